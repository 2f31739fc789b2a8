"""Seeded synthetic meshes for the simplifier workloads.

All randomness comes from splitmix64 (with Box-Muller for normals), so a seed
gives the same mesh on every machine and numpy version.

* ``heightfield(n, seed)``        -- n x n lattice over [0,1]^2, z = amp * N(0,1)
* ``fractal_heightfield(n, seed)``-- n x n lattice, z = 6-octave value noise
* ``octa_sphere(levels, seed)``   -- octahedron subdivided ``levels`` times (8*4^levels
                                     triangles, welded), radius 1 + 0.02*N(0,1), with
                                     float3 normals and equirectangular float2 UVs whose
                                     seam is split into duplicate vertices
* ``sphere_patches(count, seed)`` -- connected patches of a displaced icosphere, each
                                     with its own compact vertex buffer
"""
from __future__ import annotations

import math

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(seed: int, count: int) -> np.ndarray:
    """``count`` consecutive splitmix64 outputs for a 64-bit seed (uint64)."""
    with np.errstate(over="ignore"):
        k = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + k * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, count: int) -> np.ndarray:
    """Doubles in (0, 1) from the top 53 bits."""
    z = splitmix64(seed, count)
    return ((z >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)


def normal(seed: int, count: int) -> np.ndarray:
    """Standard normal doubles by Box-Muller (cosine branch)."""
    u = uniform(seed, 2 * count)
    u1, u2 = u[0::2], u[1::2]
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)


def grid_indices(n: int) -> np.ndarray:
    """Two triangles per quad of an n x n vertex lattice, row-major, uint32."""
    y, x = np.meshgrid(np.arange(n - 1, dtype=np.uint32), np.arange(n - 1, dtype=np.uint32), indexing="ij")
    a = (y * n + x).ravel()
    b = a + 1
    c = a + n
    d = c + 1
    tri = np.stack([a, b, c, c, b, d], axis=1).reshape(-1)
    return np.ascontiguousarray(tri, dtype=np.uint32)


def heightfield(n: int, seed: int = 1, amp: float = 0.05):
    """n x n heightfield: x, y = i/(n-1) on [0,1]^2, z = amp * N(0,1); float3 positions."""
    t = np.arange(n, dtype=np.float64) / (n - 1)
    y, x = np.meshgrid(t, t, indexing="ij")
    z = amp * normal(seed, n * n).reshape(n, n)
    pos = np.stack([x, y, z], axis=-1).reshape(-1, 3).astype(np.float32)
    return grid_indices(n), pos


def _value_noise(n: int, seed: int, octaves: int = 6, base_cells: int = 16) -> np.ndarray:
    """Fractal value noise on an n x n lattice: per octave a (cells+1)^2 lattice of
    uniform values in [-1,1], smoothstep-interpolated; frequency x2 and amplitude
    x1/2 per octave; normalised by the amplitude sum."""
    t = np.arange(n, dtype=np.float64) / (n - 1)
    total = np.zeros((n, n))
    amp, norm = 1.0, 0.0
    cells = base_cells
    for o in range(octaves):
        lat = uniform(seed * 1000003 + o, (cells + 1) * (cells + 1)).reshape(cells + 1, cells + 1) * 2.0 - 1.0
        f = t * cells
        i = np.minimum(f.astype(np.int64), cells - 1)
        s = f - i
        s = s * s * (3.0 - 2.0 * s)
        iy, ix = i[:, None], i[None, :]
        sy, sx = s[:, None], s[None, :]
        v00 = lat[iy, ix]
        v01 = lat[iy, ix + 1]
        v10 = lat[iy + 1, ix]
        v11 = lat[iy + 1, ix + 1]
        v0 = v00 + (v01 - v00) * sx
        v1 = v10 + (v11 - v10) * sx
        total += amp * (v0 + (v1 - v0) * sy)
        norm += amp
        amp *= 0.5
        cells *= 2
    return total / norm


def fractal_heightfield(n: int, seed: int = 5, amp: float = 0.05, octaves: int = 6, base_cells: int = 16):
    """n x n lattice over [0,1]^2 with z = amp * (6-octave value noise)."""
    t = np.arange(n, dtype=np.float64) / (n - 1)
    y, x = np.meshgrid(t, t, indexing="ij")
    z = amp * _value_noise(n, seed, octaves, base_cells)
    pos = np.stack([x, y, z], axis=-1).reshape(-1, 3).astype(np.float32)
    return grid_indices(n), pos


def _subdivide(verts: np.ndarray, tris: np.ndarray):
    """One 1->4 midpoint subdivision with welded midpoints projected to the unit sphere."""
    e = np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]])
    key = np.minimum(e[:, 0], e[:, 1]).astype(np.int64) * len(verts) + np.maximum(e[:, 0], e[:, 1])
    uk, inv = np.unique(key, return_inverse=True)
    a = uk // len(verts)
    b = uk % len(verts)
    mid = verts[a] + verts[b]
    mid /= np.linalg.norm(mid, axis=1, keepdims=True)
    m = inv.reshape(3, -1).T + len(verts)
    v = np.concatenate([verts, mid])
    t0, t1, t2 = tris[:, 0], tris[:, 1], tris[:, 2]
    m01, m12, m20 = m[:, 0], m[:, 1], m[:, 2]
    nt = np.stack([
        np.stack([t0, m01, m20], 1), np.stack([m01, t1, m12], 1),
        np.stack([m20, m12, t2], 1), np.stack([m01, m12, m20], 1)], 1).reshape(-1, 3)
    return v, nt


def octa_sphere(levels: int = 9, seed: int = 2, disp: float = 0.02):
    """Octahedron sphere with 8*4^levels triangles (levels=9 gives 2,097,152).

    Returns (indices uint32 [I], positions float32 [V,3], attributes float32 [V,5],
    weights float32 [5]) with attributes = (normal.xyz, u, v). The equirectangular
    UV seam (longitude pi) is split: triangles spanning it get duplicate vertices
    with the same position and u shifted by -1.
    """
    verts = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], dtype=np.float64)
    tris = np.array([[0, 2, 4], [2, 1, 4], [1, 3, 4], [3, 0, 4],
                     [2, 0, 5], [1, 2, 5], [3, 1, 5], [0, 3, 5]], dtype=np.int64)
    for _ in range(levels):
        verts, tris = _subdivide(verts, tris)
    nrm = verts / np.linalg.norm(verts, axis=1, keepdims=True)
    r = 1.0 + disp * normal(seed, len(verts))
    pos = nrm * r[:, None]
    u = np.arctan2(nrm[:, 1], nrm[:, 0]) / (2 * math.pi) + 0.5
    v = np.arccos(np.clip(nrm[:, 2], -1.0, 1.0)) / math.pi

    # seam split: in triangles whose u range exceeds 1/2, vertices with u > 1/2 get a duplicate at u - 1
    tu = u[tris]
    span = tu.max(axis=1) - tu.min(axis=1) > 0.5
    fix = span[:, None] & (tu > 0.5)
    dup_src = np.unique(tris[fix])
    dup_id = np.full(len(verts), -1, dtype=np.int64)
    dup_id[dup_src] = len(verts) + np.arange(len(dup_src))
    tris = np.where(fix, dup_id[tris], tris)
    pos = np.concatenate([pos, pos[dup_src]])
    nrm = np.concatenate([nrm, nrm[dup_src]])
    u = np.concatenate([u, u[dup_src] - 1.0])
    v = np.concatenate([v, v[dup_src]])

    attrs = np.concatenate([nrm, u[:, None], v[:, None]], axis=1).astype(np.float32)
    weights = np.array([0.5, 0.5, 0.5, 1.0, 1.0], dtype=np.float32)
    return (np.ascontiguousarray(tris.reshape(-1), dtype=np.uint32), pos.astype(np.float32), attrs, weights)


def _icosphere(levels: int):
    p = (1.0 + 5 ** 0.5) / 2
    v = np.array([[-1, p, 0], [1, p, 0], [-1, -p, 0], [1, -p, 0], [0, -1, p], [0, 1, p], [0, -1, -p], [0, 1, -p],
                  [p, 0, -1], [p, 0, 1], [-p, 0, -1], [-p, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    for _ in range(levels):
        v, f = _subdivide(v, f)
    return v, f


def sphere_patches(count: int = 4096, seed: int = 3, tmin: int = 200, tmax: int = 512, levels: int = 6, disp: float = 0.02):
    """``count`` connected triangle patches grown breadth-first from seeded triangles of a
    displaced icosphere (20*4^levels triangles); each patch's triangle count is uniform
    in [tmin, tmax]. Returns a list of (indices uint32, positions float32 [v,3]) with
    compact local vertex buffers."""
    v, f = _icosphere(levels)
    r = 1.0 + disp * normal(seed, len(v))
    pos = (v * r[:, None]).astype(np.float32)
    nt = len(f)
    # triangle adjacency through shared edges
    e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    tid = np.tile(np.arange(nt), 3)
    key = np.minimum(e[:, 0], e[:, 1]) * len(v) + np.maximum(e[:, 0], e[:, 1])
    order = np.argsort(key, kind="stable")
    ks, ts = key[order], tid[order]
    same = ks[1:] == ks[:-1]
    pa, pb = ts[:-1][same], ts[1:][same]
    nbr = [[] for _ in range(nt)]
    for a_, b_ in zip(pa.tolist(), pb.tolist()):
        nbr[a_].append(b_)
        nbr[b_].append(a_)
    u = uniform(seed + 17, 2 * count)
    out = []
    for g in range(count):
        target = tmin + int(u[2 * g] * (tmax - tmin + 1))
        start = int(u[2 * g + 1] * nt)
        seen = {start}
        queue = [start]
        head = 0
        while head < len(queue) and len(queue) < target:
            t = queue[head]
            head += 1
            for q in nbr[t]:
                if q not in seen and len(queue) < target:
                    seen.add(q)
                    queue.append(q)
        tri = f[np.array(queue)]
        uv, local = np.unique(tri.reshape(-1), return_inverse=True)
        out.append((local.astype(np.uint32), np.ascontiguousarray(pos[uv])))
    return out


def cluster_groups(levels: int = 7, group_tris: int = 1024, seed: int = 2, protect_seams: bool = True):
    """Cluster-LOD style groups over one shared vertex buffer: the octahedron sphere (normals +
    UV, seam split) cut into groups of ``group_tris`` triangles in latitude/longitude order.

    As a cluster-LOD builder prepares one level (demo/clusterlod.h lockBoundary), every
    position that two groups share is locked (bit 0 of vertex_lock) and, with protect_seams,
    vertices whose position has a duplicate with different attributes are protected (bit 1).
    Returns (groups: list of uint32 index arrays into the shared buffer, positions float32 [V,3],
    attributes float32 [V,5], weights float32 [5], lock uint8 [V])."""
    idx, pos, attr, w = octa_sphere(levels, seed=seed)
    tri = idx.reshape(-1, 3).astype(np.int64)
    c = pos[tri].mean(axis=1).astype(np.float64)
    theta = np.arccos(np.clip(c[:, 2] / np.linalg.norm(c, axis=1), -1.0, 1.0))
    phi = np.arctan2(c[:, 1], c[:, 0])
    bands = max(1, int(round(math.sqrt(len(tri) / group_tris))))
    band = np.minimum((theta / math.pi * bands).astype(np.int64), bands - 1)
    order = np.lexsort((phi, band))
    groups = [np.ascontiguousarray(tri[order[g:g + group_tris]].reshape(-1), dtype=np.uint32) for g in range(0, len(order), group_tris)]
    # position remap: the smallest vertex with the same position
    _, first, inv = np.unique(pos, axis=0, return_index=True, return_inverse=True)
    inv = inv.reshape(-1)
    remap = first[inv]
    count = np.zeros(len(pos), np.int64)
    for g in groups:
        count[np.unique(remap[g])] += 1
    lock = (count[remap] > 1).astype(np.uint8)
    if protect_seams:
        lock |= np.where(np.any(attr != attr[remap], axis=1), 2, 0).astype(np.uint8)
    return groups, pos, attr, w, lock


def lognormal_sizes(count: int, seed: int = 4, median: float = 20000.0, sigma: float = 1.0, lo: int = 1000, hi: int = 1000000):
    """Request triangle counts: lognormal(median, sigma) clipped to [lo, hi]."""
    z = normal(seed, count)
    t = np.exp(math.log(median) + sigma * z)
    return np.clip(t, lo, hi).astype(np.int64)


def target_count(index_count: int, ratio: float) -> int:
    """floor(ratio * I / 3) * 3, the target index count for a ratio of the input."""
    return int(ratio * index_count / 3) * 3


# Named workloads (sizes as the simplifier benchmarks quote them)
def config_heightfield_256():
    """256 x 256 heightfield (130,050 triangles), z = 0.05 N(0,1), 25%, error 1e-2, options 0."""
    idx, pos = heightfield(256, seed=1, amp=0.05)
    return dict(name="heightfield_256", indices=idx, positions=pos, target=target_count(len(idx), 0.25),
                error=1e-2, options=0)


def config_sphere_attr(levels: int = 9):
    """Octahedron sphere, 2,097,152 triangles at levels=9, normals (w 0.5) + UV (w 1.0), 10%, error 5e-3."""
    idx, pos, attr, w = octa_sphere(levels, seed=2)
    return dict(name=f"sphere_attr_{len(idx) // 3}", indices=idx, positions=pos, attributes=attr, weights=w,
                target=target_count(len(idx), 0.10), error=5e-3, options=0)


def config_fractal_3163(n: int = 3163):
    """3163 x 3163 fractal heightfield (19,996,488 triangles), 1%, error 5e-2."""
    idx, pos = fractal_heightfield(n, seed=5)
    return dict(name=f"fractal_{n}", indices=idx, positions=pos, target=target_count(len(idx), 0.01),
                error=5e-2, options=0)
