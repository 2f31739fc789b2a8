"""Generates the committed golden fixtures for the simplifier parity tests.

Run here, where the reference sources exist:

    make -C oracle ref clod-ref && python tests/golden/make_golden.py

It writes two files next to this script:

* ``known_answers.json`` -- the simplifier known-answer cases of the reference's own
  unit tests (demo/tests.cpp, simplify* functions). The literal vertex/index/lock
  arrays are read from that file as text; the call arguments are the ones its
  asserts use. Each case is run through the reference library compiled unmodified
  (oracle/_ref/libmeshopt_ref.so) and the expected output is recorded together with
  the assertion the reference test makes (exact buffer, count or error bound).
* ``seeded_cases.npz`` -- seeded synthetic meshes (heightfields, attribute spheres,
  lock-border patches, random lattice soups) with the reference library's outputs.
* ``clod_cases.npz`` -- two cluster-LOD levels (boundary locks from the reference builder's
  lockBoundary through oracle/clod_ref.cpp, then every group through the reference
  simplifier) over one shared vertex buffer.
* ``update_cases.npz`` -- meshopt_simplifyWithUpdate: the reference's simplifyUpdate tests
  (asserted here) and seeded meshes, with the indices, positions and attributes the reference
  leaves.
* ``meshlet_cases.npz`` -- meshopt_buildMeshletsFlex, the re-clusterization step of a
  cluster-LOD level: seeded meshes (each stored once) and the reference's meshlets for six
  parameter sets each, through the reference's own clusterizer.cpp in oracle/_ref/libclod_ref.so,
  with the meshlets after the reference's meshopt_optimizeMeshletLevel (meshletutils.cpp).
* ``compaction_cases.npz`` -- seeded inputs of the compaction step after the simplifier
  (meshopt_optimizeVertexFetchRemap, meshopt_optimizeVertexFetch,
  meshopt_generatePositionRemap) with the reference library's outputs.

The GPU machine has no reference tree; these fixtures carry its results there.
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402
from meshoptimizer_gb300 import workloads as W  # noqa: E402

REFERENCE_ROOT = os.environ.get("REFERENCE_ROOT") or os.path.join(ROOT, "..", "reference")
TESTS_CPP = os.path.join(REFERENCE_ROOT, "demo", "tests.cpp")


def _function_body(src: str, name: str) -> str:
    m = re.search(r"static void " + re.escape(name) + r"\s*\([^)]*\)\s*\{", src)
    if not m:
        raise KeyError(name)
    i, depth = m.end(), 1
    while depth:
        depth += {"{": 1, "}": -1}.get(src[i], 0)
        i += 1
    return src[m.end():i - 1]


def _eval_number(tok: str):
    tok = tok.strip()
    tok = re.sub(r"(?<=[0-9.])f\b", "", tok)
    tok = re.sub(r"(?<=[0-9])u\b", "", tok)
    return eval(tok, {"__builtins__": {}}, {})  # literal arithmetic like 0 | (9 << 28)


def _arrays(body: str) -> dict:
    """All `type name[...] = { ... };` literal arrays in a function body (flattened)."""
    out = {}
    for m in re.finditer(r"(?:const\s+)?(float|unsigned int|unsigned char)\s+(\w+)(?:\[[^\]]*\])+\s*=\s*\{", body):
        i, depth = m.end(), 1
        while depth:
            depth += {"{": 1, "}": -1}.get(body[i], 0)
            i += 1
        text = body[m.end():i - 1]
        text = re.sub(r"//[^\n]*", "", text).replace("{", " ").replace("}", " ")
        try:
            vals = [_eval_number(t) for t in text.split(",") if t.strip()]
        except SyntaxError:
            continue  # initialisers that are not literals (e.g. conditional weights) are restated by the caller
        out[m.group(2)] = (m.group(1), vals)
    return out


def _np(arrs, name):
    t, v = arrs[name]
    return np.array(v, dtype={"float": np.float32, "unsigned int": np.uint32, "unsigned char": np.uint8}[t])


def known_answer_cases():
    src = open(TESTS_CPP).read()
    cases = []

    def add(fn, name, idx, pos, stride, target, error, options=0, attrs=None, astride=0, weights=None, lock=None,
            expect=None, expect_count=None, expect_error_lt=None, expect_error_near=None):
        cases.append(dict(source=f"demo/tests.cpp:{fn}", name=name, indices=idx, positions=pos, stride=stride,
                          target=target, error=error, options=options, attributes=attrs, attr_stride=astride,
                          weights=weights, lock=lock, expect=expect, expect_count=expect_count,
                          expect_error_lt=expect_error_lt, expect_error_near=expect_error_near))

    a = _arrays(_function_body(src, "simplify"))
    add("simplify", "simplify", _np(a, "ib"), _np(a, "vb"), 12, 3, 1e-2, expect=_np(a, "expected"), expect_error_lt=1e-4)

    a = _arrays(_function_body(src, "simplifyStuck"))
    add("simplifyStuck", "stuck_tetra", _np(a, "ib1"), _np(a, "vb1"), 12, 6, 1e-3, expect_count=12)
    add("simplifyStuck", "stuck_strip_ok", _np(a, "ib2"), _np(a, "vb2"), 12, 6, 1e-3, expect_count=6)
    add("simplifyStuck", "stuck_strip_flipped", _np(a, "ib3"), _np(a, "vb2"), 12, 6, 1e-3, expect_count=9)
    add("simplifyStuck", "stuck_quad_corner", _np(a, "ib4"), _np(a, "vb4"), 12, 3, 1e-3, expect_count=6)
    add("simplifyStuck", "stuck_quad_split", _np(a, "ib5"), _np(a, "vb5"), 12, 3, 1e-3, expect_count=6)

    a = _arrays(_function_body(src, "simplifyFlip"))
    add("simplifyFlip", "flip", _np(a, "ib"), _np(a, "vb"), 12, 3, 1e-3, expect=_np(a, "expected"), expect_count=24)

    a = _arrays(_function_body(src, "simplifyDegenerate"))
    add("simplifyDegenerate", "degenerate", _np(a, "ib"), _np(a, "vb"), 12, 3, 1e-3, expect=_np(a, "expected"), expect_count=6)

    a = _arrays(_function_body(src, "simplifyLockBorder"))
    add("simplifyLockBorder", "lock_border", _np(a, "ib"), _np(a, "vb"), 12, 3, 1e-3, options=1,
        expect=_np(a, "expected"), expect_count=18)

    # simplifyAttr builds its 8x3 grid with loops; the same construction, restated
    body = _function_body(src, "simplifyAttr")
    expected = _np(_arrays(body), "expected")
    vb = np.zeros((24, 6), np.float32)
    for y in range(8):
        r = np.float32(0.8) + np.float32(y) * np.float32(0.05) if y < 4 else np.float32(0)
        b = np.float32(0) if y < 4 else np.float32(0.8) + np.float32(7 - y) * np.float32(0.05)
        for x in range(3):
            vb[y * 3 + x] = [x, y, np.float32(0.03) * x + np.float32(0.03) * (y % 2) + (x == 2 and y == 7) * np.float32(0.03), r, r, b]
    ib = []
    for y in range(7):
        for x in range(2):
            ib += [(y + 0) * 3 + (x + 0), (y + 0) * 3 + (x + 1), (y + 1) * 3 + (x + 0),
                   (y + 1) * 3 + (x + 0), (y + 0) * 3 + (x + 1), (y + 1) * 3 + (x + 1)]
    ib = np.array(ib, np.uint32)
    for skip_g in (False, True):
        w = np.array([0.5, 0.0 if skip_g else 0.5, 0.5], np.float32)
        add("simplifyAttr", f"attr_skip_g{int(skip_g)}", ib, vb.reshape(-1), 24, 18, 1e-2,
            attrs=vb.reshape(-1)[3:].copy(), astride=24, weights=w, expect=expected, expect_count=18)

    a = _arrays(_function_body(src, "simplifyLockFlags"))
    add("simplifyLockFlags", "lock_flags", _np(a, "ib"), _np(a, "vb"), 12, 3, 1e-3, lock=_np(a, "lock"),
        expect=_np(a, "expected"), expect_count=18)

    a = _arrays(_function_body(src, "simplifyLockFlagsSeam"))
    add("simplifyLockFlagsSeam", "lock_seam_none", _np(a, "ib"), _np(a, "vb"), 12, 0, 1.0, expect_count=0)
    for name, cnt in (("lock0", 12), ("lock1", 18), ("lock2", 24), ("lock3", 24)):
        add("simplifyLockFlagsSeam", f"lock_seam_{name}", _np(a, "ib"), _np(a, "vb"), 12, 0, 1.0, lock=_np(a, name), expect_count=cnt)

    a = _arrays(_function_body(src, "simplifySparse"))
    add("simplifySparse", "sparse", _np(a, "ib"), _np(a, "vb"), 12, 6, 1e-3, options=2, expect=_np(a, "expected"), expect_count=6)
    add("simplifySparse", "sparse_attr", _np(a, "ib"), _np(a, "vb"), 12, 6, 1e-1, options=2, attrs=_np(a, "vba"), astride=4,
        weights=_np(a, "aw"), lock=_np(a, "lock"), expect=_np(a, "expecteda"), expect_count=6)

    a = _arrays(_function_body(src, "simplifyErrorAbsolute"))
    add("simplifyErrorAbsolute", "error_absolute", _np(a, "ib"), _np(a, "vb"), 12, 18, 2.0, options=1 | 4,
        expect_count=18, expect_error_near=(0.85, 0.01))

    a = _arrays(_function_body(src, "simplifySeam"))
    vb = _np(a, "vb")
    add("simplifySeam", "seam", _np(a, "ib"), vb, 16, 12, 1.0, expect=_np(a, "expected"), expect_count=12,
        expect_error_near=(0.1, 0.01))
    add("simplifySeam", "seam_attr", _np(a, "ib"), vb, 16, 12, 2.0, attrs=vb[3:].copy(), astride=16,
        weights=np.array([1.0], np.float32), expect=_np(a, "expected"), expect_count=12, expect_error_near=(0.1, 0.01))

    a = _arrays(_function_body(src, "simplifySeamFake"))
    add("simplifySeamFake", "seam_fake", _np(a, "ib"), _np(a, "vb"), 16, 0, 1.0, expect_count=6)

    a = _arrays(_function_body(src, "simplifySeamAttr"))
    vb = _np(a, "vb")
    add("simplifySeamAttr", "seam_attr_lockborder", _np(a, "ib"), vb, 16, 12, 2.0, options=1, attrs=vb[3:].copy(), astride=16,
        weights=np.array([1.0], np.float32), expect=_np(a, "expected"), expect_count=18, expect_error_near=(0.35, 0.01))

    a = _arrays(_function_body(src, "simplifyPrune"))
    add("simplifyPrune", "prune", _np(a, "ib"), _np(a, "vb"), 12, 3, 1e-2, options=8, expect=_np(a, "expected"), expect_count=3,
        expect_error_lt=1e-4)
    add("simplifyPrune", "prune_subset", _np(a, "expected"), _np(a, "vb"), 12, 3, 1e-2, options=8, expect_count=3)
    add("simplifyPrune", "prune_subset_sparse", _np(a, "expected"), _np(a, "vb"), 12, 3, 1e-2, options=8 | 2, expect=_np(a, "expected"),
        expect_count=3)

    a = _arrays(_function_body(src, "simplifyPruneCleanup"))
    add("simplifyPruneCleanup", "prune_cleanup", _np(a, "ib"), _np(a, "vb"), 12, 3, 1.0, options=1 | 8, expect=_np(a, "expected"),
        expect_count=3, expect_error_near=(0.37, 0.01))

    a = _arrays(_function_body(src, "simplifyDebug"))
    add("simplifyDebug", "debug_kinds", _np(a, "ib"), _np(a, "vb"), 12, 3, 1e-2, options=1 << 30,
        expect=_np(a, "expected"), expect_count=3, expect_error_lt=1e-4)
    return cases


def _run_ref(c):
    """Calls the reference library with the case's exact buffers and strides."""
    import ctypes as C
    o = oracle.load("ref")
    idx = np.ascontiguousarray(c["indices"], np.uint32)
    pos = np.ascontiguousarray(c["positions"], np.float32)
    vcount = len(pos) * 4 // c["stride"]
    out = np.zeros(max(len(idx), 1), np.uint32)
    err = C.c_float(0)
    attrs = c["attributes"]
    weights = c["weights"]
    lock = c["lock"]
    acount = 0 if weights is None else len(weights)
    p = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)  # noqa: E731
    if attrs is None and lock is None:
        n = o._simplify(p(out), p(idx), len(idx), p(pos), vcount, c["stride"], c["target"], c["error"], c["options"], C.byref(err))
    else:
        attrs = None if attrs is None else np.ascontiguousarray(attrs, np.float32)
        n = o._simplify_attr(p(out), p(idx), len(idx), p(pos), vcount, c["stride"], p(attrs), c["attr_stride"],
                             p(weights), acount, p(lock), c["target"], c["error"], c["options"], C.byref(err))
    return out[:n].copy(), float(err.value)


def _check_expectation(c, out, err):
    if c["expect"] is not None:
        assert np.array_equal(out[:len(c["expect"])], c["expect"]), c["name"]
    if c["expect_count"] is not None:
        assert len(out) == c["expect_count"], (c["name"], len(out))
    if c["expect_error_lt"] is not None:
        assert err < c["expect_error_lt"], c["name"]
    if c["expect_error_near"] is not None:
        v, tol = c["expect_error_near"]
        assert abs(err - v) < tol, (c["name"], err)


def _listify(v):
    if isinstance(v, np.ndarray):
        if v.dtype == np.float32:
            return [float(x) for x in v]
        return [int(x) for x in v]
    return v


def seeded_cases():
    rng = np.random.default_rng(20261203)
    cases = []
    for n, amp, opt in ((9, 0.05, 0), (17, 0.05, 0), (33, 0.1, 1), (24, 0.0, 0)):
        idx, pos = W.heightfield(n, seed=n, amp=amp)
        cases.append(dict(name=f"heightfield_{n}_{opt}", indices=idx, positions=pos, target=W.target_count(len(idx), 0.25),
                          error=1e-2, options=opt))
    for lv in (2, 3, 4):
        idx, pos, attr, w = W.octa_sphere(lv, seed=lv)
        cases.append(dict(name=f"sphere_attr_{lv}", indices=idx, positions=pos, attributes=attr, weights=w,
                          target=W.target_count(len(idx), 0.10), error=5e-3, options=0))
        cases.append(dict(name=f"sphere_pos_{lv}", indices=idx, positions=pos, target=W.target_count(len(idx), 0.2),
                          error=5e-2, options=0))
    for g, (idx, pos) in enumerate(W.sphere_patches(6, seed=11, levels=5)):
        cases.append(dict(name=f"patch_{g}", indices=idx, positions=pos, target=W.target_count(len(idx), 0.5),
                          error=2e-2, options=1))
    for s in range(8):
        v = rng.integers(0, 10, size=(100, 3)).astype(np.float32)
        idx = rng.integers(0, 100, size=3 * int(rng.integers(10, 120))).astype(np.uint32)
        cases.append(dict(name=f"lattice_soup_{s}", indices=idx, positions=v, target=0, error=float(np.finfo(np.float32).max),
                          options=int([0, 1, 4, 16][s % 4])))
    for c in cases:
        out, err = oracle.simplify("ref", c["indices"], c["positions"], c["target"], c["error"], c["options"],
                                   attributes=c.get("attributes"), weights=c.get("weights"))
        c["expect"], c["expect_error"] = out, err
    return cases


def compaction_cases():
    """Seeded inputs for meshopt_optimizeVertexFetchRemap / meshopt_optimizeVertexFetch /
    meshopt_generatePositionRemap: index soups with unused vertices, a simplified heightfield,
    an empty index buffer, vertex sizes 1..256 bytes, positions with duplicates, -0 and NaN."""
    rng = np.random.default_rng(2024)
    cases = []
    for vc, ic, size in ((1, 3, 12), (17, 30, 7), (1000, 2400, 16), (300, 0, 4), (600, 3000, 256), (64, 96, 1)):
        idx = rng.integers(0, vc, size=ic).astype(np.uint32)
        verts = rng.integers(0, 256, size=(vc, size)).astype(np.uint8)
        cases.append(dict(kind="fetch", indices=idx, vertices=verts))
    hi, hp = W.heightfield(64, seed=9)
    out, _ = oracle.simplify("reference", hi, hp, W.target_count(len(hi), 0.2), 1e-2, 0)
    cases.append(dict(kind="fetch", indices=out, vertices=np.ascontiguousarray(hp).view(np.uint8).reshape(len(hp), 12)))
    for vc, k in ((1, 3), (200, 3), (3000, 4), (777, 8)):
        pos = rng.integers(-2, 3, size=(vc, k)).astype(np.float32) * 0.5
        pos[rng.random(vc) < 0.05, 0] = np.nan
        pos[rng.random(vc) < 0.1, 1] = -0.0
        cases.append(dict(kind="remap", positions=pos))
    for c in cases:
        if c["kind"] == "fetch":
            vc = c["vertices"].shape[0]
            c["remap"], c["count"] = oracle.optimize_vertex_fetch_remap("reference", c["indices"], vc)
            c["new_indices"], new_vertices, n = oracle.optimize_vertex_fetch("reference", c["indices"], c["vertices"])
            assert n == c["count"]
            # the moved vertex buffer follows from the remap (vertex v lands at remap[v])
            used = c["remap"] != 0xFFFFFFFF
            assert np.array_equal(new_vertices[c["remap"][used]], c["vertices"][used])
        else:
            c["remap"] = oracle.generate_position_remap("reference", c["positions"])
    return cases


def clod_cases():
    """Two cluster-LOD levels over the attribute sphere's shared vertex buffer: level 1 groups
    are latitude/longitude bands of triangles, level 2 groups concatenate pairs of level-1
    results. Each level runs the reference builder's lockBoundary (through the
    oracle/clod_ref.cpp harness) and then the reference simplifier on every group with
    Sparse | ErrorAbsolute | Permissive and the level's locks (demo/clusterlod.h:461-479)."""
    import clod

    rng = np.random.default_rng(77)
    cases = []
    for levels, group_tris in ((4, 64), (5, 256)):
        groups, pos, attr, w, _ = W.cluster_groups(levels, group_tris)
        remap = oracle.generate_position_remap("reference", pos)
        locks = np.where(np.any(attr != attr[remap], axis=1), 2, 0).astype(np.uint8)
        vl = rng.choice(np.array([0, 1, 2, 4], np.uint8), size=len(pos), p=[0.96, 0.01, 0.01, 0.02])
        c = dict(positions=pos, attributes=attr, weights=w, remap=remap, locks_in=locks.copy(), vertex_lock=vl,
                 options=np.array(2 | 4 | 32), error=np.array(np.finfo(np.float32).max, np.float32))
        for level in (1, 2):
            locks = clod.reference_lock_boundary(locks, groups, remap, vl)
            targets = [(len(g) // 6) * 3 for g in groups]
            outs = [oracle.simplify("reference", g, pos, t, float(c["error"]), int(c["options"]), attributes=attr, weights=w, lock=locks)
                    for g, t in zip(groups, targets)]
            off = np.zeros(len(groups) + 1, np.uint64)
            off[1:] = np.cumsum([len(g) for g in groups])
            c[f"l{level}_indices"] = np.concatenate(groups).astype(np.uint32)
            c[f"l{level}_offsets"] = off
            c[f"l{level}_targets"] = np.array(targets, np.uint64)
            c[f"l{level}_locks"] = locks.copy()
            c[f"l{level}_out"] = np.concatenate([o for o, _ in outs]).astype(np.uint32)
            c[f"l{level}_counts"] = np.array([len(o) for o, _ in outs], np.uint64)
            c[f"l{level}_errors"] = np.array([e for _, e in outs], np.float32)
            groups = [np.concatenate([outs[i][0], outs[i + 1][0]]) if i + 1 < len(outs) else outs[i][0] for i in range(0, len(outs), 2)]
        cases.append(c)
    return cases


def _parts(seed):
    """Several disconnected heightfield pieces of different sizes and scales in one buffer."""
    rng = np.random.default_rng(seed)
    parts_idx, parts_pos, base = [], [], 0
    for p in range(int(rng.integers(3, 7))):
        n = int(rng.integers(3, 14))
        idx, pos = W.heightfield(n, seed=seed * 10 + p, amp=0.05)
        pos = pos * np.float32(rng.uniform(0.05, 1.0)) + rng.uniform(-2, 2, size=3).astype(np.float32)
        parts_idx.append(idx + base)
        parts_pos.append(pos)
        base += len(pos)
    return np.concatenate(parts_idx).astype(np.uint32), np.concatenate(parts_pos).astype(np.float32)


def update_cases():
    """meshopt_simplifyWithUpdate: the reference's simplifyUpdate / simplifyUpdateLocked tests
    (demo/tests.cpp:2590-2665; one interleaved buffer, their asserts checked here) and seeded
    meshes with separate position and attribute arrays."""
    body = _function_body(open(TESTS_CPP).read(), "simplifyUpdate")
    vb = np.array(_np(_arrays(body), "vb"), np.float32)
    ib = np.array(_np(_arrays(body), "ib"), np.uint32)
    expected = np.array([0, 1, 3, 3, 1, 2, 0, 3, 2], np.uint32)
    cases = []
    for name, lock, options in (("simplifyUpdate", None, 0), ("simplifyUpdateLocked", np.array([0, 0, 0, 1, 0], np.uint8), 0),
                                ("simplifyUpdateLocked_sparse", np.array([0, 0, 0, 1, 0], np.uint8), 2)):
        out, v, err = oracle.simplify_with_update_interleaved("reference", ib, vb, 4, 3, [1.0], lock, 9, 1.0, options)
        assert np.array_equal(out, expected), name
        vv = v.reshape(-1, 4)
        assert all(abs(vv[i][3]) < 1e-6 for i in range(3)), name
        if lock is None:
            assert abs(vv[3][0] - 0.88) < 1e-2 and abs(vv[3][1] - 0.19) < 1e-2 and abs(vv[3][2] - 0.11) < 1e-2 and abs(vv[3][3] - 0.18) < 1e-2
        else:
            assert vv[3][0] == np.float32(0.9) and vv[3][1] == np.float32(0.2) and vv[3][2] == np.float32(0.1) and vv[3][3] == np.float32(0.2)
        cases.append(dict(name=name, kind="interleaved", indices=ib, vertices=vb, lock=lock, options=np.array(options), target=np.array(9),
                          error=np.array(1.0, np.float32), out=out, out_vertices=v, out_error=np.array(err, np.float32)))
    rng = np.random.default_rng(99)
    seeded = []
    for n in (16, 33):
        idx, pos = W.heightfield(n, seed=n)
        seeded.append((f"update_hf{n}", idx, pos, None, None, None, W.target_count(len(idx), 0.3), 1e-1, 0))
    for lv in (3, 4):
        idx, pos, attr, w = W.octa_sphere(lv, seed=lv)
        lock = rng.choice(np.array([0, 0, 0, 1, 2, 4], np.uint8), size=len(pos))
        seeded.append((f"update_sphere{lv}_attr", idx, pos, attr, w, None, W.target_count(len(idx), 0.25), 5e-2, 0))
        seeded.append((f"update_sphere{lv}_attr_lock_permissive", idx, pos, attr, w, lock, W.target_count(len(idx), 0.25), 5e-2, 32))
        half = idx[: (len(idx) // 6) * 3]
        seeded.append((f"update_sphere{lv}_sparse", half, pos, attr, w, None, W.target_count(len(half), 0.25), 5e-2, 2 | 4))
    # Prune (8) removes whole pieces before the solve; the debug bit (1 << 30) tags the indices after it
    # (LockBorder keeps open pieces from collapsing away on their own, so pruning decides the result)
    for seed, ratio, error, options in ((201, 0.1, 0.2, 8 | 1), (203, 0.2, 5e-2, 8 | 1), (205, 0.1, 0.5, 8 | 1 | 4), (202, 0.1, 0.2, 8 | 1)):
        idx, pos = _parts(seed)
        seeded.append((f"update_parts{seed}_prune_{options}", idx, pos, None, None, None, W.target_count(len(idx), ratio), error, options))
    idx, pos = W.heightfield(12, seed=4)
    seeded.append(("update_hf12_debug", idx, pos, None, None, None, W.target_count(len(idx), 0.3), 5e-2, 1 << 30))
    for name, idx, pos, attr, w, lock, target, error, options in seeded:
        out, p2, a2, err = oracle.simplify_with_update("reference", idx, pos, target, error, options, attributes=attr, weights=w, lock=lock)
        c = dict(name=name, kind="separate", indices=idx, positions=pos, target=np.array(target), error=np.array(error, np.float32),
                 options=np.array(options), out=out, out_positions=p2, out_error=np.array(err, np.float32))
        if attr is not None:
            c.update(attributes=attr, weights=w, out_attributes=a2)
        if lock is not None:
            c["lock"] = lock
        cases.append(c)
    return cases


def meshlet_cases():
    """meshopt_buildMeshletsFlex (src/clusterizer.cpp:1035), the reference's own build: dense and
    sparse (index subsets of a larger buffer) meshes, degenerate and zero-area triangles, a NaN
    position, and parameters from clusterlod's defaults to the extremes the asserts allow."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import meshlets as ML

    rng = np.random.default_rng(77)
    meshes = []
    idx, pos = W.heightfield(24, seed=3)
    meshes.append(("hf24", idx, pos))
    idx, pos, _, _ = W.octa_sphere(4, seed=4)
    meshes.append(("sphere4", idx, pos))
    idx, pos, _, _ = W.octa_sphere(5, seed=2)
    tri = idx.reshape(-1, 3)
    for g in range(3):
        s0 = int(rng.integers(0, len(tri) - 1100))
        meshes.append((f"sphere5_subset{g}", tri[s0:s0 + int(rng.integers(200, 1000))].reshape(-1).copy(), pos))
    idx, pos = W.heightfield(12, seed=5)
    t = idx.reshape(-1, 3).copy()
    t[::7, 1] = t[::7, 0]  # degenerate triangles (a repeated vertex)
    meshes.append(("hf12_degenerate", t.reshape(-1), pos))
    idx, pos = W.heightfield(10, seed=6, amp=0.0)
    flat = pos.copy()
    flat[:, 1] = 0.0  # every triangle has zero area
    meshes.append(("hf10_zero_area", idx, flat))
    idx, pos = W.heightfield(10, seed=7)
    nanpos = pos.copy()
    nanpos[5, 0] = np.nan
    meshes.append(("hf10_nan", idx, nanpos))
    meshes.append(("one_triangle", np.array([0, 1, 2], np.uint32), np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)))
    params = [(128, 42, 128, 0.0, 2.0), (64, 21, 64, 0.0, 2.0), (64, 16, 124, 0.25, 0.0), (255, 85, 256, 1.0, 1.5), (3, 1, 1, 0.0, 2.0),
              (256, 512, 512, 0.5, 4.0)]
    cases = []
    for j, (name, idx, pos) in enumerate(meshes):
        for mv, mint, maxt, cw, sf in params:
            m, v, tr = ML.build_meshlets_flex(idx, pos, mv, mint, maxt, cw, sf, kind="reference")
            c = dict(name=f"{name}_{mv}_{mint}_{maxt}_{cw}_{sf}", mesh=np.array(j), max_vertices=np.array(mv), min_triangles=np.array(mint),
                     max_triangles=np.array(maxt), cone_weight=np.array(cw, np.float32), split_factor=np.array(sf, np.float32), meshlets=m,
                     meshlet_vertices=v, meshlet_triangles=tr)
            # meshopt_optimizeMeshletLevel on every meshlet (src/meshletutils.cpp:366): clusterlod's
            # level 1 everywhere, levels 0 and 5 on every other case
            for level in ((1, 0, 5) if len(cases) % 2 == 0 else (1,)):
                ov, ot = ML.optimize_meshlets(m, v, tr, level, kind="reference")
                c[f"opt{level}_meshlet_vertices"] = ov
                c[f"opt{level}_meshlet_triangles"] = ot
            cases.append(c)
    return [(np.asarray(idx, np.uint32), np.asarray(pos, np.float32)) for _, idx, pos in meshes], cases


def main():
    ka = known_answer_cases()
    js = []
    for c in ka:
        out, err = _run_ref(c)
        _check_expectation(c, out, err)
        d = {k: _listify(v) for k, v in c.items()}
        d["ref_output"] = [int(x) for x in out]
        d["ref_error"] = err
        js.append(d)
    with open(os.path.join(HERE, "known_answers.json"), "w") as f:
        json.dump(js, f, indent=None, separators=(",", ":"))
    print(f"known answers: {len(js)} cases")

    sc = seeded_cases()
    blob = {}
    meta = []
    for i, c in enumerate(sc):
        for k in ("indices", "positions", "attributes", "weights", "expect"):
            if c.get(k) is not None:
                blob[f"{i}_{k}"] = np.asarray(c[k])
        meta.append(dict(name=c["name"], target=c["target"], error=c["error"], options=c["options"],
                         expect_error=c["expect_error"], has_attr=c.get("attributes") is not None))
    blob["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, "seeded_cases.npz"), **blob)
    print(f"seeded cases: {len(sc)}")

    cc = compaction_cases()
    blob = {}
    for i, c in enumerate(cc):
        for k, v in c.items():
            blob[f"{i}_{k}"] = np.asarray(v)
    blob["count"] = np.array(len(cc))
    np.savez_compressed(os.path.join(HERE, "compaction_cases.npz"), **blob)
    print(f"compaction cases: {len(cc)}")

    kc = clod_cases()
    blob = {}
    for i, c in enumerate(kc):
        for k, v in c.items():
            blob[f"{i}_{k}"] = np.asarray(v)
    blob["count"] = np.array(len(kc))
    np.savez_compressed(os.path.join(HERE, "clod_cases.npz"), **blob)
    print(f"cluster-LOD cases: {len(kc)}")

    uc = update_cases()
    blob = {}
    for i, c in enumerate(uc):
        for k, v in c.items():
            if v is not None:
                blob[f"{i}_{k}"] = np.asarray(v)
    blob["count"] = np.array(len(uc))
    np.savez_compressed(os.path.join(HERE, "update_cases.npz"), **blob)
    print(f"update cases: {len(uc)}")

    mm, mc = meshlet_cases()
    blob = {}
    for j, (idx, pos) in enumerate(mm):
        blob[f"mesh{j}_indices"] = idx
        blob[f"mesh{j}_positions"] = pos
    for i, c in enumerate(mc):
        for k, v in c.items():
            blob[f"{i}_{k}"] = np.asarray(v)
    blob["count"] = np.array(len(mc))
    np.savez_compressed(os.path.join(HERE, "meshlet_cases.npz"), **blob)
    print(f"meshlet cases: {len(mc)}")


if __name__ == "__main__":
    main()
