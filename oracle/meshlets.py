"""ctypes bindings for the re-clusterization oracle -- TEST INFRASTRUCTURE ONLY.

``kind="port"``: ``mo_buildMeshletsFlex`` in ``libmo_oracle.so`` (``mo_meshlet.c``, the plain-C
restatement of ``src/clusterizer.cpp:1035-1224``). ``kind="reference"``: the reference's own
``meshopt_buildMeshletsFlex``, compiled unmodified into ``_ref/libclod_ref.so`` (built only where
the reference sources are present). Only the tests and bench.py's CPU-baseline leg use this.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_PATH = os.path.join(HERE, "libmo_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libclod_ref.so")

_fns: dict = {}


def available(kind: str) -> bool:
    return os.path.isfile(PORT_PATH if kind == "port" else REF_PATH)


def _fn(kind):
    if kind not in _fns:
        lib = C.CDLL(PORT_PATH if kind == "port" else REF_PATH)
        prefix = "mo_" if kind == "port" else "meshopt_"
        f = getattr(lib, prefix + "buildMeshletsFlex")
        f.restype = C.c_size_t
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_size_t, C.c_size_t, C.c_size_t,
                      C.c_size_t, C.c_float, C.c_float]
        b = getattr(lib, prefix + "buildMeshletsBound")
        b.restype = C.c_size_t
        b.argtypes = [C.c_size_t, C.c_size_t, C.c_size_t]
        _fns[kind] = (f, b)
    return _fns[kind]


def bound(index_count, max_vertices, max_triangles, kind="port"):
    return int(_fn(kind)[1](index_count, max_vertices, max_triangles))


def build_meshlets_flex(indices, positions, max_vertices, min_triangles, max_triangles, cone_weight=0.0, split_factor=2.0, kind="port"):
    """Returns (meshlets [n, 4] uint32 {vertex_offset, triangle_offset, vertex_count, triangle_count},
    meshlet_vertices uint32, meshlet_triangles uint8), trimmed to what the meshlets use."""
    f, b = _fn(kind)
    idx = np.ascontiguousarray(indices, dtype=np.uint32)
    pos = np.ascontiguousarray(positions, dtype=np.float32)
    stride = pos.shape[1] * 4 if pos.ndim == 2 else 12
    n_max = int(b(len(idx), max_vertices, min_triangles))
    meshlets = np.zeros((max(n_max, 1), 4), np.uint32)
    mverts = np.zeros(max(len(idx), 1), np.uint32)
    mtris = np.zeros(max(len(idx), 1), np.uint8)
    n = int(f(meshlets.ctypes.data, mverts.ctypes.data, mtris.ctypes.data, idx.ctypes.data, len(idx), pos.ctypes.data, len(pos), stride,
              max_vertices, min_triangles, max_triangles, C.c_float(cone_weight), C.c_float(split_factor)))
    meshlets = meshlets[:n].copy()
    if n:
        last = meshlets[-1]
        mverts = mverts[: int(last[0] + last[2])].copy()
        mtris = mtris[: int(last[1] + last[3] * 3)].copy()
    else:
        mverts = mverts[:0].copy()
        mtris = mtris[:0].copy()
    return meshlets, mverts, mtris


def optimize_meshlets(meshlets, meshlet_vertices, meshlet_triangles, level, kind="port"):
    """meshopt_optimizeMeshletLevel on every meshlet of a build result (copies returned), as a
    cluster-LOD builder's clusterize step runs it (demo/clusterlod.h:292-300)."""
    v = np.array(meshlet_vertices, dtype=np.uint32, copy=True)
    t = np.array(meshlet_triangles, dtype=np.uint8, copy=True)
    m = np.ascontiguousarray(meshlets, dtype=np.uint32)
    if kind == "port":
        # the whole loop in C (mo_optimizeMeshlets), so that timing it times the port
        key = ("opt_all", kind)
        if key not in _fns:
            f = C.CDLL(PORT_PATH).mo_optimizeMeshlets
            f.restype = None
            f.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_int]
            _fns[key] = f
        if len(m):
            _fns[key](m.ctypes.data, len(m), v.ctypes.data, t.ctypes.data, int(level))
        return v, t
    key = ("opt_one", kind)
    if key not in _fns:
        f = C.CDLL(REF_PATH).meshopt_optimizeMeshletLevel
        f.restype = None
        f.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_int]
        _fns[key] = f
    for vo, to, vc, tc in m.astype(np.uint64):
        _fns[key](v.ctypes.data + int(vo) * 4, int(vc), t.ctypes.data + int(to), int(tc), int(level))
    return v, t
