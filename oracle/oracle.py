"""ctypes bindings for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Two libraries can sit behind this module:

* ``libmo_oracle.so`` -- the plain-C restatement in ``mo_oracle.c`` (``kind="port"``),
  built on any machine by ``make -C oracle``;
* ``_ref/libmeshopt_ref.so`` -- meshoptimizer's own ``src/simplifier.cpp`` and
  ``src/allocator.cpp`` compiled unmodified (``kind="reference"``), built only where
  the reference sources are present (``make -C oracle ref``).

Only the tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module; the product library never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_PATH = os.path.join(HERE, "libmo_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libmeshopt_ref.so")

MAX_PASSES = 128


class Stats(C.Structure):
    _fields_ = [
        ("passes", C.c_uint),
        ("tri", C.c_uint * MAX_PASSES),
        ("cand", C.c_uint * MAX_PASSES),
        ("evaluated", C.c_uint * MAX_PASSES),
        ("done", C.c_uint * MAX_PASSES),
        ("skipped", C.c_uint * MAX_PASSES),
        ("invalid", C.c_uint * MAX_PASSES),
        ("stop", C.c_uint * MAX_PASSES),
        ("result_error_sq", C.c_float),
        ("error_limit", C.c_float),
    ]

    def as_dict(self):
        n = min(self.passes, MAX_PASSES)
        keys = ["tri", "cand", "evaluated", "done", "skipped", "invalid", "stop"]
        d = {k: list(getattr(self, k))[:n] for k in keys}
        d["passes"] = int(self.passes)
        d["result_error_sq"] = float(self.result_error_sq)
        d["error_limit"] = float(self.error_limit)
        return d


class SetupDump(C.Structure):
    _fields_ = [
        ("remap", C.c_void_p),
        ("wedge", C.c_void_p),
        ("kind", C.c_void_p),
        ("loop", C.c_void_p),
        ("loopback", C.c_void_p),
        ("positions", C.c_void_p),
        ("quadrics", C.c_void_p),
        ("attr_quadrics", C.c_void_p),
        ("attr_gradients", C.c_void_p),
        ("capacity", C.c_size_t),
        ("scale", C.c_float),
    ]


def reference_root() -> str:
    """Where the reference's sources are: $REFERENCE_ROOT, else a `reference` checkout beside
    this repository. Only the build of the reference library and fixture generation read it."""
    return os.environ.get("REFERENCE_ROOT") or os.path.join(os.path.dirname(HERE), "..", "reference")


def build(with_reference: bool = True) -> None:
    """Compile the port and, where the reference sources exist, the reference library."""
    subprocess.run(["make", "-s", "-C", HERE, "libmo_oracle.so"], check=True)
    ref_root = reference_root()
    if with_reference and os.path.isfile(os.path.join(ref_root, "src", "simplifier.cpp")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFERENCE_ROOT={ref_root}"], check=True)
        if os.path.isfile(os.path.join(ref_root, "demo", "clusterlod.h")):
            subprocess.run(["make", "-s", "-C", HERE, "clod-ref", f"REFERENCE_ROOT={ref_root}"], check=True)


_libs: dict = {}


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _bind_simplify(lib, prefix):
    f = getattr(lib, prefix + "simplify")
    f.restype = C.c_size_t
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_size_t,
                  C.c_size_t, C.c_float, C.c_uint, C.c_void_p]
    g = getattr(lib, prefix + "simplifyWithAttributes")
    g.restype = C.c_size_t
    g.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_size_t,
                  C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p,
                  C.c_size_t, C.c_float, C.c_uint, C.c_void_p]
    s = getattr(lib, prefix + "simplifyScale")
    s.restype = C.c_float
    s.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t]
    return f, g, s


def available(kind: str) -> bool:
    return os.path.isfile(PORT_PATH if kind == "port" else REF_PATH)


def load(kind: str = "port"):
    """Returns a small object with simplify/simplifyWithAttributes/simplifyScale."""
    if kind in _libs:
        return _libs[kind]
    path = PORT_PATH if kind == "port" else REF_PATH
    if not os.path.isfile(path):
        raise FileNotFoundError(f"oracle library {path} is not built")
    lib = C.CDLL(path)
    prefix = "mo_" if kind == "port" else "meshopt_"
    f, g, s = _bind_simplify(lib, prefix)

    class _O:
        pass

    o = _O()
    o.kind = kind
    o.lib = lib
    o._simplify, o._simplify_attr, o._scale = f, g, s
    if kind == "port":
        e = lib.mo_simplify_edge
        e.restype = C.c_size_t
        e.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_size_t,
                      C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p,
                      C.c_size_t, C.c_float, C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p]
        o._edge = e
        e64 = lib.mo_simplify_edge_f64
        e64.restype = C.c_size_t
        e64.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_size_t,
                        C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p,
                        C.c_size_t, C.c_float, C.c_uint, C.c_void_p, C.c_void_p]
        o._edge64 = e64
    _libs[kind] = o
    return o


def simplify(kind, indices, positions, target_index_count, target_error, options=0,
             attributes=None, weights=None, lock=None, stats=False, dump=False, fp64=False):
    """Runs the oracle on numpy inputs.

    indices: uint32 [I]; positions: float32 [V, k>=3] (row stride = k*4 bytes);
    attributes: float32 [V, a] or None; weights: float32 [a]; lock: uint8 [V] or None.
    Returns (out_indices, result_error[, stats_dict][, dump_dict]).
    """
    o = load(kind)
    indices = np.ascontiguousarray(indices, dtype=np.uint32)
    positions = np.ascontiguousarray(positions, dtype=np.float32)
    vcount = positions.shape[0]
    pstride = positions.shape[1] * 4
    out = np.zeros(max(len(indices), 1), dtype=np.uint32)
    err = C.c_float(0)
    acount = 0
    astride = 0
    if attributes is not None:
        attributes = np.ascontiguousarray(attributes, dtype=np.float32)
        weights = np.ascontiguousarray(weights, dtype=np.float32)
        acount = attributes.shape[1]
        astride = acount * 4
    if lock is not None:
        lock = np.ascontiguousarray(lock, dtype=np.uint8)

    extra = []
    if fp64:
        err64 = C.c_double(0)
        st = Stats()
        n = o._edge64(_ptr(out), _ptr(indices), len(indices), _ptr(positions), vcount, pstride,
                      _ptr(attributes), astride, _ptr(weights), acount, _ptr(lock),
                      int(target_index_count), float(target_error), int(options), C.byref(err64), C.byref(st))
        return out[:n].copy(), float(err64.value), st.as_dict()
    if stats or dump:
        if kind != "port":
            raise ValueError("stats/dump are only available from the port")
        st = Stats()
        dp = None
        arrays = {}
        if dump:
            a = attributes.shape[1] if attributes is not None else 0
            arrays = dict(
                remap=np.zeros(vcount, np.uint32), wedge=np.zeros(vcount, np.uint32),
                kind=np.zeros(vcount, np.uint8), loop=np.zeros(vcount, np.uint32),
                loopback=np.zeros(vcount, np.uint32), positions=np.zeros((vcount, 3), np.float32),
                quadrics=np.zeros((vcount, 11), np.float32),
                attr_quadrics=np.zeros((vcount, 11), np.float32),
                attr_gradients=np.zeros((vcount, max(4 * a, 1)), np.float32))
            dp = SetupDump(**{k: v.ctypes.data for k, v in arrays.items()})
        n = o._edge(_ptr(out), _ptr(indices), len(indices), _ptr(positions), vcount, pstride,
                    _ptr(attributes), astride, _ptr(weights), acount, _ptr(lock),
                    int(target_index_count), float(target_error), int(options), C.byref(err),
                    C.byref(st), C.byref(dp) if dp is not None else None)
        res = [out[:n].copy(), float(err.value)]
        if stats:
            res.append(st.as_dict())
        if dump:
            arrays["capacity"] = int(dp.capacity)
            arrays["scale"] = float(dp.scale)
            res.append(arrays)
        return tuple(res)
    if attributes is None and lock is None:
        n = o._simplify(_ptr(out), _ptr(indices), len(indices), _ptr(positions), vcount, pstride,
                        int(target_index_count), float(target_error), int(options), C.byref(err))
    else:
        n = o._simplify_attr(_ptr(out), _ptr(indices), len(indices), _ptr(positions), vcount, pstride,
                             _ptr(attributes), astride, _ptr(weights), acount, _ptr(lock),
                             int(target_index_count), float(target_error), int(options), C.byref(err))
    return out[:n].copy(), float(err.value)


def _bind_compaction(o, prefix):
    lib = o.lib
    r = getattr(lib, prefix + "optimizeVertexFetchRemap")
    r.restype = C.c_size_t
    r.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t]
    f = getattr(lib, prefix + "optimizeVertexFetch")
    f.restype = C.c_size_t
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_size_t]
    g = getattr(lib, prefix + "generatePositionRemap")
    g.restype = None
    g.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t]
    return r, f, g


def optimize_vertex_fetch_remap(kind, indices, vertex_count):
    """meshopt_optimizeVertexFetchRemap: (remap uint32 [vertex_count], used count)."""
    o = load(kind)
    r, _, _ = _bind_compaction(o, "mo_" if kind == "port" else "meshopt_")
    indices = np.ascontiguousarray(indices, dtype=np.uint32)
    out = np.zeros(max(vertex_count, 1), np.uint32)
    n = r(_ptr(out), _ptr(indices), len(indices), vertex_count)
    return out[:vertex_count], int(n)


def optimize_vertex_fetch(kind, indices, vertices):
    """meshopt_optimizeVertexFetch on a [V, k] array of vertices (any dtype, one row per vertex):
    returns (new indices, new vertices[:used], used)."""
    o = load(kind)
    _, f, _ = _bind_compaction(o, "mo_" if kind == "port" else "meshopt_")
    idx = np.array(indices, dtype=np.uint32, copy=True)
    verts = np.ascontiguousarray(vertices)
    dst = np.zeros_like(verts)
    n = f(_ptr(dst), _ptr(idx), len(idx), _ptr(verts), verts.shape[0], verts.strides[0] if verts.ndim > 1 else verts.itemsize)
    return idx, dst[:n], int(n)


def generate_position_remap(kind, positions):
    """meshopt_generatePositionRemap: uint32 [V]."""
    o = load(kind)
    _, _, g = _bind_compaction(o, "mo_" if kind == "port" else "meshopt_")
    positions = np.ascontiguousarray(positions, dtype=np.float32)
    out = np.zeros(max(positions.shape[0], 1), np.uint32)
    g(_ptr(out), _ptr(positions), positions.shape[0], positions.shape[1] * 4)
    return out[:positions.shape[0]]


def simplify_with_update(kind, indices, positions, target_index_count, target_error, options=0, attributes=None, weights=None, lock=None):
    """meshopt_simplifyWithUpdate on copies of the inputs: returns (indices, positions, attributes,
    result_error) with the positions (and attributes) as the call leaves them."""
    o = load(kind)
    f = getattr(o.lib, ("mo_" if kind == "port" else "meshopt_") + "simplifyWithUpdate")
    f.restype = C.c_size_t
    f.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p,
                  C.c_size_t, C.c_float, C.c_uint, C.c_void_p]
    idx = np.array(indices, dtype=np.uint32, copy=True)
    pos = np.array(positions, dtype=np.float32, copy=True)
    attr = None if attributes is None else np.array(attributes, dtype=np.float32, copy=True)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float32)
    lk = None if lock is None else np.ascontiguousarray(lock, dtype=np.uint8)
    err = C.c_float(0)
    n = f(_ptr(idx), len(idx), _ptr(pos), pos.shape[0], pos.shape[1] * 4, _ptr(attr), 0 if attr is None else attr.shape[1] * 4, _ptr(w),
          0 if w is None else len(w), _ptr(lk), int(target_index_count), float(target_error), int(options), C.byref(err))
    return idx[:n].copy(), pos, attr, float(err.value)


def simplify_with_update_interleaved(kind, indices, vertices, stride_f, attr_offset, weights, lock, target_index_count, target_error, options=0):
    """meshopt_simplifyWithUpdate on one interleaved float vertex buffer (positions first, the
    attributes attr_offset floats into each stride_f-float vertex), on copies: returns
    (indices, vertices, result_error)."""
    o = load(kind)
    f = getattr(o.lib, ("mo_" if kind == "port" else "meshopt_") + "simplifyWithUpdate")
    f.restype = C.c_size_t
    f.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p,
                  C.c_size_t, C.c_float, C.c_uint, C.c_void_p]
    ib = np.array(indices, np.uint32, copy=True)
    v = np.array(vertices, np.float32, copy=True).reshape(-1)
    w = np.ascontiguousarray(weights, np.float32)
    lk = None if lock is None else np.ascontiguousarray(lock, np.uint8)
    err = C.c_float(0)
    n = f(_ptr(ib), len(ib), _ptr(v), len(v) // stride_f, stride_f * 4, v.ctypes.data + attr_offset * 4, stride_f * 4, _ptr(w), len(w), _ptr(lk),
          int(target_index_count), float(target_error), int(options), C.byref(err))
    return ib[:n].copy(), v, float(err.value)


def simplify_scale(kind, positions):
    o = load(kind)
    positions = np.ascontiguousarray(positions, dtype=np.float32)
    return float(o._scale(_ptr(positions), positions.shape[0], positions.shape[1] * 4))
