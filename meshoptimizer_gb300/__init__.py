"""GB300-native quadric edge-collapse simplifier (meshopt_simplify / meshopt_simplifyWithAttributes).

The product is the C ABI in ``include/meshopt_gb300.h``, implemented by the in-tree CUDA
library ``meshoptimizer_gb300/libmeshopt_gb300.so`` (built by ``meshoptimizer_gb300.build``).
This module is a thin ctypes mirror of that ABI for Python callers, tests and the
benchmark: same function names, same argument meaning (numpy arrays in place of host
pointers), same error behaviour (a nonzero status instead of an exception, plus
``check=True`` to raise). There is no CPU implementation behind it: if the library is
missing, ``load()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmeshopt_gb300.so")

# option bits (meshoptimizer.h:466-482)
SimplifyLockBorder = 1 << 0
SimplifySparse = 1 << 1
SimplifyErrorAbsolute = 1 << 2
SimplifyPrune = 1 << 3
SimplifyRegularize = 1 << 4
SimplifyPermissive = 1 << 5
SimplifyRegularizeLight = 1 << 6

# vertex_lock flags (meshoptimizer.h:488-495)
SimplifyVertex_Lock = 1 << 0
SimplifyVertex_Protect = 1 << 1
SimplifyVertex_Priority = 1 << 2

STATUS_OK = 0
STATUS_UNSUPPORTED = 1
STATUS_INVALID_ARGUMENT = 2
STATUS_CUDA_ERROR = 3
STATUS_OUT_OF_MEMORY = 4
STATUS_INTERNAL = 5

# every symbol include/meshopt_gb300.h declares
EXPORTS = [
    "meshopt_simplify", "meshopt_simplifyWithAttributes", "meshopt_simplifyScale", "meshopt_simplifyWithUpdate",
    "meshoptgpu_simplifyWithUpdateDevice",
    "meshoptgpu_getLastStatus", "meshoptgpu_getLastMessage", "meshoptgpu_getLastPassStats",
    "meshoptgpu_setTiming", "meshoptgpu_getLastPhaseTimes", "meshoptgpu_simplifyDevice",
    "meshoptgpu_workspaceBytes", "meshoptgpu_releaseThreadResources", "meshoptgpu_getLaunchCount",
    "meshoptgpu_setKernelProfile", "meshoptgpu_getKernelProfile", "meshoptgpu_simplifyScaleNoAlloc", "meshoptgpu_getLastPassPhaseTimes", "meshoptgpu_getTuning",
    "meshoptgpu_simplifyBatch", "meshoptgpu_simplifyBatchHost", "meshoptgpu_setBatchConfig", "meshoptgpu_getBatchThreads",
    "meshoptgpu_serverCreate", "meshoptgpu_serverDestroy", "meshoptgpu_serverSubmit", "meshoptgpu_serverWait", "meshoptgpu_serverStats",
    "meshoptgpu_getLastRoundTrace",
    "meshoptgpu_optimizeVertexFetchRemapDevice", "meshoptgpu_optimizeVertexFetchDevice", "meshoptgpu_generatePositionRemapDevice",
    "meshoptgpu_simplifyGroups", "meshoptgpu_buildMeshletsFlexGroups", "meshoptgpu_setDropinBatchLimit", "meshoptgpu_setDeviceLoop",
    "meshoptgpu_probeBarrierWait",
]


class PassStats(C.Structure):
    _fields_ = [(n, C.c_uint) for n in ("triangles", "candidates", "evaluated", "done", "skipped", "invalid", "stop", "rounds", "active", "windows")]


class BatchMesh(C.Structure):
    _fields_ = [("indices", C.c_void_p), ("index_count", C.c_size_t), ("vertex_positions", C.c_void_p),
                ("vertex_count", C.c_size_t), ("vertex_positions_stride", C.c_size_t), ("target_index_count", C.c_size_t),
                ("target_error", C.c_float), ("options", C.c_uint), ("destination", C.c_void_p),
                ("vertex_attributes", C.c_void_p), ("vertex_attributes_stride", C.c_size_t), ("attribute_weights", C.c_void_p),
                ("attribute_count", C.c_size_t), ("vertex_lock", C.c_void_p)]


class ServerConfig(C.Structure):
    _fields_ = [("memory_budget", C.c_size_t), ("batch_workers", C.c_int), ("large_workers", C.c_int),
                ("large_index_count", C.c_size_t), ("max_batch", C.c_int), ("batch_threads", C.c_int), ("plain", C.c_int),
                ("perform_blocks", C.c_int)]


class SimplifyError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"status {status}: {message}")
        self.status = status


_lib = None


def load():
    """Loads the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.isfile(LIB_PATH):
        raise FileNotFoundError(f"{LIB_PATH} is not built; run meshoptimizer_gb300.build.build()")
    lib = C.CDLL(LIB_PATH)
    vp, sz, f32, u32 = C.c_void_p, C.c_size_t, C.c_float, C.c_uint
    lib.meshopt_simplify.restype = sz
    lib.meshopt_simplify.argtypes = [vp, vp, sz, vp, sz, sz, sz, f32, u32, vp]
    lib.meshopt_simplifyWithAttributes.restype = sz
    lib.meshopt_simplifyWithAttributes.argtypes = [vp, vp, sz, vp, sz, sz, vp, sz, vp, sz, vp, sz, f32, u32, vp]
    lib.meshopt_simplifyScale.restype = f32
    lib.meshopt_simplifyScale.argtypes = [vp, sz, sz]
    lib.meshoptgpu_getLastStatus.restype = C.c_int
    lib.meshoptgpu_getLastMessage.restype = C.c_char_p
    lib.meshoptgpu_getLastPassStats.restype = C.c_int
    lib.meshoptgpu_getLastPassStats.argtypes = [vp, C.c_int]
    lib.meshoptgpu_setTiming.argtypes = [C.c_int]
    lib.meshoptgpu_getLastPhaseTimes.restype = C.c_int
    lib.meshoptgpu_getLastPhaseTimes.argtypes = [vp]
    lib.meshoptgpu_getLastPassPhaseTimes.restype = C.c_int
    lib.meshoptgpu_getLastPassPhaseTimes.argtypes = [vp, C.c_int]
    lib.meshoptgpu_getTuning.restype = C.c_int
    lib.meshoptgpu_getTuning.argtypes = [sz, sz, vp]
    lib.meshoptgpu_simplifyDevice.restype = sz
    lib.meshoptgpu_simplifyDevice.argtypes = [vp, vp, sz, vp, sz, sz, vp, sz, vp, sz, vp, sz, f32, u32, vp, vp]
    lib.meshoptgpu_workspaceBytes.restype = sz
    lib.meshoptgpu_workspaceBytes.argtypes = [sz, sz, sz]
    lib.meshoptgpu_getLaunchCount.restype = C.c_ulonglong
    lib.meshoptgpu_setKernelProfile.argtypes = [C.c_char_p]
    lib.meshoptgpu_getKernelProfile.argtypes = [vp, vp]
    lib.meshoptgpu_simplifyBatch.restype = C.c_int
    lib.meshoptgpu_simplifyBatch.argtypes = [vp, sz, vp, vp, vp]
    lib.meshoptgpu_simplifyBatchHost.restype = C.c_int
    lib.meshoptgpu_simplifyBatchHost.argtypes = [vp, sz, vp, vp]
    lib.meshoptgpu_setBatchConfig.argtypes = [C.c_int, C.c_uint]
    lib.meshoptgpu_getBatchThreads.restype = C.c_int
    lib.meshoptgpu_getLastRoundTrace.restype = C.c_int
    lib.meshoptgpu_getLastRoundTrace.argtypes = [vp, vp, C.c_int]
    lib.meshoptgpu_serverCreate.restype = C.c_void_p
    lib.meshoptgpu_serverCreate.argtypes = [vp]
    lib.meshoptgpu_serverDestroy.argtypes = [vp]
    lib.meshoptgpu_serverSubmit.restype = C.c_longlong
    lib.meshoptgpu_serverSubmit.argtypes = [vp, vp]
    lib.meshoptgpu_serverWait.restype = C.c_int
    lib.meshoptgpu_serverWait.argtypes = [vp, C.c_longlong, vp, vp, vp]
    lib.meshoptgpu_serverStats.argtypes = [vp, vp]
    lib.meshoptgpu_simplifyScaleNoAlloc.restype = C.c_int
    lib.meshoptgpu_simplifyScaleNoAlloc.argtypes = [vp, vp, sz, sz, vp]
    lib.meshoptgpu_optimizeVertexFetchRemapDevice.restype = sz
    lib.meshoptgpu_optimizeVertexFetchRemapDevice.argtypes = [vp, vp, sz, sz, vp]
    lib.meshoptgpu_optimizeVertexFetchDevice.restype = sz
    lib.meshoptgpu_optimizeVertexFetchDevice.argtypes = [vp, vp, sz, vp, sz, sz, vp]
    lib.meshoptgpu_generatePositionRemapDevice.restype = C.c_int
    lib.meshoptgpu_generatePositionRemapDevice.argtypes = [vp, vp, sz, sz, vp]
    lib.meshoptgpu_setDropinBatchLimit.argtypes = [sz]
    lib.meshopt_simplifyWithUpdate.restype = sz
    lib.meshopt_simplifyWithUpdate.argtypes = [vp, sz, vp, sz, sz, vp, sz, vp, sz, vp, sz, f32, u32, vp]
    lib.meshoptgpu_simplifyWithUpdateDevice.restype = sz
    lib.meshoptgpu_simplifyWithUpdateDevice.argtypes = [vp, sz, vp, sz, sz, vp, sz, vp, sz, vp, sz, f32, u32, vp, vp]
    lib.meshoptgpu_setDeviceLoop.restype = C.c_int
    lib.meshoptgpu_setDeviceLoop.argtypes = [C.c_int]
    lib.meshoptgpu_probeBarrierWait.restype = C.c_int
    lib.meshoptgpu_probeBarrierWait.argtypes = [C.c_int, C.c_uint, C.c_uint, C.POINTER(C.c_uint)]
    lib.meshoptgpu_simplifyGroups.restype = C.c_int
    lib.meshoptgpu_simplifyGroups.argtypes = [vp, vp, vp, sz, vp, sz, sz, vp, sz, vp, sz, vp, vp, vp, vp, f32, u32, vp, vp, vp]
    lib.meshoptgpu_buildMeshletsFlexGroups.restype = C.c_int
    lib.meshoptgpu_buildMeshletsFlexGroups.argtypes = [vp, vp, vp, vp, vp, vp, vp, sz, vp, sz, sz, sz, sz, sz, f32, f32, C.c_int, vp]
    _lib = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def last_status():
    lib = load()
    return int(lib.meshoptgpu_getLastStatus()), lib.meshoptgpu_getLastMessage().decode()


def _check(check):
    if check:
        st, msg = last_status()
        if st != STATUS_OK:
            raise SimplifyError(st, msg)


def simplify(indices, positions, target_index_count, target_error, options=0, attributes=None, weights=None, lock=None,
             destination=None, check=True):
    """meshopt_simplify / meshopt_simplifyWithAttributes on host arrays.

    indices uint32 [I]; positions float32 [V, k>=3] (stride k*4 bytes); attributes float32 [V, a]
    (or None) with weights float32 [a]; lock uint8 [V] or None. Returns (indices, result_error).
    """
    lib = load()
    indices = np.ascontiguousarray(indices, dtype=np.uint32)
    positions = np.ascontiguousarray(positions, dtype=np.float32)
    if positions.ndim == 1:
        positions = positions.reshape(-1, 3)
    out = destination if destination is not None else np.empty(max(len(indices), 1), np.uint32)
    err = C.c_float(0)
    V, pstride = positions.shape[0], positions.shape[1] * 4
    if attributes is None and lock is None:
        n = lib.meshopt_simplify(_p(out), _p(indices), len(indices), _p(positions), V, pstride, int(target_index_count),
                                 float(target_error), int(options), C.byref(err))
    else:
        a = 0
        astride = 0
        if attributes is not None:
            attributes = np.ascontiguousarray(attributes, dtype=np.float32)
            weights = np.ascontiguousarray(weights, dtype=np.float32)
            a, astride = attributes.shape[1], attributes.shape[1] * 4
        if lock is not None:
            lock = np.ascontiguousarray(lock, dtype=np.uint8)
        n = lib.meshopt_simplifyWithAttributes(_p(out), _p(indices), len(indices), _p(positions), V, pstride,
                                               _p(attributes), astride, _p(weights), a, _p(lock), int(target_index_count),
                                               float(target_error), int(options), C.byref(err))
    _check(check)
    return out[:n].copy(), float(err.value)


def simplify_with_update(indices, positions, target_index_count, target_error, options=0, attributes=None, weights=None, lock=None, check=True):
    """meshopt_simplifyWithUpdate on copies of host arrays: returns (indices, positions, attributes,
    result_error) as the call leaves them (positions float32 [V, k>=3]; attributes float32 [V, a])."""
    lib = load()
    idx = np.array(indices, dtype=np.uint32, copy=True)
    pos = np.array(positions, dtype=np.float32, copy=True)
    attr = None if attributes is None else np.array(attributes, dtype=np.float32, copy=True)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float32)
    lk = None if lock is None else np.ascontiguousarray(lock, dtype=np.uint8)
    err = C.c_float(0)
    n = lib.meshopt_simplifyWithUpdate(_p(idx), len(idx), _p(pos), pos.shape[0], pos.shape[1] * 4, _p(attr), 0 if attr is None else attr.shape[1] * 4,
                                       _p(w), 0 if w is None else len(w), _p(lk), int(target_index_count), float(target_error), int(options),
                                       C.byref(err))
    _check(check)
    return idx[:n].copy(), pos, attr, float(err.value)


def simplify_with_update_interleaved(indices, vertices, stride_f, attr_offset, weights, lock, target_index_count, target_error, options=0, check=True):
    """meshopt_simplifyWithUpdate on one interleaved float vertex buffer (positions first, the
    attributes attr_offset floats into each stride_f-float vertex), on copies: returns
    (indices, vertices, result_error)."""
    lib = load()
    ib = np.array(indices, np.uint32, copy=True)
    v = np.array(vertices, np.float32, copy=True).reshape(-1)
    w = np.ascontiguousarray(weights, np.float32)
    lk = None if lock is None else np.ascontiguousarray(lock, np.uint8)
    err = C.c_float(0)
    n = lib.meshopt_simplifyWithUpdate(_p(ib), len(ib), _p(v), len(v) // stride_f, stride_f * 4, C.c_void_p(v.ctypes.data + attr_offset * 4),
                                       stride_f * 4, _p(w), len(w), _p(lk), int(target_index_count), float(target_error), int(options), C.byref(err))
    _check(check)
    return ib[:n].copy(), v, float(err.value)


def simplify_with_update_device(d_indices, index_count, d_positions, vertex_count, positions_stride, target_index_count, target_error, options=0,
                                d_attributes=0, attributes_stride=0, weights=None, d_lock=0, stream=0, check=True):
    """meshoptgpu_simplifyWithUpdateDevice with raw device pointers (updated in place)."""
    lib = load()
    err = C.c_float(0)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float32)
    n = lib.meshoptgpu_simplifyWithUpdateDevice(C.c_void_p(d_indices), index_count, C.c_void_p(d_positions), vertex_count, positions_stride,
                                                C.c_void_p(d_attributes or None), attributes_stride, _p(w), 0 if w is None else len(w),
                                                C.c_void_p(d_lock or None), int(target_index_count), float(target_error), int(options), C.byref(err),
                                                C.c_void_p(stream or None))
    _check(check)
    return int(n), float(err.value)


def simplify_raw(destination, indices, index_count, positions, vertex_count, positions_stride, target_index_count, target_error,
                 options=0, attributes=None, attributes_stride=0, weights=None, attribute_count=0, lock=None, check=True):
    """The C signature as is (numpy buffers with explicit counts and byte strides)."""
    lib = load()
    err = C.c_float(0)
    n = lib.meshopt_simplifyWithAttributes(_p(destination), _p(indices), index_count, _p(positions), vertex_count, positions_stride,
                                           _p(attributes), attributes_stride, _p(weights), attribute_count, _p(lock),
                                           int(target_index_count), float(target_error), int(options), C.byref(err))
    _check(check)
    return int(n), float(err.value)


def simplify_scale(positions):
    lib = load()
    positions = np.ascontiguousarray(positions, dtype=np.float32)
    return float(lib.meshopt_simplifyScale(_p(positions), positions.shape[0], positions.shape[1] * 4))


def simplify_device(d_destination, d_indices, index_count, d_positions, vertex_count, positions_stride, target_index_count, target_error,
                    options=0, d_attributes=0, attributes_stride=0, weights=None, d_lock=0, stream=0, check=True):
    """meshoptgpu_simplifyDevice with raw device pointers (ints), e.g. from torch tensors' data_ptr()."""
    lib = load()
    err = C.c_float(0)
    a = 0
    if weights is not None:
        weights = np.ascontiguousarray(weights, dtype=np.float32)
        a = len(weights)
    n = lib.meshoptgpu_simplifyDevice(C.c_void_p(d_destination), C.c_void_p(d_indices), index_count, C.c_void_p(d_positions), vertex_count,
                                      positions_stride, C.c_void_p(d_attributes or None), attributes_stride, _p(weights), a,
                                      C.c_void_p(d_lock or None), int(target_index_count), float(target_error), int(options), C.byref(err),
                                      C.c_void_p(stream or None))
    _check(check)
    return int(n), float(err.value)


def last_pass_stats():
    lib = load()
    buf = (PassStats * 128)()
    n = lib.meshoptgpu_getLastPassStats(C.cast(buf, C.c_void_p), 128)
    keys = [f[0] for f in PassStats._fields_]
    return [{k: int(getattr(buf[i], k)) for k in keys} for i in range(min(n, 128))]


def set_timing(enabled: bool):
    load().meshoptgpu_setTiming(1 if enabled else 0)


def last_phase_times():
    out = (C.c_float * 16)()
    load().meshoptgpu_getLastPhaseTimes(C.cast(out, C.c_void_p))
    keys = ["setup", "adjacency", "pick", "rank", "sort", "perform", "apply", "total",
            "k_init", "k_marks", "k_rounds", "k_stop", "k_apply", "k_loops", "k_scan", "k_emit"]
    return dict(zip(keys, [float(x) for x in out]))


def last_pass_phase_times():
    """With timing on: per pass of the last single-mesh call, CUDA-event ms of its adjacency,
    pick, rank, sort and perform phases."""
    out = (C.c_float * (5 * 128))()
    n = load().meshoptgpu_getLastPassPhaseTimes(C.cast(out, C.c_void_p), 128)
    keys = ["adjacency", "pick", "rank", "sort", "perform"]
    return [dict(zip(keys, [float(out[5 * i + j]) for j in range(5)])) for i in range(min(n, 128))]


def tuning(index_count, attribute_count=0):
    """The autotuner's choices for meshes of index_count indices: pass-kernel blocks per SM, pass
    sort candidates per thread (0: by count), drop-in route (batch / single / None) and the batch
    kernel's shared-memory budget in KiB (largest size class tuned so far); None if untuned."""
    out = (C.c_int * 4)()
    found = load().meshoptgpu_getTuning(int(index_count), int(attribute_count), C.cast(out, C.c_void_p))
    route = {1: "batch", 0: "single"}.get(int(out[2]))
    return {"perform_blocks_per_sm": int(out[0]) if found else None, "sort_items": int(out[1]) if found else None,
            "dropin_route": route, "batch_smem_kib": int(out[3]) or None}


def workspace_bytes(index_count, vertex_count, attribute_count=0):
    return int(load().meshoptgpu_workspaceBytes(index_count, vertex_count, attribute_count))


def launch_count():
    """Kernels this library has launched from the calling thread."""
    return int(load().meshoptgpu_getLaunchCount())


def set_kernel_profile(name):
    """Times every launch of the kernel whose name starts with `name` (None disables)."""
    load().meshoptgpu_setKernelProfile(None if name is None else name.encode())


def kernel_profile():
    """(launches, total_ms) of the kernel selected with set_kernel_profile since selection."""
    n = C.c_ulonglong(0)
    ms = C.c_double(0)
    load().meshoptgpu_getKernelProfile(C.byref(n), C.byref(ms))
    return int(n.value), float(ms.value)


def simplify_scale_noalloc(d_extent, d_positions, vertex_count, positions_stride=12, stream=0):
    """meshoptgpu_simplifyScaleNoAlloc: writes the extent to the device float at d_extent.

    For callers that must not allocate device memory while they run (a fixed device-memory
    budget, a host that owns every allocation); it reads device positions and uses only the
    library's fixed 1 MiB scratch,
    which limits vertex_count to 67,108,864. Enqueued on `stream` without synchronising.
    Returns the status code (0 on success).
    """
    return int(load().meshoptgpu_simplifyScaleNoAlloc(C.c_void_p(d_extent), C.c_void_p(d_positions or None), vertex_count,
                                                      positions_stride, C.c_void_p(stream or None)))


def _weights(m, keep):
    w = m.get("weights")
    if w is None:
        return None, 0
    w = np.ascontiguousarray(w, dtype=np.float32)
    keep.append(w)
    return w.ctypes.data, len(w)


class HostBatch:
    """meshoptgpu_simplifyBatchHost over a fixed list of host meshes (dicts as simplify_batch takes):
    the descriptor array and the output buffers are built once; run() makes the C-ABI call, which
    packs the inputs into pinned memory, copies them to the device, simplifies, and copies the
    results back into the output buffers. outputs[i][:counts[i]] is mesh i's result."""

    def __init__(self, meshes):
        self.keep = []
        self.n = len(meshes)
        self.arr = (BatchMesh * max(self.n, 1))()
        self.outputs = []
        arrays = {}

        def shared(a, dtype):
            key = id(a)
            if key not in arrays:
                arrays[key] = np.ascontiguousarray(a, dtype=dtype)
                self.keep.append(arrays[key])
            return arrays[key]

        for i, m in enumerate(meshes):
            idx = shared(m["indices"], np.uint32)
            pos = shared(m["positions"], np.float32)
            out = np.empty(max(len(idx), 1), np.uint32)
            self.outputs.append(out)
            wp, wc = _weights(m, self.keep)
            attr = shared(m["attributes"], np.float32) if wc else None
            lock = shared(m["lock"], np.uint8) if m.get("lock") is not None else None
            self.arr[i] = BatchMesh(idx.ctypes.data, len(idx), pos.ctypes.data, pos.shape[0], pos.shape[1] * 4, int(m["target"]),
                                    float(m["error"]), int(m.get("options", 0)), out.ctypes.data, attr.ctypes.data if wc else None,
                                    attr.shape[1] * 4 if wc else 0, wp, wc, lock.ctypes.data if lock is not None else None)
        self.counts = np.zeros(max(self.n, 1), np.uint64)
        self.errors = np.zeros(max(self.n, 1), np.float32)

    def run(self, check=True):
        st = load().meshoptgpu_simplifyBatchHost(C.cast(self.arr, C.c_void_p), self.n, self.counts.ctypes.data, self.errors.ctypes.data)
        if check and st != STATUS_OK:
            raise SimplifyError(st, last_status()[1])
        return st

    def results(self):
        return [(self.outputs[i][:int(self.counts[i])].copy(), float(self.errors[i])) for i in range(self.n)]


def simplify_batch(meshes, check=True):
    """meshoptgpu_simplifyBatchHost on host arrays.

    meshes: list of dicts with indices (uint32), positions (float32 [V, k>=3]), target (index count),
    error, options, and optionally attributes (float32 [V, k>=a]), weights (a floats) and lock
    (uint8 [V]). Meshes of a sparse group may pass the same positions/attributes/lock arrays: they
    are uploaded once. Returns a list of (indices, result_error), identical to per-mesh
    meshopt_simplifyWithAttributes calls.
    """
    b = HostBatch(meshes)
    b.run(check)
    return b.results()


def _device_mesh(m, keep):
    wp, wc = _weights(m, keep)
    return BatchMesh(m["d_indices"], m["index_count"], m["d_positions"], m["vertex_count"], m.get("stride", 12), int(m["target"]),
                     float(m["error"]), int(m.get("options", 0)), m["d_destination"], m.get("d_attributes") if wc else None,
                     m.get("attr_stride", 0) if wc else 0, wp, wc, m.get("d_lock"))


class BatchDescriptors:
    """A prebuilt meshoptgpu_BatchMesh array (and the host weight arrays it points to), for callers
    that launch the same batch repeatedly without rebuilding it."""

    def __init__(self, descs):
        self.keep = []
        self.n = len(descs)
        self.arr = (BatchMesh * max(self.n, 1))()
        for i, m in enumerate(descs):
            self.arr[i] = _device_mesh(m, self.keep)


def simplify_batch_device(descs, stream=0, check=True):
    """meshoptgpu_simplifyBatch with device pointers: descs is a BatchDescriptors or a list of dicts
    with keys d_indices, index_count, d_positions, vertex_count, stride, target, error, options,
    d_destination, and optionally d_attributes, attr_stride (bytes), weights (host floats), d_lock.
    Returns (counts uint64 array, errors float32 array)."""
    lib = load()
    if not isinstance(descs, BatchDescriptors):
        descs = BatchDescriptors(descs)
    n, arr = descs.n, descs.arr
    counts = np.zeros(max(n, 1), np.uint64)
    errs = np.zeros(max(n, 1), np.float32)
    st = lib.meshoptgpu_simplifyBatch(C.cast(arr, C.c_void_p), n, counts.ctypes.data, errs.ctypes.data, C.c_void_p(stream or None))
    if check and st != STATUS_OK:
        raise SimplifyError(st, last_status()[1])
    return counts[:n], errs[:n]


def optimize_vertex_fetch_remap_device(d_destination, d_indices, index_count, vertex_count, stream=0, check=True):
    """meshoptgpu_optimizeVertexFetchRemapDevice: new index per vertex in order of first use
    (~0u unused) written to d_destination; returns the used vertex count."""
    n = load().meshoptgpu_optimizeVertexFetchRemapDevice(d_destination, d_indices, index_count, vertex_count, C.c_void_p(stream or None))
    st, msg = last_status()
    if check and st != STATUS_OK:
        raise SimplifyError(st, msg)
    return int(n)


def optimize_vertex_fetch_device(d_destination, d_indices, index_count, d_vertices, vertex_count, vertex_size, stream=0, check=True):
    """meshoptgpu_optimizeVertexFetchDevice: vertices in order of first use to d_destination (may be
    d_vertices), indices rewritten in place; returns the used vertex count."""
    n = load().meshoptgpu_optimizeVertexFetchDevice(d_destination, d_indices, index_count, d_vertices, vertex_count, vertex_size,
                                                   C.c_void_p(stream or None))
    st, msg = last_status()
    if check and st != STATUS_OK:
        raise SimplifyError(st, msg)
    return int(n)


def generate_position_remap_device(d_destination, d_positions, vertex_count, positions_stride=12, stream=0, check=True):
    """meshoptgpu_generatePositionRemapDevice: smallest vertex with an equal position, per vertex."""
    st = load().meshoptgpu_generatePositionRemapDevice(d_destination, d_positions, vertex_count, positions_stride, C.c_void_p(stream or None))
    if check and st != STATUS_OK:
        raise SimplifyError(st, last_status()[1])
    return int(st)


def simplify_groups_device(d_destination, d_indices, group_offsets, d_positions, vertex_count, positions_stride, d_remap, d_locks, targets,
                           target_error, options, d_attributes=None, attributes_stride=0, weights=None, d_vertex_lock=None, stream=0, check=True):
    """meshoptgpu_simplifyGroups: one cluster-LOD level (boundary locks, then every group simplified
    in one batch launch). group_offsets: host ints (group_count + 1); targets: host ints per group;
    weights: host floats. Returns (counts uint64 array, errors float32 array)."""
    off = np.ascontiguousarray(group_offsets, dtype=np.uint64)
    tg = np.ascontiguousarray(targets, dtype=np.uint64)
    n = len(off) - 1
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float32)
    counts = np.zeros(max(n, 1), np.uint64)
    errs = np.zeros(max(n, 1), np.float32)
    st = load().meshoptgpu_simplifyGroups(d_destination, d_indices, off.ctypes.data, n, d_positions, vertex_count, positions_stride,
                                          d_attributes if w is not None else None, attributes_stride if w is not None else 0,
                                          w.ctypes.data if w is not None else None, len(w) if w is not None else 0, d_remap, d_locks,
                                          d_vertex_lock, tg.ctypes.data, target_error, options, counts.ctypes.data, errs.ctypes.data,
                                          C.c_void_p(stream or None))
    if check and st != STATUS_OK:
        raise SimplifyError(st, last_status()[1])
    return counts[:n], errs[:n]


def meshlets_bound(index_count, max_vertices, max_triangles):
    """meshopt_buildMeshletsBound (src/clusterizer.cpp:1017-1033)."""
    by_vertices = (index_count + max_vertices - 2 - 1) // (max_vertices - 2)
    by_triangles = (index_count // 3 + max_triangles - 1) // max_triangles
    return max(by_vertices, by_triangles)


def meshlet_rows(group_offsets, max_vertices, min_triangles):
    """Row offsets (group_count + 1) with each group's meshopt_buildMeshletsBound rows."""
    off = np.asarray(group_offsets, dtype=np.int64)
    rows = [meshlets_bound(int(off[g + 1] - off[g]), max_vertices, min_triangles) for g in range(len(off) - 1)]
    return np.concatenate([[0], np.cumsum(rows, dtype=np.int64)]).astype(np.uint64)


def build_meshlets_flex_groups_device(d_meshlets, d_meshlet_vertices, d_meshlet_triangles, meshlet_offsets, d_indices, group_offsets, d_positions,
                                      vertex_count, positions_stride, max_vertices, min_triangles, max_triangles, cone_weight=0.0,
                                      split_factor=2.0, optimize_level=-1, stream=0, check=True):
    """meshoptgpu_buildMeshletsFlexGroups: meshopt_buildMeshletsFlex for every group of a level on device
    data, one warp per group, then meshopt_optimizeMeshletLevel(optimize_level) on every meshlet
    unless it is -1. meshlet_offsets / group_offsets: host ints (group_count + 1).
    Returns the meshlet count per group (uint64 array)."""
    off = np.ascontiguousarray(group_offsets, dtype=np.uint64)
    mo = np.ascontiguousarray(meshlet_offsets, dtype=np.uint64)
    n = len(off) - 1
    counts = np.zeros(max(n, 1), np.uint64)
    st = load().meshoptgpu_buildMeshletsFlexGroups(d_meshlets, d_meshlet_vertices, d_meshlet_triangles, mo.ctypes.data, counts.ctypes.data, d_indices,
                                                   off.ctypes.data, n, d_positions, vertex_count, positions_stride, max_vertices, min_triangles,
                                                   max_triangles, C.c_float(cone_weight), C.c_float(split_factor), int(optimize_level),
                                                   C.c_void_p(stream or None))
    if check and st != STATUS_OK:
        raise SimplifyError(st, last_status()[1])
    return counts[:n]


def build_meshlets_flex_groups(groups, positions, max_vertices, min_triangles, max_triangles, cone_weight=0.0, split_factor=2.0, optimize_level=-1):
    """Host convenience over build_meshlets_flex_groups_device (torch for device memory): groups is
    a list of index arrays into `positions`. Returns, per group, (meshlets [n, 4] uint32,
    meshlet_vertices uint32, meshlet_triangles uint8) trimmed as meshopt_buildMeshletsFlex leaves them."""
    import torch

    idx = [np.ascontiguousarray(g, dtype=np.uint32).reshape(-1) for g in groups]
    off = np.concatenate([[0], np.cumsum([len(g) for g in idx], dtype=np.int64)]).astype(np.uint64)
    rows = meshlet_rows(off, max_vertices, min_triangles)
    pos = np.ascontiguousarray(positions, dtype=np.float32)
    flat = np.concatenate(idx) if idx else np.zeros(0, np.uint32)
    total = max(int(off[-1]), 1)
    d_idx = torch.from_numpy(flat.view(np.int32).copy() if len(flat) else np.zeros(1, np.int32)).cuda()
    d_pos = torch.from_numpy(pos.reshape(len(pos), -1)).cuda()
    d_m = torch.zeros(max(int(rows[-1]), 1) * 4, dtype=torch.int32, device="cuda")
    d_v = torch.zeros(total, dtype=torch.int32, device="cuda")
    d_t = torch.zeros(total, dtype=torch.uint8, device="cuda")
    counts = build_meshlets_flex_groups_device(d_m.data_ptr(), d_v.data_ptr(), d_t.data_ptr(), rows, d_idx.data_ptr(), off, d_pos.data_ptr(),
                                               len(pos), pos.reshape(len(pos), -1).shape[1] * 4, max_vertices, min_triangles, max_triangles,
                                               cone_weight, split_factor, optimize_level)
    torch.cuda.synchronize()
    m = d_m.cpu().numpy().view(np.uint32).reshape(-1, 4)
    v = d_v.cpu().numpy().view(np.uint32)
    t = d_t.cpu().numpy()
    out = []
    for g in range(len(idx)):
        n = int(counts[g])
        mg = m[int(rows[g]): int(rows[g]) + n].copy()
        if n:
            last = mg[-1]
            vv = v[int(off[g]): int(off[g]) + int(last[0] + last[2])].copy()
            tt = t[int(off[g]): int(off[g]) + int(last[1] + last[3] * 3)].copy()
        else:
            vv, tt = np.zeros(0, np.uint32), np.zeros(0, np.uint8)
        out.append((mg, vv, tt))
    return out


def set_batch_config(threads=0, smem_bytes=0):
    """Threads per CTA of the batch kernel (128/256/512, 0 = autotune) and shared-memory budget."""
    load().meshoptgpu_setBatchConfig(int(threads), int(smem_bytes))


DROPIN_BATCH_LIMIT = 2 ** 64 - 1  # the library's default: the route is autotuned per size class


def set_dropin_batch_limit(max_index_count=DROPIN_BATCH_LIMIT):
    """Drop-in calls on meshes with at most this many indices run on the batch kernel (0: never;
    the default leaves the route to the autotuner)."""
    load().meshoptgpu_setDropinBatchLimit(int(max_index_count))


def probe_barrier_wait(once=False, blocks=8, wait_limit=4096):
    """meshoptgpu_probeBarrierWait: (status, timed_out) of a grid barrier that one block never reaches."""
    flag = C.c_uint(0)
    st = int(load().meshoptgpu_probeBarrierWait(int(bool(once)), int(blocks), int(wait_limit), C.byref(flag)))
    return st, int(flag.value)


def set_device_loop(enabled=True):
    """Pass loop of the single-mesh path on the device (CUDA graph, default) or driven by the host."""
    return int(load().meshoptgpu_setDeviceLoop(1 if enabled else 0))


def batch_threads():
    return int(load().meshoptgpu_getBatchThreads())


class Server:
    """Continuous-batching request server (meshoptgpu_server*): submit device-resident meshes
    without blocking, wait for tickets; latencies are measured natively from submission to
    completion."""

    def __init__(self, memory_budget=0, batch_workers=0, large_workers=0, large_index_count=0, max_batch=0, batch_threads=0, plain=False,
                 perform_blocks=0):
        self.lib = load()
        cfg = ServerConfig(memory_budget, batch_workers, large_workers, large_index_count, max_batch, batch_threads, 1 if plain else 0,
                           perform_blocks)
        self.h = self.lib.meshoptgpu_serverCreate(C.byref(cfg))
        if not self.h:
            raise SimplifyError(*last_status())

    def submit(self, d_indices, index_count, d_positions, vertex_count, target, error, options, d_destination, stride=12, d_attributes=None,
               attr_stride=0, weights=None, d_lock=None):
        keep = []
        m = _device_mesh(dict(d_indices=d_indices, index_count=index_count, d_positions=d_positions, vertex_count=vertex_count, stride=stride,
                              target=target, error=error, options=options, d_destination=d_destination, d_attributes=d_attributes,
                              attr_stride=attr_stride, weights=weights, d_lock=d_lock), keep)
        t = self.lib.meshoptgpu_serverSubmit(C.c_void_p(self.h), C.byref(m))
        if t < 0:
            raise SimplifyError(-t, last_status()[1])
        return t

    def wait(self, ticket):
        n = C.c_size_t(0)
        e = C.c_float(0)
        lat = C.c_double(0)
        st = self.lib.meshoptgpu_serverWait(C.c_void_p(self.h), ticket, C.byref(n), C.byref(e), C.byref(lat))
        return st, int(n.value), float(e.value), float(lat.value)

    def stats(self):
        out = (C.c_ulonglong * 5)()
        self.lib.meshoptgpu_serverStats(C.c_void_p(self.h), C.cast(out, C.c_void_p))
        return dict(zip(["completed", "batches", "singles", "peak_reserved", "peak_inflight"], [int(x) for x in out]))

    def close(self):
        if self.h:
            self.lib.meshoptgpu_serverDestroy(C.c_void_p(self.h))
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def last_round_trace():
    """[(active candidates, microseconds)] per decision round of the last single-mesh call."""
    n_ = (C.c_uint * 512)()
    t_ = (C.c_float * 512)()
    n = load().meshoptgpu_getLastRoundTrace(C.cast(n_, C.c_void_p), C.cast(t_, C.c_void_p), 512)
    return [(int(n_[i]), float(t_[i])) for i in range(min(n, 512))]
