"""Cluster-LOD level on top of the oracle (TEST INFRASTRUCTURE ONLY; the product never
imports it).

Restates the per-level work of the reference's cluster-LOD builder that the GPU entry
point meshoptgpu_simplifyGroups replaces: lockBoundary (demo/clusterlod.h:372-418) and the
per-group simplify call (demo/clusterlod.h:455-479, the meshopt_simplifyWithAttributes call
with the level's locks), run through the oracle's simplifier.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

import oracle

CLOD_REF_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", "libclod_ref.so")


def reference_available() -> bool:
    return os.path.isfile(CLOD_REF_PATH)


def reference_lock_boundary(locks, groups, remap, vertex_lock=None):
    """The reference builder's own lockBoundary through the oracle/clod_ref.cpp harness."""
    lib = C.CDLL(CLOD_REF_PATH)
    f = lib.clod_ref_lock_boundary
    f.restype = None
    f.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]
    out = np.array(locks, dtype=np.uint8, copy=True)
    idx = np.ascontiguousarray(np.concatenate([np.asarray(g, np.uint32) for g in groups]) if groups else np.zeros(0, np.uint32))
    off = np.zeros(len(groups) + 1, np.uint64)
    off[1:] = np.cumsum([len(g) for g in groups])
    remap = np.ascontiguousarray(remap, dtype=np.uint32)
    vl = None if vertex_lock is None else np.ascontiguousarray(vertex_lock, dtype=np.uint8)
    f(out.ctypes.data, len(out), idx.ctypes.data, off.ctypes.data, len(groups), remap.ctypes.data, None if vl is None else vl.ctypes.data)
    return out


def lock_boundary(locks, groups, remap, vertex_lock=None):
    """demo/clusterlod.h:372-418, literally: bit 7 marks a position seen by an earlier group,
    bit 0 locks it; then every vertex takes its position's lock bit and keeps its own Protect
    bit, in vertex order (so locks[remap[i]] is already rewritten when i > remap[i])."""
    locks = np.array(locks, dtype=np.uint8, copy=True)
    locks &= np.uint8(~(1 | 128) & 0xFF)
    for g in groups:
        r = remap[np.asarray(g, dtype=np.int64)]
        locks[r] |= locks[r] >> 7
        locks[r] |= 128
    out = locks
    for i in range(len(out)):
        r = int(remap[i])
        out[i] = (out[r] & 1) | (out[i] & 2)
        if vertex_lock is not None:
            out[i] |= vertex_lock[i]
    return out


def simplify_level(kind, groups, positions, attributes, weights, remap, locks, vertex_lock, targets, target_error, options):
    """(new locks, [(indices, error)] per group)."""
    new_locks = lock_boundary(locks, groups, remap, vertex_lock)
    results = []
    for g, t in zip(groups, targets):
        results.append(oracle.simplify(kind, g, positions, t, target_error, options | 2, attributes=attributes, weights=weights, lock=new_locks))
    return new_locks, results
