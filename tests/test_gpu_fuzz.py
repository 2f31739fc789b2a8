"""Randomized parity sweep, after the reference's fuzz recipe (tools/simplifyfuzz.cpp: lattice
meshes with random connectivity, every option the path has, attributes and lock flags): each
case through the batch kernel (drop-in calls up to the batch limit) and through the single-mesh
pass loop, against the oracle bit for bit (indices, count, error)."""
import numpy as np
import pytest

import meshoptimizer_gb300 as mg
from meshoptimizer_gb300 import workloads as W

pytestmark = pytest.mark.gpu

OPTION_BITS = [mg.SimplifyLockBorder, mg.SimplifySparse, mg.SimplifyErrorAbsolute, mg.SimplifyPrune, mg.SimplifyRegularize,
               mg.SimplifyPermissive, mg.SimplifyRegularizeLight]


@pytest.fixture(scope="module", autouse=True)
def built():
    from meshoptimizer_gb300 import build

    build.build()
    mg.load()


def _case(rng):
    kind = int(rng.integers(0, 3))
    if kind == 0:  # lattice soup: random triangles over integer points (duplicates, degenerates, non-manifold)
        V = int(rng.integers(8, 200))
        pos = rng.integers(0, int(rng.integers(2, 12)), size=(V, 3)).astype(np.float32)
        idx = rng.integers(0, V, size=3 * int(rng.integers(1, 300))).astype(np.uint32)
    elif kind == 1:  # a noisy heightfield patch
        n = int(rng.integers(3, 24))
        idx, pos = W.heightfield(n, seed=int(rng.integers(0, 1 << 30)), amp=float(rng.uniform(0.0, 0.2)))
    else:  # a patch of a seamed attribute sphere
        idx, pos, attr, _ = W.octa_sphere(int(rng.integers(1, 4)), seed=int(rng.integers(0, 1 << 30)))
        tri = idx.reshape(-1, 3)
        keep = rng.random(len(tri)) < rng.uniform(0.3, 1.0)
        idx = tri[keep].reshape(-1).astype(np.uint32)
        if len(idx) == 0:
            idx = tri[:1].reshape(-1).astype(np.uint32)
    V = len(pos)
    options = 0
    for bit in OPTION_BITS:
        if rng.random() < 0.3:
            options |= bit
    if rng.random() < 0.1:
        options |= 1 << 30  # the debug bit (kind and loop bits in the output indices)
    attrs = weights = lock = None
    if rng.random() < 0.5:
        ac = int(rng.integers(1, 6))
        attrs = rng.random((V, ac)).astype(np.float32)
        weights = rng.choice([0.0, 0.25, 0.5, 1.0], size=ac).astype(np.float32)
    if rng.random() < 0.4:
        lock = rng.choice(np.array([0, 0, 0, 1, 2, 4, 3, 6], np.uint8), size=V)
    target = int(rng.integers(0, len(idx) // 3 + 1)) * 3
    error = float(rng.choice([1e-3, 1e-2, 0.1, 1.0, float(np.finfo(np.float32).max)]))
    return idx, pos, attrs, weights, lock, target, error, options


def _check(port, case, batch_limit):
    idx, pos, attrs, weights, lock, target, error, options = case
    ref, ref_err = port.simplify("port", idx, pos, target, error, options, attributes=attrs, weights=weights, lock=lock)
    mg.set_dropin_batch_limit(batch_limit)
    try:
        got, err = mg.simplify(idx, pos, target, error, options, attributes=attrs, weights=weights, lock=lock)
    finally:
        mg.set_dropin_batch_limit()
    assert np.array_equal(got, ref), (options, target, error, len(idx))
    assert np.float32(err) == np.float32(ref_err) or abs(err - ref_err) <= 1e-6 * max(1.0, abs(ref_err))


@pytest.mark.parametrize("chunk", range(4))
def test_fuzz_batch_and_single_mesh(port, chunk):
    rng = np.random.default_rng(4242 + chunk)
    for _ in range(150):
        case = _case(rng)
        _check(port, case, 24000)  # meshes this small run on the batch kernel (Prune and the debug bit excepted)
        _check(port, case, 0)      # the single-mesh pass loop


def test_fuzz_update(port):
    """meshopt_simplifyWithUpdate on random cases: indices, the solved positions and attributes."""
    rng = np.random.default_rng(777)
    for _ in range(100):
        idx, pos, attrs, weights, lock, target, error, options = _case(rng)
        ref = port.simplify_with_update("port", idx, pos, target, error, options, attributes=attrs, weights=weights, lock=lock)
        got = mg.simplify_with_update(idx, pos, target, error, options, attributes=attrs, weights=weights, lock=lock)
        assert np.array_equal(got[0], ref[0]), (options, target)
        assert np.array_equal(np.asarray(got[1], np.float32).view(np.uint32), np.asarray(ref[1], np.float32).view(np.uint32))
        if attrs is not None:
            assert np.array_equal(np.asarray(got[2], np.float32).view(np.uint32), np.asarray(ref[2], np.float32).view(np.uint32))
        assert got[3] == ref[3]
