"""GPU parity: the CUDA path, called through the C ABI, against the reference's results.

Bar: the output index buffer and its count are bit-exact; result_error matches within
1e-6 relative (it is in fact compared bit for bit where the pipeline is exact). The
per-pass counters (triangles, candidates, evaluated, committed, skipped, flip-rejected,
stop reason) are compared with the oracle's as a phase-level check.
"""
import numpy as np
import pytest

import fixtures
import meshoptimizer_gb300 as mg
from meshoptimizer_gb300 import workloads as W

pytestmark = pytest.mark.gpu

REL_TOL = 1e-6
GPU_OPTIONS = (mg.SimplifyLockBorder | mg.SimplifyErrorAbsolute | mg.SimplifyRegularize | mg.SimplifyRegularizeLight | mg.SimplifySparse
               | mg.SimplifyPermissive | mg.SimplifyPrune | (1 << 30))


def close(a, b):
    return a == b or abs(a - b) <= REL_TOL * max(abs(a), abs(b))


@pytest.fixture(scope="module", autouse=True)
def built():
    from meshoptimizer_gb300 import build

    build.build()
    mg.load()
    # this module checks the multi-CTA single-mesh path (and its per-pass counters) on every
    # size; small drop-in calls routed to the batch kernel are covered by test_gpu_dropin.py
    mg.set_dropin_batch_limit(0)
    yield
    mg.set_dropin_batch_limit()


def supported(options):
    return (options & ~GPU_OPTIONS) == 0


@pytest.mark.parametrize("case", fixtures.known_answers(), ids=lambda c: c["name"])
def test_known_answers(case):
    if not supported(case["options"]):
        pytest.skip("option not implemented on the GPU path")
    idx = case["indices"]
    pos = case["positions"]
    vcount = len(pos) * 4 // case["stride"]
    out = np.zeros(max(len(idx), 1), np.uint32)
    attrs, weights, lock = case["attributes"], case["weights"], case["lock"]
    n, err = mg.simplify_raw(out, idx, len(idx), pos, vcount, case["stride"], case["target"], case["error"], case["options"],
                             attributes=attrs, attributes_stride=case["attr_stride"], weights=weights,
                             attribute_count=0 if weights is None else len(weights), lock=lock)
    assert np.array_equal(out[:n], case["ref_output"])
    assert close(err, case["ref_error"])


@pytest.mark.parametrize("case", fixtures.seeded_cases(), ids=lambda c: c["name"])
def test_seeded_fixtures(case):
    out, err = mg.simplify(case["indices"], case["positions"], case["target"], case["error"], case["options"],
                           attributes=case["attributes"], weights=case["weights"])
    assert np.array_equal(out, case["expect"])
    assert close(err, case["expect_error"])


def _compare_with_oracle(port, idx, pos, target, error, options=0, attributes=None, weights=None, lock=None, stats=True):
    ref_out, ref_err, ref_st = port.simplify("port", idx, pos, target, error, options, attributes=attributes, weights=weights,
                                              lock=lock, stats=True)
    out, err = mg.simplify(idx, pos, target, error, options, attributes=attributes, weights=weights, lock=lock)
    st = mg.last_pass_stats()
    assert len(out) == len(ref_out)
    assert np.array_equal(out, ref_out)
    assert close(err, ref_err)
    if stats:
        assert len(st) == ref_st["passes"]
        for p, s in enumerate(st):
            got = (s["triangles"], s["candidates"], s["evaluated"], s["done"], s["skipped"], s["invalid"], s["stop"])
            want = tuple(ref_st[k][p] for k in ("tri", "cand", "evaluated", "done", "skipped", "invalid", "stop"))
            assert got == want, f"pass {p}: {got} != {want}"
    return out, err


@pytest.mark.parametrize("n,opt", [(16, 0), (64, 0), (64, mg.SimplifyLockBorder), (256, 0)])
def test_heightfield(port, n, opt):
    idx, pos = W.heightfield(n, seed=n + opt, amp=0.05)
    _compare_with_oracle(port, idx, pos, W.target_count(len(idx), 0.25), 1e-2, opt)


def test_same_shape_sequence(port):
    """Calls on one mesh shape reuse the recorded pass loop: targets, error limits (including
    ErrorAbsolute, whose limit depends on the mesh extent) and lock options change per call; a
    different shape in between records a new loop."""
    idx, pos = W.heightfield(96, seed=41, amp=0.05)
    idx2, pos2 = W.heightfield(80, seed=42, amp=0.05)
    scaled = pos * np.float32(3.0)
    runs = [(idx, pos, 0.25, 1e-2, 0), (idx, pos, 0.1, 5e-2, 0), (idx, scaled, 0.1, 0.1, mg.SimplifyErrorAbsolute),
            (idx2, pos2, 0.3, 1e-2, 0), (idx, pos, 0.2, 2e-2, mg.SimplifyLockBorder), (idx, scaled, 0.05, 0.3, mg.SimplifyErrorAbsolute)]
    for i, p, ratio, error, opt in runs:
        _compare_with_oracle(port, i, p, W.target_count(len(i), ratio), error, opt)


@pytest.mark.parametrize("levels", [3, 5, 7])
def test_sphere_attributes(port, levels):
    idx, pos, attr, w = W.octa_sphere(levels, seed=levels)
    _compare_with_oracle(port, idx, pos, W.target_count(len(idx), 0.1), 5e-3, 0, attributes=attr, weights=w)


def test_sphere_attributes_2m(port):
    """The 2,097,152-triangle attribute sphere (normals w=0.5, UV w=1.0, 10%, 5e-3)."""
    c = W.config_sphere_attr(9)
    _compare_with_oracle(port, c["indices"], c["positions"], c["target"], c["error"], 0, attributes=c["attributes"],
                         weights=c["weights"])


def test_fractal_heightfield(port):
    c = W.config_fractal_3163(1024)
    _compare_with_oracle(port, c["indices"], c["positions"], c["target"], c["error"], 0)


def test_fractal_heightfield_full(port):
    """The largest single-mesh workload at its full size: the 3163 x 3163 fractal terrain
    (19,996,488 triangles, 1%, 12 passes), bit-exact with every pass's counters (the oracle
    takes about 15 s of one host core)."""
    c = W.config_fractal_3163()
    _compare_with_oracle(port, c["indices"], c["positions"], c["target"], c["error"], 0)


def test_patches_lock_border(port):
    for g, (idx, pos) in enumerate(W.sphere_patches(24, seed=5, levels=5)):
        _compare_with_oracle(port, idx, pos, W.target_count(len(idx), 0.5), 2e-2, mg.SimplifyLockBorder)


@pytest.mark.parametrize("seed", range(12))
def test_random_lattice_soup(port, seed):
    rng = np.random.default_rng(seed)
    pos = rng.integers(0, 10, size=(100, 3)).astype(np.float32)
    idx = rng.integers(0, 100, size=3 * int(rng.integers(1, 150))).astype(np.uint32)
    opt = int(rng.choice([0, mg.SimplifyLockBorder, mg.SimplifyErrorAbsolute, mg.SimplifyRegularize]))
    attrs = weights = lock = None
    if seed % 2:
        attrs = rng.random((100, 3)).astype(np.float32)
        weights = np.array([0.5, 0.0, 1.0], np.float32)
    if seed % 3 == 0:
        lock = rng.choice([0, 0, 1, 4], size=100).astype(np.uint8)
    _compare_with_oracle(port, idx, pos, 0, float(np.finfo(np.float32).max), opt, attributes=attrs, weights=weights, lock=lock)


def test_seams_and_duplicates(port):
    """Grid with duplicated vertices on a seam and random extra wedges."""
    rng = np.random.default_rng(7)
    idx, pos = W.heightfield(40, seed=7, amp=0.02)
    V = len(pos)
    dup = rng.choice(V, size=V // 5, replace=False)
    newid = {int(v): V + i for i, v in enumerate(dup)}
    pos2 = np.concatenate([pos, pos[dup]])
    tri = idx.reshape(-1, 3).copy()
    flip = rng.random(len(tri)) < 0.4
    for t in np.nonzero(flip)[0]:
        tri[t] = [newid.get(int(v), int(v)) for v in tri[t]]
    idx2 = tri.reshape(-1).astype(np.uint32)
    attrs = rng.random((len(pos2), 2)).astype(np.float32)
    _compare_with_oracle(port, idx2, pos2, W.target_count(len(idx2), 0.3), 2e-2, 0)
    _compare_with_oracle(port, idx2, pos2, W.target_count(len(idx2), 0.3), 2e-2, 0, attributes=attrs,
                         weights=np.array([1.0, 0.5], np.float32))


def test_empty_and_trivial(port):
    pos = np.zeros((3, 3), np.float32)
    out, err = mg.simplify(np.zeros(0, np.uint32), pos, 0, 1e-2)
    assert len(out) == 0 and err == 0
    idx, pos = W.heightfield(8, seed=1)
    out, err = mg.simplify(idx, pos, len(idx), 1e-2)   # target >= input: no pass runs
    assert np.array_equal(out, idx) and err == 0


def test_special_values(port):
    """NaN positions never weld, -0 welds with +0, degenerate and duplicate triangles."""
    idx, pos = W.heightfield(20, seed=3, amp=0.05)
    pos = pos.copy()
    pos[5] = [np.nan, 0.2, 0.1]
    pos[50, 0] = -0.0
    z = pos[:, 2] == 0
    pos[z, 2] = -0.0
    tri = idx.reshape(-1, 3)
    extra = np.array([[1, 1, 2], [3, 4, 3], tri[10], tri[11]], np.uint32)
    idx2 = np.concatenate([tri, extra]).reshape(-1).astype(np.uint32)
    _compare_with_oracle(port, idx2, pos, W.target_count(len(idx2), 0.25), 5e-2, 0)


def test_strided_positions_and_alias(port):
    idx, pos = W.heightfield(48, seed=9, amp=0.05)
    wide = np.concatenate([pos, np.ones((len(pos), 5), np.float32)], axis=1)  # 32-byte stride
    ref_out, ref_err = port.simplify("port", idx, wide, W.target_count(len(idx), 0.25), 1e-2, 0)
    buf = idx.copy()
    n, err = mg.simplify_raw(buf, buf, len(buf), wide, len(wide), 32, W.target_count(len(idx), 0.25), 1e-2, 0)
    assert np.array_equal(buf[:n], ref_out) and close(err, ref_err)


def test_scale():
    vb = np.array([0, 0, 0, 1, 0, 0, 0, 2, 0, 0, 0, 3], np.float32).reshape(-1, 3)
    assert mg.simplify_scale(vb) == 3.0


@pytest.mark.parametrize("seed", range(16))
def test_permissive_and_sparse(port, seed):
    """Permissive (complex collapses across attribute seams, Protect flags) and Sparse subsets."""
    rng = np.random.default_rng(100 + seed)
    if seed % 2:
        idx, pos, attr, w = W.octa_sphere(3, seed=seed)
        V = len(pos)
        opt = mg.SimplifyPermissive | (mg.SimplifySparse if seed % 4 == 1 else 0)
        lock = rng.choice([0, 0, 0, 2, 1, 4], size=V).astype(np.uint8) if seed % 3 == 0 else None
        if opt & mg.SimplifySparse:
            tri = idx.reshape(-1, 3)
            idx = tri[rng.random(len(tri)) < 0.5].reshape(-1).astype(np.uint32)
        _compare_with_oracle(port, idx, pos, W.target_count(len(idx), 0.2), 5e-2, opt, attributes=attr, weights=w, lock=lock)
    else:
        pos = rng.integers(0, 10, size=(120, 3)).astype(np.float32)
        idx = rng.integers(0, 100, size=3 * int(rng.integers(5, 150))).astype(np.uint32)
        opt = [mg.SimplifySparse, mg.SimplifyPermissive, mg.SimplifySparse | mg.SimplifyLockBorder,
               mg.SimplifyPermissive | mg.SimplifyErrorAbsolute][(seed // 2) % 4]
        attrs = rng.random((120, 2)).astype(np.float32) if seed % 4 == 0 else None
        weights = np.array([1.0, 0.5], np.float32) if attrs is not None else None
        _compare_with_oracle(port, idx, pos, 0, float(np.finfo(np.float32).max), opt, attributes=attrs, weights=weights)


def test_sparse_subset_of_large_buffer(port):
    """A cluster-sized subset of a big vertex buffer: work and error relative to the subset."""
    idx, pos = W.heightfield(200, seed=12, amp=0.05)
    tri = idx.reshape(-1, 3)[5000:5600].reshape(-1).astype(np.uint32)
    _compare_with_oracle(port, tri, pos, W.target_count(len(tri), 0.5), 1e-2, mg.SimplifySparse | mg.SimplifyLockBorder)


def test_large_dropin_overlapped_uploads(port):
    """Drop-in calls above the batch route's size limit copy their inputs on a stream of their own
    (positions, then indices, then attributes), and the setup waits for each where it first reads
    it: a whole mesh with attributes and lock flags, and a sparse subset of a larger buffer with
    attributes (the sparse path reads the indices before anything else), against the oracle."""
    idx, pos, attr, w = W.octa_sphere(7, seed=41)  # 131,072 triangles
    rng = np.random.default_rng(41)
    lock = rng.choice(np.array([0, 0, 0, 0, 1, 2, 4], np.uint8), size=len(pos))
    _compare_with_oracle(port, idx, pos, W.target_count(len(idx), 0.2), 1e-2, 0, attributes=attr, weights=w, lock=lock)
    big, bpos = W.heightfield(300, seed=42, amp=0.05)
    battr = rng.random((len(bpos), 3)).astype(np.float32)
    sub = big.reshape(-1, 3)[20000:60000].reshape(-1).astype(np.uint32)  # 120,000 indices of 536,406
    _compare_with_oracle(port, sub, bpos, W.target_count(len(sub), 0.3), 1e-2, mg.SimplifySparse, attributes=battr,
                         weights=np.array([0.5, 1.0, 0.25], np.float32))


@pytest.mark.parametrize("seed", range(10))
def test_prune(port, seed):
    """Prune: disconnected pieces of different sizes removed in the pass loop and the cleanup loop."""
    rng = np.random.default_rng(300 + seed)
    parts_idx, parts_pos, base = [], [], 0
    for p in range(int(rng.integers(2, 7))):
        n = int(rng.integers(3, 14))
        idx, pos = W.heightfield(n, seed=seed * 10 + p, amp=0.05)
        pos = pos * np.float32(rng.uniform(0.05, 1.0)) + rng.uniform(-2, 2, size=3).astype(np.float32)
        parts_idx.append(idx + base)
        parts_pos.append(pos)
        base += len(pos)
    idx = np.concatenate(parts_idx).astype(np.uint32)
    pos = np.concatenate(parts_pos).astype(np.float32)
    opt = mg.SimplifyPrune | [0, mg.SimplifyLockBorder, mg.SimplifySparse, mg.SimplifyErrorAbsolute][seed % 4]
    err = [1e-2, 5e-2, 0.2][seed % 3] * (4.0 if opt & mg.SimplifyErrorAbsolute else 1.0)
    _compare_with_oracle(port, idx, pos, W.target_count(len(idx), float(rng.uniform(0.05, 0.5))), err, opt)


def test_internal_debug_bits(port):
    idx, pos = W.heightfield(12, seed=4, amp=0.05)
    _compare_with_oracle(port, idx, pos, W.target_count(len(idx), 0.3), 1e-2, 1 << 30, stats=False)


def test_unsupported_option_reports_status():
    idx, pos = W.heightfield(8, seed=1)
    out, err = mg.simplify(idx, pos, 0, 1e-2, 1 << 29, check=False)  # the internal solve bit (simplifyWithUpdate)
    st, msg = mg.last_status()
    assert st == mg.STATUS_UNSUPPORTED and np.array_equal(out, idx)


def test_high_degree_fan(port):
    """A vertex with more corners than the per-vertex list sort takes (the stable radix sort
    builds the corner lists instead): a 300-triangle fan around one vertex plus a wavy rim."""
    n = 300
    ang = np.linspace(0, 2 * np.pi, n, endpoint=False)
    rim = np.stack([np.cos(ang), np.sin(ang), 0.05 * np.sin(7 * ang)], axis=1)
    pos = np.concatenate([[[0.0, 0.0, 0.2]], rim]).astype(np.float32)
    idx = np.array([[0, 1 + i, 1 + (i + 1) % n] for i in range(n)], np.uint32).reshape(-1)
    for opt in (0, mg.SimplifyLockBorder):
        _compare_with_oracle(port, idx, pos, W.target_count(len(idx), 0.3), 1.0, opt)


@pytest.mark.parametrize("ac", [9, 17, 32])
def test_wide_attribute_sets(port, ac):
    """Attribute counts past 8 and 16 (the wider quadric fill instantiations) up to the
    reference's limit of 32 (`kMaxAttributes`, src/simplifier.cpp:665), some weights zero, on
    the single-mesh path and on the batch kernel."""
    rng = np.random.default_rng(ac)
    idx, pos = W.heightfield(20, seed=ac, amp=0.05)
    attrs = rng.random((len(pos), ac)).astype(np.float32)
    weights = rng.choice(np.array([0.0, 0.1, 0.5, 1.0], np.float32), size=ac)
    weights[0] = 1.0
    target = W.target_count(len(idx), 0.2)
    ref, ref_err = port.simplify("port", idx, pos, target, 5e-2, 0, attributes=attrs, weights=weights)
    for limit in (0, 1 << 30):  # the pass loop, then the batch kernel (a batch of one)
        mg.set_dropin_batch_limit(limit)
        try:
            out, err = mg.simplify(idx, pos, target, 5e-2, 0, attributes=attrs, weights=weights)
        finally:
            mg.set_dropin_batch_limit(0)
        assert np.array_equal(out, ref), limit
        assert close(err, ref_err)


@pytest.mark.parametrize("ac", [2, 5])
def test_interleaved_vertex_buffer_max_stride(port, ac):
    """Positions and attributes interleaved in one 256-byte vertex record (the largest stride
    the reference accepts, src/simplifier.cpp:2349-2354), as real vertex formats lay them out:
    positions at byte 0, attributes at byte 12, both read with stride 256."""
    rng = np.random.default_rng(100 + ac)
    idx, pos = W.heightfield(24, seed=ac, amp=0.05)
    V = len(pos)
    buf = rng.random((V, 64)).astype(np.float32)  # 64 floats = 256 bytes per vertex
    buf[:, 0:3] = pos
    attrs = np.ascontiguousarray(buf[:, 3:3 + ac])
    weights = np.linspace(1.0, 0.25, ac).astype(np.float32)
    target = W.target_count(len(idx), 0.25)
    ref, ref_err = port.simplify("port", idx, pos, target, 2e-2, 0, attributes=attrs, weights=weights)
    for limit in (0, 1 << 30):  # the pass loop, then the batch kernel (a batch of one)
        mg.set_dropin_batch_limit(limit)
        try:
            out = np.zeros(len(idx), np.uint32)
            n, err = mg.simplify_raw(out, idx, len(idx), buf, V, 256, target, 2e-2, 0, attributes=buf[:, 3:], attributes_stride=256,
                                     weights=weights, attribute_count=ac)
        finally:
            mg.set_dropin_batch_limit(0)
        assert np.array_equal(out[:n], ref), limit
        assert close(err, ref_err)
