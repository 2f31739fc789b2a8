"""Batched simplification (one persistent launch, one CTA per mesh) against the oracle:
every mesh of the batch must equal its own meshopt_simplify result bit for bit, for meshes
that fit shared memory and for meshes that spill to global slabs, in every block size."""
import numpy as np
import pytest

import meshoptimizer_gb300 as mg
from meshoptimizer_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from meshoptimizer_gb300 import build

    build.build()
    mg.load()


def _meshes():
    ms = []
    for idx, pos in W.sphere_patches(48, seed=31, levels=5):
        ms.append(dict(indices=idx, positions=pos, target=W.target_count(len(idx), 0.5), error=2e-2, options=mg.SimplifyLockBorder))
    for n in (8, 16, 40):
        idx, pos = W.heightfield(n, seed=n, amp=0.05)
        ms.append(dict(indices=idx, positions=pos, target=W.target_count(len(idx), 0.25), error=1e-2, options=0))
    idx, pos = W.heightfield(72, seed=7, amp=0.05)   # workspace above the shared-memory budget -> global slab
    ms.append(dict(indices=idx, positions=pos, target=W.target_count(len(idx), 0.25), error=1e-2, options=0))
    idx, pos, _, _ = W.octa_sphere(3, seed=3)        # seam duplicates (welded by position)
    ms.append(dict(indices=idx, positions=pos, target=W.target_count(len(idx), 0.2), error=5e-2, options=0))
    rng = np.random.default_rng(5)
    for s in range(6):
        pos = rng.integers(0, 10, size=(100, 3)).astype(np.float32)
        idx = rng.integers(0, 100, size=3 * int(rng.integers(1, 120))).astype(np.uint32)
        ms.append(dict(indices=idx, positions=pos, target=0, error=float(np.finfo(np.float32).max),
                       options=[0, mg.SimplifyLockBorder, mg.SimplifyErrorAbsolute, mg.SimplifyRegularize][s % 4]))
    ms.append(dict(indices=np.zeros(0, np.uint32), positions=np.zeros((3, 3), np.float32), target=0, error=1e-2, options=0))
    idx, pos = W.heightfield(6, seed=2)
    ms.append(dict(indices=idx, positions=pos, target=len(idx), error=1e-2, options=0))  # no pass runs
    return ms


@pytest.mark.parametrize("threads", [128, 256, 512, 0])
def test_batch_matches_oracle(port, threads):
    ms = _meshes()
    mg.set_batch_config(threads)
    try:
        res = mg.simplify_batch(ms)
    finally:
        mg.set_batch_config(0)
    for i, (m, (out, err)) in enumerate(zip(ms, res)):
        ref, ref_err = port.simplify("port", m["indices"], m["positions"], m["target"], m["error"], m["options"])
        assert np.array_equal(out, ref), f"mesh {i}"
        assert err == ref_err or abs(err - ref_err) <= 1e-6 * abs(ref_err), f"mesh {i}"


def test_batch_device_pointers(port):
    torch = pytest.importorskip("torch")
    ms = _meshes()[:12]
    dev = []
    descs = []
    for m in ms:
        di = torch.from_numpy(m["indices"].view(np.int32)).cuda()
        dp = torch.from_numpy(m["positions"]).cuda()
        do = torch.empty(max(len(m["indices"]), 1), dtype=torch.int32, device="cuda")
        dev.append((di, dp, do))
        descs.append(dict(d_indices=di.data_ptr(), index_count=len(m["indices"]), d_positions=dp.data_ptr(), vertex_count=len(m["positions"]),
                          target=m["target"], error=m["error"], options=m["options"], d_destination=do.data_ptr()))
    counts, errs = mg.simplify_batch_device(descs)
    for m, (di, dp, do), n, e in zip(ms, dev, counts, errs):
        ref, ref_err = port.simplify("port", m["indices"], m["positions"], m["target"], m["error"], m["options"])
        assert np.array_equal(do[:int(n)].cpu().numpy().view(np.uint32), ref)


CLOD = mg.SimplifySparse | mg.SimplifyErrorAbsolute | mg.SimplifyPermissive
FLT_MAX = float(np.finfo(np.float32).max)


def _group_meshes(levels, group_tris, options, seed=2):
    groups, pos, attr, w, lock = W.cluster_groups(levels, group_tris, seed=seed)
    return [dict(indices=g, positions=pos, attributes=attr, weights=w, lock=lock, target=(len(g) // 6) * 3, error=FLT_MAX, options=options)
            for g in groups]


def _check(port, ms, res):
    for i, (m, (out, err)) in enumerate(zip(ms, res)):
        ref, ref_err = port.simplify("port", m["indices"], m["positions"], m["target"], m["error"], m["options"], attributes=m.get("attributes"),
                                     weights=m.get("weights"), lock=m.get("lock"))
        assert np.array_equal(out, ref), f"mesh {i}"
        assert err == ref_err or abs(err - ref_err) <= 1e-6 * abs(ref_err), f"mesh {i}: {err} vs {ref_err}"


@pytest.mark.parametrize("threads", [128, 256, 512])
@pytest.mark.parametrize("group_tris", [128, 512])
def test_batch_cluster_groups(port, threads, group_tris):
    """Cluster-LOD groups: sparse index subsets of one shared vertex buffer with attributes,
    boundary locks and protected seams, simplified to half with Sparse | ErrorAbsolute |
    Permissive (demo/clusterlod.h simplify); 128-triangle groups fit shared memory, 512-triangle
    groups take global slabs."""
    ms = _group_meshes(5 if group_tris == 128 else 6, group_tris, CLOD)
    mg.set_batch_config(threads)
    try:
        res = mg.simplify_batch(ms)
    finally:
        mg.set_batch_config(0)
    _check(port, ms, res)


def test_batch_options_mix(port):
    """Every batch option on whole meshes: attributes (with a zero weight), vertex_lock flags
    (Lock, Protect, Priority), Permissive, Regularize, Sparse over a subset, ErrorAbsolute."""
    idx, pos, attr, w = W.octa_sphere(3, seed=3)
    rng = np.random.default_rng(11)
    lock = rng.choice(np.array([0, 0, 0, 0, 1, 2, 4], np.uint8), size=len(pos))
    w0 = w.copy()
    w0[1] = 0.0
    hi, hp = W.heightfield(24, seed=4)
    ha = rng.standard_normal((len(hp), 3)).astype(np.float32)
    ms = [
        dict(indices=idx, positions=pos, attributes=attr, weights=w, target=W.target_count(len(idx), 0.2), error=5e-2, options=0),
        dict(indices=idx, positions=pos, attributes=attr, weights=w0, lock=lock, target=W.target_count(len(idx), 0.2), error=5e-2,
             options=mg.SimplifyPermissive),
        dict(indices=idx, positions=pos, lock=lock, target=W.target_count(len(idx), 0.3), error=1e-1, options=mg.SimplifyRegularize),
        dict(indices=idx[: len(idx) // 2], positions=pos, attributes=attr, weights=w, target=W.target_count(len(idx) // 2, 0.25),
             error=FLT_MAX, options=mg.SimplifySparse | mg.SimplifyErrorAbsolute),
        dict(indices=hi, positions=hp, attributes=ha, weights=np.array([1.0, 0.5, 2.0], np.float32), target=W.target_count(len(hi), 0.25),
             error=1e-2, options=mg.SimplifyLockBorder),
        dict(indices=hi, positions=hp, attributes=ha, weights=np.zeros(3, np.float32), target=W.target_count(len(hi), 0.25), error=1e-2,
             options=mg.SimplifyPermissive | mg.SimplifyRegularizeLight),
    ]
    for threads in (128, 512):
        mg.set_batch_config(threads)
        try:
            res = mg.simplify_batch(ms)
        finally:
            mg.set_batch_config(0)
        _check(port, ms, res)


def test_batch_groups_device_pointers(port):
    """The device-pointer batch entry with one shared device vertex/attribute/lock buffer."""
    torch = pytest.importorskip("torch")
    ms = _group_meshes(5, 256, CLOD)
    pos, attr, lock = ms[0]["positions"], ms[0]["attributes"], ms[0]["lock"]
    dp = torch.from_numpy(pos).cuda()
    da = torch.from_numpy(attr).cuda()
    dl = torch.from_numpy(lock).cuda()
    keep, descs = [], []
    for m in ms:
        di = torch.from_numpy(m["indices"].view(np.int32)).cuda()
        do = torch.empty(len(m["indices"]), dtype=torch.int32, device="cuda")
        keep.append((di, do))
        descs.append(dict(d_indices=di.data_ptr(), index_count=len(m["indices"]), d_positions=dp.data_ptr(), vertex_count=len(pos),
                          target=m["target"], error=m["error"], options=m["options"], d_destination=do.data_ptr(), d_attributes=da.data_ptr(),
                          attr_stride=attr.shape[1] * 4, weights=m["weights"], d_lock=dl.data_ptr()))
    counts, errs = mg.simplify_batch_device(descs)
    res = [(do[:int(n)].cpu().numpy().view(np.uint32), float(e)) for (di, do), n, e in zip(keep, counts, errs)]
    _check(port, ms, res)


def test_batch_rejects_prune():
    idx, pos = W.heightfield(8, seed=1)
    with pytest.raises(mg.SimplifyError) as e:
        mg.simplify_batch([dict(indices=idx, positions=pos, target=0, error=1e-2, options=mg.SimplifyPrune)])
    assert e.value.status == mg.STATUS_UNSUPPORTED


def test_batch_host_concurrent_callers(port):
    """Host batches from several threads at once: their packing and scattering copies share one
    pool of host threads (a caller that finds it busy copies on its own thread), and each thread
    has its own stream and scratch. Every result equals the same batch called alone, and the
    first batch's meshes equal the oracle's."""
    import threading

    sets = [[dict(indices=idx, positions=pos, target=W.target_count(len(idx), 0.5), error=2e-2, options=mg.SimplifyLockBorder)
             for idx, pos in W.sphere_patches(256, seed=70 + t, levels=7)] for t in range(4)]
    want = [mg.simplify_batch(ms) for ms in sets]
    for m, (out, err) in zip(sets[0][:16], want[0][:16]):
        ref, ref_err = port.simplify("port", m["indices"], m["positions"], m["target"], m["error"], m["options"])
        assert np.array_equal(out, ref)
    got = [[] for _ in sets]
    errors = []

    def run(t):
        try:
            for _ in range(3):
                got[t].append(mg.simplify_batch(sets[t]))
        except Exception as e:  # reported below, on the main thread
            errors.append(e)

    threads = [threading.Thread(target=run, args=(t,)) for t in range(len(sets))]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    for t, runs in enumerate(got):
        assert len(runs) == 3
        for res in runs:
            for i, ((out, err), (wout, werr)) in enumerate(zip(res, want[t])):
                assert np.array_equal(out, wout), (t, i)
                assert err == werr, (t, i)
