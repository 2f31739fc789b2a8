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
