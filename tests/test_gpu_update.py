"""meshopt_simplifyWithUpdate on the GPU against the reference library (the committed fixtures:
its simplifyUpdate tests and seeded meshes) and, on larger meshes, the oracle: the index buffer,
the positions and attributes written back, and the error, bit for bit."""
import numpy as np
import pytest

import fixtures
import meshoptimizer_gb300 as mg
from meshoptimizer_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from meshoptimizer_gb300 import build

    build.build()
    mg.load()


def _same(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


@pytest.mark.parametrize("case", fixtures.update_cases(), ids=lambda c: c["name"])
@pytest.mark.parametrize("device_loop", [True, False])
def test_update_fixtures(case, device_loop):
    mg.set_device_loop(device_loop)
    try:
        if case["kind"] == "interleaved":
            out, v, err = mg.simplify_with_update_interleaved(case["indices"], case["vertices"], 4, 3, [1.0], case.get("lock"), int(case["target"]),
                                                              float(case["error"]), int(case["options"]))
            assert np.array_equal(out, case["out"])
            assert _same(v, case["out_vertices"].reshape(-1))
        else:
            out, p2, a2, err = mg.simplify_with_update(case["indices"], case["positions"], int(case["target"]), float(case["error"]),
                                                       int(case["options"]), attributes=case.get("attributes"), weights=case.get("weights"),
                                                       lock=case.get("lock"))
            assert np.array_equal(out, case["out"])
            assert _same(p2, case["out_positions"])
            if "out_attributes" in case:
                assert _same(a2, case["out_attributes"])
        assert np.float32(err) == case["out_error"]
    finally:
        mg.set_device_loop(True)


def _cases():
    rng = np.random.default_rng(12)
    out = []
    idx, pos = W.heightfield(128, seed=5)
    out.append(("hf128", idx, pos, None, None, None, W.target_count(len(idx), 0.2), 2e-2, 0))
    idx, pos, attr, w = W.octa_sphere(6, seed=6)
    lock = rng.choice(np.array([0, 0, 0, 0, 1, 2, 4], np.uint8), size=len(pos))
    out.append(("sphere6_attr", idx, pos, attr, w, None, W.target_count(len(idx), 0.1), 5e-3, 0))
    out.append(("sphere6_attr_lock_permissive", idx, pos, attr, w, lock, W.target_count(len(idx), 0.1), 5e-3, mg.SimplifyPermissive))
    half = idx[: (len(idx) // 6) * 3]
    out.append(("sphere6_sparse_abs", half, pos, attr, w, None, W.target_count(len(half), 0.2), 1e-2, mg.SimplifySparse | mg.SimplifyErrorAbsolute))
    out.append(("sphere6_attr_debug", idx, pos, attr, w, None, W.target_count(len(idx), 0.1), 5e-3, 1 << 30))
    pidx, ppos = _parts(77)
    out.append(("parts_prune_lockborder", pidx, ppos, None, None, None, W.target_count(len(pidx), 0.05), 0.5, mg.SimplifyPrune | mg.SimplifyLockBorder))
    out.append(("parts_prune_sparse", pidx[: (len(pidx) // 6) * 3], ppos, None, None, None, W.target_count(len(pidx) // 2, 0.02), 0.5,
                mg.SimplifyPrune | mg.SimplifyLockBorder | mg.SimplifySparse))
    return out


def _parts(seed):
    """Disconnected heightfield pieces of different sizes and scales in one vertex buffer."""
    rng = np.random.default_rng(seed)
    parts_idx, parts_pos, base = [], [], 0
    for p in range(int(rng.integers(4, 9))):
        idx, pos = W.heightfield(int(rng.integers(4, 60)), seed=seed * 10 + p, amp=0.05)
        parts_idx.append(idx + base)
        parts_pos.append(pos * np.float32(rng.uniform(0.05, 1.0)) + rng.uniform(-2, 2, size=3).astype(np.float32))
        base += len(pos)
    return np.concatenate(parts_idx).astype(np.uint32), np.concatenate(parts_pos).astype(np.float32)


@pytest.mark.parametrize("name,idx,pos,attr,w,lock,target,error,options", _cases(), ids=lambda x: x if isinstance(x, str) else "")
def test_update_matches_oracle(port, name, idx, pos, attr, w, lock, target, error, options):
    ref = port.simplify_with_update("port", idx, pos, target, error, options, attributes=attr, weights=w, lock=lock)
    got = mg.simplify_with_update(idx, pos, target, error, options, attributes=attr, weights=w, lock=lock)
    assert np.array_equal(got[0], ref[0])
    assert _same(got[1], ref[1])
    if attr is not None:
        assert _same(got[2], ref[2])
    assert got[3] == ref[3]
    moved = int(np.sum(np.any(got[1].view(np.uint32) != np.asarray(pos, np.float32).view(np.uint32), axis=1)))
    assert moved > 0 or name == "hf128" or len(got[0]) == 0
    if options & mg.SimplifyPrune:
        unpruned = port.simplify_with_update("port", idx, pos, target, error, options & ~mg.SimplifyPrune)
        assert len(unpruned[0]) > len(got[0])  # the case removes pieces
    if options & (1 << 30):
        assert np.any(got[0] >> 28)


def test_update_device_entry(port):
    torch = pytest.importorskip("torch")
    idx, pos, attr, w = W.octa_sphere(5, seed=8)
    target = W.target_count(len(idx), 0.15)
    ref = port.simplify_with_update("port", idx, pos, target, 1e-2, 0, attributes=attr, weights=w)
    di = torch.from_numpy(idx.view(np.int32).copy()).cuda()
    dp = torch.from_numpy(pos.copy()).cuda()
    da = torch.from_numpy(attr.copy()).cuda()
    n, err = mg.simplify_with_update_device(di.data_ptr(), len(idx), dp.data_ptr(), len(pos), 12, target, 1e-2, 0, d_attributes=da.data_ptr(),
                                            attributes_stride=attr.shape[1] * 4, weights=w)
    assert np.array_equal(di[:n].cpu().numpy().view(np.uint32), ref[0])
    assert _same(dp.cpu().numpy(), ref[1])
    assert _same(da.cpu().numpy(), ref[2])
    assert err == ref[3]


def test_update_device_entry_prune(port):
    """Prune through the device entry: pieces removed before the solve, survivors written back."""
    torch = pytest.importorskip("torch")
    idx, pos = _parts(78)
    target = W.target_count(len(idx), 0.05)
    opts = mg.SimplifyPrune | mg.SimplifyLockBorder
    ref = port.simplify_with_update("port", idx, pos, target, 0.5, opts)
    di = torch.from_numpy(idx.view(np.int32).copy()).cuda()
    dp = torch.from_numpy(pos.copy()).cuda()
    n, err = mg.simplify_with_update_device(di.data_ptr(), len(idx), dp.data_ptr(), len(pos), 12, target, 0.5, opts)
    assert n < len(port.simplify_with_update("port", idx, pos, target, 0.5, mg.SimplifyLockBorder)[0])
    assert np.array_equal(di[:n].cpu().numpy().view(np.uint32), ref[0])
    assert _same(dp.cpu().numpy(), ref[1])
    assert err == ref[3]


def test_update_rejects_unknown_option():
    idx, pos = W.heightfield(8, seed=1)
    with pytest.raises(mg.SimplifyError) as e:
        mg.simplify_with_update(idx, pos, 0, 1e-2, 1 << 12)
    assert e.value.status == mg.STATUS_UNSUPPORTED
