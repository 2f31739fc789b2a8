"""Serving: requests of different sizes submitted concurrently to the continuous-batching
server give exactly the results each one gives alone (the oracle), on the batch path and
the single-mesh path; admission by memory budget delays but never drops requests."""
import numpy as np
import pytest

import meshoptimizer_gb300 as mg
from meshoptimizer_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    from meshoptimizer_gb300 import build

    build.build()
    mg.load()
    return t


def _requests():
    reqs = []
    rng = np.random.default_rng(11)
    for idx, pos in W.sphere_patches(40, seed=41, levels=5):
        reqs.append((idx, pos, W.target_count(len(idx), float(rng.uniform(0.1, 0.5))), 1e-2, 0))
    for n in (30, 60, 101, 160):
        idx, pos = W.heightfield(n, seed=n, amp=0.05)
        reqs.append((idx, pos, W.target_count(len(idx), float(rng.uniform(0.1, 0.5))), 1e-2, 0))
    return reqs


def _upload(torch, reqs):
    dev = []
    for idx, pos, t, e, o in reqs:
        di = torch.from_numpy(idx.view(np.int32)).cuda()
        dp = torch.from_numpy(pos).cuda()
        do = torch.empty(max(len(idx), 1), dtype=torch.int32, device="cuda")
        dev.append((di, dp, do))
    return dev


@pytest.mark.parametrize("cfg", [dict(), dict(large_index_count=3 * 5000), dict(plain=True), dict(memory_budget=64 << 20)],
                         ids=["batched", "mixed-paths", "plain", "tight-budget"])
def test_server_results_equal_standalone(port, torch, cfg):
    reqs = _requests()
    dev = _upload(torch, reqs)
    torch.cuda.synchronize()
    with mg.Server(**cfg) as srv:
        tickets = [srv.submit(di.data_ptr(), len(r[0]), dp.data_ptr(), len(r[1]), r[2], r[3], r[4], do.data_ptr())
                   for r, (di, dp, do) in zip(reqs, dev)]
        outs = [srv.wait(t) for t in tickets]
        stats = srv.stats()
    assert stats["completed"] == len(reqs)
    for (idx, pos, t, e, o), (di, dp, do), (st, n, err, lat) in zip(reqs, dev, outs):
        assert st == mg.STATUS_OK
        ref, ref_err = port.simplify("port", idx, pos, t, e, o)
        got = do[:n].cpu().numpy().view(np.uint32)
        assert np.array_equal(got, ref)
        assert err == ref_err or abs(err - ref_err) <= 1e-6 * abs(ref_err)
        assert lat >= 0


def test_server_rejects_request_over_budget(torch):
    idx, pos = W.heightfield(200, seed=1)
    di = torch.from_numpy(idx.view(np.int32)).cuda()
    dp = torch.from_numpy(pos).cuda()
    do = torch.empty(len(idx), dtype=torch.int32, device="cuda")
    with mg.Server(memory_budget=1 << 20, large_index_count=3) as srv:
        with pytest.raises(mg.SimplifyError) as e:
            srv.submit(di.data_ptr(), len(idx), dp.data_ptr(), len(pos), 1000, 1e-2, 0, do.data_ptr())
        assert e.value.status == mg.STATUS_OUT_OF_MEMORY


def test_server_attributes_locks_and_prune(port, torch):
    """Requests with attributes, vertex_lock and the cluster-LOD options take the batch kernel;
    Prune requests (which the batch kernel does not have) are routed to the single-mesh path;
    all equal the oracle."""
    groups, pos, attr, w, lock = W.cluster_groups(5, 256)
    opts = mg.SimplifySparse | mg.SimplifyErrorAbsolute | mg.SimplifyPermissive
    dp, da, dl = torch.from_numpy(pos).cuda(), torch.from_numpy(attr).cuda(), torch.from_numpy(lock).cuda()
    reqs = [(g, (len(g) // 6) * 3, float(np.finfo(np.float32).max), opts) for g in groups[:12]]
    hi, hp = W.heightfield(40, seed=8)
    pi_ = np.concatenate([hi, hi[: (len(hi) // 12) * 3] + len(hp)])  # two components: pruning removes the small one first
    pp = np.concatenate([hp, hp * 0.01 + 3.0])
    dev = []
    with mg.Server() as srv:
        tickets = []
        for g, t, e, o in reqs:
            di = torch.from_numpy(g.view(np.int32)).cuda()
            do = torch.empty(len(g), dtype=torch.int32, device="cuda")
            dev.append((di, do))
            tickets.append(srv.submit(di.data_ptr(), len(g), dp.data_ptr(), len(pos), t, e, o, do.data_ptr(), d_attributes=da.data_ptr(),
                                      attr_stride=attr.shape[1] * 4, weights=w, d_lock=dl.data_ptr()))
        di = torch.from_numpy(pi_.astype(np.uint32).view(np.int32)).cuda()
        dpp = torch.from_numpy(pp.astype(np.float32)).cuda()
        do = torch.empty(len(pi_), dtype=torch.int32, device="cuda")
        tp = srv.submit(di.data_ptr(), len(pi_), dpp.data_ptr(), len(pp), W.target_count(len(pi_), 0.3), 5e-2, mg.SimplifyPrune, do.data_ptr())
        outs = [srv.wait(t) for t in tickets]
        st, n, err, _ = srv.wait(tp)
        stats = srv.stats()
    assert stats["singles"] >= 1 and stats["batches"] >= 1
    for (g, t, e, o), (di_, do_), (s, k, er, _) in zip(reqs, dev, outs):
        assert s == mg.STATUS_OK
        ref, ref_err = port.simplify("port", g, pos, t, e, o, attributes=attr, weights=w, lock=lock)
        assert np.array_equal(do_[:k].cpu().numpy().view(np.uint32), ref)
        assert er == ref_err or abs(er - ref_err) <= 1e-6 * abs(ref_err)
    assert st == mg.STATUS_OK
    ref, ref_err = port.simplify("port", pi_.astype(np.uint32), pp.astype(np.float32), W.target_count(len(pi_), 0.3), 5e-2, mg.SimplifyPrune)
    assert np.array_equal(do[:n].cpu().numpy().view(np.uint32), ref)
