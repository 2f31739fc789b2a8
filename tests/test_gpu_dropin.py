"""Small drop-in calls routed to the batch kernel (a batch of one): the same results as the
reference (the committed fixtures) and the oracle, through meshopt_simplify /
meshopt_simplifyWithAttributes and the device-resident entry point."""
import numpy as np
import pytest

import fixtures
import meshoptimizer_gb300 as mg
from meshoptimizer_gb300 import workloads as W

pytestmark = pytest.mark.gpu

BATCH_OPTIONS = (mg.SimplifyLockBorder | mg.SimplifyErrorAbsolute | mg.SimplifyRegularize | mg.SimplifyRegularizeLight | mg.SimplifySparse
                 | mg.SimplifyPermissive)


def close(a, b):
    return a == b or abs(a - b) <= 1e-6 * max(abs(a), abs(b))


@pytest.fixture(scope="module", autouse=True)
def built():
    from meshoptimizer_gb300 import build

    build.build()
    mg.load()
    mg.set_dropin_batch_limit(24000)  # every seeded case up to 24000 indices on the batch kernel
    yield
    mg.set_dropin_batch_limit()


def _routed(call):
    mg.set_kernel_profile("kBatch")
    r = call()
    n, _ = mg.kernel_profile()
    mg.set_kernel_profile(None)
    assert n >= 1, "the call did not run on the batch kernel"
    assert mg.last_pass_stats() == []
    return r


@pytest.mark.parametrize("case", fixtures.known_answers(), ids=lambda c: c["name"])
def test_known_answers_routed(case):
    if case["options"] & ~BATCH_OPTIONS or len(case["indices"]) == 0:
        pytest.skip("option or shape that stays on the single-mesh path")
    idx, pos = case["indices"], case["positions"]
    out = np.zeros(max(len(idx), 1), np.uint32)
    weights = case["weights"]
    n, err = _routed(lambda: mg.simplify_raw(out, idx, len(idx), pos, len(pos) * 4 // case["stride"], case["stride"], case["target"],
                                             case["error"], case["options"], attributes=case["attributes"],
                                             attributes_stride=case["attr_stride"], weights=weights,
                                             attribute_count=0 if weights is None else len(weights), lock=case["lock"]))
    assert np.array_equal(out[:n], case["ref_output"])
    assert close(err, case["ref_error"])


@pytest.mark.parametrize("case", [c for c in fixtures.seeded_cases() if len(c["indices"]) <= 24000], ids=lambda c: c["name"])
def test_seeded_routed(case):
    if case["options"] & ~BATCH_OPTIONS:
        pytest.skip("option that stays on the single-mesh path")
    out, err = _routed(lambda: mg.simplify(case["indices"], case["positions"], case["target"], case["error"], case["options"],
                                           attributes=case["attributes"], weights=case["weights"]))
    assert np.array_equal(out, case["expect"])
    assert close(err, case["expect_error"])


def test_routing_limit_and_device_entry(port):
    torch = pytest.importorskip("torch")
    idx, pos, attr, w = W.octa_sphere(5, seed=6)          # 8192 triangles, 24576 indices: above the default limit
    t = W.target_count(len(idx), 0.2)
    ref, ref_err = port.simplify("port", idx, pos, t, 5e-2, 0, attributes=attr, weights=w)
    out, err = mg.simplify(idx, pos, t, 5e-2, attributes=attr, weights=w)
    assert len(mg.last_pass_stats()) > 0                   # single-mesh path
    assert np.array_equal(out, ref)
    mg.set_dropin_batch_limit(len(idx))
    try:
        out2, err2 = _routed(lambda: mg.simplify(idx, pos, t, 5e-2, attributes=attr, weights=w))
        assert np.array_equal(out2, ref) and close(err2, ref_err)
        di = torch.from_numpy(idx.view(np.int32)).cuda()
        dp = torch.from_numpy(pos).cuda()
        da = torch.from_numpy(attr).cuda()
        do = torch.empty_like(di)
        n, e = _routed(lambda: mg.simplify_device(do.data_ptr(), di.data_ptr(), len(idx), dp.data_ptr(), len(pos), 12, t, 5e-2, 0,
                                                 d_attributes=da.data_ptr(), attributes_stride=20, weights=w))
        assert np.array_equal(do[:n].cpu().numpy().view(np.uint32), ref) and close(e, ref_err)
    finally:
        mg.set_dropin_batch_limit(24000)


def test_routed_invalid_index_is_reported():
    idx = np.array([0, 1, 7], np.uint32)
    pos = np.zeros((3, 3), np.float32)
    out, err = mg.simplify(idx, pos, 0, 1e-2, check=False)
    assert mg.last_status()[0] == mg.STATUS_INVALID_ARGUMENT
    assert np.array_equal(out, idx)
