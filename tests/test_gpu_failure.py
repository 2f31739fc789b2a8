"""Failure detection without a GPU fault: the cooperative kernels' grid barriers wait a bounded
number of times. Here one block never arrives, the others' waits run out, they record the
error flag and return, and the context stays usable for the next simplification."""
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


@pytest.mark.parametrize("once", [False, True], ids=["pass-kernel barrier", "single-launch scan barrier"])
def test_barrier_wait_runs_out_and_reports(port, once):
    st, timed_out = mg.probe_barrier_wait(once=once, blocks=16, wait_limit=4096)
    assert st == mg.STATUS_OK
    assert timed_out == 1
    # the context is still usable: a simplification after the probe matches the oracle
    idx, pos = W.heightfield(48, seed=7)
    target = W.target_count(len(idx), 0.25)
    mg.set_dropin_batch_limit(0)
    try:
        out, err = mg.simplify(idx, pos, target, 1e-2)
    finally:
        mg.set_dropin_batch_limit()
    ref, ref_err = port.simplify("port", idx, pos, target, 1e-2, 0)
    assert np.array_equal(out, ref)


def test_barrier_probe_rejects_bad_arguments():
    for kw in (dict(blocks=1), dict(blocks=1 << 20), dict(wait_limit=0), dict(wait_limit=(1 << 20) + 1)):
        args = dict(once=False, blocks=8, wait_limit=64)
        args.update(kw)
        st, _ = mg.probe_barrier_wait(**args)
        assert st == mg.STATUS_INVALID_ARGUMENT, kw
