"""meshoptgpu_simplifyScaleNoAlloc, the allocation-free extent entry point.

It exists for callers that must not allocate device memory while they run (a frame loop with a
fixed device-memory budget, a plugin whose host application owns every allocation): it reads
positions already on the device and uses only the library's fixed scratch array. The checks,
through the C ABI:
  * two calls in a row on different meshes give the same extent as the existing
    meshopt_simplifyScale entry point and as the oracle's restatement of the reference's
    sequential fold (rescalePositions, src/simplifier.cpp:551-579), exact (the suite's 1e-6
    relative tolerance is never needed);
  * a mesh of more than 256 blocks of 2048 vertices, so that the last block folds several
    partials per thread, and a 20-byte stride;
  * NaN positions (skipped by the fold) and -0/+0 ties (the first in vertex order wins, which
    decides the sign of a zero extent);
  * an oversize vertex count is refused before any launch.
This file is collected last so that a run stopping at the first failure has run every other
test already; it also passes alone in a fresh process.
"""
import numpy as np
import pytest

import meshoptimizer_gb300 as mg
from meshoptimizer_gb300 import workloads as W

pytestmark = pytest.mark.gpu

REL_TOL = 1e-6


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from meshoptimizer_gb300 import build

    build.build()
    mg.load()
    return torch


@pytest.fixture(scope="module")
def port():
    import oracle

    if not oracle.available("port"):
        oracle.build(with_reference=False)
    return oracle


def _no_alloc(torch, host, stride):
    """The extent from the allocation-free entry point, for positions whose rows are `stride`
    bytes (the first 12 of each row are the position)."""
    rows = np.ascontiguousarray(host, np.float32)
    assert rows.shape[1] * 4 == stride
    dev = torch.from_numpy(rows).cuda()
    out = torch.full((1,), -1.0, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    st = mg.simplify_scale_noalloc(out.data_ptr(), dev.data_ptr(), rows.shape[0], stride, stream.cuda_stream)
    assert st == mg.STATUS_OK
    torch.cuda.synchronize()
    return float(out.item())


def _bits(x):
    return np.float32(x).view(np.uint32)


def _check(torch, port, host, stride, label):
    got = _no_alloc(torch, host, stride)
    want = port.simplify_scale("port", np.ascontiguousarray(host[:, :3]))
    existing = mg.simplify_scale(np.ascontiguousarray(host[:, :3]))
    assert mg.last_status()[0] == mg.STATUS_OK
    assert _bits(got) == _bits(want), (label, got, want)
    assert got == existing or abs(got - existing) <= REL_TOL * abs(existing), (label, got, existing)


def test_no_alloc_scale_matches_oracle_and_existing_entry_point(torch_cuda, port):
    torch = torch_cuda
    _, hf = W.heightfield(64, seed=21, amp=0.3)
    _, sph, _, _ = W.octa_sphere(5, seed=22)
    wide = np.concatenate([sph, np.full((len(sph), 1), 7.0, np.float32)], axis=1)  # 16-byte stride
    # two calls in a row on different meshes: the shared scratch keeps nothing between them
    _check(torch, port, hf, 12, "heightfield")
    _check(torch, port, wide, 16, "sphere, 16-byte stride")


def test_no_alloc_scale_many_blocks_and_stride(torch_cuda, port):
    torch = torch_cuda
    # 700,001 vertices: 342 blocks of 2048, so the last block folds two partials per thread
    # (256 threads); a 20-byte stride with unrelated data after each position
    rng = np.random.default_rng(5)
    n = 700001
    pos = (rng.standard_normal((n, 3)) * np.array([3.0, 0.5, 11.0])).astype(np.float32)
    rows = np.concatenate([pos, np.full((n, 2), -1e30, np.float32)], axis=1)
    _check(torch, port, rows, 20, "700,001 vertices, 20-byte stride")
    _check(torch, port, pos[: n // 3], 12, "a third of them")


def test_no_alloc_scale_nan_and_signed_zero(torch_cuda, port):
    torch = torch_cuda
    # NaN rows are skipped by the reference's comparisons; extremes of -0 and +0 compare equal and
    # the first in vertex order stays, so a mesh whose extent is zero keeps the sign the reference gives
    n = 5000
    pos = np.zeros((n, 3), np.float32)
    pos[1::2] = -0.0
    pos[3] = np.nan
    pos[4000, 1] = np.nan
    _check(torch, port, pos, 12, "zeros of both signs with NaN")
    pos2 = pos.copy()
    pos2[0] = -0.0
    pos2[1] = 0.0
    _check(torch, port, pos2, 12, "signs swapped")
    pos3 = np.full((n, 3), np.nan, np.float32)
    pos3[2500] = (1.0, -2.0, 0.5)
    pos3[2501] = (-1.0, 2.0, -0.0)
    _check(torch, port, pos3, 12, "NaN everywhere but two rows")


def test_no_alloc_scale_rejects_oversize(torch_cuda):
    torch = torch_cuda
    out = torch.zeros(1, dtype=torch.float32, device="cuda")
    st = mg.simplify_scale_noalloc(out.data_ptr(), 0, 67108864 + 1, 12)
    assert st == mg.STATUS_INVALID_ARGUMENT
