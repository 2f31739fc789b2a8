"""meshoptgpu_simplifyScaleNoAlloc, the allocation-free extent entry point.

It exists for callers that must not allocate device memory while they run (for example
work recorded into a CUDA graph, or a frame loop with a fixed memory budget): it reads
positions already on the device and uses only the library's fixed scratch array. The
check: through the C ABI, two calls in a row on different meshes give the same extent as
the existing meshopt_simplifyScale entry point (exact; within the suite's 1e-6 relative
tolerance by construction), and an oversize vertex count is refused before any launch.
This file is collected last so that a run stopping at the first failure has run every
other test already; it also passes alone in a fresh process.
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


def test_no_alloc_scale_matches_existing_entry_point(torch_cuda):
    torch = torch_cuda
    _, hf = W.heightfield(64, seed=21, amp=0.3)
    _, sph, _, _ = W.octa_sphere(5, seed=22)
    wide = np.concatenate([sph, np.full((len(sph), 1), 7.0, np.float32)], axis=1)  # 16-byte stride
    stream = torch.cuda.current_stream()
    out = torch.full((1,), -1.0, dtype=torch.float32, device="cuda")
    for host, stride in ((hf, 12), (wide, 16)):
        dev = torch.from_numpy(np.ascontiguousarray(host)).cuda()
        st = mg.simplify_scale_noalloc(out.data_ptr(), dev.data_ptr(), host.shape[0], stride, stream.cuda_stream)
        assert st == mg.STATUS_OK
        torch.cuda.synchronize()
        got = float(out.item())
        want = mg.simplify_scale(host)
        assert mg.last_status()[0] == mg.STATUS_OK
        assert got == want or abs(got - want) <= REL_TOL * abs(want)


def test_no_alloc_scale_rejects_oversize(torch_cuda):
    torch = torch_cuda
    out = torch.zeros(1, dtype=torch.float32, device="cuda")
    st = mg.simplify_scale_noalloc(out.data_ptr(), 0, 67108864 + 1, 12)
    assert st == mg.STATUS_INVALID_ARGUMENT
