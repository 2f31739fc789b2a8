"""One cluster-LOD level on the GPU (meshoptgpu_simplifyGroups: boundary locks, then every group
in one batch launch) against the reference builder's locks and the reference simplifier's
outputs, for two consecutive levels whose locks persist on the device."""
import numpy as np
import pytest

import meshoptimizer_gb300 as mg

from fixtures import clod_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    from meshoptimizer_gb300 import build

    build.build()
    mg.load()
    return t


def _dev(torch, a):
    a = np.ascontiguousarray(a)
    t = torch.empty(max(a.nbytes, 4), dtype=torch.uint8, device="cuda")
    if a.nbytes:
        t[: a.nbytes].copy_(torch.from_numpy(a.view(np.uint8).reshape(-1)))
    return t


@pytest.mark.parametrize("threads", [0, 128])
def test_groups_two_levels_match_reference(torch, threads):
    mg.set_batch_config(threads)
    try:
        for c in clod_cases():
            pos, attr = c["positions"], c["attributes"]
            dp, da = _dev(torch, pos), _dev(torch, attr)
            dvl = _dev(torch, c["vertex_lock"])
            dlocks = _dev(torch, c["locks_in"])
            # the position remap comes from the device too
            dremap = torch.empty(len(pos) * 4, dtype=torch.uint8, device="cuda")
            mg.generate_position_remap_device(dremap.data_ptr(), dp.data_ptr(), len(pos), 12)
            assert np.array_equal(dremap.cpu().numpy().view(np.uint32), c["remap"])
            for level in (1, 2):
                idx = c[f"l{level}_indices"]
                off = c[f"l{level}_offsets"]
                di = _dev(torch, idx)
                do = torch.empty(max(len(idx), 1) * 4, dtype=torch.uint8, device="cuda")
                counts, errs = mg.simplify_groups_device(do.data_ptr(), di.data_ptr(), off, dp.data_ptr(), len(pos), 12, dremap.data_ptr(),
                                                         dlocks.data_ptr(), c[f"l{level}_targets"], float(c["error"]), int(c["options"]),
                                                         d_attributes=da.data_ptr(), attributes_stride=attr.shape[1] * 4, weights=c["weights"],
                                                         d_vertex_lock=dvl.data_ptr())
                assert np.array_equal(dlocks[: len(pos)].cpu().numpy(), c[f"l{level}_locks"]), level
                assert np.array_equal(counts, c[f"l{level}_counts"]), level
                assert np.array_equal(errs, c[f"l{level}_errors"]), level
                got = do.cpu().numpy().view(np.uint32)
                exp = c[f"l{level}_out"]
                o = 0
                for g in range(len(off) - 1):
                    n = int(counts[g])
                    assert np.array_equal(got[int(off[g]): int(off[g]) + n], exp[o: o + n]), (level, g)
                    o += n
    finally:
        mg.set_batch_config(0)


def test_groups_reject_bad_remap(torch):
    pos = np.zeros((4, 3), np.float32)
    idx = np.array([0, 1, 2], np.uint32)
    dp, di = _dev(torch, pos), _dev(torch, idx)
    dremap = _dev(torch, np.array([0, 1, 9, 3], np.uint32))
    dl = _dev(torch, np.zeros(4, np.uint8))
    do = torch.empty(12, dtype=torch.uint8, device="cuda")
    with pytest.raises(mg.SimplifyError) as e:
        mg.simplify_groups_device(do.data_ptr(), di.data_ptr(), [0, 3], dp.data_ptr(), 4, 12, dremap.data_ptr(), dl.data_ptr(), [0], 1e-2, 0)
    assert e.value.status == mg.STATUS_INVALID_ARGUMENT
