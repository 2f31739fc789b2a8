"""The compaction step after the simplifier on device data (optimizeVertexFetchRemap,
optimizeVertexFetch, generatePositionRemap) against the reference library's outputs (the
committed fixtures) and, at a million vertices, against the oracle."""
import numpy as np
import pytest

import meshoptimizer_gb300 as mg
from meshoptimizer_gb300 import workloads as W

from fixtures import compaction_cases

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


def _host(t, dtype, count):
    return t[: count * np.dtype(dtype).itemsize].cpu().numpy().view(dtype)


def _fetch(torch, indices, vertices, in_place=False):
    vc, size = vertices.shape[0], vertices.shape[1] * vertices.itemsize
    di, dv = _dev(torch, indices), _dev(torch, vertices)
    dr = torch.empty(max(vc, 1) * 4, dtype=torch.uint8, device="cuda")
    n = mg.optimize_vertex_fetch_remap_device(dr.data_ptr(), di.data_ptr(), len(indices), vc)
    remap = _host(dr, np.uint32, vc)
    dst = dv if in_place else torch.zeros_like(dv)
    n2 = mg.optimize_vertex_fetch_device(dst.data_ptr(), di.data_ptr(), len(indices), dv.data_ptr(), vc, size)
    return remap, n, _host(di, np.uint32, len(indices)), _host(dst, np.uint8, vc * size).reshape(vc, size), n2


@pytest.mark.parametrize("in_place", [False, True])
def test_compaction_matches_golden(torch, in_place):
    for i, c in enumerate(compaction_cases()):
        if c["kind"] == "fetch":
            verts = c["vertices"]
            remap, n, idx, moved, n2 = _fetch(torch, c["indices"], verts, in_place)
            assert n == int(c["count"]) and n2 == n, i
            assert np.array_equal(remap, c["remap"]), i
            assert np.array_equal(idx, c["new_indices"]), i
            used = c["remap"] != 0xFFFFFFFF
            assert np.array_equal(moved[c["remap"][used]], verts[used]), i
        else:
            pos = np.ascontiguousarray(c["positions"], np.float32)
            dp = _dev(torch, pos)
            dr = torch.empty(max(len(pos), 1) * 4, dtype=torch.uint8, device="cuda")
            mg.generate_position_remap_device(dr.data_ptr(), dp.data_ptr(), len(pos), pos.shape[1] * 4)
            assert np.array_equal(_host(dr, np.uint32, len(pos)), c["remap"]), i


def test_compaction_after_simplify_large(torch, port):
    """A simplified 1024x1024 heightfield (2M triangles) compacted on the device: the remap,
    the rewritten indices and the moved vertices equal the oracle's; the position remap of a
    sphere with 1,023 seam duplicates equals the oracle's."""
    idx, pos = W.heightfield(1024, seed=3)
    out, _ = mg.simplify(idx, pos, W.target_count(len(idx), 0.1), 1e-2)
    remap, n, nidx, moved, n2 = _fetch(torch, out, pos)
    ref_remap, ref_n = port.optimize_vertex_fetch_remap("port", out, len(pos))
    assert n == ref_n and n2 == ref_n
    assert np.array_equal(remap, ref_remap)
    ref_idx, ref_verts, _ = port.optimize_vertex_fetch("port", out, pos)
    assert np.array_equal(nidx, ref_idx)
    assert np.array_equal(moved[:n].view(np.float32), ref_verts)
    sidx, spos, _, _ = W.octa_sphere(8, seed=2)
    dp = _dev(torch, spos)
    dr = torch.empty(len(spos) * 4, dtype=torch.uint8, device="cuda")
    mg.generate_position_remap_device(dr.data_ptr(), dp.data_ptr(), len(spos), 12)
    assert np.array_equal(_host(dr, np.uint32, len(spos)), port.generate_position_remap("port", spos))


def test_compaction_rejects_bad_input(torch):
    di = _dev(torch, np.array([0, 1, 5], np.uint32))
    dr = torch.empty(16, dtype=torch.uint8, device="cuda")
    with pytest.raises(mg.SimplifyError) as e:
        mg.optimize_vertex_fetch_remap_device(dr.data_ptr(), di.data_ptr(), 3, 4)
    assert e.value.status == mg.STATUS_INVALID_ARGUMENT
    with pytest.raises(mg.SimplifyError) as e:
        mg.optimize_vertex_fetch_device(dr.data_ptr(), di.data_ptr(), 3, dr.data_ptr(), 4, 0)
    assert e.value.status == mg.STATUS_INVALID_ARGUMENT
    remap = torch.empty(8, dtype=torch.uint8, device="cuda")
    n = mg.optimize_vertex_fetch_remap_device(remap.data_ptr(), di.data_ptr(), 0, 2)   # empty index buffer
    assert n == 0 and np.all(_host(remap, np.uint32, 2) == 0xFFFFFFFF)
