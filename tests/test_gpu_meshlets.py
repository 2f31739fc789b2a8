"""meshoptgpu_buildMeshletsFlexGroups (the re-clusterization step of a cluster-LOD level) against
the reference's own meshopt_buildMeshletsFlex (the committed fixtures) and, on cluster-LOD
groups, against the oracle restatement: meshlets, meshlet vertices and meshlet triangles, byte
for byte."""
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


def _ml():
    import meshlets as ML

    return ML


def _same(got, want, name):
    for a, b, what in zip(got, want, ("meshlets", "meshlet_vertices", "meshlet_triangles")):
        assert np.array_equal(np.asarray(a), np.asarray(b)), f"{name}: {what}"


def test_golden_cases():
    """Every fixture as a group of its own, all of one parameter set in one launch."""
    cases = fixtures.meshlet_cases()
    by_params = {}
    for c in cases:
        key = (int(c["max_vertices"]), int(c["min_triangles"]), int(c["max_triangles"]), float(c["cone_weight"]), float(c["split_factor"]))
        by_params.setdefault(key, []).append(c)
    assert len(by_params) == 6
    for key, group in by_params.items():
        # a batch shares one vertex buffer: stack the cases' buffers and offset their indices
        pos, groups, base = [], [], 0
        for c in group:
            groups.append(c["indices"].astype(np.uint32) + np.uint32(base))
            pos.append(c["positions"])
            base += len(c["positions"])
        got = mg.build_meshlets_flex_groups(groups, np.concatenate(pos), *key)
        base = 0
        for c, (m, v, t) in zip(group, got):
            _same((m, v - np.uint32(base), t), (c["meshlets"], c["meshlet_vertices"], c["meshlet_triangles"]), c["name"])
            base += len(c["positions"])


@pytest.mark.parametrize("level", [1, 0, 5])
def test_golden_cases_optimized(level):
    """The fixtures with meshopt_optimizeMeshletLevel(level) run on every meshlet afterwards."""
    cases = [c for c in fixtures.meshlet_cases() if f"opt{level}_meshlet_vertices" in c]
    assert len(cases) >= 27
    for c in cases:
        key = (int(c["max_vertices"]), int(c["min_triangles"]), int(c["max_triangles"]), float(c["cone_weight"]), float(c["split_factor"]))
        (m, v, t), = mg.build_meshlets_flex_groups([c["indices"]], c["positions"], *key, optimize_level=level)
        _same((m, v, t), (c["meshlets"], c[f"opt{level}_meshlet_vertices"], c[f"opt{level}_meshlet_triangles"]), f"{c['name']} level {level}")


def test_cluster_groups_optimized_match_oracle(port):
    """clusterlod's clusterize with its defaults: build, then optimizeMeshletLevel(1) per meshlet."""
    groups, pos, _, _, _ = W.cluster_groups(6, group_tris=512, seed=4)
    got = mg.build_meshlets_flex_groups(groups, pos, 128, 42, 128, 0.0, 2.0, optimize_level=1)
    ML = _ml()
    for g, (idx, res) in enumerate(zip(groups, got)):
        m, v, t = ML.build_meshlets_flex(idx, pos, 128, 42, 128, 0.0, 2.0, kind="port")
        v, t = ML.optimize_meshlets(m, v, t, 1, kind="port")
        _same(res, (m, v, t), f"group {g}")


@pytest.mark.parametrize("params", [(128, 42, 128, 0.0, 2.0), (64, 21, 64, 0.25, 2.0), (96, 32, 96, 0.0, 0.0)])
def test_cluster_groups_match_oracle(port, params):
    """Groups of a cluster-LOD level over one shared vertex buffer (clusterlod's default
    parameters first), against the oracle per group."""
    groups, pos, _, _, _ = W.cluster_groups(6, group_tris=512, seed=3)
    got = mg.build_meshlets_flex_groups(groups, pos, *params)
    ML = _ml()
    for g, (idx, res) in enumerate(zip(groups, got)):
        _same(res, ML.build_meshlets_flex(idx, pos, *params, kind="port"), f"group {g}")


def test_simplified_groups_match_oracle(port):
    """The input a cluster-LOD builder clusterizes: each group after the simplifier (50%)."""
    groups, pos, attr, w, lock = W.cluster_groups(6, group_tris=1024, seed=5)
    simplified = []
    for idx in groups:
        out, _ = port.simplify("port", idx, pos, W.target_count(len(idx), 0.5), 1e-2, mg.SimplifySparse | mg.SimplifyLockBorder)
        simplified.append(out)
    got = mg.build_meshlets_flex_groups(simplified, pos, 128, 42, 128, 0.0, 2.0)
    ML = _ml()
    for g, (idx, res) in enumerate(zip(simplified, got)):
        _same(res, ML.build_meshlets_flex(idx, pos, 128, 42, 128, 0.0, 2.0, kind="port"), f"group {g}")


def test_empty_and_tiny_groups(port):
    idx, pos = W.heightfield(8, seed=2)
    groups = [np.zeros(0, np.uint32), idx[:3], idx, np.zeros(0, np.uint32)]
    got = mg.build_meshlets_flex_groups(groups, pos, 64, 21, 64)
    assert len(got[0][0]) == 0 and len(got[3][0]) == 0
    ML = _ml()
    for g in (1, 2):
        _same(got[g], ML.build_meshlets_flex(groups[g], pos, 64, 21, 64, 0.0, 2.0, kind="port"), f"group {g}")


def test_nan_and_zero_area_groups(port):
    """Groups whose scores are NaN or infinite take the serial scan and still match."""
    idx, pos = W.heightfield(16, seed=4)
    bad = pos.copy()
    bad[7, 1] = np.nan
    flat = pos.copy()
    flat[:, 2] = 0.0
    flat[:, 1] = 0.0
    allpos = np.concatenate([bad, flat])
    groups = [idx, idx + np.uint32(len(pos))]
    got = mg.build_meshlets_flex_groups(groups, allpos, 64, 21, 64, 0.5, 2.0)
    ML = _ml()
    for g in range(2):
        _same(got[g], ML.build_meshlets_flex(groups[g], allpos, 64, 21, 64, 0.5, 2.0, kind="port"), f"group {g}")


def test_invalid_arguments():
    torch = pytest.importorskip("torch")
    idx, pos = W.heightfield(6, seed=1)
    d_idx = torch.from_numpy(idx.view(np.int32).copy()).cuda()
    d_pos = torch.from_numpy(pos.copy()).cuda()
    d_m = torch.zeros(4096, dtype=torch.int32, device="cuda")
    d_v = torch.zeros(len(idx), dtype=torch.int32, device="cuda")
    d_t = torch.zeros(len(idx), dtype=torch.uint8, device="cuda")
    off = np.array([0, len(idx)], np.uint64)
    rows = mg.meshlet_rows(off, 64, 21)

    def call(**kw):
        a = dict(meshlet_offsets=rows, group_offsets=off, vertex_count=len(pos), max_vertices=64, min_triangles=21, max_triangles=64,
                 optimize_level=-1)
        a.update(kw)
        return mg.build_meshlets_flex_groups_device(d_m.data_ptr(), d_v.data_ptr(), d_t.data_ptr(), a["meshlet_offsets"], d_idx.data_ptr(),
                                                    a["group_offsets"], d_pos.data_ptr(), a["vertex_count"], 12, a["max_vertices"],
                                                    a["min_triangles"], a["max_triangles"], optimize_level=a["optimize_level"], check=False)

    for kw in (dict(max_vertices=2), dict(max_vertices=257), dict(min_triangles=0), dict(min_triangles=65), dict(max_triangles=513),
               dict(group_offsets=np.array([0, len(idx) - 1], np.uint64)), dict(meshlet_offsets=np.array([0, 1], np.uint64)),
               dict(vertex_count=len(pos) - 1), dict(optimize_level=10), dict(optimize_level=-2)):
        call(**kw)
        assert mg.last_status()[0] == mg.STATUS_INVALID_ARGUMENT, kw
    call()
    assert mg.last_status()[0] == mg.STATUS_OK


def test_high_degree_fan(port):
    """A vertex shared by 2000 triangles: its list is scanned by one lane at every step."""
    n = 2000
    ang = np.linspace(0, 2 * np.pi, n, endpoint=False)
    rim = np.stack([np.cos(ang), np.sin(ang), 0.05 * np.sin(9 * ang)], axis=1)
    pos = np.concatenate([[[0.0, 0.0, 0.3]], rim]).astype(np.float32)
    idx = np.array([[0, 1 + i, 1 + (i + 1) % n] for i in range(n)], np.uint32).reshape(-1)
    ML = _ml()
    for params in ((128, 42, 128, 0.0, 2.0), (64, 16, 124, 0.25, 0.0)):
        (got,) = mg.build_meshlets_flex_groups([idx], pos, *params, optimize_level=1)
        m, v, t = ML.build_meshlets_flex(idx, pos, *params, kind="port")
        v, t = ML.optimize_meshlets(m, v, t, 1, kind="port")
        _same(got, (m, v, t), f"fan {params}")
