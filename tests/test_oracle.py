"""The CPU oracle (oracle/mo_oracle.c) pinned against the reference's own results:
the known-answer cases of demo/tests.cpp and seeded meshes run through the reference
library, both committed as fixtures under tests/golden/."""
import ctypes as C

import numpy as np
import pytest

import fixtures


def _run_port_raw(oracle, c):
    """Calls the port with the case's exact buffers and strides (interleaved layouts kept)."""
    o = oracle.load("port")
    idx = np.ascontiguousarray(c["indices"])
    pos = np.ascontiguousarray(c["positions"])
    vcount = len(pos) * 4 // c["stride"]
    out = np.zeros(max(len(idx), 1), np.uint32)
    err = C.c_float(0)
    p = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)  # noqa: E731
    attrs, weights, lock = c["attributes"], c["weights"], c["lock"]
    acount = 0 if weights is None else len(weights)
    n = o._simplify_attr(p(out), p(idx), len(idx), p(pos), vcount, c["stride"], p(attrs), c["attr_stride"],
                         p(weights), acount, p(lock), c["target"], c["error"], c["options"], C.byref(err))
    return out[:n].copy(), float(err.value)


@pytest.mark.parametrize("case", fixtures.known_answers(), ids=lambda c: c["name"])
def test_port_known_answers(port, case):
    out, err = _run_port_raw(port, case)
    assert np.array_equal(out, case["ref_output"])
    assert err == np.float32(case["ref_error"])
    if case["expect"] is not None:
        assert np.array_equal(out[:len(case["expect"])], case["expect"])
    if case["expect_count"] is not None:
        assert len(out) == case["expect_count"]
    if case["expect_error_lt"] is not None:
        assert err < case["expect_error_lt"]
    if case["expect_error_near"] is not None:
        assert abs(err - case["expect_error_near"][0]) < case["expect_error_near"][1]


@pytest.mark.parametrize("case", fixtures.seeded_cases(), ids=lambda c: c["name"])
def test_port_seeded(port, case):
    out, err = port.simplify("port", case["indices"], case["positions"], case["target"], case["error"], case["options"],
                             attributes=case["attributes"], weights=case["weights"])
    assert np.array_equal(out, case["expect"])
    assert np.float32(err) == np.float32(case["expect_error"])


def test_port_scale(port):
    vb = np.array([0, 0, 0, 1, 0, 0, 0, 2, 0, 0, 0, 3], np.float32).reshape(-1, 3)
    assert port.simplify_scale("port", vb) == 3.0  # demo/tests.cpp simplifyScale


def test_port_fp64_close(port):
    """The FP64 oracle stays within a small relative distance of the FP32 result error."""
    from meshoptimizer_gb300 import workloads as W

    idx, pos = W.heightfield(33, seed=3, amp=0.05)
    t = W.target_count(len(idx), 0.25)
    _, e32 = port.simplify("port", idx, pos, t, 1e-2, 0)
    _, e64, _ = port.simplify("port", idx, pos, t, 1e-2, 0, fp64=True)
    assert abs(e32 - e64) <= 0.05 * e64


def test_port_empty(port):
    out, err = port.simplify("port", np.zeros(0, np.uint32), np.zeros((3, 3), np.float32), 0, 1e-2, 0)
    assert len(out) == 0 and err == 0


def test_compaction_port_matches_golden(port):
    """The oracle's restatement of the compaction step after the simplifier
    (optimizeVertexFetchRemap / optimizeVertexFetch / generatePositionRemap) against the
    reference library's outputs on the committed seeded cases."""
    from fixtures import compaction_cases

    for i, c in enumerate(compaction_cases()):
        if c["kind"] == "fetch":
            remap, n = port.optimize_vertex_fetch_remap("port", c["indices"], c["vertices"].shape[0])
            assert np.array_equal(remap, c["remap"]) and n == int(c["count"]), i
            idx, verts, n2 = port.optimize_vertex_fetch("port", c["indices"], c["vertices"])
            assert np.array_equal(idx, c["new_indices"]) and n2 == n, i
            used = c["remap"] != 0xFFFFFFFF
            assert np.array_equal(verts[c["remap"][used]], c["vertices"][used]), i
        else:
            assert np.array_equal(port.generate_position_remap("port", c["positions"]), c["remap"]), i


def test_clod_level_port_matches_golden(port):
    """The oracle's cluster-LOD level (lockBoundary restatement + the port simplifier on every
    group) against the reference builder's locks and the reference simplifier's outputs."""
    import clod
    from fixtures import clod_cases

    for c in clod_cases():
        locks = c["locks_in"]
        for level in (1, 2):
            off = c[f"l{level}_offsets"].astype(np.int64)
            idx = c[f"l{level}_indices"]
            groups = [idx[off[g]:off[g + 1]] for g in range(len(off) - 1)]
            locks, res = clod.simplify_level("port", groups, c["positions"], c["attributes"], c["weights"], c["remap"], locks, c["vertex_lock"],
                                             c[f"l{level}_targets"], float(c["error"]), int(c["options"]))
            assert np.array_equal(locks, c[f"l{level}_locks"])
            assert np.array_equal(np.concatenate([o for o, _ in res]), c[f"l{level}_out"])
            assert np.array_equal(np.array([len(o) for o, _ in res]), c[f"l{level}_counts"].astype(np.int64))
            assert np.array_equal(np.array([e for _, e in res], np.float32), c[f"l{level}_errors"])


def test_update_port_matches_golden(port):
    """meshopt_simplifyWithUpdate's restatement against the reference library's indices,
    rewritten positions and attributes, and error (the reference's own simplifyUpdate tests and
    seeded meshes), bit for bit."""
    from fixtures import update_cases

    for c in update_cases():
        if c["kind"] == "interleaved":
            out, v, err = port.simplify_with_update_interleaved("port", c["indices"], c["vertices"], 4, 3, [1.0], c.get("lock"), int(c["target"]),
                                                                float(c["error"]), int(c["options"]))
            assert np.array_equal(out, c["out"]), c["name"]
            assert np.array_equal(v.view(np.uint32), c["out_vertices"].reshape(-1).view(np.uint32)), c["name"]
        else:
            out, p2, a2, err = port.simplify_with_update("port", c["indices"], c["positions"], int(c["target"]), float(c["error"]), int(c["options"]),
                                                         attributes=c.get("attributes"), weights=c.get("weights"), lock=c.get("lock"))
            assert np.array_equal(out, c["out"]), c["name"]
            assert np.array_equal(p2.view(np.uint32), c["out_positions"].view(np.uint32)), c["name"]
            if "out_attributes" in c:
                assert np.array_equal(a2.view(np.uint32), c["out_attributes"].view(np.uint32)), c["name"]
        assert np.float32(err) == c["out_error"], c["name"]


def test_meshlet_port_matches_golden(port):
    """mo_buildMeshletsFlex (oracle/mo_meshlet.c) against the reference's meshopt_buildMeshletsFlex
    outputs: the meshlets, their vertices and their triangles, byte for byte."""
    import meshlets as ML

    cases = fixtures.meshlet_cases()
    assert len(cases) >= 50
    for c in cases:
        m, v, t = ML.build_meshlets_flex(c["indices"], c["positions"], int(c["max_vertices"]), int(c["min_triangles"]), int(c["max_triangles"]),
                                         float(c["cone_weight"]), float(c["split_factor"]), kind="port")
        assert np.array_equal(m, c["meshlets"]), c["name"]
        assert np.array_equal(v, c["meshlet_vertices"]), c["name"]
        assert np.array_equal(t, c["meshlet_triangles"]), c["name"]


def test_meshlet_port_bound():
    import meshlets as ML

    # meshopt_buildMeshletsBound: the larger of the vertex-limited and triangle-limited counts
    assert ML.bound(3 * 1000, 64, 124, kind="port") == max((3000 + 61) // 62, (1000 + 123) // 124)
    assert ML.bound(0, 64, 124, kind="port") == 0


def test_meshlet_optimize_port_matches_golden(port):
    """mo_optimizeMeshletLevel against the reference's meshopt_optimizeMeshletLevel outputs."""
    import meshlets as ML

    checked = 0
    for c in fixtures.meshlet_cases():
        for level in (0, 1, 5):
            if f"opt{level}_meshlet_vertices" not in c:
                continue
            v, t = ML.optimize_meshlets(c["meshlets"], c["meshlet_vertices"], c["meshlet_triangles"], level, kind="port")
            assert np.array_equal(v, c[f"opt{level}_meshlet_vertices"]), (c["name"], level)
            assert np.array_equal(t, c[f"opt{level}_meshlet_triangles"]), (c["name"], level)
            checked += 1
    assert checked >= 100


def test_port_matches_reference_library_fuzz(port):
    """Where the reference library was built from its own sources (oracle/_ref, this container
    only), the port against it on fuzzed meshes: lattice soups with duplicates and degenerate
    triangles, every option bit, attributes with zero weights and lock flags."""
    if not port.available("ref"):
        pytest.skip("the reference library is built only where the reference sources are present")
    rng = np.random.default_rng(2024)
    bits = [1 << b for b in range(7)]  # meshoptimizer.h:469-481: LockBorder, Sparse, ErrorAbsolute, Prune, Regularize, Permissive, RegularizeLight
    for _ in range(150):
        V = int(rng.integers(4, 120))
        pos = rng.integers(0, int(rng.integers(2, 9)), size=(V, 3)).astype(np.float32)
        idx = rng.integers(0, V, size=3 * int(rng.integers(1, 200))).astype(np.uint32)
        options = 0
        for b in bits:
            if rng.random() < 0.3:
                options |= b
        attrs = weights = lock = None
        if rng.random() < 0.5:
            ac = int(rng.integers(1, 5))
            attrs = rng.random((V, ac)).astype(np.float32)
            weights = rng.choice(np.array([0.0, 0.5, 1.0], np.float32), size=ac)
        if rng.random() < 0.4:
            lock = rng.choice(np.array([0, 0, 1, 2, 4, 6], np.uint8), size=V)
        target = int(rng.integers(0, len(idx) // 3 + 1)) * 3
        error = float(rng.choice([1e-2, 0.1, float(np.finfo(np.float32).max)]))
        a = port.simplify("port", idx, pos, target, error, options, attributes=attrs, weights=weights, lock=lock)
        b = port.simplify("ref", idx, pos, target, error, options, attributes=attrs, weights=weights, lock=lock)
        assert np.array_equal(a[0], b[0]), (options, target, error)
        assert np.float32(a[1]) == np.float32(b[1])


def test_meshlet_port_matches_reference_fuzz():
    """Where the reference's clusterizer was built from its sources (this container only), the
    meshlet port against it on fuzzed groups: random subsets of a noisy heightfield and lattice
    soups, random parameter sets within the reference's asserts, and the per-meshlet reorder."""
    import meshlets as ML
    from meshoptimizer_gb300 import workloads as W

    if not (ML.available("port") and ML.available("reference")):
        pytest.skip("the reference clusterizer is built only where the reference sources are present")
    rng = np.random.default_rng(77)
    for _ in range(40):
        if rng.random() < 0.5:
            idx, pos = W.heightfield(int(rng.integers(4, 40)), seed=int(rng.integers(0, 1 << 30)), amp=float(rng.uniform(0.0, 0.3)))
            tri = idx.reshape(-1, 3)
            idx = tri[rng.random(len(tri)) < rng.uniform(0.3, 1.0)].reshape(-1).astype(np.uint32)
        else:
            V = int(rng.integers(8, 200))
            pos = rng.random((V, 3)).astype(np.float32)
            idx = rng.integers(0, V, size=3 * int(rng.integers(1, 300))).astype(np.uint32)
        max_v = int(rng.choice([16, 64, 128, 255]))
        max_t = int(rng.choice([8, 64, 124, 256, 512]))
        min_t = int(rng.integers(1, max_t + 1))
        cone = float(rng.choice([0.0, 0.25, 0.5]))
        split = float(rng.choice([0.0, 2.0]))
        a = ML.build_meshlets_flex(idx, pos, max_v, min_t, max_t, cone, split, kind="port")
        b = ML.build_meshlets_flex(idx, pos, max_v, min_t, max_t, cone, split, kind="reference")
        for x, y in zip(a, b):
            assert np.array_equal(np.asarray(x), np.asarray(y)), (max_v, min_t, max_t, cone, split)
        level = int(rng.choice([0, 1, 3]))
        oa = ML.optimize_meshlets(*a, level, kind="port")
        ob = ML.optimize_meshlets(*b, level, kind="reference")
        for x, y in zip(oa, ob):
            assert np.array_equal(np.asarray(x), np.asarray(y)), ("optimize", level)
