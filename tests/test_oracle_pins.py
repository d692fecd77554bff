"""Pins the oracle (oracle/skw_oracle.cpp) to the reference: golden vectors
generated from the reference's own code, the reference unit tests'
brute-force checks, and -- where the reference library is built here -- a
direct comparison on fresh inputs."""
from pathlib import Path

import numpy as np
import pytest

import scene_fixtures as sf
from skwarka_gb300 import scenes

GOLD = Path(__file__).resolve().parent / "golden"


def _golden_meshes(g):
    meshes, i = [], 0
    while f"mesh{i}_vertices" in g:
        meshes.append((g[f"mesh{i}_vertices"], g[f"mesh{i}_triangles"]))
        i += 1
    return meshes


def _same_tree(a, b):
    """Same nodes exactly; same triangles per leaf (order inside a leaf may
    differ, see scene_fixtures.canonical_leaf_order)."""
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(sf.canonical_leaf_order(a[1], a[2], a[3]), sf.canonical_leaf_order(b[1], b[2], b[3]))


def test_oracle_matches_golden_accel(oracle):
    g = np.load(GOLD / "accel_small.npz")
    oa = oracle.accel(_golden_meshes(g))
    _same_tree(oa.export(), (g["node_bbox"], g["node_info"], g["tri_prim"], g["tri_index"]))
    h = oa.intersect(g["rays"], threads=1)
    assert np.array_equal(h["prim"], g["hit_prim"]) and np.array_equal(h["tri"], g["hit_tri"])
    assert np.array_equal(h["t"], g["hit_t"])  # bit-exact double t
    assert np.array_equal(oa.intersect_test(g["shadow_rays"], threads=1), g["occluded"])


def test_oracle_matches_golden_knn(oracle):
    g = np.load(GOLD / "knn_small.npz")
    kd = oracle.kdtree(g["pos"], g["normal_ids"])
    assert np.array_equal(kd.perm, g["perm"]) and np.array_equal(kd.nodes, g["nodes"])
    rf = kd.knn(g["q"], g["qn"], 20, 0.15, 0.5, threads=1)
    assert np.array_equal(rf["count"], g["filt_count"])
    assert np.array_equal(rf["idx"], g["filt_idx"]) and np.array_equal(rf["d2"], g["filt_d2"])
    ru = kd.knn(g["q"], None, 20, 0.2, -1.0, threads=1)
    assert np.array_equal(ru["idx"], g["all_idx"]) and np.array_equal(ru["d2"], g["all_d2"])


def test_oracle_direction_table_golden(oracle):
    g = np.load(GOLD / "compressed_direction.npz")
    assert np.array_equal(oracle.direction_table()[g["ids"]], g["vectors"])


def test_oracle_intersect_equals_brute_force(oracle):
    """TriangleAccelerator.test.h:65-98 / 137-162: accelerator answers equal a
    brute-force double Moller-Trumbore over all triangles."""
    meshes = sf.unit_test_spheres()
    rays = sf.unit_test_rays(meshes, 1000)
    oa = oracle.accel(meshes)
    h = oa.intersect(rays)
    bp, bt, bth = oracle.brute_force(oa.tris, oa.prim, oa.tidx, rays)
    assert np.array_equal(h["prim"], bp) and np.array_equal(h["tri"], bt)
    hit = h["prim"] >= 0
    assert np.all(np.abs(h["t"][hit] - bth[hit]) <= 1e-9)
    occ = oa.intersect_test(rays)
    assert np.array_equal(occ.astype(bool), bp >= 0)


def test_oracle_knn_equals_brute_force(oracle):
    """KDTree.test.h:160-255: k-NN distance multisets equal brute force, for
    10,000 random points plus 100 duplicates and k in [1, 500]."""
    rng = np.random.default_rng(5)
    pos = rng.uniform(0, 1, size=(10_100, 3)).astype(np.float32)
    pos[10_000:] = pos[:100]
    kd = oracle.kdtree(pos)
    tree_pos = pos[kd.perm].astype(np.float64)
    for k in (1, 7, 100, 500):
        q = rng.uniform(0, 1, size=(20, 3))
        r = kd.knn(q, None, k, 10.0)
        for i in range(len(q)):
            d2 = ((tree_pos - q[i]) ** 2).sum(1)
            want = np.sort(d2)[:k]
            got = np.sort(r["d2"][i, :r["count"][i]])
            assert np.array_equal(got, want)


def test_oracle_equals_reference_fresh(oracle, reference):
    """Direct comparison with the reference's own code on fresh inputs."""
    meshes = sf.small_query_scene()
    lo, hi = scenes.scene_bounds(meshes)
    rays = scenes.uniform_rays(20_000, lo, hi, seed=41)
    srays = scenes.uniform_rays(20_000, lo, hi, seed=42, tmax_range=(0.0, 2.0))
    oa, ra = oracle.accel(meshes), reference.accel(meshes)
    _same_tree(oa.export(), ra.export())
    ho, hr = oa.intersect(rays), ra.intersect(rays)
    for key in ("prim", "tri", "t"):
        assert np.array_equal(ho[key], hr[key])
    assert np.array_equal(oa.intersect_test(srays), ra.intersect_test(srays))


def test_oracle_tree_degenerate_equals_reference(oracle, reference):
    """Zero-extent nodes (coplanar axis-aligned triangles) and the unit-test
    spheres build the same tree in the oracle and the reference."""
    for meshes in (sf.flat_tiles(), sf.unit_test_spheres()):
        oa, ra = oracle.accel(meshes), reference.accel(meshes)
        _same_tree(oa.export(), ra.export())


def test_oracle_knn_equals_reference_fresh(oracle, reference):
    rng = np.random.default_rng(77)
    pos = rng.normal(size=(6000, 3)).astype(np.float32) * 0.3
    pos[:300] = np.round(pos[:300], 1)  # many exact ties in distance
    nrm = rng.normal(size=(6000, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nids = np.array([reference.lib.skw_ref_compress_direction(*v) for v in nrm], np.uint16)
    ko, kr = oracle.kdtree(pos, nids), reference.kdtree(pos, nids)
    assert np.array_equal(ko.perm, kr.perm) and np.array_equal(ko.nodes, kr.nodes)
    q = np.round(rng.normal(size=(400, 3)) * 0.3, 1)  # queries on the tie lattice
    qn = rng.normal(size=(400, 3))
    qn /= np.linalg.norm(qn, axis=1, keepdims=True)
    for args in ((q, qn, 100, 0.3, 0.87), (q, None, 32, 0.5, -1.0), (q, qn, 1, 1.0, 0.0)):
        a, b = ko.knn(*args), kr.knn(*args)
        for key in ("idx", "d2", "count"):
            assert np.array_equal(a[key], b[key])


def test_oracle_nearest_equals_reference(oracle, reference):
    rng = np.random.default_rng(78)
    pos = rng.uniform(0, 1, size=(8000, 3)).astype(np.float32)
    ko, kr = oracle.kdtree(pos), reference.kdtree(pos)
    q = rng.uniform(-0.1, 1.1, size=(2000, 3))
    for r in (0.01, 0.05, np.inf):
        assert np.array_equal(ko.nearest(q, None, r), kr.nearest(q, r))


def test_oracle_double_rays_match_reference(oracle, reference):
    """The oracle's traversal of double rays (the reference's own Ray type)
    equals the reference's Intersect / IntersectTest bit for bit."""
    import scene_fixtures as sf
    from skwarka_gb300 import scenes
    meshes = sf.unit_test_spheres()
    lo, hi = scenes.scene_bounds(meshes)
    rng = np.random.default_rng(36)
    n = 5000
    rays = np.zeros((n, 8))
    rays[:, :3] = rng.uniform(lo, hi, size=(n, 3))
    d = rng.uniform(0, 1, size=(n, 3))
    rays[:, 3:6] = d / np.sqrt((d * d).sum(1))[:, None]
    rays[:, 6] = rng.uniform(-10, 10, n)
    rays[:, 7] = rng.uniform(100, 10000, n)
    got, want = oracle.accel(meshes).intersect_d(rays), reference.accel(meshes).intersect_d(rays)
    assert np.array_equal(got["prim"], want["prim"]) and np.array_equal(got["tri"], want["tri"])
    assert np.array_equal(got["t"].view(np.uint64), want["t"].view(np.uint64))
    assert np.array_equal(oracle.accel(meshes).intersect_test_d(rays), reference.accel(meshes).intersect_test_d(rays))
