"""The product's host tree builder (skw_flat_tree_build in libskw.so) gives
the oracle's tree node for node (and so the reference's, which the oracle
is pinned to).  Runs on CPU: the build needs no GPU."""
import numpy as np
import pytest

import scene_fixtures as sf
from skwarka_gb300.accel import Primitive, TriangleMesh, build_flat_tree
from skwarka_gb300 import _lib, scenes


def preorder_export(nodes: np.ndarray):
    """Convert the flattened device tree to the oracle's export layout
    (pre-order; bbox, flags, children L/M/R, triangle range)."""
    order, pos, st = [], {}, [0]
    kids = {}
    while st:
        i = st.pop()
        pos[i] = len(order)
        order.append(i)
        b = int(nodes[i, 7])
        if b & 3:
            m, s, ks = (b >> 2) & 7, int(nodes[i, 6]), []
            for c in range(3):
                if m & (1 << c):
                    ks.append((c, s))
                    s += 1
            kids[i] = ks
            st.extend(k for _, k in reversed(ks))
    rng = {}
    for i in reversed(order):
        b = int(nodes[i, 7])
        if b & 3:
            rs = [rng[k] for _, k in kids[i]]
            rng[i] = (rs[0][0], rs[-1][1])
        else:
            rng[i] = (int(nodes[i, 6]), int(nodes[i, 6]) + (b >> 8))
    bbox = np.zeros((len(order), 6), np.float32)
    info = np.zeros((len(order), 8), np.int32)
    for j, i in enumerate(order):
        bbox[j] = nodes[i, :6].view(np.float32)
        b = int(nodes[i, 7])
        info[j, 0] = b & 3
        info[j, 1:4] = -1
        for c, k in kids.get(i, []):
            info[j, 1 + c] = pos[k]
        info[j, 4:6] = rng[i]
    return bbox, info


def _check_same(meshes, oracle):
    ft = build_flat_tree([Primitive(TriangleMesh(v, t)) for v, t in meshes])
    ob, oi, otp, oti = oracle.accel(meshes).export()
    pb, pi = preorder_export(ft["nodes"])
    assert np.array_equal(pb, ob)
    assert np.array_equal(pi, oi)
    assert np.array_equal(ft["tri_prim"], otp) and np.array_equal(ft["tri_index"], oti)
    return ft


def test_builder_matches_oracle_query_scene(oracle):
    ft = _check_same(sf.small_query_scene(), oracle)
    assert ft["max_depth"] < 200


def test_builder_matches_oracle_unit_test_spheres(oracle):
    _check_same(sf.unit_test_spheres(), oracle)


def test_builder_matches_oracle_flat_tiles(oracle):
    """Nodes of zero extent along an axis (the NaN split-bucket path)."""
    _check_same(sf.flat_tiles(200), oracle)


def test_builder_duplicate_triangles(oracle):
    """Identical triangles cannot be separated: middle splits until the mask
    is full (leaf rule 'three middle splits')."""
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    t = np.zeros((40, 3), np.int32)
    t[:] = [0, 1, 2]
    _check_same([(v, t)], oracle)


def test_builder_tiny_and_empty(oracle):
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    _check_same([(v, np.array([[0, 1, 2]], np.int32))], oracle)
    ft = build_flat_tree([])
    assert ft["nodes"].shape[0] == 1 and ft["tris"].shape[0] == 0


def test_builder_drops_illegal_triangles_like_trianglemesh(oracle):
    """TriangleMesh drops out-of-range or repeated-index triangles and
    renumbers the rest (TriangleMesh.cpp:176-182)."""
    v, t = scenes.sphere_mesh(2)
    t = t.copy()
    t[3] = [0, 0, 1]
    t[7] = [0, 1, 10_000]
    ft = build_flat_tree([Primitive(TriangleMesh(v.astype(np.float32), t))])
    assert ft["tris"].shape[0] == t.shape[0] - 2
    assert sorted(ft["tri_index"].tolist()) == list(range(t.shape[0] - 2))
    _check_same([(v.astype(np.float32), t)], oracle)


def test_builder_transform_matches_point_transform():
    """Primitive transforms are applied like Transform::operator()(Point3D_f)."""
    v, t = scenes.sphere_mesh(1)
    v = v.astype(np.float32)
    m = np.array([[2, 0, 0, 1.5], [0, 3, 0, -2], [0, 0, 0.5, 0.25], [0, 0, 0, 1]], np.float64)
    ft = build_flat_tree([Primitive(TriangleMesh(v, t), m)])
    vd = v.astype(np.float64)
    want = (vd @ m[:3, :3].T + m[:3, 3]).astype(np.float32)
    got = ft["tris"].reshape(-1, 3, 3)
    order = ft["tri_index"]
    assert np.array_equal(got, want[t[order]])


def test_builder_parallel_split_search_matches_oracle(oracle):
    """Nodes of 2^17 triangles or more fill their split buckets on several
    threads (slices of the triangles per axis, merged); the tree stays the
    oracle's node for node.  A 262,144-triangle displaced sphere + 20,000
    random triangles: the root and its largest children take that path."""
    import time
    meshes = scenes.ray_query_scene(sphere_subdivisions=8, n_random=20_000, seed=3)
    t0 = time.perf_counter()
    ft = _check_same(meshes, oracle)
    print(f"[tree] {ft['nodes'].shape[0]} nodes, product + oracle build {time.perf_counter() - t0:.2f} s")
