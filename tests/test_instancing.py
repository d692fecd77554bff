"""Instancing (meshes shared by several primitives; TriangleAccelerator.cpp:
54-102 build, :213-233 traversal) against the reference's own accelerator
built over the same shared meshes and transforms.

CPU: the product's tree (the top tree's nodes, the triangle arrays with the
shared meshes' mesh-space triangles first, the instances' order,
primitives and world-to-mesh matrices) equals the reference's.
GPU (test_instancing_gpu.py): hits equal the reference's Intersect."""
import numpy as np
import pytest

import instancing_fixtures as inf
from skwarka_gb300.accel import Primitive, TriangleMesh, build_flat_tree


def primitives(meshes, mesh_of, xforms):
    tm = [TriangleMesh(v, t) for v, t in meshes]
    return [Primitive(tm[m], None if x is None else np.asarray(x, np.float64)) for m, x in zip(mesh_of, xforms)]


def ref_accel(reference, meshes, mesh_of, xforms):
    xf = np.stack([np.eye(4) if x is None else np.asarray(x, np.float64) for x in xforms])
    return reference.accel(meshes, mesh_of=mesh_of, xforms=xf)


def top_tree_export(ft):
    """The top tree (root 0) in pre-order: bbox, flags, children L/M/R
    (pre-order indices), triangle range and instance range (empty ranges
    as (0, 0))."""
    nodes, ext = ft["nodes"], ft["leaf_ranges"]
    order, pos, kids, st = [], {}, {}, [0]
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
    bbox = np.zeros((len(order), 6), np.float32)
    info = np.zeros((len(order), 8), np.int32)
    for j, i in enumerate(order):
        bbox[j] = nodes[i, :6].view(np.float32)
        b = int(nodes[i, 7])
        info[j, 0] = b & 3
        info[j, 1:4] = -1
        for c, k in kids.get(i, []):
            info[j, 1 + c] = pos[k]
        if not (b & 3):
            if b & 0x80:
                tf, tc, i0, ic = ext[i]
            else:
                tf, tc, i0, ic = int(nodes[i, 6]), b >> 8, 0, 0
            info[j, 4:8] = [tf, tf + tc, i0, i0 + ic]
    return bbox, info


def _canon(info):
    """Leaves only; empty ranges as (0, 0)."""
    out = info.copy()
    leaf = out[:, 0] == 0
    out[~leaf, 4:8] = 0
    for a, b in ((4, 5), (6, 7)):
        e = out[:, a] == out[:, b]
        out[e, a] = out[e, b] = 0
    return out


def address_order(ra, meshes, mesh_of, xforms):
    """The scene with its meshes renumbered and its primitives reordered in
    the reference's address order of meshes (it keys meshes by address:
    shared meshes' subtrees and unshared meshes' triangles follow that
    order), and the map from new primitive index to the original."""
    rank = ra.mesh_rank(len(meshes))
    first_use = list(dict.fromkeys(mesh_of))
    rank_of = {m: rank[i] for i, m in enumerate(first_use)}
    perm = np.array(sorted(range(len(mesh_of)), key=lambda p: (rank_of[mesh_of[p]], p)))
    new_id = {m: int(rank_of[m]) for m in first_use}
    m2 = [None] * len(first_use)
    for m in first_use:
        m2[new_id[m]] = meshes[m]
    return m2, [new_id[mesh_of[p]] for p in perm], [xforms[p] for p in perm], perm


@pytest.mark.parametrize("which", ["mixed", "tetrahedra"])
def test_instanced_tree_matches_reference(reference, which):
    meshes, mesh_of, xforms = inf.instanced_scene() if which == "mixed" else inf.tetra_instancing_test(2_000)
    ra = ref_accel(reference, meshes, mesh_of, xforms)
    m2, o2, x2, perm = address_order(ra, meshes, mesh_of, xforms)
    ft = build_flat_tree(primitives(m2, o2, x2))
    ft["tri_prim"] = np.where(ft["tri_prim"] >= 0, perm[np.maximum(ft["tri_prim"], 0)], -1)
    ft["inst_prim"] = perm[ft["inst_prim"]]
    rb, ri, rtp, rti = ra.export()
    pb, pi = top_tree_export(ft)
    n_inst = len(ft["inst_prim"])
    print(f"[instancing {which}] {pb.shape[0]} top-tree nodes, {len(ft['subtree_roots'])} shared meshes, "
          f"{n_inst} instances, {ft['tris'].shape[0]} triangle slots")
    assert n_inst > 0
    assert np.array_equal(pb, rb)
    assert np.array_equal(_canon(pi), _canon(ri))
    assert np.array_equal(ft["tri_prim"], rtp) and np.array_equal(ft["tri_index"], rti)
    p, m, c = ra.instances()
    assert np.array_equal(ft["inst_prim"], p)
    assert np.array_equal(ft["inst_world_to_mesh"].view(np.uint64), m.view(np.uint64))


def test_inverse_matches_reference_matrix4x4(reference):
    """The world-to-mesh matrices (Matrix4x4::Inverted restated) equal the
    reference's for many random transforms, bit for bit."""
    meshes, mesh_of, xforms = inf.tetra_instancing_test(500, seed=63)
    ft = build_flat_tree(primitives(meshes, mesh_of, xforms))
    p, m, _ = ref_accel(reference, meshes, mesh_of, xforms).instances()
    order = np.argsort(p)
    mine = ft["inst_world_to_mesh"][np.argsort(ft["inst_prim"])]
    assert np.array_equal(mine.view(np.uint64), m[order].view(np.uint64))
