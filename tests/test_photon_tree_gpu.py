"""The photon kd-tree built on the GPU (level by level over per-axis sorted
lists) against the host build, which restates KDTree::_Build
(Raytracer/Core/KDTree.h:428-473) with the reference's own std::nth_element:
node for node equal.  Where a node's median ties on its split axis the
reference's subtree is std::nth_element's choice among the equal points:
the device build counts those nodes and remakes their subtrees, and the
paths to them, on the host (above 256 of them, the whole tree)."""
import numpy as np
import pytest

from skwarka_gb300.kdtree import PhotonKDTree, build_device, build_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [2, 3, 17, 1000, 65_537, 1_000_000])
def test_device_tree_equals_host_tree(gpu, n):
    """Coordinates distinct on every axis (so no median can tie): the device
    tree is the host's node for node."""
    rng = np.random.default_rng(n)
    pos = np.stack([rng.permutation(n) for _ in range(3)], -1).astype(np.float32) / n
    pos[:, 2] *= 0.3  # a flatter box: the axis choice varies by node
    hp, hn = build_host(pos)
    dp, dn, tie = build_device(pos)
    assert not tie
    assert np.array_equal(hp, dp) and np.array_equal(hn, dn)


def test_device_tree_on_random_floats(gpu):
    """Random float coordinates: equal trees (with a million points some
    median usually ties: the chance that two neighbours in a sorted axis
    share a float grows with the points' density)."""
    for n in (20_000, 200_000, 1_000_000):
        pos = np.random.default_rng(n + 1).uniform(-1.0, 1.0, size=(n, 3)).astype(np.float32)
        hp, hn = build_host(pos)
        dp, dn, tie = build_device(pos)
        print(f"[device tree] n {n}: median ties {tie}")
        assert np.array_equal(hp, dp) and np.array_equal(hn, dn)


@pytest.mark.parametrize("n, n_dup", [(60_000, 20_000), (200_000, 40_000), (1_000_000, 150_000)])
def test_tied_medians_repaired(gpu, n, n_dup):
    """Some points share a coordinate with another on one axis, so a few
    medians tie: the GPU tree repaired on the host is the reference's, both
    through the device builder and in a PhotonKDTree (whose lookups index
    the tree order)."""
    rng = np.random.default_rng(n)
    pos = rng.uniform(-1.0, 1.0, size=(n, 3)).astype(np.float32)
    src, dst = rng.choice(n, n_dup, replace=False), rng.choice(n, n_dup, replace=False)
    ax = rng.integers(0, 3, n_dup)
    pos[dst, ax] = pos[src, ax]
    hp, hn = build_host(pos)
    dp, dn, tie = build_device(pos)
    print(f"[device tree] n {n}: median ties {tie}")
    assert 0 < tie <= 256
    assert np.array_equal(hp, dp) and np.array_equal(hn, dn)
    assert np.array_equal(PhotonKDTree(pos).perm, hp)


def test_median_ties_past_the_repair(gpu):
    """Points on a lattice tie at thousands of medians: the device build
    counts them and gives the host's tree."""
    g = np.arange(40, dtype=np.float32)
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    hp, hn = build_host(pos)
    dp, dn, tie = build_device(pos)
    assert tie > 256
    assert np.array_equal(hp, dp) and np.array_equal(hn, dn)
    assert np.array_equal(PhotonKDTree(pos).perm, hp)


def test_photon_maps_built_on_the_gpu(gpu):
    """The photon maps of the 1M-triangle scene (no axis-aligned surfaces):
    a map's tree comes from the GPU builder (repaired where medians tie)
    exactly when it has 16,384 photons or more and at most 256 tied
    medians, and equals the host's."""
    from skwarka_gb300 import scenes
    from skwarka_gb300.photon import PhotonMap
    from skwarka_gb300.render import RenderScene
    prims, mats, lights, _ = scenes.photon_scene(6, 2000)
    sc = RenderScene(prims, mats, lights)
    pm = PhotonMap.shoot(sc, 400_000, max_bounces=8, rr_probability=0.7, seed=4)
    info = pm.info()
    print(f"[photon trees] direct {info['n_direct']} indirect {info['n_indirect']} "
          f"trees on the GPU (bits) {info['trees_on_gpu']}")
    # a map's tree comes from the GPU exactly when the GPU build is exact
    for bit, name in ((2, "direct"), (4, "indirect")):
        pos = np.ascontiguousarray(pm.export(name)["position"])
        hp, _ = build_host(pos)
        dp, _, tie = build_device(pos)
        assert bool(info["trees_on_gpu"] & bit) == (tie <= 256 and len(pos) >= 16384)
        assert np.array_equal(hp, dp)
