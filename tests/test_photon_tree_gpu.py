"""The photon kd-tree built on the GPU (level by level over per-axis sorted
lists) against the host build, which restates KDTree::_Build
(Raytracer/Core/KDTree.h:428-473) with the reference's own std::nth_element:
node for node equal wherever no node's median ties on its split axis, and
the tie reported where one does (there the host build is used)."""
import numpy as np
import pytest

from skwarka_gb300.kdtree import build_device, build_host

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
    """Random float coordinates: equal trees whenever the device build reports
    no median tie (with a million points some median usually ties: the
    chance that two neighbours in a sorted axis share a float grows with the
    points' density)."""
    for n in (20_000, 200_000, 1_000_000):
        pos = np.random.default_rng(n + 1).uniform(-1.0, 1.0, size=(n, 3)).astype(np.float32)
        hp, hn = build_host(pos)
        dp, dn, tie = build_device(pos)
        print(f"[device tree] n {n}: median tie {tie}")
        if not tie:
            assert np.array_equal(hp, dp) and np.array_equal(hn, dn)


def test_median_ties_are_reported(gpu):
    """Points on a lattice tie at many medians: the device build says so
    (and the callers build those trees on the host)."""
    g = np.arange(40, dtype=np.float32)
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    _, _, tie = build_device(pos)
    assert tie


def test_photon_maps_built_on_the_gpu(gpu):
    """The photon maps of the 1M-triangle scene (no axis-aligned surfaces):
    a map's tree comes from the GPU builder exactly when that build reports
    no median tie, and then equals the host's."""
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
        assert bool(info["trees_on_gpu"] & bit) == (not tie and len(pos) >= 16384)
        if not tie:
            assert np.array_equal(hp, dp)
