"""CUDA closest-hit / any-hit traversal against the oracle and the
reference's golden vectors, through the C ABI.

Acceptance: hit (primitive, triangle) ids agree on >= 99.99% of rays and the
hit distance to 1e-5 relative; any-hit answers agree on >= 99.99% of rays.
Disagreements, exact-arithmetic (fp64-decided) hits and near-ties are
printed (run pytest -s to see them)."""
from pathlib import Path

import numpy as np
import pytest

import scene_fixtures as sf
from skwarka_gb300 import scenes
from skwarka_gb300.accel import Primitive, TriangleAccelerator, TriangleMesh, unpack_hits

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
T_RTOL = 1e-5
MIN_AGREE = 0.9999


def _accel(meshes):
    return TriangleAccelerator([Primitive(TriangleMesh(v, t)) for v, t in meshes])


def _gpu_hits(acc, rays):
    import torch
    r = torch.from_numpy(np.ascontiguousarray(rays, np.float32)).cuda()
    h = acc.intersect(r)
    torch.cuda.synchronize()
    return unpack_hits(h)


def _gpu_occ(acc, rays):
    import torch
    r = torch.from_numpy(np.ascontiguousarray(rays, np.float32)).cuda()
    o = acc.intersect_test(r)
    torch.cuda.synchronize()
    return o.cpu().numpy()


def compare_hits(gpu, ref, label):
    """Returns the agreement fraction; asserts t within T_RTOL where ids agree."""
    same = (gpu["prim"] == ref["prim"]) & (gpu["tri"] == ref["tri"])
    frac = same.mean()
    hit = same & (ref["prim"] >= 0)
    rel = np.abs(gpu["t"][hit].astype(np.float64) - ref["t"][hit]) / np.maximum(np.abs(ref["t"][hit]), 1e-30)
    n_fp64 = int(((gpu["flags"] & 1) != 0).sum())
    n_tie = int(((gpu["flags"] & 2) != 0).sum())
    bad = np.nonzero(~same)[0]
    print(f"[{label}] rays={len(same)} agree={frac:.6f} mismatches={len(bad)} fp64-decided={n_fp64} "
          f"near-ties={n_tie} max t rel err={rel.max() if rel.size else 0:.3g}")
    for i in bad[:10]:
        print(f"   ray {i}: gpu ({gpu['prim'][i]},{gpu['tri'][i]},t={gpu['t'][i]:.9g},flags={gpu['flags'][i]}) "
              f"ref ({ref['prim'][i]},{ref['tri'][i]},t={ref['t'][i]:.9g})")
    assert rel.size == 0 or rel.max() <= T_RTOL
    # a miss on one side must be a miss on the other wherever ids agree
    assert np.all(np.isinf(gpu["t"][same & (ref["prim"] < 0)]))
    return frac


def test_golden_vectors_on_gpu(gpu):
    g = np.load(GOLD / "accel_small.npz")
    meshes, i = [], 0
    while f"mesh{i}_vertices" in g:
        meshes.append((g[f"mesh{i}_vertices"], g[f"mesh{i}_triangles"]))
        i += 1
    acc = _accel(meshes)
    h = _gpu_hits(acc, g["rays"])
    ref = {"prim": g["hit_prim"], "tri": g["hit_tri"], "t": g["hit_t"]}
    assert compare_hits(h, ref, "golden") >= MIN_AGREE
    occ = _gpu_occ(acc, g["shadow_rays"])
    assert (occ == g["occluded"]).mean() >= MIN_AGREE


def test_unit_test_spheres_against_oracle(gpu, oracle):
    meshes = sf.unit_test_spheres()
    rays = sf.unit_test_rays(meshes, 5000)
    acc = _accel(meshes)
    ref = oracle.accel(meshes).intersect(rays)
    assert compare_hits(_gpu_hits(acc, rays), ref, "unit-test spheres") >= MIN_AGREE


def test_query_scene_against_oracle(gpu, oracle):
    meshes = sf.small_query_scene()
    lo, hi = scenes.scene_bounds(meshes)
    rays = scenes.uniform_rays(200_000, lo, hi, seed=51)
    srays = scenes.uniform_rays(200_000, lo, hi, seed=52, tmax_range=(0.0, 2.0))
    acc = _accel(meshes)
    oa = oracle.accel(meshes)
    assert compare_hits(_gpu_hits(acc, rays), oa.intersect(rays), "query scene") >= MIN_AGREE
    og, oo = _gpu_occ(acc, srays), oa.intersect_test(srays)
    frac = (og == oo).mean()
    print(f"[query scene any-hit] agree={frac:.6f} mismatches={(og != oo).sum()}")
    assert frac >= MIN_AGREE


@pytest.mark.parametrize("n", [50_000, 4_500_001, 9_437_185])
def test_host_api_equals_device_api(gpu, n):
    """The host-buffer entry points (copies in, query, copies out; above
    2^21 rays in chunks over two streams that reuse one chunk buffer each)
    equal the device ones bit for bit, including a ragged last chunk and
    more than four chunks."""
    meshes = sf.small_query_scene()
    lo, hi = scenes.scene_bounds(meshes)
    rays = scenes.uniform_rays(n, lo, hi, seed=53)
    acc = _accel(meshes)
    hd = _gpu_hits(acc, rays)
    hh = acc.intersect(rays)  # numpy -> host-buffer entry point
    for k in ("prim", "tri", "flags"):
        assert np.array_equal(hd[k], hh[k])
    assert np.array_equal(hd["t"].view(np.uint32), hh["t"].view(np.uint32))
    srays = rays.copy()
    srays[:, 7] = 1.0
    assert np.array_equal(_gpu_occ(acc, srays), acc.intersect_test(srays))


def test_edge_cases(gpu, oracle):
    # empty accelerator: everything misses
    acc0 = TriangleAccelerator([])
    rays = scenes.uniform_rays(1000, [-1, -1, -1], [1, 1, 1], seed=54)
    h = _gpu_hits(acc0, rays)
    assert np.all(h["prim"] == -1) and np.all(np.isinf(h["t"]))
    assert not _gpu_occ(acc0, rays).any()
    # zero rays
    import torch
    z = torch.zeros((0, 8), dtype=torch.float32, device="cuda")
    assert acc0.intersect(z).shape == (0, 4)
    # axis-aligned rays (zero direction components -> infinite slab
    # reciprocals), rays with tmax = 0 and rays starting on the surface
    meshes = sf.flat_tiles(300) + sf.unit_test_spheres()[:1]
    acc = _accel(meshes)
    oa = oracle.accel(meshes)
    rng = np.random.default_rng(55)
    n = 4000
    r = np.zeros((n, 8), np.float32)
    r[:, 0:2] = rng.uniform(0, 1, (n, 2))
    r[:, 2] = rng.choice([-1.0, 2.0], n)
    r[:, 5] = np.where(r[:, 2] < 0, 1.0, -1.0)
    r[:, 7] = np.where(rng.uniform(size=n) < 0.1, 0.0, np.inf)
    r[:200, 2] = 0.5  # origin in the tile plane
    assert compare_hits(_gpu_hits(acc, r), oa.intersect(r), "axis-aligned") >= MIN_AGREE
    assert (_gpu_occ(acc, r) == oa.intersect_test(r)).mean() >= MIN_AGREE
    # single-triangle scene, ray through a vertex and along an edge
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    acc1 = _accel([(v, np.array([[0, 1, 2]], np.int32))])
    oa1 = oracle.accel([(v, np.array([[0, 1, 2]], np.int32))])
    r1 = np.array([[0, 0, 1, 0, 0, -1, 0, np.inf], [0.5, 0, 1, 0, 0, -1, 0, np.inf],
                   [0.5, 0.5, 1, 0, 0, -1, 0, np.inf], [0.25, 0.25, 1, 0, 0, -1, 0, 0.5]], np.float32)
    assert compare_hits(_gpu_hits(acc1, r1), oa1.intersect(r1), "vertex/edge") == 1.0


@pytest.mark.parametrize("which", ["closest", "any"])
def test_full_size_scene_properties(gpu, oracle, which):
    """1,048,576-triangle displaced sphere + 50,000 random triangles, 4M rays:
    oracle agreement on a 100k subsample, plus size-independent properties on
    all rays -- a closest hit at t means no hit in [tmin, t*(1-1e-5)] and a hit
    in [tmin, t*(1+1e-5)]."""
    import torch
    meshes = scenes.ray_query_scene(9, 50_000, seed=3)
    lo, hi = scenes.scene_bounds(meshes)
    acc = _accel(meshes)
    if which == "closest":
        rays = scenes.uniform_rays(4_000_000, lo, hi, seed=7)
        h = _gpu_hits(acc, rays)
        sub = slice(0, 100_000)
        ref = oracle.accel(meshes).intersect(rays[sub])
        assert compare_hits({k: v[sub] for k, v in h.items()}, ref, "full scene subsample") >= MIN_AGREE
        hit = h["prim"] >= 0
        before = rays[hit].copy()
        before[:, 7] = h["t"][hit] * (1 - 1e-5)
        after = rays[hit].copy()
        after[:, 7] = h["t"][hit] * (1 + 1e-5)
        ob, oa_ = _gpu_occ(acc, before), _gpu_occ(acc, after)
        print(f"[full scene] hits={hit.sum()} occluded-before={ob.mean():.6f} occluded-after={oa_.mean():.6f}")
        assert ob.mean() <= 1 - MIN_AGREE and oa_.mean() >= MIN_AGREE
    else:
        srays = scenes.uniform_rays(4_000_000, lo, hi, seed=8, tmax_range=(0.0, 2.0))
        occ = _gpu_occ(acc, srays)
        ref = oracle.accel(meshes).intersect_test(srays[:100_000])
        frac = (occ[:100_000] == ref).mean()
        print(f"[full scene any-hit] agree={frac:.6f} occluded={occ.mean():.4f}")
        assert frac >= MIN_AGREE
