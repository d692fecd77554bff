"""CUDA photon k-NN against the reference's golden vectors and the oracle,
through the C ABI.  Acceptance: index sets (and, since the heap routines
match, their order and squared distances) bit-exact."""
from pathlib import Path

import numpy as np
import pytest

from skwarka_gb300.kdtree import PhotonKDTree, compress_directions

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()


def _same(got, want, label):
    got = {k: (v.cpu().numpy() if hasattr(v, "cpu") else v) for k, v in got.items()}
    cnt_ok = np.array_equal(got["count"], want["count"])
    idx_ok = np.array_equal(got["idx"], want["idx"])
    d2_ok = np.array_equal(got["d2"], want["d2"])
    sets_ok = all(set(got["idx"][i, :c]) == set(want["idx"][i, :c]) for i, c in enumerate(want["count"]))
    print(f"[{label}] queries={len(want['count'])} counts={cnt_ok} sets={sets_ok} order={idx_ok} d2={d2_ok} "
          f"mean found={want['count'].mean():.1f}")
    assert cnt_ok and sets_ok and idx_ok and d2_ok


def test_golden_knn_on_gpu(gpu):
    g = np.load(GOLD / "knn_small.npz")
    t = PhotonKDTree(g["pos"], g["normal_ids"])
    assert np.array_equal(t.perm, g["perm"])
    r = t.get_nearest_points(_dev(g["q"]), _dev(g["qn"]), 20, 0.15, 0.5)
    _same(r, {"idx": g["filt_idx"], "d2": g["filt_d2"], "count": g["filt_count"]}, "golden filtered")
    r = t.get_nearest_points(_dev(g["q"]), None, 20, 0.2, -1.0)
    _same(r, {"idx": g["all_idx"], "d2": g["all_d2"], "count": g["all_count"]}, "golden unfiltered")


@pytest.mark.parametrize("k,r,cos_t", [(100, 0.05, 0.87), (32, 0.1, 0.87), (1, 1.0, -1.0), (100, np.inf, -1.0),
                                       (500, 0.2, 0.5)])
def test_knn_against_oracle(gpu, oracle, k, r, cos_t):
    rng = np.random.default_rng(k + 7)
    n = 60_000
    pos = rng.uniform(0, 1, size=(n, 3)).astype(np.float32)
    pos[:2000] = np.round(pos[:2000], 2)  # coordinates on a lattice: exact distance ties
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nids = compress_directions(nrm) if cos_t >= 0 else None
    t = PhotonKDTree(pos, nids)
    ko = oracle.kdtree(pos, nids)
    assert np.array_equal(t.perm, ko.perm)
    nq = 4000
    q = rng.uniform(0, 1, size=(nq, 3))
    q[:500] = np.round(q[:500], 2)
    qn = rng.normal(size=(nq, 3))
    qn /= np.linalg.norm(qn, axis=1, keepdims=True)
    got = t.get_nearest_points(_dev(q), _dev(qn) if cos_t >= 0 else None, k, r, cos_t)
    _same(got, ko.knn(q, qn if cos_t >= 0 else None, k, r, cos_t), f"k={k} r={r} cos={cos_t}")


def test_knn_host_api_and_nearest(gpu, oracle):
    rng = np.random.default_rng(12)
    pos = rng.uniform(0, 1, size=(30_000, 3)).astype(np.float32)
    nrm = rng.normal(size=(30_000, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nids = compress_directions(nrm)
    t = PhotonKDTree(pos, nids)
    ko = oracle.kdtree(pos, nids)
    q = rng.uniform(0, 1, size=(3000, 3))
    qn = rng.normal(size=(3000, 3))
    qn /= np.linalg.norm(qn, axis=1, keepdims=True)
    _same(t.get_nearest_points(q, qn, 50, 0.08, 0.87), ko.knn(q, qn, 50, 0.08, 0.87), "host api")
    import torch
    for cos_t in (-1.0, 0.87):
        got = t.get_nearest_point(_dev(q), _dev(qn), 0.05, cos_t).cpu().numpy()
        assert np.array_equal(got, ko.nearest(q, qn, 0.05, cos_t))
    # empty tree and k = 0
    t0 = PhotonKDTree(np.zeros((0, 3), np.float32))
    r0 = t0.get_nearest_points(q[:10], None, 5, 1.0)
    assert np.all(r0["count"] == 0) and np.all(r0["idx"] == -1)
    rk = t.get_nearest_points(q[:10], None, 0, 1.0)
    assert np.all(rk["count"] == 0)


def test_photon_map_scale(gpu, oracle):
    """2M photons, k = 100 within 0.05 with the normal filter (cos 0.87), 1M
    queries: bit-exact against the oracle on a 50k subsample; properties on
    all queries (count <= k, every distance within the radius, full heaps are
    max-heaps)."""
    import torch
    rng = np.random.default_rng(13)
    n = 2_000_000
    # photons on the unit sphere surface with their outward normals
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    pos = v.astype(np.float32)
    nids = compress_directions(v[:1]) if False else None
    from skwarka_gb300.kdtree import direction_table
    t = PhotonKDTree(pos, None)
    nq = 1_000_000
    qv = rng.normal(size=(nq, 3))
    qv /= np.linalg.norm(qv, axis=1, keepdims=True)
    got = t.get_nearest_points(_dev(qv), _dev(qv), 100, 0.05, -1.0)
    torch.cuda.synchronize()
    cnt = got["count"].cpu().numpy()
    d2 = got["d2"].cpu().numpy()
    assert cnt.max() <= 100 and np.all(d2[cnt == 100] < 0.05 ** 2 + 1e-18)
    full = np.nonzero(cnt == 100)[0][:2000]
    for i in full:
        h = d2[i]
        for j in range(1, 100):
            assert h[(j - 1) // 2] >= h[j]
    ko = oracle.kdtree(pos, None)
    sub = slice(0, 50_000)
    want = ko.knn(qv[sub], None, 100, 0.05, -1.0)
    _same({k: v[sub] for k, v in got.items()}, want, "2M photons subsample")
