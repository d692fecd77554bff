"""The allocation-free k-NN entry point (skw_knn_noalloc) gives the same
results as skw_knn.

skw_knn_noalloc serves callers that cannot allocate device memory while
they query -- a renderer running inside a device-memory budget reserved up
front, or a host callback that must not block on cudaMalloc / cudaFree -- by
keeping its heaps in a static device array.  The test calls both entry
points through the C ABI on the same tree and queries, several times in a
row with different sizes (a call must not be disturbed by what the previous
one left in the shared array), for k in {0, 1, 32, 100, 150, 200} (each of
skw_knn's kernels), and compares counts, indices and squared distances
exactly (the tolerance of every k-NN test here: bit-exact); the k = 100 call
is also compared with the oracle.  It
also checks that a batch larger than the array is refused with an error.
This file is named to run last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_knn_noalloc_matches_knn_twice(gpu):
    import torch

    from skwarka_gb300 import _lib
    from skwarka_gb300.kdtree import PhotonKDTree, compress_directions

    lib = _lib.load()
    rng = np.random.default_rng(2024)
    n = 150_000
    pos = rng.uniform(0, 1, size=(n, 3)).astype(np.float32)
    pos[:3000] = np.round(pos[:3000], 2)
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    tree = PhotonKDTree(pos, compress_directions(nrm))
    s = torch.cuda.current_stream().cuda_stream

    def run(entry, q, qn, k, r, cos_t):
        nq = q.shape[0]
        idx = torch.full((nq, max(k, 1)), -7, dtype=torch.int32, device="cuda")[:, :k]
        d2 = torch.full((nq, max(k, 1)), -7.0, dtype=torch.float64, device="cuda")[:, :k]
        cnt = torch.full((nq,), -7, dtype=torch.int32, device="cuda")
        rc = entry(tree.handle, q.data_ptr(), qn.data_ptr(), nq, k, r, cos_t, idx.data_ptr(), d2.data_ptr(),
                   cnt.data_ptr(), s)
        assert rc == 0, lib.skw_last_error(tree.ctx.handle)
        torch.cuda.synchronize()
        return idx.cpu().numpy(), d2.cpu().numpy(), cnt.cpu().numpy()

    # skw_knn serves k <= 32 and k <= 128 with per-thread heaps and skips the
    # heap for k = 0; the allocation-free entry point always uses the scratch
    # heaps, so every branch of skw_knn is compared, plus the oracle once.
    cases = [(4000, 200, 0.08, 0.5), (2500, 150, 0.05, -1.0), (3000, 1, 0.1, 0.5), (3000, 32, 0.05, 0.87),
             (3000, 100, 0.06, 0.5), (3000, 0, 0.05, 0.5)]
    for call, (nq, k, r, cos_t) in enumerate(cases):
        q_np = rng.uniform(0, 1, size=(nq, 3))
        qn_np = rng.normal(size=(nq, 3))
        qn_np /= np.linalg.norm(qn_np, axis=1, keepdims=True)
        q, qn = torch.from_numpy(q_np).cuda(), torch.from_numpy(qn_np).cuda()
        a = run(lib.skw_knn, q, qn, k, r, cos_t)
        b = run(lib.skw_knn_noalloc, q, qn, k, r, cos_t)
        for x, y in zip(a, b):
            assert np.array_equal(x, y), f"call {call} (k={k}): no-allocation results differ"
        if k > 0:
            assert a[2].max() > 0
        else:
            assert (b[2] == 0).all()
        if k == 100:
            from oracle.api import Oracle
            want = Oracle().kdtree(pos, compress_directions(nrm)).knn(q_np, qn_np, k, r, cos_t)
            assert np.array_equal(b[2], want["count"])
            assert np.array_equal(b[0], want["idx"])
            assert np.array_equal(b[1].view(np.uint64), want["d2"].view(np.uint64))

    # A batch beyond the static array is refused, not truncated.
    nq, k = 10_000, 200
    q = torch.zeros((nq, 3), dtype=torch.float64, device="cuda")
    out_i = torch.empty((nq, k), dtype=torch.int32, device="cuda")
    out_d = torch.empty((nq, k), dtype=torch.float64, device="cuda")
    out_c = torch.empty((nq,), dtype=torch.int32, device="cuda")
    rc = lib.skw_knn_noalloc(tree.handle, q.data_ptr(), None, nq, k, 0.1, -1.0, out_i.data_ptr(), out_d.data_ptr(),
                             out_c.data_ptr(), s)
    assert rc == 1 and b"capacity" in lib.skw_last_error(tree.ctx.handle)
