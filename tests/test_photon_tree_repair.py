"""The host half of the GPU photon-tree build (no GPU): a tree equal to the
reference's except below nodes whose median ties on the split axis is
remade there -- the paths from the root to those nodes and their whole
subtrees, from the input order, as KDTree::_Build
(Raytracer/Core/KDTree.h:428-473) makes them -- and every other subtree is
left as it is.  The reference's tree is the host build (the same
std::nth_element calls)."""
import numpy as np
import pytest

from skwarka_gb300.kdtree import build_host, repair_host


def _tie_nodes(pos, perm, words):
    """Tree positions of the nodes whose median ties on their split axis,
    with each node's range [b, e) (node b at the range's start, left child
    [b + 1, split + 1), right [split + 1, e), split = (b + e) // 2)."""
    p = pos[perm]
    n = len(p)
    ties, ranges = [], {}
    stack = [(0, n)]
    while stack:
        b, e = stack.pop()
        ranges[b] = e
        if e - b <= 1:
            continue
        ax = int(words[b, 1] & 3)
        if np.any(p[b + 1:e, ax] == p[b, ax]):
            ties.append(b)
        s = (b + e) // 2
        stack.append((b + 1, s + 1))
        if s + 1 < e:
            stack.append((s + 1, e))
    return sorted(ties), ranges


def _paths(ties, ranges):
    """Nodes strictly above some tie node (their ranges contain one)."""
    out = set()
    for b, e in ranges.items():
        if any(b < t < e for t in ties):
            out.add(b)
    return out


def _points_with_ties(n, n_dup, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-1.0, 1.0, size=(n, 3)).astype(np.float32)
    # copy one coordinate of some points onto others: equal keys on that axis
    src, dst = rng.choice(n, n_dup, replace=False), rng.choice(n, n_dup, replace=False)
    ax = rng.integers(0, 3, n_dup)
    pos[dst, ax] = pos[src, ax]
    return pos


@pytest.mark.parametrize("n, n_dup, seed", [(5_000, 400, 1), (60_000, 20_000, 2), (200_000, 40_000, 3)])
def test_repair_remakes_tie_subtrees_and_paths(n, n_dup, seed):
    pos = _points_with_ties(n, n_dup, seed)
    hp, hn = build_host(pos)
    ties, ranges = _tie_nodes(pos, hp, hn)
    assert ties, "the case must have tied medians"
    # a tree that differs from the reference's below the tie nodes (as the
    # GPU's may): their subtrees shuffled
    rng = np.random.default_rng(seed + 100)
    bp, bn = hp.copy(), hn.copy()
    for t in ties:
        e = ranges[t]
        sh = rng.permutation(np.arange(t, e))
        bp[t:e] = hp[sh]
        bn[t:e] = hn[sh]
    assert not np.array_equal(bp, hp)
    assert _paths(ties, ranges), "some node lies above a tie node"
    rp, rn = repair_host(pos, ties, bp, bn)
    assert np.array_equal(rp, hp) and np.array_equal(rn, hn)
    print(f"[tree repair] n {n}: {len(ties)} tie nodes, largest subtree "
          f"{max(ranges[t] - t for t in ties)}")


def test_repair_without_ties_changes_nothing():
    pos = np.random.default_rng(7).uniform(size=(3000, 3)).astype(np.float32)
    hp, hn = build_host(pos)
    bp, bn = hp.copy(), hn.copy()
    leaves = np.nonzero((hn[:, 1] & 3) == 3)[0]
    bp[leaves[0]], bp[leaves[-1]] = hp[leaves[-1]], hp[leaves[0]]  # under no tie node: left as it is
    rp, rn = repair_host(pos, [], bp, bn)
    assert np.array_equal(rp, bp) and np.array_equal(rn, bn)


def test_repair_of_the_root_is_the_host_build():
    """A tie at the root: the whole tree is remade."""
    pos = _points_with_ties(2_000, 300, 9)
    hp, hn = build_host(pos)
    rp, rn = repair_host(pos, [0], np.roll(hp, 1), np.zeros_like(hn))
    assert np.array_equal(rp, hp) and np.array_equal(rn, hn)
