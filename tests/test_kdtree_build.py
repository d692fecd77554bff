"""Photon kd-tree host build and direction codec of the product library
against the oracle and the reference golden vectors (CPU only)."""
from pathlib import Path

import numpy as np

from skwarka_gb300 import kdtree

GOLD = Path(__file__).resolve().parent / "golden"


def test_build_matches_golden():
    g = np.load(GOLD / "knn_small.npz")
    perm, nodes = kdtree.build_host(g["pos"])
    assert np.array_equal(perm, g["perm"]) and np.array_equal(nodes, g["nodes"])


def test_build_matches_oracle_with_ties(oracle):
    rng = np.random.default_rng(8)
    for pos in (rng.uniform(0, 1, (20_000, 3)).astype(np.float32),
                np.round(rng.normal(size=(5000, 3)), 1).astype(np.float32),  # many equal coordinates
                np.zeros((7, 3), np.float32), rng.uniform(0, 1, (1, 3)).astype(np.float32)):
        perm, nodes = kdtree.build_host(pos)
        ko = oracle.kdtree(pos)
        assert np.array_equal(perm, ko.perm) and np.array_equal(nodes, ko.nodes)


def test_build_threads_do_not_change_result():
    pos = np.random.default_rng(9).uniform(0, 1, (300_000, 3)).astype(np.float32)
    a = kdtree.build_host(pos, threads=1)
    b = kdtree.build_host(pos, threads=0)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_direction_table_and_codec_match_golden(oracle):
    g = np.load(GOLD / "compressed_direction.npz")
    tab = kdtree.direction_table()
    assert np.array_equal(tab[g["ids"]], g["vectors"])
    assert np.array_equal(tab, oracle.direction_table())
    rng = np.random.default_rng(10)
    v = rng.normal(size=(500, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    ids = kdtree.compress_directions(v)
    # decoding an encoded direction stays within the codec's quantisation
    assert np.all((tab[ids] * v).sum(1) > 0.99)
