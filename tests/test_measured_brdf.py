"""Measured (MERL-layout) BRDF: the product's host restatement
(skw_merl_*, skwarka_gb300/csrc/merl.cpp) against the reference's
MERLMeasuredData / MERLMeasured built from its sources -- the converted
half table and the sampling segmentations bit for bit, and Evaluate, PDF
and Sample bit for bit in double on random directions (grazing ones
included).  The table is the seeded synthetic one of scenes.merl_table."""
import numpy as np
import pytest

from skwarka_gb300 import scenes
from skwarka_gb300.render import MeasuredBRDF


@pytest.fixture(scope="module")
def pair(reference):
    data = scenes.merl_table()
    return MeasuredBRDF(data, device=False), reference.merl(data)


def _dirs(rng, n, grazing=False):
    if grazing:
        th = np.radians(rng.uniform(85.0, 89.99, n))
        ph = rng.uniform(0, 2 * np.pi, n)
        v = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], 1)
        v[rng.uniform(size=n) < 0.5, 2] *= -1
        return v
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def test_tables_identical(pair):
    m, r = pair
    for a, b in zip(m.export(), r.export()):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("grazing", [False, True])
def test_eval_pdf_sample_identical(pair, grazing):
    m, r = pair
    rng = np.random.default_rng(5 + grazing)
    wi, wo = _dirs(rng, 20000, grazing), _dirs(rng, 20000)
    wo[:, 2] = np.abs(wo[:, 2]) * np.sign(wi[:, 2])
    for a, b in zip(m.eval_host(wi, wo), r.eval(wi, wo)):
        assert np.array_equal(a, b)
    u = rng.uniform(size=(20000, 2))
    for a, b in zip(m.sample_host(wi, u), r.sample(wi, u)):
        assert np.array_equal(a, b)


def test_rejects_bad_image():
    from skwarka_gb300._lib import SkwError
    with pytest.raises(SkwError):
        MeasuredBRDF(b"\x5a\x00\x00\x00" * 3 + b"\x00" * 64, device=False)
