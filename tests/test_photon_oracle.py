"""Irradiance photon map (PhotonLTEIntegrator::_ConstructIrradiancePhotonMap,
PhotonLTEIntegrator.cpp:127-245) on seeded synthetic photon maps: the
oracle's restatement and the reference itself against the golden fixture
made by the reference (tests/golden/photon_irradiance.npz), bit for bit."""
from pathlib import Path

import numpy as np

import scene_fixtures as sf

GOLD = Path(__file__).resolve().parent / "golden" / "photon_irradiance.npz"


def _check(res, g):
    pos, ext, intr, nrm, md = res
    assert np.array_equal(pos, g["pos"])
    assert np.array_equal(nrm, g["nrm"])
    assert np.array_equal(ext, g["ext"])
    assert np.array_equal(intr, g["int"])
    assert md == float(g["max_dist"])


def test_oracle_irradiance_map_matches_golden(oracle):
    from oracle.photon import irradiance_map
    maps, paths, area = sf.synthetic_photon_maps()
    g = np.load(GOLD)
    assert len(g["pos"]) == len(maps[2]) // 10
    _check(irradiance_map(oracle, maps, paths, area), g)


def test_reference_irradiance_map_matches_golden(reference):
    maps, paths, area = sf.synthetic_photon_maps()
    _check(reference.photon_irradiance(maps, paths, area), np.load(GOLD))
