"""The reference's own direct-lighting render (built from its sources into
oracle/_ref) against closed-form answers: this pins the reference build that
the render golden fixtures come from.  Skipped where the reference is not
built."""
import numpy as np

import scene_fixtures as sf


def test_reference_sphere_area_lights_known_answer(reference):
    prims, mats, cam, want = sf.sphere_area_lights_case()
    film, _ = reference.render_direct(prims, mats, [], cam, 32, 32)
    assert abs(film.mean() / want - 1.0) <= 0.02, (film.mean(), want)


def test_reference_square_light_known_answer(reference):
    """One light sample per camera sample: an estimator whose light and BSDF
    samples were not random (a sampler fed by a broken generator) lands far
    from the closed form here (about half of it)."""
    prims, mats, cam, want = sf.square_light_case()
    film, _ = reference.render_direct(prims, mats, [], cam, 32, 32, 1)
    assert abs(film.mean() / want - 1.0) <= 0.01, (film.mean(), want)
