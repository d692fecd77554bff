"""Batched multi-view render (one CUDA graph per run over all views) against
the single-camera render: every view of the batch must be bit-identical to
RenderScene.render_direct with the same seed, before and after the
autotuner changes the pass configuration, and across repeated graph
launches."""
import numpy as np
import pytest

from skwarka_gb300 import scenes
from skwarka_gb300.render import Camera, RenderBatch, RenderScene

pytestmark = pytest.mark.gpu


def _small_case():
    prims, mats = scenes.batching_scene(levels=(4, 3, 3, 2))
    cams = scenes.batching_views(n=5, seed=9, lo=8, hi=96)
    # uneven, non-square films too
    cams.append(Camera.look_at((0.1, 0.2, -0.8), (0.0, -0.5, 0.5), (0, 1, 0), np.radians(60), 37, 11))
    cams.append(Camera.look_at((-0.5, 0.5, 0.6), (0.3, -0.8, -0.2), (0, 1, 0), np.radians(80), 5, 70))
    return RenderScene(prims, mats), cams


def _plain(sc, cams, seeds, spp=(2, 2)):
    return [sc.render_direct(c, spp[0], spp[1], seed=int(s)).cpu().numpy() for c, s in zip(cams, seeds)]


def test_batch_equals_single_view_renders(gpu):
    sc, cams = _small_case()
    seeds = np.arange(len(cams), dtype=np.uint64) * 7919 + 3
    ref = _plain(sc, cams, seeds)
    # tiny passes: many passes, views split across passes, both workspaces used
    for cfg in (None, dict(samples_per_pass=4096, stack_cap=0, trace_ctas_per_sm=0, shade_block=64, overlap=1),
                dict(samples_per_pass=1000, stack_cap=0, trace_ctas_per_sm=2, shade_block=128, overlap=0)):
        b = RenderBatch(sc, cams, 2, 2, seeds=seeds, config=cfg)
        films = b.run()
        for v in range(len(cams)):
            assert np.array_equal(b.view(films, v).cpu().numpy(), ref[v]), (cfg, v)
        films2 = b.run(films)  # graph replay
        assert np.array_equal(films2.cpu().numpy(), films.cpu().numpy())


def test_batch_default_seeds_and_new_buffer(gpu):
    sc, cams = _small_case()
    b = RenderBatch(sc, cams, 1, 2, seed=40)
    ref = _plain(sc, cams, [40 + v for v in range(len(cams))], spp=(1, 2))
    f1 = b.run()
    f2 = b.run()  # a new buffer: the graph is captured again for it
    for v in range(len(cams)):
        assert np.array_equal(b.view(f1, v).cpu().numpy(), ref[v])
        assert np.array_equal(b.view(f2, v).cpu().numpy(), ref[v])


def test_autotune_keeps_results(gpu):
    sc, cams = _small_case()
    b = RenderBatch(sc, cams, 2, 2, seed=5)
    before = b.run().cpu().numpy()
    cfg, ms, n = b.autotune()
    assert n >= 3 and ms > 0
    assert cfg == b.config()
    assert np.array_equal(b.run().cpu().numpy(), before)


def test_batch_rejects_bad_config(gpu):
    from skwarka_gb300._lib import SkwError
    sc, cams = _small_case()
    with pytest.raises(SkwError):
        RenderBatch(sc, cams, 2, 2, config=dict(samples_per_pass=4096, stack_cap=47, trace_ctas_per_sm=0,
                                               shade_block=128, overlap=1))
    with pytest.raises(SkwError):
        RenderBatch(sc, cams, 2, 2, config=dict(samples_per_pass=4096, stack_cap=0, trace_ctas_per_sm=0,
                                               shade_block=96, overlap=1))


def test_batch_with_specular_and_ld_matches_single_views(gpu):
    """Specular trees inside the captured graph (device-side level lengths,
    no host round trip) and the LD sampler: every view equals the
    single-camera render with its seed up to the order of the specular
    slot's float atomics (rtol 1e-5), and a graph replay repeats the run."""
    from skwarka_gb300.render import LD, TRANSPARENT, Material
    glass = Material(kind=TRANSPARENT, kd=(1.0, 1.0, 1.0), ks=(0.9, 0.8, 0.7), refractive_index=1.5)
    prims, mats, lights, cam = scenes.glass_sphere_scene(glass, "area", (40, 24))
    sc = RenderScene(prims, mats, lights)
    sc.set_max_specular_depth(4)
    cams = [cam, Camera.look_at((-1.0, 0.9, 1.5), (0.0, 0.0, 0.4), (0, 0, 1), np.radians(50), 17, 29)]
    seeds = np.array([11, 12], dtype=np.uint64)
    for sampler in (0, LD):
        ref = [sc.render_direct(c, 2, 2, seed=int(s), sampler=sampler).cpu().numpy() for c, s in zip(cams, seeds)]
        b = RenderBatch(sc, cams, 2, 2, seeds=seeds, sampler=sampler,
                        config=dict(samples_per_pass=1024, stack_cap=0, trace_ctas_per_sm=0, shade_block=128,
                                    overlap=1))
        films = b.run()
        for v in range(len(cams)):
            got = b.view(films, v).cpu().numpy()
            assert np.allclose(got, ref[v], rtol=1e-5, atol=1e-7), (sampler, v, np.abs(got - ref[v]).max())
        again = b.run(films).cpu().numpy()
        assert np.allclose(again, films.cpu().numpy(), rtol=1e-5, atol=1e-7)
