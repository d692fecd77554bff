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
