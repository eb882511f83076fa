"""The CUDA path against the CPU oracle on seeded scenes drawn like the
benchmark configurations, from small sizes up to the full stroke-heavy
(512x512, 2048 paths) and fill-heavy prefiltered (1024x1024, 512 paths)
scenes.

Forward: every channel value within 1e-4 of the oracle's (no exceptions:
the kernels make the reference's inside / outside decisions sample for
sample, so a flipped sample is a failure).  Gradients: within 1e-3 relative
L2 (the order of the atomic accumulations differs).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FWD_TOL = 1e-4
GRAD_TOL = 1e-3


def _run(builder, spp, seed, prefilter=False, filt=None):
    import torch
    import diffvg_gb300 as dvg
    from diffvg_gb300.packing import pack_scene
    import oracle
    import native_util as nu
    w, h, shapes, groups = builder(dvg)
    pf = None if filt is None else dvg.PixelFilter(type=filt[0], radius=torch.tensor(filt[1]))
    args = dvg.RenderFunction.serialize_scene(w, h, shapes, groups, filter=pf, use_prefiltering=prefilter)
    packed = pack_scene(args)
    P = oracle.params_of(packed)
    ref = oracle.render(packed, P, w, h, spp, spp, seed, num_threads=8)
    mine = nu.render(packed, P, w, h, spp, spp, seed)
    d = np.abs(mine['image'] - ref['image'])
    nbad = int((d > FWD_TOL).sum())
    print('forward max abs %.3g, %d channel values above %.0e' % (d.max(), nbad, FWD_TOL))
    assert nbad == 0, 'forward max abs %.3g' % d.max()
    d_img = (np.arange(d.size, dtype=np.int64).reshape(d.shape) * 2654435761 % 17 - 8).astype(np.float32) / 64
    rb = oracle.render(packed, P, w, h, spp, spp, seed, forward=False, d_image=d_img, num_threads=8)
    mb = nu.render(packed, P, w, h, spp, spp, seed, d_out=d_img)
    num = np.linalg.norm(mb['d_params'] - rb['d_params'])
    den = np.linalg.norm(rb['d_params'])
    print('d_params rel L2 %.3g' % (num / den))
    assert num / den <= GRAD_TOL
    # forward then backward on one scene handle: the backward takes the
    # forward's fragment cache
    from diffvg_gb300 import _native
    sc = _native.NativeScene(packed)
    nu.render(packed, P, w, h, spp, spp, seed, scene=sc)
    mc = nu.render(packed, P, w, h, spp, spp, seed, d_out=d_img, scene=sc)
    num = np.linalg.norm(mc['d_params'] - rb['d_params'])
    print('d_params rel L2 (after forward) %.3g' % (num / den))
    assert num / den <= GRAD_TOL


def test_circle_scene():
    from diffvg_gb300 import workloads
    _run(workloads.circle_scene, 2, 0)


def test_stroke_scene_small():
    from diffvg_gb300 import workloads
    _run(lambda m: workloads.stroke_scene(m, seed=1, num_paths=256, canvas=192), 2, 1)


def test_fill_scene_prefiltered_small():
    from diffvg_gb300 import workloads
    _run(lambda m: workloads.fill_scene(m, seed=3, num_paths=48, canvas=256), 1, 3, prefilter=True)


def test_fill_scene_sampled_small():
    from diffvg_gb300 import workloads
    _run(lambda m: workloads.fill_scene(m, seed=3, num_paths=48, canvas=256), 2, 3)


def test_stroke_scene_full_size():
    """The benchmark's stroke-heavy scene at full size (512x512, 2048 paths,
    2x2 spp): 1,048,576 samples."""
    from diffvg_gb300 import workloads
    _run(lambda m: workloads.stroke_scene(m, seed=1), 2, 1)


def test_fill_scene_full_size_prefiltered():
    """The fill-heavy scene at full size (1024x1024, 512 closed paths with
    constant / linear / radial fills, 10% stroked, prefiltered, 1 spp)."""
    from diffvg_gb300 import workloads
    _run(lambda m: workloads.fill_scene(m, seed=3), 1, 3, prefilter=True)


def test_gaussian_filter_scene():
    """The Gaussian pixel filter (not in the reference; the oracle implements
    the same definition) on a stroke scene and a prefiltered fill scene."""
    import diffvg_gb300 as dvg
    from diffvg_gb300 import workloads
    g = (dvg.FilterType.gaussian, 1.25)
    _run(lambda m: workloads.stroke_scene(m, seed=7, num_paths=128, canvas=128), 2, 4, filt=g)
    _run(lambda m: workloads.fill_scene(m, seed=8, num_paths=24, canvas=128), 1, 5, prefilter=True, filt=g)


def test_deep_mixed_scene():
    """Samples under 40+ overlapping strokes and fills (96x96, 1800 paths):
    the fragment front flushes during the walk, the boundary pass settles
    fp32-decided jobs mid-walk and defers the rest, the fragment cache takes
    chunks past 16 keys, and the backward without a cache sends the deepest
    samples to the deep pass."""
    from diffvg_gb300 import workloads
    _run(lambda dvg: workloads.mixed_scene(dvg, 77, 96, 1800), 2, 5)


def test_deep_fill_scene_prefiltered():
    """Prefiltered samples under many fills (96x96, 300 fills of radius
    4-20, mean box depth 25): cache chunks past 16 fragments and the deep
    pass's regenerated runs."""
    from diffvg_gb300 import workloads
    _run(lambda dvg: workloads.fill_scene(dvg, seed=9, num_paths=300, canvas=96, radius_range=(4.0, 20.0)), 1, 9,
         prefilter=True)


def test_deep_fill_scene_sampled():
    """Sampled colours under many fills (96x96, 300 fills of radius 4-20,
    2x2 spp): a fill-heavy scene of 64 or more groups, whose forward runs
    two blocks per SM with 64 registers."""
    from diffvg_gb300 import workloads
    _run(lambda dvg: workloads.fill_scene(dvg, seed=9, num_paths=300, canvas=96, radius_range=(4.0, 20.0)), 2, 10)


def test_dense_stroke_scene():
    """Samples inside or near about 65 wide strokes each (64x64, 300 paths of
    6 cubic segments, half-widths 2-5): a stroke-only scene takes the wide
    segment-test queues, and lanes still queue more tests than they hold, so
    the walks decide the overflow one lane at a time besides the
    warp-batched decisions and the deferred root walks."""
    from diffvg_gb300 import workloads
    _run(lambda dvg: workloads.stroke_scene(dvg, seed=21, num_paths=300, canvas=64, step=12.0, num_segments=6,
                                            width_range=(2.0, 5.0)), 2, 6)
