"""Generates the full-size golden fixtures of tests/golden/full_*.npz from the
reference itself.

The three plain-method workloads at their stated sizes, rendered by the
reference's own CPU build (compiled from the reference sources by
oracle/build_ref.sh) through the reference's own pydiffvg RenderFunction:

  full_circle_mse           256x256, one circle (128,128) r 40, RGBA
                            (0.3,0.6,0.3,1), 2x2 spp, box 0.5, seed 0; MSE
                            against the circle (120,140) r 48 RGBA
                            (0.7,0.2,0.4,1) rendered the same way; stores
                            both images, the loss and the gradient of the
                            loss for every parameter
  full_stroke512            512x512, 2048 open cubic paths (seed 1), 2x2 spp
  full_fill1024_prefiltered 1024x1024, 512 closed cubic paths with constant /
                            linear / radial fills, 10% stroked (seed 3),
                            prefiltered, 1 spp

For the two large scenes the fixture holds the image quantised to steps of
1/65535 (error at most 0.5/65535 = 7.63e-6 per channel; stored as per-channel row deltas, so
that the archive stays a few MB), a SHA-256 of the exact float32 image, and
the reference's parameter gradient for the adjoint image
tests/scenes.d_image_pattern (deterministic, so it is not stored).

Each fixture also holds the same outputs from the reference built with its
one uninitialised read given a value (oracle/build_ref.sh, variant
"defined"): the quintic isolator's interval slot that the reference leaves
unset when -B/5 falls outside [0, 1] (compute_distance.h:198-201,
within_distance.h:223-226) reads whatever an earlier closest-point or stroke
evaluation on the same CPU thread left on the stack, so the stock module's
result depends on the order in which its threads visited samples, groups and
segments.  The variant reads -1 there (the slot is skipped), as this project
does.  Stored: d_params_defined, out_defined_sha256 and
defined_vs_stock_max_abs (its largest forward difference from the stock
image).

Usage (in a container that has the reference checkout):
    python tests/golden/make_full_golden.py [case ...]
"""
import hashlib
import os
import subprocess
import sys
import tempfile
import time

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import ref_loader  # noqa: E402
from diffvg_gb300 import workloads  # noqa: E402
from diffvg_gb300.packing import pack_scene  # noqa: E402
import scenes  # noqa: E402


def _scene_record(packed):
    return dict(
        canvas_width=packed.canvas_width, canvas_height=packed.canvas_height,
        num_shapes=packed.num_shapes, num_groups=packed.num_groups, num_params=packed.num_params,
        shape_info=packed.shape_info, segment_ctrl=packed.segment_ctrl, group_info=packed.group_info,
        group_shapes=packed.group_shapes, filter_type=packed.filter_type, filter_radius_off=packed.filter_radius_off,
        use_prefiltering=int(packed.use_prefiltering),
        params=np.concatenate([t.detach().reshape(-1).numpy().astype(np.float32) for t in packed.tensors]))


def _grad_args(args):
    out = []
    for i, a in enumerate(args):
        if isinstance(a, torch.Tensor) and a.dtype == torch.float32 and a.numel() > 0 and i != 6:
            a = a.detach().clone().requires_grad_(True)
        out.append(a)
    return out


def _d_params(packed, grad_args):
    d = np.zeros(max(packed.num_params, 1), np.float32)
    for sl in packed.slots:
        a = grad_args[sl.arg_index]
        g = a.grad if isinstance(a, torch.Tensor) else None
        if sl.differentiable and g is not None:
            d[sl.offset:sl.offset + sl.numel] = g.reshape(-1).numpy()
    return d


def circle_mse(pyd, keep_exact=False):
    w, h, shapes, groups = workloads.circle_scene(pyd)
    args = pyd.RenderFunction.serialize_scene(w, h, shapes, groups)
    packed = pack_scene(args)
    ga = _grad_args(args)
    img = pyd.RenderFunction.apply(w, h, 2, 2, 0, None, *ga)
    tw, th, ts, tg = workloads.circle_scene(pyd, center=(120.0, 140.0), radius=48.0, color=(0.7, 0.2, 0.4, 1.0))
    target = pyd.RenderFunction.apply(tw, th, 2, 2, 0, None,
                                      *pyd.RenderFunction.serialize_scene(tw, th, ts, tg)).detach()
    loss = ((img - target) ** 2).mean()
    loss.backward()
    rec = _scene_record(packed)
    rec.update(width=w, height=h, nsx=2, nsy=2, seed=0, out=img.detach().numpy(), target=target.numpy(),
               loss=np.float32(loss.detach()), d_params=_d_params(packed, ga))
    return rec


def quantize_image(img):
    """[H, W, C] image in [0, 1] -> [C, H, W] int16 row deltas of round(v * 65535)
    (decoded by tests/golden_util.dequantize_image)."""
    assert img.min() >= 0.0 and img.max() <= 1.0
    q = np.round(img.astype(np.float64) * 65535.0).astype(np.int32)
    d = np.diff(q.transpose(2, 0, 1), axis=2, prepend=0)
    return d.astype(np.int16)  # wraps modulo 2^16; the decoder's cumulative sum wraps back


def _pattern_case(pyd, builder, spp, seed, prefilter, keep_exact=False):
    w, h, shapes, groups = builder(pyd)
    args = pyd.RenderFunction.serialize_scene(w, h, shapes, groups, use_prefiltering=prefilter)
    packed = pack_scene(args)
    ga = _grad_args(args)
    img = pyd.RenderFunction.apply(w, h, spp, spp, seed, None, *ga)
    d_out = scenes.d_image_pattern(h, w, 4)
    img.backward(torch.from_numpy(d_out))
    out = np.ascontiguousarray(img.detach().numpy(), np.float32)
    rec = _scene_record(packed)
    rec.update(width=w, height=h, nsx=spp, nsy=spp, seed=seed, out_q16_delta=quantize_image(out),
               out_sha256=np.frombuffer(hashlib.sha256(out.tobytes()).digest(), np.uint8),
               d_params=_d_params(packed, ga))
    if keep_exact:
        rec['_out_exact'] = out
    return rec


def stroke512(pyd, keep_exact=False):
    return _pattern_case(pyd, lambda m: workloads.stroke_scene(m, seed=1), 2, 1, False, keep_exact)


def fill1024_prefiltered(pyd, keep_exact=False):
    return _pattern_case(pyd, lambda m: workloads.fill_scene(m, seed=3), 1, 3, True, keep_exact)


CASES = {'full_circle_mse': circle_mse, 'full_stroke512': stroke512,
         'full_fill1024_prefiltered': fill1024_prefiltered}


def _image(rec):
    if 'out' in rec:
        return np.asarray(rec['out'], np.float32)
    return rec['_out_exact']


def defined_worker(name, path):
    """Runs `name` on the variant with the uninitialised slot defined (its
    own process: one reference module per process) and saves its outputs."""
    pyd, _ = ref_loader.load(variant='defined')
    rec = CASES[name](pyd, keep_exact=True)
    np.savez(path, out=_image(rec), d_params=rec['d_params'])


def main():
    if len(sys.argv) == 4 and sys.argv[1] == '--defined-worker':
        defined_worker(sys.argv[2], sys.argv[3])
        return
    only = set(sys.argv[1:])
    pyd, _ = ref_loader.load()
    for name, fn in CASES.items():
        if only and name not in only:
            continue
        t0 = time.time()
        rec = fn(pyd, keep_exact=True)
        with tempfile.TemporaryDirectory() as td:
            tmp = os.path.join(td, 'defined.npz')
            subprocess.check_call([sys.executable, os.path.abspath(__file__), '--defined-worker', name, tmp])
            z = np.load(tmp)
            dout = np.ascontiguousarray(z['out'], np.float32)
            rec['d_params_defined'] = z['d_params']
            rec['out_defined_sha256'] = np.frombuffer(hashlib.sha256(dout.tobytes()).digest(), np.uint8)
            rec['defined_vs_stock_max_abs'] = np.float32(np.abs(dout - _image(rec)).max())
        rec.pop('_out_exact', None)
        path = os.path.join(HERE, name + '.npz')
        np.savez_compressed(path, **rec)
        print('%-28s %9d bytes  %.1f s  defined vs stock: forward max abs %.3g' %
              (name, os.path.getsize(path), time.time() - t0, float(rec['defined_vs_stock_max_abs'])))


if __name__ == '__main__':
    main()
