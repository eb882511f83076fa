"""Generates the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's own CPU build (compiled from the reference sources by
oracle/build_ref.sh) through the reference's own pydiffvg RenderFunction on
every scene of tests/scenes.py, and stores per case: the packed scene (the
C ABI's topology arrays and parameter arena, see diffvg_gb300/packing.py),
the render settings, the forward output, and the reference's gradients
(parameter arena, background, render_grad translation image) for the
deterministic adjoint image tests/scenes.d_image_pattern.

Usage (in a container that has the reference checkout):
    python tests/golden/make_golden.py [reference_dir [case ...]]
With case names given, only those fixtures are written.
"""
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import ref_loader  # noqa: E402
from diffvg_gb300.packing import pack_scene  # noqa: E402
import scenes  # noqa: E402


def run_case(pyd, case):
    args = scenes.serialize(pyd, pyd, case)
    packed = pack_scene(args)
    w, h, spp, seed = case['width'], case['height'], case['spp'], case['seed']
    ns = int(round(spp ** 0.5)) if spp in (1, 4, 9) else None
    nsx, nsy = (ns, ns) if ns else (spp, 1)
    bg = None
    if case['background']:
        bg = torch.from_numpy(scenes.background_pattern(h, w)).requires_grad_(True)
    grad_args = []
    for a in args:
        if isinstance(a, torch.Tensor) and a.dtype == torch.float32 and a.numel() > 0 and a is not args[6]:
            a = a.detach().clone().requires_grad_(True)
        grad_args.append(a)
    out = pyd.RenderFunction.apply(w, h, nsx, nsy, seed, bg, *grad_args)
    d_out = scenes.d_image_pattern(out.shape[0], out.shape[1] if out.dim() == 3 else 1,
                                   out.shape[-1]).reshape(out.shape)
    out.backward(torch.from_numpy(d_out))
    d_params = np.zeros(max(packed.num_params, 1), np.float32)
    for sl in packed.slots:
        g = grad_args[sl.arg_index].grad if isinstance(grad_args[sl.arg_index], torch.Tensor) else None
        if sl.differentiable and g is not None:
            d_params[sl.offset:sl.offset + sl.numel] = g.reshape(-1).numpy()
    rec = dict(
        canvas_width=packed.canvas_width, canvas_height=packed.canvas_height,
        num_shapes=packed.num_shapes, num_groups=packed.num_groups, num_params=packed.num_params,
        shape_info=packed.shape_info, segment_ctrl=packed.segment_ctrl, group_info=packed.group_info,
        group_shapes=packed.group_shapes, filter_type=packed.filter_type, filter_radius_off=packed.filter_radius_off,
        use_prefiltering=int(packed.use_prefiltering), output_sdf=int(case['output'] == 'sdf'),
        params=np.concatenate([t.detach().reshape(-1).numpy().astype(np.float32) for t in packed.tensors]),
        width=w, height=h, nsx=nsx, nsy=nsy, seed=seed, background=int(case['background']),
        out=out.detach().numpy(), d_params=d_params)
    if case['eval_positions'] is not None:
        rec['eval_positions'] = case['eval_positions'].numpy()
    if bg is not None:
        rec['d_background'] = bg.grad.numpy()
    if case['output'] == 'color' and case['eval_positions'] is None and bg is None:
        # render_grad: the translation gradient image (the reference's
        # render_grad fails with a background image: render_pytorch.py:638
        # names an undefined variable)
        args2 = scenes.serialize(pyd, pyd, case)
        dtr = pyd.RenderFunction.render_grad(torch.from_numpy(d_out), w, h, nsx, nsy, seed,
                                             None if bg is None else bg.detach(), *args2)
        rec['d_translation'] = dtr.numpy()
    return rec


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else ref_loader.reference_dir()
    only = set(sys.argv[2:])
    pyd, _ = ref_loader.load(ref)
    for builder in scenes.CASES:
        if only and builder.__name__ not in only:
            continue
        case = builder(pyd)
        rec = run_case(pyd, case)
        path = os.path.join(HERE, builder.__name__ + '.npz')
        np.savez_compressed(path, **rec)
        print('%-40s %7d bytes' % (builder.__name__, os.path.getsize(path)))


if __name__ == '__main__':
    main()
