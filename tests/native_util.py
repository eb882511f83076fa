"""Runs the CUDA path through the C ABI (libdiffvg_gb300.so via ctypes) on a
packed scene with host inputs; returns host outputs.  GPU tests only."""
import numpy as np
import torch

from diffvg_gb300 import _native


def render(packed, params, width, height, nsx, nsy, seed, background=None, eval_positions=None,
           output_sdf=False, d_out=None, want_translation=False, want_background_grad=False, scene=None,
           flags=0):
    dev = torch.device('cuda')
    sc = scene if scene is not None else _native.NativeScene(packed)
    P = torch.from_numpy(np.ascontiguousarray(params, np.float32)).to(dev)
    bg = None if background is None else torch.from_numpy(np.ascontiguousarray(background, np.float32)).to(dev)
    ev = None
    n_ev = 0
    if eval_positions is not None and np.asarray(eval_positions).size > 0:
        ev = torch.from_numpy(np.ascontiguousarray(eval_positions, np.float32).reshape(-1, 2)).to(dev)
        n_ev = ev.shape[0]
    args = _native.RenderArgs(width, height, nsx, nsy, int(seed) & (2 ** 64 - 1), int(bool(packed.use_prefiltering)),
                              n_ev, P.data_ptr(), None if bg is None else bg.data_ptr(),
                              None if ev is None else ev.data_ptr(), flags)
    stream = torch.cuda.current_stream().cuda_stream
    out = {}
    if d_out is None:
        if output_sdf:
            o = torch.empty(n_ev if ev is not None else height * width, device=dev)
            sc.forward(args, sdf_ptr=o.data_ptr(), stream=stream)
            out['sdf'] = o.cpu().numpy().reshape((-1, 1) if ev is not None else (height, width, 1))
        else:
            o = torch.empty(height, width, 4, device=dev)
            sc.forward(args, image_ptr=o.data_ptr(), stream=stream)
            out['image'] = o.cpu().numpy()
    else:
        d = torch.from_numpy(np.ascontiguousarray(d_out, np.float32)).to(dev)
        dp = torch.zeros(max(packed.num_params, 1), device=dev)
        dbg = torch.zeros_like(bg) if (want_background_grad and bg is not None) else None
        dtr = torch.zeros(height, width, 2, device=dev) if want_translation else None
        kw = dict(d_params_ptr=dp.data_ptr(), stream=stream,
                  d_background_ptr=None if dbg is None else dbg.data_ptr(),
                  d_translation_ptr=None if dtr is None else dtr.data_ptr())
        if output_sdf:
            sc.backward(args, d_sdf_ptr=d.data_ptr(), **kw)
        else:
            sc.backward(args, d_image_ptr=d.data_ptr(), **kw)
        out['d_params'] = dp.cpu().numpy()[:packed.num_params]
        out['d_background'] = None if dbg is None else dbg.cpu().numpy()
        out['d_translation'] = None if dtr is None else dtr.cpu().numpy()
    torch.cuda.synchronize()
    return out
