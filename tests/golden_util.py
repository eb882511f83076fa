"""Loading of the golden fixtures (tests/golden/*.npz) and comparison helpers."""
import glob
import os
from types import SimpleNamespace

import numpy as np

import scenes

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, '*.npz')))


def load(name):
    z = np.load(os.path.join(GOLDEN_DIR, name + '.npz'))
    g = {k: z[k] for k in z.files}
    packed = SimpleNamespace(
        canvas_width=int(g['canvas_width']), canvas_height=int(g['canvas_height']),
        num_shapes=int(g['num_shapes']), num_groups=int(g['num_groups']), num_params=int(g['num_params']),
        shape_info=g['shape_info'].astype(np.int32), segment_ctrl=g['segment_ctrl'].astype(np.int32),
        group_info=g['group_info'].astype(np.int32), group_shapes=g['group_shapes'].astype(np.int32),
        filter_type=int(g['filter_type']), filter_radius_off=int(g['filter_radius_off']),
        use_prefiltering=bool(int(g['use_prefiltering'])))
    w, h = int(g['width']), int(g['height'])
    out = g['out']
    d_out = scenes.d_image_pattern(out.shape[0], out.shape[1] if out.ndim == 3 else 1,
                                   out.shape[-1]).reshape(out.shape)
    rec = SimpleNamespace(
        name=name, packed=packed, params=g['params'].astype(np.float32), width=w, height=h,
        nsx=int(g['nsx']), nsy=int(g['nsy']), seed=int(g['seed']), output_sdf=bool(int(g['output_sdf'])),
        background=scenes.background_pattern(h, w) if int(g['background']) else None,
        eval_positions=g.get('eval_positions'), out=out, d_out=d_out, d_params=g['d_params'],
        d_background=g.get('d_background'), d_translation=g.get('d_translation'))
    return rec


def rel_l2(a, b):
    a = np.asarray(a, np.float64).reshape(-1)
    b = np.asarray(b, np.float64).reshape(-1)
    den = np.sqrt((b * b).sum())
    return float(np.sqrt(((a - b) ** 2).sum()) / max(den, 1e-12))


def image_report(mine, ref, tol=1e-4):
    d = np.abs(np.asarray(mine, np.float64) - np.asarray(ref, np.float64))
    return float(d.max()), int((d > tol).sum()), d.size
