"""Loading of the golden fixtures (tests/golden/*.npz) and comparison helpers."""
import glob
import os
from types import SimpleNamespace

import numpy as np

import scenes

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def names():
    """The per-feature fixtures (made by make_golden.py)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, '*.npz'))
                  if not os.path.basename(p).startswith('full_'))


def full_names():
    """The full-size workload fixtures (made by make_full_golden.py)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, 'full_*.npz')))


# quantisation step of the full-size fixtures' stored images and its error
# bound (half a step, plus the float64 rounding of the decode)
Q16_STEP = 1.0 / 65535.0
Q16_ERR = 0.5 / 65535.0 + 1e-12


def dequantize_image(d):
    """Inverse of make_full_golden.quantize_image: [C, H, W] int16 row deltas
    -> [H, W, C] float64 image (within Q16_ERR of the reference's)."""
    q = np.cumsum(d.astype(np.int64), axis=2) & 0xffff
    return (q.astype(np.float64) * Q16_STEP).transpose(1, 2, 0)


def load_full(name):
    z = np.load(os.path.join(GOLDEN_DIR, name + '.npz'))
    g = {k: z[k] for k in z.files}
    packed = SimpleNamespace(
        canvas_width=int(g['canvas_width']), canvas_height=int(g['canvas_height']),
        num_shapes=int(g['num_shapes']), num_groups=int(g['num_groups']), num_params=int(g['num_params']),
        shape_info=g['shape_info'].astype(np.int32), segment_ctrl=g['segment_ctrl'].astype(np.int32),
        group_info=g['group_info'].astype(np.int32), group_shapes=g['group_shapes'].astype(np.int32),
        filter_type=int(g['filter_type']), filter_radius_off=int(g['filter_radius_off']),
        use_prefiltering=bool(int(g['use_prefiltering'])))
    quantized = 'out_q16_delta' in g
    out = dequantize_image(g['out_q16_delta']) if quantized else g['out']
    return SimpleNamespace(
        name=name, packed=packed, params=g['params'].astype(np.float32), width=int(g['width']),
        height=int(g['height']), nsx=int(g['nsx']), nsy=int(g['nsy']), seed=int(g['seed']), out=out,
        out_err=Q16_ERR if quantized else 0.0, out_sha256=g.get('out_sha256'), target=g.get('target'),
        loss=g.get('loss'), d_params=g['d_params'], d_params_defined=g.get('d_params_defined'),
        out_defined_sha256=g.get('out_defined_sha256'),
        defined_vs_stock_max_abs=float(g.get('defined_vs_stock_max_abs', 0.0)))


def sha256_matches(img, digest):
    import hashlib
    if digest is None:
        return None
    return hashlib.sha256(np.ascontiguousarray(img, np.float32).tobytes()).digest() == bytes(digest)


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
