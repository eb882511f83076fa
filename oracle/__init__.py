"""TEST INFRASTRUCTURE ONLY — Python access to the CPU oracle.

The oracle (dvg_oracle.c) is a plain-C restatement of the reference render
path; this module compiles it with gcc and calls it through ctypes on packed
scenes (diffvg_gb300.packing.PackedScene).  It is imported only by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg, as the checker; the
diffvg_gb300 package never imports it.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, '_build')
LIB_PATH = os.path.join(BUILD_DIR, 'libdvg_oracle.so')
# the same source with the work counters compiled in (-DDVG_COUNT_OPS)
COUNT_LIB_PATH = os.path.join(BUILD_DIR, 'libdvg_oracle_count.so')
SOURCES = [os.path.join(HERE, 'dvg_oracle.c')]
HEADERS = [os.path.join(HERE, 'dvg_oracle.h'), os.path.join(HERE, '..', 'include', 'diffvg_gb300.h')]

_lock = threading.Lock()
_libs = {}


def build(force=False, count_ops=False):
    """Compiles the oracle into oracle/_build/libdvg_oracle.so (gcc, no GPU);
    with count_ops, the work-counting variant libdvg_oracle_count.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    path = COUNT_LIB_PATH if count_ops else LIB_PATH
    if not force and os.path.exists(path):
        newest = max(os.path.getmtime(p) for p in SOURCES + HEADERS)
        if os.path.getmtime(path) >= newest:
            return path
    tmp = path + '.%d.tmp' % os.getpid()
    cmd = ['gcc', '-O2', '-std=c11', '-ffp-contract=off', '-fno-fast-math', '-fPIC', '-shared',
           '-o', tmp] + SOURCES + ['-lm', '-lpthread'] + (['-DDVG_COUNT_OPS'] if count_ops else [])
    subprocess.check_call(cmd)
    os.replace(tmp, path)
    return path


class _SceneDesc(ctypes.Structure):
    _fields_ = [
        ('canvas_width', ctypes.c_int32), ('canvas_height', ctypes.c_int32),
        ('num_shapes', ctypes.c_int32), ('num_groups', ctypes.c_int32),
        ('num_params', ctypes.c_int32), ('total_segments', ctypes.c_int32),
        ('total_group_shapes', ctypes.c_int32), ('filter_type', ctypes.c_int32),
        ('filter_radius_off', ctypes.c_int32),
        ('shape_info', ctypes.POINTER(ctypes.c_int32)),
        ('segment_ctrl', ctypes.POINTER(ctypes.c_int32)),
        ('group_info', ctypes.POINTER(ctypes.c_int32)),
        ('group_shapes', ctypes.POINTER(ctypes.c_int32)),
    ]


_FP = ctypes.POINTER(ctypes.c_float)


class _OracleArgs(ctypes.Structure):
    _fields_ = [
        ('width', ctypes.c_int32), ('height', ctypes.c_int32),
        ('num_samples_x', ctypes.c_int32), ('num_samples_y', ctypes.c_int32),
        ('seed', ctypes.c_uint64), ('use_prefiltering', ctypes.c_int32),
        ('num_threads', ctypes.c_int32),
        ('params', _FP), ('background', _FP), ('eval_positions', _FP),
        ('num_eval_positions', ctypes.c_int32),
        ('image', _FP), ('sdf', _FP),
        ('d_image', _FP), ('d_sdf', _FP), ('d_params', _FP),
        ('d_background', _FP), ('d_translation', _FP),
        ('counters', ctypes.POINTER(ctypes.c_int64)),
    ]


def _load(count_ops=False):
    with _lock:
        if count_ops not in _libs:
            lib = ctypes.CDLL(build(count_ops=count_ops))
            lib.dvg_oracle_render.argtypes = [ctypes.POINTER(_SceneDesc), ctypes.POINTER(_OracleArgs),
                                              ctypes.c_char_p, ctypes.c_int]
            lib.dvg_oracle_render.restype = ctypes.c_int
            if count_ops:
                lib.dvg_oracle_ops.argtypes = [ctypes.POINTER(ctypes.c_uint64), ctypes.c_int]
                lib.dvg_oracle_ops.restype = None
            _libs[count_ops] = lib
    return _libs[count_ops]


PHASES = ('weight', 'render', 'resolve', 'edge')
OP_KINDS = ('fp32', 'fp64', 'transcendental')


class OracleError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status


def _ptr(a, ctype=ctypes.c_float):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def _f32(a):
    return None if a is None else np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def render(packed, params, width, height, num_samples_x, num_samples_y, seed,
           background=None, forward=True, d_image=None, d_sdf=None,
           want_translation=False, want_background_grad=False, eval_positions=None,
           output_sdf=False, num_threads=1, count_ops=False):
    """Runs the oracle on a PackedScene with host parameters `params`
    (numpy fp32, the parameter arena).  Returns a dict with 'image' or 'sdf'
    (forward) and 'd_params', 'd_background', 'd_translation' (backward).
    With count_ops the call runs the counting build and the dict also holds
    'ops': {phase: {'fp32', 'fp64', 'transcendental'}} of this call."""
    lib = _load(count_ops)
    if count_ops:
        ops = (ctypes.c_uint64 * 12)()
        lib.dvg_oracle_ops(ops, 1)
    params = _f32(params)
    si = np.ascontiguousarray(packed.shape_info.reshape(-1), dtype=np.int32)
    sc = np.ascontiguousarray(packed.segment_ctrl, dtype=np.int32)
    gi = np.ascontiguousarray(packed.group_info.reshape(-1), dtype=np.int32)
    gs = np.ascontiguousarray(packed.group_shapes, dtype=np.int32)
    # keep non-empty buffers alive for the pointers
    keep = [np.zeros(1, np.int32) if x.size == 0 else x for x in (si, sc, gi, gs)]
    desc = _SceneDesc(packed.canvas_width, packed.canvas_height, packed.num_shapes, packed.num_groups,
                      packed.num_params, int(sc.size), int(gs.size), int(packed.filter_type),
                      int(packed.filter_radius_off),
                      _ptr(keep[0], ctypes.c_int32), _ptr(keep[1], ctypes.c_int32),
                      _ptr(keep[2], ctypes.c_int32), _ptr(keep[3], ctypes.c_int32))
    bg = _f32(background)
    ev = _f32(eval_positions)
    n_ev = 0 if ev is None else ev.reshape(-1, 2).shape[0]
    out = {}
    image = sdf = dparams = dbg = dtr = None
    backward = d_image is not None or d_sdf is not None
    if forward:
        if output_sdf:
            sdf = np.zeros(n_ev if ev is not None else height * width, np.float32)
        else:
            image = np.zeros((height, width, 4), np.float32)
    di = _f32(d_image)
    ds = _f32(d_sdf)
    if backward:
        dparams = np.zeros(max(packed.num_params, 1), np.float32)
        if want_background_grad and bg is not None:
            dbg = np.zeros_like(bg)
        if want_translation:
            dtr = np.zeros((height, width, 2), np.float32)
    counters = np.zeros(8, np.int64)
    args = _OracleArgs(width, height, num_samples_x, num_samples_y, ctypes.c_uint64(int(seed) & (2**64 - 1)),
                       1 if packed.use_prefiltering else 0, int(num_threads),
                       _ptr(params), _ptr(bg), _ptr(ev), n_ev,
                       _ptr(image), _ptr(sdf), _ptr(di), _ptr(ds), _ptr(dparams), _ptr(dbg), _ptr(dtr),
                       counters.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    err = ctypes.create_string_buffer(512)
    status = lib.dvg_oracle_render(ctypes.byref(desc), ctypes.byref(args), err, 512)
    if status != 0:
        raise OracleError(status, err.value.decode(errors='replace'))
    if image is not None:
        out['image'] = image
    if sdf is not None:
        out['sdf'] = sdf.reshape(height, width, 1) if ev is None else sdf.reshape(-1, 1)
    if backward:
        out['d_params'] = dparams[:packed.num_params]
        out['d_background'] = dbg
        out['d_translation'] = dtr
    out['overflow'] = int(counters[0])
    if count_ops:
        lib.dvg_oracle_ops(ops, 1)
        out['ops'] = {ph: {k: int(ops[3 * i + j]) for j, k in enumerate(OP_KINDS)} for i, ph in enumerate(PHASES)}
    return out


def params_of(packed):
    """Host fp32 copy of a PackedScene's parameter arena."""
    if not packed.tensors:
        return np.zeros(1, np.float32)
    return np.concatenate([t.detach().cpu().reshape(-1).numpy().astype(np.float32) for t in packed.tensors])
