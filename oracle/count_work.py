"""TEST INFRASTRUCTURE ONLY — counts the algorithmic work of the benchmark
configurations with the oracle's counting build and writes
baseline/work_counts.json.

The counting build (dvg_oracle.c compiled with -DDVG_COUNT_OPS) adds, per
phase of a call, the fp32 and fp64 arithmetic (add, sub, mul, div) and the
sqrt / transcendental calls of the formulas each sample evaluates, with the
traversal replaced by exact bounding-box culls and root iterations counted as
executed.  One forward and one backward call per configuration, each on the
configuration's own inputs: the backward's image adjoint is the MSE gradient
against the configuration's target render, as in the timed step.

The phases map onto the device kernels of one step:
  forward  weight  -> weight       (filter weights per pixel)
  forward  render  -> sample_fwd   (sample colours)
  forward  resolve -> resolve      (filtered image)
  backward render  -> sample_bwd   (interior adjoint: colours, fills, strokes)
  backward edge    -> edge         (boundary term)
bench.py divides a kernel's counted ops by its measured launch time for the
fp32 / fp64 / transcendental fractions of its roofline.

Usage:
    python oracle/count_work.py [--only NAME] [--threads N]
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
OUT = os.path.join(ROOT, 'baseline', 'work_counts.json')

KERNEL_OF = {('forward', 'weight'): 'weight', ('forward', 'render'): 'sample_fwd',
             ('forward', 'resolve'): 'resolve', ('backward', 'render'): 'sample_bwd',
             ('backward', 'edge'): 'edge'}


def cases():
    """Every single-scene benchmark configuration by name: (scene, target
    scene, (nsx, nsy), seed, prefiltering)."""
    import diffvg_gb300 as dvg
    import bench
    scene, target = bench.build_workload(dvg, None)
    out = {'stroke_512_2x2': (scene, target, tuple(bench.WORKLOAD['spp']), bench.WORKLOAD['seed'], False)}
    out.update(bench.config_cases(dvg))
    return out


def count_case(case, threads):
    import numpy as np
    import diffvg_gb300 as dvg
    from diffvg_gb300.packing import pack_scene
    import oracle
    (w, h, shapes, groups), (tw, th, ts, tg), (nsx, nsy), seed, pf = case
    packed = pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups, use_prefiltering=pf))
    tpacked = pack_scene(dvg.RenderFunction.serialize_scene(tw, th, ts, tg, use_prefiltering=pf))
    P = oracle.params_of(packed)
    target = oracle.render(tpacked, oracle.params_of(tpacked), w, h, nsx, nsy, seed, num_threads=threads)['image']
    fwd = oracle.render(packed, P, w, h, nsx, nsy, seed, num_threads=threads, count_ops=True)
    d_img = ((2.0 / fwd['image'].size) * (fwd['image'] - target)).astype(np.float32)
    bwd = oracle.render(packed, P, w, h, nsx, nsy, seed, forward=False, d_image=d_img, num_threads=threads,
                        count_ops=True)
    n = w * h * nsx * nsy
    kernels = {}
    for (call, phase), kernel in KERNEL_OF.items():
        ops = (fwd if call == 'forward' else bwd)['ops'][phase]
        if any(ops.values()):
            kernels[kernel] = dict(ops, per_sample={k: round(v / n, 2) for k, v in ops.items()})
    return {'canvas': [w, h], 'spp': [nsx, nsy], 'samples': n, 'prefiltered': bool(pf),
            'path_segments': int(packed.segment_ctrl.size), 'kernels': kernels}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--only', default=None)
    ap.add_argument('--threads', type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    try:
        with open(OUT) as f:
            result = json.load(f)
    except (OSError, ValueError):
        result = {}
    result.setdefault('configs', {})
    result['definition'] = (
        'per kernel of one fwd+bwd step: fp32 and fp64 add/sub/mul/div and sqrt/transcendental calls of the '
        "reference algorithm's formulas as restated by oracle/dvg_oracle.c (OPS annotations), traversal "
        'replaced by exact bounding-box culls, root iterations as executed; counted by oracle/count_work.py')
    for name, case in cases().items():
        if args.only and name != args.only:
            continue
        t0 = time.perf_counter()
        result['configs'][name] = count_case(case, args.threads)
        print('%s: %.1f s %s' % (name, time.perf_counter() - t0,
                                 json.dumps({k: v['per_sample'] for k, v in result['configs'][name]['kernels'].items()})),
              flush=True)
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    with open(OUT, 'w') as f:
        json.dump(result, f, indent=1, sort_keys=True)
        f.write('\n')


if __name__ == '__main__':
    main()
