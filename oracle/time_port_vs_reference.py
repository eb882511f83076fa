"""TEST INFRASTRUCTURE ONLY — times the oracle port against the reference's
own CPU module on the same cores.

The reported CPU baseline (bench.py's cpu_baseline and its --impl reference
arm) runs the oracle port, because the reference's CPU module cannot be
built on the GPU host (no pybind11 there, no reference checkout).  This
script measures how the two compare where both run: the reference through
its own pydiffvg.RenderFunction (apply, then backward of an MSE loss; its
scene is rebuilt on the host in every call, as the reference does), the port
through oracle.render (forward, then backward of the same loss), both with
every host core, on the three plain-method workloads: the single circle
(256x256, 2x2 spp), the stroke-heavy scene (512x512, 2048 paths, 2x2 spp)
and the fill-heavy prefiltered scene (1024x1024, 512 paths, 1 spp).
One warm-up, then the median of `--repeats` timed steps.

Usage (in a container with the reference checkout):
    python oracle/time_port_vs_reference.py [--repeats 5]
"""
import argparse
import json
import os
import statistics
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)


def workloads_of(mod):
    from diffvg_gb300 import workloads
    return {
        'circle_256_2x2': (workloads.circle_scene(mod),
                           workloads.circle_scene(mod, center=(120.0, 140.0), radius=48.0,
                                                  color=(0.7, 0.2, 0.4, 1.0)), 2, 0, False),
        'stroke_512_2x2': (workloads.stroke_scene(mod, seed=1), workloads.stroke_scene(mod, seed=2), 2, 1, False),
        'fill_prefiltered_1024_1x1': (workloads.fill_scene(mod, seed=3), workloads.fill_scene(mod, seed=4), 1, 3, True),
    }


def time_reference(pyd, case, repeats):
    import torch
    (w, h, shapes, groups), (tw, th, ts, tg), spp, seed, pf = case
    target = pyd.RenderFunction.apply(w, h, spp, spp, seed, None,
                                      *pyd.RenderFunction.serialize_scene(tw, th, ts, tg, use_prefiltering=pf))
    for s in shapes:
        for name in ('points', 'radius', 'center', 'stroke_width'):
            t = getattr(s, name, None)
            if isinstance(t, torch.Tensor) and t.dtype == torch.float32:
                t.requires_grad_(True)

    def step():
        args = pyd.RenderFunction.serialize_scene(w, h, shapes, groups, use_prefiltering=pf)
        img = pyd.RenderFunction.apply(w, h, spp, spp, seed, None, *args)
        ((img - target) ** 2).mean().backward()

    step()
    times = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        step()
        times.append(time.perf_counter() - t0)
    return statistics.median(times)


def time_port(case, repeats, threads):
    import numpy as np
    import diffvg_gb300 as dvg
    from diffvg_gb300.packing import pack_scene
    import oracle
    (w, h, shapes, groups), (tw, th, ts, tg), spp, seed, pf = case
    packed = pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups, use_prefiltering=pf))
    tp = pack_scene(dvg.RenderFunction.serialize_scene(tw, th, ts, tg, use_prefiltering=pf))
    P = oracle.params_of(packed)
    target = oracle.render(tp, oracle.params_of(tp), w, h, spp, spp, seed, num_threads=threads)['image']

    def step():
        img = oracle.render(packed, P, w, h, spp, spp, seed, num_threads=threads)['image']
        d = ((2.0 / img.size) * (img - target)).astype(np.float32)
        oracle.render(packed, P, w, h, spp, spp, seed, forward=False, d_image=d, num_threads=threads)

    step()
    times = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        step()
        times.append(time.perf_counter() - t0)
    return statistics.median(times)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--repeats', type=int, default=5)
    args = ap.parse_args()
    from oracle import ref_loader
    import diffvg_gb300 as dvg
    pyd, _ = ref_loader.load()
    threads = os.cpu_count() or 1
    ref_cases, port_cases = workloads_of(pyd), workloads_of(dvg)
    out = {'cores': threads, 'cpu': _cpu_model(), 'repeats': args.repeats, 'configs': {}}
    for name in ref_cases:
        (w, h, _, _), _, spp, _, _ = port_cases[name]
        n = w * h * spp * spp
        tr = time_reference(pyd, ref_cases[name], args.repeats)
        tq = time_port(port_cases[name], args.repeats, threads)
        out['configs'][name] = {'samples': n, 'reference_s': round(tr, 4), 'port_s': round(tq, 4),
                                'reference_Msamples_per_s': round(n / tr / 1e6, 4),
                                'port_Msamples_per_s': round(n / tq / 1e6, 4),
                                'port_over_reference': round(tr / tq, 3)}
        print(name, json.dumps(out['configs'][name]), flush=True)
    print(json.dumps(out))


def _cpu_model():
    try:
        with open('/proc/cpuinfo') as f:
            for line in f:
                if line.startswith('model name'):
                    return line.split(':', 1)[1].strip()
    except OSError:
        pass
    return 'unknown'


if __name__ == '__main__':
    main()
