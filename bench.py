"""Benchmark of the render hot path: fwd+bwd Msamples/s.

Workload (the stroke-heavy plain-method configuration): canvas 512x512,
2x2 samples per pixel, box filter radius 0.5, seed 1; 2048 open paths of 4
cubic segments (13 control points, first point uniform in the canvas, each
later point a uniform [-20, 20]^2 step), stroke half-width U[1, 4], stroke
RGBA U[0, 1]^4, no fill.  Loss: MSE against the render of the same
generator with seed 2.  One step = forward + loss gradient + backward
(interior and boundary terms) = 1,048,576 samples.

Lines printed (one JSON line, rank 0):
  value  device-resident throughput: parameters, target and buffers live in
         HBM; each step is timed with CUDA events on the launching stream,
         the L2 is flushed (a 256 MiB write) between steps outside the timed
         events.
  e2e    the same metric through the C ABI that stands in for the
         reference's diffvg.render (dvg_render_forward / dvg_render_backward)
         with the parameter and gradient arenas in pinned host memory: the
         host-to-device copy of the parameters, the render, the loss
         gradient, the backward, the gradients and the loss copied back to
         the host are all inside the timed region (wall clock).
  e2e_render_function  the same through the PyTorch drop-in
         (RenderFunction.serialize_scene / apply / backward) with the scene
         tensors in host memory; it adds PyTorch's per-tensor work for the
         scene's 6144 leaf tensors (serialisation, autograd bookkeeping,
         one gradient view per tensor).
  e2e_render_function_fused  the drop-in with the scene's parameters
         fused into one device tensor (fuse_parameters): autograd tracks
         one tensor; the loss is read back every step.
  roofline  the dominant kernel's algorithmic bytes per launch over its
         CUDA-event time, against the measured HBM copy bandwidth.
  cpu_baseline  the CPU oracle port (oracle/, all host cores) on one full
         step of the same workload.

--impl reference times the reference algorithm on the host cores (the
oracle port; the reference's own CPU module cannot be built on the GPU
host) and prints the same line with "impl": "reference".
Under torchrun (N > 1) every rank renders its own replica of the workload
(no collective on the data path); the timed region is bracketed by barriers
and the slowest rank's time is used.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(canvas=512, num_paths=2048, spp=(2, 2), seed=1, target_seed=2, filter='box', radius=0.5)
METRIC = 'fwd+bwd Msamples/s'
UNIT = 'Msamples/s'


def launches_per_span(packed):
    """Kernel launches inside each span the scene's profile table times
    (csrc/dvg_capi.cu timed(), csrc/dvg_render.cu and dvg_prep.cu launchers):
    preparation 7 to 12 kernels (path, segment, band-list and stroke-record
    kernels only where the scene has them); the sampled
    forward, and the boundary pass of a scene of 8+ groups, add the deferred
    root walks (jobs, roots, finish)."""
    import numpy as np
    info = np.asarray(packed.shape_info).reshape(-1, 8)
    groups = np.asarray(packed.group_info).reshape(-1, 12)
    paths = bool((info[:, 0] == 2).any()) if info.size else False
    banded = bool(((info[:, 0] == 2) & (info[:, 3] >= 64)).any()) if info.size else False
    stroked = bool((groups[:, 5] != -1).any()) if groups.size else False
    prep = 7 + (1 if paths else 0) + (1 if np.asarray(packed.segment_ctrl).size else 0) + (1 if banded else 0) \
        + (2 if stroked else 0)
    defer = packed.num_groups >= 8
    return {'prepare': prep, 'weight': 1, 'sample_fwd': 4 if defer else 1, 'resolve': 1,
            'sample_bwd': 2, 'edge': 7 if defer else 4, 'sdf': 1, 'bg_combine': 1}
HEADLINE = 'stroke_512_2x2'  # the headline workload's name among the counted configurations


def _dist():
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return ws, rank, local


def aggregate_throughput(total_ms, n_samples, steps, ws, device=None):
    """Whole-job Msamples/s of replicas: every rank rendered n_samples per
    step for `steps` steps, and the job took as long as the slowest rank
    (max over ranks; the caller's process group: NCCL on the GPUs, gloo in
    the CPU tests).  Returns (value, max total_ms)."""
    if ws > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([total_ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
        dist.barrier()
    return ws * n_samples * steps / (total_ms / 1e3) / 1e6, total_ms


def _workload_config():
    return {'workload': 'stroke-heavy plain method: 512x512 canvas, 2x2 spp, box r=0.5, 2048 open cubic paths '
                        '(4 segments, 13 points), stroke half-width U[1,4], seed 1; MSE vs seed-2 target',
            'canvas': [512, 512], 'num_paths': 2048, 'samples_per_step': 512 * 512 * 4,
            'l2': 'flushed between timed steps (256 MiB write)', 'parallelism': 'replicas'}


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,'
              'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
              'clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.gpu), '--query-gpu=' + self.FIELDS,
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(',')]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == 'active':
                    reasons.add(nm)
        sm.sort()
        return {'sm_mhz': sm[len(sm) // 2] if sm else None, 'sm_max_mhz': smax, 'reasons': sorted(reasons),
                'samples': len(sm)}


def _peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            p = json.load(f)
        return float(p['hbm_gbs']), 'measured'
    except Exception:
        return 6800.0, 'fallback'


def issue_roofline(warp_instructions, avg_launch_s, num_sms, sm_mhz):
    """Issue-slot roofline of an instruction-bound kernel: warp instructions
    per launch (from an ncu capture of the same workload) over the live
    launch time, against 4 schedulers x 1 warp instruction per cycle per SM
    at the sampled SM clock.  None when an input is missing."""
    if not warp_instructions or not avg_launch_s or not num_sms or not sm_mhz:
        return None
    achieved = warp_instructions / avg_launch_s / 1e9
    peak = 4.0 * num_sms * sm_mhz / 1e3
    return {'achieved': round(achieved, 2), 'peak': round(peak, 2), 'unit': 'G warp instructions/s',
            'frac': round(achieved / peak, 4), 'warp_instructions': int(warp_instructions),
            'source': 'profiles/ncu_traffic.json (ncu smsp__inst_executed.sum per launch)'}


FP64_PEAK_OPS = 1.25e12   # GB300 nominal dense fp64 rate, ops/s (no per-pool measurement exists)


def _work_counts():
    """Counted algorithmic ops per kernel and configuration (oracle/count_work.py)."""
    try:
        with open(os.path.join(ROOT, 'baseline', 'work_counts.json')) as f:
            return json.load(f).get('configs', {})
    except Exception:
        return {}


def op_roofline(config, kernel, avg_launch_s, num_sms, sm_mhz):
    """Counted-op roofline of one kernel: the reference algorithm's fp32 ops,
    fp64 ops and sqrt / transcendental calls per launch (counted once per
    configuration by the oracle's counting build) over the live launch time.
    Peaks at the sampled SM clock: fp32 128 ops per SM per clock (one add,
    sub or mul per lane; the kernels are compiled with --fmad=false, so no
    pair fuses), transcendental 16 per SM per clock (the special-function
    units), fp64 the GB300 nominal 1.25e12 ops/s.  'fp32_fp64_as_fp32'
    counts every fp32 and fp64 op against the fp32 peak: the kernels run the
    reference's fp64 root solves as certified fp32 with rare fp64 fallbacks,
    so the fp64 fraction on its own can exceed 1.  None when a count or a
    time is missing."""
    counts = _work_counts().get(config, {}).get('kernels', {}).get(kernel)
    if not counts or not avg_launch_s or not num_sms or not sm_mhz:
        return None
    clk = sm_mhz * 1e6
    p32, ptr = 128.0 * num_sms * clk, 16.0 * num_sms * clk
    f32, f64, tr = counts['fp32'], counts['fp64'], counts['transcendental']
    return {'unit': 'Gop/s', 'source': 'baseline/work_counts.json',
            'fp32': {'achieved': round(f32 / avg_launch_s / 1e9, 2), 'peak': round(p32 / 1e9, 1),
                     'frac': round(f32 / avg_launch_s / p32, 5), 'ops': f32},
            'fp64': {'achieved': round(f64 / avg_launch_s / 1e9, 2), 'peak': FP64_PEAK_OPS / 1e9,
                     'frac': round(f64 / avg_launch_s / FP64_PEAK_OPS, 5), 'ops': f64},
            'transcendental': {'achieved': round(tr / avg_launch_s / 1e9, 3), 'peak': round(ptr / 1e9, 1),
                               'frac': round(tr / avg_launch_s / ptr, 5), 'ops': tr},
            'fp32_fp64_as_fp32': {'frac': round((f32 + f64) / avg_launch_s / p32, 5)}}


def _ncu_traffic():
    """Per-launch DRAM bytes per kernel from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, 'profiles', 'ncu_traffic.json')) as f:
            return json.load(f)
    except Exception:
        return {}


def build_workload(mod, device):
    import torch
    from diffvg_gb300 import workloads
    w, h, shapes, groups = workloads.stroke_scene(mod, seed=WORKLOAD['seed'], num_paths=WORKLOAD['num_paths'],
                                                  canvas=WORKLOAD['canvas'])
    tw, th, tshapes, tgroups = workloads.stroke_scene(mod, seed=WORKLOAD['target_seed'],
                                                      num_paths=WORKLOAD['num_paths'], canvas=WORKLOAD['canvas'])
    return (w, h, shapes, groups), (tw, th, tshapes, tgroups)


def algorithmic_bytes(kernel, packed, w, h, spp):
    """Unique bytes a launch must move: scene data read, per-pixel / per-sample
    inputs read, outputs written."""
    scene = 4 * packed.num_params + 4 * (packed.shape_info.size + packed.segment_ctrl.size +
                                         packed.group_info.size + packed.group_shapes.size)
    npx, n = w * h, w * h * spp
    if kernel == 'sample_fwd':
        return scene + 16 * n                      # sample colours out
    if kernel == 'resolve':
        return 16 * n + 4 * npx + 16 * npx         # samples + weights in, image out
    if kernel == 'weight':
        return 4 * npx
    if kernel == 'sample_bwd':
        return scene + 16 * npx + 4 * npx + 4 * packed.num_params   # d_image, weights in; d_params out
    if kernel == 'edge':
        # the boundary pass: records written and read back once (56 B per boundary sample, as the
        # reference's BoundarySample), d_image and weights in, d_params out
        return scene + 2 * 56 * n + 16 * npx + 4 * npx + 4 * packed.num_params
    return scene


def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist
    import diffvg_gb300 as dvg
    from diffvg_gb300 import _native
    from diffvg_gb300.packing import pack_scene

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    dvg.set_device(dev)
    if ws > 1:
        dist.init_process_group('nccl', device_id=dev)
    (w, h, shapes, groups), (tw, th, tshapes, tgroups) = build_workload(dvg, dev)
    nsx, nsy = WORKLOAD['spp']
    spp = nsx * nsy
    n_samples = w * h * spp
    seed = WORKLOAD['seed']

    # ---------------- device-resident step through the C ABI ----------------
    sargs = dvg.RenderFunction.serialize_scene(w, h, shapes, groups)
    packed = pack_scene(sargs)
    scene = _native.NativeScene(packed)
    arena = packed.param_arena(dev).contiguous()
    targs = dvg.RenderFunction.serialize_scene(tw, th, tshapes, tgroups)
    tpacked = pack_scene(targs)
    tscene = _native.NativeScene(tpacked)
    tarena = tpacked.param_arena(dev).contiguous()
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream
    target = torch.empty(h, w, 4, device=dev)
    ra = _native.RenderArgs(w, h, nsx, nsy, seed, 0, 0, tarena.data_ptr(), None, None, 0)
    tscene.forward(ra, image_ptr=target.data_ptr(), stream=sptr)
    img = torch.empty(h, w, 4, device=dev)
    d_img = torch.empty_like(img)
    d_params = torch.zeros(packed.num_params, device=dev)
    fwd_args = _native.RenderArgs(w, h, nsx, nsy, seed, 0, 0, arena.data_ptr(), None, None, _native.DVG_FLAG_NO_SYNC)
    bwd_args = _native.RenderArgs(w, h, nsx, nsy, seed, 0, 0, arena.data_ptr(), None, None,
                                  _native.DVG_FLAG_NO_SYNC | _native.DVG_FLAG_REUSE_PREP)
    scale = 2.0 / img.numel()
    loss_buf = torch.zeros((), device=dev)

    def step():
        scene.forward(fwd_args, image_ptr=img.data_ptr(), stream=sptr)
        torch.sub(img, target, out=d_img)
        loss_buf.copy_(torch.sum(d_img * d_img))
        d_img.mul_(scale)
        d_params.zero_()
        scene.backward(bwd_args, d_image_ptr=d_img.data_ptr(), d_params_ptr=d_params.data_ptr(), stream=sptr)

    flush = torch.empty(256 * 1024 * 1024 // 4, device=dev)
    for _ in range(max(args.warmup, 3)):
        step()
    scene.sync(sptr)
    torch.cuda.synchronize(dev)
    # forward / backward split, measured once on a warm step
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    flush.fill_(1.0)
    e0.record(stream)
    scene.forward(fwd_args, image_ptr=img.data_ptr(), stream=sptr)
    e1.record(stream)
    d_params.zero_()
    scene.backward(bwd_args, d_image_ptr=d_img.data_ptr(), d_params_ptr=d_params.data_ptr(), stream=sptr)
    e2.record(stream)
    torch.cuda.synchronize(dev)
    fwd_ms, bwd_ms = e0.elapsed_time(e1), e1.elapsed_time(e2)

    clocks = ClockSampler(local)
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize(dev)
    clocks.start()
    scene.profile(True)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    for i in range(args.steps):
        flush.fill_(float(i))          # L2 flush, outside the timed events
        starts[i].record(stream)
        step()
        ends[i].record(stream)
    torch.cuda.synchronize(dev)
    clock_info = clocks.stop()
    scene.sync(sptr)
    kernels = scene.profile_read()
    scene.profile(False)
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    value, total_ms = aggregate_throughput(float(sum(step_ms)), n_samples, args.steps, ws, dev)
    per_span = launches_per_span(packed)
    gpu_launches = 0
    for name, (cnt, _) in kernels.items():
        gpu_launches += cnt * per_span.get(name, 1)

    # ---------------- roofline of the dominant kernel ----------------
    peak, peak_kind = _peaks()
    dom = max((k for k in kernels if k != 'prepare'), key=lambda k: kernels[k][1])
    dom_cnt, dom_ms = kernels[dom]
    avg_s = dom_ms / dom_cnt / 1e3
    alg = algorithmic_bytes(dom, packed, w, h, spp)
    achieved = alg / avg_s / 1e9
    traffic = _ncu_traffic().get(dom)
    roofline = {'bound': 'hbm', 'kernel': dom, 'achieved': round(achieved, 3), 'peak': peak,
                'peak_source': peak_kind, 'unit': 'GB/s', 'frac': round(achieved / peak, 6),
                'traffic': traffic, 'algorithmic_bytes': alg, 'avg_launch_ms': round(avg_s * 1e3, 4),
                'note': 'the path is FP32/FP64-issue bound (no dense contraction); the HBM fraction is small by '
                        'construction, the issue-slot fraction is the binding one'}
    sm_mhz = clock_info.get('sm_mhz') or clock_info.get('sm_max_mhz') or 2070.0
    num_sms = torch.cuda.get_device_properties(dev).multi_processor_count
    roofline['issue'] = issue_roofline(_ncu_traffic().get(dom + '_warp_instructions'), avg_s, num_sms, sm_mhz)
    # counted-op rooflines: the dominant kernel first, then every kernel with counts
    roofline['fp32'] = op_roofline(HEADLINE, dom, avg_s, num_sms, sm_mhz)
    roofline['by_kernel'] = {k: op_roofline(HEADLINE, k, ms / cnt / 1e3, num_sms, sm_mhz)
                             for k, (cnt, ms) in kernels.items() if k != 'prepare'}

    # ---------------- end to end with host buffers ----------------
    e2e = e2e_rf = e2e_fused = None
    if not getattr(args, 'no_e2e', False):
        e2e = run_e2e_cabi(args, packed, scene, dev, target, w, h, nsx, nsy, seed, n_samples, ws)
        e2e_rf = run_e2e(args, dvg, dev, shapes, groups, target, w, h, nsx, nsy, seed, n_samples, ws)
        e2e_fused = run_e2e_fused(args, dvg, dev, target, n_samples, ws)

    out = {'metric': METRIC, 'value': round(value, 3), 'unit': UNIT, 'n_gpus': ws, 'steps': args.steps,
           'warmup': max(args.warmup, 3), 'ms_per_step': round(total_ms / args.steps, 4), 'higher_is_better': True,
           'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32 (fp64 root solves)', 'data': 'synthetic',
           'config': _workload_config(), 'e2e': e2e, 'e2e_render_function': e2e_rf,
           'e2e_render_function_fused': e2e_fused, 'roofline': roofline,
           'clocks': clock_info,
           'gpu_launches': gpu_launches, 'fwd_ms': round(fwd_ms, 4), 'bwd_ms': round(bwd_ms, 4),
           'kernels_ms_per_launch': {k: round(v[1] / v[0], 4) for k, v in kernels.items()},
           'loss': float(loss_buf.item())}
    if rank == 0 and not args.no_batched:
        out['configs'] = run_configs(dev, sm_mhz=sm_mhz, cpu=not args.no_cpu_baseline)
        out['batched'] = run_batched(dev)
        out['served'] = run_served(dev)
    if rank == 0 and not args.no_cpu_baseline:
        out['cpu_baseline'] = cpu_baseline(packed, oracle_params(packed), w, h, nsx, nsy, seed, target.cpu().numpy())
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def run_e2e_cabi(args, packed, scene, dev, target, w, h, nsx, nsy, seed, n_samples, ws):
    """The metric through the C ABI (the drop-in for the reference's
    diffvg.render) with the parameters and gradients in pinned HOST memory,
    as a native caller holds them: every step copies the parameter arena to
    the scene (dvg_scene_update_params), renders, forms the MSE gradient and
    loss on the device (dvg_mse_grad), runs the backward pass, and copies the
    gradient arena and the loss back to the host; the scene handle
    (topology) stays resident.  Wall-clock time over the steps, host
    synchronised on both sides."""
    import torch
    from diffvg_gb300 import _native
    n = packed.num_params
    h_params = packed.param_arena(torch.device('cpu')).contiguous().pin_memory()
    h_grads = torch.empty(n, dtype=torch.float32).pin_memory()
    h_loss = torch.empty(1, dtype=torch.float32).pin_memory()
    img = torch.empty(h, w, 4, device=dev)
    d_img = torch.empty_like(img)
    d_params = torch.empty(n, device=dev)
    loss = torch.empty(1, device=dev)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream
    # params None: the scene's own arena, filled by update_params
    fa = _native.RenderArgs(w, h, nsx, nsy, seed, 0, 0, None, None, None, _native.DVG_FLAG_NO_SYNC)
    ba = _native.RenderArgs(w, h, nsx, nsy, seed, 0, 0, None, None, None,
                            _native.DVG_FLAG_NO_SYNC | _native.DVG_FLAG_REUSE_PREP)

    def step():
        scene.update_params(h_params.data_ptr(), stream=sptr)
        scene.forward(fa, image_ptr=img.data_ptr(), stream=sptr)
        loss.zero_()
        _native.mse_grad(img, target, d_img, loss, stream=sptr)
        d_params.zero_()
        scene.backward(ba, d_image_ptr=d_img.data_ptr(), d_params_ptr=d_params.data_ptr(), stream=sptr)
        h_grads.copy_(d_params, non_blocking=True)
        h_loss.copy_(loss, non_blocking=True)
        scene.sync(sptr)  # waits for the stream; raises on any failure the kernels latched

    for _ in range(max(args.warmup, 3)):
        step()
    k = max(1, min(args.steps, 20))
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(k):
        step()
    torch.cuda.synchronize(dev)
    dt = time.perf_counter() - t0
    return {'value': round(ws * n_samples * k / dt / 1e6, 3), 'unit': UNIT, 'h2d_bytes_per_step': 4 * n,
            'd2h_bytes_per_step': 4 * n + 4, 'steps': k, 'ms_per_step': round(dt / k * 1e3, 3),
            'api': 'C ABI (dvg_scene_update_params, dvg_render_forward, dvg_mse_grad, dvg_render_backward, '
                   'dvg_scene_sync) with the parameter and gradient arenas in pinned host memory; scene topology '
                   'resident',
            'loss': round(float(h_loss[0]) / img.numel(), 6)}


def run_e2e(args, dvg, dev, shapes, groups, target, w, h, nsx, nsy, seed, n_samples, ws):
    """Same metric through RenderFunction (the PyTorch drop-in) with
    host-resident scene tensors: serialize_scene, apply, the loss in torch,
    backward with autograd delivering a gradient to each of the scene's
    6144 leaf tensors."""
    import torch
    params = []
    for s in shapes:
        s.points.requires_grad_(True)
        s.stroke_width.requires_grad_(True)
        params += [s.points, s.stroke_width]
    for g in groups:
        g.stroke_color.requires_grad_(True)
        params.append(g.stroke_color)
    h2d = 4 * sum(p.numel() for p in params) + 4 * (len(groups) * 9 + 1)
    d2h = 4 * sum(p.numel() for p in params) + 4

    def step():
        for p in params:
            p.grad = None
        sargs = dvg.RenderFunction.serialize_scene(w, h, shapes, groups)
        img = dvg.RenderFunction.apply(w, h, nsx, nsy, seed, None, *sargs)
        loss = ((img - target) ** 2).mean()
        loss.backward()
        return float(loss.item())

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize(dev)
    k = max(1, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(k):
        step()
    torch.cuda.synchronize(dev)
    dt = time.perf_counter() - t0
    return {'value': round(ws * n_samples * k / dt / 1e6, 3), 'unit': UNIT, 'h2d_bytes_per_step': h2d,
            'd2h_bytes_per_step': d2h, 'steps': k, 'ms_per_step': round(dt / k * 1e3, 3),
            'api': 'RenderFunction.serialize_scene + apply + MSE + backward, scene tensors in host memory'}


def run_e2e_fused(args, dvg, dev, target, n_samples, ws):
    """Same metric through RenderFunction with the scene's parameters fused
    into one device tensor (fuse_parameters): serialize_scene, apply, the
    loss in torch, backward (autograd tracks the one tensor) and the loss
    read back to the host each step.  A fresh copy of the workload's scene,
    so the other legs' objects are untouched."""
    import torch
    (w, h, shapes, groups), _ = build_workload(dvg, dev)
    nsx, nsy = WORKLOAD['spp']
    seed = WORKLOAD['seed']
    arena, filt = dvg.fuse_parameters(w, h, shapes, groups)

    def step():
        arena.grad = None
        sargs = dvg.RenderFunction.serialize_scene(w, h, shapes, groups, filter=filt)
        img = dvg.RenderFunction.apply(w, h, nsx, nsy, seed, None, *sargs)
        loss = ((img - target) ** 2).mean()
        loss.backward()
        return float(loss.item())

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize(dev)
    k = max(1, min(args.steps, 20))
    t0 = time.perf_counter()
    for _ in range(k):
        step()
    torch.cuda.synchronize(dev)
    dt = time.perf_counter() - t0
    return {'value': round(ws * n_samples * k / dt / 1e6, 3), 'unit': UNIT, 'h2d_bytes_per_step': 0,
            'd2h_bytes_per_step': 4, 'steps': k, 'ms_per_step': round(dt / k * 1e3, 3),
            'api': 'fuse_parameters + RenderFunction.serialize_scene + apply + MSE + backward, parameters in '
                   'one device tensor (one autograd leaf), loss read back each step'}


CONFIG_NAMES = ('circle_256_2x2', 'fill_prefiltered_1024_1x1', 'blob_1024_2x2', 'blob_long_1024_2x2',
                'blob_long_prefiltered_1024_1x1')


def config_cases(dvg):
    """The single-scene configurations besides the headline: (scene, target
    scene, (nsx, nsy), seed, prefiltering) by name."""
    from diffvg_gb300 import workloads
    long_segs = (200, 400)
    return {
        # the single circle (256x256, 2x2 spp; target: the circle at (120,140),
        # radius 48, colour (0.7,0.2,0.4,1))
        'circle_256_2x2': (workloads.circle_scene(dvg),
                           workloads.circle_scene(dvg, center=(120.0, 140.0), radius=48.0,
                                                  color=(0.7, 0.2, 0.4, 1.0)), (2, 2), 0, False),
        # the fill-heavy prefiltered scene (1024x1024, 1 spp, 512 closed paths of
        # 8-32 cubic segments, seed 3; target: the same generator with seed 4)
        'fill_prefiltered_1024_1x1': (workloads.fill_scene(dvg, seed=3), workloads.fill_scene(dvg, seed=4), (1, 1),
                                      3, True),
        # 512 smooth closed paths (workloads.blob_scene) of 8-32 segments and
        # of 200-400 segments (15x the segments, the same shapes' family):
        # the cost per sample against the segment count
        'blob_1024_2x2': (workloads.blob_scene(dvg, seed=5), workloads.blob_scene(dvg, seed=6), (2, 2), 3, False),
        'blob_long_1024_2x2': (workloads.blob_scene(dvg, seed=5, seg_range=long_segs),
                               workloads.blob_scene(dvg, seed=6, seg_range=long_segs), (2, 2), 3, False),
        'blob_long_prefiltered_1024_1x1': (workloads.blob_scene(dvg, seed=5, seg_range=long_segs),
                                           workloads.blob_scene(dvg, seed=6, seg_range=long_segs), (1, 1), 3, True),
    }


CPU_BASELINE_CONFIGS = ('circle_256_2x2', 'fill_prefiltered_1024_1x1')


def run_configs(dev, steps=5, warmup=3, only=None, sm_mhz=None, cpu=True):
    """Device-resident fwd+bwd Msamples/s of the other single-scene
    configurations (config_cases), through the C ABI like the headline leg.
    L2 flushed between steps, CUDA events per step; per-kernel launch times
    over the timed steps with the counted-op roofline of each kernel; for
    the circle and the fill-heavy prefiltered scene, the CPU oracle port on
    the same step (cpu_baseline)."""
    import torch
    import diffvg_gb300 as dvg
    from diffvg_gb300 import _native
    from diffvg_gb300.packing import pack_scene
    cases = config_cases(dvg)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream
    flush = torch.empty(256 * 1024 * 1024 // 4, device=dev)
    out = {}
    for name, ((w, h, shapes, groups), (tw, th, ts, tg), (nsx, nsy), seed, pf) in cases.items():
        if only is not None and name != only:
            continue
        packed = pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups, use_prefiltering=pf))
        tpacked = pack_scene(dvg.RenderFunction.serialize_scene(tw, th, ts, tg, use_prefiltering=pf))
        scene, tscene = _native.NativeScene(packed), _native.NativeScene(tpacked)
        arena, tarena = packed.param_arena(dev).contiguous(), tpacked.param_arena(dev).contiguous()
        target = torch.empty(h, w, 4, device=dev)
        tscene.forward(_native.RenderArgs(w, h, nsx, nsy, seed, int(pf), 0, tarena.data_ptr(), None, None, 0),
                       image_ptr=target.data_ptr(), stream=sptr)
        img, d_img = torch.empty(h, w, 4, device=dev), torch.empty(h, w, 4, device=dev)
        d_params = torch.zeros(max(packed.num_params, 1), device=dev)
        fa = _native.RenderArgs(w, h, nsx, nsy, seed, int(pf), 0, arena.data_ptr(), None, None,
                                _native.DVG_FLAG_NO_SYNC)
        ba = _native.RenderArgs(w, h, nsx, nsy, seed, int(pf), 0, arena.data_ptr(), None, None,
                                _native.DVG_FLAG_NO_SYNC | _native.DVG_FLAG_REUSE_PREP)
        scale = 2.0 / img.numel()

        def step():
            scene.forward(fa, image_ptr=img.data_ptr(), stream=sptr)
            torch.sub(img, target, out=d_img)
            d_img.mul_(scale)
            d_params.zero_()
            scene.backward(ba, d_image_ptr=d_img.data_ptr(), d_params_ptr=d_params.data_ptr(), stream=sptr)

        for _ in range(warmup):
            step()
        scene.sync(sptr)
        torch.cuda.synchronize(dev)
        scene.profile(True)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for i, (a, b) in enumerate(ev):
            flush.fill_(float(i))
            a.record(stream)
            step()
            b.record(stream)
        torch.cuda.synchronize(dev)
        scene.sync(sptr)
        kernels = scene.profile_read()
        scene.profile(False)
        ms = sum(a.elapsed_time(b) for a, b in ev) / steps
        n = w * h * nsx * nsy
        num_sms = torch.cuda.get_device_properties(dev).multi_processor_count
        per_launch = {k: v[1] / v[0] / 1e3 for k, v in kernels.items() if v[0]}
        dom = max((k for k in kernels if k != 'prepare'), key=lambda k: kernels[k][1])
        out[name] = {'Msamples_per_s': round(n / (ms / 1e3) / 1e6, 3), 'ms_per_step': round(ms, 4),
                     'samples_per_step': n, 'prefiltered': pf, 'steps': steps,
                     'path_segments': int(packed.segment_ctrl.size),
                     'kernels_ms_per_launch': {k: round(v * 1e3, 4) for k, v in per_launch.items()},
                     'roofline': {'kernel': dom,
                                  'fp32': op_roofline(name, dom, per_launch[dom], num_sms, sm_mhz or 2070.0),
                                  'by_kernel': {k: op_roofline(name, k, t, num_sms, sm_mhz or 2070.0)
                                                for k, t in per_launch.items() if k != 'prepare'}}}
        if cpu and name in CPU_BASELINE_CONFIGS:
            out[name]['cpu_baseline'] = cpu_baseline(packed, oracle_params(packed), w, h, nsx, nsy, seed,
                                                     target.cpu().numpy(), min_seconds=2.0)
        scene.close()
        tscene.close()
    return out


def run_batched(dev, steps=10, warmup=3, plain_steps=2):
    """The batched workload: 64 stroke scenes (seeds 100-163), canvas sizes
    drawn from {64,128,256,512}^2, path counts log-uniform in [16, 1024],
    2x2 spp, each optimised with Adam (lr 1e-2) towards a perturbed render
    of itself (points N(0, 2 px), colours N(0, 0.05)).

    The batch's step (forward, MSE gradient, backward and Adam for every
    scene, one CUDA graph) is autotuned over its candidates: per-scene
    launches on 8 streams, or persistent launches over a (scene, tile) work
    queue with 1 or 2 resident blocks per SM and 1, 2 or 4 samples per
    thread.  Reports the chosen candidate's steps/s, every candidate's time,
    and the plain per-call path (RenderFunction.apply + backward + torch Adam
    per scene) on the same scenes; equal error: every scene's loss at step
    plain_steps + 1 from the same start, batched against plain."""
    import torch
    import diffvg_gb300 as dvg
    from diffvg_gb300 import workloads
    from diffvg_gb300.batch import BatchedScenes
    seeds = list(range(100, 164))
    scenes = workloads.batched_scenes(dvg, seeds=seeds)
    args = [dvg.RenderFunction.serialize_scene(w, h, s, g) for (w, h, s, g) in scenes]
    b = BatchedScenes(args, seeds=seeds, lr=1e-2, streams=8, check_every=0)
    targets = [b.render(i, workloads.perturbed_target_params(p, b.scene_params(i), seeds[i]))
               for i, p in enumerate(b.packed)]
    b.set_targets(targets)
    candidates = [('streams', (2, 1))] + [('persistent', (c, t)) for c in (1, 2) for t in (1, 2, 4)]
    import tempfile
    with tempfile.TemporaryDirectory() as td:  # a fresh cache: every candidate is timed in this run
        timings = b.autotune(candidates=candidates, steps=3, cache_path=os.path.join(td, 'autotune.json'))
    # equal error: the batch's per-scene losses at step plain_steps + 1
    k_eq = plain_steps + 1
    for _ in range(k_eq):
        b.step()
    torch.cuda.synchronize(dev)
    batched_losses = b.loss()
    for _ in range(warmup):
        b.step()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        b.step()
    e1.record()
    torch.cuda.synchronize(dev)
    b.check()
    ms = e0.elapsed_time(e1) / steps
    n = b.samples_per_step()
    streams_ms = timings.get('streams 2 1')
    pers = {k: v for k, v in timings.items() if k.startswith('persistent')}
    best_p = min(pers, key=pers.get) if pers else None
    out = {'workload': '64 stroke scenes, canvases {64,128,256,512}^2, 16-1024 paths (log-uniform), 2x2 spp, '
                       'Adam lr 1e-2 towards perturbed self-renders', 'samples_per_step': n,
           'steps_per_s': round(1e3 / ms, 3), 'ms_per_step': round(ms, 3), 'Msamples_per_s': round(n / ms / 1e3, 3),
           'mode': b.mode, 'tuning': {'ctas_per_sm': b.tuning.ctas_per_sm,
                                      'samples_per_thread': b.tuning.samples_per_thread},
           'graph': 'one CUDA graph per step (forward, MSE gradient, backward of every scene; one Adam)',
           'autotune_ms_per_step': {k: round(v, 3) for k, v in timings.items()},
           'persistent_vs_streams': (round(streams_ms / pers[best_p], 3) if best_p and streams_ms else None)}
    # plain per-call path on the same scenes and targets, from the same start
    params, opts = [], []
    for (w, h, shapes, groups) in scenes:
        ps = []
        for s in shapes:
            s.points = s.points.to(dev).detach().requires_grad_(True)
            s.stroke_width = s.stroke_width.to(dev).detach().requires_grad_(True)
            ps += [s.points, s.stroke_width]
        for g in groups:
            g.stroke_color = g.stroke_color.to(dev).detach().requires_grad_(True)
            ps.append(g.stroke_color)
        params.append(ps)
        opts.append(torch.optim.Adam(ps, lr=1e-2))

    def plain_step():
        losses = []
        for i, (w, h, shapes, groups) in enumerate(scenes):
            opts[i].zero_grad()
            a = dvg.RenderFunction.serialize_scene(w, h, shapes, groups)
            img = dvg.RenderFunction.apply(w, h, 2, 2, seeds[i], None, *a)
            loss = ((img - targets[i]) ** 2).mean()
            loss.backward()
            opts[i].step()
            losses.append(loss.detach())
        return losses
    plain_step()  # warm-up: packing and scene handles of every scene
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(plain_steps):
        plain_losses = plain_step()
    torch.cuda.synchronize(dev)
    pms = (time.perf_counter() - t0) / plain_steps * 1e3
    plain_losses = [float(l) for l in plain_losses]
    rel = [abs(a - p) / max(abs(p), 1e-12) for a, p in zip(batched_losses, plain_losses)]
    out['plain_steps_per_s'] = round(1e3 / pms, 3)
    out['plain_ms_per_step'] = round(pms, 2)
    out['speedup_vs_plain'] = round(pms / ms, 2)
    out['equal_error_check'] = {'step': k_eq, 'scenes': len(rel), 'max_rel_loss_diff': float('%.3g' % max(rel)),
                                'mean_loss_batched': round(sum(batched_losses) / len(rel), 6),
                                'mean_loss_plain': round(sum(plain_losses) / len(rel), 6)}
    return out


def run_served(dev, rates=(2.0, 8.0, 32.0), num_requests=8, step_range=(100, 500), path_range=(64, 2048),
               plain_steps=3):
    """The served workload at its stated size, on a subsample of requests:
    per arrival rate lambda (Poisson), `num_requests` requests (canvas
    {128,256,512}^2, 64-2048 paths of mixed open strokes and closed fills,
    100-500 Adam steps at lr 1e-2 towards a different seeded scene plus
    N(0, 0.02) pixel noise), admitted under a 150 GB device budget by the
    continuous-batching server.  Reports per lambda the p50 / p99 per-step
    latency and aggregate steps/s; and the plain per-call path
    (RenderFunction + torch Adam, one request at a time, a warm-up step, then
    `plain_steps` timed steps) on the same requests.  Equal error: every
    request's loss at step plain_steps + 1, served against plain, from the
    same start."""
    import torch
    import diffvg_gb300 as dvg
    from diffvg_gb300 import serve, workloads

    def build(seed0):
        specs = workloads.served_requests(dvg, num_requests, seed0=seed0, path_range=path_range,
                                          step_range=step_range)
        out = []
        for sp in specs:
            w, h, shapes, groups = workloads.mixed_scene(dvg, sp['seed'], sp['canvas'], sp['num_paths'])
            tw, th, ts, tg = workloads.mixed_scene(dvg, sp['target_seed'], sp['canvas'], sp['num_paths'])
            targs = dvg.RenderFunction.serialize_scene(tw, th, ts, tg)
            target = workloads.noisy_target(dvg.RenderFunction.apply(tw, th, 2, 2, sp['seed'], None,
                                                                     *targs).detach(), sp['seed'])
            out.append((w, h, shapes, groups, target, sp))
        return out

    per_rate = {}
    all_scenes, all_reqs = [], []
    for k, rate in enumerate(rates):
        scenes = build(500 + 1000 * k)
        gen = torch.Generator().manual_seed(7 + k)
        gaps = torch.empty(num_requests).exponential_(rate, generator=gen).tolist()
        reqs = [serve.Request(dvg.RenderFunction.serialize_scene(w, h, shapes, groups), target, sp['steps'],
                              seed=sp['seed']) for (w, h, shapes, groups, target, sp) in scenes]
        srv = serve.Server(device=dev, memory_budget=150 * 10 ** 9)
        t = time.perf_counter()
        for r, g in zip(reqs, gaps):
            t += g
            r.arrival = t
            srv.submit(r)
        srv.run()
        st = srv.stats()
        per_rate['%g' % rate] = {'p50_step_ms': round(st['p50_step_ms'], 3), 'p99_step_ms': round(st['p99_step_ms'], 3),
                                 'steps_per_s': round(st['steps_per_s'], 2), 'steps': st['steps'],
                                 'requests': st['requests'], 'ticks': st['ticks']}
        all_scenes += scenes
        all_reqs += reqs
    # the highest rate again with no fragment cache: the same requests, each
    # holding less device memory, with a backward that recomputes its
    # fragment lists
    rate = rates[-1]
    gen = torch.Generator().manual_seed(7 + len(rates) - 1)
    gaps = torch.empty(num_requests).exponential_(rate, generator=gen).tolist()
    kw = [dict(seed=sp['seed']) for (_, _, _, _, _, sp) in scenes]
    on = [serve.Request(dvg.RenderFunction.serialize_scene(w, h, shapes, groups), target, sp['steps'], **k)
          for (w, h, shapes, groups, target, sp), k in zip(scenes, kw)]
    off = [serve.Request(dvg.RenderFunction.serialize_scene(w, h, shapes, groups), target, sp['steps'],
                         fragment_cache=False, **k) for (w, h, shapes, groups, target, sp), k in zip(scenes, kw)]
    srv = serve.Server(device=dev, memory_budget=150 * 10 ** 9)
    t = time.perf_counter()
    for r, g in zip(off, gaps):
        t += g
        r.arrival = t
        srv.submit(r)
    srv.run()
    st = srv.stats()
    cache_off = {'rate_per_s': rate, 'p50_step_ms': round(st['p50_step_ms'], 3),
                 'p99_step_ms': round(st['p99_step_ms'], 3), 'steps_per_s': round(st['steps_per_s'], 2),
                 'steps': st['steps'],
                 'mean_request_bytes': int(sum(r.device_bytes() for r in off) / len(off)),
                 'mean_request_bytes_with_cache': int(sum(r.device_bytes() for r in on) / len(on)),
                 # the same request with and without the cache, at step plain_steps + 1 (the
                 # trajectories then part by the order of the atomic sums, as any two runs do)
                 'max_rel_loss_diff_vs_cache': float('%.3g' % max(
                     abs(a.losses[plain_steps] - b.losses[plain_steps]) / max(abs(b.losses[plain_steps]), 1e-12)
                     for a, b in zip(off, reqs))),
                 'loss_diff_step': plain_steps + 1}
    # plain per-call path, one request at a time: a warm-up step (packing,
    # scene handle), then plain_steps timed steps; the loss of step
    # plain_steps + 1 is compared with the served request's
    done, t_plain, rel = 0, 0.0, []
    for (w, h, shapes, groups, target, sp), req in zip(all_scenes, all_reqs):
        ps = []
        for sh in shapes:
            sh.points = sh.points.to(dev).detach().requires_grad_(True)
            sh.stroke_width = sh.stroke_width.to(dev).detach().requires_grad_(True)
            ps += [sh.points, sh.stroke_width]
        for g in groups:
            for attr in ('fill_color', 'stroke_color'):
                c = getattr(g, attr)
                if isinstance(c, torch.Tensor):
                    setattr(g, attr, c.to(dev).detach().requires_grad_(True))
                    ps.append(getattr(g, attr))
        opt = torch.optim.Adam(ps, lr=1e-2)

        def plain_step():
            opt.zero_grad()
            a = dvg.RenderFunction.serialize_scene(w, h, shapes, groups)
            img = dvg.RenderFunction.apply(w, h, 2, 2, sp['seed'], None, *a)
            loss = ((img - target) ** 2).mean()
            loss.backward()
            opt.step()
            return loss.detach()
        plain_step()
        torch.cuda.synchronize(dev)
        t1 = time.perf_counter()
        for _ in range(plain_steps):
            loss = plain_step()
        torch.cuda.synchronize(dev)
        t_plain += time.perf_counter() - t1
        done += plain_steps
        lp = float(loss)
        ls = req.losses[plain_steps]
        rel.append(abs(ls - lp) / max(abs(lp), 1e-12))
    plain_sps = done / t_plain
    best = max(v['steps_per_s'] for v in per_rate.values())
    return {'workload': 'per arrival rate: %d requests (a subsample), canvases {128,256,512}^2, %d-%d paths (half open '
                        'strokes, half closed fills), %d-%d Adam steps each, Poisson arrivals, 150 GB admission '
                        'budget' % (num_requests, path_range[0], path_range[1], step_range[0], step_range[1]),
            'rates_per_s': list(rates), 'by_rate': per_rate,
            'plain_steps_per_s': round(plain_sps, 2),
            'speedup_vs_plain': {r: round(v['steps_per_s'] / plain_sps, 2) for r, v in per_rate.items()},
            'best_speedup_vs_plain': round(best / plain_sps, 2),
            'fragment_cache_off': cache_off,
            'equal_error_check': {'step': plain_steps + 1, 'requests': len(rel),
                                  'max_rel_loss_diff': float('%.3g' % max(rel))}}


def oracle_params(packed):
    import oracle
    return oracle.params_of(packed)


def cpu_baseline(packed, P, w, h, nsx, nsy, seed, target, threads=None, min_seconds=0.0):
    """Full fwd+bwd steps of the workload on the host cores with the oracle
    port: one step, or as many as fill min_seconds."""
    import numpy as np
    import oracle
    threads = threads or os.cpu_count() or 1
    steps = 0
    t0 = time.perf_counter()
    while True:
        fwd = oracle.render(packed, P, w, h, nsx, nsy, seed, num_threads=threads)
        d_img = (2.0 / fwd['image'].size) * (fwd['image'] - target)
        oracle.render(packed, P, w, h, nsx, nsy, seed, forward=False, d_image=d_img.astype(np.float32),
                      num_threads=threads)
        steps += 1
        dt = time.perf_counter() - t0
        if dt >= min_seconds:
            break
    n = w * h * nsx * nsy
    return {'value': round(n * steps / dt / 1e6, 4), 'unit': UNIT, 'cores': threads, 'kind': 'port',
            'sample': '%d full fwd+bwd step(s) of the workload (%d samples each), %.2f s' % (steps, n, dt)}


def run_reference(args):
    ws, rank, local = _dist()
    if rank != 0:
        return
    import numpy as np
    import torch
    import diffvg_gb300 as dvg
    from diffvg_gb300.packing import pack_scene
    import oracle
    (w, h, shapes, groups), (tw, th, tshapes, tgroups) = build_workload(dvg, None)
    nsx, nsy = WORKLOAD['spp']
    seed = WORKLOAD['seed']
    packed = pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups))
    P = oracle.params_of(packed)
    tpacked = pack_scene(dvg.RenderFunction.serialize_scene(tw, th, tshapes, tgroups))
    threads = os.cpu_count() or 1
    target = oracle.render(tpacked, oracle.params_of(tpacked), w, h, nsx, nsy, seed, num_threads=threads)['image']
    cpu_baseline(packed, P, w, h, nsx, nsy, seed, target, threads)  # one untimed warm-up step
    budget_s = 120.0
    times = []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        cpu_baseline(packed, P, w, h, nsx, nsy, seed, target, threads)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_all > budget_s:
            break
    total = sum(times)
    n = w * h * nsx * nsy
    value = n * len(times) / total / 1e6
    out = {'metric': METRIC, 'value': round(value, 4), 'unit': UNIT, 'n_gpus': ws, 'steps': len(times),
           'warmup': 1, 'ms_per_step': round(total / len(times) * 1e3, 2), 'higher_is_better': True,
           'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32 (fp64 root solves)', 'data': 'synthetic',
           'config': _workload_config(), 'impl': 'reference',
           'cpu_baseline': {'value': round(value, 4), 'unit': UNIT, 'cores': threads, 'kind': 'port',
                            'sample': 'full fwd+bwd steps of the workload on all host cores; the timed loop '
                                      'stops after %d s' % int(budget_s)},
           'e2e': {'value': round(value, 4), 'unit': UNIT, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
           'note': "the reference's own CPU module needs pybind11 and the reference checkout, neither of which "
                   "exists on the GPU host; the oracle port (oracle/dvg_oracle.c) restates its algorithm"}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=5)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--no-batched', action='store_true')
    ap.add_argument('--profile', action='store_true',
                    help='only the device-resident steps (for ncu captures): no e2e, batched, served or CPU legs')
    ap.add_argument('--config', choices=list(CONFIG_NAMES),
                    help='only this single-scene configuration (for ncu captures): target render, 3 warm-up '
                         'and 5 timed fwd+bwd steps')
    args = ap.parse_args()
    if args.config:
        import torch
        print(json.dumps({'configs': run_configs(torch.device('cuda', 0), only=args.config, cpu=False)}))
        return
    if args.profile:
        args.no_batched = args.no_cpu_baseline = True
        args.no_e2e = True
    if args.impl == 'reference':
        run_reference(args)
    else:
        run_ours(args)


if __name__ == '__main__':
    main()
