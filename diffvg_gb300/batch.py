"""Batched optimisation: many independent scenes stepped together on one GPU.

The reference optimises one scene per Python loop iteration: serialise,
build the scene on the host, render, back-propagate, copy every gradient
back to host tensors, take a torch optimiser step (apps/painterly_rendering
.py:146-192; apps/generative_models/rendering.py:46-95 loops over scenes).
Here a batch of scenes keeps everything resident on the device:

  * each scene's topology lives in its own DvgScene handle (uploaded once);
  * all scenes' parameters form one device buffer (each scene's arena is a
    16-byte aligned slice), with one gradient buffer and the Adam moments of
    the same layout;
  * one CUDA graph replays, per scene, forward render -> MSE gradient against
    the scene's target -> backward render, with the scenes spread over
    several streams so that small scenes overlap on the GPU, then one Adam
    update over the whole parameter buffer (dvg_adam_step).

A step is one graph replay; there is no host work per scene.  Failures the
kernels latch while the graph runs (a tile list outgrowing its capacity as
shapes move) are checked every `check_every` steps; a grown tile list makes
the graph be captured again.

Two ways to run the scenes' render passes inside the step:
  * mode 'streams': per-scene launches spread over several streams;
  * mode 'persistent': the forward sample pass, the interior adjoint and the
    boundary pass of all scenes each run as one persistent launch over a
    (scene, tile) work queue, largest scenes first (dvg_batch_forward /
    dvg_batch_backward), tuned by resident blocks per SM and samples per
    thread.
autotune() times the candidates on the batch itself and keeps the fastest;
its choice is cached in a JSON file by GPU and workload.
"""
import hashlib
import json
import os

import torch

from . import _native
from .packing import pack_scene

# parameter kinds that an optimisation step updates by default
DEFAULT_TRAINABLE = ('points', 'thickness', 'stroke_width', 'color', 'radius', 'center', 'corner',
                     'gradient_geometry')


def _align4(n):
    return (n + 3) // 4 * 4


class BatchedScenes:
    """A batch of scenes optimised against per-scene target images.

    scene_args: list of RenderFunction.serialize_scene argument lists.
    sizes: list of (width, height) render sizes (default: canvas sizes).
    targets: list of [H, W, 4] target images (any device), or None to set
        later with set_targets().
    """

    def __init__(self, scene_args, num_samples=(2, 2), seeds=None, sizes=None, targets=None, lr=1e-2,
                 betas=(0.9, 0.999), eps=1e-8, trainable=DEFAULT_TRAINABLE, streams=8, check_every=16,
                 device=None, mode='streams', tuning=(2, 1), fragment_cache=True):
        self.device = device or torch.device('cuda', torch.cuda.current_device())
        self.nsx, self.nsy = num_samples
        self.packed = [pack_scene(a) for a in scene_args]
        n = len(self.packed)
        self.seeds = list(seeds) if seeds is not None else list(range(n))
        self.sizes = list(sizes) if sizes is not None else [(p.canvas_width, p.canvas_height) for p in self.packed]
        self.lr, self.betas, self.eps = float(lr), betas, float(eps)
        self.check_every = check_every
        # False: no per-sample fragment cache between a scene's forward and
        # backward (the backward recomputes the fragment lists)
        self.fragment_cache = bool(fragment_cache)
        with torch.cuda.device(self.device):
            self.scenes = [_native.NativeScene(p) for p in self.packed]
        self.offsets = []
        off = 0
        for p in self.packed:
            self.offsets.append(off)
            off += _align4(max(p.num_params, 1))
        self.num_params = off
        dev = self.device
        self.params = torch.zeros(off, device=dev)
        self.lr_scale = torch.zeros(off, device=dev)
        for p, o in zip(self.packed, self.offsets):
            self.params[o:o + p.num_params] = p.param_arena(dev)[:p.num_params]
            for sl in p.slots:
                if sl.differentiable and sl.kind in trainable:
                    self.lr_scale[o + sl.offset:o + sl.offset + sl.numel] = 1.0
        self.grads = torch.zeros(off, device=dev)
        self.m = torch.zeros(off, device=dev)
        self.v = torch.zeros(off, device=dev)
        self.step_count = torch.zeros(1, dtype=torch.int32, device=dev)
        self.images = [torch.zeros(h, w, 4, device=dev) for (w, h) in self.sizes]
        self.d_images = [torch.zeros(h, w, 4, device=dev) for (w, h) in self.sizes]
        self.targets = [torch.zeros(h, w, 4, device=dev) for (w, h) in self.sizes]
        self.losses = torch.zeros(n, device=dev)
        self.streams = [torch.cuda.Stream(device=dev) for _ in range(max(1, min(streams, n)))]
        self.graph = None
        self.steps_taken = 0
        self.native_batch = None
        self.set_mode(mode, tuning)
        if targets is not None:
            self.set_targets(targets)

    def set_mode(self, mode, tuning=(2, 1)):
        """'streams' or 'persistent' (with tuning = (blocks per SM, samples
        per thread)); the next step captures its graph again."""
        if mode not in ('streams', 'persistent'):
            raise ValueError('mode must be streams or persistent')
        if mode == 'persistent' and self.native_batch is None:
            self.native_batch = _native.NativeBatch(self.scenes)
        self.mode = mode
        self.tuning = _native.BatchTuning(int(tuning[0]), int(tuning[1]))
        self.graph = None

    @property
    def num_scenes(self):
        return len(self.packed)

    def samples_per_step(self):
        return sum(w * h * self.nsx * self.nsy for (w, h) in self.sizes)

    def scene_params(self, i):
        """View of scene i's parameter arena (the layout of its packed scene)."""
        return self.params[self.offsets[i]:self.offsets[i] + self.packed[i].num_params]

    def _args(self, i, flags, params=None):
        if not self.fragment_cache:
            flags |= _native.DVG_FLAG_NO_FRAG_CACHE
        w, h = self.sizes[i]
        p = self.scene_params(i) if params is None else params
        return _native.RenderArgs(w, h, self.nsx, self.nsy, int(self.seeds[i]) & (2 ** 64 - 1),
                                  1 if self.packed[i].use_prefiltering else 0, 0, p.data_ptr(), None, None, flags)

    def set_targets(self, targets):
        for t, dst in zip(targets, self.targets):
            dst.copy_(t.to(self.device, torch.float32).reshape(dst.shape))

    def render(self, i, params=None):
        """Synchronous forward render of scene i (optionally with other parameters)."""
        out = torch.empty_like(self.images[i])
        p = self.scene_params(i) if params is None else params.to(self.device).contiguous()
        self.scenes[i].forward(self._args(i, 0, p), image_ptr=out.data_ptr(),
                               stream=torch.cuda.current_stream(self.device).cuda_stream)
        return out

    def _enqueue(self, i, stream):
        sp = stream.cuda_stream
        sc = self.scenes[i]
        o, n = self.offsets[i], self.packed[i].num_params
        sc.forward(self._args(i, _native.DVG_FLAG_NO_SYNC), image_ptr=self.images[i].data_ptr(), stream=sp)
        _native.mse_grad(self.images[i], self.targets[i], self.d_images[i], self.losses[i:i + 1], stream=sp)
        self.grads[o:o + n].zero_()
        sc.backward(self._args(i, _native.DVG_FLAG_NO_SYNC | _native.DVG_FLAG_REUSE_PREP),
                    d_image_ptr=self.d_images[i].data_ptr(), d_params_ptr=self.grads[o:o + n].data_ptr(), stream=sp)

    def _step_body(self):
        if self.mode == 'persistent':
            return self._step_body_persistent()
        main = torch.cuda.current_stream(self.device)
        self.losses.zero_()
        for st in self.streams:
            st.wait_stream(main)
        for i in range(self.num_scenes):
            st = self.streams[i % len(self.streams)]
            with torch.cuda.stream(st):
                self._enqueue(i, st)
        for st in self.streams:
            main.wait_stream(st)
        _native.adam_step(self.params, self.grads, self.m, self.v, self.step_count, self.lr, self.betas, self.eps,
                          lr_scale=self.lr_scale, stream=main.cuda_stream)

    def _step_body_persistent(self):
        main = torch.cuda.current_stream(self.device)
        sp = main.cuda_stream
        n = self.num_scenes
        self.losses.zero_()
        self.native_batch.forward([self._args(i, _native.DVG_FLAG_NO_SYNC) for i in range(n)],
                                  [im.data_ptr() for im in self.images], self.tuning, stream=sp)
        for i in range(n):
            _native.mse_grad(self.images[i], self.targets[i], self.d_images[i], self.losses[i:i + 1], stream=sp)
        self.grads.zero_()
        flags = _native.DVG_FLAG_NO_SYNC | _native.DVG_FLAG_REUSE_PREP
        self.native_batch.backward([self._args(i, flags) for i in range(n)], [d.data_ptr() for d in self.d_images],
                                   [self.grads[o:o + 1].data_ptr() for o in self.offsets], self.tuning, stream=sp)
        _native.adam_step(self.params, self.grads, self.m, self.v, self.step_count, self.lr, self.betas, self.eps,
                          lr_scale=self.lr_scale, stream=sp)

    def workload_key(self):
        """GPU name and a hash of the batch's scene and image sizes: the key of
        the autotuner's cache."""
        h = hashlib.blake2b(digest_size=8)
        h.update(repr(sorted((w, h_, self.nsx, self.nsy, p.num_shapes, int(p.segment_ctrl.size))
                             for (w, h_), p in zip(self.sizes, self.packed))).encode())
        return '%s|%s' % (torch.cuda.get_device_name(self.device), h.hexdigest())

    def autotune(self, candidates=None, steps=3, cache_path=None):
        """Times each candidate (mode, tuning) for `steps` graph replays on this
        batch, keeps the fastest, and returns {candidate: ms per step}.  The
        optimiser state is restored afterwards.  Choices are cached in
        cache_path (default: $DVG_AUTOTUNE_CACHE, else autotune.json beside the
        library) by workload_key(); a cached choice is used without timing."""
        if cache_path is None:
            cache_path = os.environ.get('DVG_AUTOTUNE_CACHE') or os.path.join(
                os.path.dirname(_native.library_path()), 'autotune.json')
        if candidates is None:
            candidates = [('streams', (2, 1))] + [('persistent', (c, t)) for c in (1, 2) for t in (1, 2, 4)]
        key = self.workload_key()
        cache = {}
        if os.path.exists(cache_path):
            try:
                with open(cache_path) as f:
                    cache = json.load(f)
            except (OSError, ValueError):
                cache = {}
        if key in cache:
            mode, tuning = cache[key]['mode'], tuple(cache[key]['tuning'])
            self.set_mode(mode, tuning)
            return dict(cache[key].get('timings_ms', {}))
        saved = (self.params.clone(), self.m.clone(), self.v.clone(), self.step_count.clone(), self.steps_taken)
        timings = {}
        for mode, tuning in candidates:
            self.set_mode(mode, tuning)
            self.step()  # capture and warm up
            torch.cuda.synchronize(self.device)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(steps):
                self.graph.replay()
            e1.record()
            torch.cuda.synchronize(self.device)
            timings['%s %d %d' % (mode, tuning[0], tuning[1])] = e0.elapsed_time(e1) / steps
        self.params.copy_(saved[0]); self.m.copy_(saved[1]); self.v.copy_(saved[2])
        self.step_count.copy_(saved[3])
        self.steps_taken = saved[4]
        best = min(timings, key=timings.get)
        mode, c, t = best.split()
        self.set_mode(mode, (int(c), int(t)))
        cache[key] = {'mode': mode, 'tuning': [int(c), int(t)], 'timings_ms': timings}
        try:
            os.makedirs(os.path.dirname(os.path.abspath(cache_path)), exist_ok=True)
            with open(cache_path, 'w') as f:
                json.dump(cache, f, indent=1, sort_keys=True)
        except OSError:
            pass
        return timings

    def check(self):
        """Waits for the device and raises a latched failure; returns True if
        a tile list was grown (the graph must be captured again)."""
        grown = False
        for sc in self.scenes:
            try:
                sc.sync(torch.cuda.current_stream(self.device).cuda_stream)
            except _native.SceneCapacityError as e:
                if 'grown' in str(e):
                    grown = True
                else:
                    raise
        return grown

    def warmup(self):
        """Synchronous calls that size every scene's arenas and tile lists
        (nothing may be allocated while the graph is captured)."""
        with torch.cuda.device(self.device):
            sp = torch.cuda.current_stream(self.device).cuda_stream
            for i, sc in enumerate(self.scenes):
                o, n = self.offsets[i], self.packed[i].num_params
                sc.forward(self._args(i, 0), image_ptr=self.images[i].data_ptr(), stream=sp)
                sc.backward(self._args(i, 0), d_image_ptr=self.d_images[i].data_ptr(),
                            d_params_ptr=self.grads[o:o + n].data_ptr(), stream=sp)
            self.grads.zero_()
            torch.cuda.synchronize(self.device)

    def capture(self):
        self.warmup()
        with torch.cuda.device(self.device):
            # one eager step on the side streams so that lazily created state exists before capture
            s = torch.cuda.Stream(device=self.device)
            s.wait_stream(torch.cuda.current_stream(self.device))
            with torch.cuda.stream(s):
                saved = (self.params.clone(), self.m.clone(), self.v.clone(), self.step_count.clone())
                self._step_body()
                self.params.copy_(saved[0]); self.m.copy_(saved[1]); self.v.copy_(saved[2])
                self.step_count.copy_(saved[3])
            torch.cuda.current_stream(self.device).wait_stream(s)
            torch.cuda.synchronize(self.device)
            self.check()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=s):
                self._step_body()
            self.graph = g

    def step(self):
        """One optimisation step of every scene (one graph replay)."""
        if self.graph is None:
            self.capture()
        self.graph.replay()
        self.steps_taken += 1
        if self.check_every and self.steps_taken % self.check_every == 0:
            if self.check():
                self.graph = None

    def step_eager(self):
        """The same step without the graph (for tests and debugging)."""
        self._step_body()
        self.steps_taken += 1

    def loss(self):
        """Per-scene mean squared error of the last step (host floats)."""
        return [float(l) / self.images[i].numel() for i, l in enumerate(self.losses.cpu())]
