"""Serving loop: continuous batching of render-and-optimise requests.

A request is a scene (RenderFunction.serialize_scene argument list), a
target image and a number of Adam steps.  The server keeps a set of active
slots on the device.  A slot holds everything a request needs between its
steps: the DvgScene handle (topology, derived scene data, tile lists,
per-sample and boundary-sample arenas), the parameter arena, its gradient,
the Adam moments, the rendered / target / adjoint images, and a CUDA graph
of one optimisation step (forward, MSE gradient, backward, Adam), captured
when the slot is admitted.

The loop runs in ticks.  Each tick replays the graph of every active slot,
spread over several streams so that the slots' kernels overlap on the GPU,
and waits for all of them; every active request advances by one step.
Between ticks, requests that have arrived are admitted while slots and the
device-memory budget allow (each request's device bytes are estimated from
its scene and image size before anything is allocated), and finished
requests are retired, which frees their memory for the next admissions.
A request admitted while others are mid-way joins the next tick.

Per-step latency is the duration of the tick a step ran in (CUDA events);
the server reports p50 / p99 over all request-steps and aggregate steps/s.
"""
import collections
import threading
import time

import torch

from . import _native
from .batch import DEFAULT_TRAINABLE
from .diffvg import ShapeType
from .packing import pack_scene


def mean_depth(packed):
    """Mean number of groups whose canvas bounding box (shapes' boxes
    grown by their stroke widths, through the group transform) covers a
    canvas point: an upper-leaning estimate of the hits per sample."""
    import numpy as np
    W, H = float(packed.canvas_width), float(packed.canvas_height)
    if packed.num_groups == 0 or W <= 0 or H <= 0:
        return 0.0
    P = np.concatenate([t.detach().reshape(-1).float().cpu().numpy() for t in packed.tensors]) \
        if packed.tensors else np.zeros(1, np.float32)
    si, gi, gs = packed.shape_info, packed.group_info, packed.group_shapes
    boxes = np.zeros((packed.num_shapes, 4))
    for s in range(packed.num_shapes):
        kind, po, npts = int(si[s, 0]), int(si[s, 1]), int(si[s, 2])
        if kind == ShapeType.circle:
            r, c = abs(P[po]), P[po + 1:po + 3]
            b = [c[0] - r, c[1] - r, c[0] + r, c[1] + r]
        elif kind == ShapeType.ellipse:
            r, c = np.abs(P[po:po + 2]), P[po + 2:po + 4]
            b = [c[0] - r[0], c[1] - r[1], c[0] + r[0], c[1] + r[1]]
        elif kind == ShapeType.path and npts > 0:
            pts = P[po:po + 2 * npts].reshape(-1, 2)
            b = [*pts.min(0), *pts.max(0)]
        elif kind == ShapeType.rect:
            b = [*np.minimum(P[po:po + 2], P[po + 2:po + 4]), *np.maximum(P[po:po + 2], P[po + 2:po + 4])]
        else:
            b = [0.0, 0.0, 0.0, 0.0]
        sw = abs(P[int(si[s, 7])]) if int(si[s, 7]) >= 0 else 0.0
        boxes[s] = [b[0] - sw, b[1] - sw, b[2] + sw, b[3] + sw]
    area = 0.0
    for g in range(packed.num_groups):
        n, off = int(gi[g, 0]), int(gi[g, 1])
        if n == 0:
            continue
        bb = boxes[gs[off:off + n]]
        lo, hi = bb[:, :2].min(0), bb[:, 2:].max(0)
        m = P[int(gi[g, 9]):int(gi[g, 9]) + 9].reshape(3, 3)
        corners = np.array([[lo[0], lo[1], 1], [hi[0], lo[1], 1], [lo[0], hi[1], 1], [hi[0], hi[1], 1]]) @ m.T
        w = corners[:, 2:3]
        if np.any(np.abs(w) < 1e-12):
            area += W * H
            continue
        c = corners[:, :2] / w
        x0, y0 = max(c[:, 0].min(), 0.0), max(c[:, 1].min(), 0.0)
        x1, y1 = min(c[:, 0].max(), W), min(c[:, 1].max(), H)
        area += max(x1 - x0, 0.0) * max(y1 - y0, 0.0)
    return area / (W * H)


def estimate_device_bytes(packed, width, height, spp, fragment_cache=True):
    """Device bytes a request holds while resident (without the per-sample
    fragment cache when `fragment_cache` is False)."""
    npx, n = width * height, width * height * spp
    P = max(packed.num_params, 1)
    nseg, ns, ng = packed.segment_ctrl.size, packed.num_shapes, packed.num_groups
    tiles = ((packed.canvas_width + 15) // 16) * ((packed.canvas_height + 15) // 16)
    params = 4 * P * 6                              # params, grads, m, v, lr scale, spare
    images = 16 * npx * 3 + 4 * npx                 # image, adjoint, target; weight image
    # forward sample colours; fragment cache per sample: 16 hit keys, or with
    # prefiltering 16 fragments of 64 B, and a count; each sample's first
    # chunk for the entries past 16, and the chunks: of 16 keys (68 B) one per
    # two samples, of 16 fragments (1028 B) one per sixteen, or as many as
    # twice the mean box depth asks for (up to what the reference's maximum
    # fragment count needs); the backward's deep-pass list
    ask = (2.0 * mean_depth(packed) - 16.0) / 16.0
    if packed.use_prefiltering:
        cache = 16 * 64 + 4 + int(1028 * min(3.0, max(1.0 / 16.0, ask)) + 0.5)
    else:
        cache = 16 * 4 + 4 + int(68 * min(15.0, max(0.5, ask)) + 0.5)
    cache = cache + 2 if fragment_cache else 0
    samples = 16 * n + (cache + 4) * n
    edges = 68 * n                                  # boundary-sample records and ordering
    if ng >= 8:  # deferred fp64 walks: jobs, per-query state and colours, fragments, deferred samples,
        # the jobs' quintics and root brackets
        edges += 32 * n + 2 * (16 + 4 + 16) * n + 4 * 8 * n + 4 * n + 40 * n + 2 * 16 * n
    scene = 4 * (8 * ns + 12 * ng + 2 * nseg + 2 * ng) + 64 * ng + 40 * ns + 48 * nseg + 4 * (10 * nseg + 8 * ns)
    scene += (8 * 33 + 4 * 64) * nseg                # tabulated subdivision trees of the segments
    tile_lists = 4 * max(65536, 32 * tiles) * 5 // 4 + 8 * tiles
    return int(params + images + samples + edges + scene + tile_lists + (1 << 20))


class Request:
    """A render-and-optimise request."""

    _ids = 0

    def __init__(self, scene_args, target, steps, num_samples=(2, 2), seed=0, lr=1e-2, betas=(0.9, 0.999),
                 eps=1e-8, trainable=DEFAULT_TRAINABLE, size=None, arrival=None, fragment_cache=True):
        Request._ids += 1
        self.id = Request._ids
        self.scene_args = scene_args
        self.target = target
        self.steps = int(steps)
        self.num_samples = num_samples
        self.seed = seed
        self.lr, self.betas, self.eps = lr, betas, eps
        self.trainable = trainable
        # False: the forward keeps no per-sample fragment cache and the
        # backward recomputes each sample's fragment list (less memory per
        # request, a slower backward)
        self.fragment_cache = bool(fragment_cache)
        self.packed = pack_scene(scene_args)
        self.size = size or (self.packed.canvas_width, self.packed.canvas_height)
        self.arrival = arrival
        self.admitted = None
        self.finished = None
        self.losses = []
        self.result = None       # final parameter arena (host tensor)
        self.step_ms = []

    @classmethod
    def from_svg(cls, filename, target, steps, use_prefiltering=False, **kw):
        """A request whose scene is read from an SVG file (svg_to_scene); the
        other arguments are those of Request."""
        from .parse_svg import svg_to_scene
        from .render_pytorch import RenderFunction
        w, h, shapes, groups = svg_to_scene(filename)
        args = RenderFunction.serialize_scene(w, h, shapes, groups, use_prefiltering=use_prefiltering)
        return cls(args, target, steps, **kw)

    def device_bytes(self):
        return estimate_device_bytes(self.packed, self.size[0], self.size[1],
                                     self.num_samples[0] * self.num_samples[1], self.fragment_cache)


class Slot:
    """The resident state of one admitted request."""

    def __init__(self, req, device, stream):
        self.req = req
        self.device = device
        w, h = req.size
        p = req.packed
        with torch.cuda.device(device):
            self.scene = _native.NativeScene(p)
        n = max(p.num_params, 1)
        self.params = p.param_arena(device)[:n].contiguous().clone()
        self.grads = torch.zeros(n, device=device)
        self.m = torch.zeros(n, device=device)
        self.v = torch.zeros(n, device=device)
        self.lr_scale = torch.zeros(n, device=device)
        for sl in p.slots:
            if sl.differentiable and sl.kind in req.trainable:
                self.lr_scale[sl.offset:sl.offset + sl.numel] = 1.0
        self.step_count = torch.zeros(1, dtype=torch.int32, device=device)
        self.image = torch.zeros(h, w, 4, device=device)
        self.d_image = torch.zeros(h, w, 4, device=device)
        self.target = req.target.to(device=device, dtype=torch.float32).reshape(h, w, 4).contiguous()
        self.loss = torch.zeros(1, device=device)
        self.stream = stream
        self.graph = None
        self.done = 0
        self._capture()

    def _args(self, flags):
        if not self.req.fragment_cache:
            flags |= _native.DVG_FLAG_NO_FRAG_CACHE
        w, h = self.req.size
        nsx, nsy = self.req.num_samples
        return _native.RenderArgs(w, h, nsx, nsy, int(self.req.seed) & (2 ** 64 - 1),
                                  1 if self.req.packed.use_prefiltering else 0, 0, self.params.data_ptr(), None, None,
                                  flags)

    def _body(self):
        sp = torch.cuda.current_stream(self.device).cuda_stream
        self.loss.zero_()
        self.scene.forward(self._args(_native.DVG_FLAG_NO_SYNC), image_ptr=self.image.data_ptr(), stream=sp)
        _native.mse_grad(self.image, self.target, self.d_image, self.loss, stream=sp)
        self.grads.zero_()
        self.scene.backward(self._args(_native.DVG_FLAG_NO_SYNC | _native.DVG_FLAG_REUSE_PREP),
                            d_image_ptr=self.d_image.data_ptr(), d_params_ptr=self.grads.data_ptr(), stream=sp)
        _native.adam_step(self.params, self.grads, self.m, self.v, self.step_count, self.req.lr, self.req.betas,
                          self.req.eps, lr_scale=self.lr_scale, stream=sp)

    def _capture(self):
        dev = self.device
        with torch.cuda.device(dev), torch.cuda.stream(self.stream):
            # synchronous calls size every arena and the tile lists before
            # capture (nothing may be allocated while the graph is captured)
            sp = self.stream.cuda_stream
            self.scene.forward(self._args(0), image_ptr=self.image.data_ptr(), stream=sp)
            self.scene.backward(self._args(0), d_image_ptr=self.d_image.data_ptr(), d_params_ptr=self.grads.data_ptr(),
                                stream=sp)
            self.grads.zero_()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=self.stream):
                self._body()
            self.graph = g

    def launch(self):
        with torch.cuda.stream(self.stream):
            self.graph.replay()

    def check(self):
        try:
            self.scene.sync(self.stream.cuda_stream)
        except _native.SceneCapacityError as e:
            if 'grown' not in str(e):
                raise
            # a tile list outgrew its capacity (shapes moved) and was grown:
            # the graph is captured again.  The steps since the last check
            # rendered this slot without gradient (their Adam updates used
            # the moments only) and are not counted as done.
            self.graph = None
            self._capture()
            return False
        return True

    def release(self):
        self.scene.close()
        self.graph = None


class Server:
    """Continuous-batching request loop on one GPU."""

    def __init__(self, device=None, memory_budget=150 * 10 ** 9, max_slots=64, streams=8, check_every=8):
        self.device = device or torch.device('cuda', torch.cuda.current_device())
        self.budget = int(memory_budget)
        self.max_slots = max_slots
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(streams)]
        self.check_every = check_every
        self.pending = collections.deque()
        self.lock = threading.Lock()
        self.active = []
        self.bytes_in_use = 0
        self.completed = []
        self.rejected = []
        self.tick_ms = []
        self.ticks = 0
        self._rr = 0

    def submit(self, req):
        """Queues a request; it is admitted at the next tick that has room.
        A request whose estimated bytes exceed the whole budget is rejected."""
        if req.device_bytes() > self.budget:
            self.rejected.append(req)
            return False
        if req.arrival is None:
            req.arrival = time.perf_counter()
        with self.lock:
            self.pending.append(req)
        return True

    def _admit(self, now):
        with self.lock:
            while self.pending and len(self.active) < self.max_slots:
                req = self.pending[0]
                if req.arrival is not None and req.arrival > now:
                    break
                b = req.device_bytes()
                if self.bytes_in_use + b > self.budget:
                    break
                self.pending.popleft()
                stream = self.streams[self._rr % len(self.streams)]
                self._rr += 1
                req.admitted = now
                req.bytes = b
                self.active.append(Slot(req, self.device, stream))
                self.bytes_in_use += b

    def _retire(self, now):
        keep = []
        for sl in self.active:
            if sl.done >= sl.req.steps:
                sl.req.result = sl.params.detach().cpu()
                sl.req.finished = now
                self.bytes_in_use -= sl.req.bytes
                sl.release()
                self.completed.append(sl.req)
            else:
                keep.append(sl)
        self.active = keep

    def tick(self):
        """Admits what fits, runs one step of every active request, retires
        finished requests.  Returns the number of steps run."""
        now = time.perf_counter()
        self._admit(now)
        if not self.active:
            return 0
        main = torch.cuda.current_stream(self.device)
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(main)
        for st in self.streams:
            st.wait_stream(main)
        for sl in self.active:
            sl.launch()
        for st in self.streams:
            main.wait_stream(st)
        end.record(main)
        losses = torch.cat([sl.loss for sl in self.active]).cpu()  # waits for the tick
        ms = start.elapsed_time(end)
        self.ticks += 1
        self.tick_ms.append(ms)
        redo = set()
        if self.check_every and self.ticks % self.check_every == 0:
            for sl in self.active:
                if not sl.check():
                    redo.add(id(sl))
        for sl, l in zip(self.active, losses.tolist()):
            if id(sl) in redo:
                continue
            sl.done += 1
            sl.req.step_ms.append(ms)
            sl.req.losses.append(l / sl.image.numel())
        n = len(self.active) - len(redo)
        self._retire(time.perf_counter())
        return n

    def run(self, until_idle=True, max_seconds=None):
        """Ticks until every submitted request is done (or time runs out)."""
        t0 = time.perf_counter()
        steps = 0
        while True:
            if max_seconds is not None and time.perf_counter() - t0 > max_seconds:
                break
            n = self.tick()
            steps += n
            if n == 0:
                with self.lock:
                    idle = not self.pending
                if idle and not self.active and until_idle:
                    break
                if not idle:
                    nxt = self.pending[0].arrival
                    delay = (nxt - time.perf_counter()) if nxt is not None else 0
                    if delay > 0:
                        time.sleep(min(delay, 0.01))
        return steps

    def stats(self):
        lat = sorted(ms for r in self.completed for ms in r.step_ms)

        def pct(q):
            if not lat:
                return None
            return lat[min(len(lat) - 1, int(round(q * (len(lat) - 1))))]
        total_steps = sum(len(r.step_ms) for r in self.completed)
        span = None
        if self.completed:
            span = max(r.finished for r in self.completed) - min(r.admitted for r in self.completed)
        return {'requests': len(self.completed), 'rejected': len(self.rejected), 'steps': total_steps,
                'p50_step_ms': pct(0.5), 'p99_step_ms': pct(0.99),
                'steps_per_s': (total_steps / span) if span else None, 'ticks': self.ticks}
