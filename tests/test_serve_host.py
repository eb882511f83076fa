"""Host-side logic of the serving loop (admission by estimated device bytes,
slot limits, retirement, latency statistics) with the device work replaced
by a stand-in slot, so it runs without a GPU."""
import types

import pytest
import torch

import diffvg_gb300 as dvg
from diffvg_gb300 import serve, workloads


class FakeSlot:
    def __init__(self, req, device, stream):
        self.req = req
        self.done = 0
        self.image = torch.zeros(req.size[1], req.size[0], 4)
        self.loss = torch.zeros(1)
        self.params = torch.zeros(3)
        self.stream = stream

    def launch(self):
        pass

    def check(self):
        return True

    def release(self):
        pass


class FakeEvent:
    def __init__(self, **kw):
        pass

    def record(self, *a):
        pass

    def elapsed_time(self, other):
        return 2.0


class FakeStream:
    cuda_stream = 0

    def wait_stream(self, other):
        pass


@pytest.fixture
def server(monkeypatch):
    monkeypatch.setattr(serve, 'Slot', FakeSlot)
    monkeypatch.setattr(serve.torch.cuda, 'Event', FakeEvent)
    monkeypatch.setattr(serve.torch.cuda, 'Stream', lambda device=None: FakeStream())
    monkeypatch.setattr(serve.torch.cuda, 'current_stream', lambda device=None: FakeStream())

    def make(budget, max_slots=64):
        return serve.Server(device=torch.device('cpu'), memory_budget=budget, max_slots=max_slots, streams=2,
                            check_every=0)
    return make


def _req(seed, canvas, paths, steps):
    w, h, shapes, groups = workloads.stroke_scene(dvg, seed=seed, num_paths=paths, canvas=canvas)
    args = dvg.RenderFunction.serialize_scene(w, h, shapes, groups)
    return serve.Request(args, torch.zeros(h, w, 4), steps)


def test_estimate_grows_with_image_and_scene():
    a = _req(1, 64, 8, 1)
    b = _req(1, 128, 8, 1)
    c = _req(1, 128, 64, 1)
    assert a.device_bytes() < b.device_bytes() < c.device_bytes()


def test_estimate_counts_the_prefiltered_fragment_cache():
    """A prefiltered request caches 16 whole fragments of 64 B per sample for
    its backward pass and chunks for the fragments past 16 (1028 B per
    sixteen samples), a sampled one 16 fragment keys of 4 B and chunks for the
    keys past 16 (68 B per two samples); both keep each sample's first chunk."""
    from diffvg_gb300.packing import pack_scene
    w, h, shapes, groups = workloads.fill_scene(dvg, seed=3, num_paths=8, canvas=128)
    plain = pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups))
    pref = pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups, use_prefiltering=True))
    n = w * h
    diff = serve.estimate_device_bytes(pref, w, h, 1) - serve.estimate_device_bytes(plain, w, h, 1)
    assert diff == (16 * 64 + 64 - (16 * 4 + 34)) * n


def test_estimate_without_the_fragment_cache():
    """A request that keeps no fragment cache saves, per sample, the 16 keys,
    the first-chunk index, the count and the chunks; the prefiltered one the 16
    fragments, the index, the count and its chunks."""
    from diffvg_gb300.packing import pack_scene
    w, h, shapes, groups = workloads.fill_scene(dvg, seed=3, num_paths=8, canvas=128)
    for pf, per in ((False, 16 * 4 + 4 + 34 + 2), (True, 16 * 64 + 4 + 64 + 2)):
        p = pack_scene(dvg.RenderFunction.serialize_scene(w, h, shapes, groups, use_prefiltering=pf))
        on = serve.estimate_device_bytes(p, w, h, 1)
        off = serve.estimate_device_bytes(p, w, h, 1, fragment_cache=False)
        assert on - off == per * w * h
    args = dvg.RenderFunction.serialize_scene(w, h, shapes, groups)
    r_on = serve.Request(args, torch.zeros(h, w, 4), 1)
    r_off = serve.Request(args, torch.zeros(h, w, 4), 1, fragment_cache=False)
    assert r_off.device_bytes() < r_on.device_bytes()


def test_budget_serialises_requests_and_all_complete(server):
    reqs = [_req(i, 64, 8, 3) for i in range(4)]
    s = server(budget=int(reqs[0].device_bytes() * 1.5))
    for r in reqs:
        assert s.submit(r)
    max_active = 0
    while s.tick():
        max_active = max(max_active, len(s.active) + 1)
    s.run()
    assert len(s.completed) == 4
    assert all(len(r.step_ms) == 3 for r in reqs)
    # never more than one request resident under this budget
    assert max(r.admitted for r in reqs[1:]) >= min(r.finished for r in reqs[:1])


def test_oversized_request_is_rejected(server):
    s = server(budget=1000)
    assert not s.submit(_req(0, 64, 8, 1))
    assert s.stats()['rejected'] == 1


def test_late_request_joins_running_ones(server):
    s = server(budget=10 ** 12)
    a = _req(0, 64, 8, 5)
    s.submit(a)
    s.tick()
    s.tick()
    b = _req(1, 64, 8, 2)
    s.submit(b)
    assert s.tick() == 2          # both advance in the same tick
    s.run()
    assert a.finished is not None and b.finished is not None
    st = s.stats()
    assert st['steps'] == 7 and st['p50_step_ms'] == 2.0 and st['p99_step_ms'] == 2.0


def test_slot_limit(server):
    s = server(budget=10 ** 12, max_slots=2)
    for i in range(5):
        s.submit(_req(i, 64, 8, 2))
    assert s.tick() == 2


def test_request_from_svg_is_served(server, tmp_path):
    """A request read from an SVG file goes through admission and completes."""
    svg = tmp_path / 'req.svg'
    svg.write_text('<svg xmlns="http://www.w3.org/2000/svg" width="32" height="24">'
                   '<path d="M2 2 C10 0 20 8 28 20" fill="none" stroke="#ff0000" stroke-width="3"/>'
                   '<circle cx="16" cy="12" r="5" fill="blue"/></svg>')
    req = serve.Request.from_svg(str(svg), torch.zeros(24, 32, 4), 2)
    assert req.size == (32, 24) and req.packed.num_shapes == 2
    srv = server(budget=1 << 40)
    assert srv.submit(req)
    srv.run()
    assert srv.completed == [req] and len(req.step_ms) == 2
