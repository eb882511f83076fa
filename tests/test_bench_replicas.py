"""bench.py's multi-GPU mode is replicas: each rank renders its own copy of
the workload, throughput is whole-job (all ranks' samples over the slowest
rank's time), and the reference arm runs on rank 0 only.  Checked with two
gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    import torch
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE='2')
    dist.init_process_group('gloo', rank=rank, world_size=2)
    value, total_ms = bench.aggregate_throughput(100.0 + 50.0 * rank, 1_000_000, 4, 2, torch.device('cpu'))
    q.put((rank, value, total_ms))
    dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_rank():
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, total_ms in out:
        assert total_ms == pytest.approx(150.0)                      # max over ranks
        assert value == pytest.approx(2 * 1_000_000 * 4 / 0.150 / 1e6)  # all ranks' samples


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    import bench
    monkeypatch.setenv('RANK', '1')
    monkeypatch.setenv('WORLD_SIZE', '2')
    assert bench.run_reference(None) is None
    assert capsys.readouterr().out == ''


def test_issue_roofline_arithmetic():
    import bench
    r = bench.issue_roofline(4.2e9, 13.8e-3, 152, 2070.0)
    assert r['peak'] == pytest.approx(4 * 152 * 2.07)              # G warp instructions / s
    assert r['achieved'] == pytest.approx(4.2e9 / 13.8e-3 / 1e9, rel=1e-3)
    assert r['frac'] == pytest.approx(r['achieved'] / r['peak'], rel=1e-3)
    assert bench.issue_roofline(None, 13.8e-3, 152, 2070.0) is None


def test_committed_profile_figures_are_present():
    import bench
    t = bench._ncu_traffic()
    assert t.get('edge', 0) > 0 and t.get('edge_warp_instructions', 0) > 0
