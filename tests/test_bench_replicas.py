"""The bench's multi-rank path on CPU (gloo, world size 2): the path is
replicated, not sharded (one independent replica per GPU, no collective in
the data path); the harness takes the slowest rank's time and reports the
whole-job rate, and the reference arm runs on rank 0 alone."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local = [2.5, 4.0][rank]                      # this replica's ms per step
    ms = bench.max_over_ranks(local, world, dist)
    value = world * 1000 / (ms * 1e-3)            # 1000 elements per replica step
    q.put((rank, ms, value))
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world_2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [4.0, 4.0]
    assert res[0][2] == pytest.approx(2 * 1000 / 4.0e-3)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    args = type("A", (), dict(warmup=3, steps=2, gpus=2, n=1024))()
    assert bench.run_reference(args) == 0
    assert capsys.readouterr().out == ""
    assert bench.max_over_ranks(3.0, 1, None) == 3.0


def test_reference_arm_line_keeps_the_contract(monkeypatch, capsys):
    # the reference arm's JSON line on a 16 x 16 plate (the sample side forced
    # small): the metric, unit and direction of the GPU arm, "impl":
    # "reference", a cpu_baseline describing the run and an e2e with no
    # host-device traffic
    import json
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "0")
    monkeypatch.setattr(bench, "cpu_sample_side", lambda nsteps, **kw: 16)
    args = type("A", (), dict(warmup=1, steps=1, gpus=1, n=16))()
    assert bench.run_reference(args) == 0
    lines = [l for l in capsys.readouterr().out.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC
    assert d["unit"] == "elements/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["config"]["same_workload"] is True and "512 triangles" in d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert cb["unit"] == "elements/s" and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "elements/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
