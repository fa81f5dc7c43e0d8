"""Multi-rank host logic of the replica path on the CPU: two gloo ranks."""
import os
import socket

import pytest

from umbreon_gb300 import replicas


def test_partition_covers_every_item_once():
    for n in (0, 1, 7, 64, 65):
        for world in (1, 2, 3, 8):
            seen = [i for r in range(world) for i in replicas.partition(n, r, world)]
            assert seen == list(range(n))
            sizes = [len(replicas.partition(n, r, world)) for r in range(world)]
            assert max(sizes) - min(sizes) <= (1 if n else 0)


def test_single_process_reduction_is_identity():
    units_s, ms = replicas.job_throughput(1000.0, 2.0)
    assert ms == 2.0 and units_s == 1000.0 / 2e-3


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ws, r, local = replicas.env_ranks()
        mine = replicas.partition(64, r, ws)
        # each rank "renders" its frames: 1,000 rays and (rank + 1) ms per frame
        units_s, ms = replicas.job_throughput(1000.0 * len(mine), float(len(mine) * (r + 1)))
        dist.barrier()
        q.put((r, list(mine), units_s, ms))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_slowest_rank_sets_the_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, f0, u0, ms0), (r1, f1, u1, ms1) = out
    assert f0 + f1 == list(range(64))
    # slowest rank: 32 frames x 2 ms; all ranks: 64,000 rays
    assert ms0 == ms1 == 64.0
    assert u0 == u1 == pytest.approx(64000.0 / 0.064)


def _timed_rank_main(rank, world, port, q):
    """One rank of the bench's replica loop with a stub render: rank r renders
    its block of the 64-frame list, each frame 1,000 rays in (r + 1) ms."""
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = replicas.partition(64, rank, world)
        calls = []

        def step():  # one "batch" = this rank's frames
            calls.append(1)
            return 1000.0 * len(mine), float(len(mine) * (rank + 1))

        job = replicas.timed_steps(step, 3)
        q.put((rank, len(calls), job))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_timed_replica_loop():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_timed_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted((q.get(timeout=120) for _ in procs), key=lambda t: t[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ncalls, job in out:
        assert ncalls == 3
        # the slowest rank (rank 1: 32 frames x 2 ms x 3 batches) sets the time;
        # units are both ranks' 3 x 64,000 rays
        assert job["ms_max"] == 3 * 32 * 2.0
        assert job["units_all"] == 3 * 64000.0
        assert job["units_per_s"] == pytest.approx(3 * 64000.0 / (3 * 32 * 2.0e-3))
    assert out[0][2]["local_units"] == 3 * 32000.0


def test_launch_command_runs_n_ranks_on_localhost():
    cmd = replicas.launch_cmd(4, "bench.py", ["--gpus", "4", "--steps", "2"], port=29999)
    assert cmd[1:3] == ["-m", "torch.distributed.run"]
    assert "--nproc-per-node=4" in cmd and "--master-addr=127.0.0.1" in cmd and "--master-port=29999" in cmd
    assert cmd[-5:] == ["bench.py", "--gpus", "4", "--steps", "2"]


def test_bench_refuses_a_rank_count_that_does_not_match_gpus(tmp_path):
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, WORLD_SIZE="1", RANK="0", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--gpus", "2", "--impl", "reference"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode != 0 and "--gpus 2 but 1 ranks" in r.stderr


def test_clock_summary_keeps_the_timed_region_samples():
    """The clock record of a bench line: the median SM clock and the throttle
    reasons of the samples taken inside the timed region; a region shorter
    than one sampling period reports the sample taken just before it."""
    import importlib.util
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    c = bench.ClockSampler(0)
    c.before = ["0, 1980, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active"]
    c.lines = ["0, 2070, 2070, 1000.0, 0x4, Not Active, Not Active, Not Active, Active",
               "0, 2040, 2070, 1100.0, 0x4, Not Active, Not Active, Not Active, Active",
               "0, 2055, 2070, 1050.0, 0x0, Not Active, Not Active, Not Active, Not Active"]
    s = c.summary()
    assert s["sm_mhz"] == 2055.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"] and s["samples"] == 3
    c.lines = []
    s = c.summary()
    assert s["sm_mhz"] == 1980.0 and s["samples"] == 0 and s["reasons"] == []
    c.before = []
    assert c.summary()["reasons"] == ["unsampled"]


def test_roofline_traffic_scales_the_capture_and_flags_stale_sources(tmp_path, monkeypatch):
    """roofline.traffic: the committed ncu capture's DRAM bytes per ray times
    the rays of the timed launch; `current` says whether the trace kernels'
    sources still match the capture's digest."""
    import importlib.util
    import json
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("bench_mod2", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    committed = json.loads(open(os.path.join(root, "profiles", "traffic.json")).read())["trace_occlusion"]
    assert committed["capture"]["rays"] > 0 and committed["capture"]["dram_bytes"] > 0
    (tmp_path / "profiles").mkdir()
    for f in bench.TRAFFIC_SOURCES:
        (tmp_path / f).parent.mkdir(parents=True, exist_ok=True)
        (tmp_path / f).write_text("kernel v1\n")
    monkeypatch.setattr(bench, "ROOT", tmp_path)
    rec = {"trace_occlusion": {"capture": {"dram_bytes": 5000, "rays": 1000, "workload": "w"},
                               "kernel_digest": bench.kernel_digest()}}
    (tmp_path / "profiles" / "traffic.json").write_text(json.dumps(rec))
    t, info = bench._traffic("trace_occlusion", 4000)
    assert t == 20000 and info["dram_bytes_per_ray"] == 5.0 and info["current"] is True
    (tmp_path / bench.TRAFFIC_SOURCES[1]).write_text("kernel v2\n")
    assert bench._traffic("trace_occlusion", 4000)[1]["current"] is False
    assert bench._traffic("trace_closest", 4000) == (None, None)
