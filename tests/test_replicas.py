"""The N > 1 path of bench.py on CPU: replicas with no data-path collective, only the timing barrier and the
max over ranks of the elapsed time (gloo, world size 2), and the reference arm under torchrun, where rank 0
alone runs and prints its line."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    r, w, _ = bench.dist()
    bench.barrier(w)
    m = bench.reduce_max(w, 1.5 * r + 0.25)
    out.put((r, w, m))
    import torch.distributed as td
    td.destroy_process_group()


def test_barrier_and_max_over_ranks_gloo():
    """Each rank's elapsed time differs; every rank gets the maximum (the value bench.py reports)."""
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(g[0] for g in got) == [0, 1]
    assert all(g[1] == 2 and g[2] == 1.75 for g in got)


def test_reference_arm_under_torchrun():
    """`bench.py --impl reference` launched like the driver's N = 2 run: one JSON line, from rank 0."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), "bench.py", "--impl", "reference",
           "--gpus", "2", "--shape", "9,13,17", "--steps", "2", "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"


def test_reference_arm_json_contract():
    """The reference arm's line at N = 1 carries the keys the bench contract names."""
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--shape", "9,13,17", "--steps", "2", "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "e2e", "cpu_baseline", "impl"):
        assert k in d, k
    assert d["n_gpus"] == 1 and d["warmup"] >= 3 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["value"] == d["value"] and d["e2e"]["value"] == d["value"]
    assert "workload" in d["config"]


def test_clock_samples_kept_for_the_timed_region():
    """bench.py's clock sampler keeps the nvidia-smi samples whose timestamps fall inside the timed region,
    reports the throttle reasons seen there, and falls back to every sample (saying so) when none does."""
    import datetime
    sys.path.insert(0, ROOT)
    import bench
    c = bench.Clocks()

    def line(t, sm, reason="Not Active"):
        stamp = datetime.datetime.fromtimestamp(t).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
        return f"{stamp}, 0, {sm}, 2070, 900.0, 0x0, {reason}, Not Active, Not Active, Not Active"

    t0 = 1_700_000_000.0
    c.lines = [line(t0 - 1.0, 345, "Active"), line(t0 + 0.1, 2070), line(t0 + 0.2, 2055), line(t0 + 0.3, 2070),
               line(t0 + 2.0, 900, "Active")]
    c.p = None
    c.t0, c.t1 = t0, t0 + 0.5

    class _Done:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    class _T:
        def join(self, timeout=None):
            pass

    c.p, c.t = _Done(), _T()
    r = c.stop()
    assert r["samples"] == 3 and r["window"] == "timed region"
    assert r["sm_mhz"] == 2070.0 and r["sm_max_mhz"] == 2070.0 and r["reasons"] == []
    c.lines = [line(t0 - 1.0, 345, "Active")]
    c.t0, c.t1 = t0, t0 + 0.5
    r = c.stop()
    assert r["samples"] == 1 and r["window"].startswith("whole") and r["reasons"] == ["hw_slowdown"]
