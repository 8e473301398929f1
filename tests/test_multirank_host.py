"""The bench's multi-rank bookkeeping on CPU with two gloo ranks: the job's
time is the max over ranks, the value counts every rank's rays, and only
rank 0 of the reference arm does work and prints (world_size 2, gloo,
127.0.0.1)."""
import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, outdir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, lr = bench.dist_info()
    ms = [40.0, 55.5][rank]
    job_ms = bench.reduce_step_time(ms, w, "cpu")
    value = bench.job_throughput(1000, w, 12, 10, job_ms)
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(outdir, f"rank{rank}.json"), "w") as f:
        json.dump({"rank": r, "world": w, "local": lr, "job_ms": job_ms, "value": value}, f)


def test_two_gloo_ranks_agree_on_the_job_time(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    assert [r["rank"] for r in res] == [0, 1] and all(r["world"] == 2 for r in res)
    assert all(r["job_ms"] == 55.5 for r in res)          # the slower rank sets the time
    assert all(abs(r["value"] - 2 * 1000 * 12 * 10 / 0.0555) < 1e-6 for r in res)


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_step_time(12.5, 1, "cpu") == 12.5
    assert bench.job_throughput(100, 1, 12, 2, 1000.0) == 100 * 12 * 2


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    bench.run_reference(bench.parse())   # returns before any CPU work
    assert capsys.readouterr().out == ""


def test_reference_arm_loads_no_product_library():
    """The reference arm (the oracle's restatement of the reference trace on
    the host cores) imports nothing of the product package and maps none of
    its libraries; its line is the contract's, with impl "reference"."""
    import json
    import subprocess
    code = ("import sys, json, io, contextlib; sys.argv = ['bench.py', '--impl', 'reference', '--nrays', '4096', "
            "'--steps', '1', '--warmup', '1']; import bench; buf = io.StringIO()\n"
            "with contextlib.redirect_stdout(buf): bench.main()\n"
            "maps = open('/proc/self/maps').read()\n"
            "print(json.dumps({'line': buf.getvalue().strip().splitlines()[-1], "
            "'imported': [m for m in sys.modules if m.startswith('batoid_gb300')], "
            "'mapped': 'libbatoid_gb300' in maps}))")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    rep = json.loads(out.stdout.strip().splitlines()[-1])
    assert rep["imported"] == [] and not rep["mapped"]
    line = json.loads(rep["line"])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
