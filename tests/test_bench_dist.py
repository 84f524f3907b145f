"""Replica (N > 1) paths of bench.py on the host: two gloo ranks launched by
torchrun on 127.0.0.1 with no GPU visible.  The path has no data exchange
between replicas; the only collectives are the barrier and the max over ranks
of the timed region."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env():
    env = dict(os.environ)
    env["CUDA_VISIBLE_DEVICES"] = ""
    env["OMP_NUM_THREADS"] = "2"
    return env


def test_two_rank_max_and_barrier(tmp_path):
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "import bench\n"
        "world, rank, local = bench.dist_setup()\n"
        "assert world == 2\n"
        "bench.dist_barrier(world)\n"
        "m = bench.dist_max(10.0 + rank, world)\n"
        "open(%r + '/rank%%d.txt' %% rank, 'w').write('RANK %%d MAX %%s' %% (rank, m))\n"
        "import torch.distributed as dist; dist.destroy_process_group()\n" % (ROOT, str(tmp_path)))
    script = tmp_path / "ranks.py"
    script.write_text(code)
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
                        "--master-addr=127.0.0.1", f"--master-port={_port()}", str(script)],
                       capture_output=True, text=True, timeout=300, env=_env(), cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    # one record file per rank (the ranks share one stdout pipe)
    found = sorted((tmp_path / f"rank{k}.txt").read_text() for k in range(2))
    assert found == ["RANK 0 MAX 11.0", "RANK 1 MAX 11.0"], (found, r.stdout)


def test_reference_arm_two_ranks_prints_once(oracle_lib):
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
                        "--master-addr=127.0.0.1", f"--master-port={_port()}", "bench.py", "--impl", "reference",
                        "--gpus", "2", "--size", "8", "--steps", "2", "--warmup", "1"],
                       capture_output=True, text=True, timeout=600, env=_env(), cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(ln) for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0


def test_gpus_flag_starts_the_ranks(oracle_lib):
    """--gpus 2 without a launcher starts two ranks itself (torchrun on
    127.0.0.1); rank 0 alone prints."""
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--size", "8",
                        "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, timeout=600, env=_env(), cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(ln) for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1 and lines[0]["n_gpus"] == 2, r.stdout


def test_cpu_sample_reports_the_steps_it_timed(oracle_lib):
    """A time budget shorter than one step times exactly one step, and the
    sample says the rate is extrapolated from fewer steps than asked."""
    sys.path.insert(0, ROOT)
    import bench
    rate, cores, secs, done = bench.cpu_oracle_rate(bench.workload(8, seed=3), 5, 0, budget_s=0.0)
    assert done == 1 and rate > 0 and secs > 0
    text = bench.sample_text(done, 5, 0, cores, secs)
    assert "1 of 5 asked" in text and "extrapolated" in text
    assert "extrapolated" not in bench.sample_text(5, 5, 0, cores, secs)
