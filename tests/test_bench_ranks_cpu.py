"""Multi-rank host logic of bench.py on CPU (gloo, world size 2): the
whole-job reduction (slowest rank's time, all ranks' events) and a torchrun
launch of the reference arm, in which rank 0 alone prints one JSON line."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, ev = bench.reduce_ranks(10.0 + 5 * rank, 1000 + rank, dist)
    dist.destroy_process_group()
    with open(os.path.join(out, "r%d.json" % rank), "w") as f:
        json.dump([ms, ev], f)


def test_reduce_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    for r in range(2):
        ms, ev = json.load(open(tmp_path / ("r%d.json" % r)))
        assert ms == 15.0 and ev == 2001


def test_reference_arm_under_torchrun(oracle_lib):
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--grid", "12"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "events/s"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    sys.path.insert(0, ROOT)
    import bench
    assert line["config"] == bench.headline_config(12, 1000, 2)
    assert line["ms_per_step"] > 0 and line["cpu_baseline"]["kind"] == "port"


def test_reference_arm_loads_no_engine_code(oracle_lib):
    """The reference arm times the CPU oracle with parameters from the
    oracle's own derivation: the engine library is never mapped."""
    code = ("import runpy, sys\n"
            "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', '--grid', '12']\n"
            "try:\n    runpy.run_path('bench.py', run_name='__main__')\nexcept SystemExit:\n    pass\n"
            "maps = open('/proc/self/maps').read()\n"
            "print('ENGINE_MAPPED' if 'libstz_gb300' in maps else 'ENGINE_NOT_MAPPED')\n"
            "print('ORACLE_MAPPED' if 'liboracle' in maps else 'ORACLE_NOT_MAPPED')\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "ENGINE_NOT_MAPPED" in r.stdout and "ORACLE_MAPPED" in r.stdout, r.stdout[-2000:]
