"""bench.py's host logic for more than one rank, on CPU (gloo, world size
2): each rank times its own region (replicas), the job's time is the
slowest rank's and its value counts every rank's cell-stages; the reference
arm runs on rank 0 alone and the other ranks exit 0 without output."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_max_over_ranks_and_whole_job_value():
    ws, port = 2, _free_port()
    procs = []
    for rank in range(ws):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, os.path.join(ROOT, "tests", "dist_rank.py")], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for o in outs:
        assert o["ms"] == 15.0  # the slowest rank
        assert o["value"] == pytest.approx(2 * 1_000_000 / 15e-3 / 1e6)


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference"], env=env,
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""


def test_reference_arm_line_on_one_rank():
    """The reference arm on rank 0 (CPU only, a tiny mesh): one JSON line
    with the ours-arm's metric, unit and workload config, impl 'reference',
    a cpu_baseline describing the run and an e2e without host transfers."""
    sys.path.insert(0, ROOT)
    import bench

    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
                        "--warmup", "3", "--n", "8"], env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr
    lines = [ln for ln in p.stdout.strip().splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"].startswith("Mcell*RK-stage/s") and d["unit"] == "Mcell*RK-stage/s"
    assert d["higher_is_better"] is True and d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # the same workload block the device arm prints for this mesh
    assert d["config"] == bench.workload_config(8, 512, 3 * 8 * 8 * 7, 1)
    assert d["steps"] == 2 and d["ms_per_step"] > 0
