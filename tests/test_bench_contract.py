"""bench.py's output line for the reference arm (the CPU restatement of the
reference's EP loop), on the small SBM workload: one JSON line with the
fields the contract names, single-process and as two gloo ranks (rank 0
alone prints).  No GPU."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _last_json(out: str) -> dict:
    lines = [x for x in out.splitlines() if x.startswith("{")]
    assert len(lines) == 1, out
    return json.loads(lines[0])


def _check_line(d: dict, n_gpus: int):
    for k, t in (("impl", str), ("metric", str), ("value", float), ("unit", str), ("n_gpus", int), ("steps", int),
                 ("warmup", int), ("ms_per_step", float), ("higher_is_better", bool), ("scaling", str),
                 ("dtype", str), ("data", str), ("config", dict), ("cpu_baseline", dict), ("e2e", dict)):
        assert isinstance(d[k], t), (k, d.get(k))
    assert d["impl"] == "reference" and d["n_gpus"] == n_gpus and d["value"] > 0 and d["unit"] == "nodes/sec"
    assert d["vs_baseline"] is None and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and "batches" in cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    assert d["config"]["workload"].startswith("sbm10k: SBM")
    # the reference arm runs none of the trainer's code: it loads the
    # workload generators and the oracle only
    libs = d["loaded_libraries"]
    assert "oracle/_build/libep_oracle.so" in libs and not any("libep_gb300" in x for x in libs), libs


def test_reference_arm_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "sbm10k", "--steps", "2",
                        "--warmup", "1"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    _check_line(_last_json(r.stdout), 1)


@pytest.mark.timeout(600)
def test_reference_arm_two_ranks():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", "29613", "bench.py", "--impl", "reference",
                        "--workload", "sbm10k", "--gpus", "2", "--steps", "2", "--warmup", "1"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    _check_line(_last_json(r.stdout), 2)
