"""CPU: the bench's CPU-baseline estimates (oracle timings scaled to the
full workload) measure real work: a positive PCG iteration time after the
warm-up solve, and finite single-thread and dense-inverse figures."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_pcg_iteration_time_is_positive(bench, sfem, coracle):
    q = sfem.meshgen.jittered_cube(ne=8)
    K = coracle.assemble(q.ne, q.NodeList, q.IEN, 3, "Q1", 3, q.ID, q.Young, 0.3, nthreads=2)
    t = bench._pcg_iteration_s(K, q, 5, 2)
    assert t > 0.0


def test_single_thread_and_dense_inverse_estimates(bench, sfem):
    st = bench.cpu_single_thread(sfem, 16, 3 * 17 ** 3, 9 * 49 ** 3, 100, sample_ne=8, sample_iters=4)
    assert st["cores"] == 1 and st["value"] > 0 and st["est_full_s"] > 0
    d = bench.dense_inverse_solve(sfem, sample_ne=4)
    assert d["est_s"] > 0 and d["threads"] >= 1 and "26,019 free" in d["problem"]


def test_reference_arm_prints_one_contract_line():
    """`bench.py --impl reference` (host cores only) prints one JSON line with
    the keys the measurement contract asks of the reference arm."""
    import json
    import subprocess
    import sys
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--ne", "12",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "DOF/s" and d["higher_is_better"]
    assert d["steps"] == 1 and d["warmup"] == 0 and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == d["value"] and cb["cores"] >= 1 and cb["sample"]
    assert cb["single_thread"]["cores"] == 1 and cb["reference_dense_solve"]["est_s"] > 0
    assert d["e2e"] == {"value": d["value"], "unit": "DOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
