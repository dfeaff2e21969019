"""CPU: the bench's host-side parts.  The reference arm times one full run
of the workload split into its K steps and reports the same config as the
GPU arm; the oracle's full run records when the residual reached the
stated tolerance; the single-thread and dense-inverse estimates measure
real work; the memory guard reads the host's free memory."""
import importlib.util
import os

import numpy as np
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


def _reference_line(ne, steps, warmup):
    import json
    import subprocess
    import sys
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--ne", str(ne),
                          "--steps", str(steps), "--warmup", str(warmup)], capture_output=True, text=True,
                         timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    return json.loads(lines[0])


@pytest.mark.parametrize("steps,warmup", [(1, 0), (4, 1)])
def test_reference_arm_prints_one_contract_line(bench, steps, warmup):
    """`bench.py --impl reference` (host cores only) prints one JSON line with
    the keys the measurement contract asks of the reference arm; its K steps
    together are one full run (the value is DOFs over their summed time)."""
    d = _reference_line(12, steps, warmup)
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "DOF/s" and d["higher_is_better"]
    assert d["steps"] == steps and d["warmup"] == warmup and d["n_gpus"] == 1
    assert len(d["step_s"]) == steps
    n_dof = 3 * 13 ** 3
    assert d["value"] == pytest.approx(n_dof / sum(d["step_s"]))
    assert d["ms_per_step"] == pytest.approx(sum(d["step_s"]) / steps * 1e3)
    assert d["relres"] <= 1e-10 and d["iterations"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == d["value"] and cb["cores"] >= 1 and "one full 12^3 run" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "DOF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}

    class A:
        ne, rtol = 12, 1e-10
    assert d["config"] == bench.headline_config(A, 1)   # the GPU arm reports the same dict


def test_oracle_full_run_marks_the_stated_tolerance(bench, sfem, coracle):
    p = sfem.meshgen.jittered_cube(ne=10)
    u, rec = bench.oracle_full_run(p, 2, rtol=1e-13, mark=1e-10)
    assert rec["relres"] <= 1e-13 and 0 < rec["iterations_to_mark"] < rec["iterations"]
    assert 0 < rec["solve_to_mark_s"] <= rec["solve_s"] and rec["cpu_s"] > rec["assemble_s"] > 0
    K = coracle.assemble(p.ne, p.NodeList, p.IEN, 3, "Q1", 3, p.ID, p.Young, 0.3, nthreads=2)
    u10, st = K.solve(p.fixed_dofs, p.fixed_vals, rtol=1e-10, nthreads=2)
    assert abs(st["iters"] - rec["iterations_to_mark"]) <= 2    # OpenMP sums may round differently
    assert np.linalg.norm(u - u10) / np.linalg.norm(u) < 1e-6


def test_oracle_solution_quad_is_the_direct_solve(bench, sfem, oracle):
    p = sfem.meshgen.quad_problem(6, 3, jitter=0.15, nu=0.4, plane="strain", e_sigma=0.5)
    u, how = bench.oracle_solution(p, 1)
    K = oracle.assemble_system(p.ne, p.NodeList, p.IEN, 2, "Q1", 2, p.ID, p.Young, 0.4, "strain")
    ref = oracle.solve_eliminated(K, p.fixed_dofs, p.fixed_vals, method="inv")
    assert "sparse LU" in how and np.linalg.norm(u - ref) / np.linalg.norm(ref) < 1e-12


def test_memory_guard(bench):
    ok, need, avail = bench._oracle_fits(10 ** 3)
    assert ok and need > 0 and avail > need
    ok, need, avail = bench._oracle_fits(10 ** 12)
    assert not ok
