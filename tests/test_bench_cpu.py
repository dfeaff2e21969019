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
