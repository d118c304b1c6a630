"""Plan search of the 2D transform (GPU): the analogue of the reference's
FFTW planner flags (core/include/hpxfft/util/adapter_fftw.hpp:13-44), where
"measure" and stronger run trial transforms (core/src/shared/loop.cpp:169-182).

"measure" times every distinct candidate plan and keeps the fastest; the
choice is cached, so a second plan of the same kind runs no trials, and it
survives a wisdom export / forget / import round trip.  Results of every
searched plan match the oracle (FP64 <= 1e-12, FP32 <= 2e-6).
"""
import numpy as np
import pytest

from gpu_helpers import padded, rel_l2, run_device, to_complex

pytestmark = pytest.mark.gpu


def oracle_fwd(oracle, x):
    p = oracle.padded(np.asarray(x, dtype=np.float64))
    oracle.fft_2d_r2c(p, nthreads=8)
    return oracle.spectrum(p)


def search_results(plan):
    n = int(plan.measurement("autotune_candidates"))
    return [plan.measurement(f"autotune_ms_{i}") for i in range(n)]


def choice(plan):
    return tuple(plan.measurement(k) for k in ("choice_columns", "choice_ff_pairs", "choice_tc_vectors",
                                               "choice_tc_rows"))


def test_measure_picks_the_fastest_candidate_and_caches_it(gpu_lib, cuda, oracle_lib, tmp_path, monkeypatch):
    from hpxfft import batch as hb

    for var in ("HPXFFT_COLUMNS", "HPXFFT_FF_PAIRS"):
        monkeypatch.delenv(var, raising=False)
    hb.wisdom_forget()
    nx = ny = 4096
    x = np.random.default_rng(21).uniform(-1, 1, (nx, ny))
    ref = oracle_fwd(oracle_lib, x)
    try:
        with gpu_lib.Plan(nx, ny + 2, 1, "f64", "measure") as plan:
            ms = search_results(plan)
            # cluster columns, four-step columns with and without the
            # float-float pair exchange
            assert len(ms) == 3 and all(m > 0 for m in ms), ms
            assert plan.measurement("autotune_best_ms") == min(ms)
            assert ms[int(plan.measurement("autotune_chosen"))] == min(ms)
            assert plan.measurement("cached_plan") == 0.0
            tuned = choice(plan)
            got = to_complex(run_device(cuda, plan, padded(x)))
            assert rel_l2(got, ref) <= 1e-12
            report = tmp_path / "plan.txt"
            plan.write_plan(str(report))
            text = report.read_text()
            assert "flag measure, from search" in text and text.count("candidate ") == 3 and "(chosen)" in text
        # the choice is cached: no trials the second time
        with gpu_lib.Plan(nx, ny + 2, 1, "f64", "measure") as plan:
            assert plan.measurement("cached_plan") == 1.0
            assert plan.measurement("autotune_candidates") == 0.0
            assert choice(plan) == tuned
        # and survives a wisdom round trip
        path = tmp_path / "wisdom.txt"
        hb.wisdom_export(str(path))
        assert "2d;p0;4096x4098;b1;full;" in path.read_text()
        hb.wisdom_forget()
        with gpu_lib.Plan(nx, ny + 2, 1, "f64", "patient") as plan:
            assert plan.measurement("cached_plan") == 0.0 and len(search_results(plan)) == 3
        hb.wisdom_forget()
        hb.wisdom_import(str(path))
        with gpu_lib.Plan(nx, ny + 2, 1, "f64", "exhaustive") as plan:
            assert plan.measurement("cached_plan") == 1.0 and choice(plan) == tuned
            got = to_complex(run_device(cuda, plan, padded(x)))
            assert rel_l2(got, ref) <= 1e-12
        # "estimate" never searches
        with gpu_lib.Plan(nx, ny + 2, 1, "f64", "estimate") as plan:
            assert plan.measurement("autotune_candidates") == 0.0
            assert plan.measurement("cached_plan") == 0.0
    finally:
        hb.wisdom_forget()


@pytest.mark.parametrize("prec,n_cand", [("f32", 2), ("bf16x3", None)])
def test_measure_other_precisions(gpu_lib, cuda, oracle_lib, monkeypatch, prec, n_cand):
    """FP32 searches the two column strategies; split-BF16 the vectors per
    CTA and tensor-core rows (its columns are always the four-step kernels)."""
    from hpxfft import batch as hb

    for var in ("HPXFFT_COLUMNS", "HPXFFT_TC_VECTORS", "HPXFFT_TC_ROWS"):
        monkeypatch.delenv(var, raising=False)
    hb.wisdom_forget()
    nx, ny = 2048, 4096
    x = np.random.default_rng(22).uniform(-1, 1, (nx, ny)).astype(np.float32)
    ref = oracle_fwd(oracle_lib, x.astype(np.float64))
    try:
        with gpu_lib.Plan(nx, ny + 2, 1, prec, "measure") as plan:
            ms = search_results(plan)
            if n_cand is not None:
                assert len(ms) == n_cand
            else:
                assert 2 <= len(ms) <= 4
            assert all(m > 0 for m in ms) and plan.measurement("autotune_best_ms") == min(ms)
            got = to_complex(run_device(cuda, plan, padded(x, np.float32)))
            assert rel_l2(got, ref) <= 2e-6
    finally:
        hb.wisdom_forget()


def test_environment_fixes_a_choice_the_search_keeps(gpu_lib, cuda, monkeypatch):
    """A choice forced through the environment is not searched over."""
    from hpxfft import batch as hb

    hb.wisdom_forget()
    monkeypatch.setenv("HPXFFT_COLUMNS", "cluster")
    try:
        with gpu_lib.Plan(4096, 4098, 1, "f64", "measure") as plan:
            assert plan.measurement("choice_columns") == 1.0
            # cluster columns leave nothing else to vary: one candidate, no trials
            assert plan.measurement("autotune_candidates") == 0.0
    finally:
        hb.wisdom_forget()
