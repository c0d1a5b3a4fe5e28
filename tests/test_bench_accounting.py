"""Host-side accounting of the benchmark and the serving driver, on the CPU: the work a GCMC
launch reports comes from the kernel's own counters (grx_gcmc_stats.trial_configs /
trial_beads), serving rates over the whole stream and over the steady window between the
10th and 90th percentile completions, and the trial energies of a serving job."""
import types

import numpy as np
import pytest

import bench
from graspa_gb300 import grx, serving


def stats(configs, beads, attempts, sum_n):
    return types.SimpleNamespace(trial_configs=configs, trial_beads=beads, attempts=attempts, sum_n=sum_n)


def test_work_counts_what_the_kernel_evaluated():
    # two chains: 100 steps at a mean loading of 20 molecules of 3 atoms, 50 steps of an empty box
    st = [stats(1500, 2400, [25, 25, 25, 25, 0], 2000.0), stats(400, 640, [10, 10, 15, 15, 0], 0.0)]
    te, pairs = bench.work_of(st, 3, 3456)
    assert te == 1900
    assert pairs == pytest.approx(2400 * (3456 + 3 * 20.0) + 640 * 3456)


def test_work_of_a_chain_that_never_moved():
    te, pairs = bench.work_of([stats(0, 0, [0, 0, 0, 0, 0], 0.0)], 3, 100)
    assert te == 0 and pairs == 0


def result(t_done, status=0):
    return types.SimpleNamespace(t_done=t_done, status=status)


def test_summary_rates_and_latencies():
    # 11 jobs arriving at t = 0, done at 1..11 s
    out = {i: (result(float(i + 1)), 0.0) for i in range(11)}
    s = serving.summarize(out)
    assert s["jobs"] == 11 and s["failed"] == 0
    assert s["makespan_s"] == pytest.approx(11.0)
    assert s["jobs_per_s"] == pytest.approx(1.0)
    assert s["p50_s"] == pytest.approx(6.0)
    lo, hi = serving.steady_window(out)
    assert (lo, hi) == (2.0, 10.0)  # the 10th and 90th percentile completions
    assert s["steady_jobs_per_s"] == pytest.approx(9 / 8.0)  # completions 2..10 over 8 s


def test_steady_window_ignores_a_long_tail():
    # 100 jobs done within the first 10 s, then 10 large jobs finishing much later
    done = list(np.linspace(0.1, 10.0, 100)) + [100.0 + k for k in range(10)]
    out = {i: (result(t), 0.0) for i, t in enumerate(done)}
    s = serving.summarize(out)
    assert s["jobs_per_s"] < 1.1                # the whole stream is set by the tail
    assert s["steady_jobs_per_s"] > 9.0         # the steady window is not


def test_failed_jobs_are_counted():
    out = {0: (result(1.0), 0.0), 1: (result(2.0, status=3), 0.0)}
    assert serving.summarize(out)["failed"] == 1


def test_trial_energies_of_a_job():
    widom = types.SimpleNamespace(kind=grx.JOB_WIDOM, widom_trial_configs=1234)
    assert serving.trial_energies_of({}, widom) == 1234
    g = [types.SimpleNamespace(trial_configs=100), types.SimpleNamespace(trial_configs=50)]
    gcmc = types.SimpleNamespace(kind=grx.JOB_GCMC, ncomp_moved=2, gcmc=g)
    assert serving.trial_energies_of({}, gcmc) == 150
