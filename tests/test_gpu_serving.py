"""The continuous-batching job server (grx_server) on the GPU.

Every job's result is the same alone and in the mix: the comparisons below are exact
(each job sees only its own box and Philox stream; the mixed and FP64 arithmetic are
deterministic), slicing a job into several launches does not change it, and a Widom
job's <W> equals the direct grx_widom_insertions of the same box and seed.
"""
import numpy as np
import pytest

from graspa_gb300 import serving, synth

pytestmark = pytest.mark.gpu


def small_jobs(n, first=0):
    return [synth.serving_job(first + j, widom_insertions=200, gcmc_cycles=15, n_atoms_range=(200, 3000))
            for j in range(n)]


def same(a, b):
    assert a.status == 0 and b.status == 0
    assert a.kind == b.kind
    if a.kind == 0:
        assert a.widom_n == b.widom_n and a.widom_mean_w == b.widom_mean_w and a.widom_mean_w2 == b.widom_mean_w2
    else:
        for k in range(a.ncomp_moved):
            assert list(a.gcmc[k].attempts) == list(b.gcmc[k].attempts)
            assert list(a.gcmc[k].accepted) == list(b.gcmc[k].accepted)
            assert a.gcmc[k].n_molecules == b.gcmc[k].n_molecules and a.gcmc[k].sum_n == b.gcmc[k].sum_n
            # the energy sum is accumulated per launch: slices round differently
            e1, e2 = a.gcmc[k].energy[3], b.gcmc[k].energy[3]
            assert abs(e1 - e2) <= 1e-9 * max(1.0, abs(e2))


@pytest.mark.parametrize("batching", [0, 1])
@pytest.mark.parametrize("prec", ["GRX_MIXED", "GRX_FP64"])
def test_results_alone_equal_results_in_the_mix(grx_lib, prec, batching):
    """batching 1: the GCMC jobs advance together in shared rounds, joining and leaving
    between rounds, each with its own step count per round."""
    jobs = small_jobs(10)
    p = getattr(grx_lib, prec)
    fp = max(grx_lib.box_footprint(J["system"], J["capacity"]) for J in jobs)
    # room for about three boxes: jobs wait for memory as well as for slots
    mix = grx_lib.Server(3.5 * fp, max_resident=6, prec=p, widom_slice=64, gcmc_slice=100, gcmc_batching=batching)
    out_mix = serving.run_stream(mix, jobs)
    mix.close()
    assert len(out_mix) == len(jobs)
    for i, J in enumerate(jobs):
        # one slice (or, batching, rounds of another length) per job, nothing else resident
        alone = grx_lib.Server(4 * fp, max_resident=1, prec=p, gcmc_slice=1000 if batching else 0,
                               gcmc_batching=batching)
        out = serving.run_stream(alone, [J])
        alone.close()
        same(out_mix[i][0], out[0][0])


def test_widom_job_equals_direct_call(grx_lib):
    J = [j for j in small_jobs(12) if j["kind"] == "widom"][0]
    srv = grx_lib.Server(64 << 20, max_resident=2, prec=grx_lib.GRX_MIXED, widom_slice=50)
    r = serving.run_stream(srv, [J])[0][0]
    srv.close()
    kind, wd, _ = serving.job_work(J)
    box = grx_lib.Box(J["system"], capacity=J["capacity"])
    box.ewald_total()
    res = box.widom(wd, 0, J["widom_insertions"], grx_lib.GRX_MIXED)
    w = res["rosenbluth"] * (res["success"] != 0)
    assert r.widom_n == J["widom_insertions"]
    assert abs(r.widom_mean_w - w.mean()) <= 1e-12 * abs(w.mean())


def drive(srv, jobs):
    for i, J in enumerate(jobs):
        serving.submit(srv, J, tag=i)
    most, done = 0, {}
    for _ in range(10_000_000):
        res, pend = srv.progress()
        most = max(most, res)
        for r in srv.poll():
            done[int(r.tag)] = r
        if len(done) == len(jobs):
            break
    return most, done


def test_admission_by_footprint_and_slots(grx_lib):
    jobs = small_jobs(8, first=20)
    big = grx_lib.Server(1 << 30, max_resident=8, prec=grx_lib.GRX_MIXED)
    _, done = drive(big, jobs)
    big.close()
    fpa = [done[i].footprint_bytes for i in range(len(jobs))]
    assert all(f > 0 for f in fpa)
    # memory-bound residency: room for every job alone, not for all of them at once. Budgets
    # come from the admission minimum (grx_box_footprint: without the voxel candidate lists,
    # which a GCMC box adds only when the arena has room for them)
    fmin = [grx_lib.box_footprint(J["system"], J["capacity"]) for J in jobs]
    budget = max(int(1.2 * max(fmin)), int(0.5 * sum(fmin)))
    srv = grx_lib.Server(budget, max_resident=8, prec=grx_lib.GRX_MIXED, widom_slice=32, gcmc_slice=50)
    most, done = drive(srv, jobs)
    srv.close()
    assert len(done) == len(jobs) and all(r.status == 0 for r in done.values())
    held = [done[i].footprint_bytes for i in range(len(jobs))]
    assert 1 <= most <= budget // min(held) and most < len(jobs)
    # slot-bound residency
    srv = grx_lib.Server(1 << 30, max_resident=3, prec=grx_lib.GRX_MIXED, widom_slice=32, gcmc_slice=50)
    most, done = drive(srv, jobs)
    srv.close()
    assert len(done) == len(jobs) and most == 3
    # a job that cannot fit even alone is reported, not queued forever
    tiny = grx_lib.Server(grx_lib.box_footprint(jobs[0]["system"], jobs[0]["capacity"]) // 4, max_resident=2,
                          prec=grx_lib.GRX_MIXED)
    out = serving.run_stream(tiny, jobs[:1])
    tiny.close()
    assert out[0][0].status == 3                          # GRX_ERR_OUT_OF_MEMORY


def test_cluster_jobs_take_the_same_decisions(grx_lib):
    """GCMC jobs whose boxes pass the cluster policy (cluster_atoms) run on thread-block
    clusters of up to 8 CTAs; in FP64 they take the same decisions as on one block, with
    energies equal to 1e-9 (the partials are summed in another order)."""
    jobs = [J for J in small_jobs(16) if J["kind"] == "gcmc"][:4]
    assert len(jobs) == 4
    natoms = [int(J["system"]["comp_start"][-1]) for J in jobs]
    assert max(natoms) >= 2 * 300   # at least one job runs on a cluster
    fp = max(grx_lib.box_footprint(J["system"], J["capacity"]) for J in jobs)
    out = []
    for cl_atoms in (300, 0):
        srv = grx_lib.Server(8 * fp, max_resident=4, prec=grx_lib.GRX_FP64, gcmc_slice=100, cluster_atoms=cl_atoms)
        out.append(serving.run_stream(srv, jobs))
        srv.close()
    for i in range(len(jobs)):
        same(out[0][i][0], out[1][i][0])
