"""Serving-stream driver over grx_server: job work descriptors, a Poisson arrival
loop, and latency / throughput summaries.

A job is a dict of graspa_gb300.synth.serving_job: one box and its Widom insertions
or GCMC steps. `run_stream` submits each job at its arrival time (seconds on the
server clock), calls grx_server_progress in a loop (continuous batching: jobs are
admitted while others run, as slots and arena memory allow) and returns the results
with per-job latency = completion - arrival.
"""
import numpy as np

from . import grx


def job_work(J, ntrials=10, norient=10):
    """(kind, widom_desc, gcmc_descs) of a serving job; the job's seed keys its Philox
    stream, so its result does not depend on what else runs."""
    s = J["system"]
    seed = 1_000_003 + int(J["seed"])
    ms = int(s["molsize"][1])
    if J["kind"] == "widom":
        return grx.JOB_WIDOM, grx.widom_desc(s, 1, ntrials=ntrials, norient=norient, seed=seed), None
    single = ms == 1
    d = grx.gcmc_desc(1, ntrials=ntrials, norient=norient, p_translation=0.25,
                      p_rotation=0.25 if single else 0.5, p_reinsertion=0.5 if single else 0.75, p_swap=1.0,
                      pressure_pa=1e5, seed=seed)
    return grx.JOB_GCMC, None, [d]


def submit(server, J, tag):
    kind, wd, gd = job_work(J)
    if kind == grx.JOB_WIDOM:
        return server.submit(J["system"], J["capacity"], kind, widom=wd, insertions=J["widom_insertions"], tag=tag)
    return server.submit(J["system"], J["capacity"], kind, gcmc=gd, steps=J["gcmc_steps"], tag=tag)


def run_stream(server, jobs, arrivals=None, timeout=600.0):
    """Submit jobs[i] at arrivals[i] (None: all at once) and drive the server until
    every job is done. Returns {tag: (result, arrival)} with tag = job index."""
    n = len(jobs)
    arrivals = np.zeros(n) if arrivals is None else np.asarray(arrivals, dtype=np.float64)
    order = np.argsort(arrivals, kind="stable")
    t0 = server.time()
    nxt = 0
    out = {}
    while len(out) < n:
        now = server.time() - t0
        while nxt < n and arrivals[order[nxt]] <= now:
            i = int(order[nxt])
            submit(server, jobs[i], tag=i)
            nxt += 1
        server.progress()
        for r in server.poll():
            out[int(r.tag)] = (r, t0 + arrivals[int(r.tag)])
        if now > timeout:
            raise TimeoutError(f"serving stream: {len(out)} of {n} jobs done after {timeout} s")
    return out


def summarize(out):
    """jobs/s over the stream and p50 / p99 latency (completion - arrival), seconds."""
    lat = np.array([r.t_done - arr for (r, arr) in out.values()])
    t_first = min(arr for (_, arr) in out.values())
    t_last = max(r.t_done for (r, _) in out.values())
    span = max(t_last - t_first, 1e-9)
    done = np.sort([r.t_done for (r, _) in out.values()])
    lo, hi = steady_window(out)
    mid = int(np.sum((done >= lo) & (done <= hi)))
    return dict(jobs=len(out), jobs_per_s=len(out) / span, p50_s=float(np.percentile(lat, 50)),
                p99_s=float(np.percentile(lat, 99)), makespan_s=span,
                steady_jobs_per_s=mid / max(hi - lo, 1e-9),
                failed=sum(1 for (r, _) in out.values() if r.status != 0))


def steady_window(out):
    """(t10, t90): the server-clock times of the 10th- and 90th-percentile completions. Rates
    over this window leave out the ramp-up and the tail of the longest jobs, which a stream of
    finite length always has."""
    done = np.sort([r.t_done for (r, _) in out.values()])
    n = len(done)
    return float(done[int(0.1 * (n - 1))]), float(done[int(0.9 * (n - 1))])


def trial_energies_of(J, r):
    """Trial-energy evaluations a finished job performed, as the device counted them:
    first-bead positions, orientations of the growths whose first bead succeeded, and the
    2 configurations of a translation / rotation."""
    if r.kind == grx.JOB_WIDOM:
        return int(r.widom_trial_configs)
    return sum(int(r.gcmc[k].trial_configs) for k in range(max(1, r.ncomp_moved)))
