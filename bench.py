"""Benchmark: CBMC trial energies/s on one GB300, mixed precision vs plain FP64,
with the p50 / p99 job latency of the serving form.

Headline workload (`--workload gcmc`, the default): GCMC of rigid CO2 in the
synthetic all-silica framework (2x2x3 cells of 20.09 x 19.74 x 13.14 A, 3456
atoms; shifted LJ + real Coulomb at 12 A; Ewald alpha 0.265, kmax 9/9/6) at 300 K
and 1e5 Pa (fugacity coefficient 1): translation : rotation : CBMC insertion :
CBMC deletion = 1:1:1:1, 10 trial positions and 10 orientations, boxes starting
empty (0-120 molecules). Independent Markov chains (three per SM, different Philox
streams) run in one persistent launch replayed as a CUDA graph; one benchmark
"step" is S Monte Carlo steps of every chain. A trial energy is one trial
configuration evaluated against every atom, as the kernel counts them: 2 per
translation / rotation, 10 first-bead positions per CBMC insertion or deletion plus
10 orientations when the first bead was grown.

  value      trial energies/s of the batched mixed-precision form, state resident
  fp64       the same batch in FP64, and the plain FP64 single-box form
  e2e        the same metric through the public C ABI (grx_gcmc_run) per step: move
             descriptors uploaded, statistics read back, host synchronised
  accuracy   energy drift (FP64 recomputed totals vs accepted energies), loading,
             and mixed-vs-FP64 decisions and energies per move
  widom      the Widom workload of the same system (20,000 CO2 insertions per step)
  serving    a bounded Poisson job stream through grx_server: jobs/s, p50 / p99
             latency, next to the one-job-at-a-time FP64 form
Reference arm (--impl reference): the FP64 C++ oracle of the same moves, one chain
per host thread on all host cores, on a bounded sample.
"""
import argparse
import concurrent.futures
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NTRIALS = 10
NORIENT = 10
FLOP_PER_PAIR_CHARGED = 70.0   # FP32-equivalent work per pair (LJ + real Coulomb), the frozen work model
FLOP_PER_PAIR_LJ = 40.0
L2_FLUSH_BYTES = 256 << 20
PEAK_FP32_NOMINAL = 152 * 128 * 2 * 2070e6 / 1e12   # TFLOP/s, 128 FMA lanes per SM at the maximum clock
# DRAM bytes (read + write) of gcmc_kernel<mixed> per chain and Monte Carlo step: ncu
# dram__bytes_read.sum + dram__bytes_write.sum = 64.98 + 104.78 MB for one launch of 456
# chains x 20 steps of the kernel of commit 5cb704c (bench.py --profile --chains 456
# --mc-steps 20, ncu --set full --clock-control none -k regex:gcmc_kernel -s 20 -c 1: the third
# warm-up launch after the 18 autotune probes), scaled by chains x steps to the timed launch.
DRAM_BYTES_PER_CHAIN_STEP = (64.982784e6 + 104.780544e6) / (456 * 20)
DRAM_CAPTURE = "ncu capture of commit 5cb704c (20-step launch of 456 chains, scaled by chain-steps)"
_FP32_PEAK = []


def _hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0


HBM_PEAK_GBS = _hbm_peak()


def fp32_peak(grx):
    """Measured FP32 FMA peak of this device (TFLOP/s), once per process."""
    if not _FP32_PEAK:
        _FP32_PEAK.append(grx.probe_fp32_fma())
    return _FP32_PEAK[0]


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def rank_seed(rank, seed=42):
    """Philox key of a rank's chains: every rank runs independent replicas (no exchange)."""
    return seed + 1000 * rank


def aggregate(torch, dist, work, seconds, device):
    """Whole-job throughput over ranks: the work summed over ranks divided by the slowest
    rank's time (max over ranks, as the timing contract asks). Without a process group the
    rank is the job."""
    if dist is None:
        return work / seconds, work, seconds
    t = torch.tensor([float(work), float(seconds)], dtype=torch.float64, device=device)
    w = t[:1].clone()
    s = t[1:].clone()
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    dist.all_reduce(s, op=dist.ReduceOp.MAX)
    return float(w.item()) / float(s.item()), float(w.item()), float(s.item())


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if not self.proc:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) >= 9:
                rows.append(p)
        os.unlink(self.path)
        if not rows:
            return out
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, n in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(n)
        out.update(sm_mhz=float(np.median(sm)) if sm else None, sm_max_mhz=max(mx) if mx else None,
                   reasons=sorted(reasons), samples=len(rows))
        return out


# ------------------------------------------------------------------ workloads
def co2_system():
    from graspa_gb300 import synth
    return synth.silica_co2(seed=42)


def gcmc_descs(grx, n, seed=42):
    """The GCMC move set: translation : rotation : insertion : deletion = 1:1:1:1."""
    return [grx.gcmc_desc(1, ntrials=NTRIALS, norient=NORIENT, p_translation=0.25, p_rotation=0.5,
                          p_reinsertion=0.5, p_swap=1.0, pressure_pa=1e5, seed=seed, stream=k) for k in range(n)]


def work_of(stats, ms, nfw):
    """(trial energies, pair evaluations) of a list of GCMC statistics, from the kernel's
    own counts: the trial configurations it evaluated (trial_configs: first-bead positions,
    orientations grown after a successful first bead, the two configurations of a
    translation / rotation) and their beads. Pairs are beads x (framework atoms + guest
    atoms at the run's mean loading)."""
    te = pairs = 0.0
    for st in stats:
        steps = max(1, sum(st.attempts))
        guests = ms * st.sum_n / steps
        te += st.trial_configs
        pairs += st.trial_beads * (nfw + guests)
    return te, pairs


def make_boxes(grx, system, n, stream_ptr, cap_molecules=160):
    """n chains of one system: a box and n-1 replicas sharing its framework (one copy
    of framework atoms, tiles and tables on the device for all chains)."""
    nfw = system["comp_start"][1]
    ms = int(system["molsize"][1])
    parent = grx.Box(system, capacity=[nfw, ms * cap_molecules])
    parent.set_stream(stream_ptr)
    parent.ewald_total()
    boxes = [parent]
    for _ in range(n - 1):
        r = parent.replica()
        r.set_stream(stream_ptr)
        boxes.append(r)
    return boxes


def close_boxes(boxes):
    for b in reversed(boxes):   # replicas before their parent
        b.close()


def total_energy(box):
    return sum(box.total_energy().values())


# ------------------------------------------------------------------ GPU arm
def timed_graph(torch, batch, stream, S, steps, warmup, flush, dist=None):
    """CUDA-event time of `steps` graph replays of S Monte Carlo steps each (L2
    flushed before each), after `warmup` replays."""
    for _ in range(warmup):
        batch.run_graph(S, 1, stream.cuda_stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    warm_stats, _ = batch.stats()
    batch.reset_stats()
    times = []
    for _ in range(steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.run_graph(S, 1, stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1000.0)
    torch.cuda.synchronize()
    stats, _ = batch.stats()
    timed_graph.warm_stats = warm_stats
    return times, stats


def bench_gcmc(args, grx, torch, stream, flush, rank, world, dist):
    system = co2_system()
    nfw = system["comp_start"][1]
    ms = int(system["molsize"][1])
    R = args.chains or 3 * torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    S = args.mc_steps
    descs = gcmc_descs(grx, R, seed=rank_seed(rank))
    out = {"chains": R, "mc_steps_per_step": S}

    # mixed, batched: the headline
    boxes = make_boxes(grx, system, R, stream.cuda_stream)
    n_drift = min(8, R)
    e0 = [total_energy(b) for b in boxes[:n_drift]]
    for b in boxes[:n_drift]:
        b.ewald_total()
    batch = grx.GcmcBatch(boxes, descs, grx.GRX_MIXED)
    shape, cand = batch.autotune(S)   # real steps at the timed launch length; picks the launch shape
    out["autotune"] = {"warps_per_box": shape[0], "chunk_mult": shape[1], "cluster": batch.cluster(),
                       "ms_per_candidate": cand}
    l0 = grx.launch_count()
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    times, stats = timed_graph(torch, batch, stream, S, args.steps, args.warmup, flush, dist)
    clk = clocks.stop()
    launches = grx.launch_count() - l0
    te, pairs = work_of(stats, ms, nfw)
    value, te_all, tot = aggregate(torch, dist, te, sum(times), "cuda")
    out.update(value=value, seconds=tot, times=times, trial_energies=te, pairs=pairs, clocks=clk,
               launches=launches)
    warm = timed_graph.warm_stats
    acc_stats, nxt = batch.stats()
    batch.close()
    if args.profile:
        close_boxes(boxes)
        return out
    # drift and loading of the timed chains (all steps since creation)
    drift = []
    beta = grx.beta_from_temperature(300.0)
    for i, b in enumerate(boxes[:n_drift]):
        e1 = total_energy(b)
        drift.append(abs((e1 - e0[i]) - (warm[i].energy[3] + acc_stats[i].energy[3])))
    loading = float(np.mean([st.n_molecules for st in acc_stats]))
    out["accuracy"] = {
        "drift_max_beta_abs": float(beta * max(drift)), "drift_max_abs_internal": float(max(drift)),
        "drift_chains": n_drift, "drift_steps": int(nxt),
        "loading_mean_molecules": loading,
        "acceptance": [float(sum(st.accepted[k] for st in acc_stats) / max(1, sum(st.attempts[k] for st in acc_stats)))
                       for k in range(4)],
    }
    close_boxes(boxes)

    # the same batch in FP64
    boxes = make_boxes(grx, system, R, stream.cuda_stream)
    batch = grx.GcmcBatch(boxes, descs, grx.GRX_FP64)
    k64 = max(1, min(args.steps, 3))
    t64, st64 = timed_graph(torch, batch, stream, S, k64, 1, flush)
    te64, _ = work_of(st64, ms, nfw)
    batch.close()
    close_boxes(boxes)
    # the plain FP64 single-box form
    box1 = make_boxes(grx, system, 1, stream.cuda_stream)
    batch = grx.GcmcBatch(box1, descs[:1], grx.GRX_FP64)
    t1, st1 = timed_graph(torch, batch, stream, S, 3, 1, flush)
    te1, _ = work_of(st1, ms, nfw)
    batch.close()
    box1[0].close()
    out["fp64"] = {"batched_value": te64 / sum(t64), "single_box_value": te1 / sum(t1),
                   "single_box_mc_steps_per_s": 3 * S / sum(t1),
                   "speedup_mixed_over_fp64_batched": out["value"] / (te64 / sum(t64)),
                   "speedup_batched_mixed_over_fp64_single_box": out["value"] / (te1 / sum(t1))}

    # per-move agreement: the same 8 chains from the same state, FP64 vs mixed
    n_cmp = min(8, R)
    res = {}
    for name, p in (("fp64", grx.GRX_FP64), ("mixed", grx.GRX_MIXED)):
        bx = make_boxes(grx, system, n_cmp, stream.cuda_stream)
        res[name] = grx.gcmc_run(bx, descs[:n_cmp], 0, 300, p)
        close_boxes(bx)
    same = [list(a.accepted) == list(b.accepted) and a.n_molecules == b.n_molecules
            for a, b in zip(res["fp64"], res["mixed"])]
    rel = [abs(a.energy[3] - b.energy[3]) / max(abs(b.energy[3]), 1.0 / beta)
           for a, b in zip(res["mixed"], res["fp64"]) if list(a.accepted) == list(b.accepted)]
    out["accuracy"].update(chains_identical_decisions_300_steps=f"{sum(same)}/{n_cmp}",
                           max_rel_energy_sum_vs_fp64=float(max(rel)) if rel else None)

    # end to end through the public C ABI (synchronous grx_gcmc_run per step)
    boxes = make_boxes(grx, system, R, stream.cuda_stream)
    e2e = []
    step0 = 0
    te_e2e = 0.0
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        st = grx.gcmc_run(boxes, descs, step0, S, grx.GRX_MIXED)
        dt = time.perf_counter() - t0
        step0 += S
        if i >= args.warmup:
            e2e.append(dt)
            te_e2e += work_of(st, ms, nfw)[0]
    close_boxes(boxes)
    h2d, d2h = grx.last_transfer()  # what one grx_gcmc_run copies (the same every step)
    out["e2e"] = {"value": aggregate(torch, dist, te_e2e, sum(e2e), "cuda")[0], "unit": "trial_energies/s",
                  "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}
    return out


def bench_widom(args, grx, torch, stream, flush, n_insert):
    system = co2_system()
    nfw = system["comp_start"][1]
    box = grx.Box(system, capacity=[nfw, 3 * 64])
    box.set_stream(stream.cuda_stream)
    box.ewald_total()
    d = grx.widom_desc(system, 1, NTRIALS, NORIENT, seed=42)
    res_dev = torch.empty(n_insert * grx.WIDOM_RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    natoms = system["comp_start"][-1]
    chain = int(system["molsize"][1]) - 1

    def work(res):
        """(trial energies, pairs) the launch evaluated: every first-bead trial, and the
        orientations of the insertions whose first bead was grown (w_first > 0)."""
        grown = int(np.count_nonzero(res["w_first"] > 0.0))
        return NTRIALS * n_insert + NORIENT * grown, (NTRIALS * n_insert + NORIENT * chain * grown) * natoms

    def run(p, steps, warmup, move):
        for _ in range(warmup):
            box.widom_async(d, move, n_insert, p, res_dev.data_ptr())
            move += n_insert
        torch.cuda.synchronize()
        times, te, pairs = [], 0, 0
        for _ in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            box.widom_async(d, move, n_insert, p, res_dev.data_ptr())
            e1.record(stream)
            move += n_insert
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1000.0)
            w = work(np.frombuffer(res_dev.cpu().numpy().tobytes(), dtype=grx.WIDOM_RESULT_DTYPE))  # after timing
            te += w[0]
            pairs += w[1]
        return times, te, pairs

    tm, te_m, pairs_m = run(grx.GRX_MIXED, args.widom_steps, 2, 0)
    t64, te_64, _ = run(grx.GRX_FP64, 2, 1, 10 ** 8)
    acc = widom_accuracy(box, grx, system)
    box.close()
    t_launch = float(np.mean(tm))
    achieved = FLOP_PER_PAIR_CHARGED * pairs_m / sum(tm) / 1e12
    peak = fp32_peak(grx)
    return {"workload": f"widom_co2_silica_3456, {n_insert} insertions per launch",
            "value": te_m / sum(tm), "unit": "trial_energies/s",
            "fp64_value": te_64 / sum(t64),
            "speedup_mixed_over_fp64": (te_m / sum(tm)) / (te_64 / sum(t64)),
            "trial_energies_per_launch": te_m / len(tm),
            "kernel_ms": 1000 * t_launch, "achieved_tflops": achieved, "frac_of_measured_fp32": achieved / peak,
            "accuracy_vs_fp64_oracle": acc}


def widom_accuracy(box, grx, system, n=200):
    """Mixed / FP32 vs the FP64 oracle on the first n insertions of the stream."""
    from oracle import oracle as O
    S = O.OracleSystem(system)
    _, s_fw, s_ads = S.ewald_total(list(system["molsize"]))
    tm = system["templates"][1]
    mp = np.ascontiguousarray(tm["pos"].reshape(-1))
    mq = np.ascontiguousarray(tm["charge"], dtype=np.float64)
    mt = np.ascontiguousarray(tm["type"], dtype=np.int64)
    intra, self_ = S.rigid_exclusion(mp, mq, np.ones(3))
    w = O.OraWidom()
    w.component, w.molsize = 1, 3
    w.mol_pos, w.mol_charge, w.mol_type = O._d(mp), O._d(mq), O._i(mt)
    w.scale = w.scale_coul = 1.0
    w.ntrials, w.norient, w.new_molid = NTRIALS, NORIENT, 0
    w.beta = grx.beta_from_temperature(300.0)
    w.excl_intra, w.excl_self = intra, self_
    w.rigid, w.has_charge = 1, 1
    w.seed, w.stream = 42, 0
    ref = S.widom(w, s_fw, s_ads, 0, n)
    R = np.array([r.rosenbluth for r in ref])
    sf = np.array([r.sel_first for r in ref])
    so = np.array([r.sel_orient for r in ref])
    E = np.array([list(r.e_first) + list(r.e_chain) for r in ref])
    out = {}
    d = grx.widom_desc(system, 1, NTRIALS, NORIENT, seed=42)
    beta = grx.beta_from_temperature(300.0)
    for name, p in (("fp64", grx.GRX_FP64), ("mixed", grx.GRX_MIXED), ("fp32", grx.GRX_FP32)):
        g = box.widom(d, 0, n, prec=p)
        same = (g["sel_first"] == sf) & (g["sel_orient"] == so)
        r = same & (R > 0)
        Eg = np.concatenate([g["e_first"], g["e_chain"]], axis=1)
        dE = np.abs(Eg[r].reshape(-1, 2, 4).sum(2) - E[r].reshape(-1, 2, 4).sum(2))
        out[name] = {"selection_agreement": float(same.mean()),
                     "max_rel_rosenbluth": float(np.max(np.abs(g["rosenbluth"][r] - R[r]) / R[r])) if r.any() else 0.0,
                     "max_beta_dE": float(beta * dE.max()) if dE.size else 0.0}
    return out


def bench_serving(args, grx):
    """The serving stream (10,000 jobs in the full sweep): jobs of Widom (5k insertions) or GCMC (2k cycles of 20
    steps), five species, frameworks of 200-20,000 atoms, through grx_server (continuous
    batching, admission by HBM footprint). First all jobs at once (saturation: jobs/s and
    trial energies/s at capacity), then Poisson arrivals at fractions of that rate (jobs/s,
    p50 / p99 latency per rate). The plain one-job-at-a-time FP64 form runs a sample of the
    same jobs with GCMC shortened to serve_fp64_cycles cycles; its trial energies/s do not
    depend on the job length, and its job rate is extrapolated to full-length jobs by the
    per-job service time scaled by steps."""
    from graspa_gb300 import serving, synth
    n = args.serve_jobs
    t0 = time.perf_counter()
    jobs = [synth.serving_job(j, widom_insertions=5000, gcmc_cycles=args.serve_gcmc_cycles) for j in range(n)]
    t_gen = time.perf_counter() - t0

    def stream(arrivals):
        srv = grx.Server(args.serve_hbm_gb * (1 << 30), max_resident=args.serve_slots, prec=grx.GRX_MIXED,
                         widom_slice=0, gcmc_slice=args.serve_gcmc_slice,
                         cluster_atoms=0 if args.serve_batching else args.serve_cluster_atoms,
                         gcmc_batching=args.serve_batching)
        out = serving.run_stream(srv, jobs, arrivals, timeout=1800.0)
        srv.close()
        summ = serving.summarize(out)
        te = sum(serving.trial_energies_of(jobs[i], r) for i, (r, _) in out.items())
        summ["trial_energies_per_s"] = te / summ["makespan_s"]
        summ["trial_energies"] = te
        lo, hi = serving.steady_window(out)
        te_mid = sum(serving.trial_energies_of(jobs[i], r) for i, (r, _) in out.items() if lo <= r.t_done <= hi)
        summ["steady_trial_energies_per_s"] = te_mid / max(hi - lo, 1e-9)
        return summ

    sat = stream(None)   # every job at t = 0: throughput at capacity
    rate_sat = sat["jobs_per_s"]
    sweep = []
    g = np.random.default_rng(7)
    for f in args.serve_rate_fractions:
        rate = f * rate_sat
        arrivals = np.cumsum(g.exponential(1.0 / rate, n))
        r = stream(arrivals)
        r.update(arrival_rate_per_s=rate, fraction_of_saturation=f)
        sweep.append(r)
    # the plain one-job-at-a-time FP64 form on a sample (GCMC shortened, scaled back by steps)
    sub = []
    for k in range(args.serve_fp64_jobs):
        J = dict(jobs[k])
        if J["kind"] == "gcmc":
            J["gcmc_steps"] = args.serve_fp64_cycles * 20
        sub.append(J)
    plain = grx.Server(args.serve_hbm_gb * (1 << 30), max_resident=1, prec=grx.GRX_FP64)
    t0 = time.perf_counter()
    out64 = serving.run_stream(plain, sub, None, timeout=1800.0)
    dt = time.perf_counter() - t0
    plain.close()
    svc, svc_full = [], []
    for i, (r, _) in out64.items():
        t = r.t_done - r.t_admit
        svc.append(t)
        svc_full.append(t * (jobs[i]["gcmc_steps"] / sub[i]["gcmc_steps"] if sub[i]["kind"] == "gcmc" else 1.0))
    te64 = sum(serving.trial_energies_of(sub[i], r) for i, (r, _) in out64.items())
    plain_te = te64 / dt
    return {"jobs": n, "slots": args.serve_slots, "gcmc_cycles": args.serve_gcmc_cycles,
            "gcmc_batching": args.serve_batching, "gcmc_slice": args.serve_gcmc_slice,
            "gcmc_steps_per_job": args.serve_gcmc_cycles * 20, "widom_insertions": 5000,
            "cluster_atoms": args.serve_cluster_atoms, "species": "CH4 CO2 N2 Xe Kr uniform",
            "framework_atoms": "200-20000 log-uniform", "job_generation_s": t_gen,
            "saturation": sat, "sweep": sweep,
            "p50_s": sweep[0]["p50_s"] if sweep else sat["p50_s"],
            "p99_s": sweep[0]["p99_s"] if sweep else sat["p99_s"],
            "plain_fp64_one_at_a_time": {
                "jobs": len(sub), "gcmc_cycles": args.serve_fp64_cycles, "trial_energies_per_s": plain_te,
                "service_p50_s": float(np.percentile(svc, 50)),
                "jobs_per_s_full_length": len(svc_full) / float(np.sum(svc_full)),
                "note": "GCMC jobs shortened to gcmc_cycles; full-length service times scaled by steps"},
            "saturation_speedup_over_plain_fp64": sat["trial_energies_per_s"] / plain_te}


def run_grx(args):
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from graspa_gb300 import grx
    grx.build()
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    if args.workload == "widom":
        w = bench_widom(args, grx, torch, stream, flush, args.insertions)
        if rank == 0:
            print(json.dumps({"metric": "CBMC trial energies/s", "value": w["value"], "unit": "trial_energies/s",
                              "n_gpus": world, "workload": "widom", **w}), flush=True)
        return
    if args.workload in ("batched", "water"):
        line = bench_other(args, grx, torch, stream, flush, args.workload)
        if rank == 0:
            print(json.dumps(line), flush=True)
        return
    if args.workload == "cluster":
        line = bench_cluster(args, grx, torch, stream, flush)
        if rank == 0:
            print(json.dumps(line), flush=True)
        return
    if args.workload == "serving":
        s = bench_serving(args, grx)
        if rank == 0:
            print(json.dumps({"metric": "serving jobs/s and p99 job latency", "n_gpus": world, **s}), flush=True)
        return

    g = bench_gcmc(args, grx, torch, stream, flush, rank, world, dist)
    if args.profile:
        if rank == 0:
            print(json.dumps({"profile_run": True, "value": g["value"], "seconds": g["seconds"],
                              "launches": int(g["launches"])}), flush=True)
        return
    line = None
    if rank == 0:
        widom = bench_widom(args, grx, torch, stream, flush, args.insertions)
        serve = bench_serving(args, grx) if args.serve_jobs > 0 else None
        cpu_val, cpu_te, cpu_dt, cores, chains, steps = cpu_gcmc_rate(args.cpu_seconds)
        t_launch = float(np.mean(g["times"]))
        achieved = FLOP_PER_PAIR_CHARGED * g["pairs"] / args.steps / t_launch / 1e12
        peak = fp32_peak(grx)
        clk = g["clocks"]
        line = {
            "metric": "CBMC trial energies/s", "value": g["value"], "unit": "trial_energies/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * g["seconds"] / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32+fp64",
            "data": "synthetic (seeded Philox framework, Philox move stream)",
            "config": {"workload": "gcmc_co2_silica_3456 (1:1:1:1 translation/rotation/insertion/deletion, "
                                   "k=10, 300 K, 1e5 Pa, boxes start empty; chains are replicas sharing one "
                                   "framework copy)",
                       "chains": g["chains"], "mc_steps_per_step": g["mc_steps_per_step"],
                       "autotune": g.get("autotune"),
                       "trial_energies_per_step": g["trial_energies"] / args.steps,
                       "framework_atoms": 3456, "precision": "mixed",
                       "launch": "one persistent kernel per step, replayed as a CUDA graph",
                       "l2": "flushed between steps (256 MB write)", "parallelism": f"replicas x{world}"},
            "fp64": g["fp64"],
            "accuracy": g["accuracy"],
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak,
                         "traffic": DRAM_BYTES_PER_CHAIN_STEP * g["chains"] * g["mc_steps_per_step"],
                         "traffic_unit": "bytes per launch (ncu DRAM read + write, 20-step capture scaled)",
                         "traffic_source": DRAM_CAPTURE,
                         "hbm_gbs_achieved": DRAM_BYTES_PER_CHAIN_STEP * g["chains"] * g["mc_steps_per_step"]
                                             / t_launch / 1e9,
                         "hbm_peak_gbs": HBM_PEAK_GBS,
                         "peak_kind": "measured FP32 FMA throughput of this GPU in this run (grx_probe_fp32_fma); "
                                      f"nominal {PEAK_FP32_NOMINAL:.1f}",
                         "kernel": "gcmc_kernel<mixed>",
                         "model": f"{FLOP_PER_PAIR_CHARGED:.0f} FLOP/pair x {g['pairs'] / args.steps:.4g} pairs "
                                  "per launch (beads x (framework + guest atoms))"},
            "cpu_baseline": {"value": cpu_val, "unit": "trial_energies/s", "cores": cores, "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": f"{chains} resident chains x {steps} GCMC steps ({cpu_te:.0f} trial "
                                       f"energies, {cpu_dt:.1f} s of moves; set-up and Ewald totals before "
                                       "timing), FP64 C++ oracle, one chain per thread"},
            "e2e": g["e2e"],
            "gpu_launches": int(g["launches"]),
            "clocks": {"sm_mhz": clk["sm_mhz"], "sm_max_mhz": clk["sm_max_mhz"], "reasons": clk["reasons"]},
            "widom": widom,
            "serving": serve,
        }
        if serve:
            line["p99_job_latency_s"] = serve["p99_s"]
            line["p50_job_latency_s"] = serve["p50_s"]
            line["latency_at"] = "Poisson arrivals at %.2f of the saturation rate" % (
                args.serve_rate_fractions[0] if args.serve_rate_fractions else 1.0)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    if line:
        print(json.dumps(line), flush=True)


def bench_other(args, grx, torch, stream, flush, which):
    """The batched line (64 CH4/Xe boxes, triclinic, LJ only, autotuned) or the water
    line (TIP4P-Ew water in the hexagonal framework) as their own JSON lines."""
    from graspa_gb300 import synth
    if which == "batched":
        systems = [synth.ch4_xe_system(k) for k in range(64)]
        descs = []
        g = np.random.default_rng(3)
        for k in range(64):
            nt = int(g.integers(8, 33))
            kw = dict(ntrials=nt, norient=1, p_translation=0.3, p_rotation=0.3, p_reinsertion=0.5, p_swap=1.0,
                      pressure_pa=1e6, max_translation=0.7, seed=42, stream=k)
            descs.append([grx.gcmc_desc(1, **kw), grx.gcmc_desc(2, **kw)])
        boxes = []
        for s in systems:
            b = grx.Box(s, capacity=[s["comp_start"][1], 256, 256])
            b.set_stream(stream.cuda_stream)
            b.ewald_total()
            boxes.append(b)
        prec = grx.GRX_MIXED
        batch = grx.GcmcBatch(boxes, descs, prec)
        chosen, cand_ms = batch.autotune(args.mc_steps)
        cluster = batch.cluster()   # 64 boxes leave SMs idle: clusters of 2 CTAs are probed
        times, stats = timed_graph(torch, batch, stream, args.mc_steps, args.steps, args.warmup, flush)
        batch.close()
        te = 0.0
        pairs = 0.0
        for k, s in enumerate(systems):
            for e in range(2):
                st = stats[2 * k + e]
                te += st.trial_configs
                pairs += st.trial_beads * (s["comp_start"][1] + st.sum_n / max(1, sum(st.attempts)))
        t = sum(times)
        for b in boxes:
            b.close()
        achieved = FLOP_PER_PAIR_LJ * pairs / t / 1e12
        return {"metric": "CBMC trial energies/s", "value": te / t, "unit": "trial_energies/s", "n_gpus": 1,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * t / args.steps,
                "workload": "batched_ch4_xe_64_triclinic (mixture GCMC, 8-32 trials, LJ only)",
                "mc_steps_per_step": args.mc_steps,
                "autotune": {"warps_per_box": chosen[0], "chunk_mult": chosen[1], "cluster": cluster,
                             "ms_per_candidate": cand_ms},
                "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak(grx), "unit": "TFLOP/s",
                             "frac": achieved / fp32_peak(grx), "model": "40 FLOP/pair (LJ only)"},
                "framework_atoms": [int(s["comp_start"][1]) for s in systems[:8]]}
    system = synth.tip4p_hex_system(n_water=0)
    nfw = system["comp_start"][1]
    R = 3 * torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    descs = [grx.gcmc_desc(1, p_translation=0.25, p_rotation=0.5, p_reinsertion=0.75, p_swap=1.0, pressure_pa=3.5e3,
                           max_translation=0.5, max_rotation=0.4, seed=42, stream=k) for k in range(R)]
    out = {}
    for name, p in (("mixed", grx.GRX_MIXED), ("fp64", grx.GRX_FP64)):
        boxes = make_boxes(grx, system, R, stream.cuda_stream, cap_molecules=400)
        e0 = [total_energy(b) for b in boxes[:4]]
        for b in boxes[:4]:
            b.ewald_total()
        batch = grx.GcmcBatch(boxes, descs, p)
        if name == "mixed":
            shape, _ = batch.autotune(args.mc_steps)
            out["autotune"] = {"warps_per_box": shape[0], "chunk_mult": shape[1]}
        else:
            batch.set_shape(*shape)
        steps = args.steps if name == "mixed" else max(1, min(args.steps, 3))
        times, stats = timed_graph(torch, batch, stream, args.mc_steps, steps, args.warmup, flush)
        warm = timed_graph.warm_stats
        acc, _ = batch.stats()
        batch.close()
        te, _ = work_of(stats, 4, nfw)
        beta = grx.beta_from_temperature(300.0)
        drift = [beta * abs((total_energy(b) - e0[i]) - (warm[i].energy[3] + acc[i].energy[3]))
                 for i, b in enumerate(boxes[:4])]
        out[name] = {"value": te / sum(times), "loading": float(np.mean([s.n_molecules for s in acc])),
                     "drift_max_beta_abs": float(max(drift))}
        close_boxes(boxes)
    return {"metric": "CBMC trial energies/s", "value": out["mixed"]["value"], "unit": "trial_energies/s",
            "n_gpus": 1, "workload": "gcmc_tip4p_ew_hexagonal_864 (alpha 0.30, kmax 10/10/8, cutoff 11 A)",
            "chains": R, "mc_steps_per_step": args.mc_steps, "autotune": out["autotune"],
            "mixed": out["mixed"], "fp64": out["fp64"],
            "speedup_mixed_over_fp64": out["mixed"]["value"] / out["fp64"]["value"]}


def bench_cluster(args, grx, torch, stream, flush):
    """Single-chain latency on thread-block clusters: one CO2 box in a charged framework of
    5,000 or 20,000 atoms (the large serving jobs; automatic Ewald set-up), 200 GCMC steps per
    launch in mixed precision, on one 24-warp block and on clusters of 2, 4 and 8 CTAs. Each
    size runs the same chain (same seed and stream) from the same start; ms per launch by CUDA
    events, L2 flushed before each launch."""
    from graspa_gb300 import synth
    S = 200
    out = {}
    for natoms in (5000, 20000):
        s = synth.adsorbate_system("CO2", 7, n_atoms=natoms)
        nfw = s["comp_start"][1]
        d = grx.gcmc_desc(1, p_translation=0.25, p_rotation=0.5, p_reinsertion=0.5, p_swap=1.0, pressure_pa=1e5,
                          seed=42, stream=0)
        row = {}
        for cl in (1, 2, 4, 8):
            box = grx.Box(s, capacity=[nfw, 3 * 200])
            box.set_stream(stream.cuda_stream)
            box.ewald_total()
            batch = grx.GcmcBatch([box], [d], grx.GRX_MIXED)
            batch.set_shape(24, 1)
            if cl > 1:
                batch.set_cluster(cl)
            times, stats = timed_graph(torch, batch, stream, S, args.steps, args.warmup, flush)
            row[f"cluster_{cl}_ms"] = 1000 * sum(times) / len(times)
            batch.close()
            box.close()
        row["speedup_8"] = row["cluster_1_ms"] / row["cluster_8_ms"]
        out[f"co2_{natoms}_atoms"] = row
    return {"metric": "ms per launch of 200 GCMC steps (one chain)", "unit": "ms", "higher_is_better": False,
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "workload": "single CO2 chain on 1 block and on clusters of 2/4/8 CTAs (mixed)", **out}


# ------------------------------------------------------------------ reference arm
def _oracle_params(desc):
    from oracle import oracle as O
    g = O.OraGcmc()
    g.component, g.ntrials, g.norient = desc.component, desc.ntrials, desc.norient
    g.p_translation, g.p_rotation, g.p_reinsertion, g.p_swap = (desc.p_translation, desc.p_rotation,
                                                                desc.p_reinsertion, desc.p_swap)
    for k in range(3):
        g.max_translation[k] = desc.max_translation[k]
        g.max_rotation[k] = desc.max_rotation[k]
    g.beta, g.pressure = desc.beta, desc.pressure
    g.fugacity_coeff, g.mol_fraction, g.ideal_rosenbluth = desc.fugacity_coeff, desc.mol_fraction, 1.0
    g.seed, g.stream = desc.seed, desc.stream
    return g


def oracle_chains(system, descs):
    """Resident FP64 oracle chains, one per move set: atoms, molecule counts and both
    structure factors stay in host memory across calls, and the full FP64 Ewald totals
    (framework exclusion included) are computed once here, outside any timing, as the
    GPU arm computes its framework S(k) once before timing."""
    from oracle import oracle as O
    osys = O.OracleSystem(system)
    _, s_fw, s_ads = osys.ewald_total(list(system["molsize"]))
    cap = [system["comp_start"][1], 3 * 160]
    return [O.OracleChain(osys, _oracle_params(d), cap, ewald=(s_fw, s_ads)) for d in descs]


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the platform string)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()


def run_oracle_slices(chains, first, n_step, threads):
    """n_step moves of every resident chain, one chain per host thread; returns (stats, s)."""
    t0 = time.perf_counter()
    with concurrent.futures.ThreadPoolExecutor(threads) as ex:
        res = list(ex.map(lambda c: c.run(first, n_step)[0], chains))
    return res, time.perf_counter() - t0


def cpu_gcmc_rate(seconds, threads=None):
    """The FP64 oracle on the same GCMC workload, one resident chain per host thread, for
    about `seconds` of moves (set-up excluded). Returns (trial energies/s, trial energies,
    seconds, threads, chains, steps)."""
    from graspa_gb300 import grx
    from oracle import oracle as O
    O.lib()
    system = co2_system()
    threads = threads or os.cpu_count() or 1
    chains = oracle_chains(system, gcmc_descs(grx, threads))
    # per-step cost of the moves alone, on resident state (warm-up steps of every chain)
    warm = 40
    _, dt = run_oracle_slices(chains, 0, warm, threads)
    chunk = int(max(20, min(5000, 0.5 * warm / max(dt, 1e-6))))   # slices of about half a second
    first, steps, te, tot = warm, 0, 0.0, 0.0
    while tot < seconds:
        res, dt = run_oracle_slices(chains, first, chunk, threads)
        first += chunk
        steps += chunk
        tot += dt
        te += work_of(res, 3, system["comp_start"][1])[0]
    return te / tot, te, tot, threads, threads, steps


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from graspa_gb300 import grx
    from oracle import oracle as O
    O.lib()
    system = co2_system()
    threads = os.cpu_count() or 1
    chains = oracle_chains(system, gcmc_descs(grx, threads))
    _, dt = run_oracle_slices(chains, 0, 20, threads)
    per_step = dt / 20
    first = 20
    n_step = int(max(10, min(args.mc_steps, 4.0 / max(per_step, 1e-9))))
    times, te_tot = [], 0.0
    for i in range(args.warmup + args.steps):
        res, dt = run_oracle_slices(chains, first, n_step, threads)
        first += n_step
        if i >= args.warmup:
            times.append(dt)
            te_tot += work_of(res, 3, system["comp_start"][1])[0]
    tot = sum(times)
    value = te_tot / tot
    model = cpu_model()
    line = {
        "metric": "CBMC trial energies/s", "value": value, "unit": "trial_energies/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * tot / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Philox)",
        "config": {"workload": "gcmc_co2_silica_3456 (1:1:1:1 translation/rotation/insertion/deletion, k=10)",
                   "chains": threads, "mc_steps_per_step": n_step},
        "cpu_baseline": {"value": value, "unit": "trial_energies/s", "cores": threads, "cpu_model": model,
                         "kind": "port",
                         "sample": f"{threads} resident chains x {n_step} GCMC steps per step (state and "
                                   "structure factors kept across steps, Ewald totals computed once before "
                                   f"timing), FP64 C++ oracle, one chain per thread on {model}"},
        "e2e": {"value": value, "unit": "trial_energies/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="grx", choices=["grx", "reference"])
    ap.add_argument("--workload", default="gcmc", choices=["gcmc", "widom", "batched", "water", "serving", "cluster"])
    ap.add_argument("--chains", type=int, default=0, help="GCMC chains (default: three per SM)")
    ap.add_argument("--mc-steps", type=int, default=100, help="Monte Carlo steps of every chain per step")
    ap.add_argument("--insertions", type=int, default=20000, help="Widom insertions per launch")
    ap.add_argument("--widom-steps", type=int, default=5)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--serve-jobs", type=int, default=500, help="jobs per stream (the full serving sweep: 10000)")
    ap.add_argument("--serve-rate-fractions", type=float, nargs="*", default=[0.5, 0.9],
                    help="Poisson arrival rates swept, as fractions of the measured saturation rate")
    ap.add_argument("--serve-slots", type=int, default=456, help="resident jobs (three chains per SM)")
    ap.add_argument("--serve-batching", type=int, default=1,
                    help="1: resident GCMC jobs advance together in shared rounds (grx_server gcmc_batching)")
    ap.add_argument("--serve-hbm-gb", type=float, default=16.0)
    ap.add_argument("--serve-gcmc-cycles", type=int, default=2000, help="GCMC cycles of 20 steps per serving job")
    ap.add_argument("--serve-gcmc-slice", type=int, default=800,
                    help="steps per launch (batching: per round, for a job of 1000 pair evaluations per step)")
    ap.add_argument("--serve-fp64-jobs", type=int, default=24)
    ap.add_argument("--serve-fp64-cycles", type=int, default=50, help="GCMC cycles of the plain FP64 sample's jobs")
    ap.add_argument("--serve-cluster-atoms", type=int, default=1000,
                    help="GCMC jobs of N atoms run on clusters of up to N / this many CTAs (0: off)")
    ap.add_argument("--profile", action="store_true", help="only the timed mixed GCMC steps (launch lists)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_grx(args)


if __name__ == "__main__":
    main()
