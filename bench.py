"""Benchmark: CBMC trial energies/s on one GB300 (batched mixed precision vs plain FP64).

Workload (one "step"): 20,000 CBMC Widom insertions of rigid CO2 into the
synthetic all-silica framework (2x2x3 cells of 20.09 x 19.74 x 13.14 A, 3456
atoms), 10 first-bead trial positions + 10 trial orientations per insertion,
shifted LJ + real-space Coulomb at 12 A, Ewald alpha 0.265 with kmax 9/9/6,
T = 300 K, Philox seed 42. One step evaluates 400,000 trial energies
(2.07e9 pair evaluations) plus 20,000 Ewald deltas.

`value`  : trial energies/s of the batched mixed-precision form, inputs resident.
`e2e`    : the same metric through the C ABI with host buffers (framework upload
           from pinned host memory, results read back), per step.
`fp64`   : the plain FP64 single-box form of the same workload (the denominator
           of the >= 5x target).
Reference arm (--impl reference): the FP64 CPU implementation of the same
routines (the test oracle, OpenMP on all host cores) on a bounded sample.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_INSERT = 20000
NTRIALS = 10
NORIENT = 10
FLOP_PER_PAIR_CHARGED = 70.0   # FP32-equivalent work model per pair (LJ + real Coulomb)
L2_FLUSH_BYTES = 256 << 20


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


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


def make_workload():
    from graspa_gb300 import synth
    return synth.silica_co2(seed=42)


def pairs_per_insertion(system):
    n_atoms = system["comp_start"][-1]
    chain = system["molsize"][1] - 1
    return (NTRIALS + NORIENT * chain) * n_atoms


def oracle_setup(system):
    from oracle import oracle as O
    S = O.OracleSystem(system)
    _, s_fw, s_ads = S.ewald_total(list(system["molsize"]))
    tm = system["templates"][1]
    mp = np.ascontiguousarray(tm["pos"].reshape(-1))
    mq = np.ascontiguousarray(tm["charge"], dtype=np.float64)
    mt = np.ascontiguousarray(tm["type"], dtype=np.int64)
    intra, self_ = S.rigid_exclusion(mp, mq, np.ones(3))
    from graspa_gb300 import grx
    w = O.OraWidom()
    w.component, w.molsize = 1, 3
    w.mol_pos, w.mol_charge, w.mol_type = O._d(mp), O._d(mq), O._i(mt)
    w.scale = w.scale_coul = 1.0
    w.ntrials, w.norient, w.new_molid = NTRIALS, NORIENT, 0
    w.beta = grx.beta_from_temperature(300.0)
    w.excl_intra, w.excl_self = intra, self_
    w.rigid, w.has_charge = 1, 1
    w.seed, w.stream = 42, 0
    return S, s_fw, s_ads, w, (mp, mq, mt)


def cpu_rate(system, seconds, first_move=10 ** 9):
    """Time the FP64 OpenMP oracle on a bounded sample; returns (trial energies/s, sample, cores)."""
    from oracle import oracle as O
    S, s_fw, s_ads, w, keep = oracle_setup(system)
    cores = int(O.lib().ora_max_threads())
    n = max(cores, 16)
    t0 = time.perf_counter()
    S.widom(w, s_fw, s_ads, first_move, n)
    dt = time.perf_counter() - t0
    n2 = int(max(n, min(200000, n * seconds / max(dt, 1e-6))))
    t0 = time.perf_counter()
    S.widom(w, s_fw, s_ads, first_move + n, n2)
    dt2 = time.perf_counter() - t0
    return (NTRIALS + NORIENT) * n2 / dt2, n2, cores, dt2


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    system = make_workload()
    from oracle import oracle as O
    S, s_fw, s_ads, w, keep = oracle_setup(system)
    cores = int(O.lib().ora_max_threads())
    # calibrate a per-step sample of about 4 s of CPU work
    t0 = time.perf_counter()
    S.widom(w, s_fw, s_ads, 0, max(cores, 16))
    per = (time.perf_counter() - t0) / max(cores, 16)
    n_step = int(max(cores, min(N_INSERT, 4.0 / max(per, 1e-9))))
    move = 1000
    for _ in range(args.warmup):
        S.widom(w, s_fw, s_ads, move, n_step)
        move += n_step
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        S.widom(w, s_fw, s_ads, move, n_step)
        times.append(time.perf_counter() - t0)
        move += n_step
    tot = sum(times)
    value = (NTRIALS + NORIENT) * n_step * args.steps / tot
    line = {
        "metric": "CBMC trial energies/s", "value": value, "unit": "trial_energies/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * tot / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Philox)",
        "config": {"workload": "widom_co2_silica_3456", "insertions_per_step": n_step,
                   "full_step_insertions": N_INSERT, "trials": NTRIALS, "orientations": NORIENT},
        "cpu_baseline": {"value": value, "unit": "trial_energies/s", "cores": cores, "kind": "port",
                         "sample": f"{n_step} insertions per step (of {N_INSERT}), FP64 C++ OpenMP oracle"},
        "e2e": {"value": value, "unit": "trial_energies/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def accuracy_check(box, grx, system, n=200):
    """Mixed / FP32 vs the FP64 oracle on the first n insertions of the stream."""
    from oracle import oracle as O
    S, s_fw, s_ads, w, keep = oracle_setup(system)
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
        tot_g = Eg[r].reshape(-1, 2, 4).sum(2)
        tot_r = E[r].reshape(-1, 2, 4).sum(2)
        dE = np.abs(tot_g - tot_r)
        out[name] = {
            "selection_agreement": float(same.mean()),
            "max_rel_rosenbluth": float(np.max(np.abs(g["rosenbluth"][r] - R[r]) / R[r])) if r.any() else 0.0,
            "max_beta_dE": float(beta * dE.max()) if dE.size else 0.0,
            "max_rel_energy_vs_max_E_kT": float(np.max(dE / np.maximum(np.abs(tot_r), 1.0 / beta))) if dE.size else 0.0,
        }
    return out


def run_grx(args):
    global N_INSERT
    N_INSERT = args.insertions
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from graspa_gb300 import grx
    grx.build()
    system = make_workload()
    nfw = system["comp_start"][1]
    box = grx.Box(system, capacity=[nfw, 3 * 64])
    stream = torch.cuda.current_stream()
    box.set_stream(stream.cuda_stream)
    box.ewald_total()
    prec = grx.PRECISIONS[args.precision]
    d = grx.widom_desc(system, 1, NTRIALS, NORIENT, seed=42, stream=rank)
    res_dev = torch.empty(N_INSERT * grx.WIDOM_RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    pairs = pairs_per_insertion(system) * N_INSERT
    te_per_step = (NTRIALS + NORIENT) * N_INSERT

    def timed_steps(p, steps, warmup, first_move):
        move = first_move
        for _ in range(warmup):
            box.widom_async(d, move, N_INSERT, p, res_dev.data_ptr())
            move += N_INSERT
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        times = []
        launches0 = grx.launch_count()
        for _ in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            box.widom_async(d, move, N_INSERT, p, res_dev.data_ptr())
            e1.record(stream)
            move += N_INSERT
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1000.0)
        torch.cuda.synchronize()
        launches = grx.launch_count() - launches0
        tot = sum(times)
        if dist:
            t = torch.tensor([tot], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            tot = float(t.item())
            dist.barrier()
        return tot, times, launches

    clocks = ClockSampler(local)
    clocks.start()
    tot, times, launches = timed_steps(prec, args.steps, args.warmup, 0)
    clk = clocks.stop()
    value = te_per_step * args.steps * world / tot
    t_launch = float(np.mean(times))
    if args.profile:
        if rank == 0:
            print(json.dumps({"profile_run": True, "value": value, "ms_per_step": 1000 * tot / args.steps,
                              "insertions": N_INSERT, "launches": int(launches)}), flush=True)
        box.close()
        return

    # plain FP64 single-box form of the same workload (fewer steps: it is slower)
    fp64_steps = max(1, min(args.steps, 3))
    tot64, _, _ = timed_steps(grx.GRX_FP64, fp64_steps, 1, 10 ** 8)
    fp64_value = te_per_step * fp64_steps * world / tot64

    # end to end through the C ABI with host buffers
    pinned = torch.empty(nfw * 8 * 8, dtype=torch.uint8, pin_memory=True)
    host_sys = dict(system)
    pn = pinned.numpy().view(np.float64)
    pn[: 3 * nfw] = np.asarray(system["pos"][:nfw]).reshape(-1)
    host_sys["pos"] = pn[: 3 * nfw].reshape(-1, 3)
    host_res = torch.empty(N_INSERT * grx.WIDOM_RESULT_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)
    res_view = host_res.numpy().view(grx.WIDOM_RESULT_DTYPE)
    box.system = host_sys
    e2e_times = []
    move = 2 * 10 ** 8
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        box.set_component(0)
        box.widom(d, move, N_INSERT, prec=prec, out=res_view)
        dt = time.perf_counter() - t0
        move += N_INSERT
        if i >= args.warmup:
            e2e_times.append(dt)
    box.system = system
    e2e_value = te_per_step * world / float(np.mean(e2e_times))
    h2d = nfw * (3 * 8 + 8 + 8 + 8 + 8 + 8)
    d2h = N_INSERT * grx.WIDOM_RESULT_DTYPE.itemsize

    if rank == 0:
        acc = accuracy_check(box, grx, system)
        cpu_val, cpu_n, cores, cpu_dt = cpu_rate(system, args.cpu_seconds)
        sm_mhz = clk["sm_mhz"] or 2070.0
        peak_fp32 = 152 * 128 * 2 * 2070e6 / 1e12
        achieved = FLOP_PER_PAIR_CHARGED * pairs / t_launch / 1e12
        line = {
            "metric": "CBMC trial energies/s", "value": value, "unit": "trial_energies/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32+fp64" if args.precision == "mixed" else args.precision,
            "data": "synthetic (seeded Philox framework, Philox trial stream)",
            "config": {"workload": "widom_co2_silica_3456", "insertions_per_step": N_INSERT, "trials": NTRIALS,
                       "orientations": NORIENT, "framework_atoms": nfw, "precision": args.precision,
                       "pairs_per_step": pairs, "l2": "flushed between steps (256 MB write)",
                       "parallelism": f"replicas x{world}"},
            "fp64": {"value": fp64_value, "unit": "trial_energies/s", "steps": fp64_steps,
                     "speedup_mixed_over_fp64": value / fp64_value},
            "accuracy_vs_fp64_oracle": acc,
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak_fp32, "unit": "TFLOP/s",
                         "frac": achieved / peak_fp32, "traffic": None,
                         "peak_kind": "nominal FP32 CUDA-core peak at 2070 MHz (no measured FP32 peak exists)",
                         "model": f"{FLOP_PER_PAIR_CHARGED:.0f} FLOP/pair x {pairs} pairs per launch"},
            "cpu_baseline": {"value": cpu_val, "unit": "trial_energies/s", "cores": cores, "kind": "port",
                             "sample": f"{cpu_n} insertions ({cpu_dt:.1f} s), FP64 C++ OpenMP oracle"},
            "e2e": {"value": e2e_value, "unit": "trial_energies/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": int(launches),
            "clocks": {"sm_mhz": clk["sm_mhz"], "sm_max_mhz": clk["sm_max_mhz"], "reasons": clk["reasons"]},
        }
        print(json.dumps(line), flush=True)
    box.close()
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="grx", choices=["grx", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64", "fp32"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--insertions", type=int, default=N_INSERT,
                    help="insertions per step (the benchmark workload is 20000)")
    ap.add_argument("--profile", action="store_true",
                    help="only the timed mixed-precision steps (for profiler launch lists)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_grx(args)


if __name__ == "__main__":
    main()
