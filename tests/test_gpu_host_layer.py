"""The C++ host layer (graspa_gb300/host: gRASPA's structs and move drivers over
the C ABI) on the GPU. Its example driver is run as a separate process on a system
file, in three modes:
  host   : RunMoves one move at a time (every energy call a libgrx call)
  device : the same moves in one grx_gcmc_run
  widom  : InsertionMove::WidomMove + the Widom statistics
FP64 host-driven moves take the same decisions as the FP64 oracle (identical move
counts, positions within 1e-9 A); the accepted-energy sum matches the drift check
of the recomputed FP64 totals to 1e-8 relative; Widom Rosenbluth weights match the
device Widom kernel to 1e-10 relative (same Philox draws, different summation order).
"""
import os
import subprocess

import numpy as np
import pytest

from graspa_gb300 import build as B
from graspa_gb300 import grx, system_file
from oracle import oracle as O
from tests.systems import co2_system
from tests.test_gpu_gcmc import ora_params, params

pytestmark = pytest.mark.gpu

CAP = 3 * 64


def run_driver(tmp_path, s, d, mode, n, prec=grx.GRX_FP64):
    f = os.path.join(tmp_path, "system.txt")
    system_file.write_system(f, s, [s["comp_start"][1], CAP], d, precision=prec)
    r = subprocess.run([B.DRIVER, f, mode, str(n)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return system_file.parse_driver_output(r.stdout)


@pytest.mark.parametrize("mode", ["host", "device"])
def test_host_layer_gcmc_matches_oracle(grx_lib, tmp_path, mode):
    s = co2_system(n_co2=4)
    d = params(grx_lib, pressure_pa=1e6)
    out = run_driver(str(tmp_path), s, d, mode, 150)
    ost, after, _ = O.OracleSystem(s).gcmc(ora_params(d), [s["comp_start"][1], CAP], 0, 150)
    assert out["attempts"] == list(ost.attempts)
    assert out["accepted"] == list(ost.accepted)
    assert int(out["n_molecules"]) == ost.n_molecules
    nfw = s["comp_start"][1]
    assert np.max(np.abs(out["positions"] - after["pos"][nfw:])) <= 1e-9
    assert abs(out["energy_sum"] - ost.energy[3]) <= 1e-9 * max(1.0, abs(ost.energy[3]))
    assert abs(out["drift"]) <= 1e-8 * max(1.0, abs(out["energy_sum"])) + 1e-6


def test_host_layer_widom_matches_device_kernel(grx_lib, tmp_path):
    s = co2_system(n_co2=0)
    d = params(grx_lib)
    out = run_driver(str(tmp_path), s, d, "widom", 40)
    box = grx_lib.Box(s, capacity=[s["comp_start"][1], CAP])
    box.ewald_total()
    wd = grx_lib.widom_desc(s, 1, ntrials=d.ntrials, norient=d.norient, seed=d.seed, stream=d.stream)
    res = box.widom(wd, 0, 40, grx_lib.GRX_FP64)
    W = np.array(out["W"])
    ref = res["rosenbluth"] * (res["success"] != 0)
    assert np.all(np.abs(W - ref) <= 1e-10 * np.maximum(np.abs(ref), 1e-300))
    # ComputeFugacity: mu_ex = -T ln<W> (block averages of equal blocks = plain mean)
    assert abs(out["widom_average_rosenbluth"] - W.mean()) <= 1e-12 * W.mean()
    assert abs(out["widom_mu_ex_K"] + 300.0 * np.log(W.mean())) <= 1e-9


def test_write_and_remove_molecule(grx_lib):
    """grx_box_write_molecule / grx_box_remove_molecule keep the device box equal
    to the same edit of the system dict (FP64 totals against the oracle)."""
    s = co2_system(n_co2=3)
    nfw = s["comp_start"][1]
    box = grx_lib.Box(s, capacity=[nfw, CAP])
    P = s["pos"].reshape(-1, 3)
    mols = [P[nfw + 3 * m: nfw + 3 * m + 3].copy() for m in range(3)]
    tm = s["templates"][1]
    box.remove_molecule(1, 0)          # the last molecule moves into slot 0
    new = mols[1] + np.array([0.5, -0.3, 0.2])
    box.write_molecule(1, 1, new, tm["charge"], tm["type"])          # overwrite in place
    box.write_molecule(1, 2, mols[0], tm["charge"], tm["type"])      # append
    expect = np.concatenate([mols[2], new, mols[0]])
    assert np.array_equal(box.positions(1), expect)
    s2 = dict(s)
    s2["pos"] = np.concatenate([P[:nfw], expect])
    t = box.total_energy()
    ref = O.OracleSystem(s2).vdw_real_total()
    got = [t[k] for k in ("hh_vdw", "hh_real", "hg_vdw", "hg_real", "gg_vdw", "gg_real")]
    assert np.all(np.abs(np.array(got) - ref) <= 1e-10 * np.maximum(np.abs(ref), 1.0))
    with pytest.raises(grx_lib.GrxError):
        box.write_molecule(1, 5, new, tm["charge"], tm["type"])   # beyond the count
    with pytest.raises(grx_lib.GrxError):
        box.remove_molecule(1, 3)


def test_host_layer_cbcf_lambda_change(grx_lib, tmp_path):
    """CBCF_LambdaChange (mc_cbcfc.h:20-124) through the host layer: molecule 0 goes
    1 -> 0.4 (lambda change), then 0.4 -> 0.1 as a CB/CFC deletion's second step whose
    Fourier part starts from the staged vector; pair and Fourier parts against the
    oracle (FP64, 1e-10 relative)."""
    import ctypes
    s = co2_system(n_co2=4)
    d = params(grx_lib, pressure_pa=1e6)
    out = run_driver(str(tmp_path), s, d, "lambda", 0)
    nfw = s["comp_start"][1]
    S = O.OracleSystem(s)
    _, s_fw, s_ads = S.ewald_total([nfw, 3])
    oi, os_ = S.rigid_exclusion(s["templates"][1]["pos"], s["templates"][1]["charge"], np.ones(3))
    pos, q, ty = s["pos"][nfw:nfw + 3], s["charge"][nfw:nfw + 3], s["type"][nfw:nfw + 3]
    staged = None
    for k, (lo, ln) in enumerate(((1.0, 0.4), (0.4, 0.1))):
        row = out["lambda"][k]
        assert row[0] == 1.0
        keep = [np.ascontiguousarray(pos.reshape(-1)), np.full(3, lo), np.ascontiguousarray(q), np.full(3, ln),
                np.ascontiguousarray(ty, dtype=np.int64)]
        to = O.OraTrials(1, 3, O._d(keep[0]), O._d(keep[1]), O._d(keep[2]), O._d(keep[1]), O._i(keep[4]), 0)
        tn = O.OraTrials(1, 3, O._d(keep[0]), O._d(keep[3]), O._d(keep[2]), O._d(keep[3]), O._i(keep[4]), 0)
        ref = np.zeros(6)
        rf = np.zeros(1, dtype=np.uint8)
        O.lib().ora_single_body(ctypes.byref(S.box), ctypes.byref(S.ff), ctypes.byref(S.atoms), ctypes.byref(to),
                                ctypes.byref(tn), 1, 1, 1, O._d(ref), rf.ctypes.data_as(O._u8p))
        got_pair = np.array(row[1:5])
        assert np.all(np.abs(got_pair - ref[2:6]) <= 1e-10 * np.maximum(np.abs(ref[2:6]), 1.0))
        ew, staged = S.ewald_delta_lambda(s_ads, s_fw, pos, q, lo, ln, oi + os_, s_temp=staged)
        assert abs(row[5] - ew[0]) <= 1e-10 * max(abs(ew[0]), 1.0) and abs(row[6] - ew[1]) <= 1e-10 * max(abs(ew[1]), 1.0)


def _round_away(x):
    return np.where(x >= 0, np.floor(x + 0.5), np.ceil(x - 0.5))


def test_host_layer_volume_move(grx_lib, tmp_path):
    """VolumeMove (mc_box.h:191-291) through the host layer: the first trial's volume is
    the Philox draw, its FP64 total equals the oracle's totals of the scaled box (cell and
    adsorbate molecules scaled, first bead by s, the other atoms at their minimum-image
    offsets; the framework unscaled, as in the reference), and the acceptance follows
    exp((N+1) ln(V'/V) - beta (dE + P dV)). Over several moves the accepted energies
    match the recomputed totals (drift)."""
    s = co2_system(n_co2=10)
    d = params(grx_lib, pressure_pa=2e7)
    out = run_driver(str(tmp_path), s, d, "volume", 8)
    nfw = s["comp_start"][1]
    cell = np.array(s["cell"], dtype=np.float64).reshape(3, 3)
    V0 = abs(np.linalg.det(cell))
    acc, newV, e_trial, overlap, e_before = out["volume"][0]
    w = O.draw(d.seed, d.stream, 0, 4098)  # GRX_SLOT_VOLUME of move 0
    V1 = np.exp(np.log(V0) + 0.05 * 2.0 * (O.u01(w[0]) - 0.5))
    assert abs(newV - V1) <= 1e-12 * V1
    sc = np.cbrt(V1 / V0)
    s2 = dict(s)
    s2["cell"] = list(np.array(s["cell"], dtype=np.float64) * sc)
    pos = np.array(s["pos"], dtype=np.float64).copy()
    Lx, Ly, Lz = s["cell"][0], s["cell"][4], s["cell"][8]
    for m in range(10):
        a0 = nfw + 3 * m
        p0 = pos[a0].copy()
        v = pos[a0:a0 + 3] - p0
        v -= _round_away(v / np.array([Lx, Ly, Lz])) * np.array([Lx, Ly, Lz])
        pos[a0:a0 + 3] = p0 * sc + v
    s2["pos"] = pos
    S2 = O.OracleSystem(s2)
    vr = S2.vdw_real_total()
    ew, _, _ = S2.ewald_total([nfw, 3])
    total = vr.sum() + (ew[1] - ew[4] + ew[6]) + ew[2] + (ew[0] + ew[1] - ew[3] + ew[5])
    assert abs(e_trial - total) <= 1e-9 * abs(total), (e_trial, total)
    assert overlap == 0.0
    lp = 11.0 * np.log(V1 / V0) - d.beta * (e_trial - e_before + d.pressure * (V1 - V0))
    pacc = np.exp(min(lp, 700.0))
    assert acc == float(O.u01(w[1]) < pacc)
    assert sum(r[0] for r in out["volume"]) >= 1  # some moves accepted at this pressure
    assert abs(out["drift"]) <= 1e-8 * max(1.0, abs(e_before)) + 1e-6


def test_host_layer_gibbs_volume_exchange(grx_lib, tmp_path):
    """NVTGibbsMove (mc_box.h:319-430) between a box and an identical copy: the total
    volume is conserved, both boxes' accepted energies match their recomputed totals."""
    s = co2_system(n_co2=10)
    d = params(grx_lib, pressure_pa=1e6)
    out = run_driver(str(tmp_path), s, d, "gibbs", 6)
    cell = np.array(s["cell"], dtype=np.float64).reshape(3, 3)
    V0 = abs(np.linalg.det(cell))
    for va, vb in out["gibbs"]:
        assert abs((va + vb) - 2 * V0) <= 1e-9 * V0
    assert out["gibbs_attempts"] == 6.0
    tol = 1e-8 * out["energy_scale"] + 1e-6
    assert abs(out["drift"]) <= tol and abs(out["drift_b"]) <= tol
