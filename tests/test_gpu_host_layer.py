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


@pytest.mark.parametrize("mode,tail", [("host", 0.0), ("device", 0.0), ("host", -200.0), ("device", -200.0)])
def test_host_layer_gcmc_matches_oracle(grx_lib, tmp_path, mode, tail):
    s = co2_system(n_co2=4)
    d = params(grx_lib, pressure_pa=1e6, tail_insert=tail)
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


def _rotate(v, u, w1, w2):
    import ctypes
    a = np.ascontiguousarray(v, dtype=np.float64).copy()
    O.lib().ora_rotate_quaternion(O._d(a), ctypes.c_double(u), ctypes.c_double(w1), ctypes.c_double(w2))
    return a


def _close(a, b, tol=1e-9):
    return abs(a - b) <= tol * max(abs(b), 1e-300)


def test_host_layer_identity_swap(grx_lib, tmp_path):
    """IdentitySwapMove (mc_swap_moves.h:199-420) in a CO2 + N2 mixture through the host layer.
    The first move is recomputed with the oracle: component and molecule picks from the Philox
    draw; the new species' single first-bead trial on the old molecule's first bead with the old
    molecule excluded (not averaged); its orientations (stored molecule 0 rotated by the
    orientation draws) and their selection; the old molecule's retrace (trial 0 its current
    configuration, the others from the retrace draws); the identity-swap Fourier delta; then
    Pacc = N_old / (N_new + 1) * W_new / W_old. Weights, Pacc and the Fourier delta agree to
    1e-9 and the decision is the same. Over the run the molecule count is conserved and the
    accepted energies match the recomputed FP64 totals."""
    from graspa_gb300 import synth
    s = synth.silica_co2_n2(n_co2=4, n_n2=4)
    d = params(grx_lib, pressure_pa=1e6)
    f = os.path.join(str(tmp_path), "system.txt")
    cs = s["comp_start"]
    system_file.write_system(f, s, [cs[1], CAP, CAP], d, precision=grx.GRX_FP64)
    r = subprocess.run([B.DRIVER, f, "swap", "60"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    out = system_file.parse_driver_output(r.stdout)
    beta = d.beta
    P, Q, T = s["pos"], s["charge"], s["type"]
    w = O.draw(d.seed, d.stream, 0, 4099)
    old = [1, 2][min(1, int(O.u01(w[0]) * 2))]
    new = 1 + min(1, int(O.u01(w[1]) * 2))
    oldmol = int(O.u01(w[2]) * 4)
    row = out["swap"][0]
    assert (int(row[0]), int(row[1]), int(row[2])) == (old, new, oldmol)
    S = O.OracleSystem(s)
    o0 = cs[old] + 3 * oldmol
    old_pos, old_q, old_t = P[o0:o0 + 3], Q[o0:o0 + 3], T[o0:o0 + 3]
    new_q, new_t = Q[cs[new]:cs[new] + 3], T[cs[new]:cs[new] + 3]
    fb = old_pos[0]
    # growth of the new species: one first-bead trial, ten orientations, the old molecule excluded
    e, fl = S.trial_energies(fb, [1.0], [new_q[0]], [1.0], [new_t[0]], 4, 1, 1, new, old, oldmol)
    assert fl[0] == 0
    W_new = np.exp(-beta * e[0].sum())
    vec = P[cs[new] + 1:cs[new] + 3] - P[cs[new]]
    tp = []
    for o in range(10):
        wo = O.draw(d.seed, d.stream, 0, 1024 + o)
        tp += [fb + _rotate(vec[a], O.u01(wo[0]), O.u01(wo[1]), O.u01(wo[2])) for a in range(2)]
    e, fl = S.trial_energies(np.array(tp), np.ones(20), np.tile(new_q[1:], 10), np.ones(20), np.tile(new_t[1:], 10),
                             4, 10, 2, new, old, oldmol)
    ok = np.flatnonzero(fl == 0)
    lw = -beta * e[ok].sum(1)
    orient = ok[O.select_trial(lw, O.u01(O.draw(d.seed, d.stream, 0, 2048)[1]))]
    W_new *= np.exp(lw).sum() / 10
    grown = np.array([fb, tp[2 * orient], tp[2 * orient + 1]])
    # retrace of the old molecule
    e, fl = S.trial_energies(fb, [1.0], [old_q[0]], [1.0], [old_t[0]], oldmol, 1, 1, old)
    W_old = np.exp(-beta * e[0].sum())
    vec = P[cs[old] + 1:cs[old] + 3] - P[cs[old]]
    tp = [old_pos[1], old_pos[2]]
    for o in range(1, 10):
        wo = O.draw(d.seed, d.stream, 0, 3072 + o)
        tp += [fb + _rotate(vec[a], O.u01(wo[0]), O.u01(wo[1]), O.u01(wo[2])) for a in range(2)]
    e, fl = S.trial_energies(np.array(tp), np.ones(20), np.tile(old_q[1:], 10), np.ones(20), np.tile(old_t[1:], 10),
                             oldmol, 10, 2, old)
    W_old *= np.exp(-beta * e[fl == 0].sum(1)).sum() / 10
    # Fourier delta: the old molecule out, the grown one in (rigid exclusions of both species)
    _, s_fw, s_ads = S.ewald_total([cs[1], 3, 3])
    ex = {c: sum(S.rigid_exclusion(P[cs[c]:cs[c] + 3], Q[cs[c]:cs[c] + 3], np.ones(3))) for c in (1, 2)}
    ew, _ = S.ewald_delta_identity_swap(s_ads, s_fw, old_pos, old_q, grown, new_q, ex[new], ex[old])
    W_new *= np.exp(-beta * (ew[0] + ew[1]))
    pacc = 4.0 / 5.0 * W_new / W_old
    assert _close(row[4], W_new) and _close(row[5], W_old) and _close(row[6], pacc)
    assert _close(row[7], ew[0]) and _close(row[8], ew[1])
    assert row[3] == float(O.u01(w[3]) < pacc)
    # the run: counts conserved, swaps accepted both ways, drift
    counts = out["count"]
    assert counts[1][0] + counts[2][0] == 8
    assert counts[1][1] + counts[2][1] >= 2 and counts[1][1] + counts[2][1] == counts[1][2] + counts[2][2]
    assert abs(out["drift"]) <= 1e-8 * max(1.0, abs(out["energy_sum"])) + 1e-6


def test_host_layer_gibbs_particle_transfer(grx_lib, tmp_path):
    """GibbsParticleTransfer (mc_swap_moves.h:51-176) between a CO2 box and an identical copy.
    First move: the box choice and the deleted molecule follow the Philox draw; the insertion
    weight equals the device Widom kernel's weight for the inserting box's stream (box b draws
    from stream + b * 2^24) and move index; Pacc = W_ins N_B V_A / (W_del (N_A + 1) V_B) and the
    decision follows it. Over the run the total count is conserved, transfers are accepted and
    both boxes' accepted energies match their recomputed totals."""
    s = co2_system(n_co2=8)
    d = params(grx_lib, pressure_pa=1e6)
    out = run_driver(str(tmp_path), s, d, "transfer", 40)
    w = O.draw(d.seed, d.stream, 0, 4100)
    A = 1 if O.u01(w[0]) > 0.5 else 0
    row = out["transfer"][0]
    assert int(row[0]) == A and int(row[1]) == int(O.u01(w[1]) * 8)
    box = grx_lib.Box(s, capacity=[s["comp_start"][1], CAP])
    box.ewald_total()
    wd = grx_lib.widom_desc(s, 1, ntrials=d.ntrials, norient=d.norient, seed=d.seed, stream=d.stream + (A << 24))
    res = box.widom(wd, 0, 1, grx_lib.GRX_FP64)
    assert res["success"][0] != 0 and _close(row[3], res["rosenbluth"][0], 1e-10)
    pacc = row[3] * 8 / (row[4] * 9)
    assert _close(row[5], pacc, 1e-12) and row[2] == float(O.u01(w[2]) < pacc)
    for r in out["transfer"]:
        assert r[6] + r[7] == 16
    assert out["transfer_attempts"] == 40.0 and out["transfer_accepted"] >= 1
    tol = 1e-8 * out["energy_scale"] + 1e-6
    assert abs(out["drift"]) <= tol and abs(out["drift_b"]) <= tol


@pytest.mark.parametrize("prec", ["GRX_FP64", "GRX_MIXED"])
def test_device_identity_swap_matches_host_layer(grx_lib, tmp_path, prec):
    """The identity swap of the device GCMC kernel (p_identity_swap) draws what the host
    layer's IdentitySwapMove draws (swap slot, orientation and retrace slots, selection word 1),
    so a device run of identity swaps only (every adsorbate component moved) equals the host
    driver's swaps move for move: FP64 the same counts, positions within 1e-9 A and energy sums
    within 1e-9 relative; mixed the same counts and positions, energies within beta*|dE| <= 1e-5."""
    from graspa_gb300 import synth
    s = synth.silica_co2_n2(n_co2=4, n_n2=4)
    d = params(grx_lib, pressure_pa=1e6)
    cs = s["comp_start"]
    f = os.path.join(str(tmp_path), "system.txt")
    system_file.write_system(f, s, [cs[1], CAP, CAP], d, precision=grx.GRX_FP64)
    fd = os.path.join(str(tmp_path), "system_dev.txt")
    system_file.write_system(fd, s, [cs[1], CAP, CAP], d, precision=getattr(grx, prec))
    runs = {}
    for mode, path in (("swap", f), ("swap_device", fd)):
        r = subprocess.run([B.DRIVER, path, mode, "60"], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        runs[mode] = system_file.parse_driver_output(r.stdout)
    host, dev = runs["swap"], runs["swap_device"]
    assert dev["count"] == host["count"]
    assert sum(v[1] for v in host["count"].values()) >= 2
    for a, b in zip(host["positions_all"], dev["positions_all"]):
        assert a.shape == b.shape and np.max(np.abs(a - b), initial=0.0) <= 1e-9
    if prec == "GRX_FP64":
        assert abs(dev["energy_sum"] - host["energy_sum"]) <= 1e-9 * max(1.0, abs(host["energy_sum"]))
        assert abs(dev["drift"]) <= 1e-8 * max(1.0, abs(dev["energy_sum"])) + 1e-6
    else:
        assert d.beta * abs(dev["energy_sum"] - host["energy_sum"]) <= 1e-5
