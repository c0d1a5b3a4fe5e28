"""GPU parity: every libgrx entry point against the FP64 oracle on the same inputs.

Tolerances (written per test):
  FP64   : |dE| <= 1e-12 * max(|E|, 1)          (the FP64 path's bar)
  MIXED  : beta*|dE| <= 1e-6 and |dE| <= 1e-6 * max(|E|, kT)   (Boltzmann weights
           exp(-beta E) agree to 1e-6 relative; energies smaller than kT are
           measured against kT)
  Ewald structure factors: |dS| <= 1e-10 (the reference's CPU/GPU check,
           ewald_preparation.h:325)
  Rosenbluth selection: identical indices in FP64 (same Philox stream).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.systems import co2_system, nist_system

pytestmark = pytest.mark.gpu

BETA300 = None
# Mixed bars are asserted per energy component (host-guest and guest-guest VDW and real
# Coulomb separately), so errors of opposite sign in two components cannot cancel.


def beta(T=300.0):
    from graspa_gb300 import grx
    return grx.beta_from_temperature(T)


def fp64_close(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.all(np.abs(a - b) <= 1e-12 * np.maximum(np.abs(b), 1.0))


def mixed_close(a, b, T=300.0):
    a, b = np.asarray(a), np.asarray(b)
    kT = 1.0 / beta(T)
    d = np.abs(a - b)
    return np.all(beta(T) * d <= 1e-6) and np.all(d <= 1e-6 * np.maximum(np.abs(b), kT))


# ---------------------------------------------------------------- Ewald totals
@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_ewald_total_nist(grx_lib, n):
    s, e = nist_system(n)
    box = grx_lib.Box(s)
    ew = box.ewald_total()
    S = O.OracleSystem(s)
    ref, s_fw, s_ads = S.ewald_total([1, 3])
    assert abs(ew[0] - e["fourier_gg"]) < 1e-5
    assert abs(ew[3] - e["self_atoms"]) < 1e-5
    assert abs(ew[5] - e["intra_exclusion"]) < 1e-5
    assert int(ew[7]) == int(ref[7])
    for k in (0, 3, 5):
        assert abs(ew[k] - ref[k]) <= 1e-12 * abs(ref[k])
    g_fw, g_ads, g_tmp = box.structure_factors()
    _, act = S.ewald_active()
    m = np.repeat(act.astype(bool), 2)
    assert np.max(np.abs(g_ads[m] - s_ads[m])) <= 1e-10
    assert np.max(np.abs(g_fw[m] - s_fw[m])) <= 1e-10


@pytest.mark.parametrize("n", [1, 4])
def test_total_energy_nist(grx_lib, n):
    s, e = nist_system(n)
    box = grx_lib.Box(s)
    t = box.total_energy()
    assert abs(t["gg_vdw"] - e["gg_vdw"]) < 1e-5
    assert abs(t["gg_real"] - e["gg_real"]) < 1e-5
    ref = O.OracleSystem(s).vdw_real_total()
    assert fp64_close([t["gg_vdw"], t["gg_real"]], ref[4:6])
    # GGEwaldE of the reference's INITIAL summary: Fourier - self - intra exclusion
    assert abs(t["gg_ewald"] - (e["fourier_gg"] - e["self_atoms"] + e["intra_exclusion"])) < 2e-5
    intra, self_ = box.exclusion(1)
    assert abs(intra - e["rigid_exclusion_intra"]) < 1e-5
    assert abs(self_ - e["rigid_exclusion_self"]) < 1e-5


# ---------------------------------------------------------------- trial energies
def _random_beads(system, comp, ntrials, chainsize, rng):
    tm = system["templates"][comp]
    cell = np.array(system["cell"]).reshape(3, 3).T
    if chainsize == 1:
        pos = (cell @ rng.uniform(0, 1, (3, ntrials))).T
        q = np.full(ntrials, tm["charge"][0])
        ty = np.full(ntrials, tm["type"][0])
    else:
        first = cell @ rng.uniform(0, 1, 3)
        pos, q, ty = [], [], []
        for o in range(ntrials):
            v = tm["pos"][1:1 + chainsize] - tm["pos"][0]
            ang = rng.uniform(0, 2 * np.pi, 3)
            for a, x in enumerate(v):
                c, s_ = np.cos(ang), np.sin(ang)
                x = np.array([x[0], c[0] * x[1] - s_[0] * x[2], s_[0] * x[1] + c[0] * x[2]])
                x = np.array([c[1] * x[0] + s_[1] * x[2], x[1], -s_[1] * x[0] + c[1] * x[2]])
                pos.append(first + x)
                q.append(tm["charge"][1 + a])
                ty.append(tm["type"][1 + a])
        pos, q, ty = np.array(pos), np.array(q), np.array(ty)
    return pos, q, ty


@pytest.mark.parametrize("n_co2,chain", [(0, 1), (0, 2), (12, 1), (12, 2)])
def test_trial_energies_co2(grx_lib, n_co2, chain):
    s = co2_system(n_co2=n_co2)
    box = grx_lib.Box(s, capacity=[len(s["pos"]) - 3 * n_co2, 3 * 64])
    S = O.OracleSystem(s)
    rng = np.random.default_rng(3)
    ntr = 10
    newmol = n_co2
    for rep in range(3):
        pos, q, ty = _random_beads(s, 1, ntr, chain, rng)
        ref, rflag = S.trial_energies(pos, np.ones(len(q)), q, np.ones(len(q)), ty, newmol, ntr, chain, 1)
        e64, f64 = box.trial_energies(pos, q, ty, newmol, ntr, chain, 1, prec=grx_lib.GRX_FP64)
        assert np.array_equal(f64, rflag)
        assert fp64_close(e64, ref), np.max(np.abs(e64 - ref))
        em, fm = box.trial_energies(pos, q, ty, newmol, ntr, chain, 1, prec=grx_lib.GRX_MIXED)
        assert np.array_equal(fm, rflag)
        ok = rflag == 0
        # every component (host-guest / guest-guest x VDW / real Coulomb) on its own
        assert mixed_close(em[ok], ref[ok]), np.max(np.abs(em[ok] - ref[ok]))
        e32, f32 = box.trial_energies(pos, q, ty, newmol, ntr, chain, 1, prec=grx_lib.GRX_FP32)
        assert np.all(np.abs(e32[ok] - ref[ok]) <= 1e-2 * np.maximum(np.abs(ref[ok]), 1.0 / beta()))


def test_trial_energies_exclusions(grx_lib):
    """Atoms of the trial molecule (component, NewMol.MolID) and of ExcludeList[0]
    are skipped (VDW_Coulomb.cu:1274-1276)."""
    s = co2_system(n_co2=8)
    box = grx_lib.Box(s, capacity=[len(s["pos"]) - 24, 3 * 32])
    S = O.OracleSystem(s)
    rng = np.random.default_rng(5)
    pos, q, ty = _random_beads(s, 1, 6, 1, rng)
    for newmol, ec, em in [(3, -1, -1), (8, 1, 5), (2, 1, 2)]:
        ref, rf = S.trial_energies(pos, np.ones(6), q, np.ones(6), ty, newmol, 6, 1, 1, ec, em)
        e, f = box.trial_energies(pos, q, ty, newmol, 6, 1, 1, prec=grx_lib.GRX_FP64, excl_comp=ec, excl_molid=em)
        assert fp64_close(e, ref)
        assert np.array_equal(f, rf)


def test_trial_energies_triclinic_water(grx_lib):
    """Guest-guest trial energies in a triclinic NIST box, all precisions."""
    s, _ = nist_system(1)
    box = grx_lib.Box(s, capacity=[1, 1500])
    S = O.OracleSystem(s)
    rng = np.random.default_rng(11)
    cell = np.array(s["cell"]).reshape(3, 3).T
    pos = (cell @ rng.uniform(0, 1, (3, 16))).T
    q = np.full(16, -0.8476)
    ty = np.zeros(16, dtype=int)
    ref, rf = S.trial_energies(pos, np.ones(16), q, np.ones(16), ty, 400, 16, 1, 1)
    e, f = box.trial_energies(pos, q, ty, 400, 16, 1, 1, prec=grx_lib.GRX_FP64)
    assert fp64_close(e, ref) and np.array_equal(f, rf)
    em, fm = box.trial_energies(pos, q, ty, 400, 16, 1, 1, prec=grx_lib.GRX_MIXED)
    ok = rf == 0
    assert np.array_equal(fm, rf)
    assert mixed_close(em[ok], ref[ok])


# ---------------------------------------------------------------- single body
def test_single_body_translation(grx_lib):
    s = co2_system(n_co2=10)
    nfw = s["comp_start"][1]
    box = grx_lib.Box(s, capacity=[nfw, 3 * 16])
    S = O.OracleSystem(s)
    rng = np.random.default_rng(2)
    for mol in (0, 4, 9):
        a0 = nfw + 3 * mol
        old = dict(pos=s["pos"][a0:a0 + 3], charge=s["charge"][a0:a0 + 3], type=s["type"][a0:a0 + 3], molid=mol)
        new = dict(old)
        new["pos"] = old["pos"] + rng.uniform(-0.5, 0.5, 3)
        got, flag = box.single_body(old, new, 1, prec=grx_lib.GRX_FP64)
        to = O.OraTrials(1, 3, O._d(np.ascontiguousarray(old["pos"].reshape(-1))), O._d(np.ones(3)),
                         O._d(np.ascontiguousarray(old["charge"])), O._d(np.ones(3)),
                         O._i(np.ascontiguousarray(old["type"], dtype=np.int64)), mol)
        npos = np.ascontiguousarray(new["pos"].reshape(-1))
        tn = O.OraTrials(1, 3, O._d(npos), O._d(np.ones(3)), O._d(np.ascontiguousarray(new["charge"])),
                         O._d(np.ones(3)), O._i(np.ascontiguousarray(new["type"], dtype=np.int64)), mol)
        ref = np.zeros(6)
        rf = np.zeros(1, dtype=np.uint8)
        import ctypes
        O.lib().ora_single_body(ctypes.byref(S.box), ctypes.byref(S.ff), ctypes.byref(S.atoms), ctypes.byref(to),
                                ctypes.byref(tn), 1, 1, 1, O._d(ref), rf.ctypes.data_as(O._u8p))
        # new - old cancels: measure against the size of the two halves
        ref_new, ref_old = np.zeros(6), np.zeros(6)
        O.lib().ora_single_body(ctypes.byref(S.box), ctypes.byref(S.ff), ctypes.byref(S.atoms), ctypes.byref(to),
                                ctypes.byref(tn), 1, 1, 0, O._d(ref_new), rf.ctypes.data_as(O._u8p))
        O.lib().ora_single_body(ctypes.byref(S.box), ctypes.byref(S.ff), ctypes.byref(S.atoms), ctypes.byref(to),
                                ctypes.byref(tn), 1, 0, 1, O._d(ref_old), rf.ctypes.data_as(O._u8p))
        scale = np.maximum(np.abs(ref_new) + np.abs(ref_old), 1.0)
        assert np.all(np.abs(got - ref) <= 1e-12 * scale), (got - ref)
        O.lib().ora_single_body(ctypes.byref(S.box), ctypes.byref(S.ff), ctypes.byref(S.atoms), ctypes.byref(to),
                                ctypes.byref(tn), 1, 1, 1, O._d(ref), rf.ctypes.data_as(O._u8p))
        assert flag == rf[0]
        gm, _ = box.single_body(old, new, 1, prec=grx_lib.GRX_MIXED)
        assert np.all(beta() * np.abs(gm - ref) <= 1e-6), gm - ref   # per component


# ---------------------------------------------------------------- Ewald delta
def test_ewald_delta_and_commit(grx_lib):
    s = co2_system(n_co2=10)
    nfw = s["comp_start"][1]
    box = grx_lib.Box(s, capacity=[nfw, 3 * 16])
    box.ewald_total()
    S = O.OracleSystem(s)
    _, s_fw, s_ads = S.ewald_total([nfw, 3])
    intra, self_ = box.exclusion(1)
    oi, os_ = S.rigid_exclusion(s["templates"][1]["pos"], s["templates"][1]["charge"], np.ones(3))
    assert abs(intra - oi) <= 1e-12 * abs(oi) and abs(self_ - os_) <= 1e-12 * abs(os_)
    rng = np.random.default_rng(8)
    mol = 3
    a0 = nfw + 3 * mol
    old = s["pos"][a0:a0 + 3]
    qs = s["charge"][a0:a0 + 3]
    new = old + rng.uniform(-1, 1, 3)
    # translation
    got = box.ewald_delta(1, grx_lib.MOVE_TRANSLATION, old, qs, new, qs)
    ref, s_new = S.ewald_delta(s_ads, s_fw, old, qs, new, qs)
    assert abs(got[0] - ref[0]) <= 1e-10 * max(abs(ref[0]), 1) and abs(got[1] - 2 * ref[1]) <= 1e-10 * max(abs(ref[1]), 1)
    # insertion: same-type delta minus rigid exclusion
    got = box.ewald_delta(1, grx_lib.MOVE_INSERTION, np.zeros((0, 3)), np.zeros(0), new, qs)
    ref, _ = S.ewald_delta(s_ads, s_fw, np.zeros((0, 3)), np.zeros(0), new, qs)
    assert abs(got[0] - (ref[0] - (oi + os_))) <= 1e-10 * max(abs(ref[0]), 1)
    # deletion
    got = box.ewald_delta(1, grx_lib.MOVE_DELETION, old, qs, np.zeros((0, 3)), np.zeros(0))
    ref, s_del = S.ewald_delta(s_ads, s_fw, old, qs, np.zeros((0, 3)), np.zeros(0))
    assert abs(got[0] - (ref[0] + (oi + os_))) <= 1e-10 * max(abs(ref[0]), 1)
    box.ewald_commit(1)
    _, g_ads, _ = box.structure_factors()
    _, act = S.ewald_active()
    m = np.repeat(act.astype(bool), 2)
    assert np.max(np.abs(g_ads[m] - s_del[m])) <= 1e-10


# ---------------------------------------------------------------- CBMC selection
def test_cbmc_select_matches_oracle(grx_lib):
    rng = np.random.default_rng(4)
    for move in range(50):
        lw = rng.normal(0, 3, 10)
        for word in (0, 1):
            sel, tot = grx_lib.cbmc_select(lw, 42, 0, move, word)
            u = O.draw(42, 0, move, 2048)[word] / 2.0 ** 32
            assert sel == O.select_trial(lw, u)
            assert abs(tot - np.exp(lw).sum()) <= 1e-13 * np.exp(lw).sum()


# ---------------------------------------------------------------- batched Widom
def oracle_widom(s, comp, n, ntrials=10, norient=10, seed=42, stream=0, first_move=0, T=300.0):
    S = O.OracleSystem(s)
    nfw = s["comp_start"][s["nhost"]]
    molsize = list(s["molsize"])
    _, s_fw, s_ads = S.ewald_total(molsize)
    tm = s["templates"][comp]
    a0, a1 = s["comp_start"][comp], s["comp_start"][comp + 1]
    ms = len(tm["charge"])
    mp = np.ascontiguousarray((s["pos"][a0:a0 + ms] if a1 > a0 else tm["pos"]).reshape(-1), dtype=np.float64)
    mq = np.ascontiguousarray(tm["charge"], dtype=np.float64)
    mt = np.ascontiguousarray(tm["type"], dtype=np.int64)
    intra, self_ = S.rigid_exclusion(mp, mq, np.ones(ms))
    w = O.OraWidom()
    w.component = comp
    w.molsize = ms
    w.mol_pos, w.mol_charge, w.mol_type = O._d(mp), O._d(mq), O._i(mt)
    w.scale = w.scale_coul = 1.0
    w.ntrials, w.norient = ntrials, norient
    w.new_molid = (a1 - a0) // ms
    w.beta = beta(T)
    w.excl_intra, w.excl_self = intra, self_
    w.tail_delta = 0.0
    w.rigid = 1
    w.has_charge = int(np.any(mq != 0))
    w.seed, w.stream = seed, stream
    res = S.widom(w, s_fw, s_ads, first_move, n)
    keep = (mp, mq, mt)
    return res, keep


def _fields(res):
    return (np.array([r.rosenbluth for r in res]), np.array([r.sel_first for r in res]),
            np.array([r.sel_orient for r in res]), np.array([r.success for r in res]),
            np.array([list(r.e_first) + list(r.e_chain) + list(r.ewald) for r in res]))


@pytest.mark.parametrize("n_co2", [0, 10])
def test_widom_fp64_bitexact_selection(grx_lib, n_co2):
    s = co2_system(n_co2=n_co2)
    nfw = s["comp_start"][1]
    box = grx_lib.Box(s, capacity=[nfw, 3 * 32])
    box.ewald_total()
    n = 300
    ref, _ = oracle_widom(s, 1, n)
    R, sf, so, ok, E = _fields(ref)
    d = grx_lib.widom_desc(s, 1, 10, 10, seed=42)
    got = box.widom(d, 0, n, prec=grx_lib.GRX_FP64)
    assert np.array_equal(got["success"], ok)
    assert np.array_equal(got["sel_first"], sf)
    assert np.array_equal(got["sel_orient"], so)
    Eg = np.concatenate([got["e_first"], got["e_chain"], got["ewald"]], axis=1)
    assert np.all(np.abs(Eg - E) <= 1e-10 * np.maximum(np.abs(E), 1.0))
    assert np.all(np.abs(got["rosenbluth"] - R) <= 1e-10 * np.maximum(R, 1e-300))
    assert ok.mean() > 0.5


def test_widom_mixed_within_tolerance(grx_lib):
    s = co2_system(n_co2=0)
    nfw = s["comp_start"][1]
    box = grx_lib.Box(s, capacity=[nfw, 3 * 32])
    box.ewald_total()
    n = 400
    ref, _ = oracle_widom(s, 1, n)
    R, sf, so, ok, E = _fields(ref)
    d = grx_lib.widom_desc(s, 1, 10, 10, seed=42)
    got = box.widom(d, 0, n, prec=grx_lib.GRX_MIXED)
    same = (got["sel_first"] == sf) & (got["sel_orient"] == so) & (got["success"] == ok)
    assert same.mean() >= 0.99
    r = same & (R > 0)
    rel = np.abs(got["rosenbluth"][r] - R[r]) / R[r]
    assert np.max(rel) <= 2e-6, np.max(rel)


def test_widom_deterministic_and_streams(grx_lib):
    s = co2_system(n_co2=0)
    nfw = s["comp_start"][1]
    box = grx_lib.Box(s, capacity=[nfw, 3 * 8])
    box.ewald_total()
    d = grx_lib.widom_desc(s, 1, 10, 10, seed=7)
    a = box.widom(d, 100, 200, prec=grx_lib.GRX_MIXED)
    b = box.widom(d, 100, 200, prec=grx_lib.GRX_MIXED)
    assert a.tobytes() == b.tobytes()
    c = box.widom(d, 150, 50, prec=grx_lib.GRX_MIXED)   # counter-based: any sub-range reproduces
    assert c.tobytes() == a[50:100].tobytes()


def test_widom_edge_cases(grx_lib):
    s = co2_system(n_co2=0)
    nfw = s["comp_start"][1]
    # every trial overlaps: construction fails, Rosenbluth 0
    s2 = dict(s)
    s2["overlap_criteria"] = -1e30
    box = grx_lib.Box(s2, capacity=[nfw, 3 * 8])
    box.ewald_total()
    got = box.widom(grx_lib.widom_desc(s2, 1, 10, 10), 0, 20, prec=grx_lib.GRX_MIXED)
    assert np.all(got["success"] == 0) and np.all(got["rosenbluth"] == 0) and np.all(got["n_ok_first"] == 0)
    # one trial, one orientation; and an uncharged system (Ewald skipped)
    s3 = dict(s)
    s3["no_charges"] = 1
    box3 = grx_lib.Box(s3, capacity=[nfw, 3 * 8])
    box3.ewald_total()
    ref, _ = oracle_widom(s3, 1, 64, ntrials=1, norient=1)
    R, sf, so, ok, E = _fields(ref)
    got = box3.widom(grx_lib.widom_desc(s3, 1, 1, 1), 0, 64, prec=grx_lib.GRX_FP64)
    assert np.array_equal(got["success"], ok)
    assert np.all(got["ewald"] == 0)
    assert np.all(np.abs(got["rosenbluth"] - R) <= 1e-10 * np.maximum(R, 1e-300))
    # zero insertions is a no-op
    assert len(box3.widom(grx_lib.widom_desc(s3, 1, 1, 1), 0, 0)) == 0


# ---------------------------------------------------------------- 12-6-4 and VDWRealBias off
def lj1264_system(n_co2=6, seed=17):
    """The CO2/silica system in the 12-6-4 form of VDW (maths.cuh:454-475): per type pair
    C12 = 4 eps sigma^12 and C6 = 4 eps sigma^6 of the LJ pair plus a seeded C4 and C10."""
    s = dict(co2_system(n_co2=n_co2))
    eps, sig = np.asarray(s["epsilon"]), np.asarray(s["sigma"])
    rng = np.random.default_rng(seed)
    nt = int(s["ntypes"])
    c4 = rng.uniform(-2000.0, 0.0, nt * nt)   # +C4 / r^4: negative C4 attracts (ion-induced dipole)
    c10 = rng.uniform(0.0, 2e5, nt * nt) * (rng.uniform(0, 1, nt * nt) < 0.5)
    c4 = 0.5 * (c4.reshape(nt, nt) + c4.reshape(nt, nt).T).reshape(-1)
    c10 = 0.5 * (c10.reshape(nt, nt) + c10.reshape(nt, nt).T).reshape(-1)
    s.update(use_1264=1, epsilon=4.0 * eps * sig ** 12, sigma=4.0 * eps * sig ** 6, z=c4, c10=c10,
             shift=np.zeros(nt * nt))
    return s


@pytest.mark.parametrize("chain", [1, 2])
def test_trial_energies_1264(grx_lib, chain):
    s = lj1264_system()
    n_co2 = 6
    box = grx_lib.Box(s, capacity=[len(s["pos"]) - 3 * n_co2, 3 * 64])
    S = O.OracleSystem(s)
    rng = np.random.default_rng(32)   # a stream whose chain trials are not all in the framework walls
    ntr = 48
    pos, q, ty = _random_beads(s, 1, ntr, chain, rng)
    ref, rflag = S.trial_energies(pos, np.ones(len(q)), q, np.ones(len(q)), ty, n_co2, ntr, chain, 1)
    e64, f64 = box.trial_energies(pos, q, ty, n_co2, ntr, chain, 1, prec=grx_lib.GRX_FP64)
    assert np.array_equal(f64, rflag)
    assert fp64_close(e64, ref), np.max(np.abs(e64 - ref))
    em, fm = box.trial_energies(pos, q, ty, n_co2, ntr, chain, 1, prec=grx_lib.GRX_MIXED)
    ok = rflag == 0
    assert ok.sum() > 0 and np.array_equal(fm, rflag)
    assert mixed_close(em[ok], ref[ok]), np.max(np.abs(em[ok] - ref[ok]))
    # the 12-6-4 terms change the energies (the test is not a plain LJ one)
    lj, _ = grx_lib.Box(co2_system(n_co2=n_co2), capacity=[len(s["pos"]) - 3 * n_co2, 3 * 64]).trial_energies(
        pos, q, ty, n_co2, ntr, chain, 1, prec=grx_lib.GRX_FP64)
    assert np.max(np.abs(lj[ok, 0] - e64[ok, 0])) > 1.0 and np.max(np.abs(lj[ok, 2] - e64[ok, 2])) > 1e-3


def test_widom_vdw_real_bias_off(grx_lib):
    """VDWRealBias = false: trials are selected on the VDW energy alone and the chosen
    trial's real-space Coulomb weight multiplies the step weight (mc_widom.h:368-369)."""
    s = dict(co2_system(n_co2=0))
    s["vdw_real_bias"] = 0
    nfw = s["comp_start"][1]
    box = grx_lib.Box(s, capacity=[nfw, 3 * 32])
    box.ewald_total()
    n = 300
    ref, _ = oracle_widom(s, 1, n)
    R, sf, so, ok, E = _fields(ref)
    d = grx_lib.widom_desc(s, 1, 10, 10, seed=42)
    got = box.widom(d, 0, n, prec=grx_lib.GRX_FP64)
    assert np.array_equal(got["success"], ok) and np.array_equal(got["sel_first"], sf)
    assert np.array_equal(got["sel_orient"], so)
    assert np.all(np.abs(got["rosenbluth"] - R) <= 1e-10 * np.maximum(R, 1e-300))
    # the selection differs from the biased one on this stream
    s_b = co2_system(n_co2=0)
    ref_b, _ = oracle_widom(s_b, 1, n)
    assert not np.array_equal(_fields(ref_b)[1], sf)
    mixed = box.widom(d, 0, n, prec=grx_lib.GRX_MIXED)
    same = (mixed["sel_first"] == sf) & (mixed["sel_orient"] == so) & (mixed["success"] == ok)
    assert same.mean() >= 0.99
    r = same & (R > 0)
    assert np.max(np.abs(mixed["rosenbluth"][r] - R[r]) / R[r]) <= 2e-6
