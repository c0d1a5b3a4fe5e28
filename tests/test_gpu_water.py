"""Charge-dominated Ewald benchmark: TIP4P-Ew water (4 sites, uncharged first bead,
three charged chain sites) in a charged hexagonal framework, alpha 0.30, kmax
10/10/8, against the FP64 oracle. Tolerances as in test_gpu_parity."""
import numpy as np
import pytest

from graspa_gb300 import synth
from oracle import oracle as O
from tests.test_gpu_gcmc import ora_params
from tests.test_gpu_parity import _fields, beta, fp64_close, mixed_close, oracle_widom

pytestmark = pytest.mark.gpu

CAP = 4 * 400


def water(n):
    return synth.tip4p_hex_system(n_water=n)


def test_water_orientation_trial_energies(grx_lib):
    s = water(30)
    nfw = s["comp_start"][1]
    box = grx_lib.Box(s, capacity=[nfw, CAP])
    S = O.OracleSystem(s)
    rng = np.random.default_rng(2)
    tm = s["templates"][1]
    cell = np.array(s["cell"]).reshape(3, 3).T
    no = 12
    first = cell @ np.array([0.02, 0.03, 0.4])     # inside the channel
    pos, q, ty = [], [], []
    for o in range(no):
        a, b_, c = rng.uniform(0, 2 * np.pi, 3)
        R = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]]) @ \
            np.array([[1, 0, 0], [0, np.cos(b_), -np.sin(b_)], [0, np.sin(b_), np.cos(b_)]])
        for k in range(1, 4):
            pos.append(first + R @ (tm["pos"][k] - tm["pos"][0]))
            q.append(tm["charge"][k])
            ty.append(tm["type"][k])
    pos, q, ty = np.array(pos), np.array(q), np.array(ty)
    n_mol = (len(s["pos"]) - nfw) // 4
    ref, rf = S.trial_energies(pos, np.ones(len(q)), q, np.ones(len(q)), ty, n_mol, no, 3, 1)
    e, f = box.trial_energies(pos, q, ty, n_mol, no, 3, 1, prec=grx_lib.GRX_FP64)
    assert np.array_equal(f, rf) and fp64_close(e, ref), np.max(np.abs(e - ref))
    em, fm = box.trial_energies(pos, q, ty, n_mol, no, 3, 1, prec=grx_lib.GRX_MIXED)
    ok = rf == 0
    assert ok.sum() > 0 and np.array_equal(fm, rf) and mixed_close(em[ok], ref[ok])   # per component


def test_water_widom_fp64_matches_oracle(grx_lib):
    s = water(20)
    box = grx_lib.Box(s, capacity=[s["comp_start"][1], CAP])
    box.ewald_total()
    n = 200
    ref, _ = oracle_widom(s, 1, n)
    R, sf, so, ok, E = _fields(ref)
    got = box.widom(grx_lib.widom_desc(s, 1, 10, 10, seed=42), 0, n, prec=grx_lib.GRX_FP64)
    assert np.array_equal(got["success"], ok) and np.array_equal(got["sel_first"], sf)
    assert np.array_equal(got["sel_orient"], so)
    Eg = np.concatenate([got["e_first"], got["e_chain"], got["ewald"]], axis=1)
    assert np.all(np.abs(Eg - E) <= 1e-10 * np.maximum(np.abs(E), 1.0))
    mixed = box.widom(grx_lib.widom_desc(s, 1, 10, 10, seed=42), 0, n, prec=grx_lib.GRX_MIXED)
    both = (mixed["success"] != 0) & (ok != 0)
    Em = np.concatenate([mixed["e_first"], mixed["e_chain"], mixed["ewald"]], axis=1)
    same_sel = both & (mixed["sel_first"] == sf) & (mixed["sel_orient"] == so)
    assert np.mean(mixed["success"] == ok) > 0.98        # failed constructions agree too
    assert same_sel.sum() > 0.95 * both.sum() and both.sum() > 0.3 * n
    assert np.all(beta() * np.abs(Em[same_sel] - E[same_sel]) <= 1e-6)   # per component


@pytest.mark.parametrize("prec", ["GRX_FP64", "GRX_MIXED"])
def test_water_gcmc(grx_lib, prec):
    s = water(25)
    nfw = s["comp_start"][1]
    d = grx_lib.gcmc_desc(1, p_translation=0.25, p_rotation=0.5, p_reinsertion=0.75, p_swap=1.0,
                          pressure_pa=3.5e3, max_translation=0.5, max_rotation=0.4)
    box = grx_lib.Box(s, capacity=[nfw, CAP])
    box.ewald_total()
    e0 = sum(box.total_energy().values())
    box.ewald_total()
    st = grx_lib.gcmc_run([box], [d], 0, 300, getattr(grx_lib, prec))[0]
    e1 = sum(box.total_energy().values())
    assert sum(st.accepted) > 30
    if prec == "GRX_FP64":
        ost, after, _ = O.OracleSystem(s).gcmc(ora_params(d), [nfw, CAP], 0, 300)
        assert list(st.attempts) == list(ost.attempts) and list(st.accepted) == list(ost.accepted)
        assert np.max(np.abs(box.positions(1) - after["pos"][nfw:])) <= 1e-9
        assert abs((e1 - e0) - st.energy[3]) <= 1e-8 * max(abs(e1), 1.0)
    else:
        assert beta() * abs((e1 - e0) - st.energy[3]) <= 1e-6 * (sum(st.accepted) + 1)
