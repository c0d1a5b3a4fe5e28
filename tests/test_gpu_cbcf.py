"""GPU parity of the CB/CFC lambda-change and identity-swap energy variants (the pair
engine and the Fourier delta with lambda scalings) against the FP64 oracle.

  - pair part of a lambda change (Calculate_Single_Body_Energy_VDWReal_LambdaChange,
    VDW_Coulomb.cu:843-1009): grx_single_body_energy with the molecule's atoms at fixed
    positions, old and new (scale, scaleCoul). FP64 within 1e-12 of the sizes of the two
    halves; mixed within beta*|dE| <= 1e-6.
  - Fourier part (GPU_EwaldDifference_LambdaChange, Ewald_Energy_Functions.h:764-789):
    grx_ewald_delta_lambda against ora_ewald_delta_lambda, also from the staged vector
    (CB/CFC deletion's second step); staged S within 1e-10.
  - identity swap (GPU_EwaldDifference_IdentitySwap, :582-634) in a two-component box
    whose components have different charges, so both exclusion terms are exercised.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from tests.systems import co2_system

pytestmark = pytest.mark.gpu


def two_component_system():
    """CO2 in silica split into component 1 (molecules 0-3) and component 2 (molecules
    4-5, charges x 0.8): same types and force field, different exclusion constants."""
    s = co2_system(n_co2=6)
    nfw = s["comp_start"][1]
    s = dict(s)
    s["charge"] = np.array(s["charge"], dtype=np.float64)
    s["molid"] = np.array(s["molid"])
    s["charge"][nfw + 12:] *= 0.8
    s["molid"][nfw + 12:] -= 4
    s["comp_start"] = [0, nfw, nfw + 12, nfw + 18]
    s["molsize"] = [nfw, 3, 3]
    t2 = dict(s["templates"][1])
    t2["charge"] = np.asarray(t2["charge"], dtype=np.float64) * 0.8
    s["templates"] = {1: s["templates"][1], 2: t2}
    return s, nfw


def trials(pos, q, ty, mol, sc, scc):
    keep = [np.ascontiguousarray(np.asarray(pos).reshape(-1)), np.full(3, sc), np.ascontiguousarray(q),
            np.full(3, scc), np.ascontiguousarray(ty, dtype=np.int64)]
    return O.OraTrials(1, 3, O._d(keep[0]), O._d(keep[1]), O._d(keep[2]), O._d(keep[3]), O._i(keep[4]), mol), keep


@pytest.mark.parametrize("lam", [(1.0, 0.35), (0.35, 0.8), (0.02, 0.6)])
def test_lambda_change_pair_energy(grx_lib, lam):
    lo, ln = lam
    s = co2_system(n_co2=8)
    nfw = s["comp_start"][1]
    box = grx_lib.Box(s, capacity=[nfw, 3 * 16])
    S = O.OracleSystem(s)
    beta = grx_lib.beta_from_temperature(300.0)
    for mol in (0, 5):
        a0 = nfw + 3 * mol
        base = dict(pos=s["pos"][a0:a0 + 3], charge=s["charge"][a0:a0 + 3], type=s["type"][a0:a0 + 3], molid=mol)
        old = dict(base, scale=np.full(3, lo), scale_coul=np.full(3, lo))
        new = dict(base, scale=np.full(3, ln), scale_coul=np.full(3, ln))
        to, k1 = trials(base["pos"], base["charge"], base["type"], mol, lo, lo)
        tn, k2 = trials(base["pos"], base["charge"], base["type"], mol, ln, ln)
        ref, ref_new, ref_old = np.zeros(6), np.zeros(6), np.zeros(6)
        rf = np.zeros(1, dtype=np.uint8)
        for out, dn, do in ((ref, 1, 1), (ref_new, 1, 0), (ref_old, 0, 1)):
            O.lib().ora_single_body(ctypes.byref(S.box), ctypes.byref(S.ff), ctypes.byref(S.atoms),
                                    ctypes.byref(to), ctypes.byref(tn), 1, dn, do, O._d(out),
                                    rf.ctypes.data_as(O._u8p))
        scale = np.maximum(np.abs(ref_new) + np.abs(ref_old), 1.0)
        got, flag = box.single_body(old, new, 1, prec=grx_lib.GRX_FP64)
        assert flag == int(rf[0])
        assert np.all(np.abs(got - ref) <= 1e-12 * scale), got - ref
        gm, _ = box.single_body(old, new, 1, prec=grx_lib.GRX_MIXED)
        assert beta * np.max(np.abs(gm - ref)) <= 1e-6, beta * np.abs(gm - ref)
    box.close()


def test_lambda_change_fourier(grx_lib):
    s = co2_system(n_co2=8)
    nfw = s["comp_start"][1]
    box = grx_lib.Box(s, capacity=[nfw, 3 * 16])
    box.ewald_total()
    S = O.OracleSystem(s)
    _, s_fw, s_ads = S.ewald_total([nfw, 3])
    intra, self_ = box.exclusion(1)
    ex = intra + self_
    _, act = S.ewald_active()
    m = np.repeat(act.astype(bool), 2)
    a0 = nfw + 3 * 2
    pos, q = s["pos"][a0:a0 + 3], s["charge"][a0:a0 + 3]
    # lambda 1 -> 0.4 from the adsorbate S(k)
    got = box.ewald_delta_lambda(1, pos, q, 1.0, 0.4)
    ref, s_04 = S.ewald_delta_lambda(s_ads, s_fw, pos, q, 1.0, 0.4, ex)
    assert abs(got[0] - ref[0]) <= 1e-10 * max(abs(ref[0]), 1) and abs(got[1] - ref[1]) <= 1e-10 * max(abs(ref[1]), 1)
    _, _, g_tmp = box.structure_factors()
    assert np.max(np.abs(g_tmp[m] - s_04[m])) <= 1e-10
    # second step from the staged vector (CB/CFC deletion), 0.4 -> 0.1
    got = box.ewald_delta_lambda(1, pos, q, 0.4, 0.1, use_staged=True)
    ref, s_01 = S.ewald_delta_lambda(s_ads, s_fw, pos, q, 0.4, 0.1, ex, s_temp=s_04)
    assert abs(got[0] - ref[0]) <= 1e-10 * max(abs(ref[0]), 1) and abs(got[1] - ref[1]) <= 1e-10 * max(abs(ref[1]), 1)
    box.ewald_commit(1)
    _, g_ads, _ = box.structure_factors()
    assert np.max(np.abs(g_ads[m] - s_01[m])) <= 1e-10
    with pytest.raises(grx_lib.GrxError):
        box.ewald_delta_lambda(0, pos, q, 1.0, 0.5)  # framework component
    box.close()


def test_identity_swap_fourier(grx_lib):
    s, nfw = two_component_system()
    box = grx_lib.Box(s, capacity=[nfw, 3 * 8, 3 * 8])
    box.ewald_total()
    S = O.OracleSystem(s)
    _, s_fw, s_ads = S.ewald_total([nfw, 3, 3])
    e1 = sum(box.exclusion(1))
    e2 = sum(box.exclusion(2))
    assert abs(e2 - 0.64 * e1) <= 1e-10 * abs(e1)  # charges x 0.8: both terms scale with q^2
    _, act = S.ewald_active()
    m = np.repeat(act.astype(bool), 2)
    rng = np.random.default_rng(11)
    # component-2 molecule 1 becomes a component-1 molecule, shifted and turned
    a0 = nfw + 12 + 3
    old_pos, old_q = s["pos"][a0:a0 + 3], s["charge"][a0:a0 + 3]
    new_pos = old_pos[::-1] + rng.uniform(-0.4, 0.4, 3)
    new_q = s["charge"][nfw:nfw + 3]
    got = box.ewald_delta_identity_swap(2, 1, old_pos, old_q, new_pos, new_q)
    ref, s_new = S.ewald_delta_identity_swap(s_ads, s_fw, old_pos, old_q, new_pos, new_q, e1, e2)
    assert abs(got[0] - ref[0]) <= 1e-10 * max(abs(ref[0]), 1) and abs(got[1] - ref[1]) <= 1e-10 * max(abs(ref[1]), 1)
    box.ewald_commit(1)
    _, g_ads, _ = box.structure_factors()
    assert np.max(np.abs(g_ads[m] - s_new[m])) <= 1e-10
    with pytest.raises(grx_lib.GrxError):
        box.ewald_delta_identity_swap(0, 1, old_pos, old_q, new_pos, new_q)
    box.close()
