"""The oracle's CB/CFC lambda-change and identity-swap Fourier deltas
(GPU_EwaldDifference_LambdaChange, Ewald_Energy_Functions.h:764-789;
GPU_EwaldDifference_IdentitySwap, :582-634) against identities of the general delta.

  - a lambda change 0 -> 1 at the inserted positions equals the insertion delta with
    its exclusion (Fourier_Ewald_Diff with no old atoms, :280-397);
  - two lambda steps 0.2 -> 0.6 -> 1.0 through the staged vector add up to 0.2 -> 1.0
    (the same-type energy is a function of S alone);
  - an identity swap to an identical molecule changes nothing but the exclusions.
Tolerance 1e-10 relative (FP64, different summation orders).
"""
import numpy as np

from oracle import oracle as O
from tests.systems import co2_system


def _setup(n_co2=6):
    s = co2_system(n_co2=n_co2)
    nfw = s["comp_start"][1]
    S = O.OracleSystem(s)
    _, s_fw, s_ads = S.ewald_total([nfw, 3])
    intra, self_ = S.rigid_exclusion(s["templates"][1]["pos"], s["templates"][1]["charge"], np.ones(3))
    return s, nfw, S, s_fw, s_ads, intra + self_


def close(a, b, tol=1e-10):
    return abs(a - b) <= tol * max(abs(a), abs(b), 1.0)


def test_lambda_zero_to_one_is_insertion():
    s, nfw, S, s_fw, s_ads, ex = _setup()
    pos = s["pos"][nfw:nfw + 3] + np.array([0.3, -0.2, 0.1])
    q = s["charge"][nfw:nfw + 3]
    lam, _ = S.ewald_delta_lambda(s_ads, s_fw, pos, q, 0.0, 1.0, ex)
    ins, _ = S.ewald_delta(s_ads, s_fw, np.zeros((0, 3)), np.zeros(0), pos, q)
    assert close(lam[0], ins[0] - ex) and close(lam[1], 2 * ins[1])


def test_lambda_steps_add_up():
    s, nfw, S, s_fw, s_ads, ex = _setup()
    a0 = nfw + 6
    pos, q = s["pos"][a0:a0 + 3], s["charge"][a0:a0 + 3]
    # the molecule currently sits at lambda 1 in S: take it to 0.2 first (staged base)
    d0, s02 = S.ewald_delta_lambda(s_ads, s_fw, pos, q, 1.0, 0.2, ex)
    d1, s06 = S.ewald_delta_lambda(s_ads, s_fw, pos, q, 0.2, 0.6, ex, s_temp=s02)
    d2, s10 = S.ewald_delta_lambda(s_ads, s_fw, pos, q, 0.6, 1.0, ex, s_temp=s06)
    d12, s10b = S.ewald_delta_lambda(s_ads, s_fw, pos, q, 0.2, 1.0, ex, s_temp=s02)
    assert close(d1[0] + d2[0], d12[0]) and close(d1[1] + d2[1], d12[1])
    assert np.max(np.abs(s10 - s10b)) <= 1e-10 and np.max(np.abs(s10 - s_ads)) <= 1e-10  # back to lambda 1
    assert close(d0[0] + d12[0], 0.0, 1e-9) and close(d0[1] + d12[1], 0.0, 1e-9)


def test_identity_swap_to_identical_molecule():
    s, nfw, S, s_fw, s_ads, ex = _setup()
    a0 = nfw + 3
    pos, q = s["pos"][a0:a0 + 3], s["charge"][a0:a0 + 3]
    out, s_new = S.ewald_delta_identity_swap(s_ads, s_fw, pos, q, pos, q, ex, 0.7 * ex)
    assert close(out[0], -ex + 0.7 * ex) and abs(out[1]) <= 1e-10
    assert np.max(np.abs(s_new - s_ads)) <= 1e-10
