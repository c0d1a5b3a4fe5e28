"""GCMC oracle self-consistency: the drift check of gRASPA (fxn_main.h:454-542,
'ENERGY DRIFT' asserted < 1e-3 by Examples/test_examples.py:61) applied to the
oracle's move deltas. Recomputing the FP64 totals after a run must reproduce the
initial totals plus the sum of the accepted move energies."""
import numpy as np

from graspa_gb300 import grx, synth
from oracle import oracle as O


def gcmc_params(seed=42, stream=0, T=300.0, pressure_pa=1e5):
    g = O.OraGcmc()
    g.component, g.ntrials, g.norient = 1, 10, 10
    g.p_translation, g.p_rotation, g.p_reinsertion, g.p_swap = 0.2, 0.4, 0.6, 1.0
    for d in range(3):
        g.max_translation[d] = 1.0
        g.max_rotation[d] = 0.5
    g.beta = grx.beta_from_temperature(T)
    g.pressure = pressure_pa / 1.6605402e7  # Pa -> internal units (fxn_main.h:120)
    g.fugacity_coeff, g.mol_fraction, g.ideal_rosenbluth = 1.0, 1.0, 1.0
    g.seed, g.stream = seed, stream
    return g


def guest_energy(system):
    """Total of every term that involves guests: HG + GG VDW/real and the guest part
    of the Ewald sum (Ewald_Total, ewald_preparation.h:5-259)."""
    S = O.OracleSystem(system)
    e6 = S.vdw_real_total()
    ew, _, _ = S.ewald_total(list(system["molsize"]))
    ewald = ew[0] + ew[2] - (ew[3] - ew[4]) + (ew[5] - ew[6])
    return e6[2] + e6[3] + e6[4] + e6[5] + ewald


def test_gcmc_energy_drift():
    s = synth.silica_co2(n_co2=5)
    e0 = guest_energy(s)
    S = O.OracleSystem(s)
    st, after, _ = S.gcmc(gcmc_params(), [s["comp_start"][1], 3 * 64], 0, 300)
    e1 = guest_energy(after)
    assert sum(st.accepted) > 40
    assert abs((e1 - e0) - st.energy[3]) < 1e-6 * max(1.0, abs(e1))


def test_gcmc_deterministic_and_resumable():
    s = synth.silica_co2(n_co2=3)
    cap = [s["comp_start"][1], 3 * 64]
    a, sa, _ = O.OracleSystem(s).gcmc(gcmc_params(), cap, 0, 120)
    b, sb, _ = O.OracleSystem(s).gcmc(gcmc_params(), cap, 0, 120)
    assert np.array_equal(sa["pos"], sb["pos"]) and a.n_molecules == b.n_molecules
    # counter-based stream: steps 0..59 then 60..119 from the saved state equal one run
    c1, mid, _ = O.OracleSystem(s).gcmc(gcmc_params(), cap, 0, 60)
    c2, end, _ = O.OracleSystem(mid).gcmc(gcmc_params(), cap, 60, 60)
    assert np.allclose(end["pos"], sa["pos"], rtol=0, atol=1e-9)
    assert c2.n_molecules == a.n_molecules


def test_gcmc_tail_correction_sign():
    """Insertion_Body multiplies the Rosenbluth weight by exp(-beta t) for the insertion
    tail difference t, and Deletion_Body divides it by exp(-beta TailE) with TailE the
    deletion difference -t (mc_swap_utilities.h:105-108, 197-200). Both acceptances
    then carry the factor of a pressure scaled by exp(-beta t): a chain with the tail
    equals the tail-free chain at that pressure, move for move."""
    s = synth.silica_co2(n_co2=3)
    cap = [s["comp_start"][1], 3 * 64]
    g = gcmc_params(pressure_pa=1e6)
    t = -200.0  # internal units; beta t ~ -0.8 at 300 K
    g.tail_insert = t
    a, sa, _ = O.OracleSystem(s).gcmc(g, cap, 0, 300)
    p = gcmc_params(pressure_pa=1e6 * np.exp(-g.beta * t))
    b, sb, _ = O.OracleSystem(s).gcmc(p, cap, 0, 300)
    c, _, _ = O.OracleSystem(s).gcmc(gcmc_params(pressure_pa=1e6), cap, 0, 300)
    assert list(a.accepted) == list(b.accepted) and a.n_molecules == b.n_molecules
    assert np.allclose(sa["pos"], sb["pos"], rtol=0, atol=1e-9)
    assert a.n_molecules > c.n_molecules  # an attractive tail raises the loading
