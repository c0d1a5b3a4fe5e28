"""GPU parity of the device GCMC run (grx_gcmc_run) against the FP64 oracle.

The oracle (ora_gcmc_run) restates RunMoves (axpy.cu:102-298) for translation,
rotation and CBMC insertion / deletion of one component; both sides draw the same
Philox counters, so in FP64 the two Markov chains must take identical decisions.
The move mix is translation : rotation : reinsertion : swap = 1 : 1 : 1 : 2.

Tolerances:
  FP64 : identical move counts and molecule numbers; positions within 1e-9 A
         (they are produced by the same FP64 expressions); accepted-energy sums
         within 1e-9 relative.
  MIXED: identical decisions on this seeded chain (the acceptance probabilities
         agree to 1e-6 relative, see the pair-energy tests); accepted-energy sums
         within beta*|dE| <= 1e-5 over the run.
  Drift: the device's recomputed FP64 total after a run equals the initial total
         plus the accepted move energies (gRASPA's ENERGY DRIFT check,
         fxn_main.h:454-542) to 1e-8 relative.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.systems import co2_system

pytestmark = pytest.mark.gpu

CAP = 3 * 64


def params(grx, **kw):
    mix = dict(p_translation=0.2, p_rotation=0.4, p_reinsertion=0.6, p_swap=1.0)
    mix.update(kw)
    return grx.gcmc_desc(1, **mix)


def ora_params(d):
    g = O.OraGcmc()
    g.component, g.ntrials, g.norient = d.component, d.ntrials, d.norient
    g.p_translation, g.p_rotation, g.p_swap = d.p_translation, d.p_rotation, d.p_swap
    g.p_reinsertion = d.p_reinsertion
    for k in range(3):
        g.max_translation[k] = d.max_translation[k]
        g.max_rotation[k] = d.max_rotation[k]
    g.beta, g.pressure = d.beta, d.pressure
    g.fugacity_coeff, g.mol_fraction, g.ideal_rosenbluth = d.fugacity_coeff, d.mol_fraction, d.ideal_rosenbluth
    g.seed, g.stream = d.seed, d.stream
    g.tail_insert = d.tail_insert
    return g


def total(box):
    t = box.total_energy()
    return sum(t[k] for k in ("hh_vdw", "hh_real", "hg_vdw", "hg_real", "gg_vdw", "gg_real", "hh_ewald",
                              "hg_ewald", "gg_ewald"))


def make_box(grx, s):
    box = grx.Box(s, capacity=[s["comp_start"][1], CAP])
    box.ewald_total()
    return box


def run_pair(grx, s, d, nsteps, prec, first=0):
    box = make_box(grx, s)
    st = grx.gcmc_run([box], [d], first, nsteps, prec)[0]
    ost, after, _ = O.OracleSystem(s).gcmc(ora_params(d), [s["comp_start"][1], CAP], first, nsteps)
    return box, st, ost, after


@pytest.mark.parametrize("n_co2", [0, 5])
def test_gcmc_fp64_matches_oracle(grx_lib, n_co2):
    s = co2_system(n_co2=n_co2)
    d = params(grx_lib, pressure_pa=1e6)
    box, st, ost, after = run_pair(grx_lib, s, d, 400, grx_lib.GRX_FP64)
    assert list(st.attempts) == list(ost.attempts)
    assert list(st.accepted) == list(ost.accepted)
    assert st.n_molecules == ost.n_molecules and st.capacity_hits == 0
    assert st.sum_n == ost.sum_n
    assert sum(st.accepted) > 40
    nfw = s["comp_start"][1]
    got = box.positions(1)
    ref = after["pos"][nfw:]
    assert got.shape == ref.shape
    assert np.max(np.abs(got - ref)) <= 1e-9
    for k in range(4):
        assert abs(st.energy[k] - ost.energy[k]) <= 1e-9 * max(1.0, abs(ost.energy[k]))


@pytest.mark.parametrize("prec", ["GRX_FP64", "GRX_MIXED"])
def test_gcmc_tail_correction_matches_oracle(grx_lib, prec):
    """A tail correction on insertion and deletion (the deletion takes the negative
    difference, mc_swap_utilities.h:197-200): the same decisions as the oracle."""
    s = co2_system(n_co2=5)
    d = params(grx_lib, pressure_pa=1e6, tail_insert=-200.0)
    box, st, ost, after = run_pair(grx_lib, s, d, 400, getattr(grx_lib, prec))
    assert list(st.attempts) == list(ost.attempts) and list(st.accepted) == list(ost.accepted)
    assert st.n_molecules == ost.n_molecules
    nfw = s["comp_start"][1]
    assert np.max(np.abs(box.positions(1) - after["pos"][nfw:])) <= 1e-9
    free = run_pair(grx_lib, s, params(grx_lib, pressure_pa=1e6), 400, grx_lib.GRX_FP64)[1]
    assert st.n_molecules > free.n_molecules


def test_gcmc_mixed_matches_oracle(grx_lib):
    s = co2_system(n_co2=5)
    d = params(grx_lib, pressure_pa=1e6)
    box, st, ost, after = run_pair(grx_lib, s, d, 400, grx_lib.GRX_MIXED)
    assert list(st.accepted) == list(ost.accepted) and st.n_molecules == ost.n_molecules
    nfw = s["comp_start"][1]
    assert np.max(np.abs(box.positions(1) - after["pos"][nfw:])) <= 1e-9
    for k in range(4):
        assert d.beta * abs(st.energy[k] - ost.energy[k]) <= 1e-5


@pytest.mark.parametrize("prec", ["GRX_FP64", "GRX_MIXED"])
def test_gcmc_energy_drift(grx_lib, prec):
    s = co2_system(n_co2=5)
    box = make_box(grx_lib, s)
    e0 = total(box)
    box.ewald_total()
    st = grx_lib.gcmc_run([box], [params(grx_lib, pressure_pa=1e6)], 0, 500, getattr(grx_lib, prec))[0]
    e1 = total(box)
    assert sum(st.accepted) > 50
    assert abs((e1 - e0) - st.energy[3]) <= 1e-8 * max(abs(e1), abs(e0))


def test_gcmc_multibox_independent_and_resumable(grx_lib):
    s = co2_system(n_co2=3)
    descs = [params(grx_lib, stream=k, pressure_pa=1e6) for k in range(4)]
    boxes = [make_box(grx_lib, s) for _ in range(4)]
    multi = grx_lib.gcmc_run(boxes, descs, 0, 200, grx_lib.GRX_FP64)
    for k in (0, 3):  # each box of the batched launch equals its own single-box run
        b = make_box(grx_lib, s)
        one = grx_lib.gcmc_run([b], [descs[k]], 0, 200, grx_lib.GRX_FP64)[0]
        assert list(one.accepted) == list(multi[k].accepted) and one.n_molecules == multi[k].n_molecules
        assert np.array_equal(b.positions(1), boxes[k].positions(1))
    assert len({tuple(m.accepted) for m in multi}) > 1  # different streams, different chains
    # steps 0..99 then 100..199 equal one run of 200 steps
    b = make_box(grx_lib, s)
    grx_lib.gcmc_run([b], [descs[1]], 0, 100, grx_lib.GRX_FP64)
    grx_lib.gcmc_run([b], [descs[1]], 100, 100, grx_lib.GRX_FP64)
    assert np.array_equal(b.positions(1), boxes[1].positions(1))


def test_gcmc_capacity_and_edges(grx_lib):
    s = co2_system(n_co2=0)
    box = grx_lib.Box(s, capacity=[s["comp_start"][1], 3 * 2])  # room for two molecules
    box.ewald_total()
    d = params(grx_lib, p_translation=0.0, p_rotation=0.0, p_reinsertion=0.0, pressure_pa=1e9)
    st = grx_lib.gcmc_run([box], [d], 0, 300, grx_lib.GRX_FP64)[0]
    assert st.n_molecules <= 2 and st.capacity_hits > 0
    assert box.component_size(1) == 3 * st.n_molecules
    # zero steps: nothing moves, counts are zero
    st0 = grx_lib.gcmc_run([box], [d], 300, 0, grx_lib.GRX_FP64)[0]
    assert sum(st0.attempts) == 0 and st0.n_molecules == st.n_molecules
    # argument errors
    bad = params(grx_lib)
    bad.component = 0
    with pytest.raises(grx_lib.GrxError):
        grx_lib.gcmc_run([box], [bad], 0, 1, grx_lib.GRX_FP64)
    bad = params(grx_lib, ntrials=65)
    with pytest.raises(grx_lib.GrxError):
        grx_lib.gcmc_run([box], [bad], 0, 1, grx_lib.GRX_FP64)
    with pytest.raises(grx_lib.GrxError):
        grx_lib.gcmc_run([box, box], [d, d], 0, 1, grx_lib.GRX_FP64)


@pytest.mark.parametrize("shape", [(8, 1), (8, 8), (12, 2), (24, 1), (24, 4)])
def test_gcmc_launch_shapes_match_oracle(grx_lib, shape):
    """Every launch shape (warps per box x items per warp of a bead pass) only changes
    how a pass is split over warps: the FP64 chain still takes the oracle's decisions."""
    s = co2_system(n_co2=5)
    d = params(grx_lib, pressure_pa=1e6)
    box = make_box(grx_lib, s)
    batch = grx_lib.GcmcBatch([box], [d], grx_lib.GRX_FP64)
    batch.set_shape(*shape)
    assert batch.shape() == shape
    batch.launch(300)
    st, nxt = batch.stats()
    batch.close()
    ost, after, _ = O.OracleSystem(s).gcmc(ora_params(d), [s["comp_start"][1], CAP], 0, 300)
    assert nxt == 300
    assert list(st[0].accepted) == list(ost.accepted) and st[0].n_molecules == ost.n_molecules
    nfw = s["comp_start"][1]
    assert np.max(np.abs(box.positions(1) - after["pos"][nfw:])) <= 1e-9
    for k in range(4):
        assert abs(st[0].energy[k] - ost.energy[k]) <= 1e-9 * max(1.0, abs(ost.energy[k]))
    with pytest.raises(grx_lib.GrxError):
        grx_lib.GcmcBatch([box], [d], grx_lib.GRX_FP64).set_shape(16, 1)


@pytest.mark.parametrize("cl,prec", [(2, "GRX_FP64"), (4, "GRX_FP64"), (8, "GRX_FP64"), (8, "GRX_MIXED")])
def test_gcmc_cluster_matches_oracle(grx_lib, cl, prec):
    """One chain per thread-block cluster of cl CTAs (24 warps each): the bead passes are
    split across the cluster and the partial sums exchanged through distributed shared
    memory, every CTA reduces them in the same order and takes the same decisions. Two
    boxes (two clusters) with different streams, each against its own oracle chain: FP64
    decisions, positions and energies as the oracle; mixed the same decisions and positions,
    energies within beta*|dE| <= 1e-5. Charged CO2, so the Ewald delta and the S(k) commit
    (computed by every CTA) are exercised with the commit barrier."""
    s = co2_system(n_co2=5)
    descs = [params(grx_lib, pressure_pa=1e6, stream=k) for k in range(2)]
    boxes = [make_box(grx_lib, s) for _ in range(2)]
    batch = grx_lib.GcmcBatch(boxes, descs, getattr(grx_lib, prec))
    batch.set_shape(24, 2)
    batch.set_cluster(cl)
    assert batch.cluster() == cl
    batch.run_graph(150, 2)
    st, nxt = batch.stats()
    batch.close()
    assert nxt == 300
    nfw = s["comp_start"][1]
    for k in range(2):
        ost, after, _ = O.OracleSystem(s).gcmc(ora_params(descs[k]), [nfw, CAP], 0, 300)
        assert list(st[k].attempts) == list(ost.attempts) and list(st[k].accepted) == list(ost.accepted)
        assert st[k].n_molecules == ost.n_molecules
        assert np.max(np.abs(boxes[k].positions(1) - after["pos"][nfw:])) <= 1e-9
        for e in range(4):
            if prec == "GRX_FP64":
                assert abs(st[k].energy[e] - ost.energy[e]) <= 1e-9 * max(1.0, abs(ost.energy[e]))
            else:
                assert descs[k].beta * abs(st[k].energy[e] - ost.energy[e]) <= 1e-5
    assert sum(st[0].accepted) > 30


def test_gcmc_cluster_shape_rules(grx_lib):
    """Clusters need 24 warps per block; a shape with fewer warps returns to one block."""
    s = co2_system(n_co2=2)
    box = make_box(grx_lib, s)
    batch = grx_lib.GcmcBatch([box], [params(grx_lib)], grx_lib.GRX_FP64)
    batch.set_shape(12, 1)
    with pytest.raises(grx_lib.GrxError):
        batch.set_cluster(2)
    with pytest.raises(grx_lib.GrxError):
        batch.set_cluster(3)
    batch.set_shape(24, 1)
    batch.set_cluster(4)
    batch.set_shape(8, 1)
    assert batch.cluster() == 1
    batch.close()


@pytest.mark.parametrize("cl", [1, 8])
def test_gcmc_mixed_ewald_row_products_match_oracle(grx_lib, cl):
    """A charged box with many k vectors per (kx, ky) row (automatic Ewald set-up of a
    2,500-atom framework: kmax 10/16/15, 8,466 active k, 23 per row) takes the row-product
    form of the double-float Ewald delta; the mixed chain still takes the oracle's exact
    decisions and positions, with energies within beta*|dE| <= 1e-5 over the run. With a
    cluster of 8 CTAs the k vectors are split across the cluster as well (each CTA stages
    and commits its own range of S(k))."""
    from graspa_gb300 import synth
    s = synth.adsorbate_system("CO2", 12, n_atoms=2500)
    S = O.OracleSystem(s)
    _, act = S.ewald_active()
    nrow = (s["kmax"][0] + 1) * (2 * s["kmax"][1] + 1)
    assert int(np.sum(act)) >= 16 * nrow  # the box qualifies for the row products
    d = params(grx_lib, pressure_pa=1e6)
    nfw = s["comp_start"][1]
    box = make_box(grx_lib, s)
    if cl == 1:
        st = grx_lib.gcmc_run([box], [d], 0, 250, grx_lib.GRX_MIXED)[0]
    else:
        batch = grx_lib.GcmcBatch([box], [d], grx_lib.GRX_MIXED)
        batch.set_shape(24, 1)
        batch.set_cluster(cl)
        batch.launch(250)
        st = batch.stats()[0][0]
        batch.close()
    ost, after, _ = S.gcmc(ora_params(d), [nfw, CAP], 0, 250)
    assert sum(st.accepted) > 20
    assert list(st.accepted) == list(ost.accepted) and st.n_molecules == ost.n_molecules
    assert np.max(np.abs(box.positions(1) - after["pos"][nfw:])) <= 1e-9
    for k in range(4):
        assert d.beta * abs(st.energy[k] - ost.energy[k]) <= 1e-5
    # the committed adsorbate S(k) (every CTA's range of k) equals S(k) recomputed from
    # the final positions
    _, s_run, _ = box.structure_factors()
    box.ewald_total()
    _, s_new, _ = box.structure_factors()
    assert np.max(np.abs(s_run - s_new)) <= 1e-9 * max(1.0, np.max(np.abs(s_new)))
    box.close()


@pytest.mark.parametrize("cl", [2, 8])
def test_identity_swaps_on_clusters(grx_lib, cl):
    """Identity swaps only (CO2 + N2 mixture, both components moved) on a thread-block cluster
    take the one-block chain's decisions in FP64: the same swap counts and molecule numbers,
    positions within 1e-9 A, energy sums within 1e-9 relative."""
    from graspa_gb300 import synth
    s = synth.silica_co2_n2(n_co2=4, n_n2=4)
    cap = [s["comp_start"][1], CAP, CAP]
    kw = dict(p_translation=0.0, p_rotation=0.0, p_reinsertion=0.0, p_identity_swap=1.0, p_swap=1.0,
              pressure_pa=1e6)
    descs = [grx_lib.gcmc_desc(1, **kw), grx_lib.gcmc_desc(2, **kw)]
    runs = []
    for c in (1, cl):
        box = grx_lib.Box(s, capacity=cap)
        box.ewald_total()
        batch = grx_lib.GcmcBatch([box], [descs], grx_lib.GRX_FP64)
        batch.set_shape(24, 1)
        if c > 1:
            batch.set_cluster(c)
        batch.launch(80)
        st, _ = batch.stats()
        batch.close()
        runs.append((st, [box.positions(1), box.positions(2)]))
        box.close()
    (a, pa), (b, pb) = runs
    for k in range(2):
        assert list(a[k].identity_in) == list(b[k].identity_in)
        assert list(a[k].identity_out) == list(b[k].identity_out)
        assert a[k].n_molecules == b[k].n_molecules
        assert abs(a[k].energy[3] - b[k].energy[3]) <= 1e-9 * max(1.0, abs(a[k].energy[3]))
    assert a[0].identity_in[1] + a[1].identity_in[1] >= 2
    for x, y in zip(pa, pb):
        assert x.shape == y.shape and np.max(np.abs(x - y), initial=0.0) <= 1e-9


def test_gcmc_vdw_real_bias_off_matches_oracle(grx_lib):
    """VDWRealBias = false in the device GCMC kernel: the oracle's decisions in FP64."""
    s = dict(co2_system(n_co2=5))
    s["vdw_real_bias"] = 0
    d = params(grx_lib, pressure_pa=1e6)
    box, st, ost, after = run_pair(grx_lib, s, d, 400, grx_lib.GRX_FP64)
    assert list(st.attempts) == list(ost.attempts)
    assert list(st.accepted) == list(ost.accepted)
    assert st.n_molecules == ost.n_molecules
    assert abs(st.energy[3] - ost.energy[3]) <= 1e-9 * max(1.0, abs(ost.energy[3]))


def test_gcmc_counts_and_rosenbluth_match_oracle(grx_lib):
    """The kernel's own work and Widom counters: trial configurations evaluated, their
    beads, and the Rosenbluth sums of the insertion attempts (RecordRosen) equal the
    oracle's over the same chain, in FP64; the mixed chain's weights agree to 1e-6."""
    s = co2_system(n_co2=5)
    d = params(grx_lib, pressure_pa=1e6)
    box, st, ost, after = run_pair(grx_lib, s, d, 400, grx_lib.GRX_FP64)
    assert st.trial_configs == ost.trial_configs and st.trial_beads == ost.trial_beads
    assert st.rosen[2] == ost.rosen[2] == st.attempts[2]
    assert abs(st.rosen[0] - ost.rosen[0]) <= 1e-10 * max(1e-300, ost.rosen[0])
    assert abs(st.rosen[1] - ost.rosen[1]) <= 1e-10 * max(1e-300, ost.rosen[1])
    # orientations are grown only after a successful first bead: fewer than 20 per growth
    assert st.trial_configs < 2 * (st.attempts[0] + st.attempts[1]) + 20 * (st.attempts[2] + st.attempts[3]) + \
        41 * st.attempts[4]
    box_m = make_box(grx_lib, s)
    sm = grx_lib.gcmc_run([box_m], [d], 0, 400, grx_lib.GRX_MIXED)[0]
    if list(sm.accepted) == list(st.accepted):
        assert abs(sm.rosen[0] - st.rosen[0]) <= 1e-6 * st.rosen[0]
