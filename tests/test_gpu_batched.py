"""Batched CBMC of the CH4 / Xe benchmark: triclinic LJ frameworks, mixture GCMC,
the prepared batch (device step counter, CUDA-graph replay) and the autotuner.

Tolerances as in test_gpu_parity: FP64 1e-12 relative (energies) and identical
decisions against the FP64 oracle; mixed beta*|dE| <= 1e-6 per trial.
"""
import numpy as np
import pytest

from graspa_gb300 import synth
from oracle import oracle as O
from tests.systems import co2_system
from tests.test_gpu_gcmc import ora_params
from tests.test_gpu_parity import beta, fp64_close, mixed_close

pytestmark = pytest.mark.gpu

CAP = 256


def mix_descs(grx, stream=0, pressure_pa=2e6, ntrials=16):
    kw = dict(p_translation=0.3, p_rotation=0.3, p_reinsertion=0.5, p_swap=1.0, pressure_pa=pressure_pa,
              ntrials=ntrials, norient=1, stream=stream, max_translation=0.7)
    return [grx.gcmc_desc(1, **kw), grx.gcmc_desc(2, **kw)]


def make_box(grx, s):
    box = grx.Box(s, capacity=[s["comp_start"][1], CAP, CAP])
    box.ewald_total()
    return box


@pytest.mark.parametrize("seed", [0, 2, 6])
def test_triclinic_trial_energies(grx_lib, seed):
    """Tile culling in general (triclinic) cells: per-trial energies of random beads
    against framework + guests equal the oracle in FP64 and within tolerance mixed."""
    s = synth.ch4_xe_system(seed, n_ch4=6, n_xe=4)
    box = make_box(grx_lib, s)
    S = O.OracleSystem(s)
    rng = np.random.default_rng(seed)
    cell = np.array(s["cell"]).reshape(3, 3).T
    ntr = 32
    pos = (cell @ rng.uniform(-0.2, 1.2, (3, ntr))).T   # also outside the stored cell
    q = np.zeros(ntr)
    ty = np.full(ntr, s["templates"][1]["type"][0])
    ref, rf = S.trial_energies(pos, np.ones(ntr), q, np.ones(ntr), ty, 6, ntr, 1, 1)
    e, f = box.trial_energies(pos, q, ty, 6, ntr, 1, 1, prec=grx_lib.GRX_FP64)
    assert np.array_equal(f, rf) and fp64_close(e, ref), np.max(np.abs(e - ref))
    em, fm = box.trial_energies(pos, q, ty, 6, ntr, 1, 1, prec=grx_lib.GRX_MIXED)
    ok = rf == 0
    assert np.array_equal(fm, rf) and mixed_close(em[ok], ref[ok])   # per component


def test_mixture_gcmc_matches_oracle(grx_lib):
    s = synth.ch4_xe_system(3, n_ch4=5, n_xe=5)
    descs = mix_descs(grx_lib)
    box = make_box(grx_lib, s)
    st = grx_lib.gcmc_run([box], [descs], 0, 400, grx_lib.GRX_FP64)
    ost, after, _ = O.OracleSystem(s).gcmc([ora_params(d) for d in descs], [s["comp_start"][1], CAP, CAP], 0, 400)
    for k in range(2):
        assert list(st[k].attempts) == list(ost[k].attempts)
        assert list(st[k].accepted) == list(ost[k].accepted)
        assert st[k].n_molecules == ost[k].n_molecules and st[k].sum_n == ost[k].sum_n
    assert sum(st[0].accepted) > 20 and sum(st[1].accepted) > 20
    for c in (1, 2):
        a, b = after["comp_start"][c], after["comp_start"][c + 1]
        assert np.max(np.abs(box.positions(c) - after["pos"][a:b]), initial=0.0) <= 1e-9


@pytest.mark.parametrize("cl", [2, 8])
def test_mixture_gcmc_on_clusters_matches_oracle(grx_lib, cl):
    """Two triclinic CH4 / Xe boxes (LJ only, two moved components each) on thread-block
    clusters: every box's FP64 chain takes its oracle chain's decisions, counts and positions."""
    seeds = (3, 5)
    systems = [synth.ch4_xe_system(k, n_ch4=5, n_xe=5) for k in seeds]
    descs = [mix_descs(grx_lib, stream=k) for k in range(2)]
    boxes = [make_box(grx_lib, s) for s in systems]
    batch = grx_lib.GcmcBatch(boxes, descs, grx_lib.GRX_FP64)
    batch.set_shape(24, 1)
    batch.set_cluster(cl)
    batch.launch(300)
    st, _ = batch.stats()
    batch.close()
    for i, s in enumerate(systems):
        ost, after, _ = O.OracleSystem(s).gcmc([ora_params(d) for d in descs[i]], [s["comp_start"][1], CAP, CAP],
                                               0, 300)
        for k in range(2):
            assert list(st[2 * i + k].attempts) == list(ost[k].attempts)
            assert list(st[2 * i + k].accepted) == list(ost[k].accepted)
            assert st[2 * i + k].n_molecules == ost[k].n_molecules and st[2 * i + k].sum_n == ost[k].sum_n
        for c in (1, 2):
            a, b = after["comp_start"][c], after["comp_start"][c + 1]
            assert np.max(np.abs(boxes[i].positions(c) - after["pos"][a:b]), initial=0.0) <= 1e-9


def test_batch_launch_graph_and_resume(grx_lib):
    seeds = [0, 3, 5, 7]
    systems = [synth.ch4_xe_system(k) for k in seeds]
    descs = [mix_descs(grx_lib, stream=k) for k in range(4)]
    ref_boxes = [make_box(grx_lib, s) for s in systems]
    ref = grx_lib.gcmc_run(ref_boxes, descs, 0, 200, grx_lib.GRX_FP64)
    # two plain launches of 100 steps
    boxes = [make_box(grx_lib, s) for s in systems]
    batch = grx_lib.GcmcBatch(boxes, descs, grx_lib.GRX_FP64)
    batch.launch(100)
    batch.launch(100)
    st, nxt = batch.stats()
    assert nxt == 200
    for a, b in zip(st, ref):
        assert list(a.attempts) == list(b.attempts) and list(a.accepted) == list(b.accepted)
        assert a.n_molecules == b.n_molecules
    for bx, rb in zip(boxes, ref_boxes):
        for c in (1, 2):
            assert np.array_equal(bx.positions(c), rb.positions(c))
    batch.close()
    # the same 200 steps as one CUDA graph of 4 launches x 50 steps
    boxes = [make_box(grx_lib, s) for s in systems]
    batch = grx_lib.GcmcBatch(boxes, descs, grx_lib.GRX_FP64)
    batch.run_graph(50, 4)
    st, nxt = batch.stats()
    assert nxt == 200
    for a, b in zip(st, ref):
        assert list(a.accepted) == list(b.accepted) and a.n_molecules == b.n_molecules
    for bx, rb in zip(boxes, ref_boxes):
        for c in (1, 2):
            assert np.array_equal(bx.positions(c), rb.positions(c))
    # replaying the graph continues the chains from step 200
    batch.reset_stats()
    batch.run_graph(50, 4)
    st2, nxt = batch.stats()
    assert nxt == 400 and sum(sum(x.attempts) for x in st2) > 0
    batch.close()


def test_autotune_keeps_chains_valid(grx_lib):
    systems = [synth.ch4_xe_system(k) for k in (2, 4)]
    boxes = [make_box(grx_lib, s) for s in systems]
    descs = [mix_descs(grx_lib, stream=k) for k in range(2)]
    totals0 = [sum(b.total_energy().values()) for b in boxes]
    for b in boxes:
        b.ewald_total()
    batch = grx_lib.GcmcBatch(boxes, descs, grx_lib.GRX_MIXED)
    chosen, ms = batch.autotune(20)
    assert chosen[0] in (8, 12, 24) and chosen[1] in (1, 2, 4) and batch.shape() == chosen
    assert len(ms) == grx_lib.GCMC_TUNE_CANDIDATES and all(m > 0 for m in ms)
    # two boxes leave SMs idle: the best shape is also probed against clusters of 8
    # (plain, cluster, cluster, plain) and the faster kept
    assert batch.cluster() in (1, 8) and (batch.cluster() == 1 or chosen[0] == 24)
    batch.launch(100)
    st, nxt = batch.stats()
    assert nxt == 2 * 20 * grx_lib.GCMC_TUNE_CANDIDATES + 4 * 20 + 100
    batch.close()
    for i, b in enumerate(boxes):
        esum = st[2 * i].energy[3] + st[2 * i + 1].energy[3]
        nacc = sum(st[2 * i].accepted) + sum(st[2 * i + 1].accepted)
        e1 = sum(b.total_energy().values())
        # mixed precision: each accepted move's dE within 1e-6 kT of FP64
        assert beta() * abs((e1 - totals0[i]) - esum) <= 1e-6 * (nacc + 1)


def test_box_step_windows_continue_each_chain(grx_lib):
    """grx_gcmc_batch_set_box_steps: boxes advanced in launches of different lengths, each
    from its own move index, take exactly the decisions of one long launch per box (FP64)."""
    s = co2_system()
    nfw = s["comp_start"][1]
    descs = [grx_lib.gcmc_desc(1, p_translation=0.25, p_rotation=0.5, p_reinsertion=0.5, p_swap=1.0,
                               pressure_pa=1e6, seed=42, stream=k) for k in range(4)]
    total = 120

    def boxes():
        parent = grx_lib.Box(s, capacity=[nfw, 3 * 64])
        parent.ewald_total()
        return [parent] + [parent.replica() for _ in range(3)]

    ref_boxes = boxes()
    ref = grx_lib.gcmc_run(ref_boxes, descs, 0, total, grx_lib.GRX_FP64)
    win_boxes = boxes()
    batch = grx_lib.GcmcBatch(win_boxes, descs, grx_lib.GRX_FP64)
    batch.set_step(10_000)   # the launch counter is unrelated to the boxes' own move indices
    done = np.zeros(4, dtype=np.int64)
    sizes = [7, 13, 40, 120]
    acc = np.zeros((4, 5), dtype=np.int64)
    while (done < total).any():
        n = np.minimum(sizes, total - done)
        batch.set_box_steps(done.astype(np.uint64), n)
        batch.launch(int(n.max()))
        st, _ = batch.stats()
        batch.reset_stats()
        for i in range(4):
            acc[i] += np.array(st[i].accepted)
        done += n
    st_final = st   # n_molecules: the counts after the last launch
    batch.close()
    for i in range(4):
        assert list(acc[i]) == list(ref[i].accepted)
        assert st_final[i].n_molecules == ref[i].n_molecules
        np.testing.assert_allclose(win_boxes[i].positions(1, 3 * ref[i].n_molecules),
                                   ref_boxes[i].positions(1, 3 * ref[i].n_molecules), atol=1e-9)
