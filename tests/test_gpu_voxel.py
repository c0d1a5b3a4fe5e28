"""Voxel candidate lists of the framework atoms (grx_voxel.cu) against the tile path they
replace: the same trial energies and overlap flags on the same beads (FP64 to 1e-12,
also against the FP64 oracle; the mixed form to the mixed bar), for beads inside the cell
and at unwrapped positions outside it, on the orthorhombic CO2/silica box and a
triclinic CH4/Xe box; and the same GCMC decisions over 300 steps of 8 chains."""
import numpy as np
import pytest

from graspa_gb300 import synth
from oracle import oracle as O
from tests.systems import co2_system

pytestmark = pytest.mark.gpu


def close(a, b, rel):
    return np.all(np.abs(a - b) <= rel * np.maximum(np.abs(b), 1.0))


def trial_beads(s, rng, ntr, chain):
    """ntr trials of `chain` beads: first beads uniform in the cell, chain beads 1-2 A away,
    a third of the trials moved by a lattice vector (unwrapped positions)."""
    cell = np.array(s["cell"]).reshape(3, 3)
    f = rng.uniform(0, 1, (ntr, 3))
    first = f @ cell
    shift = rng.integers(-1, 2, (ntr, 3)) * (rng.uniform(0, 1, (ntr, 1)) < 1 / 3)
    first = first + shift @ cell
    pos = []
    for t in range(ntr):
        pos.append(first[t])
        for _ in range(chain - 1):
            v = rng.normal(size=3)
            pos.append(first[t] + 1.5 * v / np.linalg.norm(v))
    return np.array(pos)


@pytest.mark.parametrize("which", ["co2_silica", "ch4_xe_triclinic"])
def test_voxel_lists_match_tiles_and_oracle(grx_lib, which):
    if which == "co2_silica":
        s = co2_system(n_co2=8)
        comp, chain = 1, 3
    else:
        s = synth.ch4_xe_system(5, n_ch4=6, n_xe=6)
        comp, chain = 1, 1
    nfw = s["comp_start"][1]
    caps = [nfw] + [max(64, s["comp_start"][c + 1] - s["comp_start"][c]) for c in range(1, len(s["comp_start"]) - 1)]
    vox = grx_lib.Box(s, capacity=caps)
    on, dims, entries = vox.voxel_lists()
    assert on, "voxel lists expected on this box"
    assert min(dims) >= 1 and entries > 0
    tile = grx_lib.Box(s, capacity=caps)
    tile.set_voxel_lists(0)
    assert not tile.voxel_lists()[0]
    rng = np.random.default_rng(13)
    ntr = 64
    pos = trial_beads(s, rng, ntr, chain)
    tm = s["templates"][comp]
    q = np.tile(tm["charge"][:chain], ntr)
    ty = np.tile(tm["type"][:chain], ntr)
    args = (pos, q, ty, 10 ** 6, ntr, chain, comp)
    ev, fv = vox.trial_energies(*args, prec=grx_lib.GRX_FP64)
    et, ft = tile.trial_energies(*args, prec=grx_lib.GRX_FP64)
    assert np.array_equal(fv, ft)
    assert close(ev, et, 1e-12), np.max(np.abs(ev - et))
    ora = O.OracleSystem(s)
    eo, fo = ora.trial_energies(pos, np.ones(len(q)), q, np.ones(len(q)), ty, 10 ** 6, ntr, chain, comp)
    assert np.array_equal(fv, np.asarray(fo))
    ok = np.asarray(fo) == 0
    assert close(ev[ok], np.asarray(eo)[ok], 1e-12)
    mv, mfv = vox.trial_energies(*args, prec=grx_lib.GRX_MIXED)
    mt, mft = tile.trial_energies(*args, prec=grx_lib.GRX_MIXED)
    assert np.array_equal(mfv, mft)
    beta = grx_lib.beta_from_temperature(300.0)
    assert np.max(beta * np.abs(mv[ok] - mt[ok])) < 1e-8
    assert np.max(beta * np.abs(mv[ok] - et[ok])) < 1e-6


def test_voxel_lists_same_gcmc_decisions(grx_lib):
    s = co2_system()
    nfw = s["comp_start"][1]
    res = {}
    for on in (1, 0):
        parent = grx_lib.Box(s, capacity=[nfw, 3 * 160])
        parent.set_voxel_lists(on)
        parent.ewald_total()
        boxes = [parent] + [parent.replica() for _ in range(7)]
        assert boxes[3].voxel_lists()[0] == bool(on)
        descs = [grx_lib.gcmc_desc(1, p_translation=0.25, p_rotation=0.5, p_reinsertion=0.5, p_swap=1.0,
                                   pressure_pa=1e5, seed=42, stream=k) for k in range(8)]
        res[on] = grx_lib.gcmc_run(boxes, descs, 0, 300, grx_lib.GRX_FP64)
        for b in reversed(boxes):
            b.close()
    for a, b in zip(res[1], res[0]):
        assert list(a.accepted) == list(b.accepted) and a.n_molecules == b.n_molecules
        assert abs(a.energy[3] - b.energy[3]) <= 1e-9 * max(1.0, abs(b.energy[3]))
        assert a.trial_configs == b.trial_configs
