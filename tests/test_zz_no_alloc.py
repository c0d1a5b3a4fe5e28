"""The allocation-free trial-energy entry point against the regular one.

grx_trial_energies_noalloc serves callers that cannot let a call allocate device
memory (a Monte Carlo loop that must not stall the GPU with cudaMalloc/cudaFree,
or a host application that owns all device memory through its own pool). It must
give the same energies and overlap flags as grx_trial_energies, through the C ABI,
on consecutive calls that reuse its fixed scratch array. This file is collected
last on purpose.
"""
import numpy as np
import pytest

from tests.systems import co2_system

pytestmark = pytest.mark.gpu


def _close(a, b):  # the FP64 bar of the parity tests
    return np.all(np.abs(a - b) <= 1e-12 * np.maximum(np.abs(b), 1.0))


def test_noalloc_matches_regular_entry_point(grx_lib):
    s = co2_system(n_co2=8)
    nfw = s["comp_start"][1]
    box = grx_lib.Box(s, capacity=[nfw, 3 * 32])
    rng = np.random.default_rng(21)
    cell = np.array(s["cell"]).reshape(3, 3).T
    tm = s["templates"][1]
    for call in range(2):  # two calls in a row share the scratch array
        for prec in (grx_lib.GRX_FP64, grx_lib.GRX_MIXED):
            ntr = 12
            pos = (cell @ rng.uniform(0, 1, (3, ntr))).T
            q = np.full(ntr, tm["charge"][0])
            ty = np.full(ntr, tm["type"][0])
            ref, rf = box.trial_energies(pos, q, ty, 8, ntr, 1, 1, prec=prec)
            got, gf = box.trial_energies_noalloc(pos, q, ty, 8, ntr, 1, 1, prec=prec)
            assert np.array_equal(gf, rf)
            assert _close(got, ref), np.max(np.abs(got - ref))
            # chain beads: 10 orientations x 2 beads
            first = cell @ rng.uniform(0, 1, 3)
            v = tm["pos"][1:] - tm["pos"][0]
            cp = np.concatenate([first + v @ np.linalg.qr(rng.normal(size=(3, 3)))[0].T for _ in range(10)])
            cq = np.tile(tm["charge"][1:], 10)
            ct = np.tile(tm["type"][1:], 10)
            ref, rf = box.trial_energies(cp, cq, ct, 8, 10, 2, 1, prec=prec, excl_comp=1, excl_molid=3)
            got, gf = box.trial_energies_noalloc(cp, cq, ct, 8, 10, 2, 1, prec=prec, excl_comp=1, excl_molid=3)
            assert np.array_equal(gf, rf)
            assert _close(got, ref), np.max(np.abs(got - ref))


def test_noalloc_rejects_oversized_requests(grx_lib):
    s = co2_system(n_co2=0)
    nfw = s["comp_start"][1]
    box = grx_lib.Box(s, capacity=[nfw, 3 * 8])
    n = 257  # one bead past GRX_NOALLOC_MAX_BEADS
    pos = np.zeros((n, 3)) + 5.0
    with pytest.raises(grx_lib.GrxError, match="capacity exceeded"):
        box.trial_energies_noalloc(pos, np.zeros(n), np.zeros(n, dtype=int), 0, n, 1, 1)
