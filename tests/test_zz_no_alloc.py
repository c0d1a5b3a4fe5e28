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


def test_noalloc_fp32_null_pointers_and_full_capacity(grx_lib):
    """The FP32 form, the null scale / charge / scaleCoul pointers (charges 0, scalings 1)
    and exactly GRX_NOALLOC_MAX_BEADS beads (128 trials x 2 beads: the far end of the
    scratch layout), each against grx_trial_energies."""
    s = co2_system(n_co2=8)
    nfw = s["comp_start"][1]
    box = grx_lib.Box(s, capacity=[nfw, 3 * 32])
    rng = np.random.default_rng(5)
    cell = np.array(s["cell"]).reshape(3, 3).T
    tm = s["templates"][1]
    ntr = 128
    v = tm["pos"][1:] - tm["pos"][0]
    pos = np.concatenate([cell @ rng.uniform(0, 1, 3) + v @ np.linalg.qr(rng.normal(size=(3, 3)))[0].T
                          for _ in range(ntr)])
    q = np.tile(tm["charge"][1:], ntr)
    ty = np.tile(tm["type"][1:], ntr)
    for prec in (grx_lib.GRX_FP64, grx_lib.GRX_MIXED, grx_lib.GRX_FP32):
        for call in range(2):
            ref, rf = box.trial_energies(pos, q, ty, 8, ntr, 2, 1, prec=prec)
            got, gf = box.trial_energies_noalloc(pos, q, ty, 8, ntr, 2, 1, prec=prec)
            assert np.array_equal(gf, rf)
            assert _close(got, ref), np.max(np.abs(got - ref))
        # null pointers: the regular entry point with the values they stand for
        ref, rf = box.trial_energies(pos, np.zeros(2 * ntr), ty, 8, ntr, 2, 1, prec=prec,
                                     scale=np.ones(2 * ntr), scale_coul=np.ones(2 * ntr))
        got, gf = box.trial_energies_noalloc(pos, None, ty, 8, ntr, 2, 1, prec=prec)
        assert np.array_equal(gf, rf)
        assert _close(got, ref), np.max(np.abs(got - ref))
        assert np.all(got[:, [1, 3]] == 0.0)


def test_noalloc_allocates_no_device_memory(grx_lib):
    """After a warm-up call (kernels loaded, scratch address looked up), further calls
    leave the device's free memory unchanged."""
    torch = pytest.importorskip("torch")
    s = co2_system(n_co2=8)
    nfw = s["comp_start"][1]
    box = grx_lib.Box(s, capacity=[nfw, 3 * 32])
    rng = np.random.default_rng(9)
    cell = np.array(s["cell"]).reshape(3, 3).T
    tm = s["templates"][1]
    ntr = 100
    pos = (cell @ rng.uniform(0, 1, (3, ntr))).T
    q = np.full(ntr, tm["charge"][0])
    ty = np.full(ntr, tm["type"][0])
    for prec in (grx_lib.GRX_FP64, grx_lib.GRX_MIXED, grx_lib.GRX_FP32):
        box.trial_energies_noalloc(pos, q, ty, 8, ntr, 1, 1, prec=prec)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        for prec in (grx_lib.GRX_FP64, grx_lib.GRX_MIXED, grx_lib.GRX_FP32):
            box.trial_energies_noalloc(pos, q, ty, 8, ntr, 1, 1, prec=prec)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
