"""Replica boxes (grx_box_create_replica): chains that share one framework copy give
exactly the results of independent boxes (FP64 decisions, positions, energies), and
the sharing is guarded (no framework edits or parent destruction while replicas live)."""
import numpy as np
import pytest

from tests.systems import co2_system
from tests.test_gpu_gcmc import params

pytestmark = pytest.mark.gpu


def test_replicas_equal_independent_boxes(grx_lib):
    s = co2_system(n_co2=3)
    nfw = s["comp_start"][1]
    cap = [nfw, 3 * 64]
    parent = grx_lib.Box(s, capacity=cap)
    parent.ewald_total()
    reps = [parent.replica() for _ in range(3)]
    chains = [parent] + reps
    indep = []
    for _ in range(4):
        b = grx_lib.Box(s, capacity=cap)
        b.ewald_total()
        indep.append(b)
    descs = [params(grx_lib, stream=k, pressure_pa=1e6) for k in range(4)]
    a = grx_lib.gcmc_run(chains, descs, 0, 250, grx_lib.GRX_FP64)
    b = grx_lib.gcmc_run(indep, descs, 0, 250, grx_lib.GRX_FP64)
    for x, y in zip(a, b):
        assert list(x.accepted) == list(y.accepted) and x.n_molecules == y.n_molecules
        assert x.energy[3] == y.energy[3]
    for x, y in zip(chains, indep):
        assert np.array_equal(x.positions(1), y.positions(1))
        assert np.array_equal(x.positions(0), y.positions(0))          # the shared framework
        ex, ey = x.total_energy(), y.total_energy()
        for k in ex:
            assert abs(ex[k] - ey[k]) <= 1e-9 * max(1.0, abs(ey[k]))
    # Widom on a replica equals Widom on an independent box in the same state
    d = grx_lib.widom_desc(s, 1, 10, 10, seed=5)
    ra = reps[1].widom(d, 0, 64, grx_lib.GRX_MIXED)
    rb = indep[2].widom(d, 0, 64, grx_lib.GRX_MIXED)
    assert np.array_equal(ra["rosenbluth"], rb["rosenbluth"])
    # guards
    with pytest.raises(grx_lib.GrxError):
        parent.set_component(0)
    with pytest.raises(grx_lib.GrxError):
        reps[0].replica()
    assert grx_lib.load().grx_box_destroy(parent.h) != 0              # still has replicas
    for r in reps:
        r.close()
    parent.set_component(0)                                            # allowed again
