"""The FP64 oracle against the reference's own NIST SPC/E outputs.

gRASPA's committed outputs (Examples/Reference_NIST_SPCE/Box-*/output.txt) print
every energy term with 5 decimals; the oracle must reproduce each printed value to
that precision (|diff| <= 0.5e-5 after rounding, checked as <= 1e-5), plus the
number of active wave vectors of the NIST table (readme.md:14).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.systems import nist_system

NIST_WAVE_VECTORS = {1: 831, 2: 1068, 3: 838, 4: 1028}


@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_nist_totals(n):
    s, e = nist_system(n)
    S = O.OracleSystem(s)
    assert abs(S.box.volume - e["volume"]) < 1e-5
    assert abs(S.box.reciprocal_cutoff - e["reciprocal_cutoff"]) < 1e-5
    tot = S.vdw_real_total()
    assert abs(tot[4] - e["gg_vdw"]) < 1e-5
    assert abs(tot[5] - e["gg_real"]) < 1e-5
    assert tot[0] == 0 and tot[1] == 0 and tot[2] == 0 and tot[3] == 0
    ew, s_fw, s_ads = S.ewald_total([1, 3])
    assert abs(ew[0] - e["fourier_gg"]) < 1e-5
    assert abs(ew[3] - e["self_atoms"]) < 1e-5
    assert abs(ew[5] - e["intra_exclusion"]) < 1e-5
    assert int(ew[7]) == NIST_WAVE_VECTORS[n]
    nact, act = S.ewald_active()
    assert nact == NIST_WAVE_VECTORS[n]
    assert np.all(s_fw == 0)


@pytest.mark.parametrize("n", [1, 4])
def test_nist_rigid_exclusion(n):
    s, e = nist_system(n)
    S = O.OracleSystem(s)
    intra, self_ = S.rigid_exclusion(s["pos"][:3], s["charge"][:3], np.ones(3))
    assert abs(intra - e["rigid_exclusion_intra"]) < 1e-5
    assert abs(self_ - e["rigid_exclusion_self"]) < 1e-5


def test_ewald_delta_matches_total_difference():
    """Deleting one molecule through the delta path equals the change of the FP64
    Fourier total (same-type block), the identity the reference's drift check uses."""
    s, _ = nist_system(4)
    S = O.OracleSystem(s)
    ew0, s_fw, s_ads = S.ewald_total([1, 3])
    mol = 7
    idx = np.arange(3 * mol, 3 * mol + 3)
    pos = s["pos"][idx]
    qs = s["charge"][idx]
    d, s_new = S.ewald_delta(s_ads, s_fw, pos, qs, np.zeros((0, 3)), np.zeros(0))
    keep = np.ones(len(s["charge"]), bool)
    keep[idx] = False
    s2 = dict(s)
    for k in ("pos", "scale", "charge", "scale_coul", "type", "molid"):
        s2[k] = np.asarray(s[k])[keep]
    s2["molid"] = np.repeat(np.arange(keep.sum() // 3), 3)
    s2["comp_start"] = [0, 0, int(keep.sum())]
    S2 = O.OracleSystem(s2)
    ew1, _, s_ads1 = S2.ewald_total([1, 3])
    assert abs((ew1[0] - ew0[0]) - d[0]) < 1e-8 * abs(ew0[0])
    assert np.allclose(s_new, s_ads1, atol=1e-9)
