"""gRASPA's Examples/Reference_NIST_SPCE boxes from the reference's own input files
(committed under tests/golden/nist_spce/ by tests/golden/make_nist_spce_inputs.py) through
the C++ input readers, on the CPU: graspa_run --dump reads simulation.input (RestartFile
yes), the atom-less Box-N.cif that defines the triclinic cell, SPCE.def, the force-field
files (force_field.def switches the O-O tail correction on) and the RASPA restart file
with the SPC/E molecules. The parsed molecules are the NIST configuration (up to lattice
vectors: each molecule is unwrapped around its first atom, as RestartFileParser does), the
FP64 oracle on the parsed system gives the printed VDW, real-space, Fourier, self and
intramolecular exclusion energies, and the host layer's tail correction energy equals the
printed TailE. No GPU is involved."""
import json
import os
import subprocess

import numpy as np
import pytest

from graspa_gb300 import build as B
from oracle import oracle as O
from tests.test_input_formats import system_from_dump

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIX = os.path.join(GOLD, "nist_spce")


def printed_close(x, ref):
    """the reference prints 5 decimals"""
    return abs(x - ref) <= 1e-5 + 1e-12 * abs(ref)


@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_nist_box_from_restart_file(n, tmp_path):
    B.build()
    out = tmp_path / "d.json"
    r = subprocess.run([B.RUNNER, os.path.join(FIX, f"Box-{n}"), "--dump", str(out)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    d = json.load(open(out))
    e = json.load(open(os.path.join(FIX, "expected.json")))["boxes"][f"Box-{n}"]
    ref = json.load(open(os.path.join(GOLD, f"nist_spce_box{n}.json")))
    assert d["molecules"][1] == e["molecules"]
    assert np.allclose(d["cell"], ref["cell"], rtol=0, atol=1e-12)
    assert d["kmax"] == [7, 7, 7] and d["alpha"] == 0.285
    assert printed_close(d["volume"], e["volume"])
    c = d["components"][1]
    p = np.array(c["pos"]).reshape(-1, 3)[:c["size"]]
    q = np.array(ref["pos"])
    f = (p - q) @ np.linalg.inv(np.array(d["cell"]).reshape(3, 3))
    assert np.abs(f - np.round(f)).max() < 1e-9          # the same atoms up to lattice vectors
    assert printed_close(d["tail_energy"], e["tail"])
    # the FP64 oracle on the parsed system
    s = system_from_dump(d)
    S = O.OracleSystem(s)
    vdw_real = S.vdw_real_total()
    out8, _, _ = S.ewald_total([1, 3])
    assert printed_close(vdw_real[4], e["gg_vdw"]) and printed_close(vdw_real[5], e["gg_real"])
    assert printed_close(out8[0], e["fourier_gg"])
    assert printed_close(out8[3], e["self_atoms"]) and printed_close(out8[5], e["intra_exclusion"])
