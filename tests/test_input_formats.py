"""The C++ input readers (graspa_gb300/host/graspa_input.cpp) on gRASPA's own
Examples/CO2-MFI inputs (committed under tests/golden/co2_mfi/): graspa_run --dump
parses simulation.input, the force-field files, CO2.def and the 2x2x2 MFI CIF, and the
FP64 oracle on the parsed system reproduces the reference's printed initial-stage
values (host-host Fourier energy, framework self and intramolecular exclusion energies,
CO2 rigid exclusion constants, structure-factor slots). No GPU is involved."""
import json
import os
import subprocess

import numpy as np
import pytest

from graspa_gb300 import build as B
from oracle import oracle as O

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "co2_mfi")


def system_from_dump(d):
    comps = d["components"]
    pos, q, ty, mol, starts = [], [], [], [], [0]
    for c, cc in enumerate(comps):
        n = cc["size"]
        p = np.array(cc["pos"]).reshape(-1, 3)[:n]
        pos.append(p)
        q.append(np.array(cc["charge"])[:n])
        ty.append(np.array(cc["type"], dtype=int)[:n])
        ms = cc["molsize"]
        mol.append(np.zeros(n, dtype=int) if c == 0 else np.repeat(np.arange(n // ms), ms))
        starts.append(starts[-1] + n)
    n = starts[-1]
    templates = {}
    for c in range(1, len(comps)):
        cc = comps[c]
        ms = cc["molsize"]
        templates[c] = dict(pos=np.array(cc["pos"]).reshape(-1, 3)[:ms], charge=np.array(cc["charge"])[:ms],
                            type=np.array(cc["type"], dtype=int)[:ms])
    return dict(cell=d["cell"], kmax=d["kmax"], alpha=d["alpha"], use_lammps_ewald=d["use_lammps_ewald"],
                prefactor=d["prefactor"], reciprocal_cutoff=d["reciprocal_cutoff"], ntypes=d["ntypes"],
                epsilon=np.array(d["epsilon"]), sigma=np.array(d["sigma"]), shift=np.array(d["shift"]),
                cutoff_vdw=d["cutoff_vdw"], cutoff_coul=d["cutoff_coul"], overlap_criteria=d["overlap_criteria"],
                no_charges=d["no_charges"], vdw_real_bias=1, nhost=1, comp_start=starts,
                pos=np.concatenate(pos), scale=np.ones(n), charge=np.concatenate(q), scale_coul=np.ones(n),
                type=np.concatenate(ty), molid=np.concatenate(mol), molsize=[c["molsize"] for c in comps],
                templates=templates, temperature=d["temperature"])


@pytest.fixture(scope="module")
def co2_mfi(tmp_path_factory):
    B.build()
    out = str(tmp_path_factory.mktemp("dump") / "co2_mfi.json")
    r = subprocess.run([B.RUNNER, FIX, "--dump", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return json.load(open(out)), json.load(open(os.path.join(FIX, "expected.json")))


def test_parsed_system(co2_mfi):
    d, e = co2_mfi
    assert len(d["components"][0]["pos"]) == 3 * e["framework_atoms"]
    assert d["kmax"] == [11, 11, 7] and d["use_lammps_ewald"] == 0
    assert abs(d["alpha"] - 0.26505830360350674) < 1e-15
    nv = (d["kmax"][0] + 1) * (2 * d["kmax"][1] + 1) * (2 * d["kmax"][2] + 1)
    assert nv == e["structure_factor_slots"]
    co2 = d["components"][1]
    assert co2["molsize"] == 3 and co2["charge"] == [-0.3256, 0.6512, -0.3256]
    # CIF charges: Si +2.05, O -1.025 (neutral framework)
    assert abs(sum(d["components"][0]["charge"])) < 1e-9
    assert abs(d["pressure_internal"] - 1e4 / 1.6605402e7) < 1e-15


def test_initial_stage_energies_match_reference(co2_mfi):
    d, e = co2_mfi
    s = system_from_dump(d)
    S = O.OracleSystem(s)
    ew, s_fw, _ = S.ewald_total(s["molsize"])
    assert abs(ew[1] - e["fourier_hh"]) <= 1e-5 + 1e-12 * e["fourier_hh"]
    assert abs(ew[4] - e["self_framework"]) <= 1e-10 * e["self_framework"]
    assert abs(abs(ew[6]) - e["intra_exclusion_framework"]) <= 1e-10 * e["intra_exclusion_framework"]
    tm = s["templates"][1]
    intra, self_ = S.rigid_exclusion(tm["pos"], tm["charge"], np.ones(3))
    assert abs(intra - e["co2_intra_exclusion"]) < 1e-5
    assert abs(self_ - e["co2_self_exclusion"]) < 1e-5
