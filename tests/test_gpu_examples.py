"""graspa_run (the C++ host layer's example runner) on gRASPA's Examples/CO2-MFI inputs
(committed under tests/golden/co2_mfi/) on the GPU: the device FP64 initial-stage
energies equal the reference's printed values, and a shortened GCMC run (the first
cycles of each phase) adsorbs CO2 and passes the energy drift check."""
import json
import os
import re
import subprocess

import pytest

from graspa_gb300 import build as B

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "co2_mfi")


def run(*args, timeout=900):
    B.build()
    r = subprocess.run([B.RUNNER, FIX, *args], capture_output=True, text=True, timeout=timeout)
    assert r.returncode == 0, r.stderr
    return r.stdout


def test_co2_mfi_initial_stage_on_device():
    out = run("--max-cycles", "0", "--precision", "fp64")
    e = json.load(open(os.path.join(FIX, "expected.json")))
    m = re.search(r"Fourier GG (\S+) HH (\S+) HG (\S+)", out)
    assert abs(float(m.group(2)) - e["fourier_hh"]) <= 1e-5 + 1e-12 * e["fourier_hh"]
    m = re.search(r"SelfAtomE all (\S+) host (\S+)", out)
    assert abs(float(m.group(2)) - e["self_framework"]) <= 1e-10 * e["self_framework"]
    m = re.search(r"IntraExclusionE all (\S+) host (\S+)", out)
    assert abs(abs(float(m.group(2))) - e["intra_exclusion_framework"]) <= 1e-10 * e["intra_exclusion_framework"]
    m = re.search(r"Component 1 rigid exclusion intra (\S+) self (\S+)", out)
    assert abs(float(m.group(1)) - e["co2_intra_exclusion"]) < 1e-5
    assert abs(float(m.group(2)) - e["co2_self_exclusion"]) < 1e-5
    m = re.search(r"EwaldVectors total (\d+)", out)
    assert int(m.group(1)) == e["structure_factor_slots"]


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_co2_mfi_short_run(prec):
    out = run("--max-cycles", "300", "--precision", prec)
    n = int(re.search(r"INITIALIZATION ends: molecules \[CO2\] (\d+)", out).group(1))
    assert n > 0
    moves = re.search(r"insertion (\d+)/(\d+) deletion (\d+)/(\d+)", out)
    assert int(moves.group(1)) > 0
    drift = float(re.search(r"ENERGY DRIFT (\S+)", out).group(1))
    beta = 1.0 / (1.380649e-23 / 1.6605402e-23 * 298.0)
    # FP64: summation order only; mixed: 1e-6 kT per accepted move at most
    acc = sum(int(x) for x in re.findall(r"(\d+)/\d+", out.split("moves:")[1].split("\n")[0])[::1])
    bound = 1e-7 if prec == "fp64" else 1e-6 * (acc + 1)
    assert beta * abs(drift) <= bound, (drift, acc)


NIST = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "nist_spce")


@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_nist_spce_box_end_to_end(n):
    """Examples/Reference_NIST_SPCE/Box-n from the reference's own files (restart file with
    the SPC/E molecules, atom-less CIF cell, O-O tail correction) through graspa_run: the
    device FP64 totals reproduce the values Box-n/output.txt printed (5 decimals)."""
    B.build()
    r = subprocess.run([B.RUNNER, os.path.join(NIST, f"Box-{n}"), "--max-cycles", "0", "--precision", "fp64"],
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr
    out = r.stdout
    e = json.load(open(os.path.join(NIST, "expected.json")))["boxes"][f"Box-{n}"]

    def close(x, ref):
        return abs(x - ref) <= 1e-5 + 1e-12 * abs(ref)

    m = re.search(r"Total HHVDW \S+ HHReal \S+ HGVDW \S+ HGReal \S+ GGVDW (\S+) GGReal (\S+) HHEwald \S+ HGEwald \S+ "
                  r"GGEwald (\S+)", out)
    assert close(float(m.group(1)), e["gg_vdw"]) and close(float(m.group(2)), e["gg_real"])
    assert close(float(m.group(3)), e["gg_ewald"])
    assert close(float(re.search(r"Fourier GG (\S+)", out).group(1)), e["fourier_gg"])
    assert close(float(re.search(r"SelfAtomE all (\S+)", out).group(1)), e["self_atoms"])
    assert close(abs(float(re.search(r"IntraExclusionE all (\S+)", out).group(1))), e["intra_exclusion"])
    assert close(float(re.search(r"TailE (\S+)", out).group(1)), e["tail"])
