"""The XeKr-Mixture example's inputs (committed under tests/golden/xekr/ by
tests/golden/make_xekr.py) through the C++ input readers, on the CPU: graspa_run --dump
parses simulation.input (identity-change probabilities, FugacityCoefficient PR-EOS),
the single-atom Kr.def / Xe.def, the pseudo atoms with their masses and the triclinic
25.cif, and reproduces what the reference printed for the run: the Peng-Robinson
fugacity coefficients of the 0.1/0.9 Kr/Xe mixture at 273 K and 1e5 Pa, the framework
mass, box volume and framework density. No GPU is involved."""
import json
import os
import subprocess

import pytest

from graspa_gb300 import build as B

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "xekr")


@pytest.fixture(scope="module")
def dump(tmp_path_factory):
    B.build()
    out = tmp_path_factory.mktemp("xekr") / "xekr.json"
    r = subprocess.run([B.RUNNER, FIX, "--dump", str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return json.load(open(out)), json.load(open(os.path.join(FIX, "expected.json")))


def test_pr_eos_fugacity_coefficients(dump):
    d, e = dump
    # printed with 10 decimals (output_1e5.txt:324,327)
    assert abs(d["fugacity_coeff"][1] - e["fugacity_coefficient"]["Kr"]) < 1e-10
    assert abs(d["fugacity_coeff"][2] - e["fugacity_coefficient"]["Xe"]) < 1e-10
    assert d["mol_fraction"][1:] == [0.1, 0.9]


def test_framework_mass_volume_density(dump):
    d, e = dump
    assert abs(d["framework_mass"] - e["framework_mass_g_per_mol"]) < 1e-9 * e["framework_mass_g_per_mol"]
    assert abs(d["volume"] - e["box_volume"]) < 1e-5
    assert abs(d["framework_density"] - e["widom_kr"]["framework_density_kg_m3"]) < 1e-5
    assert len(d["components"][0]["pos"]) == 3 * 1216


def test_move_probabilities_and_force_field(dump):
    d, _ = dump
    # cumulative translation, rotation, reinsertion, identity swap, swap (the reference's
    # ACCUMULATED probabilities: Kr 0.25 / 0.25 / 0.5 / 0.75 / 1, Xe 1/3 / 1/3 / 1/3 / 2/3 / 1)
    assert d["move_probabilities"][1] == pytest.approx([0.25, 0.25, 0.5, 0.75, 1.0])
    assert d["move_probabilities"][2] == pytest.approx([1 / 3, 1 / 3, 1 / 3, 2 / 3, 1.0])
    assert d["no_charges"] == 1
    nt = d["ntypes"]
    # the reference's MIXED VDW PARAMETERS: C-Xe ep 89.8401268338, sig 3.765; Xe-Kr 159.4434606674, 3.868
    C, Xe, Kr = 0, 5, 6
    assert abs(d["epsilon"][C * nt + Xe] - 89.8401268338) < 1e-9
    assert abs(d["sigma"][C * nt + Xe] - 3.765) < 1e-12
    assert abs(d["epsilon"][Xe * nt + Kr] - 159.4434606674) < 1e-9
    assert all(s == 0.0 for s in d["shift"])  # truncated, not shifted
