"""Generate the CO2-MFI known-answer fixture used to pin the input-file readers.

gRASPA's Examples/CO2-MFI is a GCMC run of CO2 in the all-silica MFI zeolite (2x2x2
P1 cell, 2304 atoms, CIF charges, RASPA-2 Ewald set-up at precision 1e-6, CutOffVDW
12.8 A, CutOffCoulomb 12 A, 298 K, 1e4 Pa). Its output.txt prints the FP64
initial-stage Ewald terms (output.txt:53-64: host-host Fourier, framework self and
intramolecular exclusion energies, CO2 rigid exclusion constants) and the number of
structure-factor slots (:80).

This script copies the example's input files (simulation.input, CO2.def,
force_field_mixing_rules.def, pseudo_atoms.def, MFI-2x2x2-P1.cif) unchanged into
tests/golden/co2_mfi/ and writes the printed values to tests/golden/co2_mfi/expected.json.
It runs only where the reference tree is mounted; the fixture is committed so nothing
at test time reads the reference.

Usage: python tests/golden/make_co2_mfi.py /path/to/gRASPA  (the reference checkout; required)
"""
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = ["simulation.input", "CO2.def", "force_field_mixing_rules.def", "pseudo_atoms.def", "MFI-2x2x2-P1.cif"]


def main(ref):
    src = os.path.join(ref, "Examples", "CO2-MFI")
    dst = os.path.join(HERE, "co2_mfi")
    os.makedirs(dst, exist_ok=True)
    for f in FILES:
        shutil.copyfile(os.path.join(src, f), os.path.join(dst, f))
    text = open(os.path.join(src, "output.txt")).read()

    def num(pattern):
        m = re.search(pattern, text)
        if not m:
            raise SystemExit(f"pattern not found: {pattern}")
        return float(m.group(1))

    exp = {
        "fourier_hh": num(r"Host-Host Fourier:\s*([-0-9.]+)"),
        "self_framework": num(r"Component: 0, SelfAtomE:\s*([-0-9.]+)"),
        "intra_exclusion_framework": num(r"Component: 0, Intra-Molecular ExclusionE:\s*([-0-9.]+)"),
        "co2_intra_exclusion": num(r"Component 1, Intra Exclusion Energy:\s*([-0-9.]+)"),
        "co2_self_exclusion": num(r"Component 1, Atom Self Exclusion Energy:\s*([-0-9.]+)"),
        "structure_factor_slots": int(num(r"CPU SF:\s*([0-9]+)")),
        "framework_atoms": 2304,
        "source": "Examples/CO2-MFI/output.txt",
    }
    with open(os.path.join(dst, "expected.json"), "w") as f:
        json.dump(exp, f, indent=1)
    print(json.dumps(exp))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_co2_mfi.py /path/to/gRASPA")
    main(sys.argv[1])
