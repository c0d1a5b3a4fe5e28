"""Generate the XeKr-Mixture statistical fixture: the reference's published GCMC run
that pins this engine's loadings and Widom statistics.

gRASPA's Examples/XeKr-Mixture is a GCMC run of a Kr/Xe mixture (mole fractions
0.1/0.9, 1e5 Pa, 273 K, PR-EOS fugacity coefficients) in the 25.cif MOF (2x2x2 triclinic
P1 cell, 1216 atoms), LJ only (ChargeMethod None, 12 A truncated cutoff), with
translation, reinsertion (Kr), identity swaps and CBMC insertion / deletion (10 trial
positions), one step per cycle. Its output_1e5.txt prints, from 1e5 initialization
and 1e6 production cycles in 5 blocks:
  * the Peng-Robinson fugacity coefficients of both components (output_1e5.txt:324-327);
  * block averages of the loadings in molecules and mol/kg (:1899-1987), whose
    "ErrorBar" is twice the population standard deviation of the 5 block averages;
  * the Rosenbluth summary of the Kr insertions (:2018-2079): per-block <W>, excess
    chemical potential and Henry coefficient, the framework density, and the averages
    with twice the population standard deviation of the blocks.

This script copies the example's input files unchanged into tests/golden/xekr/ and
writes the published numbers to tests/golden/xekr/expected.json. It runs only where the
reference tree is available; the fixture is committed, so no test reads the reference.

Usage: python tests/golden/make_xekr.py /path/to/gRASPA  (the reference checkout; required)
"""
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = ["simulation.input", "25.cif", "Kr.def", "Xe.def", "pseudo_atoms.def", "force_field_mixing_rules.def",
         "force_field.def"]


def _floats(pattern, text):
    out = []
    for x in re.findall(pattern, text):
        out.extend(float(v) for v in (x if isinstance(x, tuple) else (x,)))
    return out


def _block_section(text, title, comp):
    """Block averages and the Overall line of one component inside a BLOCK AVERAGES section."""
    sec = text.split(title, 1)[1]
    sec = sec.split("==============================================================", 1)[0]
    part = sec.split(f"COMPONENT [{comp}]", 1)[1].split("----------------------------------------------------------", 1)[0]
    blocks = _floats(r"BLOCK \[\d+\], Blocksize: \d+, Average: ([-\d.eE+]+)", part)
    m = re.search(r"Overall: Average: ([-\d.eE+]+), ErrorBar: ([-\d.eE+nan]+)", part)
    return {"blocks": blocks, "average": float(m.group(1)), "errorbar_2sigma": float(m.group(2))}


def main(ref):
    src = os.path.join(ref, "Examples", "XeKr-Mixture")
    dst = os.path.join(HERE, "xekr")
    os.makedirs(dst, exist_ok=True)
    for f in FILES:
        shutil.copyfile(os.path.join(src, f), os.path.join(dst, f))
    text = open(os.path.join(src, "output_1e5.txt")).read()
    fug = {int(a): float(b) for a, b in re.findall(r"Fugacity Coefficient for component (\d+) is ([\d.]+)", text)}
    ros = text.split("=====================Rosenbluth Summary=====================", 1)[1]
    avg = ros.split("=========================AVERAGE========================", 1)[1]
    exp = {
        "source": "Examples/XeKr-Mixture/output_1e5.txt",
        "temperature": 273.0, "pressure_pa": 1e5, "mol_fraction": {"Kr": 0.1, "Xe": 0.9},
        "cycles": {"initialization": 100000, "production": 1000000, "blocks": 5, "steps_per_cycle": 1},
        "fugacity_coefficient": {"Kr": fug[1], "Xe": fug[2]},
        "framework_mass_g_per_mol": float(re.search(r"Framework total mass: ([\d.]+)", text).group(1)),
        "box_volume": float(re.search(r"Box Volume:\s+([\d.]+)", text).group(1)),
        "loading_molecules": {"Kr": _block_section(text, "BLOCK AVERAGES (LOADING: # MOLECULES)", 1),
                              "Xe": _block_section(text, "BLOCK AVERAGES (LOADING: # MOLECULES)", 2)},
        "loading_mol_per_kg": {"Kr": _block_section(text, "BLOCK AVERAGES (LOADING: mol/kg)", 1),
                               "Xe": _block_section(text, "BLOCK AVERAGES (LOADING: mol/kg)", 2)},
        "widom_kr": {
            "insertions_per_block": _floats(r"Widom Performed: ([\d.]+)", ros),
            "framework_density_kg_m3": _floats(r"Framework Density: ([\d.]+)", ros)[0],
            "block_rosenbluth": _floats(r"\(Total\) Averaged Rosenbluth Weight: ([\d.]+)", ros),
            "block_henry": _floats(r"\(Total\) Averaged Henry Coefficient: ([\d.]+)", ros),
            "block_mu_ex_K": _floats(r"\(Total\) Averaged Excess Mu: ([-\d.]+)", ros),
            "rosenbluth": _floats(r"Averaged Rosenbluth Weight: ([\d.]+) \+/- ([\d.]+)", avg),
            "mu_ex_K": _floats(r"Averaged Excess Chemical Potential: ([-\d.]+) \+/- ([\d.]+)", avg),
            "henry_mol_kg_pa": _floats(r"Averaged Henry Coefficient \[mol/kg/Pa\]: ([\d.eE+-]+) \+/- ([\d.eE+-]+)",
                                       avg),
        },
    }
    with open(os.path.join(dst, "expected.json"), "w") as f:
        json.dump(exp, f, indent=1)
    print(json.dumps(exp, indent=1))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_xekr.py /path/to/gRASPA")
    main(sys.argv[1])
