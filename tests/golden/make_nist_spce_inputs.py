"""Copy gRASPA's Examples/Reference_NIST_SPCE input directories (one per box) for the
end-to-end runs of graspa_run on the reference's own files.

Each Box-N directory holds simulation.input (RestartFile yes, LAMMPS Ewald set-up with
alpha 0.285 and 7 k vectors per axis, 10 A cutoffs), Box-N.cif (the triclinic cell, no
framework atoms), SPCE.def, the force-field files (O-O truncated with the tail
correction, force_field.def) and RestartInitial/System_0/restartfile with the SPC/E
molecules. The files are copied unchanged to tests/golden/nist_spce/Box-N/, and
tests/golden/nist_spce/expected.json receives the values the reference printed for each
box (Box-N/output.txt, initial stage): guest-guest VDW and real-space Coulomb, the
Fourier term, the atom-self and intramolecular exclusion energies, the tail correction
energy, the number of structure-factor slots and the box volume (internal units, the
printed 5 decimals). The fixture is committed, so no test reads the reference.

Usage: python tests/golden/make_nist_spce_inputs.py /path/to/gRASPA  (the reference checkout; required)
"""
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = ["simulation.input", "SPCE.def", "force_field.def", "force_field_mixing_rules.def", "pseudo_atoms.def"]


def one(m, text):
    return float(re.search(m, text).group(1))


def main(ref):
    src_root = os.path.join(ref, "Examples", "Reference_NIST_SPCE")
    dst_root = os.path.join(HERE, "nist_spce")
    expected = {}
    for n in (1, 2, 3, 4):
        src = os.path.join(src_root, f"Box-{n}")
        dst = os.path.join(dst_root, f"Box-{n}")
        os.makedirs(os.path.join(dst, "RestartInitial", "System_0"), exist_ok=True)
        for f in FILES + [f"Box-{n}.cif"]:
            shutil.copyfile(os.path.join(src, f), os.path.join(dst, f))
        shutil.copyfile(os.path.join(src, "RestartInitial", "System_0", "restartfile"),
                        os.path.join(dst, "RestartInitial", "System_0", "restartfile"))
        text = open(os.path.join(src, "output.txt")).read()
        init = text.split("CALCULATING INITIAL STAGE ENERGY", 1)[1].split("DONE CALCULATING INITIAL STAGE ENERGY", 1)[0]
        expected[f"Box-{n}"] = {
            "gg_vdw": one(r"Guest-Guest VDW: ([-\d.]+);", init),
            "gg_real": one(r"Guest-Guest VDW: [-\d.]+; Real: ([-\d.]+)", init),
            "fourier_gg": one(r"CPU Guest-Guest Fourier: ([-\d.]+)", init),
            "self_atoms": one(r"Component: 1, SelfAtomE: ([-\d.]+)", init),
            "intra_exclusion": one(r"Component: 1, Intra-Molecular ExclusionE: ([-\d.]+)", init),
            "gg_ewald": float(re.findall(r"GGEwaldE: ([-\d.]+)", init)[-1]),
            "tail": float(re.findall(r"TailE: ([-\d.]+)", init)[-1]),
            "molecules": int(re.search(r"Component: 0\s+Adsorbate (\d+) molecules",
                                       open(os.path.join(src, "RestartInitial", "System_0", "restartfile")).read())
                             .group(1)),
        }
        vol = re.search(r"Box Volume:\s+([\d.]+)", text)
        if vol:
            expected[f"Box-{n}"]["volume"] = float(vol.group(1))
    with open(os.path.join(dst_root, "expected.json"), "w") as f:
        json.dump({"source": "Examples/Reference_NIST_SPCE/Box-*/output.txt", "boxes": expected}, f, indent=1)
    print(json.dumps(expected, indent=1))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_nist_spce_inputs.py /path/to/gRASPA")
    main(sys.argv[1])
