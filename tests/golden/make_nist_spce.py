"""Generate the NIST SPC/E known-answer fixtures used to pin the FP64 oracle.

gRASPA's own regression data for the energy path is the NIST SPC/E reference
calculation (Examples/Reference_NIST_SPCE/readme.md:7-17): four triclinic boxes of
rigid SPC/E water, LAMMPS-style Ewald (alpha = 0.285, kmax 7/7/7), 10 A cutoffs.
The per-box output.txt files hold the reference's FP64 totals in internal units
(10 J/mol), e.g. Box-1/output.txt:117 (VDW, real), :123 (Fourier), :125 (self),
:127 (intra exclusion), :131-132 (rigid-molecule exclusion constants), :61 (kmax and
reciprocal cutoff), :109 (volume).

This script reads those inputs (simulation.input, the framework .cif cell, the
RestartInitial coordinates, pseudo_atoms.def charges, force_field_mixing_rules.def
LJ parameters) and the printed totals, and writes one compact JSON per box to
tests/golden/nist_spce_box{N}.json. It runs only where the reference tree is
mounted; the JSON files are committed so nothing at test time reads the reference.

Usage: python tests/golden/make_nist_spce.py /path/to/gRASPA  (the reference checkout; required)
"""
import json
import math
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _kv(path):
    out = {}
    with open(path) as f:
        for line in f:
            t = line.split()
            if len(t) >= 2:
                out.setdefault(t[0], t[1:])
    return out


def _cell_from_cif(path):
    """Cell matrix from lengths/angles, the construction of read_data.cpp:1536-1547."""
    vals = {}
    with open(path) as f:
        for line in f:
            t = line.split()
            if len(t) >= 2 and t[0].startswith("_cell_"):
                vals[t[0]] = float(t[1])
    a, b, c = vals["_cell_length_a"], vals["_cell_length_b"], vals["_cell_length_c"]
    deg = 180.0 / 3.14159265358979323846
    al, be, ga = (vals["_cell_angle_alpha"] / deg, vals["_cell_angle_beta"] / deg,
                  vals["_cell_angle_gamma"] / deg)
    ay = b * math.sin(ga)
    tempd = (math.cos(al) - math.cos(ga) * math.cos(be)) / math.sin(ga)
    az = c * math.sqrt(1 - math.cos(be) ** 2 - tempd ** 2)
    bx = b * math.cos(ga)
    cx = c * math.cos(be)
    cy = c * tempd
    return [a, 0.0, 0.0, bx, ay, 0.0, cx, cy, az]


def _floats(line):
    return [float(x) for x in re.findall(r"[-+]?\d+\.\d+(?:[eE][-+]?\d+)?|[-+]?\d+", line)]


def make_box(ref, n):
    d = os.path.join(ref, "Examples", "Reference_NIST_SPCE", f"Box-{n}")
    sim = _kv(os.path.join(d, "simulation.input"))
    fw = sim["FrameworkName"][0]
    cell = _cell_from_cif(os.path.join(d, fw + ".cif"))

    charges = {}
    with open(os.path.join(d, "pseudo_atoms.def")) as f:
        lines = [l for l in f if l.strip() and not l.startswith("#")]
    for l in lines[1:]:
        t = l.split()
        charges[t[0]] = float(t[6])
    lj = {}
    with open(os.path.join(d, "force_field_mixing_rules.def")) as f:
        for l in f:
            t = l.split()
            if len(t) == 4 and t[1] == "lennard-jones":
                lj[t[0]] = (float(t[2]), float(t[3]))
    names = ["O_spce", "H_spce"]

    pos, types, molid = [], [], []
    with open(os.path.join(d, "RestartInitial", "System_0", "restartfile")) as f:
        for l in f:
            if l.startswith("Adsorbate-atom-position:"):
                t = l.split()
                m, a = int(t[1]), int(t[2])
                pos.append([float(t[3]), float(t[4]), float(t[5])])
                molid.append(m)
                types.append(0 if a == 0 else 1)

    with open(os.path.join(d, "output.txt")) as f:
        out = f.read().splitlines()

    def first(pattern):
        for l in out:
            if pattern in l:
                return l
        raise KeyError(pattern)

    kline = first("kmax:")
    kmax = [int(x) for x in re.findall(r"kmax: (\d+) (\d+) (\d+)", kline)[0]]
    recip = float(re.findall(r"ReciprocalCutOff: ([-\d.]+)", kline)[0])
    vol = _floats(first("Box Volume:"))[0]
    gg = first("Guest-Guest VDW:")
    gg_vdw, gg_real = [float(x) for x in re.findall(r"[-\d.]+\d", gg.split("VDW:")[1])]
    fourier = float(re.findall(r"CPU Guest-Guest Fourier: ([-\d.]+)", first("CPU Guest-Guest Fourier"))[0])
    self_e = float(re.findall(r"SelfAtomE: ([-\d.]+)", first("Component: 1, SelfAtomE"))[0])
    intra_e = float(re.findall(r"ExclusionE: ([-\d.]+)", first("Component: 1, Intra-Molecular ExclusionE"))[0])
    excl_intra = float(re.findall(r"Energy: ([-\d.]+)", first("Component 1, Intra Exclusion Energy"))[0])
    excl_self = float(re.findall(r"Energy: ([-\d.]+)", first("Component 1, Atom Self Exclusion Energy"))[0])

    eps_k, sig = lj["O_spce"]
    return {
        "source": f"Examples/Reference_NIST_SPCE/Box-{n}",
        "cell": cell,
        "cutoff": float(sim["CutOffVDW"][0]),
        "alpha": float(sim["Ewald_Alpha"][0]),
        "kmax": kmax,
        "prefactor": 138935.483496,
        "charges": [charges[nm] for nm in names],
        "type_names": names,
        "lj_eps_K": [eps_k, 0.0],
        "lj_sigma": [sig, 0.0],
        "shifted": False,
        "molsize": 3,
        "pos": pos,
        "type": types,
        "molid": molid,
        "expect": {
            "volume": vol,
            "reciprocal_cutoff": recip,
            "gg_vdw": gg_vdw,
            "gg_real": gg_real,
            "fourier_gg": fourier,
            "self_atoms": self_e,
            "intra_exclusion": intra_e,
            "rigid_exclusion_intra": excl_intra,
            "rigid_exclusion_self": excl_self,
            "decimals": 5,
        },
    }


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_nist_spce.py /path/to/gRASPA")
    ref = sys.argv[1]
    for n in (1, 2, 3, 4):
        box = make_box(ref, n)
        path = os.path.join(HERE, f"nist_spce_box{n}.json")
        with open(path, "w") as f:
            json.dump(box, f, separators=(",", ":"))
        print(path, len(box["pos"]), "atoms")


if __name__ == "__main__":
    main()
