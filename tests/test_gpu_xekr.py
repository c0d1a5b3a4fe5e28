"""Statistical parity with a published reference run: gRASPA's Examples/XeKr-Mixture
(Kr/Xe 0.1/0.9 at 1e5 Pa and 273 K in the 25.cif MOF, LJ only, translation, Kr
reinsertion, identity swaps and CBMC insertion / deletion with 10 trial positions),
through graspa_run --replicas on the GPU, in the mixed and the FP64 forms.

The reference printed (output_1e5.txt, 1e5 initialization and 1e6 production steps in 5
blocks, committed as tests/golden/xekr/expected.json) the loadings of both components
and the Widom statistics of the Kr insertions (<W>, mu_ex, Henry coefficient). Its
"ErrorBar" is twice the population standard deviation of the 5 block averages, so the
standard error of its mean is ErrorBar / 2 / sqrt(4). This engine runs many
independent replicas (one persistent launch, Philox streams) and reports the mean over
replicas with its standard error. A quantity passes when the two means differ by less
than 3 combined standard errors. The fugacity coefficients come from this engine's own
Peng-Robinson mixture (pinned to the printed values in tests/test_xekr_input.py)."""
import json
import math
import os
import re
import subprocess

import pytest

from graspa_gb300 import build as B

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "xekr")
REPLICAS = 456
INIT_STEPS = 20000
PROD_STEPS = 40000


def ref_sem(errorbar_2sigma, nblocks=5):
    return errorbar_2sigma / 2.0 / math.sqrt(nblocks - 1)


def run(prec):
    B.build()
    r = subprocess.run([B.RUNNER, FIX, "--replicas", str(REPLICAS), "--init-steps", str(INIT_STEPS), "--prod-steps",
                        str(PROD_STEPS), "--precision", prec], capture_output=True, text=True, timeout=1500)
    assert r.returncode == 0, r.stderr
    return r.stdout


def parse(out, name):
    m = re.search(rf"\[{name}\] loading (\S+) \+/- (\S+) molecules, (\S+) \+/- (\S+) mol/kg", out)
    w = re.search(rf"\[{name}\] widom <W> (\S+) \+/- (\S+) mu_ex (\S+) \+/- (\S+) K henry (\S+) \+/- (\S+)", out)
    return {"n": float(m.group(1)), "n_err": float(m.group(2)), "molkg": float(m.group(3)),
            "molkg_err": float(m.group(4)), "w": float(w.group(1)), "w_err": float(w.group(2)),
            "mu": float(w.group(3)), "mu_err": float(w.group(4)), "henry": float(w.group(5)),
            "henry_err": float(w.group(6))}


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_xekr_loadings_and_widom_match_published_run(prec):
    e = json.load(open(os.path.join(FIX, "expected.json")))
    out = run(prec)
    print(out)
    rows = []
    for name in ("Kr", "Xe"):
        g = parse(out, name)
        for key, ours, err, ref in (
                ("molecules", g["n"], g["n_err"], e["loading_molecules"][name]),
                ("mol/kg", g["molkg"], g["molkg_err"], e["loading_mol_per_kg"][name])):
            sig = math.hypot(err, ref_sem(ref["errorbar_2sigma"]))
            rows.append((name, key, ours, ref["average"], sig))
        if name == "Kr":
            wr, wr2 = e["widom_kr"]["rosenbluth"]
            rows.append((name, "<W>", g["w"], wr, math.hypot(g["w_err"], ref_sem(wr2))))
            hr, hr2 = e["widom_kr"]["henry_mol_kg_pa"]
            rows.append((name, "henry", g["henry"], hr, math.hypot(g["henry_err"], ref_sem(hr2))))
            mr, mr2 = e["widom_kr"]["mu_ex_K"]
            rows.append((name, "mu_ex", g["mu"], mr, math.hypot(g["mu_err"], ref_sem(mr2))))
    for name, key, ours, ref, sig in rows:
        print(f"{prec} {name} {key}: {ours:.6g} vs published {ref:.6g} ({(ours - ref) / sig:+.2f} sigma)")
    bad = [r for r in rows if abs(r[2] - r[3]) > 3.0 * r[4]]
    assert not bad, bad
    drift = float(re.search(r"ENERGY DRIFT (\S+)", out).group(1))
    assert abs(drift) < 1e-3 * max(1.0, abs(float(re.search(r"recomputed (\S+),", out).group(1))))
