"""CPU checks of the C++ host layer: it builds, its driver reports its usage
without touching a GPU, and the host Philox header draws the oracle's numbers."""
import os
import subprocess

import numpy as np

from graspa_gb300 import build as B
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_driver_builds_and_prints_usage():
    B.build()
    assert os.path.exists(B.DRIVER)
    r = subprocess.run([B.DRIVER], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


def test_philox_header_matches_oracle(tmp_path):
    src = os.path.join(str(tmp_path), "p.c")
    exe = os.path.join(str(tmp_path), "p")
    with open(src, "w") as f:
        f.write('#include <stdio.h>\n#include "grx_philox.h"\nint main(void){uint32_t o[4];\n'
                'for (unsigned s = 0; s < 5000; s += 997) { grx_draw(42ull + s, s % 7, 123456789012ull * s, s, o);\n'
                'printf("%u %u %u %u %.17g\\n", o[0], o[1], o[2], o[3], grx_u01(o[3])); }\nreturn 0;}\n')
    subprocess.run(["gcc", "-O2", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    for k, s in enumerate(range(0, 5000, 997)):
        ref = O.draw(42 + s, s % 7, 123456789012 * s, s)
        got = out[k].split()
        assert [int(x) for x in got[:4]] == list(ref)
        assert float(got[4]) == ref[3] * 2.0 ** -32


def test_driver_reads_system_file(tmp_path):
    """The writer and the C++ reader agree on the format: the driver parses the whole
    file and stops only where it needs a device (or runs zero steps on a GPU host)."""
    from graspa_gb300 import grx, synth, system_file
    B.build()
    s = synth.silica_co2(n_co2=2)
    d = grx.gcmc_desc(1, p_reinsertion=0.75)
    f = os.path.join(str(tmp_path), "system.txt")
    system_file.write_system(f, s, [s["comp_start"][1], 30], d)
    r = subprocess.run([B.DRIVER, f, "host", "0"], capture_output=True, text=True)
    assert (r.returncode == 1 and "grx_box_create" in r.stderr) or (r.returncode == 0 and "attempts" in r.stdout)
