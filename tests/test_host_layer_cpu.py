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


def test_philox_slots_distinct():
    """Every named Philox slot of a move is its own counter word: the per-move slots above the
    trial ranges (move, displacement, volume, identity swap, Gibbs transfer) do not collide
    with each other or with the trial, orientation, selection and retrace ranges."""
    import re
    src = open(os.path.join(ROOT, "include", "grx_philox.h")).read()
    slots = {k: int(v) for k, v in re.findall(r"#define (GRX_SLOT_[A-Z]+) (\d+)u", src)}
    singles = [slots[k] for k in ("GRX_SLOT_SELECT", "GRX_SLOT_MOVE", "GRX_SLOT_DISP", "GRX_SLOT_VOLUME",
                                  "GRX_SLOT_SWAP", "GRX_SLOT_GIBBS")]
    assert len(set(singles)) == len(singles)
    ranges = [(slots["GRX_SLOT_FIRST"], 1024), (slots["GRX_SLOT_ORIENT"], 1024), (slots["GRX_SLOT_RETRACE"], 1024)]
    for s in singles[1:]:
        assert all(not (a <= s < a + n) for a, n in ranges)


def test_parse_driver_output_new_records():
    """The driver's transfer, swap and count lines and repeated position blocks parse into
    their records."""
    from graspa_gb300 import system_file
    text = "\n".join([
        "mode swap",
        "swap 0 1 2 3 1 0.5 0.25 1.6 -1.5 0.75",
        "count 1 3 1 0",
        "count 2 5 0 1",
        "transfer 0 1 4 0 2.0 3.0 0.5 8 8",
        "positions 1", "1 2 3",
        "positions 2", "4 5 6", "7 8 9",
        "drift 1e-9"])
    out = system_file.parse_driver_output(text)
    assert out["swap"] == [[1.0, 2.0, 3.0, 1.0, 0.5, 0.25, 1.6, -1.5, 0.75]]
    assert out["count"] == {1: [3, 1, 0], 2: [5, 0, 1]}
    assert out["transfer"][0][:3] == [1.0, 4.0, 0.0]
    assert out["positions"].shape == (1, 3) and len(out["positions_all"]) == 2
    assert out["positions_all"][1].shape == (2, 3) and out["drift"] == 1e-9


def test_co2_n2_mixture_system():
    """The CO2 + N2 silica mixture: neutral, three components in storage order, N2 sites
    typed N_n2, N_n2, N_com, and the framework of the CO2 system unchanged."""
    from graspa_gb300 import synth
    s = synth.silica_co2_n2(n_co2=3, n_n2=2)
    base = synth.silica_co2()
    cs = s["comp_start"]
    assert cs[1] == base["comp_start"][1] and cs[2] - cs[1] == 9 and cs[3] - cs[2] == 6
    assert abs(float(np.sum(s["charge"]))) < 1e-12
    assert s["ntypes"] == 6 and len(s["epsilon"]) == 36 and s["molsize"] == [cs[1], 3, 3]
    assert list(s["type"][cs[2]:cs[2] + 3]) == [4, 4, 5]
    assert np.array_equal(s["pos"][:cs[1]], base["pos"][:cs[1]])
    e = np.asarray(s["epsilon"]).reshape(6, 6)
    assert np.all(e[5] == 0.0) and np.all(e[:, 5] == 0.0)   # the N2 charge site has no LJ


def test_move_probabilities_and_box_streams(tmp_path):
    """Move_Statistics::NormalizeProbabilities keeps the reference's cumulative order
    (translation, rotation, reinsertion, identity swap, swap; data_struct.h:569-608) and box b
    of a multi-box system draws from stream + b * 2^24 (box 0 keeps the stream). A C++ program
    linked against the host layer; no GPU call."""
    B.build()
    host = os.path.join(ROOT, "graspa_gb300", "host")
    src = os.path.join(str(tmp_path), "m.cpp")
    exe = os.path.join(str(tmp_path), "m")
    with open(src, "w") as f:
        f.write('#include <cstdio>\n#include "graspa_host.hpp"\nusing namespace graspa;\nint main() {\n'
                '  Move_Statistics M; M.TranslationProb = 1; M.RotationProb = 1; M.ReinsertionProb = 2;\n'
                '  M.IdentitySwapProb = 2; M.SwapProb = 2; M.NormalizeProbabilities();\n'
                '  std::printf("%.17g %.17g %.17g %.17g %.17g\\n", M.TranslationProb, M.RotationProb, M.ReinsertionProb,\n'
                '              M.IdentitySwapProb, M.SwapProb);\n'
                '  RandomNumber R; R.Stream = 7;\n'
                '  std::printf("%u %u %u\\n", R.BoxStream(0), R.BoxStream(1), R.BoxStream(2));\n  return 0;\n}\n')
    srcs = [os.path.join(host, x) for x in B.HOST_SOURCES]
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I", host, src] + srcs +
                   ["-L", B.OUT, "-lgrx", "-Wl,-rpath," + B.OUT, "-o", exe], check=True)
    lines = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    p = [float(x) for x in lines[0].split()]
    assert np.allclose(p, [0.125, 0.25, 0.5, 0.75, 1.0], rtol=0, atol=1e-15)
    assert [int(x) for x in lines[1].split()] == [7, 7 + (1 << 24), 7 + (2 << 24)]
