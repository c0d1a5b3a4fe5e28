"""The C-ABI library builds, loads without a GPU and exports every function that
include/grx.h declares (no compute call is made here)."""
import ctypes
import os
import re

from graspa_gb300 import build as B
from graspa_gb300 import grx

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "grx.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(grx_[a-z_0-9]+)\s*\(", src, flags=re.M)))


def test_header_lists_match_binding():
    assert set(declared_functions()) == set(grx.EXPORTS)


def test_library_exports_every_symbol():
    path = B.build()
    lib = ctypes.CDLL(path)
    missing = [f for f in declared_functions() if not hasattr(lib, f)]
    assert not missing, missing


def test_status_strings_without_gpu():
    L = grx.load()
    assert L.grx_status_string(0) == b"ok"
    assert L.grx_status_string(4) == b"device wait timed out"


def test_box_create_rejects_bad_desc():
    L = grx.load()
    d = grx.BoxDesc()
    d.ncomponents = 0
    h = ctypes.c_void_p()
    assert L.grx_box_create(ctypes.byref(d), ctypes.byref(h)) == 1
    assert b"ncomponents" in L.grx_last_error()


# ctypes mirror -> C typedef of include/grx.h
STRUCTS = {"BoxGeometry": "grx_box_geometry", "ForceField": "grx_forcefield", "BoxDesc": "grx_box_desc",
           "Atoms": "grx_atoms", "Trials": "grx_trials", "TrialEnergy": "grx_trial_energy", "Energy": "grx_energy",
           "WidomDesc": "grx_widom_desc", "WidomResult": "grx_widom_result", "GcmcDesc": "grx_gcmc_desc",
           "GcmcStats": "grx_gcmc_stats", "ServerConfig": "grx_server_config", "JobDesc": "grx_job_desc",
           "JobResult": "grx_job_result"}


ORACLE_STRUCTS = {"OraBox": "ora_box", "OraFF": "ora_ff", "OraAtoms": "ora_atoms", "OraTrials": "ora_trials",
                  "OraWidom": "ora_widom", "OraWidomResult": "ora_widom_result", "OraGcmc": "ora_gcmc",
                  "OraGcmcStats": "ora_gcmc_stats"}


def _check_layouts(tmp_path, module, structs, header, incdir):
    """Compiles a C program against `header` that prints every struct's size and field
    offsets, and compares them with the ctypes mirrors in `module`."""
    import subprocess
    lines = ["#include <stddef.h>", "#include <stdio.h>", f'#include "{header}"', "int main(void) {"]
    for py, c in structs.items():
        cls = getattr(module, py)
        lines.append(f'  printf("{py} __sizeof__ %zu\\n", sizeof({c}));')
        for name, _ in cls._fields_:
            lines.append(f'  printf("{py} {name} %zu\\n", offsetof({c}, {name}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", incdir, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    c_layout = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l}
    for py in structs:
        cls = getattr(module, py)
        assert ctypes.sizeof(cls) == c_layout[(py, "__sizeof__")], py
        for name, _ in cls._fields_:
            assert getattr(cls, name).offset == c_layout[(py, name)], (py, name)


def test_struct_layouts_match_header(tmp_path):
    """Every ctypes mirror of a grx.h struct has the C size and field offsets (no GPU involved)."""
    _check_layouts(tmp_path, grx, STRUCTS, "grx.h", os.path.join(ROOT, "include"))


def test_oracle_struct_layouts_match_header(tmp_path):
    """The same for the oracle's ctypes mirrors of grx_oracle.h."""
    from oracle import oracle as O
    _check_layouts(tmp_path, O, ORACLE_STRUCTS, "grx_oracle.h", os.path.join(ROOT, "oracle"))
