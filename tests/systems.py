"""System builders shared by the tests (NIST SPC/E fixtures, synthetic CO2/silica)."""
import json
import os

import numpy as np

from graspa_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def nist_system(n):
    """NIST SPC/E box n as a system dict: one empty host component, 3-site water."""
    b = json.load(open(os.path.join(GOLDEN, f"nist_spce_box{n}.json")))
    N = len(b["pos"])
    eps, sig, sh = synth.mix_lorentz_berthelot(b["lj_eps_K"], b["lj_sigma"], [0, 0], b["cutoff"])
    q = np.array([b["charges"][t] for t in b["type"]])
    s = dict(name=f"nist_spce_box{n}", cell=b["cell"], kmax=b["kmax"], alpha=b["alpha"], use_lammps_ewald=1,
             prefactor=b["prefactor"], ntypes=2, epsilon=eps, sigma=sig, shift=sh, cutoff_vdw=b["cutoff"],
             cutoff_coul=b["cutoff"], overlap_criteria=1e6, no_charges=0, vdw_real_bias=1, nhost=1,
             comp_start=[0, 0, N], pos=np.array(b["pos"]), scale=np.ones(N), charge=q, scale_coul=np.ones(N),
             type=np.array(b["type"]), molid=np.array(b["molid"]), molsize=[1, 3], temperature=300.0,
             templates={1: dict(pos=np.array(b["pos"][:3]), charge=q[:3], type=np.array(b["type"][:3]))})
    return s, b["expect"]


def co2_system(n_co2=0, seed=42):
    return synth.silica_co2(seed=seed, n_co2=n_co2)
