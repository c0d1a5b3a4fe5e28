"""Writer of the plain-text system file read by the C++ host layer's driver
(graspa_gb300/host/gcmc_driver.cpp): one box, its force field, its components
(atoms in storage order; an empty adsorbate component stores its template) and
the move set of one adsorbate component."""
import numpy as np

from . import grx


def _vals(a):
    return " ".join(repr(float(x)) for x in np.asarray(a, dtype=np.float64).reshape(-1))


def write_system(path, system, capacity, desc, precision=grx.GRX_FP64, first_step=0, temperature=None):
    """system: the system dict of graspa_gb300.synth; capacity: atoms per component;
    desc: a grx.GcmcDesc (component, trials, cumulative probabilities, state)."""
    g = grx.geometry_from_system(system)
    cs = system["comp_start"]
    ncomp = len(cs) - 1
    nt = int(system["ntypes"])
    L = []
    L.append("cell " + _vals(list(g.cell)))
    L.append("inverse_cell " + _vals(list(g.inverse_cell)))
    L.append(f"volume {float(g.volume)!r}")
    L.append(f"cubic {int(g.cubic)}")
    L.append(f"lammps_ewald {int(g.use_lammps_ewald)}")
    L.append(f"kmax {g.kmax[0]} {g.kmax[1]} {g.kmax[2]}")
    L.append(f"alpha {g.alpha!r}")
    L.append(f"prefactor {g.prefactor!r}")
    L.append(f"reciprocal_cutoff {g.reciprocal_cutoff!r}")
    L.append(f"ntypes {nt}")
    L.append("epsilon " + _vals(system["epsilon"]))
    L.append("sigma " + _vals(system["sigma"]))
    L.append("shift " + _vals(system["shift"]))
    L.append(f"cutoff_vdw_sq {float(system['cutoff_vdw']) ** 2!r}")
    L.append(f"cutoff_coul_sq {float(system['cutoff_coul']) ** 2!r}")
    L.append(f"overlap {float(system.get('overlap_criteria', 1e6))!r}")
    L.append(f"no_charges {int(system.get('no_charges', 0))}")
    L.append(f"vdw_real_bias {int(system.get('vdw_real_bias', 1))}")
    L.append(f"ncomp {ncomp}")
    L.append(f"nhost {int(system['nhost'])}")
    P = np.asarray(system["pos"], dtype=np.float64).reshape(-1, 3)
    for c in range(ncomp):
        a0, a1 = cs[c], cs[c + 1]
        ms = int(system["molsize"][c])
        n = a1 - a0
        if n == 0 and c >= int(system["nhost"]):
            tm = system["templates"][c]
            pos, q, ty, mol = np.asarray(tm["pos"]).reshape(-1, 3), tm["charge"], tm["type"], np.zeros(ms, int)
        else:
            pos = P[a0:a1]
            q = np.asarray(system["charge"])[a0:a1]
            ty = np.asarray(system["type"])[a0:a1]
            mol = np.asarray(system["molid"])[a0:a1]
        L.append(f"component {c} molsize {ms} capacity {int(max(capacity[c], len(q)))} size {n} "
                 f"stored {len(q)} rigid {1 if c >= int(system['nhost']) else 0}")
        for i in range(len(q)):
            x, y, z = (float(v) for v in pos[i])
            L.append(f"{x!r} {y!r} {z!r} {float(q[i])!r} {int(ty[i])} {int(mol[i])}")
    T = temperature if temperature is not None else system.get("temperature", 300.0)
    L.append(f"component_moved {desc.component}")
    L.append(f"beta {desc.beta!r}")
    L.append(f"temperature {float(T)!r}")
    L.append(f"pressure {desc.pressure!r}")
    L.append(f"fugacity_coeff {desc.fugacity_coeff!r}")
    L.append(f"mol_fraction {desc.mol_fraction!r}")
    L.append(f"ideal_rosenbluth {desc.ideal_rosenbluth!r}")
    L.append(f"tail_insert {desc.tail_insert!r}")
    L.append(f"ntrials {desc.ntrials}")
    L.append(f"norient {desc.norient}")
    L.append(f"cumulative_probabilities {desc.p_translation!r} {desc.p_rotation!r} {desc.p_reinsertion!r} "
             f"{desc.p_swap!r}")
    L.append("max_translation " + _vals(list(desc.max_translation)))
    L.append("max_rotation " + _vals(list(desc.max_rotation)))
    L.append(f"seed {desc.seed}")
    L.append(f"stream {desc.stream}")
    L.append(f"first_step {first_step}")
    L.append(f"precision {precision}")
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


def parse_driver_output(text):
    """Parse the driver's stdout into a dict (lists for the count lines, positions array)."""
    out = {"W": []}
    lines = text.strip().splitlines()
    i = 0
    while i < len(lines):
        parts = lines[i].split()
        k = parts[0]
        if k in ("attempts", "accepted"):
            out[k] = [int(x) for x in parts[1:]]
        elif k == "W":
            out["W"].append(float(parts[2]))
        elif k == "gibbs":  # move, volume of box 0, volume of box 1
            out.setdefault("gibbs", []).append([float(x) for x in parts[2:]])
        elif k == "volume":  # move, accepted, trial volume, trial total, overlap, total before
            out.setdefault("volume", []).append([float(x) for x in parts[2:]])
        elif k == "lambda":  # step, constructed, HGVDW HGReal GGVDW GGReal GGEwald HGEwald Tail total
            out.setdefault("lambda", []).append([float(x) for x in parts[2:]])
        elif k == "transfer":  # move, insertion box, deleted molecule, accepted, W_ins, W_del, Pacc, N0, N1
            out.setdefault("transfer", []).append([float(x) for x in parts[2:]])
        elif k == "swap":  # move, old comp, new comp, old molecule, accepted, W_new, W_old, Pacc, GGEwald, HGEwald
            out.setdefault("swap", []).append([float(x) for x in parts[2:]])
        elif k == "count":  # component: molecules, identity swaps in, identity swaps out
            out.setdefault("count", {})[int(parts[1])] = [int(x) for x in parts[2:]]
        elif k == "positions":  # one block per printed component; "positions" is the first
            n = int(parts[1])
            p = np.array([[float(x) for x in lines[i + 1 + j].split()] for j in range(n)]).reshape(-1, 3)
            out.setdefault("positions", p)
            out.setdefault("positions_all", []).append(p)
            i += n
        elif k == "mode":
            out["mode"] = parts[1]
        else:
            out[k] = float(parts[1])
        i += 1
    return out
