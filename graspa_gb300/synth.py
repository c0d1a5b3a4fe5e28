"""Seeded synthetic systems for the benchmark configurations.

No dataset is involved: each generator builds the framework, force field and
adsorbate templates from the stated sizes and distributions with a seeded
Philox bit generator (numpy.random.Philox), so the same seed gives the same
system on every machine.

A system is a plain dict (the layout the C-ABI wrapper and the test oracle both
read):
  cell[9]            column-major cell matrix (gRASPA Boxsize.Cell layout)
  kmax[3], alpha     Ewald parameters (LAMMPS-style explicit alpha/kmax)
  ntypes, type_names, epsilon/sigma/shift (ntypes^2, internal units, mixed)
  cutoff_vdw, cutoff_coul  (Angstrom, not squared)
  nhost              number of host (framework) components
  comp_start         component offsets into the atom arrays
  pos (N,3), scale, charge, scale_coul, type, molid   per atom
  molsize            atoms per molecule for every component
  templates          {component: dict(pos, charge, type)} molecule definitions
"""
import math

import numpy as np

K_PER_INTERNAL = 1.20272430057   # energy unit conversion used for epsilon (K -> 10 J/mol)
COULOMB_PREFACTOR = 138935.483496


def _rng(seed):
    return np.random.Generator(np.random.Philox(seed))


def mix_lorentz_berthelot(eps_K, sigma, shifted, cutoff):
    """Lorentz-Berthelot mixing with optional cutoff shift (gRASPA read_data.cpp
    Mixing_Rule_Epsilon / Mixing_rule_Sigma / Get_Shifted_Value)."""
    n = len(eps_K)
    eps = np.zeros(n * n)
    sig = np.zeros(n * n)
    shift = np.zeros(n * n)
    rc2 = cutoff * cutoff
    for i in range(n):
        for j in range(n):
            ep = math.sqrt(eps_K[i] * eps_K[j]) / K_PER_INTERNAL
            sg = 0.5 * (sigma[i] + sigma[j])
            eps[i * n + j] = ep
            sig[i * n + j] = sg
            if shifted[i] and shifted[j] and ep > 0.0 and sg > 0.0:
                t = rc2 / (sg * sg)
                rri3 = 1.0 / (t * t * t)
                shift[i * n + j] = 4.0 * ep * (rri3 * (rri3 - 1.0))
    return eps, sig, shift


def orthorhombic_cell(a, b, c):
    return [a, 0.0, 0.0, 0.0, b, 0.0, 0.0, 0.0, c]


def triclinic_cell(a, b, c, alpha_deg, beta_deg, gamma_deg):
    """Cell matrix from lengths and angles (gRASPA read_data.cpp:1536-1547 layout)."""
    deg = 180.0 / 3.14159265358979323846
    al, be, ga = alpha_deg / deg, beta_deg / deg, gamma_deg / deg
    ay = b * math.sin(ga)
    tempd = (math.cos(al) - math.cos(ga) * math.cos(be)) / math.sin(ga)
    az = c * math.sqrt(max(1 - math.cos(be) ** 2 - tempd ** 2, 1e-12))
    return [a, 0.0, 0.0, b * math.cos(ga), ay, 0.0, c * math.cos(be), c * tempd, az]


def perpendicular_widths(cell):
    h = np.array(cell, dtype=np.float64).reshape(3, 3).T   # columns a, b, c
    vol = abs(np.linalg.det(h))
    a, b, c = h[:, 0], h[:, 1], h[:, 2]
    return np.array([vol / np.linalg.norm(np.cross(b, c)), vol / np.linalg.norm(np.cross(c, a)),
                     vol / np.linalg.norm(np.cross(a, b))])


def co2_template():
    """Rigid linear CO2, C first then the two O at +/-1.16 A (the bead order of
    gRASPA's Examples/Henrys_coefficient/CO2.def)."""
    return dict(pos=np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 1.16], [0.0, 0.0, -1.16]]),
                charge=np.array([0.70, -0.35, -0.35]), names=["C_co2", "O_co2", "O_co2"])


SILICA_CO2_TYPES = [("Si", 22.0, 2.30), ("O", 53.0, 3.30), ("C_co2", 27.0, 2.80), ("O_co2", 79.0, 3.05)]


def silica_co2(seed=42, cells=(2, 2, 3), cutoff=12.0, alpha=0.265, kmax=(9, 9, 6), n_co2=0):
    """Widom / GCMC system of the CO2 + synthetic all-silica configuration.

    Framework: cells of 20.09 x 19.74 x 13.14 A, 96 Si + 192 O per cell. Si sit on a
    jittered lattice (+/-0.1 A): per cell a 6 x 6 x 4 grid of sites (3.35 x 3.29 x
    3.29 A spacing) whose two middle planes along a (i = 2, 3) are left empty, so
    4 x 6 x 4 = 96 sites remain and every cell carries one 10 A slit pore between
    silica walls. Every Si bonds to its +b and +c neighbours (2 bonds per Si, 192
    per cell); each bond carries one O at its midpoint (Si-O 1.65 A) jittered by
    +/-0.1 A. Charges Si +2.05, O -1.025 (neutral). LJ: Si 22 K / 2.30 A, O 53 K /
    3.30 A; CO2 C 27 K / 2.80 A, q +0.70, O 79 K / 3.05 A, q -0.35;
    Lorentz-Berthelot, shifted at the cutoff.
    """
    g = _rng(seed)
    ca, cb, cc = 20.09, 19.74, 13.14
    na, nb, nc = cells
    A, B, Cc = ca * na, cb * nb, cc * nc
    keep_i = [0, 1, 4, 5]
    gy, gz = 6 * nb, 4 * nc
    L = np.array([A, B, Cc])
    si = {}
    for ci in range(na):
        for ii in keep_i:
            for j in range(gy):
                for k in range(gz):
                    si[(ci, ii, j, k)] = np.array([(ci * 6 + ii + 0.5) * ca / 6,
                                                   (j + 0.5) * B / gy, (k + 0.5) * Cc / gz])
    keys = sorted(si)
    jit = g.uniform(-0.1, 0.1, size=(len(keys), 3))
    for n, key in enumerate(keys):
        si[key] = si[key] + jit[n]
    oxy = []
    for (ci, ii, j, k) in keys:
        p = si[(ci, ii, j, k)]
        for q in (si[(ci, ii, (j + 1) % gy, k)], si[(ci, ii, j, (k + 1) % gz)]):
            d = q - p
            d -= L * np.round(d / L)
            oxy.append(p + 0.5 * d)
    oxy = np.array(oxy) + g.uniform(-0.1, 0.1, size=(len(oxy), 3))
    si = np.array([si[k] for k in keys])
    fw = np.concatenate([si, oxy])
    fw = fw - L * np.floor(fw / L)
    nsi, no = len(si), len(oxy)
    names = [n for n, _, _ in SILICA_CO2_TYPES]
    eps_K = [e for _, e, _ in SILICA_CO2_TYPES]
    sig = [x for _, _, x in SILICA_CO2_TYPES]
    eps, sg, shift = mix_lorentz_berthelot(eps_K, sig, [1] * len(eps_K), cutoff)
    fw_type = np.array([0] * nsi + [1] * no)
    fw_q = np.array([2.05] * nsi + [-1.025] * no)
    tmpl = co2_template()
    tmpl["type"] = np.array([2, 3, 3])
    system = dict(
        name="co2_silica", cell=orthorhombic_cell(A, B, Cc), kmax=list(kmax), alpha=alpha,
        use_lammps_ewald=1, prefactor=COULOMB_PREFACTOR, ntypes=4, type_names=names,
        epsilon=eps, sigma=sg, shift=shift, cutoff_vdw=cutoff, cutoff_coul=cutoff,
        overlap_criteria=1e6, no_charges=0, vdw_real_bias=1, temperature=300.0, nhost=1,
        molsize=[len(fw), 3], templates={1: tmpl})
    _set_atoms(system, fw, fw_type, fw_q, [np.zeros((0, 3))])
    if n_co2:
        place_molecules(system, 1, n_co2, g)
    return system


def silica_co2_n2(seed=42, n_co2=0, n_n2=0):
    """The CO2 + silica system of silica_co2 with a second charged, rigid adsorbate: N2
    (two N sites, 36 K / 3.31 A, q -0.482 at +/-0.55 A, and a charge-only centre +0.964;
    the first N is the CBMC first bead). Components: 0 framework, 1 CO2, 2 N2."""
    s = silica_co2(seed=seed)
    nfw = s["comp_start"][1]
    sites = SPECIES["N2"]
    types = SILICA_CO2_TYPES + [("N_n2", 36.0, 3.31), ("N_com", 0.0, 1.0)]
    eps, sg, shift = mix_lorentz_berthelot([e for _, e, _ in types], [x for _, _, x in types], [1] * len(types),
                                           s["cutoff_vdw"])
    s.update(name="co2_n2_silica", ntypes=len(types), type_names=[n for n, _, _ in types], epsilon=eps, sigma=sg,
             shift=shift, molsize=[nfw, 3, 3])
    s["templates"][2] = dict(pos=np.array([p for (_, _, _, _, p) in sites]),
                             charge=np.array([q for (_, _, _, q, _) in sites]), type=np.array([4, 4, 5]))
    _set_atoms(s, s["pos"][:nfw], s["type"][:nfw], s["charge"][:nfw], [np.zeros((0, 3)), np.zeros((0, 3))])
    g = _rng(seed + 104729)
    if n_co2:
        place_molecules(s, 1, n_co2, g)
    if n_n2:
        place_molecules(s, 2, n_n2, g)
    return s


def _set_atoms(system, fw_pos, fw_type, fw_q, guest_pos_list):
    """Concatenate framework + guest components into the per-atom arrays."""
    pos = [np.asarray(fw_pos, dtype=np.float64)]
    typ = [np.asarray(fw_type, dtype=np.int64)]
    q = [np.asarray(fw_q, dtype=np.float64)]
    molid = [np.zeros(len(fw_pos), dtype=np.int64)]
    comp_start = [0, len(fw_pos)]
    for c, gp in enumerate(guest_pos_list, start=1):
        tm = system["templates"][c]
        ms = len(tm["charge"])
        gp = np.asarray(gp, dtype=np.float64).reshape(-1, 3)
        nmol = len(gp) // ms
        pos.append(gp)
        typ.append(np.tile(tm["type"], nmol))
        q.append(np.tile(tm["charge"], nmol))
        molid.append(np.repeat(np.arange(nmol, dtype=np.int64), ms))
        comp_start.append(comp_start[-1] + len(gp))
    system["pos"] = np.concatenate(pos)
    system["type"] = np.concatenate(typ)
    system["charge"] = np.concatenate(q)
    system["molid"] = np.concatenate(molid)
    n = len(system["pos"])
    system["scale"] = np.ones(n)
    system["scale_coul"] = np.ones(n)
    system["comp_start"] = comp_start


def guest_positions(system, comp):
    s, e = system["comp_start"][comp], system["comp_start"][comp + 1]
    return system["pos"][s:e]


def place_molecules(system, comp, n, g, min_dist=2.6, max_tries=200000):
    """Place n rigid molecules of component `comp` at random positions/orientations
    that keep every atom `min_dist` from framework and other guest atoms."""
    tm = system["templates"][comp]
    cell = np.array(system["cell"]).reshape(3, 3).T
    inv = np.linalg.inv(cell)
    fw = system["pos"][: system["comp_start"][system["nhost"]]]
    placed = [guest_positions(system, c) for c in range(1, len(system["comp_start"]) - 1)]
    new = []
    tries = 0
    while len(new) < n and tries < max_tries:
        tries += 1
        com = cell @ g.uniform(0, 1, 3)
        q = g.normal(size=4)
        q /= np.linalg.norm(q)
        w, x, y, z = q
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                      [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                      [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
        mol = (tm["pos"] - tm["pos"][0]) @ R.T + com
        others = [fw] + [p for p in placed if len(p)] + ([np.concatenate(new)] if new else [])
        allp = np.concatenate(others) if others else np.zeros((0, 3))
        ok = True
        for a in mol:
            d = allp - a
            s = d @ inv.T
            s -= np.round(s)
            d = s @ cell.T
            if len(d) and np.min(np.einsum("ij,ij->i", d, d)) < min_dist * min_dist:
                ok = False
                break
        if ok:
            new.append(mol)
    guests = []
    for c in range(1, len(system["comp_start"]) - 1):
        gp = guest_positions(system, c)
        if c == comp and new:
            gp = np.concatenate([gp] + new)
        guests.append(gp)
    fw_type = system["type"][: len(fw)]
    fw_q = system["charge"][: len(fw)]
    _set_atoms(system, fw, fw_type, fw_q, guests)
    return len(new)


# ------------------------------------------------------------------ batched CH4 / Xe
CH4_EPS_K, CH4_SIGMA = 148.0, 3.73
XE_EPS_K, XE_SIGMA = 221.0, 4.10


def _random_cell(g, edge=(10.0, 40.0), angle=(60.0, 120.0)):
    """Cell edges U[edge], angles U[angle] degrees; redrawn until the metric is valid
    (positive volume, no near-degenerate cell)."""
    while True:
        a, b, c = g.uniform(*edge, 3)
        al, be, ga = g.uniform(*angle, 3)
        ca, cb, cg = (math.cos(math.radians(x)) for x in (al, be, ga))
        v2 = 1 - ca * ca - cb * cb - cg * cg + 2 * ca * cb * cg
        if v2 > 0.15:
            return triclinic_cell(a, b, c, al, be, ga)


def lj_framework(seed, cutoff=12.0, n_atoms=None, n_types=3, rho_max=0.03):
    """Seeded LJ-only framework of the batched benchmark: a triclinic cell (edges
    10-40 A, angles 60-120 deg), N atoms log-uniform in [500, 8000]. The cell is
    replicated until every perpendicular width exceeds 2 x cutoff (and the density
    is at most rho_max atoms/A^3). The base cell holds N / replicas atoms on a
    jittered fractional lattice (random vacancies, +/-0.15 lattice spacing), with
    n_types types of eps/k U[20, 90] K and sigma U[2.5, 3.5] A.
    Returns (cell, positions, types, eps_K, sigma)."""
    g = _rng(seed)
    base = np.array(_random_cell(g)).reshape(3, 3).T
    n_target = int(round(math.exp(g.uniform(math.log(500), math.log(8000))))) if n_atoms is None else n_atoms
    w = perpendicular_widths(base.T.reshape(-1))
    reps = np.maximum(1, np.ceil(2.0 * cutoff * 1.0001 / w)).astype(int)
    vol = abs(np.linalg.det(base))
    while n_target / (vol * reps.prod()) > rho_max:
        reps[np.argmin(w * reps)] += 1
    n_base = max(1, int(round(n_target / reps.prod())))
    # lattice with >= n_base sites, spacing roughly equal along the three widths
    f = (n_base / (w[0] * w[1] * w[2])) ** (1.0 / 3.0)
    grid = np.maximum(1, np.ceil(w * f)).astype(int)
    while grid.prod() < n_base:
        grid[np.argmin(grid / w)] += 1
    idx = np.stack(np.meshgrid(*[np.arange(k) for k in grid], indexing="ij"), -1).reshape(-1, 3)
    idx = idx[g.choice(len(idx), n_base, replace=False)]
    frac = (idx + 0.5 + g.uniform(-0.15, 0.15, (n_base, 3))) / grid
    pts = frac @ base.T
    types = g.integers(0, n_types, n_base)
    eps_K = g.uniform(20.0, 90.0, n_types)
    sig = g.uniform(2.5, 3.5, n_types)
    shifts = np.stack(np.meshgrid(*[np.arange(k) for k in reps], indexing="ij"), -1).reshape(-1, 3)
    allp = (pts[None, :, :] + (shifts @ base.T)[:, None, :]).reshape(-1, 3)
    allt = np.tile(types, len(shifts))
    cell = base * reps[None, :]
    return cell.T.reshape(-1).tolist(), allp, allt, list(eps_K), list(sig)


def ch4_xe_system(seed, cutoff=12.0, n_atoms=None, n_ch4=0, n_xe=0):
    """One box of the batched CH4 / Xe benchmark on lj_framework(seed): united-atom
    CH4 (148 K, 3.73 A) and Xe (221 K, 4.10 A), no charges, Lorentz-Berthelot mixing
    shifted at the cutoff. Components: 0 framework, 1 CH4, 2 Xe (one bead each)."""
    cell, fw, ft, eps_fw, sig_fw = lj_framework(seed, cutoff=cutoff, n_atoms=n_atoms)
    nt = len(eps_fw)
    eps_K = eps_fw + [CH4_EPS_K, XE_EPS_K]
    sig = sig_fw + [CH4_SIGMA, XE_SIGMA]
    eps, sg, shift = mix_lorentz_berthelot(eps_K, sig, [1] * (nt + 2), cutoff)
    h = np.array(cell).reshape(3, 3).T
    off = abs(h[0, 1]) + abs(h[0, 2]) + abs(h[1, 2]) + abs(h[1, 0]) + abs(h[2, 0]) + abs(h[2, 1])
    templates = {1: dict(pos=np.zeros((1, 3)), charge=np.zeros(1), type=np.array([nt])),
                 2: dict(pos=np.zeros((1, 3)), charge=np.zeros(1), type=np.array([nt + 1]))}
    system = dict(
        name=f"ch4_xe_{seed}", cell=cell, kmax=[1, 1, 1], alpha=0.265, use_lammps_ewald=int(off == 0.0),
        prefactor=COULOMB_PREFACTOR, ntypes=nt + 2, epsilon=eps, sigma=sg, shift=shift, cutoff_vdw=cutoff,
        cutoff_coul=cutoff, overlap_criteria=1e6, no_charges=1, vdw_real_bias=1, temperature=300.0, nhost=1,
        molsize=[len(fw), 1, 1], templates=templates)
    _set_atoms(system, fw, ft, np.zeros(len(fw)), [np.zeros((0, 3)), np.zeros((0, 3))])
    gg = _rng(seed + 1000003)
    if n_ch4:
        place_molecules(system, 1, n_ch4, gg, min_dist=2.8)
    if n_xe:
        place_molecules(system, 2, n_xe, gg, min_dist=2.8)
    return system


# ------------------------------------------------------------------ serving jobs
KR_EPS_K, KR_SIGMA = 166.0, 3.64

SPECIES = {
    # name: list of (site, eps_K, sigma, charge, position); the first site is the CBMC first bead
    "CH4": [("CH4", CH4_EPS_K, CH4_SIGMA, 0.0, (0.0, 0.0, 0.0))],
    "Xe": [("Xe", XE_EPS_K, XE_SIGMA, 0.0, (0.0, 0.0, 0.0))],
    "Kr": [("Kr", KR_EPS_K, KR_SIGMA, 0.0, (0.0, 0.0, 0.0))],
    "CO2": [("C_co2", 27.0, 2.80, 0.70, (0.0, 0.0, 0.0)), ("O_co2", 79.0, 3.05, -0.35, (0.0, 0.0, 1.16)),
            ("O_co2", 79.0, 3.05, -0.35, (0.0, 0.0, -1.16))],
    "N2": [("N_n2", 36.0, 3.31, -0.482, (0.0, 0.0, -0.55)), ("N_n2", 36.0, 3.31, -0.482, (0.0, 0.0, 0.55)),
           ("N_com", 0.0, 1.0, 0.964, (0.0, 0.0, 0.0))],   # charge site only (eps 0)
}


def raspa_ewald(cell, cutoff, precision=1e-6):
    """Alpha, kmax and reciprocal cutoff from the Ewald precision, the automatic
    set-up of read_Ewald_Parameters_from_input (read_data.cpp:689-700)."""
    tol = math.sqrt(abs(math.log(precision * cutoff)))
    alpha = math.sqrt(abs(math.log(precision * cutoff * tol))) / cutoff
    tol1 = math.sqrt(-math.log(precision * cutoff * (2.0 * tol * alpha) ** 2))
    kmax = [int(round(0.25 + cell[k] * alpha * tol1 / math.pi)) for k in (0, 4, 8)]
    return alpha, kmax, (1.05 * max(kmax)) ** 2


def adsorbate_system(species, seed, n_atoms=None, cutoff=12.0, n_guest=0):
    """One box of `species` (a key of SPECIES) on lj_framework(seed, n_atoms). Charged
    species get framework charges U[-1.2, +1.4] e, neutralised, and the automatic Ewald
    set-up at precision 1e-6; the others run with charges off."""
    cell, fw, ft, eps_fw, sig_fw = lj_framework(seed, cutoff=cutoff, n_atoms=n_atoms)
    sites = SPECIES[species]
    charged = any(q != 0.0 for (_, _, _, q, _) in sites)
    g = _rng(seed + 7919)
    nt_fw = len(eps_fw)
    names, eps_K, sig, idx = [], list(eps_fw), list(sig_fw), []
    for name, e, s_, _, _ in sites:
        if name not in names:
            names.append(name)
            eps_K.append(e)
            sig.append(s_)
        idx.append(nt_fw + names.index(name))
    eps, sg, shift = mix_lorentz_berthelot(eps_K, sig, [1] * len(eps_K), cutoff)
    if charged:
        q = g.uniform(-1.2, 1.4, len(fw))
        q -= q.mean()
        alpha, kmax, rc = raspa_ewald(cell, cutoff)
    else:
        q = np.zeros(len(fw))
        alpha, kmax, rc = 0.265, [1, 1, 1], None
    tmpl = dict(pos=np.array([p for (_, _, _, _, p) in sites]), charge=np.array([c for (_, _, _, c, _) in sites]),
                type=np.array(idx))
    system = dict(
        name=f"{species}_{seed}", cell=cell, kmax=kmax, alpha=alpha, use_lammps_ewald=0, reciprocal_cutoff=rc,
        prefactor=COULOMB_PREFACTOR, ntypes=len(eps_K), epsilon=eps, sigma=sg, shift=shift, cutoff_vdw=cutoff,
        cutoff_coul=cutoff, overlap_criteria=1e6, no_charges=0 if charged else 1, vdw_real_bias=1,
        temperature=300.0, nhost=1, molsize=[len(fw), len(sites)], templates={1: tmpl})
    _set_atoms(system, fw, ft, q, [np.zeros((0, 3))])
    if n_guest:
        place_molecules(system, 1, n_guest, g, min_dist=2.8)
    return system


def serving_job(seed, widom_insertions=5000, gcmc_cycles=2000, steps_per_cycle=20, n_atoms_range=(200, 20000)):
    """One job of the serving stream: species uniform over CH4, CO2, N2, Xe, Kr; Widom
    (widom_insertions) or GCMC (gcmc_cycles x steps_per_cycle steps) with equal odds;
    framework atoms log-uniform in n_atoms_range. Returns a dict with the system,
    capacities and the work."""
    g = _rng(10_000_019 + seed)
    species = ["CH4", "CO2", "N2", "Xe", "Kr"][int(g.integers(0, 5))]
    kind = "widom" if g.uniform() < 0.5 else "gcmc"
    lo, hi = n_atoms_range
    n_atoms = int(round(math.exp(g.uniform(math.log(lo), math.log(hi)))))
    system = adsorbate_system(species, seed, n_atoms=n_atoms)
    ms = int(system["molsize"][1])
    return dict(seed=seed, species=species, kind=kind, n_atoms=len(system["pos"]), system=system,
                capacity=[system["comp_start"][1], ms * 256], widom_insertions=widom_insertions,
                gcmc_steps=gcmc_cycles * steps_per_cycle)


# ------------------------------------------------------------------ TIP4P-Ew water
def tip4p_ew_template():
    """TIP4P-Ew: O (81.899 K, 3.16435 A, no charge) first, then H, H (+0.52422) and the
    massless M site (-1.04844) 0.125 A from O on the bisector; O-H 0.9572 A, HOH 104.52
    deg."""
    th = math.radians(104.52 / 2.0)
    h = 0.9572
    pos = np.array([[0.0, 0.0, 0.0], [h * math.sin(th), 0.0, h * math.cos(th)],
                    [-h * math.sin(th), 0.0, h * math.cos(th)], [0.0, 0.0, 0.125]])
    return dict(pos=pos, charge=np.array([0.0, 0.52422, 0.52422, -1.04844]), names=["Ow", "Hw", "Hw", "Mw"])


def tip4p_hex_system(seed=42, n_water=0, cutoff=11.0, alpha=0.30, kmax=(10, 10, 8), cells=(1, 1, 4),
                     n_per_cell=216, n_types=4, channel_r=6.0):
    """Charge-dominated Ewald benchmark: TIP4P-Ew water in a synthetic hexagonal
    framework, a = b = 25.9 A, c = 6.9 A, gamma = 120 deg, 1 x 1 x 4 cells (864 atoms)
    on a jittered fractional lattice with random vacancies around one open channel
    (radius channel_r) along c. Framework charges
    U[-1.2, +1.4] e neutralised; LJ eps/k U[20, 100] K, sigma U[2.5, 3.5] A. The
    perpendicular width of this cell is 22.4 A, so the cutoff is 11 A (< width / 2);
    Ewald alpha 0.30 A^-1 with kmax 10/10/8 (explicit set-up)."""
    g = _rng(seed)
    base = np.array(triclinic_cell(25.9, 25.9, 6.9, 90.0, 90.0, 120.0)).reshape(3, 3).T
    grid = np.array([9, 9, 4])
    idx = np.stack(np.meshgrid(*[np.arange(k) for k in grid], indexing="ij"), -1).reshape(-1, 3)
    frac = (idx + 0.5) / grid
    # one open channel along c through the cell corner (radius channel_r): the
    # framework atoms fill the rest, as the walls of a hexagonal channel framework
    d = frac[:, :2] - np.round(frac[:, :2])
    r_xy = np.linalg.norm(np.c_[d, np.zeros(len(d))] @ base.T, axis=1)
    keep = np.where(r_xy > channel_r)[0]
    sel = keep[g.choice(len(keep), n_per_cell, replace=False)]
    frac = (idx[sel] + 0.5 + g.uniform(-0.15, 0.15, (n_per_cell, 3))) / grid
    pts = frac @ base.T
    shifts = np.stack(np.meshgrid(*[np.arange(k) for k in cells], indexing="ij"), -1).reshape(-1, 3)
    fw = (pts[None, :, :] + (shifts @ base.T)[:, None, :]).reshape(-1, 3)
    ft = np.tile(g.integers(0, n_types, n_per_cell), len(shifts))
    q = g.uniform(-1.2, 1.4, len(fw))
    q -= q.mean()
    cell = (base * np.array(cells)[None, :]).T.reshape(-1).tolist()
    eps_K = list(g.uniform(20.0, 100.0, n_types)) + [81.899, 0.0, 0.0]
    sig = list(g.uniform(2.5, 3.5, n_types)) + [3.16435, 1.0, 1.0]
    eps, sg, shift = mix_lorentz_berthelot(eps_K, sig, [1] * len(eps_K), cutoff)
    tm = tip4p_ew_template()
    tm["type"] = np.array([n_types, n_types + 1, n_types + 1, n_types + 2])
    system = dict(
        name="tip4p_hex", cell=cell, kmax=list(kmax), alpha=alpha, use_lammps_ewald=1, prefactor=COULOMB_PREFACTOR,
        ntypes=len(eps_K), epsilon=eps, sigma=sg, shift=shift, cutoff_vdw=cutoff, cutoff_coul=cutoff,
        overlap_criteria=1e6, no_charges=0, vdw_real_bias=1, temperature=300.0, nhost=1, molsize=[len(fw), 4],
        templates={1: tm})
    _set_atoms(system, fw, ft, q, [np.zeros((0, 3))])
    if n_water:
        place_molecules(system, 1, n_water, g, min_dist=2.5)
    return system
