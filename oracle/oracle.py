"""ctypes bindings of the FP64 CPU oracle (oracle/grx_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the
checker, and by bench.py for the CPU-baseline and reference legs. The product
library (graspa_gb300) never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgrx_oracle.so")

_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)
_u8p = C.POINTER(C.c_uint8)


class OraBox(C.Structure):
    _fields_ = [("cell", C.c_double * 9), ("inverse_cell", C.c_double * 9), ("volume", C.c_double),
                ("cubic", C.c_int32), ("use_lammps_ewald", C.c_int32), ("kmax", C.c_int32 * 3),
                ("pad_", C.c_int32), ("alpha", C.c_double), ("prefactor", C.c_double),
                ("reciprocal_cutoff", C.c_double)]


class OraFF(C.Structure):
    _fields_ = [("ntypes", C.c_int64), ("epsilon", _dp), ("sigma", _dp), ("z", _dp), ("shift", _dp),
                ("c10", _dp), ("use_1264", C.c_int32), ("no_charges", C.c_int32),
                ("vdw_real_bias", C.c_int32), ("pad_", C.c_int32), ("overlap_criteria", C.c_double),
                ("cutoff_vdw_sq", C.c_double), ("cutoff_coul_sq", C.c_double)]


class OraAtoms(C.Structure):
    _fields_ = [("ncomp", C.c_int64), ("nhost", C.c_int64), ("comp_start", _i64p), ("pos", _dp),
                ("scale", _dp), ("charge", _dp), ("scale_coul", _dp), ("type", _i64p), ("molid", _i64p)]


class OraTrials(C.Structure):
    _fields_ = [("ntrials", C.c_int64), ("chainsize", C.c_int64), ("pos", _dp), ("scale", _dp),
                ("charge", _dp), ("scale_coul", _dp), ("type", _i64p), ("molid", C.c_int64)]


class OraWidom(C.Structure):
    _fields_ = [("component", C.c_int64), ("molsize", C.c_int64), ("mol_pos", _dp), ("mol_charge", _dp),
                ("mol_type", _i64p), ("scale", C.c_double), ("scale_coul", C.c_double),
                ("ntrials", C.c_int64), ("norient", C.c_int64), ("new_molid", C.c_int64),
                ("beta", C.c_double), ("excl_intra", C.c_double), ("excl_self", C.c_double),
                ("tail_delta", C.c_double), ("rigid", C.c_int32), ("has_charge", C.c_int32),
                ("seed", C.c_uint64), ("stream", C.c_uint32), ("pad_", C.c_uint32)]


class OraWidomResult(C.Structure):
    _fields_ = [("rosenbluth", C.c_double), ("w_first", C.c_double), ("w_chain", C.c_double),
                ("e_first", C.c_double * 4), ("e_chain", C.c_double * 4), ("ewald", C.c_double * 2),
                ("sel_first", C.c_int64), ("sel_orient", C.c_int64), ("n_ok_first", C.c_int64),
                ("n_ok_orient", C.c_int64), ("success", C.c_int32), ("pad_", C.c_int32)]


class OraGcmc(C.Structure):
    _fields_ = [("component", C.c_int64), ("ntrials", C.c_int64), ("norient", C.c_int64),
                ("p_translation", C.c_double), ("p_rotation", C.c_double), ("p_reinsertion", C.c_double),
                ("p_swap", C.c_double), ("max_translation", C.c_double * 3), ("max_rotation", C.c_double * 3),
                ("beta", C.c_double),
                ("pressure", C.c_double), ("fugacity_coeff", C.c_double), ("mol_fraction", C.c_double),
                ("ideal_rosenbluth", C.c_double), ("seed", C.c_uint64), ("stream", C.c_uint32), ("pad_", C.c_uint32),
                ("tail_insert", C.c_double)]


class OraGcmcStats(C.Structure):
    _fields_ = [("attempts", C.c_int64 * 5), ("accepted", C.c_int64 * 5), ("n_molecules", C.c_int64),
                ("energy", C.c_double * 4), ("sum_n", C.c_double), ("rosen", C.c_double * 3),
                ("trial_configs", C.c_int64), ("trial_beads", C.c_int64), ("last_margin", C.c_double)]


def build(force=False):
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-C", HERE], check=True, stdout=subprocess.DEVNULL)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        L.ora_box_setup.argtypes = [P(OraBox)]
        L.ora_box_setup_raspa_ewald.argtypes = [P(OraBox), C.c_double, C.c_double]
        L.ora_mix_lorentz_berthelot.argtypes = [C.c_int64, _dp, _dp, P(C.c_int32), C.c_double, _dp, _dp, _dp]
        L.ora_pbc.argtypes = [P(OraBox), _dp]
        L.ora_trial_energies.argtypes = [P(OraBox), P(OraFF), P(OraAtoms), P(OraTrials), C.c_int64,
                                         C.c_int64, C.c_int64, _dp, _u8p]
        L.ora_single_body.argtypes = [P(OraBox), P(OraFF), P(OraAtoms), P(OraTrials), P(OraTrials),
                                      C.c_int64, C.c_int32, C.c_int32, _dp, _u8p]
        L.ora_vdw_real_total.argtypes = [P(OraBox), P(OraFF), P(OraAtoms), _dp]
        L.ora_ewald_nvec.argtypes = [P(OraBox)]
        L.ora_ewald_nvec.restype = C.c_int64
        L.ora_ewald_active.argtypes = [P(OraBox), _u8p]
        L.ora_ewald_active.restype = C.c_int64
        L.ora_ewald_total.argtypes = [P(OraBox), P(OraAtoms), _i64p, _dp, _dp, _dp]
        L.ora_ewald_delta.argtypes = [P(OraBox), _dp, _dp, C.c_int32, _dp, C.c_int64, _dp, _dp,
                                      C.c_int64, _dp, _dp, _dp, _dp]
        L.ora_ewald_delta_lambda.argtypes = [P(OraBox), _dp, _dp, C.c_int32, _dp, C.c_int64, _dp, _dp, C.c_double,
                                             C.c_double, C.c_double, _dp, _dp]
        L.ora_ewald_delta_identity_swap.argtypes = [P(OraBox), _dp, _dp, C.c_int64, _dp, _dp, C.c_int64, _dp, _dp,
                                                    C.c_double, C.c_double, _dp, _dp]
        L.ora_rigid_exclusion.argtypes = [P(OraBox), C.c_int64, _dp, _dp, _dp, _dp, _dp]
        L.ora_philox4x32_10.argtypes = [P(C.c_uint32), P(C.c_uint32), P(C.c_uint32)]
        L.ora_draw.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_uint32, P(C.c_uint32)]
        L.ora_select_trial.argtypes = [_dp, C.c_int64, C.c_double]
        L.ora_select_trial.restype = C.c_int64
        L.ora_rotate_quaternion.argtypes = [_dp, C.c_double, C.c_double, C.c_double]
        L.ora_widom_insertions.argtypes = [P(OraBox), P(OraFF), P(OraAtoms), _dp, _dp, P(OraWidom),
                                           C.c_uint64, C.c_int64, C.c_int32, P(OraWidomResult)]
        L.ora_max_threads.restype = C.c_int32
        L.ora_gcmc_run.argtypes = [P(OraBox), P(OraFF), _dp, _dp, _i64p, _i64p, C.c_int64, C.c_int64, _i64p, _i64p,
                                   _i64p, _dp, _dp, _i64p, C.c_double, C.c_double, _dp, _dp, P(OraGcmc), C.c_uint64,
                                   C.c_int64, P(OraGcmcStats)]
        L.ora_gcmc_run_mix.argtypes = [P(OraBox), P(OraFF), _dp, _dp, _i64p, _i64p, C.c_int64, C.c_int64, _i64p,
                                       _i64p, _i64p, P(_dp), P(_dp), P(_i64p), _dp, _dp, _dp, _dp, P(OraGcmc),
                                       C.c_int64, C.c_uint64, C.c_int64, P(OraGcmcStats)]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_i64p)


class OracleSystem:
    """Holds numpy arrays for one box in the oracle's layout (keeps them alive)."""

    def __init__(self, system):
        """`system` is a graspa_gb300-independent dict produced by tests/systems.py."""
        self.s = system
        b = OraBox()
        for i, v in enumerate(system["cell"]):
            b.cell[i] = v
        b.use_lammps_ewald = int(system.get("use_lammps_ewald", 1))
        for i in range(3):
            b.kmax[i] = int(system["kmax"][i])
        b.alpha = system["alpha"]
        b.prefactor = system.get("prefactor", 138935.483496)
        lib().ora_box_setup(C.byref(b))
        if system.get("reciprocal_cutoff") is not None:
            b.reciprocal_cutoff = system["reciprocal_cutoff"]
        self.box = b
        nt = system["ntypes"]
        self.eps = np.ascontiguousarray(system["epsilon"], dtype=np.float64)
        self.sig = np.ascontiguousarray(system["sigma"], dtype=np.float64)
        self.shift = np.ascontiguousarray(system["shift"], dtype=np.float64)
        self.zero = np.zeros(nt * nt)
        self.z = np.ascontiguousarray(system.get("z", self.zero), dtype=np.float64)
        self.c10 = np.ascontiguousarray(system.get("c10", self.zero), dtype=np.float64)
        ff = OraFF()
        ff.ntypes = nt
        ff.epsilon, ff.sigma, ff.shift = _d(self.eps), _d(self.sig), _d(self.shift)
        ff.z, ff.c10 = _d(self.z), _d(self.c10)
        ff.use_1264 = int(system.get("use_1264", 0))
        ff.no_charges = int(system.get("no_charges", 0))
        ff.vdw_real_bias = int(system.get("vdw_real_bias", 1))
        ff.overlap_criteria = system.get("overlap_criteria", 1e6)
        ff.cutoff_vdw_sq = system["cutoff_vdw"] ** 2
        ff.cutoff_coul_sq = system["cutoff_coul"] ** 2
        self.ff = ff
        self.set_atoms(system)

    def set_atoms(self, system):
        self.comp_start = np.ascontiguousarray(system["comp_start"], dtype=np.int64)
        self.pos = np.ascontiguousarray(system["pos"], dtype=np.float64).reshape(-1)
        self.scale = np.ascontiguousarray(system["scale"], dtype=np.float64)
        self.charge = np.ascontiguousarray(system["charge"], dtype=np.float64)
        self.scale_coul = np.ascontiguousarray(system["scale_coul"], dtype=np.float64)
        self.type = np.ascontiguousarray(system["type"], dtype=np.int64)
        self.molid = np.ascontiguousarray(system["molid"], dtype=np.int64)
        a = OraAtoms()
        a.ncomp = len(self.comp_start) - 1
        a.nhost = system["nhost"]
        a.comp_start = _i(self.comp_start)
        a.pos, a.scale, a.charge, a.scale_coul = _d(self.pos), _d(self.scale), _d(self.charge), _d(self.scale_coul)
        a.type, a.molid = _i(self.type), _i(self.molid)
        self.atoms = a

    # --- energies --------------------------------------------------------
    def trial_energies(self, pos, scale, charge, scale_coul, types, molid, ntrials, chainsize,
                       component, excl_comp=-1, excl_molid=-1):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        scale = np.ascontiguousarray(scale, dtype=np.float64)
        charge = np.ascontiguousarray(charge, dtype=np.float64)
        scale_coul = np.ascontiguousarray(scale_coul, dtype=np.float64)
        types = np.ascontiguousarray(types, dtype=np.int64)
        t = OraTrials(ntrials, chainsize, _d(pos), _d(scale), _d(charge), _d(scale_coul), _i(types), molid)
        out = np.zeros((ntrials, 4))
        flag = np.zeros(ntrials, dtype=np.uint8)
        lib().ora_trial_energies(C.byref(self.box), C.byref(self.ff), C.byref(self.atoms), C.byref(t),
                                 component, excl_comp, excl_molid, _d(out), flag.ctypes.data_as(_u8p))
        return out, flag

    def vdw_real_total(self):
        out = np.zeros(6)
        lib().ora_vdw_real_total(C.byref(self.box), C.byref(self.ff), C.byref(self.atoms), _d(out))
        return out

    def nvec(self):
        return lib().ora_ewald_nvec(C.byref(self.box))

    def ewald_active(self):
        act = np.zeros(self.nvec(), dtype=np.uint8)
        n = lib().ora_ewald_active(C.byref(self.box), act.ctypes.data_as(_u8p))
        return n, act

    def ewald_total(self, molsize):
        nv = self.nvec()
        s_fw = np.zeros(2 * nv)
        s_ads = np.zeros(2 * nv)
        out = np.zeros(8)
        ms = np.ascontiguousarray(molsize, dtype=np.int64)
        lib().ora_ewald_total(C.byref(self.box), C.byref(self.atoms), _i(ms), _d(s_fw), _d(s_ads), _d(out))
        return out, s_fw, s_ads

    def ewald_delta(self, s_same, s_cross, old_pos, old_qs, new_pos, new_qs):
        nv = self.nvec()
        old_pos = np.ascontiguousarray(old_pos, dtype=np.float64).reshape(-1)
        new_pos = np.ascontiguousarray(new_pos, dtype=np.float64).reshape(-1)
        old_qs = np.ascontiguousarray(old_qs, dtype=np.float64)
        new_qs = np.ascontiguousarray(new_qs, dtype=np.float64)
        s_new = np.zeros(2 * nv)
        out = np.zeros(2)
        lib().ora_ewald_delta(C.byref(self.box), _d(s_same), _d(s_cross), 0, _d(s_same),
                              len(old_qs), _d(old_pos), _d(old_qs), len(new_qs), _d(new_pos), _d(new_qs),
                              _d(s_new), _d(out))
        return out, s_new

    def ewald_delta_lambda(self, s_same, s_cross, pos, charge, scale_old, scale_new, excl, s_temp=None):
        """GPU_EwaldDifference_LambdaChange: (out2 with exclusion and the doubled cross term, S staged)."""
        nv = self.nvec()
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        q = np.ascontiguousarray(charge, dtype=np.float64)
        st = np.ascontiguousarray(s_temp if s_temp is not None else s_same, dtype=np.float64)
        s_new = np.zeros(2 * nv)
        out = np.zeros(2)
        lib().ora_ewald_delta_lambda(C.byref(self.box), _d(s_same), _d(s_cross), int(s_temp is not None), _d(st),
                                     len(q), _d(pos), _d(q), scale_old, scale_new, excl, _d(s_new), _d(out))
        return out, s_new

    def ewald_delta_identity_swap(self, s_same, s_cross, old_pos, old_qs, new_pos, new_qs, excl_new, excl_old):
        """GPU_EwaldDifference_IdentitySwap: (out2, S staged)."""
        nv = self.nvec()
        old_pos = np.ascontiguousarray(old_pos, dtype=np.float64).reshape(-1)
        new_pos = np.ascontiguousarray(new_pos, dtype=np.float64).reshape(-1)
        old_qs = np.ascontiguousarray(old_qs, dtype=np.float64)
        new_qs = np.ascontiguousarray(new_qs, dtype=np.float64)
        s_new = np.zeros(2 * nv)
        out = np.zeros(2)
        lib().ora_ewald_delta_identity_swap(C.byref(self.box), _d(s_same), _d(s_cross), len(old_qs), _d(old_pos),
                                            _d(old_qs), len(new_qs), _d(new_pos), _d(new_qs), excl_new, excl_old,
                                            _d(s_new), _d(out))
        return out, s_new

    def rigid_exclusion(self, pos, charge, scale_coul):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        charge = np.ascontiguousarray(charge, dtype=np.float64)
        scale_coul = np.ascontiguousarray(scale_coul, dtype=np.float64)
        a, b = C.c_double(), C.c_double()
        lib().ora_rigid_exclusion(C.byref(self.box), len(charge), _d(pos), _d(charge), _d(scale_coul),
                                  C.byref(a), C.byref(b))
        return a.value, b.value

    def gcmc(self, params, capacity, first_step, nsteps):
        """Run nsteps GCMC moves (oracle). params: one OraGcmc, or a list of them for a
        mixture (one per moved component). Returns (stats, system_after, s_ads_after),
        stats a list when params is a list."""
        ch = OracleChain(self, params, capacity)
        stats = ch.run(first_step, nsteps)
        return (stats if isinstance(params, (list, tuple)) else stats[0]), ch.state(), ch.s_ads

    def widom(self, params, s_fw, s_ads, first_move, n, nthreads=0):
        res = (OraWidomResult * n)()
        lib().ora_widom_insertions(C.byref(self.box), C.byref(self.ff), C.byref(self.atoms), _d(s_fw),
                                   _d(s_ads), C.byref(params), first_move, n, nthreads, res)
        return res


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().ora_philox4x32_10(c, k, o)
    return list(o)


def u01(w):
    """Uniform in [0, 1) from one Philox word (grx_u01: w * 2^-32)."""
    return float(w) * 2.3283064365386963e-10


def draw(seed, stream, move, slot):
    o = (C.c_uint32 * 4)()
    lib().ora_draw(seed, stream, move, slot, o)
    return list(o)


def select_trial(logw, u):
    lw = np.ascontiguousarray(logw, dtype=np.float64)
    return lib().ora_select_trial(_d(lw), len(lw), u)


def mix_lb(eps_K, sigma, shifted, cutoff_vdw):
    n = len(eps_K)
    e = np.ascontiguousarray(eps_K, dtype=np.float64)
    s = np.ascontiguousarray(sigma, dtype=np.float64)
    sh = np.ascontiguousarray(shifted, dtype=np.int32)
    eo, so, sho = np.zeros(n * n), np.zeros(n * n), np.zeros(n * n)
    lib().ora_mix_lorentz_berthelot(n, _d(e), _d(s), sh.ctypes.data_as(C.POINTER(C.c_int32)),
                                    cutoff_vdw ** 2, _d(eo), _d(so), _d(sho))
    return eo, so, sho


class OracleChain:
    """One GCMC chain whose state stays resident in host memory across calls: atoms,
    molecule counts, both structure factors and the slot-0 templates the orientations grow
    from. The FP64 Ewald totals (framework S(k) and the adsorbate S(k), framework
    exclusions included) are computed once here, at set-up; `run` then only makes moves,
    continuing the chain where the last call left it (the same trajectory as one long
    call)."""

    def __init__(self, osys, params, capacity, ewald=None):
        """ewald: (s_fw, s_ads) of the starting state when already known (copied), else
        computed here."""
        self.osys = osys if isinstance(osys, OracleSystem) else OracleSystem(osys)
        plist = list(params) if isinstance(params, (list, tuple)) else [params]
        sysd = self.osys.s
        cs = list(sysd["comp_start"])
        ncomp = len(cs) - 1
        sizes = np.array([cs[c + 1] - cs[c] for c in range(ncomp)], dtype=np.int64)
        offs = np.zeros(ncomp, dtype=np.int64)
        caps = [max(sizes[c], capacity[c]) for c in range(ncomp)]
        for c in range(1, ncomp):
            offs[c] = offs[c - 1] + caps[c - 1]
        tot = int(offs[-1] + caps[-1])
        self.pos = np.zeros(3 * tot)
        self.q = np.zeros(tot)
        self.ty = np.zeros(tot, dtype=np.int64)
        self.mol = np.zeros(tot, dtype=np.int64)
        P_ = np.asarray(sysd["pos"], dtype=np.float64).reshape(-1, 3)
        for c in range(ncomp):
            a, b = cs[c], cs[c + 1]
            o = offs[c]
            self.pos[3 * o:3 * (o + b - a)] = P_[a:b].reshape(-1)
            self.q[o:o + b - a] = np.asarray(sysd["charge"])[a:b]
            self.ty[o:o + b - a] = np.asarray(sysd["type"])[a:b]
            self.mol[o:o + b - a] = np.asarray(sysd["molid"])[a:b]
        self.ms = np.array(sysd["molsize"], dtype=np.int64)
        self.sizes, self.offs, self.ncomp = sizes, offs, ncomp
        self.keep = []
        mps, mqs, mts, ein, esf = [], [], [], [], []
        for pr in plist:
            comp = pr.component
            tm = sysd["templates"][comp]
            a, b = cs[comp], cs[comp + 1]
            mp = np.ascontiguousarray((P_[a:a + self.ms[comp]] if b > a else tm["pos"]).reshape(-1),
                                      dtype=np.float64).copy()
            mq = np.ascontiguousarray(tm["charge"], dtype=np.float64)
            mt = np.ascontiguousarray(tm["type"], dtype=np.int64)
            intra, self_ = self.osys.rigid_exclusion(mp, mq, np.ones(len(mq)))
            self.keep += [mp, mq, mt]
            mps.append(_d(mp))
            mqs.append(_d(mq))
            mts.append(_i(mt))
            ein.append(intra)
            esf.append(self_)
        ng = len(plist)
        self.ng = ng
        if ewald is None:
            _, self.s_fw, self.s_ads = self.osys.ewald_total(list(self.ms))
        else:
            self.s_fw, self.s_ads = np.array(ewald[0], dtype=np.float64), np.array(ewald[1], dtype=np.float64)
        self.mps = (_dp * ng)(*mps)
        self.mqs = (_dp * ng)(*mqs)
        self.mts = (_i64p * ng)(*mts)
        self.ein = (C.c_double * ng)(*ein)
        self.esf = (C.c_double * ng)(*esf)
        self.gk = (OraGcmc * ng)(*plist)

    def run(self, first_step, nsteps):
        """nsteps moves from Philox move index first_step; returns one OraGcmcStats per
        moved component, counted over this call."""
        st = (OraGcmcStats * self.ng)()
        sysd = self.osys.s
        lib().ora_gcmc_run_mix(C.byref(self.osys.box), C.byref(self.osys.ff), _d(self.pos), _d(self.q), _i(self.ty),
                               _i(self.mol), self.ncomp, sysd["nhost"], _i(self.sizes), _i(self.offs), _i(self.ms),
                               self.mps, self.mqs, self.mts, self.ein, self.esf, _d(self.s_fw), _d(self.s_ads),
                               self.gk, self.ng, first_step, nsteps, st)
        return list(st)

    def state(self):
        """The chain's atoms as a system dict (components compacted)."""
        after = dict(self.osys.s)
        newpos, newq, newt, newm = [], [], [], []
        starts = [0]
        for c in range(self.ncomp):
            o, n = self.offs[c], self.sizes[c]
            newpos.append(self.pos[3 * o:3 * (o + n)].reshape(-1, 3))
            newq.append(self.q[o:o + n])
            newt.append(self.ty[o:o + n])
            newm.append(self.mol[o:o + n])
            starts.append(starts[-1] + n)
        after["pos"] = np.concatenate(newpos)
        after["charge"] = np.concatenate(newq)
        after["type"] = np.concatenate(newt)
        after["molid"] = np.concatenate(newm)
        after["scale"] = np.ones(starts[-1])
        after["scale_coul"] = np.ones(starts[-1])
        after["comp_start"] = starts
        return after
