"""ctypes binding of libgrx.so (include/grx.h) and a small Box wrapper.

This is the Python face of the C ABI, used by the tests and the benchmark the way
gRASPA's pybind module (src_clean/pybind.h) exposes its structs. All energy work
runs in libgrx.so on the GPU; there is no CPU fallback: loading fails loudly when
the library or a CUDA device is missing.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgrx.so")

GRX_FP64, GRX_MIXED, GRX_FP32 = 0, 1, 2
PRECISIONS = {"fp64": GRX_FP64, "mixed": GRX_MIXED, "fp32": GRX_FP32}
MOVE_TRANSLATION, MOVE_ROTATION, MOVE_SINGLE_INSERTION, MOVE_SINGLE_DELETION = 0, 1, 2, 3
MOVE_INSERTION, MOVE_DELETION, MOVE_REINSERTION = 5, 6, 7
MOVE_CBCF_LAMBDACHANGE, MOVE_CBCF_INSERTION, MOVE_CBCF_DELETION, MOVE_IDENTITY_SWAP = 8, 9, 10, 11
MAX_COMPONENTS = 8

_dp = C.POINTER(C.c_double)
_szp = C.POINTER(C.c_size_t)
_u8p = C.POINTER(C.c_uint8)


class GrxError(RuntimeError):
    pass


class BoxGeometry(C.Structure):
    _fields_ = [("cell", C.c_double * 9), ("inverse_cell", C.c_double * 9), ("volume", C.c_double),
                ("cubic", C.c_int32), ("use_lammps_ewald", C.c_int32), ("kmax", C.c_int32 * 3),
                ("pad_", C.c_int32), ("alpha", C.c_double), ("prefactor", C.c_double),
                ("reciprocal_cutoff", C.c_double)]


class ForceField(C.Structure):
    _fields_ = [("ntypes", C.c_int32), ("use_1264", C.c_int32), ("epsilon", _dp), ("sigma", _dp),
                ("z", _dp), ("shift", _dp), ("c10", _dp), ("no_charges", C.c_int32),
                ("vdw_real_bias", C.c_int32), ("overlap_criteria", C.c_double),
                ("cutoff_vdw_sq", C.c_double), ("cutoff_coul_sq", C.c_double)]


class BoxDesc(C.Structure):
    _fields_ = [("geometry", BoxGeometry), ("forcefield", ForceField), ("ncomponents", C.c_int32),
                ("nhost_components", C.c_int32), ("capacity", C.c_size_t * MAX_COMPONENTS),
                ("molsize", C.c_size_t * MAX_COMPONENTS)]


class Atoms(C.Structure):
    _fields_ = [("pos", _dp), ("scale", _dp), ("charge", _dp), ("scale_coul", _dp), ("type", _szp),
                ("molid", _szp), ("size", C.c_size_t), ("n_stored", C.c_size_t)]


class Trials(C.Structure):
    _fields_ = [("pos", _dp), ("scale", _dp), ("charge", _dp), ("scale_coul", _dp), ("type", _szp),
                ("molid", C.c_size_t), ("ntrials", C.c_size_t), ("chainsize", C.c_size_t)]


class TrialEnergy(C.Structure):
    _fields_ = [("hg_vdw", C.c_double), ("hg_real", C.c_double), ("gg_vdw", C.c_double),
                ("gg_real", C.c_double)]


class Energy(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("hh_vdw", "hh_real", "hg_vdw", "hg_real", "gg_vdw", "gg_real",
                                          "hh_ewald", "hg_ewald", "gg_ewald")]


class WidomDesc(C.Structure):
    _fields_ = [("component", C.c_int32), ("ntrials", C.c_int32), ("norient", C.c_int32),
                ("pad_", C.c_int32), ("scale", C.c_double), ("scale_coul", C.c_double),
                ("beta", C.c_double), ("tail_delta", C.c_double), ("seed", C.c_uint64),
                ("stream", C.c_uint32), ("pad2_", C.c_uint32)]


class WidomResult(C.Structure):
    _fields_ = [("rosenbluth", C.c_double), ("w_first", C.c_double), ("w_chain", C.c_double),
                ("e_first", C.c_double * 4), ("e_chain", C.c_double * 4), ("ewald", C.c_double * 2),
                ("sel_first", C.c_int64), ("sel_orient", C.c_int64), ("n_ok_first", C.c_int64),
                ("n_ok_orient", C.c_int64), ("success", C.c_int32), ("pad_", C.c_int32)]


WIDOM_RESULT_DTYPE = np.dtype([("rosenbluth", "f8"), ("w_first", "f8"), ("w_chain", "f8"),
                               ("e_first", "f8", 4), ("e_chain", "f8", 4), ("ewald", "f8", 2),
                               ("sel_first", "i8"), ("sel_orient", "i8"), ("n_ok_first", "i8"),
                               ("n_ok_orient", "i8"), ("success", "i4"), ("pad_", "i4")])
assert WIDOM_RESULT_DTYPE.itemsize == C.sizeof(WidomResult)


class GcmcDesc(C.Structure):
    _fields_ = [("component", C.c_int32), ("ntrials", C.c_int32), ("norient", C.c_int32),
                ("pad_", C.c_int32), ("p_translation", C.c_double), ("p_rotation", C.c_double),
                ("p_reinsertion", C.c_double), ("p_swap", C.c_double), ("max_translation", C.c_double * 3), ("max_rotation", C.c_double * 3),
                ("beta", C.c_double), ("pressure", C.c_double), ("fugacity_coeff", C.c_double),
                ("mol_fraction", C.c_double), ("ideal_rosenbluth", C.c_double), ("tail_insert", C.c_double),
                ("seed", C.c_uint64), ("stream", C.c_uint32), ("pad2_", C.c_uint32),
                ("p_identity_swap", C.c_double)]


class GcmcStats(C.Structure):
    _fields_ = [("attempts", C.c_int64 * 5), ("accepted", C.c_int64 * 5), ("n_molecules", C.c_int64),
                ("capacity_hits", C.c_int64), ("energy", C.c_double * 4), ("sum_n", C.c_double),
                ("identity_out", C.c_int64 * 2), ("identity_in", C.c_int64 * 2),
                ("rosen", C.c_double * 3), ("trial_configs", C.c_int64),
                ("trial_beads", C.c_int64)]

JOB_WIDOM, JOB_GCMC = 0, 1
GCMC_TUNE_CANDIDATES = 9  # GRX_GCMC_TUNE_CANDIDATES: warps per box 8/12/24 x items per warp 1/2/4


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("max_resident", C.c_int32), ("precision", C.c_int32),
                ("widom_slice", C.c_int64), ("gcmc_slice", C.c_int64), ("cluster_atoms", C.c_int64),
                ("gcmc_batching", C.c_int32), ("pad_", C.c_int32)]


class JobDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("ncomp_moved", C.c_int32), ("box", C.POINTER(BoxDesc)),
                ("atoms", C.POINTER(Atoms)), ("rigid", C.POINTER(C.c_int32)), ("widom", WidomDesc),
                ("widom_insertions", C.c_int64), ("gcmc", C.POINTER(GcmcDesc)), ("gcmc_steps", C.c_int64),
                ("tag", C.c_uint64)]


class JobResult(C.Structure):
    _fields_ = [("tag", C.c_uint64), ("job_id", C.c_uint64), ("kind", C.c_int32), ("status", C.c_int32),
                ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double),
                ("footprint_bytes", C.c_size_t), ("widom_n", C.c_int64), ("widom_mean_w", C.c_double),
                ("widom_mean_w2", C.c_double), ("gcmc_steps", C.c_int64), ("ncomp_moved", C.c_int32),
                ("pad_", C.c_int32), ("gcmc", GcmcStats * 4), ("widom_trial_configs", C.c_int64)]


# every symbol include/grx.h declares
EXPORTS = [
    "grx_status_string", "grx_last_error", "grx_device_count", "grx_box_create", "grx_box_destroy",
    "grx_box_set_stream", "grx_box_set_component", "grx_box_get_component_size", "grx_box_get_positions",
    "grx_box_get_exclusion", "grx_trial_energies", "grx_single_body_energy", "grx_ewald_sizes",
    "grx_ewald_total", "grx_ewald_set_structure_factors", "grx_ewald_get_structure_factors",
    "grx_total_energy_overlap", "grx_ewald_delta", "grx_ewald_delta_lambda", "grx_ewald_delta_identity_swap", "grx_ewald_commit", "grx_total_energy", "grx_cbmc_select",
    "grx_widom_insertions", "grx_widom_insertions_async", "grx_launch_count", "grx_last_transfer", "grx_probe_fp32_fma", "grx_trial_energies_noalloc", "grx_gcmc_run",
    "grx_box_write_molecule", "grx_box_remove_molecule", "grx_gcmc_batch_create", "grx_gcmc_batch_destroy",
    "grx_gcmc_batch_set_step", "grx_gcmc_batch_launch", "grx_gcmc_batch_run_graph", "grx_gcmc_batch_stats",
    "grx_gcmc_batch_reset_stats", "grx_gcmc_batch_autotune", "grx_gcmc_batch_set_shape", "grx_gcmc_batch_get_shape",
    "grx_gcmc_batch_set_cluster", "grx_gcmc_batch_get_cluster", "grx_arena_create", "grx_arena_destroy",
    "grx_arena_usage", "grx_box_create_in", "grx_box_footprint", "grx_server_create", "grx_server_destroy",
    "grx_server_submit", "grx_server_progress", "grx_server_poll", "grx_server_time", "grx_server_launch_count",
    "grx_box_create_replica", "grx_box_set_voxel_lists", "grx_box_get_voxel_lists", "grx_gcmc_batch_set_box_steps",
    "grx_probe_df_functions",
]

_lib = None


def build():
    from . import build as _b
    return _b.build()


def load(path=LIB_PATH):
    """Load libgrx.so; raises if it is missing (no fallback path exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise GrxError(f"libgrx.so not built at {path}; run graspa_gb300.build")
    L = C.CDLL(path)
    P = C.POINTER
    L.grx_status_string.restype = C.c_char_p
    L.grx_status_string.argtypes = [C.c_int32]
    L.grx_last_error.restype = C.c_char_p
    L.grx_device_count.argtypes = [P(C.c_int32)]
    L.grx_box_create.argtypes = [P(BoxDesc), P(C.c_void_p)]
    L.grx_box_destroy.argtypes = [C.c_void_p]
    L.grx_box_set_stream.argtypes = [C.c_void_p, C.c_void_p]
    L.grx_box_set_component.argtypes = [C.c_void_p, C.c_int32, P(Atoms), C.c_int32]
    L.grx_box_get_component_size.argtypes = [C.c_void_p, C.c_int32, P(C.c_size_t)]
    L.grx_box_get_positions.argtypes = [C.c_void_p, C.c_int32, _dp, C.c_size_t]
    L.grx_box_get_exclusion.argtypes = [C.c_void_p, C.c_int32, _dp, _dp]
    L.grx_trial_energies.argtypes = [C.c_void_p, P(Trials), C.c_int32, C.c_int64, C.c_int64, C.c_int32,
                                     P(TrialEnergy), _u8p]
    L.grx_single_body_energy.argtypes = [C.c_void_p, P(Trials), P(Trials), C.c_int32, C.c_int32, C.c_int32,
                                         C.c_int32, _dp, _u8p]
    L.grx_ewald_sizes.argtypes = [C.c_void_p, P(C.c_int64), P(C.c_int64)]
    L.grx_ewald_total.argtypes = [C.c_void_p, _dp]
    L.grx_ewald_set_structure_factors.argtypes = [C.c_void_p, _dp, _dp]
    L.grx_ewald_get_structure_factors.argtypes = [C.c_void_p, _dp, _dp, _dp]
    L.grx_ewald_delta.argtypes = [C.c_void_p, C.c_int32, C.c_int32, _dp, _dp, C.c_size_t, _dp, _dp,
                                  C.c_size_t, C.c_double, _dp]
    L.grx_ewald_delta_lambda.argtypes = [C.c_void_p, C.c_int32, _dp, _dp, C.c_size_t, C.c_double, C.c_double,
                                         C.c_int32, _dp]
    L.grx_ewald_delta_identity_swap.argtypes = [C.c_void_p, C.c_int32, C.c_int32, _dp, _dp, C.c_size_t, _dp, _dp,
                                                C.c_size_t, _dp]
    L.grx_ewald_commit.argtypes = [C.c_void_p, C.c_int32]
    L.grx_total_energy.argtypes = [C.c_void_p, P(Energy)]
    L.grx_total_energy_overlap.argtypes = [C.c_void_p, P(Energy), _u8p]
    L.grx_cbmc_select.argtypes = [_dp, C.c_int32, C.c_uint64, C.c_uint32, C.c_uint64, C.c_int32,
                                  P(C.c_int32), _dp]
    L.grx_widom_insertions.argtypes = [C.c_void_p, P(WidomDesc), C.c_uint64, C.c_size_t, C.c_int32, C.c_void_p]
    L.grx_widom_insertions_async.argtypes = [C.c_void_p, P(WidomDesc), C.c_uint64, C.c_size_t, C.c_int32,
                                             C.c_void_p]
    L.grx_launch_count.restype = C.c_uint64
    L.grx_probe_fp32_fma.argtypes = [C.c_int32, P(C.c_double), P(C.c_float)]
    L.grx_last_transfer.argtypes = [P(C.c_size_t), P(C.c_size_t)]
    L.grx_trial_energies_noalloc.argtypes = [C.c_void_p, P(Trials), C.c_int32, C.c_int64, C.c_int64, C.c_int32,
                                             P(TrialEnergy), _u8p]
    L.grx_box_write_molecule.argtypes = [C.c_void_p, C.c_int32, C.c_size_t, _dp, _dp, P(C.c_size_t)]
    L.grx_box_remove_molecule.argtypes = [C.c_void_p, C.c_int32, C.c_size_t]
    L.grx_gcmc_run.argtypes = [P(C.c_void_p), C.c_int32, P(GcmcDesc), P(C.c_int32), C.c_uint64, C.c_int64,
                               C.c_int32, P(GcmcStats)]
    L.grx_gcmc_batch_create.argtypes = [P(C.c_void_p), C.c_int32, P(GcmcDesc), P(C.c_int32), C.c_int32,
                                        P(C.c_void_p)]
    L.grx_gcmc_batch_destroy.argtypes = [C.c_void_p]
    L.grx_gcmc_batch_set_step.argtypes = [C.c_void_p, C.c_uint64]
    L.grx_gcmc_batch_launch.argtypes = [C.c_void_p, C.c_int64, C.c_void_p]
    L.grx_gcmc_batch_run_graph.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_void_p]
    L.grx_gcmc_batch_stats.argtypes = [C.c_void_p, P(GcmcStats), P(C.c_uint64)]
    L.grx_gcmc_batch_reset_stats.argtypes = [C.c_void_p]
    L.grx_gcmc_batch_autotune.argtypes = [C.c_void_p, C.c_int64, P(C.c_int32), P(C.c_float)]
    L.grx_gcmc_batch_set_shape.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
    L.grx_gcmc_batch_get_shape.argtypes = [C.c_void_p, P(C.c_int32), P(C.c_int32)]
    L.grx_gcmc_batch_set_cluster.argtypes = [C.c_void_p, C.c_int32]
    L.grx_gcmc_batch_get_cluster.argtypes = [C.c_void_p, P(C.c_int32)]
    L.grx_arena_create.argtypes = [C.c_size_t, P(C.c_void_p)]
    L.grx_arena_destroy.argtypes = [C.c_void_p]
    L.grx_arena_usage.argtypes = [C.c_void_p, P(C.c_size_t), P(C.c_size_t), P(C.c_size_t)]
    L.grx_box_create_in.argtypes = [P(BoxDesc), C.c_void_p, P(C.c_void_p)]
    L.grx_box_footprint.argtypes = [P(BoxDesc), P(C.c_size_t)]
    L.grx_box_create_replica.argtypes = [C.c_void_p, P(C.c_void_p)]
    L.grx_box_set_voxel_lists.argtypes = [C.c_void_p, C.c_int32]
    L.grx_gcmc_batch_set_box_steps.argtypes = [C.c_void_p, P(C.c_uint64), P(C.c_int64)]
    L.grx_probe_df_functions.argtypes = [_dp, P(C.c_uint32), C.c_int64, _dp]
    L.grx_box_get_voxel_lists.argtypes = [C.c_void_p, P(C.c_int32), P(C.c_int32), P(C.c_int64)]
    L.grx_server_create.argtypes = [P(ServerConfig), C.c_void_p, P(C.c_void_p)]
    L.grx_server_destroy.argtypes = [C.c_void_p]
    L.grx_server_submit.argtypes = [C.c_void_p, P(JobDesc), P(C.c_uint64)]
    L.grx_server_progress.argtypes = [C.c_void_p, P(C.c_int32), P(C.c_int32)]
    L.grx_server_poll.argtypes = [C.c_void_p, P(JobResult), C.c_int32, P(C.c_int32)]
    L.grx_server_time.argtypes = [C.c_void_p, P(C.c_double)]
    L.grx_server_launch_count.argtypes = [C.c_void_p, P(C.c_uint64)]
    _lib = L
    return L


def check(status, what=""):
    if status != 0:
        L = load()
        raise GrxError(f"{what}: {L.grx_status_string(status).decode()} ({L.grx_last_error().decode()})")


def _d(a):
    return a.ctypes.data_as(_dp)


def _sz(a):
    return a.ctypes.data_as(_szp)


def geometry_from_system(system):
    """Boxsize geometry: inverse, volume, cubic flag (maths.cuh inverse_matrix /
    matrix_determinant, read_data.cpp:2020-2025) and the LAMMPS reciprocal cutoff
    (read_data.cpp:664-687)."""
    g = BoxGeometry()
    cell = np.array(system["cell"], dtype=np.float64)
    x = cell
    m11, m21, m31 = x[0], x[3], x[6]
    m12, m22, m32 = x[1], x[4], x[7]
    m13, m23, m33 = x[2], x[5], x[8]
    det = m11 * (m22 * m33 - m23 * m32) - m12 * (m21 * m33 - m23 * m31) + m13 * (m21 * m32 - m22 * m31)
    inv = [0.0] * 9
    inv[0] = (m22 * m33 - m32 * m23) / det
    inv[3] = -(m21 * m33 - m31 * m23) / det
    inv[6] = (m21 * m32 - m31 * m22) / det
    inv[1] = -(m12 * m33 - m32 * m13) / det
    inv[4] = (m11 * m33 - m31 * m13) / det
    inv[7] = -(m11 * m32 - m31 * m12) / det
    inv[2] = (m12 * m23 - m22 * m13) / det
    inv[5] = -(m11 * m23 - m21 * m13) / det
    inv[8] = (m11 * m22 - m21 * m12) / det
    for i in range(9):
        g.cell[i] = float(cell[i])
        g.inverse_cell[i] = inv[i]
    g.volume = det
    g.cubic = 0 if (abs(x[3]) + abs(x[6]) + abs(x[7])) > 1e-10 else 1
    g.use_lammps_ewald = int(system.get("use_lammps_ewald", 1))
    for i in range(3):
        g.kmax[i] = int(system["kmax"][i])
    g.alpha = float(system["alpha"])
    g.prefactor = float(system.get("prefactor", 138935.483496))
    if system.get("reciprocal_cutoff") is not None:
        g.reciprocal_cutoff = float(system["reciprocal_cutoff"])
    else:
        two_pi = 2 * 3.14159265358979323846
        lx, ly, lz = x[0], x[4], x[8]
        kvx = g.kmax[0] * (two_pi / lx)
        kvy = g.kmax[0] * (two_pi * (-0.0) / lx / ly) + g.kmax[1] * (two_pi / ly)
        kvz = g.kmax[0] * 0.0 + g.kmax[1] * 0.0 + g.kmax[2] * (two_pi / lz)
        g.reciprocal_cutoff = max(kvx * kvx, kvy * kvy, kvz * kvz) * 1.00001
    return g


def box_desc(system, capacity=None):
    """grx_box_desc of a system dict; returns (desc, keep) with `keep` owning the
    force-field arrays the descriptor points to."""
    nt = int(system["ntypes"])
    eps = np.ascontiguousarray(system["epsilon"], dtype=np.float64)
    sig = np.ascontiguousarray(system["sigma"], dtype=np.float64)
    shift = np.ascontiguousarray(system["shift"], dtype=np.float64)
    d = BoxDesc()
    d.geometry = geometry_from_system(system)
    ff = ForceField()
    ff.ntypes = nt
    # 12-6-4 mode (UseLJ1264): epsilon / sigma / z / c10 hold C12 / C6 / C4 / C10 per type pair
    ff.use_1264 = int(system.get("use_1264", 0))
    ff.epsilon, ff.sigma, ff.shift = _d(eps), _d(sig), _d(shift)
    z = np.ascontiguousarray(system.get("z", np.zeros(nt * nt)), dtype=np.float64)
    c10 = np.ascontiguousarray(system.get("c10", np.zeros(nt * nt)), dtype=np.float64)
    ff.z = _d(z) if ff.use_1264 else _dp()
    ff.c10 = _d(c10) if ff.use_1264 else _dp()
    ff.no_charges = int(system.get("no_charges", 0))
    ff.vdw_real_bias = int(system.get("vdw_real_bias", 1))
    ff.overlap_criteria = float(system.get("overlap_criteria", 1e6))
    ff.cutoff_vdw_sq = float(system["cutoff_vdw"]) ** 2
    ff.cutoff_coul_sq = float(system["cutoff_coul"]) ** 2
    d.forcefield = ff
    cs = system["comp_start"]
    ncomp = len(cs) - 1
    d.ncomponents = ncomp
    d.nhost_components = int(system["nhost"])
    for c in range(ncomp):
        n = cs[c + 1] - cs[c]
        ms = int(system["molsize"][c])
        cap = capacity[c] if capacity is not None else max(n, ms)
        d.capacity[c] = max(cap, ms)
        d.molsize[c] = ms
    return d, (eps, sig, shift, z, c10)


def component_atoms(system, c):
    """grx_atoms of component c; returns (atoms, keep). An empty adsorbate component
    stores its molecule template."""
    s = system
    a0, a1 = s["comp_start"][c], s["comp_start"][c + 1]
    n = a1 - a0
    ms = int(s["molsize"][c])
    pos = np.ascontiguousarray(np.asarray(s["pos"], dtype=np.float64)[a0:a1]).reshape(-1, 3)
    q = np.ascontiguousarray(np.asarray(s["charge"], dtype=np.float64)[a0:a1])
    ty = np.ascontiguousarray(np.asarray(s["type"])[a0:a1], dtype=np.uint64)
    mol = np.ascontiguousarray(np.asarray(s["molid"])[a0:a1], dtype=np.uint64)
    sc = np.ascontiguousarray(np.asarray(s["scale"], dtype=np.float64)[a0:a1])
    scc = np.ascontiguousarray(np.asarray(s["scale_coul"], dtype=np.float64)[a0:a1])
    stored = n
    if n == 0 and c >= int(s["nhost"]) and c in s.get("templates", {}):
        tm = s["templates"][c]
        pos = np.ascontiguousarray(tm["pos"], dtype=np.float64)
        q = np.ascontiguousarray(tm["charge"], dtype=np.float64)
        ty = np.ascontiguousarray(tm["type"], dtype=np.uint64)
        mol = np.zeros(ms, dtype=np.uint64)
        sc = np.ones(ms)
        scc = np.ones(ms)
        stored = ms
    pos = np.ascontiguousarray(pos.reshape(-1))
    return Atoms(_d(pos), _d(sc), _d(q), _d(scc), _sz(ty), _sz(mol), n, stored), (pos, q, ty, mol, sc, scc)


class Box:
    """Device-resident box (one grx_box)."""

    def __init__(self, system, capacity=None, arena=None):
        L = load()
        self.L = L
        self.system = system
        d, self._keep = box_desc(system, capacity)
        self.desc = d
        self.ncomp = d.ncomponents
        self.nhost = int(system["nhost"])
        h = C.c_void_p()
        if arena is None:
            check(L.grx_box_create(C.byref(d), C.byref(h)), "grx_box_create")
        else:
            check(L.grx_box_create_in(C.byref(d), arena.h, C.byref(h)), "grx_box_create_in")
        self.h = h
        for c in range(self.ncomp):
            self.set_component(c)

    def replica(self):
        """A new box sharing this box's framework (grx_box_create_replica)."""
        r = Box.__new__(Box)
        r.L, r.system, r.desc, r._keep = self.L, self.system, self.desc, self._keep
        r.ncomp, r.nhost = self.ncomp, self.nhost
        h = C.c_void_p()
        check(self.L.grx_box_create_replica(self.h, C.byref(h)), "grx_box_create_replica")
        r.h = h
        r.parent = self
        return r

    def close(self):
        if getattr(self, "h", None):
            self.L.grx_box_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_component(self, c, rigid=None):
        a, keep = component_atoms(self.system, c)
        if rigid is None:
            rigid = 1 if c >= self.nhost else 0
        check(self.L.grx_box_set_component(self.h, c, C.byref(a), int(rigid)), "grx_box_set_component")

    def component_size(self, c):
        n = C.c_size_t()
        check(self.L.grx_box_get_component_size(self.h, c, C.byref(n)), "grx_box_get_component_size")
        return n.value

    def positions(self, c, n=None):
        """Atom positions of component c in storage order (caller order for hosts)."""
        n = self.component_size(c) if n is None else n
        out = np.zeros(3 * n)
        check(self.L.grx_box_get_positions(self.h, c, _d(out), n), "grx_box_get_positions")
        return out.reshape(-1, 3)

    def write_molecule(self, c, mol, pos, charge, types):
        """Write adsorbate molecule `mol` of component c (mol == count appends)."""
        p = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        q = np.ascontiguousarray(charge, dtype=np.float64)
        t = np.ascontiguousarray(types, dtype=np.uint64)
        check(self.L.grx_box_write_molecule(self.h, c, mol, _d(p), _d(q), _sz(t)), "grx_box_write_molecule")

    def remove_molecule(self, c, mol):
        """Remove adsorbate molecule `mol`; the last molecule takes its slot."""
        check(self.L.grx_box_remove_molecule(self.h, c, mol), "grx_box_remove_molecule")

    # --- Ewald ---------------------------------------------------------
    def ewald_sizes(self):
        nv, na = C.c_int64(), C.c_int64()
        check(self.L.grx_ewald_sizes(self.h, C.byref(nv), C.byref(na)), "grx_ewald_sizes")
        return nv.value, na.value

    def ewald_total(self):
        out = np.zeros(8)
        check(self.L.grx_ewald_total(self.h, _d(out)), "grx_ewald_total")
        return out

    def structure_factors(self):
        nv, _ = self.ewald_sizes()
        a, b, t = np.zeros(2 * nv), np.zeros(2 * nv), np.zeros(2 * nv)
        check(self.L.grx_ewald_get_structure_factors(self.h, _d(a), _d(b), _d(t)), "get S(k)")
        return a, b, t

    def set_structure_factors(self, s_fw, s_ads):
        s_fw = np.ascontiguousarray(s_fw, dtype=np.float64)
        s_ads = np.ascontiguousarray(s_ads, dtype=np.float64)
        check(self.L.grx_ewald_set_structure_factors(self.h, _d(s_fw), _d(s_ads)), "set S(k)")

    def ewald_delta(self, comp, move_type, old_pos, old_qs, new_pos, new_qs, scale_coul_new=1.0):
        op = np.ascontiguousarray(old_pos, dtype=np.float64).reshape(-1)
        oq = np.ascontiguousarray(old_qs, dtype=np.float64)
        npos = np.ascontiguousarray(new_pos, dtype=np.float64).reshape(-1)
        nq = np.ascontiguousarray(new_qs, dtype=np.float64)
        out = np.zeros(2)
        check(self.L.grx_ewald_delta(self.h, comp, move_type, _d(op), _d(oq), len(oq), _d(npos), _d(nq), len(nq),
                                     scale_coul_new, _d(out)), "grx_ewald_delta")
        return out

    def ewald_delta_lambda(self, comp, pos, charge, scale_coul_old, scale_coul_new, use_staged=False):
        """Fourier delta of a lambda change at fixed positions (CB/CFC)."""
        p = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        q = np.ascontiguousarray(charge, dtype=np.float64)
        out = np.zeros(2)
        check(self.L.grx_ewald_delta_lambda(self.h, comp, _d(p), _d(q), len(q), scale_coul_old, scale_coul_new,
                                            int(bool(use_staged)), _d(out)), "grx_ewald_delta_lambda")
        return out

    def ewald_delta_identity_swap(self, old_comp, new_comp, old_pos, old_qs, new_pos, new_qs):
        """Fourier delta of an identity swap (old_comp molecule out, new_comp molecule in)."""
        op = np.ascontiguousarray(old_pos, dtype=np.float64).reshape(-1)
        oq = np.ascontiguousarray(old_qs, dtype=np.float64)
        npos = np.ascontiguousarray(new_pos, dtype=np.float64).reshape(-1)
        nq = np.ascontiguousarray(new_qs, dtype=np.float64)
        out = np.zeros(2)
        check(self.L.grx_ewald_delta_identity_swap(self.h, old_comp, new_comp, _d(op), _d(oq), len(oq), _d(npos),
                                                   _d(nq), len(nq), _d(out)), "grx_ewald_delta_identity_swap")
        return out

    def ewald_commit(self, comp):
        check(self.L.grx_ewald_commit(self.h, comp), "grx_ewald_commit")

    def exclusion(self, comp):
        a, b = C.c_double(), C.c_double()
        check(self.L.grx_box_get_exclusion(self.h, comp, C.byref(a), C.byref(b)), "exclusion")
        return a.value, b.value

    def total_energy(self, with_overlap=False):
        e = Energy()
        if with_overlap:
            f = np.zeros(1, dtype=np.uint8)
            check(self.L.grx_total_energy_overlap(self.h, C.byref(e), f.ctypes.data_as(_u8p)),
                  "grx_total_energy_overlap")
            return {n: getattr(e, n) for n, _ in Energy._fields_}, int(f[0])
        check(self.L.grx_total_energy(self.h, C.byref(e)), "grx_total_energy")
        return {n: getattr(e, n) for n, _ in Energy._fields_}

    # --- pair energies -------------------------------------------------
    def trial_energies(self, pos, charge, types, molid, ntrials, chainsize, component, prec=GRX_FP64,
                       scale=None, scale_coul=None, excl_comp=-1, excl_molid=-1):
        nb = ntrials * chainsize
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        charge = np.ascontiguousarray(charge, dtype=np.float64)
        types = np.ascontiguousarray(types, dtype=np.uint64)
        scale = np.ones(nb) if scale is None else np.ascontiguousarray(scale, dtype=np.float64)
        scale_coul = np.ones(nb) if scale_coul is None else np.ascontiguousarray(scale_coul, dtype=np.float64)
        t = Trials(_d(pos), _d(scale), _d(charge), _d(scale_coul), _sz(types), molid, ntrials, chainsize)
        out = (TrialEnergy * ntrials)()
        flag = np.zeros(ntrials, dtype=np.uint8)
        check(self.L.grx_trial_energies(self.h, C.byref(t), component, excl_comp, excl_molid, prec, out,
                                        flag.ctypes.data_as(_u8p)), "grx_trial_energies")
        e = np.array([[o.hg_vdw, o.hg_real, o.gg_vdw, o.gg_real] for o in out])
        return e, flag

    def trial_energies_noalloc(self, pos, charge, types, molid, ntrials, chainsize, component, prec=GRX_FP64,
                               excl_comp=-1, excl_molid=-1, scale=None, scale_coul=None):
        """grx_trial_energies_noalloc: the same call with its scratch in a fixed device array.
        charge, scale or scale_coul None pass a null pointer (charges 0, scalings 1)."""
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        types = np.ascontiguousarray(types, dtype=np.uint64)
        keep = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else None
                for a in (scale, charge, scale_coul)]
        ptr = [_d(a) if a is not None else None for a in keep]
        t = Trials(_d(pos), ptr[0], ptr[1], ptr[2], _sz(types), molid, ntrials, chainsize)
        out = (TrialEnergy * ntrials)()
        flag = np.zeros(ntrials, dtype=np.uint8)
        st = self.L.grx_trial_energies_noalloc(self.h, C.byref(t), component, excl_comp, excl_molid, prec, out,
                                               flag.ctypes.data_as(_u8p))
        check(st, "grx_trial_energies_noalloc")
        e = np.array([[o.hg_vdw, o.hg_real, o.gg_vdw, o.gg_real] for o in out])
        return e, flag

    def single_body(self, old, new, component, do_new=1, do_old=1, prec=GRX_FP64):
        """old/new: dict(pos, charge, type, molid[, scale, scale_coul])."""
        keep = []

        def mk(m):
            ms = len(m["charge"])
            pos = np.ascontiguousarray(m["pos"], dtype=np.float64).reshape(-1)
            q = np.ascontiguousarray(m["charge"], dtype=np.float64)
            ty = np.ascontiguousarray(m["type"], dtype=np.uint64)
            sc = np.ascontiguousarray(m.get("scale", np.ones(ms)), dtype=np.float64)
            scc = np.ascontiguousarray(m.get("scale_coul", np.ones(ms)), dtype=np.float64)
            keep.extend([pos, q, ty, sc, scc])
            return Trials(_d(pos), _d(sc), _d(q), _d(scc), _sz(ty), int(m["molid"]), 1, ms)
        to, tn = mk(old), mk(new)
        out = np.zeros(6)
        flag = np.zeros(1, dtype=np.uint8)
        check(self.L.grx_single_body_energy(self.h, C.byref(to), C.byref(tn), component, do_new, do_old, prec,
                                            _d(out), flag.ctypes.data_as(_u8p)), "grx_single_body_energy")
        return out, int(flag[0])

    # --- CBMC ----------------------------------------------------------
    def widom(self, desc, first_move, n, prec=GRX_MIXED, out=None):
        res = np.zeros(n, dtype=WIDOM_RESULT_DTYPE) if out is None else out
        check(self.L.grx_widom_insertions(self.h, C.byref(desc), first_move, n, prec,
                                          C.c_void_p(res.ctypes.data)), "grx_widom_insertions")
        return res

    def widom_async(self, desc, first_move, n, prec, dev_ptr):
        check(self.L.grx_widom_insertions_async(self.h, C.byref(desc), first_move, n, prec, C.c_void_p(dev_ptr)),
              "grx_widom_insertions_async")

    def set_stream(self, stream_ptr):
        check(self.L.grx_box_set_stream(self.h, C.c_void_p(stream_ptr)), "grx_box_set_stream")

    def set_voxel_lists(self, on):
        """grx_box_set_voxel_lists: 1 builds the framework's voxel candidate lists (when they
        fit), 0 frees them (the tile path)."""
        check(self.L.grx_box_set_voxel_lists(self.h, int(on)), "grx_box_set_voxel_lists")

    def voxel_lists(self):
        """(on, voxels per axis, list entries) of grx_box_get_voxel_lists."""
        on = C.c_int32()
        dims = (C.c_int32 * 3)()
        n = C.c_int64()
        check(self.L.grx_box_get_voxel_lists(self.h, C.byref(on), dims, C.byref(n)), "grx_box_get_voxel_lists")
        return bool(on.value), tuple(dims), int(n.value)


class Arena:
    """grx_arena: one reserved region of device memory that boxes are carved from."""

    def __init__(self, nbytes):
        self.L = load()
        h = C.c_void_p()
        check(self.L.grx_arena_create(int(nbytes), C.byref(h)), "grx_arena_create")
        self.h = h

    def usage(self):
        u, lf, pk = C.c_size_t(), C.c_size_t(), C.c_size_t()
        check(self.L.grx_arena_usage(self.h, C.byref(u), C.byref(lf), C.byref(pk)), "grx_arena_usage")
        return u.value, lf.value, pk.value

    def close(self):
        if getattr(self, "h", None):
            check(self.L.grx_arena_destroy(self.h), "grx_arena_destroy")
            self.h = None


def box_footprint(system, capacity=None):
    d, keep = box_desc(system, capacity)
    n = C.c_size_t()
    check(load().grx_box_footprint(C.byref(d), C.byref(n)), "grx_box_footprint")
    return n.value


class Server:
    """grx_server: continuous-batching Widom / GCMC job server."""

    def __init__(self, hbm_budget_bytes, max_resident, prec=GRX_MIXED, widom_slice=0, gcmc_slice=0,
                 cluster_atoms=0, gcmc_batching=0):
        self.L = load()
        cfg = ServerConfig(int(hbm_budget_bytes), int(max_resident), int(prec), int(widom_slice), int(gcmc_slice),
                           int(cluster_atoms), int(gcmc_batching), 0)
        h = C.c_void_p()
        check(self.L.grx_server_create(C.byref(cfg), None, C.byref(h)), "grx_server_create")
        self.h = h

    def submit(self, system, capacity, kind, widom=None, insertions=0, gcmc=None, steps=0, tag=0):
        """Copy one job (box + work) into the server's queue; returns its id."""
        d, keep_d = box_desc(system, capacity)
        ncomp = d.ncomponents
        atoms = (Atoms * ncomp)()
        keep = [keep_d]
        for c in range(ncomp):
            a, k = component_atoms(system, c)
            atoms[c] = a
            keep.append(k)
        jd = JobDesc()
        jd.kind = kind
        jd.box = C.pointer(d)
        jd.atoms = atoms
        jd.rigid = C.POINTER(C.c_int32)()
        if kind == JOB_WIDOM:
            jd.widom = widom
            jd.widom_insertions = int(insertions)
        else:
            gl = list(gcmc) if isinstance(gcmc, (list, tuple)) else [gcmc]
            arr = (GcmcDesc * len(gl))(*gl)
            keep.append(arr)
            jd.gcmc = arr
            jd.ncomp_moved = len(gl)
            jd.gcmc_steps = int(steps)
        jd.tag = int(tag)
        jid = C.c_uint64()
        check(self.L.grx_server_submit(self.h, C.byref(jd), C.byref(jid)), "grx_server_submit")
        return jid.value

    def progress(self):
        r, p = C.c_int32(), C.c_int32()
        check(self.L.grx_server_progress(self.h, C.byref(r), C.byref(p)), "grx_server_progress")
        return r.value, p.value

    def poll(self, max_results=256):
        out = (JobResult * max_results)()
        n = C.c_int32()
        check(self.L.grx_server_poll(self.h, out, max_results, C.byref(n)), "grx_server_poll")
        return [out[i] for i in range(n.value)]

    def time(self):
        t = C.c_double()
        check(self.L.grx_server_time(self.h, C.byref(t)), "grx_server_time")
        return t.value

    def launches(self):
        n = C.c_uint64()
        check(self.L.grx_server_launch_count(self.h, C.byref(n)), "grx_server_launch_count")
        return n.value

    def close(self):
        if getattr(self, "h", None):
            self.L.grx_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def beta_from_temperature(T):
    """1/(kB T) in internal units, the expression of Setup_Box_Temperature_Pressure
    (fxn_main.h:117) with the Units constants of data_struct.h:54-64."""
    kB, mass, length, time = 1.380649e-23, 1.6605402e-27, 1e-10, 1e-12
    return 1.0 / (kB / (mass * pow(length, 2) / pow(time, 2)) * T)


def widom_desc(system, component, ntrials=10, norient=10, temperature=None, seed=42, stream=0,
               scale=1.0, scale_coul=1.0, tail_delta=0.0):
    T = temperature if temperature is not None else system.get("temperature", 300.0)
    d = WidomDesc()
    d.component = component
    d.ntrials = ntrials
    d.norient = norient
    d.scale = scale
    d.scale_coul = scale_coul
    d.beta = beta_from_temperature(T)
    d.tail_delta = tail_delta
    d.seed = seed
    d.stream = stream
    return d


def gcmc_desc(component, ntrials=10, norient=10, p_translation=0.25, p_rotation=0.5, p_reinsertion=None, p_swap=1.0,
              max_translation=1.0, max_rotation=0.5, temperature=300.0, pressure_pa=1e5, fugacity_coeff=1.0,
              mol_fraction=1.0, ideal_rosenbluth=1.0, tail_insert=0.0, seed=42, stream=0, p_identity_swap=0.0):
    """GCMC move mix of one box; probabilities are cumulative as in Move_Statistics,
    pressure in Pa converted to internal units (fxn_main.h:120)."""
    d = GcmcDesc()
    d.component, d.ntrials, d.norient = component, ntrials, norient
    d.p_translation, d.p_rotation, d.p_swap = p_translation, p_rotation, p_swap
    d.p_reinsertion = p_rotation if p_reinsertion is None else p_reinsertion
    for k in range(3):
        d.max_translation[k] = max_translation
        d.max_rotation[k] = max_rotation
    d.beta = beta_from_temperature(temperature)
    d.pressure = pressure_pa / 1.6605402e7
    d.fugacity_coeff, d.mol_fraction, d.ideal_rosenbluth = fugacity_coeff, mol_fraction, ideal_rosenbluth
    d.tail_insert = tail_insert
    d.seed, d.stream = seed, stream
    d.p_identity_swap = p_identity_swap
    return d


def _moved(descs, ncomp_moved, nboxes):
    flat = [d for group in descs for d in (group if isinstance(group, (list, tuple)) else [group])]
    if ncomp_moved is None:
        ncomp_moved = [len(g) if isinstance(g, (list, tuple)) else 1 for g in descs]
    assert len(ncomp_moved) == nboxes and sum(ncomp_moved) == len(flat)
    return flat, (C.c_int32 * nboxes)(*ncomp_moved)


def gcmc_run(boxes, descs, first_step, nsteps, prec=GRX_MIXED, ncomp_moved=None):
    """Run nsteps GCMC moves on every box in one persistent launch. descs: one GcmcDesc
    per box, or a list of them for a box that moves several components. Returns one
    GcmcStats per entry (flat, box-major)."""
    L = load()
    n = len(boxes)
    flat, nm = _moved(descs, ncomp_moved, n)
    hs = (C.c_void_p * n)(*[b.h for b in boxes])
    ds = (GcmcDesc * len(flat))(*flat)
    st = (GcmcStats * len(flat))()
    check(L.grx_gcmc_run(hs, n, ds, nm, first_step, nsteps, prec, st), "grx_gcmc_run")
    return list(st)


class GcmcBatch:
    """grx_gcmc_batch: a prepared persistent GCMC launch (device step counter,
    accumulated statistics, CUDA-graph replay, autotuner)."""

    def __init__(self, boxes, descs, prec=GRX_MIXED, ncomp_moved=None):
        self.L = load()
        n = len(boxes)
        self.boxes = boxes
        flat, nm = _moved(descs, ncomp_moved, n)
        self.nentries = len(flat)
        hs = (C.c_void_p * n)(*[b.h for b in boxes])
        ds = (GcmcDesc * len(flat))(*flat)
        h = C.c_void_p()
        check(self.L.grx_gcmc_batch_create(hs, n, ds, nm, prec, C.byref(h)), "grx_gcmc_batch_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.grx_gcmc_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_step(self, step):
        check(self.L.grx_gcmc_batch_set_step(self.h, step), "grx_gcmc_batch_set_step")

    def launch(self, nsteps, stream=None):
        check(self.L.grx_gcmc_batch_launch(self.h, nsteps, C.c_void_p(stream or 0)), "grx_gcmc_batch_launch")

    def set_box_steps(self, next_move, nsteps=None):
        """grx_gcmc_batch_set_box_steps: per box, the next Philox move index and the most
        steps it takes per launch (None: every step of the launch)."""
        nm = np.ascontiguousarray(next_move, dtype=np.uint64)
        ns = None if nsteps is None else np.ascontiguousarray(nsteps, dtype=np.int64)
        check(self.L.grx_gcmc_batch_set_box_steps(self.h, nm.ctypes.data_as(C.POINTER(C.c_uint64)),
                                                  ns.ctypes.data_as(C.POINTER(C.c_int64)) if ns is not None
                                                  else C.POINTER(C.c_int64)()), "grx_gcmc_batch_set_box_steps")

    def run_graph(self, nsteps, nlaunch, stream=None):
        check(self.L.grx_gcmc_batch_run_graph(self.h, nsteps, nlaunch, C.c_void_p(stream or 0)),
              "grx_gcmc_batch_run_graph")

    def stats(self):
        st = (GcmcStats * self.nentries)()
        nxt = C.c_uint64()
        check(self.L.grx_gcmc_batch_stats(self.h, st, C.byref(nxt)), "grx_gcmc_batch_stats")
        return list(st), nxt.value

    def reset_stats(self):
        check(self.L.grx_gcmc_batch_reset_stats(self.h), "grx_gcmc_batch_reset_stats")

    def set_shape(self, nwarps, chunk_mult):
        check(self.L.grx_gcmc_batch_set_shape(self.h, nwarps, chunk_mult), "grx_gcmc_batch_set_shape")

    def shape(self):
        """(warps per box, work items per warp of a bead pass)."""
        w, m = C.c_int32(), C.c_int32()
        check(self.L.grx_gcmc_batch_get_shape(self.h, C.byref(w), C.byref(m)), "grx_gcmc_batch_get_shape")
        return w.value, m.value

    def set_cluster(self, cluster):
        """CTAs per box (1, or 2 / 4 / 8 with 24 warps per block): one chain per
        thread-block cluster."""
        check(self.L.grx_gcmc_batch_set_cluster(self.h, cluster), "grx_gcmc_batch_set_cluster")

    def cluster(self):
        c = C.c_int32()
        check(self.L.grx_gcmc_batch_get_cluster(self.h, C.byref(c)), "grx_gcmc_batch_get_cluster")
        return c.value

    def autotune(self, nsteps):
        """Times the GCMC_TUNE_CANDIDATES launch shapes on real steps (forward and
        reverse sweep, ranked by trial energies per second), then, when the boxes leave
        SMs idle, the best shape against thread-block clusters, and keeps the best:
        returns ((nwarps, chunk_mult), mean ms per plain candidate probe); the cluster
        size kept is cluster()."""
        ch = C.c_int32()
        ms = (C.c_float * GCMC_TUNE_CANDIDATES)()
        check(self.L.grx_gcmc_batch_autotune(self.h, nsteps, C.byref(ch), ms), "grx_gcmc_batch_autotune")
        rest = ch.value % 10000
        return (rest // 100, rest % 100), list(ms)


def cbmc_select(logw, seed, stream, move, word):
    L = load()
    lw = np.ascontiguousarray(logw, dtype=np.float64)
    sel = C.c_int32()
    s = C.c_double()
    check(L.grx_cbmc_select(_d(lw), len(lw), seed, stream, move, word, C.byref(sel), C.byref(s)), "grx_cbmc_select")
    return sel.value, s.value


def launch_count():
    return load().grx_launch_count()


def last_transfer():
    """(h2d, d2h) bytes of this thread's last grx_gcmc_run."""
    a, b = C.c_size_t(), C.c_size_t()
    check(load().grx_last_transfer(C.byref(a), C.byref(b)), "grx_last_transfer")
    return a.value, b.value


def probe_fp32_fma(iters=20000):
    """Measured FP32 FMA throughput of the device in TFLOP/s (grx_probe_fp32_fma)."""
    t, ms = C.c_double(), C.c_float()
    check(load().grx_probe_fp32_fma(iters, C.byref(t), C.byref(ms)), "grx_probe_fp32_fma")
    return t.value


def probe_df_functions(v, words):
    """grx_probe_df_functions: (sin 2 pi v, cos 2 pi v, rotated (1, 0.5, -0.25)) per value."""
    v = np.ascontiguousarray(v, dtype=np.float64)
    w = np.ascontiguousarray(words, dtype=np.uint32).reshape(-1)
    out = np.zeros(5 * len(v))
    check(load().grx_probe_df_functions(_d(v), w.ctypes.data_as(C.POINTER(C.c_uint32)), len(v), _d(out)),
          "grx_probe_df_functions")
    return out.reshape(-1, 5)
