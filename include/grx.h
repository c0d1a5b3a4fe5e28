/*
 * grx.h -- C ABI of the GB300 CBMC trial-energy engine (libgrx.so).
 *
 * The engine replaces the bodies of gRASPA's energy calls on the Monte Carlo hot
 * path: the CBMC trial pair energies, the single-molecule move delta, the Ewald
 * Fourier-space delta and structure-factor commit, Rosenbluth trial selection,
 * and the FP64 totals used for drift checks. Each entry point below names the
 * gRASPA interface (file:line in src_clean/) whose contract it keeps.
 *
 * Conventions (the reference's):
 *   - energies in internal units (10 J/mol); epsilon tables already divided by
 *     1.20272430057 (read_data.cpp:1200); cutoffs passed SQUARED
 *     (ForceField.CutOffVDW / CutOffCoul, data_struct.h:850-851);
 *   - cell matrices column-major as Boxsize.Cell (read_data.cpp:1545-1547);
 *   - positions are double3 triples (Atoms.pos), types and molecule ids size_t.
 *
 * Memory: every pointer argument may be host or device memory (CUDA unified
 * addressing; the library copies with cudaMemcpyDefault). The library owns all
 * device allocations of a box from grx_box_create until grx_box_destroy.
 * Errors: every call returns a grx_status; nothing calls exit() or traps.
 * Threading: a box must not be used by two host threads at once; distinct boxes
 * are independent. All work of a box is issued on the box's CUDA stream
 * (grx_box_set_stream); calls return after that work has finished unless the
 * name ends in _async.
 */
#ifndef GRX_H
#define GRX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t grx_status;
#define GRX_OK 0
#define GRX_ERR_INVALID_ARG 1
#define GRX_ERR_CUDA 2
#define GRX_ERR_OUT_OF_MEMORY 3
#define GRX_ERR_TIMEOUT 4
#define GRX_ERR_CAPACITY 5
#define GRX_ERR_NO_DEVICE 6
#define GRX_ERR_UNSUPPORTED 7

#define GRX_MAX_COMPONENTS 8
#define GRX_MAX_TYPES 32
#define GRX_MAX_TRIAL_BEADS 256
#define GRX_MAX_MOLSIZE 64

/* Arithmetic of the pair and Ewald evaluation.
 *   GRX_FP64  : every operation in FP64 (the reference's arithmetic).
 *   GRX_MIXED : FP32 cutoff screening on split hi/lo coordinates (hi on a
 *               2^-12 A grid, so hi differences are exact); pairs inside the
 *               cutoff are compacted per warp and evaluated in double-float
 *               arithmetic on the FP32 pipe (LJ and the tabulated erfc(alpha r)/r
 *               of real-space Coulomb); per-trial sums in double-float, then
 *               FP64. The Ewald delta runs in double-float against temp*S(k)
 *               tables and S(k) is updated in FP64 (compensated). FP64 is kept
 *               for self / exclusion terms and exp(-beta dE). Boltzmann weights
 *               agree with FP64 to beta*|dE| <= 1e-6.
 *   GRX_FP32  : FP32 pair math with FP64 sums; fastest, error reported, not
 *               within 1e-6 for charged systems. */
typedef enum { GRX_FP64 = 0, GRX_MIXED = 1, GRX_FP32 = 2 } grx_precision;

/* Move types, numbered as gRASPA's MoveTypes (data_struct.h:20). */
enum {
  GRX_MOVE_TRANSLATION = 0,
  GRX_MOVE_ROTATION = 1,
  GRX_MOVE_SINGLE_INSERTION = 2,
  GRX_MOVE_SINGLE_DELETION = 3,
  GRX_MOVE_SPECIAL_ROTATION = 4,
  GRX_MOVE_INSERTION = 5,
  GRX_MOVE_DELETION = 6,
  GRX_MOVE_REINSERTION = 7,
  GRX_MOVE_CBCF_LAMBDACHANGE = 8,
  GRX_MOVE_CBCF_INSERTION = 9,
  GRX_MOVE_CBCF_DELETION = 10,
  GRX_MOVE_IDENTITY_SWAP = 11
};

typedef struct grx_box grx_box; /* opaque, device-resident state of one box */

/* Geometry + Ewald parameters of a box: the fields of Boxsize
 * (data_struct.h:865-886) that the path reads. */
typedef struct {
  double cell[9];
  double inverse_cell[9];
  double volume;
  int32_t cubic;
  int32_t use_lammps_ewald;
  int32_t kmax[3];
  int32_t pad_;
  double alpha;
  double prefactor;          /* 138935.483496 (read_data.cpp:611) */
  double reciprocal_cutoff;  /* Boxsize.ReciprocalCutOff */
} grx_box_geometry;

/* Force field: ForceField (data_struct.h:838-855); tables ntypes*ntypes. */
typedef struct {
  int32_t ntypes;
  int32_t use_1264;
  const double* epsilon;
  const double* sigma;
  const double* z;     /* may be NULL (zeros) */
  const double* shift;
  const double* c10;   /* may be NULL (zeros) */
  int32_t no_charges;
  int32_t vdw_real_bias;
  double overlap_criteria;
  double cutoff_vdw_sq;
  double cutoff_coul_sq;
} grx_forcefield;

typedef struct {
  grx_box_geometry geometry;
  grx_forcefield forcefield;
  int32_t ncomponents;        /* NComponents.x */
  int32_t nhost_components;   /* NComponents.y */
  size_t capacity[GRX_MAX_COMPONENTS];  /* Atoms.Allocate_size per component */
  size_t molsize[GRX_MAX_COMPONENTS];   /* Moleculesize per component */
} grx_box_desc;

/* Atoms of one component: Atoms (data_struct.h:788-799). */
typedef struct {
  const double* pos;        /* 3*n */
  const double* scale;
  const double* charge;
  const double* scale_coul;
  const size_t* type;
  const size_t* molid;
  size_t size;              /* live atoms (Atoms.size) */
  size_t n_stored;          /* atoms present in the arrays (>= size; an empty
                               component still stores its molecule template) */
} grx_atoms;

/* Trial beads of one CBMC step: Simulations.New after
 * get_random_trial_position / get_random_trial_orientation (mc_widom.h:122-303). */
typedef struct {
  const double* pos;        /* 3 * ntrials * chainsize */
  const double* scale;
  const double* charge;
  const double* scale_coul;
  const size_t* type;
  size_t molid;             /* NewMol.MolID[0] */
  size_t ntrials;
  size_t chainsize;
} grx_trials;

typedef struct {
  double hg_vdw, hg_real, gg_vdw, gg_real;
} grx_trial_energy;

typedef struct {
  double hh_vdw, hh_real, hg_vdw, hg_real, gg_vdw, gg_real;
  double hh_ewald, hg_ewald, gg_ewald;   /* Fourier - self - exclusion, per block */
} grx_energy;

/* One batched Widom / CBMC insertion job into a static box (insertion branch of
 * Insertion_Body, mc_swap_utilities.h:3-132, called by InsertionMove::WidomMove,
 * move_struct.h:90-95). */
typedef struct {
  int32_t component;        /* inserted adsorbate component */
  int32_t ntrials;          /* NumberWidomTrials */
  int32_t norient;          /* NumberWidomTrialsOrientations */
  int32_t pad_;
  double scale;             /* proposed_scale.x (1 for a full molecule) */
  double scale_coul;        /* proposed_scale.y */
  double beta;              /* 1/(kB T), internal units */
  double tail_delta;        /* TailCorrectionDifference of one insertion */
  uint64_t seed;            /* Philox4x32-10 key */
  uint32_t stream;          /* counter word 3 (box / job id) */
  uint32_t pad2_;
} grx_widom_desc;

typedef struct {
  double rosenbluth;
  double w_first;
  double w_chain;
  double e_first[4];        /* hg_vdw hg_real gg_vdw gg_real of the chosen first bead */
  double e_chain[4];
  double ewald[2];          /* {same - exclusion, 2*cross} */
  int64_t sel_first;        /* chosen first-bead trial (index into all trials) */
  int64_t sel_orient;
  int64_t n_ok_first;       /* trials without overlap */
  int64_t n_ok_orient;
  int32_t success;
  int32_t pad_;
} grx_widom_result;

/* ---- lifecycle ---------------------------------------------------------- */
const char* grx_status_string(grx_status s);
const char* grx_last_error(void);  /* detail of the last failing call (thread-local) */
grx_status grx_device_count(int32_t* n);

/* Allocates the device state of one box (replaces the per-box allocations of
 * fxn_main.h:46-113,163-280 / main.cpp:243-300). */
grx_status grx_box_create(const grx_box_desc* desc, grx_box** out);
grx_status grx_box_destroy(grx_box* box);   /* refused while the box has live replicas */
/* A replica: a second Markov chain of the same system that shares the parent's
 * framework atoms, tiles, Coulomb table, force-field tables, k vectors and framework
 * structure factor (read-only), and owns its adsorbates, S_ads and their tables. It
 * starts as a copy of the parent's adsorbates. Many replicas keep one copy of the
 * framework in L1/L2 instead of one per chain. The parent must have current structure
 * factors, and its framework components cannot change while replicas live. No
 * counterpart in the reference (one box per simulation). */
grx_status grx_box_create_replica(grx_box* parent, grx_box** out);

/* Voxel candidate lists of the framework (host) atoms: the cell is cut into voxels of
 * about 1.5-4 A and each voxel lists every host atom within the screening radius of any
 * point of the voxel, with its periodic image, the atoms inside the cutoff for the whole
 * voxel first. The pair engine then walks a bead's voxel list instead of culling the
 * framework's 32-atom tiles (the cutoff tests stay exact, so results change only in the
 * summation order). Built by default when the lists fit 32 MB and the cell is wider than
 * twice the list radius; mode 0 frees them (tile path), mode 1 rebuilds them. Refused on
 * a box with replicas (they share the lists). No counterpart in the reference (it tests
 * every framework atom per trial). get: on (0/1), voxels per axis, list entries. */
grx_status grx_box_set_voxel_lists(grx_box* box, int32_t mode);
grx_status grx_box_get_voxel_lists(grx_box* box, int32_t* on, int32_t* dims, int64_t* entries);

/* ---- device memory arena -------------------------------------------------- */
/* One reserved region of device memory that boxes are carved from by a host-side
 * first-fit allocator (256-byte granules). A box created in an arena takes every
 * device allocation from it and returns them at grx_box_destroy without cudaFree,
 * so retiring a box does not wait on the device; a box that does not fit fails with
 * GRX_ERR_OUT_OF_MEMORY and nothing allocated. No counterpart in the reference (it
 * sizes one simulation per process); it is the admission resource of the serving
 * loop. */
typedef struct grx_arena grx_arena;
grx_status grx_arena_create(size_t bytes, grx_arena** out);
grx_status grx_arena_destroy(grx_arena* arena);      /* every box in it destroyed first */
grx_status grx_arena_usage(grx_arena* arena, size_t* in_use, size_t* largest_free, size_t* peak);
grx_status grx_box_create_in(const grx_box_desc* desc, grx_arena* arena, grx_box** out);
/* Upper estimate of the device bytes a box of this description needs, including its
 * first scratch and Widom result buffers. The framework's voxel candidate lists (up to
 * 32 MB, grx_box_set_voxel_lists) come on top when the arena or device has room for
 * them; without room the box keeps the tile path, so this is the admission minimum. */
grx_status grx_box_footprint(const grx_box_desc* desc, size_t* bytes);
/* All later work of the box goes to this stream (cudaStream_t, NULL = default). */
grx_status grx_box_set_stream(grx_box* box, void* cuda_stream);

/* Uploads one component's atoms (the device copies of Simulations.d_a[comp],
 * fxn_main.h:46-113). For rigid components the FP64 exclusion constants are
 * computed from the first molecule (Calculate_Exclusion_Energy_Rigid,
 * ewald_preparation.h:351-366). */
grx_status grx_box_set_component(grx_box* box, int32_t comp, const grx_atoms* atoms,
                                 int32_t rigid);
grx_status grx_box_get_component_size(grx_box* box, int32_t comp, size_t* size);
grx_status grx_box_get_positions(grx_box* box, int32_t comp, double* pos_out, size_t n);
grx_status grx_box_get_exclusion(grx_box* box, int32_t comp, double* intra, double* self);
/* Write the atoms of adsorbate molecule `mol` (positions 3*molsize, charges, types;
 * every atom gets MolID = mol). mol equal to the current molecule count appends a
 * molecule: Update_insertion_data_Parallel (mc_utilities.h:191-234); a smaller mol
 * overwrites it in place: update_translation_position (mc_utilities.h:285-292). */
grx_status grx_box_write_molecule(grx_box* box, int32_t comp, size_t mol, const double* pos,
                                  const double* charge, const size_t* type);
/* Remove adsorbate molecule `mol`; the component's last molecule moves into its
 * slot and takes its MolID: Update_deletion_data_Parallel (mc_utilities.h:163-189). */
grx_status grx_box_remove_molecule(grx_box* box, int32_t comp, size_t mol);

/* ---- pair energies ------------------------------------------------------ */
/* Per-trial host-guest and guest-guest VDW + real Coulomb energies and overlap
 * flags: Calculate_Multiple_Trial_Energy_VDWReal (VDW_Coulomb.cu:1183-1352) plus
 * the per-trial block sums of Host_sum_Widom_HGGG_SEPARATE (mc_widom.h:42-87),
 * i.e. the pair part of CBMC_PairwiseInteractions (mc_widom.h:89-119). Atoms of
 * (component, trials->molid) and of (exclude_comp, exclude_molid) are skipped
 * (ExcludeList[0]); pass -1 for no exclusion. */
grx_status grx_trial_energies(grx_box* box, const grx_trials* trials, int32_t component,
                              int64_t exclude_comp, int64_t exclude_molid,
                              grx_precision prec, grx_trial_energy* out, uint8_t* overlap);

/* New-minus-old energy of one moved molecule split HH/HG/GG and the overlap flag
 * of the new configuration: Calculate_Single_Body_Energy_VDWReal
 * (VDW_Coulomb.cu:626-841) with the host sums of SingleBody_Calculation
 * (mc_single_particle.h:172-200). out6 = hh_vdw hh_real hg_vdw hg_real gg_vdw gg_real. */
grx_status grx_single_body_energy(grx_box* box, const grx_trials* old_mol,
                                  const grx_trials* new_mol, int32_t component,
                                  int32_t do_new, int32_t do_old, grx_precision prec,
                                  double* out6, uint8_t* overlap);

/* ---- Ewald -------------------------------------------------------------- */
/* Number of k slots, (kmax.x+1)(2kmax.y+1)(2kmax.z+1), and of active slots. */
grx_status grx_ewald_sizes(grx_box* box, int64_t* nvec, int64_t* nactive);
/* Builds the framework and adsorbate structure factors from the current atoms in
 * FP64 and returns the Fourier totals (Ewald_Total, ewald_preparation.h:5-259,
 * device form Ewald_TotalEnergy, Ewald_Energy_Functions.h:1272).
 * out8 = fourier_gg fourier_hh fourier_hg self_all self_host excl_all excl_host n_active */
grx_status grx_ewald_total(grx_box* box, double* out8);
/* Structure factors in the reference layout (Complex[nvec], re/im interleaved):
 * Boxsize.FrameworkEik / AdsorbateEik (Allocate_Copy_Ewald_Vector, fxn_main.h:235-280). */
grx_status grx_ewald_set_structure_factors(grx_box* box, const double* s_fw, const double* s_ads);
grx_status grx_ewald_get_structure_factors(grx_box* box, double* s_fw, double* s_ads,
                                           double* s_temp);
/* Fourier delta of one move: GPU_EwaldDifference_General
 * (Ewald_Energy_Functions.h:438-580) with Initialize_WaveVector_General (:162) and
 * Fourier_Ewald_Diff (:280). old/new atoms are the moved molecule before / after
 * (positions, charge*scaleCoul). Stages S_same + dS into the temporary vector.
 * out2 = {same-type delta minus rigid exclusion, 2 * cross-type delta}. */
grx_status grx_ewald_delta(grx_box* box, int32_t component, int32_t move_type,
                           const double* old_pos, const double* old_qs, size_t n_old,
                           const double* new_pos, const double* new_qs, size_t n_new,
                           double scale_coul_new, double* out2);
/* Fourier delta of a lambda change of one fractional molecule of an adsorbate
 * component at fixed positions: GPU_EwaldDifference_LambdaChange
 * (Ewald_Energy_Functions.h:764-789) with Fourier_Ewald_Diff_LambdaChange (:636-762).
 * charge holds the atoms' charges without lambda; the old atoms carry
 * scale_coul_old, the new ones scale_coul_new. use_staged != 0 starts from the staged
 * vector instead of the adsorbate S(k) (the second step of a CB/CFC deletion, :775-778).
 * Stages S + dS. out2 = {same-type delta - (ExclusionIntra + ExclusionAtom) *
 * (scale_coul_new^2 - scale_coul_old^2), 2 * cross-type delta}. The pair part of the
 * lambda change (Calculate_Single_Body_Energy_VDWReal_LambdaChange, VDW_Coulomb.cu:843-1009)
 * is grx_single_body_energy with the same positions and the old / new scales. */
grx_status grx_ewald_delta_lambda(grx_box* box, int32_t component, const double* pos, const double* charge,
                                  size_t n, double scale_coul_old, double scale_coul_new, int32_t use_staged,
                                  double* out2);
/* Fourier delta of an identity swap (GPU_EwaldDifference_IdentitySwap,
 * Ewald_Energy_Functions.h:582-634): the molecule of old_component (positions,
 * charge*scaleCoul) leaves, the molecule of new_component arrives; atoms of an uncharged
 * side do not enter. Stages S + dS. out2 = {same-type delta - ExclusionNew +
 * ExclusionOld (rigid, charged components), 2 * cross-type delta}. The pair part of the
 * new molecule is grx_trial_energies with the old molecule excluded (ExcludeList). */
grx_status grx_ewald_delta_identity_swap(grx_box* box, int32_t old_component, int32_t new_component,
                                         const double* old_pos, const double* old_qs, size_t n_old,
                                         const double* new_pos, const double* new_qs, size_t n_new,
                                         double* out2);
/* Accept: make the staged structure factor current (Update_Vector_Ewald,
 * Ewald_Energy_Functions.h:423-433). */
grx_status grx_ewald_commit(grx_box* box, int32_t component);

/* ---- totals ------------------------------------------------------------- */
/* FP64 totals for drift checks: Total_VDW_Coulomb_Energy (VDW_Coulomb.cu:1580)
 * + Ewald_TotalEnergy (Ewald_Energy_Functions.h:1272), split as MoveEnergy. */
grx_status grx_total_energy(grx_box* box, grx_energy* out);
/* The same totals and the overlap flag of TotalVDWRealCoulomb (VDW_Coulomb.cu:1385-1386):
 * set when a pair with an adsorbate atom has an LJ energy above the overlap criterion or
 * r^2 < 0.01 A^2 (the rejection test of VolumeMove, mc_box.h:247-252). */
grx_status grx_total_energy_overlap(grx_box* box, grx_energy* out, uint8_t* overlap);

/* ---- CBMC --------------------------------------------------------------- */
/* Rosenbluth selection of SelectTrialPosition (mc_widom.h:14-39) with the
 * uniform drawn from the engine's Philox stream (seed, stream, move, slot 2048,
 * word). Returns the selected index and the unshifted weight sum. */
grx_status grx_cbmc_select(const double* logw, int32_t n, uint64_t seed, uint32_t stream,
                           uint64_t move, int32_t word, int32_t* selected, double* sum);

/* Batched CBMC Widom insertions into a static box, fully on the device: trial
 * positions, pair energies, Rosenbluth selection, orientations, pair energies,
 * selection and the Ewald delta of the chosen configuration, one result per
 * insertion (Widom_Move_FirstBead_PARTIAL + Widom_Move_Chain_PARTIAL,
 * mc_widom.h:385-614, and Insertion_Body's Ewald/tail factors,
 * mc_swap_utilities.h:94-108). Insertion i uses Philox move index first_move+i.
 * Requires current structure factors (grx_ewald_total or _set_). */
grx_status grx_widom_insertions(grx_box* box, const grx_widom_desc* desc,
                                uint64_t first_move, size_t n, grx_precision prec,
                                grx_widom_result* results);
/* Same, asynchronous on the box stream; `results` must be device memory. */
grx_status grx_widom_insertions_async(grx_box* box, const grx_widom_desc* desc,
                                      uint64_t first_move, size_t n, grx_precision prec,
                                      grx_widom_result* results);

/* ---- GCMC ----------------------------------------------------------------- */
/* Move mix and thermodynamic state of one box's GCMC run: the translation /
 * rotation / reinsertion / CBMC swap branches of RunMoves (axpy.cu:102-298) with the move
 * probabilities of Move_Statistics (cumulative, as the reference stores them),
 * get_new_position (mc_utilities.h:485-606) and GetPrefactor (mc_utilities.h:315-351). */
typedef struct {
  int32_t component;          /* the adsorbate component moved / exchanged */
  int32_t ntrials;            /* NumberOfTrialPositions */
  int32_t norient;            /* NumberOfTrialOrientations */
  int32_t pad_;
  double p_translation;       /* TranslationProb (cumulative) */
  double p_rotation;          /* RotationProb (cumulative) */
  double p_reinsertion;       /* ReinsertionProb (cumulative) */
  double p_swap;              /* SwapProb (cumulative); insertion / deletion 50:50 */
  double max_translation[3];  /* MaxTranslation, A */
  double max_rotation[3];     /* MaxRotation, rad */
  double beta;
  double pressure;            /* internal units (Pa / 1.6605402e7) */
  double fugacity_coeff;
  double mol_fraction;
  double ideal_rosenbluth;    /* IdealGasRosenbluthWeight */
  double tail_insert;         /* TailCorrectionDifference of one insertion; a
                                 deletion uses its negative (exact for the
                                 host-guest tail, which is linear in N) */
  uint64_t seed;              /* Philox key */
  uint32_t stream;            /* Philox counter word 3 (chain id) */
  uint32_t pad2_;
  double p_identity_swap;     /* IdentitySwapProb (cumulative, between reinsertion and swap;
                                 0: none). An identity swap (mc_swap_moves.h:199-420) replaces a
                                 molecule of a moved component holding molecules (uniform) by one
                                 of a moved component (uniform) grown on its first bead. Needs
                                 tail_insert 0. */
} grx_gcmc_desc;

typedef struct {
  int64_t attempts[5];        /* translation, rotation, insertion, deletion, reinsertion */
  int64_t accepted[5];
  int64_t n_molecules;        /* after the run */
  int64_t capacity_hits;      /* insertions refused for lack of component capacity */
  double energy[4];           /* sum of accepted dE: VDW, real Coulomb, Ewald Fourier, total */
  double sum_n;               /* sum over steps of N (loading average = sum_n / steps) */
  int64_t identity_out[2];    /* identity swaps removing this component: attempts, accepted */
  int64_t identity_in[2];     /* identity swaps adding this component: attempts, accepted (the
                                 accepted swaps' dE count in this entry's energy sums) */
  double rosen[3];            /* Rosenbluth weight W of every CBMC insertion attempt (W_first x
                                 W_chain x exp(-beta dE_Fourier) x exp(-beta tail), 0 when the
                                 growth fails; RecordRosen, data_struct.h:627-652): sum W,
                                 sum W^2, attempts. <W> gives mu_ex and the Henry coefficient
                                 (ComputeFugacity, print_statistics.cuh:99-109) */
  int64_t trial_configs;      /* trial configurations the kernel evaluated against every atom:
                                 first-bead positions, orientations (grown only after a
                                 successful first bead) and the two configurations of a
                                 translation / rotation (steps that picked this entry) */
  int64_t trial_beads;        /* beads of those configurations (each evaluated against every
                                 framework and guest atom) */
} grx_gcmc_stats;

/* nsteps GCMC moves on each of nboxes independent boxes (Markov chains), all on the
 * device in one persistent launch: one block per box, positions and S(k) resident.
 * Box i moves ncomp_moved[i] components (1..4; NULL: one each): its entries of descs
 * (and of stats) are consecutive, box-major, and share one seed and stream; every step
 * picks one of them uniformly (Select_Box_Component_Molecule, axpy.cu:74-100). Step s
 * of a box uses Philox move index first_step + s. stats[e] receives entry e's counts
 * for this call. Requires current structure factors (grx_ewald_total or
 * grx_ewald_set_structure_factors). */
grx_status grx_gcmc_run(grx_box* const* boxes, int32_t nboxes, const grx_gcmc_desc* descs,
                        const int32_t* ncomp_moved, uint64_t first_step, int64_t nsteps,
                        grx_precision prec, grx_gcmc_stats* stats);

/* A prepared GCMC launch over a fixed set of boxes, for long runs and CUDA graphs:
 * the per-box state, move sets, the Philox step counter (starting at 0) and running
 * statistics stay in device memory owned by the batch. Re-create the batch after
 * changing a box with any other call. */
typedef struct grx_gcmc_batch grx_gcmc_batch;
grx_status grx_gcmc_batch_create(grx_box* const* boxes, int32_t nboxes, const grx_gcmc_desc* descs,
                                 const int32_t* ncomp_moved, grx_precision prec, grx_gcmc_batch** out);
grx_status grx_gcmc_batch_destroy(grx_gcmc_batch* batch);
grx_status grx_gcmc_batch_set_step(grx_gcmc_batch* batch, uint64_t step);
/* Enqueues nsteps steps of every box on `stream` (NULL: the first box's stream) and
 * advances the device step counter; no host synchronization, so it can be captured
 * into a CUDA graph. Statistics accumulate on the device. */
grx_status grx_gcmc_batch_launch(grx_gcmc_batch* batch, int64_t nsteps, void* stream);
/* Per-box step windows for the following launches (continuous batching of jobs that
 * joined at different times): box i draws Philox move indices from next_move[i] on (its
 * own chain continues where it stopped, whatever the other boxes do) and takes at most
 * nsteps[i] steps per launch (NULL: all of the launch's steps; 0: the box idles). Waits for
 * the batch's launches. No counterpart in the reference. */
grx_status grx_gcmc_batch_set_box_steps(grx_gcmc_batch* batch, const uint64_t* next_move, const int64_t* nsteps);
/* nlaunch launches of nsteps steps each, captured once into a CUDA graph (re-captured
 * when nsteps or nlaunch change) and replayed on `stream`. */
grx_status grx_gcmc_batch_run_graph(grx_gcmc_batch* batch, int64_t nsteps, int32_t nlaunch, void* stream);
/* Waits for the device, then copies the accumulated statistics (one per entry) and
 * the next step index, and refreshes the boxes' molecule counts. */
grx_status grx_gcmc_batch_stats(grx_gcmc_batch* batch, grx_gcmc_stats* stats, uint64_t* next_step);
grx_status grx_gcmc_batch_reset_stats(grx_gcmc_batch* batch);
/* Launch shape of a batch: nwarps warps per box (8, 12 or 24; every shape keeps 24
 * warps per SM) and chunk_mult work items per warp in a bead pass (1..8). A new batch
 * takes 24 warps when its boxes fit one per SM, 12 when they fit two per SM, else 8,
 * with chunk_mult 1. */
grx_status grx_gcmc_batch_set_shape(grx_gcmc_batch* batch, int32_t nwarps, int32_t chunk_mult);
grx_status grx_gcmc_batch_get_shape(grx_gcmc_batch* batch, int32_t* nwarps, int32_t* chunk_mult);
/* Thread-block clusters: with cluster 2, 4 or 8 (nwarps must be 24) every box runs on a
 * cluster of that many CTAs, one per SM: the bead passes are split over the cluster and
 * the partial sums exchanged through distributed shared memory, so one chain spans
 * several SMs (batches with fewer boxes than SMs). Refused when not every box gets a
 * resident cluster of that size. Setting a shape with nwarps other than 24 returns to 1.
 * Same decisions as the one-block launch in the oracle tests; the summation order of the
 * partials differs. */
grx_status grx_gcmc_batch_set_cluster(grx_gcmc_batch* batch, int32_t cluster);
grx_status grx_gcmc_batch_get_cluster(grx_gcmc_batch* batch, int32_t* cluster);
/* Autotuner of the launch shape: runs nsteps real steps for each of the
 * GRX_GCMC_TUNE_CANDIDATES shapes (nwarps 8, 12, 24 x chunk_mult 1, 2, 4, in that
 * order), in a forward and a reverse sweep timed with CUDA events, and keeps the shape
 * with the most trial energies per second for this batch. When the boxes leave SMs idle
 * (clusters of 2, 4 or 8 fit, the largest is taken), the best shape is then timed
 * against that cluster size with 24 warps (order: plain, cluster, cluster, plain) and the
 * faster kept. chosen receives (cluster - 1) * 10000 + nwarps * 100 + chunk_mult;
 * ms_per_candidate receives GRX_GCMC_TUNE_CANDIDATES mean probe times of the plain shapes
 * (or NULL). The probe steps are ordinary Monte Carlo steps: the chains advance by up to
 * 2 * (GRX_GCMC_TUNE_CANDIDATES + 2) * nsteps. */
#define GRX_GCMC_TUNE_CANDIDATES 9
grx_status grx_gcmc_batch_autotune(grx_gcmc_batch* batch, int64_t nsteps, int32_t* chosen,
                                   float* ms_per_candidate);

/* ---- measurement ------------------------------------------------------------ */
/* FP32 FMA throughput of the current device (TFLOP/s, 2 FLOP per FMA): independent
 * FMA chains on every SM, timed with CUDA events over `iters` x 128 FMAs per thread.
 * The roofline denominator of the pair kernels (no gRASPA counterpart). */
grx_status grx_probe_fp32_fma(int32_t iters, double* tflops, float* ms);
/* The double-float functions of the mixed-precision CBMC stages evaluated on the device, for
 * accuracy tests: out5[5i..5i+4] = sin(2 pi v[i]), cos(2 pi v[i]) and the rotation of
 * (1, 0.5, -0.25) by the uniform quaternion of Rotate_Quaternions (mc_utilities.h:423-457)
 * whose uniforms are words[3i..3i+2] * 2^-32. No counterpart in the reference. */
grx_status grx_probe_df_functions(const double* v, const uint32_t* words, int64_t n, double* out5);

/* ---- serving ----------------------------------------------------------------- */
/* A continuous-batching job server. Each job is one box (its description and atoms,
 * copied at submission) with Widom insertions or GCMC steps to run. The caller's loop
 * calls grx_server_progress, which in one non-blocking round retires finished jobs,
 * admits queued jobs in arrival order while a slot is free and the job's box fits in
 * the server's device memory arena (admission by HBM footprint), and launches the next
 * slice of every resident job on the job's own stream, so the work of different jobs
 * overlaps on the device. A job's result does not depend on the other jobs. No
 * counterpart in the reference (one simulation per process). */
#define GRX_JOB_WIDOM 0
#define GRX_JOB_GCMC 1

typedef struct {
  size_t hbm_budget_bytes;      /* arena size when the server makes its own arena */
  int32_t max_resident;         /* job slots */
  grx_precision precision;
  int64_t widom_slice;          /* insertions per launch (<= 0: whole job) */
  int64_t gcmc_slice;           /* steps per launch (<= 0: whole job) */
  int64_t cluster_atoms;        /* > 0: a GCMC job of N atoms runs on a thread-block cluster of
                                   the largest of 8, 4, 2 CTAs not above N / cluster_atoms
                                   (grx_gcmc_batch_set_cluster; one block when it does not fit);
                                   0: one block per job */
  int32_t gcmc_batching;        /* 1: every resident GCMC job advances in one shared persistent
                                   launch per round (8 warps per job, up to 3 jobs per SM): jobs
                                   join and leave between rounds, each draws from its own move
                                   stream (grx_gcmc_batch_set_box_steps), and each takes a step
                                   count proportional to gcmc_slice / its estimated cost per step,
                                   so a round lasts about gcmc_slice steps of a job of 1000 pair
                                   evaluations per step; cluster_atoms is not used. 0: one
                                   launch per job on its own stream */
  int32_t pad_;
} grx_server_config;

typedef struct {
  int32_t kind;                 /* GRX_JOB_WIDOM or GRX_JOB_GCMC */
  int32_t ncomp_moved;          /* GCMC: entries of gcmc (1..4) */
  const grx_box_desc* box;
  const grx_atoms* atoms;       /* box->ncomponents entries (empty adsorbates store their template) */
  const int32_t* rigid;         /* per component, NULL: adsorbate components rigid */
  grx_widom_desc widom;
  int64_t widom_insertions;
  const grx_gcmc_desc* gcmc;
  int64_t gcmc_steps;
  uint64_t tag;                 /* returned with the result */
} grx_job_desc;

typedef struct {
  uint64_t tag;
  uint64_t job_id;
  int32_t kind;
  int32_t status;               /* grx_status of the job */
  double t_submit, t_admit, t_done;   /* seconds on the server clock */
  size_t footprint_bytes;       /* arena bytes the job held */
  int64_t widom_n;
  double widom_mean_w;          /* <W> over the insertions (failed constructions count as 0) */
  double widom_mean_w2;         /* <W^2> */
  int64_t gcmc_steps;
  int32_t ncomp_moved;
  int32_t pad_;
  grx_gcmc_stats gcmc[4];
  int64_t widom_trial_configs;  /* Widom: trial configurations evaluated (first-bead positions, plus
                                   the orientations of insertions whose first bead was grown) */
} grx_job_result;

typedef struct grx_server grx_server;
/* arena: NULL to make one of cfg->hbm_budget_bytes owned by the server. */
grx_status grx_server_create(const grx_server_config* cfg, grx_arena* arena, grx_server** out);
grx_status grx_server_destroy(grx_server* server);
grx_status grx_server_submit(grx_server* server, const grx_job_desc* job, uint64_t* job_id);
grx_status grx_server_progress(grx_server* server, int32_t* n_resident, int32_t* n_pending);
/* Moves up to max finished jobs' results into out; *n = how many. */
grx_status grx_server_poll(grx_server* server, grx_job_result* out, int32_t max, int32_t* n);
grx_status grx_server_time(grx_server* server, double* seconds);
grx_status grx_server_launch_count(grx_server* server, uint64_t* launches);

/* ---- allocation-free trial energies ------------------------------------- */
/* grx_trial_energies without any device allocation at call time. No counterpart
 * in the reference: it exists for callers that cannot let a call allocate device
 * memory, such as a Monte Carlo loop that must never stall the GPU (cudaMalloc and
 * cudaFree can synchronize the whole device) or a host application that owns all
 * device memory through its own pool. Same arguments, semantics and results as
 * grx_trial_energies; the scratch lives in one fixed device array of
 * GRX_NOALLOC_SCRATCH_BYTES held by every GPU that loads the library until exit.
 * Limit: ntrials * chainsize <= GRX_NOALLOC_MAX_BEADS, else GRX_ERR_CAPACITY.
 * The call works on the box's device (made current for the call, the caller's
 * device restored after). The first call on a device looks up the array's device
 * address (make it before any stream capture). All calls share the array: calls
 * that overlap on the GPU race, so issue them one after another. The box is created
 * beforehand with grx_box_create. */
#define GRX_NOALLOC_MAX_BEADS 256
#define GRX_NOALLOC_SCRATCH_BYTES 65536
grx_status grx_trial_energies_noalloc(grx_box* box, const grx_trials* trials, int32_t component,
                                      int64_t exclude_comp, int64_t exclude_molid,
                                      grx_precision prec, grx_trial_energy* out, uint8_t* overlap);

/* Number of kernel launches this process issued through the library. */
uint64_t grx_launch_count(void);
/* Bytes copied host -> device and device -> host by the calling thread's last
 * grx_gcmc_run (box state descriptors, move sets, offsets and step in; statistics and
 * molecule counts out). */
grx_status grx_last_transfer(size_t* h2d, size_t* d2h);

#ifdef __cplusplus
}
#endif
#endif /* GRX_H */
