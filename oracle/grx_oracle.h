/*
 * grx_oracle.h -- FP64 CPU oracle for the CBMC trial-energy path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain C++ restatement of gRASPA's FP64
 * arithmetic for the hot path (pair energies, Ewald Fourier delta and totals,
 * Rosenbluth selection, CBMC Widom insertion). It is the checker for the CUDA
 * library and the timed CPU baseline. Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline / reference legs may load it. The product library
 * (graspa_gb300, libgrx.so) never calls into it.
 *
 * Parity is pinned against the reference's own committed FP64 outputs for the
 * NIST SPC/E boxes (Examples/Reference_NIST_SPCE/Box-{1..4}/output.txt) through
 * tests/golden/nist_spce_box*.json.
 *
 * Conventions follow the reference: energies in internal units (10 J/mol),
 * cutoffs squared (ForceField.CutOffVDW / CutOffCoul, data_struct.h:850-851),
 * cell matrices column-major as Boxsize.Cell (read_data.cpp:1545-1547).
 */
#ifndef GRX_ORACLE_H
#define GRX_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  double cell[9];
  double inverse_cell[9];
  double volume;
  int32_t cubic;
  int32_t use_lammps_ewald;
  int32_t kmax[3];
  int32_t pad_;
  double alpha;
  double prefactor;
  double reciprocal_cutoff;
} ora_box;

typedef struct {
  int64_t ntypes;
  const double* epsilon;  /* ntypes*ntypes, internal units (K / 1.20272430057) */
  const double* sigma;
  const double* z;
  const double* shift;
  const double* c10;
  int32_t use_1264;
  int32_t no_charges;
  int32_t vdw_real_bias;
  int32_t pad_;
  double overlap_criteria;
  double cutoff_vdw_sq;
  double cutoff_coul_sq;
} ora_ff;

/* All atoms of every component, concatenated component by component (the
 * per-component Atoms arrays of Simulations.d_a, data_struct.h:788-799). */
typedef struct {
  int64_t ncomp;   /* NComponents.x */
  int64_t nhost;   /* NComponents.y */
  const int64_t* comp_start;  /* ncomp+1 offsets */
  const double* pos;          /* 3 per atom */
  const double* scale;
  const double* charge;
  const double* scale_coul;
  const int64_t* type;
  const int64_t* molid;
} ora_atoms;

/* Trial beads (Simulations.New as filled by get_random_trial_position /
 * get_random_trial_orientation, mc_widom.h:122-303). */
typedef struct {
  int64_t ntrials;
  int64_t chainsize;
  const double* pos;          /* 3 * ntrials * chainsize */
  const double* scale;
  const double* charge;
  const double* scale_coul;
  const int64_t* type;
  int64_t molid;              /* NewMol.MolID[0] */
} ora_trials;

typedef struct {
  int64_t component;          /* inserted adsorbate component */
  int64_t molsize;
  const double* mol_pos;      /* component atoms 0..molsize-1 (orientation template) */
  const double* mol_charge;
  const int64_t* mol_type;
  double scale;               /* proposed_scale.x */
  double scale_coul;          /* proposed_scale.y */
  int64_t ntrials;            /* NumberWidomTrials */
  int64_t norient;            /* NumberWidomTrialsOrientations */
  int64_t new_molid;          /* NumberOfMolecule_for_Component[component] */
  double beta;
  double excl_intra;          /* ExclusionIntra[component] */
  double excl_self;           /* ExclusionAtom[component] */
  double tail_delta;          /* TailCorrectionDifference for one insertion */
  int32_t rigid;
  int32_t has_charge;         /* hasPartialCharge[component] */
  uint64_t seed;
  uint32_t stream;
  uint32_t pad_;
} ora_widom;

typedef struct {
  double rosenbluth;
  double w_first;             /* averaged first-bead weight */
  double w_chain;             /* averaged orientation weight */
  double e_first[4];          /* selected first bead: hg_vdw hg_real gg_vdw gg_real */
  double e_chain[4];
  double ewald[2];            /* {same - exclusion, 2*cross} */
  int64_t sel_first;          /* index into the trial list (REALselected) */
  int64_t sel_orient;
  int64_t n_ok_first;
  int64_t n_ok_orient;
  int32_t success;
  int32_t pad_;
} ora_widom_result;

/* geometry / force field setup */
void ora_box_setup(ora_box* box);                 /* inverse, volume, cubic, LAMMPS cutoff */
void ora_box_setup_raspa_ewald(ora_box* box, double cutoff_coul, double precision);
void ora_mix_lorentz_berthelot(int64_t ntypes, const double* eps_K, const double* sigma,
                               const int32_t* shifted, double cutoff_vdw_sq,
                               double* eps_out, double* sig_out, double* shift_out);

/* pair math */
void ora_pbc(const ora_box* box, double* d3);
void ora_vdw(const double* ffarg, double rr, double scaling, int use_1264, double* result2);
double ora_coulomb_real(double qa, double qb, double r, double scaling, double prefactor, double alpha);

/* trial / move energies */
void ora_trial_energies(const ora_box* box, const ora_ff* ff, const ora_atoms* atoms,
                        const ora_trials* trials, int64_t component,
                        int64_t excl_comp, int64_t excl_molid,
                        double* out4, uint8_t* flag);
void ora_single_body(const ora_box* box, const ora_ff* ff, const ora_atoms* atoms,
                     const ora_trials* old_mol, const ora_trials* new_mol, int64_t component,
                     int32_t do_new, int32_t do_old, double* out6, uint8_t* flag);
void ora_vdw_real_total(const ora_box* box, const ora_ff* ff, const ora_atoms* atoms, double* out6);

/* Ewald */
int64_t ora_ewald_nvec(const ora_box* box);
int64_t ora_ewald_active(const ora_box* box, uint8_t* active);
void ora_ewald_total(const ora_box* box, const ora_atoms* atoms, const int64_t* molsize,
                     double* s_fw, double* s_ads, double* out8);
void ora_ewald_delta(const ora_box* box, const double* s_same, const double* s_cross,
                     int32_t use_temp, const double* s_temp,
                     int64_t n_old, const double* old_pos, const double* old_qs,
                     int64_t n_new, const double* new_pos, const double* new_qs,
                     double* s_new, double* out2);
void ora_ewald_delta_lambda(const ora_box* box, const double* s_same, const double* s_cross, int32_t use_temp,
                            const double* s_temp, int64_t n, const double* pos, const double* q, double scale_old,
                            double scale_new, double excl, double* s_new, double* out2);
void ora_ewald_delta_identity_swap(const ora_box* box, const double* s_same, const double* s_cross,
                                   int64_t n_old, const double* old_pos, const double* old_qs, int64_t n_new,
                                   const double* new_pos, const double* new_qs, double excl_new, double excl_old,
                                   double* s_new, double* out2);
void ora_rigid_exclusion(const ora_box* box, int64_t molsize, const double* pos,
                         const double* charge, const double* scale_coul,
                         double* intra, double* self);

/* RNG + selection */
void ora_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void ora_draw(uint64_t seed, uint32_t stream, uint64_t move, uint32_t slot, uint32_t out[4]);
int64_t ora_select_trial(const double* logw, int64_t n, double u);
void ora_rotate_quaternion(double* vec3, double u, double v, double w);

/* CBMC Widom insertion driver (Insertion_Body -> WidomMove, move_struct.h:90-95) */
void ora_widom_insertions(const ora_box* box, const ora_ff* ff, const ora_atoms* atoms,
                          const double* s_fw, const double* s_ads, const ora_widom* w,
                          uint64_t first_move, int64_t n, int32_t nthreads,
                          ora_widom_result* results);
int32_t ora_max_threads(void);


/* GCMC of one adsorbate component (RunMoves, axpy.cu:102-298, restricted to the
 * translation / rotation / reinsertion / CBMC insertion / CBMC deletion branches). */
typedef struct {
  int64_t component;
  int64_t ntrials;
  int64_t norient;
  double p_translation;   /* cumulative move probabilities (Move_Statistics) */
  double p_rotation;
  double p_reinsertion;
  double p_swap;
  double max_translation[3];
  double max_rotation[3];
  double beta;
  double pressure;        /* internal units */
  double fugacity_coeff;
  double mol_fraction;
  double ideal_rosenbluth;
  uint64_t seed;
  uint32_t stream;
  uint32_t pad_;
  double tail_insert;     /* TailCorrectionDifference of one insertion; a deletion
                             takes its negative (exact for a host-guest tail) */
} ora_gcmc;

typedef struct {
  int64_t attempts[5];    /* translation, rotation, insertion, deletion, reinsertion */
  int64_t accepted[5];
  int64_t n_molecules;
  double energy[4];       /* running sums of accepted dE: vdw, real, ewald, total */
  double sum_n;           /* sum of N after every step (loading average) */
  double rosen[3];        /* insertion attempts' Rosenbluth weights (RecordRosen): sum W, sum W^2,
                             attempts; W = 0 when the growth failed */
  int64_t trial_configs;  /* trial configurations evaluated (first beads, orientations grown after
                             a successful first bead, 2 per translation / rotation) */
  int64_t trial_beads;    /* their beads */
  double last_margin;     /* smallest decision margin of the last step (trial selections and
                             acceptance; relative weight change that flips it); test diagnostics */
} ora_gcmc_stats;

/* Runs nsteps moves on one box. atoms/s_ads are updated in place (guest component
 * region must have room for the growth: capacity atoms from comp_start). */
void ora_gcmc_run(const ora_box* box, const ora_ff* ff, double* pos, double* charge, int64_t* type,
                  int64_t* molid, int64_t ncomp, int64_t nhost, int64_t* comp_size,
                  const int64_t* comp_off, const int64_t* molsize, const double* mol_pos,
                  const double* mol_charge, const int64_t* mol_type, double excl_intra, double excl_self,
                  double* s_fw, double* s_ads, const ora_gcmc* g, uint64_t first_step,
                  int64_t nsteps, ora_gcmc_stats* stats);

/* Mixture form: ng moved components (gk[k], one template / exclusion pair each;
 * seed and stream from gk[0]); every step picks entry floor(u * ng) with word 3 of
 * the displacement slot (Select_Box_Component_Molecule, axpy.cu:74-100). stk[k]
 * receives entry k's counts. mol_pos_k[k] holds the component's slot-0 coordinates the
 * orientations grow from, in and out, so a later call continues the same chain. */
void ora_gcmc_run_mix(const ora_box* box, const ora_ff* ff, double* pos, double* charge, int64_t* type,
                      int64_t* molid, int64_t ncomp, int64_t nhost, int64_t* comp_size, const int64_t* comp_off,
                      const int64_t* molsize, double* const* mol_pos_k, const double* const* mol_charge_k,
                      const int64_t* const* mol_type_k, const double* excl_intra_k, const double* excl_self_k,
                      double* s_fw, double* s_ads, const ora_gcmc* gk, int64_t ng, uint64_t first_step,
                      int64_t nsteps, ora_gcmc_stats* stk);

#ifdef __cplusplus
}
#endif
#endif
