// graspa_host.cpp -- the reference-shaped move drivers over the libgrx C ABI.
// Each function cites the gRASPA code it restates; the energy work of every call
// runs in libgrx on the GPU.
#include "graspa_host.hpp"

#include <algorithm>
#include <cstdio>
#include <numeric>

namespace graspa {

// ------------------------------------------------------------------ small types
void MoveEnergy::take_negative() {
  HHVDW = -HHVDW; HGVDW = -HGVDW; GGVDW = -GGVDW;
  HHReal = -HHReal; HGReal = -HGReal; GGReal = -GGReal;
  HHEwaldE = -HHEwaldE; HGEwaldE = -HGEwaldE; GGEwaldE = -GGEwaldE;
  TailE = -TailE;
}
MoveEnergy& MoveEnergy::operator+=(const MoveEnergy& o) {
  HHVDW += o.HHVDW; HGVDW += o.HGVDW; GGVDW += o.GGVDW;
  HHReal += o.HHReal; HGReal += o.HGReal; GGReal += o.GGReal;
  HHEwaldE += o.HHEwaldE; HGEwaldE += o.HGEwaldE; GGEwaldE += o.GGEwaldE;
  TailE += o.TailE;
  return *this;
}
MoveEnergy& MoveEnergy::operator-=(const MoveEnergy& o) {
  MoveEnergy n = o;
  n.take_negative();
  return *this += n;
}
MoveEnergy operator+(MoveEnergy a, const MoveEnergy& b) { return a += b; }

void HostAtoms::allocate(size_t n) {
  pos.assign(n, double3{});
  scale.assign(n, 1.0);
  charge.assign(n, 0.0);
  scaleCoul.assign(n, 1.0);
  Type.assign(n, 0);
  MolID.assign(n, 0);
}

Atoms HostAtoms::view(size_t molsize, size_t size) {
  Atoms a;
  a.pos = pos.data();
  a.scale = scale.data();
  a.charge = charge.data();
  a.scaleCoul = scaleCoul.data();
  a.Type = Type.data();
  a.MolID = MolID.data();
  a.Molsize = molsize;
  a.size = size;
  a.Allocate_size = pos.size();
  return a;
}

void Move_Statistics::Record_Move_Total(int move) {
  switch (move) {
    case TRANSLATION: ++TranslationTotal; break;
    case ROTATION: ++RotationTotal; break;
    case INSERTION: ++InsertionTotal; break;
    case DELETION: ++DeletionTotal; break;
    case REINSERTION: ++ReinsertionTotal; break;
    default: break;
  }
}
void Move_Statistics::Record_Move_Accept(int move) {
  switch (move) {
    case TRANSLATION: ++TranslationAccepted; break;
    case ROTATION: ++RotationAccepted; break;
    case INSERTION: ++InsertionAccepted; break;
    case DELETION: ++DeletionAccepted; break;
    case REINSERTION: ++ReinsertionAccepted; break;
    default: break;
  }
}
void Move_Statistics::NormalizeProbabilities() {
  const double tot = TranslationProb + RotationProb + ReinsertionProb + IdentitySwapProb + SwapProb;
  if (tot > 1e-10) {
    TranslationProb /= tot; RotationProb /= tot; ReinsertionProb /= tot; IdentitySwapProb /= tot; SwapProb /= tot;
  }
  RotationProb += TranslationProb;
  ReinsertionProb += RotationProb;
  IdentitySwapProb += ReinsertionProb;
  SwapProb += IdentitySwapProb;
}

void check(grx_status st, const char* what) {
  if (st != GRX_OK) {
    throw std::runtime_error(std::string(what) + ": " + grx_status_string(st) + " (" + grx_last_error() + ")");
  }
}

static void trial_buffers(Simulations& Sims) {
  Sims.OldStore.allocate(1024);
  Sims.NewStore.allocate(1024);
  Sims.Old = Sims.OldStore.view(0, 0);
  Sims.New = Sims.NewStore.view(0, 0);
}

// ------------------------------------------------------------------ set-up
// A device box of geometry B holding `atoms` (host arrays per component, n_stored[c] atoms
// stored), with its structure factors computed (fxn_main.h:46-113 / main.cpp:243-300).
static grx_box* create_box(const Boxsize& B, const ForceField& FF, const Components& SC, const std::vector<Atoms>& atoms,
                           const std::vector<size_t>& n_stored) {
  grx_box_desc d{};
  for (int k = 0; k < 9; ++k) {
    d.geometry.cell[k] = B.Cell[k];
    d.geometry.inverse_cell[k] = B.InverseCell[k];
  }
  d.geometry.volume = B.Volume;
  d.geometry.cubic = B.Cubic;
  d.geometry.use_lammps_ewald = B.UseLAMMPSEwald;
  d.geometry.kmax[0] = B.kmax.x;
  d.geometry.kmax[1] = B.kmax.y;
  d.geometry.kmax[2] = B.kmax.z;
  d.geometry.alpha = B.Alpha;
  d.geometry.prefactor = B.Prefactor;
  d.geometry.reciprocal_cutoff = B.ReciprocalCutOff;
  d.forcefield.ntypes = (int32_t)FF.size;
  d.forcefield.use_1264 = FF.Use1264;
  d.forcefield.epsilon = FF.epsilon.data();
  d.forcefield.sigma = FF.sigma.data();
  d.forcefield.z = FF.z.empty() ? nullptr : FF.z.data();
  d.forcefield.shift = FF.shift.data();
  d.forcefield.c10 = FF.C10.empty() ? nullptr : FF.C10.data();
  d.forcefield.no_charges = FF.noCharges;
  d.forcefield.vdw_real_bias = FF.VDWRealBias;
  d.forcefield.overlap_criteria = FF.OverlapCriteria;
  d.forcefield.cutoff_vdw_sq = FF.CutOffVDW;
  d.forcefield.cutoff_coul_sq = FF.CutOffCoul;
  d.ncomponents = SC.NComponents.x;
  d.nhost_components = SC.NComponents.y;
  for (int c = 0; c < SC.NComponents.x; ++c) {
    d.capacity[c] = std::max<size_t>(1, SC.Allocate_size[c]);  // a framework may have no atoms
    d.molsize[c] = std::max<size_t>(1, SC.Moleculesize[c]);
  }
  grx_box* box = nullptr;
  check(grx_box_create(&d, &box), "grx_box_create");
  for (int c = 0; c < SC.NComponents.x; ++c) {
    const Atoms& A = atoms[c];
    grx_atoms ga{};
    ga.pos = reinterpret_cast<const double*>(A.pos);
    ga.scale = A.scale;
    ga.charge = A.charge;
    ga.scale_coul = A.scaleCoul;
    ga.type = A.Type;
    ga.molid = A.MolID;
    ga.size = A.size;
    ga.n_stored = std::max(A.size, n_stored[c]);
    const grx_status st = grx_box_set_component(box, c, &ga, c >= SC.NComponents.y && SC.rigid[c]);
    if (st) {
      grx_box_destroy(box);
      check(st, "grx_box_set_component");
    }
  }
  double out8[8];
  const grx_status st = grx_ewald_total(box, out8);
  if (st) {
    grx_box_destroy(box);
    check(st, "grx_ewald_total");
  }
  return box;
}

void Setup_Box(Variables& Vars, size_t systemId, const std::vector<size_t>& n_stored) {
  Simulations& Sims = Vars.Sims[systemId];
  Components& SC = Vars.SystemComponents[systemId];
  Boxsize& B = Sims.Box;
  SC.StoredAtoms.assign(SC.NComponents.x, 0);
  for (int c = 0; c < SC.NComponents.x; ++c) SC.StoredAtoms[c] = std::max(Sims.d_a[c].size, n_stored[c]);
  B.handle = create_box(B, Vars.device_FF, SC, Sims.d_a, SC.StoredAtoms);
  SC.ExclusionIntra.assign(SC.NComponents.x, 0.0);
  SC.ExclusionAtom.assign(SC.NComponents.x, 0.0);
  SC.hasPartialCharge.assign(SC.NComponents.x, false);
  for (int c = 0; c < SC.NComponents.x; ++c) {
    const Atoms& A = Sims.d_a[c];
    check(grx_box_get_exclusion(B.handle, c, &SC.ExclusionIntra[c], &SC.ExclusionAtom[c]), "grx_box_get_exclusion");
    for (size_t i = 0; i < SC.StoredAtoms[c]; ++i)
      if (A.charge[i] != 0.0) SC.hasPartialCharge[c] = true;
    if (c >= SC.NComponents.y) SC.NumberOfMolecule_for_Component[c] = A.size / SC.Moleculesize[c];
  }
  SC.Beta = SC.Beta > 0 ? SC.Beta : 1.0 / (1.380649e-23 / (1.6605402e-27 * 1e-20 / 1e-24) * SC.Temperature);
  trial_buffers(Sims);
}

void Destroy_Box(Variables& Vars, size_t systemId) {
  Boxsize& B = Vars.Sims[systemId].Box;
  if (B.handle) grx_box_destroy(B.handle);
  B.handle = nullptr;
}

// ------------------------------------------------------------------ energy calls
void CBMC_PairwiseInteractions(Variables& Vars, size_t systemId, Components& SC, Simulations& Sims, size_t NTrials,
                               size_t chainsize) {
  (void)systemId;
  const size_t nb = NTrials * chainsize;
  std::vector<grx_trial_energy> e(NTrials);
  std::vector<uint8_t> flag(NTrials);
  grx_trials t{};
  t.pos = reinterpret_cast<const double*>(Sims.New.pos);
  t.scale = Sims.New.scale;
  t.charge = Sims.New.charge;
  t.scale_coul = Sims.New.scaleCoul;
  t.type = Sims.New.Type;
  t.molid = Sims.New.MolID[0];
  t.ntrials = NTrials;
  t.chainsize = chainsize;
  (void)nb;
  check(grx_trial_energies(Sims.Box.handle, &t, (int32_t)SC.TempVal.component, Sims.ExcludeComponent,
                           Sims.ExcludeMolecule, Vars.Precision, e.data(), flag.data()),
        "grx_trial_energies");
  // Host_sum_Widom_HGGG_SEPARATE: keep the trials without overlap
  SC.Rosen.clear();
  SC.TrialEnergies.clear();
  SC.Trialindex.clear();
  for (size_t i = 0; i < NTrials; ++i) {
    if (flag[i]) continue;
    MoveEnergy m;
    m.HGVDW = e[i].hg_vdw;
    m.HGReal = e[i].hg_real;
    m.GGVDW = e[i].gg_vdw;
    m.GGReal = e[i].gg_real;
    double tot = m.HGVDW + m.GGVDW;
    if (Vars.device_FF.VDWRealBias) tot += m.HGReal + m.GGReal;
    SC.Rosen.push_back(-SC.Beta * tot);
    SC.TrialEnergies.push_back(m);
    SC.Trialindex.push_back(i);
  }
}

size_t SelectTrialPosition(std::vector<double>& LogBoltzmannFactors, const Variables& Vars, size_t systemId,
                           int word) {
  int32_t sel = 0;
  double sum = 0.0;
  check(grx_cbmc_select(LogBoltzmannFactors.data(), (int32_t)LogBoltzmannFactors.size(), Vars.Random.Seed,
                        Vars.Random.BoxStream(systemId), Vars.SystemComponents[systemId].Step, word, &sel, &sum),
        "grx_cbmc_select");
  return (size_t)sel;
}

// The moved molecule's atoms for the Ewald delta, per move type.
static void molecule_atoms(Simulations& Sims, Components& SC, size_t comp, size_t first_atom,
                           std::vector<double>& pos, std::vector<double>& qs) {
  const size_t ms = SC.Moleculesize[comp];
  const Atoms& A = Sims.d_a[comp];
  pos.resize(3 * ms);
  qs.resize(ms);
  for (size_t a = 0; a < ms; ++a) {
    pos[3 * a] = A.pos[first_atom + a].x;
    pos[3 * a + 1] = A.pos[first_atom + a].y;
    pos[3 * a + 2] = A.pos[first_atom + a].z;
    qs[a] = A.charge[first_atom + a] * A.scaleCoul[first_atom + a];
  }
}

// The grown configuration: first bead in Old.pos[0], chain from New at orientation `orient`.
static void grown_atoms(Simulations& Sims, Components& SC, size_t comp, size_t orient, std::vector<double>& pos,
                        std::vector<double>& qs) {
  const size_t ms = SC.Moleculesize[comp], chain = ms - 1;
  const Atoms& T = Sims.d_a[comp];  // template charges (slot 0)
  pos.resize(3 * ms);
  qs.resize(ms);
  pos[0] = Sims.Old.pos[0].x; pos[1] = Sims.Old.pos[0].y; pos[2] = Sims.Old.pos[0].z;
  qs[0] = T.charge[0];
  for (size_t a = 0; a < chain; ++a) {
    const double3& p = Sims.New.pos[orient * chain + a];
    pos[3 * (1 + a)] = p.x; pos[3 * (1 + a) + 1] = p.y; pos[3 * (1 + a) + 2] = p.z;
    qs[1 + a] = T.charge[1 + a];
  }
}

double2 GPU_EwaldDifference_General(Simulations& Sims, ForceField& FF, Components& SC, size_t comp, int MoveType,
                                    size_t Location, double2 Scale) {
  (void)FF;
  std::vector<double> op, oq, np, nq;
  switch (MoveType) {
    case TRANSLATION: case ROTATION: {
      molecule_atoms(Sims, SC, comp, Location, op, oq);
      const size_t ms = SC.Moleculesize[comp];
      np.resize(3 * ms);
      for (size_t a = 0; a < ms; ++a) {
        np[3 * a] = Sims.New.pos[a].x; np[3 * a + 1] = Sims.New.pos[a].y; np[3 * a + 2] = Sims.New.pos[a].z;
      }
      nq = oq;
      break;
    }
    case INSERTION:
      grown_atoms(Sims, SC, comp, Location, np, nq);
      break;
    case DELETION:
      molecule_atoms(Sims, SC, comp, Location, op, oq);
      break;
    case REINSERTION: {
      molecule_atoms(Sims, SC, comp, Location, op, oq);
      const size_t ms = SC.Moleculesize[comp];
      np.resize(3 * ms);
      for (size_t a = 0; a < ms; ++a) {  // tempMolStorage, staged in Old[1..ms]
        np[3 * a] = Sims.Old.pos[1 + a].x; np[3 * a + 1] = Sims.Old.pos[1 + a].y;
        np[3 * a + 2] = Sims.Old.pos[1 + a].z;
      }
      nq = oq;
      break;
    }
    default:
      throw std::runtime_error("GPU_EwaldDifference_General: move type not on this path");
  }
  double out2[2];
  check(grx_ewald_delta(Sims.Box.handle, (int32_t)comp, MoveType, op.data(), oq.data(), oq.size(), np.data(),
                        nq.data(), nq.size(), Scale.y, out2),
        "grx_ewald_delta");
  return double2{out2[0], out2[1]};
}

void Update_Vector_Ewald(Boxsize& Box, bool UseTempVector, Components& SC, size_t comp) {
  (void)UseTempVector;
  (void)SC;
  check(grx_ewald_commit(Box.handle, (int32_t)comp), "grx_ewald_commit");
}

MoveEnergy Total_Energy(Simulations& Sims) {
  grx_energy e{};
  check(grx_total_energy(Sims.Box.handle, &e), "grx_total_energy");
  MoveEnergy m;
  m.HHVDW = e.hh_vdw; m.HHReal = e.hh_real; m.HGVDW = e.hg_vdw; m.HGReal = e.hg_real;
  m.GGVDW = e.gg_vdw; m.GGReal = e.gg_real;
  m.HHEwaldE = e.hh_ewald; m.HGEwaldE = e.hg_ewald; m.GGEwaldE = e.gg_ewald;
  return m;
}

// ------------------------------------------------------------------ volume moves
// Single-image rounding of PBC (maths.cuh:427-450): cast of x +- 0.5, half away from zero.
static double round_away(double x) { return (double)(long long)(x + (x >= 0 ? 0.5 : -0.5)); }

static void pbc_host(const Boxsize& B, double3& v) {
  if (B.Cubic) {
    v.x -= round_away(v.x * B.InverseCell[0]) * B.Cell[0];
    v.y -= round_away(v.y * B.InverseCell[4]) * B.Cell[4];
    v.z -= round_away(v.z * B.InverseCell[8]) * B.Cell[8];
    return;
  }
  const double* I = B.InverseCell;
  const double* C = B.Cell;
  double s[3] = {I[0] * v.x + I[3] * v.y + I[6] * v.z, I[1] * v.x + I[4] * v.y + I[7] * v.z,
                 I[2] * v.x + I[5] * v.y + I[8] * v.z};
  for (double& x : s) x -= round_away(x);
  v = double3{C[0] * s[0] + C[3] * s[1] + C[6] * s[2], C[1] * s[0] + C[4] * s[1] + C[7] * s[2],
              C[2] * s[0] + C[5] * s[1] + C[8] * s[2]};
}

void Minimum_Image(const Boxsize& Box, double3& v) { pbc_host(Box, v); }

// The box geometry with every length scaled by s (ScalePositions :71-84): kmax from the
// precision factor tol1, or, with explicit k vectors (tol1 = 0), the same kmax and the
// LAMMPS reciprocal cutoff of the scaled cell (read_data.cpp:664-687).
static Boxsize scaled_geometry(const Boxsize& B, double s, double newV, bool charges) {
  Boxsize T = B;
  T.handle = nullptr;
  for (int k = 0; k < 9; ++k) {
    T.Cell[k] *= s;
    T.InverseCell[k] /= s;
  }
  T.Volume = newV;
  if (charges) {
    const double pi = 3.14159265358979323846;
    if (B.tol1 > 0.0) {
      T.kmax = int3{(int)std::round(0.25 + T.Cell[0] * T.Alpha * T.tol1 / pi),
                    (int)std::round(0.25 + T.Cell[4] * T.Alpha * T.tol1 / pi),
                    (int)std::round(0.25 + T.Cell[8] * T.Alpha * T.tol1 / pi)};
      T.ReciprocalCutOff = std::pow(1.05 * (double)std::max(T.kmax.x, std::max(T.kmax.y, T.kmax.z)), 2);
    } else {
      const double kvx = T.kmax.x * (2 * pi / T.Cell[0]), kvy = T.kmax.y * (2 * pi / T.Cell[4]),
                   kvz = T.kmax.z * (2 * pi / T.Cell[8]);
      T.ReciprocalCutOff = std::max(kvx * kvx, std::max(kvy * kvy, kvz * kvz)) * 1.00001;
    }
  }
  return T;
}

// One box at a scaled volume: its geometry, the scaled atoms, the device box and its totals.
struct ScaledBox {
  Boxsize Box;
  std::vector<HostAtoms> host;
  std::vector<Atoms> atoms;
  MoveEnergy E;
  bool overlap = false;
};

// ScalePositions / ScaleCopyPositions (mc_box.h:19-86): adsorbate molecules only (the
// framework is not scaled); the first bead moves to s * its position, the other atoms keep
// their minimum-image offsets from it. Then the FP64 totals of the scaled box.
static void build_scaled(Variables& Vars, size_t systemId, double s, double newV, ScaledBox& out) {
  Simulations& Sims = Vars.Sims[systemId];
  Components& SC = Vars.SystemComponents[systemId];
  const ForceField& FF = Vars.device_FF;
  for (size_t c = 0; c < SC.TailCorrectionInsert.size(); ++c)
    if (SC.TailCorrectionInsert[c] != 0.0)
      throw std::runtime_error("volume moves: tail corrections are not supported on this path");
  out.Box = scaled_geometry(Sims.Box, s, newV, !FF.noCharges);
  const int nc = SC.NComponents.x;
  out.host.assign(nc, HostAtoms());
  out.atoms.resize(nc);
  for (int c = 0; c < nc; ++c) {
    const Atoms& A = Sims.d_a[c];
    HostAtoms& H = out.host[c];
    const size_t n = SC.StoredAtoms[c];
    H.allocate(std::max(n, (size_t)1));
    for (size_t i = 0; i < n; ++i) {
      H.pos[i] = A.pos[i];
      H.scale[i] = A.scale[i];
      H.charge[i] = A.charge[i];
      H.scaleCoul[i] = A.scaleCoul[i];
      H.Type[i] = A.Type[i];
      H.MolID[i] = A.MolID[i];
    }
    if (c >= SC.NComponents.y) {
      const size_t ms = SC.Moleculesize[c];
      for (size_t m = 0; m + 1 <= A.size / ms; ++m) {
        const double3 p0 = A.pos[m * ms];
        const double3 c0{p0.x * s, p0.y * s, p0.z * s};
        for (size_t a = 0; a < ms; ++a) {
          double3 v{A.pos[m * ms + a].x - p0.x, A.pos[m * ms + a].y - p0.y, A.pos[m * ms + a].z - p0.z};
          pbc_host(Sims.Box, v);
          H.pos[m * ms + a] = double3{c0.x + v.x, c0.y + v.y, c0.z + v.z};
        }
      }
    }
    out.atoms[c] = H.view(A.Molsize, A.size);
  }
  out.Box.handle = create_box(out.Box, FF, SC, out.atoms, SC.StoredAtoms);
  grx_energy e{};
  uint8_t ovl = 0;
  const grx_status st = grx_total_energy_overlap(out.Box.handle, &e, &ovl);
  if (st) {
    grx_box_destroy(out.Box.handle);
    check(st, "grx_total_energy_overlap");
  }
  out.overlap = ovl != 0;
  out.E.HHVDW = e.hh_vdw; out.E.HHReal = e.hh_real; out.E.HGVDW = e.hg_vdw; out.E.HGReal = e.hg_real;
  out.E.GGVDW = e.gg_vdw; out.E.GGReal = e.gg_real;
  out.E.HHEwaldE = e.hh_ewald; out.E.HGEwaldE = e.hg_ewald; out.E.GGEwaldE = e.gg_ewald;
}

// Make a scaled box current: its device box replaces the old one, its atoms the mirror's.
static void adopt_scaled(Variables& Vars, size_t systemId, ScaledBox& t) {
  Simulations& Sims = Vars.Sims[systemId];
  Components& SC = Vars.SystemComponents[systemId];
  grx_box_destroy(Sims.Box.handle);
  Sims.Box = t.Box;
  t.Box.handle = nullptr;
  for (int c = SC.NComponents.y; c < SC.NComponents.x; ++c)
    for (size_t i = 0; i < SC.StoredAtoms[c]; ++i) Sims.d_a[c].pos[i] = t.host[c].pos[i];
}

// Adsorbate molecules of a box (Get_TotalNumberOfMolecule_In_Box, mc_box.h:177-189; no
// fractional molecules on this path).
static double molecules_in_box(const Components& SC) {
  double n = 0.0;
  for (int c = SC.NComponents.y; c < SC.NComponents.x; ++c) n += (double)SC.NumberOfMolecule_for_Component[c];
  return n;
}

// VolumeMove (mc_box.h:191-291). The current energy is the box's FP64 total (the reference
// uses its running sum CreateMol_Energy + deltaE, equal to it within the drift).
void VolumeMove(Variables& Vars, size_t systemId) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  SC.VolumeMoveAttempts++;
  uint32_t w[4];
  grx_draw(Vars.Random.Seed, Vars.Random.BoxStream(systemId), SC.Step, GRX_SLOT_VOLUME, w);
  const double OldV = Sims.Box.Volume;
  const double newV = std::exp(std::log(OldV) + SC.VolumeMoveMaxChange * 2.0 * (grx_u01(w[0]) - 0.5));
  const double scale = std::cbrt(newV / OldV);
  ScaledBox t;
  build_scaled(Vars, systemId, scale, newV, t);
  SC.VolumeMoveLastV = newV;
  SC.VolumeMoveLastE = t.E;
  SC.VolumeMoveLastOverlap = t.overlap;
  bool accept = false;
  MoveEnergy dE;
  if (!t.overlap) {
    const MoveEnergy cur = Total_Energy(Sims);
    dE = t.E;
    dE -= cur;
    const double pacc = std::exp((molecules_in_box(SC) + 1.0) * std::log(newV / OldV) -
                                 (dE.total() + SC.Pressure * (newV - OldV)) * SC.Beta);
    accept = grx_u01(w[1]) < pacc;
  }
  if (accept) {
    adopt_scaled(Vars, systemId, t);
    SC.VolumeMoveAccepted++;
    SC.deltaE += dE;
  } else {
    grx_box_destroy(t.Box.handle);
  }
  SC.Step++;
}

// NVTGibbsMove (mc_box.h:319-430): volume passes between boxes 0 and 1 at fixed total; the
// random numbers come from box 0's stream (box choice, ln(VA/VB) change, acceptance).
void NVTGibbsMove(Variables& Vars, Gibbs& G) {
  if (Vars.SystemComponents.size() < 2) throw std::runtime_error("NVTGibbsMove: two boxes needed");
  Components& C0 = Vars.SystemComponents[0];
  uint32_t w[4];
  grx_draw(Vars.Random.Seed, Vars.Random.BoxStream(0), C0.Step, GRX_SLOT_VOLUME, w);
  const size_t sel = grx_u01(w[2]) > 0.5 ? 1 : 0, oth = 1 - sel;
  G.GibbsBoxStats[0] += 1.0;
  const double VA = Vars.Sims[sel].Box.Volume, VB = Vars.Sims[oth].Box.Volume, TotalV = VA + VB;
  const double expdV = std::exp(std::log(VA / VB) + G.MaxGibbsBoxChange * 2.0 * (grx_u01(w[0]) - 0.5));
  const double newVA = expdV * TotalV / (1.0 + expdV), newVB = TotalV - newVA;
  const ForceField& FF = Vars.device_FF;
  const double la = std::pow(std::cbrt(newVA), 2), lb = std::pow(std::cbrt(newVB), 2);
  for (size_t b : {(size_t)0, (size_t)1}) Vars.SystemComponents[b].Step++;
  if (la < 4.0 * FF.CutOffVDW || la < 4.0 * FF.CutOffCoul || lb < 4.0 * FF.CutOffVDW || lb < 4.0 * FF.CutOffCoul)
    return;  // a box would be narrower than twice the cutoff
  const double newV[2] = {sel == 0 ? newVA : newVB, sel == 0 ? newVB : newVA};
  const double oldV[2] = {sel == 0 ? VA : VB, sel == 0 ? VB : VA};
  ScaledBox t[2];
  bool overlap = false;
  MoveEnergy dE[2];
  for (size_t b = 0; b < 2; ++b) {
    build_scaled(Vars, b, std::cbrt(newV[b] / oldV[b]), newV[b], t[b]);
    overlap = overlap || t[b].overlap;
    dE[b] = t[b].E;
    dE[b] -= Total_Energy(Vars.Sims[b]);
  }
  bool accept = false;
  if (!overlap) {
    const double beta = Vars.SystemComponents[sel].Beta;
    const double pacc = std::exp(-beta * (dE[0].total() + dE[1].total()) +
                                 (molecules_in_box(Vars.SystemComponents[sel]) + 1.0) * std::log(newV[sel] / oldV[sel]) +
                                 (molecules_in_box(Vars.SystemComponents[oth]) + 1.0) * std::log(newV[oth] / oldV[oth]));
    accept = grx_u01(w[1]) < pacc;
  }
  for (size_t b = 0; b < 2; ++b) {
    if (accept) {
      adopt_scaled(Vars, b, t[b]);
      Vars.SystemComponents[b].deltaE += dE[b];
    } else {
      grx_box_destroy(t[b].Box.handle);
    }
  }
  if (accept) G.GibbsBoxStats[1] += 1.0;
}

double GetPrefactor(Components& SC, Simulations& Sims, size_t comp, int MoveType) {
  const double bigP = SC.MolFraction[comp] * SC.Pressure * SC.FugacityCoeff[comp] * Sims.Box.Volume;
  const double N = (double)SC.NumberOfMolecule_for_Component[comp];
  if (MoveType == INSERTION) return SC.Beta * bigP / (N + 1.0);
  if (MoveType == DELETION) return N / (SC.Beta * bigP);
  return 0.0;
}

// ------------------------------------------------------------------ CBMC steps
// Rotate_Quaternions (mc_utilities.h:423-457).
static void rotate_quaternion(double3& v, double u, double w1, double w2) {
  const double pi = 3.14159265358979323846;
  const double s1 = std::sin(2 * pi * w1), c1 = std::cos(2 * pi * w1);
  const double s2 = std::sin(2 * pi * w2), c2 = std::cos(2 * pi * w2);
  const double q0 = std::sqrt(1 - u) * s1, q1 = std::sqrt(1 - u) * c1;
  const double q2 = std::sqrt(u) * s2, q3 = std::sqrt(u) * c2;
  const double a01 = q0 * q1, a02 = q0 * q2, a03 = q0 * q3;
  const double a11 = q1 * q1, a12 = q1 * q2, a13 = q1 * q3;
  const double a22 = q2 * q2, a23 = q2 * q3, a33 = q3 * q3;
  const double r0 = 1.0 - 2.0 * (a22 + a33), r1 = 2.0 * (a12 - a03), r2 = 2.0 * (a13 + a02);
  const double r3 = 2.0 * (a12 + a03), r4 = 1.0 - 2.0 * (a11 + a33), r5 = 2.0 * (a23 - a01);
  const double r6 = 2.0 * (a13 - a02), r7 = 2.0 * (a23 + a01), r8 = 1.0 - 2.0 * (a11 + a22);
  const double x = v.x * r0 + v.y * r1 + v.z * r2;
  const double y = v.x * r3 + v.y * r4 + v.z * r5;
  const double z = v.x * r6 + v.y * r7 + v.z * r8;
  v = double3{x, y, z};
}

void CBMC_FirstBead_Finish(Variables& Vars, size_t systemId, CBMC_Variables& CBMC) {
  Components& SC = Vars.SystemComponents[systemId];
  std::vector<double>& Rosen = SC.Rosen;
  bool good = false;
  size_t sel = 0;
  double W = 0.0;
  switch (CBMC.MoveType) {
    case CBMC_INSERTION: case REINSERTION_INSERTION: {
      if (Rosen.empty()) break;
      sel = SelectTrialPosition(Rosen, Vars, systemId, 0);
      for (double& r : Rosen) r = std::exp(r);
      W = std::accumulate(Rosen.begin(), Rosen.end(), 0.0);
      if (W < 1e-150) break;
      good = true;
      break;
    }
    case IDENTITY_SWAP_NEW: {  // one trial, the swapped molecule's first bead
      if (Rosen.empty()) break;
      for (double& r : Rosen) r = std::exp(r);
      W = std::accumulate(Rosen.begin(), Rosen.end(), 0.0);
      if (W < 1e-150) break;
      good = true;
      break;
    }
    default: {  // CBMC_DELETION, REINSERTION_RETRACE, IDENTITY_SWAP_OLD: the existing bead, no selection
      if (Rosen.empty()) break;
      for (double& r : Rosen) r = std::exp(r);
      W = std::accumulate(Rosen.begin(), Rosen.end(), 0.0);
      good = true;
      break;
    }
  }
  if (!good) return;
  if (CBMC.MoveType == REINSERTION_INSERTION) CBMC.StoredR = W - Rosen[sel];
  if (CBMC.MoveType == REINSERTION_RETRACE) W += CBMC.StoredR;
  // an identity swap's first bead is a single trial: not averaged (mc_widom.h:368-370)
  const bool swap = CBMC.MoveType == IDENTITY_SWAP_NEW || CBMC.MoveType == IDENTITY_SWAP_OLD;
  double avg = swap ? W : W / (double)Vars.Widom[systemId].NumberWidomTrials;
  if (!Vars.device_FF.VDWRealBias) avg *= std::exp(-SC.Beta * (SC.TrialEnergies[sel].HGReal + SC.TrialEnergies[sel].GGReal));
  CBMC.selectedTrial = SC.Trialindex[sel];
  CBMC.SuccessConstruction = true;
  CBMC.FirstBeadEnergy = SC.TrialEnergies[sel];
  CBMC.Rosenbluth = avg;
}

// mc_widom.h:385-507: trial positions (get_random_trial_position, :122-213), energies, finish.
void Widom_Move_FirstBead_PARTIAL(Variables& Vars, size_t systemId, CBMC_Variables& CBMC) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  const size_t comp = SC.TempVal.component;
  const size_t ms = SC.Moleculesize[comp];
  const Atoms& A = Sims.d_a[comp];
  size_t ntrials = Vars.Widom[systemId].NumberWidomTrials;
  size_t molid = SC.TempVal.molecule;
  const bool retrace = CBMC.MoveType == CBMC_DELETION || CBMC.MoveType == REINSERTION_RETRACE ||
                       CBMC.MoveType == IDENTITY_SWAP_OLD;
  const bool swap_new = CBMC.MoveType == IDENTITY_SWAP_NEW;
  if (CBMC.MoveType == CBMC_INSERTION || swap_new) molid = SC.NumberOfMolecule_for_Component[comp];
  if (CBMC.MoveType == REINSERTION_RETRACE || CBMC.MoveType == IDENTITY_SWAP_OLD || swap_new) ntrials = 1;
  const size_t start = SC.TempVal.molecule * ms;
  for (size_t t = 0; t < ntrials; ++t) {
    if (swap_new) {
      // the caller placed the swapped molecule's first bead in New.pos[0] (mc_swap_moves.h:267)
    } else if (retrace && t == 0) {
      Sims.New.pos[0] = A.pos[start];
    } else {
      uint32_t r[4];
      grx_draw(Vars.Random.Seed, Vars.Random.BoxStream(systemId), SC.Step, GRX_SLOT_FIRST + (uint32_t)t, r);
      Sims.New.pos[t] = double3{Sims.Box.Cell[0] * grx_u01(r[0]), Sims.Box.Cell[4] * grx_u01(r[1]),
                                Sims.Box.Cell[8] * grx_u01(r[2])};
    }
    Sims.New.scale[t] = SC.TempVal.Scale.x;
    Sims.New.scaleCoul[t] = SC.TempVal.Scale.y;
    Sims.New.charge[t] = A.charge[0];
    Sims.New.Type[t] = A.Type[0];
    Sims.New.MolID[t] = molid;
  }
  CBMC_PairwiseInteractions(Vars, systemId, SC, Sims, ntrials, 1);
  CBMC_FirstBead_Finish(Vars, systemId, CBMC);
  if (CBMC.SuccessConstruction) Sims.Old.pos[0] = Sims.New.pos[CBMC.selectedTrial];
}

// mc_widom.h:509-614 with get_random_trial_orientation (:215-303).
void Widom_Move_Chain_PARTIAL(Variables& Vars, size_t systemId, CBMC_Variables& CBMC) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  const size_t comp = SC.TempVal.component;
  const size_t ms = SC.Moleculesize[comp], chain = ms - 1;
  const size_t no = Vars.Widom[systemId].NumberWidomTrialsOrientations;
  const Atoms& A = Sims.d_a[comp];
  const bool retrace = CBMC.MoveType == CBMC_DELETION || CBMC.MoveType == REINSERTION_RETRACE ||
                       CBMC.MoveType == IDENTITY_SWAP_OLD;
  const bool grow_new = CBMC.MoveType == CBMC_INSERTION || CBMC.MoveType == IDENTITY_SWAP_NEW;
  const size_t molid = grow_new ? SC.NumberOfMolecule_for_Component[comp] : SC.TempVal.molecule;
  const size_t start = SC.TempVal.molecule * ms + 1;
  // a retrace that follows a growth in the same move draws its own orientations
  const uint32_t slot = (CBMC.MoveType == REINSERTION_RETRACE || CBMC.MoveType == IDENTITY_SWAP_OLD)
                            ? GRX_SLOT_RETRACE : GRX_SLOT_ORIENT;
  const double3 fb = Sims.Old.pos[0];
  for (size_t o = 0; o < no; ++o) {
    uint32_t r[4];
    grx_draw(Vars.Random.Seed, Vars.Random.BoxStream(systemId), SC.Step, slot + (uint32_t)o, r);
    for (size_t a = 0; a < chain; ++a) {
      const size_t i = o * chain + a;
      if (retrace && o == 0) {
        Sims.New.pos[i] = A.pos[start + a];
      } else {
        double3 v{A.pos[1 + a].x - A.pos[0].x, A.pos[1 + a].y - A.pos[0].y, A.pos[1 + a].z - A.pos[0].z};
        rotate_quaternion(v, grx_u01(r[0]), grx_u01(r[1]), grx_u01(r[2]));
        Sims.New.pos[i] = double3{fb.x + v.x, fb.y + v.y, fb.z + v.z};
      }
      Sims.New.scale[i] = SC.TempVal.Scale.x;
      Sims.New.scaleCoul[i] = SC.TempVal.Scale.y;
      Sims.New.charge[i] = A.charge[1 + a];
      Sims.New.Type[i] = A.Type[1 + a];
      Sims.New.MolID[i] = molid;
    }
  }
  CBMC_PairwiseInteractions(Vars, systemId, SC, Sims, no, chain);
  std::vector<double>& Rosen = SC.Rosen;
  bool good = false;
  size_t sel = 0;
  double W = 0.0;
  if (!Rosen.empty()) {
    if (!retrace) sel = SelectTrialPosition(Rosen, Vars, systemId, 1);
    for (double& x : Rosen) x = std::exp(x);
    W = std::accumulate(Rosen.begin(), Rosen.end(), 0.0);
    good = retrace || !(W < 1e-150);
  }
  if (!good) {
    CBMC.Rosenbluth = 0.0;
    CBMC.SuccessConstruction = false;
    return;
  }
  double avg = W / (double)no;
  if (!Vars.device_FF.VDWRealBias) avg *= std::exp(-SC.Beta * (SC.TrialEnergies[sel].HGReal + SC.TrialEnergies[sel].GGReal));
  CBMC.selectedTrialOrientation = SC.Trialindex[sel];
  CBMC.SuccessConstruction = true;
  CBMC.ChainEnergy = SC.TrialEnergies[sel];
  CBMC.Rosenbluth *= avg;
}

// ------------------------------------------------------------------ host mirror updates
static void write_molecule(Variables& Vars, size_t systemId, size_t comp, size_t mol, const std::vector<double>& pos) {
  Simulations& Sims = Vars.Sims[systemId];
  Components& SC = Vars.SystemComponents[systemId];
  const size_t ms = SC.Moleculesize[comp];
  Atoms& A = Sims.d_a[comp];
  std::vector<double> q(ms);
  std::vector<size_t> ty(ms);
  for (size_t a = 0; a < ms; ++a) {  // a molecule's charges and types follow the component's template
    q[a] = A.charge[a];
    ty[a] = A.Type[a];
  }
  check(grx_box_write_molecule(Sims.Box.handle, (int32_t)comp, mol, pos.data(), q.data(), ty.data()),
        "grx_box_write_molecule");
  for (size_t a = 0; a < ms; ++a) {
    const size_t i = mol * ms + a;
    A.pos[i] = double3{pos[3 * a], pos[3 * a + 1], pos[3 * a + 2]};
    A.charge[i] = q[a];
    A.Type[i] = ty[a];
    A.MolID[i] = mol;
    A.scale[i] = 1.0;
    A.scaleCoul[i] = 1.0;
  }
  if (mol == SC.NumberOfMolecule_for_Component[comp]) {
    SC.NumberOfMolecule_for_Component[comp]++;
    A.size += ms;
  }
}

static void remove_molecule(Variables& Vars, size_t systemId, size_t comp, size_t mol) {
  Simulations& Sims = Vars.Sims[systemId];
  Components& SC = Vars.SystemComponents[systemId];
  const size_t ms = SC.Moleculesize[comp];
  Atoms& A = Sims.d_a[comp];
  check(grx_box_remove_molecule(Sims.Box.handle, (int32_t)comp, mol), "grx_box_remove_molecule");
  const size_t last = SC.NumberOfMolecule_for_Component[comp] - 1;
  if (last != mol)
    for (size_t a = 0; a < ms; ++a) {
      const size_t d = mol * ms + a, s = last * ms + a;
      A.pos[d] = A.pos[s]; A.charge[d] = A.charge[s]; A.Type[d] = A.Type[s];
      A.scale[d] = A.scale[s]; A.scaleCoul[d] = A.scaleCoul[s]; A.MolID[d] = mol;
    }
  SC.NumberOfMolecule_for_Component[comp]--;
  A.size -= ms;
}

// ------------------------------------------------------------------ moves
// RotationAroundAxis (mc_utilities.h:459-481) for a coordinate axis.
static void rotate_axis(double3& v, double theta, int axis) {
  const double c = std::cos(theta), w = 1.0 - c, s = std::sin(theta);
  const double ax = axis == 0, ay = axis == 1, az = axis == 2;
  const double r0 = ax * ax * w + c, r1 = ax * ay * w + az * s, r2 = ax * az * w - ay * s;
  const double r3 = ax * ay * w - az * s, r4 = ay * ay * w + c, r5 = ay * az * w + ax * s;
  const double r6 = ax * az * w + ay * s, r7 = ay * az * w - ax * s, r8 = az * az * w + c;
  v = double3{v.x * r0 + v.y * r1 + v.z * r2, v.x * r3 + v.y * r4 + v.z * r5, v.x * r6 + v.y * r7 + v.z * r8};
}

double2 GPU_EwaldDifference_LambdaChange(Simulations& Sims, ForceField& FF, Components& SC, size_t comp,
                                         size_t start_position, double2 oldScale, double2 newScale, int MoveType) {
  if (FF.noCharges && !SC.hasPartialCharge[comp]) return double2{};
  const size_t ms = SC.Moleculesize[comp];
  const Atoms& A = Sims.d_a[comp];
  std::vector<double> pos(3 * ms), q(ms);
  for (size_t a = 0; a < ms; ++a) {
    pos[3 * a] = A.pos[start_position + a].x;
    pos[3 * a + 1] = A.pos[start_position + a].y;
    pos[3 * a + 2] = A.pos[start_position + a].z;
    q[a] = A.charge[start_position + a];
  }
  // the second step of a CB/CFC deletion starts from the staged vector (:775-778)
  const int use_staged = MoveType == CBCF_DELETION ? 1 : 0;
  double out2[2];
  check(grx_ewald_delta_lambda(Sims.Box.handle, (int32_t)comp, pos.data(), q.data(), ms, oldScale.y, newScale.y,
                               use_staged, out2),
        "grx_ewald_delta_lambda");
  return double2{out2[0], out2[1]};
}

double2 GPU_EwaldDifference_IdentitySwap(Simulations& Sims, ForceField& FF, Components& SC, size_t OLDComponent,
                                         size_t NEWComponent, size_t UpdateLocation,
                                         const std::vector<double3>& NewPositions) {
  if (FF.noCharges && !SC.hasPartialCharge[NEWComponent] && !SC.hasPartialCharge[OLDComponent]) return double2{};
  std::vector<double> op, oq;
  molecule_atoms(Sims, SC, OLDComponent, UpdateLocation, op, oq);
  const size_t mn = SC.Moleculesize[NEWComponent];
  const Atoms& T = Sims.d_a[NEWComponent];  // charges of the new species: its slot-0 storage
  std::vector<double> np(3 * mn), nq(mn);
  for (size_t a = 0; a < mn; ++a) {
    np[3 * a] = NewPositions[a].x; np[3 * a + 1] = NewPositions[a].y; np[3 * a + 2] = NewPositions[a].z;
    nq[a] = T.charge[a];
  }
  double out2[2];
  check(grx_ewald_delta_identity_swap(Sims.Box.handle, (int32_t)OLDComponent, (int32_t)NEWComponent, op.data(),
                                      oq.data(), oq.size(), np.data(), nq.data(), mn, out2),
        "grx_ewald_delta_identity_swap");
  return double2{out2[0], out2[1]};
}

MoveEnergy CBCF_LambdaChange(Variables& Vars, size_t systemId, size_t SelectedMolInComponent,
                             size_t SelectedComponent, double2 oldScale, double2 newScale, size_t& start_position,
                             int MoveType, bool& SuccessConstruction) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  const size_t comp = SelectedComponent, ms = SC.Moleculesize[comp];
  start_position = SelectedMolInComponent * ms;
  const Atoms& A = Sims.d_a[comp];
  // Calculate_Single_Body_Energy_VDWReal_LambdaChange (VDW_Coulomb.cu:843-1009): the same
  // positions with the stored (old) scales and with newScale
  std::vector<double> q(ms), sco(ms), scco(ms), scn(ms, newScale.x), sccn(ms, newScale.y);
  std::vector<size_t> ty(ms);
  for (size_t a = 0; a < ms; ++a) {
    q[a] = A.charge[start_position + a];
    sco[a] = A.scale[start_position + a];
    scco[a] = A.scaleCoul[start_position + a];
    ty[a] = A.Type[start_position + a];
  }
  grx_trials to{}, tn{};
  to.pos = tn.pos = reinterpret_cast<const double*>(A.pos + start_position);
  to.scale = sco.data();
  to.scale_coul = scco.data();
  tn.scale = scn.data();
  tn.scale_coul = sccn.data();
  to.charge = tn.charge = q.data();
  to.type = tn.type = ty.data();
  to.molid = tn.molid = SelectedMolInComponent;
  to.ntrials = tn.ntrials = 1;
  to.chainsize = tn.chainsize = ms;
  double e6[6];
  uint8_t flag = 0;
  check(grx_single_body_energy(Sims.Box.handle, &to, &tn, (int32_t)comp, 1, 1, Vars.Precision, e6, &flag),
        "grx_single_body_energy");
  MoveEnergy tot;
  SuccessConstruction = flag == 0;
  if (!SuccessConstruction) return tot;
  tot.HHVDW = e6[0]; tot.HHReal = e6[1]; tot.HGVDW = e6[2];
  tot.HGReal = e6[3]; tot.GGVDW = e6[4]; tot.GGReal = e6[5];
  if (!Vars.device_FF.noCharges && SC.hasPartialCharge[comp]) {
    const double2 E = GPU_EwaldDifference_LambdaChange(Sims, Vars.device_FF, SC, comp, start_position, oldScale,
                                                       newScale, MoveType);
    if (comp >= (size_t)SC.NComponents.y) { tot.GGEwaldE = E.x; tot.HGEwaldE = E.y; }
    else { tot.HHEwaldE = E.x; tot.HGEwaldE = E.y; }
  }
  // TailCorrectionDifference (TailCorrection_Energy_Functions.h:35-84): CB/CFC insertion and
  // deletion refuse tail corrections; a plain lambda change takes the insertion sign.
  const double tail = SC.TailCorrectionInsert.empty() ? 0.0 : SC.TailCorrectionInsert[comp];
  if (tail != 0.0 && (MoveType == CBCF_INSERTION || MoveType == CBCF_DELETION))
    throw std::runtime_error("TAIL CORRECTIONS NOT READY FOR CBCF MOVES!");
  tot.TailE = tail;
  return tot;
}

MoveEnergy SingleBodyMove(Variables& Vars, size_t systemId, int MoveType, double RANDOM) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  const size_t comp = SC.TempVal.component, mol = SC.TempVal.molecule;
  const size_t ms = SC.Moleculesize[comp], m0 = mol * ms;
  Move_Statistics& MS = SC.Moves[comp];
  MS.Record_Move_Total(MoveType);
  Atoms& A = Sims.d_a[comp];
  uint32_t w2[4];
  grx_draw(Vars.Random.Seed, Vars.Random.BoxStream(systemId), SC.Step, GRX_SLOT_DISP, w2);
  // get_new_position (mc_utilities.h:485-540)
  if (MoveType == TRANSLATION) {
    const double dx = MS.MaxTranslation.x * 2.0 * (grx_u01(w2[0]) - 0.5);
    const double dy = MS.MaxTranslation.y * 2.0 * (grx_u01(w2[1]) - 0.5);
    const double dz = MS.MaxTranslation.z * 2.0 * (grx_u01(w2[2]) - 0.5);
    for (size_t a = 0; a < ms; ++a)
      Sims.New.pos[a] = double3{A.pos[m0 + a].x + dx, A.pos[m0 + a].y + dy, A.pos[m0 + a].z + dz};
  } else {
    const double ang[3] = {MS.MaxRotation.x * 2.0 * (grx_u01(w2[0]) - 0.5),
                           MS.MaxRotation.y * 2.0 * (grx_u01(w2[1]) - 0.5),
                           MS.MaxRotation.z * 2.0 * (grx_u01(w2[2]) - 0.5)};
    const double3 p0 = A.pos[m0];
    for (size_t a = 0; a < ms; ++a) {
      double3 v{A.pos[m0 + a].x - p0.x, A.pos[m0 + a].y - p0.y, A.pos[m0 + a].z - p0.z};
      rotate_axis(v, ang[0], 0);
      rotate_axis(v, ang[1], 1);
      rotate_axis(v, ang[2], 2);
      Sims.New.pos[a] = double3{v.x + p0.x, v.y + p0.y, v.z + p0.z};
    }
  }
  // Calculate_Single_Body_Energy_VDWReal (VDW_Coulomb.cu:626-841) through the ABI
  std::vector<double> q(ms), ones(ms, 1.0);
  std::vector<size_t> ty(ms);
  for (size_t a = 0; a < ms; ++a) {
    q[a] = A.charge[m0 + a];
    ty[a] = A.Type[m0 + a];
  }
  grx_trials to{}, tn{};
  to.pos = reinterpret_cast<const double*>(A.pos + m0);
  tn.pos = reinterpret_cast<const double*>(Sims.New.pos);
  to.scale = tn.scale = ones.data();
  to.charge = tn.charge = q.data();
  to.scale_coul = tn.scale_coul = ones.data();
  to.type = tn.type = ty.data();
  to.molid = tn.molid = mol;
  to.ntrials = tn.ntrials = 1;
  to.chainsize = tn.chainsize = ms;
  double e6[6];
  uint8_t flag = 0;
  check(grx_single_body_energy(Sims.Box.handle, &to, &tn, (int32_t)comp, 1, 1, Vars.Precision, e6, &flag),
        "grx_single_body_energy");
  MoveEnergy energy;
  if (flag) return energy;
  energy.HHVDW = e6[0]; energy.HHReal = e6[1]; energy.HGVDW = e6[2];
  energy.HGReal = e6[3]; energy.GGVDW = e6[4]; energy.GGReal = e6[5];
  const bool charged = !Vars.device_FF.noCharges && SC.hasPartialCharge[comp];
  double ew = 0.0;
  if (charged) {
    const double2 E = GPU_EwaldDifference_General(Sims, Vars.device_FF, SC, comp, MoveType, m0, SC.TempVal.Scale);
    energy.GGEwaldE = E.x;
    energy.HGEwaldE = E.y;
    ew = E.x + E.y;
  }
  const double tot = e6[0] + e6[1] + e6[2] + e6[3] + e6[4] + e6[5] + ew;
  // SingleBody_Acceptance (mc_single_particle.h:234-293)
  if (RANDOM < std::exp(-SC.Beta * tot)) {
    std::vector<double> np(3 * ms);
    for (size_t a = 0; a < ms; ++a) {
      np[3 * a] = Sims.New.pos[a].x; np[3 * a + 1] = Sims.New.pos[a].y; np[3 * a + 2] = Sims.New.pos[a].z;
    }
    write_molecule(Vars, systemId, comp, mol, np);
    if (charged) Update_Vector_Ewald(Sims.Box, false, SC, comp);
    MS.Record_Move_Accept(MoveType);
    return energy;
  }
  return MoveEnergy();
}

// Insertion_Body (mc_swap_utilities.h:3-132)
static MoveEnergy Insertion_Body(Variables& Vars, size_t systemId, CBMC_Variables& CBMC) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  const size_t comp = SC.TempVal.component;
  CBMC.MoveType = CBMC_INSERTION;
  MoveEnergy energy;
  Widom_Move_FirstBead_PARTIAL(Vars, systemId, CBMC);
  if (!CBMC.SuccessConstruction || CBMC.Rosenbluth <= 1e-150) {
    CBMC.SuccessConstruction = false;
    return energy;
  }
  if (SC.Moleculesize[comp] > 1) {
    Widom_Move_Chain_PARTIAL(Vars, systemId, CBMC);
    if (!CBMC.SuccessConstruction || CBMC.Rosenbluth <= 1e-150) {
      CBMC.SuccessConstruction = false;
      return energy;
    }
  }
  energy = CBMC.FirstBeadEnergy + CBMC.ChainEnergy;
  if (!Vars.device_FF.noCharges && SC.hasPartialCharge[comp]) {
    const double2 E = GPU_EwaldDifference_General(Sims, Vars.device_FF, SC, comp, INSERTION,
                                                  CBMC.selectedTrialOrientation, SC.TempVal.Scale);
    energy.GGEwaldE = E.x;
    energy.HGEwaldE = E.y;
    CBMC.Rosenbluth *= std::exp(-SC.Beta * (E.x + E.y));
  }
  energy.TailE = SC.TailCorrectionInsert.empty() ? 0.0 : SC.TailCorrectionInsert[comp];
  CBMC.Rosenbluth *= std::exp(-SC.Beta * energy.TailE);
  return energy;
}

void InsertionMove::Initialize() {
  InsertionVariables.clear();
  energy.zero();
  preFactor = Pacc = 0.0;
  Accept = false;
}

void InsertionMove::Calculate(Variables& Vars, size_t systemId) {
  Components& SC = Vars.SystemComponents[systemId];
  const size_t comp = SC.TempVal.component;
  energy = Insertion_Body(Vars, systemId, InsertionVariables);
  if (!InsertionVariables.SuccessConstruction) {
    Pacc = preFactor = 0.0;
    return;
  }
  preFactor = GetPrefactor(SC, Vars.Sims[systemId], comp, INSERTION);
  Pacc = preFactor * InsertionVariables.Rosenbluth / SC.IdealRosenbluthWeight[comp];
  if (InsertionVariables.Rosenbluth <= 1e-150) Pacc = 0.0;
}

void InsertionMove::Acceptance(Variables& Vars, size_t systemId, double RANDOM) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  const size_t comp = SC.TempVal.component;
  if (!InsertionVariables.SuccessConstruction || !(RANDOM < Pacc)) {
    energy.zero();
    return;
  }
  const size_t N = SC.NumberOfMolecule_for_Component[comp];
  if ((N + 1) * SC.Moleculesize[comp] > SC.Allocate_size[comp]) {  // no room: refuse, as the device driver does
    energy.zero();
    return;
  }
  Accept = true;
  Commit(Vars, systemId);
}

// AcceptInsertion (mc_utilities.h:357-385): the grown molecule stored, S(k) committed.
void InsertionMove::Commit(Variables& Vars, size_t systemId) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  const size_t comp = SC.TempVal.component;
  std::vector<double> pos, qs;
  if (SC.Moleculesize[comp] > 1) {
    grown_atoms(Sims, SC, comp, InsertionVariables.selectedTrialOrientation, pos, qs);
  } else {
    pos = {Sims.Old.pos[0].x, Sims.Old.pos[0].y, Sims.Old.pos[0].z};
  }
  write_molecule(Vars, systemId, comp, SC.NumberOfMolecule_for_Component[comp], pos);
  if (!Vars.device_FF.noCharges && SC.hasPartialCharge[comp]) Update_Vector_Ewald(Sims.Box, false, SC, comp);
}

MoveEnergy InsertionMove::Run(Variables& Vars, size_t systemId, double RANDOM) {
  Components& SC = Vars.SystemComponents[systemId];
  const size_t comp = SC.TempVal.component;
  Initialize();
  SC.Moves[comp].Record_Move_Total(INSERTION);
  Calculate(Vars, systemId);
  if (!InsertionVariables.SuccessConstruction) return energy;
  Acceptance(Vars, systemId, RANDOM);
  if (Accept) SC.Moves[comp].Record_Move_Accept(INSERTION);
  return energy;
}

double InsertionMove::WidomMove(Variables& Vars, size_t systemId) {
  Initialize();
  Calculate(Vars, systemId);
  return InsertionVariables.SuccessConstruction ? InsertionVariables.Rosenbluth : 0.0;
}

void DeletionMove::Initialize() {
  DeletionVariables.clear();
  energy.zero();
  preFactor = Pacc = 0.0;
  Accept = false;
}

// Deletion_Body (mc_swap_utilities.h:135-225) + DeletionMove::Calculate (move_struct.h:122-132)
void DeletionMove::Calculate(Variables& Vars, size_t systemId) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  const size_t comp = SC.TempVal.component;
  CBMC_Variables& C = DeletionVariables;
  C.MoveType = CBMC_DELETION;
  Widom_Move_FirstBead_PARTIAL(Vars, systemId, C);
  if (!C.SuccessConstruction || C.Rosenbluth <= 1e-150) {
    C.SuccessConstruction = false;
    return;
  }
  if (SC.Moleculesize[comp] > 1) {
    Widom_Move_Chain_PARTIAL(Vars, systemId, C);
    if (!C.SuccessConstruction || C.Rosenbluth <= 1e-150) {
      C.SuccessConstruction = false;
      return;
    }
  }
  energy = C.FirstBeadEnergy + C.ChainEnergy;
  energy.take_negative();
  if (!Vars.device_FF.noCharges && SC.hasPartialCharge[comp]) {
    const double2 E = GPU_EwaldDifference_General(Sims, Vars.device_FF, SC, comp, DELETION,
                                                  SC.TempVal.molecule * SC.Moleculesize[comp], SC.TempVal.Scale);
    energy.GGEwaldE = E.x;
    energy.HGEwaldE = E.y;
    C.Rosenbluth /= std::exp(-SC.Beta * (E.x + E.y));
  }
  energy.TailE = SC.TailCorrectionInsert.empty() ? 0.0 : -SC.TailCorrectionInsert[comp];
  C.Rosenbluth /= std::exp(-SC.Beta * energy.TailE);  // TailE: the deletion difference (mc_swap_utilities.h:197-200)
  preFactor = GetPrefactor(SC, Sims, comp, DELETION);
  Pacc = preFactor * SC.IdealRosenbluthWeight[comp] / C.Rosenbluth;
}

void DeletionMove::Acceptance(Variables& Vars, size_t systemId, double RANDOM) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  const size_t comp = SC.TempVal.component;
  if (!DeletionVariables.SuccessConstruction || !(RANDOM < Pacc)) {
    energy.zero();
    return;
  }
  Accept = true;
  Commit(Vars, systemId);
}

// AcceptDeletion (mc_utilities.h:387-417): the last molecule moved into the slot, S(k) committed.
void DeletionMove::Commit(Variables& Vars, size_t systemId) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  const size_t comp = SC.TempVal.component;
  remove_molecule(Vars, systemId, comp, SC.TempVal.molecule);
  if (!Vars.device_FF.noCharges && SC.hasPartialCharge[comp]) Update_Vector_Ewald(Sims.Box, false, SC, comp);
}

MoveEnergy DeletionMove::Run(Variables& Vars, size_t systemId, double RANDOM) {
  Components& SC = Vars.SystemComponents[systemId];
  const size_t comp = SC.TempVal.component;
  Initialize();
  SC.Moves[comp].Record_Move_Total(DELETION);
  Calculate(Vars, systemId);
  if (!DeletionVariables.SuccessConstruction) return energy;
  Acceptance(Vars, systemId, RANDOM);
  if (Accept) SC.Moves[comp].Record_Move_Accept(DELETION);
  return energy;
}

void ReinsertionMove::Initialize() {
  InsertionVariables.clear();
  DeletionVariables.clear();
  energy.zero();
  old_energy.zero();
  Pacc = 0.0;
  Accept = false;
}

// move_struct.h:184-274
void ReinsertionMove::Calculate_Insertion(Variables& Vars, size_t systemId) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  const size_t comp = SC.TempVal.component;
  const size_t ms = SC.Moleculesize[comp];
  CBMC_Variables& C = InsertionVariables;
  C.MoveType = REINSERTION_INSERTION;
  Widom_Move_FirstBead_PARTIAL(Vars, systemId, C);
  if (C.Rosenbluth <= 1e-150) C.SuccessConstruction = false;
  if (!C.SuccessConstruction) return;
  if (ms > 1) {
    Widom_Move_Chain_PARTIAL(Vars, systemId, C);
    if (C.Rosenbluth <= 1e-150) C.SuccessConstruction = false;
    if (!C.SuccessConstruction) return;
  }
  // StoreNewLocation_Reinsertion: the grown molecule, kept while the retrace reuses New
  NewPositions.assign(ms, double3{});
  NewPositions[0] = Sims.Old.pos[0];
  for (size_t a = 1; a < ms; ++a) NewPositions[a] = Sims.New.pos[C.selectedTrialOrientation * (ms - 1) + (a - 1)];
  energy = C.FirstBeadEnergy + C.ChainEnergy;
}

// move_struct.h:276-290
void ReinsertionMove::Calculate_Deletion(Variables& Vars, size_t systemId) {
  Components& SC = Vars.SystemComponents[systemId];
  const size_t comp = SC.TempVal.component;
  CBMC_Variables& C = DeletionVariables;
  C.MoveType = REINSERTION_RETRACE;
  C.StoredR = InsertionVariables.StoredR;
  Widom_Move_FirstBead_PARTIAL(Vars, systemId, C);
  if (!C.SuccessConstruction) return;
  if (SC.Moleculesize[comp] > 1) Widom_Move_Chain_PARTIAL(Vars, systemId, C);
  old_energy = C.FirstBeadEnergy + C.ChainEnergy;
}

// move_struct.h:292-336
void ReinsertionMove::Calculate_AdjustRosenbluth(Variables& Vars, size_t systemId) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  const size_t comp = SC.TempVal.component;
  const size_t ms = SC.Moleculesize[comp];
  if (!Vars.device_FF.noCharges && SC.hasPartialCharge[comp]) {
    for (size_t a = 0; a < ms; ++a) Sims.Old.pos[1 + a] = NewPositions[a];
    const double2 E = GPU_EwaldDifference_General(Sims, Vars.device_FF, SC, comp, REINSERTION,
                                                  SC.TempVal.molecule * ms, SC.TempVal.Scale);
    energy.GGEwaldE = E.x;
    energy.HGEwaldE = E.y;
    InsertionVariables.Rosenbluth *= std::exp(-SC.Beta * (E.x + E.y));
  }
}

// move_struct.h:338-376
void ReinsertionMove::Acceptance(Variables& Vars, size_t systemId, double RANDOM) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  const size_t comp = SC.TempVal.component;
  const size_t ms = SC.Moleculesize[comp];
  Pacc = InsertionVariables.Rosenbluth / DeletionVariables.Rosenbluth;
  if (!InsertionVariables.SuccessConstruction || InsertionVariables.Rosenbluth <= 1e-150 || !(RANDOM < Pacc)) {
    energy.zero();
    return;
  }
  Accept = true;
  std::vector<double> pos(3 * ms);
  for (size_t a = 0; a < ms; ++a) {
    pos[3 * a] = NewPositions[a].x; pos[3 * a + 1] = NewPositions[a].y; pos[3 * a + 2] = NewPositions[a].z;
  }
  write_molecule(Vars, systemId, comp, SC.TempVal.molecule, pos);  // Update_Reinsertion_data
  if (!Vars.device_FF.noCharges && SC.hasPartialCharge[comp]) Update_Vector_Ewald(Sims.Box, false, SC, comp);
}

MoveEnergy ReinsertionMove::Run(Variables& Vars, size_t systemId, double RANDOM) {
  Components& SC = Vars.SystemComponents[systemId];
  const size_t comp = SC.TempVal.component;
  Initialize();
  SC.Moves[comp].Record_Move_Total(REINSERTION);
  Calculate_Insertion(Vars, systemId);
  if (!InsertionVariables.SuccessConstruction) return MoveEnergy();
  Calculate_Deletion(Vars, systemId);
  if (!DeletionVariables.SuccessConstruction) return MoveEnergy();
  energy -= old_energy;
  Calculate_AdjustRosenbluth(Vars, systemId);
  Acceptance(Vars, systemId, RANDOM);
  if (Accept) SC.Moves[comp].Record_Move_Accept(REINSERTION);
  return energy;
}

// RunMoves (axpy.cu:102-298) for the moves of this path.
MoveEnergy RunMoves(Variables& Vars, size_t systemId, size_t comp) {
  Components& SC = Vars.SystemComponents[systemId];
  Move_Statistics& MS = SC.Moves[comp];
  uint32_t w[4];
  grx_draw(Vars.Random.Seed, Vars.Random.BoxStream(systemId), SC.Step, GRX_SLOT_MOVE, w);
  const size_t N = SC.NumberOfMolecule_for_Component[comp];
  SC.TempVal.component = comp;
  SC.TempVal.molecule = (size_t)(grx_u01(w[0]) * (double)N);
  SC.TempVal.Scale = double2{1.0, 1.0};
  const double r = grx_u01(w[1]);
  const double uacc = grx_u01(w[3]);
  MoveEnergy dE;
  if (r < MS.TranslationProb) {
    if (N > 0) dE = SingleBodyMove(Vars, systemId, TRANSLATION, uacc);
  } else if (r < MS.RotationProb) {
    if (N > 0) dE = SingleBodyMove(Vars, systemId, ROTATION, uacc);
  } else if (r < MS.ReinsertionProb) {
    if (N > 0) {
      ReinsertionMove m;
      dE = m.Run(Vars, systemId, uacc);
    }
  } else if (r < MS.IdentitySwapProb) {
    dE = IdentitySwapMove(Vars, systemId);
  } else if (r < MS.SwapProb) {
    if (grx_u01(w[2]) < 0.5) {
      InsertionMove m;
      dE = m.Run(Vars, systemId, uacc);
    } else if (N > 0) {
      DeletionMove m;
      dE = m.Run(Vars, systemId, uacc);
    }
  }
  SC.deltaE += dE;
  SC.Step++;
  return dE;
}

// ------------------------------------------------------------------ identity swap, Gibbs transfer
static std::vector<double> flat_positions(const std::vector<double3>& p) {
  std::vector<double> f(3 * p.size());
  for (size_t a = 0; a < p.size(); ++a) {
    f[3 * a] = p[a].x; f[3 * a + 1] = p[a].y; f[3 * a + 2] = p[a].z;
  }
  return f;
}

// IdentitySwapMove (mc_swap_moves.h:199-420). The reference redraws the old and the new
// component together until the old one holds a molecule, so the old component is uniform over
// the adsorbate components that hold molecules and the new one uniform over all adsorbate
// components; one Philox draw (GRX_SLOT_SWAP) gives both here.
MoveEnergy IdentitySwapMove(Variables& Vars, size_t systemId) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  const size_t c0 = (size_t)SC.NComponents.y, nc = (size_t)SC.NComponents.x;
  std::vector<size_t> have;
  for (size_t c = c0; c < nc; ++c)
    if (SC.NumberOfMolecule_for_Component[c] > 0) have.push_back(c);
  if (have.empty()) return MoveEnergy();
  uint32_t w[4];
  grx_draw(Vars.Random.Seed, Vars.Random.BoxStream(systemId), SC.Step, GRX_SLOT_SWAP, w);
  const size_t OLD = have[std::min(have.size() - 1, (size_t)(grx_u01(w[0]) * (double)have.size()))];
  const size_t NEW = c0 + std::min(nc - c0 - 1, (size_t)(grx_u01(w[1]) * (double)(nc - c0)));
  const size_t oldmol = (size_t)(grx_u01(w[2]) * (double)SC.NumberOfMolecule_for_Component[OLD]);
  const size_t newmol = SC.NumberOfMolecule_for_Component[NEW];
  const size_t ms_old = SC.Moleculesize[OLD], ms_new = SC.Moleculesize[NEW];
  if (SC.TailCorrectionInsert[OLD] != 0.0 || SC.TailCorrectionInsert[NEW] != 0.0)
    throw std::runtime_error("IdentitySwapMove: tail corrections are not supported on this path");
  for (size_t c : {OLD, NEW}) {
    SC.Moves[c].IdentitySwap_Total_TO.resize(nc, 0);
    SC.Moves[c].IdentitySwap_Acc_TO.resize(nc, 0);
  }
  SC.Moves[OLD].IdentitySwapRemoveTotal++;
  SC.Moves[NEW].IdentitySwapAddTotal++;
  SC.Moves[OLD].IdentitySwap_Total_TO[NEW]++;
  Components::IdentitySwapRecord& rec = SC.LastIdentitySwap;
  rec = Components::IdentitySwapRecord{};
  rec.OldComponent = OLD;
  rec.NewComponent = NEW;
  rec.OldMolecule = oldmol;

  // the new species grown on the old molecule's first bead, the old molecule excluded
  SC.TempVal.component = NEW;
  SC.TempVal.molecule = newmol;
  SC.TempVal.Scale = double2{1.0, 1.0};
  CBMC_Variables ins;
  ins.MoveType = IDENTITY_SWAP_NEW;
  Sims.New.pos[0] = Sims.d_a[OLD].pos[oldmol * ms_old];
  Sims.ExcludeComponent = (int)OLD;
  Sims.ExcludeMolecule = (int64_t)oldmol;
  Widom_Move_FirstBead_PARTIAL(Vars, systemId, ins);
  if (ins.SuccessConstruction && ins.Rosenbluth > 1e-150 && ms_new > 1) Widom_Move_Chain_PARTIAL(Vars, systemId, ins);
  Sims.ExcludeComponent = -1;
  Sims.ExcludeMolecule = -1;
  if (!ins.SuccessConstruction || ins.Rosenbluth <= 1e-150) return MoveEnergy();
  MoveEnergy energy = ins.FirstBeadEnergy + ins.ChainEnergy;
  std::vector<double3> grown(ms_new);
  grown[0] = Sims.Old.pos[0];
  for (size_t a = 1; a < ms_new; ++a) grown[a] = Sims.New.pos[ins.selectedTrialOrientation * (ms_new - 1) + (a - 1)];

  // retrace of the old molecule (trial 0 of each stage is its current configuration)
  SC.TempVal.component = OLD;
  SC.TempVal.molecule = oldmol;
  CBMC_Variables del;
  del.MoveType = IDENTITY_SWAP_OLD;
  Widom_Move_FirstBead_PARTIAL(Vars, systemId, del);
  if (del.SuccessConstruction && ms_old > 1) Widom_Move_Chain_PARTIAL(Vars, systemId, del);
  if (!del.SuccessConstruction) return MoveEnergy();
  energy -= del.FirstBeadEnergy + del.ChainEnergy;

  if (!Vars.device_FF.noCharges) {
    const double2 E = GPU_EwaldDifference_IdentitySwap(Sims, Vars.device_FF, SC, OLD, NEW, oldmol * ms_old, grown);
    energy.GGEwaldE = E.x;
    energy.HGEwaldE = E.y;
    rec.Ewald = E;
    ins.Rosenbluth *= std::exp(-SC.Beta * (E.x + E.y));
  }
  const double pre = GetPrefactor(SC, Sims, NEW, INSERTION) * GetPrefactor(SC, Sims, OLD, DELETION);
  const double pacc = pre * (ins.Rosenbluth / SC.IdealRosenbluthWeight[NEW]) /
                      (del.Rosenbluth / SC.IdealRosenbluthWeight[OLD]);
  rec.RosenbluthNew = ins.Rosenbluth;
  rec.RosenbluthOld = del.Rosenbluth;
  rec.Pacc = pacc;
  if (!(grx_u01(w[3]) < pacc)) return MoveEnergy();
  if (NEW != OLD && (newmol + 1) * ms_new > SC.Allocate_size[NEW]) return MoveEnergy();  // no room: refused
  rec.Accepted = true;
  if (NEW != OLD) {
    remove_molecule(Vars, systemId, OLD, oldmol);
    write_molecule(Vars, systemId, NEW, newmol, flat_positions(grown));
  } else {
    write_molecule(Vars, systemId, OLD, oldmol, flat_positions(grown));
  }
  if (!Vars.device_FF.noCharges && (SC.hasPartialCharge[NEW] || SC.hasPartialCharge[OLD]))
    Update_Vector_Ewald(Sims.Box, false, SC, NEW);
  SC.Moves[NEW].IdentitySwapAddAccepted++;
  SC.Moves[OLD].IdentitySwapRemoveAccepted++;
  SC.Moves[OLD].IdentitySwap_Acc_TO[NEW]++;
  return energy;
}

// GibbsParticleTransfer (mc_swap_moves.h:51-176). The box choice, the molecule to delete and the
// acceptance come from box 0's move counter (GRX_SLOT_GIBBS); each growth draws from its own
// box's stream and counter, and both counters advance. Fractional (CB/CFC) molecules are not
// transferred on this path.
bool GibbsParticleTransfer(Variables& Vars, size_t comp, Gibbs& G) {
  if (Vars.SystemComponents.size() < 2) throw std::runtime_error("GibbsParticleTransfer: two boxes needed");
  uint32_t w[4];
  grx_draw(Vars.Random.Seed, Vars.Random.BoxStream(0), Vars.SystemComponents[0].Step, GRX_SLOT_GIBBS, w);
  G.GibbsXferStats[0] += 1.0;
  const size_t A = grx_u01(w[0]) > 0.5 ? 1 : 0, B = 1 - A;  // insert into A, delete from B
  Gibbs::TransferRecord& rec = G.LastTransfer;
  rec = Gibbs::TransferRecord{};
  rec.InsertionBox = A;
  Components& SA = Vars.SystemComponents[A];
  Components& SB = Vars.SystemComponents[B];
  bool accept = false;
  if (SB.NumberOfMolecule_for_Component[comp] >= 1) {
    SA.TempVal.component = comp;
    SA.TempVal.molecule = SA.NumberOfMolecule_for_Component[comp];
    SA.TempVal.Scale = double2{1.0, 1.0};
    InsertionMove ins;
    ins.Initialize();
    ins.Calculate(Vars, A);
    if (ins.InsertionVariables.SuccessConstruction) {
      SB.TempVal.component = comp;
      SB.TempVal.molecule = (size_t)(grx_u01(w[1]) * (double)SB.NumberOfMolecule_for_Component[comp]);
      SB.TempVal.Scale = double2{1.0, 1.0};
      DeletionMove del;
      del.Initialize();
      del.Calculate(Vars, B);
      if (del.DeletionVariables.SuccessConstruction) {
        const double NA = molecules_in_box(SA), NB = molecules_in_box(SB);
        const double pacc = (ins.InsertionVariables.Rosenbluth * NB * Vars.Sims[A].Box.Volume) /
                            (del.DeletionVariables.Rosenbluth * (NA + 1.0) * Vars.Sims[B].Box.Volume);
        const size_t N = SA.NumberOfMolecule_for_Component[comp];
        accept = grx_u01(w[2]) < pacc && (N + 1) * SA.Moleculesize[comp] <= SA.Allocate_size[comp];
        rec.DeletedMolecule = SB.TempVal.molecule;
        rec.RosenbluthInsertion = ins.InsertionVariables.Rosenbluth;
        rec.RosenbluthDeletion = del.DeletionVariables.Rosenbluth;
        rec.Pacc = pacc;
        rec.Accepted = accept;
        if (accept) {
          ins.Commit(Vars, A);
          del.Commit(Vars, B);
          SA.deltaE += ins.energy;
          SB.deltaE += del.energy;
          G.GibbsXferStats[1] += 1.0;
        }
      }
    }
  }
  for (Components& C : Vars.SystemComponents) C.Step++;
  return accept;
}

// ------------------------------------------------------------------ Widom statistics
void RecordRosen(Components& SC, size_t comp, size_t block, double W) {
  if (SC.Rosen_Widom.size() <= comp) SC.Rosen_Widom.resize(comp + 1);
  std::vector<double3>& B = SC.Rosen_Widom[comp].Blocks;
  if (B.size() < SC.Nblock) B.resize(SC.Nblock);
  if (block >= SC.Nblock) block = SC.Nblock - 1;
  B[block].x += W;
  B[block].y += W * W;
  B[block].z += 1.0;
}

double WidomAverageRosenbluth(const Components& SC, size_t comp) {
  const std::vector<double3>& B = SC.Rosen_Widom[comp].Blocks;
  double s = 0.0;
  size_t n = 0;
  for (const double3& b : B) {
    if (b.z <= 0) continue;
    s += b.x / b.z;
    ++n;
  }
  return n ? s / (double)n : 0.0;
}

// ComputeFugacity (print_statistics.cuh:100-110): mu_ex = -kT ln<W>, reported in K.
double WidomChemicalPotential(const Components& SC, size_t comp) {
  return -SC.Temperature * std::log(WidomAverageRosenbluth(SC, comp));
}

// Atoms of every pseudo-atom type in the box: framework atoms of the host mirrors plus the
// molecules of each adsorbate component (its template types times the molecule count).
static std::vector<double> type_counts(const Variables& Vars, size_t systemId, size_t extra_comp) {
  const Components& SC = Vars.SystemComponents[systemId];
  const Simulations& S = Vars.Sims[systemId];
  std::vector<double> n(Vars.device_FF.size, 0.0);
  for (int c = 0; c < SC.NComponents.x; ++c) {
    const HostAtoms& H = S.host[c];
    if (c < SC.NComponents.y) {
      for (size_t i = 0; i < SC.Moleculesize[c] && i < H.Type.size(); ++i) n[H.Type[i]] += 1.0;
    } else {
      const double nm = (double)SC.NumberOfMolecule_for_Component[c] + ((size_t)c == extra_comp ? 1.0 : 0.0);
      for (size_t a = 0; a < SC.Moleculesize[c] && a < H.Type.size(); ++a) n[H.Type[a]] += nm;
    }
  }
  return n;
}

static double tail_energy(const Variables& Vars, size_t systemId, const std::vector<double>& n) {
  const ForceField& FF = Vars.device_FF;
  if (FF.tail.empty()) return 0.0;
  const double V = Vars.Sims[systemId].Box.Volume;
  const double rc = std::sqrt(FF.CutOffVDW), rc3 = rc * rc * rc, rc9 = rc3 * rc3 * rc3;
  const double pi = 3.14159265358979323846;
  double e = 0.0;
  for (size_t i = 0; i < FF.size; ++i)
    for (size_t j = 0; j < FF.size; ++j) {
      const size_t k = i * FF.size + j;
      if (!FF.tail[k] || n[i] == 0.0 || n[j] == 0.0) continue;
      const double s3 = FF.sigma[k] * FF.sigma[k] * FF.sigma[k], s6 = s3 * s3;
      e += 2.0 * pi * n[i] * n[j] / V * 4.0 * FF.epsilon[k] * (s6 * s6 / (9.0 * rc9) - s6 / (3.0 * rc3));
    }
  return e;
}

double TailCorrectionEnergy(const Variables& Vars, size_t systemId) {
  return tail_energy(Vars, systemId, type_counts(Vars, systemId, (size_t)-1));
}

double TailCorrectionInsertion(const Variables& Vars, size_t systemId, size_t comp) {
  return tail_energy(Vars, systemId, type_counts(Vars, systemId, comp)) -
         tail_energy(Vars, systemId, type_counts(Vars, systemId, (size_t)-1));
}

double FrameworkDensity(const Components& SC, const Boxsize& Box) {
  const double avogadro = 6.02214076e23;
  return SC.FrameworkMass * 1.0e-3 / (avogadro * Box.Volume * 1.0e-30);
}

double WidomHenryCoefficient(const Components& SC, const Boxsize& Box, double AverageW) {
  const double gas_constant = 8.314462618;  // J/mol/K
  return AverageW / (gas_constant * SC.Temperature * FrameworkDensity(SC, Box));
}

// ------------------------------------------------------------------ device-resident moves
static grx_gcmc_desc device_desc(Variables& Vars, size_t systemId, size_t comp) {
  Components& SC = Vars.SystemComponents[systemId];
  const Move_Statistics& MS = SC.Moves[comp];
  grx_gcmc_desc d{};
  d.component = (int32_t)comp;
  d.ntrials = (int32_t)Vars.Widom[systemId].NumberWidomTrials;
  d.norient = (int32_t)Vars.Widom[systemId].NumberWidomTrialsOrientations;
  d.p_translation = MS.TranslationProb;
  d.p_rotation = MS.RotationProb;
  d.p_reinsertion = MS.ReinsertionProb;
  d.p_swap = MS.SwapProb;
  d.p_identity_swap = MS.IdentitySwapProb;
  d.max_translation[0] = MS.MaxTranslation.x; d.max_translation[1] = MS.MaxTranslation.y;
  d.max_translation[2] = MS.MaxTranslation.z;
  d.max_rotation[0] = MS.MaxRotation.x; d.max_rotation[1] = MS.MaxRotation.y; d.max_rotation[2] = MS.MaxRotation.z;
  d.beta = SC.Beta;
  d.pressure = SC.Pressure;
  d.fugacity_coeff = SC.FugacityCoeff[comp];
  d.mol_fraction = SC.MolFraction[comp];
  d.ideal_rosenbluth = SC.IdealRosenbluthWeight[comp];
  d.tail_insert = SC.TailCorrectionInsert.empty() ? 0.0 : SC.TailCorrectionInsert[comp];
  d.seed = Vars.Random.Seed;
  d.stream = Vars.Random.BoxStream(systemId);
  return d;
}

std::vector<grx_gcmc_desc> Device_Move_Descs(Variables& Vars, size_t systemId, std::vector<size_t>* moved) {
  Components& SC = Vars.SystemComponents[systemId];
  std::vector<grx_gcmc_desc> descs;
  if (moved) moved->clear();
  for (int c = SC.NComponents.y; c < SC.NComponents.x; ++c)
    if (SC.Moves[c].SwapProb > 1e-10) {  // cumulative: the total of this component's moves
      descs.push_back(device_desc(Vars, systemId, (size_t)c));
      if (moved) moved->push_back((size_t)c);
    }
  return descs;
}

std::vector<grx_gcmc_stats> RunMoves_Device_All(Variables& Vars, size_t systemId, int64_t nsteps,
                                                std::vector<size_t>* moved) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  std::vector<size_t> comps;
  std::vector<grx_gcmc_desc> descs = Device_Move_Descs(Vars, systemId, &comps);
  if (descs.empty()) throw std::runtime_error("RunMoves_Device_All: no component has moves");
  std::vector<grx_gcmc_stats> st(descs.size());
  grx_box* b = Sims.Box.handle;
  const int32_t nm = (int32_t)descs.size();
  check(grx_gcmc_run(&b, 1, descs.data(), &nm, SC.Step, nsteps, Vars.Precision, st.data()), "grx_gcmc_run");
  SC.Step += (uint64_t)nsteps;
  for (size_t c : comps) Sync_Host_Mirror(Vars, systemId, c);
  if (moved) *moved = comps;
  return st;
}

grx_gcmc_stats RunMoves_Device(Variables& Vars, size_t systemId, size_t comp, int64_t nsteps) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  const Move_Statistics& MS = SC.Moves[comp];
  grx_gcmc_desc d{};
  d.component = (int32_t)comp;
  d.ntrials = (int32_t)Vars.Widom[systemId].NumberWidomTrials;
  d.norient = (int32_t)Vars.Widom[systemId].NumberWidomTrialsOrientations;
  d.p_translation = MS.TranslationProb;
  d.p_rotation = MS.RotationProb;
  d.p_reinsertion = MS.ReinsertionProb;
  d.p_swap = MS.SwapProb;
  d.p_identity_swap = MS.IdentitySwapProb;
  d.max_translation[0] = MS.MaxTranslation.x; d.max_translation[1] = MS.MaxTranslation.y;
  d.max_translation[2] = MS.MaxTranslation.z;
  d.max_rotation[0] = MS.MaxRotation.x; d.max_rotation[1] = MS.MaxRotation.y; d.max_rotation[2] = MS.MaxRotation.z;
  d.beta = SC.Beta;
  d.pressure = SC.Pressure;
  d.fugacity_coeff = SC.FugacityCoeff[comp];
  d.mol_fraction = SC.MolFraction[comp];
  d.ideal_rosenbluth = SC.IdealRosenbluthWeight[comp];
  d.tail_insert = SC.TailCorrectionInsert.empty() ? 0.0 : SC.TailCorrectionInsert[comp];
  d.seed = Vars.Random.Seed;
  d.stream = Vars.Random.BoxStream(systemId);
  grx_gcmc_stats st{};
  grx_box* b = Sims.Box.handle;
  check(grx_gcmc_run(&b, 1, &d, nullptr, SC.Step, nsteps, Vars.Precision, &st), "grx_gcmc_run");
  SC.Step += (uint64_t)nsteps;
  Sync_Host_Mirror(Vars, systemId, comp);
  return st;
}

void Sync_Host_Mirror(Variables& Vars, size_t systemId, size_t comp) {
  Components& SC = Vars.SystemComponents[systemId];
  Simulations& Sims = Vars.Sims[systemId];
  const size_t ms = SC.Moleculesize[comp];
  size_t n = 0;
  check(grx_box_get_component_size(Sims.Box.handle, (int32_t)comp, &n), "grx_box_get_component_size");
  Atoms& A = Sims.d_a[comp];
  std::vector<double> pos(3 * n);
  if (n) check(grx_box_get_positions(Sims.Box.handle, (int32_t)comp, pos.data(), n), "grx_box_get_positions");
  for (size_t i = 0; i < n; ++i) {
    A.pos[i] = double3{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    A.charge[i] = A.charge[i % ms];
    A.Type[i] = A.Type[i % ms];
    A.MolID[i] = i / ms;
    A.scale[i] = 1.0;
    A.scaleCoul[i] = 1.0;
  }
  A.size = n;
  SC.NumberOfMolecule_for_Component[comp] = n / ms;
}

}  // namespace graspa
