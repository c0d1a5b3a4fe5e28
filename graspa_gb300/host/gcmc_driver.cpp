// gcmc_driver.cpp -- a reference-shaped Monte Carlo program on the C++ host layer.
//
// Reads one box (a "grx system file", written by graspa_gb300.system_file), then
//   host   <nsteps>  runs RunMoves one move at a time: every energy call is a libgrx
//                    call (CBMC_PairwiseInteractions, GPU_EwaldDifference_General, ...)
//   device <nsteps>  runs the same moves with RunMoves_Device (one grx_gcmc_run)
//   widom  <n>       runs n InsertionMove::WidomMove calls and the Widom statistics
//   volume <n>       runs n NPT VolumeMove calls (trial volume, trial energy, acceptance)
//   gibbs  <n>       runs n NVTGibbsMove calls between the box and an identical copy
//   transfer <n>     runs n GibbsParticleTransfer calls of the moved component between the
//                    box and an identical copy
//   swap   <n>       runs n IdentitySwapMove calls (every adsorbate component takes part)
//   swap_device <n>  the same identity swaps in one device run (RunMoves_Device_All, every
//                    adsorbate component with identity swaps only)
//   lambda 0         two CB/CFC lambda steps of molecule 0 (CBCF_LambdaChange)
// and prints the move statistics, the accepted-energy sum and the drift check,
// then the adsorbate positions, as plain text.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>

#include "graspa_host.hpp"

using namespace graspa;

namespace {

struct Reader {
  std::ifstream in;
  explicit Reader(const char* path) : in(path) {
    if (!in) throw std::runtime_error(std::string("cannot open ") + path);
  }
  void key(const char* k) {
    std::string s;
    in >> s;
    if (s != k) throw std::runtime_error("system file: expected '" + std::string(k) + "', found '" + s + "'");
  }
  double d() { double v; in >> v; return v; }
  long long i() { long long v; in >> v; return v; }
};

void read_system(const char* path, Variables& V, std::vector<size_t>& n_stored, size_t& comp) {
  Reader R(path);
  V.Sims.resize(1);
  V.SystemComponents.resize(1);
  V.Widom.resize(1);
  Simulations& S = V.Sims[0];
  Components& C = V.SystemComponents[0];
  Boxsize& B = S.Box;
  R.key("cell"); for (double& c : B.Cell) c = R.d();
  R.key("inverse_cell"); for (double& c : B.InverseCell) c = R.d();
  R.key("volume"); B.Volume = R.d();
  R.key("cubic"); B.Cubic = R.i() != 0;
  R.key("lammps_ewald"); B.UseLAMMPSEwald = R.i() != 0;
  R.key("kmax"); B.kmax.x = (int)R.i(); B.kmax.y = (int)R.i(); B.kmax.z = (int)R.i();
  R.key("alpha"); B.Alpha = R.d();
  R.key("prefactor"); B.Prefactor = R.d();
  R.key("reciprocal_cutoff"); B.ReciprocalCutOff = R.d();
  ForceField& FF = V.device_FF;
  R.key("ntypes"); FF.size = (size_t)R.i();
  const size_t nt2 = FF.size * FF.size;
  FF.epsilon.resize(nt2); FF.sigma.resize(nt2); FF.shift.resize(nt2);
  R.key("epsilon"); for (double& x : FF.epsilon) x = R.d();
  R.key("sigma"); for (double& x : FF.sigma) x = R.d();
  R.key("shift"); for (double& x : FF.shift) x = R.d();
  R.key("cutoff_vdw_sq"); FF.CutOffVDW = R.d();
  R.key("cutoff_coul_sq"); FF.CutOffCoul = R.d();
  R.key("overlap"); FF.OverlapCriteria = R.d();
  R.key("no_charges"); FF.noCharges = R.i() != 0;
  R.key("vdw_real_bias"); FF.VDWRealBias = R.i() != 0;
  R.key("ncomp"); C.NComponents.x = (int)R.i();
  R.key("nhost"); C.NComponents.y = (int)R.i();
  const int nc = C.NComponents.x;
  C.Moleculesize.resize(nc); C.Allocate_size.resize(nc); C.NumberOfMolecule_for_Component.resize(nc);
  C.rigid.resize(nc); C.IdealRosenbluthWeight.assign(nc, 1.0); C.FugacityCoeff.assign(nc, 1.0);
  C.MolFraction.assign(nc, 1.0); C.TailCorrectionInsert.assign(nc, 0.0); C.Moves.resize(nc);
  S.host.resize(nc); S.d_a.resize(nc);
  n_stored.assign(nc, 0);
  for (int c = 0; c < nc; ++c) {
    R.key("component"); (void)R.i();
    R.key("molsize"); C.Moleculesize[c] = (size_t)R.i();
    R.key("capacity"); C.Allocate_size[c] = (size_t)R.i();
    R.key("size"); const size_t n = (size_t)R.i();
    R.key("stored"); n_stored[c] = (size_t)R.i();
    R.key("rigid"); C.rigid[c] = R.i() != 0;
    HostAtoms& H = S.host[c];
    H.allocate(std::max<size_t>(C.Allocate_size[c], n_stored[c]));
    for (size_t a = 0; a < n_stored[c]; ++a) {
      H.pos[a].x = R.d(); H.pos[a].y = R.d(); H.pos[a].z = R.d();
      H.charge[a] = R.d();
      H.Type[a] = (size_t)R.i();
      H.MolID[a] = (size_t)R.i();
    }
    S.d_a[c] = H.view(C.Moleculesize[c], n);
  }
  R.key("component_moved"); comp = (size_t)R.i();
  C.TempVal.component = comp;
  R.key("beta"); C.Beta = R.d();
  R.key("temperature"); C.Temperature = R.d();
  R.key("pressure"); C.Pressure = R.d();
  R.key("fugacity_coeff"); C.FugacityCoeff[comp] = R.d();
  R.key("mol_fraction"); C.MolFraction[comp] = R.d();
  R.key("ideal_rosenbluth"); C.IdealRosenbluthWeight[comp] = R.d();
  R.key("tail_insert"); C.TailCorrectionInsert[comp] = R.d();
  R.key("ntrials"); V.Widom[0].NumberWidomTrials = (size_t)R.i();
  R.key("norient"); V.Widom[0].NumberWidomTrialsOrientations = (size_t)R.i();
  Move_Statistics& M = C.Moves[comp];
  R.key("cumulative_probabilities");
  M.TranslationProb = R.d(); M.RotationProb = R.d(); M.ReinsertionProb = R.d(); M.SwapProb = R.d();
  R.key("max_translation"); M.MaxTranslation.x = R.d(); M.MaxTranslation.y = R.d(); M.MaxTranslation.z = R.d();
  R.key("max_rotation"); M.MaxRotation.x = R.d(); M.MaxRotation.y = R.d(); M.MaxRotation.z = R.d();
  R.key("seed"); V.Random.Seed = (uint64_t)R.i();
  R.key("stream"); V.Random.Stream = (uint32_t)R.i();
  R.key("first_step"); C.Step = (uint64_t)R.i();
  R.key("precision"); V.Precision = (grx_precision)R.i();
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: %s <system file> host|device|widom|volume|gibbs|transfer|swap|swap_device|lambda <nsteps>\n",
                 argv[0]);
    return 2;
  }
  try {
    Variables V;
    std::vector<size_t> n_stored;
    size_t comp = 0;
    read_system(argv[1], V, n_stored, comp);
    const std::string mode = argv[2];
    const long long nsteps = std::atoll(argv[3]);
    if (mode == "gibbs" || mode == "transfer") {  // a second, identical box (arrays re-pointed at its own storage)
      V.Sims.push_back(V.Sims[0]);
      V.SystemComponents.push_back(V.SystemComponents[0]);
      V.Widom.push_back(V.Widom[0]);
      Simulations& S1 = V.Sims[1];
      for (size_t c = 0; c < S1.host.size(); ++c)
        S1.d_a[c] = S1.host[c].view(V.SystemComponents[1].Moleculesize[c], V.Sims[0].d_a[c].size);
      Setup_Box(V, 1, n_stored);
    }
    Setup_Box(V, 0, n_stored);
    Components& C = V.SystemComponents[0];
    const MoveEnergy e0 = Total_Energy(V.Sims[0]);
    std::printf("mode %s\n", mode.c_str());
    if (mode == "widom") {
      for (long long i = 0; i < nsteps; ++i) {
        C.TempVal.component = comp;
        InsertionMove m;
        const double W = m.WidomMove(V, 0);
        std::printf("W %lld %.17g\n", (long long)C.Step, W);
        RecordRosen(C, comp, (size_t)(i * (long long)C.Nblock / nsteps), W);
        C.Step++;
      }
      std::printf("widom_average_rosenbluth %.17g\n", WidomAverageRosenbluth(C, comp));
      std::printf("widom_mu_ex_K %.17g\n", WidomChemicalPotential(C, comp));
    } else if (mode == "gibbs") {
      // NVT Gibbs volume exchange between box 0 and its copy (max change of ln(VA/VB) 0.1)
      Gibbs G;
      G.MaxGibbsBoxChange = 0.1;
      const MoveEnergy e0b = Total_Energy(V.Sims[1]);
      for (long long k = 0; k < nsteps; ++k) {
        NVTGibbsMove(V, G);
        std::printf("gibbs %lld %.17g %.17g\n", k, V.Sims[0].Box.Volume, V.Sims[1].Box.Volume);
      }
      const MoveEnergy e1 = Total_Energy(V.Sims[0]), e1b = Total_Energy(V.Sims[1]);
      std::printf("gibbs_attempts %.17g\n", G.GibbsBoxStats[0]);
      std::printf("gibbs_accepted %.17g\n", G.GibbsBoxStats[1]);
      std::printf("drift %.17g\n", (e1.total() - e0.total()) - C.deltaE.total());
      std::printf("drift_b %.17g\n", (e1b.total() - e0b.total()) - V.SystemComponents[1].deltaE.total());
      std::printf("energy_scale %.17g\n", std::fabs(e1.total()) + std::fabs(e1b.total()));
      Destroy_Box(V, 1);
    } else if (mode == "transfer") {
      // Gibbs particle transfers of the moved component between box 0 and its copy
      Gibbs G;
      Components& C1 = V.SystemComponents[1];
      const MoveEnergy e0b = Total_Energy(V.Sims[1]);
      for (long long k = 0; k < nsteps; ++k) {
        GibbsParticleTransfer(V, comp, G);
        const Gibbs::TransferRecord& r = G.LastTransfer;
        std::printf("transfer %lld %zu %zu %d %.17g %.17g %.17g %zu %zu\n", k, r.InsertionBox, r.DeletedMolecule,
                    r.Accepted ? 1 : 0, r.RosenbluthInsertion, r.RosenbluthDeletion, r.Pacc,
                    C.NumberOfMolecule_for_Component[comp], C1.NumberOfMolecule_for_Component[comp]);
      }
      const MoveEnergy e1 = Total_Energy(V.Sims[0]), e1b = Total_Energy(V.Sims[1]);
      std::printf("transfer_attempts %.17g\n", G.GibbsXferStats[0]);
      std::printf("transfer_accepted %.17g\n", G.GibbsXferStats[1]);
      std::printf("drift %.17g\n", (e1.total() - e0.total()) - (C.deltaE.total() - C.deltaE.TailE));
      std::printf("drift_b %.17g\n", (e1b.total() - e0b.total()) - (C1.deltaE.total() - C1.deltaE.TailE));
      std::printf("energy_scale %.17g\n", std::fabs(e1.total()) + std::fabs(e1b.total()));
      Destroy_Box(V, 1);
    } else if (mode == "swap_device") {
      for (int c = C.NComponents.y; c < C.NComponents.x; ++c) {
        Move_Statistics& M = C.Moves[c];
        M.TranslationProb = M.RotationProb = M.ReinsertionProb = 0.0;
        M.IdentitySwapProb = M.SwapProb = 1.0;
      }
      std::vector<size_t> moved;
      const std::vector<grx_gcmc_stats> st = RunMoves_Device_All(V, 0, nsteps, &moved);
      double esum = 0.0;
      for (const grx_gcmc_stats& x : st) esum += x.energy[3];
      const MoveEnergy e1 = Total_Energy(V.Sims[0]);
      std::printf("energy_sum %.17g\n", esum);
      std::printf("drift %.17g\n", (e1.total() - e0.total()) - esum);
      for (size_t k = 0; k < moved.size(); ++k)
        std::printf("count %zu %zu %lld %lld\n", moved[k], C.NumberOfMolecule_for_Component[moved[k]],
                    (long long)st[k].identity_in[1], (long long)st[k].identity_out[1]);
      for (int c = C.NComponents.y; c < C.NComponents.x; ++c) {
        const Atoms& A = V.Sims[0].d_a[c];
        std::printf("positions %zu\n", A.size);
        for (size_t i = 0; i < A.size; ++i) std::printf("%.17g %.17g %.17g\n", A.pos[i].x, A.pos[i].y, A.pos[i].z);
      }
    } else if (mode == "swap") {
      // identity swaps among the adsorbate components
      for (long long k = 0; k < nsteps; ++k) {
        const MoveEnergy dE = IdentitySwapMove(V, 0);
        C.deltaE += dE;
        C.Step++;
        const Components::IdentitySwapRecord& r = C.LastIdentitySwap;
        std::printf("swap %lld %zu %zu %zu %d %.17g %.17g %.17g %.17g %.17g\n", k, r.OldComponent, r.NewComponent,
                    r.OldMolecule, r.Accepted ? 1 : 0, r.RosenbluthNew, r.RosenbluthOld, r.Pacc, r.Ewald.x,
                    r.Ewald.y);
      }
      const MoveEnergy e1 = Total_Energy(V.Sims[0]);
      std::printf("energy_sum %.17g\n", C.deltaE.total());
      std::printf("drift %.17g\n", (e1.total() - e0.total()) - C.deltaE.total());
      for (int c = C.NComponents.y; c < C.NComponents.x; ++c)
        std::printf("count %d %zu %zu %zu\n", c, C.NumberOfMolecule_for_Component[c],
                    C.Moves[c].IdentitySwapAddAccepted, C.Moves[c].IdentitySwapRemoveAccepted);
      for (int c = C.NComponents.y; c < C.NComponents.x; ++c) {
        const Atoms& A = V.Sims[0].d_a[c];
        std::printf("positions %zu\n", A.size);
        for (size_t i = 0; i < A.size; ++i) std::printf("%.17g %.17g %.17g\n", A.pos[i].x, A.pos[i].y, A.pos[i].z);
      }
    } else if (mode == "volume") {
      // NPT volume moves of the box (max change of ln V 0.05): per move the trial volume,
      // the trial box's FP64 total, its overlap flag, the energy before the move, acceptance
      C.VolumeMoveMaxChange = 0.05;
      for (long long k = 0; k < nsteps; ++k) {
        const double e_before = Total_Energy(V.Sims[0]).total();
        const size_t acc0 = C.VolumeMoveAccepted;
        VolumeMove(V, 0);
        std::printf("volume %lld %d %.17g %.17g %d %.17g\n", k, C.VolumeMoveAccepted > acc0 ? 1 : 0,
                    C.VolumeMoveLastV, C.VolumeMoveLastE.total(), C.VolumeMoveLastOverlap ? 1 : 0, e_before);
      }
      const MoveEnergy e1 = Total_Energy(V.Sims[0]);
      std::printf("energy_sum %.17g\n", C.deltaE.total());
      std::printf("drift %.17g\n", (e1.total() - e0.total()) - C.deltaE.total());
      std::printf("final_volume %.17g\n", V.Sims[0].Box.Volume);
      const Atoms& A = V.Sims[0].d_a[comp];
      std::printf("positions %zu\n", A.size);
      for (size_t i = 0; i < A.size; ++i) std::printf("%.17g %.17g %.17g\n", A.pos[i].x, A.pos[i].y, A.pos[i].z);
    } else if (mode == "lambda") {
      // CB/CFC lambda steps of molecule 0: 1 -> 0.4 as a lambda change, the caller's update
      // of the molecule's scales, then 0.4 -> 0.1 as the second step of a CB/CFC deletion
      // (Fourier part from the staged vector)
      const double steps[2][2] = {{1.0, 0.4}, {0.4, 0.1}};
      const int types[2] = {CBCF_LAMBDACHANGE, CBCF_DELETION};
      Atoms& A = V.Sims[0].d_a[comp];
      for (int k = 0; k < 2; ++k) {
        size_t start = 0;
        bool ok = false;
        const MoveEnergy e = CBCF_LambdaChange(V, 0, 0, comp, double2{steps[k][0], steps[k][0]},
                                               double2{steps[k][1], steps[k][1]}, start, types[k], ok);
        std::printf("lambda %d %d %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", k, ok ? 1 : 0, e.HGVDW,
                    e.HGReal, e.GGVDW, e.GGReal, e.GGEwaldE, e.HGEwaldE, e.TailE, e.total());
        for (size_t a = 0; a < C.Moleculesize[comp]; ++a) {
          A.scale[start + a] = steps[k][1];
          A.scaleCoul[start + a] = steps[k][1];
        }
      }
    } else {
      long long att[5] = {0, 0, 0, 0, 0}, acc[5] = {0, 0, 0, 0, 0};
      double esum = 0.0;
      if (mode == "host") {
        for (long long s = 0; s < nsteps; ++s) RunMoves(V, 0, comp);
        const Move_Statistics& M = C.Moves[comp];
        att[0] = M.TranslationTotal; att[1] = M.RotationTotal; att[2] = M.InsertionTotal;
        att[3] = M.DeletionTotal; att[4] = M.ReinsertionTotal;
        acc[0] = M.TranslationAccepted; acc[1] = M.RotationAccepted; acc[2] = M.InsertionAccepted;
        acc[3] = M.DeletionAccepted; acc[4] = M.ReinsertionAccepted;
        esum = C.deltaE.total() - C.deltaE.TailE;  // the FP64 totals below carry no tail term
      } else if (mode == "device") {
        const grx_gcmc_stats st = RunMoves_Device(V, 0, comp, nsteps);
        for (int k = 0; k < 5; ++k) { att[k] = st.attempts[k]; acc[k] = st.accepted[k]; }
        esum = st.energy[3];
      } else {
        throw std::runtime_error("unknown mode " + mode);
      }
      const MoveEnergy e1 = Total_Energy(V.Sims[0]);
      std::printf("attempts %lld %lld %lld %lld %lld\n", att[0], att[1], att[2], att[3], att[4]);
      std::printf("accepted %lld %lld %lld %lld %lld\n", acc[0], acc[1], acc[2], acc[3], acc[4]);
      std::printf("n_molecules %zu\n", C.NumberOfMolecule_for_Component[comp]);
      std::printf("energy_sum %.17g\n", esum);
      std::printf("drift %.17g\n", (e1.total() - e0.total()) - esum);
      const Atoms& A = V.Sims[0].d_a[comp];
      std::printf("positions %zu\n", A.size);
      for (size_t i = 0; i < A.size; ++i) std::printf("%.17g %.17g %.17g\n", A.pos[i].x, A.pos[i].y, A.pos[i].z);
    }
    Destroy_Box(V, 0);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "gcmc_driver: %s\n", e.what());
    return 1;
  }
  return 0;
}
