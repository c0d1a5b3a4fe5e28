// graspa_run.cpp -- runs a gRASPA example directory (simulation.input, force field,
// pseudo atoms, molecule .def, P1 CIF) on the GB300 engine through the C++ host layer.
//
//   graspa_run <dir> [--precision mixed|fp64] [--cycles-scale f] [--max-cycles n] [--dump file.json]
//              [--replicas R [--launch-steps L] [--init-steps n] [--prod-steps n] [--blocks b]]
//
// Prints the initial-stage energies in the terms of the reference's output (Fourier
// host-host, self and intramolecular exclusion energies, rigid exclusion constants),
// runs the initialization / equilibration / production phases (cycles of
// max(20, molecules) steps, Determine_Number_Of_Steps, axpy.cu:580-591; max translation
// and rotation adapted every 500 cycles, mc_utilities.h:612-665), and reports block
// averages of the loading, move statistics and the energy drift check. --dump writes
// the parsed system as JSON and exits before any device work.
//
// --replicas R runs R independent Markov chains of the example at once instead of one:
// the box and R - 1 replicas sharing its framework (distinct Philox streams; replica 0
// is the single-chain run), all in one persistent GCMC launch of L steps (default 500)
// at a time. The phases last the input's cycles x steps per cycle (MaxStepPerCycle with
// UseMaxStep, else 20) per replica unless --init-steps / --prod-steps say otherwise; the
// maximum translation adapts after every initialization launch (Update_Max_Translation,
// acceptance 0.5, from the translations of all replicas) and stays fixed in production.
// It reports the loadings as the mean over replicas with its standard error (the
// replicas are independent), the production block averages pooled over replicas, and the
// Widom statistics of every component's CBMC insertions (RecordRosen; ComputeFugacity:
// <W>, mu_ex, Henry coefficient).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>

#include "graspa_input.hpp"

using namespace graspa;

namespace {

void json_array(std::ofstream& o, const double* v, size_t n) {
  o << "[";
  for (size_t i = 0; i < n; ++i) {
    char buf[40];
    std::snprintf(buf, sizeof buf, "%.17g", v[i]);
    o << (i ? "," : "") << buf;
  }
  o << "]";
}

void dump_json(const std::string& path, Variables& V, const SimulationInput& in, const std::vector<size_t>& n_stored) {
  Simulations& S = V.Sims[0];
  Components& SC = V.SystemComponents[0];
  const Boxsize& B = S.Box;
  std::ofstream o(path);
  o << "{\"cell\":";
  json_array(o, B.Cell, 9);
  o << ",\"kmax\":[" << B.kmax.x << "," << B.kmax.y << "," << B.kmax.z << "]";
  char buf[200];
  std::snprintf(buf, sizeof buf, ",\"alpha\":%.17g,\"prefactor\":%.17g,\"reciprocal_cutoff\":%.17g,\"use_lammps_ewald\":%d",
                B.Alpha, B.Prefactor, B.ReciprocalCutOff, (int)B.UseLAMMPSEwald);
  o << buf;
  o << ",\"ntypes\":" << V.device_FF.size << ",\"epsilon\":";
  json_array(o, V.device_FF.epsilon.data(), V.device_FF.epsilon.size());
  o << ",\"sigma\":";
  json_array(o, V.device_FF.sigma.data(), V.device_FF.sigma.size());
  o << ",\"shift\":";
  json_array(o, V.device_FF.shift.data(), V.device_FF.shift.size());
  std::snprintf(buf, sizeof buf, ",\"cutoff_vdw\":%.17g,\"cutoff_coul\":%.17g,\"overlap_criteria\":%.17g,\"no_charges\":%d",
                in.CutOffVDW, in.CutOffCoulomb, in.OverlapCriteria, (int)V.device_FF.noCharges);
  o << buf;
  std::snprintf(buf, sizeof buf, ",\"temperature\":%.17g,\"pressure_internal\":%.17g,\"beta\":%.17g", SC.Temperature,
                SC.Pressure, SC.Beta);
  o << buf;
  std::snprintf(buf, sizeof buf, ",\"framework_mass\":%.17g,\"volume\":%.17g,\"framework_density\":%.17g",
                SC.FrameworkMass, B.Volume, FrameworkDensity(SC, B));
  o << buf;
  std::snprintf(buf, sizeof buf, ",\"tail_energy\":%.17g", TailCorrectionEnergy(V, 0));
  o << buf;
  o << ",\"molecules\":[";
  for (int c = 0; c < SC.NComponents.x; ++c) o << (c ? "," : "") << SC.NumberOfMolecule_for_Component[c];
  o << "]";
  o << ",\"fugacity_coeff\":";
  json_array(o, SC.FugacityCoeff.data(), SC.FugacityCoeff.size());
  o << ",\"mol_fraction\":";
  json_array(o, SC.MolFraction.data(), SC.MolFraction.size());
  o << ",\"move_probabilities\":[";
  for (int c = 0; c < SC.NComponents.x; ++c) {
    const Move_Statistics& M = SC.Moves[c];
    const double p[5] = {M.TranslationProb, M.RotationProb, M.ReinsertionProb, M.IdentitySwapProb, M.SwapProb};
    o << (c ? "," : "");
    json_array(o, p, 5);
  }
  o << "]";
  o << ",\"components\":[";
  for (int c = 0; c < SC.NComponents.x; ++c) {
    const Atoms& A = S.d_a[c];
    const size_t n = n_stored[c];
    std::vector<double> pos(3 * n), q(n), ty(n);
    for (size_t i = 0; i < n; ++i) {
      pos[3 * i] = A.pos[i].x; pos[3 * i + 1] = A.pos[i].y; pos[3 * i + 2] = A.pos[i].z;
      q[i] = A.charge[i];
      ty[i] = (double)A.Type[i];
    }
    o << (c ? "," : "") << "{\"molsize\":" << SC.Moleculesize[c] << ",\"size\":" << A.size << ",\"stored\":" << n
      << ",\"pos\":";
    json_array(o, pos.data(), pos.size());
    o << ",\"charge\":";
    json_array(o, q.data(), q.size());
    o << ",\"type\":";
    json_array(o, ty.data(), ty.size());
    o << "}";
  }
  o << "]}\n";
}

struct BlockStats {
  std::vector<double> sum;   // per block: sum of N over cycles
  std::vector<double> cnt;
};

struct ReplicaOptions {
  int replicas = 0;
  long long launch_steps = 500;
  long long init_steps = -1, prod_steps = -1;
  int blocks = 5;
};

double mean_of(const std::vector<double>& v) {
  double m = 0.0;
  for (double x : v) m += x;
  return v.empty() ? 0.0 : m / (double)v.size();
}

double sem_of(const std::vector<double>& v) {  // standard error of the mean of independent samples
  if (v.size() < 2) return 0.0;
  const double m = mean_of(v);
  double s = 0.0;
  for (double x : v) s += (x - m) * (x - m);
  return std::sqrt(s / (double)(v.size() - 1) / (double)v.size());
}

// R replicas of the example in one batched device launch (see the header comment).
void run_replicas(Variables& V, const SimulationInput& in, const ReplicaOptions& o) {
  Simulations& S = V.Sims[0];
  Components& SC = V.SystemComponents[0];
  const int R = o.replicas;
  std::vector<size_t> comps;
  std::vector<grx_gcmc_desc> base = Device_Move_Descs(V, 0, &comps);
  if (base.empty()) throw std::runtime_error("--replicas: no component has moves");
  const int nm = (int)base.size();
  std::vector<grx_box*> boxes(R, nullptr);
  boxes[0] = S.Box.handle;
  for (int r = 1; r < R; ++r) check(grx_box_create_replica(S.Box.handle, &boxes[r]), "grx_box_create_replica");
  const std::vector<int32_t> nmv(R, nm);
  uint64_t step = SC.Step;
  grx_gcmc_batch* batch = nullptr;
  auto make_batch = [&]() {
    if (batch) check(grx_gcmc_batch_destroy(batch), "grx_gcmc_batch_destroy");
    base = Device_Move_Descs(V, 0, nullptr);
    std::vector<grx_gcmc_desc> d;
    for (int r = 0; r < R; ++r)
      for (int k = 0; k < nm; ++k) {
        grx_gcmc_desc e = base[k];
        e.stream = V.Random.Stream + (uint32_t)r;
        d.push_back(e);
      }
    check(grx_gcmc_batch_create(boxes.data(), R, d.data(), nmv.data(), V.Precision, &batch), "grx_gcmc_batch_create");
    check(grx_gcmc_batch_set_step(batch, step), "grx_gcmc_batch_set_step");
  };
  const long long spc = in.UseMaxStep ? (long long)std::max<size_t>(1, in.MaxStepPerCycle) : 20;
  const long long init = o.init_steps >= 0 ? o.init_steps : (long long)in.NumberOfInitializationCycles * spc;
  const long long prod = o.prod_steps >= 0 ? o.prod_steps
                                           : (long long)(in.NumberOfEquilibrationCycles + in.NumberOfProductionCycles) * spc;
  const long long L = std::max(1LL, o.launch_steps);
  const int nb = std::max(1, o.blocks);
  std::printf("REPLICAS %d chains, launches of %lld steps, initialization %lld steps, production %lld steps per "
              "replica, %d blocks\n", R, L, init, prod, nb);
  double running0 = Total_Energy(S).total();
  const double e_start0 = running0;
  std::vector<grx_gcmc_stats> st((size_t)R * nm);
  make_batch();
  // initialization: launches of L steps, the maximum translation adapted after each
  for (long long done = 0; done < init;) {
    const long long n = std::min(L, init - done);
    check(grx_gcmc_batch_launch(batch, n, nullptr), "grx_gcmc_batch_launch");
    uint64_t next = 0;
    check(grx_gcmc_batch_stats(batch, st.data(), &next), "grx_gcmc_batch_stats");
    check(grx_gcmc_batch_reset_stats(batch), "grx_gcmc_batch_reset_stats");
    step = next;
    done += n;
    for (int k = 0; k < nm; ++k) running0 += st[k].energy[3];
    bool changed = false;
    for (int k = 0; k < nm; ++k) {
      long long att = 0, acc = 0;
      for (int r = 0; r < R; ++r) {
        att += st[(size_t)r * nm + k].attempts[0];
        acc += st[(size_t)r * nm + k].accepted[0];
      }
      if (att == 0) continue;
      Move_Statistics& M = SC.Moves[comps[k]];
      const double f = (double)acc / (double)att > 0.5 ? 1.05 : 0.95;
      M.MaxTranslation = double3{std::min(5.0, std::max(0.01, M.MaxTranslation.x * f)),
                                 std::min(5.0, std::max(0.01, M.MaxTranslation.y * f)),
                                 std::min(5.0, std::max(0.01, M.MaxTranslation.z * f))};
      changed = true;
    }
    if (changed && done < init) make_batch();
  }
  make_batch();
  // production: blocks of launches; per replica and component the loading sums and the
  // Rosenbluth sums of the insertions
  std::vector<double> sumn((size_t)R * nm, 0.0), nsteps((size_t)R * nm, 0.0), ws((size_t)R * nm, 0.0),
      wn((size_t)R * nm, 0.0), w2((size_t)R * nm, 0.0);
  std::vector<std::vector<double>> block_n(nm, std::vector<double>(nb, 0.0));
  std::vector<grx_gcmc_stats> tot(nm);
  const long long per_block = std::max(1LL, prod / nb);
  double wall_s = 0.0;
  for (int blk = 0; blk < nb; ++blk) {
    const long long bsteps = blk == nb - 1 ? prod - per_block * (nb - 1) : per_block;
    for (long long done = 0; done < bsteps;) {
      const long long n = std::min(L, bsteps - done);
      const auto c0 = std::chrono::steady_clock::now();
      check(grx_gcmc_batch_launch(batch, n, nullptr), "grx_gcmc_batch_launch");
      uint64_t next = 0;
      check(grx_gcmc_batch_stats(batch, st.data(), &next), "grx_gcmc_batch_stats");  // waits for the launch
      wall_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - c0).count();
      check(grx_gcmc_batch_reset_stats(batch), "grx_gcmc_batch_reset_stats");
      step = next;
      done += n;
      for (int k = 0; k < nm; ++k) running0 += st[k].energy[3];
      for (int r = 0; r < R; ++r)
        for (int k = 0; k < nm; ++k) {
          const grx_gcmc_stats& e = st[(size_t)r * nm + k];
          const size_t i = (size_t)r * nm + k;
          sumn[i] += e.sum_n;
          nsteps[i] += (double)n;
          ws[i] += e.rosen[0];
          w2[i] += e.rosen[1];
          wn[i] += e.rosen[2];
          block_n[k][blk] += e.sum_n / ((double)bsteps * R);
          grx_gcmc_stats& t = tot[k];
          for (int m = 0; m < 5; ++m) {
            t.attempts[m] += e.attempts[m];
            t.accepted[m] += e.accepted[m];
          }
          for (int m = 0; m < 2; ++m) {
            t.identity_out[m] += e.identity_out[m];
            t.identity_in[m] += e.identity_in[m];
          }
          t.trial_configs += e.trial_configs;
        }
    }
  }
  SC.Step = step;
  const double mass_kg = SC.FrameworkMass * 1e-3;  // kg per mol of frameworks
  const double rho = FrameworkDensity(SC, S.Box);
  std::printf("Framework mass %.5f g/mol density %.5f kg/m^3 volume %.5f\n", SC.FrameworkMass, rho, S.Box.Volume);
  for (int k = 0; k < nm; ++k) {
    const size_t c = comps[k];
    const char* name = in.Components[c - 1].MoleculeName.c_str();
    std::vector<double> nr, wr;
    double wsum = 0.0, wcnt = 0.0;
    for (int r = 0; r < R; ++r) {
      const size_t i = (size_t)r * nm + k;
      nr.push_back(sumn[i] / std::max(1.0, nsteps[i]));
      if (wn[i] > 0) wr.push_back(ws[i] / wn[i]);
      wsum += ws[i];
      wcnt += wn[i];
    }
    const double n_mean = mean_of(nr), n_err = sem_of(nr);
    std::printf("Component %zu [%s] loading %.6f +/- %.6f molecules, %.7f +/- %.7f mol/kg (mean over %d replicas "
                "+/- standard error)\n", c, name, n_mean, n_err, n_mean / mass_kg, n_err / mass_kg, R);
    std::printf("Component %zu [%s] block averages", c, name);
    for (int b = 0; b < nb; ++b) std::printf(" %.6f", block_n[k][b]);
    std::printf("\n");
    if (wcnt > 0) {
      const double W = wsum / wcnt, W_err = sem_of(wr);
      const double mu = -1.2027242847 / SC.Beta * std::log(W);
      const double mu_err = 1.2027242847 / SC.Beta * W_err / W;
      const double H = WidomHenryCoefficient(SC, S.Box, W), H_err = H * W_err / W;
      std::printf("Component %zu [%s] widom <W> %.8f +/- %.8f mu_ex %.6f +/- %.6f K henry %.9e +/- %.3e mol/kg/Pa "
                  "(%.0f insertions)\n", c, name, W, W_err, mu, mu_err, H, H_err, wcnt);
    }
    const grx_gcmc_stats& t = tot[k];
    std::printf("Component %zu [%s] moves: translation %lld/%lld insertion %lld/%lld deletion %lld/%lld reinsertion "
                "%lld/%lld identity-out %lld/%lld identity-in %lld/%lld trial configurations %lld\n", c, name,
                (long long)t.accepted[0], (long long)t.attempts[0], (long long)t.accepted[2], (long long)t.attempts[2],
                (long long)t.accepted[3], (long long)t.attempts[3], (long long)t.accepted[4], (long long)t.attempts[4],
                (long long)t.identity_out[1], (long long)t.identity_out[0],
                (long long)t.identity_in[1], (long long)t.identity_in[0], (long long)t.trial_configs);
    std::printf("Component %zu [%s] max translation %.6f %.6f %.6f\n", c, name, SC.Moves[c].MaxTranslation.x,
                SC.Moves[c].MaxTranslation.y, SC.Moves[c].MaxTranslation.z);
  }
  std::printf("production wall time %.3f s (%.4g replica steps/s, launches and statistics reads)\n", wall_s,
              (double)R * (double)prod / std::max(wall_s, 1e-9));
  check(grx_gcmc_batch_destroy(batch), "grx_gcmc_batch_destroy");
  const double e_end0 = Total_Energy(S).total();
  std::printf("ENERGY DRIFT %.6e (replica 0: recomputed %.6f, running %.6f, start %.6f)\n", e_end0 - running0, e_end0,
              running0, e_start0);
  for (int r = R - 1; r >= 1; --r) check(grx_box_destroy(boxes[r]), "grx_box_destroy");
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s <example dir> [--precision mixed|fp64] [--cycles-scale f] [--max-cycles n] "
                         "[--dump file.json]\n", argv[0]);
    return 2;
  }
  std::string dir = argv[1], dump;
  ReplicaOptions ro;
  double scale = 1.0;
  long long max_cycles = -1;
  grx_precision prec = GRX_MIXED;
  for (int i = 2; i < argc; ++i) {
    if (!std::strcmp(argv[i], "--precision") && i + 1 < argc) {
      prec = !std::strcmp(argv[++i], "fp64") ? GRX_FP64 : GRX_MIXED;
    } else if (!std::strcmp(argv[i], "--cycles-scale") && i + 1 < argc) {
      scale = std::atof(argv[++i]);
    } else if (!std::strcmp(argv[i], "--max-cycles") && i + 1 < argc) {
      max_cycles = std::atoll(argv[++i]);
    } else if (!std::strcmp(argv[i], "--dump") && i + 1 < argc) {
      dump = argv[++i];
    } else if (!std::strcmp(argv[i], "--replicas") && i + 1 < argc) {
      ro.replicas = std::atoi(argv[++i]);
    } else if (!std::strcmp(argv[i], "--launch-steps") && i + 1 < argc) {
      ro.launch_steps = std::atoll(argv[++i]);
    } else if (!std::strcmp(argv[i], "--init-steps") && i + 1 < argc) {
      ro.init_steps = std::atoll(argv[++i]);
    } else if (!std::strcmp(argv[i], "--prod-steps") && i + 1 < argc) {
      ro.prod_steps = std::atoll(argv[++i]);
    } else if (!std::strcmp(argv[i], "--blocks") && i + 1 < argc) {
      ro.blocks = std::atoi(argv[++i]);
    }
  }
  try {
    Variables V;
    SimulationInput in;
    std::vector<size_t> n_stored;
    Setup_From_Directory(V, dir, in, n_stored);
    V.Precision = prec;
    if (!dump.empty()) {
      dump_json(dump, V, in, n_stored);
      std::printf("dumped %s\n", dump.c_str());
      return 0;
    }
    Setup_Box(V, 0, n_stored);
    Simulations& S = V.Sims[0];
    Components& SC = V.SystemComponents[0];
    const int nc = SC.NComponents.x;
    // initial stage (Ewald_Total, ewald_preparation.h:5-259; exclusion constants :261-298)
    double ew[8];
    check(grx_ewald_total(S.Box.handle, ew), "grx_ewald_total");
    int64_t nvec = 0, nact = 0;
    check(grx_ewald_sizes(S.Box.handle, &nvec, &nact), "grx_ewald_sizes");
    std::printf("INITIAL STAGE ENERGY\n");
    std::printf("EwaldVectors total %lld active %lld alpha %.10f kmax %d %d %d\n", (long long)nvec, (long long)nact,
                S.Box.Alpha, S.Box.kmax.x, S.Box.kmax.y, S.Box.kmax.z);
    std::printf("Fourier GG %.5f HH %.5f HG %.5f\n", ew[0], ew[1], ew[2]);
    std::printf("SelfAtomE all %.5f host %.5f\n", ew[3], ew[4]);
    std::printf("IntraExclusionE all %.5f host %.5f\n", -ew[5], -ew[6]);
    for (int c = 1; c < nc; ++c)
      std::printf("Component %d rigid exclusion intra %.5f self %.5f\n", c, SC.ExclusionIntra[c], SC.ExclusionAtom[c]);
    const double tailE = TailCorrectionEnergy(V, 0);
    std::printf("TailE %.5f\n", tailE);
    // the tail difference of an insertion at the starting counts (exact for host-guest pairs)
    for (int c = 1; c < nc; ++c) SC.TailCorrectionInsert[c] = TailCorrectionInsertion(V, 0, (size_t)c);
    MoveEnergy E0 = Total_Energy(S);
    std::printf("Total HHVDW %.5f HHReal %.5f HGVDW %.5f HGReal %.5f GGVDW %.5f GGReal %.5f HHEwald %.5f HGEwald %.5f "
                "GGEwald %.5f\n", E0.HHVDW, E0.HHReal, E0.HGVDW, E0.HGReal, E0.GGVDW, E0.GGReal, E0.HHEwaldE,
                E0.HGEwaldE, E0.GGEwaldE);
    check(grx_ewald_total(S.Box.handle, ew), "grx_ewald_total");
    // CreateNumberOfMolecules: forced CBMC insertions (InsertionMove::CreateMolecule, move_struct.h:96-108)
    for (int c = 1; c < nc; ++c) {
      const size_t want = in.Components[c - 1].CreateNumberOfMolecules;
      size_t tries = 0;
      while (SC.NumberOfMolecule_for_Component[c] < want && tries < 100000) {
        SC.TempVal.component = (size_t)c;
        InsertionMove m;
        m.Run(V, 0, 0.0);
        SC.Step++;
        ++tries;
      }
    }
    for (int c = 1; c < nc; ++c)
      std::printf("Component %d [%s] fugacity coefficient %.10f mole fraction %.6f\n", c,
                  in.Components[c - 1].MoleculeName.c_str(), SC.FugacityCoeff[c], SC.MolFraction[c]);
    if (ro.replicas > 0) {
      run_replicas(V, in, ro);
      Destroy_Box(V, 0);
      return 0;
    }
    double running = Total_Energy(S).total();
    const double e_start = running;
    check(grx_ewald_total(S.Box.handle, ew), "grx_ewald_total");
    // phases
    struct Phase { const char* name; size_t cycles; bool production; };
    const Phase phases[3] = {{"INITIALIZATION", in.NumberOfInitializationCycles, false},
                             {"EQUILIBRATION", in.NumberOfEquilibrationCycles, false},
                             {"PRODUCTION", in.NumberOfProductionCycles, true}};
    std::vector<BlockStats> blocks(nc);
    std::vector<grx_gcmc_stats> totals(nc);
    std::vector<long long> tr_att(nc), tr_acc(nc), ro_att(nc), ro_acc(nc);
    long long steps_done = 0;
    for (const Phase& ph : phases) {
      size_t cycles = (size_t)std::llround((double)ph.cycles * scale);
      if (max_cycles >= 0) cycles = std::min<size_t>(cycles, (size_t)max_cycles);
      std::printf("== RUNNING %s PHASE == %zu cycles\n", ph.name, cycles);
      const size_t nblock = std::max<size_t>(1, in.NumberOfBlocks);
      const size_t bsize = std::max<size_t>(1, cycles / nblock);
      if (ph.production)
        for (int c = 0; c < nc; ++c) blocks[c] = BlockStats{std::vector<double>(nblock), std::vector<double>(nblock)};
      for (size_t cyc = 0; cyc < cycles; ++cyc) {
        size_t total_mol = 1;
        for (int c = 1; c < nc; ++c) total_mol += SC.NumberOfMolecule_for_Component[c];
        size_t steps = std::max<size_t>(20, total_mol);
        if (in.UseMaxStep && steps > in.MaxStepPerCycle) steps = in.MaxStepPerCycle;
        std::vector<size_t> moved;
        const std::vector<grx_gcmc_stats> st = RunMoves_Device_All(V, 0, (int64_t)steps, &moved);
        steps_done += (long long)steps;
        for (size_t k = 0; k < moved.size(); ++k) {
          const size_t c = moved[k];
          running += st[k].energy[3];
          for (int m = 0; m < 5; ++m) {
            totals[c].attempts[m] += st[k].attempts[m];
            totals[c].accepted[m] += st[k].accepted[m];
          }
          tr_att[c] += st[k].attempts[0]; tr_acc[c] += st[k].accepted[0];
          ro_att[c] += st[k].attempts[1]; ro_acc[c] += st[k].accepted[1];
        }
        if (cyc % 500 == 0) {  // Update_Max_Translation / Update_Max_Rotation
          for (int c = 1; c < nc; ++c) {
            Move_Statistics& M = SC.Moves[c];
            if (tr_att[c] > 0) {
              const double f = (double)tr_acc[c] / (double)tr_att[c] > 0.5 ? 1.05 : 0.95;
              M.MaxTranslation = double3{std::min(5.0, std::max(0.01, M.MaxTranslation.x * f)),
                                         std::min(5.0, std::max(0.01, M.MaxTranslation.y * f)),
                                         std::min(5.0, std::max(0.01, M.MaxTranslation.z * f))};
            }
            if (ro_att[c] > 0) {
              const double f = (double)ro_acc[c] / (double)ro_att[c] > 0.5 ? 1.05 : 0.95;
              M.MaxRotation = double3{std::min(3.14, std::max(0.01, M.MaxRotation.x * f)),
                                      std::min(3.14, std::max(0.01, M.MaxRotation.y * f)),
                                      std::min(3.14, std::max(0.01, M.MaxRotation.z * f))};
            }
            tr_att[c] = tr_acc[c] = ro_att[c] = ro_acc[c] = 0;
          }
        }
        if (ph.production) {
          const size_t blk = std::min(cyc / bsize, nblock - 1);
          for (int c = 1; c < nc; ++c) {
            blocks[c].sum[blk] += (double)SC.NumberOfMolecule_for_Component[c];
            blocks[c].cnt[blk] += 1.0;
          }
        }
      }
      std::printf("%s ends: molecules", ph.name);
      for (int c = 1; c < nc; ++c) std::printf(" [%s] %zu", in.Components[c - 1].MoleculeName.c_str(),
                                               SC.NumberOfMolecule_for_Component[c]);
      std::printf("\n");
    }
    // statistics
    for (int c = 1; c < nc; ++c) {
      const grx_gcmc_stats& t = totals[c];
      std::printf("Component %d [%s] moves: translation %lld/%lld rotation %lld/%lld insertion %lld/%lld deletion "
                  "%lld/%lld reinsertion %lld/%lld\n", c, in.Components[c - 1].MoleculeName.c_str(),
                  (long long)t.accepted[0], (long long)t.attempts[0], (long long)t.accepted[1], (long long)t.attempts[1],
                  (long long)t.accepted[2], (long long)t.attempts[2], (long long)t.accepted[3], (long long)t.attempts[3],
                  (long long)t.accepted[4], (long long)t.attempts[4]);
      const Move_Statistics& M = SC.Moves[c];
      std::printf("Component %d max translation %.6f %.6f %.6f max rotation %.6f\n", c, M.MaxTranslation.x,
                  M.MaxTranslation.y, M.MaxTranslation.z, M.MaxRotation.x);
      std::vector<double> avg;
      for (size_t b = 0; b < blocks[c].sum.size(); ++b)
        if (blocks[c].cnt[b] > 0) avg.push_back(blocks[c].sum[b] / blocks[c].cnt[b]);
      if (!avg.empty()) {
        double m = 0, v = 0;
        for (double a : avg) m += a;
        m /= (double)avg.size();
        for (double a : avg) v += (a - m) * (a - m);
        const double err = avg.size() > 1 ? std::sqrt(v / (double)(avg.size() - 1)) : 0.0;
        std::printf("Component %d average loading %.6f +/- %.6f molecules (%zu blocks)\n", c, m, err, avg.size());
      }
    }
    const double e_end = Total_Energy(S).total();
    std::printf("steps %lld\n", steps_done);
    std::printf("ENERGY DRIFT %.6e (recomputed %.6f, running %.6f, start %.6f)\n", e_end - running, e_end, running,
                e_start);
    Destroy_Box(V, 0);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "graspa_run: %s\n", e.what());
    return 1;
  }
  return 0;
}
