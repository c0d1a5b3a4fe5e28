// graspa_input.cpp -- gRASPA input files into the host layer's structs.
#include "graspa_input.hpp"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <fstream>
#include <sstream>

namespace graspa {

namespace {

std::vector<std::string> tokens(const std::string& line) {
  std::vector<std::string> t;
  std::istringstream is(line);
  std::string w;
  while (is >> w) t.push_back(w);
  return t;
}

std::vector<std::string> lines_of(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open " + path);
  std::vector<std::string> out;
  std::string s;
  while (std::getline(f, s)) {
    if (!s.empty() && s.back() == '\r') s.pop_back();
    out.push_back(s);
  }
  return out;
}

bool ieq(const std::string& a, const std::string& b) {
  if (a.size() != b.size()) return false;
  for (size_t i = 0; i < a.size(); ++i)
    if (std::tolower((unsigned char)a[i]) != std::tolower((unsigned char)b[i])) return false;
  return true;
}

bool yes(const std::string& v) { return ieq(v, "yes") || ieq(v, "true") || v == "1"; }

std::string strip_trailing_digits(std::string s) {  // remove_number_at_the_end (read_data.cpp:1407)
  while (!s.empty() && std::isdigit((unsigned char)s.back())) s.pop_back();
  return s;
}

}  // namespace

int PseudoAtomTable::index(const std::string& name) const {
  for (size_t i = 0; i < Name.size(); ++i)
    if (Name[i] == name) return (int)i;
  return -1;
}

// read_simulation_input (read_data.cpp:233-527) and the component block reader
// (read_component_values_from_simulation_input, :2298-).
SimulationInput read_simulation_input(const std::string& path) {
  SimulationInput in;
  InputComponent* cur = nullptr;
  for (const std::string& line : lines_of(path)) {
    const auto t = tokens(line);
    if (t.empty() || t[0][0] == '#') continue;
    const std::string& k = t[0];
    auto num = [&](size_t i) { return i < t.size() ? std::stod(t[i]) : 0.0; };
    if (ieq(k, "Component") && t.size() >= 4 && ieq(t[2], "MoleculeName")) {
      in.Components.emplace_back();
      cur = &in.Components.back();
      cur->MoleculeName = t[3];
      continue;
    }
    if (cur) {
      if (ieq(k, "IdealGasRosenbluthWeight")) { cur->IdealGasRosenbluthWeight = num(1); continue; }
      if (ieq(k, "FugacityCoefficient")) { cur->FugacityCoefficient = num(1); continue; }
      if (ieq(k, "MolFraction")) { cur->MolFraction = num(1); continue; }
      if (ieq(k, "TranslationProbability")) { cur->TranslationProbability = num(1); continue; }
      if (ieq(k, "RotationProbability")) { cur->RotationProbability = num(1); continue; }
      if (ieq(k, "ReinsertionProbability")) { cur->ReinsertionProbability = num(1); continue; }
      if (ieq(k, "SwapProbability")) { cur->SwapProbability = num(1); continue; }
      if (ieq(k, "WidomProbability")) { cur->WidomProbability = num(1); continue; }
      if (ieq(k, "CreateNumberOfMolecules")) { cur->CreateNumberOfMolecules = (size_t)num(1); continue; }
    }
    if (ieq(k, "NumberOfInitializationCycles")) in.NumberOfInitializationCycles = (size_t)num(1);
    else if (ieq(k, "NumberOfEquilibrationCycles")) in.NumberOfEquilibrationCycles = (size_t)num(1);
    else if (ieq(k, "NumberOfProductionCycles")) in.NumberOfProductionCycles = (size_t)num(1);
    else if (ieq(k, "NumberOfTrialPositions")) in.NumberOfTrialPositions = (size_t)num(1);
    else if (ieq(k, "NumberOfTrialOrientations")) in.NumberOfTrialOrientations = (size_t)num(1);
    else if (ieq(k, "NumberOfBlocks")) in.NumberOfBlocks = (size_t)num(1);
    else if (ieq(k, "AdsorbateAllocateSpace")) in.AdsorbateAllocateSpace = (size_t)num(1);
    else if (ieq(k, "UseMaxStep")) in.UseMaxStep = t.size() > 1 && yes(t[1]);
    else if (ieq(k, "MaxStepPerCycle")) in.MaxStepPerCycle = (size_t)num(1);
    else if (ieq(k, "UseChargesFromCIFFile")) in.UseChargesFromCIFFile = t.size() > 1 && yes(t[1]);
    else if (ieq(k, "RandomSeed")) in.RandomSeed = (uint64_t)num(1);
    else if (ieq(k, "InputFileType")) in.InputFileType = t.size() > 1 ? t[1] : "cif";
    else if (ieq(k, "FrameworkName")) in.FrameworkName = t.size() > 1 ? t[1] : "";
    else if (ieq(k, "UnitCells") && t.size() >= 5) {
      in.UnitCells[0] = (int)num(2); in.UnitCells[1] = (int)num(3); in.UnitCells[2] = (int)num(4);
    } else if (ieq(k, "ChargeMethod")) in.ChargeMethod = t.size() > 1 ? t[1] : "Ewald";
    else if (ieq(k, "Temperature")) in.Temperature = num(1);
    else if (ieq(k, "Pressure")) in.Pressure = num(1);
    else if (ieq(k, "OverlapCriteria")) in.OverlapCriteria = num(1);
    else if (ieq(k, "CutOffVDW")) in.CutOffVDW = num(1);
    else if (ieq(k, "CutOffCoulomb")) in.CutOffCoulomb = num(1);
    else if (ieq(k, "EwaldPrecision")) in.EwaldPrecision = num(1);
    else if (ieq(k, "Ewald_UseLAMMPS_Setup")) in.Ewald_UseLAMMPS_Setup = t.size() > 1 && yes(t[1]);
    else if (ieq(k, "Ewald_Alpha")) in.Ewald_Alpha = num(1);
    else if (ieq(k, "Ewald_kvectors") && t.size() >= 4) {
      in.Ewald_kvectors[0] = (int)num(1); in.Ewald_kvectors[1] = (int)num(2); in.Ewald_kvectors[2] = (int)num(3);
    }
  }
  return in;
}

// PseudoAtomParser (read_data.cpp:1324-1351): line 1 count, entries from line 3:
// name print symbol chem oxidation mass charge polarization.
PseudoAtomTable read_pseudo_atoms(const std::string& path) {
  PseudoAtomTable pa;
  const auto L = lines_of(path);
  size_t n = 0;
  for (size_t i = 0; i < L.size(); ++i) {
    const auto t = tokens(L[i]);
    if (i == 1) {
      if (t.empty()) throw std::runtime_error("pseudo_atoms.def: missing count");
      n = (size_t)std::stoul(t[0]);
    } else if (i >= 3 && pa.Name.size() < n) {
      if (t.size() < 7) throw std::runtime_error("pseudo_atoms.def: short entry: " + L[i]);
      pa.Name.push_back(t[0]);
      pa.mass.push_back(std::stod(t[5]));
      pa.charge.push_back(std::stod(t[6]));
    }
  }
  if (pa.Name.size() != n) throw std::runtime_error("pseudo_atoms.def: fewer entries than declared");
  return pa;
}

// ForceFieldParser (read_data.cpp:772-830): line 1 shifted/truncated, line 3 tail
// corrections, line 5 count, definitions from line 7 (name type eps/k sigma).
MixingRules read_mixing_rules(const std::string& path) {
  MixingRules m;
  const auto L = lines_of(path);
  size_t n = 0, got = 0;
  for (size_t i = 0; i < L.size(); ++i) {
    const auto t = tokens(L[i]);
    if (i == 1 && !t.empty()) m.shifted = t[0] == "shifted";
    else if (i == 3 && !t.empty()) m.tail = t[0] == "yes";
    else if (i == 5 && !t.empty()) n = (size_t)std::stoul(t[0]);
    else if (i >= 7 && got < n) {
      if (t.size() < 4) throw std::runtime_error("force_field_mixing_rules.def: short entry: " + L[i]);
      m.lj[t[0]] = {std::stod(t[2]), std::stod(t[3])};
      ++got;
    } else if (i >= 7 + n && !t.empty() && t[0][0] != '#') {
      m.rule = t[0];
    }
  }
  if (got != n) throw std::runtime_error("force_field_mixing_rules.def: fewer definitions than declared");
  return m;
}

// MoleculeDefinitionParser (read_data.cpp:2044-2140): line 1 Tc, 2 Pc, 3 acentric factor,
// 5 atom count, 9 rigid, positions from line 13 (index name x y z).
MoleculeDefinition read_molecule_def(const std::string& path) {
  MoleculeDefinition d;
  const auto L = lines_of(path);
  size_t n = 0;
  for (size_t i = 0; i < L.size(); ++i) {
    const auto t = tokens(L[i]);
    if (t.empty()) continue;
    if (i == 1) d.Tc = std::stod(t[0]);
    else if (i == 2) d.Pc = std::stod(t[0]);
    else if (i == 3) d.w = std::stod(t[0]);
    else if (i == 5) n = (size_t)std::stoul(t[0]);
    else if (i == 9) {
      if (!ieq(t[0], "rigid")) throw std::runtime_error(path + ": only rigid molecules are supported");
    } else if (i >= 13 && d.names.size() < n) {
      if (t.size() < 5) throw std::runtime_error(path + ": short position line: " + L[i]);
      d.names.push_back(t[1]);
      d.pos.push_back(double3{std::stod(t[2]), std::stod(t[3]), std::stod(t[4])});
    }
  }
  if (d.names.size() != n || n == 0) throw std::runtime_error(path + ": atom positions missing");
  return d;
}

// CheckFrameworkCIF (read_data.cpp:1474-1790): cell from lengths and angles times the
// unit cells; P1 atom sites, labels without their trailing digits matched to pseudo
// atoms; charges from the CIF or the pseudo atoms; replication unit cell by unit cell
// (ix, then iy, then iz) with fractional (f + n) / N.
FrameworkData read_cif(const std::string& path, const PseudoAtomTable& pa, const int uc[3], bool charges_from_cif) {
  FrameworkData F;
  const auto L = lines_of(path);
  double a = 0, b = 0, c = 0, al = 90, be = 90, ga = 90;
  for (const auto& s : L) {
    const auto t = tokens(s);
    if (t.size() < 2) continue;
    if (t[0] == "_cell_length_a") a = std::stod(t[1]);
    else if (t[0] == "_cell_length_b") b = std::stod(t[1]);
    else if (t[0] == "_cell_length_c") c = std::stod(t[1]);
    else if (t[0] == "_cell_angle_alpha") al = std::stod(t[1]);
    else if (t[0] == "_cell_angle_beta") be = std::stod(t[1]);
    else if (t[0] == "_cell_angle_gamma") ga = std::stod(t[1]);
  }
  const double deg = 180.0 / 3.14159265358979323846;
  al /= deg; be /= deg; ga /= deg;
  const double ax = a, by = b * std::sin(ga);
  const double tempd = (std::cos(al) - std::cos(ga) * std::cos(be)) / std::sin(ga);
  const double cz = c * std::sqrt(1 - std::pow(std::cos(be), 2) - std::pow(tempd, 2));
  const double bx = b * std::cos(ga), cx = c * std::cos(be), cy = c * tempd;
  double* C = F.cell;
  C[0] = uc[0] * ax; C[1] = 0.0;         C[2] = 0.0;
  C[3] = uc[1] * bx; C[4] = uc[1] * by;  C[5] = 0.0;
  C[6] = uc[2] * cx; C[7] = uc[2] * cy;  C[8] = uc[2] * cz;
  // the atom-site loop
  int col_label = -1, col_x = -1, col_y = -1, col_z = -1, col_q = -1, ncol = 0;
  size_t first = 0;
  bool in_loop = false;
  for (size_t i = 0; i < L.size(); ++i) {
    const auto t = tokens(L[i]);
    if (t.empty()) continue;
    if (t[0].rfind("_atom_site", 0) == 0) {
      in_loop = true;
      if (t[0] == "_atom_site_label") col_label = ncol;
      if (t[0] == "_atom_site_fract_x") col_x = ncol;
      if (t[0] == "_atom_site_fract_y") col_y = ncol;
      if (t[0] == "_atom_site_fract_z") col_z = ncol;
      if (t[0] == "_atom_site_charge") col_q = ncol;
      ++ncol;
      first = i + 1;
    } else if (in_loop) {
      break;
    }
  }
  if (col_label < 0 || col_x < 0 || col_y < 0 || col_z < 0)
    throw std::runtime_error(path + ": label / fract_x / fract_y / fract_z columns not found");
  std::vector<double3> fpos;
  std::vector<size_t> type;
  std::vector<double> q;
  for (size_t i = first; i < L.size(); ++i) {
    const auto t = tokens(L[i]);
    if ((int)t.size() < 4 || (int)t.size() < ncol) break;
    const std::string name = strip_trailing_digits(t[col_label]);
    const int ty = pa.index(name);
    if (ty < 0) throw std::runtime_error(path + ": atom label [" + name + "] not defined");
    fpos.push_back(double3{std::stod(t[col_x]), std::stod(t[col_y]), std::stod(t[col_z])});
    type.push_back((size_t)ty);
    q.push_back(charges_from_cif && col_q >= 0 ? std::stod(t[col_q]) : pa.charge[ty]);
  }
  const double sx = 1.0 / uc[0], sy = 1.0 / uc[1], sz = 1.0 / uc[2];
  for (int ix = 0; ix < uc[0]; ++ix)
    for (int iy = 0; iy < uc[1]; ++iy)
      for (int iz = 0; iz < uc[2]; ++iz)
        for (size_t k = 0; k < fpos.size(); ++k) {
          const double fx = (fpos[k].x + ix) * sx, fy = (fpos[k].y + iy) * sy, fz = (fpos[k].z + iz) * sz;
          F.pos.push_back(double3{fx * C[0] + fy * C[3] + fz * C[6], fx * C[1] + fy * C[4] + fz * C[7],
                                  fx * C[2] + fy * C[5] + fz * C[8]});
          F.type.push_back(type[k]);
          F.charge.push_back(q[k]);
        }
  return F;
}

void Setup_Box_Geometry(Boxsize& B, const SimulationInput& in) {
  const double* x = B.Cell;
  const double m11 = x[0], m21 = x[3], m31 = x[6], m12 = x[1], m22 = x[4], m32 = x[7];
  const double m13 = x[2], m23 = x[5], m33 = x[8];
  const double det = m11 * (m22 * m33 - m23 * m32) - m12 * (m21 * m33 - m23 * m31) + m13 * (m21 * m32 - m22 * m31);
  double* v = B.InverseCell;
  v[0] = (m22 * m33 - m32 * m23) / det;
  v[3] = -(m21 * m33 - m31 * m23) / det;
  v[6] = (m21 * m32 - m31 * m22) / det;
  v[1] = -(m12 * m33 - m32 * m13) / det;
  v[4] = (m11 * m33 - m31 * m13) / det;
  v[7] = -(m11 * m32 - m31 * m12) / det;
  v[2] = (m12 * m23 - m22 * m13) / det;
  v[5] = -(m11 * m23 - m21 * m13) / det;
  v[8] = (m11 * m22 - m21 * m12) / det;
  B.Volume = det;
  B.Cubic = std::fabs(x[3]) + std::fabs(x[6]) + std::fabs(x[7]) <= 1e-10;
  B.Prefactor = 138935.483496;
  const double pi = 3.14159265358979323846;
  if (in.Ewald_UseLAMMPS_Setup) {  // explicit alpha and kmax (read_data.cpp:632-687)
    B.UseLAMMPSEwald = true;
    B.Alpha = in.Ewald_Alpha;
    B.kmax = int3{in.Ewald_kvectors[0], in.Ewald_kvectors[1], in.Ewald_kvectors[2]};
    const double lx = x[0], ly = x[4], lz = x[8];
    const double kvx = B.kmax.x * (2 * pi / lx), kvy = B.kmax.y * (2 * pi / ly), kvz = B.kmax.z * (2 * pi / lz);
    B.ReciprocalCutOff = std::max(kvx * kvx, std::max(kvy * kvy, kvz * kvz)) * 1.00001;
  } else {  // from the precision (read_data.cpp:689-700)
    B.UseLAMMPSEwald = false;
    const double rc = in.CutOffCoulomb, p = in.EwaldPrecision;
    const double tol = std::sqrt(std::fabs(std::log(p * rc)));
    B.Alpha = std::sqrt(std::fabs(std::log(p * rc * tol))) / rc;
    const double tol1 = std::sqrt(-std::log(p * rc * std::pow(2.0 * tol * B.Alpha, 2)));
    B.tol1 = tol1;
    B.kmax = int3{(int)std::round(0.25 + x[0] * B.Alpha * tol1 / pi), (int)std::round(0.25 + x[4] * B.Alpha * tol1 / pi),
                  (int)std::round(0.25 + x[8] * B.Alpha * tol1 / pi)};
    B.ReciprocalCutOff = std::pow(1.05 * (double)std::max(B.kmax.x, std::max(B.kmax.y, B.kmax.z)), 2);
  }
}

void Setup_From_Directory(Variables& V, const std::string& dir, SimulationInput& in, std::vector<size_t>& n_stored) {
  const std::string d = dir.empty() || dir.back() == '/' ? dir : dir + "/";
  in = read_simulation_input(d + "simulation.input");
  const PseudoAtomTable pa = read_pseudo_atoms(d + "pseudo_atoms.def");
  const MixingRules mr = read_mixing_rules(d + "force_field_mixing_rules.def");
  if (!ieq(mr.rule, "Lorentz-Berthelot")) throw std::runtime_error("only Lorentz-Berthelot mixing is supported");
  V.Sims.assign(1, Simulations());
  V.SystemComponents.assign(1, Components());
  V.Widom.assign(1, WidomStruct());
  Simulations& S = V.Sims[0];
  Components& SC = V.SystemComponents[0];
  // force field in pseudo-atom order (the reference requires the two files to agree)
  ForceField& FF = V.device_FF;
  const size_t nt = pa.Name.size();
  FF.size = nt;
  FF.epsilon.assign(nt * nt, 0.0);
  FF.sigma.assign(nt * nt, 0.0);
  FF.shift.assign(nt * nt, 0.0);
  const double rc2 = in.CutOffVDW * in.CutOffVDW;
  for (size_t i = 0; i < nt; ++i)
    for (size_t j = 0; j < nt; ++j) {
      auto fi = mr.lj.find(pa.Name[i]), fj = mr.lj.find(pa.Name[j]);
      const double ei = fi == mr.lj.end() ? 0.0 : fi->second.first, si = fi == mr.lj.end() ? 0.0 : fi->second.second;
      const double ej = fj == mr.lj.end() ? 0.0 : fj->second.first, sj = fj == mr.lj.end() ? 0.0 : fj->second.second;
      const double ep = std::sqrt(ei * ej) / 1.20272430057, sg = 0.5 * (si + sj);
      FF.epsilon[i * nt + j] = ep;
      FF.sigma[i * nt + j] = sg;
      if (mr.shifted && sg > 0.0) {  // Get_Shifted_Value (read_data.cpp:737-746)
        const double t = rc2 / (sg * sg), rri3 = 1.0 / (t * t * t);
        FF.shift[i * nt + j] = 4.0 * ep * (rri3 * (rri3 - 1.0));
      }
    }
  FF.CutOffVDW = rc2;
  FF.CutOffCoul = in.CutOffCoulomb * in.CutOffCoulomb;
  FF.OverlapCriteria = in.OverlapCriteria;
  FF.noCharges = ieq(in.ChargeMethod, "None");
  FF.VDWRealBias = true;
  // framework
  const bool has_fw = !in.FrameworkName.empty() && in.InputFileType == "cif";
  FrameworkData fw;
  if (has_fw) {
    fw = read_cif(d + in.FrameworkName + ".cif", pa, in.UnitCells, in.UseChargesFromCIFFile);
    std::copy(fw.cell, fw.cell + 9, S.Box.Cell);
  } else {
    throw std::runtime_error("an example without a CIF framework needs a restart file (not supported)");
  }
  Setup_Box_Geometry(S.Box, in);
  // components: 0 framework, then the adsorbates
  const int nads = (int)in.Components.size();
  const int nc = 1 + nads;
  SC.NComponents = int3{nc, 1, nads};
  SC.Temperature = in.Temperature;
  SC.Beta = 1.0 / (1.380649e-23 / (1.6605402e-27 * std::pow(1e-10, 2) / std::pow(1e-12, 2)) * in.Temperature);
  SC.Pressure = in.Pressure / (1.6605402e-27 / (1e-10 * std::pow(1e-12, 2)));
  SC.Moleculesize.assign(nc, 0);
  SC.Allocate_size.assign(nc, 0);
  SC.NumberOfMolecule_for_Component.assign(nc, 0);
  SC.rigid.assign(nc, true);
  SC.IdealRosenbluthWeight.assign(nc, 1.0);
  SC.FugacityCoeff.assign(nc, 1.0);
  SC.MolFraction.assign(nc, 1.0);
  SC.TailCorrectionInsert.assign(nc, 0.0);
  SC.Moves.assign(nc, Move_Statistics());
  SC.Nblock = in.NumberOfBlocks;
  S.host.assign(nc, HostAtoms());
  S.d_a.assign(nc, Atoms());
  n_stored.assign(nc, 0);
  SC.Moleculesize[0] = fw.pos.size();
  SC.Allocate_size[0] = fw.pos.size();
  SC.rigid[0] = false;
  S.host[0].allocate(fw.pos.size());
  for (size_t i = 0; i < fw.pos.size(); ++i) {
    S.host[0].pos[i] = fw.pos[i];
    S.host[0].charge[i] = FF.noCharges ? 0.0 : fw.charge[i];
    S.host[0].Type[i] = fw.type[i];
    S.host[0].MolID[i] = 0;
  }
  S.d_a[0] = S.host[0].view(fw.pos.size(), fw.pos.size());
  n_stored[0] = fw.pos.size();
  for (int k = 0; k < nads; ++k) {
    const InputComponent& ic = in.Components[k];
    const int c = 1 + k;
    const MoleculeDefinition md = read_molecule_def(d + ic.MoleculeName + ".def");
    const size_t ms = md.names.size();
    SC.Moleculesize[c] = ms;
    SC.Allocate_size[c] = std::max(in.AdsorbateAllocateSpace / ms * ms, ms);
    SC.IdealRosenbluthWeight[c] = ic.IdealGasRosenbluthWeight;
    SC.FugacityCoeff[c] = ic.FugacityCoefficient;
    SC.MolFraction[c] = ic.MolFraction;
    Move_Statistics& M = SC.Moves[c];
    M.TranslationProb = ic.TranslationProbability;
    M.RotationProb = ms > 1 ? ic.RotationProbability : 0.0;
    M.ReinsertionProb = ic.ReinsertionProbability;
    M.SwapProb = ic.SwapProbability;
    M.NormalizeProbabilities();
    M.NumberOfTrials = in.NumberOfTrialPositions;
    // InitializeMaxTranslationRotation (fxn_main.h:216-228)
    M.MaxTranslation = double3{S.Box.Cell[0] * 0.1, S.Box.Cell[4] * 0.1, S.Box.Cell[8] * 0.1};
    const double r30 = 30.0 / (180 / 3.1415);
    M.MaxRotation = double3{r30, r30, r30};
    HostAtoms& H = S.host[c];
    H.allocate(SC.Allocate_size[c]);
    for (size_t a = 0; a < ms; ++a) {  // the empty component stores its template
      const int ty = pa.index(md.names[a]);
      if (ty < 0) throw std::runtime_error(ic.MoleculeName + ".def: atom [" + md.names[a] + "] not in pseudo_atoms.def");
      H.pos[a] = md.pos[a];
      H.charge[a] = FF.noCharges ? 0.0 : pa.charge[ty];
      H.Type[a] = (size_t)ty;
      H.MolID[a] = 0;
    }
    S.d_a[c] = H.view(ms, 0);
    n_stored[c] = ms;
  }
  V.Widom[0].NumberWidomTrials = in.NumberOfTrialPositions;
  V.Widom[0].NumberWidomTrialsOrientations = in.NumberOfTrialOrientations;
  V.Random.Seed = in.RandomSeed;
}

}  // namespace graspa
