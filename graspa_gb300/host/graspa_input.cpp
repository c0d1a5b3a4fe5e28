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
      if (ieq(k, "FugacityCoefficient")) {  // a number, or PR-EOS (stored as -1, the reference's flag)
        if (t.size() > 1 && ieq(t[1], "PR-EOS")) cur->FugacityCoefficient = -1.0;
        else cur->FugacityCoefficient = num(1);
        continue;
      }
      if (ieq(k, "IdentityChangeProbability")) { cur->IdentityChangeProbability = num(1); continue; }
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
    else if (ieq(k, "RestartFile")) in.RestartFile = t.size() > 1 && yes(t[1]);
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

// OverWriteFFTerms / the force_field.def reader (read_data.cpp:831-1000): a count of rule
// overrides "A B shifted|truncated yes|no" (the last word switches the tail correction), a
// count of explicit pairs "A B lennard-jones eps sigma", and a count of mixing overrides
// (only 0 is supported). Comment lines start with '#'.
PairOverrides read_force_field_overrides(const std::string& path) {
  PairOverrides o;
  std::vector<std::vector<std::string>> rows;
  for (const std::string& l : lines_of(path)) {
    const auto t = tokens(l);
    if (t.empty() || t[0][0] == '#') continue;
    rows.push_back(t);
  }
  size_t r = 0;
  auto count = [&]() -> size_t {
    if (r >= rows.size()) return 0;
    return (size_t)std::stoul(rows[r++][0]);
  };
  const size_t nrules = count();
  for (size_t k = 0; k < nrules && r < rows.size(); ++k, ++r) {
    const auto& t = rows[r];
    if (t.size() < 3) throw std::runtime_error("force_field.def: short rule: " + t[0]);
    PairOverrides::Rule x;
    x.a = t[0];
    x.b = t[1];
    x.shifted = ieq(t[2], "shifted");
    x.tail = t.size() > 3 && yes(t[3]);
    o.rules.push_back(x);
  }
  const size_t npairs = count();
  for (size_t k = 0; k < npairs && r < rows.size(); ++k, ++r) {
    const auto& t = rows[r];
    if (t.size() < 5 || !ieq(t[2], "lennard-jones"))
      throw std::runtime_error("force_field.def: only lennard-jones pairs are supported: " + t[0] + " " + t[1]);
    o.pairs.push_back({t[0], t[1], std::stod(t[3]), std::stod(t[4])});
  }
  if (count() != 0) throw std::runtime_error("force_field.def: mixing-rule overrides are not supported");
  return o;
}

std::vector<RestartComponent> read_restart(const std::string& path, size_t ncomponents) {
  std::vector<RestartComponent> out(ncomponents);
  int cur = -1;
  for (const std::string& line : lines_of(path)) {
    const auto t = tokens(line);
    if (t.empty()) continue;
    if (t[0] == "Component:" && t.size() >= 4 && t[2] == "Adsorbate") {
      cur = std::stoi(t[1]);
      if (cur < 0 || cur >= (int)ncomponents) throw std::runtime_error("restart file: unknown component " + t[1]);
      out[cur].molecules = (size_t)std::stoul(t[3]);
      continue;
    }
    if (cur < 0) continue;
    RestartComponent& R = out[cur];
    if (t[0] == "Adsorbate-atom-position:" && t.size() >= 6) {
      R.molid.push_back((size_t)std::stoul(t[1]));
      R.pos.push_back(double3{std::stod(t[3]), std::stod(t[4]), std::stod(t[5])});
    } else if (t[0] == "Adsorbate-atom-charge:" && t.size() >= 4) {
      R.charge.push_back(std::stod(t[3]));
    } else if (t[0] == "Adsorbate-atom-scaling:" && t.size() >= 4) {
      R.lambda.push_back(std::stod(t[3]));
    }
  }
  return out;
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
      // "index name x y z"; a position line without coordinates puts the atom at the origin
      // (single-atom molecules such as Kr.def of the XeKr example)
      if (t.size() < 2 || (t.size() > 2 && t.size() < 5))
        throw std::runtime_error(path + ": short position line: " + L[i]);
      d.names.push_back(t[1]);
      d.pos.push_back(t.size() >= 5 ? double3{std::stod(t[2]), std::stod(t[3]), std::stod(t[4])} : double3{0.0, 0.0, 0.0});
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
    F.mass += pa.mass[ty] * (double)(uc[0] * uc[1] * uc[2]);
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

std::vector<double> PengRobinsonFugacity(const std::vector<double>& Tc, const std::vector<double>& Pc,
                                         const std::vector<double>& w, const std::vector<double>& x, double T,
                                         double P) {
  const size_t n = Tc.size();
  double xs = 0.0;
  for (double v : x) xs += v;
  if (std::fabs(xs - 1.0) > 1e-4) throw std::runtime_error("PR-EOS: mole fractions do not sum to 1");
  // per-component attraction and co-volume in reduced form: A_i = a_i P / (R T)^2, B_i = b_i P / (R T)
  // (R cancels), a_i = 0.45724 alpha_i (R Tc_i)^2 / Pc_i, b_i = 0.07780 R Tc_i / Pc_i
  std::vector<double> A(n), B(n);
  for (size_t i = 0; i < n; ++i) {
    const double kappa = 0.37464 + 1.54226 * w[i] - 0.26992 * w[i] * w[i];
    const double sq = 1.0 + kappa * (1.0 - std::sqrt(T / Tc[i]));
    const double alpha = sq * sq;
    A[i] = 0.45724 * alpha * (Tc[i] / T) * (Tc[i] / T) * P / Pc[i];
    B[i] = 0.07780 * (Tc[i] / T) * P / Pc[i];
  }
  double Am = 0.0, Bm = 0.0;
  for (size_t i = 0; i < n; ++i) {
    Bm += x[i] * B[i];
    for (size_t j = 0; j < n; ++j) Am += x[i] * x[j] * std::sqrt(A[i] * A[j]);
  }
  // Z^3 + c2 Z^2 + c1 Z + c0 = 0, solved by the depressed cubic t^3 + p t + q (Z = t - c2/3)
  const double c2 = Bm - 1.0, c1 = Am - 3.0 * Bm * Bm - 2.0 * Bm, c0 = -(Am * Bm - Bm * Bm - Bm * Bm * Bm);
  const double p = c1 - c2 * c2 / 3.0, q = 2.0 * c2 * c2 * c2 / 27.0 - c2 * c1 / 3.0 + c0;
  const double disc = q * q / 4.0 + p * p * p / 27.0;
  std::vector<double> Z;
  if (disc > 0.0) {
    const double sd = std::sqrt(disc);
    Z.push_back(std::cbrt(-q / 2.0 + sd) + std::cbrt(-q / 2.0 - sd) - c2 / 3.0);
  } else {
    const double r = std::sqrt(-p / 3.0);
    const double cphi = r > 0.0 ? std::max(-1.0, std::min(1.0, -q / (2.0 * r * r * r))) : 0.0;
    const double phi = std::acos(cphi), pi = 3.14159265358979323846;
    for (int k = 0; k < 3; ++k) Z.push_back(2.0 * r * std::cos((phi + 2.0 * pi * k) / 3.0) - c2 / 3.0);
    std::sort(Z.begin(), Z.end(), [](double a, double b) { return a > b; });
  }
  auto phi_of = [&](size_t i, double z) {
    double sa = 0.0;
    for (size_t k = 0; k < n; ++k) sa += 2.0 * x[k] * std::sqrt(A[i] * A[k]);
    const double r2 = std::sqrt(2.0);
    return std::exp(B[i] / Bm * (z - 1.0) - std::log(z - Bm) -
                    Am / (2.0 * r2 * Bm) * (sa / Am - B[i] / Bm) * std::log((z + (1.0 + r2) * Bm) / (z + (1.0 - r2) * Bm)));
  };
  std::vector<double> out(n);
  for (size_t i = 0; i < n; ++i) {
    if (Z.size() == 1 || Z[2] <= 0.0) {
      out[i] = phi_of(i, Z[0]);
    } else {  // vapour-like and liquid-like roots: the smaller coefficient (the stable phase)
      const double f0 = phi_of(i, Z[0]), f2 = phi_of(i, Z[2]);
      out[i] = f2 < f0 ? f2 : f0;
    }
  }
  return out;
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
  // force_field.def: per-pair shifted / truncated and tail rules, explicit pairs
  FF.tail.assign(nt * nt, mr.tail ? 1 : 0);
  {
    std::ifstream probe(d + "force_field.def");
    if (probe) {
      const PairOverrides ov = read_force_field_overrides(d + "force_field.def");
      auto apply = [&](const std::string& a, const std::string& b, auto&& f) {
        const int i = pa.index(a), j = pa.index(b);
        if (i < 0 || j < 0) return;  // a pseudo atom the system does not use
        f((size_t)i * nt + (size_t)j);
        f((size_t)j * nt + (size_t)i);
      };
      for (const auto& p : ov.pairs)
        apply(p.a, p.b, [&](size_t k) {
          FF.epsilon[k] = p.eps / 1.20272430057;
          FF.sigma[k] = p.sigma;
        });
      for (const auto& x : ov.rules)
        apply(x.a, x.b, [&](size_t k) {
          FF.tail[k] = x.tail ? 1 : 0;
          FF.shift[k] = 0.0;
          if (x.shifted && FF.sigma[k] > 0.0) {
            const double tt = rc2 / (FF.sigma[k] * FF.sigma[k]), rri3 = 1.0 / (tt * tt * tt);
            FF.shift[k] = 4.0 * FF.epsilon[k] * (rri3 * (rri3 - 1.0));
          }
        });
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
    throw std::runtime_error("an example needs a CIF framework (it defines the box, possibly without atoms)");
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
  SC.Allocate_size[0] = std::max<size_t>(1, fw.pos.size());  // a CIF may only define the box
  SC.rigid[0] = false;
  S.host[0].allocate(SC.Allocate_size[0]);
  for (size_t i = 0; i < fw.pos.size(); ++i) {
    S.host[0].pos[i] = fw.pos[i];
    S.host[0].charge[i] = FF.noCharges ? 0.0 : fw.charge[i];
    S.host[0].Type[i] = fw.type[i];
    S.host[0].MolID[i] = 0;
  }
  S.d_a[0] = S.host[0].view(fw.pos.size(), fw.pos.size());
  n_stored[0] = fw.pos.size();
  std::vector<RestartComponent> restart;
  if (in.RestartFile) restart = read_restart(d + "RestartInitial/System_0/restartfile", (size_t)nads);
  size_t first_molid = 0;  // molecule ids of the file count through the components
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
    M.IdentitySwapProb = ic.IdentityChangeProbability;
    M.SwapProb = ic.SwapProbability;
    M.NormalizeProbabilities();
    M.NumberOfTrials = in.NumberOfTrialPositions;
    // InitializeMaxTranslationRotation (fxn_main.h:216-228)
    M.MaxTranslation = double3{S.Box.Cell[0] * 0.1, S.Box.Cell[4] * 0.1, S.Box.Cell[8] * 0.1};
    const double r30 = 30.0 / (180 / 3.1415);
    M.MaxRotation = double3{r30, r30, r30};
    HostAtoms& H = S.host[c];
    const RestartComponent* R = restart.empty() ? nullptr : &restart[k];
    const size_t nmol = R ? R->molecules : 0;
    if (nmol * ms > SC.Allocate_size[c]) SC.Allocate_size[c] = nmol * ms;
    H.allocate(SC.Allocate_size[c]);
    std::vector<size_t> types(ms);
    for (size_t a = 0; a < ms; ++a) {  // the empty component stores its template
      const int ty = pa.index(md.names[a]);
      if (ty < 0) throw std::runtime_error(ic.MoleculeName + ".def: atom [" + md.names[a] + "] not in pseudo_atoms.def");
      types[a] = (size_t)ty;
      H.pos[a] = md.pos[a];
      H.charge[a] = FF.noCharges ? 0.0 : pa.charge[ty];
      H.Type[a] = (size_t)ty;
      H.MolID[a] = 0;
    }
    if (nmol > 0) {
      // RestartFileParser (read_data.cpp:3085-3200): molecule ids relative to the component,
      // every atom brought to the image nearest the molecule's first atom, charges from the file
      if (R->pos.size() != nmol * ms) throw std::runtime_error("restart file: component " + std::to_string(k) +
                                                              " has the wrong number of atom positions");
      for (double l : R->lambda)
        if (l < 1.0) throw std::runtime_error("restart file: fractional molecules (lambda < 1) are not supported");
      for (size_t m = 0; m < nmol; ++m)
        for (size_t a = 0; a < ms; ++a) {
          const size_t i = m * ms + a;
          double3 p = R->pos[i];
          if (a > 0) {
            double3 dv{p.x - H.pos[m * ms].x, p.y - H.pos[m * ms].y, p.z - H.pos[m * ms].z};
            Minimum_Image(S.Box, dv);
            p = double3{H.pos[m * ms].x + dv.x, H.pos[m * ms].y + dv.y, H.pos[m * ms].z + dv.z};
          }
          H.pos[i] = p;
          H.charge[i] = FF.noCharges ? 0.0 : (R->charge.size() == R->pos.size() ? R->charge[i] : pa.charge[types[a]]);
          H.Type[i] = types[a];
          H.MolID[i] = R->molid[i] - first_molid;
        }
      first_molid += nmol;
      SC.NumberOfMolecule_for_Component[c] = nmol;
    }
    S.d_a[c] = H.view(ms, nmol * ms);
    n_stored[c] = std::max(ms, nmol * ms);
  }
  // FugacityCoefficient PR-EOS on any adsorbate: all coefficients from the Peng-Robinson
  // mixture (equations_of_state.h:130-143)
  bool need_eos = false;
  for (const InputComponent& ic : in.Components) need_eos |= ic.FugacityCoefficient < 0.0;
  SC.Tc.assign(nc, 0.0);
  SC.Pc.assign(nc, 0.0);
  SC.Accentric.assign(nc, 0.0);
  for (int k = 0; k < nads; ++k) {
    const MoleculeDefinition md = read_molecule_def(d + in.Components[k].MoleculeName + ".def");
    SC.Tc[1 + k] = md.Tc;
    SC.Pc[1 + k] = md.Pc;
    SC.Accentric[1 + k] = md.w;
  }
  if (need_eos && nads > 0) {
    std::vector<double> tc, pc, w, x;
    for (int k = 0; k < nads; ++k) {
      tc.push_back(SC.Tc[1 + k]);
      pc.push_back(SC.Pc[1 + k]);
      w.push_back(SC.Accentric[1 + k]);
      x.push_back(in.Components[k].MolFraction);
    }
    const std::vector<double> phi = PengRobinsonFugacity(tc, pc, w, x, in.Temperature, in.Pressure);
    for (int k = 0; k < nads; ++k) SC.FugacityCoeff[1 + k] = phi[k];
  }
  SC.FrameworkMass = fw.mass;
  V.Widom[0].NumberWidomTrials = in.NumberOfTrialPositions;
  V.Widom[0].NumberWidomTrialsOrientations = in.NumberOfTrialOrientations;
  V.Random.Seed = in.RandomSeed;
}

}  // namespace graspa
