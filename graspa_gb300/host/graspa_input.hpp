// graspa_input.hpp -- readers of gRASPA's input files for the C++ host layer.
//
// simulation.input (read_data.cpp:204-709), pseudo_atoms.def and
// force_field_mixing_rules.def (read_data.cpp:772-1247), molecule .def files and P1 CIF
// frameworks with UnitCells replication (read_data.cpp:1474-2196). Setup_From_Directory
// turns one example directory into a ready Variables / device box.
#pragma once

#include <map>
#include <string>
#include <vector>

#include "graspa_host.hpp"

namespace graspa {

struct InputComponent {
  std::string MoleculeName;
  double IdealGasRosenbluthWeight = 1.0;
  double FugacityCoefficient = 1.0;
  double MolFraction = 1.0;
  double TranslationProbability = 0.0, RotationProbability = 0.0, ReinsertionProbability = 0.0;
  double SwapProbability = 0.0, WidomProbability = 0.0, IdentityChangeProbability = 0.0;
  size_t CreateNumberOfMolecules = 0;
};

struct SimulationInput {
  size_t NumberOfInitializationCycles = 0, NumberOfEquilibrationCycles = 0, NumberOfProductionCycles = 0;
  size_t NumberOfTrialPositions = 10, NumberOfTrialOrientations = 10;
  size_t NumberOfBlocks = 5;
  size_t AdsorbateAllocateSpace = 10240;
  bool UseMaxStep = false;
  size_t MaxStepPerCycle = 1;
  bool UseChargesFromCIFFile = false;
  bool RestartFile = false;   // adsorbate molecules from RestartInitial/System_0/restartfile
  uint64_t RandomSeed = 0;
  std::string InputFileType = "cif";
  std::string FrameworkName;
  int UnitCells[3] = {1, 1, 1};
  std::string ChargeMethod = "Ewald";
  double Temperature = 300.0;
  double Pressure = 1e5;   // Pa
  double OverlapCriteria = 1e5;
  double CutOffVDW = 12.0, CutOffCoulomb = 12.0;
  double EwaldPrecision = 1e-6;
  bool Ewald_UseLAMMPS_Setup = false;
  double Ewald_Alpha = 0.0;
  int Ewald_kvectors[3] = {0, 0, 0};
  std::vector<InputComponent> Components;
};

struct PseudoAtomTable {
  std::vector<std::string> Name;
  std::vector<double> mass, charge;
  int index(const std::string& name) const;
};

struct MixingRules {
  bool shifted = false;
  bool tail = false;
  std::string rule = "Lorentz-Berthelot";
  std::map<std::string, std::pair<double, double>> lj;  // name -> (eps/k in K, sigma in A)
};

// force_field.def: per-pair overrides of the general rules (shifted / truncated and the tail
// correction) and explicit LJ parameters of pairs (eps/k in K, sigma in A).
struct PairOverrides {
  struct Rule { std::string a, b; bool shifted = false, tail = false; };
  struct Pair { std::string a, b; double eps = 0.0, sigma = 0.0; };
  std::vector<Rule> rules;
  std::vector<Pair> pairs;
};

// The adsorbate molecules of a RASPA restart file, per component (in file order).
struct RestartComponent {
  size_t molecules = 0;
  std::vector<double3> pos;       // molecules x atoms, as written
  std::vector<double> charge;     // empty when the file has no charge block
  std::vector<double> lambda;     // scaling per atom (1: full molecule)
  std::vector<size_t> molid;      // absolute molecule ids of the file
};

struct MoleculeDefinition {
  double Tc = 0.0, Pc = 0.0, w = 0.0;
  bool rigid = true;
  std::vector<std::string> names;
  std::vector<double3> pos;
};

struct FrameworkData {
  double cell[9] = {};
  std::vector<double3> pos;
  std::vector<size_t> type;
  std::vector<double> charge;
  double mass = 0.0;  // g/mol of all framework atoms (every unit cell)
};

// Peng-Robinson fugacity coefficients of a gas mixture (the reference's PR-EOS option,
// equations_of_state.h:120-355): critical temperatures (K), pressures (Pa), acentric
// factors and mole fractions of the adsorbates at temperature T (K) and pressure P (Pa),
// binary interaction parameters zero. The cubic in Z is solved in closed form; with
// three real roots the larger-Z and smaller-Z solutions are compared per component and
// the one with the smaller coefficient kept, as the reference does. Throws when the mole
// fractions do not sum to one.
std::vector<double> PengRobinsonFugacity(const std::vector<double>& Tc, const std::vector<double>& Pc,
                                         const std::vector<double>& w, const std::vector<double>& x, double T,
                                         double P);

SimulationInput read_simulation_input(const std::string& path);
PseudoAtomTable read_pseudo_atoms(const std::string& path);
MixingRules read_mixing_rules(const std::string& path);
PairOverrides read_force_field_overrides(const std::string& path);
// RestartFileParser (read_data.cpp:3000-3200): "Component: k ... Adsorbate N molecules" headers
// and the Adsorbate-atom-position / -charge / -scaling lines of each component.
std::vector<RestartComponent> read_restart(const std::string& path, size_t ncomponents);
MoleculeDefinition read_molecule_def(const std::string& path);
FrameworkData read_cif(const std::string& path, const PseudoAtomTable& pa, const int unit_cells[3],
                       bool charges_from_cif);

// Box geometry: inverse cell, volume, orthorhombic flag, and the Ewald parameters of the
// input (read_Ewald_Parameters_from_input, read_data.cpp:609-709).
void Setup_Box_Geometry(Boxsize& Box, const SimulationInput& in);

// Builds Variables (force field, box, components, moves) from an example directory; the
// framework, if any, is component 0. n_stored receives the stored atoms per component.
void Setup_From_Directory(Variables& V, const std::string& dir, SimulationInput& in, std::vector<size_t>& n_stored);

}  // namespace graspa
