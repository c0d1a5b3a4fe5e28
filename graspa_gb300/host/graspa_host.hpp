// graspa_host.hpp -- C++ host layer with gRASPA's state structs and move drivers,
// calling libgrx through its C ABI (include/grx.h).
//
// The structs keep the reference's names and the fields the energy path reads
// (data_struct.h: Atoms 788-799, ForceField 838-855, Boxsize 865-886,
// CBMC_Variables 889-911, Components 975-1254, Simulations 1255-1267,
// WidomStruct 1271-1278, Variables 1378-1420, MoveEnergy 416-488). The device state
// (positions, structure factors, tiles) lives in one grx_box per simulation box,
// held by Simulations::Box.handle; Simulations::d_a is the host mirror that the
// move drivers keep in step with it. The drivers restate the reference's move
// code one call at a time (mc_widom.h, move_struct.h, mc_swap_utilities.h,
// mc_single_particle.h, axpy.cu RunMoves), so a reference-shaped program keeps its
// structure and its calls: CBMC_PairwiseInteractions, GPU_EwaldDifference_General,
// Update_Vector_Ewald, SingleBody energies and the FP64 totals go to the GPU.
//
// Random numbers come from the library's Philox stream (grx_philox.h) instead of
// the reference's pre-filled table, so these host-driven moves take the same
// decisions as the device-resident driver grx_gcmc_run for the same seed.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "grx.h"
#include "grx_philox.h"

namespace graspa {

struct double2 { double x = 0.0, y = 0.0; };
struct double3 { double x = 0.0, y = 0.0, z = 0.0; };
struct int3 { int x = 0, y = 0, z = 0; };

// Move types, numbered as MoveTypes (data_struct.h:20).
enum MoveTypes {
  TRANSLATION = 0, ROTATION, SINGLE_INSERTION, SINGLE_DELETION, SPECIAL_ROTATION, INSERTION, DELETION,
  REINSERTION, CBCF_LAMBDACHANGE, CBCF_INSERTION, CBCF_DELETION, IDENTITY_SWAP
};
// CBMC step kinds (data_struct.h:21).
enum CBMC_Types {
  CBMC_INSERTION = 0, CBMC_DELETION, REINSERTION_INSERTION, REINSERTION_RETRACE, IDENTITY_SWAP_NEW,
  IDENTITY_SWAP_OLD
};

struct MoveEnergy {
  double HHVDW = 0.0, HGVDW = 0.0, GGVDW = 0.0;
  double HHReal = 0.0, HGReal = 0.0, GGReal = 0.0;
  double HHEwaldE = 0.0, HGEwaldE = 0.0, GGEwaldE = 0.0;
  double TailE = 0.0;
  double total() const {
    return HHVDW + HGVDW + GGVDW + HHReal + HGReal + GGReal + HHEwaldE + HGEwaldE + GGEwaldE + TailE;
  }
  void zero() { *this = MoveEnergy(); }
  void take_negative();
  MoveEnergy& operator+=(const MoveEnergy& o);
  MoveEnergy& operator-=(const MoveEnergy& o);
};
MoveEnergy operator+(MoveEnergy a, const MoveEnergy& b);

// Atoms of one component (or a trial buffer). Pointers refer to the owning
// vectors of HostAtoms; Type / MolID are size_t as in the reference.
struct Atoms {
  double3* pos = nullptr;
  double* scale = nullptr;
  double* charge = nullptr;
  double* scaleCoul = nullptr;
  size_t* Type = nullptr;
  size_t* MolID = nullptr;
  size_t Molsize = 0;
  size_t size = 0;
  size_t Allocate_size = 0;
};

struct HostAtoms {  // owner of one Atoms' arrays
  std::vector<double3> pos;
  std::vector<double> scale, charge, scaleCoul;
  std::vector<size_t> Type, MolID;
  void allocate(size_t n);
  Atoms view(size_t molsize, size_t size);
};

struct ForceField {
  std::vector<double> epsilon, sigma, z, shift, C10;  // size*size, internal units
  std::vector<int> tail;      // size*size: 1 where the pair has the LJ tail correction
  bool noCharges = false;
  bool VDWRealBias = true;
  bool Use1264 = false;
  size_t size = 0;
  double OverlapCriteria = 1e6;
  double CutOffVDW = 144.0;   // squared
  double CutOffCoul = 144.0;  // squared
};

struct Boxsize {
  double Cell[9] = {};
  double InverseCell[9] = {};
  double Volume = 0.0;
  double ReciprocalCutOff = 0.0;
  double Prefactor = 138935.48350;
  double Alpha = 0.265;
  bool Cubic = true;
  bool UseLAMMPSEwald = true;
  double tol1 = 0.0;          // Ewald precision factor of the automatic set-up (0: explicit kmax)
  int3 kmax;
  grx_box* handle = nullptr;  // the device box: eik tables and S(k) live here
};

struct CBMC_Variables {
  int MoveType = CBMC_INSERTION;
  double Rosenbluth = 0.0;
  double StoredR = 0.0;
  size_t selectedTrial = 0;
  size_t selectedTrialOrientation = 0;
  size_t start_position = 0;
  bool SuccessConstruction = false;
  MoveEnergy FirstBeadEnergy;
  MoveEnergy ChainEnergy;
  void clear() { *this = CBMC_Variables(); }
};

struct Move_Statistics {
  double TranslationProb = 0.0, RotationProb = 0.0, ReinsertionProb = 0.0, SwapProb = 0.0;
  double IdentitySwapProb = 0.0;         // cumulative, between reinsertion and swap (0: none)
  size_t NumberOfTrials = 10;            // first-bead trials of the CBMC moves
  size_t TranslationTotal = 0, TranslationAccepted = 0;
  size_t RotationTotal = 0, RotationAccepted = 0;
  size_t InsertionTotal = 0, InsertionAccepted = 0;
  size_t DeletionTotal = 0, DeletionAccepted = 0;
  size_t ReinsertionTotal = 0, ReinsertionAccepted = 0;
  size_t IdentitySwapRemoveTotal = 0, IdentitySwapRemoveAccepted = 0;  // this component swapped out
  size_t IdentitySwapAddTotal = 0, IdentitySwapAddAccepted = 0;        // this component swapped in
  std::vector<size_t> IdentitySwap_Total_TO, IdentitySwap_Acc_TO;      // per target component
  double3 MaxTranslation{1.0, 1.0, 1.0};
  double3 MaxRotation{0.5, 0.5, 0.5};
  void Record_Move_Total(int move);
  void Record_Move_Accept(int move);
  // cumulative as NormalizeProbabilities leaves them (data_struct.h:569-610)
  void NormalizeProbabilities();
};

// Widom statistics of one component: RecordRosen / block averages
// (data_struct.h:627-652) and ComputeFugacity (print_statistics.cuh:100-110).
struct RosenbluthWeight {
  std::vector<double3> Blocks;  // per block {sum W, sum W^2, count}
};

struct TempVals {
  size_t component = 1;
  size_t molecule = 0;
  double2 Scale{1.0, 1.0};
};

struct Components {
  int3 NComponents;                                  // x: total, y: framework components
  double Temperature = 300.0;
  double Pressure = 0.0;                             // internal units
  double Beta = 0.0;
  std::vector<size_t> Moleculesize;
  std::vector<size_t> NumberOfMolecule_for_Component;
  std::vector<size_t> Allocate_size;
  std::vector<bool> rigid, hasPartialCharge;
  std::vector<double> ExclusionIntra, ExclusionAtom;
  std::vector<double> IdealRosenbluthWeight, FugacityCoeff, MolFraction;
  std::vector<double> Tc, Pc, Accentric;             // critical constants of the molecule .def files
  double FrameworkMass = 0.0;                        // g/mol of all framework atoms (loadings per kg)
  std::vector<double> TailCorrectionInsert;          // host-guest tail delta of one insertion
  std::vector<Move_Statistics> Moves;
  std::vector<RosenbluthWeight> Rosen_Widom;
  size_t Nblock = 5;
  // CBMC scratch (mc_widom.h)
  std::vector<size_t> Trialindex;
  std::vector<double> Rosen;
  std::vector<MoveEnergy> TrialEnergies;
  TempVals TempVal;
  std::vector<size_t> StoredAtoms;                   // atoms stored per component (templates included)
  double VolumeMoveMaxChange = 0.0;                  // MaxVolumeChange of ln V
  size_t VolumeMoveAttempts = 0, VolumeMoveAccepted = 0;
  double VolumeMoveLastV = 0.0;                      // the last volume trial (reporting):
  MoveEnergy VolumeMoveLastE;                        //   its volume, FP64 totals and overlap flag
  bool VolumeMoveLastOverlap = false;
  struct IdentitySwapRecord {                        // the last identity swap (reporting)
    size_t OldComponent = 0, NewComponent = 0, OldMolecule = 0;
    double RosenbluthNew = 0.0, RosenbluthOld = 0.0, Pacc = 0.0;  // 0 where the move stopped early
    double2 Ewald;                                                // {GGEwaldE, HGEwaldE} of the trial
    bool Accepted = false;
  } LastIdentitySwap;
  MoveEnergy deltaE;                                 // running sum of accepted move energies
  uint64_t Step = 0;                                 // Philox move index of the next move
};

struct Simulations {
  std::vector<HostAtoms> host;                       // storage behind d_a
  std::vector<Atoms> d_a;                            // host mirror of the device atoms
  HostAtoms OldStore, NewStore;
  Atoms Old, New;                                    // trial buffers (1024 slots)
  Boxsize Box;
  int ExcludeComponent = -1;
  int64_t ExcludeMolecule = -1;
};

struct WidomStruct {
  size_t NumberWidomTrials = 10;
  size_t NumberWidomTrialsOrientations = 10;
};

struct RandomNumber {
  uint64_t Seed = 42;
  uint32_t Stream = 0;
  // Box b of a multi-box system draws from stream Stream + b * 2^24, so boxes at the same
  // move index never share a random number (box 0 keeps Stream).
  uint32_t BoxStream(size_t systemId) const { return Stream + ((uint32_t)systemId << 24); }
};

struct Variables {
  ForceField device_FF;
  std::vector<Simulations> Sims;
  std::vector<Components> SystemComponents;
  std::vector<WidomStruct> Widom;
  RandomNumber Random;
  grx_precision Precision = GRX_FP64;
};

// ------------------------------------------------------------------ set-up
void check(grx_status st, const char* what);
// Creates the device box of Sims[systemId] from Box, device_FF and d_a; the
// component arrays must be filled (an empty adsorbate component stores its
// molecule template, as Atoms.Allocate_size storage does in the reference).
void Setup_Box(Variables& Vars, size_t systemId, const std::vector<size_t>& n_stored);
void Destroy_Box(Variables& Vars, size_t systemId);

// ------------------------------------------------------------------ energy calls
// mc_widom.h:89-119 with Host_sum_Widom_HGGG_SEPARATE (:42-87).
void CBMC_PairwiseInteractions(Variables& Vars, size_t systemId, Components& SystemComponents,
                               Simulations& Sims, size_t NTrials, size_t chainsize);
// mc_widom.h:14-39, the uniform taken from the Philox selection slot (word).
size_t SelectTrialPosition(std::vector<double>& LogBoltzmannFactors, const Variables& Vars, size_t systemId,
                           int word);
// Ewald_Energy_Functions.h:438-580: {same-type delta minus exclusion, 2 * cross}.
double2 GPU_EwaldDifference_General(Simulations& Sims, ForceField& FF, Components& SystemComponents,
                                    size_t SelectedComponent, int MoveType, size_t Location, double2 Scale);
// Ewald_Energy_Functions.h:423-433.
void Update_Vector_Ewald(Boxsize& Box, bool UseTempVector, Components& SystemComponents, size_t SelectedComponent);
// CB/CFC and identity-swap variants of the Fourier delta (Ewald_Energy_Functions.h:582-634,764-789):
// the molecule starting at start_position changes (scale, scaleCoul) from oldScale to newScale,
// or the molecule of OLDComponent at UpdateLocation becomes one of NEWComponent at NewPositions.
double2 GPU_EwaldDifference_LambdaChange(Simulations& Sims, ForceField& FF, Components& SystemComponents,
                                         size_t SelectedComponent, size_t start_position, double2 oldScale,
                                         double2 newScale, int MoveType);
double2 GPU_EwaldDifference_IdentitySwap(Simulations& Sims, ForceField& FF, Components& SystemComponents,
                                         size_t OLDComponent, size_t NEWComponent, size_t UpdateLocation,
                                         const std::vector<double3>& NewPositions);
// Volume moves (mc_box.h:197-430) on the FP64 totals: the cell and the adsorbate
// molecules (first bead scaled, the others kept at their minimum-image offsets) are scaled,
// the totals of the scaled box decide. VolumeMove is the NPT move of one box; NVTGibbsMove
// exchanges volume between boxes 0 and 1 at fixed total volume.
struct Gibbs {
  double MaxGibbsBoxChange = 0.1;
  double GibbsBoxStats[2] = {0.0, 0.0};  // volume exchanges: attempts, accepted
  double GibbsXferStats[2] = {0.0, 0.0};  // particle transfers: attempts, accepted
  struct TransferRecord {                  // the last particle transfer (reporting)
    size_t InsertionBox = 0, DeletedMolecule = 0;
    double RosenbluthInsertion = 0.0, RosenbluthDeletion = 0.0, Pacc = 0.0;
    bool Accepted = false;
  } LastTransfer;
};
void VolumeMove(Variables& Vars, size_t systemId);
void NVTGibbsMove(Variables& Vars, Gibbs& GibbsStatistics);
// GibbsParticleTransfer (mc_swap_moves.h:51-176): a CBMC insertion of `comp` into one box
// and a CBMC deletion from the other, accepted together. Returns true when accepted.
bool GibbsParticleTransfer(Variables& Vars, size_t comp, Gibbs& GibbsStatistics);
// IdentitySwapMove (mc_swap_moves.h:199-420): one adsorbate molecule replaced by a molecule
// of another (or the same) adsorbate component grown on its first bead.
MoveEnergy IdentitySwapMove(Variables& Vars, size_t systemId);

// Energy of a lambda change of one molecule (mc_cbcfc.h:20-124): pair part over every other
// atom at fixed positions, Fourier part and tail; SuccessConstruction is false on overlap.
MoveEnergy CBCF_LambdaChange(Variables& Vars, size_t systemId, size_t SelectedMolInComponent,
                             size_t SelectedComponent, double2 oldScale, double2 newScale, size_t& start_position,
                             int MoveType, bool& SuccessConstruction);
// VDW_Coulomb.cu:1580 + Ewald_Energy_Functions.h:1272 (FP64 drift-check totals).
MoveEnergy Total_Energy(Simulations& Sims);
// The single-image rounding of PBC (maths.cuh:427-450) applied to a displacement in place.
void Minimum_Image(const Boxsize& Box, double3& v);
// LJ tail correction energy of the box (internal units): over the type pairs with the tail
// on, 2 pi N_i N_j / V * 4 eps_ij (sigma_ij^12 / (9 rc^9) - sigma_ij^6 / (3 rc^3)), N_i the
// atoms of type i in the box (framework and adsorbates), rc the VDW cutoff.
double TailCorrectionEnergy(const Variables& Vars, size_t systemId);
// The change of that energy when one molecule of component comp is inserted at the
// current counts (the TailCorrectionDifference of an insertion).
double TailCorrectionInsertion(const Variables& Vars, size_t systemId, size_t comp);
// GetPrefactor (mc_utilities.h:315-351).
double GetPrefactor(Components& SystemComponents, Simulations& Sims, size_t comp, int MoveType);

// ------------------------------------------------------------------ CBMC steps
void Widom_Move_FirstBead_PARTIAL(Variables& Vars, size_t systemId, CBMC_Variables& CBMC);
void Widom_Move_Chain_PARTIAL(Variables& Vars, size_t systemId, CBMC_Variables& CBMC);
void CBMC_FirstBead_Finish(Variables& Vars, size_t systemId, CBMC_Variables& CBMC);

// ------------------------------------------------------------------ moves
// Translation / rotation of TempVal.molecule (SingleBody_Prepare + Calculation +
// Acceptance, mc_single_particle.h:12-293); RANDOM is the acceptance uniform.
MoveEnergy SingleBodyMove(Variables& Vars, size_t systemId, int MoveType, double RANDOM);

struct InsertionMove {
  MoveEnergy energy;
  double preFactor = 0.0, Pacc = 0.0;
  bool Accept = false;
  CBMC_Variables InsertionVariables;
  void Initialize();
  void Calculate(Variables& Vars, size_t systemId);
  void Acceptance(Variables& Vars, size_t systemId, double RANDOM);
  void Commit(Variables& Vars, size_t systemId);   // store the grown molecule, commit S(k)
  MoveEnergy Run(Variables& Vars, size_t systemId, double RANDOM);
  double WidomMove(Variables& Vars, size_t systemId);
};

struct DeletionMove {
  MoveEnergy energy;
  double preFactor = 0.0, Pacc = 0.0;
  bool Accept = false;
  CBMC_Variables DeletionVariables;
  void Initialize();
  void Calculate(Variables& Vars, size_t systemId);
  void Acceptance(Variables& Vars, size_t systemId, double RANDOM);
  void Commit(Variables& Vars, size_t systemId);   // remove the molecule, commit S(k)
  MoveEnergy Run(Variables& Vars, size_t systemId, double RANDOM);
};

struct ReinsertionMove {
  MoveEnergy energy, old_energy;
  double Pacc = 0.0;
  bool Accept = false;
  CBMC_Variables InsertionVariables, DeletionVariables;
  std::vector<double3> NewPositions;  // tempMolStorage
  void Initialize();
  void Calculate_Insertion(Variables& Vars, size_t systemId);
  void Calculate_Deletion(Variables& Vars, size_t systemId);
  void Calculate_AdjustRosenbluth(Variables& Vars, size_t systemId);
  void Acceptance(Variables& Vars, size_t systemId, double RANDOM);
  MoveEnergy Run(Variables& Vars, size_t systemId, double RANDOM);
};

// One Monte Carlo step of RunMoves (axpy.cu:102-298) for component comp: the
// move is picked from the cumulative probabilities with the Philox move slot.
MoveEnergy RunMoves(Variables& Vars, size_t systemId, size_t comp);

// Widom insertions of the reference's WidomMove (move_struct.h:90-95) driven
// from the host, and the statistics of ComputeFugacity.
void RecordRosen(Components& SystemComponents, size_t comp, size_t block, double W);
double WidomChemicalPotential(const Components& SystemComponents, size_t comp);   // mu_ex in K
double WidomAverageRosenbluth(const Components& SystemComponents, size_t comp);
// FrameworkDensity (print_statistics.cuh:75-98): framework mass over the box volume, kg/m^3.
double FrameworkDensity(const Components& SystemComponents, const Boxsize& Box);
// The Henry coefficient of ComputeFugacity (print_statistics.cuh:99-109) for a rigid
// molecule: <W> / (R T rho_framework), mol/kg/Pa.
double WidomHenryCoefficient(const Components& SystemComponents, const Boxsize& Box, double AverageW);

// The same moves fully on the device: nsteps steps of grx_gcmc_run for one box.
grx_gcmc_stats RunMoves_Device(Variables& Vars, size_t systemId, size_t comp, int64_t nsteps);

// The device move set of every adsorbate component with a move probability, in component
// order (the entries RunMoves_Device_All runs); `moved` receives the components.
std::vector<grx_gcmc_desc> Device_Move_Descs(Variables& Vars, size_t systemId, std::vector<size_t>* moved);

// Every adsorbate component with a move probability, picked uniformly per step
// (Select_Box_Component_Molecule, axpy.cu:74-100): nsteps steps of grx_gcmc_run, one
// statistics entry per moved component (in `moved`).
std::vector<grx_gcmc_stats> RunMoves_Device_All(Variables& Vars, size_t systemId, int64_t nsteps,
                                                std::vector<size_t>* moved = nullptr);

// Copies the device atoms of adsorbate component comp back into the host mirror.
void Sync_Host_Mirror(Variables& Vars, size_t systemId, size_t comp);

}  // namespace graspa
