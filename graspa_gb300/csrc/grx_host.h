// grx_host.h -- host-side box object shared by the libgrx translation units.
#pragma once

#include <vector>
#include <string>

#include "grx_internal.cuh"

struct grx_box {
  grx::BoxDev dev{};
  grx_arena* arena = nullptr;  // device memory comes from here when set (else cudaMalloc)
  grx_box* parent = nullptr;   // a replica shares its parent's framework atoms, tiles and tables
  int replicas = 0;            // live replicas of this box
  cudaStream_t stream = nullptr;
  int device = 0;
  int num_sms = 0;

  // layout
  int ncomp = 0, nhost = 0;
  size_t cap[GRX_MAX_COMPONENTS] = {};
  size_t molsize[GRX_MAX_COMPONENTS] = {};
  size_t off[GRX_MAX_COMPONENTS + 1] = {};
  int size[GRX_MAX_COMPONENTS] = {};
  int rigid[GRX_MAX_COMPONENTS] = {};
  int has_charge[GRX_MAX_COMPONENTS] = {};
  size_t stored[GRX_MAX_COMPONENTS] = {};  // atoms written to storage (template included)
  double excl_intra[GRX_MAX_COMPONENTS] = {};
  double excl_self[GRX_MAX_COMPONENTS] = {};
  size_t total_cap = 0;

  // host mirrors (FP64) of the component data, for exclusion constants
  std::vector<double> h_pos, h_charge, h_scale_coul;

  // device allocations
  double4* pos64 = nullptr;
  float4* hi = nullptr;
  float4* lo = nullptr;
  int2* meta = nullptr;
  double* scale = nullptr;
  double* charge = nullptr;
  int* d_size = nullptr;
  grx::FFPair64* ff64 = nullptr;
  double* ffc10 = nullptr;
  float4* ff32 = nullptr;
  int4* kact = nullptr;
  double* ktemp = nullptr;
  double2* s_fw = nullptr;
  double2* s_ads = nullptr;
  double2* s_tmp = nullptr;
  int nvec = 0, nact = 0;
  std::vector<int4> h_kact;
  std::vector<double> h_ktemp;
  bool sk_valid = false;

  // spatial tiles of host atoms and the storage permutation of host components
  std::vector<float4> h_tile_c;
  std::vector<int4> h_tile_r;
  float4* tile_c = nullptr;
  int4* tile_r = nullptr;
  size_t tile_cap = 0;
  int ntiles = 0;
  std::vector<int> perm[GRX_MAX_COMPONENTS];  // storage slot -> caller index
  // candidate lists of host atoms per voxel (grx_voxel.cu); a replica uses its parent's
  int vox_mode = 1;          // 1: build them when they fit, 0: tile path only
  size_t vox_max_bytes = 32u << 20;  // byte cap of the lists (coarser voxels to stay below it)
  int vox_on = 0;
  int vn[3] = {0, 0, 0};
  int vchunks = 0;
  size_t vox_entries = 0;
  int4* vmeta = nullptr;
  uint32_t* vlist = nullptr;
  // double-float copies for the mixed-precision pair path
  float2* qdf = nullptr;     // q * scaleCoul per atom as hi/lo floats
  // host (framework) atoms [0, off[nhost]) as the pair engine reads them: two float4 per atom,
  // {x_hi, y_hi, z_hi, q_hi} {x_lo, y_lo, z_lo, q_lo}, and the type with bit 15 set when the
  // atom's scale is not 1 (replicas use the parent's)
  float4* hrec = nullptr;
  uint16_t* htype = nullptr;
  float4* ffdf = nullptr;    // per type pair {4eps hi, lo, 1/sigma^2 hi, lo}
  float2* ffdf2 = nullptr;   // per type pair {shift hi, lo}
  float4* ctabf = nullptr;   // Coulomb table, 4 float4 per piece
  float4* ewA = nullptr;     // per active k: temp * S_ads as double-float complex
  float4* ewF = nullptr;     // per active k: temp * S_fw
  float2* ewT = nullptr;     // per active k: temp
  bool ewdf_valid = false;
  // Coulomb table
  double* ctab = nullptr;
  int ctab_n = 0, ctab_base = 0;
  double ctab_maxrel = 0.0;

  // scratch (grown on demand)
  double* scratch = nullptr;
  size_t scratch_bytes = 0;
  void* pinned = nullptr;
  size_t pinned_bytes = 0;
  grx_widom_result* d_results = nullptr;
  size_t results_cap = 0;
};

namespace grx {
grx_status ensure_scratch(grx_box* b, size_t bytes);
grx_status ensure_pinned(grx_box* b, size_t bytes);
grx_status ensure_results(grx_box* b, size_t n);
void refresh_dev(grx_box* b);
int sm_count(grx_box* b);
void* arena_alloc(grx_arena* a, size_t bytes);
void arena_free(grx_arena* a, void* p);
// Device allocation of a box: from its arena when it has one, else cudaMalloc.
cudaError_t dev_alloc(grx_box* b, void** p, size_t bytes);
// Builds the double-float S(k) tables of a box on its stream (framework tables skipped
// for replicas) and marks them valid.
grx_status ewald_df_refresh(grx_box* b);
void dev_free(grx_box* b, void* p);
// Voxel candidate lists of the machine's host atoms (grx_voxel.cu), rebuilt after the tiles.
grx_status build_voxels(grx_box* b);
}  // namespace grx

#define GRX_CHECK_CUDA(call, what)                                    \
  do {                                                                \
    cudaError_t e_ = (call);                                          \
    if (e_ != cudaSuccess) return grx::cuda_status(e_, what);         \
  } while (0)

#define GRX_REQUIRE(cond, msg)                                        \
  do {                                                                \
    if (!(cond)) {                                                    \
      grx::set_error("%s", msg);                                      \
      return GRX_ERR_INVALID_ARG;                                     \
    }                                                                 \
  } while (0)
