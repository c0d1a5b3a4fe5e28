// grx_host.h -- host-side box object shared by the libgrx translation units.
#pragma once

#include <vector>
#include <string>

#include "grx_internal.cuh"

struct grx_box {
  grx::BoxDev dev{};
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
