// grx_gcmc_swap.cu -- launches of the persistent GCMC kernel with identity swaps (move sets
// whose p_identity_swap opens a range above p_reinsertion): one block of 8, 12 or 24 warps per
// box. A separate instantiation (IDS = true) keeps the identity-swap step out of the kernels
// of every other batch; its own translation unit compiles in parallel with the others.
#include "grx_gcmc_kernel.cuh"
#include "grx_host.h"

namespace grx {

template <int PREC, int NW>
static cudaError_t launch_ids(int nboxes, const BoxDev* dboxes, const GcmcArgs* dargs, const int* dfirst,
                              const uint64_t* dstep, int64_t nsteps, grx_gcmc_stats* dstats, size_t smem,
                              cudaStream_t stream) {
  gcmc_kernel<PREC, NW, 1, true><<<nboxes, NW * 32, smem, stream>>>(dboxes, dargs, dfirst, dstep, nsteps, dstats);
  return cudaGetLastError();
}

template <int NW>
static cudaError_t launch_prec(grx_precision prec, int nboxes, const BoxDev* dboxes, const GcmcArgs* dargs,
                               const int* dfirst, const uint64_t* dstep, int64_t nsteps, grx_gcmc_stats* dstats,
                               size_t smem, cudaStream_t stream) {
  if (prec == GRX_FP64)
    return launch_ids<GRX_FP64, NW>(nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
  if (prec == GRX_MIXED)
    return launch_ids<GRX_MIXED, NW>(nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
  return launch_ids<GRX_FP32, NW>(nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
}

cudaError_t launch_gcmc_swap(grx_precision prec, int nw, int nboxes, const BoxDev* dboxes, const GcmcArgs* dargs,
                             const int* dfirst, const uint64_t* dstep, int64_t nsteps, grx_gcmc_stats* dstats,
                             size_t smem, cudaStream_t stream) {
  if (nw == 24) return launch_prec<24>(prec, nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
  if (nw == 12) return launch_prec<12>(prec, nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
  return launch_prec<8>(prec, nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
}

template <int PREC, int NW>
static cudaError_t attr_one(size_t dyn_smem) {
  return cudaFuncSetAttribute(gcmc_kernel<PREC, NW, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)dyn_smem);
}

cudaError_t set_gcmc_swap_smem(size_t dyn_smem) {
  for (cudaError_t e : {attr_one<GRX_FP64, 8>(dyn_smem), attr_one<GRX_FP64, 12>(dyn_smem),
                        attr_one<GRX_FP64, 24>(dyn_smem), attr_one<GRX_MIXED, 8>(dyn_smem),
                        attr_one<GRX_MIXED, 12>(dyn_smem), attr_one<GRX_MIXED, 24>(dyn_smem),
                        attr_one<GRX_FP32, 8>(dyn_smem), attr_one<GRX_FP32, 12>(dyn_smem),
                        attr_one<GRX_FP32, 24>(dyn_smem)})
    if (e != cudaSuccess) return e;
  return cudaSuccess;
}

}  // namespace grx
