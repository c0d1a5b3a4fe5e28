// grx_gcmc_swap.cu -- launches of the persistent GCMC kernel with identity swaps (move sets
// whose p_identity_swap opens a range above p_reinsertion): one block of 8, 12 or 24 warps per
// box, or one thread-block cluster of 2, 4 or 8 CTAs of 24 warps. A separate instantiation
// (IDS = true) keeps the identity-swap step out of the kernels of every other batch; its own
// translation unit compiles in parallel with the others.
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

template <int PREC, int CL>
static cudaError_t launch_ids_cl(int nboxes, const BoxDev* dboxes, const GcmcArgs* dargs, const int* dfirst,
                                 const uint64_t* dstep, int64_t nsteps, grx_gcmc_stats* dstats, size_t smem,
                                 cudaStream_t stream) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(nboxes * CL));
  cfg.blockDim = dim3(24 * 32);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CL;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, gcmc_kernel<PREC, 24, CL, true>, dboxes, dargs, dfirst, dstep, nsteps, dstats);
}

template <int CL>
static cudaError_t launch_prec_cl(grx_precision prec, int nboxes, const BoxDev* dboxes, const GcmcArgs* dargs,
                                  const int* dfirst, const uint64_t* dstep, int64_t nsteps, grx_gcmc_stats* dstats,
                                  size_t smem, cudaStream_t stream) {
  if (prec == GRX_FP64)
    return launch_ids_cl<GRX_FP64, CL>(nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
  if (prec == GRX_MIXED)
    return launch_ids_cl<GRX_MIXED, CL>(nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
  return launch_ids_cl<GRX_FP32, CL>(nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
}

cudaError_t launch_gcmc_swap_cluster(grx_precision prec, int cl, int nboxes, const BoxDev* dboxes,
                                     const GcmcArgs* dargs, const int* dfirst, const uint64_t* dstep, int64_t nsteps,
                                     grx_gcmc_stats* dstats, size_t smem, cudaStream_t stream) {
  if (cl == 2) return launch_prec_cl<2>(prec, nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
  if (cl == 4) return launch_prec_cl<4>(prec, nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
  if (cl == 8) return launch_prec_cl<8>(prec, nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
  return cudaErrorInvalidValue;
}

template <int PREC, int NW, int CL = 1>
static cudaError_t attr_one(size_t dyn_smem) {
  return cudaFuncSetAttribute(gcmc_kernel<PREC, NW, CL, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)dyn_smem);
}

cudaError_t set_gcmc_swap_smem(size_t dyn_smem) {
  for (cudaError_t e : {attr_one<GRX_FP64, 8>(dyn_smem), attr_one<GRX_FP64, 12>(dyn_smem),
                        attr_one<GRX_FP64, 24>(dyn_smem), attr_one<GRX_MIXED, 8>(dyn_smem),
                        attr_one<GRX_MIXED, 12>(dyn_smem), attr_one<GRX_MIXED, 24>(dyn_smem),
                        attr_one<GRX_FP32, 8>(dyn_smem), attr_one<GRX_FP32, 12>(dyn_smem),
                        attr_one<GRX_FP32, 24>(dyn_smem), attr_one<GRX_FP64, 24, 2>(dyn_smem),
                        attr_one<GRX_FP64, 24, 4>(dyn_smem), attr_one<GRX_FP64, 24, 8>(dyn_smem),
                        attr_one<GRX_MIXED, 24, 2>(dyn_smem), attr_one<GRX_MIXED, 24, 4>(dyn_smem),
                        attr_one<GRX_MIXED, 24, 8>(dyn_smem), attr_one<GRX_FP32, 24, 2>(dyn_smem),
                        attr_one<GRX_FP32, 24, 4>(dyn_smem), attr_one<GRX_FP32, 24, 8>(dyn_smem)})
    if (e != cudaSuccess) return e;
  return cudaSuccess;
}

}  // namespace grx
