// grx_gcmc_cluster.cu -- cluster launches of the persistent GCMC kernel: one thread-block
// cluster of CL CTAs (24 warps each, CL = 2, 4 or 8) per box, so one Markov chain spans CL
// SMs. Used when a batch has fewer boxes than SMs (a few large boxes, a single serving job);
// the kernel itself is in grx_gcmc_kernel.cuh. Kept in its own translation unit so the
// cluster instantiations compile in parallel with the plain ones.
#include "grx_gcmc_kernel.cuh"
#include "grx_host.h"

namespace grx {

template <int PREC, int CL>
static cudaError_t launch_cl(int nboxes, const BoxDev* dboxes, const GcmcArgs* dargs, const int* dfirst,
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
  return cudaLaunchKernelEx(&cfg, gcmc_kernel<PREC, 24, CL>, dboxes, dargs, dfirst, dstep, nsteps, dstats);
}

template <int CL>
static cudaError_t launch_prec(grx_precision prec, int nboxes, const BoxDev* dboxes, const GcmcArgs* dargs,
                               const int* dfirst, const uint64_t* dstep, int64_t nsteps, grx_gcmc_stats* dstats,
                               size_t smem, cudaStream_t stream) {
  if (prec == GRX_FP64)
    return launch_cl<GRX_FP64, CL>(nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
  if (prec == GRX_MIXED)
    return launch_cl<GRX_MIXED, CL>(nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
  return launch_cl<GRX_FP32, CL>(nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
}

cudaError_t launch_gcmc_cluster(grx_precision prec, int cl, int nboxes, const BoxDev* dboxes, const GcmcArgs* dargs,
                                const int* dfirst, const uint64_t* dstep, int64_t nsteps, grx_gcmc_stats* dstats,
                                size_t smem, cudaStream_t stream) {
  if (cl == 2) return launch_prec<2>(prec, nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
  if (cl == 4) return launch_prec<4>(prec, nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
  if (cl == 8) return launch_prec<8>(prec, nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
  return cudaErrorInvalidValue;
}

template <int PREC, int CL>
static cudaError_t attr_one(size_t dyn_smem) {
  return cudaFuncSetAttribute(gcmc_kernel<PREC, 24, CL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_smem);
}

cudaError_t set_gcmc_cluster_smem(size_t dyn_smem) {
  for (cudaError_t e : {attr_one<GRX_FP64, 2>(dyn_smem), attr_one<GRX_FP64, 4>(dyn_smem),
                        attr_one<GRX_FP64, 8>(dyn_smem), attr_one<GRX_MIXED, 2>(dyn_smem),
                        attr_one<GRX_MIXED, 4>(dyn_smem), attr_one<GRX_MIXED, 8>(dyn_smem),
                        attr_one<GRX_FP32, 2>(dyn_smem), attr_one<GRX_FP32, 4>(dyn_smem),
                        attr_one<GRX_FP32, 8>(dyn_smem)})
    if (e != cudaSuccess) return e;
  return cudaSuccess;
}

template <int PREC, int CL>
static int active_one(size_t smem) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CL);
  cfg.blockDim = dim3(24 * 32);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CL;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, gcmc_kernel<PREC, 24, CL>, &cfg) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return n;
}

template <int CL>
static int active_prec(grx_precision prec, size_t smem) {
  if (prec == GRX_FP64) return active_one<GRX_FP64, CL>(smem);
  if (prec == GRX_MIXED) return active_one<GRX_MIXED, CL>(smem);
  return active_one<GRX_FP32, CL>(smem);
}

int gcmc_cluster_capacity(grx_precision prec, int cl, size_t smem) {
  if (cl == 2) return active_prec<2>(prec, smem);
  if (cl == 4) return active_prec<4>(prec, smem);
  if (cl == 8) return active_prec<8>(prec, smem);
  return 0;
}

}  // namespace grx
