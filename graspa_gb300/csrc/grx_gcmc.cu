// grx_gcmc.cu -- GCMC moves fully on the device: preparation of the boxes and move sets,
// persistent launches of the kernel in grx_gcmc_kernel.cuh (one block per box, or one
// thread-block cluster per box through grx_gcmc_cluster.cu), batches replayed as CUDA
// graphs, the launch-shape autotuner, and the single-molecule updates of the host layer.
#include <algorithm>
#include <cmath>
#include <vector>

#include "grx_gcmc_kernel.cuh"
#include "grx_host.h"

namespace grx {

__global__ void advance_step_kernel(uint64_t* step, int64_t nsteps) { *step += (uint64_t)nsteps; }

__global__ void ewald_df_refresh_gcmc(BoxDev b) {
  float4* ewA = const_cast<float4*>(b.ewA);
  float4* ewF = const_cast<float4*>(b.ewF);
  float2* ewT = const_cast<float2*>(b.ewT);
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < b.nact; j += gridDim.x * blockDim.x) {
    const int slot = b.kact[j].w;
    const double t = b.ktemp[j];
    const double2 sa = b.s_ads[slot], sf = b.s_fw[slot];
    const df ar = df_from(t * sa.x), ai = df_from(t * sa.y), fr = df_from(t * sf.x), fi = df_from(t * sf.y);
    ewA[j] = make_float4(ar.hi, ar.lo, ai.hi, ai.lo);
    if (b.shared_host) continue;  // a replica's framework tables are its parent's
    ewF[j] = make_float4(fr.hi, fr.lo, fi.hi, fi.lo);
    const df tt = df_from(t);
    ewT[j] = make_float2(tt.hi, tt.lo);
  }
}

grx_status ewald_df_refresh(grx_box* b) {
  refresh_dev(b);
  ewald_df_refresh_gcmc<<<std::max(1, std::min((b->nact + 255) / 256, sm_count(b))), 256, 0, b->stream>>>(b->dev);
  count_launch();
  GRX_CHECK_CUDA(cudaGetLastError(), "ewald table refresh");
  b->ewdf_valid = true;
  return GRX_OK;
}

}  // namespace grx

using namespace grx;

// A prepared persistent GCMC launch over a set of boxes (see grx.h). The per-box
// state descriptors, the move sets, the step counter and the running statistics
// live in one device allocation owned by the batch.
struct grx_gcmc_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  grx_precision prec = GRX_MIXED;
  std::vector<grx_box*> boxes;
  std::vector<grx_gcmc_desc> descs;
  std::vector<int> first;
  int nentries = 0;
  size_t smem = 0;
  int chunk_mult = 1;
  int nwarps = 8;  // warps per box (block size / 32): 8, 12 or 24
  int cluster = 1; // CTAs per box (1, or 2 / 4 / 8 with 24 warps each)
  bool swaps = false;  // a move set with identity swaps: the IDS kernel
  void* mem = nullptr;
  grx_arena* arena = nullptr;
  BoxDev* d_boxes = nullptr;
  GcmcArgs* d_args = nullptr;
  int* d_first = nullptr;
  grx_gcmc_stats* d_stats = nullptr;
  uint64_t* d_step = nullptr;
  int* d_sizes = nullptr;  // molecule counts gathered after a launch
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t graph_nsteps = 0;
  int graph_nlaunch = 0;
  cudaStream_t graph_stream = nullptr;
  cudaStream_t last_stream = nullptr;  // stream of the latest launch
  std::vector<GcmcArgs> h_args;        // host copy of the move sets (per-box step windows)
};

namespace grx {

// Dynamic shared memory of a GCMC block: eik tables of a move plus, when enabled, the
// (kx, ky) row products (at most kEwRowBytes); with the largest static workspace (24 warps)
// it stays within the 227 KB of one block.
constexpr size_t kGcmcDynSmem = 160 * 1024;

// A move set with identity swaps (a range of p_identity_swap above p_reinsertion).
static bool has_swaps(const grx_gcmc_desc* descs, int n) {
  for (int e = 0; e < n; ++e)
    if (descs[e].p_identity_swap > descs[e].p_reinsertion) return true;
  return false;
}

// Validates the boxes and move sets and fills the per-box state and per-entry args.
static grx_status prepare_gcmc(grx_box* const* boxes, int32_t nboxes, const grx_gcmc_desc* descs,
                               const int32_t* ncomp_moved, std::vector<BoxDev>& hb, std::vector<GcmcArgs>& ha,
                               std::vector<int>& first, size_t& smem, int chunk_mult, grx_precision prec) {
  GRX_REQUIRE(boxes && descs && nboxes >= 1, "grx_gcmc: bad argument");
  hb.assign(nboxes, BoxDev{});
  ha.clear();
  first.assign(nboxes + 1, 0);
  smem = 0;
  int e = 0;
  for (int i = 0; i < nboxes; ++i) {
    grx_box* b = boxes[i];
    GRX_REQUIRE(b, "grx_gcmc: null box");
    GRX_REQUIRE(b->device == boxes[0]->device, "grx_gcmc: boxes live on different devices");
    for (int j = 0; j < i; ++j) GRX_REQUIRE(boxes[j] != b, "grx_gcmc: a box appears twice");
    const int nm = ncomp_moved ? ncomp_moved[i] : 1;
    GRX_REQUIRE(nm >= 1 && nm <= kMaxMoved, "grx_gcmc: 1..4 moved components per box");
    first[i] = e;
    refresh_dev(b);
    b->dev.chunk_mult = chunk_mult;
    int msmax = 1;
    for (int k = 0; k < nm; ++k) msmax = std::max(msmax, (int)b->molsize[descs[e + k].component]);
    // row products of the Ewald delta for every move of the box, sized for its largest molecule
    b->dev.ew_rows = ew_rows_worth(b->dev.kmax, b->nact, msmax) ? 1 : 0;
    for (int k = 0; k < nm; ++k, ++e) {
      const grx_gcmc_desc& d = descs[e];
      GRX_REQUIRE(d.component >= b->nhost && d.component < b->ncomp,
                  "grx_gcmc: component must be an adsorbate component");
      for (int j = first[i]; j < e; ++j)
        GRX_REQUIRE(descs[j].component != d.component, "grx_gcmc: a component is listed twice for one box");
      GRX_REQUIRE(d.seed == descs[first[i]].seed && d.stream == descs[first[i]].stream,
                  "grx_gcmc: the entries of one box must share seed and stream");
      const int ms = (int)b->molsize[d.component];
      GRX_REQUIRE(ms >= 1 && ms <= kMolWork, "grx_gcmc: molecule size must be 1..32");
      GRX_REQUIRE(b->stored[d.component] >= (size_t)ms,
                  "grx_gcmc: the component stores no molecule template (set it with n_stored >= molsize)");
      GRX_REQUIRE(d.ntrials >= 1 && d.ntrials <= kMaxTrials, "grx_gcmc: ntrials out of range (1..64)");
      GRX_REQUIRE(ms == 1 || (d.norient >= 1 && d.norient <= kMaxTrials && d.norient * (ms - 1) <= kCbmcBeads),
                  "grx_gcmc: norient * (molecule size - 1) must be <= 128");
      GRX_REQUIRE(2 * ms <= kCbmcBeads, "grx_gcmc: molecule too large");
      GRX_REQUIRE(d.beta > 0 && d.pressure > 0 && d.ideal_rosenbluth > 0, "grx_gcmc: bad thermodynamic state");
      GRX_REQUIRE(d.p_identity_swap == 0.0 || (d.p_identity_swap >= d.p_reinsertion && d.p_identity_swap <= d.p_swap),
                  "grx_gcmc: p_identity_swap must lie between p_reinsertion and p_swap (cumulative)");
      GRX_REQUIRE(d.p_identity_swap <= d.p_reinsertion || d.tail_insert == 0.0,
                  "grx_gcmc: identity swaps with tail corrections are not supported");
      GcmcArgs a{};
      a.d = d;
      a.comp = d.component;
      a.ms = ms;
      a.off = (int)b->off[d.component];
      a.cap = (int)b->cap[d.component];
      a.rigid = b->rigid[d.component];
      a.charged = (!b->dev.no_charges && b->has_charge[d.component] && b->nact > 0) ? 1 : 0;
      a.bias = b->dev.vdw_real_bias;
      a.excl = b->excl_intra[d.component] + b->excl_self[d.component];
      a.big_p = d.mol_fraction * d.pressure * d.fugacity_coeff * b->dev.volume;
      a.step_off = 0;
      a.nsteps_cap = -1;
      ha.push_back(a);
      // eik tables of the moved atoms: FP64 (double2) in the FP64 form, double-float (float4)
      // in the others
      size_t need = (size_t)(b->dev.kmax[0] + b->dev.kmax[1] + b->dev.kmax[2] + 3) * 2 * ms *
                    (prec == GRX_FP64 ? sizeof(double2) : sizeof(float4));
      if (b->dev.ew_rows) need += (size_t)ew_rows(b->dev.kmax) * 2 * msmax * sizeof(float4);
      smem = std::max(smem, need);
    }
    if (!b->ewdf_valid && b->nact > 0) {
      grx_status st = ewald_df_refresh(b);
      if (st) return st;
    }
    hb[i] = b->dev;
  }
  first[nboxes] = e;
  GRX_REQUIRE(smem <= kGcmcDynSmem, "grx_gcmc: Ewald tables exceed the shared-memory budget");
  return GRX_OK;
}

template <int PREC, int NW>
static grx_status set_smem_one() {
  GRX_CHECK_CUDA(cudaFuncSetAttribute(gcmc_kernel<PREC, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGcmcDynSmem),
                 "gcmc shared memory attribute");
  return GRX_OK;
}

static grx_status set_gcmc_smem() {
  static bool done[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64 && done[dev]) return GRX_OK;
  grx_status st = GRX_OK;
  for (grx_status r : {set_smem_one<GRX_FP64, 8>(), set_smem_one<GRX_FP64, 12>(), set_smem_one<GRX_FP64, 24>(),
                       set_smem_one<GRX_MIXED, 8>(), set_smem_one<GRX_MIXED, 12>(), set_smem_one<GRX_MIXED, 24>(),
                       set_smem_one<GRX_FP32, 8>(), set_smem_one<GRX_FP32, 12>(), set_smem_one<GRX_FP32, 24>()})
    if (r && !st) st = r;
  if (!st) GRX_CHECK_CUDA(set_gcmc_cluster_smem(kGcmcDynSmem), "gcmc cluster shared memory attribute");
  if (!st) GRX_CHECK_CUDA(set_gcmc_swap_smem(kGcmcDynSmem), "gcmc identity-swap shared memory attribute");
  if (!st && dev >= 0 && dev < 64) done[dev] = true;
  return st;
}

// Warps per box when no shape was chosen: fill the SMs with one wave of blocks.
static int default_warps(int nboxes) {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
      sms = 1;
  }
  if (nboxes <= sms) return 24;
  if (nboxes <= 2 * sms) return 12;
  return 8;
}

template <int NW>
static void launch_shape(grx_precision prec, int nboxes, const BoxDev* dboxes, const GcmcArgs* dargs,
                         const int* dfirst, uint64_t* dstep, int64_t nsteps, grx_gcmc_stats* dstats, size_t smem,
                         cudaStream_t stream) {
  if (prec == GRX_FP64)
    gcmc_kernel<GRX_FP64, NW><<<nboxes, NW * 32, smem, stream>>>(dboxes, dargs, dfirst, dstep, nsteps, dstats);
  else if (prec == GRX_MIXED)
    gcmc_kernel<GRX_MIXED, NW><<<nboxes, NW * 32, smem, stream>>>(dboxes, dargs, dfirst, dstep, nsteps, dstats);
  else
    gcmc_kernel<GRX_FP32, NW><<<nboxes, NW * 32, smem, stream>>>(dboxes, dargs, dfirst, dstep, nsteps, dstats);
}

// Enqueues one persistent launch of nw warps per box (a cluster of cl such blocks per box
// when cl > 1, nw = 24) and the step-counter advance (no host sync).
static grx_status enqueue_gcmc(grx_precision prec, int nw, int nboxes, const BoxDev* dboxes, const GcmcArgs* dargs,
                               const int* dfirst, uint64_t* dstep, int64_t nsteps, grx_gcmc_stats* dstats,
                               size_t smem, cudaStream_t stream, int cl = 1, bool swaps = false) {
  if (swaps && cl > 1) {
    GRX_REQUIRE(nw == 24, "grx_gcmc: cluster launches use 24 warps per block");
    GRX_CHECK_CUDA(launch_gcmc_swap_cluster(prec, cl, nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem,
                                            stream),
                   "gcmc identity-swap cluster launch");
  } else if (swaps) {
    GRX_CHECK_CUDA(launch_gcmc_swap(prec, nw, nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream),
                   "gcmc identity-swap launch");
  } else if (cl > 1) {
    GRX_REQUIRE(nw == 24, "grx_gcmc: cluster launches use 24 warps per block");
    GRX_CHECK_CUDA(launch_gcmc_cluster(prec, cl, nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream),
                   "gcmc cluster launch");
  } else if (nw == 24) {
    launch_shape<24>(prec, nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
  } else if (nw == 12) {
    launch_shape<12>(prec, nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
  } else {
    launch_shape<8>(prec, nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem, stream);
  }
  advance_step_kernel<<<1, 1, 0, stream>>>(dstep, nsteps);
  count_launch();
  count_launch();
  GRX_CHECK_CUDA(cudaGetLastError(), "gcmc launch");
  return GRX_OK;
}

// Molecule counts of every box of a launch, gathered into one buffer.
__global__ void gather_sizes_kernel(const BoxDev* boxes, int nboxes, int* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nboxes * GRX_MAX_COMPONENTS) return;
  const int i = t / GRX_MAX_COMPONENTS, c = t % GRX_MAX_COMPONENTS;
  out[t] = c < boxes[i].ncomp ? boxes[i].comp_size[c] : 0;
}

// Refreshes the host copies of the boxes' molecule counts after a launch on `stream`:
// one gather kernel and one copy (dout: nboxes * GRX_MAX_COMPONENTS ints on the device).
static grx_status sync_sizes(grx_box* const* boxes, int nboxes, const grx_gcmc_desc* descs, const int* first,
                             const BoxDev* dboxes, int* dout, cudaStream_t stream) {
  std::vector<int> h((size_t)nboxes * GRX_MAX_COMPONENTS);
  gather_sizes_kernel<<<(nboxes * GRX_MAX_COMPONENTS + 255) / 256, 256, 0, stream>>>(dboxes, nboxes, dout);
  count_launch();
  GRX_CHECK_CUDA(cudaGetLastError(), "gather sizes");
  GRX_CHECK_CUDA(cudaMemcpyAsync(h.data(), dout, h.size() * sizeof(int), cudaMemcpyDeviceToHost, stream),
                 "read sizes");
  GRX_CHECK_CUDA(cudaStreamSynchronize(stream), "read sizes");
  for (int i = 0; i < nboxes; ++i) {
    grx_box* b = boxes[i];
    for (int c = 0; c < GRX_MAX_COMPONENTS; ++c) b->size[c] = h[(size_t)i * GRX_MAX_COMPONENTS + c];
    for (int e = first[i]; e < first[i + 1]; ++e) {
      const int c = descs[e].component;
      b->stored[c] = std::max(b->stored[c], (size_t)b->size[c]);
    }
  }
  return GRX_OK;
}

}  // namespace grx

extern "C" grx_status grx_gcmc_run(grx_box* const* boxes, int32_t nboxes, const grx_gcmc_desc* descs,
                                   const int32_t* ncomp_moved, uint64_t first_step, int64_t nsteps,
                                   grx_precision prec, grx_gcmc_stats* stats) {
  GRX_REQUIRE(boxes && descs && stats && nboxes >= 1, "grx_gcmc_run: bad argument");
  GRX_REQUIRE(prec == GRX_FP64 || prec == GRX_MIXED || prec == GRX_FP32, "grx_gcmc_run: bad precision");
  GRX_REQUIRE(nsteps >= 0, "grx_gcmc_run: negative step count");
  std::vector<BoxDev> hb;
  std::vector<GcmcArgs> ha;
  std::vector<int> first;
  size_t smem = 0;
  grx_status st =
      prepare_gcmc(boxes, nboxes, descs, ncomp_moved, hb, ha, first, smem, boxes[0]->dev.chunk_mult, prec);
  if (st) return st;
  const int ne = first[nboxes];
  grx_box* b0 = boxes[0];
  auto al = [](size_t n) { return (n + 255) / 256 * 256; };
  const size_t ob = 0, oa = al(nboxes * sizeof(BoxDev)), of = oa + al(ne * sizeof(GcmcArgs)),
               os = of + al((nboxes + 1) * sizeof(int)), ot = os + al(ne * sizeof(grx_gcmc_stats)),
               oz = ot + 256;
  st = ensure_scratch(b0, oz + al((size_t)nboxes * GRX_MAX_COMPONENTS * sizeof(int)));
  if (st) return st;
  char* base = (char*)b0->scratch;
  int* dsizes = (int*)(base + oz);
  BoxDev* dboxes = (BoxDev*)(base + ob);
  GcmcArgs* dargs = (GcmcArgs*)(base + oa);
  int* dfirst = (int*)(base + of);
  grx_gcmc_stats* dstats = (grx_gcmc_stats*)(base + os);
  uint64_t* dstep = (uint64_t*)(base + ot);
  GRX_CHECK_CUDA(cudaMemcpyAsync(dboxes, hb.data(), nboxes * sizeof(BoxDev), cudaMemcpyHostToDevice, b0->stream),
                 "upload boxes");
  GRX_CHECK_CUDA(cudaMemcpyAsync(dargs, ha.data(), ne * sizeof(GcmcArgs), cudaMemcpyHostToDevice, b0->stream),
                 "upload gcmc args");
  GRX_CHECK_CUDA(cudaMemcpyAsync(dfirst, first.data(), (nboxes + 1) * sizeof(int), cudaMemcpyHostToDevice,
                                 b0->stream),
                 "upload entry offsets");
  GRX_CHECK_CUDA(cudaMemcpyAsync(dstep, &first_step, sizeof(uint64_t), cudaMemcpyHostToDevice, b0->stream),
                 "upload step");
  GRX_CHECK_CUDA(cudaMemsetAsync(dstats, 0, ne * sizeof(grx_gcmc_stats), b0->stream), "clear stats");
  if (nsteps > 0) {
    st = set_gcmc_smem();
    if (st) return st;
    st = enqueue_gcmc(prec, default_warps(nboxes), nboxes, dboxes, dargs, dfirst, dstep, nsteps, dstats, smem,
                      b0->stream, 1, has_swaps(descs, ne));
    if (st) return st;
  }
  GRX_CHECK_CUDA(cudaMemcpyAsync(stats, dstats, ne * sizeof(grx_gcmc_stats), cudaMemcpyDefault, b0->stream),
                 "read gcmc stats");
  st = sync_sizes(boxes, nboxes, descs, first.data(), dboxes, dsizes, b0->stream);
  if (st) return st;
  note_transfer(nboxes * sizeof(BoxDev) + ne * sizeof(GcmcArgs) + (nboxes + 1) * sizeof(int) + sizeof(uint64_t),
                ne * sizeof(grx_gcmc_stats) + (size_t)nboxes * GRX_MAX_COMPONENTS * sizeof(int));
  if (nsteps == 0)
    for (int i = 0; i < nboxes; ++i)
      for (int e = first[i]; e < first[i + 1]; ++e)
        stats[e].n_molecules = boxes[i]->size[descs[e].component] / (int)boxes[i]->molsize[descs[e].component];
  return GRX_OK;
}

extern "C" grx_status grx_gcmc_batch_create(grx_box* const* boxes, int32_t nboxes, const grx_gcmc_desc* descs,
                                            const int32_t* ncomp_moved, grx_precision prec,
                                            grx_gcmc_batch** out) {
  GRX_REQUIRE(out, "grx_gcmc_batch_create: null output");
  GRX_REQUIRE(prec == GRX_FP64 || prec == GRX_MIXED || prec == GRX_FP32, "grx_gcmc_batch_create: bad precision");
  *out = nullptr;
  auto* B = new grx_gcmc_batch();
  B->prec = prec;
  std::vector<BoxDev> hb;
  std::vector<GcmcArgs> ha;
  grx_status st = prepare_gcmc(boxes, nboxes, descs, ncomp_moved, hb, ha, B->first, B->smem, B->chunk_mult, prec);
  if (st) { delete B; return st; }
  B->nentries = B->first[nboxes];
  B->h_args = ha;
  B->nwarps = default_warps(nboxes);
  B->boxes.assign(boxes, boxes + nboxes);
  B->descs.assign(descs, descs + B->nentries);
  B->swaps = has_swaps(descs, B->nentries);
  B->device = boxes[0]->device;
  B->stream = boxes[0]->stream;
  auto al = [](size_t n) { return (n + 255) / 256 * 256; };
  const size_t oa = al(nboxes * sizeof(BoxDev)), of = oa + al(B->nentries * sizeof(GcmcArgs)),
               os = of + al((nboxes + 1) * sizeof(int)), ot = os + al(B->nentries * sizeof(grx_gcmc_stats)),
               oz = ot + 256, total = oz + al((size_t)nboxes * GRX_MAX_COMPONENTS * sizeof(int));
  B->arena = boxes[0]->arena;  // a batch of arena boxes lives in the same arena
  if (B->arena) B->mem = arena_alloc(B->arena, total);
  else if (cudaMalloc(&B->mem, total) != cudaSuccess) B->mem = nullptr;
  if (!B->mem) {
    cudaGetLastError();
    delete B;
    set_error("grx_gcmc_batch_create: out of device memory");
    return GRX_ERR_OUT_OF_MEMORY;
  }
  char* base = (char*)B->mem;
  B->d_boxes = (BoxDev*)base;
  B->d_args = (GcmcArgs*)(base + oa);
  B->d_first = (int*)(base + of);
  B->d_stats = (grx_gcmc_stats*)(base + os);
  B->d_step = (uint64_t*)(base + ot);
  B->d_sizes = (int*)(base + oz);
  const uint64_t zero = 0;
  cudaStream_t s0 = B->stream;
  bool ok =
      cudaMemcpyAsync(B->d_boxes, hb.data(), nboxes * sizeof(BoxDev), cudaMemcpyHostToDevice, s0) == cudaSuccess &&
      cudaMemcpyAsync(B->d_args, ha.data(), B->nentries * sizeof(GcmcArgs), cudaMemcpyHostToDevice, s0) ==
          cudaSuccess &&
      cudaMemcpyAsync(B->d_first, B->first.data(), (nboxes + 1) * sizeof(int), cudaMemcpyHostToDevice, s0) ==
          cudaSuccess &&
      cudaMemsetAsync(B->d_stats, 0, B->nentries * sizeof(grx_gcmc_stats), s0) == cudaSuccess &&
      cudaMemcpyAsync(B->d_step, &zero, sizeof(uint64_t), cudaMemcpyHostToDevice, s0) == cudaSuccess &&
      cudaStreamSynchronize(s0) == cudaSuccess;
  st = set_gcmc_smem();
  if (!ok || st) {
    if (B->arena) arena_free(B->arena, B->mem);
    else cudaFree(B->mem);
    delete B;
    set_error("grx_gcmc_batch_create: device set-up failed");
    return GRX_ERR_CUDA;
  }
  *out = B;
  return GRX_OK;
}

static void drop_graph(grx_gcmc_batch* B) {
  if (B->exec) cudaGraphExecDestroy(B->exec);
  if (B->graph) cudaGraphDestroy(B->graph);
  B->exec = nullptr;
  B->graph = nullptr;
}

extern "C" grx_status grx_gcmc_batch_destroy(grx_gcmc_batch* B) {
  if (!B) return GRX_OK;
  drop_graph(B);
  if (B->arena) arena_free(B->arena, B->mem);
  else if (B->mem) cudaFree(B->mem);
  delete B;
  return GRX_OK;
}

extern "C" grx_status grx_gcmc_batch_set_step(grx_gcmc_batch* B, uint64_t step) {
  GRX_REQUIRE(B, "grx_gcmc_batch_set_step: null batch");
  GRX_CHECK_CUDA(cudaMemcpyAsync(B->d_step, &step, sizeof(uint64_t), cudaMemcpyHostToDevice, B->stream),
                 "set step");
  GRX_CHECK_CUDA(cudaStreamSynchronize(B->stream), "set step");
  return GRX_OK;
}

extern "C" grx_status grx_gcmc_batch_set_box_steps(grx_gcmc_batch* B, const uint64_t* next_move,
                                                   const int64_t* nsteps) {
  GRX_REQUIRE(B && next_move, "grx_gcmc_batch_set_box_steps: bad argument");
  GRX_CHECK_CUDA(cudaStreamSynchronize(B->stream), "set box steps");
  if (B->last_stream) GRX_CHECK_CUDA(cudaStreamSynchronize(B->last_stream), "set box steps");
  uint64_t counter = 0;  // the launch counter the next launch starts from
  GRX_CHECK_CUDA(cudaMemcpy(&counter, B->d_step, sizeof(uint64_t), cudaMemcpyDeviceToHost), "read step counter");
  const int nb = (int)B->boxes.size();
  for (int i = 0; i < nb; ++i) {
    GRX_REQUIRE(!nsteps || nsteps[i] >= 0, "grx_gcmc_batch_set_box_steps: negative step count");
    for (int e = B->first[i]; e < B->first[i + 1]; ++e) {
      B->h_args[e].step_off = (int64_t)(next_move[i] - counter);  // modulo 2^64
      B->h_args[e].nsteps_cap = nsteps ? nsteps[i] : -1;
    }
  }
  GRX_CHECK_CUDA(cudaMemcpy(B->d_args, B->h_args.data(), B->nentries * sizeof(GcmcArgs), cudaMemcpyHostToDevice),
                 "upload box steps");
  drop_graph(B);
  return GRX_OK;
}

extern "C" grx_status grx_gcmc_batch_launch(grx_gcmc_batch* B, int64_t nsteps, void* stream) {
  GRX_REQUIRE(B && nsteps >= 0, "grx_gcmc_batch_launch: bad argument");
  cudaStream_t s = stream ? (cudaStream_t)stream : B->stream;
  if (nsteps == 0) return GRX_OK;
  B->last_stream = s;
  return enqueue_gcmc(B->prec, B->nwarps, (int)B->boxes.size(), B->d_boxes, B->d_args, B->d_first, B->d_step, nsteps,
                      B->d_stats, B->smem, s, B->cluster, B->swaps);
}

extern "C" grx_status grx_gcmc_batch_run_graph(grx_gcmc_batch* B, int64_t nsteps, int32_t nlaunch, void* stream) {
  GRX_REQUIRE(B && nsteps >= 1 && nlaunch >= 1, "grx_gcmc_batch_run_graph: bad argument");
  cudaStream_t s = stream ? (cudaStream_t)stream : B->stream;
  if (!B->exec || B->graph_nsteps != nsteps || B->graph_nlaunch != nlaunch) {
    drop_graph(B);
    cudaStream_t cap = nullptr;
    GRX_CHECK_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking), "capture stream");
    GRX_CHECK_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal), "begin capture");
    grx_status st = GRX_OK;
    const uint64_t before = grx_launch_count();
    for (int k = 0; k < nlaunch && st == GRX_OK; ++k)
      st = enqueue_gcmc(B->prec, B->nwarps, (int)B->boxes.size(), B->d_boxes, B->d_args, B->d_first, B->d_step, nsteps,
                        B->d_stats, B->smem, cap, B->cluster, B->swaps);
    count_launch(0 - (grx_launch_count() - before));  // capture records the kernels, it launches nothing
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (st) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    GRX_CHECK_CUDA(ec, "end capture");
    B->graph = g;
    GRX_CHECK_CUDA(cudaGraphInstantiate(&B->exec, g, 0), "instantiate graph");
    B->graph_nsteps = nsteps;
    B->graph_nlaunch = nlaunch;
  }
  GRX_CHECK_CUDA(cudaGraphLaunch(B->exec, s), "graph launch");
  count_launch(2 * (uint64_t)nlaunch);  // the graph's kernels: one GCMC launch + one step advance each
  B->last_stream = s;
  return GRX_OK;
}

extern "C" grx_status grx_gcmc_batch_stats(grx_gcmc_batch* B, grx_gcmc_stats* stats, uint64_t* next_step) {
  GRX_REQUIRE(B, "grx_gcmc_batch_stats: null batch");
  GRX_CHECK_CUDA(cudaStreamSynchronize(B->stream), "gcmc batch sync");
  if (B->last_stream && B->last_stream != B->stream)
    GRX_CHECK_CUDA(cudaStreamSynchronize(B->last_stream), "gcmc batch sync");
  if (stats)
    GRX_CHECK_CUDA(cudaMemcpy(stats, B->d_stats, B->nentries * sizeof(grx_gcmc_stats), cudaMemcpyDeviceToHost),
                   "read stats");
  if (next_step)
    GRX_CHECK_CUDA(cudaMemcpy(next_step, B->d_step, sizeof(uint64_t), cudaMemcpyDeviceToHost), "read step");
  return sync_sizes(B->boxes.data(), (int)B->boxes.size(), B->descs.data(), B->first.data(), B->d_boxes, B->d_sizes,
                    B->stream);
}

extern "C" grx_status grx_gcmc_batch_reset_stats(grx_gcmc_batch* B) {
  GRX_REQUIRE(B, "grx_gcmc_batch_reset_stats: null batch");
  GRX_CHECK_CUDA(cudaMemsetAsync(B->d_stats, 0, B->nentries * sizeof(grx_gcmc_stats), B->stream), "clear stats");
  GRX_CHECK_CUDA(cudaStreamSynchronize(B->stream), "clear stats");
  return GRX_OK;
}

static grx_status upload_mult(grx_gcmc_batch* B, int mult) {
  const int nb = (int)B->boxes.size();
  std::vector<BoxDev> hb(nb);
  for (int i = 0; i < nb; ++i) {
    B->boxes[i]->dev.chunk_mult = mult;
    hb[i] = B->boxes[i]->dev;
  }
  GRX_CHECK_CUDA(cudaMemcpy(B->d_boxes, hb.data(), nb * sizeof(BoxDev), cudaMemcpyHostToDevice), "shape upload");
  return GRX_OK;
}

extern "C" grx_status grx_gcmc_batch_set_shape(grx_gcmc_batch* B, int32_t nwarps, int32_t chunk_mult) {
  GRX_REQUIRE(B, "grx_gcmc_batch_set_shape: null batch");
  GRX_REQUIRE(nwarps == 8 || nwarps == 12 || nwarps == 24, "grx_gcmc_batch_set_shape: nwarps must be 8, 12 or 24");
  GRX_REQUIRE(chunk_mult >= 1 && chunk_mult <= kCbmcMaxMult, "grx_gcmc_batch_set_shape: chunk_mult must be 1..8");
  GRX_CHECK_CUDA(cudaStreamSynchronize(B->stream), "set shape");
  grx_status st = upload_mult(B, chunk_mult);
  if (st) return st;
  B->nwarps = nwarps;
  B->chunk_mult = chunk_mult;
  if (nwarps != 24) B->cluster = 1;
  drop_graph(B);
  return GRX_OK;
}

extern "C" grx_status grx_gcmc_batch_get_shape(grx_gcmc_batch* B, int32_t* nwarps, int32_t* chunk_mult) {
  GRX_REQUIRE(B, "grx_gcmc_batch_get_shape: null batch");
  if (nwarps) *nwarps = B->nwarps;
  if (chunk_mult) *chunk_mult = B->chunk_mult;
  return GRX_OK;
}

// The largest cluster size (8, 4 or 2) for which every box of the batch gets its own
// resident cluster, or 1 when the boxes already fill the SMs.
static int max_cluster(const grx_gcmc_batch* B) {
  const int nb = (int)B->boxes.size();
  for (int cl : {8, 4, 2})
    if (gcmc_cluster_capacity(B->prec, cl, B->smem) >= nb) return cl;
  return 1;
}

extern "C" grx_status grx_gcmc_batch_set_cluster(grx_gcmc_batch* B, int32_t cluster) {
  GRX_REQUIRE(B, "grx_gcmc_batch_set_cluster: null batch");
  GRX_REQUIRE(cluster == 1 || cluster == 2 || cluster == 4 || cluster == 8,
              "grx_gcmc_batch_set_cluster: cluster must be 1, 2, 4 or 8");
  GRX_REQUIRE(cluster == 1 || B->nwarps == 24, "grx_gcmc_batch_set_cluster: clusters use 24 warps per block");
  GRX_CHECK_CUDA(cudaStreamSynchronize(B->stream), "set cluster");
  if (cluster > 1) {
    GRX_CHECK_CUDA(cudaSetDevice(B->device), "set device");
    grx_status st = set_gcmc_smem();
    if (st) return st;
    GRX_REQUIRE(gcmc_cluster_capacity(B->prec, cluster, B->smem) >= (int)B->boxes.size(),
                "grx_gcmc_batch_set_cluster: not every box gets a resident cluster of this size");
  }
  B->cluster = cluster;
  drop_graph(B);
  return GRX_OK;
}

extern "C" grx_status grx_gcmc_batch_get_cluster(grx_gcmc_batch* B, int32_t* cluster) {
  GRX_REQUIRE(B && cluster, "grx_gcmc_batch_get_cluster: bad argument");
  *cluster = B->cluster;
  return GRX_OK;
}

// Trial energies behind a set of statistics (one trial configuration against every
// atom: 2 per translation / rotation, trials + orientations per CBMC insertion or
// deletion, the same plus the retrace per reinsertion).
static double trial_energies(const grx_gcmc_batch* B, const std::vector<grx_gcmc_stats>& st) {
  double te = 0.0;
  for (size_t i = 0; i < B->boxes.size(); ++i)
    for (int e = B->first[i]; e < B->first[i + 1]; ++e) {
      const grx_gcmc_desc& d = B->descs[e];
      const bool chain = B->boxes[i]->molsize[d.component] > 1;
      const double grow = d.ntrials + (chain ? d.norient : 0);
      const int64_t* a = st[e].attempts;
      te += 2.0 * (a[0] + a[1]) + grow * (a[2] + a[3]) + (grow + 1 + (chain ? d.norient : 0)) * a[4];
    }
  return te;
}

// Autotuner: runs nsteps real steps of every box for each candidate launch shape
// (warps per box 8 / 12 / 24, times items per warp of a bead pass 1 / 2 / 4), timed
// with CUDA events, and keeps the shape with the most trial energies per second. The
// chains change while they are probed (boxes fill up from empty), so each candidate
// is timed twice, in a forward and a reverse sweep, and ranked by work per time.
// ms_per_candidate reports the mean time of one probe. When the boxes leave SMs idle
// (a cluster of 2, 4 or 8 CTAs per box is resident for every box), the best shape is then
// probed against clusters of 24-warp CTAs with the best 24-warp items per warp, in the
// order plain, cluster, cluster, plain, and the faster kept. The probe steps are ordinary
// Monte Carlo steps: the chains advance by up to 2 * (GRX_GCMC_TUNE_CANDIDATES + 2) * nsteps.
extern "C" grx_status grx_gcmc_batch_autotune(grx_gcmc_batch* B, int64_t nsteps, int32_t* chosen,
                                              float* ms_per_candidate) {
  GRX_REQUIRE(B && nsteps >= 1, "grx_gcmc_batch_autotune: bad argument");
  static const int warps[3] = {8, 12, 24}, mults[3] = {1, 2, 4};
  static_assert(GRX_GCMC_TUNE_CANDIDATES == 9, "candidate table");
  const int nb = (int)B->boxes.size();
  cudaEvent_t e0, e1;
  GRX_CHECK_CUDA(cudaEventCreate(&e0), "event");
  GRX_CHECK_CUDA(cudaEventCreate(&e1), "event");
  std::vector<grx_gcmc_stats> before(B->nentries), after(B->nentries);
  auto read = [&](std::vector<grx_gcmc_stats>& v) {
    return cudaMemcpy(v.data(), B->d_stats, B->nentries * sizeof(grx_gcmc_stats), cudaMemcpyDeviceToHost);
  };
  // one timed probe of a shape: adds its milliseconds and trial energies
  auto probe = [&](int nw, int mult, int cl, double& ms_acc, double& te_acc) -> grx_status {
    grx_status st = upload_mult(B, mult);
    if (st) return st;
    GRX_CHECK_CUDA(read(before), "tune stats");
    GRX_CHECK_CUDA(cudaEventRecord(e0, B->stream), "event");
    st = enqueue_gcmc(B->prec, nw, nb, B->d_boxes, B->d_args, B->d_first, B->d_step, nsteps, B->d_stats, B->smem,
                      B->stream, cl, B->swaps);
    if (st) return st;
    GRX_CHECK_CUDA(cudaEventRecord(e1, B->stream), "event");
    GRX_CHECK_CUDA(cudaEventSynchronize(e1), "event");
    float ms = 0.f;
    GRX_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1), "event");
    GRX_CHECK_CUDA(read(after), "tune stats");
    ms_acc += ms;
    te_acc += trial_energies(B, after) - trial_energies(B, before);
    return GRX_OK;
  };
  auto rate = [](double te, double ms) { return te > 0.0 ? te / ms : 1.0 / ms; };
  GRX_CHECK_CUDA(cudaStreamSynchronize(B->stream), "tune sync");
  double ms_sum[GRX_GCMC_TUNE_CANDIDATES] = {}, te_sum[GRX_GCMC_TUNE_CANDIDATES] = {};
  for (int k = 0; k < 2 * GRX_GCMC_TUNE_CANDIDATES; ++k) {
    const int c = k < GRX_GCMC_TUNE_CANDIDATES ? k : 2 * GRX_GCMC_TUNE_CANDIDATES - 1 - k;
    grx_status st = probe(warps[c / 3], mults[c % 3], 1, ms_sum[c], te_sum[c]);
    if (st) return st;
  }
  int best = 0, best24 = 6;
  for (int c = 0; c < GRX_GCMC_TUNE_CANDIDATES; ++c) {
    if (ms_per_candidate) ms_per_candidate[c] = (float)(ms_sum[c] / 2.0);
    if (rate(te_sum[c], ms_sum[c]) > rate(te_sum[best], ms_sum[best])) best = c;
    if (c >= 6 && rate(te_sum[c], ms_sum[c]) > rate(te_sum[best24], ms_sum[best24])) best24 = c;
  }
  int best_w = warps[best / 3], best_m = mults[best % 3], best_cl = 1;
  const int clmax = max_cluster(B);
  if (clmax > 1) {
    double ms_p = 0.0, te_p = 0.0, ms_c = 0.0, te_c = 0.0;
    for (int k = 0; k < 4; ++k) {
      const bool plain = k == 0 || k == 3;
      grx_status st = plain ? probe(best_w, best_m, 1, ms_p, te_p) : probe(24, mults[best24 % 3], clmax, ms_c, te_c);
      if (st) return st;
    }
    if (rate(te_c, ms_c) > rate(te_p, ms_p)) {
      best_w = 24;
      best_m = mults[best24 % 3];
      best_cl = clmax;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  grx_status st = upload_mult(B, best_m);
  if (st) return st;
  B->nwarps = best_w;
  B->chunk_mult = best_m;
  B->cluster = best_cl;
  drop_graph(B);
  if (chosen) *chosen = (best_cl - 1) * 10000 + best_w * 100 + best_m;
  return GRX_OK;
}

// ---------------------------------------------------------------- molecule updates
namespace grx {

struct MolWrite {
  double x[kMolWork], y[kMolWork], z[kMolWork], q[kMolWork];
  int type[kMolWork];
};

// Update_insertion_data_Parallel / update_translation_position (mc_utilities.h:191-234,
// 285-292): one thread per atom writes every stored representation.
__global__ void write_molecule_kernel(BoxDev b, int comp, int first, int ms, int mol, int grow, MolWrite m) {
  const int a = threadIdx.x;
  if (a < ms) store_atom(b, first + a, m.x[a], m.y[a], m.z[a], m.q[a], 1.0, 1.0, m.type[a], mol);
  if (grow && a == 0) const_cast<int*>(b.comp_size)[comp] += ms;
}

// Update_deletion_data_Parallel (mc_utilities.h:163-189): the last molecule moves
// into the removed slot, which keeps its molecule index.
__global__ void remove_molecule_kernel(BoxDev b, int comp, int dst, int src, int ms, int mol) {
  const int a = threadIdx.x;
  if (a < ms && dst != src) copy_atom(b, dst + a, src + a, mol);
  if (a == 0) const_cast<int*>(b.comp_size)[comp] -= ms;
}

}  // namespace grx

extern "C" grx_status grx_box_write_molecule(grx_box* b, int32_t comp, size_t mol, const double* pos,
                                             const double* charge, const size_t* type) {
  GRX_REQUIRE(b && pos && charge && type, "grx_box_write_molecule: null argument");
  GRX_REQUIRE(comp >= b->nhost && comp < b->ncomp, "grx_box_write_molecule: not an adsorbate component");
  const size_t ms = b->molsize[comp];
  GRX_REQUIRE(ms >= 1 && ms <= (size_t)kMolWork, "grx_box_write_molecule: molecule size must be 1..32");
  GRX_CHECK_CUDA(cudaStreamSynchronize(b->stream), "write_molecule sync");
  GRX_CHECK_CUDA(cudaMemcpy(b->size, b->d_size, GRX_MAX_COMPONENTS * sizeof(int), cudaMemcpyDeviceToHost),
                 "read sizes");
  const size_t n = (size_t)b->size[comp] / ms;
  GRX_REQUIRE(mol <= n, "grx_box_write_molecule: molecule index beyond the count");
  if ((mol + 1) * ms > b->cap[comp]) {
    set_error("grx_box_write_molecule: component %d capacity %zu exhausted", comp, b->cap[comp]);
    return GRX_ERR_CAPACITY;
  }
  MolWrite m{};
  for (size_t a = 0; a < ms; ++a) {
    m.x[a] = pos[3 * a];
    m.y[a] = pos[3 * a + 1];
    m.z[a] = pos[3 * a + 2];
    m.q[a] = charge[a];
    GRX_REQUIRE(type[a] < (size_t)b->dev.ntypes, "grx_box_write_molecule: atom type out of range");
    m.type[a] = (int)type[a];
    if (charge[a] != 0.0) b->has_charge[comp] = 1;
  }
  refresh_dev(b);
  const int grow = mol == n ? 1 : 0;
  write_molecule_kernel<<<1, 32, 0, b->stream>>>(b->dev, comp, (int)(b->off[comp] + mol * ms), (int)ms, (int)mol,
                                                 grow, m);
  count_launch();
  GRX_CHECK_CUDA(cudaGetLastError(), "write_molecule launch");
  if (grow) b->size[comp] += (int)ms;
  b->stored[comp] = std::max(b->stored[comp], (mol + 1) * ms);
  GRX_CHECK_CUDA(cudaStreamSynchronize(b->stream), "write_molecule");
  return GRX_OK;
}

extern "C" grx_status grx_box_remove_molecule(grx_box* b, int32_t comp, size_t mol) {
  GRX_REQUIRE(b, "grx_box_remove_molecule: null box");
  GRX_REQUIRE(comp >= b->nhost && comp < b->ncomp, "grx_box_remove_molecule: not an adsorbate component");
  const size_t ms = b->molsize[comp];
  GRX_CHECK_CUDA(cudaStreamSynchronize(b->stream), "remove_molecule sync");
  GRX_CHECK_CUDA(cudaMemcpy(b->size, b->d_size, GRX_MAX_COMPONENTS * sizeof(int), cudaMemcpyDeviceToHost),
                 "read sizes");
  const size_t n = (size_t)b->size[comp] / ms;
  GRX_REQUIRE(mol < n, "grx_box_remove_molecule: molecule index beyond the count");
  refresh_dev(b);
  remove_molecule_kernel<<<1, 32, 0, b->stream>>>(b->dev, comp, (int)(b->off[comp] + mol * ms),
                                                  (int)(b->off[comp] + (n - 1) * ms), (int)ms, (int)mol);
  count_launch();
  GRX_CHECK_CUDA(cudaGetLastError(), "remove_molecule launch");
  b->size[comp] -= (int)ms;
  GRX_CHECK_CUDA(cudaStreamSynchronize(b->stream), "remove_molecule");
  return GRX_OK;
}
