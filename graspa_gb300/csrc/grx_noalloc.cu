// grx_noalloc.cu -- trial energies without any device allocation at call time.
//
// grx_trial_energies grows a per-box scratch buffer with cudaMalloc when a call needs
// more than the last one. Some callers cannot allow that: a Monte Carlo loop that
// must never stall the device (cudaMalloc and cudaFree can synchronize the whole
// GPU and hold up other jobs' streams), or a host application whose device memory
// all belongs to its own pool allocator. For them, grx_trial_energies_noalloc does
// the same work with its scratch in one file-scope device array of fixed size,
// GRX_NOALLOC_SCRATCH_BYTES, which every GPU that loads this library holds until the
// process exits.
//
// Rules of use:
//  * at most GRX_NOALLOC_MAX_BEADS (= ntrials * chainsize) trial beads per call;
//    larger requests fail with GRX_ERR_CAPACITY and touch nothing;
//  * the first call on a device looks the array up with cudaGetSymbolAddress
//    (once per device, with the box's device made current for the call and the
//    caller's device restored after); make that first call before any stream capture
//    is started;
//  * all calls share the one array and it keeps the last call's contents. The
//    parts that must start at zero (overlap flags) are cleared on every call.
//    Calls that overlap on the GPU (two host threads, two streams) race on the
//    array: issue them one after another.
// The box itself is created beforehand with grx_box_create (which allocates once).
#include <mutex>

#include "grx_host.h"
#include "grx_warp.cuh"

namespace grx {

namespace {

constexpr int kNoallocBeads = GRX_NOALLOC_MAX_BEADS;

// scratch layout (byte offsets, every block 256 B aligned)
constexpr size_t kOffPos = 0;                                           // double[3*B]
constexpr size_t kOffScale = kOffPos + 3 * kNoallocBeads * 8;           // double[B]
constexpr size_t kOffCharge = kOffScale + kNoallocBeads * 8;            // double[B]
constexpr size_t kOffScaleCoul = kOffCharge + kNoallocBeads * 8;        // double[B]
constexpr size_t kOffType = kOffScaleCoul + kNoallocBeads * 8;          // size_t[B]
constexpr size_t kOffBeads = kOffType + kNoallocBeads * 8;              // Bead[B]
constexpr size_t kBeadBytes = ((kNoallocBeads * sizeof(Bead)) + 255) / 256 * 256;
constexpr size_t kOffPart = kOffBeads + kBeadBytes;                     // double[4*B]
constexpr size_t kOffFlags = kOffPart + 4 * kNoallocBeads * 8;          // int[B]
constexpr size_t kOffOut = kOffFlags + kNoallocBeads * 4;               // double[4*B]
constexpr size_t kOffOver = kOffOut + 4 * kNoallocBeads * 8;            // uint8[B]
constexpr size_t kNeed = kOffOver + kNoallocBeads;

static_assert(kNeed <= GRX_NOALLOC_SCRATCH_BYTES, "scratch array too small for its layout");
static_assert(kOffScale % 256 == 0 && kOffBeads % 256 == 0 && kOffPart % 256 == 0 && kOffOut % 256 == 0,
              "scratch blocks must stay aligned");

__device__ __align__(256) unsigned char g_noalloc_scratch[GRX_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Makes `dev` current for the life of the guard and restores the caller's device after.
struct DeviceGuard {
  int prev = -1;
  cudaError_t err = cudaSuccess;
  explicit DeviceGuard(int dev) {
    err = cudaGetDevice(&prev);
    if (err == cudaSuccess && prev != dev) err = cudaSetDevice(dev);
    else if (err == cudaSuccess) prev = -1;
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// Device address of the scratch array on device `dev`, which must be current (set-up
// once per device).
grx_status scratch_address(int dev, unsigned char** out) {
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("grx_trial_energies_noalloc: device ordinal %d out of range", dev);
    return GRX_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr)
      return cuda_status(e != cudaSuccess ? e : cudaErrorInvalidSymbol,
                         "grx_trial_energies_noalloc: cudaGetSymbolAddress");
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[dev];
  return GRX_OK;
}

// Raw trial arrays (already in the scratch array) -> Bead records, the same split
// and charge products as the staging of grx_trial_energies.
__global__ void noalloc_beads_kernel(const double* pos, const double* scale, const double* charge,
                                     const double* scale_coul, const size_t* type, int nb, int has_scale,
                                     int has_charge, int has_scale_coul, double prefactor, Bead* beads) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nb) return;
  const double sc = has_scale ? scale[j] : 1.0;
  const double q = has_charge ? charge[j] : 0.0;
  const double scc = has_scale_coul ? scale_coul[j] : 1.0;
  make_bead(beads[j], pos[3 * j], pos[3 * j + 1], pos[3 * j + 2], q * scc, sc, (int)type[j], prefactor);
}

__global__ void noalloc_reduce_kernel(const double* part, const int* flags, int nb, int chain, double* out,
                                      unsigned char* over) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  const int ntr = nb / chain;
  if (w >= ntr * 4) return;
  const int t = w >> 2, q = w & 3;
  double s = 0.0;
  for (int a = 0; a < chain; ++a) s += part[(size_t)(t * chain + a) * 4 + q];
  out[t * 4 + q] = s;
  if (q == 0) {
    int f = 0;
    for (int a = 0; a < chain; ++a) f |= flags[t * chain + a];
    over[t] = f ? 1 : 0;
  }
}

}  // namespace
}  // namespace grx

using namespace grx;

extern "C" grx_status grx_trial_energies_noalloc(grx_box* b, const grx_trials* t, int32_t component,
                                                 int64_t exclude_comp, int64_t exclude_molid,
                                                 grx_precision prec, grx_trial_energy* out,
                                                 uint8_t* overlap) {
  GRX_REQUIRE(b && t && out && overlap, "grx_trial_energies_noalloc: null argument");
  GRX_REQUIRE(t->chainsize >= 1, "grx_trial_energies_noalloc: chainsize must be >= 1");
  GRX_REQUIRE(prec == GRX_FP64 || prec == GRX_MIXED || prec == GRX_FP32,
              "grx_trial_energies_noalloc: bad precision");
  GRX_REQUIRE(component >= 0 && component < b->ncomp, "grx_trial_energies_noalloc: component out of range");
  if (t->ntrials == 0) return GRX_OK;
  GRX_REQUIRE(t->pos && t->type, "grx_trial_energies_noalloc: bead arrays missing");
  // checked before multiplying, so no trial count can wrap the product below the maximum
  if (t->chainsize > (size_t)kNoallocBeads || t->ntrials > (size_t)kNoallocBeads / t->chainsize) {
    set_error("grx_trial_energies_noalloc: %zu trials x %zu beads exceed the fixed maximum of %d trial beads",
              t->ntrials, t->chainsize, kNoallocBeads);
    return GRX_ERR_CAPACITY;
  }
  const int nb = (int)(t->ntrials * t->chainsize);
  // the box's stream belongs to the box's device: work there, whatever the caller's current device
  DeviceGuard guard(b->device);
  GRX_CHECK_CUDA(guard.err, "grx_trial_energies_noalloc: select the box's device");
  unsigned char* base = nullptr;
  grx_status st = scratch_address(b->device, &base);
  if (st) return st;
  refresh_dev(b);
  cudaStream_t s = b->stream;
  double* pos = reinterpret_cast<double*>(base + kOffPos);
  double* scale = reinterpret_cast<double*>(base + kOffScale);
  double* charge = reinterpret_cast<double*>(base + kOffCharge);
  double* scale_coul = reinterpret_cast<double*>(base + kOffScaleCoul);
  size_t* type = reinterpret_cast<size_t*>(base + kOffType);
  Bead* beads = reinterpret_cast<Bead*>(base + kOffBeads);
  double* part = reinterpret_cast<double*>(base + kOffPart);
  int* flags = reinterpret_cast<int*>(base + kOffFlags);
  double* dout = reinterpret_cast<double*>(base + kOffOut);
  unsigned char* dover = base + kOffOver;
  GRX_CHECK_CUDA(cudaMemcpyAsync(pos, t->pos, 3 * nb * sizeof(double), cudaMemcpyDefault, s), "noalloc: stage pos");
  if (t->scale)
    GRX_CHECK_CUDA(cudaMemcpyAsync(scale, t->scale, nb * sizeof(double), cudaMemcpyDefault, s), "noalloc: stage scale");
  if (t->charge)
    GRX_CHECK_CUDA(cudaMemcpyAsync(charge, t->charge, nb * sizeof(double), cudaMemcpyDefault, s), "noalloc: stage charge");
  if (t->scale_coul)
    GRX_CHECK_CUDA(cudaMemcpyAsync(scale_coul, t->scale_coul, nb * sizeof(double), cudaMemcpyDefault, s),
                   "noalloc: stage scaleCoul");
  GRX_CHECK_CUDA(cudaMemcpyAsync(type, t->type, nb * sizeof(size_t), cudaMemcpyDefault, s), "noalloc: stage type");
  GRX_CHECK_CUDA(cudaMemsetAsync(flags, 0, nb * sizeof(int), s), "noalloc: clear flags");
  noalloc_beads_kernel<<<(nb + 127) / 128, 128, 0, s>>>(pos, scale, charge, scale_coul, type, nb, t->scale != nullptr,
                                                        t->charge != nullptr, t->scale_coul != nullptr,
                                                        b->dev.prefactor, beads);
  const int ec = (int)exclude_comp, em = (int)exclude_molid, nm = (int)t->molid;
  if (prec == GRX_FP64)
    trial_bead_kernel<GRX_FP64><<<nb, GRX_THREADS, 0, s>>>(b->dev, beads, component, nm, ec, em, part, flags);
  else if (prec == GRX_MIXED)
    trial_bead_kernel<GRX_MIXED><<<nb, GRX_THREADS, 0, s>>>(b->dev, beads, component, nm, ec, em, part, flags);
  else
    trial_bead_kernel<GRX_FP32><<<nb, GRX_THREADS, 0, s>>>(b->dev, beads, component, nm, ec, em, part, flags);
  const int ntr = (int)t->ntrials;
  noalloc_reduce_kernel<<<(ntr * 4 + 127) / 128, 128, 0, s>>>(part, flags, nb, (int)t->chainsize, dout, dover);
  count_launch(3);
  GRX_CHECK_CUDA(cudaGetLastError(), "grx_trial_energies_noalloc: launch");
  GRX_CHECK_CUDA(cudaMemcpyAsync(out, dout, ntr * sizeof(grx_trial_energy), cudaMemcpyDefault, s),
                 "noalloc: read energies");
  GRX_CHECK_CUDA(cudaMemcpyAsync(overlap, dover, ntr, cudaMemcpyDefault, s), "noalloc: read flags");
  GRX_CHECK_CUDA(cudaStreamSynchronize(s), "grx_trial_energies_noalloc");
  return GRX_OK;
}
