// grx_internal.cuh -- device-side state and shared device functions of libgrx.
//
// Layout of one box in HBM (all arrays sized by component capacity, component c
// occupying [comp_off[c], comp_off[c] + capacity[c]), live atoms first):
//   pos64  double4 {x, y, z, q*scaleCoul}      FP64 path, Coulomb charges
//   hi     float4  {x_hi, y_hi, z_hi, q*sc}     hi = x rounded to a 2^-12 A grid
//   lo     float4  {x - x_hi, ..., scale}       so hi differences are exact in FP32
//   meta   int2    {type, molid}
//   scale  double  LJ lambda scaling (Atoms.scale)
// Ewald: active k list (int4 kx,ky,kz,slot + double prefactor table) and complex
// structure factors indexed by the reference's k slot.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include "../../include/grx.h"

#define GRX_THREADS 256
#define GRX_GRID_COORD 4096.0  // 2^12: hi-part grid of the split coordinates

namespace grx {

struct FFPair64 {  // per type pair, FP64: {eps or C12, sigma or C6, z or C4, shift}
  double a, b, c, shift;
};

struct BoxDev {
  // geometry
  double cell[9];
  double inv[9];
  float cell_hi[9];
  float cell_lo[9];
  float invf[9];
  int cubic;
  double alpha;
  double prefactor;
  double volume;
  // force field
  int ntypes;
  int use_1264;
  int no_charges;
  int vdw_real_bias;
  double cut_vdw2;
  double cut_coul2;
  double overlap;
  float screen2;     // FP32 screening radius^2 with guard band
  float overlapf;    // OverlapCriteria as float
  float cut_vdw2f;
  float cut_coul2f;
  const FFPair64* ff64;  // ntypes^2
  const double* ffc10;   // ntypes^2
  const float4* ff32;    // {4 eps, 1/sigma^2, shift, (1.1 sigma)^2}
  // atoms
  int ncomp;
  int nhost;
  int comp_off[GRX_MAX_COMPONENTS + 1];
  const int* comp_size;  // device, live atoms per component
  const double4* pos64;
  const float4* hi;
  const float4* lo;
  const int2* meta;
  const double* scale;
  const double* charge;  // bare charge (Atoms.charge), templates for trial beads
  int host_end;          // storage index where guest components begin
  // host (framework) atoms, index < host_end: the box's own arrays, or a parent box's
  // when the box is a replica sharing its framework (guests are always the box's own)
  const double4* hpos64;
  const float4* hhi;
  const float4* hlo;
  const int2* hmeta;
  const double* hscale;
  const float2* hqdf;
  int shared_host;       // 1: host atoms, tiles, tables and framework S(k) belong to a parent
  // spatial tiles of host atoms (32 atoms each, k-d order)
  const float4* tile_c;  // per tile: {x, y, z, bounding radius}, {box half extents, 0}
  const int4* tile_r;    // {first atom, end atom, component, 0}
  int ntiles;
  // voxel candidate lists of host atoms (grx_voxel.cu); used instead of the tiles when vox
  const float4* hrec;            // host atoms: {hi xyz, q hi}, {lo xyz, q lo} per atom
  const unsigned short* htype;   // host atoms: type | 0x8000 when scale != 1
  const int4* vmeta;     // per voxel {first entry, sure atoms, all atoms, 0}
  const unsigned* vlist; // entries: storage index | lattice shift << 20
  int vox;
  int vn[3];             // voxels along a, b, c
  int vchunks;           // 32-entry chunks of the longest list
  int cull;              // tile culling on
  float cull_r;          // screening radius used by the tile test
  float cellf[9];
  int chunk_mult;        // work items per warp and bead pass (tile-range chunking; autotuned)
  int ew_rows;           // GCMC Ewald delta through (kx, ky) row products (shared memory sized for it)
  float wperp[3];        // perpendicular widths of the cell (distances between lattice planes)
  float half_wmin2;      // (min width / 2)^2, shrunk for FP32 rounding
  // real-space Coulomb table: g(s) = erfc(alpha sqrt s)/sqrt s, piecewise quintic in
  // s = r^2, 64 pieces per octave indexed by the FP32 bit pattern of s
  const double* ctab;    // per piece {s0, 1/width, c0..c5}
  int ctab_base;
  int ctab_n;
  // double-float data of the mixed-precision dense path
  const float4* ctabf;   // per piece {s0, 1/width, c0 hi, c0 lo}, {c1 hi, lo, c2 hi, lo}, ...
  const float2* qdf;     // q * scaleCoul, hi/lo
  const float4* ffdf;    // {4 eps hi, lo, 1/sigma^2 hi, lo}
  const float2* ffdf2;   // {shift hi, lo}
  float2 cut_vdw2_df;
  float2 cut_coul2_df;
  const float4* ewA;     // per active k {re hi, re lo, im hi, im lo} of temp * S_ads
  const float4* ewF;     // ... of temp * S_fw
  const float2* ewT;     // temp as double-float
  // ewald
  int kmax[3];
  int nvec;
  int nact;
  const int4* kact;     // kx, ky, kz, slot
  const double* ktemp;  // factor * exp(-k^2/4a^2)/k^2 per active k
  double2* s_fw;
  double2* s_ads;
  double2* s_tmp;
};

// ---------------------------------------------------------------- Philox
// Philox4x32-10 (Salmon et al., SC'11). Counter {slot, move lo, move hi, stream},
// key = seed: the same stream layout as the test oracle.
__host__ __device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
    const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]);
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]);
#else
    const uint32_t hi0 = (uint32_t)(((uint64_t)0xD2511F53u * c[0]) >> 32);
    const uint32_t hi1 = (uint32_t)(((uint64_t)0xCD9E8D57u * c[2]) >> 32);
#endif
    const uint32_t lo0 = 0xD2511F53u * c[0];
    const uint32_t lo1 = 0xCD9E8D57u * c[2];
    const uint32_t n0 = hi1 ^ c[1] ^ k0;
    const uint32_t n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

__host__ __device__ inline void draw4(uint64_t seed, uint32_t stream, uint64_t move, uint32_t slot,
                                      uint32_t out[4]) {
  out[0] = slot;
  out[1] = (uint32_t)move;
  out[2] = (uint32_t)(move >> 32);
  out[3] = stream;
  philox4x32_10(out, (uint32_t)seed, (uint32_t)(seed >> 32));
}

__host__ __device__ inline double u01(uint32_t w) { return (double)w * 2.3283064365386963e-10; }

// Out-of-line forms for the per-move code of the persistent kernels: one copy of the Philox
// rounds and of the library FP64 exp serves every call site of a kernel. These run once per
// move, on few lanes, where instruction fetch rather than arithmetic sets the time, so a
// smaller kernel is a faster one. Results are those of draw4 and exp.
static __device__ __noinline__ uint4 draw4_out(uint64_t seed, uint32_t stream, uint64_t move, uint32_t slot) {
  uint32_t w[4];
  draw4(seed, stream, move, slot, w);
  return make_uint4(w[0], w[1], w[2], w[3]);
}
__device__ __forceinline__ void draw4_dev(uint64_t seed, uint32_t stream, uint64_t move, uint32_t slot,
                                          uint32_t out[4]) {
  const uint4 r = draw4_out(seed, stream, move, slot);
  out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = r.w;
}
static __device__ __noinline__ double exp_move(double x) { return exp(x); }

enum : uint32_t { SLOT_FIRST = 0u, SLOT_ORIENT = 1024u, SLOT_SELECT = 2048u, SLOT_RETRACE = 3072u };

// ---------------------------------------------------------------- geometry
// Minimum image of the reference, PBC() maths.cuh:427-450 (int-cast rounding).
__device__ __forceinline__ void pbc64(const BoxDev& b, double& x, double& y, double& z) {
  if (b.cubic) {
    x -= (double)(int)(x * b.inv[0] + ((x >= 0.0) ? 0.5 : -0.5)) * b.cell[0];
    y -= (double)(int)(y * b.inv[4] + ((y >= 0.0) ? 0.5 : -0.5)) * b.cell[4];
    z -= (double)(int)(z * b.inv[8] + ((z >= 0.0) ? 0.5 : -0.5)) * b.cell[8];
  } else {
    double sx = b.inv[0] * x + b.inv[3] * y + b.inv[6] * z;
    double sy = b.inv[1] * x + b.inv[4] * y + b.inv[7] * z;
    double sz = b.inv[2] * x + b.inv[5] * y + b.inv[8] * z;
    sx -= (double)(int)(sx + ((sx >= 0.0) ? 0.5 : -0.5));
    sy -= (double)(int)(sy + ((sy >= 0.0) ? 0.5 : -0.5));
    sz -= (double)(int)(sz + ((sz >= 0.0) ? 0.5 : -0.5));
    x = b.cell[0] * sx + b.cell[3] * sy + b.cell[6] * sz;
    y = b.cell[1] * sx + b.cell[4] * sy + b.cell[7] * sz;
    z = b.cell[2] * sx + b.cell[5] * sy + b.cell[8] * sz;
  }
}

// Split-coordinate minimum image: (dh, dl) = hi and lo parts of a displacement.
// The integer image shift is chosen from the FP32 sum with the reference's
// rounding rule; the shift is applied to both parts so dh stays exact.
__device__ __forceinline__ void pbc_split(const BoxDev& b, float3& dh, float3& dl) {
  const float x = dh.x + dl.x, y = dh.y + dl.y, z = dh.z + dl.z;
  float nx, ny, nz;
  if (b.cubic) {
    nx = (float)(int)(x * b.invf[0] + ((x >= 0.f) ? 0.5f : -0.5f));
    ny = (float)(int)(y * b.invf[4] + ((y >= 0.f) ? 0.5f : -0.5f));
    nz = (float)(int)(z * b.invf[8] + ((z >= 0.f) ? 0.5f : -0.5f));
    dh.x -= nx * b.cell_hi[0]; dl.x -= nx * b.cell_lo[0];
    dh.y -= ny * b.cell_hi[4]; dl.y -= ny * b.cell_lo[4];
    dh.z -= nz * b.cell_hi[8]; dl.z -= nz * b.cell_lo[8];
  } else {
    const float sx = b.invf[0] * x + b.invf[3] * y + b.invf[6] * z;
    const float sy = b.invf[1] * x + b.invf[4] * y + b.invf[7] * z;
    const float sz = b.invf[2] * x + b.invf[5] * y + b.invf[8] * z;
    nx = (float)(int)(sx + ((sx >= 0.f) ? 0.5f : -0.5f));
    ny = (float)(int)(sy + ((sy >= 0.f) ? 0.5f : -0.5f));
    nz = (float)(int)(sz + ((sz >= 0.f) ? 0.5f : -0.5f));
    // hi parts: cell_hi on the 2^-12 grid, small integer multiples stay exact
    dh.x -= nx * b.cell_hi[0]; dh.x -= ny * b.cell_hi[3]; dh.x -= nz * b.cell_hi[6];
    dh.y -= nx * b.cell_hi[1]; dh.y -= ny * b.cell_hi[4]; dh.y -= nz * b.cell_hi[7];
    dh.z -= nx * b.cell_hi[2]; dh.z -= ny * b.cell_hi[5]; dh.z -= nz * b.cell_hi[8];
    dl.x -= nx * b.cell_lo[0] + ny * b.cell_lo[3] + nz * b.cell_lo[6];
    dl.y -= nx * b.cell_lo[1] + ny * b.cell_lo[4] + nz * b.cell_lo[7];
    dl.z -= nx * b.cell_lo[2] + ny * b.cell_lo[5] + nz * b.cell_lo[8];
  }
}

// ---------------------------------------------------------------- potentials
// VDW(), maths.cuh:452-494 (FP64, soft-core lambda and 12-6-4 mode).
__device__ __forceinline__ double vdw64(const BoxDev& b, int row, double rr, double scaling) {
  const FFPair64 f = b.ff64[row];
  if (b.use_1264) {
    const double ri2 = 1.0 / rr;
    const double ri4 = ri2 * ri2;
    const double ri6 = ri4 * ri2;
    const double ri10 = ri4 * ri6;
    const double ri12 = ri6 * ri6;
    return scaling * (f.a * ri12 - f.b * ri6 + b.ffc10[row] * ri10 + f.c * ri4 - f.shift);
  }
  const double arg1 = 4.0 * f.a;
  const double arg2 = f.b * f.b;
  const double temp = rr / arg2;
  const double temp3 = temp * temp * temp;
  const double rri3 = 1.0 / (temp3 + 0.5 * (1.0 - scaling) * (1.0 - scaling));
  const double term = arg1 * (rri3 * (rri3 - 1.0)) - f.shift;
  return scaling * term;
}

__device__ __forceinline__ float vdw32(float4 f, float rr) {
  const float t = rr * f.y;
  const float t3 = t * t * t;
  const float rri3 = __fdividef(1.0f, t3);
  return f.x * (rri3 * (rri3 - 1.0f)) - f.z;
}

// CoulombReal(), maths.cuh:496-500, with q already multiplied by scaleCoul.
__device__ __forceinline__ double coul64(const BoxDev& b, double qq, double rr) {
  const double r = sqrt(rr);
  return b.prefactor * qq * erfc(b.alpha * r) / r;
}

__device__ __forceinline__ float coul32(const BoxDev& b, float qq, float rr) {
  const float r = sqrtf(rr);
  return (float)b.prefactor * qq * erfcf((float)b.alpha * r) / r;
}

// ---------------------------------------------------------------- bead
struct Bead {
  double x, y, z;      // FP64 position
  float3 h, l;         // split position
  double q;            // charge * scaleCoul
  double scale;        // LJ lambda
  float2 pq;           // prefactor * q as double-float
  int type;
  int unit;            // scale == 1
};

__device__ __forceinline__ void split_coord(double x, float& h, float& l) {
  const double hd = rint(x * GRX_GRID_COORD) * (1.0 / GRX_GRID_COORD);
  h = (float)hd;
  l = (float)(x - hd);
}

__device__ __forceinline__ void make_bead(Bead& bd, double x, double y, double z, double q,
                                          double scale, int type, double prefactor) {
  bd.x = x; bd.y = y; bd.z = z;
  split_coord(x, bd.h.x, bd.l.x);
  split_coord(y, bd.h.y, bd.l.y);
  split_coord(z, bd.h.z, bd.l.z);
  bd.q = q; bd.scale = scale; bd.type = type;
  const double pq = prefactor * q;
  const float ph = __double2float_rn(pq);
  bd.pq = make_float2(ph, __double2float_rn(pq - (double)ph));
  bd.unit = scale == 1.0;
}

// Energy of one (atom, bead) pair. Returns true when the pair is inside a cutoff;
// adds to vdw / real and sets `flag` on overlap (VDW_Coulomb.cu:1290-1322).
// Atom arrays by storage index: host atoms may live in a parent box (replicas).
__device__ __forceinline__ double4 atom_pos64(const BoxDev& b, int i) { return i < b.host_end ? b.hpos64[i] : b.pos64[i]; }
__device__ __forceinline__ int2 atom_meta(const BoxDev& b, int i) { return i < b.host_end ? b.hmeta[i] : b.meta[i]; }
__device__ __forceinline__ double atom_scale(const BoxDev& b, int i) { return i < b.host_end ? b.hscale[i] : b.scale[i]; }

template <int PREC>
__device__ __forceinline__ void pair_energy(const BoxDev& b, int i, const Bead& bd, int rowbase,
                                            double& vdw, double& real, int& flag) {
  const bool host = i < b.host_end;
  const double4* P64 = host ? b.hpos64 : b.pos64;
  const float4* HI = host ? b.hhi : b.hi;
  const float4* LO = host ? b.hlo : b.lo;
  const int2* META = host ? b.hmeta : b.meta;
  const double* SC = host ? b.hscale : b.scale;
  if (PREC == GRX_FP64) {
    const double4 p = P64[i];
    double x = p.x - bd.x, y = p.y - bd.y, z = p.z - bd.z;
    pbc64(b, x, y, z);
    const double rr = x * x + y * y + z * z;
    const int2 mt = META[i];
    if (rr < b.cut_vdw2) {
      const double e = vdw64(b, mt.x * b.ntypes + bd.type, rr, SC[i] * bd.scale);
      if (e > b.overlap) flag = 1;
      if (rr < 0.01) flag = 1;
      vdw += e;
    }
    if (!b.no_charges && rr < b.cut_coul2) real += coul64(b, p.w * bd.q, rr);
  } else {
    const float4 ah = HI[i];
    const float4 al = LO[i];
    float3 dh = make_float3(ah.x - bd.h.x, ah.y - bd.h.y, ah.z - bd.h.z);
    float3 dl = make_float3(al.x - bd.l.x, al.y - bd.l.y, al.z - bd.l.z);
    pbc_split(b, dh, dl);
    const float fx = dh.x + dl.x, fy = dh.y + dl.y, fz = dh.z + dl.z;
    const float rr32 = fx * fx + fy * fy + fz * fz;
    if (rr32 >= b.screen2) return;
    const int2 mt = META[i];
    const int row = mt.x * b.ntypes + bd.type;
    if (PREC == GRX_MIXED) {
      const double x = (double)dh.x + (double)dl.x;
      const double y = (double)dh.y + (double)dl.y;
      const double z = (double)dh.z + (double)dl.z;
      const double rr = x * x + y * y + z * z;
      if (rr < b.cut_vdw2) {
        const float4 f = b.ff32[row];
        const bool unit = (al.w == 1.0f) && (bd.scale == 1.0) && !b.use_1264;
        double e;
        if (unit && (float)rr > f.w) e = (double)vdw32(f, (float)rr);
        else e = vdw64(b, row, rr, SC[i] * bd.scale);
        if (e > b.overlap) flag = 1;
        if (rr < 0.01) flag = 1;
        vdw += e;
      }
      if (!b.no_charges && rr < b.cut_coul2) real += coul64(b, P64[i].w * bd.q, rr);
    } else {  // GRX_FP32
      const float sc = al.w * (float)bd.scale;
      if (rr32 < b.cut_vdw2f) {
        float e;
        if (sc == 1.0f && !b.use_1264) e = vdw32(b.ff32[row], rr32);
        else e = (float)vdw64(b, row, (double)rr32, (double)sc);
        if (e > (float)b.overlap) flag = 1;
        if (rr32 < 0.01f) flag = 1;
        vdw += (double)e;
      }
      if (!b.no_charges && rr32 < b.cut_coul2f) real += (double)coul32(b, ah.w * (float)bd.q, rr32);
    }
  }
}

// One pass of trial beads over every live atom. Thread t owns bead t % nb and lane
// t / nb; lanes (of this block, offset by lane0, strided by lane_stride across
// blocks) walk the atoms of every component. acc = {hg_vdw, hg_real, gg_vdw,
// gg_real} of the thread's bead; `flag` is set on overlap. Atoms of
// (component, newmol) and (excl_comp, excl_mol) are skipped, as in
// Calculate_Multiple_Trial_Energy_VDWReal (VDW_Coulomb.cu:1274-1276).
template <int PREC>
__device__ __forceinline__ void bead_pass(const BoxDev& b, const Bead& bd, int lane, int lane_stride,
                                          int component, int newmol, int excl_comp, int excl_mol,
                                          double acc[4], int& flag) {
  for (int c = 0; c < b.ncomp; ++c) {
    const int n = b.comp_size[c];
    const int off = b.comp_off[c];
    const bool check_mol = (c == component) || (c == excl_comp);
    double v = 0.0, r = 0.0;
#pragma unroll 2
    for (int i = lane; i < n; i += lane_stride) {
      if (check_mol) {
        const int mol = atom_meta(b, off + i).y;
        if ((c == excl_comp && mol == excl_mol) || (c == component && mol == newmol)) continue;
      }
      pair_energy<PREC>(b, off + i, bd, 0, v, r, flag);
    }
    if (c < b.nhost) { acc[0] += v; acc[1] += r; }
    else { acc[2] += v; acc[3] += r; }
  }
}

// ---------------------------------------------------------------- reductions
// Deterministic block sum of one double per thread (fixed shuffle tree).
__device__ __forceinline__ double block_sum(double v, double* sbuf) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sbuf[w] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = (l < nw) ? sbuf[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    if (l == 0) sbuf[0] = r;
  }
  __syncthreads();
  r = sbuf[0];
  __syncthreads();
  return r;
}

// Complex helpers (Ewald_Energy_Functions.h:28-40).
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

}  // namespace grx

// host-side helpers shared by the translation units
namespace grx {
struct BoxHost;
void set_error(const char* fmt, ...);
grx_status cuda_status(cudaError_t e, const char* what);
void count_launch(uint64_t n = 1);
void note_transfer(size_t h2d, size_t d2h);  // bytes the calling thread's last grx_gcmc_run copied
}  // namespace grx
