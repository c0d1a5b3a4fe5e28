// grx_warp.cuh -- the trial-bead pair engine: tile culling, FP32 screening, warp
// compaction of in-cutoff pairs and dense evaluation.
//
// A work item is (one trial bead, one range of host tiles [+ the guest atoms]) and is
// processed by one warp. For every 32-atom tile the warp first tests the tile's
// bounding sphere against the cutoff (orthorhombic cells), then screens the 32 pairs
// (split-coordinate FP32 in the mixed/FP32 forms, full FP64 in the FP64 form). Pairs
// inside the screening radius are appended to a per-warp ring buffer in shared
// memory; every 32 queued pairs are evaluated by all 32 lanes together, so the costly
// part (FP64 displacement, LJ, real-space Coulomb) runs without idle lanes. The
// order of every sum is fixed by the ballot order, so results are deterministic.
#pragma once

#include "grx_internal.cuh"
#include "grx_df.cuh"

namespace grx {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kQueue = 64;  // ring buffer entries per warp

// ---------------------------------------------------------------- voxel-list staging
// A warp walking a bead's voxel list stages the next 8 chunks (256 entries) into its own shared
// buffer with one bulk copy (cp.async.bulk, completion on an mbarrier) instead of one dependent
// global load per chunk. The copied range is rounded out to 16-byte boundaries (the list array
// carries 8 entries of padding), so the buffer holds up to 264 entries.
constexpr int kStageChunks = 8;
constexpr int kStageBuf = 32 * kStageChunks + 8;
struct alignas(16) VoxStage {
  unsigned buf[kStageBuf];
  unsigned long long mbar;
  unsigned phase;  // parity of the mbarrier phase the next copy completes
  unsigned ok;     // 0 after a wait gave up: the warp reads the lists directly from then on
};
constexpr int kStageSpin = 1 << 20;  // try_wait rounds before a wait gives up

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
// Called by one thread per stage before first use, then fenced and barrier-synchronised.
__device__ __forceinline__ void stage_init(VoxStage& st) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&st.mbar)) : "memory");
  st.phase = 0;
  st.ok = 1;
}
__device__ __forceinline__ void stage_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// Lane 0: expect `bytes` on the mbarrier and start the bulk copy of [src, src + bytes).
__device__ __forceinline__ void stage_issue(VoxStage& st, const unsigned* src, unsigned bytes) {
  const unsigned mb = smem_addr(&st.mbar);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the warp's reads of the old contents first
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_addr(st.buf)), "l"(src), "r"(bytes), "r"(mb) : "memory");
}
// Wait for the phase `parity` of the stage's mbarrier, at most kStageSpin rounds; true when done.
__device__ __forceinline__ bool stage_wait(const VoxStage& st, unsigned parity) {
  const unsigned mb = smem_addr(&st.mbar);
  for (int it = 0; it < kStageSpin; ++it) {
    unsigned done;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done) : "r"(mb), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}

// The whole warp stages list entries [a0, a1) (absolute indices): one bulk copy of the range
// rounded out to 16 bytes, issued by lane 0, awaited by every lane. Returns the first staged
// entry, or -1 when the wait gave up (after waiting once more for the copy); the stage is then
// switched off and the warp reads the lists directly. Out of line: it runs once per 8 chunks.
static __device__ __noinline__ int stage_refill(VoxStage* st, const unsigned* vlist, unsigned a0, unsigned a1) {
  const int lane = threadIdx.x & 31;
  const unsigned g0 = a0 & ~3u, g1 = (a1 + 3u) & ~3u;
  __syncwarp();
  if (lane == 0) stage_issue(*st, vlist + g0, (g1 - g0) * 4u);
  __syncwarp();
  const unsigned par = st->phase;
  const bool done = __all_sync(kFull, stage_wait(*st, par));
  if (lane == 0) st->phase = par ^ 1u;
  if (!done) {
    stage_wait(*st, par);
    if (lane == 0) st->ok = 0;
  }
  __syncwarp();
  return done ? (int)g0 : -1;
}

// g(s) = erfc(alpha sqrt s)/sqrt s from the piecewise quintic table; pieces are found
// from the FP32 bits of s. Below the table (s < 0.25 A^2) the library erfc is used.
__device__ __forceinline__ double coul_table(const BoxDev& b, float s32, double s64) {
  const int k = (__float_as_int(s32) >> 17) - b.ctab_base;
  if (k < 0 || k >= b.ctab_n) {
    const double r = sqrt(s64);
    return erfc(b.alpha * r) / r;
  }
  const double2* c = reinterpret_cast<const double2*>(b.ctab + 8 * k);
  const double2 c01 = __ldg(c), c23 = __ldg(c + 1), c45 = __ldg(c + 2), c67 = __ldg(c + 3);
  const double t = (s64 - c01.x) * c01.y;
  return c23.x + t * (c23.y + t * (c45.x + t * (c45.y + t * (c67.x + t * c67.y))));
}

// Round to the nearest integer with two FP32 instructions (|x| < 2^22): adding
// 1.5*2^23 moves the fraction out of the mantissa. Differs from the reference's
// int-cast rounding only at exact half-cell ties, which lie beyond the cutoff.
__device__ __forceinline__ float rnd(float x) {
  return __fsub_rn(__fadd_rn(x, 12582912.0f), 12582912.0f);
}

// Minimum-image displacement on split coordinates: the image shift is applied to the
// hi part with the grid-exact cell (exact) and to the lo part with the remainder.
__device__ __forceinline__ void image_split(const BoxDev& b, float3& dh, float3& dl) {
  const float x = dh.x + dl.x, y = dh.y + dl.y, z = dh.z + dl.z;
  if (b.cubic) {
    const float nx = rnd(x * b.invf[0]), ny = rnd(y * b.invf[4]), nz = rnd(z * b.invf[8]);
    dh.x = __fmaf_rn(-nx, b.cell_hi[0], dh.x); dl.x = __fmaf_rn(-nx, b.cell_lo[0], dl.x);
    dh.y = __fmaf_rn(-ny, b.cell_hi[4], dh.y); dl.y = __fmaf_rn(-ny, b.cell_lo[4], dl.y);
    dh.z = __fmaf_rn(-nz, b.cell_hi[8], dh.z); dl.z = __fmaf_rn(-nz, b.cell_lo[8], dl.z);
  } else {
    const float nx = rnd(b.invf[0] * x + b.invf[3] * y + b.invf[6] * z);
    const float ny = rnd(b.invf[1] * x + b.invf[4] * y + b.invf[7] * z);
    const float nz = rnd(b.invf[2] * x + b.invf[5] * y + b.invf[8] * z);
    dh.x = __fmaf_rn(-nz, b.cell_hi[6], __fmaf_rn(-ny, b.cell_hi[3], __fmaf_rn(-nx, b.cell_hi[0], dh.x)));
    dh.y = __fmaf_rn(-nz, b.cell_hi[7], __fmaf_rn(-ny, b.cell_hi[4], __fmaf_rn(-nx, b.cell_hi[1], dh.y)));
    dh.z = __fmaf_rn(-nz, b.cell_hi[8], __fmaf_rn(-ny, b.cell_hi[5], __fmaf_rn(-nx, b.cell_hi[2], dh.z)));
    dl.x -= nx * b.cell_lo[0] + ny * b.cell_lo[3] + nz * b.cell_lo[6];
    dl.y -= nx * b.cell_lo[1] + ny * b.cell_lo[4] + nz * b.cell_lo[7];
    dl.z -= nx * b.cell_lo[2] + ny * b.cell_lo[5] + nz * b.cell_lo[8];
  }
}

// Screening test of one pair (true when it may lie inside a cutoff). FP64 form: the
// exact FP64 test. Mixed / FP32 forms: FP32 on the hi parts alone (16 bytes per
// atom), against a radius padded for the hi rounding.
__device__ __forceinline__ bool screen_hi(const BoxDev& b, float4 ah, const Bead& bd) {
  float x = ah.x - bd.h.x, y = ah.y - bd.h.y, z = ah.z - bd.h.z;
  if (b.cubic) {
    x = __fmaf_rn(-rnd(x * b.invf[0]), b.cellf[0], x);
    y = __fmaf_rn(-rnd(y * b.invf[4]), b.cellf[4], y);
    z = __fmaf_rn(-rnd(z * b.invf[8]), b.cellf[8], z);
  } else {
    const float nx = rnd(b.invf[0] * x + b.invf[3] * y + b.invf[6] * z);
    const float ny = rnd(b.invf[1] * x + b.invf[4] * y + b.invf[7] * z);
    const float nz = rnd(b.invf[2] * x + b.invf[5] * y + b.invf[8] * z);
    x -= nx * b.cellf[0] + ny * b.cellf[3] + nz * b.cellf[6];
    y -= nx * b.cellf[1] + ny * b.cellf[4] + nz * b.cellf[7];
    z -= nx * b.cellf[2] + ny * b.cellf[5] + nz * b.cellf[8];
  }
  return x * x + y * y + z * z < b.screen2;
}

template <int PREC, bool HOST>
__device__ __forceinline__ bool pair_screen(const BoxDev& b, int i, const Bead& bd) {
  if (PREC == GRX_FP64) {
    const double4 p = (HOST ? b.hpos64 : b.pos64)[i];
    double x = p.x - bd.x, y = p.y - bd.y, z = p.z - bd.z;
    pbc64(b, x, y, z);
    const double rr = x * x + y * y + z * z;
    return rr < b.cut_vdw2 || (!b.no_charges && rr < b.cut_coul2);
  } else {
    return screen_hi(b, HOST ? b.hrec[2 * i] : b.hi[i], bd);
  }
}

// 4 eps [(sigma^2/r^2)^6 - (sigma^2/r^2)^3] - shift in double-float (full molecules),
// used by the mixed form inside 1.1 sigma where FP32 rounding of the steep repulsion
// would exceed the error budget.
__device__ __forceinline__ df lj_df(const BoxDev& b, int row, df rr) {
  const float4 f = b.ffdf[row];
  const float2 sh = b.ffdf2[row];
  const df t = df_mul(rr, df{f.z, f.w});
  const df t3 = df_mul(df_mul(t, t), t);
  const df rri3 = df_recip(t3);
  const df term = df_mul(df{f.x, f.y}, df_mul(rri3, df_add_f(rri3, -1.0f)));
  return df_add(term, df{-sh.x, -sh.y});
}

// g(s) = erfc(alpha sqrt s)/sqrt s from the double-float table. The piece width is a
// power of two, so t = (s - s0)/width is formed exactly from the two halves of s.
__device__ __forceinline__ df coul_table_df(const BoxDev& b, df s) {
  const int k = (__float_as_int(s.hi) >> 17) - b.ctab_base;
  const float4* c = b.ctabf + 4 * k;
  const float4 c0 = __ldg(c), c1 = __ldg(c + 1), c2 = __ldg(c + 2), c3 = __ldg(c + 3);
  const df t = {__fmul_rn(__fsub_rn(s.hi, c0.x), c0.y), __fmul_rn(s.lo, c0.y)};
  // Over one piece the terms of order >= 2 are ~1e-4 of g, so they are summed in
  // FP32 (error ~1e-12 of g); the first two orders are kept in double-float.
  const float tail = __fmaf_rn(__fmaf_rn(__fmaf_rn(c3.x, t.hi, c2.z), t.hi, c2.x), t.hi, c1.z);
  const df p1 = df_add(df_mul_f(t, tail), df{c1.x, c1.y});
  return df_add(df_mul(p1, t), df{c0.z, c0.w});
}

// Cold paths of the mixed-precision pair evaluation, kept out of line so the inlined copies of
// pair_dense stay small: LJ inside 1.1 sigma (double-float), LJ with a non-unit scaling or the
// 12-6-4 form, and g(s) outside the Coulomb table's range.
static __device__ __noinline__ float2 lj_df_cold(const BoxDev& b, int row, float rhi, float rlo) {
  const df e = lj_df(b, row, df{rhi, rlo});
  return make_float2(e.hi, e.lo);
}
static __device__ __noinline__ double vdw64_cold(const BoxDev& b, int row, double rr, double scaling) {
  return vdw64(b, row, rr, scaling);
}
static __device__ __noinline__ double coul_g_cold(const BoxDev& b, double rr) {
  const double r = sqrt(rr);
  return erfc(b.alpha * r) / r;
}

// Accumulators of one lane: FP64 for the FP64 and FP32 forms, double-float for mixed.
template <int PREC> struct LaneAcc { double v = 0.0, r = 0.0; };
template <> struct LaneAcc<GRX_MIXED> { df v = {0.f, 0.f}, r = {0.f, 0.f}; };

template <int PREC> __device__ __forceinline__ double acc_value(const LaneAcc<PREC>& a, bool vdw) {
  if constexpr (PREC == GRX_MIXED) return vdw ? df_to(a.v) : df_to(a.r);
  else return vdw ? a.v : a.r;
}

// Dense evaluation of one screened pair: exact cutoff tests, LJ, real Coulomb,
// overlap flag (VDW_Coulomb.cu:1287-1322). `host`: atom i is a framework (host) atom, else a
// guest atom; the arrays are selected at run time so that a work item has one inlined copy
// of this evaluation for both kinds of atoms and for full and final batches (the hot code of
// a move then fits the instruction cache better).
template <int PREC>
__device__ __forceinline__ void pair_dense(const BoxDev& b, bool host, int i, const Bead& bd, LaneAcc<PREC>& acc,
                                           int& flag) {
  if constexpr (PREC == GRX_FP64) {
    const int row = (host ? b.hmeta : b.meta)[i].x * b.ntypes + bd.type;
    const double4 p = (host ? b.hpos64 : b.pos64)[i];
    double x = p.x - bd.x, y = p.y - bd.y, z = p.z - bd.z;
    pbc64(b, x, y, z);
    const double rr = x * x + y * y + z * z;
    if (rr < b.cut_vdw2) {
      const double e = vdw64(b, row, rr, (host ? b.hscale : b.scale)[i] * bd.scale);
      if (e > b.overlap) flag = 1;
      if (rr < 0.01) flag = 1;
      acc.v += e;
    }
    if (!b.no_charges && rr < b.cut_coul2) acc.r += coul64(b, p.w * bd.q, rr);
  } else {
    // host atoms from their records (one 32-byte sector: split position and charge, plus the
    // 2-byte type); guest atoms from the per-field arrays
    float4 ah, al;
    int ty;
    bool sc1;  // the atom's scale is 1
    float2 qa;
    if (host) {
      ah = b.hrec[2 * i];
      al = b.hrec[2 * i + 1];
      const unsigned t = b.htype[i];
      ty = (int)(t & 0x7fffu);
      sc1 = !(t & 0x8000u);
      qa = make_float2(ah.w, al.w);
    } else {
      ah = b.hi[i];
      al = b.lo[i];
      ty = b.meta[i].x;
      sc1 = al.w == 1.0f;
      qa = b.qdf[i];
    }
    const int row = ty * b.ntypes + bd.type;
    float3 dh = make_float3(ah.x - bd.h.x, ah.y - bd.h.y, ah.z - bd.h.z);
    float3 dl = make_float3(al.x - bd.l.x, al.y - bd.l.y, al.z - bd.l.z);
    image_split(b, dh, dl);
    if constexpr (PREC == GRX_MIXED) {
      const df s = df_norm2_split(dh, dl);
      if (df_lt(s, df{b.cut_vdw2_df.x, b.cut_vdw2_df.y})) {
        const float4 f = b.ff32[row];
        const bool unit = sc1 && bd.unit && !b.use_1264;
        df e;
        if (unit && s.hi > f.w) e = df{vdw32(f, s.hi), 0.0f};
        else if (unit) {
          const float2 c = lj_df_cold(b, row, s.hi, s.lo);
          e = df{c.x, c.y};
        }
        else e = df_from(vdw64_cold(b, row, df_to(s), (host ? b.hscale : b.scale)[i] * bd.scale));
        if (e.hi > b.overlapf) flag = 1;
        if (s.hi < 0.01f) flag = 1;
        acc.v = df_add(acc.v, e);
      }
      if (!b.no_charges && df_lt(s, df{b.cut_coul2_df.x, b.cut_coul2_df.y})) {
        df g;
        const int k = (__float_as_int(s.hi) >> 17) - b.ctab_base;
        if (k >= 0 && k < b.ctab_n) g = coul_table_df(b, s);
        else g = df_from(coul_g_cold(b, df_to(s)));
        acc.r = df_add(acc.r, df_mul(g, df{qa.x, qa.y}));  // prefactor * q_bead applied once per item
      }
    } else {  // GRX_FP32
      const float fx = dh.x + dl.x, fy = dh.y + dl.y, fz = dh.z + dl.z;
      const float rr32 = fx * fx + fy * fy + fz * fz;
      if (rr32 < b.cut_vdw2f) {
        const float sc = (host ? (sc1 ? 1.0f : (float)b.hscale[i]) : al.w) * (float)bd.scale;
        float e;
        if (sc == 1.0f && !b.use_1264) e = vdw32(b.ff32[row], rr32);
        else e = (float)vdw64(b, row, (double)rr32, (double)sc);
        if (e > b.overlapf) flag = 1;
        if (rr32 < 0.01f) flag = 1;
        acc.v += (double)e;
      }
      if (!b.no_charges && rr32 < b.cut_coul2f) acc.r += (double)coul32(b, ah.w * (float)bd.q, rr32);
    }
  }
}

// One work item: bead `bd` against host units [t0, t1) (tiles, or with VOX 32-entry chunks
// of the bead's voxel list) and, when g1 > g0, the live guest atoms [g0, g1). hacc / gacc =
// {vdw, real} of the host and the guest atoms (valid on every lane, summed later); flag is
// per lane.
//
// A generator step screens up to 32 candidates of the current phase (host, then guests) and
// appends the ones inside the screening radius to the warp's ring buffer. Whenever 32 are
// queued, or the phase has no candidates left, the warp evaluates the next batch at the one
// dense site; a phase ends with its buffer drained. Batches are the queue order, so the sums
// do not depend on how the candidates were produced.
//
// Early overlap rejection: with `dead` (the bead's trial's flag in shared memory, null
// when the trial must be evaluated in full) the warp stops as soon as the trial is known
// to overlap: after a dense batch that set an overlap flag (it then marks the trial), or
// when another warp has marked it. An overlapping trial takes no part in the Rosenbluth
// weight, and its flag is still raised by the warp that found the overlap, so the trial
// flags (and every used energy) are the same as without the early exit.
template <int PREC, bool VOX>
__device__ __forceinline__ void warp_item(const BoxDev& b, const Bead& bd, int t0, int t1, int g0, int g1,
                                          int component, int newmol, int excl_comp, int excl_mol, int* q,
                                          LaneAcc<PREC>& hacc, LaneAcc<PREC>& gacc, int& flag,
                                          volatile int* dead, VoxStage* stage) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  unsigned head = 0, tail = 0;
  // the trial is dead (checked by lane 0, the answer shared, so the warp stays converged)
  auto is_dead = [&]() { return dead && __shfl_sync(kFull, lane == 0 ? *dead : 0, 0) > 0; };
  // after a dense batch: an overlap found by this warp kills the trial
  auto found_overlap = [&]() {
    if (!dead || !__any_sync(kFull, flag != 0)) return false;
    if (lane == 0) *dead = 1;
    return true;
  };
  auto push = [&](bool in, int i) {
    const unsigned m = __ballot_sync(kFull, in);
    if (in) q[(tail + __popc(m & lt)) & (kQueue - 1)] = i;
    tail += __popc(m);
  };
  const float bx = bd.h.x + bd.l.x, by = bd.h.y + bd.l.y, bz = bd.h.z + bd.l.z;

  // host generator state. VOX: chunks [ch, cend) of the bead's voxel list; entries below
  // vm.y are inside the cutoff for every bead of the voxel (queued unscreened), the others are
  // screened at the stored image against the bead wrapped into the home cell. Tiles: groups of
  // 32 tiles from `base`, culled one per lane; `mask` holds the group's surviving tiles.
  int ch = t0, cend = t0;
  int win_off = 0, win_end = t0;  // staged list window: entry j at buf[j + win_off], chunks below win_end
  if (stage && !stage->ok) stage = nullptr;
  int4 vm = make_int4(0, 0, 0, 0);
  float wx = 0.f, wy = 0.f, wz = 0.f;
  bool hcheck = false;
  int base = t0;
  unsigned mask = 0;
  float sx = 0.f, sy = 0.f, sz = 0.f;  // this lane's tile: image shift of the bead
  bool one_image = false;
  int4 trl = make_int4(0, 0, -1, 0);   // this lane's tile range, shuffled to the warp below
  if constexpr (VOX) {
    if (t1 > t0) {
      const float fx = b.invf[0] * bx + b.invf[3] * by + b.invf[6] * bz;
      const float fy = b.invf[1] * bx + b.invf[4] * by + b.invf[7] * bz;
      const float fz = b.invf[2] * bx + b.invf[5] * by + b.invf[8] * bz;
      const float mx = floorf(fx), my = floorf(fy), mz = floorf(fz);
      const int ix = min(b.vn[0] - 1, max(0, (int)((fx - mx) * (float)b.vn[0])));
      const int iy = min(b.vn[1] - 1, max(0, (int)((fy - my) * (float)b.vn[1])));
      const int iz = min(b.vn[2] - 1, max(0, (int)((fz - mz) * (float)b.vn[2])));
      vm = b.vmeta[(iz * b.vn[1] + iy) * b.vn[0] + ix];
      wx = bd.h.x - (mx * b.cellf[0] + my * b.cellf[3] + mz * b.cellf[6]);
      wy = bd.h.y - (mx * b.cellf[1] + my * b.cellf[4] + mz * b.cellf[7]);
      wz = bd.h.z - (mx * b.cellf[2] + my * b.cellf[5] + mz * b.cellf[8]);
      hcheck = component < b.nhost || (excl_comp >= 0 && excl_comp < b.nhost);
      cend = min(t1, (vm.z + 31) >> 5);
    }
  }
  // one host step: screen the next chunk / surviving tile; false when none is left
  auto host_step = [&]() -> bool {
    if constexpr (VOX) {
      if (ch >= cend) return false;
      if (stage && ch >= win_end) {  // stage chunks [ch, ch + 8) of the list (clipped to cend)
        const int g0 = stage_refill(stage, b.vlist, (unsigned)vm.x + 32u * (unsigned)ch,
                                    (unsigned)vm.x + (unsigned)min(32 * min(ch + kStageChunks, cend), vm.z));
        if (g0 >= 0) {
          win_off = vm.x - g0;
          win_end = min(ch + kStageChunks, cend);
        } else {
          stage = nullptr;
        }
      }
      const int j = (ch << 5) + lane;
      ++ch;
      bool in = false;
      int i = 0;
      if (j < vm.z) {
        const unsigned w = stage ? stage->buf[j + win_off] : __ldg(b.vlist + vm.x + j);
        i = (int)(w & 0xFFFFFu);
        if (j < vm.y) {
          in = true;
        } else if (PREC == GRX_FP64) {
          in = pair_screen<PREC, true>(b, i, bd);
        } else {
          const float nx = (float)((int)((w >> 20) & 7u) - 4), ny = (float)((int)((w >> 23) & 7u) - 4),
                      nz = (float)((int)((w >> 26) & 7u) - 4);
          const float4 ah = b.hrec[2 * i];
          const float x = ah.x - wx - (nx * b.cellf[0] + ny * b.cellf[3] + nz * b.cellf[6]);
          const float y = ah.y - wy - (nx * b.cellf[1] + ny * b.cellf[4] + nz * b.cellf[7]);
          const float z = ah.z - wz - (nx * b.cellf[2] + ny * b.cellf[5] + nz * b.cellf[8]);
          in = x * x + y * y + z * z < b.screen2;
        }
        if (in && hcheck) {  // a host component is moved or excluded: skip its molecule
          int tz = 0;
          while (tz + 1 < b.nhost && i >= b.comp_off[tz + 1]) ++tz;
          const int mol = b.hmeta[i].y;
          if ((tz == excl_comp && mol == excl_mol) || (tz == component && mol == newmol)) in = false;
        }
      }
      push(in, i);
      return true;
    } else {
      // Tiles are tested 32 at a time, one per lane; survivors are then screened one tile at
      // a time by the whole warp. When a tile lies inside one periodic image of the bead
      // (stored positions compact, the tile sphere clear of the rounding boundaries), the
      // image shift is applied once to the bead instead of per atom.
      while (mask == 0) {
        if (base >= t1) return false;
        const int tl = base + lane;
        base += 32;
        bool pass = tl < t1;
        sx = sy = sz = 0.f;
        one_image = false;
        trl = make_int4(0, 0, -1, 0);
        if (pass) trl = b.tile_r[tl];
        if (pass && b.cull) {
          const float4 tc = b.tile_c[2 * tl];
          float dx = tc.x - bx, dy = tc.y - by, dz = tc.z - bz;
          const float lim = b.cull_r + tc.w;
          const float m = tc.w + 1e-2f;
          if (b.cubic) {
            // Bounding box of the tile at the centre's rounded image. Per axis the distance to
            // the box bounds every atom's rounded-image distance from below: an atom whose
            // rounding differs from the centre's lies at least half a cell minus the half
            // extent away on that axis.
            const float4 th = b.tile_c[2 * tl + 1];
            const float nx = rnd(dx * b.invf[0]), ny = rnd(dy * b.invf[4]), nz = rnd(dz * b.invf[8]);
            dx = __fmaf_rn(-nx, b.cellf[0], dx);
            dy = __fmaf_rn(-ny, b.cellf[4], dy);
            dz = __fmaf_rn(-nz, b.cellf[8], dz);
            const float qx = fmaxf(fabsf(dx) - th.x, 0.f), qy = fmaxf(fabsf(dy) - th.y, 0.f),
                        qz = fmaxf(fabsf(dz) - th.z, 0.f);
            pass = qx * qx + qy * qy + qz * qz <= b.cull_r * b.cull_r;
            one_image = trl.w != 0 && fabsf(dx) + th.x + 1e-2f < 0.5f * b.cellf[0] &&
                        fabsf(dy) + th.y + 1e-2f < 0.5f * b.cellf[4] && fabsf(dz) + th.z + 1e-2f < 0.5f * b.cellf[8];
            sx = nx * b.cell_hi[0]; sy = ny * b.cell_hi[4]; sz = nz * b.cell_hi[8];
          } else {
            const float fx = b.invf[0] * dx + b.invf[3] * dy + b.invf[6] * dz;
            const float fy = b.invf[1] * dx + b.invf[4] * dy + b.invf[7] * dz;
            const float fz = b.invf[2] * dx + b.invf[5] * dy + b.invf[8] * dz;
            const float nx = rnd(fx), ny = rnd(fy), nz = rnd(fz);
            sx = nx * b.cellf[0] + ny * b.cellf[3] + nz * b.cellf[6];
            sy = nx * b.cellf[1] + ny * b.cellf[4] + nz * b.cellf[7];
            sz = nx * b.cellf[2] + ny * b.cellf[5] + nz * b.cellf[8];
            dx -= sx; dy -= sy; dz -= sz;
            const float d2 = dx * dx + dy * dy + dz * dz;
            const float rx = fabsf(fx - nx), ry = fabsf(fy - ny), rz = fabsf(fz - nz);
            if (d2 <= b.half_wmin2) {
              pass = d2 <= lim * lim;
            } else {
              const float lb = fmaxf(fmaxf(rx * b.wperp[0], ry * b.wperp[1]), rz * b.wperp[2]);
              pass = lb - 1e-3f <= lim;
            }
            one_image = trl.w != 0 && rx + m / b.wperp[0] < 0.5f - 1e-4f &&
                        ry + m / b.wperp[1] < 0.5f - 1e-4f && rz + m / b.wperp[2] < 0.5f - 1e-4f;
          }
        }
        mask = __ballot_sync(kFull, pass);
      }
      const int src = __ffs(mask) - 1;
      mask &= mask - 1;
      const int i = __shfl_sync(kFull, trl.x, src) + lane, tz = __shfl_sync(kFull, trl.z, src);
      const bool oi = __shfl_sync(kFull, one_image, src);
      const float tsx = __shfl_sync(kFull, sx, src), tsy = __shfl_sync(kFull, sy, src),
                  tsz = __shfl_sync(kFull, sz, src);
      bool in = false;
      if (i < __shfl_sync(kFull, trl.y, src)) {
        bool skip = false;
        if (tz == component || tz == excl_comp) {
          const int mol = b.hmeta[i].y;
          skip = (tz == excl_comp && mol == excl_mol) || (tz == component && mol == newmol);
        }
        if (!skip) {
          if (PREC != GRX_FP64 && oi) {
            const float4 ah = b.hrec[2 * i];
            const float x = ah.x - (bd.h.x + tsx);
            const float y = ah.y - (bd.h.y + tsy);
            const float z = ah.z - (bd.h.z + tsz);
            in = x * x + y * y + z * z < b.screen2;
          } else {
            in = pair_screen<PREC, true>(b, i, bd);
          }
        }
      }
      push(in, i);
      return true;
    }
  };
  // one batch at the phase's dense site: 32 queued pairs, or the final ones when the phase has
  // no candidates left (got false); true when the warp must stop (the trial overlaps)
  auto batch = [&](bool host, bool got, LaneAcc<PREC>& acc) -> bool {
    const unsigned avail = tail - head;
    if (avail >= 32u || (!got && avail > 0u)) {
      const int n = (int)min(avail, 32u);
      __syncwarp();
      const int j = q[(head + lane) & (kQueue - 1)];  // entries past n are stale and unused
      __syncwarp();
      if (lane < n) pair_dense<PREC>(b, host, j, bd, acc, flag);
      head += (unsigned)n;
      if (found_overlap()) return true;
    }
    return false;
  };
  if (t1 > t0) {
    for (;;) {
      if (is_dead()) return;
      const bool got = host_step();
      if (batch(true, got, hacc)) return;
      if (!got && tail == head) break;
    }
  }
  if (g1 <= g0) return;
  head = tail = 0;
  // guest atoms [g0, g1) of the concatenated adsorbate components: component gc, its atoms
  // [gi, ghi) still to screen (indices within the component), gbase = the first concatenated
  // guest index after gc
  int gc = b.nhost, gbase = 0, gi = 0, ghi = 0;
  for (;;) {
    if (is_dead()) return;
    bool got = false;
    while (gi >= ghi && gc < b.ncomp && gbase < g1) {  // next component overlapping [g0, g1)
      const int n = b.comp_size[gc];
      gi = max(g0 - gbase, 0);
      ghi = min(g1 - gbase, n);
      gbase += n;
      ++gc;
    }
    if (gi < ghi) {
      const int c = gc - 1;
      const int i = b.comp_off[c] + gi + lane;
      bool in = false;
      if (gi + lane < ghi) {
        bool skip = false;
        if (c == component || c == excl_comp) {
          const int mol = b.meta[i].y;
          skip = (c == excl_comp && mol == excl_mol) || (c == component && mol == newmol);
        }
        if (!skip) in = pair_screen<PREC, false>(b, i, bd);
      }
      gi += 32;
      push(in, i);
      got = true;
    }
    if (batch(false, got, gacc)) return;
    if (!got && tail == head) return;
  }
}

// Fixed-order warp sums (lane 0 receives the total). The double-float form keeps the
// reduction on the FP32 pipe; one conversion to FP64 happens on lane 0 only.
__device__ __forceinline__ double warp_sum(double x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(kFull, x, o);
  return x;
}

// Out of line: called once per work item and per Ewald delta, so one copy serves them all.
static __device__ __noinline__ float2 warp_sum_df_out(float hi, float lo) {
  df x = {hi, lo};
  for (int o = 16; o > 0; o >>= 1) {
    const df y = {__shfl_down_sync(kFull, x.hi, o), __shfl_down_sync(kFull, x.lo, o)};
    x = df_add(x, y);
  }
  return make_float2(x.hi, x.lo);
}

__device__ __forceinline__ df warp_sum_df(df x) {
  const float2 r = warp_sum_df_out(x.hi, x.lo);
  return df{r.x, r.y};
}

template <int PREC>
__device__ __forceinline__ void warp_store(const LaneAcc<PREC>& h, const LaneAcc<PREC>& g, double* out4, df pq,
                                           bool with_guests) {
  const int lane = threadIdx.x & 31;
  if constexpr (PREC == GRX_MIXED) {
    // the mixed form accumulates sum q_atom * g(r); the bead factor prefactor*q_bead
    // is applied here, once
    const df a = warp_sum_df(h.v), c = warp_sum_df(h.r);
    df d = {0.f, 0.f}, e = {0.f, 0.f};
    if (with_guests) { d = warp_sum_df(g.v); e = warp_sum_df(g.r); }
    if (lane == 0) {  // stored as float pairs in the 8-byte slots (item_get converts)
      float2* o = reinterpret_cast<float2*>(out4);
      const df cq = df_mul(c, pq), eq = df_mul(e, pq);
      o[0] = make_float2(a.hi, a.lo);
      o[1] = make_float2(cq.hi, cq.lo);
      o[2] = make_float2(d.hi, d.lo);
      o[3] = make_float2(eq.hi, eq.lo);
    }
  } else {
    const double a = warp_sum(h.v), c = warp_sum(h.r), d = warp_sum(g.v), e = warp_sum(g.r);
    if (lane == 0) { out4[0] = a; out4[1] = c; out4[2] = d; out4[3] = e; }
  }
}

// Live adsorbate atoms of the box, and the 32-atom work units a bead pass covers
// (host tiles plus guest atoms in groups of 32).
__device__ __forceinline__ int guest_atoms(const BoxDev& b) {
  int g = 0;
  for (int c = b.nhost; c < b.ncomp; ++c) g += b.comp_size[c];
  return g;
}
__device__ __forceinline__ int host_units(const BoxDev& b) { return b.vox ? b.vchunks : b.ntiles; }
__device__ __forceinline__ int work_tiles(const BoxDev& b) { return host_units(b) + (guest_atoms(b) + 31) / 32; }

// Work split of one bead pass. The flattened space of nb beads x nu work units (host
// tiles, then guest atoms in groups of 32) is cut into `items` contiguous ranges of equal
// size, so every warp gets the same share whatever nb is. An item that crosses a bead
// boundary stores one partial per bead it touches, in slot item + bead; these slots are
// distinct (a later item cannot reach an earlier bead), so a pass uses at most
// items + nb - 1 slots.
struct PassSplit {
  unsigned nu, items, q, r;  // units per bead, items, and T = items * q + r with T = nb * nu
  __device__ __forceinline__ void range(unsigned item, unsigned& lo, unsigned& hi) const {
    lo = item * q + min(item, r);
    hi = lo + q + (item < r ? 1u : 0u);
  }
  __device__ __forceinline__ unsigned item_of(unsigned p) const {  // the item holding unit p
    const unsigned big = r * (q + 1);
    return p < big ? p / (q + 1) : r + (p - big) / q;
  }
};

// Items of a pass: mult per warp, never more than the units of the pass (at least 1).
__device__ __forceinline__ PassSplit pass_split(const BoxDev& b, int nb, int nwarps, int mult) {
  PassSplit s;
  s.nu = (unsigned)work_tiles(b);
  const unsigned T = (unsigned)nb * s.nu;
  s.items = max(1u, min((unsigned)(mult * nwarps), T));
  s.q = T / s.items;
  s.r = T - s.q * s.items;
  return s;
}

constexpr int kMaxItems = 320;

// One pass of `nb` beads (shared memory) over every atom by a whole block. Items
// [item0, item1) (all of them when item1 < 0) are taken dynamically by warps; the partial
// of bead `bead` within item `item` lands in ipart[(item + bead)*4 + q] and
// iflag[item + bead]. Caller syncs before reading them.
template <int PREC, bool VOX>
__device__ __noinline__ void block_bead_pass_impl(const BoxDev& b, const Bead* beads, int nb, int component,
                                                     int newmol, int excl_comp, int excl_mol, int* qbuf,
                                                     double* ipart, int* iflag, int* counter, PassSplit sp,
                                                     int item0, int item1, int chain, int* dead,
                                                     VoxStage* stages) {
  if (item1 < 0) item1 = (int)sp.items;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int* q = qbuf + warp * kQueue;
  const int nt = VOX ? b.vchunks : b.ntiles;
  const int ng = guest_atoms(b);
  if (sp.nu == 0) {  // nothing to interact with: zero partials, one item per bead slot
    for (int k = threadIdx.x; k < nb * 4; k += blockDim.x) ipart[k] = 0.0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) iflag[k] = 0;
    return;
  }
  for (;;) {
    int item = 0;
    if (lane == 0) item = item0 + atomicAdd(counter, 1);
    item = __shfl_sync(kFull, item, 0);
    if (item >= item1) break;
    unsigned lo, hi;
    sp.range((unsigned)item, lo, hi);
    while (lo < hi) {
      const int bead = (int)(lo / sp.nu);
      const int u0 = (int)(lo - (unsigned)bead * sp.nu);
      const int u1 = (int)min(sp.nu, (unsigned)u0 + (hi - lo));
      // only the ranges reaching past the host tiles touch guest atoms
      const int t0 = min(u0, nt), t1 = min(u1, nt);
      const int g0 = min(32 * max(u0 - nt, 0), ng), g1 = min(32 * max(u1 - nt, 0), ng);
      // the bead is read from shared memory where it is used (fewer live registers around
      // the inlined dense evaluations: no spills in either pass)
      const Bead& bd = beads[bead];
      LaneAcc<PREC> hacc, gacc;
      int flag = 0;
      // trials of `chain` beads; dead[t] < 0: evaluated in full, else the early-exit flag
      volatile int* dt = nullptr;
      if (dead && dead[bead / chain] >= 0) dt = dead + bead / chain;
      warp_item<PREC, VOX>(b, bd, t0, t1, g0, g1, component, newmol, excl_comp, excl_mol, q, hacc, gacc, flag, dt,
                           stages ? stages + warp : nullptr);
      const unsigned fm = __ballot_sync(kFull, flag != 0);
      warp_store<PREC>(hacc, gacc, ipart + (item + bead) * 4, df{bd.pq.x, bd.pq.y}, g1 > g0);
      if (lane == 0) iflag[item + bead] = fm ? 1 : 0;
      lo += (unsigned)(u1 - u0);
    }
  }
}

// The pass through voxel lists or through tiles: two instantiations, so each keeps its own
// register allocation (the box decides, uniformly for the whole block).
// dead: per trial of `chain` beads, 0 for early overlap rejection, -1 to evaluate the trial
// in full (set by the caller before the pass; null: every trial in full).
template <int PREC>
__device__ __forceinline__ void block_bead_pass(const BoxDev& b, const Bead* beads, int nb, int component, int newmol,
                                                int excl_comp, int excl_mol, int* qbuf, double* ipart, int* iflag,
                                                int* counter, PassSplit sp, int item0 = 0, int item1 = -1,
                                                int chain = 1, int* dead = nullptr, VoxStage* stages = nullptr) {
  if (b.vox)
    block_bead_pass_impl<PREC, true>(b, beads, nb, component, newmol, excl_comp, excl_mol, qbuf, ipart, iflag,
                                     counter, sp, item0, item1, chain, dead, stages);
  else
    block_bead_pass_impl<PREC, false>(b, beads, nb, component, newmol, excl_comp, excl_mol, qbuf, ipart, iflag,
                                      counter, sp, item0, item1, chain, dead, nullptr);
}

// ---------------------------------------------------------------- thread-block clusters
// A cluster of CTAs may share one chain: each CTA evaluates a contiguous share of a pass's
// items and writes its partial slots into every peer's shared memory (PTX mapa + generic
// stores), so all CTAs reduce identical slots in identical order. barrier.cluster with
// release / acquire semantics orders those stores and the CTAs' global writes.
__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
template <class T>
__device__ __forceinline__ T* cluster_map(T* p, unsigned rank) {  // the same shared variable in CTA `rank`
  uint64_t out;
  asm volatile("mapa.u64 %0, %1, %2;" : "=l"(out) : "l"(reinterpret_cast<uint64_t>(p)), "r"(rank));
  return reinterpret_cast<T*>(out);
}

// Items of a pass for CTA `rank` of a CL-CTA cluster: [i0, i1), contiguous.
__device__ __forceinline__ void cluster_items(const PassSplit& sp, int cl, unsigned rank, int& i0, int& i1) {
  const unsigned per = (sp.items + (unsigned)cl - 1u) / (unsigned)cl;
  i0 = (int)min(sp.items, rank * per);
  i1 = (int)min(sp.items, (unsigned)i0 + per);
}

// Active k vectors of CTA `rank` of a CL-CTA cluster: [k0, k1), contiguous.
__device__ __forceinline__ void cluster_k_range(int nact, int cl, unsigned rank, int& k0, int& k1) {
  const int per = (nact + cl - 1) / cl;
  k0 = min(nact, (int)rank * per);
  k1 = min(nact, k0 + per);
}

// Item partials: FP64 in the FP64 / FP32 forms, a float pair in the mixed form.
template <int PREC>
__device__ __forceinline__ double item_get(const double* ipart, int idx) {
  if constexpr (PREC == GRX_MIXED) {
    const float2 v = reinterpret_cast<const float2*>(ipart)[idx];
    return (double)v.x + (double)v.y;
  } else {
    return ipart[idx];
  }
}

// Slots of bead `bead`: [first, last] (slot = item + bead), in unit order.
__device__ __forceinline__ void bead_slots(const PassSplit& sp, int bead, int& first, int& last) {
  if (sp.nu == 0) { first = last = bead; return; }
  const unsigned p0 = (unsigned)bead * sp.nu;
  first = (int)sp.item_of(p0) + bead;
  last = (int)sp.item_of(p0 + sp.nu - 1) + bead;
}

// Per-trial sums of one pass: trial t = beads [t*chain, (t+1)*chain), partials in order.
template <int PREC>
__device__ __forceinline__ void reduce_items(const double* ipart, const int* iflag, int ntr, int chain,
                                             const PassSplit& sp, double* te, int* tflag) {
  for (int w = threadIdx.x; w < ntr * 4; w += blockDim.x) {
    const int t = w >> 2, k = w & 3;
    int f = 0;
    if constexpr (PREC == GRX_MIXED) {
      df s = {0.f, 0.f};
#pragma unroll 1
      for (int a = 0; a < chain; ++a) {
        int s0, s1;
        bead_slots(sp, t * chain + a, s0, s1);
#pragma unroll 1
        for (int c = s0; c <= s1; ++c) {
          const float2 v = reinterpret_cast<const float2*>(ipart)[c * 4 + k];
          s = df_add(s, df{v.x, v.y});
          f |= iflag[c];
        }
      }
      te[4 * t + k] = df_to(s);
    } else {
      double s = 0.0;
#pragma unroll 1
      for (int a = 0; a < chain; ++a) {
        int s0, s1;
        bead_slots(sp, t * chain + a, s0, s1);
#pragma unroll 1
        for (int c = s0; c <= s1; ++c) {
          s += ipart[c * 4 + k];
          f |= iflag[c];
        }
      }
      te[4 * t + k] = s;
    }
    if (k == 0) tflag[t] = f;
  }
}

// Trial energies of one bead per block, the launch behind grx_trial_energies and
// grx_trial_energies_noalloc (both entry points run this one kernel, so they give the
// same sums); per-bead sums go to part[bead][4] and the overlap flag to flags[bead].
template <int PREC>
__global__ void __launch_bounds__(GRX_THREADS) trial_bead_kernel(BoxDev b, const Bead* beads, int component,
                                                                 int newmol, int excl_comp, int excl_mol,
                                                                 double* part, int* flags) {
  __shared__ double ipart[kMaxItems * 4];
  __shared__ int iflag[kMaxItems];
  __shared__ int qbuf[(GRX_THREADS / 32) * kQueue];
  __shared__ int counter;
  if (threadIdx.x == 0) counter = 0;
  __syncthreads();
  const PassSplit sp = pass_split(b, 1, GRX_THREADS / 32, 4);
  const int nch = (int)sp.items;  // one bead: slot = item
  block_bead_pass<PREC>(b, beads + blockIdx.x, 1, component, newmol, excl_comp, excl_mol, qbuf, ipart, iflag,
                        &counter, sp);
  __syncthreads();
  if (threadIdx.x < 4) {
    double s = 0.0;
    for (int c = 0; c < nch; ++c) s += item_get<PREC>(ipart, c * 4 + threadIdx.x);
    part[blockIdx.x * 4 + threadIdx.x] = s;
  }
  if (threadIdx.x == 0) {
    int f = 0;
    for (int c = 0; c < nch; ++c) f |= iflag[c];
    flags[blockIdx.x] = f;
  }
}

}  // namespace grx
