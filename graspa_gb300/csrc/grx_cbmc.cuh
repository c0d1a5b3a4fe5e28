// grx_cbmc.cuh -- block-level CBMC stages shared by the Widom and GCMC kernels.
//
// Every function here is called by all threads of a block (NW warps) with the same
// arguments; each ends with the block synchronised and its results in the
// shared-memory workspace CbmcWork<NW>. The stages restate gRASPA's CBMC move pieces:
//   gen_first_trials  get_random_trial_position      mc_widom.h:122-213
//   gen_orientations  get_random_trial_orientation   mc_widom.h:215-303
//   trial_pass        Calculate_Multiple_Trial_Energy_VDWReal + host sums
//                     (VDW_Coulomb.cu:1183-1352, mc_widom.h:42-87)
//   step_weight       SelectTrialPosition + CBMC_FirstBead_Finish / chain finish
//                     (mc_widom.h:14-39, 305-383, 568-611)
//   ewald_move        Initialize_WaveVector_General + Fourier_Ewald_Diff
//                     (Ewald_Energy_Functions.h:162-185, 280-397)
#pragma once

#include "grx_warp.cuh"

namespace grx {

constexpr int kMaxTrials = 64;
constexpr int kMolWork = 32;      // atoms of one molecule held in shared memory
constexpr int kCbmcBeads = 128;   // trial beads of one pass
constexpr int kCbmcMaxMult = 8;   // items per warp of a bead pass, at most
constexpr int kEwRowBytes = 96 * 1024;  // largest (kx, ky) row-product table of a move
constexpr int kEwRowReuse = 16;         // active k per row at which the row products pay

// Entries of the row-product table of the double-float Ewald delta: one per (kx, ky) row and
// moved atom. The host enables it for a box (BoxDev::ew_rows) when the table for 2 * molsize
// atoms (a translation) fits kEwRowBytes and the box has at least kEwRowReuse active k per
// row, and sizes dynamic shared memory for it; the kernels read the flag.
__host__ __device__ __forceinline__ int ew_rows(const int* kmax) { return (kmax[0] + 1) * (2 * kmax[1] + 1); }
__host__ __device__ __forceinline__ bool ew_rows_worth(const int* kmax, int nact, int molsize) {
  return (size_t)ew_rows(kmax) * 2 * molsize * 16 <= (size_t)kEwRowBytes && nact >= kEwRowReuse * ew_rows(kmax);
}

// Workspace of a block of NW warps. A pass uses at most items + beads - 1 partial
// slots, items = mult * NW.
template <int NW>
struct CbmcWork {
  static constexpr int kItems = kCbmcBeads + kCbmcMaxMult * NW;
  Bead beads[kCbmcBeads];
  double ipart[kItems * 4];
  int iflag[kItems];
  VoxStage vst[NW];       // per warp: voxel-list staging buffer and its mbarrier
  int tdead[kCbmcBeads];  // per trial of a pass: early overlap rejection flag (-1: evaluated in full)
  int qbuf[NW * kQueue];
  double te[kMaxTrials * 4];
  int tflag[kMaxTrials];
  double sel_ws[kMaxTrials], sel_wa[kMaxTrials];
  // moved atoms of the Ewald delta: [0, n_old) leave (charge stored negated),
  // [n_old, n_old + n_new) arrive
  double mx[2 * kMolWork], my[2 * kMolWork], mz[2 * kMolWork], mq[2 * kMolWork];
  double sbuf[32];
  double ewx[8][2];  // per-CTA Fourier partials {same, cross} of a cluster
  double wsum[2][NW];
  float2 qd[2 * kMolWork];
  int counter;
  long long cfg;    // trial configurations evaluated since the caller last cleared it
  long long cbeads; // their beads
  int ok;       // step constructed
  int sel;      // chosen (or retraced) trial index
  int nok;      // trials without overlap
  double w;     // averaged weight of the step
  double wraw;  // unaveraged weight sum of the step (reinsertion StoredR)
};

// ---------------------------------------------------------------- trials
// First-bead trial positions: Cell diagonal x Philox uniforms (mc_widom.h:133-139);
// with `retrace`, trial 0 is the existing bead (deletion, mc_widom.h:141-156).
template <class WK>
__device__ __noinline__ void gen_first_trials(const BoxDev& b, WK& W, uint64_t seed, uint32_t stream,
                                                 uint64_t move, int nt, double q, double scale, int type,
                                                 bool retrace, double ox, double oy, double oz) {
  for (int t = threadIdx.x; t < nt; t += blockDim.x) {
    if (retrace && t == 0) {
      make_bead(W.beads[0], ox, oy, oz, q, scale, type, b.prefactor);
    } else {
      uint32_t r[4];
      draw4_dev(seed, stream, move, SLOT_FIRST + t, r);
      make_bead(W.beads[t], b.cell[0] * u01(r[0]), b.cell[4] * u01(r[1]), b.cell[8] * u01(r[2]), q, scale, type,
                b.prefactor);
    }
  }
  __syncthreads();
}

// Rotate_Quaternions (mc_utilities.h:423-457): uniform rotation from (u, v, w).
__device__ __forceinline__ void rotate_quaternion(double& x, double& y, double& z, double u, double v,
                                                  double w) {
  const double pi = 3.14159265358979323846;
  double s1, c1, s2, c2;
  sincos(2 * pi * v, &s1, &c1);
  sincos(2 * pi * w, &s2, &c2);
  const double q0 = sqrt(1 - u) * s1;
  const double q1 = sqrt(1 - u) * c1;
  const double q2 = sqrt(u) * s2;
  const double q3 = sqrt(u) * c2;
  const double a01 = q0 * q1, a02 = q0 * q2, a03 = q0 * q3;
  const double a11 = q1 * q1, a12 = q1 * q2, a13 = q1 * q3;
  const double a22 = q2 * q2, a23 = q2 * q3, a33 = q3 * q3;
  const double r0 = 1.0 - 2.0 * (a22 + a33), r1 = 2.0 * (a12 - a03), r2 = 2.0 * (a13 + a02);
  const double r3 = 2.0 * (a12 + a03), r4 = 1.0 - 2.0 * (a11 + a33), r5 = 2.0 * (a23 - a01);
  const double r6 = 2.0 * (a13 - a02), r7 = 2.0 * (a23 + a01), r8 = 1.0 - 2.0 * (a11 + a22);
  const double nx = x * r0 + y * r1 + z * r2;
  const double ny = x * r3 + y * r4 + z * r5;
  const double nz = x * r6 + y * r7 + z * r8;
  x = nx; y = ny; z = nz;
}

// Trial orientations about the chosen first bead (fx, fy, fz): the vectors from the
// component's slot-0 atom to its chain atoms, rotated by Philox quaternions. With
// `retrace`, orientation 0 is the existing chain (ox/oy/oz arrays, chain atoms).
// The mixed and FP32 forms rotate in double-float on the FP32 pipe (df_rotate_quaternion),
// the FP64 form in FP64 (the oracle's arithmetic).
template <int PREC, class WK>
__device__ __noinline__ void gen_orientations(const BoxDev& b, WK& W, uint64_t seed, uint32_t stream,
                                                 uint64_t move, int no, int chain, int off, double scale_coul,
                                                 double scale, double fx, double fy, double fz, bool retrace,
                                                 const double* ox, const double* oy, const double* oz,
                                                 uint32_t slot_base = SLOT_ORIENT) {
  for (int tid = threadIdx.x; tid < no * chain; tid += blockDim.x) {
    const int o = tid / chain, at = tid % chain;
    const double q = b.charge[off + 1 + at] * scale_coul;
    const int type = b.meta[off + 1 + at].x;
    if (retrace && o == 0) {
      make_bead(W.beads[tid], ox[at], oy[at], oz[at], q, scale, type, b.prefactor);
    } else {
      uint32_t r[4];
      draw4_dev(seed, stream, move, slot_base + o, r);
      const double4 t0 = b.pos64[off];
      const double4 pa = b.pos64[off + 1 + at];
      double vx = pa.x - t0.x, vy = pa.y - t0.y, vz = pa.z - t0.z;
      if constexpr (PREC == GRX_FP64) rotate_quaternion(vx, vy, vz, u01(r[0]), u01(r[1]), u01(r[2]));
      else df_rotate_quaternion(vx, vy, vz, r[0], r[1], r[2]);
      make_bead(W.beads[tid], fx + vx, fy + vy, fz + vz, q, scale, type, b.prefactor);
    }
  }
  __syncthreads();
}

// Energies of ntr = nb / chain trials of `chain` beads each (W.beads) against every
// atom, with the atoms of (comp, newmol) and of (excl_comp, excl_mol) excluded (the
// ExcludeList of an identity swap): W.te[4 t + k], W.tflag[t]. The first `early` trials
// (all of them when early < 0) stop at their first overlap (early overlap rejection):
// their flags are exact, their energies are not computed in full and must not be used
// when flagged, which is how every CBMC step treats a flagged trial.
// With CL > 1 the block is one CTA of a cluster that shares the chain: the pass is split
// over the cluster's warps (items per warp capped so the slots fit the workspace), each
// CTA copies its slots into its peers' workspaces, and every CTA reduces all slots. The
// second cluster barrier keeps a CTA from writing the next pass's slots into a peer that
// is still reducing this one.
template <int PREC, int CL, class WK>
__device__ __forceinline__ void trial_pass_body(const BoxDev& b, WK& W, int nb, int chain, int comp, int newmol,
                                                int excl_comp, int excl_mol, int early) {
  if (threadIdx.x == 0) {
    W.counter = 0;
    W.cfg += nb / chain;
    W.cbeads += nb;
  }
  for (int t = threadIdx.x; t < nb / chain; t += blockDim.x) W.tdead[t] = (early < 0 || t < early) ? 0 : -1;
  __syncthreads();
  const int nw = (int)(blockDim.x >> 5);
  if constexpr (CL == 1) {
    const PassSplit sp = pass_split(b, nb, nw, b.chunk_mult);
    block_bead_pass<PREC>(b, W.beads, nb, comp, newmol, excl_comp, excl_mol, W.qbuf, W.ipart, W.iflag, &W.counter, sp,
                          0, -1, chain, W.tdead, W.vst);
    __syncthreads();
    reduce_items<PREC>(W.ipart, W.iflag, nb / chain, chain, sp, W.te, W.tflag);
    __syncthreads();
  } else {
    const PassSplit sp = pass_split(b, nb, nw * CL, max(1, min(b.chunk_mult, kCbmcMaxMult / CL)));
    const unsigned rank = cluster_rank();
    int i0, i1;
    cluster_items(sp, CL, rank, i0, i1);
    block_bead_pass<PREC>(b, W.beads, nb, comp, newmol, excl_comp, excl_mol, W.qbuf, W.ipart, W.iflag, &W.counter, sp,
                          i0, i1, chain, W.tdead);
    __syncthreads();
    if (sp.nu > 0 && i0 < i1) {  // this CTA's slots [s0, s0 + n): item + bead, increasing
      unsigned lo, hi;
      sp.range((unsigned)i0, lo, hi);
      const int s0 = i0 + (int)(lo / sp.nu);
      sp.range((unsigned)(i1 - 1), lo, hi);
      const int n = (i1 - 1) + (int)((hi - 1u) / sp.nu) - s0 + 1;
      const unsigned long long* src = reinterpret_cast<const unsigned long long*>(W.ipart);
      for (int k = threadIdx.x; k < (CL - 1) * n * 5; k += blockDim.x) {
        const int j = k / (n * 5), e = k - j * (n * 5);
        const unsigned peer = (unsigned)j + ((unsigned)j >= rank ? 1u : 0u);
        const int slot = s0 + e / 5, f = e % 5;
        if (f < 4) {
          cluster_map(reinterpret_cast<unsigned long long*>(W.ipart), peer)[slot * 4 + f] = src[slot * 4 + f];
        } else {
          cluster_map(W.iflag, peer)[slot] = W.iflag[slot];
        }
      }
    }
    cluster_sync_all();
    reduce_items<PREC>(W.ipart, W.iflag, nb / chain, chain, sp, W.te, W.tflag);
    __syncthreads();
    cluster_sync_all();
  }
}

template <int PREC, int CL = 1, class WK>
__device__ __noinline__ void trial_pass(const BoxDev& b, WK& W, int nb, int chain, int comp, int newmol,
                                          int early = -1) {
  trial_pass_body<PREC, CL>(b, W, nb, chain, comp, newmol, -1, -1, early);
}
// The same with a second excluded molecule (excl_comp, excl_mol).
template <int PREC, int CL = 1, class WK>
__device__ __noinline__ void trial_pass_excl(const BoxDev& b, WK& W, int nb, int chain, int comp, int newmol,
                                               int excl_comp, int excl_mol) {
  trial_pass_body<PREC, CL>(b, W, nb, chain, comp, newmol, excl_comp, excl_mol, -1);
}

// CBMC weight of one growth step (warp 0 computes, results in W.ok/sel/w/nok/wraw).
// Insertion: log-sum-exp selection with the uniform u (SelectTrialPosition) and the
// 1e-150 failure test. Retrace (deletion): the first trial without overlap is the
// existing configuration and no selection is drawn. `stored` is added to the sum
// before averaging (the reinsertion retrace's StoredR, mc_widom.h:363-366). Exponentials are evaluated one
// trial per lane; sums and the cumulative search stay sequential in trial order.
template <class WK>
__device__ __noinline__ void step_weight(WK& W, int nt, double beta, int bias, double u, double navg,
                                            bool retrace, double stored = 0.0) {
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    double lw[2];
    bool ok[2];
    double mx = -INFINITY;
    int cnt = 0;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int t = lane + 32 * r;
      ok[r] = t < nt && !W.tflag[t];
      lw[r] = -INFINITY;
      if (ok[r]) {
        double tot = W.te[4 * t] + W.te[4 * t + 2];
        if (bias) tot += W.te[4 * t + 1] + W.te[4 * t + 3];
        lw[r] = __dmul_rn(-beta, tot);
        mx = fmax(mx, lw[r]);
        ++cnt;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
#pragma unroll 1
    for (int r = 0; r < 2; ++r) {
      const int t = lane + 32 * r;
      if (t < nt) {
        W.sel_ws[t] = ok[r] ? exp_move(__dsub_rn(lw[r], mx)) : 0.0;
        W.sel_wa[t] = ok[r] ? exp_move(lw[r]) : 0.0;
      }
    }
    __syncwarp();
    if (lane == 0) {
      W.nok = cnt;
      W.ok = 0;
      if (cnt > 0) {
        int s = -1;
        if (retrace) {
#pragma unroll 1
          for (int t = 0; t < nt; ++t)
            if (!W.tflag[t]) { s = t; break; }
        } else {
          double sum = 0.0;
#pragma unroll 1
          for (int t = 0; t < nt; ++t)
            if (!W.tflag[t]) sum += W.sel_ws[t];
          const double wsel = u * sum;
          int left = cnt;
          double cum = 0.0;
#pragma unroll 1
          for (int t = 0; t < nt; ++t) {
            if (W.tflag[t]) continue;
            cum += W.sel_ws[t];
            s = t;
            --left;
            if (!(cum < wsel) || left == 0) break;
          }
        }
        double w = 0.0;
#pragma unroll 1
        for (int t = 0; t < nt; ++t)
          if (!W.tflag[t]) w += W.sel_wa[t];
        W.wraw = w;
        if (retrace || !(w < 1e-150)) {
          double avg = (w + stored) / navg;
          if (!bias) avg *= exp_move(-beta * (W.te[4 * s + 1] + W.te[4 * s + 3]));
          W.ok = 1;
          W.sel = s;
          W.w = avg;
        }
      }
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------- Ewald
// Fourier delta of the na moved atoms in W.mx/my/mz/mq (old atoms carry -q):
// dS(k) = sum q e^{ik.r}; same = sum temp (|S + dS|^2 - |S|^2), cross = sum temp
// Re(S_cross dS*), S_same = adsorbate block (guest moves). The FP64 form follows
// the reference arithmetic; the other forms evaluate dS and both sums in
// double-float on the FP32 pipe against temp*S tables (ewA, ewF). When s_out is
// given, S_same + dS is staged there (FP64) for a later commit. Results on thread 0.
// With CL > 1 each CTA of the cluster takes a contiguous range of the active k (its
// range of S is staged, and later committed, by that CTA alone); the CTAs' partial sums
// are exchanged through distributed shared memory and added in rank order by every CTA.
template <int PREC, class WK, bool ROWS = false, int CL = 1>
__device__ __noinline__ void ewald_move(const BoxDev& b, WK& W, int na, double2* eik, double2* s_out,
                                           double& same, double& cross) {
  const int tid = threadIdx.x;
  int k0 = 0, k1 = b.nact;
  if constexpr (CL > 1) cluster_k_range(b.nact, CL, cluster_rank(), k0, k1);
  const int kx1 = b.kmax[0] + 1, ky1 = b.kmax[1] + 1;
  double2* ex = eik;
  double2* ey = ex + kx1 * na;
  double2* ez = ey + ky1 * na;
  const double PI2 = 2.0 * 3.14159265358979323846;
  if (tid < 3 * na) {  // eik recurrence per atom and axis (Initialize_Vectors_thread)
    const int at = tid % na, d = tid / na;
    const double f = b.inv[d] * W.mx[at] + b.inv[3 + d] * W.my[at] + b.inv[6 + d] * W.mz[at];
    const int km = b.kmax[d];
    if constexpr (PREC == GRX_FP64) {
      double2* tab = d == 0 ? ex : (d == 1 ? ey : ez);
      tab[at] = make_double2(1.0, 0.0);
      if (km >= 1) {
        double sn, cs;
        sincos(f * PI2, &sn, &cs);
        const double2 e1 = make_double2(cs, sn);
        double2 e = e1;
        tab[at + na] = e1;
        for (int k = 2; k <= km; ++k) {
          e = cmul(e, e1);
          tab[at + k * na] = e;
        }
      }
    } else {  // straight into the double-float tables read below (the FP64 ones are not used)
      float4* f0 = reinterpret_cast<float4*>(eik);
      float4* tab = f0 + (d == 0 ? 0 : (d == 1 ? kx1 * na : (kx1 + ky1) * na));
      df_eik_row(f, km, tab + at, na);
    }
  }
  __syncthreads();
  same = 0.0;
  cross = 0.0;
  if constexpr (PREC == GRX_FP64) {
    for (int j = k0 + tid; j < k1; j += blockDim.x) {
      const int4 k = b.kact[j];
      double2 dsk = make_double2(0.0, 0.0);
      for (int at = 0; at < na; ++at) {
        double2 y = ey[at + na * abs(k.y)];
        if (k.y < 0) y.y = -y.y;
        double2 z = ez[at + na * abs(k.z)];
        if (k.z < 0) z.y = -z.y;
        const double2 t = cmul(cmul(ex[at + na * k.x], y), z);
        dsk.x += W.mq[at] * t.x;
        dsk.y += W.mq[at] * t.y;
      }
      const double tmp = b.ktemp[j];
      const double2 ov = b.s_ads[k.w];
      const double2 nv = make_double2(ov.x + dsk.x, ov.y + dsk.y);
      same += tmp * (nv.x * nv.x + nv.y * nv.y);
      same -= tmp * (ov.x * ov.x + ov.y * ov.y);
      const double2 xv = b.s_fw[k.w];
      cross += tmp * (xv.x * dsk.x + xv.y * dsk.y);
      if (s_out) s_out[k.w] = nv;
    }
    same = block_sum(same, W.sbuf);
    cross = block_sum(cross, W.sbuf);
  } else {
    float4* fx = reinterpret_cast<float4*>(eik);
    const int ntab = (b.kmax[0] + b.kmax[1] + b.kmax[2] + 3) * na;
    if (tid < na) { const df q = df_from(W.mq[tid]); W.qd[tid] = make_float2(q.hi, q.lo); }
    __syncthreads();
    const float4* fy = fx + kx1 * na;
    const float4* fz = fy + ky1 * na;
    df sm = {0.f, 0.f}, cr = {0.f, 0.f};
    if constexpr (ROWS) {
      // energy terms of one k from its dS: sm += 2 Re(temp S* dS) + temp |dS|^2,
      // cr += Re(temp S_fw* dS); optionally stage S + dS (FP64, compensated)
      auto k_energy = [&](int j, int slot, const df& cre, const df& cim) {
        const float4 A = b.ewA[j], F = b.ewF[j];
        const float2 T = b.ewT[j];
        const df reA = df_add(df_mul(df{A.x, A.y}, cre), df_mul(df{A.z, A.w}, cim));
        const df n2 = df_add(df_mul(cre, cre), df_mul(cim, cim));
        sm = df_add(sm, df_add(df{2.f * reA.hi, 2.f * reA.lo}, df_mul(df{T.x, T.y}, n2)));
        cr = df_add(cr, df_add(df_mul(df{F.x, F.y}, cre), df_mul(df{F.z, F.w}, cim)));
        if (s_out) {
          const double2 ov = b.s_ads[slot];
          s_out[slot] = make_double2(ov.x + df_to(cre), ov.y + df_to(cim));
        }
      };

      // q X(kx) Y(ky) per (kx, ky) row and atom, then one complex product with Z(kz) per
      // (k, atom); threads keep one k each, as in the direct form
      const int ny = 2 * b.kmax[1] + 1, nrow = ew_rows(b.kmax);
      float4* rxy = fx + ntab;
      for (int e = tid; e < nrow * na; e += blockDim.x) {
        const int row = e / na, at = e - row * na;
        const int kx = row / ny, ky = row - kx * ny - b.kmax[1];
        const float s = ky < 0 ? -1.f : 1.f;
        const float4 X = fx[at + na * kx], Y = fy[at + na * abs(ky)];
        const df xr = {X.x, X.y}, xi = {X.z, X.w};
        const df yr = {Y.x, Y.y}, yi = {s * Y.z, s * Y.w};
        const df q = {W.qd[at].x, W.qd[at].y};
        const df pr = df_mul(q, df_add(df_mul(xr, yr), df_mul(df{-xi.hi, -xi.lo}, yi)));
        const df pi = df_mul(q, df_add(df_mul(xr, yi), df_mul(xi, yr)));
        rxy[e] = make_float4(pr.hi, pr.lo, pi.hi, pi.lo);
      }
      __syncthreads();
      for (int j = k0 + tid; j < k1; j += blockDim.x) {
        const int4 k = b.kact[j];
        const float4* P = rxy + (k.x * ny + k.y + b.kmax[1]) * na;
        const int az = abs(k.z);
        const float sz = k.z < 0 ? -1.f : 1.f;
        df cre = {0.f, 0.f}, cim = {0.f, 0.f};
#pragma unroll 1
        for (int at = 0; at < na; ++at) {
          const float4 R = P[at], Z = fz[at + na * az];
          const df pr = {R.x, R.y}, pi = {R.z, R.w};
          const df zr = {Z.x, Z.y}, zi = {sz * Z.z, sz * Z.w};
          cre = df_add(cre, df_add(df_mul(pr, zr), df_mul(df{-pi.hi, -pi.lo}, zi)));
          cim = df_add(cim, df_add(df_mul(pr, zi), df_mul(pi, zr)));
        }
        k_energy(j, k.w, cre, cim);
      }
    } else {
      for (int j = k0 + tid; j < k1; j += blockDim.x) {
        const int4 k = b.kact[j];
        df cre = {0.f, 0.f}, cim = {0.f, 0.f};
        const int ay = abs(k.y), az = abs(k.z);
        const float sy = k.y < 0 ? -1.f : 1.f, sz = k.z < 0 ? -1.f : 1.f;
#pragma unroll 1
        for (int at = 0; at < na; ++at) {
          const float4 X = fx[at + na * k.x], Y = fy[at + na * ay], Z = fz[at + na * az];
          const df xr = {X.x, X.y}, xi = {X.z, X.w};
          const df yr = {Y.x, Y.y}, yi = {sy * Y.z, sy * Y.w};
          const df zr = {Z.x, Z.y}, zi = {sz * Z.z, sz * Z.w};
          const df pr = df_add(df_mul(xr, yr), df_mul(df{-xi.hi, -xi.lo}, yi));
          const df pi = df_add(df_mul(xr, yi), df_mul(xi, yr));
          const df tr = df_add(df_mul(pr, zr), df_mul(df{-pi.hi, -pi.lo}, zi));
          const df ti = df_add(df_mul(pr, zi), df_mul(pi, zr));
          const df q = {W.qd[at].x, W.qd[at].y};
          cre = df_add(cre, df_mul(q, tr));
          cim = df_add(cim, df_mul(q, ti));
        }
        const float4 A = b.ewA[j], F = b.ewF[j];
        const float2 T = b.ewT[j];
        const df reA = df_add(df_mul(df{A.x, A.y}, cre), df_mul(df{A.z, A.w}, cim));
        const df n2 = df_add(df_mul(cre, cre), df_mul(cim, cim));
        sm = df_add(sm, df_add(df{2.f * reA.hi, 2.f * reA.lo}, df_mul(df{T.x, T.y}, n2)));
        cr = df_add(cr, df_add(df_mul(df{F.x, F.y}, cre), df_mul(df{F.z, F.w}, cim)));
        if (s_out) {  // compensated update: FP64 S plus the double-float dS
          const double2 ov = b.s_ads[k.w];
          s_out[k.w] = make_double2(ov.x + df_to(cre), ov.y + df_to(cim));
        }
      }
    }
    sm = warp_sum_df(sm);
    cr = warp_sum_df(cr);
    if ((tid & 31) == 0) { W.wsum[0][tid >> 5] = df_to(sm); W.wsum[1][tid >> 5] = df_to(cr); }
    __syncthreads();
    if (tid == 0)
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { same += W.wsum[0][w]; cross += W.wsum[1][w]; }
  }
  if constexpr (CL > 1) {
    const unsigned rank = cluster_rank();
    if (tid == 0)
      for (unsigned p = 0; p < (unsigned)CL; ++p) {
        double* dst = cluster_map(&W.ewx[0][0], p);
        dst[2 * rank] = same;
        dst[2 * rank + 1] = cross;
      }
    cluster_sync_all();
    if (tid == 0) {
      same = 0.0;
      cross = 0.0;
      for (int p = 0; p < CL; ++p) { same += W.ewx[p][0]; cross += W.ewx[p][1]; }
    }
  }
  __syncthreads();
}

// Make the staged structure factor current and refresh its double-float table (in a
// cluster, the CTA's own range of k).
template <int CL = 1>
__device__ __noinline__ void commit_sk(const BoxDev& b, const double2* s_tmp) {
  float4* ewA = const_cast<float4*>(b.ewA);
  int k0 = 0, k1 = b.nact;
  if constexpr (CL > 1) cluster_k_range(b.nact, CL, cluster_rank(), k0, k1);
  for (int j = k0 + threadIdx.x; j < k1; j += blockDim.x) {
    const int slot = b.kact[j].w;
    const double2 v = s_tmp[slot];
    b.s_ads[slot] = v;
    const double t = b.ktemp[j];
    const df ar = df_from(t * v.x), ai = df_from(t * v.y);
    ewA[j] = make_float4(ar.hi, ar.lo, ai.hi, ai.lo);
  }
  __syncthreads();
}

// Write one atom into the box storage (all representations).
static __device__ __noinline__ void store_atom(const BoxDev& b, int idx, double x, double y, double z, double charge,
                                           double scale_coul, double scale, int type, int molid) {
  const double qe = charge * scale_coul;
  const_cast<double4*>(b.pos64)[idx] = make_double4(x, y, z, qe);
  float hx, lx, hy, ly, hz, lz;
  split_coord(x, hx, lx);
  split_coord(y, hy, ly);
  split_coord(z, hz, lz);
  const_cast<float4*>(b.hi)[idx] = make_float4(hx, hy, hz, (float)qe);
  const_cast<float4*>(b.lo)[idx] = make_float4(lx, ly, lz, (float)scale);
  const_cast<int2*>(b.meta)[idx] = make_int2(type, molid);
  const_cast<double*>(b.scale)[idx] = scale;
  const_cast<double*>(b.charge)[idx] = charge;
  const df q = df_from(qe);
  const_cast<float2*>(b.qdf)[idx] = make_float2(q.hi, q.lo);
}

}  // namespace grx
