// grx_widom.cu -- batched CBMC Widom insertions, fully on the device, and the
// stand-alone Rosenbluth selection entry point.
//
// One block per insertion (persistent grid-stride loop). Per insertion:
//   1. first-bead trial positions from Philox (get_random_trial_position),
//   2. pair energies of all trials against every atom (bead_pass),
//   3. Rosenbluth selection of the first bead (SelectTrialPosition),
//   4. trial orientations about the chosen bead (get_random_trial_orientation),
//   5. pair energies of the orientations, selection,
//   6. Ewald Fourier delta of the chosen molecule (Fourier_Ewald_Diff) and the
//      exclusion / tail factors of Insertion_Body (mc_swap_utilities.h:94-108).
#include <algorithm>
#include <cmath>
#include <vector>

#include "grx_host.h"
#include "grx_warp.cuh"

namespace grx {

constexpr int kMaxTrials = 64;
constexpr int kWidomItemsPerWarp = 1;  // work split of a bead pass (items per warp)

struct WidomArgs {
  int comp;
  int ntrials;
  int norient;
  int molsize;
  int newmol;
  int rigid;
  int charged;
  int pad_;
  double scale;
  double scale_coul;
  double beta;
  double tail;
  double excl;  // ExclusionIntra + ExclusionAtom of the component
  uint64_t seed;
  uint64_t first_move;
  int64_t n;
  uint32_t stream;
};

// Log-sum-exp selection and weight of one CBMC step (SelectTrialPosition,
// mc_widom.h:14-39, and CBMC_FirstBead_Finish :330-376, insertion branch), computed by
// warp 0: the exponentials are evaluated one trial per lane, the sums and the cumulative
// search stay sequential in trial order on lane 0, as in the reference's host loop.
// Results are valid on lane 0.
__device__ bool select_trial_warp(const double* te, const int* tflag, int nt, double beta, int bias,
                                  double u, double navg, int& sel, double& wavg, int& nok, double* ws,
                                  double* wa) {
  const int lane = threadIdx.x & 31;
  double lw[2];
  bool ok[2];
  double mx = -INFINITY;
  int cnt = 0;
  for (int r = 0; r < 2; ++r) {
    const int t = lane + 32 * r;
    ok[r] = t < nt && !tflag[t];
    lw[r] = -INFINITY;
    if (ok[r]) {
      double tot = te[4 * t] + te[4 * t + 2];
      if (bias) tot += te[4 * t + 1] + te[4 * t + 3];
      lw[r] = __dmul_rn(-beta, tot);
      mx = fmax(mx, lw[r]);
      ++cnt;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  }
  for (int r = 0; r < 2; ++r) {
    const int t = lane + 32 * r;
    if (t < nt) {
      ws[t] = ok[r] ? exp(__dsub_rn(lw[r], mx)) : 0.0;
      wa[t] = ok[r] ? exp(lw[r]) : 0.0;
    }
  }
  __syncwarp();
  nok = cnt;
  if (lane != 0 || cnt == 0) return false;
  double sum = 0.0;
  for (int t = 0; t < nt; ++t)
    if (!tflag[t]) sum += ws[t];
  const double wsel = u * sum;
  int s = -1, left = cnt;
  double cum = 0.0;
  for (int t = 0; t < nt; ++t) {
    if (tflag[t]) continue;
    cum += ws[t];
    s = t;
    --left;
    if (!(cum < wsel) || left == 0) break;
  }
  double w = 0.0;
  for (int t = 0; t < nt; ++t)
    if (!tflag[t]) w += wa[t];
  if (w < 1e-150) return false;
  sel = s;
  double avg = w / navg;
  if (!bias) avg *= exp(-beta * (te[4 * s + 1] + te[4 * s + 3]));
  wavg = avg;
  return true;
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

template <int PREC>
__global__ void __launch_bounds__(GRX_THREADS, 3) widom_kernel(BoxDev b, WidomArgs a, grx_widom_result* out) {
  __shared__ Bead beads[GRX_MAX_TRIAL_BEADS];
  __shared__ double ipart[kMaxItems * 4];
  __shared__ int iflag[kMaxItems];
  __shared__ int qbuf[(GRX_THREADS / 32) * kQueue];
  __shared__ int counter;
  __shared__ double te[kMaxTrials * 4];
  __shared__ int tflag[kMaxTrials];
  __shared__ int tdead[kMaxTrials];  // early overlap rejection flags of a pass's trials
  __shared__ double sbuf[32];
  __shared__ double newx[GRX_MAX_MOLSIZE], newy[GRX_MAX_MOLSIZE], newz[GRX_MAX_MOLSIZE], newq[GRX_MAX_MOLSIZE];
  __shared__ grx_widom_result res;
  __shared__ int s_ok;
  __shared__ double sel_ws[kMaxTrials], sel_wa[kMaxTrials];
  extern __shared__ double2 eik_s[];

  const int tid = threadIdx.x;
  const int off = b.comp_off[a.comp];
  const int ms = a.molsize, chain = ms - 1;
  const double4 t0 = b.pos64[off];
  for (int64_t m = blockIdx.x; m < a.n; m += gridDim.x) {
    const uint64_t move = a.first_move + (uint64_t)m;
    uint32_t selw[4];
    draw4(a.seed, a.stream, move, SLOT_SELECT, selw);
    if (tid == 0) {
      res = grx_widom_result{};
      res.sel_first = -1;
      res.sel_orient = -1;
      s_ok = 0;
      counter = 0;
    }
    // 1. first-bead trials (mc_widom.h:133-139)
    const int nt = a.ntrials;
    if (tid < nt) tdead[tid] = 0;
    if (tid < nt) {
      uint32_t r[4];
      draw4(a.seed, a.stream, move, SLOT_FIRST + tid, r);
      make_bead(beads[tid], b.cell[0] * u01(r[0]), b.cell[4] * u01(r[1]), b.cell[8] * u01(r[2]),
                b.charge[off] * a.scale_coul, a.scale, b.meta[off].x, b.prefactor);
    }
    __syncthreads();
    // 2. pair energies of the first-bead trials
    {
      const PassSplit sp = pass_split(b, nt, GRX_THREADS / 32, kWidomItemsPerWarp);
      block_bead_pass<PREC>(b, beads, nt, a.comp, a.newmol, -1, -1, qbuf, ipart, iflag, &counter, sp, 0, -1, 1,
                            tdead);
      __syncthreads();
      reduce_items<PREC>(ipart, iflag, nt, 1, sp, te, tflag);
      __syncthreads();
    }
    // 3. select the first bead
    if (tid < 32) {
      int sel = -1, nok = 0;
      double w = 0.0;
      const bool ok = select_trial_warp(te, tflag, nt, a.beta, b.vdw_real_bias, u01(selw[0]), (double)nt, sel, w,
                                        nok, sel_ws, sel_wa);
      if (tid == 0) res.n_ok_first = nok;
      if (ok && w > 1e-150) {
        s_ok = 1;
        res.sel_first = sel;
        res.w_first = w;
        res.rosenbluth = w;
        for (int q = 0; q < 4; ++q) res.e_first[q] = te[4 * sel + q];
        newx[0] = beads[sel].x; newy[0] = beads[sel].y; newz[0] = beads[sel].z;
        newq[0] = beads[sel].q;
      }
    }
    __syncthreads();
    if (s_ok && chain > 0) {
      // 4. orientations about the chosen first bead (mc_widom.h:255-276)
      const int no = a.norient, nb = no * chain;
      const double fx = newx[0], fy = newy[0], fz = newz[0];
      if (tid < nb) {
        const int o = tid / chain, at = tid % chain;
        uint32_t r[4];
        draw4(a.seed, a.stream, move, SLOT_ORIENT + o, r);
        const double4 pa = b.pos64[off + 1 + at];
        double vx = pa.x - t0.x, vy = pa.y - t0.y, vz = pa.z - t0.z;
        if constexpr (PREC == GRX_FP64) rotate_quaternion(vx, vy, vz, u01(r[0]), u01(r[1]), u01(r[2]));
        else df_rotate_quaternion(vx, vy, vz, r[0], r[1], r[2]);
        make_bead(beads[tid], fx + vx, fy + vy, fz + vz, b.charge[off + 1 + at] * a.scale_coul, a.scale,
                  b.meta[off + 1 + at].x, b.prefactor);
      }
      if (tid == 0) counter = 0;
      if (tid < no) tdead[tid] = 0;
      __syncthreads();
      // 5. pair energies of the orientations
      const PassSplit sp = pass_split(b, nb, GRX_THREADS / 32, kWidomItemsPerWarp);
      block_bead_pass<PREC>(b, beads, nb, a.comp, a.newmol, -1, -1, qbuf, ipart, iflag, &counter, sp, 0, -1, chain,
                            tdead);
      __syncthreads();
      reduce_items<PREC>(ipart, iflag, no, chain, sp, te, tflag);
      __syncthreads();
      if (tid < 32) {
        int sel = -1, nok = 0;
        double w = 0.0;
        const bool ok = select_trial_warp(te, tflag, no, a.beta, b.vdw_real_bias, u01(selw[1]), (double)no, sel, w,
                                          nok, sel_ws, sel_wa);
        if (tid == 0) res.n_ok_orient = nok;
        if (tid == 0 && ok) {
          res.sel_orient = sel;
          res.w_chain = w;
          for (int q = 0; q < 4; ++q) res.e_chain[q] = te[4 * sel + q];
          res.rosenbluth *= w;
          if (res.rosenbluth <= 1e-150) s_ok = 0;
          for (int at = 0; at < chain; ++at) {
            const Bead& bd = beads[sel * chain + at];
            newx[1 + at] = bd.x; newy[1 + at] = bd.y; newz[1 + at] = bd.z; newq[1 + at] = bd.q;
          }
        } else if (tid == 0) {
          s_ok = 0;
        }
      }
      __syncthreads();
    }
    // 6. Ewald delta of the chosen molecule (insertion: no old atoms)
    if (s_ok && a.charged && !b.no_charges && b.nact > 0) {
      const int kx1 = b.kmax[0] + 1, ky1 = b.kmax[1] + 1;
      double2* ex = eik_s;
      double2* ey = ex + kx1 * ms;
      double2* ez = ey + ky1 * ms;
      const double PI2 = 2.0 * 3.14159265358979323846;
      if (tid < 3 * ms) {
        const int at = tid % ms, d = tid / ms;
        const double f = b.inv[d] * newx[at] + b.inv[3 + d] * newy[at] + b.inv[6 + d] * newz[at];
        const int km = b.kmax[d];
        if constexpr (PREC == GRX_FP64) {
          double2* tab = d == 0 ? ex : (d == 1 ? ey : ez);
          tab[at] = make_double2(1.0, 0.0);
          if (km >= 1) {
            double sn, cs;
            sincos(f * PI2, &sn, &cs);
            const double2 e1 = make_double2(cs, sn);
            double2 e = e1;
            tab[at + ms] = e1;
            for (int k = 2; k <= km; ++k) {
              e = cmul(e, e1);
              tab[at + k * ms] = e;
            }
          }
        } else {  // straight into the double-float tables (after the FP64 ones)
          float4* f0 = reinterpret_cast<float4*>(ez + (b.kmax[2] + 1) * ms);
          float4* tab = f0 + (d == 0 ? 0 : (d == 1 ? kx1 * ms : (kx1 + ky1) * ms));
          df_eik_row(f, km, tab + at, ms);
        }
      }
      __syncthreads();
      double same = 0.0, cross = 0.0;
      if constexpr (PREC == GRX_FP64) {
        for (int j = tid; j < b.nact; j += blockDim.x) {
          const int4 k = b.kact[j];
          double2 cn = make_double2(0.0, 0.0);
          for (int at = 0; at < ms; ++at) {
            double2 y = ey[at + ms * abs(k.y)];
            if (k.y < 0) y.y = -y.y;
            double2 z = ez[at + ms * abs(k.z)];
            if (k.z < 0) z.y = -z.y;
            const double2 t = cmul(cmul(ex[at + ms * k.x], y), z);
            cn.x += newq[at] * t.x;
            cn.y += newq[at] * t.y;
          }
          const double tmp = b.ktemp[j];
          const double2 ov = b.s_ads[k.w];
          const double2 nv = make_double2(ov.x + cn.x, ov.y + cn.y);
          same += tmp * (nv.x * nv.x + nv.y * nv.y);
          same -= tmp * (ov.x * ov.x + ov.y * ov.y);
          const double2 xv = b.s_fw[k.w];
          cross += tmp * (xv.x * cn.x + xv.y * cn.y);
        }
        same = block_sum(same, sbuf);
        cross = block_sum(cross, sbuf);
      } else {
        // double-float copies of the eik tables (same shared buffer, after the FP64 ones)
        float4* fx = reinterpret_cast<float4*>(ez + (b.kmax[2] + 1) * ms);
        __shared__ float2 qd[GRX_MAX_MOLSIZE];
        if (tid < ms) { const df q = df_from(newq[tid]); qd[tid] = make_float2(q.hi, q.lo); }
        __syncthreads();
        const float4* fy = fx + kx1 * ms;
        const float4* fz = fy + ky1 * ms;
        df sm = {0.f, 0.f}, cr = {0.f, 0.f};
        for (int j = tid; j < b.nact; j += blockDim.x) {
          const int4 k = b.kact[j];
          df cre = {0.f, 0.f}, cim = {0.f, 0.f};
          const int ay = abs(k.y), az = abs(k.z);
          const float sy = k.y < 0 ? -1.f : 1.f, sz = k.z < 0 ? -1.f : 1.f;
          for (int at = 0; at < ms; ++at) {
            const float4 X = fx[at + ms * k.x], Y = fy[at + ms * ay], Z = fz[at + ms * az];
            const df xr = {X.x, X.y}, xi = {X.z, X.w};
            const df yr = {Y.x, Y.y}, yi = {sy * Y.z, sy * Y.w};
            const df zr = {Z.x, Z.y}, zi = {sz * Z.z, sz * Z.w};
            // (x*y)*z, then charge
            const df pr = df_add(df_mul(xr, yr), df_mul(df{-xi.hi, -xi.lo}, yi));
            const df pi = df_add(df_mul(xr, yi), df_mul(xi, yr));
            const df tr = df_add(df_mul(pr, zr), df_mul(df{-pi.hi, -pi.lo}, zi));
            const df ti = df_add(df_mul(pr, zi), df_mul(pi, zr));
            const df q = {qd[at].x, qd[at].y};
            cre = df_add(cre, df_mul(q, tr));
            cim = df_add(cim, df_mul(q, ti));
          }
          const float4 A = b.ewA[j], F = b.ewF[j];
          const float2 T = b.ewT[j];
          // same: 2 Re(A dS*) + temp |dS|^2 ; cross: Re(F dS*)
          const df reA = df_add(df_mul(df{A.x, A.y}, cre), df_mul(df{A.z, A.w}, cim));
          const df n2 = df_add(df_mul(cre, cre), df_mul(cim, cim));
          sm = df_add(sm, df_add(df{2.f * reA.hi, 2.f * reA.lo}, df_mul(df{T.x, T.y}, n2)));
          cr = df_add(cr, df_add(df_mul(df{F.x, F.y}, cre), df_mul(df{F.z, F.w}, cim)));
        }
        // block sums: warp tree in double-float, then FP64 over the 8 warp partials
        sm = warp_sum_df(sm);
        cr = warp_sum_df(cr);
        __shared__ double wsum[2][GRX_THREADS / 32];
        if ((tid & 31) == 0) { wsum[0][tid >> 5] = df_to(sm); wsum[1][tid >> 5] = df_to(cr); }
        __syncthreads();
        if (tid == 0) {
          for (int w = 0; w < GRX_THREADS / 32; ++w) { same += wsum[0][w]; cross += wsum[1][w]; }
        }
      }
      if (tid == 0) {
        if (a.rigid) same -= a.excl * (a.scale_coul * a.scale_coul - 0.0);
        res.ewald[0] = same;
        res.ewald[1] = 2.0 * cross;
        res.rosenbluth *= exp(-a.beta * (res.ewald[0] + res.ewald[1]));
      }
    }
    if (tid == 0) {
      if (s_ok) {
        res.rosenbluth *= exp(-a.beta * a.tail);
        res.success = 1;
      } else {
        res.rosenbluth = 0.0;
        res.success = 0;
      }
      out[m] = res;
    }
    __syncthreads();
  }
}

// temp * S(k) of both blocks in double-float, per active k (the box's static part of
// the Fourier delta: dE_same = sum 2 Re(A dS*) + temp |dS|^2, dE_cross = sum Re(F dS*)).
__global__ void ewald_df_refresh_kernel(BoxDev b, float4* ewA, float4* ewF, float2* ewT) {
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

__global__ void select_kernel(const double* logw, int n, double u, int* sel, double* sum) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double mx = logw[0];
  for (int i = 1; i < n; ++i) mx = fmax(mx, logw[i]);
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += exp(logw[i] - mx);
  const double ws = u * s;
  int k = 0;
  double cum = exp(logw[0] - mx);
  while (cum < ws && k + 1 < n) cum += exp(logw[++k] - mx);
  double w = 0.0;
  for (int i = 0; i < n; ++i) w += exp(logw[i]);
  *sel = k;
  *sum = w;
}

static grx_status widom_launch(grx_box* b, const grx_widom_desc* d, uint64_t first_move, size_t n,
                               grx_precision prec, grx_widom_result* dev_results) {
  GRX_REQUIRE(d->component >= b->nhost && d->component < b->ncomp,
              "grx_widom_insertions: component must be an adsorbate component");
  GRX_REQUIRE(d->ntrials >= 1 && d->ntrials <= kMaxTrials, "grx_widom_insertions: ntrials out of range (1..64)");
  const int ms = (int)b->molsize[d->component];
  GRX_REQUIRE(ms >= 1 && ms <= GRX_MAX_MOLSIZE, "grx_widom_insertions: molecule size out of range");
  if (ms > 1)
    GRX_REQUIRE(d->norient >= 1 && d->norient <= kMaxTrials && d->norient * (ms - 1) <= GRX_MAX_TRIAL_BEADS,
                "grx_widom_insertions: norient out of range");
  GRX_REQUIRE(prec == GRX_FP64 || prec == GRX_MIXED || prec == GRX_FP32, "grx_widom_insertions: bad precision");
  if (n == 0) return GRX_OK;
  refresh_dev(b);
  WidomArgs a{};
  a.comp = d->component;
  a.ntrials = d->ntrials;
  a.norient = ms > 1 ? d->norient : 0;
  a.molsize = ms;
  a.newmol = b->size[d->component] / ms;
  a.rigid = b->rigid[d->component];
  a.charged = b->has_charge[d->component];
  a.scale = d->scale;
  a.scale_coul = d->scale_coul;
  a.beta = d->beta;
  a.tail = d->tail_delta;
  a.excl = b->excl_intra[d->component] + b->excl_self[d->component];
  a.seed = d->seed;
  a.stream = d->stream;
  a.first_move = first_move;
  a.n = (int64_t)n;
  const size_t smem = (size_t)(b->dev.kmax[0] + b->dev.kmax[1] + b->dev.kmax[2] + 3) * ms *
                      (sizeof(double2) + sizeof(float4));
  if (!b->ewdf_valid && b->nact > 0) {
    ewald_df_refresh_kernel<<<std::max(1, std::min((b->nact + 255) / 256, sm_count(b))), 256, 0, b->stream>>>(
        b->dev, b->ewA, b->ewF, b->ewT);
    count_launch();
    b->ewdf_valid = true;
  }
  const int grid = (int)std::min<size_t>(n, (size_t)sm_count(b) * 3);
  if (prec == GRX_FP64) widom_kernel<GRX_FP64><<<grid, GRX_THREADS, smem, b->stream>>>(b->dev, a, dev_results);
  else if (prec == GRX_MIXED) widom_kernel<GRX_MIXED><<<grid, GRX_THREADS, smem, b->stream>>>(b->dev, a, dev_results);
  else widom_kernel<GRX_FP32><<<grid, GRX_THREADS, smem, b->stream>>>(b->dev, a, dev_results);
  count_launch();
  GRX_CHECK_CUDA(cudaGetLastError(), "widom launch");
  return GRX_OK;
}

}  // namespace grx

using namespace grx;

extern "C" {

grx_status grx_widom_insertions_async(grx_box* b, const grx_widom_desc* d, uint64_t first_move, size_t n,
                                      grx_precision prec, grx_widom_result* results) {
  GRX_REQUIRE(b && d && (results || n == 0), "grx_widom_insertions_async: null argument");
  return widom_launch(b, d, first_move, n, prec, results);
}

grx_status grx_widom_insertions(grx_box* b, const grx_widom_desc* d, uint64_t first_move, size_t n,
                                grx_precision prec, grx_widom_result* results) {
  GRX_REQUIRE(b && d && (results || n == 0), "grx_widom_insertions: null argument");
  if (n == 0) return GRX_OK;
  grx_status st = ensure_results(b, n);
  if (st) return st;
  st = widom_launch(b, d, first_move, n, prec, b->d_results);
  if (st) return st;
  GRX_CHECK_CUDA(cudaMemcpyAsync(results, b->d_results, n * sizeof(grx_widom_result), cudaMemcpyDefault, b->stream),
                 "read widom results");
  GRX_CHECK_CUDA(cudaStreamSynchronize(b->stream), "widom insertions");
  return GRX_OK;
}

grx_status grx_cbmc_select(const double* logw, int32_t n, uint64_t seed, uint32_t stream, uint64_t move,
                           int32_t word, int32_t* selected, double* sum) {
  GRX_REQUIRE(logw && selected && sum && n >= 1 && n <= 4096 && word >= 0 && word < 4,
              "grx_cbmc_select: bad argument");
  uint32_t w[4];
  draw4(seed, stream, move, SLOT_SELECT, w);
  double* d_lw = nullptr;
  GRX_CHECK_CUDA(cudaMalloc(&d_lw, n * sizeof(double) + 2 * sizeof(double)), "select scratch");
  int* d_sel = (int*)(d_lw + n);
  double* d_sum = d_lw + n + 1;
  cudaError_t e = cudaMemcpy(d_lw, logw, n * sizeof(double), cudaMemcpyDefault);
  if (e == cudaSuccess) {
    select_kernel<<<1, 32>>>(d_lw, n, u01(w[word]), d_sel, d_sum);
    count_launch();
    e = cudaGetLastError();
  }
  int s = 0;
  double sm = 0.0;
  if (e == cudaSuccess) e = cudaMemcpy(&s, d_sel, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&sm, d_sum, sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(d_lw);
  if (e != cudaSuccess) return cuda_status(e, "grx_cbmc_select");
  *selected = s;
  *sum = sm;
  return GRX_OK;
}

}  // extern "C"
