// grx_gcmc.cu -- GCMC moves fully on the device: one persistent block per box,
// looping over the box's Markov chain. A step restates RunMoves (axpy.cu:102-298)
// for one adsorbate component:
//   translation / rotation  get_new_position (mc_utilities.h:485-540), single-body
//                           energy (VDW_Coulomb.cu:626-841), Ewald delta,
//                           exp(-beta dE) (mc_single_particle.h:123-293)
//   CBMC insertion          Insertion_Body + InsertionMove (mc_swap_utilities.h:3-132,
//                           move_struct.h:18-90), Update_insertion_data_Parallel
//   CBMC deletion           Deletion_Body + DeletionMove (mc_swap_utilities.h:135-225,
//                           move_struct.h:122-167), Update_deletion_data_Parallel
// Random numbers: Philox, key = seed, counter = {slot, step lo, step hi, stream};
// slot 4096 = {molecule pick, move choice, insertion-vs-deletion, acceptance},
// slot 4097 = {three uniforms of the displacement / rotation angles}, CBMC trial
// slots 0..2047 and selection slot 2048 as in the Widom kernel.
#include <algorithm>
#include <cmath>
#include <vector>

#include "grx_cbmc.cuh"
#include "grx_host.h"

namespace grx {

enum : uint32_t { SLOT_MOVE = 4096u, SLOT_DISP = 4097u };

struct GcmcArgs {
  grx_gcmc_desc d;
  int comp;
  int ms;
  int off;
  int cap;      // component capacity in atoms
  int rigid;
  int charged;
  int bias;
  int pad_;
  double excl;  // ExclusionIntra + ExclusionAtom of the component
  double big_p; // MolFraction * Pressure * FugacityCoefficient * Volume
};

// RotationAroundAxis (mc_utilities.h:459-481) for a coordinate axis.
__device__ __forceinline__ void rotate_axis(double& x, double& y, double& z, double theta, int axis) {
  double s, c;
  sincos(theta, &s, &c);
  const double w = 1.0 - c;
  const double ax = axis == 0, ay = axis == 1, az = axis == 2;
  const double r0 = ax * ax * w + c, r1 = ax * ay * w + az * s, r2 = ax * az * w - ay * s;
  const double r3 = ax * ay * w - az * s, r4 = ay * ay * w + c, r5 = ay * az * w + ax * s;
  const double r6 = ax * az * w + ay * s, r7 = ay * az * w - ax * s, r8 = az * az * w + c;
  const double nx = x * r0 + y * r1 + z * r2;
  const double ny = x * r3 + y * r4 + z * r5;
  const double nz = x * r6 + y * r7 + z * r8;
  x = nx; y = ny; z = nz;
}

__device__ __forceinline__ void store_position(const BoxDev& b, int idx, double x, double y, double z) {
  double4* p64 = const_cast<double4*>(b.pos64);
  const double w = p64[idx].w;
  p64[idx] = make_double4(x, y, z, w);
  float hx, lx, hy, ly, hz, lz;
  split_coord(x, hx, lx);
  split_coord(y, hy, ly);
  split_coord(z, hz, lz);
  float4* hi = const_cast<float4*>(b.hi);
  float4* lo = const_cast<float4*>(b.lo);
  const float hw = hi[idx].w, lw = lo[idx].w;
  hi[idx] = make_float4(hx, hy, hz, hw);
  lo[idx] = make_float4(lx, ly, lz, lw);
}

__device__ __forceinline__ void copy_atom(const BoxDev& b, int dst, int src, int molid) {
  const_cast<double4*>(b.pos64)[dst] = b.pos64[src];
  const_cast<float4*>(b.hi)[dst] = b.hi[src];
  const_cast<float4*>(b.lo)[dst] = b.lo[src];
  const_cast<int2*>(b.meta)[dst] = make_int2(b.meta[src].x, molid);
  const_cast<double*>(b.scale)[dst] = b.scale[src];
  const_cast<double*>(b.charge)[dst] = b.charge[src];
  const_cast<float2*>(b.qdf)[dst] = b.qdf[src];
}

template <int PREC>
__global__ void __launch_bounds__(GRX_THREADS, 2) gcmc_kernel(const BoxDev* boxes, const GcmcArgs* args,
                                                              uint64_t first_step, int64_t nsteps,
                                                              grx_gcmc_stats* stats) {
  __shared__ BoxDev b;
  __shared__ GcmcArgs a;
  __shared__ CbmcWork W;
  __shared__ grx_gcmc_stats st;
  __shared__ int s_accept;
  __shared__ double s_e1[4], s_w1, s_dE[3], s_stored, s_r1[4], s_wr;
  extern __shared__ double2 eik[];
  const int tid = threadIdx.x;
  if (tid == 0) {
    b = boxes[blockIdx.x];
    a = args[blockIdx.x];
    st = grx_gcmc_stats{};
  }
  __syncthreads();
  const int comp = a.comp, ms = a.ms, chain = ms - 1, off = a.off;
  const grx_gcmc_desc& d = a.d;
  int* comp_size = const_cast<int*>(b.comp_size);
  for (int64_t step = 0; step < nsteps; ++step) {
    const uint64_t move = first_step + (uint64_t)step;
    uint32_t w[4], w2[4], ws[4];
    draw4(d.seed, d.stream, move, SLOT_MOVE, w);
    draw4(d.seed, d.stream, move, SLOT_DISP, w2);
    draw4(d.seed, d.stream, move, SLOT_SELECT, ws);
    const int N = comp_size[comp] / ms;
    const int mol = (int)(u01(w[0]) * (double)N);
    const double r = u01(w[1]);
    int kind = -1;
    if (r < d.p_translation) kind = 0;
    else if (r < d.p_rotation) kind = 1;
    else if (r < d.p_reinsertion) kind = 4;
    else if (r < d.p_swap) kind = (u01(w[2]) < 0.5) ? 2 : 3;
    const double uacc = u01(w[3]);
    if (tid == 0) s_accept = 0;

    if ((kind == 0 || kind == 1) && N > 0) {
      // ---------------------------------------------- translation / rotation
      const int m0 = off + mol * ms;
      if (tid == 0) st.attempts[kind]++;
      if (tid < ms) {
        const double4 p = b.pos64[m0 + tid];
        const double4 p0 = b.pos64[m0];
        double nx, ny, nz;
        if (kind == 0) {
          nx = p.x + d.max_translation[0] * 2.0 * (u01(w2[0]) - 0.5);
          ny = p.y + d.max_translation[1] * 2.0 * (u01(w2[1]) - 0.5);
          nz = p.z + d.max_translation[2] * 2.0 * (u01(w2[2]) - 0.5);
        } else {
          double vx = p.x - p0.x, vy = p.y - p0.y, vz = p.z - p0.z;
          rotate_axis(vx, vy, vz, d.max_rotation[0] * 2.0 * (u01(w2[0]) - 0.5), 0);
          rotate_axis(vx, vy, vz, d.max_rotation[1] * 2.0 * (u01(w2[1]) - 0.5), 1);
          rotate_axis(vx, vy, vz, d.max_rotation[2] * 2.0 * (u01(w2[2]) - 0.5), 2);
          nx = vx + p0.x; ny = vy + p0.y; nz = vz + p0.z;
        }
        W.mx[tid] = p.x; W.my[tid] = p.y; W.mz[tid] = p.z; W.mq[tid] = -p.w;
        W.mx[ms + tid] = nx; W.my[ms + tid] = ny; W.mz[ms + tid] = nz; W.mq[ms + tid] = p.w;
        const int type = b.meta[m0 + tid].x;
        const double sc = b.scale[m0 + tid];
        make_bead(W.beads[tid], nx, ny, nz, p.w, sc, type, b.prefactor);
        make_bead(W.beads[ms + tid], p.x, p.y, p.z, p.w, sc, type, b.prefactor);
      }
      __syncthreads();
      trial_pass<PREC>(b, W, 2 * ms, ms, comp, mol);  // te[0..3] new, te[4..7] old
      if (!W.tflag[0]) {
        double same = 0.0, cross = 0.0;
        if (a.charged) ewald_move<PREC>(b, W, 2 * ms, eik, b.s_tmp, same, cross);
        if (tid == 0) {
          const double dv = (W.te[0] + W.te[2]) - (W.te[4] + W.te[6]);
          const double dr = (W.te[1] + W.te[3]) - (W.te[5] + W.te[7]);
          const double ew = same + 2.0 * cross;
          const double pacc = exp(-d.beta * (dv + dr + ew));
          s_accept = uacc < pacc;
          s_dE[0] = dv; s_dE[1] = dr; s_dE[2] = ew;
        }
      }
      __syncthreads();
      if (s_accept) {
        if (tid < ms) store_position(b, m0 + tid, W.mx[ms + tid], W.my[ms + tid], W.mz[ms + tid]);
        if (a.charged) commit_sk(b, b.s_tmp);
        if (tid == 0) {
          st.accepted[kind]++;
          st.energy[0] += s_dE[0]; st.energy[1] += s_dE[1]; st.energy[2] += s_dE[2];
          st.energy[3] += s_dE[0] + s_dE[1] + s_dE[2];
        }
      }
    } else if (kind == 4 && N > 0) {
      // ---------------------------------------------- reinsertion (move_struct.h:170-406)
      const int m0 = off + mol * ms;
      if (tid == 0) st.attempts[4]++;
      if (tid < ms) {  // [0, ms): the molecule now (charge negated); [ms, 2ms): its regrowth
        const double4 p = b.pos64[m0 + tid];
        W.mx[tid] = p.x; W.my[tid] = p.y; W.mz[tid] = p.z; W.mq[tid] = -p.w;
        W.mq[ms + tid] = p.w;
      }
      __syncthreads();
      // insertion half: every trial new, the molecule itself excluded
      gen_first_trials(b, W, d.seed, d.stream, move, d.ntrials, b.charge[off], 1.0, b.meta[off].x, false, 0.0, 0.0,
                       0.0);
      trial_pass<PREC>(b, W, d.ntrials, 1, comp, mol);
      step_weight(W, d.ntrials, d.beta, a.bias, u01(ws[0]), (double)d.ntrials, false);
      bool ok = W.ok && W.w > 1e-150;
      double fx = 0, fy = 0, fz = 0;
      if (ok) {
        const Bead& fb = W.beads[W.sel];
        fx = fb.x; fy = fb.y; fz = fb.z;
        if (tid == 0) {
          for (int k = 0; k < 4; ++k) s_e1[k] = W.te[4 * W.sel + k];
          s_w1 = W.w;
          s_stored = W.wraw - W.sel_wa[W.sel];  // StoredR (mc_widom.h:363)
          W.mx[ms] = fx; W.my[ms] = fy; W.mz[ms] = fz;
        }
      }
      __syncthreads();
      double rosen = ok ? s_w1 : 0.0;
      double e2[4] = {0, 0, 0, 0};
      if (ok && chain > 0) {
        gen_orientations(b, W, d.seed, d.stream, move, d.norient, chain, off, 1.0, 1.0, fx, fy, fz, false, nullptr,
                         nullptr, nullptr);
        trial_pass<PREC>(b, W, d.norient * chain, chain, comp, mol);
        step_weight(W, d.norient, d.beta, a.bias, u01(ws[1]), (double)d.norient, false);
        ok = W.ok;
        if (ok) {
          rosen *= W.w;
          for (int k = 0; k < 4; ++k) e2[k] = W.te[4 * W.sel + k];
          if (rosen <= 1e-150) ok = false;
          if (tid < chain) {
            const Bead& bd = W.beads[W.sel * chain + tid];
            W.mx[ms + 1 + tid] = bd.x; W.my[ms + 1 + tid] = bd.y; W.mz[ms + 1 + tid] = bd.z;
          }
        }
        __syncthreads();
      }
      if (ok) {
        // retrace half: the first bead's single trial is the molecule's own, plus StoredR
        gen_first_trials(b, W, d.seed, d.stream, move, 1, b.charge[off], 1.0, b.meta[off].x, true, W.mx[0], W.my[0],
                         W.mz[0]);
        trial_pass<PREC>(b, W, 1, 1, comp, mol);
        step_weight(W, 1, d.beta, a.bias, 0.0, (double)d.ntrials, true, s_stored);
        bool ok2 = W.ok;
        if (ok2 && tid == 0) {
          for (int k = 0; k < 4; ++k) s_r1[k] = W.te[k];
          s_wr = W.w;
        }
        __syncthreads();
        double rosen_old = ok2 ? s_wr : 0.0;
        double r2[4] = {0, 0, 0, 0};
        if (ok2 && chain > 0) {
          gen_orientations(b, W, d.seed, d.stream, move, d.norient, chain, off, 1.0, 1.0, W.mx[0], W.my[0], W.mz[0],
                           true, W.mx + 1, W.my + 1, W.mz + 1, SLOT_RETRACE);
          trial_pass<PREC>(b, W, d.norient * chain, chain, comp, mol);
          step_weight(W, d.norient, d.beta, a.bias, 0.0, (double)d.norient, true);
          ok2 = W.ok;
          if (ok2) {
            rosen_old *= W.w;
            for (int k = 0; k < 4; ++k) r2[k] = W.te[4 * W.sel + k];
          }
          __syncthreads();
        }
        if (ok2) {
          double same = 0.0, cross = 0.0;
          if (a.charged) ewald_move<PREC>(b, W, 2 * ms, eik, b.s_tmp, same, cross);
          if (tid == 0) {
            const double ew = a.charged ? same + 2.0 * cross : 0.0;
            rosen *= exp(-d.beta * ew);
            const double pacc = rosen / rosen_old;
            s_accept = uacc < pacc;
            s_dE[0] = s_e1[0] + s_e1[2] + e2[0] + e2[2] - (s_r1[0] + s_r1[2] + r2[0] + r2[2]);
            s_dE[1] = s_e1[1] + s_e1[3] + e2[1] + e2[3] - (s_r1[1] + s_r1[3] + r2[1] + r2[3]);
            s_dE[2] = ew;
          }
        }
      }
      __syncthreads();
      if (s_accept) {
        if (tid < ms) store_position(b, m0 + tid, W.mx[ms + tid], W.my[ms + tid], W.mz[ms + tid]);
        if (a.charged) commit_sk(b, b.s_tmp);
        if (tid == 0) {
          st.accepted[4]++;
          st.energy[0] += s_dE[0]; st.energy[1] += s_dE[1]; st.energy[2] += s_dE[2];
          st.energy[3] += s_dE[0] + s_dE[1] + s_dE[2];
        }
      }
    } else if (kind == 2 || (kind == 3 && N > 0)) {
      // ---------------------------------------------- CBMC insertion / deletion
      const bool del = kind == 3;
      const int m0 = off + mol * ms;
      const int newmol = del ? mol : N;
      if (tid == 0) st.attempts[kind]++;
      if (del && tid < ms) {  // the molecule to retrace and remove
        const double4 p = b.pos64[m0 + tid];
        W.mx[tid] = p.x; W.my[tid] = p.y; W.mz[tid] = p.z; W.mq[tid] = -p.w;
      }
      __syncthreads();
      gen_first_trials(b, W, d.seed, d.stream, move, d.ntrials, b.charge[off], 1.0, b.meta[off].x, del,
                       W.mx[0], W.my[0], W.mz[0]);
      trial_pass<PREC>(b, W, d.ntrials, 1, comp, newmol);
      step_weight(W, d.ntrials, d.beta, a.bias, u01(ws[0]), (double)d.ntrials, del);
      bool ok = W.ok && W.w > 1e-150;
      double fx = 0, fy = 0, fz = 0;
      if (ok) {
        const Bead& fb = W.beads[W.sel];
        fx = fb.x; fy = fb.y; fz = fb.z;
        if (tid == 0) {
          for (int k = 0; k < 4; ++k) s_e1[k] = W.te[4 * W.sel + k];
          s_w1 = W.w;
        }
        if (!del && tid == 0) { W.mx[0] = fx; W.my[0] = fy; W.mz[0] = fz; W.mq[0] = b.charge[off]; }
      }
      __syncthreads();
      double rosen = ok ? s_w1 : 0.0;
      double e2[4] = {0, 0, 0, 0};
      if (ok && chain > 0) {
        gen_orientations(b, W, d.seed, d.stream, move, d.norient, chain, off, 1.0, 1.0, fx, fy, fz, del,
                         W.mx + 1, W.my + 1, W.mz + 1);
        trial_pass<PREC>(b, W, d.norient * chain, chain, comp, newmol);
        step_weight(W, d.norient, d.beta, a.bias, u01(ws[1]), (double)d.norient, del);
        ok = W.ok;
        if (ok) {
          rosen *= W.w;
          for (int k = 0; k < 4; ++k) e2[k] = W.te[4 * W.sel + k];
          if (rosen <= 1e-150) ok = false;
          if (!del && tid < chain) {
            const Bead& bd = W.beads[W.sel * chain + tid];
            W.mx[1 + tid] = bd.x; W.my[1 + tid] = bd.y; W.mz[1 + tid] = bd.z;
            W.mq[1 + tid] = b.charge[off + 1 + tid];
          }
        }
        __syncthreads();
      }
      if (ok) {
        double same = 0.0, cross = 0.0;
        if (a.charged) ewald_move<PREC>(b, W, ms, eik, b.s_tmp, same, cross);
        if (tid == 0) {
          double ew = 0.0;
          if (a.charged) {
            if (a.rigid) same -= a.excl * (del ? (0.0 - 1.0) : (1.0 - 0.0));
            ew = same + 2.0 * cross;
          }
          double pacc;
          if (!del) {
            rosen *= exp(-d.beta * ew);
            rosen *= exp(-d.beta * d.tail_insert);
            pacc = d.beta * a.big_p / (1.0 + (double)N) * rosen / d.ideal_rosenbluth;
            s_accept = rosen > 1e-150 && uacc < pacc;
            if (s_accept && (N + 1) * ms > a.cap) {
              s_accept = 0;
              st.capacity_hits++;
            }
          } else {
            rosen /= exp(-d.beta * ew);
            rosen /= exp(-d.beta * d.tail_insert);
            pacc = (double)N / (d.beta * a.big_p) * d.ideal_rosenbluth / rosen;
            s_accept = uacc < pacc;
          }
          const double ev = s_e1[0] + s_e1[2] + e2[0] + e2[2];
          const double er = s_e1[1] + s_e1[3] + e2[1] + e2[3];
          const double sg = del ? -1.0 : 1.0;
          s_dE[0] = sg * ev; s_dE[1] = sg * er; s_dE[2] = ew;
        }
      }
      __syncthreads();
      if (s_accept) {
        if (!del) {
          if (tid < ms)
            store_atom(b, off + N * ms + tid, W.mx[tid], W.my[tid], W.mz[tid], b.charge[off + tid], 1.0, 1.0,
                       b.meta[off + tid].x, N);
          __syncthreads();
          if (tid == 0) comp_size[comp] += ms;
        } else {
          const int last = off + (N - 1) * ms;
          if (m0 != last && tid < ms) copy_atom(b, m0 + tid, last + tid, mol);
          __syncthreads();
          if (tid == 0) comp_size[comp] -= ms;
        }
        if (a.charged) commit_sk(b, b.s_tmp);
        if (tid == 0) {
          st.accepted[kind]++;
          st.energy[0] += s_dE[0]; st.energy[1] += s_dE[1]; st.energy[2] += s_dE[2];
          st.energy[3] += s_dE[0] + s_dE[1] + s_dE[2];
        }
      }
    }
    __syncthreads();
    if (tid == 0) st.sum_n += (double)(comp_size[comp] / ms);
    __syncthreads();
  }
  if (tid == 0) {
    st.n_molecules = comp_size[comp] / ms;
    stats[blockIdx.x] = st;
  }
}

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
    ewF[j] = make_float4(fr.hi, fr.lo, fi.hi, fi.lo);
    const df tt = df_from(t);
    ewT[j] = make_float2(tt.hi, tt.lo);
  }
}

template <int PREC>
static grx_status launch_gcmc(grx_box* b0, int nboxes, const BoxDev* dboxes, const GcmcArgs* dargs,
                              uint64_t first_step, int64_t nsteps, grx_gcmc_stats* dstats, size_t smem) {
  GRX_CHECK_CUDA(cudaFuncSetAttribute(gcmc_kernel<PREC>, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024),
                 "gcmc shared memory attribute");
  gcmc_kernel<PREC><<<nboxes, GRX_THREADS, smem, b0->stream>>>(dboxes, dargs, first_step, nsteps, dstats);
  count_launch();
  GRX_CHECK_CUDA(cudaGetLastError(), "gcmc launch");
  return GRX_OK;
}

}  // namespace grx

using namespace grx;

extern "C" grx_status grx_gcmc_run(grx_box* const* boxes, int32_t nboxes, const grx_gcmc_desc* descs,
                                   uint64_t first_step, int64_t nsteps, grx_precision prec,
                                   grx_gcmc_stats* stats) {
  GRX_REQUIRE(boxes && descs && stats && nboxes >= 1, "grx_gcmc_run: bad argument");
  GRX_REQUIRE(prec == GRX_FP64 || prec == GRX_MIXED || prec == GRX_FP32, "grx_gcmc_run: bad precision");
  GRX_REQUIRE(nsteps >= 0, "grx_gcmc_run: negative step count");
  std::vector<BoxDev> hb(nboxes);
  std::vector<GcmcArgs> ha(nboxes);
  size_t smem = 0;
  for (int i = 0; i < nboxes; ++i) {
    grx_box* b = boxes[i];
    const grx_gcmc_desc& d = descs[i];
    GRX_REQUIRE(b, "grx_gcmc_run: null box");
    GRX_REQUIRE(b->device == boxes[0]->device, "grx_gcmc_run: boxes live on different devices");
    for (int j = 0; j < i; ++j) GRX_REQUIRE(boxes[j] != b, "grx_gcmc_run: a box appears twice");
    GRX_REQUIRE(d.component >= b->nhost && d.component < b->ncomp,
                "grx_gcmc_run: component must be an adsorbate component");
    const int ms = (int)b->molsize[d.component];
    GRX_REQUIRE(ms >= 1 && ms <= kMolWork, "grx_gcmc_run: molecule size must be 1..32");
    GRX_REQUIRE(b->stored[d.component] >= (size_t)ms,
                "grx_gcmc_run: the component stores no molecule template (set it with n_stored >= molsize)");
    GRX_REQUIRE(d.ntrials >= 1 && d.ntrials <= kMaxTrials, "grx_gcmc_run: ntrials out of range (1..64)");
    GRX_REQUIRE(ms == 1 || (d.norient >= 1 && d.norient <= kMaxTrials && d.norient * (ms - 1) <= GRX_MAX_TRIAL_BEADS),
                "grx_gcmc_run: norient out of range");
    GRX_REQUIRE(d.beta > 0 && d.pressure > 0 && d.ideal_rosenbluth > 0, "grx_gcmc_run: bad thermodynamic state");
    refresh_dev(b);
    if (!b->ewdf_valid && b->nact > 0) {
      ewald_df_refresh_gcmc<<<std::max(1, std::min((b->nact + 255) / 256, sm_count(b))), 256, 0, boxes[0]->stream>>>(
          b->dev);
      count_launch();
      b->ewdf_valid = true;
    }
    hb[i] = b->dev;
    GcmcArgs& a = ha[i];
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
    const size_t need = (size_t)(b->dev.kmax[0] + b->dev.kmax[1] + b->dev.kmax[2] + 3) * 2 * ms *
                        (sizeof(double2) + sizeof(float4));
    smem = std::max(smem, need);
  }
  GRX_REQUIRE(smem <= 64 * 1024, "grx_gcmc_run: Ewald tables exceed the shared-memory budget");
  grx_box* b0 = boxes[0];
  const size_t bbytes = (nboxes * sizeof(BoxDev) + 255) / 256 * 256;
  const size_t abytes = (nboxes * sizeof(GcmcArgs) + 255) / 256 * 256;
  grx_status st = ensure_scratch(b0, bbytes + abytes + nboxes * sizeof(grx_gcmc_stats));
  if (st) return st;
  BoxDev* dboxes = (BoxDev*)b0->scratch;
  GcmcArgs* dargs = (GcmcArgs*)((char*)b0->scratch + bbytes);
  grx_gcmc_stats* dstats = (grx_gcmc_stats*)((char*)b0->scratch + bbytes + abytes);
  GRX_CHECK_CUDA(cudaMemcpyAsync(dboxes, hb.data(), nboxes * sizeof(BoxDev), cudaMemcpyHostToDevice, b0->stream),
                 "upload boxes");
  GRX_CHECK_CUDA(cudaMemcpyAsync(dargs, ha.data(), nboxes * sizeof(GcmcArgs), cudaMemcpyHostToDevice, b0->stream),
                 "upload gcmc args");
  if (nsteps > 0) {
    if (prec == GRX_FP64) st = launch_gcmc<GRX_FP64>(b0, nboxes, dboxes, dargs, first_step, nsteps, dstats, smem);
    else if (prec == GRX_MIXED) st = launch_gcmc<GRX_MIXED>(b0, nboxes, dboxes, dargs, first_step, nsteps, dstats, smem);
    else st = launch_gcmc<GRX_FP32>(b0, nboxes, dboxes, dargs, first_step, nsteps, dstats, smem);
    if (st) return st;
    GRX_CHECK_CUDA(cudaMemcpyAsync(stats, dstats, nboxes * sizeof(grx_gcmc_stats), cudaMemcpyDefault, b0->stream),
                   "read gcmc stats");
  } else {
    for (int i = 0; i < nboxes; ++i) stats[i] = grx_gcmc_stats{};
  }
  GRX_CHECK_CUDA(cudaStreamSynchronize(b0->stream), "gcmc run");
  for (int i = 0; i < nboxes; ++i) {
    grx_box* b = boxes[i];
    GRX_CHECK_CUDA(cudaMemcpy(b->size, b->d_size, GRX_MAX_COMPONENTS * sizeof(int), cudaMemcpyDeviceToHost),
                   "read sizes");
    const int c = descs[i].component;
    b->stored[c] = std::max(b->stored[c], (size_t)b->size[c]);
    if (nsteps == 0) stats[i].n_molecules = b->size[descs[i].component] / (int)b->molsize[descs[i].component];
  }
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
