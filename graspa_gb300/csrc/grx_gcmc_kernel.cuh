// grx_gcmc_kernel.cuh -- the persistent GCMC kernel (one chain per block, or per
// thread-block cluster) shared by the plain launches (grx_gcmc.cu) and the cluster
// launches (grx_gcmc_cluster.cu). A step restates RunMoves (axpy.cu:102-298) for one
// adsorbate component:
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
#pragma once

#include "grx_cbmc.cuh"

namespace grx {

enum : uint32_t { SLOT_MOVE = 4096u, SLOT_DISP = 4097u, SLOT_SWAP = 4099u };
constexpr int kMaxMoved = 4;  // moved components per box in one GCMC run

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
  // per box (the same in all its entries): Philox move index of step s of a launch =
  // launch counter + s + step_off; steps taken = min(launch steps, nsteps_cap) (cap < 0: all)
  int64_t step_off;
  int64_t nsteps_cap;
};

// sin and cos of an angle in double-float (theta / 2 pi through df_sincos_2pi), out of line so
// the kernel body keeps its register allocation.
static __device__ __noinline__ double2 df_sincos_angle(double theta) {
  df sd, cd;
  df_sincos_2pi(df_mul(df_from(theta), df{0.15915494f, 6.4206382e-09f}), sd, cd);
  return make_double2(df_to(sd), df_to(cd));
}

// RotationAroundAxis (mc_utilities.h:459-481) for a coordinate axis; the mixed and FP32 forms
// take sin and cos in double-float, the FP64 form in FP64.
template <int PREC>
__device__ __noinline__ double4 rotate_axis_out(double x, double y, double z, double theta, int axis) {
  double s, c;
  if constexpr (PREC == GRX_FP64) sincos(theta, &s, &c);
  else {
    const double2 sc = df_sincos_angle(theta);
    s = sc.x;
    c = sc.y;
  }
  const double w = 1.0 - c;
  const double ax = axis == 0, ay = axis == 1, az = axis == 2;
  const double r0 = ax * ax * w + c, r1 = ax * ay * w + az * s, r2 = ax * az * w - ay * s;
  const double r3 = ax * ay * w - az * s, r4 = ay * ay * w + c, r5 = ay * az * w + ax * s;
  const double r6 = ax * az * w + ay * s, r7 = ay * az * w - ax * s, r8 = az * az * w + c;
  const double nx = x * r0 + y * r1 + z * r2;
  const double ny = x * r3 + y * r4 + z * r5;
  const double nz = x * r6 + y * r7 + z * r8;
  return make_double4(nx, ny, nz, 0.0);
}

template <int PREC>
__device__ __forceinline__ void rotate_axis(double& x, double& y, double& z, double theta, int axis) {
  const double4 r = rotate_axis_out<PREC>(x, y, z, theta, axis);
  x = r.x; y = r.y; z = r.z;
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

// The Fourier delta of a GCMC move, staged for commit_sk: the row-product form for boxes
// that enable it (BoxDev::ew_rows), the direct form otherwise; two instantiations, so each
// form keeps its own register allocation.
template <int PREC, int CL, class WK>
__device__ __forceinline__ void ewald_delta_move(const BoxDev& b, WK& W, int na, double2* eik, double& same,
                                                 double& cross) {
  if (b.ew_rows) ewald_move<PREC, WK, true, CL>(b, W, na, eik, b.s_tmp, same, cross);
  else ewald_move<PREC, WK, false, CL>(b, W, na, eik, b.s_tmp, same, cross);
}

// Identity swap of one step (mc_swap_moves.h:199-420), out of line so the kernel body keeps
// its register allocation. The reference redraws the old and new component until the old one
// holds a molecule: the old component is uniform over the moved components holding molecules,
// the new one uniform over all moved components. Swap slot words: {old component, new
// component, old molecule, acceptance}, as the host layer's IdentitySwapMove; the orientation
// selection takes u_orient (word 1 of the selection slot). Called by every thread of the block.
template <int PREC, int CL, class WK>
__device__ __noinline__ void identity_swap_step(const BoxDev& b, const GcmcArgs* A, int nm, grx_gcmc_stats* ST, WK& W,
                                                double2* eik, int* comp_size, uint64_t move, double beta,
                                                double u_orient, int& s_accept, double* s_e1, double& s_w1,
                                                double* s_dE, double* s_r1, double& s_wr) {
  const int tid = threadIdx.x;
  uint32_t wx[4];
  draw4_dev(A[0].d.seed, A[0].d.stream, move, SLOT_SWAP, wx);
  int have[kMaxMoved], nh = 0;
  for (int e = 0; e < nm; ++e)
    if (comp_size[A[e].comp] >= A[e].ms) have[nh++] = e;
  if (nh > 0) {
    const int eo = have[min(nh - 1, (int)(u01(wx[0]) * (double)nh))];
    const int en = min(nm - 1, (int)(u01(wx[1]) * (double)nm));
    const GcmcArgs& ao = A[eo];
    const GcmcArgs& an = A[en];
    const int mso = ao.ms, msn = an.ms;
    const int No = comp_size[ao.comp] / mso, Nn = comp_size[an.comp] / msn;
    const int omol = (int)(u01(wx[2]) * (double)No);
    const int o0 = ao.off + omol * mso;
    const bool charged = ao.charged || an.charged;
    if (tid == 0) {
      ST[eo].identity_out[0]++;
      ST[en].identity_in[0]++;
    }
    if (tid < mso) {  // [0, mso): the old molecule (charge negated); [mso, mso + msn): the new one
      const double4 p = b.pos64[o0 + tid];
      W.mx[tid] = p.x; W.my[tid] = p.y; W.mz[tid] = p.z; W.mq[tid] = -p.w;
    }
    __syncthreads();
    // the new species: one first-bead trial on the old first bead (not averaged) and its
    // orientations, the old molecule excluded
    gen_first_trials(b, W, A[0].d.seed, A[0].d.stream, move, 1, b.charge[an.off], 1.0, b.meta[an.off].x, true, W.mx[0],
                     W.my[0], W.mz[0]);
    trial_pass_excl<PREC, CL>(b, W, 1, 1, an.comp, Nn, ao.comp, omol);
    step_weight(W, 1, beta, an.bias, 0.0, 1.0, false);
    bool ok = W.ok && W.w > 1e-150;
    if (ok && tid == 0) {
      for (int k = 0; k < 4; ++k) s_e1[k] = W.te[k];
      s_w1 = W.w;
      W.mx[mso] = W.mx[0]; W.my[mso] = W.my[0]; W.mz[mso] = W.mz[0]; W.mq[mso] = b.charge[an.off];
    }
    __syncthreads();
    double rosen = ok ? s_w1 : 0.0;
    double e2[4] = {0, 0, 0, 0};
    if (ok && msn > 1) {
      gen_orientations<PREC>(b, W, A[0].d.seed, A[0].d.stream, move, an.d.norient, msn - 1, an.off, 1.0, 1.0, W.mx[0],
                       W.my[0], W.mz[0], false, nullptr, nullptr, nullptr);
      trial_pass_excl<PREC, CL>(b, W, an.d.norient * (msn - 1), msn - 1, an.comp, Nn, ao.comp, omol);
      step_weight(W, an.d.norient, beta, an.bias, u_orient, (double)an.d.norient, false);
      ok = W.ok;
      if (ok) {
        rosen *= W.w;
        for (int k = 0; k < 4; ++k) e2[k] = W.te[4 * W.sel + k];
        if (rosen <= 1e-150) ok = false;
        if (tid < msn - 1) {
          const Bead& bd = W.beads[W.sel * (msn - 1) + tid];
          W.mx[mso + 1 + tid] = bd.x; W.my[mso + 1 + tid] = bd.y; W.mz[mso + 1 + tid] = bd.z;
          W.mq[mso + 1 + tid] = b.charge[an.off + 1 + tid];
        }
      }
      __syncthreads();
    }
    if (ok) {
      // retrace of the old molecule: its own first bead (not averaged), then its orientation
      // among trials from the retrace slots
      gen_first_trials(b, W, A[0].d.seed, A[0].d.stream, move, 1, b.charge[ao.off], 1.0, b.meta[ao.off].x, true,
                       W.mx[0], W.my[0], W.mz[0]);
      trial_pass<PREC, CL>(b, W, 1, 1, ao.comp, omol);
      step_weight(W, 1, beta, ao.bias, 0.0, 1.0, true);
      bool ok2 = W.ok;
      if (ok2 && tid == 0) {
        for (int k = 0; k < 4; ++k) s_r1[k] = W.te[k];
        s_wr = W.w;
      }
      __syncthreads();
      double rosen_old = ok2 ? s_wr : 0.0;
      double r2[4] = {0, 0, 0, 0};
      if (ok2 && mso > 1) {
        gen_orientations<PREC>(b, W, A[0].d.seed, A[0].d.stream, move, ao.d.norient, mso - 1, ao.off, 1.0, 1.0, W.mx[0],
                         W.my[0], W.mz[0], true, W.mx + 1, W.my + 1, W.mz + 1, SLOT_RETRACE);
        trial_pass<PREC, CL>(b, W, ao.d.norient * (mso - 1), mso - 1, ao.comp, omol);
        step_weight(W, ao.d.norient, beta, ao.bias, 0.0, (double)ao.d.norient, true);
        ok2 = W.ok;
        if (ok2) {
          rosen_old *= W.w;
          for (int k = 0; k < 4; ++k) r2[k] = W.te[4 * W.sel + k];
        }
        __syncthreads();
      }
      if (ok2) {
        double same = 0.0, cross = 0.0;
        if (charged) ewald_delta_move<PREC, CL>(b, W, mso + msn, eik, same, cross);
        if (tid == 0) {
          double ew = 0.0;
          if (charged) {  // rigid exclusions: the new molecule arrives, the old one leaves
            if (an.rigid && an.charged) same -= an.excl;
            if (ao.rigid && ao.charged) same += ao.excl;
            ew = same + 2.0 * cross;
          }
          rosen *= exp_move(-beta * ew);
          const double pre = beta * an.big_p / (1.0 + (double)Nn) * ((double)No / (beta * ao.big_p));
          const double pacc = pre * (rosen / an.d.ideal_rosenbluth) / (rosen_old / ao.d.ideal_rosenbluth);
          s_accept = u01(wx[3]) < pacc;
          if (s_accept && an.comp != ao.comp && (Nn + 1) * msn > an.cap) {
            s_accept = 0;
            ST[en].capacity_hits++;
          }
          s_dE[0] = (s_e1[0] + s_e1[2] + e2[0] + e2[2]) - (s_r1[0] + s_r1[2] + r2[0] + r2[2]);
          s_dE[1] = (s_e1[1] + s_e1[3] + e2[1] + e2[3]) - (s_r1[1] + s_r1[3] + r2[1] + r2[3]);
          s_dE[2] = ew;
        }
      }
    }
    __syncthreads();
    if constexpr (CL > 1) cluster_sync_all();  // every CTA past its reads of this move
    if (s_accept) {
      if (an.comp != ao.comp) {  // the old molecule leaves (the last one fills its slot)
        const int last = ao.off + (No - 1) * mso;
        if (o0 != last && tid < mso) copy_atom(b, o0 + tid, last + tid, omol);
        if (tid < msn)
          store_atom(b, an.off + Nn * msn + tid, W.mx[mso + tid], W.my[mso + tid], W.mz[mso + tid],
                     b.charge[an.off + tid], 1.0, 1.0, b.meta[an.off + tid].x, Nn);
        __syncthreads();
        if (tid == 0) {
          comp_size[ao.comp] = (No - 1) * mso;
          comp_size[an.comp] = (Nn + 1) * msn;
        }
      } else if (tid < msn) {  // same species: the new configuration replaces the old one
        store_position(b, o0 + tid, W.mx[mso + tid], W.my[mso + tid], W.mz[mso + tid]);
      }
      if (charged) commit_sk<CL>(b, b.s_tmp);
      if (tid == 0) {
        ST[eo].identity_out[1]++;
        ST[en].identity_in[1]++;
        grx_gcmc_stats& sn = ST[en];
        sn.energy[0] += s_dE[0]; sn.energy[1] += s_dE[1]; sn.energy[2] += s_dE[2];
        sn.energy[3] += s_dE[0] + s_dE[1] + s_dE[2];
      }
    }
  }
}

// One block of NW warps per box (NW = 8, 12 or 24: 24 warps per SM in every shape), or,
// with CL > 1, one cluster of CL such blocks per box (launched with cluster dimension CL).
// The box's moved components are entries [first[box], first[box + 1]) of args /
// stats; every step picks one of them uniformly with word 3 of the displacement slot
// (Select_Box_Component_Molecule, axpy.cu:74-100). All entries of a box share its seed
// and stream. IDS instantiations (grx_gcmc_swap.cu) also run identity swaps
// (identity_swap_step); the others never test for them, so their code is unchanged.
//
// In a cluster every CTA runs the whole chain: the bead passes are split across the CTAs
// and their partials exchanged (trial_pass), everything else is computed redundantly from
// bitwise-identical inputs, so all CTAs take the same decisions and pass the same cluster
// barriers. Global state is written by every CTA with identical values (molecule counts
// are assigned, never incremented); a cluster barrier before each commit keeps a CTA from
// updating S(k) while a peer still reads it. Statistics are written by CTA 0.
template <int PREC, int NW, int CL = 1, bool IDS = false>
__global__ void __launch_bounds__(NW * 32, 24 / NW) gcmc_kernel(const BoxDev* boxes, const GcmcArgs* args,
                                                              const int* first, const uint64_t* step0,
                                                              int64_t nsteps, grx_gcmc_stats* stats) {
  const uint64_t first_step = *step0;
  const int box = (int)blockIdx.x / CL;
  __shared__ BoxDev b;
  __shared__ GcmcArgs A[kMaxMoved];
  __shared__ CbmcWork<NW> W;
  __shared__ grx_gcmc_stats ST[kMaxMoved];
  __shared__ int s_accept;
  __shared__ double s_e1[4], s_w1, s_dE[3], s_stored, s_r1[4], s_wr;
  extern __shared__ double2 eik[];
  const int tid = threadIdx.x;
  const int e0 = first[box], nm = first[box + 1] - e0;
  if (tid == 0) {
    b = boxes[box];
    W.cfg = 0;
    W.cbeads = 0;
  }
  if (tid < NW) stage_init(W.vst[tid]);
  stage_fence_init();
  if (tid < nm) {
    A[tid] = args[e0 + tid];
    ST[tid] = grx_gcmc_stats{};
  }
  __syncthreads();
  int* comp_size = const_cast<int*>(b.comp_size);
  const int64_t nsb = (A[0].nsteps_cap >= 0 && A[0].nsteps_cap < nsteps) ? A[0].nsteps_cap : nsteps;
  const uint64_t move0 = first_step + (uint64_t)A[0].step_off;
  for (int64_t step = 0; step < nsb; ++step) {
    const uint64_t move = move0 + (uint64_t)step;
    uint32_t w[4], w2[4], ws[4];
    draw4_dev(A[0].d.seed, A[0].d.stream, move, SLOT_MOVE, w);
    draw4_dev(A[0].d.seed, A[0].d.stream, move, SLOT_DISP, w2);
    draw4_dev(A[0].d.seed, A[0].d.stream, move, SLOT_SELECT, ws);
    const int sel = nm > 1 ? min(nm - 1, (int)(u01(w2[3]) * (double)nm)) : 0;
    const GcmcArgs& a = A[sel];
    const grx_gcmc_desc& d = a.d;
    grx_gcmc_stats& st = ST[sel];
    const int comp = a.comp, ms = a.ms, chain = ms - 1, off = a.off;
    const int N = comp_size[comp] / ms;
    const int mol = (int)(u01(w[0]) * (double)N);
    const double r = u01(w[1]);
    int kind = -1;
    if (r < d.p_translation) kind = 0;
    else if (r < d.p_rotation) kind = 1;
    else if (r < d.p_reinsertion) kind = 4;
    else if (IDS && r < d.p_identity_swap) kind = 5;
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
          rotate_axis<PREC>(vx, vy, vz, d.max_rotation[0] * 2.0 * (u01(w2[0]) - 0.5), 0);
          rotate_axis<PREC>(vx, vy, vz, d.max_rotation[1] * 2.0 * (u01(w2[1]) - 0.5), 1);
          rotate_axis<PREC>(vx, vy, vz, d.max_rotation[2] * 2.0 * (u01(w2[2]) - 0.5), 2);
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
      // te[0..3] new, te[4..7] old; the new configuration may stop at an overlap (the move is
      // then rejected), the old one is evaluated in full
      trial_pass<PREC, CL>(b, W, 2 * ms, ms, comp, mol, 1);
      if (!W.tflag[0]) {
        double same = 0.0, cross = 0.0;
        if (a.charged) ewald_delta_move<PREC, CL>(b, W, 2 * ms, eik, same, cross);
        if (tid == 0) {
          const double dv = (W.te[0] + W.te[2]) - (W.te[4] + W.te[6]);
          const double dr = (W.te[1] + W.te[3]) - (W.te[5] + W.te[7]);
          const double ew = same + 2.0 * cross;
          const double pacc = exp_move(-d.beta * (dv + dr + ew));
          s_accept = uacc < pacc;
          s_dE[0] = dv; s_dE[1] = dr; s_dE[2] = ew;
        }
      }
      __syncthreads();
      if constexpr (CL > 1) cluster_sync_all();  // every CTA past its reads of this move
      if (s_accept) {
        if (tid < ms) store_position(b, m0 + tid, W.mx[ms + tid], W.my[ms + tid], W.mz[ms + tid]);
        if (a.charged) commit_sk<CL>(b, b.s_tmp);
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
      trial_pass<PREC, CL>(b, W, d.ntrials, 1, comp, mol);
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
        gen_orientations<PREC>(b, W, d.seed, d.stream, move, d.norient, chain, off, 1.0, 1.0, fx, fy, fz, false, nullptr,
                         nullptr, nullptr);
        trial_pass<PREC, CL>(b, W, d.norient * chain, chain, comp, mol);
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
        trial_pass<PREC, CL>(b, W, 1, 1, comp, mol);
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
          gen_orientations<PREC>(b, W, d.seed, d.stream, move, d.norient, chain, off, 1.0, 1.0, W.mx[0], W.my[0], W.mz[0],
                           true, W.mx + 1, W.my + 1, W.mz + 1, SLOT_RETRACE);
          trial_pass<PREC, CL>(b, W, d.norient * chain, chain, comp, mol);
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
          if (a.charged) ewald_delta_move<PREC, CL>(b, W, 2 * ms, eik, same, cross);
          if (tid == 0) {
            const double ew = a.charged ? same + 2.0 * cross : 0.0;
            rosen *= exp_move(-d.beta * ew);
            const double pacc = rosen / rosen_old;
            s_accept = uacc < pacc;
            s_dE[0] = s_e1[0] + s_e1[2] + e2[0] + e2[2] - (s_r1[0] + s_r1[2] + r2[0] + r2[2]);
            s_dE[1] = s_e1[1] + s_e1[3] + e2[1] + e2[3] - (s_r1[1] + s_r1[3] + r2[1] + r2[3]);
            s_dE[2] = ew;
          }
        }
      }
      __syncthreads();
      if constexpr (CL > 1) cluster_sync_all();  // every CTA past its reads of this move
      if (s_accept) {
        if (tid < ms) store_position(b, m0 + tid, W.mx[ms + tid], W.my[ms + tid], W.mz[ms + tid]);
        if (a.charged) commit_sk<CL>(b, b.s_tmp);
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
      trial_pass<PREC, CL>(b, W, d.ntrials, 1, comp, newmol);
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
        gen_orientations<PREC>(b, W, d.seed, d.stream, move, d.norient, chain, off, 1.0, 1.0, fx, fy, fz, del,
                         W.mx + 1, W.my + 1, W.mz + 1);
        trial_pass<PREC, CL>(b, W, d.norient * chain, chain, comp, newmol);
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
        if (a.charged) ewald_delta_move<PREC, CL>(b, W, ms, eik, same, cross);
        if (tid == 0) {
          double ew = 0.0;
          if (a.charged) {
            if (a.rigid) same -= a.excl * (del ? (0.0 - 1.0) : (1.0 - 0.0));
            ew = same + 2.0 * cross;
          }
          double pacc;
          if (!del) {
            rosen *= exp_move(-d.beta * ew);
            rosen *= exp_move(-d.beta * d.tail_insert);
            pacc = d.beta * a.big_p / (1.0 + (double)N) * rosen / d.ideal_rosenbluth;
            s_accept = rosen > 1e-150 && uacc < pacc;
            if (s_accept && (N + 1) * ms > a.cap) {
              s_accept = 0;
              st.capacity_hits++;
            }
          } else {
            rosen /= exp_move(-d.beta * ew);
            rosen /= exp_move(d.beta * d.tail_insert);  // the deletion's tail difference is -tail_insert
            pacc = (double)N / (d.beta * a.big_p) * d.ideal_rosenbluth / rosen;
            s_accept = uacc < pacc;
          }
          const double ev = s_e1[0] + s_e1[2] + e2[0] + e2[2];
          const double er = s_e1[1] + s_e1[3] + e2[1] + e2[3];
          const double sg = del ? -1.0 : 1.0;
          s_dE[0] = sg * ev; s_dE[1] = sg * er; s_dE[2] = ew;
        }
      }
      if (!del && tid == 0) {  // RecordRosen of the insertion: W, 0 when the growth failed
        const double wr = ok ? rosen : 0.0;
        st.rosen[0] += wr;
        st.rosen[1] += wr * wr;
        st.rosen[2] += 1.0;
      }
      __syncthreads();
      if constexpr (CL > 1) cluster_sync_all();  // every CTA past its reads of this move
      if (s_accept) {
        if (!del) {
          if (tid < ms)
            store_atom(b, off + N * ms + tid, W.mx[tid], W.my[tid], W.mz[tid], b.charge[off + tid], 1.0, 1.0,
                       b.meta[off + tid].x, N);
          __syncthreads();
          if (tid == 0) comp_size[comp] = (N + 1) * ms;
        } else {
          const int last = off + (N - 1) * ms;
          if (m0 != last && tid < ms) copy_atom(b, m0 + tid, last + tid, mol);
          __syncthreads();
          if (tid == 0) comp_size[comp] = (N - 1) * ms;
        }
        if (a.charged) commit_sk<CL>(b, b.s_tmp);
        if (tid == 0) {
          st.accepted[kind]++;
          st.energy[0] += s_dE[0]; st.energy[1] += s_dE[1]; st.energy[2] += s_dE[2];
          st.energy[3] += s_dE[0] + s_dE[1] + s_dE[2];
        }
      }
    } else if (IDS && kind == 5) {
      if constexpr (IDS)
        identity_swap_step<PREC, CL>(b, A, nm, ST, W, eik, comp_size, move, d.beta, u01(ws[1]), s_accept, s_e1,
                                     s_w1, s_dE, s_r1, s_wr);
    }
    __syncthreads();
    if (tid < nm) ST[tid].sum_n += (double)(comp_size[A[tid].comp] / A[tid].ms);
    if (tid == 0) {
      st.trial_configs += W.cfg;
      st.trial_beads += W.cbeads;
      W.cfg = 0;
      W.cbeads = 0;
    }
    __syncthreads();
  }
  if (tid < nm && (CL == 1 || cluster_rank() == 0)) {  // accumulate into the caller's running statistics
    grx_gcmc_stats& o = stats[e0 + tid];
    for (int k = 0; k < 5; ++k) {
      o.attempts[k] += ST[tid].attempts[k];
      o.accepted[k] += ST[tid].accepted[k];
    }
    for (int k = 0; k < 4; ++k) o.energy[k] += ST[tid].energy[k];
    for (int k = 0; k < 3; ++k) o.rosen[k] += ST[tid].rosen[k];
    o.trial_configs += ST[tid].trial_configs;
    o.trial_beads += ST[tid].trial_beads;
    o.capacity_hits += ST[tid].capacity_hits;
    o.sum_n += ST[tid].sum_n;
    for (int k = 0; k < 2; ++k) {
      o.identity_out[k] += ST[tid].identity_out[k];
      o.identity_in[k] += ST[tid].identity_in[k];
    }
    o.n_molecules = comp_size[A[tid].comp] / A[tid].ms;
  }
}

}  // namespace grx

namespace grx {
// Cluster launches (grx_gcmc_cluster.cu): one cluster of `cl` CTAs of 24 warps per box.
cudaError_t launch_gcmc_cluster(grx_precision prec, int cl, int nboxes, const BoxDev* dboxes, const GcmcArgs* dargs,
                                const int* dfirst, const uint64_t* dstep, int64_t nsteps, grx_gcmc_stats* dstats,
                                size_t smem, cudaStream_t stream);
cudaError_t set_gcmc_cluster_smem(size_t dyn_smem);
// Launches of the kernel with identity swaps (grx_gcmc_swap.cu): one block of nw warps per box,
// or one cluster of cl CTAs of 24 warps.
cudaError_t launch_gcmc_swap(grx_precision prec, int nw, int nboxes, const BoxDev* dboxes, const GcmcArgs* dargs,
                             const int* dfirst, const uint64_t* dstep, int64_t nsteps, grx_gcmc_stats* dstats,
                             size_t smem, cudaStream_t stream);
cudaError_t launch_gcmc_swap_cluster(grx_precision prec, int cl, int nboxes, const BoxDev* dboxes,
                                     const GcmcArgs* dargs, const int* dfirst, const uint64_t* dstep, int64_t nsteps,
                                     grx_gcmc_stats* dstats, size_t smem, cudaStream_t stream);
cudaError_t set_gcmc_swap_smem(size_t dyn_smem);
// Clusters of `cl` CTAs that can be resident at once with `smem` bytes of dynamic shared memory.
int gcmc_cluster_capacity(grx_precision prec, int cl, size_t smem);
}  // namespace grx
