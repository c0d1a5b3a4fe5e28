// grx_pair.cu -- stand-alone pair-energy entry points: CBMC trial energies and the
// single-molecule move delta (the reference's per-move kernels, one call each).
#include <algorithm>
#include <cmath>
#include <vector>

#include "grx_host.h"
#include "grx_warp.cuh"

namespace grx {

// Fixed-order reduction: trial t, quantity q = sum over blocks, then chain beads.
__global__ void trial_reduce_kernel(const double* part, const int* flags, int nblk, int nb, int chain,
                                    double* out, int* tflag) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  const int ntr = nb / chain;
  if (w >= ntr * 4) return;
  const int t = w >> 2, q = w & 3;
  double s = 0.0;
  for (int a = 0; a < chain; ++a) {
    const int bead = t * chain + a;
    double sb = 0.0;
    for (int k = 0; k < nblk; ++k) sb += part[((size_t)k * nb + bead) * 4 + q];
    s += sb;
  }
  out[t * 4 + q] = s;
  if (q == 0) {
    int f = 0;
    for (int a = 0; a < chain; ++a) f |= flags[t * chain + a];
    tflag[t] = f;
  }
}

// Single-molecule delta: beads [0, ms) are the new molecule, [ms, 2 ms) the old
// one; slot of an atom: HH / HG / GG by its component and the moved component
// (mc_single_particle.h:142-170). part[block][6], flag from new beads only.
template <int PREC>
__global__ void __launch_bounds__(GRX_THREADS) single_body_kernel(BoxDev b, const Bead* beads, int ms,
                                                                  int do_new, int do_old, int component,
                                                                  int new_mol, int old_mol, double* part,
                                                                  int* flag_out) {
  __shared__ double sbuf[32];
  const int nb = 2 * ms;
  const int nl = blockDim.x / nb;
  const int tid = threadIdx.x;
  double e[6] = {0, 0, 0, 0, 0, 0};
  int flag = 0;
  if (tid < nl * nb) {
    const int bead = tid % nb;
    const bool is_new = bead < ms;
    if ((is_new && do_new) || (!is_new && do_old)) {
      const Bead bd = beads[bead];
      const bool moved_host = component < b.nhost;
      const int mol = is_new ? new_mol : old_mol;
      for (int c = 0; c < b.ncomp; ++c) {
        const bool host = c < b.nhost;
        const int slot = moved_host ? (host ? 0 : 1) : (host ? 1 : 2);
        const int n = b.comp_size[c];
        const int off = b.comp_off[c];
        double v = 0.0, r = 0.0;
        int f = 0;
        for (int i = blockIdx.x * nl + tid / nb; i < n; i += gridDim.x * nl) {
          if (c == component && b.meta[off + i].y == mol) continue;
          pair_energy<PREC>(b, off + i, bd, 0, v, r, f);
        }
        const double sg = is_new ? 1.0 : -1.0;
        e[2 * slot] += sg * v;
        e[2 * slot + 1] += sg * r;
        if (is_new) flag |= f;
      }
    }
  }
  if (flag) atomicOr(flag_out, 1);
  for (int k = 0; k < 6; ++k) {
    const double v = block_sum(e[k], sbuf);
    if (tid == 0) part[6 * blockIdx.x + k] = v;
  }
}

static void host_split(double x, float& h, float& l) {
  const double hd = std::nearbyint(x * GRX_GRID_COORD) / GRX_GRID_COORD;
  h = (float)hd;
  l = (float)(x - hd);
}

static grx_status stage_beads(const grx_trials* t, size_t first_bead, size_t nbeads, double prefactor,
                              std::vector<Bead>& out) {
  const size_t nall = t->ntrials * t->chainsize;
  std::vector<double> pos(3 * nall), sc(nall, 1.0), q(nall, 0.0), scc(nall, 1.0);
  std::vector<size_t> ty(nall, 0);
  if (nall) {
    GRX_CHECK_CUDA(cudaMemcpy(pos.data(), t->pos, 3 * nall * sizeof(double), cudaMemcpyDefault), "read bead pos");
    if (t->scale) GRX_CHECK_CUDA(cudaMemcpy(sc.data(), t->scale, nall * sizeof(double), cudaMemcpyDefault), "read bead scale");
    if (t->charge) GRX_CHECK_CUDA(cudaMemcpy(q.data(), t->charge, nall * sizeof(double), cudaMemcpyDefault), "read bead charge");
    if (t->scale_coul) GRX_CHECK_CUDA(cudaMemcpy(scc.data(), t->scale_coul, nall * sizeof(double), cudaMemcpyDefault), "read bead scaleCoul");
    GRX_CHECK_CUDA(cudaMemcpy(ty.data(), t->type, nall * sizeof(size_t), cudaMemcpyDefault), "read bead type");
  }
  out.resize(nbeads);
  for (size_t k = 0; k < nbeads; ++k) {
    const size_t j = first_bead + k;
    Bead& bd = out[k];
    bd.x = pos[3 * j]; bd.y = pos[3 * j + 1]; bd.z = pos[3 * j + 2];
    host_split(bd.x, bd.h.x, bd.l.x);
    host_split(bd.y, bd.h.y, bd.l.y);
    host_split(bd.z, bd.h.z, bd.l.z);
    bd.q = q[j] * scc[j];
    bd.scale = sc[j];
    bd.type = (int)ty[j];
    const double pq = prefactor * bd.q;
    const float ph = (float)pq;
    bd.pq = make_float2(ph, (float)(pq - (double)ph));
    bd.unit = bd.scale == 1.0;
  }
  return GRX_OK;
}

template <int PREC>
static void launch_trial_pass(grx_box* b, const Bead* beads, int nb, int comp, int newmol, int ec, int em,
                              double* part, int* flags) {
  trial_bead_kernel<PREC><<<nb, GRX_THREADS, 0, b->stream>>>(b->dev, beads, comp, newmol, ec, em, part, flags);
}

}  // namespace grx

using namespace grx;

extern "C" {

grx_status grx_trial_energies(grx_box* b, const grx_trials* t, int32_t component, int64_t exclude_comp,
                              int64_t exclude_molid, grx_precision prec, grx_trial_energy* out,
                              uint8_t* overlap) {
  GRX_REQUIRE(b && t && out && overlap, "grx_trial_energies: null argument");
  GRX_REQUIRE(t->chainsize >= 1 && t->chainsize <= GRX_MAX_TRIAL_BEADS,
              "grx_trial_energies: chainsize out of range");
  GRX_REQUIRE(t->ntrials == 0 || (t->pos && t->type), "grx_trial_energies: bead arrays missing");
  GRX_REQUIRE(prec == GRX_FP64 || prec == GRX_MIXED || prec == GRX_FP32, "grx_trial_energies: bad precision");
  GRX_REQUIRE(component >= 0 && component < b->ncomp, "grx_trial_energies: component out of range");
  if (t->ntrials == 0) return GRX_OK;
  refresh_dev(b);
  const size_t ch = t->chainsize;
  const size_t per_chunk = std::max<size_t>(1, GRX_MAX_TRIAL_BEADS / ch);
  std::vector<double> host_out;
  std::vector<int> host_flag;
  for (size_t t0 = 0; t0 < t->ntrials; t0 += per_chunk) {
    const size_t ntr = std::min(per_chunk, t->ntrials - t0);
    const int nb = (int)(ntr * ch);
    std::vector<Bead> beads;
    grx_status st = stage_beads(t, t0 * ch, nb, b->dev.prefactor, beads);
    if (st) return st;
    const int nblk = 1;
    const size_t bead_bytes = (nb * sizeof(Bead) + 255) / 256 * 256;
    const size_t part_bytes = ((size_t)nblk * nb * 4 * sizeof(double) + 255) / 256 * 256;
    const size_t flag_bytes = ((size_t)nb * sizeof(int) + 255) / 256 * 256;
    const size_t out_bytes = ntr * 4 * sizeof(double) + ntr * sizeof(int);
    st = ensure_scratch(b, bead_bytes + part_bytes + flag_bytes + out_bytes + 256);
    if (st) return st;
    char* base = (char*)b->scratch;
    Bead* d_beads = (Bead*)base;
    double* part = (double*)(base + bead_bytes);
    int* flags = (int*)(base + bead_bytes + part_bytes);
    double* d_out = (double*)(base + bead_bytes + part_bytes + flag_bytes);
    int* d_tflag = (int*)(d_out + ntr * 4);
    GRX_CHECK_CUDA(cudaMemcpyAsync(d_beads, beads.data(), nb * sizeof(Bead), cudaMemcpyHostToDevice, b->stream), "upload beads");
    GRX_CHECK_CUDA(cudaMemsetAsync(flags, 0, nb * sizeof(int), b->stream), "clear flags");
    const int ec = (int)exclude_comp, em = (int)exclude_molid;
    if (prec == GRX_FP64) launch_trial_pass<GRX_FP64>(b, d_beads, nb, component, (int)t->molid, ec, em, part, flags);
    else if (prec == GRX_MIXED) launch_trial_pass<GRX_MIXED>(b, d_beads, nb, component, (int)t->molid, ec, em, part, flags);
    else launch_trial_pass<GRX_FP32>(b, d_beads, nb, component, (int)t->molid, ec, em, part, flags);
    trial_reduce_kernel<<<(int)((ntr * 4 + 127) / 128), 128, 0, b->stream>>>(part, flags, nblk, nb, (int)ch, d_out, d_tflag);
    count_launch(2);
    GRX_CHECK_CUDA(cudaGetLastError(), "trial energy launch");
    std::vector<double> eo(ntr * 4);
    std::vector<int> fo(ntr);
    GRX_CHECK_CUDA(cudaMemcpyAsync(eo.data(), d_out, ntr * 4 * sizeof(double), cudaMemcpyDeviceToHost, b->stream), "read energies");
    GRX_CHECK_CUDA(cudaMemcpyAsync(fo.data(), d_tflag, ntr * sizeof(int), cudaMemcpyDeviceToHost, b->stream), "read flags");
    GRX_CHECK_CUDA(cudaStreamSynchronize(b->stream), "trial energies");
    host_out.insert(host_out.end(), eo.begin(), eo.end());
    host_flag.insert(host_flag.end(), fo.begin(), fo.end());
  }
  std::vector<uint8_t> f8(t->ntrials);
  for (size_t k = 0; k < t->ntrials; ++k) f8[k] = host_flag[k] ? 1 : 0;
  GRX_CHECK_CUDA(cudaMemcpy(out, host_out.data(), t->ntrials * sizeof(grx_trial_energy), cudaMemcpyDefault), "write energies");
  GRX_CHECK_CUDA(cudaMemcpy(overlap, f8.data(), t->ntrials, cudaMemcpyDefault), "write flags");
  return GRX_OK;
}

grx_status grx_single_body_energy(grx_box* b, const grx_trials* old_mol, const grx_trials* new_mol,
                                  int32_t component, int32_t do_new, int32_t do_old, grx_precision prec,
                                  double* out6, uint8_t* overlap) {
  GRX_REQUIRE(b && old_mol && new_mol && out6 && overlap, "grx_single_body_energy: null argument");
  GRX_REQUIRE(component >= 0 && component < b->ncomp, "grx_single_body_energy: component out of range");
  const size_t ms = new_mol->chainsize;
  GRX_REQUIRE(ms >= 1 && 2 * ms <= GRX_THREADS && old_mol->chainsize == ms,
              "grx_single_body_energy: molecule size out of range");
  GRX_REQUIRE(do_new || do_old, "grx_single_body_energy: nothing to do");
  refresh_dev(b);
  std::vector<Bead> nb_, ob_;
  grx_status st = stage_beads(new_mol, 0, ms, b->dev.prefactor, nb_);
  if (st) return st;
  st = stage_beads(old_mol, 0, ms, b->dev.prefactor, ob_);
  if (st) return st;
  nb_.insert(nb_.end(), ob_.begin(), ob_.end());
  size_t total_atoms = 0;
  for (int c = 0; c < b->ncomp; ++c) total_atoms += b->cap[c];
  const int nl = GRX_THREADS / (int)(2 * ms);
  int nblk = (int)std::min<size_t>((total_atoms + (size_t)nl * 16 - 1) / ((size_t)nl * 16), 2 * (size_t)sm_count(b));
  nblk = std::max(nblk, 1);
  const size_t bead_bytes = (2 * ms * sizeof(Bead) + 255) / 256 * 256;
  st = ensure_scratch(b, bead_bytes + 6 * nblk * sizeof(double) + 256);
  if (st) return st;
  Bead* d_beads = (Bead*)b->scratch;
  double* part = (double*)((char*)b->scratch + bead_bytes);
  int* d_flag = (int*)(part + 6 * nblk);
  GRX_CHECK_CUDA(cudaMemcpyAsync(d_beads, nb_.data(), 2 * ms * sizeof(Bead), cudaMemcpyHostToDevice, b->stream), "upload beads");
  GRX_CHECK_CUDA(cudaMemsetAsync(d_flag, 0, sizeof(int), b->stream), "clear flag");
  const int nm = (int)new_mol->molid, om = (int)old_mol->molid;
  if (prec == GRX_FP64)
    single_body_kernel<GRX_FP64><<<nblk, GRX_THREADS, 0, b->stream>>>(b->dev, d_beads, (int)ms, do_new, do_old, component, nm, om, part, d_flag);
  else if (prec == GRX_MIXED)
    single_body_kernel<GRX_MIXED><<<nblk, GRX_THREADS, 0, b->stream>>>(b->dev, d_beads, (int)ms, do_new, do_old, component, nm, om, part, d_flag);
  else
    single_body_kernel<GRX_FP32><<<nblk, GRX_THREADS, 0, b->stream>>>(b->dev, d_beads, (int)ms, do_new, do_old, component, nm, om, part, d_flag);
  count_launch();
  GRX_CHECK_CUDA(cudaGetLastError(), "single body launch");
  std::vector<double> parts(6 * nblk);
  int flag = 0;
  GRX_CHECK_CUDA(cudaMemcpyAsync(parts.data(), part, 6 * nblk * sizeof(double), cudaMemcpyDeviceToHost, b->stream), "read partials");
  GRX_CHECK_CUDA(cudaMemcpyAsync(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, b->stream), "read flag");
  GRX_CHECK_CUDA(cudaStreamSynchronize(b->stream), "single body");
  double e[6] = {0, 0, 0, 0, 0, 0};
  for (int k = 0; k < nblk; ++k)
    for (int q = 0; q < 6; ++q) e[q] += parts[6 * k + q];
  GRX_CHECK_CUDA(cudaMemcpy(out6, e, 6 * sizeof(double), cudaMemcpyDefault), "write energies");
  uint8_t f8 = flag ? 1 : 0;
  GRX_CHECK_CUDA(cudaMemcpy(overlap, &f8, 1, cudaMemcpyDefault), "write flag");
  return GRX_OK;
}

}  // extern "C"
