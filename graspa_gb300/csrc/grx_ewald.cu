// grx_ewald.cu -- Ewald Fourier-space kernels (structure factors, move delta,
// commit) and the FP64 totals used for drift checks.
#include <algorithm>
#include <cmath>
#include <vector>

#include "grx_host.h"

namespace grx {

constexpr int kBigMolecule = 64;  // molecules above this size get the pair-parallel exclusion

struct CompRanges {  // live atoms of every component, compact numbering
  int n;                                // total live atoms
  int ncomp, nhost;
  int off[GRX_MAX_COMPONENTS];          // storage offset
  int base[GRX_MAX_COMPONENTS + 1];     // compact offset
  int molsize[GRX_MAX_COMPONENTS];
};

__device__ __forceinline__ int comp_of(const CompRanges& r, int j, int& local) {
  int c = 0;
  while (c + 1 < r.ncomp && j >= r.base[c + 1]) ++c;
  local = j - r.base[c];
  return c;
}

// eik tables of every live atom: e^{i k s} for k = 0..kmax per axis by the
// recurrence of Initialize_Vectors (Ewald_Energy_Functions.h:42-95).
__global__ void eik_tables_kernel(BoxDev b, CompRanges r, double2* ex, double2* ey, double2* ez) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= r.n) return;
  int local;
  const int c = comp_of(r, j, local);
  const double4 p = atom_pos64(b, r.off[c] + local);
  const double PI2 = 2.0 * 3.14159265358979323846;
  double s[3];
  s[0] = (b.inv[0] * p.x + b.inv[3] * p.y + b.inv[6] * p.z) * PI2;
  s[1] = (b.inv[1] * p.x + b.inv[4] * p.y + b.inv[7] * p.z) * PI2;
  s[2] = (b.inv[2] * p.x + b.inv[5] * p.y + b.inv[8] * p.z) * PI2;
  double2* t[3] = {ex, ey, ez};
  for (int d = 0; d < 3; ++d) {
    const int km = b.kmax[d];
    const size_t n = r.n;
    t[d][j] = make_double2(1.0, 0.0);
    if (km >= 1) {
      double sn, cs;
      sincos(s[d], &sn, &cs);
      const double2 e1 = make_double2(cs, sn);
      t[d][j + n] = e1;
      double2 e = e1;
      for (int k = 2; k <= km; ++k) {
        e = cmul(e, e1);
        t[d][j + k * n] = e;
      }
    }
  }
}

__device__ __forceinline__ double2 eik_term(const double2* ex, const double2* ey, const double2* ez,
                                            size_t n, size_t j, int kx, int ky, int kz) {
  double2 y = ey[j + n * (size_t)abs(ky)];
  if (ky < 0) y.y = -y.y;
  double2 z = ez[j + n * (size_t)abs(kz)];
  if (kz < 0) z.y = -z.y;
  return cmul(cmul(ex[j + n * (size_t)kx], y), z);
}

// Structure factors per active k, split framework / adsorbate (Ewald_Total,
// ewald_preparation.h:128-147). One block per active k, deterministic sums.
__global__ void __launch_bounds__(GRX_THREADS) sk_kernel(BoxDev b, CompRanges r, const double2* ex,
                                                         const double2* ey, const double2* ez) {
  __shared__ double sbuf[32];
  const int4 k = b.kact[blockIdx.x];
  double fr = 0, fi = 0, ar = 0, ai = 0;
  const int nhost_atoms = r.base[r.nhost];
  for (int j = threadIdx.x; j < r.n; j += blockDim.x) {
    int local;
    const int c = comp_of(r, j, local);
    const double q = atom_pos64(b, r.off[c] + local).w;
    const double2 t = eik_term(ex, ey, ez, r.n, j, k.x, k.y, k.z);
    if (j < nhost_atoms) { fr += q * t.x; fi += q * t.y; }
    else { ar += q * t.x; ai += q * t.y; }
  }
  fr = block_sum(fr, sbuf);
  fi = block_sum(fi, sbuf);
  ar = block_sum(ar, sbuf);
  ai = block_sum(ai, sbuf);
  if (threadIdx.x == 0) {
    if (!b.shared_host) b.s_fw[k.w] = make_double2(fr, fi);  // a replica reads its parent's
    b.s_ads[k.w] = make_double2(ar, ai);
    b.s_tmp[k.w] = make_double2(ar, ai);
  }
}

// Self energy and intramolecular erf exclusion per atom (ewald_preparation.h:189-249),
// partial sums per block: [self_all, self_host, excl_all, excl_host].
__global__ void __launch_bounds__(GRX_THREADS) self_excl_kernel(BoxDev b, CompRanges r, double* part) {
  __shared__ double sbuf[32];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  double sa = 0, sh = 0, ea = 0, eh = 0;
  if (j < r.n) {
    int local;
    const int c = comp_of(r, j, local);
    const double4 p = atom_pos64(b, r.off[c] + local);
    const double pself = b.prefactor * b.alpha / sqrt(3.14159265358979323846);
    const double v = pself * p.w * p.w;
    sa = v;
    if (c < r.nhost) sh = v;
    const int ms = r.molsize[c];
    const int mol0 = (local / ms) * ms;
    const int lend = ms > kBigMolecule ? local + 1 : min(mol0 + ms, r.base[c + 1] - r.base[c]);
    for (int l2 = local + 1; l2 < lend; ++l2) {
      const double4 q = atom_pos64(b, r.off[c] + l2);
      double x = p.x - q.x, y = p.y - q.y, z = p.z - q.z;
      pbc64(b, x, y, z);
      const double rr = sqrt(x * x + y * y + z * z);
      const double e = b.prefactor * p.w * q.w * erf(b.alpha * rr) / rr;
      ea += e;
      if (c < r.nhost) eh += e;
    }
  }
  sa = block_sum(sa, sbuf);
  sh = block_sum(sh, sbuf);
  ea = block_sum(ea, sbuf);
  eh = block_sum(eh, sbuf);
  if (threadIdx.x == 0) {
    part[4 * blockIdx.x + 0] = sa;
    part[4 * blockIdx.x + 1] = sh;
    part[4 * blockIdx.x + 2] = ea;
    part[4 * blockIdx.x + 3] = eh;
  }
}

// Intramolecular erf exclusion of the molecules of one component with more than
// kBigMolecule atoms (a framework is one such molecule): the pairs i < j of each
// molecule spread over the whole grid instead of one thread per atom.
// part per block: [excl_all, excl_host].
__global__ void __launch_bounds__(GRX_THREADS) big_excl_kernel(BoxDev b, CompRanges r, int c, double* part) {
  __shared__ double sbuf[32];
  const int ms = r.molsize[c];
  const int n = r.base[c + 1] - r.base[c];
  const long long nmol = (n + ms - 1) / ms;
  const long long npair = nmol * (long long)ms * ms;
  double ea = 0.0;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npair;
       p += (long long)gridDim.x * blockDim.x) {
    const long long m = p / ((long long)ms * ms);
    const int rem = (int)(p - m * (long long)ms * ms);
    const int i = rem / ms, j = rem - i * ms;
    const int li = (int)(m * ms) + i, lj = (int)(m * ms) + j;
    if (j <= i || lj >= n) continue;
    const double4 a = atom_pos64(b, r.off[c] + li);
    const double4 q = atom_pos64(b, r.off[c] + lj);
    double x = a.x - q.x, y = a.y - q.y, z = a.z - q.z;
    pbc64(b, x, y, z);
    const double rr = sqrt(x * x + y * y + z * z);
    ea += b.prefactor * a.w * q.w * erf(b.alpha * rr) / rr;
  }
  ea = block_sum(ea, sbuf);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x + 0] = ea;
    part[2 * blockIdx.x + 1] = c < r.nhost ? ea : 0.0;
  }
}

// Total VDW + real Coulomb over ordered pairs with factor 0.5 (VDWReal_Total_CPU,
// VDW_Coulomb.cu:34-226; device form Total_VDW_Coulomb_Energy :1580-1665).
// part per block: hh_v hh_r hg_v hg_r gg_v gg_r, then per block an overlap flag (a pair
// with an adsorbate atom above the overlap criterion or closer than 0.1 A,
// VDWCoulEnergy_Total :1385-1386).
__global__ void __launch_bounds__(GRX_THREADS) vdw_real_total_kernel(BoxDev b, CompRanges r, double* part) {
  __shared__ double sbuf[32];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  double e[6] = {0, 0, 0, 0, 0, 0};
  int ovl = 0;
  if (j < r.n) {
    int li;
    const int ci = comp_of(r, j, li);
    const int ii = r.off[ci] + li;
    const double4 p = atom_pos64(b, ii);
    const int2 mi = atom_meta(b, ii);
    const double si = atom_scale(b, ii);
    for (int cj = 0; cj < r.ncomp; ++cj) {
      int it;
      if (ci < r.nhost || cj < r.nhost) it = (!(ci < r.nhost) || !(cj < r.nhost)) ? 1 : 0;
      else it = 2;
      const int nj = r.base[cj + 1] - r.base[cj];
      for (int lj = 0; lj < nj; ++lj) {
        const int jj = r.off[cj] + lj;
        const int2 mj = atom_meta(b, jj);
        if (mi.y == mj.y && ci == cj) continue;
        const double4 q = atom_pos64(b, jj);
        double x = p.x - q.x, y = p.y - q.y, z = p.z - q.z;
        pbc64(b, x, y, z);
        const double rr = x * x + y * y + z * z;
        if (rr < b.cut_vdw2) {
          const double ev = vdw64(b, mi.x * b.ntypes + mj.x, rr, si * atom_scale(b, jj));
          e[2 * it] += 0.5 * ev;
          if (it > 0 && (ev > b.overlap || rr < 0.01)) ovl = 1;
        }
        if (!b.no_charges && rr < b.cut_coul2) e[2 * it + 1] += 0.5 * coul64(b, p.w * q.w, rr);
      }
    }
  }
  for (int k = 0; k < 6; ++k) {
    const double v = block_sum(e[k], sbuf);
    if (threadIdx.x == 0) part[6 * blockIdx.x + k] = v;
  }
  ovl = __syncthreads_or(ovl);
  if (threadIdx.x == 0) part[6 * gridDim.x + blockIdx.x] = ovl ? 1.0 : 0.0;
}

// Fourier delta of one move (Fourier_Ewald_Diff, Ewald_Energy_Functions.h:280-397):
// every block rebuilds the eik tables of the few moved atoms in shared memory, then
// handles a strided subset of the active k. part per block: {same, cross}.
struct MoveAtoms {
  int n_old, n_new;
  double x[2 * GRX_MAX_MOLSIZE], y[2 * GRX_MAX_MOLSIZE], z[2 * GRX_MAX_MOLSIZE], q[2 * GRX_MAX_MOLSIZE];
};

__global__ void __launch_bounds__(GRX_THREADS) ewald_delta_kernel(BoxDev b, const MoveAtoms* mv,
                                                                  const double2* s_same,
                                                                  const double2* s_cross,
                                                                  double2* s_out, double* part) {
  extern __shared__ double2 eik_s[];
  __shared__ double sbuf[32];
  const int na = mv->n_old + mv->n_new;
  const int kx1 = b.kmax[0] + 1, ky1 = b.kmax[1] + 1;
  double2* ex = eik_s;
  double2* ey = ex + kx1 * na;
  double2* ez = ey + ky1 * na;
  const double PI2 = 2.0 * 3.14159265358979323846;
  for (int t = threadIdx.x; t < 3 * na; t += blockDim.x) {
    const int a = t % na, d = t / na;
    const double px = mv->x[a], py = mv->y[a], pz = mv->z[a];
    const double s = (b.inv[d] * px + b.inv[3 + d] * py + b.inv[6 + d] * pz) * PI2;
    double2* tab = d == 0 ? ex : (d == 1 ? ey : ez);
    const int km = b.kmax[d];
    tab[a] = make_double2(1.0, 0.0);
    if (km >= 1) {
      double sn, cs;
      sincos(s, &sn, &cs);
      const double2 e1 = make_double2(cs, sn);
      double2 e = e1;
      tab[a + na] = e1;
      for (int k = 2; k <= km; ++k) {
        e = cmul(e, e1);
        tab[a + k * na] = e;
      }
    }
  }
  __syncthreads();
  double same = 0.0, cross = 0.0;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < b.nact; j += gridDim.x * blockDim.x) {
    const int4 k = b.kact[j];
    double2 co = make_double2(0, 0), cn = make_double2(0, 0);
    for (int a = 0; a < na; ++a) {
      const double2 t = eik_term(ex, ey, ez, na, a, k.x, k.y, k.z);
      const double q = mv->q[a];
      if (a < mv->n_old) { co.x += q * t.x; co.y += q * t.y; }
      else { cn.x += q * t.x; cn.y += q * t.y; }
    }
    const double tmp = b.ktemp[j];
    const double2 ov = s_same[k.w];
    const double2 nv = make_double2(ov.x + cn.x - co.x, ov.y + cn.y - co.y);
    same += tmp * (nv.x * nv.x + nv.y * nv.y);
    same -= tmp * (ov.x * ov.x + ov.y * ov.y);
    s_out[k.w] = nv;
    const double2 xv = s_cross[k.w];
    cross += tmp * (xv.x * (cn.x - co.x) + xv.y * (cn.y - co.y));
  }
  same = block_sum(same, sbuf);
  cross = block_sum(cross, sbuf);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = same;
    part[2 * blockIdx.x + 1] = cross;
  }
}

__global__ void commit_kernel(BoxDev b, double2* dst, const double2* src) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < b.nact; j += gridDim.x * blockDim.x) {
    const int slot = b.kact[j].w;
    dst[slot] = src[slot];
  }
}

static CompRanges ranges(grx_box* b) {
  CompRanges r{};
  r.ncomp = b->ncomp;
  r.nhost = b->nhost;
  int acc = 0;
  for (int c = 0; c < b->ncomp; ++c) {
    r.off[c] = (int)b->off[c];
    r.base[c] = acc;
    r.molsize[c] = (int)b->molsize[c];
    acc += b->size[c];
  }
  r.base[b->ncomp] = acc;
  r.n = acc;
  return r;
}

static grx_status sync_sizes(grx_box* b) {
  GRX_CHECK_CUDA(cudaMemcpyAsync(b->size, b->d_size, GRX_MAX_COMPONENTS * sizeof(int),
                                 cudaMemcpyDeviceToHost, b->stream), "read sizes");
  GRX_CHECK_CUDA(cudaStreamSynchronize(b->stream), "sync sizes");
  return GRX_OK;
}

}  // namespace grx

using namespace grx;

extern "C" {

grx_status grx_ewald_total(grx_box* b, double* out8) {
  GRX_REQUIRE(b && out8, "grx_ewald_total: null argument");
  grx_status st = sync_sizes(b);
  if (st) return st;
  refresh_dev(b);
  CompRanges r = ranges(b);
  const size_t n = std::max(r.n, 1);
  const size_t ntab = (size_t)(b->dev.kmax[0] + b->dev.kmax[1] + b->dev.kmax[2] + 3) * n;
  const int nblk_atoms = (r.n + GRX_THREADS - 1) / GRX_THREADS;
  const int nblk_big = 4 * sm_count(b);
  const size_t part_doubles = 4 * (size_t)std::max(nblk_atoms, 1) + 2 * (size_t)nblk_big * GRX_MAX_COMPONENTS;
  st = ensure_scratch(b, ntab * sizeof(double2) + part_doubles * sizeof(double));
  if (st) return st;
  double2* ex = (double2*)b->scratch;
  double2* ey = ex + (size_t)(b->dev.kmax[0] + 1) * n;
  double2* ez = ey + (size_t)(b->dev.kmax[1] + 1) * n;
  double* part = (double*)(ex + ntab);
  if (r.n > 0) {
    eik_tables_kernel<<<nblk_atoms, GRX_THREADS, 0, b->stream>>>(b->dev, r, ex, ey, ez);
    count_launch();
  }
  if (!b->parent)  // a replica's framework structure factor is its parent's, shared by every replica
    GRX_CHECK_CUDA(cudaMemsetAsync(b->s_fw, 0, b->nvec * sizeof(double2), b->stream), "clear S_fw");
  GRX_CHECK_CUDA(cudaMemsetAsync(b->s_ads, 0, b->nvec * sizeof(double2), b->stream), "clear S_ads");
  GRX_CHECK_CUDA(cudaMemsetAsync(b->s_tmp, 0, b->nvec * sizeof(double2), b->stream), "clear S_tmp");
  if (b->nact > 0 && r.n > 0) {
    sk_kernel<<<b->nact, GRX_THREADS, 0, b->stream>>>(b->dev, r, ex, ey, ez);
    count_launch();
  }
  std::vector<double> parts(part_doubles, 0.0);
  std::vector<int> big;
  if (r.n > 0) {
    self_excl_kernel<<<nblk_atoms, GRX_THREADS, 0, b->stream>>>(b->dev, r, part);
    count_launch();
    double* pbig = part + 4 * (size_t)std::max(nblk_atoms, 1);
    for (int c = 0; c < r.ncomp; ++c) {
      if (r.molsize[c] <= kBigMolecule || r.base[c + 1] - r.base[c] < 2) continue;
      big_excl_kernel<<<nblk_big, GRX_THREADS, 0, b->stream>>>(b->dev, r, c, pbig + 2 * (size_t)nblk_big * big.size());
      count_launch();
      big.push_back(c);
    }
    GRX_CHECK_CUDA(cudaMemcpyAsync(parts.data(), part, part_doubles * sizeof(double), cudaMemcpyDeviceToHost,
                                   b->stream), "read self/exclusion");
  }
  std::vector<double2> sfw(b->nvec), sads(b->nvec);
  GRX_CHECK_CUDA(cudaMemcpyAsync(sfw.data(), b->s_fw, b->nvec * sizeof(double2), cudaMemcpyDeviceToHost, b->stream), "read S_fw");
  GRX_CHECK_CUDA(cudaMemcpyAsync(sads.data(), b->s_ads, b->nvec * sizeof(double2), cudaMemcpyDeviceToHost, b->stream), "read S_ads");
  GRX_CHECK_CUDA(cudaStreamSynchronize(b->stream), "ewald total");
  // energies in slot order, FP64 (Ewald_Total, ewald_preparation.h:150-161)
  double gg = 0, hh = 0, hg = 0;
  for (int j = 0; j < b->nact; ++j) {
    const int s = b->h_kact[j].w;
    const double t = b->h_ktemp[j];
    const double2 a = sads[s], f = sfw[s];
    gg += t * (a.x * a.x + a.y * a.y);
    hh += t * (f.x * f.x + f.y * f.y);
    hg += t * (f.x * a.x + f.y * a.y) * 2.0;
  }
  double sa = 0, sh = 0, ea = 0, eh = 0;
  for (int k = 0; k < nblk_atoms; ++k) {
    sa += parts[4 * k]; sh += parts[4 * k + 1]; ea += parts[4 * k + 2]; eh += parts[4 * k + 3];
  }
  const double* pb = parts.data() + 4 * (size_t)std::max(nblk_atoms, 1);
  for (size_t g = 0; g < big.size(); ++g)
    for (int k = 0; k < nblk_big; ++k) {
      ea += pb[2 * (nblk_big * g + k)];
      eh += pb[2 * (nblk_big * g + k) + 1];
    }
  out8[0] = gg; out8[1] = hh; out8[2] = hg;
  out8[3] = sa; out8[4] = sh; out8[5] = -ea; out8[6] = -eh;
  out8[7] = (double)b->nact;
  b->sk_valid = true;
  b->ewdf_valid = false;
  return GRX_OK;
}

grx_status grx_total_energy(grx_box* b, grx_energy* out) { return grx_total_energy_overlap(b, out, nullptr); }

grx_status grx_total_energy_overlap(grx_box* b, grx_energy* out, uint8_t* overlap) {
  GRX_REQUIRE(b && out, "grx_total_energy: null argument");
  double ew[8];
  grx_status st = grx_ewald_total(b, ew);
  if (st) return st;
  CompRanges r = ranges(b);
  const int nblk = std::max((r.n + GRX_THREADS - 1) / GRX_THREADS, 1);
  st = ensure_scratch(b, 7 * (size_t)nblk * sizeof(double));
  if (st) return st;
  double* part = b->scratch;
  std::vector<double> parts(7 * (size_t)nblk, 0.0);
  if (r.n > 0) {
    vdw_real_total_kernel<<<nblk, GRX_THREADS, 0, b->stream>>>(b->dev, r, part);
    count_launch();
    GRX_CHECK_CUDA(cudaMemcpyAsync(parts.data(), part, parts.size() * sizeof(double),
                                   cudaMemcpyDeviceToHost, b->stream), "read totals");
  }
  GRX_CHECK_CUDA(cudaStreamSynchronize(b->stream), "totals");
  double e[6] = {0, 0, 0, 0, 0, 0};
  for (int k = 0; k < nblk; ++k)
    for (int q = 0; q < 6; ++q) e[q] += parts[6 * k + q];
  if (overlap) {
    *overlap = 0;
    for (int k = 0; k < nblk; ++k)
      if (parts[6 * (size_t)nblk + k] != 0.0) *overlap = 1;
  }
  out->hh_vdw = e[0]; out->hh_real = e[1];
  out->hg_vdw = e[2]; out->hg_real = e[3];
  out->gg_vdw = e[4]; out->gg_real = e[5];
  // Ewald blocks as Ewald_Total combines them (ewald_preparation.h:170-249)
  out->hh_ewald = ew[1] - ew[4] + ew[6];
  out->hg_ewald = ew[2];
  out->gg_ewald = ew[0] + ew[1] - ew[3] + ew[5];
  return GRX_OK;
}

}  // extern "C"

namespace grx {

// Runs the Fourier delta of the staged old / new atoms (ewald_delta_kernel) against
// `same` (its S + dS staged into s_tmp) and `cross`; returns the two sums.
static grx_status ewald_delta_run(grx_box* b, const double* old_pos, const double* old_qs, size_t n_old,
                                  const double* new_pos, const double* new_qs, size_t n_new, const double2* same,
                                  const double2* cross, double& s_same, double& s_cross) {
  s_same = s_cross = 0.0;
  MoveAtoms mv{};
  mv.n_old = (int)n_old;
  mv.n_new = (int)n_new;
  std::vector<double> op(3 * n_old), oq(n_old), np_(3 * n_new), nq(n_new);
  if (n_old) {
    GRX_CHECK_CUDA(cudaMemcpy(op.data(), old_pos, 3 * n_old * sizeof(double), cudaMemcpyDefault), "read old pos");
    GRX_CHECK_CUDA(cudaMemcpy(oq.data(), old_qs, n_old * sizeof(double), cudaMemcpyDefault), "read old q");
  }
  if (n_new) {
    GRX_CHECK_CUDA(cudaMemcpy(np_.data(), new_pos, 3 * n_new * sizeof(double), cudaMemcpyDefault), "read new pos");
    GRX_CHECK_CUDA(cudaMemcpy(nq.data(), new_qs, n_new * sizeof(double), cudaMemcpyDefault), "read new q");
  }
  for (size_t a = 0; a < n_old; ++a) { mv.x[a] = op[3 * a]; mv.y[a] = op[3 * a + 1]; mv.z[a] = op[3 * a + 2]; mv.q[a] = oq[a]; }
  for (size_t a = 0; a < n_new; ++a) {
    mv.x[n_old + a] = np_[3 * a]; mv.y[n_old + a] = np_[3 * a + 1]; mv.z[n_old + a] = np_[3 * a + 2]; mv.q[n_old + a] = nq[a];
  }
  const int nblk = std::max(1, std::min((b->nact + GRX_THREADS - 1) / GRX_THREADS, sm_count(b)));
  grx_status st = ensure_scratch(b, sizeof(MoveAtoms) + 2 * (size_t)nblk * sizeof(double) + 256);
  if (st) return st;
  MoveAtoms* d_mv = (MoveAtoms*)b->scratch;
  double* part = (double*)((char*)b->scratch + (sizeof(MoveAtoms) + 255) / 256 * 256);
  GRX_CHECK_CUDA(cudaMemcpyAsync(d_mv, &mv, sizeof(MoveAtoms), cudaMemcpyHostToDevice, b->stream), "upload move");
  refresh_dev(b);
  const int na = (int)(n_old + n_new);
  const size_t smem = (size_t)(b->dev.kmax[0] + b->dev.kmax[1] + b->dev.kmax[2] + 3) * std::max(na, 1) * sizeof(double2);
  std::vector<double> parts(2 * nblk, 0.0);
  if (b->nact > 0 && na > 0) {
    ewald_delta_kernel<<<nblk, GRX_THREADS, smem, b->stream>>>(b->dev, d_mv, same, cross, b->s_tmp, part);
    count_launch();
    GRX_CHECK_CUDA(cudaGetLastError(), "ewald delta launch");
    GRX_CHECK_CUDA(cudaMemcpyAsync(parts.data(), part, 2 * nblk * sizeof(double), cudaMemcpyDeviceToHost, b->stream),
                   "read ewald partials");
  }
  GRX_CHECK_CUDA(cudaStreamSynchronize(b->stream), "ewald delta");
  for (int k = 0; k < nblk; ++k) { s_same += parts[2 * k]; s_cross += parts[2 * k + 1]; }
  return GRX_OK;
}

}  // namespace grx

extern "C" {

grx_status grx_ewald_delta(grx_box* b, int32_t comp, int32_t move_type, const double* old_pos,
                           const double* old_qs, size_t n_old, const double* new_pos,
                           const double* new_qs, size_t n_new, double scale_coul_new,
                           double* out2) {
  GRX_REQUIRE(b && out2, "grx_ewald_delta: null argument");
  GRX_REQUIRE(comp >= 0 && comp < b->ncomp, "grx_ewald_delta: component out of range");
  GRX_REQUIRE(n_old <= GRX_MAX_MOLSIZE && n_new <= GRX_MAX_MOLSIZE, "grx_ewald_delta: too many atoms");
  GRX_REQUIRE((n_old == 0 || (old_pos && old_qs)) && (n_new == 0 || (new_pos && new_qs)),
              "grx_ewald_delta: atom arrays missing");
  out2[0] = out2[1] = 0.0;
  if (b->dev.no_charges && !b->has_charge[comp]) return GRX_OK;
  const bool host_comp = comp < b->nhost;
  double s_same = 0, s_cross = 0;
  grx_status st = ewald_delta_run(b, old_pos, old_qs, n_old, new_pos, new_qs, n_new, host_comp ? b->s_fw : b->s_ads,
                                  host_comp ? b->s_ads : b->s_fw, s_same, s_cross);
  if (st) return st;
  // rigid exclusion correction of GPU_EwaldDifference_General (:548-574)
  if (b->rigid[comp]) {
    const double ex = b->excl_intra[comp] + b->excl_self[comp];
    if (move_type == GRX_MOVE_INSERTION || move_type == GRX_MOVE_SINGLE_INSERTION)
      s_same -= ex * (scale_coul_new * scale_coul_new - 0.0);
    else if (move_type == GRX_MOVE_DELETION || move_type == GRX_MOVE_SINGLE_DELETION)
      s_same -= ex * (0.0 - 1.0);
  }
  out2[0] = s_same;
  out2[1] = 2.0 * s_cross;
  return GRX_OK;
}

grx_status grx_ewald_delta_lambda(grx_box* b, int32_t comp, const double* pos, const double* charge, size_t n,
                                  double scale_coul_old, double scale_coul_new, int32_t use_staged, double* out2) {
  GRX_REQUIRE(b && out2, "grx_ewald_delta_lambda: null argument");
  GRX_REQUIRE(comp >= b->nhost && comp < b->ncomp, "grx_ewald_delta_lambda: component must be an adsorbate");
  GRX_REQUIRE(n >= 1 && n <= GRX_MAX_MOLSIZE && pos && charge, "grx_ewald_delta_lambda: bad atom arrays");
  out2[0] = out2[1] = 0.0;
  if (b->dev.no_charges && !b->has_charge[comp]) return GRX_OK;
  std::vector<double> hq(n), qo(n), qn(n);
  GRX_CHECK_CUDA(cudaMemcpy(hq.data(), charge, n * sizeof(double), cudaMemcpyDefault), "read charges");
  for (size_t a = 0; a < n; ++a) {  // Fourier_Ewald_Diff_LambdaChange: the same atoms, old and new scaleCoul
    qo[a] = hq[a] * scale_coul_old;
    qn[a] = hq[a] * scale_coul_new;
  }
  double s_same = 0, s_cross = 0;
  grx_status st = ewald_delta_run(b, pos, qo.data(), n, pos, qn.data(), n, use_staged ? b->s_tmp : b->s_ads, b->s_fw,
                                  s_same, s_cross);
  if (st) return st;
  // GPU_EwaldDifference_LambdaChange (:782-785): exclusion times the change of scaleCoul^2
  s_same -= (b->excl_intra[comp] + b->excl_self[comp]) *
            (scale_coul_new * scale_coul_new - scale_coul_old * scale_coul_old);
  out2[0] = s_same;
  out2[1] = 2.0 * s_cross;
  return GRX_OK;
}

grx_status grx_ewald_delta_identity_swap(grx_box* b, int32_t old_comp, int32_t new_comp, const double* old_pos,
                                         const double* old_qs, size_t n_old, const double* new_pos,
                                         const double* new_qs, size_t n_new, double* out2) {
  GRX_REQUIRE(b && out2, "grx_ewald_delta_identity_swap: null argument");
  GRX_REQUIRE(old_comp >= b->nhost && old_comp < b->ncomp && new_comp >= b->nhost && new_comp < b->ncomp,
              "grx_ewald_delta_identity_swap: both components must be adsorbates");
  GRX_REQUIRE(n_old <= GRX_MAX_MOLSIZE && n_new <= GRX_MAX_MOLSIZE, "grx_ewald_delta_identity_swap: too many atoms");
  GRX_REQUIRE((n_old == 0 || (old_pos && old_qs)) && (n_new == 0 || (new_pos && new_qs)),
              "grx_ewald_delta_identity_swap: atom arrays missing");
  out2[0] = out2[1] = 0.0;
  const bool q_old = b->has_charge[old_comp] != 0, q_new = b->has_charge[new_comp] != 0;
  if (b->dev.no_charges && !q_old && !q_new) return GRX_OK;
  // atoms of an uncharged side do not enter (Ewald_Energy_Functions.h:588-597)
  const size_t no = q_old ? n_old : 0, nn = q_new ? n_new : 0;
  if (no + nn == 0) return GRX_OK;
  double s_same = 0, s_cross = 0;
  grx_status st = ewald_delta_run(b, old_pos, old_qs, no, new_pos, new_qs, nn, b->s_ads, b->s_fw, s_same, s_cross);
  if (st) return st;
  if (b->rigid[new_comp] && q_new) s_same -= (b->excl_intra[new_comp] + b->excl_self[new_comp]) * 1.0;
  if (b->rigid[old_comp] && q_old) s_same -= (b->excl_intra[old_comp] + b->excl_self[old_comp]) * -1.0;
  out2[0] = s_same;
  out2[1] = 2.0 * s_cross;
  return GRX_OK;
}

grx_status grx_ewald_commit(grx_box* b, int32_t comp) {
  GRX_REQUIRE(b && comp >= 0 && comp < b->ncomp, "grx_ewald_commit: bad argument");
  if (b->nact == 0) return GRX_OK;
  refresh_dev(b);
  GRX_REQUIRE(comp >= b->nhost || !b->parent, "grx_ewald_commit: a replica cannot move its shared framework");
  double2* dst = comp < b->nhost ? b->s_fw : b->s_ads;
  commit_kernel<<<std::max(1, std::min((b->nact + 255) / 256, sm_count(b))), 256, 0, b->stream>>>(b->dev, dst, b->s_tmp);
  count_launch();
  b->ewdf_valid = false;
  GRX_CHECK_CUDA(cudaGetLastError(), "commit launch");
  GRX_CHECK_CUDA(cudaStreamSynchronize(b->stream), "commit");
  return GRX_OK;
}

}  // extern "C"
