// grx_oracle.cpp -- FP64 CPU oracle for the CBMC trial-energy path.
//
// TEST INFRASTRUCTURE ONLY (see grx_oracle.h). Every function restates the FP64
// arithmetic of the gRASPA routine named in its comment, in plain C++ with the
// same operation order where that order fixes the rounding. OpenMP parallelises
// the independent Widom insertions; nothing here touches a GPU.
#include "grx_oracle.h"

#include <cmath>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kPi = 3.14159265358979323846;

inline void mat_vec(const double* a, const double* b, double* c) {
  // matrix_multiply_by_vector, maths.cuh:133-138 (column-major 3x3 times vector)
  c[0] = a[0] * b[0] + a[3] * b[1] + a[6] * b[2];
  c[1] = a[1] * b[0] + a[4] * b[1] + a[7] * b[2];
  c[2] = a[2] * b[0] + a[5] * b[1] + a[8] * b[2];
}

struct cplx {
  double re, im;
};
inline cplx cmul(cplx a, cplx b) {  // multiply(), Ewald_Energy_Functions.h:34-40
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}

// Per-atom eik tables, recurrence of Initialize_Vectors_thread
// (Ewald_Energy_Functions.h:97-104) seeded as Initialize_WaveVector_General :162-185.
struct Eik {
  int kx, ky, kz;
  size_t n;
  std::vector<cplx> x, y, z;
  void build(const ora_box* box, size_t natoms, const double* pos) {
    kx = box->kmax[0]; ky = box->kmax[1]; kz = box->kmax[2];
    n = natoms;
    x.assign(n * (kx + 1), {0, 0});
    y.assign(n * (ky + 1), {0, 0});
    z.assign(n * (kz + 1), {0, 0});
    for (size_t i = 0; i < n; ++i) {
      double s[3];
      mat_vec(box->inverse_cell, pos + 3 * i, s);
      s[0] *= 2 * kPi; s[1] *= 2 * kPi; s[2] *= 2 * kPi;
      x[i] = {1.0, 0.0}; y[i] = {1.0, 0.0}; z[i] = {1.0, 0.0};
      if (kx >= 1) x[i + n] = {std::cos(s[0]), std::sin(s[0])};
      if (ky >= 1) y[i + n] = {std::cos(s[1]), std::sin(s[1])};
      if (kz >= 1) z[i + n] = {std::cos(s[2]), std::sin(s[2])};
      for (int k = 2; k <= kx; ++k) x[i + k * n] = cmul(x[i + (k - 1) * n], x[i + n]);
      for (int k = 2; k <= ky; ++k) y[i + k * n] = cmul(y[i + (k - 1) * n], y[i + n]);
      for (int k = 2; k <= kz; ++k) z[i + k * n] = cmul(z[i + (k - 1) * n], z[i + n]);
    }
  }
  // e^{i k.r} of atom i for signed (kx, ky, kz), as in Fourier_Ewald_Diff :336-347
  cplx term(size_t i, int a, int b, int c) const {
    cplx ey = y[i + n * (size_t)std::abs(b)];
    if (b < 0) ey.im = -ey.im;
    cplx exy = cmul(x[i + n * (size_t)a], ey);
    cplx ez = z[i + n * (size_t)std::abs(c)];
    if (c < 0) ez.im = -ez.im;
    return cmul(exy, ez);
  }
};

struct KVec {
  int kx, ky, kz;
  bool active;
  double temp;  // factor * exp(-k^2/4a^2) / k^2
};

// k-vector slot unranking and cutoff test: Fourier_Ewald_Diff
// (Ewald_Energy_Functions.h:294-333) and Ewald_Total (ewald_preparation.h:80-150).
std::vector<KVec> kvectors(const ora_box* box) {
  const int kxm = box->kmax[0], kym = box->kmax[1], kzm = box->kmax[2];
  const size_t nvec = (size_t)(kxm + 1) * (2 * kym + 1) * (2 * kzm + 1);
  std::vector<KVec> out(nvec);
  const double* ic = box->inverse_cell;
  const double ax[3] = {ic[0], ic[3], ic[6]};
  const double ay[3] = {ic[1], ic[4], ic[7]};
  const double az[3] = {ic[2], ic[5], ic[8]};
  const double alpha_sq = box->alpha * box->alpha;
  const double prefactor = box->prefactor * (2.0 * kPi / box->volume);
  for (size_t kxyz = 0; kxyz < nvec; ++kxyz) {
    int kz = (int)(kxyz % (2 * kzm + 1)) - kzm;
    int kxy = (int)(kxyz / (2 * kzm + 1));
    int kx = kxy / (2 * kym + 1);
    int ky = kxy % (2 * kym + 1) - kym;
    double ksqr = (double)(kx * kx + ky * ky + kz * kz);
    if (box->use_lammps_ewald) {
      const double* C = box->cell;
      const double lx = C[0], ly = C[4], lz = C[8], xy = C[3], xz = C[6], yz = C[7];
      const double ux = 2 * kPi / lx;
      const double uy = 2 * kPi * (-xy) / lx / ly;
      const double uz = 2 * kPi * (xy * yz - ly * xz) / lx / ly / lz;
      const double vy = 2 * kPi / ly;
      const double vz = 2 * kPi * (-yz) / ly / lz;
      const double wz = 2 * kPi / lz;
      const double kvx = kx * ux;
      const double kvy = kx * uy + ky * vy;
      const double kvz = kx * uz + ky * vz + kz * wz;
      ksqr = kvx * kvx + kvy * kvy + kvz * kvz;
    }
    KVec& k = out[kxyz];
    k.kx = kx; k.ky = ky; k.kz = kz;
    k.active = (ksqr > 1e-10) && (ksqr < box->reciprocal_cutoff);
    k.temp = 0.0;
    if (k.active) {
      double kv[3];
      for (int d = 0; d < 3; ++d)
        kv[d] = ax[d] * 2.0 * kPi * (double)kx + ay[d] * 2.0 * kPi * (double)ky +
                az[d] * 2.0 * kPi * (double)kz;
      // The reference sums the three scaled vectors component-wise: (ax*2pi*kx) +
      // (ay*2pi*ky) + (az*2pi*kz); the expression above has the same evaluation order.
      const double rksq = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
      const double factor = (kx == 0) ? (1.0 * prefactor) : (2.0 * prefactor);
      k.temp = factor * std::exp((-0.25 / alpha_sq) * rksq) / rksq;
    }
  }
  return out;
}

inline uint32_t mulhilo(uint32_t a, uint32_t b, uint32_t* hi) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  return (uint32_t)p;
}

struct TrialOut {
  double e[4];
  uint8_t flag;
};

}  // namespace

extern "C" {

int32_t ora_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// Cell inverse / volume / cubic flag: inverse_matrix and matrix_determinant
// (maths.cuh:28-59), Cubic test read_data.cpp:2024-2025; LAMMPS reciprocal cutoff
// read_data.cpp:664-687 (off-diagonal cell terms deliberately zero there).
void ora_box_setup(ora_box* box) {
  const double* x = box->cell;
  const double m11 = x[0], m21 = x[3], m31 = x[6];
  const double m12 = x[1], m22 = x[4], m32 = x[7];
  const double m13 = x[2], m23 = x[5], m33 = x[8];
  const double det = +m11 * (m22 * m33 - m23 * m32) - m12 * (m21 * m33 - m23 * m31) +
                     m13 * (m21 * m32 - m22 * m31);
  double* r = box->inverse_cell;
  r[0] = +(m22 * m33 - m32 * m23) / det;
  r[3] = -(m21 * m33 - m31 * m23) / det;
  r[6] = +(m21 * m32 - m31 * m22) / det;
  r[1] = -(m12 * m33 - m32 * m13) / det;
  r[4] = +(m11 * m33 - m31 * m13) / det;
  r[7] = -(m11 * m32 - m31 * m12) / det;
  r[2] = +(m12 * m23 - m22 * m13) / det;
  r[5] = -(m11 * m23 - m21 * m13) / det;
  r[8] = +(m11 * m22 - m21 * m12) / det;
  box->volume = det;
  box->cubic = (std::fabs(x[3]) + std::fabs(x[6]) + std::fabs(x[7])) > 1e-10 ? 0 : 1;
  if (box->use_lammps_ewald) {
    const double lx = x[0], ly = x[4], lz = x[8];
    const double xy = 0.0, xz = 0.0, yz = 0.0;
    const double ux = 2 * kPi / lx;
    const double uy = 2 * kPi * (-xy) / lx / ly;
    const double uz = 2 * kPi * (xy * yz - ly * xz) / lx / ly / lz;
    const double vy = 2 * kPi / ly;
    const double vz = 2 * kPi * (-yz) / ly / lz;
    const double wz = 2 * kPi / lz;
    const double kvx = box->kmax[0] * ux;
    const double kvy = box->kmax[0] * uy + box->kmax[1] * vy;
    const double kvz = box->kmax[0] * uz + box->kmax[1] * vz + box->kmax[2] * wz;
    box->reciprocal_cutoff = std::max(kvx * kvx, std::max(kvy * kvy, kvz * kvz)) * 1.00001;
  }
}

// RASPA-2 style automatic Ewald parameters, read_data.cpp:690-703.
void ora_box_setup_raspa_ewald(ora_box* box, double cutoff_coul, double precision) {
  const double tol = std::sqrt(std::fabs(std::log(precision * cutoff_coul)));
  const double alpha = std::sqrt(std::fabs(std::log(precision * cutoff_coul * tol))) / cutoff_coul;
  const double tol1 = std::sqrt(-std::log(precision * cutoff_coul * std::pow(2.0 * tol * alpha, 2)));
  box->alpha = alpha;
  box->kmax[0] = (int)std::round(0.25 + box->cell[0] * alpha * tol1 / kPi);
  box->kmax[1] = (int)std::round(0.25 + box->cell[4] * alpha * tol1 / kPi);
  box->kmax[2] = (int)std::round(0.25 + box->cell[8] * alpha * tol1 / kPi);
  const int km = std::max(box->kmax[0], std::max(box->kmax[1], box->kmax[2]));
  box->reciprocal_cutoff = std::pow(1.05 * (double)km, 2);
  box->use_lammps_ewald = 0;
}

// Lorentz-Berthelot mixing and cutoff shift, read_data.cpp:737-747 (shift),
// :762-770 (mixing), :1190-1243 (table fill, epsilon divided by 1.20272430057).
void ora_mix_lorentz_berthelot(int64_t ntypes, const double* eps_K, const double* sigma,
                               const int32_t* shifted, double cutoff_vdw_sq,
                               double* eps_out, double* sig_out, double* shift_out) {
  for (int64_t i = 0; i < ntypes; ++i)
    for (int64_t j = 0; j < ntypes; ++j) {
      const double ep = std::sqrt(eps_K[i] * eps_K[j]) / 1.20272430057;
      const double sg = 0.5 * (sigma[i] + sigma[j]);
      eps_out[i * ntypes + j] = ep;
      sig_out[i * ntypes + j] = sg;
      double shift = 0.0;
      if (shifted[i] && shifted[j]) {
        const double arg2 = sg * sg;
        const double temp = cutoff_vdw_sq / arg2;
        const double rri3 = 1.0 / ((temp * temp * temp) + 0.5 * (1.0 - 1.0) * (1.0 - 1.0));
        shift = 1.0 * (4.0 * ep * (rri3 * (rri3 - 1.0)));
      }
      shift_out[i * ntypes + j] = shift;
    }
}

// Minimum image, PBC() maths.cuh:427-450 (round half away from zero by int cast).
void ora_pbc(const ora_box* box, double* d) {
  const double* C = box->cell;
  const double* I = box->inverse_cell;
  if (box->cubic) {
    d[0] -= (double)(int)(d[0] * I[0] + ((d[0] >= 0.0) ? 0.5 : -0.5)) * C[0];
    d[1] -= (double)(int)(d[1] * I[4] + ((d[1] >= 0.0) ? 0.5 : -0.5)) * C[4];
    d[2] -= (double)(int)(d[2] * I[8] + ((d[2] >= 0.0) ? 0.5 : -0.5)) * C[8];
  } else {
    double s[3];
    s[0] = I[0] * d[0] + I[3] * d[1] + I[6] * d[2];
    s[1] = I[1] * d[0] + I[4] * d[1] + I[7] * d[2];
    s[2] = I[2] * d[0] + I[5] * d[1] + I[8] * d[2];
    for (int k = 0; k < 3; ++k) s[k] -= (double)(int)(s[k] + ((s[k] >= 0.0) ? 0.5 : -0.5));
    d[0] = C[0] * s[0] + C[3] * s[1] + C[6] * s[2];
    d[1] = C[1] * s[0] + C[4] * s[1] + C[7] * s[2];
    d[2] = C[2] * s[0] + C[5] * s[1] + C[8] * s[2];
  }
}

// VDW(), maths.cuh:452-494: soft-core LJ 12-6 (default) or the 12-6-4 polynomial.
void ora_vdw(const double* f, double rr, double scaling, int use_1264, double* result) {
  if (use_1264) {
    const double ri2 = 1.0 / rr;
    const double ri4 = ri2 * ri2;
    const double ri6 = ri4 * ri2;
    const double ri10 = ri4 * ri6;
    const double ri12 = ri6 * ri6;
    const double term = f[0] * ri12 - f[1] * ri6 + f[4] * ri10 + f[2] * ri4 - f[3];
    result[0] = scaling * term;
    result[1] = 0.0;
  } else {
    const double arg1 = 4.0 * f[0];
    const double arg2 = f[1] * f[1];
    const double arg3 = f[3];
    const double temp = rr / arg2;
    const double temp3 = temp * temp * temp;
    const double rri3 = 1.0 / (temp3 + 0.5 * (1.0 - scaling) * (1.0 - scaling));
    const double rri6 = rri3 * rri3;
    const double term = arg1 * (rri3 * (rri3 - 1.0)) - arg3;
    const double dl = scaling * arg1 * (rri6 * (2.0 * rri3 - 1.0));
    result[0] = scaling * term;
    result[1] = scaling < 1.0 ? term + (1.0 - scaling) * dl : 0.0;
  }
}

// CoulombReal(), maths.cuh:496-500.
double ora_coulomb_real(double qa, double qb, double r, double scaling, double prefactor,
                        double alpha) {
  const double term = qa * qb * std::erfc(alpha * r);
  return prefactor * scaling * term / r;
}

// Per-trial host-guest / guest-guest sums with exclusion rules and overlap flags:
// Calculate_Multiple_Trial_Energy_VDWReal, VDW_Coulomb.cu:1183-1352, summed per trial
// as Host_sum_Widom_HGGG_SEPARATE (mc_widom.h:42-87) does before the flag filter.
void ora_trial_energies(const ora_box* box, const ora_ff* ff, const ora_atoms* at,
                        const ora_trials* tr, int64_t component, int64_t excl_comp,
                        int64_t excl_molid, double* out4, uint8_t* flag) {
  const int64_t nt = tr->ntrials, ch = tr->chainsize;
  for (int64_t t = 0; t < nt; ++t) {
    double hg_v = 0, hg_r = 0, gg_v = 0, gg_r = 0;
    uint8_t fl = 0;
    for (int64_t comp = 0; comp < at->ncomp; ++comp) {
      const bool host = comp < at->nhost;
      for (int64_t i = at->comp_start[comp]; i < at->comp_start[comp + 1]; ++i) {
        const int64_t mol = at->molid[i];
        if (comp == excl_comp && mol == excl_molid) continue;
        if (mol == tr->molid && comp == component) continue;
        for (int64_t jj = 0; jj < ch; ++jj) {
          const int64_t j = t * ch + jj;
          double d[3] = {at->pos[3 * i] - tr->pos[3 * j], at->pos[3 * i + 1] - tr->pos[3 * j + 1],
                         at->pos[3 * i + 2] - tr->pos[3 * j + 2]};
          ora_pbc(box, d);
          const double rr = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
          double ev = 0, er = 0;
          if (rr < ff->cutoff_vdw_sq) {
            const int64_t row = at->type[i] * ff->ntypes + tr->type[j];
            const double farg[5] = {ff->epsilon[row], ff->sigma[row], ff->z ? ff->z[row] : 0.0,
                                    ff->shift[row], ff->c10 ? ff->c10[row] : 0.0};
            double res[2];
            ora_vdw(farg, rr, at->scale[i] * tr->scale[j], ff->use_1264, res);
            if (res[0] > ff->overlap_criteria) fl = 1;
            if (rr < 0.01) fl = 1;
            ev = res[0];
          }
          if (!ff->no_charges && rr < ff->cutoff_coul_sq) {
            const double r = std::sqrt(rr);
            er = ora_coulomb_real(at->charge[i], tr->charge[j], r,
                                  at->scale_coul[i] * tr->scale_coul[j], box->prefactor,
                                  box->alpha);
          }
          if (host) { hg_v += ev; hg_r += er; } else { gg_v += ev; gg_r += er; }
        }
      }
    }
    out4[4 * t + 0] = hg_v; out4[4 * t + 1] = hg_r;
    out4[4 * t + 2] = gg_v; out4[4 * t + 3] = gg_r;
    flag[t] = fl;
  }
}

// New-minus-old energy of one moved molecule split HH/HG/GG:
// Calculate_Single_Body_Energy_VDWReal (VDW_Coulomb.cu:626-841) with its block
// partition (mc_single_particle.h:142-170): a moved host molecule sees HH + HG(guests),
// a moved guest sees HG(hosts) + GG.
void ora_single_body(const ora_box* box, const ora_ff* ff, const ora_atoms* at,
                     const ora_trials* oldm, const ora_trials* newm, int64_t component,
                     int32_t do_new, int32_t do_old, double* out6, uint8_t* flag) {
  double e[6] = {0, 0, 0, 0, 0, 0};
  uint8_t fl = 0;
  const bool moved_host = component < at->nhost;
  const int64_t ms = newm->chainsize;
  for (int64_t comp = 0; comp < at->ncomp; ++comp) {
    const bool host = comp < at->nhost;
    int slot;  // 0 HH, 1 HG, 2 GG
    if (moved_host) slot = host ? 0 : 1;
    else slot = host ? 1 : 2;
    for (int64_t i = at->comp_start[comp]; i < at->comp_start[comp + 1]; ++i) {
      const int64_t mol = at->molid[i];
      for (int64_t j = 0; j < ms; ++j) {
        for (int pass = 0; pass < 2; ++pass) {
          const ora_trials* m = pass == 0 ? newm : oldm;
          if (pass == 0 && !do_new) continue;
          if (pass == 1 && !do_old) continue;
          if (mol == m->molid && comp == component) continue;
          double d[3] = {at->pos[3 * i] - m->pos[3 * j], at->pos[3 * i + 1] - m->pos[3 * j + 1],
                         at->pos[3 * i + 2] - m->pos[3 * j + 2]};
          ora_pbc(box, d);
          const double rr = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
          const double sgn = pass == 0 ? 1.0 : -1.0;
          if (rr < ff->cutoff_vdw_sq) {
            const int64_t row = at->type[i] * ff->ntypes + m->type[j];
            const double farg[5] = {ff->epsilon[row], ff->sigma[row], ff->z ? ff->z[row] : 0.0,
                                    ff->shift[row], ff->c10 ? ff->c10[row] : 0.0};
            double res[2];
            ora_vdw(farg, rr, at->scale[i] * m->scale[j], ff->use_1264, res);
            if (pass == 0) {
              if (res[0] > ff->overlap_criteria) fl = 1;
              if (rr < 0.01) fl = 1;
            }
            e[2 * slot] += sgn * res[0];
          }
          if (!ff->no_charges && rr < ff->cutoff_coul_sq) {
            const double r = std::sqrt(rr);
            e[2 * slot + 1] += sgn * ora_coulomb_real(at->charge[i], m->charge[j], r,
                                                      at->scale_coul[i] * m->scale_coul[j],
                                                      box->prefactor, box->alpha);
          }
        }
      }
    }
  }
  for (int k = 0; k < 6; ++k) out6[k] = e[k];
  *flag = fl;
}

// Total VDW + real Coulomb, VDWReal_Total_CPU (VDW_Coulomb.cu:34-226): ordered pairs
// with a factor 0.5, same-molecule pairs of the same component skipped.
void ora_vdw_real_total(const ora_box* box, const ora_ff* ff, const ora_atoms* at, double* out6) {
  const int64_t N = at->comp_start[at->ncomp];
  std::vector<int64_t> compof(N);
  for (int64_t c = 0; c < at->ncomp; ++c)
    for (int64_t i = at->comp_start[c]; i < at->comp_start[c + 1]; ++i) compof[i] = c;
  double tv[3] = {0, 0, 0}, tr[3] = {0, 0, 0};
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : tv[:3], tr[:3])
  for (int64_t i = 0; i < N; ++i) {
    const int64_t ci = compof[i];
    for (int64_t j = 0; j < N; ++j) {
      const int64_t cj = compof[j];
      if (at->molid[i] == at->molid[j] && ci == cj) continue;
      int it;
      if (ci < at->nhost || cj < at->nhost) it = (!(ci < at->nhost) || !(cj < at->nhost)) ? 1 : 0;
      else it = 2;
      double d[3] = {at->pos[3 * i] - at->pos[3 * j], at->pos[3 * i + 1] - at->pos[3 * j + 1],
                     at->pos[3 * i + 2] - at->pos[3 * j + 2]};
      ora_pbc(box, d);
      const double rr = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
      if (rr < ff->cutoff_vdw_sq) {
        const int64_t row = at->type[i] * ff->ntypes + at->type[j];
        const double farg[5] = {ff->epsilon[row], ff->sigma[row], ff->z ? ff->z[row] : 0.0,
                                ff->shift[row], ff->c10 ? ff->c10[row] : 0.0};
        double res[2];
        ora_vdw(farg, rr, at->scale[i] * at->scale[j], ff->use_1264, res);
        tv[it] += 0.5 * res[0];
      }
      if (!ff->no_charges && rr < ff->cutoff_coul_sq) {
        const double r = std::sqrt(rr);
        tr[it] += 0.5 * ora_coulomb_real(at->charge[i], at->charge[j], r,
                                         at->scale_coul[i] * at->scale_coul[j], box->prefactor,
                                         box->alpha);
      }
    }
  }
  for (int k = 0; k < 3; ++k) { out6[2 * k] = tv[k]; out6[2 * k + 1] = tr[k]; }
}

int64_t ora_ewald_nvec(const ora_box* box) {
  return (int64_t)(box->kmax[0] + 1) * (2 * box->kmax[1] + 1) * (2 * box->kmax[2] + 1);
}

int64_t ora_ewald_active(const ora_box* box, uint8_t* active) {
  auto kv = kvectors(box);
  int64_t n = 0;
  for (size_t i = 0; i < kv.size(); ++i) {
    if (active) active[i] = kv[i].active ? 1 : 0;
    n += kv[i].active ? 1 : 0;
  }
  return n;
}

// Fourier-space totals, structure factors, self and intramolecular exclusion:
// Ewald_Total, ewald_preparation.h:5-259. s_fw / s_ads receive the framework-only and
// adsorbate-only structure factors per k slot (re, im interleaved), as stored in
// SystemComponents.FrameworkEik / AdsorbateEik (:183-184, :250-256).
// out8 = {fourier_gg, fourier_hh, fourier_hg, self_all, self_host,
//         exclusion_all, exclusion_host, n_active}, where the self / exclusion entries
// are the positive amounts the reference subtracts.
void ora_ewald_total(const ora_box* box, const ora_atoms* at, const int64_t* molsize,
                     double* s_fw, double* s_ads, double* out8) {
  const int64_t N = at->comp_start[at->ncomp];
  Eik eik;
  eik.build(box, (size_t)N, at->pos);
  auto kv = kvectors(box);
  std::vector<int64_t> compof(N);
  for (int64_t c = 0; c < at->ncomp; ++c)
    for (int64_t i = at->comp_start[c]; i < at->comp_start[c + 1]; ++i) compof[i] = c;
  const bool has_fw = at->nhost > 0 && at->comp_start[at->nhost] > 0;
  double gg = 0, hh = 0, hg = 0;
  int64_t nact = 0;
  for (size_t s = 0; s < kv.size(); ++s) {
    const KVec& k = kv[s];
    cplx ads = {0, 0}, fw = {0, 0};
    if (k.active) {
      ++nact;
      for (int64_t i = 0; i < N; ++i) {
        const cplx t = eik.term((size_t)i, k.kx, k.ky, k.kz);
        const double f = at->scale_coul[i] * at->charge[i];
        ads.re += f * t.re; ads.im += f * t.im;
        if (compof[i] < at->nhost && has_fw) { fw.re += f * t.re; fw.im += f * t.im; }
      }
      if (has_fw) { ads.re -= fw.re; ads.im -= fw.im; }
      gg += k.temp * (ads.re * ads.re + ads.im * ads.im);
      hh += k.temp * (fw.re * fw.re + fw.im * fw.im);
      hg += k.temp * (fw.re * ads.re + fw.im * ads.im) * 2.0;
    }
    if (s_fw) { s_fw[2 * s] = fw.re; s_fw[2 * s + 1] = fw.im; }
    if (s_ads) { s_ads[2 * s] = ads.re; s_ads[2 * s + 1] = ads.im; }
  }
  const double pself = box->prefactor * box->alpha / std::sqrt(kPi);
  double self_all = 0, self_host = 0;
  for (int64_t i = 0; i < N; ++i) {
    const double v = pself * at->scale_coul[i] * at->charge[i] * at->scale_coul[i] * at->charge[i];
    self_all += v;
    if (compof[i] < at->nhost && has_fw) self_host += v;
  }
  double ex_all = 0, ex_host = 0;
  for (int64_t c = 0; c < at->ncomp; ++c) {
    const int64_t ms = molsize[c];
    const int64_t n = at->comp_start[c + 1] - at->comp_start[c];
    if (ms <= 0 || n == 0) continue;
    const int64_t nmol = n / ms;
    double ex_c = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : ex_c) if (ms > 64)
    for (int64_t mol = 0; mol < nmol; ++mol) {
      const int64_t a0 = at->comp_start[c] + mol * ms;
      for (int64_t i = a0; i < a0 + ms - 1; ++i) {
        const double fa = at->scale_coul[i] * at->charge[i];
        for (int64_t j = i + 1; j < a0 + ms; ++j) {
          const double fb = at->scale_coul[j] * at->charge[j];
          double d[3] = {at->pos[3 * i] - at->pos[3 * j], at->pos[3 * i + 1] - at->pos[3 * j + 1],
                         at->pos[3 * i + 2] - at->pos[3 * j + 2]};
          ora_pbc(box, d);
          const double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
          ex_c += box->prefactor * fa * fb * std::erf(box->alpha * r) / r;
        }
      }
    }
    ex_all += ex_c;
    if (c < at->nhost && has_fw) ex_host += ex_c;
  }
  out8[0] = gg; out8[1] = hh; out8[2] = hg;
  out8[3] = self_all; out8[4] = self_host;
  out8[5] = -ex_all; out8[6] = -ex_host;
  out8[7] = (double)nact;
}

// Fourier delta of one move: Fourier_Ewald_Diff (Ewald_Energy_Functions.h:280-397),
// same-type half and cross-type half. old/new qs are charge * scaleCoul per atom.
// out2 = {sum over same-type slots, sum over cross-type slots}; the move driver
// (GPU_EwaldDifference_General :438-580) subtracts exclusions from the first and
// doubles the second. s_new receives S_same + dS on active slots (tempEik).
void ora_ewald_delta(const ora_box* box, const double* s_same, const double* s_cross,
                     int32_t use_temp, const double* s_temp, int64_t n_old,
                     const double* old_pos, const double* old_qs, int64_t n_new,
                     const double* new_pos, const double* new_qs, double* s_new, double* out2) {
  const int64_t N = n_old + n_new;
  std::vector<double> pos(3 * (size_t)std::max<int64_t>(N, 1));
  for (int64_t i = 0; i < n_old; ++i) for (int d = 0; d < 3; ++d) pos[3 * i + d] = old_pos[3 * i + d];
  for (int64_t i = 0; i < n_new; ++i) for (int d = 0; d < 3; ++d) pos[3 * (n_old + i) + d] = new_pos[3 * i + d];
  Eik eik;
  eik.build(box, (size_t)N, pos.data());
  auto kv = kvectors(box);
  double same = 0, cross = 0;
  for (size_t s = 0; s < kv.size(); ++s) {
    const KVec& k = kv[s];
    if (!k.active) {
      if (s_new) { s_new[2 * s] = s_same[2 * s]; s_new[2 * s + 1] = s_same[2 * s + 1]; }
      continue;
    }
    cplx co = {0, 0}, cn = {0, 0};
    for (int64_t i = 0; i < N; ++i) {
      const cplx t = eik.term((size_t)i, k.kx, k.ky, k.kz);
      if (i < n_old) { co.re += old_qs[i] * t.re; co.im += old_qs[i] * t.im; }
      else { cn.re += new_qs[i - n_old] * t.re; cn.im += new_qs[i - n_old] * t.im; }
    }
    const double* base = use_temp ? s_temp : s_same;
    const cplx ov = {base[2 * s], base[2 * s + 1]};
    const cplx nv = {ov.re + cn.re - co.re, ov.im + cn.im - co.im};
    same += k.temp * (nv.re * nv.re + nv.im * nv.im);
    same -= k.temp * (ov.re * ov.re + ov.im * ov.im);
    if (s_new) { s_new[2 * s] = nv.re; s_new[2 * s + 1] = nv.im; }
    const cplx xv = {s_cross[2 * s], s_cross[2 * s + 1]};
    cross += k.temp * (xv.re * (cn.re - co.re) + xv.im * (cn.im - co.im));
  }
  out2[0] = same;
  out2[1] = cross;
}

// Lambda change of one fractional molecule at fixed positions: Fourier_Ewald_Diff_LambdaChange
// (Ewald_Energy_Functions.h:636-762) driven by GPU_EwaldDifference_LambdaChange (:764-789).
// q are the atoms' charges; dS = sum q (scale_new - scale_old) e^{ik.r}; use_temp starts
// from s_temp (the CB/CFC deletion's second step). out2 = {same - excl * (new^2 - old^2),
// 2 * cross}, excl = ExclusionIntra + ExclusionAtom of the component.
void ora_ewald_delta_lambda(const ora_box* box, const double* s_same, const double* s_cross, int32_t use_temp,
                            const double* s_temp, int64_t n, const double* pos, const double* q, double scale_old,
                            double scale_new, double excl, double* s_new, double* out2) {
  std::vector<double> qo((size_t)n), qn((size_t)n);
  for (int64_t i = 0; i < n; ++i) { qo[i] = q[i] * scale_old; qn[i] = q[i] * scale_new; }
  double o2[2];
  ora_ewald_delta(box, s_same, s_cross, use_temp, s_temp, n, pos, qo.data(), n, pos, qn.data(), s_new, o2);
  out2[0] = o2[0] - excl * (scale_new * scale_new - scale_old * scale_old);
  out2[1] = 2.0 * o2[1];
}

// Identity swap: GPU_EwaldDifference_IdentitySwap (Ewald_Energy_Functions.h:582-634). The old
// molecule leaves, the new one arrives (n_old / n_new already zero for an uncharged side);
// excl_new / excl_old are ExclusionIntra + ExclusionAtom of rigid charged components, else 0.
void ora_ewald_delta_identity_swap(const ora_box* box, const double* s_same, const double* s_cross,
                                   int64_t n_old, const double* old_pos, const double* old_qs, int64_t n_new,
                                   const double* new_pos, const double* new_qs, double excl_new, double excl_old,
                                   double* s_new, double* out2) {
  double o2[2];
  ora_ewald_delta(box, s_same, s_cross, 0, nullptr, n_old, old_pos, old_qs, n_new, new_pos, new_qs, s_new, o2);
  out2[0] = o2[0] - excl_new * 1.0 - excl_old * -1.0;
  out2[1] = 2.0 * o2[1];
}

// Rigid-molecule exclusion constants: Calculate_Intra_Molecule_Exclusion and
// Calculate_Self_Exclusion, ewald_preparation.h:261-298.
void ora_rigid_exclusion(const ora_box* box, int64_t ms, const double* pos, const double* q,
                         const double* sc, double* intra, double* self) {
  double e = 0.0;
  for (int64_t i = 0; i + 1 < ms; ++i) {
    const double fa = sc[i] * q[i];
    for (int64_t j = i + 1; j < ms; ++j) {
      const double fb = sc[j] * q[j];
      double d[3] = {pos[3 * i] - pos[3 * j], pos[3 * i + 1] - pos[3 * j + 1], pos[3 * i + 2] - pos[3 * j + 2]};
      ora_pbc(box, d);
      const double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      e += box->prefactor * fa * fb * std::erf(box->alpha * r) / r;
    }
  }
  *intra = e;
  const double ps = box->prefactor * box->alpha / std::sqrt(kPi);
  double s = 0.0;
  for (int64_t i = 0; i < ms; ++i) s += ps * sc[i] * q[i] * sc[i] * q[i];
  *self = s;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
// 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies with Weyl key schedule.
void ora_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, hi1;
    const uint32_t lo0 = mulhilo(0xD2511F53u, c0, &hi0);
    const uint32_t lo1 = mulhilo(0xCD9E8D57u, c2, &hi1);
    const uint32_t n0 = hi1 ^ c1 ^ k0;
    const uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// Stream layout shared with the CUDA library: key = seed, counter =
// {slot, move lo, move hi, stream}. Slots: 0..1023 first-bead trial positions,
// 1024..2047 orientation quaternions, 2048 selection/acceptance uniforms.
void ora_draw(uint64_t seed, uint32_t stream, uint64_t move, uint32_t slot, uint32_t out[4]) {
  const uint32_t ctr[4] = {slot, (uint32_t)move, (uint32_t)(move >> 32), stream};
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  ora_philox4x32_10(ctr, key, out);
}

static inline double u01(uint32_t w) { return (double)w * 2.3283064365386963e-10; }  // w / 2^32

// SelectTrialPosition, mc_widom.h:14-39: shift by the largest log-weight, cumulative
// search against u * sum (guarded against running past the end).
// Smallest decision margin of the moves since the last reset (test diagnostics): for a
// trial selection the distance of u * sum from the nearest cumulative boundary relative to
// the sum, for an acceptance |ln u - ln Pacc|; both are the relative change of the weights
// (about beta |dE|) that would flip the decision.
static thread_local double g_margin = 1e300;
static void note_margin(double m) { g_margin = std::min(g_margin, std::fabs(m)); }
static void note_acceptance(double u, double pacc) {
  if (u > 0.0 && pacc > 0.0) note_margin(std::log(u) - std::log(pacc));
}

int64_t ora_select_trial(const double* logw, int64_t n, double u) {
  if (n <= 0) return -1;
  double mx = logw[0];
  for (int64_t i = 1; i < n; ++i) mx = std::max(mx, logw[i]);
  std::vector<double> w((size_t)n);
  double sum = 0.0;
  for (int64_t i = 0; i < n; ++i) { w[i] = std::exp(logw[i] - mx); sum += w[i]; }
  int64_t sel = 0;
  double cumw = w[0];
  const double ws = u * sum;
  while (cumw < ws && sel + 1 < n) cumw += w[++sel];
  if (n > 1) {
    double m = (cumw - ws) / sum;
    if (sel > 0) m = std::min(m, (ws - (cumw - w[sel])) / sum);
    note_margin(m);
  }
  return sel;
}

// Rotate_Quaternions, mc_utilities.h:423-457 (uniform random rotation from three
// uniforms, Shoemake / Kuffner 2004).
void ora_rotate_quaternion(double* v, double u, double vv, double w) {
  const double pi = 3.14159265358979323846;
  const double q0 = std::sqrt(1 - u) * std::sin(2 * pi * vv);
  const double q1 = std::sqrt(1 - u) * std::cos(2 * pi * vv);
  const double q2 = std::sqrt(u) * std::sin(2 * pi * w);
  const double q3 = std::sqrt(u) * std::cos(2 * pi * w);
  const double a01 = q0 * q1, a02 = q0 * q2, a03 = q0 * q3;
  const double a11 = q1 * q1, a12 = q1 * q2, a13 = q1 * q3;
  const double a22 = q2 * q2, a23 = q2 * q3, a33 = q3 * q3;
  double rot[9];
  rot[0] = 1.0 - 2.0 * (a22 + a33);
  rot[1] = 2.0 * (a12 - a03);
  rot[2] = 2.0 * (a13 + a02);
  rot[3] = 2.0 * (a12 + a03);
  rot[4] = 1.0 - 2.0 * (a11 + a33);
  rot[5] = 2.0 * (a23 - a01);
  rot[6] = 2.0 * (a13 - a02);
  rot[7] = 2.0 * (a23 + a01);
  rot[8] = 1.0 - 2.0 * (a11 + a22);
  const double r = v[0] * rot[0] + v[1] * rot[1] + v[2] * rot[2];
  const double s = v[0] * rot[3] + v[1] * rot[4] + v[2] * rot[5];
  const double c = v[0] * rot[6] + v[1] * rot[7] + v[2] * rot[8];
  v[0] = r; v[1] = s; v[2] = c;
}

// Shared finisher of the first-bead and chain steps: CBMC_FirstBead_Finish
// (mc_widom.h:305-383) and the chain tail of Widom_Move_Chain_PARTIAL (:568-611),
// insertion branch. Returns false when construction fails.
static bool cbmc_finish(const ora_ff* ff, double beta, int64_t nt, const double* e4,
                        const uint8_t* flag, double u, double navg, int64_t* real_sel,
                        double* w_avg, int64_t* n_ok) {
  std::vector<double> logw;
  std::vector<int64_t> idx;
  for (int64_t t = 0; t < nt; ++t)
    if (!flag[t]) idx.push_back(t);
  for (int64_t t : idx) {
    const double* e = e4 + 4 * t;
    double tot = e[0] + e[2];
    if (ff->vdw_real_bias) tot += e[1] + e[3];
    logw.push_back(-beta * tot);
  }
  *n_ok = (int64_t)idx.size();
  if (idx.empty()) return false;
  const int64_t sel = ora_select_trial(logw.data(), (int64_t)logw.size(), u);
  double sum = 0.0;
  for (double l : logw) sum += std::exp(l);
  if (sum < 1e-150) return false;
  *real_sel = idx[(size_t)sel];
  double avg = sum / navg;
  if (!ff->vdw_real_bias) {
    const double* e = e4 + 4 * idx[(size_t)sel];
    avg *= std::exp(-beta * (e[1] + e[3]));
  }
  *w_avg = avg;
  return true;
}

// CBMC Widom insertions into a static box: InsertionMove::WidomMove
// (move_struct.h:90-95) -> Insertion_Body (mc_swap_utilities.h:3-132) ->
// Widom_Move_FirstBead_PARTIAL / Widom_Move_Chain_PARTIAL (mc_widom.h:385-614) ->
// GPU_EwaldDifference_General(INSERTION) (Ewald_Energy_Functions.h:438-580).
// Insertions are independent, so they run in parallel over OpenMP threads.
void ora_widom_insertions(const ora_box* box, const ora_ff* ff, const ora_atoms* at,
                          const double* s_fw, const double* s_ads, const ora_widom* w,
                          uint64_t first_move, int64_t n, int32_t nthreads,
                          ora_widom_result* results) {
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#endif
  const int64_t ms = w->molsize, chain = ms - 1;
  const int64_t nt = w->ntrials, no = w->norient;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
  for (int64_t m = 0; m < n; ++m) {
    ora_widom_result res;
    std::memset(&res, 0, sizeof(res));
    res.sel_first = -1; res.sel_orient = -1;
    const uint64_t move = first_move + (uint64_t)m;
    uint32_t sel_words[4];
    ora_draw(w->seed, w->stream, move, 2048u, sel_words);

    // first bead: get_random_trial_position, CBMC_INSERTION (mc_widom.h:133-139)
    std::vector<double> tp(3 * nt), tsc(nt, w->scale), tq(nt, w->mol_charge[0]),
        tscc(nt, w->scale_coul);
    std::vector<int64_t> tty(nt, w->mol_type[0]);
    for (int64_t t = 0; t < nt; ++t) {
      uint32_t r[4];
      ora_draw(w->seed, w->stream, move, (uint32_t)t, r);
      tp[3 * t + 0] = box->cell[0] * u01(r[0]);
      tp[3 * t + 1] = box->cell[4] * u01(r[1]);
      tp[3 * t + 2] = box->cell[8] * u01(r[2]);
    }
    ora_trials tr1 = {nt, 1, tp.data(), tsc.data(), tq.data(), tscc.data(), tty.data(), w->new_molid};
    std::vector<double> e1(4 * nt);
    std::vector<uint8_t> f1(nt);
    ora_trial_energies(box, ff, at, &tr1, w->component, -1, -1, e1.data(), f1.data());
    int64_t sel1 = -1;
    double w1 = 0.0;
    bool ok = cbmc_finish(ff, w->beta, nt, e1.data(), f1.data(), u01(sel_words[0]), (double)nt,
                          &sel1, &w1, &res.n_ok_first);
    if (ok && w1 <= 1e-150) ok = false;
    double rosen = 0.0;
    std::vector<double> newpos(3 * ms), newqs(ms);
    if (ok) {
      res.sel_first = sel1;
      res.w_first = w1;
      for (int k = 0; k < 4; ++k) res.e_first[k] = e1[4 * sel1 + k];
      rosen = w1;
      const double* fb = &tp[3 * sel1];
      newpos[0] = fb[0]; newpos[1] = fb[1]; newpos[2] = fb[2];
      newqs[0] = w->mol_charge[0] * w->scale_coul;
      if (ms > 1) {
        // orientations: get_random_trial_orientation (mc_widom.h:215-303)
        std::vector<double> op(3 * no * chain), osc(no * chain, w->scale), oq(no * chain),
            oscc(no * chain, w->scale_coul);
        std::vector<int64_t> oty(no * chain);
        for (int64_t o = 0; o < no; ++o) {
          uint32_t r[4];
          ora_draw(w->seed, w->stream, move, 1024u + (uint32_t)o, r);
          for (int64_t a = 0; a < chain; ++a) {
            double v[3] = {w->mol_pos[3 * (1 + a)] - w->mol_pos[0],
                           w->mol_pos[3 * (1 + a) + 1] - w->mol_pos[1],
                           w->mol_pos[3 * (1 + a) + 2] - w->mol_pos[2]};
            ora_rotate_quaternion(v, u01(r[0]), u01(r[1]), u01(r[2]));
            const int64_t j = o * chain + a;
            op[3 * j] = fb[0] + v[0]; op[3 * j + 1] = fb[1] + v[1]; op[3 * j + 2] = fb[2] + v[2];
            oq[j] = w->mol_charge[1 + a];
            oty[j] = w->mol_type[1 + a];
          }
        }
        ora_trials tr2 = {no, chain, op.data(), osc.data(), oq.data(), oscc.data(), oty.data(), w->new_molid};
        std::vector<double> e2(4 * no);
        std::vector<uint8_t> f2(no);
        ora_trial_energies(box, ff, at, &tr2, w->component, -1, -1, e2.data(), f2.data());
        int64_t sel2 = -1;
        double w2 = 0.0;
        ok = cbmc_finish(ff, w->beta, no, e2.data(), f2.data(), u01(sel_words[1]), (double)no,
                         &sel2, &w2, &res.n_ok_orient);
        if (ok) {
          res.sel_orient = sel2;
          res.w_chain = w2;
          for (int k = 0; k < 4; ++k) res.e_chain[k] = e2[4 * sel2 + k];
          rosen *= w2;
          if (rosen <= 1e-150) ok = false;
          for (int64_t a = 0; a < chain; ++a) {
            for (int d = 0; d < 3; ++d) newpos[3 * (1 + a) + d] = op[3 * (sel2 * chain + a) + d];
            newqs[1 + a] = w->mol_charge[1 + a] * w->scale_coul;
          }
        }
      }
    }
    if (ok) {
      if (!ff->no_charges && w->has_charge) {
        double d2[2];
        ora_ewald_delta(box, s_ads, s_fw, 0, nullptr, 0, nullptr, nullptr, ms, newpos.data(),
                        newqs.data(), nullptr, d2);
        double same = d2[0];
        if (w->rigid) same -= (w->excl_intra + w->excl_self) * (w->scale_coul * w->scale_coul - 0.0);
        res.ewald[0] = same;
        res.ewald[1] = 2.0 * d2[1];
        rosen *= std::exp(-w->beta * (res.ewald[0] + res.ewald[1]));
      }
      rosen *= std::exp(-w->beta * w->tail_delta);
      res.rosenbluth = rosen;
      res.success = 1;
    } else {
      res.rosenbluth = 0.0;
      res.success = 0;
    }
    results[m] = res;
  }
}

}  // extern "C"

// ----------------------------------------------------------------------------
// GCMC (test oracle): translation, rotation, CBMC insertion and CBMC deletion of
// one adsorbate component, sequential FP64, the same Philox stream layout as the
// device driver: slot 4096 = {molecule pick, move choice, insertion-vs-deletion,
// acceptance}, slot 4097 = {three uniforms of the displacement / rotation angles},
// CBMC trials in slots 0..2047 and the selection uniforms in slot 2048.
namespace {

struct GState {
  std::vector<double> pos, scale, charge, scc;
  std::vector<int64_t> type, molid;
  std::vector<int64_t> comp_start;
  int64_t ncomp = 0, nhost = 0;
  ora_atoms view() {
    ora_atoms a;
    a.ncomp = ncomp;
    a.nhost = nhost;
    a.comp_start = comp_start.data();
    a.pos = pos.data();
    a.scale = scale.data();
    a.charge = charge.data();
    a.scale_coul = scc.data();
    a.type = type.data();
    a.molid = molid.data();
    return a;
  }
};

struct Grow {
  bool ok = false;
  double rosen = 0.0;  // product of the averaged step weights
  double stored = 0.0; // reinsertion: first-bead weight sum minus the selected trial
  double e1[4] = {0, 0, 0, 0}, e2[4] = {0, 0, 0, 0};
  std::vector<double> pos, qs;  // chosen (insertion) or existing (deletion) molecule
  int64_t configs = 0, beads = 0;  // trial configurations evaluated and their beads
};

// RotationAroundAxis, mc_utilities.h:459-481, for a coordinate axis.
void rotate_axis(double* v, double theta, int axis) {
  const double c = std::cos(theta), w = 1.0 - c, s = std::sin(theta);
  double ax[3] = {0, 0, 0};
  ax[axis] = 1.0;
  double rot[9];
  rot[0] = ax[0] * ax[0] * w + c;
  rot[1] = ax[0] * ax[1] * w + ax[2] * s;
  rot[2] = ax[0] * ax[2] * w - ax[1] * s;
  rot[3] = ax[0] * ax[1] * w - ax[2] * s;
  rot[4] = ax[1] * ax[1] * w + c;
  rot[5] = ax[1] * ax[2] * w + ax[0] * s;
  rot[6] = ax[0] * ax[2] * w + ax[1] * s;
  rot[7] = ax[1] * ax[2] * w - ax[0] * s;
  rot[8] = ax[2] * ax[2] * w + c;
  const double x = v[0] * rot[0] + v[1] * rot[1] + v[2] * rot[2];
  const double y = v[0] * rot[3] + v[1] * rot[4] + v[2] * rot[5];
  const double z = v[0] * rot[6] + v[1] * rot[7] + v[2] * rot[8];
  v[0] = x; v[1] = y; v[2] = z;
}

// CBMC growth of one molecule (insertion) or retrace of an existing one (deletion):
// Widom_Move_FirstBead_PARTIAL + Widom_Move_Chain_PARTIAL (mc_widom.h:385-614) with
// CBMC_FirstBead_Finish (:305-383), insertion and deletion branches.
// mode: CBMC_INSERTION, CBMC_DELETION, REINSERTION_INSERTION (all trials new,
// StoredR = W1 - w_selected returned in g.stored) or REINSERTION_RETRACE (one
// first-bead trial at the old position, W1 += stored; orientations from the
// retrace slots).
enum { G_INSERT = 0, G_DELETE = 1, G_REINS = 2, G_RETRACE = 3 };
Grow cbmc_grow(const ora_box* box, const ora_ff* ff, const ora_atoms* at, int64_t comp, int64_t ms,
               const double* tmpl_pos, const double* tmpl_q, const int64_t* tmpl_t, int64_t nt, int64_t no,
               double beta, uint64_t seed, uint32_t stream, uint64_t move, int64_t newmol, int mode,
               const double* oldpos, double stored = 0.0) {
  Grow g;
  const bool deletion = mode == G_DELETE || mode == G_RETRACE;
  const int64_t navg1 = nt;
  if (mode == G_RETRACE) nt = 1;
  const uint32_t oslot = mode == G_RETRACE ? 3072u : 1024u;
  const int64_t chain = ms - 1;
  uint32_t sel_words[4];
  ora_draw(seed, stream, move, 2048u, sel_words);
  std::vector<double> tp(3 * nt), ones(std::max<int64_t>(nt, 1), 1.0), tq(nt, tmpl_q[0]);
  std::vector<int64_t> tty(nt, tmpl_t[0]);
  for (int64_t t = 0; t < nt; ++t) {
    if (deletion && t == 0) {
      for (int d = 0; d < 3; ++d) tp[d] = oldpos[d];
      continue;
    }
    uint32_t r[4];
    ora_draw(seed, stream, move, (uint32_t)t, r);
    tp[3 * t] = box->cell[0] * u01(r[0]);
    tp[3 * t + 1] = box->cell[4] * u01(r[1]);
    tp[3 * t + 2] = box->cell[8] * u01(r[2]);
  }
  ora_trials tr1 = {nt, 1, tp.data(), ones.data(), tq.data(), ones.data(), tty.data(), newmol};
  std::vector<double> e1(4 * nt);
  std::vector<uint8_t> f1(nt);
  ora_trial_energies(box, ff, at, &tr1, comp, -1, -1, e1.data(), f1.data());
  g.configs += nt;
  g.beads += nt;
  // log-weights of the trials without overlap (Host_sum_Widom_HGGG_SEPARATE)
  auto logw_of = [&](const std::vector<double>& e, const std::vector<uint8_t>& f, int64_t n,
                     std::vector<double>& lw, std::vector<int64_t>& idx) {
    for (int64_t t = 0; t < n; ++t) {
      if (f[t]) continue;
      double tot = e[4 * t] + e[4 * t + 2];
      if (ff->vdw_real_bias) tot += e[4 * t + 1] + e[4 * t + 3];
      lw.push_back(-beta * tot);
      idx.push_back(t);
    }
  };
  std::vector<double> lw1;
  std::vector<int64_t> idx1;
  logw_of(e1, f1, nt, lw1, idx1);
  if (idx1.empty()) return g;
  int64_t s1 = 0;
  if (!deletion) s1 = ora_select_trial(lw1.data(), (int64_t)lw1.size(), u01(sel_words[0]));
  double w1 = 0.0;
  for (double l : lw1) w1 += std::exp(l);
  if (!deletion && w1 < 1e-150) return g;
  const int64_t real1 = idx1[(size_t)s1];
  if (mode == G_REINS) g.stored = w1 - std::exp(lw1[(size_t)s1]);
  if (mode == G_RETRACE) w1 += stored;
  double avg1 = w1 / (double)navg1;
  if (!ff->vdw_real_bias) avg1 *= std::exp(-beta * (e1[4 * real1 + 1] + e1[4 * real1 + 3]));
  if (avg1 <= 1e-150) return g;
  for (int k = 0; k < 4; ++k) g.e1[k] = e1[4 * real1 + k];
  g.pos.assign(3 * ms, 0.0);
  g.qs.assign(ms, 0.0);
  const double* fb = &tp[3 * real1];
  for (int d = 0; d < 3; ++d) g.pos[d] = fb[d];
  g.qs[0] = tmpl_q[0];
  double rosen = avg1;
  if (chain > 0) {
    std::vector<double> op(3 * no * chain), oones(no * chain, 1.0), oq(no * chain);
    std::vector<int64_t> oty(no * chain);
    for (int64_t o = 0; o < no; ++o) {
      uint32_t r[4];
      ora_draw(seed, stream, move, oslot + (uint32_t)o, r);
      for (int64_t a = 0; a < chain; ++a) {
        const int64_t j = o * chain + a;
        if (deletion && o == 0) {
          for (int d = 0; d < 3; ++d) op[3 * j + d] = oldpos[3 * (1 + a) + d];
        } else {
          double v[3] = {tmpl_pos[3 * (1 + a)] - tmpl_pos[0], tmpl_pos[3 * (1 + a) + 1] - tmpl_pos[1],
                         tmpl_pos[3 * (1 + a) + 2] - tmpl_pos[2]};
          ora_rotate_quaternion(v, u01(r[0]), u01(r[1]), u01(r[2]));
          for (int d = 0; d < 3; ++d) op[3 * j + d] = fb[d] + v[d];
        }
        oq[j] = tmpl_q[1 + a];
        oty[j] = tmpl_t[1 + a];
      }
    }
    ora_trials tr2 = {no, chain, op.data(), oones.data(), oq.data(), oones.data(), oty.data(), newmol};
    std::vector<double> e2(4 * no);
    std::vector<uint8_t> f2(no);
    ora_trial_energies(box, ff, at, &tr2, comp, -1, -1, e2.data(), f2.data());
    g.configs += no;
    g.beads += no * chain;
    std::vector<double> lw2;
    std::vector<int64_t> idx2;
    logw_of(e2, f2, no, lw2, idx2);
    if (idx2.empty()) return g;
    int64_t s2 = 0;
    if (!deletion) s2 = ora_select_trial(lw2.data(), (int64_t)lw2.size(), u01(sel_words[1]));
    double w2 = 0.0;
    for (double l : lw2) w2 += std::exp(l);
    if (!deletion && w2 < 1e-150) return g;
    const int64_t real2 = idx2[(size_t)s2];
    double avg2 = w2 / (double)no;
    if (!ff->vdw_real_bias) avg2 *= std::exp(-beta * (e2[4 * real2 + 1] + e2[4 * real2 + 3]));
    for (int k = 0; k < 4; ++k) g.e2[k] = e2[4 * real2 + k];
    rosen *= avg2;
    if (rosen <= 1e-150) return g;
    for (int64_t a = 0; a < chain; ++a) {
      for (int d = 0; d < 3; ++d) g.pos[3 * (1 + a) + d] = op[3 * (real2 * chain + a) + d];
      g.qs[1 + a] = tmpl_q[1 + a];
    }
  }
  g.ok = true;
  g.rosen = rosen;
  return g;
}

}  // namespace

extern "C" void ora_gcmc_run_mix(const ora_box* box, const ora_ff* ff, double* pos, double* charge,
                                 int64_t* type, int64_t* molid, int64_t ncomp, int64_t nhost, int64_t* comp_size,
                                 const int64_t* comp_off, const int64_t* molsize, double* const* mol_pos_k,
                                 const double* const* mol_charge_k, const int64_t* const* mol_type_k,
                                 const double* excl_intra_k, const double* excl_self_k, double* s_fw, double* s_ads,
                                 const ora_gcmc* gk, int64_t ng, uint64_t first_step, int64_t nsteps,
                                 ora_gcmc_stats* stk) {
  // compact working copy of every component
  GState S;
  S.ncomp = ncomp;
  S.nhost = nhost;
  S.comp_start.assign(ncomp + 1, 0);
  for (int64_t c = 0; c < ncomp; ++c) {
    for (int64_t i = 0; i < comp_size[c]; ++i) {
      const int64_t k = comp_off[c] + i;
      for (int d = 0; d < 3; ++d) S.pos.push_back(pos[3 * k + d]);
      S.charge.push_back(charge[k]);
      S.type.push_back(type[k]);
      S.molid.push_back(molid[k]);
    }
    S.comp_start[c + 1] = S.comp_start[c] + comp_size[c];
  }
  S.scale.assign(S.charge.size(), 1.0);
  S.scc.assign(S.charge.size(), 1.0);
  const int64_t nvec = ora_ewald_nvec(box);
  std::vector<double> s_new(2 * nvec);
  const bool charged = !ff->no_charges;
  // Orientation trials grow from the coordinates stored in the component's first
  // molecule slot (AllData.pos[1+a] - AllData.pos[0], mc_widom.h:262): they follow
  // every write to slot 0 and survive the deletion of its molecule.
  std::vector<std::vector<double>> slot0s(ng);
  for (int64_t k = 0; k < ng; ++k)
    slot0s[k].assign(mol_pos_k[k], mol_pos_k[k] + 3 * molsize[gk[k].component]);
  const uint64_t seed = gk[0].seed;
  const uint32_t stream = gk[0].stream;
  for (int64_t step = 0; step < nsteps; ++step) {
    g_margin = 1e300;
    const uint64_t move = first_step + (uint64_t)step;
    uint32_t w[4], w2[4];
    ora_draw(seed, stream, move, 4096u, w);
    ora_draw(seed, stream, move, 4097u, w2);
    // Select_Box_Component_Molecule (axpy.cu:74-100): one moved component, uniformly
    const int64_t sel = ng > 1 ? std::min<int64_t>(ng - 1, (int64_t)(u01(w2[3]) * (double)ng)) : 0;
    const ora_gcmc* g = &gk[sel];
    ora_gcmc_stats* st = &stk[sel];
    const int64_t comp = g->component;
    const int64_t ms = molsize[comp];
    std::vector<double>& slot0 = slot0s[sel];
    const double* mol_charge = mol_charge_k[sel];
    const int64_t* mol_type = mol_type_k[sel];
    const double excl_intra = excl_intra_k[sel], excl_self = excl_self_k[sel];
    const double bigP = g->mol_fraction * g->pressure * g->fugacity_coeff * box->volume;
    const int64_t a0 = S.comp_start[comp];
    const int64_t n_atoms = S.comp_start[comp + 1] - a0;
    const int64_t N = n_atoms / ms;
    const int64_t mol = (int64_t)(u01(w[0]) * (double)N);
    const double r = u01(w[1]);
    int kind = -1;
    if (r < g->p_translation) kind = 0;
    else if (r < g->p_rotation) kind = 1;
    else if (r < g->p_reinsertion) kind = 4;
    else if (r < g->p_swap) kind = (u01(w[2]) < 0.5) ? 2 : 3;
    const double uacc = u01(w[3]);
    if (kind == 0 || kind == 1) {
      if (N > 0) {
        st->attempts[kind]++;
        st->trial_configs += 2;
        st->trial_beads += 2 * ms;
        const int64_t m0 = a0 + mol * ms;
        std::vector<double> oldp(S.pos.begin() + 3 * m0, S.pos.begin() + 3 * (m0 + ms)), newp(3 * ms);
        if (kind == 0) {  // get_new_position TRANSLATION (mc_utilities.h:500-515)
          double dd[3];
          for (int d = 0; d < 3; ++d) dd[d] = g->max_translation[d] * 2.0 * (u01(w2[d]) - 0.5);
          for (int64_t a = 0; a < ms; ++a)
            for (int d = 0; d < 3; ++d) newp[3 * a + d] = oldp[3 * a + d] + dd[d];
        } else {  // ROTATION (mc_utilities.h:516-540)
          double ang[3];
          for (int d = 0; d < 3; ++d) ang[d] = g->max_rotation[d] * 2.0 * (u01(w2[d]) - 0.5);
          for (int64_t a = 0; a < ms; ++a) {
            double v[3] = {oldp[3 * a] - oldp[0], oldp[3 * a + 1] - oldp[1], oldp[3 * a + 2] - oldp[2]};
            rotate_axis(v, ang[0], 0);
            rotate_axis(v, ang[1], 1);
            rotate_axis(v, ang[2], 2);
            for (int d = 0; d < 3; ++d) newp[3 * a + d] = v[d] + oldp[d];
          }
        }
        std::vector<double> q(S.charge.begin() + m0, S.charge.begin() + m0 + ms), ones(ms, 1.0);
        std::vector<int64_t> ty(S.type.begin() + m0, S.type.begin() + m0 + ms);
        ora_atoms at = S.view();
        ora_trials to = {1, ms, oldp.data(), ones.data(), q.data(), ones.data(), ty.data(), mol};
        ora_trials tn = {1, ms, newp.data(), ones.data(), q.data(), ones.data(), ty.data(), mol};
        double e6[6];
        uint8_t fl = 0;
        ora_single_body(box, ff, &at, &to, &tn, comp, 1, 1, e6, &fl);
        if (!fl) {
          double ew = 0.0;
          if (charged) {
            double d2[2];
            ora_ewald_delta(box, s_ads, s_fw, 0, nullptr, ms, oldp.data(), q.data(), ms, newp.data(), q.data(),
                            s_new.data(), d2);
            ew = d2[0] + 2.0 * d2[1];
          }
          const double tot = e6[0] + e6[1] + e6[2] + e6[3] + e6[4] + e6[5] + ew;
          const double pacc = std::exp(-g->beta * tot);
          note_acceptance(uacc, pacc);
          if (uacc < pacc) {
            st->accepted[kind]++;
            for (int64_t k = 0; k < 3 * ms; ++k) S.pos[3 * m0 + k] = newp[k];
            if (mol == 0) std::copy(newp.begin(), newp.end(), slot0.begin());
            if (charged) std::copy(s_new.begin(), s_new.end(), s_ads);
            st->energy[0] += e6[0] + e6[2] + e6[4];
            st->energy[1] += e6[1] + e6[3] + e6[5];
            st->energy[2] += ew;
            st->energy[3] += tot;
          }
        }
      }
    } else if (kind == 4 && N > 0) {  // ReinsertionMove::Run (move_struct.h:377-406)
      st->attempts[4]++;
      const int64_t m0 = a0 + mol * ms;
      std::vector<double> oldp(S.pos.begin() + 3 * m0, S.pos.begin() + 3 * (m0 + ms));
      std::vector<double> q(S.charge.begin() + m0, S.charge.begin() + m0 + ms);
      ora_atoms at = S.view();
      Grow gi = cbmc_grow(box, ff, &at, comp, ms, slot0.data(), mol_charge, mol_type, g->ntrials, g->norient,
                          g->beta, g->seed, g->stream, move, mol, G_REINS, nullptr);
      st->trial_configs += gi.configs;
      st->trial_beads += gi.beads;
      if (gi.ok) {
        Grow gr = cbmc_grow(box, ff, &at, comp, ms, slot0.data(), mol_charge, mol_type, g->ntrials, g->norient,
                            g->beta, g->seed, g->stream, move, mol, G_RETRACE, oldp.data(), gi.stored);
        st->trial_configs += gr.configs;
        st->trial_beads += gr.beads;
        if (gr.ok) {
          double rosen = gi.rosen, ew = 0.0;
          if (charged) {  // Calculate_AdjustRosenbluth: old molecule out, new in, no exclusion change
            double d2[2];
            ora_ewald_delta(box, s_ads, s_fw, 0, nullptr, ms, oldp.data(), q.data(), ms, gi.pos.data(), q.data(),
                            s_new.data(), d2);
            ew = d2[0] + 2.0 * d2[1];
            rosen *= std::exp(-g->beta * ew);
          }
          const double pacc = rosen / gr.rosen;
          note_acceptance(uacc, pacc);
          if (uacc < pacc) {
            st->accepted[4]++;
            for (int64_t k = 0; k < 3 * ms; ++k) S.pos[3 * m0 + k] = gi.pos[k];
            if (mol == 0) std::copy(gi.pos.begin(), gi.pos.end(), slot0.begin());
            if (charged) std::copy(s_new.begin(), s_new.end(), s_ads);
            const double ev = gi.e1[0] + gi.e1[2] + gi.e2[0] + gi.e2[2] - (gr.e1[0] + gr.e1[2] + gr.e2[0] + gr.e2[2]);
            const double er = gi.e1[1] + gi.e1[3] + gi.e2[1] + gi.e2[3] - (gr.e1[1] + gr.e1[3] + gr.e2[1] + gr.e2[3]);
            st->energy[0] += ev;
            st->energy[1] += er;
            st->energy[2] += ew;
            st->energy[3] += ev + er + ew;
          }
        }
      }
    } else if (kind == 2) {  // CBMC insertion (InsertionMove::Run, move_struct.h:71-89)
      st->attempts[2]++;
      ora_atoms at = S.view();
      Grow gr = cbmc_grow(box, ff, &at, comp, ms, slot0.data(), mol_charge, mol_type, g->ntrials, g->norient,
                          g->beta, g->seed, g->stream, move, N, G_INSERT, nullptr);
      st->trial_configs += gr.configs;
      st->trial_beads += gr.beads;
      double rosen_rec = 0.0;  // RecordRosen: W of the insertion, 0 when the growth failed
      if (gr.ok) {
        double ew = 0.0, rosen = gr.rosen;
        if (charged) {
          double d2[2];
          ora_ewald_delta(box, s_ads, s_fw, 0, nullptr, 0, nullptr, nullptr, ms, gr.pos.data(), gr.qs.data(),
                          s_new.data(), d2);
          const double same = d2[0] - (excl_intra + excl_self) * (1.0 - 0.0);
          ew = same + 2.0 * d2[1];
          rosen *= std::exp(-g->beta * ew);
        }
        rosen *= std::exp(-g->beta * g->tail_insert);  // Insertion_Body (mc_swap_utilities.h:105-108)
        rosen_rec = rosen;
        const double pre = g->beta * bigP / (1.0 + (double)N);  // GetPrefactor INSERTION
        const double pacc = pre * rosen / g->ideal_rosenbluth;
        note_acceptance(uacc, pacc);
        if (rosen > 1e-150 && uacc < pacc) {
          st->accepted[2]++;
          const int64_t at0 = S.comp_start[comp + 1];
          for (int64_t a = 0; a < ms; ++a) {
            for (int d = 0; d < 3; ++d) S.pos.insert(S.pos.begin() + 3 * (at0 + a) + d, gr.pos[3 * a + d]);
            S.charge.insert(S.charge.begin() + at0 + a, mol_charge[a]);
            S.type.insert(S.type.begin() + at0 + a, mol_type[a]);
            S.molid.insert(S.molid.begin() + at0 + a, N);
            S.scale.insert(S.scale.begin() + at0 + a, 1.0);
            S.scc.insert(S.scc.begin() + at0 + a, 1.0);
          }
          for (int64_t c = comp + 1; c <= ncomp; ++c) S.comp_start[c] += ms;
          if (N == 0) std::copy(gr.pos.begin(), gr.pos.end(), slot0.begin());
          if (charged) std::copy(s_new.begin(), s_new.end(), s_ads);
          const double ev = gr.e1[0] + gr.e1[2] + gr.e2[0] + gr.e2[2];
          const double er = gr.e1[1] + gr.e1[3] + gr.e2[1] + gr.e2[3];
          st->energy[0] += ev;
          st->energy[1] += er;
          st->energy[2] += ew;
          st->energy[3] += ev + er + ew;
        }
      }
      st->rosen[0] += rosen_rec;
      st->rosen[1] += rosen_rec * rosen_rec;
      st->rosen[2] += 1.0;
    } else if (kind == 3 && N > 0) {  // CBMC deletion (DeletionMove::Run, move_struct.h:148-167)
      st->attempts[3]++;
      const int64_t m0 = a0 + mol * ms;
      std::vector<double> oldp(S.pos.begin() + 3 * m0, S.pos.begin() + 3 * (m0 + ms));
      ora_atoms at = S.view();
      Grow gr = cbmc_grow(box, ff, &at, comp, ms, slot0.data(), mol_charge, mol_type, g->ntrials, g->norient,
                          g->beta, g->seed, g->stream, move, mol, G_DELETE, oldp.data());
      st->trial_configs += gr.configs;
      st->trial_beads += gr.beads;
      if (gr.ok) {
        double rosen = gr.rosen, ew = 0.0;
        std::vector<double> q(S.charge.begin() + m0, S.charge.begin() + m0 + ms);
        if (charged) {
          double d2[2];
          ora_ewald_delta(box, s_ads, s_fw, 0, nullptr, ms, oldp.data(), q.data(), 0, nullptr, nullptr,
                          s_new.data(), d2);
          const double same = d2[0] - (excl_intra + excl_self) * (0.0 - 1.0);
          ew = same + 2.0 * d2[1];
          rosen /= std::exp(-g->beta * ew);
        }
        // Deletion_Body (mc_swap_utilities.h:197-200): the weight is divided by
        // exp(-beta TailE) with TailE the deletion difference, -tail_insert here
        rosen /= std::exp(-g->beta * -g->tail_insert);
        const double pre = (double)N / (g->beta * bigP);  // GetPrefactor DELETION
        const double pacc = pre * g->ideal_rosenbluth / rosen;
        note_acceptance(uacc, pacc);
        if (uacc < pacc) {
          st->accepted[3]++;
          const int64_t last = a0 + (N - 1) * ms;
          if (mol == 0 && N > 1)
            for (int64_t k = 0; k < 3 * ms; ++k) slot0[k] = S.pos[3 * last + k];
          for (int64_t a = 0; a < ms; ++a) {  // Update_deletion_data_Parallel: last molecule into the slot
            for (int d = 0; d < 3; ++d) S.pos[3 * (m0 + a) + d] = S.pos[3 * (last + a) + d];
            S.charge[m0 + a] = S.charge[last + a];
            S.type[m0 + a] = S.type[last + a];
          }
          S.pos.erase(S.pos.begin() + 3 * last, S.pos.begin() + 3 * (last + ms));
          S.charge.erase(S.charge.begin() + last, S.charge.begin() + last + ms);
          S.type.erase(S.type.begin() + last, S.type.begin() + last + ms);
          S.molid.erase(S.molid.begin() + last, S.molid.begin() + last + ms);
          S.scale.erase(S.scale.begin() + last, S.scale.begin() + last + ms);
          S.scc.erase(S.scc.begin() + last, S.scc.begin() + last + ms);
          for (int64_t c = comp + 1; c <= ncomp; ++c) S.comp_start[c] -= ms;
          if (charged) std::copy(s_new.begin(), s_new.end(), s_ads);
          const double ev = gr.e1[0] + gr.e1[2] + gr.e2[0] + gr.e2[2];
          const double er = gr.e1[1] + gr.e1[3] + gr.e2[1] + gr.e2[3];
          st->energy[0] -= ev;
          st->energy[1] -= er;
          st->energy[2] += ew;
          st->energy[3] += -ev - er + ew;
        }
      }
    }
    for (int64_t k = 0; k < ng; ++k) {
      const int64_t ck = gk[k].component;
      stk[k].sum_n += (double)((S.comp_start[ck + 1] - S.comp_start[ck]) / molsize[ck]);
      stk[k].last_margin = g_margin;
    }
  }
  // write the state back (component regions from comp_off)
  for (int64_t c = 0; c < ncomp; ++c) {
    comp_size[c] = S.comp_start[c + 1] - S.comp_start[c];
    for (int64_t i = 0; i < comp_size[c]; ++i) {
      const int64_t k = comp_off[c] + i, j = S.comp_start[c] + i;
      for (int d = 0; d < 3; ++d) pos[3 * k + d] = S.pos[3 * j + d];
      charge[k] = S.charge[j];
      type[k] = S.type[j];
      molid[k] = S.molid[j];
    }
  }
  for (int64_t k = 0; k < ng; ++k) {
    stk[k].n_molecules = comp_size[gk[k].component] / molsize[gk[k].component];
    // the slot-0 coordinates the orientations grow from, for a later call that continues the chain
    std::copy(slot0s[k].begin(), slot0s[k].end(), mol_pos_k[k]);
  }
}

extern "C" void ora_gcmc_run(const ora_box* box, const ora_ff* ff, double* pos, double* charge, int64_t* type,
                             int64_t* molid, int64_t ncomp, int64_t nhost, int64_t* comp_size,
                             const int64_t* comp_off, const int64_t* molsize, const double* mol_pos,
                             const double* mol_charge, const int64_t* mol_type, double excl_intra,
                             double excl_self, double* s_fw, double* s_ads, const ora_gcmc* g,
                             uint64_t first_step, int64_t nsteps, ora_gcmc_stats* st) {
  std::vector<double> slot0(mol_pos, mol_pos + 3 * molsize[g->component]);
  double* slot0_p = slot0.data();
  ora_gcmc_run_mix(box, ff, pos, charge, type, molid, ncomp, nhost, comp_size, comp_off, molsize, &slot0_p,
                   &mol_charge, &mol_type, &excl_intra, &excl_self, s_fw, s_ads, g, 1, first_step, nsteps, st);
}
