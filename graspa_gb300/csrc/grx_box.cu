// grx_box.cu -- box lifecycle, component upload, Ewald k-vector table, structure
// factors and FP64 totals (drift checks).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "grx_host.h"

namespace grx {

static thread_local char g_err[512] = "";
static std::atomic<uint64_t> g_launches{0};

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

grx_status cuda_status(cudaError_t e, const char* what) {
  set_error("%s: %s", what, cudaGetErrorString(e));
  if (e == cudaErrorMemoryAllocation) return GRX_ERR_OUT_OF_MEMORY;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return GRX_ERR_NO_DEVICE;
  return GRX_ERR_CUDA;
}

void count_launch(uint64_t n) { g_launches += n; }

static thread_local size_t g_h2d = 0, g_d2h = 0;
void note_transfer(size_t h2d, size_t d2h) { g_h2d = h2d; g_d2h = d2h; }

int sm_count(grx_box* b) {
  if (!b->num_sms) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, b->device);
    b->num_sms = v > 0 ? v : 1;
  }
  return b->num_sms;
}

cudaError_t dev_alloc(grx_box* b, void** p, size_t bytes) {
  if (b->arena) {
    *p = arena_alloc(b->arena, bytes);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
  }
  return cudaMalloc(p, bytes);
}

void dev_free(grx_box* b, void* p) {
  if (!p) return;
  if (b->arena) arena_free(b->arena, p);
  else cudaFree(p);
}

grx_status ensure_scratch(grx_box* b, size_t bytes) {
  if (bytes <= b->scratch_bytes) return GRX_OK;
  dev_free(b, b->scratch);
  b->scratch = nullptr;
  b->scratch_bytes = 0;
  size_t want = std::max(bytes, (size_t)1 << 20);
  GRX_CHECK_CUDA(dev_alloc(b, (void**)&b->scratch, want), "scratch allocation");
  b->scratch_bytes = want;
  return GRX_OK;
}

grx_status ensure_pinned(grx_box* b, size_t bytes) {
  if (bytes <= b->pinned_bytes) return GRX_OK;
  if (b->pinned) cudaFreeHost(b->pinned);
  b->pinned = nullptr;
  b->pinned_bytes = 0;
  size_t want = std::max(bytes, (size_t)1 << 16);
  GRX_CHECK_CUDA(cudaMallocHost(&b->pinned, want), "pinned staging allocation");
  b->pinned_bytes = want;
  return GRX_OK;
}

grx_status ensure_results(grx_box* b, size_t n) {
  if (n <= b->results_cap) return GRX_OK;
  dev_free(b, b->d_results);
  b->d_results = nullptr;
  b->results_cap = 0;
  size_t want = std::max(n, (size_t)1024);
  GRX_CHECK_CUDA(dev_alloc(b, (void**)&b->d_results, want * sizeof(grx_widom_result)), "result buffer");
  b->results_cap = want;
  return GRX_OK;
}

void refresh_dev(grx_box* b) {
  BoxDev& d = b->dev;
  d.ncomp = b->ncomp;
  d.nhost = b->nhost;
  for (int c = 0; c <= b->ncomp; ++c) d.comp_off[c] = (int)b->off[c];
  d.comp_size = b->d_size;
  d.pos64 = b->pos64;
  d.hi = b->hi;
  d.lo = b->lo;
  d.meta = b->meta;
  d.scale = b->scale;
  d.charge = b->charge;
  d.ff64 = b->ff64;
  d.ffc10 = b->ffc10;
  d.ff32 = b->ff32;
  d.nvec = b->nvec;
  d.nact = b->nact;
  d.kact = b->kact;
  d.ktemp = b->ktemp;
  d.s_fw = b->s_fw;
  d.s_ads = b->s_ads;
  d.s_tmp = b->s_tmp;
  d.host_end = (int)b->off[b->nhost];
  d.tile_c = b->tile_c;
  d.tile_r = b->tile_r;
  d.ntiles = b->ntiles;
  d.ctab = b->ctab;
  d.ctab_base = b->ctab_base;
  d.ctab_n = b->ctab_n;
  d.ctabf = b->ctabf;
  d.qdf = b->qdf;
  d.ffdf = b->ffdf;
  d.ffdf2 = b->ffdf2;
  d.ewA = b->ewA;
  d.ewF = b->ewF;
  d.ewT = b->ewT;
  const grx_box* h = b->parent ? b->parent : b;
  d.hpos64 = h->pos64;
  d.hhi = h->hi;
  d.hlo = h->lo;
  d.hmeta = h->meta;
  d.hscale = h->scale;
  d.hqdf = h->qdf;
  d.hrec = h->hrec;
  d.htype = h->htype;
  d.shared_host = b->parent ? 1 : 0;
  d.vox = h->vox_on;
  d.vmeta = h->vmeta;
  d.vlist = h->vlist;
  for (int k = 0; k < 3; ++k) d.vn[k] = h->vn[k];
  d.vchunks = h->vchunks;
}

static float2 split_df(double x) {
  const float h = (float)x;
  return make_float2(h, (float)(x - (double)h));
}

static double hi_part(double x) { return std::nearbyint(x * GRX_GRID_COORD) / GRX_GRID_COORD; }

// Host minimum image (PBC(), maths.cuh:427-450), used for exclusion constants.
static void pbc_host(const BoxDev& b, double* d) {
  if (b.cubic) {
    for (int k = 0; k < 3; ++k) {
      const int kk = 4 * k;
      d[k] -= (double)(int)(d[k] * b.inv[kk] + ((d[k] >= 0.0) ? 0.5 : -0.5)) * b.cell[kk];
    }
  } else {
    double s[3];
    s[0] = b.inv[0] * d[0] + b.inv[3] * d[1] + b.inv[6] * d[2];
    s[1] = b.inv[1] * d[0] + b.inv[4] * d[1] + b.inv[7] * d[2];
    s[2] = b.inv[2] * d[0] + b.inv[5] * d[1] + b.inv[8] * d[2];
    for (int k = 0; k < 3; ++k) s[k] -= (double)(int)(s[k] + ((s[k] >= 0.0) ? 0.5 : -0.5));
    d[0] = b.cell[0] * s[0] + b.cell[3] * s[1] + b.cell[6] * s[2];
    d[1] = b.cell[1] * s[0] + b.cell[4] * s[1] + b.cell[7] * s[2];
    d[2] = b.cell[2] * s[0] + b.cell[5] * s[1] + b.cell[8] * s[2];
  }
}

// Real-space Coulomb kernel g(s) = erfc(alpha sqrt(s)) / sqrt(s) as piecewise quintic
// polynomials in s = r^2. Pieces follow the FP32 bit pattern of s (64 per octave) from
// s = 0.25 A^2 to just past the cutoff, so the device finds its piece with one shift of
// the FP32 bits. Each piece is the degree-5 interpolant at Chebyshev nodes, fitted in
// long double from erfcl; the worst relative error found on a dense sample is kept in
// ctab_maxrel (about 1e-14 for the benchmark systems).
struct CoulombTable {
  int base = 0, n = 0;
  double maxrel = 0.0;
  std::vector<double> tab;  // 8 per piece: s0, 1/width, 6 coefficients
  std::vector<float4> tf;   // the double-float copy
};

static void fit_coulomb_table(double alpha, double cut2, CoulombTable& T);

// The table depends on (alpha, cutoff^2) only, and its long-double fit costs tens of
// milliseconds (software quad precision on some hosts): fitted once per pair of values in
// the process, then uploaded per box.
static const CoulombTable& coulomb_table(double alpha, double cut2) {
  static std::mutex m;
  static std::map<std::pair<uint64_t, uint64_t>, CoulombTable> cache;
  uint64_t ka, kc;
  std::memcpy(&ka, &alpha, 8);
  std::memcpy(&kc, &cut2, 8);
  std::lock_guard<std::mutex> g(m);
  auto it = cache.find({ka, kc});
  if (it != cache.end()) return it->second;
  if (cache.size() >= 64) cache.clear();
  CoulombTable& T = cache[{ka, kc}];
  fit_coulomb_table(alpha, cut2, T);
  return T;
}

static grx_status build_coulomb_table(grx_box* b, double alpha, double cut2) {
  const CoulombTable& T = coulomb_table(alpha, cut2);
  b->ctab_base = T.base;
  b->ctab_n = T.n;
  b->ctab_maxrel = T.maxrel;
  GRX_CHECK_CUDA(dev_alloc(b, (void**)&b->ctab, T.tab.size() * sizeof(double)), "alloc Coulomb table");
  GRX_CHECK_CUDA(cudaMemcpy(b->ctab, T.tab.data(), T.tab.size() * sizeof(double), cudaMemcpyHostToDevice),
                 "upload Coulomb table");
  GRX_CHECK_CUDA(dev_alloc(b, (void**)&b->ctabf, T.tf.size() * sizeof(float4)), "alloc Coulomb table (float pairs)");
  GRX_CHECK_CUDA(cudaMemcpy(b->ctabf, T.tf.data(), T.tf.size() * sizeof(float4), cudaMemcpyHostToDevice),
                 "upload Coulomb table (float pairs)");
  return GRX_OK;
}

static void fit_coulomb_table(double alpha, double cut2, CoulombTable& T) {
  const float s_lo = 0.25f;
  uint32_t lo_bits, hi_bits;
  std::memcpy(&lo_bits, &s_lo, 4);
  const float s_hi = (float)(cut2 * (1.0 + 1e-4) + 1e-2);
  std::memcpy(&hi_bits, &s_hi, 4);
  const int base = (int)(lo_bits >> 17);
  const int n = (int)(hi_bits >> 17) - base + 2;
  std::vector<double> tab(8 * (size_t)n);
  const long double PI = 3.141592653589793238462643383279502884L;
  auto g = [&](long double sv) { const long double r = sqrtl(sv); return erfcl((long double)alpha * r) / r; };
  double maxrel = 0.0;
  for (int k = 0; k < n; ++k) {
    const uint32_t ab = (uint32_t)(base + k) << 17, bb = (uint32_t)(base + k + 1) << 17;
    float fa, fb;
    std::memcpy(&fa, &ab, 4);
    std::memcpy(&fb, &bb, 4);
    const long double s0 = fa, w = (long double)fb - (long double)fa;
    long double A[6][7];
    for (int j = 0; j < 6; ++j) {
      const long double t = 0.5L - 0.5L * cosl((2 * j + 1) * PI / 12.0L);
      long double p = 1.0L;
      for (int c = 0; c < 6; ++c) { A[j][c] = p; p *= t; }
      A[j][6] = g(s0 + w * t);
    }
    for (int c = 0; c < 6; ++c) {  // Gaussian elimination, partial pivoting
      int piv = c;
      for (int r = c + 1; r < 6; ++r)
        if (fabsl(A[r][c]) > fabsl(A[piv][c])) piv = r;
      for (int q = 0; q < 7; ++q) std::swap(A[c][q], A[piv][q]);
      for (int r = 0; r < 6; ++r) {
        if (r == c) continue;
        const long double f = A[r][c] / A[c][c];
        for (int q = c; q < 7; ++q) A[r][q] -= f * A[c][q];
      }
    }
    double* e = &tab[8 * (size_t)k];
    e[0] = (double)s0;
    e[1] = (double)(1.0L / w);
    for (int c = 0; c < 6; ++c) e[2 + c] = (double)(A[c][6] / A[c][c]);
    for (int m = 0; m <= 16; ++m) {
      const double sv = e[0] + (double)w * (m / 16.0);
      const double t = (sv - e[0]) * e[1];
      const double pv = e[2] + t * (e[3] + t * (e[4] + t * (e[5] + t * (e[6] + t * e[7]))));
      const long double ex = g(sv);
      maxrel = std::max(maxrel, (double)fabsl((pv - ex) / ex));
    }
  }
  T.base = base;
  T.n = n;
  T.maxrel = maxrel;
  // double-float copy: s0 and 1/width are exact floats (width is a power of two)
  std::vector<float4> tf(4 * (size_t)n);
  for (int k = 0; k < n; ++k) {
    const double* e = &tab[8 * (size_t)k];
    float2 c[6];
    for (int j = 0; j < 6; ++j) {
      const float h = (float)e[2 + j];
      c[j] = make_float2(h, (float)(e[2 + j] - (double)h));
    }
    tf[4 * k + 0] = make_float4((float)e[0], (float)e[1], c[0].x, c[0].y);
    tf[4 * k + 1] = make_float4(c[1].x, c[1].y, c[2].x, c[2].y);
    tf[4 * k + 2] = make_float4(c[3].x, c[3].y, c[4].x, c[4].y);
    tf[4 * k + 3] = make_float4(c[5].x, c[5].y, 0.0f, 0.0f);
  }
  T.tab = std::move(tab);
  T.tf = std::move(tf);
}

// Storage order of host atoms: recursive bisection of the wrapped Cartesian positions
// along the longest extent, into leaves of 32 consecutive atoms (storage slot -> caller
// index). Leaves are compact boxes, tighter than runs of a space-filling curve where a
// framework has pores.
static void kd_order(const BoxDev& d, const double* pos, size_t n, std::vector<int>& order) {
  std::vector<double> X(3 * n);
  for (size_t i = 0; i < n; ++i) {
    double s[3];
    for (int k = 0; k < 3; ++k) {
      s[k] = d.inv[k] * pos[3 * i] + d.inv[3 + k] * pos[3 * i + 1] + d.inv[6 + k] * pos[3 * i + 2];
      s[k] -= std::floor(s[k]);
    }
    for (int j = 0; j < 3; ++j) X[3 * i + j] = s[0] * d.cell[j] + s[1] * d.cell[3 + j] + s[2] * d.cell[6 + j];
  }
  order.resize(n);
  for (size_t i = 0; i < n; ++i) order[i] = (int)i;
  std::vector<std::pair<size_t, size_t>> todo = {{0, n}};
  while (!todo.empty()) {
    const auto [lo, hi] = todo.back();
    todo.pop_back();
    if (hi - lo <= 32) continue;
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (size_t j = lo; j < hi; ++j)
      for (int k = 0; k < 3; ++k) {
        mn[k] = std::min(mn[k], X[3 * order[j] + k]);
        mx[k] = std::max(mx[k], X[3 * order[j] + k]);
      }
    int ax = 0;
    for (int k = 1; k < 3; ++k)
      if (mx[k] - mn[k] > mx[ax] - mn[ax]) ax = k;
    std::stable_sort(order.begin() + lo, order.begin() + hi,
                     [&](int a, int c) { return X[3 * a + ax] < X[3 * c + ax]; });
    const size_t nl = (((hi - lo) / 32 + 1) / 2) * 32;  // left half: whole leaves
    todo.push_back({lo + nl, hi});
    todo.push_back({lo, lo + nl});
  }
}

// Tiles of 32 consecutive host atoms: two records per tile, {centre, bounding-sphere
// radius} and {half extents of the bounding box, 0}, from minimum images relative to the
// tile's first atom, rounded up.
static grx_status build_tiles(grx_box* b) {
  b->h_tile_c.clear();
  b->h_tile_r.clear();
  for (int c = 0; c < b->nhost; ++c) {
    const int n = b->size[c];
    const size_t o = b->off[c];
    for (int t0 = 0; t0 < n; t0 += 32) {
      const int t1 = std::min(n, t0 + 32);
      const double* a0 = &b->h_pos[3 * (o + t0)];
      double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
      std::vector<double> u(3 * (t1 - t0));
      int compact = 1;  // stored positions need no lattice shift relative to the first atom
      for (int i = t0; i < t1; ++i) {
        double dv[3] = {b->h_pos[3 * (o + i)] - a0[0], b->h_pos[3 * (o + i) + 1] - a0[1],
                        b->h_pos[3 * (o + i) + 2] - a0[2]};
        const double raw[3] = {dv[0], dv[1], dv[2]};
        pbc_host(b->dev, dv);
        if (raw[0] != dv[0] || raw[1] != dv[1] || raw[2] != dv[2]) compact = 0;
        for (int k = 0; k < 3; ++k) {
          u[3 * (i - t0) + k] = a0[k] + dv[k];
          lo[k] = std::min(lo[k], a0[k] + dv[k]);
          hi[k] = std::max(hi[k], a0[k] + dv[k]);
        }
      }
      const double cx = 0.5 * (lo[0] + hi[0]), cy = 0.5 * (lo[1] + hi[1]), cz = 0.5 * (lo[2] + hi[2]);
      double r2 = 0.0;
      for (int i = 0; i < t1 - t0; ++i) {
        const double dx = u[3 * i] - cx, dy = u[3 * i + 1] - cy, dz = u[3 * i + 2] - cz;
        r2 = std::max(r2, dx * dx + dy * dy + dz * dz);
      }
      const float rad = (float)(std::sqrt(r2) * (1.0 + 1e-6) + 1e-4);
      b->h_tile_c.push_back(make_float4((float)cx, (float)cy, (float)cz, rad));
      float hw[3];
      for (int k = 0; k < 3; ++k) hw[k] = (float)(0.5 * (hi[k] - lo[k]) * (1.0 + 1e-6) + 1e-4);
      b->h_tile_c.push_back(make_float4(hw[0], hw[1], hw[2], 0.0f));
      b->h_tile_r.push_back(make_int4((int)(o + t0), (int)(o + t1), c, compact));
    }
  }
  b->ntiles = (int)b->h_tile_r.size();
  // Visiting order: a stride permutation of the k-d order (stride near 0.618 nt, coprime to
  // nt). The tiles that survive a bead's cutoff cull are spatial neighbours, adjacent in k-d
  // order; scattered through the list, they spread evenly over the contiguous item ranges of
  // a bead pass instead of falling into one or two warps' items. Atoms keep their k-d order.
  const int nt = b->ntiles;
  if (nt > 2) {
    int stride = std::max(1, (int)(0.6180339887 * nt));
    auto gcd = [](int x, int y) { while (y) { const int t = x % y; x = y; y = t; } return x; };
    while (gcd(stride, nt) != 1) ++stride;
    std::vector<float4> c2(2 * (size_t)nt);
    std::vector<int4> r2(nt);
    for (int j = 0; j < nt; ++j) {
      const int t = (int)((int64_t)j * stride % nt);
      c2[2 * j] = b->h_tile_c[2 * t];
      c2[2 * j + 1] = b->h_tile_c[2 * t + 1];
      r2[j] = b->h_tile_r[t];
    }
    b->h_tile_c.swap(c2);
    b->h_tile_r.swap(r2);
  }
  if ((size_t)b->ntiles > b->tile_cap) {
    dev_free(b, b->tile_c);
    dev_free(b, b->tile_r);
    b->tile_c = nullptr;
    b->tile_r = nullptr;
    b->tile_cap = 0;
    GRX_CHECK_CUDA(dev_alloc(b, (void**)&b->tile_c, 2 * b->ntiles * sizeof(float4)), "alloc tiles");
    GRX_CHECK_CUDA(dev_alloc(b, (void**)&b->tile_r, b->ntiles * sizeof(int4)), "alloc tile ranges");
    b->tile_cap = b->ntiles;
  }
  if (b->ntiles) {
    GRX_CHECK_CUDA(cudaMemcpy(b->tile_c, b->h_tile_c.data(), 2 * b->ntiles * sizeof(float4), cudaMemcpyHostToDevice),
                   "upload tiles");
    GRX_CHECK_CUDA(cudaMemcpy(b->tile_r, b->h_tile_r.data(), b->ntiles * sizeof(int4), cudaMemcpyHostToDevice),
                   "upload tile ranges");
  }
  refresh_dev(b);
  return GRX_OK;
}

// Active k slots and their prefactors: the slot unranking and cutoff test of
// Fourier_Ewald_Diff (Ewald_Energy_Functions.h:294-333) and the factor of :359-361.
static void build_kvectors(grx_box* b, const grx_box_geometry& g) {
  const int kxm = g.kmax[0], kym = g.kmax[1], kzm = g.kmax[2];
  b->nvec = (kxm + 1) * (2 * kym + 1) * (2 * kzm + 1);
  b->h_kact.clear();
  b->h_ktemp.clear();
  const double* ic = g.inverse_cell;
  const double PI = 3.14159265358979323846;
  const double prefactor = g.prefactor * (2.0 * PI / g.volume);
  const double alpha_sq = g.alpha * g.alpha;
  for (int kxyz = 0; kxyz < b->nvec; ++kxyz) {
    const int kz = kxyz % (2 * kzm + 1) - kzm;
    const int kxy = kxyz / (2 * kzm + 1);
    const int kx = kxy / (2 * kym + 1);
    const int ky = kxy % (2 * kym + 1) - kym;
    double ksqr = (double)(kx * kx + ky * ky + kz * kz);
    if (g.use_lammps_ewald) {
      const double* C = g.cell;
      const double lx = C[0], ly = C[4], lz = C[8], xy = C[3], xz = C[6], yz = C[7];
      const double ux = 2 * PI / lx, uy = 2 * PI * (-xy) / lx / ly;
      const double uz = 2 * PI * (xy * yz - ly * xz) / lx / ly / lz;
      const double vy = 2 * PI / ly, vz = 2 * PI * (-yz) / ly / lz, wz = 2 * PI / lz;
      const double kvx = kx * ux, kvy = kx * uy + ky * vy, kvz = kx * uz + ky * vz + kz * wz;
      ksqr = kvx * kvx + kvy * kvy + kvz * kvz;
    }
    if (!((ksqr > 1e-10) && (ksqr < g.reciprocal_cutoff))) continue;
    double kv[3];
    // reciprocal vectors are the rows of the inverse cell: ax = (inv[0], inv[3], inv[6])
    const double ax[3] = {ic[0], ic[3], ic[6]};
    const double ay[3] = {ic[1], ic[4], ic[7]};
    const double az[3] = {ic[2], ic[5], ic[8]};
    for (int d = 0; d < 3; ++d)
      kv[d] = ax[d] * 2.0 * PI * (double)kx + ay[d] * 2.0 * PI * (double)ky +
              az[d] * 2.0 * PI * (double)kz;
    const double rksq = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
    const double factor = (kx == 0) ? (1.0 * prefactor) : (2.0 * prefactor);
    b->h_kact.push_back(make_int4(kx, ky, kz, kxyz));
    b->h_ktemp.push_back(factor * std::exp((-0.25 / alpha_sq) * rksq) / rksq);
  }
  b->nact = (int)b->h_kact.size();
}

}  // namespace grx

using namespace grx;

extern "C" {

const char* grx_status_string(grx_status s) {
  switch (s) {
    case GRX_OK: return "ok";
    case GRX_ERR_INVALID_ARG: return "invalid argument";
    case GRX_ERR_CUDA: return "CUDA error";
    case GRX_ERR_OUT_OF_MEMORY: return "out of device memory";
    case GRX_ERR_TIMEOUT: return "device wait timed out";
    case GRX_ERR_CAPACITY: return "capacity exceeded";
    case GRX_ERR_NO_DEVICE: return "no CUDA device";
    case GRX_ERR_UNSUPPORTED: return "unsupported";
  }
  return "unknown status";
}

const char* grx_last_error(void) { return g_err; }

uint64_t grx_launch_count(void) { return g_launches.load(); }

grx_status grx_last_transfer(size_t* h2d, size_t* d2h) {
  if (h2d) *h2d = g_h2d;
  if (d2h) *d2h = g_d2h;
  return GRX_OK;
}

grx_status grx_device_count(int32_t* n) {
  int v = 0;
  cudaError_t e = cudaGetDeviceCount(&v);
  if (e != cudaSuccess) {
    *n = 0;
    return cuda_status(e, "cudaGetDeviceCount");
  }
  *n = v;
  return GRX_OK;
}

static grx_status box_create(const grx_box_desc* desc, grx_arena* arena, grx_box** out);

grx_status grx_box_create(const grx_box_desc* desc, grx_box** out) { return box_create(desc, nullptr, out); }

grx_status grx_box_create_in(const grx_box_desc* desc, grx_arena* arena, grx_box** out) {
  GRX_REQUIRE(arena, "grx_box_create_in: null arena");
  return box_create(desc, arena, out);
}

static grx_status box_create(const grx_box_desc* desc, grx_arena* arena, grx_box** out) {
  GRX_REQUIRE(desc && out, "grx_box_create: null argument");
  *out = nullptr;
  const grx_forcefield& ff = desc->forcefield;
  const grx_box_geometry& g = desc->geometry;
  GRX_REQUIRE(desc->ncomponents >= 1 && desc->ncomponents <= GRX_MAX_COMPONENTS,
              "grx_box_create: ncomponents out of range");
  GRX_REQUIRE(desc->nhost_components >= 0 && desc->nhost_components <= desc->ncomponents,
              "grx_box_create: nhost_components out of range");
  GRX_REQUIRE(ff.ntypes >= 1 && ff.ntypes <= GRX_MAX_TYPES, "grx_box_create: ntypes out of range");
  GRX_REQUIRE(ff.epsilon && ff.sigma && ff.shift, "grx_box_create: force-field tables missing");
  GRX_REQUIRE(g.volume > 0.0, "grx_box_create: non-positive volume");
  GRX_REQUIRE(g.kmax[0] >= 0 && g.kmax[1] >= 0 && g.kmax[2] >= 0 && g.kmax[0] < 64 &&
                  g.kmax[1] < 64 && g.kmax[2] < 64,
              "grx_box_create: kmax out of range");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    set_error("grx_box_create: no CUDA device");
    return GRX_ERR_NO_DEVICE;
  }
  grx_box* b = new grx_box();
  b->arena = arena;
  cudaGetDevice(&b->device);
  b->ncomp = desc->ncomponents;
  b->nhost = desc->nhost_components;
  size_t acc = 0;
  for (int c = 0; c < b->ncomp; ++c) {
    b->cap[c] = desc->capacity[c];
    b->molsize[c] = desc->molsize[c];
    if (b->molsize[c] == 0 || b->molsize[c] > b->cap[c] + (b->cap[c] == 0)) {
      delete b;
      set_error("grx_box_create: component %d needs molsize >= 1 and capacity >= molsize", c);
      return GRX_ERR_INVALID_ARG;
    }
    b->off[c] = acc;
    acc += (b->cap[c] + 31) / 32 * 32;  // keep every component 128 B aligned
  }
  b->off[b->ncomp] = acc;
  b->total_cap = std::max<size_t>(acc, 32);
  b->h_pos.assign(3 * b->total_cap, 0.0);
  b->h_charge.assign(b->total_cap, 0.0);
  b->h_scale_coul.assign(b->total_cap, 1.0);

  BoxDev& d = b->dev;
  for (int k = 0; k < 9; ++k) {
    d.cell[k] = g.cell[k];
    d.inv[k] = g.inverse_cell[k];
    const double h = hi_part(g.cell[k]);
    d.cell_hi[k] = (float)h;
    d.cell_lo[k] = (float)(g.cell[k] - h);
    d.invf[k] = (float)g.inverse_cell[k];
  }
  d.cubic = g.cubic;
  d.alpha = g.alpha;
  d.prefactor = g.prefactor;
  d.volume = g.volume;
  d.ntypes = ff.ntypes;
  d.use_1264 = ff.use_1264;
  d.no_charges = ff.no_charges;
  d.vdw_real_bias = ff.vdw_real_bias;
  d.cut_vdw2 = ff.cutoff_vdw_sq;
  d.cut_coul2 = ff.cutoff_coul_sq;
  d.overlap = ff.overlap_criteria;
  d.overlapf = (float)ff.overlap_criteria;
  const double cmax = std::max(ff.cutoff_vdw_sq, ff.no_charges ? 0.0 : ff.cutoff_coul_sq);
  // FP32 screening on the hi parts (within 2^-13 A of the coordinates): guard band of
  // 2e-3 A on the radius covers the rounding of both atoms and the FP32 arithmetic.
  d.screen2 = (float)((std::sqrt(cmax) + 2e-3) * (std::sqrt(cmax) + 2e-3));
  d.cut_vdw2_df = split_df(ff.cutoff_vdw_sq);
  d.cut_coul2_df = split_df(ff.cutoff_coul_sq);
  d.cut_vdw2f = (float)ff.cutoff_vdw_sq;
  d.cut_coul2f = (float)ff.cutoff_coul_sq;
  for (int k = 0; k < 3; ++k) d.kmax[k] = g.kmax[k];
  for (int k = 0; k < 9; ++k) d.cellf[k] = (float)g.cell[k];
  // Tile culling needs a lower bound of the periodic distance from a bead to a tile
  // centre. Orthorhombic: the rounded image is the nearest one. General cells: the
  // rounded image e is the nearest one when |e| <= w_min/2 (any other image is at
  // least w_min - |e| away); otherwise max_k |s_k| w_k (s = fractional remainder,
  // w_k = distance between lattice planes) bounds it from below.
  d.cull = 1;
  d.chunk_mult = 1;
  d.ew_rows = 0;
  d.cull_r = (float)(std::sqrt((double)d.screen2) + 0.01);
  {
    const double* C = g.cell;
    const double a[3] = {C[0], C[1], C[2]}, bb[3] = {C[3], C[4], C[5]}, c[3] = {C[6], C[7], C[8]};
    auto cross_norm = [](const double* u, const double* v) {
      const double x = u[1] * v[2] - u[2] * v[1], y = u[2] * v[0] - u[0] * v[2], z = u[0] * v[1] - u[1] * v[0];
      return std::sqrt(x * x + y * y + z * z);
    };
    const double V = std::fabs(a[0] * (bb[1] * c[2] - bb[2] * c[1]) - a[1] * (bb[0] * c[2] - bb[2] * c[0]) +
                               a[2] * (bb[0] * c[1] - bb[1] * c[0]));
    const double w[3] = {V / cross_norm(bb, c), V / cross_norm(c, a), V / cross_norm(a, bb)};
    double wmin = w[0];
    for (int k = 0; k < 3; ++k) {
      d.wperp[k] = (float)(w[k] * (1.0 - 1e-5));
      wmin = std::min(wmin, w[k]);
    }
    const double h = 0.5 * wmin * (1.0 - 1e-4);
    d.half_wmin2 = (float)(h * h);
  }

  const int nt2 = ff.ntypes * ff.ntypes;
  std::vector<FFPair64> f64(nt2);
  std::vector<double> c10(nt2, 0.0);
  std::vector<float4> f32(nt2);
  for (int r = 0; r < nt2; ++r) {
    f64[r].a = ff.epsilon[r];
    f64[r].b = ff.sigma[r];
    f64[r].c = ff.z ? ff.z[r] : 0.0;
    f64[r].shift = ff.shift[r];
    if (ff.c10) c10[r] = ff.c10[r];
    const double s2 = ff.sigma[r] * ff.sigma[r];
    f32[r] = make_float4((float)(4.0 * ff.epsilon[r]), s2 > 0 ? (float)(1.0 / s2) : INFINITY,
                         (float)ff.shift[r], (float)(1.21 * s2));
  }
  std::vector<float4> fdf(nt2);
  std::vector<float2> fdf2(nt2);
  for (int r = 0; r < nt2; ++r) {
    const double s2 = ff.sigma[r] * ff.sigma[r];
    const float2 e4 = split_df(4.0 * ff.epsilon[r]);
    const float2 is2 = s2 > 0 ? split_df(1.0 / s2) : make_float2(INFINITY, 0.0f);
    fdf[r] = make_float4(e4.x, e4.y, is2.x, is2.y);
    fdf2[r] = split_df(ff.shift[r]);
  }
  build_kvectors(b, g);

  auto fail = [&](cudaError_t e, const char* what) {
    grx_status s = cuda_status(e, what);
    grx_box_destroy(b);
    return s;
  };
  cudaError_t e;
  const size_t n = b->total_cap;
  if ((e = dev_alloc(b, (void**)&b->pos64, n * sizeof(double4))) != cudaSuccess) return fail(e, "alloc pos64");
  if ((e = dev_alloc(b, (void**)&b->hi, n * sizeof(float4))) != cudaSuccess) return fail(e, "alloc hi");
  if ((e = dev_alloc(b, (void**)&b->lo, n * sizeof(float4))) != cudaSuccess) return fail(e, "alloc lo");
  if ((e = dev_alloc(b, (void**)&b->meta, n * sizeof(int2))) != cudaSuccess) return fail(e, "alloc meta");
  if ((e = dev_alloc(b, (void**)&b->scale, n * sizeof(double))) != cudaSuccess) return fail(e, "alloc scale");
  if ((e = dev_alloc(b, (void**)&b->charge, n * sizeof(double))) != cudaSuccess) return fail(e, "alloc charge");
  if ((e = dev_alloc(b, (void**)&b->d_size, GRX_MAX_COMPONENTS * sizeof(int))) != cudaSuccess) return fail(e, "alloc sizes");
  if ((e = dev_alloc(b, (void**)&b->ff64, nt2 * sizeof(FFPair64))) != cudaSuccess) return fail(e, "alloc ff64");
  if ((e = dev_alloc(b, (void**)&b->ffc10, nt2 * sizeof(double))) != cudaSuccess) return fail(e, "alloc ffc10");
  if ((e = dev_alloc(b, (void**)&b->ff32, nt2 * sizeof(float4))) != cudaSuccess) return fail(e, "alloc ff32");
  if ((e = dev_alloc(b, (void**)&b->ffdf, nt2 * sizeof(float4))) != cudaSuccess) return fail(e, "alloc ffdf");
  if ((e = dev_alloc(b, (void**)&b->ffdf2, nt2 * sizeof(float2))) != cudaSuccess) return fail(e, "alloc ffdf2");
  if ((e = dev_alloc(b, (void**)&b->qdf, n * sizeof(float2))) != cudaSuccess) return fail(e, "alloc qdf");
  const size_t nh = std::max<size_t>(b->off[b->nhost], 1);
  if ((e = dev_alloc(b, (void**)&b->hrec, 2 * nh * sizeof(float4))) != cudaSuccess) return fail(e, "alloc hrec");
  if ((e = dev_alloc(b, (void**)&b->htype, nh * sizeof(uint16_t))) != cudaSuccess) return fail(e, "alloc htype");
  const size_t nv = std::max(b->nvec, 1), na = std::max(b->nact, 1);
  if ((e = dev_alloc(b, (void**)&b->kact, na * sizeof(int4))) != cudaSuccess) return fail(e, "alloc kact");
  if ((e = dev_alloc(b, (void**)&b->ktemp, na * sizeof(double))) != cudaSuccess) return fail(e, "alloc ktemp");
  if ((e = dev_alloc(b, (void**)&b->s_fw, nv * sizeof(double2))) != cudaSuccess) return fail(e, "alloc s_fw");
  if ((e = dev_alloc(b, (void**)&b->s_ads, nv * sizeof(double2))) != cudaSuccess) return fail(e, "alloc s_ads");
  if ((e = dev_alloc(b, (void**)&b->s_tmp, nv * sizeof(double2))) != cudaSuccess) return fail(e, "alloc s_tmp");
  if ((e = dev_alloc(b, (void**)&b->ewA, na * sizeof(float4))) != cudaSuccess) return fail(e, "alloc ewA");
  if ((e = dev_alloc(b, (void**)&b->ewF, na * sizeof(float4))) != cudaSuccess) return fail(e, "alloc ewF");
  if ((e = dev_alloc(b, (void**)&b->ewT, na * sizeof(float2))) != cudaSuccess) return fail(e, "alloc ewT");
  cudaMemset(b->pos64, 0, n * sizeof(double4));
  cudaMemset(b->hi, 0, n * sizeof(float4));
  cudaMemset(b->lo, 0, n * sizeof(float4));
  cudaMemset(b->meta, 0, n * sizeof(int2));
  cudaMemset(b->scale, 0, n * sizeof(double));
  cudaMemset(b->charge, 0, n * sizeof(double));
  cudaMemset(b->d_size, 0, GRX_MAX_COMPONENTS * sizeof(int));
  cudaMemset(b->s_fw, 0, nv * sizeof(double2));
  cudaMemset(b->s_ads, 0, nv * sizeof(double2));
  cudaMemset(b->s_tmp, 0, nv * sizeof(double2));
  cudaMemcpy(b->ff64, f64.data(), nt2 * sizeof(FFPair64), cudaMemcpyHostToDevice);
  cudaMemcpy(b->ffc10, c10.data(), nt2 * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemcpy(b->ff32, f32.data(), nt2 * sizeof(float4), cudaMemcpyHostToDevice);
  cudaMemcpy(b->ffdf, fdf.data(), nt2 * sizeof(float4), cudaMemcpyHostToDevice);
  cudaMemcpy(b->ffdf2, fdf2.data(), nt2 * sizeof(float2), cudaMemcpyHostToDevice);
  cudaMemset(b->qdf, 0, n * sizeof(float2));
  cudaMemset(b->hrec, 0, 2 * nh * sizeof(float4));
  cudaMemset(b->htype, 0, nh * sizeof(uint16_t));
  if (b->nact) {
    cudaMemcpy(b->kact, b->h_kact.data(), b->nact * sizeof(int4), cudaMemcpyHostToDevice);
    cudaMemcpy(b->ktemp, b->h_ktemp.data(), b->nact * sizeof(double), cudaMemcpyHostToDevice);
  }
  if ((e = cudaStreamSynchronize(nullptr)) != cudaSuccess) return fail(e, "box upload");
  if (!ff.no_charges) {
    grx_status st = build_coulomb_table(b, g.alpha, ff.cutoff_coul_sq);
    if (st) {
      grx_box_destroy(b);
      return st;
    }
  }
  refresh_dev(b);
  *out = b;
  return GRX_OK;
}

grx_status grx_box_footprint(const grx_box_desc* desc, size_t* bytes) {
  GRX_REQUIRE(desc && bytes, "grx_box_footprint: null argument");
  GRX_REQUIRE(desc->ncomponents >= 1 && desc->ncomponents <= GRX_MAX_COMPONENTS, "grx_box_footprint: bad components");
  auto al = [](size_t n) { return (n + 255) / 256 * 256; };
  size_t acc = 0, ntiles = 0, nh = 0;
  for (int c = 0; c < desc->ncomponents; ++c) {
    acc += (desc->capacity[c] + 31) / 32 * 32;
    if (c < desc->nhost_components) {
      ntiles += (desc->capacity[c] + 31) / 32;
      nh += (desc->capacity[c] + 31) / 32 * 32;
    }
  }
  nh = std::max<size_t>(nh, 1);
  const size_t n = std::max<size_t>(acc, 32);
  const size_t nt2 = (size_t)desc->forcefield.ntypes * desc->forcefield.ntypes;
  grx_box tmp;
  build_kvectors(&tmp, desc->geometry);
  const size_t nv = std::max(tmp.nvec, 1), na = std::max(tmp.nact, 1);
  size_t t = al(n * sizeof(double4)) + 2 * al(n * sizeof(float4)) + al(n * sizeof(int2)) + 2 * al(n * sizeof(double)) +
             al(n * sizeof(float2)) + al(GRX_MAX_COMPONENTS * sizeof(int));
  t += al(nt2 * sizeof(FFPair64)) + al(nt2 * sizeof(double)) + 2 * al(nt2 * sizeof(float4)) + al(nt2 * sizeof(float2));
  t += al(na * sizeof(int4)) + al(na * sizeof(double)) + 3 * al(nv * sizeof(double2)) + 2 * al(na * sizeof(float4)) +
       al(na * sizeof(float2));
  t += al(ntiles * sizeof(float4)) + al(ntiles * sizeof(int4));
  t += al(2 * nh * sizeof(float4)) + al(nh * sizeof(uint16_t));  // host atom records

  if (!desc->forcefield.no_charges) {
    const float s_lo = 0.25f, s_hi = (float)(desc->forcefield.cutoff_coul_sq * (1.0 + 1e-4) + 1e-2);
    uint32_t lb, hb;
    std::memcpy(&lb, &s_lo, 4);
    std::memcpy(&hb, &s_hi, 4);
    const size_t np = (size_t)((int)(hb >> 17) - (int)(lb >> 17) + 2);
    t += al(8 * np * sizeof(double)) + al(4 * np * sizeof(float4));
  }
  t += al((size_t)1 << 20) + al(1024 * sizeof(grx_widom_result));  // first scratch and result buffers
  *bytes = t;
  return GRX_OK;
}

grx_status grx_box_create_replica(grx_box* parent, grx_box** out) {
  GRX_REQUIRE(parent && out, "grx_box_create_replica: null argument");
  GRX_REQUIRE(!parent->parent, "grx_box_create_replica: the parent is itself a replica");
  GRX_REQUIRE(parent->sk_valid, "grx_box_create_replica: the parent needs current structure factors");
  *out = nullptr;
  if (!parent->ewdf_valid && parent->nact > 0) {
    grx_status st = ewald_df_refresh(parent);
    if (st) return st;
  }
  GRX_CHECK_CUDA(cudaStreamSynchronize(parent->stream), "replica: parent ready");
  grx_box* r = new grx_box(*parent);
  r->parent = parent;
  r->replicas = 0;
  r->pos64 = nullptr; r->hi = nullptr; r->lo = nullptr; r->meta = nullptr; r->scale = nullptr;
  r->charge = nullptr; r->qdf = nullptr; r->d_size = nullptr;
  r->s_ads = nullptr; r->s_tmp = nullptr; r->ewA = nullptr;
  r->scratch = nullptr; r->scratch_bytes = 0; r->d_results = nullptr; r->results_cap = 0;
  r->pinned = nullptr; r->pinned_bytes = 0; r->tile_cap = 0;
  parent->replicas++;
  const size_t n = r->total_cap, nv = std::max(r->nvec, 1), na = std::max(r->nact, 1);
  cudaError_t e = cudaSuccess;
  auto al = [&](void** p, size_t bytes) { if (e == cudaSuccess) e = dev_alloc(r, p, bytes); };
  al((void**)&r->pos64, n * sizeof(double4));
  al((void**)&r->hi, n * sizeof(float4));
  al((void**)&r->lo, n * sizeof(float4));
  al((void**)&r->meta, n * sizeof(int2));
  al((void**)&r->scale, n * sizeof(double));
  al((void**)&r->charge, n * sizeof(double));
  al((void**)&r->qdf, n * sizeof(float2));
  al((void**)&r->d_size, GRX_MAX_COMPONENTS * sizeof(int));
  al((void**)&r->s_ads, nv * sizeof(double2));
  al((void**)&r->s_tmp, nv * sizeof(double2));
  al((void**)&r->ewA, na * sizeof(float4));
  if (e != cudaSuccess) {
    grx_status st = cuda_status(e, "replica allocation");
    grx_box_destroy(r);
    return st;
  }
  // guests (and their templates), sizes and S_ads from the parent
  const size_t g0 = r->off[r->nhost], gn = n - g0;
  auto cp = [&](void* dst, const void* src, size_t bytes) {
    if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, r->stream);
  };
  cp(r->pos64 + g0, parent->pos64 + g0, gn * sizeof(double4));
  cp(r->hi + g0, parent->hi + g0, gn * sizeof(float4));
  cp(r->lo + g0, parent->lo + g0, gn * sizeof(float4));
  cp(r->meta + g0, parent->meta + g0, gn * sizeof(int2));
  cp(r->scale + g0, parent->scale + g0, gn * sizeof(double));
  cp(r->charge + g0, parent->charge + g0, gn * sizeof(double));
  cp(r->qdf + g0, parent->qdf + g0, gn * sizeof(float2));
  cp(r->d_size, parent->d_size, GRX_MAX_COMPONENTS * sizeof(int));
  cp(r->s_ads, parent->s_ads, nv * sizeof(double2));
  cp(r->s_tmp, parent->s_tmp, nv * sizeof(double2));
  if (e == cudaSuccess) e = cudaStreamSynchronize(r->stream);
  if (e != cudaSuccess) {
    grx_status st = cuda_status(e, "replica copy");
    grx_box_destroy(r);
    return st;
  }
  r->ewdf_valid = false;  // its S_ads table; the framework tables are the parent's
  refresh_dev(r);
  *out = r;
  return GRX_OK;
}

grx_status grx_box_destroy(grx_box* b) {
  if (!b) return GRX_OK;
  GRX_REQUIRE(b->replicas == 0, "grx_box_destroy: the box still has live replicas");
  if (b->parent) {  // free only what the replica owns
    void* own[] = {b->pos64, b->hi, b->lo, b->meta, b->scale, b->charge, b->d_size, b->qdf,
                   b->s_ads, b->s_tmp, b->ewA, b->scratch, b->d_results};
    for (void* p : own) dev_free(b, p);
    if (b->pinned) cudaFreeHost(b->pinned);
    b->parent->replicas--;
    delete b;
    return GRX_OK;
  }
  void* ptrs[] = {b->pos64, b->hi, b->lo, b->meta, b->scale, b->charge, b->d_size, b->ff64,
                  b->ffc10, b->ff32, b->kact, b->ktemp, b->s_fw, b->s_ads, b->s_tmp,
                  b->scratch, b->d_results, b->tile_c, b->tile_r, b->ctab, b->ctabf, b->qdf,
                  b->ffdf, b->ffdf2, b->ewA, b->ewF, b->ewT, b->vmeta, b->vlist, b->hrec, b->htype};
  for (void* p : ptrs) dev_free(b, p);
  if (b->pinned) cudaFreeHost(b->pinned);
  delete b;
  return GRX_OK;
}

grx_status grx_box_set_stream(grx_box* b, void* s) {
  GRX_REQUIRE(b, "grx_box_set_stream: null box");
  b->stream = (cudaStream_t)s;
  return GRX_OK;
}

grx_status grx_box_set_component(grx_box* b, int32_t comp, const grx_atoms* a, int32_t rigid) {
  GRX_REQUIRE(b && a, "grx_box_set_component: null argument");
  GRX_REQUIRE(comp >= 0 && comp < b->ncomp, "grx_box_set_component: component out of range");
  GRX_REQUIRE(comp >= b->nhost || (!b->parent && b->replicas == 0),
              "grx_box_set_component: framework atoms are shared with replicas (set them on a box without any)");
  const size_t nst = std::max(a->n_stored, a->size);
  if (nst > b->cap[comp] || a->size > b->cap[comp]) {
    set_error("grx_box_set_component: %zu atoms exceed capacity %zu of component %d", nst,
              b->cap[comp], comp);
    return GRX_ERR_CAPACITY;
  }
  GRX_REQUIRE(nst == 0 || (a->pos && a->charge && a->type && a->molid),
              "grx_box_set_component: atom arrays missing");
  // stage the caller's arrays (host or device) on the host
  std::vector<double> pos(3 * nst), sc(nst, 1.0), q(nst), scc(nst, 1.0);
  std::vector<size_t> ty(nst), mol(nst);
  if (nst) {
    GRX_CHECK_CUDA(cudaMemcpy(pos.data(), a->pos, 3 * nst * sizeof(double), cudaMemcpyDefault), "read pos");
    GRX_CHECK_CUDA(cudaMemcpy(q.data(), a->charge, nst * sizeof(double), cudaMemcpyDefault), "read charge");
    GRX_CHECK_CUDA(cudaMemcpy(ty.data(), a->type, nst * sizeof(size_t), cudaMemcpyDefault), "read type");
    GRX_CHECK_CUDA(cudaMemcpy(mol.data(), a->molid, nst * sizeof(size_t), cudaMemcpyDefault), "read molid");
    if (a->scale)
      GRX_CHECK_CUDA(cudaMemcpy(sc.data(), a->scale, nst * sizeof(double), cudaMemcpyDefault), "read scale");
    if (a->scale_coul)
      GRX_CHECK_CUDA(cudaMemcpy(scc.data(), a->scale_coul, nst * sizeof(double), cudaMemcpyDefault),
                     "read scale_coul");
  }
  // rigid exclusion constants from the first molecule in caller order:
  // Calculate_Intra_Molecule_Exclusion and Calculate_Self_Exclusion
  // (ewald_preparation.h:261-298), FP64.
  b->excl_intra[comp] = 0.0;
  b->excl_self[comp] = 0.0;
  const size_t ms = b->molsize[comp];
  if (rigid && nst >= ms && ms > 0) {
    double e = 0.0;
    for (size_t i = 0; i + 1 < ms; ++i) {
      const double fa = scc[i] * q[i];
      for (size_t j = i + 1; j < ms; ++j) {
        const double fb = scc[j] * q[j];
        double dv[3] = {pos[3 * i] - pos[3 * j], pos[3 * i + 1] - pos[3 * j + 1], pos[3 * i + 2] - pos[3 * j + 2]};
        pbc_host(b->dev, dv);
        const double r = std::sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
        e += b->dev.prefactor * fa * fb * std::erf(b->dev.alpha * r) / r;
      }
    }
    const double ps = b->dev.prefactor * b->dev.alpha / std::sqrt(3.14159265358979323846);
    double sv = 0.0;
    for (size_t i = 0; i < ms; ++i) sv += ps * scc[i] * q[i] * scc[i] * q[i];
    b->excl_intra[comp] = e;
    b->excl_self[comp] = sv;
  }
  // host (framework) atoms are stored in k-d order so that 32-atom tiles are compact
  b->perm[comp].clear();
  if (comp < b->nhost && a->size > 1) {
    std::vector<int> order;
    kd_order(b->dev, pos.data(), a->size, order);
    b->perm[comp] = order;
    std::vector<double> pos2(pos), sc2(sc), q2(q), scc2(scc);
    std::vector<size_t> ty2(ty), mol2(mol);
    for (size_t j = 0; j < a->size; ++j) {
      const size_t k = (size_t)order[j];
      for (int d = 0; d < 3; ++d) pos2[3 * j + d] = pos[3 * k + d];
      sc2[j] = sc[k]; q2[j] = q[k]; scc2[j] = scc[k]; ty2[j] = ty[k]; mol2[j] = mol[k];
    }
    pos.swap(pos2); sc.swap(sc2); q.swap(q2); scc.swap(scc2); ty.swap(ty2); mol.swap(mol2);
  }
  for (size_t i = 0; i < nst; ++i)
    if (ty[i] >= (size_t)b->dev.ntypes) {
      set_error("grx_box_set_component: atom %zu has type %zu >= ntypes %d", i, ty[i], b->dev.ntypes);
      return GRX_ERR_INVALID_ARG;
    }
  std::vector<double4> p64(nst);
  std::vector<float4> h(nst), l(nst);
  std::vector<int2> m(nst);
  std::vector<float2> qd(nst);
  const size_t o = b->off[comp];
  bool charged = false;
  for (size_t i = 0; i < nst; ++i) {
    const double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
    const double qe = q[i] * scc[i];
    p64[i] = make_double4(x, y, z, qe);
    const double hx = hi_part(x), hy = hi_part(y), hz = hi_part(z);
    h[i] = make_float4((float)hx, (float)hy, (float)hz, (float)qe);
    l[i] = make_float4((float)(x - hx), (float)(y - hy), (float)(z - hz), (float)sc[i]);
    m[i] = make_int2((int)ty[i], (int)mol[i]);
    qd[i] = split_df(qe);
    if (q[i] != 0.0) charged = true;
    b->h_pos[3 * (o + i)] = x; b->h_pos[3 * (o + i) + 1] = y; b->h_pos[3 * (o + i) + 2] = z;
    b->h_charge[o + i] = q[i];
    b->h_scale_coul[o + i] = scc[i];
  }
  b->size[comp] = (int)a->size;
  b->stored[comp] = nst;
  b->rigid[comp] = rigid;
  b->has_charge[comp] = charged ? 1 : 0;
  if (nst) {
    GRX_CHECK_CUDA(cudaMemcpy(b->pos64 + o, p64.data(), nst * sizeof(double4), cudaMemcpyHostToDevice), "upload pos64");
    GRX_CHECK_CUDA(cudaMemcpy(b->hi + o, h.data(), nst * sizeof(float4), cudaMemcpyHostToDevice), "upload hi");
    GRX_CHECK_CUDA(cudaMemcpy(b->lo + o, l.data(), nst * sizeof(float4), cudaMemcpyHostToDevice), "upload lo");
    GRX_CHECK_CUDA(cudaMemcpy(b->meta + o, m.data(), nst * sizeof(int2), cudaMemcpyHostToDevice), "upload meta");
    GRX_CHECK_CUDA(cudaMemcpy(b->scale + o, sc.data(), nst * sizeof(double), cudaMemcpyHostToDevice), "upload scale");
    GRX_CHECK_CUDA(cudaMemcpy(b->charge + o, q.data(), nst * sizeof(double), cudaMemcpyHostToDevice), "upload charge");
    GRX_CHECK_CUDA(cudaMemcpy(b->qdf + o, qd.data(), nst * sizeof(float2), cudaMemcpyHostToDevice), "upload qdf");
    if (comp < b->nhost) {  // the pair engine's host records
      std::vector<float4> rec(2 * nst);
      std::vector<uint16_t> ht(nst);
      for (size_t i = 0; i < nst; ++i) {
        rec[2 * i] = make_float4(h[i].x, h[i].y, h[i].z, qd[i].x);
        rec[2 * i + 1] = make_float4(l[i].x, l[i].y, l[i].z, qd[i].y);
        ht[i] = (uint16_t)(m[i].x | (sc[i] != 1.0 ? 0x8000 : 0));
      }
      GRX_CHECK_CUDA(cudaMemcpy(b->hrec + 2 * o, rec.data(), 2 * nst * sizeof(float4), cudaMemcpyHostToDevice),
                     "upload host records");
      GRX_CHECK_CUDA(cudaMemcpy(b->htype + o, ht.data(), nst * sizeof(uint16_t), cudaMemcpyHostToDevice),
                     "upload host types");
    }
  }
  GRX_CHECK_CUDA(cudaMemcpy(b->d_size, b->size, GRX_MAX_COMPONENTS * sizeof(int), cudaMemcpyHostToDevice),
                 "upload sizes");
  if (comp < b->nhost) {
    grx_status st = build_tiles(b);
    if (st) return st;
    st = build_voxels(b);
    if (st) return st;
  }
  b->sk_valid = false;
  return GRX_OK;
}

grx_status grx_box_get_component_size(grx_box* b, int32_t comp, size_t* size) {
  GRX_REQUIRE(b && size && comp >= 0 && comp < b->ncomp, "grx_box_get_component_size: bad argument");
  int v = 0;
  GRX_CHECK_CUDA(cudaMemcpy(&v, b->d_size + comp, sizeof(int), cudaMemcpyDeviceToHost), "read size");
  b->size[comp] = v;
  *size = (size_t)v;
  return GRX_OK;
}

grx_status grx_box_get_positions(grx_box* b, int32_t comp, double* out, size_t n) {
  GRX_REQUIRE(b && out && comp >= 0 && comp < b->ncomp, "grx_box_get_positions: bad argument");
  GRX_REQUIRE(n <= b->cap[comp], "grx_box_get_positions: n exceeds capacity");
  std::vector<double4> p(n);
  const double4* src = (comp < b->nhost && b->parent) ? b->parent->pos64 : b->pos64;
  if (n)
    GRX_CHECK_CUDA(cudaMemcpy(p.data(), src + b->off[comp], n * sizeof(double4), cudaMemcpyDeviceToHost),
                   "read positions");
  std::vector<double> flat(3 * n);
  const std::vector<int>& perm = b->perm[comp];
  for (size_t i = 0; i < n; ++i) {
    const size_t k = (i < perm.size()) ? (size_t)perm[i] : i;  // storage slot -> caller index
    if (k >= n) continue;
    flat[3 * k] = p[i].x; flat[3 * k + 1] = p[i].y; flat[3 * k + 2] = p[i].z;
  }
  if (n) GRX_CHECK_CUDA(cudaMemcpy(out, flat.data(), 3 * n * sizeof(double), cudaMemcpyDefault), "write positions");
  return GRX_OK;
}

grx_status grx_box_get_exclusion(grx_box* b, int32_t comp, double* intra, double* self) {
  GRX_REQUIRE(b && intra && self && comp >= 0 && comp < b->ncomp, "grx_box_get_exclusion: bad argument");
  *intra = b->excl_intra[comp];
  *self = b->excl_self[comp];
  return GRX_OK;
}

grx_status grx_ewald_sizes(grx_box* b, int64_t* nvec, int64_t* nactive) {
  GRX_REQUIRE(b && nvec && nactive, "grx_ewald_sizes: null argument");
  *nvec = b->nvec;
  *nactive = b->nact;
  return GRX_OK;
}

grx_status grx_ewald_set_structure_factors(grx_box* b, const double* s_fw, const double* s_ads) {
  GRX_REQUIRE(b && s_fw && s_ads, "grx_ewald_set_structure_factors: null argument");
  GRX_REQUIRE(!b->parent, "grx_ewald_set_structure_factors: a replica's framework structure factor is its parent's");
  GRX_CHECK_CUDA(cudaMemcpy(b->s_fw, s_fw, b->nvec * sizeof(double2), cudaMemcpyDefault), "set S_fw");
  GRX_CHECK_CUDA(cudaMemcpy(b->s_ads, s_ads, b->nvec * sizeof(double2), cudaMemcpyDefault), "set S_ads");
  GRX_CHECK_CUDA(cudaMemcpy(b->s_tmp, s_ads, b->nvec * sizeof(double2), cudaMemcpyDefault), "set S_tmp");
  b->sk_valid = true;
  b->ewdf_valid = false;
  return GRX_OK;
}

grx_status grx_ewald_get_structure_factors(grx_box* b, double* s_fw, double* s_ads, double* s_tmp) {
  GRX_REQUIRE(b, "grx_ewald_get_structure_factors: null box");
  GRX_CHECK_CUDA(cudaStreamSynchronize(b->stream), "sync");
  if (s_fw) GRX_CHECK_CUDA(cudaMemcpy(s_fw, b->s_fw, b->nvec * sizeof(double2), cudaMemcpyDefault), "get S_fw");
  if (s_ads) GRX_CHECK_CUDA(cudaMemcpy(s_ads, b->s_ads, b->nvec * sizeof(double2), cudaMemcpyDefault), "get S_ads");
  if (s_tmp) GRX_CHECK_CUDA(cudaMemcpy(s_tmp, b->s_tmp, b->nvec * sizeof(double2), cudaMemcpyDefault), "get S_tmp");
  return GRX_OK;
}

}  // extern "C"
