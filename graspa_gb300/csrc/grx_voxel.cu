// grx_voxel.cu -- candidate lists of framework (host) atoms per voxel of the cell.
//
// The cell is cut into nv[0] x nv[1] x nv[2] voxels, parallelepipeds in fractional
// coordinates with edges near g angstrom. A voxel's list holds every host atom whose
// nearest periodic image lies within r_list = (screening radius) + (voxel bounding
// radius) + margin of the voxel centre, with the lattice shift of that image. For any
// bead inside the voxel the list therefore holds every atom within the cutoff, at the
// image the bead sees it (the cell is wider than 2 r_list, so that image is unique).
// Atoms whose image lies within (screening radius - bounding radius) of the centre are
// inside the cutoff for every bead of the voxel: they come first in the list and go to
// the dense evaluation without the FP32 screen; the others are screened with the stored
// shift. A bead pass walks its voxel's list in 32-atom chunks instead of culling the
// box's 32-atom tiles; the dense evaluation still applies the exact cutoff tests, so the
// lists change which pairs are screened, never which pairs count.
//
// Entry: bits 0-19 the atom's storage index, bits 20-28 the shift (nx + 4) | (ny + 4) << 3
// | (nz + 4) << 6, n in [-4, 3], the image being r - nx a - ny b - nz c. Lists are built on
// the host (threads over voxels; tile spheres prune the atoms) when the host atoms change,
// and shared with the box's replicas.
#include <algorithm>
#include <cmath>
#include <thread>
#include <vector>

#include "grx_host.h"

namespace grx {

namespace {

struct Geo {
  double cell[9], inv[9], w[3];
};

// Fractional rounding of the reference's PBC (round half away from zero).
inline double rnd_away(double s) { return (double)(int)(s + (s >= 0.0 ? 0.5 : -0.5)); }

// Displacement d (in) to its rounded image (out), with the lattice integers n; returns
// a lower bound of the distance to the nearest image (exact when |d_out| <= w_min / 2).
inline double image(const Geo& G, double* d, int* n, double half_wmin) {
  double s[3];
  for (int k = 0; k < 3; ++k) s[k] = G.inv[k] * d[0] + G.inv[3 + k] * d[1] + G.inv[6 + k] * d[2];
  double r[3];
  for (int k = 0; k < 3; ++k) {
    const double m = rnd_away(s[k]);
    n[k] = (int)m;
    r[k] = s[k] - m;
  }
  for (int j = 0; j < 3; ++j) d[j] = G.cell[j] * r[0] + G.cell[3 + j] * r[1] + G.cell[6 + j] * r[2];
  const double len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  if (len <= half_wmin) return len;
  return std::max(std::fabs(r[0]) * G.w[0], std::max(std::fabs(r[1]) * G.w[1], std::fabs(r[2]) * G.w[2]));
}

constexpr double kMargin = 0.02;                  // A, on the voxel bounding radius
constexpr size_t kArenaHeadroom = 4u << 20;       // arena bytes left free for the box's other buffers

}  // namespace

// Voxel grid of a cell: the finest edge g in {1.5, 2, 2.5, 3, 4} A whose lists fit the byte
// cap max_bytes (estimated from the host-atom density) and leave the cell wider than 2 r_list. Returns
// false when none does (the tile path then serves the box).
static bool choose_voxels(const double* C, double volume, int nh_atoms, double r_screen, size_t max_bytes, Geo& G,
                          double& half_wmin, int nv[3], double& h, double& est_bytes) {
  const double av[3] = {C[0], C[1], C[2]}, bv[3] = {C[3], C[4], C[5]}, cv[3] = {C[6], C[7], C[8]};
  auto cross_norm = [](const double* u, const double* v) {
    const double x = u[1] * v[2] - u[2] * v[1], y = u[2] * v[0] - u[0] * v[2], z = u[0] * v[1] - u[1] * v[0];
    return std::sqrt(x * x + y * y + z * z);
  };
  const double V = std::fabs(volume);
  G.w[0] = V / cross_norm(bv, cv);
  G.w[1] = V / cross_norm(cv, av);
  G.w[2] = V / cross_norm(av, bv);
  half_wmin = 0.5 * std::min(G.w[0], std::min(G.w[1], G.w[2]));
  const double len[3] = {std::sqrt(av[0] * av[0] + av[1] * av[1] + av[2] * av[2]),
                         std::sqrt(bv[0] * bv[0] + bv[1] * bv[1] + bv[2] * bv[2]),
                         std::sqrt(cv[0] * cv[0] + cv[1] * cv[1] + cv[2] * cv[2])};
  const double dens = (double)nh_atoms / V;
  for (double g : {1.5, 2.0, 2.5, 3.0, 4.0}) {
    int n[3];
    for (int k = 0; k < 3; ++k) n[k] = std::max(1, (int)std::ceil(len[k] / g));
    double hm = 0.0;  // half the longest body diagonal of a voxel
    for (int sy = -1; sy <= 1; sy += 2)
      for (int sz = -1; sz <= 1; sz += 2) {
        double x[3];
        for (int j = 0; j < 3; ++j) x[j] = av[j] / n[0] + sy * bv[j] / n[1] + sz * cv[j] / n[2];
        hm = std::max(hm, 0.5 * std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]));
      }
    hm += kMargin;
    if (r_screen + hm + kMargin >= half_wmin) return false;  // coarser voxels only make the bound worse
    const double rl = r_screen + hm;
    const double est = (double)n[0] * n[1] * n[2] * (dens * 4.18879 * rl * rl * rl * 1.25 + 32.0) * 4.0 +
                       (double)n[0] * n[1] * n[2] * 16.0;
    if (est <= (double)max_bytes) {
      for (int k = 0; k < 3; ++k) nv[k] = n[k];
      h = hm;
      est_bytes = est;
      return true;
    }
  }
  return false;
}

grx_status build_voxels(grx_box* b) {
  dev_free(b, b->vmeta);
  dev_free(b, b->vlist);
  b->vmeta = nullptr;
  b->vlist = nullptr;
  b->vox_on = 0;
  b->vchunks = 0;
  b->vox_entries = 0;
  const int nh_atoms = (int)b->off[b->nhost];
  if (b->vox_mode == 0 || b->nhost == 0 || nh_atoms == 0 || b->ntiles == 0 || nh_atoms >= (1 << 20)) {
    refresh_dev(b);
    return GRX_OK;
  }
  const BoxDev& d = b->dev;
  Geo G;
  for (int k = 0; k < 9; ++k) {
    G.cell[k] = d.cell[k];
    G.inv[k] = d.inv[k];
  }
  const double* C = d.cell;
  const double av[3] = {C[0], C[1], C[2]}, bv[3] = {C[3], C[4], C[5]}, cv[3] = {C[6], C[7], C[8]};
  const double r_screen = std::sqrt((double)d.screen2);
  int nv[3] = {0, 0, 0};
  double h = 0.0, half_wmin = 0.0, est = 0.0;
  if (!choose_voxels(C, d.volume, nh_atoms, r_screen, b->vox_max_bytes, G, half_wmin, nv, h, est)) {
    refresh_dev(b);
    return GRX_OK;
  }
  const double r_list = r_screen + h;
  const double r_sure = r_screen - 2e-3 - h;  // inside the largest cutoff for every bead of the voxel
  const int nvox = nv[0] * nv[1] * nv[2];
  std::vector<std::vector<uint32_t>> lists(nvox);
  std::vector<int> nsure(nvox, 0);
  const int ntile = b->ntiles;
  auto work = [&](int v0, int v1) {
    std::vector<std::pair<int, uint32_t>> sure, maybe;
    for (int v = v0; v < v1; ++v) {
      const int ix = v % nv[0], iy = (v / nv[0]) % nv[1], iz = v / (nv[0] * nv[1]);
      const double f[3] = {(ix + 0.5) / nv[0], (iy + 0.5) / nv[1], (iz + 0.5) / nv[2]};
      double c[3];
      for (int j = 0; j < 3; ++j) c[j] = av[j] * f[0] + bv[j] * f[1] + cv[j] * f[2];
      sure.clear();
      maybe.clear();
      for (int t = 0; t < ntile; ++t) {
        const float4 tc = b->h_tile_c[2 * t];
        const int4 tr = b->h_tile_r[t];
        double dv[3] = {tc.x - c[0], tc.y - c[1], tc.z - c[2]};
        int n[3];
        if (image(G, dv, n, half_wmin) - tc.w > r_list) continue;
        for (int i = tr.x; i < tr.y; ++i) {
          double da[3] = {b->h_pos[3 * i] - c[0], b->h_pos[3 * i + 1] - c[1], b->h_pos[3 * i + 2] - c[2]};
          int m[3];
          image(G, da, m, half_wmin);
          // the rounded image is the nearest one for any image within r_list < w_min / 2
          const double r = std::sqrt(da[0] * da[0] + da[1] * da[1] + da[2] * da[2]);
          if (r > r_list) continue;
          bool ok = true;
          for (int k = 0; k < 3; ++k) ok = ok && m[k] >= -4 && m[k] <= 3;
          if (!ok) continue;  // never taken: host atoms were checked to lie near the home cell
          const uint32_t e = (uint32_t)i | ((uint32_t)(m[0] + 4) << 20) | ((uint32_t)(m[1] + 4) << 23) |
                             ((uint32_t)(m[2] + 4) << 26);
          if (r <= r_sure) sure.push_back({i, e});
          else maybe.push_back({i, e});
        }
      }
      std::sort(sure.begin(), sure.end());
      std::sort(maybe.begin(), maybe.end());
      std::vector<uint32_t>& out = lists[v];
      out.reserve(sure.size() + maybe.size());
      for (const auto& p : sure) out.push_back(p.second);
      for (const auto& p : maybe) out.push_back(p.second);
      nsure[v] = (int)sure.size();
    }
  };
  // host atoms must lie within four cells of the home cell for the 3-bit shifts
  for (int i = 0; i < nh_atoms; ++i) {
    double s[3];
    for (int k = 0; k < 3; ++k)
      s[k] = G.inv[k] * b->h_pos[3 * i] + G.inv[3 + k] * b->h_pos[3 * i + 1] + G.inv[6 + k] * b->h_pos[3 * i + 2];
    for (int k = 0; k < 3; ++k)
      if (s[k] < -2.5 || s[k] > 2.5) {
        refresh_dev(b);
        return GRX_OK;
      }
  }
  const int nthr = std::max(1, std::min<int>(16, (int)std::thread::hardware_concurrency()));
  {
    std::vector<std::thread> th;
    const int per = (nvox + nthr - 1) / nthr;
    for (int k = 0; k < nthr; ++k) {
      const int v0 = k * per, v1 = std::min(nvox, v0 + per);
      if (v0 < v1) th.emplace_back(work, v0, v1);
    }
    for (auto& t : th) t.join();
  }
  std::vector<int4> meta(nvox);
  size_t total = 0;
  int maxn = 0;
  for (int v = 0; v < nvox; ++v) {
    meta[v] = make_int4((int)total, nsure[v], (int)lists[v].size(), 0);
    total += lists[v].size();
    maxn = std::max(maxn, (int)lists[v].size());
  }
  std::vector<uint32_t> flat;
  flat.reserve(total);
  for (const auto& l : lists) flat.insert(flat.end(), l.begin(), l.end());
  // 8 zero entries of padding: the pass stages list ranges with bulk copies rounded out to
  // 16-byte boundaries, which may read up to 3 entries past the last list
  flat.insert(flat.end(), 8, 0u);
  if (b->arena) {  // in an arena the lists are optional: take them only with room to spare
    size_t used = 0, largest = 0;
    grx_arena_usage(b->arena, &used, &largest, nullptr);
    if (largest < nvox * sizeof(int4) + flat.size() * sizeof(uint32_t) + kArenaHeadroom) {
      refresh_dev(b);
      return GRX_OK;
    }
  }
  if (dev_alloc(b, (void**)&b->vmeta, nvox * sizeof(int4)) != cudaSuccess ||
      dev_alloc(b, (void**)&b->vlist, flat.size() * sizeof(uint32_t)) != cudaSuccess) {
    cudaGetLastError();  // no room: the tile path serves the box
    dev_free(b, b->vmeta);
    dev_free(b, b->vlist);
    b->vmeta = nullptr;
    b->vlist = nullptr;
    refresh_dev(b);
    return GRX_OK;
  }
  GRX_CHECK_CUDA(cudaMemcpy(b->vmeta, meta.data(), nvox * sizeof(int4), cudaMemcpyHostToDevice), "upload voxels");
  GRX_CHECK_CUDA(cudaMemcpy(b->vlist, flat.data(), flat.size() * sizeof(uint32_t), cudaMemcpyHostToDevice),
                 "upload voxel lists");
  for (int k = 0; k < 3; ++k) b->vn[k] = nv[k];
  b->vchunks = (maxn + 31) / 32;
  b->vox_on = 1;
  b->vox_entries = total;
  refresh_dev(b);
  return GRX_OK;
}

}  // namespace grx

using namespace grx;

extern "C" grx_status grx_box_set_voxel_lists(grx_box* b, int32_t mode) {
  GRX_REQUIRE(b, "grx_box_set_voxel_lists: null box");
  GRX_REQUIRE(mode == 0 || mode == 1, "grx_box_set_voxel_lists: mode must be 0 or 1");
  GRX_REQUIRE(!b->parent && b->replicas == 0,
              "grx_box_set_voxel_lists: the lists are shared with replicas (set them on a box without any)");
  GRX_CHECK_CUDA(cudaStreamSynchronize(b->stream), "grx_box_set_voxel_lists");
  b->vox_mode = mode;
  return build_voxels(b);
}

extern "C" grx_status grx_box_get_voxel_lists(grx_box* b, int32_t* on, int32_t* dims, int64_t* entries) {
  GRX_REQUIRE(b && on, "grx_box_get_voxel_lists: null argument");
  const grx_box* h = b->parent ? b->parent : b;
  *on = h->vox_on;
  if (dims)
    for (int k = 0; k < 3; ++k) dims[k] = h->vox_on ? h->vn[k] : 0;
  if (entries) *entries = h->vox_on ? (int64_t)h->vox_entries : 0;
  return GRX_OK;
}
