// grx_arena.cu -- a device-memory arena: one cudaMalloc'd region of HBM carved
// into the allocations of many boxes by a host-side first-fit allocator.
//
// A serving process admits jobs by HBM footprint: each admitted box is created in
// the arena, and a box that does not fit waits. Returning a retired box's memory to
// the arena costs no cudaFree, which would wait for every stream of the device.
#include <map>
#include <mutex>
#include <unordered_map>

#include "grx_host.h"

struct grx_arena {
  int device = 0;
  char* base = nullptr;
  size_t size = 0;
  std::mutex m;
  std::map<size_t, size_t> free_;             // offset -> length, coalesced
  std::unordered_map<size_t, size_t> used_;   // offset -> length
  size_t in_use = 0;
  size_t peak = 0;
};

namespace grx {

static constexpr size_t kArenaAlign = 256;

void* arena_alloc(grx_arena* a, size_t bytes) {
  const size_t need = (std::max<size_t>(bytes, 1) + kArenaAlign - 1) / kArenaAlign * kArenaAlign;
  std::lock_guard<std::mutex> g(a->m);
  for (auto it = a->free_.begin(); it != a->free_.end(); ++it) {
    if (it->second < need) continue;
    const size_t off = it->first, len = it->second;
    a->free_.erase(it);
    if (len > need) a->free_[off + need] = len - need;
    a->used_[off] = need;
    a->in_use += need;
    a->peak = std::max(a->peak, a->in_use);
    return a->base + off;
  }
  return nullptr;
}

void arena_free(grx_arena* a, void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> g(a->m);
  const size_t off = (size_t)((char*)p - a->base);
  auto u = a->used_.find(off);
  if (u == a->used_.end()) return;
  size_t start = off, len = u->second;
  a->in_use -= len;
  a->used_.erase(u);
  auto next = a->free_.lower_bound(start);
  if (next != a->free_.end() && next->first == start + len) {
    len += next->second;
    next = a->free_.erase(next);
  }
  if (next != a->free_.begin()) {
    auto prev = std::prev(next);
    if (prev->first + prev->second == start) {
      start = prev->first;
      len += prev->second;
      a->free_.erase(prev);
    }
  }
  a->free_[start] = len;
}

}  // namespace grx

using namespace grx;

extern "C" grx_status grx_arena_create(size_t bytes, grx_arena** out) {
  GRX_REQUIRE(out && bytes > 0, "grx_arena_create: bad argument");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    set_error("grx_arena_create: no CUDA device");
    return GRX_ERR_NO_DEVICE;
  }
  auto* a = new grx_arena();
  cudaGetDevice(&a->device);
  a->size = (bytes + kArenaAlign - 1) / kArenaAlign * kArenaAlign;
  if (cudaMalloc((void**)&a->base, a->size) != cudaSuccess) {
    cudaGetLastError();
    delete a;
    set_error("grx_arena_create: cannot reserve %zu bytes of device memory", bytes);
    return GRX_ERR_OUT_OF_MEMORY;
  }
  a->free_[0] = a->size;
  *out = a;
  return GRX_OK;
}

extern "C" grx_status grx_arena_destroy(grx_arena* a) {
  if (!a) return GRX_OK;
  GRX_REQUIRE(a->used_.empty(), "grx_arena_destroy: boxes still live in the arena");
  cudaFree(a->base);
  delete a;
  return GRX_OK;
}

extern "C" grx_status grx_arena_usage(grx_arena* a, size_t* in_use, size_t* largest_free, size_t* peak) {
  GRX_REQUIRE(a, "grx_arena_usage: null arena");
  std::lock_guard<std::mutex> g(a->m);
  size_t lf = 0;
  for (const auto& f : a->free_) lf = std::max(lf, f.second);
  if (in_use) *in_use = a->in_use;
  if (largest_free) *largest_free = lf;
  if (peak) *peak = a->peak;
  return GRX_OK;
}
