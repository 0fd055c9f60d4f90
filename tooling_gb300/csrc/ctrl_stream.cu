// Control streams for served rollouts: each world's whole control sequence
// (horizon x nv generalised forces, newt's `Tree::qfrc_applied`,
// newt/src/tree.rs:207) is uploaded once into a device arena; every
// newt_gpu_apply_ctrl call then writes the next row of every stream into its
// world's qfrc row on the device and advances the stream's cursor, so a
// serving tick moves no control data across the host link.
#include <algorithm>

#include "runtime.h"

#define CKC(call)                                                               \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) { ctx->err = std::string(#call ": ") + cudaGetErrorString(e_); return NEWT_E_CUDA; } \
  } while (0)

namespace {

struct CtrlDev {
  float* qfrc;  // the world's first qfrc entry (rows are `cap` floats apart)
  int cap, nv, h, t;
  size_t off;   // the stream's first value in the arena
};

__global__ void ctrl_apply(CtrlDev* __restrict__ e, int n, const float* __restrict__ arena, int max_nv) {
  const long total = (long)n * max_nv;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int j = (int)(i / max_nv), k = (int)(i % max_nv);
    CtrlDev& d = e[j];
    if (k >= d.nv || d.t >= d.h) continue;
    d.qfrc[(size_t)k * d.cap] = arena[d.off + (size_t)d.t * d.nv + k];
  }
}

__global__ void ctrl_advance(CtrlDev* __restrict__ e, int n) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) ++e[j].t;
}

// First fit in the free list; the arena grows (keeping offsets) when nothing fits.
int arena_alloc(newt_gpu_ctx* ctx, size_t n, size_t* off) {
  auto& fl = ctx->ctrl_free;
  for (size_t i = 0; i < fl.size(); ++i)
    if (fl[i].second >= n) {
      *off = fl[i].first;
      fl[i].first += n;
      fl[i].second -= n;
      if (fl[i].second == 0) fl.erase(fl.begin() + (long)i);
      return NEWT_OK;
    }
  const size_t old = ctx->ctrl_cap;
  const size_t cap = std::max(old * 2, old + std::max(n, (size_t)1 << 20));
  float* a = nullptr;
  CKC(cudaMalloc(&a, cap * sizeof(float)));
  if (ctx->ctrl_arena) {
    CKC(cudaMemcpyAsync(a, ctx->ctrl_arena, old * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
    CKC(cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->ctrl_arena);
  }
  ctx->ctrl_arena = a;
  ctx->ctrl_cap = cap;
  // the new tail joins the free list (merged with a free block ending at `old`)
  if (!fl.empty() && fl.back().first + fl.back().second == old) fl.back().second += cap - old;
  else fl.push_back({old, cap - old});
  return arena_alloc(ctx, n, off);
}

void arena_free(newt_gpu_ctx* ctx, size_t off, size_t n) {
  auto& fl = ctx->ctrl_free;
  auto it = std::lower_bound(fl.begin(), fl.end(), std::make_pair(off, (size_t)0));
  it = fl.insert(it, {off, n});
  // merge with the neighbours
  if (it + 1 != fl.end() && it->first + it->second == (it + 1)->first) {
    it->second += (it + 1)->second;
    fl.erase(it + 1);
  }
  if (it != fl.begin() && (it - 1)->first + (it - 1)->second == it->first) {
    (it - 1)->second += it->second;
    fl.erase(it);
  }
}

}  // namespace

void ctrl_release_slot(newt_gpu_ctx* ctx, int slot) {
  if (slot < 0 || slot >= (int)ctx->ctrl_of_slot.size() || ctx->ctrl_of_slot[slot] < 0) return;
  const int j = ctx->ctrl_of_slot[slot];
  auto& e = ctx->ctrl[j];
  arena_free(ctx, e.off, (size_t)e.h * e.nv);
  ctx->ctrl_of_slot[slot] = -1;
  if (j != (int)ctx->ctrl.size() - 1) {
    ctx->ctrl[j] = ctx->ctrl.back();
    ctx->ctrl_of_slot[ctx->ctrl[j].slot] = j;
  }
  ctx->ctrl.pop_back();
  ctx->ctrl_dirty = true;
}

extern "C" {

int newt_gpu_set_ctrl_stream(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n, const float* ctrl,
                             const int32_t* horizons) {
  if (!ctx || n < 0 || (n > 0 && (!slots || !horizons))) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  size_t total = 0;
  for (int i = 0; i < n; ++i) {
    const int s = slots[i];
    if (s < 0 || s >= (int)ctx->slots.size() || !ctx->slots[s].live || horizons[i] < 0) {
      ctx->err = "bad slot or horizon";
      return NEWT_E_INVALID;
    }
    total += (size_t)horizons[i] * ctx->models[ctx->slots[s].model].nv;
  }
  if (total > 0 && !ctrl) return NEWT_E_INVALID;
  if (ctx->ctrl_of_slot.size() < ctx->slots.size()) ctx->ctrl_of_slot.resize(ctx->slots.size(), -1);
  // the trees' sequences (piles carry no generalised forces) packed into one
  // block of the arena with one copy; each stream frees its own part later
  std::vector<float> packed;
  std::vector<std::pair<int, size_t>> parts;  // (call index, offset in the block)
  size_t src = 0;
  for (int i = 0; i < n; ++i) {
    const SlotRef& r = ctx->slots[slots[i]];
    const size_t cnt = (size_t)horizons[i] * ctx->models[r.model].nv;
    ctrl_release_slot(ctx, slots[i]);
    if (ctx->groups[r.group]->soa() && cnt > 0) {
      parts.push_back({i, packed.size()});
      packed.insert(packed.end(), ctrl + src, ctrl + src + cnt);
    }
    src += cnt;
  }
  if (parts.empty()) return NEWT_OK;
  size_t base = 0;
  int rc = arena_alloc(ctx, packed.size(), &base);
  if (rc != NEWT_OK) return rc;
  CKC(cudaMemcpyAsync(ctx->ctrl_arena + base, packed.data(), packed.size() * sizeof(float), cudaMemcpyHostToDevice,
                      ctx->stream));
  for (const auto& p : parts) {
    const int s = slots[p.first];
    ctx->ctrl_of_slot[s] = (int)ctx->ctrl.size();
    ctx->ctrl.push_back({s, ctx->models[ctx->slots[s].model].nv, horizons[p.first], 0, base + p.second});
  }
  ctx->ctrl_dirty = true;
  CKC(cudaStreamSynchronize(ctx->stream));  // `packed` is pageable and local
  return NEWT_OK;
}

int newt_gpu_apply_ctrl(newt_gpu_ctx* ctx) {
  if (!ctx) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  const int n = (int)ctx->ctrl.size();
  if (n == 0) return NEWT_OK;
  int max_nv = 1;
  for (const auto& e : ctx->ctrl) max_nv = std::max(max_nv, e.nv);
  if (ctx->ctrl_dirty) {
    // entries hold device row pointers: rebuilt after streams change or a group moves
    std::vector<CtrlDev> h(n);
    for (int j = 0; j < n; ++j) {
      const auto& e = ctx->ctrl[j];
      const SlotRef& r = ctx->slots[e.slot];
      const HostGroup* g = ctx->groups[r.group].get();
      h[j] = CtrlDev{g->dF + (size_t)g->r_qfrc * g->cap + r.index, g->cap, e.nv, e.h, e.t, e.off};
    }
    if (ctx->ctrl_dev_cap < (size_t)n) {
      if (ctx->ctrl_dev) cudaFree(ctx->ctrl_dev);
      ctx->ctrl_dev = nullptr;
      ctx->ctrl_dev_cap = std::max((size_t)n, 2 * ctx->ctrl_dev_cap);
      CKC(cudaMalloc(&ctx->ctrl_dev, ctx->ctrl_dev_cap * sizeof(CtrlDev)));
    }
    CKC(cudaMemcpyAsync(ctx->ctrl_dev, h.data(), (size_t)n * sizeof(CtrlDev), cudaMemcpyHostToDevice, ctx->stream));
    CKC(cudaStreamSynchronize(ctx->stream));  // `h` is pageable and local
    ctx->ctrl_dirty = false;
  }
  const long total = (long)n * max_nv;
  const int grid = (int)std::max<long>(1, std::min<long>((total + 255) / 256, 152L * 16));
  ctrl_apply<<<grid, 256, 0, ctx->stream>>>((CtrlDev*)ctx->ctrl_dev, n, ctx->ctrl_arena, max_nv);
  ctrl_advance<<<(n + 255) / 256, 256, 0, ctx->stream>>>((CtrlDev*)ctx->ctrl_dev, n);
  ctx->launches += 2;
  for (auto& e : ctx->ctrl) ++e.t;  // the host mirror of the cursors
  CKC(cudaGetLastError());
  return NEWT_OK;
}

}  // extern "C"
