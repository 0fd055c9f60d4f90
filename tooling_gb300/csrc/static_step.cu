// Allocation-free step: newt_gpu_step_static.
//
// Some callers cannot let the step allocate device memory: a control or
// serving loop that has handed the rest of the device to another framework's
// caching pool (a cudaMalloc there fails or evicts that pool), and any loop
// that must not stall, since cudaFree waits for the whole device and a first
// step after a world change would otherwise build its tables and solver
// scratch with cudaMalloc.  This entry point runs the same kernels as the
// plain step, but the pile solver's scratch, its island work lists and its
// group tables live in one file-scope device array of fixed size
// (NEWT_STATIC_SCRATCH_BYTES); nothing is allocated per call.
//
// Setup: the first call on a device, with that device current, loads the
// pile and tree kernels and this module.  Every call then looks the array's
// address up with cudaGetSymbolAddress (a host-side lookup once the module is
// loaded, so a cudaDeviceReset between calls leaves nothing stale).  Make the
// first call on a device before any stream capture on it.
//
// Tables: the pile group table and segment table reach the device as a
// by-value kernel argument written into the array by a one-block kernel on
// the context's stream, so a call issues no host-to-device copy: it does not
// wait for the stream's earlier work, and no host buffer has to outlive it.
//
// Sharing: there is one array per device.  Two calls whose GPU work can
// overlap (two contexts on one device, or two threads) race on it; the
// caller orders them (one context, or newt_gpu_sync between contexts).
//
// What must start at zero: only the island-class counters at the end of the
// work lists, which every env-step clears on the stream before its collide
// stage.  Every other scratch word is written by the step before it is read.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "runtime.h"

extern "C" size_t newt_pile_ws_bytes(int nb, int np, int maxc);
extern "C" size_t newt_pile_list_bytes(int slots);
extern "C" cudaError_t newt_pile_prepare_kernels();
extern "C" cudaError_t newt_tree_prepare_kernels();
extern "C" int newt_launch_pile_step_serial(const PileGroupDev* dG, const int* dwseg, int ng, int total_worlds,
                                            int total_slots, int* lists, int write_diag, cudaStream_t st);

namespace {

constexpr size_t kAlign = 256;
constexpr int kMaxPileGroups = 64;  // pile groups one call can step
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[NEWT_STATIC_SCRATCH_BYTES];

std::mutex g_setup_mu;
bool g_prepared[kMaxDevices] = {};

// The pile tables of one call, passed by value (about 10 KB of kernel
// parameters; sm_90 and later take up to 32 KB).
struct StaticTables {
  PileGroupDev g[kMaxPileGroups];
  int seg[kMaxPileGroups + 1];
  int ng;
};

static_assert(sizeof(StaticTables) <= 32000, "kernel parameters are limited to 32 KB");

__global__ void static_write_tables(const StaticTables t, PileGroupDev* dG, int* dseg) {
  for (int i = threadIdx.x; i < t.ng; i += blockDim.x) dG[i] = t.g[i];
  for (int i = threadIdx.x; i <= t.ng; i += blockDim.x) dseg[i] = t.seg[i];
}

size_t round_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

int fail(newt_gpu_ctx* ctx, int code, const std::string& msg) {
  ctx->err = "newt_gpu_step_static: " + msg;
  return code;
}

// Address of this device's scratch array (the device is current); the first
// call per device loads the kernels.
int scratch_for_device(newt_gpu_ctx* ctx, unsigned char** out) {
  if (ctx->device < 0 || ctx->device >= kMaxDevices) return fail(ctx, NEWT_E_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_prepared[ctx->device]) {
    cudaError_t e = newt_pile_prepare_kernels();
    if (e == cudaSuccess) e = newt_tree_prepare_kernels();
    if (e == cudaSuccess) {
      cudaFuncAttributes a;
      e = cudaFuncGetAttributes(&a, static_write_tables);
    }
    if (e != cudaSuccess) return fail(ctx, NEWT_E_CUDA, std::string("loading step kernels: ") + cudaGetErrorString(e));
    g_prepared[ctx->device] = true;
  }
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
  if (e != cudaSuccess) return fail(ctx, NEWT_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  *out = static_cast<unsigned char*>(p);
  return NEWT_OK;
}

}  // namespace

extern "C" NEWT_API int newt_gpu_step_static(newt_gpu_ctx* ctx, int32_t n_steps) {
  if (!ctx || n_steps < 0) return NEWT_E_INVALID;
  if (n_steps == 0) return NEWT_OK;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return fail(ctx, NEWT_E_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));

  // Lay out the pile table, segment table, work lists and per-world solver
  // scratch inside the array, and refuse before any launch if they do not fit.
  StaticTables tab;
  PileGroupDev* table = tab.g;
  int* seg = tab.seg;
  size_t scr_off[kMaxPileGroups];
  int ng = 0, slots = 0;
  seg[0] = 0;
  for (auto& gp : ctx->groups) {
    const HostGroup* g = gp.get();
    if (g->n == 0) continue;
    if (g->kind == GK_TREE_CONTACT) return fail(ctx, NEWT_E_INVALID, "tree-contact worlds are not supported");
    if (g->kind != GK_PILE) continue;
    if (g->pile_newton) return fail(ctx, NEWT_E_INVALID, "pile worlds under the Newton solver are not supported");
    if (g->pile_general)
      return fail(ctx, NEWT_E_INVALID, "pile worlds with the elliptic cone or condim 1, 4, 6 are not supported");
    if (ng == kMaxPileGroups) return fail(ctx, NEWT_E_INVALID, "more than 64 pile groups (distinct body counts)");
    table[ng] = g->pile_dev();
    seg[ng + 1] = seg[ng] + g->n;
    slots += g->n * g->size;
    ++ng;
  }
  size_t off = round_up(sizeof(PileGroupDev) * (size_t)ng);
  const size_t seg_off = off;
  off += round_up(sizeof(int) * (size_t)(ng + 1));
  const size_t list_off = off;
  off += round_up(newt_pile_list_bytes(slots));
  for (int k = 0; k < ng; ++k) {
    const size_t per = newt_pile_ws_bytes(table[k].nb, table[k].np, table[k].maxc);
    scr_off[k] = off;
    table[k].sstride = (long)(per / sizeof(float));
    off += round_up(per * (size_t)table[k].n);
  }
  if (ng > 0 && off > (size_t)NEWT_STATIC_SCRATCH_BYTES)
    return fail(ctx, NEWT_E_NOMEM,
                "pile worlds need " + std::to_string(off) + " bytes of scratch; the static scratch holds " +
                    std::to_string((size_t)NEWT_STATIC_SCRATCH_BYTES) +
                    " bytes (NEWT_STATIC_SCRATCH_BYTES): step fewer pile worlds per call or use newt_gpu_step");

  unsigned char* base = nullptr;
  int rc = scratch_for_device(ctx, &base);
  if (rc != NEWT_OK) return rc;
  PileGroupDev* dG = reinterpret_cast<PileGroupDev*>(base);
  int* dseg = reinterpret_cast<int*>(base + seg_off);
  int* lists = reinterpret_cast<int*>(base + list_off);
  if (ng > 0) {
    for (int k = 0; k < ng; ++k) table[k].scr = reinterpret_cast<float*>(base + scr_off[k]);
    tab.ng = ng;
    static_write_tables<<<1, 64, 0, ctx->stream>>>(tab, dG, dseg);
    ctx->launches += 1;
  }
  // the profiling surface reads this call's island counters from the array
  ctx->last_lists.clear();
  if (ng > 0) ctx->last_lists.push_back({lists, slots});
  ctx->kev_steps = 0;
  ctx->last_fused = false;

  for (int s = 0; s < n_steps; ++s) {
    for (auto& gp : ctx->groups) {
      HostGroup* g = gp.get();
      if (g->n > 0 && g->kind == GK_TREE) {
        newt_launch_tree_plain(g->tree_dev(), ctx->stream);
        ctx->launches += 2;
      }
    }
    if (ng > 0)
      ctx->launches += newt_launch_pile_step_serial(dG, dseg, ng, seg[ng], slots, lists, s == n_steps - 1, ctx->stream);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(ctx, NEWT_E_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return NEWT_OK;
}
