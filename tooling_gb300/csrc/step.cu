// Step dispatch: the plain form (one launch per stage per step, fixed tiles,
// every group launched separately) and the batched form (one fused launch per
// kernel family over the whole horizon, work items pulled by persistent
// blocks from a device queue sorted by size class, captured once in a CUDA
// graph and replayed).
#include <algorithm>
#include <cstdio>
#include <vector>

#include "runtime.h"

#define CKS(call)                                                               \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) { ctx->err = std::string(#call ": ") + cudaGetErrorString(e_); return NEWT_E_CUDA; } \
  } while (0)

extern "C" void newt_launch_tree_persistent(const TreeGroupDev* dgroups, const int* dqueue, int* dcounter, int n_items,
                                            int bucket, int n_steps, int grid, cudaStream_t st);
extern "C" void newt_launch_pile_persistent(const PileGroupDev* dgroups, const int* dqueue, int* dcounter, int n_items,
                                            int n_steps, int grid, size_t smem, cudaStream_t st);
extern "C" int newt_tree_persistent_blocks_per_sm(int bucket);
extern "C" int newt_pile_blocks_per_sm(size_t smem);
extern "C" size_t newt_pile_ws_bytes(int nb, int np, int maxc);

static int sm_count(newt_gpu_ctx* ctx) {
  static int n = 0;
  if (n == 0) { cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, ctx->device); if (n <= 0) n = 1; }
  return n;
}
extern "C" int newt_tc_step(newt_gpu_ctx* ctx, HostGroup* g, int n_steps, int fused);

static void mark_stepped(newt_gpu_ctx* ctx) {
  for (auto& g : ctx->groups) if (g->n > 0) g->device_newer = true;
}

int step_plain(newt_gpu_ctx* ctx, int n_steps) {
  for (auto& gp : ctx->groups) {
    HostGroup* g = gp.get();
    if (g->n == 0 || g->kind != GK_PILE) continue;
    size_t need = newt_pile_plain_scratch_bytes(g->pile_dev());
    if (g->plain_scratch_bytes < need) {
      if (g->plain_scratch) cudaFree(g->plain_scratch);
      g->plain_scratch = nullptr;
      CKS(cudaMalloc(&g->plain_scratch, need));
      g->plain_scratch_bytes = need;
    }
  }
  for (int s = 0; s < n_steps; ++s) {
    for (auto& gp : ctx->groups) {
      HostGroup* g = gp.get();
      if (g->n == 0) continue;
      if (g->kind == GK_TREE) {
        newt_launch_tree_plain(g->tree_dev(), ctx->stream);
        ctx->launches += 2;
      } else if (g->kind == GK_PILE) {
        int nl = 0;
        newt_launch_pile_plain(g->pile_dev(), g->plain_scratch, ctx->stream, &nl);
        ctx->launches += nl;
      } else if (g->kind == GK_TREE_CONTACT) {
        int rc = newt_tc_step(ctx, g, 1, 0);
        if (rc != NEWT_OK) return rc;
      }
    }
  }
  mark_stepped(ctx);
  return NEWT_OK;
}

// ---------------------------------------------------------------------------
// batched: persistent kernels over a size-class-sorted device queue
// ---------------------------------------------------------------------------
struct QueueBuild {
  std::vector<int> items;  // (group slot in dev array, base, count) triples, cost-sorted
  std::vector<TreeGroupDev> tg;
  std::vector<PileGroupDev> pg;
  size_t smem = 0;  // pile scratch record bytes (largest group)
};

static int build_queue(newt_gpu_ctx* ctx, int bucket_or_pile, QueueBuild& qb) {
  // Items are chunks of worlds; bigger worlds come first so the tail of the
  // persistent grid is made of cheap items (longest-processing-time order).
  struct It { long cost; int g, base, count; };
  std::vector<It> its;
  for (auto& gp : ctx->groups) {
    HostGroup* g = gp.get();
    if (g->n == 0) continue;
    if (bucket_or_pile < 0) {
      if (g->kind != GK_PILE) continue;
      int gi = (int)qb.pg.size();
      qb.pg.push_back(g->pile_dev());
      qb.smem = std::max(qb.smem, newt_pile_ws_bytes(g->size, g->np, g->maxc));
      const int chunk = 2;  // worlds per item (one warp each)
      for (int b = 0; b < g->n; b += chunk)
        its.push_back({(long)g->size * g->size, gi, b, std::min(chunk, g->n - b)});
    } else {
      if (g->kind != GK_TREE || newt_tree_bucket(g->size) != bucket_or_pile) continue;
      int gi = (int)qb.tg.size();
      qb.tg.push_back(g->tree_dev());
      const int chunk = 64;  // worlds per item (one thread each)
      for (int b = 0; b < g->n; b += chunk) its.push_back({(long)g->size, gi, b, std::min(chunk, g->n - b)});
    }
  }
  std::stable_sort(its.begin(), its.end(), [](const It& a, const It& b) { return a.cost > b.cost; });
  for (auto& i : its) { qb.items.push_back(i.g); qb.items.push_back(i.base); qb.items.push_back(i.count); }
  return (int)its.size();
}

static int capture(newt_gpu_ctx* ctx, int n_steps) {
  std::vector<void*> bufs;
  struct Launch { int kind; int bucket; void* dg; int* dq; int* dc; int items; size_t smem; };
  std::vector<Launch> launches;
  const int buckets[4] = {8, 16, 32, 65};
  for (int bi = -1; bi < 4; ++bi) {
    QueueBuild qb;
    int nitems = build_queue(ctx, bi < 0 ? -1 : buckets[bi], qb);
    if (nitems == 0) continue;
    void* dg = nullptr;
    size_t gbytes = bi < 0 ? qb.pg.size() * sizeof(PileGroupDev) : qb.tg.size() * sizeof(TreeGroupDev);
    CKS(cudaMalloc(&dg, gbytes));
    CKS(cudaMemcpy(dg, bi < 0 ? (void*)qb.pg.data() : (void*)qb.tg.data(), gbytes, cudaMemcpyHostToDevice));
    int* dq = nullptr;
    CKS(cudaMalloc(&dq, qb.items.size() * sizeof(int)));
    CKS(cudaMemcpy(dq, qb.items.data(), qb.items.size() * sizeof(int), cudaMemcpyHostToDevice));
    int* dc = nullptr;
    CKS(cudaMalloc(&dc, sizeof(int)));
    bufs.push_back(dg); bufs.push_back(dq); bufs.push_back(dc);
    launches.push_back({bi < 0 ? GK_PILE : GK_TREE, bi < 0 ? -1 : buckets[bi], dg, dq, dc, nitems, qb.smem});
  }
  // occupancy queries and function attributes stay outside the capture
  std::vector<int> grids;
  for (auto& L : launches) {
    int per_sm = L.kind == GK_PILE ? newt_pile_blocks_per_sm(L.smem) : newt_tree_persistent_blocks_per_sm(L.bucket);
    grids.push_back(std::min(L.items, per_sm * sm_count(ctx)));
  }
  cudaGraph_t graph;
  CKS(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  for (size_t li = 0; li < launches.size(); ++li) {
    const auto& L = launches[li];
    const int grid = grids[li];
    cudaMemsetAsync(L.dc, 0, sizeof(int), ctx->stream);
    if (L.kind == GK_PILE)
      newt_launch_pile_persistent((const PileGroupDev*)L.dg, L.dq, L.dc, L.items, n_steps, grid, L.smem, ctx->stream);
    else
      newt_launch_tree_persistent((const TreeGroupDev*)L.dg, L.dq, L.dc, L.items, L.bucket, n_steps, grid, ctx->stream);
  }
  cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
  if (ce != cudaSuccess) { ctx->err = cudaGetErrorString(ce); return NEWT_E_CUDA; }
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  CKS(cudaGraphInstantiate(&ctx->graph_exec, graph, 0));
  cudaGraphDestroy(graph);
  // the graph references these buffers: keep them with the context
  for (void* p : ctx->plan_bufs) cudaFree(p);
  ctx->plan_bufs = bufs;
  ctx->graph_steps = n_steps;
  ctx->graph_dirty = false;
  ctx->queue_items = (int)launches.size();
  return NEWT_OK;
}

int step_batched(newt_gpu_ctx* ctx, int n_steps) {
  bool has_tc = false;
  for (auto& g : ctx->groups) if (g->n > 0 && g->kind == GK_TREE_CONTACT) has_tc = true;
  if (ctx->graph_dirty || ctx->graph_steps != n_steps || !ctx->graph_exec) {
    int rc = capture(ctx, n_steps);
    if (rc != NEWT_OK) return rc;
  }
  if (ctx->queue_items > 0) {
    CKS(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
    ctx->launches += ctx->queue_items;
  }
  if (has_tc) {
    for (auto& gp : ctx->groups)
      if (gp->n > 0 && gp->kind == GK_TREE_CONTACT) {
        int rc = newt_tc_step(ctx, gp.get(), n_steps, 1);
        if (rc != NEWT_OK) return rc;
      }
  }
  mark_stepped(ctx);
  return NEWT_OK;
}
