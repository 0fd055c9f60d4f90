// Step dispatch.
//
// Plain form (the drop-in baseline): every group is launched separately,
// one launch per stage per env-step with fixed tiles.
// Batched form: the whole call is captured once in a CUDA graph and
// replayed.  Trees run their horizon in one persistent launch per size
// bucket, pulling work items from a device queue sorted by size class;
// pile worlds of every size run theirs in one world-persistent launch over
// a size-sorted queue (pile_fused.cu; the island-class pipeline, one launch
// per stage per env-step, stays available to the autotuner); tree-contact
// worlds run their per-env-step kernels on a third branch of the same graph.
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
extern "C" int newt_tree_persistent_blocks_per_sm(int bucket);
extern "C" size_t newt_pile_ws_bytes(int nb, int np, int maxc);
extern "C" int newt_launch_pile_step(const PileGroupDev* dG, const int* dwseg, int ng, int total_worlds,
                                     int total_slots, int* lists, int write_diag, cudaStream_t st,
                                     const cudaStream_t* side, cudaEvent_t* ev, cudaEvent_t* kev);
extern "C" void newt_pile_init();
extern "C" int newt_pile_fused_blocks_per_sm(int shape, int nbm, int cm);
extern "C" int newt_pile_fused_worlds_per_block(int shape);
extern "C" int newt_launch_pile_fused(const PileGroupDev* dG, const int* dwseg, int ng, int* queue, int n_items,
                                      int* counter, int n_steps, int grid, unsigned long long* work, unsigned* cost,
                                      int nbm, int cm, int shape, cudaStream_t st);
extern "C" int newt_tc_prepare(newt_gpu_ctx* ctx, HostGroup* g, int n_steps);
extern "C" size_t newt_pile_newton_bytes(int maxc);
extern "C" int newt_launch_pile_solo_step(const PileGroupDev* dG, const int* dwseg, int ng, int total_worlds,
                                          int total_slots, int* lists, int write_diag, int kinds, cudaStream_t st);
extern "C" int newt_tc_launch(newt_gpu_ctx* ctx, HostGroup* g, int n_steps, cudaStream_t st, bool capturing);

// Streams and events the pile step forks its island classes onto.
static int ensure_pile_streams(newt_gpu_ctx* ctx) {
  if (ctx->pside[0]) return NEWT_OK;
  newt_pile_init();
  for (int k = 0; k < 3; ++k) CKS(cudaStreamCreateWithFlags(&ctx->pside[k], cudaStreamNonBlocking));
  for (int k = 0; k < 4; ++k) CKS(cudaEventCreateWithFlags(&ctx->pev[k], cudaEventDisableTiming));
  return NEWT_OK;
}
extern "C" size_t newt_pile_list_bytes(int slots);
extern "C" int newt_tc_step(newt_gpu_ctx* ctx, HostGroup* g, int n_steps, int fused);

static int sm_count(newt_gpu_ctx* ctx) {
  static int n = 0;
  if (n == 0) { cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, ctx->device); if (n <= 0) n = 1; }
  return n;
}

// Per-group solver scratch for pile worlds (world-major, cap worlds).
static int ensure_pile_scratch(newt_gpu_ctx* ctx, HostGroup* g) {
  int rs = ensure_pile_streams(ctx);
  if (rs != NEWT_OK) return rs;
  size_t per = newt_pile_ws_bytes(g->size, g->np, g->maxc);
  if (g->pile_newton) per += newt_pile_newton_bytes(g->maxc);  // H, its factors, the solver vectors
  size_t need = per * (size_t)g->cap;
  if (g->plain_scratch_bytes < need) {
    if (g->plain_scratch) cudaFree(g->plain_scratch);
    g->plain_scratch = nullptr;
    CKS(cudaMalloc(&g->plain_scratch, need));
    g->plain_scratch_bytes = need;
    ctx->graph_dirty = true;
    ctx->plain_dirty = true;
  }
  g->scr_stride = (long)(per / 4);
  return NEWT_OK;
}

// A device segment table over a set of pile groups.
struct PileTable {
  PileGroupDev* dG = nullptr;
  int* dseg = nullptr;   // [ng+1] cumulative world counts
  int* lists = nullptr;  // island work lists + counters
  int ng = 0, worlds = 0, slots = 0;
};

// Branch `part` of `parts` covers worlds [n*part/parts, n*(part+1)/parts) of
// every group: a view of the group with its record, int and scratch pointers
// moved to the range (pile records are world-major).
static int build_pile_table(newt_gpu_ctx* ctx, const std::vector<HostGroup*>& gs, PileTable& t,
                            std::vector<void*>& owned, int part = 0, int parts = 1) {
  std::vector<PileGroupDev> hg;
  std::vector<int> wseg{0}, iseg{0};
  for (HostGroup* g : gs) {
    int rc = ensure_pile_scratch(ctx, g);
    if (rc != NEWT_OK) return rc;
    const int a = (int)((long)g->n * part / parts), b = (int)((long)g->n * (part + 1) / parts);
    if (b <= a) continue;
    PileGroupDev d = g->pile_dev();
    d.n = b - a;
    d.F += (size_t)a * d.lay.fstride;
    d.I += (size_t)a * d.lay.istride;
    d.scr += (size_t)a * d.sstride;
    hg.push_back(d);
    wseg.push_back(wseg.back() + d.n);
    iseg.push_back(iseg.back() + d.n * g->size);
  }
  t.ng = (int)hg.size();
  t.worlds = wseg.back();
  t.slots = iseg.back();
  if (t.ng == 0) return NEWT_OK;
  CKS(cudaMalloc(&t.dG, hg.size() * sizeof(PileGroupDev)));
  CKS(cudaMalloc(&t.dseg, wseg.size() * sizeof(int)));
  CKS(cudaMalloc(&t.lists, newt_pile_list_bytes(t.slots)));
  CKS(cudaMemcpy(t.dG, hg.data(), hg.size() * sizeof(PileGroupDev), cudaMemcpyHostToDevice));
  CKS(cudaMemcpy(t.dseg, wseg.data(), wseg.size() * sizeof(int), cudaMemcpyHostToDevice));
  owned.push_back(t.dG);
  owned.push_back(t.dseg);
  owned.push_back(t.lists);
  return NEWT_OK;
}

// Timing events for the pile kernels of a captured horizon (profiling only):
// NEWT_PILE_KERNELS pairs per env-step and branch.
static int ensure_kernel_events(newt_gpu_ctx* ctx, int n_steps, int branches = 1) {
  const size_t need = (size_t)2 * NEWT_PILE_KERNELS * n_steps * branches;
  while (ctx->kev.size() < need) {
    cudaEvent_t e;
    CKS(cudaEventCreate(&e));
    ctx->kev.push_back(e);
  }
  return NEWT_OK;
}

// `n_steps` env-steps of one table on stream `st` (island classes forked to
// `side`, joined with `ev`); timing events of branch `branch` when profiling.
static void launch_pile_steps(newt_gpu_ctx* ctx, const PileTable& t, int n_steps, cudaStream_t st,
                              const cudaStream_t* side, cudaEvent_t* ev, int branch) {
  for (int s = 0; s < n_steps; ++s) {
    cudaEvent_t* kev = ctx->profile
                           ? ctx->kev.data() + (size_t)2 * NEWT_PILE_KERNELS * ((size_t)branch * n_steps + s)
                           : nullptr;
    ctx->launches += newt_launch_pile_step(t.dG, t.dseg, t.ng, t.worlds, t.slots, t.lists, s == n_steps - 1, st,
                                           side, ev, kev);
  }
}

// Streams and events of the batched form's world-range branches.
static int ensure_pile_branches(newt_gpu_ctx* ctx) {
  if (ctx->pbs[0][0]) return NEWT_OK;
  for (int b = 0; b < newt_gpu_ctx::PILE_BRANCHES; ++b) {
    for (int k = 0; k < 4; ++k) CKS(cudaStreamCreateWithFlags(&ctx->pbs[b][k], cudaStreamNonBlocking));
    for (int k = 0; k < 5; ++k) CKS(cudaEventCreateWithFlags(&ctx->pbe[b][k], cudaEventDisableTiming));
  }
  return NEWT_OK;
}

// ---------------------------------------------------------------------------
// plain
// ---------------------------------------------------------------------------
// Per-group single-entry tables (rebuilt when groups change).
static int ensure_plain_tables(newt_gpu_ctx* ctx) {
  if (ctx->plain_dirty) {
    for (void* p : ctx->plain_bufs) cudaFree(p);
    ctx->plain_bufs.clear();
    ctx->plain_tables.clear();
    for (auto& gp : ctx->groups) {
      PileTable t;
      if (gp->kind == GK_PILE && gp->n > 0) {
        int rc = build_pile_table(ctx, {gp.get()}, t, ctx->plain_bufs);
        if (rc != NEWT_OK) return rc;
      }
      ctx->plain_tables.push_back({t.dG, t.dseg, t.lists, t.ng, t.worlds, t.slots});
    }
    ctx->plain_dirty = false;
  }
  return NEWT_OK;
}

extern "C" int newt_launch_pile_resolve(const PileGroupDev* dG, const int* dwseg, int ng, int total_worlds,
                                        int total_slots, int* lists, int solve, cudaStream_t st);

// The contact sensors' re-solve of every world of pile group `g` at its
// current state, on the context's stream (pile_kernels.cu).
int pile_resolve_group(newt_gpu_ctx* ctx, HostGroup* g) {
  int rc = ensure_plain_tables(ctx);
  if (rc != NEWT_OK) return rc;
  const auto& T = ctx->plain_tables[g->id];
  ctx->launches += newt_launch_pile_resolve((const PileGroupDev*)T.dG, T.dseg, T.ng, T.worlds, T.slots, T.lists,
                                            g->pile_dev().solve, ctx->stream);
  return NEWT_OK;
}

int step_plain(newt_gpu_ctx* ctx, int n_steps) {
  int rc0 = ensure_plain_tables(ctx);
  if (rc0 != NEWT_OK) return rc0;
  ctx->last_lists.clear();
  for (const auto& T : ctx->plain_tables)
    if (T.lists) ctx->last_lists.push_back({T.lists, T.slots});
  ctx->kev_steps = 0;
  ctx->kev_branches = 1;
  ctx->last_fused = false;
  for (int s = 0; s < n_steps; ++s) {
    for (size_t gi = 0; gi < ctx->groups.size(); ++gi) {
      HostGroup* g = ctx->groups[gi].get();
      if (g->n == 0) continue;
      if (g->kind == GK_TREE) {
        newt_launch_tree_plain(g->tree_dev(), ctx->stream);
        ctx->launches += 2;
      } else if (g->kind == GK_PILE && g->pile_solo()) {
        const auto& T = ctx->plain_tables[gi];
        ctx->launches += newt_launch_pile_solo_step((const PileGroupDev*)T.dG, T.dseg, T.ng, T.worlds, T.slots,
                                                    T.lists, s == n_steps - 1, 1 << g->pile_dev().solve, ctx->stream);
      } else if (g->kind == GK_PILE) {
        const auto& T = ctx->plain_tables[gi];
        ctx->launches += newt_launch_pile_step((const PileGroupDev*)T.dG, T.dseg, T.ng, T.worlds, T.slots, T.lists,
                                               s == n_steps - 1, ctx->stream, ctx->pside, ctx->pev, nullptr);
      } else if (g->kind == GK_TREE_CONTACT) {
        int rc = newt_tc_step(ctx, g, 1, 0);
        if (rc != NEWT_OK) return rc;
      }
    }
  }
  return NEWT_OK;
}

// ---------------------------------------------------------------------------
// batched
// ---------------------------------------------------------------------------
static int capture(newt_gpu_ctx* ctx, int n_steps) {
  std::vector<void*> bufs;
  // trees: one persistent launch per size bucket over a cost-sorted queue
  struct TreeLaunch { int bucket; TreeGroupDev* dg; int* dq; int* dc; int items; int grid; };
  std::vector<TreeLaunch> tls;
  const int buckets[4] = {8, 16, 32, 65};
  for (int bucket : buckets) {
    struct It { long cost; int g, base, count; };
    std::vector<It> its;
    std::vector<TreeGroupDev> tg;
    for (auto& gp : ctx->groups) {
      HostGroup* g = gp.get();
      if (g->n == 0 || g->kind != GK_TREE || newt_tree_bucket(g->size) != bucket) continue;
      int gi = (int)tg.size();
      tg.push_back(g->tree_dev());
      const int chunk = 64;
      for (int b = 0; b < g->n; b += chunk) its.push_back({(long)g->size, gi, b, std::min(chunk, g->n - b)});
    }
    if (its.empty()) continue;
    std::stable_sort(its.begin(), its.end(), [](const It& a, const It& b) { return a.cost > b.cost; });
    std::vector<int> q;
    for (auto& i : its) { q.push_back(i.g); q.push_back(i.base); q.push_back(i.count); }
    TreeLaunch L{bucket, nullptr, nullptr, nullptr, (int)its.size(), 0};
    CKS(cudaMalloc(&L.dg, tg.size() * sizeof(TreeGroupDev)));
    CKS(cudaMemcpy(L.dg, tg.data(), tg.size() * sizeof(TreeGroupDev), cudaMemcpyHostToDevice));
    CKS(cudaMalloc(&L.dq, q.size() * sizeof(int)));
    CKS(cudaMemcpy(L.dq, q.data(), q.size() * sizeof(int), cudaMemcpyHostToDevice));
    CKS(cudaMalloc(&L.dc, sizeof(int)));
    bufs.push_back(L.dg); bufs.push_back(L.dq); bufs.push_back(L.dc);
    const int full = newt_tree_persistent_blocks_per_sm(bucket) * sm_count(ctx);
    L.grid = std::min(L.items, std::max(1, full * ctx->tune_tree_grid_pct / 100));
    tls.push_back(L);
  }
  // facet-row PGS piles, largest worlds first; the piles solved apart
  // (Newton, general rows) in their own table, stepped per env-step:
  // collide, each group's solve, integrate
  std::vector<HostGroup*> piles, npiles;
  long pile_worlds = 0;
  int solo_kinds = 0;
  for (auto& gp : ctx->groups)
    if (gp->n > 0 && gp->kind == GK_PILE) {
      if (gp->pile_solo()) {
        npiles.push_back(gp.get());
        solo_kinds |= 1 << gp->pile_dev().solve;
        continue;
      }
      piles.push_back(gp.get());
      pile_worlds += gp->n;
    }
  PileTable nt;
  if (!npiles.empty()) {
    int rc = build_pile_table(ctx, npiles, nt, bufs, 0, 1);
    if (rc != NEWT_OK) return rc;
  }
  std::stable_sort(piles.begin(), piles.end(), [](HostGroup* a, HostGroup* b) { return a->size > b->size; });
  const bool fused = ctx->tune_pile_fused != 0;
  // fused: one table over every pile group; its flat world order is the
  // queue (groups by size, largest first)
  PileTable ft;
  int* fcounter = nullptr;
  int* fqueue = nullptr;
  unsigned* fcost = nullptr;
  int fgrid = 0, fnbm = 0, fcm = 0;
  const int nbr = fused ? 0
                        : (ctx->tune_branches > 0 ? std::min(ctx->tune_branches, newt_gpu_ctx::PILE_BRANCHES)
                                                  : (int)std::max<long>(1, std::min<long>(2, pile_worlds / 4096)));
  std::vector<PileTable> pts(nbr);
  if (pile_worlds > 0) {
    int rc = ensure_pile_branches(ctx);
    if (rc != NEWT_OK) return rc;
  }
  if (fused && pile_worlds > 0) {
    int rc = build_pile_table(ctx, piles, ft, bufs, 0, 1);
    if (rc != NEWT_OK) return rc;
    CKS(cudaMalloc(&fcounter, sizeof(int)));
    CKS(cudaMalloc(&fqueue, sizeof(int) * (size_t)ft.worlds));
    CKS(cudaMalloc(&fcost, sizeof(unsigned) * (size_t)ft.worlds));
    CKS(cudaMemset(fcost, 0, sizeof(unsigned) * (size_t)ft.worlds));  // first call: any order
    bufs.push_back(fcounter);
    bufs.push_back(fqueue);
    bufs.push_back(fcost);
    if (!ctx->fused_work) CKS(cudaMalloc(&ctx->fused_work, 4 * sizeof(unsigned long long)));
    if (!ctx->fkev[0])
      for (int k = 0; k < 2; ++k) CKS(cudaEventCreate(&ctx->fkev[k]));
    for (HostGroup* g : piles) { fnbm = std::max(fnbm, g->size); fcm = std::max(fcm, g->maxc); }
    const int wpb = newt_pile_fused_worlds_per_block(ctx->tune_fused_shape);
    const int full = newt_pile_fused_blocks_per_sm(ctx->tune_fused_shape, fnbm, fcm) * sm_count(ctx);
    fgrid = std::min((ft.worlds + wpb - 1) / wpb, std::max(1, full * ctx->tune_fused_pct / 100));
  }
  for (int b = 0; b < nbr; ++b) {
    int rc = build_pile_table(ctx, piles, pts[b], bufs, b, nbr);
    if (rc != NEWT_OK) return rc;
  }
  // tree-contact groups: scratch and events before the capture
  std::vector<HostGroup*> tcs;
  for (auto& gp : ctx->groups)
    if (gp->n > 0 && gp->kind == GK_TREE_CONTACT) {
      int rc = newt_tc_prepare(ctx, gp.get(), n_steps);
      if (rc != NEWT_OK) return rc;
      tcs.push_back(gp.get());
    }
  if (!tcs.empty() && !ctx->tcstream) CKS(cudaStreamCreateWithFlags(&ctx->tcstream, cudaStreamNonBlocking));

  cudaEvent_t fork = nullptr, join = nullptr, tjoin = nullptr;
  if (!ctx->side) CKS(cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
  CKS(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  CKS(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
  CKS(cudaEventCreateWithFlags(&tjoin, cudaEventDisableTiming));
  cudaGraph_t graph;
  if (ctx->profile && nbr > 0) {
    int r = ensure_kernel_events(ctx, n_steps, nbr);
    if (r != NEWT_OK) return r;
  }
  ctx->graph_lists.clear();
  for (const PileTable& t : pts)
    if (t.ng > 0) ctx->graph_lists.push_back({t.lists, t.slots});
  CKS(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  cudaEventRecord(fork, ctx->stream);
  cudaStreamWaitEvent(ctx->side, fork, 0);
  for (auto& L : tls) {
    cudaMemsetAsync(L.dc, 0, sizeof(int), ctx->side);
    newt_launch_tree_persistent(L.dg, L.dq, L.dc, L.items, L.bucket, n_steps, L.grid, ctx->side);
  }
  cudaEventRecord(join, ctx->side);
  int tc_timed = 0;
  const int64_t l0 = ctx->launches;
  if (!tcs.empty()) {
    cudaStreamWaitEvent(ctx->tcstream, fork, 0);
    for (HostGroup* g : tcs) tc_timed = newt_tc_launch(ctx, g, n_steps, ctx->tcstream, true);
    cudaEventRecord(tjoin, ctx->tcstream);
  }
  const int tc_launches = (int)(ctx->launches - l0);
  const int64_t before = ctx->launches;
  for (int s = 0; s < n_steps && nt.ng > 0; ++s)
    ctx->launches += newt_launch_pile_solo_step(nt.dG, nt.dseg, nt.ng, nt.worlds, nt.slots, nt.lists,
                                                s == n_steps - 1, solo_kinds, ctx->stream);
  int fused_launches = 0;
  if (fused && ft.ng > 0) {
    cudaStream_t fs = ctx->pbs[0][0];
    cudaStreamWaitEvent(fs, fork, 0);
    cudaMemsetAsync(fcounter, 0, sizeof(int), fs);
    cudaMemsetAsync(ctx->fused_work, 0, 4 * sizeof(unsigned long long), fs);
    if (ctx->profile) cudaEventRecordWithFlags(ctx->fkev[0], fs, cudaEventRecordExternal);
    fused_launches = newt_launch_pile_fused(ft.dG, ft.dseg, ft.ng, fqueue, ft.worlds, fcounter, n_steps, fgrid,
                                            ctx->fused_work, fcost, fnbm, fcm, ctx->tune_fused_shape, fs);
    if (ctx->profile) cudaEventRecordWithFlags(ctx->fkev[1], fs, cudaEventRecordExternal);
    cudaEventRecord(ctx->pbe[0][4], fs);
    cudaStreamWaitEvent(ctx->stream, ctx->pbe[0][4], 0);
  }
  for (int b = 0; b < nbr; ++b) {
    if (pts[b].ng == 0) continue;
    cudaStream_t* bs = ctx->pbs[b];
    cudaStreamWaitEvent(bs[0], fork, 0);
    launch_pile_steps(ctx, pts[b], n_steps, bs[0], bs + 1, ctx->pbe[b], b);
    cudaEventRecord(ctx->pbe[b][4], bs[0]);
    cudaStreamWaitEvent(ctx->stream, ctx->pbe[b][4], 0);
  }
  const int pile_launches = (int)(ctx->launches - before) + fused_launches;
  ctx->launches = l0;
  ctx->graph_kev_steps = ctx->profile && nbr > 0 && pile_worlds > 0 ? n_steps : 0;
  ctx->graph_kev_branches = std::max(nbr, 1);
  ctx->graph_fused = fused && ft.ng > 0;
  ctx->graph_tc_steps = tc_timed;
  cudaStreamWaitEvent(ctx->stream, join, 0);
  if (!tcs.empty()) cudaStreamWaitEvent(ctx->stream, tjoin, 0);
  cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
  cudaEventDestroy(fork);
  cudaEventDestroy(join);
  cudaEventDestroy(tjoin);
  if (ce != cudaSuccess) { ctx->err = cudaGetErrorString(ce); return NEWT_E_CUDA; }
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  CKS(cudaGraphInstantiate(&ctx->graph_exec, graph, 0));
  cudaGraphDestroy(graph);
  for (void* p : ctx->plan_bufs) cudaFree(p);
  ctx->plan_bufs = bufs;
  ctx->graph_steps = n_steps;
  ctx->graph_dirty = false;
  // kernel launches one replay issues
  ctx->queue_items = (int)tls.size() + pile_launches + tc_launches;
  return NEWT_OK;
}

int step_batched(newt_gpu_ctx* ctx, int n_steps) {
  if (ctx->graph_dirty || ctx->graph_steps != n_steps || !ctx->graph_exec) {
    int rc = capture(ctx, n_steps);
    if (rc != NEWT_OK) return rc;
  }
  if (ctx->queue_items > 0) {
    CKS(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
    ctx->launches += ctx->queue_items;
  }
  ctx->last_lists = ctx->graph_lists;
  ctx->kev_steps = ctx->graph_kev_steps;
  ctx->kev_branches = ctx->graph_kev_branches;
  ctx->last_fused = ctx->graph_fused;
  ctx->tcev_steps = ctx->graph_tc_steps;
  return NEWT_OK;
}

// ---------------------------------------------------------------------------
// autotuning of the batched form's launch choices
// ---------------------------------------------------------------------------
// Every trial steps the live worlds from a snapshot of every group's records
// (model, state, status: the whole step state; solver scratch is rebuilt each
// env-step), so the worlds end where they began.  Three snapshots are timed:
// the worlds as they are, and horizon/2 and horizon env-steps later (piles
// that were falling have landed and their islands have grown); a choice is
// judged by the trapezoid average of its three times, so one that only wins
// on the early regime does not win a horizon spent mostly settled.
int autotune_batched(newt_gpu_ctx* ctx, int n_steps, int horizon, int32_t* choice) {
  if (n_steps <= 0 || horizon <= 0) return NEWT_E_INVALID;
  std::vector<std::pair<void*, size_t>> live;
  for (auto& gp : ctx->groups) {
    HostGroup* g = gp.get();
    if (g->n == 0) continue;
    live.push_back({g->dF, g->frows * (size_t)g->cap * sizeof(float)});
    live.push_back({g->dI, g->irows * (size_t)g->cap * sizeof(int)});
  }
  constexpr int NSNAP = 3;
  std::vector<void*> snap[NSNAP];
  int rc = NEWT_OK;
  auto take = [&](int k) -> int {
    for (auto& b : live) {
      void* p = nullptr;
      if (cudaMalloc(&p, b.second) != cudaSuccess) return NEWT_E_NOMEM;
      snap[k].push_back(p);
      CKS(cudaMemcpyAsync(p, b.first, b.second, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    return NEWT_OK;
  };
  auto restore = [&](int k) -> int {
    for (size_t i = 0; i < snap[k].size(); ++i)
      CKS(cudaMemcpyAsync(live[i].first, snap[k][i], live[i].second, cudaMemcpyDeviceToDevice, ctx->stream));
    return NEWT_OK;
  };
  // piles: the persistent launch in each gang shape (warps per block,
  // blocks per SM, whether the gang also meets between assembly and sweeps,
  // one or two worlds per warp), or the
  // island-class pipeline with 1, 2 or 3 world-range branches; trees: full
  // or half persistent grid
  struct Cand { int fused, shape, branches, grid_pct; };
  const Cand cands[] = {{1, 0, 0, 100},  {1, 1, 0, 100}, {1, 2, 0, 100}, {1, 3, 0, 100}, {1, 4, 0, 100},
                        {1, 5, 0, 100},  {1, 6, 0, 100}, {1, 7, 0, 100}, {1, 8, 0, 100}, {1, 9, 0, 100},
                        {1, 10, 0, 100}, {1, 11, 0, 100}, {0, 0, 1, 100}, {0, 0, 2, 100}, {0, 0, 3, 100},
                        {1, 10, 0, 50},  {0, 0, 2, 50}};
  const Cand start{ctx->tune_pile_fused, ctx->tune_fused_shape, ctx->tune_branches, ctx->tune_tree_grid_pct};
  auto set = [&](const Cand& c) {
    ctx->tune_pile_fused = c.fused;
    ctx->tune_fused_shape = c.shape;
    ctx->tune_branches = c.branches;
    ctx->tune_tree_grid_pct = c.grid_pct;
    ctx->graph_dirty = true;
  };
  // snapshots at env-steps 0, horizon/2 and horizon, stepped with the current choice
  rc = take(0);
  for (int k = 1, done = 0; k < NSNAP && rc == NEWT_OK; ++k) {
    const int target = (int)((int64_t)horizon * k / (NSNAP - 1));
    while (rc == NEWT_OK && done < target) {
      const int m = std::min(n_steps, target - done);
      rc = step_batched(ctx, m);
      done += m;
    }
    if (rc == NEWT_OK) rc = take(k);
  }
  const float weight[NSNAP] = {0.25f, 0.5f, 0.25f};
  Cand best = start;
  float best_ms = -1.f;
  for (const Cand& c : cands) {
    if (rc != NEWT_OK) break;
    set(c);
    float total = 0.f;
    for (int ph = 0; ph < NSNAP && rc == NEWT_OK; ++ph) {
      // first call captures (and warms up); the second is timed
      for (int rep = 0; rep < 2 && rc == NEWT_OK; ++rep) {
        if ((rc = restore(ph)) != NEWT_OK) break;
        cudaEventRecord(ctx->ev[0], ctx->stream);
        rc = step_batched(ctx, n_steps);
        cudaEventRecord(ctx->ev[1], ctx->stream);
      }
      if (rc != NEWT_OK) break;
      if (cudaEventSynchronize(ctx->ev[1]) != cudaSuccess) { rc = NEWT_E_CUDA; break; }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
      total += weight[ph] * ms;
    }
    if (rc != NEWT_OK) break;
    if (best_ms < 0.f || total < best_ms) { best_ms = total; best = c; }
  }
  if (!snap[0].empty() && rc == NEWT_OK) rc = restore(0);
  cudaStreamSynchronize(ctx->stream);
  for (int k = 0; k < NSNAP; ++k)
    for (void* p : snap[k]) cudaFree(p);
  set(best);
  if (choice) {
    choice[0] = best.fused ? 0 : best.branches;
    choice[1] = best.grid_pct;
    choice[2] = (int32_t)(best_ms * 1000.f);
    choice[3] = best.fused;
    choice[4] = best.shape;
  }
  return rc;
}
