// Host-side runtime structures (internal to the library).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/newt_gpu.h"
#include "groups.h"


struct HostModel {
  int kind = -1, size = 0, np = 0;
  int n_links = 0, n_bodies = 0, n_geoms = 0;
  int nq = 0, nv = 0;
  std::vector<newt_link_desc> links;
  std::vector<newt_body_desc> bodies;
  std::vector<newt_geom_desc> geoms;
  float dt = 0.005f, g[3] = {0, 0, -9.81f};
  int solver = 1, iterations = 20, self_coll = 0, integrator = NEWT_INTEGRATOR_EULER, cone = NEWT_CONE_PYRAMIDAL;
  float mag[3] = {0, -0.5f, 0};  // World::magnetic_field (magnetometers)
  bool explicit_pairs = false;    // World::pair_list given: `pairs`, in order
  std::vector<std::pair<int, int>> pairs;
  std::string key;  // topo_key(), computed once at upload
  // pile worlds whose rows are not four pyramidal facets per contact
  bool general_rows() const {
    if (cone != NEWT_CONE_PYRAMIDAL) return true;
    for (auto& gd : geoms)
      if (gd.condim != 3) return true;
    return false;
  }
  int group = -1;   // the group its worlds live in, once one exists
  // topology key: trees in one group must share parent/joint layout
  std::string topo_key() const {
    std::string k;
    for (auto& l : links) { k += std::to_string(l.parent); k += ':'; k += std::to_string(l.joint); k += ','; }
    if (kind == GK_TREE_CONTACT) {
      // shapes, attachments, condim, filters and in-tree collision fix the
      // pair list and the rows
      k += self_coll ? "s" : "n";
      k += cone == NEWT_CONE_ELLIPTIC ? "e" : "p";
      if (explicit_pairs) {  // the pair list fixes the pairs and their order
        k += "L";
        for (auto& pr : pairs) { k += std::to_string(pr.first); k += '-'; k += std::to_string(pr.second); k += ';'; }
      }
      for (auto& gd : geoms) {
        k += 'g'; k += std::to_string(gd.shape); k += '@'; k += std::to_string(gd.link);
        k += 'c'; k += std::to_string(gd.condim); k += 'f'; k += std::to_string(gd.group); k += '/';
        k += std::to_string(gd.mask);
      }
    }
    if (kind == GK_PILE) {
      // geom order fixes the pair order; shapes may differ per world; the
      // solver picks the step's kernels
      k += "np"; k += std::to_string(np);
      if (solver == NEWT_SOLVER_NEWTON) k += "newton";
      else if (general_rows()) k += "general";
    }
    return k;
  }
};

struct SlotRef {
  int group = -1, index = -1, model = -1;
  bool live = false;
};

struct newt_gpu_ctx;

struct HostGroup {
  int id = 0, kind = 0, size = 0, np = 0;
  std::string topo_key;
  int nq = 0, nv = 0;
  int cap = 0, n = 0;  // capacity and high-water mark
  std::vector<int> free_idx, slot_of;
  // float rows x cap (tree: SoA) or cap x fstride (pile: world-major)
  size_t frows = 0, irows = 0;
  float* dF = nullptr;
  int* dI = nullptr;
  int* dtopo = nullptr;
  std::vector<float> hF;  // host mirror of all float fields
  std::vector<int> hI;    // host mirror of all int fields
  std::vector<int> topo;
  std::vector<uint32_t> status_host;
  bool model_dirty = false;
  std::vector<int> pending;  // indices whose model record awaits upload
  // tree layout rows
  int r_axis = 0, r_jp = 0, r_jc = 0, r_rootq = 0, r_mass = 0, r_inert = 0, r_damp = 0, r_arm = 0, r_dtg = 0;
  int r_q = 0, r_qd = 0, r_qfrc = 0, r_qacc = 0;
  int ri_solver = 0, ri_live = 0, ri_status = 0, ri_integ = -1;
  // pile layout
  PileLayout lay{};
  int maxc = 0;
  int maxc_cap = 0;  // the context's cap on maxc for pile groups (0: none)
  // tree-contact groups: per-geom model rows, geom topology, candidate pairs
  int ng = 0, npairs = 0;
  int tc_rpc = 4, tc_cone = NEWT_CONE_PYRAMIDAL;  // tree contact: rows per contact, cone
  bool tc_general = false;  // tree contact: the elliptic cone, or condim 4 or 6 on some geom
  int r_geom = 0, ri_mode = 0, ri_iters = 0;
  std::vector<int> gtopo, gpairs;
  int* dgtopo = nullptr;
  int* dpairs = nullptr;
  bool soa() const { return kind == GK_TREE || kind == GK_TREE_CONTACT; }
  bool pile_newton = false;   // pile worlds under newt's free-body Newton solve (pile_newton.cu)
  bool pile_general = false;  // pile worlds with the elliptic cone or condim 1, 4, 6 (pile_general.cu)
  // solved apart from the facet-row PGS kernels: per env-step collide, the
  // group's own solve, integrate
  bool pile_solo() const { return pile_newton || pile_general; }
  TcGroupDev tc_dev() const;
  void setup_tc(const HostModel& m);
  void* plain_scratch = nullptr;  // pile solver scratch, cap worlds (both step forms)
  size_t plain_scratch_bytes = 0;
  long scr_stride = 0;             // floats per world in plain_scratch

  int reserve_indices(newt_gpu_ctx* ctx, int k, std::vector<int>& out);
  int* release_index(int idx);  // host side; returns the world's device live flag
  int* live_flag(int idx);      // the world's device live flag
  void write_model(newt_gpu_ctx* ctx, int idx, const HostModel& m);
  int flush_model(newt_gpu_ctx* ctx);
  // generalised force / acceleration rows of one world in the host mirror,
  // moved per world by io_scatter / io_gather (state: io_state_in/out)
  void stage_qfrc(int idx, const HostModel& m, const float* qfrc);
  void read_qacc(int idx, const HostModel& m, float* qacc) const;
  int fetch_status(newt_gpu_ctx* ctx);
  int clear_status(newt_gpu_ctx* ctx);
  int read_contacts(newt_gpu_ctx* ctx, int idx, int cap, int* n_out, int* pairs, float* data);
  int read_impulses(newt_gpu_ctx* ctx, int idx, int cap, int* n_out, float* imp);
  void release();
  // kernel argument builders
  TreeGroupDev tree_dev() const;
  PileGroupDev pile_dev() const;
  size_t bytes_per_world() const;
  // float/int element accessors (host mirror)
  float& F(size_t row, size_t w) { return soa() ? hF[row * cap + w] : hF[w * frows + row]; }
  int& I(size_t row, size_t w) { return soa() ? hI[row * cap + w] : hI[w * irows + row]; }
  float Fc(size_t row, size_t w) const { return soa() ? hF[row * cap + w] : hF[w * frows + row]; }
  int Ic(size_t row, size_t w) const { return soa() ? hI[row * cap + w] : hI[w * irows + row]; }
};

struct newt_gpu_ctx {
  int device = 0;
  int max_worlds = 0;
  int max_contacts = 0;  // pile contact capacity cap (newt_gpu_opts::max_contacts)
  uint64_t budget = 0, used = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  std::string err;
  std::vector<HostModel> models;
  std::vector<std::unique_ptr<HostGroup>> groups;
  std::vector<SlotRef> slots;
  std::vector<int> free_slots;
  void* l2buf = nullptr;
  unsigned l2flip = 0;
  int64_t launches = 0;
  // batched path
  cudaGraphExec_t graph_exec = nullptr;
  int graph_steps = -1;
  bool graph_dirty = true;
  std::vector<void*> plan_bufs;  // device queues / group tables the graph reads
  int queue_items = 0;
  cudaStream_t side = nullptr;   // second capture branch (tree persistent kernels)
  cudaStream_t pside[3] = {nullptr, nullptr, nullptr};  // pile island-class branches
  cudaEvent_t pev[4] = {nullptr, nullptr, nullptr, nullptr};
  // batched piles: world-range branches, each with its own main stream, three
  // island-class streams and four fork/join events
  static constexpr int PILE_BRANCHES = 3;
  // launch choices of the batched form (newt_gpu_autotune): pile branches
  // (0: by world count), tree persistent grid in percent of full residency
  int tune_branches = 0, tune_tree_grid_pct = 100;
  // pile worlds in the batched form: 1 = one world-persistent launch over a
  // cost-sorted queue (pile_fused.cu), 0 = the island-class pipeline per
  // env-step; the persistent launch's shape (gang size and barriers, an
  // index into pile_fused.cu's shape table) and grid in percent of full
  // residency (default: gangs of 8 warps, two per SM, meeting once per
  // env-step, the fastest shape on 8192 sixteen-body piles)
  int tune_pile_fused = 1, tune_fused_shape = 10, tune_fused_pct = 100;
  // the persistent launch of the captured graph: its timing events (external
  // records when profiling), its work counters (device: contacts, rounds,
  // levels, worlds) and whether the graph holds one; `last_fused` tells the
  // profiling surface that the last batched call ran it
  cudaEvent_t fkev[2] = {nullptr, nullptr};
  unsigned long long* fused_work = nullptr;
  bool graph_fused = false, last_fused = false;
  // tree-contact groups' branch of the captured graph, and its env-steps
  // with timing events (profiling)
  cudaStream_t tcstream = nullptr;
  int graph_tc_steps = 0;
  cudaStream_t pbs[PILE_BRANCHES][4] = {};
  cudaEvent_t pbe[PILE_BRANCHES][5] = {};
  // plain path: one single-group table per group
  struct PlainTable { void* dG; int* dseg; int* lists; int ng, worlds, slots; };
  bool plain_dirty = true;
  std::vector<PlainTable> plain_tables;
  std::vector<void*> plain_bufs;
  size_t queue_cap = 0;
  // profiling: timing events around the pile kernels of batched captures,
  // and the island work lists (pointer, slots) the last step used
  bool profile = false;
  std::vector<cudaEvent_t> kev;  // [branch][env-step][kernel][start, end]
  int kev_steps = 0, kev_branches = 1;
  std::vector<std::pair<int*, int>> last_lists;
  std::vector<std::pair<int*, int>> graph_lists;  // the captured graph's, copied to last_lists per replay
  int graph_kev_steps = 0, graph_kev_branches = 1;
  // tree-contact step timing: 3 kernels x (start, end) per env-step of the
  // last tree-contact step call, recorded when `profile` is on
  std::vector<cudaEvent_t> tcev;
  int tcev_steps = 0;
  // per-world state I/O staging (pinned host + device, same size)
  void* io_h = nullptr;
  void* io_d = nullptr;
  size_t io_bytes = 0;
  // control streams: per world a horizon x nv block of the device arena and
  // a cursor; `ctrl_of_slot` maps a slot to its entry (-1: none)
  struct CtrlEntry { int slot, nv, h, t; size_t off; };
  float* ctrl_arena = nullptr;
  size_t ctrl_cap = 0;                               // floats
  std::vector<std::pair<size_t, size_t>> ctrl_free;  // (offset, floats), sorted
  std::vector<CtrlEntry> ctrl;
  std::vector<int> ctrl_of_slot;
  void* ctrl_dev = nullptr;  // device copy of the entries, rebuilt when `ctrl_dirty`
  size_t ctrl_dev_cap = 0;
  bool ctrl_dirty = false;
};

// rows [lo, lo + cnt) of the worlds `idx` of one group (of its int block
// when `ints`, moved as raw 32-bit words)
struct RowMove {
  HostGroup* g;
  std::vector<int> idx;
  size_t lo, cnt;
  bool ints = false;
};
int io_scatter(newt_gpu_ctx* ctx, const std::vector<RowMove>& mv);  // host mirror -> device
int io_gather(newt_gpu_ctx* ctx, const std::vector<RowMove>& mv);   // device -> host mirror
int io_clear_flags(newt_gpu_ctx* ctx, const std::vector<int*>& flags);  // *flag = 0 on the device
// MuJoCo-layout state of the named worlds in and out, converted on the device
// (world_io.cu)
int io_state_in(newt_gpu_ctx* ctx, const int32_t* slots, int n, const float* qpos, const float* qvel);
int io_state_out(newt_gpu_ctx* ctx, const int32_t* slots, int n, float* qpos, float* qvel);
int io_hold_flags(newt_gpu_ctx* ctx, const std::vector<int*>& flags);   // the same, queued without a wait
void ctrl_release_slot(newt_gpu_ctx* ctx, int slot);                     // ends the slot's control stream

HostGroup* find_or_make_group(newt_gpu_ctx* ctx, HostModel& m);
int step_plain(newt_gpu_ctx* ctx, int n_steps);
int step_batched(newt_gpu_ctx* ctx, int n_steps);
int autotune_batched(newt_gpu_ctx* ctx, int n_steps, int horizon, int32_t* choice);

// kernel launchers (defined in the .cu kernel files)
extern "C" int newt_tree_bucket(int L);
extern "C" void newt_launch_tree_fused(const TreeGroupDev& g, int base, int count, int n_steps, cudaStream_t st);
extern "C" void newt_launch_tree_plain(const TreeGroupDev& g, cudaStream_t st);
extern "C" void newt_tc_offsets(int L, int nv, int ng, int maxc, int rpc, int* con, int* imp, int* misc);
extern "C" size_t newt_tc_ws_bytes(int L, int nv, int ng, int maxc, int rpc);
extern "C" size_t newt_pile_ws_bytes(int nb, int np, int maxc);
extern "C" size_t newt_pile_newton_bytes(int maxc);
