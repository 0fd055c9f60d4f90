// Host runtime behind the C ABI (include/newt_gpu.h): context, model upload
// and classification, world slots grouped by class and size, MuJoCo-layout
// state conversion, step dispatch (plain vs batched), diagnostics.
//
// The boundary mirrors newt's World API (newt/src/world.rs:325 `World::new`,
// :950-981 `add_*`, :519-623 `apply_mujoco_qpos/qvel`, :1459 `step`); errors
// that newt raises as panics come back as status codes.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/newt_gpu.h"
#include "groups.h"
#include "runtime.h"

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
static int fail(newt_gpu_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}
#define CK(call)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) return fail(ctx, NEWT_E_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

// ---------------------------------------------------------------------------
// model upload / classification
// ---------------------------------------------------------------------------
static int classify(newt_gpu_ctx* ctx, const newt_model_desc& d, HostModel& m) {
  m.n_links = d.n_links; m.n_bodies = d.n_bodies; m.n_geoms = d.n_geoms;
  m.links.assign(d.links, d.links + d.n_links);
  m.bodies.assign(d.bodies, d.bodies + d.n_bodies);
  m.geoms.assign(d.geoms, d.geoms + d.n_geoms);
  m.dt = d.dt; for (int k = 0; k < 3; ++k) m.g[k] = d.gravity[k];
  m.solver = d.solver; m.iterations = d.iterations; m.self_coll = d.tree_self_collision;
  m.integrator = d.integrator;
  m.cone = d.cone;
  for (int k = 0; k < 3; ++k) m.mag[k] = d.magnetic_field[k];
  m.explicit_pairs = d.pairs != nullptr;
  m.pairs.clear();
  if (m.explicit_pairs) {
    if (d.n_pairs < 0) return fail(ctx, NEWT_E_INVALID, "n_pairs must be >= 0");
    for (int k = 0; k < d.n_pairs; ++k) {
      const int a = d.pairs[2 * k], b = d.pairs[2 * k + 1];
      if (a < 0 || b < 0 || a >= d.n_geoms || b >= d.n_geoms || a == b)
        return fail(ctx, NEWT_E_INVALID, "pair_list entry out of range");
      m.pairs.push_back({a, b});
    }
  }
  if (!(d.dt > 0.f)) return fail(ctx, NEWT_E_INVALID, "dt must be > 0");
  if (d.cone != NEWT_CONE_PYRAMIDAL && d.cone != NEWT_CONE_ELLIPTIC) return fail(ctx, NEWT_E_INVALID, "unknown cone");
  if (d.integrator != NEWT_INTEGRATOR_EULER && d.integrator != NEWT_INTEGRATOR_RK4)
    return fail(ctx, NEWT_E_INVALID, "unknown integrator");
  if (d.solver != 0 && d.solver != NEWT_SOLVER_PGS && d.solver != NEWT_SOLVER_NEWTON)
    return fail(ctx, NEWT_E_INVALID, "unknown solver mode");
  if ((d.solver == NEWT_SOLVER_PGS || d.solver == NEWT_SOLVER_NEWTON) && d.iterations < 1)
    return fail(ctx, NEWT_E_INVALID, "solver iterations must be >= 1 (newt/src/solver.rs:127-129)");
  int nq = 7 * d.n_bodies, nv = 6 * d.n_bodies;
  for (int i = 0; i < d.n_links; ++i) {
    const newt_link_desc& L = d.links[i];
    if (i == 0 && L.parent != -1) return fail(ctx, NEWT_E_INVALID, "link 0 must be the root");
    if (i > 0 && (L.parent < 0 || L.parent >= i)) return fail(ctx, NEWT_E_INVALID, "links must be topologically sorted");
    if (i == 0 && L.joint != NEWT_JOINT_FREE && L.joint != NEWT_JOINT_FIXED)
      return fail(ctx, NEWT_E_INVALID, "root joint must be free or fixed");
    if (i > 0 && L.joint != NEWT_JOINT_HINGE && L.joint != NEWT_JOINT_SLIDE && L.joint != NEWT_JOINT_FIXED)
      return fail(ctx, NEWT_E_INVALID, "GPU path supports hinge, slide and fixed child joints");
    if (i > 0 && !(L.jp_quat[3] == 1.f && L.jc_quat[3] == 1.f))
      return fail(ctx, NEWT_E_INVALID, "child joint frames must have identity orientation (newt v0 convention)");
    if (i == 0 && L.jc_quat[3] != 1.f) return fail(ctx, NEWT_E_INVALID, "root joint_offset_in_child must be identity");
    if (!(L.mass > 0.f)) return fail(ctx, NEWT_E_INVALID, "link mass must be > 0");
    nq += L.joint == NEWT_JOINT_FREE ? 7 : (L.joint == NEWT_JOINT_FIXED ? 0 : 1);
    nv += L.joint == NEWT_JOINT_FREE ? 6 : (L.joint == NEWT_JOINT_FIXED ? 0 : 1);
  }
  m.nq = nq; m.nv = nv;
  if (d.n_links > NEWT_MAX_LINKS) return fail(ctx, NEWT_E_INVALID, "too many links");
  if (d.n_bodies > NEWT_MAX_BODIES) return fail(ctx, NEWT_E_INVALID, "too many bodies");
  // shape sizes (newt's geom constructors and loaders refuse the rest)
  for (int k = 0; k < d.n_geoms; ++k) {
    const newt_geom_desc& G = d.geoms[k];
    const float a = G.size[0], b = G.size[1], c = G.size[2];
    bool ok = true;
    switch (G.shape) {
      case NEWT_SHAPE_SPHERE: ok = a > 0.f; break;
      case NEWT_SHAPE_BOX: case NEWT_SHAPE_ELLIPSOID: ok = a > 0.f && b > 0.f && c > 0.f; break;
      case NEWT_SHAPE_CAPSULE: ok = a > 0.f && b >= 0.f; break;
      case NEWT_SHAPE_CYLINDER: ok = a > 0.f && b > 0.f; break;
      default: break;
    }
    if (!ok) return fail(ctx, NEWT_E_INVALID, "geom size out of range for its shape");
  }
  // classify
  if (d.n_links > 0 && d.n_bodies == 0 && d.n_geoms == 0) { m.kind = GK_TREE; m.size = d.n_links; return NEWT_OK; }
  if (d.n_links == 0 && d.n_bodies > 0) {
    if (m.explicit_pairs)
      return fail(ctx, NEWT_E_INVALID, "explicit pair lists are taken on tree-contact worlds (pile worlds enumerate "
                                       "their pairs on the device)");
    // piles: one geom per body plus static planes
    std::vector<int> per_body(d.n_bodies, 0);
    int np = 0;
    for (int k = 0; k < d.n_geoms; ++k) {
      const newt_geom_desc& G = d.geoms[k];
      if (G.link >= 0) return fail(ctx, NEWT_E_INVALID, "link geom in a tree-less world");
      if (G.body >= 0) {
        if (G.body >= d.n_bodies) return fail(ctx, NEWT_E_INVALID, "geom body out of range");
        if (G.shape < NEWT_SHAPE_SPHERE || G.shape > NEWT_SHAPE_ELLIPSOID)
          return fail(ctx, NEWT_E_UNSUPPORTED_PAIR,
                      "free-body geoms must be spheres, boxes, capsules, cylinders or ellipsoids on the GPU path");
        per_body[G.body]++;
      } else {
        if (G.shape != NEWT_SHAPE_PLANE) return fail(ctx, NEWT_E_UNSUPPORTED_PAIR, "static geoms must be planes");
        ++np;
      }
      if (G.condim != 1 && G.condim != 3 && G.condim != 4 && G.condim != 6)
        return fail(ctx, NEWT_E_INVALID, "condim must be 1, 3, 4 or 6 (newt/src/solver.rs:1409-1428)");
      if (d.solver == NEWT_SOLVER_NEWTON && G.condim != 3)
        return fail(ctx, NEWT_E_INVALID, "pile worlds under the Newton solver take condim 3 on the GPU path");
    }
    if (d.solver == NEWT_SOLVER_NEWTON && d.cone != NEWT_CONE_PYRAMIDAL)
      return fail(ctx, NEWT_E_INVALID, "the Newton solver takes the pyramidal cone (newt/src/solver.rs:89-91)");
    // newt has no capsule-box primitive (newt/src/contact.rs:232-257) and
    // panics when such a pair is active; the pair is refused here instead
    for (int i = 0; i < d.n_geoms; ++i)
      for (int j = i + 1; j < d.n_geoms; ++j) {
        const newt_geom_desc &A = d.geoms[i], &B = d.geoms[j];
        if (A.body < 0 || B.body < 0) continue;
        const bool cb = (A.shape == NEWT_SHAPE_CAPSULE && B.shape == NEWT_SHAPE_BOX) ||
                        (A.shape == NEWT_SHAPE_BOX && B.shape == NEWT_SHAPE_CAPSULE);
        const bool sph_round = (A.shape == NEWT_SHAPE_SPHERE && (B.shape == NEWT_SHAPE_CYLINDER || B.shape == NEWT_SHAPE_ELLIPSOID)) ||
                               (B.shape == NEWT_SHAPE_SPHERE && (A.shape == NEWT_SHAPE_CYLINDER || A.shape == NEWT_SHAPE_ELLIPSOID));
        const bool round = !sph_round && (A.shape == NEWT_SHAPE_CYLINDER || A.shape == NEWT_SHAPE_ELLIPSOID ||
                                          B.shape == NEWT_SHAPE_CYLINDER || B.shape == NEWT_SHAPE_ELLIPSOID);
        if (!(cb || round) || !((A.group & B.mask) != 0u && (B.group & A.mask) != 0u)) continue;
        if (cb) return fail(ctx, NEWT_E_UNSUPPORTED_PAIR, "capsule-box pairs are not supported (newt/src/contact.rs:232-257)");
        // cylinders and ellipsoids touch planes and spheres here; newt routes
        // their other pairs through its convex solver (contact.rs:2509-2587)
        return fail(ctx, NEWT_E_UNSUPPORTED_PAIR,
                    "cylinder and ellipsoid bodies may collide with planes and spheres on the GPU path (filter the "
                    "other body pairs)");
      }
    for (int b = 0; b < d.n_bodies; ++b) {
      if (per_body[b] != 1) return fail(ctx, NEWT_E_INVALID, "GPU piles need exactly one geom per body");
      const float* I = d.bodies[b].inertia;  // column-major; Body::new inverts it (newt/src/body.rs)
      const double det = (double)I[0] * ((double)I[4] * I[8] - (double)I[7] * I[5]) -
                         (double)I[3] * ((double)I[1] * I[8] - (double)I[7] * I[2]) +
                         (double)I[6] * ((double)I[1] * I[5] - (double)I[4] * I[2]);
      if (!(d.bodies[b].mass > 0.f) || !(det > 0.0))
        return fail(ctx, NEWT_E_INVALID, "free bodies need a positive mass and an invertible inertia");
    }
    if (np > NEWT_MAX_PLANES) return fail(ctx, NEWT_E_INVALID, "too many planes");
    if (d.solver != NEWT_SOLVER_PGS && d.solver != NEWT_SOLVER_NEWTON)
      return fail(ctx, NEWT_E_INVALID, "GPU piles need the PGS or Newton solver");
    m.kind = GK_PILE; m.size = d.n_bodies; m.np = np;
    return NEWT_OK;
  }
  if (d.n_links > 0 && d.n_bodies == 0 && d.n_geoms > 0) {
    // one tree whose link geoms (spheres, boxes, capsules) touch static planes
    if (d.n_links > 64) return fail(ctx, NEWT_E_INVALID, "tree-contact worlds have at most 64 links");
    for (int k = 0; k < d.n_geoms; ++k) {
      const newt_geom_desc& G = d.geoms[k];
      if (G.body >= 0) return fail(ctx, NEWT_E_INVALID, "body geom in a world without free bodies");
      if (G.link >= d.n_links) return fail(ctx, NEWT_E_INVALID, "geom link out of range");
      if (G.link >= 0) {
        if (G.shape < NEWT_SHAPE_SPHERE || G.shape > NEWT_SHAPE_ELLIPSOID)
          return fail(ctx, NEWT_E_UNSUPPORTED_PAIR,
                      "link geoms must be spheres, boxes, capsules, cylinders or ellipsoids on the GPU path");
      } else if (G.shape != NEWT_SHAPE_PLANE) {
        return fail(ctx, NEWT_E_UNSUPPORTED_PAIR, "static geoms must be planes");
      }
      if (G.condim != 1 && G.condim != 3 && G.condim != 4 && G.condim != 6)
        return fail(ctx, NEWT_E_INVALID, "condim must be 1, 3, 4 or 6 (newt/src/solver.rs:1409-1428)");
    }
    if (d.solver == NEWT_SOLVER_NEWTON && d.cone != NEWT_CONE_PYRAMIDAL)
      return fail(ctx, NEWT_E_INVALID, "the Newton solver takes the pyramidal cone (newt/src/solver.rs:89-91)");
    // in-tree pairs (newt collides geoms of different links of one tree unless
    // its self-collision is off, world.rs:340, 1042-1069): the shape pairs
    // newt has a routine for, as on pile worlds, plus sphere-box
    // (an explicit pair list's in-tree pairs are collided whatever the
    // filters and the switch say)
    std::vector<std::pair<int, int>> in_tree;
    if (m.explicit_pairs) {
      in_tree = m.pairs;
    } else if (d.tree_self_collision) {
      for (int i = 0; i < d.n_geoms; ++i)
        for (int j = i + 1; j < d.n_geoms; ++j)
          if ((d.geoms[i].group & d.geoms[j].mask) != 0u && (d.geoms[j].group & d.geoms[i].mask) != 0u)
            in_tree.push_back({i, j});
    }
    for (const auto& pr : in_tree) {
      const newt_geom_desc &A = d.geoms[pr.first], &B = d.geoms[pr.second];
      if (A.link < 0 || B.link < 0) continue;
      if (A.link == B.link) {
        if (m.explicit_pairs) return fail(ctx, NEWT_E_UNSUPPORTED_PAIR, "pair_list names two geoms of one link");
        continue;
      }
      const int lo = std::min(A.shape, B.shape), hi = std::max(A.shape, B.shape);
      const bool ok = (lo == NEWT_SHAPE_SPHERE && hi <= NEWT_SHAPE_ELLIPSOID) ||
                      (lo == NEWT_SHAPE_BOX && hi == NEWT_SHAPE_BOX) ||
                      (lo == NEWT_SHAPE_CAPSULE && hi == NEWT_SHAPE_CAPSULE);
      if (!ok)
        return fail(ctx, NEWT_E_UNSUPPORTED_PAIR,
                    "in-tree pairs on the GPU path: sphere with sphere, box, capsule, cylinder or ellipsoid, box-box, "
                    "capsule-capsule (filter the others or disable tree self-collision)");
    }
    if (d.solver != NEWT_SOLVER_PGS && d.solver != NEWT_SOLVER_NEWTON)
      return fail(ctx, NEWT_E_INVALID, "tree-contact worlds need the PGS or Newton solver");
    m.kind = GK_TREE_CONTACT; m.size = d.n_links;
    return NEWT_OK;
  }
  return fail(ctx, NEWT_E_INVALID, "unsupported world class (mixed trees and free bodies)");
}

// ---------------------------------------------------------------------------
// groups
// ---------------------------------------------------------------------------
HostGroup* find_or_make_group(newt_gpu_ctx* ctx, HostModel& m) {
  if (m.group >= 0) return ctx->groups[m.group].get();
  if (m.key.empty()) m.key = m.topo_key();
  for (auto& g : ctx->groups)
    if (g->kind == m.kind && g->size == m.size && g->np == m.np && g->topo_key == m.key) {
      m.group = g->id;
      return g.get();
    }
  auto g = std::make_unique<HostGroup>();
  g->kind = m.kind; g->size = m.size; g->np = m.np; g->topo_key = m.key;
  g->nq = m.nq; g->nv = m.nv;
  g->maxc_cap = ctx->max_contacts;
  g->pile_newton = m.kind == GK_PILE && m.solver == NEWT_SOLVER_NEWTON;
  g->pile_general = m.kind == GK_PILE && !g->pile_newton && m.general_rows();
  if (m.kind == GK_TREE_CONTACT) g->setup_tc(m);
  g->id = (int)ctx->groups.size();
  m.group = g->id;
  ctx->groups.push_back(std::move(g));
  return ctx->groups.back().get();
}

extern "C" {

int newt_gpu_create(const newt_gpu_opts* opts, newt_gpu_ctx** out) {
  if (!out) return NEWT_E_INVALID;
  *out = nullptr;
  auto* ctx = new newt_gpu_ctx();
  ctx->device = opts ? opts->device : 0;
  ctx->max_worlds = opts && opts->max_worlds > 0 ? opts->max_worlds : (1 << 20);
  ctx->max_contacts = opts && opts->max_contacts > 0 ? opts->max_contacts : 0;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) { delete ctx; return NEWT_E_CUDA; }
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) { delete ctx; return NEWT_E_CUDA; }
  cudaEventCreate(&ctx->ev[0]);
  cudaEventCreate(&ctx->ev[1]);
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  uint64_t reserve = (uint64_t)2 << 30;
  ctx->budget = opts && opts->hbm_budget_bytes ? opts->hbm_budget_bytes : (fr > reserve ? fr - reserve : fr / 2);
  *out = ctx;
  return NEWT_OK;
}

int newt_gpu_destroy(newt_gpu_ctx* ctx) {
  if (!ctx) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (auto& g : ctx->groups) g->release();
  if (ctx->l2buf) cudaFree(ctx->l2buf);
  if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
  for (void* p : ctx->plan_bufs) cudaFree(p);
  for (void* p : ctx->plain_bufs) cudaFree(p);
  if (ctx->side) cudaStreamDestroy(ctx->side);
  for (int k = 0; k < 3; ++k) if (ctx->pside[k]) cudaStreamDestroy(ctx->pside[k]);
  for (int k = 0; k < 4; ++k) if (ctx->pev[k]) cudaEventDestroy(ctx->pev[k]);
  for (int b = 0; b < newt_gpu_ctx::PILE_BRANCHES; ++b) {
    for (int k = 0; k < 4; ++k) if (ctx->pbs[b][k]) cudaStreamDestroy(ctx->pbs[b][k]);
    for (int k = 0; k < 5; ++k) if (ctx->pbe[b][k]) cudaEventDestroy(ctx->pbe[b][k]);
  }
  for (int k = 0; k < 2; ++k) if (ctx->fkev[k]) cudaEventDestroy(ctx->fkev[k]);
  if (ctx->fused_work) cudaFree(ctx->fused_work);
  if (ctx->tcstream) cudaStreamDestroy(ctx->tcstream);
  for (cudaEvent_t e : ctx->kev) cudaEventDestroy(e);
  for (cudaEvent_t e : ctx->tcev) cudaEventDestroy(e);
  if (ctx->io_h) cudaFreeHost(ctx->io_h);
  if (ctx->io_d) cudaFree(ctx->io_d);
  if (ctx->ctrl_arena) cudaFree(ctx->ctrl_arena);
  if (ctx->ctrl_dev) cudaFree(ctx->ctrl_dev);
  cudaEventDestroy(ctx->ev[0]);
  cudaEventDestroy(ctx->ev[1]);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return NEWT_OK;
}

const char* newt_gpu_last_error(const newt_gpu_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int newt_gpu_upload_models(newt_gpu_ctx* ctx, const newt_model_desc* models, int32_t n, int32_t* ids) {
  if (!ctx || !models || n < 0) return NEWT_E_INVALID;
  for (int i = 0; i < n; ++i) {
    HostModel m;
    int rc = classify(ctx, models[i], m);
    if (rc != NEWT_OK) return rc;
    ctx->models.push_back(std::move(m));
    if (ids) ids[i] = (int32_t)ctx->models.size() - 1;
  }
  return NEWT_OK;
}

int newt_gpu_model_dims(const newt_gpu_ctx* ctx, int32_t id, int32_t* nq, int32_t* nv) {
  if (!ctx || id < 0 || id >= (int)ctx->models.size()) return NEWT_E_INVALID;
  if (nq) *nq = ctx->models[id].nq;
  if (nv) *nv = ctx->models[id].nv;
  return NEWT_OK;
}

// Returns live slots to the free lists and clears their worlds' live flags
// on the device (one launch for the whole list).
static int release_slots(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n) {
  std::vector<int*> flags;
  flags.reserve(n);
  for (int i = 0; i < n; ++i) {
    SlotRef& r = ctx->slots[slots[i]];
    flags.push_back(ctx->groups[r.group]->release_index(r.index));
    r.live = false;
    ctx->free_slots.push_back(slots[i]);
    ctrl_release_slot(ctx, slots[i]);
  }
  return io_clear_flags(ctx, flags);
}

int newt_gpu_alloc_worlds(newt_gpu_ctx* ctx, const int32_t* model_ids, int32_t n, int32_t* slots_out) {
  if (!ctx || !model_ids || n < 0) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  // a captured step graph covers every group up to its high-water mark and
  // skips worlds that are not live, so it stays valid unless a group is
  // created or grows
  const size_t groups_before = ctx->groups.size();
  std::vector<std::pair<int, int>> extent;
  for (auto& g : ctx->groups) extent.push_back({g->n, g->cap});
  // group the request so each group grows at most once
  std::map<int, std::vector<int>> by_group;
  for (int i = 0; i < n; ++i) {
    int id = model_ids[i];
    if (id < 0 || id >= (int)ctx->models.size()) return fail(ctx, NEWT_E_INVALID, "bad model id");
    HostGroup* g = find_or_make_group(ctx, ctx->models[id]);
    by_group[g->id].push_back(i);
  }
  // all or nothing: a group that cannot grow undoes the worlds this call
  // already placed in other groups
  std::vector<int32_t> placed;
  auto finish = [&](int rc) {
    bool grew = ctx->groups.size() != groups_before;
    for (size_t k = 0; k < extent.size() && !grew; ++k)
      grew = ctx->groups[k]->n != extent[k].first || ctx->groups[k]->cap != extent[k].second;
    if (grew) {
      ctx->graph_dirty = true;
      ctx->plain_dirty = true;
      ctx->ctrl_dirty = true;  // control streams point into the groups' rows
    }
    return rc;
  };
  auto undo = [&](int rc) {
    int rc2 = release_slots(ctx, placed.data(), (int32_t)placed.size());
    return finish(rc != NEWT_OK ? rc : rc2);
  };
  for (auto& kv : by_group) {
    HostGroup* g = ctx->groups[kv.first].get();
    std::vector<int> idx;
    int rc = g->reserve_indices(ctx, (int)kv.second.size(), idx);
    if (rc != NEWT_OK) return undo(rc);
    for (size_t k = 0; k < kv.second.size(); ++k) {
      int req = kv.second[k];
      int slot = (int)ctx->slots.size();
      if (!ctx->free_slots.empty()) { slot = ctx->free_slots.back(); ctx->free_slots.pop_back(); }
      else ctx->slots.push_back(SlotRef{});
      ctx->slots[slot] = SlotRef{g->id, idx[k], model_ids[req], true};
      g->write_model(ctx, idx[k], ctx->models[model_ids[req]]);
      g->slot_of[idx[k]] = slot;
      if (slots_out) slots_out[req] = slot;
      placed.push_back(slot);
    }
    rc = g->flush_model(ctx);
    if (rc != NEWT_OK) return undo(rc);
    if (g->kind == GK_TREE_CONTACT && g->plain_scratch) {
      // a new world has no contacts until it steps: the contact sensors'
      // re-solve reads the slot's stored contact count.  Indices past the
      // scratch's current extent (the group grew) get a zeroed scratch when
      // it is next sized.
      int o_con, o_imp, o_misc;
      newt_tc_offsets(g->size, g->nv, g->ng, g->maxc, g->tc_rpc, &o_con, &o_imp, &o_misc);
      const size_t held = g->scr_stride > 0 ? g->plain_scratch_bytes / (sizeof(float) * (size_t)g->scr_stride) : 0;
      for (int i : idx)
        if ((size_t)i < held && cudaMemsetAsync((float*)g->plain_scratch + (size_t)i * g->scr_stride + o_misc, 0,
                                                sizeof(int), ctx->stream) != cudaSuccess)
          return undo(fail(ctx, NEWT_E_CUDA, "alloc_worlds: clearing the contact list"));
    }
  }
  return finish(NEWT_OK);
}

int newt_gpu_free_worlds(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n) {
  if (!ctx || (n > 0 && !slots)) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  for (int i = 0; i < n; ++i) {
    int s = slots[i];
    if (s < 0 || s >= (int)ctx->slots.size() || !ctx->slots[s].live) return fail(ctx, NEWT_E_INVALID, "bad slot");
    for (int j = 0; j < i; ++j)
      if (slots[j] == s) return fail(ctx, NEWT_E_INVALID, "slot named twice");
  }
  // the freed worlds' live flags are cleared on the device; captured graphs
  // and plain tables skip them, so neither needs rebuilding
  return release_slots(ctx, slots, n);
}

int newt_gpu_hold_worlds(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n) {
  if (!ctx || (n > 0 && !slots) || n < 0) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  std::vector<int*> flags;
  flags.reserve(n);
  for (int i = 0; i < n; ++i) {
    const int s = slots[i];
    if (s < 0 || s >= (int)ctx->slots.size() || !ctx->slots[s].live) return fail(ctx, NEWT_E_INVALID, "bad slot");
    const SlotRef& r = ctx->slots[s];
    flags.push_back(ctx->groups[r.group]->live_flag(r.index));
  }
  return io_hold_flags(ctx, flags);
}

// Collects, per group, the worlds a call names (in call order), checking
// every slot first.
static int group_worlds(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n, std::vector<std::vector<int>>& by_group) {
  by_group.assign(ctx->groups.size(), {});
  for (int i = 0; i < n; ++i) {
    int s = slots[i];
    if (s < 0 || s >= (int)ctx->slots.size() || !ctx->slots[s].live) return fail(ctx, NEWT_E_INVALID, "bad slot");
    by_group[ctx->slots[s].group].push_back(ctx->slots[s].index);
  }
  return NEWT_OK;
}

enum RowSet { ROWS_QFRC, ROWS_QACC };

static std::vector<RowMove> moves_for(newt_gpu_ctx* ctx, std::vector<std::vector<int>>& by_group, RowSet set) {
  std::vector<RowMove> mv;
  for (size_t gi = 0; gi < by_group.size(); ++gi) {
    if (by_group[gi].empty()) continue;
    HostGroup* g = ctx->groups[gi].get();
    size_t lo = 0, cnt = 0;
    if (!g->soa()) continue;  // free-body piles carry no generalised force or acceleration rows
    lo = set == ROWS_QFRC ? g->r_qfrc : g->r_qacc;
    cnt = g->nv;
    mv.push_back(RowMove{g, std::move(by_group[gi]), lo, cnt});
  }
  return mv;
}

// State goes in and out in MuJoCo layout, one copy each way, converted on the
// device (world_io.cu); only the named worlds' rows change.  The host
// mirror's state rows are not kept: every reader gathers from the device.
int newt_gpu_set_state(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n, const float* qpos, const float* qvel) {
  if (!ctx || (n > 0 && (!slots || !qpos || !qvel))) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  std::vector<std::vector<int>> by_group;
  int rc = group_worlds(ctx, slots, n, by_group);
  if (rc != NEWT_OK) return rc;
  std::vector<char> seen(ctx->slots.size(), 0);
  for (int i = 0; i < n; ++i) {
    if (seen[slots[i]]) return fail(ctx, NEWT_E_INVALID, "slot named twice");
    seen[slots[i]] = 1;
  }
  return io_state_in(ctx, slots, n, qpos, qvel);
}

int newt_gpu_get_state(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n, float* qpos, float* qvel) {
  if (!ctx || (n > 0 && (!slots || !qpos || !qvel))) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  std::vector<std::vector<int>> by_group;
  int rc = group_worlds(ctx, slots, n, by_group);
  if (rc != NEWT_OK) return rc;
  return io_state_out(ctx, slots, n, qpos, qvel);
}

int newt_gpu_set_qfrc(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n, const float* qfrc) {
  if (!ctx || (n > 0 && (!slots || !qfrc))) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  std::vector<std::vector<int>> by_group;
  int rc = group_worlds(ctx, slots, n, by_group);
  if (rc != NEWT_OK) return rc;
  long vo = 0;
  for (int i = 0; i < n; ++i) {
    const SlotRef& r = ctx->slots[slots[i]];
    const HostModel& m = ctx->models[r.model];
    ctx->groups[r.group]->stage_qfrc(r.index, m, qfrc + vo);
    vo += m.nv;
  }
  return io_scatter(ctx, moves_for(ctx, by_group, ROWS_QFRC));
}

int newt_gpu_step(newt_gpu_ctx* ctx, int32_t n_steps, int32_t mode) {
  if (!ctx || n_steps < 0) return NEWT_E_INVALID;
  if (n_steps == 0) return NEWT_OK;
  cudaSetDevice(ctx->device);
  int rc = mode == NEWT_STEP_PLAIN ? step_plain(ctx, n_steps) : step_batched(ctx, n_steps);
  if (rc != NEWT_OK) return rc;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(ctx, NEWT_E_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return NEWT_OK;
}

int newt_gpu_sync(newt_gpu_ctx* ctx, int32_t timeout_ms) {
  if (!ctx) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t e = cudaStreamQuery(ctx->stream);
    if (e == cudaSuccess) return NEWT_OK;
    if (e != cudaErrorNotReady) return fail(ctx, NEWT_E_CUDA, cudaGetErrorString(e));
    double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (timeout_ms >= 0 && ms > timeout_ms) return fail(ctx, NEWT_E_TIMEOUT, "stream did not drain in time");
    std::this_thread::yield();
  }
}

int newt_gpu_world_status(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n, uint32_t* status, int32_t clear) {
  if (!ctx || (n > 0 && (!slots || !status))) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  for (auto& g : ctx->groups) { int rc = g->fetch_status(ctx); if (rc != NEWT_OK) return rc; }
  for (int i = 0; i < n; ++i) {
    int s = slots[i];
    if (s < 0 || s >= (int)ctx->slots.size() || !ctx->slots[s].live) return fail(ctx, NEWT_E_INVALID, "bad slot");
    status[i] = ctx->groups[ctx->slots[s].group]->status_host[ctx->slots[s].index];
  }
  if (clear) for (auto& g : ctx->groups) { int rc = g->clear_status(ctx); if (rc != NEWT_OK) return rc; }
  return NEWT_OK;
}

int newt_gpu_get_qacc(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n, float* qacc) {
  if (!ctx || (n > 0 && (!slots || !qacc))) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  std::vector<std::vector<int>> by_group;
  int rc = group_worlds(ctx, slots, n, by_group);
  if (rc != NEWT_OK) return rc;
  rc = io_gather(ctx, moves_for(ctx, by_group, ROWS_QACC));
  if (rc != NEWT_OK) return rc;
  long vo = 0;
  for (int i = 0; i < n; ++i) {
    const SlotRef& r = ctx->slots[slots[i]];
    const HostModel& m = ctx->models[r.model];
    ctx->groups[r.group]->read_qacc(r.index, m, qacc + vo);
    vo += m.nv;
  }
  return NEWT_OK;
}

int newt_gpu_get_contacts(newt_gpu_ctx* ctx, int32_t slot, int32_t cap, int32_t* n_out, int32_t* pairs, float* data) {
  if (!ctx || slot < 0 || slot >= (int)ctx->slots.size() || !ctx->slots[slot].live || !n_out) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  const SlotRef& r = ctx->slots[slot];
  return ctx->groups[r.group]->read_contacts(ctx, r.index, cap, n_out, pairs, data);
}

int newt_gpu_get_impulses(newt_gpu_ctx* ctx, int32_t slot, int32_t cap, int32_t* n_out, float* imp) {
  if (!ctx || slot < 0 || slot >= (int)ctx->slots.size() || !ctx->slots[slot].live || !n_out) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  const SlotRef& r = ctx->slots[slot];
  return ctx->groups[r.group]->read_impulses(ctx, r.index, cap, n_out, imp);
}

int newt_gpu_event_record(newt_gpu_ctx* ctx, int32_t which) {
  if (!ctx || which < 0 || which > 1) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  CK(cudaEventRecord(ctx->ev[which], ctx->stream));
  return NEWT_OK;
}

int newt_gpu_event_elapsed_ms(newt_gpu_ctx* ctx, float* ms) {
  if (!ctx || !ms) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  CK(cudaEventSynchronize(ctx->ev[1]));
  CK(cudaEventElapsedTime(ms, ctx->ev[0], ctx->ev[1]));
  return NEWT_OK;
}

int newt_gpu_flush_l2(newt_gpu_ctx* ctx) {
  if (!ctx) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  const size_t bytes = (size_t)256 << 20;  // 256 MiB > 129 MB L2
  if (!ctx->l2buf) CK(cudaMalloc(&ctx->l2buf, bytes));
  CK(cudaMemsetAsync(ctx->l2buf, ctx->l2flip++ & 1, bytes, ctx->stream));
  return NEWT_OK;
}

int64_t newt_gpu_launch_count(const newt_gpu_ctx* ctx) { return ctx ? ctx->launches : -1; }

int newt_gpu_autotune(newt_gpu_ctx* ctx, int32_t n_steps, int32_t horizon, int32_t* choice) {
  if (!ctx || n_steps <= 0) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  int rc = autotune_batched(ctx, n_steps, horizon > 0 ? horizon : 8 * n_steps, choice);
  if (rc != NEWT_OK && ctx->err.empty()) ctx->err = "autotune failed";
  return rc;
}

extern "C" int newt_pile_fused_shapes();

int newt_gpu_set_launch_choice(newt_gpu_ctx* ctx, const int32_t* choice) {
  if (!ctx || !choice) return NEWT_E_INVALID;
  const int branches = choice[0], tree_pct = choice[1], fused = choice[3], shape = choice[4];
  if (branches < 0 || branches > newt_gpu_ctx::PILE_BRANCHES || tree_pct < 1 || tree_pct > 100 || fused < 0 ||
      fused > 1 || shape < 0 || shape >= newt_pile_fused_shapes()) {
    ctx->err = "newt_gpu_set_launch_choice: pile branches 0..3, tree grid percent 1..100, persistent flag 0 or 1, "
               "persistent shape 0.." + std::to_string(newt_pile_fused_shapes() - 1);
    return NEWT_E_INVALID;
  }
  ctx->tune_branches = branches;
  ctx->tune_tree_grid_pct = tree_pct;
  ctx->tune_pile_fused = fused;
  ctx->tune_fused_shape = shape;
  ctx->graph_dirty = true;
  return NEWT_OK;
}

int newt_gpu_memory(const newt_gpu_ctx* ctx, uint64_t* used, uint64_t* budget) {
  if (!ctx) return NEWT_E_INVALID;
  if (used) *used = ctx->used;
  if (budget) *budget = ctx->budget;
  return NEWT_OK;
}

int newt_gpu_tc_profile(newt_gpu_ctx* ctx, float* kernel_ms) {
  if (!ctx || !kernel_ms) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  int rc = newt_gpu_sync(ctx, 600000);
  if (rc != NEWT_OK) return rc;
  for (int k = 0; k < NEWT_TC_KERNELS; ++k) kernel_ms[k] = 0.f;
  for (int s = 0; s < ctx->tcev_steps; ++s)
    for (int k = 0; k < NEWT_TC_KERNELS; ++k) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, ctx->tcev[(size_t)6 * s + 2 * k], ctx->tcev[(size_t)6 * s + 2 * k + 1]));
      kernel_ms[k] += ms;
    }
  return NEWT_OK;
}

int newt_gpu_pile_profile(newt_gpu_ctx* ctx, int32_t enable, float* kernel_ms, int32_t* work, int32_t* launches) {
  if (!ctx) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  if (enable >= 0 && (enable != 0) != ctx->profile) {
    ctx->profile = enable != 0;
    ctx->graph_dirty = true;  // recapture with (or without) the event nodes
  }
  if (launches) *launches = ctx->kev_steps * ctx->kev_branches;
  if (!kernel_ms && !work) return NEWT_OK;
  int rc = newt_gpu_sync(ctx, 600000);
  if (rc != NEWT_OK) return rc;
  const int K = NEWT_PILE_KERNELS;
  if (kernel_ms) {
    for (int k = 0; k < K; ++k) kernel_ms[k] = 0.f;
    for (int s = 0; s < ctx->kev_steps * ctx->kev_branches; ++s)
      for (int k = 0; k < K; ++k) {
        float ms = 0.f;
        const size_t e = (size_t)2 * (K * s + k);
        CK(cudaEventElapsedTime(&ms, ctx->kev[e], ctx->kev[e + 1]));
        kernel_ms[k] += ms;
      }
  }
  if (work) {
    const int C = NEWT_PILE_ISLAND_CLASSES, n = 3 * C;
    for (int k = 0; k < n; ++k) work[k] = 0;
    for (const auto& l : ctx->last_lists) {
      int32_t h[3 * NEWT_PILE_ISLAND_CLASSES];
      CK(cudaMemcpy(h, l.first + (size_t)C * l.second, sizeof(h), cudaMemcpyDeviceToHost));
      for (int k = 0; k < n; ++k) work[k] += h[k];
    }
  }
  return NEWT_OK;
}

int newt_gpu_pile_fused_profile(newt_gpu_ctx* ctx, float* kernel_ms, uint64_t* work) {
  if (!ctx) return NEWT_E_INVALID;
  cudaSetDevice(ctx->device);
  int rc = newt_gpu_sync(ctx, 600000);
  if (rc != NEWT_OK) return rc;
  if (kernel_ms) {
    *kernel_ms = 0.f;
    if (ctx->last_fused && ctx->profile && ctx->fkev[0]) CK(cudaEventElapsedTime(kernel_ms, ctx->fkev[0], ctx->fkev[1]));
  }
  if (work) {
    for (int k = 0; k < 4; ++k) work[k] = 0;
    if (ctx->last_fused && ctx->fused_work)
      CK(cudaMemcpy(work, ctx->fused_work, 4 * sizeof(uint64_t), cudaMemcpyDeviceToHost));
  }
  return NEWT_OK;
}

}  // extern "C"
