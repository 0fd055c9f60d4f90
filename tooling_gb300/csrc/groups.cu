// World-group storage: row layouts, host mirrors, growth, model/state
// staging and MuJoCo <-> newt state conversion
// (newt/src/world.rs:519-623 apply_mujoco_qpos/qvel;
//  newt/tests/differential.rs:548-640 the inverse mapping).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "runtime.h"

#define CKG(call)                                                               \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) { ctx->err = std::string(#call ": ") + cudaGetErrorString(e_); return NEWT_E_CUDA; } \
  } while (0)

static void sym6(const float m9[9], float* o) {  // column-major 3x3 -> xx yy zz xy xz yz
  o[0] = m9[0]; o[1] = m9[4]; o[2] = m9[8]; o[3] = m9[3]; o[4] = m9[6]; o[5] = m9[7];
}
static bool inv6(const float m9[9], float* o) {
  double a = m9[0], b = m9[3], c = m9[6], d = m9[1], e = m9[4], f = m9[7], g = m9[2], h = m9[5], i = m9[8];
  double det = a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
  if (det == 0.0 || !std::isfinite(det)) return false;
  double inv = 1.0 / det;
  o[0] = (float)((e * i - f * h) * inv); o[1] = (float)((a * i - c * g) * inv); o[2] = (float)((a * e - b * d) * inv);
  o[3] = (float)((c * h - b * i) * inv); o[4] = (float)((b * f - c * e) * inv); o[5] = (float)((c * d - a * f) * inv);
  return true;
}

// ---------------------------------------------------------------------------
// layout
// ---------------------------------------------------------------------------
static void tree_rows(HostGroup& g) {
  const int L = g.size;
  size_t r = 0;
  g.r_axis = r; r += 3 * L;
  g.r_jp = r; r += 3 * L;
  g.r_jc = r; r += 3 * L;
  g.r_rootq = r; r += 4;
  g.r_mass = r; r += L;
  g.r_inert = r; r += 6 * L;
  g.r_damp = r; r += L;
  g.r_arm = r; r += L;
  g.r_dtg = r; r += 4;
  g.r_q = r; r += g.nq;
  g.r_qd = r; r += g.nv;
  g.r_qfrc = r; r += g.nv;
  g.r_qacc = r; r += g.nv;
  g.ri_solver = 0; g.ri_live = 1; g.ri_status = 2;
  g.irows = 3;
  if (g.kind == GK_TREE) {  // integrator per world (tree-contact groups: row 5)
    g.ri_integ = 3;
    g.irows = 4;
  }
  if (g.kind == GK_TREE_CONTACT) {  // per-geom model rows (TcGroupDev::geom), solver mode
    g.r_geom = r; r += 22 * g.ng;
    g.ri_mode = 3; g.ri_iters = 4; g.ri_integ = 5;
    g.irows = 6;
  }
  g.frows = r;
}

static int pile_maxc(int nb, int np) {
  int c = 6 * nb + 4 * nb * np;
  c = (c + 31) / 32 * 32;
  return std::min(std::max(c, 64), 512);
}

static void pile_rows(HostGroup& g) {
  const int nb = g.size, np = g.np, ng = nb + np;
  g.maxc = pile_maxc(nb, np);
  if (g.maxc_cap > 0)  // the context's cap, rounded up to a multiple of 32
    g.maxc = std::min(g.maxc, (g.maxc_cap + 31) / 32 * 32);
  PileLayout& l = g.lay;
  int r = 0;
  l.mass = r; r += nb;
  l.inert = r; r += 6 * nb;
  l.iinv = r; r += 6 * nb;
  l.size = r; r += 3 * nb;
  l.gpos = r; r += 3 * nb;
  l.gquat = r; r += 4 * nb;
  l.fric = r; r += ng;
  l.margin = r; r += ng;
  l.tfric = r; r += ng;
  l.rfric = r; r += ng;
  l.soft = r; r += 7;
  l.plane = r; r += 7 * np;
  l.dtg = r; r += 4;
  r = (r + 3) / 4 * 4;
  l.pos = r; r += 3 * nb;
  l.quat = r; r += 4 * nb;
  l.vel = r; r += 3 * nb;
  l.omg = r; r += 3 * nb;
  r = (r + 3) / 4 * 4;
  l.cdata = r; r += 7 * g.maxc;
  l.rpc = g.pile_general ? 6 : 4;
  l.imp = r; r += l.rpc * g.maxc;
  r = (r + 31) / 32 * 32;
  l.fstride = r;
  int q = 0;
  l.shape = q; q += nb;
  l.gent = q; q += ng;
  l.iters = q; q += 1;
  l.status = q; q += 1;
  l.ncon = q; q += 1;
  l.live = q; q += 1;
  l.integ = q; q += 1;
  l.gcond = q; q += ng;
  l.cone = q; q += 1;
  l.cpair = q; q += 2 * g.maxc;
  q = (q + 31) / 32 * 32;
  l.istride = q;
  g.frows = l.fstride;
  g.irows = l.istride;
}

// Model and state rows plus the world's solver scratch (counted against the
// admission budget; the scratch itself is allocated at the first step).
size_t HostGroup::bytes_per_world() const {
  size_t b = frows * sizeof(float) + irows * sizeof(int);
  if (kind == GK_PILE) b += newt_pile_ws_bytes(size, np, maxc);
  if (kind == GK_PILE && pile_newton) b += newt_pile_newton_bytes(maxc);
  if (kind == GK_TREE_CONTACT) b += newt_tc_ws_bytes(size, nv, ng, maxc, tc_rpc);
  return b;
}

// ---------------------------------------------------------------------------
// capacity
// ---------------------------------------------------------------------------
static int grow(newt_gpu_ctx* ctx, HostGroup& g, int need) {
  if (g.frows == 0) {
    if (g.soa()) tree_rows(g);
    else if (g.kind == GK_PILE) pile_rows(g);
  }
  if (need <= g.cap) return NEWT_OK;
  int ncap = std::max(need, std::max(64, g.cap * 2));
  if (ncap > ctx->max_worlds) ncap = std::max(need, ctx->max_worlds);
  const uint64_t bpw = g.bytes_per_world();
  if (ctx->used + (uint64_t)(ncap - g.cap) * bpw > ctx->budget) {
    // short of the doubling: take what the rest of the budget holds
    const uint64_t room = ctx->budget > ctx->used ? (ctx->budget - ctx->used) / bpw : 0;
    ncap = (int)std::min<uint64_t>((uint64_t)ncap, (uint64_t)g.cap + room);
    if (ncap < need) {
      ctx->err = "HBM admission budget exhausted";
      return NEWT_E_NOMEM;
    }
  }
  std::vector<float> nF(g.frows * (size_t)ncap, 0.f);
  std::vector<int> nI(g.irows * (size_t)ncap, 0);
  if (g.soa()) {
    for (size_t r = 0; r < g.frows; ++r)
      for (int w = 0; w < g.cap; ++w) nF[r * ncap + w] = g.hF[r * g.cap + w];
    for (size_t r = 0; r < g.irows; ++r)
      for (int w = 0; w < g.cap; ++w) nI[r * ncap + w] = g.hI[r * g.cap + w];
  } else {
    std::copy(g.hF.begin(), g.hF.end(), nF.begin());
    std::copy(g.hI.begin(), g.hI.end(), nI.begin());
  }
  // device: pull the current device contents into the new host mirror first
  if (g.dF && g.n > 0) {
    std::vector<float> cur(g.frows * (size_t)g.cap);
    std::vector<int> curI(g.irows * (size_t)g.cap);
    CKG(cudaStreamSynchronize(ctx->stream));
    CKG(cudaMemcpy(cur.data(), g.dF, cur.size() * sizeof(float), cudaMemcpyDeviceToHost));
    CKG(cudaMemcpy(curI.data(), g.dI, curI.size() * sizeof(int), cudaMemcpyDeviceToHost));
    if (g.soa()) {
      for (size_t r = 0; r < g.frows; ++r)
        for (int w = 0; w < g.cap; ++w) nF[r * ncap + w] = cur[r * g.cap + w];
      for (size_t r = 0; r < g.irows; ++r)
        for (int w = 0; w < g.cap; ++w) nI[r * ncap + w] = curI[r * g.cap + w];
    } else {
      std::copy(cur.begin(), cur.end(), nF.begin());
      std::copy(curI.begin(), curI.end(), nI.begin());
    }
  }
  if (g.dF) { cudaFree(g.dF); cudaFree(g.dI); ctx->used -= (uint64_t)g.cap * g.bytes_per_world(); }
  g.dF = nullptr; g.dI = nullptr;
  CKG(cudaMalloc(&g.dF, nF.size() * sizeof(float)));
  CKG(cudaMalloc(&g.dI, nI.size() * sizeof(int)));
  ctx->used += (uint64_t)ncap * g.bytes_per_world();
  // the host mirrors are the staging buffers of every state copy: page-lock
  // them so host<->device transfers run at full link rate
  if (!g.hF.empty()) cudaHostUnregister(g.hF.data());
  if (!g.hI.empty()) cudaHostUnregister(g.hI.data());
  g.hF.swap(nF);
  g.hI.swap(nI);
  cudaHostRegister(g.hF.data(), g.hF.size() * sizeof(float), cudaHostRegisterDefault);
  cudaHostRegister(g.hI.data(), g.hI.size() * sizeof(int), cudaHostRegisterDefault);
  cudaGetLastError();  // registration is an optimisation; ignore a refusal
  g.cap = ncap;
  g.slot_of.resize(ncap, -1);
  g.status_host.resize(ncap, 0);
  CKG(cudaMemcpyAsync(g.dF, g.hF.data(), g.hF.size() * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  CKG(cudaMemcpyAsync(g.dI, g.hI.data(), g.hI.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  CKG(cudaStreamSynchronize(ctx->stream));
  ctx->graph_dirty = true;
  ctx->plain_dirty = true;
  return NEWT_OK;
}

int HostGroup::reserve_indices(newt_gpu_ctx* ctx, int k, std::vector<int>& out) {
  out.clear();
  while ((int)out.size() < k && !free_idx.empty()) { out.push_back(free_idx.back()); free_idx.pop_back(); }
  int extra = k - (int)out.size();
  if (extra > 0) {
    int rc = grow(ctx, *this, n + extra);
    if (rc != NEWT_OK) {
      for (int i : out) free_idx.push_back(i);
      return rc;
    }
    for (int i = 0; i < extra; ++i) out.push_back(n + i);
    n += extra;
  }
  return NEWT_OK;
}

int* HostGroup::live_flag(int idx) {
  const int lrow = soa() ? ri_live : lay.live;
  return soa() ? dI + (size_t)lrow * cap + idx : dI + (size_t)idx * irows + lrow;
}

int* HostGroup::release_index(int idx) {
  int lrow = soa() ? ri_live : lay.live;
  I(lrow, idx) = 0;
  slot_of[idx] = -1;
  free_idx.push_back(idx);
  return soa() ? dI + (size_t)lrow * cap + idx : dI + (size_t)idx * irows + lrow;  // the device live flag
}

// Geom topology, candidate pairs and contact capacity of a tree-contact
// group, fixed by its first model (the topology key makes them uniform).
void HostGroup::setup_tc(const HostModel& m) {
  ng = m.n_geoms;
  // (static, link geom) pairs and, with the tree's self-collision on, the
  // pairs of geoms on different links, in newt's auto_pairs order with its
  // filter (world.rs:1042-1069)
  gtopo.assign(3 * ng, 0);
  tc_rpc = 4;
  tc_cone = m.cone;
  tc_general = m.cone != NEWT_CONE_PYRAMIDAL;
  for (int k = 0; k < ng; ++k) {
    gtopo[2 * k] = m.geoms[k].shape;
    gtopo[2 * k + 1] = m.geoms[k].link;
    gtopo[2 * ng + k] = m.geoms[k].condim;
    if (m.geoms[k].condim == 6) tc_rpc = 6;  // normal, tangent pair, torsion, rolling pair
    if (m.geoms[k].condim == 4 || m.geoms[k].condim == 6) tc_general = true;
  }
  gpairs.clear();
  maxc = 0;
  // World::pair_list, in its order and past the filters, or newt's
  // automatic pairs
  std::vector<std::pair<int, int>> cand;
  if (m.explicit_pairs) {
    cand = m.pairs;
  } else {
    for (int a = 0; a < ng; ++a)
      for (int b = a + 1; b < ng; ++b) {
        const newt_geom_desc &A = m.geoms[a], &B = m.geoms[b];
        if (A.link >= 0 && B.link >= 0 && (!m.self_coll || A.link == B.link)) continue;
        if (!((A.group & B.mask) != 0u && (B.group & A.mask) != 0u)) continue;
        cand.push_back({a, b});
      }
  }
  for (const auto& pr : cand) {
      const int a = pr.first, b = pr.second;
      const newt_geom_desc &A = m.geoms[a], &B = m.geoms[b];
      if (A.link < 0 && B.link < 0) continue;  // two static geoms: no routine, no rows
      const bool in_tree = A.link >= 0 && B.link >= 0;
      gpairs.push_back(a);
      gpairs.push_back(b);
      if (in_tree) {  // box-box up to four contacts, capsule-capsule two, sphere pairs one
        maxc += (A.shape == NEWT_SHAPE_BOX && B.shape == NEWT_SHAPE_BOX) ? 4
              : (A.shape == NEWT_SHAPE_CAPSULE && B.shape == NEWT_SHAPE_CAPSULE) ? 2 : 1;
        continue;
      }
      const int shape = A.link >= 0 ? A.shape : B.shape;
      maxc += (shape == NEWT_SHAPE_BOX || shape == NEWT_SHAPE_CYLINDER) ? 4 : (shape == NEWT_SHAPE_CAPSULE ? 2 : 1);
    }
  npairs = (int)gpairs.size() / 2;
  if (maxc < 1) maxc = 1;
  // tree structure for the mass matrix: per link its subtree (itself and its
  // descendants) as a 64-bit mask (two ints), then the link of every DoF
  const int L = m.n_links;
  std::vector<unsigned long long> desc(L, 0ull);
  for (int l = L - 1; l >= 0; --l) {
    desc[l] |= 1ull << l;
    if (m.links[l].parent >= 0) desc[m.links[l].parent] |= desc[l];
  }
  for (int l = 0; l < L; ++l) {
    gtopo.push_back((int)(unsigned)(desc[l] & 0xffffffffull));
    gtopo.push_back((int)(unsigned)(desc[l] >> 32));
  }
  for (int l = 0; l < L; ++l) {
    const int jt = m.links[l].joint;
    const int nd = jt == NEWT_JOINT_FREE ? 6 : (jt == NEWT_JOINT_FIXED ? 0 : 1);
    for (int k = 0; k < nd; ++k) gtopo.push_back(l);
  }
}

// ---------------------------------------------------------------------------
// model staging
// ---------------------------------------------------------------------------
void HostGroup::write_model(newt_gpu_ctx*, int w, const HostModel& m) {
  if (soa()) {
    const int L = size;
    if (topo.empty()) {
      topo.assign(4 * L, 0);
      int qo = 0, vo = 0;
      for (int i = 0; i < L; ++i) {
        int jt = m.links[i].joint;
        topo[4 * i] = m.links[i].parent; topo[4 * i + 1] = jt; topo[4 * i + 2] = qo; topo[4 * i + 3] = vo;
        qo += jt == NEWT_JOINT_FREE ? 7 : (jt == NEWT_JOINT_FIXED ? 0 : 1);
        vo += jt == NEWT_JOINT_FREE ? 6 : (jt == NEWT_JOINT_FIXED ? 0 : 1);
      }
    }
    for (int i = 0; i < L; ++i) {
      const newt_link_desc& l = m.links[i];
      for (int k = 0; k < 3; ++k) { F(r_axis + 3 * i + k, w) = l.axis[k]; F(r_jp + 3 * i + k, w) = l.jp_pos[k]; F(r_jc + 3 * i + k, w) = l.jc_pos[k]; }
      F(r_mass + i, w) = l.mass;
      float s6[6]; sym6(l.inertia, s6);
      for (int k = 0; k < 6; ++k) F(r_inert + 6 * i + k, w) = s6[k];
      F(r_damp + i, w) = i == 0 ? l.free_damping : l.damping;
      F(r_arm + i, w) = l.armature;
    }
    for (int k = 0; k < 4; ++k) F(r_rootq + k, w) = m.links[0].jp_quat[k];
    F(r_dtg, w) = m.dt; F(r_dtg + 1, w) = m.g[0]; F(r_dtg + 2, w) = m.g[1]; F(r_dtg + 3, w) = m.g[2];
    // default state: root pose from jp for a free root, zeros elsewhere
    for (int k = 0; k < nq; ++k) F(r_q + k, w) = 0.f;
    for (int k = 0; k < nv; ++k) { F(r_qd + k, w) = 0.f; F(r_qfrc + k, w) = 0.f; F(r_qacc + k, w) = 0.f; }
    if (m.links[0].joint == NEWT_JOINT_FREE) {
      for (int k = 0; k < 3; ++k) F(r_q + k, w) = m.links[0].jp_pos[k];
      for (int k = 0; k < 4; ++k) F(r_q + 3 + k, w) = m.links[0].jp_quat[k];
    }
    I(ri_solver, w) = m.solver != 0;
    I(ri_live, w) = 1;
    I(ri_status, w) = 0;
    if (ri_integ >= 0) I(ri_integ, w) = m.integrator;
    if (kind == GK_TREE_CONTACT) {
      for (int k = 0; k < ng; ++k) {
        const newt_geom_desc& G = m.geoms[k];
        float rec[22] = {G.size[0], G.size[1], G.size[2], G.local_pos[0], G.local_pos[1], G.local_pos[2],
                         G.local_quat[0], G.local_quat[1], G.local_quat[2], G.local_quat[3], G.friction, G.margin,
                         G.gap, G.solref[0], G.solref[1], G.solimp[0], G.solimp[1], G.solimp[2], G.solimp[3],
                         G.solimp[4], G.torsional_friction, G.rolling_friction};
        for (int f = 0; f < 22; ++f) F(r_geom + 22 * k + f, w) = rec[f];
      }
      I(ri_mode, w) = m.solver;
      I(ri_iters, w) = m.iterations;
    }
  } else if (kind == GK_PILE) {
    const int nb = size, ng = nb + np;
    const PileLayout& l = lay;
    std::vector<int> ent_of_geom(ng);
    int pi = 0;
    for (int k = 0; k < m.n_geoms; ++k) {
      const newt_geom_desc& G = m.geoms[k];
      int e = G.body >= 0 ? G.body : nb + (pi++);
      ent_of_geom[k] = e;
      I(l.gent + k, w) = e;
      F(l.fric + e, w) = G.friction;
      F(l.margin + e, w) = G.margin;
      F(l.tfric + e, w) = G.torsional_friction;
      F(l.rfric + e, w) = G.rolling_friction;
      I(l.gcond + e, w) = G.condim;
      if (G.body >= 0) {
        I(l.shape + e, w) = G.shape;
        for (int a = 0; a < 3; ++a) { F(l.size + 3 * e + a, w) = G.size[a]; F(l.gpos + 3 * e + a, w) = G.local_pos[a]; }
        for (int a = 0; a < 4; ++a) F(l.gquat + 4 * e + a, w) = G.local_quat[a];
      } else {
        int p = e - nb;
        for (int a = 0; a < 3; ++a) F(l.plane + 7 * p + a, w) = G.local_pos[a];
        for (int a = 0; a < 4; ++a) F(l.plane + 7 * p + 3 + a, w) = G.local_quat[a];
      }
    }
    // solref/solimp: the GPU pile path assumes one soft-constraint setting per world
    const newt_geom_desc& G0 = m.geoms[0];
    F(l.soft, w) = G0.solref[0]; F(l.soft + 1, w) = G0.solref[1];
    for (int a = 0; a < 5; ++a) F(l.soft + 2 + a, w) = G0.solimp[a];
    for (int b = 0; b < nb; ++b) {
      const newt_body_desc& B = m.bodies[b];
      F(l.mass + b, w) = B.mass;
      float s6[6], i6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      sym6(B.inertia, s6);
      inv6(B.inertia, i6);  // invertible: checked at upload
      for (int k = 0; k < 6; ++k) { F(l.inert + 6 * b + k, w) = s6[k]; F(l.iinv + 6 * b + k, w) = i6[k]; }
      for (int a = 0; a < 3; ++a) { F(l.pos + 3 * b + a, w) = 0.f; F(l.vel + 3 * b + a, w) = 0.f; F(l.omg + 3 * b + a, w) = 0.f; }
      F(l.quat + 4 * b, w) = 0.f; F(l.quat + 4 * b + 1, w) = 0.f; F(l.quat + 4 * b + 2, w) = 0.f; F(l.quat + 4 * b + 3, w) = 1.f;
    }
    F(l.dtg, w) = m.dt; F(l.dtg + 1, w) = m.g[0]; F(l.dtg + 2, w) = m.g[1]; F(l.dtg + 3, w) = m.g[2];
    I(l.iters, w) = m.iterations;
    I(l.status, w) = 0; I(l.ncon, w) = 0; I(l.live, w) = 1;
    I(l.integ, w) = m.integrator;
    I(l.cone, w) = m.cone;
  }
  model_dirty = true;
  pending.push_back(w);
}

int HostGroup::flush_model(newt_gpu_ctx* ctx) {
  if (soa() && !dtopo && !topo.empty()) {
    CKG(cudaMalloc(&dtopo, topo.size() * sizeof(int)));
    CKG(cudaMemcpy(dtopo, topo.data(), topo.size() * sizeof(int), cudaMemcpyHostToDevice));
  }
  if (kind == GK_TREE_CONTACT && !dgtopo && !gtopo.empty()) {
    CKG(cudaMalloc(&dgtopo, gtopo.size() * sizeof(int)));
    CKG(cudaMemcpy(dgtopo, gtopo.data(), gtopo.size() * sizeof(int), cudaMemcpyHostToDevice));
    CKG(cudaMalloc(&dpairs, std::max<size_t>(gpairs.size(), 2) * sizeof(int)));
    if (!gpairs.empty())
      CKG(cudaMemcpy(dpairs, gpairs.data(), gpairs.size() * sizeof(int), cudaMemcpyHostToDevice));
  }
  if (!model_dirty) return NEWT_OK;
  // upload only the newly written worlds (their whole records): other worlds
  // of the group may be mid-rollout on the device, with a stale host mirror;
  // one packed copy and one scatter launch per block, or one strided copy
  // when the worlds are consecutive
  std::sort(pending.begin(), pending.end());
  std::vector<RowMove> mv;
  mv.push_back(RowMove{this, pending, 0, frows, false});
  mv.push_back(RowMove{this, pending, 0, irows, true});
  const int rc = io_scatter(ctx, mv);
  if (rc != NEWT_OK) return rc;
  pending.clear();
  model_dirty = false;
  return NEWT_OK;
}

// ---------------------------------------------------------------------------
// state staging (MuJoCo layout in, newt layout on the device)
// ---------------------------------------------------------------------------
void HostGroup::stage_qfrc(int w, const HostModel& m, const float* qfrc) {
  if (soa()) for (int k = 0; k < nv; ++k) F(r_qfrc + k, w) = qfrc[k];
  (void)m;
}

void HostGroup::read_qacc(int w, const HostModel& m, float* qacc) const {
  if (soa()) for (int k = 0; k < nv; ++k) qacc[k] = Fc(r_qacc + k, w);
  else for (int k = 0; k < m.nv; ++k) qacc[k] = 0.f;
}

int HostGroup::fetch_status(newt_gpu_ctx* ctx) {
  if (n == 0) return NEWT_OK;
  // copies on the context's stream: the steps that set the status words run
  // there, and a plain cudaMemcpy does not wait for a non-blocking stream
  if (soa()) {
    CKG(cudaMemcpyAsync(hI.data() + (size_t)ri_status * cap, dI + (size_t)ri_status * cap, (size_t)cap * sizeof(int),
                        cudaMemcpyDeviceToHost, ctx->stream));
  } else {
    CKG(cudaMemcpy2DAsync(hI.data() + lay.status, irows * sizeof(int), dI + lay.status, irows * sizeof(int),
                          sizeof(int), n, cudaMemcpyDeviceToHost, ctx->stream));
  }
  CKG(cudaStreamSynchronize(ctx->stream));
  for (int w = 0; w < n; ++w)
    status_host[w] = soa() ? (uint32_t)hI[(size_t)ri_status * cap + w] : (uint32_t)hI[(size_t)w * irows + lay.status];
  return NEWT_OK;
}

int HostGroup::clear_status(newt_gpu_ctx* ctx) {
  if (n == 0) return NEWT_OK;
  if (soa()) {
    CKG(cudaMemsetAsync(dI + (size_t)ri_status * cap, 0, (size_t)cap * sizeof(int), ctx->stream));
  } else {
    CKG(cudaMemset2DAsync(dI + lay.status, irows * sizeof(int), 0, sizeof(int), n, ctx->stream));
  }
  CKG(cudaStreamSynchronize(ctx->stream));
  return NEWT_OK;
}

int HostGroup::read_contacts(newt_gpu_ctx* ctx, int w, int cap_out, int* n_out, int* pairs, float* data) {
  if (kind != GK_PILE && kind != GK_TREE_CONTACT) { *n_out = 0; return NEWT_OK; }
  if (kind == GK_TREE_CONTACT) {
    // contact records in the world's solver scratch (see newton_kernels.cu)
    int o_con, o_imp, o_misc;
    newt_tc_offsets(size, nv, ng, maxc, tc_rpc, &o_con, &o_imp, &o_misc);
    *n_out = 0;
    if (!plain_scratch) return NEWT_OK;
    const float* base = (const float*)plain_scratch + (size_t)w * scr_stride;
    std::vector<float> recs(TC_CREC * (size_t)maxc);
    int misc[2];
    CKG(cudaStreamSynchronize(ctx->stream));
    CKG(cudaMemcpy(misc, base + o_misc, sizeof(misc), cudaMemcpyDeviceToHost));
    CKG(cudaMemcpy(recs.data(), base + o_con, recs.size() * sizeof(float), cudaMemcpyDeviceToHost));
    const int nc = std::min(misc[0], maxc);
    *n_out = nc;
    for (int i = 0; i < nc && i < cap_out; ++i) {
      const float* c = recs.data() + TC_CREC * i;
      if (pairs) { std::memcpy(&pairs[2 * i], &c[0], sizeof(int)); std::memcpy(&pairs[2 * i + 1], &c[1], sizeof(int)); }
      if (data) { for (int k = 0; k < 6; ++k) data[7 * i + k] = c[4 + k]; data[7 * i + 6] = c[10]; }
    }
    return NEWT_OK;
  }
  std::vector<int> rec(irows);
  std::vector<float> frec(frows);
  CKG(cudaStreamSynchronize(ctx->stream));
  CKG(cudaMemcpy(rec.data(), dI + (size_t)w * irows, irows * sizeof(int), cudaMemcpyDeviceToHost));
  CKG(cudaMemcpy(frec.data(), dF + (size_t)w * frows, frows * sizeof(float), cudaMemcpyDeviceToHost));
  int nc = rec[lay.ncon];
  *n_out = nc;
  for (int i = 0; i < nc && i < cap_out && i < maxc; ++i) {
    if (pairs) { pairs[2 * i] = rec[lay.cpair + 2 * i]; pairs[2 * i + 1] = rec[lay.cpair + 2 * i + 1]; }
    if (data) for (int k = 0; k < 7; ++k) data[7 * i + k] = frec[lay.cdata + 7 * i + k];
  }
  return NEWT_OK;
}

int HostGroup::read_impulses(newt_gpu_ctx* ctx, int w, int cap_out, int* n_out, float* imp) {
  if (kind == GK_TREE_CONTACT) {
    int o_con, o_imp, o_misc;
    newt_tc_offsets(size, nv, ng, maxc, tc_rpc, &o_con, &o_imp, &o_misc);
    *n_out = 0;
    if (!plain_scratch) return NEWT_OK;
    const float* base = (const float*)plain_scratch + (size_t)w * scr_stride;
    int misc[2];
    CKG(cudaStreamSynchronize(ctx->stream));
    CKG(cudaMemcpy(misc, base + o_misc, sizeof(misc), cudaMemcpyDeviceToHost));
    const int nr = std::min(misc[1], tc_rpc * maxc);
    *n_out = nr;
    if (nr > 0 && imp) CKG(cudaMemcpy(imp, base + o_imp, std::min(nr, cap_out) * sizeof(float), cudaMemcpyDeviceToHost));
    return NEWT_OK;
  }
  if (kind != GK_PILE) { *n_out = 0; return NEWT_OK; }
  std::vector<int> rec(irows);
  std::vector<float> frec(frows);
  CKG(cudaStreamSynchronize(ctx->stream));
  CKG(cudaMemcpy(rec.data(), dI + (size_t)w * irows, irows * sizeof(int), cudaMemcpyDeviceToHost));
  CKG(cudaMemcpy(frec.data(), dF + (size_t)w * frows, frows * sizeof(float), cudaMemcpyDeviceToHost));
  int nc = std::min(rec[lay.ncon], maxc);
  int nr = lay.rpc * nc;
  *n_out = nr;
  for (int i = 0; i < nr && i < cap_out; ++i) imp[i] = frec[lay.imp + i];
  return NEWT_OK;
}

void HostGroup::release() {
  if (!hF.empty()) cudaHostUnregister(hF.data());
  if (!hI.empty()) cudaHostUnregister(hI.data());
  cudaGetLastError();
  if (dF) cudaFree(dF);
  if (dI) cudaFree(dI);
  if (dtopo) cudaFree(dtopo);
  if (dgtopo) cudaFree(dgtopo);
  if (dpairs) cudaFree(dpairs);
  if (plain_scratch) cudaFree(plain_scratch);
  dF = nullptr; dI = nullptr; dtopo = nullptr; dgtopo = nullptr; dpairs = nullptr; plain_scratch = nullptr;
}

TreeGroupDev HostGroup::tree_dev() const {
  TreeGroupDev d;
  d.n = n; d.cap = cap; d.L = size; d.nq = nq; d.nv = nv;
  d.topo = dtopo;
  auto row = [&](int r) { return dF + (size_t)r * cap; };
  d.axis = row(r_axis); d.jp = row(r_jp); d.jc = row(r_jc); d.rootq = row(r_rootq); d.mass = row(r_mass);
  d.inert = row(r_inert); d.damp = row(r_damp); d.arm = row(r_arm); d.dtg = row(r_dtg);
  d.solver = dI + (size_t)ri_solver * cap;
  d.live = dI + (size_t)ri_live * cap;
  d.integ = ri_integ >= 0 ? dI + (size_t)ri_integ * cap : nullptr;
  d.cfrc = nullptr; d.cstride = 0;
  d.q = row(r_q); d.qd = row(r_qd); d.qfrc = row(r_qfrc); d.qacc = row(r_qacc);
  d.status = (uint32_t*)(dI + (size_t)ri_status * cap);
  return d;
}

PileGroupDev HostGroup::pile_dev() const {
  PileGroupDev d;
  d.n = n; d.cap = cap; d.nb = size; d.np = np; d.maxc = maxc; d.lay = lay;
  d.F = dF; d.I = dI;
  d.scr = (float*)plain_scratch;
  d.sstride = scr_stride;
  d.solve = pile_newton ? PS_NEWTON : pile_general ? PS_GENERAL : PS_PGS;
  return d;
}

TcGroupDev HostGroup::tc_dev() const {
  TcGroupDev d;
  d.t = tree_dev();
  d.ng = ng; d.npairs = npairs; d.maxc = maxc;
  d.rpc = tc_rpc; d.cone = tc_cone; d.general = tc_general ? 1 : 0;
  d.gtopo = dgtopo; d.pairs = dpairs;
  d.geom = dF + (size_t)r_geom * cap;
  d.mode = dI + (size_t)ri_mode * cap;
  d.iters = dI + (size_t)ri_iters * cap;
  d.scr = (float*)plain_scratch;
  d.sstride = scr_stride;
  d.sens = nullptr;
  d.sens_stride = 0;
  return d;
}
