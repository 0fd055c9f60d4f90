// Free-body contact pipeline, solver half (the pile worlds: free spheres and
// boxes on a plane).  Per env-step, over every pile world:
//
//   K1 collide+assemble  one warp per world: load state, broadphase and
//                        narrowphase (pile_collide.cuh), soft-constraint row
//                        constants (J and M^-1 J^T of every facet row),
//                        contact islands, appended to per-class work lists
//   K2 pgs_small         one thread per island with one body and <= 4
//                        contacts (the common resting case): accumulators,
//                        Jacobians and impulses live in registers for all
//                        sweeps (classes 0-2)
//   K3 pgs_quad          multi-body islands (classes 3-5): four lanes per
//                        island, eight islands per warp; the contact sweep
//                        serial, each contact's rows spread over the lanes
//   K3c pgs_levels       long islands (class 6): one warp per island, the
//                        contacts of one dependency level solved at once
//   K4 integrate         one warp per world: semi-implicit Euler (or RK4 under
//                        the solver's wrench held over the stages), state and
//                        diagnostics back to the world record
// The class kernels touch disjoint islands and run concurrently.
//
// Restates, for FP32 on sm_103a:
//   newt/src/solver.rs:703-1257   solve_free_bodies_diag_mode (PGS branch)
//   newt/src/solver.rs:1448-1518  pgs_step_non_negative / pgs_step_pyramidal_pair
//   newt/src/solver.rs:1892-2036  row_body_diagonal, contact_regularization,
//                                 row_residual, apply_impulse_delta
//   newt/src/solver.rs:166-384    impedance, safe_solref, reference_accel
//   newt/src/solver.rs:3401-3429  pyramidal facet rows n +- mu t
//   newt/src/world.rs:3104-3112   tangent_basis
//   newt/src/world.rs:1790-1817   step_bodies_euler; world.rs:3223-3245 evaluate
//
// Gauss-Seidel is order dependent.  Rows of disjoint islands never touch the
// same body, so sweeping each island in newt's contact order (one thread per
// island) equals the serial sweep.  A facet row n + s*mu*t has Jacobian
// Jn + s*mu*Jt; each contact stores Jn, Jt1, Jt2 per side (K2 forms the rows
// on the fly) and the four rows with their M^-1 J^T (K3).  Velocity
// accumulators are kept in world frame (newt keeps the angular one in body
// frame; equal up to rounding).
#include <algorithm>

#include "../../include/newt_gpu.h"
#include "pile_solver.cuh"

using namespace pile;

namespace {

// solver-record fields (floats inside one SC block)
// (16-byte aligned: the multi-body solver reads them as float4)
enum { S_JA = 0, S_JB = 18, S_IDIAG = 36, S_BIAS = 40, S_P0 = 44, S_P1 = 48, S_REG = 52, S_MU = 53, S_IMP = 56,
       S_ROWS = 60 };
// S_ROWS: per facet row r (0..3), 32 floats at S_ROWS + 32 r: J then
//   M^-1 J^T, each as four float4 triples (side a linear, side a angular,
//   side b linear, side b angular; w = 0), zero for a static side
// pair block: h00, h11, h01, inverse determinant (0 when det <= 0)
static_assert(S_ROWS + 4 * 32 == SC, "solver record size");

// ---------------------------------------------------------------------------
// K1 part 2: row constants and islands (newt/src/solver.rs:752-1061)
// ---------------------------------------------------------------------------
// Island work lists: the PGS kernels run over compacted lists, one list per
// island class so each kernel variant is sized for its islands.
// 1 body x {1, 2, 3-4 contacts}; short multi-body islands (<= 4 contacts) with
// <= 4 or 5 bodies; long islands (5..32 contacts); the rest
constexpr int N_ICLASS = 7;
constexpr int CH_MIN = 5;    // contacts of the shortest island in the long-island class
constexpr int CH_MAXC = 8;  // contacts of the longest island solved by K3 (longer: K3c, by level)
struct IslandLists {
  int* items;   // N_ICLASS x cap entries: (world index in the table << 6) | island
  // zeroed before each step: [0, N_ICLASS) islands per class (the list
  // lengths), then contacts per class, then bodies per class (those two only
  // when `stats` is set: the last env-step of a call, for the profiling
  // surface; every world adding to the same counters costs contended atomics)
  int* counts;
  int cap;
  int stats;
};
constexpr int N_COUNTERS = 3 * N_ICLASS;

// 0-2: one body with 1, 2, 3-4 contacts (pile_k_pgs_small: everything in
// registers); 3, 4: fewer than CH_MIN contacts with up to 4 / 5 bodies; 5:
// CH_MIN..CH_MAXC contacts (pile_k_pgs_quad, sized per class); 6: the rest
// (pile_k_pgs_levels).
// An island is connected, so it has at most one body more than contacts.
NEWT_D int island_class(int nbody, int cnt) {
  if (nbody == 1 && cnt == 1) return 0;
  if (nbody == 1 && cnt == 2) return 1;
  if (nbody == 1 && cnt <= 4) return 2;
  if (cnt < CH_MIN) return nbody <= 4 ? 3 : 4;
  return (cnt <= CH_MAXC && nbody <= CH_MAXC + 1) ? 5 : 6;
}

NEWT_D void assemble(const WsLay& L, float* wf, int* wi, int lane, int t_world, const IslandLists& il) {
  const int nb = L.nb, nc = wi[L.misc + 1];
  const float dt = wf[L.dtg];
  const V3 grav = v3(wf[L.dtg + 1], wf[L.dtg + 2], wf[L.dtg + 3]);
  const float* soft = wf + L.soft;
  for (int b = lane; b < nb; b += 32) {
    M3 R = quat_mat(ld4(wf + L.quat + 4 * b));
    M3 RT{{{R.m[0][0], R.m[1][0], R.m[2][0]}, {R.m[0][1], R.m[1][1], R.m[2][1]}, {R.m[0][2], R.m[1][2], R.m[2][2]}}};
    S3 iw = sym_congr(RT, lds(wf + L.iinvb + 6 * b));
    float* o = wf + L.iinvw + 6 * b;
    o[0] = iw.xx; o[1] = iw.yy; o[2] = iw.zz; o[3] = iw.xy; o[4] = iw.xz; o[5] = iw.yz;
    st3(wf + L.dv + 3 * b, v3(0.f, 0.f, 0.f));
    st3(wf + L.dw + 3 * b, v3(0.f, 0.f, 0.f));
  }
  // active contacts (solver.rs:762-769): a dynamic side and penetration beyond the gap (gap = 0)
  for (int c = lane; c < nc; c += 32) {
    float* cf = wf + L.con + CF * c;
    const int* cc = wi + L.ci + CI * c;
    cf[C_ACT] = ((cc[2] < nb || cc[3] < nb) && cf[C_PEN] > 0.f) ? 1.f : 0.f;
    for (int k = 0; k < 6; ++k) cf[C_IMP + k] = 0.f;  // six slots: general rows read them all
  }
  __syncwarp();
  // islands, warp-parallel: each body's component as a 64-bit body mask
  // (bodies joined by active dynamic-dynamic contacts), closed by pointer
  // jumping (after r rounds a mask reaches every body within 2^r contacts);
  // an island is named by its smallest body and islands are numbered in that
  // order; bodies keep body order and contacts contact order inside an island
  // (the sweep order of newt's solver)
  unsigned* clo = reinterpret_cast<unsigned*>(wi + L.perm);  // component mask, low word (perm holds >= 2 nb)
  unsigned* chi = clo + nb;                                   // high word
  auto comp = [&](int b) { return ((unsigned long long)chi[b] << 32) | clo[b]; };
  auto active = [&](int c) { return wf[L.con + CF * c + C_ACT] != 0.f; };
  for (int b = lane; b < nb; b += 32) {
    clo[b] = b < 32 ? 1u << b : 0u;
    chi[b] = b >= 32 ? 1u << (b - 32) : 0u;
  }
  __syncwarp();
  for (int c = lane; c < nc; c += 32) {
    const int* cc = wi + L.ci + CI * c;
    if (!active(c) || cc[2] >= nb || cc[3] >= nb) continue;
    const int x = cc[2], y = cc[3];
    atomicOr(clo + x, y < 32 ? 1u << y : 0u);
    atomicOr(chi + x, y >= 32 ? 1u << (y - 32) : 0u);
    atomicOr(clo + y, x < 32 ? 1u << x : 0u);
    atomicOr(chi + y, x >= 32 ? 1u << (x - 32) : 0u);
  }
  __syncwarp();
  for (int round = 0; round < 7; ++round) {  // 2^6 >= the longest path in 64 bodies
    unsigned long long nw[2] = {0ull, 0ull};
    bool changed = false;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int b = lane + 32 * j;
      if (b >= nb) continue;
      const unsigned long long m = comp(b);
      unsigned long long acc = m;
      for (unsigned long long r = m; r; r &= r - 1) acc |= comp(__ffsll((long long)r) - 1);
      nw[j] = acc;
      changed |= acc != m;
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int b = lane + 32 * j;
      if (b < nb) { clo[b] = (unsigned)nw[j]; chi[b] = (unsigned)(nw[j] >> 32); }
    }
    __syncwarp();
    if (!__any_sync(0xffffffffu, changed)) break;
  }
  // islands exist where an active contact touches a component
  unsigned long long has = 0ull;
  for (int c = lane; c < nc; c += 32) {
    if (!active(c)) continue;
    const int* cc = wi + L.ci + CI * c;
    has |= 1ull << (__ffsll((long long)comp(cc[2] < nb ? cc[2] : cc[3])) - 1);
  }
  const unsigned long long isl_mask =
      ((unsigned long long)__reduce_or_sync(0xffffffffu, (unsigned)(has >> 32)) << 32) |
      __reduce_or_sync(0xffffffffu, (unsigned)has);
  const int nisl = __popcll((long long)isl_mask);
  auto island_of_root = [&](int r) { return __popcll((long long)(isl_mask & ((1ull << r) - 1ull))); };
  auto island_of_body = [&](int b) { return island_of_root(__ffsll((long long)comp(b)) - 1); };
  int* icount = wi + L.icount;
  int* istart = wi + L.istart;
  int* inb = wi + L.inb;
  int* ibstart = wi + L.ibstart;
  int* ibody = wi + L.ibody;
  int* blocal = wi + L.blocal;
  int* fill = wi + L.uf;  // running contact slot per island
  for (int i = lane; i < nisl; i += 32) {
    const unsigned lo = (unsigned)isl_mask, hi = (unsigned)(isl_mask >> 32);
    const int nlo = __popc(lo);
    const int r = i < nlo ? (int)__fns(lo, 0, i + 1) : 32 + (int)__fns(hi, 0, i + 1 - nlo);  // the island's root
    inb[i] = __popcll((long long)comp(r));
    icount[i] = 0;
  }
  __syncwarp();
  for (int c = lane; c < nc; c += 32) {
    if (!active(c)) continue;
    const int* cc = wi + L.ci + CI * c;
    atomicAdd(icount + island_of_body(cc[2] < nb ? cc[2] : cc[3]), 1);
  }
  __syncwarp();
  // exclusive prefix sums over islands (at most 64: two rounds of 32)
  {
    int cbase = 0, bbase = 0;
    for (int i0 = 0; i0 < nisl; i0 += 32) {
      const int i = i0 + lane;
      const int vc = i < nisl ? icount[i] : 0, vb = i < nisl ? inb[i] : 0;
      int sc = vc, sb = vb;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int tc = __shfl_up_sync(0xffffffffu, sc, o), tb = __shfl_up_sync(0xffffffffu, sb, o);
        if (lane >= o) { sc += tc; sb += tb; }
      }
      if (i < nisl) {
        istart[i] = cbase + sc - vc;
        fill[i] = cbase + sc - vc;
        ibstart[i] = bbase + sb - vb;
      }
      cbase += __shfl_sync(0xffffffffu, sc, 31);
      bbase += __shfl_sync(0xffffffffu, sb, 31);
    }
  }
  __syncwarp();
  // bodies: island-local index = rank in the component mask
  for (int b = lane; b < nb; b += 32) {
    const unsigned long long m = comp(b);
    const int r = __ffsll((long long)m) - 1;
    if (!((isl_mask >> r) & 1ull)) { blocal[b] = -1; continue; }
    const int loc = __popcll((long long)(m & ((1ull << b) - 1ull)));
    blocal[b] = loc;
    ibody[ibstart[island_of_root(r)] + loc] = b;
  }
  __syncwarp();
  // contacts: slots in island order, contact order inside an island
  int* sccon = wi + L.sccon;
  int* scid = wi + L.scid;
  const unsigned lt = (1u << lane) - 1u;
  for (int c0 = 0; c0 < nc; c0 += 32) {
    const int c = c0 + lane;
    const bool act = c < nc && active(c);
    const int* cc = wi + L.ci + CI * (act ? c : 0);
    const int isl = act ? island_of_body(cc[2] < nb ? cc[2] : cc[3]) : -1;
    const unsigned grp = __match_any_sync(0xffffffffu, isl);
    const int base = act ? fill[isl] : 0;
    __syncwarp();
    if (act) {
      const int k = base + __popc(grp & lt);
      sccon[k] = c;
      scid[2 * k] = cc[2] < nb ? blocal[cc[2]] : -1;
      scid[2 * k + 1] = cc[3] < nb ? blocal[cc[3]] : -1;
      if ((grp & lt) == 0u) fill[isl] = base + __popc(grp);
    }
    __syncwarp();
  }
  if (lane == 0) {
    wi[L.misc + 3] = nisl;
    // append this world's islands to the class work lists
    int ncls[N_ICLASS] = {}, ccls[N_ICLASS] = {}, bcls[N_ICLASS] = {};
    for (int i = 0; i < nisl; ++i) {
      const int c = island_class(inb[i], icount[i]);
      ncls[c]++;
      ccls[c] += icount[i];
      bcls[c] += inb[i];
    }
    int base[N_ICLASS];
    for (int c = 0; c < N_ICLASS; ++c) {
      base[c] = 0;
      if (!ncls[c]) continue;
      base[c] = atomicAdd(il.counts + c, ncls[c]);
      if (il.stats) {
        atomicAdd(il.counts + N_ICLASS + c, ccls[c]);
        atomicAdd(il.counts + 2 * N_ICLASS + c, bcls[c]);
      }
    }
    for (int i = 0; i < nisl; ++i) {
      const int c = island_class(inb[i], icount[i]);
      const int slot = base[c]++;
      if (slot < il.cap) il.items[(size_t)c * il.cap + slot] = (t_world << 6) | i;
    }
  }
  __syncwarp();
  // per active contact: Jacobians, regularisation, bias, pair constants
  float tc = soft[0], dr = soft[1];
  const bool direct = tc < 0.f;
  if (!direct && tc < 2.f * dt) tc = 2.f * dt;  // safe_solref (solver.rs:331-338)
  const float dmax = fminf(fmaxf(soft[3], 1.0e-4f), 0.9999f);
  const int nact = nisl > 0 ? wi[L.istart + nisl - 1] + wi[L.icount + nisl - 1] : 0;
  for (int k = lane; k < nact; k += 32) {
    const int c = wi[L.sccon + k];
    const float* cf = wf + L.con + CF * c;
    const int* cc = wi + L.ci + CI * c;
    float* sc = wf + L.sc + SC * k;
    const int ea = cc[2], eb = cc[3];
    const bool da = ea < nb, db = eb < nb;
    const float pen = cf[C_PEN], mu = cf[C_MU];
    const V3 n = ld3(cf + C_N), pos = ld3(cf + C_POS);
    V3 ref = fabsf(n.z) < 0.9f ? v3(0.f, 0.f, 1.f) : v3(1.f, 0.f, 0.f);
    V3 t1 = cross(ref, n);
    float tl = sqrtf(len2(t1));
    t1 = tl == 0.f ? v3(0.f, 0.f, 0.f) : t1 * (1.f / tl);
    const V3 t2 = cross(n, t1);
    const V3 arma = da ? pos - ld3(wf + L.pos + 3 * ea) : v3(0.f, 0.f, 0.f);
    const V3 armb = db ? pos - ld3(wf + L.pos + 3 * eb) : v3(0.f, 0.f, 0.f);
    // side Jacobians: a = (d, arm_a x d); b = -(d, arm_b x d); zero when static
    J6 Ja[3], Jb[3];
    const V3 ds[3] = {n, t1, t2};
    for (int q = 0; q < 3; ++q) {
      Ja[q] = da ? J6{ds[q], cross(arma, ds[q])} : J6{v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f)};
      Jb[q] = db ? J6{-ds[q], -cross(armb, ds[q])} : J6{v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f)};
      stj(sc + S_JA + 6 * q, Ja[q]);
      stj(sc + S_JB + 6 * q, Jb[q]);
    }
    sc[S_MU] = mu;
    const float ima = da ? 1.f / wf[L.mass + ea] : 0.f, imb = db ? 1.f / wf[L.mass + eb] : 0.f;
    const S3 Ia = da ? lds(wf + L.iinvw + 6 * ea) : S3{0, 0, 0, 0, 0, 0};
    const S3 Ib = db ? lds(wf + L.iinvw + 6 * eb) : S3{0, 0, 0, 0, 0, 0};
    const float d = impedance(-pen, soft);
    const float tran = ima + imb;
    const float reg = d > 0.f ? 2.f * mu * mu * ((1.f - d) / d * (tran * (1.f + mu * mu))) : 0.f;
    sc[S_REG] = reg;
    float b_, k_;
    if (direct) { b_ = -dr / dmax; k_ = -soft[0] / (dmax * dmax); }
    else { b_ = 2.f / (dmax * tc); k_ = d / (dmax * dmax * tc * tc * dr * dr); }
    V3 va = v3(0.f, 0.f, 0.f), vb = v3(0.f, 0.f, 0.f);
    if (da) va = ld3(wf + L.vel + 3 * ea) + cross(qrot(ld4(wf + L.quat + 4 * ea), ld3(wf + L.omg + 3 * ea)), arma);
    if (db) vb = ld3(wf + L.vel + 3 * eb) + cross(qrot(ld4(wf + L.quat + 4 * eb), ld3(wf + L.omg + 3 * eb)), armb);
    float diag[4];
    J6 Ra[4], Rb[4];
    for (int r = 0; r < 4; ++r) {
      const int q = r < 2 ? 1 : 2;
      const float s = (r & 1) ? -mu : mu;
      Ra[r] = jrow(Ja[0], Ja[q], s);
      Rb[r] = jrow(Jb[0], Jb[q], s);
      const V3 dir = n + ds[q] * s;
      // A_ii (row_body_diagonal) + regulariser
      float aii = 0.f, dvf = 0.f;
      if (da) { aii += dot(Ra[r].a, smv(Ia, Ra[r].a)) + ima; dvf += dot(grav * dt, dir); }
      if (db) { aii += dot(Rb[r].a, smv(Ib, Rb[r].a)) + imb; dvf -= dot(grav * dt, dir); }
      diag[r] = aii + reg;
      sc[S_IDIAG + r] = 1.f / diag[r];
      const float vcur = dot(va - vb, dir);
      const float aref = -b_ * vcur - k_ * (-pen);
      sc[S_BIAS + r] = dvf - aref * dt;
      sc[S_IMP + r] = 0.f;
      // a static side's row is stored as zeros, so the solvers need no masks
      float* row = sc + S_ROWS + 32 * r;
      const V3 z = v3(0.f, 0.f, 0.f);
      const V3 trip[8] = {da ? Ra[r].l : z, da ? Ra[r].a : z, db ? Rb[r].l : z, db ? Rb[r].a : z,
                          da ? Ra[r].l * ima : z, da ? smv(Ia, Ra[r].a) : z,
                          db ? Rb[r].l * imb : z, db ? smv(Ib, Rb[r].a) : z};
      for (int e = 0; e < 8; ++e) {
        row[4 * e] = trip[e].x; row[4 * e + 1] = trip[e].y; row[4 * e + 2] = trip[e].z; row[4 * e + 3] = 0.f;
      }
    }
    // pyramidal pair blocks (solver.rs:1037-1061, 1476-1518)
    for (int p = 0; p < 2; ++p) {
      const int i0 = 2 * p, i1 = i0 + 1;
      float h01 = 0.f;
      if (da) h01 += dot(Ra[i0].l, Ra[i1].l) * ima + dot(Ra[i0].a, smv(Ia, Ra[i1].a));
      if (db) h01 += dot(Rb[i0].l, Rb[i1].l) * imb + dot(Rb[i0].a, smv(Ib, Rb[i1].a));
      const float det = diag[i0] * diag[i1] - h01 * h01;
      float* pb = sc + (p ? S_P1 : S_P0);
      pb[0] = diag[i0]; pb[1] = diag[i1]; pb[2] = h01; pb[3] = det > 0.f ? 1.f / det : 0.f;
    }
  }
  __syncwarp();
}

}  // namespace

// ---------------------------------------------------------------------------
// K1: collide + assemble (one warp per world)
// ---------------------------------------------------------------------------
// Six blocks per SM (80 registers, a few spills) measured 2.6% faster on the
// 8192-world pile step than four (128 registers).
__global__ void __launch_bounds__(128, 6) pile_k_collide(const PileGroupDev* G, const int* wseg, int ng, int total,
                                                      IslandLists il) {
  const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (t >= total) return;
  const int gi = find_seg(wseg, ng, t);
  const PileGroupDev& g = G[gi];
  const int w = t - wseg[gi];
  if (w >= g.n || !g.I[(size_t)w * g.lay.istride + g.lay.live]) return;
  const WsLay L = ws_layout(g.nb, g.np, g.maxc);
  float* wf = g.scr + (size_t)w * g.sstride;
  int* wi = reinterpret_cast<int*>(wf + L.nf);
  const int lane = threadIdx.x & 31;
  ws_load(g, w, L, wf, wi, lane);
  collide(L, wf, wi, lane);
  assemble(L, wf, wi, lane, t, il);
}

// The post-step contact re-solve behind the contact sensors (newt's
// build_sensor_inputs, world.rs:1545-1612): the world's current state with
// the contacts its last step detected, which every step form leaves in the
// world record (pairs, point, normal, depth; a new world has none).  The
// scratch's contact records are rebuilt from them as the narrowphase wrote
// them (bodies from the geoms, friction the smaller of the two), then the
// rows and islands at the current state; no narrowphase runs.
__global__ void __launch_bounds__(128, 6) pile_k_reassemble(const PileGroupDev* G, const int* wseg, int ng,
                                                          int total, IslandLists il) {
  const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (t >= total) return;
  const int gi = find_seg(wseg, ng, t);
  const PileGroupDev& g = G[gi];
  const int w = t - wseg[gi];
  if (w >= g.n || !g.I[(size_t)w * g.lay.istride + g.lay.live]) return;
  const WsLay L = ws_layout(g.nb, g.np, g.maxc);
  float* wf = g.scr + (size_t)w * g.sstride;
  int* wi = reinterpret_cast<int*>(wf + L.nf);
  const int lane = threadIdx.x & 31;
  ws_load(g, w, L, wf, wi, lane);
  const PileLayout& P = g.lay;
  const float* F = g.F + (size_t)w * P.fstride;
  const int* I = g.I + (size_t)w * P.istride;
  const int nc = min(max(I[P.ncon], 0), L.maxc);
  for (int c = lane; c < nc; c += 32) {
    float* cf = wf + L.con + CF * c;
    int* cc = wi + L.ci + CI * c;
    const int ga = I[P.cpair + 2 * c], gb = I[P.cpair + 2 * c + 1];
    const int ea = wi[L.gent + ga], eb = wi[L.gent + gb];
    for (int k = 0; k < 7; ++k) cf[C_POS + k] = F[P.cdata + 7 * c + k];
    cf[C_MU] = fminf(wf[L.fric + ea], wf[L.fric + eb]);
    cc[0] = ga; cc[1] = gb; cc[2] = ea; cc[3] = eb;
  }
  if (lane == 0) {
    wi[L.misc + 1] = nc;
    wi[L.misc + 2] = 0;
  }
  __syncwarp();
  assemble(L, wf, wi, lane, t, il);
}

// Resolve a list item to its world scratch and island.
struct IslandRef {
  const PileGroupDev* g;
  int w, isl;
  float* wf;
  const int* wi;
  WsLay L;
};

NEWT_D bool island_ref(const PileGroupDev* G, const int* wseg, int ng, int item, IslandRef* r) {
  const int t = item >> 6;
  r->isl = item & 63;
  const int gi = find_seg(wseg, ng, t);
  r->g = G + gi;
  r->w = t - wseg[gi];
  r->L = ws_layout(r->g->nb, r->g->np, r->g->maxc);
  r->wf = r->g->scr + (size_t)r->w * r->g->sstride;
  r->wi = reinterpret_cast<const int*>(r->wf + r->L.nf);
  return true;
}

// ---------------------------------------------------------------------------
// K2: one-body islands with at most MC contacts; every sweep in registers
// ---------------------------------------------------------------------------
template <int MC>
__global__ void __launch_bounds__(128) pile_k_pgs_small(const PileGroupDev* G, const int* wseg, int ng,
                                                        const int* items, const int* count, int cls) {
  const int n_items = count[cls];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n_items; t += gridDim.x * blockDim.x) {
  IslandRef R;
  island_ref(G, wseg, ng, items[t], &R);
  const WsLay& L = R.L;
  float* wf = R.wf;
  const int* wi = R.wi;
  const int isl = R.isl;
  const int cnt = wi[L.icount + isl];
  const int k0 = wi[L.istart + isl];
  const int body = wi[L.ibody + wi[L.ibstart + isl]];
  const int iters = R.g->I[(size_t)R.w * R.g->lay.istride + R.g->lay.iters];
  const float im = 1.f / wf[L.mass + body];
  const S3 Iw = lds(wf + L.iinvw + 6 * body);
  J6 jn[MC], jt1[MC], jt2[MC];
  float mu[MC], idg[MC][4], bias[MC][4], reg[MC], pb[MC][8], imp[MC][4];
#pragma unroll
  for (int c = 0; c < MC; ++c) {
    if (c < cnt) {
      const float* sc = wf + L.sc + SC * (k0 + c);
      const bool sa = wi[L.scid + 2 * (k0 + c)] >= 0;
      const float* J = sc + (sa ? S_JA : S_JB);
      jn[c] = ldj(J); jt1[c] = ldj(J + 6); jt2[c] = ldj(J + 12);
      mu[c] = sc[S_MU]; reg[c] = sc[S_REG];
#pragma unroll
      for (int r = 0; r < 4; ++r) { idg[c][r] = sc[S_IDIAG + r]; bias[c][r] = sc[S_BIAS + r]; imp[c][r] = 0.f; }
#pragma unroll
      for (int q = 0; q < 8; ++q) pb[c][q] = sc[S_P0 + q];
    }
  }
  V3 dv = v3(0.f, 0.f, 0.f), dw = v3(0.f, 0.f, 0.f);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < MC; ++c) {
      if (c < cnt) {
        {
          const J6 j = jrow(jn[c], jt1[c], mu[c]);
          const float res = jdot(j, dv, dw) + reg[c] * imp[c][0] + bias[c][0];
          const float nf = RowStep::nonneg(imp[c][0], res, idg[c][0]);
          const float dl = nf - imp[c][0];
          imp[c][0] = nf;
          dv = dv + j.l * (dl * im);
          dw = dw + smv(Iw, j.a * dl);
        }
#pragma unroll
        for (int p = 0; p < 2; ++p) {
          const J6& jt = p ? jt2[c] : jt1[c];
          const J6 ji = jrow(jn[c], jt, mu[c]), jj = jrow(jn[c], jt, -mu[c]);
          const int i = 2 * p, j = i + 1;
          const float* P = pb[c] + 4 * p;
          if (P[3] == 0.f) {  // det <= 0: two half-line steps
            float res = jdot(ji, dv, dw) + reg[c] * imp[c][i] + bias[c][i];
            float nf = RowStep::nonneg(imp[c][i], res, idg[c][i]);
            float dl = nf - imp[c][i];
            imp[c][i] = nf;
            dv = dv + ji.l * (dl * im); dw = dw + smv(Iw, ji.a * dl);
            res = jdot(jj, dv, dw) + reg[c] * imp[c][j] + bias[c][j];
            nf = RowStep::nonneg(imp[c][j], res, idg[c][j]);
            dl = nf - imp[c][j];
            imp[c][j] = nf;
            dv = dv + jj.l * (dl * im); dw = dw + smv(Iw, jj.a * dl);
            continue;
          }
          const float ri = jdot(ji, dv, dw) + reg[c] * imp[c][i] + bias[c][i];
          const float rj = jdot(jj, dv, dw) + reg[c] * imp[c][j] + bias[c][j];
          float ni, nj;
          RowStep::pair(imp[c][i], imp[c][j], ri, rj, P, &ni, &nj);
          const float ai = ni - imp[c][i], aj = nj - imp[c][j];
          imp[c][i] = ni; imp[c][j] = nj;
          dv = dv + ji.l * (ai * im) + jj.l * (aj * im);
          dw = dw + smv(Iw, ji.a * ai + jj.a * aj);
        }
      }
    }
  }
#pragma unroll
  for (int c = 0; c < MC; ++c)
    if (c < cnt) {
      float* cimp = wf + L.con + CF * wi[L.sccon + k0 + c] + C_IMP;
#pragma unroll
      for (int r = 0; r < 4; ++r) cimp[r] = imp[c][r];
    }
  st3(wf + L.dv + 3 * body, dv);
  st3(wf + L.dw + 3 * body, dw);
  }
}

// ---------------------------------------------------------------------------
// K3: multi-body islands (classes 3-5), four lanes per island and eight
// islands per warp.  The contact sweep of an island stays serial (Gauss-
// Seidel order); inside one contact, lane l of the island's four holds one
// float4 triple of the 12 velocity-accumulator entries the contact touches
// (side a linear, side a angular, side b linear, side b angular) and the
// matching triples of the facet rows' J and M^-1 J^T.  A facet residual is
// a triple dot product summed over the four lanes (two shuffles; a 2x2 pair
// sums both rows at once), every lane takes the same scalar step and updates
// its own triple.  Body accumulators live in shared memory (island-local
// ids, a dummy slot for a static side), and so do the impulses of islands
// within the class's contact bound (the solver record holds them otherwise).
// The warp runs until its longest island is done; finished islands idle.
// ---------------------------------------------------------------------------
NEWT_D float dot3(const float* j, const float* a) { return (j[0] * a[0] + j[1] * a[1]) + j[2] * a[2]; }
NEWT_D float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

// One lane's share of one contact: its triple of each facet row's J and
// M^-1 J^T, the row scalars, the impulses and its side's body slot.
struct QuadContact {
  float J[4][3], W[4][3];
  float idg[4], bias[4], P[8], imp[4], reg;
  int body;
};

NEWT_D void quad_load(const float* sc, const float4* imp, const int* ids, int side, int l, int dummy,
                      QuadContact& c) {
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const float4 j = ldg4(sc + S_ROWS + 32 * r + 4 * l), w = ldg4(sc + S_ROWS + 32 * r + 16 + 4 * l);
    c.J[r][0] = j.x; c.J[r][1] = j.y; c.J[r][2] = j.z;
    c.W[r][0] = w.x; c.W[r][1] = w.y; c.W[r][2] = w.z;
  }
  const float4 d = ldg4(sc + S_IDIAG), b = ldg4(sc + S_BIAS), p0 = ldg4(sc + S_P0), p1 = ldg4(sc + S_P1);
  c.idg[0] = d.x; c.idg[1] = d.y; c.idg[2] = d.z; c.idg[3] = d.w;
  c.bias[0] = b.x; c.bias[1] = b.y; c.bias[2] = b.z; c.bias[3] = b.w;
  c.P[0] = p0.x; c.P[1] = p0.y; c.P[2] = p0.z; c.P[3] = p0.w;
  c.P[4] = p1.x; c.P[5] = p1.y; c.P[6] = p1.z; c.P[7] = p1.w;
  c.reg = __ldg(sc + S_REG);
  const float4 m = *imp;  // written by this kernel in the previous sweep
  c.imp[0] = m.x; c.imp[1] = m.y; c.imp[2] = m.z; c.imp[3] = m.w;
  const int id = __ldg(ids + side);
  c.body = id >= 0 ? id : dummy;
}

NEWT_D void quad_zero(int dummy, QuadContact& c) {
#pragma unroll
  for (int r = 0; r < 4; ++r) {
#pragma unroll
    for (int e = 0; e < 3; ++e) c.J[r][e] = c.W[r][e] = 0.f;
    c.idg[r] = c.bias[r] = c.imp[r] = 0.f;
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) c.P[i] = 0.f;
  c.reg = 0.f;
  c.body = dummy;
}

// MAXB: bodies per island; MAXC > 0: contacts per island, whose impulses are
// then kept in shared memory (0: in the solver record); WPB: warps per block.
template <int MAXB, int MAXC, int WPB>
__global__ void __launch_bounds__(32 * WPB) pile_k_pgs_quad(const PileGroupDev* G, const int* wseg, int ng,
                                                            const int* items, const int* count, int cls) {
  __shared__ float acc_s[WPB][8][MAXB + 1][6];
  __shared__ float4 imp_s[WPB][8][MAXC > 0 ? MAXC : 1];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int slot = lane >> 2, l = lane & 3, side = l >> 1, part = l & 1;
  const unsigned gm = 0xFu << (lane & ~3);  // this island's four lanes
  float(*acc)[6] = acc_s[wib][slot];
  const int n_items = count[cls];
  const int stride = gridDim.x * WPB * 8;
  for (int base = (blockIdx.x * WPB + wib) * 8; base < n_items; base += stride) {
    const int t = base + slot;
    int nbody = 0, cnt = 0, k0 = 0, b0 = 0, iters = 0;
    float* wf = nullptr;
    const int* wi = nullptr;
    WsLay L{};
    if (t < n_items) {
      IslandRef R;
      island_ref(G, wseg, ng, items[t], &R);
      L = R.L;
      wf = R.wf;
      wi = R.wi;
      nbody = wi[L.inb + R.isl];
      cnt = wi[L.icount + R.isl];
      k0 = wi[L.istart + R.isl];
      b0 = wi[L.ibstart + R.isl];
      iters = R.g->I[(size_t)R.w * R.g->lay.istride + R.g->lay.iters];
    }
    float* const sc0 = t < n_items ? wf + L.sc + SC * k0 : nullptr;
    const int* const id0 = t < n_items ? wi + L.scid + 2 * k0 : nullptr;
    float4* const imps = imp_s[wib][slot];
    // impulse of contact k: shared memory, or the solver record
    auto impk = [&](int k) -> float4* {
      return MAXC > 0 ? imps + k : reinterpret_cast<float4*>(sc0 + (size_t)SC * k + S_IMP);
    };
    for (int i = l; i < 6 * (nbody + 1); i += 4) (&acc[0][0])[i] = 0.f;
    if (MAXC > 0)
      for (int i = l; i < cnt; i += 4) imps[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    const int total = iters * cnt;
    int tmax = total;
#pragma unroll
    for (int o = 4; o < 32; o <<= 1) tmax = max(tmax, __shfl_xor_sync(0xffffffffu, tmax, o));
    __syncwarp();
    int k = 0;
    // one contact of the sweep; the next contact's values are fetched into
    // `nxt` while `cur` is solved (the loop below alternates the two)
    auto contact = [&](int step, QuadContact& cur, QuadContact& nxt) {
      const bool on = step < total;
      const int kn = k + 1 == cnt ? 0 : k + 1;
      if (step + 1 < total) quad_load(sc0 + (size_t)SC * kn, impk(kn), id0 + 2 * kn, side, l, nbody, nxt);
      const int body = on ? cur.body : 0;
      float a[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) a[c] = on ? acc[body][3 * part + c] : 0.f;
      float im[4] = {cur.imp[0], cur.imp[1], cur.imp[2], cur.imp[3]};
      auto single = [&](int r) {
        float d = dot3(cur.J[r], a);
        d += __shfl_xor_sync(gm, d, 1);
        d += __shfl_xor_sync(gm, d, 2);
        const float res = d + (cur.reg * im[r] + cur.bias[r]);
        const float nf = RowStep::nonneg(im[r], res, cur.idg[r]);
        const float dl = nf - im[r];
        im[r] = nf;
        a[0] += cur.W[r][0] * dl;
        a[1] += cur.W[r][1] * dl;
        a[2] += cur.W[r][2] * dl;
      };
      single(0);
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        const int i = 2 * p, j = i + 1;
        const float* Pp = cur.P + 4 * p;
        if (Pp[3] == 0.f) {  // uniform over the island's lanes
          single(i);
          single(j);
          continue;
        }
        float di = dot3(cur.J[i], a), dj = dot3(cur.J[j], a);
        di += __shfl_xor_sync(gm, di, 1);
        dj += __shfl_xor_sync(gm, dj, 1);
        di += __shfl_xor_sync(gm, di, 2);
        dj += __shfl_xor_sync(gm, dj, 2);
        const float ri = di + (cur.reg * im[i] + cur.bias[i]);
        const float rj = dj + (cur.reg * im[j] + cur.bias[j]);
        float ni, nj;
        RowStep::pair(im[i], im[j], ri, rj, Pp, &ni, &nj);
        const float ai = ni - im[i], aj = nj - im[j];
        im[i] = ni;
        im[j] = nj;
        a[0] += cur.W[i][0] * ai;
        a[1] += cur.W[i][1] * ai;
        a[2] += cur.W[i][2] * ai;
        a[0] += cur.W[j][0] * aj;
        a[1] += cur.W[j][1] * aj;
        a[2] += cur.W[j][2] * aj;
      }
      if (on) {
#pragma unroll
        for (int c = 0; c < 3; ++c) acc[body][3 * part + c] = a[c];
        if (l == 0) *impk(k) = make_float4(im[0], im[1], im[2], im[3]);
        if (kn == k) {  // a one-contact island reads its own update back
#pragma unroll
          for (int r = 0; r < 4; ++r) nxt.imp[r] = im[r];
        }
        k = kn;
      }
      __syncwarp();
    };
    QuadContact c0, c1;
    if (total > 0) quad_load(sc0, impk(0), id0, side, l, nbody, c0);
    else quad_zero(nbody, c0);
    quad_zero(nbody, c1);
    for (int step = 0; step < tmax; step += 2) {
      contact(step, c0, c1);
      if (step + 1 < tmax) contact(step + 1, c1, c0);
    }
    if (t < n_items) {
      for (int kk = l; kk < cnt; kk += 4) {
        const float4 m = *impk(kk);
        float* cimp = wf + L.con + CF * wi[L.sccon + k0 + kk] + C_IMP;
        cimp[0] = m.x; cimp[1] = m.y; cimp[2] = m.z; cimp[3] = m.w;
      }
      for (int b = l; b < nbody; b += 4) {
        const int bd = wi[L.ibody + b0 + b];
        st3(wf + L.dv + 3 * bd, v3(acc[b][0], acc[b][1], acc[b][2]));
        st3(wf + L.dw + 3 * bd, v3(acc[b][3], acc[b][4], acc[b][5]));
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// K3c: long islands (class 6), one warp per island, contacts solved by
// dependency level.  In newt's sweep order a contact must see the updates of
// every earlier contact that shares one of its bodies and nothing else, so
// contact k sits at level 1 + max(level of the last earlier contact on each
// of its bodies).  Contacts of one level touch disjoint bodies: the eight
// four-lane groups of the warp solve them at once (each contact exactly as
// in K3), and the levels run in order, so every body sees its contacts'
// updates in sweep order and the result equals the serial sweep.
// ---------------------------------------------------------------------------
constexpr int PL_WARPS = 4;
constexpr int PL_MAXC = 512;  // the largest contact capacity of a pile world

__global__ void __launch_bounds__(32 * PL_WARPS) pile_k_pgs_levels(const PileGroupDev* G, const int* wseg, int ng,
                                                                   const int* items, const int* count, int cls) {
  __shared__ float acc_s[PL_WARPS][NEWT_MAX_BODIES + 1][6];
  __shared__ short perm_s[PL_WARPS][PL_MAXC];      // contacts by (level, sweep order)
  __shared__ short loff_s[PL_WARPS][PL_MAXC + 1];  // level start offsets
  __shared__ short lev_s[PL_WARPS][PL_MAXC];
  __shared__ short last_s[PL_WARPS][NEWT_MAX_BODIES + 1];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int slot = lane >> 2, l = lane & 3, side = l >> 1, part = l & 1;
  const unsigned gm = 0xFu << (lane & ~3);
  float(*acc)[6] = acc_s[wib];
  short* perm = perm_s[wib];
  short* loff = loff_s[wib];
  short* lev = lev_s[wib];
  short* last = last_s[wib];
  const int n_items = count[cls];
  for (int t = blockIdx.x * PL_WARPS + wib; t < n_items; t += gridDim.x * PL_WARPS) {
    IslandRef R;
    island_ref(G, wseg, ng, items[t], &R);
    const WsLay& L = R.L;
    float* wf = R.wf;
    const int* wi = R.wi;
    const int nbody = wi[L.inb + R.isl], cnt = min(wi[L.icount + R.isl], PL_MAXC);
    const int k0 = wi[L.istart + R.isl], b0 = wi[L.ibstart + R.isl];
    const int iters = R.g->I[(size_t)R.w * R.g->lay.istride + R.g->lay.iters];
    float* const sc0 = wf + L.sc + SC * k0;
    const int* const id0 = wi + L.scid + 2 * k0;
    for (int i = lane; i < 6 * (nbody + 1); i += 32) (&acc[0][0])[i] = 0.f;
    // the level schedule: levels (lane 0), then a counting sort by level
    int nlev = 0;
    if (lane == 0) {
      for (int b = 0; b <= nbody; ++b) last[b] = 0;
      for (int k = 0; k < cnt; ++k) {
        const int la = id0[2 * k], lb = id0[2 * k + 1];
        const int lv = 1 + max(la >= 0 ? (int)last[la] : 0, lb >= 0 ? (int)last[lb] : 0);
        if (la >= 0) last[la] = (short)lv;
        if (lb >= 0) last[lb] = (short)lv;
        lev[k] = (short)lv;
        nlev = max(nlev, lv);
      }
      for (int v = 0; v <= nlev; ++v) loff[v] = 0;
      for (int k = 0; k < cnt; ++k) loff[lev[k]]++;
      int run = 0;
      for (int v = 1; v <= nlev; ++v) { const int c = loff[v]; loff[v - 1] = (short)run; run += c; }
      loff[nlev] = (short)run;
      for (int k = 0; k < cnt; ++k) perm[loff[lev[k] - 1]++] = (short)k;
      for (int v = nlev; v > 0; --v) loff[v] = loff[v - 1];  // back to level starts
      loff[0] = 0;
    }
    nlev = __shfl_sync(0xffffffffu, nlev, 0);
    __syncwarp();
    for (int it = 0; it < iters; ++it) {
      for (int v = 0; v < nlev; ++v) {
        const int s = loff[v], e = loff[v + 1];
        for (int base = s; base < e; base += 8) {
          const int idx = base + slot;
          const bool on = idx < e;
          const int k = on ? perm[idx] : 0;
          QuadContact cur;
          if (on) quad_load(sc0 + (size_t)SC * k, reinterpret_cast<const float4*>(sc0 + (size_t)SC * k + S_IMP),
                            id0 + 2 * k, side, l, nbody, cur);
          else quad_zero(nbody, cur);
          const int body = on ? cur.body : 0;
          float a[3];
#pragma unroll
          for (int c = 0; c < 3; ++c) a[c] = on ? acc[body][3 * part + c] : 0.f;
          float im[4] = {cur.imp[0], cur.imp[1], cur.imp[2], cur.imp[3]};
          auto single = [&](int r) {
            float d = dot3(cur.J[r], a);
            d += __shfl_xor_sync(gm, d, 1);
            d += __shfl_xor_sync(gm, d, 2);
            const float res = d + (cur.reg * im[r] + cur.bias[r]);
            const float nf = RowStep::nonneg(im[r], res, cur.idg[r]);
            const float dl = nf - im[r];
            im[r] = nf;
            a[0] += cur.W[r][0] * dl;
            a[1] += cur.W[r][1] * dl;
            a[2] += cur.W[r][2] * dl;
          };
          single(0);
#pragma unroll
          for (int p = 0; p < 2; ++p) {
            const int i = 2 * p, j = i + 1;
            const float* Pp = cur.P + 4 * p;
            if (Pp[3] == 0.f) {  // uniform over the contact's lanes
              single(i);
              single(j);
              continue;
            }
            float di = dot3(cur.J[i], a), dj = dot3(cur.J[j], a);
            di += __shfl_xor_sync(gm, di, 1);
            dj += __shfl_xor_sync(gm, dj, 1);
            di += __shfl_xor_sync(gm, di, 2);
            dj += __shfl_xor_sync(gm, dj, 2);
            const float ri = di + (cur.reg * im[i] + cur.bias[i]);
            const float rj = dj + (cur.reg * im[j] + cur.bias[j]);
            float ni, nj;
            RowStep::pair(im[i], im[j], ri, rj, Pp, &ni, &nj);
            const float ai = ni - im[i], aj = nj - im[j];
            im[i] = ni;
            im[j] = nj;
            a[0] += cur.W[i][0] * ai;
            a[1] += cur.W[i][1] * ai;
            a[2] += cur.W[i][2] * ai;
            a[0] += cur.W[j][0] * aj;
            a[1] += cur.W[j][1] * aj;
            a[2] += cur.W[j][2] * aj;
          }
          if (on) {
#pragma unroll
            for (int c = 0; c < 3; ++c) acc[body][3 * part + c] = a[c];
            if (l == 0)
              *reinterpret_cast<float4*>(sc0 + (size_t)SC * k + S_IMP) = make_float4(im[0], im[1], im[2], im[3]);
          }
          __syncwarp();
        }
      }
    }
    for (int kk = lane; kk < cnt; kk += 32) {
      const float* s2 = sc0 + (size_t)SC * kk;
      float* cimp = wf + L.con + CF * wi[L.sccon + k0 + kk] + C_IMP;
      for (int r = 0; r < 4; ++r) cimp[r] = s2[S_IMP + r];
    }
    for (int b = lane; b < nbody; b += 32) {
      const int bd = wi[L.ibody + b0 + b];
      st3(wf + L.dv + 3 * bd, v3(acc[b][0], acc[b][1], acc[b][2]));
      st3(wf + L.dw + 3 * bd, v3(acc[b][3], acc[b][4], acc[b][5]));
    }
    __syncwarp();
  }
}

__global__ void __launch_bounds__(128) pile_k_integrate(const PileGroupDev* G, const int* wseg, int ng, int total,
                                                        int write_diag) {
  const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (t >= total) return;
  const int gi = find_seg(wseg, ng, t);
  const PileGroupDev& g = G[gi];
  const int w = t - wseg[gi];
  if (w >= g.n || !g.I[(size_t)w * g.lay.istride + g.lay.live]) return;
  const WsLay L = ws_layout(g.nb, g.np, g.maxc);
  float* wf = g.scr + (size_t)w * g.sstride;
  const int* wi = reinterpret_cast<const int*>(wf + L.nf);
  const int lane = threadIdx.x & 31;
  const bool rk4 = g.I[(size_t)w * g.lay.istride + g.lay.integ] == NEWT_INTEGRATOR_RK4;
  const bool bad = pile_integrate_world(wf, L, rk4, lane);
  ws_store_state(g, w, L, wf, lane);
  if (write_diag) ws_store_diag(g, w, L, wf, wi, lane);
  else if (lane == 0 && wi[L.misc + 2])
    atomicOr(reinterpret_cast<unsigned*>(g.I + (size_t)w * g.lay.istride + g.lay.status), NEWT_WS_CONTACT_OVERFLOW);
  if (lane == 0 && bad)
    atomicOr(reinterpret_cast<unsigned*>(g.I + (size_t)w * g.lay.istride + g.lay.status), NEWT_WS_NONFINITE);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
extern "C" size_t newt_pile_ws_bytes(int nb, int np, int maxc) {
  WsLay L = ws_layout(nb, np, maxc);
  size_t words = (size_t)(L.nf + L.ni);
  return (words + 31) / 32 * 32 * 4;
}

// Kernel attributes and resident-grid sizes (called outside stream capture).
static int cap128 = 4096, capq[3] = {1216, 1216, 1216}, capv = 608;

// the multi-body island kernels of classes 3-6: bodies and staged contacts
// per island, warps per block
#define NEWT_QUAD_KERNELS(X) X(3, 4, CH_MIN - 1, 4) X(4, CH_MIN, CH_MIN - 1, 4) X(5, CH_MAXC + 1, CH_MAXC, 4)

extern "C" void newt_pile_init() {
  int dev = 0, sms = 1, b1 = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, pile_k_pgs_small<4>, 128, 0);
  cap128 = sms * (b1 > 0 ? b1 : 1) * 2;
#define OCC(cl, mb, mc, wpb)                                                                  \
  {                                                                                           \
    int b = 1;                                                                                \
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, pile_k_pgs_quad<mb, mc, wpb>, 32 * wpb, 0); \
    capq[cl - 3] = sms * (b > 0 ? b : 1);                                                     \
  }
  NEWT_QUAD_KERNELS(OCC)
#undef OCC
  int bv = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bv, pile_k_pgs_levels, 32 * PL_WARPS, 0);
  capv = sms * (bv > 0 ? bv : 1);
}

// Bytes of the island work lists for `slots` island slots.
extern "C" size_t newt_pile_list_bytes(int slots) { return ((size_t)N_ICLASS * (size_t)slots + 32) * sizeof(int); }

// Launches the solver of island class `cl` on stream `s`; list kernels loop
// over their items, so their grids are sized to the resident capacity.
static void launch_class(int cl, const PileGroupDev* dG, const int* dwseg, int ng, const IslandLists& il, int grid,
                         cudaStream_t s) {
  const int* items = il.items + (size_t)cl * il.cap;
  switch (cl) {
    case 0: pile_k_pgs_small<1><<<grid, 128, 0, s>>>(dG, dwseg, ng, items, il.counts, cl); break;
    case 1: pile_k_pgs_small<2><<<grid, 128, 0, s>>>(dG, dwseg, ng, items, il.counts, cl); break;
    case 2: pile_k_pgs_small<4><<<grid, 128, 0, s>>>(dG, dwseg, ng, items, il.counts, cl); break;
#define LAUNCH(c, mb, mc, wpb)                                                                                    \
  case c:                                                                                                         \
    pile_k_pgs_quad<mb, mc, wpb><<<std::min((il.cap + 8 * wpb - 1) / (8 * wpb), capq[c - 3]), 32 * wpb, 0, s>>>( \
        dG, dwseg, ng, items, il.counts, cl);                                                                     \
    break;
    NEWT_QUAD_KERNELS(LAUNCH)
#undef LAUNCH
    default:
      pile_k_pgs_levels<<<std::min((il.cap + PL_WARPS - 1) / PL_WARPS, capv), 32 * PL_WARPS, 0, s>>>(
          dG, dwseg, ng, items, il.counts, cl);
      break;
  }
}

static_assert(N_COUNTERS <= 32, "counters live in the last 32 ints of the lists");
static_assert(N_ICLASS + 2 == NEWT_PILE_KERNELS && N_ICLASS == NEWT_PILE_ISLAND_CLASSES,
              "kernel table of the profiling surface");

// One env-step of every pile world in the table.  `lists` holds the island
// work lists (newt_pile_list_bytes); its last 32 ints are the counters.
// The island classes are independent: they run on three forked streams
// (`side`, joined back with `ev[1..3]` after `ev[0]` forks them); the
// long-island chain, which bounds the step, starts first on `st`.
// `kev` (nullable): 2 * NEWT_PILE_KERNELS timing events; kernel k of the
// step (0 collide, 1 + c the solver of island class c, N_ICLASS + 1
// integrate) is bracketed by kev[2k], kev[2k+1] recorded on the stream it
// runs on (external event nodes under stream capture).
extern "C" int newt_launch_pile_step(const PileGroupDev* dG, const int* dwseg, int ng, int total_worlds,
                                     int total_slots, int* lists, int write_diag, cudaStream_t st,
                                     const cudaStream_t* side, cudaEvent_t* ev, cudaEvent_t* kev) {
  if (total_worlds <= 0) return 0;
  IslandLists il;
  il.items = lists;
  il.cap = total_slots;
  il.stats = write_diag;
  il.counts = lists + (size_t)N_ICLASS * total_slots;
  auto mark = [&](int k, int end, cudaStream_t s) {
    if (kev) cudaEventRecordWithFlags(kev[2 * k + end], s, cudaEventRecordExternal);
  };
  cudaMemsetAsync(il.counts, 0, N_COUNTERS * sizeof(int), st);
  const int wpb = 4;
  mark(0, 0, st);
  pile_k_collide<<<(total_worlds + wpb - 1) / wpb, 32 * wpb, 0, st>>>(dG, dwseg, ng, total_worlds, il);
  mark(0, 1, st);
  // list kernels loop over their items: grids sized to the resident capacity
  const int grid = std::min((total_slots + 127) / 128, cap128);
  cudaEventRecord(ev[0], st);
  for (int k = 0; k < 3; ++k) cudaStreamWaitEvent(side[k], ev[0], 0);
  // stream of each island class: the chain class first on `st`
  const int order[N_ICLASS] = {5, 6, 3, 4, 2, 1, 0};
  const cudaStream_t on[N_ICLASS] = {st, side[1], side[0], side[0], side[1], side[2], side[2]};
  for (int i = 0; i < N_ICLASS; ++i) {
    const int cl = order[i];
    mark(1 + cl, 0, on[i]);
    launch_class(cl, dG, dwseg, ng, il, grid, on[i]);
    mark(1 + cl, 1, on[i]);
  }
  for (int k = 0; k < 3; ++k) {
    cudaEventRecord(ev[1 + k], side[k]);
    cudaStreamWaitEvent(st, ev[1 + k], 0);
  }
  mark(N_ICLASS + 1, 0, st);
  pile_k_integrate<<<(total_worlds + wpb - 1) / wpb, 32 * wpb, 0, st>>>(dG, dwseg, ng, total_worlds, write_diag);
  mark(N_ICLASS + 1, 1, st);
  return N_ICLASS + 2;
}

extern "C" void newt_launch_pile_newton_solve(const PileGroupDev* dG, const int* dwseg, int ng, int total_worlds,
                                              cudaStream_t st);
extern "C" void newt_launch_pile_general_solve(const PileGroupDev* dG, const int* dwseg, int ng, int total_worlds,
                                               cudaStream_t st);

// The contact re-solve of every world of a table at its current state
// (pile_k_reassemble, then the island-class PGS solvers, the dense Newton
// solve or the general-row solve, by `solve` (PileSolve); nothing is
// integrated): the velocity changes and the contacts' impulses the contact
// sensors read.  Returns the launches issued.
extern "C" int newt_launch_pile_resolve(const PileGroupDev* dG, const int* dwseg, int ng, int total_worlds,
                                        int total_slots, int* lists, int solve, cudaStream_t st) {
  if (total_worlds <= 0) return 0;
  IslandLists il;
  il.items = lists;
  il.cap = total_slots;
  il.stats = 0;
  il.counts = lists + (size_t)N_ICLASS * total_slots;
  cudaMemsetAsync(il.counts, 0, N_COUNTERS * sizeof(int), st);
  const int wpb = 4;
  pile_k_reassemble<<<(total_worlds + wpb - 1) / wpb, 32 * wpb, 0, st>>>(dG, dwseg, ng, total_worlds, il);
  if (solve == PS_NEWTON) {
    newt_launch_pile_newton_solve(dG, dwseg, ng, total_worlds, st);
    return 2;
  }
  if (solve == PS_GENERAL) {
    newt_launch_pile_general_solve(dG, dwseg, ng, total_worlds, st);
    return 2;
  }
  const int grid = std::min((total_slots + 127) / 128, cap128);
  for (int cl = N_ICLASS - 1; cl >= 0; --cl) launch_class(cl, dG, dwseg, ng, il, grid, st);
  return 1 + N_ICLASS;
}

// Contact sensors of the named worlds from the re-solve (newt's
// sensor.rs:1030-1087 accelerometer_reading, :1103-1112 touch_reading, with
// the body accelerations of :586-600).  The velocity changes dv, dw (world
// frame) are M^-1 J^T f, so newt's wrench is F = m dv / dt and
// tau_world = I_world dw / dt; a contact's normal force is its facet
// impulses summed over dt (solver.rs:1240-1253), or its normal row's
// impulse over dt where its rows are general.  Writes only the accelerometer and touch entries
// of each output row (the state sensors' kernel writes the rest).
__global__ void __launch_bounds__(64) pile_contact_sensors_kernel(PileGroupDev g, const int* idx, int n,
                                                                 const newt_sensor_desc* S, int ns, float* out,
                                                                 int D) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int w = idx[t];
  const WsLay L = ws_layout(g.nb, g.np, g.maxc);
  const float* wf = g.scr + (size_t)w * g.sstride;
  const int* wi = reinterpret_cast<const int*>(wf + L.nf);
  const int nc = min(max(wi[L.misc + 1], 0), g.maxc);
  const float dt = wf[L.dtg];
  const V3 grav = v3(wf[L.dtg + 1], wf[L.dtg + 2], wf[L.dtg + 3]);
  float* row = out + (size_t)t * D;
  int o = 0;
  for (int k = 0; k < ns; ++k) {
    const int kind = S[k].kind;
    if (kind == NEWT_SENSOR_TOUCH) {
      float sum = 0.f;
      for (int c = 0; c < nc; ++c) {
        const int* cc = wi + L.ci + CI * c;
        if (cc[0] != S[k].index && cc[1] != S[k].index) continue;
        const float* cf = wf + L.con + CF * c;
        // the facets' impulses summed in row order, or a general block's normal row
        const float f = cf[C_ACT] == 2.f ? cf[C_IMP]
                                         : (((0.f + cf[C_IMP]) + cf[C_IMP + 1]) + cf[C_IMP + 2]) + cf[C_IMP + 3];
        sum += fabsf(f / dt);
      }
      row[o++] = sum;
      continue;
    }
    if (kind != NEWT_SENSOR_ACCELEROMETER) {
      o += kind <= NEWT_SENSOR_JOINTVEL ? 1 : (kind == NEWT_SENSOR_FRAMEQUAT ? 4 : 3);
      continue;
    }
    const int b = S[k].index;
    const Q4 q = ld4(wf + L.quat + 4 * b);
    const V3 wb = ld3(wf + L.omg + 3 * b);
    const S3 Ib = lds(wf + L.inertb + 6 * b), Ibi = lds(wf + L.iinvb + 6 * b);
    const float m = wf[L.mass + b];
    const V3 F = ld3(wf + L.dv + 3 * b) * (m / dt);
    const V3 tau_world = qrot(q, smv(Ib, qrot_inv(q, ld3(wf + L.dw + 3 * b)))) / dt;  // R Ib R^T dw / dt
    const V3 a_com = grav + F / m;
    const V3 tau_body = qrot_inv(q, tau_world);
    const V3 gyro = -cross(wb, smv(Ib, wb));
    const V3 alpha_body = smv(Ibi, tau_body + gyro);
    const V3 w_world = qrot(q, wb), a_world = qrot(q, alpha_body);
    const V3 lp = v3(S[k].local_pos[0], S[k].local_pos[1], S[k].local_pos[2]);
    const Q4 lq{S[k].local_quat[0], S[k].local_quat[1], S[k].local_quat[2], S[k].local_quat[3]};
    const V3 r = qrot(q, lp);
    const V3 a_site = a_com + cross(a_world, r) + cross(w_world, cross(w_world, r));
    const V3 v = qrot_inv(qmul(q, lq), a_site - grav);
    row[o++] = v.x; row[o++] = v.y; row[o++] = v.z;
  }
}

extern "C" void newt_launch_pile_contact_sensors(const PileGroupDev& g, const int* idx, int n,
                                                 const newt_sensor_desc* S, int ns, float* out, int D,
                                                 cudaStream_t st) {
  if (n > 0) pile_contact_sensors_kernel<<<(n + 63) / 64, 64, 0, st>>>(g, idx, n, S, ns, out, D);
}

// The collide and integrate stages alone, for the pile worlds solved apart
// (newt_launch_pile_solo_step): the island lists collide appends to are not read there,
// but their counters are zeroed so every append stays in bounds.
extern "C" void pile_k_collide_launch(const PileGroupDev* dG, const int* dwseg, int ng, int total_worlds,
                                      int total_slots, int* lists, cudaStream_t st) {
  IslandLists il;
  il.items = lists;
  il.cap = total_slots;
  il.stats = 0;
  il.counts = lists + (size_t)N_ICLASS * total_slots;
  cudaMemsetAsync(il.counts, 0, N_COUNTERS * sizeof(int), st);
  const int wpb = 4;
  pile_k_collide<<<(total_worlds + wpb - 1) / wpb, 32 * wpb, 0, st>>>(dG, dwseg, ng, total_worlds, il);
}
extern "C" void pile_k_integrate_launch(const PileGroupDev* dG, const int* dwseg, int ng, int total_worlds,
                                        int write_diag, cudaStream_t st) {
  const int wpb = 4;
  pile_k_integrate<<<(total_worlds + wpb - 1) / wpb, 32 * wpb, 0, st>>>(dG, dwseg, ng, total_worlds, write_diag);
}

// Loads every kernel of the pile step and sizes the list grids, so that the
// launches that follow create nothing on the device.  Returns the first CUDA
// error met.
extern "C" cudaError_t newt_pile_prepare_kernels() {
  newt_pile_init();
  cudaFuncAttributes a;
  const void* fns[] = {(const void*)pile_k_collide,       (const void*)pile_k_pgs_small<4>,
                       (const void*)pile_k_pgs_small<2>,    (const void*)pile_k_pgs_small<1>,
                       (const void*)pile_k_pgs_quad<4, CH_MIN - 1, 4>,
                       (const void*)pile_k_pgs_quad<CH_MIN, CH_MIN - 1, 4>,
                       (const void*)pile_k_pgs_quad<CH_MAXC + 1, CH_MAXC, 4>,
                       (const void*)pile_k_pgs_levels,
                       (const void*)pile_k_integrate};
  for (const void* f : fns) {
    cudaError_t e = cudaFuncGetAttributes(&a, f);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// The stages of newt_launch_pile_step issued in order on the one stream `st`
// (no forked streams, no events).  Results are the same: the island classes
// touch disjoint islands.
extern "C" int newt_launch_pile_step_serial(const PileGroupDev* dG, const int* dwseg, int ng, int total_worlds,
                                            int total_slots, int* lists, int write_diag, cudaStream_t st) {
  if (total_worlds <= 0) return 0;
  IslandLists il;
  il.items = lists;
  il.cap = total_slots;
  il.stats = write_diag;
  il.counts = lists + (size_t)N_ICLASS * total_slots;
  cudaMemsetAsync(il.counts, 0, N_COUNTERS * sizeof(int), st);
  const int wpb = 4;
  pile_k_collide<<<(total_worlds + wpb - 1) / wpb, 32 * wpb, 0, st>>>(dG, dwseg, ng, total_worlds, il);
  const int grid = std::min((total_slots + 127) / 128, cap128);
  for (int cl = N_ICLASS - 1; cl >= 0; --cl) launch_class(cl, dG, dwseg, ng, il, grid, st);
  pile_k_integrate<<<(total_worlds + wpb - 1) / wpb, 32 * wpb, 0, st>>>(dG, dwseg, ng, total_worlds, write_diag);
  return N_ICLASS + 2;
}
