// Free-body contact pipeline, collision half: the per-world scratch record,
// its load/store from the world record, geom poses, the sorted-AABB
// broadphase and the ordered narrowphase (one world per warp).
//
// Restates, for FP32 on sm_103a:
//   newt/src/world.rs:1459-1537      World::step phase order (Euler branch)
//   newt/src/broadphase.rs:708-756   geom_aabb; the pair set is the sorted,
//                                    deduplicated (a<b) list that naive
//                                    all-pairs would give for overlapping
//                                    boxes (newt/tests/broadphase.rs:96-118)
//   newt/src/world.rs:2476-2515      collect_contacts_full (pair order, then
//                                    emission order within a pair)
//   newt/src/contact.rs:2509-2587    dispatch + swap/relabel rule
//   newt/src/solver.rs:703-1257      solve_free_bodies_diag_mode (PGS branch)
//   newt/src/solver.rs:1448-1518     pgs_step_non_negative / pgs_step_pyramidal_pair
//   newt/src/solver.rs:1892-2036     row_body_diagonal, contact_regularization,
//                                    row_residual, apply_impulse_delta
//   newt/src/solver.rs:166-384       impedance, safe_solref, reference_accel
//   newt/src/world.rs:1790-1817      step_bodies_euler; world.rs:3223-3245 evaluate
#pragma once
#include "common.cuh"
#include "groups.h"
#include "narrowphase.cuh"

namespace pile {

constexpr int SH_PLANE = 0, SH_SPHERE = 1, SH_BOX = 2, SH_CAPSULE = 3, SH_CYLINDER = 4, SH_ELLIPSOID = 5;  // NEWT_SHAPE_*
constexpr int CF = 39;  // floats per contact in the scratch record
constexpr int CI = 4;   // ints per contact
constexpr int SC = 188;  // floats per active contact in the solver record (a multiple of 4)

// Per-world scratch record in global memory (L1/L2 resident while a world
// is being stepped).  Offsets in floats / ints.
struct WsLay {
  int nb, np, ng, maxc, pcap, words;
  // floats
  int pos, quat, vel, omg, mass, iinvb, inertb, iinvw, dv, dw, size, gpos, gquat, plane, fric, margin, aabb, con;
  int soft, dtg, sc;
  int nf;
  // ints
  int shape, gent, pairs, bits, ci, perm, lcnt, uf, misc;
  int istart, icount, inb, ibstart, ibody, blocal, scid, sccon;
  int ni;
};

__host__ __device__ inline WsLay ws_layout(int nb, int np, int maxc) {
  WsLay L;
  L.nb = nb; L.np = np; L.ng = nb + np; L.maxc = maxc;
  int all = L.ng * (L.ng - 1) / 2;
  L.pcap = all < 2 * maxc ? all : 2 * maxc;
  L.words = (L.ng + 31) / 32;
  int f = 0;
  L.pos = f; f += 3 * nb; L.quat = f; f += 4 * nb; L.vel = f; f += 3 * nb; L.omg = f; f += 3 * nb;
  L.mass = f; f += nb; L.iinvb = f; f += 6 * nb; L.inertb = f; f += 6 * nb; L.iinvw = f; f += 6 * nb;
  L.dv = f; f += 3 * nb; L.dw = f; f += 3 * nb; L.size = f; f += 3 * nb; L.gpos = f; f += 3 * nb;
  L.gquat = f; f += 4 * nb; L.plane = f; f += 7 * np; L.fric = f; f += L.ng; L.margin = f; f += L.ng;
  L.aabb = f; f += 6 * L.ng; L.soft = f; f += 7; L.dtg = f; f += 4;
  L.con = f; f += CF * maxc;
  f = (f + 3) / 4 * 4;  // 16-byte aligned solver records
  L.sc = f; f += SC * maxc;
  L.nf = (f + 3) / 4 * 4;
  int i = 0;
  L.shape = i; i += nb; L.gent = i; i += L.ng; L.pairs = i; i += 2 * L.pcap; L.bits = i; i += L.ng * L.words;
  // perm also holds the broadphase's 64 sort keys and the island masks (2 nb words)
  L.ci = i; i += CI * maxc; L.perm = i; i += max(maxc, max(64, 2 * nb)); L.lcnt = i; i += 33; L.uf = i; i += nb; L.misc = i; i += 4;
  L.istart = i; i += nb; L.icount = i; i += nb; L.inb = i; i += nb; L.ibstart = i; i += nb; L.ibody = i; i += nb;
  L.blocal = i; i += nb; L.scid = i; i += 2 * maxc; L.sccon = i; i += maxc;
  L.ni = (i + 3) / 4 * 4;
  return L;
}

// contact float fields (offsets inside one contact's CF block)
// C_IMP: the contact's row impulses (four facet rows, or up to six general
// rows: normal, two tangents, torsion, two rolling); C_ACT: 0 inactive, 1
// active with facet rows, 2 active with general rows
enum { C_POS = 0, C_N = 3, C_PEN = 6, C_MU = 7, C_IMP = 29, C_ACT = 35 };
// contact int fields: ga, gb, ea, eb
// misc ints: 0 npairs, 1 ncon, 2 overflow, 3 islands

NEWT_D V3 ld3(const float* p) { return v3(p[0], p[1], p[2]); }
NEWT_D void st3(float* p, V3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
NEWT_D Q4 ld4(const float* p) { return Q4{p[0], p[1], p[2], p[3]}; }
NEWT_D S3 lds(const float* p) { return S3{p[0], p[1], p[2], p[3], p[4], p[5]}; }

// ---------------------------------------------------------------------------
// load / store between the world record (global) and the scratch record
// ---------------------------------------------------------------------------
NEWT_D void ws_load(const PileGroupDev& g, int w, const WsLay& L, float* wf, int* wi, int lane) {
  const PileLayout& P = g.lay;
  const float* F = g.F + (size_t)w * P.fstride;
  const int* I = g.I + (size_t)w * P.istride;
  const int nb = L.nb, ng = L.ng;
  for (int k = lane; k < 3 * nb; k += 32) {
    wf[L.pos + k] = F[P.pos + k]; wf[L.vel + k] = F[P.vel + k]; wf[L.omg + k] = F[P.omg + k];
    wf[L.size + k] = F[P.size + k]; wf[L.gpos + k] = F[P.gpos + k];
  }
  for (int k = lane; k < 4 * nb; k += 32) { wf[L.quat + k] = F[P.quat + k]; wf[L.gquat + k] = F[P.gquat + k]; }
  for (int k = lane; k < 6 * nb; k += 32) { wf[L.iinvb + k] = F[P.iinv + k]; wf[L.inertb + k] = F[P.inert + k]; }
  for (int k = lane; k < nb; k += 32) { wf[L.mass + k] = F[P.mass + k]; wi[L.shape + k] = I[P.shape + k]; }
  for (int k = lane; k < 7 * L.np; k += 32) wf[L.plane + k] = F[P.plane + k];
  for (int k = lane; k < ng; k += 32) { wf[L.fric + k] = F[P.fric + k]; wf[L.margin + k] = F[P.margin + k]; wi[L.gent + k] = I[P.gent + k]; }
  if (lane < 7) wf[L.soft + lane] = F[P.soft + lane];
  if (lane < 4) wf[L.dtg + lane] = F[P.dtg + lane];
  __syncwarp();
}

NEWT_D void ws_store_state(const PileGroupDev& g, int w, const WsLay& L, const float* wf, int lane) {
  const PileLayout& P = g.lay;
  float* F = g.F + (size_t)w * P.fstride;
  for (int k = lane; k < 3 * L.nb; k += 32) { F[P.pos + k] = wf[L.pos + k]; F[P.vel + k] = wf[L.vel + k]; F[P.omg + k] = wf[L.omg + k]; }
  for (int k = lane; k < 4 * L.nb; k += 32) F[P.quat + k] = wf[L.quat + k];
}

NEWT_D void ws_store_diag(const PileGroupDev& g, int w, const WsLay& L, const float* wf, const int* wi, int lane) {
  const PileLayout& P = g.lay;
  float* F = g.F + (size_t)w * P.fstride;
  int* I = g.I + (size_t)w * P.istride;
  const int nc = wi[L.misc + 1];
  for (int c = lane; c < nc; c += 32) {
    const float* cf = wf + L.con + CF * c;
    const int* cc = wi + L.ci + CI * c;
    I[P.cpair + 2 * c] = cc[0]; I[P.cpair + 2 * c + 1] = cc[1];
    for (int k = 0; k < 7; ++k) F[P.cdata + 7 * c + k] = cf[C_POS + k];
    for (int k = 0; k < P.rpc; ++k) F[P.imp + P.rpc * c + k] = cf[C_IMP + k];
  }
  if (lane == 0) {
    I[P.ncon] = nc;
    if (wi[L.misc + 2]) I[P.status] |= NEWT_WS_CONTACT_OVERFLOW;
  }
}

NEWT_D GPose geom_pose(const WsLay& L, const float* wf, int e) {
  if (e < L.nb) {
    V3 bp = ld3(wf + L.pos + 3 * e);
    Q4 bq = ld4(wf + L.quat + 4 * e);
    return GPose{bp + qrot(bq, ld3(wf + L.gpos + 3 * e)), qmul(bq, ld4(wf + L.gquat + 4 * e))};
  }
  const float* p = wf + L.plane + 7 * (e - L.nb);
  return GPose{ld3(p), ld4(p + 3)};
}

// ---------------------------------------------------------------------------
// collision: AABBs, sort-and-sweep pair marking, ordered pair list, narrowphase
// ---------------------------------------------------------------------------
// Pairs with a capsule, cylinder or ellipsoid (sizes `za`, `zb`: radius and
// half height, or semi-axes), out of line so that the sphere/box pairs keep
// the narrowphase loop's instruction footprint.  Tries (A, B), then (B, A)
// with *flip set (the caller relabels, newt/src/contact.rs:2561-2586).
static __device__ __noinline__ int np_round_pair(int sa, int sb, GPose pa, GPose pb, const float* za, const float* zb,
                                          float margin, CRes* res, bool* flip) {
  if (sa == SH_CAPSULE && sb == SH_PLANE) return np_capsule_plane(pa, za[0], za[1], margin, pb, res);
  if (sa == SH_CYLINDER && sb == SH_PLANE) return np_cylinder_plane(pa, za[0], za[1], margin, pb, res);
  if (sa == SH_ELLIPSOID && sb == SH_PLANE) return np_ellipsoid_plane(pa, v3(za[0], za[1], za[2]), margin, pb, res);
  if (sa == SH_SPHERE && sb == SH_CYLINDER) return np_sphere_cylinder(pa.p, za[0], pb, zb[0], zb[1], margin, res);
  if (sa == SH_SPHERE && sb == SH_CAPSULE) return np_sphere_capsule(pa.p, za[0], pb, zb[0], zb[1], margin, res);
  if (sa == SH_CAPSULE && sb == SH_CAPSULE) return np_capsule_capsule(pa, za[0], za[1], pb, zb[0], zb[1], margin, res);
  if (sa == SH_SPHERE && sb == SH_ELLIPSOID) return np_sphere_ellipsoid(pa.p, za[0], pb, v3(zb[0], zb[1], zb[2]), margin, res);
  *flip = true;
  if (sb == SH_CAPSULE && sa == SH_PLANE) return np_capsule_plane(pb, zb[0], zb[1], margin, pa, res);
  if (sb == SH_CYLINDER && sa == SH_PLANE) return np_cylinder_plane(pb, zb[0], zb[1], margin, pa, res);
  if (sb == SH_ELLIPSOID && sa == SH_PLANE) return np_ellipsoid_plane(pb, v3(zb[0], zb[1], zb[2]), margin, pa, res);
  if (sb == SH_SPHERE && sa == SH_CYLINDER) return np_sphere_cylinder(pb.p, zb[0], pa, za[0], za[1], margin, res);
  if (sb == SH_SPHERE && sa == SH_CAPSULE) return np_sphere_capsule(pb.p, zb[0], pa, za[0], za[1], margin, res);
  if (sb == SH_SPHERE && sa == SH_ELLIPSOID) return np_sphere_ellipsoid(pb.p, zb[0], pa, v3(za[0], za[1], za[2]), margin, res);
  return 0;
}

NEWT_D void collide(const WsLay& L, float* wf, int* wi, int lane) {
  const int ng = L.ng, nb = L.nb, W = L.words;
  // AABBs per geom index (newt/src/broadphase.rs:708-756); planes unbounded
  for (int k = lane; k < ng; k += 32) {
    int e = wi[L.gent + k];
    float* a = wf + L.aabb + 6 * k;
    if (e >= nb) { a[0] = -INFINITY; a[1] = -INFINITY; a[2] = -INFINITY; a[3] = INFINITY; a[4] = INFINITY; a[5] = INFINITY; continue; }
    GPose p = geom_pose(L, wf, e);
    V3 ext;
    const int sh = wi[L.shape + e];
    if (sh == SH_SPHERE) { float r = wf[L.size + 3 * e]; ext = v3(r, r, r); }
    else if (sh == SH_CAPSULE) {  // |axis| h + r per component (broadphase.rs:720-729)
      const V3 ax = qrot(p.q, v3(0.f, 0.f, 1.f));
      const float r = wf[L.size + 3 * e], hh = wf[L.size + 3 * e + 1];
      ext = v3(fabsf(ax.x) * hh + r, fabsf(ax.y) * hh + r, fabsf(ax.z) * hh + r);
    } else if (sh == SH_CYLINDER) {  // (|x| + |y|) r + |z| h (broadphase.rs:731-739)
      const V3 xa = qrot(p.q, v3(1.f, 0.f, 0.f)), ya = qrot(p.q, v3(0.f, 1.f, 0.f)), za = qrot(p.q, v3(0.f, 0.f, 1.f));
      const float r = wf[L.size + 3 * e], hh = wf[L.size + 3 * e + 1];
      ext = v3((fabsf(xa.x) + fabsf(ya.x)) * r + fabsf(za.x) * hh, (fabsf(xa.y) + fabsf(ya.y)) * r + fabsf(za.y) * hh,
               (fabsf(xa.z) + fabsf(ya.z)) * r + fabsf(za.z) * hh);
    } else {  // boxes and ellipsoids: oriented extents of the half sizes
      V3 h = ld3(wf + L.size + 3 * e);
      M3 R = quat_mat(p.q);
      ext = v3(fabsf(R.m[0][0]) * h.x + fabsf(R.m[0][1]) * h.y + fabsf(R.m[0][2]) * h.z,
               fabsf(R.m[1][0]) * h.x + fabsf(R.m[1][1]) * h.y + fabsf(R.m[1][2]) * h.z,
               fabsf(R.m[2][0]) * h.x + fabsf(R.m[2][1]) * h.y + fabsf(R.m[2][2]) * h.z);
    }
    float mg = wf[L.margin + e];
    ext = ext + v3(mg, mg, mg);
    a[0] = p.p.x - ext.x; a[1] = p.p.y - ext.y; a[2] = p.p.z - ext.z;
    a[3] = p.p.x + ext.x; a[4] = p.p.y + ext.y; a[5] = p.p.z + ext.z;
  }
  for (int k = lane; k < ng * W; k += 32) wi[L.bits + k] = 0;
  __syncwarp();
  // sort geom indices by min.x (odd-even transposition over <= 64 keys held
  // two per lane), then sweep: each geom scans forward while min.x overlaps
  {
    int key0 = lane, key1 = lane + 32;
    // planes (and unused keys) sort last: only body geoms are swept
    float v0 = (key0 < ng && wi[L.gent + key0] < nb) ? wf[L.aabb + 6 * key0] : INFINITY;
    float v1 = (key1 < ng && wi[L.gent + key1] < nb) ? wf[L.aabb + 6 * key1] : INFINITY;
    int* order = wi + L.perm;  // borrows the permutation buffer (at least 64 ints)
    // bitonic sort of 64 (value, index) pairs held two per lane
    for (int size = 2; size <= 64; size <<= 1) {
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        float pv0, pv1; int pk0, pk1;
        if (stride == 32) { pv0 = v1; pk0 = key1; pv1 = v0; pk1 = key0; }
        else {
          pv0 = __shfl_xor_sync(0xffffffffu, v0, stride); pk0 = __shfl_xor_sync(0xffffffffu, key0, stride);
          pv1 = __shfl_xor_sync(0xffffffffu, v1, stride); pk1 = __shfl_xor_sync(0xffffffffu, key1, stride);
        }
        float nv[2]; int nk[2];
        for (int h = 0; h < 2; ++h) {
          const int pos = lane + 32 * h;
          const float v = h ? v1 : v0, pv = h ? pv1 : pv0;
          const int key = h ? key1 : key0, pk = h ? pk1 : pk0;
          const bool up = (pos & size) == 0;
          const bool lower = pos < (pos ^ stride);
          const bool take_min = (up == lower);
          const bool less = (pv < v) || (pv == v && pk < key);
          const bool take_partner = take_min ? less : !less;
          nv[h] = take_partner ? pv : v;
          nk[h] = take_partner ? pk : key;
        }
        v0 = nv[0]; key0 = nk[0]; v1 = nv[1]; key1 = nk[1];
      }
    }
    order[lane] = key0; order[lane + 32] = key1;
    __syncwarp();
    int nsort = 0;
    for (int k = 0; k < ng; ++k) nsort += (wi[L.gent + k] < nb);  // uniform
    for (int h = 0; h < 2; ++h) {
      int i = lane + 32 * h;
      if (i >= nsort) continue;
      int ga = order[i];
      const float* A = wf + L.aabb + 6 * ga;
      for (int j = i + 1; j < nsort; ++j) {
        int gb = order[j];
        const float* B = wf + L.aabb + 6 * gb;
        if (B[0] > A[3]) break;
        if (A[1] > B[4] || B[1] > A[4] || A[2] > B[5] || B[2] > A[5]) continue;
        int lo = ga < gb ? ga : gb, hi = ga < gb ? gb : ga;
        atomicOr(reinterpret_cast<unsigned*>(wi + L.bits + lo * W + (hi >> 5)), 1u << (hi & 31));
      }
    }
    // every body geom pairs with every plane
    for (int k = lane; k < ng; k += 32) {
      if (wi[L.gent + k] < nb) continue;
      for (int b = 0; b < ng; ++b) {
        if (b == k || wi[L.gent + b] >= nb) continue;
        int lo = b < k ? b : k, hi = b < k ? k : b;
        atomicOr(reinterpret_cast<unsigned*>(wi + L.bits + lo * W + (hi >> 5)), 1u << (hi & 31));
      }
    }
  }
  __syncwarp();
  // ordered pair list: rows a in order, bits b > a ascending (warp scan of row counts)
  int base = 0;
  for (int r0 = 0; r0 < ng; r0 += 32) {
    int a = r0 + lane;
    int cnt = 0;
    if (a < ng) for (int k = 0; k < W; ++k) cnt += __popc((unsigned)wi[L.bits + a * W + k]);
    int incl = cnt;
    for (int o = 1; o < 32; o <<= 1) { int t = __shfl_up_sync(0xffffffffu, incl, o); if (lane >= o) incl += t; }
    int off = base + incl - cnt;
    if (a < ng) {
      for (int k = 0; k < W; ++k) {
        unsigned m = (unsigned)wi[L.bits + a * W + k];
        while (m) {
          int bb = __ffs(m) - 1; m &= m - 1;
          if (off < L.pcap) { wi[L.pairs + 2 * off] = a; wi[L.pairs + 2 * off + 1] = 32 * k + bb; }
          ++off;
        }
      }
    }
    base += __shfl_sync(0xffffffffu, incl, 31);
  }
  const int npairs = base < L.pcap ? base : L.pcap;
  int overflow = base > L.pcap;
  __syncwarp();
  // narrowphase: 32 pairs per round, contacts appended in pair order
  int nc = 0;
  for (int r0 = 0; r0 < npairs; r0 += 32) {
    int pi = r0 + lane;
    CRes res[4];
    int cnt = 0, ga = 0, gb = 0;
    bool flip = false;
    if (pi < npairs) {
      ga = wi[L.pairs + 2 * pi]; gb = wi[L.pairs + 2 * pi + 1];
      int ea = wi[L.gent + ga], eb = wi[L.gent + gb];
      int sa = ea < nb ? wi[L.shape + ea] : SH_PLANE, sb = eb < nb ? wi[L.shape + eb] : SH_PLANE;
      float margin = fmaxf(wf[L.margin + ea], wf[L.margin + eb]);
      GPose pa = geom_pose(L, wf, ea), pb = geom_pose(L, wf, eb);
      // try (A, B); otherwise (B, A) and relabel (newt/src/contact.rs:2561-2586)
      if (sa >= SH_CAPSULE || sb >= SH_CAPSULE) {
        cnt = np_round_pair(sa, sb, pa, pb, wf + L.size + 3 * ea, wf + L.size + 3 * eb, margin, res, &flip);
      } else if (sa == SH_SPHERE && sb == SH_PLANE) cnt = np_sphere_plane(pa, wf[L.size + 3 * ea], margin, pb, res);
      else if (sa == SH_BOX && sb == SH_PLANE) cnt = np_box_plane(pa, ld3(wf + L.size + 3 * ea), margin, pb, res);
      else if (sa == SH_SPHERE && sb == SH_SPHERE) cnt = np_sphere_sphere(pa.p, wf[L.size + 3 * ea], pb.p, wf[L.size + 3 * eb], margin, res);
      else if (sa == SH_BOX && sb == SH_BOX) cnt = np_box_box(pa, ld3(wf + L.size + 3 * ea), pb, ld3(wf + L.size + 3 * eb), margin, res);
      else if (sa == SH_SPHERE && sb == SH_BOX) cnt = np_sphere_box(pa, wf[L.size + 3 * ea], pb, ld3(wf + L.size + 3 * eb), margin, res);
      else {
        flip = true;
        if (sb == SH_SPHERE && sa == SH_PLANE) cnt = np_sphere_plane(pb, wf[L.size + 3 * eb], margin, pa, res);
        else if (sb == SH_BOX && sa == SH_PLANE) cnt = np_box_plane(pb, ld3(wf + L.size + 3 * eb), margin, pa, res);
        else if (sb == SH_SPHERE && sa == SH_BOX) cnt = np_sphere_box(pb, wf[L.size + 3 * eb], pa, ld3(wf + L.size + 3 * ea), margin, res);
      }
    }
    int incl = cnt;
    for (int o = 1; o < 32; o <<= 1) { int t = __shfl_up_sync(0xffffffffu, incl, o); if (lane >= o) incl += t; }
    int off = nc + incl - cnt;
    for (int k = 0; k < cnt; ++k) {
      int c = off + k;
      if (c >= L.maxc) { overflow = 1; break; }
      float* cf = wf + L.con + CF * c;
      int* cc = wi + L.ci + CI * c;
      V3 n = flip ? -res[k].n : res[k].n;
      st3(cf + C_POS, res[k].pos); st3(cf + C_N, n); cf[C_PEN] = res[k].pen;
      int ea = wi[L.gent + ga], eb = wi[L.gent + gb];
      cf[C_MU] = fminf(wf[L.fric + ea], wf[L.fric + eb]);
      cc[0] = ga; cc[1] = gb; cc[2] = ea; cc[3] = eb;
    }
    nc += __shfl_sync(0xffffffffu, incl, 31);
  }
  overflow = __any_sync(0xffffffffu, overflow);
  if (lane == 0) {
    wi[L.misc] = npairs;
    wi[L.misc + 1] = nc < L.maxc ? nc : L.maxc;
    wi[L.misc + 2] = overflow;
  }
  __syncwarp();
}


}  // namespace pile
