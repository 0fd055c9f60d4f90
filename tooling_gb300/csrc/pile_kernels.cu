// Free-body contact pipeline, one world per warp (config 1 piles and the
// pile half of config 3): geom poses, sorted-AABB broadphase, narrowphase,
// soft-constraint row assembly, island-parallel projected Gauss-Seidel, and
// semi-implicit Euler integration.
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
//
// Gauss-Seidel is order dependent.  Rows of disjoint contact islands never
// touch the same body, so each lane sweeps whole islands in newt's contact
// order; the result equals the serial sweep.  Velocity accumulators are kept
// in world frame (newt keeps the angular one in body frame and rotates on
// every access; the two are equal up to rounding).
#include "common.cuh"
#include "groups.h"
#include "narrowphase.cuh"

namespace {

constexpr int SH_PLANE = 0, SH_SPHERE = 1, SH_BOX = 2;
constexpr int CF = 39;  // floats per contact in the scratch record
constexpr int CI = 4;   // ints per contact

// Per-world scratch record (shared memory in the fused kernel, global
// memory in the plain kernels).  Offsets in floats / ints.
struct WsLay {
  int nb, np, ng, maxc, pcap, words;
  // floats
  int pos, quat, vel, omg, mass, iinvb, inertb, iinvw, dv, dw, size, gpos, gquat, plane, fric, margin, aabb, con;
  int soft, dtg;
  int nf;
  // ints
  int shape, gent, pairs, bits, ci, perm, lcnt, uf, misc;
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
  L.nf = (f + 3) / 4 * 4;
  int i = 0;
  L.shape = i; i += nb; L.gent = i; i += L.ng; L.pairs = i; i += 2 * L.pcap; L.bits = i; i += L.ng * L.words;
  L.ci = i; i += CI * maxc; L.perm = i; i += maxc; L.lcnt = i; i += 33; L.uf = i; i += nb; L.misc = i; i += 4;
  L.ni = (i + 3) / 4 * 4;
  return L;
}

// contact float fields (offsets inside one contact's CF block)
enum { C_POS = 0, C_N = 3, C_PEN = 6, C_MU = 7, C_T1 = 8, C_ARMA = 11, C_ARMB = 14, C_DIAG = 17, C_REG = 21,
       C_BIAS = 25, C_IMP = 29, C_H01 = 33, C_ACT = 35, C_NR = 36 };
// contact int fields: ga, gb, ea, eb
// misc ints: 0 npairs, 1 ncon, 2 overflow

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
    for (int k = 0; k < 4; ++k) F[P.imp + 4 * c + k] = cf[C_IMP + k];
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
NEWT_D void collide(const WsLay& L, float* wf, int* wi, int lane) {
  const int ng = L.ng, nb = L.nb, W = L.words;
  // AABBs per geom index (newt/src/broadphase.rs:708-756); planes unbounded
  for (int k = lane; k < ng; k += 32) {
    int e = wi[L.gent + k];
    float* a = wf + L.aabb + 6 * k;
    if (e >= nb) { a[0] = -INFINITY; a[1] = -INFINITY; a[2] = -INFINITY; a[3] = INFINITY; a[4] = INFINITY; a[5] = INFINITY; continue; }
    GPose p = geom_pose(L, wf, e);
    V3 ext;
    if (wi[L.shape + e] == SH_SPHERE) { float r = wf[L.size + 3 * e]; ext = v3(r, r, r); }
    else {
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
    int* order = wi + L.perm;  // borrows the permutation buffer (maxc >= 64)
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
      if (sa == SH_SPHERE && sb == SH_PLANE) cnt = np_sphere_plane(pa, wf[L.size + 3 * ea], margin, pb, res);
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

// ---------------------------------------------------------------------------
// row assembly (newt/src/solver.rs:752-1061)
// ---------------------------------------------------------------------------
NEWT_D float impedance(float pos, const float* soft) {
  // effective_solimp + impedance_at_position(pos, 0) (solver.rs:301-326)
  float dmin = fminf(fmaxf(soft[2], 1.0e-4f), 0.9999f), dmax = fminf(fmaxf(soft[3], 1.0e-4f), 0.9999f);
  float width = soft[4] > 0.f ? soft[4] : 0.f, mid = fminf(fmaxf(soft[5], 1.0e-4f), 0.9999f);
  int power = soft[6] >= 1.f ? (int)soft[6] : 1;
  float x = fabsf(pos / width);
  float y;
  if (x <= 0.f) y = 0.f;
  else if (x >= 1.f) y = 1.f;
  else if (x < mid) { float r = x / mid, p = 1.f; for (int i = 0; i < power; ++i) p *= r; y = mid * p; }
  else { float r = (1.f - x) / (1.f - mid), p = 1.f; for (int i = 0; i < power; ++i) p *= r; y = 1.f - (1.f - mid) * p; }
  return dmin + (dmax - dmin) * y;
}

NEWT_D void assemble(const WsLay& L, float* wf, int* wi, int lane) {
  const int nb = L.nb, nc = wi[L.misc + 1];
  const float dt = wf[L.dtg];
  const V3 grav = v3(wf[L.dtg + 1], wf[L.dtg + 2], wf[L.dtg + 3]);
  const float* soft = wf + L.soft;
  // world inverse inertias + zeroed accumulators
  for (int b = lane; b < nb; b += 32) {
    M3 R = quat_mat(ld4(wf + L.quat + 4 * b));
    S3 ib = lds(wf + L.iinvb + 6 * b);
    S3 iw = sym_congr(M3{{{R.m[0][0], R.m[1][0], R.m[2][0]}, {R.m[0][1], R.m[1][1], R.m[2][1]}, {R.m[0][2], R.m[1][2], R.m[2][2]}}}, ib);
    float* o = wf + L.iinvw + 6 * b;
    o[0] = iw.xx; o[1] = iw.yy; o[2] = iw.zz; o[3] = iw.xy; o[4] = iw.xz; o[5] = iw.yz;
    st3(wf + L.dv + 3 * b, v3(0.f, 0.f, 0.f));
    st3(wf + L.dw + 3 * b, v3(0.f, 0.f, 0.f));
  }
  __syncwarp();
  // soft-constraint reference (solver.rs:331-384): safe_solref, direct vs positive
  float tc = soft[0], dr = soft[1];
  const bool direct = tc < 0.f;
  if (!direct && tc < 2.f * dt) tc = 2.f * dt;
  const float dmax = fminf(fmaxf(soft[3], 1.0e-4f), 0.9999f);
  for (int c = lane; c < nc; c += 32) {
    float* cf = wf + L.con + CF * c;
    const int* cc = wi + L.ci + CI * c;
    const int ea = cc[2], eb = cc[3];
    const bool da = ea < nb, db = eb < nb;
    float pen = cf[C_PEN];
    // inactive: both static or force-free gap covers the penetration (gap = 0)
    bool act = (da || db) && pen > 0.f;
    cf[C_ACT] = act ? 1.f : 0.f;
    for (int k = 0; k < 4; ++k) cf[C_IMP + k] = 0.f;
    if (!act) continue;
    V3 n = ld3(cf + C_N), pos = ld3(cf + C_POS);
    // tangent_basis (world.rs:3104-3112), t2 = n x t1 (solver.rs:3458-3463)
    V3 ref = fabsf(n.z) < 0.9f ? v3(0.f, 0.f, 1.f) : v3(1.f, 0.f, 0.f);
    V3 t1 = cross(ref, n);
    float tl = sqrtf(len2(t1));
    t1 = tl == 0.f ? v3(0.f, 0.f, 0.f) : t1 * (1.f / tl);
    V3 t2 = cross(n, t1);
    st3(cf + C_T1, t1);
    V3 arma = da ? pos - ld3(wf + L.pos + 3 * ea) : v3(0.f, 0.f, 0.f);
    V3 armb = db ? pos - ld3(wf + L.pos + 3 * eb) : v3(0.f, 0.f, 0.f);
    st3(cf + C_ARMA, arma); st3(cf + C_ARMB, armb);
    const float mu = cf[C_MU];
    const int nr = 4;  // pyramidal condim 3
    cf[C_NR] = (float)nr;
    const float d = impedance(-pen, soft);
    float tran = 0.f;
    if (da) tran += 1.f / wf[L.mass + ea];
    if (db) tran += 1.f / wf[L.mass + eb];
    const float reg = d > 0.f ? 2.f * mu * mu * ((1.f - d) / d * (tran * (1.f + mu * mu))) : 0.f;
    float b_, k_;
    if (direct) { b_ = -dr / dmax; k_ = -soft[0] / (dmax * dmax); }
    else { b_ = 2.f / (dmax * tc); k_ = d / (dmax * dmax * tc * tc * dr * dr); }
    V3 va = v3(0.f, 0.f, 0.f), vb = v3(0.f, 0.f, 0.f);
    if (da) va = ld3(wf + L.vel + 3 * ea) + cross(qrot(ld4(wf + L.quat + 4 * ea), ld3(wf + L.omg + 3 * ea)), arma);
    if (db) vb = ld3(wf + L.vel + 3 * eb) + cross(qrot(ld4(wf + L.quat + 4 * eb), ld3(wf + L.omg + 3 * eb)), armb);
    V3 dirs[4] = {n + t1 * mu, n - t1 * mu, n + t2 * mu, n - t2 * mu};
    V3 anga[4], angb[4];
    for (int r = 0; r < nr; ++r) {
      V3 dir = dirs[r];
      float aii = 0.f, dvf = 0.f;
      anga[r] = cross(arma, dir); angb[r] = cross(armb, dir);
      if (da) { aii += dot(anga[r], smv(lds(wf + L.iinvw + 6 * ea), anga[r])) + 1.f / wf[L.mass + ea]; dvf += dot(grav * dt, dir); }
      if (db) { aii += dot(angb[r], smv(lds(wf + L.iinvw + 6 * eb), angb[r])) + 1.f / wf[L.mass + eb]; dvf -= dot(grav * dt, dir); }
      float vcur = dot(va - vb, dir);
      float aref = -b_ * vcur - k_ * (-pen);
      cf[C_REG + r] = reg;
      cf[C_DIAG + r] = aii + reg;
      cf[C_BIAS + r] = dvf - aref * dt;
    }
    // pyramidal pair cross responses h01 (solver.rs:1037-1061)
    for (int p = 0; p < 2; ++p) {
      int i0 = 2 * p, i1 = 2 * p + 1;
      float h = 0.f;
      if (da) h += dot(dirs[i0], dirs[i1]) / wf[L.mass + ea] + dot(anga[i0], smv(lds(wf + L.iinvw + 6 * ea), anga[i1]));
      if (db) h += dot(dirs[i0], dirs[i1]) / wf[L.mass + eb] + dot(angb[i0], smv(lds(wf + L.iinvw + 6 * eb), angb[i1]));
      cf[C_H01 + p] = h;
    }
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------
// islands + PGS
// ---------------------------------------------------------------------------
NEWT_D int uf_find(int* uf, int x) {
  while (uf[x] != x) { uf[x] = uf[uf[x]]; x = uf[x]; }
  return x;
}

NEWT_D void islands(const WsLay& L, float* wf, int* wi, int lane) {
  const int nb = L.nb, nc = wi[L.misc + 1];
  if (lane == 0) {
    int* uf = wi + L.uf;
    for (int b = 0; b < nb; ++b) uf[b] = b;
    for (int c = 0; c < nc; ++c) {
      const float* cf = wf + L.con + CF * c;
      const int* cc = wi + L.ci + CI * c;
      if (cf[C_ACT] == 0.f || cc[2] >= nb || cc[3] >= nb) continue;
      int ra = uf_find(uf, cc[2]), rb = uf_find(uf, cc[3]);
      if (ra != rb) { if (ra < rb) uf[rb] = ra; else uf[ra] = rb; }
    }
    // island rank -> lane (round robin over roots in body order)
    int* lanemap = wi + L.lcnt;  // reuse as per-lane counters below; roots map kept in uf sign bits
    int rank = 0;
    int lane_of_root[NEWT_MAX_BODIES];
    for (int b = 0; b < nb; ++b) if (uf_find(uf, b) == b) lane_of_root[b] = (rank++) & 31;
    for (int k = 0; k < 33; ++k) lanemap[k] = 0;
    int* perm = wi + L.perm;
    // counting sort of active contacts by lane, stable in contact order
    for (int c = 0; c < nc; ++c) {
      const float* cf = wf + L.con + CF * c;
      const int* cc = wi + L.ci + CI * c;
      if (cf[C_ACT] == 0.f) continue;
      int body = cc[2] < nb ? cc[2] : cc[3];
      lanemap[lane_of_root[uf_find(uf, body)] + 1]++;
    }
    for (int k = 0; k < 32; ++k) lanemap[k + 1] += lanemap[k];
    int fill[32];
    for (int k = 0; k < 32; ++k) fill[k] = lanemap[k];
    for (int c = 0; c < nc; ++c) {
      const float* cf = wf + L.con + CF * c;
      const int* cc = wi + L.ci + CI * c;
      if (cf[C_ACT] == 0.f) continue;
      int body = cc[2] < nb ? cc[2] : cc[3];
      perm[fill[lane_of_root[uf_find(uf, body)]]++] = c;
    }
  }
  __syncwarp();
}

struct Side { bool dyn; int b; float im; V3 arm; };

NEWT_D float row_resid(const float* wf, const WsLay& L, const Side& A, const Side& B, V3 dir) {
  float s = 0.f;
  if (A.dyn) s += dot(ld3(wf + L.dv + 3 * A.b), dir) + dot(ld3(wf + L.dw + 3 * A.b), cross(A.arm, dir));
  if (B.dyn) s -= dot(ld3(wf + L.dv + 3 * B.b), dir) + dot(ld3(wf + L.dw + 3 * B.b), cross(B.arm, dir));
  return s;
}
NEWT_D void row_apply(float* wf, const WsLay& L, const Side& A, const Side& B, V3 dir, float df) {
  if (df == 0.f) return;
  if (A.dyn) {
    float* dv = wf + L.dv + 3 * A.b;
    float* dw = wf + L.dw + 3 * A.b;
    st3(dv, ld3(dv) + dir * (df * A.im));
    st3(dw, ld3(dw) + smv(lds(wf + L.iinvw + 6 * A.b), cross(A.arm, dir * df)));
  }
  if (B.dyn) {
    float* dv = wf + L.dv + 3 * B.b;
    float* dw = wf + L.dw + 3 * B.b;
    st3(dv, ld3(dv) - dir * (df * B.im));
    st3(dw, ld3(dw) + smv(lds(wf + L.iinvw + 6 * B.b), cross(B.arm, dir * (-df))));
  }
}

NEWT_D void pgs(const WsLay& L, float* wf, int* wi, int lane, int iters) {
  const int nb = L.nb;
  const int beg = wi[L.lcnt + lane], end = wi[L.lcnt + lane + 1];
  for (int it = 0; it < iters; ++it) {
    for (int k = beg; k < end; ++k) {
      const int c = wi[L.perm + k];
      float* cf = wf + L.con + CF * c;
      const int* cc = wi + L.ci + CI * c;
      Side A{cc[2] < nb, cc[2], 0.f, ld3(cf + C_ARMA)}, B{cc[3] < nb, cc[3], 0.f, ld3(cf + C_ARMB)};
      if (A.dyn) A.im = 1.f / wf[L.mass + A.b];
      if (B.dyn) B.im = 1.f / wf[L.mass + B.b];
      const V3 n = ld3(cf + C_N), t1 = ld3(cf + C_T1), t2 = cross(n, t1);
      const float mu = cf[C_MU];
      const V3 dirs[4] = {n + t1 * mu, n - t1 * mu, n + t2 * mu, n - t2 * mu};
      float* imp = cf + C_IMP;
      // normal-facet half-line step on row 0 (solver.rs:1448-1465)
      {
        float res = row_resid(wf, L, A, B, dirs[0]) + cf[C_REG] * imp[0] + cf[C_BIAS];
        float nf = imp[0] - res / cf[C_DIAG];
        float pr = nf < 0.f ? 0.f : nf;
        float dl = pr - imp[0];
        imp[0] = pr;
        row_apply(wf, L, A, B, dirs[0], dl);
      }
      // two opposing-facet pairs as 2x2 blocks (solver.rs:1476-1518)
      for (int p = 0; p < 2; ++p) {
        const int i = 2 * p, j = 2 * p + 1;
        const float h01 = cf[C_H01 + p];
        float ri = row_resid(wf, L, A, B, dirs[i]) + cf[C_REG + i] * imp[i] + cf[C_BIAS + i];
        float rj = row_resid(wf, L, A, B, dirs[j]) + cf[C_REG + j] * imp[j] + cf[C_BIAS + j];
        const float h00 = cf[C_DIAG + i], h11 = cf[C_DIAG + j];
        const float det = h00 * h11 - h01 * h01;
        if (det <= 0.f) {
          for (int q = 0; q < 2; ++q) {
            int r = q ? j : i;
            float res = row_resid(wf, L, A, B, dirs[r]) + cf[C_REG + r] * imp[r] + cf[C_BIAS + r];
            float nf = imp[r] - res / cf[C_DIAG + r];
            float pr = nf < 0.f ? 0.f : nf;
            float dl = pr - imp[r];
            imp[r] = pr;
            row_apply(wf, L, A, B, dirs[r], dl);
          }
          continue;
        }
        const float di = (-ri * h11 + h01 * rj) / det;
        const float dj = (h01 * ri - h00 * rj) / det;
        const float ni = imp[i] + di, nj = imp[j] + dj;
        float a, b;
        if (ni >= 0.f && nj >= 0.f) { a = ni; b = nj; }
        else if (ni < 0.f && nj < 0.f) { a = 0.f; b = 0.f; }
        else if (ni < 0.f) { a = 0.f; b = fmaxf(imp[j] - rj / h11, 0.f); }
        else { a = fmaxf(imp[i] - ri / h00, 0.f); b = 0.f; }
        const float ai = a - imp[i], aj = b - imp[j];
        imp[i] = a; imp[j] = b;
        row_apply(wf, L, A, B, dirs[i], ai);
        row_apply(wf, L, A, B, dirs[j], aj);
      }
    }
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------
// integration (world.rs:1790-1817, 3223-3245)
// ---------------------------------------------------------------------------
NEWT_D void integrate(const WsLay& L, float* wf, int lane, uint32_t* st) {
  const float dt = wf[L.dtg];
  const V3 grav = v3(wf[L.dtg + 1], wf[L.dtg + 2], wf[L.dtg + 3]);
  bool bad = false;
  for (int b = lane; b < L.nb; b += 32) {
    Q4 q = ld4(wf + L.quat + 4 * b);
    V3 om = ld3(wf + L.omg + 3 * b);
    V3 iw = smv(lds(wf + L.inertb + 6 * b), om);
    V3 gyro = -cross(om, iw);
    V3 dang = smv(lds(wf + L.iinvb + 6 * b), gyro);
    V3 lv = ld3(wf + L.vel + 3 * b) + grav * dt + ld3(wf + L.dv + 3 * b);
    V3 av = om + dang * dt + qrot_inv(q, ld3(wf + L.dw + 3 * b));
    V3 p = ld3(wf + L.pos + 3 * b) + lv * dt;
    Q4 nq = q_integrate(q, av, dt);
    st3(wf + L.pos + 3 * b, p); st3(wf + L.vel + 3 * b, lv); st3(wf + L.omg + 3 * b, av);
    wf[L.quat + 4 * b] = nq.x; wf[L.quat + 4 * b + 1] = nq.y; wf[L.quat + 4 * b + 2] = nq.z; wf[L.quat + 4 * b + 3] = nq.w;
    bad |= !(isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(lv.x) && isfinite(lv.y) && isfinite(lv.z) &&
             isfinite(av.x) && isfinite(av.y) && isfinite(av.z));
  }
  if (__any_sync(0xffffffffu, bad)) *st |= NEWT_WS_NONFINITE;
  __syncwarp();
}

NEWT_D void world_step(const WsLay& L, float* wf, int* wi, int lane, int iters, uint32_t* st) {
  collide(L, wf, wi, lane);
  assemble(L, wf, wi, lane);
  islands(L, wf, wi, lane);
  pgs(L, wf, wi, lane, iters);
  integrate(L, wf, lane, st);
}

}  // namespace

// ---------------------------------------------------------------------------
// fused: one warp per world, scratch record in shared memory, whole horizon
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32) pile_fused_kernel(PileGroupDev g, int base, int count, int n_steps) {
  extern __shared__ float smem[];
  const int item = blockIdx.x;
  if (item >= count) return;
  const int w = base + item;
  if (w >= g.n) return;
  const int* I = g.I + (size_t)w * g.lay.istride;
  if (!I[g.lay.live]) return;
  const WsLay L = ws_layout(g.nb, g.np, g.maxc);
  float* wf = smem;
  int* wi = reinterpret_cast<int*>(smem + L.nf);
  const int lane = threadIdx.x;
  ws_load(g, w, L, wf, wi, lane);
  const int iters = I[g.lay.iters];
  uint32_t st = 0;
  for (int s = 0; s < n_steps; ++s) world_step(L, wf, wi, lane, iters, &st);
  ws_store_state(g, w, L, wf, lane);
  ws_store_diag(g, w, L, wf, wi, lane);
  if (lane == 0 && st) atomicOr(reinterpret_cast<unsigned*>(g.I + (size_t)w * g.lay.istride + g.lay.status), st);
}

// persistent: blocks (one warp each) pull (group, base, count) items
__global__ void __launch_bounds__(32) pile_persistent_kernel(const PileGroupDev* groups, const int* queue, int* counter,
                                                             int n_items, int n_steps) {
  extern __shared__ float smem[];
  const int lane = threadIdx.x;
  for (;;) {
    int it = 0;
    if (lane == 0) it = atomicAdd(counter, 1);
    it = __shfl_sync(0xffffffffu, it, 0);
    if (it >= n_items) return;
    const PileGroupDev g = groups[queue[3 * it]];
    const int base = queue[3 * it + 1], count = queue[3 * it + 2];
    const WsLay L = ws_layout(g.nb, g.np, g.maxc);
    float* wf = smem;
    int* wi = reinterpret_cast<int*>(smem + L.nf);
    for (int k = 0; k < count; ++k) {
      const int w = base + k;
      if (w >= g.n) break;
      const int* I = g.I + (size_t)w * g.lay.istride;
      if (!I[g.lay.live]) continue;
      ws_load(g, w, L, wf, wi, lane);
      const int iters = I[g.lay.iters];
      uint32_t st = 0;
      for (int s = 0; s < n_steps; ++s) world_step(L, wf, wi, lane, iters, &st);
      ws_store_state(g, w, L, wf, lane);
      ws_store_diag(g, w, L, wf, wi, lane);
      if (lane == 0 && st) atomicOr(reinterpret_cast<unsigned*>(g.I + (size_t)w * g.lay.istride + g.lay.status), st);
      __syncwarp();
    }
  }
}

// ---------------------------------------------------------------------------
// plain: one launch per stage per step, scratch record in global memory
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool plain_world(const PileGroupDev& g, int* w_out) {
  const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  *w_out = w;
  if (w >= g.n) return false;
  return g.I[(size_t)w * g.lay.istride + g.lay.live] != 0;
}

__global__ void pile_plain_collide(PileGroupDev g, float* scr) {
  int w;
  if (!plain_world(g, &w)) return;
  const WsLay L = ws_layout(g.nb, g.np, g.maxc);
  float* wf = scr + (size_t)w * (L.nf + L.ni);
  int* wi = reinterpret_cast<int*>(wf + L.nf);
  const int lane = threadIdx.x & 31;
  ws_load(g, w, L, wf, wi, lane);
  collide(L, wf, wi, lane);
}
__global__ void pile_plain_assemble(PileGroupDev g, float* scr) {
  int w;
  if (!plain_world(g, &w)) return;
  const WsLay L = ws_layout(g.nb, g.np, g.maxc);
  float* wf = scr + (size_t)w * (L.nf + L.ni);
  int* wi = reinterpret_cast<int*>(wf + L.nf);
  assemble(L, wf, wi, threadIdx.x & 31);
}
__global__ void pile_plain_solve(PileGroupDev g, float* scr) {
  int w;
  if (!plain_world(g, &w)) return;
  const WsLay L = ws_layout(g.nb, g.np, g.maxc);
  float* wf = scr + (size_t)w * (L.nf + L.ni);
  int* wi = reinterpret_cast<int*>(wf + L.nf);
  const int lane = threadIdx.x & 31;
  islands(L, wf, wi, lane);
  pgs(L, wf, wi, lane, g.I[(size_t)w * g.lay.istride + g.lay.iters]);
}
__global__ void pile_plain_integrate(PileGroupDev g, float* scr) {
  int w;
  if (!plain_world(g, &w)) return;
  const WsLay L = ws_layout(g.nb, g.np, g.maxc);
  float* wf = scr + (size_t)w * (L.nf + L.ni);
  int* wi = reinterpret_cast<int*>(wf + L.nf);
  const int lane = threadIdx.x & 31;
  uint32_t st = 0;
  integrate(L, wf, lane, &st);
  ws_store_state(g, w, L, wf, lane);
  ws_store_diag(g, w, L, wf, wi, lane);
  if (lane == 0 && st) atomicOr(reinterpret_cast<unsigned*>(g.I + (size_t)w * g.lay.istride + g.lay.status), st);
}

extern "C" size_t newt_pile_ws_bytes(int nb, int np, int maxc) {
  WsLay L = ws_layout(nb, np, maxc);
  return (size_t)(L.nf + L.ni) * 4;
}

extern "C" size_t newt_pile_plain_scratch_bytes(const PileGroupDev& g) {
  return newt_pile_ws_bytes(g.nb, g.np, g.maxc) * (size_t)(g.cap > 0 ? g.cap : 1);
}

extern "C" void newt_launch_pile_plain(const PileGroupDev& g, void* scratch, cudaStream_t st, int* launches) {
  const int wpb = 4;  // fixed tile: 4 worlds (warps) per block
  int grid = (g.n + wpb - 1) / wpb;
  if (grid == 0) { *launches = 0; return; }
  float* s = (float*)scratch;
  pile_plain_collide<<<grid, 32 * wpb, 0, st>>>(g, s);
  pile_plain_assemble<<<grid, 32 * wpb, 0, st>>>(g, s);
  pile_plain_solve<<<grid, 32 * wpb, 0, st>>>(g, s);
  pile_plain_integrate<<<grid, 32 * wpb, 0, st>>>(g, s);
  *launches = 4;
}

static void set_smem(size_t bytes) {
  static size_t done = 0;
  if (bytes > done) {
    cudaFuncSetAttribute(pile_fused_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    cudaFuncSetAttribute(pile_persistent_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    done = bytes;
  }
}

extern "C" void newt_launch_pile_fused(const PileGroupDev& g, int base, int count, int n_steps, cudaStream_t st) {
  if (count <= 0) return;
  size_t smem = newt_pile_ws_bytes(g.nb, g.np, g.maxc);
  set_smem(smem);
  pile_fused_kernel<<<count, 32, smem, st>>>(g, base, count, n_steps);
}

extern "C" void newt_launch_pile_persistent(const PileGroupDev* dgroups, const int* dqueue, int* dcounter, int n_items,
                                            int n_steps, int grid, size_t smem, cudaStream_t st) {
  if (grid <= 0 || n_items <= 0) return;
  set_smem(smem);
  pile_persistent_kernel<<<grid, 32, smem, st>>>(dgroups, dqueue, dcounter, n_items, n_steps);
}

extern "C" int newt_pile_blocks_per_sm(size_t smem) {
  set_smem(smem);
  int nb = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, pile_persistent_kernel, 32, smem);
  return nb < 1 ? 1 : nb;
}
