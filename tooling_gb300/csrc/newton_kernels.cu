// Tree-contact step: worlds holding one articulated tree whose link geoms
// touch static planes (the quadruped workload), stepped with newt's
// semi-implicit Euler and its joint tree-contact solve.  Per env-step:
//
//   tree_aba_kernel        thread per world (tree_kernels.cu): a_free, the
//                          ABA with the implicit damping fold, into qacc
//   tc_k_solve             warp per world (this file): forward kinematics,
//                          link-plane contacts, link COM Jacobians and the
//                          mass matrix, its Cholesky factors, the Jacobian
//                          row of every cone facet, A = J M^-1 J^T, the
//                          regulariser and bias, Newton or PGS, and
//                          qacc = a_free + M^-1 J^T f / dt
//   tree_integrate_kernel  thread per world (tree_kernels.cu)
// Under RK4 (per world) a_free is the explicit ABA, the solve factors M
// without the damping term, J^T f / dt goes to the world's scratch, and the
// integrate stage runs the RK4 step with it added to qfrc.
//
// Restates, for FP32 on sm_103a:
//   newt/src/solver.rs:2805-3366  solve_tree_contacts (Euler form:
//                                 factors of M + dt*B, implicit free ABA)
//   newt/src/solver.rs:3537-3600  world_jacobian_for_side
//   newt/src/solver.rs:3719-3797  tree_body_invweight0, tree_contact_diag_approx
//   newt/src/solver.rs:1960-1974  contact_regularization_from_diag
//   newt/src/newton.rs:275-620    NewtonSystem::solve, exact_pyramidal_line_search
//   newt/src/jacobian.rs:38-120   point_jacobian
//   newt/src/dynamics.rs:474-648  mass_matrix, cholesky; tree.rs:645-684
//   newt/src/tree.rs:771-858      forward_kinematics
//   newt/src/contact.rs:269-400   sphere/box/capsule-plane contacts and the
//                                 (plane, geom) label swap of :2509-2587
// Changes that only move rounding:
//   * M = sum_l J_l^T diag(m_l, I_l) J_l from the link COM Jacobians (the CRB
//     recursion's matrix), their lever arms carried up the chain joint by
//     joint, as the recursion's local transforms carry them;
//   * A = Y^T Y with Y = L^-1 J^T (newt solves M^-1 J^T column by column);
//   * the line search walks newt's candidate set (the breakpoints where a
//     non-negative coordinate reaches zero, and each window's minimiser of
//     the piecewise-quadratic cost) with H p and H s updated one column per
//     breakpoint instead of re-multiplied per candidate; newt's
//     finite-difference slope inside a window is the masked direction used
//     here, and its window minimiser mid - g(mid).s / s.Hs equals -c1/c2;
//   * qacc adds M^-1 J^T f / dt to a_free instead of re-running the ABA with
//     the contact forces (the ABA is linear in the applied forces).
// FP64: when the FP32 Cholesky of the Newton Hessian has a pivot ratio
// (max L_ii / min L_ii)^2 above 1e6, the factor and the direction solves are
// redone in FP64 (status bit NEWT_WS_FP64_FALLBACK).  Trees above 24 DoF sum
// the mass matrix in FP64 (from the f32 Jacobians; each product is exact in
// double) and get one FP64 residual-refinement step of the mass-matrix solve
// that turns the contact impulses into accelerations: with x the FP32
// solution of M' x = J^T f / dt (M' = M + dt B, its FP64 sum rounded and
// factored in FP32), r = J^T f / dt - M' x is formed in FP64 with the FP64
// M', the correction solved in FP64 with the FP32 factor, and x += that
// correction (the mixed-precision refinement of the solve newt runs in
// cholesky_solve, dynamics.rs:630-648).  On a straight 45-DoF chain an f32
// sum of M alone leaves 3e-3 of relative error in qacc after an f32 solve,
// the FP64 sum with the refinement 1e-5.
#include <algorithm>

#include "../../include/newt_gpu.h"
#include "common.cuh"
#include "groups.h"
#include "narrowphase.cuh"
#include "newton_dense.cuh"
#include "runtime.h"

namespace {

constexpr unsigned FULL = 0xffffffffu;
using dense::warp_cholesky;
using dense::warp_dot;
using dense::warp_dot_d;
using dense::warp_llt_solve;
using dense::warp_llt_solve_mixed;
using dense::warp_matvec;
using dense::warp_sum;
using dense::warp_sumd;
constexpr int TC_WARPS = 1;  // warps (worlds) per block
constexpr int CREC = TC_CREC;  // floats per contact record
// contact record fields
// K_LINK: the link of the row's tree side with sign K_SIGN; K_LINK2: for an
// in-tree pair, the link of side b (sign -1), else -1; K_MUT, K_MUR: the
// torsional and rolling friction (min of the two geoms'); K_ROW: the first
// row, -1 for a contact without rows
enum { K_GA = 0, K_GB = 1, K_LINK = 2, K_SIGN = 3, K_POS = 4, K_N = 7, K_PEN = 10, K_GAP = 11, K_MU = 12,
       K_SR = 13, K_SI = 15, K_CONDIM = 20, K_ROW = 21, K_LINK2 = 22, K_MUT = 23, K_MUR = 24 };
static_assert(K_MUR < CREC, "contact record");
constexpr int GREC = TC_GREC;  // SoA geom model rows: size3 pos3 quat4 fric margin gap solref2 solimp5 torsional rolling
enum { G_SIZE = 0, G_POS = 3, G_QUAT = 6, G_FRIC = 10, G_MARGIN = 11, G_GAP = 12, G_SR = 13, G_SI = 15, G_TF = 20,
       G_RF = 21 };
// Row codes (rfac): 0-3 the pyramidal facets n +- mu t1, n +- mu t2 of a
// condim-3 contact; otherwise -1 - kind, kind 0 normal, 1-2 the tangents,
// 3 torsion (angular about n), 4-5 rolling (angular about t1, t2), the rows
// of contact_row_directions (newt/src/solver.rs:3401-3429).
enum { R_NORMAL = -1, R_T1 = -2, R_T2 = -3, R_TORSION = -4, R_ROLL1 = -5, R_ROLL2 = -6 };
NEWT_HD bool row_angular(int f) { return f <= R_TORSION; }
enum { JF = 0, JX = 1, JH = 2, JS = 3 };


// In-tree pairs (geoms on two links of the tree): newt's routine for the
// shape pair as (A, B), else as (B, A) with *flip set (the caller relabels,
// newt/src/contact.rs:2561-2586).  Sizes `za`, `zb`: radius / half extents /
// radius and half height.  Out of line: the solve kernel's registers stay
// sized for its own loops.
static __device__ __noinline__ int np_link_pair(int sa, int sb, GPose pa, GPose pb, V3 za, V3 zb, float margin,
                                                CRes* res, bool* flip) {
  *flip = false;
  if (sa == NEWT_SHAPE_SPHERE && sb == NEWT_SHAPE_SPHERE) return np_sphere_sphere(pa.p, za.x, pb.p, zb.x, margin, res);
  if (sa == NEWT_SHAPE_BOX && sb == NEWT_SHAPE_BOX) return np_box_box(pa, za, pb, zb, margin, res);
  if (sa == NEWT_SHAPE_SPHERE && sb == NEWT_SHAPE_BOX) return np_sphere_box(pa, za.x, pb, zb, margin, res);
  if (sa == NEWT_SHAPE_SPHERE && sb == NEWT_SHAPE_CAPSULE) return np_sphere_capsule(pa.p, za.x, pb, zb.x, zb.y, margin, res);
  if (sa == NEWT_SHAPE_SPHERE && sb == NEWT_SHAPE_CYLINDER)
    return np_sphere_cylinder(pa.p, za.x, pb, zb.x, zb.y, margin, res);
  if (sa == NEWT_SHAPE_CAPSULE && sb == NEWT_SHAPE_CAPSULE)
    return np_capsule_capsule(pa, za.x, za.y, pb, zb.x, zb.y, margin, res);
  if (sa == NEWT_SHAPE_SPHERE && sb == NEWT_SHAPE_ELLIPSOID) return np_sphere_ellipsoid(pa.p, za.x, pb, zb, margin, res);
  *flip = true;
  if (sb == NEWT_SHAPE_SPHERE && sa == NEWT_SHAPE_BOX) return np_sphere_box(pb, zb.x, pa, za, margin, res);
  if (sb == NEWT_SHAPE_SPHERE && sa == NEWT_SHAPE_CAPSULE) return np_sphere_capsule(pb.p, zb.x, pa, za.x, za.y, margin, res);
  if (sb == NEWT_SHAPE_SPHERE && sa == NEWT_SHAPE_CYLINDER)
    return np_sphere_cylinder(pb.p, zb.x, pa, za.x, za.y, margin, res);
  if (sb == NEWT_SHAPE_SPHERE && sa == NEWT_SHAPE_ELLIPSOID) return np_sphere_ellipsoid(pb.p, zb.x, pa, za, margin, res);
  return 0;  // refused at upload
}

// A contact row's direction: the normal, or facet f of the pyramid,
// n +- mu t1, n +- mu t2 (solver.rs:3401-3429, tangent_basis world.rs:3104-3112).
NEWT_D V3 row_direction(const float* cc, int f) {
  const V3 n = v3(cc[K_N], cc[K_N + 1], cc[K_N + 2]);
  if (f == R_NORMAL || f == R_TORSION) return n;
  const float mu = cc[K_MU];
  const V3 ref = fabsf(n.z) < 0.9f ? v3(0.f, 0.f, 1.f) : v3(1.f, 0.f, 0.f);
  V3 t1 = cross(ref, n);
  t1 = t1 * (1.f / sqrtf(len2(t1)));
  if (f < 0) return (f == R_T1 || f == R_ROLL1) ? t1 : cross(n, t1);
  const V3 t = f < 2 ? t1 : cross(n, t1);
  return n + t * ((f & 1) ? -mu : mu);
}

NEWT_D Q4 q_axis_angle(V3 axis, float angle) {  // math.rs:574-580
  const float l = sqrtf(len2(axis));
  const V3 a = l > 0.f ? axis * (1.f / l) : v3(0.f, 0.f, 0.f);
  float s, c;
  sincosf(angle * 0.5f, &s, &c);
  return Q4{a.x * s, a.y * s, a.z * s, c};
}
NEWT_D V3 ldv3(const float* p) { return v3(p[0], p[1], p[2]); }
NEWT_D void stv3(float* p, V3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }

// soft-constraint parameters (solver.rs:166-384)
struct Soft { float tc, dr, dmin, dmax, width, mid; int power; };
NEWT_D float clamp_imp(float v) { return v < 1.0e-4f ? 1.0e-4f : (v > 0.9999f ? 0.9999f : v); }
NEWT_D float impedance_at(float position, const Soft& s) {
  const float dmin = clamp_imp(s.dmin), dmax = clamp_imp(s.dmax), mid = clamp_imp(s.mid);
  const float width = s.width > 0.f ? s.width : 0.f;
  const int power = s.power > 1 ? s.power : 1;
  float x = position / width;
  if (x < 0.f) x = -x;
  float y;
  if (x <= 0.f) y = 0.f;
  else if (x >= 1.f) y = 1.f;
  else if (x < mid) { float r = x / mid, p = 1.f; for (int i = 0; i < power; ++i) p *= r; y = mid * p; }
  else { float r = (1.f - x) / (1.f - mid), p = 1.f; for (int i = 0; i < power; ++i) p *= r; y = 1.f - (1.f - mid) * p; }
  return dmin + (dmax - dmin) * y;
}
NEWT_D float reference_accel(float position, float velocity, float tc, float dr, const Soft& s, float dt) {
  const bool direct = tc < 0.f;
  if (!direct && tc < 2.f * dt) tc = 2.f * dt;  // safe_solref (solver.rs:331-338)
  const float dmax = clamp_imp(s.dmax);
  const float d = impedance_at(position, s);
  float b, k;
  if (direct) { b = -dr / dmax; k = -tc / (dmax * dmax); }
  else { b = 2.f / (dmax * tc); k = d / (dmax * dmax * tc * tc * dr * dr); }
  return -b * velocity - k * position;
}

// ---------------------------------------------------------------------------
// per-world scratch (world-major, floats); matrices column-major
// ---------------------------------------------------------------------------
struct TcLay {
  int L, nv, ng, maxc, ld;
  int jv, jw, iw, con, jt, j0, H, LH, LHd, imp, misc, qfc, mc, rd, words;
};
NEWT_HD int up4(int n) { return (n + 3) / 4 * 4; }
constexpr int REFINE_NV = 24;  // DoF above which M is summed and the mass-matrix solve refined in FP64
NEWT_HD TcLay tc_layout(int L, int nv, int ng, int maxc, int rpc) {
  TcLay t;
  t.L = L; t.nv = nv; t.ng = ng; t.maxc = maxc;
  t.ld = up4(rpc * maxc);
  int f = 0;
  t.jv = f; f += up4(3 * nv * L);
  t.jw = f; f += up4(3 * nv * L);
  t.iw = f; f += up4(7 * L);  // world inertias (6 per link), then link masses
  t.con = f; f += up4(CREC * maxc);
  t.jt = f; f += up4(nv * t.ld);  // J^T, then Y in place, when the rows exceed the shared tile
  t.j0 = f; f += up4(nv * t.ld);  // J^T kept for the contact force J^T f
  t.H = f; f += up4(t.ld * t.ld);
  t.LH = f; f += up4(t.ld * t.ld);       // factor of H when it exceeds the shared tile
  t.LHd = f; f += up4(2 * t.ld * t.ld);  // FP64 factor (offset is a multiple of 4 floats)
  t.imp = f; f += up4(t.ld);
  t.misc = f; f += 8;  // ncon, nrows, newton iterations
  t.qfc = f; f += up4(nv);  // RK4 worlds: J^T f / dt, held over the integrator's stages
  t.mc = f; f += nv > REFINE_NV ? up4(2 * nv * nv) : 0;  // trees above REFINE_NV DoF: M' in FP64 (lower)
  t.rd = f; f += nv > REFINE_NV ? up4(4 * nv) : 0;   // and two FP64 vectors (right-hand side, residual)
  t.words = (f + 31) / 32 * 32;
  return t;
}
// Per-world shared working set: solver vectors, row maps, link poses, the
// two mass-matrix factors, link inverse weights, a tile that first holds the
// link COM Jacobians and inertias and later the Newton factor, and the
// Jacobian rows (overwritten in place by Y = L^-1 J^T).  The tile and the rows
// live here when the active rows fit NRS (sequential Cholesky and
// triangular-solve steps then wait on shared memory instead of L2).  NRS
// trades the tile against residency: 20 rows (five contacts; a standing
// quadruped has about two) keep the block at ~12 KB, 18 warps per SM; a
// sweep of 48/32/24/20/16 rows on 16384 quadrupeds gave 7.2/7.1/8.0/8.2/8.1M
// env-steps/s.
enum { V_X = 0, V_D, V_G, V_B, V_REG, V_DIAG, V_U, V_V, V_P, V_S, N_VEC };
constexpr int NRS = 20;
struct TcSmem { int vl, ldr, nrs, vec, rmap, pose, lm, ldf, tw, lh, jy, words; };
NEWT_HD TcSmem tc_smem(int L, int nv, int maxc, int rpc) {
  TcSmem m;
  m.ldr = up4(rpc * maxc);
  m.vl = m.ldr > up4(nv) ? m.ldr : up4(nv);
  m.nrs = m.ldr < NRS ? m.ldr : NRS;
  int f = 0;
  m.vec = f; f += N_VEC * m.vl;
  m.rmap = f; f += 2 * m.ldr;
  m.pose = f; f += up4(7 * L);
  m.lm = f; f += up4(nv * nv);
  m.ldf = f; f += up4(nv * nv);
  m.tw = f; f += 2 * up4(L);  // translation, then rotation inverse weights per link
  m.lh = f; f += m.nrs * m.nrs;
  m.jy = f; f += up4(nv * m.nrs);
  m.words = f;
  return m;
}

// Two independent n x n factorisations (same order) in one pass, so the
// lanes' dependent update chains of the two matrices overlap.  Returns false
// when either has a non-positive pivot.
NEWT_D bool warp_cholesky2(float* A, float* B, int n, int ld, int lane) {
  for (int k = 0; k < n; ++k) {
    __syncwarp();
    const float akk = A[(size_t)k * ld + k], bkk = B[(size_t)k * ld + k];
    if (!(akk > 0.f) || !(bkk > 0.f)) return false;
    const float la = sqrtf(akk), lb = sqrtf(bkk);
    const float ia = 1.f / la, ib = 1.f / lb;
    __syncwarp();
    for (int i = k + 1 + lane; i < n; i += 32) {
      A[(size_t)k * ld + i] *= ia;
      B[(size_t)k * ld + i] *= ib;
    }
    if (lane == 0) {
      A[(size_t)k * ld + k] = la;
      B[(size_t)k * ld + k] = lb;
    }
    __syncwarp();
    for (int j = k + 1; j < n; ++j) {
      const float ajk = A[(size_t)k * ld + j], bjk = B[(size_t)k * ld + j];
      for (int i = j + lane; i < n; i += 32) {
        A[(size_t)j * ld + i] -= A[(size_t)k * ld + i] * ajk;
        B[(size_t)j * ld + i] -= B[(size_t)k * ld + i] * bjk;
      }
    }
  }
  __syncwarp();
  return true;
}

// Solves L^T z = rhs in place on the shared vector `v` (backward
// substitution by row dot products of the column-major factor L).
NEWT_D void warp_lt_solve(const float* Lf, int n, int ld, float* v, int lane) {
  for (int k = n - 1; k >= 0; --k) {
    __syncwarp();
    float s = 0.f;
    for (int m = k + 1 + lane; m < n; m += 32) s += Lf[(size_t)k * ld + m] * v[m];
    s = warp_sum(s);
    const float zk = (v[k] - s) / Lf[(size_t)k * ld + k];
    __syncwarp();
    if (lane == 0) v[k] = zk;
  }
  __syncwarp();
}

}  // namespace


namespace {

// Columns of the world-frame point Jacobian of link `l` at `pt`
// (jacobian.rs:38-120), walking the chain to the root; `col(k, rot, trans)`
// receives every DoF column of the chain.  The lever arm from each joint to
// `pt` is carried up the chain as `d`, the point relative to the current
// link's origin, advanced by the joint's own offsets (origin_i - origin_p =
// R_p jp (+ R_p axis q for a slide) - R_i jc); differencing world positions
// instead rounds every arm at the scale of the distance from the world
// origin, which on long chains costs most of the digits of the short arms
// between neighbouring links.
template <class F>
NEWT_D void chain_columns(const TreeGroupDev& g, int w, const float* pose, int l, V3 pt, F col) {
  const int cap = g.cap;
  V3 d = pt - ldv3(pose + 7 * l);
  for (int i = l; i >= 0; i = g.topo[4 * i]) {
    const int jt = g.topo[4 * i + 1], vo = g.topo[4 * i + 3];
    const float* pi = pose + 7 * i;
    const Q4 oi = Q4{pi[3], pi[4], pi[5], pi[6]};
    if (jt == JF) {  // the root (links 1.. have hinge, slide or fixed joints)
      for (int k = 0; k < 3; ++k) {
        const V3 aw = qrot(oi, v3(k == 0 ? 1.f : 0.f, k == 1 ? 1.f : 0.f, k == 2 ? 1.f : 0.f));
        col(vo + k, aw, cross(aw, d));
        col(vo + 3 + k, v3(0.f, 0.f, 0.f), aw);
      }
    }
    if (i == 0) break;
    const float* pp = pose + 7 * g.topo[4 * i];
    const Q4 po = Q4{pp[3], pp[4], pp[5], pp[6]};
    const V3 jp = v3(g.jp[(3 * i) * cap + w], g.jp[(3 * i + 1) * cap + w], g.jp[(3 * i + 2) * cap + w]);
    const V3 jc = v3(g.jc[(3 * i) * cap + w], g.jc[(3 * i + 1) * cap + w], g.jc[(3 * i + 2) * cap + w]);
    const V3 cw = qrot(oi, jc);  // joint anchor relative to link i's origin
    V3 step = qrot(po, jp) - cw;  // link i's origin relative to its parent's
    if (jt == JH || jt == JS) {
      const V3 ax = v3(g.axis[(3 * i) * cap + w], g.axis[(3 * i + 1) * cap + w], g.axis[(3 * i + 2) * cap + w]);
      const V3 aw = qrot(po, ax);
      if (jt == JH) {
        col(vo, aw, cross(aw, d - cw));
      } else {
        col(vo, v3(0.f, 0.f, 0.f), aw);
        step = step + qrot(po, ax * g.q[g.topo[4 * i + 2] * cap + w]);
      }
    }
    d = d + step;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// K_B: one warp per world
// ---------------------------------------------------------------------------
// REFINE: the instance for trees above REFINE_NV DoF (FP64 sum of M and the
// refinement step); the smaller trees' instance compiles without those paths.
template <bool REFINE>
__global__ void __launch_bounds__(32 * TC_WARPS) tc_k_solve(TcGroupDev G) {
  extern __shared__ __align__(16) float tcs[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w = blockIdx.x * TC_WARPS + warp;
  const TreeGroupDev& g = G.t;
  if (w >= g.n || !g.live[w]) return;  // uniform per warp
  const int cap = g.cap, L = g.L, nv = g.nv;
  const TcLay lay = tc_layout(L, nv, G.ng, G.maxc, G.rpc);
  const TcSmem sm = tc_smem(L, nv, G.maxc, G.rpc);
  const int ld = lay.ld, vl = sm.vl;
  float* wf = G.scr + (size_t)w * G.sstride;
  float* sv = tcs + (size_t)warp * sm.words;
  float* vx = sv + V_X * vl; float* vd = sv + V_D * vl; float* vg = sv + V_G * vl; float* vb = sv + V_B * vl;
  float* vreg = sv + V_REG * vl; float* vdiag = sv + V_DIAG * vl; float* vu = sv + V_U * vl;
  float* vv = sv + V_V * vl; float* vp = sv + V_P * vl; float* vs = sv + V_S * vl;
  int* rcon = reinterpret_cast<int*>(sv + sm.rmap);
  int* rfac = rcon + sm.ldr;
  const float dt = g.dtg[w];
  const bool rk4 = g.integ && g.integ[w] == NEWT_INTEGRATOR_RK4;
  uint32_t status = 0;
  const float* gm = G.geom;
  auto gv = [&](int gi, int f) { return gm[(size_t)(GREC * gi + f) * cap + w]; };

  // ---- forward kinematics (tree.rs:771-858) ----
  // Each lane loads one link's joint parameters; the chain is then walked in
  // link order by every lane (parameters arrive by shuffle), lane 0 storing
  // the poses.
  float* pose = sv + sm.pose;
  for (int base = 0; base < L; base += 32) {
    const int li = base + lane;
    float pj[3] = {0.f, 0.f, 0.f}, pc[3] = {0.f, 0.f, 0.f}, pa[3] = {0.f, 0.f, 0.f}, pq = 0.f;
    if (li < L) {
      for (int k = 0; k < 3; ++k) {
        pj[k] = g.jp[(3 * li + k) * cap + w];
        pc[k] = g.jc[(3 * li + k) * cap + w];
        pa[k] = g.axis[(3 * li + k) * cap + w];
      }
      const int jt = g.topo[4 * li + 1], qo = g.topo[4 * li + 2];
      if (jt == JH || jt == JS) pq = g.q[qo * cap + w];
    }
    const int nl = L - base < 32 ? L - base : 32;
    for (int k = 0; k < nl; ++k) {
      const int i = base + k;
      const V3 jp = v3(__shfl_sync(FULL, pj[0], k), __shfl_sync(FULL, pj[1], k), __shfl_sync(FULL, pj[2], k));
      const V3 jc = v3(__shfl_sync(FULL, pc[0], k), __shfl_sync(FULL, pc[1], k), __shfl_sync(FULL, pc[2], k));
      const V3 ax = v3(__shfl_sync(FULL, pa[0], k), __shfl_sync(FULL, pa[1], k), __shfl_sync(FULL, pa[2], k));
      const float qa = __shfl_sync(FULL, pq, k);
      const int parent = g.topo[4 * i], jt = g.topo[4 * i + 1], qo = g.topo[4 * i + 2];
      V3 p;
      Q4 o;
      if (i == 0) {
        if (jt == JF) {
          p = v3(g.q[qo * cap + w], g.q[(qo + 1) * cap + w], g.q[(qo + 2) * cap + w]);
          o = Q4{g.q[(qo + 3) * cap + w], g.q[(qo + 4) * cap + w], g.q[(qo + 5) * cap + w], g.q[(qo + 6) * cap + w]};
        } else {
          o = Q4{g.rootq[w], g.rootq[cap + w], g.rootq[2 * cap + w], g.rootq[3 * cap + w]};
          p = jp - qrot(o, jc);
        }
      } else {
        __syncwarp();
        const float* pp = pose + 7 * parent;
        const Q4 po = Q4{pp[3], pp[4], pp[5], pp[6]};
        const V3 jpw = ldv3(pp) + qrot(po, jp);
        if (jt == JH) {
          o = qmul(po, q_axis_angle(ax, qa));
          p = jpw - qrot(o, jc);
        } else if (jt == JS) {
          o = po;
          p = jpw + qrot(po, ax * qa) - qrot(o, jc);
        } else {
          o = po;
          p = jpw - qrot(o, jc);
        }
      }
      __syncwarp();
      if (lane == 0) {
        float* d = pose + 7 * i;
        stv3(d, p);
        d[3] = o.x; d[4] = o.y; d[5] = o.z; d[6] = o.w;
      }
    }
  }
  __syncwarp();

  // ---- contacts in newt's pair order (link-plane pairs, and in-tree pairs
  //      when the tree collides with itself): lane per pair, a warp scan
  //      places each pair's contacts ----
  float* con = wf + lay.con;
  const bool resolve = G.sens != nullptr;  // the contact sensors' re-solve: the last step's contacts, no detection
  int ncon = resolve ? min(max(__float_as_int(wf[lay.misc]), 0), G.maxc) : 0;
  bool overflow = false;
  auto link_geom_pose = [&](int gi) {
    const float* lp = pose + 7 * G.gtopo[2 * gi + 1];
    const Q4 lo = Q4{lp[3], lp[4], lp[5], lp[6]};
    GPose gp;
    gp.p = ldv3(lp) + qrot(lo, v3(gv(gi, G_POS), gv(gi, G_POS + 1), gv(gi, G_POS + 2)));
    gp.q = qmul(lo, Q4{gv(gi, G_QUAT), gv(gi, G_QUAT + 1), gv(gi, G_QUAT + 2), gv(gi, G_QUAT + 3)});
    return gp;
  };
  for (int base = 0; base < (resolve ? 0 : G.npairs); base += 32) {
    const int pi = base + lane;
    CRes cr[4];
    int nc = 0, a = 0, b = 0, link = 0, link2 = -1;
    bool a_static = false, flip = false;
    if (pi < G.npairs && G.gtopo[2 * G.pairs[2 * pi] + 1] >= 0 && G.gtopo[2 * G.pairs[2 * pi + 1] + 1] >= 0) {
      // in-tree pair: side a (+1) and side b (-1) both on the tree
      a = G.pairs[2 * pi];
      b = G.pairs[2 * pi + 1];
      link = G.gtopo[2 * a + 1];
      link2 = G.gtopo[2 * b + 1];
      const float margin = fmaxf(gv(a, G_MARGIN), gv(b, G_MARGIN));
      CRes ct[4];  // its own buffer: `cr` stays in registers on the link-plane path
      nc = np_link_pair(G.gtopo[2 * a], G.gtopo[2 * b], link_geom_pose(a), link_geom_pose(b),
                        v3(gv(a, G_SIZE), gv(a, G_SIZE + 1), gv(a, G_SIZE + 2)),
                        v3(gv(b, G_SIZE), gv(b, G_SIZE + 1), gv(b, G_SIZE + 2)), margin, ct, &flip);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (k < nc) cr[k] = ct[k];
    } else if (pi < G.npairs) {
      a = G.pairs[2 * pi];
      b = G.pairs[2 * pi + 1];
      a_static = G.gtopo[2 * a + 1] < 0;
      const int gl = a_static ? b : a, gp = a_static ? a : b;  // link geom, plane
      link = G.gtopo[2 * gl + 1];
      const int shape = G.gtopo[2 * gl];
      const float* lp = pose + 7 * link;
      const Q4 lo = Q4{lp[3], lp[4], lp[5], lp[6]};
      GPose gpose, ppose;
      gpose.p = ldv3(lp) + qrot(lo, v3(gv(gl, G_POS), gv(gl, G_POS + 1), gv(gl, G_POS + 2)));
      gpose.q = qmul(lo, Q4{gv(gl, G_QUAT), gv(gl, G_QUAT + 1), gv(gl, G_QUAT + 2), gv(gl, G_QUAT + 3)});
      ppose.p = v3(gv(gp, G_POS), gv(gp, G_POS + 1), gv(gp, G_POS + 2));
      ppose.q = Q4{gv(gp, G_QUAT), gv(gp, G_QUAT + 1), gv(gp, G_QUAT + 2), gv(gp, G_QUAT + 3)};
      const float margin = fmaxf(gv(a, G_MARGIN), gv(b, G_MARGIN));
      if (shape == NEWT_SHAPE_SPHERE) {
        nc = np_sphere_plane(gpose, gv(gl, G_SIZE), margin, ppose, cr);
      } else if (shape == NEWT_SHAPE_BOX) {
        nc = np_box_plane(gpose, v3(gv(gl, G_SIZE), gv(gl, G_SIZE + 1), gv(gl, G_SIZE + 2)), margin, ppose, cr);
      } else if (shape == NEWT_SHAPE_CAPSULE) {
        nc = np_capsule_plane(gpose, gv(gl, G_SIZE), gv(gl, G_SIZE + 1), margin, ppose, cr);
      } else if (shape == NEWT_SHAPE_CYLINDER) {
        nc = np_cylinder_plane(gpose, gv(gl, G_SIZE), gv(gl, G_SIZE + 1), margin, ppose, cr);
      } else if (shape == NEWT_SHAPE_ELLIPSOID) {
        nc = np_ellipsoid_plane(gpose, v3(gv(gl, G_SIZE), gv(gl, G_SIZE + 1), gv(gl, G_SIZE + 2)), margin, ppose, cr);
      }
    }
    int incl = nc;  // inclusive scan of the per-pair counts
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(FULL, incl, 31);
    const int off = ncon + incl - nc;
    for (int k = 0; k < nc; ++k) {
      if (off + k >= G.maxc) { overflow = true; break; }
      float* c = con + CREC * (off + k);
      // the narrowphase ran as (geom, plane); a pair listed as (plane, geom)
      // is relabelled with the normal flipped (contact.rs:2509-2587)
      c[K_GA] = __int_as_float(a);
      c[K_GB] = __int_as_float(b);
      c[K_LINK] = __int_as_float(link);
      c[K_LINK2] = __int_as_float(link2);
      c[K_SIGN] = a_static ? -1.f : 1.f;
      stv3(c + K_POS, cr[k].pos);
      stv3(c + K_N, (a_static || flip) ? -cr[k].n : cr[k].n);
      c[K_PEN] = cr[k].pen;
      c[K_GAP] = fmaxf(gv(a, G_GAP), gv(b, G_GAP));
      c[K_MU] = fminf(gv(a, G_FRIC), gv(b, G_FRIC));
      // combine_solref (geom.rs:156-185), combine_solimp (solver.rs:242)
      const float ta = gv(a, G_SR), tb = gv(b, G_SR), da = gv(a, G_SR + 1), db = gv(b, G_SR + 1);
      const bool dira = ta < 0.f, dirb = tb < 0.f;
      c[K_SR] = dira != dirb ? (dira ? ta : tb) : fminf(ta, tb);
      c[K_SR + 1] = dira != dirb ? (dira ? da : db) : fminf(da, db);
      for (int q = 0; q < 3; ++q) c[K_SI + q] = fminf(gv(a, G_SI + q), gv(b, G_SI + q));
      c[K_SI + 3] = gv(a, G_SI + 3);
      c[K_SI + 4] = gv(a, G_SI + 4);
      c[K_CONDIM] = (float)min(G.gtopo[2 * G.ng + a], G.gtopo[2 * G.ng + b]);
      c[K_MUT] = fminf(gv(a, G_TF), gv(b, G_TF));  // combine_torsional_friction
      c[K_MUR] = fminf(gv(a, G_RF), gv(b, G_RF));  // combine_rolling_friction
    }
    ncon = ncon + total < G.maxc ? ncon + total : G.maxc;
  }
  if (__any_sync(FULL, overflow)) status |= NEWT_WS_CONTACT_OVERFLOW;
  __syncwarp();
  // rows of the active contacts, in contact order (solver.rs:2881-2890):
  // lane per contact, a warp scan assigns the row ranges; the pyramidal
  // cone's condim-3 contacts take four facet rows, the others the normal row
  // and, by condim, the tangent pair, torsion and the rolling pair
  int nrows = 0;
  for (int base = 0; base < ncon; base += 32) {
    const int c = base + lane;
    int k = 0;
    bool facets = false;
    if (c < ncon) {
      const float* cc = con + CREC * c;
      const int cd = (int)cc[K_CONDIM];
      facets = G.cone == NEWT_CONE_PYRAMIDAL && cd == 3;
      if (cc[K_PEN] - cc[K_GAP] > 0.f) k = facets ? 4 : cd;
    }
    int incl = k;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += t;
    }
    const int start = nrows + incl - k;
    if (c < ncon) {
      con[CREC * c + K_ROW] = __int_as_float(k > 0 ? start : -1);
      for (int f = 0; f < k; ++f) { rcon[start + f] = c; rfac[start + f] = facets ? f : -1 - f; }
    }
    nrows += __shfl_sync(FULL, incl, 31);
  }
  if (lane == 0 && !resolve) {
    wf[lay.misc] = __int_as_float(ncon);
    wf[lay.misc + 1] = __int_as_float(nrows);
    wf[lay.misc + 2] = __int_as_float(0);
  }
  const int nr = nrows;
  // the re-solve's sensor inputs (solver.rs:3334-3364): per link the rows'
  // forces f / dt times their wrench axes (dir x sign, (p - c_link) x
  // dir x sign), in row order; per contact the facets' impulses summed (a
  // normal row's own) over dt
  auto sens_out = [&](int nrow) {
    float* so = G.sens + (size_t)w * G.sens_stride;
    for (int l = lane; l < L; l += 32) {
      V3 fs = v3(0.f, 0.f, 0.f), ts = v3(0.f, 0.f, 0.f);
      const V3 cl = ldv3(pose + 7 * l);
      for (int r = 0; r < nrow; ++r) {
        const float* cc = con + CREC * rcon[r];
        const int l1 = __float_as_int(cc[K_LINK]), l2 = __float_as_int(cc[K_LINK2]);
        if (l1 != l && l2 != l) continue;
        const V3 dir = row_direction(cc, rfac[r]), pt = ldv3(cc + K_POS);
        const float force = vx[r] / dt;
        const bool ang = row_angular(rfac[r]);  // wrench (0, dir sign): world_jacobian_for_side
        if (l1 == l) {
          const V3 d = dir * cc[K_SIGN];
          if (ang) {
            ts = ts + d * force;
          } else {
            fs = fs + d * force;
            ts = ts + cross(pt - cl, d) * force;
          }
        }
        if (l2 == l) {
          const V3 d = dir * -1.f;
          if (ang) {
            ts = ts + d * force;
          } else {
            fs = fs + d * force;
            ts = ts + cross(pt - cl, d) * force;
          }
        }
      }
      stv3(so + 6 * l, fs);
      stv3(so + 6 * l + 3, ts);
    }
    for (int c = lane; c < ncon; c += 32) {
      const float* cc = con + CREC * c;
      const int row = __float_as_int(cc[K_ROW]);
      float fnorm = 0.f;
      if (row >= 0 && row < nrow) {
        if (rfac[row] >= 0) for (int k = 0; k < 4; ++k) fnorm += vx[row + k];
        else fnorm = vx[row];
      }
      so[6 * L + 3 * c] = cc[K_GA];
      so[6 * L + 3 * c + 1] = cc[K_GB];
      so[6 * L + 3 * c + 2] = fnorm / dt;
    }
    if (lane == 0) so[6 * L + 3 * G.maxc] = __int_as_float(ncon);
  };
  if (nr == 0) {  // no active contact: qacc stays a_free
    if (resolve) sens_out(0);
    else if (lane == 0 && status) atomicOr(g.status + w, status);
    return;
  }

  // ---- link COM Jacobians, world inertias and masses, lane per link ----
  const bool jac_shared = 6 * nv * L + 7 * L <= sm.nrs * sm.nrs;
  float* JV = jac_shared ? sv + sm.lh : wf + lay.jv;
  float* JW = jac_shared ? JV + 3 * nv * L : wf + lay.jw;
  float* IW = jac_shared ? JW + 3 * nv * L : wf + lay.iw;  // 6 per link, then the link masses
  float* MS = IW + 6 * L;
  for (int l = lane; l < L; l += 32) {
    float* jv = JV + 3 * nv * l;
    float* jw = JW + 3 * nv * l;
    for (int k = 0; k < 3 * nv; ++k) { jv[k] = 0.f; jw[k] = 0.f; }
    const float* pl = pose + 7 * l;
    chain_columns(g, w, pose, l, ldv3(pl), [&](int k, V3 rot, V3 tr) { stv3(jw + 3 * k, rot); stv3(jv + 3 * k, tr); });
    const M3 R = quat_mat(Q4{pl[3], pl[4], pl[5], pl[6]});
    M3 RT;
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) RT.m[r][c] = R.m[c][r];
    const S3 Ib{g.inert[(6 * l) * cap + w], g.inert[(6 * l + 1) * cap + w], g.inert[(6 * l + 2) * cap + w],
                g.inert[(6 * l + 3) * cap + w], g.inert[(6 * l + 4) * cap + w], g.inert[(6 * l + 5) * cap + w]};
    const S3 Iw = sym_congr(RT, Ib);  // R I R^T
    float* iw = IW + 6 * l;
    iw[0] = Iw.xx; iw[1] = Iw.yy; iw[2] = Iw.zz; iw[3] = Iw.xy; iw[4] = Iw.xz; iw[5] = Iw.yz;
    MS[l] = g.mass[l * cap + w];
  }
  __syncwarp();

  // ---- mass matrix (lower triangle, column-major), lane per entry ----
  float* LM = sv + sm.lm;   // factor of M + dt B (response, qacc)
  float* LD = sv + sm.ldf;  // factor of M (diagApprox)
  // Only links below both DoFs' joints contribute (the others' Jacobian
  // columns are zero): entry (i, j), i >= j, sums the subtree of DoF i's link
  // when DoF j's link is an ancestor of it and is zero otherwise, in link
  // order like the full sum.
  const int* dmask = G.gtopo + 3 * G.ng;  // subtree masks (lo, hi) per link
  const int* dlink = dmask + 2 * L;      // link of each DoF
  auto subtree = [&](int a) {
    return ((unsigned long long)(unsigned)dmask[2 * a + 1] << 32) | (unsigned)dmask[2 * a];
  };
  // Trees above REFINE_NV DoF sum the entries in FP64 (every f32 product is
  // exact in double) and keep that M' for the refinement's residual: on long
  // chains the f32 sums of long-lever products lose the digits that the
  // ill-conditioned solve amplifies, and a refinement against an f32 M'
  // converges to the wrong matrix's solution.
  constexpr bool refine = REFINE;
  double* Md = refine ? reinterpret_cast<double*>(wf + lay.mc) : nullptr;
  for (int e = lane; e < nv * nv; e += 32) {
    const int i = e % nv, j = e / nv;
    if (i < j) continue;
    const int ai = dlink[i], aj = dlink[j];
    float s = 0.f;
    double sd = 0.0;
    if ((subtree(aj) >> ai) & 1ull)
      for (unsigned long long m = subtree(ai); m; m &= m - 1ull) {
        const int l = __ffsll((long long)m) - 1;
        const float* jv = JV + 3 * nv * l;
        const float* jw = JW + 3 * nv * l;
        const float* iw = IW + 6 * l;
        const S3 I{iw[0], iw[1], iw[2], iw[3], iw[4], iw[5]};
        const V3 vi = ldv3(jv + 3 * i), vj = ldv3(jv + 3 * j), wi = ldv3(jw + 3 * i), wj = ldv3(jw + 3 * j);
        if (refine) {
          const double Iwj[3] = {(double)I.xx * wj.x + (double)I.xy * wj.y + (double)I.xz * wj.z,
                                 (double)I.xy * wj.x + (double)I.yy * wj.y + (double)I.yz * wj.z,
                                 (double)I.xz * wj.x + (double)I.yz * wj.y + (double)I.zz * wj.z};
          sd += (double)MS[l] * ((double)vi.x * vj.x + (double)vi.y * vj.y + (double)vi.z * vj.z) +
                ((double)wi.x * Iwj[0] + (double)wi.y * Iwj[1] + (double)wi.z * Iwj[2]);
        } else {
          s += MS[l] * dot(vi, vj) + dot(wi, smv(I, wj));
        }
      }
    if (refine) {
      Md[(size_t)j * nv + i] = sd;
      s = (float)sd;
    }
    LD[j * nv + i] = s;
  }
  __syncwarp();
  // armature (diagonal, child joints) and, under Euler, the implicit damping
  // dt*B (tree.rs:645-684); RK4 factors M itself (solver.rs:2852-2855)
  for (int k = lane; k < nv * nv; k += 32) LM[k] = LD[k];
  __syncwarp();
  if (lane == 0) {
    for (int i = 0; i < L; ++i) {
      const int jt = g.topo[4 * i + 1], vo = g.topo[4 * i + 3];
      if (jt == JF) {
        const float dm = rk4 ? 0.f : dt * g.damp[i * cap + w];
        for (int k = 0; k < 6; ++k) {
          LM[(vo + k) * nv + vo + k] += dm;
          if (refine) Md[(size_t)(vo + k) * nv + vo + k] += (double)dm;
        }
      } else if (jt == JH || jt == JS) {
        const float arm = g.arm[i * cap + w];
        const float add = arm + (rk4 ? 0.f : dt * g.damp[i * cap + w]);
        LD[vo * nv + vo] += arm;
        LM[vo * nv + vo] += add;
        if (refine) Md[(size_t)vo * nv + vo] += (double)add;
      }
    }
  }
  __syncwarp();
  if (!warp_cholesky2(LM, LD, nv, nv, lane)) {
    if (lane == 0) atomicOr(g.status + w, status | NEWT_WS_NOT_PD);
    return;
  }

  // ---- Jacobian rows of the cone facets, velocities, lane per row ----
  const bool rows_shared = nr <= sm.nrs;
  float* Jt = rows_shared ? sv + sm.jy : wf + lay.jt;  // J^T, column-major; becomes Y
  float* J0 = wf + lay.j0;                              // J^T, kept (refined or RK4 worlds)
  const bool keep_j = refine || rk4;
  const int ldj = rows_shared ? sm.nrs : ld;
  float* tw = sv + sm.tw;  // 1 marks a link that owns rows; then its inverse weight
  float* rw = tw + up4(L);  // the rotation inverse weights (angular rows)
  for (int l = lane; l < L; l += 32) tw[l] = 0.f;
  __syncwarp();
  for (int r = lane; r < nr; r += 32) {
    const float* cc = con + CREC * rcon[r];
    const int link = __float_as_int(cc[K_LINK]), link2 = __float_as_int(cc[K_LINK2]);
    tw[link] = 1.f;
    if (link2 >= 0) tw[link2] = 1.f;
    const float sign = cc[K_SIGN];
    const V3 pt = ldv3(cc + K_POS);
    const V3 dir = row_direction(cc, rfac[r]);
    // linear rows on the point's translational columns, angular rows on the
    // link's rotational ones (world_jacobian_for_side, solver.rs:3566-3598)
    const bool ang = row_angular(rfac[r]);
    for (int k = 0; k < nv; ++k) Jt[(size_t)k * ldj + r] = 0.f;
    chain_columns(g, w, pose, link, pt, [&](int k, V3 rot, V3 tr) {
      Jt[(size_t)k * ldj + r] = dot(ang ? rot : tr, dir) * sign;
    });
    if (link2 >= 0)  // side b of an in-tree pair: the columns its chain shares with side a's take both
      chain_columns(g, w, pose, link2, pt, [&](int k, V3 rot, V3 tr) {
        Jt[(size_t)k * ldj + r] -= dot(ang ? rot : tr, dir);
      });
    float vel = 0.f, vfree = 0.f;
    for (int k = 0; k < nv; ++k) {
      const float jk = Jt[(size_t)k * ldj + r];
      if (keep_j) J0[(size_t)k * ld + r] = jk;
      vel += jk * g.qd[k * cap + w];
      vfree += jk * g.qacc[k * cap + w];
    }
    vu[r] = vel;
    vv[r] = vfree * dt;  // J . (a_free dt): the free-motion velocity change
  }
  __syncwarp();

  // ---- Y = L^-1 J^T and A = Y^T Y (solver.rs:3043-3066), lane per row ----
  float* Y = Jt;  // forward substitution in place, one row per lane
  float* H = wf + lay.H;
  for (int r = lane; r < nr; r += 32) {
    float y[NEWT_MAX_LINKS + 5];
    for (int k = 0; k < nv; ++k) {
      float s = Jt[(size_t)k * ldj + r];
      for (int m = 0; m < k; ++m) s -= LM[m * nv + k] * y[m];
      y[k] = s / LM[k * nv + k];
      Y[(size_t)k * ldj + r] = y[k];
    }
  }
  __syncwarp();
  for (int r = lane; r < nr; r += 32)
    for (int c = 0; c < nr; ++c) {
      float s = 0.f;
      for (int k = 0; k < nv; ++k) s += Y[(size_t)k * ldj + r] * Y[(size_t)k * ldj + c];
      H[(size_t)c * ld + r] = s;
    }
  // ---- mean inverse weight of each link's COM (tree_body_invweight0): three
  // lanes per link, one per axis, ten links per round; the rotation weights
  // (rows about an axis) first, for groups with angular rows ----
  if (G.general)
    for (int l0 = 0; l0 < L; l0 += 10) {
      const int l = l0 + lane / 3, axis = lane % 3;
      float s2 = 0.f;
      if (lane < 30 && l < L && tw[l] != 0.f) {
        const float* jw = JW + 3 * nv * l;
        float y[NEWT_MAX_LINKS + 5];
        for (int k = 0; k < nv; ++k) {
          float s = jw[3 * k + axis];
          for (int m = 0; m < k; ++m) s -= LD[m * nv + k] * y[m];
          y[k] = s / LD[k * nv + k];
          s2 += y[k] * y[k];
        }
      }
      const float s2y = __shfl_down_sync(0xffffffffu, s2, 1), s2z = __shfl_down_sync(0xffffffffu, s2, 2);
      if (lane < 30 && axis == 0 && l < L) rw[l] = ((s2 + s2y) + s2z) / 3.f;
    }
  __syncwarp();
  for (int l0 = 0; l0 < L; l0 += 10) {
    const int l = l0 + lane / 3, axis = lane % 3;
    float s2 = 0.f;
    if (lane < 30 && l < L && tw[l] != 0.f) {  // links that own rows
      // |L_D^-1 jv_axis|^2 = jv_axis^T M^-1 jv_axis (forward substitution only)
      const float* jv = JV + 3 * nv * l;
      float y[NEWT_MAX_LINKS + 5];
      for (int k = 0; k < nv; ++k) {
        float s = jv[3 * k + axis];
        for (int m = 0; m < k; ++m) s -= LD[m * nv + k] * y[m];
        y[k] = s / LD[k * nv + k];
        s2 += y[k] * y[k];
      }
    }
    const float s2y = __shfl_down_sync(0xffffffffu, s2, 1), s2z = __shfl_down_sync(0xffffffffu, s2, 2);
    __syncwarp();
    if (lane < 30 && axis == 0 && l < L && tw[l] != 0.f) tw[l] = ((s2 + s2y) + s2z) / 3.f;
    __syncwarp();
  }

  // ---- regulariser, diagonal and bias per row (solver.rs:3068-3121) ----
  for (int r = lane; r < nr; r += 32) {
    const float* cc = con + CREC * rcon[r];
    const float pen = cc[K_PEN] - cc[K_GAP], mu = cc[K_MU];
    const Soft s{cc[K_SR], cc[K_SR + 1], cc[K_SI], cc[K_SI + 1], cc[K_SI + 2], cc[K_SI + 3], (int)cc[K_SI + 4]};
    const float d = impedance_at(-pen, s);
    const bool pyr = rfac[r] >= 0;
    // tree_contact_diag_approx: both tree sides' translation weights, or
    // rotation weights for an angular row
    const int link2 = __float_as_int(cc[K_LINK2]);
    const float* wt = row_angular(rfac[r]) ? rw : tw;
    const float twl = wt[__float_as_int(cc[K_LINK])] + (link2 >= 0 ? wt[link2] : 0.f);
    const float base = (1.f - d) / d * (pyr ? twl * (1.f + mu * mu) : twl);
    const float reg = pyr ? 2.f * mu * mu * base : base;
    vreg[r] = reg;
    vdiag[r] = H[(size_t)r * ld + r] + reg;
    // the position term drives the facets and the normal row only
    const float position = (pyr || rfac[r] == R_NORMAL) ? -pen : 0.f;
    vb[r] = vv[r] - reference_accel(position, vu[r], s.tc, s.dr, s, dt) * dt;
    vx[r] = 0.f;
  }
  __syncwarp();

  const int mode = G.mode[w];
  const int iters = G.iters[w];
  int done_it = 0;
  if (mode == NEWT_SOLVER_PGS && !G.general) {
    // dense Gauss-Seidel, four non-negative facet steps per pyramidal block
    // (world_pgs_non_negative, solver.rs:3851-3862)
    for (int it = 0; it < iters; ++it)
      for (int r = 0; r < nr; ++r) {
        float s = 0.f;
        for (int c = lane; c < nr; c += 32) s += H[(size_t)r * ld + c] * vx[c];
        s = warp_sum(s);
        const float res = (vb[r] + s) + vreg[r] * vx[r];
        const float p = vx[r] - res / vdiag[r];
        __syncwarp();
        if (lane == 0) vx[r] = p < 0.f ? 0.f : p;
        __syncwarp();
      }
    done_it = iters;
  } else if (mode == NEWT_SOLVER_PGS) {
    // the sweep over contact blocks (solver.rs:3268-3330): the normal row,
    // then the facets, or the tangent pair capped by the normal impulse
    // (world_pgs_pair: pyramidal caps or the elliptic projection), torsion
    // (world_pgs_scalar) and the rolling pair
    auto resid = [&](int r) {  // world_pgs_residual plus the row's own reg term
      float s = 0.f;
      for (int c = lane; c < nr; c += 32) s += H[(size_t)r * ld + c] * vx[c];
      s = warp_sum(s);
      return (vb[r] + s) + vreg[r] * vx[r];
    };
    auto put = [&](int r, float v) {
      __syncwarp();
      if (lane == 0) vx[r] = v;
      __syncwarp();
    };
    auto nonneg = [&](int r) {
      const float p = vx[r] - resid(r) / vdiag[r];
      put(r, p < 0.f ? 0.f : p);
    };
    auto scalar = [&](int r, float cap) {  // project_pyramidal
      const float f = vx[r] - resid(r) / vdiag[r];
      put(r, f > cap ? cap : (f < -cap ? -cap : f));
    };
    auto pair = [&](int i, int j, float mu, float normal) {
      if (G.cone == NEWT_CONE_PYRAMIDAL) {
        scalar(i, mu * normal);
        scalar(j, mu * normal);
        return;
      }
      const float ri = resid(i), rj = resid(j);
      const float fi = vx[i] - ri / vdiag[i], fj = vx[j] - rj / vdiag[j];
      float pi = 0.f, pj = 0.f;  // project_elliptic (solver.rs:398-411), isotropic
      if (normal > 0.f && mu > 0.f) {
        const float c = mu * normal, mag2 = fi * fi + fj * fj;
        if (mag2 <= c * c) { pi = fi; pj = fj; }
        else { const float sc = c / sqrtf(mag2); pi = fi * sc; pj = fj * sc; }
      }
      __syncwarp();
      if (lane == 0) { vx[i] = pi; vx[j] = pj; }
      __syncwarp();
    };
    for (int it = 0; it < iters; ++it)
      for (int c = 0; c < ncon; ++c) {
        const float* cc = con + CREC * c;
        const int r0 = __float_as_int(cc[K_ROW]);
        if (r0 < 0) continue;
        nonneg(r0);
        if (rfac[r0] >= 0) {
          for (int k = 1; k < 4; ++k) nonneg(r0 + k);
          continue;
        }
        const int cd = (int)cc[K_CONDIM];
        if (cd < 3) continue;
        pair(r0 + 1, r0 + 2, cc[K_MU], vx[r0]);
        if (cd >= 4) scalar(r0 + 3, cc[K_MUT] * vx[r0]);
        if (cd >= 6) pair(r0 + 4, r0 + 5, cc[K_MUR], vx[r0]);
      }
    done_it = iters;
  } else {
    // ---- Newton (newton.rs:275-339) on H = A + diag(R) ----
    for (int r = lane; r < nr; r += 32) H[(size_t)r * ld + r] += vreg[r];
    __syncwarp();
    // the factor lives in the shared tile when the rows fit, else in HBM
    const bool lh_shared = nr <= sm.nrs;
    float* LH = lh_shared ? sv + sm.lh : wf + lay.LH;
    const int ldh = lh_shared ? sm.nrs : ld;
    double* LHd = reinterpret_cast<double*>(wf + lay.LHd);
    // zero-friction facets duplicate rows: newt's solver-only pivot (solver.rs:3215-3232)
    bool zero_mu = false;
    for (int r = lane; r < nr; r += 32) zero_mu = zero_mu || (rfac[r] >= 0 && con[CREC * rcon[r] + K_MU] == 0.f);
    zero_mu = __any_sync(FULL, zero_mu);
    // under the pyramidal cone the general rows' only projection is the
    // normal row's (solver.rs:3164-3196): the other rows are free
    done_it = dense::newton_solve(H, nr, ld, LH, ldh, LHd, vx, vb, vd, vg, vp, vs, vu, vv, vreg, iters, zero_mu, lane,
                                  &status, G.general ? rfac : nullptr);
  }
  __syncwarp();
  if (resolve) {  // the sensors' inputs only: the step's impulses and accelerations stay as they were
    sens_out(nr);
    return;
  }

  // ---- outputs: impulses, J^T f / dt, qacc = a_free + (M + dt B)^-1 J^T f / dt ----
  // Refined trees form the contact force from the kept J^T: Y = L^-1 J^T
  // carries the f32 rounding of the forward substitution, which L Y does not
  // undo on long chains, and the FP64 refinement below needs the true
  // right-hand side to converge to.  The rest take J^T = L Y, so
  // (L L^T)^-1 J^T f / dt = L^-T (Y f) / dt: one back substitution.  RK4
  // worlds hold J^T f / dt over the integrator's stages (from the kept J^T).
  for (int r = lane; r < nr; r += 32) wf[lay.imp + r] = vx[r];
  double* rhs = refine ? reinterpret_cast<double*>(wf + lay.rd) : nullptr;
  for (int k = lane; k < nv; k += 32) {
    if (keep_j) {
      float s = 0.f;
      double sd = 0.0;
      for (int r = 0; r < nr; ++r) {
        const float jk = J0[(size_t)k * ld + r];
        s += jk * vx[r];
        if (refine) sd += (double)jk * (double)vx[r];
      }
      if (rk4) g.cfrc[(size_t)w * g.cstride + k] = s / dt;  // the generalised force, held over the stages
      if (refine) {
        vg[k] = s / dt;
        rhs[k] = sd / dt;
      }
    }
    if (!refine) {
      float s = 0.f;
      for (int r = 0; r < nr; ++r) s += Y[(size_t)k * ldj + r] * vx[r];
      vg[k] = s / dt;
    }
  }
  __syncwarp();
  if (refine) warp_llt_solve(LM, nv, nv, vg, lane);
  else warp_lt_solve(LM, nv, nv, vg, lane);
  if (refine) {
    // r = rhs - M' x in FP64 (M' summed in FP64, symmetric, its lower
    // triangle kept), then M' d = r with the FP32 factor in FP64 arithmetic,
    // x += d
    double* r = rhs + nv;
    __syncwarp();
    for (int i = lane; i < nv; i += 32) {
      double s = rhs[i];
      for (int j = 0; j < nv; ++j) s -= (i >= j ? Md[(size_t)j * nv + i] : Md[(size_t)i * nv + j]) * (double)vg[j];
      r[i] = s;
    }
    __syncwarp();
    warp_llt_solve_mixed(LM, nv, nv, r, lane);
    for (int i = lane; i < nv; i += 32) vg[i] = (float)((double)vg[i] + r[i]);
    __syncwarp();
  }
  for (int k = lane; k < nv; k += 32) g.qacc[k * cap + w] += vg[k];
  if (lane == 0) {
    wf[lay.misc + 2] = __int_as_float(done_it);
    if (status) atomicOr(g.status + w, status);
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
extern "C" size_t newt_tc_ws_bytes(int L, int nv, int ng, int maxc, int rpc) {
  return (size_t)tc_layout(L, nv, ng, maxc, rpc).words * sizeof(float);
}
extern "C" size_t newt_tc_smem_bytes(int L, int nv, int maxc, int rpc) {
  return (size_t)TC_WARPS * tc_smem(L, nv, maxc, rpc).words * sizeof(float);
}
// Kernel attribute for the dynamic shared memory (outside stream capture).
// The limit only grows: every tree-contact group of a step is prepared before
// any of them launches, so a later, smaller group must not lower the limit an
// earlier, larger one launches with.
extern "C" cudaError_t newt_tc_init(int L, int nv, int maxc, int rpc) {
  const int bytes = (int)newt_tc_smem_bytes(L, nv, maxc, rpc);
  const bool refine = nv > REFINE_NV;
  cudaFuncAttributes fa;
  cudaError_t e = refine ? cudaFuncGetAttributes(&fa, tc_k_solve<true>) : cudaFuncGetAttributes(&fa, tc_k_solve<false>);
  if (e != cudaSuccess) return e;
  if (bytes <= fa.maxDynamicSharedSizeBytes) return cudaSuccess;
  return refine ? cudaFuncSetAttribute(tc_k_solve<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes)
                : cudaFuncSetAttribute(tc_k_solve<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}
extern "C" void newt_launch_tc_solve(const TcGroupDev& G, cudaStream_t st) {
  const int grid = (G.t.n + TC_WARPS - 1) / TC_WARPS;
  if (grid == 0) return;
  const size_t bytes = newt_tc_smem_bytes(G.t.L, G.t.nv, G.maxc, G.rpc);
  if (G.t.nv > REFINE_NV) tc_k_solve<true><<<grid, 32 * TC_WARPS, bytes, st>>>(G);
  else tc_k_solve<false><<<grid, 32 * TC_WARPS, bytes, st>>>(G);
}
extern "C" void newt_tc_offsets(int L, int nv, int ng, int maxc, int rpc, int* con, int* imp, int* misc) {
  const TcLay t = tc_layout(L, nv, ng, maxc, rpc);
  *con = t.con;
  *imp = t.imp;
  *misc = t.misc;
}

extern "C" void newt_launch_tree_aba(const TreeGroupDev& g, cudaStream_t st);
extern "C" void newt_launch_tree_integrate(const TreeGroupDev& g, cudaStream_t st);

#define CKT(call)                                                               \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) { ctx->err = std::string(#call ": ") + cudaGetErrorString(e_); return NEWT_E_CUDA; } \
  } while (0)

// Scratch, kernel attribute and (when profiling) the timing events of one
// tree-contact group for `n_steps` env-steps: everything a launch needs that
// cannot happen under stream capture.
extern "C" int newt_tc_prepare(newt_gpu_ctx* ctx, HostGroup* g, int n_steps) {
  if (g->n == 0) return NEWT_OK;
  const size_t per = newt_tc_ws_bytes(g->size, g->nv, g->ng, g->maxc, g->tc_rpc);
  const size_t need = per * (size_t)g->cap;
  if (g->plain_scratch_bytes < need) {
    if (g->plain_scratch) cudaFree(g->plain_scratch);
    g->plain_scratch = nullptr;
    g->plain_scratch_bytes = 0;
    CKT(cudaMalloc(&g->plain_scratch, need));
    CKT(cudaMemset(g->plain_scratch, 0, need));
    g->plain_scratch_bytes = need;
    ctx->graph_dirty = true;
  }
  g->scr_stride = (long)(per / sizeof(float));
  CKT(newt_tc_init(g->size, g->nv, g->maxc, g->tc_rpc));
  if (ctx->profile) {
    while (ctx->tcev.size() < (size_t)6 * n_steps) {
      cudaEvent_t e;
      CKT(cudaEventCreate(&e));
      ctx->tcev.push_back(e);
    }
  }
  return NEWT_OK;
}

// n_steps env-steps of one prepared tree-contact group on stream `st`:
// a_free, the contact solve and the integration, three launches per
// env-step.  With profiling on, every kernel is bracketed by timing events
// (recorded as external event nodes when `capturing`).
extern "C" int newt_tc_launch(newt_gpu_ctx* ctx, HostGroup* g, int n_steps, cudaStream_t st, bool capturing) {
  if (g->n == 0) return NEWT_OK;
  TcGroupDev d = g->tc_dev();
  d.t.cfrc = d.scr + tc_layout(g->size, g->nv, g->ng, g->maxc, g->tc_rpc).qfc;
  d.t.cstride = d.sstride;
  const bool timed = ctx->profile && ctx->tcev.size() >= (size_t)6 * n_steps;
  auto mark = [&](int s, int k) {
    if (!timed) return;
    if (capturing) cudaEventRecordWithFlags(ctx->tcev[(size_t)6 * s + k], st, cudaEventRecordExternal);
    else cudaEventRecord(ctx->tcev[(size_t)6 * s + k], st);
  };
  for (int s = 0; s < n_steps; ++s) {
    mark(s, 0);
    newt_launch_tree_aba(d.t, st);
    mark(s, 1);
    mark(s, 2);
    newt_launch_tc_solve(d, st);
    mark(s, 3);
    mark(s, 4);
    newt_launch_tree_integrate(d.t, st);
    mark(s, 5);
    ctx->launches += 3;
  }
  return timed ? n_steps : 0;
}

// The contact sensors' re-solve of every world of a tree-contact group at
// its current state (newt's build_sensor_inputs, world.rs:1545-1701, with
// solve_tree_contact_sensor_solution, world.rs:2252-2274): a_free at the
// state into `afree` (cap x nv, as the step's solve sees it; the group's own
// qacc rows stay the last step's), then tc_k_solve on the last step's
// contacts writing each link's contact wrench and each contact's normal
// force to `sens` (TcGroupDev::sens, `sens_stride` floats per world).
// `cfrc` (cap x nv floats) takes the RK4 worlds' held force.  Returns the
// launches issued on `st`.
extern "C" int newt_tc_resolve(newt_gpu_ctx* ctx, HostGroup* g, float* sens, long sens_stride, float* afree,
                               float* cfrc, cudaStream_t st) {
  if (g->n == 0) return 0;
  if (newt_tc_prepare(ctx, g, 0) != NEWT_OK) return -1;
  TcGroupDev d = g->tc_dev();
  d.t.qacc = afree;
  d.t.cfrc = cfrc;
  d.t.cstride = g->nv;
  d.sens = sens;
  d.sens_stride = sens_stride;
  newt_launch_tree_aba(d.t, st);
  newt_launch_tc_solve(d, st);
  return 2;
}

// Floats per world of the re-solve's output for a group of `L` links and
// contact capacity `maxc`.
extern "C" long newt_tc_sens_stride(int L, int maxc) { return (6L * L + 3L * maxc + 1 + 3) / 4 * 4; }

// n_steps env-steps of one tree-contact group on the context's stream (the
// plain form).
extern "C" int newt_tc_step(newt_gpu_ctx* ctx, HostGroup* g, int n_steps, int fused) {
  (void)fused;
  if (g->n == 0) return NEWT_OK;
  int rc = newt_tc_prepare(ctx, g, n_steps);
  if (rc != NEWT_OK) return rc;
  const int timed = newt_tc_launch(ctx, g, n_steps, ctx->stream, false);
  ctx->tcev_steps = timed;
  return NEWT_OK;
}
