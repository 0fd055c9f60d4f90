// Kinematic-tree stepping kernels: forward kinematics, the articulated-body
// algorithm with the Euler implicit-damping fold, and semi-implicit Euler
// integration, one world per thread.
//
// Restates, for FP32 on sm_103a:
//   newt/src/tree.rs:771-858    forward_kinematics_into (only the orientations
//                               are needed without contact: gravity enters ABA
//                               as a body-frame force m*R^T g)
//   newt/src/tree.rs:1021-1116  aba_with_velocity_implicit_workspace
//   newt/src/forces.rs:6-85     assemble_joint_forces (qfrc_applied - damping*qdot)
//   newt/src/aba.rs:803-1102    aba::run
//   newt/src/tree.rs:1393-1475  euler_step_with_workspace / integrate_tree_positions
//
// Two forms:
//   * fused  (`tree_fused_kernel`): the whole horizon in one launch; each
//     thread keeps its world's state in registers/local memory and reads its
//     model parameters (L1/L2-resident) every step.  Used by the batched path.
//   * plain  (`tree_fk_kernel`, `tree_aba_kernel`, `tree_integrate_kernel`):
//     one launch per stage per step with state round-tripping through HBM.
#include "common.cuh"
#include "groups.h"
#include "../../include/newt_gpu.h"

namespace {

enum { JF = 0, JX = 1, JH = 2, JS = 3 };

struct LinkScratch {
  PX X;
  SM6 S, v, c;
  SF6 U, pA;
  ABI IA;
  float D, u;
};

// Per-world ABA (forward dynamics).  q/qd/qfrc are the world's state in newt
// layout; writes qdd.  `scr` is MAXL entries of per-link scratch.
// `idt`: the step folded into the joint damping (dt for semi-implicit Euler,
// 0 for the explicit RK4 stages).
// `extb` (nullable): external wrenches per link, link frame at the COM
// (torque, force), beside gravity.
template <int MAXL>
__device__ bool tree_aba(const TreeGroupDev& g, int w, const float* q, const float* qd, const float* qfrc,
                         float* qdd, LinkScratch* scr, float idt, const SF6* extb = nullptr) {
  const int L = g.L, cap = g.cap;
  const float dt = idt;
  const V3 grav = v3(g.dtg[cap + w], g.dtg[2 * cap + w], g.dtg[3 * cap + w]);
  V3 gb[MAXL];  // gravity in each link frame
  // ---- pass 1 (root -> leaves): transforms, velocities, bias ----
  for (int i = 0; i < L; ++i) {
    const int parent = g.topo[4 * i], jt = g.topo[4 * i + 1], qo = g.topo[4 * i + 2], vo = g.topo[4 * i + 3];
    LinkScratch& s = scr[i];
    const float m = g.mass[i * cap + w];
    S3 I{g.inert[(6 * i) * cap + w], g.inert[(6 * i + 1) * cap + w], g.inert[(6 * i + 2) * cap + w],
         g.inert[(6 * i + 3) * cap + w], g.inert[(6 * i + 4) * cap + w], g.inert[(6 * i + 5) * cap + w]};
    if (i == 0) {
      Q4 ori;
      if (jt == JF) {
        ori = Q4{q[qo + 3], q[qo + 4], q[qo + 5], q[qo + 6]};
        s.v = SM6{v3(qd[vo], qd[vo + 1], qd[vo + 2]), v3(qd[vo + 3], qd[vo + 4], qd[vo + 5])};
      } else {
        ori = Q4{g.rootq[w], g.rootq[cap + w], g.rootq[2 * cap + w], g.rootq[3 * cap + w]};
        s.v = SM6{v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f)};
      }
      gb[0] = qrot_inv(ori, grav);
      s.c = SM6{v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f)};
    } else {
      const V3 jp = v3(g.jp[(3 * i) * cap + w], g.jp[(3 * i + 1) * cap + w], g.jp[(3 * i + 2) * cap + w]);
      const V3 jc = v3(g.jc[(3 * i) * cap + w], g.jc[(3 * i + 1) * cap + w], g.jc[(3 * i + 2) * cap + w]);
      const V3 ax = v3(g.axis[(3 * i) * cap + w], g.axis[(3 * i + 1) * cap + w], g.axis[(3 * i + 2) * cap + w]);
      const LinkScratch& p = scr[parent];
      if (jt == JH) {
        float an = sqrtf(len2(ax));
        V3 axn = an > 0.f ? ax * (1.f / an) : ax;
        float sn, cs;
        sincosf(-0.5f * q[qo], &sn, &cs);
        s.X.E = quat_mat(Q4{axn.x * sn, axn.y * sn, axn.z * sn, cs});
        s.X.t = jc - mv(s.X.E, jp);
        s.S = SM6{ax, cross(jc, ax)};
      } else if (jt == JS) {
        s.X.E = quat_mat(Q4{0.f, 0.f, 0.f, 1.f});
        s.X.t = (jc - jp) - ax * q[qo];
        s.S = SM6{v3(0.f, 0.f, 0.f), ax};
      } else {  // fixed (identity joint frames)
        s.X.E = quat_mat(Q4{0.f, 0.f, 0.f, 1.f});
        s.X.t = jc - jp;
        s.S = SM6{v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f)};
      }
      gb[i] = mv(s.X.E, gb[parent]);
      SM6 vp = px_motion(s.X, p.v);
      if (jt == JX) {
        s.v = vp;
        s.c = SM6{v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f)};
      } else {
        SM6 sq = smscale(s.S, qd[vo]);
        s.v = smadd(vp, sq);
        s.c = crm(s.v, sq);
      }
    }
    s.IA.A = I;
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) s.IA.B.m[r][c] = 0.f;
    s.IA.C = S3{m, m, m, 0.f, 0.f, 0.f};
    SF6 Iv = abi_mul(s.IA, s.v);
    SF6 ext{v3(0.f, 0.f, 0.f), gb[i] * m};
    if (extb) ext = sfadd(ext, extb[i]);
    s.pA = sfsub(crf(s.v, Iv), ext);
  }
  // ---- pass 2 (leaves -> root): articulated inertias and biases ----
  for (int i = L - 1; i >= 1; --i) {
    const int parent = g.topo[4 * i], jt = g.topo[4 * i + 1], vo = g.topo[4 * i + 3];
    LinkScratch& s = scr[i];
    LinkScratch& p = scr[parent];
    SF6 ps = sfadd(s.pA, abi_mul(s.IA, s.c));
    if (jt == JX) {
      abi_add(p.IA, abi_pull_back(s.IA, s.X));
      p.pA = sfadd(p.pA, px_force_T(s.X, ps));
      continue;
    }
    const float damp = g.damp[i * cap + w], arm = g.arm[i * cap + w];
    SF6 U = abi_mul(s.IA, s.S);
    float D = sdot6(s.S, U) + arm + dt * damp;
    float tau = qfrc[vo] - damp * qd[vo];
    float u = tau - sdot6(s.S, ps);
    float invD = 1.f / D;
    SF6 pfull = sfadd(ps, sfscale(U, u * invD));
    ABI Ia = s.IA;
    abi_rank1_sub(Ia, U, invD);
    s.U = U; s.D = D; s.u = u;
    abi_add(p.IA, abi_pull_back(Ia, s.X));
    p.pA = sfadd(p.pA, px_force_T(s.X, pfull));
  }
  // ---- root ----
  SM6 a0{v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f)};
  bool ok = true;
  const int jt0 = g.topo[1];
  if (jt0 == JF) {
    const int vo = g.topo[3];
    SF6 fr{v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f)};
    if (g.solver[w] != 0) fr = SF6{v3(qfrc[vo], qfrc[vo + 1], qfrc[vo + 2]), v3(qfrc[vo + 3], qfrc[vo + 4], qfrc[vo + 5])};
    SF6 rhs = sfsub(fr, scr[0].pA);
    const float fd = g.damp[w];
    ABI I0 = scr[0].IA;
    if (fd != 0.f) {
      rhs = sfsub(rhs, SF6{v3(qd[vo], qd[vo + 1], qd[vo + 2]) * fd, v3(qd[vo + 3], qd[vo + 4], qd[vo + 5]) * fd});
      float dm = dt * fd;
      I0.A.xx += dm; I0.A.yy += dm; I0.A.zz += dm; I0.C.xx += dm; I0.C.yy += dm; I0.C.zz += dm;
    }
    ok = abi_solve(I0, rhs, &a0);
    qdd[vo] = a0.w.x; qdd[vo + 1] = a0.w.y; qdd[vo + 2] = a0.w.z;
    qdd[vo + 3] = a0.v.x; qdd[vo + 4] = a0.v.y; qdd[vo + 5] = a0.v.z;
  }
  // ---- pass 3 (root -> leaves): accelerations ----
  SM6 acc[MAXL];
  acc[0] = a0;
  for (int i = 1; i < L; ++i) {
    const int parent = g.topo[4 * i], jt = g.topo[4 * i + 1], vo = g.topo[4 * i + 3];
    const LinkScratch& s = scr[i];
    SM6 xa = px_motion(s.X, acc[parent]);
    if (jt == JX) { acc[i] = smadd(xa, s.c); continue; }
    float qa = (s.u - sdot6(xa, s.U)) / s.D;
    qdd[vo] = qa;
    acc[i] = smadd(smadd(xa, s.c), smscale(s.S, qa));
  }
  return ok;
}

template <int MAXL>
__device__ void tree_integrate(const TreeGroupDev& g, int w, float* q, float* qd, const float* qdd) {
  const float dt = g.dtg[w];
  for (int k = 0; k < g.nv; ++k) qd[k] += qdd[k] * dt;
  for (int i = 0; i < g.L; ++i) {
    const int jt = g.topo[4 * i + 1], qo = g.topo[4 * i + 2], vo = g.topo[4 * i + 3];
    if (jt == JF) {
      Q4 ori{q[qo + 3], q[qo + 4], q[qo + 5], q[qo + 6]};
      V3 om = v3(qd[vo], qd[vo + 1], qd[vo + 2]);
      V3 dp = qrot(ori, v3(qd[vo + 3], qd[vo + 4], qd[vo + 5])) * dt;
      q[qo] += dp.x; q[qo + 1] += dp.y; q[qo + 2] += dp.z;
      Q4 nx = q_integrate(ori, om, dt);
      q[qo + 3] = nx.x; q[qo + 4] = nx.y; q[qo + 5] = nx.z; q[qo + 6] = nx.w;
    } else if (jt == JH || jt == JS) {
      q[qo] += qd[vo] * dt;
    }
  }
}

// One classic RK4 step (newt/src/tree.rs:1234-1364, derivative of a stage
// state tree.rs:1485-1550): four explicit ABA stages, stage states
// q0 + h dq, the weighted sum (dq1 + 2 dq2 + 2 dq3 + dq4) dt/6, then the free
// root's quaternion renormalised by division (Quat::renormalize).  `qdd`
// receives the first stage's acceleration.
template <int MAXL>
__device__ bool tree_rk4(const TreeGroupDev& g, int w, float* q, float* qd, const float* qf, float* qdd,
                         LinkScratch* scr) {
  const int L = g.L, nq = g.nq, nv = g.nv;
  const float dt = g.dtg[w];
  float q0[MAXL + 6], v0[MAXL + 5], aq[MAXL + 6], av[MAXL + 5], dq[MAXL + 6], a[MAXL + 5];
  for (int k = 0; k < nq; ++k) q0[k] = q[k];
  for (int k = 0; k < nv; ++k) v0[k] = qd[k];
  bool ok = true;
  for (int s = 0; s < 4; ++s) {
    ok = tree_aba<MAXL>(g, w, q, qd, qf, a, scr, 0.f) && ok;
    if (s == 0)
      for (int k = 0; k < nv; ++k) qdd[k] = a[k];
    for (int k = 0; k < nq; ++k) dq[k] = 0.f;
    for (int i = 0; i < L; ++i) {
      const int jt = g.topo[4 * i + 1], qo = g.topo[4 * i + 2], vo = g.topo[4 * i + 3];
      if (jt == JF) {
        const Q4 ori{q[qo + 3], q[qo + 4], q[qo + 5], q[qo + 6]};
        const V3 vw = qrot(ori, v3(qd[vo + 3], qd[vo + 4], qd[vo + 5]));
        dq[qo] = vw.x; dq[qo + 1] = vw.y; dq[qo + 2] = vw.z;
        const Q4 d = qmul(ori, Q4{qd[vo], qd[vo + 1], qd[vo + 2], 0.f});
        dq[qo + 3] = d.x * 0.5f; dq[qo + 4] = d.y * 0.5f; dq[qo + 5] = d.z * 0.5f; dq[qo + 6] = d.w * 0.5f;
      } else if (jt == JH || jt == JS) {
        dq[qo] = qd[vo];
      }
    }
    if (s == 0) {
      for (int k = 0; k < nq; ++k) aq[k] = dq[k];
      for (int k = 0; k < nv; ++k) av[k] = a[k];
    } else {
      const float wgt = s == 3 ? 1.f : 2.f;
      for (int k = 0; k < nq; ++k) aq[k] += wgt * dq[k];
      for (int k = 0; k < nv; ++k) av[k] += wgt * a[k];
    }
    if (s == 3) break;
    const float h = s < 2 ? dt * 0.5f : dt;
    for (int k = 0; k < nq; ++k) q[k] = q0[k] + dq[k] * h;
    for (int k = 0; k < nv; ++k) qd[k] = v0[k] + a[k] * h;
  }
  const float c = dt * (1.f / 6.f);
  for (int k = 0; k < nq; ++k) q[k] = q0[k] + aq[k] * c;
  for (int k = 0; k < nv; ++k) qd[k] = v0[k] + av[k] * c;
  if (g.topo[1] == JF) {
    const int o = g.topo[2] + 3;
    const float n = sqrtf(q[o] * q[o] + q[o + 1] * q[o + 1] + q[o + 2] * q[o + 2] + q[o + 3] * q[o + 3]);
    if (n == 0.f) { q[o] = 0.f; q[o + 1] = 0.f; q[o + 2] = 0.f; q[o + 3] = 1.f; }
    else { q[o] /= n; q[o + 1] /= n; q[o + 2] /= n; q[o + 3] /= n; }
  }
  return ok;
}

__device__ __forceinline__ bool is_rk4(const TreeGroupDev& g, int w) {
  return g.integ && g.integ[w] == NEWT_INTEGRATOR_RK4;
}

__device__ __forceinline__ bool finite_all(const float* a, int n) {
  bool ok = true;
  for (int k = 0; k < n; ++k) ok = ok && isfinite(a[k]);
  return ok;
}

}  // namespace

// One world's whole horizon with its state kept on-chip.
template <int MAXL>
__device__ __forceinline__ void tree_world_steps(const TreeGroupDev& g, int w, int n_steps) {
  const int cap = g.cap, nq = g.nq, nv = g.nv;
  float q[MAXL + 6], qd[MAXL + 5], qf[MAXL + 5], qdd[MAXL + 5];
  for (int k = 0; k < nq; ++k) q[k] = g.q[k * cap + w];
  for (int k = 0; k < nv; ++k) { qd[k] = g.qd[k * cap + w]; qf[k] = g.qfrc[k * cap + w]; qdd[k] = 0.f; }
  LinkScratch scr[MAXL];
  uint32_t st = 0;
  const bool rk4 = is_rk4(g, w);
  for (int s = 0; s < n_steps; ++s) {
    if (rk4) {
      if (!tree_rk4<MAXL>(g, w, q, qd, qf, qdd, scr)) st |= NEWT_WS_NOT_PD;
      continue;
    }
    if (!tree_aba<MAXL>(g, w, q, qd, qf, qdd, scr, g.dtg[w])) st |= NEWT_WS_NOT_PD;
    tree_integrate<MAXL>(g, w, q, qd, qdd);
  }
  if (!finite_all(q, nq) || !finite_all(qd, nv)) st |= NEWT_WS_NONFINITE;
  for (int k = 0; k < nq; ++k) g.q[k * cap + w] = q[k];
  for (int k = 0; k < nv; ++k) { g.qd[k * cap + w] = qd[k]; g.qacc[k * cap + w] = qdd[k]; }
  if (st) g.status[w] |= st;
}

// Whole horizon in one launch over a contiguous range of one group.
template <int MAXL>
__global__ void __launch_bounds__(64) tree_fused_kernel(TreeGroupDev g, int base, int count, int n_steps) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int w = base + t;
  if (w >= g.n || !g.live[w]) return;
  tree_world_steps<MAXL>(g, w, n_steps);
}

// Persistent form: blocks pull (group, base, count) items from a queue
// sorted by size class (largest first) until it is drained.
template <int MAXL>
__global__ void __launch_bounds__(64) tree_persistent_kernel(const TreeGroupDev* groups, const int* queue,
                                                             int* counter, int n_items, int n_steps) {
  __shared__ int item;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = item;
    if (it >= n_items) return;
    const int gi = queue[3 * it], base = queue[3 * it + 1], count = queue[3 * it + 2];
    const TreeGroupDev g = groups[gi];
    const int w = base + (int)threadIdx.x;
    if ((int)threadIdx.x < count && w < g.n && g.live[w]) tree_world_steps<MAXL>(g, w, n_steps);
  }
}

// Plain form, stage 1+2: forward dynamics from HBM state into HBM qacc.
template <int MAXL>
__global__ void __launch_bounds__(128) tree_aba_kernel(TreeGroupDev g) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= g.n || !g.live[w]) return;
  const int cap = g.cap, nq = g.nq, nv = g.nv;
  float q[MAXL + 6], qd[MAXL + 5], qf[MAXL + 5], qdd[MAXL + 5];
  for (int k = 0; k < nq; ++k) q[k] = g.q[k * cap + w];
  for (int k = 0; k < nv; ++k) { qd[k] = g.qd[k * cap + w]; qf[k] = g.qfrc[k * cap + w]; qdd[k] = 0.f; }
  LinkScratch scr[MAXL];
  const bool rk4 = is_rk4(g, w);
  if (rk4 && !g.cfrc) {  // no contacts: the whole RK4 step here; the integrate stage skips the world
    uint32_t st = tree_rk4<MAXL>(g, w, q, qd, qf, qdd, scr) ? 0u : NEWT_WS_NOT_PD;
    if (!finite_all(q, nq) || !finite_all(qd, nv)) st |= NEWT_WS_NONFINITE;
    for (int k = 0; k < nq; ++k) g.q[k * cap + w] = q[k];
    for (int k = 0; k < nv; ++k) { g.qd[k * cap + w] = qd[k]; g.qacc[k * cap + w] = qdd[k]; }
    if (st) g.status[w] |= st;
    return;
  }
  // a_free for the contact solve: with the implicit damping fold under Euler,
  // the explicit ABA under RK4 (newt/src/solver.rs:3602-3622)
  if (!tree_aba<MAXL>(g, w, q, qd, qf, qdd, scr, rk4 ? 0.f : g.dtg[w])) g.status[w] |= NEWT_WS_NOT_PD;
  for (int k = 0; k < nv; ++k) g.qacc[k * cap + w] = qdd[k];
  if (rk4)  // the solve adds J^T f / dt here when the world has contacts
    for (int k = 0; k < nv; ++k) g.cfrc[(size_t)w * g.cstride + k] = 0.f;
}

// Plain form, stage 3: Euler integration from HBM qacc; for RK4 worlds of a
// tree-contact group, the RK4 step with the contact solve's generalised force
// added to qfrc and held over the four stages (newt/src/world.rs:1826-1945).
template <int MAXL>
__global__ void __launch_bounds__(128) tree_integrate_kernel(TreeGroupDev g) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= g.n || !g.live[w]) return;
  const bool rk4 = is_rk4(g, w);
  if (rk4 && !g.cfrc) return;  // stepped whole by the ABA stage
  const int cap = g.cap, nq = g.nq, nv = g.nv;
  if (rk4) {
    float q[MAXL + 6], qd[MAXL + 5], qf[MAXL + 5], qdd[MAXL + 5];
    const float* cf = g.cfrc + (size_t)w * g.cstride;
    for (int k = 0; k < nq; ++k) q[k] = g.q[k * cap + w];
    for (int k = 0; k < nv; ++k) { qd[k] = g.qd[k * cap + w]; qf[k] = g.qfrc[k * cap + w] + cf[k]; qdd[k] = 0.f; }
    LinkScratch scr[MAXL];
    uint32_t st = tree_rk4<MAXL>(g, w, q, qd, qf, qdd, scr) ? 0u : NEWT_WS_NOT_PD;
    if (!finite_all(q, nq) || !finite_all(qd, nv)) st |= NEWT_WS_NONFINITE;
    for (int k = 0; k < nq; ++k) g.q[k * cap + w] = q[k];
    for (int k = 0; k < nv; ++k) { g.qd[k * cap + w] = qd[k]; g.qacc[k * cap + w] = qdd[k]; }
    if (st) g.status[w] |= st;
    return;
  }
  float q[MAXL + 6], qd[MAXL + 5], qdd[MAXL + 5];
  for (int k = 0; k < nq; ++k) q[k] = g.q[k * cap + w];
  for (int k = 0; k < nv; ++k) { qd[k] = g.qd[k * cap + w]; qdd[k] = g.qacc[k * cap + w]; }
  tree_integrate<MAXL>(g, w, q, qd, qdd);
  if (!finite_all(q, nq) || !finite_all(qd, nv)) g.status[w] |= NEWT_WS_NONFINITE;
  for (int k = 0; k < nq; ++k) g.q[k * cap + w] = q[k];
  for (int k = 0; k < nv; ++k) g.qd[k * cap + w] = qd[k];
}

// Host-side launchers (MAXL buckets 8, 16, 32, 65).
#define NEWT_TREE_BUCKETS(X) X(8) X(16) X(32) X(65)

extern "C" int newt_tree_bucket(int L) { return L <= 8 ? 8 : L <= 16 ? 16 : L <= 32 ? 32 : 65; }

extern "C" void newt_launch_tree_fused(const TreeGroupDev& g, int base, int count, int n_steps, cudaStream_t st) {
  const int B = 64;
  int grid = (count + B - 1) / B;
  if (grid == 0) return;
  switch (newt_tree_bucket(g.L)) {
#define X(M) case M: tree_fused_kernel<M><<<grid, B, 0, st>>>(g, base, count, n_steps); break;
    NEWT_TREE_BUCKETS(X)
#undef X
  }
}

extern "C" void newt_launch_tree_persistent(const TreeGroupDev* dgroups, const int* dqueue, int* dcounter, int n_items,
                                            int bucket, int n_steps, int grid, cudaStream_t st) {
  if (grid <= 0 || n_items <= 0) return;
  switch (bucket) {
#define X(M) case M: tree_persistent_kernel<M><<<grid, 64, 0, st>>>(dgroups, dqueue, dcounter, n_items, n_steps); break;
    NEWT_TREE_BUCKETS(X)
#undef X
  }
}

extern "C" int newt_tree_persistent_blocks_per_sm(int bucket) {
  int nb = 1;
  switch (bucket) {
#define X(M) case M: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, tree_persistent_kernel<M>, 64, 0); break;
    NEWT_TREE_BUCKETS(X)
#undef X
  }
  return nb < 1 ? 1 : nb;
}

// The sensors' dynamics pass for trees without geoms (newt/src/sensor.rs:
// 446-530, 834-1000): qddot from the explicit ABA at the world's current
// state and generalised forces, no external wrenches; then per link its
// spatial acceleration a_i = X_i a_parent + S_i qddot_i + v_i x S_i qdot_i
// (compute_link_va, the velocities and products the ABA left in its
// scratch) and the wrench its parent joint transmits, f_i = I_i a_i +
// v_i x* I_i v_i - (0, m_i R_i^T g), children pulled into parents leaves to
// root (compute_link_wrenches).  Writes 18 floats per link of each named
// world: v (angular, linear), a, f (torque, force), link frame at the COM.
// `sens` (nullable; tree-contact worlds): the contact re-solve's output
// (newt_tc_resolve), whose per-link wrenches (world force and torque about
// each COM, the first 6 L floats of each world's `sens_stride`) act as
// external wrenches in both passes.
template <int MAXL>
__global__ void __launch_bounds__(64) tree_sensor_dyn_kernel(TreeGroupDev g, const int* idx, int n, float* out,
                                                             const float* sens, long sens_stride) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int w = idx[t], cap = g.cap, nq = g.nq, nv = g.nv, L = g.L;
  float q[MAXL + 6], qd[MAXL + 5], qf[MAXL + 5], qdd[MAXL + 5];
  for (int k = 0; k < nq; ++k) q[k] = g.q[k * cap + w];
  for (int k = 0; k < nv; ++k) { qd[k] = g.qd[k * cap + w]; qf[k] = g.qfrc[k * cap + w]; qdd[k] = 0.f; }
  SF6 extb[MAXL];  // the contact wrenches in each link's frame (orientations by forward kinematics)
  if (sens) {
    const float* so = sens + (size_t)w * sens_stride;
    Q4 O[MAXL];
    for (int i = 0; i < L; ++i) {
      const int parent = g.topo[4 * i], jt = g.topo[4 * i + 1], qo = g.topo[4 * i + 2];
      if (i == 0) {
        O[0] = jt == JF ? Q4{q[qo + 3], q[qo + 4], q[qo + 5], q[qo + 6]}
                        : Q4{g.rootq[w], g.rootq[cap + w], g.rootq[2 * cap + w], g.rootq[3 * cap + w]};
      } else if (jt == JH) {
        const V3 ax = v3(g.axis[(3 * i) * cap + w], g.axis[(3 * i + 1) * cap + w], g.axis[(3 * i + 2) * cap + w]);
        const float an = sqrtf(len2(ax));
        const V3 a = an > 0.f ? ax * (1.f / an) : v3(0.f, 0.f, 0.f);
        float sn, cs;
        sincosf(q[qo] * 0.5f, &sn, &cs);
        O[i] = qmul(O[parent], Q4{a.x * sn, a.y * sn, a.z * sn, cs});
      } else {
        O[i] = O[parent];  // slide and fixed joints with identity joint frames
      }
      extb[i] = SF6{qrot_inv(O[i], v3(so[6 * i + 3], so[6 * i + 4], so[6 * i + 5])),
                    qrot_inv(O[i], v3(so[6 * i], so[6 * i + 1], so[6 * i + 2]))};
    }
  }
  LinkScratch scr[MAXL];
  tree_aba<MAXL>(g, w, q, qd, qf, qdd, scr, 0.f, sens ? extb : nullptr);
  const V3 grav = v3(g.dtg[cap + w], g.dtg[2 * cap + w], g.dtg[3 * cap + w]);
  SM6 a[MAXL];
  SF6 f[MAXL];
  V3 gb[MAXL];
  for (int i = 0; i < L; ++i) {
    const int parent = g.topo[4 * i], jt = g.topo[4 * i + 1], qo = g.topo[4 * i + 2], vo = g.topo[4 * i + 3];
    const LinkScratch& s = scr[i];
    if (i == 0) {
      const Q4 ori = jt == JF ? Q4{q[qo + 3], q[qo + 4], q[qo + 5], q[qo + 6]}
                              : Q4{g.rootq[w], g.rootq[cap + w], g.rootq[2 * cap + w], g.rootq[3 * cap + w]};
      gb[0] = qrot_inv(ori, grav);
      a[0] = jt == JF ? SM6{v3(qdd[vo], qdd[vo + 1], qdd[vo + 2]), v3(qdd[vo + 3], qdd[vo + 4], qdd[vo + 5])}
                      : SM6{v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f)};
    } else {
      gb[i] = mv(s.X.E, gb[parent]);
      const SM6 xa = px_motion(s.X, a[parent]);
      a[i] = jt == JX ? xa : smadd(smadd(xa, smscale(s.S, qdd[vo])), s.c);
    }
    const float m = g.mass[i * cap + w];
    ABI I;
    I.A = S3{g.inert[(6 * i) * cap + w], g.inert[(6 * i + 1) * cap + w], g.inert[(6 * i + 2) * cap + w],
             g.inert[(6 * i + 3) * cap + w], g.inert[(6 * i + 4) * cap + w], g.inert[(6 * i + 5) * cap + w]};
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) I.B.m[r][c] = 0.f;
    I.C = S3{m, m, m, 0.f, 0.f, 0.f};
    SF6 fe{v3(0.f, 0.f, 0.f), gb[i] * m};
    if (sens) fe = sfadd(fe, extb[i]);
    f[i] = sfsub(sfadd(abi_mul(I, a[i]), crf(s.v, abi_mul(I, s.v))), fe);
  }
  for (int i = L - 1; i >= 1; --i) f[g.topo[4 * i]] = sfadd(f[g.topo[4 * i]], px_force_T(scr[i].X, f[i]));
  float* o = out + (size_t)t * L * 18;
  for (int i = 0; i < L; ++i) {
    const V3 vv[6] = {scr[i].v.w, scr[i].v.v, a[i].w, a[i].v, f[i].t, f[i].f};
    for (int k = 0; k < 6; ++k) { o[18 * i + 3 * k] = vv[k].x; o[18 * i + 3 * k + 1] = vv[k].y; o[18 * i + 3 * k + 2] = vv[k].z; }
  }
}

extern "C" void newt_launch_tree_sensor_dyn(const TreeGroupDev& g, const int* idx, int n, float* out, const float* sens,
                                            long sens_stride, cudaStream_t st) {
  const int grid = (n + 63) / 64;
  if (grid == 0) return;
  switch (newt_tree_bucket(g.L)) {
#define X(M) case M: tree_sensor_dyn_kernel<M><<<grid, 64, 0, st>>>(g, idx, n, out, sens, sens_stride); break;
    NEWT_TREE_BUCKETS(X)
#undef X
  }
}

// Loads the plain-form kernels of every size bucket, so that their first
// launch creates nothing on the device.  Returns the first CUDA error met.
extern "C" cudaError_t newt_tree_prepare_kernels() {
  cudaFuncAttributes a;
  cudaError_t e = cudaSuccess;
#define X(M)                                                                             \
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, (const void*)tree_aba_kernel<M>);  \
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, (const void*)tree_integrate_kernel<M>);
  NEWT_TREE_BUCKETS(X)
#undef X
  return e;
}

// The two plain stages on their own (the tree-contact step runs its contact
// solve between them).
extern "C" void newt_launch_tree_aba(const TreeGroupDev& g, cudaStream_t st) {
  const int B = 128;
  const int grid = (g.n + B - 1) / B;
  if (grid == 0) return;
  switch (newt_tree_bucket(g.L)) {
#define X(M) case M: tree_aba_kernel<M><<<grid, B, 0, st>>>(g); break;
    NEWT_TREE_BUCKETS(X)
#undef X
  }
}
extern "C" void newt_launch_tree_integrate(const TreeGroupDev& g, cudaStream_t st) {
  const int B = 128;
  const int grid = (g.n + B - 1) / B;
  if (grid == 0) return;
  switch (newt_tree_bucket(g.L)) {
#define X(M) case M: tree_integrate_kernel<M><<<grid, B, 0, st>>>(g); break;
    NEWT_TREE_BUCKETS(X)
#undef X
  }
}

extern "C" void newt_launch_tree_plain(const TreeGroupDev& g, cudaStream_t st) {
  const int B = 128;
  int grid = (g.n + B - 1) / B;
  if (grid == 0) return;
  switch (newt_tree_bucket(g.L)) {
#define X(M)                                            \
  case M:                                               \
    tree_aba_kernel<M><<<grid, B, 0, st>>>(g);          \
    tree_integrate_kernel<M><<<grid, B, 0, st>>>(g);    \
    break;
    NEWT_TREE_BUCKETS(X)
#undef X
  }
}
