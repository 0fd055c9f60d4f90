// Free-body contact pipeline: the per-row and per-body pieces that every
// pile solver shares (the per-class kernels of pile_kernels.cu and the
// world-persistent kernel of pile_fused.cu), so both run the same
// arithmetic for soft-constraint parameters, PGS row steps and integration.
//
// Restates, for FP32 on sm_103a:
//   newt/src/solver.rs:301-326    impedance_at_position (effective_solimp)
//   newt/src/solver.rs:1448-1518  pgs_step_non_negative / pgs_step_pyramidal_pair
//   newt/src/world.rs:1705-1817   step_bodies_euler and the RK4 branch; world.rs:3223-3271
#pragma once
#include "../../include/newt_gpu.h"
#include "pile_collide.cuh"

namespace pile {

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

struct J6 { V3 l, a; };
NEWT_D float jdot(const J6& j, V3 dv, V3 dw) { return dot(j.l, dv) + dot(j.a, dw); }
NEWT_D J6 jrow(const J6& n, const J6& t, float s) { return J6{n.l + t.l * s, n.a + t.a * s}; }
NEWT_D J6 ldj(const float* p) { return J6{v3(p[0], p[1], p[2]), v3(p[3], p[4], p[5])}; }
NEWT_D void stj(float* p, const J6& j) { p[0] = j.l.x; p[1] = j.l.y; p[2] = j.l.z; p[3] = j.a.x; p[4] = j.a.y; p[5] = j.a.z; }

// ---------------------------------------------------------------------------
// PGS row steps (newt/src/solver.rs:1448-1518), generic over how the
// residual is read and the impulse applied.
// ---------------------------------------------------------------------------
struct RowStep {
  // returns the new impulse for a half-line (f >= 0) step
  NEWT_D static float nonneg(float imp, float res, float idiag) {
    float nf = imp - res * idiag;
    return nf < 0.f ? 0.f : nf;
  }
  // 2x2 pyramidal pair; writes the new impulses
  NEWT_D static void pair(float ii, float ij, float ri, float rj, const float* pb, float* ni_out, float* nj_out) {
    const float h00 = pb[0], h11 = pb[1], h01 = pb[2], idet = pb[3];
    const float di = (-ri * h11 + h01 * rj) * idet;
    const float dj = (h01 * ri - h00 * rj) * idet;
    const float ni = ii + di, nj = ij + dj;
    if (ni >= 0.f && nj >= 0.f) { *ni_out = ni; *nj_out = nj; }
    else if (ni < 0.f && nj < 0.f) { *ni_out = 0.f; *nj_out = 0.f; }
    else if (ni < 0.f) { *ni_out = 0.f; *nj_out = fmaxf(ij - rj / h11, 0.f); }
    else { *ni_out = fmaxf(ii - ri / h00, 0.f); *nj_out = 0.f; }
  }
};



// Map a flat index to (group, index within group) over cumulative segments.
NEWT_D int find_seg(const int* seg, int ng, int t) {
  int lo = 0, hi = ng - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (seg[mid] <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// ---------------------------------------------------------------------------
// K4: integration + write-back (world.rs:1790-1817, 3223-3245)
// ---------------------------------------------------------------------------
// One body's RK4 step under the solver's wrench held constant over the four
// stages (newt/src/world.rs:1705-1788, stage derivative world.rs:3223-3245,
// stage states world.rs:3258-3271).  The wrench comes back from the velocity
// changes the sweeps left: force / mass = dv / dt, world torque =
// R0 Ib R0^T dw / dt.  Stage orientations are not renormalised; the final one
// is, by division (newt/src/math.rs:591-598).  Returns true on a non-finite
// result.
__device__ __forceinline__ bool pile_rk4_body(float* wf, const WsLay& L, int b, float dt, V3 grav) {
  const V3 p0 = ld3(wf + L.pos + 3 * b), v0 = ld3(wf + L.vel + 3 * b), w0 = ld3(wf + L.omg + 3 * b);
  const Q4 q0 = ld4(wf + L.quat + 4 * b);
  const S3 Ib = lds(wf + L.inertb + 6 * b), Ibi = lds(wf + L.iinvb + 6 * b);
  const V3 alin = grav + ld3(wf + L.dv + 3 * b) / dt;
  const V3 tau = qrot(q0, smv(Ib, qrot_inv(q0, ld3(wf + L.dw + 3 * b)))) / dt;
  auto dang_at = [&](Q4 q, V3 om) {
    const V3 gyro = -cross(om, smv(Ib, om));
    return smv(Ibi, qrot_inv(q, tau) + gyro);
  };
  auto dori_at = [&](Q4 q, V3 om) {
    const Q4 d = qmul(q, Q4{om.x, om.y, om.z, 0.f});
    return Q4{d.x * 0.5f, d.y * 0.5f, d.z * 0.5f, d.w * 0.5f};
  };
  auto qstep = [](Q4 a, Q4 d, float h) { return Q4{a.x + d.x * h, a.y + d.y * h, a.z + d.z * h, a.w + d.w * h}; };
  // k1 at s0
  const V3 dp1 = v0, dw1 = dang_at(q0, w0);
  const Q4 dq1 = dori_at(q0, w0);
  const float h = dt * 0.5f;
  // k2 at s0 + k1 dt/2
  V3 vs = v0 + alin * h, ws = w0 + dw1 * h;
  Q4 qs = qstep(q0, dq1, h);
  const V3 dp2 = vs, dw2 = dang_at(qs, ws);
  const Q4 dq2 = dori_at(qs, ws);
  // k3 at s0 + k2 dt/2
  vs = v0 + alin * h; ws = w0 + dw2 * h; qs = qstep(q0, dq2, h);
  const V3 dp3 = vs, dw3 = dang_at(qs, ws);
  const Q4 dq3 = dori_at(qs, ws);
  // k4 at s0 + k3 dt
  vs = v0 + alin * dt; ws = w0 + dw3 * dt; qs = qstep(q0, dq3, dt);
  const V3 dp4 = vs, dw4 = dang_at(qs, ws);
  const Q4 dq4 = dori_at(qs, ws);
  const float sixth = 1.0f / 6.0f;
  const V3 dp = (dp1 + dp2 * 2.f + dp3 * 2.f + dp4) * sixth;
  const V3 dv = (alin + alin * 2.f + alin * 2.f + alin) * sixth;
  const V3 dw = (dw1 + dw2 * 2.f + dw3 * 2.f + dw4) * sixth;
  const Q4 dq{(dq1.x + dq2.x * 2.f + dq3.x * 2.f + dq4.x) * sixth, (dq1.y + dq2.y * 2.f + dq3.y * 2.f + dq4.y) * sixth,
              (dq1.z + dq2.z * 2.f + dq3.z * 2.f + dq4.z) * sixth, (dq1.w + dq2.w * 2.f + dq3.w * 2.f + dq4.w) * sixth};
  const V3 p = p0 + dp * dt, lv = v0 + dv * dt, av = w0 + dw * dt;
  Q4 nq = qstep(q0, dq, dt);
  const float n = sqrtf(nq.x * nq.x + nq.y * nq.y + nq.z * nq.z + nq.w * nq.w);
  nq = n == 0.f ? Q4{0.f, 0.f, 0.f, 1.f} : Q4{nq.x / n, nq.y / n, nq.z / n, nq.w / n};
  st3(wf + L.pos + 3 * b, p); st3(wf + L.vel + 3 * b, lv); st3(wf + L.omg + 3 * b, av);
  wf[L.quat + 4 * b] = nq.x; wf[L.quat + 4 * b + 1] = nq.y; wf[L.quat + 4 * b + 2] = nq.z; wf[L.quat + 4 * b + 3] = nq.w;
  return !(isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(lv.x) && isfinite(lv.y) && isfinite(lv.z) &&
           isfinite(av.x) && isfinite(av.y) && isfinite(av.z) && isfinite(nq.w));
}

// Semi-implicit Euler (or RK4 under the solver's wrench held over the
// stages) of every body of one world, in its scratch record, from the
// velocity changes the solver left in L.dv / L.dw (world frame); one lane
// per body.  Returns, uniformly over the warp, whether any body went
// non-finite.
NEWT_D bool pile_integrate_world(float* wf, const WsLay& L, bool rk4, int lane) {
  const float dt = wf[L.dtg];
  const V3 grav = v3(wf[L.dtg + 1], wf[L.dtg + 2], wf[L.dtg + 3]);
  bool bad = false;
  for (int b = lane; b < L.nb; b += 32) {
    if (rk4) {
      bad |= pile_rk4_body(wf, L, b, dt, grav);
      continue;
    }
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
  bad = __any_sync(0xffffffffu, bad);
  __syncwarp();
  return bad;
}

}  // namespace pile
