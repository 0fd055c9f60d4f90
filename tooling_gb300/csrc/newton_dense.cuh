// Dense warp-level linear algebra and newt's Newton solve for contact
// impulses, shared by the tree-contact kernel (newton_kernels.cu) and the
// free-body Newton kernel (pile_newton.cu).  One warp owns one system; the
// matrices are column-major in shared or global memory, a lane per row.
//
// Restates, for FP32 on sm_103a (FP64 where noted):
//   newt/src/dynamics.rs:602-648   cholesky, cholesky_solve
//   newt/src/newton.rs:275-339     NewtonSystem::solve
//   newt/src/newton.rs:386-433     project (non-negative rows)
//   newt/src/newton.rs:435-556     exact_pyramidal_line_search
//   newt/src/solver.rs:3215-3232   the zero-friction solver-only pivot
#pragma once
#include "../../include/newt_gpu.h"
#include "common.cuh"

namespace dense {

constexpr unsigned FULL = 0xffffffffu;

NEWT_D float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}
NEWT_D double warp_sumd(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

// In-place lower Cholesky of the n x n column-major matrix A (leading
// dimension ld).  Right-looking: column k is scaled, then the lanes update
// the trailing lower triangle, one lane per row.  Returns false (uniformly)
// when a pivot is not positive; reports the pivot range of L.
template <class T>
NEWT_D bool warp_cholesky(T* A, int n, int ld, int lane, T* min_piv, T* max_piv) {
  T mn = T(1e30), mx = T(0);
  for (int k = 0; k < n; ++k) {
    __syncwarp();
    const T akk = A[(size_t)k * ld + k];
    if (!(akk > T(0))) return false;
    const T lkk = sqrt(akk);
    mn = lkk < mn ? lkk : mn;
    mx = lkk > mx ? lkk : mx;
    const T inv = T(1) / lkk;
    __syncwarp();
    for (int i = k + 1 + lane; i < n; i += 32) A[(size_t)k * ld + i] *= inv;
    if (lane == 0) A[(size_t)k * ld + k] = lkk;
    __syncwarp();
    for (int j = k + 1; j < n; ++j) {
      const T ljk = A[(size_t)k * ld + j];
      for (int i = j + lane; i < n; i += 32) A[(size_t)j * ld + i] -= A[(size_t)k * ld + i] * ljk;
    }
  }
  __syncwarp();
  *min_piv = mn;
  *max_piv = mx;
  return true;
}


// Solves L L^T z = rhs in place on the shared vector `v` (length n) with the
// column-major factor L: forward substitution column by column (lanes update
// the rows below), then backward substitution by row dot products.
template <class T>
NEWT_D void warp_llt_solve(const T* Lf, int n, int ld, float* v, int lane) {
  for (int k = 0; k < n; ++k) {
    __syncwarp();
    const T yk = T(v[k]) / Lf[(size_t)k * ld + k];
    __syncwarp();
    if (lane == 0) v[k] = (float)yk;
    for (int i = k + 1 + lane; i < n; i += 32) v[i] = (float)(T(v[i]) - Lf[(size_t)k * ld + i] * yk);
  }
  for (int k = n - 1; k >= 0; --k) {
    __syncwarp();
    T s = T(0);
    for (int m = k + 1 + lane; m < n; m += 32) s += Lf[(size_t)k * ld + m] * T(v[m]);
    if (sizeof(T) == 8) s = (T)warp_sumd((double)s); else s = (T)warp_sum((float)s);
    const T zk = (T(v[k]) - s) / Lf[(size_t)k * ld + k];
    __syncwarp();
    if (lane == 0) v[k] = (float)zk;
  }
  __syncwarp();
}

// Solves L L^T z = v in FP64 with the FP32 column-major factor L (FP64
// vector `v`, in place; forward then backward substitution).
NEWT_D void warp_llt_solve_mixed(const float* Lf, int n, int ld, double* v, int lane) {
  for (int k = 0; k < n; ++k) {
    __syncwarp();
    const double yk = v[k] / (double)Lf[(size_t)k * ld + k];
    __syncwarp();
    if (lane == 0) v[k] = yk;
    for (int i = k + 1 + lane; i < n; i += 32) v[i] -= (double)Lf[(size_t)k * ld + i] * yk;
  }
  for (int k = n - 1; k >= 0; --k) {
    __syncwarp();
    double s = 0.0;
    for (int m = k + 1 + lane; m < n; m += 32) s += (double)Lf[(size_t)k * ld + m] * v[m];
    s = warp_sumd(s);
    const double zk = (v[k] - s) / (double)Lf[(size_t)k * ld + k];
    __syncwarp();
    if (lane == 0) v[k] = zk;
  }
  __syncwarp();
}

// out = H x (column-major H, lane per row; x shared).
NEWT_D void warp_matvec(const float* H, int n, int ld, const float* x, float* out, int lane) {
  __syncwarp();
  for (int r = lane; r < n; r += 32) {
    float s = 0.f;
    for (int c = 0; c < n; ++c) s += H[(size_t)c * ld + r] * x[c];
    out[r] = s;
  }
  __syncwarp();
}
NEWT_D float warp_dot(const float* a, const float* b, int n, int lane) {
  float s = 0.f;
  for (int r = lane; r < n; r += 32) s += a[r] * b[r];
  return warp_sum(s);
}
// the same dot accumulated in FP64 (each f32 product is exact in double)
NEWT_D double warp_dot_d(const float* a, const float* b, int n, int lane) {
  double s = 0.0;
  for (int r = lane; r < n; r += 32) s += (double)a[r] * (double)b[r];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

// min 1/2 x^T H x + b^T x subject to x >= 0 on every row: newt's
// NewtonSystem::solve with its exact piecewise line search, the rows being
// pyramidal facets or frictionless normals (all non-negative).  H (leading
// dimension ld) holds A + diag(R); the f32 factor goes to LH (leading
// dimension ldh, may alias shared memory), the FP64 fallback's to LHd (ld).
// When the f32 factor's pivot ratio (max L_ii / min L_ii)^2 exceeds 1e6 or
// it fails, the factor and the direction solves are redone in FP64
// (NEWT_WS_FP64_FALLBACK).  zero_mu: some row is a zero-friction facet, for
// which newt adds a solver-only pivot before it gives up on the factor.  x,
// b and the scratch vectors d, g, p, s, u, v and brk hold at least nr
// values.  Returns the iterations taken; ORs NEWT_WS_FP64_FALLBACK,
// NEWT_WS_NOT_PD (x = 0) and NEWT_WS_ITER_CAP into *status.  kinds
// (nullable: every row non-negative): per row a code whose value below -1
// marks a row without projection (newt's general contact rows under the
// pyramidal cone, whose tangent, torsion and rolling rows carry none).
NEWT_D int newton_solve(float* H, int nr, int ld, float* LH, int ldh, double* LHd, float* vx, const float* vb,
                        float* vd, float* vg, float* vp, float* vs, float* vu, float* vv, float* vbrk, int iters,
                        bool zero_mu, int lane, uint32_t* status, const int* kinds = nullptr) {
  auto projected = [&](int r) { return !kinds || kinds[r] >= -1; };
  float mn = 0.f, mx = 0.f;
  int done_it = 0;
  auto copy_h = [&]() {
    __syncwarp();
    for (int c = 0; c < nr; ++c)
      for (int r = lane; r < nr; r += 32) LH[(size_t)c * ldh + r] = H[(size_t)c * ld + r];
    __syncwarp();
  };
  copy_h();
  bool ok = warp_cholesky(LH, nr, ldh, lane, &mn, &mx);
  if (!ok) {
    // zero-friction facets duplicate rows: a solver-only pivot (solver.rs:3215-3232)
    if (zero_mu) {
      float sc = 0.f;
      for (int c = 0; c < nr; ++c)
        for (int r = lane; r < nr; r += 32) sc = fmaxf(sc, fabsf(H[(size_t)c * ld + r]));
      for (int o = 16; o > 0; o >>= 1) sc = fmaxf(sc, __shfl_xor_sync(FULL, sc, o));
      const float piv = fmaxf(sc * 1.0e-6f, 1.0e-7f);
      __syncwarp();
      for (int r = lane; r < nr; r += 32) H[(size_t)r * ld + r] += piv;
      copy_h();
      ok = warp_cholesky(LH, nr, ldh, lane, &mn, &mx);
    }
  }
  bool use64 = !ok || (mx / mn) * (mx / mn) > 1.0e6f;
  if (use64) {
    __syncwarp();
    for (int c = 0; c < nr; ++c)
      for (int r = lane; r < nr; r += 32) LHd[(size_t)c * ld + r] = (double)H[(size_t)c * ld + r];
    double mnd, mxd;
    ok = warp_cholesky(LHd, nr, ld, lane, &mnd, &mxd);
    *status |= NEWT_WS_FP64_FALLBACK;
  }
  if (!ok) {
    *status |= NEWT_WS_NOT_PD;
    for (int r = lane; r < nr; r += 32) vx[r] = 0.f;
  } else {
    // The costs that steer the line search and the stopping test are kept
    // in FP64: the window products below change by incremental updates as
    // coordinates leave the free set, and the stopping test compares cost
    // decreases at 1e-7 of the cost, the f32 rounding level of the sums.
    // The cost at the current point is evaluated afresh every iteration,
    // 0.5 x.(H x) + b.x, as newt's quad_cost does, not carried over from
    // the line search's estimate.
    double cur = 0.0;  // cost at x = 0
    const int max_it = iters > 1 ? iters : 1;
    for (int it = 0; it < max_it; ++it) {
      // gradient g = H x + b, direction d = -(L L^T)^-1 g
      warp_matvec(H, nr, ld, vx, vg, lane);
      if (it > 0) cur = 0.5 * warp_dot_d(vx, vg, nr, lane) + warp_dot_d(vx, vb, nr, lane);  // vg = H x here
      for (int r = lane; r < nr; r += 32) { vg[r] += vb[r]; vd[r] = -vg[r]; }
      __syncwarp();
      if (use64) warp_llt_solve(LHd, nr, ld, vd, lane);
      else warp_llt_solve(LH, nr, ldh, vd, lane);
      if (warp_dot(vg, vd, nr, lane) >= 0.f) break;
      // ---- exact line search over the projected path (newton.rs:435-556) ----
      for (int r = lane; r < nr; r += 32) {
        const float x = vx[r], d = vd[r];
        const bool pr = projected(r);
        const bool fr = !pr || x > 0.f || (x == 0.f && d > 0.f);
        vp[r] = fr ? x : 0.f;
        vs[r] = fr ? d : 0.f;
        const float a = (pr && x > 0.f && d < 0.f) ? -x / d : 2.f;  // where x + a d reaches zero
        vbrk[r] = (a > 0.f && a < 1.f) ? a : 2.f;
      }
      warp_matvec(H, nr, ld, vp, vu, lane);
      warp_matvec(H, nr, ld, vs, vv, lane);
      float best_a = 0.f, lo = 0.f;
      double best_c = cur;
      // cost on a window: c0 + c1 a + c2 a^2 / 2 with p = P + a S; the five
      // products are updated in O(1) when a coordinate leaves the free set
      double Pu = warp_dot_d(vp, vu, nr, lane), Pv = warp_dot_d(vp, vv, nr, lane);
      double Sv = warp_dot_d(vs, vv, nr, lane), bP = warp_dot_d(vb, vp, nr, lane), bS = warp_dot_d(vb, vs, nr, lane);
      for (int guard = 0; guard <= nr; ++guard) {
        // next breakpoint (warp argmin)
        float bm = 2.f;
        int bi = -1;
        for (int r = lane; r < nr; r += 32) if (vbrk[r] < bm) { bm = vbrk[r]; bi = r; }
        for (int o = 16; o > 0; o >>= 1) {
          const float om = __shfl_xor_sync(FULL, bm, o);
          const int oi = __shfl_xor_sync(FULL, bi, o);
          if (om < bm || (om == bm && oi >= 0 && (bi < 0 || oi < bi))) { bm = om; bi = oi; }
        }
        const float hi = bm < 1.f ? bm : 1.f;
        if (hi - lo > 1.0e-7f) {
          const double c0 = 0.5 * Pu + bP, c1 = Pv + bS, c2 = Sv;
          const float opt = c2 > 0.0 ? fminf(fmaxf((float)(-c1 / c2), lo), hi) : 0.5f * (lo + hi);
          const float cand[3] = {lo, hi, opt};
          for (int k = 0; k < 3; ++k) {
            const double a = cand[k];
            const double cost = c0 + c1 * a + 0.5 * c2 * a * a;
            if (cost < best_c) { best_c = cost; best_a = cand[k]; }
          }
        }
        if (bi < 0) break;
        // coordinate bi leaves the free set: P, S lose it, H P and H S a column
        const double xj = vp[bi], dj = vs[bi], uj = vu[bi], vj = vv[bi], bj = vb[bi];
        const double hjj = H[(size_t)bi * ld + bi];
        Pu += (xj * hjj - 2.0 * uj) * xj;
        Pv += xj * dj * hjj - xj * vj - dj * uj;
        Sv += (dj * hjj - 2.0 * vj) * dj;
        bP -= bj * xj;
        bS -= bj * dj;
        __syncwarp();
        for (int r = lane; r < nr; r += 32) {
          const float hc = H[(size_t)bi * ld + r];
          vu[r] -= (float)xj * hc;
          vv[r] -= (float)dj * hc;
        }
        if (lane == 0) { vp[bi] = 0.f; vs[bi] = 0.f; vbrk[bi] = 2.f; }
        __syncwarp();
        lo = hi;
      }
      if (best_a <= 0.f || cur - best_c <= 1.0e-7 * (1.0 + fabs(cur))) break;
      for (int r = lane; r < nr; r += 32) {
        const float x = vx[r] + best_a * vd[r];
        vx[r] = (projected(r) && x < 0.f) ? 0.f : x;
      }
      __syncwarp();
      done_it = it + 1;
    }
    if (done_it == max_it) *status |= NEWT_WS_ITER_CAP;
  }
  __syncwarp();
  return done_it;
}

}  // namespace dense
