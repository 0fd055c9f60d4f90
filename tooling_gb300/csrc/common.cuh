// Shared device-side algebra for the newt GPU kernels (sm_103a, FP32).
//
// Conventions follow newt (newt/src/math.rs, newt/src/spatial.rs):
//   * quaternions are (x, y, z, w), Hamilton product, active rotation;
//   * a spatial motion is (angular; linear), a force is (torque; linear);
//   * a Plucker transform parent->child is (E, t) with
//       motion: w' = E w,  v' = E v + t x (E w)
//       force transpose (child->parent): tau = E^T (tau' - t x f'), f = E^T f'
//     (newt/src/spatial.rs:273-311).
// Unlike the oracle, kernels are free to contract multiply-adds and to use
// cheaper but mathematically equal formulations (symmetric articulated
// inertias, block congruence transforms); parity is by tolerance.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define NEWT_HD __host__ __device__ __forceinline__
#define NEWT_D __device__ __forceinline__

struct V3 { float x, y, z; };
NEWT_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
NEWT_HD V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
NEWT_HD V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
NEWT_HD V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
NEWT_HD V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
NEWT_HD V3 operator*(float s, V3 a) { return v3(a.x * s, a.y * s, a.z * s); }
NEWT_HD V3 operator/(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
NEWT_HD V3& operator+=(V3& a, V3 b) { a = a + b; return a; }
NEWT_HD V3& operator-=(V3& a, V3 b) { a = a - b; return a; }
NEWT_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
NEWT_HD V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
NEWT_HD float len2(V3 a) { return dot(a, a); }

struct Q4 { float x, y, z, w; };
NEWT_HD Q4 qmul(Q4 a, Q4 b) {
  return Q4{a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y, a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
            a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w, a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z};
}
NEWT_HD V3 qrot(Q4 q, V3 v) {  // v + 2w (qv x v) + 2 qv x (qv x v)
  V3 qv = v3(q.x, q.y, q.z);
  V3 t = cross(qv, v) * 2.0f;
  return v + t * q.w + cross(qv, t);
}
NEWT_HD V3 qrot_inv(Q4 q, V3 v) { return qrot(Q4{-q.x, -q.y, -q.z, q.w}, v); }

// Row-major 3x3.
struct M3 { float m[3][3]; };
NEWT_HD V3 mv(const M3& a, V3 v) {
  return v3(a.m[0][0] * v.x + a.m[0][1] * v.y + a.m[0][2] * v.z, a.m[1][0] * v.x + a.m[1][1] * v.y + a.m[1][2] * v.z,
            a.m[2][0] * v.x + a.m[2][1] * v.y + a.m[2][2] * v.z);
}
NEWT_HD V3 mtv(const M3& a, V3 v) {  // a^T v
  return v3(a.m[0][0] * v.x + a.m[1][0] * v.y + a.m[2][0] * v.z, a.m[0][1] * v.x + a.m[1][1] * v.y + a.m[2][1] * v.z,
            a.m[0][2] * v.x + a.m[1][2] * v.y + a.m[2][2] * v.z);
}
NEWT_HD M3 quat_mat(Q4 q) {  // newt/src/math.rs:620-633 in row-major
  float x = q.x, y = q.y, z = q.z, w = q.w;
  M3 r;
  r.m[0][0] = 1.f - 2.f * (y * y + z * z); r.m[0][1] = 2.f * (x * y - z * w); r.m[0][2] = 2.f * (x * z + y * w);
  r.m[1][0] = 2.f * (x * y + z * w); r.m[1][1] = 1.f - 2.f * (x * x + z * z); r.m[1][2] = 2.f * (y * z - x * w);
  r.m[2][0] = 2.f * (x * z - y * w); r.m[2][1] = 2.f * (y * z + x * w); r.m[2][2] = 1.f - 2.f * (x * x + y * y);
  return r;
}

// Symmetric 3x3 stored as (xx, yy, zz, xy, xz, yz).
struct S3 { float xx, yy, zz, xy, xz, yz; };
NEWT_HD V3 smv(const S3& s, V3 v) {
  return v3(s.xx * v.x + s.xy * v.y + s.xz * v.z, s.xy * v.x + s.yy * v.y + s.yz * v.z,
            s.xz * v.x + s.yz * v.y + s.zz * v.z);
}

// Unit quaternion exponential update q * exp(w dt / 2), renormalised
// (newt/src/math.rs:648-650).  Uses CUDA's sincosf.
NEWT_D Q4 q_integrate(Q4 q, V3 om, float dt) {
  float l = sqrtf(len2(om));
  Q4 r;
  if (l > 0.f) {
    float s, c;
    sincosf(0.5f * dt * l, &s, &c);
    float k = s / l;
    r = Q4{om.x * k, om.y * k, om.z * k, c};
  } else {
    r = Q4{0.f, 0.f, 0.f, 1.f};
  }
  Q4 n = qmul(q, r);
  float nn = sqrtf(n.x * n.x + n.y * n.y + n.z * n.z + n.w * n.w);
  if (nn == 0.f) return Q4{0.f, 0.f, 0.f, 1.f};
  float inv = 1.f / nn;
  return Q4{n.x * inv, n.y * inv, n.z * inv, n.w * inv};
}

// Articulated-body inertia in block form [[A, B], [B^T, C]] acting on a
// motion (w; v): torque = A w + B v, force = B^T w + C v.  A and C symmetric.
struct ABI { S3 A; M3 B; S3 C; };

struct SM6 { V3 w, v; };  // spatial motion
struct SF6 { V3 t, f; };  // spatial force

NEWT_HD SF6 abi_mul(const ABI& I, SM6 m) {
  return SF6{smv(I.A, m.w) + mv(I.B, m.v), mtv(I.B, m.w) + smv(I.C, m.v)};
}

// Plucker transform (newt convention, see header comment).
struct PX { M3 E; V3 t; };
NEWT_HD SM6 px_motion(const PX& X, SM6 m) {
  V3 w = mv(X.E, m.w);
  return SM6{w, mv(X.E, m.v) + cross(X.t, w)};
}
NEWT_HD SF6 px_force_T(const PX& X, SF6 f) {  // child force -> parent
  return SF6{mtv(X.E, f.t - cross(X.t, f.f)), mtv(X.E, f.f)};
}

// Congruence E^T S E for symmetric S (6 unique outputs).
NEWT_HD S3 sym_congr(const M3& E, const S3& S) {
  // T = S E (3x3), then E^T T.
  M3 T;
  for (int c = 0; c < 3; ++c) {
    V3 col = v3(E.m[0][c], E.m[1][c], E.m[2][c]);
    V3 r = smv(S, col);
    T.m[0][c] = r.x; T.m[1][c] = r.y; T.m[2][c] = r.z;
  }
  S3 o;
  o.xx = E.m[0][0] * T.m[0][0] + E.m[1][0] * T.m[1][0] + E.m[2][0] * T.m[2][0];
  o.yy = E.m[0][1] * T.m[0][1] + E.m[1][1] * T.m[1][1] + E.m[2][1] * T.m[2][1];
  o.zz = E.m[0][2] * T.m[0][2] + E.m[1][2] * T.m[1][2] + E.m[2][2] * T.m[2][2];
  o.xy = E.m[0][0] * T.m[0][1] + E.m[1][0] * T.m[1][1] + E.m[2][0] * T.m[2][1];
  o.xz = E.m[0][0] * T.m[0][2] + E.m[1][0] * T.m[1][2] + E.m[2][0] * T.m[2][2];
  o.yz = E.m[0][1] * T.m[0][2] + E.m[1][1] * T.m[1][2] + E.m[2][1] * T.m[2][2];
  return o;
}
NEWT_HD M3 gen_congr(const M3& E, const M3& B) {  // E^T B E
  M3 T, o;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) T.m[r][c] = B.m[r][0] * E.m[0][c] + B.m[r][1] * E.m[1][c] + B.m[r][2] * E.m[2][c];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) o.m[r][c] = E.m[0][r] * T.m[0][c] + E.m[1][r] * T.m[1][c] + E.m[2][r] * T.m[2][c];
  return o;
}

// Pull an articulated inertia from the child frame into the parent frame:
// X^T I X (newt's `pull_back`, newt/src/spatial.rs:447-472), in block form.
// With T = skew(t):  C' = C,  B' = B - T C,  A' = A + B T - T B^T - T C T,
// and every block is then taken through E^T (.) E.
NEWT_HD ABI abi_pull_back(const ABI& I, const PX& X) {
  const V3 t = X.t;
  // TC = T * C  (T = skew(t)): row r of T C = t x (column view)
  M3 TC;
  {
    V3 c0 = v3(I.C.xx, I.C.xy, I.C.xz), c1 = v3(I.C.xy, I.C.yy, I.C.yz), c2 = v3(I.C.xz, I.C.yz, I.C.zz);
    V3 a = cross(t, c0), b = cross(t, c1), c = cross(t, c2);
    TC.m[0][0] = a.x; TC.m[1][0] = a.y; TC.m[2][0] = a.z;
    TC.m[0][1] = b.x; TC.m[1][1] = b.y; TC.m[2][1] = b.z;
    TC.m[0][2] = c.x; TC.m[1][2] = c.y; TC.m[2][2] = c.z;
  }
  M3 Bp;  // B - T C
  for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) Bp.m[r][c] = I.B.m[r][c] - TC.m[r][c];
  // A' = A + Bp T - T B^T.  (Bp T)_{rc} = (row r of Bp) x ... : (Bp T) = -(T^T Bp^T)^T ;
  // compute K = Bp * T where T = skew(t): (Bp T)[r][c] = sum_k Bp[r][k] T[k][c]
  float Tm[3][3] = {{0.f, -t.z, t.y}, {t.z, 0.f, -t.x}, {-t.y, t.x, 0.f}};
  M3 K;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) K.m[r][c] = Bp.m[r][0] * Tm[0][c] + Bp.m[r][1] * Tm[1][c] + Bp.m[r][2] * Tm[2][c];
  // T B^T = -(B T)^T ... use A' = A + K + K^T - (T C T + B T + (B T)^T - K - K^T)?  Directly:
  // A' = A + B T - T B^T - T C T = A + K + K^T  because K = B T - T C T and
  // K^T = T^T B^T - T^T C^T T^T = -T B^T - T C T  => K + K^T = B T - T B^T - 2 T C T.
  // So A' = A + K + K^T + T C T; compute T C T = (T C) T.
  M3 TCT;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) TCT.m[r][c] = TC.m[r][0] * Tm[0][c] + TC.m[r][1] * Tm[1][c] + TC.m[r][2] * Tm[2][c];
  S3 Ap;
  Ap.xx = I.A.xx + 2.f * K.m[0][0] + TCT.m[0][0];
  Ap.yy = I.A.yy + 2.f * K.m[1][1] + TCT.m[1][1];
  Ap.zz = I.A.zz + 2.f * K.m[2][2] + TCT.m[2][2];
  Ap.xy = I.A.xy + K.m[0][1] + K.m[1][0] + TCT.m[0][1];
  Ap.xz = I.A.xz + K.m[0][2] + K.m[2][0] + TCT.m[0][2];
  Ap.yz = I.A.yz + K.m[1][2] + K.m[2][1] + TCT.m[1][2];
  ABI o;
  o.A = sym_congr(X.E, Ap);
  o.B = gen_congr(X.E, Bp);
  o.C = sym_congr(X.E, I.C);
  return o;
}

NEWT_HD void abi_add(ABI& a, const ABI& b) {
  a.A.xx += b.A.xx; a.A.yy += b.A.yy; a.A.zz += b.A.zz; a.A.xy += b.A.xy; a.A.xz += b.A.xz; a.A.yz += b.A.yz;
  a.C.xx += b.C.xx; a.C.yy += b.C.yy; a.C.zz += b.C.zz; a.C.xy += b.C.xy; a.C.xz += b.C.xz; a.C.yz += b.C.yz;
  for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) a.B.m[r][c] += b.B.m[r][c];
}

// I - U U^T / D for U a spatial force (t; f) (rank-1 articulated update).
NEWT_HD void abi_rank1_sub(ABI& I, SF6 U, float invD) {
  V3 a = U.t, b = U.f;
  I.A.xx -= a.x * a.x * invD; I.A.yy -= a.y * a.y * invD; I.A.zz -= a.z * a.z * invD;
  I.A.xy -= a.x * a.y * invD; I.A.xz -= a.x * a.z * invD; I.A.yz -= a.y * a.z * invD;
  I.C.xx -= b.x * b.x * invD; I.C.yy -= b.y * b.y * invD; I.C.zz -= b.z * b.z * invD;
  I.C.xy -= b.x * b.y * invD; I.C.xz -= b.x * b.z * invD; I.C.yz -= b.y * b.z * invD;
  float av[3] = {a.x, a.y, a.z}, bv[3] = {b.x, b.y, b.z};
  for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) I.B.m[r][c] -= av[r] * bv[c] * invD;
}

NEWT_HD float sdot6(SM6 m, SF6 f) { return dot(m.w, f.t) + dot(m.v, f.f); }
NEWT_HD SM6 smadd(SM6 a, SM6 b) { return SM6{a.w + b.w, a.v + b.v}; }
NEWT_HD SM6 smscale(SM6 a, float s) { return SM6{a.w * s, a.v * s}; }
NEWT_HD SF6 sfadd(SF6 a, SF6 b) { return SF6{a.t + b.t, a.f + b.f}; }
NEWT_HD SF6 sfsub(SF6 a, SF6 b) { return SF6{a.t - b.t, a.f - b.f}; }
NEWT_HD SF6 sfscale(SF6 a, float s) { return SF6{a.t * s, a.f * s}; }
NEWT_HD SM6 crm(SM6 a, SM6 b) { return SM6{cross(a.w, b.w), cross(a.w, b.v) + cross(a.v, b.w)}; }
NEWT_HD SF6 crf(SM6 a, SF6 f) { return SF6{cross(a.w, f.t) + cross(a.v, f.f), cross(a.w, f.f)}; }

// Symmetric positive-definite 6x6 solve via LDL^T on the block ABI (root of a
// floating-base tree).  Returns false if a pivot is not positive.
NEWT_HD bool abi_solve(const ABI& I, SF6 rhs, SM6* out) {
  float a[6][6];
  a[0][0] = I.A.xx; a[1][1] = I.A.yy; a[2][2] = I.A.zz; a[0][1] = a[1][0] = I.A.xy; a[0][2] = a[2][0] = I.A.xz;
  a[1][2] = a[2][1] = I.A.yz;
  a[3][3] = I.C.xx; a[4][4] = I.C.yy; a[5][5] = I.C.zz; a[3][4] = a[4][3] = I.C.xy; a[3][5] = a[5][3] = I.C.xz;
  a[4][5] = a[5][4] = I.C.yz;
  for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) { a[r][c + 3] = I.B.m[r][c]; a[c + 3][r] = I.B.m[r][c]; }
  float b[6] = {rhs.t.x, rhs.t.y, rhs.t.z, rhs.f.x, rhs.f.y, rhs.f.z};
  // in-place Cholesky
  for (int j = 0; j < 6; ++j) {
    float s = a[j][j];
    for (int k = 0; k < j; ++k) s -= a[j][k] * a[j][k];
    if (!(s > 0.f)) return false;
    float d = sqrtf(s);
    a[j][j] = d;
    float inv = 1.f / d;
    for (int i = j + 1; i < 6; ++i) {
      float t = a[i][j];
      for (int k = 0; k < j; ++k) t -= a[i][k] * a[j][k];
      a[i][j] = t * inv;
    }
  }
  for (int i = 0; i < 6; ++i) { float s = b[i]; for (int k = 0; k < i; ++k) s -= a[i][k] * b[k]; b[i] = s / a[i][i]; }
  for (int i = 5; i >= 0; --i) { float s = b[i]; for (int k = i + 1; k < 6; ++k) s -= a[k][i] * b[k]; b[i] = s / a[i][i]; }
  out->w = v3(b[0], b[1], b[2]);
  out->v = v3(b[3], b[4], b[5]);
  return true;
}

// Bounded launch-status helpers shared by the kernels.
#define NEWT_WS_NONFINITE 0x1u
#define NEWT_WS_NOT_PD 0x2u
#define NEWT_WS_CONTACT_OVERFLOW 0x4u
#define NEWT_WS_ITER_CAP 0x8u
#define NEWT_WS_FP64_FALLBACK 0x10u
