// Oracle (test infrastructure only): scalar, vector, quaternion and spatial
// algebra restated from newt.  Nothing in the shipped GPU path includes this
// file; it is compiled into the CPU checker library and the CPU baseline.
//
// Every routine follows newt's operation order so that the `float`
// instantiation reproduces newt's f32 arithmetic bit for bit when compiled
// with -ffp-contract=off (newt never fuses multiply-adds).  The `double`
// instantiation is the FP64 oracle.
//
// Sources (paths inside hwang2409/tooling):
//   newt/src/math.rs:45-138   deterministic sin/cos (f32 polynomials)
//   newt/src/math.rs:258-665  Vec3, Mat3 (column-major), Quat (x,y,z,w)
//   newt/src/spatial.rs       Xform, SpatialInertia, Mat6
//   newt/src/aba.rs:23-665    generic Scalar algebra used by ABA
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>

namespace oracle {

// ---------------------------------------------------------------------------
// Deterministic sin/cos.  newt evaluates its own polynomials in f32
// (math.rs:45-134).  The f32 mirror reproduces them; the f64 oracle uses the
// platform's correctly rounded double sin/cos, since the f32 polynomials
// would cap its accuracy at ~1e-7.
// ---------------------------------------------------------------------------
inline float newt_sin_poly(float x) {  // math.rs:84-92
  float x2 = x * x;
  float a7 = -1.0f / 5040.0f;
  float a5 = 1.0f / 120.0f;
  float a3 = -1.0f / 6.0f;
  return x * (1.0f + x2 * (a3 + x2 * (a5 + x2 * a7)));
}
inline float newt_cos_poly(float x) {  // math.rs:96-104
  float x2 = x * x;
  float b8 = 1.0f / 40320.0f;
  float b6 = -1.0f / 720.0f;
  float b4 = 1.0f / 24.0f;
  float b2 = -1.0f / 2.0f;
  return 1.0f + x2 * (b2 + x2 * (b4 + x2 * (b6 + x2 * b8)));
}
inline void newt_reduce(float x, float* reduced, int* quadrant) {  // math.rs:113-134
  const float TWO_OVER_PI = 0.63661974f;
  const float C1 = 1.5703125f;
  const float C2 = 4.8370362e-4f;
  const float C3 = 7.5497895e-8f;
  float scaled = x * TWO_OVER_PI;
  int q = scaled >= 0.0f ? (int)(scaled + 0.5f) : (int)(scaled - 0.5f);
  float k = (float)q;
  *reduced = ((x - k * C1) - k * C2) - k * C3;
  *quadrant = q;
}
inline float newt_sin(float x) {
  float r; int q; newt_reduce(x, &r, &q);
  switch (q & 3) {
    case 0: return newt_sin_poly(r);
    case 1: return newt_cos_poly(r);
    case 2: return -newt_sin_poly(r);
    default: return -newt_cos_poly(r);
  }
}
inline float newt_cos(float x) {
  float r; int q; newt_reduce(x, &r, &q);
  switch (q & 3) {
    case 0: return newt_cos_poly(r);
    case 1: return -newt_sin_poly(r);
    case 2: return -newt_cos_poly(r);
    default: return newt_sin_poly(r);
  }
}

template <class R> struct Sc;
template <> struct Sc<float> {
  static float sin(float x) { return newt_sin(x); }
  static float cos(float x) { return newt_cos(x); }
  static float sqrt(float x) { return std::sqrt(x); }
};
template <> struct Sc<double> {
  static double sin(double x) { return std::sin(x); }
  static double cos(double x) { return std::cos(x); }
  static double sqrt(double x) { return std::sqrt(x); }
};

template <class R> inline R rabs(R x) { return x < R(0) ? -x : (x == R(0) ? R(0) : x); }

// ---------------------------------------------------------------------------
// Vec3 / Mat3 / Quat (math.rs)
// ---------------------------------------------------------------------------
template <class R> struct Vec3 {
  R x, y, z;
  Vec3() : x(0), y(0), z(0) {}
  Vec3(R a, R b, R c) : x(a), y(b), z(c) {}
  R dot(const Vec3& r) const { return x * r.x + y * r.y + z * r.z; }
  Vec3 cross(const Vec3& r) const {
    return Vec3(y * r.z - z * r.y, z * r.x - x * r.z, x * r.y - y * r.x);
  }
  R length_squared() const { return dot(*this); }
  R length() const { return Sc<R>::sqrt(length_squared()); }
  Vec3 normalize() const {
    R l = length();
    return l == R(0) ? Vec3() : Vec3(x / l, y / l, z / l);
  }
  Vec3 operator+(const Vec3& r) const { return Vec3(x + r.x, y + r.y, z + r.z); }
  Vec3 operator-(const Vec3& r) const { return Vec3(x - r.x, y - r.y, z - r.z); }
  Vec3 operator-() const { return Vec3(-x, -y, -z); }
  Vec3 operator*(R s) const { return Vec3(x * s, y * s, z * s); }
  Vec3 operator/(R s) const { return Vec3(x / s, y / s, z / s); }
  Vec3& operator+=(const Vec3& r) { *this = *this + r; return *this; }
  Vec3& operator-=(const Vec3& r) { *this = *this - r; return *this; }
  bool operator==(const Vec3& r) const { return x == r.x && y == r.y && z == r.z; }
};

// Column-major: data[c*3+r] (math.rs:377).
template <class R> struct Mat3 {
  R d[9];
  Mat3() { for (int i = 0; i < 9; ++i) d[i] = R(0); d[0] = d[4] = d[8] = R(1); }
  static Mat3 zero() { Mat3 m; for (int i = 0; i < 9; ++i) m.d[i] = R(0); return m; }
  static Mat3 diag(R a, R b, R c) { Mat3 m = zero(); m.d[0] = a; m.d[4] = b; m.d[8] = c; return m; }
  R get(int r, int c) const { return d[c * 3 + r]; }
  Mat3 transpose() const {
    Mat3 m;
    R v[9] = {get(0, 0), get(0, 1), get(0, 2), get(1, 0), get(1, 1), get(1, 2), get(2, 0), get(2, 1), get(2, 2)};
    for (int i = 0; i < 9; ++i) m.d[i] = v[i];
    return m;
  }
  static Mat3 skew(Vec3<R> v) {
    Mat3 m;
    R vals[9] = {R(0), v.z, -v.y, -v.z, R(0), v.x, v.y, -v.x, R(0)};
    for (int i = 0; i < 9; ++i) m.d[i] = vals[i];
    return m;
  }
  bool inverse(Mat3* out) const {  // math.rs:439-465
    R a = get(0, 0), b = get(0, 1), c = get(0, 2), dd = get(1, 0), e = get(1, 1), f = get(1, 2),
      g = get(2, 0), h = get(2, 1), i = get(2, 2);
    R det = a * (e * i - f * h) - b * (dd * i - f * g) + c * (dd * h - e * g);
    if (det == R(0) || !std::isfinite((double)det)) return false;
    R inv = R(1) / det;
    R v[9] = {(e * i - f * h) * inv, (f * g - dd * i) * inv, (dd * h - e * g) * inv,
              (c * h - b * i) * inv, (a * i - c * g) * inv, (b * g - a * h) * inv,
              (b * f - c * e) * inv, (c * dd - a * f) * inv, (a * e - b * dd) * inv};
    for (int k = 0; k < 9; ++k) out->d[k] = v[k];
    return true;
  }
  Vec3<R> operator*(const Vec3<R>& r) const {
    return Vec3<R>(d[0] * r.x + d[3] * r.y + d[6] * r.z, d[1] * r.x + d[4] * r.y + d[7] * r.z,
                   d[2] * r.x + d[5] * r.y + d[8] * r.z);
  }
  Mat3 operator*(const Mat3& r) const {
    Mat3 o;
    for (int col = 0; col < 3; ++col)
      for (int row = 0; row < 3; ++row) {
        R s = R(0);
        for (int k = 0; k < 3; ++k) s += get(row, k) * r.get(k, col);
        o.d[col * 3 + row] = s;
      }
    return o;
  }
  Mat3 operator+(const Mat3& r) const { Mat3 o; for (int i = 0; i < 9; ++i) o.d[i] = d[i] + r.d[i]; return o; }
  Mat3 operator*(R s) const { Mat3 o; for (int i = 0; i < 9; ++i) o.d[i] = d[i] * s; return o; }
};

template <class R> struct Quat {
  R x, y, z, w;
  Quat() : x(0), y(0), z(0), w(1) {}
  Quat(R a, R b, R c, R d) : x(a), y(b), z(c), w(d) {}
  static Quat from_axis_angle(Vec3<R> axis, R angle) {  // math.rs:574-580
    Vec3<R> a = axis.normalize();
    R half = angle * R(0.5);
    R s = Sc<R>::sin(half);
    R c = Sc<R>::cos(half);
    return Quat(a.x * s, a.y * s, a.z * s, c);
  }
  R norm_squared() const { return x * x + y * y + z * z + w * w; }
  R norm() const { return Sc<R>::sqrt(norm_squared()); }
  Quat renormalize() const {
    R n = norm();
    if (n == R(0)) return Quat();
    return Quat(x / n, y / n, z / n, w / n);
  }
  Quat conjugate() const { return Quat(-x, -y, -z, w); }
  Vec3<R> rotate(Vec3<R> v) const {  // math.rs:605-612
    Vec3<R> qv(x, y, z);
    Vec3<R> t = qv.cross(v) * R(2);
    return v + t * w + qv.cross(t);
  }
  Vec3<R> inverse_rotate(Vec3<R> v) const { return conjugate().rotate(v); }
  Mat3<R> to_mat3() const {  // math.rs:620-633
    Mat3<R> m;
    R v[9] = {R(1) - R(2) * (y * y + z * z), R(2) * (x * y + z * w), R(2) * (x * z - y * w),
              R(2) * (x * y - z * w), R(1) - R(2) * (x * x + z * z), R(2) * (y * z + x * w),
              R(2) * (x * z + y * w), R(2) * (y * z - x * w), R(1) - R(2) * (x * x + y * y)};
    for (int i = 0; i < 9; ++i) m.d[i] = v[i];
    return m;
  }
  Quat operator*(const Quat& r) const {  // math.rs:659-668
    return Quat(w * r.x + x * r.w + y * r.z - z * r.y, w * r.y - x * r.z + y * r.w + z * r.x,
                w * r.z + x * r.y - y * r.x + z * r.w, w * r.w - x * r.x - y * r.y - z * r.z);
  }
  Quat operator*(R s) const { return Quat(x * s, y * s, z * s, w * s); }
  Quat operator+(const Quat& r) const { return Quat(x + r.x, y + r.y, z + r.z, w + r.w); }
  Quat derivative(Vec3<R> om) const { return ((*this) * Quat(om.x, om.y, om.z, R(0))) * R(0.5); }
  Quat integrate_body_angular_velocity(Vec3<R> om, R dt) const {  // math.rs:648-650
    return ((*this) * from_axis_angle(om, dt * om.length())).renormalize();
  }
};

// ---------------------------------------------------------------------------
// Spatial algebra, non-generic form (spatial.rs).  Used by the CRB mass
// matrix (dynamics.rs), which goes through `Mat6::pull_back` with `Xform`.
// ---------------------------------------------------------------------------
template <class R> struct SMotion { Vec3<R> ang, lin; };
template <class R> struct SForce { Vec3<R> tau, lin; };

template <class R> inline R sdot(const SMotion<R>& m, const SForce<R>& f) {  // tree.rs:1212
  return m.ang.dot(f.tau) + m.lin.dot(f.lin);
}

template <class R> struct Xform {  // spatial.rs:241
  Mat3<R> rot;     // rot_a_to_b
  Vec3<R> trans;   // translation_a_in_b
  SMotion<R> motion(const SMotion<R>& m) const {
    Vec3<R> w = rot * m.ang;
    Vec3<R> v = rot * m.lin + trans.cross(w);
    return {w, v};
  }
  SForce<R> transpose_force(const SForce<R>& f) const {  // spatial.rs:306-311
    Mat3<R> rt = rot.transpose();
    Vec3<R> fl = rt * f.lin;
    Vec3<R> ft = rt * (f.tau - trans.cross(f.lin));
    return {ft, fl};
  }
};

template <class R> struct Mat6 {  // spatial.rs:333 (row-major rows[r][c])
  R m[6][6];
  static Mat6 zero() { Mat6 o; for (int r = 0; r < 6; ++r) for (int c = 0; c < 6; ++c) o.m[r][c] = R(0); return o; }
  static Mat6 from_spatial_inertia(R mass, Vec3<R> com, Mat3<R> icom) {  // spatial.rs:349-374
    Mat3<R> cx = Mat3<R>::skew(com);
    Mat3<R> cxcx = cx * cx;
    Mat3<R> ul = icom + (cxcx * (-mass));
    Mat3<R> ur = cx * mass;
    Mat3<R> ll = cx * (-mass);
    Mat3<R> lr = Mat3<R>::diag(mass, mass, mass);
    Mat6 o;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        o.m[r][c] = ul.get(r, c); o.m[r][c + 3] = ur.get(r, c);
        o.m[r + 3][c] = ll.get(r, c); o.m[r + 3][c + 3] = lr.get(r, c);
      }
    return o;
  }
  SForce<R> times_motion(const SMotion<R>& mv) const {  // spatial.rs:377-396
    R v[6] = {mv.ang.x, mv.ang.y, mv.ang.z, mv.lin.x, mv.lin.y, mv.lin.z};
    R out[6];
    for (int r = 0; r < 6; ++r) { R s = R(0); for (int c = 0; c < 6; ++c) s += m[r][c] * v[c]; out[r] = s; }
    return {Vec3<R>(out[0], out[1], out[2]), Vec3<R>(out[3], out[4], out[5])};
  }
  Mat6 plus(const Mat6& o) const { Mat6 r = *this; for (int i = 0; i < 6; ++i) for (int j = 0; j < 6; ++j) r.m[i][j] += o.m[i][j]; return r; }
  Mat6 pull_back(const Xform<R>& x) const {  // spatial.rs:447-472
    Mat6 o;
    for (int c = 0; c < 6; ++c) {
      SMotion<R> e;
      if (c < 3) { e.ang = Vec3<R>(c == 0 ? R(1) : R(0), c == 1 ? R(1) : R(0), c == 2 ? R(1) : R(0)); e.lin = Vec3<R>(); }
      else { e.ang = Vec3<R>(); e.lin = Vec3<R>(c == 3 ? R(1) : R(0), c == 4 ? R(1) : R(0), c == 5 ? R(1) : R(0)); }
      SMotion<R> mb = x.motion(e);
      SForce<R> fb = times_motion(mb);
      SForce<R> fa = x.transpose_force(fb);
      o.m[0][c] = fa.tau.x; o.m[1][c] = fa.tau.y; o.m[2][c] = fa.tau.z;
      o.m[3][c] = fa.lin.x; o.m[4][c] = fa.lin.y; o.m[5][c] = fa.lin.z;
    }
    return o;
  }
};

// ---------------------------------------------------------------------------
// Generic-Scalar algebra used by ABA (aba.rs:196-665).  GMat3 is row-major
// data[row][col]; its products start from zero and add terms left to right
// except the f32 `mat3_mul_vec` specialisation, which is a direct 3-term sum.
// ---------------------------------------------------------------------------
template <class R> struct GM3 {
  R a[3][3];
  static GM3 zero() { GM3 o; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) o.a[i][j] = R(0); return o; }
  static GM3 identity() { GM3 o = zero(); o.a[0][0] = o.a[1][1] = o.a[2][2] = R(1); return o; }
  static GM3 from_mat3(const Mat3<R>& m) { GM3 o; for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) o.a[r][c] = m.get(r, c); return o; }
  static GM3 quat(R x, R y, R z, R w) { return from_mat3(Quat<R>(x, y, z, w).to_mat3()); }  // aba.rs:71-78
  Vec3<R> mul_vec(const Vec3<R>& v) const {  // aba.rs:79-85 (f32 form)
    return Vec3<R>(a[0][0] * v.x + a[0][1] * v.y + a[0][2] * v.z, a[1][0] * v.x + a[1][1] * v.y + a[1][2] * v.z,
                   a[2][0] * v.x + a[2][1] * v.y + a[2][2] * v.z);
  }
  Vec3<R> transpose_mul_vec(const Vec3<R>& v) const {  // aba.rs:86-92
    return Vec3<R>(a[0][0] * v.x + a[1][0] * v.y + a[2][0] * v.z, a[0][1] * v.x + a[1][1] * v.y + a[2][1] * v.z,
                   a[0][2] * v.x + a[1][2] * v.y + a[2][2] * v.z);
  }
  GM3 mul(const GM3& r) const {  // aba.rs:379-390
    GM3 o = zero();
    for (int row = 0; row < 3; ++row)
      for (int col = 0; col < 3; ++col)
        for (int k = 0; k < 3; ++k) o.a[row][col] = o.a[row][col] + a[row][k] * r.a[k][col];
    return o;
  }
  GM3 inverse() const {  // aba.rs:391-420
    R d = a[0][0] * a[1][1] - a[0][1] * a[1][0];
    R det = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
            a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
    R inv = R(1) / det;
    GM3 o;
    o.a[0][0] = (a[1][1] * a[2][2] - a[1][2] * a[2][1]) * inv;
    o.a[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * inv;
    o.a[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) * inv;
    o.a[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) * inv;
    o.a[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) * inv;
    o.a[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * inv;
    o.a[2][0] = (a[1][0] * a[2][1] - a[1][1] * a[2][0]) * inv;
    o.a[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * inv;
    o.a[2][2] = d * inv;
    return o;
  }
};

template <class R> struct GMotion {
  Vec3<R> ang, lin;
  GMotion add(const GMotion& r) const { return {ang + r.ang, lin + r.lin}; }
  GMotion scale(R s) const { return {ang * s, lin * s}; }
  GMotion cross_motion(const GMotion& r) const {  // aba.rs:275-284
    return {ang.cross(r.ang), ang.cross(r.lin) + lin.cross(r.ang)};
  }
};
template <class R> struct GForce {
  Vec3<R> tau, lin;
  GForce add(const GForce& r) const { return {tau + r.tau, lin + r.lin}; }
  GForce sub(const GForce& r) const { return {tau - r.tau, lin - r.lin}; }
  GForce scale(R s) const { return {tau * s, lin * s}; }
};
template <class R> inline GForce<R> cross_force(const GMotion<R>& m, const GForce<R>& f) {  // aba.rs:285-293
  return {m.ang.cross(f.tau) + m.lin.cross(f.lin), m.ang.cross(f.lin)};
}
template <class R> inline R dot_force(const GMotion<R>& m, const GForce<R>& f) {  // aba.rs:1105-1108
  return m.ang.dot(f.tau) + m.lin.dot(f.lin);
}

template <class R> struct GX {  // aba.rs:423-452
  GM3<R> rot;
  Vec3<R> trans;
  static GX identity() { return {GM3<R>::identity(), Vec3<R>()}; }
  GMotion<R> motion(const GMotion<R>& m) const {
    Vec3<R> w = rot.mul_vec(m.ang);
    return {w, rot.mul_vec(m.lin) + trans.cross(w)};
  }
  GForce<R> transpose_force(const GForce<R>& f) const {
    Vec3<R> lin = rot.transpose_mul_vec(f.lin);
    Vec3<R> tau = rot.transpose_mul_vec(f.tau - trans.cross(f.lin));
    return {tau, lin};
  }
};

template <class R> struct GM6 {  // aba.rs:454-665
  R m[6][6];
  static GM6 zero() { GM6 o; for (int r = 0; r < 6; ++r) for (int c = 0; c < 6; ++c) o.m[r][c] = R(0); return o; }
  GM6 add(const GM6& o) const { GM6 r = *this; for (int i = 0; i < 6; ++i) for (int j = 0; j < 6; ++j) r.m[i][j] = r.m[i][j] + o.m[i][j]; return r; }
  GM6 sub(const GM6& o) const { GM6 r = *this; for (int i = 0; i < 6; ++i) for (int j = 0; j < 6; ++j) r.m[i][j] = r.m[i][j] - o.m[i][j]; return r; }
  GM6 scale(R s) const { GM6 r = *this; for (int i = 0; i < 6; ++i) for (int j = 0; j < 6; ++j) r.m[i][j] = r.m[i][j] * s; return r; }
  GForce<R> times_motion(const GMotion<R>& mv) const {
    R v[6] = {mv.ang.x, mv.ang.y, mv.ang.z, mv.lin.x, mv.lin.y, mv.lin.z};
    R out[6];
    for (int r = 0; r < 6; ++r) { R s = R(0); for (int c = 0; c < 6; ++c) s = s + m[r][c] * v[c]; out[r] = s; }
    return {Vec3<R>(out[0], out[1], out[2]), Vec3<R>(out[3], out[4], out[5])};
  }
  static GM6 outer(const GForce<R>& f, const GMotion<R>& mv) {
    R rr[6] = {f.tau.x, f.tau.y, f.tau.z, f.lin.x, f.lin.y, f.lin.z};
    R cc[6] = {mv.ang.x, mv.ang.y, mv.ang.z, mv.lin.x, mv.lin.y, mv.lin.z};
    GM6 o;
    for (int r = 0; r < 6; ++r) for (int c = 0; c < 6; ++c) o.m[r][c] = rr[r] * cc[c];
    return o;
  }
  GM6 pull_back(const GX<R>& x) const {
    GM6 o;
    for (int c = 0; c < 6; ++c) {
      GMotion<R> e;
      e.ang = Vec3<R>(c == 0 ? R(1) : R(0), c == 1 ? R(1) : R(0), c == 2 ? R(1) : R(0));
      e.lin = Vec3<R>(c == 3 ? R(1) : R(0), c == 4 ? R(1) : R(0), c == 5 ? R(1) : R(0));
      GMotion<R> t = x.motion(e);
      GForce<R> f = times_motion(t);
      GForce<R> p = x.transpose_force(f);
      R v[6] = {p.tau.x, p.tau.y, p.tau.z, p.lin.x, p.lin.y, p.lin.z};
      for (int r = 0; r < 6; ++r) o.m[r][c] = v[r];
    }
    return o;
  }
  // Gaussian elimination with max-|.| partial pivoting (aba.rs:614-663).
  // Rust's `max_by` keeps the LAST maximal element on ties.
  GMotion<R> solve(const GForce<R>& rhs) const {
    R vals[6] = {rhs.tau.x, rhs.tau.y, rhs.tau.z, rhs.lin.x, rhs.lin.y, rhs.lin.z};
    R a[6][7];
    for (int r = 0; r < 6; ++r) { for (int c = 0; c < 6; ++c) a[r][c] = m[r][c]; a[r][6] = vals[r]; }
    for (int col = 0; col < 6; ++col) {
      int piv = col;
      for (int r = col + 1; r < 6; ++r)
        if (!(rabs(a[r][col]) < rabs(a[piv][col]))) piv = r;
      if (piv != col) for (int k = 0; k < 7; ++k) std::swap(a[col][k], a[piv][k]);
      R scale = a[col][col];
      R inv = R(1) / scale;
      R prow[7]; for (int k = 0; k < 7; ++k) prow[k] = a[col][k];
      for (int row = 0; row < 6; ++row) {
        if (row == col) continue;
        R factor = a[row][col] * inv;
        for (int k = col; k < 7; ++k) a[row][k] = a[row][k] - factor * prow[k];
      }
    }
    return {Vec3<R>(a[0][6] / a[0][0], a[1][6] / a[1][1], a[2][6] / a[2][2]),
            Vec3<R>(a[3][6] / a[3][3], a[4][6] / a[4][4], a[5][6] / a[5][5])};
  }
};

template <class R> inline GM6<R> gm6_from_inertia(R mass, const Mat3<R>& ibody) {
  Mat6<R> m = Mat6<R>::from_spatial_inertia(mass, Vec3<R>(), ibody);
  GM6<R> o;
  for (int r = 0; r < 6; ++r) for (int c = 0; c < 6; ++c) o.m[r][c] = m.m[r][c];
  return o;
}

}  // namespace oracle
