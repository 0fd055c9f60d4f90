// Oracle (test infrastructure only): newt's GJK/EPA convex contact for the
// primitive shapes (sphere, box, capsule), restated in C++ over R = float or
// double.  It is the checker's second, independent formulation of the
// sphere-box pair (which newt routes nowhere; the closed form in
// newt_world.hpp is the first) and a cross-check of the box-box SAT.
//
// Restates newt/src/contact/ccd.rs:
//   :68-170     CcdShape centre, extent, support (sphere, box, capsule)
//   :322-344    ccd_vertex_precedes / sort_ccd_vertices (deterministic ties)
//   :360-388    ccd_support, ccd_support_normalized (Minkowski points scaled
//               by the pair extent), triple_product
//   :442-546    ccd_simplex_step (intersection GJK)
//   :658-694    ccd_closest_witness
//   :704-868    distance candidates, ccd_distance_simplex_step
//   :870-908    ccd_distance_contact
//   :910-978    ccd_distance_gjk
//   :1036-1092  ccd_face, ccd_face_precedes
//   :1106-1183  ccd_epa_fallback_contact
//   :1703-1911  ccd_convex_contact (GJK, then EPA over at most 128 vertices
//               and 512 faces)
// and newt/src/contact.rs:64-78 (lexicographic order), :2265-2318
// (closest_point_on_triangle), ccd.rs:2094-2109 (barycentric weights).
// For primitive shapes no support ties are tagged and no centred witness
// applies (ccd.rs:171-187), so witnesses are the barycentric mixes of the
// simplex's support points.
#pragma once
#include <cmath>

#include "newt_math.hpp"
#include "newt_world.hpp"

namespace oracle {
namespace ccd {

enum { SPHERE = 1, BOX = 2, CAPSULE = 3 };

template <class R> struct Shape {
  int kind;
  Vec3<R> p;
  Quat<R> q;
  Vec3<R> size;  // sphere: r; box: half extents; capsule: r, half height
};

template <class R> struct Vtx { Vec3<R> m, a, b; };
template <class R> struct Simplex { Vtx<R> p[4]; int n = 0; };
template <class R> struct Result {
  bool hit = false;
  Vec3<R> pos, n, wa, wb;  // contact point, normal (from B into A), witnesses on A and B
  R pen = R(0);
  int path = 0;  // 1 distance GJK, 2 EPA, 3 EPA fallback
};

template <class R> inline R degen2() { return R(1.0e-24); }  // (1e-12)^2

template <class R> inline bool lex_less(Vec3<R> a, Vec3<R> b) {
  if (a.x != b.x) return a.x < b.x;
  if (a.y != b.y) return a.y < b.y;
  return a.z < b.z;
}
template <class R> inline bool same(Vec3<R> a, Vec3<R> b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
template <class R> inline bool vtx_less(const Vtx<R>& a, const Vtx<R>& b) {
  if (!same(a.m, b.m)) return lex_less(a.m, b.m);
  if (!same(a.a, b.a)) return lex_less(a.a, b.a);
  if (!same(a.b, b.b)) return lex_less(a.b, b.b);
  return false;
}
template <class R> inline void sort_vtx(Vtx<R>* v, int n) {
  for (int i = 1; i < n; ++i)
    for (int k = i; k > 0 && vtx_less(v[k], v[k - 1]); --k) { Vtx<R> t = v[k]; v[k] = v[k - 1]; v[k - 1] = t; }
}

template <class R> inline R clamp01v(R x) { return x < R(0) ? R(0) : (x > R(1) ? R(1) : x); }

template <class R> R extent(const Shape<R>& s) {
  if (s.kind == SPHERE) return s.size.x * R(2);
  if (s.kind == BOX) return (s.size * R(2)).length();
  return R(2) * (s.size.y + s.size.x);
}

template <class R> Vec3<R> support(const Shape<R>& s, Vec3<R> d) {
  if (!(d.length_squared() > R(1.0e-20))) d = Vec3<R>(1, 0, 0);
  if (s.kind == SPHERE) return s.p + d.normalize() * s.size.x;
  if (s.kind == BOX) {
    Vec3<R> l = s.q.inverse_rotate(d);
    Vec3<R> c(l.x >= R(0) ? s.size.x : -s.size.x, l.y >= R(0) ? s.size.y : -s.size.y,
              l.z >= R(0) ? s.size.z : -s.size.z);
    return s.p + s.q.rotate(c);
  }
  Vec3<R> ax = s.q.rotate(Vec3<R>(0, 0, 1));
  Vec3<R> end = d.dot(ax) >= R(0) ? s.p + ax * s.size.y : s.p - ax * s.size.y;
  return end + d.normalize() * s.size.x;
}

template <class R> Vtx<R> support_pair(const Shape<R>& A, const Shape<R>& B, Vec3<R> d, R ext) {
  if (!(d.length_squared() > degen2<R>())) d = Vec3<R>(1, 0, 0);
  Vtx<R> v;
  v.a = support(A, d);
  v.b = support(B, -d);
  v.m = (v.a - v.b) / ext;
  return v;
}

template <class R> inline Vec3<R> triple(Vec3<R> a, Vec3<R> b, Vec3<R> c) { return b * a.dot(c) - a * b.dot(c); }

// intersection GJK step (ccd.rs:442-546): newest point last; true when the
// simplex encloses the origin
template <class R> bool simplex_step(Simplex<R>& s, Vec3<R>& dir) {
  const R eps2 = degen2<R>();
  const Vtx<R> a = s.p[s.n - 1];
  const Vec3<R> ao = -a.m;
  auto set = [&](std::initializer_list<Vtx<R>> l) { int k = 0; for (const auto& v : l) s.p[k++] = v; s.n = k; };
  if (s.n == 2) {
    const Vtx<R> b = s.p[0];
    const Vec3<R> ab = b.m - a.m;
    if (ab.dot(ao) > R(0)) {
      dir = triple(ab, ao, ab);
      if (dir.length_squared() <= eps2) dir = Vec3<R>(0, 0, 1);
    } else {
      set({a});
      dir = ao;
    }
  } else if (s.n == 3) {
    const Vtx<R> b = s.p[1], c = s.p[0];
    const Vec3<R> ab = b.m - a.m, ac = c.m - a.m, abc = ab.cross(ac);
    if (abc.length_squared() <= eps2) {
      set({a, b});
      const R el = ab.length_squared();
      const R t = el > eps2 ? clamp01v(-a.m.dot(ab) / el) : R(0);
      const Vec3<R> cl = a.m + ab * t;
      if (cl.length_squared() > eps2) { dir = -cl; return false; }
      Vec3<R> axis;
      if (rabs(ab.x) <= rabs(ab.y) && rabs(ab.x) <= rabs(ab.z)) axis = Vec3<R>(1, 0, 0);
      else if (rabs(ab.y) <= rabs(ab.z)) axis = Vec3<R>(0, 1, 0);
      else axis = Vec3<R>(0, 0, 1);
      dir = ab.cross(axis);
      if (dir.length_squared() <= eps2) dir = ao;
      return false;
    }
    if (abc.cross(ac).dot(ao) > R(0)) {
      if (ac.dot(ao) > R(0)) { set({a, c}); dir = triple(ac, ao, ac); }
      else if (ab.dot(ao) > R(0)) { set({a, b}); dir = triple(ab, ao, ab); }
      else { set({a}); dir = ao; }
    } else if (ab.cross(abc).dot(ao) > R(0)) {
      if (ab.dot(ao) > R(0)) { set({a, b}); dir = triple(ab, ao, ab); }
      else { set({a}); dir = ao; }
    } else if (abc.dot(ao) > R(0)) {
      dir = abc;
    } else {
      set({a, c, b});
      dir = -abc;
    }
  } else {
    const Vtx<R> b = s.p[2], c = s.p[1], d = s.p[0];
    const Vec3<R> ab = b.m - a.m, ac = c.m - a.m, ad = d.m - a.m;
    const Vec3<R> abc = ab.cross(ac), acd = ac.cross(ad), adb = ad.cross(ab);
    if (abc.dot(ao) > R(0)) { set({a, c, b}); dir = abc; }
    else if (acd.dot(ao) > R(0)) { set({a, d, c}); dir = acd; }
    else if (adb.dot(ao) > R(0)) { set({a, b, d}); dir = adb; }
    else return true;
  }
  if (dir.length_squared() <= eps2) dir = Vec3<R>(1, 0, 0);
  return false;
}

template <class R> Vec3<R> closest_on_triangle(Vec3<R> p, Vec3<R> a, Vec3<R> b, Vec3<R> c) {
  const Vec3<R> ab = b - a, ac = c - a, ap = p - a;
  const R d1 = ab.dot(ap), d2 = ac.dot(ap);
  if (d1 <= R(0) && d2 <= R(0)) return a;
  const Vec3<R> bp = p - b;
  const R d3 = ab.dot(bp), d4 = ac.dot(bp);
  if (d3 >= R(0) && d4 <= d3) return b;
  const R vc = d1 * d4 - d3 * d2;
  if (vc <= R(0) && d1 >= R(0) && d3 <= R(0)) return a + ab * (d1 / (d1 - d3));
  const Vec3<R> cp = p - c;
  const R d5 = ab.dot(cp), d6 = ac.dot(cp);
  if (d6 >= R(0) && d5 <= d6) return c;
  const R vb = d5 * d2 - d1 * d6;
  if (vb <= R(0) && d2 >= R(0) && d6 <= R(0)) return a + ac * (d2 / (d2 - d6));
  const R va = d3 * d6 - d5 * d4;
  if (va <= R(0) && (d4 - d3) >= R(0) && (d5 - d6) >= R(0)) return b + (c - b) * ((d4 - d3) / ((d4 - d3) + (d5 - d6)));
  const R den = R(1) / (va + vb + vc);
  return a + ab * (vb * den) + ac * (vc * den);
}

template <class R> void barycentric(Vec3<R> a, Vec3<R> b, Vec3<R> c, Vec3<R> p, R w[3]) {
  const Vec3<R> v0 = b - a, v1 = c - a, v2 = p - a;
  const R d00 = v0.dot(v0), d01 = v0.dot(v1), d11 = v1.dot(v1), d20 = v2.dot(v0), d21 = v2.dot(v1);
  const R den = d00 * d11 - d01 * d01;
  if (rabs(den) <= R(1.0e-12)) { w[0] = R(1); w[1] = w[2] = R(0); return; }
  const R v = (d11 * d20 - d01 * d21) / den, ww = (d00 * d21 - d01 * d20) / den;
  w[0] = R(1) - v - ww; w[1] = v; w[2] = ww;
}

template <class R> void mix(const Vtx<R>* v, const R* w, int n, Vec3<R>* pa, Vec3<R>* pb) {
  *pa = Vec3<R>(); *pb = Vec3<R>();
  for (int k = 0; k < n; ++k) { *pa += v[k].a * w[k]; *pb += v[k].b * w[k]; }
}

template <class R> void triangle_witness(const Vtx<R>& a, const Vtx<R>& b, const Vtx<R>& c, Vec3<R>* pa, Vec3<R>* pb) {
  const Vec3<R> nearest = closest_on_triangle(Vec3<R>(), a.m, b.m, c.m);
  R w[3];
  barycentric(a.m, b.m, c.m, nearest, w);
  const Vtx<R> v[3] = {a, b, c};
  mix(v, w, 3, pa, pb);
}

// ccd.rs:658-694
template <class R> bool closest_witness(const Simplex<R>& s, Vec3<R>* pa, Vec3<R>* pb) {
  if (s.n == 1) { *pa = s.p[0].a; *pb = s.p[0].b; return true; }
  if (s.n == 2) {
    const Vec3<R> e = s.p[1].m - s.p[0].m;
    const R den = e.length_squared();
    const R t = den > degen2<R>() ? clamp01v(-s.p[0].m.dot(e) / den) : R(0);
    const R w[2] = {R(1) - t, t};
    mix(s.p, w, 2, pa, pb);
    return true;
  }
  if (s.n == 3) { triangle_witness(s.p[0], s.p[1], s.p[2], pa, pb); return true; }
  if (s.n == 4) {
    const int faces[4][3] = {{0, 1, 2}, {0, 3, 1}, {0, 2, 3}, {1, 3, 2}};
    R best = R(0);
    bool have = false;
    for (auto& f : faces) {
      Vec3<R> a, b;
      triangle_witness(s.p[f[0]], s.p[f[1]], s.p[f[2]], &a, &b);
      const R d2 = (a - b).length_squared();
      if (!have || d2 < best) { best = d2; *pa = a; *pb = b; have = true; }
    }
    return have;
  }
  return false;
}

template <class R> struct Cand { Vec3<R> pt; R w[4]; Vtx<R> f[3]; int fn; };

// ccd.rs:727-792: closest point of one vertex, edge or face region
template <class R> bool candidate(const Simplex<R>& s, int mask, Cand<R>* out) {
  int idx[3], k = 0;
  for (int i = 0; i < s.n; ++i)
    if (mask & (1 << i)) { if (k == 3) return false; idx[k++] = i; }
  for (int i = 1; i < k; ++i)
    for (int p = i; p > 0 && vtx_less(s.p[idx[p]], s.p[idx[p - 1]]); --p) { int t = idx[p]; idx[p] = idx[p - 1]; idx[p - 1] = t; }
  R sw[3] = {R(1), R(0), R(0)};
  Vec3<R> pt;
  if (k == 1) pt = s.p[idx[0]].m;
  else if (k == 2) {
    const Vec3<R> a = s.p[idx[0]].m, e = s.p[idx[1]].m - a;
    const R den = e.length_squared();
    const R t = den > degen2<R>() ? clamp01v(-a.dot(e) / den) : R(0);
    pt = a + e * t; sw[0] = R(1) - t; sw[1] = t;
  } else {
    const Vec3<R> a = s.p[idx[0]].m, b = s.p[idx[1]].m, c = s.p[idx[2]].m;
    if ((b - a).cross(c - a).length_squared() <= degen2<R>()) return false;
    pt = closest_on_triangle(Vec3<R>(), a, b, c);
    barycentric(a, b, c, pt, sw);
  }
  out->pt = pt;
  for (int i = 0; i < 4; ++i) out->w[i] = R(0);
  for (int i = 0; i < k; ++i) out->w[idx[i]] = sw[i];
  for (int i = 0; i < 3; ++i) out->f[i] = s.p[idx[0]];
  for (int i = 0; i < k; ++i) out->f[i] = s.p[idx[i]];
  out->fn = k;
  return true;
}

template <class R> bool cand_less(const Cand<R>& c, const Cand<R>& d) {
  const R cd = c.pt.length_squared(), dd = d.pt.length_squared();
  if (cd != dd) return cd < dd;
  if (c.fn != d.fn) return c.fn < d.fn;
  for (int i = 0; i < c.fn; ++i) {
    if (vtx_less(c.f[i], d.f[i])) return true;
    if (vtx_less(d.f[i], c.f[i])) return false;
  }
  return lex_less(c.pt, d.pt);
}

template <class R> bool origin_in_tetra(const Simplex<R>& s) {
  const Vec3<R> a = s.p[0].m, b = s.p[1].m, c = s.p[2].m, d = s.p[3].m;
  const Vec3<R> ab = b - a, ac = c - a, ad = d - a;
  const R den = ab.cross(ac).dot(ad);
  if (rabs(den) <= degen2<R>()) return false;
  const Vec3<R> ao = -a;
  const R wb = ao.cross(ac).dot(ad) / den, wc = ab.cross(ao).dot(ad) / den, wd = ab.cross(ac).dot(ao) / den;
  const R w[4] = {R(1) - wb - wc - wd, wb, wc, wd};
  for (R x : w)
    if (!(x >= R(-1.0e-6) && x <= R(1) + R(1.0e-6))) return false;
  return true;
}

// ccd.rs:822-868: reduce to the closest feature; false when the origin is inside
template <class R> bool distance_step(Simplex<R>& s, Vec3<R>* closest) {
  if (s.n == 4 && origin_in_tetra(s)) return false;
  Cand<R> best{};
  bool have = false;
  for (int mask = 1; mask < (1 << s.n); ++mask) {
    Cand<R> c;
    if (!candidate(s, mask, &c)) continue;
    if (!have || cand_less(c, best)) { best = c; have = true; }
  }
  if (!have) return false;
  Vtx<R> sel[4];
  int k = 0;
  for (int i = 0; i < s.n; ++i)
    if (best.w[i] > R(1.0e-6)) sel[k++] = s.p[i];
  if (k == 0) {
    int li = 0;
    for (int i = 1; i < s.n; ++i) {
      const R dw = best.w[i] - best.w[li];
      if (dw > R(1.0e-6) || (rabs(dw) <= R(1.0e-6) && vtx_less(s.p[i], s.p[li]))) li = i;
    }
    sel[0] = s.p[li];
    k = 1;
  }
  sort_vtx(sel, k);
  for (int i = 0; i < k; ++i) s.p[i] = sel[i];
  s.n = k;
  *closest = best.pt;
  return true;
}

// ccd.rs:910-978 (mesh configuration: support epsilon 0, tolerance 1e-10)
template <class R> Simplex<R> distance_gjk(const Shape<R>& A, const Shape<R>& B, Simplex<R> s, R ext) {
  const R floor2 = degen2<R>(), tol = R(1.0e-10), sup_eps = R(0);
  Simplex<R> best_s = s;
  R best = R(INFINITY);
  for (int it = 0; it < 64; ++it) {
    Vec3<R> cl;
    if (!distance_step(s, &cl)) return best_s;
    const R d2 = cl.length_squared();
    if (d2 < best) { best = d2; best_s = s; }
    if (d2 <= floor2) return best_s;
    const Vec3<R> dir = -cl;
    const Vtx<R> p = support_pair(A, B, dir, ext);
    if (p.m.dot(dir) - cl.dot(dir) <= sup_eps) return best_s;
    for (int i = 0; i < s.n; ++i)
      if ((s.p[i].m - p.m).length_squared() <= floor2) return best_s;
    s.p[s.n++] = p;
    Vec3<R> nc;
    if (!distance_step(s, &nc)) return best_s;
    const R n2 = nc.length_squared();
    if (n2 < best) { best = n2; best_s = s; }
    if (d2 - n2 <= tol * (d2 > floor2 ? d2 : floor2)) return best_s;
  }
  return best_s;
}

template <class R> Result<R> distance_contact(const Simplex<R>& s, R margin) {
  Result<R> r;
  Vec3<R> pa, pb;
  if (!closest_witness(s, &pa, &pb)) return r;
  const Vec3<R> sep = pa - pb;
  const R dist = sep.length();
  const R pen = margin - dist;
  if (pen <= R(0)) return r;
  r.hit = true;
  r.wa = pa; r.wb = pb;
  r.n = dist > R(0) ? sep / dist : Vec3<R>(1, 0, 0);
  r.pos = (pa + pb) * R(0.5);
  r.pen = pen;
  r.path = 1;
  return r;
}

template <class R> struct Face { int i[3]; Vec3<R> n; R d; };

template <class R> bool make_face(const Vtx<R>* v, int a, int b, int c, Face<R>* f) {
  const Vec3<R> raw = (v[b].m - v[a].m).cross(v[c].m - v[a].m);
  if (raw.length_squared() <= degen2<R>()) return false;
  Vec3<R> n = raw.normalize();
  R d = n.dot(v[a].m);
  f->i[0] = a; f->i[1] = b; f->i[2] = c;
  if (d < R(0)) { f->i[1] = c; f->i[2] = b; n = -n; d = -d; }
  f->n = n;
  f->d = d;
  return true;
}

template <class R> bool face_less(const Vtx<R>* v, const Face<R>& c, const Face<R>& d, R tie) {
  if (c.d + tie < d.d) return true;
  if (d.d + tie < c.d) return false;
  Vtx<R> ck[3] = {v[c.i[0]], v[c.i[1]], v[c.i[2]]}, dk[3] = {v[d.i[0]], v[d.i[1]], v[d.i[2]]};
  sort_vtx(ck, 3);
  sort_vtx(dk, 3);
  for (int k = 0; k < 3; ++k) {
    if (vtx_less(ck[k], dk[k])) return true;
    if (vtx_less(dk[k], ck[k])) return false;
  }
  return false;
}

// ccd.rs:1106-1183 for primitive shapes (no mesh faces to consider)
template <class R> Result<R> epa_fallback(const Shape<R>& A, const Shape<R>& B, const Face<R>* faces, int nf, R ext,
                                          R margin) {
  bool have = false;
  Vec3<R> bax;
  R bd = R(0);
  auto consider = [&](Vec3<R> axis) {
    if (axis.length_squared() <= degen2<R>()) return;
    axis = axis.normalize();
    for (int s = 0; s < 2; ++s) {
      const Vec3<R> ax = s ? -axis : axis;
      const R dist = support_pair(A, B, ax, ext).m.dot(ax);
      if (dist <= R(0) || (have && (dist > bd || (dist == bd && !lex_less(ax, bax))))) continue;
      have = true; bax = ax; bd = dist;
    }
  };
  for (int k = 0; k < nf; ++k) consider(faces[k].n);
  consider(B.p - A.p);
  consider(Vec3<R>(1, 0, 0)); consider(Vec3<R>(0, 1, 0)); consider(Vec3<R>(0, 0, 1));
  Result<R> r;
  if (!have) return r;
  const Vec3<R> sb = support(B, -bax);
  const R pen = bd * ext + margin;
  if (!(pen > R(0))) return r;
  r.hit = true;
  r.pos = sb + bax * (bd * ext * R(0.5));
  r.n = -bax;
  r.pen = pen;
  r.wa = support(A, bax);
  r.wb = sb;
  r.path = 3;
  return r;
}

// ccd.rs:1703-1911 with the mesh configuration (EPA support epsilon 1e-7,
// at most 128 EPA iterations).  `face_eps` is how far beyond a face a new
// support point must lie for EPA to remove that face: newt's 1e-4 (relative
// to the pair extent) by default.  With it EPA stops early on curved
// features (the support point lands within 1e-4 of the closest face but not
// within the 1e-7 convergence bound, so no face changes and the point
// repeats) and returns its shallowest-axis fallback; a smaller value lets
// EPA converge there.
template <class R> Result<R> convex_contact(const Shape<R>& A, const Shape<R>& B, R margin, R face_eps = R(1.0e-4)) {
  const R ext = std::max(extent(A), extent(B));
  Result<R> none;
  if (!(ext > R(0))) return none;
  const R gjk_eps = R(0), epa_eps = R(1.0e-7);
  const int max_epa = 128;
  Vec3<R> dir = B.p - A.p;
  if (dir.length_squared() == R(0)) dir = Vec3<R>(1, 0, 0);
  Simplex<R> s;
  s.p[0] = support_pair(A, B, dir, ext);
  s.n = 1;
  dir = -s.p[0].m;
  bool enclosed = false, separated = false;
  for (int it = 0; it < 32; ++it) {
    const Vtx<R> p = support_pair(A, B, dir, ext);
    if (p.m.dot(dir) <= gjk_eps) { separated = true; break; }
    s.p[s.n++] = p;
    if (simplex_step(s, dir)) { enclosed = true; break; }
  }
  if (!enclosed && separated) s = distance_gjk(A, B, s, ext);
  if (!enclosed || s.n != 4) return distance_contact(s, margin);
  static thread_local Vtx<R> v[128];
  static thread_local Face<R> faces[512], next[512];
  static thread_local int edges[1024][2];
  for (int k = 0; k < 4; ++k) v[k] = s.p[k];
  int nv = 4, nf = 0;
  const int init[4][3] = {{0, 1, 2}, {0, 3, 1}, {0, 2, 3}, {1, 3, 2}};
  for (auto& f : init)
    if (make_face(v, f[0], f[1], f[2], &faces[nf])) ++nf;
  if (nf == 0) return distance_contact(s, margin);
  Face<R> best = faces[0];
  const R tie = face_eps;
  bool converged = false;
  for (int it = 0; it < max_epa; ++it) {
    int bi = 0;
    for (int k = 0; k < nf; ++k)
      if (face_less(v, faces[k], faces[bi], tie)) bi = k;
    best = faces[bi];
    const Vtx<R> sp = support_pair(A, B, best.n, ext);
    if (sp.m.dot(best.n) - best.d <= epa_eps) { converged = true; break; }
    if (nv == 128) break;
    bool dup = false;
    for (int k = 0; k < nv; ++k)
      if ((v[k].m - sp.m).length_squared() <= degen2<R>()) { dup = true; break; }
    if (dup) break;
    v[nv] = sp;
    const int nw = nv++;
    int nn = 0, ne = 0;
    for (int k = 0; k < nf; ++k) {
      const Face<R>& f = faces[k];
      if (f.n.dot(sp.m) > f.d + tie) {
        const int es[3][2] = {{f.i[0], f.i[1]}, {f.i[1], f.i[2]}, {f.i[2], f.i[0]}};
        for (auto& e : es) {
          int found = -1;
          for (int q = 0; q < ne; ++q)
            if (edges[q][0] == e[1] && edges[q][1] == e[0]) { found = q; break; }
          if (found >= 0) { edges[found][0] = edges[ne - 1][0]; edges[found][1] = edges[ne - 1][1]; --ne; }
          else { edges[ne][0] = e[0]; edges[ne][1] = e[1]; ++ne; }
        }
      } else {
        next[nn++] = f;
      }
    }
    for (int q = 0; q < ne; ++q) {
      if (nn == 512) break;
      if (make_face(v, edges[q][0], edges[q][1], nw, &next[nn])) ++nn;
    }
    for (int k = 0; k < nn; ++k) faces[k] = next[k];
    nf = nn;
    if (nf == 0) return none;
  }
  if (!converged) return epa_fallback(A, B, faces, nf, ext, margin);
  const Vec3<R> nearest = best.n * best.d;
  R w[3];
  barycentric(v[best.i[0]].m, v[best.i[1]].m, v[best.i[2]].m, nearest, w);
  const R sum = w[0] + w[1] + w[2];
  if (sum <= R(1.0e-8)) return none;
  for (R& x : w) x /= sum;
  const Vtx<R> f3[3] = {v[best.i[0]], v[best.i[1]], v[best.i[2]]};
  Vec3<R> pa, pb;
  mix(f3, w, 3, &pa, &pb);
  const R pen = best.d * ext + margin;
  if (pen <= R(0)) return none;
  Result<R> r;
  r.hit = true;
  r.n = -best.n;
  r.pos = (pa + pb) * R(0.5);
  r.pen = pen;
  r.wa = pa;
  r.wb = pb;
  r.path = 2;
  return r;
}

}  // namespace ccd
}  // namespace oracle
