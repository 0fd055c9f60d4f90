// GJK/EPA convex contact of two primitive shapes (sphere, box, capsule), in
// FP32 on the device: newt's general convex route, the one it runs for mesh
// pairs and height-field prisms.  The step's own narrowphase keeps the closed
// forms (narrowphase.cuh); this routine is the second formulation they are
// checked against (newt_gpu_convex_contacts).
//
// Restates newt/src/contact/ccd.rs:
//   :68-170     support of sphere, box, capsule; shape extent
//   :322-344    vertex precedence (deterministic ties)
//   :360-388    Minkowski supports scaled by the pair extent; triple product
//   :442-546    ccd_simplex_step (intersection GJK)
//   :658-694    ccd_closest_witness
//   :704-868    distance candidates and ccd_distance_simplex_step
//   :870-978    ccd_distance_contact, ccd_distance_gjk
//   :1036-1092  ccd_face, ccd_face_precedes
//   :1106-1183  ccd_epa_fallback_contact
//   :1703-1911  ccd_convex_contact (EPA over at most 128 vertices, 512 faces)
// and newt/src/contact.rs:64-78, :2265-2318, ccd.rs:2094-2109.
//
// One thread runs one pair; the EPA polytope (vertices, faces, horizon edges,
// about 25 KB) lives in the shared memory the caller hands it.  Face
// selection scans the faces in order with newt's tolerance comparison (it is
// not transitive, so a reduction tree could pick a different face).
#pragma once
#include "common.cuh"

namespace ccd {

constexpr int SPHERE = 1, BOX = 2, CAPSULE = 3;
constexpr int MAX_V = 128, MAX_F = 512, MAX_E = 1024;
constexpr float DEGEN2 = 1.0e-24f;  // (1e-12)^2

struct Shape { int kind; V3 p; Q4 q; V3 size; };  // sphere r | box half extents | capsule r, half height
struct Vtx { V3 m, a, b; };
struct Face { int i0, i1, i2; float nx, ny, nz, d; int pad; };
struct Polytope { Vtx v[MAX_V]; Face f[MAX_F]; short2 e[MAX_E]; };
struct Result { int hit, path; V3 pos, n, wa, wb; float pen; };

NEWT_D float clamp01(float x) { return x < 0.f ? 0.f : (x > 1.f ? 1.f : x); }
NEWT_D V3 normalize(V3 v) {
  const float l = sqrtf(len2(v));
  return l == 0.f ? v3(0.f, 0.f, 0.f) : v3(v.x / l, v.y / l, v.z / l);
}
NEWT_D bool lex_less(V3 a, V3 b) {
  if (a.x != b.x) return a.x < b.x;
  if (a.y != b.y) return a.y < b.y;
  return a.z < b.z;
}
NEWT_D bool same(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
NEWT_D bool vtx_less(const Vtx& a, const Vtx& b) {
  if (!same(a.m, b.m)) return lex_less(a.m, b.m);
  if (!same(a.a, b.a)) return lex_less(a.a, b.a);
  if (!same(a.b, b.b)) return lex_less(a.b, b.b);
  return false;
}
NEWT_D void sort_vtx(Vtx* v, int n) {
  for (int i = 1; i < n; ++i)
    for (int k = i; k > 0 && vtx_less(v[k], v[k - 1]); --k) { const Vtx t = v[k]; v[k] = v[k - 1]; v[k - 1] = t; }
}

NEWT_D float extent(const Shape& s) {
  if (s.kind == SPHERE) return s.size.x * 2.f;
  if (s.kind == BOX) return sqrtf(len2(s.size * 2.f));
  return 2.f * (s.size.y + s.size.x);
}

NEWT_D V3 support(const Shape& s, V3 d) {
  if (!(len2(d) > 1.0e-20f)) d = v3(1.f, 0.f, 0.f);
  if (s.kind == SPHERE) return s.p + normalize(d) * s.size.x;
  if (s.kind == BOX) {
    const V3 l = qrot_inv(s.q, d);
    const V3 c = v3(l.x >= 0.f ? s.size.x : -s.size.x, l.y >= 0.f ? s.size.y : -s.size.y,
                    l.z >= 0.f ? s.size.z : -s.size.z);
    return s.p + qrot(s.q, c);
  }
  const V3 ax = qrot(s.q, v3(0.f, 0.f, 1.f));
  const V3 end = dot(d, ax) >= 0.f ? s.p + ax * s.size.y : s.p - ax * s.size.y;
  return end + normalize(d) * s.size.x;
}

NEWT_D Vtx support_pair(const Shape& A, const Shape& B, V3 d, float ext) {
  if (!(len2(d) > DEGEN2)) d = v3(1.f, 0.f, 0.f);
  Vtx v;
  v.a = support(A, d);
  v.b = support(B, -d);
  v.m = (v.a - v.b) / ext;
  return v;
}

NEWT_D V3 triple(V3 a, V3 b, V3 c) { return b * dot(a, c) - a * dot(b, c); }

// intersection GJK step; newest point last; true when the origin is enclosed
NEWT_D bool simplex_step(Vtx* s, int& n, V3& dir) {
  const Vtx a = s[n - 1];
  const V3 ao = -a.m;
  if (n == 2) {
    const Vtx b = s[0];
    const V3 ab = b.m - a.m;
    if (dot(ab, ao) > 0.f) {
      dir = triple(ab, ao, ab);
      if (len2(dir) <= DEGEN2) dir = v3(0.f, 0.f, 1.f);
    } else {
      s[0] = a; n = 1;
      dir = ao;
    }
  } else if (n == 3) {
    const Vtx b = s[1], c = s[0];
    const V3 ab = b.m - a.m, ac = c.m - a.m, abc = cross(ab, ac);
    if (len2(abc) <= DEGEN2) {
      s[0] = a; s[1] = b; n = 2;
      const float el = len2(ab);
      const float t = el > DEGEN2 ? clamp01(-dot(a.m, ab) / el) : 0.f;
      const V3 cl = a.m + ab * t;
      if (len2(cl) > DEGEN2) { dir = -cl; return false; }
      V3 axis;
      if (fabsf(ab.x) <= fabsf(ab.y) && fabsf(ab.x) <= fabsf(ab.z)) axis = v3(1.f, 0.f, 0.f);
      else if (fabsf(ab.y) <= fabsf(ab.z)) axis = v3(0.f, 1.f, 0.f);
      else axis = v3(0.f, 0.f, 1.f);
      dir = cross(ab, axis);
      if (len2(dir) <= DEGEN2) dir = ao;
      return false;
    }
    if (dot(cross(abc, ac), ao) > 0.f) {
      if (dot(ac, ao) > 0.f) { s[0] = a; s[1] = c; n = 2; dir = triple(ac, ao, ac); }
      else if (dot(ab, ao) > 0.f) { s[0] = a; s[1] = b; n = 2; dir = triple(ab, ao, ab); }
      else { s[0] = a; n = 1; dir = ao; }
    } else if (dot(cross(ab, abc), ao) > 0.f) {
      if (dot(ab, ao) > 0.f) { s[0] = a; s[1] = b; n = 2; dir = triple(ab, ao, ab); }
      else { s[0] = a; n = 1; dir = ao; }
    } else if (dot(abc, ao) > 0.f) {
      dir = abc;
    } else {
      s[0] = a; s[1] = c; s[2] = b; n = 3;
      dir = -abc;
    }
  } else {
    const Vtx b = s[2], c = s[1], d = s[0];
    const V3 ab = b.m - a.m, ac = c.m - a.m, ad = d.m - a.m;
    const V3 abc = cross(ab, ac), acd = cross(ac, ad), adb = cross(ad, ab);
    if (dot(abc, ao) > 0.f) { s[0] = a; s[1] = c; s[2] = b; n = 3; dir = abc; }
    else if (dot(acd, ao) > 0.f) { s[0] = a; s[1] = d; s[2] = c; n = 3; dir = acd; }
    else if (dot(adb, ao) > 0.f) { s[0] = a; s[1] = b; s[2] = d; n = 3; dir = adb; }
    else return true;
  }
  if (len2(dir) <= DEGEN2) dir = v3(1.f, 0.f, 0.f);
  return false;
}

NEWT_D V3 closest_on_triangle(V3 p, V3 a, V3 b, V3 c) {
  const V3 ab = b - a, ac = c - a, ap = p - a;
  const float d1 = dot(ab, ap), d2 = dot(ac, ap);
  if (d1 <= 0.f && d2 <= 0.f) return a;
  const V3 bp = p - b;
  const float d3 = dot(ab, bp), d4 = dot(ac, bp);
  if (d3 >= 0.f && d4 <= d3) return b;
  const float vc = d1 * d4 - d3 * d2;
  if (vc <= 0.f && d1 >= 0.f && d3 <= 0.f) return a + ab * (d1 / (d1 - d3));
  const V3 cp = p - c;
  const float d5 = dot(ab, cp), d6 = dot(ac, cp);
  if (d6 >= 0.f && d5 <= d6) return c;
  const float vb = d5 * d2 - d1 * d6;
  if (vb <= 0.f && d2 >= 0.f && d6 <= 0.f) return a + ac * (d2 / (d2 - d6));
  const float va = d3 * d6 - d5 * d4;
  if (va <= 0.f && (d4 - d3) >= 0.f && (d5 - d6) >= 0.f) return b + (c - b) * ((d4 - d3) / ((d4 - d3) + (d5 - d6)));
  const float den = 1.f / (va + vb + vc);
  return a + ab * (vb * den) + ac * (vc * den);
}

NEWT_D void barycentric(V3 a, V3 b, V3 c, V3 p, float w[3]) {
  const V3 v0 = b - a, v1 = c - a, v2 = p - a;
  const float d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1), d20 = dot(v2, v0), d21 = dot(v2, v1);
  const float den = d00 * d11 - d01 * d01;
  if (fabsf(den) <= 1.0e-12f) { w[0] = 1.f; w[1] = w[2] = 0.f; return; }
  const float v = (d11 * d20 - d01 * d21) / den, ww = (d00 * d21 - d01 * d20) / den;
  w[0] = 1.f - v - ww; w[1] = v; w[2] = ww;
}

NEWT_D void mix(const Vtx* v, const float* w, int n, V3* pa, V3* pb) {
  *pa = v3(0.f, 0.f, 0.f);
  *pb = v3(0.f, 0.f, 0.f);
  for (int k = 0; k < n; ++k) { *pa = *pa + v[k].a * w[k]; *pb = *pb + v[k].b * w[k]; }
}

NEWT_D void triangle_witness(const Vtx& a, const Vtx& b, const Vtx& c, V3* pa, V3* pb) {
  const V3 nearest = closest_on_triangle(v3(0.f, 0.f, 0.f), a.m, b.m, c.m);
  float w[3];
  barycentric(a.m, b.m, c.m, nearest, w);
  const Vtx t[3] = {a, b, c};
  mix(t, w, 3, pa, pb);
}

NEWT_D bool closest_witness(const Vtx* s, int n, V3* pa, V3* pb) {
  if (n == 1) { *pa = s[0].a; *pb = s[0].b; return true; }
  if (n == 2) {
    const V3 e = s[1].m - s[0].m;
    const float den = len2(e);
    const float t = den > DEGEN2 ? clamp01(-dot(s[0].m, e) / den) : 0.f;
    const float w[2] = {1.f - t, t};
    mix(s, w, 2, pa, pb);
    return true;
  }
  if (n == 3) { triangle_witness(s[0], s[1], s[2], pa, pb); return true; }
  if (n == 4) {
    const int faces[4][3] = {{0, 1, 2}, {0, 3, 1}, {0, 2, 3}, {1, 3, 2}};
    float best = 0.f;
    for (int k = 0; k < 4; ++k) {
      V3 a, b;
      triangle_witness(s[faces[k][0]], s[faces[k][1]], s[faces[k][2]], &a, &b);
      const float d2 = len2(a - b);
      if (k == 0 || d2 < best) { best = d2; *pa = a; *pb = b; }
    }
    return true;
  }
  return false;
}

struct Cand { V3 pt; float w[4]; Vtx f[3]; int fn; };

NEWT_D bool candidate(const Vtx* s, int n, int mask, Cand* out) {
  int idx[3], k = 0;
  for (int i = 0; i < n; ++i)
    if (mask & (1 << i)) { if (k == 3) return false; idx[k++] = i; }
  for (int i = 1; i < k; ++i)
    for (int p = i; p > 0 && vtx_less(s[idx[p]], s[idx[p - 1]]); --p) { const int t = idx[p]; idx[p] = idx[p - 1]; idx[p - 1] = t; }
  float sw[3] = {1.f, 0.f, 0.f};
  V3 pt;
  if (k == 1) pt = s[idx[0]].m;
  else if (k == 2) {
    const V3 a = s[idx[0]].m, e = s[idx[1]].m - a;
    const float den = len2(e);
    const float t = den > DEGEN2 ? clamp01(-dot(a, e) / den) : 0.f;
    pt = a + e * t; sw[0] = 1.f - t; sw[1] = t;
  } else {
    const V3 a = s[idx[0]].m, b = s[idx[1]].m, c = s[idx[2]].m;
    if (len2(cross(b - a, c - a)) <= DEGEN2) return false;
    pt = closest_on_triangle(v3(0.f, 0.f, 0.f), a, b, c);
    barycentric(a, b, c, pt, sw);
  }
  out->pt = pt;
  for (int i = 0; i < 4; ++i) out->w[i] = 0.f;
  for (int i = 0; i < k; ++i) out->w[idx[i]] = sw[i];
  for (int i = 0; i < 3; ++i) out->f[i] = s[idx[0]];
  for (int i = 0; i < k; ++i) out->f[i] = s[idx[i]];
  out->fn = k;
  return true;
}

NEWT_D bool cand_less(const Cand& c, const Cand& d) {
  const float cd = len2(c.pt), dd = len2(d.pt);
  if (cd != dd) return cd < dd;
  if (c.fn != d.fn) return c.fn < d.fn;
  for (int i = 0; i < c.fn; ++i) {
    if (vtx_less(c.f[i], d.f[i])) return true;
    if (vtx_less(d.f[i], c.f[i])) return false;
  }
  return lex_less(c.pt, d.pt);
}

NEWT_D bool origin_in_tetra(const Vtx* s) {
  const V3 a = s[0].m, ab = s[1].m - a, ac = s[2].m - a, ad = s[3].m - a;
  const float den = dot(cross(ab, ac), ad);
  if (fabsf(den) <= DEGEN2) return false;
  const V3 ao = -a;
  const float wb = dot(cross(ao, ac), ad) / den, wc = dot(cross(ab, ao), ad) / den, wd = dot(cross(ab, ac), ao) / den;
  const float w[4] = {1.f - wb - wc - wd, wb, wc, wd};
  for (int k = 0; k < 4; ++k)
    if (!(w[k] >= -1.0e-6f && w[k] <= 1.f + 1.0e-6f)) return false;
  return true;
}

NEWT_D bool distance_step(Vtx* s, int& n, V3* closest) {
  if (n == 4 && origin_in_tetra(s)) return false;
  Cand best, c;
  bool have = false;
  for (int mask = 1; mask < (1 << n); ++mask) {
    if (!candidate(s, n, mask, &c)) continue;
    if (!have || cand_less(c, best)) { best = c; have = true; }
  }
  if (!have) return false;
  Vtx sel[4];
  int k = 0;
  for (int i = 0; i < n; ++i)
    if (best.w[i] > 1.0e-6f) sel[k++] = s[i];
  if (k == 0) {
    int li = 0;
    for (int i = 1; i < n; ++i) {
      const float dw = best.w[i] - best.w[li];
      if (dw > 1.0e-6f || (fabsf(dw) <= 1.0e-6f && vtx_less(s[i], s[li]))) li = i;
    }
    sel[0] = s[li];
    k = 1;
  }
  sort_vtx(sel, k);
  for (int i = 0; i < k; ++i) s[i] = sel[i];
  n = k;
  *closest = best.pt;
  return true;
}

// distance GJK (ccd.rs:910-978; support epsilon 0, tolerance 1e-10)
NEWT_D void distance_gjk(const Shape& A, const Shape& B, Vtx* s, int& n, float ext) {
  Vtx best_s[4];
  int best_n = n;
  for (int i = 0; i < n; ++i) best_s[i] = s[i];
  float best = INFINITY;
  auto keep = [&]() { best_n = n; for (int i = 0; i < n; ++i) best_s[i] = s[i]; };
  for (int it = 0; it < 64; ++it) {
    V3 cl;
    if (!distance_step(s, n, &cl)) break;
    const float d2 = len2(cl);
    if (d2 < best) { best = d2; keep(); }
    if (d2 <= DEGEN2) break;
    const V3 dir = -cl;
    const Vtx p = support_pair(A, B, dir, ext);
    if (dot(p.m, dir) - dot(cl, dir) <= 0.f) break;
    bool dup = false;
    for (int i = 0; i < n; ++i) dup |= len2(s[i].m - p.m) <= DEGEN2;
    if (dup) break;
    s[n++] = p;
    V3 nc;
    if (!distance_step(s, n, &nc)) break;
    const float n2 = len2(nc);
    if (n2 < best) { best = n2; keep(); }
    if (d2 - n2 <= 1.0e-10f * (d2 > DEGEN2 ? d2 : DEGEN2)) break;
  }
  n = best_n;
  for (int i = 0; i < n; ++i) s[i] = best_s[i];
}

NEWT_D Result distance_contact(const Vtx* s, int n, float margin) {
  Result r{};
  V3 pa, pb;
  if (!closest_witness(s, n, &pa, &pb)) return r;
  const V3 sep = pa - pb;
  const float dist = sqrtf(len2(sep));
  const float pen = margin - dist;
  if (pen <= 0.f) return r;
  r.hit = 1; r.path = 1;
  r.wa = pa; r.wb = pb;
  r.n = dist > 0.f ? sep / dist : v3(1.f, 0.f, 0.f);
  r.pos = (pa + pb) * 0.5f;
  r.pen = pen;
  return r;
}

NEWT_D bool make_face(const Vtx* v, int a, int b, int c, Face* f) {
  const V3 raw = cross(v[b].m - v[a].m, v[c].m - v[a].m);
  if (len2(raw) <= DEGEN2) return false;
  V3 n = normalize(raw);
  float d = dot(n, v[a].m);
  f->i0 = a; f->i1 = b; f->i2 = c;
  if (d < 0.f) { f->i1 = c; f->i2 = b; n = -n; d = -d; }
  f->nx = n.x; f->ny = n.y; f->nz = n.z; f->d = d;
  return true;
}

NEWT_D bool face_less(const Vtx* v, const Face& c, const Face& d, float tie) {
  if (c.d + tie < d.d) return true;
  if (d.d + tie < c.d) return false;
  Vtx ck[3] = {v[c.i0], v[c.i1], v[c.i2]}, dk[3] = {v[d.i0], v[d.i1], v[d.i2]};
  sort_vtx(ck, 3);
  sort_vtx(dk, 3);
  for (int k = 0; k < 3; ++k) {
    if (vtx_less(ck[k], dk[k])) return true;
    if (vtx_less(dk[k], ck[k])) return false;
  }
  return false;
}

NEWT_D V3 fnorm(const Face& f) { return v3(f.nx, f.ny, f.nz); }

NEWT_D Result epa_fallback(const Shape& A, const Shape& B, const Face* faces, int nf, float ext, float margin) {
  bool have = false;
  V3 bax = v3(0.f, 0.f, 0.f);
  float bd = 0.f;
  auto consider = [&](V3 axis) {
    if (len2(axis) <= DEGEN2) return;
    axis = normalize(axis);
    for (int s = 0; s < 2; ++s) {
      const V3 ax = s ? -axis : axis;
      const float dist = dot(support_pair(A, B, ax, ext).m, ax);
      if (dist <= 0.f || (have && (dist > bd || (dist == bd && !lex_less(ax, bax))))) continue;
      have = true; bax = ax; bd = dist;
    }
  };
  for (int k = 0; k < nf; ++k) consider(fnorm(faces[k]));
  consider(B.p - A.p);
  consider(v3(1.f, 0.f, 0.f)); consider(v3(0.f, 1.f, 0.f)); consider(v3(0.f, 0.f, 1.f));
  Result r{};
  if (!have) return r;
  const V3 sb = support(B, -bax);
  const float pen = bd * ext + margin;
  if (!(pen > 0.f)) return r;
  r.hit = 1; r.path = 3;
  r.pos = sb + bax * (bd * ext * 0.5f);
  r.n = -bax;
  r.pen = pen;
  r.wa = support(A, bax);
  r.wb = sb;
  return r;
}

// ccd.rs:1703-1911 with the mesh configuration (EPA support epsilon 1e-7,
// at most 128 EPA iterations); `face_eps` is EPA's face-removal threshold
// (newt: 1e-4 of the pair extent).  `P` is the caller's shared polytope.
NEWT_D Result convex_contact(const Shape& A, const Shape& B, float margin, float face_eps, Polytope* P) {
  Result none{};
  const float ext = fmaxf(extent(A), extent(B));
  if (!(ext > 0.f)) return none;
  V3 dir = B.p - A.p;
  if (len2(dir) == 0.f) dir = v3(1.f, 0.f, 0.f);
  Vtx s[4];
  int n = 1;
  s[0] = support_pair(A, B, dir, ext);
  dir = -s[0].m;
  bool enclosed = false, separated = false;
  for (int it = 0; it < 32; ++it) {
    const Vtx p = support_pair(A, B, dir, ext);
    if (dot(p.m, dir) <= 0.f) { separated = true; break; }
    s[n++] = p;
    if (simplex_step(s, n, dir)) { enclosed = true; break; }
  }
  if (!enclosed && separated) distance_gjk(A, B, s, n, ext);
  if (!enclosed || n != 4) return distance_contact(s, n, margin);
  Vtx* v = P->v;
  Face* faces = P->f;
  short2* edges = P->e;
  for (int k = 0; k < 4; ++k) v[k] = s[k];
  int nv = 4, nf = 0;
  const int init[4][3] = {{0, 1, 2}, {0, 3, 1}, {0, 2, 3}, {1, 3, 2}};
  for (int k = 0; k < 4; ++k)
    if (make_face(v, init[k][0], init[k][1], init[k][2], &faces[nf])) ++nf;
  if (nf == 0) return distance_contact(s, n, margin);
  Face best = faces[0];
  bool converged = false;
  for (int it = 0; it < 128; ++it) {
    int bi = 0;
    for (int k = 0; k < nf; ++k)
      if (face_less(v, faces[k], faces[bi], face_eps)) bi = k;
    best = faces[bi];
    const Vtx sp = support_pair(A, B, fnorm(best), ext);
    if (dot(sp.m, fnorm(best)) - best.d <= 1.0e-7f) { converged = true; break; }
    if (nv == MAX_V) break;
    bool dup = false;
    for (int k = 0; k < nv; ++k) dup |= len2(v[k].m - sp.m) <= DEGEN2;
    if (dup) break;
    v[nv] = sp;
    const int nw = nv++;
    // faces the new point sees leave (the rest keep their order); the
    // horizon is every edge of a leaving face whose reverse is not also one
    int nn = 0, ne = 0;
    for (int k = 0; k < nf; ++k) {
      const Face f = faces[k];
      if (dot(fnorm(f), sp.m) > f.d + face_eps) {
        const int es[3][2] = {{f.i0, f.i1}, {f.i1, f.i2}, {f.i2, f.i0}};
        for (int q = 0; q < 3; ++q) {
          int found = -1;
          for (int r = 0; r < ne; ++r)
            if (edges[r].x == es[q][1] && edges[r].y == es[q][0]) { found = r; break; }
          if (found >= 0) { edges[found] = edges[ne - 1]; --ne; }
          else if (ne < MAX_E) { edges[ne] = make_short2((short)es[q][0], (short)es[q][1]); ++ne; }
        }
      } else {
        faces[nn++] = f;
      }
    }
    for (int r = 0; r < ne && nn < MAX_F; ++r)
      if (make_face(v, edges[r].x, edges[r].y, nw, &faces[nn])) ++nn;
    nf = nn;
    if (nf == 0) return none;
  }
  if (!converged) return epa_fallback(A, B, faces, nf, ext, margin);
  const V3 bn = fnorm(best);
  const V3 nearest = bn * best.d;
  float w[3];
  barycentric(v[best.i0].m, v[best.i1].m, v[best.i2].m, nearest, w);
  const float sum = w[0] + w[1] + w[2];
  if (sum <= 1.0e-8f) return none;
  for (int k = 0; k < 3; ++k) w[k] /= sum;
  const Vtx f3[3] = {v[best.i0], v[best.i1], v[best.i2]};
  V3 pa, pb;
  mix(f3, w, 3, &pa, &pb);
  const float pen = best.d * ext + margin;
  if (pen <= 0.f) return none;
  Result r{};
  r.hit = 1; r.path = 2;
  r.n = -bn;
  r.pos = (pa + pb) * 0.5f;
  r.pen = pen;
  r.wa = pa;
  r.wb = pb;
  return r;
}

}  // namespace ccd
