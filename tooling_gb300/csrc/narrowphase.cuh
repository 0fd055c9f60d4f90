// Narrowphase primitives for the GPU contact pipeline (FP32, one pair per
// lane).  Contact conventions follow newt (newt/src/contact.rs:82-106): the
// normal points FROM geom B INTO geom A, `pen` = margin - raw distance, plane
// contacts sit at the MuJoCo midpoint, sphere contacts on B's surface.
//
//   sphere_plane   newt/src/contact.rs:269-301
//   box_plane      newt/src/contact.rs:311-362  (corners in bit order, first 4)
//   sphere_sphere  newt/src/contact.rs:407-470
//   box_box        newt/src/contact.rs:569-1053 (15-axis SAT, face clipping,
//                  edge-edge closest points)
//   capsule_plane  newt/src/contact.rs:367-400
//   sphere_capsule newt/src/contact.rs:473-505
//   capsule_capsule newt/src/contact.rs:1249-1272
//   cylinder_plane newt/src/contact.rs:1296-1373
//   sphere_cylinder newt/src/contact.rs:1519-1628
//   ellipsoid_plane newt/src/contact.rs:1381-1426
//   sphere_ellipsoid newt/src/contact.rs:1630-1725
//   sphere_box     extension (newt defers this pair, contact.rs:236-257):
//                  closed-form closest point on the oriented box
#pragma once
#include "common.cuh"

struct GPose { V3 p; Q4 q; };
struct CRes { V3 pos, n; float pen; };

NEWT_D V3 gx_axis(const GPose& g, int k) {
  return qrot(g.q, v3(k == 0 ? 1.f : 0.f, k == 1 ? 1.f : 0.f, k == 2 ? 1.f : 0.f));
}

NEWT_D int np_sphere_plane(const GPose& s, float r, float margin, const GPose& pl, CRes* out) {
  V3 n = qrot(pl.q, v3(0.f, 0.f, 1.f));
  float raw = dot(s.p - pl.p, n) - r;
  if (raw <= margin) {
    out[0] = CRes{s.p - n * (r + raw * 0.5f), n, margin - raw};
    return 1;
  }
  return 0;
}

NEWT_D int np_box_plane(const GPose& b, V3 h, float margin, const GPose& pl, CRes* out) {
  V3 n = qrot(pl.q, v3(0.f, 0.f, 1.f));
  float dist = dot(b.p - pl.p, n);
  int cnt = 0;
  for (int i = 0; i < 8; ++i) {
    V3 local = v3((i & 1) ? h.x : -h.x, (i & 2) ? h.y : -h.y, (i & 4) ? h.z : -h.z);
    V3 off = qrot(b.q, local);
    float ldist = dot(n, off);
    float raw = dist + ldist;
    if (raw > margin || ldist > 0.f) continue;
    if (cnt < 4) out[cnt] = CRes{(b.p + off) - n * (raw * 0.5f), n, margin - raw};
    ++cnt;
  }
  return cnt < 4 ? cnt : 4;
}

NEWT_D int np_sphere_sphere(V3 ca, float ra, V3 cb, float rb, float margin, CRes* out) {
  V3 d = ca - cb;
  float d2 = len2(d);
  float srm = (ra + rb) + margin;
  if (d2 >= srm * srm) return 0;
  float dist = sqrtf(d2);
  V3 n = dist > 0.f ? d * (1.f / dist) : v3(0.f, 0.f, 1.f);
  out[0] = CRes{cb + n * rb, n, srm - dist};
  return 1;
}

// Sphere (A) vs box (B).
NEWT_D int np_sphere_box(const GPose& s, float r, const GPose& b, V3 h, float margin, CRes* out) {
  V3 l = qrot_inv(b.q, s.p - b.p);
  float lc[3] = {l.x, l.y, l.z}, hl[3] = {h.x, h.y, h.z}, cl[3];
  bool inside = true;
  for (int k = 0; k < 3; ++k) {
    float v = lc[k];
    if (v > hl[k]) { v = hl[k]; inside = false; }
    else if (v < -hl[k]) { v = -hl[k]; inside = false; }
    cl[k] = v;
  }
  if (!inside) {
    V3 dl = v3(lc[0] - cl[0], lc[1] - cl[1], lc[2] - cl[2]);
    float d2 = len2(dl), rm = r + margin;
    if (d2 >= rm * rm) return 0;
    float dist = sqrtf(d2);
    V3 nl = dist > 0.f ? dl * (1.f / dist) : v3(0.f, 0.f, 1.f);
    out[0] = CRes{b.p + qrot(b.q, v3(cl[0], cl[1], cl[2])), qrot(b.q, nl), rm - dist};
    return 1;
  }
  int best = 0;
  float bd = hl[0] - fabsf(lc[0]);
  for (int k = 1; k < 3; ++k) { float dd = hl[k] - fabsf(lc[k]); if (dd < bd) { bd = dd; best = k; } }
  float sg = lc[best] >= 0.f ? 1.f : -1.f;
  float nl[3] = {0.f, 0.f, 0.f}, fc[3] = {lc[0], lc[1], lc[2]};
  nl[best] = sg; fc[best] = sg * hl[best];
  out[0] = CRes{b.p + qrot(b.q, v3(fc[0], fc[1], fc[2])), qrot(b.q, v3(nl[0], nl[1], nl[2])), (r + margin) + bd};
  return 1;
}

NEWT_D float clamp01f(float x) { return x < 0.f ? 0.f : (x > 1.f ? 1.f : x); }

NEWT_D void seg_closest(V3 a0, V3 a1, V3 b0, V3 b1, V3* pa, V3* pb) {  // contact.rs:2342-2387
  V3 d1 = a1 - a0, d2 = b1 - b0, r = a0 - b0;
  float a = len2(d1), e = len2(d2), f = dot(d2, r);
  const float EPS = 1.0e-12f;
  if (a <= EPS && e <= EPS) { *pa = a0; *pb = b0; return; }
  if (a <= EPS) { *pa = a0; *pb = b0 + d2 * clamp01f(f / e); return; }
  float c = dot(d1, r);
  if (e <= EPS) { *pa = a0 + d1 * clamp01f(-c / a); *pb = b0; return; }
  float b_ = dot(d1, d2), denom = a * e - b_ * b_;
  float s = denom != 0.f ? clamp01f((b_ * f - c * e) / denom) : 0.f;
  float tn = b_ * s + f, t, sf;
  if (tn < 0.f) { t = 0.f; sf = clamp01f(-c / a); }
  else if (tn > e) { t = 1.f; sf = clamp01f((b_ - c) / a); }
  else { t = tn / e; sf = s; }
  *pa = a0 + d1 * sf; *pb = b0 + d2 * t;
}

// Capsule (A, axis local z, segment -h..+h) vs plane (B): one contact per
// segment end within the margin (newt/src/contact.rs:367-400).
NEWT_D int np_capsule_plane(const GPose& c, float r, float hh, float margin, const GPose& pl, CRes* out) {
  const V3 n = qrot(pl.q, v3(0.f, 0.f, 1.f));
  const V3 ax = qrot(c.q, v3(0.f, 0.f, 1.f));
  int k = 0;
  for (int e = 0; e < 2; ++e) {
    const V3 p = e == 0 ? c.p + ax * hh : c.p - ax * hh;
    const float raw = dot(p - pl.p, n) - r;
    if (raw <= margin) out[k++] = CRes{p - n * (r + raw * 0.5f), n, margin - raw};
  }
  return k;
}

// Sphere (A) vs capsule (B): the sphere against the sphere at the axis point
// closest to its centre (contact.rs:473-505, closest_point_on_segment
// contact.rs:2313-2321).
NEWT_D int np_sphere_capsule(V3 cs, float rs, const GPose& c, float rc, float hh, float margin, CRes* out) {
  const V3 ax = qrot(c.q, v3(0.f, 0.f, 1.f));
  const V3 a = c.p - ax * hh, ab = (c.p + ax * hh) - a;
  const float den = len2(ab);
  const V3 q = den == 0.f ? a : a + ab * clamp01f(dot(cs - a, ab) / den);
  return np_sphere_sphere(cs, rs, q, rc, margin, out);
}

// Capsule (A) vs capsule (B): closest points of the two axis segments, then
// sphere vs sphere there (contact.rs:1249-1272).
NEWT_D int np_capsule_capsule(const GPose& A, float ra, float ha, const GPose& B, float rb, float hb, float margin,
                              CRes* out) {
  const V3 ax = qrot(A.q, v3(0.f, 0.f, 1.f)), bx = qrot(B.q, v3(0.f, 0.f, 1.f));
  V3 pa, pb;
  seg_closest(A.p - ax * ha, A.p + ax * ha, B.p - bx * hb, B.p + bx * hb, &pa, &pb);
  return np_sphere_sphere(pa, ra, pb, rb, margin, out);
}

// Cylinder (A, axis local z) vs plane (B): 18 samples (the two cap centres,
// then top and bottom rim points at 0, 45, ..., 315 degrees, interleaved),
// the up to four deepest with penetration > 0, deepest first with ties in
// sample order, each projected onto the plane (contact.rs:1296-1373).
NEWT_D int np_cylinder_plane(const GPose& c, float r, float hh, float margin, const GPose& pl, CRes* out) {
  const V3 n = qrot(pl.q, v3(0.f, 0.f, 1.f));
  const V3 ax = qrot(c.q, v3(0.f, 0.f, 1.f)), xl = qrot(c.q, v3(1.f, 0.f, 0.f)), yl = qrot(c.q, v3(0.f, 1.f, 0.f));
  const V3 top = c.p + ax * hh, bot = c.p - ax * hh;
  const float s = 0.70710677f;
  float best_pen[4];
  int best_i[4], nb = 0;
  for (int i = 0; i < 18; ++i) {
    V3 p;
    if (i < 2) {
      p = i == 0 ? top : bot;
    } else {
      const int k = (i - 2) >> 1;
      const float cx = (k == 0 || k == 1 || k == 7) ? 1.f : ((k == 3 || k == 4 || k == 5) ? -1.f : 0.f);
      const float cy = (k == 1 || k == 2 || k == 3) ? 1.f : ((k == 5 || k == 6 || k == 7) ? -1.f : 0.f);
      const V3 d = (k & 1) ? xl * (cx * s) + yl * (cy * s) : xl * cx + yl * cy;
      p = ((i - 2) & 1 ? bot : top) + d * r;
    }
    const float pen = margin - dot(p - pl.p, n);
    if (!(pen > 0.f)) continue;
    // keep the four deepest; a later sample displaces only a strictly shallower one
    int at = nb < 4 ? nb : 4;
    while (at > 0 && pen > best_pen[at - 1]) --at;
    if (at >= 4) continue;
    for (int j = (nb < 4 ? nb : 3); j > at; --j) { best_pen[j] = best_pen[j - 1]; best_i[j] = best_i[j - 1]; }
    best_pen[at] = pen;
    best_i[at] = i;
    if (nb < 4) ++nb;
  }
  for (int k = 0; k < nb; ++k) {
    const int i = best_i[k];
    V3 p;
    if (i < 2) {
      p = i == 0 ? top : bot;
    } else {
      const int q = (i - 2) >> 1;
      const float cx = (q == 0 || q == 1 || q == 7) ? 1.f : ((q == 3 || q == 4 || q == 5) ? -1.f : 0.f);
      const float cy = (q == 1 || q == 2 || q == 3) ? 1.f : ((q == 5 || q == 6 || q == 7) ? -1.f : 0.f);
      const V3 d = (q & 1) ? xl * (cx * s) + yl * (cy * s) : xl * cx + yl * cy;
      p = ((i - 2) & 1 ? bot : top) + d * r;
    }
    out[k] = CRes{p - n * (margin - best_pen[k]), n, best_pen[k]};
  }
  return nb;
}

// Ellipsoid (A, semi-axes e) vs plane (B): the support point along -n in the
// ellipsoid frame, (e.x^2 d.x, e.y^2 d.y, e.z^2 d.z) / |(e.x d.x, e.y d.y,
// e.z d.z)|; one contact when margin - distance >= 0 (contact.rs:1381-1426).
NEWT_D int np_ellipsoid_plane(const GPose& e, V3 ax, float margin, const GPose& pl, CRes* out) {
  const V3 n = qrot(pl.q, v3(0.f, 0.f, 1.f));
  const V3 d = qrot_inv(e.q, -n);
  const float dsq = (ax.x * d.x) * (ax.x * d.x) + (ax.y * d.y) * (ax.y * d.y) + (ax.z * d.z) * (ax.z * d.z);
  if (!(dsq > 0.f)) return 0;
  const float den = sqrtf(dsq);
  const V3 pl_ = v3(ax.x * ax.x * d.x, ax.y * ax.y * d.y, ax.z * ax.z * d.z) / den;
  const V3 sw = e.p + qrot(e.q, pl_);
  const float sg = dot(sw - pl.p, n);
  const float pen = margin - sg;
  if (!(pen >= 0.f)) return 0;
  out[0] = CRes{sw - n * (sg * 0.5f), n, pen};
  return 1;
}

// Sphere (A) vs cylinder (B): the closest point of the solid cylinder to the
// sphere centre in the cylinder frame; a centre inside leaves through the
// nearer of cap and side, the cap on ties (contact.rs:1519-1628).
NEWT_D int np_sphere_cylinder(V3 cs, float rs, const GPose& c, float rc, float hh, float margin, CRes* out) {
  const V3 pl = qrot_inv(c.q, cs - c.p);
  const float z = pl.z, dr = sqrtf(pl.x * pl.x + pl.y * pl.y);
  const bool inside = fabsf(z) <= hh && dr <= rc;
  const float ux = dr > 0.f ? pl.x / dr : 1.f, uy = dr > 0.f ? pl.y / dr : 0.f;
  V3 cl;
  if (inside) {
    cl = (hh - fabsf(z) <= rc - dr) ? v3(pl.x, pl.y, (z >= 0.f ? 1.f : -1.f) * hh) : v3(ux * rc, uy * rc, z);
  } else {
    const float zc = z > hh ? hh : (z < -hh ? -hh : z), rcl = dr > rc ? rc : dr;
    cl = v3(ux * rcl, uy * rcl, zc);
  }
  const V3 dl = pl - cl;
  const float dist = sqrtf(len2(dl));
  const float pen = (inside ? rs + dist : rs - dist) + margin;
  if (!(pen > 0.f)) return 0;
  const V3 nl = dist > 1.0e-9f ? (inside ? dl * (-1.f / dist) : dl * (1.f / dist)) : v3(0.f, 0.f, 1.f);
  out[0] = CRes{c.p + qrot(c.q, cl), qrot(c.q, nl), pen};
  return 1;
}

// Sphere (A) vs ellipsoid (B, semi-axes ax): the closest point q of the
// ellipsoid surface to the sphere centre p (ellipsoid frame) from twelve
// Newton steps from t = 0 on the Lagrange parameter t of
// q_k = ax_k^2 p_k / (ax_k^2 + t), f(t) = sum (ax_k p_k / (ax_k^2 + t))^2 - 1
// (a zero denominator nudges t and spends the step); normal (p - q) / |p - q|
// into the sphere, the contact point midway between q and the sphere's
// surface (contact.rs:1630-1725).
NEWT_D int np_sphere_ellipsoid(V3 cs, float rs, const GPose& e, V3 ax, float margin, CRes* out) {
  const V3 p = qrot_inv(e.q, cs - e.p);
  const float mx = ax.x > ax.y ? (ax.x > ax.z ? ax.x : ax.z) : (ax.y > ax.z ? ax.y : ax.z);
  if (sqrtf(len2(p)) > rs + margin + mx + 1.f) return 0;
  const float ap[3] = {ax.x * p.x, ax.y * p.y, ax.z * p.z};
  const float a2[3] = {ax.x * ax.x, ax.y * ax.y, ax.z * ax.z};
  float t = 0.f;
  for (int it = 0; it < 12; ++it) {
    float f = -1.f, fp = 0.f;
    bool nudged = false;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (nudged) continue;
      const float den = a2[k] + t;
      if (den == 0.f) { t += 1.0e-6f * (a2[k] + 1.f); nudged = true; continue; }
      const float inv = 1.f / den;
      const float num = ap[k] * inv;
      f += num * num;
      fp += -2.f * ap[k] * ap[k] * inv * inv * inv;
    }
    if (nudged) continue;
    if (fp == 0.f) break;
    t -= f / fp;
  }
  const V3 q = v3(a2[0] * p.x / (a2[0] + t), a2[1] * p.y / (a2[1] + t), a2[2] * p.z / (a2[2] + t));
  const V3 d = p - q;
  const float dist = sqrtf(len2(d));
  const float pen = rs - dist + margin;
  if (!(pen > 0.f)) return 0;
  const V3 nl = dist > 1.0e-9f ? d / dist : v3(0.f, 0.f, 1.f);
  const V3 nw = qrot(e.q, nl);
  out[0] = CRes{((e.p + qrot(e.q, q)) + (cs - nw * rs)) * 0.5f, nw, pen};
  return 1;
}

struct FV2 { float u, v, d; };

NEWT_D int np_box_box(const GPose& A, V3 half_a, const GPose& B, V3 half_b, float margin, CRes* out) {
  V3 ax[3] = {gx_axis(A, 0), gx_axis(A, 1), gx_axis(A, 2)};
  V3 bx[3] = {gx_axis(B, 0), gx_axis(B, 1), gx_axis(B, 2)};
  float ha[3] = {half_a.x, half_a.y, half_a.z}, hb[3] = {half_b.x, half_b.y, half_b.z};
  V3 delta = A.p - B.p;
  auto proj = [](V3 l, const V3* u, const float* h) {
    return h[0] * fabsf(dot(l, u[0])) + h[1] * fabsf(dot(l, u[1])) + h[2] * fabsf(dot(l, u[2]));
  };
  float best = INFINITY;
  V3 bax = v3(0.f, 0.f, 1.f);
  int kind = 0, k1 = 0, k2 = 0;
  for (int k = 0; k < 3; ++k) {
    V3 f = ax[k];
    float sg = dot(delta, f);
    float ov = proj(f, ax, ha) + proj(f, bx, hb) - fabsf(sg);
    if (ov < -margin) return 0;
    if (ov < best) { best = ov; bax = sg >= 0.f ? f : -f; kind = 0; k1 = k; }
  }
  for (int k = 0; k < 3; ++k) {
    V3 f = bx[k];
    float sg = dot(delta, f);
    float ov = proj(f, ax, ha) + proj(f, bx, hb) - fabsf(sg);
    if (ov < -margin) return 0;
    if (ov < best) { best = ov; bax = sg >= 0.f ? f : -f; kind = 1; k1 = k; }
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      V3 raw = cross(ax[i], bx[j]);
      float l2 = len2(raw);
      if (l2 < 1.0e-6f) continue;
      V3 l = raw * (1.f / sqrtf(l2));
      float sg = dot(delta, l);
      float ov = proj(l, ax, ha) + proj(l, bx, hb) - fabsf(sg);
      if (ov < -margin) return 0;
      if (ov < best) { best = ov; bax = sg >= 0.f ? l : -l; kind = 2; k1 = i; k2 = j; }
    }
  if (!isfinite(best)) return 0;
  float pen_shift = best + margin;
  if (pen_shift <= 0.f) return 0;
  if (kind == 2) {
    auto edge_mid = [](V3 c, const V3* basis, const float* h, int e, V3 dir) {
      int j = e == 0 ? 1 : 0, k = e == 2 ? 1 : 2;
      float sj = dot(dir, basis[j]) >= 0.f ? 1.f : -1.f;
      float sk = dot(dir, basis[k]) >= 0.f ? 1.f : -1.f;
      return c + basis[j] * (sj * h[j]) + basis[k] * (sk * h[k]);
    };
    V3 ma = edge_mid(A.p, ax, ha, k1, -bax), mb = edge_mid(B.p, bx, hb, k2, bax);
    V3 qa, qb;
    seg_closest(ma - ax[k1] * ha[k1], ma + ax[k1] * ha[k1], mb - bx[k2] * hb[k2], mb + bx[k2] * hb[k2], &qa, &qb);
    out[0] = CRes{qb, bax, pen_shift};
    return 1;
  }
  const bool ref_a = kind == 0;
  const V3 rc = ref_a ? A.p : B.p;
  const V3* rb = ref_a ? ax : bx;
  const float* rh = ref_a ? ha : hb;
  const V3 ic = ref_a ? B.p : A.p;
  const V3* ib = ref_a ? bx : ax;
  const float* ih = ref_a ? hb : ha;
  V3 ron = ref_a ? -bax : bax;
  float rs = dot(ron, rb[k1]) >= 0.f ? 1.f : -1.f;
  V3 rfc = rc + rb[k1] * (rs * rh[k1]);
  int ru = k1 == 0 ? 1 : 0, rv = k1 == 2 ? 1 : 2;
  int iax = 0;
  float isg = 1.f, idot = INFINITY;
  for (int k = 0; k < 3; ++k)
    for (int si = 0; si < 2; ++si) {
      float s = si == 0 ? 1.f : -1.f;
      float dd = dot(ib[k] * s, ron);
      if (dd < idot) { idot = dd; iax = k; isg = s; }
    }
  V3 ifc = ic + ib[iax] * (isg * ih[iax]);
  int iu = iax == 0 ? 1 : 0, iv = iax == 2 ? 1 : 2;
  V3 cu = ib[iu] * ih[iu], cv = ib[iv] * ih[iv];
  V3 corners[4] = {ifc - cu - cv, ifc + cu - cv, ifc + cu + cv, ifc - cu + cv};
  FV2 buf0[8], buf1[8];
  int nn = 4;
  for (int i = 0; i < 4; ++i) {
    V3 rel = corners[i] - rfc;
    buf0[i] = FV2{dot(rel, rb[ru]), dot(rel, rb[rv]), -dot(rel, ron)};
  }
  const float hu = rh[ru], hv = rh[rv];
  FV2* in = buf0;
  FV2* o = buf1;
  for (int edge = 0; edge < 4 && nn > 0; ++edge) {
    int m = 0;
    for (int i = 0; i < nn; ++i) {
      FV2 c = in[i], p = in[(i + nn - 1) % nn];
      float cs = edge == 0 ? c.u + hu : edge == 1 ? hu - c.u : edge == 2 ? c.v + hv : hv - c.v;
      float ps = edge == 0 ? p.u + hu : edge == 1 ? hu - p.u : edge == 2 ? p.v + hv : hv - p.v;
      bool ci = cs >= 0.f, pi = ps >= 0.f;
      if (ci) {
        if (!pi && m < 8) { float t = ps / (ps - cs); o[m++] = FV2{p.u + (c.u - p.u) * t, p.v + (c.v - p.v) * t, p.d + (c.d - p.d) * t}; }
        if (m < 8) o[m++] = c;
      } else if (pi && m < 8) {
        float t = ps / (ps - cs);
        o[m++] = FV2{p.u + (c.u - p.u) * t, p.v + (c.v - p.v) * t, p.d + (c.d - p.d) * t};
      }
    }
    nn = m;
    FV2* tmp = in; in = o; o = tmp;
  }
  float cpen[8];
  V3 cpos[8];
  int count = 0;
  for (int i = 0; i < nn; ++i) {
    float pen = in[i].d + margin;
    if (pen <= 0.f) continue;
    V3 por = rfc + rb[ru] * in[i].u + rb[rv] * in[i].v;
    cpen[count] = pen;
    cpos[count] = ref_a ? por + bax * (pen - margin) : por;
    if (++count == 8) break;
  }
  int order[8] = {0, 1, 2, 3, 4, 5, 6, 7};
  for (int i = 1; i < count; ++i) {
    int j = i;
    while (j > 0 && cpen[order[j]] > cpen[order[j - 1]]) { int t = order[j - 1]; order[j - 1] = order[j]; order[j] = t; --j; }
  }
  int take = count > 4 ? 4 : count;
  for (int k = 0; k < take; ++k) out[k] = CRes{cpos[order[k]], bax, cpen[order[k]]};
  return take;
}
