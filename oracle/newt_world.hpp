// Oracle (test infrastructure only): free bodies, geoms, the narrowphase
// subset, the soft-constraint PGS free-body solver, and World::step in its
// semi-implicit Euler form, restated from newt.
//
// Sources (paths inside hwang2409/tooling):
//   newt/src/body.rs:22-140          Body
//   newt/src/geom.rs:79-185,352-1009 SolRef, Geom, geom_world_pose, inertia helpers
//   newt/src/contact.rs:82-214       Contact, ContactBuf (cap 4)
//   newt/src/contact.rs:269-470      sphere_plane, box_plane, capsule_plane, sphere_sphere
//   newt/src/contact.rs:569-1247     box_box_full_manifold (SAT + face clipping)
//   newt/src/contact.rs:473-505      sphere_capsule; :1249-1272 capsule_capsule
//   newt/src/contact.rs:1296-1426    cylinder_plane, ellipsoid_plane; :1519-1628 sphere_cylinder;
//                                    :1630-1725 sphere_ellipsoid
//   newt/src/contact.rs:2313-2387    closest_point_on_segment, closest_points_on_segments
//   newt/src/contact.rs:2509-2587    dispatch / swap rule
//   newt/src/world.rs:1042-1069      auto_pairs (naive pair set; broadphase-independent contacts)
//   newt/src/world.rs:2476-2515      collect_contacts_full
//   newt/src/solver.rs:166-384       SolImp, sigmoid, impedance, safe_solref, reference_accel
//   newt/src/solver.rs:703-1257      solve_free_bodies_diag_mode (PGS branch)
//   newt/src/solver.rs:1448-1676     PGS row steps
//   newt/src/solver.rs:1892-2167     row response helpers
//   newt/src/world.rs:1459-1537      World::step (Euler branch)
//   newt/src/world.rs:1790-1817      step_bodies_euler
//   newt/src/world.rs:1952-2051      step_trees_euler
//   newt/src/world.rs:3104-3112      tangent_basis
//   newt/src/world.rs:3223-3245      evaluate
//
// Extension (no counterpart in newt): `sphere_box` contact.  newt rejects that
// shape pair (contact.rs:236-257); the restatement here is the closed-form
// sphere-vs-oriented-box closest point with newt's contact conventions
// (normal from B into A, penetration = margin - distance, contact point on
// B's surface).
#pragma once
#include <vector>
#include "newt_tree.hpp"

namespace oracle {

template <class R> struct Body {
  R mass = 1;
  Mat3<R> inertia, inertia_inv;
  Vec3<R> pos, vel;       // position, world linear velocity
  Quat<R> ori;
  Vec3<R> omega_body;     // body-frame angular velocity
};

template <class R> Body<R> make_body(R mass, Mat3<R> inertia, Vec3<R> pos, Quat<R> ori) {
  Body<R> b;
  b.mass = mass; b.inertia = inertia;
  if (!inertia.inverse(&b.inertia_inv)) b.inertia_inv = Mat3<R>::zero();
  b.pos = pos; b.ori = ori;
  return b;
}

template <class R> Mat3<R> solid_sphere_inertia(R mass, R r) {  // geom.rs:934-937
  R i = ((R(2) / R(5)) * mass * r) * r;
  return Mat3<R>::diag(i, i, i);
}
template <class R> Mat3<R> solid_box_inertia(R mass, Vec3<R> h) {  // geom.rs:939-947
  R hx2 = h.x * h.x, hy2 = h.y * h.y, hz2 = h.z * h.z;
  return Mat3<R>::diag((mass / R(3)) * (hy2 + hz2), (mass / R(3)) * (hx2 + hz2), (mass / R(3)) * (hx2 + hy2));
}
template <class R> Mat3<R> solid_capsule_inertia(R mass, R radius, R half_height) {  // geom.rs:949-966
  R r = radius, h = half_height;
  R vol_cyl = r * r * (R(2) * h);
  R vol_caps = (R(4) / R(3)) * r * r * r;
  R total = vol_cyl + vol_caps;
  R m_c = mass * (vol_cyl / total);
  R m_s = mass - m_c;
  R i_zz = R(0.5) * m_c * r * r + (R(2) / R(5)) * m_s * r * r;
  R offset = h + R(3) / R(8) * r;
  R hemi = (R(83) / R(320)) * m_s * r * r;
  R i_xx = (R(1) / R(12)) * m_c * (R(3) * r * r + R(4) * h * h) + hemi + m_s * offset * offset;
  return Mat3<R>::diag(i_xx, i_xx, i_zz);
}

enum Shape { S_PLANE = 0, S_SPHERE = 1, S_BOX = 2, S_CAPSULE = 3, S_CYLINDER = 4, S_ELLIPSOID = 5 };

template <class R> struct SolImp { R dmin = R(0.9), dmax = R(0.95), width = R(0.001), midpoint = R(0.5); int power = 2; };
template <class R> struct SolRef { R timeconst = R(0.02), dampratio = R(1); bool direct() const { return timeconst < R(0); } };

template <class R> struct Geom {
  int shape = S_SPHERE;
  R size[3] = {0, 0, 0};  // sphere: r; box: half extents; capsule: r, half_height
  int body = -1;          // free body index
  int tree = -1, link = -1;
  Vec3<R> local_pos; Quat<R> local_ori;
  R friction = 1;
  SolRef<R> solref; SolImp<R> solimp;
  R margin = 0, gap = 0;
  int condim = 3;
  unsigned group = 0xffffffffu, mask = 0xffffffffu;
  R torsional_friction = 0, rolling_friction = 0;  // geom.rs:397-409 (condim 4 / 6)
  // attachment key: 0 static, 1 body, 2 link
  int att_kind() const { return link >= 0 ? 2 : body >= 0 ? 1 : 0; }
};

template <class R> Geom<R> static_plane(Vec3<R> point, Vec3<R> normal, R friction) {  // geom.rs:494 + quat_align_z_to
  Geom<R> g; g.shape = S_PLANE; g.local_pos = point; g.friction = friction;
  Vec3<R> t = normal.normalize();
  R ct = t.z;
  if (ct > R(1) - R(1.0e-6)) g.local_ori = Quat<R>();
  else if (ct < R(-1) + R(1.0e-6)) g.local_ori = Quat<R>(1, 0, 0, 0);
  else {
    Vec3<R> ax = Vec3<R>(-t.y, t.x, R(0)).normalize();
    R hc = Sc<R>::sqrt((R(1) + ct) * R(0.5)), hs = Sc<R>::sqrt((R(1) - ct) * R(0.5));
    g.local_ori = Quat<R>(ax.x * hs, ax.y * hs, ax.z * hs, hc);
  }
  return g;
}

template <class R> struct Contact {
  int ga, gb;
  Vec3<R> pos, n;
  R pen, friction, gap;
};

template <class R> struct CBuf {  // contact.rs:115-214, capacity 4
  Contact<R> c[4];
  int len = 0;
  void push(const Contact<R>& x) { if (len < 4) c[len++] = x; }
};

template <class R> inline R cmin(R a, R b) { return a < b ? a : b; }
template <class R> inline R cmax(R a, R b) { return a > b ? a : b; }

// --------------------------------------------------------------------------
// Narrowphase primitives (contact.rs)
// --------------------------------------------------------------------------
template <class R> CBuf<R> sphere_plane(int is, const Pose<R>& sp, R radius, R fr, R margin, R gap, int ip, const Pose<R>& pp) {
  CBuf<R> out;
  Vec3<R> n = pp.o.rotate(Vec3<R>(0, 0, 1)), p0 = pp.p;
  R signed_d = (sp.p - p0).dot(n);
  R raw = signed_d - radius;
  if (raw <= margin) {
    Vec3<R> cp = sp.p - n * (radius + raw * R(0.5));
    out.push({is, ip, cp, n, margin - raw, fr, gap});
  }
  return out;
}

template <class R> CBuf<R> box_plane(int ib, const Pose<R>& bp, Vec3<R> h, R fr, R margin, R gap, int ip, const Pose<R>& pp) {
  Vec3<R> n = pp.o.rotate(Vec3<R>(0, 0, 1)), p0 = pp.p;
  CBuf<R> out;
  R dist = (bp.p - p0).dot(n);
  for (int i = 0; i < 8; ++i) {
    Vec3<R> local((i & 1) == 0 ? -h.x : h.x, (i & 2) == 0 ? -h.y : h.y, (i & 4) == 0 ? -h.z : h.z);
    Vec3<R> off = bp.o.rotate(local);
    R ldist = n.dot(off);
    R raw = dist + ldist;
    if (raw > margin || ldist > R(0)) continue;
    Vec3<R> corner = bp.p + off;
    Vec3<R> cp = corner - n * (raw * R(0.5));
    out.push({ib, ip, cp, n, margin - raw, fr, gap});
  }
  return out;
}

template <class R> CBuf<R> capsule_plane(int ic, const Pose<R>& cp_, R radius, R hh, R fr, R margin, R gap, int ip, const Pose<R>& pp) {
  Vec3<R> n = pp.o.rotate(Vec3<R>(0, 0, 1)), p0 = pp.p;
  Vec3<R> ax = cp_.o.rotate(Vec3<R>(0, 0, 1));
  Vec3<R> ends[2] = {cp_.p + ax * hh, cp_.p - ax * hh};
  CBuf<R> out;
  for (int k = 0; k < 2; ++k) {
    R raw = (ends[k] - p0).dot(n) - radius;
    if (raw <= margin) {
      Vec3<R> pt = ends[k] - n * (radius + raw * R(0.5));
      out.push({ic, ip, pt, n, margin - raw, fr, gap});
    }
  }
  return out;
}

template <class R> CBuf<R> sphere_sphere(int ia, Vec3<R> ca, R ra, int ib, Vec3<R> cb, R rb, R fr, R margin, R gap) {
  CBuf<R> out;
  Vec3<R> delta = ca - cb;
  R d2 = delta.length_squared();
  R srm = (ra + rb) + margin;
  if (d2 >= srm * srm) return out;
  R dist = Sc<R>::sqrt(d2);
  Vec3<R> n = dist > R(0) ? delta / dist : Vec3<R>(0, 0, 1);
  out.push({ia, ib, cb + n * rb, n, srm - dist, fr, gap});
  return out;
}

// Extension: sphere (A) vs box (B).  Closest point of the box to the sphere
// centre, clamped per local axis.  Centre inside the box: push out through
// the face of least depth (ties -> lowest axis, + side first).
template <class R> CBuf<R> sphere_box(int is, const Pose<R>& sp, R radius, int ib, const Pose<R>& bp, Vec3<R> h, R fr, R margin, R gap) {
  CBuf<R> out;
  Vec3<R> local = bp.o.inverse_rotate(sp.p - bp.p);
  R hl[3] = {h.x, h.y, h.z};
  R lc[3] = {local.x, local.y, local.z};
  bool inside = true;
  R cl[3];
  for (int k = 0; k < 3; ++k) {
    R v = lc[k];
    if (v > hl[k]) { v = hl[k]; inside = false; }
    else if (v < -hl[k]) { v = -hl[k]; inside = false; }
    cl[k] = v;
  }
  if (!inside) {
    Vec3<R> dl(lc[0] - cl[0], lc[1] - cl[1], lc[2] - cl[2]);
    R d2 = dl.length_squared();
    R rm = radius + margin;
    if (d2 >= rm * rm) return out;
    R dist = Sc<R>::sqrt(d2);
    Vec3<R> nl = dist > R(0) ? dl / dist : Vec3<R>(0, 0, 1);
    Vec3<R> n = bp.o.rotate(nl);
    Vec3<R> pb = bp.p + bp.o.rotate(Vec3<R>(cl[0], cl[1], cl[2]));
    out.push({is, ib, pb, n, rm - dist, fr, gap});
    return out;
  }
  int best = 0; R bestd = hl[0] - rabs(lc[0]);
  for (int k = 1; k < 3; ++k) { R dd = hl[k] - rabs(lc[k]); if (dd < bestd) { bestd = dd; best = k; } }
  R sgn = lc[best] >= R(0) ? R(1) : R(-1);
  R nl[3] = {0, 0, 0}; nl[best] = sgn;
  R face[3] = {lc[0], lc[1], lc[2]}; face[best] = sgn * hl[best];
  Vec3<R> n = bp.o.rotate(Vec3<R>(nl[0], nl[1], nl[2]));
  Vec3<R> pb = bp.p + bp.o.rotate(Vec3<R>(face[0], face[1], face[2]));
  out.push({is, ib, pb, n, (radius + margin) + bestd, fr, gap});
  return out;
}

template <class R> inline R clamp01(R x) { return x < R(0) ? R(0) : (x > R(1) ? R(1) : x); }

template <class R> void closest_points_on_segments(Vec3<R> a0, Vec3<R> a1, Vec3<R> b0, Vec3<R> b1, Vec3<R>* pa, Vec3<R>* pb) {
  Vec3<R> d1 = a1 - a0, d2 = b1 - b0, r = a0 - b0;
  R a = d1.length_squared(), e = d2.length_squared(), f = d2.dot(r);
  const R EPS = R(1.0e-12);
  if (a <= EPS && e <= EPS) { *pa = a0; *pb = b0; return; }
  if (a <= EPS) { R t = clamp01(f / e); *pa = a0; *pb = b0 + d2 * t; return; }
  R c = d1.dot(r);
  if (e <= EPS) { R s = clamp01(-c / a); *pa = a0 + d1 * s; *pb = b0; return; }
  R b_ = d1.dot(d2);
  R denom = a * e - b_ * b_;
  R s = denom != R(0) ? clamp01((b_ * f - c * e) / denom) : R(0);
  R tn = b_ * s + f;
  R t, sf;
  if (tn < R(0)) { t = R(0); sf = clamp01(-c / a); }
  else if (tn > e) { t = R(1); sf = clamp01((b_ - c) / a); }
  else { t = tn / e; sf = s; }
  *pa = a0 + d1 * sf; *pb = b0 + d2 * t;
}

// contact.rs:1296-1373 cylinder_plane: 18 samples (both cap centres, then
// the top and bottom rim points at 0, 45, ..., 315 degrees, interleaved), the
// up to four deepest with penetration > 0, deepest first (ties keep sample
// order), each projected onto the plane
template <class R> CBuf<R> cylinder_plane(int ic, const Pose<R>& cp_, R radius, R hh, R fr, R margin, R gap, int ip, const Pose<R>& pp) {
  Vec3<R> n = pp.o.rotate(Vec3<R>(0, 0, 1)), p0 = pp.p;
  Vec3<R> ax = cp_.o.rotate(Vec3<R>(0, 0, 1)), xl = cp_.o.rotate(Vec3<R>(1, 0, 0)), yl = cp_.o.rotate(Vec3<R>(0, 1, 0));
  Vec3<R> top = cp_.p + ax * hh, bot = cp_.p - ax * hh;
  const R s = R(0.70710677f);
  Vec3<R> rim[8] = {xl, xl * s + yl * s, yl, -xl * s + yl * s, -xl, -xl * s + -yl * s, -yl, xl * s + -yl * s};
  Vec3<R> smp[18];
  smp[0] = top; smp[1] = bot;
  for (int i = 0; i < 8; ++i) { smp[2 + 2 * i] = top + rim[i] * radius; smp[3 + 2 * i] = bot + rim[i] * radius; }
  R pen[18];
  int order[18], cnt = 0;
  for (int i = 0; i < 18; ++i) {
    pen[i] = margin - (smp[i] - p0).dot(n);
    if (pen[i] > R(0)) order[cnt++] = i;
  }
  for (int i = 1; i < cnt; ++i)
    for (int j = i; j > 0 && pen[order[j]] > pen[order[j - 1]]; --j) std::swap(order[j - 1], order[j]);
  CBuf<R> out;
  for (int k = 0; k < (cnt > 4 ? 4 : cnt); ++k) {
    int i = order[k];
    out.push({ic, ip, smp[i] - n * (margin - pen[i]), n, pen[i], fr, gap});
  }
  return out;
}

// contact.rs:1381-1426 ellipsoid_plane: the support point along -n,
// p = (a^2 d.x, b^2 d.y, c^2 d.z) / |(a d.x, b d.y, c d.z)| with d = -n in
// the ellipsoid frame; one contact when margin - distance >= 0
template <class R> CBuf<R> ellipsoid_plane(int ie, const Pose<R>& ep, Vec3<R> ax, R fr, R margin, R gap, int ip, const Pose<R>& pp) {
  CBuf<R> out;
  Vec3<R> n = pp.o.rotate(Vec3<R>(0, 0, 1)), p0 = pp.p;
  Vec3<R> d = ep.o.inverse_rotate(-n);
  R dsq = (ax.x * d.x) * (ax.x * d.x) + (ax.y * d.y) * (ax.y * d.y) + (ax.z * d.z) * (ax.z * d.z);
  if (dsq <= R(0)) return out;
  R den = Sc<R>::sqrt(dsq);
  Vec3<R> pl = Vec3<R>(ax.x * ax.x * d.x, ax.y * ax.y * d.y, ax.z * ax.z * d.z) / den;
  Vec3<R> sw = ep.p + ep.o.rotate(pl);
  R sg = (sw - p0).dot(n);
  R pen = margin - sg;
  if (pen >= R(0)) out.push({ie, ip, sw - n * (sg * R(0.5)), n, pen, fr, gap});
  return out;
}

// contact.rs:1519-1628 sphere_cylinder: the closest point of the solid
// cylinder to the sphere centre in the cylinder frame; a centre inside is
// pushed out through the nearer of cap and side (cap on ties)
template <class R> CBuf<R> sphere_cylinder(int is, const Pose<R>& sp, R rs, int ic, const Pose<R>& cp_, R rc, R hh, R fr, R margin, R gap) {
  Vec3<R> pl = cp_.o.inverse_rotate(sp.p - cp_.p);
  R z = pl.z;
  Vec3<R> pr(pl.x, pl.y, R(0));
  R dr = pr.length();
  bool in_ax = rabs(z) <= hh, in_rad = dr <= rc, inside = false;
  Vec3<R> cl;
  if (in_ax && in_rad) {
    inside = true;
    if (hh - rabs(z) <= rc - dr) cl = Vec3<R>(pl.x, pl.y, (z >= R(0) ? R(1) : R(-1)) * hh);
    else { Vec3<R> rd = dr > R(0) ? pr / dr : Vec3<R>(1, 0, 0); cl = Vec3<R>(rd.x * rc, rd.y * rc, z); }
  } else {
    R zc = z > hh ? hh : (z < -hh ? -hh : z);
    Vec3<R> rd = dr > R(0) ? pr / dr : Vec3<R>(1, 0, 0);
    R rcl = dr > rc ? rc : dr;
    cl = Vec3<R>(rd.x * rcl, rd.y * rcl, zc);
  }
  Vec3<R> dl = pl - cl;
  R dist = Sc<R>::sqrt(dl.length_squared());
  R pen = (inside ? rs + dist : rs - dist) + margin;
  CBuf<R> out;
  if (pen <= R(0)) return out;
  Vec3<R> nl = dist > R(1.0e-9) ? (inside ? -dl / dist : dl / dist) : Vec3<R>(0, 0, 1);
  out.push({is, ic, cp_.p + cp_.o.rotate(cl), cp_.o.rotate(nl), pen, fr, gap});
  return out;
}

// contact.rs:1630-1725 sphere_ellipsoid: the closest point q of the
// ellipsoid surface to the sphere centre p (ellipsoid frame) from twelve
// Newton steps, starting at t = 0, on the Lagrange parameter t of
// q = (a^2 p.x / (a^2 + t), b^2 p.y / (b^2 + t), c^2 p.z / (c^2 + t)) with
// f(t) = sum (a_k p_k / (a_k^2 + t))^2 - 1 (a zero denominator nudges t by
// 1e-6 (a_k^2 + 1) and spends the step); the normal (p - q) / |p - q| from
// the ellipsoid into the sphere, the contact point midway between q and the
// sphere's surface along it; nothing when the centre is farther than
// r + margin + the largest semi-axis + 1
template <class R> CBuf<R> sphere_ellipsoid(int is, const Pose<R>& sp, R rs, int ie, const Pose<R>& ep, Vec3<R> ax, R fr, R margin, R gap) {
  CBuf<R> out;
  const Vec3<R> p = ep.o.inverse_rotate(sp.p - ep.p);
  const R a = ax.x, b = ax.y, c = ax.z;
  const R mx = a > b ? (a > c ? a : c) : (b > c ? b : c);
  if (p.length() > rs + margin + mx + R(1)) return out;
  const R ap[3] = {a * p.x, b * p.y, c * p.z};
  const R a2[3] = {a * a, b * b, c * c};
  R t = R(0);
  for (int it = 0; it < 12; ++it) {
    R f = R(-1), fp = R(0);
    bool nudged = false;
    for (int k = 0; k < 3 && !nudged; ++k) {
      const R den = a2[k] + t;
      if (den == R(0)) { t += R(1.0e-6) * (a2[k] + R(1)); nudged = true; break; }
      const R inv = R(1) / den;
      const R num = ap[k] * inv;
      f += num * num;
      fp += R(-2) * ap[k] * ap[k] * inv * inv * inv;
    }
    if (nudged) continue;
    if (fp == R(0)) break;
    t -= f / fp;
  }
  const Vec3<R> q(a2[0] * p.x / (a2[0] + t), a2[1] * p.y / (a2[1] + t), a2[2] * p.z / (a2[2] + t));
  const Vec3<R> d = p - q;
  const R dist = d.length();
  const R pen = rs - dist + margin;
  if (pen <= R(0)) return out;
  const Vec3<R> nl = dist > R(1.0e-9) ? d / dist : Vec3<R>(0, 0, 1);
  const Vec3<R> nw = ep.o.rotate(nl);
  const Vec3<R> surf = ep.p + ep.o.rotate(q);
  const Vec3<R> ssurf = sp.p - nw * rs;
  out.push({is, ie, (surf + ssurf) * R(0.5), nw, pen, fr, gap});
  return out;
}

// contact.rs:2313-2321 closest_point_on_segment
template <class R> Vec3<R> closest_point_on_segment(Vec3<R> p, Vec3<R> a, Vec3<R> b) {
  Vec3<R> ab = b - a;
  R denom = ab.length_squared();
  if (denom == R(0)) return a;
  return a + ab * clamp01((p - a).dot(ab) / denom);
}

// contact.rs:473-505 sphere_capsule: sphere vs the sphere at the capsule
// axis point closest to the sphere centre (segment from -h to +h along local z)
template <class R> CBuf<R> sphere_capsule(int is, const Pose<R>& sp, R rs, int ic, const Pose<R>& cp_, R rc, R hh, R fr, R margin, R gap) {
  Vec3<R> ax = cp_.o.rotate(Vec3<R>(0, 0, 1));
  Vec3<R> closest = closest_point_on_segment(sp.p, cp_.p - ax * hh, cp_.p + ax * hh);
  return sphere_sphere(is, sp.p, rs, ic, closest, rc, fr, margin, gap);
}

// contact.rs:1249-1272 capsule_capsule: closest points of the two axis
// segments, then sphere vs sphere there
template <class R> CBuf<R> capsule_capsule(int ia, const Pose<R>& pa, R ra, R ha, int ib, const Pose<R>& pb, R rb, R hb, R fr, R margin, R gap) {
  Vec3<R> ax = pa.o.rotate(Vec3<R>(0, 0, 1)), bx = pb.o.rotate(Vec3<R>(0, 0, 1));
  Vec3<R> ca, cb;
  closest_points_on_segments(pa.p - ax * ha, pa.p + ax * ha, pb.p - bx * hb, pb.p + bx * hb, &ca, &cb);
  return sphere_sphere(ia, ca, ra, ib, cb, rb, fr, margin, gap);
}

template <class R> struct FV { R u, v, depth; };

template <class R> int sh_clip(const FV<R>* subject, R hu, R hv, FV<R>* outp) {  // contact.rs:1087-1139
  FV<R> buf[2][16];
  int n = 4;
  for (int i = 0; i < 4; ++i) buf[0][i] = subject[i];
  int cur = 0;
  for (int edge = 0; edge < 4; ++edge) {
    if (n == 0) break;
    FV<R>* in = buf[cur];
    FV<R>* out = buf[cur ^ 1];
    int m = 0;
    auto sgn = [&](const FV<R>& p) -> R {
      switch (edge) { case 0: return p.u + hu; case 1: return hu - p.u; case 2: return p.v + hv; default: return hv - p.v; }
    };
    for (int i = 0; i < n; ++i) {
      FV<R> c = in[i], p = in[(i + n - 1) % n];
      R cs = sgn(c), ps = sgn(p);
      bool ci = cs >= R(0), pi = ps >= R(0);
      auto lerp = [&](R t) { return FV<R>{p.u + (c.u - p.u) * t, p.v + (c.v - p.v) * t, p.depth + (c.depth - p.depth) * t}; };
      if (ci) {
        if (!pi) { R t = ps / (ps - cs); out[m++] = lerp(t); }
        out[m++] = c;
      } else if (pi) {
        R t = ps / (ps - cs); out[m++] = lerp(t);
      }
    }
    n = m; cur ^= 1;
  }
  for (int i = 0; i < n; ++i) outp[i] = buf[cur][i];
  return n;
}

template <class R> CBuf<R> box_box(int ia, const Pose<R>& pa, Vec3<R> half_a, int ib, const Pose<R>& pb, Vec3<R> half_b, R fr, R margin, R gap) {
  Vec3<R> ax[3] = {pa.o.rotate(Vec3<R>(1, 0, 0)), pa.o.rotate(Vec3<R>(0, 1, 0)), pa.o.rotate(Vec3<R>(0, 0, 1))};
  Vec3<R> bx[3] = {pb.o.rotate(Vec3<R>(1, 0, 0)), pb.o.rotate(Vec3<R>(0, 1, 0)), pb.o.rotate(Vec3<R>(0, 0, 1))};
  R ha[3] = {half_a.x, half_a.y, half_a.z}, hb[3] = {half_b.x, half_b.y, half_b.z};
  Vec3<R> delta = pa.p - pb.p;
  auto proj = [](Vec3<R> l, const Vec3<R>* u, const R* h) {
    return h[0] * rabs(l.dot(u[0])) + h[1] * rabs(l.dot(u[1])) + h[2] * rabs(l.dot(u[2]));
  };
  R best = R(INFINITY);
  Vec3<R> best_axis(0, 0, 1);
  int kind = 0, k1 = 0, k2 = 0;  // kind 0 faceA, 1 faceB, 2 edge
  CBuf<R> empty;
  for (int k = 0; k < 3; ++k) {
    Vec3<R> f = ax[k];
    R ov = proj(f, ax, ha) + proj(f, bx, hb) - rabs(delta.dot(f));
    R sg = delta.dot(f);
    if (ov < -margin) return empty;
    if (ov < best) { best = ov; best_axis = sg >= R(0) ? f : -f; kind = 0; k1 = k; }
  }
  for (int k = 0; k < 3; ++k) {
    Vec3<R> f = bx[k];
    R ov = proj(f, ax, ha) + proj(f, bx, hb) - rabs(delta.dot(f));
    R sg = delta.dot(f);
    if (ov < -margin) return empty;
    if (ov < best) { best = ov; best_axis = sg >= R(0) ? f : -f; kind = 1; k1 = k; }
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      Vec3<R> raw = ax[i].cross(bx[j]);
      R len2 = raw.length_squared();
      if (len2 < R(1.0e-6)) continue;
      Vec3<R> l = raw / Sc<R>::sqrt(len2);
      R sg = delta.dot(l);
      R ov = proj(l, ax, ha) + proj(l, bx, hb) - rabs(sg);
      if (ov < -margin) return empty;
      if (ov < best) { best = ov; best_axis = sg >= R(0) ? l : -l; kind = 2; k1 = i; k2 = j; }
    }
  if (!std::isfinite((double)best)) return empty;
  R pen_shift = best + margin;
  if (pen_shift <= R(0)) return empty;
  CBuf<R> out;
  if (kind == 2) {  // contact.rs:870-910
    auto edge_mid = [](Vec3<R> c, const Vec3<R>* basis, const R* h, int e, Vec3<R> dir) {
      int j = e == 0 ? 1 : 0, k = e == 2 ? 1 : 2;
      R sj = dir.dot(basis[j]) >= R(0) ? R(1) : R(-1);
      R sk = dir.dot(basis[k]) >= R(0) ? R(1) : R(-1);
      return c + basis[j] * (sj * h[j]) + basis[k] * (sk * h[k]);
    };
    Vec3<R> ma = edge_mid(pa.p, ax, ha, k1, -best_axis);
    Vec3<R> mb = edge_mid(pb.p, bx, hb, k2, best_axis);
    Vec3<R> ea0 = ma - ax[k1] * ha[k1], ea1 = ma + ax[k1] * ha[k1];
    Vec3<R> eb0 = mb - bx[k2] * hb[k2], eb1 = mb + bx[k2] * hb[k2];
    Vec3<R> qa, qb;
    closest_points_on_segments(ea0, ea1, eb0, eb1, &qa, &qb);
    out.push({ia, ib, qb, best_axis, pen_shift, fr, gap});
    return out;
  }
  // Face reference clipping (contact.rs:916-1053).
  bool ref_is_a = kind == 0;
  Vec3<R> rc = ref_is_a ? pa.p : pb.p;
  const Vec3<R>* rbasis = ref_is_a ? ax : bx;
  const R* rh = ref_is_a ? ha : hb;
  Vec3<R> icen = ref_is_a ? pb.p : pa.p;
  const Vec3<R>* ibasis = ref_is_a ? bx : ax;
  const R* ih = ref_is_a ? hb : ha;
  Vec3<R> ron = ref_is_a ? -best_axis : best_axis;
  Vec3<R> rfa = rbasis[k1];
  R rs = ron.dot(rfa) >= R(0) ? R(1) : R(-1);
  Vec3<R> rfc = rc + rfa * (rs * rh[k1]);
  int ru = k1 == 0 ? 1 : 0, rv = k1 == 2 ? 1 : 2;
  Vec3<R> ref_u = rbasis[ru], ref_v = rbasis[rv];
  R rhu = rh[ru], rhv = rh[rv];
  int iax = 0; R isg = R(1), idot = R(INFINITY);
  for (int k = 0; k < 3; ++k)
    for (int si = 0; si < 2; ++si) {
      R s = si == 0 ? R(1) : R(-1);
      R dd = (ibasis[k] * s).dot(ron);
      if (dd < idot) { idot = dd; iax = k; isg = s; }
    }
  Vec3<R> ifc = icen + ibasis[iax] * (isg * ih[iax]);
  int iu = iax == 0 ? 1 : 0, iv = iax == 2 ? 1 : 2;
  Vec3<R> inc_u = ibasis[iu], inc_v = ibasis[iv];
  R ihu = ih[iu], ihv = ih[iv];
  Vec3<R> corners[4] = {ifc - inc_u * ihu - inc_v * ihv, ifc + inc_u * ihu - inc_v * ihv,
                        ifc + inc_u * ihu + inc_v * ihv, ifc - inc_u * ihu + inc_v * ihv};
  FV<R> subj[4];
  for (int i = 0; i < 4; ++i) {
    Vec3<R> rel = corners[i] - rfc;
    subj[i] = {rel.dot(ref_u), rel.dot(ref_v), -rel.dot(ron)};
  }
  FV<R> clipped[16];
  int nc = sh_clip(subj, rhu, rhv, clipped);
  R cpen[8]; Vec3<R> cpos[8]; int count = 0;
  for (int i = 0; i < nc; ++i) {
    R pen = clipped[i].depth + margin;
    if (pen <= R(0)) continue;
    Vec3<R> por = rfc + ref_u * clipped[i].u + ref_v * clipped[i].v;
    Vec3<R> pos = ref_is_a ? por + best_axis * (pen - margin) : por;
    cpen[count] = pen; cpos[count] = pos; ++count;
    if (count == 8) break;
  }
  int order[8] = {0, 1, 2, 3, 4, 5, 6, 7};
  for (int i = 1; i < count; ++i) {
    int j = i;
    while (j > 0 && cpen[order[j]] > cpen[order[j - 1]]) { std::swap(order[j - 1], order[j]); --j; }
  }
  int take = count > 4 ? 4 : count;
  for (int k = 0; k < take; ++k) out.push({ia, ib, cpos[order[k]], best_axis, cpen[order[k]], fr, gap});
  return out;
}

// contact.rs:2509-2587 dispatch: try (A,B); otherwise (B,A) and relabel.
template <class R> bool try_np(int ia, const Geom<R>& a, const Pose<R>& pa, int ib, const Geom<R>& b, const Pose<R>& pb,
                               R fr, R margin, R gap, CBuf<R>* out) {
  if (a.shape == S_SPHERE && b.shape == S_PLANE) { *out = sphere_plane(ia, pa, a.size[0], fr, margin, gap, ib, pb); return true; }
  if (a.shape == S_BOX && b.shape == S_PLANE) { *out = box_plane(ia, pa, Vec3<R>(a.size[0], a.size[1], a.size[2]), fr, margin, gap, ib, pb); return true; }
  if (a.shape == S_CAPSULE && b.shape == S_PLANE) { *out = capsule_plane(ia, pa, a.size[0], a.size[1], fr, margin, gap, ib, pb); return true; }
  if (a.shape == S_SPHERE && b.shape == S_SPHERE) { *out = sphere_sphere(ia, pa.p, a.size[0], ib, pb.p, b.size[0], fr, margin, gap); return true; }
  if (a.shape == S_BOX && b.shape == S_BOX) {
    *out = box_box(ia, pa, Vec3<R>(a.size[0], a.size[1], a.size[2]), ib, pb, Vec3<R>(b.size[0], b.size[1], b.size[2]), fr, margin, gap);
    return true;
  }
  if (a.shape == S_CYLINDER && b.shape == S_PLANE) { *out = cylinder_plane(ia, pa, a.size[0], a.size[1], fr, margin, gap, ib, pb); return true; }
  if (a.shape == S_ELLIPSOID && b.shape == S_PLANE) {
    *out = ellipsoid_plane(ia, pa, Vec3<R>(a.size[0], a.size[1], a.size[2]), fr, margin, gap, ib, pb);
    return true;
  }
  if (a.shape == S_SPHERE && b.shape == S_CYLINDER) {
    *out = sphere_cylinder(ia, pa, a.size[0], ib, pb, b.size[0], b.size[1], fr, margin, gap);
    return true;
  }
  if (a.shape == S_SPHERE && b.shape == S_CAPSULE) {
    *out = sphere_capsule(ia, pa, a.size[0], ib, pb, b.size[0], b.size[1], fr, margin, gap);
    return true;
  }
  if (a.shape == S_SPHERE && b.shape == S_ELLIPSOID) {
    *out = sphere_ellipsoid(ia, pa, a.size[0], ib, pb, Vec3<R>(b.size[0], b.size[1], b.size[2]), fr, margin, gap);
    return true;
  }
  if (a.shape == S_CAPSULE && b.shape == S_CAPSULE) {
    *out = capsule_capsule(ia, pa, a.size[0], a.size[1], ib, pb, b.size[0], b.size[1], fr, margin, gap);
    return true;
  }
  if (a.shape == S_SPHERE && b.shape == S_BOX) {
    *out = sphere_box(ia, pa, a.size[0], ib, pb, Vec3<R>(b.size[0], b.size[1], b.size[2]), fr, margin, gap);
    return true;
  }
  return false;
}

template <class R> CBuf<R> narrow_phase(int ia, const Geom<R>& a, const Pose<R>& pa, int ib, const Geom<R>& b, const Pose<R>& pb) {
  R fr = cmin(a.friction, b.friction);
  R margin = cmax(a.margin, b.margin);
  R gap = cmax(a.gap, b.gap);
  CBuf<R> out;
  if (try_np(ia, a, pa, ib, b, pb, fr, margin, gap, &out)) return out;
  if (try_np(ib, b, pb, ia, a, pa, fr, margin, gap, &out)) {
    for (int k = 0; k < out.len; ++k) { std::swap(out.c[k].ga, out.c[k].gb); out.c[k].n = -out.c[k].n; }
    return out;
  }
  return CBuf<R>();
}

// --------------------------------------------------------------------------
// Soft-constraint parameters (solver.rs:166-384)
// --------------------------------------------------------------------------
template <class R> inline R clamp_imp(R v) { return v < R(1.0e-4) ? R(1.0e-4) : (v > R(0.9999) ? R(0.9999) : v); }
template <class R> SolImp<R> effective_solimp(SolImp<R> s) {
  SolImp<R> o;
  o.dmin = clamp_imp(s.dmin); o.dmax = clamp_imp(s.dmax);
  o.width = s.width > R(0) ? s.width : R(0);
  o.midpoint = clamp_imp(s.midpoint); o.power = s.power > 1 ? s.power : 1;
  return o;
}
template <class R> R powi(R x, int n) { R r = R(1); for (int i = 0; i < n; ++i) r *= x; return r; }
template <class R> R sigmoid(R x, int power, R mid) {
  if (x <= R(0)) return R(0);
  if (x >= R(1)) return R(1);
  if (x < mid) return mid * powi(x / mid, power);
  return R(1) - (R(1) - mid) * powi((R(1) - x) / (R(1) - mid), power);
}
template <class R> R impedance_at(R position, R margin, SolImp<R> s) {
  s = effective_solimp(s);
  R x = (position - margin) / s.width;
  if (x < R(0)) x = -x;
  R y = sigmoid(x, s.power, s.midpoint);
  return s.dmin + (s.dmax - s.dmin) * y;
}
template <class R> SolRef<R> safe_solref(SolRef<R> s, R dt) {
  if (!s.direct() && s.timeconst < R(2) * dt) { SolRef<R> o; o.timeconst = R(2) * dt; o.dampratio = s.dampratio; return o; }
  return s;
}
template <class R> R reference_accel(R position, R velocity, SolRef<R> sr, SolImp<R> si) {
  si = effective_solimp(si);
  R d = impedance_at(position, R(0), si);
  R b, k;
  if (sr.direct()) { b = -sr.dampratio / si.dmax; k = -sr.timeconst / (si.dmax * si.dmax); }
  else {
    R tc = sr.timeconst, dmax = si.dmax;
    b = R(2) / (dmax * tc);
    k = d / (dmax * dmax * tc * tc * sr.dampratio * sr.dampratio);
  }
  return -b * velocity - k * position;
}
template <class R> SolRef<R> combine_solref(SolRef<R> a, SolRef<R> b) {  // geom.rs:156-185
  if (a.direct() || b.direct()) {
    if (a.direct() && b.direct()) {
      SolRef<R> o; o.timeconst = a.timeconst <= b.timeconst ? a.timeconst : b.timeconst;
      o.dampratio = a.dampratio <= b.dampratio ? a.dampratio : b.dampratio; return o;
    }
    return a.direct() ? a : b;
  }
  SolRef<R> o;
  o.timeconst = a.timeconst <= b.timeconst ? a.timeconst : b.timeconst;
  o.dampratio = a.dampratio <= b.dampratio ? a.dampratio : b.dampratio;
  return o;
}
template <class R> SolImp<R> combine_solimp(SolImp<R> a, SolImp<R> b) {
  SolImp<R> o; o.dmin = cmin(a.dmin, b.dmin); o.dmax = cmin(a.dmax, b.dmax); o.width = cmin(a.width, b.width);
  o.midpoint = a.midpoint; o.power = a.power; return o;
}

template <class R> void tangent_basis(Vec3<R> n, Vec3<R>* t1, Vec3<R>* t2) {  // world.rs:3104-3112
  bool use_z = rabs(n.z) < R(0.9);
  Vec3<R> ref = use_z ? Vec3<R>(0, 0, 1) : Vec3<R>(1, 0, 0);
  *t1 = ref.cross(n).normalize();
  *t2 = n.cross(*t1);
}

// --------------------------------------------------------------------------
// Free-body PGS (solver.rs:703-1257), pyramidal cone, condim 3 and 1.
// --------------------------------------------------------------------------
template <class R> struct Row {  // solver.rs ConstraintRow; `ang`: RowGeom::Angular (torque about dir)
  Vec3<R> dir; int ba, bb; Vec3<R> arm_a, arm_b; R reg, diag, bias; bool ang = false;
};
template <class R> struct BDelta { Vec3<R> dv, dw; };

template <class R> struct PgsStats { int rows = 0; int contacts = 0; };

template <class R> R row_body_diagonal(const Row<R>& r, const std::vector<Body<R>>& bodies, const std::vector<Mat3<R>>& iinv) {
  R a = R(0);  // solver.rs:1892-1924
  if (r.ang) {
    if (r.ba >= 0) a += r.dir.dot(iinv[r.ba] * r.dir);
    if (r.bb >= 0) a += r.dir.dot(iinv[r.bb] * r.dir);
    return a;
  }
  if (r.ba >= 0) { Vec3<R> rc = r.arm_a.cross(r.dir); a += rc.dot(iinv[r.ba] * rc) + R(1) / bodies[r.ba].mass; }
  if (r.bb >= 0) { Vec3<R> rc = r.arm_b.cross(r.dir); a += rc.dot(iinv[r.bb] * rc) + R(1) / bodies[r.bb].mass; }
  return a;
}
template <class R> R row_residual(const Row<R>& r, const std::vector<BDelta<R>>& bd, const std::vector<Body<R>>& bodies) {
  R s = R(0);  // solver.rs:1980-2018
  if (r.ang) {
    if (r.ba >= 0) s += bodies[r.ba].ori.rotate(bd[r.ba].dw).dot(r.dir);
    if (r.bb >= 0) s -= bodies[r.bb].ori.rotate(bd[r.bb].dw).dot(r.dir);
    return s;
  }
  if (r.ba >= 0) { Vec3<R> dw = bodies[r.ba].ori.rotate(bd[r.ba].dw); Vec3<R> vp = bd[r.ba].dv + dw.cross(r.arm_a); s += vp.dot(r.dir); }
  if (r.bb >= 0) { Vec3<R> dw = bodies[r.bb].ori.rotate(bd[r.bb].dw); Vec3<R> vp = bd[r.bb].dv + dw.cross(r.arm_b); s -= vp.dot(r.dir); }
  return s;
}
template <class R> void apply_impulse(const Row<R>& r, R df, std::vector<BDelta<R>>& bd, const std::vector<Body<R>>& bodies, const std::vector<Mat3<R>>& iinv) {
  if (df == R(0)) return;  // solver.rs:2022-2066
  if (r.ang) {
    if (r.ba >= 0) { Vec3<R> tq = r.dir * df; bd[r.ba].dw += bodies[r.ba].ori.inverse_rotate(iinv[r.ba] * tq); }
    if (r.bb >= 0) { Vec3<R> tq = -r.dir * df; bd[r.bb].dw += bodies[r.bb].ori.inverse_rotate(iinv[r.bb] * tq); }
    return;
  }
  if (r.ba >= 0) {
    Vec3<R> f = r.dir * df; Vec3<R> tq = r.arm_a.cross(f);
    bd[r.ba].dv += f / bodies[r.ba].mass;
    Vec3<R> dw = iinv[r.ba] * tq;
    bd[r.ba].dw += bodies[r.ba].ori.inverse_rotate(dw);
  }
  if (r.bb >= 0) {
    Vec3<R> f = -r.dir * df; Vec3<R> tq = r.arm_b.cross(f);
    bd[r.bb].dv += f / bodies[r.bb].mass;
    Vec3<R> dw = iinv[r.bb] * tq;
    bd[r.bb].dw += bodies[r.bb].ori.inverse_rotate(dw);
  }
}
template <class R> R point_dir_velocity(const std::vector<Body<R>>& bodies, int ba, int bb, Vec3<R> arm_a, Vec3<R> arm_b, Vec3<R> n) {
  Vec3<R> va, vb;
  if (ba >= 0) { const Body<R>& b = bodies[ba]; va = b.vel + b.ori.rotate(b.omega_body).cross(arm_a); }
  if (bb >= 0) { const Body<R>& b = bodies[bb]; vb = b.vel + b.ori.rotate(b.omega_body).cross(arm_b); }
  return (va - vb).dot(n);
}

struct PgsContactInfo { int start_row; int condim; int contact_index; };

// Rows of the free-body contact system (solver.rs:752-1061): per active
// contact its facet rows (pyramidal condim 3) or normal row (condim 1), with
// regularisation, diagonal and bias; `pcs` keeps the contact blocks.
template <class R> struct FreePC {
  int ci, start, condim; SolRef<R> sr; SolImp<R> si; R pen, mu; R h01a, h01b;
  R mu_t = 0, mu_r = 0; int nrows = 1;  // torsional / rolling friction, rows of the block
};
template <class R> struct FreeSystem {
  std::vector<Row<R>> rows;
  std::vector<FreePC<R>> pcs;
  std::vector<Mat3<R>> iinv;
  int cone = 0;  // 0 pyramidal, 1 elliptic (solver.rs:75-88)
  // pyramidal condim 3: the four facet rows n +- mu t
  bool facets(const FreePC<R>& pc) const { return cone == 0 && pc.condim == 3; }
};

template <class R>
void assemble_free_rows(const std::vector<Body<R>>& bodies, const std::vector<Geom<R>>& geoms,
                        const std::vector<Contact<R>>& contacts, Vec3<R> gravity, R dt, FreeSystem<R>& sys) {
  const int nb = (int)bodies.size();
  std::vector<Row<R>>& rows = sys.rows;
  std::vector<FreePC<R>>& pcs = sys.pcs;
  rows.clear();
  pcs.clear();
  std::vector<Vec3<R>> dvfree(nb);
  for (int i = 0; i < nb; ++i) dvfree[i] = gravity * dt;
  for (int ci = 0; ci < (int)contacts.size(); ++ci) {
    const Contact<R>& c = contacts[ci];
    const Geom<R>& ga = geoms[c.ga];
    const Geom<R>& gb = geoms[c.gb];
    int ba = ga.body, bb = gb.body;
    if (ba < 0 && bb < 0) continue;
    R pen_active = c.pen - c.gap;
    if (pen_active <= R(0)) continue;
    SolRef<R> sr = combine_solref(ga.solref, gb.solref);
    SolImp<R> si = combine_solimp(ga.solimp, gb.solimp);
    R mu = cmin(ga.friction, gb.friction);
    int condim = ga.condim < gb.condim ? ga.condim : gb.condim;
    Vec3<R> n = c.n, t1, t2u;
    tangent_basis(n, &t1, &t2u);
    Vec3<R> t2 = n.cross(t1);  // solver.rs:3458-3463 fallback axes
    Vec3<R> arm_a = ba >= 0 ? c.pos - bodies[ba].pos : Vec3<R>();
    Vec3<R> arm_b = bb >= 0 ? c.pos - bodies[bb].pos : Vec3<R>();
    int start = (int)rows.size();
    FreePC<R> pc{ci, start, condim, sr, si, pen_active, mu, R(0), R(0)};
    pc.mu_t = cmin(ga.torsional_friction, gb.torsional_friction);  // combine_torsional_friction
    pc.mu_r = cmin(ga.rolling_friction, gb.rolling_friction);      // combine_rolling_friction
    // contact_row_directions (solver.rs:3401-3429) and the torsion / rolling
    // rows (:820-848); newt pushes the angular rows a second time after the
    // directions, rows that get no constants and are never swept, so only
    // the block's own rows are kept here
    if (sys.cone == 0 && condim == 3) {
      Vec3<R> dirs[4] = {n + t1 * mu, n - t1 * mu, n + t2 * mu, n - t2 * mu};
      for (int k = 0; k < 4; ++k) rows.push_back({dirs[k], ba, bb, arm_a, arm_b, R(0), R(0), R(0)});
      pc.nrows = 4;
    } else {
      rows.push_back({n, ba, bb, arm_a, arm_b, R(0), R(0), R(0)});
      if (condim >= 3) {
        rows.push_back({t1, ba, bb, arm_a, arm_b, R(0), R(0), R(0)});
        rows.push_back({t2, ba, bb, arm_a, arm_b, R(0), R(0), R(0)});
      }
      const Vec3<R> z;
      if (condim >= 4) rows.push_back({n, ba, bb, z, z, R(0), R(0), R(0), true});
      if (condim >= 6) {
        rows.push_back({t1, ba, bb, z, z, R(0), R(0), R(0), true});
        rows.push_back({t2, ba, bb, z, z, R(0), R(0), R(0), true});
      }
      pc.nrows = (int)rows.size() - start;
    }
    pcs.push_back(pc);
  }
  if (rows.empty()) return;
  sys.iinv.resize(nb);
  std::vector<Mat3<R>>& iinv = sys.iinv;
  for (int i = 0; i < nb; ++i) { Mat3<R> r = bodies[i].ori.to_mat3(); iinv[i] = r * bodies[i].inertia_inv * r.transpose(); }
  for (FreePC<R>& pc : pcs) {
    const int nr = pc.nrows;
    const bool fac = sys.facets(pc);
    for (int k = 0; k < nr; ++k) {
      Row<R>& r = rows[pc.start + k];
      R aii = row_body_diagonal(r, bodies, iinv);
      R d = impedance_at(-pc.pen, R(0), pc.si);
      // contact_regularization (solver.rs:1930-1974)
      R reg = R(0);
      if (d > R(0)) {
        R tran = R(0);
        if (r.ba >= 0) tran += R(1) / bodies[r.ba].mass;
        if (r.bb >= 0) tran += R(1) / bodies[r.bb].mass;
        R base = fac ? tran * (R(1) + pc.mu * pc.mu) : row_body_diagonal(r, bodies, iinv);
        R breg = (R(1) - d) / d * base;
        reg = fac ? R(2) * pc.mu * pc.mu * breg : breg;
      }
      r.reg = reg;
      r.diag = aii + reg;
    }
    for (int k = 0; k < nr; ++k) {
      Row<R>& r = rows[pc.start + k];
      R vcur, dvf = R(0);
      if (r.ang) {  // row_current_velocity (solver.rs:2071-2093); no angular free step (:2108-2127)
        Vec3<R> wa, wb;
        if (r.ba >= 0) wa = bodies[r.ba].ori.rotate(bodies[r.ba].omega_body);
        if (r.bb >= 0) wb = bodies[r.bb].ori.rotate(bodies[r.bb].omega_body);
        vcur = (wa - wb).dot(r.dir);
      } else {
        vcur = point_dir_velocity(bodies, r.ba, r.bb, r.arm_a, r.arm_b, r.dir);
        // free_step_velocity_contribution with zero angular free step
        if (r.ba >= 0) { Vec3<R> dw = bodies[r.ba].ori.rotate(Vec3<R>()); Vec3<R> vp = dvfree[r.ba] + dw.cross(r.arm_a); dvf += vp.dot(r.dir); }
        if (r.bb >= 0) { Vec3<R> dw = bodies[r.bb].ori.rotate(Vec3<R>()); Vec3<R> vp = dvfree[r.bb] + dw.cross(r.arm_b); dvf -= vp.dot(r.dir); }
      }
      // the penetration drives the facets and the normal row only (solver.rs:944-948)
      R position = (fac || k == 0) ? -pc.pen : R(0);
      SolRef<R> sr = safe_solref(pc.sr, dt);
      R aref = reference_accel(position, vcur, sr, pc.si);
      r.bias = dvf - aref * dt;
    }
  }
}

// Per-body wrenches (impulse / dt) from the rows' impulses (solver.rs:1204-1234).
template <class R>
void free_row_wrenches(const FreeSystem<R>& sys, const std::vector<R>& imp, R dt, std::vector<Wrench<R>>& wrenches) {
  for (int ri = 0; ri < (int)sys.rows.size(); ++ri) {
    R f = imp[ri];
    if (f == R(0)) continue;
    const Row<R>& r = sys.rows[ri];
    Vec3<R> fa = r.dir * (f / dt);
    if (r.ang) {  // a pure torque along dir
      if (r.ba >= 0) wrenches[r.ba].t += fa;
      if (r.bb >= 0) wrenches[r.bb].t += -fa;
      continue;
    }
    if (r.ba >= 0) { wrenches[r.ba].f += fa; wrenches[r.ba].t += r.arm_a.cross(fa); }
    if (r.bb >= 0) { Vec3<R> fb = -fa; wrenches[r.bb].f += fb; wrenches[r.bb].t += r.arm_b.cross(fb); }
  }
}

template <class R> void free_row_contacts(const FreeSystem<R>& sys, std::vector<int>* row_contact_out) {
  row_contact_out->assign(sys.rows.size(), -1);
  for (const FreePC<R>& pc : sys.pcs)
    for (int k = 0; k < pc.nrows; ++k) (*row_contact_out)[pc.start + k] = pc.ci;
}

// Returns per-body (force, torque) wrenches; optionally the per-row impulses
// and row metadata (for the impulse-parity tests).
template <class R>
void solve_free_bodies_pgs(const std::vector<Body<R>>& bodies, const std::vector<Geom<R>>& geoms,
                           const std::vector<Contact<R>>& contacts, Vec3<R> gravity, R dt, int iterations,
                           std::vector<Wrench<R>>& wrenches, std::vector<R>* impulses_out = nullptr,
                           std::vector<int>* row_contact_out = nullptr, int cone = 0) {
  const int nb = (int)bodies.size();
  wrenches.assign(nb, Wrench<R>{Vec3<R>(), Vec3<R>()});
  if (impulses_out) impulses_out->clear();
  if (row_contact_out) row_contact_out->clear();
  if (contacts.empty() || dt <= R(0)) return;
  FreeSystem<R> sys;
  sys.cone = cone;
  assemble_free_rows(bodies, geoms, contacts, gravity, dt, sys);
  std::vector<Row<R>>& rows = sys.rows;
  const std::vector<Mat3<R>>& iinv = sys.iinv;
  const int nrows = (int)rows.size();
  if (nrows == 0) return;
  std::vector<BDelta<R>> scratch(nb);
  for (FreePC<R>& pc : sys.pcs) {
    if (!sys.facets(pc)) continue;
    for (int pair = 0; pair < 2; ++pair) {
      const Row<R>& ri = rows[pc.start + 2 * pair];
      const Row<R>& rj = rows[pc.start + 2 * pair + 1];
      for (auto& s : scratch) s = BDelta<R>{Vec3<R>(), Vec3<R>()};
      apply_impulse(rj, R(1), scratch, bodies, iinv);
      R h = row_residual(ri, scratch, bodies);
      if (pair == 0) pc.h01a = h; else pc.h01b = h;
    }
  }
  std::vector<R> imp(nrows, R(0));
  std::vector<BDelta<R>> bd(nb, BDelta<R>{Vec3<R>(), Vec3<R>()});
  auto step_nonneg = [&](int ri) {
    const Row<R>& r = rows[ri];
    R res = row_residual(r, bd, bodies) + r.reg * imp[ri] + r.bias;
    R delta = -res / r.diag;
    R nf = imp[ri] + delta;
    R proj = nf < R(0) ? R(0) : nf;
    delta = proj - imp[ri];
    imp[ri] = proj;
    apply_impulse(r, delta, bd, bodies, iinv);
  };
  auto step_pair = [&](int ri, R h01) {  // solver.rs:1476-1518
    int rj = ri + 1;
    R res_i = row_residual(rows[ri], bd, bodies) + rows[ri].reg * imp[ri] + rows[ri].bias;
    R res_j = row_residual(rows[rj], bd, bodies) + rows[rj].reg * imp[rj] + rows[rj].bias;
    R h00 = rows[ri].diag, h11 = rows[rj].diag;
    R det = h00 * h11 - h01 * h01;
    if (det <= R(0)) { step_nonneg(ri); step_nonneg(rj); return; }
    R di = (-res_i * h11 + h01 * res_j) / det;
    R dj = (h01 * res_i - h00 * res_j) / det;
    R ni = imp[ri] + di, nj = imp[rj] + dj;
    R new_i, new_j;
    if (ni >= R(0) && nj >= R(0)) { new_i = ni; new_j = nj; }
    else if (ni < R(0) && nj < R(0)) { new_i = R(0); new_j = R(0); }
    else if (ni < R(0)) { new_i = R(0); new_j = cmax(imp[rj] - res_j / h11, R(0)); }
    else { new_i = cmax(imp[ri] - res_i / h00, R(0)); new_j = R(0); }
    R ai = new_i - imp[ri], aj = new_j - imp[rj];
    imp[ri] = new_i; imp[rj] = new_j;
    apply_impulse(rows[ri], ai, bd, bodies, iinv);
    apply_impulse(rows[rj], aj, bd, bodies, iinv);
  };
  auto step_cap = [&](int ri, R cap) {  // pgs_step_scalar_cap (solver.rs:1561-1579)
    const Row<R>& r = rows[ri];
    R res = row_residual(r, bd, bodies) + r.reg * imp[ri] + r.bias;
    R delta = -res / r.diag;
    R nf = imp[ri] + delta;
    R proj = nf > cap ? cap : (nf < -cap ? -cap : nf);  // project_pyramidal
    delta = proj - imp[ri];
    imp[ri] = proj;
    apply_impulse(r, delta, bd, bodies, iinv);
  };
  auto step_cone = [&](int r1, int r2, R cap, R mu1, R mu2) {  // pgs_step_pair_cone (solver.rs:1620-1676)
    if (sys.cone == 0) { step_cap(r1, mu1 * cap); step_cap(r2, mu2 * cap); return; }
    R res1 = row_residual(rows[r1], bd, bodies) + rows[r1].reg * imp[r1] + rows[r1].bias;
    R res2 = row_residual(rows[r2], bd, bodies) + rows[r2].reg * imp[r2] + rows[r2].bias;
    R f1 = imp[r1] - res1 / rows[r1].diag;
    R f2 = imp[r2] - res2 / rows[r2].diag;
    // project_elliptic (solver.rs:398-411); the two coefficients are equal
    // here (isotropic friction), so project_elliptic_axes is not reached
    R p1 = R(0), p2 = R(0);
    if (cap > R(0) && mu1 > R(0)) {
      const R c = mu1 * cap;
      const R mag2 = f1 * f1 + f2 * f2;
      if (mag2 <= c * c) { p1 = f1; p2 = f2; }
      else { const R sc = c / Sc<R>::sqrt(mag2); p1 = f1 * sc; p2 = f2 * sc; }
    }
    R d1 = p1 - imp[r1], d2 = p2 - imp[r2];
    imp[r1] = p1; imp[r2] = p2;
    apply_impulse(rows[r1], d1, bd, bodies, iinv);
    apply_impulse(rows[r2], d2, bd, bodies, iinv);
  };
  // solver.rs:1085-1200: per contact the normal row, then the pyramidal
  // pairs, or the tangent pair under the cone, torsion and the rolling pair,
  // every cap from the just-updated normal impulse
  for (int it = 0; it < iterations; ++it) {
    for (const FreePC<R>& pc : sys.pcs) {
      step_nonneg(pc.start);
      if (sys.facets(pc)) { step_pair(pc.start, pc.h01a); step_pair(pc.start + 2, pc.h01b); }
      else if (pc.condim >= 3) {
        const R cap = imp[pc.start];
        step_cone(pc.start + 1, pc.start + 2, cap, pc.mu, pc.mu);
        if (pc.condim >= 4) step_cap(pc.start + 3, pc.mu_t * cap);
        if (pc.condim >= 6) step_cone(pc.start + 4, pc.start + 5, cap, pc.mu_r, pc.mu_r);
      }
    }
  }
  free_row_wrenches(sys, imp, dt, wrenches);
  if (impulses_out) *impulses_out = imp;
  if (row_contact_out) free_row_contacts(sys, row_contact_out);
}

// --------------------------------------------------------------------------
// World
// --------------------------------------------------------------------------
enum SolverMode { M_PENALTY = 0, M_PGS = 1, M_NEWTON = 2 };

template <class R> struct World {
  R dt = R(0.005);
  Vec3<R> gravity = Vec3<R>(0, 0, R(-9.81));
  int solver_mode = M_PGS;
  int iterations = 20;
  int cone = 0;  // SolverConfig::cone: 0 pyramidal, 1 elliptic
  int integrator = 1;  // 0: RK4 (newt's default), 1: semi-implicit Euler (world.rs:76-84)
  std::vector<Body<R>> bodies;
  std::vector<Tree<R>> trees;
  std::vector<Geom<R>> geoms;
  std::vector<char> disabled_self_collision;  // per tree: 1 = in-tree pairs skipped
  // World::pair_list (world.rs:136-139): explicit pairs, collided in order,
  // past the filters
  bool has_pair_list = false;
  std::vector<std::pair<int, int>> pair_list;

  // world.rs:1042-1069 (naive pairs; the contact set equals the broadphase's).
  void auto_pairs(std::vector<std::pair<int, int>>& out) const {
    out.clear();
    if (has_pair_list) { out = pair_list; return; }
    int n = (int)geoms.size();
    for (int a = 0; a < n; ++a)
      for (int b = a + 1; b < n; ++b) {
        const Geom<R>& A = geoms[a]; const Geom<R>& B = geoms[b];
        int ka = A.att_kind(), kb = B.att_kind();
        bool same = ka == kb && (ka == 0 || (ka == 1 && A.body == B.body) || (ka == 2 && A.tree == B.tree && A.link == B.link));
        if (same) continue;
        if (!((A.group & B.mask) != 0u && (B.group & A.mask) != 0u)) continue;
        if (ka == 2 && kb == 2 && A.tree == B.tree && A.tree < (int)disabled_self_collision.size() && disabled_self_collision[A.tree]) continue;
        out.push_back({a, b});
      }
  }

  void geom_poses(std::vector<Pose<R>>& poses) const {
    std::vector<std::vector<Pose<R>>> tp(trees.size());
    for (size_t t = 0; t < trees.size(); ++t) forward_kinematics(trees[t], tp[t]);
    poses.resize(geoms.size());
    for (size_t i = 0; i < geoms.size(); ++i) {
      const Geom<R>& g = geoms[i];
      Vec3<R> pp; Quat<R> po;
      if (g.att_kind() == 0) { poses[i] = {g.local_pos, g.local_ori}; continue; }
      if (g.att_kind() == 1) { pp = bodies[g.body].pos; po = bodies[g.body].ori; }
      else { pp = tp[g.tree][g.link].p; po = tp[g.tree][g.link].o; }
      poses[i] = {pp + po.rotate(g.local_pos), po * g.local_ori};
    }
  }

  void detect_contacts(std::vector<Contact<R>>& out) const {  // world.rs:2476-2515
    std::vector<std::pair<int, int>> pairs;
    auto_pairs(pairs);
    std::vector<Pose<R>> poses;
    geom_poses(poses);
    out.clear();
    for (auto& pr : pairs) {
      CBuf<R> b = narrow_phase(pr.first, geoms[pr.first], poses[pr.first], pr.second, geoms[pr.second], poses[pr.second]);
      for (int k = 0; k < b.len; ++k) out.push_back(b.c[k]);
    }
  }

  // Hook for the tree-contact solve (filled in by newt_treecontact.hpp).
  std::vector<std::vector<R>> tree_qfrc;        // per tree, nv
  std::vector<Wrench<R>> tree_body_wrenches;    // per free body

  void step();  // defined after the tree-contact solver
  void step_bodies_rk4(bool solver, const std::vector<Contact<R>>& free_contacts);
};

}  // namespace oracle
