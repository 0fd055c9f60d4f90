// Oracle (test infrastructure only): the joint tree-contact solve of newt's
// World::step, for contacts between tree links and static or free-body
// geoms: pyramidal condim-3 facets, condim 1, and the general rows (normal,
// tangents, torsion, rolling) of condim 3 under the elliptic cone and of
// condim 4 and 6, with PGS or Newton.  Never linked into the shipped
// library.  Free bodies' own rolling rows (Body::rolling_friction) are not
// restated.
//
// Sources (paths inside hwang2409/tooling):
//   newt/src/solver.rs:2805-3366  solve_tree_contacts
//   newt/src/solver.rs:3401-3429  contact_row_directions
//   newt/src/solver.rs:3441-3470  contact_friction_axes (isotropic branch)
//   newt/src/solver.rs:3537-3600  world_jacobian_for_side
//   newt/src/solver.rs:3602-3622  tree_free_velocity_delta
//   newt/src/solver.rs:3624-3717  world_current_velocity, world_free_velocity,
//                                 world_velocity_from_delta
//   newt/src/solver.rs:3719-3797  tree_body_invweight0, tree_contact_diag_approx
//   newt/src/solver.rs:3799-3862  apply_world_impulse, world_pgs_non_negative
//   newt/src/solver.rs:3863-3874  world_pgs_scalar
//   newt/src/solver.rs:3973-4003  world_pgs_pair (pyramidal caps, elliptic)
//   newt/src/solver.rs:3268-3330  the PGS sweep over contact blocks
//   newt/src/solver.rs:398-411, 441-449  project_elliptic, project_pyramidal
//   newt/src/solver.rs:1960-1974  contact_regularization_from_diag
//   newt/src/newton.rs:275-620    NewtonSystem::solve, project,
//                                 exact_pyramidal_line_search (non-negative
//                                 projections: under Newton, which takes the
//                                 pyramidal cone, the general rows' only
//                                 projection is the normal row's,
//                                 solver.rs:3164-3196)
//   newt/src/jacobian.rs:38-120   point_jacobian
// Every sum runs in newt's order so the float mirror matches byte for byte.
#pragma once
#include <algorithm>
#include <cmath>
#include <stdexcept>
#include "newt_world.hpp"

namespace oracle {

// One side of a row: a free body's Jacobian, or a tree's J^T direction.
template <class R> struct TComp {
  int body = -1;             // free-body component
  int tree = -1, link = -1;  // tree component
  Vec3<R> lin, ang;          // body: Jacobian rows; tree: wrench axes
  std::vector<R> coef;       // tree: generalised coefficients (nv)
};
template <class R> struct TRow { std::vector<TComp<R>> comps; R reg = R(0), diag = R(0), bias = R(0); };
template <class R> struct TBlock {
  int contact, start, condim; SolRef<R> sr; SolImp<R> si; R pen, mu;
  R mu_t = R(0), mu_r = R(0);  // combine_torsional_friction, combine_rolling_friction (min)
  bool facets = true;          // pyramidal condim 3: the four facet rows
  int nrows = 4;
};

template <class R> Vec3<R> unit_axis(int k) { return Vec3<R>(R(k == 0), R(k == 1), R(k == 2)); }

// jacobian.rs:38-120 (world-frame columns in the tree's nv layout).
template <class R>
void point_jacobian(const Tree<R>& t, const std::vector<Pose<R>>& poses, int link, Vec3<R> point_local,
                    std::vector<Vec3<R>>& trans, std::vector<Vec3<R>>& rot) {
  const Vec3<R> point = poses[link].p + poses[link].o.rotate(point_local);
  trans.assign(t.nv(), Vec3<R>());
  rot.assign(t.nv(), Vec3<R>());
  std::vector<int> chain;
  for (int i = link; i >= 0; i = t.links[i].parent) chain.push_back(i);
  std::reverse(chain.begin(), chain.end());
  for (int i : chain) {
    const Link<R>& L = t.links[i];
    const int v = t.v_off[i];
    switch (L.type) {
      case J_FREE: {
        const Vec3<R> r = point - poses[i].p;
        for (int k = 0; k < 3; ++k) {
          const Vec3<R> aw = poses[i].o.rotate(unit_axis<R>(k));
          rot[v + k] = aw;
          trans[v + k] = aw.cross(r);
        }
        for (int k = 0; k < 3; ++k) trans[v + 3 + k] = poses[i].o.rotate(unit_axis<R>(k));
        break;
      }
      case J_HINGE: {
        const Pose<R>& P = poses[L.parent];
        const Vec3<R> jw = P.p + P.o.rotate(L.jp_pos);
        const Vec3<R> aw = P.o.rotate(L.axis);
        rot[v] = aw;
        trans[v] = aw.cross(point - jw);
        break;
      }
      case J_SLIDE: trans[v] = poses[L.parent].o.rotate(L.axis); break;
      case J_BALL: {
        const Pose<R>& P = poses[L.parent];
        const Vec3<R> jw = P.p + P.o.rotate(L.jp_pos);
        for (int k = 0; k < 3; ++k) {
          const Vec3<R> aw = poses[i].o.rotate(unit_axis<R>(k));
          rot[v + k] = aw;
          trans[v + k] = aw.cross(point - jw);
        }
        break;
      }
      default: break;
    }
  }
}

// world_jacobian_for_side (solver.rs:3537-3600): a linear row along `dir`
// at the contact point, or an angular one (torsion, rolling) about `dir`.
template <class R>
bool side_jacobian(const World<R>& w, const Geom<R>& g, R sign, Vec3<R> cpos, Vec3<R> dir,
                   const std::vector<std::vector<Pose<R>>>& tp, TComp<R>* out, bool angular = false) {
  const int kind = g.att_kind();
  if (kind == 0) return false;
  TComp<R> c;
  if (kind == 1) {
    const Body<R>& b = w.bodies[g.body];
    const Vec3<R> arm = cpos - b.pos;
    c.body = g.body;
    c.lin = angular ? Vec3<R>() : dir * sign;
    c.ang = angular ? dir * sign : arm.cross(dir) * sign;
  } else {
    const Pose<R>& P = tp[g.tree][g.link];
    const Vec3<R> local = P.o.inverse_rotate(cpos - P.p);
    std::vector<Vec3<R>> tr, rt;
    point_jacobian(w.trees[g.tree], tp[g.tree], g.link, local, tr, rt);
    c.tree = g.tree;
    c.link = g.link;
    const std::vector<Vec3<R>>& src = angular ? rt : tr;
    c.coef.resize(src.size());
    for (size_t s = 0; s < src.size(); ++s) c.coef[s] = src[s].dot(dir) * sign;
    c.lin = angular ? Vec3<R>() : dir * sign;
    c.ang = angular ? dir * sign : (cpos - P.p).cross(dir * sign);
  }
  *out = c;
  return true;
}

template <class R> R sum_products(const std::vector<R>& a, const std::vector<R>& b) {
  R s = R(0);
  for (size_t i = 0; i < a.size() && i < b.size(); ++i) s += a[i] * b[i];
  return s;
}

// tree_body_invweight0 (solver.rs:3719-3754): mean inverse weight of the
// link's COM over the three world axes, translation and rotation.
template <class R>
void tree_body_invweight0(const Tree<R>& t, const std::vector<Pose<R>>& poses, int link, const std::vector<R>& factor,
                          R* tr_out, R* rot_out) {
  std::vector<Vec3<R>> jt, jr;
  point_jacobian(t, poses, link, Vec3<R>(), jt, jr);
  const int nv = t.nv();
  R translation = R(0), rotation = R(0);
  std::vector<R> lin(nv), ang(nv), lr(nv), ar(nv);
  for (int axis = 0; axis < 3; ++axis) {
    for (int s = 0; s < nv; ++s) {
      lin[s] = axis == 0 ? jt[s].x : axis == 1 ? jt[s].y : jt[s].z;
      ang[s] = axis == 0 ? jr[s].x : axis == 1 ? jr[s].y : jr[s].z;
    }
    cholesky_solve(factor, nv, lin.data(), lr.data());
    cholesky_solve(factor, nv, ang.data(), ar.data());
    translation += sum_products(lin, lr);
    rotation += sum_products(ang, ar);
  }
  *tr_out = translation / R(3);
  *rot_out = rotation / R(3);
}

// newton.rs:386-433 for non-negative projections.
template <class R> void project_nonneg(std::vector<R>& x, const std::vector<int>& nonneg) {
  for (int i : nonneg) if (x[i] < R(0)) x[i] = R(0);
}
template <class R> void mat_vec(const std::vector<R>& m, const std::vector<R>& v, std::vector<R>& out) {
  const size_t n = v.size();
  out.assign(n, R(0));
  for (size_t i = 0; i < n; ++i)
    for (size_t j = 0; j < n; ++j) out[i] += m[i * n + j] * v[j];
}
template <class R> R quad_cost(const std::vector<R>& H, const std::vector<R>& b, const std::vector<R>& x) {
  std::vector<R> hx;
  mat_vec(H, x, hx);
  return R(0.5) * sum_products(x, hx) + sum_products(b, x);
}
template <class R> void quad_grad(const std::vector<R>& H, const std::vector<R>& b, const std::vector<R>& x, std::vector<R>& g) {
  mat_vec(H, x, g);
  for (size_t i = 0; i < g.size(); ++i) g[i] += b[i];
}
template <class R>
void affine_point(const std::vector<R>& x, const std::vector<R>& d, const std::vector<int>& nonneg, R alpha,
                  std::vector<R>& p) {
  p.resize(x.size());
  for (size_t i = 0; i < x.size(); ++i) p[i] = x[i] + alpha * d[i];
  project_nonneg(p, nonneg);
}

// newton.rs:435-556 (exact_pyramidal_line_search).
template <class R>
void line_search(const std::vector<R>& H, const std::vector<R>& b, const std::vector<int>& nonneg,
                 const std::vector<R>& x, const std::vector<R>& d, R current, R* alpha_out, R* cost_out) {
  std::vector<R> br{R(0), R(1)};
  for (int i : nonneg) {  // add_root (newton.rs:558-566)
    const R slope = d[i];
    if (slope == R(0)) continue;
    const R a = -x[i] / slope;
    if (a > R(0) && a < R(1)) br.push_back(a);
  }
  std::stable_sort(br.begin(), br.end());
  std::vector<R> breaks;
  for (R v : br)
    if (breaks.empty() || !(rabs(v - breaks.back()) <= R(1e-7))) breaks.push_back(v);
  std::vector<R> cand = breaks;
  std::vector<R> left, right, slope, zmid, lg, hs;
  for (size_t k = 0; k + 1 < breaks.size(); ++k) {
    const R lo = breaks[k], hi = breaks[k + 1];
    if (hi - lo <= R(1e-7)) continue;
    const R mid = R(0.5) * (lo + hi);
    const R eps = (hi - lo) * R(1e-4);
    const R la = std::max(mid - eps, lo);
    const R ra = std::min(mid + eps, hi);
    affine_point(x, d, nonneg, la, left);
    affine_point(x, d, nonneg, ra, right);
    const R span = ra - la;
    if (span <= R(0)) continue;
    const R scale = R(1) / span;
    slope.resize(x.size());
    for (size_t i = 0; i < x.size(); ++i) slope[i] = (right[i] - left[i]) * scale;
    affine_point(x, d, nonneg, mid, zmid);
    quad_grad(H, b, zmid, lg);
    mat_vec(H, slope, hs);
    const R den = sum_products(slope, hs);
    const R num = sum_products(lg, slope);
    R opt = mid;
    if (den > R(0)) opt = std::min(std::max(mid - num / den, lo), hi);
    cand.push_back(opt);
  }
  R best_a = R(0), best_c = current;
  std::vector<R> p;
  for (R a : cand) {
    affine_point(x, d, nonneg, a, p);
    const R c = quad_cost(H, b, p);
    if (c < best_c) { best_c = c; best_a = a; }
  }
  *alpha_out = best_a;
  *cost_out = best_c;
}

// NewtonSystem::solve (newton.rs:275-339).  Returns false when H is not PD.
template <class R>
bool newton_solve(const std::vector<R>& H, const std::vector<R>& b, const std::vector<int>& nonneg, int max_it,
                  R tol, std::vector<R>& x, int* iters_out = nullptr) {
  const int n = (int)b.size();
  x.assign(n, R(0));
  if (iters_out) *iters_out = 0;
  if (max_it == 0) return true;
  std::vector<R> L;
  if (!cholesky(H, n, L)) return false;
  R current = quad_cost(H, b, x);
  std::vector<R> g, neg(n), d(n);
  for (int it = 0; it < max_it; ++it) {
    quad_grad(H, b, x, g);
    for (int i = 0; i < n; ++i) neg[i] = -g[i];
    cholesky_solve(L, n, neg.data(), d.data());
    if (sum_products(g, d) >= R(0)) break;
    R alpha, next;
    line_search(H, b, nonneg, x, d, current, &alpha, &next);
    if (alpha <= R(0) || current - next <= tol * (R(1) + rabs(current))) break;
    for (int i = 0; i < n; ++i) x[i] += alpha * d[i];
    project_nonneg(x, nonneg);
    current = next;
    if (iters_out) *iters_out = it + 1;
  }
  return true;
}

// solve_free_body_newton_impulses (solver.rs:1295-1407) for pyramidal
// condim-3 and condim-1 contacts between free bodies: the dense response
// matrix (column j holds every row's residual after a unit impulse on row
// j, solver.rs:1303-1316), H = A + diag(R), and NewtonSystem::solve with a
// non-negative projection on every facet row and normal row, at most
// max(iterations, 1) iterations, cost tolerance 1e-7.  Returns false when H
// is not positive definite (newt panics there).
template <class R>
bool solve_free_bodies_newton(const std::vector<Body<R>>& bodies, const std::vector<Geom<R>>& geoms,
                              const std::vector<Contact<R>>& contacts, Vec3<R> gravity, R dt, int iterations,
                              std::vector<Wrench<R>>& wrenches, std::vector<R>* impulses_out = nullptr,
                              std::vector<int>* row_contact_out = nullptr) {
  const int nb = (int)bodies.size();
  wrenches.assign(nb, Wrench<R>{Vec3<R>(), Vec3<R>()});
  if (impulses_out) impulses_out->clear();
  if (row_contact_out) row_contact_out->clear();
  if (contacts.empty() || dt <= R(0)) return true;
  FreeSystem<R> sys;
  assemble_free_rows(bodies, geoms, contacts, gravity, dt, sys);
  const int n = (int)sys.rows.size();
  if (n == 0) return true;
  std::vector<R> H((size_t)n * n, R(0));
  std::vector<BDelta<R>> resp(nb);
  for (int j = 0; j < n; ++j) {
    for (auto& d : resp) d = BDelta<R>{Vec3<R>(), Vec3<R>()};
    apply_impulse(sys.rows[j], R(1), resp, bodies, sys.iinv);
    for (int i = 0; i < n; ++i) H[(size_t)i * n + j] = row_residual(sys.rows[i], resp, bodies);
  }
  for (int i = 0; i < n; ++i) H[(size_t)i * n + i] += sys.rows[i].reg;
  std::vector<int> nonneg;
  for (const FreePC<R>& pc : sys.pcs)
    for (int k = 0; k < (pc.condim == 3 ? 4 : 1); ++k) nonneg.push_back(pc.start + k);
  std::vector<R> bias(n), imp;
  for (int i = 0; i < n; ++i) bias[i] = sys.rows[i].bias;
  if (!newton_solve(H, bias, nonneg, iterations > 1 ? iterations : 1, R(1e-7), imp)) return false;
  free_row_wrenches(sys, imp, dt, wrenches);
  if (impulses_out) *impulses_out = imp;
  if (row_contact_out) free_row_contacts(sys, row_contact_out);
  return true;
}

// solve_tree_contacts (solver.rs:2805-3366).  `implicit`: the Euler form
// (factors of M + dt*B, free velocity from the implicit ABA); otherwise the
// RK4 form (factors of M, explicit ABA).  Writes w.tree_qfrc and
// w.tree_body_wrenches; the per-row impulses go to `impulses_out` if given.
template <class R>
void solve_tree_contacts(World<R>& w, const std::vector<Contact<R>>& contacts, bool use_newton, bool implicit,
                         std::vector<R>* impulses_out = nullptr, std::vector<Wrench<R>>* link_wrenches_out = nullptr,
                         std::vector<R>* normal_forces_out = nullptr) {
  if (impulses_out) impulses_out->clear();
  // the sensor inputs (solver.rs:3334-3364): each tree link's contact wrench
  // (world force and torque about its COM) and each contact's normal force
  if (link_wrenches_out && !w.trees.empty())
    link_wrenches_out->assign(w.trees[0].links.size(), Wrench<R>{Vec3<R>(), Vec3<R>()});
  if (normal_forces_out) normal_forces_out->assign(contacts.size(), R(0));
  if (contacts.empty() || w.dt <= R(0) || w.trees.empty()) return;
  const R dt = w.dt;
  const size_t ntr = w.trees.size(), nbd = w.bodies.size();
  std::vector<std::vector<Pose<R>>> tp(ntr);
  for (size_t t = 0; t < ntr; ++t) forward_kinematics(w.trees[t], tp[t]);
  std::vector<Mat3<R>> iinv(nbd);
  for (size_t i = 0; i < nbd; ++i) {
    const Mat3<R> r = w.bodies[i].ori.to_mat3();
    iinv[i] = r * w.bodies[i].inertia_inv * r.transpose();
  }
  std::vector<std::vector<R>> factor(ntr), dfactor(ntr), vfree(ntr);
  for (size_t t = 0; t < ntr; ++t) {
    const Tree<R>& tree = w.trees[t];
    const int nv = tree.nv();
    if (nv == 0) continue;
    std::vector<R> M;
    if (implicit) implicit_mass_matrix(tree, dt, M); else mass_matrix(tree, M);
    if (!cholesky(M, nv, factor[t])) throw std::runtime_error("tree contact solve: mass matrix is not positive definite");
    mass_matrix(tree, M);
    if (!cholesky(M, nv, dfactor[t])) throw std::runtime_error("tree diagApprox: mass matrix is not positive definite");
    Tree<R> free_tree = tree;  // tree_free_velocity_delta
    free_tree.disable_penalty_limits = true;
    std::vector<Pose<R>> fp;
    forward_kinematics(free_tree, fp);
    std::vector<Wrench<R>> ext(free_tree.links.size(), Wrench<R>{Vec3<R>(), Vec3<R>()});
    std::vector<R> qdd;
    aba(free_tree, fp, w.gravity, ext, implicit ? dt : R(0), qdd);
    vfree[t].resize(qdd.size());
    for (size_t s = 0; s < qdd.size(); ++s) vfree[t][s] = qdd[s] * dt;
  }
  // rows and blocks, in contact order
  std::vector<TRow<R>> rows;
  std::vector<TBlock<R>> blocks;
  for (int ci = 0; ci < (int)contacts.size(); ++ci) {
    const Contact<R>& c = contacts[ci];
    const Geom<R>& ga = w.geoms[c.ga];
    const Geom<R>& gb = w.geoms[c.gb];
    if (ga.att_kind() != 2 && gb.att_kind() != 2) continue;
    const R pen = c.pen - c.gap;
    if (pen <= R(0)) continue;
    const SolRef<R> sr = combine_solref(ga.solref, gb.solref);
    const SolImp<R> si = combine_solimp(ga.solimp, gb.solimp);
    const int condim = ga.condim < gb.condim ? ga.condim : gb.condim;
    const R mu = cmin(ga.friction, gb.friction);
    if (condim != 1 && condim != 3 && condim != 4 && condim != 6)
      throw std::runtime_error("tree contacts: condim must be 1, 3, 4 or 6");
    Vec3<R> t1, t2u;
    tangent_basis(c.n, &t1, &t2u);
    const Vec3<R> t2 = c.n.cross(t1);  // isotropic contact_friction_axes
    // contact_row_directions (solver.rs:3401-3429): direction, angular
    const bool facets = w.cone == 0 && condim == 3;
    std::vector<std::pair<Vec3<R>, bool>> dirs;
    if (facets) {
      dirs = {{c.n + t1 * mu, false}, {c.n - t1 * mu, false}, {c.n + t2 * mu, false}, {c.n - t2 * mu, false}};
    } else {
      dirs.push_back({c.n, false});
      if (condim >= 3) { dirs.push_back({t1, false}); dirs.push_back({t2, false}); }
      if (condim >= 4) dirs.push_back({c.n, true});
      if (condim >= 6) { dirs.push_back({t1, true}); dirs.push_back({t2, true}); }
    }
    std::vector<TRow<R>> brows;
    bool dynamic = false;
    for (const auto& dir : dirs) {
      TRow<R> r;
      TComp<R> comp;
      if (side_jacobian(w, ga, R(1), c.pos, dir.first, tp, &comp, dir.second)) r.comps.push_back(comp);
      if (side_jacobian(w, gb, R(-1), c.pos, dir.first, tp, &comp, dir.second)) r.comps.push_back(comp);
      if (!r.comps.empty()) dynamic = true;  // every body or non-mocap tree side is dynamic
      brows.push_back(r);
    }
    if (!dynamic) continue;
    TBlock<R> bk{ci, (int)rows.size(), condim, sr, si, pen, mu};
    bk.mu_t = cmin(ga.torsional_friction, gb.torsional_friction);
    bk.mu_r = cmin(ga.rolling_friction, gb.rolling_friction);
    bk.facets = facets;
    bk.nrows = (int)dirs.size();
    blocks.push_back(bk);
    for (auto& r : brows) rows.push_back(r);
  }
  const int n = (int)rows.size();
  if (n == 0) return;
  // response A = J M^-1 J^T, column by column (apply_world_impulse)
  std::vector<R> A((size_t)n * n, R(0));
  for (int col = 0; col < n; ++col) {
    std::vector<Vec3<R>> bdv(nbd), bdw(nbd);
    std::vector<std::vector<R>> td(ntr);
    for (size_t t = 0; t < ntr; ++t) td[t].assign(w.trees[t].nv(), R(0));
    for (const TComp<R>& cp : rows[col].comps) {
      if (cp.body >= 0) {
        const Body<R>& b = w.bodies[cp.body];
        const Vec3<R> force = cp.lin * R(1), torque = cp.ang * R(1);
        const Vec3<R> av = iinv[cp.body] * torque;
        bdv[cp.body] += force / b.mass;
        bdw[cp.body] += b.ori.inverse_rotate(av);
      }
      if (cp.tree >= 0) {
        std::vector<R> gi(cp.coef.size()), resp(cp.coef.size());
        for (size_t s = 0; s < gi.size(); ++s) gi[s] = cp.coef[s] * R(1);
        cholesky_solve(factor[cp.tree], (int)gi.size(), gi.data(), resp.data());
        for (size_t s = 0; s < resp.size(); ++s) td[cp.tree][s] += resp[s];
      }
    }
    for (int r = 0; r < n; ++r) {
      R v = R(0);
      for (const TComp<R>& cp : rows[r].comps) {
        R bv = R(0), tv = R(0);
        if (cp.body >= 0) bv = cp.lin.dot(bdv[cp.body]) + cp.ang.dot(w.bodies[cp.body].ori.rotate(bdw[cp.body]));
        if (cp.tree >= 0) tv = sum_products(cp.coef, td[cp.tree]);
        v += bv + tv;
      }
      A[(size_t)r * n + col] = v;
    }
  }
  // regularisation, diagonal and bias per row
  for (const TBlock<R>& bk : blocks) {
    const bool pyr3 = bk.facets;
    const int nr = bk.nrows;
    for (int k = 0; k < nr; ++k) {
      TRow<R>& row = rows[bk.start + k];
      const R imp = impedance_at(-bk.pen, R(0), bk.si);
      R tr = R(0), ro = R(0);  // tree_contact_diag_approx
      for (const TComp<R>& cp : row.comps) {
        if (cp.body >= 0) {
          if (!(cp.lin == Vec3<R>())) tr += R(1) / w.bodies[cp.body].mass;
          else ro += cp.ang.dot(iinv[cp.body] * cp.ang);
        }
        if (cp.tree >= 0) {
          R bt, br;
          tree_body_invweight0(w.trees[cp.tree], tp[cp.tree], cp.link, dfactor[cp.tree], &bt, &br);
          if (!(cp.lin == Vec3<R>())) tr += bt; else ro += br;
        }
      }
      const R dapprox = pyr3 ? tr * (R(1) + bk.mu * bk.mu) : tr + ro;
      const R base = (R(1) - imp) / imp * dapprox;  // contact_regularization_from_diag
      row.reg = pyr3 ? R(2) * bk.mu * bk.mu * base : base;
      row.diag = A[(size_t)(bk.start + k) * n + bk.start + k] + row.reg;
      R vel = R(0), vf = R(0);
      for (const TComp<R>& cp : row.comps) {
        R bv = R(0), tv = R(0), bf = R(0), tf = R(0);
        if (cp.body >= 0) {
          const Body<R>& b = w.bodies[cp.body];
          bv = cp.lin.dot(b.vel) + cp.ang.dot(b.ori.rotate(b.omega_body));
          bf = cp.lin.dot(w.gravity * dt);
        }
        if (cp.tree >= 0) {
          tv = sum_products(cp.coef, w.trees[cp.tree].qdot);
          tf = sum_products(cp.coef, vfree[cp.tree]);
        }
        vel += bv + tv;
        vf += bf + tf;
      }
      const R position = (pyr3 || k == 0) ? -bk.pen : R(0);  // facets and the normal row
      const R aref = reference_accel(position, vel, safe_solref(bk.sr, dt), bk.si);
      row.bias = vf - aref * dt;
    }
  }
  std::vector<R> imp(n, R(0));
  if (use_newton) {
    std::vector<R> H = A;
    for (int i = 0; i < n; ++i) H[(size_t)i * n + i] += rows[i].reg;
    // the normal row, or the four facets, non-negative; the general rows'
    // friction rows carry no projection under the pyramidal cone
    std::vector<int> nonneg;
    for (const TBlock<R>& bk : blocks)
      for (int k = 0; k < (bk.facets ? 4 : 1); ++k) nonneg.push_back(bk.start + k);
    std::vector<R> Ltest;
    bool zero_mu = false;
    for (const TBlock<R>& bk : blocks) zero_mu = zero_mu || (bk.facets && bk.mu == R(0));
    if (zero_mu && !cholesky(H, n, Ltest)) {  // solver.rs:3215-3232
      R scale = R(0);
      for (R v : H) scale = std::max(scale, rabs(v));
      const R pivot = std::max(scale * R(1e-6), R(1e-7));
      for (int i = 0; i < n; ++i) H[(size_t)i * n + i] += pivot;
    }
    std::vector<R> bias(n);
    for (int i = 0; i < n; ++i) bias[i] = rows[i].bias;
    const int max_it = w.iterations > 1 ? w.iterations : 1;
    if (!newton_solve(H, bias, nonneg, max_it, R(1e-7), imp))
      throw std::runtime_error("Newton tree contact solve: Hessian is not positive definite");
  } else {
    // world_pgs_residual (solver.rs:3838-3849) plus the row's own reg term
    auto resid = [&](int i) {
      R s = R(0);
      for (int col = 0; col < n; ++col) s += A[(size_t)i * n + col] * imp[col];
      return (rows[i].bias + s) + rows[i].reg * imp[i];
    };
    auto nonneg_step = [&](int i) {  // world_pgs_non_negative
      const R p = imp[i] - resid(i) / rows[i].diag;
      imp[i] = p < R(0) ? R(0) : p;
    };
    auto scalar_step = [&](int i, R cap) {  // world_pgs_scalar, project_pyramidal
      const R f = imp[i] - resid(i) / rows[i].diag;
      imp[i] = f > cap ? cap : (f < -cap ? -cap : f);
    };
    auto pair_step = [&](int i, int j, R mu_pair, R normal) {  // world_pgs_pair, isotropic
      if (w.cone == 0) { scalar_step(i, mu_pair * normal); scalar_step(j, mu_pair * normal); return; }
      const R ri = resid(i), rj = resid(j);
      const R fi = imp[i] - ri / rows[i].diag, fj = imp[j] - rj / rows[j].diag;
      R pi = R(0), pj = R(0);  // project_elliptic
      if (normal > R(0) && mu_pair > R(0)) {
        const R cap = mu_pair * normal;
        const R mag2 = fi * fi + fj * fj;
        if (mag2 <= cap * cap) { pi = fi; pj = fj; }
        else { const R sc = cap / Sc<R>::sqrt(mag2); pi = fi * sc; pj = fj * sc; }
      }
      imp[i] = pi;
      imp[j] = pj;
    };
    for (int it = 0; it < w.iterations; ++it)
      for (const TBlock<R>& bk : blocks) {
        const int nrm = bk.start;
        nonneg_step(nrm);
        if (bk.facets) {
          for (int k = 1; k < 4; ++k) nonneg_step(nrm + k);
        } else if (bk.condim >= 3) {
          pair_step(nrm + 1, nrm + 2, bk.mu, imp[nrm]);
          if (bk.condim >= 4) scalar_step(nrm + 3, bk.mu_t * imp[nrm]);
          if (bk.condim >= 6) pair_step(nrm + 4, nrm + 5, bk.mu_r, imp[nrm]);
        }
      }
  }
  if (impulses_out) *impulses_out = imp;
  if (normal_forces_out)
    for (const TBlock<R>& bk : blocks) {
      R fn = R(0);
      if (bk.facets) for (int k = 0; k < 4; ++k) fn += imp[bk.start + k];
      else fn = imp[bk.start];
      (*normal_forces_out)[bk.contact] = fn / dt;
    }
  for (int i = 0; i < n; ++i) {
    const R force = imp[i] / dt;
    for (const TComp<R>& cp : rows[i].comps) {
      if (cp.body >= 0) {
        w.tree_body_wrenches[cp.body].f += cp.lin * force;
        w.tree_body_wrenches[cp.body].t += cp.ang * force;
      }
      if (cp.tree >= 0)
        for (size_t s = 0; s < cp.coef.size(); ++s) w.tree_qfrc[cp.tree][s] += cp.coef[s] * force;
      if (cp.tree >= 0 && link_wrenches_out) {
        (*link_wrenches_out)[cp.link].f += cp.lin * force;
        (*link_wrenches_out)[cp.link].t += cp.ang * force;
      }
    }
  }
}

}  // namespace oracle
