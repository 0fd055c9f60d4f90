// Oracle (test infrastructure only): World::step in its semi-implicit Euler
// form, plus the free-body RK4 path with zero-order-hold solver wrenches
// (used only to replay newt's RK4 solver goldens).
//
// Sources (paths inside hwang2409/tooling):
//   newt/src/world.rs:1459-1537  World::step
//   newt/src/world.rs:1705-1788  step_bodies (RK4, solver wrenches held)
//   newt/src/world.rs:3258-3271  advance_all
//   newt/src/world.rs:1790-1817  step_bodies_euler
//   newt/src/world.rs:1952-2051  step_trees_euler
//   newt/src/world.rs:2097-2152  compute_solver_wrenches
//   newt/src/world.rs:3223-3286  evaluate, clamp_velocity
#pragma once
#include "newt_world.hpp"
#include "newt_treecontact.hpp"

namespace oracle {

template <class R> struct Deriv { Vec3<R> dlin, dang; };

template <class R> Deriv<R> evaluate(const Body<R>& s, Vec3<R> g, Vec3<R> f, Vec3<R> tq) {  // world.rs:3223-3245
  Vec3<R> dlin = g + f / s.mass;
  Vec3<R> iw = s.inertia * s.omega_body;
  Vec3<R> gyro = -(s.omega_body.cross(iw));
  Vec3<R> tb = s.ori.inverse_rotate(tq);
  Vec3<R> dang = s.inertia_inv * (tb + gyro);
  return {dlin, dang};
}

// The free-body constraint solve newt's solver mode selects (world.rs:1705-1817):
// PGS (solve_free_bodies_diag_mode) or the dense Newton solve
// (solve_free_bodies_newton, solver.rs:572 -> :1295-1407).
template <class R> void solve_free_bodies(const World<R>& w, const std::vector<Contact<R>>& contacts,
                                          std::vector<Wrench<R>>& ext) {
  if (w.solver_mode == M_NEWTON) {
    if (w.cone != 0) throw std::runtime_error("Newton takes the pyramidal cone (solver.rs:89-91)");
    for (const Contact<R>& c : contacts)
      if (std::min(w.geoms[c.ga].condim, w.geoms[c.gb].condim) >= 4)
        throw std::runtime_error("the free-body Newton solve takes condim 1 and 3 here");
    if (!solve_free_bodies_newton(w.bodies, w.geoms, contacts, w.gravity, w.dt, w.iterations, ext))
      throw std::runtime_error("Newton free-body solve failed: the Hessian is not positive definite");
  } else {
    solve_free_bodies_pgs<R>(w.bodies, w.geoms, contacts, w.gravity, w.dt, w.iterations, ext, nullptr, nullptr, w.cone);
  }
}

// step_bodies (world.rs:1705-1788): the solver wrenches are computed once at
// the start state and held over the four stages; stage states start from s0
// (advance_all, world.rs:3258-3271) and keep their orientations unnormalised.
template <class R> void World<R>::step_bodies_rk4(bool solver, const std::vector<Contact<R>>& free_contacts) {
  const size_t n = bodies.size();
  std::vector<Wrench<R>> ext(n, Wrench<R>{Vec3<R>(), Vec3<R>()});
  if (solver) {
    solve_free_bodies(*this, free_contacts, ext);
    for (size_t i = 0; i < n; ++i) { ext[i].f += tree_body_wrenches[i].f; ext[i].t += tree_body_wrenches[i].t; }
  }
  struct K { Vec3<R> dp, dv; Quat<R> dq; Vec3<R> dw; };
  auto eval = [&](const Body<R>& s, size_t i) {
    Deriv<R> d = evaluate(s, gravity, ext[i].f, ext[i].t);
    return K{s.vel, d.dlin, s.ori.derivative(s.omega_body), d.dang};
  };
  auto advance = [&](const Body<R>& o, const K& k, R h) {
    Body<R> b = o;
    b.pos = o.pos + k.dp * h;
    b.vel = o.vel + k.dv * h;
    b.ori = o.ori + k.dq * h;
    b.omega_body = o.omega_body + k.dw * h;
    return b;
  };
  const std::vector<Body<R>> s0 = bodies;
  for (size_t i = 0; i < n; ++i) {
    K k1 = eval(s0[i], i);
    K k2 = eval(advance(s0[i], k1, dt * R(0.5)), i);
    K k3 = eval(advance(s0[i], k2, dt * R(0.5)), i);
    K k4 = eval(advance(s0[i], k3, dt), i);
    const R sixth = R(1.0) / R(6.0);
    Vec3<R> dp = (k1.dp + k2.dp * R(2.0) + k3.dp * R(2.0) + k4.dp) * sixth;
    Vec3<R> dv = (k1.dv + k2.dv * R(2.0) + k3.dv * R(2.0) + k4.dv) * sixth;
    Quat<R> dq = (k1.dq + k2.dq * R(2.0) + k3.dq * R(2.0) + k4.dq) * sixth;
    Vec3<R> dw = (k1.dw + k2.dw * R(2.0) + k3.dw * R(2.0) + k4.dw) * sixth;
    Body<R>& b = bodies[i];
    b.pos = s0[i].pos + dp * dt;
    b.vel = s0[i].vel + dv * dt;
    b.ori = (s0[i].ori + dq * dt).renormalize();
    b.omega_body = s0[i].omega_body + dw * dt;
  }
}

template <class R> void World<R>::step() {
  const bool solver = solver_mode == M_PGS || solver_mode == M_NEWTON;
  std::vector<Contact<R>> contacts;
  if (solver) detect_contacts(contacts);
  // Tree-involved contacts are solved jointly first (world.rs:2154-2175).
  std::vector<Contact<R>> tree_contacts, free_contacts;
  for (const Contact<R>& c : contacts) {
    bool tl = geoms[c.ga].att_kind() == 2 || geoms[c.gb].att_kind() == 2;
    (tl ? tree_contacts : free_contacts).push_back(c);
  }
  tree_qfrc.assign(trees.size(), std::vector<R>());
  for (size_t t = 0; t < trees.size(); ++t) tree_qfrc[t].assign(trees[t].nv(), R(0));
  tree_body_wrenches.assign(bodies.size(), Wrench<R>{Vec3<R>(), Vec3<R>()});
  if (solver) solve_tree_contacts(*this, tree_contacts, solver_mode == M_NEWTON, integrator == 1);
  if (integrator == 0) {
    // RK4 (world.rs:1495-1498): step_bodies, then step_trees (world.rs:1826-1945)
    // with the solver's generalised forces held over the four stages.
    if (!bodies.empty()) step_bodies_rk4(solver, free_contacts);
    for (size_t ti = 0; ti < trees.size(); ++ti) {
      Tree<R>& tree = trees[ti];
      const bool prior = tree.disable_penalty_limits;
      if (solver) {
        for (int s = 0; s < tree.nv(); ++s) tree.qfrc_applied[s] += tree_qfrc[ti][s];
        tree.disable_penalty_limits = true;
      }
      rk4_step_tree(tree, gravity, dt);
      if (solver)
        for (int s = 0; s < tree.nv(); ++s) tree.qfrc_applied[s] -= tree_qfrc[ti][s];
      tree.disable_penalty_limits = prior;
    }
    return;
  }
  // step_trees_euler (world.rs:1952-2051)
  for (size_t ti = 0; ti < trees.size(); ++ti) {
    Tree<R>& tree = trees[ti];
    bool prior = tree.disable_penalty_limits;
    std::vector<R> delta;
    if (solver) {
      delta.assign(tree.nv(), R(0));
      for (int s = 0; s < tree.nv(); ++s) delta[s] += tree_qfrc[ti][s];
      for (int s = 0; s < tree.nv(); ++s) tree.qfrc_applied[s] += delta[s];
      tree.disable_penalty_limits = true;
    }
    euler_step_tree(tree, gravity, dt);
    for (size_t s = 0; s < delta.size(); ++s) tree.qfrc_applied[s] -= delta[s];
    tree.disable_penalty_limits = prior;
  }
  // step_bodies_euler (world.rs:1790-1817)
  std::vector<Wrench<R>> ext(bodies.size(), Wrench<R>{Vec3<R>(), Vec3<R>()});
  if (solver) {
    solve_free_bodies(*this, free_contacts, ext);
    for (size_t i = 0; i < bodies.size(); ++i) { ext[i].f += tree_body_wrenches[i].f; ext[i].t += tree_body_wrenches[i].t; }
  }
  for (size_t i = 0; i < bodies.size(); ++i) {
    Body<R>& b = bodies[i];
    Deriv<R> d = evaluate(b, gravity, ext[i].f, ext[i].t);
    Vec3<R> lv = b.vel + d.dlin * dt;
    Vec3<R> av = b.omega_body + d.dang * dt;
    b.pos += lv * dt;
    b.ori = b.ori.integrate_body_angular_velocity(av, dt);
    b.vel = lv;
    b.omega_body = av;
  }
}

}  // namespace oracle
