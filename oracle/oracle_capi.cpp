// Oracle (test infrastructure only): C entry points over the C++
// restatement of newt's step, used by the CPU test suite, the GPU parity
// tests and the benchmark's CPU-baseline leg.  Never linked into the shipped
// GPU library.
//
// Worlds are described with the same `newt_model_desc` the GPU C ABI takes
// (include/newt_gpu.h), so a test builds one description and feeds both.
// `precision` 0 runs the f32 mirror of newt's arithmetic, 1 the FP64 oracle.
// `layout` 0 = MuJoCo qpos/qvel (newt/src/world.rs:519-623), 1 = newt's own
// q/qdot order (bodies: pos, quat xyzw, v_world, omega_body).
#include <atomic>
#include <chrono>
#include <cstdio>
#include <stdexcept>
#include <thread>
#include <vector>
#include <limits>

#include "../include/newt_gpu.h"
#include "newt_ccd.hpp"
#include "newt_step.hpp"

using namespace oracle;

namespace {

template <class R> Quat<R> quat_xyzw(const float* q) { return Quat<R>(q[0], q[1], q[2], q[3]); }
template <class R> Vec3<R> v3(const float* v) { return Vec3<R>(v[0], v[1], v[2]); }
template <class R> Mat3<R> m3(const float* m) { Mat3<R> o; for (int i = 0; i < 9; ++i) o.d[i] = m[i]; return o; }

template <class R> World<R> build_world(const newt_model_desc& d) {
  World<R> w;
  w.dt = d.dt;
  w.gravity = v3<R>(d.gravity);
  w.solver_mode = d.solver == NEWT_SOLVER_NEWTON ? M_NEWTON : (d.solver == NEWT_SOLVER_PGS ? M_PGS : M_PENALTY);
  w.iterations = d.iterations;
  w.cone = d.cone;
  for (int i = 0; i < d.n_bodies; ++i) {
    const newt_body_desc& b = d.bodies[i];
    w.bodies.push_back(make_body<R>(b.mass, m3<R>(b.inertia), Vec3<R>(), Quat<R>()));
  }
  if (d.n_links > 0) {
    Tree<R> t;
    for (int i = 0; i < d.n_links; ++i) {
      const newt_link_desc& L = d.links[i];
      Link<R> l;
      l.parent = L.parent; l.type = L.joint; l.axis = v3<R>(L.axis);
      l.damping = L.damping; l.armature = L.armature; l.free_damping = L.free_damping;
      l.jp_pos = v3<R>(L.jp_pos); l.jp_ori = quat_xyzw<R>(L.jp_quat);
      l.jc_pos = v3<R>(L.jc_pos); l.jc_ori = quat_xyzw<R>(L.jc_quat);
      l.mass = L.mass; l.inertia = m3<R>(L.inertia);
      t.push_link(l);
    }
    w.trees.push_back(t);
    w.disabled_self_collision.push_back(d.tree_self_collision ? 0 : 1);
  }
  if (d.pairs) {  // World::pair_list
    w.has_pair_list = true;
    for (int k = 0; k < d.n_pairs; ++k) w.pair_list.push_back({d.pairs[2 * k], d.pairs[2 * k + 1]});
  }
  for (int i = 0; i < d.n_geoms; ++i) {
    const newt_geom_desc& G = d.geoms[i];
    Geom<R> g;
    g.shape = G.shape;
    for (int k = 0; k < 3; ++k) g.size[k] = G.size[k];
    g.body = G.body; g.link = G.link; g.tree = G.link >= 0 ? 0 : -1;
    g.local_pos = v3<R>(G.local_pos); g.local_ori = quat_xyzw<R>(G.local_quat);
    g.friction = G.friction;
    g.solref.timeconst = G.solref[0]; g.solref.dampratio = G.solref[1];
    g.solimp.dmin = G.solimp[0]; g.solimp.dmax = G.solimp[1]; g.solimp.width = G.solimp[2];
    g.solimp.midpoint = G.solimp[3]; g.solimp.power = (int)G.solimp[4];
    g.margin = G.margin; g.gap = G.gap; g.condim = G.condim;
    g.torsional_friction = G.torsional_friction; g.rolling_friction = G.rolling_friction;
    g.group = G.group; g.mask = G.mask;
    w.geoms.push_back(g);
  }
  return w;
}

template <class R> void set_state(World<R>& w, const float* qpos, const float* qvel, int layout) {
  int c = 0;
  for (Body<R>& b : w.bodies) {
    b.pos = Vec3<R>(qpos[c], qpos[c + 1], qpos[c + 2]);
    if (layout == 0) b.ori = Quat<R>(qpos[c + 4], qpos[c + 5], qpos[c + 6], qpos[c + 3]).renormalize();
    else b.ori = Quat<R>(qpos[c + 3], qpos[c + 4], qpos[c + 5], qpos[c + 6]);
    c += 7;
  }
  for (Tree<R>& t : w.trees) {
    for (size_t i = 0; i < t.links.size(); ++i) {
      int qo = t.q_off[i];
      switch (t.links[i].type) {
        case J_FREE: {
          for (int k = 0; k < 3; ++k) t.q[qo + k] = qpos[c + k];
          Quat<R> q = layout == 0 ? Quat<R>(qpos[c + 4], qpos[c + 5], qpos[c + 6], qpos[c + 3]).renormalize()
                                  : Quat<R>(qpos[c + 3], qpos[c + 4], qpos[c + 5], qpos[c + 6]);
          t.q[qo + 3] = q.x; t.q[qo + 4] = q.y; t.q[qo + 5] = q.z; t.q[qo + 6] = q.w;
          c += 7; break;
        }
        case J_BALL: {
          Quat<R> q = layout == 0 ? Quat<R>(qpos[c + 1], qpos[c + 2], qpos[c + 3], qpos[c]).renormalize()
                                  : Quat<R>(qpos[c], qpos[c + 1], qpos[c + 2], qpos[c + 3]);
          t.q[qo] = q.x; t.q[qo + 1] = q.y; t.q[qo + 2] = q.z; t.q[qo + 3] = q.w;
          c += 4; break;
        }
        case J_HINGE: case J_SLIDE: t.q[qo] = qpos[c]; c += 1; break;
        default: break;
      }
    }
  }
  c = 0;
  for (Body<R>& b : w.bodies) {
    b.vel = Vec3<R>(qvel[c], qvel[c + 1], qvel[c + 2]);
    b.omega_body = Vec3<R>(qvel[c + 3], qvel[c + 4], qvel[c + 5]);
    c += 6;
  }
  for (Tree<R>& t : w.trees) {
    for (size_t i = 0; i < t.links.size(); ++i) {
      int vo = t.v_off[i], qo = t.q_off[i];
      switch (t.links[i].type) {
        case J_FREE: {
          if (layout == 0) {
            Quat<R> o(t.q[qo + 3], t.q[qo + 4], t.q[qo + 5], t.q[qo + 6]);
            Vec3<R> vb = o.inverse_rotate(Vec3<R>(qvel[c], qvel[c + 1], qvel[c + 2]));
            R v[6] = {R(qvel[c + 3]), R(qvel[c + 4]), R(qvel[c + 5]), vb.x, vb.y, vb.z};
            for (int k = 0; k < 6; ++k) t.qdot[vo + k] = v[k];
          } else {
            for (int k = 0; k < 6; ++k) t.qdot[vo + k] = qvel[c + k];
          }
          c += 6; break;
        }
        case J_BALL: for (int k = 0; k < 3; ++k) t.qdot[vo + k] = qvel[c + k]; c += 3; break;
        case J_HINGE: case J_SLIDE: t.qdot[vo] = qvel[c]; c += 1; break;
        default: break;
      }
    }
  }
}

template <class R> void get_state(const World<R>& w, double* qpos, double* qvel, int layout) {
  int c = 0;
  for (const Body<R>& b : w.bodies) {
    qpos[c] = b.pos.x; qpos[c + 1] = b.pos.y; qpos[c + 2] = b.pos.z;
    if (layout == 0) { qpos[c + 3] = b.ori.w; qpos[c + 4] = b.ori.x; qpos[c + 5] = b.ori.y; qpos[c + 6] = b.ori.z; }
    else { qpos[c + 3] = b.ori.x; qpos[c + 4] = b.ori.y; qpos[c + 5] = b.ori.z; qpos[c + 6] = b.ori.w; }
    c += 7;
  }
  for (const Tree<R>& t : w.trees)
    for (size_t i = 0; i < t.links.size(); ++i) {
      int qo = t.q_off[i];
      switch (t.links[i].type) {
        case J_FREE:
          for (int k = 0; k < 3; ++k) qpos[c + k] = t.q[qo + k];
          if (layout == 0) { qpos[c + 3] = t.q[qo + 6]; qpos[c + 4] = t.q[qo + 3]; qpos[c + 5] = t.q[qo + 4]; qpos[c + 6] = t.q[qo + 5]; }
          else for (int k = 3; k < 7; ++k) qpos[c + k] = t.q[qo + k];
          c += 7; break;
        case J_BALL:
          if (layout == 0) { qpos[c] = t.q[qo + 3]; qpos[c + 1] = t.q[qo]; qpos[c + 2] = t.q[qo + 1]; qpos[c + 3] = t.q[qo + 2]; }
          else for (int k = 0; k < 4; ++k) qpos[c + k] = t.q[qo + k];
          c += 4; break;
        case J_HINGE: case J_SLIDE: qpos[c] = t.q[qo]; c += 1; break;
        default: break;
      }
    }
  c = 0;
  for (const Body<R>& b : w.bodies) {
    qvel[c] = b.vel.x; qvel[c + 1] = b.vel.y; qvel[c + 2] = b.vel.z;
    qvel[c + 3] = b.omega_body.x; qvel[c + 4] = b.omega_body.y; qvel[c + 5] = b.omega_body.z;
    c += 6;
  }
  for (const Tree<R>& t : w.trees)
    for (size_t i = 0; i < t.links.size(); ++i) {
      int vo = t.v_off[i], qo = t.q_off[i];
      switch (t.links[i].type) {
        case J_FREE:
          if (layout == 0) {
            Quat<R> o(t.q[qo + 3], t.q[qo + 4], t.q[qo + 5], t.q[qo + 6]);
            Vec3<R> vw = o.rotate(Vec3<R>(t.qdot[vo + 3], t.qdot[vo + 4], t.qdot[vo + 5]));
            qvel[c] = vw.x; qvel[c + 1] = vw.y; qvel[c + 2] = vw.z;
            qvel[c + 3] = t.qdot[vo]; qvel[c + 4] = t.qdot[vo + 1]; qvel[c + 5] = t.qdot[vo + 2];
          } else for (int k = 0; k < 6; ++k) qvel[c + k] = t.qdot[vo + k];
          c += 6; break;
        case J_BALL: for (int k = 0; k < 3; ++k) qvel[c + k] = t.qdot[vo + k]; c += 3; break;
        case J_HINGE: case J_SLIDE: qvel[c] = t.qdot[vo]; c += 1; break;
        default: break;
      }
    }
}

int dims(const newt_model_desc& d, int* nq, int* nv) {
  int q = 7 * d.n_bodies, v = 6 * d.n_bodies;
  for (int i = 0; i < d.n_links; ++i) { q += joint_nq(d.links[i].joint); v += joint_nv(d.links[i].joint); }
  *nq = q; *nv = v;
  return 0;
}

template <class R> void set_qfrc(World<R>& w, const float* qfrc) {
  // qfrc is nv per world in qvel order; only tree DoF carry qfrc_applied.
  int c = 6 * (int)w.bodies.size();
  for (Tree<R>& t : w.trees) for (int k = 0; k < t.nv(); ++k) t.qfrc_applied[k] = qfrc ? qfrc[c + k] : R(0);
}

template <class R>
int run_one(const newt_model_desc& d, const float* qpos, const float* qvel, const float* qfrc, int n_steps, int layout,
            int integrator,
            double* qpos_out, double* qvel_out, double* qacc_out) {
  World<R> w = build_world<R>(d);
  w.integrator = integrator;
  set_state(w, qpos, qvel, layout);
  set_qfrc(w, qfrc);
  std::vector<R> qacc;
  for (int s = 0; s < n_steps; ++s) {
    if (qacc_out && s == n_steps - 1 && !w.trees.empty() && w.geoms.empty()) {
      // one-step qacc of a contact-free tree: the ABA output the step integrates
      std::vector<Pose<R>> poses; forward_kinematics(w.trees[0], poses);
      std::vector<Wrench<R>> ext(w.trees[0].links.size(), Wrench<R>{Vec3<R>(), Vec3<R>()});
      Tree<R> t = w.trees[0];
      if (w.solver_mode != M_PENALTY) t.disable_penalty_limits = true;
      aba(t, poses, w.gravity, ext, w.dt, qacc);
    }
    w.step();
  }
  get_state(w, qpos_out, qvel_out, layout);
  if (qacc_out) {
    int nb = 6 * (int)w.bodies.size();
    for (int k = 0; k < nb; ++k) qacc_out[k] = 0.0;
    for (size_t k = 0; k < qacc.size(); ++k) qacc_out[nb + k] = qacc[k];
  }
  return 0;
}

}  // namespace

// ---- single-pair narrowphase queries (cross-checks of the contact routes) ----
// A pose is p xyz then quat x y z w; sizes as in newt_geom_desc; kinds are
// NEWT_SHAPE_* (sphere, box, capsule for GJK/EPA).
template <class R> static Pose<R> pose_of(const float* p) {
  return Pose<R>{Vec3<R>(p[0], p[1], p[2]), Quat<R>(p[3], p[4], p[5], p[6])};
}

template <class R> static int ccd_pair_t(int ka, const float* pa, const float* sa, int kb, const float* pb,
                                         const float* sb, float margin, float face_eps, double* out) {
  const ccd::Shape<R> A{ka, Vec3<R>(pa[0], pa[1], pa[2]), Quat<R>(pa[3], pa[4], pa[5], pa[6]), Vec3<R>(sa[0], sa[1], sa[2])};
  const ccd::Shape<R> B{kb, Vec3<R>(pb[0], pb[1], pb[2]), Quat<R>(pb[3], pb[4], pb[5], pb[6]), Vec3<R>(sb[0], sb[1], sb[2])};
  const ccd::Result<R> r = ccd::convex_contact(A, B, (R)margin, face_eps > 0.f ? (R)face_eps : R(1.0e-4));
  const double v[15] = {r.hit ? 1.0 : 0.0, (double)r.path, (double)r.pos.x, (double)r.pos.y, (double)r.pos.z,
                        (double)r.n.x, (double)r.n.y, (double)r.n.z, (double)r.pen, (double)r.wa.x, (double)r.wa.y,
                        (double)r.wa.z, (double)r.wb.x, (double)r.wb.y, (double)r.wb.z};
  for (int k = 0; k < 15; ++k) out[k] = v[k];
  return r.hit ? 1 : 0;
}

template <class R> static int np_pair_t(int ka, const float* pa, const float* sa, int kb, const float* pb,
                                        const float* sb, float margin, double* out) {
  Geom<R> a, b;
  a.shape = ka; b.shape = kb;
  for (int k = 0; k < 3; ++k) { a.size[k] = sa[k]; b.size[k] = sb[k]; }
  CBuf<R> buf;
  if (!try_np(0, a, pose_of<R>(pa), 1, b, pose_of<R>(pb), R(1), (R)margin, R(0), &buf)) return -1;
  for (int c = 0; c < buf.len; ++c) {
    const Contact<R>& x = buf.c[c];
    const double v[7] = {(double)x.pos.x, (double)x.pos.y, (double)x.pos.z, (double)x.n.x, (double)x.n.y,
                         (double)x.n.z, (double)x.pen};
    for (int k = 0; k < 7; ++k) out[7 * c + k] = v[k];
  }
  return buf.len;
}

// sensor.rs:834-1000 for a tree under external link wrenches `ext_in` (world
// force and torque about each COM; none: zero): qddot from the
// explicit ABA at the state, each link's spatial velocity and acceleration
// at its COM in its frame (compute_link_va: a_i = X_i a_parent + S_i qddot_i
// + v_i x S_i qdot_i), and the wrench its parent joint transmits
// (compute_link_wrenches: f_i = I_i a_i + v_i x* I_i v_i - (R_i^T t_ext,i,
// R_i^T (f_ext,i + m_i g)),
// each child's pulled into its parent, leaves to root).
template <class R> struct LinkDyn { SMotion<R> v, a; SForce<R> f; };
template <class R> SMotion<R> sm_add(const SMotion<R>& x, const SMotion<R>& y) { return {x.ang + y.ang, x.lin + y.lin}; }
template <class R> SMotion<R> sm_scale(const SMotion<R>& x, R k) { return {x.ang * k, x.lin * k}; }
template <class R> SMotion<R> sm_cross(const SMotion<R>& x, const SMotion<R>& y) {  // spatial.rs:60-65
  return {x.ang.cross(y.ang), x.ang.cross(y.lin) + x.lin.cross(y.ang)};
}
template <class R> SForce<R> sf_cross(const SMotion<R>& x, const SForce<R>& f) {  // spatial.rs:71-76
  return {x.ang.cross(f.tau) + x.lin.cross(f.lin), x.ang.cross(f.lin)};
}
template <class R> void tree_link_dynamics(const Tree<R>& t, const std::vector<Pose<R>>& poses, Vec3<R> gravity,
                                           std::vector<LinkDyn<R>>& out, const std::vector<Wrench<R>>* ext_in = nullptr) {
  const int n = (int)t.links.size();
  std::vector<Wrench<R>> ext = ext_in ? *ext_in : std::vector<Wrench<R>>(n, Wrench<R>{Vec3<R>(), Vec3<R>()});
  std::vector<R> qdd;
  aba(t, poses, gravity, ext, R(0), qdd);
  out.assign(n, LinkDyn<R>{});
  const SMotion<R> z{Vec3<R>(), Vec3<R>()};
  for (int i = 0; i < n; ++i) {
    const Link<R>& L = t.links[i];
    LinkDyn<R>& o = out[i];
    if (L.type == J_FREE) {
      const int v = t.v_off[i];
      o.v = {Vec3<R>(t.qdot[v], t.qdot[v + 1], t.qdot[v + 2]), Vec3<R>(t.qdot[v + 3], t.qdot[v + 4], t.qdot[v + 5])};
      o.a = {Vec3<R>(qdd[v], qdd[v + 1], qdd[v + 2]), Vec3<R>(qdd[v + 3], qdd[v + 4], qdd[v + 5])};
      continue;
    }
    const Xform<R> x = xup_xform(t, i);
    const SMotion<R> vp = L.parent >= 0 ? out[L.parent].v : z, ap = L.parent >= 0 ? out[L.parent].a : z;
    if (L.type == J_FIXED) { o.v = x.motion(vp); o.a = x.motion(ap); continue; }
    const SMotion<R> S = L.type == J_HINGE ? SMotion<R>{L.axis, L.jc_pos.cross(L.axis)} : SMotion<R>{Vec3<R>(), L.axis};
    const SMotion<R> sq = sm_scale(S, t.qdot[t.v_off[i]]), sqq = sm_scale(S, qdd[t.v_off[i]]);
    o.v = sm_add(x.motion(vp), sq);
    o.a = sm_add(sm_add(x.motion(ap), sqq), sm_cross(o.v, sq));
  }
  for (int i = 0; i < n; ++i) {
    const Link<R>& L = t.links[i];
    const Mat6<R> I = Mat6<R>::from_spatial_inertia(L.mass, Vec3<R>(), L.inertia);
    const SForce<R> ia = I.times_motion(out[i].a), iv = I.times_motion(out[i].v);
    const SForce<R> bias = sf_cross(out[i].v, iv);
    const Vec3<R> fb = poses[i].o.inverse_rotate(ext[i].f + gravity * L.mass), tb = poses[i].o.inverse_rotate(ext[i].t);
    out[i].f = {(ia.tau + bias.tau) - tb, (ia.lin + bias.lin) - fb};
  }
  for (int i = n - 1; i >= 1; --i) {
    const SForce<R> pulled = xup_xform(t, i).transpose_force(out[i].f);
    SForce<R>& fp = out[t.links[i].parent].f;
    fp = {fp.tau + pulled.tau, fp.lin + pulled.lin};
  }
}

extern "C" {

int oracle_model_dims(const newt_model_desc* d, int* nq, int* nv) { return dims(*d, nq, nv); }

// Steps `n_worlds` worlds independently.  World w uses models[model_of_world[w]]
// and the w-th qpos/qvel/qfrc block (blocks concatenated).  Outputs are double.
// n_threads > 1 spreads worlds over host threads dynamically: each thread
// takes the next unstarted world, so uneven per-world costs balance.
// integrator: 1 semi-implicit Euler (the stepped path), 0 RK4 (newt's default,
// used to replay its RK4 goldens).
int oracle_run_ex(const newt_model_desc* models, int n_worlds, const int* model_of_world, const float* qpos,
                  const float* qvel, const float* qfrc, int n_steps, int precision, int layout, double* qpos_out,
                  double* qvel_out, double* qacc_out, int n_threads, int integrator) {
  std::vector<long> qo(n_worlds + 1, 0), vo(n_worlds + 1, 0);
  for (int w = 0; w < n_worlds; ++w) {
    int nq, nv; dims(models[model_of_world[w]], &nq, &nv);
    qo[w + 1] = qo[w] + nq; vo[w + 1] = vo[w] + nv;
  }
  std::atomic<int> err{0};
  auto work = [&](int begin, int end) {
    for (int w = begin; w < end; ++w) {
      const newt_model_desc& d = models[model_of_world[w]];
      try {
        if (precision == 0)
          run_one<float>(d, qpos + qo[w], qvel + vo[w], qfrc ? qfrc + vo[w] : nullptr, n_steps, layout, integrator,
                         qpos_out + qo[w], qvel_out + vo[w], qacc_out ? qacc_out + vo[w] : nullptr);
        else
          run_one<double>(d, qpos + qo[w], qvel + vo[w], qfrc ? qfrc + vo[w] : nullptr, n_steps, layout, integrator,
                          qpos_out + qo[w], qvel_out + vo[w], qacc_out ? qacc_out + vo[w] : nullptr);
      } catch (const std::exception& e) {
        std::fprintf(stderr, "oracle_run world %d: %s\n", w, e.what());
        err = 1;
      }
    }
  };
  if (n_threads <= 1) work(0, n_worlds);
  else {
    std::atomic<int> next{0};
    auto pull = [&]() {
      for (int w = next.fetch_add(1); w < n_worlds; w = next.fetch_add(1)) work(w, w + 1);
    };
    std::vector<std::thread> th;
    for (int t = 0; t < n_threads; ++t) th.emplace_back(pull);
    for (auto& x : th) x.join();
  }
  return err.load();
}

int oracle_run(const newt_model_desc* models, int n_worlds, const int* model_of_world, const float* qpos,
               const float* qvel, const float* qfrc, int n_steps, int precision, int layout, double* qpos_out,
               double* qvel_out, double* qacc_out, int n_threads) {
  return oracle_run_ex(models, n_worlds, model_of_world, qpos, qvel, qfrc, n_steps, precision, layout, qpos_out,
                       qvel_out, qacc_out, n_threads, 1);
}

// Row impulses of one world's tree-contact solve at its state (MuJoCo
// layout; the Euler form of the step), in row order: 4 facet rows per
// pyramidal condim-3 contact, else the normal row, then the tangent pair
// (condim 3 and up), torsion (4 and up) and the rolling pair (6).  Also returns the
// tree's generalised contact forces (nv) when qfrc_out is non-null.
// integrator: 1 the Euler form of the solve (factors of M + dt B, implicit
// free ABA), 0 the RK4 form (factors of M, explicit free ABA).
int oracle_tree_impulses_ex(const newt_model_desc* d, const float* qpos, const float* qvel, const float* qfrc,
                            int precision, int cap, int* n_out, double* impulses, double* qfrc_out, int integrator) {
  int rc = 0;
  auto go = [&](auto tag) {
    using R = decltype(tag);
    World<R> w = build_world<R>(*d);
    set_state(w, qpos, qvel, 0);
    set_qfrc(w, qfrc);
    std::vector<Contact<R>> cs, tc;
    w.detect_contacts(cs);
    for (const Contact<R>& c : cs)
      if (w.geoms[c.ga].att_kind() == 2 || w.geoms[c.gb].att_kind() == 2) tc.push_back(c);
    w.tree_qfrc.assign(w.trees.size(), std::vector<R>());
    for (size_t t = 0; t < w.trees.size(); ++t) w.tree_qfrc[t].assign(w.trees[t].nv(), R(0));
    w.tree_body_wrenches.assign(w.bodies.size(), Wrench<R>{Vec3<R>(), Vec3<R>()});
    std::vector<R> imp;
    try {
      solve_tree_contacts(w, tc, w.solver_mode == M_NEWTON, integrator == 1, &imp);
    } catch (const std::exception& e) {
      std::fprintf(stderr, "oracle_tree_impulses: %s\n", e.what());
      rc = 1;
      return;
    }
    *n_out = (int)imp.size();
    for (int i = 0; i < (int)imp.size() && i < cap; ++i) impulses[i] = (double)imp[i];
    if (qfrc_out && !w.trees.empty())
      for (int k = 0; k < w.trees[0].nv(); ++k) qfrc_out[k] = (double)w.tree_qfrc[0][k];
  };
  if (precision == 0) go(0.0f); else go(0.0);
  return rc;
}
int oracle_tree_impulses(const newt_model_desc* d, const float* qpos, const float* qvel, const float* qfrc,
                         int precision, int cap, int* n_out, double* impulses, double* qfrc_out) {
  return oracle_tree_impulses_ex(d, qpos, qvel, qfrc, precision, cap, n_out, impulses, qfrc_out, 1);
}

// Contacts of one world at its given state (MuJoCo layout), detected exactly
// as the step's collision phase does.  data: pos xyz, normal xyz, penetration.
int oracle_contacts(const newt_model_desc* d, const float* qpos, const float* qvel, int precision, int cap,
                    int* n_out, int* pairs, double* data) {
  auto go = [&](auto tag) {
    using R = decltype(tag);
    World<R> w = build_world<R>(*d);
    set_state(w, qpos, qvel, 0);
    std::vector<Contact<R>> cs;
    w.detect_contacts(cs);
    *n_out = (int)cs.size();
    for (int i = 0; i < (int)cs.size() && i < cap; ++i) {
      pairs[2 * i] = cs[i].ga; pairs[2 * i + 1] = cs[i].gb;
      double v[7] = {(double)cs[i].pos.x, (double)cs[i].pos.y, (double)cs[i].pos.z, (double)cs[i].n.x,
                     (double)cs[i].n.y, (double)cs[i].n.z, (double)cs[i].pen};
      for (int k = 0; k < 7; ++k) data[7 * i + k] = v[k];
    }
  };
  if (precision == 0) go(0.0f); else go(0.0);
  return 0;
}

// Post-step sensors of one world at its state (MuJoCo layout), restating
// newt/src/sensor.rs:560-700 for the kinds that read the state alone, with
// site_world_pose (sensor.rs:794-806), parent_body_velocities (:812-828),
// site_velocity (:705-726), subtree_com (:728-757) and the link velocities of
// compute_link_va (:834-900) at zero acceleration.  `sensors` holds per sensor
// (kind, on_link, index) ints in `si` and (local_pos xyz, local_quat xyzw) in
// `sf`; `out` receives the concatenated values.
}  // extern "C"

// scene_query.rs:182-438 (ray_vs_geom without meshes): the distance along
// the ray (origin o, direction dv, in the geom's frame) to the first hit at
// or beyond 0, or -1.  newt returns the hit also for a ray that starts
// inside the shape (its far root).
template <class R> R ray_sphere_at(Vec3<R> c, R radius, Vec3<R> o, Vec3<R> dv) {
  const Vec3<R> off = o - c;
  const R a = dv.dot(dv);
  if (a <= R(0)) return R(-1);
  const R hb = off.dot(dv), cc = off.dot(off) - radius * radius;
  const R disc = hb * hb - a * cc;
  if (disc < R(0)) return R(-1);
  const R root = Sc<R>::sqrt(disc);
  const R nr = (-hb - root) / a, fr = (-hb + root) / a;
  const R t = nr >= R(0) ? nr : fr;
  return t >= R(0) ? t : R(-1);
}
template <class R> R ray_cyl_side(R radius, R hh, Vec3<R> o, Vec3<R> dv) {
  const R a = dv.x * dv.x + dv.y * dv.y;
  if (a <= R(1.0e-8)) return R(-1);
  const R hb = o.x * dv.x + o.y * dv.y, cc = o.x * o.x + o.y * o.y - radius * radius;
  const R disc = hb * hb - a * cc;
  if (disc < R(0)) return R(-1);
  const R root = Sc<R>::sqrt(disc);
  R best = R(-1);
  const R ts[2] = {(-hb - root) / a, (-hb + root) / a};
  for (R t : ts)
    if (t >= R(0)) {
      const R z = o.z + dv.z * t;
      if (z >= -hh && z <= hh && (best < R(0) || t < best)) best = t;
    }
  return best;
}
template <class R> R ray_geom(int shape, const R* size, Vec3<R> o, Vec3<R> dv) {
  if (!(dv.dot(dv) > R(0))) return R(-1);
  auto better = [](R cand, R best) { return cand >= R(0) && (best < R(0) || cand < best); };
  switch (shape) {
    case S_SPHERE: return ray_sphere_at(Vec3<R>(), size[0], o, dv);
    case S_PLANE: {
      if (dv.z == R(0)) return R(-1);
      const R t = -o.z / dv.z;
      return t >= R(0) ? t : R(-1);
    }
    case S_BOX: {
      R nr = -std::numeric_limits<R>::infinity(), fr = std::numeric_limits<R>::infinity();
      const R oa[3] = {o.x, o.y, o.z}, da[3] = {dv.x, dv.y, dv.z};
      for (int k = 0; k < 3; ++k) {
        if (da[k] == R(0)) {
          if (rabs(oa[k]) > size[k]) return R(-1);
          continue;
        }
        R an = (-size[k] - oa[k]) / da[k], af = (size[k] - oa[k]) / da[k];
        if (an > af) std::swap(an, af);
        if (an > nr) nr = an;
        if (af < fr) fr = af;
        if (nr > fr) return R(-1);
      }
      const R t = nr >= R(0) ? nr : fr;
      return t >= R(0) ? t : R(-1);
    }
    case S_CAPSULE: {
      R best = ray_cyl_side(size[0], size[1], o, dv);
      const R lo = ray_sphere_at(Vec3<R>(R(0), R(0), -size[1]), size[0], o, dv);
      if (better(lo, best)) best = lo;
      const R hi = ray_sphere_at(Vec3<R>(R(0), R(0), size[1]), size[0], o, dv);
      if (better(hi, best)) best = hi;
      return best;
    }
    case S_CYLINDER: {
      R best = ray_cyl_side(size[0], size[1], o, dv);
      if (dv.z != R(0))
        for (R z : {-size[1], size[1]}) {
          const R t = (z - o.z) / dv.z;
          if (t >= R(0)) {
            const R px = o.x + dv.x * t, py = o.y + dv.y * t;
            if (px * px + py * py <= size[0] * size[0] && (best < R(0) || t < best)) best = t;
          }
        }
      return best;
    }
    case S_ELLIPSOID: {
      const Vec3<R> so(o.x / size[0], o.y / size[1], o.z / size[2]), sd(dv.x / size[0], dv.y / size[1], dv.z / size[2]);
      const R a = sd.dot(sd);
      if (a <= R(0)) return R(-1);
      const R hb = so.dot(sd), cc = so.dot(so) - R(1);
      const R disc = hb * hb - a * cc;
      if (disc < R(0)) return R(-1);
      const R root = Sc<R>::sqrt(disc);
      const R nr = (-hb - root) / a, fr = (-hb + root) / a;
      const R t = nr >= R(0) ? nr : fr;
      return t >= R(0) ? t : R(-1);
    }
    default: return R(-1);
  }
}
// rangefinder_reading (sensor.rs:759-791): the nearest hit over every geom
// of the world, -1 for none.
template <class R> R rangefinder(const World<R>& w, Vec3<R> origin, Vec3<R> dir) {
  std::vector<Pose<R>> gp;
  w.geom_poses(gp);
  R nearest = R(-1);
  for (size_t i = 0; i < w.geoms.size(); ++i) {
    const Vec3<R> o = gp[i].o.inverse_rotate(origin - gp[i].p), dv = gp[i].o.inverse_rotate(dir);
    const R t = ray_geom(w.geoms[i].shape, w.geoms[i].size, o, dv);
    if (t >= R(0) && (nearest < R(0) || t < nearest)) nearest = t;
  }
  return nearest;
}

extern "C" {

int oracle_sensors(const newt_model_desc* d, const float* qpos, const float* qvel, const float* qfrc, int precision,
                   int ns, const int* si, const float* sf, double* out) {
  auto go = [&](auto tag) {
    using R = decltype(tag);
    World<R> w = build_world<R>(*d);
    set_state(w, qpos, qvel, 0);
    if (qfrc && !w.trees.empty())
      for (int k = 0; k < w.trees[0].nv(); ++k) w.trees[0].qfrc_applied[k] = qfrc[k];
    std::vector<Pose<R>> poses;
    std::vector<GMotion<R>> v;
    if (!w.trees.empty()) {
      const Tree<R>& t = w.trees[0];
      forward_kinematics(t, poses);
      const int n = (int)t.links.size();
      v.assign(n, GMotion<R>{Vec3<R>(), Vec3<R>()});
      for (int i = 0; i < n; ++i) {
        const Link<R>& L = t.links[i];
        if (L.type == J_FREE) {
          const int o = t.v_off[i];
          v[i] = {Vec3<R>(t.qdot[o], t.qdot[o + 1], t.qdot[o + 2]), Vec3<R>(t.qdot[o + 3], t.qdot[o + 4], t.qdot[o + 5])};
        } else if (L.type == J_FIXED) {
          v[i] = xup_fixed(L).motion(L.parent >= 0 ? v[L.parent] : GMotion<R>{Vec3<R>(), Vec3<R>()});
        } else {
          const GMotion<R> S = L.type == J_HINGE ? GMotion<R>{L.axis, L.jc_pos.cross(L.axis)} : GMotion<R>{Vec3<R>(), L.axis};
          v[i] = xup_joint(L, t.q[t.q_off[i]]).motion(v[L.parent]).add(S.scale(t.qdot[t.v_off[i]]));
        }
      }
    }
    std::vector<LinkDyn<R>> dyn;  // accelerometers on links, force and torque
    for (int k = 0; k < ns && !w.trees.empty() && dyn.empty(); ++k)
      if ((si[3 * k] == 9 && si[3 * k + 1]) || si[3 * k] == 11 || si[3 * k] == 12)
        tree_link_dynamics(w.trees[0], poses, w.gravity, dyn);
    int o = 0;
    for (int k = 0; k < ns; ++k) {
      const int kind = si[3 * k], on_link = si[3 * k + 1], idx = si[3 * k + 2];
      const Vec3<R> lp(sf[7 * k], sf[7 * k + 1], sf[7 * k + 2]);
      const Quat<R> lq(sf[7 * k + 3], sf[7 * k + 4], sf[7 * k + 5], sf[7 * k + 6]);
      auto put3 = [&](Vec3<R> x) { out[o++] = (double)x.x; out[o++] = (double)x.y; out[o++] = (double)x.z; };
      if (kind == 11) { put3(dyn[idx].f.lin); continue; }  // Force (sensor.rs:622-629)
      if (kind == 12) {  // Torque at the joint anchor, tau - r_jc x F (sensor.rs:630-647)
        put3(dyn[idx].f.tau - w.trees[0].links[idx].jc_pos.cross(dyn[idx].f.lin));
        continue;
      }
      if (kind == 9) {  // accelerometer on a link (sensor.rs:1030-1087, the Link branch)
        const Quat<R> ori = poses[idx].o;
        const SMotion<R>& vb = dyn[idx].v;
        const SMotion<R>& ab = dyn[idx].a;
        const Vec3<R> om = ori.rotate(vb.ang), al = ori.rotate(ab.ang);
        const Vec3<R> acom = ori.rotate(ab.lin + vb.ang.cross(vb.lin));
        const Vec3<R> r = ori.rotate(lp);
        const Vec3<R> asite = acom + al.cross(r) + om.cross(om.cross(r));
        put3((ori * lq).inverse_rotate(asite - w.gravity));
        continue;
      }
      if (kind == 0 || kind == 1) {  // JointPos / JointVel
        const Tree<R>& t = w.trees[0];
        out[o++] = (double)(kind == 0 ? t.q[t.q_off[idx]] : t.qdot[t.v_off[idx]]);
        continue;
      }
      if (kind == 8) {  // SubtreeCom
        const Tree<R>& t = w.trees[0];
        Vec3<R> acc;
        R m = R(0);
        for (int j = 0; j < (int)t.links.size(); ++j) {
          int c = j;
          bool inc = false;
          while (c >= 0) { if (c == idx) { inc = true; break; } c = t.links[c].parent; }
          if (inc) { acc = acc + poses[j].p * t.links[j].mass; m = m + t.links[j].mass; }
        }
        put3(m == R(0) ? Vec3<R>() : acc / m);
        continue;
      }
      Vec3<R> pp, wb, lin, ang;
      Quat<R> po;
      if (on_link) {
        pp = poses[idx].p; po = poses[idx].o;
        wb = v[idx].ang;
        ang = po.rotate(v[idx].ang);
        lin = po.rotate(v[idx].lin + v[idx].ang.cross(lp));
      } else {
        const Body<R>& b = w.bodies[idx];
        pp = b.pos; po = b.ori; wb = b.omega_body;
        ang = b.ori.rotate(b.omega_body);
        lin = b.vel + ang.cross(b.ori.rotate(lp));
      }
      const Quat<R> so = po * lq;
      switch (kind) {
        case 13:  // Magnetometer (sensor.rs:664-670)
          put3(so.inverse_rotate(Vec3<R>(d->magnetic_field[0], d->magnetic_field[1], d->magnetic_field[2])));
          break;
        case 14:  // Rangefinder along the site's +z (sensor.rs:671-682)
          out[o++] = (double)rangefinder(w, pp + po.rotate(lp), so.rotate(Vec3<R>(R(0), R(0), R(1))));
          break;
        case 2: put3(pp + po.rotate(lp)); break;
        case 3: out[o++] = (double)so.x; out[o++] = (double)so.y; out[o++] = (double)so.z; out[o++] = (double)so.w; break;
        case 4: put3(lq.inverse_rotate(wb)); break;
        case 5: put3(so.inverse_rotate(lin)); break;
        case 6: put3(lin); break;
        default: put3(ang); break;
      }
    }
  };
  if (precision == 0) go(0.0f); else go(0.0);
  return 0;
}

// newt's post-step contact sensors for a free-body world
// (world.rs:1545-1612 build_sensor_inputs, sensor.rs:446-757 evaluate,
// :1030-1087 accelerometer_reading, :1103-1112 touch_reading): one step from
// (qpos, qvel), then the step's contact set re-solved at the post-step
// bodies with the world's solver (solve_free_bodies_diag or its Newton
// variant, solver.rs:596-640), giving the body wrenches and the per-contact
// normal forces (the contact's row impulses summed in row order, over dt,
// solver.rs:1240-1253).  Kinds: 9 accelerometer (site on body `index`), 10
// touch (geom `index`).  Writes the readings and the post-step state
// (MuJoCo layout); returns -1 for a world with a tree or a failed Newton
// factor.
int oracle_contact_sensors(const newt_model_desc* d, const float* qpos, const float* qvel, int precision, int ns,
                           const int* si, const float* sf, double* out, double* qpos_out, double* qvel_out) {
  int rc = 0;
  auto go = [&](auto tag) {
    using R = decltype(tag);
    World<R> w = build_world<R>(*d);
    if (!w.trees.empty()) { rc = -1; return; }
    set_state(w, qpos, qvel, 0);
    std::vector<Contact<R>> contacts;
    w.detect_contacts(contacts);
    w.step();
    std::vector<Wrench<R>> wr;
    std::vector<R> imp;
    std::vector<int> row_contact;
    if (w.solver_mode == M_NEWTON) {
      if (!solve_free_bodies_newton(w.bodies, w.geoms, contacts, w.gravity, w.dt, w.iterations, wr, &imp,
                                    &row_contact)) { rc = -1; return; }
    } else {
      solve_free_bodies_pgs(w.bodies, w.geoms, contacts, w.gravity, w.dt, w.iterations, wr, &imp, &row_contact,
                            w.cone);
    }
    if (wr.empty()) wr.assign(w.bodies.size(), Wrench<R>{Vec3<R>(), Vec3<R>()});
    // the facets' impulses summed (pyramidal condim 3), else the normal row's
    std::vector<R> fn(contacts.size(), R(0));
    std::vector<char> seen(contacts.size(), 0);
    for (size_t r = 0; r < imp.size(); ++r) {
      const int c = row_contact[r];
      const bool facets = w.cone == 0 && std::min(w.geoms[contacts[c].ga].condim, w.geoms[contacts[c].gb].condim) == 3;
      if (facets || !seen[c]) fn[c] += imp[r];
      seen[c] = 1;
    }
    for (R& x : fn) x = x / w.dt;
    int o = 0;
    for (int k = 0; k < ns; ++k) {
      const int kind = si[3 * k], idx = si[3 * k + 2];
      if (kind == 10) {
        R sum = R(0);
        for (size_t c = 0; c < contacts.size(); ++c)
          if (contacts[c].ga == idx || contacts[c].gb == idx) sum += fn[c] < R(0) ? -fn[c] : fn[c];
        out[o++] = (double)sum;
        continue;
      }
      const Vec3<R> lp(sf[7 * k], sf[7 * k + 1], sf[7 * k + 2]);
      const Quat<R> lq(sf[7 * k + 3], sf[7 * k + 4], sf[7 * k + 5], sf[7 * k + 6]);
      const Body<R>& b = w.bodies[idx];
      const Vec3<R> a_com = w.gravity + wr[idx].f / b.mass;
      const Vec3<R> tau_body = b.ori.inverse_rotate(wr[idx].t);
      const Vec3<R> iw = b.inertia * b.omega_body;
      const Vec3<R> gyro = -(b.omega_body.cross(iw));
      const Vec3<R> alpha_body = b.inertia_inv * (tau_body + gyro);
      const Vec3<R> omega_world = b.ori.rotate(b.omega_body), alpha_world = b.ori.rotate(alpha_body);
      const Vec3<R> r = b.ori.rotate(lp);
      const Vec3<R> a_site = a_com + alpha_world.cross(r) + omega_world.cross(omega_world.cross(r));
      const Vec3<R> a_proper = a_site - w.gravity;
      const Vec3<R> v = (b.ori * lq).inverse_rotate(a_proper);
      out[o++] = (double)v.x; out[o++] = (double)v.y; out[o++] = (double)v.z;
    }
    get_state(w, qpos_out, qvel_out, 0);
  };
  if (precision == 0) go(0.0f); else go(0.0);
  return rc;
}

// newt's post-step contact sensors for a tree-contact world (world.rs:
// 1545-1701 build_sensor_inputs with solve_tree_contact_sensor_solution,
// world.rs:2252-2274; sensor.rs:446-1112): one step from (qpos, qvel) with
// the tree's applied forces `qfrc` (newt layout, nullable), then the step's
// tree contacts re-solved at the post-step state with the world's solver
// and integrator form, giving each link's contact wrench and each
// contact's normal force (solver.rs:3334-3364).  Kinds: 9 accelerometer on
// link `index`, 10 touch (geom `index`), 11 force and 12 torque at link
// `index`'s parent joint (the links' dynamics under those wrenches); other
// kinds read 0 here.  Writes the readings and the post-step state (MuJoCo
// layout); returns -1 for a world without a tree.
int oracle_tree_contact_sensors(const newt_model_desc* d, const float* qpos, const float* qvel, const float* qfrc,
                                int precision, int ns, const int* si, const float* sf, double* out, double* qpos_out,
                                double* qvel_out) {
  int rc = 0;
  auto go = [&](auto tag) {
    using R = decltype(tag);
    World<R> w = build_world<R>(*d);
    if (w.trees.empty()) { rc = -1; return; }
    w.integrator = d->integrator == NEWT_INTEGRATOR_RK4 ? 0 : 1;  // the model's own integrator
    set_state(w, qpos, qvel, 0);
    if (qfrc)
      for (int k = 0; k < w.trees[0].nv(); ++k) w.trees[0].qfrc_applied[k] = qfrc[k];
    std::vector<Contact<R>> contacts;
    w.detect_contacts(contacts);
    w.step();
    std::vector<Contact<R>> tc;
    for (const Contact<R>& c : contacts)
      if (w.geoms[c.ga].att_kind() == 2 || w.geoms[c.gb].att_kind() == 2) tc.push_back(c);
    w.tree_qfrc.assign(w.trees.size(), std::vector<R>());
    for (size_t t = 0; t < w.trees.size(); ++t) w.tree_qfrc[t].assign(w.trees[t].nv(), R(0));
    w.tree_body_wrenches.assign(w.bodies.size(), Wrench<R>{Vec3<R>(), Vec3<R>()});
    std::vector<Wrench<R>> lw;
    std::vector<R> fn;
    solve_tree_contacts<R>(w, tc, w.solver_mode == M_NEWTON, w.integrator == 1, nullptr, &lw, &fn);
    if (lw.empty()) lw.assign(w.trees[0].links.size(), Wrench<R>{Vec3<R>(), Vec3<R>()});
    std::vector<Pose<R>> poses;
    forward_kinematics(w.trees[0], poses);
    std::vector<LinkDyn<R>> dyn;
    tree_link_dynamics(w.trees[0], poses, w.gravity, dyn, &lw);
    int o = 0;
    for (int k = 0; k < ns; ++k) {
      const int kind = si[3 * k], idx = si[3 * k + 2];
      const Vec3<R> lp(sf[7 * k], sf[7 * k + 1], sf[7 * k + 2]);
      const Quat<R> lq(sf[7 * k + 3], sf[7 * k + 4], sf[7 * k + 5], sf[7 * k + 6]);
      auto put3 = [&](Vec3<R> x) { out[o++] = (double)x.x; out[o++] = (double)x.y; out[o++] = (double)x.z; };
      if (kind == 10) {  // touch_reading (sensor.rs:1103-1112)
        R sum = R(0);
        for (size_t c = 0; c < tc.size(); ++c)
          if (tc[c].ga == idx || tc[c].gb == idx) sum += fn[c] < R(0) ? -fn[c] : fn[c];
        out[o++] = (double)sum;
      } else if (kind == 11) {
        put3(dyn[idx].f.lin);
      } else if (kind == 12) {
        put3(dyn[idx].f.tau - w.trees[0].links[idx].jc_pos.cross(dyn[idx].f.lin));
      } else if (kind == 9) {
        const Quat<R> ori = poses[idx].o;
        const SMotion<R>& vb = dyn[idx].v;
        const SMotion<R>& ab = dyn[idx].a;
        const Vec3<R> om = ori.rotate(vb.ang), al = ori.rotate(ab.ang);
        const Vec3<R> acom = ori.rotate(ab.lin + vb.ang.cross(vb.lin));
        const Vec3<R> r = ori.rotate(lp);
        const Vec3<R> asite = acom + al.cross(r) + om.cross(om.cross(r));
        put3((ori * lq).inverse_rotate(asite - w.gravity));
      } else {
        const int dim = kind <= 1 ? 1 : (kind == 3 ? 4 : 3);
        for (int j = 0; j < dim; ++j) out[o++] = 0.0;
      }
    }
    get_state(w, qpos_out, qvel_out, 0);
  };
  if (precision == 0) go(0.0f); else go(0.0);
  return rc;
}

// PGS row impulses of one free-body world at its state (one step's solve).
int oracle_impulses(const newt_model_desc* d, const float* qpos, const float* qvel, int precision, int iterations,
                    int cap, int* n_out, double* impulses) {
  auto go = [&](auto tag) {
    using R = decltype(tag);
    World<R> w = build_world<R>(*d);
    set_state(w, qpos, qvel, 0);
    std::vector<Contact<R>> cs;
    w.detect_contacts(cs);
    std::vector<Wrench<R>> wr;
    std::vector<R> imp;
    const int its = iterations > 0 ? iterations : w.iterations;
    if (w.solver_mode == M_NEWTON) {
      if (!solve_free_bodies_newton(w.bodies, w.geoms, cs, w.gravity, w.dt, its, wr, &imp)) imp.clear();
    } else {
      solve_free_bodies_pgs(w.bodies, w.geoms, cs, w.gravity, w.dt, its, wr, &imp, nullptr, w.cone);
    }
    *n_out = (int)imp.size();
    for (int i = 0; i < (int)imp.size() && i < cap; ++i) impulses[i] = imp[i];
  };
  if (precision == 0) go(0.0f); else go(0.0);
  return 0;
}

// Dense CRB mass matrix (newt layout) of the world's tree at native q.
int oracle_mass_matrix(const newt_model_desc* d, const float* q_native, int precision, double* out) {
  auto go = [&](auto tag) {
    using R = decltype(tag);
    World<R> w = build_world<R>(*d);
    Tree<R>& t = w.trees[0];
    for (int i = 0; i < t.nq(); ++i) t.q[i] = q_native[i];
    std::vector<R> M;
    mass_matrix(t, M);
    for (size_t i = 0; i < M.size(); ++i) out[i] = M[i];
  };
  if (precision == 0) go(0.0f); else go(0.0);
  return 0;
}

// Total mechanical energy (kinetic + gravitational potential) of each world
// at the given MuJoCo-layout state, in FP64: 0.5 qd^T M qd - sum m g.p for
// the tree (CRB mass matrix, FK positions) plus 0.5 m v^2 + 0.5 w.Iw - m g.p
// for free bodies.
int oracle_energy(const newt_model_desc* models, int n_worlds, const int* model_of_world, const float* qpos,
                  const float* qvel, double* out) {
  long qo = 0, vo = 0;
  for (int w = 0; w < n_worlds; ++w) {
    const newt_model_desc& d = models[model_of_world[w]];
    int nq, nv; dims(d, &nq, &nv);
    World<double> wd = build_world<double>(d);
    set_state(wd, qpos + qo, qvel + vo, 0);
    double e = 0.0;
    for (const Body<double>& b : wd.bodies) {
      Vec3<double> iw = b.inertia * b.omega_body;
      e += 0.5 * b.mass * b.vel.dot(b.vel) + 0.5 * b.omega_body.dot(iw) - b.mass * wd.gravity.dot(b.pos);
    }
    for (const Tree<double>& t : wd.trees) {
      std::vector<double> M;
      mass_matrix(t, M);
      int n = t.nv();
      for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) e += 0.5 * t.qdot[i] * M[i * n + j] * t.qdot[j];
      std::vector<Pose<double>> poses;
      forward_kinematics(t, poses);
      for (size_t i = 0; i < t.links.size(); ++i) e -= t.links[i].mass * wd.gravity.dot(poses[i].p);
    }
    out[w] = e;
    qo += nq; vo += nv;
  }
  return 0;
}

// newt's GJK/EPA contact of one pair (newt/src/contact/ccd.rs:1703-1911).
// face_eps <= 0: newt's EPA face-removal threshold (1e-4 of the pair extent).
// out (15 doubles): hit, path (1 distance GJK, 2 EPA, 3 EPA fallback), point
// xyz, normal xyz (from B into A), penetration, witness on A, witness on B.
int oracle_ccd_pair(int precision, int kind_a, const float* pose_a, const float* size_a, int kind_b,
                    const float* pose_b, const float* size_b, float margin, float face_eps, double* out) {
  auto ok = [](int k) { return k == ccd::SPHERE || k == ccd::BOX || k == ccd::CAPSULE; };
  if (!ok(kind_a) || !ok(kind_b)) return -1;
  return precision == 0 ? ccd_pair_t<float>(kind_a, pose_a, size_a, kind_b, pose_b, size_b, margin, face_eps, out)
                        : ccd_pair_t<double>(kind_a, pose_a, size_a, kind_b, pose_b, size_b, margin, face_eps, out);
}

// The closed-form narrowphase of one pair as the step runs it (newt's
// dispatch, contact.rs:2509-2587, with the sphere-box extension), without the
// relabelling: (A, B) must be a routed order.  Up to 4 contacts of 7 doubles
// (point, normal from B into A, penetration); returns the count, -1 when
// (A, B) has no route.
int oracle_np_pair(int precision, int kind_a, const float* pose_a, const float* size_a, int kind_b,
                   const float* pose_b, const float* size_b, float margin, double* out) {
  return precision == 0 ? np_pair_t<float>(kind_a, pose_a, size_a, kind_b, pose_b, size_b, margin, out)
                        : np_pair_t<double>(kind_a, pose_a, size_a, kind_b, pose_b, size_b, margin, out);
}

// Raw f32 bits of newt's deterministic sin/cos (for the polynomial KATs).
float oracle_newt_sin(float x) { return newt_sin(x); }
float oracle_newt_cos(float x) { return newt_cos(x); }

// Wall-clock timing of the f32 mirror over `n_threads` host threads: the CPU
// baseline (worlds handed to threads one at a time).  Returns seconds.
double oracle_time_run(const newt_model_desc* models, int n_worlds, const int* model_of_world, const float* qpos,
                       const float* qvel, const float* qfrc, int n_steps, int n_threads) {
  long nq = 0, nv = 0;
  for (int w = 0; w < n_worlds; ++w) { int a, b; dims(models[model_of_world[w]], &a, &b); nq += a; nv += b; }
  std::vector<double> qo(nq), vo(nv);
  auto t0 = std::chrono::steady_clock::now();
  oracle_run(models, n_worlds, model_of_world, qpos, qvel, qfrc, n_steps, 0, 0, qo.data(), vo.data(), nullptr, n_threads);
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"
