// Oracle (test infrastructure only): kinematic trees, forward kinematics,
// the articulated-body algorithm, the CRB mass matrix, Cholesky, and the
// semi-implicit Euler tree step, restated from newt.
//
// Sources (paths inside hwang2409/tooling):
//   newt/src/tree.rs:79-237     Link / Tree layout (q, qdot, qfrc_applied)
//   newt/src/tree.rs:771-858    forward_kinematics_into
//   newt/src/tree.rs:1021-1116  aba_with_velocity_implicit_workspace
//   newt/src/forces.rs:6-85     assemble_joint_forces
//   newt/src/aba.rs:803-1102    aba::run (three passes)
//   newt/src/tree.rs:1393-1475  euler_step_with_workspace, integrate_tree_positions
//   newt/src/dynamics.rs:474-648 mass_matrix, cholesky, cholesky_solve
//   newt/src/tree.rs:645-684    implicit_mass_matrix
#pragma once
#include <array>
#include <vector>
#include "newt_math.hpp"

namespace oracle {

enum JointType { J_FREE = 0, J_FIXED = 1, J_HINGE = 2, J_SLIDE = 3, J_BALL = 4 };

inline int joint_nq(int t) { return t == J_FREE ? 7 : t == J_FIXED ? 0 : t == J_BALL ? 4 : 1; }
inline int joint_nv(int t) { return t == J_FREE ? 6 : t == J_FIXED ? 0 : t == J_BALL ? 3 : 1; }

template <class R> struct Link {
  int parent = -1;
  int type = J_FIXED;
  Vec3<R> axis;            // hinge / slide axis in the parent frame
  R damping = 0, armature = 0, free_damping = 0;
  Vec3<R> jp_pos; Quat<R> jp_ori;   // joint_offset_in_parent
  Vec3<R> jc_pos; Quat<R> jc_ori;   // joint_offset_in_child
  R mass = 1;
  Mat3<R> inertia, inertia_inv;
};

template <class R> struct Tree {
  std::vector<Link<R>> links;
  std::vector<int> q_off, v_off;
  std::vector<R> q, qdot, qfrc_applied;
  bool disable_penalty_limits = false;
  int nq() const { return (int)q.size(); }
  int nv() const { return (int)qdot.size(); }
  // tree.rs:275-331: append a link and grow the state vectors.
  int push_link(Link<R> l) {
    if (!l.inertia.inverse(&l.inertia_inv)) l.inertia_inv = Mat3<R>::zero();
    int idx = (int)links.size();
    q_off.push_back((int)q.size());
    v_off.push_back((int)qdot.size());
    switch (l.type) {
      case J_FREE: { Vec3<R> p = l.jp_pos; Quat<R> o = l.jp_ori; R v[7] = {p.x, p.y, p.z, o.x, o.y, o.z, o.w}; q.insert(q.end(), v, v + 7); break; }
      case J_HINGE: case J_SLIDE: q.push_back(R(0)); break;
      case J_BALL: { R v[4] = {0, 0, 0, 1}; q.insert(q.end(), v, v + 4); break; }
      default: break;
    }
    for (int i = 0; i < joint_nv(l.type); ++i) { qdot.push_back(R(0)); qfrc_applied.push_back(R(0)); }
    links.push_back(l);
    return idx;
  }
};

template <class R> struct Pose { Vec3<R> p; Quat<R> o; };

// tree.rs:771-858
template <class R> void forward_kinematics(const Tree<R>& t, std::vector<Pose<R>>& out) {
  out.clear();
  for (size_t i = 0; i < t.links.size(); ++i) {
    const Link<R>& L = t.links[i];
    Pose<R> pose;
    switch (L.type) {
      case J_FREE: {
        int o = t.q_off[i];
        pose.p = Vec3<R>(t.q[o], t.q[o + 1], t.q[o + 2]);
        pose.o = Quat<R>(t.q[o + 3], t.q[o + 4], t.q[o + 5], t.q[o + 6]);
        break;
      }
      case J_FIXED: {
        Pose<R> par = L.parent >= 0 ? out[L.parent] : Pose<R>{Vec3<R>(), Quat<R>()};
        Vec3<R> jpw = par.p + par.o.rotate(L.jp_pos);
        Quat<R> jow = par.o * L.jp_ori;
        Quat<R> co = jow * L.jc_ori.conjugate();
        pose.p = jpw - co.rotate(L.jc_pos);
        pose.o = co;
        break;
      }
      case J_HINGE: {
        Pose<R> par = out[L.parent];
        R qa = t.q[t.q_off[i]];
        Vec3<R> jpw = par.p + par.o.rotate(L.jp_pos);
        Quat<R> jr = Quat<R>::from_axis_angle(L.axis, qa);
        Quat<R> co = par.o * jr;
        pose.p = jpw - co.rotate(L.jc_pos);
        pose.o = co;
        break;
      }
      case J_SLIDE: {
        Pose<R> par = out[L.parent];
        R qs = t.q[t.q_off[i]];
        Quat<R> co = par.o;
        Vec3<R> jpw = par.p + par.o.rotate(L.jp_pos);
        Vec3<R> sw = par.o.rotate(L.axis * qs);
        pose.p = jpw + sw - co.rotate(L.jc_pos);
        pose.o = co;
        break;
      }
      case J_BALL: {
        Pose<R> par = out[L.parent];
        int o = t.q_off[i];
        Quat<R> qb(t.q[o], t.q[o + 1], t.q[o + 2], t.q[o + 3]);
        Vec3<R> jpw = par.p + par.o.rotate(L.jp_pos);
        Quat<R> co = par.o * qb;
        pose.p = jpw - co.rotate(L.jc_pos);
        pose.o = co;
        break;
      }
    }
    out.push_back(pose);
  }
}

// tree.rs:1120-1127 (Fixed child) as a GX.
template <class R> GX<R> xup_fixed(const Link<R>& L) {
  Quat<R> rel = L.jp_ori * L.jc_ori.conjugate();
  Mat3<R> rot = rel.conjugate().to_mat3();
  Vec3<R> t = L.jc_pos - rot * L.jp_pos;
  return {GM3<R>::from_mat3(rot), t};
}

// aba.rs:744-787 `transform` for hinge / slide.
template <class R> GX<R> xup_joint(const Link<R>& L, R q) {
  if (L.type == J_HINGE) {
    Vec3<R> ax = L.axis.normalize();
    R half = (R(0) - q) * R(0.5);
    R s = Sc<R>::sin(half), c = Sc<R>::cos(half);
    GM3<R> rot = GM3<R>::quat(ax.x * s, ax.y * s, ax.z * s, c);
    return {rot, L.jc_pos - rot.mul_vec(L.jp_pos)};
  }
  // slide
  return {GM3<R>::identity(), (L.jc_pos - L.jp_pos) - L.axis * q};
}

// Per-link world-frame external wrench at the COM: (force, torque).
template <class R> struct Wrench { Vec3<R> f, t; };

// ABA with the Euler velocity-implicit fold (tree.rs:1021-1116 + aba.rs:803-1102).
// `implicit_dt` = 0 selects the explicit form.
template <class R>
void aba(const Tree<R>& t, const std::vector<Pose<R>>& poses, Vec3<R> gravity,
         const std::vector<Wrench<R>>& ext, R implicit_dt, std::vector<R>& qacc) {
  const int n = (int)t.links.size();
  const int nv = t.nv();
  // assemble_joint_forces (forces.rs:6-85); no tendons, limits or actuators.
  std::vector<R> scalar(n, R(0));
  std::vector<Vec3<R>> ball(n);
  GForce<R> freef{Vec3<R>(), Vec3<R>()};
  for (int i = 0; i < n; ++i) {
    const Link<R>& L = t.links[i];
    if (L.type == J_FREE && i == 0) {
      bool ap = t.disable_penalty_limits;
      R z = R(0);
      freef.tau = Vec3<R>(z + (ap ? t.qfrc_applied[0] : z), z + (ap ? t.qfrc_applied[1] : z), z + (ap ? t.qfrc_applied[2] : z));
      freef.lin = Vec3<R>(z + (ap ? t.qfrc_applied[3] : z), z + (ap ? t.qfrc_applied[4] : z), z + (ap ? t.qfrc_applied[5] : z));
    } else if (L.type == J_HINGE || L.type == J_SLIDE) {
      int vo = t.v_off[i];
      R qd = t.qdot[vo];
      // qfrc_applied + tendon(0) - damping*qdot + limit(0) + actuators(-0)
      scalar[i] = ((t.qfrc_applied[vo] + R(0)) - L.damping * qd) + R(0);
    } else if (L.type == J_BALL) {
      int o = t.v_off[i];
      ball[i] = Vec3<R>((t.qfrc_applied[o] + R(0)) - L.damping * t.qdot[o],
                        (t.qfrc_applied[o + 1] + R(0)) - L.damping * t.qdot[o + 1],
                        (t.qfrc_applied[o + 2] + R(0)) - L.damping * t.qdot[o + 2]);
    }
  }
  std::vector<GForce<R>> ext_body(n);
  std::vector<R> dmass(n, R(0));
  for (int i = 0; i < n; ++i) {
    const Link<R>& L = t.links[i];
    // tree.rs:1060-1064: applied_wrenches are zero in this restatement.
    Vec3<R> fb = poses[i].o.inverse_rotate((ext[i].f + Vec3<R>()) + gravity * L.mass);
    Vec3<R> tb = poses[i].o.inverse_rotate(ext[i].t + Vec3<R>());
    ext_body[i] = {tb, fb};
    switch (L.type) {
      case J_HINGE: case J_SLIDE: dmass[i] = implicit_dt == R(0) ? R(0) : implicit_dt * (L.damping + R(0)); break;
      case J_BALL: dmass[i] = implicit_dt * L.damping; break;
      case J_FREE: dmass[i] = implicit_dt * L.free_damping; break;
      default: dmass[i] = R(0);
    }
  }
  // aba::run
  std::vector<GX<R>> xup(n, GX<R>::identity());
  std::vector<GMotion<R>> S(n), v(n), c(n), a(n);
  std::vector<std::array<GMotion<R>, 3>> S3(n);
  std::vector<GM6<R>> IA(n);
  std::vector<GForce<R>> pA(n), IAs(n);
  std::vector<R> d(n, R(0)), tau(n, R(0));
  std::vector<GM3<R>> d3inv(n, GM3<R>::zero());
  const GMotion<R> zm{Vec3<R>(), Vec3<R>()};
  for (int i = 0; i < n; ++i) {
    const Link<R>& L = t.links[i];
    switch (L.type) {
      case J_FREE: {
        int o = t.v_off[i];
        xup[i] = GX<R>::identity();
        v[i] = {Vec3<R>(t.qdot[o], t.qdot[o + 1], t.qdot[o + 2]), Vec3<R>(t.qdot[o + 3], t.qdot[o + 4], t.qdot[o + 5])};
        c[i] = zm;
        break;
      }
      case J_FIXED: {
        xup[i] = xup_fixed(L);
        GMotion<R> pv = L.parent >= 0 ? v[L.parent] : zm;
        v[i] = xup[i].motion(pv);
        c[i] = zm;
        break;
      }
      case J_HINGE: case J_SLIDE: {
        GX<R> x = xup_joint(L, t.q[t.q_off[i]]);
        xup[i] = x;
        if (L.type == J_HINGE) S[i] = {L.axis, L.jc_pos.cross(L.axis)};
        else S[i] = {Vec3<R>(), L.axis};
        GMotion<R> sq = S[i].scale(t.qdot[t.v_off[i]]);
        v[i] = x.motion(v[L.parent]).add(sq);
        c[i] = v[i].cross_motion(sq);
        break;
      }
      case J_BALL: {
        int o = t.q_off[i];
        GM3<R> rot = GM3<R>::quat(R(0) - t.q[o], R(0) - t.q[o + 1], R(0) - t.q[o + 2], t.q[o + 3]);
        xup[i] = {rot, L.jc_pos - rot.mul_vec(L.jp_pos)};
        Vec3<R> r = L.jc_pos;
        for (int k = 0; k < 3; ++k) {
          Vec3<R> e(k == 0 ? R(1) : R(0), k == 1 ? R(1) : R(0), k == 2 ? R(1) : R(0));
          S3[i][k] = {e, r.cross(e)};
        }
        int vo = t.v_off[i];
        GMotion<R> sq = S3[i][0].scale(t.qdot[vo]).add(S3[i][1].scale(t.qdot[vo + 1])).add(S3[i][2].scale(t.qdot[vo + 2]));
        v[i] = xup[i].motion(v[L.parent]).add(sq);
        c[i] = v[i].cross_motion(sq);
        break;
      }
    }
  }
  for (int i = 0; i < n; ++i) {
    GM6<R> I = gm6_from_inertia(t.links[i].mass, t.links[i].inertia);
    IA[i] = I;
    pA[i] = cross_force(v[i], I.times_motion(v[i])).sub(ext_body[i]);
  }
  for (int i = n - 1; i >= 1; --i) {
    const Link<R>& L = t.links[i];
    int p = L.parent;
    if (L.type == J_FIXED) {
      IA[p] = IA[p].add(IA[i].pull_back(xup[i]));
      pA[p] = pA[p].add(xup[i].transpose_force(pA[i].add(IA[i].times_motion(c[i]))));
    } else if (L.type == J_HINGE || L.type == J_SLIDE) {
      GForce<R> ias = IA[i].times_motion(S[i]);
      R dd = (dot_force(S[i], ias) + L.armature) + dmass[i];
      GForce<R> ps = pA[i].add(IA[i].times_motion(c[i]));
      R u = scalar[i] - dot_force(S[i], ps);
      R qdd = u / dd;
      GForce<R> pfull = ps.add(ias.scale(qdd));
      R invd = R(1) / dd;
      GM6<R> ifull = IA[i].sub(GM6<R>::outer(ias, GMotion<R>{ias.tau, ias.lin}).scale(invd));
      IAs[i] = ias; d[i] = dd; tau[i] = scalar[i];
      IA[p] = IA[p].add(ifull.pull_back(xup[i]));
      pA[p] = pA[p].add(xup[i].transpose_force(pfull));
    } else if (L.type == J_BALL) {
      std::array<GMotion<R>, 3>& s3 = S3[i];
      GForce<R> is3[3] = {IA[i].times_motion(s3[0]), IA[i].times_motion(s3[1]), IA[i].times_motion(s3[2])};
      GM3<R> D = GM3<R>::zero();
      for (int r = 0; r < 3; ++r) for (int cc = 0; cc < 3; ++cc) D.a[r][cc] = dot_force(s3[r], is3[cc]);
      for (int k = 0; k < 3; ++k) D.a[k][k] = (D.a[k][k] + L.armature) + dmass[i];
      GM3<R> Dinv = D.inverse();
      GForce<R> ps = pA[i].add(IA[i].times_motion(c[i]));
      Vec3<R> sp(dot_force(s3[0], ps), dot_force(s3[1], ps), dot_force(s3[2], ps));
      Vec3<R> qdd = Dinv.mul_vec(ball[i] - sp);
      GForce<R> pfull = ps.add(is3[0].scale(qdd.x)).add(is3[1].scale(qdd.y)).add(is3[2].scale(qdd.z));
      GM6<R> ifull = IA[i];
      for (int cc = 0; cc < 3; ++cc) {
        GForce<R> acol{Vec3<R>(), Vec3<R>()};
        for (int r = 0; r < 3; ++r) acol = acol.add(is3[r].scale(Dinv.a[r][cc]));
        ifull = ifull.sub(GM6<R>::outer(acol, GMotion<R>{is3[cc].tau, is3[cc].lin}));
      }
      d3inv[i] = Dinv;
      IA[p] = IA[p].add(ifull.pull_back(xup[i]));
      pA[p] = pA[p].add(xup[i].transpose_force(pfull));
    }
  }
  qacc.assign(nv, R(0));
  if (t.links[0].type == J_FREE) {
    GForce<R> rhs = freef.sub(pA[0]);
    R damping = t.links[0].free_damping;
    if (damping != R(0)) {
      int o = t.v_off[0];
      Vec3<R> wa(t.qdot[o], t.qdot[o + 1], t.qdot[o + 2]), wl(t.qdot[o + 3], t.qdot[o + 4], t.qdot[o + 5]);
      rhs = rhs.sub(GForce<R>{wa * damping, wl * damping});
      for (int k = 0; k < 6; ++k) IA[0].m[k][k] = IA[0].m[k][k] + dmass[0];
    }
    GMotion<R> root = IA[0].solve(rhs);
    a[0] = root;
    int o = t.v_off[0];
    qacc[o] = root.ang.x; qacc[o + 1] = root.ang.y; qacc[o + 2] = root.ang.z;
    qacc[o + 3] = root.lin.x; qacc[o + 4] = root.lin.y; qacc[o + 5] = root.lin.z;
  } else {
    a[0] = zm;
  }
  for (int i = 1; i < n; ++i) {
    const Link<R>& L = t.links[i];
    int p = L.parent;
    if (L.type == J_FIXED) {
      a[i] = xup[i].motion(a[p]);
    } else if (L.type == J_HINGE || L.type == J_SLIDE) {
      GMotion<R> prime = xup[i].motion(a[p]).add(c[i]);
      GForce<R> inner = IA[i].times_motion(prime).add(pA[i]);
      R qdd = (scalar[i] - dot_force(S[i], inner)) / d[i];
      a[i] = prime.add(S[i].scale(qdd));
      qacc[t.v_off[i]] = qdd;
    } else if (L.type == J_BALL) {
      GMotion<R> prime = xup[i].motion(a[p]).add(c[i]);
      GForce<R> inner = IA[i].times_motion(prime).add(pA[i]);
      std::array<GMotion<R>, 3>& s3 = S3[i];
      Vec3<R> rhs(ball[i].x - dot_force(s3[0], inner), ball[i].y - dot_force(s3[1], inner), ball[i].z - dot_force(s3[2], inner));
      Vec3<R> qdd = d3inv[i].mul_vec(rhs);
      a[i] = prime.add(s3[0].scale(qdd.x)).add(s3[1].scale(qdd.y)).add(s3[2].scale(qdd.z));
      int o = t.v_off[i];
      qacc[o] = qdd.x; qacc[o + 1] = qdd.y; qacc[o + 2] = qdd.z;
    }
  }
}

// tree.rs:1422-1475
template <class R> void integrate_tree_positions(Tree<R>& t, R dt) {
  for (size_t i = 0; i < t.links.size(); ++i) {
    const Link<R>& L = t.links[i];
    int qo = t.q_off[i], vo = t.v_off[i];
    switch (L.type) {
      case J_FREE: {
        Quat<R> ori(t.q[qo + 3], t.q[qo + 4], t.q[qo + 5], t.q[qo + 6]);
        Vec3<R> om(t.qdot[vo], t.qdot[vo + 1], t.qdot[vo + 2]);
        Vec3<R> vel(t.qdot[vo + 3], t.qdot[vo + 4], t.qdot[vo + 5]);
        Vec3<R> dp = ori.rotate(vel) * dt;
        t.q[qo] += dp.x; t.q[qo + 1] += dp.y; t.q[qo + 2] += dp.z;
        Quat<R> nx = ori.integrate_body_angular_velocity(om, dt);
        t.q[qo + 3] = nx.x; t.q[qo + 4] = nx.y; t.q[qo + 5] = nx.z; t.q[qo + 6] = nx.w;
        break;
      }
      case J_HINGE: case J_SLIDE: t.q[qo] += t.qdot[vo] * dt; break;
      case J_BALL: {
        Quat<R> ori(t.q[qo], t.q[qo + 1], t.q[qo + 2], t.q[qo + 3]);
        Vec3<R> om(t.qdot[vo], t.qdot[vo + 1], t.qdot[vo + 2]);
        Quat<R> nx = ori.integrate_body_angular_velocity(om, dt);
        t.q[qo] = nx.x; t.q[qo + 1] = nx.y; t.q[qo + 2] = nx.z; t.q[qo + 3] = nx.w;
        break;
      }
      default: break;
    }
  }
}

// tree.rs:1485-1550 (tree_deriv): dq from the stage state, dv = qddot.
template <class R> void tree_deriv(const Tree<R>& t, const std::vector<R>& qdd, std::vector<R>& dq, std::vector<R>& dv) {
  dq.assign(t.q.size(), R(0));
  dv = qdd;
  for (size_t i = 0; i < t.links.size(); ++i) {
    const int qo = t.q_off[i], vo = t.v_off[i];
    switch (t.links[i].type) {
      case J_FREE: {
        const Quat<R> ori(t.q[qo + 3], t.q[qo + 4], t.q[qo + 5], t.q[qo + 6]);
        const Vec3<R> wb(t.qdot[vo], t.qdot[vo + 1], t.qdot[vo + 2]);
        const Vec3<R> vb(t.qdot[vo + 3], t.qdot[vo + 4], t.qdot[vo + 5]);
        const Vec3<R> vw = ori.rotate(vb);
        dq[qo] = vw.x; dq[qo + 1] = vw.y; dq[qo + 2] = vw.z;
        const Quat<R> d = ori.derivative(wb);
        dq[qo + 3] = d.x; dq[qo + 4] = d.y; dq[qo + 5] = d.z; dq[qo + 6] = d.w;
        break;
      }
      case J_HINGE: case J_SLIDE: dq[qo] = t.qdot[vo]; break;
      case J_BALL: {
        const Quat<R> qb(t.q[qo], t.q[qo + 1], t.q[qo + 2], t.q[qo + 3]);
        const Quat<R> d = qb.derivative(Vec3<R>(t.qdot[vo], t.qdot[vo + 1], t.qdot[vo + 2]));
        dq[qo] = d.x; dq[qo + 1] = d.y; dq[qo + 2] = d.z; dq[qo + 3] = d.w;
        break;
      }
      default: break;
    }
  }
}

// tree.rs:1234-1364 (rk4_step_with_workspace): four explicit ABA stages with
// the external wrenches held at zero (solver mode), then quaternion
// renormalisation of free and ball joints.  No actuators, no mocap roots.
template <class R> void rk4_step_tree(Tree<R>& t, Vec3<R> gravity, R dt) {
  const std::vector<R> q0 = t.q, v0 = t.qdot;
  const std::vector<Wrench<R>> ext(t.links.size(), Wrench<R>{Vec3<R>(), Vec3<R>()});
  std::vector<Pose<R>> poses;
  std::vector<R> qdd, dq[4], dv[4];
  for (int s = 0; s < 4; ++s) {
    forward_kinematics(t, poses);
    aba(t, poses, gravity, ext, R(0), qdd);
    tree_deriv(t, qdd, dq[s], dv[s]);
    if (s == 3) break;
    const R h = s < 2 ? dt * R(0.5) : dt;
    for (size_t j = 0; j < q0.size(); ++j) t.q[j] = q0[j] + dq[s][j] * h;
    for (size_t j = 0; j < v0.size(); ++j) t.qdot[j] = v0[j] + dv[s][j] * h;
  }
  const R sixth = R(1) / R(6);
  for (size_t j = 0; j < q0.size(); ++j)
    t.q[j] = q0[j] + (dq[0][j] + R(2) * dq[1][j] + R(2) * dq[2][j] + dq[3][j]) * (dt * sixth);
  for (size_t j = 0; j < v0.size(); ++j)
    t.qdot[j] = v0[j] + (dv[0][j] + R(2) * dv[1][j] + R(2) * dv[2][j] + dv[3][j]) * (dt * sixth);
  for (size_t i = 0; i < t.links.size(); ++i) {
    const int type = t.links[i].type;
    if (!(type == J_FREE && i == 0) && type != J_BALL) continue;
    const int o = t.q_off[i] + (type == J_FREE ? 3 : 0);
    const Quat<R> q = Quat<R>(t.q[o], t.q[o + 1], t.q[o + 2], t.q[o + 3]).renormalize();
    t.q[o] = q.x; t.q[o + 1] = q.y; t.q[o + 2] = q.z; t.q[o + 3] = q.w;
  }
}

// tree.rs:1393-1420 (non-implicit-fast Euler; no mocap roots).  Returns the
// qacc used for the step through `qacc_out` when it is non-null.
template <class R> void euler_step_tree(Tree<R>& t, Vec3<R> gravity, R dt, std::vector<R>* qacc_out = nullptr) {
  std::vector<Pose<R>> poses;
  forward_kinematics(t, poses);
  std::vector<Wrench<R>> ext(t.links.size(), Wrench<R>{Vec3<R>(), Vec3<R>()});
  std::vector<R> qdd;
  aba(t, poses, gravity, ext, dt, qdd);
  for (int i = 0; i < t.nv(); ++i) t.qdot[i] += qdd[i] * dt;
  integrate_tree_positions(t, dt);
  if (qacc_out) *qacc_out = qdd;
}

// ---------------------------------------------------------------------------
// CRB mass matrix + Cholesky (dynamics.rs)
// ---------------------------------------------------------------------------
template <class R> Xform<R> xup_xform(const Tree<R>& t, int i) {  // dynamics.rs:151-180
  const Link<R>& L = t.links[i];
  Xform<R> x{Mat3<R>(), Vec3<R>()};
  switch (L.type) {
    case J_FREE: break;
    case J_FIXED: {
      Quat<R> rel = L.jp_ori * L.jc_ori.conjugate();
      x.rot = rel.conjugate().to_mat3();
      x.trans = L.jc_pos - x.rot * L.jp_pos;
      break;
    }
    case J_HINGE: {  // tree.rs:1130-1136
      x.rot = Quat<R>::from_axis_angle(L.axis, -t.q[t.q_off[i]]).to_mat3();
      x.trans = L.jc_pos - x.rot * L.jp_pos;
      break;
    }
    case J_SLIDE: x.trans = L.jc_pos - L.jp_pos - L.axis * t.q[t.q_off[i]]; break;
    case J_BALL: {
      int o = t.q_off[i];
      Quat<R> qb(t.q[o], t.q[o + 1], t.q[o + 2], t.q[o + 3]);
      x.rot = qb.conjugate().to_mat3();
      x.trans = L.jc_pos - x.rot * L.jp_pos;
      break;
    }
  }
  return x;
}

template <class R> void mass_matrix(const Tree<R>& t, std::vector<R>& M) {  // dynamics.rs:474-578
  const int n = (int)t.links.size(), nv = t.nv();
  M.assign((size_t)nv * nv, R(0));
  if (nv == 0) return;
  std::vector<Xform<R>> xup(n);
  for (int i = 0; i < n; ++i) xup[i] = xup_xform(t, i);
  std::vector<Mat6<R>> ic(n);
  for (int i = 0; i < n; ++i) ic[i] = Mat6<R>::from_spatial_inertia(t.links[i].mass, Vec3<R>(), t.links[i].inertia);
  for (int i = n - 1; i >= 1; --i) {
    int p = t.links[i].parent;
    if (p >= 0) ic[p] = ic[p].plus(ic[i].pull_back(xup[i]));
  }
  if (t.links[0].type == J_FREE) {
    int o = t.v_off[0];
    for (int r = 0; r < 6; ++r) for (int c = 0; c < 6; ++c) M[(o + r) * nv + o + c] = ic[0].m[r][c];
  }
  for (int i = 1; i < n; ++i) {
    const Link<R>& L = t.links[i];
    int vi = t.v_off[i];
    std::vector<SMotion<R>> cols;
    if (L.type == J_FIXED) continue;
    if (L.type == J_HINGE) cols.push_back({L.axis, L.jc_pos.cross(L.axis)});
    else if (L.type == J_SLIDE) cols.push_back({Vec3<R>(), L.axis});
    else if (L.type == J_BALL) for (int k = 0; k < 3; ++k) { Vec3<R> e(k == 0, k == 1, k == 2); cols.push_back({e, L.jc_pos.cross(e)}); }
    for (size_t k = 0; k < cols.size(); ++k) {
      SForce<R> f = ic[i].times_motion(cols[k]);
      for (size_t kp = 0; kp < cols.size(); ++kp) M[(vi + kp) * nv + vi + k] = sdot(cols[kp], f);
      M[(vi + k) * nv + vi + k] += L.armature;
      int jc = i;
      while (t.links[jc].parent >= 0) {
        int j = t.links[jc].parent;
        f = xup[jc].transpose_force(f);
        jc = j;
        int vj = t.v_off[j];
        const Link<R>& PL = t.links[j];
        if (PL.type == J_HINGE || PL.type == J_SLIDE) {
          SMotion<R> s = PL.type == J_HINGE ? SMotion<R>{PL.axis, PL.jc_pos.cross(PL.axis)} : SMotion<R>{Vec3<R>(), PL.axis};
          R val = sdot(s, f);
          M[vj * nv + vi + k] = val; M[(vi + k) * nv + vj] = val;
        } else if (PL.type == J_BALL) {
          for (int kk = 0; kk < 3; ++kk) {
            Vec3<R> e(kk == 0, kk == 1, kk == 2);
            R val = sdot(SMotion<R>{e, PL.jc_pos.cross(e)}, f);
            M[(vj + kk) * nv + vi + k] = val; M[(vi + k) * nv + vj + kk] = val;
          }
        } else if (PL.type == J_FREE) {
          R fc[6] = {f.tau.x, f.tau.y, f.tau.z, f.lin.x, f.lin.y, f.lin.z};
          for (int kk = 0; kk < 6; ++kk) { M[(vj + kk) * nv + vi + k] = fc[kk]; M[(vi + k) * nv + vj + kk] = fc[kk]; }
        }
      }
    }
  }
}

// tree.rs:645-684 with implicit_fast = false.
template <class R> void implicit_mass_matrix(const Tree<R>& t, R dt, std::vector<R>& M) {
  mass_matrix(t, M);
  const int nv = t.nv();
  if (nv == 0 || dt == R(0)) return;
  for (size_t i = 0; i < t.links.size(); ++i) {
    const Link<R>& L = t.links[i];
    int o = t.v_off[i];
    R dmp;
    if (L.type == J_FREE) dmp = L.free_damping;
    else if (L.type == J_HINGE || L.type == J_SLIDE) dmp = L.damping + R(0);
    else if (L.type == J_BALL) dmp = L.damping;
    else continue;
    for (int s = o; s < o + joint_nv(L.type); ++s) M[s * nv + s] += dt * dmp;
  }
}

template <class R> bool cholesky(const std::vector<R>& a, int n, std::vector<R>& l) {  // dynamics.rs:602-622
  l.assign((size_t)n * n, R(0));
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= i; ++j) {
      R sum = a[i * n + j];
      for (int k = 0; k < j; ++k) sum -= l[i * n + k] * l[j * n + k];
      if (i == j) {
        if (sum <= R(0)) return false;
        l[i * n + i] = Sc<R>::sqrt(sum);
      } else {
        l[i * n + j] = sum / l[j * n + j];
      }
    }
  return true;
}

template <class R> void cholesky_solve(const std::vector<R>& l, int n, const R* b, R* x) {  // dynamics.rs:626-648
  std::vector<R> y(n);
  for (int i = 0; i < n; ++i) {
    R sum = b[i];
    for (int k = 0; k < i; ++k) sum -= l[i * n + k] * y[k];
    y[i] = sum / l[i * n + i];
  }
  for (int i = n - 1; i >= 0; --i) {
    R sum = y[i];
    for (int k = i + 1; k < n; ++k) sum -= l[k * n + i] * x[k];
    x[i] = sum / l[i * n + i];
  }
}

}  // namespace oracle
