// Post-step sensors: one thread per world walks the tree (forward kinematics
// and link velocities) or reads the free bodies, then writes every requested
// sensor's values into the world's output row.  Accelerometer and touch
// readings on pile worlds come from newt's post-step contact re-solve
// (pile_kernels.cu: pile_k_reassemble, the solvers, then
// pile_contact_sensors_kernel), run for the group before its sensors;
// accelerometer, force and torque readings on trees from the links' dynamics
// pass (tree_kernels.cu: tree_sensor_dyn_kernel), on tree-contact worlds
// under the wrenches of the contact re-solve (newton_kernels.cu:
// newt_tc_resolve), which also gives their touch readings.
//
// Restates, for FP32 on sm_103a:
//   newt/src/sensor.rs:560-700   evaluate (JointPos, JointVel, FramePos,
//                                FrameQuat, Gyro, Velocimeter, SubtreeCom,
//                                FrameLinVel, FrameAngVel)
//   newt/src/sensor.rs:705-757   site_velocity, subtree_com
//   newt/src/sensor.rs:794-828   site_world_pose, parent_body_velocities
//   newt/src/tree.rs:771-858     forward_kinematics (link poses)
// Link velocities are propagated in the world frame (angular rate and the link
// origin's velocity) and rotated into the link frame at the end; newt
// propagates the body-frame spatial velocity (sensor.rs:834-900).  Both give
// the same vectors up to rounding.
#include <vector>

#include "../../include/newt_gpu.h"
#include "common.cuh"
#include "groups.h"
#include "runtime.h"

namespace {

enum { JF = 0, JX = 1, JH = 2, JS = 3 };

__host__ __device__ int sensor_dim(int kind) {
  return kind <= NEWT_SENSOR_JOINTVEL || kind == NEWT_SENSOR_TOUCH || kind == NEWT_SENSOR_RANGEFINDER
             ? 1 : (kind == NEWT_SENSOR_FRAMEQUAT ? 4 : 3);
}
__host__ __device__ bool contact_sensor(int kind) {
  return kind == NEWT_SENSOR_ACCELEROMETER || kind == NEWT_SENSOR_TOUCH;
}
// kinds read from the links' dynamics pass on trees (tree_sensor_dyn_kernel)
__host__ __device__ bool dyn_sensor(int kind) {
  return kind == NEWT_SENSOR_ACCELEROMETER || kind == NEWT_SENSOR_FORCE || kind == NEWT_SENSOR_TORQUE;
}

NEWT_D Q4 axis_angle(V3 axis, float angle) {  // newt/src/math.rs:574-580
  const float l = sqrtf(len2(axis));
  const V3 a = l > 0.f ? axis * (1.f / l) : v3(0.f, 0.f, 0.f);
  float s, c;
  sincosf(angle * 0.5f, &s, &c);
  return Q4{a.x * s, a.y * s, a.z * s, c};
}

// The site's parent frame: pose, world angular velocity, the velocity of its
// origin (the body's or link's centre of mass), and the body-frame angular
// velocity.
struct Frame { V3 p; Q4 o; V3 w_world, v_world, w_body; };

// ray_vs_geom (newt/src/scene_query.rs:182-438, no meshes): the distance
// along the ray (origin o, direction dv, in the geom's frame) to its first
// hit at or beyond 0 -- the far root when the ray starts inside -- or -1.
NEWT_D float ray_sphere_at(V3 c, float r, V3 o, V3 dv) {
  const V3 off = o - c;
  const float a = dot(dv, dv);
  if (a <= 0.f) return -1.f;
  const float hb = dot(off, dv), cc = dot(off, off) - r * r;
  const float disc = hb * hb - a * cc;
  if (disc < 0.f) return -1.f;
  const float root = sqrtf(disc);
  const float nr = (-hb - root) / a, fr = (-hb + root) / a;
  const float t = nr >= 0.f ? nr : fr;
  return t >= 0.f ? t : -1.f;
}
NEWT_D float ray_cyl_side(float r, float hh, V3 o, V3 dv) {
  const float a = dv.x * dv.x + dv.y * dv.y;
  if (a <= 1.0e-8f) return -1.f;
  const float hb = o.x * dv.x + o.y * dv.y, cc = o.x * o.x + o.y * o.y - r * r;
  const float disc = hb * hb - a * cc;
  if (disc < 0.f) return -1.f;
  const float root = sqrtf(disc);
  float best = -1.f;
  const float ts[2] = {(-hb - root) / a, (-hb + root) / a};
  for (int k = 0; k < 2; ++k) {
    const float t = ts[k];
    if (t >= 0.f) {
      const float z = o.z + dv.z * t;
      if (z >= -hh && z <= hh && (best < 0.f || t < best)) best = t;
    }
  }
  return best;
}
NEWT_D float ray_geom(int shape, V3 sz, V3 o, V3 dv) {
  if (!(dot(dv, dv) > 0.f)) return -1.f;
  switch (shape) {
    case NEWT_SHAPE_SPHERE: return ray_sphere_at(v3(0.f, 0.f, 0.f), sz.x, o, dv);
    case NEWT_SHAPE_PLANE: {
      if (dv.z == 0.f) return -1.f;
      const float t = -o.z / dv.z;
      return t >= 0.f ? t : -1.f;
    }
    case NEWT_SHAPE_BOX: {
      float nr = -INFINITY, fr = INFINITY;
      const float oa[3] = {o.x, o.y, o.z}, da[3] = {dv.x, dv.y, dv.z}, ea[3] = {sz.x, sz.y, sz.z};
      for (int k = 0; k < 3; ++k) {
        if (da[k] == 0.f) {
          if (fabsf(oa[k]) > ea[k]) return -1.f;
          continue;
        }
        float an = (-ea[k] - oa[k]) / da[k], af = (ea[k] - oa[k]) / da[k];
        if (an > af) { const float x = an; an = af; af = x; }
        if (an > nr) nr = an;
        if (af < fr) fr = af;
        if (nr > fr) return -1.f;
      }
      const float t = nr >= 0.f ? nr : fr;
      return t >= 0.f ? t : -1.f;
    }
    case NEWT_SHAPE_CAPSULE: {
      float best = ray_cyl_side(sz.x, sz.y, o, dv);
      const float lo = ray_sphere_at(v3(0.f, 0.f, -sz.y), sz.x, o, dv);
      if (lo >= 0.f && (best < 0.f || lo < best)) best = lo;
      const float hi = ray_sphere_at(v3(0.f, 0.f, sz.y), sz.x, o, dv);
      if (hi >= 0.f && (best < 0.f || hi < best)) best = hi;
      return best;
    }
    case NEWT_SHAPE_CYLINDER: {
      float best = ray_cyl_side(sz.x, sz.y, o, dv);
      if (dv.z != 0.f)
        for (int k = 0; k < 2; ++k) {
          const float t = ((k ? sz.y : -sz.y) - o.z) / dv.z;
          if (t >= 0.f) {
            const float px = o.x + dv.x * t, py = o.y + dv.y * t;
            if (px * px + py * py <= sz.x * sz.x && (best < 0.f || t < best)) best = t;
          }
        }
      return best;
    }
    case NEWT_SHAPE_ELLIPSOID: {
      const V3 so = v3(o.x / sz.x, o.y / sz.y, o.z / sz.z), sd = v3(dv.x / sz.x, dv.y / sz.y, dv.z / sz.z);
      const float a = dot(sd, sd);
      if (a <= 0.f) return -1.f;
      const float hb = dot(so, sd), cc = dot(so, so) - 1.f;
      const float disc = hb * hb - a * cc;
      if (disc < 0.f) return -1.f;
      const float root = sqrtf(disc);
      const float nr = (-hb - root) / a, fr = (-hb + root) / a;
      const float t = nr >= 0.f ? nr : fr;
      return t >= 0.f ? t : -1.f;
    }
    default: return -1.f;
  }
}
// The nearest hit over a world's geoms (rangefinder_reading,
// sensor.rs:759-791): `geom(i, &shape, &size, &pose)` gives geom i's world pose.
template <class G>
NEWT_D float rangefinder(int ng, G geom, V3 origin, V3 dir) {
  float nearest = -1.f;
  for (int i = 0; i < ng; ++i) {
    int shape;
    V3 sz, gp;
    Q4 go;
    geom(i, &shape, &sz, &gp, &go);
    const float t = ray_geom(shape, sz, qrot_inv(go, origin - gp), qrot_inv(go, dir));
    if (t >= 0.f && (nearest < 0.f || t < nearest)) nearest = t;
  }
  return nearest;
}

// `mag`: the world's magnetic field; `ng`, `geom`: its geoms (rangefinder).
template <class G>
NEWT_D void write_sensors(const newt_sensor_desc* S, int ns, const Frame* frames, const float* q, const float* qd,
                          const int* qoff, const int* voff, float* row, const V3* subtree_com, V3 mag, int ng,
                          G geom) {
  int o = 0;
  for (int k = 0; k < ns; ++k) {
    const newt_sensor_desc& s = S[k];
    const int kind = s.kind;
    if (contact_sensor(kind) || dyn_sensor(kind)) { o += sensor_dim(kind); continue; }  // written apart
    if (kind == NEWT_SENSOR_JOINTPOS) { row[o++] = q[qoff[s.index]]; continue; }
    if (kind == NEWT_SENSOR_JOINTVEL) { row[o++] = qd[voff[s.index]]; continue; }
    if (kind == NEWT_SENSOR_SUBTREECOM) {
      const V3 c = subtree_com[k];
      row[o++] = c.x; row[o++] = c.y; row[o++] = c.z;
      continue;
    }
    const Frame& f = frames[k];
    const V3 lp = v3(s.local_pos[0], s.local_pos[1], s.local_pos[2]);
    const Q4 lq{s.local_quat[0], s.local_quat[1], s.local_quat[2], s.local_quat[3]};
    V3 r;
    switch (kind) {
      case NEWT_SENSOR_FRAMEPOS: r = f.p + qrot(f.o, lp); break;
      case NEWT_SENSOR_FRAMEQUAT: {
        const Q4 so = qmul(f.o, lq);
        row[o++] = so.x; row[o++] = so.y; row[o++] = so.z; row[o++] = so.w;
        continue;
      }
      case NEWT_SENSOR_GYRO: r = qrot_inv(lq, f.w_body); break;
      case NEWT_SENSOR_MAGNETOMETER: r = qrot_inv(qmul(f.o, lq), mag); break;  // sensor.rs:664-670
      case NEWT_SENSOR_RANGEFINDER:  // along the site's +z (sensor.rs:671-682)
        row[o++] = rangefinder(ng, geom, f.p + qrot(f.o, lp), qrot(qmul(f.o, lq), v3(0.f, 0.f, 1.f)));
        continue;
      case NEWT_SENSOR_FRAMEANGVEL: r = f.w_world; break;
      default: {  // site linear velocity: origin velocity plus w x (R lp)
        const V3 lin = f.v_world + cross(f.w_world, qrot(f.o, lp));
        r = kind == NEWT_SENSOR_VELOCIMETER ? qrot_inv(qmul(f.o, lq), lin) : lin;
      }
    }
    row[o++] = r.x; row[o++] = r.y; row[o++] = r.z;
  }
}

// Tree worlds (trees without geoms and tree-contact worlds): newt layout q/qd
// in the group's SoA rows.  Frames for link sensors and subtree centres are
// collected per sensor as the links are walked.
// `dyn` (when an accelerometer, force or torque sensor is asked for): the
// links' dynamics pass, 18 floats per link of each world.  `sens`
// (tree-contact worlds, when a contact-dependent sensor is asked for): the
// contact re-solve's output (newt_tc_resolve), `sens_stride` floats per
// world, its contact list after 6 L floats of link wrenches, the count at
// 6 L + 3 maxc.
template <int MAXL>
__global__ void __launch_bounds__(64) tree_sensors_kernel(TreeGroupDev g, const int* idx, int n,
                                                         const newt_sensor_desc* S, int ns, float* out, int D,
                                                         const float* dyn, const float* sens, long sens_stride,
                                                         int maxc, const float* mag, const float* tgeom,
                                                         const int* tgtopo, int tng) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int w = idx[t], cap = g.cap, L = g.L;
  float q[MAXL + 6], qd[MAXL + 5];
  for (int k = 0; k < g.nq; ++k) q[k] = g.q[k * cap + w];
  for (int k = 0; k < g.nv; ++k) qd[k] = g.qd[k * cap + w];
  V3 P[MAXL], Wn[MAXL], Vn[MAXL];
  Q4 O[MAXL];
  int qoff[MAXL], voff[MAXL];
  for (int i = 0; i < L; ++i) {
    const int parent = g.topo[4 * i], jt = g.topo[4 * i + 1], qo = g.topo[4 * i + 2], vo = g.topo[4 * i + 3];
    qoff[i] = qo; voff[i] = vo;
    const V3 jp = v3(g.jp[(3 * i) * cap + w], g.jp[(3 * i + 1) * cap + w], g.jp[(3 * i + 2) * cap + w]);
    const V3 jc = v3(g.jc[(3 * i) * cap + w], g.jc[(3 * i + 1) * cap + w], g.jc[(3 * i + 2) * cap + w]);
    if (i == 0) {
      if (jt == JF) {
        P[0] = v3(q[qo], q[qo + 1], q[qo + 2]);
        O[0] = Q4{q[qo + 3], q[qo + 4], q[qo + 5], q[qo + 6]};
        Wn[0] = qrot(O[0], v3(qd[vo], qd[vo + 1], qd[vo + 2]));
        Vn[0] = qrot(O[0], v3(qd[vo + 3], qd[vo + 4], qd[vo + 5]));
      } else {
        O[0] = Q4{g.rootq[w], g.rootq[cap + w], g.rootq[2 * cap + w], g.rootq[3 * cap + w]};
        P[0] = jp - qrot(O[0], jc);
        Wn[0] = v3(0.f, 0.f, 0.f);
        Vn[0] = v3(0.f, 0.f, 0.f);
      }
      continue;
    }
    const V3 ax = v3(g.axis[(3 * i) * cap + w], g.axis[(3 * i + 1) * cap + w], g.axis[(3 * i + 2) * cap + w]);
    const Q4 po = O[parent];
    const V3 anchor = P[parent] + qrot(po, jp);
    V3 wrel = v3(0.f, 0.f, 0.f), vrel = v3(0.f, 0.f, 0.f);
    if (jt == JH) {
      O[i] = qmul(po, axis_angle(ax, q[qo]));
      P[i] = anchor - qrot(O[i], jc);
      wrel = qrot(po, ax) * qd[vo];
      vrel = cross(wrel, P[i] - anchor);
    } else if (jt == JS) {
      O[i] = po;
      P[i] = anchor + qrot(po, ax * q[qo]) - qrot(O[i], jc);
      vrel = qrot(po, ax) * qd[vo];
    } else {
      O[i] = po;
      P[i] = anchor - qrot(O[i], jc);
    }
    Wn[i] = Wn[parent] + wrel;
    Vn[i] = Vn[parent] + cross(Wn[parent], P[i] - P[parent]) + vrel;
  }
  Frame fr[16];
  V3 com[16];
  for (int k = 0; k < ns && k < 16; ++k) {
    const newt_sensor_desc& s = S[k];
    const int l = s.index;
    if (s.kind == NEWT_SENSOR_SUBTREECOM) {  // sensor.rs:728-757: links whose parent chain reaches l
      V3 acc = v3(0.f, 0.f, 0.f);
      float m = 0.f;
      for (int j = 0; j < L; ++j) {
        int c = j;
        while (c > l) c = g.topo[4 * c];
        if (c != l) continue;
        const float mj = g.mass[j * cap + w];
        acc = acc + P[j] * mj;
        m += mj;
      }
      com[k] = m == 0.f ? v3(0.f, 0.f, 0.f) : acc / m;
      continue;
    }
    if (s.kind <= NEWT_SENSOR_JOINTVEL || contact_sensor(s.kind) || dyn_sensor(s.kind)) continue;
    fr[k] = Frame{P[l], O[l], Wn[l], Vn[l], qrot_inv(O[l], Wn[l])};
  }
  float* row = out + (size_t)t * D;
  // the world's geoms (tree-contact worlds; a tree without geoms has none)
  auto geom = [&](int i, int* shape, V3* sz, V3* gp, Q4* go) {
    auto gv = [&](int f) { return tgeom[(size_t)(TC_GREC * i + f) * cap + w]; };
    *shape = tgtopo[2 * i];
    const int link = tgtopo[2 * i + 1];
    *sz = v3(gv(0), gv(1), gv(2));
    const V3 lp = v3(gv(3), gv(4), gv(5));
    const Q4 lq{gv(6), gv(7), gv(8), gv(9)};
    if (link < 0) { *gp = lp; *go = lq; }
    else { *gp = P[link] + qrot(O[link], lp); *go = qmul(O[link], lq); }
  };
  write_sensors(S, ns, fr, q, qd, qoff, voff, row, com, v3(mag[3 * t], mag[3 * t + 1], mag[3 * t + 2]), tng, geom);
  if (sens) {  // touch: the re-solved normal forces of the geom's contacts (sensor.rs:1103-1112)
    const float* so = sens + (size_t)w * sens_stride;
    const int nc = min(max(__float_as_int(so[6 * L + 3 * maxc]), 0), maxc);
    int o = 0;
    for (int k = 0; k < ns; ++k) {
      if (S[k].kind == NEWT_SENSOR_TOUCH) {
        float sum = 0.f;
        for (int c = 0; c < nc; ++c) {
          const float* cc = so + 6 * L + 3 * c;
          if (__float_as_int(cc[0]) == S[k].index || __float_as_int(cc[1]) == S[k].index) sum += fabsf(cc[2]);
        }
        row[o] = sum;
      }
      o += sensor_dim(S[k].kind);
    }
  }
  if (!dyn) return;
  // sensor.rs:620-647 (force; torque at the joint anchor, tau - r_jc x F)
  // and :1030-1087 (accelerometer, the link branch: the spatial acceleration
  // made classical with w x v, then the site's point acceleration less g)
  const V3 grav = v3(g.dtg[cap + w], g.dtg[2 * cap + w], g.dtg[3 * cap + w]);
  int o = 0;
  for (int k = 0; k < ns; ++k) {
    const newt_sensor_desc& s = S[k];
    const int dim = sensor_dim(s.kind);
    if (!dyn_sensor(s.kind)) { o += dim; continue; }
    const int l = s.index;
    const float* d = dyn + ((size_t)t * L + l) * 18;
    const V3 vw = v3(d[0], d[1], d[2]), vv = v3(d[3], d[4], d[5]), aw = v3(d[6], d[7], d[8]), av = v3(d[9], d[10], d[11]);
    const V3 ft = v3(d[12], d[13], d[14]), ff = v3(d[15], d[16], d[17]);
    V3 r;
    if (s.kind == NEWT_SENSOR_FORCE) {
      r = ff;
    } else if (s.kind == NEWT_SENSOR_TORQUE) {
      r = ft - cross(v3(g.jc[(3 * l) * cap + w], g.jc[(3 * l + 1) * cap + w], g.jc[(3 * l + 2) * cap + w]), ff);
    } else {
      const Q4 ori = O[l];
      const V3 om = qrot(ori, vw), al = qrot(ori, aw), acom = qrot(ori, av + cross(vw, vv));
      const V3 rs = qrot(ori, v3(s.local_pos[0], s.local_pos[1], s.local_pos[2]));
      const V3 asite = acom + cross(al, rs) + cross(om, cross(om, rs));
      r = qrot_inv(qmul(ori, Q4{s.local_quat[0], s.local_quat[1], s.local_quat[2], s.local_quat[3]}), asite - grav);
    }
    row[o] = r.x; row[o + 1] = r.y; row[o + 2] = r.z;
    o += dim;
  }
}

// Pile worlds: free-body poses and velocities from the world-major record.
__global__ void __launch_bounds__(64) pile_sensors_kernel(PileGroupDev g, const int* idx, int n,
                                                         const newt_sensor_desc* S, int ns, float* out, int D,
                                                         const float* mag) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float* F = g.F + (size_t)idx[t] * g.lay.fstride;
  const int* I = g.I + (size_t)idx[t] * g.lay.istride;
  Frame fr[16];
  for (int k = 0; k < ns && k < 16; ++k) {
    const int b = S[k].index;
    if (S[k].kind == NEWT_SENSOR_TOUCH) continue;  // a geom index, read by the contact sensors' kernel
    const Q4 o{F[g.lay.quat + 4 * b], F[g.lay.quat + 4 * b + 1], F[g.lay.quat + 4 * b + 2], F[g.lay.quat + 4 * b + 3]};
    const V3 wb = v3(F[g.lay.omg + 3 * b], F[g.lay.omg + 3 * b + 1], F[g.lay.omg + 3 * b + 2]);
    fr[k] = Frame{v3(F[g.lay.pos + 3 * b], F[g.lay.pos + 3 * b + 1], F[g.lay.pos + 3 * b + 2]), o, qrot(o, wb),
                  v3(F[g.lay.vel + 3 * b], F[g.lay.vel + 3 * b + 1], F[g.lay.vel + 3 * b + 2]), wb};
  }
  // the world's geoms: one per body, then the static planes
  auto geom = [&](int i, int* shape, V3* sz, V3* gp, Q4* go) {
    if (i < g.nb) {
      const Q4 bo{F[g.lay.quat + 4 * i], F[g.lay.quat + 4 * i + 1], F[g.lay.quat + 4 * i + 2], F[g.lay.quat + 4 * i + 3]};
      const V3 bp = v3(F[g.lay.pos + 3 * i], F[g.lay.pos + 3 * i + 1], F[g.lay.pos + 3 * i + 2]);
      const Q4 lq{F[g.lay.gquat + 4 * i], F[g.lay.gquat + 4 * i + 1], F[g.lay.gquat + 4 * i + 2], F[g.lay.gquat + 4 * i + 3]};
      *shape = I[g.lay.shape + i];
      *sz = v3(F[g.lay.size + 3 * i], F[g.lay.size + 3 * i + 1], F[g.lay.size + 3 * i + 2]);
      *gp = bp + qrot(bo, v3(F[g.lay.gpos + 3 * i], F[g.lay.gpos + 3 * i + 1], F[g.lay.gpos + 3 * i + 2]));
      *go = qmul(bo, lq);
    } else {
      const float* p = F + g.lay.plane + 7 * (i - g.nb);
      *shape = NEWT_SHAPE_PLANE;
      *sz = v3(0.f, 0.f, 0.f);
      *gp = v3(p[0], p[1], p[2]);
      *go = Q4{p[3], p[4], p[5], p[6]};
    }
  };
  write_sensors(S, ns, fr, nullptr, nullptr, nullptr, nullptr, out + (size_t)t * D, nullptr,
                v3(mag[3 * t], mag[3 * t + 1], mag[3 * t + 2]), g.nb + g.np, geom);
}

int bad(newt_gpu_ctx* ctx, const char* msg) {
  ctx->err = msg;
  return NEWT_E_INVALID;
}

}  // namespace

extern "C" int newt_tree_bucket(int L);
extern "C" void newt_launch_tree_sensor_dyn(const TreeGroupDev& g, const int* idx, int n, float* out, const float* sens,
                                            long sens_stride, cudaStream_t st);
extern "C" int newt_tc_resolve(newt_gpu_ctx* ctx, HostGroup* g, float* sens, long sens_stride, float* afree,
                               float* cfrc, cudaStream_t st);
extern "C" long newt_tc_sens_stride(int L, int maxc);
extern "C" void newt_launch_pile_contact_sensors(const PileGroupDev& g, const int* idx, int n,
                                                 const newt_sensor_desc* S, int ns, float* out, int D,
                                                 cudaStream_t st);
int pile_resolve_group(newt_gpu_ctx* ctx, HostGroup* g);

int newt_gpu_read_sensors(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n, const newt_sensor_desc* sensors,
                          int32_t n_sensors, float* out) {
  if (!ctx || n < 0 || n_sensors < 0 || (n > 0 && (!slots || !out)) || (n_sensors > 0 && !sensors))
    return NEWT_E_INVALID;
  if (n_sensors > 16) return bad(ctx, "at most 16 sensors per call");
  if (n == 0 || n_sensors == 0) return NEWT_OK;
  cudaSetDevice(ctx->device);
  int D = 0;
  bool needs_resolve = false, needs_dyn = false;
  for (int k = 0; k < n_sensors; ++k) {
    if (sensors[k].kind < NEWT_SENSOR_JOINTPOS || sensors[k].kind > NEWT_SENSOR_RANGEFINDER)
      return bad(ctx, "unknown sensor kind");
    D += sensor_dim(sensors[k].kind);
    needs_resolve = needs_resolve || contact_sensor(sensors[k].kind);
    needs_dyn = needs_dyn || dyn_sensor(sensors[k].kind);
  }
  // validate every world against every sensor, and group the worlds
  std::vector<std::vector<int>> idx(ctx->groups.size()), rows(ctx->groups.size());
  for (int i = 0; i < n; ++i) {
    const int s = slots[i];
    if (s < 0 || s >= (int)ctx->slots.size() || !ctx->slots[s].live) return bad(ctx, "bad slot");
    const SlotRef& r = ctx->slots[s];
    const HostModel& m = ctx->models[r.model];
    const bool tree = m.kind != GK_PILE;
    for (int k = 0; k < n_sensors; ++k) {
      const newt_sensor_desc& d = sensors[k];
      const bool link_only = d.kind <= NEWT_SENSOR_JOINTVEL || d.kind == NEWT_SENSOR_SUBTREECOM ||
                             d.kind == NEWT_SENSOR_FORCE || d.kind == NEWT_SENSOR_TORQUE;
      if (d.kind == NEWT_SENSOR_TOUCH && m.kind == GK_TREE)
        return bad(ctx, "touch sensors read worlds with contacts (piles, tree-contact worlds)");
      if ((d.on_link != 0) != tree || (link_only && !d.on_link))
        return bad(ctx, "sensor attachment does not match the world (links for trees, bodies for piles)");
      const int lim = d.kind == NEWT_SENSOR_TOUCH ? m.n_geoms : (tree ? m.n_links : m.n_bodies);
      if (d.index < 0 || d.index >= lim) return bad(ctx, "sensor index out of range");
      if (d.kind <= NEWT_SENSOR_JOINTVEL && m.links[d.index].joint != NEWT_JOINT_HINGE &&
          m.links[d.index].joint != NEWT_JOINT_SLIDE)
        return bad(ctx, "joint sensors read hinge or slide links");
    }
    idx[r.group].push_back(r.index);
    rows[r.group].push_back(i);
  }
  // each device row's magnetic field (its world's model), rows grouped as dI
  std::vector<float> hmag;
  hmag.reserve(3 * (size_t)n);
  for (size_t gi = 0; gi < rows.size(); ++gi)
    for (int i : rows[gi]) {
      const HostModel& m = ctx->models[ctx->slots[slots[i]].model];
      hmag.insert(hmag.end(), m.mag, m.mag + 3);
    }
  cudaStream_t st = ctx->stream;
  newt_sensor_desc* dS = nullptr;
  int* dI = nullptr;
  float* dO = nullptr;
  float* dM = nullptr;
  cudaError_t e = cudaMallocAsync(&dS, sizeof(newt_sensor_desc) * n_sensors, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&dM, sizeof(float) * 3 * (size_t)n, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dM, hmag.data(), sizeof(float) * hmag.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&dI, sizeof(int) * n, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&dO, sizeof(float) * (size_t)n * D, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dS, sensors, sizeof(newt_sensor_desc) * n_sensors, cudaMemcpyHostToDevice, st);
  std::vector<int> order;  // the device rows' order: grouped
  int resolve_rc = NEWT_OK;
  std::vector<float> host((size_t)n * D);
  size_t base = 0;
  for (size_t gi = 0; gi < idx.size() && e == cudaSuccess; ++gi) {
    const int cnt = (int)idx[gi].size();
    if (cnt == 0) continue;
    e = cudaMemcpyAsync(dI + base, idx[gi].data(), sizeof(int) * cnt, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) break;
    HostGroup* g = ctx->groups[gi].get();
    const int grid = (cnt + 63) / 64;
    float* o = dO + base * D;
    if (g->kind == GK_PILE) {
      pile_sensors_kernel<<<grid, 64, 0, st>>>(g->pile_dev(), dI + base, cnt, dS, n_sensors, o, D, dM + 3 * base);
      if (needs_resolve) {
        resolve_rc = pile_resolve_group(ctx, g);
        if (resolve_rc != NEWT_OK) break;
        newt_launch_pile_contact_sensors(g->pile_dev(), dI + base, cnt, dS, n_sensors, o, D, st);
        ctx->launches += 1;
      }
    } else {
      const TreeGroupDev td = g->tree_dev();
      // tree-contact worlds: the last step's contacts re-solved at the
      // current state, for the touch readings and as the links' external
      // wrenches in the dynamics pass
      float *sens = nullptr, *afree = nullptr, *cfrc = nullptr;
      long sstride = 0;
      if (g->kind == GK_TREE_CONTACT && (needs_dyn || needs_resolve)) {
        sstride = newt_tc_sens_stride(td.L, g->maxc);
        e = cudaMallocAsync(&sens, sizeof(float) * (size_t)sstride * g->cap, st);
        if (e == cudaSuccess) e = cudaMallocAsync(&afree, sizeof(float) * (size_t)g->nv * g->cap, st);
        if (e == cudaSuccess) e = cudaMallocAsync(&cfrc, sizeof(float) * (size_t)g->nv * g->cap, st);
        if (e != cudaSuccess) break;
        const int nl = newt_tc_resolve(ctx, g, sens, sstride, afree, cfrc, st);
        if (nl < 0) { resolve_rc = NEWT_E_CUDA; break; }
        ctx->launches += nl;
      }
      float* dyn = nullptr;  // the links' dynamics pass, when a sensor reads it
      if (needs_dyn) {
        e = cudaMallocAsync(&dyn, sizeof(float) * 18 * (size_t)cnt * td.L, st);
        if (e != cudaSuccess) break;
        newt_launch_tree_sensor_dyn(td, dI + base, cnt, dyn, sens, sstride, st);
        ctx->launches += 1;
      }
      const int mc = g->maxc;
      const float* mg = dM + 3 * base;
      // tree-contact worlds' geoms for the rangefinder
      const bool tc = g->kind == GK_TREE_CONTACT;
      const float* tg = tc ? g->tc_dev().geom : nullptr;
      const int* tt = tc ? g->tc_dev().gtopo : nullptr;
      const int tn = tc ? g->ng : 0;
      switch (newt_tree_bucket(td.L)) {
        case 8: tree_sensors_kernel<8><<<grid, 64, 0, st>>>(td, dI + base, cnt, dS, n_sensors, o, D, dyn, sens, sstride, mc, mg, tg, tt, tn); break;
        case 16: tree_sensors_kernel<16><<<grid, 64, 0, st>>>(td, dI + base, cnt, dS, n_sensors, o, D, dyn, sens, sstride, mc, mg, tg, tt, tn); break;
        case 32: tree_sensors_kernel<32><<<grid, 64, 0, st>>>(td, dI + base, cnt, dS, n_sensors, o, D, dyn, sens, sstride, mc, mg, tg, tt, tn); break;
        default: tree_sensors_kernel<65><<<grid, 64, 0, st>>>(td, dI + base, cnt, dS, n_sensors, o, D, dyn, sens, sstride, mc, mg, tg, tt, tn); break;
      }
      if (dyn) cudaFreeAsync(dyn, st);
      if (sens) cudaFreeAsync(sens, st);
      if (afree) cudaFreeAsync(afree, st);
      if (cfrc) cudaFreeAsync(cfrc, st);
    }
    e = cudaGetLastError();
    ctx->launches += 1;
    order.insert(order.end(), rows[gi].begin(), rows[gi].end());
    base += cnt;
  }
  if (e == cudaSuccess && resolve_rc == NEWT_OK)
    e = cudaMemcpyAsync(host.data(), dO, sizeof(float) * host.size(), cudaMemcpyDeviceToHost, st);
  if (dS) cudaFreeAsync(dS, st);
  if (dM) cudaFreeAsync(dM, st);
  if (dI) cudaFreeAsync(dI, st);
  if (dO) cudaFreeAsync(dO, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (resolve_rc != NEWT_OK) return resolve_rc;  // its message is in ctx->err
  if (e != cudaSuccess) {
    ctx->err = std::string("read_sensors: ") + cudaGetErrorString(e);
    return NEWT_E_CUDA;
  }
  for (size_t j = 0; j < order.size(); ++j)
    std::copy(host.begin() + j * D, host.begin() + (j + 1) * D, out + (size_t)order[j] * D);
  return NEWT_OK;
}
