// Device-side layout of world groups (shared by the kernels and the host
// runtime).  A group holds worlds of one class and one size.
//
//   * Tree groups are structure-of-arrays across worlds (one world per
//     thread): element k of a per-world field lives at  f[k * cap + w], so a
//     warp of 32 consecutive worlds reads 128 contiguous bytes.
//   * Pile groups are world-major (one world per warp): world w's record is
//     the contiguous range F[w * fstride, (w+1) * fstride), which the warp
//     stages into shared memory with coalesced loads.
#pragma once
#include <stdint.h>

#define NEWT_MAX_LINKS 65
#define NEWT_MAX_BODIES 64
#define NEWT_MAX_PLANES 4

enum GroupKind { GK_TREE = 0, GK_PILE = 1, GK_TREE_CONTACT = 2 };

// Kinematic tree without contact (config 0 chains, config 3 chains).
struct TreeGroupDev {
  int n;        // worlds stepped (indices 0..n-1; freed indices are masked by `live`)
  int cap;      // SoA stride
  int L, nq, nv;
  const int* topo;  // [4*L]: parent, joint type, q offset, v offset (same for all worlds)
  // per-world model (SoA)
  const float* axis;   // 3L
  const float* jp;     // 3L   joint_offset_in_parent position
  const float* jc;     // 3L   joint_offset_in_child position
  const float* rootq;  // 4    root orientation (x y z w) for a fixed root
  const float* mass;   // L
  const float* inert;  // 6L   xx yy zz xy xz yz
  const float* damp;   // L    hinge/slide damping (link 0: free_damping)
  const float* arm;    // L    armature
  const float* dtg;    // 4    dt, gx, gy, gz
  const int* solver;   // 1    nonzero enables free-root qfrc (newt/src/forces.rs:16-31)
  const int* live;     // 1    nonzero for allocated worlds
  const int* integ;    // 1    NEWT_INTEGRATOR_* (null: Euler for every world)
  float* cfrc;         // tree-contact groups: the contact solve's J^T f / dt (nv per world, stride
  long cstride;        // `cstride` floats, in the solver scratch); null for trees without geoms
  // per-world state (SoA)
  float* q;     // nq  (newt layout: free root p xyz, quat xyzw; hinge angle)
  float* qd;    // nv  (free root: omega_body, v_body; hinge rate)
  float* qfrc;  // nv
  float* qacc;  // nv  (last step)
  uint32_t* status;
};

// A tree whose link geoms touch static planes (quadruped worlds): the tree
// group's SoA layout plus per-geom model rows, the solver mode and a
// world-major solver scratch.
// Floats per tree-contact record in the solver scratch (newton_kernels.cu),
// SoA geom model rows per geom of a tree-contact world (size3 pos3 quat4
// fric margin gap solref2 solimp5 torsional rolling).
constexpr int TC_CREC = 28;
constexpr int TC_GREC = 22;

struct TcGroupDev {
  TreeGroupDev t;
  int ng;            // geoms per world (link geoms and static planes, model order)
  int npairs;        // candidate (static, link geom) pairs, newt's pair order
  int maxc;          // contact capacity per world
  int rpc;           // row capacity per contact: 6 when a geom has condim 6, else 4
  int cone;          // NEWT_CONE_* (uniform over the group)
  int general;       // some contact's rows are not four pyramidal facets or one normal row
  const int* gtopo;  // [2*ng] shape, link (-1 static); [ng] condim; [2*L] subtree masks (lo, hi);
                     // [nv] the link of each DoF
  const int* pairs;  // [2*npairs] geom indices (a < b)
  const float* geom; // 22 SoA rows per geom: size3 pos3 quat4 fric margin gap solref2 solimp5
                     // torsional rolling
  const int* mode;   // per world: NEWT_SOLVER_PGS | NEWT_SOLVER_NEWTON
  const int* iters;  // per world
  float* scr;        // world-major solver scratch
  long sstride;      // floats per world in `scr`
  // the contact sensors' re-solve (null in a step): the last step's contacts
  // solved again at the current state; per world (stride `sens_stride`)
  // each link's contact wrench (world force, torque about its COM), then per
  // contact slot (geom a, geom b as int bits, normal force), then the count
  float* sens;
  long sens_stride;
};

// Field offsets (in floats / ints) inside one pile world's record.
struct PileLayout {
  int fstride, istride;
  // float fields
  int mass, inert, iinv, size, gpos, gquat, fric, margin, soft, plane, dtg;
  int tfric, rfric;  // per entity: torsional and rolling friction
  int pos, quat, vel, omg;
  int cdata, imp;
  int rpc;  // impulse slots per contact in `imp`: 4 (facet rows), 6 on general-row groups
  // int fields
  int shape, gent, iters, status, ncon, cpair, live, integ;
  int gcond, cone;  // per entity: condim; the world's friction cone (NEWT_CONE_*)
};

// How a pile group's contacts are solved: PGS over the pyramidal facet rows
// (condim 3 everywhere, the island-class and world-persistent kernels), the
// dense Newton solve (pile_newton.cu), or PGS over newt's general rows
// (elliptic cone, condim 1, 4 or 6: pile_general.cu).
enum PileSolve { PS_PGS = 0, PS_NEWTON = 1, PS_GENERAL = 2 };

// Free bodies with one geom each plus static planes (config 1 piles).
struct PileGroupDev {
  int n, cap;
  int nb;        // bodies per world
  int np;        // static planes per world
  int maxc;      // contact capacity per world
  PileLayout lay;
  float* F;      // world-major float records
  int* I;        // world-major int records
  float* scr;    // per-world solver scratch (world-major)
  long sstride;  // floats per world in `scr`
  int solve;     // PileSolve
};
