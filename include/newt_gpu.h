/*
 * newt_gpu.h - C ABI of the GB300 batched stepping engine for newt.
 *
 * newt (hwang2409/tooling, newt/) is a single-world, single-threaded Rust
 * rigid-body engine whose public surface is `World::step(&mut self)`
 * (newt/src/world.rs:1459), scene loading (newt/src/model.rs:179,
 * newt/src/mjcf.rs:119) and MuJoCo-layout state setters
 * (newt/src/world.rs:519-623).  It has no FFI (newt/Cargo.toml:9-10) and
 * reports errors by panicking.  This header is the drop-in boundary a newt
 * caller binds with `extern "C"`: plain pointers and sizes, int status codes,
 * no C++ exceptions and no device traps crossing it.
 *
 * Ownership: the library owns model and world state on the device.  Host
 * buffers passed in are caller-owned, copied during the call and never
 * retained.  One context = one CUDA stream; a context is not thread-safe.
 *
 * State layout (MuJoCo convention, the one newt's differential tests use,
 * newt/tests/differential.rs:548-640):
 *   qpos: free bodies first (pos xyz, quat wxyz), then the tree joints in link
 *         order (free root: pos xyz + quat wxyz; hinge/slide: 1; ball: quat wxyz).
 *   qvel: free bodies (v_world xyz, omega_body xyz), then tree joints
 *         (free root: v_world xyz, omega_body xyz; hinge/slide: 1; ball: 3).
 */
#ifndef NEWT_GPU_H
#define NEWT_GPU_H

#include <stdint.h>

#if defined(__GNUC__)
#define NEWT_API __attribute__((visibility("default")))
#else
#define NEWT_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (replace newt's panics, newt/src/world.rs:874-894,
 *      newt/src/solver.rs:2856-2858, newt/src/world.rs:1462-1464) ---------- */
#define NEWT_OK 0
#define NEWT_E_INVALID 1          /* bad argument / malformed model */
#define NEWT_E_UNSUPPORTED_PAIR 2 /* shape pair with no narrowphase (world.rs:874) */
#define NEWT_E_NOT_PD 3           /* mass matrix or Hessian factorisation failed */
#define NEWT_E_OVERFLOW 4         /* a per-world contact buffer overflowed */
#define NEWT_E_TIMEOUT 5          /* a bounded device wait gave up */
#define NEWT_E_CUDA 6             /* CUDA runtime error */
#define NEWT_E_NOMEM 7            /* device memory / admission budget exhausted */
#define NEWT_E_NOT_FINITE 8       /* NaN or Inf produced in a world */

/* per-world status bits (newt_gpu_world_status) */
#define NEWT_WS_NONFINITE 0x1u
#define NEWT_WS_NOT_PD 0x2u
#define NEWT_WS_CONTACT_OVERFLOW 0x4u
#define NEWT_WS_ITER_CAP 0x8u
#define NEWT_WS_FP64_FALLBACK 0x10u

/* ---- model description (flattened newt `World`; newt/src/tree.rs:79-237,
 *      newt/src/body.rs:22-47, newt/src/geom.rs:352) ----------------------- */
#define NEWT_JOINT_FREE 0
#define NEWT_JOINT_FIXED 1
#define NEWT_JOINT_HINGE 2
#define NEWT_JOINT_SLIDE 3
#define NEWT_JOINT_BALL 4

#define NEWT_SHAPE_PLANE 0
#define NEWT_SHAPE_SPHERE 1
#define NEWT_SHAPE_BOX 2
#define NEWT_SHAPE_CAPSULE 3   /* size: radius, half height along local z */
#define NEWT_SHAPE_CYLINDER 4  /* size: radius, half height along local z */
#define NEWT_SHAPE_ELLIPSOID 5 /* size: semi-axes */

#define NEWT_SOLVER_PGS 1
#define NEWT_SOLVER_NEWTON 2
#define NEWT_CONE_PYRAMIDAL 0
#define NEWT_CONE_ELLIPTIC 1

/* Semi-implicit Euler (the configs' integrator, implicit joint damping) or
 * classic RK4 (newt's default: four explicit ABA stages, root quaternion
 * renormalised after the step, newt/src/tree.rs:1234-1364).  Under RK4 the
 * contact solve runs once at the start of the step and its result is held over
 * the four stages: per-body wrenches for free-body piles
 * (newt/src/world.rs:1705-1788), J^T f / dt added to qfrc for tree-contact
 * worlds, whose solve then factors M and uses the explicit free ABA
 * (world.rs:1826-1945, solver.rs:2852-2855,3602-3622).  A tree's qacc is the
 * first stage's. */
#define NEWT_INTEGRATOR_EULER 0
#define NEWT_INTEGRATOR_RK4 1

typedef struct newt_link_desc {      /* newt::tree::Link */
  int32_t parent;                    /* -1 for the root (link 0) */
  int32_t joint;                     /* NEWT_JOINT_* */
  float axis[3];                     /* hinge/slide axis, parent frame */
  float damping;                     /* hinge/slide/ball joint damping */
  float armature;
  float free_damping;                /* free root only */
  float jp_pos[3], jp_quat[4];       /* joint_offset_in_parent, quat xyzw */
  float jc_pos[3], jc_quat[4];       /* joint_offset_in_child, quat xyzw */
  float mass;
  float inertia[9];                  /* about the COM, body axes, column-major */
} newt_link_desc;

typedef struct newt_body_desc {      /* newt::body::Body (free rigid body) */
  float mass;
  float inertia[9];                  /* column-major */
} newt_body_desc;

typedef struct newt_geom_desc {      /* newt::geom::Geom */
  int32_t shape;                     /* NEWT_SHAPE_* */
  int32_t body;                      /* free-body index, or -1 */
  int32_t link;                      /* link index in the world's tree, or -1 */
  float size[3];                     /* sphere r | box half extents | capsule r, half_height */
  float local_pos[3], local_quat[4]; /* offset in the body/link frame; static: world pose */
  float friction;
  float solref[2];                   /* timeconst, dampratio */
  float solimp[5];                   /* dmin, dmax, width, midpoint, power */
  float margin, gap;
  int32_t condim;                    /* 1, 3, 4 or 6 (newt/src/solver.rs:1409-1428) */
  uint32_t group, mask;              /* collision filter (newt/src/broadphase.rs:16) */
  float torsional_friction;          /* condim >= 4: torsion cap mu_t f_n (geom.rs:397-403) */
  float rolling_friction;            /* condim 6: rolling cap mu_r f_n (geom.rs:404-409) */
} newt_geom_desc;

typedef struct newt_model_desc {     /* one world's model: at most one tree */
  int32_t n_links, n_bodies, n_geoms;
  const newt_link_desc* links;
  const newt_body_desc* bodies;
  const newt_geom_desc* geoms;
  float dt;
  float gravity[3];
  int32_t solver;                    /* NEWT_SOLVER_PGS | NEWT_SOLVER_NEWTON */
  int32_t iterations;                /* PGS sweeps / Newton iteration cap */
  int32_t tree_self_collision;       /* nonzero (newt's default, world.rs:340): geoms on different links of
                                      * the tree collide; 0: those pairs are skipped */
  int32_t integrator;                /* NEWT_INTEGRATOR_*: World::integrator (newt/src/world.rs:76-84) */
  int32_t cone;                      /* NEWT_CONE_*: SolverConfig::cone (newt/src/solver.rs:75-110);
                                      * elliptic under PGS (Newton takes the pyramidal cone) */
  float magnetic_field[3];           /* World::magnetic_field, world frame, read by magnetometers
                                      * (newt/src/world.rs:118-119; World::new sets (0, -0.5, 0)) */
  int32_t n_pairs;                   /* World::pair_list (world.rs:136-139): with `pairs` non-null, the */
  const int32_t* pairs;              /* world collides exactly these n_pairs geom pairs (a, b), in this
                                      * order, past the group/mask filter and the tree's self-collision
                                      * switch; null: the automatic pairs.  Tree-contact worlds only. */
} newt_model_desc;

/* ---- context ------------------------------------------------------------ */
typedef struct newt_gpu_ctx newt_gpu_ctx;

typedef struct newt_gpu_opts {
  int32_t device;                    /* CUDA device ordinal */
  int32_t max_worlds;                /* slot capacity */
  uint64_t hbm_budget_bytes;         /* 0 = free HBM at creation minus a reserve */
  int32_t max_contacts;              /* pile worlds: contacts kept per world (0 = sized from the body
                                      * count, 6 nb + 4 nb np, 64..512), rounded up to a multiple of
                                      * 32.  Contacts past it are dropped in pair order and the world's
                                      * status gets NEWT_WS_CONTACT_OVERFLOW (newt's contact list
                                      * grows without bound, world.rs:2476-2515) */
} newt_gpu_opts;

/* Replaces building a `World` (newt/src/world.rs:325). */
NEWT_API int newt_gpu_create(const newt_gpu_opts* opts, newt_gpu_ctx** out);
NEWT_API int newt_gpu_destroy(newt_gpu_ctx* ctx);
NEWT_API const char* newt_gpu_last_error(const newt_gpu_ctx* ctx);

/* Replaces the loaders' `World::add_tree/add_body/add_geom`
 * (newt/src/world.rs:950-981): validates and copies `n` models to the device.
 * Rejects unsupported shape pairs with NEWT_E_UNSUPPORTED_PAIR (the
 * deferred-pair panic of newt/src/world.rs:874-894). */
NEWT_API int newt_gpu_upload_models(newt_gpu_ctx* ctx, const newt_model_desc* models, int32_t n,
                           int32_t* model_ids_out);
/* MuJoCo-layout dimensions of a model: nq, nv (and nu = nv actuated DoF). */
NEWT_API int newt_gpu_model_dims(const newt_gpu_ctx* ctx, int32_t model_id, int32_t* nq, int32_t* nv);

/* Allocate world slots for models (admission by the HBM budget). */
NEWT_API int newt_gpu_alloc_worlds(newt_gpu_ctx* ctx, const int32_t* model_ids, int32_t n, int32_t* slots_out);
NEWT_API int newt_gpu_free_worlds(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n);

/* State in/out, MuJoCo layout, the worlds' vectors concatenated in `slots`
 * order.  Mirrors `World::apply_mujoco_qpos/qvel` (newt/src/world.rs:519-623).
 * Each call makes one host<->device copy per array and converts between the
 * layouts on the device; arrays in page-locked host memory (cudaMallocHost,
 * cudaHostRegister) are copied by DMA as they are, others through the
 * context's staging buffer.  Both return once the caller's arrays are free
 * again; a slot named twice in newt_gpu_set_state is refused. */
NEWT_API int newt_gpu_set_state(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n, const float* qpos,
                       const float* qvel);
NEWT_API int newt_gpu_get_state(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n, float* qpos, float* qvel);
/* Generalised applied forces (`Tree::qfrc_applied`, newt/src/tree.rs:207),
 * nv per world, concatenated; persists across steps like newt's field. */
NEWT_API int newt_gpu_set_qfrc(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n, const float* qfrc);

/* Replaces `World::step()` (newt/src/world.rs:1459) for every live world.
 * mode NEWT_STEP_PLAIN: one launch per stage per step, fixed tiles.
 * mode NEWT_STEP_BATCHED: the whole call captured in one CUDA graph and
 *   replayed: trees run the horizon in one persistent launch per size bucket
 *   over a cost-sorted queue; pile worlds of every size run theirs in one
 *   world-persistent launch (a warp per world for the whole horizon, worlds
 *   pulled from a queue sorted by the previous call's cost, most costly
 *   first); tree-contact worlds run their three kernels per env-step on a
 *   branch of the graph.  newt_gpu_autotune may instead pick the
 *   island-class pipeline for piles (collide, island-class solvers on forked
 *   streams, integrate, per env-step).  Pile worlds under the Newton solver
 *   (solve_free_body_newton_impulses, newt/src/solver.rs:1295-1407) run
 *   collide, a dense Newton solve (a warp per world) and integrate per
 *   env-step in both modes. */
#define NEWT_STEP_PLAIN 0
#define NEWT_STEP_BATCHED 1
NEWT_API int newt_gpu_step(newt_gpu_ctx* ctx, int32_t n_steps, int32_t mode);
/* Allocation-free plain step.  No counterpart in the reference (newt steps
 * one world on the host and has no device memory to manage).
 * Same kernels and results as newt_gpu_step(ctx, n, NEWT_STEP_PLAIN), all on
 * the context's stream, but the pile solver's scratch, island work lists and
 * group tables sit in one fixed device array of NEWT_STATIC_SCRATCH_BYTES per
 * device instead of buffers from cudaMalloc: for callers that must not
 * allocate or free device memory while they step.  About 131 KB per
 * 16-body pile world (some 250 such worlds fit); a context that needs more
 * gets NEWT_E_NOMEM before anything is launched.  Tree worlds need no
 * scratch; tree-contact worlds and pile worlds under the Newton solver are
 * refused (NEWT_E_INVALID).
 * The first call on a device sets up (symbol lookup, kernel loading): make it
 * before any stream capture.  There is one array per device, so calls whose
 * GPU work can overlap (two contexts or threads on one device) race; order
 * them (newt_gpu_sync between contexts). */
#define NEWT_STATIC_SCRATCH_BYTES (32u * 1024u * 1024u)
NEWT_API int newt_gpu_step_static(newt_gpu_ctx* ctx, int32_t n_steps);
/* Stops the named worlds from being stepped, on the device and without a
 * host wait: ordered on the context's stream after the work already issued,
 * so a caller that queues several step calls can end one world's horizon
 * between two of them.  The worlds keep their state (newt_gpu_get_state
 * reads it) and their slots until newt_gpu_free_worlds.  No counterpart in
 * newt, whose caller simply stops calling World::step. */
NEWT_API int newt_gpu_hold_worlds(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n);
/* Waits for the context's stream (bounded host wait; NEWT_E_TIMEOUT). */
NEWT_API int newt_gpu_sync(newt_gpu_ctx* ctx, int32_t timeout_ms);

/* Per-world status words (NEWT_WS_*), accumulated since the last clear. */
NEWT_API int newt_gpu_world_status(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n, uint32_t* status,
                          int32_t clear);

/* ---- convex contact queries -------------------------------------------------
 * newt's general convex route, GJK then EPA (newt/src/contact/ccd.rs:1703-1911,
 * the path newt takes for mesh pairs), run on the device for arbitrary pairs
 * of spheres, boxes and capsules.  The step's narrowphase keeps its closed
 * forms; this entry point is their second formulation (a cross-check) and a
 * device query for callers.  A pose is position x y z, then quaternion
 * x y z w; sizes as in newt_geom_desc.  `face_eps` is EPA's face-removal
 * threshold relative to the pair extent (<= 0: newt's 1e-4; EPA then ends in
 * newt's shallowest-axis fallback on curved features, and a threshold of
 * 1e-7 lets it converge there).  Result: hit, path (1 distance GJK, 2 EPA,
 * 3 EPA fallback), contact point, normal (from B into A), penetration and
 * the witness points on A and B.  Pairs with another shape get
 * NEWT_E_UNSUPPORTED_PAIR before anything runs. */
typedef struct newt_convex_query {
  int32_t shape_a, shape_b;          /* NEWT_SHAPE_SPHERE | _BOX | _CAPSULE */
  float pose_a[7], size_a[3];
  float pose_b[7], size_b[3];
  float margin;
} newt_convex_query;
typedef struct newt_convex_result {
  int32_t hit, path;
  float pos[3], normal[3];
  float penetration;
  float witness_a[3], witness_b[3];
} newt_convex_result;
NEWT_API int newt_gpu_convex_contacts(newt_gpu_ctx* ctx, const newt_convex_query* queries, int32_t n, float face_eps,
                                      newt_convex_result* out);

/* ---- diagnostics (parity surfaces) -------------------------------------- */
/* Generalised acceleration of the last step, newt layout (qdot order), nv per
 * world.  Mirrors the qacc that `euler_step_with_workspace` integrates
 * (newt/src/tree.rs:1406-1417). */
NEWT_API int newt_gpu_get_qacc(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n, float* qacc);
/* Post-step sensors that read the state alone (newt/src/sensor.rs:153-196,
 * evaluated as World::evaluate_sensors does after a step, sensor.rs:446-700).
 * A site frame is (local_pos, local_quat x y z w) in its parent: free body
 * `index` (on_link 0) or link `index` of the world's tree (on_link 1).
 *   JOINTPOS / JOINTVEL  hinge or slide coordinate and rate of link `index` (1)
 *   FRAMEPOS             site position, world (3)
 *   FRAMEQUAT            site orientation x y z w, world (4)
 *   GYRO                 parent's body-frame angular velocity in the site frame (3)
 *   VELOCIMETER          site linear velocity in the site frame (3)
 *   FRAMELINVEL          site linear velocity, world (3)
 *   FRAMEANGVEL          parent's angular velocity, world (3)
 *   SUBTREECOM           mass-weighted centre of link `index` and its descendants (3)
 *   ACCELEROMETER        specific force at the site on free body or link `index`, site frame (3)
 *   TOUCH                summed normal-force magnitudes of the contacts of geom `index` (1)
 *   FORCE                force link `index`'s parent joint transmits to it, link frame (3)
 *   TORQUE               the matching torque about the joint anchor, link frame (3)
 *   MAGNETOMETER         the model's magnetic_field in the site frame (3)
 *   RANGEFINDER          distance along the site's +z to the nearest geom of the world, the
 *                        site's own included (a ray that starts inside a shape hits its far
 *                        side), -1 when the ray meets none (1; sensor.rs:759-791,
 *                        scene_query.rs:182-438)
 * ACCELEROMETER and TOUCH are read on pile worlds as newt's World::step reads
 * them (world.rs:1545-1612, sensor.rs:586-600, 1030-1112): the contacts of
 * the world's last step (any step form) are re-solved at its current state
 * with its solver, giving the body wrenches (F/m + g, Euler's equations) and
 * the normal forces (a contact's row impulses over dt).  A world read before
 * its first step sees no contacts.  ACCELEROMETER on a link, FORCE and
 * TORQUE are read on trees (sensor.rs:446-530, 620-647, 834-1000): qddot
 * from the explicit ABA at the current state with the world's generalised
 * forces, the links' spatial accelerations, and the RNE wrench each parent
 * joint transmits.  On tree-contact worlds the last step's contacts are
 * first re-solved at the current state with the world's solver
 * (world.rs:2252-2300, solver.rs:3334-3364): the rows' forces give each
 * link's external wrench, which the ABA and the RNE take in, and each
 * contact's normal force, which TOUCH sums. */
#define NEWT_SENSOR_JOINTPOS 0
#define NEWT_SENSOR_JOINTVEL 1
#define NEWT_SENSOR_FRAMEPOS 2
#define NEWT_SENSOR_FRAMEQUAT 3
#define NEWT_SENSOR_GYRO 4
#define NEWT_SENSOR_VELOCIMETER 5
#define NEWT_SENSOR_FRAMELINVEL 6
#define NEWT_SENSOR_FRAMEANGVEL 7
#define NEWT_SENSOR_SUBTREECOM 8
#define NEWT_SENSOR_ACCELEROMETER 9
#define NEWT_SENSOR_TOUCH 10
#define NEWT_SENSOR_FORCE 11
#define NEWT_SENSOR_TORQUE 12
#define NEWT_SENSOR_MAGNETOMETER 13
#define NEWT_SENSOR_RANGEFINDER 14
typedef struct newt_sensor_desc {
  int32_t kind;        /* NEWT_SENSOR_* */
  int32_t on_link;     /* 1: `index` is a link of the world's tree, 0: a free body */
  int32_t index;
  float local_pos[3];
  float local_quat[4]; /* x y z w */
} newt_sensor_desc;
/* Evaluates `n_sensors` sensors on each of `n` worlds at their current state,
 * on the device; `out` receives n rows of the sensors' values concatenated in
 * order (the layout of newt's SensorBank::data, sensor.rs:370-400). */
NEWT_API int newt_gpu_read_sensors(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n, const newt_sensor_desc* sensors,
                                   int32_t n_sensors, float* out);

/* Contacts detected at the start of the last step for one world:
 * per contact (geom_a, geom_b) pairs into `pairs` (2*cap ints) and
 * pos xyz, normal xyz, penetration into `data` (7*cap floats). */
NEWT_API int newt_gpu_get_contacts(newt_gpu_ctx* ctx, int32_t slot, int32_t cap, int32_t* n_out,
                          int32_t* pairs, float* data);
/* Row impulses of the last step's constraint solve for one world, in the
 * solver's row order (newt's impulses, solver.rs:1204-1257), per detected
 * contact (zeros for an inactive one): 4 pyramidal facet rows; on pile
 * worlds with the elliptic cone or a condim other than 3, 6 slots per
 * contact holding its rows first (facets, or normal, tangents, torsion,
 * rolling as its condim has them) and zeros after.  On tree-contact worlds
 * the rows of the active contacts only, in contact order, with the same
 * rows per contact (solver.rs:2880-2990). */
NEWT_API int newt_gpu_get_impulses(newt_gpu_ctx* ctx, int32_t slot, int32_t cap, int32_t* n_out, float* impulses);

/* ---- timing helpers for the benchmark (CUDA events on the ctx stream) ---- */
NEWT_API int newt_gpu_event_record(newt_gpu_ctx* ctx, int32_t which);          /* which: 0 start, 1 stop */
NEWT_API int newt_gpu_event_elapsed_ms(newt_gpu_ctx* ctx, float* ms);
NEWT_API int newt_gpu_flush_l2(newt_gpu_ctx* ctx);                              /* writes a buffer > L2 */
/* Kernel launches issued by this context since creation. */
NEWT_API int64_t newt_gpu_launch_count(const newt_gpu_ctx* ctx);
/* Times the batched step's launch choices on the live worlds (piles in the
 * world-persistent launch in each of its shapes -- gangs of 4 to 32 warps,
 * one to four gangs per SM, with or without a barrier between assembly and
 * sweeps, one or two worlds per warp --
 * or in the island-class pipeline with 1, 2 or 3 world-range branches; tree
 * persistent grid at full or half residency), `n_steps` env-steps per trial,
 * and keeps the fastest for later NEWT_STEP_BATCHED calls.  `horizon` is how
 * many env-steps the caller means to run next (<= 0: 8 x n_steps): every
 * choice is timed from three snapshots of every world -- as they are, and
 * horizon/2 and horizon env-steps later (falling piles land and their
 * islands grow) -- and judged by the trapezoid average over the horizon
 * (weights 1/4, 1/2, 1/4).  Every world's state is left as it was.
 * `choice` (nullable, 5 ints): pile branches (0 for the persistent launch),
 * tree grid percent, the winner's averaged time per trial in microseconds,
 * 1 if piles use the persistent launch, its shape index (0: 16 warps; 1: 12
 * warps; 2: 12 warps, one barrier per env-step; 3: 8 warps; 4: 24 warps; 5:
 * 32 warps).  No counterpart in newt. */
NEWT_API int newt_gpu_autotune(newt_gpu_ctx* ctx, int32_t n_steps, int32_t horizon, int32_t* choice);
/* Sets the batched step's launch choices directly, in newt_gpu_autotune's
 * `choice` layout: [0] pile world-range branches of the island-class
 * pipeline (0: by world count), [1] tree persistent grid percent, [2]
 * ignored, [3] 1 for the world-persistent pile launch, 0 for the pipeline,
 * [4] its shape index (newt_gpu_autotune).  No counterpart in newt. */
NEWT_API int newt_gpu_set_launch_choice(newt_gpu_ctx* ctx, const int32_t* choice);
/* Device bytes the world groups hold (capacity x bytes per world: model,
 * state, contact and solver buffers) and the admission budget they are
 * checked against. */
NEWT_API int newt_gpu_memory(const newt_gpu_ctx* ctx, uint64_t* used, uint64_t* budget);

/* Control streams.  A world's whole control sequence (horizon x nv
 * generalised forces, `Tree::qfrc_applied`, newt/src/tree.rs:207) is
 * uploaded once and kept on the device; each newt_gpu_apply_ctrl call writes
 * the next row of every stream into its world's qfrc and advances the
 * stream's cursor (past the horizon qfrc keeps its last row).  `ctrl` holds
 * the worlds' sequences concatenated in `slots` order.  Worlds without
 * generalised forces (free-body piles) are skipped; a new stream replaces a
 * world's old one, and freeing the world ends it. */
NEWT_API int newt_gpu_set_ctrl_stream(newt_gpu_ctx* ctx, const int32_t* slots, int32_t n, const float* ctrl,
                                      const int32_t* horizons);
NEWT_API int newt_gpu_apply_ctrl(newt_gpu_ctx* ctx);

/* ---- served rollouts ------------------------------------------------------
 * No counterpart in newt, whose callers (the examples in newt/examples,
 * sandbox/src/main.rs:601) own one World and call World::step in their own
 * loop.  newt_gpu_serve is that loop for many requests at once: a request
 * (model, initial state, control sequence, horizon) is admitted into a free
 * world slot once it has arrived and the device budget allows
 * (newt_gpu_alloc_worlds answers NEWT_E_NOMEM past it; the request then
 * waits), its state stays on the device, every admitted world advances by
 * one env-step per step call, `steps_per_tick` of them per tick (requests
 * join and leave between ticks), row t of its controls is applied as qfrc
 * at its step t,
 * and its final state is read back when its horizon completes (a horizon of
 * 0 returns the initial state without admission).  Latency = completion -
 * arrival (completion - call start when real_time is 0). */
typedef struct newt_serve_request {
  int32_t model_id;        /* an uploaded model */
  int32_t horizon;         /* env-steps */
  double arrival_s;        /* seconds after the call starts */
  const float* qpos;       /* initial state, MuJoCo layout (nq, nv) */
  const float* qvel;
  const float* ctrl;       /* horizon x nv generalised forces, row t at step t; NULL = none */
  float* qpos_out;         /* final state written at completion (nullable) */
  float* qvel_out;
  double admit_s;          /* out: admission time */
  double done_s;           /* out: completion time */
} newt_serve_request;
typedef struct newt_serve_opts {
  int32_t max_active;      /* cap on admitted requests (0: the device budget only) */
  int32_t real_time;       /* 1: arrivals follow the wall clock; 0: all present at start */
  int32_t step_mode;       /* NEWT_STEP_BATCHED or NEWT_STEP_PLAIN */
  int32_t steps_per_tick;  /* env-steps per tick (0 or 1: one).  Above one, a
                            * tick queues that many env-steps (each with its
                            * control row) without a host wait between them,
                            * holds every world whose horizon ends inside the
                            * tick at that env-step (newt_gpu_hold_worlds), and
                            * admits and completes requests once per tick:
                            * results are unchanged, host round trips per
                            * env-step fall by that factor, and a request
                            * waits up to a tick for admission. */
} newt_serve_opts;
typedef struct newt_serve_stats {
  int32_t completed, peak_active;
  int64_t ticks;
  double wall_s;           /* call start to last completion */
  double env_steps;        /* sum of the completed horizons */
  double mean_active;      /* admitted requests per tick, averaged */
  double p50_ms, p99_ms, max_ms, mean_ms;  /* latency */
  /* host wall time per phase, summed over ticks: admission (alloc + state
   * upload), controls (qfrc upload), step (launch to completion), and
   * completion (state read-back + release) */
  double admit_s, ctrl_s, step_s, complete_s;
} newt_serve_stats;
NEWT_API int newt_gpu_serve(newt_gpu_ctx* ctx, newt_serve_request* reqs, int32_t n, const newt_serve_opts* opts,
                            newt_serve_stats* stats);

/* Profiling surface of the free-body contact step (no counterpart in newt,
 * whose per-phase timing lives in newt/benches/newt_perf.rs).
 * enable >= 0 sets whether later batched steps bracket every pile kernel with
 * a pair of timing events on the stream that kernel runs on (two event nodes
 * per kernel in the captured graph); enable < 0 leaves the setting.
 * Outputs (each nullable) describe the last newt_gpu_step call, after waiting
 * for it:
 *   kernel_ms[NEWT_PILE_KERNELS]  device time of each pile kernel summed over
 *       that call's launches, in launch-table order: collide, the solvers of
 *       island classes 0..6, integrate (zeros unless timing was on for a
 *       batched step);
 *   work[3 * NEWT_PILE_ISLAND_CLASSES]  islands, then contacts, then bodies
 *       per island class in that call's last env-step;
 *   launches  launches of each kernel summed in kernel_ms (env-steps times
 *       the world-range branches of the batched form). */
#define NEWT_PILE_KERNELS 9
#define NEWT_PILE_ISLAND_CLASSES 7
NEWT_API int newt_gpu_pile_profile(newt_gpu_ctx* ctx, int32_t enable, float* kernel_ms, int32_t* work,
                                   int32_t* launches);

/* Profiling surface of the world-persistent pile launch (no counterpart in
 * newt).  After waiting for the last newt_gpu_step call: `kernel_ms` (nullable)
 * its device time, when timing is on (newt_gpu_pile_profile's `enable`) and
 * that call was batched with piles in the persistent launch, else 0; `work`
 * (nullable, 4 counters, zero unless that call ran the launch): active
 * contacts summed over every world's env-steps, contact-update rounds (a
 * dependency level's groups of eight contacts) summed over the sweeps,
 * dependency levels summed over env-steps, worlds stepped. */
NEWT_API int newt_gpu_pile_fused_profile(newt_gpu_ctx* ctx, float* kernel_ms, uint64_t* work);

/* Profiling surface of the tree-contact step (quadruped worlds).  With
 * timing on (newt_gpu_pile_profile's `enable`), every tree-contact env-step
 * brackets its kernels with timing events on the context's stream; this
 * returns, after waiting for the last newt_gpu_step call, each kernel's
 * device time summed over that call: unconstrained ABA, contact solve,
 * integration (NEWT_TC_KERNELS entries). */
#define NEWT_TC_KERNELS 3
NEWT_API int newt_gpu_tc_profile(newt_gpu_ctx* ctx, float* kernel_ms);

#ifdef __cplusplus
}
#endif
#endif /* NEWT_GPU_H */
