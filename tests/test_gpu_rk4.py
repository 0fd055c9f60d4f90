"""RK4 (newt's default integrator) on the GPU: trees without geoms, and
free-body piles with the PGS wrench held over the stages.

Pinned to newt's own output: the joints golden (newt/tests/joints_golden.rs:
a fixed-root hinge chain and a floating box with an arm) after 100 and 1000
steps; the free-body integrator golden (integrators_golden.rs); the PGS
solver goldens (solver_golden.rs: a three-box stack and a box on an incline,
solved once per step and held over the RK4 stages).  The stack is chaotic (the
FP64 oracle and newt's f32 run drift 2 cm apart by step 200), so it is held
to one-step parity from newt's own snapshots and to that FP64 window over 1000
steps.  Tree-contact worlds hold the joint solve's generalised force over
the stages, here against the FP64 oracle's RK4; newt's own tree-contact
goldens (solver_tree.bin, solver_newton_tree.bin, with their in-tree box
pair) are held on the GPU in tests/test_gpu_intree.py."""
import numpy as np
import pytest

import oracle_py
from test_oracle_golden import _joints_chain, _joints_floating, _read_f32
from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN, scenes
from tooling_gb300 import model as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from tooling_gb300 import build as B
    B.build()
    e = Engine(device=0)
    yield e
    e.close()


def _rot(q_xyzw):
    x, y, z, w = (float(c) for c in q_xyzw)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _floating_to_mujoco(q, v):
    """newt layout (pos, quat xyzw, hinge; omega_body, v_body, rate) to
    MuJoCo layout (pos, quat wxyz, hinge; v_world, omega_body, rate)."""
    q = np.asarray(q, np.float64)
    v = np.asarray(v, np.float64)
    qm = np.concatenate([q[:3], [q[6]], q[3:6], q[7:]])
    vm = np.concatenate([_rot(q[3:7]) @ v[3:6], v[:3], v[6:]])
    return qm, vm


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
def test_joints_golden_rk4(eng, mode):
    gold = _read_f32("joints_chain_and_floating.bin").reshape(3, 21).astype(np.float64)
    wc, qc, vc = _joints_chain()
    wf = _joints_floating(gold[0, 9:13].astype(np.float32))
    for w in (wc, wf):
        w.integrator = M.INTEGRATOR_RK4
    slots = eng.alloc(eng.upload(M.PackedModels([wc, wf])))
    q0f, v0f = _floating_to_mujoco(gold[0, 6:14], gold[0, 14:21])
    eng.set_state(slots, np.concatenate([qc, q0f]).astype(np.float32), np.concatenate([vc, v0f]).astype(np.float32))
    done = 0
    for row, n, tol in ((1, 100, 2e-5), (2, 1000, 2e-3)):
        eng.step(n - done, mode)
        done = n
        q, v = eng.get_state(slots, 3 + 8, 3 + 7)
        # chain: hinge angles and rates, identical in both layouts
        assert np.abs(q[:3] - gold[row, 0:3]).max() < tol
        assert np.abs(v[:3] - gold[row, 3:6]).max() < tol
        qm, vm = _floating_to_mujoco(gold[row, 6:14], gold[row, 14:21])
        assert np.abs(q[3:] - qm).max() < tol, (np.abs(q[3:] - qm).max(), n)
        assert np.abs(v[3:] - vm).max() < tol, (np.abs(v[3:] - vm).max(), n)
    eng.free(slots)


def test_rk4_chains_track_fp64_oracle(eng):
    b = scenes.chain_batch(n_worlds=64, first_world=3000)
    rk = M.Batch(b.links, b.n_links, b.bodies, b.n_bodies, b.geoms, b.n_geoms, 1e-3, (0.0, 0.0, -9.81),
                 M.SOLVER_PGS, 20, integrator=M.INTEGRATOR_RK4)
    rk.qpos[:], rk.qvel[:], rk.qfrc[:] = b.qpos, b.qvel, b.qfrc
    slots = eng.alloc(eng.upload(rk))
    eng.set_state(slots, rk.qpos, rk.qvel)
    eng.set_qfrc(slots, rk.qfrc)
    eng.step(50, STEP_BATCHED)
    q, v = eng.get_state(slots, int(rk.nq.sum()), int(rk.nv.sum()))
    eng.free(slots)
    rq, rv = oracle_py.run(rk, np.arange(len(rk)), rk.qpos, rk.qvel, rk.qfrc, 50, precision=1, integrator=0)
    assert np.abs(q - rq).max() < 1e-3 and np.abs(v - rv).max() < 1e-2
    # and it is not the Euler answer
    eq, ev = oracle_py.run(rk, np.arange(len(rk)), rk.qpos, rk.qvel, rk.qfrc, 50, precision=1, integrator=1)
    assert np.abs(q - eq).max() > 10 * np.abs(q - rq).max()


def _damped_chain_contact(solver):
    """newt's tree-chain contact scene with joint damping (hinge 0.4, free
    root 0.2), so that the RK4 form of the joint solve (factors of M, the
    explicit free ABA) differs from the Euler form (M + dt B, the implicit
    one)."""
    from test_oracle_golden import _tree_chain_contact
    w = _tree_chain_contact(solver)
    w.links[1].damping = 0.4
    w.links[0].free_damping = 0.2
    w.integrator = M.INTEGRATOR_RK4
    return w


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
@pytest.mark.parametrize("solver", [M.SOLVER_NEWTON, M.SOLVER_PGS])
def test_tree_contact_rk4_tracks_fp64_oracle(eng, solver, mode):
    """The contact solve once per step, its J^T f / dt held over the RK4
    stages (newt/src/world.rs:1826-1945): within 1e-3 m / 1e-2 m/s of the
    FP64 oracle over 800 steps of falling, landing and rolling (the f32 and
    FP64 oracles agree to 2e-6 here; Euler lands 7e-3 to 5e-2 m away)."""
    w = _damped_chain_contact(solver)
    P = M.PackedModels([w])
    q0 = np.array([0.0, 0.0, 1.35, 1.0, 0.0, 0.0, 0.0, 0.0], np.float32)
    v0 = np.array([0.3, 0.0, 0.0, 0.0, 0.5, 0.0, 2.0], np.float32)
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q0, v0)
    done, errs = 0, []
    for n in (300, 500, 800):
        eng.step(n - done, mode)
        done = n
        gq, gv = eng.get_state(slots, 8, 7)
        rq, rv = oracle_py.run(P, np.zeros(1, np.int32), q0, v0, None, n, precision=1, integrator=0)
        eq, _ = oracle_py.run(P, np.zeros(1, np.int32), q0, v0, None, n, precision=1, integrator=1)
        errs.append((n, float(np.abs(gq - rq).max()), float(np.abs(gv - rv).max()), float(np.abs(eq - rq).max())))
    assert not (eng.status(slots) & 0x7).any()
    eng.free(slots)
    assert all(dq < 1e-3 and dv < 1e-2 for _, dq, dv, _ in errs), errs
    assert max(e for *_, e in errs) > 5e-3, errs  # the oracle's two integrators do differ here


@pytest.mark.parametrize("solver", [M.SOLVER_NEWTON, M.SOLVER_PGS])
def test_tree_contact_rk4_impulses_match_oracle(eng, solver):
    """One RK4 step from a resting state with eight contacts: row impulses
    within 1e-3 relative of the oracle's RK4-form solve."""
    w = _damped_chain_contact(solver)
    P = M.PackedModels([w])
    q0 = np.array([0.0, 0.0, 1.35, 1.0, 0.0, 0.0, 0.0, 0.0], np.float32)
    v0 = np.array([0.3, 0.0, 0.0, 0.0, 0.5, 0.0, 2.0], np.float32)
    rq, rv = oracle_py.run(P, np.zeros(1, np.int32), q0, v0, None, 800, precision=1, integrator=0)
    q, v = rq.astype(np.float32), rv.astype(np.float32)
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q, v)
    eng.step(1, STEP_PLAIN)
    eng.sync()
    g = eng.impulses(int(slots[0]))
    eng.free(slots)
    ref, _ = oracle_py.tree_impulses(P, 0, q, v, None, integrator=0)
    assert len(ref) >= 8 and len(g) == len(ref)
    assert np.abs(g - ref).max() / np.abs(ref).max() < 1e-3


@pytest.mark.parametrize("solver", [M.SOLVER_NEWTON, M.SOLVER_PGS])
def test_quadrupeds_rk4_short_trajectory(eng, solver):
    """Settled quadrupeds with controls, ten RK4 steps: within 2e-3 m /
    5e-2 m/s of the FP64 oracle (the tree-contact Euler bar)."""
    b = scenes.quadruped_batch(n_worlds=16, first_world=300, solver=solver)
    rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, None, 300, precision=1)
    b.qpos[:], b.qvel[:] = rq.astype(np.float32), rv.astype(np.float32)
    b.qfrc[:] = scenes.quadruped_controls(len(b), 0, first_world=300)
    for i in range(len(b)):
        b.descs[i].integrator = M.INTEGRATOR_RK4
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, b.qpos, b.qvel)
    eng.set_qfrc(slots, b.qfrc)
    eng.step(10, STEP_BATCHED)
    gq, gv = eng.get_state(slots, int(b.nq.sum()), int(b.nv.sum()))
    assert not (eng.status(slots) & 0x7).any()
    eng.free(slots)
    oq, ov = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, b.qfrc, 10, precision=1, integrator=0)
    assert np.abs(gq - oq).max() < 2e-3 and np.abs(gv - ov).max() < 5e-2


def _mj(q_newt, nb):
    """newt free-body layout (pos, quat xyzw) to MuJoCo's (pos, quat wxyz);
    the velocity layouts (v_world, omega_body) agree."""
    q = np.asarray(q_newt, np.float32).reshape(nb, 7)
    return np.concatenate([q[:, :3], q[:, 6:7], q[:, 3:6]], axis=1).reshape(-1)


def _pile_world(name):
    from test_oracle_golden import _integrator_scene, _solver_box_scene
    if name == "integrator":
        w, q, v = _integrator_scene()
        # the pile path wants one geom per body: a sphere with nothing to touch
        w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, body=0, size=(0.05, 0.0, 0.0)))
        w.solver, w.iterations = M.SOLVER_PGS, 1  # no contacts: a zero wrench, as in newt's penalty mode
        gold = _read_f32("integrator_rk4.bin").reshape(3, 1, 13)
        return w, q, v, gold, (20, 100)
    w, q, v = _solver_box_scene(name)
    gold = _read_f32(f"solver_{name}.bin").reshape(4, len(w.bodies), 13)
    return w, q, v, gold, (50, 200, 1000)


def _track(eng, name, mode):
    w, q, v, gold, marks = _pile_world(name)
    w.integrator = M.INTEGRATOR_RK4
    nb = len(w.bodies)
    slots = eng.alloc(eng.upload(M.PackedModels([w])))
    eng.set_state(slots, _mj(q, nb), v)
    done, errs = 0, []
    for row, n in enumerate(marks, start=1):
        eng.step(n - done, mode)
        done = n
        gq, gv = eng.get_state(slots, 7 * nb, 6 * nb)
        errs.append((n, float(np.abs(gq - _mj(gold[row][:, :7], nb)).max()),
                     float(np.abs(gv - gold[row][:, 7:].reshape(-1)).max())))
    assert not (eng.status(slots) & 0x5).any()
    eng.free(slots)
    return errs


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
@pytest.mark.parametrize("name,qtol,vtol", [("integrator", 2e-6, 2e-6), ("incline", 5e-4, 5e-3)])
def test_pile_rk4_tracks_newt_goldens(eng, name, qtol, vtol, mode):
    errs = _track(eng, name, mode)
    assert all(dq < qtol and dv < vtol for _, dq, dv in errs), errs


def _stack_envelope(n_runs=48, nudge=1e-7):
    """How far newt's own f32 arithmetic lands from newt's stack snapshots
    when the start positions move by 1e-7 m: the oracle's float mirror (byte-
    identical to newt unperturbed) over `n_runs` nudged starts, the largest
    position and velocity distances at each snapshot."""
    w, q, v, gold, marks = _pile_world("stack")
    w.integrator = M.INTEGRATOR_RK4
    nb = len(w.bodies)
    rng = np.random.default_rng(7)
    qs = np.tile(np.asarray(q, np.float32).reshape(nb, 7), (n_runs, 1, 1))
    qs[:, :, :3] += rng.uniform(-nudge, nudge, (n_runs, nb, 3)).astype(np.float32)
    vs = np.tile(np.asarray(v, np.float32), n_runs)
    packed = M.PackedModels([w])
    env, done = [], 0
    qc, vc = qs.reshape(-1), vs
    for row, n in enumerate(marks, start=1):
        qo, vo = oracle_py.run(packed, np.zeros(n_runs, np.int32), qc, vc, None, n - done, precision=0, layout=1,
                               integrator=0, n_threads=8)
        done = n
        qc, vc = qo.astype(np.float32), vo.astype(np.float32)
        dq = np.abs(qc.reshape(n_runs, nb, 7) - gold[row][None, :, :7]).max()
        dv = np.abs(vc.reshape(n_runs, nb * 6) - gold[row][:, 7:].reshape(-1)[None, :]).max()
        env.append((n, float(dq), float(dv)))
    return env


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
def test_pile_rk4_stack_stays_in_newts_envelope(eng, mode):
    """newt's box stack is chaotic: 48 f32 runs of newt's own arithmetic from
    start positions nudged by 1e-7 m spread up to a few cm and about 0.3 m/s
    from newt's snapshot at step 1000.  The GPU run must stay within 5 cm, or
    1.25 times that spread if larger, of newt's positions at every snapshot,
    and within 1.25 times the velocity spread once the stack has settled
    (step 1000)."""
    errs = _track(eng, "stack", mode)
    env = _stack_envelope()
    ok_q = all(dq < max(5e-2, 1.25 * eq) for (_, dq, _), (_, eq, _) in zip(errs, env))
    assert ok_q and errs[-1][2] < 1.25 * env[-1][2], (errs, env)


def test_pile_rk4_one_step_from_newt_snapshots(eng):
    """From each of newt's stack snapshots, one GPU RK4 step against one step
    of the f32 oracle (itself byte-identical to newt over 1000 steps)."""
    from test_oracle_golden import _solver_box_scene
    w, _, _ = _solver_box_scene("stack")
    w.integrator = M.INTEGRATOR_RK4
    gold = _read_f32("solver_stack.bin").reshape(4, 3, 13)
    packed = M.PackedModels([w])
    ids = eng.upload(packed)
    for row in range(4):
        q = np.ascontiguousarray(gold[row][:, :7]).reshape(-1)
        v = np.ascontiguousarray(gold[row][:, 7:]).reshape(-1)
        slots = eng.alloc(ids)
        eng.set_state(slots, _mj(q, 3), v)
        eng.step(1, STEP_BATCHED)
        gq, gv = eng.get_state(slots, 21, 18)
        eng.free(slots)
        rq, rv = oracle_py.run(packed, np.zeros(1, np.int32), q, v, None, 1, precision=0, layout=1, integrator=0)
        assert np.abs(gq - _mj(rq, 3)).max() < 2e-6 and np.abs(gv - rv).max() < 2e-4, row


def test_pile_rk4_batch_tracks_fp64_oracle(eng):
    """A settled 48-world pile batch stepped 20 times with RK4: within
    1e-3 m / 1e-2 m/s of the FP64 oracle's RK4."""
    b = scenes.pile_batch(n_worlds=48, first_world=500)
    rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, None, 300, precision=1)
    rk = M.Batch(b.links, b.n_links, b.bodies, b.n_bodies, b.geoms, b.n_geoms, 2e-3, (0.0, 0.0, -9.81),
                 M.SOLVER_PGS, 50, integrator=M.INTEGRATOR_RK4)
    rk.qpos[:], rk.qvel[:] = rq.astype(np.float32), rv.astype(np.float32)
    slots = eng.alloc(eng.upload(rk))
    eng.set_state(slots, rk.qpos, rk.qvel)
    eng.step(20, STEP_BATCHED)
    gq, gv = eng.get_state(slots, int(rk.nq.sum()), int(rk.nv.sum()))
    eng.free(slots)
    oq, ov = oracle_py.run(rk, np.arange(len(rk)), rk.qpos, rk.qvel, None, 20, precision=1, integrator=0)
    assert np.abs(gq - oq).max() < 1e-3 and np.abs(gv - ov).max() < 1e-2
    eq, _ = oracle_py.run(rk, np.arange(len(rk)), rk.qpos, rk.qvel, None, 20, precision=1, integrator=1)
    assert np.abs(oq - eq).max() > 0  # the two integrators differ on this state
