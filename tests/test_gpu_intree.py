"""In-tree geom pairs on the GPU (a tree that collides with itself, newt's
default, world.rs:340, 1042-1069), through the C ABI, pinned to newt's own
tree-contact goldens.

newt/tests/solver_golden.rs:93-144, 260-297: a free-root tree with one hinge
child, a box on each link (the two boxes a parent-child pair that newt
collides), resting on a plane; q and qdot after 0, 50, 200 and 1000 RK4
steps, under PGS (solver_tree.bin) and Newton (solver_newton_tree.bin).  The
oracle's f32 mirror is byte-identical to both (tests/test_oracle_golden.py).

The two boxes touch between newt's snapshots: the in-tree pair is active
over steps 89-98 and 113-123 of the PGS run and in four windows between
steps 60 and 153 of the Newton run.

Bars: from each of newt's snapshots and from the oracle's f32 states inside
those windows, one GPU step no further from the FP64 oracle's step than
twice newt's own f32 step is (the oracle's float mirror), or within 2e-6
(positions) and 2e-4 (velocities) where newt's is closer; from the start,
the GPU at steps 50, 200 and 1000 within 1.25 times the larger of the spread
of newt's own f32 runs from starts nudged by 1e-7 m and the FP64 oracle's
distance from the snapshot (under Newton newt's f32 line search moves the
first step 2.8e-4 m/s from FP64, and the GPU, whose line-search costs are in
FP64, follows the FP64 run), or within 5e-4 / 5e-3; the in-tree pair's
contacts present in the GPU's contact list, as the oracle lists them, at
those window states."""
import functools

import numpy as np
import pytest

import oracle_py
from test_gpu_rk4 import _floating_to_mujoco
from test_oracle_golden import _read_f32, _tree_contact_scene
from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN
from tooling_gb300 import model as M

pytestmark = pytest.mark.gpu
GOLDENS = [(M.SOLVER_PGS, "solver_tree.bin"), (M.SOLVER_NEWTON, "solver_newton_tree.bin")]
# steps of newt's runs at which the in-tree pair is active (the oracle's f32 run, byte-identical to newt)
IN_TREE_STEPS = {M.SOLVER_PGS: (90, 94, 98, 115, 120), M.SOLVER_NEWTON: (61, 66, 112, 136, 150)}


@pytest.fixture(scope="module")
def eng():
    from tooling_gb300 import build as B
    B.build()
    e = Engine(device=0)
    yield e
    e.close()


def _scene(solver):
    w, q0, v0 = _tree_contact_scene(solver)
    w.integrator = M.INTEGRATOR_RK4
    return w, q0, v0


def _mj(row):
    q, v = _floating_to_mujoco(row[:8], row[8:])
    return q.astype(np.float32), v.astype(np.float32)


def _oracle(P, q, v, n, precision=0):
    rq, rv = oracle_py.run(P, np.zeros(1, np.int32), q, v, None, n, precision=precision, integrator=0)
    return rq.astype(np.float32), rv.astype(np.float32)


@functools.lru_cache(maxsize=None)
def _window_states(solver, name):
    """The oracle's f32 states (newt's arithmetic) at IN_TREE_STEPS."""
    w, _, _ = _scene(solver)
    P = M.PackedModels([w])
    q, v = _mj(_read_f32(name).reshape(4, 15)[0])
    out, done = [], 0
    for n in IN_TREE_STEPS[solver]:
        q, v = _oracle(P, q, v, n - done)
        done = n
        out.append((q, v))
    return out


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
@pytest.mark.parametrize("solver,name", GOLDENS)
def test_one_step_from_newt_snapshots(eng, solver, name, mode):
    w, _, _ = _scene(solver)
    P = M.PackedModels([w])
    gold = _read_f32(name).reshape(4, 15)
    ids = eng.upload(P)
    states = [_mj(gold[row]) for row in range(4)] + _window_states(solver, name)
    for row, (q, v) in enumerate(states):
        slots = eng.alloc(ids)
        eng.set_state(slots, q, v)
        eng.step(1, mode)
        gq, gv = eng.get_state(slots, 8, 7)
        st = int(eng.status(slots)[0])
        eng.free(slots)
        q32, v32 = _oracle(P, q, v, 1)
        q64, v64 = _oracle(P, q, v, 1, precision=1)
        assert not st & 0x3, (row, hex(st))
        gpu = (np.abs(gq - q64).max(), np.abs(gv - v64).max())
        newt = (np.abs(q32 - q64).max(), np.abs(v32 - v64).max())
        assert gpu[0] <= max(2e-6, 2.0 * newt[0]) and gpu[1] <= max(2e-4, 2.0 * newt[1]), (row, gpu, newt)


@pytest.mark.parametrize("solver,name", GOLDENS)
def test_in_tree_contacts_listed_like_the_oracle(eng, solver, name):
    """Inside the windows the two link boxes touch each other: the GPU lists
    the same pairs as the oracle, the in-tree pair among them, with the same
    depths and normals."""
    w, _, _ = _scene(solver)
    P = M.PackedModels([w])
    seen_in_tree = False
    for q, v in _window_states(solver, name):
        slots = eng.alloc(eng.upload(P))
        eng.set_state(slots, q, v)
        eng.step(1, STEP_PLAIN)
        gp, gd = eng.contacts(int(slots[0]))
        eng.free(slots)
        rp, rd = oracle_py.contacts(P, 0, q, v)
        if len(rd) and (np.abs(rd[:, 6]) < 1e-6).any():
            continue
        assert gp.tolist() == rp.tolist()
        if len(rd):
            assert np.abs(gd[:, 6] - rd[:, 6]).max() < 1e-5 and np.abs(gd[:, 3:6] - rd[:, 3:6]).max() < 1e-4
        seen_in_tree |= any(a > 0 and b > 0 for a, b in gp.tolist())  # geom 0 is the plane
    assert seen_in_tree


@functools.lru_cache(maxsize=None)
def _envelope(solver, name, n_runs=32, nudge=1e-7, marks=(50, 200, 1000)):
    """How far newt's own f32 arithmetic lands from its snapshots when the
    root's start position moves by up to `nudge` m, and how far the FP64
    oracle lands (MuJoCo layout): per mark, the larger of the two."""
    w, _, _ = _scene(solver)
    P = M.PackedModels([w])
    gold = _read_f32(name).reshape(4, 15)
    q0, v0 = _mj(gold[0])
    rng = np.random.default_rng(11)
    qs = np.tile(q0, (n_runs, 1))
    qs[:, :3] += rng.uniform(-nudge, nudge, (n_runs, 3)).astype(np.float32)
    qc, vc, done, env = qs.reshape(-1), np.tile(v0, n_runs), 0, []
    for row, n in enumerate(marks, start=1):
        qo, vo = oracle_py.run(P, np.zeros(n_runs, np.int32), qc, vc, None, n - done, precision=0, integrator=0,
                               n_threads=8)
        done = n
        qc, vc = qo.astype(np.float32), vo.astype(np.float32)
        gq, gvv = _mj(gold[row])
        q64, v64 = _oracle(P, q0, v0, n, precision=1)
        env.append((max(float(np.abs(qc.reshape(n_runs, 8) - gq[None]).max()), float(np.abs(q64 - gq).max())),
                    max(float(np.abs(vc.reshape(n_runs, 7) - gvv[None]).max()), float(np.abs(v64 - gvv).max()))))
    return env


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
@pytest.mark.parametrize("solver,name", GOLDENS)
def test_goldens_stay_in_newts_envelope(eng, solver, name, mode):
    w, _, _ = _scene(solver)
    gold = _read_f32(name).reshape(4, 15)
    q0, v0 = _mj(gold[0])
    slots = eng.alloc(eng.upload(M.PackedModels([w])))
    eng.set_state(slots, q0, v0)
    done, errs = 0, []
    for row, n in enumerate((50, 200, 1000), start=1):
        eng.step(n - done, mode)
        done = n
        gq, gv = eng.get_state(slots, 8, 7)
        rq, rv = _mj(gold[row])
        errs.append((float(np.abs(gq - rq).max()), float(np.abs(gv - rv).max())))
    assert not (eng.status(slots) & 0x7).any()
    eng.free(slots)
    env = _envelope(solver, name)
    for (dq, dv), (eq, ev) in zip(errs, env):
        assert dq <= max(5e-4, 1.25 * eq) and dv <= max(5e-3, 1.25 * ev), (errs, env)
