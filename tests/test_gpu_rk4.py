"""RK4 (newt's default integrator) for trees without geoms on the GPU.

Pinned to newt's own output: the joints golden (newt/tests/joints_golden.rs:
a fixed-root hinge chain and a floating box with an arm, RK4, f32) after 100
and 1000 steps; and tracked against the FP64 oracle's RK4 on the 7-link
chains.  Worlds with geoms stay on Euler (their contacts use it)."""
import numpy as np
import pytest

import oracle_py
from test_oracle_golden import _joints_chain, _joints_floating, _read_f32
from tooling_gb300 import Engine, NewtError, STEP_BATCHED, STEP_PLAIN, scenes
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


def test_rk4_refused_for_worlds_with_geoms(eng):
    p = scenes.pile_batch(n_worlds=1)
    rk = M.Batch(p.links, p.n_links, p.bodies, p.n_bodies, p.geoms, p.n_geoms, 2e-3, (0.0, 0.0, -9.81),
                 M.SOLVER_PGS, 50, integrator=M.INTEGRATOR_RK4)
    with pytest.raises(NewtError):
        eng.upload(rk)
