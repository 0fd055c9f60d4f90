"""Accelerometer and touch sensors on the GPU (newt_gpu_read_sensors on pile
worlds: the last step's contacts re-solved at the post-step state, as newt's
World::step evaluates them) against the oracle, whose readings hold newt's
anchors (tests/test_oracle_contact_sensors.py).

Bars: on a resting sphere, the FP64 oracle's readings within 1e-3 (m/s^2,
N); on settled 16-body piles under PGS (plain and batched forms) and under
Newton, every reading no further from the FP64 oracle than twice newt's own
f32 arithmetic, or 1e-3 of the largest reading of its kind where newt's is
closer."""
import numpy as np
import pytest

import oracle_py
from test_oracle_contact_sensors import SENS, resting_sphere, _settle
from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN, scenes
from tooling_gb300 import api as A
from tooling_gb300 import model as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from tooling_gb300 import build as B
    B.build()
    e = Engine(device=0)
    yield e
    e.close()


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
@pytest.mark.parametrize("solver", [M.SOLVER_PGS, M.SOLVER_NEWTON])
def test_resting_sphere_matches_oracle(eng, solver, mode):
    w, q, v = resting_sphere(solver)
    q, v = _settle(w, q, v)
    packed = M.PackedModels([w])
    slots = eng.alloc(eng.upload(packed))
    eng.set_state(slots, q, v)
    eng.step(1, mode)
    got = eng.read_sensors(slots, SENS)[0]
    eng.free(slots)
    ref, _, _ = oracle_py.contact_sensors(packed, 0, q, v, SENS)
    np.testing.assert_allclose(got, ref, atol=1e-3)
    np.testing.assert_allclose(got[0:3], [0.0, 0.0, 9.81], atol=2e-3)
    assert abs(got[6] - 9.81) < 2e-2


def test_reads_no_contacts_before_a_first_step(eng):
    w, q, v = resting_sphere()
    q, v = _settle(w, q, v)
    slots = eng.alloc(eng.upload(M.PackedModels([w])))
    eng.set_state(slots, q, v)
    got = eng.read_sensors(slots, SENS)[0]
    eng.free(slots)
    assert got[6] == 0.0 and got[7] == 0.0
    np.testing.assert_allclose(got[0:3], 0.0, atol=1e-6)  # no contact force: free fall


def _pile_sensors(nb=16):
    specs = [(A.SENSOR_TOUCH, 0, 0)]
    for b in range(0, nb, 3):
        specs.append((A.SENSOR_ACCELEROMETER, 0, b, (0.05, -0.02, 0.03)))
        specs.append((A.SENSOR_TOUCH, 0, b + 1))
    return A.sensors(*specs)


def _settled(solver):
    b = scenes.pile_batch(n_worlds=12, first_world=1500)
    rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, None, 300, precision=1)
    nw = M.Batch(b.links, b.n_links, b.bodies, b.n_bodies, b.geoms, b.n_geoms, 2e-3, (0.0, 0.0, -9.81), solver,
                 50 if solver == M.SOLVER_PGS else 20)
    nw.qpos[:] = rq.astype(np.float32)
    nw.qvel[:] = rv.astype(np.float32)
    return nw


@pytest.mark.parametrize("solver,mode", [(M.SOLVER_PGS, STEP_PLAIN), (M.SOLVER_PGS, STEP_BATCHED),
                                         (M.SOLVER_NEWTON, STEP_BATCHED)])
def test_settled_piles_match_fp64(eng, solver, mode):
    b = _settled(solver)
    sens = _pile_sensors()
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, b.qpos, b.qvel)
    eng.step(1, mode)
    got = eng.read_sensors(slots, sens)
    eng.free(slots)
    touch = np.array([k == A.SENSOR_TOUCH for k in sens["kind"] for _ in range(1 if k == A.SENSOR_TOUCH else 3)])
    worst, checked = 0.0, 0
    for w in range(len(b)):
        qp = b.qpos[b.q_off[w]:b.q_off[w] + b.nq[w]]
        qv = b.qvel[b.v_off[w]:b.v_off[w] + b.nv[w]]
        rp, rd = oracle_py.contacts(b, w, qp, qv)
        if len(rd) and (np.abs(rd[:, 6]) < 1e-6).any():
            continue  # a contact at the margin: the two sides may see different sets
        r64, _, _ = oracle_py.contact_sensors(b, w, qp, qv, sens, precision=1)
        r32, _, _ = oracle_py.contact_sensors(b, w, qp, qv, sens, precision=0)
        for part in (touch, ~touch):
            scale = max(np.abs(r64[part]).max(), 1.0)
            gpu = np.abs(got[w][part] - r64[part]).max()
            newt = np.abs(r32[part] - r64[part]).max()
            assert gpu <= max(1e-3 * scale, 2.0 * newt), (w, part.sum(), gpu, newt, scale)
            worst = max(worst, gpu / scale)
        checked += 1
    assert checked >= 8, checked
    assert got[:, 0].min() > 0.0  # every pile rests on the plane
