"""Post-step sensors on the GPU (newt_gpu_read_sensors) against the oracle's
restatement of newt/src/sensor.rs, evaluated at the GPU's own state so that
only the sensor evaluation is compared: within 2e-5 (positions, quaternions)
and 2e-4 relative (velocities) on 7-link chains, quadrupeds (tree-contact
worlds) and piles; newt's posed-arm anchor (tip at (0, 1, 1),
sensors_battery.rs:432-555) on the GPU; attachment errors refused."""
import numpy as np
import pytest

import oracle_py
from test_oracle_sensors import ARM_SENSORS, posed_arm
from tooling_gb300 import Engine, NewtError, STEP_BATCHED, scenes
from tooling_gb300 import api as A
from tooling_gb300 import model as M

pytestmark = pytest.mark.gpu

FRAME = ((0.03, -0.02, 0.05), (0.1, 0.2, -0.3, 0.9273618))  # a site off the parent's origin, turned


@pytest.fixture(scope="module")
def eng():
    from tooling_gb300 import build as B
    B.build()
    e = Engine(device=0)
    yield e
    e.close()


def _site_sensors(on_link, idx):
    lp, lq = FRAME
    lq = tuple(np.asarray(lq) / np.linalg.norm(lq))
    return [(k, on_link, idx, lp, lq) for k in (A.SENSOR_FRAMEPOS, A.SENSOR_FRAMEQUAT, A.SENSOR_GYRO,
                                                  A.SENSOR_VELOCIMETER, A.SENSOR_FRAMELINVEL,
                                                  A.SENSOR_FRAMEANGVEL)]


def _compare(eng, b, slots, sens):
    q, v = eng.get_state(slots, int(b.nq.sum()), int(b.nv.sum()))
    got = eng.read_sensors(slots, sens)
    worst = 0.0
    for w in range(len(slots)):
        qp, qv = q[b.q_off[w]:b.q_off[w] + b.nq[w]], v[b.v_off[w]:b.v_off[w] + b.nv[w]]
        ref = oracle_py.sensors(b, w, qp, qv, sens)
        scale = np.maximum(1.0, np.abs(ref))
        worst = max(worst, float((np.abs(got[w] - ref) / scale).max()))
    return worst


def test_posed_arm_anchor_on_gpu(eng):
    w, q = posed_arm()
    P = M.PackedModels([w])
    slots = eng.alloc(eng.upload(P))
    qd = np.array([1.0, 0.0], np.float32)
    eng.set_state(slots, q, qd)
    got = eng.read_sensors(slots, ARM_SENSORS)[0]
    eng.free(slots)
    ref = oracle_py.sensors(P, 0, q, qd, ARM_SENSORS)
    np.testing.assert_allclose(got[0:3], [0.0, 1.0, 1.0], atol=1e-6)
    np.testing.assert_allclose(got, ref, atol=2e-6)


def test_chain_sensors_match_oracle(eng):
    b = scenes.chain_batch(n_worlds=64, first_world=100)
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, b.qpos, b.qvel)
    eng.set_qfrc(slots, b.qfrc)
    eng.step(30, STEP_BATCHED)
    sens = A.sensors(*_site_sensors(1, 7), (A.SENSOR_JOINTPOS, 1, 4), (A.SENSOR_JOINTVEL, 1, 7),
                     (A.SENSOR_SUBTREECOM, 1, 2), (A.SENSOR_SUBTREECOM, 1, 0))
    worst = _compare(eng, b, slots, sens)
    eng.free(slots)
    assert worst < 2e-4, worst


def test_quadruped_sensors_match_oracle(eng):
    b = scenes.quadruped_batch(n_worlds=32, first_world=300, solver=M.SOLVER_NEWTON)
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, b.qpos, b.qvel)
    eng.step(200, STEP_BATCHED)  # standing on the plane by now
    sens = A.sensors(*_site_sensors(1, 12), (A.SENSOR_GYRO, 1, 0), (A.SENSOR_JOINTPOS, 1, 5),
                     (A.SENSOR_JOINTVEL, 1, 5), (A.SENSOR_SUBTREECOM, 1, 0), (A.SENSOR_SUBTREECOM, 1, 1))
    worst = _compare(eng, b, slots, sens)
    eng.free(slots)
    assert worst < 2e-4, worst


def test_pile_sensors_match_oracle(eng):
    b = scenes.pile_batch(n_worlds=48, first_world=500)
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, b.qpos, b.qvel)
    eng.step(200, STEP_BATCHED)
    sens = A.sensors(*_site_sensors(0, 3), *_site_sensors(0, 15)[:2])
    worst = _compare(eng, b, slots, sens)
    eng.free(slots)
    assert worst < 2e-4, worst


def test_sensor_attachment_errors(eng):
    b = scenes.pile_batch(n_worlds=1)
    slots = eng.alloc(eng.upload(b))
    with pytest.raises(NewtError):  # a link sensor on a free-body world
        eng.read_sensors(slots, A.sensors((A.SENSOR_FRAMEPOS, 1, 0)))
    with pytest.raises(NewtError):  # body index out of range
        eng.read_sensors(slots, A.sensors((A.SENSOR_FRAMEPOS, 0, 16)))
    eng.free(slots)
    w, _ = posed_arm()
    slots = eng.alloc(eng.upload(M.PackedModels([w])))
    with pytest.raises(NewtError):  # joint sensors read hinge or slide links, not the fixed root
        eng.read_sensors(slots, A.sensors((A.SENSOR_JOINTPOS, 1, 0)))
    eng.free(slots)
