"""Accelerometers on links, force and torque sensors on the GPU (trees
without geoms; tree_sensor_dyn_kernel and tree_sensors_kernel), through
newt_gpu_read_sensors, against the oracle, which holds newt's anchors
(tests/test_oracle_tree_dyn_sensors.py).

Bars: newt's anchors on the GPU (the elbow's statics within 0.05, the
free-falling link's accelerometer at its COM below 5e-3, link and body
accelerometer paths within 1e-3) and the FP64 oracle within 1e-4 there; on
64 seven-link chains with random joint torques and on floating trees with a
swinging arm, every reading no further from the FP64 oracle than twice
newt's own f32 arithmetic, or within 1e-4 of the reading's size (floor 1)
where newt's is closer; the forms the GPU refuses (touch on a tree without
geoms, force sensors on bodies) are refused.  Tree-contact worlds:
tests/test_gpu_tree_contact_sensors.py."""
import numpy as np
import pytest

import oracle_py
from f32util import quat_from_axis_angle
from test_oracle_golden import _joints_floating
from test_oracle_tree_dyn_sensors import ELBOW, bias_forces, body_path_reading, elbow_arm, free_link, _rot
from tooling_gb300 import Engine, NewtError, STEP_BATCHED, scenes
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


def _read(eng, P, q, v, sens, qfrc=None):
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q, v)
    if qfrc is not None:
        eng.set_qfrc(slots, qfrc)
    got = eng.read_sensors(slots, sens)[0]
    eng.free(slots)
    return got


def test_elbow_statics_on_gpu(eng):
    w, q, v = elbow_arm()
    P = M.PackedModels([w])
    h = bias_forces(P, q, v)
    got = _read(eng, P, q, v, ELBOW, h)
    ref = oracle_py.sensors(P, 0, q, v, ELBOW, qfrc=h)
    assert np.abs(got[0:3] - np.array([0.0, 9.81, 0.0])).max() < 0.05, got
    assert np.abs(got[3:6] - np.array([4.905, 0.0, 0.0])).max() < 0.05, got
    assert np.abs(got - ref).max() < 1e-4, (got, ref)


def test_free_fall_link_accelerometer_on_gpu(eng):
    quat = quat_from_axis_angle((1.0, 0.4, -0.2), 0.6)
    w, q, v = free_link((0.5, -0.3, 2.0), quat, (1.2, -0.7, 0.9), _rot(quat) @ np.array([0.4, 0.6, -0.3]))
    sens = A.sensors((A.SENSOR_ACCELEROMETER, 1, 0, (0.0, 0.0, 0.0), quat_from_axis_angle((0.0, 1.0, 0.0), np.pi / 6)))
    P = M.PackedModels([w])
    got = _read(eng, P, q, v, sens)
    assert np.abs(got).max() < 5e-3, got
    assert np.abs(got - oracle_py.sensors(P, 0, q, v, sens)).max() < 1e-4


def test_link_and_body_accelerometer_paths_agree_on_gpu(eng):
    quat = quat_from_axis_angle((0.4, 1.0, -0.3), 0.7)
    omega_body, offset = (0.8, -0.4, 1.1), (0.15, -0.1, 0.2)
    site_quat = quat_from_axis_angle((0.0, 1.0, 0.0), np.pi / 6)
    w, q, v = free_link((1.3, -0.5, 4.0), quat, omega_body, (0.3, 0.4, -0.5))
    got = _read(eng, M.PackedModels([w]), q, v, A.sensors((A.SENSOR_ACCELEROMETER, 1, 0, offset, site_quat)))
    ref = body_path_reading(quat, omega_body, (0.4, 0.6, 0.5), offset, site_quat)
    assert np.abs(got - ref).max() < 1e-3, (got, ref)


def _against_fp64(eng, b, slots, sens, qfrc):
    q, v = eng.get_state(slots, int(b.nq.sum()), int(b.nv.sum()))
    got = eng.read_sensors(slots, sens)
    worst = 0.0
    for w in range(len(slots)):
        qp, qv = q[b.q_off[w]:b.q_off[w] + b.nq[w]], v[b.v_off[w]:b.v_off[w] + b.nv[w]]
        qf = qfrc[b.v_off[w]:b.v_off[w] + b.nv[w]]
        r64 = oracle_py.sensors(b, w, qp, qv, sens, precision=1, qfrc=qf)
        r32 = oracle_py.sensors(b, w, qp, qv, sens, precision=0, qfrc=qf)
        scale = np.maximum(1.0, np.abs(r64))
        gpu, newt = np.abs(got[w] - r64), np.abs(r32 - r64)
        assert (gpu <= np.maximum(1e-4 * scale, 2.0 * newt)).all(), (w, gpu, newt, r64)
        worst = max(worst, float((gpu / scale).max()))
    return worst


def test_chain_force_torque_accelerometer_match_fp64(eng):
    b = scenes.chain_batch(n_worlds=64, first_world=700)
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, b.qpos, b.qvel)
    eng.set_qfrc(slots, b.qfrc)
    eng.step(30, STEP_BATCHED)
    sens = A.sensors((A.SENSOR_FORCE, 1, 1), (A.SENSOR_TORQUE, 1, 1), (A.SENSOR_FORCE, 1, 4),
                     (A.SENSOR_TORQUE, 1, 7), (A.SENSOR_ACCELEROMETER, 1, 3, (0.02, -0.03, 0.1)),
                     (A.SENSOR_ACCELEROMETER, 1, 7, (0.0, 0.01, -0.05), (0.1, 0.2, -0.3, 0.9273618)),
                     (A.SENSOR_JOINTPOS, 1, 2))
    _against_fp64(eng, b, slots, sens, b.qfrc)
    eng.free(slots)


def test_floating_tree_sensors_match_fp64(eng):
    rng = np.random.default_rng(17)
    worlds, qs, vs = [], [], []
    for k in range(8):
        quat = quat_from_axis_angle(tuple(rng.normal(size=3)), float(rng.uniform(0.1, 2.0)))
        w = _joints_floating(quat)
        w.gravity = (0.0, 0.0, -9.81)
        worlds.append(w)
        x, y, z, ww = quat
        qs.append(np.array([0.5, -1.0, 4.5, ww, x, y, z, rng.uniform(-1, 1)], np.float32))
        vs.append(rng.normal(0.0, 1.0, 7).astype(np.float32))
    b = M.PackedModels(worlds)
    q, v = np.concatenate(qs), np.concatenate(vs)
    qfrc = np.zeros(len(v), np.float32)
    qfrc[6::7] = rng.normal(0.0, 0.5, len(worlds))  # the arm's hinge only
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, q, v)
    eng.set_qfrc(slots, qfrc)
    sens = A.sensors((A.SENSOR_FORCE, 1, 1), (A.SENSOR_TORQUE, 1, 1), (A.SENSOR_FORCE, 1, 0),
                     (A.SENSOR_ACCELEROMETER, 1, 0, (0.1, 0.05, -0.1)), (A.SENSOR_ACCELEROMETER, 1, 1))
    _against_fp64(eng, _Offsets(b, worlds), slots, sens, qfrc)
    eng.free(slots)


class _Offsets:
    """The batch's per-world state offsets, for a PackedModels."""

    def __init__(self, packed, worlds):
        self.descs = packed.descs
        self.nq = np.array([w.nq for w in worlds])
        self.nv = np.array([w.nv for w in worlds])
        self.q_off = np.concatenate([[0], np.cumsum(self.nq)[:-1]])
        self.v_off = np.concatenate([[0], np.cumsum(self.nv)[:-1]])


def test_refusals(eng):
    c = scenes.chain_batch(n_worlds=2, first_world=5)
    slots = eng.alloc(eng.upload(c))
    with pytest.raises(NewtError):
        eng.read_sensors(slots, A.sensors((A.SENSOR_TOUCH, 1, 0)))
    with pytest.raises(NewtError):
        eng.read_sensors(slots, A.sensors((A.SENSOR_FORCE, 0, 1)))
    eng.free(slots)
