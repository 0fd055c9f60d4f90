"""The oracle's post-step contact sensors (accelerometer, touch) against
newt's anchors (CPU).

newt/tests/sensors_battery.rs:41-108: a sphere (radius 0.5, 1 kg) resting on
a plane reads (0, 0, +9.81) on an accelerometer at its centre, and
(0, 9.81, 0) when the site is turned 90 degrees about x; :111-160: a body
spinning at 3 rad/s about z with no gravity and no contact reads the
centripetal (-4.5, 0, 0) at the site (0.5, 0, 0); :696-719: touch on the
resting sphere under PGS reads about m g (newt's band: 0.4 to 3 m g).  The
oracle re-solves the step's contacts at the post-step state, as newt does
(world.rs:1545-1612)."""
import numpy as np
import pytest

import oracle_py
from f32util import quat_from_axis_angle
from tooling_gb300 import api as A
from tooling_gb300 import model as M


def resting_sphere(solver=M.SOLVER_PGS, gravity=-9.81):
    """sensors_battery.rs:24-37: a 1 kg sphere of radius 0.5 on a plane
    (friction 0.5), here under PGS 40 (or Newton) and dt 2e-3."""
    w = M.WorldModel(dt=0.002, gravity=(0.0, 0.0, gravity), solver=solver, iterations=40)
    w.add_geom(M.static_plane(friction=0.5))
    b = w.add_body(1.0, M.solid_sphere_inertia(1.0, 0.5))
    w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, body=b, size=(0.5, 0.0, 0.0), friction=0.5))
    qpos = np.array([0.0, 0.0, 0.5, 1.0, 0.0, 0.0, 0.0], np.float32)  # MuJoCo layout (quat w x y z)
    return w, qpos, np.zeros(6, np.float32)


def _settle(w, qpos, qvel, n=800, precision=1):
    q, v = oracle_py.run(M.PackedModels([w]), np.zeros(1, np.int32), qpos, qvel, None, n, precision=precision)
    return q.astype(np.float32), v.astype(np.float32)


SENS = A.sensors(
    (A.SENSOR_ACCELEROMETER, 0, 0),
    (A.SENSOR_ACCELEROMETER, 0, 0, (0.0, 0.0, 0.0), tuple(quat_from_axis_angle((1.0, 0.0, 0.0), np.pi / 2))),
    (A.SENSOR_TOUCH, 0, 1),
    (A.SENSOR_TOUCH, 0, 0),
)


@pytest.mark.parametrize("solver", [M.SOLVER_PGS, M.SOLVER_NEWTON])
@pytest.mark.parametrize("precision", [0, 1])
def test_resting_sphere_reads_plus_g_and_mg(solver, precision):
    w, q, v = resting_sphere(solver)
    q, v = _settle(w, q, v, precision=precision)
    r, _, _ = oracle_py.contact_sensors(M.PackedModels([w]), 0, q, v, SENS, precision=precision)
    np.testing.assert_allclose(r[0:3], [0.0, 0.0, 9.81], atol=1e-3)
    np.testing.assert_allclose(r[3:6], [0.0, 9.81, 0.0], atol=1e-3)
    # the sphere's geom and the plane see the same contact: m g at rest
    assert abs(r[6] - 9.81) < 1e-2 and abs(r[7] - 9.81) < 1e-2, r[6:8]


def test_spinning_body_reads_centripetal():
    w = M.WorldModel(dt=0.005, gravity=(0.0, 0.0, 0.0), solver=M.SOLVER_PGS, iterations=10)
    w.add_geom(M.static_plane(point=(0.0, 0.0, -10.0)))
    b = w.add_body(1.0, M.solid_sphere_inertia(1.0, 0.25))
    w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, body=b, size=(0.25, 0.0, 0.0)))
    q = np.array([0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0], np.float32)
    v = np.array([0.0, 0.0, 0.0, 0.0, 0.0, 3.0], np.float32)  # v_world, omega_body
    sens = A.sensors((A.SENSOR_ACCELEROMETER, 0, 0, (0.5, 0.0, 0.0)))
    r, _, _ = oracle_py.contact_sensors(M.PackedModels([w]), 0, q, v, sens)
    # the site turned with the body through one step: the reading stays in
    # the site frame, where the centripetal acceleration points at the axis
    np.testing.assert_allclose(r, [-4.5, 0.0, 0.0], atol=1e-9)


def test_falling_body_reads_zero_and_touch_reads_nothing():
    w, q, v = resting_sphere()
    q = q.copy()
    q[2] = 3.0  # well above the plane: free fall, no contact
    r, _, _ = oracle_py.contact_sensors(M.PackedModels([w]), 0, q, v, SENS)
    np.testing.assert_allclose(r[0:6], 0.0, atol=1e-9)
    assert r[6] == 0.0 and r[7] == 0.0
