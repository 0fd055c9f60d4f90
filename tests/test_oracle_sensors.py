"""The oracle's post-step sensors against newt's hand-derived anchors (CPU).

newt/tests/sensors_battery.rs:432-555 poses a two-link arm (both hinges at
pi/2 about +x, rods of length 1): the tip site reads (0, 1, 1) and the
orientation +-(1, 0, 0, 0).  sensors_battery.rs:306-375: a gyro whose site is
turned 90 degrees about z reads (-0.7, -0.5, 1.1) for a body spinning at
(0.5, -0.7, 1.1).  The velocity and subtree-centre cases below are derived by
hand the same way.
"""
import numpy as np

import oracle_py
from f32util import quat_from_axis_angle
from tooling_gb300 import api as A
from tooling_gb300 import model as M


def posed_arm():
    """sensors_battery.rs:442-480: fixed root at the origin, two unit rods
    hinged about +x, each COM 0.5 from its joint."""
    w = M.WorldModel(dt=0.005, gravity=(0.0, 0.0, 0.0), solver=0)
    w.push_link(M.Link(parent=-1, joint=M.JOINT_FIXED, mass=1.0, inertia=M._diag9(1.0, 1.0, 1.0)))
    w.push_link(M.Link(parent=0, joint=M.JOINT_HINGE, axis=(1.0, 0.0, 0.0), jc_pos=(0.0, 0.0, 0.5), mass=1.0,
                       inertia=M._diag9(1e-3, 1e-3, 1e-3)))
    w.push_link(M.Link(parent=1, joint=M.JOINT_HINGE, axis=(1.0, 0.0, 0.0), jp_pos=(0.0, 0.0, -0.5),
                       jc_pos=(0.0, 0.0, 0.5), mass=1.0, inertia=M._diag9(1e-3, 1e-3, 1e-3)))
    return w, np.array([np.pi / 2, np.pi / 2], np.float32)


ARM_SENSORS = A.sensors(
    (A.SENSOR_FRAMEPOS, 1, 2, (0.0, 0.0, -0.5)),
    (A.SENSOR_FRAMEQUAT, 1, 2, (0.0, 0.0, -0.5)),
    (A.SENSOR_JOINTPOS, 1, 1),
    (A.SENSOR_JOINTVEL, 1, 2),
    (A.SENSOR_SUBTREECOM, 1, 1),
    (A.SENSOR_SUBTREECOM, 1, 0),
    (A.SENSOR_FRAMELINVEL, 1, 1),
    (A.SENSOR_FRAMEANGVEL, 1, 1),
    (A.SENSOR_GYRO, 1, 1),
    (A.SENSOR_VELOCIMETER, 1, 2, (0.0, 0.0, -0.5)),
)


def test_posed_arm_anchors():
    w, q = posed_arm()
    qd = np.array([1.0, 0.0], np.float32)
    r = oracle_py.sensors(M.PackedModels([w]), 0, q, qd, ARM_SENSORS)
    np.testing.assert_allclose(r[0:3], [0.0, 1.0, 1.0], atol=1e-6)  # the tip
    quat = r[3:7]
    assert min(np.abs(quat - [1, 0, 0, 0]).max(), np.abs(quat + [1, 0, 0, 0]).max()) < 1e-6
    assert r[7] == np.float32(np.pi / 2) and r[8] == 0.0
    # rod COMs at (0, .5, 0) and (0, 1, .5), root at the origin, unit masses
    np.testing.assert_allclose(r[9:12], [0.0, 0.75, 0.25], atol=1e-6)
    np.testing.assert_allclose(r[12:15], [0.0, 0.5, 0.5 / 3.0], atol=1e-6)
    # shoulder turning at 1 rad/s about +x: rod 1's COM at (0, .5, 0) moves at (0, 0, .5)
    np.testing.assert_allclose(r[15:18], [0.0, 0.0, 0.5], atol=1e-6)
    np.testing.assert_allclose(r[18:21], [1.0, 0.0, 0.0], atol=1e-6)
    # rod 1 is turned pi/2 about x: its body-frame rate is still (1, 0, 0)
    np.testing.assert_allclose(r[21:24], [1.0, 0.0, 0.0], atol=1e-6)
    # the tip (0, 1, 1) turns about the origin: (1,0,0) x (0,1,1) = (0,-1,1) in
    # the world; the tip frame is Rot_x(pi): (0, 1, -1) in it
    np.testing.assert_allclose(r[24:27], [0.0, 1.0, -1.0], atol=1e-6)


def _spinning_body():
    w = M.WorldModel(dt=0.005, gravity=(0.0, 0.0, 0.0), solver=M.SOLVER_PGS, iterations=1)
    w.add_body(1.0, M._diag9(1.0, 2.0, 3.0))
    w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, body=0, size=(0.05, 0.0, 0.0)))
    qpos = np.array([0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0], np.float32)
    qvel = np.array([0.0, 0.0, 0.0, 0.5, -0.7, 1.1], np.float32)
    return w, qpos, qvel


def test_gyro_site_rotation_anchor():
    w, qpos, qvel = _spinning_body()
    rot = quat_from_axis_angle((0.0, 0.0, 1.0), np.pi / 2)
    s = A.sensors((A.SENSOR_GYRO, 0, 0, (0.1, 0.2, 0.3), tuple(float(x) for x in rot)))
    r = oracle_py.sensors(M.PackedModels([w]), 0, qpos, qvel, s)
    np.testing.assert_allclose(r, [-0.7, -0.5, 1.1], atol=1e-6)


def test_body_site_velocity_anchor():
    """A body at rest translating at (1, 0, 0) and spinning at 2 rad/s about
    z; a site 1 m out along x moves at (1, 2, 0); the velocimeter of a site
    turned 90 degrees about z reads (2, -1, 0)."""
    w, qpos, _ = _spinning_body()
    qvel = np.array([1.0, 0.0, 0.0, 0.0, 0.0, 2.0], np.float32)
    rot = tuple(float(x) for x in quat_from_axis_angle((0.0, 0.0, 1.0), np.pi / 2))
    s = A.sensors((A.SENSOR_FRAMELINVEL, 0, 0, (1.0, 0.0, 0.0)), (A.SENSOR_FRAMEANGVEL, 0, 0),
                  (A.SENSOR_VELOCIMETER, 0, 0, (1.0, 0.0, 0.0), rot), (A.SENSOR_FRAMEPOS, 0, 0, (1.0, 0.0, 0.0)))
    r = oracle_py.sensors(M.PackedModels([w]), 0, qpos, qvel, s)
    np.testing.assert_allclose(r, [1.0, 2.0, 0.0, 0.0, 0.0, 2.0, 2.0, -1.0, 0.0, 1.0, 0.0, 0.0], atol=1e-6)
