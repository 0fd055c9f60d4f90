"""The oracle's accelerometer on links and its force and torque sensors on
trees without geoms (newt/src/sensor.rs:446-530, 620-647, 834-1087)
against newt's anchors (CPU).

sensors_battery.rs:729-877: a horizontal two-link arm held static by
qfrc_applied = the bias forces h(q, 0): the forearm's elbow reads force
(0, 9.81, 0) and torque (4.905, 0, 0) within 0.05.  sensors_battery.rs:
188-218: an accelerometer at the COM of a free-root link, spinning and
translating in free fall, reads zero within 5e-3.  sensors_battery.rs:
220-305: a free-root link and a free body in the same state read the same
accelerometer at an offset site within 1e-3; the body's reading is taken
here from Newton's and Euler's equations directly (a = g, alpha = I^-1
(-w x I w)), evaluated in double.
"""
import numpy as np
import pytest

import oracle_py
from f32util import quat_from_axis_angle
from tooling_gb300 import api as A
from tooling_gb300 import model as M

G = (0.0, 0.0, -9.81)


def elbow_arm():
    """sensors_battery.rs:776-816: fixed root at the origin, rod 1 hinged
    about +x at the root with its COM 0.5 from the joint, rod 2 hinged at
    rod 1's far end; q1 = pi/2, q2 = 0 (the arm horizontal along +y)."""
    w = M.WorldModel(dt=0.005, gravity=G, solver=0)
    w.push_link(M.Link(parent=-1, joint=M.JOINT_FIXED, mass=1.0, inertia=M._diag9(1.0, 1.0, 1.0)))
    w.push_link(M.Link(parent=0, joint=M.JOINT_HINGE, axis=(1.0, 0.0, 0.0), jc_pos=(0.0, 0.0, 0.5), mass=1.0,
                       inertia=M._diag9(1e-3, 1e-3, 1e-3)))
    w.push_link(M.Link(parent=1, joint=M.JOINT_HINGE, axis=(1.0, 0.0, 0.0), jp_pos=(0.0, 0.0, -0.5),
                       jc_pos=(0.0, 0.0, 0.5), mass=1.0, inertia=M._diag9(1e-3, 1e-3, 1e-3)))
    return w, np.array([np.pi / 2, 0.0], np.float32), np.zeros(2, np.float32)


def bias_forces(P, q, v):
    """h(q, v) = -M qacc(q, v, qfrc = 0): with qfrc_applied = h the ABA's
    qddot is zero (newt's bias_forces, dynamics.rs)."""
    _, _, qacc = oracle_py.run(P, np.zeros(1, np.int32), q, v, None, 1, precision=1, want_qacc=True)
    Mm = oracle_py.mass_matrix(P, 0, q, len(v))
    return (-(Mm @ qacc)).astype(np.float32)


ELBOW = A.sensors((A.SENSOR_FORCE, 1, 2), (A.SENSOR_TORQUE, 1, 2))


@pytest.mark.parametrize("precision", [0, 1])
def test_elbow_force_torque_match_statics(precision):
    w, q, v = elbow_arm()
    P = M.PackedModels([w])
    h = bias_forces(P, q, v)
    r = oracle_py.sensors(P, 0, q, v, ELBOW, precision=precision, qfrc=h)
    assert np.abs(r[0:3] - np.array([0.0, 9.81, 0.0])).max() < 0.05, r
    assert np.abs(r[3:6] - np.array([4.905, 0.0, 0.0])).max() < 0.05, r


def free_link(pos, quat_xyzw, omega_body, v_world, mass=1.5, inertia=(0.4, 0.6, 0.5)):
    w = M.WorldModel(dt=0.005, gravity=G, solver=0)
    w.push_link(M.Link(parent=-1, joint=M.JOINT_FREE, mass=mass, inertia=M._diag9(*inertia)))
    x, y, z, ww = quat_xyzw
    q = np.array(list(pos) + [ww, x, y, z], np.float32)
    v = np.array(list(v_world) + list(omega_body), np.float32)
    return w, q, v


@pytest.mark.parametrize("precision", [0, 1])
def test_free_fall_link_accelerometer_at_com_reads_zero(precision):
    quat = quat_from_axis_angle((1.0, 0.4, -0.2), 0.6)
    Rm = _rot(quat)
    w, q, v = free_link((0.5, -0.3, 2.0), quat, (1.2, -0.7, 0.9), Rm @ np.array([0.4, 0.6, -0.3]))
    sens = A.sensors((A.SENSOR_ACCELEROMETER, 1, 0, (0.0, 0.0, 0.0), quat_from_axis_angle((0.0, 1.0, 0.0), np.pi / 6)))
    r = oracle_py.sensors(M.PackedModels([w]), 0, q, v, sens, precision=precision)
    assert np.abs(r).max() < 5e-3, r


def _rot(q_xyzw):
    x, y, z, w = (float(c) for c in q_xyzw)
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def body_path_reading(quat, omega_body, inertia, offset, site_quat):
    """A free body's accelerometer with no contacts (sensor.rs:528-548,
    1030-1087): a_com = g, alpha_body = I^-1 (-w x I w)."""
    Rm = _rot(quat)
    I = np.diag(inertia)
    wb = np.array(omega_body, np.float64)
    alpha_b = np.linalg.solve(I, -np.cross(wb, I @ wb))
    om, al, r = Rm @ wb, Rm @ alpha_b, Rm @ np.array(offset, np.float64)
    a_site = np.array(G) + np.cross(al, r) + np.cross(om, np.cross(om, r))
    return (Rm @ _rot(site_quat)).T @ (a_site - np.array(G))


@pytest.mark.parametrize("precision", [0, 1])
def test_link_and_body_accelerometer_paths_agree(precision):
    quat = quat_from_axis_angle((0.4, 1.0, -0.3), 0.7)
    omega_body, offset = (0.8, -0.4, 1.1), (0.15, -0.1, 0.2)
    site_quat = quat_from_axis_angle((0.0, 1.0, 0.0), np.pi / 6)
    w, q, v = free_link((1.3, -0.5, 4.0), quat, omega_body, (0.3, 0.4, -0.5))
    sens = A.sensors((A.SENSOR_ACCELEROMETER, 1, 0, offset, site_quat))
    r = oracle_py.sensors(M.PackedModels([w]), 0, q, v, sens, precision=precision)
    ref = body_path_reading(quat, omega_body, (0.4, 0.6, 0.5), offset, site_quat)
    assert np.abs(r - ref).max() < 1e-3, (r, ref)
