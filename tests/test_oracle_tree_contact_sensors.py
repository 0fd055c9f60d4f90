"""The oracle's contact sensors on tree-contact worlds (CPU): touch, link
accelerometers, force and torque readings under the wrenches of newt's
contact re-solve (newt/src/world.rs:2252-2300, solver.rs:3334-3364,
sensor.rs:1103-1112).

sensors_battery.rs:646-692: a free-root link carrying a sphere of radius
0.4 and mass 1.25, dropped from 0.01 above a plane, reads touch = m g
within 0.8 after 800 steps.  newt runs that anchor under its penalty
contact model; the batched path has no penalty mode, so the same scene runs
here under PGS (40 iterations, the iteration count of newt's PGS touch
anchor, sensors_battery.rs:696-720).  At rest the link's accelerometer
reads +g along its up axis and the free root's force sensor reads the zero
net wrench, both within the same 0.8.

tree_contacts_solver.rs:366-403: two spheres on one free-root link, the
upper one inside its contact gap above a second plane: the force-free gap
contact comes first in the contact list and the lower sphere's touch still
reads its contact's force (above 1).  newt picks the two pairs with an
explicit pair list; collision groups and masks pick the same two here."""
import numpy as np
import pytest

import oracle_py
from tooling_gb300 import api as A
from tooling_gb300 import model as M

MASS, RADIUS = 1.25, 0.4


def resting_sphere_link(solver=M.SOLVER_PGS):
    """sensors_battery.rs:650-680 under PGS: plane geom 0, sphere geom 1."""
    w = M.WorldModel(dt=0.005, gravity=(0.0, 0.0, -9.81), solver=solver, iterations=40)
    w.push_link(M.Link(parent=-1, joint=M.JOINT_FREE, mass=MASS, inertia=M.solid_sphere_inertia(MASS, RADIUS)))
    w.add_geom(M.static_plane(friction=0.5))
    w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, link=0, size=(RADIUS, 0.0, 0.0), friction=0.5))
    q = np.array([0.0, 0.0, RADIUS + 0.01, 1.0, 0.0, 0.0, 0.0], np.float32)
    return w, q, np.zeros(6, np.float32)


RESTING = A.sensors((A.SENSOR_TOUCH, 1, 1), (A.SENSOR_ACCELEROMETER, 1, 0), (A.SENSOR_FORCE, 1, 0),
                    (A.SENSOR_TORQUE, 1, 0))


def settle(P, q, v, n, precision):
    qo, vo = oracle_py.run(P, np.zeros(1, np.int32), q, v, None, n, precision=precision)
    return qo.astype(np.float32), vo.astype(np.float32)


@pytest.mark.parametrize("precision", [0, 1])
def test_link_attached_sphere_resting_on_plane_reads_mg(precision):
    w, q, v = resting_sphere_link()
    P = M.PackedModels([w])
    q, v = settle(P, q, v, 799, precision)
    r, _, _ = oracle_py.tree_contact_sensors(P, 0, q, v, RESTING, precision=precision)
    mg = MASS * 9.81
    assert abs(r[0] - mg) < 0.8, r
    assert np.abs(r[1:4] - np.array([0.0, 0.0, 9.81])).max() < 0.8, r
    assert np.abs(r[4:7]).max() < 0.8, r
    assert np.abs(r[7:10]).max() < 0.8, r


def gap_alignment_scene():
    """tree_contacts_solver.rs:366-390: a free-root link at height 0.45,
    friction-free planes at 0.97 (geom 0) and 0 (geom 1), a sphere of radius
    0.5 at the link's +1.0 (geom 2, gap 0.1) and one at its origin (geom 3)."""
    w = M.WorldModel(dt=0.005, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=40)
    w.push_link(M.Link(parent=-1, joint=M.JOINT_FREE, mass=1.0, inertia=M.solid_sphere_inertia(1.0, 0.5)))
    upper, lower = 1, 2  # collision groups: each plane meets its own sphere only
    w.add_geom(M.Geom(shape=M.SHAPE_PLANE, local_pos=(0.0, 0.0, 0.97), friction=0.0, group=upper, mask=upper))
    w.add_geom(M.Geom(shape=M.SHAPE_PLANE, friction=0.0, group=lower, mask=lower))
    w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, link=0, size=(0.5, 0.0, 0.0), local_pos=(0.0, 0.0, 1.0), friction=0.0,
                      gap=0.1, group=upper, mask=upper))
    w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, link=0, size=(0.5, 0.0, 0.0), friction=0.0, group=lower, mask=lower))
    return w, np.array([0.0, 0.0, 0.45, 1.0, 0.0, 0.0, 0.0], np.float32), np.zeros(6, np.float32)


GAP = A.sensors((A.SENSOR_TOUCH, 1, 3), (A.SENSOR_TOUCH, 1, 2))


@pytest.mark.parametrize("precision", [0, 1])
def test_touch_keeps_force_free_gap_contact_alignment(precision):
    w, q, v = gap_alignment_scene()
    r, _, _ = oracle_py.tree_contact_sensors(M.PackedModels([w]), 0, q, v, GAP, precision=precision)
    assert r[0] > 1.0, r
    assert r[1] == 0.0, r


def gap_alignment_pair_list_scene():
    """tree_contacts_solver.rs:366-390 as newt states it: no filters, the two
    pairs (upper plane, upper sphere) and (lower plane, lower sphere) given
    as the world's explicit pair list (world.rs:136-139)."""
    w, q, v = gap_alignment_scene()
    for g in w.geoms:
        g.group = g.mask = 0xFFFFFFFF
    w.pair_list = [(0, 2), (1, 3)]
    return w, q, v


@pytest.mark.parametrize("precision", [0, 1])
def test_touch_alignment_with_newts_pair_list(precision):
    w, q, v = gap_alignment_pair_list_scene()
    r, _, _ = oracle_py.tree_contact_sensors(M.PackedModels([w]), 0, q, v, GAP, precision=precision)
    assert r[0] > 1.0 and r[1] == 0.0, r
