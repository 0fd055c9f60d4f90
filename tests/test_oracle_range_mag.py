"""The oracle's rangefinder and magnetometer (newt/src/sensor.rs:664-682,
759-791; scene_query.rs:182-438) against newt's anchors (CPU).

apis.rs:97-130: a body at z = -1 under a plane at z = 0, the site at the
body's origin: the rangefinder reads 1 within 1e-6 and the magnetometer the
world field (0, -0.5, 0).  apis.rs:320-420: a probe body at the origin and a
target at z = 2 (a plane at z = 2, or a sphere, box, capsule, cylinder or
ellipsoid of size 0.5 on the target): the rangefinder reads 2, 1.5, 1.5, 1,
1.5, 1.5 within 1e-5, and -1 in a world without geoms.  Beyond newt's
anchors: a body turned a quarter turn about z reads the field rotated into
its frame, and a site inside a geom reads the distance to that geom's far
side (newt's ray test takes the far root for a ray that starts inside)."""
import numpy as np
import pytest

import oracle_py
from f32util import quat_from_axis_angle
from tooling_gb300 import api as A
from tooling_gb300 import model as M


def probe_world(kind=None):
    w = M.WorldModel()
    w.add_body(1.0, M._diag9(1.0, 1.0, 1.0))  # the probe, at the origin
    if kind == "plane":
        w.add_geom(M.Geom(shape=M.SHAPE_PLANE, local_pos=(0.0, 0.0, 2.0), friction=0.0))
    elif kind is not None:
        t = w.add_body(1.0, M._diag9(1.0, 1.0, 1.0))
        shape, size = {"sphere": (M.SHAPE_SPHERE, (0.5, 0.0, 0.0)), "box": (M.SHAPE_BOX, (0.5, 0.5, 0.5)),
                       "capsule": (M.SHAPE_CAPSULE, (0.5, 0.5, 0.0)), "cylinder": (M.SHAPE_CYLINDER, (0.5, 0.5, 0.0)),
                       "ellipsoid": (M.SHAPE_ELLIPSOID, (0.5, 0.5, 0.5))}[kind]
        w.add_geom(M.Geom(shape=shape, body=t, size=size, friction=0.0))
    nb = len(w.bodies)
    q = np.zeros(7 * nb, np.float32)
    q[3::7] = 1.0
    if nb > 1:
        q[7 + 2] = 2.0
    return w, q, np.zeros(6 * nb, np.float32)


ANCHORS = [("plane", 2.0), ("sphere", 1.5), ("box", 1.5), ("capsule", 1.0), ("cylinder", 1.5), ("ellipsoid", 1.5)]


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("kind,expected", ANCHORS)
def test_rangefinder_hits_each_shape(kind, expected, precision):
    w, q, v = probe_world(kind)
    r = oracle_py.sensors(M.PackedModels([w]), 0, q, v, A.sensors((A.SENSOR_RANGEFINDER, 0, 0)), precision=precision)
    assert abs(r[0] - expected) < 1e-5, (kind, r)


def test_rangefinder_without_geoms_reads_minus_one():
    w, q, v = probe_world(None)
    r = oracle_py.sensors(M.PackedModels([w]), 0, q, v, A.sensors((A.SENSOR_RANGEFINDER, 0, 0)))
    assert r[0] == -1.0


@pytest.mark.parametrize("precision", [0, 1])
def test_rangefinder_and_magnetometer_use_site_frame(precision):
    w = M.WorldModel(magnetic_field=(0.0, -0.5, 0.0))
    w.add_body(1.0, M._diag9(1.0, 1.0, 1.0))
    w.add_geom(M.static_plane(friction=0.0))
    q = np.array([0.0, 0.0, -1.0, 1.0, 0.0, 0.0, 0.0], np.float32)
    s = A.sensors((A.SENSOR_RANGEFINDER, 0, 0), (A.SENSOR_MAGNETOMETER, 0, 0))
    r = oracle_py.sensors(M.PackedModels([w]), 0, q, np.zeros(6, np.float32), s, precision=precision)
    assert abs(r[0] - 1.0) < 1e-6, r
    assert np.array_equal(r[1:], [0.0, -0.5, 0.0]), r


def test_magnetometer_turns_with_the_site_and_rangefinder_far_side():
    w = M.WorldModel(magnetic_field=(0.0, -0.5, 0.0))
    b = w.add_body(1.0, M.solid_sphere_inertia(1.0, 0.1))
    w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, body=b, size=(0.1, 0.0, 0.0)))
    x, y, z, ww = quat_from_axis_angle((0.0, 0.0, 1.0), np.pi / 2)
    q = np.array([0.0, 0.0, 1.0, ww, x, y, z], np.float32)
    s = A.sensors((A.SENSOR_MAGNETOMETER, 0, 0), (A.SENSOR_RANGEFINDER, 0, 0, (0.0, 0.0, 0.03)))
    r = oracle_py.sensors(M.PackedModels([w]), 0, q, np.zeros(6, np.float32), s)
    assert np.abs(r[:3] - np.array([-0.5, 0.0, 0.0])).max() < 1e-6, r
    assert abs(r[3] - 0.07) < 1e-6, r
