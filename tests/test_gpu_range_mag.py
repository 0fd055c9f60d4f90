"""Rangefinder and magnetometer on the GPU (write_sensors' ray casts over the
world's geoms, sensors.cu) against the oracle, which holds newt's anchors
(tests/test_oracle_range_mag.py).

The GPU's pile worlds give every body one geom, so the anchors' probe body
carries a sphere of radius 0.05 and the site sits 0.1 above its centre: each
reading is newt's expected value less 0.1 (within 1e-5, as newt's bar), and
-1 where nothing lies ahead.  On settled piles and on quadrupeds (a
tree-contact world: the torso box, leg capsules and the plane), rangefinders
at random site frames and magnetometers read no further from the FP64
oracle than twice newt's own f32 arithmetic or 1e-4 of the reading (floor
1)."""
import numpy as np
import pytest

import oracle_py
from f32util import quat_from_axis_angle
from test_oracle_range_mag import ANCHORS, probe_world
from tooling_gb300 import Engine, scenes
from tooling_gb300 import api as A
from tooling_gb300 import model as M

pytestmark = pytest.mark.gpu
UP = (0.0, 0.0, 0.1)


@pytest.fixture(scope="module")
def eng():
    from tooling_gb300 import build as B
    B.build()
    e = Engine(device=0)
    yield e
    e.close()


def _read(eng, P, q, v, sens):
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q, v)
    got = eng.read_sensors(slots, sens)
    eng.free(slots)
    return got


def _with_probe_geom(w):
    w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, body=0, size=(0.05, 0.0, 0.0), friction=0.0))
    return w


@pytest.mark.parametrize("kind,expected", ANCHORS + [(None, -1.0)])
def test_rangefinder_anchors_on_gpu(eng, kind, expected):
    w, q, v = probe_world(kind)
    P = M.PackedModels([_with_probe_geom(w)])
    s = A.sensors((A.SENSOR_RANGEFINDER, 0, 0, UP))
    got = _read(eng, P, q, v, s)[0]
    want = expected - 0.1 if expected > 0 else -1.0
    assert abs(got[0] - want) < 1e-5, (kind, got, want)
    assert abs(got[0] - oracle_py.sensors(P, 0, q, v, s)[0]) < 1e-5


def test_site_frame_anchor_on_gpu(eng):
    w = M.WorldModel(magnetic_field=(0.0, -0.5, 0.0))
    w.add_body(1.0, M._diag9(1.0, 1.0, 1.0))
    w.add_geom(M.static_plane(friction=0.0))
    _with_probe_geom(w)
    x, y, z, ww = quat_from_axis_angle((0.0, 0.0, 1.0), np.pi / 2)
    P = M.PackedModels([w])
    v = np.zeros(6, np.float32)
    s = A.sensors((A.SENSOR_RANGEFINDER, 0, 0, UP), (A.SENSOR_MAGNETOMETER, 0, 0))
    got = _read(eng, P, np.array([0.0, 0.0, -1.0, 1.0, 0.0, 0.0, 0.0], np.float32), v, s)[0]
    assert abs(got[0] - 0.9) < 1e-5 and np.array_equal(got[1:], [0.0, -0.5, 0.0]), got
    got = _read(eng, P, np.array([0.0, 0.0, -1.0, ww, x, y, z], np.float32), v, s)[0]
    assert np.abs(got[1:] - np.array([-0.5, 0.0, 0.0])).max() < 1e-6, got


def _random_sites(rng, n, on_link, index_hi):
    items = []
    for _ in range(n):
        quat = quat_from_axis_angle(tuple(rng.normal(size=3)), float(rng.uniform(0.0, np.pi)))
        pos = tuple(rng.uniform(-0.1, 0.1, 3))
        idx = int(rng.integers(0, index_hi))
        items.append((A.SENSOR_RANGEFINDER, on_link, idx, pos, quat))
        items.append((A.SENSOR_MAGNETOMETER, on_link, idx, pos, quat))
    return A.sensors(*items)


def _against_fp64(got, b, w, q, v, sens):
    r64 = oracle_py.sensors(b, w, q, v, sens, precision=1)
    r32 = oracle_py.sensors(b, w, q, v, sens, precision=0)
    gpu, newt = np.abs(got - r64), np.abs(r32 - r64)
    assert (gpu <= np.maximum(1e-4 * np.maximum(1.0, np.abs(r64)), 2.0 * newt)).all(), (w, got, r64, r32)
    return int((r64[::4] >= 0).sum())


@pytest.mark.parametrize("which", ["pile", "quadruped"])
def test_random_sites_match_fp64(eng, which):
    rng = np.random.default_rng(41)
    if which == "pile":
        b = scenes.pile_batch(n_worlds=12, first_world=3300)
        rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, None, 200, precision=1)
        on_link, hi = 0, 16
    else:
        b = scenes.quadruped_batch(n_worlds=12, first_world=3300)
        rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, None, 100, precision=1)
        on_link, hi = 1, 13
    b.qpos[:] = rq.astype(np.float32)
    b.qvel[:] = rv.astype(np.float32)
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, b.qpos, b.qvel)
    hits = 0
    for _ in range(2):
        sens = _random_sites(rng, 8, on_link, hi)
        got = eng.read_sensors(slots, sens)
        for w in range(len(b)):
            q, v = b.qpos[b.q_off[w]:b.q_off[w] + b.nq[w]], b.qvel[b.v_off[w]:b.v_off[w] + b.nv[w]]
            hits += _against_fp64(got[w], b, w, q, v, sens)
    eng.free(slots)
    assert hits > 0
