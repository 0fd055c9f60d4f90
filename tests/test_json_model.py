"""newt's packaged JSON models through the JSON-subset loader (CPU).

newt/tests/model_load.rs builds the same worlds in code and holds the loaded
ones equal to them (stack.json :194-260, pendulum.json :385-470); the loader
is held to those programmatic builds field by field here.  arm.json
(position actuators) and pile.json (meshes) are outside the GPU subset and
refused.
"""
import json
import os

import numpy as np
import pytest

from test_mjcf import _same_model
from test_oracle_golden import GOLD
from tooling_gb300 import model as M
from tooling_gb300.json_model import JsonUnsupported, load_json


def _path(name):
    return os.path.join(GOLD, name + ".json")


def _stack_programmatic():
    """model_load.rs:202-222: plane (friction 0.6) and three solid boxes of
    half-extent 0.35 dropped at z = 0.5, 1.7, 2.9; the middle one shifted
    0.02 in x, the top one spinning at 0.3 rad/s about body y; World::new
    defaults (penalty contacts, RK4)."""
    w = M.WorldModel(dt=0.005, gravity=(0.0, 0.0, -9.81), solver=0, iterations=20, integrator=M.INTEGRATOR_RK4)
    plane = M.static_plane(friction=0.6)
    plane.group, plane.mask = 0xFFFFFFFF, 0xFFFFFFFF
    w.add_geom(plane)
    h = (0.35, 0.35, 0.35)
    qpos, qvel = [], []
    for mass, pos, om in ((1.2, (0.0, 0.0, 0.5), (0.0, 0.0, 0.0)), (0.9, (0.02, 0.0, 1.7), (0.0, 0.0, 0.0)),
                          (1.5, (0.0, 0.0, 2.9), (0.0, 0.3, 0.0))):
        b = w.add_body(mass, M.solid_box_inertia(mass, h))
        g = M.Geom(shape=M.SHAPE_BOX, body=b, size=h, friction=0.6)
        g.group, g.mask = 0xFFFFFFFF, 0xFFFFFFFF
        w.add_geom(g)
        qpos += list(pos) + [1.0, 0.0, 0.0, 0.0]
        qvel += [0.0, 0.0, 0.0] + list(om)
    return w, np.array(qpos, np.float32), np.array(qvel, np.float32)


def _pendulum_programmatic():
    """model_load.rs:385-418."""
    w = M.WorldModel(dt=0.005, gravity=(0.0, 0.0, -9.81), solver=0, iterations=20, integrator=M.INTEGRATOR_RK4)
    w.push_link(M.Link(parent=-1, joint=M.JOINT_FIXED, jp_pos=(0.0, 0.0, 1.5), mass=1.0,
                       inertia=M._diag9(1.0, 1.0, 1.0)))
    w.push_link(M.Link(parent=0, joint=M.JOINT_HINGE, axis=(1.0, 0.0, 0.0), jc_pos=(0.0, 0.0, 0.45), mass=1.3,
                       inertia=M._diag9(0.08775, 0.08775, 1e-6)))
    w.push_link(M.Link(parent=1, joint=M.JOINT_HINGE, axis=(1.0, 0.0, 0.0), jp_pos=(0.0, 0.0, -0.45),
                       jc_pos=(0.0, 0.0, 0.3), mass=0.7, inertia=M._diag9(0.021, 0.021, 1e-6)))
    return w


def test_stack_json_matches_programmatic_build():
    s = load_json(_path("stack"))
    w, q, v = _stack_programmatic()
    _same_model(s.model, w)
    assert s.model.integrator == M.INTEGRATOR_RK4 and s.model.solver == 0
    np.testing.assert_array_equal(s.qpos0, q)
    np.testing.assert_array_equal(s.qvel0, v)
    assert s.body_names == ["bottom", "middle", "top"]


def test_pendulum_json_matches_programmatic_build():
    s = load_json(_path("pendulum"))
    _same_model(s.model, _pendulum_programmatic())
    assert s.link_names == ["pivot", "upper", "lower"] and s.site_names == ["tip"]
    assert s.qpos0.tolist() == [0.0, 0.0] and s.qvel0.tolist() == [0.0, 0.0]


@pytest.mark.parametrize("name", ["arm", "pile"])
def test_models_outside_the_subset_are_refused(name):
    with pytest.raises(JsonUnsupported):
        load_json(_path(name))


def test_options_reach_the_model():
    s = load_json('{"integrator": "Euler", "solver": {"mode": "pgs", "iterations": 30}, "timestep": 0.002}')
    assert (s.model.integrator, s.model.solver, s.model.iterations) == (M.INTEGRATOR_EULER, M.SOLVER_PGS, 30)
    assert s.model.dt == pytest.approx(0.002)
    with pytest.raises(JsonUnsupported):
        load_json('{"integrator": "implicitfast"}')
    with pytest.raises(JsonUnsupported):
        load_json('{"solver": {"mode": "pgs", "cone": "conical"}}')


def test_cone_and_explicit_contact_pairs_are_read():
    """model.rs:1557-1597 (solver.cone) and 1033-1041, 3208-3250
    (contact_pairs.explicit, each pair stored as (min, max) in list order)."""
    with open(os.path.join(GOLD, "stack.json")) as f:
        root = json.load(f)
    root["solver"] = {"mode": "pgs", "iterations": 30, "cone": "elliptic"}
    root["contact_pairs"] = {"explicit": [{"a": "middle_box", "b": "ground"}, {"a": "bottom_box", "b": "top_box"}]}
    w = load_json(json.dumps(root)).model
    assert w.cone == M.CONE_ELLIPTIC
    assert w.pair_list == [(0, 2), (1, 3)]
    root["contact_pairs"] = {"disable": [{"a": "middle_box", "b": "ground"}]}
    with pytest.raises(JsonUnsupported):
        load_json(json.dumps(root))
