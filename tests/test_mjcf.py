"""newt's reference MJCF scenes through the MJCF-subset loader (CPU).

The loader must build the same worlds newt's MJCF loader builds: the scenes
are checked field by field against the hand-restated ones the golden tests
use, then stepped by the FP64 oracle from the MuJoCo captures' first frames
and held to newt's matched-Euler windows (newt/tests/differential.rs)."""
import os

import numpy as np
import pytest

import oracle_py
from test_oracle_golden import (GOLD, _double_pendulum, _free_body_scene, _tree_chain_contact, read_newtdif)
from tooling_gb300 import model as M
from tooling_gb300.mjcf import MjcfUnsupported, load_mjcf


def _xml(name):
    return os.path.join(GOLD, name + ".xml")


def _same_model(a: M.WorldModel, b: M.WorldModel):
    assert a.dt == pytest.approx(b.dt) and tuple(a.gravity) == pytest.approx(tuple(b.gravity))
    assert a.solver == b.solver and a.iterations == b.iterations
    assert a.tree_self_collision == b.tree_self_collision
    assert len(a.links) == len(b.links) and len(a.bodies) == len(b.bodies) and len(a.geoms) == len(b.geoms)
    f32 = lambda v: np.asarray(v, np.float32)  # noqa: E731  (the descriptors are f32)
    for la, lb in zip(a.links, b.links):
        assert (la.parent, la.joint) == (lb.parent, lb.joint)
        for k in ("axis", "jp_pos", "jp_quat", "jc_pos", "jc_quat", "inertia"):
            np.testing.assert_array_equal(f32(getattr(la, k)), f32(getattr(lb, k)), err_msg=k)
        assert np.float32(la.mass) == np.float32(lb.mass)
        assert np.float32(la.damping) == np.float32(lb.damping)
    for (ma, ia), (mb, ib) in zip(a.bodies, b.bodies):
        assert np.float32(ma) == np.float32(mb)
        np.testing.assert_array_equal(f32(ia), f32(ib))
    for ga, gb in zip(a.geoms, b.geoms):
        assert (ga.shape, ga.body, ga.link, ga.condim) == (gb.shape, gb.body, gb.link, gb.condim)
        for k in ("size", "local_pos", "local_quat", "solref", "solimp"):
            np.testing.assert_array_equal(f32(getattr(ga, k)), f32(getattr(gb, k)), err_msg=k)
        assert np.float32(ga.friction) == np.float32(gb.friction)
        assert (ga.margin, ga.gap) == (gb.margin, gb.gap)
    # contype / conaffinity 1 (MJCF) and all-ones filters collide the same pairs
    pairs = lambda w: [(i, j) for i in range(len(w.geoms)) for j in range(i + 1, len(w.geoms))  # noqa: E731
                       if w.geoms[i].group & w.geoms[j].mask and w.geoms[j].group & w.geoms[i].mask]
    assert pairs(a) == pairs(b)


@pytest.mark.parametrize("name", ["ballistic", "sphere_drop", "box_stack"])
def test_free_body_scenes_load_like_newt(name):
    s = load_mjcf(_xml(name))
    w, q0, _ = _free_body_scene(name)
    if name == "ballistic":  # no geoms: the hand scene has none either
        assert not s.model.geoms
    _same_model(s.model, w)
    np.testing.assert_allclose(s.qpos0, np.asarray(q0, np.float32), atol=0)
    assert s.integrator == "RK4"  # the XMLs keep MuJoCo's RK4; newt's matched rows switch to Euler


def test_double_pendulum_loads_like_newt():
    s = load_mjcf(_xml("double_pendulum"))
    _same_model(s.model, _double_pendulum())
    assert s.qpos0.size == 2 and not s.qpos0.any()


def test_tree_chain_contact_loads_like_newt():
    s = load_mjcf(_xml("tree_chain_contact"))
    _same_model(s.model, _tree_chain_contact(M.SOLVER_NEWTON))
    assert s.integrator == "Euler"
    np.testing.assert_allclose(s.qpos0[:3], [0.0, 0.0, 1.35])


def test_defaults_reach_geoms():
    stiff, soft = load_mjcf(_xml("sphere_drop_stiff")), load_mjcf(_xml("sphere_drop_soft"))
    for s, tc in ((stiff, 0.010), (soft, 0.050)):
        assert [g.solref[0] for g in s.model.geoms] == pytest.approx([tc, tc])


@pytest.mark.parametrize("name,qtol,vtol", [("ballistic", 3.0e-5, 8.0e-5), ("sphere_drop", 1.5e-2, 9.0e-1),
                                             ("box_stack", 2.0e-2, 5.0e-1), ("double_pendulum", 4.0e-7, 1.0e-6)])
def test_loaded_scenes_within_mujoco_windows(name, qtol, vtol):
    """The matched-Euler rows (differential.rs:1272-1295) from the loaded
    scenes, initial state from the capture's first frame."""
    s = load_mjcf(_xml(name))
    ref = read_newtdif(f"{name}_euler.bin")
    packed = M.PackedModels([s.model])
    q0 = ref["qpos"][0].astype(np.float32)
    v0 = ref["qvel"][0].astype(np.float32)
    worst_q = worst_v = 0.0
    for k, step in enumerate(ref["steps"]):
        qo, vo = oracle_py.run(packed, np.zeros(1, np.int32), q0, v0, None, step, precision=1)
        worst_q = max(worst_q, np.abs(qo - ref["qpos"][k]).max())
        worst_v = max(worst_v, np.abs(vo - ref["qvel"][k]).max())
    assert worst_q <= qtol and worst_v <= vtol, (worst_q, worst_v)


def test_integrator_option_reaches_the_model():
    """mjcf.rs:727-742: RK4 (also when no option is given) or Euler; the
    GPU path has no implicitfast."""
    base = '<mujoco><compiler angle="radian"/>{}<worldbody/></mujoco>'
    assert load_mjcf(base.format("")).model.integrator == M.INTEGRATOR_RK4
    assert load_mjcf(base.format('<option integrator="RK4"/>')).model.integrator == M.INTEGRATOR_RK4
    assert load_mjcf(base.format('<option integrator="Euler"/>')).model.integrator == M.INTEGRATOR_EULER
    with pytest.raises(MjcfUnsupported):
        load_mjcf(base.format('<option integrator="implicitfast"/>'))


def test_outside_the_subset_is_refused():
    with pytest.raises(MjcfUnsupported):
        load_mjcf('<mujoco><compiler angle="radian"/><worldbody><body name="b"><freejoint/>'
                  '<inertial mass="1" diaginertia="1 1 1"/><geom type="cylinder" size="0.1 0.2"/></body>'
                  '</worldbody></mujoco>')
    with pytest.raises(MjcfUnsupported):  # MuJoCo's default angle unit (degrees) is not taken
        load_mjcf('<mujoco><worldbody/></mujoco>')
