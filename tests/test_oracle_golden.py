"""Pins the oracle to newt's own golden vectors (CPU only).

The f32 mirror must reproduce newt's byte goldens exactly; the FP64 oracle
must stay inside the windows newt's differential tests allow against MuJoCo.
"""
import os

import numpy as np
import pytest

import oracle_py
from f32util import f32, quat_from_axis_angle
from tooling_gb300 import model as M

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _read_f32(name):
    return np.fromfile(os.path.join(GOLD, name), dtype="<f4")


def _integrator_scene():
    # newt/tests/integrators_golden.rs:10-25
    w = M.WorldModel(dt=0.005, gravity=(0.0, 0.0, -9.81), solver=0)
    w.add_body(1.25, M._diag9(0.7, 1.3, 2.1))
    q = quat_from_axis_angle((1.0, 0.2, -0.4), 0.6)
    qpos = np.array([0.4, -0.7, 2.0] + q, dtype=np.float32)
    qvel = np.array([0.8, -0.4, 1.2, 0.4, 1.1, -0.3], dtype=np.float32)
    return w, qpos, qvel


def test_integrator_euler_golden_is_byte_identical():
    """newt/tests/integrators_golden.rs:84-91 (Euler)."""
    w, qpos, qvel = _integrator_scene()
    packed = M.PackedModels([w])
    gold = _read_f32("integrator_euler.bin").reshape(3, 13)
    got = [np.concatenate([qpos, qvel])]
    for n in (20, 100):
        qo, vo = oracle_py.run(packed, np.zeros(1, np.int32), qpos, qvel, None, n, precision=0, layout=1)
        got.append(np.concatenate([qo, vo]).astype(np.float32))
    got = np.stack(got)
    assert got.tobytes() == gold.tobytes(), np.abs(got - gold).max()


def test_integrator_rk4_golden_is_byte_identical():
    """newt/tests/integrators_golden.rs:84-91 (RK4, newt's default): the
    free-body RK4 of world.rs:1705-1788 with no contacts."""
    w, qpos, qvel = _integrator_scene()
    packed = M.PackedModels([w])
    gold = _read_f32("integrator_rk4.bin").reshape(3, 13)
    got = [np.concatenate([qpos, qvel])]
    for n in (20, 100):
        qo, vo = oracle_py.run(packed, np.zeros(1, np.int32), qpos, qvel, None, n, precision=0, layout=1, integrator=0)
        got.append(np.concatenate([qo, vo]).astype(np.float32))
    got = np.stack(got)
    assert got.tobytes() == gold.tobytes(), np.abs(got - gold).max()


def _solver_box_scene(name, solver=M.SOLVER_PGS):
    """newt/tests/solver_golden.rs:27-91: the stack (three unit boxes with
    1 cm x offsets) and the incline (one asymmetric box under tilted gravity),
    World::new() defaults (RK4, pyramidal cone), solref (0.05, 1.5) on every
    geom, PGS or (newton_stack_scene, newton_incline_scene) Newton.  Returns
    (model, qpos, qvel) in newt's layout."""
    sr = (0.05, 1.5)
    if name == "stack":
        w = M.WorldModel(dt=0.005, gravity=(0.0, 0.0, -9.81), solver=solver, iterations=30)
        fric, halves = 0.8, [(0.25, 0.25, 0.25)] * 3
        poses = [(f32(0.01) * f32(k), 0.0, f32(0.25) + f32(0.5) * f32(k)) for k in range(3)]
    else:
        L = oracle_py.lib()
        ang = f32(f32(32.0) * f32(np.pi)) / f32(180.0)
        g = f32(9.81)
        gz = -(g * f32(L.oracle_newt_cos(float(ang))))
        w = M.WorldModel(dt=0.005, gravity=(float(g * f32(L.oracle_newt_sin(float(ang)))), 0.0, float(gz)),
                         solver=solver, iterations=30)
        fric, halves, poses = 0.5, [(0.2, 0.21, 0.19)], [(0.01, 0.0, 0.2)]
    plane = M.static_plane(friction=fric)
    plane.solref = sr
    w.add_geom(plane)
    qpos, qvel = [], []
    for h, p in zip(halves, poses):
        b = w.add_body(1.0, M.solid_box_inertia(1.0, h))
        w.add_geom(M.Geom(shape=M.SHAPE_BOX, body=b, size=h, friction=fric, solref=sr))
        qpos += [float(x) for x in p] + [0.0, 0.0, 0.0, 1.0]
        qvel += [0.0] * 6
    return w, np.array(qpos, np.float32), np.array(qvel, np.float32)


@pytest.mark.parametrize("solver,file", [(M.SOLVER_PGS, ""), (M.SOLVER_NEWTON, "newton_")])
@pytest.mark.parametrize("name", ["stack", "incline"])
def test_solver_rk4_zoh_goldens_are_byte_identical(name, solver, file):
    """newt/tests/solver_golden.rs:164-258: free-body PGS, or the dense
    free-body Newton solve, solved once per step and held over the RK4
    stages, snapshots after 0, 50, 200 and 1000 steps."""
    w, qpos, qvel = _solver_box_scene(name, solver)
    nb = len(w.bodies)
    gold = _read_f32(f"solver_{file}{name}.bin").reshape(4, nb, 13)
    got = [np.concatenate([qpos.reshape(nb, 7), qvel.reshape(nb, 6)], axis=1)]
    packed = M.PackedModels([w])
    for n in (50, 200, 1000):
        qo, vo = oracle_py.run(packed, np.zeros(1, np.int32), qpos, qvel, None, n, precision=0, layout=1, integrator=0)
        got.append(np.concatenate([qo.reshape(nb, 7), vo.reshape(nb, 6)], axis=1).astype(np.float32))
    got = np.stack(got)
    assert got.tobytes() == gold.tobytes(), np.abs(got - gold).max(axis=(1, 2))


def _renormalize(q):
    n = np.sqrt(f32(f32(f32(q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3]))
    return [x / n for x in q]


def _box_inertia(mass, hx, hy, hz):
    m3 = f32(mass) / f32(3.0)
    hx2, hy2, hz2 = f32(hx) * f32(hx), f32(hy) * f32(hy), f32(hz) * f32(hz)
    return M._diag9(m3 * (hy2 + hz2), m3 * (hx2 + hz2), m3 * (hx2 + hy2))


def _mixed_tree():
    """newt/tests/dynamics_golden.rs:28-89."""
    from f32util import normalize
    w = M.WorldModel()
    w.push_link(M.Link(parent=-1, joint=M.JOINT_FIXED, mass=1.0, inertia=M._diag9(1.0, 1.0, 1.0)))
    w.push_link(M.Link(parent=0, joint=M.JOINT_HINGE, axis=normalize((1.0, 0.3, -0.2)), armature=0.02,
                       jp_pos=(0.05, 0.0, -0.1), jc_pos=(-0.15, 0.0, 0.3), mass=0.9,
                       inertia=_box_inertia(0.9, 0.15, 0.1, 0.3)))
    w.push_link(M.Link(parent=1, joint=M.JOINT_SLIDE, axis=normalize((0.2, 1.0, 0.4)), armature=0.05,
                       jp_pos=(0.0, 0.0, -0.3), jc_pos=(0.1, -0.2, 0.15), mass=0.7,
                       inertia=_box_inertia(0.7, 0.1, 0.2, 0.15)))
    w.push_link(M.Link(parent=2, joint=M.JOINT_BALL, armature=0.01, jp_pos=(0.1, -0.2, -0.15),
                       jc_pos=(-0.05, 0.1, 0.2), mass=0.5, inertia=M._diag9(0.02, 0.03, 0.04)))
    ball = _renormalize(quat_from_axis_angle(normalize((0.4, 1.0, -0.3)), 0.55))
    q_native = np.array([0.35, 0.12] + ball, dtype=np.float32)
    return w, q_native


def test_mass_matrix_golden_is_byte_identical():
    """CRB mass matrix part of newt/tests/goldens/dynamics_mass_bias.bin."""
    w, q = _mixed_tree()
    packed = M.PackedModels([w])
    got = oracle_py.mass_matrix(packed, 0, q, 5, precision=0).astype(np.float32)
    gold = _read_f32("dynamics_mass_bias.bin")[:25].reshape(5, 5)
    assert got.tobytes() == gold.tobytes(), np.abs(got - gold).max()


def read_newtdif(name):
    """NEWTDIF1 reader (newt/tests/differential.rs:239-301)."""
    import struct
    d = open(os.path.join(GOLD, name), "rb").read()
    assert d[:8] == b"NEWTDIF1"
    n = struct.unpack("<I", d[8:12])[0]
    o = 12 + n
    nq, nv, stride, ns, nsteps = struct.unpack("<5I", d[o:o + 20])
    o += 20
    steps, qpos, qvel = [], [], []
    for _ in range(ns):
        steps.append(struct.unpack("<I", d[o:o + 4])[0]); o += 4
        qpos.append(np.frombuffer(d, "<f8", nq, o)); o += 8 * nq
        qvel.append(np.frombuffer(d, "<f8", nv, o)); o += 8 * nv
    return dict(stride=stride, n_steps=nsteps, steps=steps, qpos=np.array(qpos), qvel=np.array(qvel))


def _double_pendulum():
    """tests/references/double_pendulum.xml as newt's MJCF loader builds it
    (newt/src/mjcf.rs:1079-1110 root, :1258-1262 joint offsets)."""
    w = M.WorldModel(dt=0.002, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=20)
    w.push_link(M.Link(parent=-1, joint=M.JOINT_FIXED, jp_pos=(0.0, 0.0, 1.5), mass=1.0,
                       inertia=M._diag9(1.0, 1.0, 1.0)))
    w.push_link(M.Link(parent=0, joint=M.JOINT_HINGE, axis=(1.0, 0.0, 0.0),
                       jp_pos=(0.0, 0.0, float(f32(-0.45) + f32(0.45))), jc_pos=(0.0, 0.0, 0.45), mass=1.3,
                       inertia=M._diag9(0.08775, 0.08775, 1e-6)))
    w.push_link(M.Link(parent=1, joint=M.JOINT_HINGE, axis=(1.0, 0.0, 0.0),
                       jp_pos=(0.0, 0.0, float(f32(-0.75) + f32(0.3))), jc_pos=(0.0, 0.0, 0.3), mass=0.7,
                       inertia=M._diag9(0.021, 0.021, 1e-6)))
    return w


@pytest.mark.parametrize("precision,qtol,vtol", [(0, 4.0e-7, 1.0e-6), (1, 4.0e-7, 1.0e-6)])
def test_double_pendulum_euler_matches_mujoco_capture(precision, qtol, vtol):
    """Matched-Euler row of newt/tests/differential.rs:1594-1599 (window :1281-1284)."""
    ref = read_newtdif("double_pendulum_euler.bin")
    packed = M.PackedModels([_double_pendulum()])
    qpos = np.array([0.35, -0.15], np.float32)
    qvel = np.zeros(2, np.float32)
    worst_q = worst_v = 0.0
    for k, step in enumerate(ref["steps"]):
        qo, vo = oracle_py.run(packed, np.zeros(1, np.int32), qpos, qvel, None, step, precision=precision)
        worst_q = max(worst_q, np.abs(qo - ref["qpos"][k]).max())
        worst_v = max(worst_v, np.abs(vo - ref["qvel"][k]).max())
    assert worst_q <= qtol and worst_v <= vtol, (worst_q, worst_v)


def _tree_contact_scene(solver):
    """newt/tests/solver_golden.rs:93-144: a free-root tree with one hinge
    child, a box on each link, resting on a plane (newt's default RK4)."""
    w = M.WorldModel(dt=0.005, gravity=(0.0, 0.0, -9.81), solver=solver, iterations=30,
                     tree_self_collision=1)  # newt collides in-tree pairs by default (world.rs:340)
    plane = M.static_plane(friction=0.7)
    plane.solref = (0.05, 1.5)
    w.add_geom(plane)
    gold = _read_f32("solver_tree.bin").reshape(4, 15)
    root_q = [float(x) for x in gold[0, 3:7]]  # Quat::from_axis_angle(normalize(1, 0.4, -0.2), 0.35)
    w.push_link(M.Link(parent=-1, joint=M.JOINT_FREE, jp_pos=(0.13, -0.07, 0.78), jp_quat=root_q, mass=1.2,
                       inertia=M._diag9(0.08, 0.09, 0.1)))
    w.push_link(M.Link(parent=0, joint=M.JOINT_HINGE, axis=(0.0, 1.0, 0.0), jp_pos=(0.0, 0.0, -0.3),
                       jc_pos=(0.0, 0.0, 0.22), mass=0.75, inertia=M._diag9(0.02, 0.025, 0.018)))
    w.add_geom(M.Geom(shape=M.SHAPE_BOX, link=0, size=(0.22, 0.17, 0.19), local_pos=(0.08, -0.06, 0.0),
                      local_quat=quat_from_axis_angle((0.0, 1.0, 0.0), 0.2), friction=0.7))
    w.add_geom(M.Geom(shape=M.SHAPE_BOX, link=1, size=(0.14, 0.12, 0.24), local_pos=(0.0, 0.0, -0.18),
                      local_quat=quat_from_axis_angle((1.0, 0.0, 0.0), -0.15), friction=0.7))
    q0 = np.concatenate([gold[0, :7], [0.37]]).astype(np.float32)
    v0 = np.array([0, 0, 0, 0, 0, 0, -0.25], np.float32)
    return w, q0, v0


@pytest.mark.parametrize("solver,name", [(M.SOLVER_PGS, "solver_tree.bin"), (M.SOLVER_NEWTON, "solver_newton_tree.bin")])
def test_tree_contact_solver_golden_is_byte_identical(solver, name):
    """newt/tests/solver_golden.rs:260-297: q and qdot after 0, 50, 200 and
    1000 RK4 steps with the joint tree-contact solve held over each step."""
    w, q0, v0 = _tree_contact_scene(solver)
    packed = M.PackedModels([w])
    gold = _read_f32(name).reshape(4, 15)
    assert np.concatenate([q0, v0]).tobytes() == gold[0].tobytes()
    got = [np.concatenate([q0, v0])]
    for n in (50, 200, 1000):
        qo, vo = oracle_py.run(packed, np.zeros(1, np.int32), q0, v0, None, n, precision=0, layout=1, integrator=0)
        got.append(np.concatenate([qo, vo]).astype(np.float32))
    got = np.stack(got)
    assert got.tobytes() == gold.tobytes(), np.abs(got - gold).max(axis=1)


def _joints_chain():
    """newt/tests/joints_golden.rs:23-60: fixed root and three X hinges."""
    w = M.WorldModel(dt=0.005, gravity=(0.0, 0.0, -9.81), solver=0)
    w.push_link(M.Link(parent=-1, joint=M.JOINT_FIXED, mass=1.0, inertia=M._diag9(1.0, 1.0, 1.0)))
    masses, lengths = [f32(1.1), f32(0.7), f32(1.3)], [f32(0.6), f32(0.4), f32(0.5)]
    for i in range(3):
        m, l = masses[i], lengths[i]
        ip = f32(f32(f32(f32(1.0) / f32(12.0)) * m) * l) * l
        anchor = (0.0, 0.0, 0.0) if i == 0 else (0.0, 0.0, float(-lengths[i - 1] * f32(0.5)))
        w.push_link(M.Link(parent=i, joint=M.JOINT_HINGE, axis=(1.0, 0.0, 0.0), jp_pos=anchor,
                           jc_pos=(0.0, 0.0, float(l * f32(0.5))), mass=float(m),
                           inertia=M._diag9(float(ip), float(ip), 1e-6)))
    return w, np.array([0.4, -0.3, 0.2], np.float32), np.array([0.0, 0.5, 0.0], np.float32)


def _joints_floating(q0):
    """newt/tests/joints_golden.rs:62-103: free box with a swinging arm, no gravity."""
    from f32util import normalize
    w = M.WorldModel(dt=0.005, gravity=(0.0, 0.0, 0.0), solver=0)
    hx, hy, hz, m0 = f32(0.3), f32(0.2), f32(0.15), f32(2.0)
    m3 = m0 / f32(3.0)
    box_i = M._diag9(float(m3 * (hy * hy + hz * hz)), float(m3 * (hx * hx + hz * hz)), float(m3 * (hx * hx + hy * hy)))
    w.push_link(M.Link(parent=-1, joint=M.JOINT_FREE, jp_pos=(0.5, -1.0, 4.5), jp_quat=[float(x) for x in q0],
                       mass=2.0, inertia=box_i))
    l, m1 = f32(0.8), f32(0.7)
    ip = f32(f32(f32(f32(1.0) / f32(12.0)) * m1) * l) * l
    w.push_link(M.Link(parent=0, joint=M.JOINT_HINGE, axis=[float(x) for x in normalize((1.0, 0.3, 0.0))],
                       jp_pos=(0.0, 0.0, float(-hz)), jc_pos=(0.0, 0.0, float(l * f32(0.5))), mass=float(m1),
                       inertia=M._diag9(float(ip), float(ip), 1e-4)))
    return w


def test_joints_chain_and_floating_golden_is_byte_identical():
    """newt/tests/joints_golden.rs:105-170: tree RK4 (explicit ABA) after 0,
    100 and 1000 steps for a hinge chain and a floating base with an arm."""
    gold = _read_f32("joints_chain_and_floating.bin").reshape(3, 21)
    wc, qc, vc = _joints_chain()
    wf = _joints_floating(gold[0, 9:13])  # Quat::from_axis_angle((1, 0.4, -0.3), 0.6)
    qf = gold[0, 6:14].copy()
    vf = np.array([0, 0, 0, 0, 0, 0, 4.0], np.float32)
    assert np.concatenate([qc, vc, qf, vf]).tobytes() == gold[0].tobytes()
    got = [gold[0]]
    for n in (100, 1000):
        row = []
        for w, q, v in ((wc, qc, vc), (wf, qf, vf)):
            qo, vo = oracle_py.run(M.PackedModels([w]), np.zeros(1, np.int32), q, v, None, n, precision=0, layout=1,
                                   integrator=0)
            row += [qo, vo]
        got.append(np.concatenate(row).astype(np.float32))
    got = np.stack(got)
    assert got.tobytes() == gold.tobytes(), np.abs(got - gold).max(axis=1)


def _tree_chain_contact(solver):
    """tests/references/tree_chain_contact.xml as newt's MJCF loader builds
    it: a free root sphere and a hinged sphere below it, falling on a plane
    (Euler, dt 2e-3, 20 solver iterations)."""
    w = M.WorldModel(dt=0.002, gravity=(0.0, 0.0, -9.81), solver=solver, iterations=20)
    w.add_geom(M.static_plane(friction=0.6))
    w.push_link(M.Link(parent=-1, joint=M.JOINT_FREE, jp_pos=(0.0, 0.0, 1.35), mass=1.1,
                       inertia=M._diag9(0.08, 0.09, 0.1)))
    w.push_link(M.Link(parent=0, joint=M.JOINT_HINGE, axis=(0.0, 1.0, 0.0), jp_pos=(0.0, 0.0, -0.25),
                       jc_pos=(0.0, 0.0, 0.25), mass=0.8, inertia=M._diag9(0.025, 0.03, 0.02)))
    w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, link=0, size=(0.24, 0.0, 0.0), friction=0.6))
    w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, link=1, size=(0.19, 0.0, 0.0), friction=0.6))
    return w


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("solver,name,qtol,vtol", [
    (M.SOLVER_NEWTON, "tree_chain_contact_newton_euler.bin", 8.0e-2, 1.3),
    (M.SOLVER_PGS, "tree_chain_contact_pgs_euler.bin", 7.0e-2, 0.7)])
def test_tree_chain_contact_euler_matches_mujoco_capture(precision, solver, name, qtol, vtol):
    """Tree-contact rows of newt/tests/differential.rs:1411-1446 (the Euler
    form of the joint solve), inside newt's own windows against MuJoCo."""
    ref = read_newtdif(name)
    packed = M.PackedModels([_tree_chain_contact(solver)])
    qpos = ref["qpos"][0].astype(np.float32)
    qvel = ref["qvel"][0].astype(np.float32)
    worst_q = worst_v = 0.0
    for k, step in enumerate(ref["steps"]):
        qo, vo = oracle_py.run(packed, np.zeros(1, np.int32), qpos, qvel, None, step, precision=precision)
        worst_q = max(worst_q, np.abs(qo - ref["qpos"][k]).max())
        worst_v = max(worst_v, np.abs(vo - ref["qvel"][k]).max())
    assert worst_q <= qtol and worst_v <= vtol, (worst_q, worst_v)


def _free_body_scene(name):
    """The free-body differential scenes as newt's MJCF loader builds them:
    a free-jointed top-level body without children becomes a World body
    (newt/src/mjcf.rs:889-1010), geoms at the body origin, default solref
    and solimp, margin 0, condim 3; initial state from scenarios.json.
    Returns (model, qpos0, qvel0) in MuJoCo layout."""
    if name == "ballistic":  # tests/references/ballistic.xml
        w = M.WorldModel(dt=0.005, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=20)
        w.add_body(1.0, M._diag9(0.05, 0.06, 0.07))
        return w, [0.1, -0.2, 3.0, 1.0, 0.0, 0.0, 0.0], [3.0, -1.5, 5.0, 0.0, 0.0, 0.0]
    w = M.WorldModel(dt=0.002, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=20)
    if name == "sphere_drop":  # tests/references/sphere_drop.xml
        w.add_geom(M.static_plane(friction=0.8))
        b = w.add_body(0.5, M._diag9(0.002, 0.002, 0.002))
        w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, body=b, size=(0.1, 0.0, 0.0), friction=0.8))
        return w, [0.0, 0.0, 0.6, 1.0, 0.0, 0.0, 0.0], [0.0] * 6
    assert name == "box_stack"  # tests/references/box_stack.xml
    w.add_geom(M.static_plane(friction=0.6))
    qpos = []
    for mass, inert, pos in ((1.2, 0.098, (0.0, 0.0, 0.5)), (0.9, 0.0735, (0.02, 0.0, 1.25)),
                             (1.5, 0.1225, (0.0, 0.0, 2.0))):
        b = w.add_body(mass, M._diag9(inert, inert, inert))
        w.add_geom(M.Geom(shape=M.SHAPE_BOX, body=b, size=(0.35, 0.35, 0.35), friction=0.6))
        qpos += list(pos) + [1.0, 0.0, 0.0, 0.0]
    return w, qpos, [0.0] * 18


# matched-Euler windows against MuJoCo 3.11.0 (newt/tests/differential.rs:1272-1295)
FREE_BODY_WINDOWS = [("ballistic", 3.0e-5, 8.0e-5), ("sphere_drop", 1.5e-2, 9.0e-1), ("box_stack", 2.0e-2, 5.0e-1)]


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name,qtol,vtol", FREE_BODY_WINDOWS)
def test_free_body_euler_matches_mujoco_capture(precision, name, qtol, vtol):
    """Free-body rows of newt's matched-Euler differential test
    (differential.rs:1593-1599): the pile path's integrator, contacts and PGS
    stay inside newt's own windows against the MuJoCo captures."""
    ref = read_newtdif(f"{name}_euler.bin")
    w, q0, v0 = _free_body_scene(name)
    packed = M.PackedModels([w])
    qpos = np.array(q0, np.float32)
    qvel = np.array(v0, np.float32)
    assert np.abs(qpos - ref["qpos"][0]).max() < 1e-7 and np.abs(qvel - ref["qvel"][0]).max() == 0
    worst_q = worst_v = 0.0
    for k, step in enumerate(ref["steps"]):
        qo, vo = oracle_py.run(packed, np.zeros(1, np.int32), qpos, qvel, None, step, precision=precision)
        worst_q = max(worst_q, np.abs(qo - ref["qpos"][k]).max())
        worst_v = max(worst_v, np.abs(vo - ref["qvel"][k]).max())
    assert worst_q <= qtol and worst_v <= vtol, (worst_q, worst_v)
