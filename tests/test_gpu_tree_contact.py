"""GPU parity for tree-contact worlds (quadrupeds on a plane, Newton or PGS)
through the C ABI, against the FP64 oracle.

Bars (stated here, checked below):
  * contact pair lists identical to the oracle's wherever no penetration lies
    within 1e-6 of the margin;
  * row impulses, same solver and iteration cap, within 1e-3 of each row's
    own FP64 value plus an absolute floor of 1e-4 of the world's largest
    impulse (newt's own f32 arithmetic, the oracle's float mirror, uses 0.25
    of that bar under Newton and 0.67 under PGS on these worlds);
  * short-horizon trajectories within 2e-3 m / 5e-2 m/s;
  * the MuJoCo capture of newt's tree-chain contact scene inside newt's own
    differential windows (qpos 8e-2 / 7e-2, qvel 1.3 / 0.7).
"""
import os
import sys

import numpy as np
import pytest

import oracle_py
from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN, scenes
from tooling_gb300 import model as M

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from test_oracle_golden import _tree_chain_contact, read_newtdif  # noqa: E402

pytestmark = pytest.mark.gpu

IMPULSE_RTOL = 1e-3
IMPULSE_FLOOR = 1e-4  # of the world's largest impulse
MARGIN_BAND = 1e-6


@pytest.fixture(scope="module")
def eng():
    from tooling_gb300 import build as B
    B.build()
    e = Engine(device=0)
    yield e
    e.close()


def _settled(solver, n=24, steps=300, first=300):
    """Quadrupeds advanced by the FP64 oracle until they lie on the plane
    with 4-12 contacts each."""
    b = scenes.quadruped_batch(n_worlds=n, first_world=first, solver=solver)
    rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, None, steps, precision=1)
    b.qpos[:] = rq.astype(np.float32)
    b.qvel[:] = rv.astype(np.float32)
    return b


@pytest.fixture(scope="module")
def settled_newton():
    return _settled(M.SOLVER_NEWTON)


@pytest.fixture(scope="module")
def settled_pgs():
    return _settled(M.SOLVER_PGS)


def _load(eng, b):
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, b.qpos, b.qvel)
    if b.qfrc.any():
        eng.set_qfrc(slots, b.qfrc)
    return slots


def _world(b, w):
    return (b.qpos[b.q_off[w]:b.q_off[w] + b.nq[w]], b.qvel[b.v_off[w]:b.v_off[w] + b.nv[w]],
            b.qfrc[b.v_off[w]:b.v_off[w] + b.nv[w]])


def test_contact_pair_lists_match_oracle(eng, settled_newton):
    b = settled_newton
    slots = _load(eng, b)
    eng.step(1, STEP_PLAIN)
    eng.sync()
    compared = 0
    for w in range(len(b)):
        qp, qv, _ = _world(b, w)
        rp, rd = oracle_py.contacts(b, w, qp, qv)
        if len(rd) and (np.abs(rd[:, 6]) < MARGIN_BAND).any():
            continue
        gp, gd = eng.contacts(int(slots[w]))
        assert np.array_equal(gp, rp), f"world {w}"
        if len(rd):
            assert np.abs(gd[:, 6] - rd[:, 6]).max() < 1e-4
            assert np.abs(gd[:, :3] - rd[:, :3]).max() < 1e-4
            assert np.abs(gd[:, 3:6] - rd[:, 3:6]).max() < 1e-5
        compared += 1
    assert compared >= len(b) // 2
    eng.free(slots)


@pytest.mark.parametrize("which", ["newton", "pgs"])
def test_impulses_match_oracle(eng, settled_newton, settled_pgs, which):
    b = settled_newton if which == "newton" else settled_pgs
    slots = _load(eng, b)
    eng.step(1, STEP_PLAIN)
    eng.sync()
    worst, rows = 0.0, 0
    for w in range(len(b)):
        qp, qv, qf = _world(b, w)
        rp, rd = oracle_py.contacts(b, w, qp, qv)
        if len(rd) and (np.abs(rd[:, 6]) < MARGIN_BAND).any():
            continue
        ref, _ = oracle_py.tree_impulses(b, w, qp, qv, qf)
        g = eng.impulses(int(slots[w]))
        assert len(g) == len(ref), f"world {w}"
        if len(ref):
            tol = IMPULSE_RTOL * np.abs(ref) + IMPULSE_FLOOR * np.abs(ref).max()
            worst = max(worst, float((np.abs(g - ref) / tol).max()))
            rows += len(ref)
    assert rows > 0
    assert worst <= 1.0, worst
    st = eng.status(slots)
    assert not (st & 0x7).any(), st  # no NaN, no factorisation failure, no overflow
    eng.free(slots)


def test_short_trajectory_tracks_oracle(eng, settled_newton):
    b = settled_newton
    b.qfrc[:] = scenes.quadruped_controls(len(b), 0, first_world=300)
    slots = _load(eng, b)
    eng.step(10, STEP_PLAIN)
    qp, qv = eng.get_state(slots, int(b.nq.sum()), int(b.nv.sum()))
    rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, b.qfrc, 10, precision=1)
    assert np.abs(qp - rq).max() < 2e-3
    assert np.abs(qv - rv).max() < 5e-2
    b.qfrc[:] = 0.0
    eng.free(slots)


def test_plain_and_batched_agree(eng, settled_newton):
    b = settled_newton
    s1 = _load(eng, b)
    eng.step(5, STEP_PLAIN)
    q1, v1 = eng.get_state(s1, int(b.nq.sum()), int(b.nv.sum()))
    eng.free(s1)
    s2 = _load(eng, b)
    eng.step(5, STEP_BATCHED)
    q2, v2 = eng.get_state(s2, int(b.nq.sum()), int(b.nv.sum()))
    eng.free(s2)
    assert np.abs(q1 - q2).max() < 1e-5 and np.abs(v1 - v2).max() < 1e-4


@pytest.mark.parametrize("solver,name,qtol,vtol", [
    (M.SOLVER_NEWTON, "tree_chain_contact_newton_euler.bin", 8.0e-2, 1.3),
    (M.SOLVER_PGS, "tree_chain_contact_pgs_euler.bin", 7.0e-2, 0.7)])
def test_tree_chain_contact_within_mujoco_windows(eng, solver, name, qtol, vtol):
    """The GPU step on newt's tree-chain contact scene stays inside the
    windows newt's differential tests allow against MuJoCo
    (newt/tests/differential.rs:1411-1446)."""
    ref = read_newtdif(name)
    packed = M.PackedModels([_tree_chain_contact(solver)])
    slots = eng.alloc(eng.upload(packed))
    eng.set_state(slots, ref["qpos"][0].astype(np.float32), ref["qvel"][0].astype(np.float32))
    worst_q = worst_v = 0.0
    prev = 0
    for k, step in enumerate(ref["steps"]):
        if step > prev:
            eng.step(step - prev, STEP_PLAIN)
            prev = step
        qp, qv = eng.get_state(slots, 8, 7)
        worst_q = max(worst_q, np.abs(qp - ref["qpos"][k]).max())
        worst_v = max(worst_v, np.abs(qv - ref["qvel"][k]).max())
    eng.free(slots)
    assert worst_q <= qtol and worst_v <= vtol, (worst_q, worst_v)


def _snake(n_hinges, foot_every=5):
    """A free root and `n_hinges` hinged links in a line along x, axes
    alternating z and y, masses alternating 1 and 0.05 kg, sphere feet on
    every fifth link resting 0.5 mm into the plane; Newton, dt 2e-3."""
    w = M.WorldModel(dt=0.002, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_NEWTON, iterations=20)
    w.add_geom(M.static_plane(friction=0.8))
    for i in range(n_hinges + 1):
        m = 1.0 if i % 2 == 0 else 0.05
        inert = 0.4 * m * 0.03 ** 2 + m * 0.05 ** 2 / 3
        if i == 0:
            w.push_link(M.Link(parent=-1, joint=M.JOINT_FREE, mass=m, inertia=M._diag9(inert, inert, inert)))
        else:
            ax = (0.0, 0.0, 1.0) if i % 2 else (0.0, 1.0, 0.0)
            w.push_link(M.Link(parent=i - 1, joint=M.JOINT_HINGE, axis=ax, jp_pos=(0.05, 0.0, 0.0),
                               jc_pos=(-0.05, 0.0, 0.0), mass=m, inertia=M._diag9(inert, inert, inert),
                               damping=0.01))
        if i % foot_every == 0:
            w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, link=i, size=(0.03, 0.0, 0.0), friction=0.8))
    rng = np.random.default_rng(n_hinges)
    qpos = np.zeros(w.nq, np.float32)  # straight, every foot 0.5 mm into the plane
    qpos[2], qpos[3] = 0.0295, 1.0
    qvel = rng.normal(0.0, 0.1, w.nv).astype(np.float32)
    return w, qpos, qvel


@pytest.mark.parametrize("n_hinges", [25, 39])
def test_long_chain_contact_qacc_matches_fp64(eng, n_hinges):
    """Trees above 24 DoF sum the mass matrix in FP64 and take one FP64
    residual-refinement step of the mass-matrix solve (M + dt B) x = J^T f /
    dt.  On a 31-DoF and a 45-DoF snake lying straight with every foot in
    contact (6 and 8), the contact pairs equal the oracle's and the one-step
    qacc ((qvel' - qvel) / dt, the same layout on both sides) is no further
    (max-norm relative) from the FP64 oracle's than 1e-4 or newt's own f32
    arithmetic (the f32 oracle), whichever is larger: newt's is 4.0e-5 and
    1.6e-4 away, this path 2.7e-5 and 1.4e-4 (with an f32 sum of M it was
    4e-4 and 3e-3).  The impulses of these
    ill-conditioned Newton systems are held to twice newt's own f32 distance
    from FP64 on the per-row bar (0.54 and 0.99 bar units), and never less
    than the bar itself."""
    w, qpos, qvel = _snake(n_hinges)
    packed = M.PackedModels([w])
    rp, _ = oracle_py.contacts(packed, 0, qpos, qvel)
    assert len(rp) == n_hinges // 5 + 1  # every foot
    slots = eng.alloc(eng.upload(packed))
    eng.set_state(slots, qpos, qvel)
    eng.step(1, STEP_PLAIN)
    _, v_gpu = eng.get_state(slots, w.nq, w.nv)
    st = int(eng.status(slots)[0])
    gp, _ = eng.contacts(int(slots[0]))
    g_imp = eng.impulses(int(slots[0]))
    eng.free(slots)
    assert not st & 0x3, hex(st)
    assert np.array_equal(gp, rp)

    def bar_units(imp, ref):
        return (np.abs(imp - ref) / (IMPULSE_RTOL * np.abs(ref) + IMPULSE_FLOOR * np.abs(ref).max())).max()

    ref_imp, _ = oracle_py.tree_impulses(packed, 0, qpos, qvel, None, precision=1)
    f32_imp, _ = oracle_py.tree_impulses(packed, 0, qpos, qvel, None, precision=0)
    newt_units = bar_units(f32_imp, ref_imp)
    gpu_units = bar_units(g_imp, ref_imp)
    assert gpu_units <= max(1.0, 2.0 * newt_units), (w.nv, gpu_units, newt_units)
    _, v64 = oracle_py.run(packed, np.zeros(1, np.int32), qpos, qvel, None, 1, precision=1)
    q0 = qvel.astype(np.float64)
    ref = (v64 - q0) / w.dt  # semi-implicit Euler: qvel += qacc dt
    got = (v_gpu.astype(np.float64) - q0) / w.dt
    rel = np.abs(got - ref).max() / np.abs(ref).max()
    _, v32 = oracle_py.run(packed, np.zeros(1, np.int32), qpos, qvel, None, 1, precision=0)
    newt_rel = np.abs((v32 - q0) / w.dt - ref).max() / np.abs(ref).max()
    assert rel <= max(1e-4, newt_rel), (w.nv, rel, newt_rel)
