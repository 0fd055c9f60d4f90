"""The oracle's tree-contact rows beyond pyramidal condim 3 (CPU): the
elliptic cone and torsional (condim 4) and rolling (condim 6) friction on
tree links (newt/src/solver.rs:2880-3330: contact_row_directions' general
rows with the links' rotational Jacobians for the angular rows,
tree_contact_diag_approx's rotation weight, world_pgs_pair and
world_pgs_scalar; under Newton the general rows' only projection is the
normal row's, solver.rs:3164-3196).

newt's condim and cone anchors are stated on free bodies
(condim_torsional.rs:60-140, condim_rolling.rs:60-110,
solver_friction_incline.rs:41-105; tests/test_oracle_cones.py); here each
scene's body is a free-root link carrying the same geom, and the link meets
the same bands: the spin of a sphere on a condim-4 plane decays
monotonically to under 5% in 0.4 s (mu_t 0.5) and stays above 5% (mu_t
0.005) or half (condim 3); a ball rolling on a condim-6 plane slows
monotonically to under half its speed in 4 s and keeps over half with
condim 3; a box on a mu 0.5 incline holds at 22 degrees and slides at 32
under either cone.  Where only the contact's normal row carries force (the
spinning sphere) the link's trajectory equals the body's, which is pinned
byte for byte to newt's condim_torsional.bin, within 1e-9."""
import copy

import numpy as np
import pytest

import oracle_py
from test_oracle_cones import condim_golden_scene, incline, roller, spinner
from tooling_gb300 import model as M

RK4 = 0


def as_tree(w, solver=None):
    """The world with its one free body turned into a free-root link that
    carries the body's geoms."""
    t = M.WorldModel(dt=w.dt, gravity=w.gravity, solver=w.solver if solver is None else solver,
                     iterations=w.iterations, integrator=w.integrator, cone=w.cone)
    mass, inertia = w.bodies[0]
    t.push_link(M.Link(parent=-1, joint=M.JOINT_FREE, mass=mass, inertia=list(inertia)))
    for g in w.geoms:
        g2 = copy.copy(g)
        if g2.body == 0:
            g2.body, g2.link = -1, 0
        t.add_geom(g2)
    return t


def run(w, q, v, n, precision=1):
    qo, vo = oracle_py.run(M.PackedModels([w]), np.zeros(1, np.int32), q, v, None, n, precision=precision,
                           integrator=RK4)
    return qo.astype(np.float32), vo.astype(np.float32)


def spin_history(condim, mu_t, cone=M.CONE_PYRAMIDAL, solver=None, chunks=8, per=10):
    w, q, v = spinner(condim, mu_t, cone)
    t = as_tree(w, solver)
    q, v = run(t, q, v, 200)
    v[3:6] = (0.0, 0.0, 8.0)  # settle, then spin about z (body frame; the sphere sits upright)
    out = [8.0]
    for _ in range(chunks):
        q, v = run(t, q, v, per)
        out.append(abs(float(v[5])))
    return out


@pytest.mark.parametrize("cone", [M.CONE_PYRAMIDAL, M.CONE_ELLIPTIC])
def test_link_spin_decays_with_condim_4(cone):
    h = spin_history(4, 0.5, cone)
    assert all(b <= a + 0.01 for a, b in zip(h, h[1:])), h
    assert h[-1] < 0.05 * h[0], h


def test_link_weak_torsion_and_condim_3_keep_spinning():
    assert spin_history(4, 0.005)[-1] > 0.05 * 8.0
    assert spin_history(3, 0.5)[-1] > 0.5 * 8.0


def test_link_spin_decays_under_newton():
    """Under Newton the torsion row has no cap (no projection), so the spin
    stops at least as fast as under PGS."""
    h = spin_history(4, 0.5, solver=M.SOLVER_NEWTON)
    assert h[-1] < 0.05 * h[0], h


@pytest.mark.parametrize("cone", [M.CONE_PYRAMIDAL, M.CONE_ELLIPTIC])
def test_link_rolling_ball_slows_with_condim_6(cone):
    w, q, v = roller(6, cone)
    t = as_tree(w)
    q, v = run(t, q, v, 50)
    v0 = float(np.hypot(v[0], v[1]))
    last = v0
    for _ in range(8):
        q, v = run(t, q, v, 100)
        now = float(np.hypot(v[0], v[1]))
        assert now <= last + 0.02, (now, last)
        last = now
    assert last < 0.5 * v0, (v0, last)


def test_link_ball_keeps_rolling_with_condim_3():
    w, q, v = roller(3)
    t = as_tree(w)
    q, v = run(t, q, v, 50)
    v0 = float(np.hypot(v[0], v[1]))
    q, v = run(t, q, v, 800)
    assert float(np.hypot(v[0], v[1])) > 0.5 * v0


@pytest.mark.parametrize("cone", [M.CONE_PYRAMIDAL, M.CONE_ELLIPTIC])
def test_link_box_holds_at_22_slides_at_32(cone):
    w, q, v = incline(22.0, 0.5, cone)
    qo, _ = run(as_tree(w), q, v, 800)
    assert abs(qo[0] - q[0]) < 0.20, qo[0]
    w, q, v = incline(32.0, 0.5, cone)
    qo, _ = run(as_tree(w), q, v, 800)
    assert qo[0] - q[0] > 1.0, qo[0]


def test_link_and_body_spin_agree():
    w, q, v = condim_golden_scene("torsional")
    qm = np.array([q[0], q[1], q[2], q[6], q[3], q[4], q[5]], np.float32)  # MuJoCo layout
    for cone in (M.CONE_PYRAMIDAL, M.CONE_ELLIPTIC):
        w.cone = cone
        for n in (50, 200, 400):
            a, b = (np.concatenate(oracle_py.run(M.PackedModels([x]), np.zeros(1, np.int32), qm, v, None, n,
                                                 precision=1, integrator=RK4)) for x in (w, as_tree(w)))
            assert np.abs(a - b).max() < 1e-9, (cone, n, a, b)
