"""The oracle's free-body rows beyond pyramidal condim 3 against newt's
anchors (CPU): the elliptic cone, condim 1, torsional (condim 4) and rolling
(condim 6) friction, all under PGS and RK4 (World::new's integrator).

newt/tests/solver_friction_incline.rs:41-105: a box on a mu 0.5 incline holds
at 22 degrees (drift under 0.2 m in 800 steps) and slides at 32 degrees (over
1 m), under either cone.  solver_free_bodies.rs:147-190: a condim-1 block
slides on a shallow tilt that friction would hold.
condim_torsional.rs:60-140: a spinning sphere's spin decays monotonically to
under 5% in 0.4 s with condim 4 (mu_t 0.5), stays above 5% with mu_t 0.005,
and above half with condim 3.  condim_rolling.rs:60-110: a rolling sphere
slows monotonically to under half its speed in 4 s with condim 6 (mu_r 0.1)
and keeps over half with condim 3.  newt states these as bands; the oracle
meets them, and its elliptic and pyramidal incline runs differ (the cones
are not the same rule).  equality_golden.rs:189-258, 395-420: the oracle's
f32 mirror is byte-identical to newt's condim_torsional.bin (a sphere spun
at 8 rad/s on a condim-4 plane, mu_t 0.5) and condim_rolling.bin (a sphere
rolling at 1 m/s on a condim-6 plane, mu_r 0.1) after 0, 50, 200 and 1000
RK4 steps under PGS 30."""
import numpy as np
import pytest

import oracle_py
from test_oracle_golden import _read_f32
from tooling_gb300 import model as M

RK4 = 0


def incline(angle_deg, mu, cone, condim=3):
    a = np.float32(angle_deg) * np.float32(np.pi) / np.float32(180.0)
    g = np.float32(9.81)
    L = oracle_py.lib()
    w = M.WorldModel(dt=0.005, gravity=(float(g * np.float32(L.oracle_newt_sin(float(a)))), 0.0,
                                        float(-g * np.float32(L.oracle_newt_cos(float(a))))),
                     solver=M.SOLVER_PGS, iterations=30, integrator=M.INTEGRATOR_RK4, cone=cone)
    plane = M.static_plane(friction=mu)
    plane.condim = condim
    w.add_geom(plane)
    b = w.add_body(1.0, M.solid_box_inertia(1.0, (0.2, 0.2, 0.2)))
    w.add_geom(M.Geom(shape=M.SHAPE_BOX, body=b, size=(0.2, 0.2, 0.2), friction=mu, condim=condim))
    q = np.array([0.0, 0.0, 0.2, 1.0, 0.0, 0.0, 0.0], np.float32)
    return w, q, np.zeros(6, np.float32)


def _run(w, q, v, n, precision=1):
    qo, vo = oracle_py.run(M.PackedModels([w]), np.zeros(1, np.int32), q, v, None, n, precision=precision,
                           integrator=RK4)
    return qo.astype(np.float32), vo.astype(np.float32)


@pytest.mark.parametrize("cone", [M.CONE_PYRAMIDAL, M.CONE_ELLIPTIC])
def test_incline_holds_at_22_slides_at_32(cone):
    w, q, v = incline(22.0, 0.5, cone)
    qo, _ = _run(w, q, v, 800)
    assert abs(qo[0] - q[0]) < 0.20, qo[0]
    w, q, v = incline(32.0, 0.5, cone)
    qo, _ = _run(w, q, v, 800)
    assert qo[0] - q[0] > 1.0, qo[0]


def test_elliptic_and_pyramidal_cones_differ():
    runs = []
    for cone in (M.CONE_PYRAMIDAL, M.CONE_ELLIPTIC):
        w, q, v = incline(32.0, 0.5, cone)
        runs.append(_run(w, q, v, 200)[0])
    assert np.abs(runs[0] - runs[1]).max() > 1e-3


def test_condim_1_block_slides_on_a_shallow_tilt():
    w, q, v = incline(10.0, 1.0, M.CONE_PYRAMIDAL, condim=1)
    qo, _ = _run(w, q, v, 200)
    assert qo[0] - q[0] > 0.05, qo[0]  # condim 3 with mu 1 would hold at 10 degrees
    w, q, v = incline(10.0, 1.0, M.CONE_PYRAMIDAL, condim=3)
    qo3, _ = _run(w, q, v, 200)
    assert abs(qo3[0] - q[0]) < 0.01, qo3[0]


def spinner(condim, mu_t, cone=M.CONE_PYRAMIDAL):
    """condim_torsional.rs:12-52: a 1 kg sphere of radius 0.1 on a mu 0.8
    plane, solref (0.02, 1), PGS 30, dt 5e-3."""
    w = M.WorldModel(dt=0.005, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=30,
                     integrator=M.INTEGRATOR_RK4, cone=cone)
    plane = M.static_plane(friction=0.8)
    plane.condim, plane.torsional_friction = condim, mu_t
    w.add_geom(plane)
    b = w.add_body(1.0, M.solid_sphere_inertia(1.0, 0.1))
    w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, body=b, size=(0.1, 0.0, 0.0), friction=0.8, condim=condim,
                      torsional_friction=mu_t))
    return w, np.array([0.0, 0.0, 0.5, 1.0, 0.0, 0.0, 0.0], np.float32), np.zeros(6, np.float32)


def _spin_history(condim, mu_t, chunks=8, per=10, cone=M.CONE_PYRAMIDAL):
    w, q, v = spinner(condim, mu_t, cone)
    q, v = _run(w, q, v, 200)
    v[3:6] = (0.0, 0.0, 8.0)  # settle, then spin about z (body frame; the sphere sits upright)
    out = [8.0]
    for _ in range(chunks):
        q, v = _run(w, q, v, per)
        out.append(abs(float(v[5])))
    return out


@pytest.mark.parametrize("cone", [M.CONE_PYRAMIDAL, M.CONE_ELLIPTIC])
def test_condim_4_spin_decays(cone):
    h = _spin_history(4, 0.5, cone=cone)
    assert all(b <= a + 0.01 for a, b in zip(h, h[1:])), h
    assert h[-1] < 0.05 * h[0], h


def test_weak_torsion_and_condim_3_keep_spinning():
    assert _spin_history(4, 0.005)[-1] > 0.05 * 8.0
    assert _spin_history(3, 0.5)[-1] > 0.5 * 8.0


def roller(condim, cone=M.CONE_PYRAMIDAL):
    """condim_rolling.rs:12-50: a 1 kg sphere of radius 0.1 rolling at 1 m/s
    (10 rad/s about y) on a mu 0.9 plane, mu_r 0.1."""
    w = M.WorldModel(dt=0.005, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=30,
                     integrator=M.INTEGRATOR_RK4, cone=cone)
    plane = M.static_plane(friction=0.9)
    plane.condim, plane.rolling_friction = condim, 0.1
    w.add_geom(plane)
    b = w.add_body(1.0, M.solid_sphere_inertia(1.0, 0.1))
    w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, body=b, size=(0.1, 0.0, 0.0), friction=0.9, condim=condim,
                      rolling_friction=0.1))
    q = np.array([0.0, 0.0, 0.1, 1.0, 0.0, 0.0, 0.0], np.float32)
    v = np.array([1.0, 0.0, 0.0, 0.0, 10.0, 0.0], np.float32)
    return w, q, v


@pytest.mark.parametrize("cone", [M.CONE_PYRAMIDAL, M.CONE_ELLIPTIC])
def test_condim_6_rolling_ball_slows(cone):
    w, q, v = roller(6, cone)
    q, v = _run(w, q, v, 50)
    v0 = float(np.hypot(v[0], v[1]))
    last = v0
    for _ in range(8):
        q, v = _run(w, q, v, 100)
        now = float(np.hypot(v[0], v[1]))
        assert now <= last + 0.02, (now, last)
        last = now
    assert last < 0.5 * v0, (v0, last)


def test_condim_3_ball_keeps_rolling():
    w, q, v = roller(3)
    q, v = _run(w, q, v, 50)
    v0 = float(np.hypot(v[0], v[1]))
    q, v = _run(w, q, v, 800)
    assert float(np.hypot(v[0], v[1])) > 0.5 * v0


def condim_golden_scene(kind):
    """equality_golden.rs:189-258: World::new() (RK4, PGS 30, pyramidal), a
    1 kg sphere of radius 0.1 on a plane, solref (0.02, 1), the default
    solimp; newt layout (pos, quat xyzw; v_world, omega_body)."""
    fr, cd = (0.9, 6) if kind == "rolling" else (0.8, 4)
    w = M.WorldModel(dt=0.005, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=30,
                     integrator=M.INTEGRATOR_RK4, cone=M.CONE_PYRAMIDAL)
    plane = M.static_plane(friction=fr)
    g = M.Geom(shape=M.SHAPE_SPHERE, body=0, size=(0.1, 0.0, 0.0), friction=fr)
    for geom in (plane, g):
        geom.solref, geom.condim = (0.02, 1.0), cd
        if kind == "rolling":
            geom.rolling_friction = 0.1
        else:
            geom.torsional_friction = 0.5
    w.add_geom(plane)
    w.add_body(1.0, M.solid_sphere_inertia(1.0, 0.1))
    w.add_geom(g)
    if kind == "rolling":
        q, v = [0.0, 0.01, 0.1, 0.0, 0.0, 0.0, 1.0], [1.0, 0.0, 0.0, 0.0, 10.0, 0.0]
    else:
        q, v = [0.01, 0.0, 0.5, 0.0, 0.0, 0.0, 1.0], [0.0, 0.0, 0.0, 0.0, 0.0, 8.0]
    return w, np.array(q, np.float32), np.array(v, np.float32)


@pytest.mark.parametrize("kind", ["torsional", "rolling"])
def test_condim_goldens_are_byte_identical(kind):
    w, q, v = condim_golden_scene(kind)
    gold = _read_f32(f"condim_{kind}.bin").reshape(4, 13)
    P = M.PackedModels([w])
    got = [np.concatenate([q, v])]
    for n in (50, 200, 1000):
        qo, vo = oracle_py.run(P, np.zeros(1, np.int32), q, v, None, n, precision=0, layout=1, integrator=0)
        got.append(np.concatenate([qo, vo]).astype(np.float32))
    got = np.stack(got)
    assert got.tobytes() == gold.tobytes(), np.abs(got - gold).max(axis=1)
