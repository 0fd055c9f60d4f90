"""The elliptic cone and condim 1, 4 and 6 on tree links on the GPU
(tc_k_solve's general rows: the tangent pair, torsion and rolling rows, the
links' rotational Jacobians for the angular rows, the sweep over contact
blocks, free friction rows under Newton), through the C ABI, against the
oracle, whose tree rows meet newt's condim and cone bands on free-root links
(tests/test_oracle_tree_cones.py).

Bars:
  * newt's anchors (condim_torsional.rs, condim_rolling.rs,
    solver_friction_incline.rs) met by GPU runs of free-root links: condim-4
    spin decays monotonically below 5% (and stays above it with mu_t 0.005)
    under either cone, the condim-6 ball slows below half, the box holds on
    the 22-degree incline and slides on the 32-degree one under either cone;
  * from states along those runs, one GPU step no further from the FP64
    oracle's step than twice newt's own f32 step (the oracle's float mirror),
    or within 2e-6 m and 2e-4 m/s where newt's is closer;
  * on settled quadrupeds whose geoms take condim 3 (torso), 4 (hips), 1
    (thighs) and 6 (shanks), under PGS with either cone and under Newton: per
    row the impulses no further from FP64 than twice newt's f32 or within
    1e-3 of the row plus 1e-4 of the world's largest impulse; the touch
    readings likewise (1e-3 of the reading, floor 1); ten controlled steps
    within 2e-3 m and 5e-2 m/s of the FP64 oracle; the batched form within
    1e-5 m and 1e-4 m/s of the plain one."""
import numpy as np
import pytest

import oracle_py
from test_oracle_cones import incline, roller, spinner
from test_oracle_tree_cones import as_tree, run
from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN, scenes
from tooling_gb300 import api as A
from tooling_gb300 import model as M

pytestmark = pytest.mark.gpu
MARGIN_BAND = 1e-6


@pytest.fixture(scope="module")
def eng():
    from tooling_gb300 import build as B
    B.build()
    e = Engine(device=0)
    yield e
    e.close()


def _gpu_run(eng, t, q, v, n, mode=STEP_PLAIN):
    slots = eng.alloc(eng.upload(M.PackedModels([t])))
    eng.set_state(slots, q, v)
    eng.step(n, mode)
    gq, gv = eng.get_state(slots, 7, 6)
    st = int(eng.status(slots)[0])
    eng.free(slots)
    assert not st & 0x3, hex(st)
    return gq, gv


def _gpu_spin(eng, mu_t, cone, chunks=8, per=10):
    w, q, v = spinner(4, mu_t, cone)
    t = as_tree(w)
    q, v = _gpu_run(eng, t, q, v, 200)
    v = v.copy()
    v[3:6] = (0.0, 0.0, 8.0)
    out = [8.0]
    for _ in range(chunks):
        q, v = _gpu_run(eng, t, q, v, per)
        out.append(abs(float(v[5])))
    return out


@pytest.mark.parametrize("cone", [M.CONE_PYRAMIDAL, M.CONE_ELLIPTIC])
def test_link_spin_decays(eng, cone):
    h = _gpu_spin(eng, 0.5, cone)
    assert all(b <= a + 0.01 for a, b in zip(h, h[1:])), h
    assert h[-1] < 0.05 * h[0], h
    assert _gpu_spin(eng, 0.005, cone)[-1] > 0.05 * 8.0


@pytest.mark.parametrize("cone", [M.CONE_PYRAMIDAL, M.CONE_ELLIPTIC])
def test_link_rolling_ball_slows(eng, cone):
    w, q, v = roller(6, cone)
    t = as_tree(w)
    q, v = _gpu_run(eng, t, q, v, 50)
    v0 = float(np.hypot(v[0], v[1]))
    last = v0
    for _ in range(8):
        q, v = _gpu_run(eng, t, q, v, 100)
        now = float(np.hypot(v[0], v[1]))
        assert now <= last + 0.02, (now, last)
        last = now
    assert last < 0.5 * v0, (v0, last)


@pytest.mark.parametrize("cone", [M.CONE_PYRAMIDAL, M.CONE_ELLIPTIC])
def test_link_box_holds_at_22_slides_at_32(eng, cone):
    w, q, v = incline(22.0, 0.5, cone)
    gq, _ = _gpu_run(eng, as_tree(w), q, v, 800)
    assert abs(gq[0] - q[0]) < 0.20, gq[0]
    w, q, v = incline(32.0, 0.5, cone)
    gq, _ = _gpu_run(eng, as_tree(w), q, v, 800)
    assert gq[0] - q[0] > 1.0, gq[0]


def _scenes():
    out = []
    for cone in (M.CONE_PYRAMIDAL, M.CONE_ELLIPTIC):
        out.append(("incline32", cone) + incline(32.0, 0.5, cone))
        out.append(("spin4", cone) + spinner(4, 0.5, cone))
        out.append(("roll6", cone) + roller(6, cone))
    return out


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
def test_one_step_matches_fp64_along_the_runs(eng, mode):
    for name, cone, w, q, v in _scenes():
        t = as_tree(w)
        if name.startswith("spin"):
            q, v = run(t, q, v, 200)
            v[3:6] = (0.0, 0.0, 8.0)
        for k in range(4):
            gq, gv = _gpu_run(eng, t, q, v, 1, mode)
            q64, v64 = oracle_py.run(M.PackedModels([t]), np.zeros(1, np.int32), q, v, None, 1, precision=1,
                                     integrator=0)
            q32, v32 = run(t, q, v, 1, precision=0)
            gpu_q, gpu_v = np.abs(gq - q64).max(), np.abs(gv - v64).max()
            newt_q, newt_v = np.abs(q32 - q64).max(), np.abs(v32 - v64).max()
            assert gpu_q <= max(2e-6, 2 * newt_q) and gpu_v <= max(2e-4, 2 * newt_v), \
                (name, cone, k, gpu_q, newt_q, gpu_v, newt_v)
            q, v = run(t, q, v, 40)


# condim per geom of a quadruped world: plane, torso, then (hip, thigh, shank)
# per leg; a contact takes the smaller of its two geoms'
QUAD_CONDIM = np.array([6, 3] + [4, 1, 6] * 4, np.int32)


def _general_quads(solver, cone, n=16, first=300, steps=300):
    """Quadrupeds with QUAD_CONDIM, torsional friction 0.02 and rolling
    friction 0.01, advanced by the FP64 oracle until they lie on the plane."""
    b = scenes.quadruped_batch(n_worlds=n, first_world=first, solver=solver)
    g = b.geoms.copy()
    g["condim"] = np.tile(QUAD_CONDIM, n)
    g["torsional_friction"] = 0.02
    g["rolling_friction"] = 0.01
    q = M.Batch(b.links, b.n_links, b.bodies, b.n_bodies, g, b.n_geoms, 2e-3, (0.0, 0.0, -9.81), solver, 20,
                cone=cone)
    rq, rv = oracle_py.run(q, np.arange(n), b.qpos, b.qvel, None, steps, precision=1)
    q.qpos[:] = rq.astype(np.float32)
    q.qvel[:] = rv.astype(np.float32)
    return q


CASES = [(M.SOLVER_PGS, M.CONE_PYRAMIDAL), (M.SOLVER_PGS, M.CONE_ELLIPTIC), (M.SOLVER_NEWTON, M.CONE_PYRAMIDAL)]


@pytest.fixture(scope="module", params=CASES, ids=["pgs-pyramidal", "pgs-elliptic", "newton"])
def quads(request):
    return _general_quads(*request.param)


def _load(eng, b):
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, b.qpos, b.qvel)
    eng.set_qfrc(slots, b.qfrc)
    return slots


def _world(b, w):
    return (b.qpos[b.q_off[w]:b.q_off[w] + b.nq[w]], b.qvel[b.v_off[w]:b.v_off[w] + b.nv[w]],
            b.qfrc[b.v_off[w]:b.v_off[w] + b.nv[w]])


TOUCH = A.sensors(*[(A.SENSOR_TOUCH, 1, g) for g in range(1, 14)])  # reading j: geom j + 1
HIPS_AND_SHANKS = [g - 1 for g in (2, 5, 8, 11, 4, 7, 10, 13)]


def test_impulses_and_touch_match_fp64(eng, quads):
    b = quads
    slots = _load(eng, b)
    eng.step(1, STEP_PLAIN)
    touch = eng.read_sensors(slots, TOUCH)
    rows = general = 0
    for w in range(len(b)):
        qp, qv, qf = _world(b, w)
        _, rd = oracle_py.contacts(b, w, qp, qv)
        if len(rd) and (np.abs(rd[:, 6]) < MARGIN_BAND).any():
            continue
        r64, _ = oracle_py.tree_impulses(b, w, qp, qv, qf, precision=1)
        r32, _ = oracle_py.tree_impulses(b, w, qp, qv, qf, precision=0)
        g = eng.impulses(int(slots[w]))
        assert len(g) == len(r64), (w, len(g), len(r64))
        if len(r64):
            tol = np.maximum(1e-3 * np.abs(r64) + 1e-4 * np.abs(r64).max(), 2.0 * np.abs(r32 - r64))
            assert (np.abs(g - r64) <= tol).all(), (w, g, r64, r32)
            rows += len(r64)
        t64, _, _ = oracle_py.tree_contact_sensors(b, w, qp, qv, TOUCH, precision=1, qfrc=qf)
        t32, _, _ = oracle_py.tree_contact_sensors(b, w, qp, qv, TOUCH, precision=0, qfrc=qf)
        assert (np.abs(touch[w] - t64) <= np.maximum(1e-3 * np.maximum(1.0, np.abs(t64)),
                                                     2.0 * np.abs(t32 - t64))).all(), (w, touch[w], t64)
        general += int((t64[HIPS_AND_SHANKS] > 0).sum())
    assert rows > 0
    assert general > 0  # some hip or shank (condim 4 / 6) contact carries force
    st = eng.status(slots)
    assert not (st & 0x7).any(), st
    eng.free(slots)


def test_short_trajectory_tracks_fp64(eng, quads):
    b = quads
    b.qfrc[:] = scenes.quadruped_controls(len(b), 0, first_world=300)
    slots = _load(eng, b)
    eng.step(10, STEP_PLAIN)
    qp, qv = eng.get_state(slots, int(b.nq.sum()), int(b.nv.sum()))
    rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, b.qfrc, 10, precision=1)
    b.qfrc[:] = 0.0
    eng.free(slots)
    assert np.abs(qp - rq).max() < 2e-3
    assert np.abs(qv - rv).max() < 5e-2


def test_plain_and_batched_agree(eng, quads):
    b = quads
    s1 = _load(eng, b)
    eng.step(5, STEP_PLAIN)
    q1, v1 = eng.get_state(s1, int(b.nq.sum()), int(b.nv.sum()))
    eng.free(s1)
    s2 = _load(eng, b)
    eng.step(5, STEP_BATCHED)
    q2, v2 = eng.get_state(s2, int(b.nq.sum()), int(b.nv.sum()))
    eng.free(s2)
    assert np.abs(q1 - q2).max() < 1e-5 and np.abs(v1 - v2).max() < 1e-4


def _run_engine(items, mode, n=20):
    """Fresh context: upload and place each (model, qpos, qvel, nq, nv) in
    order, step n env-steps, return each one's state."""
    e = Engine(device=0)
    try:
        slots = []
        for P, q, v, nq, nv in items:
            s = e.alloc(e.upload(P))
            e.set_state(s, q, v)
            slots.append((s, nq, nv))
        e.step(n, mode)
        return [e.get_state(s, nq, nv) for s, nq, nv in slots]
    finally:
        e.close()


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
def test_tree_contact_groups_of_different_sizes_step_together(mode):
    """A larger tree-contact group placed before a smaller one: both are
    prepared before either launches, and each steps as it does alone."""
    b = scenes.quadruped_batch(n_worlds=4, first_world=50)
    w, q1, v1 = spinner(4, 0.5, M.CONE_ELLIPTIC)
    quad = (b, b.qpos, b.qvel, int(b.nq.sum()), int(b.nv.sum()))
    link = (M.PackedModels([as_tree(w)]), q1, v1, 7, 6)
    together = _run_engine([quad, link], mode)
    alone = [_run_engine([quad], mode)[0], _run_engine([link], mode)[0]]
    for (qa, va), (qt, vt) in zip(alone, together):
        assert np.abs(qa - qt).max() < 1e-5 and np.abs(va - vt).max() < 1e-4
