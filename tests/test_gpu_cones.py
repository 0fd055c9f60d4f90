"""The elliptic friction cone and condim 1, 4 and 6 on the GPU (pile worlds
solved over newt's general rows, pile_general.cu), through the C ABI,
against the oracle, whose free-body rows hold newt's anchors
(tests/test_oracle_cones.py).

Bars:
  * newt's condim goldens (condim_torsional.bin, condim_rolling.bin, the
    oracle byte-identical to both): from each snapshot one GPU step within
    2e-6 m and 2e-4 m/s of the oracle's f32 step, and from the start the GPU
    within 5e-4 m and 5e-3 m/s of newt's snapshots at steps 50, 200, 1000;
  * newt's anchors (solver_friction_incline.rs, solver_free_bodies.rs,
    condim_torsional.rs, condim_rolling.rs) met by GPU runs: the incline
    holds at 22 and slides at 32 degrees under either cone, the condim-1
    block slides, condim-4 spin decays monotonically below 5% (and stays
    above it with mu_t 0.005), the condim-6 ball slows below half;
  * from states along those runs, one GPU step within 2e-6 m and 2e-4 m/s
    of the oracle's f32 step (newt's arithmetic; the PGS goldens' bars);
  * on settled 16-body piles with a condim drawn per geom from {1, 3, 4, 6}
    under either cone: the contact pairs equal, per row the impulses, and
    the one-step velocities, no further from the FP64 oracle than twice
    newt's own f32 arithmetic (or within 1e-3 relative per row and 1e-4
    m/s); the touch sensors likewise;
  * the batched form equal to the plain one, with facet-row PGS piles and
    Newton piles stepped alongside;
  * the forms the GPU path refuses are refused at upload."""
import numpy as np
import pytest

import oracle_py
from test_oracle_cones import RK4, _run, condim_golden_scene, incline, roller, spinner
from test_oracle_golden import _read_f32
from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN, scenes
from tooling_gb300 import api as A
from tooling_gb300 import model as M

pytestmark = pytest.mark.gpu
IMPULSE_RTOL, IMPULSE_FLOOR = 1e-3, 2e-5
MARGIN_BAND = 1e-6


@pytest.fixture(scope="module")
def eng():
    from tooling_gb300 import build as B
    B.build()
    e = Engine(device=0)
    yield e
    e.close()


def _gpu_run(eng, w, q, v, n, mode=STEP_PLAIN):
    nb = len(w.bodies)
    slots = eng.alloc(eng.upload(M.PackedModels([w])))
    eng.set_state(slots, q, v)
    eng.step(n, mode)
    gq, gv = eng.get_state(slots, 7 * nb, 6 * nb)
    st = int(eng.status(slots)[0])
    eng.free(slots)
    assert not st & 0x3, hex(st)
    return gq, gv


def _mj_body(row):
    """newt's body snapshot (pos, quat xyzw, v_world, omega_body) in MuJoCo
    layout (pos, quat wxyz; v_world, omega_body)."""
    return (np.array([row[0], row[1], row[2], row[6], row[3], row[4], row[5]], np.float32),
            np.array(row[7:13], np.float32))


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
@pytest.mark.parametrize("kind", ["torsional", "rolling"])
def test_condim_goldens(eng, kind, mode):
    w, _, _ = condim_golden_scene(kind)
    gold = _read_f32(f"condim_{kind}.bin").reshape(4, 13)
    P = M.PackedModels([w])
    for row in range(4):
        q, v = _mj_body(gold[row])
        gq, gv = _gpu_run(eng, w, q, v, 1, mode)
        rq, rv = oracle_py.run(P, np.zeros(1, np.int32), q, v, None, 1, precision=0, integrator=RK4)
        assert np.abs(gq - rq).max() < 2e-6 and np.abs(gv - rv).max() < 2e-4, (row, np.abs(gq - rq).max(),
                                                                                np.abs(gv - rv).max())
    q, v = _mj_body(gold[0])
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q, v)
    done = 0
    for row, n in enumerate((50, 200, 1000), start=1):
        eng.step(n - done, mode)
        done = n
        gq, gv = eng.get_state(slots, 7, 6)
        rq, rv = _mj_body(gold[row])
        assert np.abs(gq - rq).max() < 5e-4 and np.abs(gv - rv).max() < 5e-3, (n, np.abs(gq - rq).max(),
                                                                                np.abs(gv - rv).max())
    eng.free(slots)


@pytest.mark.parametrize("cone", [M.CONE_PYRAMIDAL, M.CONE_ELLIPTIC])
def test_incline_holds_at_22_slides_at_32(eng, cone):
    # the pyramidal condim-3 incline runs the facet-row kernels, the elliptic one the general rows
    w, q, v = incline(22.0, 0.5, cone)
    gq, _ = _gpu_run(eng, w, q, v, 800)
    assert abs(gq[0] - q[0]) < 0.20, gq[0]
    w, q, v = incline(32.0, 0.5, cone)
    gq, _ = _gpu_run(eng, w, q, v, 800)
    assert gq[0] - q[0] > 1.0, gq[0]
    rq, _ = _run(w, q, v, 800)
    assert abs(gq[0] - rq[0]) < 1e-2 * abs(rq[0] - q[0]), (gq[0], rq[0])


def test_condim_1_block_slides_on_a_shallow_tilt(eng):
    w, q, v = incline(10.0, 1.0, M.CONE_PYRAMIDAL, condim=1)
    gq, _ = _gpu_run(eng, w, q, v, 200)
    assert gq[0] - q[0] > 0.05, gq[0]
    rq, _ = _run(w, q, v, 200)
    assert abs(gq[0] - rq[0]) < 1e-2 * abs(rq[0] - q[0]), (gq[0], rq[0])


def _gpu_spin(eng, condim, mu_t, cone, chunks=8, per=10):
    w, q, v = spinner(condim, mu_t, cone)
    q, v = _gpu_run(eng, w, q, v, 200)
    v = v.copy()
    v[3:6] = (0.0, 0.0, 8.0)
    out = [8.0]
    for _ in range(chunks):
        q, v = _gpu_run(eng, w, q, v, per)
        out.append(abs(float(v[5])))
    return out


@pytest.mark.parametrize("cone", [M.CONE_PYRAMIDAL, M.CONE_ELLIPTIC])
def test_condim_4_spin_decays(eng, cone):
    h = _gpu_spin(eng, 4, 0.5, cone)
    assert all(b <= a + 0.01 for a, b in zip(h, h[1:])), h
    assert h[-1] < 0.05 * h[0], h
    assert _gpu_spin(eng, 4, 0.005, cone)[-1] > 0.05 * 8.0


@pytest.mark.parametrize("cone", [M.CONE_PYRAMIDAL, M.CONE_ELLIPTIC])
def test_condim_6_rolling_ball_slows(eng, cone):
    w, q, v = roller(6, cone)
    q, v = _gpu_run(eng, w, q, v, 50)
    v0 = float(np.hypot(v[0], v[1]))
    last = v0
    for _ in range(8):
        q, v = _gpu_run(eng, w, q, v, 100)
        now = float(np.hypot(v[0], v[1]))
        assert now <= last + 0.02, (now, last)
        last = now
    assert last < 0.5 * v0, (v0, last)


def _scenes():
    out = []
    for cone in (M.CONE_PYRAMIDAL, M.CONE_ELLIPTIC):
        out.append(("incline32", cone) + incline(32.0, 0.5, cone))
        out.append(("spin4", cone) + spinner(4, 0.5, cone))
        out.append(("roll6", cone) + roller(6, cone))
    out.append(("incline_condim1", M.CONE_PYRAMIDAL) + incline(10.0, 1.0, M.CONE_PYRAMIDAL, condim=1))
    return out


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
def test_one_step_matches_newt_along_the_runs(eng, mode):
    worst = []
    for name, cone, w, q, v in _scenes():
        if name.startswith("spin"):
            q, v = _run(w, q, v, 200)
            v[3:6] = (0.0, 0.0, 8.0)
        for k in range(4):
            gq, gv = _gpu_run(eng, w, q, v, 1, mode)
            rq, rv = _run(w, q, v, 1)
            dq, dv = float(np.abs(gq - rq).max()), float(np.abs(gv - rv).max())
            worst.append((name, cone, k, dq, dv))
            assert dq < 2e-6 and dv < 2e-4, worst[-1]
            q, v = _run(w, q, v, 40)


def _general(b, cone, seed=5):
    """The batch with a condim drawn per geom from {1, 3, 4, 6}, torsional
    friction 0.02 and rolling friction 0.01, under `cone`."""
    g = b.geoms.copy()
    rng = np.random.default_rng(seed)
    g["condim"] = rng.choice(np.array([1, 3, 4, 6], np.int32), size=len(g))
    g["torsional_friction"] = 0.02
    g["rolling_friction"] = 0.01
    return M.Batch(b.links, b.n_links, b.bodies, b.n_bodies, g, b.n_geoms, 2e-3, (0.0, 0.0, -9.81), M.SOLVER_PGS,
                   50, cone=cone)


@pytest.fixture(scope="module")
def settled():
    b = scenes.pile_batch(n_worlds=16, first_world=2100)
    rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, None, 300, precision=1)
    return b, rq.astype(np.float32), rv.astype(np.float32)


def _rows(b, w, cone, pairs):
    """Rows per contact of newt's general assembly (solver.rs:752-848)."""
    cd = b.geoms["condim"][b.geom_off[w]:b.geom_off[w] + b.n_geoms[w]]
    out = []
    for ga, gb in pairs:
        c = int(min(cd[ga], cd[gb]))
        out.append(4 if (cone == M.CONE_PYRAMIDAL and c == 3) else c)
    return out


def _world(b, w):
    return b.qpos[b.q_off[w]:b.q_off[w] + b.nq[w]], b.qvel[b.v_off[w]:b.v_off[w] + b.nv[w]]


@pytest.mark.parametrize("cone", [M.CONE_PYRAMIDAL, M.CONE_ELLIPTIC])
def test_general_piles_impulses_and_step_match_fp64(eng, settled, cone):
    b0, q0, v0 = settled
    b = _general(b0, cone)
    b.qpos[:] = q0
    b.qvel[:] = v0
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, b.qpos, b.qvel)
    eng.step(1, STEP_PLAIN)
    _, gv_all = eng.get_state(slots, int(b.nq.sum()), int(b.nv.sum()))
    st = eng.status(slots)
    rows, checked, kinds = 0, 0, set()
    for w in range(len(b)):
        qp, qv = _world(b, w)
        rp, rd = oracle_py.contacts(b, w, qp, qv)
        if len(rd) and (np.abs(rd[:, 6]) < MARGIN_BAND).any():
            continue
        gp, _ = eng.contacts(int(slots[w]))
        assert gp.tolist() == rp.tolist(), f"world {w}"
        active = rd[:, 6] > 0 if len(rd) else np.zeros(0, bool)
        nr = _rows(b, w, cone, rp[active])
        kinds.update(nr)
        gi = eng.impulses(int(slots[w])).reshape(-1, 6)[active]
        g = np.concatenate([gi[k, :n] for k, n in enumerate(nr)]) if nr else np.zeros(0)
        ref = oracle_py.impulses(b, w, qp, qv, precision=1)
        f32 = oracle_py.impulses(b, w, qp, qv, precision=0)
        assert len(g) == len(ref), f"world {w}"
        if len(ref):
            tol = IMPULSE_RTOL * np.abs(ref) + IMPULSE_FLOOR * np.abs(ref).max()
            gpu_u, newt_u = (np.abs(g - ref) / tol).max(), (np.abs(f32 - ref) / tol).max()
            assert gpu_u <= max(1.0, 2.0 * newt_u), (w, gpu_u, newt_u)
            rows += len(ref)
        _, v64 = oracle_py.run(b, np.array([w], np.int32), qp, qv, None, 1, precision=1)
        _, v32 = oracle_py.run(b, np.array([w], np.int32), qp, qv, None, 1, precision=0)
        gv = gv_all[b.v_off[w]:b.v_off[w] + b.nv[w]]
        gpu_d, newt_d = np.abs(gv - v64).max(), np.abs(v32 - v64).max()
        assert gpu_d <= max(1e-4, 2.0 * newt_d), (w, gpu_d, newt_d)
        checked += 1
    eng.free(slots)
    assert not (st & 0x3).any(), st
    assert checked >= 12 and rows > 300, (checked, rows)
    assert {1, 3, 6}.issubset(kinds) or {1, 4, 6}.issubset(kinds), kinds


def test_general_piles_batched_equal_plain_beside_other_piles(eng, settled):
    b0, q0, v0 = settled
    gen = _general(b0, M.CONE_ELLIPTIC)
    gen.qpos[:] = q0
    gen.qvel[:] = v0
    pgs = scenes.pile_batch(n_worlds=16, first_world=1200)
    nwt = M.Batch(b0.links, b0.n_links, b0.bodies, b0.n_bodies, b0.geoms, b0.n_geoms, 2e-3, (0.0, 0.0, -9.81),
                  M.SOLVER_NEWTON, 20)
    nwt.qpos[:] = q0
    nwt.qvel[:] = v0
    out = {}
    for mode in (STEP_PLAIN, STEP_BATCHED):
        ss = [eng.alloc(eng.upload(x)) for x in (pgs, nwt, gen)]
        for s, x in zip(ss, (pgs, nwt, gen)):
            eng.set_state(s, x.qpos, x.qvel)
        eng.step(10, mode)
        out[mode] = [eng.get_state(s, int(x.nq.sum()), int(x.nv.sum())) for s, x in zip(ss, (pgs, nwt, gen))]
        for s in ss:
            assert not (eng.status(s) & 0x3).any()
            eng.free(s)
    for (pq, pv), (bq, bv) in zip(out[STEP_PLAIN][1:], out[STEP_BATCHED][1:]):
        assert np.abs(pq - bq).max() < 1e-6 and np.abs(pv - bv).max() < 1e-5  # the same kernels in both forms
    (pq, pv), (bq, bv) = out[STEP_PLAIN][0], out[STEP_BATCHED][0]
    assert np.abs(pq - bq).max() < 1e-5 and np.abs(pv - bv).max() < 1e-4


def test_touch_on_general_piles_matches_fp64(eng, settled):
    b0, q0, v0 = settled
    b = _general(b0, M.CONE_ELLIPTIC)
    b.qpos[:] = q0
    b.qvel[:] = v0
    specs = [(A.SENSOR_TOUCH, 0, 0)]
    for k in range(0, 16, 3):
        specs.append((A.SENSOR_ACCELEROMETER, 0, k, (0.05, -0.02, 0.03)))
        specs.append((A.SENSOR_TOUCH, 0, k + 1))
    sens = A.sensors(*specs)
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, b.qpos, b.qvel)
    eng.step(1, STEP_PLAIN)
    got = eng.read_sensors(slots, sens)
    eng.free(slots)
    touch = np.array([k == A.SENSOR_TOUCH for k in sens["kind"] for _ in range(1 if k == A.SENSOR_TOUCH else 3)])
    checked = 0
    for w in range(len(b)):
        qp, qv = _world(b, w)
        _, rd = oracle_py.contacts(b, w, qp, qv)
        if len(rd) and (np.abs(rd[:, 6]) < MARGIN_BAND).any():
            continue
        r64, _, _ = oracle_py.contact_sensors(b, w, qp, qv, sens, precision=1)
        r32, _, _ = oracle_py.contact_sensors(b, w, qp, qv, sens, precision=0)
        for part in (touch, ~touch):
            scale = max(np.abs(r64[part]).max(), 1.0)
            gpu = np.abs(got[w][part] - r64[part]).max()
            newt = np.abs(r32[part] - r64[part]).max()
            assert gpu <= max(1e-3 * scale, 2.0 * newt), (w, part.sum(), gpu, newt, scale)
        checked += 1
    assert checked >= 8, checked
    assert got[:, 0].min() > 0.0


def _refused(eng, w):
    with pytest.raises(A.NewtError):
        eng.upload(M.PackedModels([w]))


def test_refusals(eng):
    w, _, _ = incline(22.0, 0.5, M.CONE_PYRAMIDAL, condim=2)
    _refused(eng, w)
    w, _, _ = incline(22.0, 0.5, M.CONE_ELLIPTIC)
    w.solver = M.SOLVER_NEWTON
    _refused(eng, w)  # solver.rs:89-91: Newton takes the pyramidal cone
    w, _, _ = incline(22.0, 0.5, M.CONE_PYRAMIDAL, condim=4)
    w.solver = M.SOLVER_NEWTON
    _refused(eng, w)
    # the allocation-free step takes facet-row piles only (a fresh context:
    # no other group to refuse first)
    e2 = Engine(device=0)
    w, q, v = incline(22.0, 0.5, M.CONE_ELLIPTIC)
    slots = e2.alloc(e2.upload(M.PackedModels([w])))
    e2.set_state(slots, q, v)
    with pytest.raises(A.NewtError, match="elliptic"):
        e2.step_static(1)
    e2.close()
