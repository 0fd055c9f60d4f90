"""Free-body piles under newt's Newton solve on the GPU (pile_newton.cu),
through the C ABI, against the oracle.  The oracle's free-body Newton
(solve_free_body_newton_impulses, newt/src/solver.rs:1295-1407) is
byte-identical to newt's solver_newton_stack.bin and
solver_newton_incline.bin (tests/test_oracle_golden.py), so one step of its
f32 instantiation is newt's own step.

Bars: from each of newt's Newton snapshots, one GPU step within 2e-6 m and
2e-4 m/s of newt's (the bars of the PGS goldens); the incline and the stack
tracked to newt's snapshots at steps 50, 200 and 1000 inside the envelope of
newt's own f32 runs from nudged starts (both are chaotic under Newton); on
settled 16-body piles, the contact pairs equal, the impulses per row and the
one-step velocities no further from the FP64 oracle than twice newt's own
f32 arithmetic (and within the per-row bar and 1e-4 m/s where newt's is);
the batched form equal to the plain one, with PGS piles stepped alongside."""
import functools

import numpy as np
import pytest

import oracle_py
from test_gpu_rk4 import _mj
from test_oracle_golden import _read_f32, _solver_box_scene
from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN, scenes
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


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
@pytest.mark.parametrize("name", ["stack", "incline"])
def test_newton_one_step_from_newt_snapshots(eng, name, mode):
    w, _, _ = _solver_box_scene(name, M.SOLVER_NEWTON)
    w.integrator = M.INTEGRATOR_RK4
    nb = len(w.bodies)
    gold = _read_f32(f"solver_newton_{name}.bin").reshape(4, nb, 13)
    packed = M.PackedModels([w])
    ids = eng.upload(packed)
    for row in range(4):
        q = np.ascontiguousarray(gold[row][:, :7]).reshape(-1)
        v = np.ascontiguousarray(gold[row][:, 7:]).reshape(-1)
        slots = eng.alloc(ids)
        eng.set_state(slots, _mj(q, nb), v)
        eng.step(1, mode)
        gq, gv = eng.get_state(slots, 7 * nb, 6 * nb)
        st = int(eng.status(slots)[0])
        eng.free(slots)
        rq, rv = oracle_py.run(packed, np.zeros(1, np.int32), q, v, None, 1, precision=0, layout=1, integrator=0)
        assert not st & 0x3, (row, hex(st))
        assert np.abs(gq - _mj(rq, nb)).max() < 2e-6 and np.abs(gv - rv).max() < 2e-4, row


@functools.lru_cache(maxsize=None)
def _envelope(name, n_runs=48, nudge=1e-7, marks=(50, 200, 1000)):
    """How far newt's own f32 arithmetic (the oracle's float mirror, byte-
    identical to newt unperturbed) lands from newt's Newton snapshots when
    the start positions move by up to `nudge` m: per snapshot, the largest
    position and velocity distances over `n_runs` nudged starts."""
    w, q, v = _solver_box_scene(name, M.SOLVER_NEWTON)
    w.integrator = M.INTEGRATOR_RK4
    nb = len(w.bodies)
    gold = _read_f32(f"solver_newton_{name}.bin").reshape(4, nb, 13)
    rng = np.random.default_rng(7)
    qs = np.tile(np.asarray(q, np.float32).reshape(nb, 7), (n_runs, 1, 1))
    qs[:, :, :3] += rng.uniform(-nudge, nudge, (n_runs, nb, 3)).astype(np.float32)
    packed = M.PackedModels([w])
    qc, vc, done, env = qs.reshape(-1), np.tile(np.asarray(v, np.float32), n_runs), 0, []
    for row, n in enumerate(marks, start=1):
        qo, vo = oracle_py.run(packed, np.zeros(n_runs, np.int32), qc, vc, None, n - done, precision=0, layout=1,
                               integrator=0, n_threads=8)
        done = n
        qc, vc = qo.astype(np.float32), vo.astype(np.float32)
        env.append((float(np.abs(qc.reshape(n_runs, nb, 7) - gold[row][None, :, :7]).max()),
                     float(np.abs(vc.reshape(n_runs, nb * 6) - gold[row][:, 7:].reshape(-1)[None, :]).max())))
    return env


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
@pytest.mark.parametrize("name,qfloor,vfloor", [("incline", 5e-4, 5e-3), ("stack", 5e-2, 0.5)])
def test_newton_goldens_stay_in_newts_envelope(eng, name, qfloor, vfloor, mode):
    """Under Newton the incline's box tumbles down the slope and the stack
    topples: both are chaotic.  newt's own f32 runs from starts nudged by
    1e-7 m spread by up to 1.8 m and 13 m/s (incline) and 0.8 m and 2 m/s
    (stack) at step 1000, and by micrometres on the incline at steps 50 and
    200.  The GPU run stays within 1.25 times that spread of newt's snapshots
    at steps 50, 200 and 1000, or within the floors (the PGS goldens' bars)
    where the spread is smaller."""
    w, q, v = _solver_box_scene(name, M.SOLVER_NEWTON)
    w.integrator = M.INTEGRATOR_RK4
    nb = len(w.bodies)
    gold = _read_f32(f"solver_newton_{name}.bin").reshape(4, nb, 13)
    slots = eng.alloc(eng.upload(M.PackedModels([w])))
    eng.set_state(slots, _mj(q, nb), v)
    done, errs = 0, []
    for row, n in enumerate((50, 200, 1000), start=1):
        eng.step(n - done, mode)
        done = n
        gq, gv = eng.get_state(slots, 7 * nb, 6 * nb)
        errs.append((float(np.abs(gq - _mj(gold[row][:, :7], nb)).max()),
                     float(np.abs(gv - gold[row][:, 7:].reshape(-1)).max())))
    assert not (eng.status(slots) & 0x7).any()
    eng.free(slots)
    env = _envelope(name)
    for (dq, dv), (eq, ev) in zip(errs, env):
        assert dq <= max(qfloor, 1.25 * eq) and dv <= max(vfloor, 1.25 * ev), (errs, env)


@pytest.fixture(scope="module")
def newton_piles():
    """16-body pile worlds settled by 300 FP64 PGS steps, then given newt's
    Newton solve (20 iterations)."""
    b = scenes.pile_batch(n_worlds=16, first_world=900)
    rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, None, 300, precision=1)
    nw = M.Batch(b.links, b.n_links, b.bodies, b.n_bodies, b.geoms, b.n_geoms, 2e-3, (0.0, 0.0, -9.81),
                 M.SOLVER_NEWTON, 20)
    nw.qpos[:] = rq.astype(np.float32)
    nw.qvel[:] = rv.astype(np.float32)
    return nw


def _world(b, w):
    return (b.qpos[b.q_off[w]:b.q_off[w] + b.nq[w]], b.qvel[b.v_off[w]:b.v_off[w] + b.nv[w]])


def test_newton_pile_impulses_and_step_match_fp64(eng, newton_piles):
    b = newton_piles
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, b.qpos, b.qvel)
    eng.step(1, STEP_PLAIN)
    _, gv_all = eng.get_state(slots, int(b.nq.sum()), int(b.nv.sum()))
    st = eng.status(slots)
    rows, checked = 0, 0
    for w in range(len(b)):
        qp, qv = _world(b, w)
        rp, rd = oracle_py.contacts(b, w, qp, qv)
        if len(rd) and (np.abs(rd[:, 6]) < MARGIN_BAND).any():
            continue
        gp, _ = eng.contacts(int(slots[w]))
        assert gp.tolist() == rp.tolist(), f"world {w}"
        ref = oracle_py.impulses(b, w, qp, qv, precision=1)
        f32 = oracle_py.impulses(b, w, qp, qv, precision=0)
        active = rd[:, 6] > 0 if len(rd) else np.zeros(0, bool)
        g = eng.impulses(int(slots[w])).reshape(-1, 4)[active].reshape(-1)
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
    assert not (st & 0x3).any(), st
    assert checked >= 12 and rows > 300, (checked, rows)
    eng.free(slots)


def test_newton_piles_batched_equal_plain_beside_pgs_piles(eng, newton_piles):
    """A context holding PGS piles and Newton piles: 10 batched env-steps
    (PGS piles in the persistent launch, Newton piles on their own table)
    equal 10 plain ones."""
    nwt = newton_piles
    pgs = scenes.pile_batch(n_worlds=16, first_world=1200)
    out = {}
    for mode in (STEP_PLAIN, STEP_BATCHED):
        s1 = eng.alloc(eng.upload(pgs))
        s2 = eng.alloc(eng.upload(nwt))
        eng.set_state(s1, pgs.qpos, pgs.qvel)
        eng.set_state(s2, nwt.qpos, nwt.qvel)
        eng.step(10, mode)
        out[mode] = (eng.get_state(s1, int(pgs.nq.sum()), int(pgs.nv.sum())),
                     eng.get_state(s2, int(nwt.nq.sum()), int(nwt.nv.sum())))
        assert not (eng.status(s2) & 0x3).any()
        eng.free(s1)
        eng.free(s2)
    (pq, pv), (nq, nv) = out[STEP_PLAIN]
    (bq, bv), (mq, mv) = out[STEP_BATCHED]
    assert np.abs(nq - mq).max() < 1e-6 and np.abs(nv - mv).max() < 1e-5  # the same kernels in both forms
    assert np.abs(pq - bq).max() < 1e-5 and np.abs(pv - bv).max() < 1e-4
