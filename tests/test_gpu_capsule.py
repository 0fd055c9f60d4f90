"""GPU parity for free capsules in piles (sphere-capsule, capsule-capsule,
capsule-plane contacts) through the C ABI, against the FP64 oracle.

Bars, as for the sphere/box piles: contact pair lists identical wherever no
penetration lies within 1e-6 of the margin; PGS impulses within 1e-3
relative at equal iterations; 20-step trajectories within 1e-3 m /
1e-2 m/s.  Capsule-box pairs, which newt has no primitive for, are refused
at upload."""
import numpy as np
import pytest

import oracle_py
from tooling_gb300 import Engine, NewtError, STEP_BATCHED, STEP_PLAIN, scenes
from tooling_gb300 import model as M

pytestmark = pytest.mark.gpu

IMPULSE_RTOL = 1e-3
MARGIN_BAND = 1e-6


@pytest.fixture(scope="module")
def eng():
    from tooling_gb300 import build as B
    B.build()
    e = Engine(device=0)
    yield e
    e.close()


@pytest.fixture(scope="module")
def settled():
    b = scenes.capsule_pile_batch(n_worlds=48, first_world=40)
    rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, None, 400, precision=1)
    b.qpos[:] = rq.astype(np.float32)
    b.qvel[:] = rv.astype(np.float32)
    return b


def _load(eng, b):
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, b.qpos, b.qvel)
    return slots


def _state(b, w):
    return b.qpos[b.q_off[w]:b.q_off[w] + b.nq[w]], b.qvel[b.v_off[w]:b.v_off[w] + b.nv[w]]


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
def test_capsule_contacts_match_oracle(eng, settled, mode):
    b = settled
    slots = _load(eng, b)
    eng.step(1, mode)
    eng.sync()
    total, kinds = 0, set()
    for w in range(len(b)):
        qp, qv = _state(b, w)
        rp, rd = oracle_py.contacts(b, w, qp, qv)
        if len(rd) and (np.abs(rd[:, 6]) < MARGIN_BAND).any():
            continue
        gp, gd = eng.contacts(int(slots[w]))
        assert gp.tolist() == rp.tolist(), f"world {w}"
        if len(rd):
            assert np.abs(gd[:, 6] - rd[:, 6]).max() < 1e-4
            assert np.abs(gd[:, 3:6] - rd[:, 3:6]).max() < 1e-3
            assert np.abs(gd[:, 0:3] - rd[:, 0:3]).max() < 1e-4
        g0 = int(b.geom_off[w])
        for ga, gb in rp:
            kinds.add(tuple(sorted((int(b.geoms["shape"][g0 + ga]), int(b.geoms["shape"][g0 + gb])))))
        total += len(rp)
    assert total > 100
    assert {(M.SHAPE_PLANE, M.SHAPE_CAPSULE), (M.SHAPE_SPHERE, M.SHAPE_CAPSULE),
            (M.SHAPE_CAPSULE, M.SHAPE_CAPSULE)} <= kinds, kinds
    eng.free(slots)


def test_capsule_impulses_match_oracle(eng, settled):
    b = settled
    slots = _load(eng, b)
    eng.step(1, STEP_BATCHED)
    eng.sync()
    worst, rows = 0.0, 0
    for w in range(len(b)):
        qp, qv = _state(b, w)
        rp, rd = oracle_py.contacts(b, w, qp, qv)
        if len(rd) and (np.abs(rd[:, 6]) < MARGIN_BAND).any():
            continue
        ref = oracle_py.impulses(b, w, qp, qv)
        gimp = eng.impulses(int(slots[w])).reshape(-1, 4)
        active = rd[:, 6] > 0 if len(rd) else np.zeros(0, bool)
        g = gimp[active].reshape(-1)
        assert len(g) == len(ref), f"world {w}"
        if len(ref):
            worst = max(worst, np.abs(g - ref).max() / max(1e-9, np.abs(ref).max()))
            rows += len(ref)
    assert rows > 0 and worst <= IMPULSE_RTOL, (rows, worst)
    eng.free(slots)


def test_capsule_trajectory_tracks_oracle(eng, settled):
    b = settled
    slots = _load(eng, b)
    eng.step(20, STEP_BATCHED)
    qp, qv = eng.get_state(slots, int(b.nq.sum()), int(b.nv.sum()))
    assert not (eng.status(slots) & 0x5).any()
    eng.free(slots)
    rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, None, 20, precision=1)
    assert np.abs(qp - rq).max() < 1e-3 and np.abs(qv - rv).max() < 1e-2


def test_capsule_piles_plain_and_batched_agree(eng, settled):
    b = settled
    s1 = _load(eng, b)
    eng.step(10, STEP_PLAIN)
    q1, v1 = eng.get_state(s1, int(b.nq.sum()), int(b.nv.sum()))
    eng.free(s1)
    s2 = _load(eng, b)
    eng.step(10, STEP_BATCHED)
    q2, v2 = eng.get_state(s2, int(b.nq.sum()), int(b.nv.sum()))
    eng.free(s2)
    assert np.abs(q1 - q2).max() < 1e-5 and np.abs(v1 - v2).max() < 1e-4


def test_capsule_box_pair_is_refused(eng):
    w = M.WorldModel(dt=2e-3, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=20)
    w.add_geom(M.static_plane())
    a = w.add_body(1.0, M._diag9(0.01, 0.01, 0.01))
    c = w.add_body(1.0, M._diag9(0.01, 0.01, 0.01))
    w.add_geom(M.Geom(shape=M.SHAPE_BOX, body=a, size=(0.1, 0.1, 0.1)))
    w.add_geom(M.Geom(shape=M.SHAPE_CAPSULE, body=c, size=(0.05, 0.1, 0.0)))
    with pytest.raises(NewtError):
        eng.upload(M.PackedModels([w]))
    w.geoms[2].group, w.geoms[2].mask = 2, 2  # filtered out against the box (group 1): accepted
    w.geoms[1].group, w.geoms[1].mask = 1, 1
    eng.upload(M.PackedModels([w]))
