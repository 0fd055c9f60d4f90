"""Failure surfaces of the GPU step, each made to happen on purpose without
faulting the GPU, through the C ABI:

  * a bounded host wait that runs out: newt_gpu_sync with a 1 ms limit on a
    long step answers NEWT_E_TIMEOUT, the context stays usable, and a second
    wait drains the stream with the step's results intact;
  * a contact buffer that overflows: a context whose pile contact capacity
    is forced down to 64 (newt_gpu_opts::max_contacts) steps settled 64-body
    piles (about 100 contacts each) beside small piles; the big worlds carry
    NEWT_WS_CONTACT_OVERFLOW and keep the first 64 contacts in newt's pair
    order, the small worlds are bit-identical to an uncapped context;
  * the Newton solver's FP64 fallback: a tree whose free root weighs 1000 kg
    and whose hinged foot weighs 1e-5 kg, both touching the plane, gives a
    Hessian whose FP32 Cholesky pivot ratio exceeds 1e6; the status word
    reports NEWT_WS_FP64_FALLBACK and every row of both contacts (impulses
    8 orders of magnitude apart) matches the FP64 oracle within 1e-3 of its
    own contact's largest row.
"""
import math

import numpy as np
import pytest

import oracle_py
from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN, scenes
from tooling_gb300 import model as M
from tooling_gb300.api import NewtError

pytestmark = pytest.mark.gpu

NEWT_E_TIMEOUT = 5
WS_CONTACT_OVERFLOW, WS_FP64_FALLBACK = 0x4, 0x10
ROW_RTOL = 1e-3


@pytest.fixture(scope="module")
def built():
    from tooling_gb300 import build as B
    B.build()


def _load(eng, b):
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, b.qpos, b.qvel)
    return slots


def test_sync_times_out_then_recovers(built):
    b = scenes.pile_batch(n_worlds=8192, first_world=20000)
    eng = Engine(device=0)
    try:
        slots = _load(eng, b)
        eng.step(1, STEP_BATCHED)  # capture outside the timed wait
        eng.sync()
        eng.step(200, STEP_BATCHED)  # 8192 worlds x 200 env-steps: far longer than 1 ms
        with pytest.raises(NewtError) as ei:
            eng.sync(timeout_ms=1)
        assert ei.value.code == NEWT_E_TIMEOUT
        eng.sync()  # the second wait drains it
        q, v = eng.get_state(slots, int(b.nq.sum()), int(b.nv.sum()))
        assert np.isfinite(q).all() and np.isfinite(v).all()
        assert not (eng.status(slots) & 0x1).any()
        eng.step(1, STEP_BATCHED)  # and the context keeps stepping
        eng.sync()
    finally:
        eng.close()


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
def test_contact_overflow_is_flagged_and_isolated(built, mode):
    big = scenes.pile_batch(n_worlds=4, n_bodies=64, first_world=50)
    small = scenes.pile_batch(n_worlds=16, n_bodies=3, first_world=80)
    ref, cap = Engine(device=0), Engine(device=0, max_contacts=64)
    try:
        rs = [_load(ref, big), _load(ref, small)]
        ref.step(400, STEP_PLAIN)  # settle: every body lands on the plane
        settled = [ref.get_state(s, int(b.nq.sum()), int(b.nv.sum())) for s, b in zip(rs, (big, small))]
        cs = [cap.alloc(cap.upload(b)) for b in (big, small)]
        for c, r, (q, v) in zip(cs, rs, settled):  # both contexts start from the same host state
            cap.set_state(c, q, v)
            ref.set_state(r, q, v)
        cap.step(1, mode)
        ref.step(1, mode)
        st_big, st_small = cap.status(cs[0]), cap.status(cs[1])
        assert (st_big & WS_CONTACT_OVERFLOW).all(), st_big
        assert not (st_small & WS_CONTACT_OVERFLOW).any(), st_small
        # the big worlds keep the first 64 contacts of the pair-ordered list
        for w in range(len(big)):
            qp = settled[0][0][big.q_off[w]:big.q_off[w] + big.nq[w]]
            qv = settled[0][1][big.v_off[w]:big.v_off[w] + big.nv[w]]
            rp, _ = oracle_py.contacts(big, w, qp, qv)
            assert len(rp) > 80, len(rp)
            gp, _ = cap.contacts(int(cs[0][w]))
            assert len(gp) == 64
            assert gp.tolist() == rp[:64].tolist(), f"world {w}"
        qb, vb = cap.get_state(cs[0], int(big.nq.sum()), int(big.nv.sum()))
        assert np.isfinite(qb).all() and np.isfinite(vb).all()
        # the small worlds in the capped context: the uncapped context's result, bit for bit
        q1, v1 = cap.get_state(cs[1], int(small.nq.sum()), int(small.nv.sum()))
        q2, v2 = ref.get_state(rs[1], int(small.nq.sum()), int(small.nv.sum()))
        np.testing.assert_array_equal(q1, q2)
        np.testing.assert_array_equal(v1, v2)
    finally:
        cap.close()
        ref.close()


def _ill_conditioned(solver=M.SOLVER_NEWTON):
    """A 1000 kg free sphere resting on the plane with a 1e-5 kg sphere
    hinged to it, also touching the plane."""
    w = M.WorldModel(dt=0.002, gravity=(0.0, 0.0, -9.81), solver=solver, iterations=20)
    w.add_geom(M.static_plane(friction=0.6))
    m_h, m_l = 1000.0, 1e-5
    i_h, i_l = 0.4 * m_h * 0.24 ** 2, 0.4 * m_l * 0.05 ** 2
    w.push_link(M.Link(parent=-1, joint=M.JOINT_FREE, mass=m_h, inertia=M._diag9(i_h, i_h, i_h)))
    w.push_link(M.Link(parent=0, joint=M.JOINT_HINGE, axis=(0.0, 1.0, 0.0), jp_pos=(0.15, 0.0, 0.0),
                       jc_pos=(-0.2, 0.0, 0.0), mass=m_l, inertia=M._diag9(i_l, i_l, i_l)))
    w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, link=0, size=(0.24, 0.0, 0.0), friction=0.6))
    w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, link=1, size=(0.05, 0.0, 0.0), friction=0.6))
    # root 0.5 mm into the plane; the hinge angle puts the foot's centre 0.19 m below the hinge
    qpos = np.array([0.0, 0.0, 0.2395, 1.0, 0.0, 0.0, 0.0, math.asin(0.19 / 0.2)], np.float32)
    return M.PackedModels([w]), qpos, np.zeros(7, np.float32)


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
def test_newton_fp64_fallback_matches_oracle(built, mode):
    packed, qpos, qvel = _ill_conditioned()
    rp, _ = oracle_py.contacts(packed, 0, qpos, qvel)
    assert len(rp) == 2  # root-plane and foot-plane
    ref, _ = oracle_py.tree_impulses(packed, 0, qpos, qvel, None, precision=1)
    ref = ref.reshape(2, 4)
    assert ref[0].max() / ref[1].max() > 1e6  # rows of very different scale
    eng = Engine(device=0)
    try:
        slots = eng.alloc(eng.upload(packed))
        eng.set_state(slots, qpos, qvel)
        eng.step(1, mode)
        st = int(eng.status(slots)[0])
        assert st & WS_FP64_FALLBACK, hex(st)
        assert not st & 0x3, hex(st)  # finite, factorised
        g = eng.impulses(int(slots[0])).reshape(2, 4)
        for c in range(2):
            err = np.abs(g[c] - ref[c]) / np.abs(ref[c]).max()
            assert err.max() <= ROW_RTOL, (c, g[c], ref[c])
    finally:
        eng.close()
