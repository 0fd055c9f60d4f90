"""Served rollouts (newt_gpu_serve): requests of mixed kinds (hinge chains,
free-body piles, quadrupeds with contacts) join and leave a resident batch
between env-steps.  A request's result must not depend on what it was
batched with: each final state equals, bit for bit, the same rollout run
alone (one world, the same per-step controls, the same step form).

Also covered: several env-steps per tick (worlds held where their horizon
ends), slot reuse under a captured step graph, admission against a device
budget, Poisson arrivals on the wall clock, and the plain step form."""
import numpy as np
import pytest

from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def worlds():
    u = scenes.uneven_batch(n_worlds=40, first_world=12288)
    q = scenes.quadruped_batch(n_worlds=12, first_world=700)
    return u, q


@pytest.fixture(scope="module")
def eng(worlds):
    from tooling_gb300 import build as B
    B.build()
    e = Engine(device=0)
    u, q = worlds
    ids = np.concatenate([e.upload(u), e.upload(q)])
    yield e, ids
    e.close()


def _states(b):
    return [(b.qpos[b.q_off[i]:b.q_off[i] + b.nq[i]], b.qvel[b.v_off[i]:b.v_off[i] + b.nv[i]]) for i in range(len(b))]


def _requests(eng, ids, worlds, n, seed, h_lo=3, h_hi=40):
    e, _ = eng
    u, q = worlds
    init = _states(u) + _states(q)
    rng = np.random.default_rng(seed)
    pick = rng.integers(0, len(ids), n)
    hz = rng.integers(h_lo, h_hi, n)
    nv = np.array([e.dims(int(ids[k]))[1] for k in pick])
    pool = rng.standard_normal(1 << 16).astype(np.float32)
    coff = np.array([rng.integers(0, pool.size - h * v) for h, v in zip(hz, nv)])
    qp = np.concatenate([init[k][0] for k in pick])
    qv = np.concatenate([init[k][1] for k in pick])
    return ids[pick], hz, qp, qv, pool, coff, nv, [init[k] for k in pick]


def _alone(e, mid, h, q0, v0, ctrl, mode=STEP_BATCHED, chunks=None):
    """One world through the same step calls: one env-step per call with
    control row t before step t, or the given step counts per call."""
    nq, nv = e.dims(int(mid))
    s = e.alloc([mid])
    e.set_state(s, q0, v0)
    if chunks is not None:
        for c in chunks:
            e.step(c, mode)
    for t in range(h):
        if ctrl is not None:
            e.set_qfrc(s, ctrl[t * nv:(t + 1) * nv])
        e.step(1, mode)
    q, v = e.get_state(s, nq, nv)
    e.free(s)
    return q, v


def _split(e, mids, flat_q, flat_v):
    out, oq, ov = [], 0, 0
    for m in mids:
        nq, nv = e.dims(int(m))
        out.append((flat_q[oq:oq + nq], flat_v[ov:ov + nv]))
        oq += nq
        ov += nv
    return out


def _check_alone(e, mids, hz, init, pool, coff, nv, got, sample, mode=STEP_BATCHED):
    for i in sample:
        ctrl = pool[coff[i]:coff[i] + hz[i] * nv[i]]
        q, v = _alone(e, mids[i], int(hz[i]), init[i][0], init[i][1], ctrl, mode)
        np.testing.assert_array_equal(got[i][0], q, err_msg=f"request {i} qpos")
        np.testing.assert_array_equal(got[i][1], v, err_msg=f"request {i} qvel")


def test_served_results_equal_alone(eng, worlds):
    e, ids = eng
    mids, hz, qp, qv, pool, coff, nv, init = _requests(eng, ids, worlds, 60, seed=11)
    oq, ov, st, admit, done = e.serve(mids, hz, np.zeros(len(mids)), qp, qv, pool, coff, max_active=16,
                                      real_time=False)
    assert st["completed"] == len(mids) and st["peak_active"] == 16
    assert st["env_steps"] == hz.sum()
    assert (admit >= 0).all() and (done >= admit).all()
    assert e.memory()[0] > 0
    got = _split(e, mids, oq, ov)
    _check_alone(e, mids, hz, init, pool, coff, nv, got, range(len(mids)))


@pytest.mark.parametrize("k", [4, 7])
def test_multi_step_ticks_equal_alone(eng, worlds, k):
    """steps_per_tick = k: a tick queues k env-steps (each with its control
    row) without a host wait and holds every world whose horizon ends inside
    it at that env-step.  Every result still equals its rollout run alone, bit
    for bit, and the ticks fall by about k."""
    e, ids = eng
    mids, hz, qp, qv, pool, coff, nv, init = _requests(eng, ids, worlds, 60, seed=11)
    _, _, one, _, _ = e.serve(mids, hz, np.zeros(len(mids)), qp, qv, pool, coff, max_active=16, real_time=False)
    oq, ov, st, admit, done = e.serve(mids, hz, np.zeros(len(mids)), qp, qv, pool, coff, max_active=16,
                                      real_time=False, steps_per_tick=k)
    assert st["completed"] == len(mids) and st["env_steps"] == hz.sum()
    assert (admit >= 0).all() and (done >= admit).all()
    assert st["ticks"] * k >= one["ticks"] and st["ticks"] < one["ticks"] / (k / 2.0), (st["ticks"], one["ticks"])
    _check_alone(e, mids, hz, init, pool, coff, nv, _split(e, mids, oq, ov), range(len(mids)))


def test_plain_step_form(eng, worlds):
    e, ids = eng
    mids, hz, qp, qv, pool, coff, nv, init = _requests(eng, ids, worlds, 12, seed=12)
    oq, ov, st, _, _ = e.serve(mids, hz, np.zeros(len(mids)), qp, qv, pool, coff, max_active=5, real_time=False,
                               mode=STEP_PLAIN)
    assert st["completed"] == len(mids)
    _check_alone(e, mids, hz, init, pool, coff, nv, _split(e, mids, oq, ov), range(len(mids)), STEP_PLAIN)


def test_zero_horizon_returns_initial_state(eng, worlds):
    e, ids = eng
    mids, hz, qp, qv, pool, coff, nv, init = _requests(eng, ids, worlds, 6, seed=13)
    hz[::2] = 0
    oq, ov, st, _, _ = e.serve(mids, hz, np.zeros(len(mids)), qp, qv, pool, coff, real_time=False)
    assert st["completed"] == 6
    got = _split(e, mids, oq, ov)
    for i in range(0, 6, 2):
        np.testing.assert_array_equal(got[i][0], init[i][0])
        np.testing.assert_array_equal(got[i][1], init[i][1])
    _check_alone(e, mids, hz, init, pool, coff, nv, got, range(1, 6, 2))


def test_slot_reuse_keeps_captured_graph_correct(eng, worlds):
    e, ids = eng
    u, q = worlds
    init = _states(u) + _states(q)
    k = len(ids)
    slots = e.alloc(ids)
    e.set_state(slots, np.concatenate([x[0] for x in init]), np.concatenate([x[1] for x in init]))
    e.step(5, STEP_BATCHED)
    gone = np.arange(0, k, 2)
    e.free(slots[gone])
    again = e.alloc(ids[gone])  # the freed group indices come back: no group grows
    e.set_state(again, np.concatenate([init[i][0] for i in gone]), np.concatenate([init[i][1] for i in gone]))
    e.step(5, STEP_BATCHED)
    dims = [e.dims(int(m)) for m in ids]
    kept = np.arange(1, k, 2)
    qk, vk = e.get_state(slots[kept], sum(dims[i][0] for i in kept), sum(dims[i][1] for i in kept))
    qa, va = e.get_state(again, sum(dims[i][0] for i in gone), sum(dims[i][1] for i in gone))
    e.free(np.concatenate([slots[kept], again]))
    for sel, fq, fv, chunks in ((kept, qk, vk, [5, 5]), (gone, qa, va, [5])):
        got = _split(e, ids[sel], fq, fv)
        for j, i in enumerate(sel[:8]):
            q0, v0 = _alone(e, ids[i], 0, init[i][0], init[i][1], None, chunks=chunks)
            np.testing.assert_array_equal(got[j][0], q0)
            np.testing.assert_array_equal(got[j][1], v0)


def test_admission_waits_for_the_budget(worlds):
    _, q = worlds
    probe = Engine(device=0)
    pid = probe.upload(q)
    probe.alloc(pid[:1])
    per_world = probe.memory()[0] // 64  # a new group takes 64 worlds when the budget allows
    probe.close()
    e = Engine(device=0, hbm_budget_bytes=int(6.5 * per_world))
    try:
        ids = e.upload(q)
        init = _states(q)
        rng = np.random.default_rng(5)
        pick = rng.integers(0, len(ids), 20)
        hz = rng.integers(2, 12, 20)
        qp = np.concatenate([init[k][0] for k in pick])
        qv = np.concatenate([init[k][1] for k in pick])
        oq, ov, st, admit, done = e.serve(ids[pick], hz, np.zeros(20), qp, qv, real_time=False)
        assert st["completed"] == 20 and st["peak_active"] == 6
        assert e.memory()[0] <= e.memory()[1]
        got = _split(e, ids[pick], oq, ov)
        for i in range(0, 20, 4):
            q0, v0 = _alone(e, ids[pick[i]], int(hz[i]), init[pick[i]][0], init[pick[i]][1], None)
            np.testing.assert_array_equal(got[i][0], q0)
            np.testing.assert_array_equal(got[i][1], v0)
    finally:
        e.close()


def test_poisson_arrivals_on_the_wall_clock(eng, worlds):
    e, ids = eng
    n = 400
    mids, _, qp, qv, pool, coff, nv, init = _requests(eng, ids, worlds, n, seed=14)
    rng = np.random.default_rng(15)
    arrivals = np.cumsum(rng.exponential(1.0 / 2000.0, n))
    hz = np.floor(np.exp(rng.uniform(np.log(10), np.log(101), n))).astype(np.int32)
    coff = np.array([rng.integers(0, pool.size - h * v) for h, v in zip(hz, nv)])
    oq, ov, st, admit, done = e.serve(mids, hz, arrivals, qp, qv, pool, coff)
    assert st["completed"] == n and st["env_steps"] == hz.sum()
    assert (admit >= arrivals - 1e-9).all() and (done >= admit).all()
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    assert st["wall_s"] >= arrivals[-1]
    _check_alone(e, mids, hz, init, pool, coff, nv, _split(e, mids, oq, ov), range(0, n, 40))


def test_control_streams_survive_group_growth(worlds):
    """Control streams live on the device and point into their worlds' qfrc
    rows; a group that grows (and moves) between calls must not lose them:
    each env-step's qfrc equals the stream's next row, as with set_qfrc."""
    _, q = worlds
    e = Engine(device=0)
    try:
        ids = e.upload(q)
        init = _states(q)
        rng = np.random.default_rng(21)
        h = 12
        nv = q.nv[0]
        ctrl = rng.standard_normal((4, h * nv)).astype(np.float32)
        s = e.alloc(ids[:4])
        e.set_state(s, np.concatenate([init[i][0] for i in range(4)]), np.concatenate([init[i][1] for i in range(4)]))
        e.set_ctrl_stream(s, ctrl.reshape(-1), [h] * 4)
        for t in range(h):
            if t == 5:  # more worlds of the same group: it grows past its first capacity
                extra = e.alloc(np.repeat(ids[4:], 12))
            e.apply_ctrl()
            e.step(1, STEP_BATCHED)
        got = e.get_state(s, int(q.nq[:4].sum()), int(q.nv[:4].sum()))
        e.free(extra)
        e.free(s)
        for i in range(4):
            q0, v0 = _alone(e, ids[i], h, init[i][0], init[i][1], ctrl[i])
            np.testing.assert_array_equal(got[0][i * q.nq[0]:(i + 1) * q.nq[0]], q0)
            np.testing.assert_array_equal(got[1][i * nv:(i + 1) * nv], v0)
    finally:
        e.close()
