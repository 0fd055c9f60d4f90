"""GPU parity for free-body contact worlds (pile workload) through the C ABI.

Bars (stated here, checked below):
  * contact pair lists identical to the FP64 oracle's wherever no
    penetration lies within 1e-6 of the margin (ties at the activation
    threshold may legitimately flip);
  * PGS row impulses at equal iteration counts within 1e-3 of each row's own
    FP64 value plus an absolute floor of 2e-5 of the world's largest impulse
    (newt's own f32 arithmetic, the oracle's float mirror, stays within
    1e-3 |row| + 1e-5 max on these worlds), for every solver path: the plain
    form's island-class kernels, the batched form's world-persistent kernel
    (one and two worlds per warp) and the batched island-class pipeline;
  * every launch shape of the world-persistent kernel bit-identical;
  * short-horizon trajectories within 1e-3 m / 1e-2 m/s.
"""
import numpy as np
import pytest

import oracle_py
from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN, scenes

pytestmark = pytest.mark.gpu

IMPULSE_RTOL = 1e-3
IMPULSE_FLOOR = 2e-5  # of the world's largest impulse
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
    """Pile worlds advanced 300 steps by the FP64 oracle: a state with
    resting, stacked and sliding contacts."""
    b = scenes.pile_batch(n_worlds=48, first_world=500)
    rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, None, 300, precision=1)
    b.qpos[:] = rq.astype(np.float32)
    b.qvel[:] = rv.astype(np.float32)
    return b


def _load(eng, b):
    ids = eng.upload(b)
    slots = eng.alloc(ids)
    eng.set_state(slots, b.qpos, b.qvel)
    return slots


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
def test_contact_pair_lists_match_oracle(eng, settled, mode):
    b = settled
    slots = _load(eng, b)
    eng.step(1, mode)
    eng.sync()
    total = 0
    for w in range(len(b)):
        qp = b.qpos[b.q_off[w]:b.q_off[w] + b.nq[w]]
        qv = b.qvel[b.v_off[w]:b.v_off[w] + b.nv[w]]
        rp, rd = oracle_py.contacts(b, w, qp, qv)
        gp, gd = eng.contacts(int(slots[w]))
        near = np.abs(rd[:, 6]) < MARGIN_BAND if len(rd) else np.zeros(0, bool)
        if near.any():
            continue
        assert gp.tolist() == rp.tolist(), f"world {w}"
        if len(rd):
            assert np.abs(gd[:, 6] - rd[:, 6]).max() < 1e-4
            assert np.abs(gd[:, 3:6] - rd[:, 3:6]).max() < 1e-3
        total += len(rp)
    assert total > 100
    eng.free(slots)


@pytest.mark.parametrize("path", ["plain", "persistent", "persistent_pairs", "pipeline"])
def test_pgs_impulses_match_oracle_at_equal_iterations(eng, settled, path):
    b = settled
    slots = _load(eng, b)
    # shape 6: gangs of 12 warps, two worlds per warp
    eng.set_launch_choice(persistent=path != "pipeline", persistent_shape=6 if path == "persistent_pairs" else 2)
    try:
        eng.step(1, STEP_PLAIN if path == "plain" else STEP_BATCHED)
        eng.sync()
        if path.startswith("persistent"):
            _, fw = eng.fused_profile()
            assert fw["worlds"] == len(b) and fw["contacts"] > 0, fw
        else:
            _, work = eng.pile_profile()
            # the one-body kernels, the short multi-body kernel and the long-island
            # chain kernel all have islands to solve here
            assert (work["islands"][[0, 1, 2, 3, 5]] > 0).all(), work["islands"]
    finally:
        eng.set_launch_choice(persistent=True)
    worst, rows = 0.0, 0
    for w in range(len(b)):
        qp = b.qpos[b.q_off[w]:b.q_off[w] + b.nq[w]]
        qv = b.qvel[b.v_off[w]:b.v_off[w] + b.nv[w]]
        rp, rd = oracle_py.contacts(b, w, qp, qv)
        if len(rd) and (np.abs(rd[:, 6]) < MARGIN_BAND).any():
            continue
        ref = oracle_py.impulses(b, w, qp, qv)
        gimp = eng.impulses(int(slots[w])).reshape(-1, 4)
        active = rd[:, 6] > 0 if len(rd) else np.zeros(0, bool)
        g = gimp[active].reshape(-1)
        assert len(g) == len(ref), f"world {w}"
        if len(ref):
            tol = IMPULSE_RTOL * np.abs(ref) + IMPULSE_FLOOR * np.abs(ref).max()
            worst = max(worst, float((np.abs(g - ref) / tol).max()))
            rows += len(ref)
    assert rows > 1000
    assert worst <= 1.0, worst
    eng.free(slots)


def test_short_trajectory_tracks_oracle(eng, settled):
    b = settled
    slots = _load(eng, b)
    eng.step(20, STEP_BATCHED)
    qp, qv = eng.get_state(slots, int(b.nq.sum()), int(b.nv.sum()))
    rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, None, 20, precision=1)
    assert np.abs(qp - rq).max() < 1e-3
    assert np.abs(qv - rv).max() < 1e-2
    st = eng.status(slots)
    assert not (st & 0x5).any()  # no NaN, no contact overflow
    eng.free(slots)


def test_plain_and_batched_agree(eng, settled):
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


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
@pytest.mark.parametrize("name,qtol,vtol", [("ballistic", 3.0e-5, 8.0e-5), ("sphere_drop", 1.5e-2, 9.0e-1),
                                             ("box_stack", 2.0e-2, 5.0e-1)])
def test_free_body_scenes_within_mujoco_windows(eng, name, qtol, vtol, mode):
    """newt's matched-Euler free-body rows (differential.rs:1272-1295,
    1593-1599) run on the GPU pile path: every captured frame inside newt's
    own windows against MuJoCo 3.11.0."""
    from test_oracle_golden import _free_body_scene, read_newtdif
    from tooling_gb300 import model as M
    ref = read_newtdif(f"{name}_euler.bin")
    w, q0, v0 = _free_body_scene(name)
    if not w.geoms:  # the pile path wants one geom per body: a sphere with nothing to touch
        w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, body=0, size=(0.05, 0.0, 0.0)))
    slots = eng.alloc(eng.upload(M.PackedModels([w])))
    eng.set_state(slots, np.array(q0, np.float32), np.array(v0, np.float32))
    worst_q = worst_v = 0.0
    done = 0
    for k, step in enumerate(ref["steps"]):
        if step > done:
            eng.step(step - done, mode)
            done = step
        q, v = eng.get_state(slots, w.nq, w.nv)
        worst_q = max(worst_q, np.abs(q - ref["qpos"][k]).max())
        worst_v = max(worst_v, np.abs(v - ref["qvel"][k]).max())
    eng.free(slots)
    assert worst_q <= qtol and worst_v <= vtol, (worst_q, worst_v)


def test_persistent_shapes_agree_bit_for_bit(eng, settled):
    """Every launch shape of the world-persistent kernel (gang size, the
    barrier between assembly and sweeps, one or two worlds per warp, with
    rounds of eight or four contacts) runs the same arithmetic per world: a
    body's contacts keep their order in any round schedule.  20 batched
    env-steps from the settled state agree bit for bit across shapes."""
    from tooling_gb300 import api as A
    b = settled
    nq, nv = int(b.nq.sum()), int(b.nv.sum())
    ref, shape = None, 0
    try:
        while True:
            try:
                eng.set_launch_choice(persistent=True, persistent_shape=shape)
            except A.NewtError:
                break
            slots = _load(eng, b)
            eng.step(20, STEP_BATCHED)
            q, v = eng.get_state(slots, nq, nv)
            st = eng.status(slots)
            eng.free(slots)
            assert not (st & 0x5).any(), (shape, st)
            if ref is None:
                ref = (q, v)
            else:
                np.testing.assert_array_equal(q, ref[0], err_msg=f"shape {shape}")
                np.testing.assert_array_equal(v, ref[1], err_msg=f"shape {shape}")
            shape += 1
    finally:
        eng.set_launch_choice(persistent=True)
    assert shape >= 9, shape


def test_world_range_branches_match_plain(eng):
    """The batched island-class pipeline splits every group into world-range
    branches on their own streams; each world's arithmetic is unchanged, so
    it and the plain form agree bit for bit."""
    b = scenes.pile_batch(n_worlds=8300, first_world=9000)
    slots = _load(eng, b)
    nq, nv = int(b.nq.sum()), int(b.nv.sum())
    eng.set_launch_choice(persistent=False, pile_branches=2)
    try:
        eng.step(30, STEP_BATCHED)
    finally:
        eng.set_launch_choice(persistent=True)
    qb, vb = eng.get_state(slots, nq, nv)
    eng.set_state(slots, b.qpos, b.qvel)
    eng.step(30, STEP_PLAIN)
    qp, vp = eng.get_state(slots, nq, nv)
    eng.free(slots)
    np.testing.assert_array_equal(qb, qp)
    np.testing.assert_array_equal(vb, vp)


def test_persistent_kernel_tracks_oracle_from_the_drop(eng):
    """The world-persistent kernel over a whole horizon (one launch for 150
    env-steps: the drop, the first impacts, the settling) against the FP64
    oracle over the same horizon, on worlds where the trajectories are not
    yet chaotic: positions within 1e-3 m over 60 env-steps, and every world
    still finite and without overflow after 150."""
    b = scenes.pile_batch(n_worlds=64, first_world=3000)
    slots = _load(eng, b)
    nq, nv = int(b.nq.sum()), int(b.nv.sum())
    eng.step(60, STEP_BATCHED)
    q, v = eng.get_state(slots, nq, nv)
    rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, None, 60, precision=1)
    assert np.abs(q - rq).max() < 1e-3
    assert np.abs(v - rv).max() < 1e-2
    eng.step(90, STEP_BATCHED)
    _, fw = eng.fused_profile()
    assert fw["worlds"] == len(b) and fw["contacts"] > 0 and fw["levels"] > 0
    st = eng.status(slots)
    assert not (st & 0x5).any()
    eng.free(slots)
