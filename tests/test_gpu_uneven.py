"""The uneven workload (chains and piles of 2..64 bodies in one batch): the
batched form and the plain form agree, and both track the FP64 oracle.

Bars: batched vs plain within 1e-5 m / 1e-4 m/s after 10 env-steps; a
sample of worlds within 1e-3 m / 1e-2 m/s of the oracle after 20 env-steps
(piles settle through PGS, chains free-swing)."""
import numpy as np
import pytest

import oracle_py
from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch():
    return scenes.uneven_batch(n_worlds=192, first_world=4096)


@pytest.fixture(scope="module")
def eng():
    from tooling_gb300 import build as B
    B.build()
    e = Engine(device=0)
    yield e
    e.close()


def _run(eng, b, n, mode):
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, b.qpos, b.qvel)
    eng.set_qfrc(slots, b.qfrc)
    eng.step(n, mode)
    q, v = eng.get_state(slots, int(b.nq.sum()), int(b.nv.sum()))
    st = eng.status(slots)
    eng.free(slots)
    return q, v, st


def test_batch_mixes_sizes_and_kinds(batch):
    chains = batch.n_links > 0
    assert chains.any() and (~chains).any()
    sizes = np.where(chains, batch.n_links - 1, batch.n_bodies)
    assert sizes.min() >= 2 and sizes.max() <= 64 and len(np.unique(sizes)) > 20


def test_batched_and_plain_agree(eng, batch):
    q1, v1, s1 = _run(eng, batch, 10, STEP_PLAIN)
    q2, v2, s2 = _run(eng, batch, 10, STEP_BATCHED)
    assert not (s1 & 0x1).any() and not (s2 & 0x1).any()
    assert np.abs(q1 - q2).max() < 1e-5 and np.abs(v1 - v2).max() < 1e-4


def test_tracks_fp64_oracle(eng, batch):
    q, v, _ = _run(eng, batch, 20, STEP_BATCHED)
    rq, rv = oracle_py.run(batch, np.arange(len(batch)), batch.qpos, batch.qvel, batch.qfrc, 20, precision=1)
    assert np.abs(q - rq).max() < 1e-3
    assert np.abs(v - rv).max() < 1e-2


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
def test_status_reports_blow_up_right_after_the_step(eng, mode):
    """A 56-link chain of the workload diverges near step 125 at dt 2e-3 (the
    FP64 oracle does too); the status word must say so when read straight
    after the step call, with no state read in between."""
    b = scenes.uneven_batch(n_worlds=1, first_world=6326)
    rq, _ = oracle_py.run(b, np.zeros(1, np.int32), b.qpos, b.qvel, b.qfrc, 150, precision=1)
    assert not np.isfinite(rq).all()
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, b.qpos, b.qvel)
    eng.set_qfrc(slots, b.qfrc)
    for _ in range(6):
        eng.step(25, mode)
    assert int(eng.status(slots)[0]) & 0x1
    eng.free(slots)


def test_autotune_keeps_state_and_results(eng, batch):
    """newt_gpu_autotune times the batched form's launch choices on the live
    worlds from three snapshots over a 20-env-step horizon: the worlds end
    where they began, and the chosen form still agrees with the plain one."""
    slots = eng.alloc(eng.upload(batch))
    eng.set_state(slots, batch.qpos, batch.qvel)
    eng.set_qfrc(slots, batch.qfrc)
    nq, nv = int(batch.nq.sum()), int(batch.nv.sum())
    q0, v0 = eng.get_state(slots, nq, nv)
    choice = eng.autotune(5, horizon=20)
    q1, v1 = eng.get_state(slots, nq, nv)
    np.testing.assert_array_equal(q0, q1)
    np.testing.assert_array_equal(v0, v1)
    assert choice["pile_persistent"] or choice["pile_branches"] in (1, 2, 3)
    assert choice["tree_grid_pct"] in (50, 100)
    eng.step(10, STEP_BATCHED)
    qb, vb = eng.get_state(slots, nq, nv)
    eng.set_state(slots, q0, v0)
    eng.step(10, STEP_PLAIN)
    qp, vp = eng.get_state(slots, nq, nv)
    eng.free(slots)
    assert np.abs(qb - qp).max() < 1e-5 and np.abs(vb - vp).max() < 1e-4
