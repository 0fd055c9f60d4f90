"""GPU parity for contact-free trees (chain workload) through the C ABI.

Tolerances: one-step qacc relative error <= 1e-4 against the FP64 oracle;
trajectories compared in MuJoCo layout."""
import numpy as np
import pytest

import oracle_py
from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN, scenes

pytestmark = pytest.mark.gpu

QACC_RTOL = 1e-4


@pytest.fixture(scope="module")
def eng():
    from tooling_gb300 import build as B
    B.build()
    e = Engine(device=0)
    yield e
    e.close()


def _load(eng, b):
    ids = eng.upload(b)
    slots = eng.alloc(ids)
    eng.set_state(slots, b.qpos, b.qvel)
    eng.set_qfrc(slots, b.qfrc)
    return slots


def _rel(a, ref):
    return np.abs(a - ref).max() / max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
def test_chain_one_step_qacc_matches_fp64_oracle(eng, mode):
    b = scenes.chain_batch(n_worlds=256)
    slots = _load(eng, b)
    eng.step(1, mode)
    eng.sync()
    qacc = eng.get_qacc(slots, int(b.nv.sum()))
    _, _, ref = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, b.qfrc, 1, precision=1, want_qacc=True)
    per_world = [np.abs(qacc[o:o + n] - ref[o:o + n]).max() / max(1e-6, np.abs(ref[o:o + n]).max())
                 for o, n in zip(b.v_off, b.nv)]
    assert max(per_world) <= QACC_RTOL, max(per_world)
    eng.free(slots)


def test_chain_trajectory_tracks_fp64_oracle(eng):
    b = scenes.chain_batch(n_worlds=64)
    slots = _load(eng, b)
    eng.step(100, STEP_BATCHED)
    qp, qv = eng.get_state(slots, int(b.nq.sum()), int(b.nv.sum()))
    rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, b.qfrc, 100, precision=1)
    assert np.abs(qp - rq).max() < 5e-3
    assert np.abs(qv - rv).max() < 5e-2
    eng.free(slots)


def test_plain_and_batched_agree(eng):
    b = scenes.chain_batch(n_worlds=128, first_world=1000)
    s1 = _load(eng, b)
    eng.step(50, STEP_PLAIN)
    q1, v1 = eng.get_state(s1, int(b.nq.sum()), int(b.nv.sum()))
    eng.free(s1)
    s2 = _load(eng, b)
    eng.step(50, STEP_BATCHED)
    q2, v2 = eng.get_state(s2, int(b.nq.sum()), int(b.nv.sum()))
    eng.free(s2)
    assert np.abs(q1 - q2).max() < 1e-5 and np.abs(v1 - v2).max() < 1e-4


def test_frictionless_energy_drift_1000_steps(eng):
    """Undamped, unactuated chains: energy drift over 1000 semi-implicit
    Euler steps stays within the FP64 oracle's own drift plus 1e-3 relative."""
    b = scenes.chain_batch(n_worlds=32, damping=False, torque=False, first_world=77)
    slots = _load(eng, b)
    eng.step(1000, STEP_BATCHED)
    qp, qv = eng.get_state(slots, int(b.nq.sum()), int(b.nv.sum()))
    rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, b.qfrc, 1000, precision=1)
    e0 = oracle_py.energy(b, np.arange(len(b)), b.qpos, b.qvel)
    eg = oracle_py.energy(b, np.arange(len(b)), qp, qv)
    er = oracle_py.energy(b, np.arange(len(b)), rq.astype(np.float32), rv.astype(np.float32))
    scale = np.maximum(1.0, np.abs(e0))
    gpu_drift = np.abs(eg - e0) / scale
    ref_drift = np.abs(er - e0) / scale
    assert np.all(gpu_drift <= ref_drift + 1e-3), (gpu_drift.max(), ref_drift.max())
    eng.free(slots)
