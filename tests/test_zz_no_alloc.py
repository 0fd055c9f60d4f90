"""Allocation-free step (newt_gpu_step_static) against the plain step.

newt_gpu_step_static runs the plain step's kernels with the pile solver's
scratch in a fixed device array instead of cudaMalloc'd buffers.  Bars:
  * two calls in a row each land within the plain-vs-batched tolerance of
    newt_gpu_step(PLAIN) from the same state (1e-5 m, 1e-4 m/s), for pile
    worlds and chain worlds stepped in one context;
  * a context whose pile worlds need more than NEWT_STATIC_SCRATCH_BYTES is
    refused with NEWT_E_NOMEM before anything runs;
  * stepping allocates nothing: after the first call (the per-device setup),
    the device's free memory (cudaMemGetInfo) is the same before and after
    further calls on a context whose worlds were just placed.
The file name sorts last so the test also runs after every other GPU test.
"""
import numpy as np
import pytest

from tooling_gb300 import Engine, STEP_PLAIN, scenes
from tooling_gb300.api import NewtError

pytestmark = pytest.mark.gpu

QPOS_ATOL = 1e-5
QVEL_ATOL = 1e-4
NEWT_E_NOMEM = 7


@pytest.fixture(scope="module")
def built():
    from tooling_gb300 import build as B
    B.build()


def _load(eng, batches):
    out = []
    for b in batches:
        ids = eng.upload(b)
        slots = eng.alloc(ids)
        eng.set_state(slots, b.qpos, b.qvel)
        out.append(slots)
    return out


def _state(eng, batches, slots):
    qs, vs = [], []
    for b, s in zip(batches, slots):
        q, v = eng.get_state(s, int(b.nq.sum()), int(b.nv.sum()))
        qs.append(q)
        vs.append(v)
    return np.concatenate(qs), np.concatenate(vs)


def test_static_step_matches_plain_on_two_calls(built):
    batches = [scenes.pile_batch(n_worlds=48, first_world=700), scenes.chain_batch(n_worlds=64, first_world=900)]
    ref, eng = Engine(device=0), Engine(device=0)
    try:
        rs, es = _load(ref, batches), _load(eng, batches)
        before = eng.launch_count()
        for n in (150, 10):  # the first call lands bodies on the plane, the second steps resting contacts
            ref.step(n, STEP_PLAIN)
            eng.step_static(n)
            q1, v1 = _state(ref, batches, rs)
            q2, v2 = _state(eng, batches, es)
            assert np.abs(q1 - q2).max() < QPOS_ATOL
            assert np.abs(v1 - v2).max() < QVEL_ATOL
        assert eng.launch_count() > before
        assert sum(len(eng.contacts(int(s))[0]) for s in es[0]) > 0  # the contact solver ran
        assert not (eng.status(es[0]) & 0x5).any()
    finally:
        eng.close()
        ref.close()


def _device_free_bytes():
    """cudaMemGetInfo through the CUDA runtime the library already loaded."""
    import ctypes as C
    rt = C.CDLL("libcudart.so.13")
    free, total = C.c_size_t(), C.c_size_t()
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


def test_static_step_allocates_nothing(built):
    b = scenes.pile_batch(n_worlds=96, first_world=1500)
    eng = Engine(device=0)
    try:
        (slots,) = _load(eng, [b])
        eng.step_static(1)  # the first call on the device sets up
        eng.sync()
        fresh = scenes.pile_batch(n_worlds=32, first_world=1700)
        (s2,) = _load(eng, [fresh])  # new worlds, not stepped yet: a plain step would allocate scratch now
        eng.sync()
        before = _device_free_bytes()
        for n in (5, 3):
            eng.step_static(n)
            eng.sync()
        after = _device_free_bytes()
        assert after == before, (before, after)
        q, v = eng.get_state(s2, int(fresh.nq.sum()), int(fresh.nv.sum()))
        assert np.isfinite(q).all() and np.isfinite(v).all()
    finally:
        eng.close()


def test_static_step_refuses_oversize_context(built):
    b = scenes.pile_batch(n_worlds=300, first_world=1200)  # about 131 KB of scratch each: over 32 MiB
    eng = Engine(device=0)
    try:
        (slots,) = _load(eng, [b])
        q0, v0 = eng.get_state(slots, int(b.nq.sum()), int(b.nv.sum()))
        with pytest.raises(NewtError) as ei:
            eng.step_static(1)
        assert ei.value.code == NEWT_E_NOMEM
        assert "NEWT_STATIC_SCRATCH_BYTES" in str(ei.value)
        q, v = eng.get_state(slots, int(b.nq.sum()), int(b.nv.sum()))
        assert np.array_equal(q, q0) and np.array_equal(v, v0)  # nothing ran
    finally:
        eng.close()
