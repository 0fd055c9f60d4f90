"""newt's stack.json loaded by the JSON-subset loader and stepped on the GPU
with PGS (the file keeps newt's default penalty contacts, which the GPU path
does not have) under its own RK4: the run turns chaotic at the first impacts
(f32 and FP64 oracles drift 8 cm apart by step 100), so each GPU step is held
to the f32 oracle's step from the same state at steps 0, 100, 200 and 400:
within 2e-6 m and 2e-4 m/s."""
import numpy as np
import pytest

import oracle_py
from test_json_model import _path
from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN
from tooling_gb300 import model as M
from tooling_gb300.json_model import load_json

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from tooling_gb300 import build as B
    B.build()
    e = Engine(device=0)
    yield e
    e.close()


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
def test_stack_json_one_step_parity(eng, mode):
    s = load_json(_path("stack"))
    s.model.solver, s.model.iterations = M.SOLVER_PGS, 30
    P = M.PackedModels([s.model])
    ids = eng.upload(P)
    for n in (0, 100, 200, 400):
        q, v = oracle_py.run(P, np.zeros(1, np.int32), s.qpos0, s.qvel0, None, n, precision=0, integrator=0)
        q, v = q.astype(np.float32), v.astype(np.float32)
        slots = eng.alloc(ids)
        eng.set_state(slots, q, v)
        eng.step(1, mode)
        gq, gv = eng.get_state(slots, 21, 18)
        eng.free(slots)
        rq, rv = oracle_py.run(P, np.zeros(1, np.int32), q, v, None, 1, precision=0, integrator=0)
        assert np.abs(gq - rq).max() < 2e-6 and np.abs(gv - rv).max() < 2e-4, (n, np.abs(gq - rq).max(),
                                                                               np.abs(gv - rv).max())
