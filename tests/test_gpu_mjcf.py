"""newt's reference MJCF scenes, loaded by the MJCF-subset loader and stepped
on the GPU through the C ABI: every captured frame inside newt's own
matched-Euler windows against MuJoCo 3.11.0 (newt/tests/differential.rs)."""
import numpy as np
import pytest

from test_mjcf import _xml
from test_oracle_golden import read_newtdif
from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN
from tooling_gb300 import model as M
from tooling_gb300.mjcf import load_mjcf

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from tooling_gb300 import build as B
    B.build()
    e = Engine(device=0)
    yield e
    e.close()


def _run(eng, model, ref, mode):
    model.integrator = M.INTEGRATOR_EULER  # newt's matched rows step Euler (differential.rs:1272-1295)
    slots = eng.alloc(eng.upload(M.PackedModels([model])))
    eng.set_state(slots, ref["qpos"][0].astype(np.float32), ref["qvel"][0].astype(np.float32))
    worst_q = worst_v = 0.0
    done = 0
    for k, step in enumerate(ref["steps"]):
        if step > done:
            eng.step(step - done, mode)
            done = step
        q, v = eng.get_state(slots, model.nq, model.nv)
        worst_q = max(worst_q, np.abs(q - ref["qpos"][k]).max())
        worst_v = max(worst_v, np.abs(v - ref["qvel"][k]).max())
    eng.free(slots)
    return worst_q, worst_v


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
def test_box_stack_xml_on_the_pile_path(eng, mode):
    wq, wv = _run(eng, load_mjcf(_xml("box_stack")).model, read_newtdif("box_stack_euler.bin"), mode)
    assert wq <= 2.0e-2 and wv <= 5.0e-1, (wq, wv)


@pytest.mark.parametrize("solver,name,qtol,vtol", [
    (M.SOLVER_NEWTON, "tree_chain_contact_newton_euler.bin", 8.0e-2, 1.3),
    (M.SOLVER_PGS, "tree_chain_contact_pgs_euler.bin", 7.0e-2, 0.7)])
def test_tree_chain_contact_xml_on_the_tree_contact_path(eng, solver, name, qtol, vtol):
    model = load_mjcf(_xml("tree_chain_contact")).model
    model.solver = solver  # the PGS capture runs the same scene with newt's PGS mode
    wq, wv = _run(eng, model, read_newtdif(name), STEP_BATCHED)
    assert wq <= qtol and wv <= vtol, (wq, wv)
