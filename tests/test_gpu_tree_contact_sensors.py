"""Contact sensors on tree-contact worlds on the GPU (newt_gpu_read_sensors:
the contact re-solve in tc_k_solve's resolve mode, then
tree_sensor_dyn_kernel and tree_sensors_kernel) against the oracle, which
holds newt's anchors (tests/test_oracle_tree_contact_sensors.py).

Each GPU reading is taken after one GPU step from a state read back from
the device; the oracle steps once from that same state and re-solves the
step's contacts at its own post-step state.

Bars: newt's anchors on the GPU (the link-attached sphere's touch = m g
within 0.8, its accelerometer +g and its free root's zero force within the
same; the gap contact's alignment); on quadrupeds under PGS and Newton with
random hip and knee torques, every touch, accelerometer, force and torque
reading no further from the FP64 oracle than twice newt's own f32 arithmetic
(the oracle's float mirror), or within 1e-3 of the reading's size (floor 1)
where newt's is closer."""
import numpy as np
import pytest

import oracle_py
from test_oracle_tree_contact_sensors import MASS, RESTING, GAP, gap_alignment_scene, resting_sphere_link
from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN, scenes
from tooling_gb300 import api as A
from tooling_gb300 import model as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    from tooling_gb300 import build as B
    B.build()
    e = Engine(device=0)
    yield e
    e.close()


def _read_after_step(eng, slots, nq, nv, sens, mode=STEP_BATCHED):
    q, v = eng.get_state(slots, nq, nv)
    eng.step(1, mode)
    return q, v, eng.read_sensors(slots, sens)


def test_resting_link_sphere_reads_mg_on_gpu(eng):
    w, q, v = resting_sphere_link()
    P = M.PackedModels([w])
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q, v)
    eng.step(799, STEP_BATCHED)
    q0, v0, got = _read_after_step(eng, slots, 7, 6, RESTING)
    eng.free(slots)
    got = got[0]
    assert abs(got[0] - MASS * 9.81) < 0.8, got
    assert np.abs(got[1:4] - np.array([0.0, 0.0, 9.81])).max() < 0.8, got
    assert np.abs(got[4:10]).max() < 0.8, got
    r64, _, _ = oracle_py.tree_contact_sensors(P, 0, q0, v0, RESTING, precision=1)
    assert np.abs(got - r64).max() < 1e-3, (got, r64)


def test_gap_contact_alignment_on_gpu(eng):
    w, q, v = gap_alignment_scene()
    P = M.PackedModels([w])
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q, v)
    eng.step(1, STEP_PLAIN)
    got = eng.read_sensors(slots, GAP)[0]
    eng.free(slots)
    r64, _, _ = oracle_py.tree_contact_sensors(P, 0, q, v, GAP, precision=1)
    assert got[0] > 1.0 and got[1] == 0.0, got
    assert abs(got[0] - r64[0]) < 1e-3 * max(1.0, abs(r64[0])), (got, r64)


def test_fresh_world_reads_no_contacts(eng):
    """A world that has not stepped since it was placed has no contacts,
    even in a slot whose previous world had some."""
    w, q, v = resting_sphere_link()
    P = M.PackedModels([w])
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q, v)
    eng.step(200, STEP_BATCHED)
    assert eng.read_sensors(slots, RESTING)[0][0] > 1.0
    eng.free(slots)
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q, v)
    assert eng.read_sensors(slots, RESTING)[0][0] == 0.0
    eng.free(slots)


# touch on the torso and every leg capsule (geoms 1-13), the torso's
# accelerometer at an offset site, the free root's net force, a thigh's and a
# shank's joint force and torque, a shank's accelerometer; two read calls (at
# most 16 sensors per call)
QUAD_TOUCH = A.sensors(*[(A.SENSOR_TOUCH, 1, g) for g in range(1, 14)])
QUAD_DYN = A.sensors((A.SENSOR_ACCELEROMETER, 1, 0, (0.05, -0.02, 0.03)), (A.SENSOR_FORCE, 1, 0),
                     (A.SENSOR_FORCE, 1, 2), (A.SENSOR_TORQUE, 1, 2), (A.SENSOR_FORCE, 1, 9), (A.SENSOR_TORQUE, 1, 9),
                     (A.SENSOR_ACCELEROMETER, 1, 12, (0.0, 0.0, -0.1)))
QUAD = np.concatenate([QUAD_TOUCH, QUAD_DYN])


@pytest.mark.parametrize("solver", [M.SOLVER_PGS, M.SOLVER_NEWTON])
def test_quadruped_contact_sensors_match_fp64(eng, solver):
    n = 24
    b = scenes.quadruped_batch(n_worlds=n, first_world=300, solver=solver)
    rng = np.random.default_rng(23)
    qfrc = np.zeros(int(b.nv.sum()), np.float32)
    for w in range(n):  # hip and knee torques; the free root's six DoFs unforced
        qfrc[b.v_off[w] + 6:b.v_off[w] + b.nv[w]] = rng.normal(0.0, 2.0, b.nv[w] - 6)
    slots = eng.alloc(eng.upload(b))
    eng.set_state(slots, b.qpos, b.qvel)
    eng.set_qfrc(slots, qfrc)
    eng.step(119, STEP_BATCHED)
    q, v, touch = _read_after_step(eng, slots, int(b.nq.sum()), int(b.nv.sum()), QUAD_TOUCH)
    got = np.concatenate([touch, eng.read_sensors(slots, QUAD_DYN)], 1)
    eng.free(slots)
    touching = 0
    for w in range(n):
        qp, qv = q[b.q_off[w]:b.q_off[w] + b.nq[w]], v[b.v_off[w]:b.v_off[w] + b.nv[w]]
        qf = qfrc[b.v_off[w]:b.v_off[w] + b.nv[w]]
        r64, _, _ = oracle_py.tree_contact_sensors(b, w, qp, qv, QUAD, precision=1, qfrc=qf)
        r32, _, _ = oracle_py.tree_contact_sensors(b, w, qp, qv, QUAD, precision=0, qfrc=qf)
        scale = np.maximum(1.0, np.abs(r64))
        gpu, newt = np.abs(got[w] - r64), np.abs(r32 - r64)
        assert (gpu <= np.maximum(1e-3 * scale, 2.0 * newt)).all(), (w, gpu, newt, r64)
        touching += int((r64[:13] > 0.0).sum())
    assert touching >= n, touching  # the legs have landed: about 50 geoms press on the plane


def test_gap_alignment_with_pair_list_on_gpu(eng):
    from test_oracle_tree_contact_sensors import gap_alignment_pair_list_scene
    w, q, v = gap_alignment_pair_list_scene()
    P = M.PackedModels([w])
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q, v)
    eng.step(1, STEP_PLAIN)
    got = eng.read_sensors(slots, GAP)[0]
    gp, _ = eng.contacts(int(slots[0]))
    eng.free(slots)
    r64, _, _ = oracle_py.tree_contact_sensors(P, 0, q, v, GAP, precision=1)
    assert got[0] > 1.0 and got[1] == 0.0, got
    assert abs(got[0] - r64[0]) < 1e-3 * max(1.0, abs(r64[0])), (got, r64)
    rp, _ = oracle_py.contacts(P, 0, q, v)
    assert np.array_equal(gp, rp), (gp, rp)  # the list's order: the gap contact first


def test_explicit_pair_list_order_on_quadrupeds(eng):
    """An explicit list naming the four shank-plane pairs in reverse order:
    the GPU's contacts come in that order, as the oracle's, and the step
    matches the FP64 oracle's within 2e-3 m and 5e-2 m/s."""
    b = scenes.quadruped_batch(n_worlds=1, first_world=300)
    rq, rv = oracle_py.run(b, np.arange(1), b.qpos, b.qvel, None, 300, precision=1)
    w = M.WorldModel(dt=2e-3, solver=M.SOLVER_PGS, iterations=20)
    for k in range(b.n_links[0]):
        L = b.links[k]
        w.push_link(M.Link(parent=int(L["parent"]), joint=int(L["joint"]), axis=tuple(L["axis"]),
                           jp_pos=tuple(L["jp_pos"]), jp_quat=tuple(L["jp_quat"]), jc_pos=tuple(L["jc_pos"]),
                           mass=float(L["mass"]), inertia=list(L["inertia"])))
    for k in range(b.n_geoms[0]):
        G = b.geoms[k]
        w.add_geom(M.Geom(shape=int(G["shape"]), link=int(G["link"]), size=tuple(G["size"]),
                          local_pos=tuple(G["local_pos"]), local_quat=tuple(G["local_quat"]),
                          friction=float(G["friction"])))
    w.pair_list = [(13, 0), (10, 0), (7, 0), (4, 0)]  # shank-plane pairs, last leg first, plane second
    P = M.PackedModels([w])
    q, v = rq.astype(np.float32), rv.astype(np.float32)
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q, v)
    eng.step(1, STEP_PLAIN)
    gp, _ = eng.contacts(int(slots[0]))
    eng.step(9, STEP_PLAIN)
    gq, gv = eng.get_state(slots, len(q), len(v))
    eng.free(slots)
    rp, _ = oracle_py.contacts(P, 0, q, v)
    assert np.array_equal(gp, rp), (gp, rp)
    oq, ov = oracle_py.run(P, np.zeros(1, np.int32), q, v, None, 10, precision=1)
    assert np.abs(gq - oq).max() < 2e-3 and np.abs(gv - ov).max() < 5e-2
