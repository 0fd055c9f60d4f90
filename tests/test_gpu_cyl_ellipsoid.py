"""GPU parity for cylinder and ellipsoid geoms against planes
(newt/src/contact.rs:1296-1426) through the C ABI, against the FP64 oracle:
free bodies in a pile whose body pairs are filtered out (group/mask), and the
links of a tree on the tree-contact path.  Bars as for the other piles:
contact lists identical away from the activation threshold, 20-step
trajectories within 1e-3 m / 1e-2 m/s.  Spheres dropped on ellipsoids
(sphere-ellipsoid, contact.rs:1630-1725, the oracle pinned to newt's anchors
in tests/test_oracle_cyl_ellipsoid.py): the same bars.  A cylinder or
ellipsoid body left free to touch a body other than a sphere is refused at
upload."""
import numpy as np
import pytest

import oracle_py
from test_oracle_golden import _tree_chain_contact
from tooling_gb300 import Engine, NewtError, STEP_BATCHED, STEP_PLAIN
from tooling_gb300 import model as M

pytestmark = pytest.mark.gpu

MARGIN_BAND = 1e-6


@pytest.fixture(scope="module")
def eng():
    from tooling_gb300 import build as B
    B.build()
    e = Engine(device=0)
    yield e
    e.close()


def _round_pile(seed, n=8):
    """n cylinders and ellipsoids dropped on a plane; bodies collide with the
    plane only (body geoms group 2 / mask 1, plane group 1 / mask 2)."""
    rng = np.random.default_rng(seed)
    w = M.WorldModel(dt=2e-3, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=50)
    plane = M.static_plane(friction=0.8)
    plane.group, plane.mask = 1, 2
    w.add_geom(plane)
    qpos = []
    for k in range(n):
        if k % 2 == 0:
            r, h = rng.uniform(0.05, 0.15), rng.uniform(0.05, 0.2)
            m = float(np.float32(1000.0 * np.pi * r * r * 2 * h))
            b = w.add_body(m, M.solid_cylinder_inertia(m, r, h))
            g = M.Geom(shape=M.SHAPE_CYLINDER, body=b, size=(r, h, 0.0), friction=float(rng.uniform(0.4, 1.0)))
        else:
            ax = rng.uniform(0.05, 0.2, 3)
            m = float(np.float32(1000.0 * 4.0 / 3.0 * np.pi * ax.prod()))
            b = w.add_body(m, M.solid_ellipsoid_inertia(m, ax))
            g = M.Geom(shape=M.SHAPE_ELLIPSOID, body=b, size=tuple(float(x) for x in ax),
                       friction=float(rng.uniform(0.4, 1.0)))
        g.group, g.mask = 2, 1
        w.add_geom(g)
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        qpos += [float(rng.uniform(-1.5, 1.5)), float(rng.uniform(-1.5, 1.5)), float(rng.uniform(0.3, 0.8))] + list(q)
    return w, np.array(qpos, np.float32), np.zeros(6 * n, np.float32)


@pytest.fixture(scope="module")
def settled_pile():
    worlds, qs, vs = [], [], []
    for s in range(16):
        w, q, v = _round_pile(100 + s)
        P = M.PackedModels([w])
        rq, rv = oracle_py.run(P, np.zeros(1, np.int32), q, v, None, 250, precision=1)
        worlds.append(w)
        qs.append(rq.astype(np.float32))
        vs.append(rv.astype(np.float32))
    return M.PackedModels(worlds), np.concatenate(qs), np.concatenate(vs), worlds


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
def test_round_pile_contacts_match_oracle(eng, settled_pile, mode):
    P, q, v, worlds = settled_pile
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q, v)
    eng.step(1, mode)
    eng.sync()
    nq, nv = 7 * 8, 6 * 8
    total, shapes = 0, set()
    for w in range(len(slots)):
        qp, qv = q[w * nq:(w + 1) * nq], v[w * nv:(w + 1) * nv]
        rp, rd = oracle_py.contacts(P, w, qp, qv)
        if len(rd) and (np.abs(rd[:, 6]) < MARGIN_BAND).any():
            continue
        gp, gd = eng.contacts(int(slots[w]))
        assert gp.tolist() == rp.tolist(), f"world {w}"
        if len(rd):
            assert np.abs(gd[:, 6] - rd[:, 6]).max() < 1e-4
            assert np.abs(gd[:, 0:6] - rd[:, 0:6]).max() < 1e-4
        shapes |= {worlds[w].geoms[int(gb)].shape for _, gb in rp}
        total += len(rp)
    eng.free(slots)
    assert total > 100 and {M.SHAPE_CYLINDER, M.SHAPE_ELLIPSOID} <= shapes


def test_round_pile_trajectory_tracks_oracle(eng, settled_pile):
    P, q, v, _ = settled_pile
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q, v)
    eng.step(20, STEP_BATCHED)
    gq, gv = eng.get_state(slots, len(q), len(v))
    assert not (eng.status(slots) & 0x5).any()
    eng.free(slots)
    rq, rv = oracle_py.run(P, np.arange(len(slots)), q, v, None, 20, precision=1)
    assert np.abs(gq - rq).max() < 1e-3 and np.abs(gv - rv).max() < 1e-2


@pytest.mark.parametrize("solver", [M.SOLVER_NEWTON, M.SOLVER_PGS])
def test_tree_with_cylinder_and_ellipsoid_links(eng, solver):
    """newt's tree-chain contact scene with a cylinder root geom and an
    ellipsoid child geom: 300 oracle steps to land, then 20 GPU steps
    against 20 oracle steps."""
    w = _tree_chain_contact(solver)
    w.geoms[1] = M.Geom(shape=M.SHAPE_CYLINDER, link=0, size=(0.22, 0.12, 0.0), friction=0.6)
    w.geoms[2] = M.Geom(shape=M.SHAPE_ELLIPSOID, link=1, size=(0.12, 0.16, 0.2), friction=0.6)
    P = M.PackedModels([w])
    q0 = np.array([0.0, 0.0, 1.35, 0.9950042, 0.0998334, 0.0, 0.0, 0.3], np.float32)
    v0 = np.array([0.2, 0.0, 0.0, 0.0, 0.4, 0.0, 1.0], np.float32)
    rq, rv = oracle_py.run(P, np.zeros(1, np.int32), q0, v0, None, 300, precision=1)
    q, v = rq.astype(np.float32), rv.astype(np.float32)
    pairs, _ = oracle_py.contacts(P, 0, q, v)
    assert len(pairs) > 0
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q, v)
    eng.step(20, STEP_BATCHED)
    gq, gv = eng.get_state(slots, 8, 7)
    assert not (eng.status(slots) & 0x7).any()
    eng.free(slots)
    oq, ov = oracle_py.run(P, np.zeros(1, np.int32), q, v, None, 20, precision=1)
    assert np.abs(gq - oq).max() < 1e-3 and np.abs(gv - ov).max() < 1e-2


def _sphere_cylinder_pile(seed, n=10):
    """spheres and cylinders on a plane; cylinder pairs filtered (cylinder
    geoms group 2 / mask 5, spheres group 1, plane group 4)."""
    rng = np.random.default_rng(seed)
    w = M.WorldModel(dt=2e-3, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=50)
    plane = M.static_plane(friction=0.8)
    plane.group, plane.mask = 4, 0xFF
    w.add_geom(plane)
    qpos = []
    for k in range(n):
        if k % 2 == 0:
            r, h = rng.uniform(0.08, 0.2), rng.uniform(0.05, 0.2)
            m = float(np.float32(1000.0 * np.pi * r * r * 2 * h))
            b = w.add_body(m, M.solid_cylinder_inertia(m, r, h))
            g = M.Geom(shape=M.SHAPE_CYLINDER, body=b, size=(r, h, 0.0), friction=0.7)
            g.group, g.mask = 2, 5
        else:
            r = rng.uniform(0.05, 0.15)
            m = float(np.float32(1000.0 * 4.0 / 3.0 * np.pi * r ** 3))
            b = w.add_body(m, M.solid_sphere_inertia(m, r))
            g = M.Geom(shape=M.SHAPE_SPHERE, body=b, size=(r, 0.0, 0.0), friction=0.7)
            g.group, g.mask = 1, 0xFF
        w.add_geom(g)
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        qpos += [float(rng.uniform(-0.5, 0.5)), float(rng.uniform(-0.5, 0.5)), float(0.3 + 0.35 * k)] + list(q)
    return w, np.array(qpos, np.float32), np.zeros(6 * n, np.float32)


def test_sphere_cylinder_pile_matches_oracle(eng):
    """contact.rs:1519-1628 on the pile path: 300 oracle steps of spheres
    falling onto cylinders, then contact lists and 20 GPU steps against the
    oracle."""
    worlds, qs, vs = [], [], []
    for s in range(12):
        w, q, v = _sphere_cylinder_pile(200 + s)
        rq, rv = oracle_py.run(M.PackedModels([w]), np.zeros(1, np.int32), q, v, None, 300, precision=1)
        worlds.append(w)
        qs.append(rq.astype(np.float32))
        vs.append(rv.astype(np.float32))
    P, q, v = M.PackedModels(worlds), np.concatenate(qs), np.concatenate(vs)
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q, v)
    eng.step(1, STEP_BATCHED)
    eng.sync()
    nq, nv, kinds = 70, 60, 0
    for w in range(len(worlds)):
        qp, qv = q[w * nq:(w + 1) * nq], v[w * nv:(w + 1) * nv]
        rp, rd = oracle_py.contacts(P, w, qp, qv)
        if len(rd) and (np.abs(rd[:, 6]) < MARGIN_BAND).any():
            continue
        gp, gd = eng.contacts(int(slots[w]))
        assert gp.tolist() == rp.tolist(), f"world {w}"
        if len(rd):
            assert np.abs(gd[:, 0:7] - rd[:, 0:7]).max() < 1e-4
        kinds += sum(1 for a, b in rp if {worlds[w].geoms[a].shape, worlds[w].geoms[b].shape}
                     == {M.SHAPE_SPHERE, M.SHAPE_CYLINDER})
    eng.free(slots)
    assert kinds > 5
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q, v)
    eng.step(20, STEP_BATCHED)
    gq, gv = eng.get_state(slots, len(q), len(v))
    eng.free(slots)
    rq, rv = oracle_py.run(P, np.arange(len(worlds)), q, v, None, 20, precision=1)
    assert np.abs(gq - rq).max() < 1e-3 and np.abs(gv - rv).max() < 1e-2


def test_unfiltered_cylinder_body_pair_is_refused(eng):
    w = M.WorldModel(dt=2e-3, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=20)
    w.add_geom(M.static_plane())
    a = w.add_body(1.0, M._diag9(0.01, 0.01, 0.01))
    c = w.add_body(1.0, M._diag9(0.01, 0.01, 0.01))
    w.add_geom(M.Geom(shape=M.SHAPE_BOX, body=a, size=(0.1, 0.1, 0.1)))
    w.add_geom(M.Geom(shape=M.SHAPE_CYLINDER, body=c, size=(0.05, 0.1, 0.0)))
    with pytest.raises(NewtError):
        eng.upload(M.PackedModels([w]))


def _sphere_on_ellipsoid_pile(seed):
    """Two ellipsoids lying on a plane and six spheres dropped onto them;
    ellipsoid-ellipsoid pairs filtered out (ellipsoids group 2 / mask 5,
    spheres group 4 / mask 7, plane group 1 / mask 6)."""
    rng = np.random.default_rng(seed)
    w = M.WorldModel(dt=2e-3, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=50)
    plane = M.static_plane(friction=0.8)
    plane.group, plane.mask = 1, 6
    w.add_geom(plane)
    qpos = []
    for k in range(2):
        ax = np.array([rng.uniform(0.2, 0.3), rng.uniform(0.12, 0.2), rng.uniform(0.08, 0.12)])
        m = float(np.float32(1000.0 * 4.0 / 3.0 * np.pi * ax.prod()))
        b = w.add_body(m, M.solid_ellipsoid_inertia(m, ax))
        g = M.Geom(shape=M.SHAPE_ELLIPSOID, body=b, size=tuple(float(x) for x in ax), friction=0.7)
        g.group, g.mask = 2, 5
        w.add_geom(g)
        yaw = rng.uniform(0.0, np.pi)
        qpos += [0.35 * (2 * k - 1), 0.0, float(ax[2]) + 0.01, np.cos(yaw / 2), 0.0, 0.0, np.sin(yaw / 2)]
    for k in range(6):
        r = rng.uniform(0.04, 0.08)
        m = float(np.float32(1000.0 * 4.0 / 3.0 * np.pi * r ** 3))
        b = w.add_body(m, M.solid_sphere_inertia(m, r))
        g = M.Geom(shape=M.SHAPE_SPHERE, body=b, size=(r, 0.0, 0.0), friction=float(rng.uniform(0.4, 1.0)))
        g.group, g.mask = 4, 7
        w.add_geom(g)
        qpos += [float(rng.uniform(-0.55, 0.55)), float(rng.uniform(-0.15, 0.15)), float(rng.uniform(0.35, 0.9)),
                 1.0, 0.0, 0.0, 0.0]
    return w, np.array(qpos, np.float32), np.zeros(6 * 8, np.float32)


@pytest.fixture(scope="module")
def ell_piles():
    """After 150 FP64 oracle steps: spheres landed on (and rolling off) the
    ellipsoids."""
    worlds, qs, vs = [], [], []
    for s in range(16):
        w, q, v = _sphere_on_ellipsoid_pile(400 + s)
        P = M.PackedModels([w])
        rq, rv = oracle_py.run(P, np.zeros(1, np.int32), q, v, None, 150, precision=1)
        worlds.append(w)
        qs.append(rq.astype(np.float32))
        vs.append(rv.astype(np.float32))
    return M.PackedModels(worlds), np.concatenate(qs), np.concatenate(vs), worlds


@pytest.mark.parametrize("mode", [STEP_PLAIN, STEP_BATCHED])
def test_sphere_ellipsoid_contacts_match_oracle(eng, ell_piles, mode):
    P, q, v, worlds = ell_piles
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q, v)
    eng.step(1, mode)
    eng.sync()
    nq, nv = 7 * 8, 6 * 8
    sph_ell = 0
    for w in range(len(slots)):
        qp, qv = q[w * nq:(w + 1) * nq], v[w * nv:(w + 1) * nv]
        rp, rd = oracle_py.contacts(P, w, qp, qv)
        if len(rd) and (np.abs(rd[:, 6]) < MARGIN_BAND).any():
            continue
        gp, gd = eng.contacts(int(slots[w]))
        assert gp.tolist() == rp.tolist(), f"world {w}"
        if len(rd):
            assert np.abs(gd[:, 6] - rd[:, 6]).max() < 1e-4
            assert np.abs(gd[:, 0:6] - rd[:, 0:6]).max() < 1e-4
        shp = [w_.shape for w_ in worlds[w].geoms]
        sph_ell += sum(1 for a, b in rp if {shp[a], shp[b]} == {M.SHAPE_SPHERE, M.SHAPE_ELLIPSOID})
    eng.free(slots)
    assert sph_ell >= 8, sph_ell


def test_sphere_ellipsoid_trajectory_tracks_oracle(eng, ell_piles):
    P, q, v, _ = ell_piles
    slots = eng.alloc(eng.upload(P))
    eng.set_state(slots, q, v)
    eng.step(20, STEP_BATCHED)
    gq, gv = eng.get_state(slots, len(q), len(v))
    assert not (eng.status(slots) & 0x5).any()
    eng.free(slots)
    rq, rv = oracle_py.run(P, np.arange(len(slots)), q, v, None, 20, precision=1)
    assert np.abs(gq - rq).max() < 1e-3 and np.abs(gv - rv).max() < 1e-2


def test_unfiltered_ellipsoid_pair_is_refused(eng):
    w = M.WorldModel(dt=2e-3, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=20)
    w.add_geom(M.static_plane())
    for _ in range(2):
        b = w.add_body(1.0, M._diag9(0.01, 0.01, 0.01))
        w.add_geom(M.Geom(shape=M.SHAPE_ELLIPSOID, body=b, size=(0.1, 0.08, 0.05)))
    with pytest.raises(NewtError):
        eng.upload(M.PackedModels([w]))
