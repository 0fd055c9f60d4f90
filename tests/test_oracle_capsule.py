"""Known-answer checks of the oracle's capsule pairs (CPU only).

newt's sphere-capsule (newt/src/contact.rs:473-505) and capsule-capsule
(contact.rs:1249-1272) reduce to sphere-vs-sphere at the closest points of
the axis segments; newt's own tests hold no golden for either pair, so the
oracle is checked here against an independent formulation: the distance
between the segments found by dense sampling refined with a bounded scalar
minimisation, penetration = r_a + r_b - distance whenever that is positive,
normal from B into A, the point on B's surface.  Capsule-plane is pinned by
the tree-contact goldens (both segment ends, contact.rs:367-400).
"""
import numpy as np
from scipy.optimize import minimize_scalar

import oracle_py
from tooling_gb300 import model as M


def _rotmat(q_wxyz):
    w, x, y, z = q_wxyz
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def _seg(c, q, hh):
    ax = _rotmat(q) @ np.array([0.0, 0.0, 1.0])
    return c - ax * hh, c + ax * hh


def _point_seg_dist(p, a, b):
    ab = b - a
    den = ab @ ab
    t = 0.0 if den == 0 else np.clip((p - a) @ ab / den, 0.0, 1.0)
    return np.linalg.norm(p - (a + ab * t))


def _seg_seg_dist(a0, a1, b0, b1):
    f = lambda s: _point_seg_dist(a0 + (a1 - a0) * s, b0, b1)  # noqa: E731  (convex in s)
    grid = np.linspace(0.0, 1.0, 201)
    k = int(np.argmin([f(s) for s in grid]))
    lo, hi = grid[max(k - 1, 0)], grid[min(k + 1, 200)]
    return min(minimize_scalar(f, bounds=(lo, hi), method="bounded", options={"xatol": 1e-12}).fun, f(0.0), f(1.0))


def _world(shape_a, size_a, shape_b, size_b):
    w = M.WorldModel(dt=2e-3, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=20)
    a = w.add_body(1.0, M._diag9(1.0, 1.0, 1.0))
    b = w.add_body(1.0, M._diag9(1.0, 1.0, 1.0))
    w.add_geom(M.Geom(shape=shape_a, body=a, size=size_a))
    w.add_geom(M.Geom(shape=shape_b, body=b, size=size_b))
    return w


def _unit(rng):
    q = rng.normal(size=4)
    return q / np.linalg.norm(q)


def _check(kind, n=300, seed=3):
    rng = np.random.default_rng(seed)
    hits = 0
    for _ in range(n):
        ra, rb = rng.uniform(0.05, 0.2, 2)
        ha, hb = rng.uniform(0.0, 0.3, 2)
        qa, qb = _unit(rng), _unit(rng)
        ca = rng.uniform(-0.3, 0.3, 3)
        cb = ca + rng.uniform(-0.4, 0.4, 3)
        if kind == "sphere_capsule":
            w = _world(M.SHAPE_SPHERE, (ra, 0.0, 0.0), M.SHAPE_CAPSULE, (rb, hb, 0.0))
        else:
            w = _world(M.SHAPE_CAPSULE, (ra, ha, 0.0), M.SHAPE_CAPSULE, (rb, hb, 0.0))
        qpos = np.concatenate([ca, qa, cb, qb]).astype(np.float32)
        pairs, data = oracle_py.contacts(M.PackedModels([w]), 0, qpos, np.zeros(12, np.float32), precision=1)
        # the geometry the oracle saw (f32 inputs, quaternions normalised)
        q32 = qpos.astype(np.float64)
        ca64, cb64 = q32[0:3], q32[7:10]
        qa64, qb64 = q32[3:7] / np.linalg.norm(q32[3:7]), q32[10:14] / np.linalg.norm(q32[10:14])
        ra32, rb32 = float(np.float32(ra)), float(np.float32(rb))
        ha32, hb32 = float(np.float32(ha)), float(np.float32(hb))
        b0, b1 = _seg(cb64, qb64, hb32)
        if kind == "sphere_capsule":
            dist = _point_seg_dist(ca64, b0, b1)
        else:
            a0, a1 = _seg(ca64, qa64, ha32)
            dist = _seg_seg_dist(a0, a1, b0, b1)
        pen = ra32 + rb32 - dist
        if abs(pen) < 1e-7:
            continue  # on the activation threshold either answer is right
        if pen < 0:
            assert len(pairs) == 0, (kind, pen, data)
            continue
        hits += 1
        assert len(pairs) == 1 and tuple(pairs[0]) == (0, 1)
        pos, nrm, got = data[0, 0:3], data[0, 3:6], data[0, 6]
        assert abs(got - pen) < 1e-8, (kind, got, pen)
        assert abs(np.linalg.norm(nrm) - 1.0) < 1e-12
        # the point is on B's surface: radius rb from B's axis segment
        assert abs(_point_seg_dist(pos, b0, b1) - rb32) < 1e-8
        # the normal points from B into A: moving A along it separates them
        if kind == "sphere_capsule":
            moved = _point_seg_dist(ca64 + nrm * 1e-4, b0, b1)
        else:
            moved = _seg_seg_dist(a0 + nrm * 1e-4, a1 + nrm * 1e-4, b0, b1)
        assert moved > dist
    assert hits > 40
    return hits


def test_sphere_capsule_matches_segment_distance():
    _check("sphere_capsule")


def test_capsule_capsule_matches_segment_distance():
    _check("capsule_capsule")


def test_capsule_pile_scene_produces_all_capsule_pairs():
    """The sphere/capsule pile settles into sphere-capsule, capsule-capsule and
    capsule-plane contacts (the pairs the GPU parity tests then compare)."""
    from tooling_gb300 import scenes
    b = scenes.capsule_pile_batch(n_worlds=8, first_world=40)
    rq, rv = oracle_py.run(b, np.arange(len(b)), b.qpos, b.qvel, None, 400, precision=1)
    kinds = set()
    for w in range(len(b)):
        qp = rq[b.q_off[w]:b.q_off[w] + b.nq[w]].astype(np.float32)
        qv = rv[b.v_off[w]:b.v_off[w] + b.nv[w]].astype(np.float32)
        pairs, _ = oracle_py.contacts(b, w, qp, qv)
        g0 = int(b.geom_off[w])
        for ga, gb in pairs:
            sa, sb = int(b.geoms["shape"][g0 + ga]), int(b.geoms["shape"][g0 + gb])
            kinds.add(tuple(sorted((sa, sb))))
    assert {(M.SHAPE_PLANE, M.SHAPE_CAPSULE), (M.SHAPE_SPHERE, M.SHAPE_CAPSULE),
            (M.SHAPE_CAPSULE, M.SHAPE_CAPSULE)} <= kinds, kinds
