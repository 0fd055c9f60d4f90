"""Known-answer checks of the oracle's cylinder-plane, ellipsoid-plane,
sphere-cylinder and sphere-ellipsoid contacts (CPU only;
newt/src/contact.rs:1296-1426, 1519-1725).

Cylinder: an upright cylinder sunk by d gives four contacts of depth d, the
bottom cap centre and the bottom rim at 0, 45 and 90 degrees (newt's tie
order); for random poses the contacts equal an independent evaluation of
newt's rule (18 samples, the four deepest with penetration > 0, projected
onto the plane).  Ellipsoid: the penetration equals the depth of the
deepest surface point found by a dense search over the surface, and the
contact lies midway between that point and the plane.  Sphere-ellipsoid:
newt's anchors (contacts_geoms_v1.rs:1414-1446, 1470-1500: depth 0.1 within
1e-6, normal +X, point (0.45, 0, 0) within 2e-3) in either geom order, and
for sphere centres outside the ellipsoid the penetration, normal and point
against the nearest surface point from a bisection on the Lagrange
parameter in double (an independent solve): within 1e-6 (FP64) and 2e-5
(f32, newt's arithmetic).
"""
import numpy as np
import pytest

import oracle_py
from tooling_gb300 import model as M


def _rotmat(q_wxyz):
    w, x, y, z = q_wxyz
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def _one(shape, size, pos, quat):
    w = M.WorldModel(dt=2e-3, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=20)
    w.add_geom(M.static_plane())
    b = w.add_body(1.0, M._diag9(0.01, 0.01, 0.01))
    w.add_geom(M.Geom(shape=shape, body=b, size=size))
    qpos = np.array(list(pos) + list(quat), np.float32)
    pairs, data = oracle_py.contacts(M.PackedModels([w]), 0, qpos, np.zeros(6, np.float32), precision=1)
    return pairs, data, qpos


def test_upright_cylinder_gives_newts_four_tied_contacts():
    r, h, d = 0.3, 0.2, 0.01
    pairs, data, _ = _one(M.SHAPE_CYLINDER, (r, h, 0.0), (0.0, 0.0, h - d), (1.0, 0.0, 0.0, 0.0))
    # labels follow the pair order (plane first), the normal from the cylinder
    # into the plane (newt's swap rule, contact.rs:2575-2586)
    assert [tuple(p) for p in pairs] == [(0, 1)] * 4
    s = np.float32(0.70710677)
    expect = np.array([[0.0, 0.0, 0.0], [r, 0.0, 0.0], [r * s, r * s, 0.0], [0.0, r, 0.0]])
    np.testing.assert_allclose(data[:, 0:3], expect, atol=1e-6)
    np.testing.assert_allclose(data[:, 6], d, atol=1e-6)
    np.testing.assert_allclose(data[:, 3:6], [[0.0, 0.0, -1.0]] * 4, atol=1e-12)


def test_cylinder_contacts_follow_the_sampling_rule():
    rng = np.random.default_rng(11)
    seen = 0
    for _ in range(300):
        r, h = rng.uniform(0.05, 0.3), rng.uniform(0.05, 0.3)
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        pos = (rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(-0.1, 0.35))
        pairs, data, qpos = _one(M.SHAPE_CYLINDER, (r, h, 0.0), pos, q)
        Rm = _rotmat(qpos[3:7].astype(np.float64) / np.linalg.norm(qpos[3:7].astype(np.float64)))
        c = qpos[0:3].astype(np.float64)
        r32, h32 = float(np.float32(r)), float(np.float32(h))
        ax, xl, yl = Rm[:, 2], Rm[:, 0], Rm[:, 1]
        top, bot = c + ax * h32, c - ax * h32
        ang = np.deg2rad(45.0 * np.arange(8))
        dirs = [xl * np.cos(t) + yl * np.sin(t) for t in ang]
        smp = [top, bot] + [p for dd in dirs for p in (top + dd * r32, bot + dd * r32)]
        pen = np.array([-p[2] for p in smp])
        idx = [i for i in np.argsort(-pen, kind="stable") if pen[i] > 0][:4]
        if any(abs(pen[i]) < 1e-6 for i in range(18)):
            continue  # a sample on the plane: the strict threshold may go either way
        assert len(pairs) == len(idx)
        for k, i in enumerate(idx):
            assert abs(data[k, 6] - pen[i]) < 1e-6
            assert np.abs(data[k, 0:3] - (smp[i] - np.array([0.0, 0.0, smp[i][2]]))).max() < 1e-6
        seen += len(idx) > 0
    assert seen > 50


def _ellipsoid_surface(n=400):
    u = np.linspace(0.0, np.pi, n)
    v = np.linspace(0.0, 2.0 * np.pi, 2 * n)
    U, V = np.meshgrid(u, v)
    return np.stack([np.sin(U) * np.cos(V), np.sin(U) * np.sin(V), np.cos(U)], -1).reshape(-1, 3)


def test_ellipsoid_depth_matches_surface_search():
    rng = np.random.default_rng(5)
    sphere = _ellipsoid_surface()
    hits = 0
    for _ in range(60):
        ax = rng.uniform(0.05, 0.3, 3)
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        pos = (rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(-0.05, 0.3))
        pairs, data, qpos = _one(M.SHAPE_ELLIPSOID, tuple(ax), pos, q)
        Rm = _rotmat(qpos[3:7].astype(np.float64) / np.linalg.norm(qpos[3:7].astype(np.float64)))
        a32 = np.array([float(np.float32(x)) for x in ax])
        pts = qpos[0:3].astype(np.float64) + (sphere * a32) @ Rm.T
        deepest = pts[np.argmin(pts[:, 2])]
        depth = -deepest[2]
        if abs(depth) < 1e-3:
            continue
        if depth < 0:
            assert len(pairs) == 0
            continue
        hits += 1
        assert len(pairs) == 1 and tuple(pairs[0]) == (0, 1)
        assert data[0, 6] >= depth - 1e-9 and data[0, 6] - depth < 2e-4 * a32.max()
        mid = deepest.copy()
        mid[2] *= 0.5
        assert np.abs(data[0, 0:3] - mid).max() < 2e-2 * a32.max()
    assert hits > 15


def test_sphere_cylinder_matches_signed_distance():
    """contact.rs:1519-1628 against the signed distance of the sphere centre
    to the solid cylinder: outside, |(max(r_xy - R, 0), max(|z| - h, 0))|;
    inside, -min(R - r_xy, h - |z|); penetration = r_s - signed distance."""
    rng = np.random.default_rng(9)
    hits = 0
    for _ in range(400):
        rs, rc, hh = rng.uniform(0.05, 0.2), rng.uniform(0.05, 0.3), rng.uniform(0.05, 0.3)
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        w = M.WorldModel(dt=2e-3, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=20)
        a = w.add_body(1.0, M._diag9(0.01, 0.01, 0.01))
        c = w.add_body(1.0, M._diag9(0.01, 0.01, 0.01))
        w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, body=a, size=(rs, 0.0, 0.0)))
        w.add_geom(M.Geom(shape=M.SHAPE_CYLINDER, body=c, size=(rc, hh, 0.0)))
        cc = rng.uniform(-0.3, 0.3, 3)
        cs = cc + rng.uniform(-0.5, 0.5, 3)
        qpos = np.concatenate([cs, [1.0, 0.0, 0.0, 0.0], cc, q]).astype(np.float32)
        pairs, data = oracle_py.contacts(M.PackedModels([w]), 0, qpos, np.zeros(12, np.float32), precision=1)
        Rm = _rotmat(qpos[10:14].astype(np.float64) / np.linalg.norm(qpos[10:14].astype(np.float64)))
        pl = Rm.T @ (qpos[0:3].astype(np.float64) - qpos[7:10].astype(np.float64))
        R32, h32, r32 = (float(np.float32(x)) for x in (rc, hh, rs))
        rxy, az = np.hypot(pl[0], pl[1]), abs(pl[2])
        if rxy <= R32 and az <= h32:
            sd = -min(R32 - rxy, h32 - az)
        else:
            sd = np.hypot(max(rxy - R32, 0.0), max(az - h32, 0.0))
        pen = r32 - sd
        if abs(pen) < 1e-7:
            continue
        if pen < 0:
            assert len(pairs) == 0
            continue
        hits += 1
        assert len(pairs) == 1 and tuple(pairs[0]) == (0, 1)
        assert abs(data[0, 6] - pen) < 1e-8, (data[0, 6], pen)
        assert abs(np.linalg.norm(data[0, 3:6]) - 1.0) < 1e-9
    assert hits > 60


def _sphere_ellipsoid(rs, sp, ax, ep, eq, ell_first=False, precision=1):
    w = M.WorldModel(dt=2e-3, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=20)
    a = w.add_body(1.0, M._diag9(0.01, 0.01, 0.01))
    b = w.add_body(1.0, M._diag9(0.01, 0.01, 0.01))
    gs = M.Geom(shape=M.SHAPE_SPHERE, body=a, size=(rs, 0.0, 0.0))
    ge = M.Geom(shape=M.SHAPE_ELLIPSOID, body=b, size=tuple(float(x) for x in ax))
    for g in ((ge, gs) if ell_first else (gs, ge)):
        w.add_geom(g)
    qpos = np.concatenate([sp, [1.0, 0.0, 0.0, 0.0], ep, eq]).astype(np.float32)
    return oracle_py.contacts(M.PackedModels([w]), 0, qpos, np.zeros(12, np.float32), precision=precision), qpos


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("ell_first", [False, True])
def test_sphere_ellipsoid_anchor(precision, ell_first):
    (pairs, data), _ = _sphere_ellipsoid(0.2, (0.6, 0.0, 0.0), (0.5, 0.3, 0.2), (0.0, 0.0, 0.0), (1.0, 0.0, 0.0, 0.0),
                                         ell_first, precision)
    assert len(pairs) == 1
    sgn = -1.0 if ell_first else 1.0  # newt relabels (B, A) pairs with the normal flipped
    assert tuple(pairs[0]) == (0, 1)
    assert abs(data[0, 6] - 0.1) < 1e-6
    assert np.abs(data[0, 3:6] - sgn * np.array([1.0, 0.0, 0.0])).max() < 1e-6
    assert np.abs(data[0, 0:3] - np.array([0.45, 0.0, 0.0])).max() < 2e-3


def _nearest_on_ellipsoid(p, a):
    """The surface point nearest an outside point p by bisection on the
    Lagrange parameter t of q = a^2 p / (a^2 + t) (f(t) = sum (a p / (a^2 +
    t))^2 - 1 falls from f(0) > 0 to -1), in double: an independent solve of
    the problem newt's twelve Newton steps address."""
    f = lambda t: ((a * p / (a * a + t)) ** 2).sum() - 1.0
    lo, hi = 0.0, 1.0
    while f(hi) > 0.0:
        hi *= 2.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        lo, hi = (mid, hi) if f(mid) > 0.0 else (lo, mid)
    return a * a * p / (a * a + lo)


@pytest.mark.parametrize("precision,ptol,ntol", [(1, 1e-6, 1e-4), (0, 2e-5, 1e-3)])
def test_sphere_ellipsoid_matches_nearest_point(precision, ptol, ntol):
    rng = np.random.default_rng(21)
    hits = 0
    for _ in range(300):
        ax = rng.uniform(0.08, 0.3, 3)
        rs = rng.uniform(0.05, 0.15)
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        ep = rng.uniform(-0.2, 0.2, 3)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        sp = ep + d * (ax.min() + (ax.max() - ax.min() + rs) * rng.uniform(0.0, 1.2))
        (pairs, data), qpos = _sphere_ellipsoid(rs, sp, ax, ep, q, precision=precision)
        Rm = _rotmat(qpos[10:14].astype(np.float64) / np.linalg.norm(qpos[10:14].astype(np.float64)))
        a32 = np.array([float(np.float32(x)) for x in ax])
        p = Rm.T @ (qpos[0:3].astype(np.float64) - qpos[7:10].astype(np.float64))
        if ((p / a32) ** 2).sum() <= 1.0:
            continue  # newt's solver addresses centres outside the ellipsoid
        qn = _nearest_on_ellipsoid(p, a32)
        dist = np.linalg.norm(p - qn)
        pen = float(np.float32(rs)) - dist
        if abs(pen) < 1e-5:
            continue
        if pen < 0:
            assert len(pairs) == 0
            continue
        hits += 1
        assert len(pairs) == 1 and tuple(pairs[0]) == (0, 1)
        assert abs(data[0, 6] - pen) < ptol, (data[0, 6], pen)
        nrm = Rm @ ((p - qn) / dist)
        assert np.abs(data[0, 3:6] - nrm).max() < ntol
        surf = qpos[7:10].astype(np.float64) + Rm @ qn
        mid = 0.5 * (surf + (qpos[0:3].astype(np.float64) - nrm * float(np.float32(rs))))
        assert np.abs(data[0, 0:3] - mid).max() < 10 * ptol
    assert hits > 60
