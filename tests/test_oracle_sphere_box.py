"""Known-answer check of the oracle's sphere-box contact (CPU only).

newt defers the sphere-box pair (newt/src/contact.rs:236-257), so no newt
golden covers it; the oracle restates it as the closed-form closest point on
the oriented box with newt's contact conventions (normal from the box into
the sphere, penetration = margin - distance, point on the box surface).  Here
it is checked against an independent formulation: the signed distance of the
sphere centre to the box, sd = |max(q, 0)| + min(max_i q_i, 0) with
q = |p_local| - h, so penetration = r - sd whenever sd < r.
"""
import numpy as np

import oracle_py
from tooling_gb300 import model as M


def _rotmat(q_wxyz):
    w, x, y, z = q_wxyz
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def test_sphere_box_penetration_matches_signed_distance():
    rng = np.random.default_rng(7)
    checked = hits = 0
    for _ in range(300):
        r = float(rng.uniform(0.05, 0.2))
        h = rng.uniform(0.05, 0.2, 3)
        w = M.WorldModel(dt=2e-3, gravity=(0.0, 0.0, -9.81), solver=M.SOLVER_PGS, iterations=50)
        s = w.add_body(1.0, M._diag9(1.0, 1.0, 1.0))
        b = w.add_body(1.0, M._diag9(1.0, 1.0, 1.0))
        w.add_geom(M.Geom(shape=M.SHAPE_SPHERE, body=s, size=(r, 0.0, 0.0)))
        w.add_geom(M.Geom(shape=M.SHAPE_BOX, body=b, size=tuple(float(x) for x in h)))
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        cb = rng.uniform(-0.5, 0.5, 3)
        local = rng.uniform(-1.0, 1.0, 3) * (h + 1.5 * r)
        cs = cb + _rotmat(q) @ local
        qpos = np.concatenate([cs, [1.0, 0.0, 0.0, 0.0], cb, q]).astype(np.float32)
        qvel = np.zeros(12, np.float32)
        # the distance the oracle sees (its inputs are float32)
        qq = qpos[10:14].astype(np.float64)
        qq /= np.linalg.norm(qq)
        p_local = _rotmat(qq).T @ (qpos[0:3].astype(np.float64) - qpos[7:10].astype(np.float64))
        hq = np.abs(p_local) - h.astype(np.float32).astype(np.float64)
        sd = np.linalg.norm(np.maximum(hq, 0.0)) + min(hq.max(), 0.0)
        r32 = float(np.float32(r))
        pairs, data = oracle_py.contacts(M.PackedModels([w]), 0, qpos, qvel, precision=1)
        checked += 1
        if abs(sd - r32) < 1e-6:
            continue  # on the activation threshold either answer is right
        if sd >= r32:
            assert len(pairs) == 0, (sd, r32, data)
            continue
        hits += 1
        assert len(pairs) == 1 and tuple(pairs[0]) == (0, 1)
        pos, n, pen = data[0, 0:3], data[0, 3:6], data[0, 6]
        assert abs(pen - (r32 - sd)) < 1e-7, (pen, r32 - sd)
        assert abs(np.linalg.norm(n) - 1.0) < 1e-12
        # the point lies on the box surface, the normal points out of the box
        pl = _rotmat(qq).T @ (pos - qpos[7:10].astype(np.float64))
        assert np.all(np.abs(pl) <= h.astype(np.float32) + 1e-6)
        assert np.isclose(np.max(np.abs(pl) - h.astype(np.float32)), 0.0, atol=1e-6)
        assert n @ (qpos[0:3].astype(np.float64) - pos) >= -1e-6 or sd < 0
    assert checked == 300 and hits > 50
