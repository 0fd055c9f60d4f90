"""The device GJK/EPA (newt_gpu_convex_contacts) against the oracle's FP64
restatement of newt's routine and against the closed forms, through the C
ABI, on the headline generator's settled sphere-box and box-box pairs and on
random sphere/box/capsule placements.

Bars: the same hit/miss on every pair; where both hit and both took the
same converging path (distance GJK, or EPA run to its 1e-7 bound),
penetration within 2e-5 m and normal within 3e-3 rad.  The path itself is
precision-sensitive: newt's routine in the oracle's own f32 and FP64 takes
the same path on 87% of the random pairs with EPA allowed to converge, and
where it ends in its shallowest-axis fallback (newt's face threshold) the
f32 and FP64 answers differ by up to 0.4 rad, so fallback contacts are
compared with the oracle's f32 instantiation for hit/miss only.  With EPA
allowed to converge, sphere-box depth within 2e-5 m of the closed form."""
import numpy as np
import pytest

import oracle_py
from pile_pairs import BOX, SPHERE, settled_pairs
from tooling_gb300 import Engine
from tooling_gb300.api import CONVEX_QUERY_DTYPE

pytestmark = pytest.mark.gpu
CAPSULE = 3


@pytest.fixture(scope="module")
def eng():
    from tooling_gb300 import build as B
    B.build()
    e = Engine(device=0)
    yield e
    e.close()


def _random_pairs(n=400, seed=11):
    """Shapes of sizes 0.05..0.2 around the origin, random orientations,
    their centres 0.6..1.1 of the sum of bounding radii apart."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        ka, kb = rng.choice([SPHERE, BOX, CAPSULE], 2)
        sz = []
        for k in (ka, kb):
            if k == SPHERE:
                sz.append(np.array([rng.uniform(0.05, 0.2), 0, 0], np.float32))
            elif k == BOX:
                sz.append(rng.uniform(0.05, 0.2, 3).astype(np.float32))
            else:
                sz.append(np.array([rng.uniform(0.03, 0.1), rng.uniform(0.05, 0.2), 0], np.float32))
        bound = lambda k, z: z[0] if k == SPHERE else (np.linalg.norm(z) if k == BOX else z[0] + z[1])
        dirn = rng.normal(size=3)
        dirn /= np.linalg.norm(dirn)
        dist = rng.uniform(0.6, 1.1) * (bound(ka, sz[0]) + bound(kb, sz[1]))
        poses = []
        for c in (np.zeros(3), dirn * dist):
            qv = rng.normal(size=4)
            qv /= np.linalg.norm(qv)
            poses.append(np.r_[c, qv].astype(np.float32))
        out.append((int(ka), poses[0], sz[0], int(kb), poses[1], sz[1]))
    return out


def _queries(pairs):
    q = np.zeros(len(pairs), CONVEX_QUERY_DTYPE)
    for i, (ka, pa, za, kb, pb, zb) in enumerate(pairs):
        q[i] = (ka, kb, pa, za, pb, zb, 0.0)
    return q


def _compare(eng, pairs, face_eps, precision):
    got = eng.convex_contacts(_queries(pairs), face_eps=face_eps)
    same_path, total = 0, 0
    for g, (ka, pa, za, kb, pb, zb) in zip(got, pairs):
        ref = oracle_py.ccd_pair(ka, pa, za, kb, pb, zb, face_eps=face_eps, precision=precision)
        assert bool(g["hit"]) == (ref is not None), (ka, kb, g, ref)
        if ref is None:
            continue
        total += 1
        if g["path"] != ref["path"]:
            continue
        same_path += 1
        if ref["path"] == 3:  # the fallback: precision-sensitive (module docstring)
            continue
        assert abs(g["penetration"] - ref["pen"]) < 2e-5, (ka, kb, g["penetration"], ref["pen"])
        assert np.abs(g["normal"] - ref["normal"]).max() < 3e-3, (ka, kb, g["normal"], ref["normal"])
    return same_path, total


def test_device_gjk_epa_converged_matches_fp64_oracle(eng):
    same, total = _compare(eng, _random_pairs(), 1e-7, precision=1)
    assert total >= 100 and same >= 0.8 * total, (same, total)


def test_device_gjk_epa_at_newts_threshold_matches_f32_oracle(eng):
    same, total = _compare(eng, _random_pairs(), 0.0, precision=0)
    assert total >= 100 and same >= 0.9 * total, (same, total)


def test_device_gjk_epa_on_generator_pairs(eng):
    sb, bb = settled_pairs()
    pairs = [(SPHERE, a, b, BOX, c, d) for a, b, c, d in sb] + [(BOX, a, b, BOX, c, d) for a, b, c, d in bb]
    same, total = _compare(eng, pairs, 1e-7, precision=1)
    assert total >= 40 and same >= 0.8 * total, (same, total)
    # sphere-box: the converged device EPA against the closed form
    got = eng.convex_contacts(_queries(pairs[:len(sb)]), face_eps=1e-7)
    n = 0
    for g, (ps, zs, pb, zb) in zip(got, sb):
        c = oracle_py.np_pair(SPHERE, ps, zs, BOX, pb, zb)
        if len(c) == 0:
            assert not g["hit"]
            continue
        assert g["hit"] and abs(g["penetration"] - c[0, 6]) < 2e-5
        n += 1
    assert n >= 30
