"""The device GJK/EPA (newt_gpu_convex_contacts) against the oracle's
restatements of newt's routine and against the closed forms, through the C
ABI, on the headline generator's settled sphere-box and box-box pairs and on
random sphere/box/capsule placements.

Bars: bit-exact with the oracle's f32 instantiation (newt's own arithmetic:
every product and sum rounded on its own, IEEE division and square root) in
hit/miss, path, depth, normal, position and witnesses, at newt's face
threshold (1e-4 of the pair extent) and at 1e-7, where EPA runs to its
convergence bound.  Bit parity is the bar because the routine is
precision-sensitive: its face test at 1e-7 sits at the f32 rounding level,
and a build that fuses multiply-adds takes other polytope paths and on some
curved pairs reports a converged depth for a face that is not the nearest
(a 0.082 m sphere-sphere depth where the exact one is 0.067 m).  Against
the FP64 oracle, wherever both took the same converging path (distance GJK,
or EPA to 1e-7): depth within 2e-5 m and normal within 3e-3; sphere-box depth
within 2e-5 m of the closed form."""
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


def _check_bits(g, ref):
    """One device result equals the f32 oracle's bit for bit."""
    assert bool(g["hit"]) == (ref is not None), (g, ref)
    if ref is None:
        return
    f = lambda x: np.asarray(x, np.float64).astype(np.float32)
    assert int(g["path"]) == ref["path"], (g, ref)
    assert g["penetration"] == f(ref["pen"]), (g["penetration"], ref["pen"])
    for k_dev, k_ref in (("normal", "normal"), ("pos", "pos"), ("witness_a", "witness_a"), ("witness_b", "witness_b")):
        assert np.array_equal(g[k_dev], f(ref[k_ref])), (k_dev, g[k_dev], ref[k_ref])


def _all_pairs():
    sb, bb = settled_pairs()
    gen = [(SPHERE, a, b, BOX, c, d) for a, b, c, d in sb] + [(BOX, a, b, BOX, c, d) for a, b, c, d in bb]
    return _random_pairs() + gen


@pytest.mark.parametrize("face_eps", [0.0, 1e-7])
def test_device_gjk_epa_is_bit_exact_with_newts_f32(eng, face_eps):
    pairs = _all_pairs()
    got = eng.convex_contacts(_queries(pairs), face_eps=face_eps)
    hits = 0
    for g, (ka, pa, za, kb, pb, zb) in zip(got, pairs):
        ref = oracle_py.ccd_pair(ka, pa, za, kb, pb, zb, face_eps=face_eps, precision=0)
        _check_bits(g, ref)
        hits += ref is not None
    assert hits >= 200


def test_device_gjk_epa_converged_matches_fp64_oracle(eng):
    pairs = _all_pairs()
    got = eng.convex_contacts(_queries(pairs), face_eps=1e-7)
    same_path, total = 0, 0
    for g, (ka, pa, za, kb, pb, zb) in zip(got, pairs):
        ref = oracle_py.ccd_pair(ka, pa, za, kb, pb, zb, face_eps=1e-7, precision=1)
        assert bool(g["hit"]) == (ref is not None), (ka, kb, g, ref)
        if ref is None:
            continue
        total += 1
        if g["path"] != ref["path"] or ref["path"] == 3:
            continue
        same_path += 1
        assert abs(g["penetration"] - ref["pen"]) < 2e-5, (ka, kb, g["penetration"], ref["pen"])
        assert np.abs(g["normal"] - ref["normal"]).max() < 3e-3, (ka, kb, g["normal"], ref["normal"])
    assert total >= 200 and same_path >= 0.8 * total, (same_path, total)


def test_device_gjk_epa_sphere_box_matches_closed_form(eng):
    sb, _ = settled_pairs()
    pairs = [(SPHERE, a, b, BOX, c, d) for a, b, c, d in sb]
    got = eng.convex_contacts(_queries(pairs), face_eps=1e-7)
    n = 0
    for g, (ps, zs, pb, zb) in zip(got, sb):
        c = oracle_py.np_pair(SPHERE, ps, zs, BOX, pb, zb)
        if len(c) == 0:
            assert not g["hit"]
            continue
        assert g["hit"] and abs(g["penetration"] - c[0, 6]) < 2e-5
        n += 1
    assert n >= 30
