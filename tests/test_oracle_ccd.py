"""newt's GJK/EPA (the oracle's restatement of newt/src/contact/ccd.rs) as a
second formulation of the narrowphase, against the closed forms the step
uses, on known placements and on the headline generator's settled pairs.

Bars:
  * known placements (sphere on a box face, sphere-sphere, box on box,
    separated pairs): the same contact, depth within 1e-7 m;
  * box-box on the generator's pairs: EPA converges and its depth equals the
    SAT manifold's deepest point within 1e-5 m;
  * sphere-box on the generator's pairs: with EPA allowed to converge (face
    threshold 1e-7) every pair takes the EPA path and its depth equals the
    closed form's within 1e-6 m, its normal within 2e-3 rad (EPA's face
    normal on the rounded edges and corners of the Minkowski sum); with
    newt's own threshold (1e-4) EPA ends in its shallowest-axis fallback on
    almost every pair and the depth still agrees within 1e-4 m."""
import numpy as np
import pytest

import oracle_py
from pile_pairs import BOX, SPHERE, settled_pairs

CAPSULE = 3
ID = [0.0, 0.0, 0.0, 1.0]


@pytest.fixture(scope="module")
def pairs():
    return settled_pairs()


def test_sphere_on_box_face_known_answer():
    box = [0.0, 0.0, 0.0] + ID
    for face_eps in (0.0, 1e-7):
        r = oracle_py.ccd_pair(SPHERE, [0.05, -0.02, 0.299] + ID, [0.1, 0, 0], BOX, box, [0.3, 0.3, 0.2],
                               face_eps=face_eps)
        assert r is not None and abs(r["pen"] - 0.001) < 1e-7
        np.testing.assert_allclose(r["normal"], [0, 0, 1], atol=1e-7)
    assert oracle_py.ccd_pair(SPHERE, [0, 0, 0.31] + ID, [0.1, 0, 0], BOX, box, [0.3, 0.3, 0.2]) is None


def test_sphere_sphere_and_capsule_pairs_match_closed_forms():
    a, b = [0.0, 0.0, 0.0] + ID, [0.25, 0.1, -0.05] + ID
    r = oracle_py.ccd_pair(SPHERE, a, [0.15, 0, 0], SPHERE, b, [0.14, 0, 0], face_eps=1e-7)
    c = oracle_py.np_pair(SPHERE, a, [0.15, 0, 0], SPHERE, b, [0.14, 0, 0])
    assert r is not None and len(c) == 1
    assert abs(r["pen"] - c[0, 6]) < 1e-6
    np.testing.assert_allclose(r["normal"], c[0, 3:6], atol=1e-4)
    # capsule lying across a sphere
    cap = [0.0, 0.0, 0.18, 0.7071068, 0.0, 0.0, 0.7071068]
    r = oracle_py.ccd_pair(SPHERE, a, [0.1, 0, 0], CAPSULE, cap, [0.09, 0.2, 0], face_eps=1e-7)
    c = oracle_py.np_pair(SPHERE, a, [0.1, 0, 0], CAPSULE, cap, [0.09, 0.2, 0])
    assert r is not None and len(c) == 1 and abs(r["pen"] - c[0, 6]) < 1e-6


def test_box_on_box_known_answer():
    lower = [0.0, 0.0, 0.0] + ID
    upper = [0.02, -0.01, 0.399] + ID  # 1 mm into the lower box's top face
    r = oracle_py.ccd_pair(BOX, upper, [0.2, 0.2, 0.2], BOX, lower, [0.3, 0.3, 0.2])
    c = oracle_py.np_pair(BOX, upper, [0.2, 0.2, 0.2], BOX, lower, [0.3, 0.3, 0.2])
    assert r is not None and r["path"] == 2
    assert abs(r["pen"] - 0.001) < 1e-7 and abs(c[:, 6].max() - 0.001) < 1e-7
    np.testing.assert_allclose(r["normal"], [0, 0, 1], atol=1e-7)


def test_box_box_epa_matches_sat_on_generator_pairs(pairs):
    _, bb = pairs
    n = 0
    for pa, za, pb, zb in bb:
        c = oracle_py.np_pair(BOX, pa, za, BOX, pb, zb)
        r = oracle_py.ccd_pair(BOX, pa, za, BOX, pb, zb)
        if len(c) == 0:
            assert r is None or r["pen"] < 1e-6
            continue
        assert r is not None and r["path"] == 2
        assert abs(r["pen"] - c[:, 6].max()) < 1e-5
        n += 1
    assert n >= 10, n


def test_sphere_box_gjk_epa_matches_closed_form_on_generator_pairs(pairs):
    sb, _ = pairs
    n, fallback = 0, 0
    for ps, zs, pb, zb in sb:
        c = oracle_py.np_pair(SPHERE, ps, zs, BOX, pb, zb)
        conv = oracle_py.ccd_pair(SPHERE, ps, zs, BOX, pb, zb, face_eps=1e-7)
        newt = oracle_py.ccd_pair(SPHERE, ps, zs, BOX, pb, zb)
        if len(c) == 0:
            assert conv is None and newt is None
            continue
        assert conv is not None and conv["path"] == 2
        assert abs(conv["pen"] - c[0, 6]) < 1e-6
        assert np.abs(conv["normal"] - c[0, 3:6]).max() < 2e-3
        assert newt is not None and abs(newt["pen"] - c[0, 6]) < 1e-4
        fallback += newt["path"] == 3
        n += 1
    assert n >= 30, n
    assert fallback >= n // 2  # newt's threshold: the fallback is the common ending on these pairs
