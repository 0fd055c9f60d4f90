"""Seeded synthetic worlds for the five benchmark workloads.

No dataset is involved: every world is drawn from a seeded generator with the
shapes, sizes and distributions the workloads specify.  Seeds:
``splitmix64(0x6e657774 + config_index)`` per workload and
``splitmix64(config_seed ^ world_id)`` per world, so any world can be rebuilt
alone (the serving tests rely on that).

Workloads
  chain     : 7-link serial hinge pendulum, no contact (dt 1e-3)
  pile      : 16 free spheres/boxes above a plane, PGS 50 (dt 2e-3)
  quadruped : floating-base 18-DoF quadruped on a plane, Newton <= 20 (dt 2e-3)
  uneven    : 50/50 chains and piles, 2..64 bodies (log-uniform), PGS 50
"""
from __future__ import annotations

import math
from typing import Optional

import numpy as np

from . import model as M

MASK64 = (1 << 64) - 1
DEFAULT_SOLREF = (0.02, 1.0)
DEFAULT_SOLIMP = (0.9, 0.95, 0.001, 0.5, 2.0)


def splitmix64(x: int) -> int:
    x = (x + 0x9E3779B97F4A7C15) & MASK64
    z = x
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return z ^ (z >> 31)


def config_seed(index: int) -> int:
    return splitmix64(0x6E657774 + index)


def world_rng(cfg_seed: int, world_id: int) -> np.random.Generator:
    return np.random.default_rng(splitmix64(cfg_seed ^ world_id))


def _f32(x):
    return np.float32(x)


def _diag9(a, b, c):
    return np.array([a, 0, 0, 0, b, 0, 0, 0, c], np.float32)


def capsule_inertia(mass, radius, half_height):
    return np.array(M.solid_capsule_inertia(mass, radius, half_height), np.float32)


def sphere_inertia(mass, r):
    return np.array(M.solid_sphere_inertia(mass, r), np.float32)


def box_inertia(mass, h):
    return np.array(M.solid_box_inertia(mass, h), np.float32)


def _geom(shape, body=-1, link=-1, size=(0, 0, 0), pos=(0, 0, 0), quat=(0, 0, 0, 1), friction=1.0, condim=3):
    g = np.zeros((), M.GEOM_DT)
    g["shape"], g["body"], g["link"] = shape, body, link
    g["size"] = size
    g["local_pos"] = pos
    g["local_quat"] = quat
    g["friction"] = friction
    g["solref"] = DEFAULT_SOLREF
    g["solimp"] = DEFAULT_SOLIMP
    g["condim"] = condim
    g["group"] = 0xFFFFFFFF
    g["mask"] = 0xFFFFFFFF
    return g


def _link(parent, joint, axis=(0, 0, 1), damping=0.0, jp=(0, 0, 0), jpq=(0, 0, 0, 1), jc=(0, 0, 0), mass=1.0,
          inertia=None):
    l = np.zeros((), M.LINK_DT)
    l["parent"], l["joint"] = parent, joint
    l["axis"] = axis
    l["damping"] = damping
    l["jp_pos"] = jp
    l["jp_quat"] = jpq
    l["jc_pos"] = jc
    l["jc_quat"] = (0, 0, 0, 1)
    l["mass"] = mass
    l["inertia"] = inertia if inertia is not None else _diag9(1, 1, 1)
    return l


# ---------------------------------------------------------------------------
# chain: serial hinge pendulum
# ---------------------------------------------------------------------------
CHAIN_RADIUS = 0.03


def _chain_world(rng: np.random.Generator, n_hinges: int, damping: bool = True):
    """Fixed root at the origin + n hinge links about x, joint at each capsule's
    top (joint_offset_in_child = (0,0,L/2), parent offset (0,0,-L_parent/2))."""
    links = [_link(-1, M.JOINT_FIXED, mass=1.0, inertia=_diag9(1, 1, 1))]
    masses = rng.uniform(0.5, 2.0, n_hinges)
    lengths = rng.uniform(0.2, 0.5, n_hinges)
    damp = rng.uniform(0.0, 0.1, n_hinges) if damping else np.zeros(n_hinges)
    prev_half = 0.0
    for i in range(n_hinges):
        half = float(_f32(lengths[i]) * _f32(0.5))
        links.append(_link(i, M.JOINT_HINGE, axis=(1.0, 0.0, 0.0), damping=float(damp[i]),
                           jp=(0.0, 0.0, -prev_half), jc=(0.0, 0.0, half), mass=float(masses[i]),
                           inertia=capsule_inertia(masses[i], CHAIN_RADIUS, half)))
        prev_half = half
    q = rng.uniform(-math.pi, math.pi, n_hinges)
    qd = rng.normal(0.0, 1.0, n_hinges)
    tau = rng.normal(0.0, 0.5, n_hinges)
    return links, q, qd, tau


def chain_batch(n_worlds: int = 4096, n_hinges: int = 7, seed_index: int = 0, dt: float = 1e-3,
                damping: bool = True, torque: bool = True, first_world: int = 0) -> M.Batch:
    cs = config_seed(seed_index)
    all_links, qs, qds, taus = [], [], [], []
    for w in range(first_world, first_world + n_worlds):
        links, q, qd, tau = _chain_world(world_rng(cs, w), n_hinges, damping)
        all_links += links
        qs.append(q); qds.append(qd); taus.append(tau if torque else np.zeros_like(tau))
    b = M.Batch(np.stack(all_links), [n_hinges + 1] * n_worlds, np.zeros(0, M.BODY_DT), [0] * n_worlds,
                np.zeros(0, M.GEOM_DT), [0] * n_worlds, dt, (0.0, 0.0, -9.81), M.SOLVER_PGS, 50)
    b.qpos[:] = np.concatenate(qs)
    b.qvel[:] = np.concatenate(qds)
    b.qfrc[:] = np.concatenate(taus)
    return b


# ---------------------------------------------------------------------------
# pile: free spheres and boxes above a plane
# ---------------------------------------------------------------------------
def _random_quat(rng):
    # uniform unit quaternion (Shoemake); returned as w, x, y, z (MuJoCo order)
    u1, u2, u3 = rng.random(3)
    a, b = math.sqrt(1 - u1), math.sqrt(u1)
    x, y = a * math.sin(2 * math.pi * u2), a * math.cos(2 * math.pi * u2)
    z, w = b * math.sin(2 * math.pi * u3), b * math.cos(2 * math.pi * u3)
    return (w, x, y, z)


def _pile_world(rng: np.random.Generator, n_bodies: int, box_lo=(-1.0, -1.0, 0.3), box_hi=(1.0, 1.0, 2.3)):
    """n free bodies: 50% spheres r~U(.05,.2), 50% boxes half-extents~U(.05,.2);
    density 1000; positions uniform in the box, rejection-sampled so bounding
    spheres do not overlap; uniform random orientations; zero velocity."""
    bodies, geoms = [], [_geom(M.SHAPE_PLANE, friction=1.0)]
    qpos = []
    centers, radii = [], []
    for b in range(n_bodies):
        sphere = rng.random() < 0.5
        if sphere:
            r = float(rng.uniform(0.05, 0.2))
            mass = float(_f32(1000.0) * _f32(4.0 / 3.0 * math.pi * r ** 3))
            inertia = sphere_inertia(mass, r)
            size = (r, 0.0, 0.0)
            bound = r
        else:
            h = rng.uniform(0.05, 0.2, 3)
            mass = float(_f32(1000.0 * 8.0 * h[0] * h[1] * h[2]))
            inertia = box_inertia(mass, h)
            size = tuple(float(v) for v in h)
            bound = float(np.linalg.norm(h))
        mu = float(rng.uniform(0.3, 1.0))
        C_arr = np.asarray(centers).reshape(-1, 3)
        R_arr = np.asarray(radii)
        for _ in range(1000):
            p = rng.uniform(box_lo, box_hi)
            if not len(C_arr) or np.all(np.sqrt(((C_arr - p) ** 2).sum(axis=1)) > bound + R_arr):
                break
        centers.append(p)
        radii.append(bound)
        bd = np.zeros((), M.BODY_DT)
        bd["mass"] = mass
        bd["inertia"] = inertia
        bodies.append(bd)
        geoms.append(_geom(M.SHAPE_SPHERE if sphere else M.SHAPE_BOX, body=b, size=size, friction=mu))
        qpos.append(np.concatenate([p, _random_quat(rng)]))
    return bodies, geoms, np.concatenate(qpos)


def _capsule_pile_world(rng: np.random.Generator, n_bodies: int, box_lo=(-0.8, -0.8, 0.3), box_hi=(0.8, 0.8, 2.0)):
    """n free bodies: 50% spheres r~U(.05,.2), 50% capsules r~U(.04,.12),
    half-height~U(.05,.2) along local z; density 1000; placed like the box
    piles (non-overlapping bounding spheres, random orientations, at rest)."""
    bodies, geoms = [], [_geom(M.SHAPE_PLANE, friction=1.0)]
    qpos, centers, radii = [], [], []
    for b in range(n_bodies):
        sphere = rng.random() < 0.5
        if sphere:
            r = float(rng.uniform(0.05, 0.2))
            mass = float(_f32(1000.0) * _f32(4.0 / 3.0 * math.pi * r ** 3))
            inertia, size, bound = sphere_inertia(mass, r), (r, 0.0, 0.0), r
        else:
            r, hh = float(rng.uniform(0.04, 0.12)), float(rng.uniform(0.05, 0.2))
            mass = float(_f32(1000.0 * (math.pi * r * r * 2.0 * hh + 4.0 / 3.0 * math.pi * r ** 3)))
            inertia = np.array(M.solid_capsule_inertia(mass, r, hh), np.float32)
            size, bound = (r, hh, 0.0), r + hh
        mu = float(rng.uniform(0.3, 1.0))
        C_arr, R_arr = np.asarray(centers).reshape(-1, 3), np.asarray(radii)
        for _ in range(1000):
            p = rng.uniform(box_lo, box_hi)
            if not len(C_arr) or np.all(np.sqrt(((C_arr - p) ** 2).sum(axis=1)) > bound + R_arr):
                break
        centers.append(p)
        radii.append(bound)
        bd = np.zeros((), M.BODY_DT)
        bd["mass"], bd["inertia"] = mass, inertia
        bodies.append(bd)
        geoms.append(_geom(M.SHAPE_SPHERE if sphere else M.SHAPE_CAPSULE, body=b, size=size, friction=mu))
        qpos.append(np.concatenate([p, _random_quat(rng)]))
    return bodies, geoms, np.concatenate(qpos)


def capsule_pile_batch(n_worlds: int = 1024, n_bodies: int = 12, seed_index: int = 5, dt: float = 2e-3,
                       iterations: int = 50, first_world: int = 0) -> M.Batch:
    """Piles of free spheres and capsules on a plane (sphere-capsule,
    capsule-capsule and capsule-plane contacts), PGS."""
    cs = config_seed(seed_index)
    bodies, geoms, qps = [], [], []
    for w in range(first_world, first_world + n_worlds):
        b, g, qp = _capsule_pile_world(world_rng(cs, w), n_bodies)
        bodies += b; geoms += g; qps.append(qp)
    batch = M.Batch(np.zeros(0, M.LINK_DT), [0] * n_worlds, np.stack(bodies), [n_bodies] * n_worlds,
                    np.stack(geoms), [n_bodies + 1] * n_worlds, dt, (0.0, 0.0, -9.81), M.SOLVER_PGS, iterations)
    batch.qpos[:] = np.concatenate(qps)
    return batch


def pile_batch(n_worlds: int = 8192, n_bodies: int = 16, seed_index: int = 1, dt: float = 2e-3,
               iterations: int = 50, first_world: int = 0) -> M.Batch:
    cs = config_seed(seed_index)
    bodies, geoms, qps = [], [], []
    for w in range(first_world, first_world + n_worlds):
        b, g, qp = _pile_world(world_rng(cs, w), n_bodies)
        bodies += b; geoms += g; qps.append(qp)
    batch = M.Batch(np.zeros(0, M.LINK_DT), [0] * n_worlds, np.stack(bodies), [n_bodies] * n_worlds,
                    np.stack(geoms), [n_bodies + 1] * n_worlds, dt, (0.0, 0.0, -9.81), M.SOLVER_PGS, iterations)
    batch.qpos[:] = np.concatenate(qps)
    return batch


# ---------------------------------------------------------------------------
# quadruped: floating-base torso with 4 x 3 revolute legs on a plane
# ---------------------------------------------------------------------------
QUAD_TORSO_HALF = (0.2, 0.1, 0.05)  # 0.4 x 0.2 x 0.1 m box
QUAD_TORSO_MASS = 5.0
QUAD_LINK_HALF = 0.1                # capsule links 0.2 m long
QUAD_LINK_RADIUS = 0.02
QUAD_LINK_MASS = 0.5
QUAD_MU = 0.8
QUAD_CROUCH = (0.0, 0.9, -1.8)      # hip-ab, hip-flex, knee nominal angles
QUAD_HIPS = ((0.15, 1.0), (0.15, -1.0), (-0.15, 1.0), (-0.15, -1.0))  # (x, side)


def _rot(axis, a):
    c, s = math.cos(a), math.sin(a)
    if axis == 0:
        return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])


def _quad_lowest_point(base_z, q):
    """Lowest point of the legs' capsules (forward kinematics with the torso
    level at height base_z; used to reject initial penetration)."""
    low = np.inf
    for leg, (hx, side) in enumerate(QUAD_HIPS):
        ab, flex, knee = q[3 * leg:3 * leg + 3]
        # link 1: hinge about x at the torso side, capsule along y, outward
        R1 = _rot(0, ab)
        j1 = np.array([hx, side * QUAD_TORSO_HALF[1], base_z])
        p1 = j1 + R1 @ np.array([0.0, side * QUAD_LINK_HALF, 0.0])
        e1 = [p1 + R1 @ np.array([0.0, s * QUAD_LINK_HALF, 0.0]) for s in (1, -1)]
        # link 2: hip flexion about y at link 1's outer end, hanging down
        j2 = p1 + R1 @ np.array([0.0, side * QUAD_LINK_HALF, 0.0])
        R2 = R1 @ _rot(1, flex)
        p2 = j2 - R2 @ np.array([0.0, 0.0, QUAD_LINK_HALF])
        j3 = p2 - R2 @ np.array([0.0, 0.0, QUAD_LINK_HALF])
        R3 = R2 @ _rot(1, knee)
        p3 = j3 - R3 @ np.array([0.0, 0.0, QUAD_LINK_HALF])
        ends = e1 + [p2 + R2 @ np.array([0, 0, s * QUAD_LINK_HALF]) for s in (1, -1)]
        ends += [p3 + R3 @ np.array([0, 0, s * QUAD_LINK_HALF]) for s in (1, -1)]
        low = min(low, min(e[2] for e in ends) - QUAD_LINK_RADIUS)
    return low


def _quad_world(rng: np.random.Generator, max_tries: int = 100):
    """Torso box (5 kg) with a free joint; per leg a hip-ab link (hinge x, a
    lateral capsule), a thigh (hinge y) and a shank (hinge y), capsules 0.2 m
    x r 0.02 m, 0.5 kg.  Base height U(0.3, 0.5); joint angles = nominal crouch
    + N(0, 0.2), resampled until no capsule starts below the plane (straight
    0.6 m legs cannot stand under a 0.3-0.5 m base)."""
    cap_i = capsule_inertia(QUAD_LINK_MASS, QUAD_LINK_RADIUS, QUAD_LINK_HALF)
    # a capsule along the link's y axis: its z axis turned onto y
    lat_q = (-math.sin(math.pi / 4), 0.0, 0.0, math.cos(math.pi / 4))
    links = [_link(-1, M.JOINT_FREE, mass=QUAD_TORSO_MASS, inertia=box_inertia(QUAD_TORSO_MASS, QUAD_TORSO_HALF))]
    geoms = [_geom(M.SHAPE_PLANE, friction=QUAD_MU),
             _geom(M.SHAPE_BOX, link=0, size=QUAD_TORSO_HALF, friction=QUAD_MU)]
    for leg, (hx, side) in enumerate(QUAD_HIPS):
        l1, l2, l3 = 1 + 3 * leg, 2 + 3 * leg, 3 + 3 * leg
        links.append(_link(0, M.JOINT_HINGE, axis=(1.0, 0.0, 0.0), jp=(hx, side * QUAD_TORSO_HALF[1], 0.0),
                           jc=(0.0, -side * QUAD_LINK_HALF, 0.0), mass=QUAD_LINK_MASS, inertia=cap_i))
        links.append(_link(l1, M.JOINT_HINGE, axis=(0.0, 1.0, 0.0), jp=(0.0, side * QUAD_LINK_HALF, 0.0),
                           jc=(0.0, 0.0, QUAD_LINK_HALF), mass=QUAD_LINK_MASS, inertia=cap_i))
        links.append(_link(l2, M.JOINT_HINGE, axis=(0.0, 1.0, 0.0), jp=(0.0, 0.0, -QUAD_LINK_HALF),
                           jc=(0.0, 0.0, QUAD_LINK_HALF), mass=QUAD_LINK_MASS, inertia=cap_i))
        geoms.append(_geom(M.SHAPE_CAPSULE, link=l1, size=(QUAD_LINK_RADIUS, QUAD_LINK_HALF, 0.0), quat=lat_q,
                           friction=QUAD_MU))
        for l in (l2, l3):
            geoms.append(_geom(M.SHAPE_CAPSULE, link=l, size=(QUAD_LINK_RADIUS, QUAD_LINK_HALF, 0.0),
                               friction=QUAD_MU))
    base = float(rng.uniform(0.3, 0.5))
    nominal = np.tile(QUAD_CROUCH, 4)
    for _ in range(max_tries):
        q = nominal + rng.normal(0.0, 0.2, 12)
        if _quad_lowest_point(base, q) > 1e-3:
            break
    else:
        q = nominal
    qpos = np.concatenate([[0.0, 0.0, base, 1.0, 0.0, 0.0, 0.0], q])
    return links, geoms, qpos


def quadruped_batch(n_worlds: int = 16384, seed_index: int = 2, dt: float = 2e-3, iterations: int = 20,
                    solver: int = M.SOLVER_NEWTON, first_world: int = 0) -> M.Batch:
    cs = config_seed(seed_index)
    links, geoms, qps = [], [], []
    for w in range(first_world, first_world + n_worlds):
        l, g, qp = _quad_world(world_rng(cs, w))
        links += l; geoms += g; qps.append(qp)
    b = M.Batch(np.stack(links), [13] * n_worlds, np.zeros(0, M.BODY_DT), [0] * n_worlds, np.stack(geoms),
                [14] * n_worlds, dt, (0.0, 0.0, -9.81), solver, iterations)
    b.qpos[:] = np.concatenate(qps)
    return b


def quadruped_controls(n_worlds: int, block: int, seed_index: int = 2, first_world: int = 0) -> np.ndarray:
    """Joint torques tau ~ N(0, 2) for the 12 actuated DoF of every world,
    for control block `block` (controls are resampled every 20 steps);
    MuJoCo qvel order, the 6 free-root entries zero.  One generator per
    (workload, block, first world) draws the whole block."""
    cs = config_seed(seed_index)
    rng = np.random.default_rng([cs, block, first_world])
    out = np.zeros((n_worlds, 18), np.float32)
    out[:, 6:] = rng.normal(0.0, 2.0, (n_worlds, 12))
    return out.reshape(-1)


# ---------------------------------------------------------------------------
# uneven: a mixed batch of chains and piles with 2..64 bodies
# ---------------------------------------------------------------------------
def uneven_sizes(n_worlds: int, seed_index: int = 3, first_world: int = 0):
    """(kind, n) per world: n = floor(exp(U(ln 2, ln 65))) in [2, 64], kind
    'chain' or 'pile' with probability 1/2 each."""
    cs = config_seed(seed_index)
    out = []
    for w in range(first_world, first_world + n_worlds):
        rng = world_rng(cs, w)
        n = int(math.floor(math.exp(rng.uniform(math.log(2.0), math.log(65.0)))))
        out.append(("chain" if rng.random() < 0.5 else "pile", min(max(n, 2), 64)))
    return out


def _pack(items, dtype):
    out = np.empty(len(items), dtype)
    for i, x in enumerate(items):
        out[i] = x
    return out


def _uneven_chunk(args):
    """Worlds [first, first + count) of the uneven workload as packed arrays."""
    seed_index, first, count = args
    cs = config_seed(seed_index)
    links, bodies, geoms, nl, nb, ng, qps, qvs, taus = [], [], [], [], [], [], [], [], []
    for w in range(first, first + count):
        rng = world_rng(cs, w)
        n = int(math.floor(math.exp(rng.uniform(math.log(2.0), math.log(65.0)))))
        n = min(max(n, 2), 64)
        if rng.random() < 0.5:
            l, q, qd, tau = _chain_world(rng, n)
            links += l; nl.append(len(l)); nb.append(0); ng.append(0)
            qps.append(q); qvs.append(qd); taus.append(tau)
        else:
            b, g, qp = _pile_world(rng, n)
            bodies += b; geoms += g; nl.append(0); nb.append(n); ng.append(len(g))
            qps.append(qp); qvs.append(np.zeros(6 * n)); taus.append(np.zeros(6 * n))
    return (_pack(links, M.LINK_DT), nl, _pack(bodies, M.BODY_DT), nb, _pack(geoms, M.GEOM_DT), ng,
            np.concatenate(qps), np.concatenate(qvs), np.concatenate(taus))


def uneven_batch(n_worlds: int = 32768, seed_index: int = 3, dt: float = 2e-3, iterations: int = 50,
                 first_world: int = 0, workers: int = 0) -> M.Batch:
    """Chains (the chain generator with n hinges) and piles (the pile
    generator with n bodies) mixed in one batch, PGS 50, dt 2e-3; every
    world is rebuilt from its own seed.  Large batches are generated in
    chunks by a spawn-started process pool (`workers` 0 = all cores)."""
    chunk = 1024
    jobs = [(seed_index, f, min(chunk, first_world + n_worlds - f))
            for f in range(first_world, first_world + n_worlds, chunk)]
    if len(jobs) > 1:
        import concurrent.futures as cf
        import multiprocessing as mp
        import os
        nw = workers or min(len(jobs), os.cpu_count() or 1)
        with cf.ProcessPoolExecutor(max_workers=nw, mp_context=mp.get_context("spawn")) as ex:
            parts = list(ex.map(_uneven_chunk, jobs))
    else:
        parts = [_uneven_chunk(j) for j in jobs]
    cat = lambda k: np.concatenate([p[k] for p in parts])
    nl = sum((list(p[1]) for p in parts), [])
    nb = sum((list(p[3]) for p in parts), [])
    ng = sum((list(p[5]) for p in parts), [])
    batch = M.Batch(cat(0), nl, cat(2), nb, cat(4), ng, dt, (0.0, 0.0, -9.81), M.SOLVER_PGS, iterations)
    batch.qpos[:] = cat(6)
    batch.qvel[:] = cat(7)
    batch.qfrc[:] = cat(8)
    return batch
