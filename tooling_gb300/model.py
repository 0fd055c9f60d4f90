"""Host-side model description for the newt GPU C ABI (include/newt_gpu.h).

The ctypes structures below are the exact layout of ``newt_link_desc``,
``newt_body_desc``, ``newt_geom_desc`` and ``newt_model_desc``.  ``WorldModel``
is a small builder that mirrors how a newt ``World`` is assembled
(``World::add_body`` / ``add_tree`` / ``add_geom``, newt/src/world.rs:950-981;
``Tree::push_link``, newt/src/tree.rs:275-331; the ``Geom`` constructors,
newt/src/geom.rs:494-760), so a scene written against newt reads the same
here.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

JOINT_FREE, JOINT_FIXED, JOINT_HINGE, JOINT_SLIDE, JOINT_BALL = 0, 1, 2, 3, 4
SHAPE_PLANE, SHAPE_SPHERE, SHAPE_BOX, SHAPE_CAPSULE, SHAPE_CYLINDER, SHAPE_ELLIPSOID = 0, 1, 2, 3, 4, 5
SOLVER_PGS, SOLVER_NEWTON = 1, 2
CONE_PYRAMIDAL, CONE_ELLIPTIC = 0, 1
INTEGRATOR_EULER, INTEGRATOR_RK4 = 0, 1
JOINT_NQ = {JOINT_FREE: 7, JOINT_FIXED: 0, JOINT_HINGE: 1, JOINT_SLIDE: 1, JOINT_BALL: 4}
JOINT_NV = {JOINT_FREE: 6, JOINT_FIXED: 0, JOINT_HINGE: 1, JOINT_SLIDE: 1, JOINT_BALL: 3}


class LinkDesc(C.Structure):
    _fields_ = [
        ("parent", C.c_int32), ("joint", C.c_int32), ("axis", C.c_float * 3),
        ("damping", C.c_float), ("armature", C.c_float), ("free_damping", C.c_float),
        ("jp_pos", C.c_float * 3), ("jp_quat", C.c_float * 4),
        ("jc_pos", C.c_float * 3), ("jc_quat", C.c_float * 4),
        ("mass", C.c_float), ("inertia", C.c_float * 9),
    ]


class BodyDesc(C.Structure):
    _fields_ = [("mass", C.c_float), ("inertia", C.c_float * 9)]


class GeomDesc(C.Structure):
    _fields_ = [
        ("shape", C.c_int32), ("body", C.c_int32), ("link", C.c_int32), ("size", C.c_float * 3),
        ("local_pos", C.c_float * 3), ("local_quat", C.c_float * 4), ("friction", C.c_float),
        ("solref", C.c_float * 2), ("solimp", C.c_float * 5), ("margin", C.c_float), ("gap", C.c_float),
        ("condim", C.c_int32), ("group", C.c_uint32), ("mask", C.c_uint32),
        ("torsional_friction", C.c_float), ("rolling_friction", C.c_float),
    ]


class ModelDesc(C.Structure):
    _fields_ = [
        ("n_links", C.c_int32), ("n_bodies", C.c_int32), ("n_geoms", C.c_int32),
        ("links", C.POINTER(LinkDesc)), ("bodies", C.POINTER(BodyDesc)), ("geoms", C.POINTER(GeomDesc)),
        ("dt", C.c_float), ("gravity", C.c_float * 3), ("solver", C.c_int32), ("iterations", C.c_int32),
        ("tree_self_collision", C.c_int32), ("integrator", C.c_int32), ("cone", C.c_int32),
        ("magnetic_field", C.c_float * 3), ("n_pairs", C.c_int32), ("pairs", C.POINTER(C.c_int32)),
    ]


def _diag9(a, b, c):
    return [a, 0.0, 0.0, 0.0, b, 0.0, 0.0, 0.0, c]


def solid_sphere_inertia(mass: float, r: float) -> List[float]:
    """newt/src/geom.rs:934-937 (evaluated in f32)."""
    f = np.float32
    i = f(f(f(f(2.0) / f(5.0)) * f(mass)) * f(r)) * f(r)
    return _diag9(i, i, i)


def solid_box_inertia(mass: float, h: Sequence[float]) -> List[float]:
    """newt/src/geom.rs:939-947 (evaluated in f32)."""
    f = np.float32
    hx2, hy2, hz2 = f(h[0]) * f(h[0]), f(h[1]) * f(h[1]), f(h[2]) * f(h[2])
    m3 = f(mass) / f(3.0)
    return _diag9(m3 * (hy2 + hz2), m3 * (hx2 + hz2), m3 * (hx2 + hy2))


def solid_cylinder_inertia(mass: float, radius: float, half_height: float) -> List[float]:
    """newt/src/geom.rs:993-999 (evaluated in f32)."""
    f = np.float32
    m, r2, h2 = f(mass), f(radius) * f(radius), f(half_height) * f(half_height)
    i_zz = f(0.5) * m * r2
    i_xx = (f(1.0) / f(12.0)) * m * (f(3.0) * r2 + f(4.0) * h2)
    return _diag9(i_xx, i_xx, i_zz)


def solid_ellipsoid_inertia(mass: float, semi_axes: Sequence[float]) -> List[float]:
    """newt/src/geom.rs:1009-1017 (evaluated in f32)."""
    f = np.float32
    m = f(mass)
    a2, b2, c2 = (f(x) * f(x) for x in semi_axes)
    k = f(1.0) / f(5.0)
    return _diag9(k * m * (b2 + c2), k * m * (a2 + c2), k * m * (a2 + b2))


def solid_capsule_inertia(mass: float, radius: float, half_height: float) -> List[float]:
    """newt/src/geom.rs:949-966 (evaluated in f32)."""
    f = np.float32
    r, h, m = f(radius), f(half_height), f(mass)
    vol_cyl = r * r * (f(2.0) * h)
    vol_caps = (f(4.0) / f(3.0)) * r * r * r
    total = vol_cyl + vol_caps
    m_c = m * (vol_cyl / total)
    m_s = m - m_c
    i_zz = f(0.5) * m_c * r * r + (f(2.0) / f(5.0)) * m_s * r * r
    offset = h + f(3.0) / f(8.0) * r
    hemi = (f(83.0) / f(320.0)) * m_s * r * r
    i_xx = (f(1.0) / f(12.0)) * m_c * (f(3.0) * r * r + f(4.0) * h * h) + hemi + m_s * offset * offset
    return _diag9(i_xx, i_xx, i_zz)


@dataclass
class Link:
    parent: int
    joint: int
    axis: Sequence[float] = (0.0, 0.0, 1.0)
    damping: float = 0.0
    armature: float = 0.0
    free_damping: float = 0.0
    jp_pos: Sequence[float] = (0.0, 0.0, 0.0)
    jp_quat: Sequence[float] = (0.0, 0.0, 0.0, 1.0)
    jc_pos: Sequence[float] = (0.0, 0.0, 0.0)
    jc_quat: Sequence[float] = (0.0, 0.0, 0.0, 1.0)
    mass: float = 1.0
    inertia: Sequence[float] = tuple(_diag9(1.0, 1.0, 1.0))


@dataclass
class Geom:
    shape: int
    body: int = -1
    link: int = -1
    size: Sequence[float] = (0.0, 0.0, 0.0)
    local_pos: Sequence[float] = (0.0, 0.0, 0.0)
    local_quat: Sequence[float] = (0.0, 0.0, 0.0, 1.0)
    friction: float = 1.0
    solref: Sequence[float] = (0.02, 1.0)
    solimp: Sequence[float] = (0.9, 0.95, 0.001, 0.5, 2.0)
    margin: float = 0.0
    gap: float = 0.0
    condim: int = 3
    group: int = 0xFFFFFFFF
    mask: int = 0xFFFFFFFF
    torsional_friction: float = 0.0  # condim >= 4 (newt Geom::torsional_friction)
    rolling_friction: float = 0.0    # condim 6 (newt Geom::rolling_friction)


@dataclass
class WorldModel:
    """One world's model: at most one kinematic tree plus free bodies and geoms."""

    dt: float = 0.005
    gravity: Sequence[float] = (0.0, 0.0, -9.81)
    solver: int = SOLVER_PGS
    iterations: int = 20
    tree_self_collision: int = 0
    integrator: int = 0  # INTEGRATOR_EULER or INTEGRATOR_RK4
    cone: int = CONE_PYRAMIDAL  # SolverConfig::cone
    magnetic_field: Sequence[float] = (0.0, -0.5, 0.0)  # World::new's (newt/src/world.rs:332)
    pair_list: Optional[List[Tuple[int, int]]] = None  # World::pair_list: explicit geom pairs, in order
    links: List[Link] = field(default_factory=list)
    bodies: List[tuple] = field(default_factory=list)  # (mass, inertia9)
    geoms: List[Geom] = field(default_factory=list)

    def add_body(self, mass: float, inertia9: Sequence[float]) -> int:
        self.bodies.append((float(mass), list(inertia9)))
        return len(self.bodies) - 1

    def push_link(self, link: Link) -> int:
        self.links.append(link)
        return len(self.links) - 1

    def add_geom(self, g: Geom) -> int:
        self.geoms.append(g)
        return len(self.geoms) - 1

    # MuJoCo-layout dimensions (include/newt_gpu.h header comment)
    @property
    def nq(self) -> int:
        return 7 * len(self.bodies) + sum(JOINT_NQ[l.joint] for l in self.links)

    @property
    def nv(self) -> int:
        return 6 * len(self.bodies) + sum(JOINT_NV[l.joint] for l in self.links)


class PackedModels:
    """ctypes arrays for a list of WorldModel, kept alive with the descriptors."""

    def __init__(self, models: Sequence[WorldModel]):
        self._keep = []
        self.descs = (ModelDesc * len(models))()
        for i, m in enumerate(models):
            links = (LinkDesc * max(1, len(m.links)))()
            for k, l in enumerate(m.links):
                d = links[k]
                d.parent, d.joint = l.parent, l.joint
                d.axis[:] = list(l.axis)
                d.damping, d.armature, d.free_damping = l.damping, l.armature, l.free_damping
                d.jp_pos[:] = list(l.jp_pos); d.jp_quat[:] = list(l.jp_quat)
                d.jc_pos[:] = list(l.jc_pos); d.jc_quat[:] = list(l.jc_quat)
                d.mass = l.mass
                d.inertia[:] = list(l.inertia)
            bodies = (BodyDesc * max(1, len(m.bodies)))()
            for k, (mass, inertia) in enumerate(m.bodies):
                bodies[k].mass = mass
                bodies[k].inertia[:] = list(inertia)
            geoms = (GeomDesc * max(1, len(m.geoms)))()
            for k, g in enumerate(m.geoms):
                d = geoms[k]
                d.shape, d.body, d.link = g.shape, g.body, g.link
                d.size[:] = list(g.size)
                d.local_pos[:] = list(g.local_pos); d.local_quat[:] = list(g.local_quat)
                d.friction = g.friction
                d.solref[:] = list(g.solref); d.solimp[:] = list(g.solimp)
                d.margin, d.gap, d.condim = g.margin, g.gap, g.condim
                d.group, d.mask = g.group & 0xFFFFFFFF, g.mask & 0xFFFFFFFF
                d.torsional_friction, d.rolling_friction = g.torsional_friction, g.rolling_friction
            self._keep += [links, bodies, geoms]
            md = self.descs[i]
            md.n_links, md.n_bodies, md.n_geoms = len(m.links), len(m.bodies), len(m.geoms)
            md.links = C.cast(links, C.POINTER(LinkDesc))
            md.bodies = C.cast(bodies, C.POINTER(BodyDesc))
            md.geoms = C.cast(geoms, C.POINTER(GeomDesc))
            md.dt = m.dt
            md.gravity[:] = list(m.gravity)
            md.solver, md.iterations = m.solver, m.iterations
            md.tree_self_collision = m.tree_self_collision
            md.integrator = m.integrator
            md.cone = m.cone
            md.magnetic_field[:] = list(m.magnetic_field)
            if m.pair_list is not None:
                pl = (C.c_int32 * max(1, 2 * len(m.pair_list)))(*[int(x) for pr in m.pair_list for x in pr])
                self._keep.append(pl)
                md.n_pairs = len(m.pair_list)
                md.pairs = C.cast(pl, C.POINTER(C.c_int32))

    def __len__(self) -> int:
        return len(self.descs)


def static_plane(point=(0.0, 0.0, 0.0), normal=(0.0, 0.0, 1.0), friction: float = 1.0) -> Geom:
    """``Geom::static_plane`` (newt/src/geom.rs:494) for an upward normal."""
    n = np.asarray(normal, dtype=np.float64)
    n = n / np.linalg.norm(n)
    if n[2] > 1.0 - 1e-6:
        quat = (0.0, 0.0, 0.0, 1.0)
    else:
        raise ValueError("only +Z planes are used by this package's scenes")
    return Geom(shape=SHAPE_PLANE, local_pos=tuple(point), local_quat=quat, friction=friction)


def _np_dtype(struct):
    """numpy structured dtype with the exact layout of a ctypes Structure."""
    names, formats, offsets = [], [], []
    for name, ctype in struct._fields_:
        f = getattr(struct, name)
        names.append(name)
        offsets.append(f.offset)
        if hasattr(ctype, "_length_"):
            base = ctype._type_
            formats.append((np.dtype(base), (ctype._length_,)))
        else:
            formats.append(np.dtype(ctype))
    return np.dtype({"names": names, "formats": formats, "offsets": offsets, "itemsize": C.sizeof(struct)})


LINK_DT = _np_dtype(LinkDesc)
BODY_DT = _np_dtype(BodyDesc)
GEOM_DT = _np_dtype(GeomDesc)


class Batch:
    """Many worlds described by flat numpy arrays (vectorised scene building).

    ``links``/``bodies``/``geoms`` are structured arrays with the C layout;
    world ``w`` owns ``links[link_off[w]:link_off[w]+n_links[w]]`` and so on.
    ``descs`` is a ctypes ``ModelDesc`` array pointing into those buffers: one
    model per world.  ``qpos``/``qvel``/``qfrc`` are MuJoCo-layout state blocks
    concatenated in world order.
    """

    def __init__(self, links, n_links, bodies, n_bodies, geoms, n_geoms, dt, gravity, solver, iterations,
                 self_coll=0, integrator=INTEGRATOR_EULER, cone=CONE_PYRAMIDAL, magnetic_field=(0.0, -0.5, 0.0)):
        self.links = np.ascontiguousarray(links)
        self.bodies = np.ascontiguousarray(bodies)
        self.geoms = np.ascontiguousarray(geoms)
        W = len(n_links)
        self.n_worlds = W
        self.n_links = np.asarray(n_links, np.int64)
        self.n_bodies = np.asarray(n_bodies, np.int64)
        self.n_geoms = np.asarray(n_geoms, np.int64)
        self.link_off = np.concatenate([[0], np.cumsum(self.n_links)[:-1]]).astype(np.int64)
        self.body_off = np.concatenate([[0], np.cumsum(self.n_bodies)[:-1]]).astype(np.int64)
        self.geom_off = np.concatenate([[0], np.cumsum(self.n_geoms)[:-1]]).astype(np.int64)
        nq = 7 * self.n_bodies.copy()
        nv = 6 * self.n_bodies.copy()
        if len(self.links):
            jt = self.links["joint"]
            jq = np.select([jt == JOINT_FREE, jt == JOINT_FIXED, jt == JOINT_BALL], [7, 0, 4], 1)
            jv = np.select([jt == JOINT_FREE, jt == JOINT_FIXED, jt == JOINT_BALL], [6, 0, 3], 1)
            cq = np.concatenate([[0], np.cumsum(jq)])
            cv = np.concatenate([[0], np.cumsum(jv)])
            nq += cq[self.link_off + self.n_links] - cq[self.link_off]
            nv += cv[self.link_off + self.n_links] - cv[self.link_off]
        self.nq = nq
        self.nv = nv
        self.q_off = np.concatenate([[0], np.cumsum(nq)[:-1]]).astype(np.int64)
        self.v_off = np.concatenate([[0], np.cumsum(nv)[:-1]]).astype(np.int64)
        self.descs = (ModelDesc * W)()
        lp = self.links.ctypes.data if len(self.links) else 0
        bp = self.bodies.ctypes.data if len(self.bodies) else 0
        gp = self.geoms.ctypes.data if len(self.geoms) else 0
        dt = np.broadcast_to(np.asarray(dt, np.float32), (W,))
        iters = np.broadcast_to(np.asarray(iterations, np.int32), (W,))
        solver = np.broadcast_to(np.asarray(solver, np.int32), (W,))
        for w in range(W):
            d = self.descs[w]
            d.n_links, d.n_bodies, d.n_geoms = int(self.n_links[w]), int(self.n_bodies[w]), int(self.n_geoms[w])
            d.links = C.cast(lp + int(self.link_off[w]) * LINK_DT.itemsize, C.POINTER(LinkDesc))
            d.bodies = C.cast(bp + int(self.body_off[w]) * BODY_DT.itemsize, C.POINTER(BodyDesc))
            d.geoms = C.cast(gp + int(self.geom_off[w]) * GEOM_DT.itemsize, C.POINTER(GeomDesc))
            d.dt = float(dt[w])
            d.gravity[0], d.gravity[1], d.gravity[2] = gravity
            d.solver, d.iterations, d.tree_self_collision = int(solver[w]), int(iters[w]), int(self_coll)
            d.integrator = int(integrator)
            d.cone = int(cone)
            d.magnetic_field[:] = [float(x) for x in magnetic_field]
        self.qpos = np.zeros(int(nq.sum()), np.float32)
        self.qvel = np.zeros(int(nv.sum()), np.float32)
        self.qfrc = np.zeros(int(nv.sum()), np.float32)

    def __len__(self) -> int:
        return self.n_worlds

    def subset(self, idx):
        """Views of the state blocks for a list of worlds (for oracle calls)."""
        idx = np.asarray(idx)
        qp = np.concatenate([self.qpos[self.q_off[w]:self.q_off[w] + self.nq[w]] for w in idx])
        qv = np.concatenate([self.qvel[self.v_off[w]:self.v_off[w] + self.nv[w]] for w in idx])
        qf = np.concatenate([self.qfrc[self.v_off[w]:self.v_off[w] + self.nv[w]] for w in idx])
        return qp, qv, qf
