"""MJCF scenes onto the GPU path: the subset of newt's MJCF loader
(newt/src/mjcf.rs) that produces worlds the GPU step supports.

Follows newt's conventions, restated:
  * a free-jointed top-level body without child bodies is a free `Body`;
    any other top-level body is the root of a tree (free root with a
    <freejoint>, fixed root without joint) (mjcf.rs:889-924);
  * a tree's root link takes the body pose as its joint offset in the parent;
    a child body's link takes body pos + joint pos as its offset in the parent
    and the joint pos as its offset in the child, identity orientations
    (mjcf.rs:1080-1120, 1192-1280); trees do not collide with themselves
    (mjcf.rs:1047);
  * <inertial> gives mass and a diagonal or full inertia about the body origin
    (mjcf.rs:1371-1460);
  * geoms: sphere / box / capsule (size form) / plane, friction defaults to
    0.5, contype / conaffinity to 1, condim to 3, margin and gap to 0,
    solref / solimp to MuJoCo's defaults (mjcf.rs:1891-2035);
  * <default> classes for geom and joint attributes, class / childclass
    lookup (mjcf.rs:364-510);
  * <option> timestep, gravity, iterations, solver, integrator, cone and
    <compiler angle> (mjcf.rs:652-843).
Anything outside the subset raises `MjcfUnsupported`.  Arithmetic that newt
does in f32 (the joint offset sums) is done in f32 here.
"""
from __future__ import annotations

import math
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import model as M


class MjcfUnsupported(ValueError):
    pass


@dataclass
class MjcfScene:
    model: M.WorldModel
    qpos0: np.ndarray        # MuJoCo layout, from the body poses
    qvel0: np.ndarray
    integrator: str = "RK4"  # the XML's option (MuJoCo's default RK4); also set on `model`
    body_names: List[str] = field(default_factory=list)
    link_names: List[str] = field(default_factory=list)


def _floats(s: str) -> List[float]:
    return [float(x) for x in s.split()]


def _f32(x) -> np.ndarray:
    return np.asarray(x, dtype=np.float32)


class _Defaults:
    """`<default>` classes: per class, per element kind, an attribute map
    inherited from the enclosing class ("main" at the top)."""

    def __init__(self, root: ET.Element):
        self.classes: Dict[str, Dict[str, Dict[str, str]]] = {"main": {}}
        top = root.find("default")
        if top is not None:
            self._walk(top, "main", {})

    def _walk(self, e: ET.Element, name: str, parent: Dict[str, Dict[str, str]]):
        own = {k: dict(v) for k, v in parent.items()}
        for c in e:
            if c.tag == "default":
                continue
            own.setdefault(c.tag, {}).update(c.attrib)
        self.classes[name] = own
        for c in e:
            if c.tag == "default":
                self._walk(c, c.attrib.get("class", name), own)

    def attr(self, e: ET.Element, kind: str, key: str, cls: str) -> Optional[str]:
        if key in e.attrib:
            return e.attrib[key]
        c = self.classes.get(e.attrib.get("class", cls), self.classes["main"])
        return c.get(kind, {}).get(key)


def _quat_wxyz(s: str) -> List[float]:
    w, x, y, z = _floats(s)
    n = math.sqrt(w * w + x * x + y * y + z * z)
    if n < 1e-6:
        raise MjcfUnsupported("quaternion has zero norm")
    return [x / n, y / n, z / n, w / n]  # xyzw


def _orientation(e: ET.Element) -> List[float]:
    if "euler" in e.attrib or "axisangle" in e.attrib:
        raise MjcfUnsupported("euler / axisangle orientations are outside the GPU subset (use quat)")
    return _quat_wxyz(e.attrib["quat"]) if "quat" in e.attrib else [0.0, 0.0, 0.0, 1.0]


def _inertial(body: ET.Element):
    ins = body.findall("inertial")
    if len(ins) != 1:
        raise MjcfUnsupported(f"body {body.attrib.get('name')!r}: one <inertial> is required in the GPU subset")
    ine = ins[0]
    if "pos" in ine.attrib and any(v != 0.0 for v in _floats(ine.attrib["pos"])):
        raise MjcfUnsupported("inertial pos must be 0 (newt keeps the COM at the body origin)")
    if "quat" in ine.attrib and _quat_wxyz(ine.attrib["quat"]) != [0.0, 0.0, 0.0, 1.0]:
        raise MjcfUnsupported("inertial quat is not supported (inertia in body axes)")
    mass = float(ine.attrib["mass"])
    if mass <= 0.0:
        raise MjcfUnsupported("mass must be > 0")
    if "diaginertia" in ine.attrib:
        a, b, c = _floats(ine.attrib["diaginertia"])
        inertia = M._diag9(a, b, c)
    elif "fullinertia" in ine.attrib:
        xx, yy, zz, xy, xz, yz = _floats(ine.attrib["fullinertia"])
        inertia = [xx, xy, xz, xy, yy, yz, xz, yz, zz]
    else:
        raise MjcfUnsupported("inertial needs diaginertia or fullinertia")
    return mass, inertia


class _Loader:
    def __init__(self, root: ET.Element):
        self.root = root
        self.defaults = _Defaults(root)
        # World::new() steps RK4 unless <option integrator> says otherwise
        self.scene = MjcfScene(M.WorldModel(integrator=M.INTEGRATOR_RK4), np.zeros(0, np.float32),
                               np.zeros(0, np.float32))
        self.qpos: List[float] = []
        self.qvel: List[float] = []
        self.tree_qpos: List[float] = []
        self.tree_qvel: List[float] = []

    # -- options ---------------------------------------------------------------
    def options(self):
        w = self.scene.model
        comp = self.root.find("compiler")
        if comp is not None and comp.attrib.get("angle", "degree") != "radian":
            raise MjcfUnsupported("only <compiler angle=\"radian\"> is supported")
        if comp is None:
            raise MjcfUnsupported("only <compiler angle=\"radian\"> is supported")
        opt = self.root.find("option")
        a = opt.attrib if opt is not None else {}
        w.dt = float(a.get("timestep", "0.002"))
        w.gravity = tuple(_floats(a.get("gravity", "0 0 -9.81")))
        w.iterations = int(a.get("iterations", "100"))
        solver = a.get("solver", "Newton")
        if solver not in ("PGS", "Newton"):
            raise MjcfUnsupported(f"solver {solver!r}: PGS or Newton")
        w.solver = M.SOLVER_PGS if solver == "PGS" else M.SOLVER_NEWTON
        if a.get("cone", "pyramidal") != "pyramidal":
            raise MjcfUnsupported("only the pyramidal cone is on the GPU path")
        # mjcf.rs:727-742; implicitfast is not on the GPU path
        name = a.get("integrator", "RK4")
        if name in ("RK4", "rk4"):
            self.scene.integrator, w.integrator = "RK4", M.INTEGRATOR_RK4
        elif name in ("Euler", "euler"):
            self.scene.integrator, w.integrator = "Euler", M.INTEGRATOR_EULER
        else:
            raise MjcfUnsupported(f"option integrator={name!r}: RK4 or Euler on the GPU path")

    # -- geoms -----------------------------------------------------------------
    def geom(self, e: ET.Element, cls: str, body: int = -1, link: int = -1) -> M.Geom:
        d = lambda k: self.defaults.attr(e, "geom", k, cls)  # noqa: E731
        ty = d("type") or "sphere"
        if "fromto" in e.attrib:
            raise MjcfUnsupported("geom fromto is outside the GPU subset")
        size = _floats(d("size") or "0")
        shape = {"sphere": M.SHAPE_SPHERE, "box": M.SHAPE_BOX, "capsule": M.SHAPE_CAPSULE,
                 "plane": M.SHAPE_PLANE}.get(ty)
        if shape is None:
            raise MjcfUnsupported(f"geom type {ty!r} is outside the GPU subset")
        if shape == M.SHAPE_PLANE:
            sz = (0.0, 0.0, 0.0)
        elif shape == M.SHAPE_SPHERE:
            sz = (size[0], 0.0, 0.0)
        elif shape == M.SHAPE_BOX:
            sz = tuple(size[:3])
        else:
            sz = (size[0], size[1], 0.0)
        fr = d("friction")
        friction = _floats(fr)[0] if fr is not None else 0.5
        g = M.Geom(shape=shape, body=body, link=link, size=sz,
                   local_pos=tuple(_floats(d("pos"))) if d("pos") else (0.0, 0.0, 0.0),
                   local_quat=tuple(_quat_wxyz(d("quat"))) if d("quat") else (0.0, 0.0, 0.0, 1.0),
                   friction=friction)
        if d("solref"):
            g.solref = tuple(_floats(d("solref")))
        if d("solimp"):
            si = _floats(d("solimp"))
            g.solimp = tuple(si + list(g.solimp[len(si):]))
        g.margin = float(d("margin") or 0.0)
        g.gap = float(d("gap") or 0.0)
        g.condim = int(d("condim") or 3)
        g.group = int(d("contype") or 1)
        g.mask = int(d("conaffinity") or 1)
        return g

    # -- bodies ----------------------------------------------------------------
    def worldbody(self):
        wb = self.root.find("worldbody")
        trees = 0
        for e in wb:
            if e.tag == "geom":
                g = self.geom(e, "main")
                if g.shape != M.SHAPE_PLANE:
                    raise MjcfUnsupported("static geoms must be planes on the GPU path")
                if g.local_quat != (0.0, 0.0, 0.0, 1.0):
                    raise MjcfUnsupported("only +Z planes are supported")
                self.scene.model.add_geom(g)
            elif e.tag == "body":
                free = [c for c in e if c.tag == "freejoint" or (c.tag == "joint" and c.attrib.get("type") == "free")]
                children = [c for c in e if c.tag == "body"]
                if free and not children:
                    self.free_body(e)
                else:
                    trees += 1
                    if trees > 1:
                        raise MjcfUnsupported("one tree per world on the GPU path")
                    self.tree(e, bool(free))
            elif e.tag in ("light", "camera", "site"):
                continue
            else:
                raise MjcfUnsupported(f"<{e.tag}> under <worldbody> is outside the GPU subset")

    def free_body(self, e: ET.Element):
        cls = e.attrib.get("childclass", "main")
        mass, inertia = _inertial(e)
        w = self.scene.model
        b = w.add_body(mass, inertia)
        self.scene.body_names.append(e.attrib.get("name", f"body{b}"))
        for c in e:
            if c.tag == "geom":
                w.add_geom(self.geom(c, cls, body=b))
            elif c.tag not in ("inertial", "freejoint", "joint", "site"):
                raise MjcfUnsupported(f"<{c.tag}> in a free body is outside the GPU subset")
        pos = _floats(e.attrib.get("pos", "0 0 0"))
        x, y, z, qw = _orientation(e)
        self.qpos += pos + [qw, x, y, z]
        self.qvel += [0.0] * 6

    def tree(self, e: ET.Element, free_root: bool):
        w = self.scene.model
        w.tree_self_collision = 0  # MJCF trees skip in-tree pairs (mjcf.rs:1047)
        cls = e.attrib.get("childclass", "main")
        mass, inertia = _inertial(e)
        pos = _floats(e.attrib.get("pos", "0 0 0"))
        quat = _orientation(e)
        w.push_link(M.Link(parent=-1, joint=M.JOINT_FREE if free_root else M.JOINT_FIXED, jp_pos=tuple(pos),
                           jp_quat=tuple(quat), mass=mass, inertia=inertia))
        self.scene.link_names.append(e.attrib.get("name", "root"))
        if free_root:
            x, y, z, qw = quat
            self.tree_qpos += pos + [qw, x, y, z]
            self.tree_qvel += [0.0] * 6
        self.link_children(e, 0, cls)

    def link_children(self, e: ET.Element, link: int, cls: str):
        w = self.scene.model
        for c in e:
            if c.tag == "geom":
                w.add_geom(self.geom(c, cls, link=link))
            elif c.tag == "body":
                self.child_body(c, link, c.attrib.get("childclass", cls))
            elif c.tag not in ("inertial", "freejoint", "joint", "site"):
                raise MjcfUnsupported(f"<{c.tag}> in a tree body is outside the GPU subset")

    def child_body(self, e: ET.Element, parent: int, cls: str):
        w = self.scene.model
        if _orientation(e) != [0.0, 0.0, 0.0, 1.0]:
            raise MjcfUnsupported("non-root bodies need identity orientation (newt v1 subset)")
        mass, inertia = _inertial(e)
        joints = [c for c in e if c.tag in ("joint", "freejoint")]
        if len(joints) > 1:
            raise MjcfUnsupported("one joint per body")
        body_pos = _f32(_floats(e.attrib.get("pos", "0 0 0")))
        jpos = np.zeros(3, np.float32)
        kind, axis, damping, armature = M.JOINT_FIXED, (0.0, 0.0, 1.0), 0.0, 0.0
        if joints:
            j = joints[0]
            d = lambda k: self.defaults.attr(j, "joint", k, cls)  # noqa: E731
            ty = d("type") or "hinge"
            if j.tag == "freejoint" or ty not in ("hinge", "slide"):
                raise MjcfUnsupported(f"joint type {ty!r} below the root is outside the GPU subset")
            if d("ref") and float(d("ref")) != 0.0:
                raise MjcfUnsupported("joint ref must be 0")
            if d("range") and (d("limited") or "true") == "true":
                raise MjcfUnsupported("joint limits are outside the GPU subset")
            kind = M.JOINT_HINGE if ty == "hinge" else M.JOINT_SLIDE
            a = _f32(_floats(d("axis")))
            n = float(np.sqrt(np.float32(a @ a)))
            axis = tuple(float(x) for x in (a / np.float32(n)))
            damping = float(d("damping") or 0.0)
            armature = float(d("armature") or 0.0)
            if d("pos"):
                jpos = _f32(_floats(d("pos")))
        jp = body_pos + jpos  # f32, as newt adds the two Vec3s
        w.push_link(M.Link(parent=parent, joint=kind, axis=axis, damping=damping, armature=armature,
                           jp_pos=tuple(float(x) for x in jp), jc_pos=tuple(float(x) for x in jpos), mass=mass,
                           inertia=inertia))
        link = len(w.links) - 1
        self.scene.link_names.append(e.attrib.get("name", f"link{link}"))
        if kind != M.JOINT_FIXED:
            self.tree_qpos.append(0.0)
            self.tree_qvel.append(0.0)
        self.link_children(e, link, cls)


def load_mjcf(source: str) -> MjcfScene:
    """Parse an MJCF document (a string, or a path ending in .xml)."""
    if source.lstrip().startswith("<"):
        root = ET.fromstring(source)
    else:
        root = ET.parse(source).getroot()
    if root.tag != "mujoco":
        raise MjcfUnsupported("the document root must be <mujoco>")
    for c in root:
        if c.tag not in ("compiler", "option", "default", "worldbody", "size", "visual", "statistic"):
            raise MjcfUnsupported(f"<{c.tag}> is outside the GPU subset")
    ld = _Loader(root)
    ld.options()
    ld.worldbody()
    s = ld.scene
    # MuJoCo layout: free bodies first (World::mujoco_qpos order), then the tree
    s.qpos0 = np.asarray(ld.qpos + ld.tree_qpos, np.float32)
    s.qvel0 = np.asarray(ld.qvel + ld.tree_qvel, np.float32)
    return s
