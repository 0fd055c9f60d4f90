"""newt's JSON scene format (the subset the GPU path steps) -> WorldModel.

Follows newt/src/model.rs (load_from_path :185, build_scene :778-1142):
  * root: version, gravity, timestep, integrator (RK4 | Euler, default RK4 as
    World::new; implicitfast refused, :1536-1562), solver {mode penalty | pgs |
    newton, iterations, cone pyramidal} (:1564-1614), bodies, trees, geoms,
    sites (names kept, frames unused);
  * bodies (:1143-1186): mass > 0, inertia diag | tensor | solid {box, sphere,
    capsule, cylinder, ellipsoid} evaluated in f32 by newt's formulas
    (:326-477), pose {position, orientation [x, y, z, w] renormalised |
    orientation_axis_angle} (:479-528), velocity {linear, angular_body};
  * one tree (:1188-1399): links with name, parent (by name, earlier links),
    joint free | fixed | hinge | slide {axis, damping, armature} (:530-776),
    joint offsets (identity orientations below the root), mass, inertia;
    self_collide (default false);
  * geoms (:1417-1519): shape plane | sphere | box | capsule | cylinder |
    ellipsoid (:1787-1904), attach static | body | link (:1906-1962), local
    offset / orientation, friction (default 0.5), solref {timeconst,
    dampratio}, solimp {dmin, dmax, width, midpoint, power}, margin, gap,
    condim; collision group and mask all ones.
Also the solver's cone (model.rs:1557-1597) and explicit contact pairs
(`contact_pairs.explicit`, model.rs:1033-1041, 3208-3250; taken by
tree-contact worlds).  Anything else (meshes, height fields, actuators,
auto-pair exclusions, equalities, sensors, tendons, ball joints, joint
limits, mocap, rolling or torsional friction, more than one tree) raises
`JsonUnsupported`.  Axis-angle
orientations use numpy's f32 sin/cos (newt's polynomial may differ by an ulp).
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field
from typing import Dict, List

import numpy as np

from . import model as M

f32 = np.float32
_ROOT_KEYS = {"version", "gravity", "timestep", "integrator", "solver", "bodies", "trees", "geoms", "sites",
              "contact_pairs"}


class JsonUnsupported(ValueError):
    pass


@dataclass
class JsonScene:
    model: M.WorldModel
    qpos0: np.ndarray  # MuJoCo layout
    qvel0: np.ndarray
    body_names: List[str] = field(default_factory=list)
    link_names: List[str] = field(default_factory=list)
    geom_names: List[str] = field(default_factory=list)
    site_names: List[str] = field(default_factory=list)


def _keys(obj: dict, allowed, where: str):
    extra = set(obj) - set(allowed)
    if extra:
        raise JsonUnsupported(f"{where}: {sorted(extra)} outside the GPU subset")


def _vec3(v, where):
    if not isinstance(v, list) or len(v) != 3:
        raise JsonUnsupported(f"{where}: expected 3 numbers")
    return [float(f32(x)) for x in v]


def _renorm(q):  # Quat::renormalize in f32 (math.rs:591-598)
    q = [f32(x) for x in q]
    n = np.sqrt(f32(f32(f32(q[0] * q[0] + q[1] * q[1]) + q[2] * q[2]) + q[3] * q[3]))
    if n == 0:
        return [0.0, 0.0, 0.0, 1.0]
    return [float(x / n) for x in q]


def _axis_angle(axis, angle):  # Quat::from_axis_angle (math.rs:574-580)
    a = [f32(x) for x in axis]
    n = np.sqrt(f32(f32(a[0] * a[0] + a[1] * a[1]) + a[2] * a[2]))
    a = [x / n for x in a]
    half = f32(angle) * f32(0.5)
    s, c = np.sin(half, dtype=np.float32), np.cos(half, dtype=np.float32)
    return [float(a[0] * s), float(a[1] * s), float(a[2] * s), float(c)]


def _pose(v, where):
    if v is None:
        return [0.0, 0.0, 0.0], [0.0, 0.0, 0.0, 1.0]
    _keys(v, ("position", "orientation", "orientation_axis_angle"), where)
    pos = _vec3(v.get("position", [0.0, 0.0, 0.0]), where + ".position")
    if "orientation" in v and "orientation_axis_angle" in v:
        raise JsonUnsupported(f"{where}: orientation given twice")
    if "orientation" in v:
        return pos, _renorm(v["orientation"])
    if "orientation_axis_angle" in v:
        aa = v["orientation_axis_angle"]
        return pos, _axis_angle(aa["axis"], aa["angle"])
    return pos, [0.0, 0.0, 0.0, 1.0]


def _inertia(v, mass, where):
    kind = v.get("kind")
    if kind == "diag":
        a, b, c = _vec3(v["values"], where)
        return M._diag9(a, b, c)
    if kind == "tensor":
        xx, yy, zz, xy, xz, yz = (float(f32(x)) for x in v["values"])
        return [xx, xy, xz, xy, yy, yz, xz, yz, zz]
    if kind == "solid":
        s = v["shape"]
        k = s.get("kind")
        if k == "box":
            return M.solid_box_inertia(mass, _vec3(s["half_extents"], where))
        if k == "sphere":
            return M.solid_sphere_inertia(mass, s["radius"])
        if k == "capsule":
            return M.solid_capsule_inertia(mass, s["radius"], s["half_height"])
        if k == "cylinder":
            return M.solid_cylinder_inertia(mass, s["radius"], s["half_height"])
        if k == "ellipsoid":
            return M.solid_ellipsoid_inertia(mass, _vec3(s["semi_axes"], where))
    raise JsonUnsupported(f"{where}: inertia kind {kind!r}")


_SHAPES = {"plane": M.SHAPE_PLANE, "sphere": M.SHAPE_SPHERE, "box": M.SHAPE_BOX, "capsule": M.SHAPE_CAPSULE,
           "cylinder": M.SHAPE_CYLINDER, "ellipsoid": M.SHAPE_ELLIPSOID}


def _shape(s, where):
    k = s.get("kind")
    if k not in _SHAPES:
        raise JsonUnsupported(f"{where}: shape {k!r} outside the GPU subset")
    if k == "plane":
        return M.SHAPE_PLANE, (0.0, 0.0, 0.0)
    if k == "sphere":
        return M.SHAPE_SPHERE, (float(f32(s["radius"])), 0.0, 0.0)
    if k in ("box", "ellipsoid"):
        return _SHAPES[k], tuple(_vec3(s["half_extents" if k == "box" else "semi_axes"], where))
    return _SHAPES[k], (float(f32(s["radius"])), float(f32(s["half_height"])), 0.0)


def load_json(source: str) -> JsonScene:
    """Parse a newt JSON scene (a path or the JSON text itself)."""
    text = source if source.lstrip().startswith("{") else open(source).read()
    root = json.loads(text)
    _keys(root, _ROOT_KEYS, "root")
    w = M.WorldModel(integrator=M.INTEGRATOR_RK4, solver=0, iterations=20)
    w.gravity = tuple(_vec3(root.get("gravity", [0.0, 0.0, -9.81]), "gravity"))
    w.dt = float(f32(root.get("timestep", 0.005)))
    integ = root.get("integrator", "RK4")
    if integ in ("RK4", "rk4"):
        w.integrator = M.INTEGRATOR_RK4
    elif integ in ("Euler", "euler"):
        w.integrator = M.INTEGRATOR_EULER
    else:
        raise JsonUnsupported(f"integrator {integ!r}: RK4 or Euler on the GPU path")
    if "solver" in root:
        sv = root["solver"]
        _keys(sv, ("mode", "iterations", "cone"), "solver")
        mode = sv.get("mode", "penalty")
        w.solver = {"penalty": 0, "pgs": M.SOLVER_PGS, "newton": M.SOLVER_NEWTON}[mode]
        w.iterations = int(sv.get("iterations", 20))
        cone = sv.get("cone", "pyramidal")  # model.rs:1557-1597
        if cone not in ("pyramidal", "elliptic"):
            raise JsonUnsupported(f"solver.cone {cone!r}")
        w.cone = M.CONE_ELLIPTIC if cone == "elliptic" else M.CONE_PYRAMIDAL
    scene = JsonScene(w, np.zeros(0, np.float32), np.zeros(0, np.float32))
    qpos, qvel = [], []
    bodies: Dict[str, int] = {}
    for i, b in enumerate(root.get("bodies", [])):
        where = f"bodies[{i}]"
        _keys(b, ("name", "mass", "inertia", "pose", "velocity"), where)
        mass = float(f32(b["mass"]))
        if not mass > 0:
            raise JsonUnsupported(f"{where}: mass must be > 0")
        bi = w.add_body(mass, _inertia(b["inertia"], mass, where + ".inertia"))
        bodies[b.get("name", f"body{i}")] = bi
        scene.body_names.append(b.get("name", ""))
        pos, ori = _pose(b.get("pose"), where + ".pose")
        vel = b.get("velocity", {})
        _keys(vel, ("linear", "angular_body"), where + ".velocity")
        qpos += pos + [ori[3], ori[0], ori[1], ori[2]]
        qvel += _vec3(vel.get("linear", [0.0, 0.0, 0.0]), where) + _vec3(vel.get("angular_body", [0.0, 0.0, 0.0]), where)
    links: Dict[str, int] = {}
    trees = root.get("trees", [])
    if len(trees) > 1:
        raise JsonUnsupported("one tree per world on the GPU path")
    tree_name = None
    for t in trees:
        _keys(t, ("name", "self_collide", "links"), "trees[0]")
        tree_name = t["name"]
        w.tree_self_collision = int(bool(t.get("self_collide", False)))
        for i, l in enumerate(t["links"]):
            where = f"trees[0].links[{i}]"
            _keys(l, ("name", "parent", "joint", "joint_offset_in_parent", "joint_offset_in_child", "mass", "inertia"),
                  where)
            j = l["joint"]
            kind = j.get("kind")
            parent = -1 if i == 0 else links[l["parent"]]
            jp_pos, jp_quat = _pose(l.get("joint_offset_in_parent"), where + ".joint_offset_in_parent")
            jc_pos, jc_quat = _pose(l.get("joint_offset_in_child"), where + ".joint_offset_in_child")
            mass = float(f32(l["mass"]))
            link = M.Link(parent=parent, joint=M.JOINT_FIXED, jp_pos=tuple(jp_pos), jp_quat=list(jp_quat),
                          jc_pos=tuple(jc_pos), jc_quat=list(jc_quat), mass=mass,
                          inertia=_inertia(l["inertia"], mass, where + ".inertia"))
            if kind == "free":
                _keys(j, ("kind", "damping"), where + ".joint")
                link.joint, link.free_damping = M.JOINT_FREE, float(f32(j.get("damping", 0.0)))
            elif kind in ("hinge", "slide"):
                _keys(j, ("kind", "axis", "damping", "armature"), where + ".joint")
                link.joint = M.JOINT_HINGE if kind == "hinge" else M.JOINT_SLIDE
                link.axis = tuple(_vec3(j["axis"], where + ".joint.axis"))
                link.damping = float(f32(j.get("damping", 0.0)))
                link.armature = float(f32(j.get("armature", 0.0)))
            elif kind != "fixed":
                raise JsonUnsupported(f"{where}: joint {kind!r} outside the GPU subset")
            w.push_link(link)
            links[l["name"]] = i
            scene.link_names.append(l["name"])
            if kind == "free":
                qpos += jp_pos + [jp_quat[3], jp_quat[0], jp_quat[1], jp_quat[2]]
                qvel += [0.0] * 6
            elif kind in ("hinge", "slide"):
                qpos.append(0.0)
                qvel.append(0.0)
    for i, g in enumerate(root.get("geoms", [])):
        where = f"geoms[{i}]"
        _keys(g, ("name", "shape", "attach", "local_offset", "local_orientation", "friction", "solref", "solimp",
                  "margin", "gap", "condim"), where)
        shape, size = _shape(g["shape"], where + ".shape")
        at = g["attach"]
        body = link = -1
        if at["kind"] == "body":
            body = bodies[at["body"]]
        elif at["kind"] == "link":
            if at["tree"] != tree_name:
                raise JsonUnsupported(f"{where}: unknown tree {at['tree']!r}")
            link = links[at["link"]]
        elif at["kind"] != "static":
            raise JsonUnsupported(f"{where}: attach {at['kind']!r}")
        geom = M.Geom(shape=shape, body=body, link=link, size=size, friction=float(f32(g.get("friction", 0.5))),
                      local_pos=tuple(_vec3(g.get("local_offset", [0.0, 0.0, 0.0]), where)),
                      local_quat=tuple(_renorm(g["local_orientation"]) if "local_orientation" in g
                                       else (0.0, 0.0, 0.0, 1.0)))
        if "solref" in g:
            geom.solref = (float(f32(g["solref"]["timeconst"])), float(f32(g["solref"]["dampratio"])))
        if "solimp" in g:
            si = g["solimp"]
            geom.solimp = tuple(float(f32(si[k])) for k in ("dmin", "dmax", "width", "midpoint", "power"))
        geom.margin, geom.gap = float(f32(g.get("margin", 0.0))), float(f32(g.get("gap", 0.0)))
        geom.condim = int(g.get("condim", 3))
        geom.group, geom.mask = 0xFFFFFFFF, 0xFFFFFFFF
        w.add_geom(geom)
        scene.geom_names.append(g["name"])
    if "contact_pairs" in root:  # model.rs:1033-1041, 3208-3250: explicit pairs, as (min, max)
        cp = root["contact_pairs"]
        _keys(cp, ("explicit",), "contact_pairs")  # "disable" (auto-pair exclusions) is outside the subset
        index = {n: k for k, n in enumerate(scene.geom_names)}
        pairs = []
        for i, pr in enumerate(cp.get("explicit", [])):
            _keys(pr, ("a", "b"), f"contact_pairs.explicit[{i}]")
            a, b = index[pr["a"]], index[pr["b"]]
            pairs.append((min(a, b), max(a, b)))
        w.pair_list = pairs
    scene.site_names = [s.get("name", "") for s in root.get("sites", [])]
    scene.qpos0 = np.array(qpos, np.float32)
    scene.qvel0 = np.array(qvel, np.float32)
    return scene
