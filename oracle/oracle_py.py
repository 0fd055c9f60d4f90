"""Oracle (test infrastructure only): ctypes bindings to ``liboracle.so``.

Only the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  The shipped GPU path never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH) or _stale():
        subprocess.check_call(["make", "-s", "-C", HERE])
    return LIB_PATH


def _stale() -> bool:
    t = os.path.getmtime(LIB_PATH)
    srcs = [os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith((".hpp", ".cpp"))]
    srcs.append(os.path.join(HERE, "..", "include", "newt_gpu.h"))
    return any(os.path.getmtime(s) > t for s in srcs)


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        L.oracle_run.argtypes = [P, C.c_int, P, P, P, P, C.c_int, C.c_int, C.c_int, P, P, P, C.c_int]
        L.oracle_run.restype = C.c_int
        L.oracle_run_ex.argtypes = [P, C.c_int, P, P, P, P, C.c_int, C.c_int, C.c_int, P, P, P, C.c_int, C.c_int]
        L.oracle_run_ex.restype = C.c_int
        L.oracle_tree_impulses.argtypes = [P, P, P, P, C.c_int, C.c_int, P, P, P]
        L.oracle_tree_impulses.restype = C.c_int
        L.oracle_tree_impulses_ex.argtypes = [P, P, P, P, C.c_int, C.c_int, P, P, P, C.c_int]
        L.oracle_tree_impulses_ex.restype = C.c_int
        L.oracle_sensors.argtypes = [P, P, P, P, C.c_int, C.c_int, P, P, P]
        L.oracle_sensors.restype = C.c_int
        L.oracle_contact_sensors.argtypes = [P, P, P, C.c_int, C.c_int, P, P, P, P, P]
        L.oracle_tree_contact_sensors.argtypes = [P, P, P, P, C.c_int, C.c_int, P, P, P, P, P]
        L.oracle_tree_contact_sensors.restype = C.c_int
        L.oracle_contact_sensors.restype = C.c_int
        L.oracle_ccd_pair.argtypes = [C.c_int, C.c_int, P, P, C.c_int, P, P, C.c_float, C.c_float, P]
        L.oracle_ccd_pair.restype = C.c_int
        L.oracle_np_pair.argtypes = [C.c_int, C.c_int, P, P, C.c_int, P, P, C.c_float, P]
        L.oracle_np_pair.restype = C.c_int
        L.oracle_contacts.argtypes = [P, P, P, C.c_int, C.c_int, P, P, P]
        L.oracle_impulses.argtypes = [P, P, P, C.c_int, C.c_int, C.c_int, P, P]
        L.oracle_mass_matrix.argtypes = [P, P, C.c_int, P]
        L.oracle_newt_sin.argtypes = [C.c_float]
        L.oracle_newt_sin.restype = C.c_float
        L.oracle_newt_cos.argtypes = [C.c_float]
        L.oracle_newt_cos.restype = C.c_float
        L.oracle_time_run.argtypes = [P, C.c_int, P, P, P, P, C.c_int, C.c_int]
        L.oracle_time_run.restype = C.c_double
        _lib = L
    return _lib


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def run(packed, model_of_world: np.ndarray, qpos: np.ndarray, qvel: np.ndarray, qfrc: Optional[np.ndarray],
        n_steps: int, precision: int = 1, layout: int = 0, want_qacc: bool = False, n_threads: int = 1,
        integrator: int = 1):
    """Step worlds on the CPU; returns (qpos, qvel[, qacc]) as float64 arrays.
    integrator 1 = semi-implicit Euler (the GPU path), 0 = RK4 (newt's default)."""
    mow = np.ascontiguousarray(model_of_world, dtype=np.int32)
    qpos = np.ascontiguousarray(qpos, dtype=np.float32)
    qvel = np.ascontiguousarray(qvel, dtype=np.float32)
    qf = None if qfrc is None else np.ascontiguousarray(qfrc, dtype=np.float32)
    qo = np.zeros(qpos.shape[0], dtype=np.float64)
    vo = np.zeros(qvel.shape[0], dtype=np.float64)
    qa = np.zeros(qvel.shape[0], dtype=np.float64) if want_qacc else None
    rc = lib().oracle_run_ex(C.cast(packed.descs, C.c_void_p), len(mow), _ptr(mow), _ptr(qpos), _ptr(qvel), _ptr(qf),
                             int(n_steps), int(precision), int(layout), _ptr(qo), _ptr(vo), _ptr(qa), int(n_threads),
                             int(integrator))
    if rc != 0:
        raise RuntimeError("oracle_run failed")
    return (qo, vo, qa) if want_qacc else (qo, vo)


def contacts(packed, index: int, qpos: np.ndarray, qvel: np.ndarray, precision: int = 1, cap: int = 4096):
    qpos = np.ascontiguousarray(qpos, dtype=np.float32)
    qvel = np.ascontiguousarray(qvel, dtype=np.float32)
    n = C.c_int(0)
    pairs = np.zeros(2 * cap, dtype=np.int32)
    data = np.zeros(7 * cap, dtype=np.float64)
    d = C.cast(C.byref(packed.descs[index]), C.c_void_p)
    lib().oracle_contacts(d, _ptr(qpos), _ptr(qvel), precision, cap, C.byref(n), _ptr(pairs), _ptr(data))
    k = min(n.value, cap)
    return pairs[: 2 * k].reshape(k, 2), data[: 7 * k].reshape(k, 7)


def impulses(packed, index: int, qpos: np.ndarray, qvel: np.ndarray, precision: int = 1, iterations: int = 0,
             cap: int = 16384):
    qpos = np.ascontiguousarray(qpos, dtype=np.float32)
    qvel = np.ascontiguousarray(qvel, dtype=np.float32)
    n = C.c_int(0)
    out = np.zeros(cap, dtype=np.float64)
    d = C.cast(C.byref(packed.descs[index]), C.c_void_p)
    lib().oracle_impulses(d, _ptr(qpos), _ptr(qvel), precision, iterations, cap, C.byref(n), _ptr(out))
    return out[: min(n.value, cap)]


def tree_impulses(packed, index: int, qpos: np.ndarray, qvel: np.ndarray, qfrc: Optional[np.ndarray] = None,
                  precision: int = 1, cap: int = 4096, integrator: int = 1):
    """Row impulses and generalised contact forces of one world's tree-contact
    solve at its state (integrator 1: the Euler form, 0: the RK4 form);
    returns (impulses, qfrc_contact)."""
    qpos = np.ascontiguousarray(qpos, dtype=np.float32)
    qvel = np.ascontiguousarray(qvel, dtype=np.float32)
    qf = None if qfrc is None else np.ascontiguousarray(qfrc, dtype=np.float32)
    n = C.c_int(0)
    out = np.zeros(cap, dtype=np.float64)
    qc = np.zeros(qvel.shape[0], dtype=np.float64)
    d = C.cast(C.byref(packed.descs[index]), C.c_void_p)
    if lib().oracle_tree_impulses_ex(d, _ptr(qpos), _ptr(qvel), _ptr(qf), precision, cap, C.byref(n), _ptr(out),
                                     _ptr(qc), int(integrator)):
        raise RuntimeError("oracle_tree_impulses failed")
    return out[: min(n.value, cap)], qc


def contact_sensors(packed, index: int, qpos: np.ndarray, qvel: np.ndarray, sens: np.ndarray, precision: int = 1):
    """newt's post-step contact sensors of one free-body world: one step from
    (qpos, qvel) (MuJoCo layout), the step's contacts re-solved at the
    post-step state; kinds 9 accelerometer (3), 10 touch (1).  Returns the
    readings and the post-step (qpos, qvel)."""
    qpos = np.ascontiguousarray(qpos, dtype=np.float32)
    qvel = np.ascontiguousarray(qvel, dtype=np.float32)
    si = np.ascontiguousarray(np.stack([sens["kind"], sens["on_link"], sens["index"]], 1), np.int32)
    sf = np.ascontiguousarray(np.concatenate([sens["local_pos"], sens["local_quat"]], 1), np.float32)
    D = int(sum(1 if k == 10 else 3 for k in sens["kind"]))
    out = np.zeros(D, dtype=np.float64)
    qo = np.zeros(qpos.size, dtype=np.float64)
    vo = np.zeros(qvel.size, dtype=np.float64)
    d = C.cast(C.byref(packed.descs[index]), C.c_void_p)
    rc = lib().oracle_contact_sensors(d, _ptr(qpos), _ptr(qvel), precision, len(sens), _ptr(si), _ptr(sf), _ptr(out),
                                      _ptr(qo), _ptr(vo))
    if rc < 0:
        raise ValueError("contact sensors take free-body worlds (and a positive definite Newton factor)")
    return out, qo, vo


def tree_contact_sensors(packed, index: int, qpos: np.ndarray, qvel: np.ndarray, sens: np.ndarray, precision: int = 1,
                         qfrc: Optional[np.ndarray] = None):
    """newt's post-step contact sensors of one tree-contact world: one step
    from (qpos, qvel) (MuJoCo layout) with the tree's applied forces `qfrc`,
    the step's tree contacts re-solved at the post-step state; kinds 9
    accelerometer on a link, 10 touch, 11 force, 12 torque (others read 0).
    Returns the readings and the post-step (qpos, qvel)."""
    qpos = np.ascontiguousarray(qpos, dtype=np.float32)
    qvel = np.ascontiguousarray(qvel, dtype=np.float32)
    qfrc = None if qfrc is None else np.ascontiguousarray(qfrc, dtype=np.float32)
    si = np.ascontiguousarray(np.stack([sens["kind"], sens["on_link"], sens["index"]], 1), np.int32)
    sf = np.ascontiguousarray(np.concatenate([sens["local_pos"], sens["local_quat"]], 1), np.float32)
    D = int(sum(1 if (k <= 1 or k in (10, 14)) else (4 if k == 3 else 3) for k in sens["kind"]))
    out = np.zeros(D, dtype=np.float64)
    qo = np.zeros(len(qpos), np.float64)
    vo = np.zeros(len(qvel), np.float64)
    d = C.cast(C.byref(packed.descs[index]), C.c_void_p)
    rc = lib().oracle_tree_contact_sensors(d, _ptr(qpos), _ptr(qvel), _ptr(qfrc), precision, len(sens), _ptr(si),
                                           _ptr(sf), _ptr(out), _ptr(qo), _ptr(vo))
    if rc != 0:
        raise RuntimeError("oracle_tree_contact_sensors failed")
    return out, qo, vo

def sensors(packed, index: int, qpos: np.ndarray, qvel: np.ndarray, sens: np.ndarray, precision: int = 1,
            qfrc: Optional[np.ndarray] = None) -> np.ndarray:
    """Post-step sensor values of one world at its state (MuJoCo layout);
    `sens` is an array with the fields kind, on_link, index, local_pos,
    local_quat (the newt_sensor_desc layout); `qfrc` the tree's applied
    generalised forces (newt layout), read by the accelerometer on a link
    and the force and torque sensors.  Kinds 13 magnetometer and 14
    rangefinder read the world's magnetic field and geoms."""
    qpos = np.ascontiguousarray(qpos, dtype=np.float32)
    qvel = np.ascontiguousarray(qvel, dtype=np.float32)
    qfrc = None if qfrc is None else np.ascontiguousarray(qfrc, dtype=np.float32)
    si = np.ascontiguousarray(np.stack([sens["kind"], sens["on_link"], sens["index"]], 1), np.int32)
    sf = np.ascontiguousarray(np.concatenate([sens["local_pos"], sens["local_quat"]], 1), np.float32)
    D = int(sum(1 if (k <= 1 or k in (10, 14)) else (4 if k == 3 else 3) for k in sens["kind"]))
    out = np.zeros(D, dtype=np.float64)
    d = C.cast(C.byref(packed.descs[index]), C.c_void_p)
    lib().oracle_sensors(d, _ptr(qpos), _ptr(qvel), _ptr(qfrc), precision, len(sens), _ptr(si), _ptr(sf), _ptr(out))
    return out


def _pose7(pose) -> np.ndarray:
    p = np.ascontiguousarray(pose, dtype=np.float32)
    assert p.shape == (7,), "pose: position xyz, quaternion x y z w"
    return p


def ccd_pair(kind_a: int, pose_a, size_a, kind_b: int, pose_b, size_b, margin: float = 0.0, precision: int = 1,
             face_eps: float = 0.0):
    """newt's GJK/EPA contact of two primitive shapes (sphere, box, capsule).
    Poses are (x, y, z, qx, qy, qz, qw).  face_eps: EPA's face-removal
    threshold (0: newt's 1e-4 of the pair extent).  Returns None (no contact)
    or a dict: path (1 distance GJK, 2 EPA, 3 EPA fallback), pos, normal (from
    B into A), pen, witness_a, witness_b."""
    out = np.zeros(15, np.float64)
    sa = np.ascontiguousarray(size_a, np.float32)
    sb = np.ascontiguousarray(size_b, np.float32)
    rc = lib().oracle_ccd_pair(int(precision), int(kind_a), _ptr(_pose7(pose_a)), _ptr(sa), int(kind_b),
                               _ptr(_pose7(pose_b)), _ptr(sb), C.c_float(margin), C.c_float(face_eps), _ptr(out))
    if rc < 0:
        raise ValueError("GJK/EPA takes spheres, boxes and capsules")
    if rc == 0:
        return None
    return {"path": int(out[1]), "pos": out[2:5].copy(), "normal": out[5:8].copy(), "pen": float(out[8]),
            "witness_a": out[9:12].copy(), "witness_b": out[12:15].copy()}


def np_pair(kind_a: int, pose_a, size_a, kind_b: int, pose_b, size_b, margin: float = 0.0,
            precision: int = 1) -> np.ndarray:
    """The step's closed-form narrowphase for one routed pair (A, B): an
    (n, 7) array of point, normal (from B into A), penetration."""
    out = np.zeros(28, np.float64)
    sa = np.ascontiguousarray(size_a, np.float32)
    sb = np.ascontiguousarray(size_b, np.float32)
    n = lib().oracle_np_pair(int(precision), int(kind_a), _ptr(_pose7(pose_a)), _ptr(sa), int(kind_b),
                             _ptr(_pose7(pose_b)), _ptr(sb), C.c_float(margin), _ptr(out))
    if n < 0:
        raise ValueError("no narrowphase route for this (A, B) order")
    return out[: 7 * n].reshape(n, 7)


def mass_matrix(packed, index: int, q_native: np.ndarray, nv: int, precision: int = 1) -> np.ndarray:
    q = np.ascontiguousarray(q_native, dtype=np.float32)
    out = np.zeros(nv * nv, dtype=np.float64)
    d = C.cast(C.byref(packed.descs[index]), C.c_void_p)
    lib().oracle_mass_matrix(d, _ptr(q), precision, _ptr(out))
    return out.reshape(nv, nv)


def energy(packed, model_of_world, qpos, qvel) -> np.ndarray:
    mow = np.ascontiguousarray(model_of_world, dtype=np.int32)
    qpos = np.ascontiguousarray(qpos, dtype=np.float32)
    qvel = np.ascontiguousarray(qvel, dtype=np.float32)
    out = np.zeros(len(mow), np.float64)
    L = lib()
    L.oracle_energy.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.oracle_energy(C.cast(packed.descs, C.c_void_p), len(mow), _ptr(mow), _ptr(qpos), _ptr(qvel), _ptr(out))
    return out


def time_run(packed, model_of_world, qpos, qvel, qfrc, n_steps: int, n_threads: int) -> float:
    mow = np.ascontiguousarray(model_of_world, dtype=np.int32)
    qpos = np.ascontiguousarray(qpos, dtype=np.float32)
    qvel = np.ascontiguousarray(qvel, dtype=np.float32)
    qf = None if qfrc is None else np.ascontiguousarray(qfrc, dtype=np.float32)
    return lib().oracle_time_run(C.cast(packed.descs, C.c_void_p), len(mow), _ptr(mow), _ptr(qpos), _ptr(qvel),
                                 _ptr(qf), int(n_steps), int(n_threads))
