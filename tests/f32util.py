"""f32 helpers that reproduce newt's scalar arithmetic for building test scenes."""
import numpy as np

import oracle_py

f32 = np.float32


def normalize(v):
    v = [f32(x) for x in v]
    l = np.sqrt(f32(f32(v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]))
    if l == 0:
        return [f32(0), f32(0), f32(0)]
    return [x / l for x in v]


def quat_from_axis_angle(axis, angle):
    """Quat::from_axis_angle (newt/src/math.rs:574-580), x y z w in f32."""
    a = normalize(axis)
    half = f32(angle) * f32(0.5)
    L = oracle_py.lib()
    s = f32(L.oracle_newt_sin(float(half)))
    c = f32(L.oracle_newt_cos(float(half)))
    return [a[0] * s, a[1] * s, a[2] * s, c]
