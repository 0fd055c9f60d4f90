"""Python host binding of the newt GPU C ABI (include/newt_gpu.h).

This is a thin ctypes layer: every call goes straight to ``libnewt_gpu.so``.
There is no CPU fallback; constructing an :class:`Engine` without the built
library or without a CUDA device raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

from . import model as M

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnewt_gpu.so")

OK = 0
ERRORS = {1: "NEWT_E_INVALID", 2: "NEWT_E_UNSUPPORTED_PAIR", 3: "NEWT_E_NOT_PD", 4: "NEWT_E_OVERFLOW",
          5: "NEWT_E_TIMEOUT", 6: "NEWT_E_CUDA", 7: "NEWT_E_NOMEM", 8: "NEWT_E_NOT_FINITE"}
STEP_PLAIN, STEP_BATCHED = 0, 1
WS_NONFINITE, WS_NOT_PD, WS_CONTACT_OVERFLOW, WS_ITER_CAP, WS_FP64_FALLBACK = 0x1, 0x2, 0x4, 0x8, 0x10

EXPORTED = [
    "newt_gpu_create", "newt_gpu_destroy", "newt_gpu_last_error", "newt_gpu_upload_models", "newt_gpu_model_dims",
    "newt_gpu_alloc_worlds", "newt_gpu_free_worlds", "newt_gpu_set_state", "newt_gpu_get_state",
    "newt_gpu_set_qfrc", "newt_gpu_step", "newt_gpu_sync", "newt_gpu_world_status", "newt_gpu_get_qacc",
    "newt_gpu_get_contacts", "newt_gpu_get_impulses", "newt_gpu_event_record", "newt_gpu_event_elapsed_ms",
    "newt_gpu_flush_l2", "newt_gpu_launch_count", "newt_gpu_step_static", "newt_gpu_pile_profile",
    "newt_gpu_tc_profile", "newt_gpu_serve", "newt_gpu_memory", "newt_gpu_autotune",
    "newt_gpu_set_ctrl_stream", "newt_gpu_apply_ctrl", "newt_gpu_read_sensors", "newt_gpu_pile_fused_profile",
    "newt_gpu_set_launch_choice", "newt_gpu_convex_contacts", "newt_gpu_hold_worlds",
]
# newt_sensor_desc (include/newt_gpu.h)
SENSOR_DTYPE = np.dtype([("kind", np.int32), ("on_link", np.int32), ("index", np.int32),
                         ("local_pos", np.float32, 3), ("local_quat", np.float32, 4)])
SENSOR_JOINTPOS, SENSOR_JOINTVEL, SENSOR_FRAMEPOS, SENSOR_FRAMEQUAT, SENSOR_GYRO = 0, 1, 2, 3, 4
SENSOR_VELOCIMETER, SENSOR_FRAMELINVEL, SENSOR_FRAMEANGVEL, SENSOR_SUBTREECOM = 5, 6, 7, 8
SENSOR_ACCELEROMETER, SENSOR_TOUCH, SENSOR_FORCE, SENSOR_TORQUE = 9, 10, 11, 12
SENSOR_MAGNETOMETER, SENSOR_RANGEFINDER = 13, 14
SENSOR_DIM = {SENSOR_JOINTPOS: 1, SENSOR_JOINTVEL: 1, SENSOR_FRAMEQUAT: 4, SENSOR_TOUCH: 1, SENSOR_RANGEFINDER: 1}


def sensors(*specs) -> np.ndarray:
    """Sensor descriptors from (kind, on_link, index[, local_pos[, local_quat xyzw]]) tuples."""
    out = np.zeros(len(specs), SENSOR_DTYPE)
    for i, sp in enumerate(specs):
        out[i]["kind"], out[i]["on_link"], out[i]["index"] = sp[0], sp[1], sp[2]
        out[i]["local_pos"] = sp[3] if len(sp) > 3 else (0.0, 0.0, 0.0)
        out[i]["local_quat"] = sp[4] if len(sp) > 4 else (0.0, 0.0, 0.0, 1.0)
    return out
# newt_convex_query / newt_convex_result (include/newt_gpu.h)
CONVEX_QUERY_DTYPE = np.dtype([("shape_a", np.int32), ("shape_b", np.int32), ("pose_a", np.float32, 7),
                               ("size_a", np.float32, 3), ("pose_b", np.float32, 7), ("size_b", np.float32, 3),
                               ("margin", np.float32)])
CONVEX_RESULT_DTYPE = np.dtype([("hit", np.int32), ("path", np.int32), ("pos", np.float32, 3),
                                ("normal", np.float32, 3), ("penetration", np.float32),
                                ("witness_a", np.float32, 3), ("witness_b", np.float32, 3)])
TC_KERNELS = ["tree_aba_kernel", "tc_k_solve", "tree_integrate_kernel"]
PILE_KERNELS = ["pile_k_collide", "pile_k_pgs_small<1>", "pile_k_pgs_small<2>", "pile_k_pgs_small<4>",
                "pile_k_pgs_quad[3]", "pile_k_pgs_quad[4]", "pile_k_pgs_quad[5]", "pile_k_pgs_levels[6]",
                "pile_k_integrate"]
PILE_ISLAND_CLASSES = 7


class NewtError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Opts(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_worlds", C.c_int32), ("hbm_budget_bytes", C.c_uint64),
                ("max_contacts", C.c_int32)]


class ServeRequest(C.Structure):
    _fields_ = [("model_id", C.c_int32), ("horizon", C.c_int32), ("arrival_s", C.c_double),
                ("qpos", C.c_void_p), ("qvel", C.c_void_p), ("ctrl", C.c_void_p),
                ("qpos_out", C.c_void_p), ("qvel_out", C.c_void_p), ("admit_s", C.c_double), ("done_s", C.c_double)]


class ServeOpts(C.Structure):
    _fields_ = [("max_active", C.c_int32), ("real_time", C.c_int32), ("step_mode", C.c_int32),
                ("steps_per_tick", C.c_int32)]


# newt_serve_request as a numpy record (same layout), so request tables are
# built without a Python loop
SERVE_DTYPE = np.dtype([("model_id", "<i4"), ("horizon", "<i4"), ("arrival_s", "<f8"), ("qpos", "<u8"),
                        ("qvel", "<u8"), ("ctrl", "<u8"), ("qpos_out", "<u8"), ("qvel_out", "<u8"),
                        ("admit_s", "<f8"), ("done_s", "<f8")], align=True)


class ServeStats(C.Structure):
    _fields_ = [("completed", C.c_int32), ("peak_active", C.c_int32), ("ticks", C.c_int64), ("wall_s", C.c_double),
                ("env_steps", C.c_double), ("mean_active", C.c_double), ("p50_ms", C.c_double),
                ("p99_ms", C.c_double), ("max_ms", C.c_double), ("mean_ms", C.c_double), ("admit_s", C.c_double),
                ("ctrl_s", C.c_double), ("step_s", C.c_double), ("complete_s", C.c_double)]


_lib = None


def load_library(path: str = LIB_PATH):
    """Load the shared library (never builds; call ``tooling_gb300.build.build()``)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: run tooling_gb300.build.build() first (no CPU fallback)")
    L = C.CDLL(path)
    P, I32 = C.c_void_p, C.c_int32
    sig = {
        "newt_gpu_create": ([P, P], C.c_int),
        "newt_gpu_destroy": ([P], C.c_int),
        "newt_gpu_last_error": ([P], C.c_char_p),
        "newt_gpu_upload_models": ([P, P, I32, P], C.c_int),
        "newt_gpu_model_dims": ([P, I32, P, P], C.c_int),
        "newt_gpu_alloc_worlds": ([P, P, I32, P], C.c_int),
        "newt_gpu_free_worlds": ([P, P, I32], C.c_int),
        "newt_gpu_set_state": ([P, P, I32, P, P], C.c_int),
        "newt_gpu_get_state": ([P, P, I32, P, P], C.c_int),
        "newt_gpu_set_qfrc": ([P, P, I32, P], C.c_int),
        "newt_gpu_step": ([P, I32, I32], C.c_int),
        "newt_gpu_sync": ([P, I32], C.c_int),
        "newt_gpu_world_status": ([P, P, I32, P, I32], C.c_int),
        "newt_gpu_get_qacc": ([P, P, I32, P], C.c_int),
        "newt_gpu_get_contacts": ([P, I32, I32, P, P, P], C.c_int),
        "newt_gpu_get_impulses": ([P, I32, I32, P, P], C.c_int),
        "newt_gpu_event_record": ([P, I32], C.c_int),
        "newt_gpu_event_elapsed_ms": ([P, P], C.c_int),
        "newt_gpu_flush_l2": ([P], C.c_int),
        "newt_gpu_launch_count": ([P], C.c_int64),
        "newt_gpu_step_static": ([P, I32], C.c_int),
        "newt_gpu_pile_profile": ([P, I32, P, P, P], C.c_int),
        "newt_gpu_tc_profile": ([P, P], C.c_int),
        "newt_gpu_serve": ([P, P, I32, P, P], C.c_int),
        "newt_gpu_memory": ([P, P, P], C.c_int),
        "newt_gpu_autotune": ([P, I32, I32, P], C.c_int),
        "newt_gpu_set_ctrl_stream": ([P, P, I32, P, P], C.c_int),
        "newt_gpu_apply_ctrl": ([P], C.c_int),
        "newt_gpu_pile_fused_profile": ([P, P, P], C.c_int),
        "newt_gpu_set_launch_choice": ([P, P], C.c_int),
        "newt_gpu_hold_worlds": ([P, P, I32], C.c_int),
        "newt_gpu_convex_contacts": ([P, P, I32, C.c_float, P], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Engine:
    """One context = one CUDA stream on one device (not thread-safe)."""

    def __init__(self, device: int = 0, max_worlds: int = 0, hbm_budget_bytes: int = 0, max_contacts: int = 0):
        self.L = load_library()
        self.ctx = C.c_void_p()
        o = Opts(device, max_worlds, hbm_budget_bytes, max_contacts)
        rc = self.L.newt_gpu_create(C.byref(o), C.byref(self.ctx))
        if rc != OK:
            raise NewtError(rc, "newt_gpu_create failed (is a CUDA device visible?)")
        self._dims = {}

    def _ck(self, rc: int):
        if rc != OK:
            raise NewtError(rc, self.L.newt_gpu_last_error(self.ctx).decode())

    def close(self):
        if self.ctx:
            self.L.newt_gpu_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- models / worlds ----------------------------------------------------
    def upload(self, packed: "M.PackedModels") -> np.ndarray:
        ids = np.zeros(len(packed), np.int32)
        self._ck(self.L.newt_gpu_upload_models(self.ctx, C.cast(packed.descs, C.c_void_p), len(packed), _p(ids)))
        return ids

    def dims(self, model_id: int):
        if model_id not in self._dims:
            nq, nv = C.c_int32(), C.c_int32()
            self._ck(self.L.newt_gpu_model_dims(self.ctx, int(model_id), C.byref(nq), C.byref(nv)))
            self._dims[model_id] = (nq.value, nv.value)
        return self._dims[model_id]

    def alloc(self, model_ids: Sequence[int]) -> np.ndarray:
        ids = np.ascontiguousarray(model_ids, np.int32)
        slots = np.zeros(len(ids), np.int32)
        self._ck(self.L.newt_gpu_alloc_worlds(self.ctx, _p(ids), len(ids), _p(slots)))
        return slots

    def free(self, slots: Sequence[int]):
        s = np.ascontiguousarray(slots, np.int32)
        self._ck(self.L.newt_gpu_free_worlds(self.ctx, _p(s), len(s)))

    def hold(self, slots: Sequence[int]):
        """Stop stepping these worlds from the next step call on (queued on
        the device, no wait); they keep their state until freed."""
        s = np.ascontiguousarray(slots, np.int32)
        self._ck(self.L.newt_gpu_hold_worlds(self.ctx, _p(s), len(s)))

    # -- state --------------------------------------------------------------
    def set_state(self, slots, qpos: np.ndarray, qvel: np.ndarray):
        s = np.ascontiguousarray(slots, np.int32)
        qp = np.ascontiguousarray(qpos, np.float32)
        qv = np.ascontiguousarray(qvel, np.float32)
        self._ck(self.L.newt_gpu_set_state(self.ctx, _p(s), len(s), _p(qp), _p(qv)))

    def get_state(self, slots, nq_total: int, nv_total: int, out=None):
        """MuJoCo-layout state of the worlds, into new arrays or into `out`
        (a pair of contiguous float32 arrays; page-locked ones are filled by
        DMA directly)."""
        s = np.ascontiguousarray(slots, np.int32)
        if out is None:
            qp = np.zeros(nq_total, np.float32)
            qv = np.zeros(nv_total, np.float32)
        else:
            qp, qv = out
            if not (qp.dtype == np.float32 and qv.dtype == np.float32 and qp.flags.c_contiguous
                    and qv.flags.c_contiguous and qp.size >= nq_total and qv.size >= nv_total):
                raise ValueError("out must be two contiguous float32 arrays large enough for the state")
        self._ck(self.L.newt_gpu_get_state(self.ctx, _p(s), len(s), _p(qp), _p(qv)))
        return qp, qv

    def set_qfrc(self, slots, qfrc: np.ndarray):
        s = np.ascontiguousarray(slots, np.int32)
        q = np.ascontiguousarray(qfrc, np.float32)
        self._ck(self.L.newt_gpu_set_qfrc(self.ctx, _p(s), len(s), _p(q)))

    def set_ctrl_stream(self, slots, ctrl: np.ndarray, horizons):
        """Upload each world's horizon x nv control sequence (concatenated in
        slot order) to the device; apply_ctrl writes the next row into qfrc."""
        s = np.ascontiguousarray(slots, np.int32)
        h = np.ascontiguousarray(horizons, np.int32)
        c = np.ascontiguousarray(ctrl, np.float32)
        self._ck(self.L.newt_gpu_set_ctrl_stream(self.ctx, _p(s), len(s), _p(c), _p(h)))

    def apply_ctrl(self):
        self._ck(self.L.newt_gpu_apply_ctrl(self.ctx))

    def get_qacc(self, slots, nv_total: int) -> np.ndarray:
        s = np.ascontiguousarray(slots, np.int32)
        out = np.zeros(nv_total, np.float32)
        self._ck(self.L.newt_gpu_get_qacc(self.ctx, _p(s), len(s), _p(out)))
        return out

    def read_sensors(self, slots, sens: np.ndarray) -> np.ndarray:
        """Evaluate `sens` (a SENSOR_DTYPE array) on each world at its current
        state, on the device; returns (len(slots), total sensor dim)."""
        s = np.ascontiguousarray(slots, np.int32)
        sens = np.ascontiguousarray(sens, SENSOR_DTYPE)
        D = sum(SENSOR_DIM.get(int(k), 3) for k in sens["kind"])
        out = np.zeros((len(s), D), np.float32)
        self._ck(self.L.newt_gpu_read_sensors(self.ctx, _p(s), len(s), _p(sens), len(sens), _p(out)))
        return out

    # -- stepping -------------------------------------------------------------
    def step(self, n_steps: int = 1, mode: int = STEP_BATCHED):
        self._ck(self.L.newt_gpu_step(self.ctx, int(n_steps), int(mode)))

    def step_static(self, n_steps: int = 1):
        """Plain step whose solver scratch is a fixed device array (no allocation)."""
        self._ck(self.L.newt_gpu_step_static(self.ctx, int(n_steps)))

    def sync(self, timeout_ms: int = 600000):
        self._ck(self.L.newt_gpu_sync(self.ctx, int(timeout_ms)))

    def status(self, slots, clear: bool = False) -> np.ndarray:
        s = np.ascontiguousarray(slots, np.int32)
        out = np.zeros(len(s), np.uint32)
        self._ck(self.L.newt_gpu_world_status(self.ctx, _p(s), len(s), _p(out), int(clear)))
        return out

    # -- served rollouts -------------------------------------------------------
    def serve(self, model_ids, horizons, arrivals_s, qpos: np.ndarray, qvel: np.ndarray,
              ctrl: Optional[np.ndarray] = None, ctrl_off=None, max_active: int = 0,
              real_time: bool = True, mode: int = STEP_BATCHED, steps_per_tick: int = 1):
        """Serve rollout requests through the native loop (newt_gpu_serve).

        qpos / qvel: the requests' initial states concatenated in request
        order (MuJoCo layout).  ctrl: one flat float32 array; request i reads
        horizon_i x nv_i values from element ctrl_off[i] (-1: no controls).
        steps_per_tick: env-steps queued per tick (worlds that finish inside
        a tick are held at their last env-step).  Returns (final qpos, final
        qvel) concatenated like the inputs, a stats dict, and the admission
        and completion times (s)."""
        n = len(model_ids)
        ids = np.ascontiguousarray(model_ids, np.int32)
        hz = np.ascontiguousarray(horizons, np.int32)
        dims = np.array([self.dims(int(m)) for m in ids], np.int64).reshape(n, 2)
        qoff = np.concatenate([[0], np.cumsum(dims[:, 0])])
        voff = np.concatenate([[0], np.cumsum(dims[:, 1])])
        qp = np.ascontiguousarray(qpos, np.float32)
        qv = np.ascontiguousarray(qvel, np.float32)
        if qp.size != qoff[-1] or qv.size != voff[-1]:
            raise ValueError("qpos/qvel sizes do not match the requests' models")
        oq, ov = np.zeros(qoff[-1], np.float32), np.zeros(voff[-1], np.float32)
        r = np.zeros(n, SERVE_DTYPE)
        r["model_id"], r["horizon"], r["arrival_s"] = ids, hz, np.asarray(arrivals_s, np.float64)
        r["qpos"] = qp.ctypes.data + 4 * qoff[:-1]
        r["qvel"] = qv.ctypes.data + 4 * voff[:-1]
        r["qpos_out"] = oq.ctypes.data + 4 * qoff[:-1]
        r["qvel_out"] = ov.ctypes.data + 4 * voff[:-1]
        if ctrl is not None:
            c = np.ascontiguousarray(ctrl, np.float32)
            co = np.asarray(ctrl_off, np.int64)
            need = co + hz.astype(np.int64) * dims[:, 1]
            if np.any((co >= 0) & (need > c.size)):
                raise ValueError("a control window runs past the end of ctrl")
            r["ctrl"] = np.where(co >= 0, c.ctypes.data + 4 * np.maximum(co, 0), 0).astype(np.uint64)
        opts = ServeOpts(int(max_active), int(bool(real_time)), int(mode), int(steps_per_tick))
        st = ServeStats()
        self._ck(self.L.newt_gpu_serve(self.ctx, r.ctypes.data, n, C.byref(opts), C.byref(st)))
        stats = {k: getattr(st, k) for k, _ in ServeStats._fields_}
        return oq, ov, stats, r["admit_s"].copy(), r["done_s"].copy()

    def convex_contacts(self, queries: np.ndarray, face_eps: float = 0.0) -> np.ndarray:
        """GJK/EPA contacts of sphere/box/capsule pairs on the device
        (`queries`: CONVEX_QUERY_DTYPE records); CONVEX_RESULT_DTYPE records."""
        q = np.ascontiguousarray(queries, CONVEX_QUERY_DTYPE)
        out = np.zeros(len(q), CONVEX_RESULT_DTYPE)
        self._ck(self.L.newt_gpu_convex_contacts(self.ctx, _p(q), len(q), C.c_float(face_eps), _p(out)))
        return out

    # -- diagnostics ----------------------------------------------------------
    def contacts(self, slot: int, cap: int = 1024):
        n = C.c_int32()
        pairs = np.zeros(2 * cap, np.int32)
        data = np.zeros(7 * cap, np.float32)
        self._ck(self.L.newt_gpu_get_contacts(self.ctx, int(slot), cap, C.byref(n), _p(pairs), _p(data)))
        k = min(n.value, cap)
        return pairs[: 2 * k].reshape(k, 2), data[: 7 * k].reshape(k, 7)

    def impulses(self, slot: int, cap: int = 4096) -> np.ndarray:
        n = C.c_int32()
        out = np.zeros(cap, np.float32)
        self._ck(self.L.newt_gpu_get_impulses(self.ctx, int(slot), cap, C.byref(n), _p(out)))
        return out[: min(n.value, cap)]

    # -- timing ---------------------------------------------------------------
    def event(self, which: int):
        self._ck(self.L.newt_gpu_event_record(self.ctx, int(which)))

    def elapsed_ms(self) -> float:
        ms = C.c_float()
        self._ck(self.L.newt_gpu_event_elapsed_ms(self.ctx, C.byref(ms)))
        return ms.value

    def flush_l2(self):
        self._ck(self.L.newt_gpu_flush_l2(self.ctx))

    def autotune(self, n_steps: int = 25, horizon: int = 0) -> dict:
        """Pick the batched step's launch choices by timing them on the live
        worlds, `n_steps` env-steps per trial, averaged over the next
        `horizon` env-steps (0: 8 x n_steps); the worlds' state is left
        unchanged."""
        c = np.zeros(5, np.int32)
        self._ck(self.L.newt_gpu_autotune(self.ctx, int(n_steps), int(horizon), _p(c)))
        return {"pile_persistent": bool(c[3]), "persistent_shape": int(c[4]), "pile_branches": int(c[0]),
                "tree_grid_pct": int(c[1]), "best_ms": c[2] / 1000.0}

    def set_launch_choice(self, persistent: bool = True, persistent_shape: int = 10, pile_branches: int = 0,
                          tree_grid_pct: int = 100):
        """Pin the batched step's launch choices (what autotune() would pick):
        piles in the world-persistent launch of shape `persistent_shape`, or
        in the island-class pipeline with `pile_branches` world-range
        branches (0: by world count)."""
        c = np.array([pile_branches, tree_grid_pct, 0, int(bool(persistent)), persistent_shape], np.int32)
        self._ck(self.L.newt_gpu_set_launch_choice(self.ctx, _p(c)))

    def memory(self):
        """(device bytes held by the world groups, admission budget)."""
        u, b = C.c_uint64(), C.c_uint64()
        self._ck(self.L.newt_gpu_memory(self.ctx, C.byref(u), C.byref(b)))
        return u.value, b.value

    def launch_count(self) -> int:
        return int(self.L.newt_gpu_launch_count(self.ctx))

    def tc_profile(self) -> dict:
        """Per-kernel ms of the last step call's tree-contact env-steps
        (timing is switched on with pile_profile(1))."""
        ms = np.zeros(len(TC_KERNELS), np.float32)
        self._ck(self.L.newt_gpu_tc_profile(self.ctx, _p(ms)))
        return dict(zip(TC_KERNELS, ms.tolist()))

    def fused_profile(self):
        """(device ms of the last batched call's world-persistent pile launch,
        or 0 when it was not timed; {contacts, rounds, levels, worlds} summed
        over that launch's worlds and env-steps)."""
        ms = C.c_float()
        w = np.zeros(4, np.uint64)
        self._ck(self.L.newt_gpu_pile_fused_profile(self.ctx, C.byref(ms), _p(w)))
        return ms.value, {"contacts": int(w[0]), "rounds": int(w[1]), "levels": int(w[2]), "worlds": int(w[3])}

    def pile_profile(self, enable: int = -1):
        """(per-kernel ms summed over the last step call's launches, {islands,
        contacts, bodies per island class of its last env-step, launches per
        kernel}); enable 1/0 switches kernel timing for later batched steps,
        -1 leaves it."""
        ms = np.zeros(len(PILE_KERNELS), np.float32)
        work = np.zeros(3 * PILE_ISLAND_CLASSES, np.int32)
        n = C.c_int32()
        self._ck(self.L.newt_gpu_pile_profile(self.ctx, int(enable), _p(ms), _p(work), C.byref(n)))
        w = work.reshape(3, PILE_ISLAND_CLASSES)
        return dict(zip(PILE_KERNELS, ms.tolist())), {"islands": w[0], "contacts": w[1], "bodies": w[2],
                                                      "launches": n.value}
