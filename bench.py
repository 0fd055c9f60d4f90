"""Benchmark: batched GPU stepping of newt worlds on GB300.

Workload (the metric's headline configuration): 8192 independent worlds, each
16 free bodies (50% spheres, 50% boxes, density 1000) above a plane, pyramidal
friction, PGS 50 iterations, dt = 2e-3 -- seeded synthetic worlds.

A bench step advances every world by `--substeps` env-steps with one call of
the C ABI's batched step (one CUDA-graph replay of one world-persistent
launch: a warp per world runs collide, PGS and integration for every
env-step of the call, worlds pulled from a queue).  The same line carries the
plain form (one launch per stage per env-step) on the same worlds and horizon,
the one-step error against the FP64 oracle on a sample of the timed region's
start state, and two compact runs of the other metric configurations: the
uneven batch (batched vs plain, finite worlds counted apart) and a served
Poisson stream (p50/p99 latency).
Other workloads: --workload quadruped (16384 quadrupeds, Newton), uneven
(32768 chains and piles of 2..64 bodies, batched vs plain), serve (Poisson
request streams through the served-rollout loop).  Timing:
  value : device time with CUDA events on the engine's stream, L2 flushed
          between timed steps, state resident in HBM;
  e2e   : wall time of set_state (host->device) + step + get_state
          (device->host) through the C ABI with host buffers, every step.
The reference arm (`--impl reference`) times newt's algorithm on the host
cores: the C++ restatement of newt's f32 step (newt itself is Rust and no
Rust toolchain exists on these machines).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
# FP32 pipe peak of a GB300 derived from its datasheet figures: 152 SMs x 128
# FP32 lanes x 2 FLOP per fused multiply-add x 2.07 GHz maximum SM clock
FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12
# newt's PGS work per active contact and sweep (5 row updates x ~235 FLOP,
# newt/src/solver.rs:1448-1518 with the residuals of :1980 and the impulse
# application of :2022)
PGS_FLOP_PER_CONTACT_SWEEP = 5 * 235
# DRAM bytes (read + write) per world and env-step of pile_k_fused, from the
# ncu capture summarised in profiles/pile_k_fused_2048worlds_settled_full.md
# (2048 settled worlds, one launch of 25 env-steps: 28.8 MB read + 272.5 MB
# written), scaled by worlds x env-steps
FUSED_DRAM_BYTES_PER_WORLD_STEP = (28.797696e6 + 272.532224e6) / (2048 * 25)


def pinned_like(a):
    """A page-locked host copy of float32 array `a` (torch's pinned allocator),
    or a plain copy where torch cannot pin."""
    try:
        import torch
        t = torch.empty(a.size, dtype=torch.float32, pin_memory=True)
        out = t.numpy()
        out[:] = a
        pinned_like.keep.append(t)  # the numpy view does not own the buffer
        return out
    except Exception:
        return np.array(a, dtype=np.float32, copy=True)


pinned_like.keep = []


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--substeps", type=int, default=25)
    ap.add_argument("--worlds", type=int, default=8192)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-plain", action="store_true", help="skip timing the plain (per-stage launch) form")
    ap.add_argument("--no-extras", action="store_true",
                    help="headline only: skip the FP64 error sample and the uneven / served sub-runs")
    ap.add_argument("--rates", default="1000,5000,10000,20000,50000",
                    help="serve workload: Poisson request rates (req/s), one timed run each")
    ap.add_argument("--duration", type=float, default=1.5, help="serve workload: seconds of arrivals per rate")
    ap.add_argument("--steps-per-tick", type=int, default=8,
                    help="served rollouts: env-steps queued per serving tick (worlds held where their horizon ends)")
    ap.add_argument("--workload", default="pile", choices=["pile", "quadruped", "uneven", "serve"],
                    help="pile: 16 free bodies on a plane (default); quadruped: Newton tree contact; "
                         "uneven: chains and piles of 2..64 bodies, batched vs plain")
    return ap.parse_args()


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return rank, ws, local, dist
    return rank, ws, local, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def peaks():
    try:
        with open(PEAKS_PATH) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix="newt_clocks_", suffix=".csv")
        os.close(fd)

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            lines = f.readlines()
        os.unlink(self.path)
        for line in lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1])); smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


ROW_WORDS = 117  # solver words per active contact: 4 facet rows x (J, M^-1 J^T) x 2 sides + 21 constants


def pile_kernel_bytes(kernel: str, n_worlds: int, nb: int, work: dict) -> float:
    """Algorithmic HBM bytes of one launch (one env-step) of a pile kernel:
    what the kernel must read and write at least once, from the per-class
    work of the step (islands, contacts, bodies per island class).
      collide: each world record read (per body: position, velocity, angular
        velocity, size, geom offset 3 each; orientation, geom orientation 4
        each; inverse and body inertia 6 each; mass, shape; per geom friction,
        margin, filter; plane 7, soft parameters 7, dt and gravity 4) and the
        solver rows of every active contact written;
      class-c solver: the rows of its contacts read, 4 impulses per contact
        and 6 velocity deltas per body written;
      integrate: 13 state words read and written and 6 deltas read per body."""
    contacts, bodies = work["contacts"], work["bodies"]
    if kernel == "pile_k_collide":
        rec = nb * 37 + 7 + 3 * (nb + 1) + 7 + 4
        return 4.0 * (n_worlds * rec + int(contacts.sum()) * (ROW_WORDS + 1))
    if kernel == "pile_k_integrate":
        return 4.0 * n_worlds * nb * (13 + 6 + 13)
    from tooling_gb300.api import PILE_KERNELS
    c = PILE_KERNELS.index(kernel) - 1
    return 4.0 * (int(contacts[c]) * (ROW_WORDS + 4) + int(bodies[c]) * 6)


def fused_kernel_bytes(n_worlds: int, nb: int, contacts_last_step: float) -> float:
    """Algorithmic HBM bytes of one pile_k_fused launch: every world record
    read once (per body: position, velocity, angular velocity, size, geom
    offset 3 each; orientation, geom orientation 4 each; inverse and body
    inertia 6 each; mass, shape; per geom friction, margin, filter; plane 7,
    soft parameters 7, dt and gravity 4), the 13 state words per body written
    once, and the last env-step's contacts (pair 2, point, normal, depth 7,
    impulses 4) written once.  The per-env-step solver records live in the
    world's scratch and are not algorithmic traffic."""
    rec = nb * 37 + 7 + 3 * (nb + 1) + 7 + 4
    return 4.0 * (n_worlds * (rec + 13 * nb) + contacts_last_step * 13)


def fp64_one_step_error(eng, batch, slots, start_qpos, start_qvel, n_sample=64):
    """One env-step from the timed region's start state: the GPU's velocity
    change against the FP64 oracle's on a spread sample of worlds, as the
    relative error of the generalised acceleration (qacc = dv / dt) per world,
    max-norm over the world's DoF."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py
    from tooling_gb300 import STEP_BATCHED
    W = len(batch)
    idx = np.unique(np.linspace(0, W - 1, min(n_sample, W)).astype(np.int64))
    eng.set_state(slots, start_qpos, start_qvel)
    eng.step(1, STEP_BATCHED)
    q1, v1 = eng.get_state(slots, int(batch.nq.sum()), int(batch.nv.sum()))
    qp = np.concatenate([start_qpos[batch.q_off[w]:batch.q_off[w] + batch.nq[w]] for w in idx])
    qv = np.concatenate([start_qvel[batch.v_off[w]:batch.v_off[w] + batch.nv[w]] for w in idx])
    rq, rv = oracle_py.run(batch, idx, qp, qv, None, 1, precision=1, n_threads=os.cpu_count() or 1)
    rel, dq = [], []
    vo = 0
    qo = 0
    for w in idx:
        nv, nq = int(batch.nv[w]), int(batch.nq[w])
        v0 = start_qvel[batch.v_off[w]:batch.v_off[w] + nv].astype(np.float64)
        dg = v1[batch.v_off[w]:batch.v_off[w] + nv] - v0
        dr = rv[vo:vo + nv] - v0
        rel.append(float(np.abs(dg - dr).max() / max(np.abs(dr).max(), 1e-30)))
        dq.append(float(np.abs(q1[batch.q_off[w]:batch.q_off[w] + nq] - rq[qo:qo + nq]).max()))
        vo += nv
        qo += nq
    rel = np.array(rel)
    return {"worlds": int(len(idx)), "qacc_rel_max": float(rel.max()), "qacc_rel_median": float(np.median(rel)),
            "worlds_within_1e-4": int((rel <= 1e-4).sum()), "qpos_abs_max": float(max(dq)),
            "what": "one env-step from the timed region's start state; qacc = dv/dt per world, max-norm relative "
                    "error against the FP64 oracle (oracle/, newt's step in double)"}


def run_gpu(args, rank, ws, local, dist):
    from tooling_gb300 import build as B
    B.build()
    from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN, scenes
    W = args.worlds
    batch = scenes.pile_batch(n_worlds=W, first_world=rank * W)
    eng = Engine(device=local)
    ids = eng.upload(batch)
    slots = eng.alloc(ids)
    eng.set_state(slots, batch.qpos, batch.qvel)
    S = args.substeps
    nq_t, nv_t = int(batch.nq.sum()), int(batch.nv.sum())
    # the persistent launch's timing events ride in the captured graph
    eng.pile_profile(1)
    # warm-up (also captures the CUDA graph), then the launch-choice autotuner
    # (it leaves the worlds' state as it found it)
    for _ in range(max(3, args.warmup)):
        eng.step(S, STEP_BATCHED)
    tuned = eng.autotune(S, horizon=S * args.steps)
    eng.sync()
    start_qpos, start_qvel = eng.get_state(slots, nq_t, nv_t)
    launches0 = eng.launch_count()
    clocks = Clocks(local)
    clocks.start()
    per_step, fused_ms, kernel_ms = [], 0.0, {}
    fwork = {"contacts": 0, "rounds": 0, "levels": 0, "worlds": 0}
    n_launch = 0
    barrier(dist)
    eng.sync()
    for _ in range(args.steps):
        eng.flush_l2()
        eng.event(0)
        eng.step(S, STEP_BATCHED)
        eng.event(1)
        per_step.append(eng.elapsed_ms())
        ms, fw = eng.fused_profile()
        fused_ms += ms
        for k in fwork:
            fwork[k] += fw[k]
        kms, work = eng.pile_profile()
        n_launch += work["launches"]
        for k, v in kms.items():
            kernel_ms[k] = kernel_ms.get(k, 0.0) + v
    eng.sync()
    barrier(dist)
    clk = clocks.stop()
    launches = eng.launch_count() - launches0
    total_ms = max_over_ranks(dist, float(sum(per_step)))
    env_steps = W * S * args.steps * ws
    value = env_steps / (total_ms / 1e3)
    st = eng.status(slots)
    # e2e: host buffers in, host buffers out, every step (page-locked host
    # buffers: the state moves by DMA, converted on the device)
    qp = pinned_like(start_qpos)
    qv = pinned_like(start_qvel)
    h2d = (qp.nbytes + qv.nbytes)
    d2h = h2d
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.set_state(slots, qp, qv)
        eng.step(S, STEP_BATCHED)
        eng.get_state(slots, nq_t, nv_t, out=(qp, qv))
    eng.sync()
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
    e2e = env_steps / e2e_s
    plain = None
    if not args.no_plain:
        # the same timed horizon from the same start state, plain form
        eng.set_state(slots, start_qpos, start_qvel)
        eng.step(1, STEP_PLAIN)
        eng.set_state(slots, start_qpos, start_qvel)
        eng.sync()
        pms = 0.0
        for _ in range(args.steps):
            eng.flush_l2()
            eng.event(0)
            eng.step(S, STEP_PLAIN)
            eng.event(1)
            pms += eng.elapsed_ms()
        plain = W * S * args.steps / (max_over_ranks(dist, pms) / 1e3)
    err = None
    if not args.no_extras and rank == 0:
        err = fp64_one_step_error(eng, batch, slots, start_qpos, start_qvel)
    hbm, src = peaks()
    avg_ms = total_ms / args.steps
    nb = int(batch.n_bodies[0])
    persistent = fwork["worlds"] > 0
    if persistent:
        # the world-persistent kernel: FP32 work of newt's PGS over the
        # contacts it solved, per launch, against the FP32 pipe's peak
        dom, dom_ms = "pile_k_fused", fused_ms / args.steps
        flops = PGS_FLOP_PER_CONTACT_SWEEP * 50 * fwork["contacts"] / args.steps
        achieved = flops / (dom_ms / 1e3) / 1e12 if dom_ms > 0 else None
        contacts_last = fwork["contacts"] / (args.steps * S)
        alg = fused_kernel_bytes(W, nb, contacts_last)
        hbm_ach = alg / (dom_ms / 1e3) / 1e9 if dom_ms > 0 else None
        traffic = (FUSED_DRAM_BYTES_PER_WORLD_STEP * W * S) if FUSED_DRAM_BYTES_PER_WORLD_STEP else None
        roof = {"bound": "fp32", "kernel": dom, "achieved": achieved, "peak": FP32_PEAK_TFLOPS, "unit": "TFLOP/s",
                "frac": achieved / FP32_PEAK_TFLOPS if achieved else None, "traffic": traffic,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one settled 2048-world "
                                  "launch (profiles/pile_k_fused_2048worlds_settled_full.md), per world-step, "
                                  "scaled to this launch's worlds x env-steps",
                "peak_source": "derived from datasheet figures (152 SMs x 128 FP32 lanes x 2 x 2.07 GHz); "
                               "MEASURED_PEAKS.json has no FP32 figure",
                "flop_per_launch": flops, "flop_formula": "5 x 235 FLOP x 50 sweeps per active contact and env-step "
                                                          "(newt's PGS row updates), contacts counted by the kernel",
                "ms_per_launch": dom_ms, "active_contacts_per_world_step": fwork["contacts"] / (W * S * args.steps),
                "dependency_rounds_per_world_sweep": fwork["rounds"] / (50.0 * W * S * args.steps),
                "hbm": {"achieved": hbm_ach, "peak": hbm, "unit": "GB/s", "frac": hbm_ach / hbm if hbm_ach else None,
                        "peak_source": src, "algorithmic_bytes_per_launch": alg},
                "note": "one launch per bench step (all worlds, all env-steps), timed live by an event pair on its "
                        "stream inside the graph"}
        kernels = {"pile_k_fused": {"ms_per_launch": dom_ms, "share": 1.0, "algorithmic_bytes": alg}}
        mode = ("batched: one world-persistent launch per bench step (a warp per world for all its env-steps, "
                "worlds from a size-sorted queue), CUDA graph")
    else:
        branches = n_launch / (args.steps * S)
        dom = max(kernel_ms, key=kernel_ms.get)
        dom_ms = kernel_ms[dom] / n_launch
        alg = pile_kernel_bytes(dom, W, nb, work) / branches
        achieved = alg / (dom_ms / 1e3) / 1e9 if dom_ms > 0 else None
        roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm if achieved else None, "traffic": None, "peak_source": src,
                "algorithmic_bytes_per_launch": alg, "ms_per_launch": dom_ms}
        tot_k = sum(kernel_ms.values())
        kernels = {k: {"ms_per_launch": v / n_launch, "share": v / tot_k if tot_k else None,
                       "algorithmic_bytes": pile_kernel_bytes(k, W, nb, work) / branches}
                   for k, v in kernel_ms.items()}
        mode = "batched: island-class pipeline, per env-step and world-range branch, CUDA graph"
    out = {
        "metric": "env-steps/s", "value": value, "unit": "env-steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": avg_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
        "config": {"workload": "pile: 16 free spheres/boxes on a plane per world, PGS 50 iterations, dt 2e-3",
                   "worlds_per_gpu": W, "bodies_per_world": 16, "env_steps_per_bench_step": S,
                   "mode": mode, "autotuned": tuned,
                   "l2": "flushed between timed steps", "parallelism": f"replicas x{ws}"},
        "e2e": {"value": e2e, "unit": "env-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clk,
        "roofline": roof,
        "kernels": kernels,
        "status_flags": int(np.bitwise_or.reduce(st)) if len(st) else 0,
    }
    if plain is not None:
        out["plain_value"] = plain
        out["batched_over_plain"] = value / ws / plain
    if err is not None:
        out["error_vs_fp64"] = err
    eng.close()
    return out, (batch, start_qpos, start_qvel)


def run_uneven_compact(rank, ws, local, dist, n_worlds=32768, substeps=25, steps=8):
    """The uneven configuration in brief for the headline line: 32768 chains
    and piles of 2..64 bodies, env-steps 0..200 from the start state, the
    batched form (autotuned) against the plain form on the same worlds,
    throughput over all worlds and over the worlds that stayed finite."""
    from tooling_gb300 import scenes
    batch = scenes.uneven_batch(n_worlds=n_worlds, first_world=rank * n_worlds)
    from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN
    eng = Engine(device=local)
    slots = eng.alloc(eng.upload(batch))
    nq, nv = int(batch.nq.sum()), int(batch.nv.sum())

    def reset():
        eng.set_state(slots, batch.qpos, batch.qvel)
        eng.set_qfrc(slots, batch.qfrc)
        eng.status(slots, clear=True)

    reset()
    eng.step(substeps, STEP_BATCHED)
    tuned = eng.autotune(substeps, horizon=substeps * steps)
    out = {"worlds": n_worlds, "env_steps": substeps * steps, "autotuned": tuned}
    for name, mode in (("batched", STEP_BATCHED), ("plain", STEP_PLAIN)):
        reset()
        eng.step(1, mode)  # captures / builds tables outside the timing
        reset()
        eng.sync()
        barrier(dist)
        ms = 0.0
        for _ in range(steps):
            eng.flush_l2()
            eng.event(0)
            eng.step(substeps, mode)
            eng.event(1)
            ms += eng.elapsed_ms()
        ms = max_over_ranks(dist, ms)
        st = eng.status(slots)
        finite = int(((st & 0x1) == 0).sum())
        out[name] = {"value": n_worlds * substeps * steps * ws / (ms / 1e3),
                     "finite_value": finite * substeps * steps * ws / (ms / 1e3),
                     "finite_worlds": finite, "status_flags": int(np.bitwise_or.reduce(st)), "ms": ms}
    out["batched_over_plain"] = out["batched"]["value"] / out["plain"]["value"]
    out["note"] = ("worlds flagged NEWT_WS_NONFINITE are long chains that newt's own algorithm also blows up on "
                   "at dt 2e-3 (the FP64 oracle diverges on the same worlds); finite_value counts the others only")
    eng.close()
    return out


def run_served_compact(rank, ws, local, dist, rate=10000.0, duration=1.0, pool_worlds=4096, steps_per_tick=8):
    """The served configuration in brief: one Poisson stream at `rate` req/s
    over a pool of uneven worlds, horizons log-uniform in 10..1000, tau ~
    N(0,1) per DoF per env-step, through newt_gpu_serve with
    `steps_per_tick` env-steps per serving tick; p50/p99 latency."""
    from tooling_gb300 import scenes
    pool = scenes.uneven_batch(n_worlds=pool_worlds, first_world=rank * pool_worlds)
    from tooling_gb300 import Engine
    eng = Engine(device=local)
    ids = eng.upload(pool)
    nv = pool.nv.astype(np.int64)
    rng = np.random.default_rng(scenes.config_seed(4) + rank)
    tau = rng.standard_normal(1 << 22).astype(np.float32)

    def one(d):
        arrivals, world, hz, coff = serve_requests(rng, len(pool), nv, rate, d, tau)
        qp = np.concatenate([pool.qpos[pool.q_off[w]:pool.q_off[w] + pool.nq[w]] for w in world])
        qv = np.concatenate([pool.qvel[pool.v_off[w]:pool.v_off[w] + pool.nv[w]] for w in world])
        oq, ov, st, _, _ = eng.serve(ids[world], hz, arrivals, qp, qv, tau, coff, steps_per_tick=steps_per_tick)
        qo = np.concatenate([[0], np.cumsum(pool.nq[world])])
        bad = np.add.reduceat((~np.isfinite(oq)).astype(np.int64), qo[:-1]) if len(world) else np.zeros(0)
        st["requests"] = len(world)
        st["nonfinite_requests"] = int((bad > 0).sum())
        return st

    one(0.2)  # warm-up: groups grown, graph captured
    barrier(dist)
    st = one(duration)
    keep = ["requests", "completed", "p50_ms", "p99_ms", "max_ms", "mean_active", "ticks", "wall_s",
            "nonfinite_requests"]
    out = {k: st[k] for k in keep}
    out["rate_req_per_s"] = rate
    out["steps_per_tick"] = steps_per_tick
    out["env_steps_per_s"] = st["env_steps"] / st["wall_s"] if st["wall_s"] > 0 else 0.0
    eng.close()
    return out


def tc_kernel_bytes(kernel: str, n_worlds: int, batch, contacts_per_world: float) -> float:
    """Algorithmic HBM bytes of one launch (one env-step) of a tree-contact
    kernel for quadruped worlds (13 links, 14 geoms, nq 19, nv 18).
      tree_aba_kernel: per link model (axis, joint offsets, mass, inertia,
        damping, armature: 18 words), q, qdot and qfrc read, qacc written;
      tc_k_solve: the same model plus 20 words per geom, q, qdot and a_free
        read, qacc written, and per contact its 24-word record and 4 impulses
        written;
      tree_integrate_kernel: q, qdot, qacc read, q and qdot written."""
    L, G, nq, nv = int(batch.n_links[0]), int(batch.n_geoms[0]), int(batch.nq[0]), int(batch.nv[0])
    if kernel == "tree_aba_kernel":
        words = 18 * L + nq + 2 * nv + nv
    elif kernel == "tc_k_solve":
        words = 18 * L + 20 * G + nq + 2 * nv + nv + contacts_per_world * 28
    else:
        words = nq + 2 * nv + nq + nv
    return 4.0 * n_worlds * words


def run_gpu_quadruped(args, rank, ws, local, dist):
    """Quadrupeds on a plane, Newton <= 20 iterations, dt 2e-3: one bench
    step is one control block of 20 env-steps (the torques are resampled
    every 20 steps and uploaded before the block)."""
    from tooling_gb300 import build as B
    B.build()
    from tooling_gb300 import Engine, STEP_BATCHED, scenes
    eng = Engine(device=local)
    W = args.worlds
    batch = scenes.quadruped_batch(n_worlds=W, first_world=rank * W)
    slots = eng.alloc(eng.upload(batch))
    eng.set_state(slots, batch.qpos, batch.qvel)
    S = 20
    n_blocks = max(3, args.warmup) + 2 * args.steps
    ctrl = [scenes.quadruped_controls(W, k, first_world=rank * W) for k in range(n_blocks)]
    eng.pile_profile(1)
    blk = 0
    for _ in range(max(3, args.warmup)):
        eng.set_qfrc(slots, ctrl[blk]); blk += 1
        eng.step(S, STEP_BATCHED)
    eng.sync()
    start_qpos, start_qvel = eng.get_state(slots, int(batch.nq.sum()), int(batch.nv.sum()))
    launches0 = eng.launch_count()
    clocks = Clocks(local)
    clocks.start()
    per_step, kernel_ms = [], {}
    barrier(dist)
    eng.sync()
    for _ in range(args.steps):
        eng.set_qfrc(slots, ctrl[blk]); blk += 1  # the control block, uploaded before the timed step
        eng.flush_l2()
        eng.event(0)
        eng.step(S, STEP_BATCHED)
        eng.event(1)
        per_step.append(eng.elapsed_ms())
        for k, v in eng.tc_profile().items():
            kernel_ms[k] = kernel_ms.get(k, 0.0) + v
    eng.sync()
    barrier(dist)
    clk = clocks.stop()
    launches = eng.launch_count() - launches0
    total_ms = max_over_ranks(dist, float(sum(per_step)))
    value = W * S * args.steps * ws / (total_ms / 1e3)
    st = eng.status(slots)
    sample = slots[:: max(1, W // 64)]
    contacts = float(np.mean([len(eng.contacts(int(s))[0]) for s in sample]))
    # e2e: host state and controls in, host state out, every bench step
    qp, qv = pinned_like(start_qpos), pinned_like(start_qvel)
    h2d = qp.nbytes + qv.nbytes + ctrl[0].nbytes
    d2h = qp.nbytes + qv.nbytes
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.set_state(slots, qp, qv)
        eng.set_qfrc(slots, ctrl[blk]); blk += 1
        eng.step(S, STEP_BATCHED)
        eng.get_state(slots, int(batch.nq.sum()), int(batch.nv.sum()), out=(qp, qv))
    eng.sync()
    e2e = W * S * args.steps * ws / max_over_ranks(dist, time.perf_counter() - t0)
    hbm, src = peaks()
    n_launch = args.steps * S
    dom = max(kernel_ms, key=kernel_ms.get)
    dom_ms = kernel_ms[dom] / n_launch
    alg = tc_kernel_bytes(dom, W, batch, contacts)
    achieved = alg / (dom_ms / 1e3) / 1e9 if dom_ms > 0 else None
    tot_k = sum(kernel_ms.values())
    avg_ms = total_ms / args.steps
    out = {
        "metric": "env-steps/s", "value": value, "unit": "env-steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": avg_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
        "config": {"workload": "quadruped: floating torso + 4x3 revolute legs on a plane, Newton <= 20 iterations, "
                               "dt 2e-3, tau ~ N(0,2) resampled every 20 steps",
                   "worlds_per_gpu": W, "dof": int(batch.nv[0]), "env_steps_per_bench_step": S,
                   "mode": "3 kernels per env-step (ABA, warp-per-world contact solve, integrate)",
                   "l2": "flushed between timed steps (working set also exceeds L2)",
                   "parallelism": f"replicas x{ws}", "contacts_per_world_end": contacts},
        "e2e": {"value": e2e, "unit": "env-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clk,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm if achieved else None, "traffic": None, "peak_source": src,
                     "algorithmic_bytes_per_launch": alg, "ms_per_launch": dom_ms,
                     "note": "dense per-world Newton solves, latency-bound; timed live by event pairs on the "
                             "launching stream"},
        "kernels": {k: {"ms_per_launch": v / n_launch, "share": v / tot_k if tot_k else None,
                        "algorithmic_bytes": tc_kernel_bytes(k, W, batch, contacts)} for k, v in kernel_ms.items()},
        "status_flags": int(np.bitwise_or.reduce(st)) if len(st) else 0,
    }
    eng.close()
    return out, (batch, start_qpos, start_qvel, ctrl[0])


def run_gpu_uneven(args, rank, ws, local, dist):
    """Uneven batch: chains and piles with 2..64 bodies (log-uniform), PGS 50,
    dt 2e-3.  The batched form (tree persistent kernels per size bucket plus
    one pile table over every size, captured in a CUDA graph) is timed beside
    the plain form (one launch per stage per size group) on the same worlds
    from the same start state."""
    from tooling_gb300 import build as B
    B.build()
    from tooling_gb300 import scenes
    batch = scenes.uneven_batch(n_worlds=args.worlds, first_world=rank * args.worlds)  # before the first GPU call
    from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN
    eng = Engine(device=local)
    W = args.worlds
    slots = eng.alloc(eng.upload(batch))
    eng.set_state(slots, batch.qpos, batch.qvel)
    eng.set_qfrc(slots, batch.qfrc)
    S = args.substeps
    eng.pile_profile(1)
    # warm-up (graph capture, first-touch) and the launch-choice autotuner,
    # then back to the start state: the timed steps cover env-steps
    # 0 .. steps x substeps of every world
    for _ in range(max(3, args.warmup)):
        eng.step(S, STEP_BATCHED)
    tuned = eng.autotune(S, horizon=S * args.steps)
    eng.step(S, STEP_BATCHED)
    eng.sync()
    nq, nv = int(batch.nq.sum()), int(batch.nv.sum())
    start_qpos, start_qvel = batch.qpos.copy(), batch.qvel.copy()
    eng.set_state(slots, start_qpos, start_qvel)
    eng.sync()
    launches0 = eng.launch_count()
    clocks = Clocks(local)
    clocks.start()
    per_step, kernel_ms, work, n_launch = [], {}, None, 0
    barrier(dist)
    eng.sync()
    for _ in range(args.steps):
        eng.flush_l2()
        eng.event(0)
        eng.step(S, STEP_BATCHED)
        eng.event(1)
        per_step.append(eng.elapsed_ms())
        kms, work = eng.pile_profile()
        n_launch += work["launches"]
        for k, v in kms.items():
            kernel_ms[k] = kernel_ms.get(k, 0.0) + v
    eng.sync()
    barrier(dist)
    clk = clocks.stop()
    launches = eng.launch_count() - launches0
    total_ms = max_over_ranks(dist, float(sum(per_step)))
    value = W * S * args.steps * ws / (total_ms / 1e3)
    st = eng.status(slots)
    # plain form, same worlds, same start state
    eng.set_state(slots, start_qpos, start_qvel)
    eng.step(1, STEP_PLAIN)  # builds the per-group tables (allocation outside the timed region)
    eng.set_state(slots, start_qpos, start_qvel)
    eng.sync()
    plain_launch0 = eng.launch_count()
    pms = 0.0
    for _ in range(args.steps):
        eng.flush_l2()
        eng.event(0)
        eng.step(S, STEP_PLAIN)
        eng.event(1)
        pms += eng.elapsed_ms()
    plain_launches = eng.launch_count() - plain_launch0
    plain = W * S * args.steps / (max_over_ranks(dist, pms) / 1e3)
    # e2e through the C ABI with host buffers, batched form
    qp, qv = pinned_like(start_qpos), pinned_like(start_qvel)
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.set_state(slots, qp, qv)
        eng.step(S, STEP_BATCHED)
        eng.get_state(slots, nq, nv, out=(qp, qv))
    eng.sync()
    e2e = W * S * args.steps * ws / max_over_ranks(dist, time.perf_counter() - t0)
    hbm, src = peaks()
    branches = n_launch / (args.steps * S) if n_launch else 1.0
    dom = max(kernel_ms, key=kernel_ms.get)
    dom_ms = kernel_ms[dom] / max(n_launch, 1)
    n_piles = int((batch.n_bodies > 0).sum())
    # pile kernels see the pile worlds only; the mean body count stands in for every world's
    mean_nb = int(round(float(batch.n_bodies[batch.n_bodies > 0].mean()))) if n_piles else 0
    alg = pile_kernel_bytes(dom, n_piles, mean_nb, work) / branches
    achieved = alg / (dom_ms / 1e3) / 1e9 if dom_ms > 0 else None
    out = {
        "metric": "env-steps/s", "value": value, "unit": "env-steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
        "config": {"workload": "uneven: 50/50 chains and piles, 2..64 bodies log-uniform, PGS 50, dt 2e-3",
                   "worlds_per_gpu": W, "chains": W - n_piles, "piles": n_piles, "env_steps_per_bench_step": S,
                   "horizon": f"env-steps 0..{S * args.steps} from the start state (piles fall and settle)",
                   "autotuned": tuned,
                   "mode": "batched: tree persistent kernels per size bucket + one pile table, CUDA graph",
                   "l2": "flushed between timed steps", "parallelism": f"replicas x{ws}"},
        "plain_value": plain, "batched_over_plain": value / ws / plain,
        "plain_launches_per_bench_step": plain_launches / args.steps,
        "e2e": {"value": e2e, "unit": "env-steps/s", "h2d_bytes_per_step": qp.nbytes + qv.nbytes,
                "d2h_bytes_per_step": qp.nbytes + qv.nbytes},
        "gpu_launches": launches,
        "clocks": clk,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm if achieved else None, "traffic": None, "peak_source": src,
                     "algorithmic_bytes_per_launch": alg, "ms_per_launch": dom_ms,
                     "note": "pile kernels timed live inside the graph; the tree persistent kernels run "
                             "concurrently on a second branch"},
        "status_flags": int(np.bitwise_or.reduce(st)) if len(st) else 0,
    }
    eng.close()
    return out


def serve_requests(rng, n_pool, nv, rate, duration, tau):
    """Poisson arrivals over `duration` s at `rate` req/s; each request is one
    pool world with horizon floor(exp(U(ln 10, ln 1001))) and a window of
    N(0,1) controls (horizon x nv) from a shared seeded pool."""
    gaps = rng.exponential(1.0 / rate, int(rate * duration * 1.3) + 16)
    arrivals = np.cumsum(gaps)
    arrivals = arrivals[arrivals < duration]
    n = len(arrivals)
    world = rng.integers(0, n_pool, n)
    hz = np.floor(np.exp(rng.uniform(np.log(10.0), np.log(1001.0), n))).astype(np.int32)
    need = hz.astype(np.int64) * nv[world]
    coff = (rng.random(n) * (tau.size - need)).astype(np.int64)
    return arrivals, world, hz, coff


def run_gpu_serve(args, rank, ws, local, dist):
    """Served rollouts: Poisson request streams over a pool of uneven worlds
    (chains and piles, 2..64 bodies), each request an initial state, a
    control sequence tau ~ N(0,1) per DoF per env-step and a log-uniform
    horizon in 10..1000; admitted into free world slots, stepped with every
    other admitted request (--steps-per-tick env-steps per serving tick, a
    world held at the env-step its horizon ends), read back at completion.
    Timed on the wall clock through newt_gpu_serve (host buffers in and out)."""
    from tooling_gb300 import build as B
    B.build()
    from tooling_gb300 import scenes
    pool = scenes.uneven_batch(n_worlds=args.worlds, first_world=rank * args.worlds)  # before the first GPU call
    from tooling_gb300 import Engine, STEP_BATCHED, STEP_PLAIN
    eng = Engine(device=local)
    ids = eng.upload(pool)
    nv = pool.nv.astype(np.int64)
    rng = np.random.default_rng(scenes.config_seed(4) + rank)
    tau = rng.standard_normal(1 << 24).astype(np.float32)
    rates = [float(r) for r in args.rates.split(",") if r]

    def inputs(world):
        qp = np.concatenate([pool.qpos[pool.q_off[w]:pool.q_off[w] + pool.nq[w]] for w in world])
        qv = np.concatenate([pool.qvel[pool.v_off[w]:pool.v_off[w] + pool.nv[w]] for w in world])
        return qp, qv

    def serve(rate, duration, mode=STEP_BATCHED, k=args.steps_per_tick):
        arrivals, world, hz, coff = serve_requests(rng, len(pool), nv, rate, duration, tau)
        qp, qv = inputs(world)
        barrier(dist)
        l0 = eng.launch_count()
        oq, ov, st, admit, done = eng.serve(ids[world], hz, arrivals, qp, qv, tau, coff, mode=mode,
                                            steps_per_tick=k)
        st["launches"] = eng.launch_count() - l0
        st["requests"] = len(world)
        st["rate"] = rate
        st["env_steps_per_s"] = st["env_steps"] / st["wall_s"] if st["wall_s"] > 0 else 0.0
        st["h2d_bytes"] = int(qp.nbytes + qv.nbytes + 4 * int((hz.astype(np.int64) * nv[world]).sum()))
        st["d2h_bytes"] = int(oq.nbytes + ov.nbytes)
        qo = np.concatenate([[0], np.cumsum(pool.nq[world])])
        bad = np.add.reduceat((~np.isfinite(oq)).astype(np.int64), qo[:-1]) if len(world) else np.zeros(0)
        st["nonfinite_requests"] = int((bad > 0).sum())
        return st

    # rates in increasing order, each after a short warm-up at its own rate
    # (grows the world groups to that rate's working set and captures the
    # one-env-step graph); the clocks are sampled over the timed runs only
    rates = sorted(rates)
    runs, clk_runs = [], []
    for r in rates:
        for _ in range(max(3, args.warmup)):
            serve(r, min(0.2, args.duration))
        clocks = Clocks(local)
        clocks.start()
        runs.append(serve(r, args.duration))
        clk_runs.append(clocks.stop())
    clk = clk_runs[-1]
    clk["reasons"] = sorted(set(x for c in clk_runs for x in c.get("reasons", [])))
    top = runs[-1]
    plain = serve(top["rate"], args.duration, STEP_PLAIN) if not args.no_plain else None
    one_step = serve(top["rate"], args.duration, k=1) if args.steps_per_tick > 1 else None
    ticks = max(1, top["ticks"])
    value = max_over_ranks(dist, 1.0 / top["env_steps_per_s"]) if top["env_steps_per_s"] > 0 else 0.0
    value = ws / value if value > 0 else 0.0
    keep = ["rate", "requests", "completed", "env_steps_per_s", "p50_ms", "p99_ms", "max_ms", "mean_ms",
            "mean_active", "peak_active", "ticks", "wall_s", "admit_s", "ctrl_s", "step_s", "complete_s",
            "nonfinite_requests"]
    out = {
        "metric": "env-steps/s", "value": value, "unit": "env-steps/s", "n_gpus": ws, "steps": len(rates),
        "warmup": max(3, args.warmup), "ms_per_step": 1e3 * top["wall_s"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
        "config": {"workload": "served rollouts: Poisson arrivals, uneven worlds (chains and piles, 2..64 "
                               "bodies), tau ~ N(0,1) per DoF per env-step, horizon log-uniform 10..1000",
                   "world_pool": len(pool), "rates_req_per_s": rates, "seconds_of_arrivals": args.duration,
                   "step": f"{args.steps_per_tick} env-steps queued per tick (worlds held where their horizon "
                           "ends), one step call per env-step, batched form (CUDA graph)",
                   "l2": "inputs resident; working set above L2 at the top rates",
                   "parallelism": f"replicas x{ws}"},
        "served": [{k: r[k] for k in keep} for r in runs],
        "e2e": {"value": top["env_steps_per_s"] * ws, "unit": "env-steps/s",
                "h2d_bytes_per_step": top["h2d_bytes"] / ticks, "d2h_bytes_per_step": top["d2h_bytes"] / ticks,
                "note": "value and e2e are both the served wall-clock rate at the top request rate: the serve "
                        "loop is itself the end-to-end path (a step here is one tick)"},
        "gpu_launches": int(sum(r["launches"] for r in runs)),
        "clocks": clk,
    }
    if one_step is not None:
        out["one_step_ticks"] = {k: one_step[k] for k in keep}
    if plain is not None:
        out["plain_served"] = {k: plain[k] for k in keep}
        out["batched_over_plain"] = top["env_steps_per_s"] / plain["env_steps_per_s"] if plain["env_steps_per_s"] else None
    eng.close()
    return out


def cpu_baseline_quadruped(batch, qpos, qvel, qfrc, n_worlds=256, steps=40):
    """The f32 restatement of newt's step (Newton tree-contact solve) on all
    host cores, on a sample of the quadrupeds from the timed region's start."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py
    from tooling_gb300 import scenes
    cores = os.cpu_count() or 1
    n = min(n_worlds, len(batch))
    sub = scenes.quadruped_batch(n_worlds=n)
    qp = qpos[: int(sub.nq.sum())]
    qv = qvel[: int(sub.nv.sum())]
    qf = qfrc[: int(sub.nv.sum())]
    secs = oracle_py.time_run(sub, np.arange(n), qp, qv, qf, steps, cores)
    return {"value": n * steps / secs, "unit": "env-steps/s", "cores": cores, "kind": "port",
            "sample": f"{n} quadruped worlds x {steps} env-steps from the bench's start state, f32 restatement of "
                      f"newt's step (Newton tree-contact solve), {cores} host threads"}


def cpu_baseline(batch, qpos, qvel, S, n_worlds=256, steps=500):
    """The f32 restatement of newt's step on the host cores: one world per
    thread, static partition, all cores; a sample of the worlds over the same
    horizon the GPU timed region covers."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py
    from tooling_gb300 import model as M
    cores = os.cpu_count() or 1
    idx = np.arange(min(n_worlds, len(batch)))
    qp = np.concatenate([qpos[batch.q_off[w]:batch.q_off[w] + batch.nq[w]] for w in idx])
    qv = np.concatenate([qvel[batch.v_off[w]:batch.v_off[w] + batch.nv[w]] for w in idx])
    n_steps = steps or S
    # a ModelDesc array for just the sampled worlds
    sub = M.Batch(batch.links, batch.n_links[idx], batch.bodies[:int(batch.n_bodies[idx].sum())], batch.n_bodies[idx],
                  batch.geoms[:int(batch.n_geoms[idx].sum())], batch.n_geoms[idx], 2e-3, (0.0, 0.0, -9.81),
                  M.SOLVER_PGS, 50)
    secs = oracle_py.time_run(sub, np.arange(len(idx)), qp, qv, None, n_steps, cores)
    return {"value": len(idx) * n_steps / secs, "unit": "env-steps/s", "cores": cores, "kind": "port",
            "sample": f"{len(idx)} pile worlds x {n_steps} env-steps from the bench's start state, f32 restatement of "
                      f"newt's step, {cores} host threads"}


def run_reference(args, rank, ws, local, dist):
    """newt's algorithm on the host cores for the chosen workload: the float
    restatement (newt is Rust and cannot be built here), all host threads, a
    bounded sample of the workload's worlds advancing `substeps` env-steps per
    bench step from the GPU arm's start phase."""
    if rank != 0:
        return None
    from tooling_gb300 import scenes
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py
    cores = os.cpu_count() or 1
    line = {"impl": "reference", "metric": "env-steps/s", "unit": "env-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator)"}
    if args.workload == "serve":
        line["unavailable"] = ("newt has no serving loop; its per-world step on the host cores is timed by "
                               "--impl reference --workload uneven")
        return line
    S, qfrc = args.substeps, None
    if args.workload == "quadruped":
        n, S = min(args.worlds, 64), 20
        batch = scenes.quadruped_batch(n_worlds=n)
        qfrc = scenes.quadruped_controls(n, 0)
        config = {"workload": "quadruped: 13-link trees on a plane, Newton <= 20, dt 2e-3",
                  "worlds_per_gpu": args.worlds}
    elif args.workload == "uneven":
        n = min(args.worlds, 256)
        batch = scenes.uneven_batch(n_worlds=n)
        qfrc = batch.qfrc
        config = {"workload": "uneven: 50/50 chains and piles, 2..64 bodies log-uniform, PGS 50, dt 2e-3",
                  "worlds_per_gpu": args.worlds}
    else:
        n = min(args.worlds, 256)
        batch = scenes.pile_batch(n_worlds=n)
        config = {"workload": "pile: free spheres/boxes on a plane, PGS 50 iterations, dt 2e-3",
                  "worlds_per_gpu": args.worlds, "bodies_per_world": 16}
    idx = np.arange(n)
    # advance the sample to the GPU arm's start phase (its warm-up horizon), untimed
    qo, vo = oracle_py.run(batch, idx, batch.qpos, batch.qvel, qfrc, max(3, args.warmup) * S, precision=0,
                           n_threads=cores)
    qp, qv = qo.astype(np.float32), vo.astype(np.float32)
    vals = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        qo, vo = oracle_py.run(batch, idx, qp, qv, qfrc, S, precision=0, n_threads=cores)
        vals.append(n * S / (time.perf_counter() - t0))
        qp, qv = qo.astype(np.float32), vo.astype(np.float32)
    v = statistics.median(vals)
    sample = (f"{n} worlds x {S} env-steps per step, advancing from the GPU arm's start phase, f32 restatement of "
              f"newt's step, {cores} host threads; newt is Rust and cannot be built here (no cargo), so its "
              f"arithmetic runs through the byte-identical C++ restatement")
    line.update({"value": v, "config": config,
                 "cpu_baseline": {"value": v, "unit": "env-steps/s", "cores": cores, "kind": "port", "sample": sample},
                 "e2e": {"value": v, "unit": "env-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
    return line


def main():
    args = parse()
    rank, ws, local, dist = dist_setup()
    if "--worlds" not in sys.argv:  # each workload's configured world count
        args.worlds = {"uneven": 32768, "quadruped": 16384}.get(args.workload, args.worlds)
    if args.impl == "reference":
        out = run_reference(args, rank, ws, local, dist)
        if out is not None:
            print(json.dumps(out))
        return
    if args.workload == "serve":
        out = run_gpu_serve(args, rank, ws, local, dist)
        if rank == 0:
            print(json.dumps(out))
        return
    if args.workload == "uneven":
        out = run_gpu_uneven(args, rank, ws, local, dist)
        if rank == 0:
            print(json.dumps(out))
        return
    if args.workload == "quadruped":
        out, (batch, qp, qv, qf) = run_gpu_quadruped(args, rank, ws, local, dist)
        if rank == 0:
            if not args.no_cpu and ws == 1:
                out["cpu_baseline"] = cpu_baseline_quadruped(batch, qp, qv, qf)
            print(json.dumps(out))
        return
    out, (batch, qp, qv) = run_gpu(args, rank, ws, local, dist)
    if not args.no_extras:
        out["uneven"] = run_uneven_compact(rank, ws, local, dist)
        out["served"] = run_served_compact(rank, ws, local, dist, steps_per_tick=args.steps_per_tick)
    if rank == 0:
        if not args.no_cpu and ws == 1:
            out["cpu_baseline"] = cpu_baseline(batch, qp, qv, args.substeps, steps=args.substeps * args.steps)
        print(json.dumps(out))


if __name__ == "__main__":
    main()
