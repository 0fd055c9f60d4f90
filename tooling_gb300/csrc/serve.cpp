// Served rollouts: the request loop above the C ABI (include/newt_gpu.h,
// newt_gpu_serve).  It plays the role of newt's callers, which own a World
// and call World::step in their own loop (sandbox/src/main.rs:601), for many
// requests at once, and uses only the public entry points:
//
//   admission   requests that have arrived join in arrival order while the
//               active count is under `max_active` and newt_gpu_alloc_worlds
//               finds room in the device budget (NEWT_E_NOMEM: the request
//               waits for completions); freed world slots are reused, so the
//               captured step graph stays valid while no group grows
//   tick        `steps_per_tick` times: the next row of each admitted
//               request's control stream (uploaded once at admission,
//               newt_gpu_set_ctrl_stream) goes to its qfrc on the device,
//               then one step call of one env-step advances every admitted
//               world together (continuous batching); the env-steps of a
//               tick are queued without a host wait, and a world whose
//               horizon ends inside the tick is held at that env-step
//               (newt_gpu_hold_worlds)
//   completion  a request whose horizon is reached has its final state read
//               back and its slot freed; latency = completion - arrival
#include <algorithm>
#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/newt_gpu.h"

namespace {

struct Active {
  int req;
  int32_t slot;
  int32_t nq, nv;
  int32_t t;  // env-steps done
};

double percentile(std::vector<double> v, double p) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = p * (double)(v.size() - 1);
  const size_t lo = (size_t)pos, hi = std::min(lo + 1, v.size() - 1);
  return v[lo] + (pos - (double)lo) * (v[hi] - v[lo]);
}

}  // namespace

extern "C" NEWT_API int newt_gpu_serve(newt_gpu_ctx* ctx, newt_serve_request* reqs, int32_t n,
                                       const newt_serve_opts* opts, newt_serve_stats* stats) {
  if (!ctx || n < 0 || (n > 0 && !reqs) || !stats) return NEWT_E_INVALID;
  const int max_active = opts && opts->max_active > 0 ? opts->max_active : (1 << 30);
  const bool real_time = !opts || opts->real_time != 0;
  const int mode = opts ? opts->step_mode : NEWT_STEP_BATCHED;
  const int ksteps = opts && opts->steps_per_tick > 1 ? opts->steps_per_tick : 1;
  if (mode != NEWT_STEP_BATCHED && mode != NEWT_STEP_PLAIN) return NEWT_E_INVALID;
  std::memset(stats, 0, sizeof(*stats));
  for (int i = 0; i < n; ++i) {
    if (reqs[i].horizon < 0 || !reqs[i].qpos || !reqs[i].qvel) return NEWT_E_INVALID;
    reqs[i].admit_s = -1.0;
    reqs[i].done_s = -1.0;
  }
  // arrival order
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return reqs[a].arrival_s < reqs[b].arrival_s; });
  const auto t0 = std::chrono::steady_clock::now();
  auto now = [&]() { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); };

  std::vector<Active> active;
  std::vector<double> lat;
  size_t next = 0;
  int done = 0;
  double active_sum = 0.0;
  std::vector<int32_t> ids, slots, hold;
  std::vector<float> qp, qv, qf;
  bool full = false;  // the budget refused a world: wait for a completion
  // on an error the admitted worlds are released before returning
  auto bail = [&](int rc) {
    std::vector<int32_t> held;
    for (const Active& a : active) held.push_back(a.slot);
    if (!held.empty()) newt_gpu_free_worlds(ctx, held.data(), (int32_t)held.size());
    return rc;
  };
  while (done < n) {
    // ---- admission ----
    const double tn = now();
    ids.clear();
    std::vector<int> admit;
    while (!full && next < order.size() && (int)(active.size() + admit.size()) < max_active &&
           (!real_time || reqs[order[next]].arrival_s <= tn)) {
      newt_serve_request& r = reqs[order[next]];
      ++next;
      if (r.horizon == 0) {  // nothing to step: the initial state is the result
        int32_t nq = 0, nv = 0;
        int rc = newt_gpu_model_dims(ctx, r.model_id, &nq, &nv);
        if (rc != NEWT_OK) return bail(rc);
        if (r.qpos_out) std::memcpy(r.qpos_out, r.qpos, nq * sizeof(float));
        if (r.qvel_out) std::memcpy(r.qvel_out, r.qvel, nv * sizeof(float));
        r.admit_s = r.done_s = now();
        lat.push_back(1e3 * (r.done_s - (real_time ? r.arrival_s : 0.0)));
        ++done;
        continue;
      }
      admit.push_back(order[next - 1]);
      ids.push_back(r.model_id);
    }
    if (!admit.empty()) {
      slots.assign(admit.size(), -1);
      int rc = newt_gpu_alloc_worlds(ctx, ids.data(), (int32_t)ids.size(), slots.data());
      if (rc == NEWT_E_NOMEM) {
        // admit one at a time until the budget refuses; the rest wait
        size_t k = 0;
        for (; k < admit.size(); ++k) {
          rc = newt_gpu_alloc_worlds(ctx, &ids[k], 1, &slots[k]);
          if (rc != NEWT_OK) break;
        }
        if (rc != NEWT_OK && rc != NEWT_E_NOMEM) {
          if (k > 0) newt_gpu_free_worlds(ctx, slots.data(), (int32_t)k);
          return bail(rc);
        }
        if (k == 0 && active.empty()) return NEWT_E_NOMEM;  // can never fit
        // the refused requests go back to the head of the queue, in order
        for (size_t j = admit.size(); j-- > k;) order[--next] = admit[j];
        admit.resize(k);
        slots.resize(k);
        full = true;
      } else if (rc != NEWT_OK) {
        return bail(rc);
      }
      qp.clear();
      qv.clear();
      for (size_t k = 0; k < admit.size(); ++k) {
        newt_serve_request& r = reqs[admit[k]];
        int32_t nq = 0, nv = 0;
        newt_gpu_model_dims(ctx, r.model_id, &nq, &nv);
        qp.insert(qp.end(), r.qpos, r.qpos + nq);
        qv.insert(qv.end(), r.qvel, r.qvel + nv);
        r.admit_s = now();
        active.push_back(Active{admit[k], slots[k], nq, nv, 0});
      }
      if (!admit.empty()) {
        int rc2 = newt_gpu_set_state(ctx, slots.data(), (int32_t)slots.size(), qp.data(), qv.data());
        if (rc2 != NEWT_OK) return bail(rc2);
        // the admitted requests' whole control sequences go to the device once
        std::vector<int32_t> cs, hz;
        qf.clear();
        for (size_t k = 0; k < admit.size(); ++k) {
          const newt_serve_request& r = reqs[admit[k]];
          if (!r.ctrl || r.horizon == 0) continue;
          cs.push_back(slots[k]);
          hz.push_back(r.horizon);
          qf.insert(qf.end(), r.ctrl, r.ctrl + (size_t)r.horizon * active[active.size() - admit.size() + k].nv);
        }
        if (!cs.empty()) {
          rc2 = newt_gpu_set_ctrl_stream(ctx, cs.data(), (int32_t)cs.size(), qf.data(), hz.data());
          if (rc2 != NEWT_OK) return bail(rc2);
        }
      }
    }
    stats->admit_s += now() - tn;
    if (active.empty()) {
      if (next < order.size() && real_time) {  // idle until the next arrival
        const double wait = reqs[order[next]].arrival_s - now();
        if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.01)));
      }
      continue;
    }
    // ---- tick: kt env-steps, each the next control row of every stream and
    //      one step call, queued without a host wait; a world whose horizon
    //      ends inside the tick is held at that env-step ----
    int kt = 1;
    for (const Active& a : active) kt = std::max(kt, std::min(ksteps, reqs[a.req].horizon - a.t));
    int rc = NEWT_OK;
    for (int s = 0; s < kt && rc == NEWT_OK; ++s) {
      const double tc = now();
      rc = newt_gpu_apply_ctrl(ctx);
      const double ts = now();
      stats->ctrl_s += ts - tc;
      if (rc == NEWT_OK) rc = newt_gpu_step(ctx, 1, mode);
      if (rc == NEWT_OK && s + 1 < kt) {
        hold.clear();
        for (const Active& a : active)
          if (a.t + s + 1 == reqs[a.req].horizon) hold.push_back(a.slot);
        if (!hold.empty()) rc = newt_gpu_hold_worlds(ctx, hold.data(), (int32_t)hold.size());
      }
      stats->step_s += now() - ts;
    }
    if (rc == NEWT_OK) {
      const double ts = now();
      rc = newt_gpu_sync(ctx, 600000);
      stats->step_s += now() - ts;
    }
    if (rc != NEWT_OK) return bail(rc);
    stats->ticks += 1;
    active_sum += (double)active.size();
    stats->peak_active = std::max<int32_t>(stats->peak_active, (int32_t)active.size());
    // ---- completions ----
    std::vector<size_t> fin;
    for (size_t k = 0; k < active.size(); ++k) {
      active[k].t = std::min(active[k].t + kt, reqs[active[k].req].horizon);
      if (active[k].t >= reqs[active[k].req].horizon) fin.push_back(k);
    }
    if (fin.empty()) continue;
    const double tf = now();
    slots.clear();
    int32_t tq = 0, tv = 0;
    for (size_t k : fin) { slots.push_back(active[k].slot); tq += active[k].nq; tv += active[k].nv; }
    qp.assign(tq, 0.f);
    qv.assign(tv, 0.f);
    rc = newt_gpu_get_state(ctx, slots.data(), (int32_t)slots.size(), qp.data(), qv.data());
    if (rc != NEWT_OK) return bail(rc);
    const double tdone = now();
    size_t oq = 0, ov = 0;
    for (size_t k : fin) {
      newt_serve_request& r = reqs[active[k].req];
      if (r.qpos_out) std::memcpy(r.qpos_out, qp.data() + oq, active[k].nq * sizeof(float));
      if (r.qvel_out) std::memcpy(r.qvel_out, qv.data() + ov, active[k].nv * sizeof(float));
      oq += active[k].nq;
      ov += active[k].nv;
      r.done_s = tdone;
      lat.push_back(1e3 * (tdone - (real_time ? r.arrival_s : 0.0)));
      stats->env_steps += (double)r.horizon;
      ++done;
    }
    rc = newt_gpu_free_worlds(ctx, slots.data(), (int32_t)slots.size());
    if (rc != NEWT_OK) return rc;
    full = false;
    std::vector<Active> keep;
    keep.reserve(active.size());
    for (size_t k = 0, f = 0; k < active.size(); ++k) {
      if (f < fin.size() && fin[f] == k) { ++f; continue; }
      keep.push_back(active[k]);
    }
    active.swap(keep);
    stats->complete_s += now() - tf;
  }
  stats->completed = done;
  stats->wall_s = now();
  stats->mean_active = stats->ticks ? active_sum / (double)stats->ticks : 0.0;
  stats->p50_ms = percentile(lat, 0.50);
  stats->p99_ms = percentile(lat, 0.99);
  stats->max_ms = lat.empty() ? 0.0 : *std::max_element(lat.begin(), lat.end());
  double s = 0.0;
  for (double x : lat) s += x;
  stats->mean_ms = lat.empty() ? 0.0 : s / (double)lat.size();
  return NEWT_OK;
}
