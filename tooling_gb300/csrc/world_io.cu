// Per-world state I/O: moves chosen rows of the named worlds between the
// host mirror and the device, so a call that touches k worlds moves k worlds'
// rows (what newt's World::apply_mujoco_qpos/qvel, newt/src/world.rs:519-623,
// touches for one world) instead of whole groups.
//
// One call packs every group's segment into one pinned staging buffer, makes
// one copy and one scatter (or gather) launch per group, then synchronises
// once; a group whose named worlds are consecutive indices skips the packing
// and moves by one strided copy.  The packed order follows the device layout so both sides of each
// launch are coalesced: tree groups keep fields as rows x cap (packed as
// rows x k), pile groups keep worlds contiguous (packed as k x rows).
#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "runtime.h"

#define CKW(call)                                                               \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) { ctx->err = std::string(#call ": ") + cudaGetErrorString(e_); return NEWT_E_CUDA; } \
  } while (0)

namespace {

__global__ void rows_scatter(float* __restrict__ dF, int soa, int cap, int frows, int lo, int cnt,
                             const int* __restrict__ idx, int k, const float* __restrict__ src) {
  const long total = (long)k * cnt;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    if (soa) {
      const int r = (int)(t / k), j = (int)(t % k);
      dF[(size_t)(lo + r) * cap + idx[j]] = src[t];
    } else {
      const int j = (int)(t / cnt), r = (int)(t % cnt);
      dF[(size_t)idx[j] * frows + lo + r] = src[t];
    }
  }
}

__global__ void rows_gather(const float* __restrict__ dF, int soa, int cap, int frows, int lo, int cnt,
                            const int* __restrict__ idx, int k, float* __restrict__ dst) {
  const long total = (long)k * cnt;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    if (soa) {
      const int r = (int)(t / k), j = (int)(t % k);
      dst[t] = dF[(size_t)(lo + r) * cap + idx[j]];
    } else {
      const int j = (int)(t / cnt), r = (int)(t % cnt);
      dst[t] = dF[(size_t)idx[j] * frows + lo + r];
    }
  }
}

__global__ void flags_clear(int* const* __restrict__ flags, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) *flags[i] = 0;
}

int grid_for(long total) {
  const long b = (total + 255) / 256;
  return (int)std::max<long>(1, std::min<long>(b, 152L * 16));
}

// staging: [idx ints | floats], both for every segment of the call
int ensure_staging(newt_gpu_ctx* ctx, size_t n_idx, size_t n_f) {
  const size_t bytes = ((n_idx * sizeof(int) + 255) & ~(size_t)255) + n_f * sizeof(float);
  if (bytes <= ctx->io_bytes) return NEWT_OK;
  size_t want = std::max<size_t>(bytes, 2 * ctx->io_bytes);
  want = std::max<size_t>(want, 1 << 20);
  if (ctx->io_h) cudaFreeHost(ctx->io_h);
  if (ctx->io_d) cudaFree(ctx->io_d);
  ctx->io_h = nullptr;
  ctx->io_d = nullptr;
  ctx->io_bytes = 0;
  CKW(cudaMallocHost(&ctx->io_h, want));
  CKW(cudaMalloc(&ctx->io_d, want));
  ctx->io_bytes = want;
  return NEWT_OK;
}

struct Layout {
  size_t idx_bytes;
  std::vector<size_t> ioff, foff;
  size_t n_idx = 0, n_f = 0;
};

Layout layout(const std::vector<RowMove>& mv) {
  Layout L;
  for (const RowMove& m : mv) {
    L.ioff.push_back(L.n_idx);
    L.foff.push_back(L.n_f);
    L.n_idx += m.idx.size();
    L.n_f += m.idx.size() * m.cnt;
  }
  L.idx_bytes = (L.n_idx * sizeof(int) + 255) & ~(size_t)255;
  return L;
}

// A world list that is one run of consecutive indices moves as one strided
// copy straight between the host mirror and the device, with no packing.
bool consecutive(const std::vector<int>& idx) {
  for (size_t j = 1; j < idx.size(); ++j)
    if (idx[j] != idx[0] + (int)j) return false;
  return !idx.empty();
}

cudaError_t copy_run(const RowMove& m, cudaStream_t st, bool to_device) {
  HostGroup& g = *m.g;
  const size_t a = (size_t)m.idx[0], k = m.idx.size();
  float* h = m.ints ? reinterpret_cast<float*>(g.hI.data()) : g.hF.data();
  float* d = m.ints ? reinterpret_cast<float*>(g.dI) : g.dF;
  const size_t rows = m.ints ? g.irows : g.frows;
  if (g.soa()) {  // cnt rows of k consecutive worlds, row pitch cap
    const size_t off = m.lo * g.cap + a, pitch = g.cap * sizeof(float);
    return to_device ? cudaMemcpy2DAsync(d + off, pitch, h + off, pitch, k * sizeof(float), m.cnt,
                                         cudaMemcpyHostToDevice, st)
                     : cudaMemcpy2DAsync(h + off, pitch, d + off, pitch, k * sizeof(float), m.cnt,
                                         cudaMemcpyDeviceToHost, st);
  }
  const size_t off = a * rows + m.lo, pitch = rows * sizeof(float);  // k worlds of cnt values
  return to_device ? cudaMemcpy2DAsync(d + off, pitch, h + off, pitch, m.cnt * sizeof(float), k,
                                       cudaMemcpyHostToDevice, st)
                   : cudaMemcpy2DAsync(h + off, pitch, d + off, pitch, m.cnt * sizeof(float), k,
                                       cudaMemcpyDeviceToHost, st);
}

}  // namespace

int io_scatter(newt_gpu_ctx* ctx, const std::vector<RowMove>& all) {
  std::vector<RowMove> mv;
  for (const RowMove& m : all) {
    if (consecutive(m.idx)) CKW(copy_run(m, ctx->stream, true));
    else mv.push_back(m);
  }
  if (mv.empty()) {
    CKW(cudaStreamSynchronize(ctx->stream));
    return NEWT_OK;
  }
  const Layout L = layout(mv);
  int rc = ensure_staging(ctx, L.n_idx, L.n_f);
  if (rc != NEWT_OK) return rc;
  int* hi = (int*)ctx->io_h;
  float* hf = (float*)((char*)ctx->io_h + L.idx_bytes);
  for (size_t s = 0; s < mv.size(); ++s) {
    const RowMove& m = mv[s];
    const HostGroup& g = *m.g;
    const size_t k = m.idx.size();
    std::copy(m.idx.begin(), m.idx.end(), hi + L.ioff[s]);
    float* out = hf + L.foff[s];
    for (size_t j = 0; j < k; ++j)
      for (size_t r = 0; r < m.cnt; ++r) {
        float v;
        if (m.ints) { const int iv = g.Ic(m.lo + r, m.idx[j]); std::memcpy(&v, &iv, sizeof(v)); }
        else v = g.Fc(m.lo + r, m.idx[j]);
        if (g.soa()) out[r * k + j] = v; else out[j * m.cnt + r] = v;
      }
  }
  CKW(cudaMemcpyAsync(ctx->io_d, ctx->io_h, L.idx_bytes + L.n_f * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  const int* di = (const int*)ctx->io_d;
  const float* df = (const float*)((char*)ctx->io_d + L.idx_bytes);
  for (size_t s = 0; s < mv.size(); ++s) {
    const RowMove& m = mv[s];
    const long total = (long)m.idx.size() * m.cnt;
    if (total == 0) continue;
    rows_scatter<<<grid_for(total), 256, 0, ctx->stream>>>(m.ints ? reinterpret_cast<float*>(m.g->dI) : m.g->dF,
                                                            m.g->soa() ? 1 : 0, m.g->cap,
                                                            (int)(m.ints ? m.g->irows : m.g->frows),
                                                            (int)m.lo, (int)m.cnt, di + L.ioff[s], (int)m.idx.size(),
                                                            df + L.foff[s]);
    ctx->launches++;
  }
  CKW(cudaGetLastError());
  CKW(cudaStreamSynchronize(ctx->stream));  // the pinned staging is reused by the next call
  return NEWT_OK;
}

int io_gather(newt_gpu_ctx* ctx, const std::vector<RowMove>& all) {
  std::vector<RowMove> mv;
  for (const RowMove& m : all) {
    if (consecutive(m.idx)) CKW(copy_run(m, ctx->stream, false));
    else mv.push_back(m);
  }
  if (mv.empty()) {
    CKW(cudaStreamSynchronize(ctx->stream));
    return NEWT_OK;
  }
  const Layout L = layout(mv);
  int rc = ensure_staging(ctx, L.n_idx, L.n_f);
  if (rc != NEWT_OK) return rc;
  int* hi = (int*)ctx->io_h;
  for (size_t s = 0; s < mv.size(); ++s) std::copy(mv[s].idx.begin(), mv[s].idx.end(), hi + L.ioff[s]);
  CKW(cudaMemcpyAsync(ctx->io_d, ctx->io_h, L.n_idx * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  const int* di = (const int*)ctx->io_d;
  float* df = (float*)((char*)ctx->io_d + L.idx_bytes);
  for (size_t s = 0; s < mv.size(); ++s) {
    const RowMove& m = mv[s];
    const long total = (long)m.idx.size() * m.cnt;
    if (total == 0) continue;
    rows_gather<<<grid_for(total), 256, 0, ctx->stream>>>(m.ints ? reinterpret_cast<const float*>(m.g->dI) : m.g->dF,
                                                           m.g->soa() ? 1 : 0, m.g->cap,
                                                           (int)(m.ints ? m.g->irows : m.g->frows),
                                                           (int)m.lo, (int)m.cnt, di + L.ioff[s], (int)m.idx.size(),
                                                           df + L.foff[s]);
    ctx->launches++;
  }
  CKW(cudaGetLastError());
  float* hf = (float*)((char*)ctx->io_h + L.idx_bytes);
  CKW(cudaMemcpyAsync(hf, df, L.n_f * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  CKW(cudaStreamSynchronize(ctx->stream));
  for (size_t s = 0; s < mv.size(); ++s) {
    const RowMove& m = mv[s];
    HostGroup& g = *m.g;
    const size_t k = m.idx.size();
    const float* in = hf + L.foff[s];
    for (size_t j = 0; j < k; ++j)
      for (size_t r = 0; r < m.cnt; ++r) {
        const float v = g.soa() ? in[r * k + j] : in[j * m.cnt + r];
        if (m.ints) std::memcpy(&g.I(m.lo + r, m.idx[j]), &v, sizeof(v));
        else g.F(m.lo + r, m.idx[j]) = v;
      }
  }
  return NEWT_OK;
}

// ---------------------------------------------------------------------------
// state in MuJoCo layout, converted on the device
// ---------------------------------------------------------------------------
// newt_gpu_set_state / newt_gpu_get_state move the caller's MuJoCo-layout
// arrays in one copy each way and convert them here, a warp per world:
// quaternions reordered (wxyz <-> xyzw) and, on the way in, normalised; a
// free root's linear velocity rotated between world and body frame (newt's
// apply_mujoco_qpos/qvel, world.rs:519-623, and its inverse).  A free root's
// and a hinge's MuJoCo offsets equal newt's (7 and 1 coordinates, 6 and 1
// rates), so a link's `topo` offsets index both layouts.
namespace {

struct StateGroup {
  float* F;
  int soa, cap, size;  // tree SoA (row * cap + w) or pile world-major (w * frows + row); bodies or links
  long frows;
  int pos, quat, vel, omg;  // pile rows
  int rq, rqd;              // tree rows
  const int* topo;          // tree: parent, joint, q offset, v offset per link
};
struct StateWorld { int g, w, qoff, voff; };

NEWT_D float& frow(const StateGroup& g, int row, int w) {
  return g.soa ? g.F[(size_t)row * g.cap + w] : g.F[(size_t)w * g.frows + row];
}
NEWT_D Q4 qnorm_or_identity(Q4 q) {  // the host's q_norm: a zero quaternion becomes the identity
  const float n = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
  return n == 0.f ? Q4{0.f, 0.f, 0.f, 1.f} : Q4{q.x / n, q.y / n, q.z / n, q.w / n};
}

__global__ void state_in(const StateGroup* __restrict__ G, const StateWorld* __restrict__ W, int n,
                         const float* __restrict__ qpos, const float* __restrict__ qvel) {
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (t >= n) return;
  const StateWorld sw = W[t];
  const StateGroup g = G[sw.g];
  const float* qp = qpos + sw.qoff;
  const float* qv = qvel + sw.voff;
  for (int i = lane; i < g.size; i += 32) {
    if (!g.soa) {  // free body i
      const float* p = qp + 7 * i;
      const float* v = qv + 6 * i;
      const Q4 q = qnorm_or_identity(Q4{p[4], p[5], p[6], p[3]});
      for (int k = 0; k < 3; ++k) {
        frow(g, g.pos + 3 * i + k, sw.w) = p[k];
        frow(g, g.vel + 3 * i + k, sw.w) = v[k];
        frow(g, g.omg + 3 * i + k, sw.w) = v[3 + k];
      }
      frow(g, g.quat + 4 * i, sw.w) = q.x; frow(g, g.quat + 4 * i + 1, sw.w) = q.y;
      frow(g, g.quat + 4 * i + 2, sw.w) = q.z; frow(g, g.quat + 4 * i + 3, sw.w) = q.w;
      continue;
    }
    const int jt = g.topo[4 * i + 1], qo = g.topo[4 * i + 2], vo = g.topo[4 * i + 3];
    if (jt == NEWT_JOINT_FREE) {  // pos, quat xyzw; omega_body, v_body
      const Q4 q = qnorm_or_identity(Q4{qp[qo + 4], qp[qo + 5], qp[qo + 6], qp[qo + 3]});
      const V3 vb = qrot_inv(q, v3(qv[vo], qv[vo + 1], qv[vo + 2]));
      for (int k = 0; k < 3; ++k) frow(g, g.rq + qo + k, sw.w) = qp[qo + k];
      frow(g, g.rq + qo + 3, sw.w) = q.x; frow(g, g.rq + qo + 4, sw.w) = q.y;
      frow(g, g.rq + qo + 5, sw.w) = q.z; frow(g, g.rq + qo + 6, sw.w) = q.w;
      for (int k = 0; k < 3; ++k) frow(g, g.rqd + vo + k, sw.w) = qv[vo + 3 + k];
      frow(g, g.rqd + vo + 3, sw.w) = vb.x; frow(g, g.rqd + vo + 4, sw.w) = vb.y; frow(g, g.rqd + vo + 5, sw.w) = vb.z;
    } else if (jt == NEWT_JOINT_HINGE || jt == NEWT_JOINT_SLIDE) {
      frow(g, g.rq + qo, sw.w) = qp[qo];
      frow(g, g.rqd + vo, sw.w) = qv[vo];
    }
  }
}

__global__ void state_out(const StateGroup* __restrict__ G, const StateWorld* __restrict__ W, int n,
                          float* __restrict__ qpos, float* __restrict__ qvel) {
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (t >= n) return;
  const StateWorld sw = W[t];
  const StateGroup g = G[sw.g];
  float* qp = qpos + sw.qoff;
  float* qv = qvel + sw.voff;
  for (int i = lane; i < g.size; i += 32) {
    if (!g.soa) {
      float* p = qp + 7 * i;
      float* v = qv + 6 * i;
      for (int k = 0; k < 3; ++k) {
        p[k] = frow(g, g.pos + 3 * i + k, sw.w);
        v[k] = frow(g, g.vel + 3 * i + k, sw.w);
        v[3 + k] = frow(g, g.omg + 3 * i + k, sw.w);
      }
      p[3] = frow(g, g.quat + 4 * i + 3, sw.w); p[4] = frow(g, g.quat + 4 * i, sw.w);
      p[5] = frow(g, g.quat + 4 * i + 1, sw.w); p[6] = frow(g, g.quat + 4 * i + 2, sw.w);
      continue;
    }
    const int jt = g.topo[4 * i + 1], qo = g.topo[4 * i + 2], vo = g.topo[4 * i + 3];
    if (jt == NEWT_JOINT_FREE) {
      const Q4 q{frow(g, g.rq + qo + 3, sw.w), frow(g, g.rq + qo + 4, sw.w), frow(g, g.rq + qo + 5, sw.w),
                 frow(g, g.rq + qo + 6, sw.w)};
      for (int k = 0; k < 3; ++k) qp[qo + k] = frow(g, g.rq + qo + k, sw.w);
      qp[qo + 3] = q.w; qp[qo + 4] = q.x; qp[qo + 5] = q.y; qp[qo + 6] = q.z;
      const V3 vw = qrot(q, v3(frow(g, g.rqd + vo + 3, sw.w), frow(g, g.rqd + vo + 4, sw.w),
                               frow(g, g.rqd + vo + 5, sw.w)));
      qv[vo] = vw.x; qv[vo + 1] = vw.y; qv[vo + 2] = vw.z;
      for (int k = 0; k < 3; ++k) qv[vo + 3 + k] = frow(g, g.rqd + vo + k, sw.w);
    } else if (jt == NEWT_JOINT_HINGE || jt == NEWT_JOINT_SLIDE) {
      qp[qo] = frow(g, g.rq + qo, sw.w);
      qv[vo] = frow(g, g.rqd + vo, sw.w);
    }
  }
}

bool host_pinned(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
  return a.type == cudaMemoryTypeHost;
}

// The call's worlds: per distinct group a StateGroup, per world its entry,
// in the staging's head; returns the offsets of qpos and qvel in the staging.
struct StatePlan { std::vector<StateGroup> groups; std::vector<StateWorld> worlds; long nq = 0, nv = 0; };
StatePlan plan_state(newt_gpu_ctx* ctx, const int32_t* slots, int n) {
  StatePlan P;
  std::vector<int> gslot(ctx->groups.size(), -1);
  for (int i = 0; i < n; ++i) {
    const SlotRef& r = ctx->slots[slots[i]];
    const HostModel& m = ctx->models[r.model];
    if (gslot[r.group] < 0) {
      const HostGroup& hg = *ctx->groups[r.group];
      StateGroup g{};
      g.F = hg.dF;
      g.soa = hg.soa() ? 1 : 0;
      g.cap = hg.cap;
      g.size = hg.size;
      g.frows = (long)hg.frows;
      g.pos = hg.lay.pos; g.quat = hg.lay.quat; g.vel = hg.lay.vel; g.omg = hg.lay.omg;
      g.rq = hg.r_q; g.rqd = hg.r_qd;
      g.topo = hg.dtopo;
      gslot[r.group] = (int)P.groups.size();
      P.groups.push_back(g);
    }
    P.worlds.push_back(StateWorld{gslot[r.group], r.index, (int)P.nq, (int)P.nv});
    P.nq += m.nq;
    P.nv += m.nv;
  }
  return P;
}

size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

int io_state_in(newt_gpu_ctx* ctx, const int32_t* slots, int n, const float* qpos, const float* qvel) {
  if (n <= 0) return NEWT_OK;
  const StatePlan P = plan_state(ctx, slots, n);
  const size_t gb = up256(P.groups.size() * sizeof(StateGroup)), wb = up256(P.worlds.size() * sizeof(StateWorld));
  const size_t qb = up256(P.nq * sizeof(float)), vb = P.nv * sizeof(float);
  int rc = ensure_staging(ctx, 0, (gb + wb + qb + vb) / sizeof(float) + 1);
  if (rc != NEWT_OK) return rc;
  char* h = (char*)ctx->io_h;
  char* d = (char*)ctx->io_d;
  std::memcpy(h, P.groups.data(), P.groups.size() * sizeof(StateGroup));
  std::memcpy(h + gb, P.worlds.data(), P.worlds.size() * sizeof(StateWorld));
  CKW(cudaMemcpyAsync(d, h, gb + wb, cudaMemcpyHostToDevice, ctx->stream));
  // page-locked caller arrays go by DMA as they are; others through the staging
  const bool pinned = host_pinned(qpos) && host_pinned(qvel);
  if (!pinned) {
    std::memcpy(h + gb + wb, qpos, P.nq * sizeof(float));
    std::memcpy(h + gb + wb + qb, qvel, vb);
  }
  CKW(cudaMemcpyAsync(d + gb + wb, pinned ? (const void*)qpos : (const void*)(h + gb + wb), P.nq * sizeof(float),
                      cudaMemcpyHostToDevice, ctx->stream));
  CKW(cudaMemcpyAsync(d + gb + wb + qb, pinned ? (const void*)qvel : (const void*)(h + gb + wb + qb), vb,
                      cudaMemcpyHostToDevice, ctx->stream));
  const long threads = 32L * n;
  state_in<<<(int)((threads + 255) / 256), 256, 0, ctx->stream>>>((const StateGroup*)d, (const StateWorld*)(d + gb), n,
                                                                   (const float*)(d + gb + wb),
                                                                   (const float*)(d + gb + wb + qb));
  ctx->launches++;
  CKW(cudaGetLastError());
  CKW(cudaStreamSynchronize(ctx->stream));  // the caller's arrays and the staging are free again
  return NEWT_OK;
}

int io_state_out(newt_gpu_ctx* ctx, const int32_t* slots, int n, float* qpos, float* qvel) {
  if (n <= 0) return NEWT_OK;
  const StatePlan P = plan_state(ctx, slots, n);
  const size_t gb = up256(P.groups.size() * sizeof(StateGroup)), wb = up256(P.worlds.size() * sizeof(StateWorld));
  const size_t qb = up256(P.nq * sizeof(float)), vb = P.nv * sizeof(float);
  int rc = ensure_staging(ctx, 0, (gb + wb + qb + vb) / sizeof(float) + 1);
  if (rc != NEWT_OK) return rc;
  char* h = (char*)ctx->io_h;
  char* d = (char*)ctx->io_d;
  std::memcpy(h, P.groups.data(), P.groups.size() * sizeof(StateGroup));
  std::memcpy(h + gb, P.worlds.data(), P.worlds.size() * sizeof(StateWorld));
  CKW(cudaMemcpyAsync(d, h, gb + wb, cudaMemcpyHostToDevice, ctx->stream));
  const long threads = 32L * n;
  state_out<<<(int)((threads + 255) / 256), 256, 0, ctx->stream>>>((const StateGroup*)d, (const StateWorld*)(d + gb),
                                                                    n, (float*)(d + gb + wb), (float*)(d + gb + wb + qb));
  ctx->launches++;
  CKW(cudaGetLastError());
  const bool pinned = host_pinned(qpos) && host_pinned(qvel);
  CKW(cudaMemcpyAsync(pinned ? (void*)qpos : (void*)(h + gb + wb), d + gb + wb, P.nq * sizeof(float),
                      cudaMemcpyDeviceToHost, ctx->stream));
  CKW(cudaMemcpyAsync(pinned ? (void*)qvel : (void*)(h + gb + wb + qb), d + gb + wb + qb, vb, cudaMemcpyDeviceToHost,
                      ctx->stream));
  CKW(cudaStreamSynchronize(ctx->stream));
  if (!pinned) {
    std::memcpy(qpos, h + gb + wb, P.nq * sizeof(float));
    std::memcpy(qvel, h + gb + wb + qb, vb);
  }
  return NEWT_OK;
}

// Up to 1024 live flags cleared by one launch with the pointers passed by
// value (8 KB of parameters): nothing to stage, so the call returns at once.
struct HoldList {
  int n;
  int* f[1024];
};
__global__ void flags_hold(HoldList L) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < L.n) *L.f[i] = 0;
}

int io_hold_flags(newt_gpu_ctx* ctx, const std::vector<int*>& flags) {
  for (size_t a = 0; a < flags.size(); a += 1024) {
    HoldList L;
    L.n = (int)std::min<size_t>(1024, flags.size() - a);
    for (int i = 0; i < L.n; ++i) L.f[i] = flags[a + i];
    flags_hold<<<(L.n + 255) / 256, 256, 0, ctx->stream>>>(L);
    ctx->launches++;
    CKW(cudaGetLastError());
  }
  return NEWT_OK;
}

int io_clear_flags(newt_gpu_ctx* ctx, const std::vector<int*>& flags) {
  if (flags.empty()) return NEWT_OK;
  int rc = ensure_staging(ctx, 0, 2 * flags.size());  // one pointer = two floats' room
  if (rc != NEWT_OK) return rc;
  std::copy(flags.begin(), flags.end(), (int**)ctx->io_h);
  CKW(cudaMemcpyAsync(ctx->io_d, ctx->io_h, flags.size() * sizeof(int*), cudaMemcpyHostToDevice, ctx->stream));
  flags_clear<<<grid_for((long)flags.size()), 256, 0, ctx->stream>>>((int* const*)ctx->io_d, (int)flags.size());
  ctx->launches++;
  CKW(cudaGetLastError());
  CKW(cudaStreamSynchronize(ctx->stream));
  return NEWT_OK;
}
