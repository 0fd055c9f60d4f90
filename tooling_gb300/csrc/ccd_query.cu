// newt_gpu_convex_contacts: the device GJK/EPA routine (ccd.cuh) as a batch
// query over pairs of primitive shapes.  One block per pair; its thread runs
// GJK and, for overlapping pairs, EPA over a polytope in the block's shared
// memory (newt's caps: 128 vertices, 512 faces, 1024 horizon edges).
#include <string>

#include "../../include/newt_gpu.h"
#include "ccd.cuh"
#include "runtime.h"

namespace {

__global__ void __launch_bounds__(1) ccd_query_kernel(const newt_convex_query* q, int n, float face_eps,
                                                      newt_convex_result* out) {
  __shared__ ccd::Polytope P;
  const int i = blockIdx.x;
  if (i >= n) return;
  const newt_convex_query& Q = q[i];
  auto shape = [](int kind, const float* pose, const float* size) {
    return ccd::Shape{kind, v3(pose[0], pose[1], pose[2]), Q4{pose[3], pose[4], pose[5], pose[6]},
                      v3(size[0], size[1], size[2])};
  };
  const ccd::Result r = ccd::convex_contact(shape(Q.shape_a, Q.pose_a, Q.size_a), shape(Q.shape_b, Q.pose_b, Q.size_b),
                                            Q.margin, face_eps, &P);
  newt_convex_result& o = out[i];
  o.hit = r.hit;
  o.path = r.path;
  const V3 vs[4] = {r.pos, r.n, r.wa, r.wb};
  float* dst[4] = {o.pos, o.normal, o.witness_a, o.witness_b};
  for (int k = 0; k < 4; ++k) { dst[k][0] = vs[k].x; dst[k][1] = vs[k].y; dst[k][2] = vs[k].z; }
  o.penetration = r.pen;
}

bool primitive(int k) { return k == NEWT_SHAPE_SPHERE || k == NEWT_SHAPE_BOX || k == NEWT_SHAPE_CAPSULE; }

}  // namespace

extern "C" NEWT_API int newt_gpu_convex_contacts(newt_gpu_ctx* ctx, const newt_convex_query* queries, int32_t n,
                                                 float face_eps, newt_convex_result* out) {
  if (!ctx || n < 0 || (n > 0 && (!queries || !out))) return NEWT_E_INVALID;
  if (n == 0) return NEWT_OK;
  for (int i = 0; i < n; ++i)
    if (!primitive(queries[i].shape_a) || !primitive(queries[i].shape_b)) {
      ctx->err = "newt_gpu_convex_contacts: pair " + std::to_string(i) + " is not a sphere, box or capsule pair";
      return NEWT_E_UNSUPPORTED_PAIR;
    }
  cudaError_t e = cudaSetDevice(ctx->device);
  newt_convex_query* dq = nullptr;
  newt_convex_result* dr = nullptr;
  auto fail = [&](const char* what) {
    ctx->err = std::string("newt_gpu_convex_contacts: ") + what + ": " + cudaGetErrorString(e);
    if (dq) cudaFree(dq);
    if (dr) cudaFree(dr);
    return NEWT_E_CUDA;
  };
  if (e != cudaSuccess) return fail("cudaSetDevice");
  if ((e = cudaMalloc(&dq, sizeof(newt_convex_query) * (size_t)n)) != cudaSuccess) return fail("cudaMalloc");
  if ((e = cudaMalloc(&dr, sizeof(newt_convex_result) * (size_t)n)) != cudaSuccess) return fail("cudaMalloc");
  if ((e = cudaMemcpyAsync(dq, queries, sizeof(newt_convex_query) * (size_t)n, cudaMemcpyHostToDevice, ctx->stream)) !=
      cudaSuccess)
    return fail("upload");
  ccd_query_kernel<<<n, 1, 0, ctx->stream>>>(dq, n, face_eps > 0.f ? face_eps : 1.0e-4f, dr);
  ctx->launches += 1;
  if ((e = cudaGetLastError()) != cudaSuccess) return fail("launch");
  if ((e = cudaMemcpyAsync(out, dr, sizeof(newt_convex_result) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream)) !=
      cudaSuccess)
    return fail("read-back");
  if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return fail("sync");
  cudaFree(dq);
  cudaFree(dr);
  return NEWT_OK;
}
