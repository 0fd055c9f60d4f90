// World-persistent free-body step: the batched form's pile kernel.
//
// One warp owns one pile world at a time and runs the whole call's horizon
// for it.  Per env-step, inside the warp and the world's scratch record:
//   collide        AABBs, sorted sweep, ordered pair list and narrowphase
//                  (pile_collide.cuh, unchanged);
//   assemble       the active contacts in contact order and, per contact, a
//                  compact row record (below);
//   rounds         contact k goes to the first round after the rounds of
//                  the last earlier contacts on its dynamic bodies that still
//                  has one of the warp's eight four-lane groups free;
//   sweeps         PGS: rounds in order, the contacts of one round (they touch
//                  disjoint bodies) on the warp's four-lane groups;
//   integrate      semi-implicit Euler or RK4 (pile_solver.cuh, unchanged).
// The state stays in the scratch record between env-steps and goes back to
// the world record once, after the last one.
//
// Scheduling.  One block of GANG warps runs per SM and takes GANG worlds at
// a time from a device queue; the gang's warps move through each phase of an
// env-step together (a block barrier after collide and assembly, after the
// sweeps and after integration), so every warp on the SM executes the same
// code region and the instruction caches hold it (with warps spread over the
// whole kernel, instruction fetch was the dominant stall).  The queue is
// sorted by each world's measured cost from the previous call, most costly
// first (pile_k_queue_sort, a one-block counting sort at the head of the
// call), so the worlds of a gang cost about the same (short barrier waits)
// and the last gangs to start are the cheapest (a short tail).  No world ever
// waits on another world's env-step.
//
// Restates, for FP32 on sm_103a:
//   newt/src/world.rs:1459-1537   World::step phase order (Euler branch)
//   newt/src/solver.rs:703-1257   solve_free_bodies_diag_mode, PGS branch: rows,
//                                 regularisation, bias (:752-1061) and the
//                                 sweeps (:1085-1200)
//   newt/src/solver.rs:1448-1518  pgs_step_non_negative, pgs_step_pyramidal_pair
//   newt/src/solver.rs:1892-2036  row_body_diagonal, row_residual,
//                                 apply_impulse_delta
//   newt/src/solver.rs:3401-3429  pyramidal facet rows n +- mu t
//   newt/src/world.rs:3104-3112   tangent_basis
//
// Gauss-Seidel order.  newt sweeps each island's contacts in contact order.
// A contact update reads the velocity accumulators of its (at most two)
// dynamic bodies, which only earlier contacts on the same bodies have
// changed; running the rounds in order therefore reproduces the serial
// sweep of every island exactly (islands never share a body).
//
// Row record.  A pyramidal contact has four facet rows r = n + s_r mu t_q(r)
// (s = +, -, +, -; q = 1, 1, 2, 2).  The record keeps the Jacobian of the
// normal and of both tangents and their M^-1 J^T per lane triple (side a
// linear, side a angular, side b linear, side b angular; zero for a static
// side, so the four lanes of a contact run one code path), the exact
// row-space block A_rs = J_r M^-1 J_s^T, newt's row diagonals
// (row_body_diagonal plus the regulariser), the biases and the pair
// determinants.  One contact update
// takes three four-lane dot products (J_n.v, J_t1.v, J_t2.v) for the four
// facet residuals, runs newt's row steps in registers -- the non-negative
// step on row 0, then the pyramidal pairs (0,1) and (2,3) -- advancing the
// residuals by A after every step (what re-reading J_r . v gives, up to
// rounding), and applies the summed impulse changes to the bodies once.
#include <algorithm>

#include "../../include/newt_gpu.h"
#include "pile_solver.cuh"

using namespace pile;

namespace {

constexpr unsigned FULL = 0xffffffffu;
// gang sizes (warps per block, one block per SM): 32 warps run at 64
// registers and 24 at 80 (both spilling), 16 at 128 (spilling in the
// sweeps), 12 at 168 and 8 at 182 without
constexpr int F_MAXC = 512;   // the largest contact capacity of a pile world
constexpr int N_BUCKET = 256; // cost classes of the queue sort

// compact row record (floats, 16-byte aligned)
enum {
  R_TRI = 0,    // per lane triple l (0 side a linear, 1 side a angular, 2 side b
                // linear, 3 side b angular), 20 floats at R_TRI + 20 l: J of n,
                // t1, t2, then M^-1 J^T of each, 2 pad (zero for a static side)
  R_A = 80,     // A00 A01 A02 A03 | A11 A12 A13 A22 | A23 A33 reg mu
  R_B = 92,     // bias of rows 0..3
  R_DG = 96,    // newt's row diagonals (A_rr by row_body_diagonal, plus reg)
  R_IDG = 100,  // their inverses
  R_MISC = 104, // 1/det of pair (0,1), of pair (2,3) (0 when det <= 0), body slot a, body slot b (int bits)
  R_IMP = 108,  // impulses of rows 0..3
  FR = 112
};
static_assert(FR % 4 == 0, "records are read as float4");
static_assert(FR <= SC, "the compact record fits the solver record's slot");

NEWT_D float4 ld4g(const float* p) { return *reinterpret_cast<const float4*>(p); }
NEWT_D void st4g(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }

// ---------------------------------------------------------------------------
// assemble: active contacts in contact order and their row records
// (newt/src/solver.rs:752-1061)
// ---------------------------------------------------------------------------
NEWT_D int fused_assemble(const WsLay& L, float* wf, int* wi, int lane, float (*acc)[6]) {
  const int nb = L.nb, nc = wi[L.misc + 1];
  const float dt = wf[L.dtg];
  const V3 grav = v3(wf[L.dtg + 1], wf[L.dtg + 2], wf[L.dtg + 3]);
  const float* soft = wf + L.soft;
  for (int b = lane; b < nb; b += 32) {
    M3 R = quat_mat(ld4(wf + L.quat + 4 * b));
    M3 RT{{{R.m[0][0], R.m[1][0], R.m[2][0]}, {R.m[0][1], R.m[1][1], R.m[2][1]}, {R.m[0][2], R.m[1][2], R.m[2][2]}}};
    S3 iw = sym_congr(RT, lds(wf + L.iinvb + 6 * b));
    float* o = wf + L.iinvw + 6 * b;
    o[0] = iw.xx; o[1] = iw.yy; o[2] = iw.zz; o[3] = iw.xy; o[4] = iw.xz; o[5] = iw.yz;
  }
  for (int i = lane; i < 6 * (nb + 1); i += 32) (&acc[0][0])[i] = 0.f;
  // active contacts (solver.rs:762-769): a dynamic side and penetration beyond the gap (gap = 0)
  int* sccon = wi + L.sccon;
  const unsigned lt = (1u << lane) - 1u;
  int nact = 0;
  for (int c0 = 0; c0 < nc; c0 += 32) {
    const int c = c0 + lane;
    bool act = false;
    if (c < nc) {
      float* cf = wf + L.con + CF * c;
      const int* cc = wi + L.ci + CI * c;
      act = (cc[2] < nb || cc[3] < nb) && cf[C_PEN] > 0.f;
      cf[C_ACT] = act ? 1.f : 0.f;
      for (int k = 0; k < 4; ++k) cf[C_IMP + k] = 0.f;
    }
    const unsigned m = __ballot_sync(FULL, act);
    if (act) sccon[nact + __popc(m & lt)] = c;
    nact += __popc(m);
  }
  __syncwarp();
  float tc = soft[0], dr = soft[1];
  const bool direct = tc < 0.f;
  if (!direct && tc < 2.f * dt) tc = 2.f * dt;  // safe_solref (solver.rs:331-338)
  const float dmax = fminf(fmaxf(soft[3], 1.0e-4f), 0.9999f);
  float b_, k0;
  for (int k = lane; k < nact; k += 32) {
    const int c = sccon[k];
    const float* cf = wf + L.con + CF * c;
    const int* cc = wi + L.ci + CI * c;
    float* rec = wf + L.sc + FR * k;
    const int ea = cc[2], eb = cc[3];
    const bool da = ea < nb, db = eb < nb;
    const float pen = cf[C_PEN], mu = cf[C_MU];
    const V3 n = ld3(cf + C_N), pos = ld3(cf + C_POS);
    V3 ref = fabsf(n.z) < 0.9f ? v3(0.f, 0.f, 1.f) : v3(1.f, 0.f, 0.f);
    V3 t1 = cross(ref, n);
    const float tl = sqrtf(len2(t1));
    t1 = tl == 0.f ? v3(0.f, 0.f, 0.f) : t1 * (1.f / tl);
    const V3 t2 = cross(n, t1);
    const V3 z = v3(0.f, 0.f, 0.f);
    const V3 arma = da ? pos - ld3(wf + L.pos + 3 * ea) : z;
    const V3 armb = db ? pos - ld3(wf + L.pos + 3 * eb) : z;
    const float ima = da ? 1.f / wf[L.mass + ea] : 0.f, imb = db ? 1.f / wf[L.mass + eb] : 0.f;
    const S3 Ia = da ? lds(wf + L.iinvw + 6 * ea) : S3{0, 0, 0, 0, 0, 0};
    const S3 Ib = db ? lds(wf + L.iinvw + 6 * eb) : S3{0, 0, 0, 0, 0, 0};
    const V3 ds[3] = {n, t1, t2};
    V3 ja[3], jb[3];
    for (int q = 0; q < 3; ++q) {
      ja[q] = da ? cross(arma, ds[q]) : z;
      jb[q] = db ? -cross(armb, ds[q]) : z;
    }
    // the four lane triples: J of n, t1, t2, then M^-1 J^T of each
    for (int q = 0; q < 3; ++q) {
      const V3 la = da ? ds[q] : z, lb = db ? -ds[q] : z;
      st3(rec + R_TRI + 3 * q, la);      st3(rec + R_TRI + 9 + 3 * q, la * ima);
      st3(rec + R_TRI + 20 + 3 * q, ja[q]); st3(rec + R_TRI + 29 + 3 * q, smv(Ia, ja[q]));
      st3(rec + R_TRI + 40 + 3 * q, lb);  st3(rec + R_TRI + 49 + 3 * q, lb * imb);
      st3(rec + R_TRI + 60 + 3 * q, jb[q]); st3(rec + R_TRI + 69 + 3 * q, smv(Ib, jb[q]));
    }
    for (int t = 0; t < 4; ++t) rec[R_TRI + 20 * t + 18] = rec[R_TRI + 20 * t + 19] = 0.f;
    // facet rows: side Jacobians as in newt's row assembly
    J6 Ra[4], Rb[4];
    float diag[4];
    const float d = impedance(-pen, soft);
    const float tran = ima + imb;
    const float reg = d > 0.f ? 2.f * mu * mu * ((1.f - d) / d * (tran * (1.f + mu * mu))) : 0.f;
    if (direct) { b_ = -dr / dmax; k0 = -soft[0] / (dmax * dmax); }
    else { b_ = 2.f / (dmax * tc); k0 = d / (dmax * dmax * tc * tc * dr * dr); }
    V3 va = z, vb = z;
    if (da) va = ld3(wf + L.vel + 3 * ea) + cross(qrot(ld4(wf + L.quat + 4 * ea), ld3(wf + L.omg + 3 * ea)), arma);
    if (db) vb = ld3(wf + L.vel + 3 * eb) + cross(qrot(ld4(wf + L.quat + 4 * eb), ld3(wf + L.omg + 3 * eb)), armb);
    for (int r = 0; r < 4; ++r) {
      const int q = r < 2 ? 1 : 2;
      const float s = (r & 1) ? -mu : mu;
      const V3 dir = n + ds[q] * s;
      Ra[r] = J6{dir, ja[0] + ja[q] * s};
      Rb[r] = J6{-dir, jb[0] + jb[q] * s};
      float aii = 0.f, dvf = 0.f;
      if (da) { aii += dot(Ra[r].a, smv(Ia, Ra[r].a)) + ima; dvf += dot(grav * dt, dir); }
      if (db) { aii += dot(Rb[r].a, smv(Ib, Rb[r].a)) + imb; dvf -= dot(grav * dt, dir); }
      diag[r] = aii + reg;
      const float vcur = dot(va - vb, dir);
      const float aref = -b_ * vcur - k0 * (-pen);
      rec[R_B + r] = dvf - aref * dt;
      rec[R_DG + r] = diag[r];
      rec[R_IDG + r] = 1.f / diag[r];
      rec[R_IMP + r] = 0.f;
    }
    // exact row-space block A_rs = J_r M^-1 J_s^T
    auto arow = [&](int r, int s) {
      float h = 0.f;
      if (da) h += dot(Ra[r].l, Ra[s].l) * ima + dot(Ra[r].a, smv(Ia, Ra[s].a));
      if (db) h += dot(Rb[r].l, Rb[s].l) * imb + dot(Rb[r].a, smv(Ib, Rb[s].a));
      return h;
    };
    const float a01 = arow(0, 1), a23 = arow(2, 3);
    rec[R_A + 0] = arow(0, 0); rec[R_A + 1] = a01; rec[R_A + 2] = arow(0, 2); rec[R_A + 3] = arow(0, 3);
    rec[R_A + 4] = arow(1, 1); rec[R_A + 5] = arow(1, 2); rec[R_A + 6] = arow(1, 3); rec[R_A + 7] = arow(2, 2);
    rec[R_A + 8] = a23; rec[R_A + 9] = arow(3, 3); rec[R_A + 10] = reg; rec[R_A + 11] = mu;
    // pyramidal pair blocks (solver.rs:1037-1061)
    const float det0 = diag[0] * diag[1] - a01 * a01, det1 = diag[2] * diag[3] - a23 * a23;
    rec[R_MISC + 0] = det0 > 0.f ? 1.f / det0 : 0.f;
    rec[R_MISC + 1] = det1 > 0.f ? 1.f / det1 : 0.f;
    rec[R_MISC + 2] = __int_as_float(da ? ea : nb);
    rec[R_MISC + 3] = __int_as_float(db ? eb : nb);
  }
  __syncwarp();
  return nact;
}

// ---------------------------------------------------------------------------
// levels: lane 0 assigns each record its round (at most `cap` records, on
// disjoint bodies: the four-lane groups the world has, eight on a whole
// warp, four on a half) and counting-sorts the records by round (sweep
// order inside a round); `loff` gets the round starts and the end.
// Returns the round count.
// ---------------------------------------------------------------------------
NEWT_D int fused_levels(const WsLay& L, const float* wf, int nact, int lane, short* last, short* lev, short* perm,
                        short* loff, int cap) {
  int nlev = 0;
  for (int v = lane; v <= nact; v += 32) loff[v] = 0;  // contacts per round
  __syncwarp();
  if (lane == 0) {
    // List scheduling with `cap` contacts per round: contact k takes the first round after the last rounds of its
    // bodies that still has a free group.  Every body still sees its
    // contacts in contact order and no round holds two contacts of one
    // body, so the sweep equals the serial one; islands fill each other's
    // rounds instead of spilling a crowded level into a second round.
    const int nb = L.nb;
    for (int b = 0; b <= nb; ++b) last[b] = 0;
    for (int k = 0; k < nact; ++k) {
      const float* rec = wf + L.sc + FR * k;
      const int ba = __float_as_int(rec[R_MISC + 2]), bb = __float_as_int(rec[R_MISC + 3]);
      int lv = 1 + max(ba < nb ? (int)last[ba] : 0, bb < nb ? (int)last[bb] : 0);
      while (loff[lv] >= cap) ++lv;  // lv <= k + 1 <= nact: rounds 1..k hold at most k contacts
      loff[lv]++;
      if (ba < nb) last[ba] = (short)lv;
      if (bb < nb) last[bb] = (short)lv;
      lev[k] = (short)lv;
      nlev = max(nlev, lv);
    }
    int run = 0;
    for (int v = 1; v <= nlev; ++v) { const int c = loff[v]; loff[v - 1] = (short)run; run += c; }
    loff[nlev] = (short)run;
    for (int k = 0; k < nact; ++k) perm[loff[lev[k] - 1]++] = (short)k;
    for (int v = nlev; v > 0; --v) loff[v] = loff[v - 1];  // back to level starts
    loff[0] = 0;
  }
  nlev = __shfl_sync(FULL, nlev, 0);
  __syncwarp();
  return nlev;
}

// newt's pyramidal pair step (RowStep::pair, solver.rs:1476-1518) with its
// four cases chosen by selects rather than branches (the eight contacts of a
// round take different cases) and the one-row fallbacks' division by the row
// diagonal done as a product with its stored inverse.
NEWT_D void pair_select(float ii, float ij, float ri, float rj, float h00, float h11, float h01, float idet,
                        float i00, float i11, float* ni, float* nj) {
  const float ui = ii + (-ri * h11 + h01 * rj) * idet;
  const float uj = ij + (h01 * ri - h00 * rj) * idet;
  const float si = fmaxf(ii - ri * i00, 0.f), sj = fmaxf(ij - rj * i11, 0.f);
  const bool pi = ui >= 0.f, pj = uj >= 0.f;
  *ni = pi ? (pj ? ui : si) : 0.f;  // both >= 0: the pair; one < 0: it is 0 and the other steps alone
  *nj = pj ? (pi ? uj : sj) : 0.f;
}

// ---------------------------------------------------------------------------
// one contact update on the calling four-lane group (lane l of the group
// holds triple l: side a linear, side a angular, side b linear, side b
// angular); newt/src/solver.rs:1085-1200, 1448-1518
// ---------------------------------------------------------------------------
NEWT_D void fused_contact(float* rec, int l, unsigned gm, int nb, float (*acc)[6]) {
  const int side = l >> 1, part = l & 1;
  const float4 s0 = ld4g(rec + R_A), s1 = ld4g(rec + R_A + 4), s2 = ld4g(rec + R_A + 8);
  const float4 bs = ld4g(rec + R_B), dg = ld4g(rec + R_DG), ig = ld4g(rec + R_IDG), ms = ld4g(rec + R_MISC);
  const float4 f4 = ld4g(rec + R_IMP);
  const int body = __float_as_int(side ? ms.w : ms.z);
  const float* blk = rec + R_TRI + 20 * l;
  const float4 a0 = ld4g(blk), a1 = ld4g(blk + 4), a2 = ld4g(blk + 8), a3 = ld4g(blk + 12), a4 = ld4g(blk + 16);
  const float J[3][3] = {{a0.x, a0.y, a0.z}, {a0.w, a1.x, a1.y}, {a1.z, a1.w, a2.x}};
  const float W[3][3] = {{a2.y, a2.z, a2.w}, {a3.x, a3.y, a3.z}, {a3.w, a4.x, a4.y}};
  float a[3];
#pragma unroll
  for (int e = 0; e < 3; ++e) a[e] = acc[body][3 * part + e];
  float dn = (J[0][0] * a[0] + J[0][1] * a[1]) + J[0][2] * a[2];
  float d1 = (J[1][0] * a[0] + J[1][1] * a[1]) + J[1][2] * a[2];
  float d2 = (J[2][0] * a[0] + J[2][1] * a[1]) + J[2][2] * a[2];
  dn += __shfl_xor_sync(gm, dn, 1);
  d1 += __shfl_xor_sync(gm, d1, 1);
  d2 += __shfl_xor_sync(gm, d2, 1);
  dn += __shfl_xor_sync(gm, dn, 2);
  d1 += __shfl_xor_sync(gm, d1, 2);
  d2 += __shfl_xor_sync(gm, d2, 2);
  const float mu = s2.w, reg = s2.z;
  // symmetric 4x4 row block
  const float A[4][4] = {{s0.x, s0.y, s0.z, s0.w}, {s0.y, s1.x, s1.y, s1.z}, {s0.z, s1.y, s1.w, s2.x},
                         {s0.w, s1.z, s2.x, s2.y}};
  const float b[4] = {bs.x, bs.y, bs.z, bs.w}, diag[4] = {dg.x, dg.y, dg.z, dg.w}, idg[4] = {ig.x, ig.y, ig.z, ig.w};
  const float idet[2] = {ms.x, ms.y};
  float d[4] = {dn + mu * d1, dn - mu * d1, dn + mu * d2, dn - mu * d2};
  const float f0[4] = {f4.x, f4.y, f4.z, f4.w};
  float f[4] = {f4.x, f4.y, f4.z, f4.w};
  auto advance = [&](int s, float delta) {
#pragma unroll
    for (int r = 0; r < 4; ++r) d[r] += A[r][s] * delta;
  };
  auto single = [&](int r) {
    const float res = d[r] + (reg * f[r] + b[r]);
    const float nf = RowStep::nonneg(f[r], res, idg[r]);
    const float delta = nf - f[r];
    f[r] = nf;
    advance(r, delta);
  };
  single(0);
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    const int i = 2 * p, j = i + 1;
    if (idet[p] == 0.f) {  // det <= 0: two half-line steps
      single(i);
      single(j);
      continue;
    }
    const float ri = d[i] + (reg * f[i] + b[i]);
    const float rj = d[j] + (reg * f[j] + b[j]);
    float ni, nj;
    pair_select(f[i], f[j], ri, rj, diag[i], diag[j], A[i][j], idet[p], idg[i], idg[j], &ni, &nj);
    const float di = ni - f[i], dj = nj - f[j];
    f[i] = ni;
    f[j] = nj;
    advance(i, di);
    advance(j, dj);
  }
  // velocity change: sum_r W_r df_r = W_n sum df + mu W_t1 (df0 - df1) + mu W_t2 (df2 - df3)
  const float e0 = f[0] - f0[0], e1 = f[1] - f0[1], e2 = f[2] - f0[2], e3 = f[3] - f0[3];
  const float Fn = (e0 + e1) + (e2 + e3), F1 = mu * (e0 - e1), F2 = mu * (e2 - e3);
  if (body < nb) {
#pragma unroll
    for (int e = 0; e < 3; ++e) acc[body][3 * part + e] = a[e] + (W[0][e] * Fn + W[1][e] * F1 + W[2][e] * F2);
  }
  if (l == 0) st4g(rec + R_IMP, make_float4(f[0], f[1], f[2], f[3]));
}

}  // namespace

// ---------------------------------------------------------------------------
// the queue: worlds sorted by last call's cost, most costly first
// ---------------------------------------------------------------------------
// Counting sort by cost class (4 classes per octave of cost); the order
// inside a class is unspecified, which changes which warp steps a world and
// never what it computes.  One block.
__global__ void __launch_bounds__(1024) pile_k_queue_sort(const unsigned* __restrict__ cost, int n,
                                                          int* __restrict__ queue) {
  __shared__ int hist[N_BUCKET];
  auto bucket = [](unsigned c) {
    const float l = log2f((float)c + 1.f) * 4.f;
    const int b = (int)l;
    return b < N_BUCKET ? b : N_BUCKET - 1;
  };
  for (int b = threadIdx.x; b < N_BUCKET; b += blockDim.x) hist[b] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) atomicAdd(&hist[bucket(cost[i])], 1);
  __syncthreads();
  if (threadIdx.x == 0) {  // exclusive starts, most costly class first
    int run = 0;
    for (int b = N_BUCKET - 1; b >= 0; --b) { const int c = hist[b]; hist[b] = run; run += c; }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) queue[atomicAdd(&hist[bucket(cost[i])], 1)] = i;
}

// Shared memory of one warp: velocity accumulators (nb + 1 bodies, the last
// a static side's zero), the round schedule (last round per body, round per
// record, records by round, round starts), each part 16-byte aligned.
struct WarpSmem {
  int acc, last, lev, perm, loff, bytes;
};
NEWT_HD int up16(int b) { return (b + 15) / 16 * 16; }
NEWT_HD WarpSmem warp_smem(int nbm, int cm) {
  WarpSmem w;
  int o = 0;
  w.acc = o; o += up16((nbm + 1) * 6 * 4);
  w.last = o; o += up16((nbm + 1) * 2);
  w.lev = o; o += up16(cm * 2);
  w.perm = o; o += up16(cm * 2);
  w.loff = o; o += up16((cm + 1) * 2);
  w.bytes = o;
  return w;
}

// ---------------------------------------------------------------------------
// the phases of one env-step around the sweeps, out of line: each rebuilds
// the world's scratch layout itself, so the sweep loop keeps only a few
// registers live across them
// ---------------------------------------------------------------------------
// collide, assemble and levels; returns (active contacts, levels) and ORs
// the contact-overflow flag into *overflow
__device__ __noinline__ int2 fused_prepare(const PileGroupDev* g, int w, int lane, float (*acc)[6], short* last,
                                           short* lev, short* perm, short* loff, int* overflow, int cap) {
  const WsLay L = ws_layout(g->nb, g->np, g->maxc);
  float* wf = g->scr + (size_t)w * g->sstride;
  int* wi = reinterpret_cast<int*>(wf + L.nf);
  collide(L, wf, wi, lane);
  *overflow |= wi[L.misc + 2];
  const int nact = min(fused_assemble(L, wf, wi, lane, acc), F_MAXC);
  const int nlev = fused_levels(L, wf, nact, lane, last, lev, perm, loff, cap);
  return make_int2(nact, nlev);
}

// the sweeps' velocity changes to the integrator, the impulses of the last
// env-step back to the contact records (the diagnostics surface), then the
// integration; returns whether a body went non-finite
__device__ __noinline__ bool fused_finish(const PileGroupDev* g, int w, int lane, float (*acc)[6], int nact,
                                          bool last_step, bool rk4) {
  const WsLay L = ws_layout(g->nb, g->np, g->maxc);
  float* wf = g->scr + (size_t)w * g->sstride;
  const int* wi = reinterpret_cast<const int*>(wf + L.nf);
  for (int b = lane; b < L.nb; b += 32) {
    st3(wf + L.dv + 3 * b, v3(acc[b][0], acc[b][1], acc[b][2]));
    st3(wf + L.dw + 3 * b, v3(acc[b][3], acc[b][4], acc[b][5]));
  }
  if (last_step)
    for (int k = lane; k < nact; k += 32) {
      const float* rec = wf + L.sc + FR * k;
      float* cimp = wf + L.con + CF * wi[L.sccon + k] + C_IMP;
      for (int r = 0; r < 4; ++r) cimp[r] = rec[R_IMP + r];
    }
  __syncwarp();
  return pile_integrate_world(wf, L, rk4, lane);
}

// the sweeps of one env-step on the calling lane's four-lane group (its
// half's world); out of line, so that only the sweep's own registers are
// live in it (the collide phase needs about twice as many)
__device__ __noinline__ void fused_sweeps(float* sc, const short* perm, const short* loff, float (*acc)[6], int nb,
                                          int iters, int nlev, int itmax, int nlmax, int slot, int l, unsigned gm) {
  for (int it = 0; it < itmax; ++it)
    for (int v = 0; v < nlmax; ++v) {
      if (it < iters && v < nlev) {
        const int idx = loff[v] + slot;
        if (idx < loff[v + 1]) fused_contact(sc + FR * perm[idx], l, gm, nb, acc);
      }
      __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// the kernel: gangs of warps over the world queue
// ---------------------------------------------------------------------------
// work (nullable): [0] active contacts summed over every world's env-steps,
// [1] contact-update rounds summed over sweeps, [2] rounds summed over
// env-steps, [3] worlds stepped.  cost (per flat world index): this call's
// contact-update rounds plus 64 per contact, the sort key of the next
// call's queue.  nbm / cm: the table's largest body count and contact
// capacity (they size the shared memory).
// GANG: warps per block; MID: a block barrier between assembly and the
// sweeps as well as after integration (otherwise only after integration);
// MINB: blocks per SM the registers are sized for (smaller gangs wait at
// their barrier on fewer worlds; several gangs share an SM);
// WPW: worlds per warp.  With two, the warp takes two consecutive worlds of
// the queue (of about the same cost), runs collide, assembly and
// integration for each in turn on all 32 lanes, and sweeps both at once,
// each on a half-warp with rounds of at most four contacts: the rounds of a
// settled pile fill five of eight groups on average, so two half-filled
// worlds share one warp's instructions.  A body's contacts keep their order
// under either round capacity, so the results are the same.
// Per-world bookkeeping of a warp's worlds, in shared memory (written by
// lane 0, read by all) so that the sweep keeps only its own registers live.
struct FusedSlot {
  const PileGroupDev* g;  // null: no world
  int w, t, iters, rk4, bad, overflow, nact, nlev;
  unsigned long long n_con, n_rounds, n_lev;
};

template <int GANG, bool MID, int WPW, int MINB>
__global__ void __launch_bounds__(32 * GANG, MINB) pile_k_fused(const PileGroupDev* G, const int* wseg, int ng,
                                                             const int* queue, int n_items, int* counter, int n_steps,
                                                             unsigned long long* work, unsigned* cost, int nbm,
                                                             int cm) {
  static_assert(WPW == 1 || WPW == 2, "one or two worlds per warp");
  static_assert(GANG * WPW <= 32, "slots per block");
  extern __shared__ __align__(16) unsigned char fsm[];
  __shared__ int gang_base;
  __shared__ FusedSlot fslot[32];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int half = WPW == 2 ? lane >> 4 : 0;  // the world this lane sweeps
  const int slot = (lane >> 2) & (8 / WPW - 1), l = lane & 3;
  const int cap = 8 / WPW;                    // contacts per round
  const unsigned gm = 0xFu << (lane & ~3);
  const WarpSmem ws = warp_smem(nbm, cm);
  FusedSlot* my = fslot + WPW * wib;
  auto region = [&](int j) { return fsm + (size_t)(WPW * wib + j) * ws.bytes; };
  auto acc_of = [&](int j) { return reinterpret_cast<float(*)[6]>(region(j) + ws.acc); };
  auto sh_of = [&](int j, int off) { return reinterpret_cast<short*>(region(j) + off); };
  for (;;) {
    __syncthreads();  // every warp is done with the previous gang's base
    if (threadIdx.x == 0) gang_base = atomicAdd(counter, WPW * GANG);
    __syncthreads();
    if (gang_base >= n_items) break;  // uniform over the block
    // this warp's worlds, if any (a gang at the end of the queue is partial)
    for (int j = 0; j < WPW; ++j) {
      const int item = gang_base + WPW * wib + j;
      const int t = item < n_items ? (queue ? queue[item] : item) : -1;
      const PileGroupDev* g = nullptr;
      int w = 0;
      if (t >= 0 && t < wseg[ng]) {
        const int gi = find_seg(wseg, ng, t);
        g = G + gi;
        w = t - wseg[gi];
        if (w >= g->n || !g->I[(size_t)w * g->lay.istride + g->lay.live]) g = nullptr;
      }
      if (lane == 0) {
        FusedSlot f{};
        f.g = g;
        f.w = w;
        f.t = t;
        if (g) {
          f.iters = g->I[(size_t)w * g->lay.istride + g->lay.iters];
          f.rk4 = g->I[(size_t)w * g->lay.istride + g->lay.integ] == NEWT_INTEGRATOR_RK4;
        }
        my[j] = f;
      }
      if (g) {  // uniform over the warp
        const WsLay L = ws_layout(g->nb, g->np, g->maxc);
        float* wf = g->scr + (size_t)w * g->sstride;
        ws_load(*g, w, L, wf, reinterpret_cast<int*>(wf + L.nf), lane);
      }
    }
    __syncwarp();
    for (int s = 0; s < n_steps; ++s) {
      for (int j = 0; j < WPW; ++j) {
        const PileGroupDev* g = my[j].g;
        if (!g) continue;
        int ovf = 0;
        const int2 nn = fused_prepare(g, my[j].w, lane, acc_of(j), sh_of(j, ws.last), sh_of(j, ws.lev),
                                      sh_of(j, ws.perm), sh_of(j, ws.loff), &ovf, cap);
        if (lane == 0) {
          const short* loff = sh_of(j, ws.loff);
          int rounds = 0;
          for (int v = 0; v < nn.y; ++v) rounds += (loff[v + 1] - loff[v] + cap - 1) / cap;
          FusedSlot& f = my[j];
          f.overflow |= ovf;
          f.nact = nn.x;
          f.nlev = nn.y;
          f.n_con += (unsigned long long)nn.x;
          f.n_rounds += (unsigned long long)rounds * (unsigned long long)f.iters;
          f.n_lev += (unsigned long long)nn.y;
        }
        __syncwarp();
      }
      if (MID) __syncthreads();  // the gang leaves collide and assembly together
      {
        // the sweeps: each lane's four-lane group on its half's world
        int itmax = 0, nlmax = 0;
        for (int j = 0; j < WPW; ++j)
          if (my[j].g) { itmax = max(itmax, my[j].iters); nlmax = max(nlmax, my[j].nlev); }
        const PileGroupDev* mg = my[half].g;
        const int my_it = mg ? my[half].iters : 0, my_nl = mg ? my[half].nlev : 0, my_nb = mg ? mg->nb : 0;
        float* my_sc = nullptr;
        if (mg) my_sc = mg->scr + (size_t)my[half].w * mg->sstride + ws_layout(mg->nb, mg->np, mg->maxc).sc;
        fused_sweeps(my_sc, sh_of(half, ws.perm), sh_of(half, ws.loff), acc_of(half), my_nb, my_it, my_nl, itmax,
                     nlmax, slot, l, gm);
      }
      if (MID) __syncthreads();  // and the sweeps
      for (int j = 0; j < WPW; ++j) {
        const PileGroupDev* g = my[j].g;
        if (!g) continue;
        const bool b = fused_finish(g, my[j].w, lane, acc_of(j), my[j].nact, s == n_steps - 1, my[j].rk4);
        if (lane == 0) my[j].bad |= b;
        __syncwarp();
      }
      if (!MID) __syncthreads();  // one barrier per env-step
    }
    for (int j = 0; j < WPW; ++j) {
      const PileGroupDev* g = my[j].g;
      if (!g) continue;
      const int w = my[j].w;
      const WsLay L = ws_layout(g->nb, g->np, g->maxc);
      float* wf = g->scr + (size_t)w * g->sstride;
      ws_store_state(*g, w, L, wf, lane);
      ws_store_diag(*g, w, L, wf, reinterpret_cast<const int*>(wf + L.nf), lane);
      if (lane == 0) {
        const FusedSlot& f = my[j];
        unsigned st = 0u;
        if (f.overflow) st |= NEWT_WS_CONTACT_OVERFLOW;
        if (f.bad) st |= NEWT_WS_NONFINITE;
        if (st) atomicOr(reinterpret_cast<unsigned*>(g->I + (size_t)w * g->lay.istride + g->lay.status), st);
        if (cost) cost[f.t] = (unsigned)min(f.n_rounds + 64ull * f.n_con, 0xffffffffull);
        if (work) {
          atomicAdd(work + 0, f.n_con);
          atomicAdd(work + 1, f.n_rounds);
          atomicAdd(work + 2, f.n_lev);
          atomicAdd(work + 3, 1ull);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// The launch shapes the autotuner chooses among: (gang warps, barrier between
// assembly and sweeps, worlds per warp, blocks per SM the registers are
// sized for).  On 8192 sixteen-body piles over env-steps 125..625 the gangs
// of 8 warps, two per SM (shape 10), run 4% faster than one gang of 12;
// more warps per SM at 80 or 64 registers run slower (the worlds' solver
// records no longer fit in L1), and two worlds per warp 13% slower.
namespace {
struct FusedShape { int gang; bool mid; int wpw; int minb; };
constexpr FusedShape kShapes[] = {{16, true, 1, 1}, {12, true, 1, 1}, {12, false, 1, 1}, {8, true, 1, 1},
                                  {24, true, 1, 1}, {32, true, 1, 1}, {12, false, 2, 1}, {4, false, 1, 3},
                                  {6, false, 1, 2},  {4, false, 1, 4}, {8, false, 1, 2},  {7, false, 1, 4}};
constexpr int kNumShapes = sizeof(kShapes) / sizeof(kShapes[0]);
template <class F> void with_kernel(int shape, F f) {
  switch (shape) {
    case 0: f(pile_k_fused<16, true, 1, 1>, 16, 1); break;
    case 1: f(pile_k_fused<12, true, 1, 1>, 12, 1); break;
    case 2: f(pile_k_fused<12, false, 1, 1>, 12, 1); break;
    case 3: f(pile_k_fused<8, true, 1, 1>, 8, 1); break;
    case 4: f(pile_k_fused<24, true, 1, 1>, 24, 1); break;
    case 5: f(pile_k_fused<32, true, 1, 1>, 32, 1); break;
    case 6: f(pile_k_fused<12, false, 2, 1>, 12, 2); break;
    case 7: f(pile_k_fused<4, false, 1, 3>, 4, 1); break;
    case 8: f(pile_k_fused<6, false, 1, 2>, 6, 1); break;
    case 9: f(pile_k_fused<4, false, 1, 4>, 4, 1); break;
    case 10: f(pile_k_fused<8, false, 1, 2>, 8, 1); break;
    default: f(pile_k_fused<7, false, 1, 4>, 7, 1); break;
  }
}
}  // namespace

extern "C" int newt_pile_fused_shapes() { return kNumShapes; }

// Warps per block of launch shape `shape`.
extern "C" int newt_pile_fused_warps_per_block(int shape) { return kShapes[shape % kNumShapes].gang; }

// Worlds in flight per block of launch shape `shape`.
extern "C" int newt_pile_fused_worlds_per_block(int shape) {
  return kShapes[shape % kNumShapes].gang * kShapes[shape % kNumShapes].wpw;
}

// Dynamic shared memory of one block holding `worlds` worlds in flight for a
// table whose largest world has `nbm` bodies and contact capacity `cm`.
extern "C" size_t newt_pile_fused_smem_bytes(int worlds, int nbm, int cm) {
  return (size_t)worlds * warp_smem(nbm, cm).bytes;
}

// Resident blocks per SM of launch shape `shape` for that table (outside
// stream capture; sets the kernel's dynamic shared memory limit first).
extern "C" int newt_pile_fused_blocks_per_sm(int shape, int nbm, int cm) {
  int b = 1;
  with_kernel(shape, [&](auto kern, int gang, int wpw) {
    const int bytes = (int)newt_pile_fused_smem_bytes(gang * wpw, nbm, cm);
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, -1);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, 32 * gang, bytes) != cudaSuccess || b < 1) b = 1;
    // The smallest shared-memory carve-out that holds those b blocks: the
    // rest of the SM's unified 256 KB stays L1, where the worlds' solver
    // records (about 12 KB per settled world) live across the sweeps.
    int dev = 0, per_sm = 0, reserved = 0;
    cudaFuncAttributes fa;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) == cudaSuccess &&
        cudaFuncGetAttributes(&fa, kern) == cudaSuccess && per_sm > 0) {
      const long need = (long)b * ((long)bytes + (long)fa.sharedSizeBytes + reserved);
      const int pct = (int)std::min(100L, (need * 100 + per_sm - 1) / per_sm);
      int b2 = 0;
      if (cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, pct) != cudaSuccess ||
          cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, kern, 32 * gang, bytes) != cudaSuccess || b2 < b)
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, -1);
    }
  });
  return b;
}

// Loads the kernels (so a later launch under stream capture creates nothing).
extern "C" cudaError_t newt_pile_fused_prepare() {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, pile_k_queue_sort);
  for (int k = 0; k < kNumShapes && e == cudaSuccess; ++k)
    with_kernel(k, [&](auto kern, int, int) { e = cudaFuncGetAttributes(&a, kern); });
  return e;
}

// One call's launches on `st`: the queue sort by last call's costs (when
// `cost` and `queue` are given), then the gangs of launch shape `shape`.
// `counter` must be zero when the gangs start (the caller clears it on `st`
// first).  Every live world of the table advances `n_steps` env-steps.
extern "C" int newt_launch_pile_fused(const PileGroupDev* dG, const int* dwseg, int ng, int* queue, int n_items,
                                      int* counter, int n_steps, int grid, unsigned long long* work, unsigned* cost,
                                      int nbm, int cm, int shape, cudaStream_t st) {
  if (n_items <= 0 || grid <= 0) return 0;
  int launches = 0;
  if (queue && cost) {
    pile_k_queue_sort<<<1, 1024, 0, st>>>(cost, n_items, queue);
    ++launches;
  }
  with_kernel(shape, [&](auto kern, int gang, int wpw) {
    kern<<<grid, 32 * gang, newt_pile_fused_smem_bytes(gang * wpw, nbm, cm), st>>>(dG, dwseg, ng, queue, n_items,
                                                                                   counter, n_steps, work, cost, nbm,
                                                                                   cm);
  });
  return launches + 1;
}
