// Free-body Newton: the contact solve of pile worlds whose solver is Newton.
//
// Per env-step (newt_launch_pile_solo_step, pile_general.cu): pile_k_collide
// as for PGS (contacts, the active set, per contact the facet rows' J and M^-1 J^T and
// the row constants), then one warp per world here, then pile_k_integrate
// with the velocity changes this kernel leaves (Euler, or RK4 with the
// solver's wrench held over the stages).
//
// The warp's solve restates newt/src/solver.rs:1295-1407
// (solve_free_body_newton_impulses): the rows in contact order (four
// pyramidal facets per condim-3 contact), the dense response
// H_ij = J_i M^-1 J_j^T (column j of newt's matrix is every row's residual
// after a unit impulse on row j), the regulariser on its diagonal, the bias,
// and newt's NewtonSystem::solve with every row non-negative
// (newton_dense.cuh), then the bodies' velocity changes M^-1 J^T f (newt's
// wrenches J^T f / dt, integrated over dt).  H is formed from the records'
// J and M^-1 J^T triples: row i meets column j through every dynamic body
// the two contacts share.
//
// Scratch: past each world's pile scratch, H, its f32 factor, the FP64
// factor and the solver vectors, sized by the world's contact capacity
// (four rows per contact).
#include <algorithm>

#include "../../include/newt_gpu.h"
#include "newton_dense.cuh"
#include "pile_solver.cuh"

using namespace pile;

namespace {

// solver-record fields of pile_k_collide (pile_kernels.cu) that the solve reads
constexpr int S_BIAS = 40, S_REG = 52, S_MU = 53, S_ROWS = 60;

NEWT_HD int up4n(int n) { return (n + 3) / 4 * 4; }

// Newton region of one world, in floats past its pile scratch.
struct NewtonLay {
  int nrc;  // row capacity (4 x contact capacity, a multiple of 4)
  int H, LH, LHd, vec, order, words;
};
NEWT_HD NewtonLay newton_layout(int maxc) {
  NewtonLay n;
  n.nrc = up4n(4 * maxc);
  const int m = n.nrc * n.nrc;
  int f = 0;
  n.H = f; f += m;
  n.LH = f; f += m;
  n.LHd = f; f += 2 * m;    // doubles (the offset is a multiple of 16 floats)
  n.vec = f; f += 9 * n.nrc;  // x, b, d, g, p, s, u, v, breakpoints
  n.order = f; f += up4n(maxc);  // records in contact order (ints)
  n.words = (f + 31) / 32 * 32;
  return n;
}
NEWT_HD int pile_words(const WsLay& L) { return (L.nf + L.ni + 31) / 32 * 32; }

NEWT_D float dot4(float4 a, float4 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
NEWT_D float4 ldg4f(const float* p) { return *reinterpret_cast<const float4*>(p); }

__global__ void __launch_bounds__(32) pile_k_newton(const PileGroupDev* G, const int* wseg, int ng, int total) {
  const int t = blockIdx.x;
  if (t >= total) return;
  const int gi = find_seg(wseg, ng, t);
  const PileGroupDev& g = G[gi];
  if (g.solve != PS_NEWTON) return;
  const int w = t - wseg[gi];
  if (w >= g.n || !g.I[(size_t)w * g.lay.istride + g.lay.live]) return;
  const int lane = threadIdx.x;
  const WsLay L = ws_layout(g.nb, g.np, g.maxc);
  float* wf = g.scr + (size_t)w * g.sstride;
  int* wi = reinterpret_cast<int*>(wf + L.nf);
  const int nb = L.nb;
  const int nisl = wi[L.misc + 3];
  const int nact = nisl > 0 ? wi[L.istart + nisl - 1] + wi[L.icount + nisl - 1] : 0;
  if (nact == 0) return;  // the velocity changes stay zero
  const NewtonLay N = newton_layout(g.maxc);
  float* nw = wf + pile_words(L);
  const int ld = N.nrc, nr = 4 * nact;
  float* H = nw + N.H;
  float* LH = nw + N.LH;
  double* LHd = reinterpret_cast<double*>(nw + N.LHd);
  float* v = nw + N.vec;
  float *vx = v, *vb = v + ld, *vd = v + 2 * ld, *vg = v + 3 * ld, *vp = v + 4 * ld, *vs = v + 5 * ld,
        *vu = v + 6 * ld, *vv = v + 7 * ld, *vbrk = v + 8 * ld;
  int* ord = reinterpret_cast<int*>(nw + N.order);
  const int* sccon = wi + L.sccon;
  const float* sc0 = wf + L.sc;

  // records in contact order: record k's rank is the number of active
  // contacts with a smaller index (sccon holds them in island order)
  for (int k = lane; k < nact; k += 32) {
    const int c = sccon[k];
    int rank = 0;
    for (int q = 0; q < nact; ++q) rank += sccon[q] < c;
    ord[rank] = k;
  }
  __syncwarp();
  auto bodies = [&](int k, int* ba, int* bb) {
    const int* cc = wi + L.ci + CI * sccon[k];
    *ba = cc[2];
    *bb = cc[3];
  };
  // H (column-major, every entry: newt's matrix is J_i M^-1 J_j^T entry by
  // entry, its factor reads the lower triangle and its products the whole),
  // the bias and a zero-friction flag
  bool zero_mu = false;
  for (int e = lane; e < nr * nr; e += 32) {
    const int i = e % nr, j = e / nr;
    const int ki = ord[i >> 2], kj = ord[j >> 2];
    const float* ri = sc0 + (size_t)SC * ki + S_ROWS + 32 * (i & 3);       // J of row i
    const float* rj = sc0 + (size_t)SC * kj + S_ROWS + 32 * (j & 3) + 16;  // M^-1 J^T of row j
    int ia[2], ja[2];
    bodies(ki, &ia[0], &ia[1]);
    bodies(kj, &ja[0], &ja[1]);
    float h = 0.f;
    for (int si = 0; si < 2; ++si) {
      if (ia[si] >= nb) continue;  // a static side's row is zero
      for (int sj = 0; sj < 2; ++sj) {
        if (ja[sj] != ia[si]) continue;
        h += dot4(ldg4f(ri + 8 * si), ldg4f(rj + 8 * sj)) + dot4(ldg4f(ri + 8 * si + 4), ldg4f(rj + 8 * sj + 4));
      }
    }
    if (i == j) h += sc0[(size_t)SC * ki + S_REG];
    H[(size_t)j * ld + i] = h;
  }
  for (int i = lane; i < nr; i += 32) {
    const float* s = sc0 + (size_t)SC * ord[i >> 2];
    vb[i] = s[S_BIAS + (i & 3)];
    vx[i] = 0.f;
    zero_mu = zero_mu || s[S_MU] == 0.f;
  }
  zero_mu = __any_sync(dense::FULL, zero_mu);
  __syncwarp();
  const int iters = g.I[(size_t)w * g.lay.istride + g.lay.iters];
  uint32_t status = 0;
  dense::newton_solve(H, nr, ld, LH, ld, LHd, vx, vb, vd, vg, vp, vs, vu, vv, vbrk, iters, zero_mu, lane, &status);

  // the bodies' velocity changes M^-1 J^T f (world frame), and the impulses
  // to the contact records (the diagnostics surface)
  for (int b = lane; b < nb; b += 32) {
    float dvx = 0.f, dvy = 0.f, dvz = 0.f, dwx = 0.f, dwy = 0.f, dwz = 0.f;
    for (int i = 0; i < nr; ++i) {
      const int k = ord[i >> 2];
      int ba, bb;
      bodies(k, &ba, &bb);
      const float f = vx[i];
      const float* r = sc0 + (size_t)SC * k + S_ROWS + 32 * (i & 3) + 16;
      for (int s = 0; s < 2; ++s) {
        if ((s ? bb : ba) != b) continue;
        const float4 wl = ldg4f(r + 8 * s), wa = ldg4f(r + 8 * s + 4);
        dvx += wl.x * f; dvy += wl.y * f; dvz += wl.z * f;
        dwx += wa.x * f; dwy += wa.y * f; dwz += wa.z * f;
      }
    }
    st3(wf + L.dv + 3 * b, v3(dvx, dvy, dvz));
    st3(wf + L.dw + 3 * b, v3(dwx, dwy, dwz));
  }
  for (int i = lane; i < nr; i += 32) wf[L.con + CF * sccon[ord[i >> 2]] + C_IMP + (i & 3)] = vx[i];
  if (lane == 0 && status)
    atomicOr(reinterpret_cast<unsigned*>(g.I + (size_t)w * g.lay.istride + g.lay.status), status);
}

}  // namespace

// Floats of one world's Newton region (past its pile scratch).
extern "C" size_t newt_pile_newton_bytes(int maxc) { return (size_t)newton_layout(maxc).words * sizeof(float); }

// The dense Newton solve (the solo step's and the contact sensors' re-solve).
extern "C" void newt_launch_pile_newton_solve(const PileGroupDev* dG, const int* dwseg, int ng, int total_worlds,
                                              cudaStream_t st) {
  if (total_worlds > 0) pile_k_newton<<<total_worlds, 32, 0, st>>>(dG, dwseg, ng, total_worlds);
}
