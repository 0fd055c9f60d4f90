// General contact rows: the contact solve of PGS pile worlds whose rows are
// not four pyramidal facets per contact -- the elliptic friction cone, or
// condim 1 (normal only), 4 (plus torsion) or 6 (plus rolling).
//
// Per env-step (newt_launch_pile_solo_step): pile_k_collide as for every
// pile (contacts, the active set, islands with their contacts in contact
// order), then one warp per world here, then pile_k_integrate with the
// velocity changes this kernel leaves.
//
// Restates newt/src/solver.rs:703-1257 (solve_free_bodies_diag_mode, PGS
// branch) for these rows:
//   :752-848    per active contact the block's rows: the facets n +- mu t
//               (pyramidal condim 3), else the normal, the tangents t1 t2
//               (condim >= 3), the torsion about n (condim >= 4) and the
//               rolling rows about t1 t2 (condim 6), the last three angular
//   :1892-1974  row_body_diagonal, contact_regularization (the facets'
//               base tran (1 + mu^2) with the 2 mu^2 factor, every other
//               row's its own diagonal)
//   :944-948    the penetration drives the facets and the normal row only
//   :1085-1200  the sweep: per contact the normal row (non-negative), then
//               the facet pairs, or the tangent pair under the cone
//               (pgs_step_pair_cone, :1620-1676; project_elliptic,
//               :398-411), the torsion cap mu_t f_n (pgs_step_scalar_cap,
//               :1561-1579) and the rolling pair under mu_r f_n, every cap
//               from the normal impulse just updated
// with the combined torsional and rolling coefficients the smaller of the
// two geoms' (geom.rs:397-409) and the block's condim the smaller of theirs.
//
// Contacts of disjoint islands never share a body, so each lane sweeps one
// island (its contacts in contact order, newt's order restricted to the
// island) with the body velocity changes in world frame in the scratch
// record.  The rows sit in the world's solver records (one record of SC
// floats per active contact, island order).
#include "../../include/newt_gpu.h"
#include "pile_solver.cuh"

using namespace pile;

namespace {

// One active contact's block in its SC record: a header, then up to six
// rows of GR floats: J of side a (linear, angular), J of side b, M^-1 J^T of
// side a, of side b (zero for a static side), the diagonal with its
// regulariser, the regulariser, the bias.
enum { G_NR = 0, G_COND = 1, G_FAC = 2, G_MU = 3, G_MUT = 4, G_MUR = 5, G_H01A = 6, G_H01B = 7, G_ROWS = 8 };
constexpr int GR = 28;
enum { R_JA = 0, R_JB = 6, R_WA = 12, R_WB = 18, R_DIAG = 24, R_REG = 25, R_BIAS = 26 };
static_assert(G_ROWS + 6 * GR <= SC, "general rows fit the solver record");

NEWT_D J6 side_j(bool dyn, bool ang, V3 dir, V3 arm, float sgn) {
  if (!dyn) return J6{v3(0.f, 0.f, 0.f), v3(0.f, 0.f, 0.f)};
  if (ang) return J6{v3(0.f, 0.f, 0.f), dir * sgn};
  return J6{dir * sgn, cross(arm, dir) * sgn};
}

// Rows, regularisers, biases and facet pair couplings of active contact k.
NEWT_D void assemble_block(const PileGroupDev& g, int w, const WsLay& L, float* wf, const int* wi, int k) {
  const PileLayout& P = g.lay;
  const float* F = g.F + (size_t)w * P.fstride;
  const int* I = g.I + (size_t)w * P.istride;
  const int nb = L.nb;
  const int c = wi[L.sccon + k];
  float* cf = wf + L.con + CF * c;
  const int* cc = wi + L.ci + CI * c;
  float* blk = wf + L.sc + SC * k;
  const int ea = cc[2], eb = cc[3];
  const bool da = ea < nb, db = eb < nb;
  const float dt = wf[L.dtg];
  const V3 grav = v3(wf[L.dtg + 1], wf[L.dtg + 2], wf[L.dtg + 3]);
  const float* soft = wf + L.soft;
  const int condim = min(I[P.gcond + ea], I[P.gcond + eb]);
  const bool fac = I[P.cone] == NEWT_CONE_PYRAMIDAL && condim == 3;
  const float pen = cf[C_PEN], mu = cf[C_MU];
  const float mut = fminf(F[P.tfric + ea], F[P.tfric + eb]), mur = fminf(F[P.rfric + ea], F[P.rfric + eb]);
  const V3 n = ld3(cf + C_N), pos = ld3(cf + C_POS);
  // tangent_basis (world.rs:3104-3112)
  V3 ref = fabsf(n.z) < 0.9f ? v3(0.f, 0.f, 1.f) : v3(1.f, 0.f, 0.f);
  V3 t1 = cross(ref, n);
  const float tl = sqrtf(len2(t1));
  t1 = tl == 0.f ? v3(0.f, 0.f, 0.f) : t1 * (1.f / tl);
  const V3 t2 = cross(n, t1);
  const V3 arma = da ? pos - ld3(wf + L.pos + 3 * ea) : v3(0.f, 0.f, 0.f);
  const V3 armb = db ? pos - ld3(wf + L.pos + 3 * eb) : v3(0.f, 0.f, 0.f);
  V3 dirs[6];
  bool ang[6] = {false, false, false, false, false, false};
  int nr = 0;
  if (fac) {
    dirs[0] = n + t1 * mu; dirs[1] = n - t1 * mu; dirs[2] = n + t2 * mu; dirs[3] = n - t2 * mu;
    nr = 4;
  } else {
    dirs[nr++] = n;
    if (condim >= 3) { dirs[nr++] = t1; dirs[nr++] = t2; }
    if (condim >= 4) { ang[nr] = true; dirs[nr++] = n; }
    if (condim >= 6) { ang[nr] = true; dirs[nr++] = t1; ang[nr] = true; dirs[nr++] = t2; }
  }
  const float ima = da ? 1.f / wf[L.mass + ea] : 0.f, imb = db ? 1.f / wf[L.mass + eb] : 0.f;
  const S3 Ia = da ? lds(wf + L.iinvw + 6 * ea) : S3{0, 0, 0, 0, 0, 0};
  const S3 Ib = db ? lds(wf + L.iinvw + 6 * eb) : S3{0, 0, 0, 0, 0, 0};
  const float d = impedance(-pen, soft);
  // reference_accel (solver.rs:340-384) with safe_solref (:331-338)
  float tc = soft[0];
  const float dr = soft[1];
  const bool direct = tc < 0.f;
  if (!direct && tc < 2.f * dt) tc = 2.f * dt;
  const float dmax = fminf(fmaxf(soft[3], 1.0e-4f), 0.9999f);
  float b_, k_;
  if (direct) { b_ = -dr / dmax; k_ = -soft[0] / (dmax * dmax); }
  else { b_ = 2.f / (dmax * tc); k_ = d / (dmax * dmax * tc * tc * dr * dr); }
  V3 va = v3(0.f, 0.f, 0.f), vb = v3(0.f, 0.f, 0.f), wa = v3(0.f, 0.f, 0.f), wb = v3(0.f, 0.f, 0.f);
  if (da) {
    wa = qrot(ld4(wf + L.quat + 4 * ea), ld3(wf + L.omg + 3 * ea));
    va = ld3(wf + L.vel + 3 * ea) + cross(wa, arma);
  }
  if (db) {
    wb = qrot(ld4(wf + L.quat + 4 * eb), ld3(wf + L.omg + 3 * eb));
    vb = ld3(wf + L.vel + 3 * eb) + cross(wb, armb);
  }
  const float tran = ima + imb;
  for (int r = 0; r < nr; ++r) {
    const J6 ja = side_j(da, ang[r], dirs[r], arma, 1.f), jb = side_j(db, ang[r], dirs[r], armb, -1.f);
    const J6 wa_ = J6{ja.l * ima, smv(Ia, ja.a)}, wb_ = J6{jb.l * imb, smv(Ib, jb.a)};
    float* row = blk + G_ROWS + GR * r;
    stj(row + R_JA, ja); stj(row + R_JB, jb); stj(row + R_WA, wa_); stj(row + R_WB, wb_);
    // row_body_diagonal: the angular rows carry no mass term
    float aii = 0.f;
    if (da) aii += dot(ja.a, smv(Ia, ja.a)) + (ang[r] ? 0.f : ima);
    if (db) aii += dot(jb.a, smv(Ib, jb.a)) + (ang[r] ? 0.f : imb);
    float reg = 0.f;
    if (d > 0.f) {
      const float breg = (1.f - d) / d * (fac ? tran * (1.f + mu * mu) : aii);
      reg = fac ? 2.f * mu * mu * breg : breg;
    }
    row[R_DIAG] = aii + reg;
    row[R_REG] = reg;
    // the free step moves the linear rows by g dt; the angular rows have none
    float vcur, dvf = 0.f;
    if (ang[r]) {
      vcur = dot(wa - wb, dirs[r]);
    } else {
      vcur = dot(va - vb, dirs[r]);
      if (da) dvf += dot(grav * dt, dirs[r]);
      if (db) dvf -= dot(grav * dt, dirs[r]);
    }
    const float position = (fac || r == 0) ? -pen : 0.f;
    const float aref = -b_ * vcur - k_ * position;
    row[R_BIAS] = dvf - aref * dt;
    row[GR - 1] = 0.f;
  }
  // facet pair couplings h01: row i's residual after a unit impulse on row i + 1
  float h01[2] = {0.f, 0.f};
  if (fac)
    for (int p = 0; p < 2; ++p) {
      const float* ri = blk + G_ROWS + GR * (2 * p);
      const float* rj = blk + G_ROWS + GR * (2 * p + 1);
      const J6 jia = ldj(ri + R_JA), jib = ldj(ri + R_JB), wja = ldj(rj + R_WA), wjb = ldj(rj + R_WB);
      if (da) h01[p] += dot(jia.l, wja.l) + dot(jia.a, wja.a);
      if (db) h01[p] += dot(jib.l, wjb.l) + dot(jib.a, wjb.a);
    }
  blk[G_NR] = (float)nr; blk[G_COND] = (float)condim; blk[G_FAC] = fac ? 1.f : 0.f;
  blk[G_MU] = mu; blk[G_MUT] = mut; blk[G_MUR] = mur; blk[G_H01A] = h01[0]; blk[G_H01B] = h01[1];
  cf[C_ACT] = fac ? 1.f : 2.f;
  for (int q = 0; q < 6; ++q) cf[C_IMP + q] = 0.f;
}

// The island's body velocity changes (world frame, in the scratch record)
// as the sweep reads and moves them.
struct Acc {
  float* dv;
  float* dw;
  int nb;
  NEWT_D float residual(const float* row, int ea, int eb) const {
    float s = 0.f;
    if (ea < nb) s += jdot(ldj(row + R_JA), ld3(dv + 3 * ea), ld3(dw + 3 * ea));
    if (eb < nb) s += jdot(ldj(row + R_JB), ld3(dv + 3 * eb), ld3(dw + 3 * eb));
    return s;
  }
  NEWT_D void apply(const float* row, int ea, int eb, float df) const {
    if (df == 0.f) return;
    if (ea < nb) {
      const J6 m = ldj(row + R_WA);
      st3(dv + 3 * ea, ld3(dv + 3 * ea) + m.l * df);
      st3(dw + 3 * ea, ld3(dw + 3 * ea) + m.a * df);
    }
    if (eb < nb) {
      const J6 m = ldj(row + R_WB);
      st3(dv + 3 * eb, ld3(dv + 3 * eb) + m.l * df);
      st3(dw + 3 * eb, ld3(dw + 3 * eb) + m.a * df);
    }
  }
};

// One contact's rows, one sweep (solver.rs:1085-1200).
NEWT_D void sweep_block(const Acc& acc, const float* blk, float* imp, int ea, int eb, int elliptic) {
  const float* rows = blk + G_ROWS;
  auto res = [&](int r) {
    const float* row = rows + GR * r;
    return acc.residual(row, ea, eb) + row[R_REG] * imp[r] + row[R_BIAS];
  };
  auto set = [&](int r, float f) {
    const float df = f - imp[r];
    imp[r] = f;
    acc.apply(rows + GR * r, ea, eb, df);
  };
  auto nonneg = [&](int r) {  // pgs_step_non_negative (solver.rs:1448-1474)
    const float nf = imp[r] - res(r) / rows[GR * r + R_DIAG];
    set(r, nf < 0.f ? 0.f : nf);
  };
  auto cap = [&](int r, float c) {  // pgs_step_scalar_cap, project_pyramidal
    const float nf = imp[r] - res(r) / rows[GR * r + R_DIAG];
    set(r, nf > c ? c : (nf < -c ? -c : nf));
  };
  auto pair = [&](int i, float h01) {  // pgs_step_pyramidal_pair (solver.rs:1476-1518)
    const int j = i + 1;
    const float ri = res(i), rj = res(j);
    const float h00 = rows[GR * i + R_DIAG], h11 = rows[GR * j + R_DIAG];
    const float det = h00 * h11 - h01 * h01;
    if (det <= 0.f) { nonneg(i); nonneg(j); return; }
    const float di = (-ri * h11 + h01 * rj) / det, dj = (h01 * ri - h00 * rj) / det;
    const float ni = imp[i] + di, nj = imp[j] + dj;
    float fi, fj;
    if (ni >= 0.f && nj >= 0.f) { fi = ni; fj = nj; }
    else if (ni < 0.f && nj < 0.f) { fi = 0.f; fj = 0.f; }
    else if (ni < 0.f) { fi = 0.f; fj = fmaxf(imp[j] - rj / h11, 0.f); }
    else { fi = fmaxf(imp[i] - ri / h00, 0.f); fj = 0.f; }
    set(i, fi);
    set(j, fj);
  };
  auto cone = [&](int r1, float c, float m) {  // pgs_step_pair_cone (solver.rs:1620-1676)
    const int r2 = r1 + 1;
    if (!elliptic) { cap(r1, m * c); cap(r2, m * c); return; }
    const float f1 = imp[r1] - res(r1) / rows[GR * r1 + R_DIAG];
    const float f2 = imp[r2] - res(r2) / rows[GR * r2 + R_DIAG];
    // project_elliptic (solver.rs:398-411), equal coefficients on both axes
    float p1 = 0.f, p2 = 0.f;
    if (c > 0.f && m > 0.f) {
      const float lim = m * c, mag2 = f1 * f1 + f2 * f2;
      if (mag2 <= lim * lim) { p1 = f1; p2 = f2; }
      else { const float s = lim / sqrtf(mag2); p1 = f1 * s; p2 = f2 * s; }
    }
    set(r1, p1);
    set(r2, p2);
  };
  nonneg(0);
  if (blk[G_FAC] != 0.f) {
    pair(0, blk[G_H01A]);
    pair(2, blk[G_H01B]);
    return;
  }
  const int condim = (int)blk[G_COND];
  if (condim < 3) return;
  const float fn = imp[0];
  cone(1, fn, blk[G_MU]);
  if (condim >= 4) cap(3, blk[G_MUT] * fn);
  if (condim >= 6) cone(4, fn, blk[G_MUR]);
}

__global__ void __launch_bounds__(32) pile_k_general(const PileGroupDev* G, const int* wseg, int ng, int total) {
  const int t = blockIdx.x;
  if (t >= total) return;
  const int gi = find_seg(wseg, ng, t);
  const PileGroupDev& g = G[gi];
  if (g.solve != PS_GENERAL) return;
  const int w = t - wseg[gi];
  if (w >= g.n || !g.I[(size_t)w * g.lay.istride + g.lay.live]) return;
  const int lane = threadIdx.x;
  const WsLay L = ws_layout(g.nb, g.np, g.maxc);
  float* wf = g.scr + (size_t)w * g.sstride;
  const int* wi = reinterpret_cast<const int*>(wf + L.nf);
  const int nisl = wi[L.misc + 3];
  const int nact = nisl > 0 ? wi[L.istart + nisl - 1] + wi[L.icount + nisl - 1] : 0;
  if (nact == 0) return;  // the velocity changes stay zero
  for (int k = lane; k < nact; k += 32) assemble_block(g, w, L, wf, wi, k);
  __syncwarp();
  const int iters = g.I[(size_t)w * g.lay.istride + g.lay.iters];
  const int elliptic = g.I[(size_t)w * g.lay.istride + g.lay.cone] == NEWT_CONE_ELLIPTIC;
  const Acc acc{wf + L.dv, wf + L.dw, L.nb};
  for (int i = lane; i < nisl; i += 32) {
    const int k0 = wi[L.istart + i], kn = wi[L.icount + i];
    for (int it = 0; it < iters; ++it)
      for (int k = k0; k < k0 + kn; ++k) {
        const int c = wi[L.sccon + k];
        const int* cc = wi + L.ci + CI * c;
        sweep_block(acc, wf + L.sc + SC * k, wf + L.con + CF * c + C_IMP, cc[2], cc[3], elliptic);
      }
  }
}

}  // namespace

extern "C" void pile_k_collide_launch(const PileGroupDev* dG, const int* dwseg, int ng, int total_worlds,
                                      int total_slots, int* lists, cudaStream_t st);
extern "C" void pile_k_integrate_launch(const PileGroupDev* dG, const int* dwseg, int ng, int total_worlds,
                                        int write_diag, cudaStream_t st);
extern "C" void newt_launch_pile_newton_solve(const PileGroupDev* dG, const int* dwseg, int ng, int total_worlds,
                                              cudaStream_t st);

// The general-row solve alone (the contact sensors' re-solve).
extern "C" void newt_launch_pile_general_solve(const PileGroupDev* dG, const int* dwseg, int ng, int total_worlds,
                                               cudaStream_t st) {
  if (total_worlds > 0) pile_k_general<<<total_worlds, 32, 0, st>>>(dG, dwseg, ng, total_worlds);
}

// One env-step of a table of pile groups solved apart from the facet-row
// PGS kernels, on `st`: collide, the solve of each group's kind (`kinds`:
// bit PS_NEWTON for the dense Newton solve, bit PS_GENERAL for the general
// rows; each kernel passes over the other kind's worlds), integrate.
// Returns the launches issued.
extern "C" int newt_launch_pile_solo_step(const PileGroupDev* dG, const int* dwseg, int ng, int total_worlds,
                                          int total_slots, int* lists, int write_diag, int kinds, cudaStream_t st) {
  if (total_worlds <= 0) return 0;
  int n = 2;
  pile_k_collide_launch(dG, dwseg, ng, total_worlds, total_slots, lists, st);
  if (kinds & (1 << PS_NEWTON)) { newt_launch_pile_newton_solve(dG, dwseg, ng, total_worlds, st); ++n; }
  if (kinds & (1 << PS_GENERAL)) { newt_launch_pile_general_solve(dG, dwseg, ng, total_worlds, st); ++n; }
  pile_k_integrate_launch(dG, dwseg, ng, total_worlds, write_diag, st);
  return n;
}
