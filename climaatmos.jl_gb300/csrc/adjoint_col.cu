// Reverse (adjoint) kernel of the implicit column stage.
//
// The forward stage (kernels_colg.cu) maps the assembled stage state U^ to
//   U   = filter(U^ - W(U^)^-1 R(U^)) with the van Leer minus central
//         correction of rho e_tot added (implicit_tendency.jl:322-339),
//   T_imp = (U - U^) / dtgamma,
// where R = dtgamma T_imp(U0) + (U^ - U0), U0 = filter(U^), is the residual of
// implicit_tendency! (implicit_tendency.jl:185-298) and W the manual Jacobian
// (manual_sparse_jacobian.jl:713-870) solved by BlockArrowheadSolve (:580-583).
// This kernel is the exact reverse mode of that map, including the
// dependence of W on the state: with x = W^-1 R,
//   cotangent(U^) = (dR/dU^)^T y - (d(W x)/dU^)^T y,   y = W^-T cotangent(x),
// so it solves the transposed Schur-complement tridiagonal system and runs the
// Jacobian-entry, residual and thermodynamic formulas backwards.  It then
// distributes cotangent(U^) to u_n and to the stage tendencies it was
// assembled from (U^ = u_n + dt sum_j (a~_ij T_exp_j + a_ij T_imp_j)) and
// accumulates d/d(sponge rate) (beta_w = rate s(z)).
//
// One thread per column with serial sweeps over the levels (the forward and
// transposed tridiagonal solves by the Thomas algorithm); the per-column
// intermediates live in a column-major global scratch so that the threads of
// a warp access consecutive words.
#include <cstdlib>
#include <type_traits>

#include "colcore.cuh"

namespace gb {

namespace {

// scratch arrays (each [Nf][ncols])
enum ColScr {
  // centres
  S_R0 = 0, S_RE, S_U1, S_U2, S_K, S_H, S_PI, S_THV, S_THVR, S_PHID, S_RJ, S_IJ, S_RR, S_RES, S_RN, S_REN,
  S_HN, S_RJN,
  S_BR, S_BRE, S_BU1, S_BU2, S_BK, S_BH, S_BPI, S_BTHV, S_BTHVR, S_BPHIR, S_BRJ, S_BRN, S_BREN, S_BHN, S_BRJN,
  S_BRR, S_BRES, S_BRU0, S_BRU1, S_BEU0, S_BEU1,
  // faces (forward values, then the cotangents S_BU3 .. S_BFHB, which the reverse pass zeroes)
  S_U3, S_H4, S_A, S_B, S_C, S_D, S_CP, S_DP, S_X, S_U3N, S_FR, S_FHB,
  S_BU3, S_BH4, S_BX, S_BD, S_BU3N, S_BF, S_BFH, S_BFR, S_BFHB,
  S_NUM
};

template <class FT>
struct ColVjpArgs {
  StageArgs<FT> A;        // the forward stage's sources and coefficients (U_c etc. unused)
  const FT *Ub_c, *Ub_f;  // cotangent of U (4 centre fields, faces)
  const FT *Tb_c, *Tb_f;  // cotangent of T_imp (rho, rho e_tot; faces)
  FT *Yb_c, *Yb_f;        // cotangent of u_n (accumulated)
  FT *Teb_c[4], *Teb_f[4];  // cotangents of the explicit tendencies (accumulated)
  FT *Tib_c[4], *Tib_f[4];  // cotangents of the implicit tendencies (accumulated)
  FT *scr;
  double *dalpha;         // per-column d/d(sponge rate), accumulated (RSlot<FT> entries)
  // when set: the recorded stage output U and implicit tendency T_imp, from which
  // U^ = U - dtgamma T_imp (the stage leaves u_h unchanged) replaces the assembly
  const FT *Uo_c, *Uo_f, *Tio_c, *Tio_f;
  // init: the tendency cotangents are written, each initialised from the cotangent of
  // u_n as it is on entry (the final-combination transpose's dt b_j Ybar): Teb_j =
  // e0[j] Yb + ce_j U^bar, Tib_j = i0[j] Yb + ci_j U^bar
  int init;
  FT e0[4], i0[4];
  // tby: the cotangent of T_imp is tbs times that of u_n as it is on entry (Tb_c, Tb_f
  // unused): the last stage's implicit tendency enters the final combination with
  // coefficient dt b_4, so its cotangent is read in place instead of materialised
  int tby;
  FT tbs;
};

// Cotangent of T_imp at level k of row 0 (rho) or 1 (rho e_tot), and at face k; rb, cb
// and fb are the column's offsets in the two-row, the four-row and the face layouts.
template <class FT>
__device__ __forceinline__ FT tb_cen(const ColVjpArgs<FT> &V, size_t rb, size_t cb, size_t sc, int row, int k) {
  return V.tby ? V.tbs * V.Yb_c[cb + (size_t)(row ? 3 : 0) * sc + k] : V.Tb_c[rb + (size_t)(row ? sc : 0) + k];
}
template <class FT>
__device__ __forceinline__ FT tb_face(const ColVjpArgs<FT> &V, size_t fb, int k) {
  return V.tby ? V.tbs * V.Yb_f[fb + k] : V.Tb_f[fb + k];
}

template <class FT>
__device__ __forceinline__ FT vl_value(FT u, FT am2, FT am1, FT a0, FT ap1, bool near, FT dtm) {
  const bool pos = u >= FT(0);
  const FT lo = pos ? am2 : am1, c = pos ? am1 : a0, hi = pos ? a0 : ap1;
  if (near) return u * c;
  const FT da = (hi - lo) / FT(2);
  const FT mn = fmin(lo, fmin(c, hi)), mx = fmax(lo, fmax(c, hi));
  const FT sl = copysign(fmin(fabs(da), fmin(FT(2) * (c - mn), FT(2) * (mx - c))), da);
  const FT half = sl * (FT(1) - fabs(u) * dtm) / FT(2);
  return u * (pos ? c + half : c - half);
}

// Partial derivatives of vl_value (piecewise: the active branch of the limiter).
// dh[0..3] are the derivatives with respect to (am2, am1, a0, ap1).
template <class FT>
__device__ __forceinline__ void vl_grad(FT u, FT am2, FT am1, FT a0, FT ap1, bool near, FT dtm, FT &du, FT (&dh)[4]) {
  const bool pos = u >= FT(0);
  const int ilo = pos ? 0 : 1, ic = pos ? 1 : 2, ihi = pos ? 2 : 3;
  const FT lo = pos ? am2 : am1, c = pos ? am1 : a0, hi = pos ? a0 : ap1;
  dh[0] = dh[1] = dh[2] = dh[3] = FT(0);
  if (near) {
    du = c;
    dh[ic] = u;
    return;
  }
  const FT da = (hi - lo) / FT(2);
  const FT mn = fmin(lo, fmin(c, hi)), mx = fmax(lo, fmax(c, hi));
  const FT m1 = fabs(da), m2 = FT(2) * (c - mn), m3 = FT(2) * (mx - c);
  const FT sgn = copysign(FT(1), da);
  // d sl / d (lo, c, hi)
  FT dl[3] = {FT(0), FT(0), FT(0)};
  FT sl;
  if (m1 <= m2 && m1 <= m3) {
    sl = da;
    dl[0] = -FT(0.5);
    dl[2] = FT(0.5);
  } else if (m2 <= m3) {
    sl = sgn * m2;
    dl[1] += FT(2) * sgn;
    const int imn = (lo <= c && lo <= hi) ? 0 : (c <= hi ? 1 : 2);
    dl[imn] -= FT(2) * sgn;
  } else {
    sl = sgn * m3;
    dl[1] -= FT(2) * sgn;
    const int imx = (lo >= c && lo >= hi) ? 0 : (c >= hi ? 1 : 2);
    dl[imx] += FT(2) * sgn;
  }
  const FT f = (FT(1) - fabs(u) * dtm) / FT(2);
  const FT half = sl * f;
  const FT s = pos ? FT(1) : FT(-1);  // value = u (c + s half)
  du = c + s * half + u * s * sl * (-copysign(FT(1), u) * dtm / FT(2));
  const FT k = u * s * f;  // d value / d sl
  dh[ilo] += k * dl[0];
  dh[ic] += u + k * dl[1];
  dh[ihi] += k * dl[2];
}

template <class FT>
__global__ void __launch_bounds__(128) k_col_stage_vjp(DevParams<FT> P, ColVjpArgs<FT> V) {
  const int ncols = P.Nh * NN;
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncols) return;
  const StageArgs<FT> &A = V.A;
  const int e = col >> 4, n = col & 15, Nv = P.Nv, Nf = P.Nf;
  FT *const scr = V.scr;
  auto S = [&](int q, int k) -> FT & { return scr[((size_t)q * Nf + k) * ncols + col]; };
  ColGeo<FT> G;
  G.load(P, e, n);
  const FT dtg = A.dtg, idtg = A.idtg, kap = P.Rd * P.icvd;
  const size_t cb = (size_t)e * 4 * NN * Nv + (size_t)n * Nv, rb = (size_t)e * 2 * NN * Nv + (size_t)n * Nv;
  const size_t fb = ((size_t)e * NN + n) * Nf;
  const int sc = NN * Nv;
  // ------------------------------------------------ forward recompute
  // stage assembly (the forward kernel's order of additions)
  for (int v = 0; v < Nv; ++v) {
    FT h[4];
    for (int c = 0; c < 4; ++c) h[c] = A.un_c[cb + (size_t)c * sc + v];
    for (int j = 0; j < A.nsrc; ++j) {
      for (int c = 0; c < 4; ++c) {
        h[c] += A.ce[j] * A.te_c[j][cb + (size_t)c * sc + v];
        if (j >= 1 && (c == 0 || c == 3)) h[c] += A.ci[j] * A.ti_c[j][rb + (size_t)(c == 0 ? 0 : sc) + v];
      }
    }
    S(S_R0, v) = h[0];
    S(S_U1, v) = h[1];
    S(S_U2, v) = h[2];
    S(S_RE, v) = h[3];
  }
  for (int f = 0; f < Nf; ++f) {
    FT h = A.un_f[fb + f];
    for (int j = 0; j < A.nsrc; ++j) {
      h += A.ce[j] * A.te_f[j][fb + f];
      if (j >= 1) h += A.ci[j] * A.ti_f[j][fb + f];
    }
    S(S_H4, f) = h;
    S(S_U3, f) = (f == 0 || f == Nv) ? FT(0) : h;
  }
  auto g33 = [&](int f) { return P.lf4[f].x; };
  // centre diagnostics of U0
  for (int v = 0; v < Nv; ++v) {
    const Lev4<FT> L = P.lc4[v];
    const FT u1 = S(S_U1, v), u2 = S(S_U2, v), a = S(S_U3, v), b = S(S_U3, v + 1);
    const FT c1 = (G.gu0 * u1 + G.gu1 * u2) * L.z, c2 = (G.gu1 * u1 + G.gu2 * u2) * L.z;
    const FT K = (u1 * c1 + u2 * c2 + (a * (a * g33(v)) + b * (b * g33(v + 1))) / FT(2)) / FT(2);
    Thermo<FT> th;
    thermo(P, S(S_R0, v), S(S_RE, v), K, L.w, P.lr4[v], th);
    S(S_K, v) = K;
    S(S_H, v) = th.h;
    S(S_PI, v) = th.Pi;
    S(S_THV, v) = th.thv;
    S(S_THVR, v) = th.thvr;
    S(S_PHID, v) = th.phid;
    S(S_RJ, v) = S(S_R0, v) * (G.Jh * L.x);
    S(S_IJ, v) = G.iJh * L.y;
  }
  // face fluxes (zero on the boundary faces)
  auto face_F = [&](int f, FT &F, FT &Fh, FT &fr, FT &fhb) {
    if (f == 0 || f >= Nv) { F = Fh = fr = fhb = FT(0); return; }
    const FT rJb = (S(S_RJ, f - 1) + S(S_RJ, f)) / FT(2), hb = (S(S_H, f - 1) + S(S_H, f)) / FT(2);
    F = rJb * (S(S_U3, f) * g33(f));
    Fh = F * hb;
    fr = rJb * g33(f);
    fhb = hb;
  };
  for (int f = 0; f < Nf; ++f) {
    FT F, Fh, fr, fhb;
    face_F(f, F, Fh, fr, fhb);
    S(S_FR, f) = fr;
    S(S_FHB, f) = fhb;
  }
  // centre rows: residual and (scalar, u_3) blocks
  auto crow = [&](int v, FT &ru0, FT &ru1, FT &eu0, FT &eu1) {
    const FT iJ = S(S_IJ, v);
    ru0 = dtg * (S(S_FR, v) * iJ);
    ru1 = dtg * (-S(S_FR, v + 1) * iJ);
    eu0 = dtg * (S(S_FR, v) * iJ * S(S_FHB, v));
    eu1 = dtg * (-S(S_FR, v + 1) * iJ * S(S_FHB, v + 1));
  };
  for (int v = 0; v < Nv; ++v) {
    FT Fa, Fha, fra, fhba, Fb, Fhb, frb, fhbb;
    face_F(v, Fa, Fha, fra, fhba);
    face_F(v + 1, Fb, Fhb, frb, fhbb);
    S(S_RR, v) = dtg * (-((Fb - Fa) * S(S_IJ, v)));
    S(S_RES, v) = dtg * (-((Fhb - Fha) * S(S_IJ, v)));
  }
  // face rows of W and R, Schur complement onto u_3
  struct FRow { FT ur0, ur1, ue0, uu0, uu1, uu2, T3; };
  auto frow = [&](int f) {
    FRow r;
    const FT beta = P.lf4[f].y;
    const FT u3 = S(S_U3, f);
    if (f == 0 || f >= Nv) {
      r.ur0 = r.ur1 = r.ue0 = r.uu0 = r.uu2 = FT(0);
      r.uu1 = -dtg * beta - FT(1);
      r.T3 = -beta * u3;
      return r;
    }
    const int a = f - 1, b = f;
    const FT ra = S(S_R0, a), rbv = S(S_R0, b);
    const FT irb = FT(1) / ((ra + rbv) / FT(2));
    const FT dpa = kap * (P.T0 * P.cpd - S(S_K, a) - P.lc4[a].w);
    const FT dpb = kap * (P.T0 * P.cpd - S(S_K, b) - P.lc4[b].w);
    const FT buoy = P.cpd * ((S(S_THV, a) + S(S_THV, b)) / FT(2)) * (S(S_PI, b) - S(S_PI, a)) * irb;
    r.ur0 = dtg * (dpa * irb + buoy / FT(2));
    r.ur1 = dtg * (-dpb * irb + buoy / FT(2));
    r.ue0 = dtg * (kap * irb);
    const FT u3cm = S(S_U3, f - 1) * g33(f - 1), u3c = u3 * g33(f), u3cp = S(S_U3, f + 1) * g33(f + 1);
    r.uu0 = dtg * (-kap * ra * u3cm * (irb / FT(2)));
    r.uu1 = dtg * (kap * (rbv - ra) * u3c * (irb / FT(2)) - beta) - FT(1);
    r.uu2 = dtg * (kap * rbv * u3cp * (irb / FT(2)));
    const FT thd = ((S(S_THV, a) - S(S_THVR, a)) + (S(S_THV, b) - S(S_THVR, b))) / FT(2);
    r.T3 = -((S(S_PHID, b) - S(S_PHID, a)) + P.cpd * thd * (S(S_PI, b) - S(S_PI, a))) - beta * u3;
    return r;
  };
  for (int f = 0; f < Nf; ++f) {
    const FRow r = frow(f);
    FT aa = r.uu0, bb = r.uu1, cc = r.uu2, rhs = dtg * r.T3 + (S(S_H4, f) - S(S_U3, f));
    if (f >= 1) {
      FT ru0, ru1, eu0, eu1;
      crow(f - 1, ru0, ru1, eu0, eu1);
      aa += r.ur0 * ru0 + r.ue0 * eu0;
      bb += r.ur0 * ru1 + r.ue0 * eu1;
      rhs += r.ur0 * S(S_RR, f - 1) + r.ue0 * S(S_RES, f - 1);
    }
    if (f < Nv) {
      FT ru0, ru1, eu0, eu1;
      crow(f, ru0, ru1, eu0, eu1);
      bb += r.ur1 * ru0 - r.ue0 * eu0;
      cc += r.ur1 * ru1 - r.ue0 * eu1;
      rhs += r.ur1 * S(S_RR, f) - r.ue0 * S(S_RES, f);
    }
    S(S_A, f) = aa;
    S(S_B, f) = bb;
    S(S_C, f) = cc;
    S(S_D, f) = rhs;
  }
  // Thomas solve A x = D
  {
    FT cp = S(S_C, 0) / S(S_B, 0), dp = S(S_D, 0) / S(S_B, 0);
    S(S_CP, 0) = cp;
    S(S_DP, 0) = dp;
    for (int f = 1; f < Nf; ++f) {
      const FT m = S(S_B, f) - S(S_A, f) * cp;
      cp = S(S_C, f) / m;
      dp = (S(S_D, f) - S(S_A, f) * dp) / m;
      S(S_CP, f) = cp;
      S(S_DP, f) = dp;
    }
    FT x = dp;
    S(S_X, Nf - 1) = x;
    for (int f = Nf - 2; f >= 0; --f) {
      x = S(S_DP, f) - S(S_CP, f) * x;
      S(S_X, f) = x;
    }
  }
  // back-substitution
  for (int v = 0; v < Nv; ++v) {
    FT ru0, ru1, eu0, eu1;
    crow(v, ru0, ru1, eu0, eu1);
    const FT xa = S(S_X, v), xb = S(S_X, v + 1);
    S(S_RN, v) = S(S_R0, v) - (ru0 * xa + ru1 * xb - S(S_RR, v));
    S(S_REN, v) = S(S_RE, v) - (eu0 * xa + eu1 * xb - S(S_RES, v));
  }
  for (int f = 0; f < Nf; ++f) S(S_U3N, f) = (f == 0 || f >= Nv) ? FT(0) : S(S_U3, f) - S(S_X, f);
  // van Leer forward quantities at the Newton result
  for (int v = 0; v < Nv; ++v) {
    const Lev4<FT> L = P.lc4[v];
    const FT u1 = S(S_U1, v), u2 = S(S_U2, v), a = S(S_U3N, v), b = S(S_U3N, v + 1);
    const FT c1 = (G.gu0 * u1 + G.gu1 * u2) * L.z, c2 = (G.gu1 * u1 + G.gu2 * u2) * L.z;
    const FT K = (u1 * c1 + u2 * c2 + (a * (a * g33(v)) + b * (b * g33(v + 1))) / FT(2)) / FT(2);
    Thermo<FT> th;
    thermo(P, S(S_RN, v), S(S_REN, v), K, L.w, P.lr4[v], th);
    S(S_HN, v) = th.h;
    S(S_RJN, v) = S(S_RN, v) * (G.Jh * L.x);
  }
  // ------------------------------------------------ reverse
  for (int v = 0; v < Nv; ++v)
    for (int q = S_BR; q <= S_BEU1; ++q) S(q, v) = FT(0);
  for (int f = 0; f < Nf; ++f)
    for (int q = S_BU3; q <= S_BFHB; ++q) S(q, f) = FT(0);
  CSum<FT> dal;
  // output cotangents: U and T_imp = (U - U^) / dtgamma
  for (int v = 0; v < Nv; ++v) {
    S(S_BRN, v) = V.Ub_c[cb + v] + tb_cen(V, rb, cb, sc, 0, v) * idtg;
    S(S_BREN, v) = V.Ub_c[cb + (size_t)3 * sc + v] + tb_cen(V, rb, cb, sc, 1, v) * idtg;
  }
  for (int f = 0; f < Nf; ++f) S(S_BU3N, f) = V.Ub_f[fb + f] + tb_face(V, fb, f) * idtg;
  // (a) van Leer correction: rhoe_out = rhoe_n + dtgamma corr(state_n)
  if (P.upwinding) {
    for (int f = 1; f < Nv; ++f) {
      FT cb_ = FT(0);  // cotangent of fup(f); that of fcen(f) is -cb_
      if (f < Nv) cb_ += dtg * S(S_BREN, f) * S(S_IJ, f);
      cb_ -= dtg * S(S_BREN, f - 1) * S(S_IJ, f - 1);
      const FT u = S(S_U3N, f) * g33(f);
      const FT rJb = (S(S_RJN, f - 1) + S(S_RJN, f)) / FT(2);
      const bool near = f == 1 || f == Nv - 1;
      const FT hm2 = f >= 2 ? S(S_HN, f - 2) : FT(0), hm1 = S(S_HN, f - 1), h0 = S(S_HN, f);
      const FT hp1 = f + 1 < Nv ? S(S_HN, f + 1) : FT(0);
      const FT vl = vl_value(u, hm2, hm1, h0, hp1, near, P.dt_model);
      FT du, dh[4];
      vl_grad(u, hm2, hm1, h0, hp1, near, P.dt_model, du, dh);
      const FT hm = (hm1 + h0) / FT(2);
      const FT rJbb = cb_ * vl - cb_ * u * hm;
      S(S_BRJN, f - 1) += rJbb / FT(2);
      S(S_BRJN, f) += rJbb / FT(2);
      const FT ub = cb_ * rJb * du - cb_ * rJb * hm;
      S(S_BU3N, f) += ub * g33(f);
      if (f >= 2) S(S_BHN, f - 2) += cb_ * rJb * dh[0];
      S(S_BHN, f - 1) += cb_ * rJb * dh[1] - cb_ * rJb * u / FT(2);
      S(S_BHN, f) += cb_ * rJb * dh[2] - cb_ * rJb * u / FT(2);
      if (f + 1 < Nv) S(S_BHN, f + 1) += cb_ * rJb * dh[3];
    }
    for (int v = 0; v < Nv; ++v) {
      const Lev4<FT> L = P.lc4[v];
      const FT u1 = S(S_U1, v), u2 = S(S_U2, v), a = S(S_U3N, v), b = S(S_U3N, v + 1);
      const FT c1 = (G.gu0 * u1 + G.gu1 * u2) * L.z, c2 = (G.gu1 * u1 + G.gu2 * u2) * L.z;
      const FT K = (u1 * c1 + u2 * c2 + (a * (a * g33(v)) + b * (b * g33(v + 1))) / FT(2)) / FT(2);
      ThermoBar<FT> tb{};
      tb.h = S(S_BHN, v);
      FT rb_, reb, Kb;
      thermo_vjp(P, S(S_RN, v), S(S_REN, v), K, L.w, tb, rb_, reb, Kb);
      S(S_BRN, v) += rb_ + (G.Jh * L.x) * S(S_BRJN, v);
      S(S_BREN, v) += reb;
      S(S_BU1, v) += c1 * Kb;
      S(S_BU2, v) += c2 * Kb;
      S(S_BU3N, v) += Kb * a * g33(v) / FT(2);
      S(S_BU3N, v + 1) += Kb * b * g33(v + 1) / FT(2);
    }
  }
  // (b) back-substitution
  for (int v = 0; v < Nv; ++v) {
    S(S_BR, v) += S(S_BRN, v);
    S(S_BRE, v) += S(S_BREN, v);
    S(S_BRR, v) += S(S_BRN, v);
    S(S_BRES, v) += S(S_BREN, v);
    S(S_BRU0, v) -= S(S_BRN, v) * S(S_X, v);
    S(S_BRU1, v) -= S(S_BRN, v) * S(S_X, v + 1);
    S(S_BEU0, v) -= S(S_BREN, v) * S(S_X, v);
    S(S_BEU1, v) -= S(S_BREN, v) * S(S_X, v + 1);
  }
  for (int f = 0; f < Nf; ++f) {
    FT xb = FT(0);
    if (f < Nv) {
      FT ru0, ru1, eu0, eu1;
      crow(f, ru0, ru1, eu0, eu1);
      xb -= S(S_BRN, f) * ru0 + S(S_BREN, f) * eu0;
    }
    if (f >= 1) {
      FT ru0, ru1, eu0, eu1;
      crow(f - 1, ru0, ru1, eu0, eu1);
      xb -= S(S_BRN, f - 1) * ru1 + S(S_BREN, f - 1) * eu1;
    }
    const bool inner = f > 0 && f < Nv;
    if (inner) {
      xb -= S(S_BU3N, f);
      S(S_BU3, f) += S(S_BU3N, f);
    }
    S(S_BX, f) = xb;
  }
  // (c) transposed solve A^T dbar = xbar  (A^T: sub C[f-1], diagonal B[f], super A[f+1])
  {
    FT cp = (Nf > 1 ? S(S_A, 1) : FT(0)) / S(S_B, 0), dp = S(S_BX, 0) / S(S_B, 0);
    S(S_CP, 0) = cp;
    S(S_DP, 0) = dp;
    for (int f = 1; f < Nf; ++f) {
      const FT sub = S(S_C, f - 1);
      const FT m = S(S_B, f) - sub * cp;
      cp = (f + 1 < Nf ? S(S_A, f + 1) : FT(0)) / m;
      dp = (S(S_BX, f) - sub * dp) / m;
      S(S_CP, f) = cp;
      S(S_DP, f) = dp;
    }
    FT y = dp;
    S(S_BD, Nf - 1) = y;
    for (int f = Nf - 2; f >= 0; --f) {
      y = S(S_DP, f) - S(S_CP, f) * y;
      S(S_BD, f) = y;
    }
  }
  // (d) Schur rows, Jacobian entries and the u_3 tendency
  for (int f = 0; f < Nf; ++f) {
    const FT db = S(S_BD, f);
    const FT ab = f >= 1 ? -db * S(S_X, f - 1) : FT(0);
    const FT bbb = -db * S(S_X, f);
    const FT cbb = f + 1 < Nf ? -db * S(S_X, f + 1) : FT(0);
    const FRow r = frow(f);
    FT ur0b = FT(0), ur1b = FT(0), ue0b = FT(0);
    if (f >= 1) {
      FT ru0, ru1, eu0, eu1;
      crow(f - 1, ru0, ru1, eu0, eu1);
      ur0b += ru0 * ab + ru1 * bbb + S(S_RR, f - 1) * db;
      ue0b += eu0 * ab + eu1 * bbb + S(S_RES, f - 1) * db;
      S(S_BRU0, f - 1) += r.ur0 * ab;
      S(S_BRU1, f - 1) += r.ur0 * bbb;
      S(S_BEU0, f - 1) += r.ue0 * ab;
      S(S_BEU1, f - 1) += r.ue0 * bbb;
      S(S_BRR, f - 1) += r.ur0 * db;
      S(S_BRES, f - 1) += r.ue0 * db;
    }
    if (f < Nv) {
      FT ru0, ru1, eu0, eu1;
      crow(f, ru0, ru1, eu0, eu1);
      ur1b += ru0 * bbb + ru1 * cbb + S(S_RR, f) * db;
      ue0b -= eu0 * bbb + eu1 * cbb + S(S_RES, f) * db;
      S(S_BRU0, f) += r.ur1 * bbb;
      S(S_BRU1, f) += r.ur1 * cbb;
      S(S_BEU0, f) -= r.ue0 * bbb;
      S(S_BEU1, f) -= r.ue0 * cbb;
      S(S_BRR, f) += r.ur1 * db;
      S(S_BRES, f) -= r.ue0 * db;
    }
    // rhs = dtgamma T3 + (U^_3 - U0_3)
    const FT T3b = dtg * db;
    S(S_BH4, f) += db;
    S(S_BU3, f) -= db;
    const FT spg = P.levf[LF_SPG * Nf + f], beta = P.lf4[f].y;
    const FT u3 = S(S_U3, f);
    S(S_BU3, f) -= beta * T3b;
    dal.add(-mul_rn(spg * u3, T3b));
    dal.add(-mul_rn(dtg * spg, bbb));  // uu1 = dtgamma (... - beta) - 1
    if (f == 0 || f >= Nv) continue;
    const int a = f - 1, b = f;
    // T3 = -(dPhi - (Phi_r(b) - Phi_r(a)) + cp thd (Pi(b) - Pi(a))) - beta u3
    const FT dPi = S(S_PI, b) - S(S_PI, a);
    const FT thd = ((S(S_THV, a) - S(S_THVR, a)) + (S(S_THV, b) - S(S_THVR, b))) / FT(2);
    S(S_BPHIR, b) += T3b;
    S(S_BPHIR, a) -= T3b;
    const FT thdb = -P.cpd * dPi * T3b;
    S(S_BPI, b) -= P.cpd * thd * T3b;
    S(S_BPI, a) += P.cpd * thd * T3b;
    S(S_BTHV, a) += thdb / FT(2);
    S(S_BTHVR, a) -= thdb / FT(2);
    S(S_BTHV, b) += thdb / FT(2);
    S(S_BTHVR, b) -= thdb / FT(2);
    // Jacobian entries
    const FT uu0b = ab, uu1b = bbb, uu2b = cbb;
    const FT ra = S(S_R0, a), rbv = S(S_R0, b);
    const FT irb = FT(1) / ((ra + rbv) / FT(2));
    const FT dpa = kap * (P.T0 * P.cpd - S(S_K, a) - P.lc4[a].w);
    const FT dpb = kap * (P.T0 * P.cpd - S(S_K, b) - P.lc4[b].w);
    const FT thvb = (S(S_THV, a) + S(S_THV, b)) / FT(2);
    const FT buoy = P.cpd * thvb * dPi * irb;
    const FT u3cm = S(S_U3, f - 1) * g33(f - 1), u3c = u3 * g33(f), u3cp = S(S_U3, f + 1) * g33(f + 1);
    const FT dpab = dtg * irb * ur0b, dpbb = -dtg * irb * ur1b, buoyb = dtg * (ur0b + ur1b) / FT(2);
    FT irbb = dtg * (dpa * ur0b - dpb * ur1b) + dtg * kap * ue0b;
    irbb += dtg * (-kap * ra * u3cm / FT(2)) * uu0b + dtg * (kap * (rbv - ra) * u3c / FT(2)) * uu1b +
            dtg * (kap * rbv * u3cp / FT(2)) * uu2b;
    irbb += buoyb * P.cpd * thvb * dPi;
    const FT thvbb = buoyb * P.cpd * dPi * irb, dPib = buoyb * P.cpd * thvb * irb;
    S(S_BR, a) += dtg * (-kap * u3cm * irb / FT(2)) * uu0b - dtg * kap * u3c * irb / FT(2) * uu1b;
    S(S_BR, b) += dtg * kap * u3c * irb / FT(2) * uu1b + dtg * kap * u3cp * irb / FT(2) * uu2b;
    S(S_BU3, f - 1) += dtg * (-kap * ra * irb / FT(2)) * uu0b * g33(f - 1);
    S(S_BU3, f) += dtg * kap * (rbv - ra) * irb / FT(2) * uu1b * g33(f);
    S(S_BU3, f + 1) += dtg * kap * rbv * irb / FT(2) * uu2b * g33(f + 1);
    S(S_BK, a) -= kap * dpab;
    S(S_BK, b) -= kap * dpbb;
    const FT rbarb = -irb * irb * irbb;
    S(S_BR, a) += rbarb / FT(2);
    S(S_BR, b) += rbarb / FT(2);
    S(S_BTHV, a) += thvbb / FT(2);
    S(S_BTHV, b) += thvbb / FT(2);
    S(S_BPI, b) += dPib;
    S(S_BPI, a) -= dPib;
  }
  // (e) centre rows: R_rho = dtgamma T_rho, blocks from fr, fhb
  for (int v = 0; v < Nv; ++v) {
    const FT iJ = S(S_IJ, v);
    const FT Trb = dtg * S(S_BRR, v), Teb = dtg * S(S_BRES, v);
    S(S_BF, v + 1) -= Trb * iJ;
    S(S_BF, v) += Trb * iJ;
    S(S_BFH, v + 1) -= Teb * iJ;
    S(S_BFH, v) += Teb * iJ;
    S(S_BFR, v) += dtg * iJ * S(S_BRU0, v) + dtg * iJ * S(S_FHB, v) * S(S_BEU0, v);
    S(S_BFR, v + 1) -= dtg * iJ * S(S_BRU1, v) + dtg * iJ * S(S_FHB, v + 1) * S(S_BEU1, v);
    S(S_BFHB, v) += dtg * S(S_FR, v) * iJ * S(S_BEU0, v);
    S(S_BFHB, v + 1) -= dtg * S(S_FR, v + 1) * iJ * S(S_BEU1, v);
  }
  // (f) face fluxes F = rJb u3c, Fh = F hb, fr = rJb g33, fhb = hb
  for (int f = 1; f < Nv; ++f) {
    FT F, Fh, fr, fhb;
    face_F(f, F, Fh, fr, fhb);
    const FT rJb = (S(S_RJ, f - 1) + S(S_RJ, f)) / FT(2), hb = fhb;
    const FT Fb = S(S_BF, f) + S(S_BFH, f) * hb;
    const FT hbb = S(S_BFH, f) * F + S(S_BFHB, f);
    const FT rJbb = Fb * (S(S_U3, f) * g33(f)) + S(S_BFR, f) * g33(f);
    S(S_BU3, f) += Fb * rJb * g33(f);
    S(S_BH, f - 1) += hbb / FT(2);
    S(S_BH, f) += hbb / FT(2);
    S(S_BRJ, f - 1) += rJbb / FT(2);
    S(S_BRJ, f) += rJbb / FT(2);
  }
  // (g) centre diagnostics of U0
  for (int v = 0; v < Nv; ++v) {
    const Lev4<FT> L = P.lc4[v];
    const FT u1 = S(S_U1, v), u2 = S(S_U2, v), a = S(S_U3, v), b = S(S_U3, v + 1);
    const FT c1 = (G.gu0 * u1 + G.gu1 * u2) * L.z, c2 = (G.gu1 * u1 + G.gu2 * u2) * L.z;
    ThermoBar<FT> tb{};
    tb.h = S(S_BH, v);
    tb.Pi = S(S_BPI, v);
    tb.thv = S(S_BTHV, v);
    tb.thvr = S(S_BTHVR, v);
    tb.phir = S(S_BPHIR, v);
    FT rb_, reb, Kb;
    thermo_vjp(P, S(S_R0, v), S(S_RE, v), S(S_K, v), L.w, tb, rb_, reb, Kb);
    S(S_BR, v) += rb_ + (G.Jh * L.x) * S(S_BRJ, v);
    S(S_BRE, v) += reb;
    const FT Kt = Kb + S(S_BK, v);
    S(S_BU1, v) += c1 * Kt;
    S(S_BU2, v) += c2 * Kt;
    S(S_BU3, v) += Kt * a * g33(v) / FT(2);
    S(S_BU3, v + 1) += Kt * b * g33(v + 1) / FT(2);
  }
  // ------------------------------------------------ cotangent of U^ and its distribution
  for (int v = 0; v < Nv; ++v) {
    const FT hb[4] = {S(S_BR, v) - tb_cen(V, rb, cb, sc, 0, v) * idtg, S(S_BU1, v) + V.Ub_c[cb + (size_t)sc + v],
                      S(S_BU2, v) + V.Ub_c[cb + (size_t)2 * sc + v], S(S_BRE, v) - tb_cen(V, rb, cb, sc, 1, v) * idtg};
    FT y0[4];
    for (int c = 0; c < 4; ++c) {
      y0[c] = V.Yb_c[cb + (size_t)c * sc + v];
      V.Yb_c[cb + (size_t)c * sc + v] = y0[c] + hb[c];
    }
    for (int j = 0; j < A.nsrc; ++j) {
      // init: written from the cotangent of u_n on entry (see ColVjpArgs)
      const FT ke = V.init ? V.e0[j] : FT(0), ki = V.init ? V.i0[j] : FT(0);
      for (int c = 0; c < 4; ++c) {
        FT &t = V.Teb_c[j][cb + (size_t)c * sc + v];
        t = (V.init ? ke * y0[c] : t) + A.ce[j] * hb[c];
      }
      if (j >= 1) {
        FT &t0 = V.Tib_c[j][rb + v], &t3 = V.Tib_c[j][rb + (size_t)sc + v];
        t0 = (V.init ? ki * y0[0] : t0) + A.ci[j] * hb[0];
        t3 = (V.init ? ki * y0[3] : t3) + A.ci[j] * hb[3];
      }
    }
  }
  for (int f = 0; f < Nf; ++f) {
    const bool inner = f > 0 && f < Nv;
    const FT hb = S(S_BH4, f) + (inner ? S(S_BU3, f) : FT(0)) - tb_face(V, fb, f) * idtg;
    const FT y0 = V.Yb_f[fb + f];
    V.Yb_f[fb + f] = y0 + hb;
    for (int j = 0; j < A.nsrc; ++j) {
      FT &t = V.Teb_f[j][fb + f];
      t = (V.init ? V.e0[j] * y0 : t) + A.ce[j] * hb;
      if (j >= 1) {
        FT &u = V.Tib_f[j][fb + f];
        u = (V.init ? V.i0[j] * y0 : u) + A.ci[j] * hb;
      }
    }
  }
  RSlot<FT>::put(&V.dalpha[col], dal, false);  // accumulated over the launches of a reverse pass (zeroed by the host)
}


// ============================================================================ lane-parallel form
// The same reverse pass with a column held by G lanes, CM levels per lane (the
// forward stage kernel's layout): the forward is recomputed in registers, the
// transposed tridiagonal system is solved by the lane-parallel cyclic
// reduction, and every scatter to a neighbouring level becomes a local add
// plus one shuffle ("fold") per halo.
namespace lp {

using col::up;
using col::down;

// Value of level r0 - 1 (previous lane's last) and r0 + CM (next lane's first); 0 past the column.
template <int G, int CM, class FT>
__device__ __forceinline__ FT prv(const FT (&x)[CM], int gl) {
  const FT v = up<G>(x[CM - 1], 1);
  return gl > 0 ? v : FT(0);
}
template <int G, int CM, class FT>
__device__ __forceinline__ FT prv2(const FT (&x)[CM], int gl) {
  const FT v = up<G>(x[CM - 2], 1);
  return gl > 0 ? v : FT(0);
}
template <int G, int CM, class FT>
__device__ __forceinline__ FT nxt(const FT (&x)[CM], int gl) {
  const FT v = down<G>(x[0], 1);
  return gl + 1 < G ? v : FT(0);
}
template <int G, int CM, class FT>
__device__ __forceinline__ FT nxt2(const FT (&x)[CM], int gl) {
  const FT v = down<G>(x[1], 1);
  return gl + 1 < G ? v : FT(0);
}
// own[] += the contributions neighbours computed for this lane's levels:
// toPrev is this lane's contribution to level r0 - 1, toNext to level r0 + CM.
template <int G, int CM, class FT>
__device__ __forceinline__ void fold1(FT (&own)[CM], FT toPrev, FT toNext, int gl) {
  const FT fn = down<G>(toPrev, 1), fp = up<G>(toNext, 1);
  if (gl + 1 < G) own[CM - 1] += fn;
  if (gl > 0) own[0] += fp;
}
// halo 2: toPrev2 -> r0 - 2, toPrev1 -> r0 - 1, toNext0 -> r0 + CM, toNext1 -> r0 + CM + 1
template <int G, int CM, class FT>
__device__ __forceinline__ void fold2(FT (&own)[CM], FT toPrev2, FT toPrev1, FT toNext0, FT toNext1, int gl) {
  const FT a = down<G>(toPrev2, 1), b = down<G>(toPrev1, 1), c = up<G>(toNext0, 1), d = up<G>(toNext1, 1);
  if (gl + 1 < G) { own[CM - 2] += a; own[CM - 1] += b; }
  if (gl > 0) { own[0] += c; own[1] += d; }
}

// thermo_vjp at the lane's CM levels, with the cotangent of h alone (FULL = false) or of
// (h, Pi, thv, thvr, Phi_r); FP32 with two levels per lane: one packed pair.
template <bool FULL, class FT, int CM>
__device__ __forceinline__ void thermo_vjp_lane(const DevParams<FT> &P, const FT (&rho)[CM], const FT (&rhoe)[CM],
                                                const FT (&K)[CM], const FT (&Phi)[CM], const FT (&bh)[CM],
                                                const FT (&bPi)[CM], const FT (&bthv)[CM], const FT (&bthvr)[CM],
                                                const FT (&bphir)[CM], FT (&rb)[CM], FT (&reb)[CM], FT (&Kb)[CM]) {
  if constexpr (std::is_same<FT, float>::value && CM == 2) {
    ThermoBar2 tb;
    tb.T = tb.p = tb.Tr = bc2(0.0f);
    tb.h = make_float2(bh[0], bh[1]);
    tb.Pi = FULL ? make_float2(bPi[0], bPi[1]) : bc2(0.0f);
    tb.thv = FULL ? make_float2(bthv[0], bthv[1]) : bc2(0.0f);
    tb.thvr = FULL ? make_float2(bthvr[0], bthvr[1]) : bc2(0.0f);
    tb.phir = FULL ? make_float2(bphir[0], bphir[1]) : bc2(0.0f);
    float2 r, re, k;
    thermo_vjp_pair(P, make_float2(rho[0], rho[1]), make_float2(rhoe[0], rhoe[1]), make_float2(K[0], K[1]),
                    make_float2(Phi[0], Phi[1]), tb, r, re, k);
    rb[0] = r.x; rb[1] = r.y; reb[0] = re.x; reb[1] = re.y; Kb[0] = k.x; Kb[1] = k.y;
  } else {
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      ThermoBar<FT> tb{};
      tb.h = bh[k];
      if (FULL) {
        tb.Pi = bPi[k];
        tb.thv = bthv[k];
        tb.thvr = bthvr[k];
        tb.phir = bphir[k];
      }
      thermo_vjp(P, rho[k], rhoe[k], K[k], Phi[k], tb, rb[k], reb[k], Kb[k]);
    }
  }
}

// Default register cap: FP32 at 128 registers (four resident 128-thread CTAs per SM), FP64
// uncapped; the FP32 32-lane, two-levels-per-lane form (z_elem < 64) is launched at six CTAs
// per SM instead (launch_column_stage_vjp).
template <class FT>
struct VjpMinBlocks {
  static constexpr int value = sizeof(FT) == 4 ? 4 : 1;
};

// REC: the stage's recorded output U and implicit tendency T_imp are given (V.Uo_c, V.Tio_c):
// the stage input is U - dtgamma T_imp and the Newton update at the inner faces is
// x = U^ - U = -dtgamma T_imp (the update of u_3 is all the stage does to it), so the forward
// tridiagonal solve is not repeated: the boundary rows of the Schur system are diagonal,
// and rho, rho e_tot after the update follow from x by the back-substitution formulas.
template <class FT, int G, int CM, int MINB = VjpMinBlocks<FT>::value, bool REC = false>
__global__ void __launch_bounds__(128, MINB) k_col_stage_vjp_g(DevParams<FT> P, ColVjpArgs<FT> V) {
  const int lane = threadIdx.x & 31, gl = lane % G;
  const int col0 = (blockIdx.x * 4 + (threadIdx.x >> 5)) * (32 / G) + lane / G;
  const int ncols = P.Nh * NN;
  const bool colv = col0 < ncols;
  const int col = colv ? col0 : ncols - 1;
  const StageArgs<FT> &A = V.A;
  const int e = col >> 4, n = col & 15, Nv = P.Nv, Nf = P.Nf, r0 = gl * CM, sc = NN * Nv;
  ColGeo<FT> Gm;
  Gm.load(P, e, n);
  const FT dtg = A.dtg, idtg = A.idtg, kap = P.Rd * P.icvd;
  const size_t cb = (size_t)e * 4 * NN * Nv + (size_t)n * Nv + r0, rb = (size_t)e * 2 * NN * Nv + (size_t)n * Nv + r0;
  const size_t fb = ((size_t)e * NN + n) * Nf + r0;
  const col::ColLev<FT> L{P.lc4, P.lf4, P.lr4, Nv, Nf};
  // The cotangent inputs and the accumulation targets are first touched after
  // the forward recompute: start their lines towards L2 now (one prefetch per
  // field and warp covers the column: the lanes' levels are contiguous).
  if (r0 < Nv) {
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      prefetch_l2(V.Ub_c + cb + (size_t)c * sc);
      prefetch_l2(V.Yb_c + cb + (size_t)c * sc);
    }
    if (!V.tby) {
      prefetch_l2(V.Tb_c + rb);
      prefetch_l2(V.Tb_c + rb + sc);
    }
    for (int j = 0; !V.init && j < A.nsrc; ++j) {  // (init: the tendency cotangents are only written)
      if (V.Teb_c[j])
        for (int c = 0; c < 4; ++c) prefetch_l2(V.Teb_c[j] + cb + (size_t)c * sc);
      if (j >= 1 && V.Tib_c[j]) {
        prefetch_l2(V.Tib_c[j] + rb);
        prefetch_l2(V.Tib_c[j] + rb + sc);
      }
    }
  }
  if (r0 < Nf) {
    prefetch_l2(V.Ub_f + fb);
    if (!V.tby) prefetch_l2(V.Tb_f + fb);
    prefetch_l2(V.Yb_f + fb);
    for (int j = 0; !V.init && j < A.nsrc; ++j) {
      if (V.Teb_f[j]) prefetch_l2(V.Teb_f[j] + fb);
      if (j >= 1 && V.Tib_f[j]) prefetch_l2(V.Tib_f[j] + fb);
    }
  }
  // ---------------------------------------------------------------- forward recompute
  FT H[5][CM], tif[CM];
  if constexpr (REC) {
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const bool okc = r0 + k < Nv, okf = r0 + k < Nf;
      tif[k] = okf ? V.Tio_f[fb + k] : FT(0);
      H[0][k] = okc ? V.Uo_c[cb + k] - dtg * V.Tio_c[rb + k] : FT(0);
      H[1][k] = okc ? V.Uo_c[cb + (size_t)sc + k] : FT(0);
      H[2][k] = okc ? V.Uo_c[cb + (size_t)2 * sc + k] : FT(0);
      H[3][k] = okc ? V.Uo_c[cb + (size_t)3 * sc + k] - dtg * V.Tio_c[rb + (size_t)sc + k] : FT(0);
      H[4][k] = okf ? V.Uo_f[fb + k] - dtg * tif[k] : FT(0);
    }
  } else {
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const bool okc = r0 + k < Nv, okf = r0 + k < Nf;
#pragma unroll
    for (int c = 0; c < 4; ++c) H[c][k] = okc ? A.un_c[cb + (size_t)c * sc + k] : FT(0);
    H[4][k] = okf ? A.un_f[fb + k] : FT(0);
  }
  for (int j = 0; j < A.nsrc; ++j) {
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const bool okc = r0 + k < Nv, okf = r0 + k < Nf;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        H[c][k] += A.ce[j] * (okc ? A.te_c[j][cb + (size_t)c * sc + k] : FT(0));
        if (j >= 1 && (c == 0 || c == 3))
          H[c][k] += A.ci[j] * (okc ? A.ti_c[j][rb + (size_t)(c == 0 ? 0 : sc) + k] : FT(0));
      }
      H[4][k] += A.ce[j] * (okf ? A.te_f[j][fb + k] : FT(0));
      if (j >= 1) H[4][k] += A.ci[j] * (okf ? A.ti_f[j][fb + k] : FT(0));
    }
  }
  }
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    if (r0 + k >= Nv) { H[0][k] = FT(1); H[1][k] = FT(0); H[2][k] = FT(0); H[3][k] = FT(1); }
    if (r0 + k >= Nf) H[4][k] = FT(0);
  }
  FT u3[CM], g33[CM], beta[CM], spg[CM];
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const int f = r0 + k;
    u3[k] = (f == 0 || f >= Nv) ? FT(0) : H[4][k];
    const Lev4<FT> lf = P.lf4[min(f, Nf - 1)];
    g33[k] = lf.x;
    beta[k] = lf.y;
    spg[k] = P.levf[LF_SPG * Nf + min(f, Nf - 1)];
  }
  const FT u3n0 = nxt<G, CM>(u3, gl), g33n0 = nxt<G, CM>(g33, gl);
  const FT u3p = prv<G, CM>(u3, gl), g33p = prv<G, CM>(g33, gl);
  // centre diagnostics of U0
  FT K[CM], h[CM], Pi[CM], thv[CM], thvr[CM], phid[CM], rJ[CM], iJ[CM], c1[CM], c2[CM], Jc[CM], phi[CM];
  {
    FT ub[CM], gb[CM];
    col::Cen<FT> cc[CM];
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      ub[k] = k + 1 < CM ? u3[k + 1] : u3n0;
      gb[k] = k + 1 < CM ? g33[k + 1] : g33n0;
    }
    col::cdiag_lane<FT, CM>(P, Gm, L, r0, H, u3, ub, g33, gb, cc);
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const Lev4<FT> Lc = P.lc4[min(r0 + k, Nv - 1)];
      c1[k] = (Gm.gu0 * H[1][k] + Gm.gu1 * H[2][k]) * Lc.z;
      c2[k] = (Gm.gu1 * H[1][k] + Gm.gu2 * H[2][k]) * Lc.z;
      K[k] = cc[k].K; h[k] = cc[k].h; Pi[k] = cc[k].Pi; thv[k] = cc[k].thv; thvr[k] = cc[k].thvr;
      phid[k] = cc[k].phid; rJ[k] = cc[k].rJ; iJ[k] = cc[k].iJ; Jc[k] = Gm.Jh * Lc.x; phi[k] = cc[k].phi;
    }
  }
  // previous-level (centre r0 - 1) values
  const FT rJp = prv<G, CM>(rJ, gl), hp = prv<G, CM>(h, gl), Kp = prv<G, CM>(K, gl), Pip = prv<G, CM>(Pi, gl);
  const FT thvp = prv<G, CM>(thv, gl), thvrp = prv<G, CM>(thvr, gl), phidp = prv<G, CM>(phid, gl);
  const FT rhop = prv<G, CM>(H[0], gl), phip = prv<G, CM>(phi, gl);
  auto cprev = [&](const FT (&x)[CM], int k, FT pv) { return k > 0 ? x[k - 1] : pv; };
  // face fluxes and rows
  FT fr[CM], fhb[CM], F[CM], Fh[CM], T3[CM], ur0[CM], ur1[CM], ue0[CM], uu0[CM], uu1[CM], uu2[CM];
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const int f = r0 + k;
    const bool inner = f > 0 && f < Nv;
    const FT rJa = cprev(rJ, k, rJp), ha = cprev(h, k, hp);
    const FT rJb = (rJa + rJ[k]) / FT(2), hb = (ha + h[k]) / FT(2);
    F[k] = inner ? rJb * (u3[k] * g33[k]) : FT(0);
    Fh[k] = F[k] * hb;
    fr[k] = inner ? rJb * g33[k] : FT(0);
    fhb[k] = inner ? hb : FT(0);
    if (inner) {
      const FT ra = cprev(H[0], k, rhop), rbv = H[0][k];
      const FT irb = FT(1) / ((ra + rbv) / FT(2));
      const FT dpa = kap * (P.T0 * P.cpd - cprev(K, k, Kp) - cprev(phi, k, phip));
      const FT dpb = kap * (P.T0 * P.cpd - K[k] - phi[k]);
      const FT thva = cprev(thv, k, thvp), Pia = cprev(Pi, k, Pip);
      const FT buoy = P.cpd * ((thva + thv[k]) / FT(2)) * (Pi[k] - Pia) * irb;
      ur0[k] = dtg * (dpa * irb + buoy / FT(2));
      ur1[k] = dtg * (-dpb * irb + buoy / FT(2));
      ue0[k] = dtg * (kap * irb);
      const FT u3cm = cprev(u3, k, u3p) * cprev(g33, k, g33p), u3c = u3[k] * g33[k];
      const FT u3cp = (k + 1 < CM ? u3[k + 1] : u3n0) * (k + 1 < CM ? g33[k + 1] : g33n0);
      uu0[k] = dtg * (-kap * ra * u3cm * (irb / FT(2)));
      uu1[k] = dtg * (kap * (rbv - ra) * u3c * (irb / FT(2)) - beta[k]) - FT(1);
      uu2[k] = dtg * (kap * rbv * u3cp * (irb / FT(2)));
      const FT thd = ((thva - cprev(thvr, k, thvrp)) + (thv[k] - thvr[k])) / FT(2);
      T3[k] = -((phid[k] - cprev(phid, k, phidp)) + P.cpd * thd * (Pi[k] - Pia)) - beta[k] * u3[k];
    } else {
      ur0[k] = ur1[k] = ue0[k] = uu0[k] = uu2[k] = FT(0);
      uu1[k] = f <= Nv ? -dtg * beta[k] - FT(1) : FT(1);
      T3[k] = -beta[k] * u3[k];
    }
  }
  const FT Fn = nxt<G, CM>(F, gl), Fhn = nxt<G, CM>(Fh, gl), frn = nxt<G, CM>(fr, gl), fhbn = nxt<G, CM>(fhb, gl);
  auto fnext = [&](const FT (&x)[CM], int k, FT nv) { return k + 1 < CM ? x[k + 1] : nv; };
  FT Rr[CM], Re[CM], ru0[CM], ru1[CM], eu0[CM], eu1[CM];
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const bool cv = r0 + k < Nv;
    Rr[k] = cv ? dtg * (-((fnext(F, k, Fn) - F[k]) * iJ[k])) : FT(0);
    Re[k] = cv ? dtg * (-((fnext(Fh, k, Fhn) - Fh[k]) * iJ[k])) : FT(0);
    ru0[k] = cv ? dtg * (fr[k] * iJ[k]) : FT(0);
    ru1[k] = cv ? dtg * (-fnext(fr, k, frn) * iJ[k]) : FT(0);
    eu0[k] = cv ? dtg * (fr[k] * iJ[k] * fhb[k]) : FT(0);
    eu1[k] = cv ? dtg * (-fnext(fr, k, frn) * iJ[k] * fnext(fhb, k, fhbn)) : FT(0);
  }
  const FT ru0p = prv<G, CM>(ru0, gl), ru1p = prv<G, CM>(ru1, gl), eu0p = prv<G, CM>(eu0, gl);
  const FT eu1p = prv<G, CM>(eu1, gl), Rrp = prv<G, CM>(Rr, gl), Rep = prv<G, CM>(Re, gl);
  FT Sa[CM], Sb[CM], Sc[CM], Sd[CM];
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const int f = r0 + k;
    FT aa = uu0[k], bb = uu1[k], cc = uu2[k], rhs = f < Nf ? dtg * T3[k] + (H[4][k] - u3[k]) : FT(0);
    if (f >= 1 && f - 1 < Nv) {
      aa += ur0[k] * cprev(ru0, k, ru0p) + ue0[k] * cprev(eu0, k, eu0p);
      bb += ur0[k] * cprev(ru1, k, ru1p) + ue0[k] * cprev(eu1, k, eu1p);
      rhs += ur0[k] * cprev(Rr, k, Rrp) + ue0[k] * cprev(Re, k, Rep);
    }
    if (f < Nv) {
      bb += ur1[k] * ru0[k] - ue0[k] * eu0[k];
      cc += ur1[k] * ru1[k] - ue0[k] * eu1[k];
      rhs += ur1[k] * Rr[k] - ue0[k] * Re[k];
    }
    if (f >= Nf) { aa = FT(0); bb = FT(1); cc = FT(0); rhs = FT(0); }
    Sa[k] = aa; Sb[k] = bb; Sc[k] = cc; Sd[k] = rhs;
  }
  FT x[CM];
  if constexpr (REC) {
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const int f = r0 + k;
      x[k] = f >= Nf ? FT(0) : (f == 0 || f == Nv) ? Sd[k] / Sb[k] : -dtg * tif[k];
    }
  } else {
    FT a_[CM], b_[CM], c_[CM], d_[CM];
#pragma unroll
    for (int k = 0; k < CM; ++k) { a_[k] = Sa[k]; b_[k] = Sb[k]; c_[k] = Sc[k]; d_[k] = Sd[k]; }
    col::solve_lanes<FT, G, CM>(a_, b_, c_, d_, x, gl);
  }
  const FT xn0 = nxt<G, CM>(x, gl), xp = prv<G, CM>(x, gl);
  FT RN[CM], REN[CM], U3N[CM];
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const int f = r0 + k;
    const FT xu = fnext(x, k, xn0);
    RN[k] = H[0][k] - (ru0[k] * x[k] + ru1[k] * xu - Rr[k]);
    REN[k] = H[3][k] - (eu0[k] * x[k] + eu1[k] * xu - Re[k]);
    if (f >= Nv) { RN[k] = FT(1); REN[k] = FT(1); }
    U3N[k] = (f == 0 || f >= Nv) ? FT(0) : u3[k] - x[k];
  }
  // ---------------------------------------------------------------- reverse
  FT bRN[CM], bREN[CM], bU3N[CM], bU1[CM], bU2[CM];
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const bool okc = r0 + k < Nv, okf = r0 + k < Nf;
    bRN[k] = okc ? V.Ub_c[cb + k] + tb_cen(V, rb, cb, sc, 0, k) * idtg : FT(0);
    bREN[k] = okc ? V.Ub_c[cb + (size_t)3 * sc + k] + tb_cen(V, rb, cb, sc, 1, k) * idtg : FT(0);
    bU3N[k] = okf ? V.Ub_f[fb + k] + tb_face(V, fb, k) * idtg : FT(0);
    bU1[k] = FT(0);
    bU2[k] = FT(0);
  }
  // (a) van Leer minus central correction at the Newton result
  if (P.upwinding) {
    FT hn[CM], rJn[CM], cn1[CM], cn2[CM], Kn[CM];
    const FT U3Nn = nxt<G, CM>(U3N, gl);
    {
      FT Un[5][CM], wn[CM], gb[CM];
      col::Cen<FT> cc[CM];
#pragma unroll
      for (int k = 0; k < CM; ++k) {
        Un[0][k] = RN[k]; Un[1][k] = H[1][k]; Un[2][k] = H[2][k]; Un[3][k] = REN[k]; Un[4][k] = U3N[k];
        wn[k] = fnext(U3N, k, U3Nn);
        gb[k] = fnext(g33, k, g33n0);
      }
      col::cdiag_lane<FT, CM>(P, Gm, L, r0, Un, U3N, wn, g33, gb, cc);
#pragma unroll
      for (int k = 0; k < CM; ++k) {
        hn[k] = cc[k].h;
        rJn[k] = cc[k].rJ;
        Kn[k] = cc[k].K;
        cn1[k] = c1[k];
        cn2[k] = c2[k];
      }
    }
    const FT hnp = prv<G, CM>(hn, gl), hnp2 = prv2<G, CM>(hn, gl), hnn = nxt<G, CM>(hn, gl), hnn2 = nxt2<G, CM>(hn, gl);
    const FT rJnp = prv<G, CM>(rJn, gl);
    const FT bRENp = prv<G, CM>(bREN, gl), iJp = prv<G, CM>(iJ, gl);
    // contributions: h to levels f-2 .. f+1 (array index j + 2 -> level r0 + j), rJ to f-1, f
    FT accH[CM + 4], accR[CM + 2];
#pragma unroll
    for (int j = 0; j < CM + 4; ++j) accH[j] = FT(0);
#pragma unroll
    for (int j = 0; j < CM + 2; ++j) accR[j] = FT(0);
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const int f = r0 + k;
      if (!(f >= 1 && f < Nv)) continue;
      FT cbv = dtg * bREN[k] * iJ[k];
      cbv -= dtg * cprev(bREN, k, bRENp) * cprev(iJ, k, iJp);
      const FT u = U3N[k] * g33[k];
      const FT hA1 = k >= 1 ? hn[k - 1] : hnp;
      const FT hA2 = k >= 2 ? hn[k - 2] : (k == 1 ? hnp : hnp2);
      const FT h0 = hn[k], hP1 = k + 1 < CM ? hn[k + 1] : hnn;
      const FT rJb = (cprev(rJn, k, rJnp) + rJn[k]) / FT(2);
      const bool near = f == 1 || f == Nv - 1;
      const FT vl = vl_value(u, f >= 2 ? hA2 : FT(0), hA1, h0, f + 1 < Nv ? hP1 : FT(0), near, P.dt_model);
      FT du, dh[4];
      vl_grad(u, f >= 2 ? hA2 : FT(0), hA1, h0, f + 1 < Nv ? hP1 : FT(0), near, P.dt_model, du, dh);
      const FT hm = (hA1 + h0) / FT(2);
      const FT rJbb = cbv * vl - cbv * u * hm;
      accR[k] += rJbb / FT(2);      // level f - 1 (index k - 1 + 1)
      accR[k + 1] += rJbb / FT(2);  // level f
      bU3N[k] += (cbv * rJb * du - cbv * rJb * hm) * g33[k];
      if (f >= 2) accH[k] += cbv * rJb * dh[0];  // level f - 2 (index k - 2 + 2)
      accH[k + 1] += cbv * rJb * dh[1] - cbv * rJb * u / FT(2);
      accH[k + 2] += cbv * rJb * dh[2] - cbv * rJb * u / FT(2);
      if (f + 1 < Nv) accH[k + 3] += cbv * rJb * dh[3];
    }
    FT bHN[CM], bRJN[CM];
#pragma unroll
    for (int k = 0; k < CM; ++k) { bHN[k] = accH[k + 2]; bRJN[k] = accR[k + 1]; }
    fold2<G, CM>(bHN, accH[0], accH[1], accH[CM + 2], accH[CM + 3], gl);
    fold1<G, CM>(bRJN, accR[0], accR[CM + 1], gl);
    FT toNextU3 = FT(0);
    FT tvr[CM], tvre[CM], tvK[CM];
    thermo_vjp_lane<false>(P, RN, REN, Kn, phi, bHN, bHN, bHN, bHN, bHN, tvr, tvre, tvK);
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      if (r0 + k >= Nv) continue;
      const FT rb_ = tvr[k], reb = tvre[k], Kb = tvK[k];
      bRN[k] += rb_ + Jc[k] * bRJN[k];
      bREN[k] += reb;
      bU1[k] += cn1[k] * Kb;
      bU2[k] += cn2[k] * Kb;
      bU3N[k] += Kb * U3N[k] * g33[k] / FT(2);
      const FT cUp = Kb * fnext(U3N, k, U3Nn) * fnext(g33, k, g33n0) / FT(2);
      if (k + 1 < CM) bU3N[k + 1] += cUp; else toNextU3 = cUp;
    }
    fold1<G, CM>(bU3N, FT(0), toNextU3, gl);
  }
  // (b) back-substitution: U = U0 - dY
  FT bR0[CM], bRE0[CM], bRr[CM], bRe[CM], bru0[CM], bru1[CM], beu0[CM], beu1[CM], bX[CM], bU3[CM];
  {
    const FT bRNp = prv<G, CM>(bRN, gl), bRENp = prv<G, CM>(bREN, gl);
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const int f = r0 + k;
      const bool cv = f < Nv, inner = f > 0 && f < Nv;
      const FT xu = fnext(x, k, xn0);
      bR0[k] = cv ? bRN[k] : FT(0);
      bRE0[k] = cv ? bREN[k] : FT(0);
      bRr[k] = bR0[k];
      bRe[k] = bRE0[k];
      bru0[k] = -bR0[k] * x[k];
      bru1[k] = -bR0[k] * xu;
      beu0[k] = -bRE0[k] * x[k];
      beu1[k] = -bRE0[k] * xu;
      FT xb = FT(0);
      if (cv) xb -= bRN[k] * ru0[k] + bREN[k] * eu0[k];
      if (f >= 1 && f - 1 < Nv) xb -= cprev(bRN, k, bRNp) * cprev(ru1, k, ru1p) + cprev(bREN, k, bRENp) * cprev(eu1, k, eu1p);
      bU3[k] = FT(0);
      if (inner) {
        xb -= bU3N[k];
        bU3[k] = bU3N[k];
      }
      bX[k] = f < Nf ? xb : FT(0);
    }
  }
  // (c) transposed solve A^T dbar = xbar (sub C[f-1], diagonal B[f], super A[f+1])
  FT bD[CM];
  {
    const FT Scp = prv<G, CM>(Sc, gl), San = nxt<G, CM>(Sa, gl);
    FT a_[CM], b_[CM], c_[CM], d_[CM];
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const int f = r0 + k;
      a_[k] = f >= 1 ? cprev(Sc, k, Scp) : FT(0);
      b_[k] = Sb[k];
      c_[k] = f + 1 < Nf ? fnext(Sa, k, San) : FT(0);
      d_[k] = bX[k];
      if (f >= Nf) { a_[k] = FT(0); b_[k] = FT(1); c_[k] = FT(0); d_[k] = FT(0); }
    }
    col::solve_lanes<FT, G, CM>(a_, b_, c_, d_, bD, gl);
  }
  // (d) Schur rows, Jacobian entries, u_3 tendency
  FT bH4[CM], bK[CM], bH[CM], bPI[CM], bTHV[CM], bTHVR[CM], bPHIR[CM], bRJ[CM];
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    bH4[k] = bK[k] = bH[k] = bPI[k] = bTHV[k] = bTHVR[k] = bPHIR[k] = bRJ[k] = FT(0);
  }
  CSum<FT> dal;
  {
    // contributions to the centre below the face (f - 1) go to the previous level
    FT pR0 = 0, pK = 0, pTHV = 0, pTHVR = 0, pPI = 0, pPHIR = 0, pru0 = 0, pru1 = 0, peu0 = 0, peu1 = 0, pRr = 0, pRe = 0;
    FT toPrevU3 = 0, toNextU3 = 0;
    // this lane's own contributions accumulate straight into the cotangent arrays (no
    // separate accumulators live through the loop); those of the level below the lane's
    // first go to the previous lane (pXX) and are folded in after the loop
    FT (&cR0)[CM] = bR0, (&cK)[CM] = bK, (&cTHV)[CM] = bTHV, (&cTHVR)[CM] = bTHVR, (&cPI)[CM] = bPI;
    FT (&cPHIR)[CM] = bPHIR, (&cru0)[CM] = bru0, (&cru1)[CM] = bru1, (&ceu0)[CM] = beu0, (&ceu1)[CM] = beu1;
    FT (&cRr)[CM] = bRr, (&cRe)[CM] = bRe;
    const FT xpv = xp;
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const int f = r0 + k;
      if (f >= Nf) continue;
      const FT db = bD[k];
      const FT ab = f >= 1 ? -db * cprev(x, k, xpv) : FT(0);
      const FT bbb = -db * x[k];
      const FT cbb = f + 1 < Nf ? -db * fnext(x, k, xn0) : FT(0);
      FT ur0b = 0, ur1b = 0, ue0b = 0;
      // (scalar, u_3) rows of the centre below (f - 1): its index is k - 1 (this lane) or the previous lane's last
      auto addA = [&](FT (&arr)[CM], FT &pv, FT val) {
        if (k >= 1) arr[k - 1] += val; else pv += val;
      };
      if (f >= 1 && f - 1 < Nv) {
        ur0b += cprev(ru0, k, ru0p) * ab + cprev(ru1, k, ru1p) * bbb + cprev(Rr, k, Rrp) * db;
        ue0b += cprev(eu0, k, eu0p) * ab + cprev(eu1, k, eu1p) * bbb + cprev(Re, k, Rep) * db;
        addA(cru0, pru0, ur0[k] * ab);
        addA(cru1, pru1, ur0[k] * bbb);
        addA(ceu0, peu0, ue0[k] * ab);
        addA(ceu1, peu1, ue0[k] * bbb);
        addA(cRr, pRr, ur0[k] * db);
        addA(cRe, pRe, ue0[k] * db);
      }
      if (f < Nv) {
        ur1b += ru0[k] * bbb + ru1[k] * cbb + Rr[k] * db;
        ue0b -= eu0[k] * bbb + eu1[k] * cbb + Re[k] * db;
        cru0[k] += ur1[k] * bbb;
        cru1[k] += ur1[k] * cbb;
        ceu0[k] -= ue0[k] * bbb;
        ceu1[k] -= ue0[k] * cbb;
        cRr[k] += ur1[k] * db;
        cRe[k] -= ue0[k] * db;
      }
      const FT T3b = dtg * db;
      bH4[k] += db;
      bU3[k] -= db;
      bU3[k] -= beta[k] * T3b;
      dal.add(-mul_rn(spg[k] * u3[k], T3b));
      dal.add(-mul_rn(dtg * spg[k], bbb));
      if (!(f > 0 && f < Nv)) continue;
      // T3 = -(dPhi - (Phi_r(b) - Phi_r(a)) + cp thd (Pi(b) - Pi(a))) - beta u3
      const FT Pia = cprev(Pi, k, Pip), dPi = Pi[k] - Pia;
      const FT thva = cprev(thv, k, thvp), thvra = cprev(thvr, k, thvrp);
      const FT thd = ((thva - thvra) + (thv[k] - thvr[k])) / FT(2);
      cPHIR[k] += T3b;
      addA(cPHIR, pPHIR, -T3b);
      const FT thdb = -P.cpd * dPi * T3b;
      cPI[k] -= P.cpd * thd * T3b;
      addA(cPI, pPI, P.cpd * thd * T3b);
      addA(cTHV, pTHV, thdb / FT(2));
      addA(cTHVR, pTHVR, -thdb / FT(2));
      cTHV[k] += thdb / FT(2);
      cTHVR[k] -= thdb / FT(2);
      // Jacobian entries
      const FT uu0b = ab, uu1b = bbb, uu2b = cbb;
      const FT ra = cprev(H[0], k, rhop), rbv = H[0][k];
      const FT irb = FT(1) / ((ra + rbv) / FT(2));
      const FT dpa = kap * (P.T0 * P.cpd - cprev(K, k, Kp) - cprev(phi, k, phip));
      const FT dpb = kap * (P.T0 * P.cpd - K[k] - phi[k]);
      const FT thvb = (thva + thv[k]) / FT(2);
      const FT u3cm = cprev(u3, k, u3p) * cprev(g33, k, g33p), u3c = u3[k] * g33[k];
      const FT u3cp = fnext(u3, k, u3n0) * fnext(g33, k, g33n0);
      const FT dpab = dtg * irb * ur0b, dpbb = -dtg * irb * ur1b, buoyb = dtg * (ur0b + ur1b) / FT(2);
      FT irbb = dtg * (dpa * ur0b - dpb * ur1b) + dtg * kap * ue0b;
      irbb += dtg * (-kap * ra * u3cm / FT(2)) * uu0b + dtg * (kap * (rbv - ra) * u3c / FT(2)) * uu1b +
              dtg * (kap * rbv * u3cp / FT(2)) * uu2b;
      irbb += buoyb * P.cpd * thvb * dPi;
      const FT thvbb = buoyb * P.cpd * dPi * irb, dPib = buoyb * P.cpd * thvb * irb;
      const FT rbarb = -irb * irb * irbb;
      addA(cR0, pR0, dtg * (-kap * u3cm * irb / FT(2)) * uu0b - dtg * kap * u3c * irb / FT(2) * uu1b + rbarb / FT(2));
      cR0[k] += dtg * kap * u3c * irb / FT(2) * uu1b + dtg * kap * u3cp * irb / FT(2) * uu2b + rbarb / FT(2);
      const FT tp = dtg * (-kap * ra * irb / FT(2)) * uu0b * cprev(g33, k, g33p);
      if (k >= 1) bU3[k - 1] += tp; else toPrevU3 += tp;
      bU3[k] += dtg * kap * (rbv - ra) * irb / FT(2) * uu1b * g33[k];
      const FT tn = dtg * kap * rbv * irb / FT(2) * uu2b * fnext(g33, k, g33n0);
      if (k + 1 < CM) bU3[k + 1] += tn; else toNextU3 += tn;
      addA(cK, pK, -kap * dpab);
      cK[k] -= kap * dpbb;
      addA(cTHV, pTHV, thvbb / FT(2));
      cTHV[k] += thvbb / FT(2);
      cPI[k] += dPib;
      addA(cPI, pPI, -dPib);
    }
    fold1<G, CM>(cR0, pR0, FT(0), gl);
    fold1<G, CM>(cK, pK, FT(0), gl);
    fold1<G, CM>(cTHV, pTHV, FT(0), gl);
    fold1<G, CM>(cTHVR, pTHVR, FT(0), gl);
    fold1<G, CM>(cPI, pPI, FT(0), gl);
    fold1<G, CM>(cPHIR, pPHIR, FT(0), gl);
    fold1<G, CM>(cru0, pru0, FT(0), gl);
    fold1<G, CM>(cru1, pru1, FT(0), gl);
    fold1<G, CM>(ceu0, peu0, FT(0), gl);
    fold1<G, CM>(ceu1, peu1, FT(0), gl);
    fold1<G, CM>(cRr, pRr, FT(0), gl);
    fold1<G, CM>(cRe, pRe, FT(0), gl);
    fold1<G, CM>(bU3, toPrevU3, toNextU3, gl);
  }
  // (e) centre rows: contributions to the face cotangents of F, F h, fr, fhb at faces v, v+1
  FT bF[CM], bFh[CM], bfr[CM], bfhb[CM];
  {
    FT nF = 0, nFh = 0, nfr = 0, nfhb = 0;
#pragma unroll
    for (int k = 0; k < CM; ++k) bF[k] = bFh[k] = bfr[k] = bfhb[k] = FT(0);
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      if (r0 + k >= Nv) continue;
      const FT Trb = dtg * bRr[k], Teb = dtg * bRe[k];
      bF[k] += Trb * iJ[k];
      bFh[k] += Teb * iJ[k];
      bfr[k] += dtg * iJ[k] * bru0[k] + dtg * iJ[k] * fhb[k] * beu0[k];
      bfhb[k] += dtg * fr[k] * iJ[k] * beu0[k];
      const FT frU = fnext(fr, k, frn), fhbU = fnext(fhb, k, fhbn);
      const FT uF = -Trb * iJ[k], uFh = -Teb * iJ[k];
      const FT ufr = -(dtg * iJ[k] * bru1[k] + dtg * iJ[k] * fhbU * beu1[k]);
      const FT ufhb = -dtg * frU * iJ[k] * beu1[k];
      if (k + 1 < CM) { bF[k + 1] += uF; bFh[k + 1] += uFh; bfr[k + 1] += ufr; bfhb[k + 1] += ufhb; }
      else { nF = uF; nFh = uFh; nfr = ufr; nfhb = ufhb; }
    }
    fold1<G, CM>(bF, FT(0), nF, gl);
    fold1<G, CM>(bFh, FT(0), nFh, gl);
    fold1<G, CM>(bfr, FT(0), nfr, gl);
    fold1<G, CM>(bfhb, FT(0), nfhb, gl);
  }
  // (f) face fluxes F = rJb u3c, Fh = F hb, fr = rJb g33, fhb = hb -> rho J and h of the centres f-1, f
  {
    FT pH = 0, pRJ = 0;
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const int f = r0 + k;
      if (!(f > 0 && f < Nv)) continue;
      const FT rJb = (cprev(rJ, k, rJp) + rJ[k]) / FT(2), hb = fhb[k];
      const FT Fb = bF[k] + bFh[k] * hb;
      const FT hbb = bFh[k] * F[k] + bfhb[k];
      const FT rJbb = Fb * (u3[k] * g33[k]) + bfr[k] * g33[k];
      bU3[k] += Fb * rJb * g33[k];
      bH[k] += hbb / FT(2);
      bRJ[k] += rJbb / FT(2);
      if (k >= 1) { bH[k - 1] += hbb / FT(2); bRJ[k - 1] += rJbb / FT(2); }
      else { pH += hbb / FT(2); pRJ += rJbb / FT(2); }
    }
    fold1<G, CM>(bH, pH, FT(0), gl);
    fold1<G, CM>(bRJ, pRJ, FT(0), gl);
  }
  // (g) centre diagnostics of U0
  {
    FT toNextU3 = 0;
    FT tvr[CM], tvre[CM], tvK[CM];
    thermo_vjp_lane<true>(P, H[0], H[3], K, phi, bH, bPI, bTHV, bTHVR, bPHIR, tvr, tvre, tvK);
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      if (r0 + k >= Nv) continue;
      const FT rb_ = tvr[k], reb = tvre[k], Kb = tvK[k];
      bR0[k] += rb_ + Jc[k] * bRJ[k];
      bRE0[k] += reb;
      const FT Kt = Kb + bK[k];
      bU1[k] += c1[k] * Kt;
      bU2[k] += c2[k] * Kt;
      bU3[k] += Kt * u3[k] * g33[k] / FT(2);
      const FT cu = Kt * fnext(u3, k, u3n0) * fnext(g33, k, g33n0) / FT(2);
      if (k + 1 < CM) bU3[k + 1] += cu; else toNextU3 = cu;
    }
    fold1<G, CM>(bU3, FT(0), toNextU3, gl);
  }
  // ---------------------------------------------------------------- cotangent of U^ and its distribution
  // Per level, every load (the cotangents of u_n, U and T_imp and, when accumulating, those
  // of the earlier stages' tendencies) is issued before the first store: the stores may
  // alias later loads as far as the compiler knows, so interleaved they would serialise one
  // memory round trip per tendency.
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const int v = r0 + k;
    const bool cen = colv && v < Nv, fac = colv && v < Nf, acc = !V.init;
    FT y0[4] = {0, 0, 0, 0}, ub1 = 0, ub2 = 0, t0 = 0, t1 = 0, te[4][4], ti[4][2];
    FT yf = 0, tf = 0, tef[4], tif[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      tef[j] = tif[j] = ti[j][0] = ti[j][1] = FT(0);
#pragma unroll
      for (int c = 0; c < 4; ++c) te[j][c] = FT(0);
    }
    if (cen) {
#pragma unroll
      for (int c = 0; c < 4; ++c) y0[c] = V.Yb_c[cb + (size_t)c * sc + k];
      ub1 = V.Ub_c[cb + (size_t)sc + k];
      ub2 = V.Ub_c[cb + (size_t)2 * sc + k];
      t0 = tb_cen(V, rb, cb, sc, 0, k);
      t1 = tb_cen(V, rb, cb, sc, 1, k);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (!acc || j >= A.nsrc) continue;
#pragma unroll
        for (int c = 0; c < 4; ++c) te[j][c] = V.Teb_c[j][cb + (size_t)c * sc + k];
        if (j >= 1) {
          ti[j][0] = V.Tib_c[j][rb + k];
          ti[j][1] = V.Tib_c[j][rb + (size_t)sc + k];
        }
      }
    }
    if (fac) {
      yf = V.Yb_f[fb + k];
      tf = tb_face(V, fb, k);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (!acc || j >= A.nsrc) continue;
        tef[j] = V.Teb_f[j][fb + k];
        if (j >= 1) tif[j] = V.Tib_f[j][fb + k];
      }
    }
    if (cen) {
      const FT hb[4] = {bR0[k] - t0 * idtg, bU1[k] + ub1, bU2[k] + ub2, bRE0[k] - t1 * idtg};
#pragma unroll
      for (int c = 0; c < 4; ++c) V.Yb_c[cb + (size_t)c * sc + k] = y0[c] + hb[c];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (j >= A.nsrc) continue;
        const FT ke = acc ? FT(1) : V.e0[j], ki = acc ? FT(1) : V.i0[j];
#pragma unroll
        for (int c = 0; c < 4; ++c) V.Teb_c[j][cb + (size_t)c * sc + k] = (acc ? te[j][c] : ke * y0[c]) + A.ce[j] * hb[c];
        if (j >= 1) {
          V.Tib_c[j][rb + k] = (acc ? ti[j][0] : ki * y0[0]) + A.ci[j] * hb[0];
          V.Tib_c[j][rb + (size_t)sc + k] = (acc ? ti[j][1] : ki * y0[3]) + A.ci[j] * hb[3];
        }
      }
    }
    if (fac) {
      const bool inner = v > 0 && v < Nv;
      const FT hb = bH4[k] + (inner ? bU3[k] : FT(0)) - tf * idtg;
      V.Yb_f[fb + k] = yf + hb;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (j >= A.nsrc) continue;
        V.Teb_f[j][fb + k] = (acc ? tef[j] : V.e0[j] * yf) + A.ce[j] * hb;
        if (j >= 1) V.Tib_f[j][fb + k] = (acc ? tif[j] : V.i0[j] * yf) + A.ci[j] * hb;
      }
    }
  }
  col::group_sum1<G>(dal);
  if (gl == 0 && colv) RSlot<FT>::put(&V.dalpha[col], dal, false);
}

}  // namespace lp

}  // namespace

size_t col_vjp_scratch_words(int Nh, int Nv) { return (size_t)S_NUM * (Nv + 1) * (size_t)Nh * NN; }

template <class FT>
void launch_column_stage_vjp(const DevParams<FT> &P, const StageArgs<FT> &A, const FT *Ub_c, const FT *Ub_f,
                             const FT *Tb_c, const FT *Tb_f, FT *Yb_c, FT *Yb_f, FT *const Teb[4], FT *const Tib[4],
                             size_t NC, size_t NR, FT *scr, double *dalpha, cudaStream_t s, const FT *Uo,
                             const FT *Tio, const FT *e0, const FT *i0, const FT *tbs) {
  ColVjpArgs<FT> V{};
  V.A = A;
  if (tbs) {
    V.tby = 1;
    V.tbs = *tbs;
  }
  if (e0 && i0) {
    V.init = 1;
    for (int j = 0; j < 4; ++j) {
      V.e0[j] = e0[j];
      V.i0[j] = i0[j];
    }
  }
  if (Uo && Tio) {
    V.Uo_c = Uo; V.Uo_f = Uo + NC; V.Tio_c = Tio; V.Tio_f = Tio + NR;
  }
  V.Ub_c = Ub_c; V.Ub_f = Ub_f; V.Tb_c = Tb_c; V.Tb_f = Tb_f; V.Yb_c = Yb_c; V.Yb_f = Yb_f;
  for (int j = 0; j < 4; ++j) {
    V.Teb_c[j] = Teb[j];
    V.Teb_f[j] = Teb[j] ? Teb[j] + NC : nullptr;
    V.Tib_c[j] = Tib[j];
    V.Tib_f[j] = Tib[j] ? Tib[j] + NR : nullptr;
  }
  V.scr = scr;
  V.dalpha = dalpha;
  const int ncols = P.Nh * NN;
  // lane-parallel form by default; GBDYCORE_COLUMN_VJP=serial selects the one-thread-per-column form
  static const bool serial = [] {
    const char *e = getenv("GBDYCORE_COLUMN_VJP");
    return e && e[0] == 's';
  }();
  if (serial) {
    k_col_stage_vjp<FT><<<(ncols + 127) / 128, 128, 0, s>>>(P, V);
    return;
  }
  auto grid = [&](int G) { return (ncols + 4 * (32 / G) - 1) / (4 * (32 / G)); };
  auto go = [&](auto rec) {
    constexpr bool R = decltype(rec)::value;
    constexpr int M6 = sizeof(FT) == 4 ? 6 : 1;
    constexpr int MD = lp::VjpMinBlocks<FT>::value;
    if (P.Nf <= 16) lp::k_col_stage_vjp_g<FT, 8, 2, MD, R><<<grid(8), 128, 0, s>>>(P, V);
    else if (P.Nf <= 32) lp::k_col_stage_vjp_g<FT, 16, 2, MD, R><<<grid(16), 128, 0, s>>>(P, V);
    // FP32, two levels per lane: six resident CTAs per SM (an 85-register cap; measured at
    // z_elem = 63: 0.531 ms at 4 CTAs, 0.518 at 5, 0.506 at 6, 0.516 at 7, 0.571 at 8)
    else if (P.Nf <= 64) lp::k_col_stage_vjp_g<FT, 32, 2, M6, R><<<grid(32), 128, 0, s>>>(P, V);
    else lp::k_col_stage_vjp_g<FT, 32, 4, MD, R><<<grid(32), 128, 0, s>>>(P, V);
  };
  if (V.Uo_c) go(std::true_type{});
  else go(std::false_type{});
}

template void launch_column_stage_vjp<float>(const DevParams<float> &, const StageArgs<float> &, const float *,
                                             const float *, const float *, const float *, float *, float *,
                                             float *const[4], float *const[4], size_t, size_t, float *, double *,
                                             cudaStream_t, const float *, const float *, const float *,
                                             const float *, const float *);
template void launch_column_stage_vjp<double>(const DevParams<double> &, const StageArgs<double> &, const double *,
                                              const double *, const double *, const double *, double *, double *,
                                              double *const[4], double *const[4], size_t, size_t, double *,
                                              double *, cudaStream_t, const double *, const double *,
                                              const double *, const double *, const double *);

}  // namespace gb
