// Column kernel of the implicit vertical-acoustic solve: one warp per column,
// each lane owning M consecutive levels (level index = lane*M + k, centre and
// face of the same index, the face below the centre).
//
// COL_STAGE fuses, for one implicit ARS343 stage, what ClimaTimeSteppers does
// through the hooks (src/simulation/integrator.jl:189-225):
//   stage assembly U^ = u_n + dt sum_j (a~_ij T_exp_j + a_ij T_imp_j),
//   set_implicit_precomputed_quantities! (precomputed_quantities.jl:698-831,
//     impenetrable filter :486-553),
//   implicit_tendency! (implicit_tendency.jl:185-298) -> residual
//     R = U^ + dtgamma T_imp(U) - U,
//   update_jacobian! (manual_sparse_jacobian.jl:713-870, dry, no topography),
//   ldiv! with BlockArrowheadSolve(rho, rho e_tot; alg2 = u_h)
//     (manual_sparse_jacobian.jl:580-583): Schur complement onto u_3 (a
//     tridiagonal face system), solved by parallel cyclic reduction across
//     the warp, then back-substitution for rho and rho e_tot,
//   U -= dY; filter; correct_implicit_advection_tendency! (van Leer minus
//     central, implicit_tendency.jl:322-339) applied as U += dtgamma * corr,
//   T_imp_i = (U - U^) / dtgamma, and the FP64 residual sums of squares.
// The other modes are the individual hooks.
#include <type_traits>

#include "colcore.cuh"

namespace gb {

namespace {

constexpr int COL_THREADS = 128;  // 4 columns per CTA

// value of x at level (own level + D) for the compile-time slot K
template <int M, int K, int D, class FT>
__device__ __forceinline__ FT nb(const FT (&x)[M]) {
  constexpr int kk = K + D;
  if constexpr (kk >= 0 && kk < M) {
    return x[kk];
  } else if constexpr (kk < 0) {
    constexpr int L = (-kk + M - 1) / M;
    return shfl_up(x[kk + L * M], L);
  } else {
    constexpr int L = kk / M;
    return shfl_down(x[kk - L * M], L);
  }
}

template <int M, int D, class FT>
__device__ __forceinline__ void nb_all(const FT (&x)[M], FT (&o)[M]) {
  if constexpr (M >= 1) o[0] = nb<M, 0, D>(x);
  if constexpr (M >= 2) o[1] = nb<M, 1, D>(x);
  if constexpr (M >= 3) o[2] = nb<M, 2, D>(x);
  if constexpr (M >= 4) o[3] = nb<M, 3, D>(x);
}

// Parallel cyclic reduction of the 32*M-row tridiagonal system held by the warp
// (rows outside the column are identity rows).  Leaves x = d / b.
template <class FT, int M, int S>
__device__ __forceinline__ void pcr_level(FT (&a)[M], FT (&b)[M], FT (&c)[M], FT (&d)[M], int lane) {
  FT am[M], bm[M], cm[M], dm[M], ap[M], bp[M], cp[M], dp[M];
  nb_all<M, -S>(a, am); nb_all<M, -S>(b, bm); nb_all<M, -S>(c, cm); nb_all<M, -S>(d, dm);
  nb_all<M, S>(a, ap); nb_all<M, S>(b, bp); nb_all<M, S>(c, cp); nb_all<M, S>(d, dp);
#pragma unroll
  for (int k = 0; k < M; ++k) {
    const int r = lane * M + k;
    const bool hm = r - S >= 0, hp = r + S < 32 * M;
    const FT al = hm ? -gdiv(a[k], bm[k]) : FT(0);
    const FT ga = hp ? -gdiv(c[k], bp[k]) : FT(0);
    const FT na = hm ? al * am[k] : FT(0);
    const FT nc = hp ? ga * cp[k] : FT(0);
    FT nbv = b[k], ndv = d[k];
    if (hm) { nbv += al * cm[k]; ndv += al * dm[k]; }
    if (hp) { nbv += ga * ap[k]; ndv += ga * dp[k]; }
    a[k] = na; b[k] = nbv; c[k] = nc; d[k] = ndv;
  }
}

template <class FT, int M>
__device__ __forceinline__ void pcr_solve(FT (&a)[M], FT (&b)[M], FT (&c)[M], FT (&d)[M], FT (&x)[M], int lane) {
  pcr_level<FT, M, 1>(a, b, c, d, lane);
  pcr_level<FT, M, 2>(a, b, c, d, lane);
  pcr_level<FT, M, 4>(a, b, c, d, lane);
  pcr_level<FT, M, 8>(a, b, c, d, lane);
  pcr_level<FT, M, 16>(a, b, c, d, lane);
  if constexpr (M >= 2) pcr_level<FT, M, 32>(a, b, c, d, lane);
  if constexpr (M >= 4) pcr_level<FT, M, 64>(a, b, c, d, lane);
#pragma unroll
  for (int k = 0; k < M; ++k) x[k] = gdiv(d[k], b[k]);
}

// Two rows per lane: one cyclic-reduction level eliminates the odd rows
// (row 2l-1 comes from the previous lane), parallel cyclic reduction solves
// the 32 even rows across the warp, and the odd rows are back-substituted.
template <class FT>
__device__ __forceinline__ void crpcr_solve2(FT (&a)[2], FT (&b)[2], FT (&c)[2], FT (&d)[2], FT (&x)[2], int lane) {
  const FT ap = shfl_up(a[1], 1), bp = shfl_up(b[1], 1), cp = shfl_up(c[1], 1), dp = shfl_up(d[1], 1);
  const bool hm0 = lane > 0;
  const FT al0 = hm0 ? -gdiv(a[0], bp) : FT(0);
  const FT ga0 = -gdiv(c[0], b[1]);
  FT A = hm0 ? al0 * ap : FT(0);
  FT C = ga0 * c[1];
  FT B = b[0] + ga0 * a[1];
  FT Dd = d[0] + ga0 * d[1];
  if (hm0) { B += al0 * cp; Dd += al0 * dp; }
#pragma unroll
  for (int s = 1; s < 32; s <<= 1) {
    const FT Am = shfl_up(A, s), Bm = shfl_up(B, s), Cm = shfl_up(C, s), Dm = shfl_up(Dd, s);
    const FT Ap = shfl_down(A, s), Bp = shfl_down(B, s), Cp = shfl_down(C, s), Dp = shfl_down(Dd, s);
    const bool hm = lane >= s, hp = lane + s < 32;
    const FT al = hm ? -gdiv(A, Bm) : FT(0);
    const FT ga = hp ? -gdiv(C, Bp) : FT(0);
    FT nB = B, nD = Dd;
    if (hm) { nB += al * Cm; nD += al * Dm; }
    if (hp) { nB += ga * Ap; nD += ga * Dp; }
    A = hm ? al * Am : FT(0);
    C = hp ? ga * Cp : FT(0);
    B = nB;
    Dd = nD;
  }
  const FT xe = gdiv(Dd, B);
  const FT xn = shfl_down(xe, 1);
  x[0] = xe;
  x[1] = gdiv(d[1] - a[1] * xe - (lane < 31 ? c[1] * xn : FT(0)), b[1]);
}

// Column-local thermodynamic state at the owned levels.
template <class FT, int M>
struct ColState {
  FT rho[M], u1[M], u2[M], rhoe[M], u3[M];
  FT rhoq[M];  // moist 0M: rho q_tot
};
// Over terrain-following levels (TOPO) also: w3c = g^33 u_3 of the faces (u3c is then the full
// u^3 = u_h^3 + g^33 u_3), ct3 = CT3(u_h) of the centres, the face's g^33 and the centre's Phi.
template <class FT, int M>
struct ColDiag {
  FT c1[M], c2[M], K[M], T[M], h[M], Pi[M], thv[M], thvr[M], phid[M], rJ[M], u3c[M], J[M], iJ[M];
  FT w3c[M], ct3[M], g33[M], phi[M];
  // moist 0M: q = specific(rho q_tot, rho), kappa_m, dp/d(rho q_tot)
  FT q[M], km[M], dpq[M];
};

// The impenetrable filter over terrain on a state held M levels per lane: u_3 = -CT3(u_h) / g^33
// of the adjacent centre on the bottom and top faces, 0 beyond the column.
template <class FT, int M>
__device__ __forceinline__ void col_filter_topo(const col::ColLevT<FT> &T, ColState<FT, M> &S, int lane) {
  const int Nv = T.Nv, Nf = T.Nf;
  FT ct3[M], ctm[M];
#pragma unroll
  for (int k = 0; k < M; ++k) {
    const int v = min(lane * M + k, Nv - 1);
    FT g31, g32, phis;
    T.ct(v, g31, g32, phis);
    ct3[k] = g31 * S.u1[k] + g32 * S.u2[k];
  }
  nb_all<M, -1>(ct3, ctm);
#pragma unroll
  for (int k = 0; k < M; ++k) {
    const int f = lane * M + k;
    if (f == 0) S.u3[k] = -ct3[k] / T.f4(0).x;
    else if (f == Nv) S.u3[k] = -ctm[k] / T.f4(Nv).x;
    else if (f > Nv) S.u3[k] = FT(0);
  }
  (void)Nf;
}

template <class FT, int M, bool TOPO, bool MOIST, class LV>
__device__ __forceinline__ void col_diag(const DevParams<FT> &P, const ColGeo<FT> &G, const LV &T,
                                         const ColState<FT, M> &S, ColDiag<FT, M> &Dg, int lane) {
  const int Nv = P.Nv, Nf = P.Nf;
#pragma unroll
  for (int k = 0; k < M; ++k) {
    const int f = min(lane * M + k, Nf - 1);
    if constexpr (TOPO) {
      Dg.g33[k] = T.f4(f).x;
      Dg.w3c[k] = S.u3[k] * Dg.g33[k];
    } else {
      Dg.u3c[k] = S.u3[k] * P.levf[LF_G33 * Nf + f];
    }
  }
  FT u3n[M], u3cn[M];
  nb_all<M, 1>(S.u3, u3n);
  nb_all<M, 1>(TOPO ? Dg.w3c : Dg.u3c, u3cn);
#pragma unroll
  for (int k = 0; k < M; ++k) {
    const int v = min(lane * M + k, Nv - 1);
    if constexpr (TOPO) {
      // the column's own metric; K takes 2 CT3(u_h) I^c(u_3) (compute_kinetic, utilities.jl:194-206)
      // and CT12(ᶜu) takes g^a3 I^c(u_3)
      FT g31, g32, phis;
      const Lev4<FT> c4 = T.c4ct(v, g31, g32, phis);
      const FT gu0 = G.gu0 * c4.z, gu1 = G.gu1 * c4.z, gu2 = G.gu2 * c4.z;
      const FT h1 = gu0 * S.u1[k] + gu1 * S.u2[k], h2 = gu1 * S.u1[k] + gu2 * S.u2[k];
      const FT ct3 = g31 * S.u1[k] + g32 * S.u2[k], ub3 = (S.u3[k] + u3n[k]) / FT(2);
      const FT kv = (S.u3[k] * Dg.w3c[k] + u3n[k] * u3cn[k]) / FT(2);
      const FT K = (S.u1[k] * h1 + S.u2[k] * h2 + kv + FT(2) * ct3 * ub3) / FT(2);
      Thermo<FT> th;
      thermo(P, S.rho[k], S.rhoe[k], K, c4.w, P.lr4[v], th);
      Dg.c1[k] = h1 + g31 * ub3; Dg.c2[k] = h2 + g32 * ub3; Dg.K[k] = K; Dg.T[k] = th.T; Dg.h[k] = th.h;
      Dg.Pi[k] = th.Pi; Dg.thv[k] = th.thv; Dg.thvr[k] = th.thvr; Dg.phid[k] = th.phid + phis;
      Dg.ct3[k] = ct3;
      Dg.phi[k] = c4.w;
      Dg.J[k] = G.Jh * c4.x;
      Dg.iJ[k] = G.iJh * c4.y;
      Dg.rJ[k] = S.rho[k] * Dg.J[k];
    } else {
      const FT r2 = P.levc[LC_R2 * Nv + v], dz = P.levc[LC_DZ * Nv + v], Phi = P.levc[LC_PHI * Nv + v];
      const FT ir2 = P.levc[LC_IR2 * Nv + v];
      const FT gu0 = G.gu0 * ir2, gu1 = G.gu1 * ir2, gu2 = G.gu2 * ir2;
      const FT c1 = gu0 * S.u1[k] + gu1 * S.u2[k], c2 = gu1 * S.u1[k] + gu2 * S.u2[k];
      const FT kv = (S.u3[k] * Dg.u3c[k] + u3n[k] * u3cn[k]) / FT(2);
      const FT K = (S.u1[k] * c1 + S.u2[k] * c2 + kv) / FT(2);
      Thermo<FT> th;
      if constexpr (MOIST) thermo_moist(P, S.rho[k], S.rhoe[k], S.rhoq[k], K, Phi, P.lr4[v], th, Dg.q[k], Dg.km[k], Dg.dpq[k]);
      else thermo(P, S.rho[k], S.rhoe[k], K, Phi, P.lr4[v], th);
      Dg.c1[k] = c1; Dg.c2[k] = c2; Dg.K[k] = K; Dg.T[k] = th.T; Dg.h[k] = th.h; Dg.Pi[k] = th.Pi;
      Dg.thv[k] = th.thv; Dg.thvr[k] = th.thvr; Dg.phid[k] = th.phid;
      Dg.J[k] = G.Jh * r2 * dz;
      Dg.iJ[k] = G.iJh * ir2 * P.levc[LC_IDZ * Nv + v];
      Dg.rJ[k] = S.rho[k] * Dg.J[k];
    }
  }
  if constexpr (TOPO) {
    // u^3 = ᶠwinterp(rho J, CT3(u_h)) + g^33 u_3 (the adjacent centre's CT3 on the boundary faces)
    FT rJm[M], ctm[M];
    nb_all<M, -1>(Dg.rJ, rJm);
    nb_all<M, -1>(Dg.ct3, ctm);
#pragma unroll
    for (int k = 0; k < M; ++k) {
      const int f = lane * M + k;
      FT uh3;
      if (f == 0) uh3 = Dg.ct3[k];
      else if (f >= Nv) uh3 = ctm[k];
      else uh3 = (rJm[k] * ctm[k] + Dg.rJ[k] * Dg.ct3[k]) / (rJm[k] + Dg.rJ[k]);
      Dg.u3c[k] = uh3 + Dg.w3c[k];
    }
  }
}

// implicit tendency (rho, rho e_tot, u_3; moist: rho q_tot) at the owned levels
template <class FT, int M, bool TOPO, bool MOIST, class LV>
__device__ __forceinline__ void col_implicit(const DevParams<FT> &P, const ColGeo<FT> &G, const LV &Tg,
                                             const ColState<FT, M> &S, const ColDiag<FT, M> &Dg, FT (&Tr)[M],
                                             FT (&Te)[M], FT (&T3)[M], FT (&Tq)[M], int lane) {
  const int Nv = P.Nv, Nf = P.Nf;
  FT rJm[M], hm[M], phm[M], Pim[M], thm[M], thrm[M], qm[M];
  nb_all<M, -1>(Dg.rJ, rJm); nb_all<M, -1>(Dg.h, hm); nb_all<M, -1>(Dg.phid, phm);
  nb_all<M, -1>(Dg.Pi, Pim); nb_all<M, -1>(Dg.thv, thm); nb_all<M, -1>(Dg.thvr, thrm);
  if constexpr (MOIST) nb_all<M, -1>(Dg.q, qm);
  FT flux[M], fh[M], fq[M];
#pragma unroll
  for (int k = 0; k < M; ++k) {
    const int f = lane * M + k;
    const bool inner = f > 0 && f < Nv;
    const int fc = min(f, Nf - 1);
    const FT rJ = (rJm[k] + Dg.rJ[k]) / FT(2);
    const FT F = rJ * Dg.u3c[k];   // ᶜadvdivᵥ(ᶠinterp(ρJ)/ᶠJ u³): the face Jacobian cancels
    const FT hb = (hm[k] + Dg.h[k]) / FT(2);
    flux[k] = inner ? F : FT(0);
    fh[k] = inner ? F * hb : FT(0);
    // central transport of q_tot (implicit_tendency.jl:211-215)
    if constexpr (MOIST) fq[k] = inner ? F * ((qm[k] + Dg.q[k]) / FT(2)) : FT(0);
    FT val = 0;
    if (inner) {
      // ᶠgradᵥ(Phi) - ᶠgradᵥ(Phi_r) as the difference of Phi - Phi_r between the levels
      const FT gPhid = Dg.phid[k] - phm[k];
      const FT thd = ((thm[k] - thrm[k]) + (Dg.thv[k] - Dg.thvr[k])) / FT(2);
      const FT gPi = Dg.Pi[k] - Pim[k];
      val = -(gPhid + P.cpd * thd * gPi);
    }
    if constexpr (TOPO) val -= Tg.f4(fc).y * S.u3[k];
    else val -= P.levf[LF_BETA * Nf + fc] * S.u3[k];
    T3[k] = val;
  }
  FT fln[M], fhn[M], fqn[M];
  nb_all<M, 1>(flux, fln);
  nb_all<M, 1>(fh, fhn);
  if constexpr (MOIST) nb_all<M, 1>(fq, fqn);
#pragma unroll
  for (int k = 0; k < M; ++k) {
    Tr[k] = -((fln[k] - flux[k]) * Dg.iJ[k]);
    Te[k] = -((fhn[k] - fh[k]) * Dg.iJ[k]);
    Tq[k] = MOIST ? -((fqn[k] - fq[k]) * Dg.iJ[k]) : FT(0);
  }
}

// Jacobian blocks at the owned levels (centre rows: Mru/Meu for faces v, v+1;
// face rows: Mur/Mue/Muh for centres k-1, k, Muu for faces k-1, k, k+1).
// Over terrain six more quantities per centre v carry the (rho, u_h) and (rho e_tot, u_h) blocks
// (manual_sparse_jacobian.jl:150-187, 745-786): the interior face k's flux rho-bar J u^3 holds
// 1/2 sum_c rho_c J_c CT3(u_h)_c over its two centres, so with ct_c = g^31_c x_1,c + g^32_c x_2,c
//   d(rho_t)_v . x   = dtγ [hm (ct_{v-1} + ... ) ...] = wm ct_{v-1} + (w0m - w0p) ct_v - wp ct_{v+1}
//   d(rhoe_t)_v . x  = hb0 (wm ct_{v-1} + w0m ct_v) - hb1 (w0p ct_v + wp ct_{v+1})
// with wm = dtγ rho_{v-1} J_{v-1} / (2 J_v) (face v interior), w0m = dtγ rho_v / 2 (face v
// interior), w0p = dtγ rho_v / 2 (face v+1 interior), wp = dtγ rho_{v+1} J_{v+1} / (2 J_v) (face
// v+1 interior), hb0, hb1 the face means of h_tot; g^3a is geometry and is recomputed where used.
template <class FT, int M>
struct ColJac {
  FT ru0[M], ru1[M], eu0[M], eu1[M];
  FT ur0[M], ur1[M], ue0[M], ue1[M], uh0[M], uh1[M], uh2[M], uh3[M], uu0[M], uu1[M], uu2[M];
  FT wm[M], w0m[M], w0p[M], wp[M], hb0[M], hb1[M];
  // moist 0M: (rho q_tot, u_3) of centre v for faces v, v+1 and (u_3, rho q_tot) of face k for
  // centres k-1, k
  FT qu0[M], qu1[M], uq0[M], uq1[M];
};

// Moist 0M (manual_sparse_jacobian.jl:646-685, 770-831): kappa_m of each centre replaces the
// dry R_d / cv_d, dp/drho gains (R_d - kappa_m cv_d) T, and the (rho q_tot, u_3) and
// (u_3, rho q_tot) blocks are the (rho e_tot, u_3) block with ᶠinterp(q_tot) and the
// (u_3, rho e_tot) block with dp/d(rho q_tot).
template <class FT, int M, bool TOPO, bool MOIST, class LV>
__device__ __forceinline__ void col_jacobian(const DevParams<FT> &P, const ColGeo<FT> &G, const LV &Tg,
                                             const ColState<FT, M> &S, const ColDiag<FT, M> &Dg, FT dtg,
                                             ColJac<FT, M> &Jc, int lane) {
  const int Nv = P.Nv, Nf = P.Nf;
  const FT kap = P.Rd * P.icvd;
  FT rJm[M], hm[M], rhom[M], Km[M], thm[M], Pim[M], c1m[M], c2m[M], u3cm[M], u3cp[M];
  nb_all<M, -1>(Dg.rJ, rJm); nb_all<M, -1>(Dg.h, hm); nb_all<M, -1>(S.rho, rhom); nb_all<M, -1>(Dg.K, Km);
  nb_all<M, -1>(Dg.thv, thm); nb_all<M, -1>(Dg.Pi, Pim); nb_all<M, -1>(Dg.c1, c1m); nb_all<M, -1>(Dg.c2, c2m);
  // (u_3, u_3) uses g^33 u_3 of the neighbouring faces (u3c over a flat surface, w3c over terrain)
  nb_all<M, -1>(TOPO ? Dg.w3c : Dg.u3c, u3cm); nb_all<M, 1>(TOPO ? Dg.w3c : Dg.u3c, u3cp);
  FT ctm[M], phim[M];
  if constexpr (TOPO) {
    nb_all<M, -1>(Dg.ct3, ctm);
    nb_all<M, -1>(Dg.phi, phim);
  }
  FT kmm[M], Tmm[M], dqm[M], qm[M];
  if constexpr (MOIST) {
    nb_all<M, -1>(Dg.km, kmm); nb_all<M, -1>(Dg.T, Tmm); nb_all<M, -1>(Dg.dpq, dqm); nb_all<M, -1>(Dg.q, qm);
  }
  // face quantities needed by centre rows: rJbar*g33 and hbar at faces
  FT fr[M], fhb[M], fqb[M];
#pragma unroll
  for (int k = 0; k < M; ++k) {
    const int f = lane * M + k;
    const bool inner = f > 0 && f < Nv;
    const int fc = min(f, Nf - 1);
    const FT g33 = TOPO ? Dg.g33[k] : P.levf[LF_G33 * Nf + fc];
    const FT rJ = (rJm[k] + Dg.rJ[k]) / FT(2);
    fr[k] = inner ? rJ * g33 : FT(0);
    fhb[k] = (hm[k] + Dg.h[k]) / FT(2);
    if constexpr (MOIST) fqb[k] = (qm[k] + Dg.q[k]) / FT(2);
  }
  FT frn[M], fhbn[M], fqbn[M];
  nb_all<M, 1>(fr, frn);
  nb_all<M, 1>(fhb, fhbn);
  if constexpr (MOIST) nb_all<M, 1>(fqb, fqbn);
#pragma unroll
  for (int k = 0; k < M; ++k) {
    const FT v0 = fr[k] * Dg.iJ[k], v1 = -frn[k] * Dg.iJ[k];
    Jc.ru0[k] = dtg * v0;
    Jc.ru1[k] = dtg * v1;
    Jc.eu0[k] = dtg * (v0 * fhb[k]);
    Jc.eu1[k] = dtg * (v1 * fhbn[k]);
    if constexpr (MOIST) {
      Jc.qu0[k] = dtg * (v0 * fqb[k]);
      Jc.qu1[k] = dtg * (v1 * fqbn[k]);
    }
    const int f = lane * M + k;
    const int fc = min(f, Nf - 1);
    const FT beta = TOPO ? Tg.f4(fc).y : P.levf[LF_BETA * Nf + fc];
    if (f > 0 && f < Nv) {
      const int va = f - 1;
      const FT ra = rhom[k], rb = S.rho[k];
      const FT rbar = (ra + rb) / FT(2);
      const FT irb = grcp(rbar);
      const FT phia = TOPO ? phim[k] : P.levc[LC_PHI * Nv + va], phib = TOPO ? Dg.phi[k] : P.levc[LC_PHI * Nv + f];
      // kappa_m of the centres below (a) and above (b) the face: R_d / cv_d for dry air
      const FT ka = MOIST ? kmm[k] : kap, kb = MOIST ? Dg.km[k] : kap;
      FT dpa = ka * (P.T0 * P.cpd - Km[k] - phia);
      FT dpb = kb * (P.T0 * P.cpd - Dg.K[k] - phib);
      if constexpr (MOIST) {
        dpa += (P.Rd - ka * P.cvd) * Tmm[k];
        dpb += (P.Rd - kb * P.cvd) * Dg.T[k];
        Jc.uq0[k] = dtg * (dqm[k] * irb);
        Jc.uq1[k] = dtg * (-Dg.dpq[k] * irb);
      }
      const FT thvb = (thm[k] + Dg.thv[k]) / FT(2);
      const FT gPi = Dg.Pi[k] - Pim[k];
      const FT buoy = P.cpd * thvb * gPi * irb;
      Jc.ur0[k] = dtg * (dpa * irb + buoy / FT(2));
      Jc.ur1[k] = dtg * (-dpb * irb + buoy / FT(2));
      Jc.ue0[k] = dtg * (ka * irb);
      Jc.ue1[k] = dtg * (-kb * irb);
      Jc.uh0[k] = dtg * (-ka * ra * irb) * c1m[k];
      Jc.uh1[k] = dtg * (-ka * ra * irb) * c2m[k];
      Jc.uh2[k] = dtg * (kb * rb * irb) * Dg.c1[k];
      Jc.uh3[k] = dtg * (kb * rb * irb) * Dg.c2[k];
      if constexpr (TOPO) {
        // dK_v/du_3,f = (g^33 u_3)_f / 2 + CT3(u_h)_v / 2 (manual_sparse_jacobian.jl:754-756)
        Jc.uu0[k] = dtg * (-kap * ra * (u3cm[k] + ctm[k]) * (irb / FT(2)));
        Jc.uu1[k] = dtg * (kap * (rb * (Dg.w3c[k] + Dg.ct3[k]) - ra * (Dg.w3c[k] + ctm[k])) * (irb / FT(2)) - beta) - FT(1);
        Jc.uu2[k] = dtg * (kap * rb * (u3cp[k] + Dg.ct3[k]) * (irb / FT(2)));
      } else if constexpr (MOIST) {
        Jc.uu0[k] = dtg * (-ka * ra * u3cm[k] * (irb / FT(2)));
        Jc.uu1[k] = dtg * ((kb * rb - ka * ra) * Dg.u3c[k] * (irb / FT(2)) - beta) - FT(1);
        Jc.uu2[k] = dtg * (kb * rb * u3cp[k] * (irb / FT(2)));
      } else {
        Jc.uu0[k] = dtg * (-kap * ra * u3cm[k] * (irb / FT(2)));
        Jc.uu1[k] = dtg * (kap * (rb - ra) * Dg.u3c[k] * (irb / FT(2)) - beta) - FT(1);
        Jc.uu2[k] = dtg * (kap * rb * u3cp[k] * (irb / FT(2)));
      }
    } else {
      if constexpr (MOIST) Jc.uq0[k] = Jc.uq1[k] = FT(0);
      Jc.ur0[k] = Jc.ur1[k] = Jc.ue0[k] = Jc.ue1[k] = FT(0);
      Jc.uh0[k] = Jc.uh1[k] = Jc.uh2[k] = Jc.uh3[k] = FT(0);
      Jc.uu0[k] = Jc.uu2[k] = FT(0);
      Jc.uu1[k] = f <= Nv ? -dtg * beta - FT(1) : FT(1);  // identity rows beyond the column
    }
  }
  if constexpr (TOPO) {
    FT rJp[M], hp[M];
    nb_all<M, 1>(Dg.rJ, rJp);
    nb_all<M, 1>(Dg.h, hp);
#pragma unroll
    for (int k = 0; k < M; ++k) {
      const int v = lane * M + k;
      const bool lo = v >= 1 && v < Nv, hi = v + 1 <= Nv - 1;
      const FT half = dtg / FT(2);
      Jc.wm[k] = lo ? half * rJm[k] * Dg.iJ[k] : FT(0);
      Jc.w0m[k] = lo ? half * S.rho[k] : FT(0);
      Jc.w0p[k] = hi ? half * S.rho[k] : FT(0);
      Jc.wp[k] = hi ? half * rJp[k] * Dg.iJ[k] : FT(0);
      Jc.hb0[k] = (hm[k] + Dg.h[k]) / FT(2);
      Jc.hb1[k] = (Dg.h[k] + hp[k]) / FT(2);
    }
  }
}

// Solve W dY = R with the Schur complement onto u_3.  Moist 0M: the rho q_tot row is a third
// scalar row with a -I diagonal block, as rho and rho e_tot (the reference's
// ApproximateBlockArrowheadIterativeSolve, manual_sparse_jacobian.jl:539-584, is then exact in
// its first preconditioner application).
template <class FT, int M, bool TOPO, bool MOIST, class LV>
__device__ __forceinline__ void col_ldiv(const DevParams<FT> &P, const LV &Tg, const ColJac<FT, M> &Jc,
                                         const FT (&Rr0)[M], const FT (&Re0)[M], const FT (&Rq)[M],
                                         const FT (&Ru1)[M], const FT (&Ru2)[M], const FT (&R3)[M], FT (&Xr)[M],
                                         FT (&Xe)[M], FT (&Xq)[M], FT (&X3)[M], int lane) {
  const int Nv = P.Nv, Nf = P.Nf;
  // over terrain the (rho, u_h), (rho e_tot, u_h) blocks times Δu_h = -R_u_h move to the right-hand
  // sides of the scalar rows: R_x + M_x,uh R_uh
  FT Rr[M], Re[M];
  if constexpr (TOPO) {
    FT ct[M], ctm[M], ctp[M];
#pragma unroll
    for (int k = 0; k < M; ++k) {
      const int v = min(lane * M + k, Nv - 1);
      FT g31, g32, phis;
      Tg.ct(v, g31, g32, phis);
      ct[k] = lane * M + k < Nv ? g31 * Ru1[k] + g32 * Ru2[k] : FT(0);
    }
    nb_all<M, -1>(ct, ctm);
    nb_all<M, 1>(ct, ctp);
#pragma unroll
    for (int k = 0; k < M; ++k) {
      Rr[k] = Rr0[k] + (Jc.wm[k] * ctm[k] + (Jc.w0m[k] - Jc.w0p[k]) * ct[k] - Jc.wp[k] * ctp[k]);
      Re[k] = Re0[k] + (Jc.hb0[k] * (Jc.wm[k] * ctm[k] + Jc.w0m[k] * ct[k]) -
                        Jc.hb1[k] * (Jc.w0p[k] * ct[k] + Jc.wp[k] * ctp[k]));
    }
  } else {
#pragma unroll
    for (int k = 0; k < M; ++k) {
      Rr[k] = Rr0[k];
      Re[k] = Re0[k];
    }
  }
  FT ru0m[M], ru1m[M], eu0m[M], eu1m[M], Rrm[M], Rem[M], Ru1m[M], Ru2m[M];
  nb_all<M, -1>(Jc.ru0, ru0m); nb_all<M, -1>(Jc.ru1, ru1m); nb_all<M, -1>(Jc.eu0, eu0m); nb_all<M, -1>(Jc.eu1, eu1m);
  nb_all<M, -1>(Rr, Rrm); nb_all<M, -1>(Re, Rem); nb_all<M, -1>(Ru1, Ru1m); nb_all<M, -1>(Ru2, Ru2m);
  FT qu0m[M], qu1m[M], Rqm[M];
  if constexpr (MOIST) {
    nb_all<M, -1>(Jc.qu0, qu0m); nb_all<M, -1>(Jc.qu1, qu1m); nb_all<M, -1>(Rq, Rqm);
  }
  FT a[M], b[M], c[M], d[M], x[M];
#pragma unroll
  for (int k = 0; k < M; ++k) {
    const int f = lane * M + k;
    FT aa = Jc.uu0[k], bb = Jc.uu1[k], cc = Jc.uu2[k];
    FT rhs = f < Nf ? R3[k] : FT(0);
    if (f >= 1 && f - 1 < Nv) {  // centre f-1 (slot s = 0)
      const FT cr = Jc.ur0[k], ce = Jc.ue0[k];
      aa += cr * ru0m[k] + ce * eu0m[k];
      bb += cr * ru1m[k] + ce * eu1m[k];
      rhs += cr * Rrm[k] + ce * Rem[k];
      rhs += Jc.uh0[k] * Ru1m[k] + Jc.uh1[k] * Ru2m[k];
      if constexpr (MOIST) {
        const FT cq = Jc.uq0[k];
        aa += cq * qu0m[k];
        bb += cq * qu1m[k];
        rhs += cq * Rqm[k];
      }
    }
    if (f < Nv) {  // centre f (slot s = 1)
      const FT cr = Jc.ur1[k], ce = Jc.ue1[k];
      bb += cr * Jc.ru0[k] + ce * Jc.eu0[k];
      cc += cr * Jc.ru1[k] + ce * Jc.eu1[k];
      rhs += cr * Rr[k] + ce * Re[k];
      rhs += Jc.uh2[k] * Ru1[k] + Jc.uh3[k] * Ru2[k];
      if constexpr (MOIST) {
        const FT cq = Jc.uq1[k];
        bb += cq * Jc.qu0[k];
        cc += cq * Jc.qu1[k];
        rhs += cq * Rq[k];
      }
    }
    if (f >= Nf) { aa = FT(0); bb = FT(1); cc = FT(0); rhs = FT(0); }
    a[k] = aa; b[k] = bb; c[k] = cc; d[k] = rhs;
  }
  if constexpr (M == 2) crpcr_solve2<FT>(a, b, c, d, x, lane);
  else pcr_solve<FT, M>(a, b, c, d, x, lane);
  FT xn[M];
  nb_all<M, 1>(x, xn);
#pragma unroll
  for (int k = 0; k < M; ++k) {
    X3[k] = x[k];
    Xr[k] = Jc.ru0[k] * x[k] + Jc.ru1[k] * xn[k] - Rr[k];
    Xe[k] = Jc.eu0[k] * x[k] + Jc.eu1[k] * xn[k] - Re[k];
    Xq[k] = MOIST ? Jc.qu0[k] * x[k] + Jc.qu1[k] * xn[k] - Rq[k] : FT(0);
  }
}

// Lin et al. (1994) van Leer face value times u, with their monotonicity
// constraint and first-order one-sided values next to the boundaries.
template <class FT>
__device__ __forceinline__ FT vanleer(FT u, FT am2, FT am1, FT a0, FT ap1, bool near, FT dtm) {
  // face between centres (am1 below) and (a0 above); am2 below am1, ap1 above a0
  if (u >= FT(0)) {
    if (near) return u * am1;
    const FT lo = am2, c = am1, hi = a0;
    const FT da = (hi - lo) / FT(2);
    const FT mn = fmin(lo, fmin(c, hi)), mx = fmax(lo, fmax(c, hi));
    const FT sl = copysign(fmin(fabs(da), fmin(FT(2) * (c - mn), FT(2) * (mx - c))), da);
    return u * (c + sl * (FT(1) - fabs(u) * dtm) / FT(2));
  } else {
    if (near) return u * a0;
    const FT lo = am1, c = a0, hi = ap1;
    const FT da = (hi - lo) / FT(2);
    const FT mn = fmin(lo, fmin(c, hi)), mx = fmax(lo, fmax(c, hi));
    const FT sl = copysign(fmin(fabs(da), fmin(FT(2) * (c - mn), FT(2) * (mx - c))), da);
    return u * (c - sl * (FT(1) - fabs(u) * dtm) / FT(2));
  }
}

// a: the transported specific quantity of the centres (h_tot for rho e_tot, q_tot for rho q_tot)
template <class FT, int M>
__device__ __forceinline__ void col_correction(const DevParams<FT> &P, const ColGeo<FT> &G, const ColDiag<FT, M> &Dg,
                                               const FT (&a)[M], FT (&corr)[M], int lane) {
  const int Nv = P.Nv, Nf = P.Nf;
  FT hm1[M], hm2[M], hp1[M], rJm[M];
  nb_all<M, -1>(a, hm1); nb_all<M, -2>(a, hm2); nb_all<M, 1>(a, hp1);
  nb_all<M, -1>(Dg.rJ, rJm);
  FT fup[M], fcen[M];
#pragma unroll
  for (int k = 0; k < M; ++k) {
    const int f = lane * M + k;
    const bool inner = f > 0 && f < Nv;
    const FT rJ = (rJm[k] + Dg.rJ[k]) / FT(2);
    const FT u = Dg.u3c[k];
    const bool near = f == 1 || f == Nv - 1;
    const FT vl = vanleer(u, hm2[k], hm1[k], a[k], hp1[k], near, P.dt_model);
    fup[k] = inner ? rJ * vl : FT(0);
    fcen[k] = inner ? rJ * (u * (hm1[k] + a[k]) / FT(2)) : FT(0);
  }
  FT fupn[M], fcn[M];
  nb_all<M, 1>(fup, fupn);
  nb_all<M, 1>(fcen, fcn);
#pragma unroll
  for (int k = 0; k < M; ++k) {
    const FT vup = -((fupn[k] - fup[k]) * Dg.iJ[k]);
    const FT vc = -((fcn[k] - fcen[k]) * Dg.iJ[k]);
    corr[k] = vup - vc;
  }
}

// centre block [e][NFC][16][Nv]: NFC = 4 (rho, u_1, u_2, rho e_tot), 5 with rho q_tot
template <class FT, int NFC = 4>
__device__ __forceinline__ size_t cidx(int e, int c, int n, int v, int Nv) { return (((size_t)e * NFC + c) * NN + n) * Nv + v; }
template <class FT>
__device__ __forceinline__ size_t ridx(int e, int c, int n, int v, int Nv) { return (((size_t)e * 2 + c) * NN + n) * Nv + v; }

// Individual hooks: implicit tendency, Jacobian, ldiv, post-Newton correction.  MOIST: the
// centre block carries rho q_tot as its fifth component (never with TOPO).
template <class FT, int M, int MODE, bool TOPO, bool MOIST>
__global__ void __launch_bounds__(COL_THREADS) k_col_hook(DevParams<FT> P, ColArgs<FT> A) {
  static_assert(!(TOPO && MOIST), "moist 0M is not built over terrain");
  constexpr int NFC = MOIST ? 5 : 4;
  const int lane = threadIdx.x & 31;
  const int col = blockIdx.x * (COL_THREADS / 32) + (threadIdx.x >> 5);
  const int ncols = P.Nh * NN;
  if (col >= ncols) return;
  const int e = col >> 4, n = col & 15, Nv = P.Nv, Nf = P.Nf;
  ColGeo<FT> G;
  G.load(P, e, n);
  constexpr int NQJ = TOPO ? JAC_QT : (MOIST ? JAC_QM : JAC_Q);
  using LV = std::conditional_t<TOPO, col::ColLevT<FT>, col::ColLev<FT>>;
  LV Tg;
  if constexpr (TOPO) Tg.load(P, e, n);
  else Tg = col::ColLev<FT>{P.lc4, P.lf4, P.lr4, Nv, Nf};
  ColState<FT, M> S;
#pragma unroll
  for (int k = 0; k < M; ++k) {
    const int v = lane * M + k;
    const bool cv = v < Nv, fv = v < Nf;
    S.rho[k] = cv ? A.Y_c[cidx<FT, NFC>(e, 0, n, v, Nv)] : (MODE == COL_LDIV ? FT(0) : FT(1));
    S.u1[k] = cv ? A.Y_c[cidx<FT, NFC>(e, 1, n, v, Nv)] : FT(0);
    S.u2[k] = cv ? A.Y_c[cidx<FT, NFC>(e, 2, n, v, Nv)] : FT(0);
    S.rhoe[k] = cv ? A.Y_c[cidx<FT, NFC>(e, 3, n, v, Nv)] : (MODE == COL_LDIV ? FT(0) : FT(1));
    S.rhoq[k] = MOIST && cv ? A.Y_c[cidx<FT, NFC>(e, 4, n, v, Nv)] : FT(0);
    S.u3[k] = fv ? A.Y_f[((size_t)e * NN + n) * Nf + v] : FT(0);
    if (!TOPO && MODE != COL_LDIV && (v == 0 || v >= Nv)) S.u3[k] = FT(0);  // impenetrable filter
  }
  if constexpr (TOPO) {
    if (MODE != COL_LDIV) col_filter_topo<FT, M>(Tg, S, lane);  // -u_h^3 / g^33 on the boundary faces
  }
  FT *jac = A.jac + (size_t)col * NQJ * Nf;
  FT o0[M], o1[M], o2[M], o3[M], o4[M], o5[M];
  if constexpr (MODE == COL_LDIV) {
    ColJac<FT, M> Jc;
#pragma unroll
    for (int k = 0; k < M; ++k) {
      const int f = lane * M + k;
      const int fc = min(f, Nf - 1);
      FT *q[JAC_QT] = {Jc.ru0, Jc.ru1, Jc.eu0, Jc.eu1, Jc.ur0, Jc.ur1, Jc.ue0, Jc.ue1,
                       Jc.uh0, Jc.uh1, Jc.uh2, Jc.uh3, Jc.uu0, Jc.uu1, Jc.uu2,
                       TOPO ? Jc.wm : Jc.qu0, TOPO ? Jc.w0m : Jc.qu1, TOPO ? Jc.w0p : Jc.uq0, TOPO ? Jc.wp : Jc.uq1,
                       Jc.hb0, Jc.hb1};
      for (int t = 0; t < NQJ; ++t) q[t][k] = jac[t * Nf + fc];
      if (f >= Nf) {
        for (int t = 0; t < NQJ; ++t) q[t][k] = FT(0);
        Jc.uu1[k] = FT(1);
      }
    }
    col_ldiv<FT, M, TOPO, MOIST>(P, Tg, Jc, S.rho, S.rhoe, S.rhoq, S.u1, S.u2, S.u3, o0, o3, o5, o4, lane);
#pragma unroll
    for (int k = 0; k < M; ++k) { o1[k] = -S.u1[k]; o2[k] = -S.u2[k]; }
  } else {
    ColDiag<FT, M> Dg;
    col_diag<FT, M, TOPO, MOIST>(P, G, Tg, S, Dg, lane);
    if constexpr (MODE == COL_IMPLICIT) {
      col_implicit<FT, M, TOPO, MOIST>(P, G, Tg, S, Dg, o0, o3, o4, o5, lane);
#pragma unroll
      for (int k = 0; k < M; ++k) { o1[k] = FT(0); o2[k] = FT(0); }
    } else if constexpr (MODE == COL_POSTIMP) {
      FT corr[M], corq[M];
      if (P.upwinding) {
        col_correction<FT, M>(P, G, Dg, Dg.h, corr, lane);
        if constexpr (MOIST) col_correction<FT, M>(P, G, Dg, Dg.q, corq, lane);
      }
#pragma unroll
      for (int k = 0; k < M; ++k) {
        o0[k] = o1[k] = o2[k] = o4[k] = FT(0);
        o3[k] = P.upwinding ? corr[k] : FT(0);
        o5[k] = MOIST && P.upwinding ? corq[k] : FT(0);
      }
    } else {  // COL_JACOBIAN
      ColJac<FT, M> Jc;
      col_jacobian<FT, M, TOPO, MOIST>(P, G, Tg, S, Dg, A.dtg, Jc, lane);
#pragma unroll
      for (int k = 0; k < M; ++k) {
        const int f = lane * M + k;
        if (f < Nf) {
          if constexpr (TOPO) {
            const FT q[JAC_QT] = {Jc.ru0[k], Jc.ru1[k], Jc.eu0[k], Jc.eu1[k], Jc.ur0[k], Jc.ur1[k], Jc.ue0[k],
                                  Jc.ue1[k], Jc.uh0[k], Jc.uh1[k], Jc.uh2[k], Jc.uh3[k], Jc.uu0[k], Jc.uu1[k],
                                  Jc.uu2[k], Jc.wm[k], Jc.w0m[k], Jc.w0p[k], Jc.wp[k], Jc.hb0[k], Jc.hb1[k]};
            for (int t = 0; t < JAC_QT; ++t) jac[t * Nf + f] = q[t];
          } else if constexpr (MOIST) {
            const FT q[JAC_QM] = {Jc.ru0[k], Jc.ru1[k], Jc.eu0[k], Jc.eu1[k], Jc.ur0[k], Jc.ur1[k], Jc.ue0[k],
                                  Jc.ue1[k], Jc.uh0[k], Jc.uh1[k], Jc.uh2[k], Jc.uh3[k], Jc.uu0[k], Jc.uu1[k],
                                  Jc.uu2[k], Jc.qu0[k], Jc.qu1[k], Jc.uq0[k], Jc.uq1[k]};
            for (int t = 0; t < JAC_QM; ++t) jac[t * Nf + f] = q[t];
          } else {
            const FT q[JAC_Q] = {Jc.ru0[k], Jc.ru1[k], Jc.eu0[k], Jc.eu1[k], Jc.ur0[k], Jc.ur1[k], Jc.ue0[k], Jc.ue1[k],
                                 Jc.uh0[k], Jc.uh1[k], Jc.uh2[k], Jc.uh3[k], Jc.uu0[k], Jc.uu1[k], Jc.uu2[k]};
            for (int t = 0; t < JAC_Q; ++t) jac[t * Nf + f] = q[t];
          }
        }
      }
      return;
    }
  }
#pragma unroll
  for (int k = 0; k < M; ++k) {
    const int v = lane * M + k;
    if (v < Nv) {
      A.O_c[cidx<FT, NFC>(e, 0, n, v, Nv)] = o0[k];
      A.O_c[cidx<FT, NFC>(e, 1, n, v, Nv)] = o1[k];
      A.O_c[cidx<FT, NFC>(e, 2, n, v, Nv)] = o2[k];
      A.O_c[cidx<FT, NFC>(e, 3, n, v, Nv)] = o3[k];
      if constexpr (MOIST) A.O_c[cidx<FT, NFC>(e, 4, n, v, Nv)] = o5[k];
    }
    if (v < Nf) A.O_f[((size_t)e * NN + n) * Nf + v] = o4[k];
  }
}

inline int levels_per_lane(int Nf) { return Nf <= 32 ? 1 : (Nf <= 64 ? 2 : 4); }

}  // namespace

template <class FT, int M, bool TOPO, bool MOIST>
void launch_hook_mt(const DevParams<FT> &P, int mode, const ColArgs<FT> &A, int grid, cudaStream_t s) {
  switch (mode) {
    case COL_IMPLICIT: k_col_hook<FT, M, COL_IMPLICIT, TOPO, MOIST><<<grid, COL_THREADS, 0, s>>>(P, A); break;
    case COL_JACOBIAN: k_col_hook<FT, M, COL_JACOBIAN, TOPO, MOIST><<<grid, COL_THREADS, 0, s>>>(P, A); break;
    case COL_LDIV: k_col_hook<FT, M, COL_LDIV, TOPO, MOIST><<<grid, COL_THREADS, 0, s>>>(P, A); break;
    default: k_col_hook<FT, M, COL_POSTIMP, TOPO, MOIST><<<grid, COL_THREADS, 0, s>>>(P, A); break;
  }
}
template <class FT, int M>
void launch_hook_m(const DevParams<FT> &P, int mode, const ColArgs<FT> &A, int grid, cudaStream_t s) {
  if (P.topo) launch_hook_mt<FT, M, true, false>(P, mode, A, grid, s);
  else if (P.moist) launch_hook_mt<FT, M, false, true>(P, mode, A, grid, s);
  else launch_hook_mt<FT, M, false, false>(P, mode, A, grid, s);
}

template <class FT>
void launch_column(const DevParams<FT> &P, int mode, const ColArgs<FT> &A, cudaStream_t s) {
  const int ncols = P.Nh * NN, grid = (ncols + COL_THREADS / 32 - 1) / (COL_THREADS / 32);
  switch (levels_per_lane(P.Nf)) {
    case 1: launch_hook_m<FT, 1>(P, mode, A, grid, s); break;
    case 2: launch_hook_m<FT, 2>(P, mode, A, grid, s); break;
    default: launch_hook_m<FT, 4>(P, mode, A, grid, s); break;
  }
}

template void launch_column<float>(const DevParams<float> &, int, const ColArgs<float> &, cudaStream_t);
template void launch_column<double>(const DevParams<double> &, int, const ColArgs<double> &, cudaStream_t);

}  // namespace gb
