// Device core of the implicit column solve, shared by the IMEX stage kernel and
// the batched standalone-column kernels.
//
// A column of Nv centres / Nv+1 faces is held by a group of G lanes, CM
// consecutive levels per lane (lane gl holds levels gl*CM .. gl*CM+CM-1); the
// only cross-lane traffic is a one-level halo per quantity and the tridiagonal
// solve.  One call of newton_core is one Newton iteration of ClimaTimeSteppers'
// NewtonsMethod on the implicit stage equation (integrator.jl:63-120):
//   R = U^ + dtgamma T_imp(U) - U              (implicit_tendency.jl:185-298)
//   W = dtgamma dT_imp/dU - I at U             (manual_sparse_jacobian.jl:713-870,
//                                               dry, no topography)
//   U <- U - W^-1 R                            (BlockArrowheadSolve(rho, rho e_tot;
//                                               alg2 = u_h), manual_sparse_jacobian.jl:580-583)
// with the impenetrable filter (precomputed_quantities.jl:486-553) on u_3.
#pragma once
#include "kernels.cuh"
#include "topo.cuh"

namespace gb {
namespace col {

template <int G, class FT>
__device__ __forceinline__ FT up(FT v, int d) { return __shfl_up_sync(0xffffffffu, v, d, G); }
template <int G, class FT>
__device__ __forceinline__ FT down(FT v, int d) { return __shfl_down_sync(0xffffffffu, v, d, G); }

// Level geometry of one column: lc4[v] = {r^2 dz, 1/(r^2 dz), 1/r^2, Phi},
// lf4[f] = {g^33, beta_w, Phi_c(f) - Phi_c(f-1) (0 on the boundary faces), 0},
// lr4[v] = the level's reference record {p0, 1/p0, cp_d (T_sfc - T_min) / 7 Pi0^7, 0}.
template <class FT>
struct ColLev {
  const Lev4<FT> *lc4, *lf4, *lr4;
  int Nv, Nf;
  static constexpr bool TOPO = false;
  __device__ Lev4<FT> c4(int v) const { return lc4[v]; }
  __device__ Lev4<FT> f4(int k) const { return lf4[k]; }
  __device__ Lev4<FT> r4(int v) const { return lr4[v]; }
};

// The level geometry of one column over terrain-following levels, with the interface of
// ColLev: c4(v) = {r^2 dz, 1/(r^2 dz), 1/r^2, Phi} and f4(k) = {g^33, beta_w, 0, 0} of the
// column's own points (topo.cuh), r4(v) the flat level's reference record; ct(v) gives the
// centre's (g^31, g^32) and g z_s b, the geopotential above the flat level's.
template <class FT>
struct ColLevT {
  const Lev4<FT> *ltc, *ltf, *lr4;
  int Nv, Nf;
  FT zs, d1, d2, gs0, gs1, gs2, iR, grav, aw, zd, sk;
  static constexpr bool TOPO = true;
  __device__ void load(const DevParams<FT> &P, int e, int n) {
    ltc = P.ltc;
    ltf = P.ltf;
    lr4 = P.lr4;
    Nv = P.Nv;
    Nf = P.Nf;
    iR = P.iR;
    grav = P.grav;
    aw = P.spg_aw;
    zd = P.spg_zd;
    sk = P.spg_k;
    const FT *tg = P.tgeo + (size_t)e * TG_N * NN, *hg = P.hgeo + (size_t)e * HG_N * NN;
    zs = tg[TG_ZS * NN + n];
    d1 = tg[TG_D1 * NN + n];
    d2 = tg[TG_D2 * NN + n];
    gs0 = hg[HG_GU0 * NN + n];
    gs1 = hg[HG_GU1 * NN + n];
    gs2 = hg[HG_GU2 * NN + n];
  }
  __device__ TPoint<FT> pt(const Lev4<FT> &L) const {
    TPoint<FT> o;
    o.zsb = zs * L.y;
    o.z = L.x + o.zsb;
    o.r = FT(1) + o.z * iR;
    o.ir = grcp(o.r);
    o.r2 = o.r * o.r;
    o.ir2 = o.ir * o.ir;
    o.dz = L.z + zs * L.w;
    o.idz = grcp(o.dz);
    o.s1 = L.y * d1;
    o.s2 = L.y * d2;
    return o;
  }
  __device__ Lev4<FT> c4(int v) const {
    const TPoint<FT> t = pt(ltc[v]);
    const FT x = t.r2 * t.dz;
    return Lev4<FT>{x, grcp(x), t.ir2, grav * t.z};
  }
  __device__ Lev4<FT> f4(int k) const {
    const TPoint<FT> t = pt(ltf[k]);
    FT beta = FT(0);
    if (aw != FT(0) && t.z > zd) {
      const FT s = gsin(sk * (t.z - zd));
      beta = aw * s * s;
    }
    return Lev4<FT>{tmetric_up(t, gs0, gs1, gs2).g33, beta, FT(0), FT(0)};
  }
  __device__ Lev4<FT> r4(int v) const { return lr4[v]; }
  __device__ void ct(int v, FT &g31, FT &g32, FT &phis) const {
    const TPoint<FT> t = pt(ltc[v]);
    const TMetricUp<FT> m = tmetric_up(t, gs0, gs1, gs2);
    g31 = m.g13;
    g32 = m.g23;
    phis = grav * t.zsb;
  }
  // c4 and ct of one centre from one evaluation of its point terms
  __device__ Lev4<FT> c4ct(int v, FT &g31, FT &g32, FT &phis) const {
    const TPoint<FT> t = pt(ltc[v]);
    const TMetricUp<FT> m = tmetric_up(t, gs0, gs1, gs2);
    g31 = m.g13;
    g32 = m.g23;
    phis = grav * t.zsb;
    const FT x = t.r2 * t.dz;
    return Lev4<FT>{x, grcp(x), t.ir2, grav * t.z};
  }
};

// Centre diagnostics of one level from (rho, u_1, u_2, rho e_tot), the u_3 of
// the faces below/above and their g^33.  ct3 = CT3(u_h) (0 over a flat surface).
template <class FT>
struct Cen {
  FT rJ, h, phid, Pi, thv, thvr, K, iJ, phi, ct3;
};
template <class FT, class LV>
__device__ __forceinline__ Cen<FT> cdiag(const DevParams<FT> &P, const ColGeo<FT> &G, const LV &L, int v,
                                         FT rho, FT u1, FT u2, FT rhoe, FT u3a, FT u3b, FT g33a, FT g33b) {
  const int vc = min(max(v, 0), L.Nv - 1);
  FT phis = FT(0), g31 = FT(0), g32 = FT(0);
  Lev4<FT> Lc;
  if constexpr (LV::TOPO) Lc = L.c4ct(vc, g31, g32, phis);
  else Lc = L.c4(vc);
  const FT c1 = (G.gu0 * u1 + G.gu1 * u2) * Lc.z, c2 = (G.gu1 * u1 + G.gu2 * u2) * Lc.z;
  const FT kv = (u3a * (u3a * g33a) + u3b * (u3b * g33b)) / FT(2);
  Cen<FT> o;
  if constexpr (LV::TOPO) {
    // over terrain K takes 2 CT3(u_h) I^c(u_3) (compute_kinetic, utilities.jl:194-206)
    o.ct3 = g31 * u1 + g32 * u2;
    o.K = (u1 * c1 + u2 * c2 + kv + FT(2) * o.ct3 * ((u3a + u3b) / FT(2))) / FT(2);
  } else {
    o.ct3 = FT(0);
    o.K = (u1 * c1 + u2 * c2 + kv) / FT(2);
  }
  Thermo<FT> th;
  thermo(P, rho, rhoe, o.K, Lc.w, L.r4(vc), th);
  o.h = th.h;
  o.phid = LV::TOPO ? th.phid + phis : th.phid;
  o.Pi = th.Pi;
  o.thv = th.thv;
  o.thvr = th.thvr;
  o.iJ = G.iJh * Lc.y;
  o.rJ = rho * (G.Jh * Lc.x);
  o.phi = Lc.w;
  return o;
}

// The centre diagnostics of the lane's CM levels r0 .. r0 + CM - 1 from the state U
// (rho, u_1, u_2, rho e_tot), the u_3 of the faces below (u3a) and above (u3b) each level
// and their g^33.  FP32 with two levels per lane: both levels at once, the same quantities
// with packed arithmetic (thermo_pair).
template <class FT, int CM, class LV>
__device__ __forceinline__ void cdiag_lane(const DevParams<FT> &P, const ColGeo<FT> &G, const LV &L, int r0,
                                           const FT (&U)[5][CM], const FT (&u3a)[CM], const FT (&u3b)[CM],
                                           const FT (&g33a)[CM], const FT (&g33b)[CM], Cen<FT> (&o)[CM]) {
#pragma unroll
  for (int k = 0; k < CM; ++k)
    o[k] = cdiag(P, G, L, r0 + k, U[0][k], U[1][k], U[2][k], U[3][k], u3a[k], u3b[k], g33a[k], g33b[k]);
}
template <>
__device__ __forceinline__ void cdiag_lane<float, 2, ColLev<float>>(const DevParams<float> &P, const ColGeo<float> &G,
                                                     const ColLev<float> &L, int r0, const float (&U)[5][2],
                                                     const float (&u3a)[2], const float (&u3b)[2],
                                                     const float (&g33a)[2], const float (&g33b)[2],
                                                     Cen<float> (&o)[2]) {
  const int v0 = min(max(r0, 0), L.Nv - 1), v1 = min(max(r0 + 1, 0), L.Nv - 1);
  const Lev4<float> C0 = L.lc4[v0], C1 = L.lc4[v1], R0 = L.lr4[v0], R1 = L.lr4[v1];
  const float2 rho = make_float2(U[0][0], U[0][1]), u1 = make_float2(U[1][0], U[1][1]);
  const float2 u2 = make_float2(U[2][0], U[2][1]), rhoe = make_float2(U[3][0], U[3][1]);
  const float2 a = make_float2(u3a[0], u3a[1]), b = make_float2(u3b[0], u3b[1]);
  const float2 ga = make_float2(g33a[0], g33a[1]), gb = make_float2(g33b[0], g33b[1]);
  const float2 ir2 = make_float2(C0.z, C1.z), phi = make_float2(C0.w, C1.w);
  const float2 c1 = __fmul2_rn(__ffma2_rn(bc2(G.gu1), u2, __fmul2_rn(bc2(G.gu0), u1)), ir2);
  const float2 c2 = __fmul2_rn(__ffma2_rn(bc2(G.gu2), u2, __fmul2_rn(bc2(G.gu1), u1)), ir2);
  const float2 kv = __fmul2_rn(__ffma2_rn(b, __fmul2_rn(b, gb), __fmul2_rn(a, __fmul2_rn(a, ga))), bc2(0.5f));
  const float2 K = __fmul2_rn(__fadd2_rn(__ffma2_rn(u2, c2, __fmul2_rn(u1, c1)), kv), bc2(0.5f));
  float2 T, p, h, Pi, thv, thvr, phid, Tr;
  thermo_pair(P, rho, rhoe, K, phi, make_float2(R0.y, R1.y), make_float2(R0.z, R1.z), T, p, h, Pi, thv, thvr, phid, Tr);
  const float2 iJ = __fmul2_rn(bc2(G.iJh), make_float2(C0.y, C1.y));
  const float2 rJ = __fmul2_rn(rho, __fmul2_rn(bc2(G.Jh), make_float2(C0.x, C1.x)));
  o[0].K = K.x; o[1].K = K.y;
  o[0].h = h.x; o[1].h = h.y;
  o[0].phid = phid.x; o[1].phid = phid.y;
  o[0].Pi = Pi.x; o[1].Pi = Pi.y;
  o[0].thv = thv.x; o[1].thv = thv.y;
  o[0].thvr = thvr.x; o[1].thvr = thvr.y;
  o[0].iJ = iJ.x; o[1].iJ = iJ.y;
  o[0].rJ = rJ.x; o[1].rJ = rJ.y;
  o[0].phi = phi.x; o[1].phi = phi.y;
  o[0].ct3 = o[1].ct3 = 0.0f;
}

// Tridiagonal solve of the CM*G rows held CM per lane by a G-lane group:
// log2(CM) in-lane cyclic-reduction levels reduce each lane's rows to one,
// parallel cyclic reduction solves the G reduced rows across the group, and
// the eliminated rows are back-substituted in-lane.
template <class FT, int G, int CM>
__device__ __forceinline__ void solve_lanes(FT (&a)[CM], FT (&b)[CM], FT (&c)[CM], FT (&d)[CM], FT (&x)[CM], int gl) {
#pragma unroll
  for (int s = 1; s < CM; s <<= 1) {
    const FT pa = up<G>(a[CM - s], 1), pb = up<G>(b[CM - s], 1), pc = up<G>(c[CM - s], 1), pd = up<G>(d[CM - s], 1);
#pragma unroll
    for (int k = 0; k < CM; k += 2 * s) {
      const bool hl = (k - s >= 0) || gl > 0;
      const FT la = k - s >= 0 ? a[k - s] : pa, lb = k - s >= 0 ? b[k - s] : pb;
      const FT lc = k - s >= 0 ? c[k - s] : pc, ld = k - s >= 0 ? d[k - s] : pd;
      const FT al = hl ? -gdiv(a[k], lb) : FT(0);
      const FT ga = -gdiv(c[k], b[k + s]);
      FT nb = b[k] + ga * a[k + s], nd = d[k] + ga * d[k + s];
      if (hl) { nb += al * lc; nd += al * ld; }
      a[k] = hl ? al * la : FT(0);
      c[k] = ga * c[k + s];
      b[k] = nb;
      d[k] = nd;
    }
  }
  FT A = a[0], B = b[0], C = c[0], D = d[0];
#pragma unroll
  for (int s = 1; s < G; s <<= 1) {
    const FT Am = up<G>(A, s), Bm = up<G>(B, s), Cm = up<G>(C, s), Dm = up<G>(D, s);
    const FT Ap = down<G>(A, s), Bp = down<G>(B, s), Cp = down<G>(C, s), Dp = down<G>(D, s);
    const bool hm = gl >= s, hp = gl + s < G;
    const FT al = hm ? -gdiv(A, Bm) : FT(0);
    const FT ga = hp ? -gdiv(C, Bp) : FT(0);
    FT nB = B, nD = D;
    if (hm) { nB += al * Cm; nD += al * Dm; }
    if (hp) { nB += ga * Ap; nD += ga * Dp; }
    A = hm ? al * Am : FT(0);
    C = hp ? ga * Cp : FT(0);
    B = nB;
    D = nD;
  }
  x[0] = gdiv(D, B);
  const FT xns = down<G>(x[0], 1);  // every lane shuffles; the column's last lane discards it
  const FT xn = gl + 1 < G ? xns : FT(0);
#pragma unroll
  for (int s = CM / 2; s >= 1; s >>= 1) {
#pragma unroll
    for (int m = s; m < CM; m += 2 * s) {
      const FT xu = m + s < CM ? x[m + s] : xn;
      x[m] = gdiv(d[m] - a[m] * x[m - s] - c[m] * xu, b[m]);
    }
  }
}

// Face value of the van Leer (Mono5-limited) reconstruction times u
// (abbreviations.jl:250-256 ᶠlin_vanleer; first order next to the boundary).
template <class FT>
__device__ __forceinline__ FT vanleer_g(FT u, FT am2, FT am1, FT a0, FT ap1, bool near, FT dtm) {
  const bool pos = u >= FT(0);
  const FT lo = pos ? am2 : am1, c = pos ? am1 : a0, hi = pos ? a0 : ap1;
  if (near) return u * c;
  const FT da = (hi - lo) / FT(2);
  const FT mn = fmin(lo, fmin(c, hi)), mx = fmax(lo, fmax(c, hi));
  const FT sl = copysign(fmin(fabs(da), fmin(FT(2) * (c - mn), FT(2) * (mx - c))), da);
  const FT half = sl * (FT(1) - fabs(u) * dtm) / FT(2);
  return u * (pos ? c + half : c - half);
}

// One Newton iteration on the column held by this lane group.
//   Hh: U^ per level (rho, u_1, u_2, rho e_tot at centres r0..r0+CM-1; u_3 at faces r0..)
//   U:  the iterate; on return U[0], U[3] are updated and U[4] holds the filtered u_3
//   (levels past the column hold rho = rho e_tot = 1 and u_3 = 0).
// HAT = false asserts U == U^ on entry (the first iteration of an IMEX stage),
// which drops the U^ - U terms of the residual.
// ss accumulates the FP64 sums of squares of the residual (rho, rho e_tot, u_3),
// iJc receives 1/J of the lane's centres.
// Over terrain-following levels (LV::TOPO) u^3 = u_h^3 + g^33 u_3 with
// u_h^3 = ᶠwinterp(rho J, CT3(u_h)) (compute_ᶠuₕ³, precomputed_quantities.jl:473-476), the
// filter sets u_3 = -u_h^3 / g^33 on the bottom and top faces, and the (u_3, u_3) block takes
// dK/du_3 = (g^33 u_3)_f / 2 + CT3(u_h)_v / 2 (∂ᶜK_∂ᶠu₃, manual_sparse_jacobian.jl:754-756).
// The (rho, u_h), (rho e_tot, u_h) and (u_3, u_h) blocks multiply R_u_h = 0 here.
template <class FT, int G, int CM, bool HAT, class LV>
__device__ __forceinline__ void newton_core(const DevParams<FT> &P, const ColGeo<FT> &Gm, const LV &L, int gl,
                                            FT dtg, const FT (&Hh)[5][CM], FT (&U)[5][CM], CSum<FT> (&ss)[3],
                                            bool &finite, FT (&iJc)[CM]) {
  const int Nv = L.Nv, Nf = L.Nf;
  const int r0 = gl * CM;
  // face geometry of faces r0 .. r0 + CM and g^33 of face r0 - 1
  Lev4<FT> LF[CM + 1];
#pragma unroll
  for (int k = 0; k <= CM; ++k) LF[k] = L.f4(min(r0 + k, Nf - 1));
  const FT g33m = L.f4(min(max(r0 - 1, 0), Nf - 1)).x;
  // halo: centre -1 and face -1 from the previous lane, face r0 + CM from the next lane
  const FT hr = up<G>(U[0][CM - 1], 1), hu1 = up<G>(U[1][CM - 1], 1), hu2 = up<G>(U[2][CM - 1], 1);
  // ---- filtered state: u_3 = 0 on the boundary faces (-u_h^3 / g^33 over terrain)
  FT u3[CM];
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const int f = r0 + k;
    if constexpr (LV::TOPO) {
      if (f == 0 || f == Nv) {
        const int v = f == 0 ? 0 : Nv - 1;
        const FT a1 = f == 0 ? U[1][k] : (k > 0 ? U[1][k > 0 ? k - 1 : 0] : hu1);
        const FT a2 = f == 0 ? U[2][k] : (k > 0 ? U[2][k > 0 ? k - 1 : 0] : hu2);
        FT g31, g32, phis;
        L.ct(v, g31, g32, phis);
        u3[k] = -(g31 * a1 + g32 * a2) / LF[k].x;
      } else {
        u3[k] = f > Nv ? FT(0) : U[4][k];
      }
    } else {
      u3[k] = (f == 0 || f >= Nv) ? FT(0) : U[4][k];
    }
  }
  const FT he = up<G>(U[3][CM - 1], 1), h3 = up<G>(u3[CM - 1], 1);
  const FT n3 = down<G>(u3[0], 1);  // every lane shuffles; the column's last lane discards it
  const FT u3n = gl + 1 < G ? n3 : FT(0);
  // ---- centre diagnostics r0-1 .. r0+CM-1 and face quantities r0 .. r0+CM-1 (streamed)
  FT F[CM + 1], Fh[CM + 1], fr[CM + 1], fhb[CM + 1];
  FT T3[CM], ur0[CM], ur1[CM], ue0[CM], uu0[CM], uu1[CM], uu2[CM];
  const FT kap = P.Rd * P.icvd;
  const FT h3m = gl > 0 ? h3 : FT(0);
  Cen<FT> prev = cdiag(P, Gm, L, r0 - 1, gl > 0 ? hr : FT(1), hu1, hu2, gl > 0 ? he : FT(1), h3m, u3[0], g33m, LF[0].x);
  FT rhoPrev = gl > 0 ? hr : FT(1);
  FT u3cPrev = h3m * g33m;
  Cen<FT> cen[CM];
  {
    FT u3b[CM], ga[CM], gb[CM];
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      u3b[k] = k + 1 < CM ? u3[k + 1] : u3n;
      ga[k] = LF[k].x;
      gb[k] = LF[k + 1].x;
    }
    cdiag_lane<FT, CM>(P, Gm, L, r0, U, u3, u3b, ga, gb, cen);
  }
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const int f = r0 + k;
    const FT u3next = k + 1 < CM ? u3[k + 1] : u3n;
    const Cen<FT> cur = cen[k];
    iJc[k] = cur.iJ;
    const bool inner = f > 0 && f < Nv;
    const FT g33 = LF[k].x;
    const FT u3c = u3[k] * g33;
    const FT rJb = (prev.rJ + cur.rJ) / FT(2);
    const FT hb = (prev.h + cur.h) / FT(2);
    if constexpr (LV::TOPO) {
      const FT uh3 = (prev.rJ * prev.ct3 + cur.rJ * cur.ct3) / (prev.rJ + cur.rJ);
      F[k] = inner ? rJb * (uh3 + u3c) : FT(0);
    } else {
      F[k] = inner ? rJb * u3c : FT(0);
    }
    Fh[k] = F[k] * hb;
    fr[k] = inner ? rJb * g33 : FT(0);
    fhb[k] = hb;
    const FT beta = LF[k].y;
    FT t3 = FT(0);
    if (inner) {
      const FT thd = ((prev.thv - prev.thvr) + (cur.thv - cur.thvr)) / FT(2);
      // ᶠgradᵥ(Phi) - ᶠgradᵥ(Phi_r): the difference of Phi - Phi_r between the levels
      t3 = -((cur.phid - prev.phid) + P.cpd * thd * (cur.Pi - prev.Pi));
    }
    T3[k] = t3 - beta * u3[k];
    if (inner) {
      const FT ra = rhoPrev, rbv = U[0][k];
      const FT irb = grcp((ra + rbv) / FT(2));
      const FT dpa = kap * (P.T0 * P.cpd - prev.K - prev.phi);
      const FT dpb = kap * (P.T0 * P.cpd - cur.K - cur.phi);
      const FT buoy = P.cpd * ((prev.thv + cur.thv) / FT(2)) * (cur.Pi - prev.Pi) * irb;
      ur0[k] = dtg * (dpa * irb + buoy / FT(2));
      ur1[k] = dtg * (-dpb * irb + buoy / FT(2));
      ue0[k] = dtg * (kap * irb);
      const FT u3cn = u3next * LF[k + 1].x;
      if constexpr (LV::TOPO) {
        uu0[k] = dtg * (-kap * ra * (u3cPrev + prev.ct3) * (irb / FT(2)));
        uu1[k] = dtg * (kap * (rbv * (u3c + cur.ct3) - ra * (u3c + prev.ct3)) * (irb / FT(2)) - beta) - FT(1);
        uu2[k] = dtg * (kap * rbv * (u3cn + cur.ct3) * (irb / FT(2)));
      } else {
        uu0[k] = dtg * (-kap * ra * u3cPrev * (irb / FT(2)));
        uu1[k] = dtg * (kap * (rbv - ra) * u3c * (irb / FT(2)) - beta) - FT(1);
        uu2[k] = dtg * (kap * rbv * u3cn * (irb / FT(2)));
      }
    } else {
      ur0[k] = ur1[k] = ue0[k] = uu0[k] = uu2[k] = FT(0);
      uu1[k] = f <= Nv ? -dtg * beta - FT(1) : FT(1);
    }
    prev = cur;
    rhoPrev = U[0][k];
    u3cPrev = u3c;
  }
  // face r0 + CM belongs to the next lane (its face quantities at k = 0)
  {
    const FT sF = down<G>(F[0], 1), sFh = down<G>(Fh[0], 1), sfr = down<G>(fr[0], 1), sfhb = down<G>(fhb[0], 1);
    const bool nx = gl + 1 < G;
    F[CM] = nx ? sF : FT(0);
    Fh[CM] = nx ? sFh : FT(0);
    fr[CM] = nx ? sfr : FT(0);
    fhb[CM] = sfhb;
  }
  // ---- centre rows r0 .. r0+CM-1: residual and the (scalar, u_3) blocks
  FT Rr[CM], Re[CM], ru0[CM], ru1[CM], eu0[CM], eu1[CM];
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const int v = r0 + k;
    const bool cv = v < Nv;
    const FT Tr = -((F[k + 1] - F[k]) * iJc[k]);
    const FT Te = -((Fh[k + 1] - Fh[k]) * iJc[k]);
    FT rr = dtg * Tr, re = dtg * Te;
    if (HAT) {
      rr += Hh[0][k] - U[0][k];
      re += Hh[3][k] - U[3][k];
    }
    Rr[k] = cv ? rr : FT(0);
    Re[k] = cv ? re : FT(0);
    const FT v0 = fr[k] * iJc[k], v1 = -fr[k + 1] * iJc[k];
    ru0[k] = cv ? dtg * v0 : FT(0);
    ru1[k] = cv ? dtg * v1 : FT(0);
    eu0[k] = cv ? dtg * (v0 * fhb[k]) : FT(0);
    eu1[k] = cv ? dtg * (v1 * fhb[k + 1]) : FT(0);
    ss[0].add(mul_rn(Rr[k], Rr[k]));
    ss[1].add(mul_rn(Re[k], Re[k]));
    finite = finite && isfinite(Rr[k]) && isfinite(Re[k]);
  }
  // ---- Schur complement rows onto u_3 (faces r0 .. r0+CM-1); centre r0-1 rows from the previous lane
  FT a[CM], b[CM], c[CM], d[CM];
  {
    const FT pRr = up<G>(Rr[CM - 1], 1), pRe = up<G>(Re[CM - 1], 1);
    const FT pru0 = up<G>(ru0[CM - 1], 1), pru1 = up<G>(ru1[CM - 1], 1);
    const FT peu0 = up<G>(eu0[CM - 1], 1), peu1 = up<G>(eu1[CM - 1], 1);
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const int f = r0 + k;
      FT R3 = FT(0);
      if (f < Nf) R3 = dtg * T3[k] + (Hh[4][k] - u3[k]);
      ss[2].add(mul_rn(R3, R3));
      finite = finite && isfinite(R3);
      FT aa = uu0[k], bb = uu1[k], cc = uu2[k], rhs = R3;
      const FT mr0 = k > 0 ? ru0[k - 1] : pru0, mr1 = k > 0 ? ru1[k - 1] : pru1;
      const FT me0 = k > 0 ? eu0[k - 1] : peu0, me1 = k > 0 ? eu1[k - 1] : peu1;
      const FT mRr = k > 0 ? Rr[k - 1] : pRr, mRe = k > 0 ? Re[k - 1] : pRe;
      if (f >= 1 && f - 1 < Nv) {
        aa += ur0[k] * mr0 + ue0[k] * me0;
        bb += ur0[k] * mr1 + ue0[k] * me1;
        rhs += ur0[k] * mRr + ue0[k] * mRe;
      }
      if (f < Nv) {
        bb += ur1[k] * ru0[k] - ue0[k] * eu0[k];
        cc += ur1[k] * ru1[k] - ue0[k] * eu1[k];
        rhs += ur1[k] * Rr[k] - ue0[k] * Re[k];
      }
      if (f >= Nf) { aa = FT(0); bb = FT(1); cc = FT(0); rhs = FT(0); }
      a[k] = aa; b[k] = bb; c[k] = cc; d[k] = rhs;
    }
  }
  FT x[CM];
  solve_lanes<FT, G, CM>(a, b, c, d, x, gl);
  const FT xns = down<G>(x[0], 1);
  const FT xn = gl + 1 < G ? xns : FT(0);
  // ---- back-substitution and update; u_3 filtered again
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const int f = r0 + k;
    const FT xu = k + 1 < CM ? x[k + 1] : xn;
    FT rho = U[0][k] - (ru0[k] * x[k] + ru1[k] * xu - Rr[k]);
    FT rhoe = U[3][k] - (eu0[k] * x[k] + eu1[k] * xu - Re[k]);
    if (f >= Nv) { rho = FT(1); rhoe = FT(1); }
    U[0][k] = rho;
    U[3][k] = rhoe;
    if constexpr (LV::TOPO) U[4][k] = (f == 0 || f == Nv) ? u3[k] : (f > Nv ? FT(0) : u3[k] - x[k]);
    else U[4][k] = (f == 0 || f >= Nv) ? FT(0) : u3[k] - x[k];
  }
}

// Post-Newton van Leer minus central correction of rho e_tot
// (correct_implicit_advection_tendency!, implicit_tendency.jl:322-339), added
// as rhoe += dtgamma * corr.  U holds the Newton result (filtered u_3).
template <class FT, int G, int CM, class LV>
__device__ __forceinline__ void vanleer_correct(const DevParams<FT> &P, const ColGeo<FT> &Gm, const LV &L,
                                                int gl, FT dtg, FT (&U)[5][CM], const FT (&iJc)[CM]) {
  const int Nv = L.Nv, Nf = L.Nf;
  const int r0 = gl * CM;
  const FT w3ns = down<G>(U[4][0], 1);
  const FT w3n = gl + 1 < G ? w3ns : FT(0);
  FT g33[CM + 1];
#pragma unroll
  for (int k = 0; k <= CM; ++k) g33[k] = L.f4(min(r0 + k, Nf - 1)).x;
  FT hh[CM], rJ[CM], ct[CM];
  {
    FT w3a[CM], w3b[CM], ga[CM], gb[CM];
    Cen<FT> cc[CM];
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      w3a[k] = U[4][k];
      w3b[k] = k + 1 < CM ? U[4][k + 1] : w3n;
      ga[k] = g33[k];
      gb[k] = g33[k + 1];
    }
    cdiag_lane<FT, CM>(P, Gm, L, r0, U, w3a, w3b, ga, gb, cc);
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      hh[k] = cc[k].h;
      rJ[k] = cc[k].rJ;
      ct[k] = cc[k].ct3;
    }
  }
  const FT hm2 = up<G>(hh[CM - 2], 1), hm1 = up<G>(hh[CM - 1], 1), rJm = up<G>(rJ[CM - 1], 1);
  const FT hp0 = down<G>(hh[0], 1), hp1 = down<G>(hh[1], 1), rJp = down<G>(rJ[0], 1);
  FT ctm = FT(0), ctp = FT(0);
  if constexpr (LV::TOPO) {
    ctm = up<G>(ct[CM - 1], 1);
    ctp = down<G>(ct[0], 1);
  }
  FT fup[CM + 1], fcen[CM + 1];
#pragma unroll
  for (int k = 0; k <= CM; ++k) {
    const int f = r0 + k;
    const bool inner = f > 0 && f < Nv;
    const FT hA2 = k >= 2 ? hh[k - 2] : (k == 1 ? hm1 : hm2);
    const FT hA1 = k >= 1 ? hh[k - 1] : hm1;
    const FT h0 = k < CM ? hh[k] : hp0;
    const FT hP1 = k + 1 < CM ? hh[k + 1] : (k + 1 == CM ? hp0 : hp1);
    const FT rA = k >= 1 ? rJ[k - 1] : rJm;
    const FT r0v = k < CM ? rJ[k] : rJp;
    const FT wk = k < CM ? U[4][k] : w3n;
    FT u = wk * g33[k];
    if constexpr (LV::TOPO) {
      // u^3 = ᶠwinterp(rho J, CT3(u_h)) + g^33 u_3
      const FT cA = k >= 1 ? ct[k >= 1 ? k - 1 : 0] : ctm, c0 = k < CM ? ct[k < CM ? k : 0] : ctp;
      u += (rA * cA + r0v * c0) / (rA + r0v);
    }
    const FT rJb = (rA + r0v) / FT(2);
    const bool near = f == 1 || f == Nv - 1;
    fup[k] = inner ? rJb * vanleer_g(u, hA2, hA1, h0, hP1, near, P.dt_model) : FT(0);
    fcen[k] = inner ? rJb * (u * (hA1 + h0) / FT(2)) : FT(0);
  }
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const FT corr = -((fup[k + 1] - fup[k]) * iJc[k]) + ((fcen[k + 1] - fcen[k]) * iJc[k]);
    U[3][k] += dtg * corr;
  }
}

// Sums over the lane group, the same in every lane (TwoSum is exact, so the
// butterfly's operand order does not matter); every lane of the warp calls it.
template <int G, class FT>
__device__ __forceinline__ void group_sum(CSum<FT> (&ss)[3]) {
#pragma unroll
  for (int q = 0; q < 3; ++q)
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) ss[q].add(ss[q].xor_shfl(o, G));
}

// The column's sums over its lane group for the stage kernel's residual norms: each lane's
// compensated pair is rounded to one value and the group adds those in plain arithmetic
// (a butterfly, the same in every lane).  In FP32 the column sum then carries a relative
// error of at most ~log2(G) + 1 roundings (<= 4e-7), against ~2^-44 for the compensated
// butterfly of group_sum at about a third of its instructions; the sums across columns
// stay compensated.  In FP64 it is the plain sum.
template <int G, class FT>
__device__ __forceinline__ void group_sum_rounded(CSum<FT> (&ss)[3]) {
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    FT v = ss[q].hi + ss[q].lo;
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, G);
    ss[q].hi = v;
    ss[q].lo = FT(0);
  }
}

template <int G, class FT>
__device__ __forceinline__ void group_sum1(CSum<FT> &v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v.add(v.xor_shfl(o, G));
}

}  // namespace col
}  // namespace gb
