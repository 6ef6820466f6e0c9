// Implicit stage kernel: G lanes per column, CM (2 or 4) consecutive levels per lane.
//
// Fuses, for one implicit ARS343 stage, what ClimaTimeSteppers does through
// the hooks (src/simulation/integrator.jl:189-225):
//   stage assembly U^ = u_n + dt sum_j (a~_ij T_exp_j + a_ij T_imp_j),
//   impenetrable filter (precomputed_quantities.jl:486-553),
//   implicit_tendency! residual R = U^ + dtgamma T_imp(U) - U
//     (implicit_tendency.jl:185-298),
//   update_jacobian! blocks (manual_sparse_jacobian.jl:713-870, dry, no
//     topography; the (u_3, u_h) block multiplies R_uh = 0 and is skipped),
//   ldiv! with BlockArrowheadSolve(rho, rho e_tot; alg2 = u_h)
//     (manual_sparse_jacobian.jl:580-583): Schur complement onto u_3,
//   U -= dY; filter; van Leer minus central post-Newton correction
//     (implicit_tendency.jl:322-339) applied as U += dtgamma * corr,
//   T_imp_i = (U - U^) / dtgamma and FP64 residual sums of squares.
// Each lane streams its CM levels in registers; the only cross-lane traffic is
// a one-level halo per quantity and the tridiagonal solve: log2(CM) in-lane
// cyclic-reduction levels reduce the lane's CM rows to one, parallel cyclic
// reduction solves the G reduced rows across the lane group, and the
// eliminated rows are back-substituted in-lane.
#include <cstdio>
#include <cstdlib>

#include "kernels.cuh"

namespace gb {

namespace {

constexpr int CG_THREADS = 128;

template <int G, class FT>
__device__ __forceinline__ FT up(FT v, int d) { return __shfl_up_sync(0xffffffffu, v, d, G); }
template <int G, class FT>
__device__ __forceinline__ FT down(FT v, int d) { return __shfl_down_sync(0xffffffffu, v, d, G); }

// Centre diagnostics of one level from (rho, u_1, u_2, rho e_tot), the u_3 of
// the faces below/above and their g^33.
template <class FT>
struct Cen {
  FT rJ, h, phir, Pi, thv, thvr, K, iJ, phi;
};
template <class FT>
__device__ __forceinline__ Cen<FT> cdiag(const DevParams<FT> &P, const ColGeo<FT> &G, int v, FT rho, FT u1, FT u2,
                                         FT rhoe, FT u3a, FT u3b, FT g33a, FT g33b) {
  const Lev4<FT> L = P.lc4[min(max(v, 0), P.Nv - 1)];
  const FT c1 = (G.gu0 * u1 + G.gu1 * u2) * L.z, c2 = (G.gu1 * u1 + G.gu2 * u2) * L.z;
  const FT kv = (u3a * (u3a * g33a) + u3b * (u3b * g33b)) / FT(2);
  Cen<FT> o;
  o.K = (u1 * c1 + u2 * c2 + kv) / FT(2);
  Thermo<FT> th;
  thermo(P, rho, rhoe, o.K, L.w, th);
  o.h = th.h;
  o.phir = th.phir;
  o.Pi = th.Pi;
  o.thv = th.thv;
  o.thvr = th.thvr;
  o.iJ = G.iJh * L.y;
  o.rJ = rho * (G.Jh * L.x);
  o.phi = L.w;
  return o;
}

// Tridiagonal solve of the CM*G rows held CM per lane by a G-lane group.
template <class FT, int G, int CM>
__device__ __forceinline__ void solve8(FT (&a)[CM], FT (&b)[CM], FT (&c)[CM], FT (&d)[CM], FT (&x)[CM], int gl) {
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
  const FT x8s = down<G>(x[0], 1);  // every lane shuffles; the column's last lane discards it
  const FT x8 = gl + 1 < G ? x8s : FT(0);
#pragma unroll
  for (int s = CM / 2; s >= 1; s >>= 1) {
#pragma unroll
    for (int m = s; m < CM; m += 2 * s) {
      const FT xu = m + s < CM ? x[m + s] : x8;
      x[m] = gdiv(d[m] - a[m] * x[m - s] - c[m] * xu, b[m]);
    }
  }
}

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

template <class FT, int G, int CM, int STG, int MINB>
__global__ void __launch_bounds__(CG_THREADS, MINB) k_col_stage_g(DevParams<FT> P, StageArgs<FT> A) {
  const int lane = threadIdx.x & 31, gl = lane % G;
  const int col0 = (blockIdx.x * (CG_THREADS / 32) + (threadIdx.x >> 5)) * (32 / G) + lane / G;
  const int ncols = P.Nh * NN;
  const bool colv = col0 < ncols;
  const int col = colv ? col0 : ncols - 1;  // idle groups compute on a valid column, write nothing
  const int e = col >> 4, n = col & 15, Nv = P.Nv, Nf = P.Nf;
  const int r0 = gl * CM;   // first level of this lane
  const int sc = NN * Nv;   // component stride of the centre fields
  ColGeo<FT> Gm;
  Gm.load(P, e, n);
  const FT dtg = A.dtg;
  // per-lane bases: level r0 of this column; levels past the column are not read
  const size_t cb = (size_t)e * 4 * NN * Nv + (size_t)n * Nv + r0, rb = (size_t)e * 2 * NN * Nv + (size_t)n * Nv + r0;
  const size_t fb = ((size_t)e * NN + n) * Nf + r0;
  // ---- stage assembly U^ = u_n + sum_j (dt a~_ij T_exp_j + dt a_ij T_imp_j)
  FT H[5][CM];
  {
    const FT *pc = A.un_c + cb, *pf = A.un_f + fb;
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const bool okc = r0 + k < Nv, okf = r0 + k < Nf;
#pragma unroll
      for (int c = 0; c < 4; ++c) H[c][k] = okc ? pc[c * sc + k] : FT(0);
      H[4][k] = okf ? pf[k] : FT(0);
    }
  }
  // sources one at a time, summed in the tableau order
#pragma unroll
  for (int j = 0; j < STG; ++j) {
    FT t[5][CM];
    const FT *tc = A.te_c[j] + cb, *tf = A.te_f[j] + fb;
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const bool okc = r0 + k < Nv, okf = r0 + k < Nf;
#pragma unroll
      for (int c = 0; c < 4; ++c) t[c][k] = okc ? tc[c * sc + k] : FT(0);
      t[4][k] = okf ? tf[k] : FT(0);
    }
    FT q[3][CM];
    if (j >= 1) {
      const FT *qc = A.ti_c[j] + rb, *qf = A.ti_f[j] + fb;
#pragma unroll
      for (int k = 0; k < CM; ++k) {
        const bool okc = r0 + k < Nv, okf = r0 + k < Nf;
        q[0][k] = okc ? qc[k] : FT(0);
        q[1][k] = okc ? qc[sc + k] : FT(0);
        q[2][k] = okf ? qf[k] : FT(0);
      }
    }
#pragma unroll
    for (int k = 0; k < CM; ++k) {
#pragma unroll
      for (int c = 0; c < 5; ++c) {
        H[c][k] += A.ce[j] * t[c][k];
        if (j >= 1 && c != 1 && c != 2) H[c][k] += A.ci[j] * q[c == 0 ? 0 : (c == 3 ? 1 : 2)][k];
      }
    }
  }
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const int v = r0 + k;
    if (v >= Nv) { H[0][k] = FT(1); H[1][k] = FT(0); H[2][k] = FT(0); H[3][k] = FT(1); }
    if (v >= Nf) H[4][k] = FT(0);
  }
  // face geometry of faces r0 .. r0 + CM and g^33 of face r0 - 1
  Lev4<FT> LF[CM + 1];
#pragma unroll
  for (int k = 0; k <= CM; ++k) LF[k] = P.lf4[min(r0 + k, Nf - 1)];
  const FT g33m = P.lf4[min(max(r0 - 1, 0), Nf - 1)].x;
  // ---- filtered state U: u_3 = 0 on the boundary faces
  FT u3[CM];
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const int f = r0 + k;
    u3[k] = (f == 0 || f >= Nv) ? FT(0) : H[4][k];
  }
  // halo: centre -1 and face -1 from the previous lane, face r0 + CM from the next lane
  const FT hr = up<G>(H[0][CM - 1], 1), hu1 = up<G>(H[1][CM - 1], 1), hu2 = up<G>(H[2][CM - 1], 1);
  const FT he = up<G>(H[3][CM - 1], 1), h3 = up<G>(u3[CM - 1], 1);
  const FT n3 = down<G>(u3[0], 1);  // every lane shuffles; the column's last lane discards it
  const FT u3n = gl + 1 < G ? n3 : FT(0);
  // ---- centre diagnostics r0-1 .. r0+CM-1 and face quantities r0 .. r0+CM-1 (streamed)
  FT F[CM + 1], Fh[CM + 1], fr[CM + 1], fhb[CM + 1];
  FT T3[CM], ur0[CM], ur1[CM], ue0[CM], uu0[CM], uu1[CM], uu2[CM];
  FT iJc[CM];
  const FT kap = P.Rd * P.icvd;
  const FT h3m = gl > 0 ? h3 : FT(0);
  Cen<FT> prev = cdiag(P, Gm, r0 - 1, gl > 0 ? hr : FT(1), hu1, hu2, gl > 0 ? he : FT(1), h3m, u3[0], g33m, LF[0].x);
  FT rhoPrev = gl > 0 ? hr : FT(1);
  FT u3cPrev = h3m * g33m;
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const int f = r0 + k;
    const FT u3next = k + 1 < CM ? u3[k + 1] : u3n;
    const Cen<FT> cur = cdiag(P, Gm, f, H[0][k], H[1][k], H[2][k], H[3][k], u3[k], u3next, LF[k].x, LF[k + 1].x);
    iJc[k] = cur.iJ;
    const bool inner = f > 0 && f < Nv;
    const FT g33 = LF[k].x;
    const FT u3c = u3[k] * g33;
    const FT rJb = (prev.rJ + cur.rJ) / FT(2);
    const FT hb = (prev.h + cur.h) / FT(2);
    F[k] = inner ? rJb * u3c : FT(0);
    Fh[k] = F[k] * hb;
    fr[k] = inner ? rJb * g33 : FT(0);
    fhb[k] = hb;
    const FT beta = LF[k].y;
    FT t3 = FT(0);
    if (inner) {
      const FT thd = ((prev.thv - prev.thvr) + (cur.thv - cur.thvr)) / FT(2);
      t3 = -(LF[k].z - (cur.phir - prev.phir) + P.cpd * thd * (cur.Pi - prev.Pi));
    }
    T3[k] = t3 - beta * u3[k];
    if (inner) {
      const FT ra = rhoPrev, rbv = H[0][k];
      const FT irb = grcp((ra + rbv) / FT(2));
      const FT dpa = kap * (P.T0 * P.cpd - prev.K - prev.phi);
      const FT dpb = kap * (P.T0 * P.cpd - cur.K - cur.phi);
      const FT buoy = P.cpd * ((prev.thv + cur.thv) / FT(2)) * (cur.Pi - prev.Pi) * irb;
      ur0[k] = dtg * (dpa * irb + buoy / FT(2));
      ur1[k] = dtg * (-dpb * irb + buoy / FT(2));
      ue0[k] = dtg * (kap * irb);
      const FT u3cn = u3next * LF[k + 1].x;
      uu0[k] = dtg * (-kap * ra * u3cPrev * (irb / FT(2)));
      uu1[k] = dtg * (kap * (rbv - ra) * u3c * (irb / FT(2)) - beta) - FT(1);
      uu2[k] = dtg * (kap * rbv * u3cn * (irb / FT(2)));
    } else {
      ur0[k] = ur1[k] = ue0[k] = uu0[k] = uu2[k] = FT(0);
      uu1[k] = f <= Nv ? -dtg * beta - FT(1) : FT(1);
    }
    prev = cur;
    rhoPrev = H[0][k];
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
  double ss[3] = {0, 0, 0};
  bool finite = true;
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const int v = r0 + k;
    const bool cv = v < Nv;
    const FT Tr = -((F[k + 1] - F[k]) * iJc[k]);
    const FT Te = -((Fh[k + 1] - Fh[k]) * iJc[k]);
    Rr[k] = cv ? dtg * Tr : FT(0);
    Re[k] = cv ? dtg * Te : FT(0);
    const FT v0 = fr[k] * iJc[k], v1 = -fr[k + 1] * iJc[k];
    ru0[k] = cv ? dtg * v0 : FT(0);
    ru1[k] = cv ? dtg * v1 : FT(0);
    eu0[k] = cv ? dtg * (v0 * fhb[k]) : FT(0);
    eu1[k] = cv ? dtg * (v1 * fhb[k + 1]) : FT(0);
    ss[0] += (double)(Rr[k] * Rr[k]);
    ss[1] += (double)(Re[k] * Re[k]);
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
      if (f < Nf) R3 = dtg * T3[k] + (H[4][k] - u3[k]);
      ss[2] += (double)(R3 * R3);
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
  solve8<FT, G, CM>(a, b, c, d, x, gl);
  const FT x8s = down<G>(x[0], 1);
  const FT x8 = gl + 1 < G ? x8s : FT(0);
  // ---- back-substitution and update; U.u_3 filtered again
  FT rho[CM], rhoe[CM], w3[CM];
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const int f = r0 + k;
    const FT xu = k + 1 < CM ? x[k + 1] : x8;
    rho[k] = H[0][k] - (ru0[k] * x[k] + ru1[k] * xu - Rr[k]);
    rhoe[k] = H[3][k] - (eu0[k] * x[k] + eu1[k] * xu - Re[k]);
    w3[k] = (f == 0 || f >= Nv) ? FT(0) : u3[k] - x[k];
    if (f >= Nv) { rho[k] = FT(1); rhoe[k] = FT(1); }
  }
  // ---- post-Newton van Leer correction of rho e_tot
  if (P.upwinding) {
    const FT w3ns = down<G>(w3[0], 1);
    const FT w3n = gl + 1 < G ? w3ns : FT(0);
    FT hh[CM], rJ[CM];
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const FT wn = k + 1 < CM ? w3[k + 1] : w3n;
      const Cen<FT> cc = cdiag(P, Gm, r0 + k, rho[k], H[1][k], H[2][k], rhoe[k], w3[k], wn, LF[k].x, LF[k + 1].x);
      hh[k] = cc.h;
      rJ[k] = cc.rJ;
    }
    const FT hm2 = up<G>(hh[CM - 2], 1), hm1 = up<G>(hh[CM - 1], 1), rJm = up<G>(rJ[CM - 1], 1);
    const FT hp0 = down<G>(hh[0], 1), hp1 = down<G>(hh[1], 1), rJp = down<G>(rJ[0], 1);
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
      const FT wk = k < CM ? w3[k] : w3n;
      const FT u = wk * LF[k].x;
      const FT rJb = (rA + r0v) / FT(2);
      const bool near = f == 1 || f == Nv - 1;
      fup[k] = inner ? rJb * vanleer_g(u, hA2, hA1, h0, hP1, near, P.dt_model) : FT(0);
      fcen[k] = inner ? rJb * (u * (hA1 + h0) / FT(2)) : FT(0);
    }
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const FT corr = -((fup[k + 1] - fup[k]) * iJc[k]) + ((fcen[k + 1] - fcen[k]) * iJc[k]);
      rhoe[k] += dtg * corr;
    }
  }
  // ---- outputs (u_h passes through the implicit stage unchanged)
  const FT idtg = A.idtg;
  {
    FT *uc = A.U_c + cb, *uf = A.U_f + fb, *tc = A.Ti_c + rb, *tf = A.Ti_f + fb;
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const int v = r0 + k;
      if (colv && v < Nv) {
        uc[k] = rho[k];
        uc[sc + k] = H[1][k];
        uc[2 * sc + k] = H[2][k];
        uc[3 * sc + k] = rhoe[k];
        tc[k] = (rho[k] - H[0][k]) * idtg;
        tc[sc + k] = (rhoe[k] - H[3][k]) * idtg;
      }
      if (colv && v < Nf) {
        uf[k] = w3[k];
        tf[k] = (w3[k] - H[4][k]) * idtg;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 3; ++q)
    for (int o = G / 2; o > 0; o >>= 1) ss[q] += __shfl_xor_sync(0xffffffffu, ss[q], o, G);
  finite = __all_sync(0xffffffffu, finite);
  if (gl == 0 && colv) {
    if (A.rnorm)
      for (int q = 0; q < 3; ++q) A.rnorm[(size_t)col * 3 + q] = (A.first ? 0.0 : A.rnorm[(size_t)col * 3 + q]) + ss[q];
  }
  if (lane == 0 && !finite) atomicOr(P.status, ST_NONFINITE);
}

template <class FT, int G, int CM, int MINB>
void launch_g(const DevParams<FT> &P, const StageArgs<FT> &A, cudaStream_t s) {
  const int ncols = P.Nh * NN, per_cta = (CG_THREADS / 32) * (32 / G);
  const int grid = (ncols + per_cta - 1) / per_cta;
  switch (A.nsrc) {
    case 1: k_col_stage_g<FT, G, CM, 1, MINB><<<grid, CG_THREADS, 0, s>>>(P, A); break;
    case 2: k_col_stage_g<FT, G, CM, 2, MINB><<<grid, CG_THREADS, 0, s>>>(P, A); break;
    default: k_col_stage_g<FT, G, CM, 3, MINB><<<grid, CG_THREADS, 0, s>>>(P, A); break;
  }
}

// Levels per lane CM and the register cap (min resident CTAs per SM) of a variant.
template <class FT, int CM, int MINB>
void launch_cm(const DevParams<FT> &P, const StageArgs<FT> &A, cudaStream_t s) {
  // G lanes x CM levels >= Nv + 1 faces, G a power of two in 4..32
  const int need = (P.Nf + CM - 1) / CM;
  if (need <= 4) launch_g<FT, 4, CM, MINB>(P, A, s);
  else if (need <= 8) launch_g<FT, 8, CM, MINB>(P, A, s);
  else if (need <= 16) launch_g<FT, 16, CM, MINB>(P, A, s);
  else launch_g<FT, 32, CM, MINB>(P, A, s);
}

int column_variant_env() {
  static const int v = [] {
    const char *e = getenv("GBDYCORE_COLUMN_VARIANT");
    return e ? atoi(e) : -1;
  }();
  return v;
}

}  // namespace

// A.nsrc = stage index (1..3); all explicit sources j < nsrc and implicit
// sources 1 <= j < nsrc must be present (the ARS343 nonzero pattern).
template <class FT>
void launch_column_stage(const DevParams<FT> &P, const StageArgs<FT> &A, cudaStream_t s) {
  // the kernel reads every source below nsrc unconditionally: refuse a missing one
  bool ok = A.nsrc >= 1 && A.nsrc <= 3 && A.un_c && A.un_f && A.U_c && A.U_f && A.Ti_c && A.Ti_f;
  for (int j = 0; ok && j < A.nsrc; ++j) ok = A.te_c[j] && A.te_f[j] && (j == 0 || (A.ti_c[j] && A.ti_f[j]));
  if (!ok) {
    fprintf(stderr, "gbdycore: column stage launched with a missing source (nsrc=%d); not launched\n", A.nsrc);
    return;
  }
  // Variants (levels per lane CM, register cap as min resident 128-thread CTAs per SM).
  // Measured on GB300 at z_elem = 63, FP32, stage 4: CM 4 uncapped (160 registers)
  // 0.272 ms, CM 4 / 4 CTAs 0.205 ms, CM 2 uncapped 0.259 ms, CM 2 / 6 CTAs 0.174 ms.
  // Default: CM 2 / 6 CTAs when two levels per lane cover the column (Nf <= 64),
  // else CM 4 / 4 CTAs.  GBDYCORE_COLUMN_VARIANT=0..6 overrides it for tuning.
  int v = column_variant_env();
  if (v < 0 || v > 6) v = P.Nf <= 64 ? 3 : 1;
  if ((v == 2 || v == 3 || v == 4 || v == 6) && P.Nf > 64) v = 1;  // CM 2 covers at most 64 faces
  switch (v) {
    case 0: launch_cm<FT, 4, 1>(P, A, s); break;
    case 2: launch_cm<FT, 2, 1>(P, A, s); break;
    case 3: launch_cm<FT, 2, 6>(P, A, s); break;
    case 4: launch_cm<FT, 2, 8>(P, A, s); break;
    case 5: launch_cm<FT, 4, 5>(P, A, s); break;
    case 6: launch_cm<FT, 2, 7>(P, A, s); break;
    default: launch_cm<FT, 4, 4>(P, A, s); break;
  }
}

template void launch_column_stage<float>(const DevParams<float> &, const StageArgs<float> &, cudaStream_t);
template void launch_column_stage<double>(const DevParams<double> &, const StageArgs<double> &, cudaStream_t);

}  // namespace gb
