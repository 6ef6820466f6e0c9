// Shared device-side definitions of the GB300 dry dynamical core.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "geometry.h"

namespace gb {

// Device status word bits (read back by the host).
enum : int { ST_TIMEOUT = 1, ST_NONFINITE = 2 };
// Time limit (ns, device global timer) of every bounded wait on an mbarrier.
constexpr unsigned long long WAIT_LIMIT_NS = 1000000000ull;

// Four per-level values in one aligned 16-byte (FP32) or 32-byte (FP64) load.
template <class FT>
struct alignas(4 * sizeof(FT)) Lev4 {
  FT x, y, z, w;
};

template <class FT>
struct DevParams {
  int Nh, Nv, Nf, ngroups;
  FT grav, Rd, cpd, cvd, T0, pref, kappa, Tmin_ref, Tsfc_ref, Tmin_sgs, icvd, ipref;
  FT nu_v, nu_s, div_damp, dt_model;
  int upwinding;
  // Held-Suarez forcing: k_a, k_s - k_a, k_f; sigma_b, 1 / (1 - sigma_b); Delta T_y, T_equator,
  // Delta theta_z, T_min; 1 / p_ref_theta, 1 / MSLP
  int hs;
  FT hs_ka, hs_dk, hs_kf, hs_sb, hs_isb, hs_dTy, hs_Teq, hs_dthz, hs_Tmin, hs_ip0, hs_iMSLP;
  FT W[NN], iW[NN];
  alignas(16) FT D[NQ * NQ];   // D[i*4+k] = l_k'(xi_i)
  alignas(16) FT DT[NQ * NQ];  // the transpose, DT[k*4+i] = D[i*4+k] (pairs of rows of a column)
  const FT *hgeo;  // [Nh][HG_N][16]
  const FT *levc;  // [LC_N][Nv]
  const FT *levf;  // [LF_N][Nf]
  const Lev4<FT> *lc4;  // [Nv] centres: {r^2 dz, 1 / (r^2 dz), 1 / r^2, Phi}
  const Lev4<FT> *lf4;  // [Nf] faces: {g^33, beta_w, Phi_c(v) - Phi_c(v-1) (0 on the boundary faces), 0}
  // [Nv] centres: the level's reference record {p0, 1 / p0, cp_d (T_sfc - T_min) / 7 Pi0^7, 0}
  // (reference_level, geometry.h) for Phi - Phi_r in deviation form
  const Lev4<FT> *lr4;
  FT cpTmin;  // cp_d T_min_ref
  const int *goff, *gcopy;
  const FT *gw, *ecov, *econ;  // ecov/econ: [Nh*16][6]
  int *status;
  // Terrain-following levels (topo = 1): per node z_s and its xi^1, xi^2 derivatives in the
  // element ([Nh][TG_N][16]); per level the warp records {zeta, b, dzeta, db} of the centres
  // (ltc [Nv]) and faces (ltf [Nf]), so that a point's height is zeta + z_s b and its layer
  // thickness dzeta + z_s db; 1 / R; the Rayleigh sponge of each point, beta = alpha
  // sin^2(spg_k (z - spg_zd)) above spg_zd (spg_k = pi / (2 (z_max - z_d))).
  int topo;
  const FT *tgeo;
  const Lev4<FT> *ltc, *ltf;
  FT iR, spg_auh, spg_aw, spg_zd, spg_k;
  // Moist 0M (moist = 1): R_v; cv of vapour, liquid and ice; cp_v - cp_l, cp_v - cp_i; L_v0,
  // L_s0; 1 / T_triple, p_triple; T_freeze, T_icenuc, 1 / (T_freeze - T_icenuc), pow_icenuc;
  // e_int_v0 = L_v0 - R_v T_0, e_int_i0 = L_s0 - L_v0; Newton iterations of the adjustment
  int moist, sa_iters;
  FT Rv, cvv, cvl, cvi, dcl, dci, Lv0, Ls0, iTtr, ptr, Tfrz, Tice, iTrng, pice, ev0, ei0;
};

// ---------------------------------------------------------------- math
// FP32 uses the hardware approximations (ex2/lg2/rcp based, a few ulp); FP64
// keeps the correctly rounded library functions and IEEE division.
__device__ __forceinline__ float gpow(float x, float y) { return __powf(x, y); }
__device__ __forceinline__ double gpow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float glog(float x) { return __logf(x); }
__device__ __forceinline__ double glog(double x) { return log(x); }
__device__ __forceinline__ float gdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double gdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float grcp(float a) { return __fdividef(1.0f, a); }
__device__ __forceinline__ double grcp(double a) { return 1.0 / a; }
__device__ __forceinline__ float gsin(float x) { return sinf(x); }
__device__ __forceinline__ double gsin(double x) { return sin(x); }
// ln(p / p0) for p near p0, and exp(x) - 1 for small x.  FP64: the library's log1p and expm1
// (accurate near 0).  FP32: the hardware ln of the ratio p (1/p0), whose absolute error
// (~2e-7) is below what the FP32 pressure itself carries (~3e-7 relative), and exp - 1 by
// the hardware exp (absolute error ~2e-7 on a term scaled by cp (T_sfc - T_min) Pi0^7 / 7,
// i.e. a few 1e-3 J/kg): a few instructions instead of two full function evaluations.
__device__ __forceinline__ float glog_ratio(float p, float p0, float ip0) {
  (void)p0;
  return __logf(p * ip0);
}
__device__ __forceinline__ double glog_ratio(double p, double p0, double ip0) { return log1p((p - p0) * ip0); }
__device__ __forceinline__ float gexpm1(float x) { return __expf(x) - 1.0f; }
__device__ __forceinline__ double gexpm1(double x) { return expm1(x); }
__device__ __forceinline__ float gexp(float x) { return __expf(x); }
__device__ __forceinline__ double gexp(double x) { return exp(x); }

template <class FT>
__device__ __forceinline__ FT shfl(FT v, int src, int width) {
  return __shfl_sync(0xffffffffu, v, src, width);
}
template <class FT>
__device__ __forceinline__ FT shfl_up(FT v, int d) {
  return __shfl_up_sync(0xffffffffu, v, d);
}
template <class FT>
__device__ __forceinline__ FT shfl_down(FT v, int d) {
  return __shfl_down_sync(0xffffffffu, v, d);
}

// Dry thermodynamics of Thermodynamics.jl with e_int = cv_d (T - T_0) - R_d T_0,
// and the hydrostatic reference state of src/utils/refstate_thermodynamics.jl.
// phid = Phi - Phi_r(Pi), the geopotential less the reference state's at the point's
// Exner pressure, which the pressure-gradient and hyperdiffusion terms take
// (advection.jl:82-88, implicit_tendency.jl:286-293, hyperdiffusion.jl:142-147).
// It is formed as a deviation from the level's reference record rl (Phi_r(Pi0) = Phi at
// p0 = rl.x): with ln x = kappa ln(p / p0),
//   Phi - Phi_r(Pi) = cp_d T_min ln x + cp_d (T_sfc - T_min) / 7 Pi0^7 expm1(7 ln x),
// the same quantity as Phi - Phi_r(Pi) written directly, without the cancellation of two
// O(1e5) J/kg terms that costs FP32 most of its precision there.
template <class FT>
struct Thermo {
  FT T, p, h, Pi, thv, thvr, phid, Tr;
};
template <class FT>
__device__ __forceinline__ void thermo(const DevParams<FT> &P, FT rho, FT rhoe, FT K, FT Phi, const Lev4<FT> &rl,
                                       Thermo<FT> &o) {
  FT e_tot = gdiv(rhoe, rho);
  FT eint = e_tot - K - Phi;
  FT T = P.T0 + (eint + P.Rd * P.T0) * P.icvd;
  T = T > P.Tmin_sgs ? T : P.Tmin_sgs;
  FT p = rho * P.Rd * T;
  FT Pi = gpow(p * P.ipref, P.kappa);
  FT Pi2 = Pi * Pi, Pi7 = Pi2 * Pi2 * Pi2 * Pi;
  FT Tr = P.Tmin_ref + (P.Tsfc_ref - P.Tmin_ref) * Pi7;
  FT iPi = grcp(Pi);
  o.T = T;
  o.p = p;
  o.h = e_tot + P.Rd * T;
  o.Pi = Pi;
  o.thv = T * iPi;
  o.thvr = Tr * iPi;
  o.Tr = Tr;
  const FT lx = P.kappa * glog_ratio(p, rl.x, rl.y);
  o.phid = P.cpTmin * lx + rl.z * gexpm1(FT(7) * lx);
}
// thermo() for two points at once in FP32 (packed multiplies and adds; the hardware ln, exp,
// power and reciprocal per point): geopotential Phi and the reference record's 1/p0 (ip0)
// and cp_d (T_sfc - T_min) / 7 Pi0^7 (rz) per point, so the two may sit on different levels.
__device__ __forceinline__ float2 bc2(float x) { return make_float2(x, x); }
__device__ __forceinline__ void thermo_pair(const DevParams<float> &P, float2 rho, float2 rhoe, float2 K, float2 Phi,
                                            float2 ip0, float2 rz, float2 &T, float2 &p, float2 &h, float2 &Pi,
                                            float2 &thv, float2 &thvr, float2 &phid, float2 &Tr) {
  const float2 e = make_float2(gdiv(rhoe.x, rho.x), gdiv(rhoe.y, rho.y));
  const float2 eint = __ffma2_rn(Phi, bc2(-1.0f), __ffma2_rn(K, bc2(-1.0f), e));
  T = __ffma2_rn(__fadd2_rn(eint, bc2(P.Rd * P.T0)), bc2(P.icvd), bc2(P.T0));
  T = make_float2(T.x > P.Tmin_sgs ? T.x : P.Tmin_sgs, T.y > P.Tmin_sgs ? T.y : P.Tmin_sgs);
  p = __fmul2_rn(__fmul2_rn(rho, bc2(P.Rd)), T);
  const float2 x = __fmul2_rn(p, bc2(P.ipref));
  Pi = make_float2(gpow(x.x, P.kappa), gpow(x.y, P.kappa));
  const float2 Pi2 = __fmul2_rn(Pi, Pi), Pi4 = __fmul2_rn(Pi2, Pi2), Pi7 = __fmul2_rn(__fmul2_rn(Pi4, Pi2), Pi);
  Tr = __ffma2_rn(bc2(P.Tsfc_ref - P.Tmin_ref), Pi7, bc2(P.Tmin_ref));
  const float2 iPi = make_float2(grcp(Pi.x), grcp(Pi.y));
  h = __ffma2_rn(bc2(P.Rd), T, e);
  thv = __fmul2_rn(T, iPi);
  thvr = __fmul2_rn(Tr, iPi);
  // Phi - Phi_r(Pi) as the deviation from the level's reference record (see thermo())
  const float2 r = __fmul2_rn(p, ip0);
  const float2 lx = __fmul2_rn(bc2(P.kappa), make_float2(__logf(r.x), __logf(r.y)));
  const float2 e7 = __fmul2_rn(lx, bc2(7.0f));
  const float2 em = __fadd2_rn(make_float2(__expf(e7.x), __expf(e7.y)), bc2(-1.0f));
  phid = __ffma2_rn(rz, em, __fmul2_rn(bc2(P.cpTmin), lx));
}

// ---- moist thermodynamics (EquilibriumMicrophysics0M) ----
// The formulation of Thermodynamics.jl 1.3.0 that the reference's Jacobian assumes (its dp/drho
// and dp/d(rho q_tot), manual_sparse_jacobian.jl:646-685, follow from these definitions):
//   cv_m  = cv_d + (cv_v - cv_d) q_t + (cv_l - cv_v) q_l + (cv_i - cv_v) q_i
//   R_m   = R_d (1 - q_t) + R_v (q_t - q_l - q_i)
//   e_int = cv_m (T - T_0) + q_v e_int_v0 - q_i e_int_i0 - (1 - q_t) R_d T_0
//   q_v*  = p_v*(T) / (rho R_v T),  p_v* = p_tr (T / T_tr)^(dcp / R_v) exp((L_0 - dcp T_0) / R_v (1 / T_tr - 1 / T))
//           with L_0 and dcp the liquid-fraction weighted latent heat and cp_v - cp_(l,i)
//   lam(T) = 1 above T_freeze, 0 at or below T_icenuc, ((T - T_icenuc) / (T_freeze - T_icenuc))^pow between.
// The liquid fraction and its T-derivative.
template <class FT>
__device__ __forceinline__ FT liq_frac(const DevParams<FT> &P, FT T, FT &dl) {
  if (T > P.Tfrz) { dl = FT(0); return FT(1); }
  if (!(T > P.Tice)) { dl = FT(0); return FT(0); }
  const FT x = (T - P.Tice) * P.iTrng;
  if (P.pice == FT(1)) { dl = P.iTrng; return x; }
  dl = P.pice * gpow(x, P.pice - FT(1)) * P.iTrng;
  return gpow(x, P.pice);
}
// q_v*(T, rho) and d ln q_v* / dT (the L_0 and dcp weights follow lam(T) too)
template <class FT>
__device__ __forceinline__ FT qsat(const DevParams<FT> &P, FT T, FT rho, FT &dlnq) {
  FT dl;
  const FT lam = liq_frac(P, T, dl);
  const FT iRv = grcp(P.Rv), iT = grcp(T);
  const FT dcp = lam * P.dcl + (FT(1) - lam) * P.dci, L0 = lam * P.Lv0 + (FT(1) - lam) * P.Ls0;
  const FT a = dcp * iRv, b = (L0 - dcp * P.T0) * iRv, sd = P.iTtr - iT;
  const FT lt = glog(T * P.iTtr);
  const FT ps = P.ptr * gexp(a * lt + b * sd);
  const FT dd = P.dcl - P.dci;
  const FT dlp = a * iT + b * iT * iT + dl * (dd * iRv * lt + ((P.Lv0 - P.Ls0) - dd * P.T0) * iRv * sd);
  dlnq = dlp - iT;
  return gdiv(ps, rho * P.Rv * T);
}
// The saturation adjustment in (rho, e_int, q_tot) (TD.saturation_adjustment with TD.ρe(),
// precomputed_quantities.jl:734-747): the all-vapour temperature T_u if the point is unsaturated
// there, else sa_iters safeguarded Newton iterations on f(T) = e_int(T) - e_int with the saturated
// partition q_c = q_t - q_v*(T) continued smoothly where q_v* > q_t (the clamped function's kink
// makes plain Newton cycle).  f increases with T and
// [T_u, max(T_u + q_t (e_int_v0 + e_int_i0) / cv_d, T_0) + 1] brackets its root; a step outside
// the current bracket becomes a bisection.  A lane stops once a step moves T by no more than
// 1e-9 K (FP64) or 1e-3 K (FP32) (Newton's error after it is of the order of its square).  The
// partition is that of the final T.
template <class FT>
__device__ __forceinline__ void sat_adjust(const DevParams<FT> &P, FT rho, FT eint, FT q, FT &T, FT &ql, FT &qi) {
  const FT cvm0 = P.cvd + (P.cvv - P.cvd) * q;
  T = P.T0 + gdiv(eint - q * P.ev0 + (FT(1) - q) * P.Rd * P.T0, cvm0);
  T = T > P.Tmin_sgs ? T : P.Tmin_sgs;
  FT dlnq;
  ql = qi = FT(0);
  if (q <= qsat(P, T, rho, dlnq)) return;
  FT lo = T, hi = fmax(T + gdiv(q * (P.ev0 + P.ei0), P.cvd), P.T0) + FT(1);
  for (int it = 0; it < P.sa_iters; ++it) {
    FT dl;
    const FT lam = liq_frac(P, T, dl);
    const FT qs = qsat(P, T, rho, dlnq);
    const FT qc = q - qs;
    const FT l = lam * qc, i = (FT(1) - lam) * qc;
    const FT cvm = P.cvd + (P.cvv - P.cvd) * q + (P.cvl - P.cvv) * l + (P.cvi - P.cvv) * i;
    const FT f = cvm * (T - P.T0) + qs * P.ev0 - i * P.ei0 - (FT(1) - q) * P.Rd * P.T0 - eint;
    const FT dqc = -qs * dlnq;
    const FT dql = dl * qc + lam * dqc, dqi = -dl * qc + (FT(1) - lam) * dqc;
    const FT df = cvm + (T - P.T0) * ((P.cvl - P.cvv) * dql + (P.cvi - P.cvv) * dqi) - dqc * P.ev0 - dqi * P.ei0;
    if (f < FT(0)) lo = T;
    else hi = T;
    FT Tn = T - gdiv(f, df);
    if (!(Tn >= lo && Tn <= hi)) Tn = (lo + hi) / FT(2);
    const FT dT = Tn - T;
    T = Tn;
    if (fabs(dT) <= (sizeof(FT) == 8 ? FT(1e-9) : FT(1e-3))) break;
  }
  FT dl;
  const FT lam = liq_frac(P, T, dl);
  const FT qc = fmax(FT(0), q - qsat(P, T, rho, dlnq));
  ql = lam * qc;
  qi = (FT(1) - lam) * qc;
}
// thermo() of moist air: T from the saturation adjustment of max(0, q_tot), p = rho R_m T,
// h_tot = e_tot + R_m T, theta_v = T R_m / (Pi R_d) (refstate_thermodynamics.jl:58-63); also
// q = specific(rho q_tot, rho), kappa_m = R_m / cv_m (ᶜkappa_m_field!) and dp/d(rho q_tot) at
// constant rho and rho e_tot (ᶜ∂p∂ρq_tot_field!, manual_sparse_jacobian.jl:646-685).
template <class FT>
__device__ __forceinline__ void thermo_moist(const DevParams<FT> &P, FT rho, FT rhoe, FT rhoq, FT K, FT Phi,
                                             const Lev4<FT> &rl, Thermo<FT> &o, FT &q, FT &kapm, FT &dpdq) {
  const FT irho = grcp(rho);
  const FT e_tot = rhoe * irho;
  const FT eint = e_tot - K - Phi;
  q = rhoq * irho;
  const FT qn = fmax(FT(0), q);
  FT T, ql, qi;
  sat_adjust(P, rho, eint, qn, T, ql, qi);
  const FT Rm = P.Rd * (FT(1) - qn) + P.Rv * (qn - ql - qi);
  const FT cvm = P.cvd + (P.cvv - P.cvd) * qn + (P.cvl - P.cvv) * ql + (P.cvi - P.cvv) * qi;
  const FT p = rho * Rm * T;
  const FT Pi = gpow(p * P.ipref, P.kappa);
  const FT Pi2 = Pi * Pi, Pi7 = Pi2 * Pi2 * Pi2 * Pi;
  const FT Tr = P.Tmin_ref + (P.Tsfc_ref - P.Tmin_ref) * Pi7;
  const FT iPi = grcp(Pi);
  o.T = T;
  o.p = p;
  o.h = e_tot + Rm * T;
  o.Pi = Pi;
  o.thv = gdiv(T * Rm, Pi * P.Rd);
  o.thvr = Tr * iPi;
  o.Tr = Tr;
  const FT lx = P.kappa * glog_ratio(p, rl.x, rl.y);
  o.phid = P.cpTmin * lx + rl.z * gexpm1(FT(7) * lx);
  kapm = gdiv(Rm, cvm);
  dpdq = kapm * (-P.ev0 - P.Rd * P.T0 - (P.cvv - P.cvd) * (T - P.T0)) + (P.Rv - P.Rd) * T;
}

// Reverse mode of thermo(): the cotangents of its outputs (T, p, h, Pi, thv,
// thvr, phir) and of the reference temperature T_r(Pi) give those of
// (rho, rho e_tot, K).  Uses dPi/dp = kappa Pi / p, dT_r/dPi = 7 (T_sfc - T_min) Pi^6,
// dPhi_r/dPi = -cp T_r / Pi; T has no sensitivity where it is clamped at T_min_sgs.
template <class FT>
struct ThermoBar {
  FT T, p, h, Pi, thv, thvr, phir, Tr;
};
template <class FT>
__device__ __forceinline__ void thermo_vjp(const DevParams<FT> &P, FT rho, FT rhoe, FT K, FT Phi,
                                           const ThermoBar<FT> &b, FT &rho_b, FT &rhoe_b, FT &K_b) {
  const FT e = gdiv(rhoe, rho);
  const FT Tu = P.T0 + (e - K - Phi + P.Rd * P.T0) * P.icvd;
  const bool clamped = !(Tu > P.Tmin_sgs);
  const FT T = clamped ? P.Tmin_sgs : Tu;
  const FT p = rho * P.Rd * T;
  const FT Pi = gpow(p * P.ipref, P.kappa);
  const FT Pi2 = Pi * Pi, Pi7 = Pi2 * Pi2 * Pi2 * Pi;
  const FT dT = P.Tsfc_ref - P.Tmin_ref;
  const FT Tr = P.Tmin_ref + dT * Pi7;
  const FT iPi = grcp(Pi), iPi2 = iPi * iPi;
  const FT Pib = b.Pi - T * iPi2 * b.thv + (FT(7) * dT * Pi7 - Tr) * iPi2 * b.thvr - P.cpd * Tr * iPi * b.phir +
                 FT(7) * dT * Pi7 * iPi * b.Tr;
  const FT pb = b.p + P.kappa * Pi * gdiv(Pib, p);
  const FT Tb = b.T + iPi * b.thv + P.Rd * b.h + rho * P.Rd * pb;
  FT eb = b.h;
  FT Kb = FT(0);
  if (!clamped) {
    eb += Tb * P.icvd;
    Kb = -Tb * P.icvd;
  }
  rho_b = P.Rd * T * pb - gdiv(eb * e, rho);
  rhoe_b = gdiv(eb, rho);
  K_b = Kb;
}

// thermo_vjp for two points at once in FP32: the same formulas with packed multiplies and
// adds, one reciprocal of rho per point in place of the three divisions (the hardware
// power and reciprocals per point).  Cotangents as float2 pairs.
struct ThermoBar2 {
  float2 T, p, h, Pi, thv, thvr, phir, Tr;
};
__device__ __forceinline__ void thermo_vjp_pair(const DevParams<float> &P, float2 rho, float2 rhoe, float2 K,
                                                float2 Phi, const ThermoBar2 &b, float2 &rho_b, float2 &rhoe_b,
                                                float2 &K_b) {
  const float2 m1 = bc2(-1.0f);
  const float2 irho = make_float2(grcp(rho.x), grcp(rho.y));
  const float2 e = __fmul2_rn(rhoe, irho);
  const float2 eint = __ffma2_rn(Phi, m1, __ffma2_rn(K, m1, e));
  const float2 Tu = __ffma2_rn(__fadd2_rn(eint, bc2(P.Rd * P.T0)), bc2(P.icvd), bc2(P.T0));
  const bool cx = !(Tu.x > P.Tmin_sgs), cy = !(Tu.y > P.Tmin_sgs);
  const float2 T = make_float2(cx ? P.Tmin_sgs : Tu.x, cy ? P.Tmin_sgs : Tu.y);
  const float2 p = __fmul2_rn(__fmul2_rn(rho, bc2(P.Rd)), T);
  const float2 x = __fmul2_rn(p, bc2(P.ipref));
  const float2 Pi = make_float2(gpow(x.x, P.kappa), gpow(x.y, P.kappa));
  const float2 Pi2 = __fmul2_rn(Pi, Pi), Pi4 = __fmul2_rn(Pi2, Pi2), Pi7 = __fmul2_rn(__fmul2_rn(Pi4, Pi2), Pi);
  const float dT = P.Tsfc_ref - P.Tmin_ref;
  const float2 Tr = __ffma2_rn(bc2(dT), Pi7, bc2(P.Tmin_ref));
  const float2 iPi = make_float2(grcp(Pi.x), grcp(Pi.y)), iPi2 = __fmul2_rn(iPi, iPi);
  const float2 s7 = __fmul2_rn(bc2(7.0f * dT), Pi7);
  // Pib = b.Pi - T iPi^2 b.thv + (7 dT Pi^7 - T_r) iPi^2 b.thvr - cp T_r iPi b.phir + 7 dT Pi^7 iPi b.Tr
  float2 Pib = __ffma2_rn(__fmul2_rn(__fmul2_rn(T, iPi2), m1), b.thv, b.Pi);
  Pib = __ffma2_rn(__fmul2_rn(__ffma2_rn(Tr, m1, s7), iPi2), b.thvr, Pib);
  Pib = __ffma2_rn(__fmul2_rn(__fmul2_rn(bc2(-P.cpd), Tr), iPi), b.phir, Pib);
  Pib = __ffma2_rn(__fmul2_rn(s7, iPi), b.Tr, Pib);
  const float2 ip = make_float2(grcp(p.x), grcp(p.y));
  const float2 pb = __ffma2_rn(__fmul2_rn(bc2(P.kappa), Pi), __fmul2_rn(Pib, ip), b.p);
  float2 Tb = __ffma2_rn(iPi, b.thv, b.T);
  Tb = __ffma2_rn(bc2(P.Rd), b.h, Tb);
  Tb = __ffma2_rn(__fmul2_rn(rho, bc2(P.Rd)), pb, Tb);
  const float2 ti = __fmul2_rn(Tb, bc2(P.icvd));
  const float2 tic = make_float2(cx ? 0.0f : ti.x, cy ? 0.0f : ti.y);
  const float2 eb = __fadd2_rn(b.h, tic);
  K_b = __fmul2_rn(tic, m1);
  rhoe_b = __fmul2_rn(eb, irho);
  rho_b = __ffma2_rn(__fmul2_rn(rhoe_b, m1), e, __fmul2_rn(__fmul2_rn(bc2(P.Rd), T), pb));
}

// The hyperdiffused dry static energy less its reference value,
// s_d - s_d,r = cp_d (T - T_0) + Phi - (cp_d (T_r - T_0) + Phi_r) = cp_d (T - T_r) + phid
// (TD.dry_static_energy and sd_r, hyperdiffusion.jl:142-147, refstate_thermodynamics.jl).
template <class FT>
__device__ __forceinline__ FT sd_dev(const DevParams<FT> &P, const Thermo<FT> &th) {
  return P.cpd * (th.T - th.Tr) + th.phid;
}

// Per-column horizontal geometry (surface metric of one node).
template <class FT>
struct ColGeo {
  FT Jh, iJh, gu0, gu1, gu2;
  __device__ void load(const DevParams<FT> &P, int e, int n) {
    const FT *hg = P.hgeo + (size_t)e * HG_N * NN;
    Jh = hg[HG_JH * NN + n];
    iJh = hg[HG_IJH * NN + n];
    gu0 = hg[HG_GU0 * NN + n];
    gu1 = hg[HG_GU1 * NN + n];
    gu2 = hg[HG_GU2 * NN + n];
  }
};

// ---------------------------------------------------------------- TMA (bulk copy) + mbarrier
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Start a global line towards L2 (no register written, no wait).
__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
// Compensated sum of FT values.  In FP32 a (hi, lo) pair: every addition is
// Knuth's TwoSum (error-free), its rounding error carried in lo, so the sum
// keeps about twice FP32's precision without FP64 instructions (GB300 issues
// FP64 at 1/64 of its FP32 rate; FP64 accumulators made that pipe the
// bottleneck of the column kernels).  value() rounds hi + lo to FP64.  In FP64
// a plain double.  Products fed to add() are rounded first (mul_rn), so that
// no multiply-add contraction splits them between the TwoSum's operations.
template <class FT>
struct CSum;
template <>
struct CSum<float> {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float s = hi + x, v = s - hi;
    lo += (hi - (s - v)) + (x - v);
    hi = s;
  }
  __device__ __forceinline__ void add(const CSum &o) {
    const float s = hi + o.hi, v = s - hi;
    const float e = ((hi - (s - v)) + (o.hi - v)) + (lo + o.lo);
    hi = s + e;
    lo = e - (hi - s);
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
  __device__ __forceinline__ CSum xor_shfl(int o, int width) const {
    CSum r;
    r.hi = __shfl_xor_sync(0xffffffffu, hi, o, width);
    r.lo = __shfl_xor_sync(0xffffffffu, lo, o, width);
    return r;
  }
};
template <>
struct CSum<double> {
  double hi = 0.0, lo = 0.0;  // lo stays zero
  __device__ __forceinline__ void add(double x) { hi += x; }
  __device__ __forceinline__ void add(const CSum &o) { hi += o.hi; }
  __device__ __forceinline__ double value() const { return hi; }
  __device__ __forceinline__ CSum xor_shfl(int o, int width) const {
    CSum r;
    r.hi = __shfl_xor_sync(0xffffffffu, hi, o, width);
    return r;
  }
};
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

// A column's residual sum of squares as kept between kernels, in one 8-byte
// slot: the compensated pair itself in FP32 runs (so that the column kernels
// issue no FP64 instruction: on this pipe a warp instruction costs its full
// issue time even with one lane active), a double in FP64 runs.  get() is the
// FP64 value; put() stores v (first) or adds it to the stored sum.
template <class FT>
struct RSlot;
template <>
struct RSlot<float> {
  static __device__ __forceinline__ void put(double *p, const CSum<float> &v, bool first) {
    float2 *q = reinterpret_cast<float2 *>(p);
    CSum<float> t = v;
    if (!first) {
      const float2 o = *q;
      CSum<float> a;
      a.hi = o.x;
      a.lo = o.y;
      t.add(a);
    }
    *q = make_float2(t.hi, t.lo);
  }
  static __device__ __forceinline__ CSum<float> load(const double *p) {
    const float2 q = *reinterpret_cast<const float2 *>(p);
    CSum<float> r;
    r.hi = q.x;
    r.lo = q.y;
    return r;
  }
};
template <>
struct RSlot<double> {
  static __device__ __forceinline__ void put(double *p, const CSum<double> &v, bool first) {
    *p = first ? v.hi : *p + v.hi;
  }
  static __device__ __forceinline__ CSum<double> load(const double *p) {
    CSum<double> r;
    r.hi = *p;
    return r;
  }
};

// Sum over a block of 256 threads of three compensated sums each, in a fixed
// order (deterministic); the result is valid in thread 0.
template <class FT>
__device__ __forceinline__ void block_sum3(CSum<FT> (&v)[3]) {
  __shared__ FT sh_hi[3][256], sh_lo[3][256];
  for (int q = 0; q < 3; ++q) {
    sh_hi[q][threadIdx.x] = v[q].hi;
    sh_lo[q][threadIdx.x] = v[q].lo;
  }
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
      for (int q = 0; q < 3; ++q) {
        CSum<FT> a, b;
        a.hi = sh_hi[q][threadIdx.x];
        a.lo = sh_lo[q][threadIdx.x];
        b.hi = sh_hi[q][threadIdx.x + o];
        b.lo = sh_lo[q][threadIdx.x + o];
        a.add(b);
        sh_hi[q][threadIdx.x] = a.hi;
        sh_lo[q][threadIdx.x] = a.lo;
      }
    __syncthreads();
  }
  for (int q = 0; q < 3; ++q) {
    v[q].hi = sh_hi[q][0];
    v[q].lo = sh_lo[q][0];
  }
}

// L2 prefetch of a contiguous range by the copy engine (16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_prefetch_l2(const void *p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// 1-D TMA bulk copy global -> shared, completing on an mbarrier.  dst, src and
// bytes must be multiples of 16.
__device__ __forceinline__ void tma_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// 1-D TMA bulk copy shared -> global (bulk-group completion).
__device__ __forceinline__ void tma_store(void *dst, const void *src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_store_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void tma_store_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// all but the most recent committed store group have finished reading shared memory
__device__ __forceinline__ void tma_store_wait_read_1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
__device__ __forceinline__ void tma_store_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// Bounded wait: returns false (and flags ST_TIMEOUT) if the phase did not
// complete within limit_ns (WAIT_LIMIT_NS by default); the caller then waits
// once more, with the same limit, for its own copies and skips its work.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, int *status,
                                                  unsigned long long limit_ns = WAIT_LIMIT_NS) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (global_ns() - t0 < limit_ns)
    if (mbar_try_wait(bar, parity)) return true;
  if (status) atomicOr(status, ST_TIMEOUT);
  const unsigned long long t1 = global_ns();
  while (global_ns() - t1 < limit_ns)
    if (mbar_try_wait(bar, parity)) break;
  return false;
}

__host__ __device__ constexpr size_t align16(size_t b) { return (b + 15) & ~size_t(15); }

}  // namespace gb
