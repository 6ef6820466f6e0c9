// CPU ORACLE for the ClimaAtmos dry dynamical-core IMEX step.
//
// TEST INFRASTRUCTURE ONLY: the parity tests, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py use this file for the results to compare with and
// as the timed CPU port.  Nothing in the product library links or calls it.
//
// Parity status: the reference's arithmetic lives in ClimaCore 0.15.1,
// ClimaTimeSteppers 0.10.6 and Thermodynamics 1.3.0 (pinned in
// .buildkite/Manifest-v1.11.toml, not vendored) and no Julia toolchain exists
// here, so this restatement is pinned by the reference's own invariants
// (sponge known answers, impenetrable-boundary filter, post-Newton identity,
// mass/energy conservation, Jacobian vs finite differences) and NOT by
// ClimaCore outputs: parity with ClimaCore itself is unpinned.
//
// The code follows the reference statement by statement, as full-field
// operations, in the order the reference issues them:
//   remaining_tendency!            src/prognostic_equations/remaining_tendency.jl:48-58
//   horizontal_dynamics_tendency!  src/prognostic_equations/advection.jl:36-91
//   prep/apply hyperdiffusion      src/prognostic_equations/hyperdiffusion.jl:116-147, 247-307
//   explicit_vertical_advection!   src/prognostic_equations/advection.jl:205-290 (deep branch)
//   Rayleigh sponge                src/parameterized_tendencies/sponge/rayleigh_sponge.jl:7-57
//   Held-Suarez forcing            src/parameterized_tendencies/radiation/held_suarez.jl:98-296
//   implicit tendency              src/prognostic_equations/implicit/implicit_tendency.jl:185-298
//   post-Newton correction         src/prognostic_equations/implicit/implicit_tendency.jl:322-339
//   Jacobian blocks                src/prognostic_equations/implicit/manual_sparse_jacobian.jl:713-870
//   BlockArrowheadSolve (dry)      src/prognostic_equations/implicit/manual_sparse_jacobian.jl:580-583
//   precomputed quantities         src/cache/precomputed_quantities.jl:473-571, 698-831
//   kinetic energy                 src/utils/utilities.jl:194-206
//   reference state                src/utils/refstate_thermodynamics.jl:58-166
//   operators and their BCs        src/utils/abbreviations.jl:72-290
// Operators are restated from docs/src/discretization.md:60-420 and the
// spectral-element weak/strong forms (Taylor & Fournier 2010); ARS343 is the
// Ascher-Ruuth-Spiteri (1997) (3,4,3) tableau; the van Leer face
// reconstruction is Lin et al. (1994) with their monotonicity constraint.
//
// Layout (same as the product's C-ABI): centre block [elem][comp][node][level]
// with comp = (rho, u_1, u_2, rho e_tot); face block [elem][node][face].
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {
struct OracleParams {
  double grav, omega, R_d, cp_d, cv_d, T_0, p_ref, T_min_ref, T_surf_ref, T_min_sgs, radius;
  double nu_v, nu_s, div_damp;
  double sponge_zd, alpha_uh, alpha_w;
  double z_max;
  double dt_model;  // the model time step used by the van Leer Courant factor
  int upwinding;    // 0: central only (no post-Newton correction), 1: van Leer
  int dss_stage1;   // 1: DSS the first stage as well (ClimaTimeSteppers does)
  int held_suarez;  // 1: Held-Suarez forcing in the remaining tendency
  double hs_day, hs_sigma_b, hs_dT_y, hs_T_equator, hs_dtheta_z, hs_T_min, hs_p_ref_theta, hs_MSLP;
  // Moist 0M (EquilibriumMicrophysics0M): moist = 1 adds the centre component rho q_tot (comp 4)
  // to the column operators; the moist thermodynamic constants (Thermodynamics.jl names) and the
  // Newton iterations of the saturation adjustment
  int moist;
  double R_v, cp_v, cp_l, cp_i, LH_v0, LH_s0, T_triple, press_triple, T_freeze, T_icenuc, pow_icenuc;
  int sa_iters;
};
struct OracleGeom {
  int Nh, Nv, ngroups;
  const double *W, *D, *Jh, *gup, *gdn, *sinlat, *fh0, *ecov, *econ, *zf;
  const int *dss_off, *dss_copy;
  const double *dss_w;
  // Terrain-following geometry (all null over a flat surface), per point: heights
  // zc [Nh][16][Nv] and zf [Nh][16][Nf]; Jacobians Jc, Jf; contravariant metrics
  // guc, guf [..][6] = (g^11, g^12, g^22, g^13, g^23, g^33); covariant metric of the
  // centres gdc [..][6] = (g_11, g_12, g_22, g_13, g_23, g_33); the Coriolis f^3 of the
  // centres and (f^1, f^2) of the faces; the covariant and contravariant basis of the
  // centres Ecc, Ecn [..][3][3] (row i = E_i or E^i, Cartesian) for the vector DSS.
  const double *t_zc, *t_zf, *t_Jc, *t_Jf, *t_guc, *t_guf, *t_gdc, *t_f3c, *t_f12f, *t_Ecc, *t_Ecn;
};
}

namespace {

constexpr int NQ = 4, NN = 16;

template <class FT>
struct Oracle {
  int Nh, Nv, Nf;
  // parameters
  FT grav, omega, Rd, cpd, cvd, T0, pref, Tmin_ref, Tsfc_ref, Tmin_sgs, R;
  FT nu_v, nu_s, div_damp, zd, a_uh, a_w, zmax, dt_model, kappa;
  int upwinding, dss_stage1;
  int hs = 0;  // Held-Suarez forcing
  // moist 0M: centre components per element (4 dry, 5 with rho q_tot) and the moist constants:
  // cv of vapour, liquid and ice, latent heats at T_0, the triple point, the freezing and
  // homogeneous-nucleation temperatures of the liquid fraction, e_int_v0 = L_v0 - R_v T_0,
  // e_int_i0 = L_s0 - L_v0
  int moist = 0, nfc = 4, sa_iters = 0;
  FT Rv, cvv, cvl, cvi, cpv, cpl, cpi, Lv0, Ls0, Ttr, ptr, Tfrz, Tice, pice, ev0, ei0;
  FT hs_day, hs_sb, hs_dTy, hs_Teq, hs_dthz, hs_Tmin, hs_p0, hs_MSLP;
  // geometry
  FT W[NN], D[NQ][NQ];
  std::vector<FT> Jh, gup, gdn, sinlat, fh0, ecov, econ;
  std::vector<FT> zf, zc, dzc, dzf, rc, rf;
  std::vector<int> goff, gcopy;
  std::vector<FT> gw;
  // terrain-following geometry per point (topo = 1), see OracleGeom
  int topo = 0;
  std::vector<FT> tzc, tzf, tJc, tJf, tguc, tguf, tgdc, tf3c, tf12f, tEcc, tEcn;

  size_t ncen() const { return (size_t)Nh * nfc * NN * Nv; }
  size_t nfac() const { return (size_t)Nh * NN * Nf; }
  size_t npt() const { return (size_t)Nh * NN * Nv; }
  size_t ci(int e, int c, int n, int v) const { return (((size_t)e * nfc + c) * NN + n) * Nv + v; }
  size_t fi(int e, int n, int k) const { return ((size_t)e * NN + n) * Nf + k; }
  size_t pi(int e, int n, int v) const { return ((size_t)e * NN + n) * Nv + v; }
  size_t hn(int e, int n) const { return (size_t)e * NN + n; }

  // ---- pointwise geometry (per level over a flat surface, per point over terrain) ----
  FT Jc(int e, int n, int v) const { return topo ? tJc[pi(e, n, v)] : Jh[hn(e, n)] * rc[v] * rc[v] * dzc[v]; }
  FT Jfc(int e, int n, int k) const { return topo ? tJf[fi(e, n, k)] : Jh[hn(e, n)] * rf[k] * rf[k] * dzf[k]; }
  FT zcp(int e, int n, int v) const { return topo ? tzc[pi(e, n, v)] : zc[v]; }
  FT zfp(int e, int n, int k) const { return topo ? tzf[fi(e, n, k)] : zf[k]; }
  // g^33 of a face and the (g^31, g^32) of a centre
  FT g33f(int e, int n, int k) const { return topo ? tguf[fi(e, n, k) * 6 + 5] : FT(1) / (dzf[k] * dzf[k]); }
  FT g31c(int e, int n, int v) const { return topo ? tguc[pi(e, n, v) * 6 + 3] : FT(0); }
  FT g32c(int e, int n, int v) const { return topo ? tguc[pi(e, n, v) * 6 + 4] : FT(0); }
  FT gu(int e, int n, int c, FT r) const { return gup[hn(e, n) * 3 + c] / (r * r); }
  FT gd(int e, int n, int c, FT r) const { return gdn[hn(e, n) * 3 + c] * (r * r); }

  // ---- thermodynamics (Thermodynamics.jl dry air; e_int = cv_d (T - T_0) - R_d T_0) ----
  FT exner(FT p) const { return std::pow(p / pref, kappa); }
  FT T_ref(FT Pi) const { return Tmin_ref + (Tsfc_ref - Tmin_ref) * std::pow(Pi, FT(7)); }
  FT phi_r(FT Pi) const {
    return -cpd * (Tmin_ref * std::log(Pi) + (Tsfc_ref - Tmin_ref) / FT(7) * (std::pow(Pi, FT(7)) - FT(1)));
  }
  FT sd_r(FT Pi) const { return cpd * (T_ref(Pi) - T0) + phi_r(Pi); }
  FT beta_sponge(FT z, FT alpha) const {
    if (!(z > zd) || alpha == FT(0)) return FT(0);
    FT s = std::sin(FT(M_PI) * (z - zd) / (zmax - zd) / FT(2));
    return alpha * s * s;
  }

  // ---- precomputed quantities (set_implicit_precomputed_quantities!) ----
  struct Pre {
    std::vector<FT> ub3, K, T, p, h, Pi, thv, thvr, phir, uc1, uc2, u3c;  // u3c = contravariant u^3 at faces
    // ct3 = CT3(u_h) = g^31 u_1 + g^32 u_2 at centres (0 over a flat surface); w3c = g^33 u_3 at faces
    std::vector<FT> ct3, w3c;
    // moist: q = specific(rho q_tot, rho); kapm = R_m / cv_m; dpdq = dp/d(rho q_tot) at constant
    // rho and rho e_tot
    std::vector<FT> q, kapm, dpdq;
  } pre;

  // ---- moist thermodynamics (EquilibriumMicrophysics0M) ----
  // Restated from the published formulation of Thermodynamics.jl 1.3.0 (not vendored here; parity
  // with it is unpinned), as the reference's Jacobian assumes it (manual_sparse_jacobian.jl:646-684:
  // its dp/drho and dp/d(rho q_tot) follow from these definitions):
  //   cv_m  = cv_d + (cv_v - cv_d) q_t + (cv_l - cv_v) q_l + (cv_i - cv_v) q_i
  //   R_m   = R_d (1 - q_t) + R_v (q_t - q_l - q_i)
  //   e_int = cv_m (T - T_0) + q_v e_int_v0 - q_i e_int_i0 - (1 - q_t) R_d T_0
  //   p_v*(T) = p_tr (T / T_tr)^(dcp / R_v) exp((L_0 - dcp T_0) / R_v (1 / T_tr - 1 / T)),
  //     L_0 = lam L_v0 + (1 - lam) L_s0, dcp = lam (cp_v - cp_l) + (1 - lam) (cp_v - cp_i)
  //   q_v* = p_v* / (rho R_v T)
  //   lam(T) = 1 above T_freeze, 0 below T_icenuc, ((T - T_icenuc) / (T_freeze - T_icenuc))^pow between
  // The saturation adjustment (precomputed_quantities.jl:734-747, TD.saturation_adjustment with
  // TD.ρe()): the all-vapour temperature T_u if the point is unsaturated there, else sa_iters
  // safeguarded Newton iterations on f(T) = e_int(T) - e_int with the saturated partition
  // q_c = q_t - q_v*(T) split by lam(T), continued smoothly (q_c < 0) where q_v* > q_t: the
  // clamped function's kink there makes plain Newton cycle between T_u and an unsaturated
  // iterate.  f increases with T, f(T_u) < 0 and f(T_b) > 0 at
  // T_b = max(T_u + q_t (e_int_v0 + e_int_i0) / cv_d, T_0) + 1; a Newton step outside the
  // current bracket is replaced by bisection.  The iterations stop early once a step moves T by
  // no more than 1e-9 K (FP64) or 1e-3 K (FP32): Newton's error after such a step is of the order
  // of its square.  The partition returned is that of the final T.
  FT liq_frac(FT T, FT &dl) const {
    if (T > Tfrz) { dl = FT(0); return FT(1); }
    if (!(T > Tice)) { dl = FT(0); return FT(0); }
    const FT x = (T - Tice) / (Tfrz - Tice);
    dl = pice * std::pow(x, pice - FT(1)) / (Tfrz - Tice);
    return std::pow(x, pice);
  }
  // q_v*(T, rho) and d ln q_v* / dT
  FT qsat(FT T, FT rho, FT &dlnq) const {
    FT dl;
    const FT lam = liq_frac(T, dl);
    const FT dcl = cpv - cpl, dci = cpv - cpi;
    const FT dcp = lam * dcl + (FT(1) - lam) * dci, L0 = lam * Lv0 + (FT(1) - lam) * Ls0;
    const FT a = dcp / Rv, b = (L0 - dcp * T0) / Rv, s = FT(1) / Ttr - FT(1) / T;
    const FT lt = std::log(T / Ttr);
    const FT ps = ptr * std::exp(a * lt + b * s);
    // d ln p_v* / dT, with the dependence of L_0 and dcp on lam(T)
    const FT dlp = a / T + b / (T * T) + dl * ((dcl - dci) / Rv * lt + ((Lv0 - Ls0) - (dcl - dci) * T0) / Rv * s);
    dlnq = dlp - FT(1) / T;
    return ps / (rho * Rv * T);
  }
  struct Sat {
    FT T, ql, qi;
  };
  Sat sat_adjust(FT rho, FT eint, FT q) const {
    const FT cvm0 = cvd + (cvv - cvd) * q;
    FT T = T0 + (eint - q * ev0 + (FT(1) - q) * Rd * T0) / cvm0;
    T = std::max(Tmin_sgs, T);
    FT dlnq;
    if (q <= qsat(T, rho, dlnq)) return {T, FT(0), FT(0)};
    FT lo = T, hi = std::max(T + q * (ev0 + ei0) / cvd, T0) + FT(1);
    for (int it = 0; it < sa_iters; ++it) {
      FT dl;
      const FT lam = liq_frac(T, dl);
      const FT qs = qsat(T, rho, dlnq);
      const FT qc = q - qs;
      const FT ql = lam * qc, qi = (FT(1) - lam) * qc;
      const FT cvm = cvd + (cvv - cvd) * q + (cvl - cvv) * ql + (cvi - cvv) * qi;
      const FT f = cvm * (T - T0) + qs * ev0 - qi * ei0 - (FT(1) - q) * Rd * T0 - eint;
      const FT dqc = -qs * dlnq;
      const FT dql = dl * qc + lam * dqc, dqi = -dl * qc + (FT(1) - lam) * dqc;
      const FT df = cvm + (T - T0) * ((cvl - cvv) * dql + (cvi - cvv) * dqi) - dqc * ev0 - dqi * ei0;
      if (f < FT(0)) lo = T;
      else hi = T;
      FT Tn = T - f / df;
      if (!(Tn >= lo && Tn <= hi)) Tn = (lo + hi) / FT(2);
      const FT dT = Tn - T;
      T = Tn;
      if (std::fabs(dT) <= (sizeof(FT) == 8 ? FT(1e-9) : FT(1e-3))) break;
    }
    FT dl;
    const FT lam = liq_frac(T, dl);
    const FT qc = std::max(FT(0), q - qsat(T, rho, dlnq));
    return {T, lam * qc, (FT(1) - lam) * qc};
  }
#ifdef ORACLE_PHID
  // per level: the reference pressure p0 = p_ref Pi0^(1/kappa) and Pi0^7, Phi_r(Pi0) = g z_c (Newton, FP64)
  std::vector<FT> p0v, pi07;
  void ref_levels() {
    p0v.resize(Nv);
    pi07.resize(Nv);
    const double cp = cpd, tm = Tmin_ref, dT = (double)Tsfc_ref - (double)Tmin_ref;
    for (int v = 0; v < Nv; ++v) {
      const double gz = (double)grav * (double)zc[v];
      // Newton's method in x = ln P (decreasing, concave: monotone from x = 0; in P itself the
      // first step overshoots below zero for levels near 30 km)
      double x = 0.0;
      for (int it = 0; it < 100; ++it) {
        const double e7 = std::exp(7.0 * x);
        x -= (-cp * (tm * x + dT / 7.0 * (e7 - 1.0)) - gz) / (-cp * (tm + dT * e7));
      }
      const double P = std::exp(x);
      p0v[v] = (FT)((double)pref * std::pow(P, 1.0 / (double)kappa));
      pi07[v] = (FT)std::pow(P, 7.0);
    }
  }
#endif

  void alloc_pre() {
    size_t P = npt();
    for (auto *v : {&pre.ub3, &pre.K, &pre.T, &pre.p, &pre.h, &pre.Pi, &pre.thv, &pre.thvr, &pre.phir, &pre.uc1, &pre.uc2,
                    &pre.ct3})
      v->assign(P, FT(0));
    pre.u3c.assign(nfac(), FT(0));
    pre.w3c.assign(nfac(), FT(0));
    if (moist)
      for (auto *v : {&pre.q, &pre.kapm, &pre.dpdq}) v->assign(P, FT(0));
#ifdef ORACLE_PHID
    ref_levels();
#endif
  }

  // impenetrable-boundary filter: u_3 = -u_h^3 / g^33 at the bottom and top faces
  // (set_velocity_at_surface! / set_velocity_at_top!, precomputed_quantities.jl:486-553),
  // u_h^3 = ᶠwinterp(rho J, CT3(u_h)), which at the boundary faces is the adjacent centre's
  // CT3(u_h) (Extrapolate); over a flat surface u_h^3 = 0.
  void bc_filter(const FT *Yc, FT *Yf) const {
#pragma omp parallel for
    for (int e = 0; e < Nh; ++e)
      for (int n = 0; n < NN; ++n) {
        if (!topo) {
          Yf[fi(e, n, 0)] = FT(0);
          Yf[fi(e, n, Nv)] = FT(0);
          continue;
        }
        const FT b = g31c(e, n, 0) * Yc[ci(e, 1, n, 0)] + g32c(e, n, 0) * Yc[ci(e, 2, n, 0)];
        const FT t = g31c(e, n, Nv - 1) * Yc[ci(e, 1, n, Nv - 1)] + g32c(e, n, Nv - 1) * Yc[ci(e, 2, n, Nv - 1)];
        Yf[fi(e, n, 0)] = -b / g33f(e, n, 0);
        Yf[fi(e, n, Nv)] = -t / g33f(e, n, Nv);
      }
  }

  void set_precomputed(FT *Yc, FT *Yf) {
    bc_filter(Yc, Yf);
#pragma omp parallel for
    for (int e = 0; e < Nh; ++e)
      for (int n = 0; n < NN; ++n) {
        for (int k = 0; k < Nf; ++k)
          pre.u3c[fi(e, n, k)] = topo ? Yf[fi(e, n, k)] * g33f(e, n, k) : Yf[fi(e, n, k)] / (dzf[k] * dzf[k]);
        if (topo) {
          // CT3(u_h) at the centres; u^3 = ᶠwinterp(rho J, CT3(u_h)) + g^33 u_3 at the faces
          // (compute_ᶠuₕ³ and set_velocity_quantities!, precomputed_quantities.jl:473-476, 560-571)
          for (int v = 0; v < Nv; ++v)
            pre.ct3[pi(e, n, v)] = g31c(e, n, v) * Yc[ci(e, 1, n, v)] + g32c(e, n, v) * Yc[ci(e, 2, n, v)];
          for (int k = 0; k < Nf; ++k) {
            FT uh3;
            if (k == 0) uh3 = pre.ct3[pi(e, n, 0)];
            else if (k == Nv) uh3 = pre.ct3[pi(e, n, Nv - 1)];
            else {
              const FT wa = Yc[ci(e, 0, n, k - 1)] * Jc(e, n, k - 1), wb = Yc[ci(e, 0, n, k)] * Jc(e, n, k);
              uh3 = (wa * pre.ct3[pi(e, n, k - 1)] + wb * pre.ct3[pi(e, n, k)]) / (wa + wb);
            }
            pre.w3c[fi(e, n, k)] = pre.u3c[fi(e, n, k)];
            pre.u3c[fi(e, n, k)] = uh3 + pre.w3c[fi(e, n, k)];
          }
        } else {
          for (int k = 0; k < Nf; ++k) pre.w3c[fi(e, n, k)] = pre.u3c[fi(e, n, k)];
        }
        for (int v = 0; v < Nv; ++v) {
          size_t q = pi(e, n, v);
          FT rho = Yc[ci(e, 0, n, v)], u1 = Yc[ci(e, 1, n, v)], u2 = Yc[ci(e, 2, n, v)], rhoe = Yc[ci(e, 3, n, v)];
          FT a = Yf[fi(e, n, v)], b = Yf[fi(e, n, v + 1)];
          FT c1, c2, K;
          pre.ub3[q] = (a + b) / FT(2);
          if (topo) {
            // ᶜu = C123(u_h) + ᶜinterp(C123(u_3)); CT12(ᶜu) = g^ab u_b + g^a3 I^c(u_3);
            // K = 1/2 (C123(u_h) . CT123(u_h) + I^c(u_3 g^33 u_3) + 2 CT3(u_h) I^c(u_3))
            // (compute_kinetic, utilities.jl:194-206)
            const FT *G = &tguc[q * 6];
            const FT h1 = G[0] * u1 + G[1] * u2, h2 = G[1] * u1 + G[2] * u2;
            c1 = h1 + G[3] * pre.ub3[q];
            c2 = h2 + G[4] * pre.ub3[q];
            const FT kv = (a * pre.w3c[fi(e, n, v)] + b * pre.w3c[fi(e, n, v + 1)]) / FT(2);
            K = (u1 * h1 + u2 * h2 + kv + FT(2) * pre.ct3[q] * pre.ub3[q]) / FT(2);
          } else {
            FT r = rc[v];
            c1 = gu(e, n, 0, r) * u1 + gu(e, n, 1, r) * u2;
            c2 = gu(e, n, 1, r) * u1 + gu(e, n, 2, r) * u2;
            // K = 1/2 (u_h . u_h + I^c(u_3 u^3) + 2 u_h^3 I^c(u_3)); u_h^3 = 0 here
            FT kv = (a * pre.u3c[fi(e, n, v)] + b * pre.u3c[fi(e, n, v + 1)]) / FT(2);
            K = (u1 * c1 + u2 * c2 + kv) / FT(2);
          }
          pre.uc1[q] = c1;
          pre.uc2[q] = c2;
          pre.K[q] = K;
          FT Phi = grav * zcp(e, n, v);
          FT eint = rhoe / rho - K - Phi;
          FT T, Rm = Rd;
          if (moist) {
            // precomputed_quantities.jl:734-747: q_tot_nonneg = max(0, specific(rho q_tot, rho)),
            // the saturation adjustment, p = rho R_m T (EquilibriumMicrophysics0M)
            const FT qt = Yc[ci(e, 4, n, v)] / rho, qn = std::max(FT(0), qt);
            const Sat sa = sat_adjust(rho, eint, qn);
            T = sa.T;
            Rm = Rd * (FT(1) - qn) + Rv * (qn - sa.ql - sa.qi);
            const FT cvm = cvd + (cvv - cvd) * qn + (cvl - cvv) * sa.ql + (cvi - cvv) * sa.qi;
            const FT km = Rm / cvm;
            pre.q[q] = qt;
            pre.kapm[q] = km;
            // ᶜ∂p∂ρq_tot (manual_sparse_jacobian.jl:670-685)
            pre.dpdq[q] = km * (-ev0 - Rd * T0 - (cvv - cvd) * (T - T0)) + (Rv - Rd) * T;
          } else {
            T = std::max(Tmin_sgs, T0 + (eint + Rd * T0) / cvd);
          }
          FT p = rho * Rm * T;
          FT Pi = exner(p);
          pre.T[q] = T;
          pre.p[q] = p;
          pre.h[q] = rhoe / rho + Rm * T;
          pre.Pi[q] = Pi;
          // theta_v = T R_m / (Pi R_d) (refstate_thermodynamics.jl:58-63)
          pre.thv[q] = moist ? T * Rm / (Pi * Rd) : T / Pi;
          pre.thvr[q] = T_ref(Pi) / Pi;
#ifdef ORACLE_PHID
          // precision-study build: phir holds the deviation g z - Phi_r(Pi), formed from the
          // level's reference Exner Pi0 (Phi_r(Pi0) = g z) so that no O(1e5) terms cancel:
          // g z - Phi_r(Pi) = cp (T_min ln x + (T_sfc - T_min) / 7 Pi0^7 (x^7 - 1)), x = Pi / Pi0
          FT lx = kappa * std::log1p((p - p0v[v]) / p0v[v]);
          pre.phir[q] = cpd * (Tmin_ref * lx + (Tsfc_ref - Tmin_ref) / FT(7) * pi07[v] * std::expm1(FT(7) * lx));
#else
          pre.phir[q] = phi_r(Pi);
#endif
        }
      }
  }

  // ---- spectral-element operators on one (element, level) slab ----
  // d1 f[i,j] = sum_k D[i][k] f[k,j]; d2 f[i,j] = sum_k D[j][k] f[i,k]
  void d1(const FT *f, FT *o) const {
    for (int j = 0; j < NQ; ++j)
      for (int i = 0; i < NQ; ++i) {
        FT s = 0;
        for (int k = 0; k < NQ; ++k) s += D[i][k] * f[k + NQ * j];
        o[i + NQ * j] = s;
      }
  }
  void d2(const FT *f, FT *o) const {
    for (int j = 0; j < NQ; ++j)
      for (int i = 0; i < NQ; ++i) {
        FT s = 0;
        for (int k = 0; k < NQ; ++k) s += D[j][k] * f[i + NQ * k];
        o[i + NQ * j] = s;
      }
  }
  // transposes: t1 f[i,j] = sum_k D[k][i] f[k,j]; t2 f[i,j] = sum_k D[k][j] f[i,k]
  void t1(const FT *f, FT *o) const {
    for (int j = 0; j < NQ; ++j)
      for (int i = 0; i < NQ; ++i) {
        FT s = 0;
        for (int k = 0; k < NQ; ++k) s += D[k][i] * f[k + NQ * j];
        o[i + NQ * j] = s;
      }
  }
  void t2(const FT *f, FT *o) const {
    for (int j = 0; j < NQ; ++j)
      for (int i = 0; i < NQ; ++i) {
        FT s = 0;
        for (int k = 0; k < NQ; ++k) s += D[k][j] * f[i + NQ * k];
        o[i + NQ * j] = s;
      }
  }
  // Geometry of one slab.  Over a flat surface the metric is block diagonal (g^33 and g_33
  // per level); over terrain (t = true) it is the full per-node 3x3 metric: gu3, gu4, gu5 =
  // g^13, g^23, g^33 and gd3, gd4, gd5 = g_13, g_23, g_33 (centres only: the faces need J).
  struct Slab {
    FT J[NN], WJ[NN], gu0[NN], gu1[NN], gu2[NN], gd0[NN], gd1[NN], gd2[NN], g33, G33;
    bool t = false;
    FT gu3[NN], gu4[NN], gu5[NN], gd3[NN], gd4[NN], gd5[NN];
  };
  void slab(int e, FT r, FT dz, Slab &s) const {
    for (int n = 0; n < NN; ++n) {
      s.J[n] = Jh[hn(e, n)] * r * r * dz;
      s.WJ[n] = W[n] * s.J[n];
      s.gu0[n] = gu(e, n, 0, r); s.gu1[n] = gu(e, n, 1, r); s.gu2[n] = gu(e, n, 2, r);
      s.gd0[n] = gd(e, n, 0, r); s.gd1[n] = gd(e, n, 1, r); s.gd2[n] = gd(e, n, 2, r);
    }
    s.g33 = FT(1) / (dz * dz);
    s.G33 = dz * dz;
    s.t = false;
  }
  void slab_c(int e, int v, Slab &s) const {
    if (!topo) return slab(e, rc[v], dzc[v], s);
    s.t = true;
    for (int n = 0; n < NN; ++n) {
      const size_t q = pi(e, n, v);
      const FT *G = &tguc[q * 6], *H = &tgdc[q * 6];
      s.J[n] = tJc[q];
      s.WJ[n] = W[n] * s.J[n];
      s.gu0[n] = G[0]; s.gu1[n] = G[1]; s.gu2[n] = G[2]; s.gu3[n] = G[3]; s.gu4[n] = G[4]; s.gu5[n] = G[5];
      s.gd0[n] = H[0]; s.gd1[n] = H[1]; s.gd2[n] = H[2]; s.gd3[n] = H[3]; s.gd4[n] = H[4]; s.gd5[n] = H[5];
    }
  }
  void slab_f(int e, int k, Slab &s) const {
    if (!topo) return slab(e, rf[k], dzf[k], s);
    s.t = true;
    for (int n = 0; n < NN; ++n) {
      const size_t q = fi(e, n, k);
      const FT *G = &tguf[q * 6];
      s.J[n] = tJf[q];
      s.WJ[n] = W[n] * s.J[n];
      s.gu0[n] = G[0]; s.gu1[n] = G[1]; s.gu2[n] = G[2]; s.gu3[n] = G[3]; s.gu4[n] = G[4]; s.gu5[n] = G[5];
      s.gd0[n] = s.gd1[n] = s.gd2[n] = s.gd3[n] = s.gd4[n] = s.gd5[n] = FT(0);
    }
  }
  // strong divergence of contravariant (F1, F2): (1/J) d_i (J F^i)
  void div_h(const Slab &s, const FT *F1, const FT *F2, FT *o) const {
    FT a[NN], b[NN], da[NN], db[NN];
    for (int n = 0; n < NN; ++n) { a[n] = s.J[n] * F1[n]; b[n] = s.J[n] * F2[n]; }
    d1(a, da); d2(b, db);
    for (int n = 0; n < NN; ++n) o[n] = (da[n] + db[n]) / s.J[n];
  }
  // weak divergence: -(1/WJ) sum D^T (WJ F)
  void wdiv_h(const Slab &s, const FT *F1, const FT *F2, FT *o) const {
    FT a[NN], b[NN], da[NN], db[NN];
    for (int n = 0; n < NN; ++n) { a[n] = s.WJ[n] * F1[n]; b[n] = s.WJ[n] * F2[n]; }
    t1(a, da); t2(b, db);
    for (int n = 0; n < NN; ++n) o[n] = -(da[n] + db[n]) / s.WJ[n];
  }
  // strong gradient (covariant components)
  void grad_h(const FT *f, FT *o1, FT *o2) const { d1(f, o1); d2(f, o2); }
  // weak gradient (covariant components): -(1/W) sum D^T (W f)
  void wgrad_h(const FT *f, FT *o1, FT *o2) const {
    FT a[NN], da[NN], db[NN];
    for (int n = 0; n < NN; ++n) a[n] = W[n] * f[n];
    t1(a, da); t2(a, db);
    for (int n = 0; n < NN; ++n) { o1[n] = -da[n] / W[n]; o2[n] = -db[n] / W[n]; }
  }
  // strong curl of a covariant (c1, c2, c3): contravariant result
  void curl_h(const Slab &s, const FT *c1, const FT *c2, const FT *c3, FT *o1, FT *o2, FT *o3) const {
    FT a[NN], b[NN];
    d1(c2, a); d2(c1, b);
    for (int n = 0; n < NN; ++n) o3[n] = (a[n] - b[n]) / s.J[n];
    if (c3) {
      d2(c3, a); d1(c3, b);
      for (int n = 0; n < NN; ++n) { o1[n] = a[n] / s.J[n]; o2[n] = -b[n] / s.J[n]; }
    }
  }
  // weak curl of a covariant (c1, c2, c3): contravariant result
  void wcurl_h(const Slab &s, const FT *c1, const FT *c2, const FT *c3, FT *o1, FT *o2, FT *o3) const {
    FT a[NN], b[NN], ta[NN], tb[NN];
    if (c1 && c2) {
      for (int n = 0; n < NN; ++n) { a[n] = W[n] * c2[n]; b[n] = W[n] * c1[n]; }
      t1(a, ta); t2(b, tb);
      for (int n = 0; n < NN; ++n) o3[n] = (-ta[n] + tb[n]) / s.WJ[n];
    }
    if (c3) {
      for (int n = 0; n < NN; ++n) a[n] = W[n] * c3[n];
      t2(a, tb); t1(a, ta);
      for (int n = 0; n < NN; ++n) { o1[n] = -tb[n] / s.WJ[n]; o2[n] = ta[n] / s.WJ[n]; }
    }
  }

  // ---- vector Laplacian  L(u) = C123(wgrad(div u)) * fdiv - C123(wcurl(C123(curl u))) ----
  // input covariant (c1, c2, c3) on the slab; output covariant (o1, o2, o3)
  // Over terrain every metric conversion takes the full 3x3 metric: the divergence reads
  // the contravariant (u^1, u^2) of the C123 input, g^a1 c_1 + g^a2 c_2 + g^a3 c_3, and the
  // covariant (C123) forms of the curls take g_ij over all three components.
  void vec_lap(const Slab &s, const FT *c1, const FT *c2, const FT *c3, FT fdiv, FT *o1, FT *o2, FT *o3) const {
    FT F1[NN], F2[NN], dv[NN], w1[NN], w2[NN];
    for (int n = 0; n < NN; ++n) {
      F1[n] = s.gu0[n] * c1[n] + s.gu1[n] * c2[n];
      F2[n] = s.gu1[n] * c1[n] + s.gu2[n] * c2[n];
      if (s.t) {
        F1[n] += s.gu3[n] * c3[n];
        F2[n] += s.gu4[n] * c3[n];
      }
    }
    div_h(s, F1, F2, dv);
    wgrad_h(dv, w1, w2);
    FT k1[NN], k2[NN], k3[NN];
    curl_h(s, c1, c2, c3, k1, k2, k3);
    FT z1[NN], z2[NN], z3[NN];
    for (int n = 0; n < NN; ++n) {  // C123 of the contravariant curl
      if (s.t) {
        z1[n] = s.gd0[n] * k1[n] + s.gd1[n] * k2[n] + s.gd3[n] * k3[n];
        z2[n] = s.gd1[n] * k1[n] + s.gd2[n] * k2[n] + s.gd4[n] * k3[n];
        z3[n] = s.gd3[n] * k1[n] + s.gd4[n] * k2[n] + s.gd5[n] * k3[n];
      } else {
        z1[n] = s.gd0[n] * k1[n] + s.gd1[n] * k2[n];
        z2[n] = s.gd1[n] * k1[n] + s.gd2[n] * k2[n];
        z3[n] = s.G33 * k3[n];
      }
    }
    FT q1[NN], q2[NN], q3[NN];
    wcurl_h(s, z1, z2, z3, q1, q2, q3);
    for (int n = 0; n < NN; ++n) {
      if (s.t) {
        o1[n] = fdiv * w1[n] - (s.gd0[n] * q1[n] + s.gd1[n] * q2[n] + s.gd3[n] * q3[n]);
        o2[n] = fdiv * w2[n] - (s.gd1[n] * q1[n] + s.gd2[n] * q2[n] + s.gd4[n] * q3[n]);
        o3[n] = -(s.gd3[n] * q1[n] + s.gd4[n] * q2[n] + s.gd5[n] * q3[n]);
      } else {
        o1[n] = fdiv * w1[n] - (s.gd0[n] * q1[n] + s.gd1[n] * q2[n]);
        o2[n] = fdiv * w2[n] - (s.gd1[n] * q1[n] + s.gd2[n] * q2[n]);
        o3[n] = -s.G33 * q3[n];
      }
    }
  }

  // ---- DSS (Spaces.weighted_dss!): J-weighted average over collocated nodes; the
  // covariant horizontal vector (comps 1, 2 of a centre block) is averaged in
  // Cartesian components.  Centre block comps: 0 scalar, 1-2 vector, 3 scalar.
  // c123: comps 1-3 of the block are one covariant 3-vector (the Laplacian block of
  // remaining_tendency: (L_s, C123 of the vector Laplacian)).  Over terrain its third
  // basis vector E^3 leans with the level, so the vector is projected to Cartesian
  // components with each copy's full contravariant basis, averaged, and projected back on
  // each copy's covariant basis (ClimaCore's dss_transform / dss_untransform of a
  // Covariant123Vector); over a flat surface that reduces to the horizontal vector and a
  // scalar third component.
  void dss_center_c123(FT *C, int levels) const {
    int G = (int)goff.size() - 1;
#pragma omp parallel for
    for (int g = 0; g < G; ++g) {
      for (int v = 0; v < levels; ++v) {
        FT s0 = 0, X[3] = {0, 0, 0};
        for (int c = goff[g]; c < goff[g + 1]; ++c) {
          int idx = gcopy[c], e = idx / NN, n = idx % NN;
          FT w = gw[c];
          s0 += w * C[ci(e, 0, n, v)];
          const FT *En = &tEcn[pi(e, n, v) * 9];
          for (int d = 0; d < 3; ++d)
            X[d] += w * (C[ci(e, 1, n, v)] * En[d] + C[ci(e, 2, n, v)] * En[3 + d] + C[ci(e, 3, n, v)] * En[6 + d]);
        }
        for (int c = goff[g]; c < goff[g + 1]; ++c) {
          int idx = gcopy[c], e = idx / NN, n = idx % NN;
          const FT *Ec = &tEcc[pi(e, n, v) * 9];
          C[ci(e, 0, n, v)] = s0;
          for (int i = 0; i < 3; ++i) C[ci(e, 1 + i, n, v)] = Ec[3 * i] * X[0] + Ec[3 * i + 1] * X[1] + Ec[3 * i + 2] * X[2];
        }
      }
    }
  }
  void dss_center(FT *C, int levels, bool c123 = false) const {
    if (c123 && topo) return dss_center_c123(C, levels);
    int G = (int)goff.size() - 1;
#pragma omp parallel for
    for (int g = 0; g < G; ++g) {
      for (int v = 0; v < levels; ++v) {
        // the weighted sums as fused multiply-adds in ascending copy order (an exact
        // rounding recipe, so that a GPU DSS doing the same operations agrees bit for bit)
        // (moist: ρq_tot, centre component 4, is a scalar like ρ and ρe_tot)
        FT s0 = 0, s3 = 0, s4 = 0, X[3] = {0, 0, 0};
        for (int c = goff[g]; c < goff[g + 1]; ++c) {
          int idx = gcopy[c], e = idx / NN, n = idx % NN;
          FT w = gw[c];
          s0 = std::fma(w, C[ci(e, 0, n, v)], s0);
          s3 = std::fma(w, C[ci(e, 3, n, v)], s3);
          if (nfc == 5) s4 = std::fma(w, C[ci(e, 4, n, v)], s4);
          FT u1 = C[ci(e, 1, n, v)], u2 = C[ci(e, 2, n, v)];
          const FT *ec = &econ[hn(e, n) * 6];
          for (int d = 0; d < 3; ++d) X[d] = std::fma(w, std::fma(u2, ec[3 + d], u1 * ec[d]), X[d]);
        }
        for (int c = goff[g]; c < goff[g + 1]; ++c) {
          int idx = gcopy[c], e = idx / NN, n = idx % NN;
          C[ci(e, 0, n, v)] = s0;
          C[ci(e, 3, n, v)] = s3;
          if (nfc == 5) C[ci(e, 4, n, v)] = s4;
          const FT *eo = &ecov[hn(e, n) * 6];
          C[ci(e, 1, n, v)] = std::fma(eo[2], X[2], std::fma(eo[1], X[1], eo[0] * X[0]));
          C[ci(e, 2, n, v)] = std::fma(eo[5], X[2], std::fma(eo[4], X[1], eo[3] * X[0]));
        }
      }
    }
  }
  void dss_face(FT *F) const {
    int G = (int)goff.size() - 1;
#pragma omp parallel for
    for (int g = 0; g < G; ++g)
      for (int k = 0; k < Nf; ++k) {
        FT s = 0;
        for (int c = goff[g]; c < goff[g + 1]; ++c) {
          int idx = gcopy[c];
          s = std::fma(gw[c], F[fi(idx / NN, idx % NN, k)], s);
        }
        for (int c = goff[g]; c < goff[g + 1]; ++c) {
          int idx = gcopy[c];
          F[fi(idx / NN, idx % NN, k)] = s;
        }
      }
  }
  void dss(FT *Yc, FT *Yf) const { dss_center(Yc, Nv); dss_face(Yf); }

  // ---- the horizontal Laplacians alone (analytic tests of the operators) ----
  // X is a centre block [Nh][4][16][Nv] holding a scalar f (comp 0) and a covariant
  // horizontal vector (u_1, u_2) (comps 1-2).  O receives, per level and after the DSS,
  // comp 0 = wdiv_h(grad_h f) (the scalar Laplacian of prep_hyperdiffusion_tendency!,
  // hyperdiffusion.jl:141-147) and comps 1-2 = the vector Laplacian of (u_1, u_2, 0)
  // with unit divergence factor (hyperdiffusion.jl:140), comp 3 = 0.
  void laplacians(const FT *X, FT *O) const {
#pragma omp parallel for
    for (int e = 0; e < Nh; ++e)
      for (int v = 0; v < Nv; ++v) {
        Slab s;
        slab_c(e, v, s);
        FT f[NN], u1[NN], u2[NN], u3[NN], g1[NN], g2[NN], F1[NN], F2[NN], Ls[NN], o1[NN], o2[NN], o3[NN];
        for (int n = 0; n < NN; ++n) {
          f[n] = X[ci(e, 0, n, v)];
          u1[n] = X[ci(e, 1, n, v)];
          u2[n] = X[ci(e, 2, n, v)];
          u3[n] = FT(0);
        }
        grad_h(f, g1, g2);
        for (int n = 0; n < NN; ++n) {
          F1[n] = s.gu0[n] * g1[n] + s.gu1[n] * g2[n];
          F2[n] = s.gu1[n] * g1[n] + s.gu2[n] * g2[n];
        }
        wdiv_h(s, F1, F2, Ls);
        vec_lap(s, u1, u2, u3, FT(1), o1, o2, o3);
        for (int n = 0; n < NN; ++n) {
          O[ci(e, 0, n, v)] = Ls[n];
          O[ci(e, 1, n, v)] = o1[n];
          O[ci(e, 2, n, v)] = o2[n];
          O[ci(e, 3, n, v)] = FT(0);
        }
      }
    dss_center(O, Nv);
  }

  // ---- remaining_tendency! ----
  std::vector<FT> Lap;  // [e][4][n][v]: (Ls, L1, L2, L3) so comps 1-2 are the C12 vector
  void remaining_tendency(FT *Tc, FT *Tf, const FT *Yc, const FT *Yf) {
    std::fill(Tc, Tc + ncen(), FT(0));
    std::fill(Tf, Tf + nfac(), FT(0));
    Lap.assign(ncen(), FT(0));
    // horizontal_dynamics_tendency! + prep_hyperdiffusion_tendency! (element-local)
#pragma omp parallel for
    for (int e = 0; e < Nh; ++e) {
      Slab s;
      for (int v = 0; v < Nv; ++v) {
        slab_c(e, v, s);
        FT rho[NN], F1[NN], F2[NN], h[NN], tmp[NN], a1[NN], a2[NN], u1[NN], u2[NN], u3[NN];
        for (int n = 0; n < NN; ++n) {
          size_t q = pi(e, n, v);
          rho[n] = Yc[ci(e, 0, n, v)];
          u1[n] = Yc[ci(e, 1, n, v)]; u2[n] = Yc[ci(e, 2, n, v)]; u3[n] = pre.ub3[q];
          F1[n] = rho[n] * pre.uc1[q]; F2[n] = rho[n] * pre.uc2[q];
          h[n] = pre.h[q];
        }
        // Yt.rho -= split_div(rho u, 1) = wdiv(rho u)
        FT dm[NN];
        wdiv_h(s, F1, F2, dm);
        for (int n = 0; n < NN; ++n) Tc[ci(e, 0, n, v)] -= dm[n];
        // Yt.rhoe -= split_div(rho u, h) = 1/2 wdiv(rho u h) + 1/2 (h wdiv(rho u) + rho u . grad h)
        FT G1[NN], G2[NN], dmh[NN];
        for (int n = 0; n < NN; ++n) { G1[n] = F1[n] * h[n]; G2[n] = F2[n] * h[n]; }
        wdiv_h(s, G1, G2, dmh);
        grad_h(h, a1, a2);
        for (int n = 0; n < NN; ++n)
          Tc[ci(e, 3, n, v)] -= (dmh[n] + h[n] * dm[n] + F1[n] * a1[n] + F2[n] * a2[n]) / FT(2);
        // Yt.u_h -= grad(K + Phi - Phi_r) + cp_d (th' grad Pi + grad(th' Pi) - Pi grad th') / 2
        FT Pi[NN], thp[NN], b1[NN], b2[NN], c1[NN], c2[NN], d1_[NN], d2_[NN];
        for (int n = 0; n < NN; ++n) {
          size_t q = pi(e, n, v);
#ifdef ORACLE_PHID
          tmp[n] = pre.K[q] + pre.phir[q];
#else
          tmp[n] = pre.K[q] + grav * zcp(e, n, v) - pre.phir[q];
#endif
          Pi[n] = pre.Pi[q];
          thp[n] = pre.thv[q] - pre.thvr[q];
        }
        grad_h(tmp, a1, a2);
        grad_h(Pi, b1, b2);
        FT tp[NN];
        for (int n = 0; n < NN; ++n) tp[n] = thp[n] * Pi[n];
        grad_h(tp, c1, c2);
        grad_h(thp, d1_, d2_);
        for (int n = 0; n < NN; ++n) {
          Tc[ci(e, 1, n, v)] -= a1[n] + cpd * (thp[n] * b1[n] + c1[n] - Pi[n] * d1_[n]) / FT(2);
          Tc[ci(e, 2, n, v)] -= a2[n] + cpd * (thp[n] * b2[n] + c2[n] - Pi[n] * d2_[n]) / FT(2);
        }
        // prep hyperdiffusion: grad/curl Laplacian of u_bar, scalar Laplacian of s_d - s_d,r
        FT o1[NN], o2[NN], o3[NN];
        vec_lap(s, u1, u2, u3, FT(1), o1, o2, o3);
        FT sd[NN], g1[NN], g2[NN], Ls[NN];
        for (int n = 0; n < NN; ++n) {
          size_t q = pi(e, n, v);
#ifdef ORACLE_PHID
          sd[n] = cpd * (pre.T[q] - T_ref(pre.Pi[q])) + pre.phir[q];
#else
          sd[n] = cpd * (pre.T[q] - T0) + grav * zcp(e, n, v) - sd_r(pre.Pi[q]);
#endif
        }
        grad_h(sd, g1, g2);
        for (int n = 0; n < NN; ++n) {
          FT x1 = s.gu0[n] * g1[n] + s.gu1[n] * g2[n], x2 = s.gu1[n] * g1[n] + s.gu2[n] * g2[n];
          g1[n] = x1; g2[n] = x2;
        }
        wdiv_h(s, g1, g2, Ls);
        for (int n = 0; n < NN; ++n) {
          Lap[ci(e, 0, n, v)] = Ls[n];
          Lap[ci(e, 1, n, v)] = o1[n];
          Lap[ci(e, 2, n, v)] = o2[n];
          Lap[ci(e, 3, n, v)] = o3[n];
        }
      }
    }
    // weighted_dss! of the Laplacians (remaining_tendency.jl:18-21)
    dss_center(Lap.data(), Nv, true);
    // apply_hyperdiffusion_tendency!
    std::vector<FT> L4u3(npt());
#pragma omp parallel for
    for (int e = 0; e < Nh; ++e) {
      Slab s;
      for (int v = 0; v < Nv; ++v) {
        slab_c(e, v, s);
        FT l1[NN], l2[NN], l3[NN], ls[NN], o1[NN], o2[NN], o3[NN];
        for (int n = 0; n < NN; ++n) {
          ls[n] = Lap[ci(e, 0, n, v)]; l1[n] = Lap[ci(e, 1, n, v)];
          l2[n] = Lap[ci(e, 2, n, v)]; l3[n] = Lap[ci(e, 3, n, v)];
        }
        vec_lap(s, l1, l2, l3, div_damp, o1, o2, o3);
        FT g1[NN], g2[NN], hd[NN];
        grad_h(ls, g1, g2);
        for (int n = 0; n < NN; ++n) {
          FT rho = Yc[ci(e, 0, n, v)];
          FT x1 = s.gu0[n] * g1[n] + s.gu1[n] * g2[n], x2 = s.gu1[n] * g1[n] + s.gu2[n] * g2[n];
          g1[n] = rho * x1; g2[n] = rho * x2;
        }
        wdiv_h(s, g1, g2, hd);
        for (int n = 0; n < NN; ++n) {
          Tc[ci(e, 1, n, v)] -= nu_v * o1[n];
          Tc[ci(e, 2, n, v)] -= nu_v * o2[n];
          Tc[ci(e, 3, n, v)] -= nu_s * hd[n];
          L4u3[pi(e, n, v)] = o3[n];
        }
      }
    }
    // Yt.u3 -= nu ᶠwinterp(ᶜJ ρ, C3(∇⁴u))  (extrapolated at the boundary faces)
#pragma omp parallel for
    for (int e = 0; e < Nh; ++e)
      for (int n = 0; n < NN; ++n) {
        for (int k = 0; k < Nf; ++k) {
          FT val;
          if (k == 0) val = L4u3[pi(e, n, 0)];
          else if (k == Nv) val = L4u3[pi(e, n, Nv - 1)];
          else {
            FT wa = Jc(e, n, k - 1) * Yc[ci(e, 0, n, k - 1)], wb = Jc(e, n, k) * Yc[ci(e, 0, n, k)];
            val = (wa * L4u3[pi(e, n, k - 1)] + wb * L4u3[pi(e, n, k)]) / (wa + wb);
          }
          Tf[fi(e, n, k)] -= nu_v * val;
        }
      }
    // explicit_vertical_advection_tendency! (deep atmosphere)
    std::vector<FT> om3(npt()), fo1(nfac()), fo2(nfac());
#pragma omp parallel for
    for (int e = 0; e < Nh; ++e) {
      Slab s;
      for (int v = 0; v < Nv; ++v) {  // ᶜω³ = wcurl(u_h)
        slab_c(e, v, s);
        FT u1[NN], u2[NN], o1[NN], o2[NN], o3[NN];
        for (int n = 0; n < NN; ++n) { u1[n] = Yc[ci(e, 1, n, v)]; u2[n] = Yc[ci(e, 2, n, v)]; }
        wcurl_h(s, u1, u2, nullptr, o1, o2, o3);
        for (int n = 0; n < NN; ++n) om3[pi(e, n, v)] = o3[n];
      }
      for (int k = 0; k < Nf; ++k) {  // ᶠω¹² = ᶠcurlᵥ(u_h) + CT12(wcurl(u_3))
        slab_f(e, k, s);
        FT w3[NN], o1[NN], o2[NN], o3[NN];
        for (int n = 0; n < NN; ++n) w3[n] = Yf[fi(e, n, k)];
        wcurl_h(s, nullptr, nullptr, w3, o1, o2, o3);
        for (int n = 0; n < NN; ++n) {
          FT cv1 = 0, cv2 = 0;
          if (k > 0 && k < Nv) {
            FT J = s.J[n];
            cv1 = -(Yc[ci(e, 2, n, k)] - Yc[ci(e, 2, n, k - 1)]) / J;
            cv2 = (Yc[ci(e, 1, n, k)] - Yc[ci(e, 1, n, k - 1)]) / J;
          }
          FT fh = FT(1) / rf[k];
          // Coriolis f^a = grad(xi^a) . 2 Omega z_hat: fh0 / r over a flat surface, per point over terrain
          const FT f1 = topo ? tf12f[fi(e, n, k) * 2 + 0] : fh0[hn(e, n) * 2 + 0] * fh;
          const FT f2 = topo ? tf12f[fi(e, n, k) * 2 + 1] : fh0[hn(e, n) * 2 + 1] * fh;
          fo1[fi(e, n, k)] = f1 + cv1 + o1[n];
          fo2[fi(e, n, k)] = f2 + cv2 + o2[n];
        }
      }
    }
#pragma omp parallel for
    for (int e = 0; e < Nh; ++e)
      for (int n = 0; n < NN; ++n) {
        // face cross product X = (f12 + w12) x (I^f(rho J) u^3)  -> C12, times face J
        std::vector<FT> X1(Nf), X2(Nf);
        for (int k = 0; k < Nf; ++k) {
          FT rJ;
          if (k == 0) rJ = Yc[ci(e, 0, n, 0)] * Jc(e, n, 0);
          else if (k == Nv) rJ = Yc[ci(e, 0, n, Nv - 1)] * Jc(e, n, Nv - 1);
          else rJ = (Yc[ci(e, 0, n, k - 1)] * Jc(e, n, k - 1) + Yc[ci(e, 0, n, k)] * Jc(e, n, k)) / FT(2);
          FT b3 = rJ * pre.u3c[fi(e, n, k)];
          FT Jf = Jfc(e, n, k);
          X1[k] = Jf * (fo2[fi(e, n, k)] * b3);
          X2[k] = Jf * (-fo1[fi(e, n, k)] * b3);
        }
        for (int v = 0; v < Nv; ++v) {
          size_t q = pi(e, n, v);
          FT rJ = Yc[ci(e, 0, n, v)] * Jc(e, n, v);
          FT t1v = (X1[v] + X1[v + 1]) / FT(2) / rJ;
          FT t2v = (X2[v] + X2[v + 1]) / FT(2) / rJ;
          // (f3 + w3) x CT12(u) -> C12 = J (-a3 u^2, a3 u^1)
          // f^3 = grad(xi^3) . 2 Omega z_hat: 2 Omega sin(lat) / dz over a flat surface
          FT a3 = (topo ? tf3c[q] : FT(2) * omega * sinlat[hn(e, n)] / dzc[v]) + om3[q];
          FT J = Jc(e, n, v);
          t1v += J * (-a3 * pre.uc2[q]);
          t2v += J * (a3 * pre.uc1[q]);
          Tc[ci(e, 1, n, v)] -= t1v;
          Tc[ci(e, 2, n, v)] -= t2v;
        }
        for (int k = 0; k < Nf; ++k) {
          // (f12 + w12) x I^f(CT12(u)) -> C3 = J (a1 c2 - a2 c1); plus ᶠgradᵥ(K)
          FT c1, c2, gK = 0;
          if (k == 0) { c1 = pre.uc1[pi(e, n, 0)]; c2 = pre.uc2[pi(e, n, 0)]; }
          else if (k == Nv) { c1 = pre.uc1[pi(e, n, Nv - 1)]; c2 = pre.uc2[pi(e, n, Nv - 1)]; }
          else {
            c1 = (pre.uc1[pi(e, n, k - 1)] + pre.uc1[pi(e, n, k)]) / FT(2);
            c2 = (pre.uc2[pi(e, n, k - 1)] + pre.uc2[pi(e, n, k)]) / FT(2);
            gK = pre.K[pi(e, n, k)] - pre.K[pi(e, n, k - 1)];
          }
          FT Jf = Jfc(e, n, k);
          Tf[fi(e, n, k)] -= Jf * (fo1[fi(e, n, k)] * c2 - fo2[fi(e, n, k)] * c1) + gK;
        }
        // additional_tendency!: Rayleigh sponge on u_h
        for (int v = 0; v < Nv; ++v) {
          FT b = beta_sponge(zcp(e, n, v), a_uh);
          Tc[ci(e, 1, n, v)] -= b * Yc[ci(e, 1, n, v)];
          Tc[ci(e, 2, n, v)] -= b * Yc[ci(e, 2, n, v)];
        }
        // Held-Suarez forcing (remaining_tendency.jl:154-172; held_suarez.jl:98-120 compute_dRhoT,
        // :122-141 compute_sigma / height_factor, :160-225 the rho e_tot relaxation times cv_d,
        // :230-296 the boundary-layer drag k_f = 1/day).  Flat surface: sigma = p / MSLP;
        // T = p / (rho R_d); latitude from the node's sin(lat).
        if (hs) {
          const FT s2 = sinlat[hn(e, n)] * sinlat[hn(e, n)], c2 = FT(1) - s2;
          const FT ka = FT(1) / (FT(40) * hs_day), ks = FT(1) / (FT(4) * hs_day), kf = FT(1) / hs_day;
          for (int v = 0; v < Nv; ++v) {
            const FT rho = Yc[ci(e, 0, n, v)], p = pre.p[pi(e, n, v)];
            const FT hf = std::max(FT(0), (p / hs_MSLP - hs_sb) / (FT(1) - hs_sb));
            const FT kT = ka + (ks - ka) * hf * (c2 * c2);
            const FT pr = p / hs_p0;
            const FT Teq = std::max(hs_Tmin, (hs_Teq - hs_dTy * s2 - hs_dthz * std::log(pr) * c2) * std::pow(pr, kappa));
            Tc[ci(e, 3, n, v)] -= kT * rho * (p / (rho * Rd) - Teq) * cvd;
            Tc[ci(e, 1, n, v)] -= kf * hf * Yc[ci(e, 1, n, v)];
            Tc[ci(e, 2, n, v)] -= kf * hf * Yc[ci(e, 2, n, v)];
          }
        }
      }
  }

  // ---- implicit_tendency! (implicit_vertical_advection_tendency!) ----
  // needs set_precomputed at Y first
  void implicit_tendency(FT *Tc, FT *Tf, const FT *Yc, const FT *Yf) {
    std::fill(Tc, Tc + ncen(), FT(0));
    std::fill(Tf, Tf + nfac(), FT(0));
#pragma omp parallel for
    for (int e = 0; e < Nh; ++e)
      for (int n = 0; n < NN; ++n) {
        std::vector<FT> flux(Nf), fh(Nf), fq(Nf, FT(0));
        for (int k = 0; k < Nf; ++k) {
          if (k == 0 || k == Nv) { flux[k] = 0; fh[k] = 0; continue; }
          FT rJ = (Yc[ci(e, 0, n, k - 1)] * Jc(e, n, k - 1) + Yc[ci(e, 0, n, k)] * Jc(e, n, k)) / FT(2);
          FT Jf = Jfc(e, n, k);
          FT F = rJ / Jf * pre.u3c[fi(e, n, k)];
          FT hb = (pre.h[pi(e, n, k - 1)] + pre.h[pi(e, n, k)]) / FT(2);
          flux[k] = Jf * F;       // ᶜadvdivᵥ multiplies the face value by ᶠJ
          fh[k] = Jf * F * hb;
          // central transport of q_tot = specific(rho q_tot, rho) (implicit_tendency.jl:211-215)
          if (moist) fq[k] = Jf * F * ((pre.q[pi(e, n, k - 1)] + pre.q[pi(e, n, k)]) / FT(2));
        }
        for (int v = 0; v < Nv; ++v) {
          FT J = Jc(e, n, v);
          Tc[ci(e, 0, n, v)] -= (flux[v + 1] - flux[v]) / J;
          Tc[ci(e, 3, n, v)] -= (fh[v + 1] - fh[v]) / J;
          if (moist) Tc[ci(e, 4, n, v)] -= (fq[v + 1] - fq[v]) / J;
        }
        for (int k = 0; k < Nf; ++k) {
          FT val = 0;
          if (k > 0 && k < Nv) {
            size_t a = pi(e, n, k - 1), b = pi(e, n, k);
#ifdef ORACLE_PHID
            FT gPhi = pre.phir[b] - pre.phir[a], gPhir = 0;
#else
            FT gPhi = grav * (zcp(e, n, k) - zcp(e, n, k - 1));
            FT gPhir = pre.phir[b] - pre.phir[a];
#endif
            FT thd = ((pre.thv[a] - pre.thvr[a]) + (pre.thv[b] - pre.thvr[b])) / FT(2);
            FT gPi = pre.Pi[b] - pre.Pi[a];
            val = -(gPhi - gPhir + cpd * thd * gPi);
          }
          val -= beta_sponge(zfp(e, n, k), a_w) * Yf[fi(e, n, k)];
          Tf[fi(e, n, k)] = val;
        }
      }
  }

  // ---- Jacobian (update_advection_jacobian!, dry, no topography) ----
  struct Jac {
    std::vector<FT> Mru, Meu;             // [col][v][2]  (u3 faces v, v+1)
    std::vector<FT> Mur, Mue;             // [col][k][2]  (centres k-1, k)
    std::vector<FT> Muh;                  // [col][k][2][2] (centres k-1, k; comps 1, 2)
    std::vector<FT> Muu;                  // [col][k][3]  (faces k-1, k, k+1)
    std::vector<FT> Mrh, Meh;             // terrain: [col][v][3][2] (centres v-1, v, v+1; comps 1, 2)
    std::vector<FT> Mqu;                  // moist: [col][v][2] (rho q_tot, u3 faces v, v+1)
    std::vector<FT> Muq;                  // moist: [col][k][2] (u3, rho q_tot of centres k-1, k)
  } jac;

  void update_jacobian(const FT *Yc, const FT *Yf, FT dtg) {
    size_t C = (size_t)Nh * NN;
    jac.Mru.assign(C * Nv * 2, 0); jac.Meu.assign(C * Nv * 2, 0);
    jac.Mur.assign(C * Nf * 2, 0); jac.Mue.assign(C * Nf * 2, 0);
    jac.Muh.assign(C * Nf * 4, 0); jac.Muu.assign(C * Nf * 3, 0);
    if (topo) { jac.Mrh.assign(C * Nv * 6, 0); jac.Meh.assign(C * Nv * 6, 0); }
    if (moist) { jac.Mqu.assign(C * Nv * 2, 0); jac.Muq.assign(C * Nf * 2, 0); }
    const FT kapd = Rd / cvd;  // kappa_m for dry air
    // moist: kappa_m = R_m / cv_m of each centre (ᶜkappa_m_field!, manual_sparse_jacobian.jl:646-662)
    auto kapc = [&](size_t q) { return moist ? pre.kapm[q] : kapd; };
#pragma omp parallel for
    for (int e = 0; e < Nh; ++e)
      for (int n = 0; n < NN; ++n) {
        size_t col = hn(e, n);
        // centre rows: d(rho_t)/d(u3), d(rhoe_t)/d(u3)
        for (int v = 0; v < Nv; ++v) {
          FT J = Jc(e, n, v);
          for (int s = 0; s < 2; ++s) {
            int k = v + s;
            FT val = 0, vh = 0, vq = 0;
            if (k > 0 && k < Nv) {
              FT rJ = (Yc[ci(e, 0, n, k - 1)] * Jc(e, n, k - 1) + Yc[ci(e, 0, n, k)] * Jc(e, n, k)) / FT(2);
              FT g33 = g33f(e, n, k);
              FT sign = s ? FT(-1) : FT(1);  // -ᶜadvdivᵥ: -(+ at v+1, - at v)/J
              val = sign * rJ * g33 / J;
              FT hb = (pre.h[pi(e, n, k - 1)] + pre.h[pi(e, n, k)]) / FT(2);
              vh = val * hb;
              // (rho q_tot, u_3): the same with ᶠinterp(q_tot) (manual_sparse_jacobian.jl:770-783)
              if (moist) vq = val * ((pre.q[pi(e, n, k - 1)] + pre.q[pi(e, n, k)]) / FT(2));
            }
            jac.Mru[(col * Nv + v) * 2 + s] = dtg * val;
            jac.Meu[(col * Nv + v) * 2 + s] = dtg * vh;
            if (moist) jac.Mqu[(col * Nv + v) * 2 + s] = dtg * vq;
          }
        }
        for (int k = 0; k < Nf; ++k) {
          FT beta = beta_sponge(zfp(e, n, k), a_w);
          if (k == 0 || k == Nv) {
            jac.Muu[(col * Nf + k) * 3 + 1] = -dtg * beta - FT(1);
            continue;
          }
          size_t a = pi(e, n, k - 1), b = pi(e, n, k);
          FT ra = Yc[ci(e, 0, n, k - 1)], rb = Yc[ci(e, 0, n, k)];
          FT rbar = (ra + rb) / FT(2);
          const FT ka = kapc(a), kb = kapc(b);
          // ᶜ∂p∂ρ = kappa_m (T_0 cp_d - K - Phi) + (R_d - kappa_m cv_d) T; the second term is 0
          // for dry air (manual_sparse_jacobian.jl:817-819)
          auto dpdr = [&](size_t q, FT km) {
            const FT d = km * (T0 * cpd - pre.K[q] - grav * zcp(e, n, (int)(q % Nv)));
            return moist ? d + (Rd - km * cvd) * pre.T[q] : d;
          };
          FT thvb = (pre.thv[a] + pre.thv[b]) / FT(2);
          FT gPi = pre.Pi[b] - pre.Pi[a];
          FT buoy = cpd * thvb * gPi / rbar;  // times ᶠinterp_matrix (1/2, 1/2)
          // ᶠp_grad_matrix = diag(-1/ρ̄) ᶠgradᵥ_matrix  (−1 at k−1, +1 at k)
          jac.Mur[(col * Nf + k) * 2 + 0] = dtg * (dpdr(a, ka) / rbar + buoy / FT(2));
          jac.Mur[(col * Nf + k) * 2 + 1] = dtg * (-dpdr(b, kb) / rbar + buoy / FT(2));
          jac.Mue[(col * Nf + k) * 2 + 0] = dtg * (ka / rbar);
          jac.Mue[(col * Nf + k) * 2 + 1] = dtg * (-kb / rbar);
          if (moist) {
            // (u_3, rho q_tot) = dtγ ᶠp_grad_matrix ⋅ diag(ᶜ∂p∂ρq_tot) (manual_sparse_jacobian.jl:827-831)
            jac.Muq[(col * Nf + k) * 2 + 0] = dtg * (pre.dpdq[a] / rbar);
            jac.Muq[(col * Nf + k) * 2 + 1] = dtg * (-pre.dpdq[b] / rbar);
          }
          // (u3, u_h): p_grad * diag(-kappa rho) * dK/du_h,  dK/du_i = u^i
          jac.Muh[(col * Nf + k) * 4 + 0] = dtg * (-ka * ra / rbar) * pre.uc1[a];
          jac.Muh[(col * Nf + k) * 4 + 1] = dtg * (-ka * ra / rbar) * pre.uc2[a];
          jac.Muh[(col * Nf + k) * 4 + 2] = dtg * (kb * rb / rbar) * pre.uc1[b];
          jac.Muh[(col * Nf + k) * 4 + 3] = dtg * (kb * rb / rbar) * pre.uc2[b];
          // (u3, u3): p_grad * diag(-kappa rho) * dK/du3 - beta - I ; dK_v/du3_f = u^3_f / 2
          if (topo) {
            // over terrain dK_v/du3_f = (g^33 u_3)_f / 2 + CT3(u_h)_v / 2 (∂ᶜK_∂ᶠu₃,
            // manual_sparse_jacobian.jl:754-756)
            const FT wm = pre.w3c[fi(e, n, k - 1)], w0 = pre.w3c[fi(e, n, k)], wp = pre.w3c[fi(e, n, k + 1)];
            const FT ca = pre.ct3[a], cb = pre.ct3[b];
            jac.Muu[(col * Nf + k) * 3 + 0] = dtg * (-kapd * ra * (wm + ca) / (FT(2) * rbar));
            jac.Muu[(col * Nf + k) * 3 + 1] =
                dtg * (kapd * (rb * (w0 + cb) - ra * (w0 + ca)) / (FT(2) * rbar) - beta) - FT(1);
            jac.Muu[(col * Nf + k) * 3 + 2] = dtg * (kapd * rb * (wp + cb) / (FT(2) * rbar));
          } else if (moist) {
            FT um = pre.u3c[fi(e, n, k - 1)], u0 = pre.u3c[fi(e, n, k)], up = pre.u3c[fi(e, n, k + 1)];
            jac.Muu[(col * Nf + k) * 3 + 0] = dtg * (-ka * ra * um / (FT(2) * rbar));
            jac.Muu[(col * Nf + k) * 3 + 1] = dtg * ((kb * rb - ka * ra) * u0 / (FT(2) * rbar) - beta) - FT(1);
            jac.Muu[(col * Nf + k) * 3 + 2] = dtg * (kb * rb * up / (FT(2) * rbar));
          } else {
            FT um = pre.u3c[fi(e, n, k - 1)], u0 = pre.u3c[fi(e, n, k)], up = pre.u3c[fi(e, n, k + 1)];
            jac.Muu[(col * Nf + k) * 3 + 0] = dtg * (-kapd * ra * um / (FT(2) * rbar));
            jac.Muu[(col * Nf + k) * 3 + 1] = dtg * (kapd * (rb - ra) * u0 / (FT(2) * rbar) - beta) - FT(1);
            jac.Muu[(col * Nf + k) * 3 + 2] = dtg * (kapd * rb * up / (FT(2) * rbar));
          }
        }
        if (topo) {
          // (rho, u_h) and (rho e_tot, u_h) over terrain (manual_sparse_jacobian.jl:761-763, 771-775):
          // dtγ ᶜadvection_matrix ⋅ [diag(ᶠinterp(h_tot))] ⋅ ᶠwinterp_matrix(ᶜJ ρ) ⋅ diag(g^3h).
          // The interior face k's flux ρ̄J u^3 holds ½ Σ_c ρJ_c CT3(u_h)_c over its two centres,
          // so d(flux_k)/du_a,c = ½ ρ_c J_c g^3a_c; the boundary faces carry no flux.
          for (int v = 0; v < Nv; ++v) {
            const FT iJ = FT(1) / Jc(e, n, v);
            for (int t = 0; t < 3; ++t) {
              const int c = v - 1 + t;
              FT wr = 0, we = 0;
              if (c >= 0 && c < Nv) {
                const FT half_rJ = Yc[ci(e, 0, n, c)] * Jc(e, n, c) / FT(2);
                // face v (below centre v, +) and face v + 1 (above, -)
                if ((c == v - 1 || c == v) && v >= 1) {
                  const FT hb = (pre.h[pi(e, n, v - 1)] + pre.h[pi(e, n, v)]) / FT(2);
                  wr += half_rJ * iJ;
                  we += half_rJ * iJ * hb;
                }
                if ((c == v || c == v + 1) && v + 1 <= Nv - 1) {
                  const FT hb = (pre.h[pi(e, n, v)] + pre.h[pi(e, n, v + 1)]) / FT(2);
                  wr -= half_rJ * iJ;
                  we -= half_rJ * iJ * hb;
                }
              }
              for (int a2 = 0; a2 < 2; ++a2) {
                const FT g3a = c >= 0 && c < Nv ? (a2 == 0 ? g31c(e, n, c) : g32c(e, n, c)) : FT(0);
                jac.Mrh[((col * Nv + v) * 3 + t) * 2 + a2] = dtg * wr * g3a;
                jac.Meh[((col * Nv + v) * 3 + t) * 2 + a2] = dtg * we * g3a;
              }
            }
          }
        }
      }
  }
  // The (rho, u_h) and (rho e_tot, u_h) blocks applied to V_uh, per centre (terrain only).
  void uh_coupling(int e, int n, const FT *Vc, int v, FT &gr, FT &ge) const {
    gr = ge = FT(0);
    if (!topo) return;
    const size_t col = hn(e, n);
    for (int t = 0; t < 3; ++t) {
      const int c = v - 1 + t;
      if (c < 0 || c >= Nv) continue;
      for (int a2 = 0; a2 < 2; ++a2) {
        const FT x = Vc[ci(e, 1 + a2, n, c)];
        gr += jac.Mrh[((col * Nv + v) * 3 + t) * 2 + a2] * x;
        ge += jac.Meh[((col * Nv + v) * 3 + t) * 2 + a2] * x;
      }
    }
  }

  // ---- ldiv!: BlockArrowheadSolve(rho, rhoe; alg2 = BlockLowerTriangularSolve(u_h)) ----
  // Moist 0M: the reference solves with ApproximateBlockArrowheadIterativeSolve over (rho, rho e_tot,
  // rho q_tot) (manual_sparse_jacobian.jl:539-584) because diffusion and sedimentation may fill the
  // scalar blocks; with 0M and neither, those blocks are -I ((rho e_tot, rho q_tot) = 0,
  // manual_sparse_jacobian.jl:906-910), its block-arrowhead Schur preconditioner is the exact
  // inverse, and the solve is the same Schur complement onto u_3 with a third scalar row.
  void ldiv(FT *Xc, FT *Xf, const FT *Rc, const FT *Rf) const {
#pragma omp parallel for
    for (int e = 0; e < Nh; ++e)
      for (int n = 0; n < NN; ++n) {
        size_t col = hn(e, n);
        std::vector<FT> A(Nf), B(Nf), Cc(Nf), Dd(Nf);
        // Δu_h = -R_uh
        for (int v = 0; v < Nv; ++v) {
          Xc[ci(e, 1, n, v)] = -Rc[ci(e, 1, n, v)];
          Xc[ci(e, 2, n, v)] = -Rc[ci(e, 2, n, v)];
        }
        // over terrain the (rho, u_h), (rho e_tot, u_h) blocks times Δu_h = -R_uh move to the
        // right-hand sides of the scalar rows: R_x + M_x,uh R_uh
        std::vector<FT> Rr(Nv), Re(Nv), Rq(Nv, FT(0));
        for (int v = 0; v < Nv; ++v) {
          FT gr, ge;
          uh_coupling(e, n, Rc, v, gr, ge);
          Rr[v] = topo ? Rc[ci(e, 0, n, v)] + gr : Rc[ci(e, 0, n, v)];
          Re[v] = topo ? Rc[ci(e, 3, n, v)] + ge : Rc[ci(e, 3, n, v)];
          if (moist) Rq[v] = Rc[ci(e, 4, n, v)];
        }
        for (int k = 0; k < Nf; ++k) {
          const FT *mu = &jac.Muu[(col * Nf + k) * 3];
          const FT *mr = &jac.Mur[(col * Nf + k) * 2];
          const FT *me = &jac.Mue[(col * Nf + k) * 2];
          const FT *mh = &jac.Muh[(col * Nf + k) * 4];
          FT a = mu[0], b = mu[1], c = mu[2];
          FT rhs = Rf[fi(e, n, k)];
          for (int s = 0; s < 2; ++s) {
            int v = k - 1 + s;
            if (v < 0 || v >= Nv) continue;
            // S += M_u,x M_x,u ; rhs += M_u,x R_x
            const FT *mru = &jac.Mru[(col * Nv + v) * 2];
            const FT *meu = &jac.Meu[(col * Nv + v) * 2];
            // centre v couples faces v (slot 0) and v+1 (slot 1)
            FT cr = mr[s], ce = me[s];
            // face v = k - 1 + s; offset of face v relative to k: s - 1
            // face v+1 relative to k: s
            FT t0 = cr * mru[0] + ce * meu[0];  // -> face v
            FT t1 = cr * mru[1] + ce * meu[1];  // -> face v+1
            if (moist) {
              const FT cq = jac.Muq[(col * Nf + k) * 2 + s];
              const FT *mqu = &jac.Mqu[(col * Nv + v) * 2];
              t0 += cq * mqu[0];
              t1 += cq * mqu[1];
              rhs += cq * Rq[v];
            }
            if (s == 0) { a += t0; b += t1; } else { b += t0; c += t1; }
            rhs += cr * Rr[v] + ce * Re[v];
            rhs += mh[2 * s] * Rc[ci(e, 1, n, v)] + mh[2 * s + 1] * Rc[ci(e, 2, n, v)];
          }
          A[k] = a; B[k] = b; Cc[k] = c; Dd[k] = rhs;
        }
        // Thomas algorithm
        std::vector<FT> cp(Nf), dp(Nf), x(Nf);
        cp[0] = Cc[0] / B[0]; dp[0] = Dd[0] / B[0];
        for (int k = 1; k < Nf; ++k) {
          FT m = B[k] - A[k] * cp[k - 1];
          cp[k] = Cc[k] / m;
          dp[k] = (Dd[k] - A[k] * dp[k - 1]) / m;
        }
        x[Nf - 1] = dp[Nf - 1];
        for (int k = Nf - 2; k >= 0; --k) x[k] = dp[k] - cp[k] * x[k + 1];
        for (int k = 0; k < Nf; ++k) Xf[fi(e, n, k)] = x[k];
        for (int v = 0; v < Nv; ++v) {
          const FT *mru = &jac.Mru[(col * Nv + v) * 2];
          const FT *meu = &jac.Meu[(col * Nv + v) * 2];
          Xc[ci(e, 0, n, v)] = mru[0] * x[v] + mru[1] * x[v + 1] - Rr[v];
          Xc[ci(e, 3, n, v)] = meu[0] * x[v] + meu[1] * x[v + 1] - Re[v];
          if (moist) {
            const FT *mqu = &jac.Mqu[(col * Nv + v) * 2];
            Xc[ci(e, 4, n, v)] = mqu[0] * x[v] + mqu[1] * x[v + 1] - Rq[v];
          }
        }
      }
  }

  // W V with the stored blocks (W = dtγ ∂T/∂Y − I restricted to the manual sparsity)
  void jac_apply(FT *Oc, FT *Of, const FT *Vc, const FT *Vf) const {
#pragma omp parallel for
    for (int e = 0; e < Nh; ++e)
      for (int n = 0; n < NN; ++n) {
        size_t col = hn(e, n);
        for (int v = 0; v < Nv; ++v) {
          const FT *mru = &jac.Mru[(col * Nv + v) * 2];
          const FT *meu = &jac.Meu[(col * Nv + v) * 2];
          FT a = Vf[fi(e, n, v)], b = Vf[fi(e, n, v + 1)];
          Oc[ci(e, 0, n, v)] = -Vc[ci(e, 0, n, v)] + mru[0] * a + mru[1] * b;
          Oc[ci(e, 3, n, v)] = -Vc[ci(e, 3, n, v)] + meu[0] * a + meu[1] * b;
          if (topo) {
            FT gr, ge;
            uh_coupling(e, n, Vc, v, gr, ge);
            Oc[ci(e, 0, n, v)] += gr;
            Oc[ci(e, 3, n, v)] += ge;
          }
          Oc[ci(e, 1, n, v)] = -Vc[ci(e, 1, n, v)];
          Oc[ci(e, 2, n, v)] = -Vc[ci(e, 2, n, v)];
          if (moist) {
            const FT *mqu = &jac.Mqu[(col * Nv + v) * 2];
            Oc[ci(e, 4, n, v)] = -Vc[ci(e, 4, n, v)] + mqu[0] * a + mqu[1] * b;
          }
        }
        for (int k = 0; k < Nf; ++k) {
          const FT *mu = &jac.Muu[(col * Nf + k) * 3];
          const FT *mr = &jac.Mur[(col * Nf + k) * 2];
          const FT *me = &jac.Mue[(col * Nf + k) * 2];
          const FT *mh = &jac.Muh[(col * Nf + k) * 4];
          FT s = mu[1] * Vf[fi(e, n, k)];
          if (k > 0) s += mu[0] * Vf[fi(e, n, k - 1)];
          if (k < Nv) s += mu[2] * Vf[fi(e, n, k + 1)];
          for (int t = 0; t < 2; ++t) {
            int v = k - 1 + t;
            if (v < 0 || v >= Nv) continue;
            s += mr[t] * Vc[ci(e, 0, n, v)] + me[t] * Vc[ci(e, 3, n, v)];
            s += mh[2 * t] * Vc[ci(e, 1, n, v)] + mh[2 * t + 1] * Vc[ci(e, 2, n, v)];
            if (moist) s += jac.Muq[(col * Nf + k) * 2 + t] * Vc[ci(e, 4, n, v)];
          }
          Of[fi(e, n, k)] = s;
        }
      }
  }

  // ---- correct_implicit_advection_tendency! (van Leer minus central; ρe_tot, and ρq_tot when moist) ----
  FT vanleer_face(FT u, const FT *a, int k) const {
    // a: centre values of the column; face k between centres k-1 and k (interior)
    bool near = (k == 1 || k == Nv - 1);
    if (u >= 0) {
      FT a0 = a[k - 1];
      if (near) return u * a0;
      FT am = a[k - 2], ap = a[k];
      FT da = (ap - am) / FT(2);
      FT mn = std::min(am, std::min(a0, ap)), mx = std::max(am, std::max(a0, ap));
      FT sl = std::copysign(std::min(std::fabs(da), std::min(FT(2) * (a0 - mn), FT(2) * (mx - a0))), da);
      return u * (a0 + sl * (FT(1) - std::fabs(u) * dt_model) / FT(2));
    } else {
      FT a0 = a[k];
      if (near) return u * a0;
      FT am = a[k - 1], ap = a[k + 1];
      FT da = (ap - am) / FT(2);
      FT mn = std::min(am, std::min(a0, ap)), mx = std::max(am, std::max(a0, ap));
      FT sl = std::copysign(std::min(std::fabs(da), std::min(FT(2) * (a0 - mn), FT(2) * (mx - a0))), da);
      return u * (a0 - sl * (FT(1) - std::fabs(u) * dt_model) / FT(2));
    }
  }
  void correct_implicit(FT *Tc, FT *Tf, const FT *Yc, const FT *Yf) {
    std::fill(Tc, Tc + ncen(), FT(0));
    std::fill(Tf, Tf + nfac(), FT(0));
    if (!upwinding) return;
#pragma omp parallel for
    for (int e = 0; e < Nh; ++e)
      for (int n = 0; n < NN; ++n) {
        std::vector<FT> h(Nv), fup(Nf, 0), fc(Nf, 0);
        for (int comp = 3; comp <= (moist ? 4 : 3); ++comp) {
          // the transported specific quantity: h_tot for rho e_tot, q_tot for rho q_tot
          for (int v = 0; v < Nv; ++v) h[v] = comp == 3 ? pre.h[pi(e, n, v)] : pre.q[pi(e, n, v)];
          for (int k = 1; k < Nv; ++k) {
            FT rJ = (Yc[ci(e, 0, n, k - 1)] * Jc(e, n, k - 1) + Yc[ci(e, 0, n, k)] * Jc(e, n, k)) / FT(2);
            FT u = pre.u3c[fi(e, n, k)];
            FT Jf = Jfc(e, n, k);
            fup[k] = Jf * (rJ / Jf * vanleer_face(u, h.data(), k));
            fc[k] = Jf * (rJ / Jf * (u * (h[k - 1] + h[k]) / FT(2)));
          }
          for (int v = 0; v < Nv; ++v) {
            FT J = Jc(e, n, v);
            FT vup = -(fup[v + 1] - fup[v]) / J;
            FT vc = -(fc[v + 1] - fc[v]) / J;
            Tc[ci(e, comp, n, v)] = vup - vc;
          }
        }
      }
  }

  // ---- ARS343 IMEX step with one Newton iteration (ClimaTimeSteppers stage loop) ----
  FT ae[4][4], ai[4][4], be[4], bi[4];
  void tableau() {
    double g = 0.4358665215084590;
    double a42 = 0.5529291480359398, a43 = a42;
    double b1 = -1.5 * g * g + 4 * g - 0.25, b2 = 1.5 * g * g - 5 * g + 1.25;
    double a31 = (1 - 4.5 * g + 1.5 * g * g) * a42 + (2.75 - 10.5 * g + 3.75 * g * g) * a43 - 3.5 + 13 * g - 4.5 * g * g;
    double a32 = (-1 + 4.5 * g - 1.5 * g * g) * a42 + (-2.75 + 10.5 * g - 3.75 * g * g) * a43 + 4 - 12.5 * g + 4.5 * g * g;
    double a41 = 1 - a42 - a43;
    double E[4][4] = {{0, 0, 0, 0}, {g, 0, 0, 0}, {a31, a32, 0, 0}, {a41, a42, a43, 0}};
    double I[4][4] = {{0, 0, 0, 0}, {0, g, 0, 0}, {0, (1 - g) / 2, g, 0}, {0, b1, b2, g}};
    double B[4] = {0, b1, b2, g};
    for (int i = 0; i < 4; ++i) {
      for (int j = 0; j < 4; ++j) { ae[i][j] = (FT)E[i][j]; ai[i][j] = (FT)I[i][j]; }
      be[i] = (FT)B[i]; bi[i] = (FT)B[i];
    }
  }

  std::vector<FT> Te_c[4], Te_f[4], Ti_c[4], Ti_f[4], Uc, Uf, Hc, Hf, Rc_, Rf_, Xc_, Xf_, Kc, Kf;
  // ORACLE_STORE32 (a separate build for the precision study only): every field the step
  // stores (stage states, tendencies, the state) is rounded to FP32 while the arithmetic
  // stays in FT, which separates the FP32 storage error from the FP32 arithmetic error.
#ifdef ORACLE_STORE32
  static void R32v(std::vector<FT> &v) { for (auto &x : v) x = (FT)(float)x; }
  static void R32p(FT *p, size_t n) { for (size_t i = 0; i < n; ++i) p[i] = (FT)(float)p[i]; }
#else
  static void R32v(std::vector<FT> &) {}
  static void R32p(FT *, size_t) {}
#endif
  void step(FT *Yc, FT *Yf, double dt_) {
    FT dt = (FT)dt_;
    size_t NC = ncen(), NF = nfac();
    for (int i = 0; i < 4; ++i) {
      Te_c[i].assign(NC, 0); Te_f[i].assign(NF, 0); Ti_c[i].assign(NC, 0); Ti_f[i].assign(NF, 0);
    }
    Uc.resize(NC); Uf.resize(NF); Hc.resize(NC); Hf.resize(NF);
    Rc_.resize(NC); Rf_.resize(NF); Xc_.resize(NC); Xf_.resize(NF); Kc.resize(NC); Kf.resize(NF);
    for (int i = 0; i < 4; ++i) {
      // U = u + dt sum_j (ã_ij T_exp_j + a_ij T_imp_j)
#pragma omp parallel for
      for (size_t q = 0; q < NC; ++q) {
        FT s = Yc[q];
        for (int j = 0; j < i; ++j) {
          if (ae[i][j] != FT(0)) s += dt * ae[i][j] * Te_c[j][q];
          if (ai[i][j] != FT(0)) s += dt * ai[i][j] * Ti_c[j][q];
        }
        Uc[q] = s;
      }
#pragma omp parallel for
      for (size_t q = 0; q < NF; ++q) {
        FT s = Yf[q];
        for (int j = 0; j < i; ++j) {
          if (ae[i][j] != FT(0)) s += dt * ae[i][j] * Te_f[j][q];
          if (ai[i][j] != FT(0)) s += dt * ai[i][j] * Ti_f[j][q];
        }
        Uf[q] = s;
      }
      R32v(Uc); R32v(Uf);
      if (i > 0 || dss_stage1) dss(Uc.data(), Uf.data());
      R32v(Uc); R32v(Uf);
      FT aii = ai[i][i];
      if (aii != FT(0)) {
        FT dtg = dt * aii;
        Hc = Uc; Hf = Uf;  // Û (temp)
        // Newton, one iteration
        set_precomputed(Uc.data(), Uf.data());  // cache_imp!
        implicit_tendency(Kc.data(), Kf.data(), Uc.data(), Uf.data());
        for (size_t q = 0; q < NC; ++q) Rc_[q] = Hc[q] + dtg * Kc[q] - Uc[q];
        for (size_t q = 0; q < NF; ++q) Rf_[q] = Hf[q] + dtg * Kf[q] - Uf[q];
        update_jacobian(Uc.data(), Uf.data(), dtg);
        ldiv(Xc_.data(), Xf_.data(), Rc_.data(), Rf_.data());
        for (size_t q = 0; q < NC; ++q) Uc[q] -= Xc_[q];
        for (size_t q = 0; q < NF; ++q) Uf[q] -= Xf_[q];
        set_precomputed(Uc.data(), Uf.data());  // cache! after the solve
        if (upwinding) {
          correct_implicit(Kc.data(), Kf.data(), Uc.data(), Uf.data());
          for (size_t q = 0; q < NC; ++q) Uc[q] += dtg * Kc[q];
          set_precomputed(Uc.data(), Uf.data());
        }
        R32v(Uc); R32v(Uf);
        for (size_t q = 0; q < NC; ++q) Ti_c[i][q] = (Uc[q] - Hc[q]) / dtg;
        for (size_t q = 0; q < NF; ++q) Ti_f[i][q] = (Uf[q] - Hf[q]) / dtg;
        R32v(Ti_c[i]); R32v(Ti_f[i]);
      } else {
        set_precomputed(Uc.data(), Uf.data());  // cache!
      }
      remaining_tendency(Te_c[i].data(), Te_f[i].data(), Uc.data(), Uf.data());
      R32v(Te_c[i]); R32v(Te_f[i]);
    }
#pragma omp parallel for
    for (size_t q = 0; q < NC; ++q) {
      FT s = Yc[q];
      for (int j = 0; j < 4; ++j) {
        if (be[j] != FT(0)) s += dt * be[j] * Te_c[j][q];
        if (bi[j] != FT(0)) s += dt * bi[j] * Ti_c[j][q];
      }
      Yc[q] = s;
    }
#pragma omp parallel for
    for (size_t q = 0; q < NF; ++q) {
      FT s = Yf[q];
      for (int j = 0; j < 4; ++j) {
        if (be[j] != FT(0)) s += dt * be[j] * Te_f[j][q];
        if (bi[j] != FT(0)) s += dt * bi[j] * Ti_f[j][q];
      }
      Yf[q] = s;
    }
    R32p(Yc, NC); R32p(Yf, NF);
    dss(Yc, Yf);
    R32p(Yc, NC); R32p(Yf, NF);
    set_precomputed(Yc, Yf);
  }

  // ∫ rho dV, ∫ rho e_tot dV (and, moist, ∫ rho q_tot dV: the three sums of
  // check_conservation, solve.jl:216-265) with compensated (Neumaier) FP64 summation
  void global_sums(const FT *Yc, double *out) const {
    for (int c = 0; c < (nfc == 5 ? 3 : 2); ++c) {
      const int comp = c == 0 ? 0 : c == 1 ? 3 : 4;
      double s = 0, comp_ = 0;
      for (int e = 0; e < Nh; ++e)
        for (int n = 0; n < NN; ++n)
          for (int v = 0; v < Nv; ++v) {
            double x = (double)Yc[ci(e, comp, n, v)] * (double)W[n] *
                       (topo ? (double)tJc[pi(e, n, v)] : ((double)Jh[hn(e, n)] * rc[v] * rc[v] * dzc[v]));
            double t = s + x;
            if (std::fabs(s) >= std::fabs(x)) comp_ += (s - t) + x; else comp_ += (x - t) + s;
            s = t;
          }
      out[c] = s + comp_;
    }
  }

  void init(const OracleGeom *g, const OracleParams *p) {
    Nh = g->Nh; Nv = g->Nv; Nf = Nv + 1;
    grav = p->grav; omega = p->omega; Rd = p->R_d; cpd = p->cp_d; cvd = p->cv_d; T0 = p->T_0; pref = p->p_ref;
    Tmin_ref = p->T_min_ref; Tsfc_ref = p->T_surf_ref; Tmin_sgs = p->T_min_sgs; R = p->radius;
    nu_v = p->nu_v; nu_s = p->nu_s; div_damp = p->div_damp; zd = p->sponge_zd; a_uh = p->alpha_uh; a_w = p->alpha_w;
    zmax = p->z_max; dt_model = p->dt_model; upwinding = p->upwinding; dss_stage1 = p->dss_stage1;
    kappa = Rd / cpd;
    hs = p->held_suarez; hs_day = p->hs_day; hs_sb = p->hs_sigma_b; hs_dTy = p->hs_dT_y; hs_Teq = p->hs_T_equator;
    hs_dthz = p->hs_dtheta_z; hs_Tmin = p->hs_T_min; hs_p0 = p->hs_p_ref_theta; hs_MSLP = p->hs_MSLP;
    moist = p->moist;
    nfc = moist ? 5 : 4;
    if (moist) {
      Rv = p->R_v; cpv = p->cp_v; cpl = p->cp_l; cpi = p->cp_i;
      cvv = cpv - Rv; cvl = cpl; cvi = cpi;
      Lv0 = p->LH_v0; Ls0 = p->LH_s0; Ttr = p->T_triple; ptr = p->press_triple;
      Tfrz = p->T_freeze; Tice = p->T_icenuc; pice = p->pow_icenuc;
      ev0 = Lv0 - Rv * T0; ei0 = Ls0 - Lv0;
      sa_iters = p->sa_iters;
    }
    for (int n = 0; n < NN; ++n) W[n] = g->W[n];
    for (int i = 0; i < NQ; ++i) for (int k = 0; k < NQ; ++k) D[i][k] = g->D[i * NQ + k];
    size_t H = (size_t)Nh * NN;
    Jh.assign(g->Jh, g->Jh + H);
    gup.assign(g->gup, g->gup + 3 * H); gdn.assign(g->gdn, g->gdn + 3 * H);
    sinlat.assign(g->sinlat, g->sinlat + H); fh0.assign(g->fh0, g->fh0 + 2 * H);
    ecov.assign(g->ecov, g->ecov + 6 * H); econ.assign(g->econ, g->econ + 6 * H);
    zf.assign(g->zf, g->zf + Nf);
    zc.resize(Nv); dzc.resize(Nv); rc.resize(Nv); dzf.resize(Nf); rf.resize(Nf);
    for (int v = 0; v < Nv; ++v) {
      zc[v] = (FT)((g->zf[v] + g->zf[v + 1]) / 2);
      dzc[v] = (FT)(g->zf[v + 1] - g->zf[v]);
      rc[v] = (FT)((p->radius + (g->zf[v] + g->zf[v + 1]) / 2) / p->radius);
    }
    for (int k = 0; k < Nf; ++k) {
      double d;
      if (k == 0) d = g->zf[1] - g->zf[0];
      else if (k == Nv) d = g->zf[Nv] - g->zf[Nv - 1];
      else d = (g->zf[k] + g->zf[k + 1]) / 2 - (g->zf[k - 1] + g->zf[k]) / 2;
      dzf[k] = (FT)d;
      rf[k] = (FT)((p->radius + g->zf[k]) / p->radius);
    }
    topo = g->t_zc != nullptr;
    if (topo) {
      const size_t P = npt(), F = nfac();
      auto cp = [](std::vector<FT> &d, const double *s, size_t n) { d.assign(s, s + n); };
      cp(tzc, g->t_zc, P); cp(tzf, g->t_zf, F); cp(tJc, g->t_Jc, P); cp(tJf, g->t_Jf, F);
      cp(tguc, g->t_guc, 6 * P); cp(tguf, g->t_guf, 6 * F); cp(tgdc, g->t_gdc, 6 * P);
      cp(tf3c, g->t_f3c, P); cp(tf12f, g->t_f12f, 2 * F); cp(tEcc, g->t_Ecc, 9 * P); cp(tEcn, g->t_Ecn, 9 * P);
    }
    goff.assign(g->dss_off, g->dss_off + g->ngroups + 1);
    gcopy.assign(g->dss_copy, g->dss_copy + goff.back());
    gw.assign(g->dss_w, g->dss_w + goff.back());
    tableau();
    alloc_pre();
  }
};

struct Handle {
  int ft;
  Oracle<double> *d = nullptr;
  Oracle<float> *f = nullptr;
};

}  // namespace

#define DISPATCH(h, CALL)                         \
  do {                                            \
    if ((h)->ft == 8) { auto &o = *(h)->d; CALL; } \
    else { auto &o = *(h)->f; CALL; }             \
  } while (0)

extern "C" {

void *oracle_create(const OracleGeom *g, const OracleParams *p, int ft_bytes) {
  Handle *h = new Handle();
  h->ft = ft_bytes;
  if (ft_bytes == 8) { h->d = new Oracle<double>(); h->d->init(g, p); }
  else { h->f = new Oracle<float>(); h->f->init(g, p); }
  return h;
}
void oracle_destroy(void *hh) {
  Handle *h = (Handle *)hh;
  delete h->d; delete h->f; delete h;
}
void oracle_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int oracle_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
// All state pointers are FT arrays in the C-ABI layout; FT = ft_bytes of the handle.
void oracle_set_precomputed(void *hh, void *Yc, void *Yf) {
  Handle *h = (Handle *)hh;
  DISPATCH(h, (o.set_precomputed((decltype(o.R) *)Yc, (decltype(o.R) *)Yf)));
}
// The precomputed pressure at Y (centres, [Nh][16][Nv] in the oracle's precision).
void oracle_pressure(void *hh, void *Yc, void *Yf, void *p_out) {
  Handle *h = (Handle *)hh;
  DISPATCH(h, (o.set_precomputed((decltype(o.R) *)Yc, (decltype(o.R) *)Yf),
               std::copy(o.pre.p.begin(), o.pre.p.end(), (decltype(o.R) *)p_out)));
}
void oracle_remaining_tendency(void *hh, void *Tc, void *Tf, void *Yc, void *Yf) {
  Handle *h = (Handle *)hh;
  DISPATCH(h, (o.set_precomputed((decltype(o.R) *)Yc, (decltype(o.R) *)Yf),
               o.remaining_tendency((decltype(o.R) *)Tc, (decltype(o.R) *)Tf, (decltype(o.R) *)Yc, (decltype(o.R) *)Yf)));
}
void oracle_implicit_tendency(void *hh, void *Tc, void *Tf, void *Yc, void *Yf) {
  Handle *h = (Handle *)hh;
  DISPATCH(h, (o.set_precomputed((decltype(o.R) *)Yc, (decltype(o.R) *)Yf),
               o.implicit_tendency((decltype(o.R) *)Tc, (decltype(o.R) *)Tf, (decltype(o.R) *)Yc, (decltype(o.R) *)Yf)));
}
void oracle_update_jacobian(void *hh, void *Yc, void *Yf, double dtg) {
  Handle *h = (Handle *)hh;
  DISPATCH(h, (o.set_precomputed((decltype(o.R) *)Yc, (decltype(o.R) *)Yf),
               o.update_jacobian((decltype(o.R) *)Yc, (decltype(o.R) *)Yf, (decltype(o.R))dtg)));
}
void oracle_ldiv(void *hh, void *Xc, void *Xf, void *Rc, void *Rf) {
  Handle *h = (Handle *)hh;
  DISPATCH(h, (o.ldiv((decltype(o.R) *)Xc, (decltype(o.R) *)Xf, (const decltype(o.R) *)Rc, (const decltype(o.R) *)Rf)));
}
void oracle_correct_implicit(void *hh, void *Tc, void *Tf, void *Yc, void *Yf) {
  Handle *h = (Handle *)hh;
  DISPATCH(h, (o.set_precomputed((decltype(o.R) *)Yc, (decltype(o.R) *)Yf),
               o.correct_implicit((decltype(o.R) *)Tc, (decltype(o.R) *)Tf, (decltype(o.R) *)Yc, (decltype(o.R) *)Yf)));
}
void oracle_jac_apply(void *hh, void *Oc, void *Of, void *Vc, void *Vf) {
  Handle *h = (Handle *)hh;
  DISPATCH(h, (o.jac_apply((decltype(o.R) *)Oc, (decltype(o.R) *)Of, (const decltype(o.R) *)Vc, (const decltype(o.R) *)Vf)));
}
void oracle_dss(void *hh, void *Yc, void *Yf) {
  Handle *h = (Handle *)hh;
  DISPATCH(h, (o.dss((decltype(o.R) *)Yc, (decltype(o.R) *)Yf)));
}
// The DSS of a centre block whose comps 1-3 are one covariant 3-vector (the Laplacians).
void oracle_dss_c123(void *hh, void *C) {
  Handle *h = (Handle *)hh;
  DISPATCH(h, (o.dss_center((decltype(o.R) *)C, o.Nv, true)));
}
void oracle_step(void *hh, void *Yc, void *Yf, double dt, int nsteps) {
  Handle *h = (Handle *)hh;
  for (int s = 0; s < nsteps; ++s) DISPATCH(h, (o.step((decltype(o.R) *)Yc, (decltype(o.R) *)Yf, dt)));
}
void oracle_laplacians(void *hh, void *X, void *O) {
  Handle *h = (Handle *)hh;
  DISPATCH(h, (o.laplacians((const decltype(o.R) *)X, (decltype(o.R) *)O)));
}
// The saturation adjustment of n points (moist handles): T, q_liq, q_ice from (rho, e_int, q_tot).
void oracle_sat_adjust(void *hh, int n, const double *rho, const double *eint, const double *q, double *T,
                       double *ql, double *qi) {
  Handle *h = (Handle *)hh;
  for (int i = 0; i < n; ++i)
    DISPATCH(h, ({
      using F = decltype(o.R);
      const auto r = o.sat_adjust((F)rho[i], (F)eint[i], (F)q[i]);
      T[i] = r.T; ql[i] = r.ql; qi[i] = r.qi;
    }));
}
void oracle_global_sums(void *hh, void *Yc, double *out) {
  Handle *h = (Handle *)hh;
  DISPATCH(h, (o.global_sums((const decltype(o.R) *)Yc, out)));
}
}
