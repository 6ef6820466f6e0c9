// Host-side grid generation (FP64): equiangular cubed sphere with Nq = 4 GLL
// nodes, deep-atmosphere metric terms, vertical mesh, and the DSS plan.
//
// Restates what SphereGrid (src/simulation/grids.jl:42-89) obtains from
// ClimaCore: EquiangularCubedSphere, nh_poly = 3, DeepSphericalGlobalGeometry
// (horizontal metric scaled by (R + z) / R), and the tanh stretching of
// get_stretching (grids.jl:356).  The DSS plan lists, for every set of
// collocated element nodes, its copies in ascending element*16 + node order
// with J-weights; collocated nodes are found exactly on the integer node
// lattice of the cube (each coordinate in 0..3*h_elem).
//
// The tables are built in the caller's element layout when gb_config gives one
// (elem_map / elem_orient): element e of the caller is library element
// elem_map[e] with its (xi^1, xi^2) frame turned by elem_orient[e] quarter
// turns, so every per-node quantity is stored at the caller's (element, node)
// and expressed on the caller's covariant basis.  The copies of a DSS group
// are kept in the library's order whatever the caller's layout, so the DSS
// sums add the same values in the same order for any element numbering.
#include "geometry.h"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace gb {

namespace {
// Panel frames (normal, t1, t2) with t1 x t2 = normal.
const int PANEL[6][3][3] = {
    {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},  {{0, 1, 0}, {-1, 0, 0}, {0, 0, 1}},
    {{-1, 0, 0}, {0, -1, 0}, {0, 0, 1}}, {{0, -1, 0}, {1, 0, 0}, {0, 0, 1}},
    {{0, 0, 1}, {0, 1, 0}, {-1, 0, 0}}, {{0, 0, -1}, {0, 1, 0}, {1, 0, 0}},
};

void gll4(double *x, double *w, double D[NQ][NQ]) {
  const double s = 1.0 / std::sqrt(5.0);
  const double xs[NQ] = {-1.0, -s, s, 1.0};
  const double ws[NQ] = {1.0 / 6.0, 5.0 / 6.0, 5.0 / 6.0, 1.0 / 6.0};
  double lam[NQ];
  for (int j = 0; j < NQ; ++j) {
    double p = 1.0;
    for (int m = 0; m < NQ; ++m)
      if (m != j) p *= xs[j] - xs[m];
    lam[j] = 1.0 / p;
  }
  for (int i = 0; i < NQ; ++i) {
    x[i] = xs[i];
    w[i] = ws[i];
    double diag = 0;
    for (int k = 0; k < NQ; ++k) {
      if (k == i) continue;
      D[i][k] = (lam[k] / lam[i]) / (xs[i] - xs[k]);
      diag -= D[i][k];
    }
    D[i][i] = diag;
  }
}

}  // namespace

std::vector<double> vertical_faces(const gb_config &c) {
  const int N = c.z_elem;
  std::vector<double> zf(N + 1);
  if (!c.z_stretch) {
    for (int k = 0; k <= N; ++k) zf[k] = c.z_max * k / N;
    return zf;
  }
  // z(zeta) = z_max (1 + tanh(gamma (zeta - 1)) / tanh(gamma)); gamma from z(1/N) = dz_bottom
  const double target = c.dz_bottom / c.z_max;
  auto first = [&](double g) { return 1.0 + std::tanh(g * (1.0 / N - 1.0)) / std::tanh(g); };
  double lo = 1e-8, hi = 50.0;
  for (int it = 0; it < 200; ++it) {
    double mid = 0.5 * (lo + hi);
    if (first(mid) > target) lo = mid; else hi = mid;
  }
  const double g = 0.5 * (lo + hi);
  for (int k = 0; k <= N; ++k) zf[k] = c.z_max * (1.0 + std::tanh(g * ((double)k / N - 1.0)) / std::tanh(g));
  zf[0] = 0.0;
  zf[N] = c.z_max;
  return zf;
}

double beta_sponge(double z, double zd, double zmax, double alpha) {
  if (!(z > zd) || alpha == 0.0) return 0.0;
  double s = std::sin(M_PI * (z - zd) / (zmax - zd) / 2.0);
  return alpha * s * s;
}

void reference_level(const gb_config &c, double Phi, double out[3]) {
  const double cp = c.cp_d, tm = c.T_min_ref, dT = c.T_surf_ref - c.T_min_ref, kappa = c.R_d / c.cp_d;
  // Newton's method in x = ln Pi0 on f(x) = Phi_r - Phi = -cp (T_min x + dT / 7 (e^{7x} - 1)) - Phi,
  // which is decreasing and concave: from x = 0 (Phi_r = 0 <= Phi) the iterates decrease
  // monotonically to the root and stay finite (Newton in Pi itself overshoots below 0 for
  // levels near 30 km).
  double x = 0.0;
  for (int it = 0; it < 100; ++it) {
    const double e7 = std::exp(7.0 * x);
    const double f = -cp * (tm * x + dT / 7.0 * (e7 - 1.0)) - Phi;
    const double df = -cp * (tm + dT * e7);
    const double step = f / df;
    x -= step;
    if (std::fabs(step) < 1e-15 * (1.0 + std::fabs(x))) break;
  }
  const double P = std::exp(x);
  const double p0 = c.p_ref * std::pow(P, 1.0 / kappa);
  out[0] = p0;
  out[1] = 1.0 / p0;
  out[2] = cp * dT / 7.0 * std::pow(P, 7.0);
}

void caller_node(int o, int i, int j, int &ic, int &jc) {
  // the caller's (i', j') of library node (i, j) in a frame turned by o quarter turns
  switch (o & 3) {
    case 0: ic = i; jc = j; break;
    case 1: ic = j; jc = 3 - i; break;
    case 2: ic = 3 - i; jc = 3 - j; break;
    default: ic = 3 - j; jc = i; break;
  }
}

bool validate_config(const gb_config &c, const char **why) {
  if (c.h_elem < 1 || c.h_elem > 512) { *why = "h_elem must be in [1, 512]"; return false; }
  if (c.z_elem < 2 || c.z_elem > 127) { *why = "z_elem must be in [2, 127]"; return false; }
  if (c.ft_bytes != 4 && c.ft_bytes != 8) { *why = "ft_bytes must be 4 or 8"; return false; }
  if (!(c.z_max > 0) || (c.z_stretch && !(c.dz_bottom > 0 && c.dz_bottom < c.z_max / c.z_elem))) {
    *why = "invalid vertical mesh (z_max, dz_bottom)";
    return false;
  }
  if (!(c.radius > 0) || !(c.R_d > 0) || !(c.cp_d > c.R_d) || !(c.cv_d > 0) || !(c.p_ref > 0)) {
    *why = "invalid physical constants";
    return false;
  }
  if (c.upwinding != 0 && c.upwinding != 1) { *why = "upwinding must be 0 or 1"; return false; }
  if (c.held_suarez != 0 && c.held_suarez != 1) { *why = "held_suarez must be 0 or 1"; return false; }
  if (c.held_suarez && (!(c.hs_day > 0) || !(c.hs_sigma_b >= 0 && c.hs_sigma_b < 1) || !(c.hs_p_ref_theta > 0) ||
                        !(c.hs_MSLP > 0))) {
    *why = "invalid Held-Suarez parameters";
    return false;
  }
  if (c.test_dycore_consistency != 0 && c.test_dycore_consistency != 1) {
    *why = "test_dycore_consistency must be 0 or 1";
    return false;
  }
  if (c.z_surface) {
    if (c.warp != 0 && c.warp != 1) { *why = "warp must be 0 (linear) or 1 (SLEVE)"; return false; }
    if (c.warp == 1 && !(c.sleve_eta > 0 && c.sleve_eta <= 1 && c.sleve_s > 0)) {
      *why = "SLEVE warp: sleve_eta must be in (0, 1] and sleve_s > 0";
      return false;
    }
    if (c.held_suarez) { *why = "the Held-Suarez forcing is not available over terrain"; return false; }
    const size_t H = (size_t)6 * c.h_elem * c.h_elem * 16;
    double zmx = 0;
    for (size_t q = 0; q < H; ++q) {
      if (!std::isfinite(c.z_surface[q]) || !(c.z_surface[q] > -0.5 * c.z_max)) {
        *why = "z_surface: a surface elevation is not finite or lies below -z_max / 2";
        return false;
      }
      zmx = std::max(zmx, c.z_surface[q]);
    }
    if (c.warp == 1 && !(c.sleve_s * c.z_max > zmx)) {
      *why = "SLEVE warp: sleve_s * z_max must exceed the highest surface (topography.jl:295-297)";
      return false;
    }
  }
  if (c.moist != 0 && c.moist != 1) { *why = "moist must be 0 or 1"; return false; }
  if (c.moist) {
    if (c.z_surface) { *why = "moist 0M is not available over terrain"; return false; }
    if (c.held_suarez) { *why = "the Held-Suarez forcing is a dry configuration (moist = 0)"; return false; }
    if (!(c.R_v > 0) || !(c.cp_v > c.R_v) || !(c.cp_l > 0) || !(c.cp_i > 0) || !(c.LH_v0 > 0) ||
        !(c.LH_s0 > c.LH_v0) || !(c.T_triple > 0) || !(c.press_triple > 0) || !(c.T_freeze > c.T_icenuc) ||
        !(c.T_icenuc > 0) || !(c.pow_icenuc > 0) || c.sa_iters < 1 || c.sa_iters > 100) {
      *why = "invalid moist thermodynamic constants or sa_iters";
      return false;
    }
  }
  if ((c.elem_map == nullptr) != (c.elem_orient == nullptr)) {
    *why = "elem_map and elem_orient must both be given or both be NULL";
    return false;
  }
  if (c.elem_map) {
    const int Nh = 6 * c.h_elem * c.h_elem;
    std::vector<char> seen(Nh, 0);
    for (int e = 0; e < Nh; ++e) {
      const int m = c.elem_map[e], o = c.elem_orient[e];
      if (m < 0 || m >= Nh || seen[m]) { *why = "elem_map is not a permutation of the elements"; return false; }
      if (o < 0 || o > 3) { *why = "elem_orient entries must be in 0..3"; return false; }
      seen[m] = 1;
    }
  }
  return true;
}

void build_geometry(const gb_config &c, HostGeometry &g) {
  const int h = c.h_elem, Nh = 6 * h * h, Nv = c.z_elem, Nf = Nv + 1;
  const double R = c.radius;
  g.h = h; g.Nh = Nh; g.Nv = Nv; g.R = R;
  gll4(g.xg, g.wg, g.D);
  for (int n = 0; n < NN; ++n) g.W[n] = g.wg[n % NQ] * g.wg[n / NQ];
  const size_t H = (size_t)Nh * NN;
  g.xyz.assign(H * 3, 0); g.ecov.assign(H * 6, 0); g.econ.assign(H * 6, 0);
  g.Jh.assign(H, 0); g.gup.assign(H * 3, 0); g.gdn.assign(H * 3, 0);
  g.sinlat.assign(H, 0); g.fh0.assign(H * 2, 0);
  const double dal = (M_PI / 2.0) / h;
  std::vector<long long> key(H);
  std::vector<int> libidx(H);  // library element*16 + node of each stored (caller) node
  // the caller's element and frame of each library element
  std::vector<int> slot(Nh), orient(Nh, 0);
  for (int e = 0; e < Nh; ++e) slot[e] = e;
  if (c.elem_map)
    for (int e = 0; e < Nh; ++e) {
      slot[c.elem_map[e]] = e;
      orient[c.elem_map[e]] = c.elem_orient[e];
    }
  const int M = 3 * h;
  for (int p = 0; p < 6; ++p)
    for (int ey = 0; ey < h; ++ey)
      for (int ex = 0; ex < h; ++ex) {
        const int el = (p * h + ey) * h + ex;
        const int e = slot[el], o = orient[el];
        for (int j = 0; j < NQ; ++j)
          for (int i = 0; i < NQ; ++i) {
            int ic, jc;
            caller_node(o, i, j, ic, jc);
            const int n = ic + NQ * jc;
            const size_t q = (size_t)e * NN + n;
            libidx[q] = el * NN + i + NQ * j;
            const double al = -M_PI / 4 + (ex + (g.xg[i] + 1) / 2) * dal;
            const double be = -M_PI / 4 + (ey + (g.xg[j] + 1) / 2) * dal;
            const double ta = std::tan(al), tb = std::tan(be);
            double P[3], t1[3], t2[3];
            for (int d = 0; d < 3; ++d) {
              t1[d] = PANEL[p][1][d];
              t2[d] = PANEL[p][2][d];
              P[d] = PANEL[p][0][d] + ta * t1[d] + tb * t2[d];
            }
            const double r2 = P[0] * P[0] + P[1] * P[1] + P[2] * P[2], rn = std::sqrt(r2);
            for (int d = 0; d < 3; ++d) g.xyz[q * 3 + d] = P[d] / rn;
            // e_k = R (dal/2) d(P/|P|)/dalpha_k with dP/dalpha = sec^2 * t (library frame)
            double el_k[2][3];
            for (int k = 0; k < 2; ++k) {
              const double *tv = k == 0 ? t1 : t2;
              const double tt = k == 0 ? ta : tb;
              double dP[3], pd = 0;
              for (int d = 0; d < 3; ++d) { dP[d] = (1.0 + tt * tt) * tv[d]; pd += P[d] * dP[d]; }
              for (int d = 0; d < 3; ++d) el_k[k][d] = R * (dal / 2.0) * (dP[d] / rn - P[d] * pd / (rn * r2));
            }
            // the caller's basis: its frame turned by o quarter turns against the library's
            // (o = 1: e'_1 = e_2, e'_2 = -e_1; o = 2: -e_1, -e_2; o = 3: -e_2, e_1)
            for (int d = 0; d < 3; ++d) {
              double a = el_k[0][d], b = el_k[1][d];
              switch (o) {
                case 1: { const double t = a; a = b; b = -t; break; }
                case 2: a = -a; b = -b; break;
                case 3: { const double t = a; a = -b; b = t; break; }
                default: break;
              }
              g.ecov[q * 6 + d] = a;
              g.ecov[q * 6 + 3 + d] = b;
            }
            const double *e1 = &g.ecov[q * 6], *e2 = &g.ecov[q * 6 + 3];
            const double g11 = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
            const double g12 = e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2];
            const double g22 = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
            const double det = g11 * g22 - g12 * g12;
            g.Jh[q] = std::sqrt(det);
            g.gdn[q * 3 + 0] = g11; g.gdn[q * 3 + 1] = g12; g.gdn[q * 3 + 2] = g22;
            const double u11 = g22 / det, u12 = -g12 / det, u22 = g11 / det;
            g.gup[q * 3 + 0] = u11; g.gup[q * 3 + 1] = u12; g.gup[q * 3 + 2] = u22;
            for (int d = 0; d < 3; ++d) {
              g.econ[q * 6 + d] = u11 * e1[d] + u12 * e2[d];
              g.econ[q * 6 + 3 + d] = u12 * e1[d] + u22 * e2[d];
            }
            const double X = g.xyz[q * 3], Y = g.xyz[q * 3 + 1], Z = g.xyz[q * 3 + 2];
            g.sinlat[q] = Z;
            const double coslat = std::sqrt(std::max(X * X + Y * Y, 0.0));
            const double lon = std::atan2(Y, X);
            const double north[3] = {-Z * std::cos(lon), -Z * std::sin(lon), coslat};
            // covariant components of 2 Omega cos(lat) north, raised with g^ij
            double fc[2];
            for (int k = 0; k < 2; ++k) {
              const double *ek = &g.ecov[q * 6 + k * 3];
              fc[k] = 2.0 * c.omega * coslat * (ek[0] * north[0] + ek[1] * north[1] + ek[2] * north[2]);
            }
            g.fh0[q * 2 + 0] = u11 * fc[0] + u12 * fc[1];
            g.fh0[q * 2 + 1] = u12 * fc[0] + u22 * fc[1];
            // integer lattice point of this node on the cube [0, M]^3
            const int a = 3 * ex + i, b = 3 * ey + j;
            int L[3];
            for (int d = 0; d < 3; ++d) {
              if (PANEL[p][0][d]) L[d] = PANEL[p][0][d] > 0 ? M : 0;
              else if (PANEL[p][1][d]) L[d] = PANEL[p][1][d] > 0 ? a : M - a;
              else L[d] = PANEL[p][2][d] > 0 ? b : M - b;
            }
            key[q] = ((long long)L[0] * (M + 1) + L[1]) * (M + 1) + L[2];
          }
      }
  // DSS groups: copies sharing a lattice point, each in the library's node order,
  // the groups ordered by their first copy in that order
  std::vector<int> order(H);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return key[x] < key[y]; });
  std::vector<std::vector<int>> groups;
  auto lib_less = [&](int x, int y) { return libidx[x] < libidx[y]; };
  for (size_t s = 0; s < H;) {
    size_t t = s;
    while (t < H && key[order[t]] == key[order[s]]) ++t;
    if (t - s > 1) {
      std::vector<int> gset(order.begin() + s, order.begin() + t);
      std::sort(gset.begin(), gset.end(), lib_less);
      groups.push_back(gset);
    }
    s = t;
  }
  std::sort(groups.begin(), groups.end(),
            [&](const std::vector<int> &x, const std::vector<int> &y) { return libidx[x[0]] < libidx[y[0]]; });
  g.grp_off.assign(1, 0);
  g.grp_copy.clear();
  g.grp_w.clear();
  for (auto &gs : groups) {
    double s = 0;
    for (int idx : gs) s += g.Jh[idx];
    for (int idx : gs) {
      g.grp_copy.push_back(idx);
      g.grp_w.push_back(g.Jh[idx] / s);
    }
    g.grp_off.push_back((int)g.grp_copy.size());
  }
  // vertical mesh
  g.zf = vertical_faces(c);
  g.zc.resize(Nv); g.dzc.resize(Nv); g.rc.resize(Nv); g.dzf.resize(Nf); g.rf.resize(Nf);
  for (int v = 0; v < Nv; ++v) {
    g.zc[v] = (g.zf[v] + g.zf[v + 1]) / 2;
    g.dzc[v] = g.zf[v + 1] - g.zf[v];
    g.rc[v] = (R + g.zc[v]) / R;
  }
  for (int k = 0; k < Nf; ++k) {
    if (k == 0) g.dzf[k] = g.dzc[0];
    else if (k == Nv) g.dzf[k] = g.dzc[Nv - 1];
    else g.dzf[k] = g.zc[k] - g.zc[k - 1];
    g.rf[k] = (R + g.zf[k]) / R;
  }
  // kernel-side arrays
  g.hgeo.assign((size_t)Nh * HG_N * NN, 0);
  for (int e = 0; e < Nh; ++e)
    for (int n = 0; n < NN; ++n) {
      const size_t q = (size_t)e * NN + n;
      double *o = &g.hgeo[(size_t)e * HG_N * NN];
      o[HG_JH * NN + n] = g.Jh[q];
      for (int k = 0; k < 3; ++k) {
        o[(HG_GU0 + k) * NN + n] = g.gup[q * 3 + k];
        o[(HG_GD0 + k) * NN + n] = g.gdn[q * 3 + k];
      }
      o[HG_F3 * NN + n] = 2.0 * c.omega * g.sinlat[q];
      o[HG_FH1 * NN + n] = g.fh0[q * 2];
      o[HG_FH2 * NN + n] = g.fh0[q * 2 + 1];
      o[HG_IJH * NN + n] = 1.0 / g.Jh[q];
      o[HG_S2 * NN + n] = g.sinlat[q] * g.sinlat[q];
    }
  g.levc.assign((size_t)LC_N * Nv, 0);
  for (int v = 0; v < Nv; ++v) {
    g.levc[LC_Z * Nv + v] = g.zc[v];
    g.levc[LC_R2 * Nv + v] = g.rc[v] * g.rc[v];
    g.levc[LC_DZ * Nv + v] = g.dzc[v];
    g.levc[LC_PHI * Nv + v] = c.grav * g.zc[v];
    g.levc[LC_BETA * Nv + v] = beta_sponge(g.zc[v], c.sponge_zd, c.z_max, c.alpha_uh);
    g.levc[LC_IR2 * Nv + v] = 1.0 / (g.rc[v] * g.rc[v]);
    g.levc[LC_IDZ * Nv + v] = 1.0 / g.dzc[v];
    g.levc[LC_SPG * Nv + v] = beta_sponge(g.zc[v], c.sponge_zd, c.z_max, 1.0);
    double ref[3];
    reference_level(c, c.grav * g.zc[v], ref);
    g.levc[LC_P0 * Nv + v] = ref[0];
    g.levc[LC_IP0 * Nv + v] = ref[1];
    g.levc[LC_RB * Nv + v] = ref[2];
  }
  g.levf.assign((size_t)LF_N * Nf, 0);
  for (int k = 0; k < Nf; ++k) {
    g.levf[LF_Z * Nf + k] = g.zf[k];
    g.levf[LF_R2 * Nf + k] = g.rf[k] * g.rf[k];
    g.levf[LF_DZ * Nf + k] = g.dzf[k];
    g.levf[LF_RINV * Nf + k] = 1.0 / g.rf[k];
    g.levf[LF_BETA * Nf + k] = beta_sponge(g.zf[k], c.sponge_zd, c.z_max, c.alpha_w);
    g.levf[LF_DPHI * Nf + k] = (k > 0 && k < Nv) ? c.grav * (g.zc[k] - g.zc[k - 1]) : 0.0;
    g.levf[LF_IR2 * Nf + k] = 1.0 / (g.rf[k] * g.rf[k]);
    g.levf[LF_IDZ * Nf + k] = 1.0 / g.dzf[k];
    g.levf[LF_G33 * Nf + k] = 1.0 / (g.dzf[k] * g.dzf[k]);
    g.levf[LF_SPG * Nf + k] = beta_sponge(g.zf[k], c.sponge_zd, c.z_max, 1.0);
  }
}

double warp_factor(const gb_config &c, double zeta) {
  if (c.warp == 0) return 1.0 - zeta / c.z_max;
  const double eta = zeta / c.z_max;
  if (eta > c.sleve_eta) return 0.0;
  return std::sinh((c.sleve_eta - eta) / (c.sleve_s * c.sleve_eta)) / std::sinh(1.0 / c.sleve_s);
}

// Terrain tables of build_geometry (gb_config.z_surface given): the per-node surface and its
// element-local GLL derivatives (in the caller's element frame, where the kernels differentiate),
// and the per-level warp records.  Returns false if a warped layer would have no thickness.
static bool build_terrain(const gb_config &c, HostGeometry &g, const char **why) {
  const int Nh = g.Nh, Nv = g.Nv, Nf = Nv + 1;
  g.topo = true;
  g.tgeo.assign((size_t)Nh * TG_N * NN, 0.0);
  for (int e = 0; e < Nh; ++e) {
    const double *z = c.z_surface + (size_t)e * NN;
    double *o = &g.tgeo[(size_t)e * TG_N * NN];
    for (int j = 0; j < NQ; ++j)
      for (int i = 0; i < NQ; ++i) {
        double a = 0, b = 0;
        for (int k = 0; k < NQ; ++k) {
          a += g.D[i][k] * z[k + NQ * j];
          b += g.D[j][k] * z[i + NQ * k];
        }
        const int n = i + NQ * j;
        o[TG_ZS * NN + n] = z[n];
        o[TG_D1 * NN + n] = a;
        o[TG_D2 * NN + n] = b;
      }
  }
  std::vector<double> bf(Nf), bc(Nv);
  for (int k = 0; k < Nf; ++k) bf[k] = warp_factor(c, g.zf[k]);
  for (int v = 0; v < Nv; ++v) bc[v] = (bf[v] + bf[v + 1]) / 2;
  g.ltc.assign((size_t)4 * Nv, 0.0);
  g.ltf.assign((size_t)4 * Nf, 0.0);
  for (int v = 0; v < Nv; ++v) {
    g.ltc[4 * v + 0] = g.zc[v];
    g.ltc[4 * v + 1] = bc[v];
    g.ltc[4 * v + 2] = g.dzc[v];
    g.ltc[4 * v + 3] = bf[v + 1] - bf[v];
  }
  for (int k = 0; k < Nf; ++k) {
    const int v = k == 0 ? 0 : (k == Nv ? Nv - 1 : -1);
    g.ltf[4 * k + 0] = g.zf[k];
    g.ltf[4 * k + 1] = bf[k];
    g.ltf[4 * k + 2] = g.dzf[k];
    g.ltf[4 * k + 3] = v >= 0 ? g.ltc[4 * v + 3] : bc[k] - bc[k - 1];
  }
  // every warped centre and face keeps a positive thickness
  for (size_t q = 0; q < (size_t)Nh * NN; ++q) {
    const double zs = c.z_surface[q];
    for (int v = 0; v < Nv; ++v)
      if (!(g.ltc[4 * v + 2] + zs * g.ltc[4 * v + 3] > 0)) {
        *why = "z_surface: the terrain-following levels cross (a layer of non-positive thickness)";
        return false;
      }
    for (int k = 0; k < Nf; ++k)
      if (!(g.ltf[4 * k + 2] + zs * g.ltf[4 * k + 3] > 0)) {
        *why = "z_surface: the terrain-following levels cross (a layer of non-positive thickness)";
        return false;
      }
  }
  return true;
}

bool build_terrain_tables(const gb_config &c, HostGeometry &g, const char **why) {
  g.topo = false;
  g.tgeo.clear();
  g.ltc.clear();
  g.ltf.clear();
  return c.z_surface ? build_terrain(c, g, why) : true;
}

bool match_elements(const gb_config &c, const double *xyz, int *elem_map, int *elem_orient, const char **why) {
  gb_config lc = c;
  lc.elem_map = nullptr;
  lc.elem_orient = nullptr;
  HostGeometry g;
  build_geometry(lc, g);
  const int h = c.h_elem, Nh = g.Nh;
  const double dal = (M_PI / 2.0) / h, tol = 1e-9;
  std::vector<char> seen(Nh, 0);
  for (int e = 0; e < Nh; ++e) {
    // unit vectors of the caller's 16 nodes; the element is found from the mean of its
    // four interior nodes, which lies inside one element of one panel
    double u[NN][3], cen[3] = {0, 0, 0};
    for (int n = 0; n < NN; ++n) {
      const double *x = xyz + ((size_t)e * NN + n) * 3;
      const double r = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
      if (!(r > 0)) { *why = "gb_match_elements: a node position is zero or not finite"; return false; }
      for (int d = 0; d < 3; ++d) u[n][d] = x[d] / r;
    }
    for (int n : {5, 6, 9, 10})
      for (int d = 0; d < 3; ++d) cen[d] += u[n][d];
    int p = -1;
    double best = -1;
    for (int q = 0; q < 6; ++q) {
      const double dot = PANEL[q][0][0] * cen[0] + PANEL[q][0][1] * cen[1] + PANEL[q][0][2] * cen[2];
      if (dot > best) { best = dot; p = q; }
    }
    double ta = 0, tb = 0;
    for (int d = 0; d < 3; ++d) {
      ta += PANEL[p][1][d] * cen[d] / best;
      tb += PANEL[p][2][d] * cen[d] / best;
    }
    const int ex = std::min(h - 1, std::max(0, (int)std::floor((std::atan(ta) + M_PI / 4) / dal)));
    const int ey = std::min(h - 1, std::max(0, (int)std::floor((std::atan(tb) + M_PI / 4) / dal)));
    const int el = (p * h + ey) * h + ex;
    int found = -1;
    for (int o = 0; o < 4 && found < 0; ++o) {
      double err = 0;
      for (int j = 0; j < NQ; ++j)
        for (int i = 0; i < NQ; ++i) {
          int ic, jc;
          caller_node(o, i, j, ic, jc);
          const double *a = u[ic + NQ * jc], *b = &g.xyz[((size_t)el * NN + i + NQ * j) * 3];
          for (int d = 0; d < 3; ++d) err = std::max(err, std::fabs(a[d] - b[d]));
        }
      if (err < tol) found = o;
    }
    if (found < 0) {
      *why = "gb_match_elements: an element's nodes are not the GLL nodes of an equiangular cubed-sphere "
             "element at this h_elem in a rotated frame";
      return false;
    }
    if (seen[el]) { *why = "gb_match_elements: two elements are the same element"; return false; }
    seen[el] = 1;
    elem_map[e] = el;
    elem_orient[e] = found;
  }
  return true;
}

}  // namespace gb
