// Host-side (FP64) grid generation for the GB300 dry dynamical core.
#pragma once
#include <vector>

#include "gbdycore.h"

namespace gb {

constexpr int NQ = 4;
constexpr int NN = 16;

// Per-node horizontal geometry quantities stored for the kernels ([elem][q][node]).
// HG_S2: sin^2 of the node's latitude (Held-Suarez forcing)
enum HGeo { HG_JH = 0, HG_GU0, HG_GU1, HG_GU2, HG_GD0, HG_GD1, HG_GD2, HG_F3, HG_FH1, HG_FH2, HG_IJH, HG_S2, HG_N };
// Per-level centre quantities ([q][Nv]).
// LC_SPG / LF_SPG: the sponge shape s(z) (beta = alpha s(z)), for the sponge-rate derivative.
// LC_P0, LC_IP0, LC_RB: the level's reference record (reference_level()): the pressure p0 of
// the hydrostatic reference state at the level's geopotential, 1 / p0, and
// cp_d (T_sfc - T_min) / 7 Pi0^7.
enum LevC { LC_Z = 0, LC_R2, LC_DZ, LC_PHI, LC_BETA, LC_IR2, LC_IDZ, LC_SPG, LC_P0, LC_IP0, LC_RB, LC_N };
// Per-level face quantities ([q][Nv+1]).
enum LevF { LF_Z = 0, LF_R2, LF_DZ, LF_RINV, LF_BETA, LF_DPHI, LF_IR2, LF_IDZ, LF_G33, LF_SPG, LF_N };

// Per-node terrain quantities ([elem][q][node], terrain-following levels only): the surface
// elevation z_s and its derivatives along xi^1 and xi^2 in the element (the GLL derivative
// matrix applied to the element's 16 nodal values), padded to four rows.
enum TGeo { TG_ZS = 0, TG_D1, TG_D2, TG_PAD, TG_N };

struct HostGeometry {
  int h = 0, Nh = 0, Nv = 0;
  double R = 0;
  double xg[NQ], wg[NQ], W[NN], D[NQ][NQ];
  std::vector<double> xyz, ecov, econ, Jh, gup, gdn, sinlat, fh0;
  std::vector<double> zf, zc, dzc, dzf, rc, rf;
  std::vector<int> grp_off, grp_copy;
  std::vector<double> grp_w;
  std::vector<double> hgeo;  // [Nh][HG_N][16]
  std::vector<double> levc;  // [LC_N][Nv]
  std::vector<double> levf;  // [LF_N][Nv+1]
  // terrain-following levels: z = zeta + z_s b(zeta) per point.  ltc[v] = {zeta_c, b_c,
  // dzeta_c, db_c} (the centre midway between warped faces: b_c the mean of its faces' b,
  // the thickness dzeta_c + z_s db_c), ltf[k] = {zeta_f, b_f, dzeta_f, db_f} (the face's
  // distance between centres, the adjacent thickness on the boundary faces).
  bool topo = false;
  std::vector<double> tgeo;  // [Nh][TG_N][16]
  std::vector<double> ltc;   // [Nv][4]
  std::vector<double> ltf;   // [Nv+1][4]
};

// The warp factor b(zeta) of the terrain-following levels (gb_config.warp).
double warp_factor(const gb_config &cfg, double zeta);
// The terrain tables (tgeo, ltc, ltf) of a built geometry when cfg.z_surface is given (the
// surface in the caller's element and node order); false, with a message, if the warped
// levels cross.
bool build_terrain_tables(const gb_config &cfg, HostGeometry &g, const char **why);

// Returns false (with a message) on an invalid configuration.
bool validate_config(const gb_config &cfg, const char **why);
void build_geometry(const gb_config &cfg, HostGeometry &g);
// The caller's node (ic, jc) of library node (i, j) in a frame turned by o quarter turns.
void caller_node(int o, int i, int j, int &ic, int &jc);
// gb_match_elements: the caller's element layout from its node positions.
bool match_elements(const gb_config &cfg, const double *xyz, int *elem_map, int *elem_orient, const char **why);

// Face heights z_0 = 0 .. z_{z_elem} = z_max: uniform, or tanh-stretched with the
// first layer dz_bottom (ClimaCore's HyperbolicTangentStretching, grids.jl:356).
std::vector<double> vertical_faces(const gb_config &cfg);
// Rayleigh sponge rate alpha sin^2(pi/2 (z - z_d)/(z_max - z_d)) above z_d (rayleigh_sponge.jl:39-44).
double beta_sponge(double z, double zd, double zmax, double alpha);
// The reference record of a level of geopotential Phi: the Exner value Pi0 at which the
// reference state's geopotential Phi_r(Pi0) = -cp_d (T_min ln Pi0 + (T_sfc - T_min) / 7 (Pi0^7 - 1))
// (src/utils/refstate_thermodynamics.jl:58-166) equals Phi, found by Newton's method in FP64;
// out = {p0 = p_ref Pi0^(1/kappa), 1 / p0, cp_d (T_sfc - T_min) / 7 Pi0^7}.  The kernels form
// Phi - Phi_r(Pi) as a deviation from it, cp_d T_min ln x + out[2] (x^7 - 1) with
// x = Pi / Pi0 = (p / p0)^kappa, so that no two O(1e5) terms cancel in FP32.
void reference_level(const gb_config &cfg, double Phi, double out[3]);

}  // namespace gb
