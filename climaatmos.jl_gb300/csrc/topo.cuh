// Terrain-following geometry of one point, computed where it is used.
//
// Over terrain the height of a point is z = zeta + z_s b(zeta) (the warp of the flat level
// zeta by the surface z_s under the node), its layer thickness dz = dzeta + z_s db, and the
// covariant basis E_a = r e_a + s_a x_hat (a = 1, 2), E_3 = dz x_hat with r = 1 + z / R, e_a
// the surface basis and s_a = dz/dxi^a = b dz_s/dxi^a the slope of the level in the element.
// So the metric of every point follows from a few per-node values (J_h, the surface metric,
// z_s and its two element derivatives) and the level's warp record {zeta, b, dzeta, db}:
//   J     = J_h r^2 dz
//   g^ab  = g_s^ab / r^2,  g^a3 = -g^ab s_b / dz,  g^33 = (1 + s_a g^ab s_b) / dz^2
//   g_ab  = r^2 g_s,ab + s_a s_b,  g_a3 = s_a dz,  g_33 = dz^2
// (the inverse of [[r^2 g_s + s s^T, s dz], [s^T dz, dz^2]]), and the Coriolis components
// f^a = (2 Omega z_hat . e^a) / r and f^3 = (2 Omega sin(lat) - s_a f^a) / dz
// (grad(xi^3) = (x_hat - s_a grad(xi^a)) / dz).  Nothing of this is stored per point.
#pragma once
#include "common.cuh"

namespace gb {

template <class FT>
struct TPoint {
  FT z, zsb, r, ir, r2, ir2, dz, idz, s1, s2;
};

// The point of node (z_s, d1 = dz_s/dxi^1, d2 = dz_s/dxi^2) on the level with warp record L.
template <class FT>
__device__ __forceinline__ TPoint<FT> tpoint(const DevParams<FT> &P, FT zs, FT d1, FT d2, const Lev4<FT> &L) {
  TPoint<FT> o;
  o.zsb = zs * L.y;
  o.z = L.x + o.zsb;
  o.r = FT(1) + o.z * P.iR;
  o.ir = grcp(o.r);
  o.r2 = o.r * o.r;
  o.ir2 = o.ir * o.ir;
  o.dz = L.z + zs * L.w;
  o.idz = grcp(o.dz);
  o.s1 = L.y * d1;
  o.s2 = L.y * d2;
  return o;
}

// The contravariant metric of a point from the surface g_s^ab (gs0, gs1, gs2 = 11, 12, 22).
template <class FT>
struct TMetricUp {
  FT g11, g12, g22, g13, g23, g33;
};
template <class FT>
__device__ __forceinline__ TMetricUp<FT> tmetric_up(const TPoint<FT> &t, FT gs0, FT gs1, FT gs2) {
  TMetricUp<FT> m;
  m.g11 = gs0 * t.ir2;
  m.g12 = gs1 * t.ir2;
  m.g22 = gs2 * t.ir2;
  const FT h1 = m.g11 * t.s1 + m.g12 * t.s2, h2 = m.g12 * t.s1 + m.g22 * t.s2;
  m.g13 = -h1 * t.idz;
  m.g23 = -h2 * t.idz;
  m.g33 = (FT(1) + t.s1 * h1 + t.s2 * h2) * (t.idz * t.idz);
  return m;
}

// Rayleigh sponge rate of a point at height z (rayleigh_sponge.jl:39-44).
template <class FT>
__device__ __forceinline__ FT tsponge(const DevParams<FT> &P, FT z, FT alpha) {
  if (!(alpha != FT(0)) || !(z > P.spg_zd)) return FT(0);
  const FT s = gsin(P.spg_k * (z - P.spg_zd));
  return alpha * s * s;
}

}  // namespace gb
