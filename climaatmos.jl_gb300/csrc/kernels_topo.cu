// Spectral-element slab kernels of the explicit tendency over terrain-following levels.
//
// The same work as k_passA / k_passB (remaining_tendency!: prep_hyperdiffusion_tendency!,
// horizontal_dynamics_tendency!, apply_hyperdiffusion_tendency!,
// explicit_vertical_advection_tendency! and the Rayleigh sponge on u_h) with the metric of
// every point (topo.cuh) in place of the per-level scaling of the surface metric:
//  - the contravariant (u^1, u^2) of the centre velocity C123(u_h) + I^c(C123(u_3)) take
//    g^a3 I^c(u_3), and u^3 on a face takes u_h^3 = ᶠwinterp(rho J, CT3(u_h))
//    (compute_ᶠuₕ³, precomputed_quantities.jl:473-476);
//  - the kinetic energy takes 2 CT3(u_h) I^c(u_3) (compute_kinetic, utilities.jl:194-206);
//  - the geopotential g z, the Rayleigh sponge and the Coriolis f^3 are per point;
//  - every C123 <-> CT123 conversion of the vector Laplacians takes the full 3x3 metric;
//  - u_3 on the bottom and top faces is the impenetrable value -u_h^3 / g^33 (formed here
//    from u_h of the adjacent centre, so the kernels read the filtered state whatever the
//    stored boundary values).
// The vector Laplacian is a covariant 3-vector whose DSS projects to Cartesian components
// with each copy's basis, whose E^3 leans with the level over terrain.  Pass A therefore
// stores (L_s, L_1 - (s_1 / dz) L_3, L_2 - (s_2 / dz) L_3, L_3): the horizontal part of the
// Cartesian vector in covariant form, which the ordinary DSS averages as a horizontal vector
// (and L_3 as a scalar, dz being the same for every copy), and pass B adds (s_a / dz) L_3
// back on its own copy's slopes; that is the Cartesian DSS of the 3-vector.
#include "se_ops.cuh"
#include "topo.cuh"

namespace gb {

namespace {

using namespace se;

constexpr int TS_THREADS = 256;
constexpr int TS_LEVELS = TS_THREADS / 4;
// Resident CTAs per SM the terrain slab kernels are compiled for: two in FP32 (the 128-register
// cap: pass A fits it, 94 -> 80 us at h_elem 30, z_elem 63; pass B spills ten words with its
// centre phase ordered hyperdiffusion first), one in FP64.
template <class FT>
struct TsMinBlocks {
  static constexpr int value = sizeof(FT) == 4 ? 2 : 1;
};

template <class FT>
struct TopoALayout {
  size_t y[2], f[2], g[2], t[2], out, w, gf, bar, total;
  __host__ __device__ TopoALayout(int Nv, int nbuf) {
    const int Nf = Nv + 1;
    size_t o = 0;
    for (int b = 0; b < 2; ++b) {
      if (b < nbuf) {
        y[b] = o; o += align16(sizeof(FT) * 64 * Nv);
        f[b] = o; o += align16(sizeof(FT) * 16 * Nf);
        g[b] = o; o += align16(sizeof(FT) * HG_N * 16);
        t[b] = o; o += align16(sizeof(FT) * TG_N * 16);
      } else {
        y[b] = y[0]; f[b] = f[0]; g[b] = g[0]; t[b] = t[0];
      }
    }
    out = o; o += align16(sizeof(FT) * 64 * Nv);
    w = o; o += align16(sizeof(FT) * 2 * 16);     // GLL weights W, 1/W
    gf = o; o += align16(sizeof(FT) * 16 * Nf);   // g^33 of every face [Nf][16]
    bar = o; o += 16;
    total = o;
  }
};

// Level-major scratch rows of the terrain pass B ((f Nv + v) 16 + n).
enum TopoBScratch { TB_C1 = 0, TB_C2, TB_K, TB_RJ, TB_L4, TB_Q1, TB_Q2, TB_CT3, TB_N };

template <class FT>
struct TopoBLayout {
  size_t y[2], f[2], g[2], t[2], lap[2], s, x1, x2, w, gf, bar, total;
  __host__ __device__ TopoBLayout(int Nv, int nbuf) {
    const int Nf = Nv + 1;
    size_t o = 0;
    for (int b = 0; b < 2; ++b) {
      if (b < nbuf) {
        y[b] = o; o += align16(sizeof(FT) * 64 * Nv);
        f[b] = o; o += align16(sizeof(FT) * 16 * Nf);
        g[b] = o; o += align16(sizeof(FT) * HG_N * 16);
        t[b] = o; o += align16(sizeof(FT) * TG_N * 16);
        lap[b] = o; o += align16(sizeof(FT) * 64 * Nv);
      } else {
        y[b] = y[0]; f[b] = f[0]; g[b] = g[0]; t[b] = t[0]; lap[b] = lap[0];
      }
    }
    s = o; o += align16(sizeof(FT) * TB_N * 16 * Nv);
    x1 = o; o += align16(sizeof(FT) * 16 * Nf);
    x2 = o; o += align16(sizeof(FT) * 16 * Nf);
    w = o; o += align16(sizeof(FT) * 2 * 16);
    gf = o; o += align16(sizeof(FT) * 16 * Nf);   // g^33 of every face [Nf][16]
    bar = o; o += 16;
    total = o;
  }
};

// Row helpers of the terrain kernels: the arithmetic over the row's four nodes goes through the
// vector helpers (two nodes per packed instruction in FP32).
template <class FT>
__device__ __forceinline__ void vbc(FT c, FT (&o)[4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i) o[i] = c;
}
template <class FT>
__device__ __forceinline__ void vrcp(const FT (&a)[4], FT (&o)[4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i) o[i] = grcp(a[i]);
}
// thermo() for the row's nodes, each with its own geopotential Phi[i], on the level with the
// reference record rl (FP32: two nodes at a time)
template <class FT>
__device__ __forceinline__ void thermo_row_pt(const DevParams<FT> &P, const FT (&rho)[4], const FT (&rhoe)[4],
                                              const FT (&K)[4], const FT (&Phi)[4], const Lev4<FT> &rl,
                                              ThermoRow<FT> &o) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    Thermo<FT> th;
    thermo(P, rho[i], rhoe[i], K[i], Phi[i], rl, th);
    o.T[i] = th.T; o.p[i] = th.p; o.h[i] = th.h; o.Pi[i] = th.Pi;
    o.thv[i] = th.thv; o.thvr[i] = th.thvr; o.phid[i] = th.phid; o.Tr[i] = th.Tr;
  }
}
__device__ __forceinline__ void thermo_row_pt(const DevParams<float> &P, const float (&rho)[4], const float (&rhoe)[4],
                                              const float (&K)[4], const float (&Phi)[4], const Lev4<float> &rl,
                                              ThermoRow<float> &o) {
  float2 T[2], p[2], h[2], Pi[2], thv[2], thvr[2], phid[2], Tr[2];
  const float2 ip0 = bc2(rl.y), rz = bc2(rl.z);
  thermo_pair(P, lo2(rho), lo2(rhoe), lo2(K), lo2(Phi), ip0, rz, T[0], p[0], h[0], Pi[0], thv[0], thvr[0], phid[0], Tr[0]);
  thermo_pair(P, hi2(rho), hi2(rhoe), hi2(K), hi2(Phi), ip0, rz, T[1], p[1], h[1], Pi[1], thv[1], thvr[1], phid[1], Tr[1]);
  put2(T[0], T[1], o.T); put2(p[0], p[1], o.p); put2(h[0], h[1], o.h); put2(Pi[0], Pi[1], o.Pi);
  put2(thv[0], thv[1], o.thv); put2(thvr[0], thvr[1], o.thvr); put2(phid[0], phid[1], o.phid); put2(Tr[0], Tr[1], o.Tr);
}

// The point terms of the row's nodes on the level with warp record L: z_s b, height z, 1/r, r^2,
// 1/r^2, layer thickness dz, 1/dz and the slopes s_a (tpoint, four nodes).
template <class FT>
struct TPoint4 {
  FT zsb[4], z[4], ir[4], r2[4], ir2[4], dz[4], idz[4], s1[4], s2[4];
};
template <class FT>
__device__ __forceinline__ void tpoint4(const DevParams<FT> &P, const FT (&zs)[4], const FT (&d1)[4], const FT (&d2)[4],
                                        const Lev4<FT> &L, TPoint4<FT> &t) {
  FT a[4], r[4];
  vmuls(zs, L.y, t.zsb);
  vbc(L.x, a);
  vadd(a, t.zsb, t.z);
  vbc(FT(1), a);
  vfmas(t.z, P.iR, a, r);
  vrcp(r, t.ir);
  vmul(r, r, t.r2);
  vmul(t.ir, t.ir, t.ir2);
  vbc(L.z, a);
  vfmas(zs, L.w, a, t.dz);
  vrcp(t.dz, t.idz);
  vmuls(d1, L.y, t.s1);
  vmuls(d2, L.y, t.s2);
}
// the contravariant metric g^ij (tmetric_up, four nodes) from the surface g_s^ab
template <class FT>
__device__ __forceinline__ void tmetric_up4(const TPoint4<FT> &t, const FT (&a0)[4], const FT (&a1)[4],
                                            const FT (&a2)[4], FT (&g11)[4], FT (&g12)[4], FT (&g22)[4],
                                            FT (&g13)[4], FT (&g23)[4], FT *g33) {
  FT h1[4], h2[4], x[4];
  vmul(a0, t.ir2, g11);
  vmul(a1, t.ir2, g12);
  vmul(a2, t.ir2, g22);
  vmul(g12, t.s2, x);
  vfma(g11, t.s1, x, h1);
  vmul(g22, t.s2, x);
  vfma(g12, t.s1, x, h2);
  vmul(h1, t.idz, g13);
  vmuls(g13, FT(-1), g13);
  vmul(h2, t.idz, g23);
  vmuls(g23, FT(-1), g23);
  if (g33) {
    FT one[4], q[4], i2[4], o[4];
    vbc(FT(1), one);
    vfma(t.s1, h1, one, q);
    vfma(t.s2, h2, q, q);
    vmul(t.idz, t.idz, i2);
    vmul(q, i2, o);
#pragma unroll
    for (int i = 0; i < 4; ++i) g33[i] = o[i];
  }
}

// The geometry of the thread's row (4 nodes) at one centre level.
template <class FT>
struct TRow {
  FT J[4], iJ[4], WJ[4], iWJ[4];
  FT u11[4], u12[4], u22[4], u13[4], u23[4];  // g^ij (g^33 of centres is not used)
  FT z[4], zsb[4], ir[4], s1i[4], s2i[4], idz[4];  // height, z_s b, 1 / r, s_a / dz, 1 / dz
};

// The covariant metric g_ij of the row's nodes at the centre level with warp record L (formed
// only where the vector Laplacians' curls take it, so that it is not held across the pass).
template <class FT>
struct TCov {
  FT d11[4], d12[4], d22[4], d13[4], d23[4], d33[4];
};
template <class FT>
__device__ __forceinline__ void trow_cov(const DevParams<FT> &P, const FT *sG, const FT *sT, int j, const Lev4<FT> &L,
                                         TCov<FT> &o) {
  FT b0[4], b1[4], b2[4], zs[4], e1[4], e2[4];
  ld_row(sG + HG_GD0 * NN + NQ * j, b0);
  ld_row(sG + HG_GD1 * NN + NQ * j, b1);
  ld_row(sG + HG_GD2 * NN + NQ * j, b2);
  ld_row(sT + TG_ZS * NN + NQ * j, zs);
  ld_row(sT + TG_D1 * NN + NQ * j, e1);
  ld_row(sT + TG_D2 * NN + NQ * j, e2);
  TPoint4<FT> t;
  tpoint4(P, zs, e1, e2, L, t);
  FT x[4];
  vmul(t.s1, t.s1, x);
  vfma(t.r2, b0, x, o.d11);
  vmul(t.s1, t.s2, x);
  vfma(t.r2, b1, x, o.d12);
  vmul(t.s2, t.s2, x);
  vfma(t.r2, b2, x, o.d22);
  vmul(t.s1, t.dz, o.d13);
  vmul(t.s2, t.dz, o.d23);
  vmul(t.dz, t.dz, o.d33);
}

// Node rows of the element slab: sG the horizontal geometry, sT the terrain, sW = (W, 1/W).
template <class FT>
__device__ __forceinline__ void trow_centre(const DevParams<FT> &P, const FT *sG, const FT *sT, const FT *sW, int j,
                                            const Lev4<FT> &L, TRow<FT> &o) {
  FT Jh[4], a0[4], a1[4], a2[4], zs[4], e1[4], e2[4], W[4];
  ld_row(sG + HG_JH * NN + NQ * j, Jh);
  ld_row(sG + HG_GU0 * NN + NQ * j, a0);
  ld_row(sG + HG_GU1 * NN + NQ * j, a1);
  ld_row(sG + HG_GU2 * NN + NQ * j, a2);
  ld_row(sT + TG_ZS * NN + NQ * j, zs);
  ld_row(sT + TG_D1 * NN + NQ * j, e1);
  ld_row(sT + TG_D2 * NN + NQ * j, e2);
  ld_row(sW + NQ * j, W);
  TPoint4<FT> t;
  tpoint4(P, zs, e1, e2, L, t);
  tmetric_up4(t, a0, a1, a2, o.u11, o.u12, o.u22, o.u13, o.u23, (FT *)nullptr);
  vmul(Jh, t.r2, o.J);
  vmul(o.J, t.dz, o.J);
  vrcp(o.J, o.iJ);
  vmul(W, o.J, o.WJ);
  vrcp(o.WJ, o.iWJ);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    o.z[i] = t.z[i];
    o.zsb[i] = t.zsb[i];
    o.ir[i] = t.ir[i];
    o.idz[i] = t.idz[i];
  }
  vmul(t.s1, t.idz, o.s1i);
  vmul(t.s2, t.idz, o.s2i);
}

// g^33 of the row's nodes on a face with warp record L (and, optionally, J, 1/J, 1/r).
template <class FT>
__device__ __forceinline__ void trow_face(const DevParams<FT> &P, const FT *sG, const FT *sT, int j, const Lev4<FT> &L,
                                          FT (&g33)[4], FT *J = nullptr, FT *iJ = nullptr, FT *ir = nullptr) {
  FT Jh[4], a0[4], a1[4], a2[4], zs[4], e1[4], e2[4];
  ld_row(sG + HG_GU0 * NN + NQ * j, a0);
  ld_row(sG + HG_GU1 * NN + NQ * j, a1);
  ld_row(sG + HG_GU2 * NN + NQ * j, a2);
  ld_row(sT + TG_ZS * NN + NQ * j, zs);
  ld_row(sT + TG_D1 * NN + NQ * j, e1);
  ld_row(sT + TG_D2 * NN + NQ * j, e2);
  if (J) ld_row(sG + HG_JH * NN + NQ * j, Jh);
  TPoint4<FT> t;
  tpoint4(P, zs, e1, e2, L, t);
  FT g11[4], g12[4], g22[4], g13[4], g23[4];
  tmetric_up4(t, a0, a1, a2, g11, g12, g22, g13, g23, g33);
  if (J) {
    FT x[4];
    vmul(Jh, t.r2, x);
    vmul(x, t.dz, x);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      J[i] = x[i];
      iJ[i] = grcp(x[i]);
      ir[i] = t.ir[i];
    }
  }
}

// g^33 of every face of the element into sG33 [Nf][16] (one row per thread and face slot);
// the caller synchronises before the rows are read.
template <class FT>
__device__ __forceinline__ void face_g33_rows(const DevParams<FT> &P, const FT *sG, const FT *sT, FT *sG33, int j,
                                              int vl) {
  for (int k = vl; k < P.Nf; k += TS_LEVELS) {
    FT g33[4];
    trow_face(P, sG, sT, j, P.ltf[k], g33);
    st_row(sG33 + (size_t)k * NN + NQ * j, g33);
  }
}

// C123(wgrad(div u)) fdiv - C123(wcurl(C123(curl u))) of a covariant (c1, c2, c3) with the full
// metric of the row (the oracle's vec_lap over terrain).
template <class FT>
__device__ __forceinline__ void tvec_lap(const DevParams<FT> &P, const Row<FT> &R, const TRow<FT> &G, const FT *sG,
                                         const FT *sT, int j, const Lev4<FT> &L, const FT (&W)[4], const FT (&iW)[4],
                                         const FT (&c1)[4], const FT (&c2)[4], const FT (&c3)[4], FT fdiv,
                                         FT (&o1)[4], FT (&o2)[4], FT (&o3)[4]) {
  FT a[4], b[4], da[4], db[4], w1[4], w2[4], x[4];
  vmul(G.u13, c3, x);
  vfma(G.u12, c2, x, x);
  vfma(G.u11, c1, x, x);
  vmul(G.J, x, a);
  vmul(G.u23, c3, x);
  vfma(G.u22, c2, x, x);
  vfma(G.u12, c1, x, x);
  vmul(G.J, x, b);
  d1(P, a, da);
  d2(R, b, db);
  vadd(da, db, x);
  vmul(x, G.iJ, x);
  vmul(W, x, a);
  t1(P, a, w1);
  t2(R, a, w2);
  FT e1[4], e2[4], e3[4], e4[4];
  d1(P, c2, e1);
  d2(R, c1, e2);
  d2(R, c3, e3);
  d1(P, c3, e4);
  TCov<FT> Gd;
  trow_cov(P, sG, sT, j, L, Gd);
  FT z1[4], z2[4], z3[4];
  {
    FT k1[4], k2[4], k3[4];
    vmul(e3, G.iJ, k1);
    vmul(e4, G.iJ, k2);
    vmuls(k2, FT(-1), k2);
    vsub(e1, e2, k3);
    vmul(k3, G.iJ, k3);
    vmul(Gd.d13, k3, x);
    vfma(Gd.d12, k2, x, x);
    vfma(Gd.d11, k1, x, x);
    vmul(W, x, z1);
    vmul(Gd.d23, k3, x);
    vfma(Gd.d22, k2, x, x);
    vfma(Gd.d12, k1, x, x);
    vmul(W, x, z2);
    vmul(Gd.d33, k3, x);
    vfma(Gd.d23, k2, x, x);
    vfma(Gd.d13, k1, x, x);
    vmul(W, x, z3);
  }
  FT f1[4], f2[4], f3[4], f4[4];
  t1(P, z2, f1);
  t2(R, z1, f2);
  t2(R, z3, f3);
  t1(P, z3, f4);
  FT q1[4], q2[4], q3[4], y[4];
  vmul(f3, G.iWJ, q1);
  vmuls(q1, FT(-1), q1);
  vmul(f4, G.iWJ, q2);
  vsub(f2, f1, q3);
  vmul(q3, G.iWJ, q3);
  // o1 = -fdiv (w1 / W) - (d11 q1 + d12 q2 + d13 q3), o2 alike
  vmul(w1, iW, y);
  vmul(Gd.d13, q3, x);
  vfma(Gd.d12, q2, x, x);
  vfma(Gd.d11, q1, x, x);
  vmuls(x, FT(-1), x);
  vfmas(y, -fdiv, x, o1);
  vmul(w2, iW, y);
  vmul(Gd.d23, q3, x);
  vfma(Gd.d22, q2, x, x);
  vfma(Gd.d12, q1, x, x);
  vmuls(x, FT(-1), x);
  vfmas(y, -fdiv, x, o2);
  vmul(Gd.d33, q3, x);
  vfma(Gd.d23, q2, x, x);
  vfma(Gd.d13, q1, x, x);
  vmuls(x, FT(-1), o3);
}

// weak divergence -(1/WJ) (D^T (WJ F1) + ...) with the row's per-node WJ
template <class FT>
__device__ __forceinline__ void twdiv(const DevParams<FT> &P, const Row<FT> &R, const TRow<FT> &G, const FT (&F1)[4],
                                      const FT (&F2)[4], FT (&o)[4]) {
  FT a[4], b[4], ta[4], tb[4];
  vmul(G.WJ, F1, a);
  vmul(G.WJ, F2, b);
  t1(P, a, ta);
  t2(R, b, tb);
  vadd(ta, tb, a);
  vmul(a, G.iWJ, a);
  vmuls(a, FT(-1), o);
}

// The centre state of the row at level v with the filtered face u_3 below and above:
// ct3 = CT3(u_h), ub3 = I^c(u_3), h = CT12(u_h) and K.
template <class FT>
struct TCen {
  FT rho[4], u1[4], u2[4], rhoe[4], ct3[4], ub3[4], h1[4], h2[4], K[4];
};
template <class FT>
__device__ __forceinline__ void tcentre(const DevParams<FT> &P, const FT *sY, const FT *sF, const FT *sG33, int j,
                                        int v, const TRow<FT> &G, TCen<FT> &c) {
  const int Nv = P.Nv, Nf = P.Nf;
  FT ga[4], gb[4], fa[4], fb[4], x[4];
  ld_row(sG33 + (size_t)v * NN + NQ * j, ga);
  ld_row(sG33 + (size_t)(v + 1) * NN + NQ * j, gb);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int q = (NQ * j + i) * Nv + v;
    c.rho[i] = sY[q];
    c.u1[i] = sY[16 * Nv + q];
    c.u2[i] = sY[32 * Nv + q];
    c.rhoe[i] = sY[48 * Nv + q];
  }
  vmul(G.u23, c.u2, x);
  vfma(G.u13, c.u1, x, c.ct3);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int n = NQ * j + i;
    // the impenetrable value on the bottom and top faces (u^3 = 0 there)
    fa[i] = v == 0 ? -gdiv(c.ct3[i], ga[i]) : sF[n * Nf + v];
    fb[i] = v + 1 == Nv ? -gdiv(c.ct3[i], gb[i]) : sF[n * Nf + v + 1];
  }
  vadd(fa, fb, c.ub3);
  vmuls(c.ub3, FT(0.5), c.ub3);
  vmul(G.u12, c.u2, x);
  vfma(G.u11, c.u1, x, c.h1);
  vmul(G.u22, c.u2, x);
  vfma(G.u12, c.u1, x, c.h2);
  // K = (u_1 h1 + u_2 h2 + (fa^2 ga + fb^2 gb) / 2 + 2 ct3 ub3) / 2
  FT kv[4], y[4];
  vmul(fb, gb, y);
  vmul(fb, y, kv);
  vmul(fa, ga, y);
  vfma(fa, y, kv, kv);
  vmul(c.ct3, c.ub3, y);
  vmuls(y, FT(4), y);
  vadd(kv, y, kv);                   // fa^2 ga + fb^2 gb + 4 ct3 ub3
  vmul(c.u2, c.h2, y);
  vfma(c.u1, c.h1, y, y);
  vfmas(kv, FT(0.5), y, y);
  vmuls(y, FT(0.5), c.K);
}

template <class FT>
__global__ void __launch_bounds__(TS_THREADS, TsMinBlocks<FT>::value) k_topo_passA(DevParams<FT> P, int nbuf, const FT *__restrict__ Yc,
                                                             const FT *__restrict__ Yf, FT *__restrict__ Lout) {
  extern __shared__ __align__(128) unsigned char sm[];
  const int Nv = P.Nv, Nf = P.Nf;
  const TopoALayout<FT> Lo(Nv, nbuf);
  auto at = [&](const size_t (&off)[2], int b) { return (FT *)(sm + (b ? off[1] : off[0])); };
  FT *sO = (FT *)(sm + Lo.out), *sW = (FT *)(sm + Lo.w), *sG33 = (FT *)(sm + Lo.gf);
  uint64_t *bar = (uint64_t *)(sm + Lo.bar);
  const uint32_t by = uint32_t(sizeof(FT) * 64 * Nv), bf = uint32_t(sizeof(FT) * 16 * Nf);
  const uint32_t bg = uint32_t(sizeof(FT) * HG_N * 16), bt = uint32_t(sizeof(FT) * TG_N * 16);
  auto issue = [&](int b, int e) {
    uint64_t *bb = b ? &bar[1] : &bar[0];
    mbar_expect_tx(bb, by + bf + bg + bt);
    tma_load(at(Lo.y, b), Yc + (size_t)e * 64 * Nv, by, bb);
    tma_load(at(Lo.f, b), Yf + (size_t)e * 16 * Nf, bf, bb);
    tma_load(at(Lo.g, b), P.hgeo + (size_t)e * HG_N * 16, bg, bb);
    tma_load(at(Lo.t, b), P.tgeo + (size_t)e * TG_N * 16, bt, bb);
  };
  if (threadIdx.x < NN) {
    sW[threadIdx.x] = P.W[threadIdx.x];
    sW[NN + threadIdx.x] = P.iW[threadIdx.x];
  }
  slab_init_bars(bar);
  int e = blockIdx.x;
  if (threadIdx.x == 0 && e < P.Nh) issue(0, e);
  const int j = threadIdx.x & 3, vl = threadIdx.x >> 2, vs = level_slot(vl);
  Row<FT> R;
  R.init(P, j);
  FT W[4], iW[4];
  ld_row(sW + NQ * j, W);
  ld_row(sW + NN + NQ * j, iW);
  for (int it = 0; e < P.Nh; ++it, e += gridDim.x) {
    int b;
    if (!slab_begin(bar, nbuf, it, e, P.Nh, P.status, issue, b)) break;
    const FT *sY = at(Lo.y, b), *sF = at(Lo.f, b), *sG = at(Lo.g, b), *sT = at(Lo.t, b);
    face_g33_rows(P, sG, sT, sG33, j, vl);
    __syncthreads();
    for (int v0 = 0; v0 < Nv; v0 += TS_LEVELS) {
      const int v = min(v0 + vs, Nv - 1);
      const bool act = v0 + vs < Nv;
      TRow<FT> G;
      trow_centre(P, sG, sT, sW, j, P.ltc[v], G);
      TCen<FT> c;
      tcentre(P, sY, sF, sG33, j, v, G, c);
      FT sd[4];
      {
        // s_d - s_d,r = cp_d (T - T_r) + (Phi - Phi_r(Pi)); the level record's deviation is for
        // the flat level's geopotential g zeta, the point is g z_s b higher
        FT Phi[4], t[4], x[4];
        ThermoRow<FT> th;
        vmuls(G.z, P.grav, Phi);
        thermo_row_pt(P, c.rho, c.rhoe, c.K, Phi, P.lr4[v], th);
        vsub(th.T, th.Tr, t);
        vfmas(G.zsb, P.grav, th.phid, x);
        vfmas(t, P.cpd, x, sd);
      }
      FT o1[4], o2[4], o3[4];
      tvec_lap(P, R, G, sG, sT, j, P.ltc[v], W, iW, c.u1, c.u2, c.ub3, FT(1), o1, o2, o3);
      FT g1[4], g2[4], x1[4], x2[4], Ls[4];
      d1(P, sd, g1);
      d2(R, sd, g2);
      {
        FT t[4];
        vmul(G.u12, g2, t);
        vfma(G.u11, g1, t, x1);
        vmul(G.u22, g2, t);
        vfma(G.u12, g1, t, x2);
      }
      twdiv(P, R, G, x1, x2, Ls);
      if (act) {
        FT t[4];
        vmul(G.s1i, o3, t);
        vsub(o1, t, o1);
        vmul(G.s2i, o3, t);
        vsub(o2, t, o2);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = (NQ * j + i) * Nv + v;
          sO[q] = Ls[i];
          sO[16 * Nv + q] = o1[i];
          sO[32 * Nv + q] = o2[i];
          sO[48 * Nv + q] = o3[i];
        }
      }
    }
    fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      tma_store(Lout + (size_t)e * 64 * Nv, sO, by);
      tma_store_commit();
    }
  }
  if (threadIdx.x == 0) tma_store_wait_all();
}

template <class FT>
struct alignas(16) TV16 {
  FT v[16 / sizeof(FT)];
};

// out = U + c_3 T + sum_j c_j T_j over one slab of n values in 16-byte vectors (T in shared
// memory, overwritten; U and the T_j at offset off in global memory): the final combination of
// a stiffly accurate step, as the flat pass B folds it.
template <class FT>
__device__ __forceinline__ void tfin_combine(FT *sT, const FT *U, const FT *const (&Tj)[3], const FinArgs<FT> &F,
                                             size_t off, int n) {
  constexpr int E = 16 / sizeof(FT);
  TV16<FT> *sv = reinterpret_cast<TV16<FT> *>(sT);
  const TV16<FT> *u = reinterpret_cast<const TV16<FT> *>(U + off);
  for (int i = threadIdx.x; i < n / E; i += TS_THREADS) {
    TV16<FT> r = u[i];
    const TV16<FT> t = sv[i];
#pragma unroll
    for (int k = 0; k < E; ++k) r.v[k] += F.c[3] * t.v[k];
#pragma unroll
    for (int q = 0; q < 3; ++q)
      if (Tj[q]) {
        const TV16<FT> a = reinterpret_cast<const TV16<FT> *>(Tj[q] + off)[i];
#pragma unroll
        for (int k = 0; k < E; ++k) r.v[k] += F.c[q] * a.v[k];
      }
    sv[i] = r;
  }
}

// FIN: the slab written is the step's final combination (FinArgs) of the stage state Yc/Yf,
// the earlier tendencies and this tendency (its u_3 on the bottom and top faces is then set by
// the filter after the state's DSS).
template <class FT, bool FIN>
__global__ void __launch_bounds__(TS_THREADS, TsMinBlocks<FT>::value) k_topo_passB(DevParams<FT> P, int nbuf, const FT *__restrict__ Yc,
                                                             const FT *__restrict__ Yf, const FT *__restrict__ Lin,
                                                             FT *__restrict__ Tc, FT *__restrict__ Tf, FinArgs<FT> Fa) {
  extern __shared__ __align__(128) unsigned char sm[];
  const int Nv = P.Nv, Nf = P.Nf;
  const TopoBLayout<FT> Lo(Nv, nbuf);
  auto at = [&](const size_t (&off)[2], int b) { return (FT *)(sm + (b ? off[1] : off[0])); };
  FT *sS = (FT *)(sm + Lo.s), *sX1 = (FT *)(sm + Lo.x1), *sX2 = (FT *)(sm + Lo.x2), *sW = (FT *)(sm + Lo.w);
  FT *sG33 = (FT *)(sm + Lo.gf);
  uint64_t *bar = (uint64_t *)(sm + Lo.bar);
  const uint32_t by = uint32_t(sizeof(FT) * 64 * Nv), bf = uint32_t(sizeof(FT) * 16 * Nf);
  const uint32_t bg = uint32_t(sizeof(FT) * HG_N * 16), bt = uint32_t(sizeof(FT) * TG_N * 16);
  auto issue = [&](int b, int e) {
    uint64_t *bb = b ? &bar[1] : &bar[0];
    mbar_expect_tx(bb, 2 * by + bf + bg + bt);
    tma_load(at(Lo.y, b), Yc + (size_t)e * 64 * Nv, by, bb);
    tma_load(at(Lo.f, b), Yf + (size_t)e * 16 * Nf, bf, bb);
    tma_load(at(Lo.g, b), P.hgeo + (size_t)e * HG_N * 16, bg, bb);
    tma_load(at(Lo.t, b), P.tgeo + (size_t)e * TG_N * 16, bt, bb);
    tma_load(at(Lo.lap, b), Lin + (size_t)e * 64 * Nv, by, bb);
  };
  if (threadIdx.x < NN) {
    sW[threadIdx.x] = P.W[threadIdx.x];
    sW[NN + threadIdx.x] = P.iW[threadIdx.x];
  }
  slab_init_bars(bar);
  int e = blockIdx.x;
  if (threadIdx.x == 0 && e < P.Nh) issue(0, e);
  const int j = threadIdx.x & 3, vl = threadIdx.x >> 2, vs = level_slot(vl);
  auto row = [&](FT *base, int f, int v) { return base + ((size_t)f * Nv + v) * NN + NQ * j; };
  Row<FT> R;
  R.init(P, j);
  for (int it = 0; e < P.Nh; ++it, e += gridDim.x) {
    int b;
    if (!slab_begin(bar, nbuf, it, e, P.Nh, P.status, issue, b)) break;
    FT *sY = at(Lo.y, b), *sF = at(Lo.f, b);
    const FT *sG = at(Lo.g, b), *sT = at(Lo.t, b), *sL = at(Lo.lap, b);
    FT W[4], iW[4];
    ld_row(sW + NQ * j, W);
    ld_row(sW + NN + NQ * j, iW);
    if (FIN && threadIdx.x == 0) {
      // the final combination's other operands, into L2 while the tendency is computed
      bulk_prefetch_l2(Yc + (size_t)e * 64 * Nv, by);
      bulk_prefetch_l2(Yf + (size_t)e * 16 * Nf, bf);
      for (int q = 0; q < 3; ++q)
        if (Fa.te_c[q]) {
          bulk_prefetch_l2(Fa.te_c[q] + (size_t)e * 64 * Nv, by);
          bulk_prefetch_l2(Fa.te_f[q] + (size_t)e * 16 * Nf, bf);
        }
    }
    face_g33_rows(P, sG, sT, sG33, j, vl);
    __syncthreads();
    // ---- P1: centre levels, ordered so that each group of intermediates dies before the
    // next is formed: the hyperdiffusion of u (the largest) first, then the state's diagnostics
    for (int v0 = 0; v0 < Nv; v0 += TS_LEVELS) {
      const int v = min(v0 + vs, Nv - 1);
      const bool act = v0 + vs < Nv;
      TRow<FT> G;
      trow_centre(P, sG, sT, sW, j, P.ltc[v], G);
      // hyperdiffusion of u: the Laplacian's covariant 3-vector back on this copy's slopes
      FT Q1[4], Q2[4];
      {
        FT L1[4], L2[4], L3[4], o1[4], o2[4], o3[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = (NQ * j + i) * Nv + v;
          L3[i] = sL[48 * Nv + q];
          L1[i] = sL[16 * Nv + q];
          L2[i] = sL[32 * Nv + q];
        }
        vfma(G.s1i, L3, L1, L1);
        vfma(G.s2i, L3, L2, L2);
        tvec_lap(P, R, G, sG, sT, j, P.ltc[v], W, iW, L1, L2, L3, P.div_damp, o1, o2, o3);
        vmuls(o1, -P.nu_v, Q1);
        vmuls(o2, -P.nu_v, Q2);
        if (act) st_row(row(sS, TB_L4, v), o3);
      }
      TCen<FT> c;
      tcentre(P, sY, sF, sG33, j, v, G, c);
      // rho e_tot: -nu_s wdiv(rho grad L_s)
      FT Trhoe[4];
      {
        FT Ls[4], g1[4], g2[4], x1[4], x2[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) Ls[i] = sL[(NQ * j + i) * Nv + v];
        d1(P, Ls, g1);
        d2(R, Ls, g2);
        vcontract(G.u11, G.u12, g1, g2, c.rho, x1);
        vcontract(G.u12, G.u22, g1, g2, c.rho, x2);
        twdiv(P, R, G, x1, x2, Trhoe);
        vmuls(Trhoe, -P.nu_s, Trhoe);
      }
      FT h[4], Pi[4], thp[4], gg[4], c1[4], c2[4];
      {
        FT Phi[4], t[4];
        ThermoRow<FT> th;
        vmuls(G.z, P.grav, Phi);
        thermo_row_pt(P, c.rho, c.rhoe, c.K, Phi, P.lr4[v], th);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          h[i] = th.h[i];
          Pi[i] = th.Pi[i];
        }
        vsub(th.thv, th.thvr, thp);
        // K + Phi - Phi_r(Pi) + (cp_d / 2) th' Pi: one gradient for grad(K + Phi - Phi_r) and
        // the (cp_d / 2) grad(th' Pi) of the Exner-split pressure gradient
        vfmas(G.zsb, P.grav, th.phid, t);
        vadd(c.K, t, gg);
        vmul(thp, Pi, t);
        vfmas(t, P.cpd * FT(0.5), gg, gg);
        vfma(G.u13, c.ub3, c.h1, c1);
        vfma(G.u23, c.ub3, c.h2, c2);
      }
      // vorticity w^3 = wcurl(u_h), Coriolis f^3, (f^3 + w^3) x CT12(u) -> C12, the sponge
      {
        FT a[4], bb[4], ta[4], tb[4], f3[4], fh1[4], fh2[4];
        vmul(W, c.u2, a);
        vmul(W, c.u1, bb);
        t1(P, a, ta);
        t2(R, bb, tb);
        ld_row(sG + HG_F3 * NN + NQ * j, f3);
        ld_row(sG + HG_FH1 * NN + NQ * j, fh1);
        ld_row(sG + HG_FH2 * NN + NQ * j, fh2);
        // om = (tb - ta) / (W J); f^3 = f3 / dz - (s1 fh1 + s2 fh2) / (r dz); a3J = J (f^3 + om)
        FT om[4], fc[4], x[4], a3J[4], damp[4];
        vsub(tb, ta, om);
        vmul(om, G.iWJ, om);
        vmul(G.s2i, fh2, x);
        vfma(G.s1i, fh1, x, x);
        vmul(x, G.ir, x);
        vmul(f3, G.idz, fc);
        vsub(fc, x, fc);
        vadd(fc, om, x);
        vmul(G.J, x, a3J);
#pragma unroll
        for (int i = 0; i < 4; ++i) damp[i] = tsponge(P, G.z[i], P.spg_auh);
        // Q1 += a3J c2 - damp u1, Q2 += -a3J c1 - damp u2
        vmul(damp, c.u1, x);
        vsub(Q1, x, Q1);
        vfma(a3J, c2, Q1, Q1);
        vmul(damp, c.u2, x);
        vsub(Q2, x, Q2);
        vmul(a3J, c1, x);
        vsub(Q2, x, Q2);
      }
      // rho: -wdiv(rho u); rho e_tot: -split_div(rho u, h)
      FT dm[4];
      {
        FT F1[4], F2[4], G1[4], G2[4], dmh[4], ha[4], hb[4], x[4];
        vmul(c.rho, c1, F1);
        vmul(c.rho, c2, F2);
        vmul(F1, h, G1);
        vmul(F2, h, G2);
        twdiv(P, R, G, F1, F2, dm);
        twdiv(P, R, G, G1, G2, dmh);
        d1(P, h, ha);
        d2(R, h, hb);
        // T_rhoe -= (wdiv(F h) + h wdiv(F) + F . grad h) / 2
        vmul(F2, hb, x);
        vfma(F1, ha, x, x);
        vfma(h, dm, x, x);
        vadd(dmh, x, x);
        vfmas(x, FT(-0.5), Trhoe, Trhoe);
      }
      // u_h: -[grad(K + Phi - Phi_r) + cp_d (th' grad Pi + grad(th' Pi) - Pi grad th') / 2]
      {
        FT a1[4], a2[4], b1[4], b2[4], f1[4], f2[4];
        d1(P, gg, a1);
        d2(R, gg, a2);
        d1(P, Pi, b1);
        d2(R, Pi, b2);
        d1(P, thp, f1);
        d2(R, thp, f2);
        // Q -= a + (cp_d / 2) (th' b - Pi f)
        FT t[4], x[4];
        vmul(Pi, f1, t);
        vmuls(t, FT(-1), t);
        vfma(thp, b1, t, t);
        vfmas(t, P.cpd * FT(0.5), a1, x);
        vsub(Q1, x, Q1);
        vmul(Pi, f2, t);
        vmuls(t, FT(-1), t);
        vfma(thp, b2, t, t);
        vfmas(t, P.cpd * FT(0.5), a2, x);
        vsub(Q2, x, Q2);
      }
      if (act) {
        FT rJ[4];
        vmul(c.rho, G.J, rJ);
        st_row(row(sS, TB_C1, v), c1);
        st_row(row(sS, TB_C2, v), c2);
        st_row(row(sS, TB_K, v), c.K);
        st_row(row(sS, TB_RJ, v), rJ);
        st_row(row(sS, TB_Q1, v), Q1);
        st_row(row(sS, TB_Q2, v), Q2);
        st_row(row(sS, TB_CT3, v), c.ct3);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = (NQ * j + i) * Nv + v;
          sY[q] = -dm[i];        // the tendency over the (read) state entries
          sY[48 * Nv + q] = Trhoe[i];
        }
      }
    }
    __syncthreads();
    // ---- P2: faces (f^12 + w^12, cross products, the u_3 tendency)
    for (int k0 = 0; k0 < Nf; k0 += TS_LEVELS) {
      const int k = min(k0 + vl, Nf - 1);
      const bool act = k0 + vl < Nf;
      const bool inner = k > 0 && k < Nv;
      const int va = k > 0 ? k - 1 : 0, vb = k < Nv ? k : Nv - 1;
      FT g33[4], g33r[4], Jf[4], iJf[4], irf[4];
      trow_face(P, sG, sT, j, P.ltf[k], g33r, Jf, iJf, irf);
      ld_row(sG33 + (size_t)k * NN + NQ * j, g33);
      FT C1a[4], C1b[4], C2a[4], C2b[4], Ka[4], Kb[4], Ra[4], Rb[4], La[4], Lb[4], CTa[4], CTb[4];
      ld_row(row(sS, TB_C1, va), C1a);
      ld_row(row(sS, TB_C1, vb), C1b);
      ld_row(row(sS, TB_C2, va), C2a);
      ld_row(row(sS, TB_C2, vb), C2b);
      ld_row(row(sS, TB_K, va), Ka);
      ld_row(row(sS, TB_K, vb), Kb);
      ld_row(row(sS, TB_RJ, va), Ra);
      ld_row(row(sS, TB_RJ, vb), Rb);
      ld_row(row(sS, TB_L4, va), La);
      ld_row(row(sS, TB_L4, vb), Lb);
      ld_row(row(sS, TB_CT3, va), CTa);
      ld_row(row(sS, TB_CT3, vb), CTb);
      FT u3[4], Wu[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        u3[i] = inner ? sF[(NQ * j + i) * Nf + k] : -gdiv(CTa[i], g33[i]);
        Wu[i] = W[i] * u3[i];
      }
      FT ta[4], tb[4];
      t2(R, Wu, tb);
      t1(P, Wu, ta);
      if (act) {
        FT fh1[4], fh2[4];
        ld_row(sG + HG_FH1 * NN + NQ * j, fh1);
        ld_row(sG + HG_FH2 * NN + NQ * j, fh2);
        FT T3[4], X1[4], X2[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int n = NQ * j + i;
          const FT iWJf = iW[i] * iJf[i];
          FT cv1 = 0, cv2 = 0, gK = 0, cc1, cc2, l4, rJ, uh3;
          if (inner) {
            const int qa = n * Nv + va, qb = n * Nv + vb;
            cv1 = (sY[32 * Nv + qa] - sY[32 * Nv + qb]) * iJf[i];   // -(d u_2 / d xi^3) / J_f
            cv2 = (sY[16 * Nv + qb] - sY[16 * Nv + qa]) * iJf[i];   // (d u_1 / d xi^3) / J_f
            cc1 = (C1a[i] + C1b[i]) / FT(2);
            cc2 = (C2a[i] + C2b[i]) / FT(2);
            gK = Kb[i] - Ka[i];
            const FT iRab = grcp(Ra[i] + Rb[i]);
            l4 = (Ra[i] * La[i] + Rb[i] * Lb[i]) * iRab;
            uh3 = (Ra[i] * CTa[i] + Rb[i] * CTb[i]) * iRab;
            rJ = (Ra[i] + Rb[i]) / FT(2);
          } else {
            cc1 = C1a[i];
            cc2 = C2a[i];
            l4 = La[i];
            uh3 = CTa[i];
            rJ = Ra[i];
          }
          const FT fo1 = fh1[i] * irf[i] + cv1 - tb[i] * iWJf;
          const FT fo2 = fh2[i] * irf[i] + cv2 + ta[i] * iWJf;
          const FT b3 = rJ * (uh3 + g33[i] * u3[i]);
          T3[i] = -P.nu_v * l4 - (Jf[i] * (fo1 * cc2 - fo2 * cc1) + gK);
          X1[i] = Jf[i] * (fo2 * b3);
          X2[i] = -(Jf[i] * (fo1 * b3));
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) sF[(NQ * j + i) * Nf + k] = T3[i];
        st_row(sX1 + (size_t)k * NN + NQ * j, X1);
        st_row(sX2 + (size_t)k * NN + NQ * j, X2);
      }
    }
    __syncthreads();
    // ---- P3: centre u_h part of the face cross products
    for (int v0 = 0; v0 < Nv; v0 += TS_LEVELS) {
      const int v = v0 + vs;
      if (v < Nv) {
        FT Xa1[4], Xb1[4], Xa2[4], Xb2[4], rJ[4], Q1[4], Q2[4];
        ld_row(sX1 + (size_t)v * NN + NQ * j, Xa1);
        ld_row(sX1 + (size_t)(v + 1) * NN + NQ * j, Xb1);
        ld_row(sX2 + (size_t)v * NN + NQ * j, Xa2);
        ld_row(sX2 + (size_t)(v + 1) * NN + NQ * j, Xb2);
        ld_row(row(sS, TB_RJ, v), rJ);
        ld_row(row(sS, TB_Q1, v), Q1);
        ld_row(row(sS, TB_Q2, v), Q2);
        FT irJ[4], t1v[4], t2v[4];
        vrcp(rJ, irJ);
        vadd(Xa1, Xb1, t1v);
        vmul(t1v, irJ, t1v);
        vfmas(t1v, FT(-0.5), Q1, t1v);
        vadd(Xa2, Xb2, t2v);
        vmul(t2v, irJ, t2v);
        vfmas(t2v, FT(-0.5), Q2, t2v);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = (NQ * j + i) * Nv + v;
          sY[16 * Nv + q] = t1v[i];
          sY[32 * Nv + q] = t2v[i];
        }
      }
    }
    if (FIN) {
      __syncthreads();
      tfin_combine<FT>(sY, Yc, Fa.te_c, Fa, (size_t)e * 64 * Nv, 64 * Nv);
      tfin_combine<FT>(sF, Yf, Fa.te_f, Fa, (size_t)e * 16 * Nf, 16 * Nf);
    }
    fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      tma_store(Tc + (size_t)e * 64 * Nv, sY, by);
      tma_store(Tf + (size_t)e * 16 * Nf, sF, bf);
      tma_store_commit();
    }
  }
  if (threadIdx.x == 0) tma_store_wait_all();
}

// The impenetrable filter over terrain (set_velocity_at_surface!, set_velocity_at_top!,
// precomputed_quantities.jl:486-553): u_3 = -u_h^3 / g^33 on the bottom and top faces, with
// u_h^3 the adjacent centre's CT3(u_h) (ᶠwinterp extrapolates at the boundary).  One thread
// per column and boundary.
template <class FT>
__global__ void k_topo_filter(DevParams<FT> P, const FT *__restrict__ Yc, FT *__restrict__ Yf) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int ncols = P.Nh * NN;
  if (t >= 2 * ncols) return;
  const int col = t >> 1, top = t & 1;
  const int e = col >> 4, n = col & 15, Nv = P.Nv, Nf = P.Nf;
  const int v = top ? Nv - 1 : 0, k = top ? Nv : 0;
  const FT *hg = P.hgeo + (size_t)e * HG_N * NN, *tg = P.tgeo + (size_t)e * TG_N * NN;
  const FT zs = tg[TG_ZS * NN + n], d1v = tg[TG_D1 * NN + n], d2v = tg[TG_D2 * NN + n];
  const FT a0 = hg[HG_GU0 * NN + n], a1 = hg[HG_GU1 * NN + n], a2 = hg[HG_GU2 * NN + n];
  const TMetricUp<FT> mc = tmetric_up(tpoint(P, zs, d1v, d2v, P.ltc[v]), a0, a1, a2);
  const TMetricUp<FT> mf = tmetric_up(tpoint(P, zs, d1v, d2v, P.ltf[k]), a0, a1, a2);
  const size_t cb = ((size_t)e * 4 * NN + n) * Nv + v;
  const FT ct3 = mc.g13 * Yc[cb + 16 * Nv] + mc.g23 * Yc[cb + 32 * Nv];
  Yf[(size_t)col * Nf + k] = -ct3 / mf.g33;
}

// DSS of the reduced implicit tendencies (rho, rho e_tot at the centres: [Nh][2][16][Nv]; u_3
// at the faces), the J-weighted average of collocated copies in the fixed copy order.  Over
// terrain the implicit tendency of a column depends on its element's slopes (through u_h^3),
// so collocated copies differ; the stage states the reference assembles from them are DSSed
// (ClimaTimeSteppers' dss! after each stage), which DSSing the tendencies reproduces.
template <class FT>
__global__ void __launch_bounds__(256) k_dss_reduced(DevParams<FT> P, FT *__restrict__ C, FT *__restrict__ F) {
  const int lane = threadIdx.x & 31;
  const int g = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (g >= P.ngroups) return;
  const int Nv = P.Nv, Nf = P.Nf;
  const int o0 = P.goff[g], o1 = P.goff[g + 1];
  for (int k = lane; k < Nf; k += 32) {
    FT s0 = 0, s1 = 0, sf = 0;
    for (int c = o0; c < o1; ++c) {
      const int idx = P.gcopy[c], e = idx >> 4, n = idx & 15;
      const FT w = P.gw[c];
      if (k < Nv) {
        const size_t b = ((size_t)e * 2 * NN + n) * Nv + k;
        s0 = fma(w, C[b], s0);
        s1 = fma(w, C[b + 16 * Nv], s1);
      }
      sf = fma(w, F[(size_t)idx * Nf + k], sf);
    }
    for (int c = o0; c < o1; ++c) {
      const int idx = P.gcopy[c], e = idx >> 4, n = idx & 15;
      if (k < Nv) {
        const size_t b = ((size_t)e * 2 * NN + n) * Nv + k;
        C[b] = s0;
        C[b + 16 * Nv] = s1;
      }
      F[(size_t)idx * Nf + k] = sf;
    }
  }
}

struct TsDev {
  int nsm = 0, optin = 0, per_sm = 0;
};
const TsDev &ts_dev() {
  static const TsDev d = [] {
    TsDev x;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&x.nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&x.optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&x.per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (x.nsm <= 0) x.nsm = 1;
    return x;
  }();
  return d;
}

// Buffering and resident CTAs per SM: at the compiled residency (two in FP32) double-buffered
// slabs if two CTAs' fit the SM (1 KB per CTA reserved), else single-buffered; else one CTA.
template <class FT, class L>
void ts_shape(int Nv, int &nbuf, size_t &smem, int &ctas) {
  const size_t two = L(Nv, 2).total, one = L(Nv, 1).total, per_sm = (size_t)ts_dev().per_sm;
  if (TsMinBlocks<FT>::value >= 2) {
    if (2 * (two + 1024) <= per_sm) { nbuf = 2; smem = two; ctas = 2; return; }
    if (2 * (one + 1024) <= per_sm) { nbuf = 1; smem = one; ctas = 2; return; }
  }
  ctas = 1;
  if (two <= (size_t)ts_dev().optin) { nbuf = 2; smem = two; }
  else { nbuf = 1; smem = one; }
}

}  // namespace

template <class FT>
size_t topo_smem(int Nv) { return TopoBLayout<FT>(Nv, 1).total; }

template <class FT>
cudaError_t configure_topo(int Nv) {
  (void)Nv;
  cudaError_t e = cudaFuncSetAttribute(k_topo_passA<FT>, cudaFuncAttributeMaxDynamicSharedMemorySize, ts_dev().optin);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_topo_passB<FT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, ts_dev().optin);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_topo_passB<FT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, ts_dev().optin);
}

template <class FT>
void launch_topo_passA(const DevParams<FT> &P, const FT *Yc, const FT *Yf, FT *L, cudaStream_t s) {
  int nbuf, ctas;
  size_t smem;
  ts_shape<FT, TopoALayout<FT>>(P.Nv, nbuf, smem, ctas);
  const int grid = min(P.Nh, ts_dev().nsm * ctas);
  k_topo_passA<FT><<<grid, TS_THREADS, smem, s>>>(P, nbuf, Yc, Yf, L);
}
template <class FT>
void launch_topo_passB(const DevParams<FT> &P, const FT *Yc, const FT *Yf, const FT *L, FT *Tc, FT *Tf, cudaStream_t s,
                       const FinArgs<FT> *fin) {
  int nbuf, ctas;
  size_t smem;
  ts_shape<FT, TopoBLayout<FT>>(P.Nv, nbuf, smem, ctas);
  const int grid = min(P.Nh, ts_dev().nsm * ctas);
  const FinArgs<FT> F = fin ? *fin : FinArgs<FT>{};
  if (fin) k_topo_passB<FT, true><<<grid, TS_THREADS, smem, s>>>(P, nbuf, Yc, Yf, L, Tc, Tf, F);
  else k_topo_passB<FT, false><<<grid, TS_THREADS, smem, s>>>(P, nbuf, Yc, Yf, L, Tc, Tf, F);
}
template <class FT>
void launch_topo_filter(const DevParams<FT> &P, const FT *Yc, FT *Yf, cudaStream_t s) {
  const int n = 2 * P.Nh * NN;
  k_topo_filter<FT><<<(n + 255) / 256, 256, 0, s>>>(P, Yc, Yf);
}
template <class FT>
void launch_dss_reduced(const DevParams<FT> &P, FT *C, FT *F, cudaStream_t s) {
  k_dss_reduced<FT><<<(P.ngroups + 7) / 8, 256, 0, s>>>(P, C, F);
}

#define INST(FT)                                                                                                  \
  template size_t topo_smem<FT>(int);                                                                             \
  template cudaError_t configure_topo<FT>(int);                                                                   \
  template void launch_topo_passA<FT>(const DevParams<FT> &, const FT *, const FT *, FT *, cudaStream_t);         \
  template void launch_topo_passB<FT>(const DevParams<FT> &, const FT *, const FT *, const FT *, FT *, FT *,       \
                                      cudaStream_t, const FinArgs<FT> *);                                         \
  template void launch_topo_filter<FT>(const DevParams<FT> &, const FT *, FT *, cudaStream_t);                    \
  template void launch_dss_reduced<FT>(const DevParams<FT> &, FT *, FT *, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace gb
