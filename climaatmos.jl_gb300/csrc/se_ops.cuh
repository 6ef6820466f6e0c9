// Element-slab spectral-element operators shared by the forward slab kernels
// and their reverse (adjoint) kernels.
//
// Thread mapping: one thread per (level, row j), holding the four nodes
// n = 4 j + i of that row; xi^1 derivatives are register-local 4x4 products,
// xi^2 derivatives gather the other rows with shuffles inside the level's
// 4-lane group.  The transposes pair up: d1^T = t1 and d2^T = t2.
#pragma once
#include "kernels.cuh"

namespace gb {
namespace se {

// Packed FP32: the pair (a[0], a[1]) or (a[2], a[3]) of a 4-node row, and back.
__device__ __forceinline__ float2 lo2(const float (&a)[4]) { return make_float2(a[0], a[1]); }
__device__ __forceinline__ float2 hi2(const float (&a)[4]) { return make_float2(a[2], a[3]); }
__device__ __forceinline__ void put2(float2 lo, float2 hi, float (&o)[4]) {
  o[0] = lo.x; o[1] = lo.y; o[2] = hi.x; o[3] = hi.y;
}
__device__ __forceinline__ float2 ld2(const float *p) { return *reinterpret_cast<const float2 *>(p); }

// Element-wise arithmetic on a 4-node row: FP64 one operation per node, FP32 two packed
// (f32x2) operations per row.  o may alias an input.
template <class FT>
__device__ __forceinline__ void vmul(const FT (&a)[4], const FT (&b)[4], FT (&o)[4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i) o[i] = a[i] * b[i];
}
__device__ __forceinline__ void vmul(const float (&a)[4], const float (&b)[4], float (&o)[4]) {
  put2(__fmul2_rn(lo2(a), lo2(b)), __fmul2_rn(hi2(a), hi2(b)), o);
}
template <class FT>
__device__ __forceinline__ void vmuls(const FT (&a)[4], FT c, FT (&o)[4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i) o[i] = a[i] * c;
}
__device__ __forceinline__ void vmuls(const float (&a)[4], float c, float (&o)[4]) {
  put2(__fmul2_rn(lo2(a), bc2(c)), __fmul2_rn(hi2(a), bc2(c)), o);
}
// o = a b + c
template <class FT>
__device__ __forceinline__ void vfma(const FT (&a)[4], const FT (&b)[4], const FT (&c)[4], FT (&o)[4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i) o[i] = fma(a[i], b[i], c[i]);
}
__device__ __forceinline__ void vfma(const float (&a)[4], const float (&b)[4], const float (&c)[4], float (&o)[4]) {
  put2(__ffma2_rn(lo2(a), lo2(b), lo2(c)), __ffma2_rn(hi2(a), hi2(b), hi2(c)), o);
}
// o = a s + c
template <class FT>
__device__ __forceinline__ void vfmas(const FT (&a)[4], FT sc, const FT (&c)[4], FT (&o)[4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i) o[i] = fma(a[i], sc, c[i]);
}
__device__ __forceinline__ void vfmas(const float (&a)[4], float sc, const float (&c)[4], float (&o)[4]) {
  put2(__ffma2_rn(lo2(a), bc2(sc), lo2(c)), __ffma2_rn(hi2(a), bc2(sc), hi2(c)), o);
}
template <class FT>
__device__ __forceinline__ void vadd(const FT (&a)[4], const FT (&b)[4], FT (&o)[4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i) o[i] = a[i] + b[i];
}
__device__ __forceinline__ void vadd(const float (&a)[4], const float (&b)[4], float (&o)[4]) {
  put2(__fadd2_rn(lo2(a), lo2(b)), __fadd2_rn(hi2(a), hi2(b)), o);
}
template <class FT>
__device__ __forceinline__ void vsub(const FT (&a)[4], const FT (&b)[4], FT (&o)[4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i) o[i] = a[i] - b[i];
}
__device__ __forceinline__ void vsub(const float (&a)[4], const float (&b)[4], float (&o)[4]) {
  const float2 m = bc2(-1.0f);
  put2(__ffma2_rn(lo2(b), m, lo2(a)), __ffma2_rn(hi2(b), m, hi2(a)), o);
}
// o = (a x + b y) s, the metric contraction of a covariant pair (x, y) with weight s per node
template <class FT>
__device__ __forceinline__ void vcontract(const FT (&a)[4], const FT (&b)[4], const FT (&x)[4], const FT (&y)[4],
                                          const FT (&w)[4], FT (&o)[4]) {
  FT t[4];
  vmul(b, y, t);
  vfma(a, x, t, t);
  vmul(w, t, o);
}

// thermo() for the 4 nodes of a row.  FP64: per node.  FP32: the same operations two nodes
// at a time (packed multiplies and adds; the hardware ln, exp, power and reciprocal per
// node), with the level's geopotential Phi and reference record rl.
template <class FT>
struct ThermoRow {
  FT T[4], p[4], h[4], Pi[4], thv[4], thvr[4], phid[4], Tr[4];
};
template <class FT>
__device__ __forceinline__ void thermo_row(const DevParams<FT> &P, const FT (&rho)[4], const FT (&rhoe)[4],
                                           const FT (&K)[4], FT Phi, const Lev4<FT> &rl, ThermoRow<FT> &o) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    Thermo<FT> th;
    thermo(P, rho[i], rhoe[i], K[i], Phi, rl, th);
    o.T[i] = th.T; o.p[i] = th.p; o.h[i] = th.h; o.Pi[i] = th.Pi;
    o.thv[i] = th.thv; o.thvr[i] = th.thvr; o.phid[i] = th.phid; o.Tr[i] = th.Tr;
  }
}
template <>
__device__ __forceinline__ void thermo_row<float>(const DevParams<float> &P, const float (&rho)[4],
                                                  const float (&rhoe)[4], const float (&K)[4], float Phi,
                                                  const Lev4<float> &rl, ThermoRow<float> &o) {
  float2 T[2], p[2], h[2], Pi[2], thv[2], thvr[2], phid[2], Tr[2];
  const float2 ph = bc2(Phi), ip0 = bc2(rl.y), rz = bc2(rl.z);
  thermo_pair(P, lo2(rho), lo2(rhoe), lo2(K), ph, ip0, rz, T[0], p[0], h[0], Pi[0], thv[0], thvr[0], phid[0], Tr[0]);
  thermo_pair(P, hi2(rho), hi2(rhoe), hi2(K), ph, ip0, rz, T[1], p[1], h[1], Pi[1], thv[1], thvr[1], phid[1], Tr[1]);
  put2(T[0], T[1], o.T); put2(p[0], p[1], o.p); put2(h[0], h[1], o.h); put2(Pi[0], Pi[1], o.Pi);
  put2(thv[0], thv[1], o.thv); put2(thvr[0], thvr[1], o.thvr); put2(phid[0], phid[1], o.phid);
  put2(Tr[0], Tr[1], o.Tr);
}

// thermo_vjp for the 4 nodes of a row with the cotangents of (h, Pi, thv - thvr, Phi_r):
// FP64 per node, FP32 two nodes at a time (thermo_vjp_pair).
template <class FT>
__device__ __forceinline__ void thermo_vjp_row(const DevParams<FT> &P, const FT (&rho)[4], const FT (&rhoe)[4],
                                               const FT (&K)[4], FT Phi, const FT (&hb)[4], const FT (&Pib)[4],
                                               const FT (&thpb)[4], const FT (&phirb)[4], FT (&rb)[4],
                                               FT (&reb)[4], FT (&kb)[4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    ThermoBar<FT> tb{};
    tb.h = hb[i];
    tb.Pi = Pib[i];
    tb.thv = thpb[i];
    tb.thvr = -thpb[i];
    tb.phir = phirb[i];
    thermo_vjp(P, rho[i], rhoe[i], K[i], Phi, tb, rb[i], reb[i], kb[i]);
  }
}
template <>
__device__ __forceinline__ void thermo_vjp_row<float>(const DevParams<float> &P, const float (&rho)[4],
                                                      const float (&rhoe)[4], const float (&K)[4], float Phi,
                                                      const float (&hb)[4], const float (&Pib)[4],
                                                      const float (&thpb)[4], const float (&phirb)[4],
                                                      float (&rb)[4], float (&reb)[4], float (&kb)[4]) {
  float2 r[2], re[2], k[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int i = 2 * h;
    ThermoBar2 tb;
    tb.T = tb.p = tb.Tr = bc2(0.0f);
    tb.h = make_float2(hb[i], hb[i + 1]);
    tb.Pi = make_float2(Pib[i], Pib[i + 1]);
    tb.thv = make_float2(thpb[i], thpb[i + 1]);
    tb.thvr = make_float2(-thpb[i], -thpb[i + 1]);
    tb.phir = make_float2(phirb[i], phirb[i + 1]);
    thermo_vjp_pair(P, make_float2(rho[i], rho[i + 1]), make_float2(rhoe[i], rhoe[i + 1]),
                    make_float2(K[i], K[i + 1]), bc2(Phi), tb, r[h], re[h], k[h]);
  }
  put2(r[0], r[1], rb);
  put2(re[0], re[1], reb);
  put2(k[0], k[1], kb);
}

// Row helper: the thread's row j and its xi^2 derivative coefficients.
template <class FT>
struct Row {
  int j;
  // xi^2 coefficients ordered by partner row j ^ m (m = 0: the thread's own row):
  // dX[m] = D[j][j ^ m], tX[m] = D[j ^ m][j]
  FT dX[NQ], tX[NQ];
  __device__ void init(const DevParams<FT> &P, int jj) {
    j = jj;
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      dX[m] = P.D[j * NQ + (j ^ m)];
      tX[m] = P.D[(j ^ m) * NQ + j];
    }
  }
};

// o[i] = sum_k D[i][k] f[k]   (d/dxi^1, register-local)
template <class FT>
__device__ __forceinline__ void d1(const DevParams<FT> &P, const FT (&f)[4], FT (&o)[4]) {
#pragma unroll
  for (int i = 0; i < NQ; ++i) {
    FT s = 0;
#pragma unroll
    for (int k = 0; k < NQ; ++k) s += P.D[i * NQ + k] * f[k];
    o[i] = s;
  }
}
// FP32: two outputs per packed multiply-add, the same operations in the same order per lane
// (so the same bits as the scalar form)
template <>
__device__ __forceinline__ void d1<float>(const DevParams<float> &P, const float (&f)[4], float (&o)[4]) {
  float2 lo = __fmul2_rn(ld2(&P.DT[0]), bc2(f[0])), hi = __fmul2_rn(ld2(&P.DT[2]), bc2(f[0]));
#pragma unroll
  for (int k = 1; k < NQ; ++k) {
    lo = __ffma2_rn(ld2(&P.DT[k * NQ]), bc2(f[k]), lo);
    hi = __ffma2_rn(ld2(&P.DT[k * NQ + 2]), bc2(f[k]), hi);
  }
  put2(lo, hi, o);
}
// o[i] = sum_k D[k][i] f[k]   (transpose: weak forms)
template <class FT>
__device__ __forceinline__ void t1(const DevParams<FT> &P, const FT (&f)[4], FT (&o)[4]) {
#pragma unroll
  for (int i = 0; i < NQ; ++i) {
    FT s = 0;
#pragma unroll
    for (int k = 0; k < NQ; ++k) s += P.D[k * NQ + i] * f[k];
    o[i] = s;
  }
}
template <>
__device__ __forceinline__ void t1<float>(const DevParams<float> &P, const float (&f)[4], float (&o)[4]) {
  float2 lo = __fmul2_rn(ld2(&P.D[0]), bc2(f[0])), hi = __fmul2_rn(ld2(&P.D[2]), bc2(f[0]));
#pragma unroll
  for (int k = 1; k < NQ; ++k) {
    lo = __ffma2_rn(ld2(&P.D[k * NQ]), bc2(f[k]), lo);
    hi = __ffma2_rn(ld2(&P.D[k * NQ + 2]), bc2(f[k]), hi);
  }
  put2(lo, hi, o);
}
// o[i] = sum_m C[m] f(i, row j ^ m): the thread's own row plus three xor
// partners of its level's 4-lane group (12 shuffles for the 4 outputs)
template <class FT>
__device__ __forceinline__ void across(const FT (&C)[NQ], const FT (&f)[4], FT (&o)[4]) {
#pragma unroll
  for (int i = 0; i < NQ; ++i) {
    FT s = C[0] * f[i];
#pragma unroll
    for (int m = 1; m < NQ; ++m) s += C[m] * __shfl_xor_sync(0xffffffffu, f[i], m, 4);
    o[i] = s;
  }
}
__device__ __forceinline__ void across(const float (&C)[NQ], const float (&f)[4], float (&o)[4]) {
  float g[NQ][4];
#pragma unroll
  for (int m = 1; m < NQ; ++m)
#pragma unroll
    for (int i = 0; i < NQ; ++i) g[m][i] = __shfl_xor_sync(0xffffffffu, f[i], m, 4);
  float2 lo = __fmul2_rn(bc2(C[0]), lo2(f)), hi = __fmul2_rn(bc2(C[0]), hi2(f));
#pragma unroll
  for (int m = 1; m < NQ; ++m) {
    lo = __ffma2_rn(bc2(C[m]), lo2(g[m]), lo);
    hi = __ffma2_rn(bc2(C[m]), hi2(g[m]), hi);
  }
  put2(lo, hi, o);
}
template <class FT>
__device__ __forceinline__ void d2(const Row<FT> &R, const FT (&f)[4], FT (&o)[4]) { across(R.dX, f, o); }
template <class FT>
__device__ __forceinline__ void t2(const Row<FT> &R, const FT (&f)[4], FT (&o)[4]) { across(R.tX, f, o); }

// Level slot of the 4-lane group vl (0..63) of a 256-thread slab sweep: warp
// w takes levels 4 (w mod 4) + 32 (w / 4) + {0..3, 16..19}.  A [node][level]
// slab with an odd level count Nv is then read and written without bank
// conflicts: node rows are 4 Nv = 4 (Nv mod 8) banks apart, and the shifts of
// the four rows carry the two 4-bank chunks onto all eight.
__device__ __forceinline__ int level_slot(int vl) {
  const int w = vl >> 3, g = vl & 7;
  return ((w & 3) << 2) + ((w >> 2) << 5) + (g < 4 ? g : g + 12);
}

// The four nodes of a row as one 16-byte vector access (two in FP64);
// p must be 16-byte aligned.
__device__ __forceinline__ void st_row(float *p, const float (&a)[4]) {
  *reinterpret_cast<float4 *>(p) = make_float4(a[0], a[1], a[2], a[3]);
}
__device__ __forceinline__ void st_row(double *p, const double (&a)[4]) {
  reinterpret_cast<double2 *>(p)[0] = make_double2(a[0], a[1]);
  reinterpret_cast<double2 *>(p)[1] = make_double2(a[2], a[3]);
}
__device__ __forceinline__ void ld_row(const float *p, float (&a)[4]) {
  const float4 t = *reinterpret_cast<const float4 *>(p);
  a[0] = t.x; a[1] = t.y; a[2] = t.z; a[3] = t.w;
}
__device__ __forceinline__ void ld_row(const double *p, double (&a)[4]) {
  const double2 t0 = reinterpret_cast<const double2 *>(p)[0], t1 = reinterpret_cast<const double2 *>(p)[1];
  a[0] = t0.x; a[1] = t0.y; a[2] = t1.x; a[3] = t1.y;
}

// A row load that is issued at every use: the compiler may neither merge it
// with an earlier load of the same row nor hold the value in registers
// between uses (trading a 16-byte shared-memory read for register pressure).
__device__ __forceinline__ void ld_row_v(const float *p, float (&a)[4]) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(p));
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(a[0]), "=f"(a[1]), "=f"(a[2]), "=f"(a[3])
               : "r"(sa));
}
__device__ __forceinline__ void ld_row_v(const double *p, double (&a)[4]) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(p));
  asm volatile("ld.shared.v2.f64 {%0, %1}, [%2];" : "=d"(a[0]), "=d"(a[1]) : "r"(sa));
  asm volatile("ld.shared.v2.f64 {%0, %1}, [%2+16];" : "=d"(a[2]), "=d"(a[3]) : "r"(sa));
}

// Per-node horizontal geometry of the thread's row (loaded once per element
// and held in registers).  The accessors give the operators one interface
// for this and for SlabGeo.
template <class FT>
struct RowGeo {
  FT Jh[4], iJh[4], gu0[4], gu1[4], gu2[4], gd0[4], gd1[4], gd2[4], W[4], iW[4];
  __device__ void load(const FT *sG, const DevParams<FT> &P, int j) {
#pragma unroll
    for (int i = 0; i < NQ; ++i) {
      const int n = NQ * j + i;
      Jh[i] = sG[HG_JH * NN + n];
      iJh[i] = sG[HG_IJH * NN + n];
      gu0[i] = sG[HG_GU0 * NN + n];
      gu1[i] = sG[HG_GU1 * NN + n];
      gu2[i] = sG[HG_GU2 * NN + n];
      gd0[i] = sG[HG_GD0 * NN + n];
      gd1[i] = sG[HG_GD1 * NN + n];
      gd2[i] = sG[HG_GD2 * NN + n];
      W[i] = P.W[n];
      iW[i] = P.iW[n];
    }
  }
  __device__ void gu(FT (&a)[4], FT (&b)[4], FT (&c)[4]) const {
#pragma unroll
    for (int i = 0; i < 4; ++i) { a[i] = gu0[i]; b[i] = gu1[i]; c[i] = gu2[i]; }
  }
  __device__ void gd(FT (&a)[4], FT (&b)[4], FT (&c)[4]) const {
#pragma unroll
    for (int i = 0; i < 4; ++i) { a[i] = gd0[i]; b[i] = gd1[i]; c[i] = gd2[i]; }
  }
  __device__ void w(FT (&a)[4]) const {
#pragma unroll
    for (int i = 0; i < 4; ++i) a[i] = W[i];
  }
  __device__ void iw(FT (&a)[4]) const {
#pragma unroll
    for (int i = 0; i < 4; ++i) a[i] = iW[i];
  }
};

// The same geometry re-read from the element's shared-memory slab at each use
// (one 16-byte row per field; the GLL weights W and 1/W are staged per CTA).
template <class FT>
struct SlabGeo {
  const FT *g;   // element slab + 4 j: field f of the row at g + 16 f
  const FT *wt;  // W[16] then 1/W[16], + 4 j
  __device__ void row(int f, FT (&a)[4]) const { ld_row_v(g + f * NN, a); }
  __device__ void gu(FT (&a)[4], FT (&b)[4], FT (&c)[4]) const {
    row(HG_GU0, a);
    row(HG_GU1, b);
    row(HG_GU2, c);
  }
  __device__ void gd(FT (&a)[4], FT (&b)[4], FT (&c)[4]) const {
    row(HG_GD0, a);
    row(HG_GD1, b);
    row(HG_GD2, c);
  }
  __device__ void w(FT (&a)[4]) const { ld_row_v(wt, a); }
  __device__ void iw(FT (&a)[4]) const { ld_row_v(wt + NN, a); }
};

// Geometry of the row at one level (deep-atmosphere scaling r^2, layer thickness dz).
template <class FT>
struct LevRow {
  FT J[4], iJ[4], WJ[4], iWJ[4];
  FT ir2, r2, G33;
  __device__ void set_rows(const FT (&Jh)[4], const FT (&iJh)[4], const FT (&W)[4], const FT (&iW)[4], FT r2_,
                           FT ir2_, FT dz, FT idz) {
    r2 = r2_;
    ir2 = ir2_;
    G33 = dz * dz;
    vmuls(Jh, r2 * dz, J);
    vmuls(iJh, ir2 * idz, iJ);
    vmul(W, J, WJ);
    vmul(iW, iJ, iWJ);
  }
  __device__ void set(const RowGeo<FT> &g, FT r2_, FT ir2_, FT dz, FT idz) {
    set_rows(g.Jh, g.iJh, g.W, g.iW, r2_, ir2_, dz, idz);
  }
};

// C123(wgrad(div u)) * fdiv - C123(wcurl(C123(curl u))) for covariant (c1, c2, c3)
template <class FT, class G>
__device__ __forceinline__ void vec_lap(const DevParams<FT> &P, const Row<FT> &R, const G &g,
                                        const LevRow<FT> &s, const FT (&c1)[4], const FT (&c2)[4],
                                        const FT (&c3)[4], FT fdiv, FT (&o1)[4], FT (&o2)[4], FT (&o3)[4]) {
  // the metric of the level is the surface metric scaled by r^-2 (g^ij) or r^2 (g_ij): the
  // scale is folded into the per-node weight of each contraction
  FT a[4], b[4], da[4], db[4];
  {
    FT gu0[4], gu1[4], gu2[4], Jr[4];
    g.gu(gu0, gu1, gu2);
    vmuls(s.J, s.ir2, Jr);
    vcontract(gu0, gu1, c1, c2, Jr, a);   // J (g^11 c1 + g^12 c2)
    vcontract(gu1, gu2, c1, c2, Jr, b);   // J (g^12 c1 + g^22 c2)
  }
  d1(P, a, da);
  d2(R, b, db);
  FT wdv[4], w1[4], w2[4];
  {
    FT W[4];
    g.w(W);
    vadd(da, db, wdv);
    vmul(wdv, s.iJ, wdv);
    vmul(W, wdv, wdv);
  }
  t1(P, wdv, w1);
  t2(R, wdv, w2);
  FT e1[4], e2[4], e3[4], e4[4];
  d1(P, c2, e1);
  d2(R, c1, e2);
  d2(R, c3, e3);
  d1(P, c3, e4);
  FT Wz1[4], Wz2[4], Wz3[4];
  {
    FT gd0[4], gd1[4], gd2[4], W[4], WiJ[4], k2[4];
    g.gd(gd0, gd1, gd2);
    g.w(W);
    vmul(W, s.iJ, WiJ);
    vsub(e1, e2, Wz3);
    vmul(Wz3, WiJ, Wz3);
    vmuls(Wz3, s.G33, Wz3);               // W G33 (e1 - e2) / J
    vmuls(WiJ, s.r2, WiJ);
    vmuls(e4, FT(-1), k2);
    vcontract(gd0, gd1, e3, k2, WiJ, Wz1);  // W r^2 (g_11 k1 + g_12 k2), k = (e3, -e4) / J
    vcontract(gd1, gd2, e3, k2, WiJ, Wz2);
  }
  FT f1[4], f2[4], f3[4], f4[4];
  t1(P, Wz2, f1);
  t2(R, Wz1, f2);
  t2(R, Wz3, f3);
  t1(P, Wz3, f4);
  {
    FT gd0[4], gd1[4], gd2[4], iW[4], q1[4], q3[4], r2iWJ[4], t[4];
    g.gd(gd0, gd1, gd2);
    g.iw(iW);
    vsub(f2, f1, q3);
    vmul(q3, s.iWJ, q3);
    vmuls(q3, -s.G33, o3);
    vmuls(s.iWJ, s.r2, r2iWJ);
    vmuls(f3, FT(-1), q1);                  // q = (-f3, f4) / (W J); the contraction takes r^2
    vcontract(gd0, gd1, q1, f4, r2iWJ, t);
    vmul(w1, iW, o1);
    vmuls(o1, -fdiv, o1);
    vsub(o1, t, o1);
    vcontract(gd1, gd2, q1, f4, r2iWJ, t);
    vmul(w2, iW, o2);
    vmuls(o2, -fdiv, o2);
    vsub(o2, t, o2);
  }
}

// The third output of vec_lap alone (it depends on c3 only): the same
// operations in the same order as in vec_lap.
template <class FT, class G>
__device__ __forceinline__ void vec_lap_o3(const DevParams<FT> &P, const Row<FT> &R, const G &g,
                                           const LevRow<FT> &s, const FT (&c3)[4], FT (&o3)[4]) {
  FT e3[4], e4[4], Wz1[4], Wz2[4];
  d2(R, c3, e3);
  d1(P, c3, e4);
  {
    FT gd0[4], gd1[4], gd2[4], W[4], WiJ[4], k2[4];
    g.gd(gd0, gd1, gd2);
    g.w(W);
    vmul(W, s.iJ, WiJ);
    vmuls(WiJ, s.r2, WiJ);
    vmuls(e4, FT(-1), k2);
    vcontract(gd0, gd1, e3, k2, WiJ, Wz1);
    vcontract(gd1, gd2, e3, k2, WiJ, Wz2);
  }
  FT f1[4], f2[4], q3[4];
  t1(P, Wz2, f1);
  t2(R, Wz1, f2);
  vsub(f2, f1, q3);
  vmul(q3, s.iWJ, q3);
  vmuls(q3, -s.G33, o3);
}

// weak divergence -(1/WJ) (D^T (WJ F1) along xi^1 + along xi^2)
template <class FT>
__device__ __forceinline__ void wdiv(const DevParams<FT> &P, const Row<FT> &R, const LevRow<FT> &s,
                                     const FT (&F1)[4], const FT (&F2)[4], FT (&o)[4]) {
  FT a[4], b[4], ta[4], tb[4];
  vmul(s.WJ, F1, a);
  vmul(s.WJ, F2, b);
  t1(P, a, ta);
  t2(R, b, tb);
  vadd(ta, tb, o);
  vmul(o, s.iWJ, o);
  vmuls(o, FT(-1), o);
}

// ---------------------------------------------------------------- reverse (adjoint) forms
// Transpose of vec_lap: given the cotangents (ob1, ob2, ob3) of (o1, o2, o3),
// returns the cotangents (cb1, cb2, cb3) of (c1, c2, c3).  The forward sequence
// run backwards, with d1 <-> t1 and d2 <-> t2.
template <class FT, class G>
__device__ __forceinline__ void vec_lap_t(const DevParams<FT> &P, const Row<FT> &R, const G &g,
                                          const LevRow<FT> &s, const FT (&ob1)[4], const FT (&ob2)[4],
                                          const FT (&ob3)[4], FT fdiv, FT (&cb1)[4], FT (&cb2)[4], FT (&cb3)[4]) {
  // element-wise steps in the packed helpers; the metric scales (r^2, r^-2, G33) are folded
  // into the per-node weights of the contractions, as in vec_lap
  FT f1b[4], f2b[4], f3b[4], f4b[4], w1b[4], w2b[4];
  {
    FT gd0[4], gd1[4], gd2[4], iW[4], wq[4];
    g.gd(gd0, gd1, gd2);
    g.iw(iW);
    vmuls(s.iWJ, s.r2, wq);
    vcontract(gd0, gd1, ob1, ob2, wq, f3b);   // -q1b iWJ, q1b = -r^2 (g_11 ob1 + g_12 ob2)
    vmuls(wq, FT(-1), wq);
    vcontract(gd1, gd2, ob1, ob2, wq, f4b);   // q2b iWJ
    vmuls(s.iWJ, s.G33, wq);
    vmul(ob3, wq, f1b);                       // -q3b iWJ, q3b = -G33 ob3
    vmuls(f1b, FT(-1), f2b);
    vmuls(iW, -fdiv, wq);
    vmul(wq, ob1, w1b);
    vmul(wq, ob2, w2b);
  }
  FT Wz1b[4], Wz2b[4], Wz3b[4], tmp[4];
  d1(P, f1b, Wz2b);
  d2(R, f2b, Wz1b);
  d2(R, f3b, Wz3b);
  d1(P, f4b, tmp);
  FT e1b[4], e2b[4], e3b[4], e4b[4];
  {
    FT gd0[4], gd1[4], gd2[4], W[4], WiJ[4], wk[4];
    g.gd(gd0, gd1, gd2);
    g.w(W);
    vadd(Wz3b, tmp, Wz3b);
    vmul(W, s.iJ, WiJ);
    vmuls(WiJ, s.r2, wk);
    vcontract(gd0, gd1, Wz1b, Wz2b, wk, e3b);  // k1b / J, k1b = W r^2 (g_11 Wz1b + g_12 Wz2b)
    vmuls(wk, FT(-1), wk);
    vcontract(gd1, gd2, Wz1b, Wz2b, wk, e4b);  // -k2b / J
    vmuls(WiJ, s.G33, wk);
    vmul(Wz3b, wk, e1b);                       // k3b / J, k3b = W G33 Wz3b
    vmuls(e1b, FT(-1), e2b);
  }
  t1(P, e1b, cb2);
  t2(R, e2b, cb1);
  t2(R, e3b, cb3);
  t1(P, e4b, tmp);
  FT wdvb[4], t2b[4];
  d1(P, w1b, wdvb);
  d2(R, w2b, t2b);
  FT dab[4];
  {
    FT W[4];
    g.w(W);
    vadd(cb3, tmp, cb3);
    vadd(wdvb, t2b, dab);
    vmul(dab, s.iJ, dab);
    vmul(W, dab, dab);
  }
  FT ab[4], bb[4];
  t1(P, dab, ab);
  t2(R, dab, bb);
  {
    FT gu0[4], gu1[4], gu2[4], Jr[4], t[4];
    g.gu(gu0, gu1, gu2);
    vmuls(s.J, s.ir2, Jr);
    vcontract(gu0, gu1, ab, bb, Jr, t);
    vadd(cb1, t, cb1);
    vcontract(gu1, gu2, ab, bb, Jr, t);
    vadd(cb2, t, cb2);
  }
}

// Transpose of wdiv: cotangents (Fb1, Fb2) of (F1, F2) from the cotangent ob of o.
template <class FT>
__device__ __forceinline__ void wdiv_t(const DevParams<FT> &P, const Row<FT> &R, const LevRow<FT> &s,
                                       const FT (&ob)[4], FT (&Fb1)[4], FT (&Fb2)[4]) {
  FT tb[4];
  vmul(ob, s.iWJ, tb);
  vmuls(tb, FT(-1), tb);
  d1(P, tb, Fb1);
  d2(R, tb, Fb2);
  vmul(Fb1, s.WJ, Fb1);
  vmul(Fb2, s.WJ, Fb2);
}

// Transpose of the gradient (d1 f, d2 f): fb = t1(gb1) + t2(gb2).
template <class FT>
__device__ __forceinline__ void grad_t(const DevParams<FT> &P, const Row<FT> &R, const FT (&gb1)[4],
                                       const FT (&gb2)[4], FT (&fb)[4]) {
  FT a[4];
  t1(P, gb1, fb);
  t2(R, gb2, a);
  vadd(fb, a, fb);
}

// Transpose of the scalar Laplacian Ls = wdiv(g^-1 grad sd) (with the row's g^ij / r^2).
template <class FT, class G>
__device__ __forceinline__ void lap_t(const DevParams<FT> &P, const Row<FT> &R, const G &g,
                                      const LevRow<FT> &s, const FT (&Lb)[4], FT (&sdb)[4]) {
  FT xb1[4], xb2[4], gb1[4], gb2[4];
  wdiv_t(P, R, s, Lb, xb1, xb2);
  {
    FT gu0[4], gu1[4], gu2[4], w[4];
    g.gu(gu0, gu1, gu2);
#pragma unroll
    for (int i = 0; i < 4; ++i) w[i] = s.ir2;
    vcontract(gu0, gu1, xb1, xb2, w, gb1);
    vcontract(gu1, gu2, xb1, xb2, w, gb2);
  }
  grad_t(P, R, gb1, gb2, sdb);
}

}  // namespace se
}  // namespace gb

namespace gb {
namespace se {

// ---------------------------------------------------------------- TMA slab pipeline
// Shared by slab kernels whose output store reads from a load buffer (an
// input slab accumulated in place and stored back).  One mbarrier per buffer.
__device__ __forceinline__ void slab_init_bars(uint64_t *bar) {
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
}

// Start of element iteration `it` (element e): thread 0 first retires the
// reads of the previous element's store (it may read the buffer about to be
// refilled), then prefetches the next element into the other buffer (double
// buffering) or loads this one (single buffering; iteration 0 was issued
// before the loop).  issue(buffer, element) issues the TMA loads.  Returns
// false, in every thread, if the bounded wait for this element gave up.
template <class Issue>
__device__ __forceinline__ bool slab_begin(uint64_t *bar, int nbuf, int it, int e, int Nh, int *status,
                                           const Issue &issue, int &b) {
  b = nbuf == 2 ? (it & 1) : 0;
  if (threadIdx.x == 0) {
    tma_store_wait_read();
    if (nbuf == 2) {
      const int en = e + (int)gridDim.x;
      if (en < Nh) issue(b ^ 1, en);
    } else if (it > 0) {
      issue(0, e);
    }
  }
  const uint32_t parity = nbuf == 2 ? ((it >> 1) & 1) : (it & 1);
  const bool ok = mbar_wait_bounded(b ? &bar[1] : &bar[0], parity, status);
  return __syncthreads_and(ok) != 0;
}

// slab_begin for the kernels whose tendency overwrites their own input slabs and whose first
// phase is long enough to cover the next element's loads: double-buffered, the prefetch of the
// next element (into the buffer holding the previous element's output until that element's
// store has read it) is left to slab_prefetch, called after that first phase, when the store has
// long finished, instead of holding every thread at the start while the store reads.
// Single-buffered, as slab_begin.
template <class Issue>
__device__ __forceinline__ bool slab_begin_deferred(uint64_t *bar, int nbuf, int it, int e, int *status,
                                                    const Issue &issue, int &b) {
  b = nbuf == 2 ? (it & 1) : 0;
  if (threadIdx.x == 0 && nbuf != 2) {
    tma_store_wait_read();
    if (it > 0) issue(0, e);
  }
  const uint32_t parity = nbuf == 2 ? ((it >> 1) & 1) : (it & 1);
  const bool ok = mbar_wait_bounded(b ? &bar[1] : &bar[0], parity, status);
  return __syncthreads_and(ok) != 0;
}
template <class Issue>
__device__ __forceinline__ void slab_prefetch(int nbuf, int b, int e, int Nh, const Issue &issue) {
  if (threadIdx.x == 0 && nbuf == 2) {
    tma_store_wait_read();
    const int en = e + (int)gridDim.x;
    if (en < Nh) issue(b ^ 1, en);
  }
}

// The element's face block (16 nodes x Nf faces) into the padded face slab (face_rows): one TMA
// copy per node row j (4 Nf elements: a multiple of 16 bytes at 16-byte aligned addresses on both
// sides), and back.
template <class FT>
__device__ __forceinline__ void load_faces(FT *sF, const FT *Yf, int e, int Nf, uint64_t *bar) {
  const int FR = face_rows<FT>(Nf);
  const uint32_t b4 = uint32_t(sizeof(FT) * 4 * Nf);
#pragma unroll
  for (int j = 0; j < NQ; ++j) tma_load(sF + (size_t)j * FR, Yf + ((size_t)e * 16 + 4 * j) * Nf, b4, bar);
}
template <class FT>
__device__ __forceinline__ void store_faces(FT *Yf, const FT *sF, int e, int Nf) {
  const int FR = face_rows<FT>(Nf);
  const uint32_t b4 = uint32_t(sizeof(FT) * 4 * Nf);
#pragma unroll
  for (int j = 0; j < NQ; ++j) tma_store(Yf + ((size_t)e * 16 + 4 * j) * Nf, sF + (size_t)j * FR, b4);
}

}  // namespace se
}  // namespace gb
