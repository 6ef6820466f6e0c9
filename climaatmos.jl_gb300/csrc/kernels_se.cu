// Spectral-element slab kernels of the explicit tendency (remaining_tendency!).
//
// One CTA per element: the Nq=4 GLL slab of all levels (state, DSSed
// Laplacians, per-node metric terms) is staged into shared memory by 1-D TMA
// bulk copies, horizontal derivatives apply the 4x4 derivative matrix with
// warp shuffles inside 16-lane groups (one level of one element per group),
// vertical (face/centre) operators read neighbouring levels from shared memory
// in a level-fastest mapping, and the finished slab leaves by a TMA bulk store.
//
// pass A = prep_hyperdiffusion_tendency! (src/prognostic_equations/hyperdiffusion.jl:116-147):
//   L = (grad/curl Laplacian of u_bar, scalar Laplacian of s_d - s_d,r)
// pass B = horizontal_dynamics_tendency! (advection.jl:36-91)
//        + apply_hyperdiffusion_tendency! (hyperdiffusion.jl:247-307)
//        + explicit_vertical_advection_tendency! (advection.jl:205-290, deep branch)
//        + Rayleigh sponge on u_h (remaining_tendency.jl:119-166, rayleigh_sponge.jl:39-44)
#include "kernels.cuh"

namespace gb {

namespace {

constexpr int SE_THREADS = 256;  // 16 nodes x 16 levels per sweep

// Per-lane nodal derivative helper (lane holds node n = i + 4 j of one level).
template <class FT>
struct Nodal {
  int i, j;
  FT dA[NQ], dB[NQ], tA[NQ], tB[NQ];  // D[i][k], D[j][k], D[k][i], D[k][j]
  __device__ void init(const DevParams<FT> &P, int n) {
    i = n & 3;
    j = n >> 2;
#pragma unroll
    for (int k = 0; k < NQ; ++k) {
      dA[k] = P.D[i * NQ + k];
      dB[k] = P.D[j * NQ + k];
      tA[k] = P.D[k * NQ + i];
      tB[k] = P.D[k * NQ + j];
    }
  }
  // d1 f = sum_k D[i][k] f(k,j)
  __device__ FT d1(FT f) const {
    FT s = 0;
#pragma unroll
    for (int k = 0; k < NQ; ++k) s += dA[k] * shfl(f, NQ * j + k, 16);
    return s;
  }
  __device__ FT d2(FT f) const {
    FT s = 0;
#pragma unroll
    for (int k = 0; k < NQ; ++k) s += dB[k] * shfl(f, i + NQ * k, 16);
    return s;
  }
  // t1 f = sum_k D[k][i] f(k,j)
  __device__ FT t1(FT f) const {
    FT s = 0;
#pragma unroll
    for (int k = 0; k < NQ; ++k) s += tA[k] * shfl(f, NQ * j + k, 16);
    return s;
  }
  __device__ FT t2(FT f) const {
    FT s = 0;
#pragma unroll
    for (int k = 0; k < NQ; ++k) s += tB[k] * shfl(f, i + NQ * k, 16);
    return s;
  }
};

template <class FT>
struct NodeGeo {
  FT Jh, iJh, gu0, gu1, gu2, gd0, gd1, gd2, f3, fh1, fh2, W, iW;
  __device__ void load(const FT *sG, const DevParams<FT> &P, int n) {
    Jh = sG[HG_JH * NN + n];
    iJh = sG[HG_IJH * NN + n];
    iW = P.iW[n];
    gu0 = sG[HG_GU0 * NN + n]; gu1 = sG[HG_GU1 * NN + n]; gu2 = sG[HG_GU2 * NN + n];
    gd0 = sG[HG_GD0 * NN + n]; gd1 = sG[HG_GD1 * NN + n]; gd2 = sG[HG_GD2 * NN + n];
    f3 = sG[HG_F3 * NN + n]; fh1 = sG[HG_FH1 * NN + n]; fh2 = sG[HG_FH2 * NN + n];
    W = P.W[n];
  }
};

// Slab geometry at one level: full Jacobian and metric with deep-atmosphere scaling.
template <class FT>
struct LevGeo {
  FT J, iJ, WJ, iWJ, gu0, gu1, gu2, gd0, gd1, gd2, G33;
  __device__ void set(const NodeGeo<FT> &g, FT r2, FT ir2, FT dz, FT idz) {
    J = g.Jh * r2 * dz;
    iJ = g.iJh * ir2 * idz;
    WJ = g.W * J;
    iWJ = g.iW * iJ;
    gu0 = g.gu0 * ir2; gu1 = g.gu1 * ir2; gu2 = g.gu2 * ir2;
    gd0 = g.gd0 * r2; gd1 = g.gd1 * r2; gd2 = g.gd2 * r2;
    G33 = dz * dz;
  }
};

// C123(wgrad(div u)) * fdiv - C123(wcurl(C123(curl u))) for covariant (c1, c2, c3)
template <class FT>
__device__ __forceinline__ void vec_lap(const Nodal<FT> &N, const LevGeo<FT> &s, FT W, FT iW, FT c1, FT c2, FT c3,
                                        FT fdiv, FT &o1, FT &o2, FT &o3) {
  FT F1 = s.gu0 * c1 + s.gu1 * c2, F2 = s.gu1 * c1 + s.gu2 * c2;
  FT dv = (N.d1(s.J * F1) + N.d2(s.J * F2)) * s.iJ;
  FT wdv = W * dv;
  FT w1 = -N.t1(wdv) * iW, w2 = -N.t2(wdv) * iW;
  FT k3 = (N.d1(c2) - N.d2(c1)) * s.iJ;
  FT k1 = N.d2(c3) * s.iJ, k2 = -N.d1(c3) * s.iJ;
  FT z1 = s.gd0 * k1 + s.gd1 * k2, z2 = s.gd1 * k1 + s.gd2 * k2, z3 = s.G33 * k3;
  FT q3 = (-N.t1(W * z2) + N.t2(W * z1)) * s.iWJ;
  FT Wz3 = W * z3;
  FT q1 = -N.t2(Wz3) * s.iWJ, q2 = N.t1(Wz3) * s.iWJ;
  o1 = fdiv * w1 - (s.gd0 * q1 + s.gd1 * q2);
  o2 = fdiv * w2 - (s.gd1 * q1 + s.gd2 * q2);
  o3 = -s.G33 * q3;
}

// Stage one element's slabs into shared memory; returns false on a TMA timeout.
template <class FT>
__device__ bool stage_in(uint64_t *bar, int nbuf, void *const *dst, const void *const *src, const uint32_t *bytes,
                         int *status) {
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t tot = 0;
    for (int b = 0; b < nbuf; ++b) tot += bytes[b];
    mbar_expect_tx(bar, tot);
    for (int b = 0; b < nbuf; ++b) tma_load(dst[b], src[b], bytes[b], bar);
  }
  bool ok = mbar_wait_bounded(bar, 0, status);
  return __syncthreads_and(ok) != 0;
}

template <class FT>
__device__ void stage_out(int nbuf, void *const *dst, const void *const *src, const uint32_t *bytes) {
  fence_proxy_async();
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int b = 0; b < nbuf; ++b) tma_store(dst[b], src[b], bytes[b]);
    tma_store_commit();
    tma_store_wait_all();
  }
  __syncthreads();
}

// u_bar_3 = I^c(u_3) and the face part of K, I^c(u_3 u^3) / ... with the
// impenetrable filter (u_3 = 0 on the boundary faces), level-fastest mapping.
template <class FT>
__device__ void centre_from_faces(const DevParams<FT> &P, const FT *sF, FT *sU3, FT *sKv) {
  const int Nv = P.Nv, Nf = P.Nf;
  for (int idx = threadIdx.x; idx < NN * Nv; idx += blockDim.x) {
    const int n = idx / Nv, v = idx - n * Nv;
    FT a = v == 0 ? FT(0) : sF[n * Nf + v];
    FT b = v + 1 == Nv ? FT(0) : sF[n * Nf + v + 1];
    FT ua = a * P.levf[LF_G33 * Nf + v], ub = b * P.levf[LF_G33 * Nf + v + 1];
    sU3[idx] = (a + b) / FT(2);
    sKv[idx] = (a * ua + b * ub) / FT(2);
  }
}

template <class FT>
__global__ void __launch_bounds__(SE_THREADS) k_passA(DevParams<FT> P, const FT *__restrict__ Yc,
                                                      const FT *__restrict__ Yf, FT *__restrict__ Lout) {
  extern __shared__ __align__(128) unsigned char sm[];
  const int Nv = P.Nv, Nf = P.Nf, e = blockIdx.x;
  const PassALayout<FT> Lo(Nv);
  FT *sY = (FT *)(sm + Lo.y), *sF = (FT *)(sm + Lo.f), *sG = (FT *)(sm + Lo.g);
  FT *sU3 = (FT *)(sm + Lo.u3), *sKv = (FT *)(sm + Lo.kv), *sO = (FT *)(sm + Lo.out);
  uint64_t *bar = (uint64_t *)(sm + Lo.bar);
  {
    void *dst[3] = {sY, sF, sG};
    const void *src[3] = {Yc + (size_t)e * 64 * Nv, Yf + (size_t)e * 16 * Nf, P.hgeo + (size_t)e * HG_N * 16};
    uint32_t by[3] = {uint32_t(sizeof(FT) * 64 * Nv), uint32_t(sizeof(FT) * 16 * Nf), uint32_t(sizeof(FT) * HG_N * 16)};
    if (!stage_in<FT>(bar, 3, dst, src, by, P.status)) return;
  }
  centre_from_faces(P, sF, sU3, sKv);
  __syncthreads();

  const int n = threadIdx.x & 15, vl = threadIdx.x >> 4, nlev = blockDim.x >> 4;
  Nodal<FT> N;
  N.init(P, n);
  NodeGeo<FT> g;
  g.load(sG, P, n);
  for (int v0 = 0; v0 < Nv; v0 += nlev) {
    const int v = min(v0 + vl, Nv - 1);
    const bool act = v0 + vl < Nv;
    LevGeo<FT> s;
    s.set(g, P.levc[LC_R2 * Nv + v], P.levc[LC_IR2 * Nv + v], P.levc[LC_DZ * Nv + v], P.levc[LC_IDZ * Nv + v]);
    const FT Phi = P.levc[LC_PHI * Nv + v];
    const int q = n * Nv + v;
    const FT rho = sY[q], u1 = sY[16 * Nv + q], u2 = sY[32 * Nv + q], rhoe = sY[48 * Nv + q];
    const FT ub3 = sU3[q], kv = sKv[q];
    const FT c1 = s.gu0 * u1 + s.gu1 * u2, c2 = s.gu1 * u1 + s.gu2 * u2;
    const FT K = (u1 * c1 + u2 * c2 + kv) / FT(2);
    Thermo<FT> th;
    thermo(P, rho, rhoe, K, Phi, th);
    FT o1, o2, o3;
    vec_lap(N, s, g.W, g.iW, u1, u2, ub3, FT(1), o1, o2, o3);
    const FT sd = P.cpd * (th.T - P.T0) + Phi - sd_r(P, th.Pi, th.phir);
    const FT g1 = N.d1(sd), g2 = N.d2(sd);
    const FT x1 = s.gu0 * g1 + s.gu1 * g2, x2 = s.gu1 * g1 + s.gu2 * g2;
    const FT Ls = -(N.t1(s.WJ * x1) + N.t2(s.WJ * x2)) * s.iWJ;
    if (act) {
      sO[q] = Ls;
      sO[16 * Nv + q] = o1;
      sO[32 * Nv + q] = o2;
      sO[48 * Nv + q] = o3;
    }
  }
  void *dst[1] = {Lout + (size_t)e * 64 * Nv};
  const void *src[1] = {sO};
  uint32_t by[1] = {uint32_t(sizeof(FT) * 64 * Nv)};
  stage_out<FT>(1, dst, src, by);
}

template <class FT>
__global__ void __launch_bounds__(SE_THREADS) k_passB(DevParams<FT> P, const FT *__restrict__ Yc,
                                                      const FT *__restrict__ Yf, const FT *__restrict__ Lin,
                                                      FT *__restrict__ Tc, FT *__restrict__ Tf) {
  extern __shared__ __align__(128) unsigned char sm[];
  const int Nv = P.Nv, Nf = P.Nf, e = blockIdx.x;
  const PassBLayout<FT> Lo(Nv);
  FT *sY = (FT *)(sm + Lo.y), *sF = (FT *)(sm + Lo.f), *sG = (FT *)(sm + Lo.g), *sL = (FT *)(sm + Lo.lap);
  FT *sU3 = (FT *)(sm + Lo.u3), *sKv = (FT *)(sm + Lo.kv);
  FT *sC1 = (FT *)(sm + Lo.c1), *sC2 = (FT *)(sm + Lo.c2), *sK = (FT *)(sm + Lo.k), *sRJ = (FT *)(sm + Lo.rj);
  FT *sL4 = (FT *)(sm + Lo.l4), *sO = (FT *)(sm + Lo.out), *sOf = (FT *)(sm + Lo.outf);
  FT *sCr1 = sU3, *sCr2 = sKv;          // centre cross terms overwrite u_bar_3 / K_v point by point
  FT *sX1 = sL, *sX2 = sL + 16 * Nf;    // face cross products reuse the Laplacian buffer after P1
  uint64_t *bar = (uint64_t *)(sm + Lo.bar);
  {
    void *dst[4] = {sY, sF, sG, sL};
    const void *src[4] = {Yc + (size_t)e * 64 * Nv, Yf + (size_t)e * 16 * Nf, P.hgeo + (size_t)e * HG_N * 16,
                          Lin + (size_t)e * 64 * Nv};
    uint32_t by[4] = {uint32_t(sizeof(FT) * 64 * Nv), uint32_t(sizeof(FT) * 16 * Nf),
                      uint32_t(sizeof(FT) * HG_N * 16), uint32_t(sizeof(FT) * 64 * Nv)};
    if (!stage_in<FT>(bar, 4, dst, src, by, P.status)) return;
  }
  centre_from_faces(P, sF, sU3, sKv);
  __syncthreads();

  const int n = threadIdx.x & 15, vl = threadIdx.x >> 4, nlev = blockDim.x >> 4;
  Nodal<FT> N;
  N.init(P, n);
  NodeGeo<FT> g;
  g.load(sG, P, n);
  // ---- P1: centre-level horizontal work
  for (int v0 = 0; v0 < Nv; v0 += nlev) {
    const int v = min(v0 + vl, Nv - 1);
    const bool act = v0 + vl < Nv;
    LevGeo<FT> s;
    const FT dz = P.levc[LC_DZ * Nv + v], idz = P.levc[LC_IDZ * Nv + v];
    s.set(g, P.levc[LC_R2 * Nv + v], P.levc[LC_IR2 * Nv + v], dz, idz);
    const FT Phi = P.levc[LC_PHI * Nv + v];
    const int q = n * Nv + v;
    const FT rho = sY[q], u1 = sY[16 * Nv + q], u2 = sY[32 * Nv + q], rhoe = sY[48 * Nv + q];
    const FT kv = sKv[q];
    const FT c1 = s.gu0 * u1 + s.gu1 * u2, c2 = s.gu1 * u1 + s.gu2 * u2;
    const FT K = (u1 * c1 + u2 * c2 + kv) / FT(2);
    Thermo<FT> th;
    thermo(P, rho, rhoe, K, Phi, th);
    const FT h = th.h;
    // rho: -split_div(rho u, 1) = -wdiv(rho u)
    const FT F1 = rho * c1, F2 = rho * c2;
    const FT dm = -(N.t1(s.WJ * F1) + N.t2(s.WJ * F2)) * s.iWJ;
    FT Trho = -dm;
    // rho e_tot: -split_div(rho u, h)
    const FT dmh = -(N.t1(s.WJ * (F1 * h)) + N.t2(s.WJ * (F2 * h))) * s.iWJ;
    const FT ha = N.d1(h), hb = N.d2(h);
    FT Trhoe = -((dmh + h * dm + F1 * ha + F2 * hb) / FT(2));
    // u_h: -[grad(K + Phi - Phi_r) + cp_d (th' grad Pi + grad(th' Pi) - Pi grad th') / 2]
    const FT tmp = K + Phi - th.phir;
    const FT thp = th.thv - th.thvr;
    const FT a1 = N.d1(tmp), a2 = N.d2(tmp);
    const FT b1 = N.d1(th.Pi), b2 = N.d2(th.Pi);
    const FT tp = thp * th.Pi;
    const FT e1 = N.d1(tp), e2 = N.d2(tp);
    const FT f1 = N.d1(thp), f2 = N.d2(thp);
    FT Tu1 = -(a1 + P.cpd * (thp * b1 + e1 - th.Pi * f1) / FT(2));
    FT Tu2 = -(a2 + P.cpd * (thp * b2 + e2 - th.Pi * f2) / FT(2));
    // hyperdiffusion: nu (div_damp C123(wgrad div L) - C123(wcurl C123(curl L)))
    const FT Ls = sL[q], L1 = sL[16 * Nv + q], L2 = sL[32 * Nv + q], L3 = sL[48 * Nv + q];
    FT o1, o2, o3;
    vec_lap(N, s, g.W, g.iW, L1, L2, L3, P.div_damp, o1, o2, o3);
    const FT g1 = N.d1(Ls), g2 = N.d2(Ls);
    const FT x1 = rho * (s.gu0 * g1 + s.gu1 * g2), x2 = rho * (s.gu1 * g1 + s.gu2 * g2);
    const FT hd = -(N.t1(s.WJ * x1) + N.t2(s.WJ * x2)) * s.iWJ;
    Tu1 -= P.nu_v * o1;
    Tu2 -= P.nu_v * o2;
    Trhoe -= P.nu_s * hd;
    // vorticity: w^3 = wcurl(u_h); (f^3 + w^3) x CT12(u) -> C12
    const FT om3 = (-N.t1(g.W * u2) + N.t2(g.W * u1)) * s.iWJ;
    const FT a3 = g.f3 * idz + om3;
    __syncwarp();
    if (act) {
      sO[q] = Trho;
      sO[16 * Nv + q] = Tu1;
      sO[32 * Nv + q] = Tu2;
      sO[48 * Nv + q] = Trhoe;
      sC1[q] = c1;
      sC2[q] = c2;
      sK[q] = K;
      sRJ[q] = rho * s.J;
      sL4[q] = o3;
      sCr1[q] = s.J * (-a3 * c2);
      sCr2[q] = s.J * (a3 * c1);
    }
  }
  __syncthreads();
  // ---- P2: face-level work (f^12 + w^12, cross products, u_3 tendency)
  for (int k0 = 0; k0 < Nf; k0 += nlev) {
    const int k = min(k0 + vl, Nf - 1);
    const bool act = k0 + vl < Nf;
    const bool inner = k > 0 && k < Nv;
    const FT u3 = inner ? sF[n * Nf + k] : FT(0);
    const FT r2 = P.levf[LF_R2 * Nf + k], dzf = P.levf[LF_DZ * Nf + k], rinv = P.levf[LF_RINV * Nf + k];
    const FT Jf = g.Jh * r2 * dzf;
    const FT iJf = g.iJh * P.levf[LF_IR2 * Nf + k] * P.levf[LF_IDZ * Nf + k], iWJf = g.iW * iJf;
    const FT Wu = g.W * u3;
    const FT w1 = -N.t2(Wu) * iWJf, w2 = N.t1(Wu) * iWJf;
    FT cv1 = 0, cv2 = 0, gK = 0, cc1, cc2, l4, rJ;
    const int qa = n * Nv + (k > 0 ? k - 1 : 0), qb = n * Nv + (k < Nv ? k : Nv - 1);
    if (inner) {
      cv1 = -(sY[32 * Nv + qb] - sY[32 * Nv + qa]) * iJf;
      cv2 = (sY[16 * Nv + qb] - sY[16 * Nv + qa]) * iJf;
      cc1 = (sC1[qa] + sC1[qb]) / FT(2);
      cc2 = (sC2[qa] + sC2[qb]) / FT(2);
      gK = sK[qb] - sK[qa];
      const FT wa = sRJ[qa], wb = sRJ[qb];
      l4 = gdiv(wa * sL4[qa] + wb * sL4[qb], wa + wb);
      rJ = (wa + wb) / FT(2);
    } else {
      const int qq = k == 0 ? qb : qa;
      cc1 = sC1[qq];
      cc2 = sC2[qq];
      l4 = sL4[qq];
      rJ = sRJ[qq];
    }
    const FT fo1 = g.fh1 * rinv + cv1 + w1, fo2 = g.fh2 * rinv + cv2 + w2;
    const FT b3 = rJ * (u3 * P.levf[LF_G33 * Nf + k]);
    FT T3 = -(P.nu_v * l4);
    T3 -= Jf * (fo1 * cc2 - fo2 * cc1) + gK;
    if (act) {
      sX1[n * Nf + k] = Jf * (fo2 * b3);
      sX2[n * Nf + k] = Jf * (-fo1 * b3);
      sOf[n * Nf + k] = T3;
    }
  }
  __syncthreads();
  // ---- P3: centre u_h part of the face cross products and the sponge (level-fastest)
  for (int idx = threadIdx.x; idx < NN * Nv; idx += blockDim.x) {
    const int nn = idx / Nv, v = idx - nn * Nv;
    const FT irJ = grcp(sRJ[idx]);
    const FT t1v = (sX1[nn * Nf + v] + sX1[nn * Nf + v + 1]) / FT(2) * irJ + sCr1[idx];
    const FT t2v = (sX2[nn * Nf + v] + sX2[nn * Nf + v + 1]) / FT(2) * irJ + sCr2[idx];
    const FT beta = P.levc[LC_BETA * Nv + v];
    FT a = sO[16 * Nv + idx] - t1v;
    FT b = sO[32 * Nv + idx] - t2v;
    a -= beta * sY[16 * Nv + idx];
    b -= beta * sY[32 * Nv + idx];
    sO[16 * Nv + idx] = a;
    sO[32 * Nv + idx] = b;
  }
  void *dst[2] = {Tc + (size_t)e * 64 * Nv, Tf + (size_t)e * 16 * Nf};
  const void *src[2] = {sO, sOf};
  uint32_t by[2] = {uint32_t(sizeof(FT) * 64 * Nv), uint32_t(sizeof(FT) * 16 * Nf)};
  stage_out<FT>(2, dst, src, by);
}

}  // namespace

template <class FT>
size_t passA_smem(int Nv) { return PassALayout<FT>(Nv).total; }
template <class FT>
size_t passB_smem(int Nv) { return PassBLayout<FT>(Nv).total; }

// Raise the dynamic shared-memory limit of the slab kernels to the device's
// opt-in maximum once (contexts with different level counts may coexist).
template <class FT>
void configure_se(int Nv) {
  (void)Nv;
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncSetAttribute(k_passA<FT>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
  cudaFuncSetAttribute(k_passB<FT>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
}

template <class FT>
void launch_passA(const DevParams<FT> &P, const FT *Yc, const FT *Yf, FT *L, cudaStream_t s) {
  k_passA<FT><<<P.Nh, SE_THREADS, passA_smem<FT>(P.Nv), s>>>(P, Yc, Yf, L);
}
template <class FT>
void launch_passB(const DevParams<FT> &P, const FT *Yc, const FT *Yf, const FT *L, FT *Tc, FT *Tf, cudaStream_t s) {
  k_passB<FT><<<P.Nh, SE_THREADS, passB_smem<FT>(P.Nv), s>>>(P, Yc, Yf, L, Tc, Tf);
}

#define INST(FT)                                                                                             \
  template size_t passA_smem<FT>(int);                                                                       \
  template size_t passB_smem<FT>(int);                                                                       \
  template void configure_se<FT>(int);                                                                       \
  template void launch_passA<FT>(const DevParams<FT> &, const FT *, const FT *, FT *, cudaStream_t);         \
  template void launch_passB<FT>(const DevParams<FT> &, const FT *, const FT *, const FT *, FT *, FT *, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace gb
