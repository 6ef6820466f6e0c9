// Reverse (adjoint) kernels of the spectral-element slab passes.
//
// pass A^T: cotangent of prep_hyperdiffusion_tendency!'s Laplacians
//   (hyperdiffusion.jl:141-147) -> cotangent of the state.
// pass B^T: cotangent of the explicit tendency (horizontal_dynamics_tendency!,
//   advection.jl:36-91; apply_hyperdiffusion_tendency!, hyperdiffusion.jl:273-307;
//   explicit_vertical_advection_tendency!, advection.jl:205-290; Rayleigh
//   sponge on u_h, rayleigh_sponge.jl:39-44) -> cotangents of the state and of
//   the DSSed Laplacians, plus d/dnu and d/d(sponge rate).
//
// Both recompute the forward intermediates of one element from the state
// slab and run the forward sequence backwards (the SE operators transpose as
// d1 <-> t1, d2 <-> t2).  One CTA per element at a time, 256 threads in the
// forward (level, row) mapping; slabs are read with coalesced loads into
// shared memory.  The state cotangent is accumulated (+=) element by element:
// each element owns its nodes, so there are no write conflicts; the DSS
// transpose that precedes/follows is a separate kernel.
#include <algorithm>

#include "se_ops.cuh"

namespace gb {

namespace {

using namespace se;

constexpr int AD_THREADS = 256;
constexpr int AD_LEVELS = AD_THREADS / 4;
// Resident CTAs per SM the pass B reverse is compiled for: two in FP32 (a
// 128-register cap), one in FP64.
template <class FT>
struct AdMinBlocks {
  static constexpr int value = sizeof(FT) == 4 ? 2 : 1;
};

template <class FT>
__device__ __forceinline__ void load_slab(FT *dst, const FT *src, int n) {
  for (int q = threadIdx.x; q < n; q += blockDim.x) dst[q] = src[q];
}

// Per-level forward quantities of one row at centre level v.
template <class FT>
__device__ __forceinline__ void level_geo(const DevParams<FT> &P, const RowGeo<FT> &g, int v, LevRow<FT> &s) {
  const int Nv = P.Nv;
  s.set(g, P.levc[LC_R2 * Nv + v], P.levc[LC_IR2 * Nv + v], P.levc[LC_DZ * Nv + v], P.levc[LC_IDZ * Nv + v]);
}

// Device shape shared by the reverse slab kernels.
struct AdDev {
  int nsm = 0, optin = 0, per_sm = 0;
};
AdDev &ad_dev() {
  static AdDev d;
  if (!d.nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&d.nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&d.optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&d.per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (d.nsm <= 0) d.nsm = 1;
  }
  return d;
}
// Buffering and resident CTAs per SM of a TMA slab kernel (1 KB per CTA is
// reserved by the hardware): double buffering at `minb` CTAs if it fits,
// else single buffering at `minb`, else one double- or single-buffered CTA.
struct AdShape {
  int nbuf, ctas;
  size_t smem;
};
template <class L>
AdShape ad_shape(int Nv, int minb) {
  const AdDev &d = ad_dev();
  const size_t two = L(Nv, 2).total, one = L(Nv, 1).total, per_sm = (size_t)d.per_sm;
  if (minb >= 2) {
    if (2 * (two + 1024) <= per_sm) return {2, 2, two};
    if (2 * (one + 1024) <= per_sm) return {1, 2, one};
  }
  if (two <= (size_t)d.optin) return {2, 1, two};
  return {1, 1, one};
}

// ----------------------------------------------------------------------------- pass A^T
// Per buffer: the state Y (64 Nv) and faces (16 Nf), the element geometry,
// the Laplacian cotangent Lb (64 Nv) and the state cotangent (64 Nv, 16 Nf),
// which is accumulated in place and stored back.  Scratch: the face parts of
// each level's cotangent, level-major rows [Nv][16] (lower, upper face).
template <class FT>
struct AvLayout {
  size_t y[2], f[2], g[2], lb[2], yb[2], fb[2], lo, hi, bar, total;
  __host__ __device__ AvLayout(int Nv, int nbuf) {
    const int Nf = Nv + 1;
    size_t o = 0;
    for (int b = 0; b < 2; ++b) {
      if (b < nbuf) {
        y[b] = o; o += align16(sizeof(FT) * 64 * Nv);
        f[b] = o; o += align16(sizeof(FT) * 16 * Nf);
        g[b] = o; o += align16(sizeof(FT) * HG_N * 16);
        lb[b] = o; o += align16(sizeof(FT) * 64 * Nv);
        yb[b] = o; o += align16(sizeof(FT) * 64 * Nv);
        fb[b] = o; o += align16(sizeof(FT) * 16 * Nf);
      } else {
        y[b] = y[0]; f[b] = f[0]; g[b] = g[0]; lb[b] = lb[0]; yb[b] = yb[0]; fb[b] = fb[0];
      }
    }
    lo = o; o += align16(sizeof(FT) * 16 * Nv);
    hi = o; o += align16(sizeof(FT) * 16 * Nv);
    bar = o; o += 16;
    total = o;
  }
};

template <class FT>
__global__ void __launch_bounds__(AD_THREADS, AdMinBlocks<FT>::value)
    k_passA_vjp(DevParams<FT> P, int nbuf, const FT *__restrict__ Yc, const FT *__restrict__ Yf,
                const FT *__restrict__ Lb, FT *__restrict__ Ybc, FT *__restrict__ Ybf) {
  extern __shared__ __align__(128) unsigned char sm[];
  const int Nv = P.Nv, Nf = P.Nf;
  const AvLayout<FT> Lo(Nv, nbuf);
  // slab x of buffer b (selects, not a runtime-indexed array)
  auto at = [&](const size_t (&off)[2], int b) { return (FT *)(sm + (b ? off[1] : off[0])); };
  FT *sLo = (FT *)(sm + Lo.lo), *sHi = (FT *)(sm + Lo.hi);
  uint64_t *bar = (uint64_t *)(sm + Lo.bar);
  const uint32_t by = uint32_t(sizeof(FT) * 64 * Nv), bf = uint32_t(sizeof(FT) * 16 * Nf);
  const uint32_t bg = uint32_t(sizeof(FT) * HG_N * 16);
  auto issue = [&](int b, int e) {
    mbar_expect_tx(b ? &bar[1] : &bar[0], 3 * by + 2 * bf + bg);
    uint64_t *bb = b ? &bar[1] : &bar[0];
    tma_load(at(Lo.y, b), Yc + (size_t)e * 64 * Nv, by, bb);
    tma_load(at(Lo.f, b), Yf + (size_t)e * 16 * Nf, bf, bb);
    tma_load(at(Lo.g, b), P.hgeo + (size_t)e * HG_N * 16, bg, bb);
    tma_load(at(Lo.lb, b), Lb + (size_t)e * 64 * Nv, by, bb);
    tma_load(at(Lo.yb, b), Ybc + (size_t)e * 64 * Nv, by, bb);
    tma_load(at(Lo.fb, b), Ybf + (size_t)e * 16 * Nf, bf, bb);
  };
  slab_init_bars(bar);
  int e = blockIdx.x;
  if (threadIdx.x == 0 && e < P.Nh) issue(0, e);
  const int j = threadIdx.x & 3, vl = threadIdx.x >> 2, vs = level_slot(vl);
  Row<FT> R;
  R.init(P, j);
  for (int it = 0; e < P.Nh; ++it, e += gridDim.x) {
    int b;
    if (!slab_begin(bar, nbuf, it, e, P.Nh, P.status, issue, b)) break;
    const FT *sY = at(Lo.y, b), *sF = at(Lo.f, b), *sG = at(Lo.g, b), *sL = at(Lo.lb, b);
    FT *sB = at(Lo.yb, b), *sBf = at(Lo.fb, b);
    RowGeo<FT> g;
    g.load(sG, P, j);
    for (int v0 = 0; v0 < Nv; v0 += AD_LEVELS) {
      const int v = min(v0 + vs, Nv - 1);
      const bool act = v0 + vs < Nv;
      LevRow<FT> s;
      level_geo(P, g, v, s);
      const FT Phi = P.levc[LC_PHI * Nv + v];
      const FT g3a = P.levf[LF_G33 * Nf + v], g3b = P.levf[LF_G33 * Nf + v + 1];
      FT Lsb[4], L1b[4], L2b[4], L3b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int q = (NQ * j + i) * Nv + v;
        Lsb[i] = sL[q];
        L1b[i] = sL[16 * Nv + q];
        L2b[i] = sL[32 * Nv + q];
        L3b[i] = sL[48 * Nv + q];
      }
      FT u1b[4], u2b[4], ub3b[4], sdb[4];
      vec_lap_t(P, R, g, s, L1b, L2b, L3b, FT(1), u1b, u2b, ub3b);
      lap_t(P, R, g, s, Lsb, sdb);
      FT lo[4], hi[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int n = NQ * j + i;
        const int q = n * Nv + v;
        const FT rho = sY[q], u1 = sY[16 * Nv + q], u2 = sY[32 * Nv + q], rhoe = sY[48 * Nv + q];
        const FT gu0 = g.gu0[i] * s.ir2, gu1 = g.gu1[i] * s.ir2, gu2 = g.gu2[i] * s.ir2;
        const FT c1 = gu0 * u1 + gu1 * u2, c2 = gu1 * u1 + gu2 * u2;
        // faces v, v+1 (u_3 = 0 on the boundary faces): u_bar_3 = (a + b)/2, Kv = (a^2 g33_a + b^2 g33_b)/2
        const FT fa = v == 0 ? FT(0) : sF[n * Nf + v], fb = v + 1 == Nv ? FT(0) : sF[n * Nf + v + 1];
        const FT kv = (fa * (fa * g3a) + fb * (fb * g3b)) / FT(2);
        const FT K = (u1 * c1 + u2 * c2 + kv) / FT(2);
        // sd = cp (T - T_r(Pi)) + Phi - Phi_r(Pi)
        ThermoBar<FT> tb{};
        tb.T = P.cpd * sdb[i];
        tb.Tr = -P.cpd * sdb[i];
        tb.phir = -sdb[i];
        FT rb, reb, Kb;
        thermo_vjp(P, rho, rhoe, K, Phi, tb, rb, reb, Kb);
        // K = (u . c + Kv) / 2: dK/du_h = c, dK/dKv = 1/2
        if (act) {
          sB[q] += rb;
          sB[16 * Nv + q] += u1b[i] + c1 * Kb;
          sB[32 * Nv + q] += u2b[i] + c2 * Kb;
          sB[48 * Nv + q] += reb;
        }
        const FT Kvb = Kb / FT(2);
        lo[i] = v == 0 ? FT(0) : ub3b[i] / FT(2) + Kvb * fa * g3a;
        hi[i] = v + 1 == Nv ? FT(0) : ub3b[i] / FT(2) + Kvb * fb * g3b;
      }
      if (act) {
        st_row(sLo + (size_t)v * NN + NQ * j, lo);
        st_row(sHi + (size_t)v * NN + NQ * j, hi);
      }
    }
    __syncthreads();
    // inner face k gathers the upper part of level k-1 and the lower part of level k
    for (int k0 = 1; k0 < Nv; k0 += AD_LEVELS) {
      const int k = k0 + vl;
      if (k < Nv) {
        FT hi[4], lo[4];
        ld_row(sHi + (size_t)(k - 1) * NN + NQ * j, hi);
        ld_row(sLo + (size_t)k * NN + NQ * j, lo);
#pragma unroll
        for (int i = 0; i < 4; ++i) sBf[(NQ * j + i) * Nf + k] += hi[i] + lo[i];
      }
    }
    fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      tma_store(Ybc + (size_t)e * 64 * Nv, sB, by);
      tma_store(Ybf + (size_t)e * 16 * Nf, sBf, bf);
      tma_store_commit();
    }
  }
  if (threadIdx.x == 0) tma_store_wait_all();
}

// ----------------------------------------------------------------------------- pass B^T
// Shared memory (FT words): Y 64Nv, F 16Nf, geometry HG_N*16 (the Laplacians
// and the tendency cotangent are read from global memory); centre scratch
// Kv, c1, c2, K, rho J, o3, a3 (7 x 16Nv), lower/upper face parts (2 x 16Nv);
// face scratch X1, X2, and the face cotangents cc1, cc2, gK, l4, rJ, cv1, cv2,
// u3 (10 x 16Nf).
template <class FT>
__host__ __device__ inline size_t passB_vjp_words(int Nv) {
  const size_t Nf = Nv + 1;
  return 64 * (size_t)Nv + 16 * Nf + HG_N * 16 + 9 * 16 * (size_t)Nv + 10 * 16 * Nf;
}

template <class FT>
__global__ void __launch_bounds__(AD_THREADS, AdMinBlocks<FT>::value) k_passB_vjp(DevParams<FT> P, const FT *__restrict__ Yc,
                                                          const FT *__restrict__ Yf, const FT *__restrict__ Lc,
                                                          const FT *__restrict__ Tbc, const FT *__restrict__ Tbf,
                                                          FT *__restrict__ Ybc, FT *__restrict__ Ybf,
                                                          FT *__restrict__ Lbc, double *__restrict__ dpar) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  FT *sm = (FT *)sm_raw;
  const int Nv = P.Nv, Nf = P.Nf;
  FT *sY = sm, *sF = sY + 64 * Nv;
  FT *sG = sF + 16 * Nf;
  FT *sKv = sG + HG_N * 16, *sC1 = sKv + 16 * Nv, *sC2 = sC1 + 16 * Nv, *sK = sC2 + 16 * Nv;
  FT *sRJ = sK + 16 * Nv, *sL4 = sRJ + 16 * Nv, *sA3 = sL4 + 16 * Nv, *sLo = sA3 + 16 * Nv, *sHi = sLo + 16 * Nv;
  FT *sX1 = sHi + 16 * Nv, *sX2 = sX1 + 16 * Nf, *bCc1 = sX2 + 16 * Nf, *bCc2 = bCc1 + 16 * Nf;
  FT *bGK = bCc2 + 16 * Nf, *bL4 = bGK + 16 * Nf, *bRJ = bL4 + 16 * Nf, *bCv1 = bRJ + 16 * Nf;
  FT *bCv2 = bCv1 + 16 * Nf, *bU3 = bCv2 + 16 * Nf;
  const int j = threadIdx.x & 3, vl = threadIdx.x >> 2;
  Row<FT> R;
  R.init(P, j);
  const FT nu = P.nu_v, nus = P.nu_s;
  const FT rpr = nu != FT(0) ? nus / nu : FT(1);  // d nu_s / d nu = 1 / Prandtl
  double dnu = 0, dal = 0;
  for (int e = blockIdx.x; e < P.Nh; e += gridDim.x) {
    load_slab(sY, Yc + (size_t)e * 64 * Nv, 64 * Nv);
    load_slab(sF, Yf + (size_t)e * 16 * Nf, 16 * Nf);
    load_slab(sG, P.hgeo + (size_t)e * HG_N * 16, HG_N * 16);
    // the Laplacians and the tendency cotangent are read in place (L1-cached)
    const FT *sL = Lc + (size_t)e * 64 * Nv, *sT = Tbc + (size_t)e * 64 * Nv, *sTf = Tbf + (size_t)e * 16 * Nf;
    __syncthreads();
    centre_from_faces<FT>(P, sF, nullptr, sKv);
    __syncthreads();
    RowGeo<FT> g;
    g.load(sG, P, j);
    // ---- C: forward centre quantities used by the face phase and the P3 transpose
    for (int v0 = 0; v0 < Nv; v0 += AD_LEVELS) {
      const int v = min(v0 + vl, Nv - 1);
      const bool act = v0 + vl < Nv;
      LevRow<FT> s;
      level_geo(P, g, v, s);
      const FT idz = P.levc[LC_IDZ * Nv + v];
      FT rho[4], u1[4], u2[4], L1[4], L2[4], L3[4], Ls[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int q = (NQ * j + i) * Nv + v;
        rho[i] = sY[q];
        u1[i] = sY[16 * Nv + q];
        u2[i] = sY[32 * Nv + q];
        Ls[i] = sL[q];
        L1[i] = sL[16 * Nv + q];
        L2[i] = sL[32 * Nv + q];
        L3[i] = sL[48 * Nv + q];
      }
      FT o1[4], o2[4], o3[4];
      vec_lap(P, R, g, s, L1, L2, L3, P.div_damp, o1, o2, o3);
      FT g1[4], g2[4], x1[4], x2[4], hd[4];
      d1(P, Ls, g1);
      d2(R, Ls, g2);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const FT gu0 = g.gu0[i] * s.ir2, gu1 = g.gu1[i] * s.ir2, gu2 = g.gu2[i] * s.ir2;
        x1[i] = rho[i] * (gu0 * g1[i] + gu1 * g2[i]);
        x2[i] = rho[i] * (gu1 * g1[i] + gu2 * g2[i]);
      }
      wdiv(P, R, s, x1, x2, hd);
      FT om[4];
      {
        FT Wu1[4], Wu2[4], ta[4], tb[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          Wu1[i] = g.W[i] * u1[i];
          Wu2[i] = g.W[i] * u2[i];
        }
        t1(P, Wu2, ta);
        t2(R, Wu1, tb);
#pragma unroll
        for (int i = 0; i < 4; ++i) om[i] = (-ta[i] + tb[i]) * s.iWJ[i];
      }
      if (act) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int n = NQ * j + i, q = n * Nv + v;
          const FT gu0 = g.gu0[i] * s.ir2, gu1 = g.gu1[i] * s.ir2, gu2 = g.gu2[i] * s.ir2;
          const FT c1 = gu0 * u1[i] + gu1 * u2[i], c2 = gu1 * u1[i] + gu2 * u2[i];
          sC1[q] = c1;
          sC2[q] = c2;
          sK[q] = (u1[i] * c1 + u2[i] * c2 + sKv[q]) / FT(2);
          sRJ[q] = rho[i] * s.J[i];
          sL4[q] = o3[i];
          sA3[q] = sG[HG_F3 * NN + n] * idz + om[i];
          dnu -= (double)(o1[i] * sT[16 * Nv + q] + o2[i] * sT[32 * Nv + q] + rpr * hd[i] * sT[48 * Nv + q]);
        }
      }
    }
    __syncthreads();
    // ---- D: face phase, forward and reverse (the P3 cotangent of X is known from Tb and rho J)
    for (int k0 = 0; k0 < Nf; k0 += AD_LEVELS) {
      const int k = min(k0 + vl, Nf - 1);
      const bool act = k0 + vl < Nf;
      const bool inner = k > 0 && k < Nv;
      const FT r2 = P.levf[LF_R2 * Nf + k], dzf = P.levf[LF_DZ * Nf + k], rinv = P.levf[LF_RINV * Nf + k];
      const FT ir2f = P.levf[LF_IR2 * Nf + k], idzf = P.levf[LF_IDZ * Nf + k], g33 = P.levf[LF_G33 * Nf + k];
      FT Wu[4], u3[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        u3[i] = inner ? sF[(NQ * j + i) * Nf + k] : FT(0);
        Wu[i] = g.W[i] * u3[i];
      }
      FT ta[4], tb[4];
      t2(R, Wu, tb);
      t1(P, Wu, ta);
      const int va = k > 0 ? k - 1 : 0, vb = k < Nv ? k : Nv - 1;
      FT tab[4], tbb[4], u3d[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int n = NQ * j + i;
        const int qa = n * Nv + va, qb = n * Nv + vb;
        const FT Jf = g.Jh[i] * r2 * dzf;
        const FT iJf = g.iJh[i] * ir2f * idzf, iWJf = g.iW[i] * iJf;
        const FT w1 = -tb[i] * iWJf, w2 = ta[i] * iWJf;
        FT cv1 = 0, cv2 = 0, cc1, cc2, l4, rJ;
        if (inner) {
          cv1 = -(sY[32 * Nv + qb] - sY[32 * Nv + qa]) * iJf;
          cv2 = (sY[16 * Nv + qb] - sY[16 * Nv + qa]) * iJf;
          cc1 = (sC1[qa] + sC1[qb]) / FT(2);
          cc2 = (sC2[qa] + sC2[qb]) / FT(2);
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
        const FT fo1 = sG[HG_FH1 * NN + n] * rinv + cv1 + w1, fo2 = sG[HG_FH2 * NN + n] * rinv + cv2 + w2;
        const FT b3 = rJ * (u3[i] * g33);
        // X-cotangents from P3: t_i(v) = (X_i(v) + X_i(v+1)) / (2 rho J(v)) + ..., T_u_i -= t_i
        FT Xb1 = 0, Xb2 = 0;
        if (k >= 1) {
          Xb1 -= sT[16 * Nv + qa] / (FT(2) * sRJ[qa]);
          Xb2 -= sT[32 * Nv + qa] / (FT(2) * sRJ[qa]);
        }
        if (k < Nv) {
          Xb1 -= sT[16 * Nv + qb] / (FT(2) * sRJ[qb]);
          Xb2 -= sT[32 * Nv + qb] / (FT(2) * sRJ[qb]);
        }
        const FT T3b = sTf[n * Nf + k];
        const FT b3b = Jf * (fo2 * Xb1 - fo1 * Xb2);
        const FT fo1b = -Jf * b3 * Xb2 - Jf * cc2 * T3b;
        const FT fo2b = Jf * b3 * Xb1 + Jf * cc1 * T3b;
        if (act) {
          sX1[n * Nf + k] = Jf * (fo2 * b3);
          sX2[n * Nf + k] = Jf * (-fo1 * b3);
          bCc1[n * Nf + k] = Jf * fo2 * T3b;
          bCc2[n * Nf + k] = -Jf * fo1 * T3b;
          bGK[n * Nf + k] = inner ? -T3b : FT(0);
          bL4[n * Nf + k] = -nu * T3b;
          bRJ[n * Nf + k] = b3b * u3[i] * g33;
          bCv1[n * Nf + k] = inner ? fo1b * iJf : FT(0);
          bCv2[n * Nf + k] = inner ? fo2b * iJf : FT(0);
          dnu -= (double)(l4 * T3b);
        }
        u3d[i] = inner ? b3b * rJ * g33 : FT(0);
        // w1 = -tb iWJf, w2 = ta iWJf  ->  cotangents of tb, ta
        tbb[i] = -fo1b * iWJf;
        tab[i] = fo2b * iWJf;
      }
      FT Wb[4], Wb2[4];
      d1(P, tab, Wb);
      d2(R, tbb, Wb2);
      if (act) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int n = NQ * j + i;
          bU3[n * Nf + k] = inner ? u3d[i] + g.W[i] * (Wb[i] + Wb2[i]) : FT(0);
        }
      }
    }
    __syncthreads();
    // ---- G: centre phase: P3 and face gathers, then the P1 transpose
    FT *yb = Ybc + (size_t)e * 64 * Nv, *lb = Lbc + (size_t)e * 64 * Nv;
    for (int v0 = 0; v0 < Nv; v0 += AD_LEVELS) {
      const int v = min(v0 + vl, Nv - 1);
      const bool act = v0 + vl < Nv;
      LevRow<FT> s;
      level_geo(P, g, v, s);
      const FT Phi = P.levc[LC_PHI * Nv + v], beta = P.levc[LC_BETA * Nv + v], spg = P.levc[LC_SPG * Nv + v];
      FT rho[4], u1[4], u2[4], rhoe[4], c1[4], c2[4], K[4];
      FT Trb[4], Tu1b[4], Tu2b[4], Teb[4];
      FT rhob[4], u1b[4], u2b[4], c1b[4], c2b[4], Kb[4], L4b[4], omb[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int n = NQ * j + i, q = n * Nv + v;
        rho[i] = sY[q];
        u1[i] = sY[16 * Nv + q];
        u2[i] = sY[32 * Nv + q];
        rhoe[i] = sY[48 * Nv + q];
        c1[i] = sC1[q];
        c2[i] = sC2[q];
        K[i] = sK[q];
        Trb[i] = sT[q];
        Tu1b[i] = sT[16 * Nv + q];
        Tu2b[i] = sT[32 * Nv + q];
        Teb[i] = sT[48 * Nv + q];
        const FT RJ = sRJ[q], iRJ = FT(1) / RJ;
        // P3: t_i = (X_i(v) + X_i(v+1)) / 2 / rho J + Cr_i, T_u_i -= t_i + beta u_i
        const FT X1s = (sX1[n * Nf + v] + sX1[n * Nf + v + 1]) / FT(2);
        const FT X2s = (sX2[n * Nf + v] + sX2[n * Nf + v + 1]) / FT(2);
        const FT t1b = -Tu1b[i], t2b = -Tu2b[i];
        FT RJb = -(X1s * t1b + X2s * t2b) * iRJ * iRJ;
        const FT a3 = sA3[q];
        // Cr1 = J (-a3 c2), Cr2 = J (a3 c1)
        omb[i] = s.J[i] * (c1[i] * t2b - c2[i] * t1b);
        c1b[i] = s.J[i] * a3 * t2b;
        c2b[i] = -s.J[i] * a3 * t1b;
        u1b[i] = -beta * Tu1b[i];
        u2b[i] = -beta * Tu2b[i];
        if (act) dal -= (double)(spg * (u1[i] * Tu1b[i] + u2[i] * Tu2b[i]));
        Kb[i] = FT(0);
        // gathers from face v (this centre is its upper neighbour) and face v+1 (lower neighbour)
        const int fl = n * Nf + v, fu = n * Nf + v + 1;
        const FT L4v = sL4[q];
        FT l4b = FT(0);
        if (v > 0) {
          const FT wa = sRJ[q - 1], wb = RJ, ws = wa + wb;
          const FT l4 = (wa * sL4[q - 1] + wb * L4v) / ws;
          c1b[i] += bCc1[fl] / FT(2);
          c2b[i] += bCc2[fl] / FT(2);
          Kb[i] += bGK[fl];
          l4b += bL4[fl] * wb / ws;
          RJb += bL4[fl] * (L4v - l4) / ws + bRJ[fl] / FT(2);
          u1b[i] += bCv2[fl];
          u2b[i] -= bCv1[fl];
        } else {
          c1b[i] += bCc1[fl];
          c2b[i] += bCc2[fl];
          l4b += bL4[fl];
          RJb += bRJ[fl];
        }
        if (v + 1 < Nv) {
          const FT wa = RJ, wb = sRJ[q + 1], ws = wa + wb;
          const FT l4 = (wa * L4v + wb * sL4[q + 1]) / ws;
          c1b[i] += bCc1[fu] / FT(2);
          c2b[i] += bCc2[fu] / FT(2);
          Kb[i] -= bGK[fu];
          l4b += bL4[fu] * wa / ws;
          RJb += bL4[fu] * (L4v - l4) / ws + bRJ[fu] / FT(2);
          u1b[i] -= bCv2[fu];
          u2b[i] += bCv1[fu];
        } else {
          c1b[i] += bCc1[fu];
          c2b[i] += bCc2[fu];
          l4b += bL4[fu];
          RJb += bRJ[fu];
        }
        L4b[i] = l4b;
        rhob[i] = s.J[i] * RJb;
      }
      // ---- hyperdiffusion: T_u -= nu o(L), T_rhoe -= nu_s wdiv(rho g^-1 grad L_s), o3 -> faces (L4)
      {
        FT o1b[4], o2b[4], L1b[4], L2b[4], L3b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          o1b[i] = -nu * Tu1b[i];
          o2b[i] = -nu * Tu2b[i];
        }
        vec_lap_t(P, R, g, s, o1b, o2b, L4b, P.div_damp, L1b, L2b, L3b);
        FT hdb[4], xb1[4], xb2[4], Ls[4], g1[4], g2[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          hdb[i] = -nus * Teb[i];
          Ls[i] = sL[(NQ * j + i) * Nv + v];
        }
        wdiv_t(P, R, s, hdb, xb1, xb2);
        d1(P, Ls, g1);
        d2(R, Ls, g2);
        FT gb1[4], gb2[4], Lsb[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const FT gu0 = g.gu0[i] * s.ir2, gu1 = g.gu1[i] * s.ir2, gu2 = g.gu2[i] * s.ir2;
          rhob[i] += (gu0 * g1[i] + gu1 * g2[i]) * xb1[i] + (gu1 * g1[i] + gu2 * g2[i]) * xb2[i];
          gb1[i] = rho[i] * (gu0 * xb1[i] + gu1 * xb2[i]);
          gb2[i] = rho[i] * (gu1 * xb1[i] + gu2 * xb2[i]);
        }
        grad_t(P, R, gb1, gb2, Lsb);
        if (act) {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int q = (NQ * j + i) * Nv + v;
            lb[q] = Lsb[i];
            lb[16 * Nv + q] = L1b[i];
            lb[32 * Nv + q] = L2b[i];
            lb[48 * Nv + q] = L3b[i];
          }
        }
      }
      // ---- vorticity: om = (-t1(W u2) + t2(W u1)) / WJ
      {
        FT tab[4], tbb[4], da[4], db[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          tab[i] = -omb[i] * s.iWJ[i];
          tbb[i] = omb[i] * s.iWJ[i];
        }
        d1(P, tab, da);
        d2(R, tbb, db);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          u2b[i] += g.W[i] * da[i];
          u1b[i] += g.W[i] * db[i];
        }
      }
      // ---- forward thermodynamics and the horizontal-dynamics transpose
      FT h[4], Pi[4], thp[4], tp[4], F1[4], F2[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        Thermo<FT> th;
        thermo(P, rho[i], rhoe[i], K[i], Phi, th);
        h[i] = th.h;
        Pi[i] = th.Pi;
        thp[i] = th.thv - th.thvr;
        tp[i] = thp[i] * Pi[i];
        F1[i] = rho[i] * c1[i];
        F2[i] = rho[i] * c2[i];
      }
      FT hb_[4], Pib[4], thpb[4], phirb[4];
      {
        // T_u_i = -(a_i + cp (thp b_i + e_i - Pi f_i) / 2), a = grad tmp, b = grad Pi, e = grad tp, f = grad thp
        FT b1[4], b2[4], f1[4], f2[4];
        d1(P, Pi, b1);
        d2(R, Pi, b2);
        d1(P, thp, f1);
        d2(R, thp, f2);
        FT ab1[4], ab2[4], bb1[4], bb2[4], eb1[4], eb2[4], fb1[4], fb2[4];
        const FT hc = P.cpd / FT(2);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          ab1[i] = -Tu1b[i];
          ab2[i] = -Tu2b[i];
          bb1[i] = -hc * thp[i] * Tu1b[i];
          bb2[i] = -hc * thp[i] * Tu2b[i];
          eb1[i] = -hc * Tu1b[i];
          eb2[i] = -hc * Tu2b[i];
          fb1[i] = hc * Pi[i] * Tu1b[i];
          fb2[i] = hc * Pi[i] * Tu2b[i];
          thpb[i] = -hc * (b1[i] * Tu1b[i] + b2[i] * Tu2b[i]);
          Pib[i] = hc * (f1[i] * Tu1b[i] + f2[i] * Tu2b[i]);
        }
        FT tmpb[4], x[4], tpb[4];
        grad_t(P, R, ab1, ab2, tmpb);
        grad_t(P, R, bb1, bb2, x);
        grad_t(P, R, eb1, eb2, tpb);
#pragma unroll
        for (int i = 0; i < 4; ++i) Pib[i] += x[i];
        grad_t(P, R, fb1, fb2, x);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          thpb[i] += x[i] + Pi[i] * tpb[i];
          Pib[i] += thp[i] * tpb[i];
          Kb[i] += tmpb[i];
          phirb[i] = -tmpb[i];
        }
      }
      {
        // T_rho = -dm, T_rhoe = -(dmh + h dm + F . grad h) / 2, dm = wdiv(F), dmh = wdiv(F h)
        FT dm[4], ha[4], hbv[4];
        wdiv(P, R, s, F1, F2, dm);
        d1(P, h, ha);
        d2(R, h, hbv);
        FT dmb[4], dmhb[4], hab[4], hbb[4], F1b[4], F2b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const FT q = Teb[i] / FT(2);
          dmb[i] = -Trb[i] - h[i] * q;
          dmhb[i] = -q;
          hb_[i] = -dm[i] * q;
          F1b[i] = -ha[i] * q;
          F2b[i] = -hbv[i] * q;
          hab[i] = -F1[i] * q;
          hbb[i] = -F2[i] * q;
        }
        FT x[4], y1[4], y2[4];
        grad_t(P, R, hab, hbb, x);
        wdiv_t(P, R, s, dmb, y1, y2);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          hb_[i] += x[i];
          F1b[i] += y1[i];
          F2b[i] += y2[i];
        }
        wdiv_t(P, R, s, dmhb, y1, y2);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          F1b[i] += h[i] * y1[i];
          F2b[i] += h[i] * y2[i];
          hb_[i] += F1[i] * y1[i] + F2[i] * y2[i];
          rhob[i] += c1[i] * F1b[i] + c2[i] * F2b[i];
          c1b[i] += rho[i] * F1b[i];
          c2b[i] += rho[i] * F2b[i];
        }
      }
      if (act) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int n = NQ * j + i, q = n * Nv + v;
          ThermoBar<FT> tb{};
          tb.h = hb_[i];
          tb.Pi = Pib[i];
          tb.thv = thpb[i];
          tb.thvr = -thpb[i];
          tb.phir = phirb[i];
          FT rb, reb, kb;
          thermo_vjp(P, rho[i], rhoe[i], K[i], Phi, tb, rb, reb, kb);
          const FT Kt = Kb[i] + kb;
          const FT gu0 = g.gu0[i] * s.ir2, gu1 = g.gu1[i] * s.ir2, gu2 = g.gu2[i] * s.ir2;
          yb[q] += rhob[i] + rb;
          yb[16 * Nv + q] += u1b[i] + c1[i] * Kt + gu0 * c1b[i] + gu1 * c2b[i];
          yb[32 * Nv + q] += u2b[i] + c2[i] * Kt + gu1 * c1b[i] + gu2 * c2b[i];
          yb[48 * Nv + q] += reb;
          const FT a = v == 0 ? FT(0) : sF[n * Nf + v], bt = v + 1 == Nv ? FT(0) : sF[n * Nf + v + 1];
          const FT Kvb = Kt / FT(2);
          sLo[q] = v == 0 ? FT(0) : Kvb * a * P.levf[LF_G33 * Nf + v];
          sHi[q] = v + 1 == Nv ? FT(0) : Kvb * bt * P.levf[LF_G33 * Nf + v + 1];
        }
      }
    }
    __syncthreads();
    FT *fb = Ybf + (size_t)e * 16 * Nf;
    for (int idx = threadIdx.x; idx < 16 * Nf; idx += blockDim.x) {
      const int n = idx / Nf, f = idx - n * Nf;
      if (f > 0 && f < Nv) fb[idx] += bU3[idx] + sHi[n * Nv + f - 1] + sLo[n * Nv + f];
    }
    __syncthreads();
  }
  // parameter cotangents: block sums in a fixed order, one slot per CTA
  __shared__ double red[2][AD_THREADS];
  red[0][threadIdx.x] = dnu;
  red[1][threadIdx.x] = dal;
  __syncthreads();
  for (int o = AD_THREADS / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      red[0][threadIdx.x] += red[0][threadIdx.x + o];
      red[1][threadIdx.x] += red[1][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {  // accumulated over the launches of a reverse pass (zeroed by the host)
    dpar[2 * blockIdx.x] += red[0][0];
    dpar[2 * blockIdx.x + 1] += red[1][0];
  }
}

}  // namespace

template <class FT>
size_t passA_vjp_smem(int Nv) {
  return AvLayout<FT>(Nv, 1).total;
}
template <class FT>
size_t passB_vjp_smem(int Nv) {
  return sizeof(FT) * passB_vjp_words<FT>(Nv);
}

template <class FT>
void configure_adjoint_se(int Nv) {
  (void)Nv;
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  // the dynamic limit is the opt-in maximum less the kernel's static shared memory
  cudaFuncAttributes fa{};
  cudaFuncGetAttributes(&fa, k_passA_vjp<FT>);
  cudaFuncSetAttribute(k_passA_vjp<FT>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
  cudaFuncGetAttributes(&fa, k_passB_vjp<FT>);
  cudaFuncSetAttribute(k_passB_vjp<FT>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
}

// Persistent grids: the resident CTAs of each kernel at its shared-memory size.
template <class K>
int resident_grid(K kern, size_t smem, int Nh) {
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  }
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, AD_THREADS, smem);
  return std::max(1, std::min(Nh, nsm * std::max(1, b)));
}

template <class FT>
void launch_passA_vjp(const DevParams<FT> &P, const FT *Yc, const FT *Yf, const FT *Lb, FT *Ybc, FT *Ybf, int grid,
                      cudaStream_t s) {
  (void)grid;
  const AdShape sh = ad_shape<AvLayout<FT>>(P.Nv, AdMinBlocks<FT>::value);
  const int g = std::max(1, std::min(P.Nh, ad_dev().nsm * sh.ctas));
  k_passA_vjp<FT><<<g, AD_THREADS, sh.smem, s>>>(P, sh.nbuf, Yc, Yf, Lb, Ybc, Ybf);
}
// grid: the number of parameter-partial slots (CTAs) the caller allocated.
template <class FT>
void launch_passB_vjp(const DevParams<FT> &P, const FT *Yc, const FT *Yf, const FT *L, const FT *Tbc, const FT *Tbf,
                      FT *Ybc, FT *Ybf, FT *Lb, double *dpar, int grid, cudaStream_t s) {
  const size_t sm = passB_vjp_smem<FT>(P.Nv);
  const int g = std::min(grid, resident_grid(k_passB_vjp<FT>, sm, P.Nh));
  k_passB_vjp<FT><<<g, AD_THREADS, sm, s>>>(P, Yc, Yf, L, Tbc, Tbf, Ybc, Ybf, Lb, dpar);
}

#define INST(FT)                                                                                             \
  template size_t passA_vjp_smem<FT>(int);                                                                   \
  template size_t passB_vjp_smem<FT>(int);                                                                   \
  template void configure_adjoint_se<FT>(int);                                                               \
  template void launch_passA_vjp<FT>(const DevParams<FT> &, const FT *, const FT *, const FT *, FT *, FT *, int, \
                                     cudaStream_t);                                                          \
  template void launch_passB_vjp<FT>(const DevParams<FT> &, const FT *, const FT *, const FT *, const FT *,      \
                                     const FT *, FT *, FT *, FT *, double *, int, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace gb
