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
// forward (level, row) mapping; the slabs of each element arrive by TMA bulk
// copies.  The state cotangent is accumulated (or, by pass B^T on request,
// written) element by element: each element owns its nodes, so there are no
// write conflicts; the DSS transposes before and after are separate kernels.
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
// Read once (a function-local static: thread-safe initialisation).
const AdDev &ad_dev() {
  static const AdDev d = [] {
    AdDev x;
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
// ADD: a further cotangent slab (xb, xf) is loaded and added as well.
template <class FT, bool ADD = false>
struct AvLayout {
  size_t y[2], f[2], g[2], lb[2], yb[2], fb[2], xb[2], xf[2], lo, hi, bar, total;
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
        xb[b] = xf[b] = 0;
        if (ADD) {
          xb[b] = o; o += align16(sizeof(FT) * 64 * Nv);
          xf[b] = o; o += align16(sizeof(FT) * 16 * Nf);
        }
      } else {
        y[b] = y[0]; f[b] = f[0]; g[b] = g[0]; lb[b] = lb[0]; yb[b] = yb[0]; fb[b] = fb[0];
        xb[b] = xb[0]; xf[b] = xf[0];
      }
    }
    lo = o; o += align16(sizeof(FT) * 16 * Nv);
    hi = o; o += align16(sizeof(FT) * 16 * Nv);
    bar = o; o += 16;
    total = o;
  }
};

// ADD: Ybar += Xbar + the pass's own contribution (Xbar, a further cotangent of
// the state, e.g. pass B^T's, is read by TMA with the other slabs).
template <class FT, bool ADD>
__global__ void __launch_bounds__(AD_THREADS, AdMinBlocks<FT>::value)
    k_passA_vjp(DevParams<FT> P, int nbuf, const FT *__restrict__ Yc, const FT *__restrict__ Yf,
                const FT *__restrict__ Lb, FT *__restrict__ Ybc, FT *__restrict__ Ybf, const FT *__restrict__ Xbc,
                const FT *__restrict__ Xbf) {
  extern __shared__ __align__(128) unsigned char sm[];
  const int Nv = P.Nv, Nf = P.Nf;
  const AvLayout<FT, ADD> Lo(Nv, nbuf);
  // slab x of buffer b (selects, not a runtime-indexed array)
  auto at = [&](const size_t (&off)[2], int b) { return (FT *)(sm + (b ? off[1] : off[0])); };
  FT *sLo = (FT *)(sm + Lo.lo), *sHi = (FT *)(sm + Lo.hi);
  uint64_t *bar = (uint64_t *)(sm + Lo.bar);
  const uint32_t by = uint32_t(sizeof(FT) * 64 * Nv), bf = uint32_t(sizeof(FT) * 16 * Nf);
  const uint32_t bg = uint32_t(sizeof(FT) * HG_N * 16);
  auto issue = [&](int b, int e) {
    mbar_expect_tx(b ? &bar[1] : &bar[0], ADD ? 4 * by + 3 * bf + bg : 3 * by + 2 * bf + bg);
    uint64_t *bb = b ? &bar[1] : &bar[0];
    tma_load(at(Lo.y, b), Yc + (size_t)e * 64 * Nv, by, bb);
    tma_load(at(Lo.f, b), Yf + (size_t)e * 16 * Nf, bf, bb);
    tma_load(at(Lo.g, b), P.hgeo + (size_t)e * HG_N * 16, bg, bb);
    tma_load(at(Lo.lb, b), Lb + (size_t)e * 64 * Nv, by, bb);
    tma_load(at(Lo.yb, b), Ybc + (size_t)e * 64 * Nv, by, bb);
    tma_load(at(Lo.fb, b), Ybf + (size_t)e * 16 * Nf, bf, bb);
    if (ADD) {
      tma_load(at(Lo.xb, b), Xbc + (size_t)e * 64 * Nv, by, bb);
      tma_load(at(Lo.xf, b), Xbf + (size_t)e * 16 * Nf, bf, bb);
    }
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
    const FT *sX = at(Lo.xb, b), *sXf = at(Lo.xf, b);
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
          if (ADD) {
            sB[q] += sX[q] + rb;
            sB[16 * Nv + q] += sX[16 * Nv + q] + (u1b[i] + c1 * Kb);
            sB[32 * Nv + q] += sX[32 * Nv + q] + (u2b[i] + c2 * Kb);
            sB[48 * Nv + q] += sX[48 * Nv + q] + reb;
          } else {
            sB[q] += rb;
            sB[16 * Nv + q] += u1b[i] + c1 * Kb;
            sB[32 * Nv + q] += u2b[i] + c2 * Kb;
            sB[48 * Nv + q] += reb;
          }
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
        for (int i = 0; i < 4; ++i) {
          const int idx = (NQ * j + i) * Nf + k;
          sBf[idx] += ADD ? sXf[idx] + (hi[i] + lo[i]) : hi[i] + lo[i];
        }
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
// Per buffer: the state Y (64 Nv) and faces (16 Nf), the element geometry,
// the DSSed Laplacians L (64 Nv) and the tendency cotangent Tb (64 Nv, 16 Nf).
// Scratch, level-major rows ([Nv][16] or [Nf][16], one 16-byte row per
// thread): the forward centre values c1, c2, K, rho J, o3; the forward face
// cross products X1, X2 and the face cotangents; the K_v cotangent.  The
// state cotangent goes to global memory, added (accum) or written; the
// Laplacian cotangent is written.
enum BvCentre { BC_C1 = 0, BC_C2, BC_K, BC_RJ, BC_L4, BC_N };
enum BvFace { BF_X1 = 0, BF_X2, BF_CC1, BF_CC2, BF_RJ, BF_CV1, BF_CV2, BF_U3, BF_N };

// GL: the Laplacians and the tendency cotangent are read from global memory
// instead of being staged (tall columns, where the staged slabs do not fit).
template <class FT, bool GL = false>
struct BvLayout {
  size_t y[2], f[2], g[2], lap[2], tb[2], tbf[2], c, fc, kvb, w, red, bar, total;
  __host__ __device__ BvLayout(int Nv, int nbuf) {
    const int Nf = Nv + 1;
    size_t o = 0;
    for (int b = 0; b < 2; ++b) {
      if (b < nbuf) {
        y[b] = o; o += align16(sizeof(FT) * 64 * Nv);
        f[b] = o; o += align16(sizeof(FT) * 16 * Nf);
        g[b] = o; o += align16(sizeof(FT) * HG_N * 16);
        lap[b] = tb[b] = tbf[b] = 0;
        if (!GL) {
          lap[b] = o; o += align16(sizeof(FT) * 64 * Nv);
          tb[b] = o; o += align16(sizeof(FT) * 64 * Nv);
          tbf[b] = o; o += align16(sizeof(FT) * 16 * Nf);
        }
      } else {
        y[b] = y[0]; f[b] = f[0]; g[b] = g[0]; lap[b] = lap[0]; tb[b] = tb[0]; tbf[b] = tbf[0];
      }
    }
    c = o; o += align16(sizeof(FT) * BC_N * 16 * Nv);
    fc = o; o += align16(sizeof(FT) * BF_N * 16 * Nf);
    kvb = o; o += align16(sizeof(FT) * 16 * Nv);
    w = o; o += align16(sizeof(FT) * 2 * 16);
    red = o; o += align16(sizeof(double) * 2 * (AD_THREADS / 32));
    bar = o; o += 16;
    total = o;
  }
};

// HS: the Held-Suarez forcing's pullback is compiled in (a separate instantiation).
template <class FT, bool HS, bool GL>
__global__ void __launch_bounds__(AD_THREADS, AdMinBlocks<FT>::value)
    k_passB_vjp(DevParams<FT> P, int nbuf, const FT *__restrict__ Yc, const FT *__restrict__ Yf,
                const FT *__restrict__ Lc, const FT *__restrict__ Tbc, const FT *__restrict__ Tbf,
                FT *__restrict__ Ybc, FT *__restrict__ Ybf, FT *__restrict__ Lbc, double *__restrict__ dpar,
                int accum, FT tsc) {
  extern __shared__ __align__(128) unsigned char sm[];
  const int Nv = P.Nv, Nf = P.Nf;
  const BvLayout<FT, GL> Lo(Nv, nbuf);
  auto at = [&](const size_t (&off)[2], int b) { return (FT *)(sm + (b ? off[1] : off[0])); };
  FT *sC = (FT *)(sm + Lo.c), *sFc = (FT *)(sm + Lo.fc), *sKvb = (FT *)(sm + Lo.kvb), *sW = (FT *)(sm + Lo.w);
  double *red = (double *)(sm + Lo.red);
  uint64_t *bar = (uint64_t *)(sm + Lo.bar);
  const uint32_t by = uint32_t(sizeof(FT) * 64 * Nv), bf = uint32_t(sizeof(FT) * 16 * Nf);
  const uint32_t bg = uint32_t(sizeof(FT) * HG_N * 16);
  auto issue = [&](int b, int e) {
    uint64_t *bb = b ? &bar[1] : &bar[0];
    mbar_expect_tx(bb, GL ? by + bf + bg : 3 * by + 2 * bf + bg);
    tma_load(at(Lo.y, b), Yc + (size_t)e * 64 * Nv, by, bb);
    tma_load(at(Lo.f, b), Yf + (size_t)e * 16 * Nf, bf, bb);
    tma_load(at(Lo.g, b), P.hgeo + (size_t)e * HG_N * 16, bg, bb);
    if (!GL) {
      tma_load(at(Lo.lap, b), Lc + (size_t)e * 64 * Nv, by, bb);
      tma_load(at(Lo.tb, b), Tbc + (size_t)e * 64 * Nv, by, bb);
      tma_load(at(Lo.tbf, b), Tbf + (size_t)e * 16 * Nf, bf, bb);
    }
  };
  if (threadIdx.x < NN) {
    sW[threadIdx.x] = P.W[threadIdx.x];
    sW[NN + threadIdx.x] = P.iW[threadIdx.x];
  }
  slab_init_bars(bar);
  int e = blockIdx.x;
  if (threadIdx.x == 0 && e < P.Nh) issue(0, e);
  const int j = threadIdx.x & 3, vl = threadIdx.x >> 2, vs = level_slot(vl);
  // the thread's row of centre scratch field f at level v / face field f at face k
  auto crow = [&](int f, int v) { return sC + ((size_t)f * Nv + v) * NN + NQ * j; };
  auto frow = [&](int f, int k) { return sFc + ((size_t)f * Nf + k) * NN + NQ * j; };
  Row<FT> R;
  R.init(P, j);
  const FT nu = P.nu_v, nus = P.nu_s;
  const FT rpr = nu != FT(0) ? nus / nu : FT(1);  // d nu_s / d nu = 1 / Prandtl
  const FT hc = P.cpd / FT(2);
  CSum<FT> dnu, dal;
  const FT inu = nu != FT(0) ? FT(1) / nu : FT(0);  // the Laplacian terms of d/dnu carry 1 / nu
  for (int it = 0; e < P.Nh; ++it, e += gridDim.x) {
    int b;
    if (!slab_begin(bar, nbuf, it, e, P.Nh, P.status, issue, b)) break;
    const FT *sY = at(Lo.y, b), *sF = at(Lo.f, b), *sG = at(Lo.g, b);
    const FT *sL = GL ? Lc + (size_t)e * 64 * Nv : at(Lo.lap, b);
    const FT *sT = GL ? Tbc + (size_t)e * 64 * Nv : at(Lo.tb, b);
    const FT *sTf = GL ? Tbf + (size_t)e * 16 * Nf : at(Lo.tbf, b);
    const SlabGeo<FT> g{sG + NQ * j, sW + NQ * j};
    auto levrow = [&](int v, LevRow<FT> &s) {
      FT Jh[4], iJh[4], W[4], iW[4];
      g.row(HG_JH, Jh);
      g.row(HG_IJH, iJh);
      g.w(W);
      g.iw(iW);
      s.set_rows(Jh, iJh, W, iW, P.levc[LC_R2 * Nv + v], P.levc[LC_IR2 * Nv + v], P.levc[LC_DZ * Nv + v],
                 P.levc[LC_IDZ * Nv + v]);
    };
    // ---- C: forward centre values used by the face phase and the centre transpose
    for (int v0 = 0; v0 < Nv; v0 += AD_LEVELS) {
      const int v = min(v0 + vs, Nv - 1);
      const bool act = v0 + vs < Nv;
      LevRow<FT> s;
      levrow(v, s);
      const FT g3a = P.levf[LF_G33 * Nf + v], g3b = P.levf[LF_G33 * Nf + v + 1];
      FT rho[4];
      {
        FT c1[4], c2[4], K[4], rJ[4], gu0[4], gu1[4], gu2[4];
        g.gu(gu0, gu1, gu2);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int n = NQ * j + i, q = n * Nv + v;
          rho[i] = sY[q];
          const FT u1 = sY[16 * Nv + q], u2 = sY[32 * Nv + q];
          const FT x0 = gu0[i] * s.ir2, x1 = gu1[i] * s.ir2, x2 = gu2[i] * s.ir2;
          c1[i] = x0 * u1 + x1 * u2;
          c2[i] = x1 * u1 + x2 * u2;
          const FT fa = v == 0 ? FT(0) : sF[n * Nf + v], fb = v + 1 == Nv ? FT(0) : sF[n * Nf + v + 1];
          const FT kv = (fa * (fa * g3a) + fb * (fb * g3b)) / FT(2);
          K[i] = (u1 * c1[i] + u2 * c2[i] + kv) / FT(2);
          rJ[i] = rho[i] * s.J[i];
        }
        if (act) {
          st_row(crow(BC_C1, v), c1);
          st_row(crow(BC_C2, v), c2);
          st_row(crow(BC_K, v), K);
          st_row(crow(BC_RJ, v), rJ);
        }
      }
      if (nu != FT(0)) {
        // only o3 (face phase) is needed: the d/dnu terms of o1, o2 and the rho e_tot
        // hyperdiffusion follow from the transposes in the centre phase (adjoint identity)
        FT L3[4], o3[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) L3[i] = sL[48 * Nv + (NQ * j + i) * Nv + v];
        vec_lap_o3(P, R, g, s, L3, o3);
        if (act) st_row(crow(BC_L4, v), o3);
        continue;
      }
      FT o1[4], o2[4], o3[4];
      {
        FT L1[4], L2[4], L3[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = (NQ * j + i) * Nv + v;
          L1[i] = sL[16 * Nv + q];
          L2[i] = sL[32 * Nv + q];
          L3[i] = sL[48 * Nv + q];
        }
        vec_lap(P, R, g, s, L1, L2, L3, P.div_damp, o1, o2, o3);
      }
      if (act) st_row(crow(BC_L4, v), o3);
      FT hd[4];
      {
        FT Ls[4], g1[4], g2[4], x1[4], x2[4], gu0[4], gu1[4], gu2[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) Ls[i] = sL[(NQ * j + i) * Nv + v];
        d1(P, Ls, g1);
        d2(R, Ls, g2);
        g.gu(gu0, gu1, gu2);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const FT y0 = gu0[i] * s.ir2, y1 = gu1[i] * s.ir2, y2 = gu2[i] * s.ir2;
          x1[i] = rho[i] * (y0 * g1[i] + y1 * g2[i]);
          x2[i] = rho[i] * (y1 * g1[i] + y2 * g2[i]);
        }
        wdiv(P, R, s, x1, x2, hd);
      }
      if (act) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = (NQ * j + i) * Nv + v;
          dnu.add(-(o1[i] * sT[16 * Nv + q] + o2[i] * sT[32 * Nv + q] + rpr * hd[i] * sT[48 * Nv + q]));
        }
      }
    }
    __syncthreads();
    // ---- D: face phase, forward and reverse (the cotangent of X follows from Tb and rho J)
    for (int k0 = 0; k0 < Nf; k0 += AD_LEVELS) {
      const int k = min(k0 + vl, Nf - 1);
      const bool act = k0 + vl < Nf;
      const bool inner = k > 0 && k < Nv;
      const FT r2 = P.levf[LF_R2 * Nf + k], dzf = P.levf[LF_DZ * Nf + k], rinv = P.levf[LF_RINV * Nf + k];
      const FT ir2f = P.levf[LF_IR2 * Nf + k], idzf = P.levf[LF_IDZ * Nf + k], g33 = P.levf[LF_G33 * Nf + k];
      FT u3[4], ta[4], tb[4];
      {
        FT W[4], Wu[4];
        g.w(W);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          u3[i] = inner ? sF[(NQ * j + i) * Nf + k] : FT(0);
          Wu[i] = W[i] * u3[i];
        }
        t2(R, Wu, tb);
        t1(P, Wu, ta);
      }
      // the levels below and above the face (both the adjacent level on a boundary face)
      const int va = k > 0 ? k - 1 : 0, vb = k < Nv ? k : Nv - 1;
      FT X1[4], X2[4], Cc1[4], Cc2[4], RJb[4], Cv1[4], Cv2[4], u3d[4], tab[4], tbb[4];
      {
        FT C1a[4], C1b[4], C2a[4], C2b[4], Ra[4], Rb[4], La[4], Lb[4];
        ld_row(crow(BC_C1, va), C1a);
        ld_row(crow(BC_C1, vb), C1b);
        ld_row(crow(BC_C2, va), C2a);
        ld_row(crow(BC_C2, vb), C2b);
        ld_row(crow(BC_RJ, va), Ra);
        ld_row(crow(BC_RJ, vb), Rb);
        ld_row(crow(BC_L4, va), La);
        ld_row(crow(BC_L4, vb), Lb);
        FT Jh[4], iJh[4], iW[4], fh1[4], fh2[4];
        g.row(HG_JH, Jh);
        g.row(HG_IJH, iJh);
        g.iw(iW);
        g.row(HG_FH1, fh1);
        g.row(HG_FH2, fh2);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int n = NQ * j + i;
          const int qa = n * Nv + va, qb = n * Nv + vb;
          const FT Jf = Jh[i] * r2 * dzf;
          const FT iJf = iJh[i] * ir2f * idzf, iWJf = iW[i] * iJf;
          const FT w1 = -tb[i] * iWJf, w2 = ta[i] * iWJf;
          FT cv1 = 0, cv2 = 0, cc1, cc2, l4, rJ;
          if (inner) {
            cv1 = -(sY[32 * Nv + qb] - sY[32 * Nv + qa]) * iJf;
            cv2 = (sY[16 * Nv + qb] - sY[16 * Nv + qa]) * iJf;
            cc1 = (C1a[i] + C1b[i]) / FT(2);
            cc2 = (C2a[i] + C2b[i]) / FT(2);
            l4 = gdiv(Ra[i] * La[i] + Rb[i] * Lb[i], Ra[i] + Rb[i]);
            rJ = (Ra[i] + Rb[i]) / FT(2);
          } else {
            cc1 = C1a[i];
            cc2 = C2a[i];
            l4 = La[i];
            rJ = Ra[i];
          }
          const FT fo1 = fh1[i] * rinv + cv1 + w1, fo2 = fh2[i] * rinv + cv2 + w2;
          const FT b3 = rJ * (u3[i] * g33);
          // X-cotangents from P3: t_i(v) = (X_i(v) + X_i(v+1)) / (2 rho J(v)) + ..., T_u_i -= t_i
          FT Xb1 = 0, Xb2 = 0;
          if (k >= 1) {
            const FT ia = grcp(FT(2) * Ra[i]);
            Xb1 -= sT[16 * Nv + qa] * ia;
            Xb2 -= sT[32 * Nv + qa] * ia;
          }
          if (k < Nv) {
            const FT ib = grcp(FT(2) * Rb[i]);
            Xb1 -= sT[16 * Nv + qb] * ib;
            Xb2 -= sT[32 * Nv + qb] * ib;
          }
          const FT T3b = sTf[n * Nf + k];
          const FT b3b = Jf * (fo2 * Xb1 - fo1 * Xb2);
          const FT fo1b = -Jf * b3 * Xb2 - Jf * cc2 * T3b;
          const FT fo2b = Jf * b3 * Xb1 + Jf * cc1 * T3b;
          X1[i] = Jf * (fo2 * b3);
          X2[i] = Jf * (-fo1 * b3);
          Cc1[i] = Jf * fo2 * T3b;
          Cc2[i] = -Jf * fo1 * T3b;
          RJb[i] = b3b * u3[i] * g33;
          Cv1[i] = inner ? fo1b * iJf : FT(0);
          Cv2[i] = inner ? fo2b * iJf : FT(0);
          if (act) dnu.add(-mul_rn(l4, T3b));
          u3d[i] = inner ? b3b * rJ * g33 : FT(0);
          // w1 = -tb iWJf, w2 = ta iWJf  ->  cotangents of tb, ta
          tbb[i] = -fo1b * iWJf;
          tab[i] = fo2b * iWJf;
        }
      }
      FT Wb[4], Wb2[4], U3b[4];
      d1(P, tab, Wb);
      d2(R, tbb, Wb2);
      {
        FT W[4];
        g.w(W);
#pragma unroll
        for (int i = 0; i < 4; ++i) U3b[i] = inner ? u3d[i] + W[i] * (Wb[i] + Wb2[i]) : FT(0);
      }
      if (act) {
        st_row(frow(BF_X1, k), X1);
        st_row(frow(BF_X2, k), X2);
        st_row(frow(BF_CC1, k), Cc1);
        st_row(frow(BF_CC2, k), Cc2);
        st_row(frow(BF_RJ, k), RJb);
        st_row(frow(BF_CV1, k), Cv1);
        st_row(frow(BF_CV2, k), Cv2);
        st_row(frow(BF_U3, k), U3b);
      }
    }
    __syncthreads();
    // ---- G: centre transpose (P3 and the face gathers, vorticity, hyperdiffusion,
    // horizontal dynamics, thermodynamics), intermediates dying group by group
    FT *yb = Ybc + (size_t)e * 64 * Nv, *lb = Lbc + (size_t)e * 64 * Nv;
    for (int v0 = 0; v0 < Nv; v0 += AD_LEVELS) {
      const int v = min(v0 + vs, Nv - 1);
      const bool act = v0 + vs < Nv;
      LevRow<FT> s;
      levrow(v, s);
      const FT idz = P.levc[LC_IDZ * Nv + v];
      const FT beta = P.levc[LC_BETA * Nv + v], spg = P.levc[LC_SPG * Nv + v];
      const int vm = v > 0 ? v - 1 : v, vp = v + 1 < Nv ? v + 1 : v;
      FT rhob[4], u1b[4], u2b[4], c1b[4], c2b[4], Kb[4], L4b[4];
      {
        FT Tu1b[4], Tu2b[4], RJv[4], RJb[4], omb[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = (NQ * j + i) * Nv + v;
          Tu1b[i] = sT[16 * Nv + q];
          Tu2b[i] = sT[32 * Nv + q];
        }
        ld_row(crow(BC_RJ, v), RJv);
        // P3: t_i = (X_i(v) + X_i(v+1)) / 2 / rho J + Cr_i, T_u_i -= t_i + beta u_i
        {
          FT Xa1[4], Xb1[4], Xa2[4], Xb2[4];
          ld_row(frow(BF_X1, v), Xa1);
          ld_row(frow(BF_X1, v + 1), Xb1);
          ld_row(frow(BF_X2, v), Xa2);
          ld_row(frow(BF_X2, v + 1), Xb2);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const FT iRJ = grcp(RJv[i]);
            const FT X1s = (Xa1[i] + Xb1[i]) / FT(2), X2s = (Xa2[i] + Xb2[i]) / FT(2);
            RJb[i] = -(X1s * (-Tu1b[i]) + X2s * (-Tu2b[i])) * iRJ * iRJ;
          }
        }
        // Cr1 = J (-a3 c2), Cr2 = J (a3 c1) with a3 = f^3 + w^3, w^3 = wcurl(u_h) recomputed
        {
          FT u1[4], u2[4], om[4], C1v[4], C2v[4], f3[4];
          {
            FT W[4], Wu1[4], Wu2[4], ta[4], tb[4];
            g.w(W);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              const int q = (NQ * j + i) * Nv + v;
              u1[i] = sY[16 * Nv + q];
              u2[i] = sY[32 * Nv + q];
              Wu1[i] = W[i] * u1[i];
              Wu2[i] = W[i] * u2[i];
            }
            t1(P, Wu2, ta);
            t2(R, Wu1, tb);
#pragma unroll
            for (int i = 0; i < 4; ++i) om[i] = (-ta[i] + tb[i]) * s.iWJ[i];
          }
          ld_row(crow(BC_C1, v), C1v);
          ld_row(crow(BC_C2, v), C2v);
          g.row(HG_F3, f3);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const FT a3 = f3[i] * idz + om[i];
            const FT t1b = -Tu1b[i], t2b = -Tu2b[i];
            omb[i] = s.J[i] * (C1v[i] * t2b - C2v[i] * t1b);
            c1b[i] = s.J[i] * a3 * t2b;
            c2b[i] = -s.J[i] * a3 * t1b;
            u1b[i] = -beta * Tu1b[i];
            u2b[i] = -beta * Tu2b[i];
            if (act) dal.add(-mul_rn(spg, u1[i] * Tu1b[i] + u2[i] * Tu2b[i]));
            Kb[i] = FT(0);
          }
        }
        // gathers from face v (this centre is its upper neighbour) and face v+1 (lower neighbour)
        {
          FT RJm[4], RJp[4], L4m[4], L4v[4], L4p[4];
          ld_row(crow(BC_RJ, vm), RJm);
          ld_row(crow(BC_RJ, vp), RJp);
          ld_row(crow(BC_L4, vm), L4m);
          ld_row(crow(BC_L4, v), L4v);
          ld_row(crow(BC_L4, vp), L4p);
          FT cc1l[4], cc1u[4], cc2l[4], cc2u[4], rjl[4], rju[4], cv1l[4], cv1u[4], cv2l[4], cv2u[4];
          ld_row(frow(BF_CC1, v), cc1l);
          ld_row(frow(BF_CC1, v + 1), cc1u);
          ld_row(frow(BF_CC2, v), cc2l);
          ld_row(frow(BF_CC2, v + 1), cc2u);
          ld_row(frow(BF_RJ, v), rjl);
          ld_row(frow(BF_RJ, v + 1), rju);
          ld_row(frow(BF_CV1, v), cv1l);
          ld_row(frow(BF_CV1, v + 1), cv1u);
          ld_row(frow(BF_CV2, v), cv2l);
          ld_row(frow(BF_CV2, v + 1), cv2u);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int n = NQ * j + i;
            // face cotangents of gK (-T3b on inner faces) and l4 (-nu T3b)
            const FT T3l = sTf[n * Nf + v], T3u = sTf[n * Nf + v + 1];
            const FT bl4l = -nu * T3l, bl4u = -nu * T3u;
            FT l4b = FT(0);
            if (v > 0) {
              const FT wa = RJm[i], wb = RJv[i], iws = grcp(wa + wb);
              const FT l4 = (wa * L4m[i] + wb * L4v[i]) * iws;
              c1b[i] += cc1l[i] / FT(2);
              c2b[i] += cc2l[i] / FT(2);
              Kb[i] += -T3l;
              l4b += bl4l * wb * iws;
              RJb[i] += bl4l * (L4v[i] - l4) * iws + rjl[i] / FT(2);
              u1b[i] += cv2l[i];
              u2b[i] -= cv1l[i];
            } else {
              c1b[i] += cc1l[i];
              c2b[i] += cc2l[i];
              l4b += bl4l;
              RJb[i] += rjl[i];
            }
            if (v + 1 < Nv) {
              const FT wa = RJv[i], wb = RJp[i], iws = grcp(wa + wb);
              const FT l4 = (wa * L4v[i] + wb * L4p[i]) * iws;
              c1b[i] += cc1u[i] / FT(2);
              c2b[i] += cc2u[i] / FT(2);
              Kb[i] -= -T3u;
              l4b += bl4u * wa * iws;
              RJb[i] += bl4u * (L4v[i] - l4) * iws + rju[i] / FT(2);
              u1b[i] -= cv2u[i];
              u2b[i] += cv1u[i];
            } else {
              c1b[i] += cc1u[i];
              c2b[i] += cc2u[i];
              l4b += bl4u;
              RJb[i] += rju[i];
            }
            L4b[i] = l4b;
            rhob[i] = s.J[i] * RJb[i];
          }
        }
        // vorticity: om = (-t1(W u2) + t2(W u1)) / WJ
        {
          FT tab[4], tbb[4], da[4], db[4], W[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            tab[i] = -omb[i] * s.iWJ[i];
            tbb[i] = omb[i] * s.iWJ[i];
          }
          d1(P, tab, da);
          d2(R, tbb, db);
          g.w(W);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            u2b[i] += W[i] * da[i];
            u1b[i] += W[i] * db[i];
          }
        }
      }
      // ---- hyperdiffusion: T_u -= nu o(L), T_rhoe -= nu_s wdiv(rho g^-1 grad L_s), o3 -> faces (L4)
      {
        FT o1b[4], o2b[4], L1b[4], L2b[4], L3b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = (NQ * j + i) * Nv + v;
          o1b[i] = -nu * sT[16 * Nv + q];
          o2b[i] = -nu * sT[32 * Nv + q];
        }
        vec_lap_t(P, R, g, s, o1b, o2b, L4b, P.div_damp, L1b, L2b, L3b);
        if (act) {
          FT o3[4];
          ld_row(crow(BC_L4, v), o3);
          FT dl = 0;  // sum L . Lb - o3 . L4b = sum (o1 o1b + o2 o2b), o_ib = -nu T_u_i
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int q = (NQ * j + i) * Nv + v;
            lb[16 * Nv + q] = tsc * L1b[i];
            lb[32 * Nv + q] = tsc * L2b[i];
            lb[48 * Nv + q] = tsc * L3b[i];
            dl += sL[16 * Nv + q] * L1b[i] + sL[32 * Nv + q] * L2b[i] + sL[48 * Nv + q] * L3b[i] - o3[i] * L4b[i];
          }
          dnu.add(mul_rn(dl, inu));
        }
      }
      {
        FT hdb[4], xb1[4], xb2[4], Ls[4], g1[4], g2[4], gb1[4], gb2[4], Lsb[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = (NQ * j + i) * Nv + v;
          hdb[i] = -nus * sT[48 * Nv + q];
          Ls[i] = sL[q];
        }
        wdiv_t(P, R, s, hdb, xb1, xb2);
        d1(P, Ls, g1);
        d2(R, Ls, g2);
        FT gu0[4], gu1[4], gu2[4];
        g.gu(gu0, gu1, gu2);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const FT rho = sY[(NQ * j + i) * Nv + v];
          const FT x0 = gu0[i] * s.ir2, x1 = gu1[i] * s.ir2, x2 = gu2[i] * s.ir2;
          rhob[i] += (x0 * g1[i] + x1 * g2[i]) * xb1[i] + (x1 * g1[i] + x2 * g2[i]) * xb2[i];
          gb1[i] = rho * (x0 * xb1[i] + x1 * xb2[i]);
          gb2[i] = rho * (x1 * xb1[i] + x2 * xb2[i]);
        }
        grad_t(P, R, gb1, gb2, Lsb);
        if (act) {
          FT dl = 0;  // sum Ls . Lsb = sum hd . hdb, hdb = -nu_s T_rhoe
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            lb[(NQ * j + i) * Nv + v] = tsc * Lsb[i];
            dl += Ls[i] * Lsb[i];
          }
          dnu.add(mul_rn(dl, inu));
        }
      }
      // ---- forward thermodynamics and the horizontal-dynamics transpose
      const FT Phi = P.levc[LC_PHI * Nv + v];
      FT rho[4], rhoe[4], K[4], c1[4], c2[4], h[4], Pi[4], thp[4], pH[4];
      ld_row(crow(BC_K, v), K);
      ld_row(crow(BC_C1, v), c1);
      ld_row(crow(BC_C2, v), c2);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int q = (NQ * j + i) * Nv + v;
        rho[i] = sY[q];
        rhoe[i] = sY[48 * Nv + q];
      }
      {
        ThermoRow<FT> th;
        thermo_row(P, rho, rhoe, K, Phi, P.lr4[v], th);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          h[i] = th.h[i];
          Pi[i] = th.Pi[i];
          if (HS) pH[i] = th.p[i];
        }
        vsub(th.thv, th.thvr, thp);
      }
      FT hb_[4], Pib[4], thpb[4], phirb[4];
      {
        // T_u_i = -(g_i + cp (thp b_i - Pi f_i) / 2), g = grad(K + Phi - Phi_r + cp thp Pi / 2),
        // b = grad Pi, f = grad thp
        FT Tu1b[4], Tu2b[4], b1[4], b2[4], f1[4], f2[4], x1[4], x2[4], x[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = (NQ * j + i) * Nv + v;
          Tu1b[i] = sT[16 * Nv + q];
          Tu2b[i] = sT[32 * Nv + q];
        }
        d1(P, Pi, b1);
        d2(R, Pi, b2);
        d1(P, thp, f1);
        d2(R, thp, f2);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          thpb[i] = -hc * (b1[i] * Tu1b[i] + b2[i] * Tu2b[i]);
          Pib[i] = hc * (f1[i] * Tu1b[i] + f2[i] * Tu2b[i]);
          x1[i] = -Tu1b[i];
          x2[i] = -Tu2b[i];
        }
        FT gb[4];  // cotangent of the fused gradient's argument
        grad_t(P, R, x1, x2, gb);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          x1[i] = -hc * thp[i] * Tu1b[i];
          x2[i] = -hc * thp[i] * Tu2b[i];
        }
        grad_t(P, R, x1, x2, x);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          Pib[i] += x[i];
          x1[i] = hc * Pi[i] * Tu1b[i];
          x2[i] = hc * Pi[i] * Tu2b[i];
        }
        grad_t(P, R, x1, x2, x);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const FT tpb = hc * gb[i];  // of th' Pi
          thpb[i] += x[i] + Pi[i] * tpb;
          Pib[i] += thp[i] * tpb;
          Kb[i] += gb[i];
          phirb[i] = -gb[i];
        }
      }
      {
        // T_rho = -dm, T_rhoe = -(dmh + h dm + F . grad h) / 2, dm = wdiv(F), dmh = wdiv(F h)
        FT F1[4], F2[4], dm[4], ha[4], hbv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          F1[i] = rho[i] * c1[i];
          F2[i] = rho[i] * c2[i];
        }
        wdiv(P, R, s, F1, F2, dm);
        d1(P, h, ha);
        d2(R, h, hbv);
        FT dmb[4], dmhb[4], hab[4], hbb[4], F1b[4], F2b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = (NQ * j + i) * Nv + v;
          const FT qq = sT[48 * Nv + q] / FT(2);
          dmb[i] = -sT[q] - h[i] * qq;
          dmhb[i] = -qq;
          hb_[i] = -dm[i] * qq;
          F1b[i] = -ha[i] * qq;
          F2b[i] = -hbv[i] * qq;
          hab[i] = -F1[i] * qq;
          hbb[i] = -F2[i] * qq;
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
        FT kvb[4], gu0[4], gu1[4], gu2[4], s2[4];
        g.gu(gu0, gu1, gu2);
        if (HS) g.row(HG_S2, s2);
        FT rbv[4], rebv[4], kbv[4];
        if (!HS) thermo_vjp_row(P, rho, rhoe, K, Phi, hb_, Pib, thpb, phirb, rbv, rebv, kbv);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = (NQ * j + i) * Nv + v;
          ThermoBar<FT> tb{};
          tb.h = hb_[i];
          tb.Pi = Pib[i];
          tb.thv = thpb[i];
          tb.thvr = -thpb[i];
          tb.phir = phirb[i];
          if (HS) {
            // Held-Suarez: T_rhoe -= E = cv_d k_T (p / R_d - rho T_eq), T_u -= k_f hf u,
            // hf = max(0, (p / MSLP - sigma_b) / (1 - sigma_b)); cotangents of p, rho and u_h
            const FT p = pH[i], c2l = FT(1) - s2[i];
            const FT xs = (p * P.hs_iMSLP - P.hs_sb) * P.hs_isb;
            const FT hf = fmax(FT(0), xs), dhf = xs > FT(0) ? P.hs_isb * P.hs_iMSLP : FT(0);
            const FT kT = P.hs_ka + P.hs_dk * hf * (c2l * c2l), dkT = P.hs_dk * (c2l * c2l) * dhf;
            const FT pr = p * P.hs_ip0, pk = gpow(pr, P.kappa);
            const FT A = P.hs_Teq - P.hs_dTy * s2[i] - P.hs_dthz * glog(pr) * c2l;
            const FT raw = A * pk;
            const FT Teq = fmax(P.hs_Tmin, raw);
            const FT dTeq = raw > P.hs_Tmin ? P.hs_ip0 * gdiv(pk, pr) * (P.kappa * A - P.hs_dthz * c2l) : FT(0);
            const FT Teb = sT[48 * Nv + q], Tu1b = sT[16 * Nv + q], Tu2b = sT[32 * Nv + q];
            const FT u1 = sY[16 * Nv + q], u2 = sY[32 * Nv + q];
            const FT dEdp = P.cvd * (dkT * (p / P.Rd - rho[i] * Teq) + kT * (FT(1) / P.Rd - rho[i] * dTeq));
            tb.p = -Teb * dEdp - P.hs_kf * dhf * (u1 * Tu1b + u2 * Tu2b);
            rhob[i] += Teb * P.cvd * kT * Teq;
            u1b[i] -= P.hs_kf * hf * Tu1b;
            u2b[i] -= P.hs_kf * hf * Tu2b;
          }
          FT rb = rbv[i], reb = rebv[i], kb = kbv[i];
          if (HS) thermo_vjp(P, rho[i], rhoe[i], K[i], Phi, tb, rb, reb, kb);
          const FT Kt = Kb[i] + kb;
          const FT x0 = gu0[i] * s.ir2, x1 = gu1[i] * s.ir2, x2 = gu2[i] * s.ir2;
          const FT o0 = tsc * (rhob[i] + rb), o1 = tsc * (u1b[i] + c1[i] * Kt + x0 * c1b[i] + x1 * c2b[i]);
          const FT o2 = tsc * (u2b[i] + c2[i] * Kt + x1 * c1b[i] + x2 * c2b[i]), o3 = tsc * reb;
          if (accum) {
            yb[q] += o0;
            yb[16 * Nv + q] += o1;
            yb[32 * Nv + q] += o2;
            yb[48 * Nv + q] += o3;
          } else {
            yb[q] = o0;
            yb[16 * Nv + q] = o1;
            yb[32 * Nv + q] = o2;
            yb[48 * Nv + q] = o3;
          }
          kvb[i] = Kt / FT(2);
        }
        st_row(sKvb + (size_t)v * NN + NQ * j, kvb);
      }
    }
    __syncthreads();
    // inner face k: the face-phase cotangent of u_3 and the K_v cotangents of levels k-1, k
    FT *fb = Ybf + (size_t)e * 16 * Nf;
    for (int k0 = 1; k0 < Nv; k0 += AD_LEVELS) {
      const int k = k0 + vl;
      if (k < Nv) {
        FT U3b[4], Km[4], Kp[4];
        ld_row(frow(BF_U3, k), U3b);
        ld_row(sKvb + (size_t)(k - 1) * NN + NQ * j, Km);
        ld_row(sKvb + (size_t)k * NN + NQ * j, Kp);
        const FT g33 = P.levf[LF_G33 * Nf + k];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int idx = (NQ * j + i) * Nf + k;
          const FT u3 = sF[idx];
          const FT o = tsc * (U3b[i] + Km[i] * u3 * g33 + Kp[i] * u3 * g33);
          if (accum) fb[idx] += o;
          else fb[idx] = o;
        }
      }
    }
    // overwrite: the boundary faces have no cotangent
    if (!accum && vl == 0) {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        fb[(NQ * j + i) * Nf] = FT(0);
        fb[(NQ * j + i) * Nf + Nv] = FT(0);
      }
    }
    // every thread is done with this element's slabs before they are refilled
    __syncthreads();
  }
  // parameter cotangents: warp sums, then the warps in a fixed order; one slot per CTA
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    dnu.add(dnu.xor_shfl(o, 32));
    dal.add(dal.xor_shfl(o, 32));
  }
  const int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red[warp] = dnu.value();
    red[AD_THREADS / 32 + warp] = dal.value();
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // accumulated over the launches of a reverse pass (zeroed by the host)
    double a = 0, c = 0;
    for (int w = 0; w < AD_THREADS / 32; ++w) {
      a += red[w];
      c += red[AD_THREADS / 32 + w];
    }
    dpar[2 * blockIdx.x] += (double)tsc * a;
    dpar[2 * blockIdx.x + 1] += (double)tsc * c;
  }
}

}  // namespace

template <class FT>
size_t passA_vjp_smem(int Nv) {
  return AvLayout<FT, false>(Nv, 1).total;
}
// Whether pass A^T can also take a further cotangent slab (shared memory).
template <class FT>
bool passA_vjp_add_fits(int Nv) {
  return AvLayout<FT, true>(Nv, 1).total <= (size_t)ad_dev().optin;
}
// Whether pass B^T stages the Laplacians and the tendency cotangent (they fit).
template <class FT>
bool passB_vjp_staged(int Nv) {
  return BvLayout<FT, false>(Nv, 1).total <= (size_t)ad_dev().optin;
}
template <class FT>
size_t passB_vjp_smem(int Nv) {
  return passB_vjp_staged<FT>(Nv) ? BvLayout<FT, false>(Nv, 1).total : BvLayout<FT, true>(Nv, 1).total;
}

template <class FT>
void configure_adjoint_se(int Nv) {
  (void)Nv;
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  // the dynamic limit is the opt-in maximum less the kernel's static shared memory
  cudaFuncAttributes fa{};
  cudaFuncGetAttributes(&fa, k_passA_vjp<FT, false>);
  cudaFuncSetAttribute(k_passA_vjp<FT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
  cudaFuncGetAttributes(&fa, k_passA_vjp<FT, true>);
  cudaFuncSetAttribute(k_passA_vjp<FT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
  auto raise = [&](auto kern) {
    cudaFuncGetAttributes(&fa, kern);
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
  };
  raise(k_passB_vjp<FT, false, false>);
  raise(k_passB_vjp<FT, true, false>);
  raise(k_passB_vjp<FT, false, true>);
  raise(k_passB_vjp<FT, true, true>);
}

template <class FT>
void launch_passA_vjp(const DevParams<FT> &P, const FT *Yc, const FT *Yf, const FT *Lb, FT *Ybc, FT *Ybf, int grid,
                      cudaStream_t s, const FT *Xbc, const FT *Xbf) {
  (void)grid;
  if (Xbc && Xbf) {
    const AdShape sh = ad_shape<AvLayout<FT, true>>(P.Nv, AdMinBlocks<FT>::value);
    const int g = std::max(1, std::min(P.Nh, ad_dev().nsm * sh.ctas));
    k_passA_vjp<FT, true><<<g, AD_THREADS, sh.smem, s>>>(P, sh.nbuf, Yc, Yf, Lb, Ybc, Ybf, Xbc, Xbf);
  } else {
    const AdShape sh = ad_shape<AvLayout<FT, false>>(P.Nv, AdMinBlocks<FT>::value);
    const int g = std::max(1, std::min(P.Nh, ad_dev().nsm * sh.ctas));
    k_passA_vjp<FT, false><<<g, AD_THREADS, sh.smem, s>>>(P, sh.nbuf, Yc, Yf, Lb, Ybc, Ybf, nullptr, nullptr);
  }
}
// grid: the number of parameter-partial slots (CTAs) the caller allocated.
template <class FT>
void launch_passB_vjp(const DevParams<FT> &P, const FT *Yc, const FT *Yf, const FT *L, const FT *Tbc, const FT *Tbf,
                      FT *Ybc, FT *Ybf, FT *Lb, double *dpar, int grid, bool accum, cudaStream_t s, FT tsc) {
  const bool staged = passB_vjp_staged<FT>(P.Nv);
  const AdShape sh = staged ? ad_shape<BvLayout<FT, false>>(P.Nv, AdMinBlocks<FT>::value)
                            : ad_shape<BvLayout<FT, true>>(P.Nv, AdMinBlocks<FT>::value);
  const int g = std::max(1, std::min({grid, P.Nh, ad_dev().nsm * sh.ctas}));
  const int ac = accum ? 1 : 0;
  if (staged) {
    if (P.hs) k_passB_vjp<FT, true, false><<<g, AD_THREADS, sh.smem, s>>>(P, sh.nbuf, Yc, Yf, L, Tbc, Tbf, Ybc, Ybf, Lb, dpar, ac, tsc);
    else k_passB_vjp<FT, false, false><<<g, AD_THREADS, sh.smem, s>>>(P, sh.nbuf, Yc, Yf, L, Tbc, Tbf, Ybc, Ybf, Lb, dpar, ac, tsc);
  } else {
    if (P.hs) k_passB_vjp<FT, true, true><<<g, AD_THREADS, sh.smem, s>>>(P, sh.nbuf, Yc, Yf, L, Tbc, Tbf, Ybc, Ybf, Lb, dpar, ac, tsc);
    else k_passB_vjp<FT, false, true><<<g, AD_THREADS, sh.smem, s>>>(P, sh.nbuf, Yc, Yf, L, Tbc, Tbf, Ybc, Ybf, Lb, dpar, ac, tsc);
  }
}

#define INST(FT)                                                                                             \
  template size_t passA_vjp_smem<FT>(int);                                                                   \
  template bool passA_vjp_add_fits<FT>(int);                                                                 \
  template size_t passB_vjp_smem<FT>(int);                                                                   \
  template void configure_adjoint_se<FT>(int);                                                               \
  template void launch_passA_vjp<FT>(const DevParams<FT> &, const FT *, const FT *, const FT *, FT *, FT *, int, \
                                     cudaStream_t, const FT *, const FT *);                                  \
  template void launch_passB_vjp<FT>(const DevParams<FT> &, const FT *, const FT *, const FT *, const FT *,      \
                                     const FT *, FT *, FT *, FT *, double *, int, bool, cudaStream_t, FT);
INST(float)
INST(double)
#undef INST

}  // namespace gb
