// Spectral-element slab kernels of the explicit tendency (remaining_tendency!).
//
// Persistent CTAs walk the elements.  For each element the Nq=4 GLL slab of
// all levels (state, DSSed Laplacians, per-node metric terms) is staged into
// shared memory by 1-D TMA bulk copies, double-buffered where shared memory
// allows so that the next element's slab streams in while the current one is
// computed; the finished slab leaves by a TMA bulk store.
//
// Thread mapping of the horizontal work: one thread per (level, row j),
// holding the four nodes n = 4 j + i of that row.  Derivatives along xi^1 are
// 4x4 matrix-vector products in registers (D from the constant bank);
// derivatives along xi^2 gather the other rows with shuffles inside the 4-lane
// group of the level.  Vertical (face/centre) operators read neighbouring
// levels from shared memory in a level-fastest mapping.
//
// pass A = prep_hyperdiffusion_tendency! (src/prognostic_equations/hyperdiffusion.jl:116-147):
//   L = (grad/curl Laplacian of u_bar, scalar Laplacian of s_d - s_d,r)
// pass B = horizontal_dynamics_tendency! (advection.jl:36-91)
//        + apply_hyperdiffusion_tendency! (hyperdiffusion.jl:247-307)
//        + explicit_vertical_advection_tendency! (advection.jl:205-290, deep branch)
//        + Rayleigh sponge on u_h (remaining_tendency.jl:119-166, rayleigh_sponge.jl:39-44)
#include <cstdlib>

#include "se_ops.cuh"

namespace gb {

namespace {

using namespace se;

constexpr int SE_THREADS = 256;          // 64 level slots x 4 rows per sweep
constexpr int SE_LEVELS = SE_THREADS / 4;

// TMA loads of one element's input slabs into buffer set b (thread 0 only).
template <class FT>
__device__ __forceinline__ void issue_slab(const DevParams<FT> &P, uint64_t *bar, int e, FT *sY, FT *sF, FT *sG,
                                           FT *sL, const FT *Yc, const FT *Yf, const FT *Lin) {
  const int Nv = P.Nv, Nf = P.Nf;
  const uint32_t by = uint32_t(sizeof(FT) * 64 * Nv), bf = uint32_t(sizeof(FT) * 16 * Nf);
  const uint32_t bg = uint32_t(sizeof(FT) * HG_N * 16);
  mbar_expect_tx(bar, by + bf + bg + (sL ? by : 0u));
  tma_load(sY, Yc + (size_t)e * 64 * Nv, by, bar);
  load_faces(sF, Yf, e, Nf, bar);
  tma_load(sG, P.hgeo + (size_t)e * HG_N * 16, bg, bar);
  if (sL) tma_load(sL, Lin + (size_t)e * 64 * Nv, by, bar);
}

__device__ __forceinline__ void init_bars(uint64_t *bar) {
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
}

// Start of one element iteration: prefetch the next element (double
// buffering) or load this one (single buffering), retire the previous
// output store, and wait for this element's slabs.  Returns false if a
// bounded wait gave up (every thread then leaves the element loop).
template <class T>
__device__ __forceinline__ T *pick(int b, T *p0, T *p1) { return b ? p1 : p0; }

template <class FT>
__device__ __forceinline__ bool begin_element(const DevParams<FT> &P, uint64_t *bar, int nbuf, int it, int e,
                                              FT *const (&sY)[2], FT *const (&sF)[2], FT *const (&sG)[2],
                                              FT *const (&sL)[2], bool withL, const FT *Yc, const FT *Yf,
                                              const FT *Lin, int &b) {
  b = nbuf == 2 ? (it & 1) : 0;
  if (threadIdx.x == 0) {
    if (nbuf == 2) {
      const int en = e + gridDim.x;
      const int o = b ^ 1;
      if (en < P.Nh)
        issue_slab<FT>(P, &bar[o], en, pick(o, sY[0], sY[1]), pick(o, sF[0], sF[1]), pick(o, sG[0], sG[1]),
                       withL ? pick(o, sL[0], sL[1]) : nullptr, Yc, Yf, Lin);
    } else if (it > 0) {
      issue_slab<FT>(P, &bar[0], e, sY[0], sF[0], sG[0], withL ? sL[0] : nullptr, Yc, Yf, Lin);
    }
    // the output slab this element writes was last stored two elements ago (double-buffered
    // output) or by the previous element
    if (nbuf == 2) tma_store_wait_read_1();
    else tma_store_wait_read();
  }
  const uint32_t parity = nbuf == 2 ? ((it >> 1) & 1) : (it & 1);
  const bool ok = mbar_wait_bounded(pick(b, &bar[0], &bar[1]), parity, P.status);
  return __syncthreads_and(ok) != 0;
}

// MB: the resident CTAs per SM the kernel is compiled for (its register cap): two in FP32 (a
// 128-register cap; one CTA computes while the other's slabs stream in) or three, one in FP64
// (whose register demand would spill heavily under the cap).
template <class FT, int MB>
__global__ void __launch_bounds__(SE_THREADS, MB) k_passA(DevParams<FT> P, int nbuf, const FT *__restrict__ Yc,
                                                         const FT *__restrict__ Yf, FT *__restrict__ Lout) {
  extern __shared__ __align__(128) unsigned char sm[];
  const int Nv = P.Nv;
  const int Nf = P.Nf, FR = face_rows<FT>(Nf);
  const PassALayout<FT> Lo(Nv, nbuf);
  FT *sYb[2] = {(FT *)(sm + Lo.y[0]), (FT *)(sm + Lo.y[1])};
  FT *sFb[2] = {(FT *)(sm + Lo.f[0]), (FT *)(sm + Lo.f[1])};
  FT *sGb[2] = {(FT *)(sm + Lo.g[0]), (FT *)(sm + Lo.g[1])};
  FT *sOb[2] = {(FT *)(sm + Lo.out[0]), (FT *)(sm + Lo.out[1])};
  uint64_t *bar = (uint64_t *)(sm + Lo.bar);
  init_bars(bar);
  int e = blockIdx.x;
  if (threadIdx.x == 0 && e < P.Nh) issue_slab<FT>(P, &bar[0], e, sYb[0], sFb[0], sGb[0], nullptr, Yc, Yf, nullptr);
  const int j = threadIdx.x & 3, vs = level_slot(threadIdx.x >> 2);
  Row<FT> R;
  R.init(P, j);
  for (int it = 0; e < P.Nh; ++it, e += gridDim.x) {
    int b;
    if (!begin_element<FT>(P, bar, nbuf, it, e, sYb, sFb, sGb, sGb, false, Yc, Yf, nullptr, b)) break;
    const FT *sY = pick(b, sYb[0], sYb[1]), *sF = pick(b, sFb[0], sFb[1]), *sG = pick(b, sGb[0], sGb[1]);
    FT *sO = pick(b, sOb[0], sOb[1]);
    RowGeo<FT> g;
    g.load(sG, P, j);
    for (int v0 = 0; v0 < Nv; v0 += SE_LEVELS) {
      const int v = min(v0 + vs, Nv - 1);
      const bool act = v0 + vs < Nv;
      LevRow<FT> s;
      s.set(g, P.levc[LC_R2 * Nv + v], P.levc[LC_IR2 * Nv + v], P.levc[LC_DZ * Nv + v], P.levc[LC_IDZ * Nv + v]);
      const FT Phi = P.levc[LC_PHI * Nv + v];
      const Lev4<FT> rl = P.lr4[v];
      const FT g3a = P.levf[LF_G33 * Nf + v], g3b = P.levf[LF_G33 * Nf + v + 1];
      FT u1[4], u2[4], ub3[4], sd[4], K[4];
      {
        FT rho[4], rhoe[4], fa[4], fb[4], t[4], c1[4], c2[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int n = NQ * j + i;
          const int q = n * Nv + v;
          rho[i] = sY[q];
          rhoe[i] = sY[48 * Nv + q];
          u1[i] = sY[16 * Nv + q];
          u2[i] = sY[32 * Nv + q];
          // u_3 of the faces below and above (0 on the boundary faces)
          fa[i] = v == 0 ? FT(0) : sF[fslot(n, v, Nf, FR)];
          fb[i] = v + 1 == Nv ? FT(0) : sF[fslot(n, v + 1, Nf, FR)];
        }
        // u_bar_3 = I^c(u_3); CT12(u_h) with the level's g^ij = r^-2 g^ij(surface); K
        vadd(fa, fb, ub3);
        vmuls(ub3, FT(0.5), ub3);
        vmul(g.gu1, u2, t);
        vfma(g.gu0, u1, t, t);
        vmuls(t, s.ir2, c1);
        vmul(g.gu2, u2, t);
        vfma(g.gu1, u1, t, t);
        vmuls(t, s.ir2, c2);
        FT kv2[4];
        vmuls(fb, g3b, kv2);
        vmul(fb, kv2, kv2);
        vmuls(fa, g3a, t);
        vfma(fa, t, kv2, kv2);
        vmul(u2, c2, t);
        vfma(u1, c1, t, t);
        vfmas(kv2, FT(0.5), t, K);
        vmuls(K, FT(0.5), K);
        // s_d - s_d,r = cp_d (T - T_r) + (Phi - Phi_r)
        ThermoRow<FT> th;
        thermo_row(P, rho, rhoe, K, Phi, rl, th);
        vsub(th.T, th.Tr, t);
        vfmas(t, P.cpd, th.phid, sd);
      }
      FT o1[4], o2[4], o3[4];
      vec_lap(P, R, g, s, u1, u2, ub3, FT(1), o1, o2, o3);
      FT g1[4], g2[4], x1[4], x2[4], Ls[4];
      d1(P, sd, g1);
      d2(R, sd, g2);
      {
        FT t[4];
        vmul(g.gu1, g2, t);
        vfma(g.gu0, g1, t, t);
        vmuls(t, s.ir2, x1);
        vmul(g.gu2, g2, t);
        vfma(g.gu1, g1, t, t);
        vmuls(t, s.ir2, x2);
      }
      wdiv(P, R, s, x1, x2, Ls);
      if (act) {
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
      tma_store(Lout + (size_t)e * 64 * Nv, sO, uint32_t(sizeof(FT) * 64 * Nv));
      tma_store_commit();
    }
  }
  if (threadIdx.x == 0) tma_store_wait_all();
}

template <class FT>
struct alignas(16) V16 {
  FT v[16 / sizeof(FT)];
};

// out = U + c_3 T + sum_j c_j T_j over one slab of n values in 16-byte vectors
// (T in shared memory, overwritten; U and the T_j at offset off in global memory).  Vector i
// of the slab sits at shared-memory vector i + (i / rowv) padv: the padded face slab (rowv
// vectors per node row, padv vectors of padding after each); rowv = n / E, padv = 0 for the
// unpadded centre slab.
template <class FT>
__device__ __forceinline__ void fin_combine(FT *sT, const FT *U, const FT *const (&Tj)[3], const FinArgs<FT> &F,
                                            size_t off, int n, int rowv, int padv) {
  constexpr int E = 16 / sizeof(FT);
  V16<FT> *s = reinterpret_cast<V16<FT> *>(sT);
  const V16<FT> *u = reinterpret_cast<const V16<FT> *>(U + off);
#pragma unroll 2
  for (int i = threadIdx.x; i < n / E; i += SE_THREADS) {
    V16<FT> r = u[i];
    const int si = i + (i / rowv) * padv;
    const V16<FT> t = s[si];
#pragma unroll
    for (int k = 0; k < E; ++k) r.v[k] += F.c[3] * t.v[k];
#pragma unroll
    for (int q = 0; q < 3; ++q)
      if (Tj[q]) {
        const V16<FT> a = reinterpret_cast<const V16<FT> *>(Tj[q] + off)[i];
#pragma unroll
        for (int k = 0; k < E; ++k) r.v[k] += F.c[q] * a.v[k];
      }
    s[si] = r;
  }
}

// HS: the Held-Suarez forcing is compiled in (a separate instantiation, so that
// the default kernel carries none of its registers or instructions).
// FIN: the slab written is the step's final combination (FinArgs) of the stage
// state Yc/Yf, earlier tendencies and this tendency, instead of the tendency.
template <class FT, bool HS, bool FIN, int MB>
__global__ void __launch_bounds__(SE_THREADS, MB) k_passB(DevParams<FT> P, int nbuf, const FT *__restrict__ Yc,
                                                         const FT *__restrict__ Yf, const FT *__restrict__ Lin,
                                                         FT *__restrict__ Tc, FT *__restrict__ Tf, FinArgs<FT> F) {
  extern __shared__ __align__(128) unsigned char sm[];
  const int Nv = P.Nv, Nf = P.Nf, FR = face_rows<FT>(Nf);
  const PassBLayout<FT> Lo(Nv, nbuf);
  auto at = [&](const size_t (&off)[2], int b) { return (FT *)(sm + (b ? off[1] : off[0])); };
  FT *sS = (FT *)(sm + Lo.s), *sX1 = (FT *)(sm + Lo.x1), *sX2 = (FT *)(sm + Lo.x2), *sW = (FT *)(sm + Lo.w);
  uint64_t *bar = (uint64_t *)(sm + Lo.bar);
  const uint32_t by = uint32_t(sizeof(FT) * 64 * Nv), bf = uint32_t(sizeof(FT) * 16 * Nf);
  const uint32_t bg = uint32_t(sizeof(FT) * HG_N * 16);
  auto issue = [&](int b, int e) {
    uint64_t *bb = b ? &bar[1] : &bar[0];
    mbar_expect_tx(bb, 2 * by + bf + bg);
    tma_load(at(Lo.y, b), Yc + (size_t)e * 64 * Nv, by, bb);
    load_faces(at(Lo.f, b), Yf, e, Nf, bb);
    tma_load(at(Lo.g, b), P.hgeo + (size_t)e * HG_N * 16, bg, bb);
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
  // the thread's row of scratch field f at level (or face) v
  auto row = [&](FT *base, int f, int v) { return base + ((size_t)f * Nv + v) * NN + NQ * j; };
  Row<FT> R;
  R.init(P, j);
  for (int it = 0; e < P.Nh; ++it, e += gridDim.x) {
    // the tendency overwrites this element's slabs: the next element is prefetched after the
    // centre phase (slab_prefetch below)
    int b;
    if (!slab_begin_deferred(bar, nbuf, it, e, P.status, issue, b)) break;
    if (FIN && threadIdx.x == 0) {
      // the final combination's other operands, into L2 while the tendency is computed
      bulk_prefetch_l2(Yc + (size_t)e * 64 * Nv, by);
      bulk_prefetch_l2(Yf + (size_t)e * 16 * Nf, bf);
      for (int q = 0; q < 3; ++q)
        if (F.te_c[q]) {
          bulk_prefetch_l2(F.te_c[q] + (size_t)e * 64 * Nv, by);
          bulk_prefetch_l2(F.te_f[q] + (size_t)e * 16 * Nf, bf);
        }
    }
    // the tendency overwrites the state and face slabs in place: each entry is
    // written by the thread that read it, after its last read
    FT *sY = at(Lo.y, b), *sF = at(Lo.f, b);
    const FT *sG = at(Lo.g, b), *sL = at(Lo.lap, b);
    FT *sO = sY, *sOf = sF;
    const SlabGeo<FT> g{sG + NQ * j, sW + NQ * j};
    // ---- P1: centre-level horizontal work, ordered so that each group of
    // intermediate fields dies before the next is formed; per-level results
    // go to the level-major scratch rows for the face pass
    for (int v0 = 0; v0 < Nv; v0 += SE_LEVELS) {
      const int v = min(v0 + vs, Nv - 1);
      const bool act = v0 + vs < Nv;
      const FT idz = P.levc[LC_IDZ * Nv + v];
      const FT Phi = P.levc[LC_PHI * Nv + v], beta = P.levc[LC_BETA * Nv + v];
      const Lev4<FT> rl = P.lr4[v];
      const FT g3a = P.levf[LF_G33 * Nf + v], g3b = P.levf[LF_G33 * Nf + v + 1];
      LevRow<FT> s;
      {
        FT Jh[4], iJh[4], W[4], iW[4];
        g.row(HG_JH, Jh);
        g.row(HG_IJH, iJh);
        g.w(W);
        g.iw(iW);
        s.set_rows(Jh, iJh, W, iW, P.levc[LC_R2 * Nv + v], P.levc[LC_IR2 * Nv + v], P.levc[LC_DZ * Nv + v], idz);
      }
      // Q: the u_h tendency less the face cross products (added in P3)
      FT rho[4], h[4], Pi[4], thp[4], gg[4], F1[4], F2[4], Q1[4], Q2[4];
      FT hsk[4] = {0, 0, 0, 0};  // Held-Suarez drag rate k_f max(0, (sigma - sigma_b) / (1 - sigma_b))
      {
        FT u1[4], u2[4], c1[4], c2[4], K[4], phid[4];
        {
          FT gu0[4], gu1[4], gu2[4], s2[4], rhoe[4], fa[4], fb[4], t[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int n = NQ * j + i;
            const int q = n * Nv + v;
            rho[i] = sY[q];
            u1[i] = sY[16 * Nv + q];
            u2[i] = sY[32 * Nv + q];
            rhoe[i] = sY[48 * Nv + q];
            // u_3 of the faces below and above (0 on the boundary faces)
            fa[i] = v == 0 ? FT(0) : sF[fslot(n, v, Nf, FR)];
            fb[i] = v + 1 == Nv ? FT(0) : sF[fslot(n, v + 1, Nf, FR)];
          }
          // CT12(u_h) = g^ij u_j with the level's g^ij = r^-2 g^ij(surface)
          g.gu(gu0, gu1, gu2);
          vmul(gu1, u2, t);
          vfma(gu0, u1, t, t);
          vmuls(t, s.ir2, c1);
          vmul(gu2, u2, t);
          vfma(gu1, u1, t, t);
          vmuls(t, s.ir2, c2);
          // K = (u_h . CT12(u_h) + I^c(u_3 u^3)) / 2, I^c(u_3 u^3) = (fa^2 g33_a + fb^2 g33_b) / 2
          FT kv2[4];
          vmuls(fb, g3b, kv2);
          vmul(fb, kv2, kv2);
          vmuls(fa, g3a, t);
          vfma(fa, t, kv2, kv2);
          vmul(u2, c2, t);
          vfma(u1, c1, t, t);
          vfmas(kv2, FT(0.5), t, K);
          vmuls(K, FT(0.5), K);
          if (HS) g.row(HG_S2, s2);
          ThermoRow<FT> th4;
          thermo_row(P, rho, rhoe, K, Phi, rl, th4);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            h[i] = th4.h[i];
            Pi[i] = th4.Pi[i];
            phid[i] = th4.phid[i];
          }
          vsub(th4.thv, th4.thvr, thp);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int q = (NQ * j + i) * Nv + v;
            if (HS) {
              Thermo<FT> th;
              th.p = th4.p[i];
              // Held-Suarez forcing (held_suarez.jl:98-141, 203-225, 279-295), flat surface:
              // sigma = p / MSLP; rho e_tot relaxes with -cv_d k_T rho (p / (rho R_d) - T_eq)
              const FT c2l = FT(1) - s2[i];
              const FT hf = fmax(FT(0), (th.p * P.hs_iMSLP - P.hs_sb) * P.hs_isb);
              const FT kT = P.hs_ka + P.hs_dk * hf * (c2l * c2l);
              const FT pr = th.p * P.hs_ip0;
              const FT Teq =
                  fmax(P.hs_Tmin, (P.hs_Teq - P.hs_dTy * s2[i] - P.hs_dthz * glog(pr) * c2l) * gpow(pr, P.kappa));
              hsk[i] = P.hs_kf * hf;
              // parked in the (already read) rho e_tot entry of the slab until the tendency is written
              if (act) sY[48 * Nv + q] = kT * rho[i] * (th.p / (rho[i] * P.Rd) - Teq) * P.cvd;
            }
          }
          // grad(K + Phi - Phi_r) and (cp_d / 2) grad(th' Pi) taken as one gradient
          vmul(thp, Pi, t);
          vadd(K, phid, gg);
          vfmas(t, P.cpd * FT(0.5), gg, gg);
        }
        // vorticity w^3 = wcurl(u_h); (f^3 + w^3) x CT12(u) -> C12, and the sponge
        FT om[4];
        {
          FT W[4], Wu1[4], Wu2[4], ta[4], tb[4];
          g.w(W);
          vmul(W, u1, Wu1);
          vmul(W, u2, Wu2);
          t1(P, Wu2, ta);
          t2(R, Wu1, tb);
          vsub(tb, ta, om);
          vmul(om, s.iWJ, om);
        }
        FT f3[4], rJ[4], a3J[4], damp[4];
        g.row(HG_F3, f3);
        vfmas(f3, idz, om, a3J);            // f^3 + w^3
        vmul(a3J, s.J, a3J);                // J (f^3 + w^3)
#pragma unroll
        for (int i = 0; i < 4; ++i) damp[i] = HS ? beta + hsk[i] : beta;  // sponge (+ Held-Suarez drag)
        // Q1 = J a3 c2 - damp u1, Q2 = -J a3 c1 - damp u2
        vmul(damp, u1, Q1);
        vmuls(Q1, FT(-1), Q1);
        vfma(a3J, c2, Q1, Q1);
        vmul(a3J, c1, Q2);
        vfma(damp, u2, Q2, Q2);
        vmuls(Q2, FT(-1), Q2);
        vmul(rho, c1, F1);
        vmul(rho, c2, F2);
        vmul(rho, s.J, rJ);
        if (act) {
          st_row(row(sS, SB_C1, v), c1);
          st_row(row(sS, SB_C2, v), c2);
          st_row(row(sS, SB_K, v), K);
          st_row(row(sS, SB_RJ, v), rJ);
        }
      }
      // rho: -wdiv(rho u); rho e_tot: -split_div(rho u, h)
      FT Trhoe[4];
      {
        FT G1[4], G2[4], dm[4], dmh[4], ha[4], hb[4];
        vmul(F1, h, G1);
        vmul(F2, h, G2);
        wdiv(P, R, s, F1, F2, dm);
        wdiv(P, R, s, G1, G2, dmh);
        d1(P, h, ha);
        d2(R, h, hb);
        // T_rhoe = -(wdiv(F h) + h wdiv(F) + F . grad h) / 2
        vmul(F2, hb, Trhoe);
        vfma(F1, ha, Trhoe, Trhoe);
        vfma(h, dm, Trhoe, Trhoe);
        vadd(dmh, Trhoe, Trhoe);
        vmuls(Trhoe, FT(-0.5), Trhoe);
        if (act) {
#pragma unroll
          for (int i = 0; i < 4; ++i) sO[(NQ * j + i) * Nv + v] = -dm[i];
        }
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
        FT t[4];
        vmul(Pi, f1, t);
        vmuls(t, FT(-1), t);
        vfma(thp, b1, t, t);
        vfmas(t, P.cpd * FT(0.5), a1, t);
        vsub(Q1, t, Q1);
        vmul(Pi, f2, t);
        vmuls(t, FT(-1), t);
        vfma(thp, b2, t, t);
        vfmas(t, P.cpd * FT(0.5), a2, t);
        vsub(Q2, t, Q2);
      }
      // hyperdiffusion: nu (div_damp C123(wgrad div L) - C123(wcurl C123(curl L)))
      {
        FT L1[4], L2[4], L3[4], o1[4], o2[4], o3[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = (NQ * j + i) * Nv + v;
          L1[i] = sL[16 * Nv + q];
          L2[i] = sL[32 * Nv + q];
          L3[i] = sL[48 * Nv + q];
        }
        vec_lap(P, R, g, s, L1, L2, L3, P.div_damp, o1, o2, o3);
        vfmas(o1, -P.nu_v, Q1, Q1);
        vfmas(o2, -P.nu_v, Q2, Q2);
        if (act) {
          st_row(row(sS, SB_L4, v), o3);
          st_row(row(sS, SB_Q1, v), Q1);
          st_row(row(sS, SB_Q2, v), Q2);
        }
      }
      {
        FT Ls[4], g1[4], g2[4], x1[4], x2[4], hd[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) Ls[i] = sL[(NQ * j + i) * Nv + v];
        d1(P, Ls, g1);
        d2(R, Ls, g2);
        {
          // rho g^ij d_j L_s with the level's g^ij = r^-2 g^ij(surface)
          FT gu0[4], gu1[4], gu2[4], rr[4];
          g.gu(gu0, gu1, gu2);
          vmuls(rho, s.ir2, rr);
          vcontract(gu0, gu1, g1, g2, rr, x1);
          vcontract(gu1, gu2, g1, g2, rr, x2);
        }
        wdiv(P, R, s, x1, x2, hd);
        if (act) {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int q = 48 * Nv + (NQ * j + i) * Nv + v;
            const FT t = Trhoe[i] - P.nu_s * hd[i];
            sO[q] = HS ? t - sO[q] : t;
          }
        }
      }
    }
    __syncthreads();
    slab_prefetch(nbuf, b, e, P.Nh, issue);
    // ---- P2: face-level work (f^12 + w^12, cross products, u_3 tendency)
    for (int k0 = 0; k0 < Nf; k0 += SE_LEVELS) {
      // faces in level_slot order, as the centre levels: the face slab reads are then free of
      // bank conflicts (its padded rows) and so are the row-vector scratch accesses
      const int k = min(k0 + vs, Nf - 1);
      const bool act = k0 + vs < Nf;
      const bool inner = k > 0 && k < Nv;
      const FT r2 = P.levf[LF_R2 * Nf + k], dzf = P.levf[LF_DZ * Nf + k], rinv = P.levf[LF_RINV * Nf + k];
      const FT ir2f = P.levf[LF_IR2 * Nf + k], idzf = P.levf[LF_IDZ * Nf + k], g33 = P.levf[LF_G33 * Nf + k];
      FT Wu[4], u3[4];
      {
        FT W[4];
        g.w(W);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          u3[i] = inner ? sF[j * FR + i * Nf + k] : FT(0);
          Wu[i] = W[i] * u3[i];
        }
      }
      FT ta[4], tb[4];
      t2(R, Wu, tb);
      t1(P, Wu, ta);
      // the levels below and above the face (both the adjacent level on a boundary face)
      const int va = k > 0 ? k - 1 : 0, vb = k < Nv ? k : Nv - 1;
      if (act) {
        FT C1a[4], C1b[4], C2a[4], C2b[4], Ka[4], Kb[4], Ra[4], Rb[4], La[4], Lb[4];
        ld_row(row(sS, SB_C1, va), C1a);
        ld_row(row(sS, SB_C1, vb), C1b);
        ld_row(row(sS, SB_C2, va), C2a);
        ld_row(row(sS, SB_C2, vb), C2b);
        ld_row(row(sS, SB_K, va), Ka);
        ld_row(row(sS, SB_K, vb), Kb);
        ld_row(row(sS, SB_RJ, va), Ra);
        ld_row(row(sS, SB_RJ, vb), Rb);
        ld_row(row(sS, SB_L4, va), La);
        ld_row(row(sS, SB_L4, vb), Lb);
        FT Jh[4], iJh[4], iW[4], fh1[4], fh2[4];
        g.row(HG_JH, Jh);
        g.row(HG_IJH, iJh);
        g.iw(iW);
        g.row(HG_FH1, fh1);
        g.row(HG_FH2, fh2);
        // face Jacobian, its inverse and the weak-curl weight of the face
        FT Jf[4], iJf[4], iWJf[4], w1[4], w2[4];
        vmuls(Jh, r2 * dzf, Jf);
        vmuls(iJh, ir2f * idzf, iJf);
        vmul(iW, iJf, iWJf);
        vmul(tb, iWJf, w1);
        vmuls(w1, FT(-1), w1);
        vmul(ta, iWJf, w2);
        FT cv1[4] = {0, 0, 0, 0}, cv2[4] = {0, 0, 0, 0}, gK[4] = {0, 0, 0, 0}, cc1[4], cc2[4], l4[4], rJ[4];
        if (inner) {
          // u_h of the levels below and above (not yet overwritten: P3 writes them)
          FT a1[4], b1[4], a2[4], b2[4], num[4], den[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int n = NQ * j + i;
            const int qa = n * Nv + va, qb = n * Nv + vb;
            a1[i] = sY[16 * Nv + qa];
            b1[i] = sY[16 * Nv + qb];
            a2[i] = sY[32 * Nv + qa];
            b2[i] = sY[32 * Nv + qb];
          }
          vsub(a2, b2, cv1);
          vmul(cv1, iJf, cv1);   // -(d u_2 / d xi^3) / J_f
          vsub(b1, a1, cv2);
          vmul(cv2, iJf, cv2);   // (d u_1 / d xi^3) / J_f
          vadd(C1a, C1b, cc1);
          vmuls(cc1, FT(0.5), cc1);
          vadd(C2a, C2b, cc2);
          vmuls(cc2, FT(0.5), cc2);
          vsub(Kb, Ka, gK);
          vmul(Rb, Lb, num);
          vfma(Ra, La, num, num);
          vadd(Ra, Rb, den);
#pragma unroll
          for (int i = 0; i < 4; ++i) l4[i] = gdiv(num[i], den[i]);
          vmuls(den, FT(0.5), rJ);
        } else {
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            cc1[i] = C1a[i];
            cc2[i] = C2a[i];
            l4[i] = La[i];
            rJ[i] = Ra[i];
          }
        }
        // (f^12 + w^12) on the face, the u_3 tendency and the face cross products
        FT fo1[4], fo2[4], b3[4], t[4], T3[4], X1[4], X2[4];
        vfmas(fh1, rinv, cv1, fo1);
        vadd(fo1, w1, fo1);
        vfmas(fh2, rinv, cv2, fo2);
        vadd(fo2, w2, fo2);
        FT u3g[4];
        vmuls(u3, g33, u3g);
        vmul(rJ, u3g, b3);
        vmul(fo2, cc1, t);
        vmuls(t, FT(-1), t);
        vfma(fo1, cc2, t, t);
        vfma(Jf, t, gK, t);
        vmuls(l4, -P.nu_v, T3);
        vsub(T3, t, T3);
        vmul(fo2, b3, X1);
        vmul(Jf, X1, X1);
        vmul(fo1, b3, X2);
        vmul(Jf, X2, X2);
        vmuls(X2, FT(-1), X2);
#pragma unroll
        for (int i = 0; i < 4; ++i) sOf[j * FR + i * Nf + k] = T3[i];
        st_row(sX1 + (size_t)k * NN + NQ * j, X1);
        st_row(sX2 + (size_t)k * NN + NQ * j, X2);
      }
    }
    __syncthreads();
    // ---- P3: centre u_h part of the face cross products (the sponge is in Q)
    for (int v0 = 0; v0 < Nv; v0 += SE_LEVELS) {
      const int v = v0 + vs;
      if (v < Nv) {
        FT Xa1[4], Xb1[4], Xa2[4], Xb2[4], rJ[4], Q1[4], Q2[4];
        ld_row(sX1 + (size_t)v * NN + NQ * j, Xa1);
        ld_row(sX1 + (size_t)(v + 1) * NN + NQ * j, Xb1);
        ld_row(sX2 + (size_t)v * NN + NQ * j, Xa2);
        ld_row(sX2 + (size_t)(v + 1) * NN + NQ * j, Xb2);
        ld_row(row(sS, SB_RJ, v), rJ);
        ld_row(row(sS, SB_Q1, v), Q1);
        ld_row(row(sS, SB_Q2, v), Q2);
        FT irJ[4], t1v[4], t2v[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) irJ[i] = grcp(rJ[i]);
        vadd(Xa1, Xb1, t1v);
        vmul(t1v, irJ, t1v);
        vfmas(t1v, FT(-0.5), Q1, t1v);
        vadd(Xa2, Xb2, t2v);
        vmul(t2v, irJ, t2v);
        vfmas(t2v, FT(-0.5), Q2, t2v);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int q = (NQ * j + i) * Nv + v;
          sO[16 * Nv + q] = t1v[i];
          sO[32 * Nv + q] = t2v[i];
        }
      }
    }
    if (FIN) {
      __syncthreads();
      constexpr int E = 16 / sizeof(FT);
      fin_combine<FT>(sO, Yc, F.te_c, F, (size_t)e * 64 * Nv, 64 * Nv, 64 * Nv / E, 0);
      fin_combine<FT>(sOf, Yf, F.te_f, F, (size_t)e * 16 * Nf, 16 * Nf, 4 * Nf / E, (FR - 4 * Nf) / E);
      __syncthreads();
      // impenetrable filter: u_3 = 0 on the bottom and top faces (thread t < 32: node t / 2)
      if (threadIdx.x < 32) sOf[fslot(threadIdx.x >> 1, (threadIdx.x & 1) ? Nv : 0, Nf, FR)] = FT(0);
    }
    fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      tma_store(Tc + (size_t)e * 64 * Nv, sO, by);
      store_faces(Tf, sOf, e, Nf);
      tma_store_commit();
    }
  }
  if (threadIdx.x == 0) tma_store_wait_all();
}

struct SeLaunch {
  int nsm = 0, optin = 0, per_sm = 0;
};
// The device attributes the slab launches need, read once (a function-local
// static: its initialisation is thread-safe); every device of one process is
// taken to be the same GPU model.
const SeLaunch &se_dev() {
  static const SeLaunch d = [] {
    SeLaunch x;
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

// Buffering and resident CTAs per SM of a slab kernel compiled for `ctas` resident CTAs (1 KB
// per CTA is reserved by the hardware): double buffering if that many such CTAs fit, else
// single buffering at that many, else one double- or single-buffered CTA.
struct SeShape {
  int nbuf, ctas;
  size_t smem;
};
template <class FT, class L>
SeShape se_shape(int Nv, int ctas) {
  const size_t two = L(Nv, 2).total, one = L(Nv, 1).total, per_sm = (size_t)se_dev().per_sm;
  if (ctas >= 2) {
    if (ctas * (two + 1024) <= per_sm) return {2, ctas, two};
    if (ctas * (one + 1024) <= per_sm) return {1, ctas, one};
  }
  if (two <= (size_t)se_dev().optin) return {2, 1, two};
  return {1, 1, one};
}

// Resident CTAs per SM of the FP32 slab kernels: two (a 128-register cap) by default; three (an
// 85-register cap, single-buffered slabs) with GBDYCORE_SE_CTAS=3.
int se_ctas_env() {
  static const int v = [] {
    const char *e = getenv("GBDYCORE_SE_CTAS");
    return e && atoi(e) == 3 ? 3 : 2;
  }();
  return v;
}

}  // namespace

template <class FT>
size_t passA_smem(int Nv) { return PassALayout<FT>(Nv, 1).total; }
template <class FT>
size_t passB_smem(int Nv) { return PassBLayout<FT>(Nv, 1).total; }

// Raise the dynamic shared-memory limit of the slab kernels to the device's
// opt-in maximum once (contexts with different level counts may coexist).
template <class FT, int MB>
void configure_se_mb() {
  cudaFuncSetAttribute(k_passA<FT, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, se_dev().optin);
  cudaFuncSetAttribute(k_passB<FT, false, false, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, se_dev().optin);
  cudaFuncSetAttribute(k_passB<FT, true, false, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, se_dev().optin);
  cudaFuncSetAttribute(k_passB<FT, false, true, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, se_dev().optin);
  cudaFuncSetAttribute(k_passB<FT, true, true, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, se_dev().optin);
}
template <class FT>
void configure_se(int Nv) {
  (void)Nv;
  if constexpr (sizeof(FT) == 4) {
    configure_se_mb<FT, 2>();
    configure_se_mb<FT, 3>();
  } else {
    configure_se_mb<FT, 1>();
  }
}

template <class FT, int MB>
void launch_passA_mb(const DevParams<FT> &P, const FT *Yc, const FT *Yf, FT *L, cudaStream_t s) {
  const SeShape sh = se_shape<FT, PassALayout<FT>>(P.Nv, MB);
  const int grid = min(P.Nh, se_dev().nsm * sh.ctas);
  k_passA<FT, MB><<<grid, SE_THREADS, sh.smem, s>>>(P, sh.nbuf, Yc, Yf, L);
}
template <class FT>
void launch_passA(const DevParams<FT> &P, const FT *Yc, const FT *Yf, FT *L, cudaStream_t s) {
  if constexpr (sizeof(FT) == 4) {
    if (se_ctas_env() == 3) launch_passA_mb<FT, 3>(P, Yc, Yf, L, s);
    else launch_passA_mb<FT, 2>(P, Yc, Yf, L, s);
  } else {
    launch_passA_mb<FT, 1>(P, Yc, Yf, L, s);
  }
}
template <class FT, int MB>
void launch_passB_mb(const DevParams<FT> &P, const FT *Yc, const FT *Yf, const FT *L, FT *Tc, FT *Tf, cudaStream_t s,
                     const FinArgs<FT> *fin) {
  const SeShape sh = se_shape<FT, PassBLayout<FT>>(P.Nv, MB);
  const int grid = min(P.Nh, se_dev().nsm * sh.ctas);
  const FinArgs<FT> F = fin ? *fin : FinArgs<FT>{};
  if (fin) {
    if (P.hs) k_passB<FT, true, true, MB><<<grid, SE_THREADS, sh.smem, s>>>(P, sh.nbuf, Yc, Yf, L, Tc, Tf, F);
    else k_passB<FT, false, true, MB><<<grid, SE_THREADS, sh.smem, s>>>(P, sh.nbuf, Yc, Yf, L, Tc, Tf, F);
  } else {
    if (P.hs) k_passB<FT, true, false, MB><<<grid, SE_THREADS, sh.smem, s>>>(P, sh.nbuf, Yc, Yf, L, Tc, Tf, F);
    else k_passB<FT, false, false, MB><<<grid, SE_THREADS, sh.smem, s>>>(P, sh.nbuf, Yc, Yf, L, Tc, Tf, F);
  }
}
template <class FT>
void launch_passB(const DevParams<FT> &P, const FT *Yc, const FT *Yf, const FT *L, FT *Tc, FT *Tf, cudaStream_t s,
                  const FinArgs<FT> *fin) {
  if constexpr (sizeof(FT) == 4) {
    if (se_ctas_env() == 3) launch_passB_mb<FT, 3>(P, Yc, Yf, L, Tc, Tf, s, fin);
    else launch_passB_mb<FT, 2>(P, Yc, Yf, L, Tc, Tf, s, fin);
  } else {
    launch_passB_mb<FT, 1>(P, Yc, Yf, L, Tc, Tf, s, fin);
  }
}

#define INST(FT)                                                                                             \
  template size_t passA_smem<FT>(int);                                                                       \
  template size_t passB_smem<FT>(int);                                                                       \
  template void configure_se<FT>(int);                                                                       \
  template void launch_passA<FT>(const DevParams<FT> &, const FT *, const FT *, FT *, cudaStream_t);         \
  template void launch_passB<FT>(const DevParams<FT> &, const FT *, const FT *, const FT *, FT *, FT *, cudaStream_t, \
                                 const FinArgs<FT> *);
INST(float)
INST(double)
#undef INST

}  // namespace gb
