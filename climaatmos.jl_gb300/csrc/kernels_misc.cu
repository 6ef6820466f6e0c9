// DSS, final stage combination, boundary filter and compensated global sums.
#include "kernels.cuh"

namespace gb {

namespace {

constexpr int DSS_THREADS = 256;  // 8 groups per CTA, one warp per group

// Direct stiffness summation (Spaces.weighted_dss!, constrain_state.jl:59-64 and
// remaining_tendency.jl:18-21): each group of collocated element nodes gets the
// J-weighted average of its copies, summed in the fixed ascending copy order
// (deterministic, no atomics).  Centre block components: 0 scalar, 1-2 covariant
// horizontal vector (averaged in Cartesian components), 3 scalar.  One warp
// per group, lanes over levels.  Q5 (moist 0M): a fifth centre component,
// rho*q_tot, averaged as a scalar (element block stride 5 * 16 * Nv).
// Two levels per lane (v0 + lane and v0 + 32 + lane), so that each lane has
// two independent gathers in flight; per level the sums run in the same copy
// order as with one level per lane.  Every product and sum is an explicit
// fused multiply-add or rounded product, so the rounding does not depend on
// the compiler's contraction choices (the oracle's DSS does the same
// operations in the same order and matches bit for bit).
template <class FT, bool Q5 = false>
__global__ void __launch_bounds__(DSS_THREADS) k_dss(DevParams<FT> P, FT *__restrict__ C, FT *__restrict__ F) {
  constexpr int NFC = Q5 ? 5 : 4;
  const int lane = threadIdx.x & 31;
  const int g = blockIdx.x * (DSS_THREADS / 32) + (threadIdx.x >> 5);
  if (g >= P.ngroups) return;
  const int Nv = P.Nv, Nf = P.Nf;
  const int o0 = P.goff[g], o1 = P.goff[g + 1];
  if (C) {
    for (int v0 = 0; v0 < Nv; v0 += 64) {
      const int v[2] = {v0 + lane, v0 + 32 + lane};
      const bool ok[2] = {v[0] < Nv, v[1] < Nv};
      FT s0[2] = {0, 0}, s3[2] = {0, 0}, s4[2] = {0, 0}, X0[2] = {0, 0}, X1[2] = {0, 0}, X2[2] = {0, 0};
      for (int c = o0; c < o1; ++c) {
        const int idx = P.gcopy[c], e = idx >> 4, n = idx & 15;
        const FT w = P.gw[c];
        const FT *ec = P.econ + (size_t)idx * 6;
        const size_t b0 = ((size_t)e * NFC * NN + n) * Nv;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          if (!ok[h]) continue;
          const size_t b = b0 + v[h];
          s0[h] = fma(w, C[b], s0[h]);
          s3[h] = fma(w, C[b + 48 * Nv], s3[h]);
          if (Q5) s4[h] = fma(w, C[b + 64 * Nv], s4[h]);
          const FT u1 = C[b + 16 * Nv], u2 = C[b + 32 * Nv];
          X0[h] = fma(w, fma(u2, ec[3], mul_rn(u1, ec[0])), X0[h]);
          X1[h] = fma(w, fma(u2, ec[4], mul_rn(u1, ec[1])), X1[h]);
          X2[h] = fma(w, fma(u2, ec[5], mul_rn(u1, ec[2])), X2[h]);
        }
      }
      for (int c = o0; c < o1; ++c) {
        const int idx = P.gcopy[c], e = idx >> 4, n = idx & 15;
        const FT *eo = P.ecov + (size_t)idx * 6;
        const size_t b0 = ((size_t)e * NFC * NN + n) * Nv;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          if (!ok[h]) continue;
          const size_t b = b0 + v[h];
          C[b] = s0[h];
          C[b + 48 * Nv] = s3[h];
          if (Q5) C[b + 64 * Nv] = s4[h];
          C[b + 16 * Nv] = fma(eo[2], X2[h], fma(eo[1], X1[h], mul_rn(eo[0], X0[h])));
          C[b + 32 * Nv] = fma(eo[5], X2[h], fma(eo[4], X1[h], mul_rn(eo[3], X0[h])));
        }
      }
    }
  }
  if (F) {
    for (int k0 = 0; k0 < Nf; k0 += 64) {
      const int k[2] = {k0 + lane, k0 + 32 + lane};
      const bool ok[2] = {k[0] < Nf, k[1] < Nf};
      FT sf[2] = {0, 0};
      for (int c = o0; c < o1; ++c) {
        const FT w = P.gw[c];
        const size_t b0 = (size_t)P.gcopy[c] * Nf;
#pragma unroll
        for (int h = 0; h < 2; ++h)
          if (ok[h]) sf[h] = fma(w, F[b0 + k[h]], sf[h]);
      }
      for (int c = o0; c < o1; ++c) {
        const size_t b0 = (size_t)P.gcopy[c] * Nf;
#pragma unroll
        for (int h = 0; h < 2; ++h)
          if (ok[h]) F[b0 + k[h]] = sf[h];
      }
    }
  }
}

// Transpose of k_dss (the reverse pass of the DSS projection).  The forward
// map gives every copy c of a group out_c = sum_k w_k in_k (vectors: the
// covariant basis of c applied to sum_k w_k (contravariant basis of k . u_k)),
// so its transpose gives every copy k in_k = w_k sum_c out_c (vectors: w_k
// times the contravariant basis of k applied to sum_c (covariant basis of c
// . u_c)).  Same group order and summation order as k_dss.
template <class FT>
__global__ void __launch_bounds__(DSS_THREADS) k_dss_t(DevParams<FT> P, FT *__restrict__ C, FT *__restrict__ F) {
  const int lane = threadIdx.x & 31;
  const int g = blockIdx.x * (DSS_THREADS / 32) + (threadIdx.x >> 5);
  if (g >= P.ngroups) return;
  const int Nv = P.Nv, Nf = P.Nf;
  const int o0 = P.goff[g], o1 = P.goff[g + 1];
  if (C) {
    for (int v0 = 0; v0 < Nv; v0 += 64) {
      const int v[2] = {v0 + lane, v0 + 32 + lane};
      const bool ok[2] = {v[0] < Nv, v[1] < Nv};
      FT s0[2] = {0, 0}, s3[2] = {0, 0}, X0[2] = {0, 0}, X1[2] = {0, 0}, X2[2] = {0, 0};
      for (int c = o0; c < o1; ++c) {
        const int idx = P.gcopy[c], e = idx >> 4, n = idx & 15;
        const FT *eo = P.ecov + (size_t)idx * 6;
        const size_t b0 = ((size_t)e * 4 * NN + n) * Nv;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          if (!ok[h]) continue;
          const size_t b = b0 + v[h];
          s0[h] += C[b];
          s3[h] += C[b + 48 * Nv];
          const FT u1 = C[b + 16 * Nv], u2 = C[b + 32 * Nv];
          X0[h] += u1 * eo[0] + u2 * eo[3];
          X1[h] += u1 * eo[1] + u2 * eo[4];
          X2[h] += u1 * eo[2] + u2 * eo[5];
        }
      }
      for (int c = o0; c < o1; ++c) {
        const int idx = P.gcopy[c], e = idx >> 4, n = idx & 15;
        const FT w = P.gw[c];
        const FT *ec = P.econ + (size_t)idx * 6;
        const size_t b0 = ((size_t)e * 4 * NN + n) * Nv;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          if (!ok[h]) continue;
          const size_t b = b0 + v[h];
          C[b] = w * s0[h];
          C[b + 48 * Nv] = w * s3[h];
          C[b + 16 * Nv] = w * (ec[0] * X0[h] + ec[1] * X1[h] + ec[2] * X2[h]);
          C[b + 32 * Nv] = w * (ec[3] * X0[h] + ec[4] * X1[h] + ec[5] * X2[h]);
        }
      }
    }
  }
  if (F) {
    for (int k0 = 0; k0 < Nf; k0 += 64) {
      const int k[2] = {k0 + lane, k0 + 32 + lane};
      const bool ok[2] = {k[0] < Nf, k[1] < Nf};
      FT sf[2] = {0, 0};
      for (int c = o0; c < o1; ++c) {
        const size_t b0 = (size_t)P.gcopy[c] * Nf;
#pragma unroll
        for (int h = 0; h < 2; ++h)
          if (ok[h]) sf[h] += F[b0 + k[h]];
      }
      for (int c = o0; c < o1; ++c) {
        const FT w = P.gw[c];
        const size_t b0 = (size_t)P.gcopy[c] * Nf;
#pragma unroll
        for (int h = 0; h < 2; ++h)
          if (ok[h]) F[b0 + k[h]] = w * sf[h];
      }
    }
  }
}

// u_{n+1} = u_n + dt sum_j (b~_j T_exp_j + b_j T_imp_j), then the impenetrable filter.
template <class FT>
__global__ void k_final(DevParams<FT> P, StageArgs<FT> A, FT *__restrict__ Yc, FT *__restrict__ Yf) {
  const int Nv = P.Nv, Nf = P.Nf;
  const size_t NC = (size_t)P.Nh * 4 * NN * Nv, NF = (size_t)P.Nh * NN * Nf;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < NC + NF; q += (size_t)gridDim.x * blockDim.x) {
    if (q < NC) {
      const size_t row = q / Nv;
      const int v = (int)(q - row * Nv);
      const int n = (int)(row % NN), c = (int)((row / NN) % 4);
      const size_t e = row / (4 * NN);
      FT s = Yc[q];
      for (int j = 0; j < A.nsrc; ++j) {
        if (A.te_c[j]) s += A.ce[j] * A.te_c[j][q];
        if (A.ti_c[j] && (c == 0 || c == 3)) s += A.ci[j] * A.ti_c[j][((e * 2 + (c == 3)) * NN + n) * Nv + v];
      }
      Yc[q] = s;
    } else {
      const size_t r = q - NC;
      const int k = (int)(r % Nf);
      FT s = Yf[r];
      for (int j = 0; j < A.nsrc; ++j) {
        if (A.te_f[j]) s += A.ce[j] * A.te_f[j][r];
        if (A.ti_f[j]) s += A.ci[j] * A.ti_f[j][r];
      }
      Yf[r] = (k == 0 || k == Nv) ? FT(0) : s;
    }
  }
}

// Transpose of k_final: the filter zeroes the boundary-face cotangent of
// u_{n+1}; u_n receives it unchanged and every tendency j its coefficient
// times it.  The tendency cotangents are written (this is their first
// contribution in a reverse step); a zero coefficient writes zeros.
template <class FT>
__global__ void k_final_t(DevParams<FT> P, CotArgs<FT> A, FT *__restrict__ Ybc, FT *__restrict__ Ybf) {
  const int Nv = P.Nv, Nf = P.Nf;
  const size_t NC = (size_t)P.Nh * 4 * NN * Nv, NF = (size_t)P.Nh * NN * Nf;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < NC + NF; q += (size_t)gridDim.x * blockDim.x) {
    if (q < NC) {
      const size_t row = q / Nv;
      const int v = (int)(q - row * Nv);
      const int n = (int)(row % NN), c = (int)((row / NN) % 4);
      const size_t e = row / (4 * NN);
      const FT yb = Ybc[q];
      for (int j = 0; j < A.nsrc; ++j) {
        if (A.te_c[j]) A.te_c[j][q] = A.ce[j] * yb;
        if (A.ti_c[j] && (c == 0 || c == 3)) A.ti_c[j][((e * 2 + (c == 3)) * NN + n) * Nv + v] = A.ci[j] * yb;
      }
    } else {
      const size_t r = q - NC;
      const int k = (int)(r % Nf);
      const FT yb = (k == 0 || k == Nv) ? FT(0) : Ybf[r];
      Ybf[r] = yb;
      for (int j = 0; j < A.nsrc; ++j) {
        if (A.te_f[j]) A.te_f[j][r] = A.ce[j] * yb;
        if (A.ti_f[j]) A.ti_f[j][r] = A.ci[j] * yb;
      }
    }
  }
}


// acc[o] += sum_i part[i * stride + o] for o < nout, in a fixed order (one block).
__global__ void k_accum(const double *__restrict__ part, int n, int stride, int nout, double *__restrict__ acc) {
  __shared__ double sh[256];
  for (int o = 0; o < nout; ++o) {
    double s = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[(size_t)i * stride + o];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) acc[o] += sh[0];
    __syncthreads();
  }
}

// acc[0] += the sum of n RSlot<FT> entries, in a fixed order: one block of ACC_THREADS
// threads, each with four independent compensated sums fed four loads at a time (the
// loads of one thread are in flight together), then the lanes and the warps in order.
constexpr int ACC_THREADS = 1024;
template <class FT>
__global__ void __launch_bounds__(ACC_THREADS) k_accum_slots(const double *__restrict__ part, int n,
                                                             double *__restrict__ acc) {
  __shared__ FT sh[2][ACC_THREADS / 32];
  CSum<FT> s[4];
  int i = threadIdx.x;
  for (; i + 3 * ACC_THREADS < n; i += 4 * ACC_THREADS) {
    CSum<FT> x[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) x[u] = RSlot<FT>::load(&part[i + u * ACC_THREADS]);
#pragma unroll
    for (int u = 0; u < 4; ++u) s[u].add(x[u]);
  }
  for (; i < n; i += ACC_THREADS) s[0].add(RSlot<FT>::load(&part[i]));
  s[0].add(s[1]);
  s[2].add(s[3]);
  s[0].add(s[2]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s[0].add(s[0].xor_shfl(o, 32));
  if ((threadIdx.x & 31) == 0) {
    sh[0][threadIdx.x >> 5] = s[0].hi;
    sh[1][threadIdx.x >> 5] = s[0].lo;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    CSum<FT> t;
    for (int w = 0; w < ACC_THREADS / 32; ++w) {
      CSum<FT> a;
      a.hi = sh[0][w];
      a.lo = sh[1][w];
      t.add(a);
    }
    acc[0] += t.value();
  }
}

template <class FT>
__global__ void k_bc_filter(int ncols, int Nf, FT *__restrict__ Yf) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncols) {
    Yf[(size_t)c * Nf] = FT(0);
    Yf[(size_t)c * Nf + Nf - 1] = FT(0);
  }
}

// Neumaier (compensated) FP64 summation
__device__ __forceinline__ void two_sum_acc(double &s, double &cmp, double x) {
  const double t = s + x;
  if (fabs(s) >= fabs(x)) cmp += (s - t) + x; else cmp += (x - t) + s;
  s = t;
}

constexpr int SUM_THREADS = 256;

// Block partial sums of rho*WJ and rhoe*WJ, and with Q5 (moist 0M) of
// rhoq_tot*WJ, the fifth centre component (fixed order -> deterministic).
// Each block writes NS (sum, compensation) pairs at part[block * 6].
template <class FT, bool Q5 = false>
__global__ void __launch_bounds__(SUM_THREADS) k_sums_partial(DevParams<FT> P, const FT *__restrict__ Yc, double *__restrict__ part) {
  constexpr int NS = Q5 ? 3 : 2, NFC = Q5 ? 5 : 4;
  __shared__ double sh[2 * NS][SUM_THREADS];
  const int Nv = P.Nv;
  const size_t npt = (size_t)P.Nh * NN * Nv;
  double s[NS] = {}, c[NS] = {};
  for (size_t p = blockIdx.x * (size_t)SUM_THREADS + threadIdx.x; p < npt; p += (size_t)gridDim.x * SUM_THREADS) {
    const size_t col = p / Nv;
    const int v = (int)(p - col * Nv);
    const int n = (int)(col % NN);
    const size_t e = col / NN;
    const double Jh = (double)P.hgeo[(e * HG_N + HG_JH) * NN + n];
    double WJ;
    if (P.topo) {
      // terrain-following levels: J = J_h r^2 dz of the point (topo.cuh), in FP64
      const Lev4<FT> L = P.ltc[v];
      const double zs = (double)P.tgeo[(e * TG_N + TG_ZS) * NN + n];
      const double r = 1.0 + ((double)L.x + zs * (double)L.y) * (double)P.iR;
      WJ = (double)P.W[n] * (Jh * (r * r) * ((double)L.z + zs * (double)L.w));
    } else {
      WJ = (double)P.W[n] * (Jh * (double)P.levc[LC_R2 * Nv + v] * (double)P.levc[LC_DZ * Nv + v]);
    }
    const size_t b = (e * NFC * NN + n) * Nv + v;
    two_sum_acc(s[0], c[0], (double)Yc[b] * WJ);
    two_sum_acc(s[1], c[1], (double)Yc[b + 48 * Nv] * WJ);
    if (Q5) two_sum_acc(s[NS - 1], c[NS - 1], (double)Yc[b + 64 * Nv] * WJ);
  }
#pragma unroll
  for (int q = 0; q < NS; ++q) {
    sh[2 * q][threadIdx.x] = s[q];
    sh[2 * q + 1][threadIdx.x] = c[q];
  }
  __syncthreads();
  if (threadIdx.x < NS) {
    double ss = 0, cc = 0;
    for (int t = 0; t < SUM_THREADS; ++t) {
      two_sum_acc(ss, cc, sh[2 * threadIdx.x][t]);
      cc += sh[2 * threadIdx.x + 1][t];
    }
    part[blockIdx.x * 6 + 2 * threadIdx.x] = ss;
    part[blockIdx.x * 6 + 2 * threadIdx.x + 1] = cc;
  }
}

__global__ void k_sums_final(const double *__restrict__ part, int nblocks, int nsums, double *__restrict__ out) {
  if (threadIdx.x < nsums) {
    double ss = 0, cc = 0;
    for (int b = 0; b < nblocks; ++b) {
      two_sum_acc(ss, cc, part[b * 6 + 2 * threadIdx.x]);
      cc += part[b * 6 + 2 * threadIdx.x + 1];
    }
    out[threadIdx.x] = ss + cc;
  }
}

template <class FT>
__global__ void __launch_bounds__(256) k_reduce_rnorm(const double *__restrict__ r, int ncols, double *__restrict__ out) {
  CSum<FT> s[3];
  for (int c = threadIdx.x; c < ncols; c += blockDim.x)
    for (int q = 0; q < 3; ++q) s[q].add(RSlot<FT>::load(&r[(size_t)c * 3 + q]));
  block_sum3<FT>(s);
  if (threadIdx.x == 0)
    for (int q = 0; q < 3; ++q) out[q] = s[q].value();
}

// The failure-detection self-test: an mbarrier phase that announces a 16-byte
// transfer which nothing issues can never complete, so every lane's bounded
// wait runs out after limit_ns and flags ST_TIMEOUT, exactly as a wait on a
// copy that never lands would.  Nothing is in flight when the kernel ends.
__global__ void k_selftest_wait(int *status, unsigned long long limit_ns) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_expect_tx(&bar, 16u);
  __syncwarp();
  mbar_wait_bounded(&bar, 0u, status, limit_ns);
}

}  // namespace

void launch_selftest_wait(int *status, unsigned long long limit_ns, cudaStream_t s) {
  k_selftest_wait<<<1, 32, 0, s>>>(status, limit_ns);
}

template <class FT>
void launch_dss(const DevParams<FT> &P, FT *C, FT *F, cudaStream_t s) {
  const int grid = (P.ngroups + DSS_THREADS / 32 - 1) / (DSS_THREADS / 32);
  if (grid > 0) k_dss<FT><<<grid, DSS_THREADS, 0, s>>>(P, C, F);
}
template <class FT>
void launch_dss_state(const DevParams<FT> &P, FT *C, FT *F, cudaStream_t s) {
  const int grid = (P.ngroups + DSS_THREADS / 32 - 1) / (DSS_THREADS / 32);
  if (grid <= 0) return;
  if (P.moist) k_dss<FT, true><<<grid, DSS_THREADS, 0, s>>>(P, C, F);
  else k_dss<FT><<<grid, DSS_THREADS, 0, s>>>(P, C, F);
}
template <class FT>
void launch_dss_transpose(const DevParams<FT> &P, FT *C, FT *F, cudaStream_t s) {
  const int grid = (P.ngroups + DSS_THREADS / 32 - 1) / (DSS_THREADS / 32);
  if (grid > 0) k_dss_t<FT><<<grid, DSS_THREADS, 0, s>>>(P, C, F);
}
template <class FT>
void launch_final(const DevParams<FT> &P, const StageArgs<FT> &A, FT *Yc, FT *Yf, cudaStream_t s) {
  k_final<FT><<<152 * 8, 256, 0, s>>>(P, A, Yc, Yf);
}
template <class FT>
void launch_final_transpose(const DevParams<FT> &P, const CotArgs<FT> &A, FT *Ybc, FT *Ybf, cudaStream_t s) {
  k_final_t<FT><<<152 * 8, 256, 0, s>>>(P, A, Ybc, Ybf);
}
template <class FT>
void launch_accum_slots(const double *part, int n, double *acc, cudaStream_t s) {
  k_accum_slots<FT><<<1, ACC_THREADS, 0, s>>>(part, n, acc);
}
void launch_accum(const double *part, int n, int stride, int nout, double *acc, cudaStream_t s) {
  k_accum<<<1, 256, 0, s>>>(part, n, stride, nout, acc);
}
template <class FT>
void launch_bc_filter(const DevParams<FT> &P, FT *Yf, cudaStream_t s) {
  const int ncols = P.Nh * NN;
  k_bc_filter<FT><<<(ncols + 255) / 256, 256, 0, s>>>(ncols, P.Nf, Yf);
}
template <class FT>
void launch_global_sums(const DevParams<FT> &P, const FT *Yc, double *partials, int nblocks, double *out, cudaStream_t s) {
  if (P.moist) k_sums_partial<FT, true><<<nblocks, SUM_THREADS, 0, s>>>(P, Yc, partials);
  else k_sums_partial<FT><<<nblocks, SUM_THREADS, 0, s>>>(P, Yc, partials);
  k_sums_final<<<1, 32, 0, s>>>(partials, nblocks, P.moist ? 3 : 2, out);
}
template <class FT>
void launch_reduce_rnorm(const double *rnorm, int ncols, double *out, cudaStream_t s) {
  k_reduce_rnorm<FT><<<1, 256, 0, s>>>(rnorm, ncols, out);
}

#define INST(FT)                                                                                          \
  template void launch_dss<FT>(const DevParams<FT> &, FT *, FT *, cudaStream_t);                          \
  template void launch_dss_state<FT>(const DevParams<FT> &, FT *, FT *, cudaStream_t);                    \
  template void launch_dss_transpose<FT>(const DevParams<FT> &, FT *, FT *, cudaStream_t);                \
  template void launch_final<FT>(const DevParams<FT> &, const StageArgs<FT> &, FT *, FT *, cudaStream_t); \
  template void launch_final_transpose<FT>(const DevParams<FT> &, const CotArgs<FT> &, FT *, FT *, cudaStream_t); \
  template void launch_bc_filter<FT>(const DevParams<FT> &, FT *, cudaStream_t);                          \
  template void launch_global_sums<FT>(const DevParams<FT> &, const FT *, double *, int, double *, cudaStream_t); \
  template void launch_reduce_rnorm<FT>(const double *, int, double *, cudaStream_t);             \
  template void launch_accum_slots<FT>(const double *, int, double *, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace gb
