// Implicit stage kernel: G lanes per column, CM (2 or 4) consecutive levels per lane.
//
// Fuses, for one implicit ARS343 stage, what ClimaTimeSteppers does through
// the hooks (src/simulation/integrator.jl:189-225):
//   stage assembly U^ = u_n + dt sum_j (a~_ij T_exp_j + a_ij T_imp_j),
//   impenetrable filter (precomputed_quantities.jl:486-553),
//   one Newton iteration: implicit_tendency! residual (implicit_tendency.jl:185-298),
//     update_jacobian! blocks (manual_sparse_jacobian.jl:713-870, dry, no
//     topography; the (u_3, u_h) block multiplies R_uh = 0 and is skipped),
//     ldiv! with BlockArrowheadSolve(rho, rho e_tot; alg2 = u_h)
//     (manual_sparse_jacobian.jl:580-583): Schur complement onto u_3,
//   U -= dY; filter; van Leer minus central post-Newton correction
//     (implicit_tendency.jl:322-339) applied as U += dtgamma * corr,
//   T_imp_i = (U - U^) / dtgamma and FP64 residual sums of squares.
// The column arithmetic is the shared core in colcore.cuh.
#include <cstdio>
#include <cstdlib>
#include <type_traits>

#include "colcore.cuh"

namespace gb {

namespace {

constexpr int CG_THREADS = 128;

// H += ce t (all five fields) + ci q (rho, rho e_tot, u_3), level by level; FP32 with two
// levels per lane: both levels in one packed multiply-add.
template <class FT, int CM>
__device__ __forceinline__ void stage_accumulate(FT (&H)[5][CM], const FT (&t)[5][CM], const FT (&q)[3][CM], FT ce,
                                                 FT ci) {
#pragma unroll
  for (int k = 0; k < CM; ++k)
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      H[c][k] += ce * t[c][k];
      if (ci != FT(0) && c != 1 && c != 2) H[c][k] += ci * q[c == 0 ? 0 : (c == 3 ? 1 : 2)][k];
    }
}
template <>
__device__ __forceinline__ void stage_accumulate<float, 2>(float (&H)[5][2], const float (&t)[5][2],
                                                           const float (&q)[3][2], float ce, float ci) {
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    float2 h = __ffma2_rn(bc2(ce), make_float2(t[c][0], t[c][1]), make_float2(H[c][0], H[c][1]));
    if (ci != 0.0f && c != 1 && c != 2) {
      const int m = c == 0 ? 0 : (c == 3 ? 1 : 2);
      h = __ffma2_rn(bc2(ci), make_float2(q[m][0], q[m][1]), h);
    }
    H[c][0] = h.x;
    H[c][1] = h.y;
  }
}

// TOPO: terrain-following levels (the column's own metric, col::ColLevT).
template <class FT, int G, int CM, int STG, int MINB, bool TOPO>
__global__ void __launch_bounds__(CG_THREADS, MINB) k_col_stage_g(DevParams<FT> P, StageArgs<FT> A) {
  const int lane = threadIdx.x & 31, gl = lane % G;
  const int col0 = (blockIdx.x * (CG_THREADS / 32) + (threadIdx.x >> 5)) * (32 / G) + lane / G;
  const int ncols = P.Nh * NN;
  const bool colv = col0 < ncols;
  const int col = colv ? col0 : ncols - 1;  // idle groups compute on a valid column, write nothing
  const int e = col >> 4, n = col & 15, Nv = P.Nv, Nf = P.Nf;
  const int r0 = gl * CM;   // first level of this lane
  const int sc = NN * Nv;   // component stride of the centre fields
  ColGeo<FT> Gm;
  Gm.load(P, e, n);
  const FT dtg = A.dtg;
  // per-lane bases: level r0 of this column; levels past the column are not read
  const size_t cb = (size_t)e * 4 * NN * Nv + (size_t)n * Nv + r0, rb = (size_t)e * 2 * NN * Nv + (size_t)n * Nv + r0;
  const size_t fb = ((size_t)e * NN + n) * Nf + r0;
  // ---- stage assembly U^ = u_n + sum_j (dt a~_ij T_exp_j + dt a_ij T_imp_j)
  FT H[5][CM];
  {
    const FT *pc = A.un_c + cb, *pf = A.un_f + fb;
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const bool okc = r0 + k < Nv, okf = r0 + k < Nf;
#pragma unroll
      for (int c = 0; c < 4; ++c) H[c][k] = okc ? pc[c * sc + k] : FT(0);
      H[4][k] = okf ? pf[k] : FT(0);
    }
  }
  // sources one at a time, summed in the tableau order
#pragma unroll
  for (int j = 0; j < STG; ++j) {
    FT t[5][CM];
    const FT *tc = A.te_c[j] + cb, *tf = A.te_f[j] + fb;
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const bool okc = r0 + k < Nv, okf = r0 + k < Nf;
#pragma unroll
      for (int c = 0; c < 4; ++c) t[c][k] = okc ? tc[c * sc + k] : FT(0);
      t[4][k] = okf ? tf[k] : FT(0);
    }
    FT q[3][CM];
    if (j >= 1) {
      const FT *qc = A.ti_c[j] + rb, *qf = A.ti_f[j] + fb;
#pragma unroll
      for (int k = 0; k < CM; ++k) {
        const bool okc = r0 + k < Nv, okf = r0 + k < Nf;
        q[0][k] = okc ? qc[k] : FT(0);
        q[1][k] = okc ? qc[sc + k] : FT(0);
        q[2][k] = okf ? qf[k] : FT(0);
      }
    }
    stage_accumulate<FT, CM>(H, t, q, A.ce[j], j >= 1 ? A.ci[j] : FT(0));
  }
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const int v = r0 + k;
    if (v >= Nv) { H[0][k] = FT(1); H[1][k] = FT(0); H[2][k] = FT(0); H[3][k] = FT(1); }
    if (v >= Nf) H[4][k] = FT(0);
  }
  // ---- one Newton iteration from U = U^, then the post-Newton correction
  using LV = std::conditional_t<TOPO, col::ColLevT<FT>, col::ColLev<FT>>;
  LV L;
  if constexpr (TOPO) L.load(P, e, n);
  else L = col::ColLev<FT>{P.lc4, P.lf4, P.lr4, Nv, Nf};
  FT U[5][CM];
#pragma unroll
  for (int c = 0; c < 5; ++c)
#pragma unroll
    for (int k = 0; k < CM; ++k) U[c][k] = H[c][k];
  CSum<FT> ss[3];
  bool finite = true;
  FT iJc[CM];
  col::newton_core<FT, G, CM, false>(P, Gm, L, gl, dtg, H, U, ss, finite, iJc);
  if (P.upwinding) col::vanleer_correct<FT, G, CM>(P, Gm, L, gl, dtg, U, iJc);
  // ---- outputs (u_h passes through the implicit stage unchanged)
  const FT idtg = A.idtg;
  {
    FT *uc = A.U_c + cb, *uf = A.U_f + fb, *tc = A.Ti_c + rb, *tf = A.Ti_f + fb;
#pragma unroll
    for (int k = 0; k < CM; ++k) {
      const int v = r0 + k;
      if (colv && v < Nv) {
        uc[k] = U[0][k];
        uc[sc + k] = H[1][k];
        uc[2 * sc + k] = H[2][k];
        uc[3 * sc + k] = U[3][k];
        tc[k] = (U[0][k] - H[0][k]) * idtg;
        tc[sc + k] = (U[3][k] - H[3][k]) * idtg;
      }
      if (colv && v < Nf) {
        uf[k] = U[4][k];
        tf[k] = (U[4][k] - H[4][k]) * idtg;
      }
    }
  }
  col::group_sum_rounded<G>(ss);
  finite = __all_sync(0xffffffffu, finite);
  if (gl == 0 && colv) {
    if (A.rnorm)
      for (int q = 0; q < 3; ++q) RSlot<FT>::put(&A.rnorm[(size_t)col * 3 + q], ss[q], A.first != 0);
  }
  if (lane == 0 && !finite) atomicOr(P.status, ST_NONFINITE);
}

template <class FT, int G, int CM, int MINB, bool TOPO>
void launch_gt(const DevParams<FT> &P, const StageArgs<FT> &A, cudaStream_t s) {
  const int ncols = P.Nh * NN, per_cta = (CG_THREADS / 32) * (32 / G);
  const int grid = (ncols + per_cta - 1) / per_cta;
  switch (A.nsrc) {
    case 1: k_col_stage_g<FT, G, CM, 1, MINB, TOPO><<<grid, CG_THREADS, 0, s>>>(P, A); break;
    case 2: k_col_stage_g<FT, G, CM, 2, MINB, TOPO><<<grid, CG_THREADS, 0, s>>>(P, A); break;
    default: k_col_stage_g<FT, G, CM, 3, MINB, TOPO><<<grid, CG_THREADS, 0, s>>>(P, A); break;
  }
}
// Over terrain the column's metric is computed per level from a few per-column values (no spill
// at the flat variants' register caps).
template <class FT, int G, int CM, int MINB>
void launch_g(const DevParams<FT> &P, const StageArgs<FT> &A, cudaStream_t s) {
  if (P.topo) launch_gt<FT, G, CM, MINB, true>(P, A, s);
  else launch_gt<FT, G, CM, MINB, false>(P, A, s);
}

// Levels per lane CM and the register cap (min resident CTAs per SM) of a variant.
template <class FT, int CM, int MINB>
void launch_cm(const DevParams<FT> &P, const StageArgs<FT> &A, cudaStream_t s) {
  // G lanes x CM levels >= Nv + 1 faces, G a power of two in 4..32
  const int need = (P.Nf + CM - 1) / CM;
  if (need <= 4) launch_g<FT, 4, CM, MINB>(P, A, s);
  else if (need <= 8) launch_g<FT, 8, CM, MINB>(P, A, s);
  else if (need <= 16) launch_g<FT, 16, CM, MINB>(P, A, s);
  else launch_g<FT, 32, CM, MINB>(P, A, s);
}

int column_variant_env() {
  static const int v = [] {
    const char *e = getenv("GBDYCORE_COLUMN_VARIANT");
    return e ? atoi(e) : -1;
  }();
  return v;
}

}  // namespace

// A.nsrc = stage index (1..3); all explicit sources j < nsrc and implicit
// sources 1 <= j < nsrc must be present (the ARS343 nonzero pattern).
template <class FT>
void launch_column_stage(const DevParams<FT> &P, const StageArgs<FT> &A, cudaStream_t s) {
  // the kernel reads every source below nsrc unconditionally: refuse a missing one
  bool ok = A.nsrc >= 1 && A.nsrc <= 3 && A.un_c && A.un_f && A.U_c && A.U_f && A.Ti_c && A.Ti_f;
  for (int j = 0; ok && j < A.nsrc; ++j) ok = A.te_c[j] && A.te_f[j] && (j == 0 || (A.ti_c[j] && A.ti_f[j]));
  if (!ok) {
    fprintf(stderr, "gbdycore: column stage launched with a missing source (nsrc=%d); not launched\n", A.nsrc);
    return;
  }
  // Variants (levels per lane CM, register cap as min resident 128-thread CTAs per SM).
  // Measured on GB300 at z_elem = 63, FP32, stage 4: CM 4 uncapped (160 registers)
  // 0.272 ms, CM 4 / 4 CTAs 0.205 ms, CM 2 uncapped 0.259 ms, CM 2 / 6 CTAs 0.174 ms
  // (7 and 8 CTAs: 0.172-0.174 ms with spills).  Default: CM 2 / 6 CTAs when two
  // levels per lane cover the column (Nf <= 64), else CM 4 / 4 CTAs.
  // GBDYCORE_COLUMN_VARIANT=0..3 overrides it for tuning.
  int v = column_variant_env();
  if (v < 0 || v > 3) v = P.Nf <= 64 ? 3 : 1;
  if ((v == 2 || v == 3) && P.Nf > 64) v = 1;  // CM 2 covers at most 64 faces
  switch (v) {
    case 0: launch_cm<FT, 4, 1>(P, A, s); break;
    case 2: launch_cm<FT, 2, 1>(P, A, s); break;
    case 3: launch_cm<FT, 2, 6>(P, A, s); break;
    default: launch_cm<FT, 4, 4>(P, A, s); break;
  }
}

template void launch_column_stage<float>(const DevParams<float> &, const StageArgs<float> &, cudaStream_t);
template void launch_column_stage<double>(const DevParams<double> &, const StageArgs<double> &, cudaStream_t);

}  // namespace gb
