// Launch wrappers of the GB300 dry dynamical-core kernels.
#pragma once
#include "common.cuh"

namespace gb {

// Face slab of the flat slab kernels in shared memory: the element's four node rows j (nodes
// 4j..4j+3, Nf faces each, as in global memory) at j * face_rows<FT>(Nf) elements.  In FP32 the
// row stride is padded to 4 banks modulo 32, so that the four rows' threads of a warp reading
// one node each at the eight levels of a level_slot group hit 32 distinct banks (unpadded, the
// rows of Nf = 64 faces all start on bank 0: 4-way conflicts); FP64 keeps the global layout.
template <class FT>
__host__ __device__ inline int face_rows(int Nf) {
  return sizeof(FT) == 4 ? 4 * Nf + ((4 - 4 * Nf) % 32 + 32) % 32 : 4 * Nf;
}
// element index of (node n, face k) in that slab; FR = face_rows<FT>(Nf)
__host__ __device__ inline int fslot(int n, int k, int Nf, int FR) { return (n >> 2) * FR + (n & 3) * Nf + k; }

// Shared-memory layouts of the element-slab kernels (byte offsets).  The
// input slabs are double-buffered (nbuf = 2) when they fit, else single.
// Pass A's output slab is double-buffered with its inputs: the store of one element's
// Laplacians then reads its slab while the next element is computed into the other.
template <class FT>
struct PassALayout {
  size_t y[2], f[2], g[2], out[2], bar, total;
  __host__ __device__ PassALayout(int Nv, int nbuf) {
    const int Nf = Nv + 1;
    size_t o = 0;
    for (int b = 0; b < 2; ++b) {
      if (b < nbuf) {
        y[b] = o; o += align16(sizeof(FT) * 64 * Nv);
        f[b] = o; o += align16(sizeof(FT) * 4 * face_rows<FT>(Nf));
        g[b] = o; o += align16(sizeof(FT) * HG_N * 16);
      } else {
        y[b] = y[0]; f[b] = f[0]; g[b] = g[0];
      }
    }
    out[0] = o; o += align16(sizeof(FT) * 64 * Nv);
    if (nbuf == 2) {
      out[1] = o; o += align16(sizeof(FT) * 64 * Nv);
    } else {
      out[1] = out[0];
    }
    bar = o; o += 16;
    total = o;
  }
};

// Level-major scratch rows of pass B: field f of level v, node n at
// (f Nv + v) 16 + n, so the thread of (level v, row j) reads or writes its
// four nodes as one 16-byte row vector (bank-conflict free).
enum PassBScratch { SB_C1 = 0, SB_C2, SB_K, SB_RJ, SB_L4, SB_Q1, SB_Q2, SB_N };

// Pass B's shared memory: per buffer the input slabs (state, faces, geometry,
// Laplacians); the tendency is written in place over the state and face slabs
// of the element being computed and stored from there.
template <class FT>
struct PassBLayout {
  size_t y[2], f[2], g[2], lap[2], s, x1, x2, w, bar, total;
  __host__ __device__ PassBLayout(int Nv, int nbuf) {
    const int Nf = Nv + 1;
    size_t o = 0;
    for (int b = 0; b < 2; ++b) {
      if (b < nbuf) {
        y[b] = o; o += align16(sizeof(FT) * 64 * Nv);
        f[b] = o; o += align16(sizeof(FT) * 4 * face_rows<FT>(Nf));
        g[b] = o; o += align16(sizeof(FT) * HG_N * 16);
        lap[b] = o; o += align16(sizeof(FT) * 64 * Nv);
      } else {
        y[b] = y[0]; f[b] = f[0]; g[b] = g[0]; lap[b] = lap[0];
      }
    }
    s = o; o += align16(sizeof(FT) * SB_N * 16 * Nv);
    x1 = o; o += align16(sizeof(FT) * 16 * Nf);   // face rows [Nf][16]
    x2 = o; o += align16(sizeof(FT) * 16 * Nf);
    w = o; o += align16(sizeof(FT) * 2 * 16);     // GLL weights W, 1/W
    bar = o; o += 16;
    total = o;
  }
};

// Sources of a stage assembly  U = u_n + sum_j (ce[j] T_exp[j] + ci[j] T_imp[j]).
template <class FT>
struct StageArgs {
  const FT *un_c, *un_f;
  const FT *te_c[4], *te_f[4];
  const FT *ti_c[4], *ti_f[4];  // reduced implicit tendencies ([e][2][16][Nv], faces)
  FT ce[4], ci[4];
  int nsrc;
  FT *U_c, *U_f;    // stage state out
  FT *Ti_c, *Ti_f;  // implicit tendency of this stage out (reduced)
  FT dtg, idtg;
  double *rnorm;    // [ncols][3] residual sums of squares (accumulated; RSlot<FT> entries)
  int first;        // 1: overwrite rnorm, 0: accumulate
};

// Final combination of a stiffly accurate step folded into the last stage's
// explicit tendency: out = U + sum_{j<3} c_j T_j + c_3 T, with U the stage
// state (the pass's own input), T_j earlier (DSSed) explicit tendencies and T
// the tendency the pass computes.
// The bottom and top faces of u_3 are zero (the impenetrable filter, as in the
// stage combination kernel).
template <class FT>
struct FinArgs {
  const FT *te_c[3], *te_f[3];
  FT c[4];
};

// Cotangents of the tendencies a transposed stage combination accumulates into.
template <class FT>
struct CotArgs {
  FT *te_c[4], *te_f[4];
  FT *ti_c[4], *ti_f[4];
  FT ce[4], ci[4];
  int nsrc;
};

enum ColMode { COL_STAGE = 0, COL_IMPLICIT = 1, COL_JACOBIAN = 2, COL_LDIV = 3, COL_POSTIMP = 4 };
constexpr int JAC_Q = 15;  // stored Jacobian quantities per level
constexpr int JAC_QT = JAC_Q + 6;  // over terrain: with the (rho, u_h), (rho e_tot, u_h) blocks
constexpr int JAC_QM = JAC_Q + 4;  // moist 0M: with the (rho q_tot, u_3) and (u_3, rho q_tot) blocks

template <class FT>
struct ColArgs {
  const FT *Y_c, *Y_f;  // input state (or R for ldiv)
  FT *O_c, *O_f;        // output (tendency, or dY for ldiv)
  FT *jac;              // [ncols][JAC_Q][Nf]
  FT dtg;
};

template <class FT> void launch_passA(const DevParams<FT> &P, const FT *Yc, const FT *Yf, FT *L, cudaStream_t s);
template <class FT> void launch_passB(const DevParams<FT> &P, const FT *Yc, const FT *Yf, const FT *L, FT *Tc, FT *Tf, cudaStream_t s, const FinArgs<FT> *fin = nullptr);
template <class FT> void launch_dss(const DevParams<FT> &P, FT *C, FT *F, cudaStream_t s);
// the DSS of a state (Y.c with the context's centre components: 5 when moist)
template <class FT> void launch_dss_state(const DevParams<FT> &P, FT *C, FT *F, cudaStream_t s);
template <class FT> void launch_dss_transpose(const DevParams<FT> &P, FT *C, FT *F, cudaStream_t s);
template <class FT> void launch_column_stage(const DevParams<FT> &P, const StageArgs<FT> &A, cudaStream_t s);
template <class FT> void launch_column(const DevParams<FT> &P, int mode, const ColArgs<FT> &A, cudaStream_t s);
template <class FT> void launch_final(const DevParams<FT> &P, const StageArgs<FT> &A, FT *Yc, FT *Yf, cudaStream_t s);
// ---- reverse (adjoint) kernels
template <class FT> void launch_final_transpose(const DevParams<FT> &P, const CotArgs<FT> &A, FT *Ybc, FT *Ybf, cudaStream_t s);
void launch_accum(const double *part, int n, int stride, int nout, double *acc, cudaStream_t s);
template <class FT> bool passA_vjp_add_fits(int Nv);
template <class FT> size_t passA_vjp_smem(int Nv);
template <class FT> size_t passB_vjp_smem(int Nv);
template <class FT> void configure_adjoint_se(int Nv);
template <class FT> void launch_passA_vjp(const DevParams<FT> &P, const FT *Yc, const FT *Yf, const FT *Lb, FT *Ybc, FT *Ybf, int grid, cudaStream_t s, const FT *Xbc = nullptr, const FT *Xbf = nullptr);
// tsc scales the tendency cotangent: the result is that of tsc * (Tbc, Tbf), formed by
// scaling the outputs (the pullback is linear in the cotangent).
template <class FT> void launch_passB_vjp(const DevParams<FT> &P, const FT *Yc, const FT *Yf, const FT *L, const FT *Tbc, const FT *Tbf, FT *Ybc, FT *Ybf, FT *Lb, double *dpar, int grid, bool accum, cudaStream_t s, FT tsc = FT(1));
size_t col_vjp_scratch_words(int Nh, int Nv);
// Uo, Tio (optional): the recorded stage output and implicit tendency (U^ = U - dtgamma T_imp
// then replaces the stage assembly in the forward recompute).  e0, i0 (optional): the
// tendency cotangents are written, initialised as e0[j] Yb / i0[j] Yb from Yb on entry.
// tbs: when given, the cotangent of T_imp is *tbs times Yb on entry (Tb_c, Tb_f unused).
template <class FT> void launch_column_stage_vjp(const DevParams<FT> &P, const StageArgs<FT> &A, const FT *Ub_c, const FT *Ub_f, const FT *Tb_c, const FT *Tb_f, FT *Yb_c, FT *Yb_f, FT *const Teb[4], FT *const Tib[4], size_t NC, size_t NR, FT *scr, double *dalpha, cudaStream_t s, const FT *Uo = nullptr, const FT *Tio = nullptr, const FT *e0 = nullptr, const FT *i0 = nullptr, const FT *tbs = nullptr);
template <class FT> void launch_bc_filter(const DevParams<FT> &P, FT *Yf, cudaStream_t s);
// Failure-detection self-test: one warp waits on an mbarrier whose transfer is announced but
// never issued, so the bounded wait gives up after limit_ns and sets ST_TIMEOUT in *status.
void launch_selftest_wait(int *status, unsigned long long limit_ns, cudaStream_t s);
template <class FT> void launch_global_sums(const DevParams<FT> &P, const FT *Yc, double *partials, int nblocks, double *out, cudaStream_t s);
template <class FT> void launch_reduce_rnorm(const double *rnorm, int ncols, double *out, cudaStream_t s);
template <class FT> void launch_accum_slots(const double *part, int n, double *acc, cudaStream_t s);

// ---- terrain-following levels (kernels_topo.cu)
template <class FT> size_t topo_smem(int Nv);
template <class FT> cudaError_t configure_topo(int Nv);
template <class FT> void launch_topo_passA(const DevParams<FT> &P, const FT *Yc, const FT *Yf, FT *L, cudaStream_t s);
template <class FT> void launch_topo_passB(const DevParams<FT> &P, const FT *Yc, const FT *Yf, const FT *L, FT *Tc, FT *Tf, cudaStream_t s, const FinArgs<FT> *fin = nullptr);
// u_3 = -u_h^3 / g^33 on the bottom and top faces of every column (reads u_h of Yc)
template <class FT> void launch_topo_filter(const DevParams<FT> &P, const FT *Yc, FT *Yf, cudaStream_t s);
// DSS of the reduced implicit tendencies ([Nh][2][16][Nv] centres, faces)
template <class FT> void launch_dss_reduced(const DevParams<FT> &P, FT *C, FT *F, cudaStream_t s);

// Shared memory needed by the slab kernels with single input buffers (the
// minimum; double buffering is used when it fits).
template <class FT> size_t passA_smem(int Nv);
template <class FT> size_t passB_smem(int Nv);
template <class FT> void configure_se(int Nv);

}  // namespace gb
