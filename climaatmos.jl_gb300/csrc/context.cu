// C ABI of the GB300 dry dynamical core: context, hooks and the fused ARS343
// step (see include/gbdycore.h for the interface and its reference citations).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "gbdycore.h"
#include "kernels.cuh"
#include "trace.h"

using namespace gb;

// Scratch of gb_jacobian_solve_noalloc: the Jacobian blocks live in this
// file-scope device array instead of memory allocated by the library.  In
// host code the name is only a stand-in; its device address comes from
// cudaGetSymbolAddress (per device, see noalloc_scratch()).
static __device__ __align__(256) unsigned char g_noalloc_scratch[GB_NOALLOC_SCRATCH_BYTES];

namespace {

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  ~DevBuf() { if (p) cudaFree(p); }
};

struct ImplBase {
  virtual ~ImplBase() {}
};

template <class FT>
struct Impl : ImplBase {
  DevParams<FT> P{};
  DevBuf hgeo, levc, levf, lc4, lf4, lr4, goff, gcopy, gw, ecov, econ, status, tgeo, ltc, ltf;
  DevBuf lap, U, Te[4], Ti[4], jac, rnorm, partials, sums, rsum;
  size_t NC = 0, NF = 0, NR = 0;  // centre, face and reduced-centre element counts
  int nsum_blocks = 0;
  bool jac_valid = false;
  // ARS343 tableau (explicit a~, implicit a, weights b~ = b)
  double ae[4][4], ai[4][4], be[4], bi[4];
  bool stiffly_accurate = false;  // b = the last row of the implicit tableau
  // reverse mode (allocated on first use)
  // A captured launch sequence and the arguments it was captured for.
  struct Graph {
    cudaGraphExec_t exec = nullptr;
    const void *a = nullptr, *b = nullptr;
    double dt = 0;
    ~Graph() {
      if (exec) cudaGraphExecDestroy(exec);
    }
  };
  struct Record {  // forward data of one step kept for its reverse pass
    DevBuf Y, U[4], L[4], Te[4], Ti[4];
    Graph fwd, rev;  // this record's recording step and reverse step, captured on first use
  };
  struct Adjoint {
    std::vector<std::unique_ptr<Record>> rec;
    std::vector<std::unique_ptr<DevBuf>> ckpt;
    DevBuf Ub, Lb, Teb[4], Tib[4], zero, dummy, scr, dparB, dal, dacc, work, yb;
    int nsteps = 0, every = 0, grid = 0;
    int rec_first = -1;  // the first of the trailing segments whose stage records the forward pass kept
    int keep = 1;        // trailing segments the forward pass records (gb_adjoint_set_record_segments)
    double dt = 0;
    bool ready = false;
    size_t bytes = 0, rec_bytes = 0;
  };
  std::unique_ptr<Adjoint> adj;
  // captured step graph
  cudaGraphExec_t gexec = nullptr;
  cudaStream_t cap = nullptr;  // private stream the step graph is captured on
  void *g_c = nullptr, *g_f = nullptr;
  double g_dt = 0;
  ~Impl() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (cap) cudaStreamDestroy(cap);
  }
};

}  // namespace

struct gb_ctx {
  gb_config cfg{};
  HostGeometry geo;
  cudaStream_t stream = nullptr;
  ImplBase *impl = nullptr;
  std::string err;
  int last = GB_OK;
  ~gb_ctx() { delete impl; }
};

namespace {

int fail(gb_ctx *c, int code, const std::string &msg) {
  if (c) {
    c->err = msg;
    c->last = code;
  }
  return code;
}

#define CK(call)                                                                                \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) return fail(ctx, GB_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

template <class FT>
int upload(gb_ctx *ctx, DevBuf &b, const std::vector<double> &v) {
  std::vector<FT> t(v.begin(), v.end());
  b.bytes = t.size() * sizeof(FT);
  if (cudaMalloc(&b.p, b.bytes ? b.bytes : 16) != cudaSuccess) return fail(ctx, GB_ERR_NOMEM, "cudaMalloc failed");
  CK(cudaMemcpy(b.p, t.data(), b.bytes, cudaMemcpyHostToDevice));
  return GB_OK;
}
int upload_i(gb_ctx *ctx, DevBuf &b, const std::vector<int> &v) {
  b.bytes = v.size() * sizeof(int);
  if (cudaMalloc(&b.p, b.bytes ? b.bytes : 16) != cudaSuccess) return fail(ctx, GB_ERR_NOMEM, "cudaMalloc failed");
  CK(cudaMemcpy(b.p, v.data(), b.bytes, cudaMemcpyHostToDevice));
  return GB_OK;
}
int alloc(gb_ctx *ctx, DevBuf &b, size_t bytes) {
  b.bytes = bytes;
  if (cudaMalloc(&b.p, bytes ? bytes : 16) != cudaSuccess)
    return fail(ctx, GB_ERR_NOMEM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed");
  CK(cudaMemset(b.p, 0, bytes ? bytes : 16));
  return GB_OK;
}

void ars343(double ae[4][4], double ai[4][4], double be[4], double bi[4]) {
  // Ascher, Ruuth & Spiteri (1997), the (3,4,3) scheme
  const double g = 0.4358665215084590;
  const double a42 = 0.5529291480359398, a43 = a42;
  const double b1 = -1.5 * g * g + 4 * g - 0.25, b2 = 1.5 * g * g - 5 * g + 1.25;
  const double a31 = (1 - 4.5 * g + 1.5 * g * g) * a42 + (2.75 - 10.5 * g + 3.75 * g * g) * a43 - 3.5 + 13 * g - 4.5 * g * g;
  const double a32 = (-1 + 4.5 * g - 1.5 * g * g) * a42 + (-2.75 + 10.5 * g - 3.75 * g * g) * a43 + 4 - 12.5 * g + 4.5 * g * g;
  const double a41 = 1 - a42 - a43;
  const double E[4][4] = {{0, 0, 0, 0}, {g, 0, 0, 0}, {a31, a32, 0, 0}, {a41, a42, a43, 0}};
  const double I[4][4] = {{0, 0, 0, 0}, {0, g, 0, 0}, {0, (1 - g) / 2, g, 0}, {0, b1, b2, g}};
  const double B[4] = {0, b1, b2, g};
  for (int i = 0; i < 4; ++i) {
    for (int j = 0; j < 4; ++j) { ae[i][j] = E[i][j]; ai[i][j] = I[i][j]; }
    be[i] = B[i]; bi[i] = B[i];
  }
}

template <class FT>
int create_impl(gb_ctx *ctx) {
  auto *I = new (std::nothrow) Impl<FT>();
  if (!I) return fail(ctx, GB_ERR_NOMEM, "host allocation failed");
  ctx->impl = I;
  const HostGeometry &g = ctx->geo;
  const gb_config &c = ctx->cfg;
  int r;
  if ((r = upload<FT>(ctx, I->hgeo, g.hgeo))) return r;
  if ((r = upload<FT>(ctx, I->levc, g.levc))) return r;
  if ((r = upload<FT>(ctx, I->levf, g.levf))) return r;
  {
    const int nv = g.Nv, nf = nv + 1;
    std::vector<double> c4((size_t)4 * nv), f4((size_t)4 * nf, 0.0), r4((size_t)4 * nv, 0.0);
    for (int v = 0; v < nv; ++v) {
      const double r2dz = g.levc[LC_R2 * nv + v] * g.levc[LC_DZ * nv + v];
      c4[4 * v + 0] = r2dz;
      c4[4 * v + 1] = 1.0 / r2dz;
      c4[4 * v + 2] = g.levc[LC_IR2 * nv + v];
      c4[4 * v + 3] = g.levc[LC_PHI * nv + v];
      r4[4 * v + 0] = g.levc[LC_P0 * nv + v];
      r4[4 * v + 1] = g.levc[LC_IP0 * nv + v];
      r4[4 * v + 2] = g.levc[LC_RB * nv + v];
    }
    for (int f = 0; f < nf; ++f) {
      f4[4 * f + 0] = g.levf[LF_G33 * nf + f];
      f4[4 * f + 1] = g.levf[LF_BETA * nf + f];
      f4[4 * f + 2] = g.levf[LF_DPHI * nf + f];
    }
    if ((r = upload<FT>(ctx, I->lc4, c4))) return r;
    if ((r = upload<FT>(ctx, I->lf4, f4))) return r;
    if ((r = upload<FT>(ctx, I->lr4, r4))) return r;
  }
  if ((r = upload_i(ctx, I->goff, g.grp_off))) return r;
  if ((r = upload_i(ctx, I->gcopy, g.grp_copy))) return r;
  if ((r = upload<FT>(ctx, I->gw, g.grp_w))) return r;
  if ((r = upload<FT>(ctx, I->ecov, g.ecov))) return r;
  if ((r = upload<FT>(ctx, I->econ, g.econ))) return r;
  if (g.topo) {
    if ((r = upload<FT>(ctx, I->tgeo, g.tgeo))) return r;
    if ((r = upload<FT>(ctx, I->ltc, g.ltc))) return r;
    if ((r = upload<FT>(ctx, I->ltf, g.ltf))) return r;
  }
  if ((r = alloc(ctx, I->status, 16))) return r;
  const int Nh = g.Nh, Nv = g.Nv, Nf = Nv + 1;
  I->NC = (size_t)Nh * 4 * NN * Nv;
  I->NF = (size_t)Nh * NN * Nf;
  I->NR = (size_t)Nh * 2 * NN * Nv;
  if ((r = alloc(ctx, I->lap, I->NC * sizeof(FT)))) return r;
  if ((r = alloc(ctx, I->U, (I->NC + I->NF) * sizeof(FT)))) return r;
  for (int s = 0; s < 4; ++s)
    if ((r = alloc(ctx, I->Te[s], (I->NC + I->NF) * sizeof(FT)))) return r;
  for (int s = 1; s < 4; ++s)
    if ((r = alloc(ctx, I->Ti[s], (I->NR + I->NF) * sizeof(FT)))) return r;
  if ((r = alloc(ctx, I->rnorm, (size_t)Nh * NN * 3 * sizeof(double)))) return r;
  I->nsum_blocks = 152 * 4;
  if ((r = alloc(ctx, I->partials, (size_t)I->nsum_blocks * 6 * sizeof(double)))) return r;
  if ((r = alloc(ctx, I->sums, 4 * sizeof(double)))) return r;
  if ((r = alloc(ctx, I->rsum, 4 * sizeof(double)))) return r;
  DevParams<FT> &P = I->P;
  P.Nh = Nh; P.Nv = Nv; P.Nf = Nf; P.ngroups = (int)g.grp_off.size() - 1;
  P.grav = (FT)c.grav; P.Rd = (FT)c.R_d; P.cpd = (FT)c.cp_d; P.cvd = (FT)c.cv_d; P.T0 = (FT)c.T_0;
  P.pref = (FT)c.p_ref; P.kappa = (FT)c.R_d / (FT)c.cp_d; P.Tmin_ref = (FT)c.T_min_ref;
  P.Tsfc_ref = (FT)c.T_surf_ref; P.Tmin_sgs = (FT)c.T_min_sgs;
  P.icvd = (FT)(1.0 / c.cv_d); P.ipref = (FT)(1.0 / c.p_ref);
  P.cpTmin = (FT)(c.cp_d * c.T_min_ref);
  P.nu_v = (FT)c.nu_v; P.nu_s = (FT)c.nu_s; P.div_damp = (FT)c.div_damp; P.dt_model = (FT)c.dt;
  P.hs = c.held_suarez ? 1 : 0;
  if (P.hs) {
    P.hs_ka = (FT)(1.0 / (40.0 * c.hs_day));
    P.hs_dk = (FT)(1.0 / (4.0 * c.hs_day) - 1.0 / (40.0 * c.hs_day));
    P.hs_kf = (FT)(1.0 / c.hs_day);
    P.hs_sb = (FT)c.hs_sigma_b;
    P.hs_isb = (FT)(1.0 / (1.0 - c.hs_sigma_b));
    P.hs_dTy = (FT)c.hs_dT_y; P.hs_Teq = (FT)c.hs_T_equator; P.hs_dthz = (FT)c.hs_dtheta_z;
    P.hs_Tmin = (FT)c.hs_T_min; P.hs_ip0 = (FT)(1.0 / c.hs_p_ref_theta); P.hs_iMSLP = (FT)(1.0 / c.hs_MSLP);
  }
  P.upwinding = c.upwinding;
  for (int n = 0; n < NN; ++n) { P.W[n] = (FT)g.W[n]; P.iW[n] = (FT)(1.0 / g.W[n]); }
  for (int i = 0; i < NQ; ++i)
    for (int k = 0; k < NQ; ++k) {
      P.D[i * NQ + k] = (FT)g.D[i][k];
      P.DT[k * NQ + i] = (FT)g.D[i][k];
    }
  P.hgeo = (const FT *)I->hgeo.p; P.levc = (const FT *)I->levc.p; P.levf = (const FT *)I->levf.p;
  P.lc4 = (const Lev4<FT> *)I->lc4.p; P.lf4 = (const Lev4<FT> *)I->lf4.p; P.lr4 = (const Lev4<FT> *)I->lr4.p;
  P.goff = (const int *)I->goff.p; P.gcopy = (const int *)I->gcopy.p; P.gw = (const FT *)I->gw.p;
  P.ecov = (const FT *)I->ecov.p; P.econ = (const FT *)I->econ.p;
  P.status = (int *)I->status.p;
  P.topo = g.topo ? 1 : 0;
  P.tgeo = (const FT *)I->tgeo.p;
  P.ltc = (const Lev4<FT> *)I->ltc.p;
  P.ltf = (const Lev4<FT> *)I->ltf.p;
  P.iR = (FT)(1.0 / c.radius);
  P.spg_auh = (FT)c.alpha_uh;
  P.spg_aw = (FT)c.alpha_w;
  P.spg_zd = (FT)c.sponge_zd;
  P.spg_k = (FT)(M_PI / (2.0 * (c.z_max - c.sponge_zd)));
  P.moist = c.moist ? 1 : 0;
  if (P.moist) {
    P.sa_iters = c.sa_iters;
    P.Rv = (FT)c.R_v;
    P.cvv = (FT)(c.cp_v - c.R_v); P.cvl = (FT)c.cp_l; P.cvi = (FT)c.cp_i;
    P.dcl = (FT)(c.cp_v - c.cp_l); P.dci = (FT)(c.cp_v - c.cp_i);
    P.Lv0 = (FT)c.LH_v0; P.Ls0 = (FT)c.LH_s0;
    P.iTtr = (FT)(1.0 / c.T_triple); P.ptr = (FT)c.press_triple;
    P.Tfrz = (FT)c.T_freeze; P.Tice = (FT)c.T_icenuc; P.iTrng = (FT)(1.0 / (c.T_freeze - c.T_icenuc));
    P.pice = (FT)c.pow_icenuc;
    P.ev0 = (FT)(c.LH_v0 - c.R_v * c.T_0); P.ei0 = (FT)(c.LH_s0 - c.LH_v0);
  }
  ars343(I->ae, I->ai, I->be, I->bi);
  I->stiffly_accurate = true;
  for (int j = 0; j < 4; ++j) I->stiffly_accurate = I->stiffly_accurate && I->bi[j] == I->ai[3][j];
  int dev = 0, optin = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (passB_smem<FT>(Nv) > (size_t)optin)
    return fail(ctx, GB_ERR_ARG, "z_elem too large for the element-slab kernels at this precision (shared memory)");
  configure_se<FT>(Nv);
  if (g.topo) {
    if (topo_smem<FT>(Nv) > (size_t)optin)
      return fail(ctx, GB_ERR_ARG, "z_elem too large for the terrain slab kernels at this precision (shared memory)");
    const cudaError_t e = configure_topo<FT>(Nv);
    if (e != cudaSuccess)
      return fail(ctx, GB_ERR_CUDA, std::string("terrain slab kernels: ") + cudaGetErrorString(e));
  }
  CK(cudaGetLastError());
  return GB_OK;
}

template <class FT>
Impl<FT> *impl(gb_ctx *ctx) { return static_cast<Impl<FT> *>(ctx->impl); }

int check_launch(gb_ctx *ctx) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(ctx, GB_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  return GB_OK;
}

// test_dycore_consistency: NaN (all bits set, in FP32 and FP64) in every scratch
// buffer the tendencies and the step fill before they read it (fill_with_nans!,
// src/utils/debug_utils.jl:58-70).  The Jacobian blocks are not scratch: ldiv
// reads the blocks of the last update_jacobian, as CTS's Jacobian object.
template <class FT>
void poison_scratch(gb_ctx *ctx, cudaStream_t s) {
  if (!ctx->cfg.test_dycore_consistency) return;
  Impl<FT> *I = impl<FT>(ctx);
  DevBuf *bufs[] = {&I->lap, &I->U, &I->Te[0], &I->Te[1], &I->Te[2], &I->Te[3],
                    &I->Ti[1], &I->Ti[2], &I->Ti[3], &I->rnorm};
  for (DevBuf *b : bufs)
    if (b->p) cudaMemsetAsync(b->p, 0xFF, b->bytes, s);
}

template <class FT>
int remaining_tendency_t(gb_ctx *ctx, gb_fieldvec Yt, gb_fieldvec Y) {
  Impl<FT> *I = impl<FT>(ctx);
  poison_scratch<FT>(ctx, ctx->stream);
  if (I->P.topo) {
    launch_topo_passA<FT>(I->P, (const FT *)Y.c, (const FT *)Y.f, (FT *)I->lap.p, ctx->stream);
    launch_dss<FT>(I->P, (FT *)I->lap.p, nullptr, ctx->stream);
    launch_topo_passB<FT>(I->P, (const FT *)Y.c, (const FT *)Y.f, (const FT *)I->lap.p, (FT *)Yt.c, (FT *)Yt.f,
                          ctx->stream);
    return check_launch(ctx);
  }
  launch_passA<FT>(I->P, (const FT *)Y.c, (const FT *)Y.f, (FT *)I->lap.p, ctx->stream);
  launch_dss<FT>(I->P, (FT *)I->lap.p, nullptr, ctx->stream);
  launch_passB<FT>(I->P, (const FT *)Y.c, (const FT *)Y.f, (const FT *)I->lap.p, (FT *)Yt.c, (FT *)Yt.f, ctx->stream);
  return check_launch(ctx);
}

template <class FT>
int column_hook_t(gb_ctx *ctx, int mode, gb_fieldvec O, gb_fieldvec Y, double dtg) {
  Impl<FT> *I = impl<FT>(ctx);
  if (mode == COL_JACOBIAN && !I->jac.p) {
    const int nq = I->P.topo ? JAC_QT : (I->P.moist ? JAC_QM : JAC_Q);
    int r = alloc(ctx, I->jac, (size_t)I->P.Nh * NN * nq * I->P.Nf * sizeof(FT));
    if (r) return r;
  }
  if (mode == COL_LDIV && !I->jac_valid) return fail(ctx, GB_ERR_STATE, "gb_ldiv called before gb_update_jacobian");
  if (mode == COL_IMPLICIT) poison_scratch<FT>(ctx, ctx->stream);
  ColArgs<FT> A{};
  A.Y_c = (const FT *)Y.c; A.Y_f = (const FT *)Y.f;
  A.O_c = (FT *)O.c; A.O_f = (FT *)O.f;
  A.jac = (FT *)I->jac.p;
  A.dtg = (FT)dtg;
  launch_column<FT>(I->P, mode, A, ctx->stream);
  if (mode == COL_JACOBIAN) I->jac_valid = true;
  return check_launch(ctx);
}

// The final combination of a stiffly accurate step written from the last stage
// state U_4 = u_n + dt sum_j (a~_4j T_exp_j + b_j T_imp_j):
// u_{n+1} = U_4 + dt sum_j (b~_j - a~_4j) T_exp_j, with u_3 = 0 on the bottom
// and top faces, folded into the last pass B.  The last T_exp enters before its
// DSS, and the sum is DSSed as a whole (the reference's final dss!): for a
// continuous u_n that equals U_4 + ... + DSS(T_exp_4).
template <class FT>
FinArgs<FT> fin_args(const Impl<FT> *I, FT dt, FT *const (&tc)[4], FT *const (&tf)[4]) {
  FinArgs<FT> F{};
  for (int j = 0; j < 3; ++j) {
    const double c = I->be[j] - I->ae[3][j];
    F.c[j] = dt * (FT)c;
    F.te_c[j] = c != 0 ? tc[j] : nullptr;
    F.te_f[j] = c != 0 ? tf[j] : nullptr;
  }
  F.c[3] = dt * (FT)I->be[3];
  return F;
}

// One fused ARS343 step (stage loop of ClimaTimeSteppers' IMEX ARK with one
// Newton iteration per implicit stage); T_exp_j is DSSed once right after it
// is computed, so every stage state assembled from u_n (continuous), DSSed
// explicit tendencies and column-local implicit tendencies is continuous.
// The step over terrain-following levels: the terrain slab kernels for the explicit
// tendencies; the implicit tendencies are DSSed too (a column's implicit tendency depends on
// its element's slopes through u_h^3, so collocated copies differ, and the reference DSSes
// every assembled stage state); the unfolded final combination, its DSS and the impenetrable
// filter u_3 = -u_h^3 / g^33 of the new state (the reference's dss! then cache!).
template <class FT>
void enqueue_step_topo(gb_ctx *ctx, FT *Yc, FT *Yf, double dt_, cudaStream_t s) {
  Impl<FT> *I = impl<FT>(ctx);
  const DevParams<FT> &P = I->P;
  const FT dt = (FT)dt_;
  FT *lap = (FT *)I->lap.p;
  auto tec = [&](int j) { return (FT *)I->Te[j].p; };
  auto tef = [&](int j) { return (FT *)I->Te[j].p + I->NC; };
  auto tic = [&](int j) { return (FT *)I->Ti[j].p; };
  auto tif = [&](int j) { return (FT *)I->Ti[j].p + I->NR; };
  FT *Uc = (FT *)I->U.p, *Uf = Uc + I->NC;
  poison_scratch<FT>(ctx, s);
  launch_topo_passA<FT>(P, Yc, Yf, lap, s);
  launch_dss<FT>(P, lap, nullptr, s);
  launch_topo_passB<FT>(P, Yc, Yf, lap, tec(0), tef(0), s);
  launch_dss<FT>(P, tec(0), tef(0), s);
  for (int i = 1; i < 4; ++i) {
    StageArgs<FT> A{};
    A.un_c = Yc; A.un_f = Yf;
    A.nsrc = i;
    for (int j = 0; j < i; ++j) {
      A.te_c[j] = I->ae[i][j] != 0 ? tec(j) : nullptr;
      A.te_f[j] = I->ae[i][j] != 0 ? tef(j) : nullptr;
      A.ce[j] = dt * (FT)I->ae[i][j];
      A.ti_c[j] = I->ai[i][j] != 0 ? tic(j) : nullptr;
      A.ti_f[j] = I->ai[i][j] != 0 ? tif(j) : nullptr;
      A.ci[j] = dt * (FT)I->ai[i][j];
    }
    A.U_c = Uc; A.U_f = Uf;
    A.Ti_c = tic(i); A.Ti_f = tif(i);
    A.dtg = dt * (FT)I->ai[i][i];
    A.idtg = (FT)1 / A.dtg;
    A.rnorm = (double *)I->rnorm.p;
    A.first = i == 1;
    launch_column_stage<FT>(P, A, s);
    launch_topo_passA<FT>(P, Uc, Uf, lap, s);
    launch_dss<FT>(P, lap, nullptr, s);
    if (i == 3 && I->stiffly_accurate) {
      // the final combination folded into the last pass B, as in the flat step; the last
      // implicit tendency is inside U_4, and the DSS of the whole sum replaces its DSS
      FT *const c4[4] = {tec(0), tec(1), tec(2), tec(3)}, *const f4[4] = {tef(0), tef(1), tef(2), tef(3)};
      const FinArgs<FT> F = fin_args<FT>(I, dt, c4, f4);
      launch_topo_passB<FT>(P, Uc, Uf, lap, Yc, Yf, s, &F);
      launch_dss<FT>(P, Yc, Yf, s);
      launch_topo_filter<FT>(P, Yc, Yf, s);
      return;
    }
    launch_dss_reduced<FT>(P, tic(i), tif(i), s);
    launch_topo_passB<FT>(P, Uc, Uf, lap, tec(i), tef(i), s);
    launch_dss<FT>(P, tec(i), tef(i), s);
  }
  StageArgs<FT> A{};
  A.nsrc = 4;
  for (int j = 0; j < 4; ++j) {
    A.te_c[j] = I->be[j] != 0 ? tec(j) : nullptr;
    A.te_f[j] = I->be[j] != 0 ? tef(j) : nullptr;
    A.ce[j] = dt * (FT)I->be[j];
    A.ti_c[j] = I->bi[j] != 0 ? tic(j) : nullptr;
    A.ti_f[j] = I->bi[j] != 0 ? tif(j) : nullptr;
    A.ci[j] = dt * (FT)I->bi[j];
  }
  launch_final<FT>(P, A, Yc, Yf, s);
  launch_dss<FT>(P, Yc, Yf, s);
  launch_topo_filter<FT>(P, Yc, Yf, s);
}

template <class FT>
void enqueue_step(gb_ctx *ctx, FT *Yc, FT *Yf, double dt_, cudaStream_t s) {
  Impl<FT> *I = impl<FT>(ctx);
  if (I->P.topo) return enqueue_step_topo<FT>(ctx, Yc, Yf, dt_, s);
  const DevParams<FT> &P = I->P;
  const FT dt = (FT)dt_;
  FT *lap = (FT *)I->lap.p;
  auto tec = [&](int j) { return (FT *)I->Te[j].p; };
  auto tef = [&](int j) { return (FT *)I->Te[j].p + I->NC; };
  auto tic = [&](int j) { return (FT *)I->Ti[j].p; };
  auto tif = [&](int j) { return (FT *)I->Ti[j].p + I->NR; };
  FT *Uc = (FT *)I->U.p, *Uf = Uc + I->NC;
  poison_scratch<FT>(ctx, s);
  // stage 1: U_1 = u_n
  launch_passA<FT>(P, Yc, Yf, lap, s);
  launch_dss<FT>(P, lap, nullptr, s);
  launch_passB<FT>(P, Yc, Yf, lap, tec(0), tef(0), s);
  launch_dss<FT>(P, tec(0), tef(0), s);
  for (int i = 1; i < 4; ++i) {
    StageArgs<FT> A{};
    A.un_c = Yc; A.un_f = Yf;
    A.nsrc = i;
    for (int j = 0; j < i; ++j) {
      A.te_c[j] = I->ae[i][j] != 0 ? tec(j) : nullptr;
      A.te_f[j] = I->ae[i][j] != 0 ? tef(j) : nullptr;
      A.ce[j] = dt * (FT)I->ae[i][j];
      A.ti_c[j] = I->ai[i][j] != 0 ? tic(j) : nullptr;
      A.ti_f[j] = I->ai[i][j] != 0 ? tif(j) : nullptr;
      A.ci[j] = dt * (FT)I->ai[i][j];
    }
    A.U_c = Uc; A.U_f = Uf;
    A.Ti_c = tic(i); A.Ti_f = tif(i);
    A.dtg = dt * (FT)I->ai[i][i];
    A.idtg = (FT)1 / A.dtg;
    A.rnorm = (double *)I->rnorm.p;
    A.first = i == 1;
    launch_column_stage<FT>(P, A, s);
    launch_passA<FT>(P, Uc, Uf, lap, s);
    launch_dss<FT>(P, lap, nullptr, s);
    if (i == 3 && I->stiffly_accurate) {
      FT *const c4[4] = {tec(0), tec(1), tec(2), tec(3)}, *const f4[4] = {tef(0), tef(1), tef(2), tef(3)};
      const FinArgs<FT> F = fin_args<FT>(I, dt, c4, f4);
      launch_passB<FT>(P, Uc, Uf, lap, Yc, Yf, s, &F);
      launch_dss<FT>(P, Yc, Yf, s);
      return;
    }
    launch_passB<FT>(P, Uc, Uf, lap, tec(i), tef(i), s);
    launch_dss<FT>(P, tec(i), tef(i), s);
  }
  StageArgs<FT> A{};
  A.nsrc = 4;
  for (int j = 0; j < 4; ++j) {
    A.te_c[j] = I->be[j] != 0 ? tec(j) : nullptr;
    A.te_f[j] = I->be[j] != 0 ? tef(j) : nullptr;
    A.ce[j] = dt * (FT)I->be[j];
    A.ti_c[j] = I->bi[j] != 0 ? tic(j) : nullptr;
    A.ti_f[j] = I->bi[j] != 0 ? tif(j) : nullptr;
    A.ci[j] = dt * (FT)I->bi[j];
  }
  launch_final<FT>(P, A, Yc, Yf, s);
}

// Run the launches enqueue(stream) as a CUDA graph: captured (on the private capture stream)
// when g holds none for the arguments (a, b, dt), then launched on the context's stream.
template <class FT, class F>
int graph_run(gb_ctx *ctx, typename Impl<FT>::Graph &g, const void *a, const void *b, double dt, F &&enqueue) {
  Impl<FT> *I = impl<FT>(ctx);
  if (!g.exec || g.a != a || g.b != b || g.dt != dt) {
    if (g.exec) { cudaGraphExecDestroy(g.exec); g.exec = nullptr; }
    if (!I->cap) CK(cudaStreamCreateWithFlags(&I->cap, cudaStreamNonBlocking));
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(I->cap, cudaStreamCaptureModeThreadLocal));
    enqueue(I->cap);
    cudaError_t le = cudaGetLastError();
    cudaError_t ce = cudaStreamEndCapture(I->cap, &graph);
    if (le != cudaSuccess) return fail(ctx, GB_ERR_CUDA, std::string("capture launch: ") + cudaGetErrorString(le));
    if (ce != cudaSuccess) return fail(ctx, GB_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ce));
    cudaError_t ie = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) { g.exec = nullptr; return fail(ctx, GB_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie)); }
    g.a = a; g.b = b; g.dt = dt;
  }
  CK(cudaGraphLaunch(g.exec, ctx->stream));
  return GB_OK;
}

template <class FT>
int step_t(gb_ctx *ctx, gb_fieldvec Y, double dt, int nsteps, int use_graph) {
  Impl<FT> *I = impl<FT>(ctx);
  FT *Yc = (FT *)Y.c, *Yf = (FT *)Y.f;
  if (!use_graph) {
    for (int s = 0; s < nsteps; ++s) enqueue_step<FT>(ctx, Yc, Yf, dt, ctx->stream);
    return check_launch(ctx);
  }
  if (!I->gexec || I->g_c != Y.c || I->g_f != Y.f || I->g_dt != dt) {
    if (I->gexec) { cudaGraphExecDestroy(I->gexec); I->gexec = nullptr; }
    // capture on a private stream (the caller's stream may be the legacy
    // default stream, which cannot be captured); replay on the caller's stream
    if (!I->cap) CK(cudaStreamCreateWithFlags(&I->cap, cudaStreamNonBlocking));
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(I->cap, cudaStreamCaptureModeThreadLocal));
    enqueue_step<FT>(ctx, Yc, Yf, dt, I->cap);
    cudaError_t le = cudaGetLastError();
    cudaError_t ce = cudaStreamEndCapture(I->cap, &graph);
    if (le != cudaSuccess) return fail(ctx, GB_ERR_CUDA, std::string("capture launch: ") + cudaGetErrorString(le));
    if (ce != cudaSuccess) return fail(ctx, GB_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ce));
    cudaError_t ie = cudaGraphInstantiate(&I->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) { I->gexec = nullptr; return fail(ctx, GB_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie)); }
    I->g_c = Y.c; I->g_f = Y.f; I->g_dt = dt;
  }
  for (int s = 0; s < nsteps; ++s) CK(cudaGraphLaunch(I->gexec, ctx->stream));
  return GB_OK;
}

template <class FT>
int read_status(gb_ctx *ctx) {
  Impl<FT> *I = impl<FT>(ctx);
  int st = 0;
  CK(cudaMemcpyAsync(&st, I->status.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (st) CK(cudaMemsetAsync(I->status.p, 0, sizeof(int), ctx->stream));  // reported once
  if (st & ST_TIMEOUT) return fail(ctx, GB_ERR_TIMEOUT, "a bounded device wait timed out");
  if (st & ST_NONFINITE) return fail(ctx, GB_ERR_NONFINITE, "non-finite Newton residual");
  return GB_OK;
}

// The integrals of rho and rho e_tot, and (moist) of rho q_tot: nout of them are copied out.
template <class FT>
int global_sums_t(gb_ctx *ctx, gb_fieldvec Y, double *out, int nout) {
  Impl<FT> *I = impl<FT>(ctx);
  launch_global_sums<FT>(I->P, (const FT *)Y.c, (double *)I->partials.p, I->nsum_blocks, (double *)I->sums.p, ctx->stream);
  int r = check_launch(ctx);
  if (r) return r;
  CK(cudaMemcpyAsync(out, I->sums.p, nout * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return GB_OK;
}

template <class FT>
int residual_t(gb_ctx *ctx, double *out) {
  Impl<FT> *I = impl<FT>(ctx);
  launch_reduce_rnorm<FT>((const double *)I->rnorm.p, I->P.Nh * NN, (double *)I->rsum.p, ctx->stream);
  int r = check_launch(ctx);
  if (r) return r;
  CK(cudaMemcpyAsync(out, I->rsum.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return read_status<FT>(ctx);
}

template <class FT>
int ensure_adjoint(gb_ctx *ctx);
template <class FT>
StageArgs<FT> single_stage_args(Impl<FT> *I, const FT *Uhc, const FT *Uhf, double dtg);

template <class FT>
int time_kernel_t(gb_ctx *ctx, int kernel, gb_fieldvec Y, int reps, double *ms) {
  Impl<FT> *I = impl<FT>(ctx);
  const DevParams<FT> &P = I->P;
  cudaStream_t s = ctx->stream;
  FT *Yc = (FT *)Y.c, *Yf = (FT *)Y.f;
  FT *lap = (FT *)I->lap.p;
  FT *Tc = (FT *)I->Te[0].p, *Tf = Tc + I->NC;
  StageArgs<FT> A{};
  const FT dt = (FT)ctx->cfg.dt;
  if (kernel == GB_K_COLUMN || kernel == GB_K_FINAL) {
    const int i = kernel == GB_K_COLUMN ? 3 : 4;
    A.un_c = Yc; A.un_f = Yf; A.nsrc = i;
    for (int j = 0; j < i; ++j) {
      const double e = i < 4 ? I->ae[i][j] : I->be[j], m = i < 4 ? I->ai[i][j] : I->bi[j];
      A.te_c[j] = e != 0 ? (FT *)I->Te[j].p : nullptr;
      A.te_f[j] = e != 0 ? (FT *)I->Te[j].p + I->NC : nullptr;
      A.ce[j] = dt * (FT)e;
      A.ti_c[j] = m != 0 ? (FT *)I->Ti[j].p : nullptr;
      A.ti_f[j] = m != 0 ? (FT *)I->Ti[j].p + I->NR : nullptr;
      A.ci[j] = dt * (FT)m;
    }
    A.U_c = (FT *)I->U.p; A.U_f = (FT *)I->U.p + I->NC;
    A.Ti_c = (FT *)I->Ti[3].p; A.Ti_f = (FT *)I->Ti[3].p + I->NR;
    A.dtg = dt * (FT)I->ai[3][3];
    A.idtg = (FT)1 / A.dtg;
    A.rnorm = (double *)I->rnorm.p;
    A.first = 1;
  }
  // reverse kernels: cotangent inputs are the tendency and Laplacian buffers of
  // the last step (finite values), outputs the reverse-mode scratch
  const bool rev = kernel >= GB_K_PASSA_VJP && kernel <= GB_K_DSS_T;
  if (P.topo && (rev || kernel == GB_K_PASSB_FINAL))
    return fail(ctx, GB_ERR_ARG, "gb_time_kernel: the reverse kernels and the folded final pass are not built over terrain");
  if (rev) {
    int r = ensure_adjoint<FT>(ctx);
    if (r) return r;
  }
  FT *Ubc = rev ? (FT *)I->adj->Ub.p : nullptr, *Ubf = rev ? Ubc + I->NC : nullptr;
  FT *Lbc = rev ? (FT *)I->adj->Lb.p : nullptr;
  StageArgs<FT> SA{};
  // the implicit-tendency cotangent input: stage 1's buffer (stage 0 has no implicit tendency)
  if (kernel == GB_K_COLUMN_VJP) {
    if (!I->Ti[1].p) return fail(ctx, GB_ERR_ARG, "implicit tendency buffers not allocated");
    SA = single_stage_args<FT>(I, Yc, Yf, (double)dt * I->ai[1][1]);
  }
  FT *Teb[4] = {rev ? (FT *)I->adj->dummy.p : nullptr, nullptr, nullptr, nullptr};
  FT *Tibs[4] = {nullptr, nullptr, nullptr, nullptr};
  auto launch = [&]() {
    switch (kernel) {
      case GB_K_PASSA:
        if (P.topo) launch_topo_passA<FT>(P, Yc, Yf, lap, s);
        else launch_passA<FT>(P, Yc, Yf, lap, s);
        break;
      case GB_K_PASSB:
        if (P.topo) launch_topo_passB<FT>(P, Yc, Yf, lap, Tc, Tf, s);
        else launch_passB<FT>(P, Yc, Yf, lap, Tc, Tf, s);
        break;
      case GB_K_COLUMN: launch_column_stage<FT>(P, A, s); break;
      case GB_K_DSS: launch_dss<FT>(P, Yc, Yf, s); break;
      case GB_K_PASSA_VJP: launch_passA_vjp<FT>(P, Yc, Yf, lap, Ubc, Ubf, I->adj->grid, s); break;
      case GB_K_PASSB_VJP:
        launch_passB_vjp<FT>(P, Yc, Yf, lap, Tc, Tf, Ubc, Ubf, Lbc, (double *)I->adj->dparB.p, I->adj->grid, false, s);
        break;
      case GB_K_COLUMN_VJP:
        // as in a reverse step: the stage's recorded output and implicit tendency given
        // (here the stage buffer and the last implicit tendency; finite values)
        launch_column_stage_vjp<FT>(P, SA, Tc, Tf, (const FT *)I->Ti[1].p, (const FT *)I->Ti[1].p + I->NR, Ubc, Ubf,
                                    Teb, Tibs, I->NC, I->NR, (FT *)I->adj->scr.p, (double *)I->adj->dal.p, s,
                                    (const FT *)I->U.p, (const FT *)I->Ti[3].p);
        break;
      case GB_K_DSS_T: launch_dss_transpose<FT>(P, Ubc, Ubf, s); break;
      case GB_K_PASSB_FINAL: {
        // U = Y + the final combination's terms; Y and the tendency buffers are read
        FT *const c4[4] = {(FT *)I->Te[0].p, (FT *)I->Te[1].p, (FT *)I->Te[2].p, (FT *)I->Te[3].p};
        FT *const f4[4] = {c4[0] + I->NC, c4[1] + I->NC, c4[2] + I->NC, c4[3] + I->NC};
        const FinArgs<FT> F = fin_args<FT>(I, dt, c4, f4);
        launch_passB<FT>(P, Yc, Yf, lap, (FT *)I->U.p, (FT *)I->U.p + I->NC, s, &F);
        break;
      }
      default: launch_final<FT>(P, A, (FT *)I->U.p, (FT *)I->U.p + I->NC, s); break;
    }
  };
  launch();  // warm-up
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  CK(cudaEventRecord(a, s));
  for (int r = 0; r < reps; ++r) launch();
  CK(cudaEventRecord(b, s));
  int rc = check_launch(ctx);
  CK(cudaEventSynchronize(b));
  float t = 0;
  CK(cudaEventElapsedTime(&t, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = reps > 0 ? t / reps : 0.0;
  return rc;
}

// Device address of g_noalloc_scratch on the current device, resolved once per
// device (with that device current) on the first call.
constexpr int NOALLOC_MAX_DEVICES = 64;
void *g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};
std::mutex g_noalloc_mu;

// ---------------------------------------------------------------- reverse mode
template <class FT>
int alloc_z(gb_ctx *ctx, DevBuf &b, size_t bytes, size_t &total) {
  int r = alloc(ctx, b, bytes);
  total += bytes;
  return r;
}

template <class FT>
int ensure_adjoint(gb_ctx *ctx) {
  Impl<FT> *I = impl<FT>(ctx);
  if (I->adj) return GB_OK;
  int dev = 0, optin = 0, nsm = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  if (passB_vjp_smem<FT>(I->P.Nv) > (size_t)optin ||
      passA_vjp_smem<FT>(I->P.Nv) > (size_t)optin)
    return fail(ctx, GB_ERR_ARG, "z_elem too large for the reverse-mode slab kernels at this precision (shared memory)");
  configure_adjoint_se<FT>(I->P.Nv);
  auto A = std::make_unique<typename Impl<FT>::Adjoint>();
  const size_t S = (I->NC + I->NF) * sizeof(FT), R = (I->NR + I->NF) * sizeof(FT);
  const int ncols = I->P.Nh * NN;
  A->grid = std::min(I->P.Nh, 4 * nsm);  // parameter-partial slots: at most 4 resident CTAs per SM
  size_t &t = A->bytes;
  int r;
  if ((r = alloc_z<FT>(ctx, A->Ub, S, t)) ||
      (r = alloc_z<FT>(ctx, A->Lb, I->NC * sizeof(FT), t)) || (r = alloc_z<FT>(ctx, A->zero, S, t)) ||
      (r = alloc_z<FT>(ctx, A->dummy, S, t)) || (r = alloc_z<FT>(ctx, A->work, S, t)) ||
      (r = alloc_z<FT>(ctx, A->scr, col_vjp_scratch_words(I->P.Nh, I->P.Nv) * sizeof(FT), t)) ||
      (r = alloc_z<FT>(ctx, A->dparB, (size_t)A->grid * 2 * sizeof(double), t)) ||
      (r = alloc_z<FT>(ctx, A->dal, (size_t)ncols * sizeof(double), t)) ||
      (r = alloc_z<FT>(ctx, A->dacc, 4 * sizeof(double), t)))
    return r;
  for (int j = 0; j < 4; ++j)
    if ((r = alloc_z<FT>(ctx, A->Teb[j], S, t))) return r;
  for (int j = 1; j < 4; ++j)
    if ((r = alloc_z<FT>(ctx, A->Tib[j], R, t))) return r;
  I->adj = std::move(A);
  return GB_OK;
}

template <class FT>
int ensure_records(gb_ctx *ctx, int n) {
  Impl<FT> *I = impl<FT>(ctx);
  auto &A = *I->adj;
  const size_t S = (I->NC + I->NF) * sizeof(FT), R = (I->NR + I->NF) * sizeof(FT), L = I->NC * sizeof(FT);
  while ((int)A.rec.size() < n) {
    auto rc = std::make_unique<typename Impl<FT>::Record>();
    size_t t = 0;
    int r;
    if ((r = alloc_z<FT>(ctx, rc->Y, S, t))) return r;
    for (int i = 0; i < 4; ++i) {
      if ((r = alloc_z<FT>(ctx, rc->L[i], L, t)) || (r = alloc_z<FT>(ctx, rc->Te[i], S, t))) return r;
      if (i >= 1 && ((r = alloc_z<FT>(ctx, rc->U[i], S, t)) || (r = alloc_z<FT>(ctx, rc->Ti[i], R, t)))) return r;
    }
    A.rec_bytes = t;
    A.bytes += t;
    A.rec.push_back(std::move(rc));
  }
  return GB_OK;
}

// Sources of implicit stage i (1..3) as the fused step assembles them.
template <class FT>
StageArgs<FT> stage_args(Impl<FT> *I, int i, FT dt, const FT *Yc, const FT *Yf, FT *const Te[4], FT *const Ti[4]) {
  StageArgs<FT> A{};
  A.un_c = Yc; A.un_f = Yf;
  A.nsrc = i;
  for (int j = 0; j < i; ++j) {
    A.te_c[j] = I->ae[i][j] != 0 ? Te[j] : nullptr;
    A.te_f[j] = I->ae[i][j] != 0 ? Te[j] + I->NC : nullptr;
    A.ce[j] = dt * (FT)I->ae[i][j];
    A.ti_c[j] = I->ai[i][j] != 0 ? Ti[j] : nullptr;
    A.ti_f[j] = I->ai[i][j] != 0 ? Ti[j] + I->NR : nullptr;
    A.ci[j] = dt * (FT)I->ai[i][j];
  }
  A.dtg = dt * (FT)I->ai[i][i];
  A.idtg = (FT)1 / A.dtg;
  A.rnorm = (double *)I->rnorm.p;
  A.first = i == 1;
  return A;
}

// One fused ARS343 step on Y (the arithmetic of enqueue_step) that keeps the
// stage states, Laplacians and tendencies in rec.
template <class FT>
void record_step(gb_ctx *ctx, FT *Yc, FT *Yf, double dt_, typename Impl<FT>::Record &rec, cudaStream_t s) {
  Impl<FT> *I = impl<FT>(ctx);
  const DevParams<FT> &P = I->P;
  const FT dt = (FT)dt_;
  cudaMemcpyAsync(rec.Y.p, Yc, I->NC * sizeof(FT), cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync((FT *)rec.Y.p + I->NC, Yf, I->NF * sizeof(FT), cudaMemcpyDeviceToDevice, s);
  FT *Te[4], *Ti[4] = {nullptr, nullptr, nullptr, nullptr};
  for (int j = 0; j < 4; ++j) {
    Te[j] = (FT *)rec.Te[j].p;
    if (j >= 1) Ti[j] = (FT *)rec.Ti[j].p;
  }
  for (int i = 0; i < 4; ++i) {
    FT *Uc = Yc, *Uf = Yf;
    if (i >= 1) {
      StageArgs<FT> A = stage_args<FT>(I, i, dt, Yc, Yf, Te, Ti);
      Uc = (FT *)rec.U[i].p;
      Uf = Uc + I->NC;
      A.U_c = Uc; A.U_f = Uf;
      A.Ti_c = Ti[i]; A.Ti_f = Ti[i] + I->NR;
      launch_column_stage<FT>(P, A, s);
    }
    FT *L = (FT *)rec.L[i].p;
    launch_passA<FT>(P, Uc, Uf, L, s);
    launch_dss<FT>(P, L, nullptr, s);
    if (i == 3 && I->stiffly_accurate) {
      // as enqueue_step (the reverse pass reads no T_exp of the last stage)
      FT *const c4[4] = {Te[0], Te[1], Te[2], Te[3]};
      FT *const f4[4] = {Te[0] + I->NC, Te[1] + I->NC, Te[2] + I->NC, Te[3] + I->NC};
      const FinArgs<FT> F = fin_args<FT>(I, dt, c4, f4);
      launch_passB<FT>(P, Uc, Uf, L, Yc, Yf, s, &F);
      launch_dss<FT>(P, Yc, Yf, s);
      return;
    }
    launch_passB<FT>(P, Uc, Uf, L, Te[i], Te[i] + I->NC, s);
    launch_dss<FT>(P, Te[i], Te[i] + I->NC, s);
  }
  StageArgs<FT> A{};
  A.nsrc = 4;
  for (int j = 0; j < 4; ++j) {
    A.te_c[j] = I->be[j] != 0 ? Te[j] : nullptr;
    A.te_f[j] = I->be[j] != 0 ? Te[j] + I->NC : nullptr;
    A.ce[j] = dt * (FT)I->be[j];
    A.ti_c[j] = I->bi[j] != 0 && Ti[j] ? Ti[j] : nullptr;
    A.ti_f[j] = I->bi[j] != 0 && Ti[j] ? Ti[j] + I->NR : nullptr;
    A.ci[j] = dt * (FT)I->bi[j];
  }
  launch_final<FT>(P, A, Yc, Yf, s);
}

// Reverse of the explicit tendency of one stage state U: Ub (+)= (dT/dU)^T Tb,
// where Tb is the cotangent of the DSSed tendency (dss_out, as inside the step;
// Tb is then DSS-transposed in place) or of the tendency as
// gb_remaining_tendency returns it (not DSSed; Tb is only read).  accum adds
// to Ub, else Ub is overwritten.  With Yc_add: Yc_add (+)= (dT/dU)^T Tb instead,
// Ub being scratch (pass B^T writes it, pass A^T adds it and its own part).  The
// cotangent is tsc Tb (pass B^T scales its outputs).
template <class FT>
void tendency_vjp(gb_ctx *ctx, const FT *Uc, const FT *Uf, const FT *L, FT *Tb_c, FT *Tb_f, FT *Ubc, FT *Ubf,
                  bool dss_out, bool accum, cudaStream_t s, FT *Yc_add = nullptr, FT *Yf_add = nullptr,
                  FT tsc = FT(1)) {
  Impl<FT> *I = impl<FT>(ctx);
  auto &A = *I->adj;
  const DevParams<FT> &P = I->P;
  FT *Lb = (FT *)A.Lb.p;
  if (dss_out) launch_dss_transpose<FT>(P, Tb_c, Tb_f, s);
  if (Yc_add && passA_vjp_add_fits<FT>(P.Nv)) {
    launch_passB_vjp<FT>(P, Uc, Uf, L, Tb_c, Tb_f, Ubc, Ubf, Lb, (double *)A.dparB.p, A.grid, false, s, tsc);
    launch_dss_transpose<FT>(P, Lb, nullptr, s);
    launch_passA_vjp<FT>(P, Uc, Uf, Lb, Yc_add, Yf_add, A.grid, s, Ubc, Ubf);
    return;
  }
  if (Yc_add) {
    Ubc = Yc_add;
    Ubf = Yf_add;
    accum = true;
  }
  launch_passB_vjp<FT>(P, Uc, Uf, L, Tb_c, Tb_f, Ubc, Ubf, Lb, (double *)A.dparB.p, A.grid, accum, s, tsc);
  launch_dss_transpose<FT>(P, Lb, nullptr, s);
  launch_passA_vjp<FT>(P, Uc, Uf, Lb, Ubc, Ubf, A.grid, s);
}

// Reverse of one recorded step: Yb holds the cotangent of u_{n+1} on entry and
// that of u_n on return; d/dnu and d/d(sponge rate) accumulate in dacc.
template <class FT>
void reverse_step(gb_ctx *ctx, typename Impl<FT>::Record &rec, double dt_, FT *Ybc, FT *Ybf, cudaStream_t s) {
  Impl<FT> *I = impl<FT>(ctx);
  auto &A = *I->adj;
  const DevParams<FT> &P = I->P;
  const FT dt = (FT)dt_;
  FT *Teb[4], *Tib[4] = {nullptr, nullptr, nullptr, nullptr}, *Te[4], *Ti[4] = {nullptr, nullptr, nullptr, nullptr};
  for (int j = 0; j < 4; ++j) {
    Teb[j] = (FT *)A.Teb[j].p;
    Te[j] = (FT *)rec.Te[j].p;
    if (j >= 1) {
      Tib[j] = (FT *)A.Tib[j].p;
      Ti[j] = (FT *)rec.Ti[j].p;
    }
  }
  // final combination u_{n+1} = u_n + dt sum_j b_j (T_exp_j + T_imp_j), filtered.  Its
  // transpose gives every tendency j the cotangent dt b_j Ybar: written here for the last
  // stage only; the last stage's column pullback writes those of the earlier stages
  // (dt b_j Ybar plus its own part, Ybar read once).
  CotArgs<FT> F{};
  F.nsrc = 4;
  FT e0[4], i0[4];
  for (int j = 0; j < 4; ++j) {
    F.te_c[j] = j == 3 ? Teb[j] : nullptr;
    F.te_f[j] = j == 3 ? Teb[j] + I->NC : nullptr;
    F.ce[j] = dt * (FT)I->be[j];
    F.ti_c[j] = j == 3 ? Tib[j] : nullptr;
    F.ti_f[j] = j == 3 ? Tib[j] + I->NR : nullptr;
    F.ci[j] = dt * (FT)I->bi[j];
    e0[j] = F.ce[j];
    i0[j] = F.ci[j];
  }
  // the step's own final DSS (the combination folded into the last pass B, then
  // DSSed as a whole): its transpose first, then that of the impenetrability filter.
  // The last stage's tendency cotangents, dt b~_4 Ybar and dt b_4 Ybar, are then not
  // materialised: its pullbacks read Ybar in place with those factors, and they need no
  // second transposed DSS (the DSS is a projection).
  const bool fold = I->stiffly_accurate;
  if (fold) {
    launch_dss_transpose<FT>(P, Ybc, Ybf, s);
    launch_bc_filter<FT>(P, Ybf, s);
  } else {
    launch_final_transpose<FT>(P, F, Ybc, Ybf, s);
  }
  const FT *Yc = (const FT *)rec.Y.p, *Yf = Yc + I->NC;
  FT *Ubc = (FT *)A.Ub.p, *Ubf = Ubc + I->NC;
  for (int i = 3; i >= 0; --i) {
    const FT *Uc = i == 0 ? Yc : (const FT *)rec.U[i].p, *Uf = Uc + I->NC;
    if (i == 0) {
      // stage 0 is u_n itself: its tendency cotangent adds straight into the caller's Yb
      tendency_vjp<FT>(ctx, Uc, Uf, (const FT *)rec.L[i].p, Teb[i], Teb[i] + I->NC, Ubc, Ubf, true, false, s, Ybc,
                       Ybf);
    } else {
      const bool last = i == 3 && fold;
      if (last)
        tendency_vjp<FT>(ctx, Uc, Uf, (const FT *)rec.L[i].p, Ybc, Ybf, Ubc, Ubf, false, false, s, nullptr, nullptr,
                         F.ce[3]);
      else
        tendency_vjp<FT>(ctx, Uc, Uf, (const FT *)rec.L[i].p, Teb[i], Teb[i] + I->NC, Ubc, Ubf, true, false, s);
      const StageArgs<FT> SA = stage_args<FT>(I, i, dt, Yc, Yf, Te, Ti);
      launch_column_stage_vjp<FT>(P, SA, Ubc, Ubf, Tib[i], Tib[i] + I->NR, Ybc, Ybf, Teb, Tib, I->NC, I->NR,
                                  (FT *)A.scr.p, (double *)A.dal.p, s, (const FT *)rec.U[i].p,
                                  (const FT *)rec.Ti[i].p, i == 3 ? e0 : nullptr, i == 3 ? i0 : nullptr,
                                  last ? &F.ci[3] : nullptr);
    }
  }
}

template <class FT>
int dss_transpose_t(gb_ctx *ctx, gb_fieldvec X) {
  launch_dss_transpose<FT>(impl<FT>(ctx)->P, (FT *)X.c, (FT *)X.f, ctx->stream);
  return check_launch(ctx);
}

// Zero the parameter partials (per-CTA of the pass B reverse, per column of
// the column reverse) at the start of a reverse pass.
template <class FT>
void zero_dpar(gb_ctx *ctx, cudaStream_t s) {
  auto &A = *impl<FT>(ctx)->adj;
  cudaMemsetAsync(A.dacc.p, 0, 4 * sizeof(double), s);
  cudaMemsetAsync(A.dparB.p, 0, (size_t)A.grid * 2 * sizeof(double), s);
  cudaMemsetAsync(A.dal.p, 0, (size_t)impl<FT>(ctx)->P.Nh * NN * sizeof(double), s);
}

// Reduce the partials (fixed order) and read (d/dnu, d/d rate).
template <class FT>
int read_dacc(gb_ctx *ctx, double *dpar, bool add) {
  Impl<FT> *I = impl<FT>(ctx);
  auto &A = *I->adj;
  launch_accum((const double *)A.dparB.p, A.grid, 2, 2, (double *)A.dacc.p, ctx->stream);
  launch_accum_slots<FT>((const double *)A.dal.p, I->P.Nh * NN, (double *)A.dacc.p + 1, ctx->stream);
  double h[2];
  CK(cudaMemcpyAsync(h, I->adj->dacc.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (dpar) {
    dpar[0] = (add ? dpar[0] : 0.0) + h[0];
    dpar[1] = (add ? dpar[1] : 0.0) + h[1];
  }
  return GB_OK;
}

template <class FT>
int remaining_tendency_vjp_t(gb_ctx *ctx, gb_fieldvec Yb, gb_fieldvec Tb, gb_fieldvec Y, double *dpar) {
  int r = ensure_adjoint<FT>(ctx);
  if (r) return r;
  Impl<FT> *I = impl<FT>(ctx);
  cudaStream_t s = ctx->stream;
  zero_dpar<FT>(ctx, s);
  // forward Laplacians at Y (DSSed), then the reverse
  FT *L = (FT *)I->lap.p;
  launch_passA<FT>(I->P, (const FT *)Y.c, (const FT *)Y.f, L, s);
  launch_dss<FT>(I->P, L, nullptr, s);
  tendency_vjp<FT>(ctx, (const FT *)Y.c, (const FT *)Y.f, L, (FT *)Tb.c, (FT *)Tb.f, (FT *)Yb.c, (FT *)Yb.f, false,
                   true, s);
  if ((r = check_launch(ctx))) return r;
  return read_dacc<FT>(ctx, dpar, true);
}

template <class FT>
StageArgs<FT> single_stage_args(Impl<FT> *I, const FT *Uhc, const FT *Uhf, double dtg) {
  // U^ given directly: one source, the zero field, with coefficient 0
  StageArgs<FT> A{};
  A.un_c = Uhc; A.un_f = Uhf;
  A.nsrc = 1;
  A.te_c[0] = (const FT *)I->adj->zero.p;
  A.te_f[0] = (const FT *)I->adj->zero.p + I->NC;
  A.ce[0] = FT(0);
  A.dtg = (FT)dtg;
  A.idtg = (FT)1 / A.dtg;
  A.rnorm = (double *)I->rnorm.p;
  A.first = 1;
  return A;
}

template <class FT>
int implicit_stage_t(gb_ctx *ctx, gb_fieldvec U, gb_fieldvec Ti, gb_fieldvec Uh, double dtg) {
  int r = ensure_adjoint<FT>(ctx);
  if (r) return r;
  Impl<FT> *I = impl<FT>(ctx);
  StageArgs<FT> A = single_stage_args<FT>(I, (const FT *)Uh.c, (const FT *)Uh.f, dtg);
  A.U_c = (FT *)U.c; A.U_f = (FT *)U.f;
  A.Ti_c = (FT *)Ti.c; A.Ti_f = (FT *)Ti.f;
  launch_column_stage<FT>(I->P, A, ctx->stream);
  return check_launch(ctx);
}

template <class FT>
int implicit_stage_vjp_t(gb_ctx *ctx, gb_fieldvec Uhb, gb_fieldvec Ub, gb_fieldvec Tib, gb_fieldvec Uh, double dtg,
                         double *dpar) {
  int r = ensure_adjoint<FT>(ctx);
  if (r) return r;
  Impl<FT> *I = impl<FT>(ctx);
  cudaStream_t s = ctx->stream;
  zero_dpar<FT>(ctx, s);
  const StageArgs<FT> A = single_stage_args<FT>(I, (const FT *)Uh.c, (const FT *)Uh.f, dtg);
  FT *Teb[4] = {(FT *)I->adj->dummy.p, nullptr, nullptr, nullptr}, *Tibs[4] = {nullptr, nullptr, nullptr, nullptr};
  launch_column_stage_vjp<FT>(I->P, A, (const FT *)Ub.c, (const FT *)Ub.f, (const FT *)Tib.c, (const FT *)Tib.f,
                              (FT *)Uhb.c, (FT *)Uhb.f, Teb, Tibs, I->NC, I->NR, (FT *)I->adj->scr.p,
                              (double *)I->adj->dal.p, s);
  if ((r = check_launch(ctx))) return r;
  return read_dacc<FT>(ctx, dpar, true);
}

template <class FT>
int step_vjp_t(gb_ctx *ctx, gb_fieldvec Yb, gb_fieldvec Y, double dt, double *dpar) {
  int r = ensure_adjoint<FT>(ctx);
  if (r || (r = ensure_records<FT>(ctx, 1))) return r;
  Impl<FT> *I = impl<FT>(ctx);
  cudaStream_t s = ctx->stream;
  auto &A = *I->adj;
  FT *W = (FT *)A.work.p;
  CK(cudaMemcpyAsync(W, Y.c, I->NC * sizeof(FT), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(W + I->NC, Y.f, I->NF * sizeof(FT), cudaMemcpyDeviceToDevice, s));
  zero_dpar<FT>(ctx, s);
  A.rec_first = -1;  // record 0 is reused here
  record_step<FT>(ctx, W, W + I->NC, dt, *A.rec[0], s);
  reverse_step<FT>(ctx, *A.rec[0], dt, (FT *)Yb.c, (FT *)Yb.f, s);
  if ((r = check_launch(ctx))) return r;
  if ((r = read_dacc<FT>(ctx, dpar, true))) return r;
  return read_status<FT>(ctx);
}

template <class FT>
int adjoint_forward_t(gb_ctx *ctx, gb_fieldvec Y, double dt, int nsteps, int every) {
  int r = ensure_adjoint<FT>(ctx);
  if (r) return r;
  Impl<FT> *I = impl<FT>(ctx);
  auto &A = *I->adj;
  const size_t SB = (I->NC + I->NF) * sizeof(FT);
  const int nck = (nsteps + every - 1) / every;
  while ((int)A.ckpt.size() < nck) {
    auto b = std::make_unique<DevBuf>();
    if ((r = alloc_z<FT>(ctx, *b, SB, A.bytes))) return r;
    A.ckpt.push_back(std::move(b));
  }
  // the last `keep` segments' stage data is recorded on the way (the reverse pass starts
  // there and needs no recompute for them); the same kernels in the same order as the step.
  // Segment g (of the kept ones) uses the records from (nck - 1 - g) * every on.
  const int keep = std::max(1, std::min(A.keep, nck));
  if ((r = ensure_records<FT>(ctx, keep * every))) return r;
  const int first = nck - keep;
  A.rec_first = -1;
  cudaStream_t s = ctx->stream;
  FT *Yc = (FT *)Y.c, *Yf = (FT *)Y.f;
  for (int k = 0; k < nsteps; ++k) {
    const int g = k / every;
    if (k % every == 0) {
      FT *ck = (FT *)A.ckpt[g]->p;
      CK(cudaMemcpyAsync(ck, Yc, I->NC * sizeof(FT), cudaMemcpyDeviceToDevice, s));
      CK(cudaMemcpyAsync(ck + I->NC, Yf, I->NF * sizeof(FT), cudaMemcpyDeviceToDevice, s));
    }
    if (g >= first) {
      auto &rc = *A.rec[(nck - 1 - g) * every + (k - g * every)];
      r = graph_run<FT>(ctx, rc.fwd, Yc, Yf, dt, [&](cudaStream_t cs) { record_step<FT>(ctx, Yc, Yf, dt, rc, cs); });
      if (r) return r;
    } else {
      enqueue_step<FT>(ctx, Yc, Yf, dt, s);
    }
  }
  A.rec_first = first;
  A.nsteps = nsteps;
  A.every = every;
  A.dt = dt;
  A.ready = true;
  if ((r = check_launch(ctx))) return r;
  return read_status<FT>(ctx);
}

template <class FT>
int adjoint_reverse_t(gb_ctx *ctx, gb_fieldvec Yb, double *dpar, size_t *peak) {
  Impl<FT> *I = impl<FT>(ctx);
  if (!I->adj || !I->adj->ready) return fail(ctx, GB_ERR_STATE, "gb_adjoint_reverse called before gb_adjoint_forward");
  auto &A = *I->adj;
  int r = ensure_records<FT>(ctx, A.every);
  if (r) return r;
  cudaStream_t s = ctx->stream;
  const size_t SB = (I->NC + I->NF) * sizeof(FT);
  FT *W = (FT *)A.work.p;
  // the cotangent is carried in a library buffer, so that each record's recording and
  // reverse steps are captured once as CUDA graphs and replayed (fixed arguments)
  if (!A.yb.p && (r = alloc_z<FT>(ctx, A.yb, SB, A.bytes))) return r;
  FT *ybc = (FT *)A.yb.p, *ybf = ybc + I->NC;
  CK(cudaMemcpyAsync(ybc, Yb.c, I->NC * sizeof(FT), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(ybf, Yb.f, I->NF * sizeof(FT), cudaMemcpyDeviceToDevice, s));
  zero_dpar<FT>(ctx, s);
  const int nseg = (A.nsteps + A.every - 1) / A.every;
  for (int g = nseg - 1; g >= 0; --g) {
    const int s0 = g * A.every, s1 = std::min(A.nsteps, s0 + A.every);
    // a kept segment's records start at (nseg - 1 - g) * every; a recomputed one reuses the
    // first record set (its segment was reversed first)
    const bool kept = A.rec_first >= 0 && g >= A.rec_first;
    const int base = kept ? (nseg - 1 - g) * A.every : 0;
    if (!kept) {
      CK(cudaMemcpyAsync(W, A.ckpt[g]->p, SB, cudaMemcpyDeviceToDevice, s));
      for (int k = s0; k < s1; ++k) {
        auto &rc = *A.rec[base + k - s0];
        r = graph_run<FT>(ctx, rc.fwd, W, W + I->NC, A.dt,
                          [&](cudaStream_t cs) { record_step<FT>(ctx, W, W + I->NC, A.dt, rc, cs); });
        if (r) return r;
      }
    }
    for (int k = s1 - 1; k >= s0; --k) {
      auto &rc = *A.rec[base + k - s0];
      r = graph_run<FT>(ctx, rc.rev, ybc, ybf, A.dt,
                        [&](cudaStream_t cs) { reverse_step<FT>(ctx, rc, A.dt, ybc, ybf, cs); });
      if (r) return r;
    }
    if ((r = check_launch(ctx))) return r;
  }
  CK(cudaMemcpyAsync(Yb.c, ybc, I->NC * sizeof(FT), cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(Yb.f, ybf, I->NF * sizeof(FT), cudaMemcpyDeviceToDevice, s));
  if ((r = read_dacc<FT>(ctx, dpar, false))) return r;
  if (peak) {
    size_t base = 0;
    base += (I->NC + I->NF) * sizeof(FT) * (2 + 4) + (I->NR + I->NF) * sizeof(FT) * 3 + I->NC * sizeof(FT);
    *peak = base + A.bytes;
  }
  A.ready = false;
  return read_status<FT>(ctx);
}

int noalloc_scratch(gb_ctx *ctx, void **out) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return fail(ctx, GB_ERR_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(ctx, GB_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return GB_OK;
}

template <class FT>
int jacobian_solve_noalloc_t(gb_ctx *ctx, gb_fieldvec dY, gb_fieldvec Y, gb_fieldvec R, double dtg) {
  Impl<FT> *I = impl<FT>(ctx);
  const size_t need = (size_t)I->P.Nh * NN * (I->P.moist ? JAC_QM : JAC_Q) * I->P.Nf * sizeof(FT);
  if (need > (size_t)GB_NOALLOC_SCRATCH_BYTES)
    return fail(ctx, GB_ERR_ARG, "gb_jacobian_solve_noalloc: Jacobian needs " + std::to_string(need) +
                                     " bytes, more than GB_NOALLOC_SCRATCH_BYTES (" +
                                     std::to_string((size_t)GB_NOALLOC_SCRATCH_BYTES) + ")");
  void *scratch = nullptr;
  int r = noalloc_scratch(ctx, &scratch);
  if (r) return r;
  ColArgs<FT> A{};
  A.jac = (FT *)scratch;
  A.dtg = (FT)dtg;
  A.Y_c = (const FT *)Y.c; A.Y_f = (const FT *)Y.f;
  launch_column<FT>(I->P, COL_JACOBIAN, A, ctx->stream);
  A.Y_c = (const FT *)R.c; A.Y_f = (const FT *)R.f;
  A.O_c = (FT *)dY.c; A.O_f = (FT *)dY.f;
  launch_column<FT>(I->P, COL_LDIV, A, ctx->stream);
  return check_launch(ctx);
}

bool aligned(const void *p) { return ((uintptr_t)p & 15) == 0; }
bool fv_ok(gb_fieldvec v) { return v.c && v.f && aligned(v.c) && aligned(v.f); }

#define DISPATCH(ctx, fn, ...) ((ctx)->cfg.ft_bytes == 8 ? fn<double>(__VA_ARGS__) : fn<float>(__VA_ARGS__))

#define GUARD(ctx)                                           \
  do {                                                       \
    if (!(ctx)) return GB_ERR_ARG;                           \
  } while (0)

// Entry points not built for terrain-following levels refuse a terrain context.
#define NO_TERRAIN(ctx, what)                                                                       \
  do {                                                                                              \
    if ((ctx)->geo.topo) return fail((ctx), GB_ERR_ARG, what " is not available over terrain");   \
  } while (0)

// A moist 0M context supports the column hooks (gb_set_precomputed_quantities,
// gb_implicit_tendency, gb_update_jacobian, gb_ldiv, gb_correct_implicit_advection_tendency,
// gb_jacobian_solve_noalloc), the state DSS and the conservation sums.
#define NO_MOIST(ctx, what)                                                                            \
  do {                                                                                                 \
    if ((ctx) && (ctx)->cfg.moist) return fail((ctx), GB_ERR_ARG, what " is not available with moist = 1"); \
  } while (0)

}  // namespace

extern "C" {

int gb_sizes(const gb_config *cfg, size_t *n_center, size_t *n_face, int *n_groups, int *n_copies) {
  GB_RANGE();
  if (!cfg) return GB_ERR_ARG;
  const char *why = nullptr;
  if (!validate_config(*cfg, &why)) return GB_ERR_ARG;
  const size_t Nh = 6 * (size_t)cfg->h_elem * cfg->h_elem;
  if (n_center) *n_center = Nh * (cfg->moist ? 5 : 4) * NN * cfg->z_elem;
  if (n_face) *n_face = Nh * NN * (cfg->z_elem + 1);
  if (n_groups || n_copies || cfg->z_surface) {
    HostGeometry g;
    build_geometry(*cfg, g);
    // over terrain the warped levels must not cross
    if (!build_terrain_tables(*cfg, g, &why)) return GB_ERR_ARG;
    if (n_groups) *n_groups = (int)g.grp_off.size() - 1;
    if (n_copies) *n_copies = (int)g.grp_copy.size();
  }
  return GB_OK;
}

int gb_geometry_export(const gb_config *cfg, gb_geometry_host *out) {
  GB_RANGE();
  if (!cfg || !out) return GB_ERR_ARG;
  const char *why = nullptr;
  if (!validate_config(*cfg, &why)) return GB_ERR_ARG;
  try {
    HostGeometry g;
    build_geometry(*cfg, g);
    auto cp = [](double *dst, const std::vector<double> &v) { if (dst) std::memcpy(dst, v.data(), v.size() * sizeof(double)); };
    cp(out->xyz, g.xyz); cp(out->ecov, g.ecov); cp(out->Jh, g.Jh); cp(out->gup, g.gup); cp(out->fh0, g.fh0); cp(out->zf, g.zf);
    cp(out->econ, g.econ); cp(out->dss_w, g.grp_w);
    if (out->dss_off) std::memcpy(out->dss_off, g.grp_off.data(), g.grp_off.size() * sizeof(int));
    if (out->dss_copy) std::memcpy(out->dss_copy, g.grp_copy.data(), g.grp_copy.size() * sizeof(int));
  } catch (...) {
    return GB_ERR_NOMEM;
  }
  return GB_OK;
}

int gb_ctx_create(const gb_config *cfg, gb_ctx **out) {
  GB_RANGE();
  if (!cfg || !out) return GB_ERR_ARG;
  *out = nullptr;
  const char *why = nullptr;
  if (!validate_config(*cfg, &why)) return GB_ERR_ARG;
  gb_ctx *ctx = new (std::nothrow) gb_ctx();
  if (!ctx) return GB_ERR_NOMEM;
  ctx->cfg = *cfg;
  int r;
  try {
    build_geometry(*cfg, ctx->geo);
    if (!build_terrain_tables(*cfg, ctx->geo, &why)) {
      delete ctx;
      return GB_ERR_ARG;
    }
    // the layout and the surface are now in the geometry tables; the caller's arrays are not kept
    ctx->cfg.elem_map = nullptr;
    ctx->cfg.elem_orient = nullptr;
    ctx->cfg.z_surface = nullptr;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { delete ctx; return GB_ERR_CUDA; }
    r = cfg->ft_bytes == 8 ? create_impl<double>(ctx) : create_impl<float>(ctx);
  } catch (...) {
    r = GB_ERR_NOMEM;
  }
  if (r) { delete ctx; return r; }
  *out = ctx;
  return GB_OK;
}

int gb_ctx_destroy(gb_ctx *ctx) {
  GB_RANGE();
  if (!ctx) return GB_ERR_ARG;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  else cudaDeviceSynchronize();
  delete ctx;
  return GB_OK;
}

int gb_set_stream(gb_ctx *ctx, void *stream) {
  GB_RANGE();
  GUARD(ctx);
  ctx->stream = (cudaStream_t)stream;
  return GB_OK;
}

int gb_last_error(gb_ctx *ctx, char *buf, size_t len) {
  GB_RANGE();
  GUARD(ctx);
  if (buf && len) {
    std::strncpy(buf, ctx->err.c_str(), len - 1);
    buf[len - 1] = 0;
  }
  return ctx->last;
}

int gb_set_precomputed_quantities(gb_ctx *ctx, gb_fieldvec Y, double t) {
  GB_RANGE();
  GUARD(ctx);
  (void)t;
  if (!fv_ok(Y)) return fail(ctx, GB_ERR_ARG, "Y: null or misaligned pointer");
  if (ctx->geo.topo) {
    if (ctx->cfg.ft_bytes == 8) launch_topo_filter<double>(impl<double>(ctx)->P, (const double *)Y.c, (double *)Y.f, ctx->stream);
    else launch_topo_filter<float>(impl<float>(ctx)->P, (const float *)Y.c, (float *)Y.f, ctx->stream);
    return check_launch(ctx);
  }
  if (ctx->cfg.ft_bytes == 8) launch_bc_filter<double>(impl<double>(ctx)->P, (double *)Y.f, ctx->stream);
  else launch_bc_filter<float>(impl<float>(ctx)->P, (float *)Y.f, ctx->stream);
  return check_launch(ctx);
}

int gb_remaining_tendency(gb_ctx *ctx, gb_fieldvec Yt, gb_fieldvec Y, double t) {
  GB_RANGE();
  NO_MOIST(ctx, "gb_remaining_tendency");
  GUARD(ctx);
  (void)t;
  if (!fv_ok(Y) || !fv_ok(Yt)) return fail(ctx, GB_ERR_ARG, "null or misaligned pointer");
  return DISPATCH(ctx, remaining_tendency_t, ctx, Yt, Y);
}

int gb_implicit_tendency(gb_ctx *ctx, gb_fieldvec Yt, gb_fieldvec Y, double t) {
  GB_RANGE();
  GUARD(ctx);
  (void)t;
  if (!fv_ok(Y) || !fv_ok(Yt)) return fail(ctx, GB_ERR_ARG, "null or misaligned pointer");
  return DISPATCH(ctx, column_hook_t, ctx, (int)COL_IMPLICIT, Yt, Y, 0.0);
}

int gb_update_jacobian(gb_ctx *ctx, gb_fieldvec Y, double dtgamma, double t) {
  GB_RANGE();
  GUARD(ctx);
  (void)t;
  if (!fv_ok(Y)) return fail(ctx, GB_ERR_ARG, "null or misaligned pointer");
  gb_fieldvec none{nullptr, nullptr};
  return DISPATCH(ctx, column_hook_t, ctx, (int)COL_JACOBIAN, none, Y, dtgamma);
}

int gb_ldiv(gb_ctx *ctx, gb_fieldvec dY, gb_fieldvec R) {
  GB_RANGE();
  GUARD(ctx);
  if (!fv_ok(dY) || !fv_ok(R)) return fail(ctx, GB_ERR_ARG, "null or misaligned pointer");
  return DISPATCH(ctx, column_hook_t, ctx, (int)COL_LDIV, dY, R, 0.0);
}

int gb_correct_implicit_advection_tendency(gb_ctx *ctx, gb_fieldvec Yt, gb_fieldvec Y, double t) {
  GB_RANGE();
  GUARD(ctx);
  (void)t;
  if (!fv_ok(Y) || !fv_ok(Yt)) return fail(ctx, GB_ERR_ARG, "null or misaligned pointer");
  return DISPATCH(ctx, column_hook_t, ctx, (int)COL_POSTIMP, Yt, Y, 0.0);
}

int gb_dss(gb_ctx *ctx, gb_fieldvec Y) {
  GB_RANGE();
  GUARD(ctx);
  if (!fv_ok(Y)) return fail(ctx, GB_ERR_ARG, "null or misaligned pointer");
  if (ctx->cfg.ft_bytes == 8) launch_dss_state<double>(impl<double>(ctx)->P, (double *)Y.c, (double *)Y.f, ctx->stream);
  else launch_dss_state<float>(impl<float>(ctx)->P, (float *)Y.c, (float *)Y.f, ctx->stream);
  return check_launch(ctx);
}

int gb_step(gb_ctx *ctx, gb_fieldvec Y, double t, double dt, int nsteps, int use_graph) {
  GB_RANGE();
  NO_MOIST(ctx, "gb_step");
  GUARD(ctx);
  (void)t;
  if (!fv_ok(Y)) return fail(ctx, GB_ERR_ARG, "null or misaligned pointer");
  if (nsteps < 0 || !(dt > 0)) return fail(ctx, GB_ERR_ARG, "nsteps must be >= 0 and dt > 0");
  if (dt != ctx->cfg.dt)
    return fail(ctx, GB_ERR_ARG, "dt differs from gb_config.dt (the van Leer Courant factor uses the model time step)");
  return DISPATCH(ctx, step_t, ctx, Y, dt, nsteps, use_graph);
}

int gb_global_sums(gb_ctx *ctx, gb_fieldvec Y, double out[2]) {
  GB_RANGE();
  GUARD(ctx);
  if (!fv_ok(Y) || !out) return fail(ctx, GB_ERR_ARG, "null or misaligned pointer");
  return DISPATCH(ctx, global_sums_t, ctx, Y, out, 2);
}

int gb_conservation_sums(gb_ctx *ctx, gb_fieldvec Y, double out[3]) {
  GB_RANGE();
  GUARD(ctx);
  if (!fv_ok(Y) || !out) return fail(ctx, GB_ERR_ARG, "null or misaligned pointer");
  out[2] = 0.0;
  return DISPATCH(ctx, global_sums_t, ctx, Y, out, ctx->cfg.moist ? 3 : 2);
}

int gb_newton_residual(gb_ctx *ctx, double out[3]) {
  GB_RANGE();
  GUARD(ctx);
  if (!out) return fail(ctx, GB_ERR_ARG, "null pointer");
  return DISPATCH(ctx, residual_t, ctx, out);
}

int gb_jacobian_solve_noalloc(gb_ctx *ctx, gb_fieldvec dY, gb_fieldvec Y, gb_fieldvec R, double dtgamma) {
  GB_RANGE();
  GUARD(ctx);
  NO_TERRAIN(ctx, "gb_jacobian_solve_noalloc");
  if (!fv_ok(dY) || !fv_ok(Y) || !fv_ok(R)) return fail(ctx, GB_ERR_ARG, "null or misaligned pointer");
  return DISPATCH(ctx, jacobian_solve_noalloc_t, ctx, dY, Y, R, dtgamma);
}

int gb_dss_transpose(gb_ctx *ctx, gb_fieldvec X) {
  GB_RANGE();
  NO_MOIST(ctx, "gb_dss_transpose");
  if (!ctx || !X.c || !X.f) return GB_ERR_ARG;
  return ctx->cfg.ft_bytes == 8 ? dss_transpose_t<double>(ctx, X) : dss_transpose_t<float>(ctx, X);
}

int gb_remaining_tendency_vjp(gb_ctx *ctx, gb_fieldvec Ybar, gb_fieldvec Tbar, gb_fieldvec Y, double t,
                              double dparams[2]) {
  GB_RANGE();
  NO_MOIST(ctx, "gb_remaining_tendency_vjp");
  if (ctx && ctx->geo.topo) return fail(ctx, GB_ERR_ARG, "gb_remaining_tendency_vjp is not available over terrain");
  (void)t;
  if (!ctx || !fv_ok(Ybar) || !fv_ok(Tbar) || !fv_ok(Y)) return GB_ERR_ARG;
  return ctx->cfg.ft_bytes == 8 ? remaining_tendency_vjp_t<double>(ctx, Ybar, Tbar, Y, dparams)
                                : remaining_tendency_vjp_t<float>(ctx, Ybar, Tbar, Y, dparams);
}

int gb_implicit_stage(gb_ctx *ctx, gb_fieldvec U, gb_fieldvec Timp, gb_fieldvec Uhat, double dtgamma) {
  GB_RANGE();
  NO_MOIST(ctx, "gb_implicit_stage");
  if (!ctx || !U.c || !U.f || !Timp.c || !Timp.f || !Uhat.c || !Uhat.f || !(dtgamma > 0)) return GB_ERR_ARG;
  return ctx->cfg.ft_bytes == 8 ? implicit_stage_t<double>(ctx, U, Timp, Uhat, dtgamma)
                                : implicit_stage_t<float>(ctx, U, Timp, Uhat, dtgamma);
}

int gb_implicit_stage_vjp(gb_ctx *ctx, gb_fieldvec Uhat_bar, gb_fieldvec Ubar, gb_fieldvec Timp_bar, gb_fieldvec Uhat,
                          double dtgamma, double dparams[2]) {
  GB_RANGE();
  NO_MOIST(ctx, "gb_implicit_stage_vjp");
  if (ctx && ctx->geo.topo) return fail(ctx, GB_ERR_ARG, "gb_implicit_stage_vjp is not available over terrain");
  if (!ctx || !Uhat_bar.c || !Ubar.c || !Timp_bar.c || !Uhat.c || !(dtgamma > 0)) return GB_ERR_ARG;
  return ctx->cfg.ft_bytes == 8 ? implicit_stage_vjp_t<double>(ctx, Uhat_bar, Ubar, Timp_bar, Uhat, dtgamma, dparams)
                                : implicit_stage_vjp_t<float>(ctx, Uhat_bar, Ubar, Timp_bar, Uhat, dtgamma, dparams);
}

int gb_step_vjp(gb_ctx *ctx, gb_fieldvec Ybar, gb_fieldvec Y, double t, double dt, double dparams[2]) {
  GB_RANGE();
  NO_MOIST(ctx, "gb_step_vjp");
  if (ctx && ctx->geo.topo) return fail(ctx, GB_ERR_ARG, "gb_step_vjp is not available over terrain");
  (void)t;
  if (!ctx || !fv_ok(Ybar) || !fv_ok(Y) || !(dt > 0)) return GB_ERR_ARG;
  return ctx->cfg.ft_bytes == 8 ? step_vjp_t<double>(ctx, Ybar, Y, dt, dparams)
                                : step_vjp_t<float>(ctx, Ybar, Y, dt, dparams);
}

int gb_adjoint_forward(gb_ctx *ctx, gb_fieldvec Y, double t0, double dt, int nsteps, int checkpoint_every) {
  GB_RANGE();
  NO_MOIST(ctx, "gb_adjoint_forward");
  if (ctx && ctx->geo.topo) return fail(ctx, GB_ERR_ARG, "gb_adjoint_forward is not available over terrain");
  (void)t0;
  if (!ctx || !fv_ok(Y) || !(dt > 0) || nsteps < 1 || checkpoint_every < 1) return GB_ERR_ARG;
  return ctx->cfg.ft_bytes == 8 ? adjoint_forward_t<double>(ctx, Y, dt, nsteps, checkpoint_every)
                                : adjoint_forward_t<float>(ctx, Y, dt, nsteps, checkpoint_every);
}

int gb_adjoint_reverse(gb_ctx *ctx, gb_fieldvec Ybar, double dparams[2], size_t *peak_bytes) {
  GB_RANGE();
  NO_MOIST(ctx, "gb_adjoint_reverse");
  if (ctx && ctx->geo.topo) return fail(ctx, GB_ERR_ARG, "gb_adjoint_reverse is not available over terrain");
  if (!ctx || !fv_ok(Ybar)) return GB_ERR_ARG;
  return ctx->cfg.ft_bytes == 8 ? adjoint_reverse_t<double>(ctx, Ybar, dparams, peak_bytes)
                                : adjoint_reverse_t<float>(ctx, Ybar, dparams, peak_bytes);
}

int gb_adjoint_set_record_segments(gb_ctx *ctx, int segments) {
  GB_RANGE();
  NO_MOIST(ctx, "gb_adjoint_set_record_segments");
  GUARD(ctx);
  if (segments < 1) return fail(ctx, GB_ERR_ARG, "gb_adjoint_set_record_segments: segments must be >= 1");
  if (ctx->geo.topo) return fail(ctx, GB_ERR_ARG, "gb_adjoint_set_record_segments is not available over terrain");
  const int r = ctx->cfg.ft_bytes == 8 ? ensure_adjoint<double>(ctx) : ensure_adjoint<float>(ctx);
  if (r) return r;
  if (ctx->cfg.ft_bytes == 8) impl<double>(ctx)->adj->keep = segments;
  else impl<float>(ctx)->adj->keep = segments;
  return GB_OK;
}

int gb_match_elements(const gb_config *cfg, const double *xyz, int *elem_map, int *elem_orient) {
  GB_RANGE();
  if (!cfg || !xyz || !elem_map || !elem_orient) return GB_ERR_ARG;
  gb_config c = *cfg;
  c.elem_map = nullptr;
  c.elem_orient = nullptr;
  const char *why = nullptr;
  if (!validate_config(c, &why)) return GB_ERR_ARG;
  try {
    return match_elements(c, xyz, elem_map, elem_orient, &why) ? GB_OK : GB_ERR_ARG;
  } catch (...) {
    return GB_ERR_NOMEM;
  }
}

int gb_selftest_bounded_wait(gb_ctx *ctx, double limit_s) {
  GB_RANGE();
  GUARD(ctx);
  if (!(limit_s > 0) || limit_s > 1.0) return fail(ctx, GB_ERR_ARG, "limit_s must be in (0, 1]");
  int *status = ctx->cfg.ft_bytes == 8 ? impl<double>(ctx)->P.status : impl<float>(ctx)->P.status;
  launch_selftest_wait(status, (unsigned long long)(limit_s * 1e9), ctx->stream);
  int r = check_launch(ctx);
  if (r) return r;
  return DISPATCH(ctx, read_status, ctx);
}

int gb_time_kernel(gb_ctx *ctx, int kernel, gb_fieldvec Y, int reps, double *ms) {
  GB_RANGE();
  NO_MOIST(ctx, "gb_time_kernel");
  GUARD(ctx);
  if (!fv_ok(Y) || !ms || reps < 0 || kernel < 0 || kernel > GB_K_PASSB_FINAL) return fail(ctx, GB_ERR_ARG, "bad gb_time_kernel arguments");
  return DISPATCH(ctx, time_kernel_t, ctx, kernel, Y, reps, ms);
}

}  // extern "C"
