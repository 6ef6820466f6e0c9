// Batched standalone columns of uneven height (gb_columns_* in gbdycore.h).
//
// Independent dry ColumnGrid columns (src/simulation/grids.jl:93-127, flat
// metric), each with its own z_elem, solved by Newton on the implicit stage
// equation U = U^ + dtgamma T_imp(U) with the column core of colcore.cuh (one
// call of col::newton_core per iteration: implicit_tendency! residual,
// update_jacobian! blocks, BlockArrowheadSolve).
//
// Schedule.  Columns are sorted tallest first and cut into work items: groups
// of 32/G columns of one height class, a class being the lane-group shape
// (G lanes x CM levels per lane >= z_elem + 1 faces).  The persistent kernel
// runs as many CTAs as are resident; each warp takes the next item from a
// work counter (longest first, so the tail is short) and solves its columns
// with all Newton iterations in registers.  The plain form launches one grid
// per distinct z_elem instead.  gb_columns_autotune times the persistent
// variants (CTA size x register cap x levels per lane) on the caller's data.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "colcore.cuh"
#include "geometry.h"
#include "trace.h"

namespace gb {

namespace {

constexpr int MAX_ITERS = 8;

template <class FT>
struct BatchArgs {
  int ncols, nitems, iters, ctot;
  FT dtg;
  const int4 *items;        // {first slot in order[], columns, class, 0}
  const int *order;         // columns, tallest first
  const int *nv;            // z_elem per column
  const int *coff;          // centre offset per column (its faces start at coff + column)
  const int *lco, *lfo;     // offsets of the column's level tables
  const Lev4<FT> *lc4, *lf4, *lr4;  // lr4: the levels' reference records (offsets of lc4)
  const FT *hat_c, *hat_f;  // U^
  FT *u_c, *u_f;            // the iterate
  double *rnorm;            // [ncols][MAX_ITERS][3]
  int *queue;               // work counter of the persistent form
};

// One work item: 32/G columns of one class, all Newton iterations.
template <class FT, int G, int CM>
__device__ __forceinline__ void solve_item(const DevParams<FT> &P, const BatchArgs<FT> &B, int4 w, int lane) {
  const int gl = lane % G, slot = lane / G;
  const bool colv = slot < w.y;
  const int c = B.order[w.x + (colv ? slot : 0)];  // idle groups repeat the item's first column, write nothing
  const int Nv = B.nv[c], Nf = Nv + 1, r0 = gl * CM;
  const col::ColLev<FT> L{B.lc4 + B.lco[c], B.lf4 + B.lfo[c], B.lr4 + B.lco[c], Nv, Nf};
  ColGeo<FT> Gm;  // flat column: J_h = 1, g^ij = identity
  Gm.Jh = FT(1); Gm.iJh = FT(1); Gm.gu0 = FT(1); Gm.gu1 = FT(0); Gm.gu2 = FT(1);
  const size_t cb = (size_t)B.coff[c] + r0, fb = (size_t)B.coff[c] + c + r0, sc = (size_t)B.ctot;
  FT H[5][CM], U[5][CM];
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    const bool okc = r0 + k < Nv, okf = r0 + k < Nf;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      H[q][k] = okc ? B.hat_c[q * sc + cb + k] : FT(0);
      U[q][k] = okc ? B.u_c[q * sc + cb + k] : FT(0);
    }
    H[4][k] = okf ? B.hat_f[fb + k] : FT(0);
    U[4][k] = okf ? B.u_f[fb + k] : FT(0);
    if (!okc) { H[0][k] = H[3][k] = U[0][k] = U[3][k] = FT(1); }
  }
  bool finite = true;
  for (int it = 0; it < B.iters; ++it) {
    CSum<FT> ss[3];
    FT iJc[CM];
    col::newton_core<FT, G, CM, true>(P, Gm, L, gl, B.dtg, H, U, ss, finite, iJc);
    // u_h: T_imp = 0 and its Jacobian block is -I, so Newton sets it to U^'s
#pragma unroll
    for (int k = 0; k < CM; ++k) { U[1][k] = H[1][k]; U[2][k] = H[2][k]; }
    col::group_sum<G>(ss);
    if (gl == 0 && colv)
      for (int q = 0; q < 3; ++q) RSlot<FT>::put(&B.rnorm[((size_t)c * MAX_ITERS + it) * 3 + q], ss[q], true);
  }
  finite = __all_sync(0xffffffffu, finite);
  if (lane == 0 && !finite) atomicOr(P.status, ST_NONFINITE);
#pragma unroll
  for (int k = 0; k < CM; ++k) {
    if (colv && r0 + k < Nv) {
      B.u_c[cb + k] = U[0][k];
      B.u_c[sc + cb + k] = U[1][k];
      B.u_c[2 * sc + cb + k] = U[2][k];
      B.u_c[3 * sc + cb + k] = U[3][k];
    }
    if (colv && r0 + k < Nf) B.u_f[fb + k] = U[4][k];
  }
}

// Height classes: with CM2, G = 8 / 16 / 32 lanes x 2 levels for up to 16 / 32 / 64
// faces and 32 x 4 above; without, G = 4 / 8 / 16 / 32 lanes x 4 levels.
template <class FT, bool CM2>
__device__ __forceinline__ void dispatch(const DevParams<FT> &P, const BatchArgs<FT> &B, int4 w, int lane) {
  if (CM2) {
    switch (w.z) {
      case 0: solve_item<FT, 8, 2>(P, B, w, lane); break;
      case 1: solve_item<FT, 16, 2>(P, B, w, lane); break;
      case 2: solve_item<FT, 32, 2>(P, B, w, lane); break;
      default: solve_item<FT, 32, 4>(P, B, w, lane); break;
    }
  } else {
    switch (w.z) {
      case 0: solve_item<FT, 4, 4>(P, B, w, lane); break;
      case 1: solve_item<FT, 8, 4>(P, B, w, lane); break;
      case 2: solve_item<FT, 16, 4>(P, B, w, lane); break;
      default: solve_item<FT, 32, 4>(P, B, w, lane); break;
    }
  }
}

int height_class(int Nf, bool cm2) {
  if (cm2) {  // 8, 16, 32 lanes x 2 levels; 32 x 4 above 64 faces
    if (Nf <= 16) return 0;
    if (Nf <= 32) return 1;
    if (Nf <= 64) return 2;
    return 3;
  }
  if (Nf <= 16) return 0;  // 4, 8, 16, 32 lanes x 4 levels
  if (Nf <= 32) return 1;
  if (Nf <= 64) return 2;
  return 3;
}
int class_lanes(int cls, bool cm2) {
  static const int g2[4] = {8, 16, 32, 32}, g4[4] = {4, 8, 16, 32};
  return cm2 ? g2[cls] : g4[cls];
}

template <class FT, int THREADS, int MINB, bool CM2>
__global__ void __launch_bounds__(THREADS, MINB) k_col_batch(DevParams<FT> P, BatchArgs<FT> B) {
  const int lane = threadIdx.x & 31;
  // a warp takes at most nitems items, so the loop ends even if the counter misbehaves
  for (int n = 0; n < B.nitems; ++n) {
    int it = 0;
    if (lane == 0) it = atomicAdd(B.queue, 1);
    it = __shfl_sync(0xffffffffu, it, 0);
    if (it >= B.nitems) break;
    dispatch<FT, CM2>(P, B, B.items[it], lane);
  }
}

// Plain form: one warp per item of one height group.
template <class FT, int G>
__global__ void __launch_bounds__(128, 4) k_col_group(DevParams<FT> P, BatchArgs<FT> B, int item0, int nitem) {
  const int it = blockIdx.x * 4 + (threadIdx.x >> 5);
  if (it >= nitem) return;  // warp-uniform
  solve_item<FT, G, 4>(P, B, B.items[item0 + it], threadIdx.x & 31);
}

// rsum[it][q] = sum over columns of rnorm[c][it][q] (fixed order: deterministic;
// compensated FP32 pairs in FP32 runs, FP64 once at the end)
template <class FT>
__global__ void __launch_bounds__(256) k_batch_rsum(const double *rnorm, int ncols, double *out) {
  const int it = blockIdx.x;
  CSum<FT> s[3];
  for (int c = threadIdx.x; c < ncols; c += blockDim.x)
    for (int q = 0; q < 3; ++q) s[q].add(RSlot<FT>::load(&rnorm[((size_t)c * MAX_ITERS + it) * 3 + q]));
  block_sum3<FT>(s);
  if (threadIdx.x == 0)
    for (int q = 0; q < 3; ++q) out[it * 3 + q] = s[q].value();
}

// ---------------------------------------------------------------- host side
struct Buf {
  void *p = nullptr;
  ~Buf() { if (p) cudaFree(p); }
};

struct VariantInfo {
  int threads, minb;
  bool cm2;
};
const VariantInfo kVariants[GB_COLUMNS_VARIANTS] = {
    {128, 4, false}, {128, 4, true}, {128, 6, true}, {256, 2, true}, {64, 8, true}};
constexpr int kDefaultVariant = 1;

struct ColBase {
  virtual ~ColBase() {}
};

template <class FT>
struct ColImpl : ColBase {
  DevParams<FT> P{};
  Buf lc4, lf4, lr4, nv, coff, lco, lfo, order, items[2], pitems, rnorm, rsum, queue, status;
  int nitems[2] = {0, 0};
  struct Group { int item0, nitem, G; };
  std::vector<Group> groups;  // plain form: one per distinct z_elem
  int grid[GB_COLUMNS_VARIANTS] = {0};
  cudaGraphExec_t gexec = nullptr;
  cudaStream_t cap = nullptr;
  struct Key {
    const void *a, *b, *c, *d;
    double dtg;
    int iters, variant;
    bool operator==(const Key &o) const {
      return a == o.a && b == o.b && c == o.c && d == o.d && dtg == o.dtg && iters == o.iters && variant == o.variant;
    }
  } key{};
  ~ColImpl() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (cap) cudaStreamDestroy(cap);
  }
};

}  // namespace
}  // namespace gb

struct gb_columns {
  gb_config cfg{};
  int ncols = 0;
  long long ctot = 0;
  std::vector<int> z;
  int variant = gb::kDefaultVariant;
  cudaStream_t stream = nullptr;
  std::string err;
  gb::ColBase *impl = nullptr;
  ~gb_columns() { delete impl; }
};

namespace gb {
namespace {

int cfail(gb_columns *c, int code, const std::string &m) {
  if (c) c->err = m;
  return code;
}
#define CCK(x)                                                                  \
  do {                                                                          \
    cudaError_t e_ = (x);                                                       \
    if (e_ != cudaSuccess) return cfail(cols, GB_ERR_CUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
  } while (0)

int balloc(gb_columns *cols, Buf &b, size_t bytes) {
  if (cudaMalloc(&b.p, bytes ? bytes : 16) != cudaSuccess) return cfail(cols, GB_ERR_NOMEM, "cudaMalloc failed");
  return GB_OK;
}
template <class T>
int bupload(gb_columns *cols, Buf &b, const std::vector<T> &v) {
  int r = balloc(cols, b, v.size() * sizeof(T));
  if (r) return r;
  CCK(cudaMemcpy(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return GB_OK;
}

template <class FT>
ColImpl<FT> *cimpl(gb_columns *c) { return static_cast<ColImpl<FT> *>(c->impl); }

template <class FT>
int create_t(gb_columns *cols) {
  auto *I = new (std::nothrow) ColImpl<FT>();
  if (!I) return cfail(cols, GB_ERR_NOMEM, "host allocation failed");
  cols->impl = I;
  const gb_config &c = cols->cfg;
  const int n = cols->ncols;
  // level tables, one per distinct z_elem
  std::map<int, std::pair<int, int>> tab;  // z_elem -> (centre offset, face offset)
  std::vector<double> c4, f4, r4;
  for (int z : cols->z) {
    if (tab.count(z)) continue;
    gb_config cz = c;
    cz.z_elem = z;
    const std::vector<double> zf = vertical_faces(cz);
    tab[z] = {(int)(c4.size() / 4), (int)(f4.size() / 4)};
    std::vector<double> zc(z);
    for (int v = 0; v < z; ++v) {
      zc[v] = (zf[v] + zf[v + 1]) / 2;
      const double dz = zf[v + 1] - zf[v];
      c4.insert(c4.end(), {dz, 1.0 / dz, 1.0, c.grav * zc[v]});
      double ref[3];
      reference_level(c, c.grav * zc[v], ref);
      r4.insert(r4.end(), {ref[0], ref[1], ref[2], 0.0});
    }
    for (int k = 0; k <= z; ++k) {
      const double d = k == 0 ? zf[1] - zf[0] : k == z ? zf[z] - zf[z - 1] : (zf[k + 1] - zf[k - 1]) / 2;
      const double dphi = (k > 0 && k < z) ? c.grav * (zc[k] - zc[k - 1]) : 0.0;
      f4.insert(f4.end(), {1.0 / (d * d), beta_sponge(zf[k], c.sponge_zd, c.z_max, c.alpha_w), dphi, 0.0});
    }
  }
  std::vector<FT> c4t(c4.begin(), c4.end()), f4t(f4.begin(), f4.end()), r4t(r4.begin(), r4.end());
  std::vector<int> coff(n), lco(n), lfo(n);
  long long o = 0;
  for (int i = 0; i < n; ++i) {
    coff[i] = (int)o;
    o += cols->z[i];
    lco[i] = tab[cols->z[i]].first;
    lfo[i] = tab[cols->z[i]].second;
  }
  // schedule: tallest first (ties by index), items of one class
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cols->z[a] > cols->z[b]; });
  std::vector<int4> items[2];
  for (int f = 0; f < 2; ++f) {
    const bool cm2 = f == 1;
    for (int s = 0; s < n;) {
      const int cls = height_class(cols->z[order[s]] + 1, cm2), per = 32 / class_lanes(cls, cm2);
      int t = s;
      while (t < n && t - s < per && height_class(cols->z[order[t]] + 1, cm2) == cls) ++t;
      items[f].push_back(make_int4(s, t - s, cls, 0));
      s = t;
    }
  }
  std::vector<int4> pitems;  // plain form: items of one z_elem
  for (int s = 0; s < n;) {
    const int z = cols->z[order[s]], cls = height_class(z + 1, false), G = class_lanes(cls, false);
    typename ColImpl<FT>::Group g{(int)pitems.size(), 0, G};
    int t = s;
    while (t < n && cols->z[order[t]] == z) {
      int u = t;
      while (u < n && u - t < 32 / G && cols->z[order[u]] == z) ++u;
      pitems.push_back(make_int4(t, u - t, cls, 0));
      t = u;
    }
    g.nitem = (int)pitems.size() - g.item0;
    I->groups.push_back(g);
    s = t;
  }
  int r;
  if ((r = bupload(cols, I->lc4, c4t)) || (r = bupload(cols, I->lf4, f4t)) || (r = bupload(cols, I->lr4, r4t)) ||
      (r = bupload(cols, I->nv, cols->z)) ||
      (r = bupload(cols, I->coff, coff)) || (r = bupload(cols, I->lco, lco)) || (r = bupload(cols, I->lfo, lfo)) ||
      (r = bupload(cols, I->order, order)) || (r = bupload(cols, I->items[0], items[0])) ||
      (r = bupload(cols, I->items[1], items[1])) || (r = bupload(cols, I->pitems, pitems)))
    return r;
  I->nitems[0] = (int)items[0].size();
  I->nitems[1] = (int)items[1].size();
  if ((r = balloc(cols, I->rnorm, (size_t)n * MAX_ITERS * 3 * sizeof(double))) ||
      (r = balloc(cols, I->rsum, MAX_ITERS * 3 * sizeof(double))) || (r = balloc(cols, I->queue, 16)) ||
      (r = balloc(cols, I->status, 16)))
    return r;
  CCK(cudaMemset(I->rnorm.p, 0, (size_t)n * MAX_ITERS * 3 * sizeof(double)));
  CCK(cudaMemset(I->status.p, 0, 16));
  DevParams<FT> &P = I->P;
  P.grav = (FT)c.grav; P.Rd = (FT)c.R_d; P.cpd = (FT)c.cp_d; P.cvd = (FT)c.cv_d; P.T0 = (FT)c.T_0;
  P.pref = (FT)c.p_ref; P.kappa = (FT)c.R_d / (FT)c.cp_d; P.Tmin_ref = (FT)c.T_min_ref;
  P.Tsfc_ref = (FT)c.T_surf_ref; P.Tmin_sgs = (FT)c.T_min_sgs;
  P.icvd = (FT)(1.0 / c.cv_d); P.ipref = (FT)(1.0 / c.p_ref);
  P.cpTmin = (FT)(c.cp_d * c.T_min_ref);
  P.status = (int *)I->status.p;
  // resident CTAs of every persistent variant
  int dev = 0, nsm = 0;
  CCK(cudaGetDevice(&dev));
  CCK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  auto occ = [&](auto kern, int threads) {
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, threads, 0);
    return std::max(1, b) * nsm;
  };
  I->grid[0] = occ(k_col_batch<FT, 128, 4, false>, 128);
  I->grid[1] = occ(k_col_batch<FT, 128, 4, true>, 128);
  I->grid[2] = occ(k_col_batch<FT, 128, 6, true>, 128);
  I->grid[3] = occ(k_col_batch<FT, 256, 2, true>, 256);
  I->grid[4] = occ(k_col_batch<FT, 64, 8, true>, 64);
  CCK(cudaGetLastError());
  CCK(cudaStreamCreateWithFlags(&I->cap, cudaStreamNonBlocking));
  return GB_OK;
}

template <class FT>
BatchArgs<FT> args_for(gb_columns *cols, gb_fieldvec U, gb_fieldvec Uh, double dtg, int iters, const int4 *items,
                       int nitems) {
  ColImpl<FT> *I = cimpl<FT>(cols);
  BatchArgs<FT> B{};
  B.ncols = cols->ncols; B.nitems = nitems; B.iters = iters; B.ctot = (int)cols->ctot; B.dtg = (FT)dtg;
  B.items = items; B.order = (const int *)I->order.p; B.nv = (const int *)I->nv.p;
  B.coff = (const int *)I->coff.p; B.lco = (const int *)I->lco.p; B.lfo = (const int *)I->lfo.p;
  B.lc4 = (const Lev4<FT> *)I->lc4.p; B.lf4 = (const Lev4<FT> *)I->lf4.p; B.lr4 = (const Lev4<FT> *)I->lr4.p;
  B.hat_c = (const FT *)Uh.c; B.hat_f = (const FT *)Uh.f; B.u_c = (FT *)U.c; B.u_f = (FT *)U.f;
  B.rnorm = (double *)I->rnorm.p; B.queue = (int *)I->queue.p;
  return B;
}

// The persistent form's launch sequence: counter reset, kernel, residual reduction.
template <class FT>
void enqueue_persistent(gb_columns *cols, int variant, gb_fieldvec U, gb_fieldvec Uh, double dtg, int iters,
                        cudaStream_t s) {
  ColImpl<FT> *I = cimpl<FT>(cols);
  const bool cm2 = kVariants[variant].cm2;
  const BatchArgs<FT> B = args_for<FT>(cols, U, Uh, dtg, iters, (const int4 *)I->items[cm2].p, I->nitems[cm2]);
  cudaMemsetAsync(I->queue.p, 0, sizeof(int), s);
  const int g = I->grid[variant];
  switch (variant) {
    case 0: k_col_batch<FT, 128, 4, false><<<g, 128, 0, s>>>(I->P, B); break;
    case 1: k_col_batch<FT, 128, 4, true><<<g, 128, 0, s>>>(I->P, B); break;
    case 2: k_col_batch<FT, 128, 6, true><<<g, 128, 0, s>>>(I->P, B); break;
    case 3: k_col_batch<FT, 256, 2, true><<<g, 256, 0, s>>>(I->P, B); break;
    default: k_col_batch<FT, 64, 8, true><<<g, 64, 0, s>>>(I->P, B); break;
  }
  k_batch_rsum<FT><<<iters, 256, 0, s>>>((const double *)I->rnorm.p, cols->ncols, (double *)I->rsum.p);
}

template <class FT>
void enqueue_per_height(gb_columns *cols, gb_fieldvec U, gb_fieldvec Uh, double dtg, int iters, cudaStream_t s) {
  ColImpl<FT> *I = cimpl<FT>(cols);
  const BatchArgs<FT> B = args_for<FT>(cols, U, Uh, dtg, iters, (const int4 *)I->pitems.p, 0);
  for (const auto &g : I->groups) {
    const int grid = (g.nitem + 3) / 4;
    switch (g.G) {
      case 4: k_col_group<FT, 4><<<grid, 128, 0, s>>>(I->P, B, g.item0, g.nitem); break;
      case 8: k_col_group<FT, 8><<<grid, 128, 0, s>>>(I->P, B, g.item0, g.nitem); break;
      case 16: k_col_group<FT, 16><<<grid, 128, 0, s>>>(I->P, B, g.item0, g.nitem); break;
      default: k_col_group<FT, 32><<<grid, 128, 0, s>>>(I->P, B, g.item0, g.nitem); break;
    }
  }
  k_batch_rsum<FT><<<iters, 256, 0, s>>>((const double *)I->rnorm.p, cols->ncols, (double *)I->rsum.p);
}

template <class FT>
int read_status(gb_columns *cols) {
  ColImpl<FT> *I = cimpl<FT>(cols);
  int st = 0;
  CCK(cudaMemcpyAsync(&st, I->status.p, sizeof(int), cudaMemcpyDeviceToHost, cols->stream));
  CCK(cudaStreamSynchronize(cols->stream));
  if (st) {
    CCK(cudaMemsetAsync(I->status.p, 0, sizeof(int), cols->stream));
    CCK(cudaStreamSynchronize(cols->stream));
    if (st & ST_NONFINITE) return cfail(cols, GB_ERR_NONFINITE, "non-finite Newton residual in a column");
  }
  return GB_OK;
}

template <class FT>
int solve_t(gb_columns *cols, gb_fieldvec U, gb_fieldvec Uh, double dtg, int iters, int mode, double *rnorm) {
  ColImpl<FT> *I = cimpl<FT>(cols);
  cudaStream_t s = cols->stream;
  if (mode == GB_COLUMNS_PER_HEIGHT) {
    enqueue_per_height<FT>(cols, U, Uh, dtg, iters, s);
  } else if (mode == GB_COLUMNS_PERSISTENT) {
    enqueue_persistent<FT>(cols, cols->variant, U, Uh, dtg, iters, s);
  } else {
    const typename ColImpl<FT>::Key k{U.c, U.f, Uh.c, Uh.f, dtg, iters, cols->variant};
    if (!I->gexec || !(k == I->key)) {
      if (I->gexec) { cudaGraphExecDestroy(I->gexec); I->gexec = nullptr; }
      cudaGraph_t graph = nullptr;
      CCK(cudaStreamBeginCapture(I->cap, cudaStreamCaptureModeThreadLocal));
      enqueue_persistent<FT>(cols, cols->variant, U, Uh, dtg, iters, I->cap);
      CCK(cudaStreamEndCapture(I->cap, &graph));
      const cudaError_t e = cudaGraphInstantiate(&I->gexec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) { I->gexec = nullptr; return cfail(cols, GB_ERR_CUDA, cudaGetErrorString(e)); }
      I->key = k;
    }
    CCK(cudaGraphLaunch(I->gexec, s));
  }
  CCK(cudaGetLastError());
  if (rnorm) {
    CCK(cudaMemcpyAsync(rnorm, I->rsum.p, (size_t)iters * 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
    return read_status<FT>(cols);
  }
  return GB_OK;
}

template <class FT>
int autotune_t(gb_columns *cols, gb_fieldvec U, gb_fieldvec Uh, double dtg, int iters, int reps, int *choice,
               double *ms) {
  cudaStream_t s = cols->stream;
  const size_t cb = (size_t)cols->ctot * 4 * sizeof(FT), fb = (size_t)(cols->ctot + cols->ncols) * sizeof(FT);
  Buf wc, wf;
  int r;
  if ((r = balloc(cols, wc, cb)) || (r = balloc(cols, wf, fb))) return r;
  const gb_fieldvec W{wc.p, wf.p};
  cudaEvent_t a = nullptr, b = nullptr;
  CCK(cudaEventCreate(&a));
  CCK(cudaEventCreate(&b));
  double best = 1e30;
  int bi = kDefaultVariant;
  for (int v = 0; v < GB_COLUMNS_VARIANTS; ++v) {
    float tot = 0;
    for (int k = 0; k <= reps; ++k) {  // k = 0 is the warm-up
      cudaMemcpyAsync(wc.p, U.c, cb, cudaMemcpyDeviceToDevice, s);
      cudaMemcpyAsync(wf.p, U.f, fb, cudaMemcpyDeviceToDevice, s);
      cudaEventRecord(a, s);
      enqueue_persistent<FT>(cols, v, W, Uh, dtg, iters, s);
      cudaEventRecord(b, s);
      cudaEventSynchronize(b);
      float t = 0;
      cudaEventElapsedTime(&t, a, b);
      if (k > 0) tot += t;
    }
    const double m = tot / std::max(1, reps);
    if (ms) ms[v] = m;
    if (m < best) { best = m; bi = v; }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  CCK(cudaGetLastError());
  r = read_status<FT>(cols);
  if (r) return r;
  cols->variant = bi;
  if (choice) *choice = bi;
  return GB_OK;
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" {

int gb_columns_create(const gb_config *cfg, int ncols, const int *z_elem, gb_columns **out) {
  GB_RANGE();
  if (!out) return GB_ERR_ARG;
  *out = nullptr;
  // the batched columns are dry (moist 0M is built for the column hooks of a context)
  if (!cfg || ncols <= 0 || !z_elem || (cfg->ft_bytes != 4 && cfg->ft_bytes != 8) || !(cfg->z_max > 0) || cfg->moist)
    return GB_ERR_ARG;
  auto *c = new (std::nothrow) gb_columns();
  if (!c) return GB_ERR_NOMEM;
  c->cfg = *cfg;
  c->ncols = ncols;
  c->z.assign(z_elem, z_elem + ncols);
  for (int z : c->z) {
    if (z < 2 || z > 127 || (cfg->z_stretch && !(cfg->dz_bottom > 0 && cfg->dz_bottom < cfg->z_max / z))) {
      delete c;
      return GB_ERR_ARG;
    }
    c->ctot += z;
  }
  if (c->ctot + ncols >= (1ll << 31)) { delete c; return GB_ERR_ARG; }
  const int r = cfg->ft_bytes == 4 ? create_t<float>(c) : create_t<double>(c);
  if (r) { delete c; return r; }
  *out = c;
  return GB_OK;
}

int gb_columns_destroy(gb_columns *cols) {
  GB_RANGE();
  delete cols;
  return GB_OK;
}

int gb_columns_set_stream(gb_columns *cols, void *cuda_stream) {
  GB_RANGE();
  if (!cols) return GB_ERR_ARG;
  cols->stream = (cudaStream_t)cuda_stream;
  return GB_OK;
}

int gb_columns_size(const gb_columns *cols, long long *centres, long long *faces) {
  GB_RANGE();
  if (!cols) return GB_ERR_ARG;
  if (centres) *centres = cols->ctot;
  if (faces) *faces = cols->ctot + cols->ncols;
  return GB_OK;
}

int gb_columns_solve(gb_columns *cols, gb_fieldvec U, gb_fieldvec Uhat, double dtgamma, int newton_iters, int mode,
                     double *rnorm) {
  GB_RANGE();
  if (!cols) return GB_ERR_ARG;
  if (!U.c || !U.f || !Uhat.c || !Uhat.f || newton_iters < 1 || newton_iters > MAX_ITERS || mode < 0 || mode > 2 ||
      !(dtgamma > 0))
    return cfail(cols, GB_ERR_ARG, "gb_columns_solve: invalid argument");
  return cols->cfg.ft_bytes == 4 ? solve_t<float>(cols, U, Uhat, dtgamma, newton_iters, mode, rnorm)
                                 : solve_t<double>(cols, U, Uhat, dtgamma, newton_iters, mode, rnorm);
}

int gb_columns_autotune(gb_columns *cols, gb_fieldvec U, gb_fieldvec Uhat, double dtgamma, int newton_iters,
                        int reps, int *choice, double *ms) {
  GB_RANGE();
  if (!cols) return GB_ERR_ARG;
  if (!U.c || !U.f || !Uhat.c || !Uhat.f || newton_iters < 1 || newton_iters > MAX_ITERS || reps < 1 || !(dtgamma > 0))
    return cfail(cols, GB_ERR_ARG, "gb_columns_autotune: invalid argument");
  return cols->cfg.ft_bytes == 4 ? autotune_t<float>(cols, U, Uhat, dtgamma, newton_iters, reps, choice, ms)
                                 : autotune_t<double>(cols, U, Uhat, dtgamma, newton_iters, reps, choice, ms);
}

int gb_columns_set_variant(gb_columns *cols, int variant) {
  GB_RANGE();
  if (!cols || variant < 0 || variant >= GB_COLUMNS_VARIANTS) return GB_ERR_ARG;
  cols->variant = variant;
  return GB_OK;
}

int gb_columns_last_error(const gb_columns *cols, char *buf, size_t len) {
  GB_RANGE();
  if (!cols || !buf || len == 0) return GB_ERR_ARG;
  snprintf(buf, len, "%s", cols->err.c_str());
  return GB_OK;
}

}  // extern "C"
