// Tree tensor network algorithms on the device: operator application,
// orthogonalisation and truncation, inner products, integral of O f.
//
// Reference: operate (src/elementary_operators.jl:294-319) hands O and f to
// ITensorNetworks.contract(...; alg="fit", init=f), a variational fit that
// starts from f's bond dimensions; truncate (src/itensornetworkfunction.jl:
// 114-118) calls ITensorNetworks.truncate (QR toward a root, SVD per bond with
// a relative discarded-weight cutoff).  Here O f is formed exactly (bond dims
// multiply) and then truncated -- the result the fit converges to.
//
// Truncation of a tree: (1) QR every vertex toward its root, children first;
// (2) depth-first from the root: at vertex v (the orthogonality centre) SVD
// the bond to child c, keep the rank allowed by cutoff / maxdim, move the
// centre into c (S V^H absorbed), recurse, then QR c back toward v.  Every
// SVD therefore sees the exact Schmidt spectrum of its bond.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdlib>
#include <functional>
#include <numeric>

#include "evaluate.cuh"
#include "linalg.cuh"

namespace tnfa {

tnfa_net* site_reduced_net(tnfa_ctx* ctx, const tnfa_net* net, int take_sum);  // integrate.cu

namespace {

inline double habs2(double x) { return x * x; }
inline double habs2(cplx x) { return x.re * x.re + x.im * x.im; }
template <class T> inline T hreal(double a);
template <> inline double hreal<double>(double a) { return a; }
template <> inline cplx hreal<cplx>(double a) { return {a, 0.0}; }
__device__ inline double dmul(double x, double s) { return x * s; }
__device__ inline cplx dmul(cplx x, double s) { return {x.re * s, x.im * s}; }

template <class T>
__global__ void k_scale_by(T* x, int64_t n, double s) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = dmul(x[i], s);
}

// Diagnostics: with TNFA_DEBUG_NAN set, every step of the truncation checks
// its output for NaN / Inf and fails naming the first step that produced one.
inline bool nan_debug() {
  static const char* e = getenv("TNFA_DEBUG_NAN");
  return e && *e;
}

template <class T>
void nan_check(tnfa_ctx* ctx, const void* p, int64_t n, const char* what, int v) {
  if (!nan_debug() || n <= 0) return;
  std::vector<T> h(n);
  TNFA_CUDA(cudaMemcpyAsync(h.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int64_t i = 0; i < n; ++i) {
    double a = habs2(h[i]);
    if (!std::isfinite(a))
      fail(TNFA_ERR_CUDA, std::string("non-finite value after ") + what + " at vertex " +
                              std::to_string(v) + ", element " + std::to_string(i) + " of " +
                              std::to_string(n));
  }
}

template <class T>
struct Work {
  tnfa_ctx* ctx;
  Topo topo;
  std::vector<DBuf> t;  // per-vertex tensors, canonical layout

  std::vector<int> shape(int v) const {
    std::vector<int> s{topo.site_dim[v], topo.link[v]};
    for (int c : topo.children[v]) s.push_back(topo.link[c]);
    return s;
  }
  int64_t size(int v) const {
    int64_t n = 1;
    for (int d : shape(v)) n *= d;
    return n;
  }
  int child_axis(int v, int c) const {
    const auto& ch = topo.children[v];
    return 2 + (int)(std::find(ch.begin(), ch.end(), c) - ch.begin());
  }
};

template <class T>
Work<T> load_work(tnfa_ctx* ctx, const tnfa_net* net) {
  Work<T> w{ctx, net->topo, {}};
  w.t.reserve(net->topo.V);
  for (int v = 0; v < net->topo.V; ++v) {
    const int64_t n = net->topo.size(v);
    w.t.emplace_back(ctx, (size_t)n * sizeof(T));
    TNFA_CUDA(cudaMemcpyAsync(w.t.back().p, (const T*)net->d + net->topo.off[v], n * sizeof(T),
                              cudaMemcpyDeviceToDevice, ctx->stream));
    nan_check<T>(ctx, w.t.back().p, n, "load", v);
  }
  return w;
}

template <class T>
tnfa_net* store_work(Work<T>& w, int dtype) {
  w.topo.finalize();
  tnfa_net* out = new_net(w.ctx, w.topo, dtype);
  for (int v = 0; v < w.topo.V; ++v)
    TNFA_CUDA(cudaMemcpyAsync((T*)out->d + w.topo.off[v], w.t[v].p, w.size(v) * sizeof(T),
                              cudaMemcpyDeviceToDevice, w.ctx->stream));
  return out;
}

// dst = src with axis `ax` moved to position `to` (dims `shp`).
template <class T>
void move_axis(tnfa_ctx* ctx, const void* src, void* dst, const std::vector<int>& shp, int ax,
               int to) {
  la::PermJob j{};
  j.src = src;
  j.dst = dst;
  j.nd = (int)shp.size();
  TNFA_CHECK(j.nd <= la::MAXD, TNFA_ERR_UNSUPPORTED, "tensor order above 16");
  std::vector<int> order(j.nd);
  std::iota(order.begin(), order.end(), 0);
  order.erase(order.begin() + ax);
  order.insert(order.begin() + to, ax);
  j.n = 1;
  for (int a = 0; a < j.nd; ++a) {
    j.shape[a] = shp[a];
    j.perm[a] = order[a];
    j.n *= shp[a];
  }
  if (ax == to) {
    TNFA_CUDA(cudaMemcpyAsync(dst, src, j.n * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
    return;
  }
  la::permute<T>(ctx, {j});
}

// T_v <- M x_ax T_v : contract axis `ax` of v's tensor with the columns of M
// (newdim x shape[ax]).
template <class T>
void absorb(Work<T>& w, int v, int ax, const void* M, int newdim) {
  tnfa_ctx* ctx = w.ctx;
  std::vector<int> shp = w.shape(v);
  const int old = shp[ax];
  const int64_t rest = w.size(v) / old;
  DBuf a(ctx, (size_t)w.size(v) * sizeof(T));
  move_axis<T>(ctx, w.t[v].p, a.p, shp, ax, 0);  // [old][rest]
  DBuf b(ctx, (size_t)newdim * rest * sizeof(T));
  la::GemmJob g{M, a.p, b.p, newdim, (int)rest, old, old, (int)rest, (int)rest, 0, 0, 1.0, 0.0};
  la::gemm<T>(ctx, {g});
  std::vector<int> nshp = shp;
  nshp.erase(nshp.begin() + ax);
  nshp.insert(nshp.begin(), newdim);  // current layout [newdim][rest...]
  nan_check<T>(ctx, a.p, w.size(v), "absorb/permute-in", v);
  nan_check<T>(ctx, M, (int64_t)newdim * old, "absorb/matrix", v);
  nan_check<T>(ctx, b.p, newdim * rest, "absorb/gemm", v);
  DBuf c(ctx, (size_t)newdim * rest * sizeof(T));
  move_axis<T>(ctx, b.p, c.p, nshp, 0, ax);
  nan_check<T>(ctx, c.p, newdim * rest, "absorb/permute-out", v);
  w.t[v] = std::move(c);
}

// Thin QR of v's tensor with axis `ax` as the columns: T = Q R.  v keeps Q
// (axis ax now of dim k = min(rows, cols)); R (k x cols) is returned.
template <class T>
int qr_axis(Work<T>& w, int v, int ax, DBuf& R) {
  tnfa_ctx* ctx = w.ctx;
  std::vector<int> shp = w.shape(v);
  const int cols = shp[ax];
  const int64_t rows = w.size(v) / cols;
  TNFA_CHECK(rows < (int64_t(1) << 31), TNFA_ERR_UNSUPPORTED, "matrix too large");
  const int k = (int)std::min<int64_t>(rows, cols);
  DBuf M(ctx, (size_t)w.size(v) * sizeof(T));
  move_axis<T>(ctx, w.t[v].p, M.p, shp, ax, (int)shp.size() - 1);  // [rest][cols]
  DBuf Q(ctx, (size_t)rows * k * sizeof(T));
  R = DBuf(ctx, (size_t)k * cols * sizeof(T));
  DBuf tau(ctx, (size_t)k * sizeof(T));
  nan_check<T>(ctx, M.p, w.size(v), "qr_axis/permute-in", v);
  la::qr<T>(ctx, {la::QrJob{M.p, Q.p, R.p, tau.p, (int)rows, cols}});
  nan_check<T>(ctx, Q.p, rows * k, "qr_axis/Q", v);
  nan_check<T>(ctx, R.p, (int64_t)k * cols, "qr_axis/R", v);
  std::vector<int> qshp = shp;
  qshp.erase(qshp.begin() + ax);
  qshp.push_back(k);
  DBuf back(ctx, (size_t)rows * k * sizeof(T));
  move_axis<T>(ctx, Q.p, back.p, qshp, (int)qshp.size() - 1, ax);
  w.t[v] = std::move(back);
  return k;
}

template <class T>
void orthogonalize_to_roots(Work<T>& w) {
  for (int v = w.topo.V - 1; v >= 0; --v) {
    const int p = w.topo.parent[v];
    if (p < 0) continue;
    DBuf R;
    const int ax_p = w.child_axis(p, v);
    const int k = qr_axis(w, v, 1, R);
    absorb(w, p, ax_p, R.p, k);
    w.topo.link[v] = k;
  }
}

struct TruncStats {
  double max_discarded = 0.0;  // largest relative discarded weight of a bond
  int max_sweeps = 0;
  bool nonconv = false;
};

// SVD of v's tensor across the bond to child c, truncated; the centre moves
// into c.
template <class T>
void split_bond(Work<T>& w, int v, int c, const tnfa_trunc_params& prm, TruncStats& st) {
  tnfa_ctx* ctx = w.ctx;
  const int ax = w.child_axis(v, c);
  const std::vector<int> shp = w.shape(v);
  const int cols = shp[ax];
  const int64_t rows64 = w.size(v) / cols;
  TNFA_CHECK(rows64 < (int64_t(1) << 31), TNFA_ERR_UNSUPPORTED, "matrix too large");
  const int rows = (int)rows64;
  DBuf M(ctx, (size_t)w.size(v) * sizeof(T));
  move_axis<T>(ctx, w.t[v].p, M.p, shp, ax, (int)shp.size() - 1);  // [rows][cols]
  std::vector<la::FactorResult> res;
  la::trunc_factor<T>(ctx, {la::FactorJob{M.p, rows, cols}}, prm.cutoff, prm.maxdim, prm.mindim,
                      prm.precision, res);
  la::FactorResult& o = res[0];
  if (o.sweeps < 0) st.nonconv = true;
  st.max_sweeps = std::max(st.max_sweeps, o.sweeps);
  st.max_discarded = std::max(st.max_discarded, o.discarded);
  const int r = o.r;
  std::vector<int> nshp = shp;
  nshp.erase(nshp.begin() + ax);
  nshp.push_back(r);
  DBuf back(ctx, (size_t)rows * r * sizeof(T));
  move_axis<T>(ctx, o.L.p, back.p, nshp, (int)nshp.size() - 1, ax);
  w.t[v] = std::move(back);
  absorb(w, c, 1, o.X.p, r);
  w.topo.link[c] = r;
}

template <class T>
void truncate_from(Work<T>& w, int v, const tnfa_trunc_params& prm, TruncStats& st) {
  const std::vector<int> kids = w.topo.children[v];
  for (int c : kids) {
    split_bond(w, v, c, prm, st);
    truncate_from(w, c, prm, st);
    DBuf R;  // move the centre back to v
    const int ax = w.child_axis(v, c);
    const int k = qr_axis(w, c, 1, R);
    absorb(w, v, ax, R.p, k);
    w.topo.link[c] = k;
  }
}

// ------------------------------------------------------ exact apply ----
constexpr int AP_MAXD = 10;
// Y[s_out][(aO af)][(cO cf)...] = sum_{s_in} O[(s_out, s_in) fused per leg][aO][cO..] f[s_in][af][cf..]
struct ApplyJob {
  int64_t ooff, foff, yoff, n;
  int nd;                 // axes: site + bonds
  int dO[AP_MAXD], dF[AP_MAXD];
  int nlegs;
  int base[8];
  // k_apply_exact: this vertex's operator, function and output tensors, and
  // the first of its blocks in the flat grid (ascending over the job list)
  const void* o;
  const void* f;
  void* y;
  int64_t first_block;
};

constexpr int AP_THREADS = 256;
constexpr int AP_PER_BLOCK = 4 * AP_THREADS;  // outputs per block

// The job that owns flat block b: the last one whose first block is <= b.
template <class Job>
__device__ __forceinline__ const Job& job_of_block(const Job* __restrict__ jobs, int njobs, int64_t b) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].first_block <= b)
      lo = mid;
    else
      hi = mid - 1;
  }
  return jobs[lo];
}

// Every vertex of every listed (operator, function) pair in one launch: the
// jobs' outputs are cut into runs of AP_PER_BLOCK entries, one block each.
template <class T>
__global__ void __launch_bounds__(AP_THREADS) k_apply_exact(const ApplyJob* __restrict__ jobs, int njobs) {
  const int64_t b = blockIdx.x;
  const ApplyJob& jb = job_of_block(jobs, njobs, b);
  const T* __restrict__ O = (const T*)jb.o;
  const T* __restrict__ F = (const T*)jb.f;
  T* __restrict__ Y = (T*)jb.y;
  int64_t obond = 1, fbond = 1;
  for (int a = 1; a < jb.nd; ++a) {
    obond *= jb.dO[a];
    fbond *= jb.dF[a];
  }
  const int sdim = jb.dF[0];
  const int64_t i0 = (b - jb.first_block) * AP_PER_BLOCK;
  const int64_t i1 = i0 + AP_PER_BLOCK < jb.n ? i0 + AP_PER_BLOCK : jb.n;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += AP_THREADS) {
    int64_t r = i, oi = 0, fi = 0, os = 1, fs = 1;
    for (int a = jb.nd - 1; a >= 1; --a) {
      const int64_t d = (int64_t)jb.dO[a] * jb.dF[a];
      const int64_t x = r % d;
      r /= d;
      oi += (x / jb.dF[a]) * os;
      fi += (x % jb.dF[a]) * fs;
      os *= jb.dO[a];
      fs *= jb.dF[a];
    }
    const int s_out = (int)r;
    T acc = Sc<T>::zero();
    for (int s_in = 0; s_in < sdim; ++s_in) {
      // fused operator site index: per leg (out * b + in), first leg most significant
      int so = s_out, si = s_in, osite = 0, mul = 1;
      for (int l = jb.nlegs - 1; l >= 0; --l) {
        const int bb = jb.base[l];
        const int o = so % bb, in = si % bb;
        so /= bb;
        si /= bb;
        osite += (o * bb + in) * mul;
        mul *= bb * bb;
      }
      acc = Sc<T>::fma(O[osite * obond + oi], F[s_in * fbond + fi], acc);
    }
    Y[i] = acc;
  }
}

// Contiguous copies of many tensors in one launch (runs of AP_PER_BLOCK
// elements, one block each).
struct CopyRun {
  const void* src;
  void* dst;
  int64_t n;  // elements
  int64_t first_block;
};

template <class T>
__global__ void __launch_bounds__(AP_THREADS) k_copy_runs(const CopyRun* __restrict__ runs, int nruns) {
  const int64_t b = blockIdx.x;
  const CopyRun& c = job_of_block(runs, nruns, b);
  const T* __restrict__ src = (const T*)c.src;
  T* __restrict__ dst = (T*)c.dst;
  const int64_t i0 = (b - c.first_block) * AP_PER_BLOCK;
  const int64_t i1 = i0 + AP_PER_BLOCK < c.n ? i0 + AP_PER_BLOCK : c.n;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += AP_THREADS) dst[i] = src[i];
}

// Adjoint of k_apply_exact with respect to f:
//   dF[s_in][fi] += sum_{s_out, oi} O[(s_out, s_in)][oi] dY[s_out][(oi, fi)]
// (the (oi, fi) pairs fused per bond axis, operator index major, as in Y).
template <class T>
__global__ void k_apply_vjp(const T* __restrict__ O, const T* __restrict__ dY, T* __restrict__ dF,
                            const ApplyJob* __restrict__ jobs) {
  const ApplyJob& jb = jobs[blockIdx.y];
  int64_t obond = 1, fbond = 1;
  for (int a = 1; a < jb.nd; ++a) {
    obond *= jb.dO[a];
    fbond *= jb.dF[a];
  }
  const int sdim = jb.dF[0];
  const int64_t nf = (int64_t)sdim * fbond;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nf;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int s_in = (int)(i / fbond);
    const int64_t fi = i % fbond;
    T acc = Sc<T>::zero();
    for (int s_out = 0; s_out < sdim; ++s_out) {
      int so = s_out, si = s_in, osite = 0, mul = 1;
      for (int l = jb.nlegs - 1; l >= 0; --l) {
        const int b = jb.base[l];
        const int o = so % b, in = si % b;
        so /= b;
        si /= b;
        osite += (o * b + in) * mul;
        mul *= b * b;
      }
      const T* orow = O + jb.ooff + (int64_t)osite * obond;
      const T* yrow = dY + jb.yoff + (int64_t)s_out * obond * fbond;
      for (int64_t oi = 0; oi < obond; ++oi) {
        // Y bond index per axis: o_a * dF[a] + f_a, row-major over the axes
        int64_t yi = 0, ro = oi, rf = fi, ym = 1;
        for (int a = jb.nd - 1; a >= 1; --a) {
          const int64_t oa = ro % jb.dO[a], fa = rf % jb.dF[a];
          ro /= jb.dO[a];
          rf /= jb.dF[a];
          yi += (oa * jb.dF[a] + fa) * ym;
          ym *= (int64_t)jb.dO[a] * jb.dF[a];
        }
        acc = Sc<T>::fma(orow[oi], yrow[yi], acc);
      }
    }
    dF[jb.foff + i] += acc;
  }
}

// O'[s_in][rest] = w * sum_{s_out} O[(s_out, s_in)][rest]: the out legs of an
// operator contracted with the uniform integration weights.
struct RowJob {
  int64_t ooff, doff, rest;
  int nlegs;
  int base[8];
  double w;
};

template <class T>
__global__ void k_reduce_out(const T* __restrict__ O, T* __restrict__ D,
                             const RowJob* __restrict__ jobs) {
  const RowJob& jb = jobs[blockIdx.y];
  int sdim = 1;
  for (int l = 0; l < jb.nlegs; ++l) sdim *= jb.base[l];
  const int64_t n = (int64_t)sdim * jb.rest;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int s_in = (int)(i / jb.rest);
    const int64_t q = i % jb.rest;
    T acc = Sc<T>::zero();
    for (int s_out = 0; s_out < sdim; ++s_out) {
      int so = s_out, si = s_in, osite = 0, mul = 1;
      for (int l = jb.nlegs - 1; l >= 0; --l) {
        const int b = jb.base[l];
        osite += ((so % b) * b + si % b) * mul;
        so /= b;
        si /= b;
        mul *= b * b;
      }
      acc = acc + O[jb.ooff + (int64_t)osite * jb.rest + q];
    }
    D[jb.doff + i] = dmul(acc, jb.w);
  }
}

template <class Job>
DBuf upload_jobs(tnfa_ctx* ctx, const std::vector<Job>& jobs) {
  DBuf d(ctx, jobs.size() * sizeof(Job));
  h2d(ctx, d.p, jobs.data(), jobs.size() * sizeof(Job));
  return d;
}

void check_same_tree(const Topo& A, const Topo& B, const char* what) {
  TNFA_CHECK(A.V == B.V && A.parent == B.parent && A.nlegs == B.nlegs, TNFA_ERR_SHAPE,
             std::string(what) + ": operator and function live on different trees");
}

void check_apply(const Topo& A, const Topo& B) {
  check_same_tree(A, B, "apply");
  for (int l = 0; l < A.leg_off[A.V]; ++l) {
    TNFA_CHECK(A.leg_kind[l] == TNFA_LEG_OPERATOR, TNFA_ERR_INVALID_ARGUMENT,
               "apply: first argument is not an operator");
    TNFA_CHECK(B.leg_kind[l] != TNFA_LEG_OPERATOR, TNFA_ERR_INVALID_ARGUMENT,
               "apply: second argument is an operator");
    TNFA_CHECK(A.leg_dim[l] == B.leg_dim[l] * B.leg_dim[l], TNFA_ERR_SHAPE,
               "apply: operator leg dim must be base^2 of the function's");
  }
}

// One job per vertex of y = O f: offsets and axis dimensions of O, f and Y
// (Y's topology is f's with every bond multiplied by the operator's).
std::vector<ApplyJob> apply_jobs(const Topo& A, const Topo& B, Topo& Y) {
  Y = B;
  for (int v = 0; v < B.V; ++v) Y.link[v] = A.link[v] * B.link[v];
  Y.finalize();
  std::vector<ApplyJob> jobs;
  for (int v = 0; v < B.V; ++v) {
    ApplyJob j{};
    j.ooff = A.off[v];
    j.foff = B.off[v];
    j.yoff = Y.off[v];
    j.n = Y.size(v);
    j.nd = 2 + (int)B.children[v].size();
    TNFA_CHECK(j.nd <= AP_MAXD && B.nlegs[v] <= 8, TNFA_ERR_UNSUPPORTED, "vertex degree too high");
    j.dO[0] = A.site_dim[v];
    j.dF[0] = B.site_dim[v];
    j.dO[1] = A.link[v];
    j.dF[1] = B.link[v];
    for (size_t i = 0; i < B.children[v].size(); ++i) {
      j.dO[2 + i] = A.link[B.children[v][i]];
      j.dF[2 + i] = B.link[B.children[v][i]];
    }
    j.nlegs = B.nlegs[v];
    for (int l = 0; l < j.nlegs; ++l) j.base[l] = B.leg_dim[B.leg_off[v] + l];
    jobs.push_back(j);
  }
  return jobs;
}

// Give every job its first block in the flat grid; the total block count.
template <class Job>
int64_t number_blocks(std::vector<Job>& jobs) {
  int64_t nb = 0;
  for (auto& j : jobs) {
    j.first_block = nb;
    nb += (j.n + AP_PER_BLOCK - 1) / AP_PER_BLOCK;
  }
  TNFA_CHECK(nb < (int64_t(1) << 31), TNFA_ERR_UNSUPPORTED, "too many blocks for one launch");
  return nb;
}

// y_i = O_i f_i exactly, vertex by vertex, for every pair in one launch; each
// W[i] receives y_i's per-vertex tensors, written in place by the kernel.
template <class T>
void apply_exact_many(tnfa_ctx* ctx, int n, const tnfa_net* const* ops, const tnfa_net* const* fs,
                      std::vector<Work<T>>& W) {
  W.clear();
  W.reserve(n);
  std::vector<ApplyJob> jobs;
  double fl = 0;
  for (int i = 0; i < n; ++i) {
    const Topo& A = ops[i]->topo;
    const Topo& B = fs[i]->topo;
    check_apply(A, B);
    Topo Y;
    std::vector<ApplyJob> ji = apply_jobs(A, B, Y);
    W.push_back(Work<T>{ctx, Y, {}});
    Work<T>& w = W.back();
    w.t.reserve(Y.V);
    for (int v = 0; v < Y.V; ++v) {
      w.t.emplace_back(ctx, (size_t)Y.size(v) * sizeof(T));
      ApplyJob& j = ji[v];
      j.o = (const T*)ops[i]->d + j.ooff;
      j.f = (const T*)fs[i]->d + j.foff;
      j.y = w.t.back().p;
      fl += 2.0 * j.n * j.dF[0];
      jobs.push_back(j);
    }
  }
  if (jobs.empty()) return;
  const int64_t nb = number_blocks(jobs);
  DBuf dj = upload_jobs(ctx, jobs);
  KernelScope ks(ctx, "apply_exact", fl, 0.0);
  k_apply_exact<T><<<(unsigned)nb, AP_THREADS, 0, ctx->stream>>>(dj.as<ApplyJob>(), (int)jobs.size());
  TNFA_LAUNCH_CHECK();
}

template <class T>
Work<T> apply_exact(tnfa_ctx* ctx, const tnfa_net* op, const tnfa_net* f) {
  std::vector<Work<T>> W;
  apply_exact_many<T>(ctx, 1, &op, &f, W);
  return std::move(W[0]);
}

// One network per Work (canonical layout), all tensors copied in one launch.
template <class T>
void store_works(std::vector<Work<T>>& W, int dtype, tnfa_net** outs) {
  if (W.empty()) return;
  tnfa_ctx* ctx = W[0].ctx;
  std::vector<CopyRun> runs;
  for (size_t i = 0; i < W.size(); ++i) {
    Work<T>& w = W[i];
    w.topo.finalize();
    outs[i] = new_net(ctx, w.topo, dtype);
    for (int v = 0; v < w.topo.V; ++v)
      runs.push_back({w.t[v].p, (T*)outs[i]->d + w.topo.off[v], w.size(v), 0});
  }
  const int64_t nb = number_blocks(runs);
  DBuf dr = upload_jobs(ctx, runs);
  k_copy_runs<T><<<(unsigned)nb, AP_THREADS, 0, ctx->stream>>>(dr.as<CopyRun>(), (int)runs.size());
  TNFA_LAUNCH_CHECK();
}

// df += J^T dy for y = apply_exact(op, f) (dy in y's canonical layout).
template <class T>
void apply_vjp(tnfa_ctx* ctx, const tnfa_net* op, const tnfa_net* f, const void* dy, int dy_mem,
               void* df, int df_mem) {
  const Topo& A = op->topo;
  const Topo& B = f->topo;
  check_apply(A, B);
  Topo Y;
  std::vector<ApplyJob> jobs = apply_jobs(A, B, Y);
  int64_t nmax = 1;
  for (int v = 0; v < B.V; ++v) nmax = std::max<int64_t>(nmax, B.size(v));
  DBuf dyb, dfb;
  const T* dyd = (const T*)dy;
  T* dfd = (T*)df;
  if (dy_mem == TNFA_MEM_HOST) {
    dyb = DBuf(ctx, (size_t)Y.n_elem * sizeof(T));
    TNFA_CUDA(cudaMemcpyAsync(dyb.p, dy, (size_t)Y.n_elem * sizeof(T), cudaMemcpyHostToDevice,
                              ctx->stream));
    dyd = dyb.as<T>();
  }
  if (df_mem == TNFA_MEM_HOST) {
    dfb = DBuf(ctx, (size_t)B.n_elem * sizeof(T));
    TNFA_CUDA(cudaMemcpyAsync(dfb.p, df, (size_t)B.n_elem * sizeof(T), cudaMemcpyHostToDevice,
                              ctx->stream));
    dfd = dfb.as<T>();
  }
  DBuf dj = upload_jobs(ctx, jobs);
  dim3 grid(grid_for(nmax, 256, 4096), B.V);
  {
    double fl = 0;
    for (auto& j : jobs) fl += 2.0 * j.n * j.dF[0];
    KernelScope ks(ctx, "apply_vjp", fl, 0.0);
    k_apply_vjp<T><<<grid, 256, 0, ctx->stream>>>((const T*)op->d, dyd, dfd, dj.as<ApplyJob>());
    TNFA_LAUNCH_CHECK();
  }
  if (df_mem == TNFA_MEM_HOST)
    TNFA_CUDA(cudaMemcpyAsync(df, dfd, (size_t)B.n_elem * sizeof(T), cudaMemcpyDeviceToHost,
                              ctx->stream));
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
}

template <class T>
double host_norm(tnfa_ctx* ctx, const DBuf& b, int64_t n) {
  std::vector<T> h(n);
  TNFA_CUDA(cudaMemcpyAsync(h.data(), b.p, n * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  double s = 0;
  for (auto& x : h) s += habs2(x);
  return std::sqrt(s);
}

template <class T>
tnfa_net* truncate_work(Work<T>& w, int dtype, const tnfa_trunc_params& prm) {
  orthogonalize_to_roots(w);
  TruncStats st;
  for (int r : w.topo.roots()) truncate_from(w, r, prm, st);
  TNFA_CHECK(!st.nonconv, TNFA_ERR_NOT_CONVERGED, "Jacobi SVD hit its sweep cap");
  if (prm.normalize) {
    for (int r : w.topo.roots()) {
      const double nrm = host_norm<T>(w.ctx, w.t[r], w.size(r));
      if (nrm > 0) {
        k_scale_by<T><<<grid_for(w.size(r), 256, 1024), 256, 0, w.ctx->stream>>>(
            w.t[r].template as<T>(), w.size(r), 1.0 / nrm);
        TNFA_LAUNCH_CHECK();
      }
    }
  }
  return store_work(w, dtype);
}

void check_params(const tnfa_trunc_params* p) {
  TNFA_CHECK(p != nullptr, TNFA_ERR_INVALID_ARGUMENT, "null truncation parameters");
  TNFA_CHECK(p->cutoff >= 0.0 && std::isfinite(p->cutoff), TNFA_ERR_INVALID_ARGUMENT,
             "cutoff must be finite and >= 0");
  TNFA_CHECK(p->maxdim >= 0 && p->mindim >= 0, TNFA_ERR_INVALID_ARGUMENT, "negative maxdim/mindim");
}

// ------------------------------------------------------------- inner ----
// Message of vertex v toward its parent: M[ag][af] = sum conj?(F) G over the
// site and children legs (children already contracted with their messages).
template <class T>
void contract_pair(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_net* g, bool conjF, double* out) {
  const Topo& A = f->topo;
  const Topo& B = g->topo;
  check_same_tree(A, B, "inner");
  TNFA_CHECK(A.site_dim == B.site_dim, TNFA_ERR_SHAPE, "inner: site dimensions differ");
  std::vector<DBuf> msg(A.V);
  T total = hreal<T>(1.0);
  for (int v = A.V - 1; v >= 0; --v) {
    // G with every child leg cg_j replaced by cf_j
    std::vector<int> shp{B.site_dim[v], B.link[v]};
    for (int c : B.children[v]) shp.push_back(B.link[c]);
    int64_t n = B.size(v);
    DBuf G(ctx, (size_t)n * sizeof(T));
    TNFA_CUDA(cudaMemcpyAsync(G.p, (const T*)g->d + B.off[v], n * sizeof(T),
                              cudaMemcpyDeviceToDevice, ctx->stream));
    for (size_t j = 0; j < B.children[v].size(); ++j) {
      const int c = B.children[v][j];
      const int ax = 2 + (int)j;
      const int oldd = shp[ax], newd = A.link[c];
      const int64_t rest = n / oldd;
      DBuf a(ctx, (size_t)n * sizeof(T));
      move_axis<T>(ctx, G.p, a.p, shp, ax, 0);  // [cg][rest]
      DBuf b(ctx, (size_t)newd * rest * sizeof(T));
      // b[cf][rest] = sum_cg M_c[cg][cf] a[cg][rest]  (M_c is cg x cf)
      la::gemm<T>(ctx, {la::GemmJob{msg[c].p, a.p, b.p, newd, (int)rest, oldd, newd, (int)rest,
                                    (int)rest, 1, 0, 1.0, 0.0}});
      std::vector<int> nshp = shp;
      nshp.erase(nshp.begin() + ax);
      nshp.insert(nshp.begin(), newd);
      shp[ax] = newd;
      n = newd * rest;
      G = DBuf(ctx, (size_t)n * sizeof(T));
      move_axis<T>(ctx, b.p, G.p, nshp, 0, ax);
      msg[c].reset();
    }
    // M[ag][af] = sum_R G[ag][R] conj?(F[af][R])
    std::vector<int> fshp{A.site_dim[v], A.link[v]};
    for (int c : A.children[v]) fshp.push_back(A.link[c]);
    DBuf Fm(ctx, (size_t)A.size(v) * sizeof(T)), Gm(ctx, (size_t)n * sizeof(T));
    move_axis<T>(ctx, (const T*)f->d + A.off[v], Fm.p, fshp, 1, 0);
    move_axis<T>(ctx, G.p, Gm.p, shp, 1, 0);
    const int ag = B.link[v], af = A.link[v];
    const int64_t R = n / ag;
    msg[v] = DBuf(ctx, (size_t)ag * af * sizeof(T));
    la::gemm<T>(ctx, {la::GemmJob{Gm.p, Fm.p, msg[v].p, ag, af, (int)R, (int)R, (int)R, af, 0,
                                  conjF ? 2 : 1, 1.0, 0.0}});
    if (B.parent[v] < 0) {
      T val;
      TNFA_CUDA(cudaMemcpyAsync(&val, msg[v].p, sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
      TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
      total = total * val;
      msg[v].reset();
    }
  }
  if constexpr (sizeof(T) == 16) {
    out[0] = ((cplx*)&total)->re;
    out[1] = ((cplx*)&total)->im;
  } else {
    out[0] = (double)total;
    out[1] = 0.0;
  }
}

tnfa_net* reduce_out_legs(tnfa_ctx* ctx, const tnfa_net* op, int take_sum) {
  const Topo& A = op->topo;
  Topo D = A;
  for (int l = 0; l < A.leg_off[A.V]; ++l) {
    int b = 1;
    while (b * b < A.leg_dim[l]) ++b;
    TNFA_CHECK(b * b == A.leg_dim[l] && A.leg_kind[l] == TNFA_LEG_OPERATOR, TNFA_ERR_INVALID_ARGUMENT,
               "integrate(O, f): O is not an operator network");
    D.leg_dim[l] = b;
    D.leg_kind[l] = TNFA_LEG_REAL;
  }
  D.finalize();
  tnfa_net* out = new_net(ctx, D, op->dtype);
  std::vector<RowJob> jobs;
  int64_t nmax = 1;
  for (int v = 0; v < A.V; ++v) {
    RowJob j{};
    j.ooff = A.off[v];
    j.doff = D.off[v];
    j.rest = A.size(v) / A.site_dim[v];
    j.nlegs = A.nlegs[v];
    TNFA_CHECK(j.nlegs <= 8, TNFA_ERR_UNSUPPORTED, "too many legs");
    j.w = 1.0;
    for (int l = 0; l < j.nlegs; ++l) {
      j.base[l] = D.leg_dim[D.leg_off[v] + l];
      if (!take_sum) j.w /= j.base[l];
    }
    jobs.push_back(j);
    nmax = std::max<int64_t>(nmax, D.size(v));
  }
  DBuf dj = upload_jobs(ctx, jobs);
  dim3 grid(grid_for(nmax, 256, 1024), A.V);
  if (op->dtype == TNFA_F64)
    k_reduce_out<double><<<grid, 256, 0, ctx->stream>>>((const double*)op->d, (double*)out->d,
                                                         dj.as<RowJob>());
  else if (op->dtype == TNFA_C128)
    k_reduce_out<cplx><<<grid, 256, 0, ctx->stream>>>((const cplx*)op->d, (cplx*)out->d,
                                                       dj.as<RowJob>());
  else
    fail(TNFA_ERR_DTYPE, "integrate(O, f) needs FP64 or complex128 networks");
  TNFA_LAUNCH_CHECK();
  return out;
}

// --------------------------------------------- batched paths (MPS) ----
// Many independent path networks (vertex i's only child is i + 1) truncated
// step by step together: step t handles one vertex of every network that has
// it, so each primitive (permute, QR, SVD, GEMM) runs once per step for the
// whole batch with per-problem shapes.

bool is_rooted_path(const Topo& T) {
  if (T.V < 1 || T.parent[0] != -1) return false;
  for (int v = 1; v < T.V; ++v)
    if (T.parent[v] != v - 1) return false;
  return true;
}

struct MoveJob {
  const void* src;
  void* dst;
  std::vector<int> shp;
  int ax, to;
};

template <class T>
void move_axes(tnfa_ctx* ctx, const std::vector<MoveJob>& mv) {
  std::vector<la::PermJob> jobs;
  for (const auto& m : mv) {
    la::PermJob j{};
    j.src = m.src;
    j.dst = m.dst;
    j.nd = (int)m.shp.size();
    TNFA_CHECK(j.nd <= la::MAXD, TNFA_ERR_UNSUPPORTED, "tensor order above 16");
    std::vector<int> order(j.nd);
    std::iota(order.begin(), order.end(), 0);
    order.erase(order.begin() + m.ax);
    order.insert(order.begin() + m.to, m.ax);
    j.n = 1;
    for (int a = 0; a < j.nd; ++a) {
      j.shape[a] = m.shp[a];
      j.perm[a] = order[a];
      j.n *= m.shp[a];
    }
    jobs.push_back(j);
  }
  for (size_t i = 0; i < jobs.size(); i += 60000)
    la::permute<T>(ctx, std::vector<la::PermJob>(jobs.begin() + i,
                                                 jobs.begin() + std::min(jobs.size(), i + 60000)));
}

struct BSlot {
  int net, v;
};

// QR of the listed vertices with their parent axis (1) as columns; each keeps
// Q and returns R (k x old) in Rs[i]; ks[i] = k.  With reveal_tol > 0 the
// factorisation is rank revealing (column pivoting): k is the numerical rank,
// the directions left out holding at most reveal_tol of the matrix's
// Frobenius norm.
template <class T>
void qr_parent_axis_batched(std::vector<Work<T>>& W, const std::vector<BSlot>& sl,
                            std::vector<DBuf>& Rs, std::vector<int>& ks, double reveal_tol = 0.0) {
  if (sl.empty()) return;
  tnfa_ctx* ctx = W[sl[0].net].ctx;
  const size_t n = sl.size();
  std::vector<DBuf> M(n), Q(n), tau(n), back(n);
  Rs.clear();
  Rs.resize(n);
  ks.assign(n, 0);
  std::vector<MoveJob> mv;
  std::vector<la::QrJob> qj;
  std::vector<std::vector<int>> shp(n);
  for (size_t i = 0; i < n; ++i) {
    Work<T>& w = W[sl[i].net];
    const int v = sl[i].v;
    shp[i] = w.shape(v);
    const int cols = shp[i][1];
    const int64_t rows = w.size(v) / cols;
    TNFA_CHECK(rows < (int64_t(1) << 31), TNFA_ERR_UNSUPPORTED, "matrix too large");
    ks[i] = (int)std::min<int64_t>(rows, cols);
    M[i] = DBuf(ctx, (size_t)w.size(v) * sizeof(T));
    Q[i] = DBuf(ctx, (size_t)rows * ks[i] * sizeof(T));
    Rs[i] = DBuf(ctx, (size_t)ks[i] * cols * sizeof(T));
    tau[i] = DBuf(ctx, (size_t)ks[i] * sizeof(T));
    mv.push_back({w.t[v].p, M[i].p, shp[i], 1, (int)shp[i].size() - 1});
    qj.push_back({M[i].p, Q[i].p, Rs[i].p, tau[i].p, (int)rows, cols});
  }
  move_axes<T>(ctx, mv);
  if (reveal_tol > 0.0)
    la::qr_rank<T>(ctx, qj, reveal_tol, ks);
  else
    la::qr<T>(ctx, qj);
  mv.clear();
  for (size_t i = 0; i < n; ++i) {
    std::vector<int> qshp = shp[i];
    qshp.erase(qshp.begin() + 1);
    qshp.push_back(ks[i]);
    const int64_t rows = W[sl[i].net].size(sl[i].v) / shp[i][1];
    back[i] = DBuf(ctx, (size_t)rows * ks[i] * sizeof(T));
    mv.push_back({Q[i].p, back[i].p, qshp, (int)qshp.size() - 1, 1});
  }
  move_axes<T>(ctx, mv);
  for (size_t i = 0; i < n; ++i) W[sl[i].net].t[sl[i].v] = std::move(back[i]);
}

// T_v <- M x_ax T_v for every listed vertex (M newdims[i] x old).
template <class T>
void absorb_batched(std::vector<Work<T>>& W, const std::vector<BSlot>& sl, const std::vector<int>& ax,
                    const std::vector<const void*>& Ms, const std::vector<int>& newd) {
  if (sl.empty()) return;
  tnfa_ctx* ctx = W[sl[0].net].ctx;
  const size_t n = sl.size();
  std::vector<DBuf> a(n), b(n), c(n);
  std::vector<MoveJob> mv;
  std::vector<la::GemmJob> gj;
  std::vector<std::vector<int>> shp(n);
  for (size_t i = 0; i < n; ++i) {
    Work<T>& w = W[sl[i].net];
    const int v = sl[i].v;
    shp[i] = w.shape(v);
    const int old = shp[i][ax[i]];
    const int64_t rest = w.size(v) / old;
    a[i] = DBuf(ctx, (size_t)w.size(v) * sizeof(T));
    b[i] = DBuf(ctx, (size_t)newd[i] * rest * sizeof(T));
    mv.push_back({w.t[v].p, a[i].p, shp[i], ax[i], 0});
    gj.push_back({Ms[i], a[i].p, b[i].p, newd[i], (int)rest, old, old, (int)rest, (int)rest, 0, 0,
                  1.0, 0.0});
  }
  move_axes<T>(ctx, mv);
  for (size_t i = 0; i < gj.size(); i += 60000)
    la::gemm<T>(ctx, std::vector<la::GemmJob>(gj.begin() + i, gj.begin() + std::min(gj.size(), i + 60000)));
  mv.clear();
  for (size_t i = 0; i < n; ++i) {
    std::vector<int> nshp = shp[i];
    const int64_t rest = W[sl[i].net].size(sl[i].v) / nshp[ax[i]];
    nshp.erase(nshp.begin() + ax[i]);
    nshp.insert(nshp.begin(), newd[i]);
    c[i] = DBuf(ctx, (size_t)newd[i] * rest * sizeof(T));
    mv.push_back({b[i].p, c[i].p, nshp, 0, ax[i]});
  }
  move_axes<T>(ctx, mv);
  for (size_t i = 0; i < n; ++i) W[sl[i].net].t[sl[i].v] = std::move(c[i]);
}

// Relative Frobenius weight below which the batched orthogonalisation drops
// directions (a few hundred times the FP64 rounding of a QR step).
constexpr double kRevealTol = 1e-13;

template <class T>
void truncate_paths_batched(std::vector<Work<T>>& W, const tnfa_trunc_params& prm) {
  if (W.empty()) return;
  tnfa_ctx* ctx = W[0].ctx;
  int maxV = 0;
  for (auto& w : W) maxV = std::max(maxV, w.topo.V);
  // (1) orthogonalise toward vertex 0, from the far end of every path.  The
  // QR is rank revealing: an operator's exact product carries bonds of D chi
  // whose numerical rank is often far lower (a shift adds one direction per
  // bond), and dropping the directions at the FP64 rounding floor here
  // shrinks every later factorisation.
  for (int t = 0; t + 1 < maxV; ++t) {
    std::vector<BSlot> sl;
    for (int i = 0; i < (int)W.size(); ++i) {
      const int v = W[i].topo.V - 1 - t;
      if (v >= 1) sl.push_back({i, v});
    }
    std::vector<DBuf> Rs;
    std::vector<int> ks;
    qr_parent_axis_batched(W, sl, Rs, ks, kRevealTol);
    std::vector<BSlot> ps;
    std::vector<int> ax;
    std::vector<const void*> Ms;
    for (size_t q = 0; q < sl.size(); ++q) {
      ps.push_back({sl[q].net, sl[q].v - 1});
      ax.push_back(2);
      Ms.push_back(Rs[q].p);
    }
    absorb_batched(W, ps, ax, Ms, ks);
    for (size_t q = 0; q < sl.size(); ++q) W[sl[q].net].topo.link[sl[q].v] = ks[q];
  }
  // (2) SVD sweep from vertex 0: bond (t, t + 1) of every path at step t
  for (int t = 0; t + 1 < maxV; ++t) {
    std::vector<BSlot> sl;
    for (int i = 0; i < (int)W.size(); ++i)
      if (t + 1 < W[i].topo.V) sl.push_back({i, t});
    const size_t n = sl.size();
    std::vector<DBuf> M(n), back(n);
    std::vector<int> rows(n), cols(n), r(n);
    std::vector<std::vector<int>> shp(n);
    std::vector<MoveJob> mv;
    std::vector<la::FactorJob> fj;
    for (size_t q = 0; q < n; ++q) {
      Work<T>& w = W[sl[q].net];
      const int v = sl[q].v;
      shp[q] = w.shape(v);
      cols[q] = shp[q][2];
      const int64_t r64 = w.size(v) / cols[q];
      TNFA_CHECK(r64 < (int64_t(1) << 31), TNFA_ERR_UNSUPPORTED, "matrix too large");
      rows[q] = (int)r64;
      M[q] = DBuf(ctx, (size_t)w.size(v) * sizeof(T));
      mv.push_back({w.t[v].p, M[q].p, shp[q], 2, (int)shp[q].size() - 1});
      fj.push_back({M[q].p, rows[q], cols[q]});
    }
    move_axes<T>(ctx, mv);
    std::vector<la::FactorResult> res;
    la::trunc_factor<T>(ctx, fj, prm.cutoff, prm.maxdim, prm.mindim, prm.precision, res, kRevealTol);
    mv.clear();
    for (size_t q = 0; q < n; ++q) {
      TNFA_CHECK(res[q].sweeps >= 0, TNFA_ERR_NOT_CONVERGED, "Jacobi SVD hit its sweep cap");
      r[q] = res[q].r;
      std::vector<int> nshp = shp[q];
      nshp.erase(nshp.begin() + 2);
      nshp.push_back(r[q]);
      back[q] = DBuf(ctx, (size_t)rows[q] * r[q] * sizeof(T));
      mv.push_back({res[q].L.p, back[q].p, nshp, (int)nshp.size() - 1, 2});
    }
    move_axes<T>(ctx, mv);
    std::vector<BSlot> cs;
    std::vector<int> ax;
    std::vector<const void*> Ms;
    for (size_t q = 0; q < n; ++q) {
      W[sl[q].net].t[sl[q].v] = std::move(back[q]);
      cs.push_back({sl[q].net, sl[q].v + 1});
      ax.push_back(1);
      Ms.push_back(res[q].X.p);
    }
    absorb_batched(W, cs, ax, Ms, r);
    for (size_t q = 0; q < n; ++q) W[sl[q].net].topo.link[sl[q].v + 1] = r[q];
  }
  if (prm.normalize) {
    // the centre ends at the last vertex of every path
    for (auto& w : W) {
      const int c = w.topo.V - 1;
      const double nrm = host_norm<T>(ctx, w.t[c], w.size(c));
      if (nrm > 0) {
        k_scale_by<T><<<grid_for(w.size(c), 256, 1024), 256, 0, ctx->stream>>>(
            w.t[c].template as<T>(), w.size(c), 1.0 / nrm);
        TNFA_LAUNCH_CHECK();
      }
    }
  }
}

template <class T>
void batch_apply_truncate(tnfa_ctx* ctx, int n, const tnfa_net* const* ops, const tnfa_net* const* fs,
                          const tnfa_trunc_params& prm, int dtype, tnfa_net** outs) {
  std::vector<Work<T>> W;
  if (ops) {
    apply_exact_many<T>(ctx, n, ops, fs, W);
  } else {
    W.reserve(n);
    for (int i = 0; i < n; ++i) W.push_back(load_work<T>(ctx, fs[i]));
  }
  truncate_paths_batched(W, prm);
  store_works(W, dtype, outs);
}

// ------------------------------------------------------------ linsolve ----
// Two-site alternating linear solver on a path (the sweep of
// ITensorNetworks.linsolve / dmrg with nsites = 2): every update solves the
// system projected onto the current left / right bases exactly,
//   (a0 I + a1 LA_i A_i A_{i+1} RA_{i+2}) v = Lb_i b_i b_{i+1} Rb_{i+2},
// splits v by a truncated SVD and moves the orthogonality centre on.  The
// residual ||(a0 + a1 A) x - b|| / ||b|| is formed exactly as a network and
// normed through a QR sweep after every half sweep.

tnfa_net* direct_sum_ext(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_net* g);

// Path order of a connected tree with all degrees <= 2, from its
// lowest-numbered end: ord[k] is the vertex at position k.
std::vector<int> path_order(const Topo& T) {
  TNFA_CHECK(T.roots().size() == 1, TNFA_ERR_UNSUPPORTED, "linsolve needs a connected path");
  std::vector<std::vector<int>> adj(T.V);
  for (int v = 0; v < T.V; ++v)
    if (T.parent[v] >= 0) {
      adj[v].push_back(T.parent[v]);
      adj[T.parent[v]].push_back(v);
    }
  int end = -1;
  for (int v = 0; v < T.V; ++v) {
    TNFA_CHECK(adj[v].size() <= 2, TNFA_ERR_UNSUPPORTED,
               "linsolve needs a path graph (vertex " + std::to_string(v) +
                   " has more than two neighbours)");
    if (adj[v].size() <= 1 && end < 0) end = v;
  }
  std::vector<int> ord;
  for (int prev = -1, v = end; v >= 0;) {
    ord.push_back(v);
    int nxt = -1;
    for (int u : adj[v])
      if (u != prev) nxt = u;
    prev = v;
    v = nxt;
  }
  return ord;
}

// T re-rooted at ord[0]: vertex k of the result is T's vertex ord[k], with
// parent k - 1; bonds and site legs are carried over.
Topo path_topo(const Topo& T, const std::vector<int>& ord) {
  Topo P;
  P.V = T.V;
  P.parent.resize(T.V);
  P.link.resize(T.V);
  P.nlegs.resize(T.V);
  for (int k = 0; k < T.V; ++k) {
    const int c = ord[k];
    P.parent[k] = k - 1;
    if (k == 0) {
      P.link[k] = 1;
    } else {
      const int cp = ord[k - 1];
      P.link[k] = T.parent[c] == cp ? T.link[c] : T.link[cp];
    }
    P.nlegs[k] = T.nlegs[c];
    for (int l = T.leg_off[c]; l < T.leg_off[c + 1]; ++l) {
      P.leg_dim.push_back(T.leg_dim[l]);
      P.leg_var.push_back(T.leg_var[l]);
      P.leg_digit.push_back(T.leg_digit[l]);
      P.leg_kind.push_back(T.leg_kind[l]);
    }
  }
  P.finalize();
  return P;
}

// The tensors (cur, data) laid out for tgt, the same tree rooted elsewhere and
// numbered so that tgt's vertex t is cur's vertex cur_of[t]: every tensor is
// permuted to [site, parent, children ascending] of tgt.  A dim-1 parent axis
// appears (new root) or disappears (old root) without moving memory.
template <class T>
Work<T> relayout(tnfa_ctx* ctx, const Topo& cur, const void* data, const Topo& tgt,
                 const std::vector<int>& cur_of) {
  Work<T> w{ctx, tgt, {}};
  std::vector<int> tgt_of(cur.V);
  for (int t = 0; t < tgt.V; ++t) tgt_of[cur_of[t]] = t;
  std::vector<la::PermJob> jobs;
  w.t.reserve(tgt.V);
  for (int t = 0; t < tgt.V; ++t) {
    const int c = cur_of[t];
    const bool cur_root = cur.parent[c] < 0;
    // axes of the current tensor without a root's dim-1 parent axis, each
    // tagged with the tgt vertex across it (-1: the site axis)
    std::vector<int> shp{cur.site_dim[c]}, nb{-1};
    if (!cur_root) {
      shp.push_back(cur.link[c]);
      nb.push_back(tgt_of[cur.parent[c]]);
    }
    for (int ch : cur.children[c]) {
      shp.push_back(cur.link[ch]);
      nb.push_back(tgt_of[ch]);
    }
    auto axis_of = [&](int u) { return (int)(std::find(nb.begin(), nb.end(), u) - nb.begin()); };
    std::vector<int> perm{0};
    if (tgt.parent[t] >= 0) perm.push_back(axis_of(tgt.parent[t]));
    for (int ch : tgt.children[t]) perm.push_back(axis_of(ch));
    TNFA_CHECK(perm.size() == shp.size() && (int)shp.size() <= la::MAXD, TNFA_ERR_UNSUPPORTED,
               "relayout: trees differ");
    for (int a : perm) TNFA_CHECK(a < (int)shp.size(), TNFA_ERR_UNSUPPORTED, "relayout: trees differ");
    const int64_t n = cur.size(c);
    TNFA_CHECK(n == tgt.size(t), TNFA_ERR_SHAPE, "relayout: sizes differ");
    w.t.emplace_back(ctx, (size_t)n * sizeof(T));
    la::PermJob j{};
    j.src = (const T*)data + cur.off[c];
    j.dst = w.t.back().p;
    j.nd = (int)shp.size();
    j.n = n;
    for (int a = 0; a < j.nd; ++a) {
      j.shape[a] = shp[a];
      j.perm[a] = perm[a];
    }
    jobs.push_back(j);
  }
  la::permute<T>(ctx, jobs);
  return w;
}

// A dense FP64 tensor on the device with its shape.
struct Dense {
  DBuf b;
  std::vector<int> shp;
  double* p() const { return b.as<double>(); }
};

Dense permuted(tnfa_ctx* ctx, const double* src, const std::vector<int>& shp,
               const std::vector<int>& order) {
  Dense d;
  d.shp.resize(order.size());
  int64_t n = 1;
  for (size_t a = 0; a < order.size(); ++a) {
    d.shp[a] = shp[order[a]];
    n *= shp[a];
  }
  TNFA_CHECK(shp.size() == order.size() && (int)shp.size() <= la::MAXD, TNFA_ERR_UNSUPPORTED,
             "permute: tensor order above 16");
  d.b = DBuf(ctx, (size_t)n * 8);
  la::PermJob j{};
  j.src = src;
  j.dst = d.b.p;
  j.nd = (int)shp.size();
  j.n = n;
  for (int a = 0; a < j.nd; ++a) {
    j.shape[a] = shp[a];
    j.perm[a] = order[a];
  }
  la::permute<double>(ctx, {j});
  return d;
}

// C (m x n) = op(A) op(B), row-major, inner dimension k; C gets shape shp.
Dense mm(tnfa_ctx* ctx, const double* A, const double* B, int m, int n, int k, int opA, int opB,
         std::vector<int> shp) {
  Dense d;
  d.shp = std::move(shp);
  d.b = DBuf(ctx, (size_t)m * n * 8);
  const int lda = opA ? m : k, ldb = opB ? k : n;
  la::gemm<double>(ctx, {la::GemmJob{A, B, d.b.p, m, n, k, lda, ldb, n, opA, opB, 1.0, 0.0}});
  return d;
}

Dense ones(tnfa_ctx* ctx, std::vector<int> shp) {
  Dense d;
  d.shp = std::move(shp);
  d.b = DBuf(ctx, 8);
  const double one = 1.0;
  TNFA_CUDA(cudaMemcpyAsync(d.b.p, &one, 8, cudaMemcpyHostToDevice, ctx->stream));
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  return d;
}

// Path tensors: x and b are [s][l][r], A is [o][i][wl][wr] (the fused
// operator leg out * d + in); r = 1 past the last vertex.
struct LinsolveState {
  tnfa_ctx* ctx;
  int L, d;
  Work<double> x, A, b;
  // environments at bond k (between vertices k-1 and k; k = 0 and L are the
  // open ends): LA/RA [bra][operator][ket], Lb/Rb [x bond][b bond]
  std::vector<Dense> LA, RA, Lb, Rb;
  bool has_b = true;  // false: no right-hand side (eigenproblem)
  int bond(const Work<double>& w, int k) const {
    return k >= 1 && k < L && k < (int)w.topo.link.size() ? w.topo.link[k] : 1;
  }
};

// LA_{i+1} and Lb_{i+1} from LA_i, Lb_i and the left-orthonormal x_i.
void left_env(LinsolveState& S, int i) {
  tnfa_ctx* ctx = S.ctx;
  const int d = S.d;
  const int l = S.bond(S.x, i), r = S.bond(S.x, i + 1);
  const int wl = S.bond(S.A, i), wr = S.bond(S.A, i + 1);
  const double* xi = S.x.t[i].as<double>();
  Dense xp = permuted(ctx, xi, {d, l, r}, {1, 0, 2});                     // [l][s][r]
  Dense t1 = mm(ctx, S.LA[i].p(), xp.p(), l * wl, d * r, l, 0, 0, {l, wl, d, r});  // [l'][wl][s][r]
  Dense t1p = permuted(ctx, t1.p(), t1.shp, {0, 3, 1, 2});                // [l'][r][wl][s]
  Dense Ap = permuted(ctx, S.A.t[i].as<double>(), {d, d, wl, wr}, {2, 1, 0, 3});  // [wl][s][o][wr]
  Dense t2 = mm(ctx, t1p.p(), Ap.p(), l * r, d * wr, wl * d, 0, 0, {l, r, d, wr});  // [l'][r][o][wr]
  Dense t2p = permuted(ctx, t2.p(), t2.shp, {2, 0, 3, 1});                // [o][l'][wr][r]
  S.LA[i + 1] = mm(ctx, xi, t2p.p(), r, wr * r, d * l, 1, 0, {r, wr, r});
  if (!S.has_b) return;
  const int bl = S.bond(S.b, i), br = S.bond(S.b, i + 1);
  Dense bp = permuted(ctx, S.b.t[i].as<double>(), {d, bl, br}, {1, 0, 2});  // [bl][s][br]
  Dense u1 = mm(ctx, S.Lb[i].p(), bp.p(), l, d * br, bl, 0, 0, {l, d, br});   // [l'][s][br]
  Dense u1p = permuted(ctx, u1.p(), u1.shp, {1, 0, 2});                   // [s][l'][br]
  S.Lb[i + 1] = mm(ctx, xi, u1p.p(), r, br, d * l, 1, 0, {r, br});
}

// RA_i and Rb_i from RA_{i+1}, Rb_{i+1} and the right-orthonormal x_i.
void right_env(LinsolveState& S, int i) {
  tnfa_ctx* ctx = S.ctx;
  const int d = S.d;
  const int l = S.bond(S.x, i), r = S.bond(S.x, i + 1);
  const int wl = S.bond(S.A, i), wr = S.bond(S.A, i + 1);
  const double* xi = S.x.t[i].as<double>();
  Dense Rp = permuted(ctx, S.RA[i + 1].p(), S.RA[i + 1].shp, {2, 0, 1});  // [r][r'][wr]
  Dense t1 = mm(ctx, xi, Rp.p(), d * l, r * wr, r, 0, 0, {d, l, r, wr});  // [s][l][r'][wr]
  Dense t1p = permuted(ctx, t1.p(), t1.shp, {0, 3, 1, 2});                // [s][wr][l][r']
  Dense Ap = permuted(ctx, S.A.t[i].as<double>(), {d, d, wl, wr}, {0, 2, 1, 3});  // [o][wl][s][wr]
  Dense t2 = mm(ctx, Ap.p(), t1p.p(), d * wl, l * r, d * wr, 0, 0, {d, wl, l, r});  // [o][wl][l][r']
  Dense t2p = permuted(ctx, t2.p(), t2.shp, {0, 3, 1, 2});                // [o][r'][wl][l]
  Dense xp = permuted(ctx, xi, {d, l, r}, {1, 0, 2});                     // [l'][o][r']
  S.RA[i] = mm(ctx, xp.p(), t2p.p(), l, wl * l, d * r, 0, 0, {l, wl, l});
  if (!S.has_b) return;
  const int bl = S.bond(S.b, i), br = S.bond(S.b, i + 1);
  Dense v1 = mm(ctx, S.b.t[i].as<double>(), S.Rb[i + 1].p(), d * bl, r, br, 0, 1, {d, bl, r});
  Dense v1p = permuted(ctx, v1.p(), v1.shp, {0, 2, 1});                   // [s][r'][bl]
  S.Rb[i] = mm(ctx, xp.p(), v1p.p(), l, bl, d * r, 0, 0, {l, bl});
}

// y += a x
__global__ void k_axpy(double* __restrict__ y, const double* __restrict__ x, int64_t n, double a) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}

__global__ void k_shift_diag(double* H, int n, double a0, double a1) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn;
       i += (int64_t)gridDim.x * blockDim.x)
    H[i] = a1 * H[i] + ((i / n) == (i % n) ? a0 : 0.0);
}

constexpr int kLocalDenseMax = 8192;    // largest two-site system solved densely
constexpr int kLocalDenseSmall = 4096;  // above this the eigensolver goes matrix-free

// TNFA_LOCAL_MATRIX_FREE=1 selects the matrix-free two-site operator at every
// size (the dense one is the default where it fits).
bool force_matrix_free() {
  static const bool on = getenv("TNFA_LOCAL_MATRIX_FREE") && *getenv("TNFA_LOCAL_MATRIX_FREE") == '1';
  return on;
}

// a0 I + a1 LA_i A_i A_{i+1} RA_{i+2} as a dense n x n matrix, rows
// [l' s1' s2' r'] and columns [l s1 s2 r].
Dense local_H(LinsolveState& S, int i, double a0, double a1, const char* what) {
  tnfa_ctx* ctx = S.ctx;
  const int d = S.d;
  const int l = S.bond(S.x, i), r = S.bond(S.x, i + 2);
  const int wl = S.bond(S.A, i), wm = S.bond(S.A, i + 1), wr = S.bond(S.A, i + 2);
  const int64_t n64 = (int64_t)l * d * d * r;
  TNFA_CHECK(n64 <= kLocalDenseMax, TNFA_ERR_UNSUPPORTED,
             std::string(what) + ": two-site problem of dimension " + std::to_string(n64) +
                 " above the dense limit " + std::to_string(kLocalDenseMax) + " (lower maxdim)");
  const int n = (int)n64;
  // H[l' s1' s2' r'][l s1 s2 r] = LA_i A_i A_{i+1} RA_{i+2}
  Dense Lp = permuted(ctx, S.LA[i].p(), S.LA[i].shp, {0, 2, 1});                       // [l'][l][wl]
  Dense A1 = permuted(ctx, S.A.t[i].as<double>(), {d, d, wl, wm}, {2, 0, 1, 3});      // [wl][o][in][wm]
  Dense P1 = mm(ctx, Lp.p(), A1.p(), l * l, d * d * wm, wl, 0, 0, {l, l, d, d, wm});
  Dense A2 = permuted(ctx, S.A.t[i + 1].as<double>(), {d, d, wm, wr}, {2, 0, 1, 3});  // [wm][o][in][wr]
  Dense Rp = permuted(ctx, S.RA[i + 2].p(), S.RA[i + 2].shp, {1, 0, 2});              // [wr][r'][r]
  Dense P2 = mm(ctx, A2.p(), Rp.p(), wm * d * d, r * r, wr, 0, 0, {wm, d, d, r, r});
  Dense Hr = mm(ctx, P1.p(), P2.p(), l * l * d * d, d * d * r * r, wm, 0, 0,
                {l, l, d, d, d, d, r, r});  // [l'][l][s1'][s1][s2'][s2][r'][r]
  Dense H = permuted(ctx, Hr.p(), Hr.shp, {0, 2, 4, 6, 1, 3, 5, 7});
  k_shift_diag<<<grid_for(n64 * n64, 256, 8192), 256, 0, ctx->stream>>>(H.p(), n, a0, a1);
  TNFA_LAUNCH_CHECK();
  return H;
}


// Write v [l][s1][s2][r] back as x_i x_{i+1} through a truncated SVD; the
// centre ends in x_{i+1} (toward_right) or in x_i.
void store_two_site(LinsolveState& S, int i, const Dense& v, const tnfa_trunc_params& tp,
                    TruncStats& st, bool toward_right) {
  tnfa_ctx* ctx = S.ctx;
  const int d = S.d;
  const int l = S.bond(S.x, i), r = S.bond(S.x, i + 2);
  // a two-vertex work: vertex 0 = v as [(l s1)][1][(s2 r)], vertex 1 = the
  // identity on (s2 r); split_bond leaves U in vertex 0 and S V^T in vertex 1
  Work<double> two{ctx, Topo{}, {}};
  two.topo.V = 2;
  two.topo.parent = {-1, 0};
  two.topo.link = {1, d * r};
  two.topo.nlegs = {0, 0};
  two.topo.finalize();
  two.topo.site_dim = {l * d, d * r};
  const int64_t nv = (int64_t)l * d * d * r;
  two.t.emplace_back(ctx, (size_t)nv * 8);
  TNFA_CUDA(cudaMemcpyAsync(two.t[0].p, v.p(), (size_t)nv * 8, cudaMemcpyDeviceToDevice, ctx->stream));
  {
    const int q = d * r;
    std::vector<double> eye((size_t)q * q, 0.0);
    for (int k = 0; k < q; ++k) eye[(size_t)k * q + k] = 1.0;
    two.t.emplace_back(ctx, eye.size() * 8);
    TNFA_CUDA(cudaMemcpyAsync(two.t[1].p, eye.data(), eye.size() * 8, cudaMemcpyHostToDevice,
                              ctx->stream));
    TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  split_bond(two, 0, 1, tp, st);
  const int k = two.topo.link[1];
  Dense x0 = permuted(ctx, two.t[0].as<double>(), {l, d, k}, {1, 0, 2});  // [s1][l][k]
  Dense x1 = permuted(ctx, two.t[1].as<double>(), {d, r, k}, {0, 2, 1});  // [s2][k][r]
  S.x.t[i] = std::move(x0.b);
  S.x.t[i + 1] = std::move(x1.b);
  S.x.topo.link[i + 1] = k;
  if (!toward_right) {
    // x_{i+1} = Q R with Q right-orthonormal; R moves into x_i
    DBuf R;
    const int kq = qr_axis(S.x, i + 1, 1, R);
    absorb(S.x, i, 2, R.p, kq);
    S.x.topo.link[i + 1] = kq;
  }
  S.x.topo.finalize();
}

// Matrix-free two-site operator: y = a0 v + a1 LA_i A_i A_{i+1} RA_{i+2} v
// for v [l][s1][s2][r], as four GEMMs and three transposes per product; the
// operator pieces are transposed once per two-site problem.  Used when the
// dense two-site matrix would be large.
struct LocalOp {
  tnfa_ctx* ctx;
  int l, r, d, wl, wm, wr;
  double a0, a1;
  const double* LA;  // [l'][wl][l]
  Dense A1p, A2p, RAp;
  LocalOp(LinsolveState& S, int i, double a0_, double a1_) : ctx(S.ctx), a0(a0_), a1(a1_) {
    d = S.d;
    l = S.bond(S.x, i);
    r = S.bond(S.x, i + 2);
    wl = S.bond(S.A, i);
    wm = S.bond(S.A, i + 1);
    wr = S.bond(S.A, i + 2);
    LA = S.LA[i].p();
    A1p = permuted(ctx, S.A.t[i].as<double>(), {d, d, wl, wm}, {2, 1, 0, 3});      // [wl][in][o][wm]
    A2p = permuted(ctx, S.A.t[i + 1].as<double>(), {d, d, wm, wr}, {2, 1, 0, 3});  // [wm][in][o][wr]
    RAp = permuted(ctx, S.RA[i + 2].p(), S.RA[i + 2].shp, {1, 2, 0});              // [wr][r][r']
  }
  int n() const { return l * d * d * r; }
  void operator()(const double* v, double* y) const {
    Dense t1 = mm(ctx, LA, v, l * wl, d * d * r, l, 0, 0, {l, wl, d, d, r});        // [l'][wl][s1][s2][r]
    Dense t1p = permuted(ctx, t1.p(), t1.shp, {0, 3, 4, 1, 2});                      // [l'][s2][r][wl][s1]
    Dense t2 = mm(ctx, t1p.p(), A1p.p(), l * d * r, d * wm, wl * d, 0, 0, {l, d, r, d, wm});  // [l'][s2][r][s1'][wm]
    Dense t2p = permuted(ctx, t2.p(), t2.shp, {0, 2, 3, 4, 1});                      // [l'][r][s1'][wm][s2]
    Dense t3 = mm(ctx, t2p.p(), A2p.p(), l * r * d, d * wr, wm * d, 0, 0, {l, r, d, d, wr});  // [l'][r][s1'][s2'][wr]
    Dense t3p = permuted(ctx, t3.p(), t3.shp, {0, 2, 3, 4, 1});                      // [l'][s1'][s2'][wr][r]
    la::gemm<double>(ctx, {la::GemmJob{t3p.p(), RAp.p(), y, l * d * d, r, wr * r, wr * r, r, r, 0, 0, a1, 0.0}});
    if (a0 != 0.0) {
      const int64_t nn = n();
      k_axpy<<<grid_for(nn, 256, 1024), 256, 0, ctx->stream>>>(y, v, nn, a0);
      TNFA_LAUNCH_CHECK();
    }
  }
};

// ------------------------------------------------------------------ dmrg --
// Lowest eigenpair of the dense symmetric local operator by Lanczos with full
// re-orthogonalisation (two classical Gram-Schmidt passes per step, as GEMMs
// on the device) and restarts from the Ritz vector; the small projected
// matrix is diagonalised on the host by cyclic Jacobi.

__global__ void k_scale_copy(double* __restrict__ dst, const double* __restrict__ src, int64_t n, double a) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = a * src[i];
}

// Smallest eigenvalue of the symmetric m x m matrix T (row-major) and its
// eigenvector, by cyclic Jacobi rotations.
void sym_eig_min(std::vector<double> T, int m, double& theta, std::vector<double>& y) {
  std::vector<double> Vm((size_t)m * m, 0.0);
  for (int i = 0; i < m; ++i) Vm[(size_t)i * m + i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) (i == j ? tot : off) += T[(size_t)i * m + j] * T[(size_t)i * m + j];
    if (off <= 1e-30 * (tot + off)) break;
    for (int p = 0; p < m - 1; ++p)
      for (int q = p + 1; q < m; ++q) {
        const double apq = T[(size_t)p * m + q];
        if (apq == 0.0) continue;
        const double app = T[(size_t)p * m + p], aqq = T[(size_t)q * m + q];
        const double tau = (aqq - app) / (2.0 * apq);
        const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        const double c = 1.0 / std::sqrt(1.0 + t * t), sn = t * c;
        for (int k = 0; k < m; ++k) {  // rows / columns p, q of T
          const double tkp = T[(size_t)k * m + p], tkq = T[(size_t)k * m + q];
          T[(size_t)k * m + p] = c * tkp - sn * tkq;
          T[(size_t)k * m + q] = sn * tkp + c * tkq;
        }
        for (int k = 0; k < m; ++k) {
          const double tpk = T[(size_t)p * m + k], tqk = T[(size_t)q * m + k];
          T[(size_t)p * m + k] = c * tpk - sn * tqk;
          T[(size_t)q * m + k] = sn * tpk + c * tqk;
        }
        for (int k = 0; k < m; ++k) {
          const double vkp = Vm[(size_t)k * m + p], vkq = Vm[(size_t)k * m + q];
          Vm[(size_t)k * m + p] = c * vkp - sn * vkq;
          Vm[(size_t)k * m + q] = sn * vkp + c * vkq;
        }
      }
  }
  int best = 0;
  for (int i = 1; i < m; ++i)
    if (T[(size_t)i * m + i] < T[(size_t)best * m + best]) best = i;
  theta = T[(size_t)best * m + best];
  y.assign(m, 0.0);
  for (int k = 0; k < m; ++k) y[k] = Vm[(size_t)k * m + best];
}

double dev_dot(tnfa_ctx* ctx, const double* a, const double* b, int n, DBuf& scratch) {
  la::gemm<double>(ctx, {la::GemmJob{a, b, scratch.p, 1, 1, n, n, 1, 1, 0, 0, 1.0, 0.0}});
  double h = 0.0;
  TNFA_CUDA(cudaMemcpyAsync(&h, scratch.p, 8, cudaMemcpyDeviceToHost, ctx->stream));
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  return h;
}

using MatVec = std::function<void(const double*, double*)>;  // y = H x on the device

// v (device, n): start vector in, lowest eigenvector out (unit norm).
double lanczos_min(tnfa_ctx* ctx, const MatVec& H, int n, double* v, int kdim, int restarts, double tol) {
  kdim = std::max(2, std::min(kdim, n));
  DBuf V(ctx, (size_t)(kdim + 1) * n * 8), w(ctx, (size_t)n * 8), h(ctx, (size_t)(kdim + 1) * 8), one(ctx, 8);
  double theta = 0.0;
  for (int rs = 0; rs <= restarts; ++rs) {
    double nv = std::sqrt(dev_dot(ctx, v, v, n, one));
    TNFA_CHECK(nv > 0 && std::isfinite(nv), TNFA_ERR_NOT_CONVERGED, "dmrg: zero or non-finite start vector");
    const unsigned g = grid_for(n, 256, 1024);
    k_scale_copy<<<g, 256, 0, ctx->stream>>>(V.as<double>(), v, n, 1.0 / nv);
    TNFA_LAUNCH_CHECK();
    std::vector<double> T((size_t)kdim * kdim, 0.0);
    int m = 0;
    double beta_last = 0.0;
    for (int j = 0; j < kdim; ++j) {
      const double* vj = V.as<double>() + (int64_t)j * n;
      H(vj, w.as<double>());
      std::vector<double> hh(j + 1, 0.0);
      for (int pass = 0; pass < 2; ++pass) {  // w -= V^T (V w), twice
        la::gemm<double>(ctx, {la::GemmJob{V.p, w.p, h.p, j + 1, 1, n, n, 1, 1, 0, 0, 1.0, 0.0}});
        la::gemm<double>(ctx, {la::GemmJob{V.p, h.p, w.p, n, 1, j + 1, n, 1, 1, 1, 0, -1.0, 1.0}});
        std::vector<double> hp(j + 1);
        TNFA_CUDA(cudaMemcpyAsync(hp.data(), h.p, (j + 1) * 8, cudaMemcpyDeviceToHost, ctx->stream));
        TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
        for (int k = 0; k <= j; ++k) hh[k] += hp[k];
      }
      for (int k = 0; k <= j; ++k) {
        T[(size_t)k * kdim + j] = hh[k];
        T[(size_t)j * kdim + k] = hh[k];
      }
      m = j + 1;
      const double beta = std::sqrt(std::max(0.0, dev_dot(ctx, w.as<double>(), w.as<double>(), n, one)));
      beta_last = beta;
      if (j + 1 == kdim || beta <= 1e-14 * (std::fabs(hh[j]) + 1e-300)) break;
      T[(size_t)j * kdim + j + 1] = T[(size_t)(j + 1) * kdim + j] = beta;
      k_scale_copy<<<g, 256, 0, ctx->stream>>>(V.as<double>() + (int64_t)(j + 1) * n, w.as<double>(), n, 1.0 / beta);
      TNFA_LAUNCH_CHECK();
    }
    std::vector<double> Tm((size_t)m * m);
    for (int a = 0; a < m; ++a)
      for (int b = 0; b < m; ++b) Tm[(size_t)a * m + b] = T[(size_t)a * kdim + b];
    std::vector<double> y;
    sym_eig_min(Tm, m, theta, y);
    // v = V^T y
    DBuf dy(ctx, (size_t)m * 8);
    TNFA_CUDA(cudaMemcpyAsync(dy.p, y.data(), m * 8, cudaMemcpyHostToDevice, ctx->stream));
    la::gemm<double>(ctx, {la::GemmJob{V.p, dy.p, v, n, 1, m, n, 1, 1, 1, 0, 1.0, 0.0}});
    TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
    const double resid = beta_last * std::fabs(y[m - 1]);
    if (resid <= tol * std::max(1.0, std::fabs(theta)) || m < kdim) break;
  }
  const double nv = std::sqrt(dev_dot(ctx, v, v, n, one));
  k_scale_copy<<<grid_for(n, 256, 1024), 256, 0, ctx->stream>>>(v, v, n, 1.0 / nv);
  TNFA_LAUNCH_CHECK();
  return theta;
}

// Solve A x = g (device vectors of length n) by restarted GMRES(m) from the
// given x, Arnoldi with two classical Gram-Schmidt passes, Givens rotations
// on the host; stops when the residual estimate is <= tol |g|.
void gmres(tnfa_ctx* ctx, const MatVec& A, int n, const double* g, double* x, int m, int restarts,
           double tol) {
  m = std::max(1, std::min(m, n));
  DBuf V(ctx, (size_t)(m + 1) * n * 8), w(ctx, (size_t)n * 8), h(ctx, (size_t)(m + 1) * 8), one(ctx, 8);
  const double gn = std::sqrt(dev_dot(ctx, g, g, n, one));
  if (gn == 0.0) {
    TNFA_CUDA(cudaMemsetAsync(x, 0, (size_t)n * 8, ctx->stream));
    return;
  }
  const unsigned gr = grid_for(n, 256, 1024);
  for (int rs = 0; rs <= restarts; ++rs) {
    // r = g - A x
    A(x, w.as<double>());
    k_scale_copy<<<gr, 256, 0, ctx->stream>>>(w.as<double>(), w.as<double>(), n, -1.0);
    k_axpy<<<gr, 256, 0, ctx->stream>>>(w.as<double>(), g, n, 1.0);
    TNFA_LAUNCH_CHECK();
    const double beta = std::sqrt(dev_dot(ctx, w.as<double>(), w.as<double>(), n, one));
    if (beta <= tol * gn) return;
    k_scale_copy<<<gr, 256, 0, ctx->stream>>>(V.as<double>(), w.as<double>(), n, 1.0 / beta);
    TNFA_LAUNCH_CHECK();
    std::vector<double> Hh((size_t)(m + 1) * m, 0.0), cs(m, 0.0), sn(m, 0.0), sv(m + 1, 0.0);
    sv[0] = beta;
    int k = 0;
    for (int j = 0; j < m; ++j) {
      A(V.as<double>() + (int64_t)j * n, w.as<double>());
      std::vector<double> hh(j + 1, 0.0);
      for (int pass = 0; pass < 2; ++pass) {
        la::gemm<double>(ctx, {la::GemmJob{V.p, w.p, h.p, j + 1, 1, n, n, 1, 1, 0, 0, 1.0, 0.0}});
        la::gemm<double>(ctx, {la::GemmJob{V.p, h.p, w.p, n, 1, j + 1, n, 1, 1, 1, 0, -1.0, 1.0}});
        std::vector<double> hp(j + 1);
        TNFA_CUDA(cudaMemcpyAsync(hp.data(), h.p, (j + 1) * 8, cudaMemcpyDeviceToHost, ctx->stream));
        TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
        for (int q = 0; q <= j; ++q) hh[q] += hp[q];
      }
      const double hn = std::sqrt(std::max(0.0, dev_dot(ctx, w.as<double>(), w.as<double>(), n, one)));
      for (int q = 0; q <= j; ++q) Hh[(size_t)q * m + j] = hh[q];
      Hh[(size_t)(j + 1) * m + j] = hn;
      for (int q = 0; q < j; ++q) {  // earlier rotations on the new column
        const double a = Hh[(size_t)q * m + j], b = Hh[(size_t)(q + 1) * m + j];
        Hh[(size_t)q * m + j] = cs[q] * a + sn[q] * b;
        Hh[(size_t)(q + 1) * m + j] = -sn[q] * a + cs[q] * b;
      }
      const double a = Hh[(size_t)j * m + j], b = Hh[(size_t)(j + 1) * m + j];
      const double rr = std::hypot(a, b);
      cs[j] = rr > 0 ? a / rr : 1.0;
      sn[j] = rr > 0 ? b / rr : 0.0;
      Hh[(size_t)j * m + j] = rr;
      Hh[(size_t)(j + 1) * m + j] = 0.0;
      sv[j + 1] = -sn[j] * sv[j];
      sv[j] = cs[j] * sv[j];
      k = j + 1;
      if (std::fabs(sv[j + 1]) <= tol * gn || hn <= 1e-300) break;
      k_scale_copy<<<gr, 256, 0, ctx->stream>>>(V.as<double>() + (int64_t)(j + 1) * n, w.as<double>(), n,
                                                1.0 / hn);
      TNFA_LAUNCH_CHECK();
    }
    // y = R^-1 s, x += V^T y
    std::vector<double> y(k, 0.0);
    for (int q = k - 1; q >= 0; --q) {
      double t = sv[q];
      for (int c = q + 1; c < k; ++c) t -= Hh[(size_t)q * m + c] * y[c];
      y[q] = Hh[(size_t)q * m + q] != 0.0 ? t / Hh[(size_t)q * m + q] : 0.0;
    }
    DBuf dy(ctx, (size_t)k * 8);
    TNFA_CUDA(cudaMemcpyAsync(dy.p, y.data(), k * 8, cudaMemcpyHostToDevice, ctx->stream));
    la::gemm<double>(ctx, {la::GemmJob{V.p, dy.p, x, n, 1, k, n, 1, 1, 1, 0, 1.0, 1.0}});
    TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
    if (std::fabs(sv[k]) <= tol * gn) return;
  }
}

// x_i x_{i+1} as v [l][s1][s2][r].
Dense two_site(LinsolveState& S, int i) {
  tnfa_ctx* ctx = S.ctx;
  const int d = S.d;
  const int l = S.bond(S.x, i), k = S.bond(S.x, i + 1), r = S.bond(S.x, i + 2);
  Dense a = permuted(ctx, S.x.t[i].as<double>(), {d, l, k}, {1, 0, 2});      // [l][s1][k]
  Dense b = permuted(ctx, S.x.t[i + 1].as<double>(), {d, k, r}, {1, 0, 2});  // [k][s2][r]
  return mm(ctx, a.p(), b.p(), l * d, d * r, k, 0, 0, {l, d, d, r});
}

// Solve the projected system at bond (i, i+1); returns v [l][s1][s2][r].
Dense local_solve(LinsolveState& S, int i, double a0, double a1) {
  tnfa_ctx* ctx = S.ctx;
  const int d = S.d;
  const int l = S.bond(S.x, i), r = S.bond(S.x, i + 2);
  const int64_t n64 = (int64_t)l * d * d * r;
  TNFA_CHECK(n64 < (int64_t(1) << 31), TNFA_ERR_UNSUPPORTED, "linsolve: two-site system too large");
  const int n = (int)n64;
  // g[l][s1][s2][r] = Lb_i b_i b_{i+1} Rb_{i+2}
  const int bl = S.bond(S.b, i), bm = S.bond(S.b, i + 1), br = S.bond(S.b, i + 2);
  Dense b1 = permuted(ctx, S.b.t[i].as<double>(), {d, bl, bm}, {1, 0, 2});      // [bl][s][bm]
  Dense G1 = mm(ctx, S.Lb[i].p(), b1.p(), l, d * bm, bl, 0, 0, {l, d, bm});
  Dense b2 = permuted(ctx, S.b.t[i + 1].as<double>(), {d, bm, br}, {1, 0, 2});  // [bm][s][br]
  Dense G2 = mm(ctx, G1.p(), b2.p(), l * d, d * br, bm, 0, 0, {l, d, d, br});
  Dense g = mm(ctx, G2.p(), S.Rb[i + 2].p(), l * d * d, r, br, 0, 1, {l, d, d, r});
  if (n64 <= kLocalDenseMax && !force_matrix_free()) {
    Dense H = local_H(S, i, a0, a1, "linsolve");
    TNFA_CHECK(la::lu_solve(ctx, H.p(), g.p(), n), TNFA_ERR_NOT_CONVERGED,
               "linsolve: singular two-site system at bond " + std::to_string(i + 1));
    return g;
  }
  // large two-site systems: matrix-free GMRES from the current two-site tensor
  Dense x = two_site(S, i);
  LocalOp op(S, i, a0, a1);
  gmres(ctx, [&](const double* u, double* y) { op(u, y); }, n, g.p(), x.p(), 40, 20, 1e-12);
  return x;
}

// ||net|| through a QR sweep toward the root (backward stable).
double qr_norm(tnfa_ctx* ctx, const tnfa_net* net) {
  Work<double> w = load_work<double>(ctx, net);
  orthogonalize_to_roots(w);
  double s2 = 0;
  for (int r : w.topo.roots()) {
    const double x = host_norm<double>(ctx, w.t[r], w.size(r));
    s2 += x * x;
  }
  return std::sqrt(s2);
}

struct NetHold {
  tnfa_net* p = nullptr;
  NetHold() = default;
  explicit NetHold(tnfa_net* q) : p(q) {}
  NetHold(const NetHold&) = delete;
  NetHold& operator=(const NetHold&) = delete;
  ~NetHold() {
    if (p) tnfa_net_destroy(p);
  }
};

void abi(tnfa_ctx* ctx, int status) {
  if (status != TNFA_OK) fail(status, ctx->last_error);
}

// (a0 + a1 A) x - b as a network (bond dims add up; nothing truncated).
tnfa_net* residual_network(tnfa_ctx* ctx, const tnfa_net* A, const tnfa_net* b, Work<double>& x,
                           double a0, double a1) {
  NetHold xr(store_work(x, TNFA_F64));
  Work<double> ax = apply_exact<double>(ctx, A, xr.p);
  NetHold y(store_work(ax, TNFA_F64));
  abi(ctx, tnfa_net_scale(ctx, y.p, 0, a1, 0.0));
  NetHold bneg;
  abi(ctx, tnfa_net_copy(ctx, b, &bneg.p));
  abi(ctx, tnfa_net_scale(ctx, bneg.p, 0, -1.0, 0.0));
  NetHold r1(direct_sum_ext(ctx, y.p, bneg.p));
  if (a0 == 0.0) {
    tnfa_net* out = r1.p;
    r1.p = nullptr;
    return out;
  }
  abi(ctx, tnfa_net_scale(ctx, xr.p, 0, a0, 0.0));
  return direct_sum_ext(ctx, r1.p, xr.p);
}

// ||(a0 + a1 A) x - b|| / ||b|| (A, b and x on one layout).
double residual(tnfa_ctx* ctx, const tnfa_net* A, const tnfa_net* b, Work<double>& x, double a0,
                double a1, double bnorm) {
  NetHold r(residual_network(ctx, A, b, x, a0, a1));
  return qr_norm(ctx, r.p) / bnorm;
}

}  // namespace

tnfa_net* apply_truncate(tnfa_ctx* ctx, const tnfa_net* op, const tnfa_net* f,
                         const tnfa_trunc_params& prm) {
  TNFA_CHECK(op->dtype == f->dtype, TNFA_ERR_DTYPE, "apply: operator and function types differ");
  if (f->dtype == TNFA_F64) {
    Work<double> w = apply_exact<double>(ctx, op, f);
    return truncate_work(w, TNFA_F64, prm);
  }
  if (f->dtype == TNFA_C128) {
    Work<cplx> w = apply_exact<cplx>(ctx, op, f);
    return truncate_work(w, TNFA_C128, prm);
  }
  fail(TNFA_ERR_DTYPE, "apply: FP64 or complex128 networks");
}

tnfa_net* truncate_net(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_trunc_params& prm) {
  if (f->dtype == TNFA_F64) {
    Work<double> w = load_work<double>(ctx, f);
    return truncate_work(w, TNFA_F64, prm);
  }
  if (f->dtype == TNFA_C128) {
    Work<cplx> w = load_work<cplx>(ctx, f);
    return truncate_work(w, TNFA_C128, prm);
  }
  fail(TNFA_ERR_DTYPE, "truncate: FP64 or complex128 networks");
}

tnfa_net* direct_sum(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_net* g);  // algebra.cu

namespace {
tnfa_net* direct_sum_ext(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_net* g) {
  return direct_sum(ctx, f, g);
}
}  // namespace

tnfa_net* linsolve_path(tnfa_ctx* ctx, const tnfa_net* A, const tnfa_net* b, const tnfa_net* x0,
                        const tnfa_linsolve_params& prm, double* rel_res) {
  TNFA_CHECK(A->dtype == TNFA_F64 && b->dtype == TNFA_F64 && x0->dtype == TNFA_F64, TNFA_ERR_DTYPE,
             "linsolve works on FP64 networks");
  check_same_tree(A->topo, b->topo, "linsolve (A, b)");
  check_same_tree(x0->topo, b->topo, "linsolve (x0, b)");
  TNFA_CHECK(b->topo.V >= 2, TNFA_ERR_UNSUPPORTED, "linsolve needs at least two vertices");
  for (int v = 0; v < b->topo.V; ++v)
    TNFA_CHECK(b->topo.nlegs[v] == 1, TNFA_ERR_UNSUPPORTED, "linsolve needs one site leg per vertex");
  for (int l = 0; l < b->topo.leg_off[b->topo.V]; ++l) {
    TNFA_CHECK(A->topo.leg_kind[l] == TNFA_LEG_OPERATOR && b->topo.leg_kind[l] != TNFA_LEG_OPERATOR &&
                   x0->topo.leg_kind[l] != TNFA_LEG_OPERATOR,
               TNFA_ERR_INVALID_ARGUMENT, "linsolve(A, b, x0): A an operator, b and x0 functions");
    TNFA_CHECK(b->topo.leg_dim[l] == b->topo.leg_dim[0] && x0->topo.leg_dim[l] == b->topo.leg_dim[l] &&
                   A->topo.leg_dim[l] == b->topo.leg_dim[l] * b->topo.leg_dim[l],
               TNFA_ERR_SHAPE, "linsolve: site dimensions of A, b, x0 disagree");
  }
  const std::vector<int> ord = path_order(b->topo);
  const int L = b->topo.V;
  LinsolveState S{ctx, L, b->topo.leg_dim[0],
                  relayout<double>(ctx, x0->topo, x0->d, path_topo(x0->topo, ord), ord),
                  relayout<double>(ctx, A->topo, A->d, path_topo(A->topo, ord), ord),
                  relayout<double>(ctx, b->topo, b->d, path_topo(b->topo, ord), ord),
                  {}, {}, {}, {}};
  NetHold An(store_work(S.A, TNFA_F64)), bn(store_work(S.b, TNFA_F64));
  const double bnorm = qr_norm(ctx, bn.p);
  TNFA_CHECK(bnorm > 0, TNFA_ERR_INVALID_ARGUMENT, "linsolve: b is zero");
  orthogonalize_to_roots(S.x);  // right-orthonormal, centre at vertex 0
  S.x.topo.finalize();
  S.LA.resize(L + 1);
  S.RA.resize(L + 1);
  S.Lb.resize(L + 1);
  S.Rb.resize(L + 1);
  S.LA[0] = ones(ctx, {1, 1, 1});
  S.RA[L] = ones(ctx, {1, 1, 1});
  S.Lb[0] = ones(ctx, {1, 1});
  S.Rb[L] = ones(ctx, {1, 1});
  for (int i = L - 1; i >= 2; --i) right_env(S, i);
  const tnfa_trunc_params tp{prm.cutoff, prm.maxdim, 1, 0, TNFA_PREC_F64};
  TruncStats st;
  double res = residual(ctx, An.p, bn.p, S.x, prm.a0, prm.a1, bnorm);
  for (int sweep = 0; sweep < prm.nsweeps && res > prm.tol; ++sweep) {
    for (int dir = 0; dir < 2 && res > prm.tol; ++dir) {
      for (int step = 0; step + 1 < L; ++step) {
        const int i = dir == 0 ? step : L - 2 - step;
        Dense v = local_solve(S, i, prm.a0, prm.a1);
        store_two_site(S, i, v, tp, st, dir == 0);
        if (dir == 0) left_env(S, i);
        else right_env(S, i + 1);
      }
      res = residual(ctx, An.p, bn.p, S.x, prm.a0, prm.a1, bnorm);
    }
  }
  if (rel_res) *rel_res = res;
  // back to the caller's numbering and rooting
  NetHold xp(store_work(S.x, TNFA_F64));
  Topo back = x0->topo;
  for (int k = 1; k < L; ++k) {
    const int c = ord[k], cp = ord[k - 1];
    (back.parent[c] == cp ? back.link[c] : back.link[cp]) = S.x.topo.link[k];
  }
  back.finalize();
  std::vector<int> pos(L);
  for (int k = 0; k < L; ++k) pos[ord[k]] = k;
  Work<double> wb = relayout<double>(ctx, xp.p->topo, xp.p->d, back, pos);
  return store_work(wb, TNFA_F64);
}

tnfa_net* linsolve_any(tnfa_ctx* ctx, const tnfa_net* A, const tnfa_net* b, const tnfa_net* x0,
                       const tnfa_linsolve_params& prm, double* rel_res);

// linsolve (path or tree sweep) followed by iterative refinement on the
// caller's layout.
tnfa_net* linsolve_refined(tnfa_ctx* ctx, const tnfa_net* A, const tnfa_net* b, const tnfa_net* x0,
                           const tnfa_linsolve_params& prm, double* rel_res) {
  double res = 0.0;
  NetHold x(linsolve_any(ctx, A, b, x0, prm, &res));
  if (prm.refinements > 0 && res > prm.tol) {
    const double bnorm = qr_norm(ctx, b);
    const tnfa_trunc_params tr{prm.refine_cutoff, prm.maxdim, 1, 0, TNFA_PREC_F64};
    tnfa_linsolve_params pe = prm;
    pe.refinements = 0;
    pe.tol = 0.0;
    for (int k = 0; k < prm.refinements && res > prm.tol; ++k) {
      // e solves (a0 + a1 A) e = b - (a0 + a1 A) x
      Work<double> xw = load_work<double>(ctx, x.p);
      NetHold r(residual_network(ctx, A, b, xw, prm.a0, prm.a1));
      abi(ctx, tnfa_net_scale(ctx, r.p, 0, -1.0, 0.0));
      NetHold rt(truncate_net(ctx, r.p, tr));
      double eres = 0.0;
      NetHold e(linsolve_any(ctx, A, rt.p, rt.p, pe, &eres));
      NetHold sum(direct_sum_ext(ctx, x.p, e.p));
      NetHold xn(truncate_net(ctx, sum.p, tr));
      Work<double> xnw = load_work<double>(ctx, xn.p);
      const double rn = residual(ctx, A, b, xnw, prm.a0, prm.a1, bnorm);
      if (!(rn < res)) break;  // no progress: keep the previous solution
      std::swap(x.p, xn.p);
      res = rn;
    }
  }
  if (rel_res) *rel_res = res;
  tnfa_net* out = x.p;
  x.p = nullptr;
  return out;
}

// Two-site DMRG for the lowest eigenpair of a symmetric operator on a path.
tnfa_net* dmrg_path(tnfa_ctx* ctx, const tnfa_net* A, const tnfa_net* x0, const tnfa_dmrg_params& prm,
                    double* energy) {
  TNFA_CHECK(A->dtype == TNFA_F64 && x0->dtype == TNFA_F64, TNFA_ERR_DTYPE, "dmrg works on FP64 networks");
  check_same_tree(A->topo, x0->topo, "dmrg (H, psi0)");
  TNFA_CHECK(x0->topo.V >= 2, TNFA_ERR_UNSUPPORTED, "dmrg needs at least two vertices");
  for (int v = 0; v < x0->topo.V; ++v)
    TNFA_CHECK(x0->topo.nlegs[v] == 1, TNFA_ERR_UNSUPPORTED, "dmrg needs one site leg per vertex");
  for (int l = 0; l < x0->topo.leg_off[x0->topo.V]; ++l) {
    TNFA_CHECK(A->topo.leg_kind[l] == TNFA_LEG_OPERATOR && x0->topo.leg_kind[l] != TNFA_LEG_OPERATOR,
               TNFA_ERR_INVALID_ARGUMENT, "dmrg(H, psi0): H an operator, psi0 a function");
    TNFA_CHECK(x0->topo.leg_dim[l] == x0->topo.leg_dim[0] &&
                   A->topo.leg_dim[l] == x0->topo.leg_dim[l] * x0->topo.leg_dim[l],
               TNFA_ERR_SHAPE, "dmrg: site dimensions of H and psi0 disagree");
  }
  const std::vector<int> ord = path_order(x0->topo);
  const int L = x0->topo.V;
  LinsolveState S{ctx, L, x0->topo.leg_dim[0],
                  relayout<double>(ctx, x0->topo, x0->d, path_topo(x0->topo, ord), ord),
                  relayout<double>(ctx, A->topo, A->d, path_topo(A->topo, ord), ord),
                  Work<double>{ctx, Topo{}, {}}, {}, {}, {}, {}};
  S.has_b = false;
  orthogonalize_to_roots(S.x);
  S.x.topo.finalize();
  S.LA.resize(L + 1);
  S.RA.resize(L + 1);
  S.LA[0] = ones(ctx, {1, 1, 1});
  S.RA[L] = ones(ctx, {1, 1, 1});
  for (int i = L - 1; i >= 2; --i) right_env(S, i);
  const tnfa_trunc_params tp{prm.cutoff, prm.maxdim, 1, 0, TNFA_PREC_F64};
  TruncStats st;
  double E = 0.0, Eprev = 0.0;
  for (int sweep = 0; sweep < std::max(1, prm.nsweeps); ++sweep) {
    for (int dir = 0; dir < 2; ++dir) {
      for (int step = 0; step + 1 < L; ++step) {
        const int i = dir == 0 ? step : L - 2 - step;
        Dense v = two_site(S, i);
        const int64_t n64 = (int64_t)S.bond(S.x, i) * S.d * S.d * S.bond(S.x, i + 2);
        TNFA_CHECK(n64 < (int64_t(1) << 31), TNFA_ERR_UNSUPPORTED, "dmrg: two-site problem too large");
        const int n = (int)n64;
        const int kd = prm.krylov_dim > 0 ? prm.krylov_dim : 30;
        if (n64 <= kLocalDenseSmall && !force_matrix_free()) {
          Dense H = local_H(S, i, 0.0, 1.0, "dmrg");
          const double* Hp = H.p();
          E = lanczos_min(
              ctx,
              [&](const double* x, double* y) {
                la::gemm<double>(ctx, {la::GemmJob{Hp, x, y, n, 1, n, n, 1, 1, 0, 0, 1.0, 0.0}});
              },
              n, v.p(), kd, std::max(0, prm.restarts), 1e-12);
        } else {
          LocalOp op(S, i, 0.0, 1.0);
          E = lanczos_min(ctx, [&](const double* x, double* y) { op(x, y); }, n, v.p(), kd,
                          std::max(0, prm.restarts), 1e-12);
        }
        store_two_site(S, i, v, tp, st, dir == 0);
        // keep the state normalised after truncation: rescale the centre
        const int c = dir == 0 ? i + 1 : i;
        const double nc = host_norm<double>(ctx, S.x.t[c], S.x.size(c));
        if (nc > 0)
          k_scale_copy<<<grid_for(S.x.size(c), 256, 1024), 256, 0, ctx->stream>>>(
              S.x.t[c].as<double>(), S.x.t[c].as<double>(), S.x.size(c), 1.0 / nc);
        if (dir == 0) left_env(S, i);
        else right_env(S, i + 1);
      }
    }
    if (sweep > 0 && std::fabs(E - Eprev) <= prm.tol * std::max(1.0, std::fabs(E))) break;
    Eprev = E;
  }
  if (energy) *energy = E;
  NetHold xp(store_work(S.x, TNFA_F64));
  Topo back = x0->topo;
  for (int k = 1; k < L; ++k) {
    const int c = ord[k], cp = ord[k - 1];
    (back.parent[c] == cp ? back.link[c] : back.link[cp]) = S.x.topo.link[k];
  }
  back.finalize();
  std::vector<int> pos(L);
  for (int k = 0; k < L; ++k) pos[ord[k]] = k;
  Work<double> wb = relayout<double>(ctx, xp.p->topo, xp.p->d, back, pos);
  return store_work(wb, TNFA_F64);
}

// ------------------------------------------------------- tree solvers ----
// linsolve and dmrg on any tree (vertices of any degree, one site leg each),
// the sweep ITensorNetworks runs with nsites = 2 on a TreeTensorNetwork:
// the orthogonality centre walks a depth-first tour from the root, every
// edge (u, c) is updated twice per sweep (on the way down the centre moves
// to c, on the way back to u), and each update solves the system projected
// onto the environments of all other edges, then splits the two-site tensor
// by a truncated SVD.  Environments are kept per directed edge (a -> b: the
// part of the network on a's side); those pointing at the centre stay valid
// along the tour.  Contractions are labelled: every tensor carries one label
// per axis and a pairwise contraction (permute + GEMM on the device) sums
// over the labels the two share.

// A device tensor with labelled axes; views (LV) borrow the data.
struct LT {
  Dense d;
  std::vector<int> lab;
};
struct LV {
  const double* p;
  std::vector<int> shp, lab;
};
LV view(const LT& t) { return {t.d.p(), t.d.shp, t.lab}; }

int64_t numel(const std::vector<int>& s) {
  int64_t n = 1;
  for (int x : s) n *= x;
  return n;
}

// Axes of A put in label order `order`.
LT lt_perm(tnfa_ctx* ctx, const LV& A, const std::vector<int>& order) {
  TNFA_CHECK(order.size() == A.lab.size(), TNFA_ERR_INVALID_ARGUMENT, "tree solver: label count");
  std::vector<int> p(order.size());
  for (size_t i = 0; i < order.size(); ++i) {
    const auto it = std::find(A.lab.begin(), A.lab.end(), order[i]);
    TNFA_CHECK(it != A.lab.end(), TNFA_ERR_INVALID_ARGUMENT, "tree solver: missing label");
    p[i] = (int)(it - A.lab.begin());
  }
  return LT{permuted(ctx, A.p, A.shp, p), order};
}

// Sum over the labels A and B share; result axes: A's other labels, then B's.
LT lt_contract(tnfa_ctx* ctx, const LV& A, const LV& B) {
  std::vector<int> sh, fa, fb, sa_dims, fa_dims, fb_dims;
  for (size_t i = 0; i < A.lab.size(); ++i) {
    const auto it = std::find(B.lab.begin(), B.lab.end(), A.lab[i]);
    if (it == B.lab.end()) {
      fa.push_back(A.lab[i]);
      fa_dims.push_back(A.shp[i]);
    } else {
      TNFA_CHECK(B.shp[it - B.lab.begin()] == A.shp[i], TNFA_ERR_SHAPE, "tree solver: bond dims disagree");
      sh.push_back(A.lab[i]);
      sa_dims.push_back(A.shp[i]);
    }
  }
  for (size_t i = 0; i < B.lab.size(); ++i)
    if (std::find(A.lab.begin(), A.lab.end(), B.lab[i]) == A.lab.end()) {
      fb.push_back(B.lab[i]);
      fb_dims.push_back(B.shp[i]);
    }
  const int64_t m = numel(fa_dims), k = numel(sa_dims), n = numel(fb_dims);
  TNFA_CHECK(m < (int64_t(1) << 31) && n < (int64_t(1) << 31) && k < (int64_t(1) << 31),
             TNFA_ERR_UNSUPPORTED, "tree solver: contraction too large");
  // A as [free][shared] (or [shared][free], transposed), B as [shared][free]
  // (or [free][shared]); permute only when neither order holds
  auto cat = [](std::vector<int> a, const std::vector<int>& b) {
    a.insert(a.end(), b.begin(), b.end());
    return a;
  };
  LT ta, tb;
  const double* pa = A.p;
  const double* pb = B.p;
  int opA = 0, opB = 0;
  if (A.lab == cat(fa, sh)) {
    opA = 0;
  } else if (A.lab == cat(sh, fa)) {
    opA = 1;
  } else {
    ta = lt_perm(ctx, A, cat(fa, sh));
    pa = ta.d.p();
  }
  if (B.lab == cat(sh, fb)) {
    opB = 0;
  } else if (B.lab == cat(fb, sh)) {
    opB = 1;
  } else {
    tb = lt_perm(ctx, B, cat(sh, fb));
    pb = tb.d.p();
  }
  LT out;
  out.lab = cat(fa, fb);
  out.d = mm(ctx, pa, pb, (int)m, (int)n, (int)k, opA, opB, cat(fa_dims, fb_dims));
  return out;
}

struct TreeSolve {
  tnfa_ctx* ctx;
  int V, d, root;
  Work<double> x, A, b;
  bool has_b = true;
  std::map<std::pair<int, int>, LT> EA, Eb;  // directed edge (from, to); from -1: the root's open end
  enum { S = 0, SP = 1, K = 2, KP = 3, W = 4, B = 5 };
  int lab(int kind, int id) const { return kind * V + id; }  // id: a vertex or an edge (its child)
  // edges of u: (edge id, neighbour); the edge to the parent has u's id (the
  // root's is its open end, neighbour -1), the edge to a child that child's
  std::vector<std::pair<int, int>> edges(int u) const {
    std::vector<std::pair<int, int>> e{{u, x.topo.parent[u]}};
    for (int c : x.topo.children[u]) e.push_back({c, c});
    return e;
  }
  std::vector<int> xlab(int u, int ks = K, int ss = S) const {
    std::vector<int> l{lab(ss, u), lab(ks, u)};
    for (int c : x.topo.children[u]) l.push_back(lab(ks, c));
    return l;
  }
  LV xv(int u) const { return {x.t[u].as<double>(), x.shape(u), xlab(u)}; }
  LV xbra(int u) const { return {x.t[u].as<double>(), x.shape(u), xlab(u, KP, SP)}; }
  LV av(int u) const {
    std::vector<int> shp = A.shape(u);
    shp.erase(shp.begin());
    shp.insert(shp.begin(), {d, d});  // fused site leg out * d + in
    std::vector<int> l{lab(SP, u), lab(S, u), lab(W, u)};
    for (int c : A.topo.children[u]) l.push_back(lab(W, c));
    return {A.t[u].as<double>(), shp, l};
  }
  LV bv(int u) const {
    std::vector<int> l{lab(S, u), lab(B, u)};
    for (int c : b.topo.children[u]) l.push_back(lab(B, c));
    return {b.t[u].as<double>(), b.shape(u), l};
  }
  // environments of the edge from a toward `to` (a is orthonormal toward it)
  void env(int a, int to) {
    const int e = to == x.topo.parent[a] ? a : to;
    LT T{Dense{}, {}};
    bool have = false;
    auto cur = [&](const LV& base) { return have ? view(T) : base; };
    const LV xa = xv(a);
    for (auto [f, w] : edges(a)) {
      if (f == e) continue;
      LT n = lt_contract(ctx, cur(xa), view(EA.at({w, a})));
      T = std::move(n);
      have = true;
    }
    {
      LT n = lt_contract(ctx, cur(xa), av(a));
      T = std::move(n);
      have = true;
    }
    LT n = lt_contract(ctx, view(T), xbra(a));
    EA[{a, to}] = lt_perm(ctx, view(n), {lab(KP, e), lab(W, e), lab(K, e)});
    if (!has_b) return;
    have = false;
    const LV ba = bv(a);
    for (auto [f, w] : edges(a)) {
      if (f == e) continue;
      LT m = lt_contract(ctx, cur(ba), view(Eb.at({w, a})));
      T = std::move(m);
      have = true;
    }
    LT m = lt_contract(ctx, cur(ba), xa);
    Eb[{a, to}] = lt_perm(ctx, view(m), {lab(K, e), lab(B, e)});
  }
  void open_end() {
    LT ea{ones(ctx, {1, 1, 1}), {lab(KP, root), lab(W, root), lab(K, root)}};
    EA[{-1, root}] = std::move(ea);
    if (has_b) {
      LT eb{ones(ctx, {1, 1}), {lab(K, root), lab(B, root)}};
      Eb[{-1, root}] = std::move(eb);
    }
  }
  // the external edges of the two-site block (u, c): (edge, neighbour, owner)
  std::vector<std::array<int, 3>> outer(int u, int c) const {
    std::vector<std::array<int, 3>> o;
    for (auto [f, w] : edges(u))
      if (f != c) o.push_back({f, w, u});
    for (int g : x.topo.children[c]) o.push_back({g, g, c});
    return o;
  }
  // y = a0 th + a1 H th for a two-site tensor with labels tl
  void matvec(int u, int c, const std::vector<int>& tl, const std::vector<int>& ts, const double* th,
              double* y, double a0, double a1) {
    // u's environments, then A_u, then c's environments, then A_c: keeps the
    // intermediate's order low on high-degree vertices
    LT T{Dense{}, {}};
    bool have = false;
    const LV t0{th, ts, tl};
    for (int side = 0; side < 2; ++side) {
      const int owner = side == 0 ? u : c;
      for (auto& o : outer(u, c)) {
        if (o[2] != owner) continue;
        LT n = lt_contract(ctx, have ? view(T) : t0, view(EA.at({o[1], o[2]})));
        T = std::move(n);
        have = true;
      }
      LT n = lt_contract(ctx, have ? view(T) : t0, av(owner));
      T = std::move(n);
      have = true;
    }
    // primed labels back to unprimed, axes in the order of th
    for (int& l : T.lab) {
      const int kind = l / V, id = l % V;
      if (kind == SP) l = lab(S, id);
      if (kind == KP) l = lab(K, id);
    }
    LT r = lt_perm(ctx, view(T), tl);
    const int64_t n = numel(ts);
    TNFA_CUDA(cudaMemcpyAsync(y, r.d.p(), n * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    if (a1 != 1.0) {
      k_scale_copy<<<grid_for(n, 256, 1024), 256, 0, ctx->stream>>>(y, y, n, a1);
      TNFA_LAUNCH_CHECK();
    }
    if (a0 != 0.0) {
      k_axpy<<<grid_for(n, 256, 1024), 256, 0, ctx->stream>>>(y, th, n, a0);
      TNFA_LAUNCH_CHECK();
    }
  }
  // two-site right-hand side with labels tl
  LT rhs(int u, int c, const std::vector<int>& tl) {
    LT T = lt_contract(ctx, bv(u), bv(c));
    for (auto& o : outer(u, c)) {
      LT n = lt_contract(ctx, view(T), view(Eb.at({o[1], o[2]})));
      T = std::move(n);
    }
    return lt_perm(ctx, view(T), tl);
  }
  // update of edge (u, c) (c a child of u), the centre moving to c (down) or
  // back to u; returns the local eigenvalue for dmrg
  double update(int u, int c, bool down, double a0, double a1, const tnfa_trunc_params& tp, int kdim,
                int restarts) {
    LT th = lt_contract(ctx, xv(u), xv(c));
    const std::vector<int> tl = th.lab, ts = th.d.shp;
    const int64_t n64 = numel(ts);
    TNFA_CHECK(n64 < (int64_t(1) << 31), TNFA_ERR_UNSUPPORTED, "tree solver: two-site problem too large");
    const int n = (int)n64;
    double E = 0.0;
    MatVec H = [&](const double* in, double* out) { matvec(u, c, tl, ts, in, out, a0, a1); };
    if (has_b) {
      LT g = rhs(u, c, tl);
      gmres(ctx, H, n, g.d.p(), th.d.p(), 40, 20, 1e-12);
    } else {
      E = lanczos_min(ctx, H, n, th.d.p(), kdim, restarts, 1e-12);
    }
    // split: rows are the side that keeps orthonormal columns
    std::vector<int> ul{lab(S, u), lab(K, u)}, cl{lab(S, c)};
    for (int w : x.topo.children[u])
      if (w != c) ul.push_back(lab(K, w));
    for (int g : x.topo.children[c]) cl.push_back(lab(K, g));
    const std::vector<int>& rl = down ? ul : cl;
    const std::vector<int>& kl = down ? cl : ul;
    std::vector<int> order = rl;
    order.insert(order.end(), kl.begin(), kl.end());
    LT M = lt_perm(ctx, view(th), order);
    int64_t rows = 1, cols = 1;
    for (size_t i = 0; i < rl.size(); ++i) rows *= M.d.shp[i];
    for (size_t i = rl.size(); i < order.size(); ++i) cols *= M.d.shp[i];
    std::vector<la::FactorResult> res;
    la::trunc_factor<double>(ctx, {la::FactorJob{M.d.p(), (int)rows, (int)cols}}, tp.cutoff, tp.maxdim,
                             tp.mindim, TNFA_PREC_F64, res);
    TNFA_CHECK(res[0].sweeps >= 0, TNFA_ERR_NOT_CONVERGED, "Jacobi SVD hit its sweep cap");
    const int r = res[0].r;
    std::vector<int> lshp(M.d.shp.begin(), M.d.shp.begin() + rl.size());
    lshp.push_back(r);
    std::vector<int> xshp{r};
    xshp.insert(xshp.end(), M.d.shp.begin() + rl.size(), M.d.shp.end());
    std::vector<int> llab = rl;
    llab.push_back(lab(K, c));
    std::vector<int> xlb{lab(K, c)};
    xlb.insert(xlb.end(), kl.begin(), kl.end());
    x.topo.link[c] = r;
    const int ortho = down ? u : c, centre = down ? c : u;
    LT no = lt_perm(ctx, LV{res[0].L.as<double>(), lshp, llab}, xlab(ortho));
    LT nc = lt_perm(ctx, LV{res[0].X.as<double>(), xshp, xlb}, xlab(centre));
    x.t[ortho] = std::move(no.d.b);
    x.t[centre] = std::move(nc.d.b);
    if (!has_b) {
      // keep the state normalised after truncation: rescale the centre
      const int64_t nn = x.size(centre);
      const double nr = host_norm<double>(ctx, x.t[centre], nn);
      if (nr > 0) {
        k_scale_copy<<<grid_for(nn, 256, 1024), 256, 0, ctx->stream>>>(x.t[centre].as<double>(),
                                                                         x.t[centre].as<double>(), nn, 1.0 / nr);
        TNFA_LAUNCH_CHECK();
      }
    }
    env(ortho, centre);
    return E;
  }
  double tour(int u, double a0, double a1, const tnfa_trunc_params& tp, int kdim, int restarts) {
    double E = 0.0;
    for (int c : x.topo.children[u]) {
      E = update(u, c, true, a0, a1, tp, kdim, restarts);
      const double Ec = tour(c, a0, a1, tp, kdim, restarts);
      if (!x.topo.children[c].empty()) E = Ec;
      E = update(u, c, false, a0, a1, tp, kdim, restarts);
    }
    return E;
  }
  void init() {
    orthogonalize_to_roots(x);  // every vertex orthonormal toward its parent, centre at the root
    x.topo.finalize();
    open_end();
    for (int v = V - 1; v >= 0; --v)  // children have larger indices than their parent
      if (v != root) env(v, x.topo.parent[v]);
  }
};

bool path_shaped(const Topo& T) {
  if (T.roots().size() != 1) return false;
  for (int v = 0; v < T.V; ++v)
    if ((int)T.children[v].size() + (T.parent[v] >= 0 ? 1 : 0) > 2) return false;
  return true;
}

void check_tree_solve(const tnfa_net* A, const tnfa_net* f, const char* what) {
  TNFA_CHECK(A->dtype == TNFA_F64 && f->dtype == TNFA_F64, TNFA_ERR_DTYPE,
             std::string(what) + " works on FP64 networks");
  check_same_tree(A->topo, f->topo, what);
  TNFA_CHECK(f->topo.V >= 2 && f->topo.roots().size() == 1, TNFA_ERR_UNSUPPORTED,
             std::string(what) + " needs one connected tree of at least two vertices");
  TNFA_CHECK(f->topo.roots()[0] == 0, TNFA_ERR_TOPOLOGY, std::string(what) + ": the root must be vertex 0");
  for (int v = 0; v < f->topo.V; ++v)
    TNFA_CHECK(f->topo.nlegs[v] == 1, TNFA_ERR_UNSUPPORTED, std::string(what) + " needs one site leg per vertex");
  for (int l = 0; l < f->topo.leg_off[f->topo.V]; ++l) {
    TNFA_CHECK(A->topo.leg_kind[l] == TNFA_LEG_OPERATOR && f->topo.leg_kind[l] != TNFA_LEG_OPERATOR,
               TNFA_ERR_INVALID_ARGUMENT, std::string(what) + ": an operator and a function");
    TNFA_CHECK(f->topo.leg_dim[l] == f->topo.leg_dim[0] && A->topo.leg_dim[l] == f->topo.leg_dim[l] * f->topo.leg_dim[l],
               TNFA_ERR_SHAPE, std::string(what) + ": site dimensions disagree");
  }
}

tnfa_net* linsolve_tree(tnfa_ctx* ctx, const tnfa_net* A, const tnfa_net* b, const tnfa_net* x0,
                        const tnfa_linsolve_params& prm, double* rel_res) {
  check_tree_solve(A, b, "linsolve (A, b)");
  check_same_tree(x0->topo, b->topo, "linsolve (x0, b)");
  TNFA_CHECK(x0->dtype == TNFA_F64, TNFA_ERR_DTYPE, "linsolve works on FP64 networks");
  TreeSolve S{ctx, b->topo.V, b->topo.leg_dim[0], 0, load_work<double>(ctx, x0), load_work<double>(ctx, A),
              load_work<double>(ctx, b)};
  const double bnorm = qr_norm(ctx, b);
  TNFA_CHECK(bnorm > 0, TNFA_ERR_INVALID_ARGUMENT, "linsolve: b is zero");
  S.init();
  const tnfa_trunc_params tp{prm.cutoff, prm.maxdim, 1, 0, TNFA_PREC_F64};
  double res = residual(ctx, A, b, S.x, prm.a0, prm.a1, bnorm);
  for (int sweep = 0; sweep < prm.nsweeps && res > prm.tol; ++sweep) {
    S.tour(S.root, prm.a0, prm.a1, tp, 0, 0);
    res = residual(ctx, A, b, S.x, prm.a0, prm.a1, bnorm);
  }
  if (rel_res) *rel_res = res;
  return store_work(S.x, TNFA_F64);
}

tnfa_net* dmrg_tree(tnfa_ctx* ctx, const tnfa_net* H, const tnfa_net* x0, const tnfa_dmrg_params& prm,
                    double* energy) {
  check_tree_solve(H, x0, "dmrg (H, psi0)");
  TreeSolve S{ctx, x0->topo.V, x0->topo.leg_dim[0], 0, load_work<double>(ctx, x0), load_work<double>(ctx, H),
              Work<double>{ctx, Topo{}, {}}};
  S.has_b = false;
  S.init();
  const tnfa_trunc_params tp{prm.cutoff, prm.maxdim, 1, 0, TNFA_PREC_F64};
  const int kd = prm.krylov_dim > 0 ? prm.krylov_dim : 30;
  double E = 0.0, Eprev = 0.0;
  for (int sweep = 0; sweep < std::max(1, prm.nsweeps); ++sweep) {
    E = S.tour(S.root, 0.0, 1.0, tp, kd, std::max(0, prm.restarts));
    if (sweep > 0 && std::fabs(E - Eprev) <= prm.tol * std::max(1.0, std::fabs(E))) break;
    Eprev = E;
  }
  if (energy) *energy = E;
  return store_work(S.x, TNFA_F64);
}

tnfa_net* linsolve_any(tnfa_ctx* ctx, const tnfa_net* A, const tnfa_net* b, const tnfa_net* x0,
                       const tnfa_linsolve_params& prm, double* rel_res) {
  return path_shaped(b->topo) ? linsolve_path(ctx, A, b, x0, prm, rel_res)
                              : linsolve_tree(ctx, A, b, x0, prm, rel_res);
}

void inner_product(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_net* g, bool conjF, double* out) {
  TNFA_CHECK(f->dtype == g->dtype, TNFA_ERR_DTYPE, "inner: element types differ");
  if (f->dtype == TNFA_F64) contract_pair<double>(ctx, f, g, conjF, out);
  else if (f->dtype == TNFA_C128) contract_pair<cplx>(ctx, f, g, conjF, out);
  else fail(TNFA_ERR_DTYPE, "inner: FP64 or complex128 networks");
}

}  // namespace tnfa

using namespace tnfa;

extern "C" {

int tnfa_apply(tnfa_ctx* ctx, const tnfa_net* op, const tnfa_net* f,
               const tnfa_trunc_params* params, tnfa_net** out) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(op, "apply operator");
  require_net(f, "apply function");
  check_params(params);
  TNFA_CHECK(out, TNFA_ERR_INVALID_ARGUMENT, "null out");
  *out = apply_truncate(ctx, op, f, *params);
  TNFA_API_END
}

int tnfa_apply_exact(tnfa_ctx* ctx, const tnfa_net* op, const tnfa_net* f, tnfa_net** out) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(op, "apply operator");
  require_net(f, "apply function");
  TNFA_CHECK(out, TNFA_ERR_INVALID_ARGUMENT, "null out");
  TNFA_CHECK(op->dtype == f->dtype, TNFA_ERR_DTYPE, "apply: operator and function types differ");
  if (f->dtype == TNFA_F64) {
    Work<double> w = apply_exact<double>(ctx, op, f);
    *out = store_work(w, TNFA_F64);
  } else if (f->dtype == TNFA_C128) {
    Work<cplx> w = apply_exact<cplx>(ctx, op, f);
    *out = store_work(w, TNFA_C128);
  } else {
    fail(TNFA_ERR_DTYPE, "apply: FP64 or complex128 networks");
  }
  TNFA_API_END
}

int tnfa_apply_vjp(tnfa_ctx* ctx, const tnfa_net* op, const tnfa_net* f, const void* dy,
                   int dy_memory, void* df, int df_memory) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(op, "apply_vjp operator");
  require_net(f, "apply_vjp function");
  TNFA_CHECK(dy && df, TNFA_ERR_INVALID_ARGUMENT, "null dy or df");
  TNFA_CHECK((dy_memory == TNFA_MEM_HOST || dy_memory == TNFA_MEM_DEVICE) &&
                 (df_memory == TNFA_MEM_HOST || df_memory == TNFA_MEM_DEVICE),
             TNFA_ERR_INVALID_ARGUMENT, "bad memory kind");
  TNFA_CHECK(op->dtype == f->dtype, TNFA_ERR_DTYPE, "apply_vjp: operator and function types differ");
  if (f->dtype == TNFA_F64)
    apply_vjp<double>(ctx, op, f, dy, dy_memory, df, df_memory);
  else if (f->dtype == TNFA_C128)
    apply_vjp<cplx>(ctx, op, f, dy, dy_memory, df, df_memory);
  else
    fail(TNFA_ERR_DTYPE, "apply_vjp: FP64 or complex128 networks");
  TNFA_API_END
}

int tnfa_apply_batched(tnfa_ctx* ctx, int32_t n, const tnfa_net* const* ops,
                       const tnfa_net* const* fs, const tnfa_trunc_params* params,
                       tnfa_net** outs) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  check_params(params);
  TNFA_CHECK(n >= 0 && (n == 0 || (ops && fs && outs)), TNFA_ERR_INVALID_ARGUMENT, "null arrays");
  for (int i = 0; i < n; ++i) outs[i] = nullptr;
  try {
    bool paths = n > 0;
    for (int i = 0; i < n; ++i) {
      require_net(ops[i], "apply_batched operator");
      require_net(fs[i], "apply_batched function");
      paths = paths && is_rooted_path(fs[i]->topo) && fs[i]->dtype == fs[0]->dtype &&
              ops[i]->dtype == fs[i]->dtype;
    }
    if (paths && fs[0]->dtype == TNFA_F64)
      batch_apply_truncate<double>(ctx, n, ops, fs, *params, TNFA_F64, outs);
    else if (paths && fs[0]->dtype == TNFA_C128)
      batch_apply_truncate<cplx>(ctx, n, ops, fs, *params, TNFA_C128, outs);
    else
      for (int i = 0; i < n; ++i) outs[i] = apply_truncate(ctx, ops[i], fs[i], *params);
  } catch (...) {
    for (int i = 0; i < n; ++i)
      if (outs[i]) {
        tnfa_net_destroy(outs[i]);
        outs[i] = nullptr;
      }
    throw;
  }
  TNFA_API_END
}

int tnfa_truncate(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_trunc_params* params,
                  tnfa_net** out) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(f, "truncate");
  check_params(params);
  TNFA_CHECK(out, TNFA_ERR_INVALID_ARGUMENT, "null out");
  *out = truncate_net(ctx, f, *params);
  TNFA_API_END
}

int tnfa_truncate_batched(tnfa_ctx* ctx, int32_t n, const tnfa_net* const* fs,
                          const tnfa_trunc_params* params, tnfa_net** outs) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  check_params(params);
  TNFA_CHECK(n >= 0 && (n == 0 || (fs && outs)), TNFA_ERR_INVALID_ARGUMENT, "null arrays");
  for (int i = 0; i < n; ++i) outs[i] = nullptr;
  try {
    bool paths = n > 0;
    for (int i = 0; i < n; ++i) {
      require_net(fs[i], "truncate_batched");
      paths = paths && is_rooted_path(fs[i]->topo) && fs[i]->dtype == fs[0]->dtype;
    }
    if (paths && fs[0]->dtype == TNFA_F64)
      batch_apply_truncate<double>(ctx, n, nullptr, fs, *params, TNFA_F64, outs);
    else if (paths && fs[0]->dtype == TNFA_C128)
      batch_apply_truncate<cplx>(ctx, n, nullptr, fs, *params, TNFA_C128, outs);
    else
      for (int i = 0; i < n; ++i) outs[i] = truncate_net(ctx, fs[i], *params);
  } catch (...) {
    for (int i = 0; i < n; ++i)
      if (outs[i]) {
        tnfa_net_destroy(outs[i]);
        outs[i] = nullptr;
      }
    throw;
  }
  TNFA_API_END
}

int tnfa_inner(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_net* g, double* out) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(f, "inner f");
  require_net(g, "inner g");
  TNFA_CHECK(out, TNFA_ERR_INVALID_ARGUMENT, "null out");
  inner_product(ctx, f, g, true, out);
  TNFA_API_END
}

int tnfa_linsolve(tnfa_ctx* ctx, const tnfa_net* A, const tnfa_net* b, const tnfa_net* x0,
                  const tnfa_linsolve_params* params, tnfa_net** x, double* rel_residual) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(A, "linsolve A");
  require_net(b, "linsolve b");
  require_net(x0, "linsolve x0");
  TNFA_CHECK(params && x, TNFA_ERR_INVALID_ARGUMENT, "null params or out");
  TNFA_CHECK(params->maxdim >= 0 && params->cutoff >= 0 && params->tol >= 0, TNFA_ERR_INVALID_ARGUMENT,
             "negative linsolve parameter");
  double rr = 0;
  TNFA_CHECK(params->refinements >= 0 && params->refine_cutoff >= 0, TNFA_ERR_INVALID_ARGUMENT,
             "negative refinement parameter");
  *x = linsolve_refined(ctx, A, b, x0, *params, &rr);
  if (rel_residual) *rel_residual = rr;
  TNFA_API_END
}

int tnfa_dmrg(tnfa_ctx* ctx, const tnfa_net* H, const tnfa_net* psi0, const tnfa_dmrg_params* params,
              tnfa_net** psi, double* energy) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(H, "dmrg H");
  require_net(psi0, "dmrg psi0");
  TNFA_CHECK(params && psi, TNFA_ERR_INVALID_ARGUMENT, "null params or out");
  TNFA_CHECK(params->maxdim >= 0 && params->cutoff >= 0 && params->tol >= 0, TNFA_ERR_INVALID_ARGUMENT,
             "negative dmrg parameter");
  *psi = path_shaped(psi0->topo) ? dmrg_path(ctx, H, psi0, *params, energy)
                                 : dmrg_tree(ctx, H, psi0, *params, energy);
  TNFA_API_END
}

int tnfa_integrate_operator(tnfa_ctx* ctx, const tnfa_net* op, const tnfa_net* f, int take_sum,
                            double* out) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(op, "integrate operator");
  require_net(f, "integrate function");
  TNFA_CHECK(out, TNFA_ERR_INVALID_ARGUMENT, "null out");
  TNFA_CHECK(op->dtype == f->dtype, TNFA_ERR_DTYPE, "integrate(O, f): element types differ");
  tnfa_net* row = reduce_out_legs(ctx, op, take_sum);
  try {
    inner_product(ctx, row, f, false, out);
  } catch (...) {
    tnfa_net_destroy(row);
    throw;
  }
  tnfa_net_destroy(row);
  TNFA_API_END
}

}  // extern "C"
