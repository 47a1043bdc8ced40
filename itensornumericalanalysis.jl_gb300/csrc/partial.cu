// Partial integration of a tree tensor network function.
//
// Reference: partial_integrate (src/integration.jl:35-54) multiplies every
// site index of the integrated variables by the constant vector c = 1/base
// (1 with take_sum) and then calls merge_internal_tensors
// (src/utils.jl:99-113), which contracts every tensor left without site
// indices into its first neighbour, or, when it has no neighbour left,
// multiplies its scalar into the first vertex that still has site indices.
//
// Here: one pass reduces the integrated legs of every vertex (a strided sum
// over the dropped digits), the merges run as permute + GEMM on the device,
// and the survivors are written out in canonical layout, numbered breadth
// first with vertices ordered by a caller-given rank (the vertex order of the
// caller's graph), so the caller's layout rule reproduces the numbering.
#include <algorithm>
#include <numeric>

#include "common.cuh"
#include "linalg.cuh"

namespace tnfa {
namespace {

constexpr int PI_MAXLEGS = 8;

struct PReduceJob {
  const void* src;
  void* dst;
  int64_t slice, n;  // n = kept site dim * slice
  int nlegs;
  int dim[PI_MAXLEGS];
  int keep[PI_MAXLEGS];
  double w;
};

__device__ inline double mul_real(double x, double w) { return x * w; }
__device__ inline float mul_real(float x, double w) { return (float)(x * w); }
__device__ inline cplx mul_real(cplx x, double w) { return {x.re * w, x.im * w}; }

template <class T>
__global__ void k_partial_reduce(const PReduceJob* __restrict__ jobs) {
  const PReduceJob jb = jobs[blockIdx.y];
  const T* src = (const T*)jb.src;
  T* dst = (T*)jb.dst;
  int64_t ndrop = 1;
  for (int l = 0; l < jb.nlegs; ++l)
    if (!jb.keep[l]) ndrop *= jb.dim[l];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < jb.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = i % jb.slice;
    int64_t rem = i / jb.slice;
    int dig[PI_MAXLEGS];
    for (int l = jb.nlegs - 1; l >= 0; --l)
      if (jb.keep[l]) {
        dig[l] = (int)(rem % jb.dim[l]);
        rem /= jb.dim[l];
      }
    T acc = Sc<T>::zero();
    for (int64_t c = 0; c < ndrop; ++c) {
      int64_t r2 = c;
      for (int l = jb.nlegs - 1; l >= 0; --l)
        if (!jb.keep[l]) {
          dig[l] = (int)(r2 % jb.dim[l]);
          r2 /= jb.dim[l];
        }
      int64_t s = 0;
      for (int l = 0; l < jb.nlegs; ++l) s = s * jb.dim[l] + dig[l];
      acc += src[s * jb.slice + q];
    }
    dst[i] = mul_real(acc, jb.w);
  }
}

// x[0..n) *= *s (a scalar held on the device).
template <class T>
__global__ void k_scale_by_scalar(T* __restrict__ x, int64_t n, const T* __restrict__ s) {
  const T f = *s;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = x[i] * f;
}

// A tensor of the network being merged: [site][bond axes...], each bond axis
// labelled with the (input) vertex across it.
struct Node {
  bool alive = true;
  DBuf t;
  int site = 1;
  std::vector<int> legs;  // input leg ids still attached
  std::vector<int> nb, dim;
  int64_t size() const {
    int64_t s = site;
    for (int d : dim) s *= d;
    return s;
  }
};

template <class T>
void permute_to(tnfa_ctx* ctx, const void* src, void* dst, const std::vector<int>& shp,
                const std::vector<int>& order) {
  la::PermJob j{};
  j.src = src;
  j.dst = dst;
  j.nd = (int)shp.size();
  TNFA_CHECK(j.nd <= la::MAXD, TNFA_ERR_UNSUPPORTED, "partial_integrate: tensor order above 10");
  j.n = 1;
  for (int a = 0; a < j.nd; ++a) {
    j.shape[a] = shp[a];
    j.perm[a] = order[a];
    j.n *= shp[a];
  }
  la::permute<T>(ctx, {j});
}

template <class T>
tnfa_net* partial_integrate_impl(tnfa_ctx* ctx, const tnfa_net* net, const std::vector<int>& vars,
                                 bool take_sum, bool merge, const std::vector<int>& rank,
                                 std::vector<int>& out_vertex_of) {
  const Topo& I = net->topo;
  const int V = I.V;
  std::vector<Node> nodes(V);
  // (1) reduce the integrated legs
  std::vector<PReduceJob> jobs;
  int64_t nmax = 1;
  for (int v = 0; v < V; ++v) {
    Node& nd = nodes[v];
    const int nl = I.nlegs[v];
    TNFA_CHECK(nl <= PI_MAXLEGS, TNFA_ERR_UNSUPPORTED, "partial_integrate: more than 8 legs on a vertex");
    PReduceJob j{};
    j.src = (const T*)net->d + I.off[v];
    j.nlegs = nl;
    j.w = 1.0;
    for (int k = 0; k < nl; ++k) {
      const int l = I.leg_off[v] + k;
      j.dim[k] = I.leg_dim[l];
      const bool drop = std::find(vars.begin(), vars.end(), I.leg_var[l]) != vars.end();
      j.keep[k] = !drop;
      if (drop) {
        if (!take_sum) j.w /= I.leg_dim[l];
      } else {
        nd.site *= I.leg_dim[l];
        nd.legs.push_back(l);
      }
    }
    if (I.parent[v] >= 0) {
      nd.nb.push_back(I.parent[v]);
      nd.dim.push_back(I.link[v]);
    }
    for (int c : I.children[v]) {
      nd.nb.push_back(c);
      nd.dim.push_back(I.link[c]);
    }
    j.slice = I.size(v) / I.site_dim[v];
    j.n = nd.site * j.slice;
    nd.t = DBuf(ctx, (size_t)j.n * sizeof(T));
    j.dst = nd.t.p;
    jobs.push_back(j);
    nmax = std::max(nmax, j.n);
  }
  {
    DBuf dj(ctx, jobs.size() * sizeof(PReduceJob));
    TNFA_CUDA(cudaMemcpyAsync(dj.p, jobs.data(), jobs.size() * sizeof(PReduceJob),
                              cudaMemcpyHostToDevice, ctx->stream));
    TNFA_CHECK(V <= 65535, TNFA_ERR_UNSUPPORTED, "more than 65535 vertices");
    KernelScope ks(ctx, "partial_reduce", (double)I.n_elem, (double)sizeof(T) * (double)I.n_elem);
    dim3 grid(grid_for(nmax, 256, 1024), V);
    k_partial_reduce<T><<<grid, 256, 0, ctx->stream>>>(dj.as<PReduceJob>());
    TNFA_LAUNCH_CHECK();
  }
  // (2) merge the vertices left without legs, in rank order
  std::vector<int> by_rank(V);
  std::iota(by_rank.begin(), by_rank.end(), 0);
  std::stable_sort(by_rank.begin(), by_rank.end(), [&](int a, int b) { return rank[a] < rank[b]; });
  auto first_by_rank = [&](const std::vector<int>& vs) {
    int best = -1;
    for (int u : vs)
      if (best < 0 || rank[u] < rank[best]) best = u;
    return best;
  };
  for (int v : by_rank) {
    Node& nv = nodes[v];
    if (!merge || !nv.alive || !nv.legs.empty()) continue;
    if (nv.nb.empty()) {
      // a scalar: multiply it into the first vertex that still has legs
      int e = -1;
      for (int u : by_rank)
        if (u != v && nodes[u].alive && !nodes[u].legs.empty()) {
          e = u;
          break;
        }
      TNFA_CHECK(e >= 0, TNFA_ERR_INVALID_ARGUMENT,
                 "partial_integrate over every variable leaves a scalar: use integrate");
      Node& ne = nodes[e];
      k_scale_by_scalar<T><<<grid_for(ne.size(), 256, 1024), 256, 0, ctx->stream>>>(
          ne.t.template as<T>(), ne.size(), nv.t.template as<T>());
      TNFA_LAUNCH_CHECK();
      nv.alive = false;
      nv.t.reset();
      continue;
    }
    const int u = first_by_rank(nv.nb);
    Node& nu = nodes[u];
    const int a = (int)(std::find(nu.nb.begin(), nu.nb.end(), v) - nu.nb.begin());
    const int b = (int)(std::find(nv.nb.begin(), nv.nb.end(), u) - nv.nb.begin());
    const int d = nu.dim[a];
    // u -> [site_u, others_u..., bond], v -> [bond, others_v...]
    std::vector<int> ushp{nu.site}, uord{0};
    for (size_t k = 0; k < nu.dim.size(); ++k) ushp.push_back(nu.dim[k]);
    for (int k = 0; k < (int)nu.dim.size(); ++k)
      if (k != a) uord.push_back(1 + k);
    uord.push_back(1 + a);
    std::vector<int> vshp(nv.dim), vord{b};
    for (int k = 0; k < (int)nv.dim.size(); ++k)
      if (k != b) vord.push_back(k);
    const int64_t rows = nu.size() / d, cols = nv.size() / d;
    DBuf pu(ctx, (size_t)nu.size() * sizeof(T)), pv(ctx, (size_t)nv.size() * sizeof(T));
    permute_to<T>(ctx, nu.t.p, pu.p, ushp, uord);
    permute_to<T>(ctx, nv.t.p, pv.p, vshp, vord);
    TNFA_CHECK(rows < (int64_t(1) << 31) && cols < (int64_t(1) << 31), TNFA_ERR_UNSUPPORTED,
               "partial_integrate: merged tensor too large");
    DBuf merged(ctx, (size_t)(rows * cols) * sizeof(T));
    la::gemm<T>(ctx, {la::GemmJob{pu.p, pv.p, merged.p, (int)rows, (int)cols, d, d, (int)cols,
                                  (int)cols, 0, 0, 1.0, 0.0}});
    std::vector<int> nnb, ndim;
    for (int k = 0; k < (int)nu.nb.size(); ++k)
      if (k != a) nnb.push_back(nu.nb[k]), ndim.push_back(nu.dim[k]);
    for (int k = 0; k < (int)nv.nb.size(); ++k)
      if (k != b) {
        const int w = nv.nb[k];
        nnb.push_back(w);
        ndim.push_back(nv.dim[k]);
        for (int& x : nodes[w].nb)
          if (x == v) x = u;
      }
    nu.nb = nnb;
    nu.dim = ndim;
    nu.t = std::move(merged);
    nv.alive = false;
    nv.t.reset();
  }
  // (3) survivors, breadth first in rank order
  std::vector<int> pos(V, -1);
  std::vector<int> order, parent;
  for (int r : by_rank) {
    if (!nodes[r].alive || pos[r] >= 0) continue;
    pos[r] = (int)order.size();
    order.push_back(r);
    parent.push_back(-1);
    for (size_t h = pos[r]; h < order.size(); ++h) {
      std::vector<int> nbs = nodes[order[h]].nb;
      std::stable_sort(nbs.begin(), nbs.end(), [&](int x, int y) { return rank[x] < rank[y]; });
      for (int w : nbs)
        if (pos[w] < 0) {
          pos[w] = (int)order.size();
          order.push_back(w);
          parent.push_back((int)h);
        }
    }
  }
  const int W = (int)order.size();
  Topo O;
  O.V = W;
  O.parent = parent;
  O.link.assign(W, 1);
  O.nlegs.assign(W, 0);
  for (int k = 0; k < W; ++k) {
    const Node& n = nodes[order[k]];
    if (parent[k] >= 0) {
      const int p = order[parent[k]];
      O.link[k] = n.dim[std::find(n.nb.begin(), n.nb.end(), p) - n.nb.begin()];
    }
    O.nlegs[k] = (int)n.legs.size();
    for (int l : n.legs) {
      O.leg_dim.push_back(I.leg_dim[l]);
      O.leg_var.push_back(I.leg_var[l]);
      O.leg_digit.push_back(I.leg_digit[l]);
      O.leg_kind.push_back(I.leg_kind[l]);
    }
  }
  O.finalize();
  tnfa_net* out = new_net(ctx, O, net->dtype);
  try {
    for (int k = 0; k < W; ++k) {
      const Node& n = nodes[order[k]];
      std::vector<int> shp{n.site}, ord{0};
      for (int x : n.dim) shp.push_back(x);
      std::vector<int> want;
      if (parent[k] >= 0) want.push_back(order[parent[k]]);
      for (int c : O.children[k]) want.push_back(order[c]);
      for (int w : want) ord.push_back(1 + (int)(std::find(n.nb.begin(), n.nb.end(), w) - n.nb.begin()));
      TNFA_CHECK(ord.size() == shp.size(), TNFA_ERR_UNSUPPORTED, "partial_integrate: merge bookkeeping");
      permute_to<T>(ctx, n.t.p, (T*)out->d + O.off[k], shp, ord);
    }
  } catch (...) {
    tnfa_net_destroy(out);
    throw;
  }
  out_vertex_of = order;
  return out;
}

}  // namespace
}  // namespace tnfa

using namespace tnfa;

extern "C" {

int tnfa_partial_integrate(tnfa_ctx* ctx, const tnfa_net* net, int32_t n_vars, const int32_t* vars,
                           int take_sum, int merge_vertices, const int32_t* vertex_rank,
                           tnfa_net** out, int32_t* out_vertex_of) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(net, "partial_integrate");
  TNFA_CHECK(out && (n_vars == 0 || vars), TNFA_ERR_INVALID_ARGUMENT, "null argument");
  std::vector<int> vs(vars, vars + n_vars);
  std::vector<int> rank(net->topo.V);
  for (int v = 0; v < net->topo.V; ++v) rank[v] = vertex_rank ? vertex_rank[v] : v;
  std::vector<int> ov;
  if (net->dtype == TNFA_F64)
    *out = partial_integrate_impl<double>(ctx, net, vs, take_sum != 0, merge_vertices != 0, rank, ov);
  else if (net->dtype == TNFA_C128)
    *out = partial_integrate_impl<cplx>(ctx, net, vs, take_sum != 0, merge_vertices != 0, rank, ov);
  else
    fail(TNFA_ERR_DTYPE, "partial_integrate: FP64 or complex128 networks");
  if (out_vertex_of)
    for (size_t k = 0; k < ov.size(); ++k) out_vertex_of[k] = ov[k];
  TNFA_API_END
}

}  // extern "C"
