// Network algebra on the device: direct sum (f + g), Hadamard product (f * g),
// diag(f) as an operator, forest union and element-type conversion.
#include <algorithm>
#include <type_traits>

#include "common.cuh"

namespace tnfa {

constexpr int ALG_MAXD = 12;  // tensor order handled by the index kernels

// Per-vertex block copy: dst[o + idx(src)] (+)= src, with src dims d[], dst
// dims D[] and per-axis offsets o[].
struct EmbedJob {
  int64_t soff, doff, n;
  int nd;
  int accumulate;
  int d[ALG_MAXD], D[ALG_MAXD], o[ALG_MAXD];
};

template <class T>
__global__ void k_embed(const T* __restrict__ src, T* __restrict__ dst,
                        const EmbedJob* __restrict__ jobs) {
  const EmbedJob& jb = jobs[blockIdx.y];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < jb.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i, di = 0, stride = 1;
    for (int a = jb.nd - 1; a >= 0; --a) {
      int64_t x = r % jb.d[a];
      r /= jb.d[a];
      di += (x + jb.o[a]) * stride;
      stride *= jb.D[a];
    }
    T v = src[jb.soff + i];
    if (jb.accumulate)
      dst[jb.doff + di] = dst[jb.doff + di] + v;
    else
      dst[jb.doff + di] = v;
  }
}

// out[(i_f, i_g) per axis] = f[i_f] * g[i_g]; axis 0 (site) is shared.
struct HadamardJob {
  int64_t foff, goff, ooff, n;
  int nd;
  int df[ALG_MAXD], dg[ALG_MAXD];
};

template <class T>
__global__ void k_hadamard(const T* __restrict__ f, const T* __restrict__ g, T* __restrict__ o,
                           const HadamardJob* __restrict__ jobs) {
  const HadamardJob& jb = jobs[blockIdx.y];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < jb.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i, fi = 0, gi = 0, fs = 1, gs = 1;
    for (int a = jb.nd - 1; a >= 1; --a) {
      int64_t dd = (int64_t)jb.df[a] * jb.dg[a];
      int64_t x = r % dd;
      r /= dd;
      fi += (x / jb.dg[a]) * fs;
      gi += (x % jb.dg[a]) * gs;
      fs *= jb.df[a];
      gs *= jb.dg[a];
    }
    fi += r * fs;  // shared site axis
    gi += r * gs;
    o[jb.ooff + i] = f[jb.foff + fi] * g[jb.goff + gi];
  }
}

// diag: O[(s_l * b_l + s_l) over legs][rest] = f[s][rest]; other entries 0.
struct ProjJob {
  int64_t foff, ooff, rest, n;
  int nlegs;
  int b[ALG_MAXD];
};

template <class T>
__global__ void k_proj(const T* __restrict__ f, T* __restrict__ o, const ProjJob* __restrict__ jobs) {
  const ProjJob& jb = jobs[blockIdx.y];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < jb.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t s = i / jb.rest, q = i % jb.rest;
    int64_t os = 0, ostride = 1;
    for (int l = jb.nlegs - 1; l >= 0; --l) {
      int64_t x = s % jb.b[l];
      s /= jb.b[l];
      os += (x * jb.b[l] + x) * ostride;
      ostride *= (int64_t)jb.b[l] * jb.b[l];
    }
    o[jb.ooff + os * jb.rest + q] = f[jb.foff + i];
  }
}

template <class S, class D>
__global__ void k_convert(const S* __restrict__ s, D* __restrict__ d, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if constexpr (std::is_same<D, cplx>::value)
      d[i] = cplx{(double)s[i], 0.0};
    else
      d[i] = (D)s[i];
  }
}

// Strided broadcast gather: dst[i] = src[sum_a x_a(i) * st[a]] over the
// output axes (x_a the coordinates of i); an output vertex without a source
// is all ones.
struct GatherJob {
  int64_t soff, doff, n;
  int nd;
  int has_src;
  int d[ALG_MAXD];
  int64_t st[ALG_MAXD];
};

template <class T>
__global__ void k_gather(const T* __restrict__ src, T* __restrict__ dst,
                         const GatherJob* __restrict__ jobs) {
  const GatherJob& jb = jobs[blockIdx.y];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < jb.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (!jb.has_src) {
      dst[jb.doff + i] = Sc<T>::one();
      continue;
    }
    int64_t r = i, si = 0;
    for (int a = jb.nd - 1; a >= 0; --a) {
      const int64_t x = r % jb.d[a];
      r /= jb.d[a];
      si += x * jb.st[a];
    }
    dst[jb.doff + i] = src[jb.soff + si];
  }
}

// Axis dims of v's tensor: [site, parent, children...].
static std::vector<int> axes(const Topo& T, int v) {
  std::vector<int> a{T.site_dim[v], T.link[v]};
  for (int c : T.children[v]) a.push_back(T.link[c]);
  return a;
}

static void same_shape(const Topo& A, const Topo& B, const char* what) {
  bool ok = A.V == B.V && A.parent == B.parent && A.nlegs == B.nlegs && A.leg_dim == B.leg_dim;
  TNFA_CHECK(ok, TNFA_ERR_SHAPE, std::string(what) + ": networks have different trees or site legs");
}

template <class Job>
static DBuf upload_jobs(tnfa_ctx* ctx, const std::vector<Job>& jobs) {
  DBuf d(ctx, jobs.size() * sizeof(Job));
  h2d(ctx, d.p, jobs.data(), jobs.size() * sizeof(Job));
  return d;
}

#define TNFA_DISPATCH(dtype, T, ...)            \
  do {                                          \
    if ((dtype) == TNFA_F64) {                  \
      using T = double;                         \
      __VA_ARGS__;                              \
    } else if ((dtype) == TNFA_F32) {           \
      using T = float;                          \
      __VA_ARGS__;                              \
    } else {                                    \
      using T = cplx;                           \
      __VA_ARGS__;                              \
    }                                           \
  } while (0)

tnfa_net* direct_sum(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_net* g) {
  const Topo& A = f->topo;
  const Topo& B = g->topo;
  same_shape(A, B, "add");
  TNFA_CHECK(f->dtype == g->dtype, TNFA_ERR_DTYPE, "add: element types differ");
  TNFA_CHECK(A.roots().size() == 1, TNFA_ERR_UNSUPPORTED, "add of a forest (several roots)");
  Topo O = A;
  for (int v = 0; v < A.V; ++v)
    if (A.parent[v] >= 0) O.link[v] = A.link[v] + B.link[v];
  O.finalize();
  tnfa_net* out = new_net(ctx, O, f->dtype);
  size_t es = dtype_size(f->dtype);
  TNFA_CUDA(cudaMemsetAsync(out->d, 0, (size_t)O.n_elem * es, ctx->stream));
  std::vector<EmbedJob> jf, jg;
  int64_t nmax = 1;
  for (int v = 0; v < A.V; ++v) {
    std::vector<int> da = axes(A, v), db = axes(B, v), dd = axes(O, v);
    TNFA_CHECK((int)da.size() <= ALG_MAXD, TNFA_ERR_UNSUPPORTED, "vertex degree too high");
    bool isolated = (A.parent[v] < 0 && A.children[v].empty());
    EmbedJob a{}, b{};
    a.soff = A.off[v];
    b.soff = B.off[v];
    a.doff = b.doff = O.off[v];
    a.n = A.size(v);
    b.n = B.size(v);
    a.nd = b.nd = (int)da.size();
    a.accumulate = 0;
    b.accumulate = isolated ? 1 : 0;
    for (int i = 0; i < a.nd; ++i) {
      a.d[i] = da[i];
      b.d[i] = db[i];
      a.D[i] = b.D[i] = dd[i];
      a.o[i] = 0;
      // g's block starts after f's on every bond axis (axis 0 is the site;
      // the parent axis of a root has dimension 1 in all three tensors).
      b.o[i] = (i == 0 || (i == 1 && A.parent[v] < 0) || isolated) ? 0 : da[i];
    }
    jf.push_back(a);
    jg.push_back(b);
    nmax = std::max(nmax, std::max(a.n, b.n));
  }
  DBuf df = upload_jobs(ctx, jf), dg = upload_jobs(ctx, jg);
  dim3 grid(grid_for(nmax, 256, 1024), A.V);
  TNFA_DISPATCH(f->dtype, T, {
    k_embed<T><<<grid, 256, 0, ctx->stream>>>((const T*)f->d, (T*)out->d, df.as<EmbedJob>());
    k_embed<T><<<grid, 256, 0, ctx->stream>>>((const T*)g->d, (T*)out->d, dg.as<EmbedJob>());
  });
  TNFA_LAUNCH_CHECK();
  return out;
}

tnfa_net* hadamard(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_net* g) {
  const Topo& A = f->topo;
  const Topo& B = g->topo;
  same_shape(A, B, "multiply");
  TNFA_CHECK(f->dtype == g->dtype, TNFA_ERR_DTYPE, "multiply: element types differ");
  Topo O = A;
  for (int v = 0; v < A.V; ++v) O.link[v] = A.link[v] * B.link[v];
  O.finalize();
  tnfa_net* out = new_net(ctx, O, f->dtype);
  std::vector<HadamardJob> jobs;
  int64_t nmax = 1;
  for (int v = 0; v < A.V; ++v) {
    std::vector<int> da = axes(A, v), db = axes(B, v);
    TNFA_CHECK((int)da.size() <= ALG_MAXD, TNFA_ERR_UNSUPPORTED, "vertex degree too high");
    HadamardJob h{};
    h.foff = A.off[v];
    h.goff = B.off[v];
    h.ooff = O.off[v];
    h.n = O.size(v);
    h.nd = (int)da.size();
    for (int i = 0; i < h.nd; ++i) {
      h.df[i] = da[i];
      h.dg[i] = db[i];
    }
    jobs.push_back(h);
    nmax = std::max(nmax, h.n);
  }
  DBuf dj = upload_jobs(ctx, jobs);
  dim3 grid(grid_for(nmax, 256, 1024), A.V);
  TNFA_DISPATCH(f->dtype, T, {
    k_hadamard<T><<<grid, 256, 0, ctx->stream>>>((const T*)f->d, (const T*)g->d, (T*)out->d,
                                                 dj.as<HadamardJob>());
  });
  TNFA_LAUNCH_CHECK();
  return out;
}

tnfa_net* operator_proj(tnfa_ctx* ctx, const tnfa_net* f) {
  const Topo& A = f->topo;
  Topo O = A;
  for (int l = 0; l < A.leg_off[A.V]; ++l) {
    TNFA_CHECK(A.leg_kind[l] != TNFA_LEG_OPERATOR, TNFA_ERR_INVALID_ARGUMENT,
               "operator_proj needs a function network");
    O.leg_dim[l] = A.leg_dim[l] * A.leg_dim[l];
    O.leg_kind[l] = TNFA_LEG_OPERATOR;
  }
  O.finalize();
  tnfa_net* out = new_net(ctx, O, f->dtype);
  TNFA_CUDA(cudaMemsetAsync(out->d, 0, (size_t)O.n_elem * dtype_size(f->dtype), ctx->stream));
  std::vector<ProjJob> jobs;
  int64_t nmax = 1;
  for (int v = 0; v < A.V; ++v) {
    TNFA_CHECK(A.nlegs[v] <= ALG_MAXD, TNFA_ERR_UNSUPPORTED, "too many legs");
    ProjJob p{};
    p.foff = A.off[v];
    p.ooff = O.off[v];
    p.n = A.size(v);
    p.rest = A.size(v) / A.site_dim[v];
    p.nlegs = A.nlegs[v];
    for (int l = 0; l < p.nlegs; ++l) p.b[l] = A.leg_dim[A.leg_off[v] + l];
    jobs.push_back(p);
    nmax = std::max(nmax, p.n);
  }
  DBuf dj = upload_jobs(ctx, jobs);
  dim3 grid(grid_for(nmax, 256, 1024), A.V);
  TNFA_DISPATCH(f->dtype, T, {
    k_proj<T><<<grid, 256, 0, ctx->stream>>>((const T*)f->d, (T*)out->d, dj.as<ProjJob>());
  });
  TNFA_LAUNCH_CHECK();
  return out;
}

tnfa_net* concat(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_net* g) {
  TNFA_CHECK(f->dtype == g->dtype, TNFA_ERR_DTYPE, "concat: element types differ");
  const Topo& A = f->topo;
  const Topo& B = g->topo;
  Topo O;
  O.V = A.V + B.V;
  O.parent = A.parent;
  for (int v = 0; v < B.V; ++v) O.parent.push_back(B.parent[v] < 0 ? -1 : B.parent[v] + A.V);
  O.link = A.link;
  O.link.insert(O.link.end(), B.link.begin(), B.link.end());
  O.nlegs = A.nlegs;
  O.nlegs.insert(O.nlegs.end(), B.nlegs.begin(), B.nlegs.end());
  auto cat = [](std::vector<int> a, const std::vector<int>& b) {
    a.insert(a.end(), b.begin(), b.end());
    return a;
  };
  O.leg_dim = cat(A.leg_dim, B.leg_dim);
  O.leg_var = cat(A.leg_var, B.leg_var);
  O.leg_digit = cat(A.leg_digit, B.leg_digit);
  O.leg_kind = cat(A.leg_kind, B.leg_kind);
  O.finalize();
  tnfa_net* out = new_net(ctx, O, f->dtype);
  size_t es = dtype_size(f->dtype);
  TNFA_CUDA(cudaMemcpyAsync(out->d, f->d, (size_t)A.n_elem * es, cudaMemcpyDeviceToDevice,
                            ctx->stream));
  TNFA_CUDA(cudaMemcpyAsync((char*)out->d + (size_t)A.n_elem * es, g->d, (size_t)B.n_elem * es,
                            cudaMemcpyDeviceToDevice, ctx->stream));
  return out;
}

tnfa_net* convert(tnfa_ctx* ctx, const tnfa_net* f, int dtype) {
  TNFA_CHECK(dtype == TNFA_F64 || dtype == TNFA_F32 || dtype == TNFA_C128, TNFA_ERR_DTYPE,
             "bad dtype");
  TNFA_CHECK(!(f->dtype == TNFA_C128 && dtype != TNFA_C128), TNFA_ERR_DTYPE,
             "complex networks cannot be converted to a real type");
  tnfa_net* out = new_net(ctx, f->topo, dtype);
  int64_t n = f->topo.n_elem;
  unsigned g = grid_for(n, 256, 4096);
  if (f->dtype == dtype) {
    TNFA_CUDA(cudaMemcpyAsync(out->d, f->d, (size_t)n * dtype_size(dtype), cudaMemcpyDeviceToDevice,
                              ctx->stream));
  } else if (f->dtype == TNFA_F64 && dtype == TNFA_F32) {
    k_convert<double, float><<<g, 256, 0, ctx->stream>>>((const double*)f->d, (float*)out->d, n);
  } else if (f->dtype == TNFA_F32 && dtype == TNFA_F64) {
    k_convert<float, double><<<g, 256, 0, ctx->stream>>>((const float*)f->d, (double*)out->d, n);
  } else if (f->dtype == TNFA_F64 && dtype == TNFA_C128) {
    k_convert<double, cplx><<<g, 256, 0, ctx->stream>>>((const double*)f->d, (cplx*)out->d, n);
  } else {
    k_convert<float, cplx><<<g, 256, 0, ctx->stream>>>((const float*)f->d, (cplx*)out->d, n);
  }
  TNFA_LAUNCH_CHECK();
  return out;
}

Topo topo_from_abi(const tnfa_topology* t);  // core.cu

tnfa_net* gather(tnfa_ctx* ctx, const tnfa_net* f, const Topo& O, const int32_t* src_vertex,
                 const int64_t* strides) {
  const Topo& S = f->topo;
  TNFA_CHECK(src_vertex && strides, TNFA_ERR_INVALID_ARGUMENT, "gather: null arrays");
  tnfa_net* out = new_net(ctx, O, f->dtype);
  std::vector<GatherJob> jobs;
  int64_t nmax = 1, k = 0;
  try {
    for (int t = 0; t < O.V; ++t) {
      GatherJob j{};
      j.doff = O.off[t];
      j.n = O.size(t);
      const int sv = src_vertex[t];
      TNFA_CHECK(sv >= -1 && sv < S.V, TNFA_ERR_INVALID_ARGUMENT, "gather: source vertex out of range");
      j.has_src = sv >= 0;
      j.soff = sv >= 0 ? S.off[sv] : 0;
      std::vector<int> d;
      for (int l = O.leg_off[t]; l < O.leg_off[t + 1]; ++l) d.push_back(O.leg_dim[l]);
      d.push_back(O.link[t]);
      for (int c : O.children[t]) d.push_back(O.link[c]);
      TNFA_CHECK((int)d.size() <= ALG_MAXD, TNFA_ERR_UNSUPPORTED, "gather: vertex order above 12");
      j.nd = (int)d.size();
      int64_t reach = 0;
      for (int a = 0; a < j.nd; ++a) {
        j.d[a] = d[a];
        j.st[a] = strides[k++];
        TNFA_CHECK(j.st[a] >= 0, TNFA_ERR_INVALID_ARGUMENT, "gather: negative stride");
        reach += (int64_t)(d[a] - 1) * j.st[a];
      }
      // every read stays inside the source vertex's tensor
      TNFA_CHECK(sv < 0 || reach < S.size(sv), TNFA_ERR_INVALID_ARGUMENT,
                 "gather: strides of vertex " + std::to_string(t) + " reach past its source tensor");
      jobs.push_back(j);
      nmax = std::max(nmax, j.n);
    }
    DBuf dj = upload_jobs(ctx, jobs);
    dim3 grid(grid_for(nmax, 256, 1024), O.V);
    TNFA_CHECK(O.V <= 65535, TNFA_ERR_UNSUPPORTED, "more than 65535 vertices");
    TNFA_DISPATCH(f->dtype, T, {
      k_gather<T><<<grid, 256, 0, ctx->stream>>>((const T*)f->d, (T*)out->d, dj.as<GatherJob>());
    });
    TNFA_LAUNCH_CHECK();
  } catch (...) {
    tnfa_net_destroy(out);
    throw;
  }
  return out;
}

}  // namespace tnfa

using namespace tnfa;

extern "C" {

int tnfa_add(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_net* g, tnfa_net** out) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(f, "add f");
  require_net(g, "add g");
  TNFA_CHECK(out, TNFA_ERR_INVALID_ARGUMENT, "null out");
  *out = direct_sum(ctx, f, g);
  TNFA_API_END
}

int tnfa_multiply(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_net* g, tnfa_net** out) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(f, "multiply f");
  require_net(g, "multiply g");
  TNFA_CHECK(out, TNFA_ERR_INVALID_ARGUMENT, "null out");
  *out = hadamard(ctx, f, g);
  TNFA_API_END
}

int tnfa_operator_proj(tnfa_ctx* ctx, const tnfa_net* f, tnfa_net** out) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(f, "operator_proj");
  TNFA_CHECK(out, TNFA_ERR_INVALID_ARGUMENT, "null out");
  *out = operator_proj(ctx, f);
  TNFA_API_END
}

int tnfa_net_concat(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_net* g, tnfa_net** out) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(f, "concat f");
  require_net(g, "concat g");
  TNFA_CHECK(out, TNFA_ERR_INVALID_ARGUMENT, "null out");
  *out = concat(ctx, f, g);
  TNFA_API_END
}

int tnfa_net_gather(tnfa_ctx* ctx, const tnfa_net* f, const tnfa_topology* target,
                    const int32_t* src_vertex, const int64_t* strides, tnfa_net** out) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(f, "gather");
  TNFA_CHECK(out, TNFA_ERR_INVALID_ARGUMENT, "null out");
  Topo O = topo_from_abi(target);
  *out = gather(ctx, f, O, src_vertex, strides);
  TNFA_API_END
}

int tnfa_net_convert(tnfa_ctx* ctx, const tnfa_net* f, int dtype, tnfa_net** out) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(f, "convert");
  TNFA_CHECK(out, TNFA_ERR_INVALID_ARGUMENT, "null out");
  *out = convert(ctx, f, dtype);
  TNFA_API_END
}

}  // extern "C"
