// Integration of a tree tensor network function over [0,1)^n.
//
// Reference: integrate (src/integration.jl:6-17) multiplies every vertex by
// ITensor(c, site_inds...) with c = 1/base (1 with take_sum) and contracts the
// network with belief propagation.  Here (tnfa_integrate): the vertices by
// height, leaves first, one HBM-streaming launch per level over all SMs that
// reads each tensor once and contracts it at the same time with the site
// weights and the children's messages (k_integrate_level); messages are kept
// in FP64 (or complex FP64) with a power-of-two exponent per vertex.
// site_reduced_net (the site-reduced network as a network) serves the
// operator and partial integrals.
#include <cmath>

#include "evaluate.cuh"

namespace tnfa {

struct ReduceJob {
  int64_t soff, doff, slice;
  int sd;
  double w;
};

// dst_v[i] = w_v * sum_s src_v[s * slice + i] for every vertex v (blockIdx.y).
template <class T>
__global__ void k_site_reduce(const T* __restrict__ src, T* __restrict__ dst,
                              const ReduceJob* __restrict__ jobs) {
  const ReduceJob jb = jobs[blockIdx.y];
  const T* s = src + jb.soff;
  T* d = dst + jb.doff;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < jb.slice;
       i += (int64_t)gridDim.x * blockDim.x) {
    T acc = Sc<T>::zero();
    for (int q = 0; q < jb.sd; ++q) acc += s[(int64_t)q * jb.slice + i];
    d[i] = acc * (T)jb.w;
  }
}
template <>
__global__ void k_site_reduce<cplx>(const cplx* __restrict__ src, cplx* __restrict__ dst,
                                    const ReduceJob* __restrict__ jobs) {
  const ReduceJob jb = jobs[blockIdx.y];
  const cplx* s = src + jb.soff;
  cplx* d = dst + jb.doff;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < jb.slice;
       i += (int64_t)gridDim.x * blockDim.x) {
    cplx acc{0.0, 0.0};
    for (int q = 0; q < jb.sd; ++q) acc += s[(int64_t)q * jb.slice + i];
    d[i] = cplx{acc.re * jb.w, acc.im * jb.w};
  }
}

// ----------------------------------------------------- tnfa_integrate ----
template <class T> struct IntAcc { using type = double; };
template <> struct IntAcc<cplx> { using type = cplx; };
__device__ inline void atomicAddAcc(double* a, double v) { atomicAdd(a, v); }
__device__ inline void atomicAddAcc(cplx* a, cplx v) {
  atomicAdd(&a->re, v.re);
  atomicAdd(&a->im, v.im);
}
__device__ inline double mulw(double x, double w) { return x * w; }
__device__ inline cplx mulw(cplx x, double w) { return cplx{x.re * w, x.im * w}; }
__device__ inline double to_acc(float x, double) { return (double)x; }
__device__ inline double to_acc(double x, double) { return x; }
__device__ inline cplx to_acc(cplx x, cplx) { return x; }
__device__ inline float to_dot(double x, float) { return (float)x; }
__device__ inline double to_dot(double x, double) { return x; }
__device__ inline cplx to_dot(cplx x, cplx) { return x; }

struct IntVertex {
  int64_t off;       // tensor offset (elements)
  int sd, chi_a, nchild, last;  // last: entries of the last child (1 without children)
  int64_t rows;      // sd * chi_a * prod(children but the last)
  int ch[EVAL_MAXC], dim[EVAL_MAXC];
  int v;
  double w;          // site weight: prod of 1 / leg dim (1 with take_sum)
};

// Vertices are processed by height (leaves first); one level is two launches.
// k_integrate_norm: a CTA per vertex copies its children's messages,
// normalised by a power of two, to cm[v] in the tensor's own type (FP32
// networks stay on the FP32 pipe, GB300 runs FP64 at 1/64 of it) and sets the
// vertex exponent.
template <class T, class A>
__global__ void __launch_bounds__(256) k_integrate_norm(const IntVertex* __restrict__ lv,
                                                        const A* __restrict__ msgs, int* exps,
                                                        T* __restrict__ cm, int chimax) {
  const IntVertex iv = lv[blockIdx.x];
  __shared__ int cex[EVAL_MAXC];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  T* dst = cm + (int64_t)iv.v * EVAL_MAXC * chimax;
  for (int c = warp; c < iv.nchild; c += nw) {
    const A* src = msgs + (int64_t)iv.ch[c] * chimax;
    double mx = 0.0;
    for (int i = lane; i < iv.dim[c]; i += 32) mx = fmax(mx, Sc<A>::absmax(src[i]));
    for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    int ex = 0;
    if (mx > 0) frexp(mx, &ex);
    for (int i = lane; i < iv.dim[c]; i += 32) dst[c * chimax + i] = to_dot(Sc<A>::scale2(src[i], -ex), T{});
    if (lane == 0) cex[c] = ex + exps[iv.ch[c]];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int e = 0;
    for (int c = 0; c < iv.nchild; ++c) e += cex[c];
    exps[iv.v] = e;
  }
}

// k_integrate_level: out_v[a] += w_v * sum over rows (s, a, k) of
// prod_{c < last} m_c[k_c] * sum_j T_v[row][j] m_last[j] for every vertex of
// the level.  A warp task is a run of INT_KB consecutive rows of one vertex
// with the same (s, a) (contiguous bytes); tasks of all the level's vertices
// are numbered consecutively (task_start).  Each lane keeps one partial sum
// over its entries j = lane + 32 i; one warp reduction and one atomic per
// task.  Rows are read four at a time so that their loads overlap.
constexpr int INT_KB = 16;
template <class T>
__global__ void __launch_bounds__(256) k_integrate_level(const T* __restrict__ tensors,
                                                         const IntVertex* __restrict__ lv, int nv,
                                                         const int64_t* __restrict__ task_start,
                                                         typename IntAcc<T>::type* msgs,
                                                         const T* __restrict__ cm, int chimax) {
  using A = typename IntAcc<T>::type;
  using D = T;  // type of the row dots and the task's partial sum
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int64_t ntask = task_start[nv];
  int vi = 0;
  for (int64_t t = (int64_t)blockIdx.x * nw + warp; t < ntask; t += (int64_t)gridDim.x * nw) {
    while (vi + 1 < nv && task_start[vi + 1] <= t) ++vi;  // tasks ascend per warp
    while (vi > 0 && task_start[vi] > t) --vi;
    const IntVertex& iv = lv[vi];
    const D* cv = cm + (int64_t)iv.v * EVAL_MAXC * chimax;
    const int64_t Kouter = iv.rows / ((int64_t)iv.sd * iv.chi_a);
    const int64_t nkb = (Kouter + INT_KB - 1) / INT_KB;
    const int64_t tl = t - task_start[vi];
    const int64_t sa = tl / nkb;  // (s, a) block
    const int a = (int)(sa % iv.chi_a);
    const int64_t k0 = (tl - sa * nkb) * INT_KB;
    const int64_t k1 = min(Kouter, k0 + INT_KB);
    const int last = iv.last;
    // the task in the tensor's own type (FP32 rows stay on the FP32 pipe),
    // its sum added to the FP64 (or complex FP64) message once
    D mlr[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int j = lane + 32 * i;
      mlr[i] = iv.nchild == 0 ? (j == 0 ? Sc<D>::one() : Sc<D>::zero())
                              : (j < last ? cv[(iv.nchild - 1) * chimax + j] : Sc<D>::zero());
    }
    const T* base = tensors + iv.off + sa * Kouter * last;
    D partial = Sc<D>::zero();
    for (int64_t k = k0; k < k1; k += 4) {
      D dot[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) dot[u] = Sc<D>::zero();
      if (last <= 256) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if (k + u < k1) {
            const T* row = base + (k + u) * last;
#pragma unroll
            for (int i = 0; i < 8; ++i) {
              const int j = lane + 32 * i;
              if (j < last) dot[u] = Sc<D>::fma(row[j], mlr[i], dot[u]);
            }
          }
        }
      } else {
        for (int u = 0; u < 4 && k + u < k1; ++u) {
          const T* row = base + (k + u) * last;
          for (int j = lane; j < last; j += 32)
            dot[u] = Sc<D>::fma(row[j], cv[(iv.nchild - 1) * chimax + j], dot[u]);
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if (k + u >= k1) break;
        // weight: the entries of the children but the last at k + u (mixed
        // radix; with two children simply the first child's entry k + u)
        D wgt;
        if (iv.nchild <= 1) {
          wgt = Sc<D>::one();
        } else if (iv.nchild == 2) {
          wgt = cv[(int)(k + u)];
        } else {
          wgt = Sc<D>::one();
          int kk = (int)(k + u);
          for (int c = iv.nchild - 2; c >= 0; --c) {
            const int d = iv.dim[c];
            wgt = wgt * cv[c * chimax + kk % d];
            kk /= d;
          }
        }
        partial = Sc<D>::fma(wgt, dot[u], partial);
      }
    }
    for (int o = 16; o; o >>= 1) {
      if constexpr (sizeof(D) == 16) {
        cplx z = *(cplx*)&partial;
        z.re += __shfl_xor_sync(0xffffffffu, z.re, o);
        z.im += __shfl_xor_sync(0xffffffffu, z.im, o);
        partial = *(D*)&z;
      } else {
        partial = partial + __shfl_xor_sync(0xffffffffu, partial, o);
      }
    }
    if (lane == 0) atomicAddAcc(&msgs[(int64_t)iv.v * chimax + a], mulw(to_acc(partial, A{}), iv.w));
  }
}

// A network with the same bonds and no site legs: the site-reduced tensors.
tnfa_net* site_reduced_net(tnfa_ctx* ctx, const tnfa_net* net, int take_sum) {
  const Topo& T = net->topo;
  Topo R = T;
  R.nlegs.assign(T.V, 0);
  R.leg_dim.clear();
  R.leg_var.clear();
  R.leg_digit.clear();
  R.leg_kind.clear();
  R.finalize();
  tnfa_net* out = new_net(ctx, R, net->dtype);
  std::vector<ReduceJob> jobs(T.V);
  int64_t maxslice = 1;
  for (int v = 0; v < T.V; ++v) {
    double w = 1.0;
    if (!take_sum)
      for (int l = T.leg_off[v]; l < T.leg_off[v + 1]; ++l) w /= T.leg_dim[l];
    jobs[v] = {T.off[v], R.off[v], R.size(v), T.site_dim[v], w};
    maxslice = std::max<int64_t>(maxslice, R.size(v));
  }
  DBuf dj(ctx, jobs.size() * sizeof(ReduceJob));
  TNFA_CUDA(cudaMemcpyAsync(dj.p, jobs.data(), jobs.size() * sizeof(ReduceJob),
                            cudaMemcpyHostToDevice, ctx->stream));
  TNFA_CHECK(T.V <= 65535, TNFA_ERR_UNSUPPORTED, "more than 65535 vertices");
  dim3 grid(grid_for(maxslice, 256, std::max(1, 4 * ctx->sm_count)), T.V);
  KernelScope ks(ctx, "site_reduce", (double)T.n_elem,
                 (double)dtype_size(net->dtype) * (double)(T.n_elem + R.n_elem));
  if (net->dtype == TNFA_F64)
    k_site_reduce<double><<<grid, 256, 0, ctx->stream>>>((const double*)net->d, (double*)out->d,
                                                         dj.as<ReduceJob>());
  else if (net->dtype == TNFA_F32)
    k_site_reduce<float><<<grid, 256, 0, ctx->stream>>>((const float*)net->d, (float*)out->d,
                                                        dj.as<ReduceJob>());
  else
    k_site_reduce<cplx><<<grid, 256, 0, ctx->stream>>>((const cplx*)net->d, (cplx*)out->d,
                                                       dj.as<ReduceJob>());
  TNFA_LAUNCH_CHECK();
  return out;
}

template <class T>
void integrate_stream(tnfa_ctx* ctx, const tnfa_net* net, int take_sum, double* out) {
  using A = typename IntAcc<T>::type;
  const Topo& Tp = net->topo;
  const int V = Tp.V;
  int chimax = 1;
  for (int v = 0; v < V; ++v) chimax = std::max(chimax, Tp.link[v]);
  // heights: leaves 0, a vertex one more than its highest child
  std::vector<int> height(V, 0);
  int hmax = 0;
  for (int v = V - 1; v >= 0; --v) {  // children have larger indices than their parent
    for (int c : Tp.children[v]) height[v] = std::max(height[v], height[c] + 1);
    hmax = std::max(hmax, height[v]);
  }
  std::vector<std::vector<IntVertex>> levels(hmax + 1);
  for (int v = 0; v < V; ++v) {
    IntVertex iv{};
    iv.off = Tp.off[v];
    iv.sd = Tp.site_dim[v];
    iv.chi_a = Tp.link[v];
    iv.nchild = (int)Tp.children[v].size();
    TNFA_CHECK(iv.nchild <= EVAL_MAXC, TNFA_ERR_UNSUPPORTED, "vertex degree too high");
    int64_t kout = 1;
    for (int c = 0; c < iv.nchild; ++c) {
      iv.ch[c] = Tp.children[v][c];
      iv.dim[c] = Tp.link[iv.ch[c]];
      if (c + 1 < iv.nchild) kout *= iv.dim[c];
    }
    iv.last = iv.nchild ? iv.dim[iv.nchild - 1] : 1;
    iv.rows = (int64_t)iv.sd * iv.chi_a * kout;
    iv.v = v;
    iv.w = 1.0;
    if (!take_sum)
      for (int l = Tp.leg_off[v]; l < Tp.leg_off[v + 1]; ++l) iv.w /= Tp.leg_dim[l];
    levels[height[v]].push_back(iv);
  }
  // one upload: per level its vertices and task prefix sums
  std::vector<IntVertex> allv;
  std::vector<int64_t> allts;
  std::vector<size_t> vbase, tbase;
  for (const auto& lv : levels) {
    vbase.push_back(allv.size());
    tbase.push_back(allts.size());
    int64_t acc = 0;
    for (const auto& iv : lv) {
      allv.push_back(iv);
      allts.push_back(acc);
      const int64_t kout = iv.rows / ((int64_t)iv.sd * iv.chi_a);
      acc += (int64_t)iv.sd * iv.chi_a * ((kout + INT_KB - 1) / INT_KB);
    }
    allts.push_back(acc);
  }
  DBuf msgs(ctx, (size_t)V * chimax * sizeof(A)), exps(ctx, (size_t)V * sizeof(int));
  DBuf cm(ctx, (size_t)V * EVAL_MAXC * chimax * sizeof(T));
  DBuf dv(ctx, allv.size() * sizeof(IntVertex)), dt(ctx, allts.size() * sizeof(int64_t));
  TNFA_CUDA(cudaMemcpyAsync(dv.p, allv.data(), allv.size() * sizeof(IntVertex), cudaMemcpyHostToDevice,
                            ctx->stream));
  TNFA_CUDA(cudaMemcpyAsync(dt.p, allts.data(), allts.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                            ctx->stream));
  TNFA_CUDA(cudaMemsetAsync(msgs.p, 0, (size_t)V * chimax * sizeof(A), ctx->stream));
  TNFA_CUDA(cudaMemsetAsync(exps.p, 0, (size_t)V * sizeof(int), ctx->stream));
  KernelScope ks(ctx, "integrate", 2.0 * (double)Tp.n_elem, (double)dtype_size(net->dtype) * Tp.n_elem);
  for (size_t h = 0; h < levels.size(); ++h) {
    const int nv = (int)levels[h].size();
    if (nv == 0) continue;
    const IntVertex* lv = dv.as<IntVertex>() + vbase[h];
    const int64_t* ts = dt.as<int64_t>() + tbase[h];
    if (h > 0) {
      k_integrate_norm<T, A><<<nv, 256, 0, ctx->stream>>>(lv, msgs.as<A>(), exps.as<int>(), cm.as<T>(),
                                                          chimax);
      TNFA_LAUNCH_CHECK();
    }
    const int64_t ntask = allts[tbase[h] + nv];
    const unsigned grid = grid_for(ntask, 8, std::max(1, 8 * ctx->sm_count));
    k_integrate_level<T><<<grid, 256, 0, ctx->stream>>>((const T*)net->d, lv, nv, ts, msgs.as<A>(),
                                                        cm.as<T>(), chimax);
    TNFA_LAUNCH_CHECK();
  }
  const std::vector<int> roots = Tp.roots();
  std::vector<A> hm((size_t)V * chimax);
  std::vector<int> he(V);
  TNFA_CUDA(cudaMemcpyAsync(hm.data(), msgs.p, hm.size() * sizeof(A), cudaMemcpyDeviceToHost, ctx->stream));
  TNFA_CUDA(cudaMemcpyAsync(he.data(), exps.p, he.size() * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  // product over the roots of the forest, exponents applied at the end
  double re = 1.0, im = 0.0;
  int e = 0;
  for (int r : roots) {
    double vr, vi;
    if constexpr (sizeof(A) == 16) {
      const cplx z = *(const cplx*)&hm[(size_t)r * chimax];
      vr = z.re;
      vi = z.im;
    } else {
      vr = *(const double*)&hm[(size_t)r * chimax];
      vi = 0.0;
    }
    const double nr = re * vr - im * vi, ni = re * vi + im * vr;
    re = nr;
    im = ni;
    e += he[r];
  }
  out[0] = std::ldexp(re, e);
  if (net->dtype == TNFA_C128) out[1] = std::ldexp(im, e);
}

}  // namespace tnfa

using namespace tnfa;

extern "C" int tnfa_integrate(tnfa_ctx* ctx, const tnfa_net* net, int take_sum, double* out) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(net, "integrate");
  TNFA_CHECK(out, TNFA_ERR_INVALID_ARGUMENT, "null out");
  const Topo& T = net->topo;
  for (int l = 0; l < T.leg_off[T.V]; ++l)
    TNFA_CHECK(T.leg_kind[l] != TNFA_LEG_OPERATOR, TNFA_ERR_INVALID_ARGUMENT,
               "integrate needs a function network, got an operator");
  if (net->dtype == TNFA_F64)
    integrate_stream<double>(ctx, net, take_sum, out);
  else if (net->dtype == TNFA_F32)
    integrate_stream<float>(ctx, net, take_sum, out);
  else
    integrate_stream<cplx>(ctx, net, take_sum, out);
  TNFA_API_END
}
