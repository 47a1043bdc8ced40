// Integration of a tree tensor network function over [0,1)^n.
//
// Reference: integrate (src/integration.jl:6-17) multiplies every vertex by
// ITensor(c, site_inds...) with c = 1/base (1 with take_sum) and contracts the
// network with belief propagation.  Here: one HBM-streaming pass reduces the
// site axis of every tensor (the only pass that touches all tensor bytes),
// then the bond-only forest is contracted by the evaluation engine at a
// single point.
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
  tnfa_net* r = site_reduced_net(ctx, net, take_sum);
  try {
    contract_scalar(ctx, r, out);
  } catch (...) {
    tnfa_net_destroy(r);
    throw;
  }
  tnfa_net_destroy(r);
  TNFA_API_END
}
