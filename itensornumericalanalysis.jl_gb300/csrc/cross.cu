// Cross approximation (adaptive cross with full pivoting) of a sampled block,
// the factorisation step of tensor cross interpolation.
//
// Reference: the TCI extension (ext/ITensorNumericalAnalysisTCIExt/
// tci_util.jl:21-55) hands the interpolation to ITensorTCI, whose two-site
// update factorises each sampled bond matrix by cross; this is that step.
// One CTA holds the residual R (in shared memory when it fits, else in a
// global-memory copy) and repeats: the entry of largest magnitude (the
// smallest flat index among equal ones) becomes the pivot (i, j) unless it is
// at most tol * max|M|, then R <- R - R[:, j] R[i, :] / R[i, j].  The update
// is computed as R - (c * r) / p in FP64, the same operations in the same
// order as a straightforward host implementation, so pivots agree exactly.
#include <cfloat>

#include "common.cuh"

namespace tnfa {
namespace {

constexpr int CROSS_THREADS = 1024;
constexpr int64_t CROSS_SMEM_ELEMS = 24 * 1024;  // 192 KB of FP64 residual

__device__ inline void arg_better(double v, int64_t k, double& bv, int64_t& bk) {
  if (v > bv || (v == bv && k < bk)) {
    bv = v;
    bk = k;
  }
}

__global__ void __launch_bounds__(CROSS_THREADS) k_cross_full(const double* __restrict__ M, double* Rg,
                                                             int rows, int cols, double tol, int maxrank,
                                                             int* __restrict__ out, double* __restrict__ outd,
                                                             int in_smem) {
  extern __shared__ double cross_smem[];
  __shared__ double wv[32];
  __shared__ long long wk[32];
  __shared__ double s_scale, s_piv;
  __shared__ int s_i, s_j, s_stop;
  const int64_t n = (int64_t)rows * cols;
  double* R = in_smem ? cross_smem : Rg;
  double* colbuf = in_smem ? cross_smem + n : Rg + n;  // rows entries
  double* rowbuf = colbuf + rows;                      // cols entries
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t k = threadIdx.x; k < n; k += blockDim.x) R[k] = M[k];
  __syncthreads();
  auto argmax = [&](double& bv, int64_t& bk) {
    bv = -1.0;
    bk = INT64_MAX;
    for (int64_t k = threadIdx.x; k < n; k += blockDim.x) arg_better(fabs(R[k]), k, bv, bk);
    for (int o = 16; o; o >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const long long ok = __shfl_xor_sync(0xffffffffu, (long long)bk, o);
      arg_better(ov, ok, bv, bk);
    }
    if (lane == 0) {
      wv[warp] = bv;
      wk[warp] = bk;
    }
    __syncthreads();
    if (warp == 0) {
      bv = lane < nw ? wv[lane] : -1.0;
      bk = lane < nw ? wk[lane] : INT64_MAX;
      for (int o = 16; o; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const long long ok = __shfl_xor_sync(0xffffffffu, (long long)bk, o);
        arg_better(ov, ok, bv, bk);
      }
      if (lane == 0) {
        wv[0] = bv;
        wk[0] = bk;
      }
    }
    __syncthreads();
    bv = wv[0];
    bk = wk[0];
    __syncthreads();
  };
  double bv;
  int64_t bk;
  argmax(bv, bk);
  if (threadIdx.x == 0) s_scale = bv;
  __syncthreads();
  const double scale = s_scale;
  const int kmax = min(maxrank, min(rows, cols));
  int r = 0;
  double err = scale;
  while (r < kmax) {
    if (r > 0) argmax(bv, bk);
    if (threadIdx.x == 0) {
      s_i = (int)(bk / cols);
      s_j = (int)(bk % cols);
      s_piv = R[bk];
      s_stop = (scale == 0.0 || fabs(R[bk]) <= tol * scale) ? 1 : 0;
    }
    __syncthreads();
    err = fabs(s_piv);
    if (s_stop) break;
    const int pi = s_i, pj = s_j;
    const double piv = s_piv;
    if (threadIdx.x == 0) {
      out[1 + r] = pi;
      out[1 + kmax + r] = pj;
    }
    for (int a = threadIdx.x; a < rows; a += blockDim.x) colbuf[a] = R[(int64_t)a * cols + pj];
    for (int b = threadIdx.x; b < cols; b += blockDim.x) rowbuf[b] = R[(int64_t)pi * cols + b];
    __syncthreads();
    for (int64_t k = threadIdx.x; k < n; k += blockDim.x) {
      const int a = (int)(k / cols), b = (int)(k % cols);
      const double prod = __dmul_rn(colbuf[a], rowbuf[b]);
      R[k] = __dsub_rn(R[k], __ddiv_rn(prod, piv));
    }
    __syncthreads();
    ++r;
  }
  if (r == kmax && kmax > 0) {
    argmax(bv, bk);
    err = n ? bv : 0.0;
  }
  if (threadIdx.x == 0) {
    out[0] = r;
    outd[0] = err;
    outd[1] = scale;
  }
}

}  // namespace
}  // namespace tnfa

using namespace tnfa;

int tnfa_cross(tnfa_ctx* ctx, const double* block, int mem, int32_t rows, int32_t cols, double tol,
               int32_t maxrank, int32_t* piv_rows, int32_t* piv_cols, int32_t* rank, double* err) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  TNFA_CHECK(block && piv_rows && piv_cols && rank, TNFA_ERR_INVALID_ARGUMENT, "cross: null argument");
  TNFA_CHECK(rows >= 1 && cols >= 1 && maxrank >= 0 && tol >= 0, TNFA_ERR_INVALID_ARGUMENT,
             "cross: rows, cols >= 1, maxrank, tol >= 0");
  TNFA_CHECK(mem == TNFA_MEM_HOST || mem == TNFA_MEM_DEVICE, TNFA_ERR_INVALID_ARGUMENT, "cross: bad memory kind");
  const int64_t n = (int64_t)rows * cols;
  TNFA_CHECK(n < (int64_t(1) << 31), TNFA_ERR_UNSUPPORTED, "cross: block too large");
  const int kmax = std::min<int>(maxrank, std::min(rows, cols));
  const bool smem = n + rows + cols <= CROSS_SMEM_ELEMS;
  DBuf dM(ctx, mem == TNFA_MEM_HOST ? (size_t)n * 8 : 0);
  const double* M = block;
  if (mem == TNFA_MEM_HOST) {
    TNFA_CUDA(cudaMemcpyAsync(dM.p, block, (size_t)n * 8, cudaMemcpyHostToDevice, ctx->stream));
    M = dM.as<double>();
  }
  DBuf Rg(ctx, smem ? 0 : (size_t)(n + rows + cols) * 8);
  DBuf outi(ctx, (size_t)(1 + 2 * std::max(kmax, 1)) * 4), outd(ctx, 16);
  const size_t shm = smem ? (size_t)(n + rows + cols) * 8 : 0;
  {
    KernelScope ks(ctx, "cross", 3.0 * (double)n * kmax, 8.0 * (double)n);
    TNFA_CUDA(cudaFuncSetAttribute(k_cross_full, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(CROSS_SMEM_ELEMS * 8)));
    k_cross_full<<<1, CROSS_THREADS, shm, ctx->stream>>>(M, Rg.as<double>(), rows, cols, tol, maxrank,
                                                         outi.as<int>(), outd.as<double>(), smem ? 1 : 0);
    TNFA_LAUNCH_CHECK();
  }
  std::vector<int> hi(1 + 2 * std::max(kmax, 1));
  double hd[2];
  TNFA_CUDA(cudaMemcpyAsync(hi.data(), outi.p, hi.size() * 4, cudaMemcpyDeviceToHost, ctx->stream));
  TNFA_CUDA(cudaMemcpyAsync(hd, outd.p, 16, cudaMemcpyDeviceToHost, ctx->stream));
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  const int r = hi[0];
  for (int q = 0; q < r; ++q) {
    piv_rows[q] = hi[1 + q];
    piv_cols[q] = hi[1 + kmax + q];
  }
  *rank = r;
  if (err) {
    err[0] = hd[0];
    err[1] = hd[1];
  }
  TNFA_API_END
}
