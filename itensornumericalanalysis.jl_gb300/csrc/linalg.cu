// Batched dense linear algebra kernels (FP64 real and complex128).
//
//   permute  : general tensor transpose (up to 10 axes)
//   gemm     : tiled SIMT GEMM, 64x64 tiles, op(A) op(B) with N/T/C
//   qr       : Householder QR, one CTA per matrix, column-major workspace
//   svd      : one-sided Jacobi (Hestenes) SVD, round-robin pair ordering,
//              one CTA per matrix, columns contiguous in the workspace
// Every problem of a batch may have its own shape; one launch covers them all.
#include <algorithm>
#include <cmath>
#include <cstdlib>

#include <cooperative_groups.h>

#include "linalg.cuh"

namespace cg = cooperative_groups;

namespace tnfa {
namespace la {

// ---------------------------------------------------------- scalar ops --
__host__ __device__ inline double re(double x) { return x; }
__host__ __device__ inline double re(cplx x) { return x.re; }
__host__ __device__ inline double abs2(double x) { return x * x; }
__host__ __device__ inline double abs2(cplx x) { return x.re * x.re + x.im * x.im; }
__host__ __device__ inline double conj(double x) { return x; }
__host__ __device__ inline cplx conj(cplx x) { return {x.re, -x.im}; }
__host__ __device__ inline double scal(double x, double a) { return x * a; }
__host__ __device__ inline cplx scal(cplx x, double a) { return {x.re * a, x.im * a}; }
template <class T> __host__ __device__ inline T from_real(double a);
template <> __host__ __device__ inline double from_real<double>(double a) { return a; }
template <> __host__ __device__ inline cplx from_real<cplx>(double a) { return {a, 0.0}; }
__host__ __device__ inline float re(float x) { return x; }
__host__ __device__ inline float abs2(float x) { return x * x; }
__host__ __device__ inline float conj(float x) { return x; }
__host__ __device__ inline float scal(float x, float a) { return x * a; }
template <> __host__ __device__ inline float from_real<float>(double a) { return (float)a; }
__device__ inline float shfl_xor(float v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ inline float phase(float x) { return x < 0 ? -1.0f : 1.0f; }
__device__ inline double shfl_xor(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ inline cplx shfl_xor(cplx v, int o) {
  return {__shfl_xor_sync(0xffffffffu, v.re, o), __shfl_xor_sync(0xffffffffu, v.im, o)};
}
template <class T>
__device__ inline T warp_sum(T v) {
  for (int o = 16; o; o >>= 1) v = v + shfl_xor(v, o);
  return v;
}
// x / |x| (1 for x = 0)
__device__ inline double phase(double x) { return x < 0 ? -1.0 : 1.0; }
__device__ inline cplx phase(cplx x) {
  double a = sqrt(abs2(x));
  return a > 0 ? cplx{x.re / a, x.im / a} : cplx{1.0, 0.0};
}

template <class Job>
static DBuf upload(tnfa_ctx* ctx, const std::vector<Job>& jobs) {
  DBuf d(ctx, jobs.size() * sizeof(Job));
  TNFA_CUDA(cudaMemcpyAsync(d.p, jobs.data(), jobs.size() * sizeof(Job), cudaMemcpyHostToDevice,
                            ctx->stream));
  return d;
}

// ------------------------------------------------------------- permute --
template <class T>
__global__ void k_permute(const PermJob* __restrict__ jobs) {
  const PermJob& jb = jobs[blockIdx.y];
  int64_t sstride[MAXD];
  int64_t st = 1;
  for (int a = jb.nd - 1; a >= 0; --a) {
    sstride[a] = st;
    st *= jb.shape[a];
  }
  const T* src = (const T*)jb.src;
  T* dst = (T*)jb.dst;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < jb.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = i, si = 0;
    for (int a = jb.nd - 1; a >= 0; --a) {
      const int sa = jb.perm[a];
      const int64_t x = r % jb.shape[sa];
      r /= jb.shape[sa];
      si += x * sstride[sa];
    }
    dst[i] = src[si];
  }
}

template <class T>
void permute(tnfa_ctx* ctx, const std::vector<PermJob>& jobs) {
  if (jobs.empty()) return;
  int64_t nmax = 1;
  for (const auto& j : jobs) nmax = std::max(nmax, j.n);
  TNFA_CHECK(jobs.size() <= 65535, TNFA_ERR_UNSUPPORTED, "permute batch too large");
  DBuf d = upload(ctx, jobs);
  dim3 grid(grid_for(nmax, 256, 2048), (unsigned)jobs.size());
  KernelScope ks(ctx, "permute", 0.0, 2.0 * sizeof(T) * nmax * jobs.size());
  k_permute<T><<<grid, 256, 0, ctx->stream>>>(d.as<PermJob>());
  TNFA_LAUNCH_CHECK();
}

// ---------------------------------------------------------------- gemm --
template <class T>
__device__ inline T opget(const T* X, int ld, int op, int r, int c) {
  // element (r, c) of op(X)
  if (op == 0) return X[(int64_t)r * ld + c];
  T v = X[(int64_t)c * ld + r];
  return op == 2 ? conj(v) : v;
}

template <class T>
__global__ void __launch_bounds__(256) k_gemm(const GemmJob* __restrict__ jobs) {
  constexpr int BM = 64, BN = 64, BK = 16;
  const GemmJob& jb = jobs[blockIdx.z];
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  if (m0 >= jb.m || n0 >= jb.n) return;
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const T* A = (const T*)jb.A;
  const T* B = (const T*)jb.B;
  T* C = (T*)jb.C;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = from_real<T>(0.0);
  for (int k0 = 0; k0 < jb.k; k0 += BK) {
    for (int idx = threadIdx.x; idx < BM * BK; idx += 256) {
      int r, kk;
      if (jb.opA == 0) { r = idx / BK; kk = idx % BK; }   // contiguous along k
      else { kk = idx / BM; r = idx % BM; }              // contiguous along m
      const int gr = m0 + r, gk = k0 + kk;
      As[kk][r] = (gr < jb.m && gk < jb.k) ? opget(A, jb.lda, jb.opA, gr, gk) : from_real<T>(0.0);
    }
    for (int idx = threadIdx.x; idx < BN * BK; idx += 256) {
      int c, kk;
      if (jb.opB == 0) { kk = idx / BN; c = idx % BN; }   // contiguous along n
      else { c = idx / BK; kk = idx % BK; }              // contiguous along k
      const int gc = n0 + c, gk = k0 + kk;
      Bs[kk][c] = (gc < jb.n && gk < jb.k) ? opget(B, jb.ldb, jb.opB, gk, gc) : from_real<T>(0.0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = Sc<T>::fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = m0 + ty + 16 * i;
    if (r >= jb.m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = n0 + tx + 16 * j;
      if (c >= jb.n) continue;
      T v = scal(acc[i][j], jb.alpha);
      T* cp = C + (int64_t)r * jb.ldc + c;
      *cp = jb.beta == 0.0 ? v : v + scal(*cp, jb.beta);
    }
  }
}

template <class T>
void gemm(tnfa_ctx* ctx, const std::vector<GemmJob>& jobs) {
  if (jobs.empty()) return;
  int mt = 1, nt = 1;
  double fl = 0;
  for (const auto& j : jobs) {
    mt = std::max(mt, (j.m + 63) / 64);
    nt = std::max(nt, (j.n + 63) / 64);
    fl += 2.0 * j.m * j.n * j.k;
  }
  TNFA_CHECK(jobs.size() <= 65535 && mt <= 65535, TNFA_ERR_UNSUPPORTED, "gemm batch too large");
  DBuf d = upload(ctx, jobs);
  dim3 grid(nt, mt, (unsigned)jobs.size());
  KernelScope ks(ctx, sizeof(T) == 8 ? "gemm_f64" : "gemm_c128", fl, 0.0);
  k_gemm<T><<<grid, 256, 0, ctx->stream>>>(d.as<GemmJob>());
  TNFA_LAUNCH_CHECK();
}

template <class Job>
std::string size_note(const std::vector<Job>& jobs) {
  int mm = 0, mn = 0;
  double work = 0;
  for (const auto& j : jobs) {
    mm = std::max(mm, j.m);
    mn = std::max(mn, j.n);
    work += (double)j.m * j.n * j.n;
  }
  char b[160];
  snprintf(b, sizeof b, "jobs=%zu max_m=%d max_n=%d sum_mn2=%.3g", jobs.size(), mm, mn, work);
  return b;
}

// ------------------------------------------------------------------ qr --
template <class T>
__device__ inline T block_sum(T v, T* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    T t = lane < nw ? red[lane] : from_real<T>(0.0);
    t = warp_sum(t);
    if (lane == 0) red[0] = t;
  }
  __syncthreads();
  T r = red[0];
  __syncthreads();
  return r;
}

// Workspace per job: A copied column-major into W (m*n), Q column-major
// into Qw (m*kq); reflector j is stored in W column j rows j..m-1.
template <class T>
__global__ void __launch_bounds__(512) k_qr(const QrJob* __restrict__ jobs, T* __restrict__ work,
                                            const int64_t* __restrict__ woff) {
  const QrJob jb = jobs[blockIdx.x];
  const int m = jb.m, n = jb.n, kq = min(m, n);
  T* W = work + woff[blockIdx.x];
  T* Qw = W + (int64_t)m * n;
  T* tau = (T*)jb.tau;
  const T* A = (const T*)jb.A;
  __shared__ T red[32];
  __shared__ T alpha_sh;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t i = threadIdx.x; i < (int64_t)m * n; i += blockDim.x) {
    const int r = (int)(i / n), c = (int)(i % n);
    W[(int64_t)c * m + r] = A[i];
  }
  __syncthreads();
  T* R = (T*)jb.R;
  for (int j = 0; j < kq; ++j) {
    T* x = W + (int64_t)j * m;
    double part = 0.0;
    for (int r = j + threadIdx.x; r < m; r += blockDim.x) part += abs2(x[r]);
    const double nrm2 = re(block_sum<T>(from_real<T>(part), red));
    if (threadIdx.x == 0) {
      const T x0 = x[j];
      const double nrm = sqrt(nrm2);
      if (!(nrm > 1e-150)) {
        // an (almost) eliminated column: no reflection.  A residue this small
        // (rounding left by earlier steps) would make 2 / |v|^2 overflow.
        tau[j] = from_real<T>(0.0);
        alpha_sh = x0;
      } else {
        const T alpha = scal(phase(x0), -nrm);
        const T v0 = x0 - alpha;
        const double vn2 = nrm2 - abs2(x0) + abs2(v0);
        tau[j] = from_real<T>(vn2 > 0.0 ? 2.0 / vn2 : 0.0);
        x[j] = v0;
        alpha_sh = alpha;
      }
    }
    __syncthreads();
    const double beta = re(tau[j]);
    const T alpha = alpha_sh;
    if (beta != 0.0) {
      for (int c = j + 1 + warp; c < n; c += nw) {
        T* y = W + (int64_t)c * m;
        T w = from_real<T>(0.0);
        for (int r = j + lane; r < m; r += 32) w = Sc<T>::fma(conj(x[r]), y[r], w);
        w = warp_sum(w);
        const T bw = scal(w, beta);
        for (int r = j + lane; r < m; r += 32) y[r] = y[r] - x[r] * bw;
      }
    }
    __syncthreads();
    // R row j: diagonal alpha, then the updated row j of the trailing block
    for (int c = threadIdx.x; c < n; c += blockDim.x)
      R[(int64_t)j * n + c] = c < j ? from_real<T>(0.0) : (c == j ? alpha : W[(int64_t)c * m + j]);
    __syncthreads();
  }
  // Q = H_0 ... H_{kq-1} [I; 0]
  for (int64_t i = threadIdx.x; i < (int64_t)m * kq; i += blockDim.x) {
    const int c = (int)(i / m), r = (int)(i % m);
    Qw[i] = from_real<T>(r == c ? 1.0 : 0.0);
  }
  __syncthreads();
  for (int j = kq - 1; j >= 0; --j) {
    const double beta = re(tau[j]);
    if (beta != 0.0) {
      const T* x = W + (int64_t)j * m;
      for (int c = j + warp; c < kq; c += nw) {
        T* y = Qw + (int64_t)c * m;
        T w = from_real<T>(0.0);
        for (int r = j + lane; r < m; r += 32) w = Sc<T>::fma(conj(x[r]), y[r], w);
        w = warp_sum(w);
        const T bw = scal(w, beta);
        for (int r = j + lane; r < m; r += 32) y[r] = y[r] - x[r] * bw;
      }
    }
    __syncthreads();
  }
  T* Q = (T*)jb.Q;
  for (int64_t i = threadIdx.x; i < (int64_t)m * kq; i += blockDim.x) {
    const int r = (int)(i / kq), c = (int)(i % kq);
    Q[i] = Qw[(int64_t)c * m + r];
  }
}

template <class T>
void qr(tnfa_ctx* ctx, const std::vector<QrJob>& jobs) {
  if (jobs.empty()) return;
  std::vector<int64_t> woff(jobs.size() + 1, 0);
  double fl = 0;
  for (size_t i = 0; i < jobs.size(); ++i) {
    const int64_t m = jobs[i].m, n = jobs[i].n, k = std::min(m, n);
    woff[i + 1] = woff[i] + m * n + m * k;
    fl += 4.0 * m * n * k;
  }
  DBuf work(ctx, (size_t)woff.back() * sizeof(T));
  DBuf dw = upload(ctx, woff);
  DBuf d = upload(ctx, jobs);
  KernelScope ks(ctx, sizeof(T) == 8 ? "qr_f64" : "qr_c128", fl, 0.0);
  if (trace_on()) ks.note = size_note(jobs);
  k_qr<T><<<(unsigned)jobs.size(), 512, 0, ctx->stream>>>(d.as<QrJob>(), work.as<T>(),
                                                          dw.as<int64_t>());
  TNFA_LAUNCH_CHECK();
}

// ----------------------------------------------------------------- svd --
void trace_sweeps(tnfa_ctx* ctx, const std::vector<SvdJob>& jobs) {
  int mx = 0, capped = 0, cnt = 0;
  long tot = 0;
  for (const auto& j : jobs) {
    if (!j.sweeps) continue;
    int sw = 0;
    TNFA_CUDA(cudaMemcpyAsync(&sw, j.sweeps, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
    if (sw < 0) ++capped;
    else mx = std::max(mx, sw), tot += sw, ++cnt;
  }
  fprintf(stderr, "tnfa-trace svd-sweeps max=%d mean=%.2f capped=%d\n", mx, cnt ? (double)tot / cnt : 0.0,
          capped);
}

// Round-robin pairing of n2 (even) players: round r, slot i.
__device__ inline void rr_pair(int n2, int r, int i, int& p, int& q) {
  if (i == 0) {
    p = n2 - 1;
    q = r;
  } else {
    p = (r + i) % (n2 - 1);
    q = (r - i + (n2 - 1)) % (n2 - 1);
  }
  if (p > q) {
    int t = p;
    p = q;
    q = t;
  }
}

template <class T>
__global__ void __launch_bounds__(512) k_svd(const SvdJob* __restrict__ jobs, T* __restrict__ work,
                                             const int64_t* __restrict__ woff, int max_sweeps) {
  const SvdJob jb = jobs[blockIdx.x];
  const int m = jb.m, n = jb.n;
  T* U = work + woff[blockIdx.x];     // column-major m x n (columns contiguous)
  T* V = U + (int64_t)m * n;          // column-major n x n
  double* sig = (double*)(V + (int64_t)n * n);
  int* rank = (int*)(sig + n);
  const T* A = (const T*)jb.A;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __shared__ int rotated;
  for (int64_t i = threadIdx.x; i < (int64_t)m * n; i += blockDim.x) {
    const int r = (int)(i / n), c = (int)(i % n);
    U[(int64_t)c * m + r] = A[i];
  }
  for (int64_t i = threadIdx.x; i < (int64_t)n * n; i += blockDim.x)
    V[i] = from_real<T>((i / n) == (i % n) ? 1.0 : 0.0);
  __shared__ double red[32];
  double part = 0.0;
  for (int64_t i = threadIdx.x; i < (int64_t)m * n; i += blockDim.x) part += abs2(A[i]);
  const double fro2 = block_sum<double>(part, red);
  // columns below this are rounding noise of the whole matrix
  const double negl = 1e-30 * fro2;
  const int n2 = (n + 1) & ~1;
  int sweep = 0;
  bool converged = (n < 2);
  // pairs count as orthogonal once |g| <= tol sqrt(a b); the rounding floor of
  // a length-m dot product is ~sqrt(m) eps
  const double tol = 8.0 * sqrt((double)m) * 2.220446049250313e-16;
  while (!converged && sweep < max_sweeps) {
    if (threadIdx.x == 0) rotated = 0;
    __syncthreads();
    for (int r = 0; r < n2 - 1; ++r) {
      for (int slot = warp; slot < n2 / 2; slot += nw) {
        int p, q;
        rr_pair(n2, r, slot, p, q);
        if (q >= n) continue;
        T* up = U + (int64_t)p * m;
        T* uq = U + (int64_t)q * m;
        double a = 0.0, b = 0.0;
        T g = from_real<T>(0.0);
        for (int i = lane; i < m; i += 32) {
          a += abs2(up[i]);
          b += abs2(uq[i]);
          g = Sc<T>::fma(conj(up[i]), uq[i], g);
        }
        a = warp_sum(a);
        b = warp_sum(b);
        g = warp_sum(g);
        const double ag = sqrt(abs2(g));
        // a negligible column carries no singular value worth orthogonalising
        // against; skipping it also avoids zeta^2 overflow on extreme ratios
        if (ag <= tol * sqrt(a * b) || ag == 0.0 || a < negl || b < negl) continue;
        const double zeta = (b - a) / (2.0 * ag);
        const double t = fabs(zeta) > 1e150
                             ? 0.5 / zeta
                             : (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        if (t == 0.0) continue;
        const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
        const T e = phase(g);  // g / |g|
        const T se = scal(e, s), sec = scal(conj(e), s);
        for (int i = lane; i < m; i += 32) {
          const T xp = up[i], xq = uq[i];
          up[i] = scal(xp, c) - sec * xq;
          uq[i] = se * xp + scal(xq, c);
        }
        T* vp = V + (int64_t)p * n;
        T* vq = V + (int64_t)q * n;
        for (int i = lane; i < n; i += 32) {
          const T xp = vp[i], xq = vq[i];
          vp[i] = scal(xp, c) - sec * xq;
          vq[i] = se * xp + scal(xq, c);
        }
        if (lane == 0) rotated = 1;
      }
      __syncthreads();
    }
    ++sweep;
    converged = (rotated == 0);
    __syncthreads();
  }
  // singular values, ranks (descending, stable), normalised outputs
  for (int c = warp; c < n; c += nw) {
    double s2 = 0.0;
    for (int i = lane; i < m; i += 32) s2 += abs2(U[(int64_t)c * m + i]);
    s2 = warp_sum(s2);
    if (lane == 0) sig[c] = sqrt(s2);
  }
  __syncthreads();
  for (int c = threadIdx.x; c < n; c += blockDim.x) {
    int rk = 0;
    for (int d = 0; d < n; ++d) rk += (sig[d] > sig[c]) || (sig[d] == sig[c] && d < c);
    rank[c] = rk;
    jb.S[rk] = sig[c];
  }
  __syncthreads();
  T* Uo = (T*)jb.U;
  T* Vo = (T*)jb.V;
  for (int64_t i = threadIdx.x; i < (int64_t)m * n; i += blockDim.x) {
    const int c = (int)(i / m), r = (int)(i % m);
    const double s = sig[c];
    Uo[(int64_t)r * n + rank[c]] = s > 0 ? scal(U[i], 1.0 / s) : from_real<T>(0.0);
  }
  for (int64_t i = threadIdx.x; i < (int64_t)n * n; i += blockDim.x) {
    const int c = (int)(i / n), r = (int)(i % n);
    Vo[(int64_t)r * n + rank[c]] = V[i];
  }
  if (threadIdx.x == 0 && jb.sweeps) *jb.sweeps = converged ? sweep : -1;
}

// The same Jacobi iteration spread over a thread-block cluster: the pairs of a
// round are shared by the warps of all CTAs of the cluster, the columns live
// in global memory (L2-resident; loads and stores bypass L1), and a cluster
// barrier (release / acquire at cluster scope) separates the rounds.  The
// convergence decision of a sweep is read by every CTA from one global flag
// after the sweep's last barrier, so all CTAs leave the loop together; flag
// k % 3 is cleared two sweeps before it is reused, after every CTA has read it.
template <class T> struct RealOf { using type = double; };
template <> struct RealOf<float> { using type = float; };

__device__ inline double ldcg(const double* p) { return __ldcg(p); }
__device__ inline float ldcg(const float* p) { return __ldcg(p); }
__device__ inline cplx ldcg(const cplx* p) {
  const double2 v = __ldcg((const double2*)p);
  return {v.x, v.y};
}
__device__ inline void stcg(double* p, double v) { __stcg(p, v); }
__device__ inline void stcg(float* p, float v) { __stcg(p, v); }
__device__ inline void stcg(cplx* p, cplx v) { __stcg((double2*)p, make_double2(v.re, v.im)); }
__device__ inline float fmaT(float a, float b, float c) { return fmaf(a, b, c); }
__device__ inline double fmaT(double a, double b, double c) { return fma(a, b, c); }
__device__ inline cplx fmaT(cplx a, cplx b, cplx c) { return Sc<cplx>::fma(a, b, c); }

template <class T>
__global__ void __launch_bounds__(512) k_svd_cluster(const SvdJob* __restrict__ jobs, T* __restrict__ work,
                                                     const int64_t* __restrict__ woff, int* __restrict__ flags,
                                                     int max_sweeps, int init_v) {
  using R = typename RealOf<T>::type;
  cg::cluster_group cl = cg::this_cluster();
  const int C = (int)cl.num_blocks(), crank = (int)cl.block_rank();
  const int ji = blockIdx.x / C;
  const SvdJob jb = jobs[ji];
  const int m = jb.m, n = jb.n;
  T* U = work + woff[ji];
  T* V = U + (int64_t)m * n;
  double* sig = (double*)(V + (int64_t)n * n);
  int* rank = (int*)(sig + n);
  int* flag = flags + 3 * ji;
  const T* A = (const T*)jb.A;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int64_t gt = (int64_t)crank * blockDim.x + threadIdx.x, gs = (int64_t)C * blockDim.x;
  for (int64_t i = gt; i < (int64_t)m * n; i += gs) {
    const int r = (int)(i / n), c = (int)(i % n);
    stcg(U + (int64_t)c * m + r, A[i]);
  }
  // V starts as the identity, or (init_v) as jb.V given row-major
  for (int64_t i = gt; i < (int64_t)n * n; i += gs) {
    const int c = (int)(i / n), r = (int)(i % n);
    stcg(V + i, init_v ? ((const T*)jb.V)[(int64_t)r * n + c] : from_real<T>(r == c ? 1.0 : 0.0));
  }
  __shared__ double red[32];
  double part = 0.0;
  for (int64_t i = threadIdx.x; i < (int64_t)m * n; i += blockDim.x) part += (double)abs2(A[i]);
  const double fro2 = block_sum<double>(part, red);
  const double eps = sizeof(R) == 4 ? 1.1920929e-7 : 2.220446049250313e-16;
  const double negl = (sizeof(R) == 4 ? 1e-13 : 1e-30) * fro2;
  const R tol = (R)(8.0 * sqrt((double)m) * eps);
  const int n2 = (n + 1) & ~1;
  const int gw = crank * nw + warp, nwc = C * nw;
  int sweep = 0;
  bool converged = (n < 2);
  cl.sync();
  while (!converged && sweep < max_sweeps) {
    if (crank == 0 && threadIdx.x == 0) flag[(sweep + 1) % 3] = 0;
    int rotated_here = 0;
    for (int r = 0; r < n2 - 1; ++r) {
      for (int slot = gw; slot < n2 / 2; slot += nwc) {
        int p, q;
        rr_pair(n2, r, slot, p, q);
        if (q >= n) continue;
        T* up = U + (int64_t)p * m;
        T* uq = U + (int64_t)q * m;
        R a = 0, b = 0;
        T g = from_real<T>(0.0);
        for (int i = lane; i < m; i += 32) {
          const T xp = ldcg(up + i), xq = ldcg(uq + i);
          a += abs2(xp);
          b += abs2(xq);
          g = fmaT(conj(xp), xq, g);
        }
        a = warp_sum(a);
        b = warp_sum(b);
        g = warp_sum(g);
        const R ag = sqrt(abs2(g));
        if (ag <= tol * sqrt(a * b) || ag == (R)0 || (double)a < negl || (double)b < negl) continue;
        const R zeta = (b - a) / ((R)2 * ag);
        const R big = sizeof(R) == 4 ? (R)1e18 : (R)1e150;
        const R t = fabs(zeta) > big ? (R)0.5 / zeta
                                     : (zeta >= 0 ? (R)1 : (R)-1) / (fabs(zeta) + sqrt((R)1 + zeta * zeta));
        if (t == (R)0) continue;
        const R c = (R)1 / sqrt((R)1 + t * t), sn = c * t;
        const T e = phase(g);
        const T se = scal(e, sn), sec = scal(conj(e), sn);
        for (int i = lane; i < m; i += 32) {
          const T xp = ldcg(up + i), xq = ldcg(uq + i);
          stcg(up + i, scal(xp, c) - sec * xq);
          stcg(uq + i, se * xp + scal(xq, c));
        }
        T* vp = V + (int64_t)p * n;
        T* vq = V + (int64_t)q * n;
        for (int i = lane; i < n; i += 32) {
          const T xp = ldcg(vp + i), xq = ldcg(vq + i);
          stcg(vp + i, scal(xp, c) - sec * xq);
          stcg(vq + i, se * xp + scal(xq, c));
        }
        rotated_here = 1;
      }
      cl.sync();
    }
    // (a flag store after the round's barrier would still precede the read
    // below only through the next barrier, so it is stored before the last one)
    if (rotated_here && lane == 0) atomicOr(flag + sweep % 3, 1);
    cl.sync();
    converged = (__ldcg(flag + sweep % 3) == 0);
    ++sweep;
  }
  for (int c = gw; c < n; c += nwc) {
    double s2 = 0.0;
    for (int i = lane; i < m; i += 32) s2 += (double)abs2(ldcg(U + (int64_t)c * m + i));
    s2 = warp_sum(s2);
    if (lane == 0) __stcg(sig + c, sqrt(s2));
  }
  cl.sync();
  for (int64_t c = gt; c < n; c += gs) {
    const double sc = __ldcg(sig + c);
    int rk = 0;
    for (int d = 0; d < n; ++d) {
      const double sd = __ldcg(sig + d);
      rk += (sd > sc) || (sd == sc && d < c);
    }
    __stcg(rank + c, rk);
    jb.S[rk] = sc;
  }
  cl.sync();
  T* Uo = (T*)jb.U;
  T* Vo = (T*)jb.V;
  for (int64_t i = gt; i < (int64_t)m * n; i += gs) {
    const int c = (int)(i / m), r = (int)(i % m);
    const double sc = __ldcg(sig + c);
    Uo[(int64_t)r * n + __ldcg(rank + c)] = sc > 0 ? scal(ldcg(U + i), (R)(1.0 / sc)) : from_real<T>(0.0);
  }
  for (int64_t i = gt; i < (int64_t)n * n; i += gs) {
    const int c = (int)(i / n), r = (int)(i % n);
    Vo[(int64_t)r * n + __ldcg(rank + c)] = ldcg(V + i);
  }
  if (crank == 0 && threadIdx.x == 0 && jb.sweeps) *jb.sweeps = converged ? sweep : -1;
}

constexpr int SVD_CLUSTER = 8;  // CTAs (SMs) per large matrix

// A job goes to the cluster kernel when its Jacobi work is large enough to
// pay for a cluster barrier per round.
inline bool svd_big(const SvdJob& j) { return j.n >= 96 && (double)j.m * j.n * j.n >= 2.0e6; }

template <class T>
void launch_svd(tnfa_ctx* ctx, const std::vector<SvdJob>& jobs, int max_sweeps, bool init_v,
                const char* family) {
  std::vector<SvdJob> big, small;
  for (const auto& j : jobs) (svd_big(j) ? big : small).push_back(j);
  for (int pass = 0; pass < 2; ++pass) {
    const std::vector<SvdJob>& js = pass == 0 ? big : small;
    if (js.empty()) continue;
    std::vector<int64_t> woff(js.size() + 1, 0);
    double fl = 0;
    for (size_t i = 0; i < js.size(); ++i) {
      TNFA_CHECK(js[i].m >= js[i].n, TNFA_ERR_INVALID_ARGUMENT, "svd needs m >= n");
      const int64_t m = js[i].m, n = js[i].n;
      // U, V in T; sig (n doubles) and rank (n ints) rounded up to T slots
      woff[i + 1] = woff[i] + m * n + n * n + (int64_t)((n * 12 + sizeof(T) - 1) / sizeof(T)) + 2;
      fl += 6.0 * m * n * n * 8;  // ~8 sweeps
    }
    DBuf work(ctx, (size_t)woff.back() * sizeof(T));
    DBuf dw = upload(ctx, woff);
    DBuf d = upload(ctx, js);
    KernelScope ks(ctx, family, fl, 0.0);
    if (trace_on()) ks.note = (pass == 0 ? "cluster " : "single ") + size_note(js);
    if (pass == 0) {
      DBuf flags(ctx, js.size() * 3 * sizeof(int));
      TNFA_CUDA(cudaMemsetAsync(flags.p, 0, js.size() * 3 * sizeof(int), ctx->stream));
      cudaLaunchConfig_t cfg{};
      cfg.gridDim = dim3((unsigned)(js.size() * SVD_CLUSTER));
      cfg.blockDim = dim3(512);
      cfg.stream = ctx->stream;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = SVD_CLUSTER;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      TNFA_CUDA(cudaLaunchKernelEx(&cfg, k_svd_cluster<T>, (const SvdJob*)d.as<SvdJob>(), work.as<T>(),
                                   (const int64_t*)dw.as<int64_t>(), flags.as<int>(), max_sweeps,
                                   init_v ? 1 : 0));
    } else {
      TNFA_CHECK(!init_v, TNFA_ERR_UNSUPPORTED, "svd: initial V needs the cluster kernel");
      k_svd<T><<<(unsigned)js.size(), 512, 0, ctx->stream>>>(d.as<SvdJob>(), work.as<T>(),
                                                             dw.as<int64_t>(), max_sweeps);
    }
    TNFA_LAUNCH_CHECK();
  }
}

template <class T>
void svd(tnfa_ctx* ctx, const std::vector<SvdJob>& jobs, int max_sweeps) {
  if (jobs.empty()) return;
  launch_svd<T>(ctx, jobs, max_sweeps, false, sizeof(T) == 8 ? "svd_f64" : "svd_c128");
  if (trace_on()) trace_sweeps(ctx, jobs);
  // Diagnostics: with TNFA_DEBUG_DIR set, the input of every SVD that hit the
  // sweep cap is written there (int32 m, int32 n, element size, then data).
  static const char* dbg = getenv("TNFA_DEBUG_DIR");
  if (dbg && *dbg) {
    static int counter = 0;
    for (const auto& j : jobs) {
      if (!j.sweeps) continue;
      int sw = 0;
      TNFA_CUDA(cudaMemcpyAsync(&sw, j.sweeps, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
      if (sw >= 0) continue;
      std::vector<T> h((size_t)j.m * j.n);
      TNFA_CUDA(cudaMemcpyAsync(h.data(), j.A, h.size() * sizeof(T), cudaMemcpyDeviceToHost,
                                ctx->stream));
      TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
      char path[1024];
      snprintf(path, sizeof path, "%s/svd_nonconv_%d.bin", dbg, counter++);
      if (FILE* fp = fopen(path, "wb")) {
        int hdr[3] = {j.m, j.n, (int)sizeof(T)};
        fwrite(hdr, sizeof(int), 3, fp);
        fwrite(h.data(), sizeof(T), h.size(), fp);
        fclose(fp);
      }
    }
  }
}

// ------------------------------------------------------------------ lu --
constexpr int LU_NB = 32;

// Factor columns k..k+kb-1 (rows k..n-1); row swaps inside the panel only.
__global__ void __launch_bounds__(512) k_lu_panel(double* A, int n, int k, int kb, int* piv,
                                                  int* singular) {
  __shared__ double vmax[32];
  __shared__ int imax[32];
  __shared__ int p_sh;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = k; j < k + kb; ++j) {
    double best = -1.0;
    int bi = j;
    for (int r = j + threadIdx.x; r < n; r += blockDim.x) {
      const double a = fabs(A[(int64_t)r * n + j]);
      if (a > best) {
        best = a;
        bi = r;
      }
    }
    for (int o = 16; o; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    if (lane == 0) {
      vmax[warp] = best;
      imax[warp] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double b = -1.0;
      int i = j;
      for (int w = 0; w < nw; ++w)
        if (vmax[w] > b || (vmax[w] == b && imax[w] < i)) {
          b = vmax[w];
          i = imax[w];
        }
      p_sh = i;
      piv[j] = i;
      if (!(b > 0.0)) *singular = 1;
    }
    __syncthreads();
    const int p = p_sh;
    if (p != j)
      for (int c = k + threadIdx.x; c < k + kb; c += blockDim.x) {
        const double t = A[(int64_t)j * n + c];
        A[(int64_t)j * n + c] = A[(int64_t)p * n + c];
        A[(int64_t)p * n + c] = t;
      }
    __syncthreads();
    const double d = A[(int64_t)j * n + j];
    if (d != 0.0) {
      for (int r = j + 1 + threadIdx.x; r < n; r += blockDim.x) {
        double* row = A + (int64_t)r * n;
        const double l = row[j] / d;
        row[j] = l;
        for (int c = j + 1; c < k + kb; ++c) row[c] -= l * A[(int64_t)j * n + c];
      }
    }
    __syncthreads();
  }
}

// Apply the panel's row swaps to the columns outside it.
__global__ void k_lu_swap(double* A, int n, int k, int kb, const int* piv) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    if (c >= k && c < k + kb) continue;
    for (int j = k; j < k + kb; ++j) {
      const int p = piv[j];
      if (p != j) {
        const double t = A[(int64_t)j * n + c];
        A[(int64_t)j * n + c] = A[(int64_t)p * n + c];
        A[(int64_t)p * n + c] = t;
      }
    }
  }
}

// U12 = L11^{-1} A12 (unit lower triangular L11), one column per thread.
__global__ void k_lu_trsm(double* A, int n, int k, int kb) {
  for (int c = k + kb + blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
    for (int r = k + 1; r < k + kb; ++r) {
      double acc = A[(int64_t)r * n + c];
      for (int t = k; t < r; ++t) acc -= A[(int64_t)r * n + t] * A[(int64_t)t * n + c];
      A[(int64_t)r * n + c] = acc;
    }
}

// Swaps on b, then L y = b (unit diagonal) and U x = y, one CTA.
__global__ void __launch_bounds__(512) k_lu_subst(const double* A, int n, const int* piv, double* b) {
  __shared__ double red[32];
  if (threadIdx.x == 0)
    for (int j = 0; j < n; ++j) {
      const int p = piv[j];
      if (p != j) {
        const double t = b[j];
        b[j] = b[p];
        b[p] = t;
      }
    }
  __syncthreads();
  for (int r = 1; r < n; ++r) {
    double part = 0.0;
    for (int t = threadIdx.x; t < r; t += blockDim.x) part += A[(int64_t)r * n + t] * b[t];
    const double s = block_sum<double>(part, red);
    if (threadIdx.x == 0) b[r] -= s;
    __syncthreads();
  }
  for (int r = n - 1; r >= 0; --r) {
    double part = 0.0;
    for (int t = r + 1 + threadIdx.x; t < n; t += blockDim.x) part += A[(int64_t)r * n + t] * b[t];
    const double s = block_sum<double>(part, red);
    if (threadIdx.x == 0) b[r] = (b[r] - s) / A[(int64_t)r * n + r];
    __syncthreads();
  }
}

bool lu_solve(tnfa_ctx* ctx, double* A, double* b, int n) {
  if (n <= 0) return true;
  DBuf piv(ctx, (size_t)n * sizeof(int)), sing(ctx, sizeof(int));
  TNFA_CUDA(cudaMemsetAsync(sing.p, 0, sizeof(int), ctx->stream));
  KernelScope ks(ctx, "lu_f64", 2.0 / 3.0 * (double)n * n * n, 0.0);
  for (int k = 0; k < n; k += LU_NB) {
    const int kb = std::min(LU_NB, n - k);
    k_lu_panel<<<1, 512, 0, ctx->stream>>>(A, n, k, kb, piv.as<int>(), sing.as<int>());
    k_lu_swap<<<grid_for(n, 256, 1024), 256, 0, ctx->stream>>>(A, n, k, kb, piv.as<int>());
    if (k + kb < n) {
      k_lu_trsm<<<grid_for(n - k - kb, 128, 1024), 128, 0, ctx->stream>>>(A, n, k, kb);
      const int m2 = n - k - kb;
      GemmJob g{A + (int64_t)(k + kb) * n + k, A + (int64_t)k * n + k + kb,
                A + (int64_t)(k + kb) * n + k + kb, m2, m2, kb, n, n, n, 0, 0, -1.0, 1.0};
      gemm<double>(ctx, {g});
    }
    TNFA_LAUNCH_CHECK();
  }
  k_lu_subst<<<1, 512, 0, ctx->stream>>>(A, n, piv.as<int>(), b);
  TNFA_LAUNCH_CHECK();
  int hs = 0;
  TNFA_CUDA(cudaMemcpyAsync(&hs, sing.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  return hs == 0;
}

int truncation_rank(const double* s, int n, double cutoff, int maxdim, int mindim) {
  if (n <= 0) return 0;
  double total = 0.0;
  for (int i = 0; i < n; ++i) total += s[i] * s[i];
  int r = n;
  if (total > 0.0 && cutoff > 0.0) {
    double dropped = 0.0;
    while (r > 1 && dropped + s[r - 1] * s[r - 1] <= cutoff * total) {
      dropped += s[r - 1] * s[r - 1];
      --r;
    }
  }
  if (maxdim > 0) r = std::min(r, maxdim);
  r = std::max(r, std::min(std::max(mindim, 1), n));
  return r;
}

template void permute<double>(tnfa_ctx*, const std::vector<PermJob>&);
template void permute<cplx>(tnfa_ctx*, const std::vector<PermJob>&);
template void permute<float>(tnfa_ctx*, const std::vector<PermJob>&);
template void gemm<double>(tnfa_ctx*, const std::vector<GemmJob>&);
template void gemm<cplx>(tnfa_ctx*, const std::vector<GemmJob>&);
template void qr<double>(tnfa_ctx*, const std::vector<QrJob>&);
template void qr<cplx>(tnfa_ctx*, const std::vector<QrJob>&);
template void svd<double>(tnfa_ctx*, const std::vector<SvdJob>&, int);
template void svd<cplx>(tnfa_ctx*, const std::vector<SvdJob>&, int);

}  // namespace la
}  // namespace tnfa
