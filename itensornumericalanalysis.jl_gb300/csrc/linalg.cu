// Batched dense linear algebra kernels (FP64 real and complex128; FP32 for
// the first passes of the mixed factorisation).
//
//   permute      : general tensor transpose (up to 10 axes)
//   gemm         : tiled SIMT GEMM, 64x64 tiles, op(A) op(B) with N/T/C
//   qr           : Householder QR, one CTA per matrix or an 8-CTA cluster
//                  per large matrix, column-major workspace
//   jacobi       : one-sided Jacobi (Hestenes) SVD, round-robin pairs, one
//                  CTA or an 8-CTA cluster per matrix, register-cached columns
//   trunc_factor : the SVD step of truncation (QR + Jacobi without V, plain
//                  or FP32-preconditioned)
//   lu_solve     : blocked LU with partial pivoting for one dense system
// Every problem of a batch may have its own shape; one launch covers them all.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <type_traits>

#include <cooperative_groups.h>

#include "linalg.cuh"

namespace cg = cooperative_groups;

namespace tnfa {
namespace la {

// ------------------------------------------------------ double-float --
// x = hi + lo (FP32 pair, |lo| <= ulp(hi) / 2): about 48 significant bits
// from FP32 arithmetic, with the error-free sum of Knuth (TAOCP vol. 2,
// 4.2.2) and the error-free product by FMA (after Dekker 1971); division and
// square root take one Newton correction of the FP32 quotient / root.  Used
// where GB300's FP64 rate (1/64 of its FP32 rate) would bound a kernel; the
// range is FP32's, so callers scale by powers of two.
struct dfl {
  float hi, lo;
  __host__ __device__ dfl() : hi(0.f), lo(0.f) {}
  __host__ __device__ constexpr dfl(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ dfl(int x) : hi((float)x), lo(0.f) {}
  __host__ __device__ explicit dfl(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};
__device__ __forceinline__ dfl df_fast2sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dfl df_2sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  const dfl s = df_2sum(a.hi, b.hi);
  return df_fast2sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ dfl operator-(dfl a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__device__ __forceinline__ dfl& operator+=(dfl& a, dfl b) { return a = a + b; }
__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_fast2sum(p, e);
}
__device__ __forceinline__ dfl operator/(dfl a, dfl b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const dfl r = a - b * dfl(q1, 0.f);
  return df_fast2sum(q1, __fdiv_rn(r.hi, b.hi));
}
__device__ __forceinline__ bool operator<(dfl a, dfl b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(dfl a, dfl b) { return b < a; }
__device__ __forceinline__ bool operator<=(dfl a, dfl b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(dfl a, dfl b) { return !(a < b); }
__device__ __forceinline__ bool operator==(dfl a, dfl b) { return a.hi == b.hi && a.lo == b.lo; }
using ::fabs;
using ::sqrt;
__device__ __forceinline__ dfl fabs(dfl a) { return a.hi < 0.f ? -a : a; }
__device__ __forceinline__ dfl sqrt(dfl a) {
  if (!(a.hi > 0.f)) return dfl(0.f, 0.f);
  const float x = __fsqrt_rn(a.hi);
  const float xx = __fmul_rn(x, x);
  const dfl r = a - dfl(xx, __fmaf_rn(x, x, -xx));
  return df_fast2sum(x, __fdiv_rn(r.hi, __fmul_rn(2.f, x)));
}


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
__device__ inline float absval(float x) { return fabsf(x); }
__device__ inline double absval(double x) { return fabs(x); }
__device__ inline double absval(cplx x) { return hypot(x.re, x.im); }
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
  double a = hypot(x.re, x.im);
  return a > 0 ? cplx{x.re / a, x.im / a} : cplx{1.0, 0.0};
}
__device__ inline dfl re(dfl x) { return x; }
__device__ inline dfl abs2(dfl x) { return x * x; }
__device__ inline dfl conj(dfl x) { return x; }
__device__ inline dfl scal(dfl x, dfl a) { return x * a; }
template <> __host__ __device__ inline dfl from_real<dfl>(double a) { return dfl(a); }
__device__ inline dfl absval(dfl x) { return fabs(x); }
__device__ inline dfl phase(dfl x) { return x.hi < 0.f ? dfl(-1) : dfl(1); }
__device__ inline dfl shfl_xor(dfl v, int o) {
  return {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
}

template <class Job>
static DBuf upload(tnfa_ctx* ctx, const std::vector<Job>& jobs) {
  DBuf d(ctx, jobs.size() * sizeof(Job));
  h2d(ctx, d.p, jobs.data(), jobs.size() * sizeof(Job));
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
  for (const auto& j : jobs)
    TNFA_CHECK(j.nd >= 1 && j.nd <= MAXD, TNFA_ERR_UNSUPPORTED, "permute: tensor order above 16");
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

// Loads and stores that bypass L1 (data shared between the CTAs of a
// cluster through L2).
__device__ inline double ldcg(const double* p) { return __ldcg(p); }
__device__ inline float ldcg(const float* p) { return __ldcg(p); }
__device__ inline cplx ldcg(const cplx* p) {
  const double2 v = __ldcg((const double2*)p);
  return {v.x, v.y};
}
__device__ inline void stcg(double* p, double v) { __stcg(p, v); }
__device__ inline void stcg(float* p, float v) { __stcg(p, v); }
__device__ inline void stcg(cplx* p, cplx v) { __stcg((double2*)p, make_double2(v.re, v.im)); }
__device__ inline dfl ldcg(const dfl* p) {
  const float2 v = __ldcg((const float2*)p);
  return {v.x, v.y};
}
__device__ inline void stcg(dfl* p, dfl v) { __stcg((float2*)p, make_float2(v.hi, v.lo)); }
__device__ inline float fmaT(float a, float b, float c) { return fmaf(a, b, c); }
__device__ inline double fmaT(double a, double b, double c) { return fma(a, b, c); }
__device__ inline cplx fmaT(cplx a, cplx b, cplx c) { return Sc<cplx>::fma(a, b, c); }
__device__ inline dfl fmaT(dfl a, dfl b, dfl c) { return a * b + c; }

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
//
// Columns are dealt round-robin to the CTAs of a cluster (CL; one CTA
// otherwise): the owner of column j builds reflector j in place, a barrier
// publishes it, and every CTA applies it to the columns it owns; Q is then
// formed column by column by the owners without further barriers.
template <bool CL>
__device__ inline void qsync() {
  if constexpr (CL)
    cg::this_cluster().sync();
  else
    __syncthreads();
}

template <class T, bool CL>
__global__ void __launch_bounds__(512) k_qr(const QrJob* __restrict__ jobs, T* __restrict__ work,
                                            const int64_t* __restrict__ woff) {
  int C = 1, crank = 0;
  if constexpr (CL) {
    C = (int)cg::this_cluster().num_blocks();
    crank = (int)cg::this_cluster().block_rank();
  }
  const int ji = blockIdx.x / C;
  const QrJob jb = jobs[ji];
  const int m = jb.m, n = jb.n, kq = min(m, n);
  T* W = work + woff[ji];
  T* Qw = W + (int64_t)m * n;
  T* alpha_g = Qw + (int64_t)m * kq;  // kq diagonal entries of R
  T* tau = (T*)jb.tau;
  const T* A = (const T*)jb.A;
  __shared__ T red[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t i = threadIdx.x; i < (int64_t)m * n; i += blockDim.x) {
    const int r = (int)(i / n), c = (int)(i % n);
    if (c % C == crank) W[(int64_t)c * m + r] = A[i];
  }
  __syncthreads();
  T* R = (T*)jb.R;
  for (int j = 0; j < kq; ++j) {
    T* x = W + (int64_t)j * m;
    if (j % C == crank) {
      double part = 0.0;
      for (int r = j + threadIdx.x; r < m; r += blockDim.x) part += abs2(x[r]);
      const double nrm2 = re(block_sum<T>(from_real<T>(part), red));
      if (threadIdx.x == 0) {
        const T x0 = x[j];
        const double nrm = sqrt(nrm2);
        if (!(nrm > 1e-150)) {
          // an (almost) eliminated column: no reflection.  A residue this
          // small (rounding left by earlier steps) would make 2 / |v|^2 overflow.
          stcg(tau + j, from_real<T>(0.0));
          stcg(alpha_g + j, x0);
        } else {
          const T alpha = scal(phase(x0), -nrm);
          const T v0 = x0 - alpha;
          const double vn2 = nrm2 - abs2(x0) + abs2(v0);
          stcg(tau + j, from_real<T>(vn2 > 0.0 ? 2.0 / vn2 : 0.0));
          stcg(x + j, v0);
          stcg(alpha_g + j, alpha);
        }
      }
    }
    qsync<CL>();
    const double beta = re(ldcg(tau + j));
    if (beta != 0.0) {
      // this CTA's columns c > j: c = crank + C * k
      const int c0 = j + 1 + ((crank - (j + 1)) % C + C) % C;
      for (int c = c0 + C * warp; c < n; c += C * nw) {
        T* y = W + (int64_t)c * m;
        T w = from_real<T>(0.0);
        for (int r = j + lane; r < m; r += 32) w = Sc<T>::fma(conj(ldcg(x + r)), y[r], w);
        w = warp_sum(w);
        const T bw = scal(w, beta);
        for (int r = j + lane; r < m; r += 32) y[r] = y[r] - ldcg(x + r) * bw;
      }
    }
    __syncthreads();
    // R row j: diagonal alpha, then the updated row j of this CTA's columns
    for (int c = crank + C * threadIdx.x; c < n; c += C * blockDim.x)
      R[(int64_t)j * n + c] = c < j ? from_real<T>(0.0) : (c == j ? ldcg(alpha_g + j) : W[(int64_t)c * m + j]);
  }
  // Q = H_0 ... H_{kq-1} [I; 0], columns owned as above
  for (int c = crank + C * warp; c < kq; c += C * nw) {
    T* y = Qw + (int64_t)c * m;
    for (int r = lane; r < m; r += 32) y[r] = from_real<T>(r == c ? 1.0 : 0.0);
  }
  __syncthreads();
  for (int j = kq - 1; j >= 0; --j) {
    const double beta = re(ldcg(tau + j));
    if (beta == 0.0) continue;
    const T* x = W + (int64_t)j * m;
    // a column stays with one warp for all j (no barrier between the j)
    for (int c = crank + C * warp; c < kq; c += C * nw) {
      if (c < j) continue;
      T* y = Qw + (int64_t)c * m;
      T w = from_real<T>(0.0);
      for (int r = j + lane; r < m; r += 32) w = Sc<T>::fma(conj(ldcg(x + r)), y[r], w);
      w = warp_sum(w);
      const T bw = scal(w, beta);
      for (int r = j + lane; r < m; r += 32) y[r] = y[r] - ldcg(x + r) * bw;
    }
  }
  __syncthreads();
  T* Q = (T*)jb.Q;
  for (int64_t i = threadIdx.x; i < (int64_t)m * kq; i += blockDim.x) {
    const int r = (int)(i / kq), c = (int)(i % kq);
    if (c % C == crank) Q[i] = Qw[(int64_t)c * m + r];
  }
}

constexpr int QR_CLUSTER = 8;

template <class T>
void qr(tnfa_ctx* ctx, const std::vector<QrJob>& jobs) {
  if (jobs.empty()) return;
  std::vector<QrJob> big, small;
  // clusters for large factorisations, and for every job of at least 32
  // columns when the batch is too small to fill the GPU (see svd_big)
  const bool few = jobs.size() * 8 <= (size_t)ctx->sm_count;
  for (const auto& j : jobs)
    (((double)j.m * j.n * std::min(j.m, j.n) >= 4.0e6 && std::min(j.m, j.n) >= 64) ||
             (few && std::min(j.m, j.n) >= 32)
         ? big
         : small)
        .push_back(j);
  for (int pass = 0; pass < 2; ++pass) {
    const std::vector<QrJob>& js = pass == 0 ? big : small;
    if (js.empty()) continue;
    std::vector<int64_t> woff(js.size() + 1, 0);
    double fl = 0;
    for (size_t i = 0; i < js.size(); ++i) {
      const int64_t m = js[i].m, n = js[i].n, k = std::min(m, n);
      // W, Qw, the k diagonal entries of R
      woff[i + 1] = woff[i] + m * n + m * k + k;
      fl += 4.0 * m * n * k;
    }
    DBuf work(ctx, (size_t)woff.back() * sizeof(T));
    DBuf dw = upload(ctx, woff);
    DBuf d = upload(ctx, js);
    KernelScope ks(ctx, sizeof(T) == 8 ? "qr_f64" : "qr_c128", fl, 0.0);
    if (trace_on()) ks.note = (pass == 0 ? "cluster " : "single ") + size_note(js);
    if (pass == 0) {
      cudaLaunchConfig_t cfg{};
      cfg.gridDim = dim3((unsigned)(js.size() * QR_CLUSTER));
      cfg.blockDim = dim3(512);
      cfg.stream = ctx->stream;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = QR_CLUSTER;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      TNFA_CUDA(cudaLaunchKernelEx(&cfg, k_qr<T, true>, (const QrJob*)d.as<QrJob>(), work.as<T>(),
                                   (const int64_t*)dw.as<int64_t>()));
    } else {
      k_qr<T, false><<<(unsigned)js.size(), 512, 0, ctx->stream>>>(d.as<QrJob>(), work.as<T>(),
                                                                  dw.as<int64_t>());
    }
    TNFA_LAUNCH_CHECK();
  }
}

// ------------------------------------------------------------- qr_rank --
// Householder QR with column pivoting that stops once the columns left over
// hold no more than tol^2 of the matrix's squared Frobenius norm: A ~= Q R
// with Q (m x r, orthonormal) and R (r x n) in A's own column order, r the
// numerical rank.  Step j reflects the remaining column of largest norm;
// columns never move (each stays with the CTA that owns it), so R row j holds
// alpha_j at the pivot column, the reflected row j at the columns not yet
// pivoted and zeros at the earlier pivots.  The column norms below the
// current row are recomputed exactly while each column is reflected.  In a
// cluster every CTA posts its best column and its share of the remaining
// norm to a slot in global memory; all CTAs reduce the slots in the same
// order, so they take identical pivot and stop decisions.
//
// Workspace: W (m*n) + Qw (m*kq) + alpha (kq) in T as for k_qr; in doubles
// the column norms (n; -1 marks a pivoted column) and 2 x C slots of
// (best norm, its column, remaining norm).
constexpr int QRCP_MAXK = 1024;

__device__ inline void block_argmax_sum(double& best, int& idx, double& sum, double* sb, int* si,
                                        double* ss) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o; o >>= 1) {
    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
    sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (ob > best || (ob == best && oi < idx)) {
      best = ob;
      idx = oi;
    }
  }
  __syncthreads();
  if (lane == 0) {
    sb[warp] = best;
    si[warp] = idx;
    ss[warp] = sum;
  }
  __syncthreads();
  if (warp == 0) {
    best = lane < nw ? sb[lane] : -1.0;
    idx = lane < nw ? si[lane] : INT_MAX;
    sum = lane < nw ? ss[lane] : 0.0;
    for (int o = 16; o; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
      sum += __shfl_xor_sync(0xffffffffu, sum, o);
      if (ob > best || (ob == best && oi < idx)) {
        best = ob;
        idx = oi;
      }
    }
    if (lane == 0) {
      sb[0] = best;
      si[0] = idx;
      ss[0] = sum;
    }
  }
  __syncthreads();
  best = sb[0];
  idx = si[0];
  sum = ss[0];
  __syncthreads();
}

template <class T, bool CL>
__global__ void __launch_bounds__(512) k_qrcp(const QrJob* __restrict__ jobs, T* __restrict__ work,
                                              const int64_t* __restrict__ woff, double* __restrict__ dwork,
                                              const int64_t* __restrict__ doff, double tol2,
                                              int* __restrict__ ranks) {
  int C = 1, crank = 0;
  if constexpr (CL) {
    C = (int)cg::this_cluster().num_blocks();
    crank = (int)cg::this_cluster().block_rank();
  }
  const int ji = blockIdx.x / C;
  const QrJob jb = jobs[ji];
  const int m = jb.m, n = jb.n, kq = min(m, n);
  T* W = work + woff[ji];
  T* Qw = W + (int64_t)m * n;
  T* alpha_g = Qw + (int64_t)m * kq;
  T* tau = (T*)jb.tau;
  double* nrm = dwork + doff[ji];
  double* slot = nrm + n;  // [2][C][3]
  const T* A = (const T*)jb.A;
  __shared__ T red[32];
  __shared__ double sb[32], ss[32];
  __shared__ int si[32];
  __shared__ int piv[QRCP_MAXK];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t i = threadIdx.x; i < (int64_t)m * n; i += blockDim.x) {
    const int r = (int)(i / n), c = (int)(i % n);
    if (c % C == crank) W[(int64_t)c * m + r] = A[i];
  }
  __syncthreads();
  for (int c = crank + C * warp; c < n; c += C * nw) {
    const T* y = W + (int64_t)c * m;
    double s = 0.0;
    for (int r = lane; r < m; r += 32) s += abs2(y[r]);
    s = warp_sum(s);
    if (lane == 0) nrm[c] = s;
  }
  __syncthreads();
  double total;
  {
    double part = 0.0;
    for (int c = crank + C * threadIdx.x; c < n; c += C * blockDim.x) part += nrm[c];
    double b = -1.0;
    int bi = INT_MAX;
    block_argmax_sum(b, bi, part, sb, si, ss);
    if (threadIdx.x == 0) stcg(slot + crank, part);
    qsync<CL>();
    total = 0.0;
    for (int i = 0; i < C; ++i) total += ldcg(slot + i);
    qsync<CL>();
  }
  const double thr = tol2 * total;
  T* R = (T*)jb.R;
  int r_keep = kq;
  for (int j = 0; j < kq; ++j) {
    double best = -1.0, sum = 0.0;
    int bi = INT_MAX;
    for (int c = crank + C * threadIdx.x; c < n; c += C * blockDim.x) {
      const double v = nrm[c];
      if (v >= 0.0) {
        sum += v;
        if (v > best || (v == best && c < bi)) {
          best = v;
          bi = c;
        }
      }
    }
    block_argmax_sum(best, bi, sum, sb, si, ss);
    double* my = slot + ((int64_t)(j & 1) * C + crank) * 3;
    if (threadIdx.x == 0) {
      stcg(my, best);
      stcg(my + 1, (double)bi);
      stcg(my + 2, sum);
    }
    qsync<CL>();
    double gbest = -1.0, gsum = 0.0;
    int p = INT_MAX;
    for (int i = 0; i < C; ++i) {
      const double* o = slot + ((int64_t)(j & 1) * C + i) * 3;
      const double ob = ldcg(o);
      const int oi = (int)ldcg(o + 1);
      gsum += ldcg(o + 2);
      if (ob > gbest || (ob == gbest && oi < p)) {
        gbest = ob;
        p = oi;
      }
    }
    if (p >= n || (j > 0 && (gsum <= thr || !(gbest > 0.0)))) {
      r_keep = j;  // 0 only when no column has a finite norm
      break;
    }
    if (threadIdx.x == 0) piv[j] = p;
    T* x = W + (int64_t)p * m;
    if (p % C == crank) {
      double part = 0.0;
      for (int r = j + threadIdx.x; r < m; r += blockDim.x) part += abs2(x[r]);
      const double nrm2 = re(block_sum<T>(from_real<T>(part), red));
      if (threadIdx.x == 0) {
        const T x0 = x[j];
        const double nv = sqrt(nrm2);
        if (!(nv > 1e-150)) {
          stcg(tau + j, from_real<T>(0.0));
          stcg(alpha_g + j, x0);
        } else {
          const T alpha = scal(phase(x0), -nv);
          const T v0 = x0 - alpha;
          const double vn2 = nrm2 - abs2(x0) + abs2(v0);
          stcg(tau + j, from_real<T>(vn2 > 0.0 ? 2.0 / vn2 : 0.0));
          stcg(x + j, v0);
          stcg(alpha_g + j, alpha);
        }
        nrm[p] = -1.0;
      }
    }
    qsync<CL>();
    const double beta = re(ldcg(tau + j));
    for (int c = crank + C * warp; c < n; c += C * nw) {
      if (nrm[c] < 0.0) continue;  // pivoted earlier (or now, by this CTA)
      T* y = W + (int64_t)c * m;
      double s = 0.0;
      if (beta != 0.0) {
        T w = from_real<T>(0.0);
        for (int r = j + lane; r < m; r += 32) w = Sc<T>::fma(conj(ldcg(x + r)), y[r], w);
        w = warp_sum(w);
        const T bw = scal(w, beta);
        for (int r = j + lane; r < m; r += 32) {
          const T v = y[r] - ldcg(x + r) * bw;
          y[r] = v;
          if (r > j) s += abs2(v);
        }
      } else {
        for (int r = j + 1 + lane; r < m; r += 32) s += abs2(y[r]);
      }
      s = warp_sum(s);
      if (lane == 0) nrm[c] = s;
    }
    __syncthreads();
    const T aj = ldcg(alpha_g + j);
    for (int c = crank + C * threadIdx.x; c < n; c += C * blockDim.x)
      R[(int64_t)j * n + c] = c == p ? aj : (nrm[c] >= 0.0 ? W[(int64_t)c * m + j] : from_real<T>(0.0));
  }
  __syncthreads();
  // Q = H_0 ... H_{r-1} [I; 0] (m x r), columns owned round-robin
  for (int c = crank + C * warp; c < r_keep; c += C * nw) {
    T* y = Qw + (int64_t)c * m;
    for (int r = lane; r < m; r += 32) y[r] = from_real<T>(r == c ? 1.0 : 0.0);
  }
  __syncthreads();
  for (int j = r_keep - 1; j >= 0; --j) {
    const double beta = re(ldcg(tau + j));
    if (beta == 0.0) continue;
    const T* x = W + (int64_t)piv[j] * m;
    for (int c = crank + C * warp; c < r_keep; c += C * nw) {
      if (c < j) continue;
      T* y = Qw + (int64_t)c * m;
      T w = from_real<T>(0.0);
      for (int r = j + lane; r < m; r += 32) w = Sc<T>::fma(conj(ldcg(x + r)), y[r], w);
      w = warp_sum(w);
      const T bw = scal(w, beta);
      for (int r = j + lane; r < m; r += 32) y[r] = y[r] - ldcg(x + r) * bw;
    }
  }
  __syncthreads();
  T* Q = (T*)jb.Q;
  for (int64_t i = threadIdx.x; i < (int64_t)m * r_keep; i += blockDim.x) {
    const int r = (int)(i / r_keep), c = (int)(i % r_keep);
    if (c % C == crank) Q[i] = Qw[(int64_t)c * m + r];
  }
  if (crank == 0 && threadIdx.x == 0) ranks[ji] = r_keep;
}

template <class T>
void qr_rank(tnfa_ctx* ctx, const std::vector<QrJob>& jobs, double tol, std::vector<int>& ranks) {
  ranks.assign(jobs.size(), 0);
  if (jobs.empty()) return;
  std::vector<size_t> big, small;
  const bool few = jobs.size() * 8 <= (size_t)ctx->sm_count;
  for (size_t i = 0; i < jobs.size(); ++i) {
    const QrJob& j = jobs[i];
    TNFA_CHECK(std::min(j.m, j.n) <= QRCP_MAXK, TNFA_ERR_UNSUPPORTED,
               "rank-revealing QR handles at most 1024 reflectors");
    (((double)j.m * j.n * std::min(j.m, j.n) >= 4.0e6 && std::min(j.m, j.n) >= 64) ||
             (few && std::min(j.m, j.n) >= 32)
         ? big
         : small)
        .push_back(i);
  }
  // ranks of the cluster launch first, then of the single-CTA launch
  DBuf rk(ctx, jobs.size() * sizeof(int));
  for (int pass = 0; pass < 2; ++pass) {
    const std::vector<size_t>& idx = pass == 0 ? big : small;
    if (idx.empty()) continue;
    const int C = pass == 0 ? QR_CLUSTER : 1;
    int* rl = rk.as<int>() + (pass == 0 ? 0 : big.size());
    std::vector<QrJob> js;
    std::vector<int64_t> woff(idx.size() + 1, 0), doff(idx.size() + 1, 0);
    double fl = 0;
    for (size_t i = 0; i < idx.size(); ++i) {
      js.push_back(jobs[idx[i]]);
      const int64_t m = js[i].m, n = js[i].n, k = std::min(m, n);
      woff[i + 1] = woff[i] + m * n + m * k + k;
      doff[i + 1] = doff[i] + n + 6 * C;
      fl += 4.0 * m * n * k;
    }
    DBuf work(ctx, (size_t)woff.back() * sizeof(T));
    DBuf dwork(ctx, (size_t)doff.back() * sizeof(double));
    DBuf dw = upload(ctx, woff);
    DBuf dd = upload(ctx, doff);
    DBuf d = upload(ctx, js);
    KernelScope ks(ctx, sizeof(T) == 8 ? "qr_rank_f64" : "qr_rank_c128", fl, 0.0);
    if (trace_on()) ks.note = (pass == 0 ? "cluster " : "single ") + size_note(js);
    if (pass == 0) {
      cudaLaunchConfig_t cfg{};
      cfg.gridDim = dim3((unsigned)(js.size() * QR_CLUSTER));
      cfg.blockDim = dim3(512);
      cfg.stream = ctx->stream;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = QR_CLUSTER;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      TNFA_CUDA(cudaLaunchKernelEx(&cfg, k_qrcp<T, true>, (const QrJob*)d.as<QrJob>(), work.as<T>(),
                                   (const int64_t*)dw.as<int64_t>(), dwork.as<double>(),
                                   (const int64_t*)dd.as<int64_t>(), tol * tol, rl));
    } else {
      k_qrcp<T, false><<<(unsigned)js.size(), 512, 0, ctx->stream>>>(
          d.as<QrJob>(), work.as<T>(), dw.as<int64_t>(), dwork.as<double>(), dd.as<int64_t>(), tol * tol,
          rl);
    }
    TNFA_LAUNCH_CHECK();
  }
  std::vector<int> h(jobs.size());
  TNFA_CUDA(cudaMemcpyAsync(h.data(), rk.p, jobs.size() * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  for (size_t i = 0; i < big.size(); ++i) ranks[big[i]] = h[i];
  for (size_t i = 0; i < small.size(); ++i) ranks[small[i]] = h[big.size() + i];
  for (int r : ranks)
    TNFA_CHECK(r >= 1, TNFA_ERR_DOMAIN, "rank-revealing QR: no column with a finite norm (NaN or Inf input)");
  if (trace_on()) {
    long sr = 0, sk = 0, mx_m = 0, mx_n = 0, mx_r = 0;
    for (size_t i = 0; i < jobs.size(); ++i) {
      sr += ranks[i];
      sk += std::min(jobs[i].m, jobs[i].n);
      mx_m = std::max<long>(mx_m, jobs[i].m);
      mx_n = std::max<long>(mx_n, jobs[i].n);
      mx_r = std::max<long>(mx_r, ranks[i]);
    }
    char b[200];
    snprintf(b, sizeof b, "qr_rank ranks jobs=%zu sum_r=%ld sum_minmn=%ld max_m=%ld max_n=%ld max_r=%ld",
             jobs.size(), sr, sk, mx_m, mx_n, mx_r);
    trace_line(b);
  }
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

// One-sided (Hestenes) Jacobi: rotate column pairs (p, q) of U until every
// pair is orthogonal to tol = 8 sqrt(m) eps relative to |u_p| |u_q|; the
// singular values are the final column norms.  Round-robin pairing: the n/2
// pairs of a round are disjoint, so the warps of a round run them in
// parallel.  The columns live in global memory (L2-resident; loads and
// stores bypass L1); with MAXR > 0 each lane keeps its MAXR elements of the
// two columns in registers between the dot products and the rotation.
//
// CL: the job is spread over a thread-block cluster -- the warps of all its
// CTAs share the pairs of a round and a cluster barrier (release / acquire at
// cluster scope) separates the rounds.  The stop decision of a sweep is read
// by every CTA from one global flag after the sweep's last barrier, so all
// CTAs leave the loop together; flag k % 3 is cleared two sweeps before it is
// reused, after every CTA has read it.
//
// A sweep ends the iteration when no pair had |g| > stop sqrt(a b) with
// stop = max(tol, stop_rel): Jacobi converges quadratically near the end, so
// after a sweep whose rotations were all below ~1e-10 the next one would
// change nothing above rounding.
//
// Deflation (small_rel > 0): a pair whose columns both weigh less than
// small_rel |A|_F^2 / n is skipped.  The columns above that bound end up
// orthogonal to each other and to the rest, so their norms are singular
// values and the rest spans the complementary subspace with a known total
// weight below small_rel |A|_F^2; a truncation whose budget exceeds that
// drops all of it, and decides exactly like on the full decomposition.
template <class T> struct RealOf { using type = double; };
template <> struct RealOf<float> { using type = float; };
template <> struct RealOf<dfl> { using type = dfl; };

// Per arithmetic: unit roundoff, the weight (relative to |A|_F^2) below which
// a column is rounding noise, and the largest |zeta| handled directly.
template <class R> struct JacobiTraits {
  static constexpr double eps = 2.220446049250313e-16, negl = 1e-30, big = 1e150;
};
template <> struct JacobiTraits<float> {
  static constexpr double eps = 1.1920929e-7, negl = 1e-13, big = 1e18;
};
template <> struct JacobiTraits<dfl> {  // 2^-46: the pair arithmetic's error with some margin
  static constexpr double eps = 1.4210854715202004e-14, negl = 1e-26, big = 1e18;
};

struct JacobiOpts {
  double stop_rel;   // sweep-level stop threshold (relative |g| / sqrt(a b))
  double small_rel;  // deflation bound (relative to |A|_F^2 / n); 0: none
};



template <bool CL>
__device__ inline void jsync() {
  if constexpr (CL)
    cg::this_cluster().sync();
  else
    __syncthreads();
}

template <class T, bool CL, int MAXR>
__global__ void __launch_bounds__(512) k_jacobi(const SvdJob* __restrict__ jobs, T* __restrict__ work,
                                                const int64_t* __restrict__ woff, int* __restrict__ flags,
                                                int max_sweeps, JacobiOpts opt) {
  using R = typename RealOf<T>::type;
  int C = 1, crank = 0;
  if constexpr (CL) {
    C = (int)cg::this_cluster().num_blocks();
    crank = (int)cg::this_cluster().block_rank();
  }
  const int ji = blockIdx.x / C;
  const SvdJob jb = jobs[ji];
  const int m = jb.m, n = jb.n;
  const bool want_v = jb.V != nullptr;
  T* U = work + woff[ji];  // column-major m x n
  T* V = U + (int64_t)m * n;  // column-major n x n (when wanted)
  // sig (n doubles) starts on an 8-byte boundary (job bases are 16-byte
  // aligned; for 4-byte T the offset is rounded up to an even count)
  constexpr int64_t al = sizeof(T) >= 8 ? 1 : 8 / sizeof(T);
  const int64_t soff = ((int64_t)m * n + (want_v ? (int64_t)n * n : 0) + al - 1) / al * al;
  double* sig = (double*)(U + soff);
  int* rank = (int*)(sig + n);
  int* flag = flags + 3 * ji;
  const T* A = (const T*)jb.A;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int64_t gt = (int64_t)crank * blockDim.x + threadIdx.x, gs = (int64_t)C * blockDim.x;
  for (int64_t i = gt; i < (int64_t)m * n; i += gs) {
    const int r = (int)(i / n), c = (int)(i % n);
    stcg(U + (int64_t)c * m + r, A[i]);
  }
  if (want_v)
    for (int64_t i = gt; i < (int64_t)n * n; i += gs)
      stcg(V + i, from_real<T>((i / n) == (i % n) ? 1.0 : 0.0));
  __shared__ double red[32];
  double part = 0.0;
  for (int64_t i = threadIdx.x; i < (int64_t)m * n; i += blockDim.x) part += (double)abs2(A[i]);
  const double fro2 = block_sum<double>(part, red);
  const double eps = JacobiTraits<R>::eps;
  // columns below this are rounding noise of the whole matrix
  const double negl = JacobiTraits<R>::negl * fro2;
  const R tol = (R)(8.0 * sqrt((double)m) * eps);
  const R stop = (R)fmax((double)tol, opt.stop_rel);
  // pairs of columns both below this are left alone (deflation for truncation)
  const double small = opt.small_rel * fro2 / n;
  const int n2 = (n + 1) & ~1;
  const int gw = crank * nw + warp, nwc = C * nw;
  int sweep = 0;
  bool converged = (n < 2);
  jsync<CL>();
  while (!converged && sweep < max_sweeps) {
    if (crank == 0 && threadIdx.x == 0) flag[(sweep + 1) % 3] = 0;
    int busy = 0;
    for (int r = 0; r < n2 - 1; ++r) {
      for (int slot = gw; slot < n2 / 2; slot += nwc) {
        int p, q;
        rr_pair(n2, r, slot, p, q);
        if (q >= n) continue;
        T* up = U + (int64_t)p * m;
        T* uq = U + (int64_t)q * m;
        R a = 0, b = 0;
        T g = from_real<T>(0.0);
        T xp[MAXR > 0 ? MAXR : 1], xq[MAXR > 0 ? MAXR : 1];
        if constexpr (MAXR > 0) {
#pragma unroll
          for (int k = 0; k < MAXR; ++k) {
            const int i = lane + 32 * k;
            xp[k] = i < m ? ldcg(up + i) : from_real<T>(0.0);
            xq[k] = i < m ? ldcg(uq + i) : from_real<T>(0.0);
            a += abs2(xp[k]);
            b += abs2(xq[k]);
            g = fmaT(conj(xp[k]), xq[k], g);
          }
        } else {
          for (int i = lane; i < m; i += 32) {
            const T x = ldcg(up + i), y = ldcg(uq + i);
            a += abs2(x);
            b += abs2(y);
            g = fmaT(conj(x), y, g);
          }
        }
        a = warp_sum(a);
        b = warp_sum(b);
        g = warp_sum(g);
        const R ag = absval(g);  // |g| without squaring (|g|^2 underflows at small scales)
        // a negligible column carries no singular value worth orthogonalising
        // against; skipping it also avoids zeta^2 overflow on extreme ratios
        if ((double)a < negl || (double)b < negl) continue;
        if ((double)a < small && (double)b < small) continue;
        const R nab = sqrt(a) * sqrt(b);
        if (ag > stop * nab) busy = 1;
        if (ag <= tol * nab || ag == (R)0) continue;
        const R zeta = (b - a) / ((R)2 * ag);
        const R big = (R)JacobiTraits<R>::big;
        const R t = fabs(zeta) > big ? (R)0.5 / zeta
                                     : (zeta >= 0 ? (R)1 : (R)-1) / (fabs(zeta) + sqrt((R)1 + zeta * zeta));
        if (t == (R)0) continue;
        const R c = (R)1 / sqrt((R)1 + t * t), sn = c * t;
        const T e = phase(g);  // g / |g|
        const T se = scal(e, sn), sec = scal(conj(e), sn);
        if constexpr (MAXR > 0) {
#pragma unroll
          for (int k = 0; k < MAXR; ++k) {
            const int i = lane + 32 * k;
            if (i < m) {
              stcg(up + i, scal(xp[k], c) - sec * xq[k]);
              stcg(uq + i, se * xp[k] + scal(xq[k], c));
            }
          }
        } else {
          for (int i = lane; i < m; i += 32) {
            const T x = ldcg(up + i), y = ldcg(uq + i);
            stcg(up + i, scal(x, c) - sec * y);
            stcg(uq + i, se * x + scal(y, c));
          }
        }
        if (want_v) {
          T* vp = V + (int64_t)p * n;
          T* vq = V + (int64_t)q * n;
          for (int i = lane; i < n; i += 32) {
            const T x = ldcg(vp + i), y = ldcg(vq + i);
            stcg(vp + i, scal(x, c) - sec * y);
            stcg(vq + i, se * x + scal(y, c));
          }
        }
      }
      jsync<CL>();
    }
    if (busy && lane == 0) atomicOr(flag + sweep % 3, 1);
    jsync<CL>();
    converged = (__ldcg(flag + sweep % 3) == 0);
    ++sweep;
  }
  // singular values, ranks (descending, stable), normalised outputs
  for (int c = gw; c < n; c += nwc) {
    double s2 = 0.0;
    for (int i = lane; i < m; i += 32) s2 += (double)abs2(ldcg(U + (int64_t)c * m + i));
    s2 = warp_sum(s2);
    if (lane == 0) __stcg(sig + c, sqrt(s2));
  }
  jsync<CL>();
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
  jsync<CL>();
  T* Uo = (T*)jb.U;
  for (int64_t i = gt; i < (int64_t)m * n; i += gs) {
    const int c = (int)(i / m), r = (int)(i % m);
    const double sc = __ldcg(sig + c);
    // a negligible column was never orthogonalised: it leaves U as zeros
    Uo[(int64_t)r * n + __ldcg(rank + c)] =
        sc * sc > negl && sc > 0 ? scal(ldcg(U + i), (R)(1.0 / sc)) : from_real<T>(0.0);
  }
  if (want_v) {
    T* Vo = (T*)jb.V;
    for (int64_t i = gt; i < (int64_t)n * n; i += gs) {
      const int c = (int)(i / n), r = (int)(i % n);
      Vo[(int64_t)r * n + __ldcg(rank + c)] = ldcg(V + i);
    }
  }
  if (crank == 0 && threadIdx.x == 0 && jb.sweeps) *jb.sweeps = converged ? sweep : -1;
}

constexpr int SVD_CLUSTER = 8;  // CTAs (SMs) per large matrix

// A job goes to the cluster kernel when its Jacobi work is large enough to
// pay for a cluster barrier per round -- or, in a batch too small to fill the
// GPU with one CTA per job (the tail of an uneven batch), when it has enough
// column pairs to share between the CTAs of a cluster.
inline bool svd_big(const SvdJob& j, size_t njobs, int sms) {
  if (j.n >= 96 && (double)j.m * j.n * j.n >= 2.0e6) return true;
  return njobs * 8 <= (size_t)sms && j.n >= 32;
}

template <class T, bool CL, int MAXR>
void launch_jacobi(tnfa_ctx* ctx, const SvdJob* d, T* work, const int64_t* woff, int* flags, int njobs,
                   int max_sweeps, JacobiOpts stop_rel) {
  if constexpr (CL) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)(njobs * SVD_CLUSTER));
    cfg.blockDim = dim3(512);
    cfg.stream = ctx->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = SVD_CLUSTER;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    TNFA_CUDA(cudaLaunchKernelEx(&cfg, k_jacobi<T, true, MAXR>, d, work, woff, flags, max_sweeps, stop_rel));
  } else {
    k_jacobi<T, false, MAXR><<<(unsigned)njobs, 512, 0, ctx->stream>>>(d, work, woff, flags, max_sweeps,
                                                                       stop_rel);
  }
  TNFA_LAUNCH_CHECK();
}

// Registers per lane and column kept by the Jacobi kernels (0: reload).
template <class T> constexpr int jacobi_maxr() { return sizeof(T) == 16 ? 8 : 16; }

template <class T>
void jacobi(tnfa_ctx* ctx, const std::vector<SvdJob>& jobs, int max_sweeps, JacobiOpts stop_rel,
            const char* family) {
  if (ctx->jacobi_sweep_cap > 0) max_sweeps = std::min(max_sweeps, ctx->jacobi_sweep_cap);
  std::vector<SvdJob> big, small;
  for (const auto& j : jobs) (svd_big(j, jobs.size(), ctx->sm_count) ? big : small).push_back(j);
  for (int pass = 0; pass < 2; ++pass) {
    const std::vector<SvdJob>& js = pass == 0 ? big : small;
    if (js.empty()) continue;
    std::vector<int64_t> woff(js.size() + 1, 0);
    double fl = 0;
    int maxm = 0;
    for (size_t i = 0; i < js.size(); ++i) {
      TNFA_CHECK(js[i].m >= js[i].n, TNFA_ERR_INVALID_ARGUMENT, "svd needs m >= n");
      const int64_t m = js[i].m, n = js[i].n;
      maxm = std::max(maxm, js[i].m);
      // U (and V) in T; sig (n doubles) and rank (n ints) rounded up to T
      // slots, with slack for aligning sig; every job base 16-byte aligned
      const int64_t al = (int64_t)(16 / sizeof(T) > 0 ? 16 / sizeof(T) : 1);
      const int64_t need = m * n + (js[i].V ? n * n : 0) + (int64_t)((n * 12 + sizeof(T) - 1) / sizeof(T)) + 4;
      woff[i + 1] = woff[i] + (need + al - 1) / al * al;
      fl += 5.0 * m * n * n * 8;  // ~8 sweeps of 3 dots + 2 rotations per pair
    }
    DBuf work(ctx, (size_t)woff.back() * sizeof(T));
    DBuf dw = upload(ctx, woff);
    DBuf d = upload(ctx, js);
    DBuf flags(ctx, js.size() * 3 * sizeof(int));
    TNFA_CUDA(cudaMemsetAsync(flags.p, 0, js.size() * 3 * sizeof(int), ctx->stream));
    KernelScope ks(ctx, family, fl, 0.0);
    if (trace_on()) ks.note = (pass == 0 ? "cluster " : "single ") + size_note(js);
    const int need = (maxm + 31) / 32;  // column elements per lane
    const SvdJob* dj = d.as<SvdJob>();
    const int nj = (int)js.size();
    T* w = work.as<T>();
    const int64_t* wo = dw.as<int64_t>();
    int* fl_ = flags.as<int>();
    if (pass == 0) {
      if (need <= 4)
        launch_jacobi<T, true, 4>(ctx, dj, w, wo, fl_, nj, max_sweeps, stop_rel);
      else if (need <= jacobi_maxr<T>())
        launch_jacobi<T, true, jacobi_maxr<T>()>(ctx, dj, w, wo, fl_, nj, max_sweeps, stop_rel);
      else
        launch_jacobi<T, true, 0>(ctx, dj, w, wo, fl_, nj, max_sweeps, stop_rel);
    } else {
      if (need <= 4)
        launch_jacobi<T, false, 4>(ctx, dj, w, wo, fl_, nj, max_sweeps, stop_rel);
      else if (need <= jacobi_maxr<T>())
        launch_jacobi<T, false, jacobi_maxr<T>()>(ctx, dj, w, wo, fl_, nj, max_sweeps, stop_rel);
      else
        launch_jacobi<T, false, 0>(ctx, dj, w, wo, fl_, nj, max_sweeps, stop_rel);
    }
  }
  if (trace_on()) trace_sweeps(ctx, jobs);
  // Diagnostics: with TNFA_DEBUG_DIR set, the input of every Jacobi job that
  // hit the sweep cap (or, with TNFA_DEBUG_SWEEPS=k, took k sweeps or more) is
  // written there: int32 m, n, element size, sweeps, then the matrix.
  static const char* dbg = getenv("TNFA_DEBUG_DIR");
  static const int thr = getenv("TNFA_DEBUG_SWEEPS") ? atoi(getenv("TNFA_DEBUG_SWEEPS")) : 0;
  if (dbg && *dbg) {
    static int counter = 0;
    for (const auto& j : jobs) {
      if (!j.sweeps) continue;
      int sw = 0;
      TNFA_CUDA(cudaMemcpyAsync(&sw, j.sweeps, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
      if (sw >= 0 && !(thr > 0 && sw >= thr)) continue;
      if (counter >= 64) break;
      std::vector<T> h((size_t)j.m * j.n);
      TNFA_CUDA(cudaMemcpyAsync(h.data(), j.A, h.size() * sizeof(T), cudaMemcpyDeviceToHost,
                                ctx->stream));
      TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
      char path[1024];
      snprintf(path, sizeof path, "%s/jacobi_%s_%d.bin", dbg, family, counter++);
      if (FILE* fp = fopen(path, "wb")) {
        int hdr[4] = {j.m, j.n, (int)sizeof(T), sw};
        fwrite(hdr, sizeof(int), 4, fp);
        fwrite(h.data(), sizeof(T), h.size(), fp);
        fclose(fp);
      }
    }
  }
}


// ------------------------------------------------------------------ lu --
constexpr int LU_NB = 32;

// Factor columns k..k+kb-1 (rows k..n-1); row swaps inside the panel only.
// For each column the pivot row's panel segment goes to shared memory and
// every thread loads the whole panel segment of each of its rows at once
// (LU_NB independent loads), so a column step costs one memory latency per
// row a thread owns rather than one per entry.
__global__ void __launch_bounds__(256) k_lu_panel(double* A, int n, int k, int kb, int* piv,
                                                  int* singular) {
  __shared__ double vmax[32];
  __shared__ int imax[32];
  __shared__ int p_sh;
  __shared__ double prow[LU_NB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int jj = 0; jj < kb; ++jj) {
    const int j = k + jj;
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
      double bb = -1.0;
      int i = j;
      for (int w = 0; w < nw; ++w)
        if (vmax[w] > bb || (vmax[w] == bb && imax[w] < i)) {
          bb = vmax[w];
          i = imax[w];
        }
      p_sh = i;
      piv[j] = i;
      if (!(bb > 0.0)) *singular = 1;
    }
    __syncthreads();
    const int p = p_sh;
    if (threadIdx.x < kb) {
      const int c = k + threadIdx.x;
      const double tj = A[(int64_t)j * n + c], tp = A[(int64_t)p * n + c];
      if (p != j) {
        A[(int64_t)j * n + c] = tp;
        A[(int64_t)p * n + c] = tj;
      }
      prow[threadIdx.x] = tp;
    }
    __syncthreads();
    const double d = prow[jj];
    if (d != 0.0) {
      for (int r = j + 1 + threadIdx.x; r < n; r += blockDim.x) {
        double* row = A + (int64_t)r * n + k;
        double v[LU_NB];
#pragma unroll
        for (int c = 0; c < LU_NB; ++c) v[c] = (c >= jj && c < kb) ? row[c] : 0.0;
        double vj = 0.0;  // v[jj] by selection, so that v stays in registers
#pragma unroll
        for (int c = 0; c < LU_NB; ++c) vj = c == jj ? v[c] : vj;
        const double l = vj / d;
#pragma unroll
        for (int c = 0; c < LU_NB; ++c)
          if (c > jj && c < kb) row[c] = v[c] - l * prow[c];
        row[jj] = l;
      }
    }
    __syncthreads();
  }
}

// The same panel factorisation with the panel (rows k..n-1, kb columns) held
// in shared memory, row stride kb + 1 doubles: one read and one write-back of
// the panel, every column step in shared memory.  1024 threads.
__global__ void __launch_bounds__(1024) k_lu_panel_smem(double* A, int n, int k, int kb, int* piv,
                                                        int* singular) {
  extern __shared__ __align__(16) double P[];
  __shared__ double vmax[32];
  __shared__ int imax[32];
  __shared__ int p_sh;
  const int rows = n - k, ld = kb + 1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i = threadIdx.x; i < rows * kb; i += blockDim.x) {
    const int r = i / kb, c = i - r * kb;
    P[r * ld + c] = A[(int64_t)(k + r) * n + k + c];
  }
  __syncthreads();
  for (int jj = 0; jj < kb; ++jj) {
    double best = -1.0;
    int bi = jj;
    for (int r = jj + threadIdx.x; r < rows; r += blockDim.x) {
      const double a = fabs(P[r * ld + jj]);
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
      double bb = -1.0;
      int i = jj;
      for (int w = 0; w < nw; ++w)
        if (vmax[w] > bb || (vmax[w] == bb && imax[w] < i)) {
          bb = vmax[w];
          i = imax[w];
        }
      p_sh = i;
      piv[k + jj] = k + i;
      if (!(bb > 0.0)) *singular = 1;
    }
    __syncthreads();
    const int pr = p_sh;
    if (pr != jj && threadIdx.x < kb) {
      const double t = P[jj * ld + threadIdx.x];
      P[jj * ld + threadIdx.x] = P[pr * ld + threadIdx.x];
      P[pr * ld + threadIdx.x] = t;
    }
    __syncthreads();
    const double d = P[jj * ld + jj];
    if (d != 0.0)
      for (int r = jj + 1 + threadIdx.x; r < rows; r += blockDim.x) {
        double* row = P + r * ld;
        const double l = row[jj] / d;
        row[jj] = l;
        for (int c = jj + 1; c < kb; ++c) row[c] -= l * P[jj * ld + c];
      }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < rows * kb; i += blockDim.x) {
    const int r = i / kb, c = i - r * kb;
    A[(int64_t)(k + r) * n + k + c] = P[r * ld + c];
  }
}

// Register-resident panel for at most 2 x 512 rows and LU_RB = 16 columns:
// thread t owns rows t and t + 512 of the panel, their 16 entries in
// registers for the whole factorisation.  A column step is a register pivot
// search, an exchange of the two swapped rows through shared memory, and a
// register update against the pivot row broadcast from shared memory.
constexpr int LU_RB = 16;
__global__ void __launch_bounds__(512) k_lu_panel_reg(double* A, int n, int k, int kb, int* piv,
                                                      int* singular) {
  __shared__ double prow[LU_RB], jrow[LU_RB];
  __shared__ double vmax[16];
  __shared__ int imax[16];
  __shared__ int p_sh;
  const int rows = n - k;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double v[2][LU_RB];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int r = threadIdx.x + h * 512;
#pragma unroll
    for (int c = 0; c < LU_RB; ++c)
      v[h][c] = (r < rows && c < kb) ? A[(int64_t)(k + r) * n + k + c] : 0.0;
  }
  for (int jj = 0; jj < kb; ++jj) {
    // pivot: the largest |entry| of column jj among rows >= jj
    double best = -1.0;
    int bi = jj;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int r = threadIdx.x + h * 512;
      double a = 0.0;
#pragma unroll
      for (int c = 0; c < LU_RB; ++c) a = c == jj ? v[h][c] : a;
      a = fabs(a);
      if (r >= jj && r < rows && a > best) {
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
      double bb = -1.0;
      int i = jj;
      for (int w = 0; w < nw; ++w)
        if (vmax[w] > bb || (vmax[w] == bb && imax[w] < i)) {
          bb = vmax[w];
          i = imax[w];
        }
      p_sh = i;
      piv[k + jj] = k + i;
      if (!(bb > 0.0)) *singular = 1;
    }
    __syncthreads();
    const int pr = p_sh;
    // rows jj and pr trade places: their owners publish them in shared
    // memory (prow = the new row jj), then each takes the other's values
    const int hp = pr >> 9, tp = pr & 511;
    const int hj = jj >> 9, tj = jj & 511;
    if (threadIdx.x == tp) {
#pragma unroll
      for (int c = 0; c < LU_RB; ++c) prow[c] = hp ? v[1][c] : v[0][c];
    }
    if (pr != jj && threadIdx.x == tj) {
#pragma unroll
      for (int c = 0; c < LU_RB; ++c) jrow[c] = hj ? v[1][c] : v[0][c];
    }
    __syncthreads();
    if (pr != jj) {
      if (threadIdx.x == tj) {
#pragma unroll
        for (int c = 0; c < LU_RB; ++c) {
          if (hj) v[1][c] = prow[c];
          else v[0][c] = prow[c];
        }
      }
      if (threadIdx.x == tp) {
#pragma unroll
        for (int c = 0; c < LU_RB; ++c) {
          if (hp) v[1][c] = jrow[c];
          else v[0][c] = jrow[c];
        }
      }
    }
    const double d = prow[jj];
    if (d != 0.0) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = threadIdx.x + h * 512;
        if (r > jj && r < rows) {
          double a = 0.0;
#pragma unroll
          for (int c = 0; c < LU_RB; ++c) a = c == jj ? v[h][c] : a;
          const double l = a / d;
#pragma unroll
          for (int c = 0; c < LU_RB; ++c) {
            if (c > jj) v[h][c] -= l * prow[c];
            if (c == jj) v[h][c] = l;
          }
        }
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int r = threadIdx.x + h * 512;
    if (r < rows)
#pragma unroll
      for (int c = 0; c < LU_RB; ++c)
        if (c < kb) A[(int64_t)(k + r) * n + k + c] = v[h][c];
  }
}

// Shared-memory panel: rows x (kb + 1) doubles within this budget.
constexpr size_t LU_SMEM_PANEL = 220 * 1024;

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

// U12 = L11^{-1} A12 with L11 (unit lower, kb <= KB) in shared memory and each
// thread's column of A12 in registers.
template <int KB>
__global__ void __launch_bounds__(128) k_lu_trsm_reg(double* A, int n, int k, int kb) {
  __shared__ double Ls[KB][KB];
  for (int i = threadIdx.x; i < KB * KB; i += blockDim.x) {
    const int r = i / KB, t = i - r * KB;
    Ls[r][t] = (r < kb && t < kb) ? A[(int64_t)(k + r) * n + k + t] : 0.0;
  }
  __syncthreads();
  for (int c = k + kb + blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    double v[KB];
#pragma unroll
    for (int r = 0; r < KB; ++r) v[r] = r < kb ? A[(int64_t)(k + r) * n + c] : 0.0;
#pragma unroll
    for (int r = 1; r < KB; ++r)
#pragma unroll
      for (int t = 0; t < r; ++t) v[r] -= Ls[r][t] * v[t];
#pragma unroll
    for (int r = 0; r < KB; ++r)
      if (r < kb) A[(int64_t)(k + r) * n + c] = v[r];
  }
}

// Swaps on b, then L y = b (unit diagonal) and U x = y, one CTA, by blocks
// of 32 rows: the block's right-hand side first takes the product with the
// solved part (all warps, one row each), then one warp solves the 32 x 32
// triangle with shuffles.
__global__ void __launch_bounds__(512) k_lu_subst(const double* A, int n, const int* piv, double* b) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
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
  // forward: rows r0..r0+31 after rows < r0 are final
  for (int r0 = 0; r0 < n; r0 += 32) {
    const int rb = min(32, n - r0);
    for (int i = warp; i < rb; i += nw) {
      const double* Ar = A + (int64_t)(r0 + i) * n;
      double part = 0.0;
      for (int t = lane; t < r0; t += 32) part += Ar[t] * b[t];
      for (int o = 16; o; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
      if (lane == 0) b[r0 + i] -= part;
    }
    __syncthreads();
    if (warp == 0) {
      double y = lane < rb ? b[r0 + lane] : 0.0;
      for (int i = 0; i < rb; ++i) {
        const double yi = __shfl_sync(0xffffffffu, y, i);
        if (lane > i && lane < rb) y -= A[(int64_t)(r0 + lane) * n + r0 + i] * yi;
      }
      if (lane < rb) b[r0 + lane] = y;
    }
    __syncthreads();
  }
  // backward: rows r0..r0+rb-1 (from the bottom) after rows >= r0 + rb are final
  for (int r1 = n; r1 > 0; r1 -= 32) {
    const int r0 = max(0, r1 - 32), rb = r1 - r0;
    for (int i = warp; i < rb; i += nw) {
      const double* Ar = A + (int64_t)(r0 + i) * n;
      double part = 0.0;
      for (int t = r1 + lane; t < n; t += 32) part += Ar[t] * b[t];
      for (int o = 16; o; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
      if (lane == 0) b[r0 + i] -= part;
    }
    __syncthreads();
    if (warp == 0) {
      double y = lane < rb ? b[r0 + lane] : 0.0;
      for (int i = rb - 1; i >= 0; --i) {
        const double di = A[(int64_t)(r0 + i) * n + r0 + i];
        if (lane == i) y /= di;
        const double yi = __shfl_sync(0xffffffffu, y, i);
        if (lane < i) y -= A[(int64_t)(r0 + lane) * n + r0 + i] * yi;
      }
      if (lane < rb) b[r0 + lane] = y;
    }
    __syncthreads();
  }
}

bool lu_solve(tnfa_ctx* ctx, double* A, double* b, int n) {
  if (n <= 0) return true;
  DBuf piv(ctx, (size_t)n * sizeof(int)), sing(ctx, sizeof(int));
  TNFA_CUDA(cudaMemsetAsync(sing.p, 0, sizeof(int), ctx->stream));
  KernelScope ks(ctx, "lu_f64", 2.0 / 3.0 * (double)n * n * n, 0.0);
  TNFA_CUDA(cudaFuncSetAttribute(k_lu_panel_smem, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)LU_SMEM_PANEL));
  for (int k = 0; k < n;) {
    // panel width: 32 columns, or 16 when only that lets the panel sit in
    // shared memory; the global-memory panel beyond that
    // the panel in registers (at most 1024 rows left, 16 columns), in shared
    // memory (at most 1600 rows, 16 columns), else in global memory (32)
    const int rows = n - k;
    int kb;
    if (rows <= 1024) {
      kb = std::min(LU_RB, rows);
      k_lu_panel_reg<<<1, 512, 0, ctx->stream>>>(A, n, k, kb, piv.as<int>(), sing.as<int>());
    } else if ((size_t)rows * 17 * 8 <= LU_SMEM_PANEL) {
      kb = 16;
      k_lu_panel_smem<<<1, 1024, (size_t)rows * (kb + 1) * 8, ctx->stream>>>(A, n, k, kb, piv.as<int>(),
                                                                           sing.as<int>());
    } else {
      kb = LU_NB;
      k_lu_panel<<<1, 256, 0, ctx->stream>>>(A, n, k, kb, piv.as<int>(), sing.as<int>());
    }
    k_lu_swap<<<grid_for(n, 256, 1024), 256, 0, ctx->stream>>>(A, n, k, kb, piv.as<int>());
    if (k + kb < n) {
      if (kb <= 16)
        k_lu_trsm_reg<16><<<grid_for(n - k - kb, 128, 1024), 128, 0, ctx->stream>>>(A, n, k, kb);
      else
        k_lu_trsm_reg<32><<<grid_for(n - k - kb, 128, 1024), 128, 0, ctx->stream>>>(A, n, k, kb);
      const int m2 = n - k - kb;
      GemmJob g{A + (int64_t)(k + kb) * n + k, A + (int64_t)k * n + k + kb,
                A + (int64_t)(k + kb) * n + k + kb, m2, m2, kb, n, n, n, 0, 0, -1.0, 1.0};
      gemm<double>(ctx, {g});
    }
    TNFA_LAUNCH_CHECK();
    k += kb;
  }
  k_lu_subst<<<1, 512, 0, ctx->stream>>>(A, n, piv.as<int>(), b);
  TNFA_LAUNCH_CHECK();
  int hs = 0;
  TNFA_CUDA(cudaMemcpyAsync(&hs, sing.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  return hs == 0;
}

// --------------------------------------------------------- factorise --
// Batched block copy with element conversion: dst[(r, c) or (c, r)] =
// conv(src[r * lds + c]), conjugated on request.
struct CopyJob {
  const void* src;
  void* dst;
  int rows, cols, lds, ldd;
  int trans, conj;
  // when set: multiply by the power of two that brings sqrt(*sumsq) into
  // [1, 2) (keeps FP32 copies of tiny or huge blocks in range, exactly)
  const double* sumsq = nullptr;
};

__device__ inline double pow2_scale(const double* ss) {
  if (!ss) return 1.0;
  const double f = sqrt(*ss);
  return f > 0 && isfinite(f) ? ldexp(1.0, -ilogb(f)) : 1.0;
}

// Per-job sum of squares of an m x k block (one CTA per job).
struct SumsqJob {
  const void* src;
  int64_t n;
  double* out;
};

__global__ void k_sumsq(const SumsqJob* __restrict__ jobs) {
  const SumsqJob jb = jobs[blockIdx.x];
  const double* x = (const double*)jb.src;
  double part = 0.0;
  for (int64_t i = threadIdx.x; i < jb.n; i += blockDim.x) part += x[i] * x[i];
  __shared__ double red[32];
  const double t = block_sum<double>(part, red);
  if (threadIdx.x == 0) *jb.out = t;
}

__device__ inline double cvt(double x, double*) { return x; }
__device__ inline float cvt(double x, float*) { return (float)x; }
__device__ inline double cvt(float x, double*) { return (double)x; }
__device__ inline cplx cvt(cplx x, cplx*) { return x; }
__device__ inline dfl cvt(double x, dfl*) { return dfl(x); }
__device__ inline double cvt(dfl x, double*) { return (double)x; }

template <class S, class D>
__global__ void k_copy_block(const CopyJob* __restrict__ jobs) {
  const CopyJob jb = jobs[blockIdx.y];
  const S* src = (const S*)jb.src;
  D* dst = (D*)jb.dst;
  const int64_t n = (int64_t)jb.rows * jb.cols;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / jb.cols), c = (int)(i % jb.cols);
    S v = src[(int64_t)r * jb.lds + c];
    if (jb.conj) v = conj(v);
    if (jb.sumsq) v = scal(v, (decltype(re(v)))pow2_scale(jb.sumsq));
    const int64_t o = jb.trans ? (int64_t)c * jb.ldd + r : (int64_t)r * jb.ldd + c;
    dst[o] = cvt(v, (D*)nullptr);
  }
}

template <class S, class D>
void copy_blocks(tnfa_ctx* ctx, const std::vector<CopyJob>& jobs) {
  if (jobs.empty()) return;
  int64_t nmax = 1;
  for (const auto& j : jobs) nmax = std::max<int64_t>(nmax, (int64_t)j.rows * j.cols);
  TNFA_CHECK(jobs.size() <= 65535, TNFA_ERR_UNSUPPORTED, "more than 65535 copies in one batch");
  DBuf d = upload(ctx, jobs);
  k_copy_block<S, D><<<dim3(grid_for(nmax, 256, 1024), (unsigned)jobs.size()), 256, 0, ctx->stream>>>(
      d.as<CopyJob>());
  TNFA_LAUNCH_CHECK();
}

template <class T>
void trunc_factor(tnfa_ctx* ctx, const std::vector<FactorJob>& jobs, double cutoff, int maxdim,
                  int mindim, int precision, std::vector<FactorResult>& out, double reveal_tol) {
  const size_t nj = jobs.size();
  out.clear();
  out.resize(nj);
  if (!nj) return;
  constexpr bool real64 = std::is_same<T, double>::value;
  const bool mixed = real64 && (precision == TNFA_PREC_MIXED || precision == TNFA_PREC_F32);
  // Per job the core C (cm x k) that Jacobi diagonalises, and how L and X
  // follow from its left vectors U_r:
  //   tall, QR  : M = Q R, C = R (k x k),   L = Q U_r, X = U_r^H R
  //   tall, none: C = M (rows x k) [mixed], L = U_r,   X = U_r^H M
  //   wide      : M^H = Q R, C = R^H,       L = U_r,   X = U_r^H M
  std::vector<int> n(nj), cm(nj), ku(nj);
  std::vector<char> tall(nj), useq(nj);
  std::vector<DBuf> Q(nj), R(nj), tau(nj), Mt(nj), J(nj), U(nj);
  std::vector<const void*> core(nj);
  std::vector<CopyJob> adj;
  std::vector<QrJob> qj;
  // singular values and sweep counts of all jobs in two buffers, so that the
  // host reads them back with one copy each
  std::vector<size_t> soff(nj + 1, 0);
  for (size_t q = 0; q < nj; ++q) soff[q + 1] = soff[q] + (size_t)std::min(jobs[q].rows, jobs[q].cols);
  DBuf Sall(ctx, std::max<size_t>(soff[nj], 1) * sizeof(double));
  DBuf swall(ctx, nj * sizeof(int));
  auto S_of = [&](size_t q) { return Sall.as<double>() + soff[q]; };
  auto sw_of = [&](size_t q) { return swall.as<int>() + q; };
  // Rank-revealing front end (reveal_tol > 0, tall jobs): M = Q1 R1 by
  // pivoted QR with R1 (r x cols), r the numerical rank; when r < cols the
  // square core is R2^H from R1^H = Q2 R2, else R1 itself.  The left vectors
  // of M are Q1 times those of the core, so L = Q1 U_r and X = U_r^H R1, as
  // for the plain tall case with (Q, R) = (Q1, R1).
  std::vector<char> rev(nj, 0);
  if (reveal_tol > 0.0) {
    std::vector<QrJob> pj;
    std::vector<size_t> pidx;
    for (size_t q = 0; q < nj; ++q) {
      const FactorJob& f = jobs[q];
      if (f.rows < f.cols) continue;
      rev[q] = 1;
      Q[q] = DBuf(ctx, (size_t)f.rows * f.cols * sizeof(T));
      R[q] = DBuf(ctx, (size_t)f.cols * f.cols * sizeof(T));
      tau[q] = DBuf(ctx, (size_t)f.cols * sizeof(T));
      pj.push_back({f.M, Q[q].p, R[q].p, tau[q].p, f.rows, f.cols});
      pidx.push_back(q);
    }
    std::vector<int> rk;
    qr_rank<T>(ctx, pj, reveal_tol, rk);
    // R1^H = Q2 R2 for the jobs with r < cols; the core is R2^H
    std::vector<DBuf> Rt(nj), Q2(nj), R2(nj), t2(nj);
    std::vector<CopyJob> tr, back;
    std::vector<QrJob> lq;
    for (size_t i = 0; i < pidx.size(); ++i) {
      const size_t q = pidx[i];
      const int r = rk[i], cols = jobs[q].cols;
      n[q] = cm[q] = r;
      tall[q] = useq[q] = 1;
      if (r == cols) {
        core[q] = R[q].p;
        continue;
      }
      Rt[q] = DBuf(ctx, (size_t)cols * r * sizeof(T));
      Q2[q] = DBuf(ctx, (size_t)cols * r * sizeof(T));
      R2[q] = DBuf(ctx, (size_t)r * r * sizeof(T));
      t2[q] = DBuf(ctx, (size_t)r * sizeof(T));
      tr.push_back({R[q].p, Rt[q].p, r, cols, cols, r, 1, 1});
      lq.push_back({Rt[q].p, Q2[q].p, R2[q].p, t2[q].p, cols, r});
      J[q] = DBuf(ctx, (size_t)r * r * sizeof(T));
      back.push_back({R2[q].p, J[q].p, r, r, r, r, 1, 1});
      core[q] = J[q].p;
    }
    copy_blocks<T, T>(ctx, tr);
    qr<T>(ctx, lq);
    copy_blocks<T, T>(ctx, back);
  }
  for (size_t q = 0; q < nj; ++q) {
    const FactorJob& f = jobs[q];
    if (rev[q]) continue;
    tall[q] = f.rows >= f.cols;
    n[q] = std::min(f.rows, f.cols);
    const int k = n[q];
    useq[q] = tall[q] && !mixed;
    if (tall[q] && mixed) {
      core[q] = f.M;
      cm[q] = f.rows;
      continue;
    }
    R[q] = DBuf(ctx, (size_t)k * k * sizeof(T));
    tau[q] = DBuf(ctx, (size_t)k * sizeof(T));
    cm[q] = k;
    if (tall[q]) {
      Q[q] = DBuf(ctx, (size_t)f.rows * k * sizeof(T));
      qj.push_back({f.M, Q[q].p, R[q].p, tau[q].p, f.rows, f.cols});
      core[q] = R[q].p;
    } else {
      Mt[q] = DBuf(ctx, (size_t)f.rows * f.cols * sizeof(T));
      adj.push_back({f.M, Mt[q].p, f.rows, f.cols, f.cols, f.rows, 1, 1});
      Q[q] = DBuf(ctx, (size_t)f.cols * k * sizeof(T));
      qj.push_back({Mt[q].p, Q[q].p, R[q].p, tau[q].p, f.cols, f.rows});
      J[q] = DBuf(ctx, (size_t)k * k * sizeof(T));
      core[q] = J[q].p;
    }
  }
  copy_blocks<T, T>(ctx, adj);
  qr<T>(ctx, qj);
  adj.clear();
  for (size_t q = 0; q < nj; ++q)
    if (!tall[q]) adj.push_back({R[q].p, J[q].p, n[q], n[q], n[q], n[q], 1, 1});
  copy_blocks<T, T>(ctx, adj);
  const JacobiOpts opts{1e-10, cutoff > 0 ? cutoff * 1e-2 : 0.0};
  // the polish starts from FP32-converged columns (offsets ~1e-7), already in
  // the quadratic regime: the sweep whose rotations were all below 1e-6
  // leaves ~1e-12, so it is the last one
  const JacobiOpts polish{1e-6, opts.small_rel};
  // (2) Jacobi on the core: U (cm x ku); extra[q] = weight outside U's span
  std::vector<double> extra(nj, 0.0);
  std::vector<double> polish_scale;  // mixed: sum of squares of each polish input
  std::vector<SvdJob> sj;
  if (!mixed) {
    for (size_t q = 0; q < nj; ++q) {
      ku[q] = n[q];
      U[q] = DBuf(ctx, (size_t)cm[q] * n[q] * sizeof(T));
      sj.push_back({core[q], U[q].p, S_of(q), nullptr, cm[q], n[q], sw_of(q)});
    }
    jacobi<T>(ctx, sj, 60, opts, real64 ? "svd_f64" : "svd_c128");
  } else {
    // Two FP32 passes, each followed by an FP64 change of basis X <- X V.
    // Pass 1 finds the directions worth keeping; pass 2 runs on X = C V,
    // whose columns are already scaled by their singular values, so its FP32
    // rounding is relative to each column and the small directions (which
    // pass 1 cannot resolve below ~sqrt(eps32) of the largest) come out
    // right.  FP64 Jacobi then converges in two or three sweeps.
    std::vector<DBuf> X(nj);
    std::vector<int> w(nj);
    std::vector<const void*> xin(core);
    // |C|_F^2 and |C V_kept|_F^2 in FP64: their difference is the weight of
    // the directions dropped after pass 1, exact to FP64 rounding
    std::vector<double> ss_in(nj), ss_kept(nj);
    DBuf ss_keep;  // pass 2's sums of squares, read after the passes
    for (size_t q = 0; q < nj; ++q) w[q] = n[q];
    for (int pass = 0; pass < 2; ++pass) {
      std::vector<DBuf> C32(nj), U32(nj), V32(nj), V(nj), G(nj), Y(nj), Xn(nj);
      DBuf S32all(ctx, std::max<size_t>(soff[nj], 1) * sizeof(double));
      DBuf sw32all(ctx, nj * sizeof(int));
      std::vector<CopyJob> down, up;
      std::vector<SvdJob> s32;
      // FP32 copies scaled by a power of two to unit size
      DBuf ss(ctx, nj * sizeof(double));
      {
        std::vector<SumsqJob> sq;
        for (size_t q = 0; q < nj; ++q)
          sq.push_back({xin[q], (int64_t)cm[q] * w[q], ss.as<double>() + q});
        DBuf dq = upload(ctx, sq);
        k_sumsq<<<(unsigned)nj, 256, 0, ctx->stream>>>(dq.as<SumsqJob>());
        TNFA_LAUNCH_CHECK();
      }
      for (size_t q = 0; q < nj; ++q) {
        const int k = w[q], m = cm[q];
        C32[q] = DBuf(ctx, (size_t)m * k * sizeof(float));
        U32[q] = DBuf(ctx, (size_t)m * k * sizeof(float));
        V32[q] = DBuf(ctx, (size_t)k * k * sizeof(float));
        down.push_back({xin[q], C32[q].p, m, k, k, k, 0, 0, ss.as<double>() + q});
        s32.push_back({C32[q].p, U32[q].p, S32all.as<double>() + soff[q], V32[q].p, m, k,
                       sw32all.as<int>() + q});
      }
      copy_blocks<double, float>(ctx, down);
      // pass 1 only has to split kept from dropped directions and hand pass 2
      // a nearly diagonal start: stop at 1e-4; pass 2 runs to FP32 accuracy
      jacobi<float>(ctx, s32, 60, JacobiOpts{pass == 0 ? 1e-4 : 0.0, opts.small_rel}, "svd_f32");
      if (pass == 0) {
        // keep the FP32 directions that a 10^6 times smaller cutoff would
        // keep (all of them without a cutoff).  What pass 1 drops cannot be
        // recovered: a kept direction s_k tilts by ~eps32 s_max / s_k into
        // the dropped span, losing ~eps32 s_drop / s_k of itself, so the
        // dropped weight must sit far below the truncation budget (here
        // 1e-6 of it: the FP64 rule below drops it too, and the loss stays
        // near 1e-10 of the norm).  Exactly-deficient ranks still fall away.
        // (the sums of squares are read here, where the host waits anyway: a
        // copy to pageable memory returns only once it has completed)
        std::vector<double> sv32(soff[nj]);
        const std::vector<double>& hss = ss_in;
        TNFA_CUDA(cudaMemcpyAsync(ss_in.data(), ss.p, nj * sizeof(double), cudaMemcpyDeviceToHost,
                                  ctx->stream));
        TNFA_CUDA(cudaMemcpyAsync(sv32.data(), S32all.p, soff[nj] * sizeof(double),
                                  cudaMemcpyDeviceToHost, ctx->stream));
        TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
        for (size_t q = 0; q < nj; ++q) {
          const int k = n[q];
          double* sq = sv32.data() + soff[q];
          // undo the power-of-two scaling of the FP32 copy
          const double f = std::sqrt(hss[q]);
          const double back = f > 0 && std::isfinite(f) ? std::ldexp(1.0, std::ilogb(f)) : 1.0;
          for (int i = 0; i < k; ++i) sq[i] *= back;
          int keep = cutoff > 0 ? truncation_rank(sq, k, cutoff * 1e-6, 0, 1) : k;
          if (maxdim > 0) keep = std::min(keep, std::min(k, maxdim + 8));
          keep = std::max(keep, std::min(k, std::max(mindim, 1)));
          ku[q] = keep;
        }
      }
      for (size_t q = 0; q < nj; ++q) {
        const int k = w[q], c = ku[q];
        V[q] = DBuf(ctx, (size_t)k * c * sizeof(double));
        up.push_back({V32[q].p, V[q].p, k, c, k, c, 0, 0});
      }
      copy_blocks<float, double>(ctx, up);
      // V <- V (3 I - V^T V) / 2, twice: orthonormal columns to rounding
      for (int it = 0; it < 2; ++it) {
        std::vector<GemmJob> g1, g2;
        std::vector<CopyJob> cp;
        for (size_t q = 0; q < nj; ++q) {
          const int k = w[q], c = ku[q];
          G[q] = DBuf(ctx, (size_t)c * c * sizeof(double));
          Y[q] = DBuf(ctx, (size_t)k * c * sizeof(double));
          g1.push_back({V[q].p, V[q].p, G[q].p, c, c, k, c, c, c, 1, 0, 1.0, 0.0});
          cp.push_back({V[q].p, Y[q].p, k, c, c, c, 0, 0});
          g2.push_back({V[q].p, G[q].p, Y[q].p, k, c, c, c, c, c, 0, 0, -0.5, 1.5});
        }
        gemm<double>(ctx, g1);
        copy_blocks<double, double>(ctx, cp);
        gemm<double>(ctx, g2);
        for (size_t q = 0; q < nj; ++q) std::swap(V[q], Y[q]);
      }
      std::vector<GemmJob> gw;
      for (size_t q = 0; q < nj; ++q) {
        const int k = w[q], c = ku[q], m = cm[q];
        Xn[q] = DBuf(ctx, (size_t)m * c * sizeof(double));
        gw.push_back({xin[q], V[q].p, Xn[q].p, m, c, k, k, c, c, 0, 0, 1.0, 0.0});
      }
      gemm<double>(ctx, gw);
      for (size_t q = 0; q < nj; ++q) {
        X[q] = std::move(Xn[q]);
        xin[q] = X[q].p;
        w[q] = ku[q];
      }
      if (pass == 1) ss_keep = std::move(ss);
    }
    TNFA_CUDA(cudaMemcpyAsync(ss_kept.data(), ss_keep.p, nj * sizeof(double), cudaMemcpyDeviceToHost,
                              ctx->stream));
    TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
    for (size_t q = 0; q < nj; ++q) extra[q] = std::max(0.0, ss_in[q] - ss_kept[q]);
    // The polish in double-float (FP32 pairs, ~48 bits) on the FP32 pipe:
    // X is scaled by a power of two to unit size on the way in, U comes back
    // to FP64, and the singular values are scaled back on the host.
    DBuf ssx(ctx, nj * sizeof(double));
    {
      std::vector<SumsqJob> sq;
      for (size_t q = 0; q < nj; ++q) sq.push_back({X[q].p, (int64_t)cm[q] * ku[q], ssx.as<double>() + q});
      DBuf dq = upload(ctx, sq);
      k_sumsq<<<(unsigned)nj, 256, 0, ctx->stream>>>(dq.as<SumsqJob>());
      TNFA_LAUNCH_CHECK();
    }
    std::vector<DBuf> Xd(nj), Ud(nj);
    std::vector<CopyJob> dn, upj;
    for (size_t q = 0; q < nj; ++q) {
      const size_t ne = (size_t)cm[q] * ku[q];
      Xd[q] = DBuf(ctx, ne * sizeof(dfl));
      Ud[q] = DBuf(ctx, ne * sizeof(dfl));
      U[q] = DBuf(ctx, ne * sizeof(T));
      dn.push_back({X[q].p, Xd[q].p, cm[q], ku[q], ku[q], ku[q], 0, 0, ssx.as<double>() + q});
      sj.push_back({Xd[q].p, Ud[q].p, S_of(q), nullptr, cm[q], ku[q], sw_of(q)});
      upj.push_back({Ud[q].p, U[q].p, cm[q], ku[q], ku[q], ku[q], 0, 0});
    }
    copy_blocks<double, dfl>(ctx, dn);
    jacobi<dfl>(ctx, sj, 60, polish, "svd_polish_df");
    copy_blocks<dfl, double>(ctx, upj);
    polish_scale.resize(nj);
    TNFA_CUDA(cudaMemcpyAsync(polish_scale.data(), ssx.p, nj * sizeof(double), cudaMemcpyDeviceToHost,
                              ctx->stream));
    // Diagnostics (TNFA_DEBUG_DIR with TNFA_DEBUG_SWEEPS=k): the FP64 core of
    // every mixed job whose polish took k sweeps or more, with its polish input
    static const char* dbg = getenv("TNFA_DEBUG_DIR");
    static const int thr = getenv("TNFA_DEBUG_SWEEPS") ? atoi(getenv("TNFA_DEBUG_SWEEPS")) : 0;
    if (dbg && *dbg && thr > 0) {
      static int counter = 0;
      for (size_t q = 0; q < nj && counter < 32; ++q) {
        int swq = 0;
        TNFA_CUDA(cudaMemcpyAsync(&swq, sw_of(q), sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
        if (swq >= 0 && swq < thr) continue;
        const int m = cm[q], k = n[q], c = ku[q];
        std::vector<double> hc((size_t)m * k), hx((size_t)m * c);
        TNFA_CUDA(cudaMemcpyAsync(hc.data(), core[q], hc.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
        TNFA_CUDA(cudaMemcpyAsync(hx.data(), X[q].p, hx.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
        TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
        char path[1024];
        snprintf(path, sizeof path, "%s/mixed_core_%d.bin", dbg, counter++);
        if (FILE* fp = fopen(path, "wb")) {
          int hdr[4] = {m, k, c, swq};
          fwrite(hdr, sizeof(int), 4, fp);
          fwrite(hc.data(), 8, hc.size(), fp);
          fwrite(hx.data(), 8, hx.size(), fp);
          fclose(fp);
        }
      }
    }
  }
  // (3) ranks on the host (one read-back of every job's values and sweeps)
  if (!polish_scale.empty())
    TNFA_CUDA(cudaStreamSynchronize(ctx->stream));  // polish_scale arrives with the values
  {
    std::vector<double> hs(soff[nj]);
    std::vector<int> hsw(nj);
    TNFA_CUDA(cudaMemcpyAsync(hs.data(), Sall.p, soff[nj] * sizeof(double), cudaMemcpyDeviceToHost,
                              ctx->stream));
    TNFA_CUDA(cudaMemcpyAsync(hsw.data(), swall.p, nj * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
    for (size_t q = 0; q < nj; ++q) {
      out[q].s.assign(hs.begin() + soff[q], hs.begin() + soff[q] + ku[q]);
      out[q].sweeps = hsw[q];
      if (!polish_scale.empty()) {
        // undo the power of two the polish input was scaled by
        const double f = std::sqrt(polish_scale[q]);
        const double back = f > 0 && std::isfinite(f) ? std::ldexp(1.0, std::ilogb(f)) : 1.0;
        for (double& x : out[q].s) x *= back;
      }
    }
  }
  std::vector<GemmJob> gl, gx;
  std::vector<CopyJob> cl;
  for (size_t q = 0; q < nj; ++q) {
    FactorResult& o = out[q];
    const FactorJob& f = jobs[q];
    const int k = n[q], c = ku[q], m = cm[q];
    double tot = extra[q];
    for (int i = 0; i < c; ++i) tot += o.s[i] * o.s[i];
    int r = c;
    double drop = extra[q];
    if (tot > 0.0 && cutoff > 0.0)
      while (r > 1 && drop + o.s[r - 1] * o.s[r - 1] <= cutoff * tot) {
        --r;
        drop += o.s[r] * o.s[r];
      }
    if (maxdim > 0) r = std::min(r, maxdim);
    // never keep directions at the rounding floor: Jacobi leaves them
    // unorthogonalised (zero columns of U)
    int nz = 0;
    while (nz < c && o.s[nz] * o.s[nz] > 1e-28 * tot) ++nz;
    r = std::min(r, std::max(nz, 1));
    r = std::max(r, std::min(std::max(mindim, 1), c));
    drop = extra[q];
    for (int i = r; i < c; ++i) drop += o.s[i] * o.s[i];
    o.r = r;
    o.discarded = tot > 0 ? drop / tot : 0.0;
    o.L = DBuf(ctx, (size_t)f.rows * r * sizeof(T));
    o.X = DBuf(ctx, (size_t)r * f.cols * sizeof(T));
    if (useq[q]) {
      gl.push_back({Q[q].p, U[q].p, o.L.p, f.rows, r, k, k, c, r, 0, 0, 1.0, 0.0});
      gx.push_back({U[q].p, R[q].p, o.X.p, r, f.cols, k, c, f.cols, f.cols, 2, 0, 1.0, 0.0});
    } else {
      cl.push_back({U[q].p, o.L.p, m, r, c, r, 0, 0});
      gx.push_back({U[q].p, f.M, o.X.p, r, f.cols, m, c, f.cols, f.cols, 2, 0, 1.0, 0.0});
    }
  }
  gemm<T>(ctx, gl);
  copy_blocks<T, T>(ctx, cl);
  gemm<T>(ctx, gx);
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
template void qr_rank<double>(tnfa_ctx*, const std::vector<QrJob>&, double, std::vector<int>&);
template void qr_rank<cplx>(tnfa_ctx*, const std::vector<QrJob>&, double, std::vector<int>&);
template void trunc_factor<double>(tnfa_ctx*, const std::vector<FactorJob>&, double, int, int, int,
                                   std::vector<FactorResult>&, double);
template void trunc_factor<cplx>(tnfa_ctx*, const std::vector<FactorJob>&, double, int, int, int,
                                 std::vector<FactorResult>&, double);

}  // namespace la
}  // namespace tnfa
