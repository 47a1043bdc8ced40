// Batched dense linear algebra on the device (row-major matrices).  Every
// routine takes a vector of independent problems of possibly different sizes
// and runs them in one launch (one CTA, or one CTA tile set, per problem).
#pragma once
#include "common.cuh"

namespace tnfa {
namespace la {

constexpr int MAXD = 16;  // tensor order handled by permute

// dst = transpose of src: dst axis i is src axis perm[i].
struct PermJob {
  const void* src;
  void* dst;
  int nd;
  int shape[MAXD];  // src shape
  int perm[MAXD];
  int64_t n;
};
template <class T>
void permute(tnfa_ctx* ctx, const std::vector<PermJob>& jobs);

// C = alpha * op(A) * op(B) + beta * C; op(X) = X, X^T or X^H (conj).
struct GemmJob {
  const void* A;
  const void* B;
  void* C;
  int m, n, k;
  int lda, ldb, ldc;
  int opA, opB;  // 0: N, 1: T, 2: C (conjugate transpose)
  double alpha, beta;
};
template <class T>
void gemm(tnfa_ctx* ctx, const std::vector<GemmJob>& jobs);

// Householder QR of A (m x n, lda = n, destroyed): Q (m x kq, kq = min(m, n))
// and R (kq x n) written to separate buffers.
struct QrJob {
  void* A;
  void* Q;
  void* R;
  void* tau;  // kq scalars of workspace
  int m, n;
};
template <class T>
void qr(tnfa_ctx* ctx, const std::vector<QrJob>& jobs);

// Rank-revealing QR (Householder with column pivoting) of the same jobs:
// A ~= Q R with Q (m x r, orthonormal, written row-major m x r into the Q
// buffer) and R (r x n, A's column order, the first r rows of the R buffer),
// where r >= 1 is the first step at which the columns not yet pivoted hold
// at most tol^2 of |A|_F^2 (r = min(m, n) if none).  ranks[i] = r of job i.
template <class T>
void qr_rank(tnfa_ctx* ctx, const std::vector<QrJob>& jobs, double tol, std::vector<int>& ranks);

// One job of the one-sided Jacobi SVD used by trunc_factor: A (m x n, m >=
// n, lda = n, read only) = U diag(S) V^H with U (m x n, orthonormal columns
// where S > 0), S (n, real, descending), V (n x n; not accumulated when V is
// null).  sweeps receives the sweep count, or -1 when the sweep cap was hit.
struct SvdJob {
  const void* A;
  void* U;
  double* S;
  void* V;
  int m, n;
  int* sweeps;
};

// Solve A x = b for one dense n x n FP64 system (A row-major, destroyed; b
// overwritten by x): blocked right-looking LU with partial pivoting (panel
// kernel, row swaps, triangular solve, trailing update by the batched GEMM),
// then forward / back substitution.  Returns false if a pivot is exactly 0.
bool lu_solve(tnfa_ctx* ctx, double* A, double* b, int n);

// Truncated factorisation of bond matrices, the SVD step of truncation:
// M (rows x cols, row-major; overwritten) ~= L X with L (rows x r) having
// orthonormal columns and X (r x cols), r = truncation_rank of M's singular
// values.  The square core J (R of M = QR when rows >= cols, else R^H of
// M^H = QR) is diagonalised by one-sided Jacobi without accumulating V:
// L = Q U_r (or U_r) and X = U_r^H R (or U_r^H M).  precision MIXED / F32
// (real FP64 only): Jacobi first runs in FP32 with V accumulated, V is
// re-orthonormalised in FP64 (two Newton-Schulz steps), and Jacobi on J V
// in double-float (FP32 pairs, about 48 bits, on the FP32 pipe) polishes U
// and the singular values in a few sweeps.
struct FactorJob {
  void* M;
  int rows, cols;
};
struct FactorResult {
  DBuf L, X;
  int r = 0;
  double discarded = 0.0;  // relative discarded weight
  int sweeps = 0;          // FP64 Jacobi sweeps; -1: the sweep cap was hit
  std::vector<double> s;   // singular values, descending
};
// reveal_tol > 0: tall jobs first go through the rank-revealing QR (qr_rank
// with that tolerance) and the core is the square factor of its numerical
// rank, so the SVD runs on r x r rather than cols x cols.
template <class T>
void trunc_factor(tnfa_ctx* ctx, const std::vector<FactorJob>& jobs, double cutoff, int maxdim,
                  int mindim, int precision, std::vector<FactorResult>& out, double reveal_tol = 0.0);

// Rank kept by the reference truncation rule: smallest r >= mindim with
// sum_{i >= r} s_i^2 <= cutoff * sum s_i^2, capped by maxdim (> 0).
int truncation_rank(const double* s, int n, double cutoff, int maxdim, int mindim);

}  // namespace la
}  // namespace tnfa
