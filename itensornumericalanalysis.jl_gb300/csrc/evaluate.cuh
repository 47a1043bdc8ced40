// Internal interface of the batched evaluation engine (shared by the SIMT
// kernels in evaluate.cu and the tensor-core kernels in evaluate_tc.cu).
#pragma once
#include <cuda.h>

#include "common.cuh"

namespace tnfa {

constexpr int EVAL_MAXC = 8;  // children per vertex handled by one contraction

// Where a child's message row for point p comes from: a message buffer
// (row p of a Pc x dim matrix plus a base-2 exponent per row) or, for a leaf
// child fused into its parent, row S[p] of the leaf tensor itself.
template <class T>
struct ChildSrc {
  const T* ptr;
  const int* exps;     // null for a fused leaf
  const uint8_t* S;    // site index of the leaf per point; null for a message
  int dim;
};

// One vertex contraction over all points of a chunk:
//   out[p, a] = sum_k A[p, k] * T_v[s_p][a][k],  A[p, k] = prod_c m_c[p, k_c]
// (k = mixed radix over the children, first child most significant), with
// the points grouped by their site value s_p (grp_*) so that a tile of rows
// shares one slice T_v[s].
template <class T>
struct VertexJob {
  int nchild;
  ChildSrc<T> ch[EVAL_MAXC];
  int K, chi_a, site_dim;
  const T* B;          // T_v, canonical layout [site][parent][children...]
  T* out;              // Pc x chi_a, natural point order
  int* out_exp;        // Pc
  const int* perm;     // grouped order -> point; null = identity
  const int* grp_off;  // [ngroups]
  const int* grp_cnt;  // [ngroups]
  const int* tile_start;  // [ngroups + 1]
  int ngroups;
  int Pc;
};

// Per-vertex grouping metadata lives in one int buffer:
//   [grp_off | grp_cnt | tile_start (ng+1) | cursor]  (ng = site_dim)
inline size_t group_meta_ints(int ng) { return (size_t)4 * ng + 1; }

// Tensor-core contraction of one vertex (evaluate_tc.cu).  Returns false when
// the shapes are outside what the tcgen05 kernel handles; the caller then
// uses the FP32 SIMT kernel.
bool tc_vertex_eligible(int nchild, const int* child_dims, int chi_a);
void tc_prepare_net(tnfa_ctx* ctx, const tnfa_net* net);  // BF16 hi/lo copies
void tc_contract_vertex(tnfa_ctx* ctx, const tnfa_net* net, int v, const VertexJob<float>& job,
                        int tile_rows, int* err);
int tc_tile_rows();
// 3-D BF16 tensor map {x_dim, y_dim, z_dim} (x contiguous) with a box of
// {64, box_y, box_z} elements and 128-byte swizzle.
CUtensorMap tc_make_map3(const void* base, int x_dim, int y_dim, int64_t z_dim, int box_y,
                         int box_z);

// Error-free sliced tensor-core contraction (evaluate_oz.cu): a vertex of two
// children evaluated from FP64 messages to FP64 messages on tcgen05.
bool oz_vertex_eligible(int nchild, const int* child_dims, int chi_a);
void oz_prepare_net(tnfa_ctx* ctx, const tnfa_net* net);  // digit planes of the tensors
void oz_contract_vertex(tnfa_ctx* ctx, const tnfa_net* net, int v, const VertexJob<double>& job,
                        int tile_rows, int* err);
int oz_tile_rows();

}  // namespace tnfa

