// Batched point evaluation of a tree tensor network function.
//
// Reference path (ITensorNumericalAnalysis.jl): evaluate
// (src/itensornetworkfunction.jl:96-112) = calculate_ind_values (digits by
// greedy subtraction, src/IndexMaps/abstractindexmap.jl:121-138) -> project
// (one-hot slice of every site leg, :84-94) -> scalar(tn; alg="bp") (exact on
// a tree).  It handles one point per call.
//
// Here all points of a chunk go through the tree vertex by vertex (children
// before parents):
//   1. k_digitize: coordinates -> site value s_v(p) of every vertex (u8).
//   2. per vertex: group the points by s_v (count / scan / scatter), so that a
//      tile of points shares one slice T_v[s].
//   3. per vertex: out[p, a] = sum_k A[p, k] T_v[s][a][k] with A the row-wise
//      Kronecker product of the children's messages.  Leaves are never
//      materialised: a parent reads the leaf slice T_leaf[s_leaf(p)] directly.
//      Each message row is rescaled by a power of two when it is read (exact)
//      and the exponent is carried per point, so deep trees neither underflow
//      nor overflow.
//   4. k_combine: product over the roots of the forest, times 2^exponent.
#include <algorithm>
#include <type_traits>

#include "evaluate.cuh"

namespace tnfa {

// ----------------------------------------------------------- digitize ----
struct DigitEntry {
  int col;     // column of X
  int base;
  int vertex;
  int stride;  // weight of this leg inside the vertex's site value
  double invb; // base^-digit, correctly rounded
  int start;   // first digit of a (variable, part): reload the remainder
};

__global__ void k_digitize(const double* __restrict__ X, int ncols, int Pc,
                           const DigitEntry* __restrict__ prog, int nprog, uint8_t* __restrict__ S,
                           int64_t ldS, int* __restrict__ err) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < Pc; p += gridDim.x * blockDim.x) {
    double xr = 0.0;
    for (int e = 0; e < nprog; ++e) {
      DigitEntry d = prog[e];
      if (d.start) {
        xr = X[(int64_t)p * ncols + d.col];
        if (!(xr >= 0.0) || !isfinite(xr)) {
          atomicOr(err, 1);
          xr = 0.0;
        }
      }
      // Largest digit value v with xr >= v * base^-digit; subtract it.
      int dig = 0;
      for (int v = d.base - 1; v >= 1; --v) {
        double t = (double)v * d.invb;
        if (xr >= t) {
          dig = v;
          xr -= t;
          break;
        }
      }
      uint8_t* sp = S + (int64_t)d.vertex * ldS + p;
      *sp = (uint8_t)(*sp + dig * d.stride);
    }
  }
}

// ----------------------------------------------------------- grouping ----
__global__ void k_group_count(const uint8_t* __restrict__ S, int Pc, int ng, int* __restrict__ cnt) {
  __shared__ int h[256];
  for (int i = threadIdx.x; i < ng; i += blockDim.x) h[i] = 0;
  __syncthreads();
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < Pc; p += gridDim.x * blockDim.x)
    atomicAdd(&h[S[p]], 1);
  __syncthreads();
  for (int i = threadIdx.x; i < ng; i += blockDim.x)
    if (h[i]) atomicAdd(&cnt[i], h[i]);
}

// Single thread: offsets, tile starts and scatter cursors from the counts.
__global__ void k_group_scan(int* meta, int ng, int tp) {
  int* off = meta;
  int* cnt = meta + ng;
  int* ts = meta + 2 * ng;
  int* cur = meta + 3 * ng + 1;
  int o = 0, t = 0;
  for (int g = 0; g < ng; ++g) {
    off[g] = o;
    cur[g] = o;
    ts[g] = t;
    o += cnt[g];
    t += (cnt[g] + tp - 1) / tp;
  }
  ts[ng] = t;
}

// Identity grouping (vertex without site legs).
__global__ void k_group_identity(int* meta, int Pc, int tp) {
  meta[0] = 0;
  meta[1] = Pc;
  meta[2] = 0;
  meta[3] = (Pc + tp - 1) / tp;
  meta[4] = 0;
}

constexpr int SCATTER_ITEMS = 8;
__global__ void k_group_scatter(const uint8_t* __restrict__ S, int Pc, int ng, int* __restrict__ cur,
                                int* __restrict__ perm) {
  __shared__ int h[256];
  __shared__ int base[256];
  for (int i = threadIdx.x; i < ng; i += blockDim.x) h[i] = 0;
  __syncthreads();
  int p0 = blockIdx.x * blockDim.x * SCATTER_ITEMS;
  int loc[SCATTER_ITEMS];
  int grp[SCATTER_ITEMS];
#pragma unroll
  for (int i = 0; i < SCATTER_ITEMS; ++i) {
    int p = p0 + i * blockDim.x + threadIdx.x;
    grp[i] = -1;
    if (p < Pc) {
      grp[i] = S[p];
      loc[i] = atomicAdd(&h[grp[i]], 1);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < ng; i += blockDim.x) base[i] = h[i] ? atomicAdd(&cur[i], h[i]) : 0;
  __syncthreads();
#pragma unroll
  for (int i = 0; i < SCATTER_ITEMS; ++i) {
    int p = p0 + i * blockDim.x + threadIdx.x;
    if (grp[i] >= 0) perm[base[grp[i]] + loc[i]] = p;
  }
}

// ------------------------------------------------------- contraction ----
template <class T>
__device__ inline bool locate_tile(const VertexJob<T>& j, int tp, int b, int& row0, int& nrows,
                                   int& g) {
  int ng = j.ngroups;
  if (b >= j.tile_start[ng]) return false;
  int gg = 0;
  while (gg + 1 < ng && j.tile_start[gg + 1] <= b) ++gg;
  g = gg;
  row0 = j.grp_off[gg] + (b - j.tile_start[gg]) * tp;
  nrows = min(tp, j.grp_off[gg] + j.grp_cnt[gg] - row0);
  return nrows > 0;
}

template <class T> struct Frexp;
template <> struct Frexp<double> {
  __device__ static int e(double m) {
    int ex = 0;
    frexp(m, &ex);
    return ex;
  }
};
template <> struct Frexp<float> {
  __device__ static int e(float m) {
    int ex = 0;
    frexpf(m, &ex);
    return ex;
  }
};

// Load the message rows of every child for the tile's points into shared
// memory (child c at rows + choff_c * tp, row-major tp x dim_c), rescale each
// row by 2^-e so that its largest entry lies in [0.5, 1), and accumulate the
// exponents of the tile's points into eacc.  The gather issues LU loads per
// thread before storing any, so that a tile's rows are in flight together
// rather than one load latency per element.
template <class T>
__device__ void load_children(const VertexJob<T>& j, const int* pts, int nrows, int tp, T* rows,
                              int* eacc) {
  constexpr int LU = 8;
  int off = 0;
  for (int c = 0; c < j.nchild; ++c) {
    const ChildSrc<T> s = j.ch[c];
    T* dst = rows + (int64_t)off * tp;
    const int n = tp * s.dim;
    for (int i0 = threadIdx.x; i0 < n; i0 += blockDim.x * LU) {
      T v[LU];
#pragma unroll
      for (int u = 0; u < LU; ++u) {
        const int idx = i0 + u * (int)blockDim.x;
        const int r = idx / s.dim, i = idx - r * s.dim;
        v[u] = Sc<T>::zero();
        if (idx < n && r < nrows) {
          const int p = pts[r];
          v[u] = s.S ? s.ptr[(int64_t)s.S[p] * s.dim + i] : s.ptr[(int64_t)p * s.dim + i];
        }
      }
#pragma unroll
      for (int u = 0; u < LU; ++u) {
        const int idx = i0 + u * (int)blockDim.x;
        if (idx < n) dst[idx] = v[u];
      }
    }
    off += s.dim;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  off = 0;
  for (int c = 0; c < j.nchild; ++c) {
    const ChildSrc<T> s = j.ch[c];
    T* base = rows + (int64_t)off * tp;
    for (int r = warp; r < nrows; r += nw) {
      T* row = base + (int64_t)r * s.dim;
      decltype(Sc<T>::absmax(Sc<T>::zero())) m = 0;
      for (int i = lane; i < s.dim; i += 32) m = max(m, Sc<T>::absmax(row[i]));
      for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
      int ex = (m > 0) ? Frexp<decltype(m)>::e(m) : 0;
      if (ex != 0)
        for (int i = lane; i < s.dim; i += 32) row[i] = Sc<T>::scale2(row[i], -ex);
      if (lane == 0) atomicAdd(&eacc[r], ex + (s.exps ? s.exps[pts[r]] : 0));
    }
    off += s.dim;
  }
  __syncthreads();
}

// A[r, k] for the tile: product of the children's row entries.
template <class T>
__device__ inline T kr_entry(const VertexJob<T>& j, const T* rows, int tp, int r, int k) {
  T a = Sc<T>::one();
  int off_end = 0;
  for (int c = 0; c < j.nchild; ++c) off_end += j.ch[c].dim;
  int off = off_end;
  for (int c = j.nchild - 1; c >= 0; --c) {
    int d = j.ch[c].dim;
    off -= d;
    int kc = k % d;
    k /= d;
    a = a * rows[(int64_t)off * tp + (int64_t)r * d + kc];
  }
  return a;
}

// General SIMT contraction: CTA tile = TP points x TA output columns, 256
// threads as (256 / (TA / 4)) row threads x (TA / 4) column threads, each
// with a (TP / row threads) x 4 register micro-tile; K streamed in chunks of
// 16.  TA follows the parent bond (32, 64 or 128) so that thin bonds do not
// pay for idle columns.
template <class T, int TP, int TA>
__global__ void __launch_bounds__(256) k_contract_gemm(const VertexJob<T> j) {
  constexpr int KC = 16, CT = TA / 4, RT = 256 / CT, RM = TP / RT;
  static_assert(RM >= 1 && RM * RT == TP, "tile rows must cover the row threads");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int row0, nrows, g;
  if (!locate_tile(j, TP, blockIdx.x, row0, nrows, g)) return;
  const int a0 = blockIdx.y * TA;
  int sumdim = 0;
  for (int c = 0; c < j.nchild; ++c) sumdim += j.ch[c].dim;
  T* rows = (T*)smem_raw;
  T* As = rows + (int64_t)sumdim * TP;  // [KC][TP]
  T* Bs = As + KC * TP;                 // [KC][TA]
  int* pts = (int*)(Bs + KC * TA);
  int* eacc = pts + TP;
  for (int r = threadIdx.x; r < TP; r += blockDim.x) {
    pts[r] = r < nrows ? (j.perm ? j.perm[row0 + r] : row0 + r) : 0;
    eacc[r] = 0;
  }
  __syncthreads();
  load_children(j, pts, nrows, TP, rows, eacc);

  const T* Bg = j.B + (int64_t)g * j.chi_a * j.K;
  const int tx = threadIdx.x % CT, ty = threadIdx.x / CT;
  T acc[RM][4];
#pragma unroll
  for (int i = 0; i < RM; ++i)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[i][q] = Sc<T>::zero();

  for (int k0 = 0; k0 < j.K; k0 += KC) {
    for (int idx = threadIdx.x; idx < KC * TP; idx += blockDim.x) {
      int kk = idx / TP, r = idx - kk * TP;
      int k = k0 + kk;
      As[idx] = (k < j.K && r < nrows) ? kr_entry(j, rows, TP, r, k) : Sc<T>::zero();
    }
    for (int idx = threadIdx.x; idx < KC * TA; idx += blockDim.x) {
      int a = idx / KC, kk = idx - a * KC;
      int k = k0 + kk, aa = a0 + a;
      Bs[kk * TA + a] = (k < j.K && aa < j.chi_a) ? Bg[(int64_t)aa * j.K + k] : Sc<T>::zero();
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < KC; ++kk) {
      T av[RM], bv[4];
#pragma unroll
      for (int i = 0; i < RM; ++i) av[i] = As[kk * TP + ty * RM + i];
#pragma unroll
      for (int q = 0; q < 4; ++q) bv[q] = Bs[kk * TA + tx + CT * q];
#pragma unroll
      for (int i = 0; i < RM; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[i][q] = Sc<T>::fma(av[i], bv[q], acc[i][q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < RM; ++i) {
    int r = ty * RM + i;
    if (r >= nrows) continue;
    int p = pts[r];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int a = a0 + tx + CT * q;
      if (a < j.chi_a) j.out[(int64_t)p * j.chi_a + a] = acc[i][q];
    }
  }
  if (blockIdx.y == 0)
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) j.out_exp[pts[r]] = eacc[r];
}

// Narrow outputs (chi_a <= 16): one warp per point, lanes split K, shuffle
// reduction.  Used at the roots (chi_a = 1) and on thin bonds.
template <class T, int NA>
__global__ void __launch_bounds__(256) k_contract_narrow(const VertexJob<T> j) {
  constexpr int TP = 8;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int row0, nrows, g;
  if (!locate_tile(j, TP, blockIdx.x, row0, nrows, g)) return;
  int sumdim = 0;
  for (int c = 0; c < j.nchild; ++c) sumdim += j.ch[c].dim;
  T* rows = (T*)smem_raw;
  int* pts = (int*)(rows + (int64_t)sumdim * TP);
  int* eacc = pts + TP;
  for (int r = threadIdx.x; r < TP; r += blockDim.x) {
    pts[r] = r < nrows ? (j.perm ? j.perm[row0 + r] : row0 + r) : 0;
    eacc[r] = 0;
  }
  __syncthreads();
  load_children(j, pts, nrows, TP, rows, eacc);
  const int lane = threadIdx.x & 31, r = threadIdx.x >> 5;
  if (r >= nrows) return;
  const T* Bg = j.B + (int64_t)g * j.chi_a * j.K;
  T acc[NA];
#pragma unroll
  for (int q = 0; q < NA; ++q) acc[q] = Sc<T>::zero();
  const int dl = j.nchild ? j.ch[j.nchild - 1].dim : 1;
  if (j.nchild >= 1 && j.nchild <= 2 && dl >= 16) {
    // lanes over the last child's entries, a loop over the other child's:
    // no index decoding in the loop
    const int offl = sumdim - dl;
    const int Ko = j.K / dl;
    const T* ml = rows + (int64_t)offl * TP + (int64_t)r * dl;
    const T* m0 = rows + (int64_t)r * (j.nchild == 2 ? j.ch[0].dim : 0);
    for (int ko = 0; ko < Ko; ++ko) {
      const T ao = j.nchild == 2 ? m0[ko] : Sc<T>::one();
      const T* Bk = Bg + (int64_t)ko * dl;
      for (int kl = lane; kl < dl; kl += 32) {
        const T a = ao * ml[kl];
#pragma unroll
        for (int q = 0; q < NA; ++q)
          acc[q] = Sc<T>::fma(a, q < j.chi_a ? Bk[(int64_t)q * j.K + kl] : Sc<T>::zero(), acc[q]);
      }
    }
  } else {
    for (int k = lane; k < j.K; k += 32) {
      T a = kr_entry(j, rows, TP, r, k);
#pragma unroll
      for (int q = 0; q < NA; ++q)
        acc[q] = Sc<T>::fma(a, q < j.chi_a ? Bg[(int64_t)q * j.K + k] : Sc<T>::zero(), acc[q]);
    }
  }
  int p = pts[r];
#pragma unroll
  for (int q = 0; q < NA; ++q) {
    if (q >= j.chi_a) continue;
    T v = acc[q];
    for (int o = 16; o; o >>= 1) {
      if constexpr (sizeof(T) == 16) {
        cplx z = *(cplx*)&v;
        z.re += __shfl_xor_sync(0xffffffffu, z.re, o);
        z.im += __shfl_xor_sync(0xffffffffu, z.im, o);
        v = *(T*)&z;
      } else {
        v = v + __shfl_xor_sync(0xffffffffu, v, o);
      }
    }
    if (lane == 0) j.out[(int64_t)p * j.chi_a + q] = v;
  }
  if (lane == 0) j.out_exp[p] = eacc[r];
}

// ------------------------------------------------------------ combine ----
template <class T>
__device__ inline void write_out(void* out, int kind, int64_t p, int64_t P, T v, int e);
template <>
__device__ inline void write_out<double>(void* out, int kind, int64_t p, int64_t P, double v, int e) {
  if (kind == TNFA_OUT_F64) {
    ((double*)out)[p] = scalbn(v, e);
  } else if (kind == TNFA_OUT_F32) {
    ((float*)out)[p] = (float)scalbn(v, e);
  } else {  // scaled f32
    int ex = 0;
    double m = frexp(v, &ex);
    ((float*)out)[p] = (float)m;
    ((int*)((float*)out + P))[p] = (v == 0.0) ? 0 : e + ex;
  }
}
template <>
__device__ inline void write_out<float>(void* out, int kind, int64_t p, int64_t P, float v, int e) {
  write_out<double>(out, kind, p, P, (double)v, e);
}
template <>
__device__ inline void write_out<cplx>(void* out, int kind, int64_t p, int64_t P, cplx v, int e) {
  ((cplx*)out)[p] = cplx{scalbn(v.re, e), scalbn(v.im, e)};
}

template <class T>
__global__ void k_combine(const T* __restrict__ rootv, const int* __restrict__ roote, int nroots,
                          int Pc, void* out, int kind, int64_t P, int64_t p0) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < Pc; p += gridDim.x * blockDim.x) {
    T v = Sc<T>::one();
    int e = 0;
    for (int r = 0; r < nroots; ++r) {
      v = v * rootv[(int64_t)r * Pc + p];
      e += roote[(int64_t)r * Pc + p];
    }
    write_out<T>(out, kind, p0 + p, P, v, e);
  }
}

// --------------------------------------------- fused small-bond path ----
// For networks whose bonds are all small (chi <= 16, or chi <= 32 on paths),
// one thread walks its point through the whole tree: digits from the digit
// program, then the vertices in post-order, each a chain of small
// matrix-vector products against the network's tensors held in shared
// memory, the messages in shared memory ([slot][entry][thread], conflict
// free), each message rescaled by a power of two with the exponent carried.
// One launch per chunk instead of about four per vertex, and no message
// traffic through HBM.
struct FusedStep {
  int off;       // element offset of the vertex tensor in the shared copy
  int vertex;
  int chi_a;     // parent bond (1 at a root)
  int nchild;    // 0, 1 or 2
  int d1, d2;    // child bonds (1 when absent)
  int in1, in2;  // message slots of the children
  int out;       // message slot of this vertex; -1 at a root
};
constexpr int FUSED_MAXV = 128;

template <class T, int CHI>
__global__ void __launch_bounds__(128) k_eval_fused(
    const double* __restrict__ X, int ncols, int Pc, const DigitEntry* __restrict__ prog, int nprog,
    const FusedStep* __restrict__ steps, int nsteps, const T* __restrict__ tensors, int n_elem,
    int V, int nslots, size_t off_msg, size_t off_prog, size_t off_steps, void* out, int kind,
    int64_t P, int64_t p0, int* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // the tensors in shared memory when they fit (off_msg > 0), else read in
  // place (a few hundred KB at most: they stay in L1 / L2)
  const T* ts = off_msg ? (const T*)smem_raw : tensors;
  T* msg = (T*)(smem_raw + off_msg);
  DigitEntry* pg = (DigitEntry*)(smem_raw + off_prog);
  FusedStep* st = (FusedStep*)(smem_raw + off_steps);
  if (off_msg)
    for (int i = threadIdx.x; i < n_elem; i += blockDim.x) ((T*)smem_raw)[i] = tensors[i];
  for (int i = threadIdx.x; i < nprog; i += blockDim.x) pg[i] = prog[i];
  for (int i = threadIdx.x; i < nsteps; i += blockDim.x) st[i] = steps[i];
  __syncthreads();
  const int tpb = blockDim.x, tid = threadIdx.x;
  auto M = [&](int slot, int k) -> T& { return msg[((size_t)slot * CHI + k) * tpb + tid]; };
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < Pc; p += gridDim.x * blockDim.x) {
    uint8_t dg[FUSED_MAXV];
    for (int v = 0; v < V; ++v) dg[v] = 0;
    double xr = 0.0;
    for (int e = 0; e < nprog; ++e) {
      const DigitEntry d = pg[e];
      if (d.start) {
        xr = X[(int64_t)p * ncols + d.col];
        if (!(xr >= 0.0) || !isfinite(xr)) {
          atomicOr(err, 1);
          xr = 0.0;
        }
      }
      int dig = 0;
      for (int v = d.base - 1; v >= 1; --v) {
        const double t = (double)v * d.invb;
        if (xr >= t) {
          dig = v;
          xr -= t;
          break;
        }
      }
      dg[d.vertex] = (uint8_t)(dg[d.vertex] + dig * d.stride);
    }
    T val = Sc<T>::one();
    int ex_acc = 0;
    for (int i = 0; i < nsteps; ++i) {
      const FusedStep s = st[i];
      const int K = s.d1 * s.d2;
      const T* Tv = ts + s.off + (int64_t)dg[s.vertex] * s.chi_a * K;
      // the last child's message in registers; the first child's (two
      // children) read from its slot inside the loop, which the output slot
      // never aliases (it is taken before the children's slots are freed)
      const int dl = s.nchild == 2 ? s.d2 : s.d1;
      const int il = s.nchild == 2 ? s.in2 : s.in1;
      T ml[CHI];
#pragma unroll
      for (int c = 0; c < CHI; ++c) ml[c] = (s.nchild > 0 && c < dl) ? M(il, c) : Sc<T>::zero();
      decltype(Sc<T>::absmax(Sc<T>::zero())) mx = 0;
      T rv = Sc<T>::zero();
      for (int a = 0; a < s.chi_a; ++a) {
        const T* Ta = Tv + (int64_t)a * K;
        T acc = Sc<T>::zero();
        if (s.nchild == 0) {
          acc = Ta[0];
        } else if (s.nchild == 1) {
#pragma unroll
          for (int c = 0; c < CHI; ++c)
            if (c < dl) acc = Sc<T>::fma(Ta[c], ml[c], acc);
        } else {
          for (int b = 0; b < s.d1; ++b) {
            const T* Tb = Ta + b * dl;
            T in = Sc<T>::zero();
#pragma unroll
            for (int c = 0; c < CHI; ++c)
              if (c < dl) in = Sc<T>::fma(Tb[c], ml[c], in);
            acc = Sc<T>::fma(M(s.in1, b), in, acc);
          }
        }
        if (s.out < 0) {
          rv = acc;  // a root: its parent bond is 1
        } else {
          M(s.out, a) = acc;
          mx = max(mx, Sc<T>::absmax(acc));
        }
      }
      if (s.out < 0) {
        val = val * rv;
        continue;
      }
      const int ex = mx > 0 ? Frexp<decltype(mx)>::e(mx) : 0;
      ex_acc += ex;
      if (ex != 0)
        for (int a = 0; a < s.chi_a; ++a) M(s.out, a) = Sc<T>::scale2(M(s.out, a), -ex);
    }
    write_out<T>(out, kind, p0 + p, P, val, ex_acc);
  }
}

struct FusedPlan {
  bool ok = false;
  int chi = 0;  // CHI of the kernel
  int nslots = 0, tpb = 0;
  std::vector<FusedStep> steps;
  size_t off_msg = 0, off_prog = 0, off_steps = 0, smem = 0;
};

// Whether the fused kernel takes this network, and its schedule (post-order,
// message slots recycled as children are consumed) and shared-memory layout.
static FusedPlan make_fused_plan(const Topo& T, size_t tsize, size_t nprog, int64_t npoints) {
  FusedPlan F;
  const char* env = getenv("TNFA_EVAL_FUSED");
  if (env && *env == '0') return F;
  if (T.V > FUSED_MAXV) return F;
  int chimax = 1, maxch = 0;
  for (int v = 0; v < T.V; ++v) {
    chimax = std::max(chimax, T.link[v]);
    maxch = std::max(maxch, (int)T.children[v].size());
    if (T.site_dim[v] > 256) return F;
  }
  if (maxch > 2 || chimax > 32 || (chimax > 16 && maxch > 1)) return F;
  // a thread per point: above chi 8 a few thousand points leave the GPU
  // mostly idle, where the per-vertex kernels spread a point over a warp
  if (chimax > 8 && npoints < 32768) return F;
  if (T.n_elem * (int64_t)tsize > 4 * 1024 * 1024) return F;
  F.chi = chimax <= 2 ? 2 : chimax <= 4 ? 4 : chimax <= 8 ? 8 : chimax <= 16 ? 16 : 32;
  std::vector<int> slot(T.V, -1), free_slots;
  int n = 0;
  for (int r : T.roots()) {
    std::vector<std::pair<int, int>> stack{{r, 0}};
    while (!stack.empty()) {
      auto& [v, i] = stack.back();
      if (i < (int)T.children[v].size()) {
        const int c = T.children[v][i++];
        stack.push_back({c, 0});
        continue;
      }
      FusedStep s{};
      s.off = (int)T.off[v];
      s.vertex = v;
      s.chi_a = T.link[v];
      s.nchild = (int)T.children[v].size();
      s.d1 = s.nchild >= 1 ? T.link[T.children[v][0]] : 1;
      s.d2 = s.nchild >= 2 ? T.link[T.children[v][1]] : 1;
      s.in1 = s.nchild >= 1 ? slot[T.children[v][0]] : 0;
      s.in2 = s.nchild >= 2 ? slot[T.children[v][1]] : 0;
      // the output slot is taken before the children's are released, so it
      // never aliases a message the step still reads
      if (T.parent[v] >= 0) {
        if (free_slots.empty()) free_slots.push_back(n++);
        s.out = slot[v] = free_slots.back();
        free_slots.pop_back();
      } else {
        s.out = -1;
      }
      for (int c : T.children[v]) free_slots.push_back(slot[c]);
      F.steps.push_back(s);
      stack.pop_back();
    }
  }
  F.nslots = std::max(n, 1);
  auto al = [](size_t x) { return (x + 15) & ~(size_t)15; };
  // threads per block: as many as keep the messages within 64 KB, 32..128
  const size_t per_thread = (size_t)F.nslots * F.chi * tsize;
  F.tpb = (int)std::min<size_t>(128, std::max<size_t>(32, (64 * 1024 / per_thread) / 32 * 32));
  if ((size_t)F.tpb * per_thread > 64 * 1024) return F;
  const bool ts_smem = (size_t)T.n_elem * tsize <= 96 * 1024;
  F.off_msg = ts_smem ? al((size_t)T.n_elem * tsize) : 0;
  F.off_prog = al(F.off_msg + (size_t)F.tpb * per_thread);
  F.off_steps = al(F.off_prog + nprog * sizeof(DigitEntry));
  F.smem = F.off_steps + F.steps.size() * sizeof(FusedStep);
  F.ok = F.smem <= 200 * 1024;
  return F;
}

template <class T>
static void launch_fused(tnfa_ctx* ctx, const FusedPlan& F, const FusedStep* dsteps, const T* tensors,
                         const Topo& Tp, const double* Xc, int ncols, int Pc,
                         const DigitEntry* dprog, int nprog, void* o, int kind, int64_t Pout,
                         int64_t pofs, int* derr) {
  const int tpb = F.tpb;
  const unsigned grid = grid_for(Pc, tpb, ctx->sm_count * (2048 / tpb));
  double fl = 0;
  for (const auto& s : F.steps) fl += 2.0 * s.chi_a * s.d1 * s.d2;
  KernelScope ks(ctx, "eval_fused", fl * Pc, (double)Pc * (ncols * 8.0 + 8.0));
  auto go = [&](auto kern) {
    TNFA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)F.smem));
    kern<<<grid, tpb, F.smem, ctx->stream>>>(Xc, ncols, Pc, dprog, nprog, dsteps, (int)F.steps.size(),
                                             tensors, (int)Tp.n_elem, Tp.V, F.nslots, F.off_msg,
                                             F.off_prog, F.off_steps, o, kind, Pout, pofs, derr);
  };
  switch (F.chi) {
    case 2: go(k_eval_fused<T, 2>); break;
    case 4: go(k_eval_fused<T, 4>); break;
    case 8: go(k_eval_fused<T, 8>); break;
    case 16: go(k_eval_fused<T, 16>); break;
    default: go(k_eval_fused<T, 32>); break;
  }
  TNFA_LAUNCH_CHECK();
}

// -------------------------------------------------------------- driver ----
struct EvalPlan {
  std::vector<int> order;        // vertices computed, children before parents
  std::vector<char> fused_leaf;  // non-root leaf read directly by its parent
  std::vector<int> slot;         // message slot of a computed non-root vertex
  int nslots = 0;
  std::vector<int> roots;
  int chimax = 1;
};

// A vertex's output slot is taken while its children still hold theirs, so
// that it never shares memory with the messages it reads: the contraction
// kernels write their output as they go (tiles split over columns, the
// sliced kernel's two phases) and the autotuner runs one contraction several
// times over the same inputs.
static EvalPlan make_plan(const Topo& T) {
  EvalPlan P;
  P.fused_leaf.assign(T.V, 0);
  P.slot.assign(T.V, -1);
  P.roots = T.roots();
  for (int v = 0; v < T.V; ++v)
    if (T.parent[v] >= 0 && T.children[v].empty()) P.fused_leaf[v] = 1;
  // Post-order DFS per root keeps the number of live messages near the depth.
  for (int r : P.roots) {
    std::vector<std::pair<int, int>> st{{r, 0}};
    while (!st.empty()) {
      auto& [v, i] = st.back();
      if (i < (int)T.children[v].size()) {
        int c = T.children[v][i++];
        st.push_back({c, 0});
      } else {
        if (!P.fused_leaf[v]) P.order.push_back(v);
        st.pop_back();
      }
    }
  }
  std::vector<int> free_slots;
  int n = 0;
  for (int v : P.order) {
    if (T.parent[v] >= 0) {
      if (free_slots.empty()) free_slots.push_back(n++);
      P.slot[v] = free_slots.back();
      free_slots.pop_back();
      P.chimax = std::max(P.chimax, T.link[v]);
    }
    for (int c : T.children[v])
      if (!P.fused_leaf[c]) free_slots.push_back(P.slot[c]);
  }
  P.nslots = n;
  return P;
}

// Tile of k_contract_gemm for a parent bond chi_a > 16 and children rows of
// sumdim entries: TP x TA with TA the smallest of 32 / 64 / 128 covering
// chi_a, and TP = 4096 / TA (a 4 x 4 micro-tile per thread) while the
// children rows of the tile fit in shared memory, else TP = 1024 / TA (one
// row per thread).
struct GemmTile {
  int tp, ta;
};
static GemmTile gemm_tile(int chi_a, int sumdim, size_t tsize) {
  const size_t row_bytes = (size_t)sumdim * tsize;
  const int ta = chi_a <= 32 ? 32 : chi_a <= 64 ? 64 : 128;
  const int tp = 4096 / ta;
  if (row_bytes * tp + (size_t)16 * (tp + ta) * tsize <= 160 * 1024) return {tp, ta};
  return {1024 / ta, ta};
}

// Tiles worth timing against each other for one shape: the rule's choice
// first, then a 4 x 4 micro-tile at each other column width that fits.
static std::vector<GemmTile> gemm_tile_candidates(int chi_a, int sumdim, size_t tsize) {
  std::vector<GemmTile> c{gemm_tile(chi_a, sumdim, tsize)};
  const size_t row_bytes = (size_t)sumdim * tsize;
  for (int ta : {32, 64, 128}) {
    const int tp = 4096 / ta;
    if (row_bytes * tp + (size_t)16 * (tp + ta) * tsize > 160 * 1024) continue;
    if (tp == c[0].tp && ta == c[0].ta) continue;
    c.push_back({tp, ta});
  }
  return c;
}

template <class T> struct FamilyName;
template <> struct FamilyName<double> { static constexpr const char* v = "contract_f64"; };
template <> struct FamilyName<float> { static constexpr const char* v = "contract_f32"; };
template <> struct FamilyName<cplx> { static constexpr const char* v = "contract_c128"; };

template <class T>
static void launch_contract(tnfa_ctx* ctx, const VertexJob<T>& j, int Pc,
                            const GemmTile* tile = nullptr) {
  int sumdim = 0;
  for (int c = 0; c < j.nchild; ++c) sumdim += j.ch[c].dim;
  KernelScope ks(ctx, FamilyName<T>::v, 2.0 * Pc * (double)j.K * j.chi_a,
                 (double)sizeof(T) * ((double)Pc * (sumdim + j.chi_a) +
                                      (double)j.site_dim * j.chi_a * j.K));
  if (j.chi_a <= 16) {
    constexpr int TP = 8;
    size_t sm = (size_t)sumdim * TP * sizeof(T) + 2 * TP * sizeof(int);
    TNFA_CHECK(sm <= 200 * 1024, TNFA_ERR_UNSUPPORTED, "children bonds too large for evaluation");
    if (sm > 48 * 1024)
      for (auto kern : {k_contract_narrow<T, 1>, k_contract_narrow<T, 4>, k_contract_narrow<T, 16>})
        TNFA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    unsigned gx = (unsigned)((Pc + TP - 1) / TP + j.ngroups);
    // accumulators per lane: as many as the parent bond, so that they stay in registers
    if (j.chi_a == 1) k_contract_narrow<T, 1><<<gx, 256, sm, ctx->stream>>>(j);
    else if (j.chi_a <= 4) k_contract_narrow<T, 4><<<gx, 256, sm, ctx->stream>>>(j);
    else k_contract_narrow<T, 16><<<gx, 256, sm, ctx->stream>>>(j);
  } else {
    const GemmTile t = tile ? *tile : gemm_tile(j.chi_a, sumdim, sizeof(T));
    const size_t sm = (size_t)sumdim * sizeof(T) * t.tp + (size_t)16 * (t.tp + t.ta) * sizeof(T) +
                      2 * t.tp * sizeof(int);
    TNFA_CHECK(sm <= 200 * 1024, TNFA_ERR_UNSUPPORTED, "children bonds too large for evaluation");
    dim3 grid((unsigned)((Pc + t.tp - 1) / t.tp + j.ngroups), (unsigned)((j.chi_a + t.ta - 1) / t.ta));
    auto go = [&](auto kern) {
      if (sm > 48 * 1024)
        TNFA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      kern<<<grid, 256, sm, ctx->stream>>>(j);
    };
    if (t.ta == 32) t.tp == 128 ? go(k_contract_gemm<T, 128, 32>) : go(k_contract_gemm<T, 32, 32>);
    else if (t.ta == 64) t.tp == 64 ? go(k_contract_gemm<T, 64, 64>) : go(k_contract_gemm<T, 16, 64>);
    else t.tp == 32 ? go(k_contract_gemm<T, 32, 128>) : go(k_contract_gemm<T, 8, 128>);
  }
  TNFA_LAUNCH_CHECK();
}

static int contract_tile_rows(int chi_a, int sumdim, size_t tsize) {
  return chi_a <= 16 ? 8 : gemm_tile(chi_a, sumdim, tsize).tp;
}

template <class T>
static void evaluate_impl(tnfa_ctx* ctx, const tnfa_net* net, const T* tensors, const double* X,
                          int64_t P, int ncols, const std::vector<DigitEntry>& prog, int xmem,
                          void* out, int out_kind, int out_mem, bool use_tc,
                          bool use_oz = false) {
  const Topo& Tp = net->topo;
  const int V = Tp.V;
  EvalPlan plan = make_plan(Tp);
  const int nroots = (int)plan.roots.size();
  size_t out_elem = out_kind == TNFA_OUT_F64 ? 8 : out_kind == TNFA_OUT_F32 ? 4
                    : out_kind == TNFA_OUT_F32_SCALED ? 8 : 16;
  size_t per_point = (size_t)plan.nslots * (plan.chimax * sizeof(T) + sizeof(int)) + V + 4 +
                     (xmem == TNFA_MEM_HOST ? ncols * 8 : 0) + nroots * (sizeof(T) + 4) +
                     (out_mem == TNFA_MEM_HOST ? out_elem : 0);
  int64_t Pc_max = (int64_t)(ctx->eval_budget / per_point);
  Pc_max = std::max<int64_t>(256, std::min<int64_t>(Pc_max, int64_t(1) << 30));
  Pc_max = (Pc_max / 256) * 256;
  const int64_t Pc_alloc = std::min<int64_t>(P, Pc_max);
  const int Pcap = (int)std::max<int64_t>(Pc_alloc, 1);

  DBuf dprog(ctx, prog.size() * sizeof(DigitEntry));
  if (!prog.empty())
    TNFA_CUDA(cudaMemcpyAsync(dprog.p, prog.data(), prog.size() * sizeof(DigitEntry),
                              cudaMemcpyHostToDevice, ctx->stream));
  DBuf dS(ctx, (size_t)V * Pcap);
  DBuf dperm(ctx, (size_t)Pcap * 4);
  int maxsd = 1;
  for (int v = 0; v < V; ++v) maxsd = std::max(maxsd, Tp.site_dim[v]);
  DBuf dmeta(ctx, group_meta_ints(maxsd) * 4);
  DBuf derr(ctx, 4);
  TNFA_CUDA(cudaMemsetAsync(derr.p, 0, 4, ctx->stream));
  const size_t slot_vals = (size_t)Pcap * plan.chimax;
  DBuf dslots(ctx, (size_t)plan.nslots * slot_vals * sizeof(T));
  DBuf dslote(ctx, (size_t)plan.nslots * Pcap * sizeof(int));
  DBuf droot(ctx, (size_t)nroots * Pcap * sizeof(T));
  DBuf droote(ctx, (size_t)nroots * Pcap * sizeof(int));
  DBuf dX(ctx, xmem == TNFA_MEM_HOST ? (size_t)Pcap * ncols * 8 : 0);
  DBuf dout(ctx, out_mem == TNFA_MEM_HOST ? (size_t)Pcap * out_elem : 0);
  std::vector<int> root_index(V, -1);
  for (int r = 0; r < nroots; ++r) root_index[plan.roots[r]] = r;
  // small bonds everywhere: the whole tree per thread in one launch
  const FusedPlan F = make_fused_plan(Tp, sizeof(T), prog.size(), std::min<int64_t>(P, Pcap));
  DBuf dsteps;
  if (F.ok) {
    dsteps = DBuf(ctx, F.steps.size() * sizeof(FusedStep));
    TNFA_CUDA(cudaMemcpyAsync(dsteps.p, F.steps.data(), F.steps.size() * sizeof(FusedStep),
                              cudaMemcpyHostToDevice, ctx->stream));
  }

  for (int64_t p0 = 0; p0 < P; p0 += Pcap) {
    const int Pc = (int)std::min<int64_t>(Pcap, P - p0);
    const double* Xc;
    if (xmem == TNFA_MEM_HOST) {
      TNFA_CUDA(cudaMemcpyAsync(dX.p, X + p0 * ncols, (size_t)Pc * ncols * 8,
                                cudaMemcpyHostToDevice, ctx->stream));
      Xc = dX.as<double>();
    } else {
      Xc = X + p0 * ncols;
    }
    if (F.ok) {
      void* o = out_mem == TNFA_MEM_HOST ? dout.p : out;
      launch_fused<T>(ctx, F, dsteps.as<FusedStep>(), tensors, Tp, Xc, ncols, Pc,
                      dprog.as<DigitEntry>(), (int)prog.size(), o, out_kind,
                      out_mem == TNFA_MEM_HOST ? Pc : P, out_mem == TNFA_MEM_HOST ? 0 : p0,
                      derr.as<int>());
    } else {
    TNFA_CUDA(cudaMemsetAsync(dS.p, 0, (size_t)V * Pcap, ctx->stream));
    if (!prog.empty()) {
      KernelScope ks(ctx, "digitize", 0.0, (double)Pc * (ncols * 8.0 + V));
      k_digitize<<<grid_for(Pc, 256, 8 * 152 * 8), 256, 0, ctx->stream>>>(
          Xc, ncols, Pc, dprog.as<DigitEntry>(), (int)prog.size(), dS.as<uint8_t>(), (int64_t)Pcap,
          derr.as<int>());
      TNFA_LAUNCH_CHECK();
    }
    for (int v : plan.order) {
      VertexJob<T> j{};
      j.nchild = (int)Tp.children[v].size();
      TNFA_CHECK(j.nchild <= EVAL_MAXC, TNFA_ERR_UNSUPPORTED,
                 "vertex degree above " + std::to_string(EVAL_MAXC) + " children");
      int64_t K = 1;
      int sumdim = 0;
      int cdims[EVAL_MAXC];
      for (int i = 0; i < j.nchild; ++i) {
        int c = Tp.children[v][i];
        ChildSrc<T>& s = j.ch[i];
        s.dim = Tp.link[c];
        cdims[i] = s.dim;
        sumdim += s.dim;
        K *= s.dim;
        if (plan.fused_leaf[c]) {
          s.ptr = tensors + Tp.off[c];
          s.exps = nullptr;
          s.S = dS.as<uint8_t>() + (int64_t)c * Pcap;
        } else {
          s.ptr = (const T*)dslots.p + (size_t)plan.slot[c] * slot_vals;
          s.exps = dslote.as<int>() + (size_t)plan.slot[c] * Pcap;
          s.S = nullptr;
        }
      }
      TNFA_CHECK(K < (int64_t(1) << 31), TNFA_ERR_UNSUPPORTED, "contraction too large");
      j.K = (int)K;
      j.chi_a = Tp.link[v];
      j.site_dim = Tp.site_dim[v];
      j.B = tensors + Tp.off[v];
      j.Pc = Pc;
      if (Tp.parent[v] < 0) {
        j.out = (T*)droot.p + (size_t)root_index[v] * Pcap;
        j.out_exp = droote.as<int>() + (size_t)root_index[v] * Pcap;
      } else {
        j.out = (T*)dslots.p + (size_t)plan.slot[v] * slot_vals;
        j.out_exp = dslote.as<int>() + (size_t)plan.slot[v] * Pcap;
      }
      const bool tc = use_tc && j.site_dim <= 256 && tc_vertex_eligible(j.nchild, cdims, j.chi_a);
      const bool oz = use_oz && oz_vertex_eligible(j.nchild, cdims, j.chi_a);
      // SIMT shapes: the tile kept by the autotuner for this shape, else the rule's
      std::vector<GemmTile> cand;
      std::string key;
      int tp = tc   ? tc_tile_rows()
               : oz ? oz_tile_rows()
                    : contract_tile_rows(j.chi_a, sumdim, sizeof(T));
      if (!tc && !oz && j.chi_a > 16) {
        cand = gemm_tile_candidates(j.chi_a, sumdim, sizeof(T));
        key = std::string("simt:") + FamilyName<T>::v + ":" + std::to_string(j.chi_a) + ":";
        for (int i = 0; i < j.nchild; ++i) key += std::to_string(cdims[i]) + (i + 1 < j.nchild ? "x" : "");
        const int kept = tuned_choice(ctx, key);
        tp = cand[kept >= 0 ? kept : 0].tp;
      }
      const int ng = j.site_dim;
      int* meta = dmeta.as<int>();
      j.ngroups = ng;
      j.grp_off = meta;
      j.grp_cnt = meta + ng;
      j.tile_start = meta + 2 * ng;
      if (ng == 1) {
        KernelScope ks(ctx, "group", 0.0, 0.0);
        k_group_identity<<<1, 1, 0, ctx->stream>>>(meta, Pc, tp);
        TNFA_LAUNCH_CHECK();
        j.perm = nullptr;
      } else {
        TNFA_CHECK(ng <= 256, TNFA_ERR_UNSUPPORTED, "site dimension above 256 per vertex");
        const uint8_t* Sv = dS.as<uint8_t>() + (int64_t)v * Pcap;
        TNFA_CUDA(cudaMemsetAsync(meta + ng, 0, ng * sizeof(int), ctx->stream));
        KernelScope ks(ctx, "group", 0.0, (double)Pc * 6.0);
        k_group_count<<<grid_for(Pc, 256, 4 * 152), 256, 0, ctx->stream>>>(Sv, Pc, ng, meta + ng);
        k_group_scan<<<1, 1, 0, ctx->stream>>>(meta, ng, tp);
        unsigned gs = (unsigned)((Pc + 256 * SCATTER_ITEMS - 1) / (256 * SCATTER_ITEMS));
        k_group_scatter<<<gs, 256, 0, ctx->stream>>>(Sv, Pc, ng, meta + 3 * ng + 1, dperm.as<int>());
        TNFA_LAUNCH_CHECK();
        j.perm = dperm.as<int>();
      }
      if constexpr (std::is_same<T, float>::value) {
        if (tc) {
          tc_contract_vertex(ctx, net, v, j, tp, derr.as<int>());
          continue;
        }
      }
      if constexpr (std::is_same<T, double>::value) {
        if (oz) {
          oz_contract_vertex(ctx, net, v, j, tp, derr.as<int>());
          continue;
        }
      }
      if (cand.empty()) {
        launch_contract<T>(ctx, j, Pc);
        continue;
      }
      int cur_tp = tp;
      tune(ctx, key, (int)cand.size(), 2.0 * Pc * (double)j.K * j.chi_a, [&](int i) {
        if (cand[i].tp != cur_tp) {  // tile table for this candidate's rows per tile
          if (ng == 1) k_group_identity<<<1, 1, 0, ctx->stream>>>(meta, Pc, cand[i].tp);
          else k_group_scan<<<1, 1, 0, ctx->stream>>>(meta, ng, cand[i].tp);
          TNFA_LAUNCH_CHECK();
          cur_tp = cand[i].tp;
        }
        launch_contract<T>(ctx, j, Pc, &cand[i]);
      });
    }
    void* o = out_mem == TNFA_MEM_HOST ? dout.p : out;
    int64_t Pout = out_mem == TNFA_MEM_HOST ? Pc : P;
    int64_t pofs = out_mem == TNFA_MEM_HOST ? 0 : p0;
    KernelScope ksc(ctx, "combine", 0.0, (double)Pc * nroots * (sizeof(T) + 4.0));
    k_combine<T><<<grid_for(Pc, 256, 8192), 256, 0, ctx->stream>>>(
        (const T*)droot.p, droote.as<int>(), nroots, Pc, o, out_kind, Pout, pofs);
    TNFA_LAUNCH_CHECK();
    }
    if (out_mem == TNFA_MEM_HOST) {
      if (out_kind == TNFA_OUT_F32_SCALED) {
        TNFA_CUDA(cudaMemcpyAsync((float*)out + p0, dout.p, (size_t)Pc * 4, cudaMemcpyDeviceToHost,
                                  ctx->stream));
        TNFA_CUDA(cudaMemcpyAsync((int*)((float*)out + P) + p0, (float*)dout.p + Pc, (size_t)Pc * 4,
                                  cudaMemcpyDeviceToHost, ctx->stream));
      } else {
        TNFA_CUDA(cudaMemcpyAsync((char*)out + p0 * out_elem, dout.p, (size_t)Pc * out_elem,
                                  cudaMemcpyDeviceToHost, ctx->stream));
      }
    }
  }
  int herr = 0;
  TNFA_CUDA(cudaMemcpyAsync(&herr, derr.p, 4, cudaMemcpyDeviceToHost, ctx->stream));
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  TNFA_CHECK((herr & 2) == 0, TNFA_ERR_TIMEOUT,
             "a tensor-core pipeline wait ran out of its iteration budget");
  TNFA_CHECK(herr == 0, TNFA_ERR_DOMAIN,
             "a coordinate is negative or not finite (the digit map needs x >= 0)");
}

// Digit program of a network for the given variable list.
static std::vector<DigitEntry> make_digit_program(const Topo& T, int n_dims, const int32_t* dims,
                                                  int* ncols_out) {
  bool has_imag = false;
  int L = T.leg_off[T.V];
  for (int l = 0; l < L; ++l) {
    TNFA_CHECK(T.leg_kind[l] != TNFA_LEG_OPERATOR, TNFA_ERR_INVALID_ARGUMENT,
               "evaluate needs a function network, got an operator");
    if (T.leg_kind[l] == TNFA_LEG_IMAG) has_imag = true;
  }
  const int ncols = has_imag ? 2 * n_dims : n_dims;
  *ncols_out = ncols;
  struct LegRef {
    int var, kind, digit, leg, vertex, stride;
  };
  std::vector<LegRef> refs;
  for (int v = 0; v < T.V; ++v) {
    int stride = 1;
    for (int l = T.leg_off[v + 1] - 1; l >= T.leg_off[v]; --l) {
      refs.push_back({T.leg_var[l], T.leg_kind[l], T.leg_digit[l], l, v, stride});
      stride *= T.leg_dim[l];
    }
  }
  std::sort(refs.begin(), refs.end(), [](const LegRef& a, const LegRef& b) {
    if (a.var != b.var) return a.var < b.var;
    if (a.kind != b.kind) return a.kind < b.kind;
    return a.digit < b.digit;
  });
  std::vector<DigitEntry> prog;
  for (size_t i = 0; i < refs.size(); ++i) {
    const LegRef& r = refs[i];
    bool start = (i == 0 || refs[i - 1].var != r.var || refs[i - 1].kind != r.kind);
    int expect = start ? 1 : refs[i - 1].digit + 1;
    TNFA_CHECK(r.digit == expect, TNFA_ERR_TOPOLOGY,
               "digits of variable " + std::to_string(r.var) +
                   " are not 1..L (missing or repeated digit " + std::to_string(expect) + ")");
    int col = -1;
    for (int j = 0; j < n_dims; ++j)
      if (dims[j] == r.var) col = j;
    TNFA_CHECK(col >= 0, TNFA_ERR_INVALID_ARGUMENT,
               "variable " + std::to_string(r.var) + " has digits but is not listed in dims");
    int base = T.leg_dim[r.leg];
    TNFA_CHECK(base >= 2 && base <= 255, TNFA_ERR_UNSUPPORTED, "digit base outside 2..255");
    double bk = 1.0;
    for (int k = 0; k < r.digit; ++k) bk *= base;
    TNFA_CHECK(bk < 9007199254740992.0, TNFA_ERR_UNSUPPORTED, "base^digit above 2^53");
    DigitEntry d;
    d.col = has_imag ? 2 * col + (r.kind == TNFA_LEG_IMAG ? 1 : 0) : col;
    d.base = base;
    d.vertex = r.vertex;
    d.stride = r.stride;
    d.invb = 1.0 / bk;
    d.start = start ? 1 : 0;
    prog.push_back(d);
  }
  return prog;
}

}  // namespace tnfa

using namespace tnfa;

extern "C" int tnfa_evaluate(tnfa_ctx* ctx, const tnfa_net* net, const double* X, int64_t n_points,
                             int32_t n_dims, const int32_t* dims, int x_memory, void* out,
                             int out_kind, int out_memory, int precision) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(net, "evaluate");
  TNFA_CHECK(n_points >= 0, TNFA_ERR_INVALID_ARGUMENT, "n_points < 0");
  if (n_points == 0) return TNFA_OK;
  TNFA_CHECK(X && out && (n_dims == 0 || dims), TNFA_ERR_INVALID_ARGUMENT, "null X, out or dims");
  TNFA_CHECK(n_dims >= 0 && n_dims <= 64, TNFA_ERR_INVALID_ARGUMENT, "n_dims out of range");
  TNFA_CHECK(x_memory == TNFA_MEM_HOST || x_memory == TNFA_MEM_DEVICE, TNFA_ERR_INVALID_ARGUMENT,
             "bad x_memory");
  TNFA_CHECK(out_memory == TNFA_MEM_HOST || out_memory == TNFA_MEM_DEVICE,
             TNFA_ERR_INVALID_ARGUMENT, "bad out_memory");
  for (int v = 0; v < net->topo.V; ++v)
    TNFA_CHECK(net->topo.site_dim[v] <= 256, TNFA_ERR_UNSUPPORTED, "site dimension above 256");
  int ncols = 0;
  std::vector<DigitEntry> prog = make_digit_program(net->topo, n_dims, dims, &ncols);
  if (net->dtype == TNFA_C128) {
    TNFA_CHECK(out_kind == TNFA_OUT_C128, TNFA_ERR_DTYPE, "complex networks need TNFA_OUT_C128");
    TNFA_CHECK(precision == TNFA_PREC_F64, TNFA_ERR_UNSUPPORTED,
               "complex networks evaluate in TNFA_PREC_F64 only");
    evaluate_impl<cplx>(ctx, net, (const cplx*)net->d, X, n_points, ncols, prog, x_memory, out,
                        out_kind, out_memory, false);
  } else {
    TNFA_CHECK(out_kind == TNFA_OUT_F64 || out_kind == TNFA_OUT_F32 ||
                   out_kind == TNFA_OUT_F32_SCALED,
               TNFA_ERR_DTYPE, "real networks need a real output kind");
    if (precision == TNFA_PREC_F64) {
      TNFA_CHECK(net->dtype == TNFA_F64, TNFA_ERR_DTYPE, "TNFA_PREC_F64 needs an FP64 network");
      evaluate_impl<double>(ctx, net, (const double*)net->d, X, n_points, ncols, prog, x_memory,
                            out, out_kind, out_memory, false);
    } else if (precision == TNFA_PREC_MIXED) {
      // FP64 messages; two-child vertices of tensor-core shape take the
      // error-free sliced products, the rest the FP64 kernels
      oz_prepare_net(ctx, net);
      const double* t64 =
          net->dtype == TNFA_F64 ? (const double*)net->d : (const double*)net->d_f64;
      evaluate_impl<double>(ctx, net, t64, X, n_points, ncols, prog, x_memory, out, out_kind,
                            out_memory, false, true);
    } else if (precision == TNFA_PREC_F32 || precision == TNFA_PREC_MIXED_FAST) {
      const float* t32;
      if (net->dtype == TNFA_F32) {
        t32 = (const float*)net->d;
      } else {
        if (!net->d_f32) {
          net->d_f32 = dalloc(ctx, (size_t)net->topo.n_elem * 4);
          convert_f64_to_f32(ctx, (const double*)net->d, (float*)net->d_f32, net->topo.n_elem);
        }
        t32 = (const float*)net->d_f32;
      }
      if (precision == TNFA_PREC_MIXED_FAST) tc_prepare_net(ctx, net);
      evaluate_impl<float>(ctx, net, t32, X, n_points, ncols, prog, x_memory, out, out_kind,
                           out_memory, precision == TNFA_PREC_MIXED_FAST);
    } else {
      fail(TNFA_ERR_INVALID_ARGUMENT, "unknown precision");
    }
  }
  TNFA_API_END
}

// ------------------------------------------ evaluation without allocation ----
// tnfa_evaluate_noalloc: the same digitize / group / contract / combine
// kernels as tnfa_evaluate, with every scratch buffer carved out of one
// file-scope device array instead of the stream-ordered allocator.
#include <array>
#include <mutex>

namespace tnfa {
namespace {

constexpr size_t NOALLOC_BYTES = (size_t)32 << 20;  // 32 MiB, held by every device
__device__ __align__(256) unsigned char noalloc_scratch[NOALLOC_BYTES];

// Host code cannot use the array's name as a device address; this looks the
// address up once per device (with that device current) and caches it.
unsigned char* noalloc_base(int device) {
  static std::mutex mu;
  static std::vector<unsigned char*> addr;
  std::lock_guard<std::mutex> lock(mu);
  if ((int)addr.size() <= device) addr.resize(device + 1, nullptr);
  if (!addr[device]) {
    // the look-up needs `device` current; the caller's current device is
    // put back afterwards
    int prev = -1;
    TNFA_CUDA(cudaGetDevice(&prev));
    if (prev != device) TNFA_CUDA(cudaSetDevice(device));
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, noalloc_scratch);
    if (prev != device) TNFA_CUDA(cudaSetDevice(prev));
    TNFA_CUDA(e);
    addr[device] = (unsigned char*)p;
  }
  return addr[device];
}

struct Carve {
  unsigned char* base;
  size_t cap, used = 0;
  size_t take_off(size_t bytes) {
    const size_t off = (used + 255) & ~(size_t)255;
    used = off + bytes;
    return off;
  }
  void* take(size_t bytes) {
    const size_t off = take_off(bytes);
    TNFA_CHECK(used <= cap, TNFA_ERR_INVALID_ARGUMENT, "scratch overflow");
    return base + off;
  }
};

// The pieces evaluate_noalloc_impl carves for P points, in order: digit
// program, fused schedule, digits, permutation, group tables, error flag,
// message slots, slot exponents, root values, root exponents.  The fused
// small-bond path needs only the program, its schedule and the error flag.
template <class T>
std::array<size_t, 10> noalloc_sizes(const tnfa_net* net, const EvalPlan& plan, int64_t P,
                                     size_t prog_entries, const FusedPlan& F) {
  const Topo& Tp = net->topo;
  const int V = Tp.V;
  const int nroots = (int)plan.roots.size();
  int maxsd = 1;
  for (int v = 0; v < V; ++v) maxsd = std::max(maxsd, Tp.site_dim[v]);
  const size_t slot_vals = (size_t)P * plan.chimax;
  if (F.ok)
    return {prog_entries * sizeof(DigitEntry), F.steps.size() * sizeof(FusedStep), 0, 0, 0, 4,
            0, 0, 0, 0};
  return {prog_entries * sizeof(DigitEntry),
          0,
          (size_t)V * P,
          (size_t)P * 4,
          group_meta_ints(maxsd) * 4,
          4,
          (size_t)plan.nslots * slot_vals * sizeof(T),
          (size_t)plan.nslots * P * sizeof(int),
          (size_t)nroots * P * sizeof(T),
          (size_t)nroots * P * sizeof(int)};
}

// Scratch bytes evaluate_noalloc_impl carves for P points (256-byte aligned pieces).
template <class T>
size_t noalloc_bytes(const tnfa_net* net, int64_t P, size_t prog_entries) {
  Carve dry{nullptr, ~(size_t)0};
  const FusedPlan F = make_fused_plan(net->topo, sizeof(T), prog_entries, P);
  for (size_t s : noalloc_sizes<T>(net, make_plan(net->topo), P, prog_entries, F)) dry.take_off(s);
  return dry.used;
}

// The evaluation kernels over scratch carved from [base, base + cap).  With
// check, the digit program is copied in from the host and the call ends by
// reading the error flag (a host sync); without it (stream capture), the
// program must already sit at the start of the scratch and the call only
// enqueues work.  *err_flag receives the device address of the error flag.
template <class T>
void evaluate_noalloc_impl(tnfa_ctx* ctx, const tnfa_net* net, const T* tensors, const double* X,
                           int64_t P64, int ncols, const std::vector<DigitEntry>& prog, void* out,
                           int out_kind, unsigned char* base, size_t cap, bool check,
                           int** err_flag = nullptr) {
  const Topo& Tp = net->topo;
  const int V = Tp.V;
  EvalPlan plan = make_plan(Tp);
  const int nroots = (int)plan.roots.size();
  // Dry run of the carving to size the request before touching the device.
  const int64_t P = P64;
  const size_t slot_vals = (size_t)P * plan.chimax;
  const FusedPlan F = make_fused_plan(Tp, sizeof(T), prog.size(), P);
  const std::array<size_t, 10> sizes = noalloc_sizes<T>(net, plan, P, prog.size(), F);
  Carve dry{nullptr, cap};
  for (size_t s : sizes) dry.take_off(s);
  if (dry.used > cap) {
    const size_t per_point = (dry.used - prog.size() * sizeof(DigitEntry)) / (size_t)std::max<int64_t>(P, 1) + 1;
    fail(TNFA_ERR_INVALID_ARGUMENT,
         "tnfa_evaluate_noalloc: " + std::to_string(P) + " points need " +
             std::to_string(dry.used) + " bytes of scratch, above the fixed " +
             std::to_string(cap) + "; this network allows about " +
             std::to_string(cap / per_point) + " points per call");
  }
  Carve cv{base, cap};
  DigitEntry* dprog = (DigitEntry*)cv.take(sizes[0]);
  FusedStep* dsteps = (FusedStep*)cv.take(sizes[1]);
  uint8_t* dS = (uint8_t*)cv.take(sizes[2]);
  int* dperm = (int*)cv.take(sizes[3]);
  int* meta = (int*)cv.take(sizes[4]);
  int* derr = (int*)cv.take(sizes[5]);
  T* slots = (T*)cv.take(sizes[6]);
  int* slote = (int*)cv.take(sizes[7]);
  T* rootv = (T*)cv.take(sizes[8]);
  int* roote = (int*)cv.take(sizes[9]);
  const int Pc = (int)P;
  // the array keeps the previous call's contents: clear what must start at 0
  if (err_flag) *err_flag = derr;
  TNFA_CUDA(cudaMemsetAsync(derr, 0, 4, ctx->stream));
  if (F.ok) {
    if (check) {
      if (!prog.empty())
        TNFA_CUDA(cudaMemcpyAsync(dprog, prog.data(), sizes[0], cudaMemcpyHostToDevice, ctx->stream));
      TNFA_CUDA(cudaMemcpyAsync(dsteps, F.steps.data(), sizes[1], cudaMemcpyHostToDevice, ctx->stream));
    }
    launch_fused<T>(ctx, F, dsteps, tensors, Tp, X, ncols, Pc, dprog, (int)prog.size(), out, out_kind,
                    P, 0, derr);
  } else {
  TNFA_CUDA(cudaMemsetAsync(dS, 0, (size_t)V * P, ctx->stream));
  if (!prog.empty()) {
    if (check)
      TNFA_CUDA(cudaMemcpyAsync(dprog, prog.data(), sizes[0], cudaMemcpyHostToDevice, ctx->stream));
    k_digitize<<<grid_for(Pc, 256, 8 * 152 * 8), 256, 0, ctx->stream>>>(
        X, ncols, Pc, dprog, (int)prog.size(), dS, (int64_t)P, derr);
    TNFA_LAUNCH_CHECK();
  }
  std::vector<int> root_index(V, -1);
  for (int r = 0; r < nroots; ++r) root_index[plan.roots[r]] = r;
  for (int v : plan.order) {
    VertexJob<T> j{};
    j.nchild = (int)Tp.children[v].size();
    TNFA_CHECK(j.nchild <= EVAL_MAXC, TNFA_ERR_UNSUPPORTED, "vertex degree too high");
    int64_t K = 1;
    int sumdim = 0;
    for (int i = 0; i < j.nchild; ++i) {
      const int c = Tp.children[v][i];
      ChildSrc<T>& s = j.ch[i];
      s.dim = Tp.link[c];
      sumdim += s.dim;
      K *= s.dim;
      if (plan.fused_leaf[c]) {
        s.ptr = tensors + Tp.off[c];
        s.exps = nullptr;
        s.S = dS + (int64_t)c * P;
      } else {
        s.ptr = slots + (size_t)plan.slot[c] * slot_vals;
        s.exps = slote + (size_t)plan.slot[c] * P;
        s.S = nullptr;
      }
    }
    TNFA_CHECK(K < (int64_t(1) << 31), TNFA_ERR_UNSUPPORTED, "contraction too large");
    j.K = (int)K;
    j.chi_a = Tp.link[v];
    j.site_dim = Tp.site_dim[v];
    j.B = tensors + Tp.off[v];
    j.Pc = Pc;
    if (Tp.parent[v] < 0) {
      j.out = rootv + (size_t)root_index[v] * P;
      j.out_exp = roote + (size_t)root_index[v] * P;
    } else {
      j.out = slots + (size_t)plan.slot[v] * slot_vals;
      j.out_exp = slote + (size_t)plan.slot[v] * P;
    }
    const int tp = contract_tile_rows(j.chi_a, sumdim, sizeof(T));
    const int ng = j.site_dim;
    j.ngroups = ng;
    j.grp_off = meta;
    j.grp_cnt = meta + ng;
    j.tile_start = meta + 2 * ng;
    if (ng == 1) {
      k_group_identity<<<1, 1, 0, ctx->stream>>>(meta, Pc, tp);
      TNFA_LAUNCH_CHECK();
      j.perm = nullptr;
    } else {
      TNFA_CHECK(ng <= 256, TNFA_ERR_UNSUPPORTED, "site dimension above 256 per vertex");
      const uint8_t* Sv = dS + (int64_t)v * P;
      TNFA_CUDA(cudaMemsetAsync(meta + ng, 0, ng * sizeof(int), ctx->stream));
      k_group_count<<<grid_for(Pc, 256, 4 * 152), 256, 0, ctx->stream>>>(Sv, Pc, ng, meta + ng);
      k_group_scan<<<1, 1, 0, ctx->stream>>>(meta, ng, tp);
      const unsigned gs = (unsigned)((Pc + 256 * SCATTER_ITEMS - 1) / (256 * SCATTER_ITEMS));
      k_group_scatter<<<gs, 256, 0, ctx->stream>>>(Sv, Pc, ng, meta + 3 * ng + 1, dperm);
      TNFA_LAUNCH_CHECK();
      j.perm = dperm;
    }
    launch_contract<T>(ctx, j, Pc);
  }
  k_combine<T><<<grid_for(Pc, 256, 8192), 256, 0, ctx->stream>>>(rootv, roote, nroots, Pc, out,
                                                                   out_kind, P, 0);
  TNFA_LAUNCH_CHECK();
  }
  if (!check) return;
  int herr = 0;
  TNFA_CUDA(cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, ctx->stream));
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  TNFA_CHECK(herr == 0, TNFA_ERR_DOMAIN,
             "a coordinate is negative or not finite (the digit map needs x >= 0)");
}

}  // namespace
}  // namespace tnfa

extern "C" int tnfa_evaluate_noalloc(tnfa_ctx* ctx, const tnfa_net* net, const double* X,
                                     int64_t n_points, int32_t n_dims, const int32_t* dims,
                                     void* out, int out_kind, int precision) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(net, "evaluate_noalloc");
  TNFA_CHECK(n_points >= 0, TNFA_ERR_INVALID_ARGUMENT, "n_points < 0");
  if (n_points == 0) return TNFA_OK;
  TNFA_CHECK(X && out && (n_dims == 0 || dims), TNFA_ERR_INVALID_ARGUMENT, "null X, out or dims");
  TNFA_CHECK(n_dims >= 0 && n_dims <= 64, TNFA_ERR_INVALID_ARGUMENT, "n_dims out of range");
  TNFA_CHECK(n_points < (int64_t(1) << 31), TNFA_ERR_INVALID_ARGUMENT, "too many points");
  for (int v = 0; v < net->topo.V; ++v)
    TNFA_CHECK(net->topo.site_dim[v] <= 256, TNFA_ERR_UNSUPPORTED, "site dimension above 256");
  int ncols = 0;
  std::vector<DigitEntry> prog = make_digit_program(net->topo, n_dims, dims, &ncols);
  if (net->dtype == TNFA_C128) {
    TNFA_CHECK(out_kind == TNFA_OUT_C128 && precision == TNFA_PREC_F64, TNFA_ERR_DTYPE,
               "complex networks: TNFA_OUT_C128 and TNFA_PREC_F64");
    evaluate_noalloc_impl<cplx>(ctx, net, (const cplx*)net->d, X, n_points, ncols, prog, out,
                                out_kind, noalloc_base(ctx->device), NOALLOC_BYTES, true);
  } else {
    TNFA_CHECK(out_kind == TNFA_OUT_F64 || out_kind == TNFA_OUT_F32 ||
                   out_kind == TNFA_OUT_F32_SCALED,
               TNFA_ERR_DTYPE, "real networks need a real output kind");
    if (precision == TNFA_PREC_F64 && net->dtype == TNFA_F64)
      evaluate_noalloc_impl<double>(ctx, net, (const double*)net->d, X, n_points, ncols, prog, out,
                                    out_kind, noalloc_base(ctx->device), NOALLOC_BYTES, true);
    else if (precision == TNFA_PREC_F32 && net->dtype == TNFA_F32)
      evaluate_noalloc_impl<float>(ctx, net, (const float*)net->d, X, n_points, ncols, prog, out,
                                   out_kind, noalloc_base(ctx->device), NOALLOC_BYTES, true);
    else
      fail(TNFA_ERR_UNSUPPORTED,
           "tnfa_evaluate_noalloc computes in the network's own type: TNFA_PREC_F64 on FP64 "
           "networks or TNFA_PREC_F32 on FP32 networks");
  }
  TNFA_API_END
}

// ------------------------------------------------ captured evaluation ----
// tnfa_eval_plan: the no-allocation kernel sequence for fixed device buffers
// (X, out) and a fixed point count, captured once into a CUDA graph over
// scratch the plan owns, then replayed with one graph launch per call.  For
// small batches evaluation is launch-bound (about four launches per vertex),
// and the replay removes the per-launch host cost.
struct tnfa_eval_plan {
  tnfa_ctx* ctx = nullptr;
  const tnfa_net* net = nullptr;
  void* scratch = nullptr;
  int* derr = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t n_points = 0;
};

namespace tnfa {
namespace {
void plan_free(tnfa_eval_plan* p) {
  if (!p) return;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->scratch) cudaFree(p->scratch);
  if (p->ctx) ctx_release(p->ctx);
  delete p;
}

template <class T>
void plan_build(tnfa_eval_plan* p, const T* tensors, const double* X, int ncols,
                const std::vector<DigitEntry>& prog, void* out, int out_kind) {
  tnfa_ctx* ctx = p->ctx;
  const size_t bytes = noalloc_bytes<T>(p->net, p->n_points, prog.size());
  TNFA_CUDA(cudaMalloc(&p->scratch, bytes));
  // one eager run: validates the inputs, sets kernel attributes, stages the
  // digit program at the start of the scratch (where the capture expects it)
  evaluate_noalloc_impl<T>(ctx, p->net, tensors, X, p->n_points, ncols, prog, out, out_kind,
                           (unsigned char*)p->scratch, bytes, true, &p->derr);
  cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
  TNFA_CUDA(cudaStreamBeginCapture(ctx->stream, mode));
  ctx->capturing = true;
  try {
    evaluate_noalloc_impl<T>(ctx, p->net, tensors, X, p->n_points, ncols, prog, out, out_kind,
                             (unsigned char*)p->scratch, bytes, false);
  } catch (...) {
    ctx->capturing = false;
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(ctx->stream, &g);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    throw;
  }
  ctx->capturing = false;
  TNFA_CUDA(cudaStreamEndCapture(ctx->stream, &p->graph));
  TNFA_CUDA(cudaGraphInstantiate(&p->exec, p->graph, 0));
}
}  // namespace
}  // namespace tnfa

extern "C" int tnfa_eval_plan_create(tnfa_ctx* ctx, const tnfa_net* net, const double* X,
                                     int64_t n_points, int32_t n_dims, const int32_t* dims,
                                     void* out, int out_kind, int precision,
                                     tnfa_eval_plan** plan) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(net, "eval_plan_create");
  TNFA_CHECK(plan, TNFA_ERR_INVALID_ARGUMENT, "null plan");
  *plan = nullptr;
  TNFA_CHECK(n_points > 0 && n_points < (int64_t(1) << 31), TNFA_ERR_INVALID_ARGUMENT,
             "n_points must be in [1, 2^31)");
  TNFA_CHECK(X && out && (n_dims == 0 || dims), TNFA_ERR_INVALID_ARGUMENT, "null X, out or dims");
  TNFA_CHECK(n_dims >= 0 && n_dims <= 64, TNFA_ERR_INVALID_ARGUMENT, "n_dims out of range");
  for (int v = 0; v < net->topo.V; ++v)
    TNFA_CHECK(net->topo.site_dim[v] <= 256, TNFA_ERR_UNSUPPORTED, "site dimension above 256");
  int ncols = 0;
  std::vector<DigitEntry> prog = make_digit_program(net->topo, n_dims, dims, &ncols);
  tnfa_eval_plan* p = new tnfa_eval_plan;
  p->ctx = ctx;
  ctx->refs += 1;
  p->net = net;
  p->n_points = n_points;
  try {
    if (net->dtype == TNFA_C128) {
      TNFA_CHECK(out_kind == TNFA_OUT_C128 && precision == TNFA_PREC_F64, TNFA_ERR_DTYPE,
                 "complex networks: TNFA_OUT_C128 and TNFA_PREC_F64");
      plan_build<cplx>(p, (const cplx*)net->d, X, ncols, prog, out, out_kind);
    } else {
      TNFA_CHECK(out_kind == TNFA_OUT_F64 || out_kind == TNFA_OUT_F32 ||
                     out_kind == TNFA_OUT_F32_SCALED,
                 TNFA_ERR_DTYPE, "real networks need a real output kind");
      if (precision == TNFA_PREC_F64 && net->dtype == TNFA_F64)
        plan_build<double>(p, (const double*)net->d, X, ncols, prog, out, out_kind);
      else if (precision == TNFA_PREC_F32 && net->dtype == TNFA_F32)
        plan_build<float>(p, (const float*)net->d, X, ncols, prog, out, out_kind);
      else
        fail(TNFA_ERR_UNSUPPORTED,
             "an evaluation plan computes in the network's own type: TNFA_PREC_F64 on FP64 "
             "networks or TNFA_PREC_F32 on FP32 networks");
    }
  } catch (...) {
    plan_free(p);
    throw;
  }
  *plan = p;
  TNFA_API_END
}

extern "C" int tnfa_eval_plan_launch(tnfa_ctx* ctx, tnfa_eval_plan* plan) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  TNFA_CHECK(plan && plan->exec && plan->ctx == ctx, TNFA_ERR_INVALID_ARGUMENT,
             "not a plan of this context");
  TNFA_CUDA(cudaGraphLaunch(plan->exec, ctx->stream));
  TNFA_API_END
}

extern "C" int tnfa_eval_plan_check(tnfa_ctx* ctx, tnfa_eval_plan* plan) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  TNFA_CHECK(plan && plan->derr && plan->ctx == ctx, TNFA_ERR_INVALID_ARGUMENT,
             "not a plan of this context");
  int herr = 0;
  TNFA_CUDA(cudaMemcpyAsync(&herr, plan->derr, 4, cudaMemcpyDeviceToHost, ctx->stream));
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  TNFA_CHECK(herr == 0, TNFA_ERR_DOMAIN,
             "a coordinate is negative or not finite (the digit map needs x >= 0)");
  TNFA_API_END
}

extern "C" int tnfa_eval_plan_destroy(tnfa_eval_plan* plan) {
  if (!plan) return TNFA_OK;
  cudaStreamSynchronize(plan->ctx->stream);
  tnfa::plan_free(plan);
  return TNFA_OK;
}

// ----------------------------------------------- vector-Jacobian product ----
// d/dT of sum_p dout_p f(x_p).  For vertex v with outside message E_v (the
// contraction of everything but v's subtree, as a vector over v's parent
// bond) and inside messages m_c of its children,
//   dT_v[s][a][c1..ck] += sum_{p: s_v(p) = s} dout_p E_v[p][a] prod_j m_cj[p][c_j].
// Inside messages come from the forward contraction (kept for every vertex);
// E of a child is the same contraction with that child's bond as the output
// (the vertex tensor with the child's axis moved first, E_v as one more input);
// the accumulation treats E_v as one more Kronecker factor and reduces over
// the points of each digit group (split over point tiles, atomics per tile).
#include "linalg.cuh"

namespace tnfa {
namespace {

template <class T>
__device__ inline void atomic_add_T(T* a, T v);
template <>
__device__ inline void atomic_add_T<double>(double* a, double v) { atomicAdd(a, v); }
template <>
__device__ inline void atomic_add_T<float>(float* a, float v) { atomicAdd(a, v); }
template <>
__device__ inline void atomic_add_T<cplx>(cplx* a, cplx v) {
  atomicAdd(&a->re, v.re);
  atomicAdd(&a->im, v.im);
}

// dT_v[g][k] += sum over the points p of site value g of scale_p * prod_c m_c[p][k_c]
// (k decoded as the mixed-radix tuple of the child entries, last child
// fastest).  Each CTA walks a contiguous run of tiles of tiles_per_cta point
// tiles, keeps its partial sums in registers and adds them to dT once per site
// value it met, so the atomics on the few thousand dT entries stay far from
// the point count.
template <class T, int TP, int KQ>
__global__ void __launch_bounds__(256) k_grad_acc(const VertexJob<T> j, T* __restrict__ dT,
                                                  int tiles_per_cta) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int sumdim = 0;
  for (int c = 0; c < j.nchild; ++c) sumdim += j.ch[c].dim;
  T* rows = (T*)smem_raw;
  T* scale = rows + (int64_t)sumdim * TP;
  int* pts = (int*)(scale + TP);
  int* eacc = pts + TP;
  // KQ entries k = blockIdx.y * 256 KQ + threadIdx.x + 256 q per thread, each
  // with its child row offsets decoded once
  int kq[KQ], off0[KQ], off1[KQ];
#pragma unroll
  for (int q = 0; q < KQ; ++q) {
    kq[q] = blockIdx.y * blockDim.x * KQ + threadIdx.x + blockDim.x * q;
    int kk = kq[q] < j.K ? kq[q] : 0;
    // the general product below decodes per point; two children (the common
    // case: the outside message and one child) keep both offsets here
    const int d1 = j.nchild > 1 ? j.ch[1].dim : 1;
    off0[q] = (kk / d1);
    off1[q] = j.ch[0].dim * TP + kk % d1;
  }
  const int ntiles = j.tile_start[j.ngroups];
  const int b0 = blockIdx.x * tiles_per_cta;
  const int b1 = min(ntiles, b0 + tiles_per_cta);
  T acc[KQ];
#pragma unroll
  for (int q = 0; q < KQ; ++q) acc[q] = Sc<T>::zero();
  int gcur = -1;
  for (int b = b0; b < b1; ++b) {
    int row0, nrows, g;
    if (!locate_tile(j, TP, b, row0, nrows, g)) continue;  // uniform over the CTA
    if (g != gcur) {
      if (gcur >= 0)
#pragma unroll
        for (int q = 0; q < KQ; ++q)
          if (kq[q] < j.K) atomic_add_T<T>(dT + (int64_t)gcur * j.K + kq[q], acc[q]);
#pragma unroll
      for (int q = 0; q < KQ; ++q) acc[q] = Sc<T>::zero();
      gcur = g;
    }
    __syncthreads();  // the previous tile's rows are no longer read
    for (int r = threadIdx.x; r < TP; r += blockDim.x) {
      pts[r] = r < nrows ? (j.perm ? j.perm[row0 + r] : row0 + r) : 0;
      eacc[r] = 0;
    }
    __syncthreads();
    load_children(j, pts, nrows, TP, rows, eacc);
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) scale[r] = Sc<T>::scale2(Sc<T>::one(), eacc[r]);
    __syncthreads();
    if (j.nchild == 2) {
      const int d0 = j.ch[0].dim, d1 = j.ch[1].dim;
      for (int r = 0; r < nrows; ++r) {
        const T sc = scale[r];
        const T* r0 = rows + r * d0;
        const T* r1 = rows + r * d1;
#pragma unroll
        for (int q = 0; q < KQ; ++q) acc[q] = Sc<T>::fma(sc * r0[off0[q]], r1[off1[q]], acc[q]);
      }
    } else {
#pragma unroll
      for (int q = 0; q < KQ; ++q) {
        if (kq[q] >= j.K) continue;
        for (int r = 0; r < nrows; ++r) {
          T a = scale[r];
          int kk = kq[q], off = sumdim;
          for (int c = j.nchild - 1; c >= 0; --c) {
            const int d = j.ch[c].dim;
            off -= d;
            a = a * rows[off * TP + r * d + kk % d];
            kk /= d;
          }
          acc[q] = acc[q] + a;
        }
      }
    }
  }
  if (gcur >= 0)
#pragma unroll
    for (int q = 0; q < KQ; ++q)
      if (kq[q] < j.K) atomic_add_T<T>(dT + (int64_t)gcur * j.K + kq[q], acc[q]);
}

template <class T>
__global__ void k_vjp_seed(const double* __restrict__ dout, const T* __restrict__ rootv,
                           const int* __restrict__ roote, int nroots, int r, int Pc, T* __restrict__ E,
                           int* __restrict__ Eexp) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < Pc; p += gridDim.x * blockDim.x) {
    T v = Sc<T>::one();
    if constexpr (sizeof(T) == 16)
      v = T{dout[p], 0.0};
    else
      v = (T)dout[p];
    int e = 0;
    for (int q = 0; q < nroots; ++q) {
      if (q == r) continue;
      v = v * rootv[(int64_t)q * Pc + p];
      e += roote[(int64_t)q * Pc + p];
    }
    E[p] = v;
    Eexp[p] = e;
  }
}

// Group the points of a chunk by the site value of vertex v (fills the job's
// group fields; tp = tile rows of the kernel that will consume them).
template <class T>
void group_by_site(tnfa_ctx* ctx, VertexJob<T>& j, const uint8_t* Sv, int Pc, int ng, int tp,
                   int* meta, int* perm) {
  j.ngroups = ng;
  j.grp_off = meta;
  j.grp_cnt = meta + ng;
  j.tile_start = meta + 2 * ng;
  if (ng == 1) {
    k_group_identity<<<1, 1, 0, ctx->stream>>>(meta, Pc, tp);
    TNFA_LAUNCH_CHECK();
    j.perm = nullptr;
    return;
  }
  TNFA_CHECK(ng <= 256, TNFA_ERR_UNSUPPORTED, "site dimension above 256 per vertex");
  TNFA_CUDA(cudaMemsetAsync(meta + ng, 0, ng * sizeof(int), ctx->stream));
  KernelScope ks(ctx, "group", 0.0, (double)Pc * 6.0);
  k_group_count<<<grid_for(Pc, 256, 4 * 152), 256, 0, ctx->stream>>>(Sv, Pc, ng, meta + ng);
  k_group_scan<<<1, 1, 0, ctx->stream>>>(meta, ng, tp);
  const unsigned gs = (unsigned)((Pc + 256 * SCATTER_ITEMS - 1) / (256 * SCATTER_ITEMS));
  k_group_scatter<<<gs, 256, 0, ctx->stream>>>(Sv, Pc, ng, meta + 3 * ng + 1, perm);
  TNFA_LAUNCH_CHECK();
  j.perm = perm;
}

template <class T>
void vjp_impl(tnfa_ctx* ctx, const tnfa_net* net, const T* tensors, const double* X, int64_t P,
              int ncols, const std::vector<DigitEntry>& prog, int xmem, const double* dout,
              int dout_mem, T* dT) {
  const Topo& Tp = net->topo;
  const int V = Tp.V;
  EvalPlan plan = make_plan(Tp);
  const int nroots = (int)plan.roots.size();
  std::vector<int> root_index(V, -1);
  for (int r = 0; r < nroots; ++r) root_index[plan.roots[r]] = r;
  size_t per_point = V + 4 + (xmem == TNFA_MEM_HOST ? ncols * 8 : 0) +
                     (dout_mem == TNFA_MEM_HOST ? 8 : 0) + nroots * (sizeof(T) + 4);
  for (int v = 0; v < V; ++v) per_point += 2 * ((size_t)Tp.link[v] * sizeof(T) + 4);
  int64_t Pc_max = (int64_t)(ctx->eval_budget / per_point);
  Pc_max = std::max<int64_t>(256, std::min<int64_t>(Pc_max, int64_t(1) << 30));
  const int Pcap = (int)std::max<int64_t>(std::min<int64_t>(P, (Pc_max / 256) * 256), 1);
  int maxsd = 1;
  for (int v = 0; v < V; ++v) maxsd = std::max(maxsd, Tp.site_dim[v]);
  DBuf dprog(ctx, prog.size() * sizeof(DigitEntry));
  if (!prog.empty())
    TNFA_CUDA(cudaMemcpyAsync(dprog.p, prog.data(), prog.size() * sizeof(DigitEntry),
                              cudaMemcpyHostToDevice, ctx->stream));
  DBuf dS(ctx, (size_t)V * Pcap), dperm(ctx, (size_t)Pcap * 4);
  DBuf dmeta(ctx, group_meta_ints(maxsd) * 4), derr(ctx, 4);
  TNFA_CUDA(cudaMemsetAsync(derr.p, 0, 4, ctx->stream));
  std::vector<DBuf> in(V), ine(V), E(V), Ee(V);
  for (int v = 0; v < V; ++v) {
    if (!plan.fused_leaf[v]) {
      in[v] = DBuf(ctx, (size_t)Pcap * Tp.link[v] * sizeof(T));
      ine[v] = DBuf(ctx, (size_t)Pcap * 4);
    }
    E[v] = DBuf(ctx, (size_t)Pcap * Tp.link[v] * sizeof(T));
    Ee[v] = DBuf(ctx, (size_t)Pcap * 4);
  }
  DBuf droot(ctx, (size_t)nroots * Pcap * sizeof(T)), droote(ctx, (size_t)nroots * Pcap * 4);
  DBuf dX(ctx, xmem == TNFA_MEM_HOST ? (size_t)Pcap * ncols * 8 : 0);
  DBuf ddout(ctx, dout_mem == TNFA_MEM_HOST ? (size_t)Pcap * 8 : 0);
  int* meta = dmeta.as<int>();
  auto inside_src = [&](int c) {
    ChildSrc<T> s{};
    s.dim = Tp.link[c];
    if (plan.fused_leaf[c]) {
      s.ptr = tensors + Tp.off[c];
      s.exps = nullptr;
      s.S = dS.as<uint8_t>() + (int64_t)c * Pcap;
    } else {
      s.ptr = in[c].as<T>();
      s.exps = ine[c].as<int>();
      s.S = nullptr;
    }
    return s;
  };
  for (int64_t p0 = 0; p0 < P; p0 += Pcap) {
    const int Pc = (int)std::min<int64_t>(Pcap, P - p0);
    const double* Xc = X + p0 * ncols;
    if (xmem == TNFA_MEM_HOST) {
      TNFA_CUDA(cudaMemcpyAsync(dX.p, Xc, (size_t)Pc * ncols * 8, cudaMemcpyHostToDevice, ctx->stream));
      Xc = dX.as<double>();
    }
    const double* dc = dout + p0;
    if (dout_mem == TNFA_MEM_HOST) {
      TNFA_CUDA(cudaMemcpyAsync(ddout.p, dc, (size_t)Pc * 8, cudaMemcpyHostToDevice, ctx->stream));
      dc = ddout.as<double>();
    }
    TNFA_CUDA(cudaMemsetAsync(dS.p, 0, (size_t)V * Pcap, ctx->stream));
    if (!prog.empty()) {
      KernelScope ks(ctx, "digitize", 0.0, (double)Pc * (ncols * 8.0 + V));
      k_digitize<<<grid_for(Pc, 256, 8 * 152 * 8), 256, 0, ctx->stream>>>(
          Xc, ncols, Pc, dprog.as<DigitEntry>(), (int)prog.size(), dS.as<uint8_t>(), (int64_t)Pcap,
          derr.as<int>());
      TNFA_LAUNCH_CHECK();
    }
    // forward: inside messages of every non-leaf vertex
    for (int v : plan.order) {
      VertexJob<T> j{};
      j.nchild = (int)Tp.children[v].size();
      TNFA_CHECK(j.nchild <= EVAL_MAXC, TNFA_ERR_UNSUPPORTED, "vertex degree too high");
      int64_t K = 1;
      int sumdim = 0;
      for (int i = 0; i < j.nchild; ++i) {
        j.ch[i] = inside_src(Tp.children[v][i]);
        K *= j.ch[i].dim;
        sumdim += j.ch[i].dim;
      }
      j.K = (int)K;
      j.chi_a = Tp.link[v];
      j.site_dim = Tp.site_dim[v];
      j.B = tensors + Tp.off[v];
      j.Pc = Pc;
      if (Tp.parent[v] < 0) {
        j.out = (T*)droot.p + (size_t)root_index[v] * Pcap;
        j.out_exp = droote.as<int>() + (size_t)root_index[v] * Pcap;
      } else {
        j.out = in[v].as<T>();
        j.out_exp = ine[v].as<int>();
      }
      group_by_site(ctx, j, dS.as<uint8_t>() + (int64_t)v * Pcap, Pc, j.site_dim,
                    contract_tile_rows(j.chi_a, sumdim, sizeof(T)), meta, dperm.as<int>());
      launch_contract<T>(ctx, j, Pc);
    }
    // seeds: E of a root = dout times the other roots' values
    for (int r = 0; r < nroots; ++r)
      k_vjp_seed<T><<<grid_for(Pc, 256, 4096), 256, 0, ctx->stream>>>(
          dc, (const T*)droot.p, droote.as<int>(), nroots, r, Pcap, E[plan.roots[r]].as<T>(),
          Ee[plan.roots[r]].as<int>());
    TNFA_LAUNCH_CHECK();
    // top-down: outside messages of every child
    for (int v = 0; v < V; ++v) {
      const auto& kids = Tp.children[v];
      std::vector<int> shp{Tp.site_dim[v], Tp.link[v]};
      for (int c : kids) shp.push_back(Tp.link[c]);
      for (size_t jx = 0; jx < kids.size(); ++jx) {
        const int c = kids[jx];
        // T_v with child c's axis moved to position 1: [s][c][parent][others]
        DBuf perm_t(ctx, (size_t)Tp.size(v) * sizeof(T));
        la::PermJob pj{};
        pj.src = tensors + Tp.off[v];
        pj.dst = perm_t.p;
        pj.nd = (int)shp.size();
        TNFA_CHECK(pj.nd <= la::MAXD, TNFA_ERR_UNSUPPORTED, "vertex degree too high");
        std::vector<int> order;
        order.push_back(0);
        order.push_back(2 + (int)jx);
        for (int a = 1; a < pj.nd; ++a)
          if (a != 2 + (int)jx) order.push_back(a);
        pj.n = Tp.size(v);
        for (int a = 0; a < pj.nd; ++a) {
          pj.shape[a] = shp[a];
          pj.perm[a] = order[a];
        }
        la::permute<T>(ctx, {pj});
        VertexJob<T> j{};
        j.nchild = 0;
        ChildSrc<T> e{};
        e.ptr = E[v].as<T>();
        e.exps = Ee[v].as<int>();
        e.S = nullptr;
        e.dim = Tp.link[v];
        j.ch[j.nchild++] = e;
        int64_t K = e.dim;
        int sumdim = e.dim;
        for (size_t q = 0; q < kids.size(); ++q) {
          if (q == jx) continue;
          TNFA_CHECK(j.nchild < EVAL_MAXC, TNFA_ERR_UNSUPPORTED, "vertex degree too high");
          j.ch[j.nchild++] = inside_src(kids[q]);
          K *= Tp.link[kids[q]];
          sumdim += Tp.link[kids[q]];
        }
        j.K = (int)K;
        j.chi_a = Tp.link[c];
        j.site_dim = Tp.site_dim[v];
        j.B = perm_t.as<T>();
        j.Pc = Pc;
        j.out = E[c].as<T>();
        j.out_exp = Ee[c].as<int>();
        group_by_site(ctx, j, dS.as<uint8_t>() + (int64_t)v * Pcap, Pc, j.site_dim,
                      contract_tile_rows(j.chi_a, sumdim, sizeof(T)), meta, dperm.as<int>());
        launch_contract<T>(ctx, j, Pc);
      }
    }
    // accumulation: dT_v[s][(a, c...)] += sum_p E_v[p][a] prod m_c[p][c]
    for (int v = 0; v < V; ++v) {
      VertexJob<T> j{};
      ChildSrc<T> e{};
      e.ptr = E[v].as<T>();
      e.exps = Ee[v].as<int>();
      e.S = nullptr;
      e.dim = Tp.link[v];
      j.ch[j.nchild++] = e;
      int64_t K = e.dim;
      int sumdim = e.dim;
      for (int c : Tp.children[v]) {
        TNFA_CHECK(j.nchild < EVAL_MAXC, TNFA_ERR_UNSUPPORTED, "vertex degree too high");
        j.ch[j.nchild++] = inside_src(c);
        K *= Tp.link[c];
        sumdim += Tp.link[c];
      }
      TNFA_CHECK(K < (int64_t(1) << 31), TNFA_ERR_UNSUPPORTED, "gradient block too large");
      j.K = (int)K;
      j.chi_a = 1;
      j.site_dim = Tp.site_dim[v];
      j.Pc = Pc;
      constexpr int TP = 64;
      group_by_site(ctx, j, dS.as<uint8_t>() + (int64_t)v * Pcap, Pc, j.site_dim, TP, meta,
                    dperm.as<int>());
      const size_t sm = (size_t)sumdim * TP * sizeof(T) + TP * sizeof(T) + 2 * TP * sizeof(int);
      TNFA_CHECK(sm <= 200 * 1024, TNFA_ERR_UNSUPPORTED, "bonds too large for the gradient kernel");
      constexpr int KQ = 4;
      auto kern = k_grad_acc<T, TP, KQ>;
      if (sm > 48 * 1024)
        TNFA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      // one wave of resident CTAs, each over a run of consecutive tiles
      int occ = 0, nsm = 0, dev = 0;
      TNFA_CUDA(cudaGetDevice(&dev));
      TNFA_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
      TNFA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 256, sm));
      const int ntiles = (int)((Pc + TP - 1) / TP + j.ngroups);
      const int ky = (int)((K + 256 * KQ - 1) / (256 * KQ));
      const int want = std::max(1, std::max(occ, 1) * nsm / ky);
      const int per = std::max(1, (ntiles + want - 1) / want);
      dim3 grid((unsigned)((ntiles + per - 1) / per), (unsigned)ky);
      KernelScope ks(ctx, "grad_acc", 2.0 * Pc * (double)K, 0.0);
      kern<<<grid, 256, sm, ctx->stream>>>(j, dT + Tp.off[v], per);
      TNFA_LAUNCH_CHECK();
    }
  }
  int herr = 0;
  TNFA_CUDA(cudaMemcpyAsync(&herr, derr.p, 4, cudaMemcpyDeviceToHost, ctx->stream));
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  TNFA_CHECK(herr == 0, TNFA_ERR_DOMAIN,
             "a coordinate is negative or not finite (the digit map needs x >= 0)");
}

}  // namespace
}  // namespace tnfa

extern "C" int tnfa_evaluate_vjp(tnfa_ctx* ctx, const tnfa_net* net, const double* X,
                                 int64_t n_points, int32_t n_dims, const int32_t* dims,
                                 int x_memory, const double* dout, int dout_memory, void* dtensors,
                                 int dtensors_memory) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(net, "evaluate_vjp");
  TNFA_CHECK(n_points >= 0, TNFA_ERR_INVALID_ARGUMENT, "n_points < 0");
  if (n_points == 0) return TNFA_OK;
  TNFA_CHECK(X && dout && dtensors && (n_dims == 0 || dims), TNFA_ERR_INVALID_ARGUMENT,
             "null X, dout, dtensors or dims");
  for (int m : {x_memory, dout_memory, dtensors_memory})
    TNFA_CHECK(m == TNFA_MEM_HOST || m == TNFA_MEM_DEVICE, TNFA_ERR_INVALID_ARGUMENT, "bad memory kind");
  for (int v = 0; v < net->topo.V; ++v)
    TNFA_CHECK(net->topo.site_dim[v] <= 256, TNFA_ERR_UNSUPPORTED, "site dimension above 256");
  int ncols = 0;
  std::vector<DigitEntry> prog = make_digit_program(net->topo, n_dims, dims, &ncols);
  const size_t es = dtype_size(net->dtype);
  const size_t bytes = (size_t)net->topo.n_elem * es;
  DBuf acc;
  void* dT = dtensors;
  if (dtensors_memory == TNFA_MEM_HOST) {
    acc = DBuf(ctx, bytes);
    TNFA_CUDA(cudaMemcpyAsync(acc.p, dtensors, bytes, cudaMemcpyHostToDevice, ctx->stream));
    dT = acc.p;
  }
  if (net->dtype == TNFA_F64)
    vjp_impl<double>(ctx, net, (const double*)net->d, X, n_points, ncols, prog, x_memory, dout,
                     dout_memory, (double*)dT);
  else if (net->dtype == TNFA_F32)
    vjp_impl<float>(ctx, net, (const float*)net->d, X, n_points, ncols, prog, x_memory, dout,
                    dout_memory, (float*)dT);
  else
    vjp_impl<cplx>(ctx, net, (const cplx*)net->d, X, n_points, ncols, prog, x_memory, dout,
                   dout_memory, (cplx*)dT);
  if (dtensors_memory == TNFA_MEM_HOST) {
    TNFA_CUDA(cudaMemcpyAsync(dtensors, acc.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  TNFA_API_END
}
