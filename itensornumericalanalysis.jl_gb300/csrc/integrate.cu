// Integration of a tree tensor network function over [0,1)^n.
//
// Reference: integrate (src/integration.jl:6-17) multiplies every vertex by
// ITensor(c, site_inds...) with c = 1/base (1 with take_sum) and contracts the
// network with belief propagation.  Here (tnfa_integrate): one persistent,
// HBM-streaming launch (k_integrate) reads each tensor once and contracts it
// at the same time with the site weights and the children's messages,
// vertices taken leaves first; messages are kept in FP64 (or complex FP64)
// with a power-of-two exponent per vertex.
// site_reduced_net (the site-reduced network as a network) serves the
// operator and partial integrals.
#include <cmath>

#include "evaluate.cuh"
#include "tc_ptx.cuh"

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
// One persistent launch contracts the whole network.  A task is a run of up
// to kb consecutive rows (s, a, k) of one vertex with the same (s, a), kb
// chosen per level so that every level has about two tasks per resident warp;
// tasks are numbered leaves first, level by level (a vertex's height is one
// more than its highest child's), and warps take them in that order from one
// atomic counter (the next task is taken while the current one runs).  So
// when a warp holds a task of height h every task of lower height has been
// taken by a running warp, and waiting for a child never blocks on work that
// has not started.  A task first issues the loads of its first rows, then
// waits (bounded) for its vertex's children to be ready, contracts its rows
// with the last child's message (each row weighted by the other children's
// entries) and adds the sum to its vertex's FP64 (complex FP64) message with
// one atomic.  The warp that completes a vertex's last task finishes the
// vertex: it scales the message by a power of two into [1/2, 1) (stored in
// the tensors' own type, so FP32 networks keep the FP32 pipe), records the
// exponent and sets the vertex's ready flag.  A leaf is one task.
//
// Row loads are 16-byte vectors (4 FP32, 2 FP64 or 1 complex value per
// lane) when the vertex's rows allow it; NCH vectors cover a row of up to
// 32 * NCH * VE entries and 8 / NCH rows are in flight per warp.
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
__device__ inline float ldcg_acc(const float* p) { return __ldcg(p); }
__device__ inline double ldcg_acc(const double* p) { return __ldcg(p); }
__device__ inline cplx ldcg_acc(const cplx* p) {
  const double2 v = __ldcg((const double2*)p);
  return {v.x, v.y};
}

template <class T> struct Vec;
template <> struct Vec<float> {
  static constexpr int VE = 4;
  __device__ static void load(const float* p, float* e) {
    const float4 v = __ldcs((const float4*)p);
    e[0] = v.x;
    e[1] = v.y;
    e[2] = v.z;
    e[3] = v.w;
  }
};
template <> struct Vec<double> {
  static constexpr int VE = 2;
  __device__ static void load(const double* p, double* e) {
    const double2 v = __ldcs((const double2*)p);
    e[0] = v.x;
    e[1] = v.y;
  }
};
template <> struct Vec<cplx> {
  static constexpr int VE = 1;
  __device__ static void load(const cplx* p, cplx* e) {
    const double2 v = __ldcs((const double2*)p);
    e[0] = cplx{v.x, v.y};
  }
};

__device__ inline int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}


struct IntVertex {
  int64_t off;     // tensor offset (elements)
  int64_t task0;   // its first task
  int64_t kouter;  // rows per (s, a): product of the children's dims but the last
  int64_t nkb;     // tasks per (s, a)
  int64_t ntask;   // tasks of the vertex
  int64_t kb;      // rows per task
  int sd, chi_a, nchild, last;  // last: entries of the last child (1 without children)
  int ch[EVAL_MAXC], dim[EVAL_MAXC];
  int v, root;  // root: position among the forest's roots, -1 otherwise
  int vec;      // rows are read as 16-byte vectors
  double w;     // site weight: prod of 1 / leg dim (1 with take_sum)
};

template <class T>
struct IntState {
  using A = typename IntAcc<T>::type;
  A* msgs;    // V x chimax accumulators (zeroed)
  int* done;  // tasks completed per vertex (zeroed)
  int* ready; // vertex finished (zeroed)
  unsigned long long* next;  // task counter (zeroed)
  A* res;     // per root: its message entry 0
  int* rexp;  // per root: the exponent that goes with it
  int* err;   // nonzero: a wait gave up (zeroed)
  int* exps;  // per vertex: exponent of its normalised message
  T* cm;      // V x chimax normalised messages
  int chimax, nv;
  int64_t ntask;
  uint32_t wait_limit;
};

template <class T>
__device__ void integrate_finish(const IntVertex& iv, const IntState<T>& st) {
  using A = typename IntAcc<T>::type;
  const int lane = threadIdx.x & 31;
  __syncwarp();
  __threadfence();
  int X = 0;
  for (int c = 0; c < iv.nchild; ++c) X += __ldcg(st.exps + iv.ch[c]);
  const A* raw = st.msgs + (int64_t)iv.v * st.chimax;
  double mx = 0.0;
  for (int i = lane; i < iv.chi_a; i += 32) mx = fmax(mx, Sc<A>::absmax(ldcg_acc(raw + i)));
  for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  int ex = 0;
  if (mx > 0) frexp(mx, &ex);
  T* dst = st.cm + (int64_t)iv.v * st.chimax;
  for (int i = lane; i < iv.chi_a; i += 32) dst[i] = to_dot(Sc<A>::scale2(ldcg_acc(raw + i), -ex), T{});
  __syncwarp();
  if (lane == 0) {
    st.exps[iv.v] = ex + X;
    if (iv.root >= 0) {
      st.res[iv.root] = ldcg_acc(raw);
      st.rexp[iv.root] = X;
    }
    __threadfence();
    atomicExch(st.ready + iv.v, 1);
  }
  __syncwarp();
}

// The bulk-copy pipeline of one CTA (one per SM): a producer thread takes
// tasks from the global counter and, for each, copies the task's rows (one
// contiguous run of bytes) into the next of INT_STAGES shared-memory stages
// with cp.async.bulk, completing on the stage's full barrier; each stage has
// INT_CPS consumer warps (one takes the even rows, one the odd): they wait
// for the fill, wait for the task's children, read their rows from shared
// memory, release the stage on its empty barrier and then add their sums to
// the vertex's message.  The producer fills whichever stage is released
// first, so a consumer that waits for its children holds up no other stage.  About INT_STAGES x 32 KB are in
// flight per SM, which keeps HBM busy without the register cost of loads in
// flight.  Rows that are not 16-byte aligned, and leaves, are read from
// global memory by the consumer (the stage then carries only the task).
constexpr int INT_STAGES = 6;
constexpr int INT_STAGE_BYTES = 32 * 1024;
constexpr int INT_CPS = 2;  // consumer warps per stage (even / odd rows)
constexpr int INT_THREADS = 32 * (1 + INT_STAGES * INT_CPS);
constexpr int INT_SMEM = INT_STAGES * INT_STAGE_BYTES + 128;
constexpr int INT_GRAB = 4;  // tasks claimed per atomic by a producer

struct IntSlot {
  long long t;  // task; -1: no more tasks
  int vi, a;
  long long k0, k1;
};

// Vector load of VE entries from shared memory.
__device__ inline void lds_vec(const float* p, float* e) {
  const float4 v = *(const float4*)p;
  e[0] = v.x;
  e[1] = v.y;
  e[2] = v.z;
  e[3] = v.w;
}
__device__ inline void lds_vec(const double* p, double* e) {
  const double2 v = *(const double2*)p;
  e[0] = v.x;
  e[1] = v.y;
}
__device__ inline void lds_vec(const cplx* p, cplx* e) {
  const double2 v = *(const double2*)p;
  e[0] = cplx{v.x, v.y};
}

template <class T>
__device__ inline T shfl_t(T v, int src) {
  if constexpr (sizeof(T) == 16) {
    cplx z = *(cplx*)&v;
    z.re = __shfl_sync(0xffffffffu, z.re, src);
    z.im = __shfl_sync(0xffffffffu, z.im, src);
    return *(T*)&z;
  } else {
    return __shfl_sync(0xffffffffu, v, src);
  }
}

template <class T, int NCH>
__global__ void __launch_bounds__(INT_THREADS, 1) k_integrate(const T* __restrict__ tensors,
                                                             const IntVertex* __restrict__ vt, IntState<T> st) {
  using namespace ptx;
  using A = typename IntAcc<T>::type;
  using D = T;
  constexpr int VE = Vec<T>::VE;
  extern __shared__ unsigned char int_smem[];
  __shared__ uint64_t full[INT_STAGES], empty[INT_STAGES];
  __shared__ IntSlot slot[INT_STAGES];
  unsigned char* stages = (unsigned char*)(((uintptr_t)int_smem + 127) & ~(uintptr_t)127);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int i = 0; i < INT_STAGES; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], INT_CPS);
    }
    fence_mbar_init();
  }
  __syncthreads();
  if (warp == 0) {
    if (lane != 0) return;
    // ---------------- producer ----------------
    // Each task goes to whichever stage its consumer has released (a
    // consumer that waits for its children does not hold up the others).
    int vi = 0;
    unsigned pending = 0;  // stages with a copy the consumer has not released
    unsigned sent = 0;     // stages that got their end-of-work fill
    int fills[INT_STAGES];
    for (int i = 0; i < INT_STAGES; ++i) fills[i] = 0;
    bool exhausted = false;
    // tasks are taken INT_GRAB at a time; the next batch is claimed while the
    // current one is placed, so the atomic's round trip is off the copy path
    long long tq = (long long)atomicAdd(st.next, (unsigned long long)INT_GRAB);
    long long tq_end = tq + INT_GRAB;
    long long tq_next = (long long)atomicAdd(st.next, (unsigned long long)INT_GRAB);
    uint32_t idle = 0;
    int rot = 0;
    bool failed = false;
    while (sent != (1u << INT_STAGES) - 1) {
      int sidx = -1;
      for (int q = 0; q < INT_STAGES; ++q) {
        const int c = (rot + q) % INT_STAGES;
        if (sent & (1u << c)) continue;
        if (fills[c] == 0 || mbar_test(&empty[c], (fills[c] - 1) & 1)) {
          sidx = c;
          break;
        }
      }
      if (sidx < 0) {
        if (++idle > st.wait_limit) {
          atomicOr(st.err, 1);
          failed = true;
          break;
        }
        __nanosleep(32);
        continue;
      }
      idle = 0;
      rot = sidx + 1;
      pending &= ~(1u << sidx);
      const int n = fills[sidx];
      long long t = (long long)st.ntask;
      if (!exhausted) {
        if (tq == tq_end) {
          tq = tq_next;
          tq_end = tq + INT_GRAB;
          if (tq < st.ntask) tq_next = (long long)atomicAdd(st.next, (unsigned long long)INT_GRAB);
        }
        t = tq++;
      }
      if (t >= st.ntask) {
        exhausted = true;
        slot[sidx].t = -1;
        fills[sidx] = n + 1;
        sent |= 1u << sidx;
        mbar_arrive(&full[sidx]);
        continue;
      }
      while (vi + 1 < st.nv && vt[vi + 1].task0 <= t) ++vi;
      const IntVertex& iv = vt[vi];
      IntSlot sl;
      sl.t = t;
      sl.vi = vi;
      sl.a = 0;
      sl.k0 = sl.k1 = 0;
      long long sa = 0;
      if (iv.nchild) {
        const long long tl = t - iv.task0;
        sa = tl / iv.nkb;
        sl.a = (int)(sa % iv.chi_a);
        sl.k0 = (tl - sa * iv.nkb) * iv.kb;
        sl.k1 = min((long long)iv.kouter, sl.k0 + iv.kb);
      }
      slot[sidx] = sl;
      fills[sidx] = n + 1;
      if (iv.nchild && iv.vec) {
        const T* src = tensors + iv.off + (sa * iv.kouter + sl.k0) * iv.last;
        const uint32_t bytes = (uint32_t)((sl.k1 - sl.k0) * iv.last * (long long)sizeof(T));
        mbar_arrive_expect_tx(&full[sidx], bytes);
        bulk_load(stages + (size_t)sidx * INT_STAGE_BYTES, src, bytes, &full[sidx]);
        pending |= 1u << sidx;
      } else {
        mbar_arrive(&full[sidx]);
      }
    }
    (void)failed;
    // after a timeout: let the copies still in flight land before the CTA exits
    for (int i = 0; i < INT_STAGES; ++i)
      if (pending & (1u << i)) mbar_wait(&full[i], (fills[i] - 1) & 1, st.wait_limit);
    return;
  }
  // ---------------- consumers ----------------
  const int sidx = (warp - 1) / INT_CPS, part = (warp - 1) % INT_CPS;
  const T* sbuf = (const T*)(stages + (size_t)sidx * INT_STAGE_BYTES);
  int ready_vi = -1;
  // The completion count of a task is read after the next fill has arrived
  // (the atomic's round trip overlaps the copy); the warp that completed a
  // vertex finishes it then.
  int pend_vi = -1, pend_old = 0;
  auto settle = [&]() {
    if (pend_vi < 0) return;
    int fin = 0;
    if (lane == 0) fin = pend_old == (int)(vt[pend_vi].ntask * INT_CPS - 1);
    fin = __shfl_sync(0xffffffffu, fin, 0);
    if (fin) integrate_finish<T>(vt[pend_vi], st);
    pend_vi = -1;
  };
  for (int n = 0;; ++n) {
    if (!mbar_wait(&full[sidx], n & 1, st.wait_limit)) {
      if (lane == 0) atomicOr(st.err, 1);
      settle();
      break;
    }
    settle();
    const IntSlot sl = slot[sidx];
    if (sl.t < 0) break;
    const IntVertex& iv = vt[sl.vi];
    if (iv.nchild == 0) {
      // a leaf: msg[a] = w sum_s T[s, a], the vertex's only task
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[sidx]);
      if (part != 0) continue;
      const T* base = tensors + iv.off;
      A* out = st.msgs + (int64_t)iv.v * st.chimax;
      for (int a = lane; a < iv.chi_a; a += 32) {
        D acc = Sc<D>::zero();
        for (int s = 0; s < iv.sd; ++s) acc += base[(int64_t)s * iv.chi_a + a];
        out[a] = mulw(to_acc(acc, A{}), iv.w);
      }
      integrate_finish<T>(iv, st);
      continue;
    }
    const int last = iv.last;
    if (ready_vi != sl.vi) {
      // lane c watches child c (bounded)
      int ok = 1;
      if (lane < iv.nchild) {
        uint32_t it = 0;
        while (ld_acquire(st.ready + iv.ch[lane]) == 0) {
          if (++it > st.wait_limit) {
            atomicOr(st.err, 1);
            ok = 0;
            break;
          }
          __nanosleep(64);
        }
      }
      ok = __all_sync(0xffffffffu, ok);
      if (ok) ready_vi = sl.vi;
    }
    const D* cl = st.cm + (int64_t)iv.ch[iv.nchild - 1] * st.chimax;  // last child's message
    const D* c0 = st.cm + (int64_t)iv.ch[0] * st.chimax;
    D partial = Sc<D>::zero();
    if (ready_vi == sl.vi) {
      if (iv.vec) {
        D ml[NCH][VE];
#pragma unroll
        for (int c = 0; c < NCH; ++c)
#pragma unroll
          for (int e = 0; e < VE; ++e) {
            const int j = (lane + 32 * c) * VE + e;
            ml[c][e] = j < last ? ldcg_acc(cl + j) : Sc<D>::zero();
          }
        const int nr = (int)(sl.k1 - sl.k0);
        // first-child weights of the rows (two children), 32 rows per register
        D w2[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const long long r = sl.k0 + lane + 32 * i;
          w2[i] = iv.nchild == 2 && r < sl.k1 ? ldcg_acc(c0 + r) : Sc<D>::one();
        }
#pragma unroll 4
        for (int r = part; r < nr; r += INT_CPS) {
          D dot = Sc<D>::zero();
          const T* row = sbuf + (size_t)r * last;
#pragma unroll
          for (int c = 0; c < NCH; ++c) {
            const int j = (lane + 32 * c) * VE;
            if (j < last) {
              D e[VE];
              lds_vec(row + j, e);
#pragma unroll
              for (int q = 0; q < VE; ++q) dot = Sc<D>::fma(e[q], ml[c][q], dot);
            }
          }
          D wgt;
          if (iv.nchild <= 1) {
            wgt = Sc<D>::one();
          } else if (iv.nchild == 2) {
            const int i = r >> 5;
            const D wr = i == 0 ? w2[0] : i == 1 ? w2[1] : i == 2 ? w2[2] : w2[3];
            wgt = shfl_t(wr, r & 31);
          } else {
            wgt = Sc<D>::one();
            int kk = (int)(sl.k0 + r);
            for (int c = iv.nchild - 2; c >= 0; --c) {
              const int d = iv.dim[c];
              wgt = wgt * ldcg_acc(st.cm + (int64_t)iv.ch[c] * st.chimax + kk % d);
              kk /= d;
            }
          }
          partial = Sc<D>::fma(wgt, dot, partial);
        }
      } else {
        // rows that are not 16-byte aligned or too long for a stage
        const long long sa = (sl.t - iv.task0) / iv.nkb;
        const T* base = tensors + iv.off + sa * iv.kouter * last;
        for (long long r = sl.k0 + part; r < sl.k1; r += INT_CPS) {
          const T* row = base + r * last;
          D dot = Sc<D>::zero();
          for (int j = lane; j < last; j += 32) dot = Sc<D>::fma(row[j], ldcg_acc(cl + j), dot);
          D wgt = Sc<D>::one();
          int kk = (int)r;
          for (int c = iv.nchild - 2; c >= 0; --c) {
            const int d = iv.dim[c];
            wgt = wgt * ldcg_acc(st.cm + (int64_t)iv.ch[c] * st.chimax + kk % d);
            kk /= d;
          }
          partial = Sc<D>::fma(wgt, dot, partial);
        }
      }
    }
    // the stage is free as soon as its rows are read
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[sidx]);
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
    if (lane == 0) {
      atomicAddAcc(&st.msgs[(int64_t)iv.v * st.chimax + sl.a], mulw(to_acc(partial, A{}), iv.w));
      // release: the message add is visible before the count; the finisher
      // acquires (integrate_finish begins with a fence)
      asm volatile("atom.add.release.gpu.global.s32 %0, [%1], 1;" : "=r"(pend_old) : "l"(st.done + iv.v) : "memory");
    }
    pend_vi = sl.vi;
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
  constexpr int VE = Vec<T>::VE;
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
  const std::vector<int> roots = Tp.roots();
  std::vector<int> root_of(V, -1);
  for (size_t i = 0; i < roots.size(); ++i) root_of[roots[i]] = (int)i;
  int maxlast = 1;
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
    iv.kouter = kout;
    iv.v = v;
    iv.root = root_of[v];
    iv.w = 1.0;
    if (!take_sum)
      for (int l = Tp.leg_off[v]; l < Tp.leg_off[v + 1]; ++l) iv.w /= Tp.leg_dim[l];
    if (iv.nchild) maxlast = std::max(maxlast, iv.last);
    levels[height[v]].push_back(iv);
  }
  // vectors per lane covering the longest row (longer rows, and rows that
  // are not 16-byte aligned, take the global-memory path)
  int nch = 1;
  while (nch < 8 && 32 * VE * nch < maxlast) nch *= 2;
  // rows per task: about two tasks per consumer warp in every level, between
  // 1 and 128 rows, and no more than one stage holds
  const int64_t warps = (int64_t)ctx->sm_count * INT_STAGES;
  for (auto& lv : levels) {
    int64_t rows = 0;
    for (const auto& iv : lv)
      if (iv.nchild) rows += (int64_t)iv.sd * iv.chi_a * iv.kouter;
    int64_t kb = 1;
    while (kb < 128 && kb * 2 <= rows / (2 * warps)) kb *= 2;
    for (auto& iv : lv) {
      iv.vec = iv.nchild > 0 && iv.off % VE == 0 && iv.last % VE == 0 && iv.last <= 32 * VE * nch &&
               (int64_t)iv.last * (int64_t)sizeof(T) <= INT_STAGE_BYTES;
      int64_t k = std::min<int64_t>(kb, iv.kouter);
      if (iv.vec)
        while (k > 1 && k * iv.last * (int64_t)sizeof(T) > INT_STAGE_BYTES) k /= 2;
      iv.kb = std::max<int64_t>(k, 1);
      iv.nkb = (iv.kouter + iv.kb - 1) / iv.kb;
      iv.ntask = iv.nchild ? (int64_t)iv.sd * iv.chi_a * iv.nkb : 1;
    }
  }
  std::vector<IntVertex> allv;
  int64_t ntask = 0;
  for (auto& lv : levels)
    for (auto& iv : lv) {
      iv.task0 = ntask;
      ntask += iv.ntask;
      allv.push_back(iv);
    }
  const int nr = (int)roots.size();
  // scratch: zeroed [msgs | done | ready | next | res | rexp | err], then [exps | cm]
  auto up = [](size_t x) { return (x + 15) & ~(size_t)15; };
  const size_t o_done = up((size_t)V * chimax * sizeof(A));
  const size_t o_ready = o_done + up((size_t)V * sizeof(int));
  const size_t o_next = o_ready + up((size_t)V * sizeof(int));
  const size_t o_res = o_next + 16;
  const size_t o_rexp = o_res + (size_t)nr * sizeof(A);
  const size_t o_err = o_rexp + (size_t)nr * sizeof(int);
  const size_t zeroed = up(o_err + sizeof(int));
  const size_t o_exps = zeroed;
  const size_t o_cm = o_exps + up((size_t)V * sizeof(int));
  const size_t total = o_cm + (size_t)V * chimax * sizeof(T);
  DBuf scratch(ctx, total);
  DBuf dv(ctx, allv.size() * sizeof(IntVertex));
  unsigned char* sb = (unsigned char*)scratch.p;
  TNFA_CUDA(cudaMemcpyAsync(dv.p, allv.data(), allv.size() * sizeof(IntVertex), cudaMemcpyHostToDevice,
                            ctx->stream));
  TNFA_CUDA(cudaMemsetAsync(sb, 0, zeroed, ctx->stream));
  IntState<T> st;
  st.msgs = (A*)sb;
  st.done = (int*)(sb + o_done);
  st.ready = (int*)(sb + o_ready);
  st.next = (unsigned long long*)(sb + o_next);
  st.res = (A*)(sb + o_res);
  st.rexp = (int*)(sb + o_rexp);
  st.err = (int*)(sb + o_err);
  st.exps = (int*)(sb + o_exps);
  st.cm = (T*)(sb + o_cm);
  st.chimax = chimax;
  st.nv = (int)allv.size();
  st.ntask = ntask;
  st.wait_limit = ctx->tc_wait_limit;
  // one CTA per SM (the stages take most of its shared memory)
  const unsigned grid = (unsigned)std::max<int64_t>(
      1, std::min<int64_t>((ntask + INT_STAGES - 1) / INT_STAGES, ctx->sm_count));
  {
    KernelScope ks(ctx, "integrate", 2.0 * (double)Tp.n_elem, (double)dtype_size(net->dtype) * Tp.n_elem);
    const T* d = (const T*)net->d;
    const IntVertex* pv = dv.as<IntVertex>();
    auto launch = [&](auto kern) {
      TNFA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, INT_SMEM));
      kern<<<grid, INT_THREADS, INT_SMEM, ctx->stream>>>(d, pv, st);
    };
    switch (nch) {
      case 1: launch(k_integrate<T, 1>); break;
      case 2: launch(k_integrate<T, 2>); break;
      case 4: launch(k_integrate<T, 4>); break;
      default: launch(k_integrate<T, 8>); break;
    }
    TNFA_LAUNCH_CHECK();
  }
  // one read-back: the roots' values and exponents and the error word
  std::vector<unsigned char> hb(zeroed - o_res);
  TNFA_CUDA(cudaMemcpyAsync(hb.data(), sb + o_res, hb.size(), cudaMemcpyDeviceToHost, ctx->stream));
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  int herr;
  std::memcpy(&herr, hb.data() + (o_err - o_res), sizeof(int));
  TNFA_CHECK(herr == 0, TNFA_ERR_TIMEOUT, "integrate: a wait for a child vertex ran out of its budget");
  // product over the roots of the forest, exponents applied at the end
  double re = 1.0, im = 0.0;
  int e = 0;
  for (int i = 0; i < nr; ++i) {
    A val;
    int ex;
    std::memcpy(&val, hb.data() + i * sizeof(A), sizeof(A));
    std::memcpy(&ex, hb.data() + (o_rexp - o_res) + i * sizeof(int), sizeof(int));
    double vr, vi;
    if constexpr (sizeof(A) == 16) {
      const cplx z = *(const cplx*)&val;
      vr = z.re;
      vi = z.im;
    } else {
      vr = *(const double*)&val;
      vi = 0.0;
    }
    const double nr_ = re * vr - im * vi, ni = re * vi + im * vr;
    re = nr_;
    im = ni;
    e += ex;
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
