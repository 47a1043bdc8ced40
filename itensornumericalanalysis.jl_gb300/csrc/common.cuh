// Shared internals of libtnfa: error plumbing, context / network objects,
// scalar types and small device helpers.  Nothing here is part of the ABI.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <functional>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/tnfa.h"

namespace tnfa {

// ---------------------------------------------------------------- errors --
// Internal code throws tnfa::Error; every extern "C" entry point catches it
// (TNFA_API_BEGIN/END) and turns it into a status plus a context message.
struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

[[noreturn]] inline void fail(int status, const std::string& msg) { throw Error(status, msg); }

inline void check_cuda(cudaError_t e, const char* what, const char* file, int line) {
  if (e != cudaSuccess) {
    char buf[512];
    snprintf(buf, sizeof buf, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    fail(e == cudaErrorMemoryAllocation ? TNFA_ERR_OUT_OF_MEMORY : TNFA_ERR_CUDA, buf);
  }
}
#define TNFA_CUDA(call) ::tnfa::check_cuda((call), #call, __FILE__, __LINE__)
#define TNFA_CHECK(cond, status, msg)  \
  do {                                  \
    if (!(cond)) ::tnfa::fail((status), (msg)); \
  } while (0)
#define TNFA_LAUNCH_CHECK() TNFA_CUDA(cudaGetLastError())

// ---------------------------------------------------------------- scalars --
struct cplx {
  double re, im;
};
__host__ __device__ inline cplx operator+(cplx a, cplx b) { return {a.re + b.re, a.im + b.im}; }
__host__ __device__ inline cplx operator-(cplx a, cplx b) { return {a.re - b.re, a.im - b.im}; }
__host__ __device__ inline cplx operator*(cplx a, cplx b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__host__ __device__ inline cplx& operator+=(cplx& a, cplx b) {
  a.re += b.re;
  a.im += b.im;
  return a;
}

template <class T> struct Sc;
template <> struct Sc<double> {
  __host__ __device__ static double zero() { return 0.0; }
  __host__ __device__ static double one() { return 1.0; }
  __device__ static double absmax(double x) { return fabs(x); }
  __device__ static double scale2(double x, int e) { return scalbn(x, e); }
  __device__ static double fma(double a, double b, double c) { return ::fma(a, b, c); }
  __host__ __device__ static double conj(double x) { return x; }
};
template <> struct Sc<float> {
  __host__ __device__ static float zero() { return 0.0f; }
  __host__ __device__ static float one() { return 1.0f; }
  __device__ static float absmax(float x) { return fabsf(x); }
  __device__ static float scale2(float x, int e) { return scalbnf(x, e); }
  __device__ static float fma(float a, float b, float c) { return fmaf(a, b, c); }
  __host__ __device__ static float conj(float x) { return x; }
};
template <> struct Sc<cplx> {
  __host__ __device__ static cplx zero() { return {0.0, 0.0}; }
  __host__ __device__ static cplx one() { return {1.0, 0.0}; }
  __device__ static double absmax(cplx z) { return fmax(fabs(z.re), fabs(z.im)); }
  __device__ static cplx scale2(cplx z, int e) { return {scalbn(z.re, e), scalbn(z.im, e)}; }
  __device__ static cplx fma(cplx a, cplx b, cplx c) {
    return {::fma(a.re, b.re, ::fma(-a.im, b.im, c.re)), ::fma(a.re, b.im, ::fma(a.im, b.re, c.im))};
  }
  __host__ __device__ static cplx conj(cplx z) { return {z.re, -z.im}; }
};

inline size_t dtype_size(int dtype) {
  switch (dtype) {
    case TNFA_F64: return 8;
    case TNFA_F32: return 4;
    case TNFA_C128: return 16;
  }
  fail(TNFA_ERR_DTYPE, "unknown dtype " + std::to_string(dtype));
}

// ------------------------------------------------------------- objects --
struct Ctx;

// Host-side description of a forest plus its device tensors.
struct Topo {
  int V = 0;
  std::vector<int> parent, link, nlegs, leg_off;  // leg_off[v]: first leg of v
  std::vector<int> leg_dim, leg_var, leg_digit, leg_kind;
  std::vector<std::vector<int>> children;  // ascending
  std::vector<int> site_dim;               // product of the leg dims of v
  std::vector<int64_t> off;                // element offset of v's tensor
  int64_t n_elem = 0;

  int64_t size(int v) const {
    int64_t s = (int64_t)site_dim[v] * link[v];
    for (int c : children[v]) s *= link[c];
    return s;
  }
  void finalize();  // children, site_dim, off, n_elem from the arrays above
  void validate() const;
  std::vector<int> roots() const {
    std::vector<int> r;
    for (int v = 0; v < V; ++v)
      if (parent[v] < 0) r.push_back(v);
    return r;
  }
};

}  // namespace tnfa

namespace tnfa {
// Per-family launch accounting of a context (see tnfa_ctx_kernel_stats).
struct KernelFamily {
  std::string name;
  int64_t launches = 0;
  double flops = 0, bytes = 0;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> events;  // unresolved
  double ms = 0;
};
}  // namespace tnfa

struct tnfa_ctx {
  // One reference for the caller's handle plus one per live network: the
  // context (and its stream) is released only when the last one goes, so a
  // network may be destroyed after tnfa_ctx_destroy without touching freed
  // memory.
  int refs = 1;
  bool closed = false;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int sm_count = 0;
  size_t eval_budget = 0;  // bytes of device scratch an evaluate call may hold
  std::string last_error;
  bool timing = false;
  bool capturing = false;  // a stream capture is open: no events, no syncs
  // autotuning of interchangeable launch variants (tnfa::tune)
  int autotune = -1;            // -1: from TNFA_AUTOTUNE (default on), 0 off, 1 on
  double autotune_min_work = 2e9;  // algorithmic flops below which the rule choice stands
  std::map<std::string, int> tuned;
  std::map<std::string, std::vector<float>> tuned_ms;
  std::vector<tnfa::KernelFamily> families;
  std::vector<cudaEvent_t> event_pool;
  // tensor-core pipelines: try_wait polls before an mbarrier wait gives up,
  // and a test switch that withholds one arrive so that a wait runs out
  uint32_t tc_wait_limit = 1u << 26;
  int tc_drop_arrive = 0;
  // fault injection for tests: device allocations left before one fails
  // (-1: never), and a cap on Jacobi sweeps (0: the built-in caps)
  int64_t alloc_countdown = -1;
  int jacobi_sweep_cap = 0;
  // Blocks freed back to this context, by size class, for reuse by later
  // work on its stream (stream order makes the reuse safe); block -> class
  // size of every block handed out through the cache.
  std::map<size_t, std::vector<void*>> free_blocks;
  std::unordered_map<void*, size_t> block_size;
  size_t cached_bytes = 0;
  // Pinned host blocks that stage large host -> device uploads (tnfa::h2d);
  // a block is free again once the event recorded after its copy completes.
  struct PinnedBlock {
    void* p;
    size_t bytes;
    cudaEvent_t ev;
  };
  std::vector<PinnedBlock> pinned;
  size_t pinned_bytes = 0;
};

struct tnfa_net {
  tnfa_ctx* ctx = nullptr;
  tnfa::Topo topo;
  int dtype = TNFA_F64;
  void* d = nullptr;  // device tensors, canonical layout
  // Lazily built derived copies (invalidated by any in-place change).
  mutable void* d_f32 = nullptr;   // FP32 copy of a real network
  mutable void* d_bhi = nullptr;   // BF16 hi part (tensor-core evaluation)
  mutable void* d_blo = nullptr;   // BF16 lo part
  mutable void* d_f64 = nullptr;   // FP64 copy of an FP32 network (accurate mixed path)
  mutable void* d_oz = nullptr;    // BF16 digit planes of two-child vertices (evaluate_oz.cu)
  mutable int* d_ozexp = nullptr;  // their per-(site value, parent index) exponents
  void invalidate_caches() const;
};

namespace tnfa {

// Device memory from the stream-ordered allocator of the context's stream.
void* dalloc(tnfa_ctx* ctx, size_t bytes);
void dfree(tnfa_ctx* ctx, void* p);

// Host -> device copy of host data (job tables and the like) on the
// context's stream that returns without waiting for the stream: the source
// may be reused as soon as the call returns.
void h2d(tnfa_ctx* ctx, void* dst, const void* src, size_t bytes);

// RAII scratch buffer.
struct DBuf {
  tnfa_ctx* ctx = nullptr;
  void* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(tnfa_ctx* c, size_t bytes) : ctx(c), n(bytes) { p = bytes ? dalloc(c, bytes) : nullptr; }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : ctx(o.ctx), p(o.p), n(o.n) { o.p = nullptr; }
  DBuf& operator=(DBuf&& o) noexcept {
    reset();
    ctx = o.ctx;
    p = o.p;
    n = o.n;
    o.p = nullptr;
    return *this;
  }
  ~DBuf() { reset(); }
  void reset() {
    if (p) dfree(ctx, p);
    p = nullptr;
  }
  template <class T> T* as() const { return (T*)p; }
};

tnfa_net* new_net(tnfa_ctx* ctx, const Topo& topo, int dtype);  // allocates d
void ctx_release(tnfa_ctx* ctx);  // drop one reference (frees at zero)
void require_net(const tnfa_net* net, const char* what);
void require_ctx(const tnfa_ctx* ctx);

// Element-type conversions on the device.
void convert_f64_to_f32(tnfa_ctx* ctx, const double* src, float* dst, int64_t n);

// Measured choice among ncand interchangeable variants of one launch (tile
// shapes, formulations) that compute the same result.  The first call for a
// key whose algorithmic work reaches ctx->autotune_min_work times every
// variant once on the context's stream (CUDA events), keeps the fastest for
// the key and leaves its result in place (re-running it when another variant
// ran last); later calls run the kept variant directly.  Below the work
// threshold, with autotuning off, or inside a stream capture, variant 0 (the
// rule-based default) runs and nothing is recorded.  run(i) enqueues variant
// i.  Returns the variant that produced the result.
int tune(tnfa_ctx* ctx, const std::string& key, int ncand, double work,
         const std::function<void(int)>& run);
// The variant kept for key, or -1.
int tuned_choice(const tnfa_ctx* ctx, const std::string& key);

// Launch accounting: construct before a launch, destroy after it.  Counts
// the launch and its algorithmic work; records CUDA events when timing is on.
// With the environment variable TNFA_TRACE set (to a file path, or to 1 for
// stderr) every launch is also timed and written out as one line: family,
// algorithmic flops, milliseconds and the launcher's note.
struct KernelScope {
  tnfa_ctx* ctx;
  int fam;
  double flops;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  std::string note;
  KernelScope(tnfa_ctx* c, const char* family, double flops, double bytes);
  ~KernelScope();
};
bool trace_on();
void trace_line(const std::string& line);  // one line to the trace, if tracing

inline unsigned grid_for(int64_t n, int block, int cap = 1 << 20) {
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (unsigned)g;
}

}  // namespace tnfa

// Entry-point wrappers: map exceptions to statuses, record the message.
// Every entry point is an NVTX range named after the function, so a
// profiler's timeline (ncu --nvtx, Nsight Systems) shows the C-ABI calls
// around their kernels; without a profiler attached the push / pop cost a
// branch each.
namespace tnfa {
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
}  // namespace tnfa

#define TNFA_API_BEGIN(ctxp)              \
  tnfa::NvtxRange __tnfa_nvtx(__func__); \
  tnfa_ctx* __tnfa_ctx = (ctxp);         \
  try {
#define TNFA_API_END                                                   \
  }                                                                    \
  catch (const tnfa::Error& e) {                                       \
    if (__tnfa_ctx) __tnfa_ctx->last_error = e.what();                 \
    return e.status;                                                   \
  }                                                                    \
  catch (const std::bad_alloc&) {                                      \
    if (__tnfa_ctx) __tnfa_ctx->last_error = "host allocation failed"; \
    return TNFA_ERR_OUT_OF_MEMORY;                                     \
  }                                                                    \
  catch (const std::exception& e) {                                    \
    if (__tnfa_ctx) __tnfa_ctx->last_error = e.what();                 \
    return TNFA_ERR_INVALID_ARGUMENT;                                  \
  }                                                                    \
  if (__tnfa_ctx) __tnfa_ctx->last_error.clear();                      \
  return TNFA_OK;
