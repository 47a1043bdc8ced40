// Context and network objects of libtnfa: creation, validation, transfer,
// copies and scalar scaling.
#include <cstring>

#include "common.cuh"

namespace tnfa {

void Topo::finalize() {
  children.assign(V, {});
  site_dim.assign(V, 1);
  leg_off.assign(V + 1, 0);
  for (int v = 0; v < V; ++v) leg_off[v + 1] = leg_off[v] + nlegs[v];
  for (int v = 0; v < V; ++v)
    if (parent[v] >= 0 && parent[v] < v) children[parent[v]].push_back(v);
  for (int v = 0; v < V; ++v)
    for (int l = leg_off[v]; l < leg_off[v + 1]; ++l) site_dim[v] *= leg_dim[l];
  off.assign(V + 1, 0);
  for (int v = 0; v < V; ++v) off[v + 1] = off[v] + size(v);
  n_elem = off[V];
}

void Topo::validate() const {
  TNFA_CHECK(V >= 1, TNFA_ERR_TOPOLOGY, "network needs at least one vertex");
  for (int v = 0; v < V; ++v) {
    TNFA_CHECK(parent[v] == -1 || (parent[v] >= 0 && parent[v] < v), TNFA_ERR_TOPOLOGY,
               "parent[" + std::to_string(v) + "] = " + std::to_string(parent[v]) +
                   " breaks the order parent[v] < v (or -1 for a root)");
    TNFA_CHECK(link[v] >= 1, TNFA_ERR_TOPOLOGY, "link_dim must be >= 1");
    TNFA_CHECK(parent[v] >= 0 || link[v] == 1, TNFA_ERR_TOPOLOGY,
               "a root (vertex " + std::to_string(v) + ") must have link_dim 1");
    TNFA_CHECK(nlegs[v] >= 0, TNFA_ERR_TOPOLOGY, "n_legs must be >= 0");
  }
  int L = leg_off[V];
  for (int l = 0; l < L; ++l) {
    TNFA_CHECK(leg_dim[l] >= 1, TNFA_ERR_TOPOLOGY, "leg_dim must be >= 1");
    TNFA_CHECK(leg_kind[l] >= 0 && leg_kind[l] <= 2, TNFA_ERR_TOPOLOGY, "bad leg_kind");
  }
  for (int v = 0; v < V; ++v)
    TNFA_CHECK(size(v) > 0 && size(v) < (int64_t(1) << 40), TNFA_ERR_SHAPE, "tensor too large");
}

// Device memory: stream-ordered allocations (cudaMallocAsync) behind a
// per-context cache of freed blocks.  The batched factorisations allocate and
// free thousands of small per-problem buffers per sweep step; handing a freed
// block to the next request of its size class is safe because every launch
// of the context runs on its one stream, so the earlier user of the block has
// finished before the next one starts.  Classes: powers of two from 512 B to
// 1 MiB, then multiples of 2 MiB up to 64 MiB; larger requests are not
// cached.  While a stream capture is open the cache is bypassed (blocks
// freed then go back with cudaFreeAsync, as captured graphs require).
namespace {
constexpr size_t kCacheMaxBlock = size_t(64) << 20;
constexpr size_t kCacheMaxBytes = size_t(2) << 30;

size_t size_class(size_t bytes) {
  if (bytes > (size_t(1) << 20)) return (bytes + (size_t(2) << 20) - 1) & ~((size_t(2) << 20) - 1);
  size_t c = 512;
  while (c < bytes) c <<= 1;
  return c;
}

void drop_cache(tnfa_ctx* ctx) {
  for (auto& kv : ctx->free_blocks)
    for (void* p : kv.second) cudaFreeAsync(p, ctx->stream);
  ctx->free_blocks.clear();
  ctx->cached_bytes = 0;
}
}  // namespace

void* dalloc(tnfa_ctx* ctx, size_t bytes) {
  void* p = nullptr;
  if (bytes == 0) return nullptr;
  if (ctx->alloc_countdown == 0)
    fail(TNFA_ERR_OUT_OF_MEMORY, "device allocation of " + std::to_string(bytes) +
                                     " bytes failed: injected failure (tnfa_ctx_inject_faults)");
  if (ctx->alloc_countdown > 0) --ctx->alloc_countdown;
  const bool cache = !ctx->capturing && bytes <= kCacheMaxBlock;
  const size_t cls = cache ? size_class(bytes) : bytes;
  if (cache) {
    auto it = ctx->free_blocks.find(cls);
    if (it != ctx->free_blocks.end() && !it->second.empty()) {
      p = it->second.back();
      it->second.pop_back();
      ctx->cached_bytes -= cls;
      ctx->block_size[p] = cls;
      return p;
    }
  }
  cudaError_t e = cudaMallocAsync(&p, cls, ctx->stream);
  if (e != cudaSuccess && !ctx->capturing && ctx->cached_bytes > 0) {
    cudaGetLastError();
    drop_cache(ctx);  // give the cached blocks back to the pool and retry once
    e = cudaMallocAsync(&p, cls, ctx->stream);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    fail(TNFA_ERR_OUT_OF_MEMORY, "device allocation of " + std::to_string(bytes) +
                                     " bytes failed: " + cudaGetErrorString(e));
  }
  if (cache) ctx->block_size[p] = cls;
  return p;
}

void dfree(tnfa_ctx* ctx, void* p) {
  if (!p) return;
  auto it = ctx->block_size.find(p);
  if (it == ctx->block_size.end()) {
    cudaFreeAsync(p, ctx->stream);
    return;
  }
  const size_t cls = it->second;
  ctx->block_size.erase(it);
  if (ctx->capturing || ctx->cached_bytes + cls > kCacheMaxBytes) {
    cudaFreeAsync(p, ctx->stream);
    return;
  }
  ctx->free_blocks[cls].push_back(p);
  ctx->cached_bytes += cls;
}

// A copy from pageable host memory returns at once only up to 64 KB (the
// driver stages it); a larger one returns after the stream has drained, so
// every large job table would stall the host behind the GPU.  Those go
// through pinned blocks instead: copied in, sent with an asynchronous copy,
// and reused only after the event recorded behind that copy has completed.
// Inside a stream capture (where a captured copy would read the block again
// at every replay) and beyond the pinned cap the plain copy is used.
constexpr size_t kPageableAsyncMax = size_t(64) << 10;
constexpr size_t kPinnedMaxBytes = size_t(256) << 20;

void h2d(tnfa_ctx* ctx, void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (bytes > kPageableAsyncMax && !ctx->capturing)
    TNFA_CUDA(cudaStreamIsCapturing(ctx->stream, &cap));
  if (bytes <= kPageableAsyncMax || ctx->capturing || cap != cudaStreamCaptureStatusNone) {
    TNFA_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return;
  }
  tnfa_ctx::PinnedBlock* blk = nullptr;
  for (auto& b : ctx->pinned) {
    if (b.bytes < bytes) continue;
    const cudaError_t q = cudaEventQuery(b.ev);
    if (q == cudaSuccess) {
      blk = &b;
      break;
    }
    if (q != cudaErrorNotReady) TNFA_CUDA(q);
    // "not ready" is a status, not a failure: keep it out of the error state
    if (cudaPeekAtLastError() == cudaErrorNotReady) cudaGetLastError();
  }
  if (!blk) {
    size_t cls = size_t(128) << 10;
    while (cls < bytes) cls <<= 1;
    if (ctx->pinned_bytes + cls > kPinnedMaxBytes) {
      TNFA_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
      return;
    }
    void* p = nullptr;
    if (cudaMallocHost(&p, cls) != cudaSuccess) {
      cudaGetLastError();
      TNFA_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
      return;
    }
    cudaEvent_t ev = nullptr;
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      cudaFreeHost(p);
      TNFA_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
      return;
    }
    ctx->pinned.push_back({p, cls, ev});
    ctx->pinned_bytes += cls;
    blk = &ctx->pinned.back();
  }
  std::memcpy(blk->p, src, bytes);
  TNFA_CUDA(cudaMemcpyAsync(dst, blk->p, bytes, cudaMemcpyHostToDevice, ctx->stream));
  TNFA_CUDA(cudaEventRecord(blk->ev, ctx->stream));
}

void require_ctx(const tnfa_ctx* ctx) {
  TNFA_CHECK(ctx != nullptr, TNFA_ERR_INVALID_ARGUMENT, "null context");
}

void require_net(const tnfa_net* net, const char* what) {
  TNFA_CHECK(net != nullptr && net->d != nullptr, TNFA_ERR_INVALID_ARGUMENT,
             std::string("null network: ") + what);
}

tnfa_net* new_net(tnfa_ctx* ctx, const Topo& topo, int dtype) {
  tnfa_net* n = new tnfa_net;
  n->ctx = ctx;
  n->topo = topo;
  n->dtype = dtype;
  try {
    n->d = dalloc(ctx, (size_t)topo.n_elem * dtype_size(dtype));
  } catch (...) {
    delete n;
    throw;
  }
  ctx->refs += 1;
  return n;
}

static void ctx_free(tnfa_ctx* ctx) {
  drop_cache(ctx);
  cudaStreamSynchronize(ctx->stream);
  for (auto& f : ctx->families)
    for (auto& ev : f.events) {
      cudaEventDestroy(ev.first);
      cudaEventDestroy(ev.second);
    }
  for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
  for (auto& b : ctx->pinned) {
    cudaEventDestroy(b.ev);
    cudaFreeHost(b.p);
  }
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

void ctx_release(tnfa_ctx* ctx) {
  if (--ctx->refs == 0) ctx_free(ctx);
}

__global__ void k_f64_to_f32(const double* __restrict__ s, float* __restrict__ d, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    d[i] = (float)s[i];
}

void convert_f64_to_f32(tnfa_ctx* ctx, const double* src, float* dst, int64_t n) {
  k_f64_to_f32<<<grid_for(n, 256, 4096), 256, 0, ctx->stream>>>(src, dst, n);
  TNFA_LAUNCH_CHECK();
}

template <class T>
__global__ void k_scale(T* x, int64_t n, T s) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = x[i] * s;
}

Topo topo_from_abi(const tnfa_topology* t) {
  TNFA_CHECK(t && t->parent && t->link_dim && t->n_legs, TNFA_ERR_INVALID_ARGUMENT,
             "topology has null arrays");
  Topo T;
  T.V = t->n_vertices;
  TNFA_CHECK(T.V >= 1, TNFA_ERR_TOPOLOGY, "n_vertices must be >= 1");
  T.parent.assign(t->parent, t->parent + T.V);
  T.link.assign(t->link_dim, t->link_dim + T.V);
  T.nlegs.assign(t->n_legs, t->n_legs + T.V);
  int64_t L = 0;
  for (int v = 0; v < T.V; ++v) {
    TNFA_CHECK(T.nlegs[v] >= 0 && T.nlegs[v] <= 16, TNFA_ERR_TOPOLOGY, "n_legs out of range");
    L += T.nlegs[v];
  }
  if (L > 0)
    TNFA_CHECK(t->leg_dim && t->leg_var && t->leg_digit && t->leg_kind, TNFA_ERR_INVALID_ARGUMENT,
               "topology has legs but null leg arrays");
  T.leg_dim.assign(t->leg_dim, t->leg_dim + L);
  T.leg_var.assign(t->leg_var, t->leg_var + L);
  T.leg_digit.assign(t->leg_digit, t->leg_digit + L);
  T.leg_kind.assign(t->leg_kind, t->leg_kind + L);
  T.leg_off.assign(T.V + 1, 0);
  for (int v = 0; v < T.V; ++v) T.leg_off[v + 1] = T.leg_off[v] + T.nlegs[v];
  for (int v = 0; v < T.V; ++v)
    TNFA_CHECK(T.parent[v] == -1 || (T.parent[v] >= 0 && T.parent[v] < v), TNFA_ERR_TOPOLOGY,
               "parent[" + std::to_string(v) + "] = " + std::to_string(T.parent[v]) +
                   " breaks the order parent[v] < v (or -1 for a root)");
  for (int v = 0; v < T.V; ++v) TNFA_CHECK(T.link[v] >= 1, TNFA_ERR_TOPOLOGY, "link_dim < 1");
  for (int64_t l = 0; l < L; ++l) TNFA_CHECK(T.leg_dim[l] >= 1, TNFA_ERR_TOPOLOGY, "leg_dim < 1");
  T.finalize();
  T.validate();
  return T;
}

static cudaEvent_t take_event(tnfa_ctx* ctx) {
  if (!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return e;
}

namespace {
FILE* trace_file() {
  static FILE* f = [] {
    const char* t = getenv("TNFA_TRACE");
    if (!t || !*t || !strcmp(t, "0")) return (FILE*)nullptr;
    if (!strcmp(t, "1")) return stderr;
    FILE* g = fopen(t, "a");
    return g ? g : stderr;
  }();
  return f;
}
}  // namespace

bool trace_on() { return trace_file() != nullptr; }

void trace_line(const std::string& line) {
  if (FILE* f = trace_file()) {
    fprintf(f, "tnfa-trace %s\n", line.c_str());
    fflush(f);
  }
}

static bool autotune_on(tnfa_ctx* ctx) {
  if (ctx->autotune < 0) {
    const char* e = getenv("TNFA_AUTOTUNE");
    ctx->autotune = (e && *e == '0') ? 0 : 1;
  }
  return ctx->autotune == 1;
}

int tuned_choice(const tnfa_ctx* ctx, const std::string& key) {
  auto it = ctx->tuned.find(key);
  return it == ctx->tuned.end() ? -1 : it->second;
}

int tune(tnfa_ctx* ctx, const std::string& key, int ncand, double work,
         const std::function<void(int)>& run) {
  if (ncand <= 1) {
    run(0);
    return 0;
  }
  const int kept = tuned_choice(ctx, key);
  if (kept >= 0) {
    run(kept);
    return kept;
  }
  if (ctx->capturing || !autotune_on(ctx) || work < ctx->autotune_min_work) {
    run(0);
    return 0;
  }
  cudaEvent_t e0 = take_event(ctx), e1 = take_event(ctx);
  TNFA_CHECK(e0 && e1, TNFA_ERR_CUDA, "autotune: no CUDA events");
  std::vector<float> ms(ncand, -1.0f);
  for (int i = 0; i < ncand; ++i) {
    TNFA_CUDA(cudaEventRecord(e0, ctx->stream));
    run(i);
    TNFA_CUDA(cudaEventRecord(e1, ctx->stream));
    TNFA_CUDA(cudaEventSynchronize(e1));
    TNFA_CUDA(cudaEventElapsedTime(&ms[i], e0, e1));
  }
  ctx->event_pool.push_back(e0);
  ctx->event_pool.push_back(e1);
  int best = 0;
  for (int i = 1; i < ncand; ++i)
    if (ms[i] < ms[best]) best = i;
  if (best != ncand - 1) run(best);
  ctx->tuned[key] = best;
  ctx->tuned_ms[key] = ms;
  if (trace_on()) {
    fprintf(trace_file(), "tnfa-tune %s ->%d", key.c_str(), best);
    for (float m : ms) fprintf(trace_file(), " %.4f", m);
    fprintf(trace_file(), "\n");
    fflush(trace_file());
  }
  return best;
}

KernelScope::KernelScope(tnfa_ctx* c, const char* family, double fl, double bytes)
    : ctx(c), flops(fl) {
  fam = -1;
  for (size_t i = 0; i < ctx->families.size(); ++i)
    if (ctx->families[i].name == family) fam = (int)i;
  if (fam < 0) {
    ctx->families.push_back(KernelFamily{});
    ctx->families.back().name = family;
    fam = (int)ctx->families.size() - 1;
  }
  KernelFamily& f = ctx->families[fam];
  f.launches += 1;
  f.flops += fl;
  f.bytes += bytes;
  if (!ctx->capturing && (ctx->timing || trace_on())) {
    e0 = take_event(ctx);
    e1 = take_event(ctx);
    if (e0 && e1) cudaEventRecord(e0, ctx->stream);
  }
}

KernelScope::~KernelScope() {
  if (e0 && e1 && trace_on()) {
    cudaEventRecord(e1, ctx->stream);
    float ms = -1.0f;
    if (cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    fprintf(trace_file(), "tnfa-trace %s flops=%.4g ms=%.4f %s\n", ctx->families[fam].name.c_str(),
            flops, ms, note.c_str());
    fflush(trace_file());
    if (ctx->timing) {
      ctx->families[fam].events.push_back({e0, e1});
    } else {
      ctx->event_pool.push_back(e0);
      ctx->event_pool.push_back(e1);
    }
  } else if (e0 && e1) {
    cudaEventRecord(e1, ctx->stream);
    ctx->families[fam].events.push_back({e0, e1});
  } else {
    if (e0) ctx->event_pool.push_back(e0);
    if (e1) ctx->event_pool.push_back(e1);
  }
}

}  // namespace tnfa

void tnfa_net::invalidate_caches() const {
  if (d_f32) tnfa::dfree(ctx, d_f32);
  if (d_bhi) tnfa::dfree(ctx, d_bhi);
  if (d_blo) tnfa::dfree(ctx, d_blo);
  if (d_f64) tnfa::dfree(ctx, d_f64);
  if (d_oz) tnfa::dfree(ctx, d_oz);
  if (d_ozexp) tnfa::dfree(ctx, d_ozexp);
  d_f32 = d_bhi = d_blo = d_f64 = d_oz = nullptr;
  d_ozexp = nullptr;
}

using namespace tnfa;

extern "C" {

const char* tnfa_version(void) { return "tnfa 0.1.0 sm_103a"; }

int tnfa_ctx_create(int device, void* stream, tnfa_ctx** out) {
  if (!out) return TNFA_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  tnfa_ctx* c = new (std::nothrow) tnfa_ctx;
  if (!c) return TNFA_ERR_OUT_OF_MEMORY;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    delete c;
    return TNFA_ERR_CUDA;
  }
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess) {
    delete c;
    return TNFA_ERR_CUDA;
  }
  if (stream) {
    c->stream = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete c;
      return TNFA_ERR_CUDA;
    }
    c->own_stream = true;
  }
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  size_t cap = (size_t)6 << 30;
  c->eval_budget = fr / 3 < cap ? fr / 3 : cap;
  if (c->eval_budget < ((size_t)64 << 20)) c->eval_budget = (size_t)64 << 20;
  *out = c;
  return TNFA_OK;
}

int tnfa_ctx_set_timing(tnfa_ctx* ctx, int enable) {
  if (!ctx) return TNFA_ERR_INVALID_ARGUMENT;
  ctx->timing = enable != 0;
  return TNFA_OK;
}

int tnfa_ctx_set_autotune(tnfa_ctx* ctx, int enable, double min_work, int forget) {
  if (!ctx) return TNFA_ERR_INVALID_ARGUMENT;
  if (enable >= 0) ctx->autotune = enable != 0 ? 1 : 0;
  if (min_work >= 0) ctx->autotune_min_work = min_work;
  if (forget) {
    ctx->tuned.clear();
    ctx->tuned_ms.clear();
  }
  return TNFA_OK;
}

int tnfa_ctx_tuning_report(tnfa_ctx* ctx, char* buf, int64_t size, int64_t* needed) {
  if (!ctx) return TNFA_ERR_INVALID_ARGUMENT;
  std::string r;
  for (const auto& kv : ctx->tuned) {
    r += kv.first + " " + std::to_string(kv.second);
    for (float m : ctx->tuned_ms[kv.first]) {
      char b[32];
      snprintf(b, sizeof b, " %.4f", m);
      r += b;
    }
    r += "\n";
  }
  if (needed) *needed = (int64_t)r.size() + 1;
  if (buf && size > 0) {
    const size_t n = std::min<size_t>((size_t)size - 1, r.size());
    memcpy(buf, r.data(), n);
    buf[n] = 0;
  }
  return TNFA_OK;
}

int tnfa_ctx_kernel_stats(tnfa_ctx* ctx, int32_t max, char* names, int64_t* launches, double* ms,
                          double* flops, double* bytes, int32_t* n_families, int reset) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  for (auto& f : ctx->families) {
    for (auto& ev : f.events) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, ev.first, ev.second) == cudaSuccess) f.ms += t;
      cudaGetLastError();
      ctx->event_pool.push_back(ev.first);
      ctx->event_pool.push_back(ev.second);
    }
    f.events.clear();
  }
  int n = (int)ctx->families.size();
  if (n_families) *n_families = n;
  for (int i = 0; i < n && i < max; ++i) {
    const auto& f = ctx->families[i];
    if (names) {
      memset(names + 32 * i, 0, 32);
      strncpy(names + 32 * i, f.name.c_str(), 31);
    }
    if (launches) launches[i] = f.launches;
    if (ms) ms[i] = f.ms;
    if (flops) flops[i] = f.flops;
    if (bytes) bytes[i] = f.bytes;
  }
  if (reset) ctx->families.clear();
  TNFA_API_END
}

int tnfa_ctx_inject_faults(tnfa_ctx* ctx, int64_t fail_alloc_after, int32_t jacobi_sweep_cap) {
  if (!ctx) return TNFA_ERR_INVALID_ARGUMENT;
  ctx->alloc_countdown = fail_alloc_after < 0 ? -1 : fail_alloc_after;
  ctx->jacobi_sweep_cap = jacobi_sweep_cap > 0 ? jacobi_sweep_cap : 0;
  return TNFA_OK;
}

int tnfa_ctx_set_wait_budget(tnfa_ctx* ctx, uint32_t polls, int drop_arrive) {
  if (!ctx) return TNFA_ERR_INVALID_ARGUMENT;
  if (polls) ctx->tc_wait_limit = polls;
  ctx->tc_drop_arrive = drop_arrive ? 1 : 0;
  return TNFA_OK;
}

int tnfa_ctx_destroy(tnfa_ctx* ctx) {
  if (!ctx || ctx->closed) return TNFA_ERR_INVALID_ARGUMENT;
  ctx->closed = true;
  cudaStreamSynchronize(ctx->stream);
  ctx_release(ctx);
  return TNFA_OK;
}

int tnfa_ctx_synchronize(tnfa_ctx* ctx) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  TNFA_API_END
}

const char* tnfa_last_error_string(const tnfa_ctx* ctx) {
  return ctx ? ctx->last_error.c_str() : "null context";
}

int tnfa_net_create(tnfa_ctx* ctx, const tnfa_topology* topo, int dtype, const void* tensors,
                    int memory, tnfa_net** out) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  TNFA_CHECK(out && tensors, TNFA_ERR_INVALID_ARGUMENT, "null tensors or out");
  *out = nullptr;
  TNFA_CHECK(dtype == TNFA_F64 || dtype == TNFA_F32 || dtype == TNFA_C128, TNFA_ERR_DTYPE,
             "dtype must be TNFA_F64, TNFA_F32 or TNFA_C128");
  TNFA_CHECK(memory == TNFA_MEM_HOST || memory == TNFA_MEM_DEVICE, TNFA_ERR_INVALID_ARGUMENT,
             "memory must be TNFA_MEM_HOST or TNFA_MEM_DEVICE");
  Topo T = topo_from_abi(topo);
  tnfa_net* n = new_net(ctx, T, dtype);
  size_t bytes = (size_t)T.n_elem * dtype_size(dtype);
  cudaError_t e = cudaMemcpyAsync(n->d, tensors, bytes,
                                  memory == TNFA_MEM_HOST ? cudaMemcpyHostToDevice
                                                          : cudaMemcpyDeviceToDevice,
                                  ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    dfree(ctx, n->d);
    delete n;
    check_cuda(e, "upload of network tensors", __FILE__, __LINE__);
  }
  *out = n;
  TNFA_API_END
}

int tnfa_net_destroy(tnfa_net* net) {
  if (!net) return TNFA_ERR_INVALID_ARGUMENT;
  tnfa_ctx* ctx = net->ctx;
  net->invalidate_caches();
  if (net->d) dfree(ctx, net->d);
  delete net;
  if (ctx) ctx_release(ctx);
  return TNFA_OK;
}

int tnfa_net_info(const tnfa_net* net, int32_t* n_vertices, int32_t* dtype, int64_t* n_elements,
                  int32_t* link_dim_out) {
  if (!net) return TNFA_ERR_INVALID_ARGUMENT;
  if (n_vertices) *n_vertices = net->topo.V;
  if (dtype) *dtype = net->dtype;
  if (n_elements) *n_elements = net->topo.n_elem;
  if (link_dim_out)
    for (int v = 0; v < net->topo.V; ++v) link_dim_out[v] = net->topo.link[v];
  return TNFA_OK;
}

int tnfa_net_topology(const tnfa_net* net, int32_t* parent, int32_t* link_dim, int32_t* n_legs,
                      int32_t* leg_dim, int32_t* leg_var, int32_t* leg_digit, int32_t* leg_kind,
                      int32_t* n_legs_total) {
  if (!net) return TNFA_ERR_INVALID_ARGUMENT;
  const Topo& T = net->topo;
  int L = T.leg_off[T.V];
  for (int v = 0; v < T.V; ++v) {
    if (parent) parent[v] = T.parent[v];
    if (link_dim) link_dim[v] = T.link[v];
    if (n_legs) n_legs[v] = T.nlegs[v];
  }
  for (int l = 0; l < L; ++l) {
    if (leg_dim) leg_dim[l] = T.leg_dim[l];
    if (leg_var) leg_var[l] = T.leg_var[l];
    if (leg_digit) leg_digit[l] = T.leg_digit[l];
    if (leg_kind) leg_kind[l] = T.leg_kind[l];
  }
  if (n_legs_total) *n_legs_total = L;
  return TNFA_OK;
}

int tnfa_net_download(tnfa_ctx* ctx, const tnfa_net* net, void* tensors, int memory) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(net, "download");
  TNFA_CHECK(tensors, TNFA_ERR_INVALID_ARGUMENT, "null destination");
  size_t bytes = (size_t)net->topo.n_elem * dtype_size(net->dtype);
  TNFA_CUDA(cudaMemcpyAsync(tensors, net->d, bytes,
                            memory == TNFA_MEM_HOST ? cudaMemcpyDeviceToHost
                                                    : cudaMemcpyDeviceToDevice,
                            ctx->stream));
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
  TNFA_API_END
}

int tnfa_net_copy(tnfa_ctx* ctx, const tnfa_net* net, tnfa_net** out) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(net, "copy");
  TNFA_CHECK(out, TNFA_ERR_INVALID_ARGUMENT, "null out");
  tnfa_net* n = new_net(ctx, net->topo, net->dtype);
  TNFA_CUDA(cudaMemcpyAsync(n->d, net->d, (size_t)net->topo.n_elem * dtype_size(net->dtype),
                            cudaMemcpyDeviceToDevice, ctx->stream));
  *out = n;
  TNFA_API_END
}

int tnfa_net_scale(tnfa_ctx* ctx, tnfa_net* net, int32_t vertex, double re, double im) {
  TNFA_API_BEGIN(ctx);
  require_ctx(ctx);
  require_net(net, "scale");
  const Topo& T = net->topo;
  TNFA_CHECK(vertex >= 0 && vertex < T.V, TNFA_ERR_INVALID_ARGUMENT, "vertex out of range");
  int64_t n = T.size(vertex);
  unsigned g = grid_for(n, 256, 1024);
  if (net->dtype == TNFA_F64) {
    TNFA_CHECK(im == 0.0, TNFA_ERR_DTYPE, "complex factor on a real network");
    k_scale<double><<<g, 256, 0, ctx->stream>>>((double*)net->d + T.off[vertex], n, re);
  } else if (net->dtype == TNFA_F32) {
    TNFA_CHECK(im == 0.0, TNFA_ERR_DTYPE, "complex factor on a real network");
    k_scale<float><<<g, 256, 0, ctx->stream>>>((float*)net->d + T.off[vertex], n, (float)re);
  } else {
    k_scale<cplx><<<g, 256, 0, ctx->stream>>>((cplx*)net->d + T.off[vertex], n, cplx{re, im});
  }
  TNFA_LAUNCH_CHECK();
  net->invalidate_caches();
  TNFA_API_END
}

}  // extern "C"
