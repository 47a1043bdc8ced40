// Tensor-core (tcgen05) vertex contraction for batched evaluation, sm_103a.
//
// One CTA computes a tile of 128 points (rows) of one vertex:
//   out[p, a] = sum_{b, c} m1[p, b] m2[p, c] T_s[a][b * chi2 + c]
// i.e. D[128 x N] = A[128 x K] * B[N x K]^T with K = chi1 * chi2, A the row-wise
// Kronecker product of the two child messages (never stored in global memory)
// and B the slice T_s of the vertex tensor (canonical layout, K-major).
//
// Precision: split BF16.  A = A_hi + A_lo, B = B_hi + B_lo (each BF16), and
// D = A_hi B_hi + A_hi B_lo + A_lo B_hi accumulated in FP32 in tensor memory;
// the dropped A_lo B_lo term is ~2^-16 relative.
//
// Roles (320 threads):
//   warps 0-7  producers: thread (row m, half h) keeps half of its m2 row in
//              registers and writes 32 of the 64 columns of every A chunk (hi and
//              lo) into 128B-swizzled shared memory; afterwards they run the
//              epilogue (TMEM -> registers, power-of-two row rescaling, store).
//   warp 8     TMA: streams the B_hi / B_lo chunk [N x 64] of every K step.
//   warp 9     MMA: one lane issues tcgen05.mma (M=128, N, K=16) x 12 per chunk.
// Stages are guarded by mbarriers; every wait is bounded and a timeout sets an
// error bit and unwinds (TMEM is always released).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "evaluate.cuh"
#include "tc_ptx.cuh"

namespace tnfa {

namespace {

constexpr int TC_M = 128;         // rows per tile (points)
constexpr int TC_KC = 64;         // K elements per chunk (128 bytes of BF16)
constexpr int TC_PRODUCERS = 256; // warps 0-7
constexpr int TC_THREADS = 320;
using namespace ptx;
constexpr int TC_ERR_TIMEOUT = ptx::ERR_TIMEOUT;

struct TcParams {
  const float* m1_ptr;   // child 1 rows (message or leaf tensor); null: chi1 = 1
  const int* m1_exp;
  const uint8_t* m1_S;
  const float* m2_ptr;   // child 2 rows
  const int* m2_exp;
  const uint8_t* m2_S;
  int chi1, chi2, N, K;
  float* out;
  int* out_exp;
  const int* perm;
  const int* grp_off;
  const int* grp_cnt;
  const int* tile_start;
  int ngroups;
  int* err;
  uint32_t wait_limit;  // try_wait polls before a wait gives up
};

// BILIN = false: Kronecker mode above (output N = chi_a columns).
// BILIN = true : root of two children (chi_a = 1): A = m2 rows (K = chi2),
//                N = chi1, and the epilogue contracts D[p, :] with m1[p, :].
template <int N, int CHI2, int STAGES, bool BILIN>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_contract_tc(const __grid_constant__ CUtensorMap map_hi,
                  const __grid_constant__ CUtensorMap map_lo, const TcParams P) {
  constexpr int A_BYTES = TC_M * TC_KC * 2;  // 16 KB
  constexpr int B_BYTES = N * TC_KC * 2;
  constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
  constexpr int HALF = CHI2 / 2;  // m2 values per producer thread
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[STAGES], empty_bar[STAGES], acc_bar;
  __shared__ uint32_t tmem_base_sh;
  __shared__ float rowmax[2][TC_M];
  __shared__ int sh_abort;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  unsigned char* smem =
      (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);

  // ---- tile lookup (same grouping as the SIMT kernels) ----
  const int b = blockIdx.x;
  const int ng = P.ngroups;
  if (b >= P.tile_start[ng]) return;
  int g = 0;
  while (g + 1 < ng && P.tile_start[g + 1] <= b) ++g;
  const int row0 = P.grp_off[g] + (b - P.tile_start[g]) * TC_M;
  const int nrows = min(TC_M, P.grp_off[g] + P.grp_cnt[g] - row0);
  if (nrows <= 0) return;

  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full_bar[s], TC_PRODUCERS + 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&acc_bar, 1);
    sh_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 8) {  // TMEM allocation: N fp32 columns (power of two >= 32)
    constexpr uint32_t ncols = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base_sh)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base_sh;
  const int nk = P.K / TC_KC;

  if (warp < 8) {
    // ------------------------------------------------------ producers ----
    const int m = (warp & 3) * 32 + lane;
    const int h = warp >> 2;
    const bool valid = m < nrows;
    const int p = valid ? (P.perm ? P.perm[row0 + m] : row0 + m) : 0;
    float m2r[HALF];
    const float* m2row = P.m2_S ? P.m2_ptr + (int64_t)P.m2_S[p] * CHI2
                                : P.m2_ptr + (int64_t)p * CHI2;
#pragma unroll
    for (int j = 0; j < HALF; ++j) {
      // columns [32h, 32h+32) of every 64-wide block of c
      int c = (j / 32) * 64 + 32 * h + (j % 32);
      m2r[j] = valid ? m2row[c] : 0.0f;
    }
    const float* m1row = nullptr;
    if (P.m1_ptr)
      m1row = P.m1_S ? P.m1_ptr + (int64_t)P.m1_S[p] * P.chi1 : P.m1_ptr + (int64_t)p * P.chi1;
    const int nb = BILIN ? 1 : P.chi1;
    const int e_in = valid ? ((P.m1_exp ? P.m1_exp[p] : 0) + (P.m2_exp ? P.m2_exp[p] : 0)) : 0;
    constexpr int CPB = CHI2 / TC_KC;  // chunks per value of b
    bool ok = true;
    // m1[p, b] is consumed once per b; it is loaded four at a time one group
    // ahead so the global-load latency hides behind the previous group.
    const bool use_m1 = !BILIN && m1row && valid;
    const bool vec4 = use_m1 && (P.chi1 % 4 == 0);
    float4 grp = make_float4(1.f, 1.f, 1.f, 1.f), nxt = grp;
    if (vec4) nxt = *reinterpret_cast<const float4*>(m1row);
    for (int bb = 0; bb < nb && ok; ++bb) {
      float a1;
      if (vec4) {
        if ((bb & 3) == 0) {
          grp = nxt;
          if (bb + 4 < nb) nxt = *reinterpret_cast<const float4*>(m1row + bb + 4);
        }
        const int q4 = bb & 3;
        a1 = q4 == 0 ? grp.x : q4 == 1 ? grp.y : q4 == 2 ? grp.z : grp.w;
      } else {
        a1 = use_m1 ? m1row[bb] : (valid ? 1.0f : 0.0f);
      }
#pragma unroll
      for (int cblk = 0; cblk < CPB; ++cblk) {
        const int kc = bb * CPB + cblk;
        const int s = kc % STAGES, use = kc / STAGES;
        if (use > 0 && !mbar_wait(&empty_bar[s], (use - 1) & 1, P.wait_limit)) {
          ok = false;
          break;
        }
        unsigned char* Ahi = smem + s * STAGE_BYTES;
        unsigned char* Alo = Ahi + A_BYTES;
#pragma unroll
        for (int q = 0; q < 4; ++q) {  // 4 x 16-byte chunks of 8 values
          uint32_t hw[4], lw[4];
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            float x0 = a1 * m2r[cblk * 32 + q * 8 + 2 * t];
            float x1 = a1 * m2r[cblk * 32 + q * 8 + 2 * t + 1];
            __nv_bfloat162 hh = __floats2bfloat162_rn(x0, x1);
            float2 hf = __bfloat1622float2(hh);
            hw[t] = *reinterpret_cast<uint32_t*>(&hh);
            lw[t] = pack_bf16(x0 - hf.x, x1 - hf.y);
          }
          const int chunk = (4 * h + q) ^ (m & 7);
          const int off = m * 128 + chunk * 16;
          *reinterpret_cast<uint4*>(Ahi + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
          *reinterpret_cast<uint4*>(Alo + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        }
        fence_proxy_async();
        mbar_arrive(&full_bar[s]);
      }
    }
    if (!ok) {
      atomicOr(P.err, TC_ERR_TIMEOUT);
      sh_abort = 1;
    }
    // ------------------------------------------------------- epilogue ----
    const bool acc_ok = mbar_wait(&acc_bar, 0, P.wait_limit);
    if (!acc_ok) {
      atomicOr(P.err, TC_ERR_TIMEOUT);
      sh_abort = 1;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    float v[N / 2];
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
#pragma unroll
    for (int cc = 0; cc < N / 2; cc += 32)
      tmem_ld32(tmem + lane_base + (uint32_t)(h * (N / 2) + cc), v + cc);
    if constexpr (BILIN) {
      // out[p] = sum_b D[p, b] m1[p, b]
      float part = 0.f;
      if (valid) {
        const float* mrow = m1row + h * (N / 2);
#pragma unroll
        for (int i = 0; i < N / 2; ++i) part = fmaf(v[i], mrow[i], part);
      }
      rowmax[h][m] = part;
      asm volatile("bar.sync 1, 256;" ::: "memory");
      if (h == 0 && valid && acc_ok) {
        const float tot = rowmax[0][m] + rowmax[1][m];
        int ex = 0;
        if (tot != 0.f) frexpf(tot, &ex);
        P.out[p] = scalbnf(tot, -ex);
        P.out_exp[p] = e_in + ex;
      }
    } else {
      float mx = 0.f;
#pragma unroll
      for (int i = 0; i < N / 2; ++i) mx = fmaxf(mx, fabsf(v[i]));
      rowmax[h][m] = mx;
      asm volatile("bar.sync 1, 256;" ::: "memory");
      mx = fmaxf(rowmax[0][m], rowmax[1][m]);
      int ex = 0;
      if (mx > 0.f) frexpf(mx, &ex);
      if (valid && acc_ok) {
        float* dst = P.out + (int64_t)p * N + h * (N / 2);
#pragma unroll
        for (int i = 0; i < N / 2; i += 4)
          *reinterpret_cast<float4*>(dst + i) =
              make_float4(scalbnf(v[i], -ex), scalbnf(v[i + 1], -ex), scalbnf(v[i + 2], -ex),
                          scalbnf(v[i + 3], -ex));
        if (h == 0) P.out_exp[p] = e_in + ex;
      }
    }
  } else if (warp == 8) {
    // ------------------------------------------------------------ TMA ----
    if (lane == 0) {
      bool ok = true;
      for (int kc = 0; kc < nk; ++kc) {
        const int s = kc % STAGES, use = kc / STAGES;
        if (use > 0 && !mbar_wait(&empty_bar[s], (use - 1) & 1, P.wait_limit)) {
          ok = false;
          break;
        }
        unsigned char* Bhi = smem + s * STAGE_BYTES + 2 * A_BYTES;
        unsigned char* Blo = Bhi + B_BYTES;
        mbar_arrive_expect_tx(&full_bar[s], 2 * B_BYTES);
        tma_load_2d(Bhi, &map_hi, &full_bar[s], kc * TC_KC, g * N);
        tma_load_2d(Blo, &map_lo, &full_bar[s], kc * TC_KC, g * N);
      }
      if (!ok) atomicOr(P.err, TC_ERR_TIMEOUT);
    }
  } else {
    // ------------------------------------------------------------ MMA ----
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16(TC_M, N);
      bool ok = true;
      for (int kc = 0; kc < nk; ++kc) {
        const int s = kc % STAGES, use = kc / STAGES;
        if (!mbar_wait(&full_bar[s], use & 1, P.wait_limit)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        unsigned char* Ahi = smem + s * STAGE_BYTES;
        unsigned char* Alo = Ahi + A_BYTES;
        unsigned char* Bhi = Alo + A_BYTES;
        unsigned char* Blo = Bhi + B_BYTES;
        const uint64_t dah = sw128_desc(Ahi), dal = sw128_desc(Alo);
        const uint64_t dbh = sw128_desc(Bhi), dbl = sw128_desc(Blo);
#pragma unroll
        for (int k = 0; k < TC_KC / 16; ++k) {
          const uint64_t adv = (uint64_t)(k * 32) >> 4;  // 16 BF16 along K
          mma_bf16(tmem, dah + adv, dbh + adv, idesc, (kc | k) != 0);
          mma_bf16(tmem, dah + adv, dbl + adv, idesc, 1);
          mma_bf16(tmem, dal + adv, dbh + adv, idesc, 1);
        }
        mma_commit(&empty_bar[s]);
      }
      if (!ok) atomicOr(P.err, TC_ERR_TIMEOUT);
      mma_commit(&acc_bar);  // arrives once every issued MMA has completed
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 8) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    constexpr uint32_t ncols = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
  }
}

// ---------------------------------------------------------------------------
// Second formulation for a vertex with two children (chi_a in {64, 128},
// chi2 in {64, 128}): contract the second child first,
//   Y[p, (a, b)] = sum_c m2[p, c] T_s[a][b][c]           (tensor cores)
//   out[p, a]    = sum_b m1[p, b] Y[p, (a, b)]            (epilogue, CUDA cores)
// The A operand is then the m2 rows of the tile -- written to shared memory
// once (hi and lo BF16, K = chi2) and reused by every MMA -- and B streams
// T_s as N-tiles of 256 rows (a, b) x 64 columns c through a 3-D TMA box
// {64 c, 256 / chi_a b, chi_a a}.  Per N-tile the MMA warp issues
// 3 x 4 x (chi2 / 64) MMAs of M = 128, N = 256 into one of two TMEM buffers
// (2 x 256 columns); the eight epilogue warps read the other buffer and fold
// it into per-thread accumulators out[p, a] with m1[p, b].  Compared to the
// Kronecker formulation this removes the per-chunk A writes (producers ran
// 32 KB per 6.3 MFLOP through shared memory) and halves the A reads per flop
// (N = 256), the shared-memory traffic that bounded the tensor pipe at ~60 %.
//
// Roles (320 threads): warps 0-7 build A then run the epilogue (thread: row
// m = 32 (w % 4) + lane, half h = w / 4 of the 256 columns); warp 8 TMA;
// warp 9 MMA.  Every wait is bounded; a timeout sets an error bit, stops the
// role's loop and the CTA still releases TMEM.
constexpr int T2_N = 256;

template <int CHIA, int CHI2>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_contract_tc2(const __grid_constant__ CUtensorMap map_hi,
                   const __grid_constant__ CUtensorMap map_lo, const TcParams P) {
  constexpr int NBT = T2_N / CHIA;            // values of b per N-tile
  constexpr int KCH = CHI2 / TC_KC;           // K chunks per N-tile
  constexpr int A_CHUNK = TC_M * TC_KC * 2;   // 16 KB: 128 rows x 64 BF16
  constexpr int A_BYTES = 2 * KCH * A_CHUNK;  // hi and lo, all chunks
  constexpr int B_BYTES = T2_N * TC_KC * 2;   // 32 KB per chunk and part
  constexpr int STAGES = 2;
  constexpr int STAGE_BYTES = 2 * B_BYTES;
  constexpr int ACC = CHIA / 2;               // accumulators per thread
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[STAGES], empty_bar[STAGES], tfull[2], tempty[2],
      a_ready;
  __shared__ uint32_t tmem_base_sh;
  __shared__ float rowmax[2][TC_M];
  __shared__ int sh_abort;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* Asm = smem;
  unsigned char* Bsm = smem + A_BYTES;

  const int blk = blockIdx.x;
  const int ng = P.ngroups;
  if (blk >= P.tile_start[ng]) return;
  int g = 0;
  while (g + 1 < ng && P.tile_start[g + 1] <= blk) ++g;
  const int row0 = P.grp_off[g] + (blk - P.tile_start[g]) * TC_M;
  const int nrows = min(TC_M, P.grp_off[g] + P.grp_cnt[g] - row0);
  if (nrows <= 0) return;
  const int ntiles = P.chi1 / NBT;

  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], TC_PRODUCERS);
    }
    mbar_init(&a_ready, TC_PRODUCERS);
    sh_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 8) {  // TMEM: two accumulators of 256 FP32 columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base_sh)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base_sh;

  if (warp < 8) {
    // ------------------------------------------- A = m2 rows, then epilogue ----
    const int m = (warp & 3) * 32 + lane;
    const int h = warp >> 2;
    const bool valid = m < nrows;
    const int p = valid ? (P.perm ? P.perm[row0 + m] : row0 + m) : 0;
    const float* m2row =
        P.m2_S ? P.m2_ptr + (int64_t)P.m2_S[p] * CHI2 : P.m2_ptr + (int64_t)p * CHI2;
    // thread (m, h) writes columns [32h, 32h + 32) of every 64-wide chunk
#pragma unroll
    for (int kc = 0; kc < KCH; ++kc) {
      unsigned char* Ahi = Asm + kc * 2 * A_CHUNK;
      unsigned char* Alo = Ahi + A_CHUNK;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        float x[8];
        if (valid) {
          const float4 u = *reinterpret_cast<const float4*>(m2row + kc * 64 + 32 * h + q * 8);
          const float4 w = *reinterpret_cast<const float4*>(m2row + kc * 64 + 32 * h + q * 8 + 4);
          x[0] = u.x, x[1] = u.y, x[2] = u.z, x[3] = u.w, x[4] = w.x, x[5] = w.y, x[6] = w.z, x[7] = w.w;
        } else {
#pragma unroll
          for (int t = 0; t < 8; ++t) x[t] = 0.f;
        }
        uint32_t hw[4], lw[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          __nv_bfloat162 hh = __floats2bfloat162_rn(x[2 * t], x[2 * t + 1]);
          float2 hf = __bfloat1622float2(hh);
          hw[t] = *reinterpret_cast<uint32_t*>(&hh);
          lw[t] = pack_bf16(x[2 * t] - hf.x, x[2 * t + 1] - hf.y);
        }
        const int chunk = (4 * h + q) ^ (m & 7);
        const int off = m * 128 + chunk * 16;
        *reinterpret_cast<uint4*>(Ahi + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        *reinterpret_cast<uint4*>(Alo + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
      }
    }
    fence_proxy_async();
    mbar_arrive(&a_ready);

    const float* m1row =
        P.m1_S ? P.m1_ptr + (int64_t)P.m1_S[p] * P.chi1 : P.m1_ptr + (int64_t)p * P.chi1;
    const int e_in = valid ? ((P.m1_exp ? P.m1_exp[p] : 0) + (P.m2_exp ? P.m2_exp[p] : 0)) : 0;
    float acc[ACC];
#pragma unroll
    for (int i = 0; i < ACC; ++i) acc[i] = 0.f;
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    bool ok = true;
    float mb[NBT], mbn[NBT];
#pragma unroll
    for (int i = 0; i < NBT; ++i) mbn[i] = valid ? m1row[i] : 0.f;
    for (int t = 0; t < ntiles; ++t) {
#pragma unroll
      for (int i = 0; i < NBT; ++i) mb[i] = mbn[i];
      if (t + 1 < ntiles) {
#pragma unroll
        for (int i = 0; i < NBT; ++i) mbn[i] = valid ? m1row[(t + 1) * NBT + i] : 0.f;
      }
      const int buf = t & 1;
      if (!mbar_wait(&tfull[buf], (t >> 1) & 1, P.wait_limit)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int cc = 0; cc < 4; ++cc) {
        float v[32];
        tmem_ld32(tmem + lane_base + (uint32_t)(buf * T2_N + h * 128 + cc * 32), v);
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int jl = cc * 32 + j;  // column within this half
          acc[jl / NBT] = fmaf(v[j], mb[jl % NBT], acc[jl / NBT]);
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(&tempty[buf]);
    }
    if (!ok) {
      atomicOr(P.err, TC_ERR_TIMEOUT);
      sh_abort = 1;
    }
    // power-of-two row normalisation across both halves, then store
    float mx = 0.f;
#pragma unroll
    for (int i = 0; i < ACC; ++i) mx = fmaxf(mx, fabsf(acc[i]));
    rowmax[h][m] = mx;
    asm volatile("bar.sync 1, 256;" ::: "memory");
    mx = fmaxf(rowmax[0][m], rowmax[1][m]);
    int ex = 0;
    if (mx > 0.f) frexpf(mx, &ex);
    if (valid && ok) {
      float* dst = P.out + (int64_t)p * CHIA + h * ACC;
#pragma unroll
      for (int i = 0; i < ACC; i += 4)
        *reinterpret_cast<float4*>(dst + i) = make_float4(
            scalbnf(acc[i], -ex), scalbnf(acc[i + 1], -ex), scalbnf(acc[i + 2], -ex), scalbnf(acc[i + 3], -ex));
      if (h == 0) P.out_exp[p] = e_in + ex;
    }
  } else if (warp == 8) {
    // ------------------------------------------------------------ TMA ----
    if (lane == 0) {
      bool ok = true;
      const int nst = ntiles * KCH;
      for (int si = 0; si < nst; ++si) {
        const int s = si % STAGES, use = si / STAGES;
        if (use > 0 && !mbar_wait(&empty_bar[s], (use - 1) & 1, P.wait_limit)) {
          ok = false;
          break;
        }
        unsigned char* Bhi = Bsm + s * STAGE_BYTES;
        unsigned char* Blo = Bhi + B_BYTES;
        const int t = si / KCH, kc = si % KCH;
        mbar_arrive_expect_tx(&full_bar[s], 2 * B_BYTES);
        tma_load_3d(Bhi, &map_hi, &full_bar[s], kc * TC_KC, t * NBT, g * CHIA);
        tma_load_3d(Blo, &map_lo, &full_bar[s], kc * TC_KC, t * NBT, g * CHIA);
      }
      if (!ok) atomicOr(P.err, TC_ERR_TIMEOUT);
    }
  } else {
    // ------------------------------------------------------------ MMA ----
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16(TC_M, T2_N);
      bool ok = mbar_wait(&a_ready, 0, P.wait_limit);
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      for (int t = 0; t < ntiles && ok; ++t) {
        const int buf = t & 1;
        if (t >= 2 && !mbar_wait(&tempty[buf], ((t >> 1) - 1) & 1, P.wait_limit)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dcol = tmem + (uint32_t)(buf * T2_N);
        for (int kc = 0; kc < KCH; ++kc) {
          const int si = t * KCH + kc;
          const int s = si % STAGES, use = si / STAGES;
          if (!mbar_wait(&full_bar[s], use & 1, P.wait_limit)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          unsigned char* Ahi = Asm + kc * 2 * A_CHUNK;
          unsigned char* Alo = Ahi + A_CHUNK;
          unsigned char* Bhi = Bsm + s * STAGE_BYTES;
          unsigned char* Blo = Bhi + B_BYTES;
          const uint64_t dah = sw128_desc(Ahi), dal = sw128_desc(Alo);
          const uint64_t dbh = sw128_desc(Bhi), dbl = sw128_desc(Blo);
#pragma unroll
          for (int k = 0; k < TC_KC / 16; ++k) {
            const uint64_t adv = (uint64_t)(k * 32) >> 4;
            mma_bf16(dcol, dah + adv, dbh + adv, idesc, (kc | k) != 0);
            mma_bf16(dcol, dah + adv, dbl + adv, idesc, 1);
            mma_bf16(dcol, dal + adv, dbh + adv, idesc, 1);
          }
          mma_commit(&empty_bar[s]);
        }
        if (ok) mma_commit(&tfull[buf]);
      }
      if (!ok) atomicOr(P.err, TC_ERR_TIMEOUT);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 8) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
  }
}

// BF16 hi / lo split of the FP32 tensors, per-vertex offsets padded to 64
// elements so every vertex base is 128-byte aligned for TMA.
__global__ void k_split_bf16(const float* __restrict__ src, __nv_bfloat16* __restrict__ hi,
                             __nv_bfloat16* __restrict__ lo, const int64_t* __restrict__ soff,
                             const int64_t* __restrict__ doff, int V) {
  const int v = blockIdx.y;
  const int64_t n = soff[v + 1] - soff[v];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float x = src[soff[v] + i];
    __nv_bfloat16 h = __float2bfloat16_rn(x);
    hi[doff[v] + i] = h;
    lo[doff[v] + i] = __float2bfloat16_rn(x - __bfloat162float(h));
  }
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    cudaGetLastError();
  });
  return fn;
}

CUtensorMap make_map(const void* base, int64_t K, int64_t rows, int box_rows) {
  auto enc = get_encode();
  TNFA_CHECK(enc != nullptr, TNFA_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
  CUtensorMap m;
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  cuuint32_t box[2] = {(cuuint32_t)TC_KC, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides,
                   box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  TNFA_CHECK(r == CUDA_SUCCESS, TNFA_ERR_CUDA,
             "cuTensorMapEncodeTiled failed with code " + std::to_string((int)r));
  return m;
}

// 3-D map of one vertex's slice stack T[s][a][b][c] (BF16): dims {chi2,
// chi1, S * chi_a}, box {64, 256 / chi_a, chi_a}.
CUtensorMap make_map3(const void* base, int chi2, int chi1, int64_t sa, int box_b, int box_a) {
  auto enc = get_encode();
  TNFA_CHECK(enc != nullptr, TNFA_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
  CUtensorMap m;
  cuuint64_t dims[3] = {(cuuint64_t)chi2, (cuuint64_t)chi1, (cuuint64_t)sa};
  cuuint64_t strides[2] = {(cuuint64_t)chi2 * 2, (cuuint64_t)chi2 * chi1 * 2};
  cuuint32_t box[3] = {(cuuint32_t)TC_KC, (cuuint32_t)box_b, (cuuint32_t)box_a};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides,
                   box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  TNFA_CHECK(r == CUDA_SUCCESS, TNFA_ERR_CUDA,
             "cuTensorMapEncodeTiled (3-D) failed with code " + std::to_string((int)r));
  return m;
}

template <int CHIA, int CHI2>
void launch_tc2(tnfa_ctx* ctx, const CUtensorMap& mh, const CUtensorMap& ml, const TcParams& p,
                unsigned grid) {
  constexpr int KCH = CHI2 / TC_KC;
  const int smem = 2 * KCH * TC_M * TC_KC * 2 + 2 * 2 * T2_N * TC_KC * 2 + 1024;
  TNFA_CUDA(cudaFuncSetAttribute(k_contract_tc2<CHIA, CHI2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem));
  k_contract_tc2<CHIA, CHI2><<<grid, TC_THREADS, smem, ctx->stream>>>(mh, ml, p);
  TNFA_LAUNCH_CHECK();
}

template <int N, int CHI2, int STAGES, bool BILIN>
void launch_tc(tnfa_ctx* ctx, const CUtensorMap& mh, const CUtensorMap& ml, const TcParams& p,
               unsigned grid) {
  constexpr int STAGE_BYTES = 2 * TC_M * TC_KC * 2 + 2 * N * TC_KC * 2;
  const int smem = STAGES * STAGE_BYTES + 1024;
  TNFA_CUDA(cudaFuncSetAttribute(k_contract_tc<N, CHI2, STAGES, BILIN>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  k_contract_tc<N, CHI2, STAGES, BILIN><<<grid, TC_THREADS, smem, ctx->stream>>>(mh, ml, p);
  TNFA_LAUNCH_CHECK();
}

struct TcCache {
  std::vector<int64_t> doff;  // padded offsets of the BF16 copies
};

}  // namespace

CUtensorMap tc_make_map3(const void* base, int x_dim, int y_dim, int64_t z_dim, int box_y,
                         int box_z) {
  return make_map3(base, x_dim, y_dim, z_dim, box_y, box_z);
}

bool tc_vertex_eligible(int nchild, const int* child_dims, int chi_a) {
  if (nchild < 1 || nchild > 2) return false;
  const int chi2 = child_dims[nchild - 1];
  if (chi2 != 64 && chi2 != 128) return false;
  if (chi_a == 1)  // root of two children: bilinear mode, N = chi1
    return nchild == 2 && (child_dims[0] == 64 || child_dims[0] == 128);
  if (chi_a != 64 && chi_a != 128) return false;
  if (nchild == 2 && (child_dims[0] < 1 || child_dims[0] > 4096)) return false;
  return true;
}

int tc_tile_rows() { return TC_M; }

static std::vector<int64_t> padded_offsets(const Topo& T) {
  std::vector<int64_t> d(T.V + 1, 0);
  for (int v = 0; v < T.V; ++v) d[v + 1] = d[v] + ((T.size(v) + 63) / 64) * 64;
  return d;
}

void tc_prepare_net(tnfa_ctx* ctx, const tnfa_net* net) {
  if (net->d_bhi) return;
  const Topo& T = net->topo;
  const float* src = net->dtype == TNFA_F32 ? (const float*)net->d : (const float*)net->d_f32;
  TNFA_CHECK(src != nullptr, TNFA_ERR_INVALID_ARGUMENT, "no FP32 tensors for the split");
  std::vector<int64_t> doff = padded_offsets(T);
  std::vector<int64_t> soff(T.off.begin(), T.off.end());
  DBuf ds(ctx, soff.size() * 8), dd(ctx, doff.size() * 8);
  TNFA_CUDA(cudaMemcpyAsync(ds.p, soff.data(), soff.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
  TNFA_CUDA(cudaMemcpyAsync(dd.p, doff.data(), doff.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
  net->d_bhi = dalloc(ctx, (size_t)doff[T.V] * 2);
  net->d_blo = dalloc(ctx, (size_t)doff[T.V] * 2);
  int64_t maxn = 1;
  for (int v = 0; v < T.V; ++v) maxn = std::max<int64_t>(maxn, T.size(v));
  dim3 grid(grid_for(maxn, 256, 2048), T.V);
  k_split_bf16<<<grid, 256, 0, ctx->stream>>>(src, (__nv_bfloat16*)net->d_bhi,
                                               (__nv_bfloat16*)net->d_blo, ds.as<int64_t>(),
                                               dd.as<int64_t>(), T.V);
  TNFA_LAUNCH_CHECK();
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
}

void tc_contract_vertex(tnfa_ctx* ctx, const tnfa_net* net, int v, const VertexJob<float>& j,
                        int tile_rows, int* err) {
  TNFA_CHECK(tile_rows == TC_M, TNFA_ERR_INVALID_ARGUMENT, "tile rows mismatch");
  const Topo& T = net->topo;
  std::vector<int64_t> doff = padded_offsets(T);
  const __nv_bfloat16* hi = (const __nv_bfloat16*)net->d_bhi + doff[v];
  const __nv_bfloat16* lo = (const __nv_bfloat16*)net->d_blo + doff[v];
  const bool bilin = j.chi_a == 1;
  const int N = bilin ? j.ch[0].dim : j.chi_a;
  const int K = bilin ? j.ch[1].dim : j.K;
  CUtensorMap mh = make_map(hi, K, (int64_t)j.site_dim * N, N);
  CUtensorMap ml = make_map(lo, K, (int64_t)j.site_dim * N, N);
  TcParams p{};
  const ChildSrc<float>& c2 = j.ch[j.nchild - 1];
  p.m2_ptr = c2.ptr;
  p.m2_exp = c2.exps;
  p.m2_S = c2.S;
  p.chi2 = c2.dim;
  if (j.nchild == 2) {
    p.m1_ptr = j.ch[0].ptr;
    p.m1_exp = j.ch[0].exps;
    p.m1_S = j.ch[0].S;
    p.chi1 = j.ch[0].dim;
  } else {
    p.chi1 = 1;
  }
  p.N = N;
  p.K = K;
  p.out = j.out;
  p.out_exp = j.out_exp;
  p.perm = j.perm;
  p.grp_off = j.grp_off;
  p.grp_cnt = j.grp_cnt;
  p.tile_start = j.tile_start;
  p.ngroups = j.ngroups;
  p.err = err;
  p.wait_limit = ctx->tc_wait_limit;
  const unsigned grid = (unsigned)((j.Pc + TC_M - 1) / TC_M + j.ngroups);
  KernelScope ks(ctx, "contract_tc", 2.0 * j.Pc * (double)j.K * j.chi_a,
                 4.0 * ((double)j.Pc * (p.chi1 + p.chi2 + j.chi_a)) +
                     4.0 * j.site_dim * (double)j.chi_a * j.K);
  // Two children: the second child first (k_contract_tc2) or the Kronecker
  // formulation (k_contract_tc); the autotuner times both per shape, the
  // default is tc2, and TNFA_TC_KRON=1 forces the Kronecker form.
  static const bool kron_only = getenv("TNFA_TC_KRON") && *getenv("TNFA_TC_KRON") == '1';
  auto kron = [&]() {
    if (N == 128 && p.chi2 == 128) launch_tc<128, 128, 3, false>(ctx, mh, ml, p, grid);
    else if (N == 128 && p.chi2 == 64) launch_tc<128, 64, 3, false>(ctx, mh, ml, p, grid);
    else if (N == 64 && p.chi2 == 128) launch_tc<64, 128, 4, false>(ctx, mh, ml, p, grid);
    else if (N == 64 && p.chi2 == 64) launch_tc<64, 64, 4, false>(ctx, mh, ml, p, grid);
    else fail(TNFA_ERR_UNSUPPORTED, "tensor-core shape");
  };
  if (!bilin && !kron_only && j.nchild == 2 && p.chi1 % (T2_N / N) == 0) {
    const int nbt = T2_N / N;
    CUtensorMap h3 = make_map3(hi, p.chi2, p.chi1, (int64_t)j.site_dim * N, nbt, N);
    CUtensorMap l3 = make_map3(lo, p.chi2, p.chi1, (int64_t)j.site_dim * N, nbt, N);
    auto tc2 = [&]() {
      if (N == 128 && p.chi2 == 128) launch_tc2<128, 128>(ctx, h3, l3, p, grid);
      else if (N == 128 && p.chi2 == 64) launch_tc2<128, 64>(ctx, h3, l3, p, grid);
      else if (N == 64 && p.chi2 == 128) launch_tc2<64, 128>(ctx, h3, l3, p, grid);
      else launch_tc2<64, 64>(ctx, h3, l3, p, grid);
    };
    const std::string key = "tc:" + std::to_string(N) + ":" + std::to_string(p.chi1) + "x" +
                            std::to_string(p.chi2);
    tune(ctx, key, 2, 2.0 * j.Pc * (double)j.K * j.chi_a, [&](int i) { i == 0 ? tc2() : kron(); });
    return;
  }
  if (!bilin) {
    kron();
  } else {
    if (N == 128 && p.chi2 == 128) launch_tc<128, 128, 3, true>(ctx, mh, ml, p, grid);
    else if (N == 128 && p.chi2 == 64) launch_tc<128, 64, 3, true>(ctx, mh, ml, p, grid);
    else if (N == 64 && p.chi2 == 128) launch_tc<64, 128, 4, true>(ctx, mh, ml, p, grid);
    else if (N == 64 && p.chi2 == 64) launch_tc<64, 64, 4, true>(ctx, mh, ml, p, grid);
    else fail(TNFA_ERR_UNSUPPORTED, "tensor-core shape");
  }
}

}  // namespace tnfa
