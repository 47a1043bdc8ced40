// Accurate mixed-precision vertex contraction for batched evaluation: the
// tensor-core product made error free by integer slicing (tcgen05, sm_103a).
//
// A vertex with two children contracts, for the points p of one site value s,
//   out[p, a] = sum_b m1[p, b] sum_c m2[p, c] T_s[a][b][c]
// from FP64 messages m1, m2 to an FP64 message out.  The inner contraction
// runs on the tensor cores on slices of the operands (the error-free
// splitting of Ozaki, Ogita, Oishi & Rump, Numer. Algorithms 59 (2012), in
// the tensor-core form of Mukunoki, Ozaki, Ogita & Imamura, ISC 2020):
//   m2[p, c]     = 2^E2(p)   * sum_{i=1..6} dA_i[p, c] 2^(-8i)
//   T_s[a][b][c] = 2^eB(s,a) * sum_{j=1..6} dB_j[s][a][b][c] 2^(-8j)
// Every digit is an integer with |d_1| <= 256 and |d_i| <= 128 (i > 1), exact
// in BF16, so each MMA product is exact and a sum over K <= 128 of them stays
// within 2^24: the FP32 accumulation in tensor memory is exact too.  Digit
// pairs with the same i + j = k share one accumulator (at most 2^24 by the
// digit bounds); pairs with i + j > 8 are left out.  That is 26 pair passes
// of M = 128 points x N = 256 columns x K per product.  The epilogue folds
// each group into
//   out[p, a] += 2^(-8k) sum_b m1[p, b] acc_k[p, (a, b)]
// in double-float (FP32 pairs: error-free products and sums) for the groups
// k <= 4 and plain FP32 into the pair's low word for k >= 5 (at most 2^-24
// of the result), the pair renormalised after every group; each N-tile's pair
// sums (8 values of b) go to FP64 once.  The
// contraction is accurate to a few units of 2^-48 of the result's norm
// (relative), within a small factor of an FP64 evaluation.
//
// Shared memory holds six A plane-chunks of 128 points x 64 K (96 KB): all
// six digit planes when K = 64, three at a time when K = 128 (two phases over
// the digit planes; the partial result of phase 0 waits in the output
// message).  B (the digit planes of T_s) streams through four 32 KB stages as
// N-tiles of 32 parent values a x 8 first-child values b by 64 K (3-D TMA
// box {64 c, 8 b, 32 a}), one load per digit pair.  Two tensor-memory
// accumulators of 256 columns alternate between the MMA issuer and the
// epilogue.
//
// Roles (320 threads): warps 0-7 build the A planes, then run the epilogue
// (thread: point row m = 32 (w % 4) + lane, column half h = w / 4, i.e. 16
// values of a x 8 of b per N-tile); warp 8 issues the TMA loads; warp 9
// issues the MMAs.  Every mbarrier wait is bounded by the context's wait
// budget; a timeout sets an error bit, the role stops, the TMA and MMA roles
// wait (again bounded) for their copies and MMAs in flight, and the CTA
// releases its tensor memory.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <climits>

#include "evaluate.cuh"
#include "tc_ptx.cuh"

namespace tnfa {

namespace {

using namespace ptx;

constexpr int OZ_M = 128;                        // points per tile
constexpr int OZ_NA = 32, OZ_NB = 8;             // an N-tile: 32 values of a x 8 of b
constexpr int OZ_N = OZ_NA * OZ_NB;              // 256 columns
constexpr int OZ_KC = 64;                        // K elements per chunk (128 B of BF16)
constexpr int OZ_DIG = 6;                        // digits per operand
constexpr int OZ_KMAX = 8;                       // digit pairs with i + j <= 8
constexpr int OZ_SLOTS = 6;                      // A plane-chunks in shared memory
constexpr int OZ_SLOT_BYTES = OZ_M * OZ_KC * 2;  // 16 KB
constexpr int OZ_STAGES = 4;
constexpr int OZ_B_BYTES = OZ_N * OZ_KC * 2;     // 32 KB
constexpr int OZ_THREADS = 320;
constexpr int OZ_SMEM = OZ_SLOTS * OZ_SLOT_BYTES + OZ_STAGES * OZ_B_BYTES + 1024;

struct OzParams {
  const double* m1_ptr;  // first child: message rows or (fused leaf) tensor rows
  const int* m1_exp;
  const uint8_t* m1_S;
  const double* m2_ptr;  // second child
  const int* m2_exp;
  const uint8_t* m2_S;
  int chi_a, chi1, site_dim;
  const int* bexp;  // [site][chi_a] base-2 exponents of the tensor slabs
  double* out;      // Pc x chi_a
  int* out_exp;
  const int* perm;
  const int* grp_off;
  const int* grp_cnt;
  const int* tile_start;
  int ngroups;
  int* err;
  uint32_t wait_limit;  // try_wait polls before a wait gives up
  int drop_arrive;      // nonzero: the A-ready arrive of phase 0 is withheld (timeout test)
};

// x 2^-E as an FP32 pair hi + lo: hi is x 2^-E with its significand cut to
// 24 bits, lo the remaining 29 bits rounded to 24 (48 bits in all), built
// from the FP64 bit pattern with integer and FP32 operations only (GB300
// runs FP64 arithmetic and FP64 conversions at 1/64 of the FP32 rate).
// Results below 2^-126 (far below the row maximum 2^E) flush to zero.
__device__ __forceinline__ void split_f64(double x, int E, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned w1 = (unsigned)(b >> 32), w0 = (unsigned)b;
  const int be = (int)((w1 >> 20) & 0x7FF);
  const int e = be - 1023 - E;  // exponent of x 2^-E
  if (be == 0 || e < -126 || e > 127) {
    hi = lo = 0.f;
    return;
  }
  const unsigned sign = w1 & 0x80000000u;
  hi = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | ((w1 & 0xFFFFFu) << 3) | (w0 >> 29));
  const unsigned rem = w0 & 0x1FFFFFFFu;  // weight 2^(e - 52)
  if (rem == 0 || e - 52 < -126) {
    lo = 0.f;
    return;
  }
  // float(rem) by the 2^23 bias trick on its two parts, one rounding
  const float rl = __fsub_rn(__uint_as_float(0x4B000000u | (rem & 0x7FFFFFu)), 8388608.f);
  const float rh = __fsub_rn(__uint_as_float(0x4B000000u | (rem >> 23)), 8388608.f);
  const float r = __fmaf_rn(rh, 8388608.f, rl);
  lo = __uint_as_float(__float_as_uint(__fmul_rn(r, __uint_as_float((unsigned)(e - 52 + 127) << 23))) | sign);
}

// The PP digits first+1 .. first+PP (1-based) of xs = r + l, |xs| < 1 (an
// FP32 pair, 48 bits): xs = sum_i d_i 2^(-8i) + O(2^-48).  Each digit is the
// rounded leading part of the pair times 256, taken off exactly, and the
// pair is renormalised by an error-free sum.
template <int PP>
__device__ __forceinline__ void oz_digits(float r, float l, int first, float (&d)[PP]) {
#pragma unroll
  for (int o = 0; o < PP; ++o) d[o] = 0.f;
#pragma unroll
  for (int i = 0; i < OZ_DIG; ++i) {
    r = __fmul_rn(r, 256.f);
    l = __fmul_rn(l, 256.f);
    const float di = rintf(r);
    r = __fsub_rn(r, di);
    const float s = __fadd_rn(r, l);
    const float bp = __fsub_rn(s, r);
    l = __fadd_rn(__fsub_rn(r, __fsub_rn(s, bp)), __fsub_rn(l, bp));
    r = s;
#pragma unroll
    for (int o = 0; o < PP; ++o) d[o] = (i == first + o) ? di : d[o];
  }
}

// Exact widening of an FP32 value by its bit pattern (no FP64 conversion
// unit); FP32 subnormals, far below every sum here, widen to zero.
__device__ __forceinline__ double f2d(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned e = (u >> 23) & 0xFFu;
  if (e == 0) return 0.0;
  return __longlong_as_double((long long)(((unsigned long long)(u & 0x80000000u) << 32) |
                                          ((unsigned long long)(e + 896u) << 52) |
                                          ((unsigned long long)(u & 0x7FFFFFu) << 29)));
}

// s + e = a + b exactly (Knuth's two-sum, no ordering assumption).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  const float t = __fadd_rn(a, b);
  const float bp = __fsub_rn(t, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(t, bp)), __fsub_rn(b, bp));
  s = t;
}

// Digit groups k = i + j of a phase, in issue order.  Phase 0 holds every
// group 2..8; its double-float groups (k <= 4, the slow drains) alternate
// with FP32 ones so that a long drain overlaps a long MMA unit in the
// two-buffer pipeline.  Later phases hold k = ph * PP + 2 .. 8 in order.
__device__ __forceinline__ int oz_ngroups(int ph, int pp) {
  return ph == 0 ? OZ_KMAX - 1 : OZ_KMAX - (ph * pp + 2) + 1;
}
__device__ __forceinline__ int oz_group(int ph, int gi, int pp) {
  if (ph == 0) {
    constexpr int order = 0x8763542;  // 2, 4, 5, 3, 6, 7, 8 (a nibble each, lowest first)
    return (order >> (4 * gi)) & 0xF;
  }
  return ph * pp + 2 + gi;
}

// (ah, al) += (bh, bl) in double-float with the accurate addition (Joldes,
// Muller & Popescu, ACM TOMS 44 (2017), algorithm 6): relative error about
// 3 * 2^-48.
__device__ __forceinline__ void dd_add(float& ah, float& al, float bh, float bl) {
  float s, e, t, f;
  two_sum(ah, bh, s, e);
  two_sum(al, bl, t, f);
  e = __fadd_rn(e, t);
  const float s2 = __fadd_rn(s, e);
  e = __fsub_rn(e, __fsub_rn(s2, s));
  e = __fadd_rn(e, f);
  ah = __fadd_rn(s2, e);
  al = __fsub_rn(e, __fsub_rn(ah, s2));
}

template <int KCH>
__global__ void __launch_bounds__(OZ_THREADS, 1)
    k_contract_oz(const __grid_constant__ CUtensorMap mapB, const OzParams P) {
  constexpr int PP = OZ_DIG / KCH;  // digit planes resident per phase
  constexpr int NPH = KCH;          // phases over the digit planes of A
  constexpr int CHI2 = KCH * OZ_KC;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[OZ_STAGES], empty_bar[OZ_STAGES], tfull[2], tempty[2],
      a_ready, mma_done;
  __shared__ uint32_t tmem_base_sh;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* Asm = smem;
  unsigned char* Bsm = smem + OZ_SLOTS * OZ_SLOT_BYTES;

  const int blk = blockIdx.x;
  const int ng = P.ngroups;
  if (blk >= P.tile_start[ng]) return;
  int g = 0;
  while (g + 1 < ng && P.tile_start[g + 1] <= blk) ++g;
  const int row0 = P.grp_off[g] + (blk - P.tile_start[g]) * OZ_M;
  const int nrows = min(OZ_M, P.grp_off[g] + P.grp_cnt[g] - row0);
  if (nrows <= 0) return;
  const int nab = P.chi_a / OZ_NA, nbb = P.chi1 / OZ_NB;
  const uint32_t lim = P.wait_limit;

  if (tid == 0) {
    for (int s = 0; s < OZ_STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 256);
    }
    mbar_init(&a_ready, 256);
    mbar_init(&mma_done, 1);
    fence_mbar_init();
  }
  if (warp == 8) tmem_alloc(&tmem_base_sh, 2 * OZ_N);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_sh;

  if (warp < 8) {
    // ---------------------------------------- A digit planes + epilogue ----
    const int m = (warp & 3) * 32 + lane;
    const int h = warp >> 2;
    const bool valid = m < nrows;
    const int p = valid ? (P.perm ? P.perm[row0 + m] : row0 + m) : 0;
    const double* m1row =
        P.m1_S ? P.m1_ptr + (int64_t)P.m1_S[p] * P.chi1 : P.m1_ptr + (int64_t)p * P.chi1;
    const double* m2row =
        P.m2_S ? P.m2_ptr + (int64_t)P.m2_S[p] * CHI2 : P.m2_ptr + (int64_t)p * CHI2;
    // Row exponents: 2^E bounds |row| strictly.  The two threads of a row
    // scan one half each and meet in shared memory (the start of the A
    // region, free until the planes are written).
    int* rexp = reinterpret_cast<int*>(Asm);  // [m1 | m2][h][row]
    {
      double mx1 = 0.0, mx2 = 0.0;
      if (valid) {
        const int n1 = P.chi1 / 2;
        for (int b = h * n1; b < (h + 1) * n1; ++b) mx1 = fmax(mx1, fabs(m1row[b]));
        for (int c = h * (CHI2 / 2); c < (h + 1) * (CHI2 / 2); ++c) mx2 = fmax(mx2, fabs(m2row[c]));
      }
      // ilogb(x) + 1 is frexp's exponent: 2^(e-1) <= |x| < 2^e
      const int e1 = mx1 > 0.0 ? ilogb(mx1) + 1 : INT_MIN;
      const int e2 = mx2 > 0.0 ? ilogb(mx2) + 1 : INT_MIN;
      rexp[(0 * 2 + h) * OZ_M + m] = e1;
      rexp[(1 * 2 + h) * OZ_M + m] = e2;
    }
    asm volatile("bar.sync 1, 256;" ::: "memory");
    int E1 = max(rexp[(0 * 2 + 0) * OZ_M + m], rexp[(0 * 2 + 1) * OZ_M + m]);
    int E2 = max(rexp[(1 * 2 + 0) * OZ_M + m], rexp[(1 * 2 + 1) * OZ_M + m]);
    if (E1 == INT_MIN) E1 = 0;
    if (E2 == INT_MIN) E2 = 0;
    asm volatile("bar.sync 1, 256;" ::: "memory");  // every row read before A overwrites
    const int e_in = valid ? ((P.m1_exp ? P.m1_exp[p] : 0) + (P.m2_exp ? P.m2_exp[p] : 0)) : 0;
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    bool ok = true;
    uint32_t u = 0;  // accumulator unit, in the MMA issuer's order

#pragma unroll 1
    for (int ph = 0; ph < NPH && ok; ++ph) {
      // thread (m, h) writes 16-byte chunks 4h .. 4h+3 (columns 32h .. 32h+31)
      // of every 64-wide K chunk, 128-byte swizzled, for the phase's planes
#pragma unroll
      for (int kc = 0; kc < KCH; ++kc) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int off = m * 128 + (((4 * h + q) ^ (m & 7)) * 16);
#pragma unroll
          for (int t = 0; t < 8; t += 2) {
            const int c = kc * OZ_KC + 32 * h + q * 8 + t;
            float d0[PP], d1[PP], r0 = 0.f, l0 = 0.f, r1 = 0.f, l1 = 0.f;
            if (valid) {
              split_f64(m2row[c], E2, r0, l0);
              split_f64(m2row[c + 1], E2, r1, l1);
            }
            oz_digits<PP>(r0, l0, ph * PP, d0);
            oz_digits<PP>(r1, l1, ph * PP, d1);
#pragma unroll
            for (int i = 0; i < PP; ++i)
              *reinterpret_cast<uint32_t*>(Asm + (i * KCH + kc) * OZ_SLOT_BYTES + off + 2 * t) =
                  pack_bf16(d0[i], d1[i]);
          }
        }
      }
      fence_proxy_async();
      if (!(P.drop_arrive && ph == 0)) mbar_arrive(&a_ready);

      for (int ab = 0; ab < nab && ok; ++ab) {
        float ah[16], al[16];  // the a-block's sums (double-float)
        float sh[16], sl[16];  // the current four N-tiles' sums
#pragma unroll
        for (int i = 0; i < 16; ++i) ah[i] = al[i] = sh[i] = sl[i] = 0.f;
        // m1 of the next N-tile is loaded one N-tile ahead (its latency hides
        // behind the current N-tile's groups)
        double m1n[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) m1n[t] = valid ? m1row[t] : 0.0;
        for (int bb = 0; bb < nbb && ok; ++bb) {
          float m1h[8], m1l[8];
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            m1h[t] = m1l[t] = 0.f;
            split_f64(m1n[t], E1, m1h[t], m1l[t]);
          }
          if (bb + 1 < nbb) {
#pragma unroll
            for (int t = 0; t < 8; ++t) m1n[t] = valid ? m1row[(bb + 1) * OZ_NB + t] : 0.0;
          }
          for (int gi = 0; gi < oz_ngroups(ph, PP); ++gi) {
            const int k = oz_group(ph, gi, PP);
            const int buf = u & 1;
            const bool got = mbar_wait(&tfull[buf], (u >> 1) & 1, lim);
            if (!__all_sync(0xffffffffu, got)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t col = tmem + lane_base + (uint32_t)(buf * OZ_N + h * 128);
            // double-float fold of the groups k <= 4; the k >= 5 groups (at most
            // 2^-24 of the result) only need FP32 and ride in the low word
            const float w = __int_as_float((127 - 8 * (k - 2)) << 23);  // 2^(-8(k-2))
            const bool pair = k <= 4;
            float mw[8];  // m1 high words times the group's weight (exact)
#pragma unroll
            for (int t = 0; t < 8; ++t) mw[t] = __fmul_rn(m1h[t], w);
#pragma unroll
            for (int cc = 0; cc < 8; ++cc) {  // 2 values of a x 8 of b per load
              float v[16];
              tmem_ld16(col + cc * 16, v);
#pragma unroll
              for (int q = 0; q < 2; ++q) {
                const int ai = cc * 2 + q;
                if (pair) {
                  // error-free products, summed pairwise (a tree of depth 3,
                  // so that the dependency chains stay short), then into the
                  // pair; every rounding error goes to the low word
                  float pr[8], lo = 0.f;
#pragma unroll
                  for (int bl = 0; bl < 8; ++bl) {
                    const float x = __fmul_rn(v[q * 8 + bl], w);  // exact: a power of two
                    pr[bl] = __fmul_rn(m1h[bl], x);
                    float pe = __fmaf_rn(m1h[bl], x, -pr[bl]);
                    pe = __fmaf_rn(m1l[bl], x, pe);
                    lo = __fadd_rn(lo, pe);
                  }
#pragma unroll
                  for (int st = 1; st < 8; st *= 2)
#pragma unroll
                    for (int bl = 0; bl < 8; bl += 2 * st) {
                      float e;
                      two_sum(pr[bl], pr[bl + st], pr[bl], e);
                      lo = __fadd_rn(lo, e);
                    }
                  float e;
                  two_sum(sh[ai], pr[0], sh[ai], e);
                  sl[ai] = __fadd_rn(sl[ai], __fadd_rn(lo, e));
                } else {
#pragma unroll
                  for (int bl = 0; bl < 8; ++bl) sl[ai] = __fmaf_rn(mw[bl], v[q * 8 + bl], sl[ai]);
                }
              }
            }
            tc_fence_before();
            mbar_arrive(&tempty[buf]);
            ++u;
            // renormalise each pair (error free) so that the low word starts
            // the next group small
#pragma unroll
            for (int i = 0; i < 16; ++i) {
              const float t = __fadd_rn(sh[i], sl[i]);
              sl[i] = __fsub_rn(sl[i], __fsub_rn(t, sh[i]));
              sh[i] = t;
            }
          }
          // every four N-tiles (32 values of b) the sums join the a-block's by
          // an accurate double-float addition
          if ((bb & 3) == 3 || bb == nbb - 1) {
#pragma unroll
            for (int i = 0; i < 16; ++i) {
              dd_add(ah[i], al[i], sh[i], sl[i]);
              sh[i] = sl[i] = 0.f;
            }
          }
        }
        if (ok && valid) {
          double* dst = P.out + (int64_t)p * P.chi_a + ab * OZ_NA + h * 16;
          const int* be = P.bexp + (int64_t)g * P.chi_a + ab * OZ_NA + h * 16;
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            double t = f2d(ah[i]) + f2d(al[i]);
            if (ph > 0) t += dst[i];  // phase 0's partial sum of this entry
            // the slab exponent and the digit weight 2^-16 (the rows' 2^(E1+E2)
            // goes to the message exponent)
            if (ph == NPH - 1) t *= __longlong_as_double((long long)(be[i] - 16 + 1023) << 52);
            dst[i] = t;
          }
        }
      }
    }
    if (!ok) atomicOr(P.err, ERR_TIMEOUT);
    if (ok && valid && h == 0) P.out_exp[p] = e_in + E1 + E2;
  } else if (warp == 8) {
    // ------------------------------------------------------------ TMA ----
    if (lane == 0) {
      bool ok = true;
      uint32_t si = 0;
      for (int ph = 0; ph < NPH && ok; ++ph)
        for (int ab = 0; ab < nab && ok; ++ab)
          for (int bb = 0; bb < nbb && ok; ++bb)
            for (int gi = 0; gi < oz_ngroups(ph, PP) && ok; ++gi) {
              const int k = oz_group(ph, gi, PP);
              const int ilo = max(ph * PP + 1, k - OZ_DIG), ihi = min(ph * PP + PP, k - 1);
              for (int i = ilo; i <= ihi && ok; ++i)
                for (int kc = 0; kc < KCH; ++kc) {
                  const int s = si % OZ_STAGES;
                  const uint32_t use = si / OZ_STAGES;
                  if (use > 0 && !mbar_wait(&empty_bar[s], (use - 1) & 1, lim)) {
                    ok = false;
                    break;
                  }
                  const int j = k - i;
                  mbar_arrive_expect_tx(&full_bar[s], OZ_B_BYTES);
                  tma_load_3d(Bsm + s * OZ_B_BYTES, &mapB, &full_bar[s], kc * OZ_KC, bb * OZ_NB,
                              ((j - 1) * P.site_dim + g) * P.chi_a + ab * OZ_NA);
                  ++si;
                }
            }
      if (!ok) atomicOr(P.err, ERR_TIMEOUT);
      // the copies still in flight land before the CTA exits
      for (int s = 0; s < OZ_STAGES; ++s)
        if (si > (uint32_t)s) mbar_wait(&full_bar[s], ((si - 1 - s) / OZ_STAGES) & 1, lim);
    }
  } else {
    // ------------------------------------------------------------ MMA ----
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16(OZ_M, OZ_N);
      bool ok = true;
      uint32_t si = 0, u = 0;
      for (int ph = 0; ph < NPH && ok; ++ph) {
        if (!mbar_wait(&a_ready, ph & 1, lim)) {
          ok = false;
          break;
        }
        tc_fence_after();
        for (int ab = 0; ab < nab && ok; ++ab)
          for (int bb = 0; bb < nbb && ok; ++bb)
            for (int gi = 0; gi < oz_ngroups(ph, PP) && ok; ++gi) {
              const int k = oz_group(ph, gi, PP);
              const int buf = u & 1;
              if (u >= 2 && !mbar_wait(&tempty[buf], ((u >> 1) - 1) & 1, lim)) {
                ok = false;
                break;
              }
              tc_fence_after();
              const uint32_t dcol = tmem + (uint32_t)(buf * OZ_N);
              uint32_t accum = 0;
              const int ilo = max(ph * PP + 1, k - OZ_DIG), ihi = min(ph * PP + PP, k - 1);
              for (int i = ilo; i <= ihi && ok; ++i)
                for (int kc = 0; kc < KCH; ++kc) {
                  const int s = si % OZ_STAGES;
                  const uint32_t use = si / OZ_STAGES;
                  if (!mbar_wait(&full_bar[s], use & 1, lim)) {
                    ok = false;
                    break;
                  }
                  tc_fence_after();
                  const uint64_t da =
                      sw128_desc(Asm + ((i - 1 - ph * PP) * KCH + kc) * OZ_SLOT_BYTES);
                  const uint64_t db = sw128_desc(Bsm + s * OZ_B_BYTES);
#pragma unroll
                  for (int k16 = 0; k16 < OZ_KC / 16; ++k16) {
                    const uint64_t adv = (uint64_t)(k16 * 32) >> 4;  // 16 BF16 along K
                    mma_bf16(dcol, da + adv, db + adv, idesc, accum);
                    accum = 1;
                  }
                  mma_commit(&empty_bar[s]);
                  ++si;
                }
              if (ok) mma_commit(&tfull[buf]);
              ++u;
            }
      }
      if (!ok) atomicOr(P.err, ERR_TIMEOUT);
      mma_commit(&mma_done);  // every MMA issued above has completed when this arrives
      mbar_wait(&mma_done, 0, lim);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 8) {
    tc_fence_after();
    tmem_dealloc(tmem, 2 * OZ_N);
  }
}

// Digit planes of one vertex's tensor: slab (s, a) = T[s][a][:][:] gets the
// exponent eB = exponent of its largest entry (2^eB > |slab|), and digit j of
// entry x is the j-th signed base-256 digit of x 2^-eB (exact in FP64).
// Planes are [6][S][chi_a][chi1][chi2] BF16.
template <class T>
__global__ void k_oz_split(const T* __restrict__ src, __nv_bfloat16* __restrict__ planes,
                           int* __restrict__ bexp, int chi_a, int64_t slab, int64_t plane) {
  const int a = blockIdx.x, s = blockIdx.y;
  const int64_t base = ((int64_t)s * chi_a + a) * slab;
  __shared__ double red[32];
  double mx = 0.0;
  for (int64_t i = threadIdx.x; i < slab; i += blockDim.x) mx = fmax(mx, fabs((double)src[base + i]));
  for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) {
    mx = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (threadIdx.x == 0) red[0] = mx;
  }
  __syncthreads();
  mx = red[0];
  int e = 0;
  if (mx > 0.0) frexp(mx, &e);
  if (threadIdx.x == 0) bexp[(int64_t)s * chi_a + a] = e;
  const double sc = ldexp(1.0, -e);
  for (int64_t i = threadIdx.x; i < slab; i += blockDim.x) {
    double r = (double)src[base + i] * sc;
#pragma unroll
    for (int j = 0; j < OZ_DIG; ++j) {
      r *= 256.0;
      const double d = rint(r);
      r -= d;
      planes[(int64_t)j * plane + base + i] = __float2bfloat16_rn((float)d);
    }
  }
}

__global__ void k_f32_to_f64(const float* __restrict__ src, double* __restrict__ dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}

// Element offsets of every eligible vertex's digit planes (padded to 64
// elements, so that each plane base stays 128-byte aligned) and of its
// exponents; -1 for the other vertices.
struct OzLayout {
  std::vector<int64_t> doff, eoff;
  int64_t nplanes = 0, nexp = 0;
};

OzLayout oz_layout(const Topo& T) {
  OzLayout L;
  L.doff.assign(T.V, -1);
  L.eoff.assign(T.V, -1);
  for (int v = 0; v < T.V; ++v) {
    const int nc = (int)T.children[v].size();
    if (nc != 2) continue;
    const int cd[2] = {T.link[T.children[v][0]], T.link[T.children[v][1]]};
    if (!oz_vertex_eligible(nc, cd, T.link[v])) continue;
    L.doff[v] = L.nplanes;
    L.nplanes += ((OZ_DIG * T.size(v) + 63) / 64) * 64;
    L.eoff[v] = L.nexp;
    L.nexp += (int64_t)T.site_dim[v] * T.link[v];
  }
  return L;
}

template <int KCH>
void launch_oz(tnfa_ctx* ctx, const CUtensorMap& map, const OzParams& p, unsigned grid) {
  TNFA_CUDA(cudaFuncSetAttribute(k_contract_oz<KCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 OZ_SMEM));
  k_contract_oz<KCH><<<grid, OZ_THREADS, OZ_SMEM, ctx->stream>>>(map, p);
  TNFA_LAUNCH_CHECK();
}

}  // namespace

bool oz_vertex_eligible(int nchild, const int* cd, int chi_a) {
  if (nchild != 2) return false;
  if (cd[1] != 64 && cd[1] != 128) return false;
  if (cd[0] < OZ_NB || cd[0] % OZ_NB != 0 || cd[0] > 4096) return false;
  return chi_a >= OZ_NA && chi_a % OZ_NA == 0 && chi_a <= 4096;
}

int oz_tile_rows() { return OZ_M; }

void oz_prepare_net(tnfa_ctx* ctx, const tnfa_net* net) {
  if (net->d_oz) return;
  const Topo& T = net->topo;
  TNFA_CHECK(net->dtype == TNFA_F64 || net->dtype == TNFA_F32, TNFA_ERR_DTYPE,
             "sliced tensor-core evaluation needs a real network");
  if (net->dtype == TNFA_F32 && !net->d_f64) {
    net->d_f64 = dalloc(ctx, (size_t)T.n_elem * 8);
    k_f32_to_f64<<<grid_for(T.n_elem, 256, 8192), 256, 0, ctx->stream>>>(
        (const float*)net->d, (double*)net->d_f64, T.n_elem);
    TNFA_LAUNCH_CHECK();
  }
  const OzLayout L = oz_layout(T);
  net->d_oz = dalloc(ctx, (size_t)std::max<int64_t>(L.nplanes, 64) * 2);
  net->d_ozexp = (int*)dalloc(ctx, (size_t)std::max<int64_t>(L.nexp, 1) * 4);
  for (int v = 0; v < T.V; ++v) {
    if (L.doff[v] < 0) continue;
    const int chi_a = T.link[v];
    const int64_t slab = (int64_t)T.link[T.children[v][0]] * T.link[T.children[v][1]];
    __nv_bfloat16* planes = (__nv_bfloat16*)net->d_oz + L.doff[v];
    int* be = net->d_ozexp + L.eoff[v];
    dim3 grid((unsigned)chi_a, (unsigned)T.site_dim[v]);
    if (net->dtype == TNFA_F64)
      k_oz_split<double><<<grid, 256, 0, ctx->stream>>>((const double*)net->d + T.off[v], planes, be,
                                                       chi_a, slab, T.size(v));
    else
      k_oz_split<float><<<grid, 256, 0, ctx->stream>>>((const float*)net->d + T.off[v], planes, be,
                                                      chi_a, slab, T.size(v));
    TNFA_LAUNCH_CHECK();
  }
  TNFA_CUDA(cudaStreamSynchronize(ctx->stream));
}

void oz_contract_vertex(tnfa_ctx* ctx, const tnfa_net* net, int v, const VertexJob<double>& j,
                        int tile_rows, int* err) {
  TNFA_CHECK(tile_rows == OZ_M, TNFA_ERR_INVALID_ARGUMENT, "tile rows mismatch");
  TNFA_CHECK(net->d_oz != nullptr, TNFA_ERR_INVALID_ARGUMENT, "digit planes not prepared");
  const Topo& T = net->topo;
  const OzLayout L = oz_layout(T);
  TNFA_CHECK(L.doff[v] >= 0 && j.nchild == 2, TNFA_ERR_UNSUPPORTED,
             "vertex shape outside the sliced tensor-core kernel");
  const int chi1 = j.ch[0].dim, chi2 = j.ch[1].dim;
  const __nv_bfloat16* planes = (const __nv_bfloat16*)net->d_oz + L.doff[v];
  const CUtensorMap map =
      tc_make_map3(planes, chi2, chi1, (int64_t)OZ_DIG * j.site_dim * j.chi_a, OZ_NB, OZ_NA);
  OzParams p{};
  p.m1_ptr = j.ch[0].ptr;
  p.m1_exp = j.ch[0].exps;
  p.m1_S = j.ch[0].S;
  p.m2_ptr = j.ch[1].ptr;
  p.m2_exp = j.ch[1].exps;
  p.m2_S = j.ch[1].S;
  p.chi_a = j.chi_a;
  p.chi1 = chi1;
  p.site_dim = j.site_dim;
  p.bexp = net->d_ozexp + L.eoff[v];
  p.out = j.out;
  p.out_exp = j.out_exp;
  p.perm = j.perm;
  p.grp_off = j.grp_off;
  p.grp_cnt = j.grp_cnt;
  p.tile_start = j.tile_start;
  p.ngroups = j.ngroups;
  p.err = err;
  p.wait_limit = ctx->tc_wait_limit;
  p.drop_arrive = ctx->tc_drop_arrive;
  const unsigned grid = (unsigned)((j.Pc + OZ_M - 1) / OZ_M + j.ngroups);
  // 26 digit-pair passes per product (the algorithmic count is one)
  KernelScope ks(ctx, "contract_oz", 2.0 * j.Pc * (double)j.K * j.chi_a,
                 8.0 * ((double)j.Pc * (chi1 + chi2 + j.chi_a)) +
                     2.0 * OZ_DIG * j.site_dim * (double)j.chi_a * j.K);
  if (chi2 == 128) launch_oz<2>(ctx, map, p, grid);
  else launch_oz<1>(ctx, map, p, grid);
}

}  // namespace tnfa
