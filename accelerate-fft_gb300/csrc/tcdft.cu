// Split-FP16 dense DFT of contiguous rows on the 5th-generation tensor cores.
//
// For a row x of length n (Complex Float) let h = ceil(n/2) - 1 index pairs
// (j, n-j), 1 <= j <= h, and P = floor(n/2) + 1.  With C[p][k] =
// cos(2*pi*p*k/n), S[p][k] = sin(2*pi*p*k/n) and the folded row
//   p = 0:             a = Re x_0, c = Im x_0, b = d = 0
//   1 <= p <= h:       a = Re(x_p + x_{n-p}), b = Re(x_p - x_{n-p}),
//                      c = Im(x_p + x_{n-p}), d = Im(x_p - x_{n-p})
//   p = n/2 (n even):  a = Re x_p, c = Im x_p, b = d = 0
// the forward DFT X_k = sum_j x_j e^{-2 pi i jk/n} is, for 0 <= k < P,
//   Re X_k = (aC)_k + (dS)_k      Im X_k = (cC)_k - (bS)_k
// and for 1 <= k <= h
//   Re X_{n-k} = (aC)_k - (dS)_k  Im X_{n-k} = (cC)_k + (bS)_k
// so a batch of rows is four real GEMMs [rows x P] x [P x P] -- n^2 real
// multiply-adds per row instead of the 4n^2 of a complex DFT matrix.  This is
// the tensor-core form for lengths the Stockham kernels can only reach by
// Bluestein (primes such as 1009): one direct product replaces two padded
// transforms and the chirp and filter multiplies.
//
// Precision: every operand is split in FP16 as v = hi + lo (each row scaled by
// a power of two that puts its largest component in [2^12, 2^13), so every
// folded value stays below 2^14) and the three products hi*hi + hi*lo + lo*hi
// are accumulated in FP32 in tensor memory -- the large hi*hi term in its own
// accumulator, the two small correction terms in a second one, because the
// tensor cores' accumulation loses about a third of a unit in the last place
// per product instruction (measured: with all three in one accumulator a
// 1009-point row lost 1.9e-6 relative L2, 2047 points 3.7e-6; the error grows
// with the number of instructions per accumulator).  The scale is undone in
// the epilogue.
//
// Two kernels:
//  * tcdft_fold_kernel: one warp per row (8 rows per CTA) stages the row in
//    shared memory, finds its largest component, and writes the folded,
//    scaled, split operand tiles (8 arrays: a, b, c, d x hi, lo) in the
//    tensor cores' K-major core-matrix layout, one 32 KiB block per 128 rows
//    and 16 folded indices, plus the row's inverse scale.
//  * tcdft_mma_kernel: one CTA per (128 rows, 64 output frequencies); the
//    CTAs of up to 8 frequency chunks of one row tile form a cluster and
//    share every operand block through multicast bulk copies (each CTA
//    fetches one eighth and the copy lands in all of them), while each
//    fetches its own cos/sin block; a four-stage ring.  One thread issues
//    tcgen05.mma (M = 128, K = 16; per step and quantity one N = 128 product
//    into [main | correction] and one N = 64 product into the correction)
//    into four accumulator pairs that fill the SM's 512 TMEM columns; eight
//    epilogue warps read them back with tcgen05.ld and write X_k and X_{n-k}.
// Every wait is bounded: on timeout the kernel records GBFFT_ERR_TIMEOUT in
// the plan's status word, drains its own bulk copies, frees its tensor memory
// and returns.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "butterflies.cuh"
#include "gbfft.h"
#include "gbfft_internal.h"
#include "plan_internal.h"
#include "tma.cuh"

namespace gbfft {
namespace {

constexpr int kM = 128;                         // rows per tile = TMEM lanes
constexpr int kKc = 16;                         // folded indices per K chunk (one MMA step)
constexpr int kNc = 64;                         // output frequencies per CTA
constexpr uint32_t kTile = kM * kKc * 2;        // one [128 x 16] FP16 tile: 4 KiB
constexpr uint32_t kABlk = 8 * kTile;           // a, b, c, d x hi, lo: 32 KiB
constexpr uint32_t kBBlk = 2 * kTile;           // [C_hi; C_lo], [S_hi; S_lo]: 8 KiB
constexpr uint32_t kStage = kABlk + kBBlk;      // 40 KiB
constexpr int kStages = 4;
constexpr int kFoldRows = 8;                    // rows (warps) per fold CTA
constexpr int kMmaThreads = 320;                // producer, MMA, 8 epilogue warps
constexpr int kMaxCluster = 4;                  // CTAs (frequency chunks) sharing operand blocks

// byte offset of element (m, k) in a [rows x 16] K-major tile of core
// matrices (8 rows x 16 bytes each, no swizzle): LBO 128 B along K, SBO
// 256 B along M
__host__ __device__ __forceinline__ uint32_t cm_off(int m, int k) {
  return uint32_t((m >> 3) * 256 + (k >> 3) * 128 + (m & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: start, LBO 128 B, SBO 256 B, version 1,
// no swizzle
__device__ __forceinline__ uint64_t mat_desc(uint32_t saddr) {
  return uint64_t((saddr >> 4) & 0x3FFF) | (uint64_t(128 >> 4) << 16) | (uint64_t(256 >> 4) << 32) |
         (uint64_t(1) << 46);
}
// instruction descriptors, kind::f16: D f32, A = B = f16, both K-major, M = 128, N = 128 / 64
constexpr uint32_t kIdesc128 = (1u << 4) | ((128u >> 3) << 17) | ((uint32_t(kM) >> 4) << 24);
constexpr uint32_t kIdesc64 = (1u << 4) | ((64u >> 3) << 17) | ((uint32_t(kM) >> 4) << 24);

// padded shared-memory index of element j of a staged row: one gap every
// 8 elements keeps the fold's stride-8 reads free of bank conflicts
__device__ __forceinline__ int pidx(int j) { return j + (j >> 3); }

// a = hi.x + lo.x, b = hi.y + lo.y in FP16 pairs (a in the low half), both
// rounded to nearest: one pair conversion each way instead of four scalar ones
__device__ __forceinline__ void split_pair(float a, float b, uint32_t& hi, uint32_t& lo) {
  const __half2 h = __floats2half2_rn(a, b);
  const float2 hf = __half22float2(h);
  const __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
  hi = *reinterpret_cast<const uint32_t*>(&h);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}

// ---- step 1: fold, scale and split ------------------------------------------
// d.in: rows (row stride in_cs elements); d.out: operand blocks of the
// scratch, then one float per padded row (its inverse scale); d.ncols rows;
// rows beyond d.ncols up to the tile boundary get zero operands.
__global__ void __launch_bounds__(kFoldRows * 32) tcdft_fold_kernel(const PassDesc d) {
  extern __shared__ __align__(16) float2 srow_all[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n = d.n, P = d.tc_p, KC = d.tc_kc;
  const int h = (n - 1) / 2;  // index pairs (j, n-j)
  const int64_t r = int64_t(blockIdx.x) * kFoldRows + warp;
  const bool live = r < d.ncols;
  float2* sr = srow_all + size_t(warp) * size_t(pidx(n) + 1);
  const float2* __restrict__ in = static_cast<const float2*>(d.in) + (live ? r * d.in_cs : 0);
  const bool conj = (d.flags & F_CONJ_IN) != 0;
  float mx = 0.f;
  // 16 loads in flight per lane before any use
  for (int j0 = 0; j0 < n; j0 += 32 * 16) {
    float2 xs[16];
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int j = j0 + lane + 32 * u;
      xs[u] = (live && j < n) ? in[j] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      const int j = j0 + lane + 32 * u;
      float2 x = xs[u];
      if (conj) x.y = -x.y;
      if (j < n) sr[pidx(j)] = x;
      mx = fmaxf(mx, fmaxf(fabsf(x.x), fabsf(x.y)));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  __syncwarp();
  // power-of-two scale: max |x| * s in [2^12, 2^13), so every folded value
  // (a sum of two components) stays below 2^14
  int sh = 0;
  if (mx > 0.f) {
    int e;
    frexpf(mx, &e);  // mx = f * 2^e, f in [0.5, 1)
    sh = max(-126, min(126, 13 - e));
  }
  const float s = ldexpf(1.f, sh);
  unsigned char* A = static_cast<unsigned char*>(d.out);
  const int64_t mt = r / kM;
  const int m = int(r % kM);
  // item = (K chunk, group of 8 folded indices): 8 arrays x 16 bytes
  for (int it = lane; it < KC * 2; it += 32) {
    const int kc = it >> 1, g = it & 1;
    uint32_t w[8][4];
#pragma unroll
    for (int q = 0; q < 8; q += 2) {
      float v[2][4];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int p = kc * kKc + g * 8 + q + u;
        float a = 0.f, b = 0.f, c = 0.f, dd = 0.f;
        if (p == 0 || (p < P && p > h)) {  // unpaired: x_0, and x_{n/2} for even n
          const float2 x = sr[pidx(p)];
          a = x.x * s;
          c = x.y * s;
        } else if (p <= h) {
          const float2 x1 = sr[pidx(p)], x2 = sr[pidx(n - p)];
          const float r1 = x1.x * s, r2 = x2.x * s, i1 = x1.y * s, i2 = x2.y * s;
          a = r1 + r2;
          b = r1 - r2;
          c = i1 + i2;
          dd = i1 - i2;
        }
        v[u][0] = a;
        v[u][1] = b;
        v[u][2] = c;
        v[u][3] = dd;
      }
#pragma unroll
      for (int t = 0; t < 4; ++t) split_pair(v[0][t], v[1][t], w[2 * t][q >> 1], w[2 * t + 1][q >> 1]);
    }
    unsigned char* blk = A + (size_t(mt) * size_t(KC) + size_t(kc)) * kABlk + cm_off(m, g * 8);
#pragma unroll
    for (int t = 0; t < 8; ++t)
      *reinterpret_cast<uint4*>(blk + size_t(t) * kTile) = make_uint4(w[t][0], w[t][1], w[t][2], w[t][3]);
  }
  if (lane == 0) {
    const int64_t mtiles = (d.ncols + kM - 1) / kM;
    float* rowinfo = reinterpret_cast<float*>(A + size_t(mtiles) * size_t(KC) * kABlk);
    rowinfo[r] = ldexpf(1.f, -sh);
  }
}

// ---- step 2: the four GEMMs and the output combination -------------------------
__device__ __forceinline__ void mma_f16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(da), "l"(db), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
// arrive on the barrier at this offset in every CTA of `mask` once the
// products issued so far have completed
__device__ __forceinline__ void mma_commit_mc(uint64_t* bar, uint16_t mask) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
          smem_u32(bar)),
      "h"(mask)
      : "memory");
}
// bulk copy delivered to the same shared-memory offset of every CTA of
// `mask`, completing on the barrier at the same offset in each
__device__ __forceinline__ void tma_load_1d_mc(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                               uint16_t mask) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.multicast::cluster [%0], [%1], %2, [%3], "
      "%4;" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar)), "h"(mask)
      : "memory");
}
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
#define GBFFT_LD8(r, addr)                                                                   \
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"      \
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), \
                 "=r"(r[7])                                                                  \
               : "r"(addr)                                                                   \
               : "memory")


// d.in: the operand blocks written by the fold (then the inverse scales);
// d.tw: cos/sin blocks [NCp][KC] of 8 KiB; d.out: output rows (row stride
// out_cs); d.ncols rows; d.tc_nc = NCp (frequency chunks, padded to a
// multiple of the cluster size).  Grid (row tiles, NCp); a cluster is CS
// consecutive frequency chunks of one row tile, CS = d.W.
//
// Per K chunk of 16 folded indices the four quantities' products are
//   D_q[0:128)  += A_hi(q) x [B_hi(q); B_lo(q)]   (N = 128: main | correction)
//   D_q[64:128) += A_lo(q) x  B_hi(q)             (N = 64: correction)
// so the large main accumulator takes one rounding per K step; the two
// correction products (2^-11 of it) share the second half.  Accumulators at
// columns 128q (q = aC, dS, cC, bS) fill the 512 TMEM columns.
__global__ void __launch_bounds__(kMmaThreads, 1) tcdft_mma_kernel(const PassDesc d) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages], accf;
  __shared__ uint32_t s_tbase;
  __shared__ int s_fail, s_issued, s_consumed;
  // the ring starts on a 1 KiB boundary of the shared window (the launch
  // requests 1 KiB more than the ring); the offset is the same in every CTA
  // of the cluster, as multicast copies require
  unsigned char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int KC = d.tc_kc, P = d.tc_p, n = d.n, CS = d.W;
  const int64_t mt = blockIdx.x;
  const int nc = int(blockIdx.y);
  const uint32_t crank = cluster_rank();
  const uint16_t cmask = uint16_t((1u << CS) - 1u);
  const unsigned char* A = static_cast<const unsigned char*>(d.in) + size_t(mt) * size_t(KC) * kABlk;
  const unsigned char* Bm = static_cast<const unsigned char*>(d.tw) + size_t(nc) * size_t(KC) * kBBlk;
  if (threadIdx.x == 0) {
    s_fail = 0;
    s_issued = 0;
    s_consumed = 0;
    for (int i = 0; i < kStages; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], uint32_t(CS));  // one arrival per CTA of the cluster
    }
    mbar_init(&accf, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&s_tbase))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  // every CTA's barriers exist before any multicast copy or arrival lands
  cluster_sync_all();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = s_tbase;

  if (warp == 0) {
    if (lane == 0) {
      // producer: operand tiles t = crank, crank + CS, ... of each chunk go to
      // every CTA of the cluster; this CTA's own cos/sin block to itself.
      // Chunks in a rotated order per row tile (spreads the reads of the
      // shared cos/sin blocks over time).
      const int k0 = int(mt % KC);
      int kc = 0;
      for (; kc < KC; ++kc) {
        const int st = kc % kStages;
        if (kc >= kStages &&
            !mbar_wait_bounded(&empty[st], uint32_t(kc / kStages - 1) & 1u, d.status)) {
          atomicExch(&s_fail, 1);
          break;
        }
        const int kk = (kc + k0) % KC;
        unsigned char* dst = smem + st * kStage;
        mbar_expect_tx(&full[st], kStage);
        for (int t = int(crank); t < 8; t += CS)
          tma_load_1d_mc(dst + t * kTile, A + size_t(kk) * kABlk + size_t(t) * kTile, kTile, &full[st], cmask);
        tma_load_1d(dst + kABlk, Bm + size_t(kk) * kBBlk, kBBlk, &full[st]);
      }
      s_issued = kc;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const int ta[4] = {0, 6, 4, 2};  // hi tile of a, d, c, b (lo = +1)
      const int tb[4] = {0, 1, 0, 1};  // [C_hi; C_lo], [S_hi; S_lo], ...
      int kc = 0;
      for (; kc < KC; ++kc) {
        const int st = kc % kStages;
        if (!mbar_wait_bounded(&full[st], uint32_t(kc / kStages) & 1u, d.status)) {
          atomicExch(&s_fail, 1);
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t sa = smem_u32(smem + st * kStage), sb = sa + kABlk;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const uint32_t acc = tmem + uint32_t(q * 128);
          const uint64_t ah = mat_desc(sa + ta[q] * kTile), al = mat_desc(sa + (ta[q] + 1) * kTile);
          const uint64_t bb = mat_desc(sb + tb[q] * kTile);
          mma_f16(acc, ah, bb, kIdesc128, kc ? 1u : 0u);
          mma_f16(acc + 64, al, bb, kIdesc64, 1u);
        }
        // the stage is free in every CTA once all CTAs' products have read it
        mma_commit_mc(&empty[st], cmask);
      }
      s_consumed = kc;
      mma_commit(&accf);  // arrives when every product issued above has completed
    }
  } else {
    // epilogue: warp w reads TMEM lanes 32*(w % 4) .. +31; warps 2..5 take
    // frequency columns 0..31 of the chunk, warps 6..9 columns 32..63
    bool ok = mbar_wait_bounded(&accf, 0u, d.status);
    ok = ok && s_fail == 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int quarter = warp & 3;
    const int m = quarter * 32 + lane;
    const int64_t row = mt * kM + m;
    const int64_t mtiles = (d.ncols + kM - 1) / kM;
    const float* rowinfo = reinterpret_cast<const float*>(static_cast<const unsigned char*>(d.in) +
                                                          size_t(mtiles) * size_t(KC) * kABlk);
    const bool live = ok && row < d.ncols;
    const float inv = live ? rowinfo[row] * ((d.flags & F_SCALE) ? float(d.scale) : 1.f) : 0.f;
    const float sgn = (d.flags & F_CONJ_OUT) ? -1.f : 1.f;
    const int h = (n - 1) / 2;
    float2* __restrict__ out = static_cast<float2*>(d.out) + (live ? row * d.out_cs : 0);
    const int c0 = (warp < 6) ? 0 : 32;
    const uint32_t lane_base = tmem + (uint32_t(quarter * 32) << 16);
    for (int cc = c0; cc < c0 + 32; cc += 8) {
      // main and correction halves of the four accumulators
      uint32_t r0[8], r1[8], r2[8], r3[8], e0[8], e1[8], e2[8], e3[8];
      GBFFT_LD8(r0, lane_base + uint32_t(0 * 128 + cc));
      GBFFT_LD8(e0, lane_base + uint32_t(0 * 128 + 64 + cc));
      GBFFT_LD8(r1, lane_base + uint32_t(1 * 128 + cc));
      GBFFT_LD8(e1, lane_base + uint32_t(1 * 128 + 64 + cc));
      GBFFT_LD8(r2, lane_base + uint32_t(2 * 128 + cc));
      GBFFT_LD8(e2, lane_base + uint32_t(2 * 128 + 64 + cc));
      GBFFT_LD8(r3, lane_base + uint32_t(3 * 128 + cc));
      GBFFT_LD8(e3, lane_base + uint32_t(3 * 128 + 64 + cc));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (!live) continue;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const int k = nc * kNc + cc + c;
        if (k >= P) break;
        const float u = __uint_as_float(r0[c]) + __uint_as_float(e0[c]);   // aC
        const float v = __uint_as_float(r1[c]) + __uint_as_float(e1[c]);   // dS
        const float w = __uint_as_float(r2[c]) + __uint_as_float(e2[c]);   // cC
        const float z = __uint_as_float(r3[c]) + __uint_as_float(e3[c]);   // bS
        out[k] = make_float2((u + v) * inv, sgn * (w - z) * inv);
        if (k >= 1 && k <= h) out[n - k] = make_float2((u - v) * inv, sgn * (w + z) * inv);
      }
    }
  }
  // every tensor-memory read above, and every product, has completed; drain
  // bulk copies that were issued but never consumed (a timeout path only)
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int kc = s_consumed; kc < s_issued; ++kc)
      mbar_wait_bounded(&full[kc % kStages], uint32_t(kc / kStages) & 1u, d.status);
  }
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
  // no CTA leaves while another may still deliver copies or arrivals to it
  cluster_sync_all();
}

size_t fold_smem(int n) { return size_t(kFoldRows) * size_t(n + (n >> 3) + 2) * sizeof(float2); }

// ---- fused two-stage form: n = 8 * n2, n2 odd, (n2 + 1) / 2 <= 64 ----------
// j = n2*j1 + j2, k = k1 + 8*k2.  A radix-8 DFT over j1 and the twiddle
// W_n^(j2*k1) run on the CUDA cores; the DFT over j2 for each (row, k1) runs
// on the tensor cores in the folded form above (P2 = (n2 + 1) / 2 folded
// indices, h2 = P2 - 1 pairs).  One persistent CTA of 16 warps works on tiles
// of 16 rows: GEMM row m = 8*r + k1 (128 TMEM lanes), K = folded j2 index
// (two halves of 32), N = k2 (64 columns, four accumulators = 256 TMEM
// columns, so two CTAs share an SM).  Per tile:
//   1. warp r reads row r once, coalesced, for its largest component (the
//      row's power-of-two scale puts it in [2^9, 2^10); the radix-8 stage,
//      the twiddle and the fold grow a component at most 16*sqrt(2)-fold, so
//      every folded value stays below 2^15);
//   2. per K half, lane p loads x[n2*j1 + j2] for j2 = p and n2 - p (L2 hits),
//      runs the two radix-8 DFTs and twiddles, folds, splits hi/lo and stores
//      one 16-byte vector per operand array: the 8 values k1 = 0..7 of GEMM
//      rows 8r..8r+7, i.e. the operand is stored MN-major;
//   3. one thread issues the 24 products of the half (M = 128, N = 64,
//      K = 16) and commits; the CTA waits before the next half reuses the
//      operand buffer;
//   4. all 16 warps read the accumulators back (warp w: lanes of quarter
//      w % 4, 16 of the 64 columns) and store X[k1 + 8*k2] and
//      X[k1 + 8*(n2 - k2)]: eight consecutive k1 form a 64-byte segment.
constexpr int kS_Rows = 16;
constexpr int kS_Threads = 512;
constexpr uint32_t kS_ATile = 128 * 32 * 2;          // [128 m x 32 K] f16: 8 KiB
constexpr uint32_t kS_BTile = 64 * 32 * 2;           // [64 k2 x 32 K] f16: 4 KiB
constexpr uint32_t kS_BBytes = 2 * 4 * kS_BTile;     // K halves x (C, S) x (hi, lo): 32 KiB
constexpr uint32_t kS_Smem = 8 * kS_ATile + kS_BBytes + 1024 * 8;  // + W_n table (n <= 1024)
// MN-major operand tiles: core matrix = 8 K rows x 16 bytes (8 consecutive
// m); consecutive K groups 128 B apart, consecutive m groups 512 B apart
constexpr uint32_t kS_AKStride = 128, kS_AMStride = 512;
constexpr uint32_t kS_ALbo = kS_AKStride, kS_ASbo = kS_AMStride;
// instruction descriptor: D f32, A = B = f16, A MN-major (bit 15), B K-major, N = 64, M = 128
constexpr uint32_t kS_Idesc = (1u << 4) | (1u << 15) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ uint64_t mat_desc2(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return uint64_t((saddr >> 4) & 0x3FFF) | (uint64_t(lbo >> 4) << 16) | (uint64_t(sbo >> 4) << 32) |
         (uint64_t(1) << 46);
}
__device__ __forceinline__ void mma_f16_s(uint32_t tmem, uint64_t da, uint64_t db, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(da), "l"(db), "r"(kS_Idesc), "r"(acc)
      : "memory");
}

// d.tw: B tiles (kS_BBytes) followed by W_n^(j2*k1) at (k1 - 1)*n2 + j2 (Complex Float);
// d.tc_nc = n2, d.tc_p = P2; rows d.ncols, strides in_cs / out_cs.
__global__ void __launch_bounds__(kS_Threads, 2) tcdft8_kernel(const PassDesc d) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t s_tbase;
  __shared__ float s_inv[kS_Rows];
  unsigned char* sm = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  unsigned char* As = sm;
  unsigned char* Bs = sm + 8 * kS_ATile;
  float2* Ws = reinterpret_cast<float2*>(Bs + kS_BBytes);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int n = d.n, n2 = d.tc_nc, P2 = d.tc_p, h2 = P2 - 1;
  {
    const uint4* src = static_cast<const uint4*>(d.tw);
    uint4* dst = reinterpret_cast<uint4*>(Bs);
    const int words = int((kS_BBytes + uint32_t(n) * 8u + 15u) / 16u);
    for (int i = tid; i < words; i += kS_Threads) dst[i] = src[i];
  }
  if (tid == 0) {
    mbar_init(&mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(&s_tbase))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_async_smem();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = s_tbase;
  const bool conj_in = (d.flags & F_CONJ_IN) != 0;
  const float osc = (d.flags & F_SCALE) ? float(d.scale) : 1.f;
  const float sgn = (d.flags & F_CONJ_OUT) ? -1.f : 1.f;
  const int64_t tiles = (d.ncols + kS_Rows - 1) / kS_Rows;
  const bool vec_rows = ((reinterpret_cast<uintptr_t>(d.in) & 15) == 0) && (d.in_cs % 2 == 0);
  uint32_t phase = 0;
  bool fail = false;
  for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int64_t row = tile * kS_Rows + warp;
    const bool live = row < d.ncols;
    const float2* __restrict__ in = static_cast<const float2*>(d.in) + (live ? row * d.in_cs : 0);
    // 1. the row's largest component
    float mx = 0.f;
    if (live && vec_rows) {
      // pairs of elements as 16-byte loads (n is even, rows 16-byte aligned)
      const float4* in4 = reinterpret_cast<const float4*>(in);
      for (int j0 = 0; j0 < n / 2; j0 += 32 * 16) {
        float4 xs[16];  // 16 loads in flight per lane before any use
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int j = j0 + lane + 32 * u;
          xs[u] = j < n / 2 ? in4[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 16; ++u)
          mx = fmaxf(mx, fmaxf(fmaxf(fabsf(xs[u].x), fabsf(xs[u].y)), fmaxf(fabsf(xs[u].z), fabsf(xs[u].w))));
      }
    } else if (live) {
      for (int j0 = 0; j0 < n; j0 += 32 * 16) {
        float2 xs[16];  // 16 loads in flight per lane before any use
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int j = j0 + lane + 32 * u;
          xs[u] = j < n ? in[j] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 16; ++u) mx = fmaxf(mx, fmaxf(fabsf(xs[u].x), fabsf(xs[u].y)));
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    int sh = 0;
    if (mx > 0.f) {
      int e;
      frexpf(mx, &e);  // mx in [2^(e-1), 2^e): mx * s in [2^9, 2^10)
      sh = max(-126, min(126, 10 - e));
    }
    const float s = ldexpf(1.f, sh);
    if (lane == 0) s_inv[warp] = ldexpf(1.f, -sh);
    for (int hh = 0; hh < 2; ++hh) {
      // 2. folded index p = 32*hh + lane: j2 = p (and n2 - p when paired)
      const int p = hh * 32 + lane;
      const bool pair = p >= 1 && p <= h2;
      const bool one = p == 0 || pair;
      float2 z0[8], z1[8];
#pragma unroll
      for (int j1 = 0; j1 < 8; ++j1) {
        z0[j1] = (live && one) ? in[n2 * j1 + p] : make_float2(0.f, 0.f);
        z1[j1] = (live && pair) ? in[n2 * j1 + n2 - p] : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int j1 = 0; j1 < 8; ++j1) {
        if (conj_in) {
          z0[j1].y = -z0[j1].y;
          z1[j1].y = -z1[j1].y;
        }
        z0[j1] = make_float2(z0[j1].x * s, z0[j1].y * s);
        z1[j1] = make_float2(z1[j1].x * s, z1[j1].y * s);
      }
      dft8(z0);
      dft8(z1);
      // twiddle W_n^(j2*k1) from the table [k1 - 1][j2] (consecutive lanes,
      // consecutive entries)
      {
        const int ja = one ? p : 0, jb = pair ? n2 - p : 0;
#pragma unroll
        for (int k1 = 1; k1 < 8; ++k1) {
          z0[k1] = cmul(z0[k1], Ws[(k1 - 1) * n2 + ja]);
          z1[k1] = cmul(z1[k1], Ws[(k1 - 1) * n2 + jb]);
        }
      }
      // fold, split, store: quantity q = a, b, c, d; arrays 2q (hi) and 2q + 1
      // (lo), one 16-byte vector of the 8 values k1 = 0..7 each.  An unpaired
      // index (p = 0) has no odd part: b = d = 0.
      {
        unsigned char* dst = As + uint32_t(warp) * kS_AMStride + uint32_t(lane >> 3) * kS_AKStride +
                             uint32_t(lane & 7) * 16u;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          uint32_t hi[4], lo[4];
#pragma unroll
          for (int k1 = 0; k1 < 8; k1 += 2) {
            float v[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
              const float2 x1 = z0[k1 + u], x2 = z1[k1 + u];  // z1 is zero when unpaired
              const float f = (q == 0) ? x1.x + x2.x : (q == 1) ? x1.x - x2.x : (q == 2) ? x1.y + x2.y : x1.y - x2.y;
              v[u] = ((q & 1) && !pair) ? 0.f : f;
            }
            split_pair(v[0], v[1], hi[k1 >> 1], lo[k1 >> 1]);
          }
          *reinterpret_cast<uint4*>(dst + (2 * q) * kS_ATile) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
          *reinterpret_cast<uint4*>(dst + (2 * q + 1) * kS_ATile) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
        }
      }
      fence_async_smem();
      __syncthreads();
      // 3. the half's products: accumulators aC | dS | cC | bS at columns 0 | 64 | 128 | 192
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int ta[4] = {0, 6, 4, 2};
        const int tb[4] = {0, 2, 0, 2};
        const uint32_t sa = smem_u32(As), sb = smem_u32(Bs) + uint32_t(hh) * 4u * kS_BTile;
#pragma unroll
        for (int ks = 0; ks < 2; ++ks)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const uint32_t acc = tmem + uint32_t(q * 64);
            const uint64_t ah = mat_desc2(sa + ta[q] * kS_ATile + ks * 2 * kS_AKStride, kS_ALbo, kS_ASbo);
            const uint64_t al = mat_desc2(sa + (ta[q] + 1) * kS_ATile + ks * 2 * kS_AKStride, kS_ALbo, kS_ASbo);
            const uint64_t bh = mat_desc2(sb + tb[q] * kS_BTile + ks * 256, 128, 512);
            const uint64_t bl = mat_desc2(sb + (tb[q] + 1) * kS_BTile + ks * 256, 128, 512);
            mma_f16_s(acc, ah, bh, (hh | ks) ? 1u : 0u);
            mma_f16_s(acc, ah, bl, 1u);
            mma_f16_s(acc, al, bh, 1u);
          }
        mma_commit(&mbar);
      }
      const bool timed_out = !mbar_wait_bounded(&mbar, phase, d.status);
      phase ^= 1u;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (__syncthreads_or(timed_out)) {  // a uniform decision across the CTA
        fail = true;
        break;
      }
    }
    if (fail) break;
    // 4. epilogue, 8 columns at a time (register budget of two CTAs per SM)
    {
      const int quarter = warp & 3, cg = warp >> 2;
      const int m = quarter * 32 + lane;
      const int r = m >> 3, k1 = m & 7;
      const int64_t orow = tile * kS_Rows + r;
      const bool live_o = orow < d.ncols;
      const float inv = s_inv[r] * osc;
      float2* __restrict__ out = static_cast<float2*>(d.out) + (live_o ? orow * d.out_cs : 0) + k1;
#pragma unroll
      for (int c0 = 0; c0 < 16; c0 += 8) {
        uint32_t rA[8], rD[8], rC[8], rB[8];
        const uint32_t base = tmem + (uint32_t(quarter * 32) << 16) + uint32_t(cg * 16 + c0);
        GBFFT_LD8(rA, base + 0);
        GBFFT_LD8(rD, base + 64);
        GBFFT_LD8(rC, base + 128);
        GBFFT_LD8(rB, base + 192);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (live_o) {
#pragma unroll
          for (int c = 0; c < 8; ++c) {
            const int k2 = cg * 16 + c0 + c;
            const float u = __uint_as_float(rA[c]), v = __uint_as_float(rD[c]);
            const float w2 = __uint_as_float(rC[c]), z = __uint_as_float(rB[c]);
            if (k2 < P2) out[8 * k2] = make_float2((u + v) * inv, sgn * (w2 - z) * inv);
            if (k2 >= 1 && k2 <= h2) out[8 * (n2 - k2)] = make_float2((u - v) * inv, sgn * (w2 + z) * inv);
          }
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();  // accumulators and s_inv are free for the next tile
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem) : "memory");
  }
}

int g_tc_sms = 0;

}  // namespace

cudaError_t prepare_tcdft_kernels() {
  cudaError_t e = cudaFuncSetAttribute(tcdft_fold_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(fold_smem(kTcDftMaxN)));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(tcdft_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           int(kStages * kStage + 1024));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(tcdft8_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kS_Smem + 1024));
  if (e != cudaSuccess) return e;
  int dev = 0;
  cudaGetDevice(&dev);
  return cudaDeviceGetAttribute(&g_tc_sms, cudaDevAttrMultiProcessorCount, dev);
}

cudaError_t launch_tcdft(const PassDesc& d, cudaStream_t s) {
  if (d.ncols <= 0) return cudaSuccess;
  if (d.kernel == K_TC_DFT8) {
    const int64_t tiles = (d.ncols + kS_Rows - 1) / kS_Rows;
    // two CTAs per SM by design (256 TMEM columns and ~105 KiB of shared
    // memory each); CTAs beyond the resident ones simply start later
    const int64_t cap = int64_t(std::max(1, g_tc_sms)) * 2;
    tcdft8_kernel<<<unsigned(std::min(tiles, cap)), kS_Threads, kS_Smem + 1024, s>>>(d);
    return cudaGetLastError();
  }
  const int64_t mtiles = (d.ncols + kM - 1) / kM;
  if (d.kernel == K_TC_FOLD) {
    const int64_t grid = mtiles * (kM / kFoldRows);
    tcdft_fold_kernel<<<unsigned(grid), kFoldRows * 32, fold_smem(d.n), s>>>(d);
  } else {
    // 1 KiB beyond the ring: room to align its start (see the kernel); a
    // cluster of d.W consecutive frequency chunks shares the operand blocks
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(mtiles), unsigned(d.tc_nc), 1);
    cfg.blockDim = dim3(kMmaThreads, 1, 1);
    cfg.dynamicSmemBytes = kStages * kStage + 1024;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 1;
    attr[0].val.clusterDim.y = unsigned(d.W);
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, tcdft_mma_kernel, d);
  }
  return cudaGetLastError();
}

// ---- host side: cos/sin operand blocks and the two passes --------------------

bool tcdft_available(int64_t n) { return n >= 3 && n <= kTcDftMaxN; }

// n = 8 * n2 with n2 odd, 3 <= n2 <= 127: the fused radix-8 + dense form
bool tcdft8_available(int64_t n) {
  if (n % 8) return false;
  const int64_t n2 = n / 8;
  return (n2 & 1) && n2 >= 3 && n2 <= 127;
}

// One pass of the fused form (no scratch): the cos/sin operand tiles of the
// odd stage and the table W_n^t go into B's blob.
int tcdft8_add_pass(Builder& B, int64_t n, int64_t rows, int64_t in_cs, int64_t out_cs, int src, int dst,
                    std::vector<PassSpec>& passes) {
  if (!tcdft8_available(n) || rows <= 0) return GBFFT_ERR_UNSUPPORTED;
  const int n2 = int(n / 8), P2 = (n2 + 1) / 2;
  std::vector<unsigned char> tb(kS_BBytes + size_t(n) * 8 + 16, 0);
  for (int k2 = 0; k2 < P2; ++k2)
    for (int p = 0; p < P2; ++p) {
      const cd w = unit_root((int64_t(p) * k2) % n2, n2);  // cos - i sin
      const double vals[2] = {w.real(), -w.imag()};
      const int hh = p / 32;
      // [64 k2 x 32 K] K-major core matrices: LBO 128 B (K), SBO 512 B (k2)
      const uint32_t off = uint32_t((k2 >> 3) * 512 + ((p % 32) >> 3) * 128 + (k2 & 7) * 16 + (p % 8) * 2);
      for (int u = 0; u < 2; ++u) {
        const __half hi = __float2half_rn(float(vals[u]));
        const __half lo = __float2half_rn(float(vals[u] - double(__half2float(hi))));
        std::memcpy(tb.data() + size_t(hh * 4 + 2 * u) * kS_BTile + off, &hi, 2);
        std::memcpy(tb.data() + size_t(hh * 4 + 2 * u + 1) * kS_BTile + off, &lo, 2);
      }
    }
  // radix-8 twiddles W_n^(j2*k1) at (k1 - 1)*n2 + j2, k1 = 1..7, j2 < n2
  // (7*n2 < n entries)
  for (int k1 = 1; k1 < 8; ++k1)
    for (int j2 = 0; j2 < n2; ++j2) {
      const cd w = unit_root((int64_t(j2) * k1) % n, n);
      const float v[2] = {float(w.real()), float(w.imag())};
      std::memcpy(tb.data() + kS_BBytes + (size_t(k1 - 1) * size_t(n2) + size_t(j2)) * 8, v, 8);
    }
  while (B.blob.size() % 256) B.blob.push_back(0);
  const size_t off = B.blob.size();
  B.blob.insert(B.blob.end(), tb.begin(), tb.end());
  PassSpec g;
  std::memset(&g.d, 0, sizeof(PassDesc));
  g.d.kernel = K_TC_DFT8;
  g.d.n = int(n);
  g.d.ncols = rows;
  g.d.nbatch = g.d.nb_lo = 1;
  g.d.scale = 1.0;
  g.d.tw4_n = 1;
  g.d.tc_p = P2;
  g.d.tc_nc = n2;
  g.d.in_cs = in_cs;
  g.d.out_cs = out_cs;
  g.src = src;
  g.dst = dst;
  g.tw_off = int64_t(off);
  g.axis_final = true;
  g.rot_ok = false;
  g.axis_n = n;
  passes.push_back(g);
  return GBFFT_OK;
}

size_t tcdft_scratch_bytes(int64_t n, int64_t rows) {
  const int64_t P = n / 2 + 1, KC = (P + kKc - 1) / kKc;  // operand blocks of 16 folded indices
  const int64_t mtiles = (rows + kM - 1) / kM;
  return size_t(mtiles) * size_t(KC) * kABlk + size_t(mtiles) * kM * sizeof(float);
}

// Appends the fold and product passes for `rows` rows of length n (row
// strides in_cs / out_cs elements) reading role src and writing role dst, the
// operand blocks in scratch role R_S1; the cos/sin blocks go into B's blob.
int tcdft_add_passes(Builder& B, int64_t n, int64_t rows, int64_t in_cs, int64_t out_cs, int src, int dst,
                     std::vector<PassSpec>& passes) {
  if (!tcdft_available(n) || rows <= 0) return GBFFT_ERR_UNSUPPORTED;
  const int P = int(n / 2 + 1);
  const int KC = (P + kKc - 1) / kKc, NC = (P + kNc - 1) / kNc;
  // frequency chunks per cluster (1, 2, 4 or 8) and chunks padded to a multiple of it
  const int CS = NC >= kMaxCluster ? kMaxCluster : NC > 2 ? 4 : NC;
  const int NCp = (NC + CS - 1) / CS * CS;
  // cos/sin blocks [NCp][KC]: tiles [C_hi; C_lo] and [S_hi; S_lo] of
  // [128 x 16]: rows 0..63 hi and 64..127 lo of the chunk's 64 frequencies
  std::vector<unsigned char> mats(size_t(NCp) * size_t(KC) * kBBlk, 0);
  for (int k = 0; k < P; ++k)
    for (int p = 0; p < P; ++p) {
      const cd w = unit_root((int64_t(p) * k) % n, n);  // cos - i sin
      const double vals[2] = {w.real(), -w.imag()};
      const int nc = k / kNc, kc = p / kKc;
      unsigned char* blk = mats.data() + (size_t(nc) * size_t(KC) + size_t(kc)) * kBBlk;
      for (int u = 0; u < 2; ++u) {
        const __half hi = __float2half_rn(float(vals[u]));
        const __half lo = __float2half_rn(float(vals[u] - double(__half2float(hi))));
        std::memcpy(blk + size_t(u) * kTile + cm_off(k % kNc, p % kKc), &hi, 2);
        std::memcpy(blk + size_t(u) * kTile + cm_off(kNc + k % kNc, p % kKc), &lo, 2);
      }
    }
  while (B.blob.size() % 256) B.blob.push_back(0);
  const size_t mat_off = B.blob.size();
  B.blob.insert(B.blob.end(), mats.begin(), mats.end());

  PassSpec f, g;
  std::memset(&f.d, 0, sizeof(PassDesc));
  std::memset(&g.d, 0, sizeof(PassDesc));
  for (PassSpec* ps : {&f, &g}) {
    ps->d.n = int(n);
    ps->d.ncols = rows;
    ps->d.nbatch = ps->d.nb_lo = 1;
    ps->d.scale = 1.0;
    ps->d.tw4_n = 1;
    ps->d.tc_p = P;
    ps->d.tc_kc = KC;
    ps->d.tc_nc = NCp;
    ps->d.W = CS;
  }
  f.d.kernel = K_TC_FOLD;
  f.d.in_cs = in_cs;
  f.src = src;
  f.dst = R_S1;
  g.d.kernel = K_TC_DFT;
  g.d.out_cs = out_cs;
  g.src = R_S1;
  g.dst = dst;
  g.tw_off = int64_t(mat_off);
  // the axis index of an output element is k itself (a fused output shift
  // would rotate it), but the product writes X_k and X_{n-k} from one
  // column: no rotation is offered
  g.axis_final = true;
  g.rot_ok = false;
  g.axis_n = n;
  passes.push_back(f);
  passes.push_back(g);
  return GBFFT_OK;
}

}  // namespace gbfft
