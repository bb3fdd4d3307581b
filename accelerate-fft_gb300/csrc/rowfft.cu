// Register-resident Stockham transform of contiguous rows (the innermost
// axis: fft / fft1D, and the first pass of fft2D / fft3D).
//
// Each row of N elements is owned by TH = N/E threads holding E elements
// each in registers.  Stage s of radix R gives every thread E/R butterflies
// j = t + TH*q.  Shared memory only carries the exchanges between stages;
// exchanges use an XOR swizzle (bits 1-3 of the element index flipped by
// bits 4-6) that keeps every access pattern of these stages conflict-free and
// keeps element pairs adjacent, so the first stage's outputs are written as
// 16-byte vectors.  The radix list is a template parameter equal to the
// planner's factorisation (factor_device), so the kernels share the stage
// twiddle table layout ([r - 1][p] per stage) of the generic pencil kernel.
//
// Two variants:
//  * rowfft_kernel: one chunk of ROWS rows per CTA, the first stage loading
//    x[t + TH*m] straight from global memory.
//  * rowfft_tma_kernel (Complex Float): persistent CTAs; a chunk of ROWS
//    contiguous rows is fetched into shared memory by one cp.async.bulk
//    (TMA) completing on an mbarrier, double buffered, so the next chunk
//    streams in while the current one is transformed.  Waits are bounded: on
//    timeout the kernel records GBFFT_ERR_TIMEOUT in the plan's status word
//    and stops.
#include <cuda_fp16.h>

#include <algorithm>

#include "butterflies.cuh"
#include "gbfft_internal.h"
#include "strided_tile.cuh"
#include "tma.cuh"

namespace gbfft {

namespace {

// Double-buffered exchanges (bufs = 2 regions of PITCH elements).
template <int N, int E, int NS, int OFF, int BUF, int PITCH, typename C, int R, int... Rest>
__device__ __forceinline__ void row_stages2(C (&v)[E], C* bufs, const C* __restrict__ tw, int t,
                                            RL<R, Rest...>) {
  row_compute<N, E, NS, R>(v, tw + OFF, t);
  if constexpr (sizeof...(Rest) > 0) {
    C* b = bufs + BUF * PITCH;
    row_write<N, E, NS, R>(v, b, t);
    __syncthreads();
    constexpr int R2 = rl_first(RL<Rest...>{});
    row_read<N, E, R2>(v, b, t);
    row_stages2<N, E, NS * R, OFF + tw_entries<R>(NS), 1 - BUF, PITCH>(v, bufs, tw, t, RL<Rest...>{});
  }
}

// Single-buffered exchanges in `b` (two barriers per exchange); ends with a
// barrier after the last read so the caller may reuse `b`.
template <int N, int E, int NS, int OFF, typename C, int R, int... Rest>
__device__ __forceinline__ void row_stages1(C (&v)[E], C* b, const C* __restrict__ tw, int t,
                                            RL<R, Rest...>) {
  row_compute<N, E, NS, R>(v, tw + OFF, t);
  if constexpr (sizeof...(Rest) > 0) {
    row_write<N, E, NS, R>(v, b, t);
    __syncthreads();
    constexpr int R2 = rl_first(RL<Rest...>{});
    row_read<N, E, R2>(v, b, t);
    __syncthreads();
    row_stages1<N, E, NS * R, OFF + tw_entries<R>(NS)>(v, b, tw, t, RL<Rest...>{});
  }
}

template <typename T, int N, int E, int ROWS, int MINB, int... Rs>
__global__ void __launch_bounds__(ROWS*(N / E), MINB) rowfft_kernel(const PassDesc d) {
  using C = typename CxT<T>::type;
  constexpr int TH = N / E;
  constexpr int R0 = rl_first(RL<Rs...>{});
  constexpr int RZ = rl_last(RL<Rs...>{});
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int slot = threadIdx.x / TH;
  const int t = threadIdx.x - slot * TH;
  // two exchange regions of ROWS rows; row `slot` at offset slot*row_pitch
  C* bufs = reinterpret_cast<C*>(smem_raw) + slot * row_pitch<N>();
  const int64_t row = int64_t(blockIdx.x) * ROWS + slot;
  const bool ok = row < d.ncols;
  const uint32_t fl = d.flags;
  const C* __restrict__ in = static_cast<const C*>(d.in) + row * d.in_cs;
  C* __restrict__ out = static_cast<C*>(d.out) + row * d.out_cs;

  // the flag handling sits in uniform branches outside the element loops
  C v[E];
#pragma unroll
  for (int q = 0; q < E / R0; ++q)
#pragma unroll
    for (int r = 0; r < R0; ++r) v[q * R0 + r] = ok ? in[t + TH * (q + r * (E / R0))] : cmake<C>(T(0), T(0));
  if (fl & F_CONJ_IN) {
#pragma unroll
    for (int e = 0; e < E; ++e) v[e].y = -v[e].y;
  }
  row_stages2<N, E, 1, 0, 0, ROWS * row_pitch<N>()>(v, bufs, static_cast<const C*>(d.tw), t,
                                                   RL<Rs...>{});
  if (!ok) return;
  if (fl & (F_SCALE | F_CONJ_OUT)) {
    const T s = (fl & F_SCALE) ? T(d.scale) : T(1);
    const T cy = (fl & F_CONJ_OUT) ? -s : s;
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = cmake<C>(v[e].x * s, v[e].y * cy);
  }
  if (fl & F_ROT_OUT) {
#pragma unroll
    for (int q = 0; q < E / RZ; ++q)
#pragma unroll
      for (int r = 0; r < RZ; ++r) {
        const int k = t + TH * (q + r * (E / RZ));
        out[k + rot_delta(d, k)] = v[q * RZ + r];
      }
  } else {
#pragma unroll
    for (int q = 0; q < E / RZ; ++q)
#pragma unroll
      for (int r = 0; r < RZ; ++r) out[t + TH * (q + r * (E / RZ))] = v[q * RZ + r];
  }
}

// Variant with one exchange buffer (half the shared memory, two barriers per
// exchange) so more CTAs fit on an SM.
template <typename T, int N, int E, int ROWS, int MINB, int... Rs>
__global__ void __launch_bounds__(ROWS*(N / E), MINB) rowfft1_kernel(const PassDesc d) {
  using C = typename CxT<T>::type;
  constexpr int TH = N / E;
  constexpr int R0 = rl_first(RL<Rs...>{});
  constexpr int RZ = rl_last(RL<Rs...>{});
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int slot = threadIdx.x / TH;
  const int t = threadIdx.x - slot * TH;
  C* b = reinterpret_cast<C*>(smem_raw) + slot * row_pitch<N>();
  const int64_t row = int64_t(blockIdx.x) * ROWS + slot;
  const bool ok = row < d.ncols;
  const uint32_t fl = d.flags;
  const C* __restrict__ in = static_cast<const C*>(d.in) + row * d.in_cs;
  C* __restrict__ out = static_cast<C*>(d.out) + row * d.out_cs;
  C v[E];
  const bool stream_in = (fl & F_L2_IN_FIRST) != 0;
  const uint64_t ipol = stream_in ? l2_policy_first() : 0;
#pragma unroll
  for (int q = 0; q < E / R0; ++q)
#pragma unroll
    for (int r = 0; r < R0; ++r) {
      C x = cmake<C>(T(0), T(0));
      if (ok) {
        const C* a = in + t + TH * (q + r * (E / R0));
        x = stream_in ? ld_l2hint(a, ipol) : *a;
      }
      if (fl & F_CONJ_IN) x.y = -x.y;
      v[q * R0 + r] = x;
    }
  row_stages1<N, E, 1, 0>(v, b, static_cast<const C*>(d.tw), t, RL<Rs...>{});
  if (!ok) return;
  const T s = T(d.scale);
  const bool keep = (fl & F_L2_OUT_LAST) != 0;
  const uint64_t pol = keep ? l2_policy_last() : 0;
#pragma unroll
  for (int q = 0; q < E / RZ; ++q)
#pragma unroll
    for (int r = 0; r < RZ; ++r) {
      C x = v[q * RZ + r];
      if (fl & F_SCALE) x = cscale(x, s);
      if (fl & F_CONJ_OUT) x.y = -x.y;
      const int k = t + TH * (q + r * (E / RZ));
      C* o = out + k + rot_delta(d, k);
      if (keep)
        st_l2hint(o, x, pol);
      else
        *o = x;
    }
}

// Bluestein over contiguous rows in one pass: the chirped row (n_in
// elements, zero padded) is transformed at the padded length N in
// registers, multiplied by the filter spectrum and conjugated, transformed
// again straight from registers, and the first n_out outputs are
// conjugated, multiplied by the chirp and stored.  (Both transforms are
// forward DFTs: the inverse is taken as conj(DFT(conj(.))).)
template <typename T, int N, int E, int ROWS, int MINB, int... Rs>
__global__ void __launch_bounds__(ROWS*(N / E), MINB) rowblue_kernel(const PassDesc d) {
  using C = typename CxT<T>::type;
  constexpr int TH = N / E;
  constexpr int R0 = rl_first(RL<Rs...>{});
  constexpr int RZ = rl_last(RL<Rs...>{});
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int slot = threadIdx.x / TH;
  const int t = threadIdx.x - slot * TH;
  C* b = reinterpret_cast<C*>(smem_raw) + slot * row_pitch<N>();
  const int64_t row = int64_t(blockIdx.x) * ROWS + slot;
  const bool ok = row < d.ncols;
  const uint32_t fl = d.flags;
  const C* __restrict__ in = static_cast<const C*>(d.in) + row * d.in_cs;
  C* __restrict__ out = static_cast<C*>(d.out) + row * d.out_cs;
  const C* __restrict__ chirp = static_cast<const C*>(d.chirp);
  const C* __restrict__ filt = static_cast<const C*>(d.filter);
  const C* __restrict__ tw = static_cast<const C*>(d.tw);
  const int nin = int(d.n_in), nout = int(d.n_out);
  C v[E];
  // all loads of the row first, then the chirp products
#pragma unroll
  for (int q = 0; q < E / R0; ++q)
#pragma unroll
    for (int r = 0; r < R0; ++r) {
      const int i = t + TH * (q + r * (E / R0));
      v[q * R0 + r] = (ok && i < nin) ? in[i] : cmake<C>(T(0), T(0));
    }
#pragma unroll
  for (int q = 0; q < E / R0; ++q)
#pragma unroll
    for (int r = 0; r < R0; ++r) {
      const int i = t + TH * (q + r * (E / R0));
      C x = v[q * R0 + r];
      if (fl & F_CONJ_IN) x.y = -x.y;
      v[q * R0 + r] = i < nin ? cmul(x, chirp[i]) : x;
    }
  row_stages1<N, E, 1, 0>(v, b, tw, t, RL<Rs...>{});
  // v[q*RZ + r] holds X[k], k = t + TH*(q + r*E/RZ); the second transform's
  // first stage wants element t + TH*(q' + r'*E/R0) in v[q'*R0 + r']
  C u[E];
#pragma unroll
  for (int q = 0; q < E / RZ; ++q)
#pragma unroll
    for (int r = 0; r < RZ; ++r) {
      const int m = q + r * (E / RZ);
      u[(m % (E / R0)) * R0 + m / (E / R0)] = cconj(cmul(v[q * RZ + r], filt[t + TH * m]));
    }
#pragma unroll
  for (int i = 0; i < E; ++i) v[i] = u[i];
  row_stages1<N, E, 1, 0>(v, b, tw, t, RL<Rs...>{});
  if (!ok) return;
  const T s = T(d.scale);
#pragma unroll
  for (int q = 0; q < E / RZ; ++q)
#pragma unroll
    for (int r = 0; r < RZ; ++r) {
      const int k = t + TH * (q + r * (E / RZ));
      if (k >= nout) continue;
      C x = cmul(cconj(v[q * RZ + r]), chirp[k]);
      if (fl & F_SCALE) x = cscale(x, s);
      if (fl & F_CONJ_OUT) x.y = -x.y;
      out[k + rot_delta(d, k)] = x;
    }
}

// ---- TMA-fed persistent variant (Complex Float) ----------------------------
template <int N, int E, int ROWS, int MINB, int... Rs>
__global__ void __launch_bounds__(ROWS*(N / E), MINB) rowfft_tma_kernel(const PassDesc d) {
  using C = float2;
  constexpr int TH = N / E;
  constexpr int P = row_pitch<N>();  // slot pitch: the exchanges' swizzle spans whole 16-element blocks
  constexpr int CH = ROWS * P;
  constexpr int R0 = rl_first(RL<Rs...>{});
  constexpr int RZ = rl_last(RL<Rs...>{});
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[2];
  C* buf0 = reinterpret_cast<C*>(smem_raw);
  const int slot = threadIdx.x / TH;
  const int t = threadIdx.x - slot * TH;
  const int64_t rows = d.ncols;
  const int64_t nchunks = (rows + ROWS - 1) / ROWS;
  const C* __restrict__ in = static_cast<const C*>(d.in);
  C* __restrict__ out = static_cast<C*>(d.out);
  const C* __restrict__ tw = static_cast<const C*>(d.tw);
  const uint32_t fl = d.flags;
  const float s = float(d.scale);

  auto issue = [&](int64_t c, int b) {
    const int64_t r0 = c * ROWS;
    const int64_t nr = (rows - r0 < ROWS) ? rows - r0 : ROWS;
    const uint32_t bytes = uint32_t(nr * N * sizeof(C));
    mbar_expect_tx(&bars[b], bytes);
    if constexpr (P == N) {
      tma_load_1d(buf0 + b * CH, in + r0 * N, bytes, &bars[b]);
    } else {
      // one copy per row into its pitched slot (N * 8 bytes, a multiple of 16)
      for (int j = 0; j < int(nr); ++j)
        tma_load_1d(buf0 + b * CH + j * P, in + (r0 + j) * N, uint32_t(N * sizeof(C)), &bars[b]);
    }
  };

  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < 2; ++k) {
      const int64_t c = int64_t(blockIdx.x) + int64_t(k) * gridDim.x;
      if (c < nchunks) issue(c, k);
    }
  }
  int it = 0;
  for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x, ++it) {
    const int b = it & 1;
    const uint32_t par = uint32_t(it >> 1) & 1u;
    // every thread observes the completed phase (acquire) before reading;
    // the abort decision is made uniformly across the CTA
    const bool timed_out = !mbar_wait_bounded(&bars[b], par, d.status);
    if (__syncthreads_or(timed_out)) break;
    C* sb = buf0 + b * CH + slot * P;
    const int64_t row = c * ROWS + slot;
    const bool ok = row < rows;
    C v[E];
#pragma unroll
    for (int q = 0; q < E / R0; ++q)
#pragma unroll
      for (int r = 0; r < R0; ++r) {
        C x = sb[t + TH * (q + r * (E / R0))];
        if (fl & F_CONJ_IN) x.y = -x.y;
        v[q * R0 + r] = x;
      }
    __syncthreads();  // stage-1 inputs consumed; the chunk buffer becomes the exchange buffer
    row_stages1<N, E, 1, 0>(v, sb, tw, t, RL<Rs...>{});
    // the buffer is free again: prefetch the chunk after next into it
    if (threadIdx.x == 0) {
      const int64_t cn = c + 2 * int64_t(gridDim.x);
      fence_async_smem();
      if (cn < nchunks) issue(cn, b);
    }
    if (ok) {
      C* o = out + row * N;
#pragma unroll
      for (int q = 0; q < E / RZ; ++q)
#pragma unroll
        for (int r = 0; r < RZ; ++r) {
          C x = v[q * RZ + r];
          if (fl & F_SCALE) x = cscale(x, s);
          if (fl & F_CONJ_OUT) x.y = -x.y;
          const int k = t + TH * (q + r * (E / RZ));
          o[k + rot_delta(d, k)] = x;
        }
    }
  }
  // drain: do not exit with a bulk copy still targeting this CTA's smem
  if (threadIdx.x == 0) {
    int it2 = it;
    for (int k = 0; k < 2; ++k, ++it2) {
      const int64_t c = int64_t(blockIdx.x) + int64_t(it2) * gridDim.x;
      if (c < nchunks) mbar_wait_bounded(&bars[it2 & 1], uint32_t(it2 >> 1) & 1u, d.status);
    }
  }
}

// ---- split-FP16 tensor-core variant (Complex Float) --------------------------
// Every radix-16 stage runs as a GEMM on the 5th-generation tensor cores:
// the 128 butterflies of a warpgroup form the rows of A (128 x 32: real then
// imaginary parts of the 16 inputs), D is the 32 x 32 real form of the
// forward DFT-16, and Y^T = A * D^T is accumulated in FP32 in tensor memory
// (tcgen05.mma kind::f16, M = 128, N = 32, K = 32).  Inputs are split as
// x*s = hi + lo in FP16 with a per-butterfly power-of-two scale s (rows are
// independent, so the scale is exact to undo) and D = D_hi + D_lo; three
// products hi*hi + hi*lo + lo*hi recover FP32 accuracy.  TMEM lane r of the
// accumulator is row r, which is the butterfly of thread r of the warpgroup,
// so tcgen05.ld 32x32b returns every thread its own 32 outputs.  Twiddles
// and the radix-8/4/2 stages stay in FP32 on the CUDA cores.
__device__ __forceinline__ int cm_off(int m, int k) {  // no-swizzle K-major core matrices
  return (m >> 3) * 512 + (k >> 3) * 128 + (m & 7) * 16 + (k & 7) * 2;
}
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
  // start address, leading byte offset 128 (K), stride byte offset 512 (M/N),
  // descriptor version 1, no swizzle
  return uint64_t((saddr >> 4) & 0x3FFF) | (uint64_t(128 >> 4) << 16) | (uint64_t(512 >> 4) << 32) |
         (uint64_t(1) << 46);
}
constexpr uint32_t kTcIdesc = (1u << 4) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

struct TcCtx {
  unsigned char* a_hi;  // 8 KiB, this warpgroup's A (hi)
  unsigned char* a_lo;  // 8 KiB (lo)
  uint32_t b_hi, b_lo;  // shared addresses of D_hi, D_lo (2 KiB each)
  uint64_t* mbar;
  uint32_t phase;
  uint32_t taddr;  // this warpgroup's accumulator columns, lane 0
  int row;         // thread's row in the warpgroup (0..127)
  int wg;          // warpgroup index in the CTA
  int* status;
};

__device__ __forceinline__ void tc_dft16(float2 (&v)[16], TcCtx& c) {
  // per-butterfly power-of-two scale: max |x*s| in [2^13, 2^14)
  float mx = 0.f;
#pragma unroll
  for (int k = 0; k < 16; ++k) mx = fmaxf(mx, fmaxf(fabsf(v[k].x), fabsf(v[k].y)));
  const int ex = mx > 0.f ? ((__float_as_int(mx) >> 23) & 0xFF) - 127 : 0;
  const int sh = max(-100, min(100, 13 - ex));
  const float s = ldexpf(1.f, sh), inv = ldexpf(1.f, -sh);
#pragma unroll
  for (int kc = 0; kc < 4; ++kc) {
    __align__(16) __half hi[8], lo[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int k = kc * 8 + q;
      const float x = (k < 16 ? v[k].x : v[k - 16].y) * s;
      const __half h = __float2half_rn(x);
      hi[q] = h;
      lo[q] = __float2half_rn(x - __half2float(h));
    }
    *reinterpret_cast<uint4*>(c.a_hi + cm_off(c.row, kc * 8)) = *reinterpret_cast<const uint4*>(hi);
    *reinterpret_cast<uint4*>(c.a_lo + cm_off(c.row, kc * 8)) = *reinterpret_cast<const uint4*>(lo);
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("bar.sync %0, 128;" ::"r"(1 + c.wg) : "memory");
  if (c.row == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t ahi = smem_u32(c.a_hi), alo = smem_u32(c.a_lo);
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
      const uint64_t dah = umma_desc(ahi + ks * 256), dal = umma_desc(alo + ks * 256);
      const uint64_t dbh = umma_desc(c.b_hi + ks * 256), dbl = umma_desc(c.b_lo + ks * 256);
      const uint32_t acc0 = ks > 0 ? 1u : 0u;
      asm volatile(
          "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
          " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(c.taddr),
          "l"(dah), "l"(dbh), "r"(kTcIdesc), "r"(acc0)
          : "memory");
      asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, 1;\n" ::"r"(c.taddr), "l"(dah),
                   "l"(dbl), "r"(kTcIdesc)
                   : "memory");
      asm volatile("tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, 1;\n" ::"r"(c.taddr), "l"(dal),
                   "l"(dbh), "r"(kTcIdesc)
                   : "memory");
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(c.mbar))
                 : "memory");
  }
  if (!mbar_wait_bounded(c.mbar, c.phase, c.status)) {
    // the product never completed: leave the inputs in place (the status
    // word records the timeout) rather than read an unfinished accumulator
    c.phase ^= 1u;
    return;
  }
  c.phase ^= 1u;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  uint32_t r[32];
  const uint32_t lane_base = uint32_t((c.row >> 5) * 32) << 16;
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
        "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
        "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(c.taddr + lane_base)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = make_float2(__uint_as_float(r[k]) * inv, __uint_as_float(r[k + 16]) * inv);
}

template <int N, int E, int NS, int R>
__device__ __forceinline__ void row_compute_tc(float2 (&v)[E], const float2* __restrict__ tw, int t,
                                               TcCtx& c) {
  if constexpr (R == 16 && E == 16) {
    if constexpr (NS > 1) {
      const int p = t % NS;
      float2 w[17];
      derive_tw<16, NS>(w, tw + p);
#pragma unroll
      for (int r = 1; r < 16; ++r) v[r] = cmul(v[r], w[r]);
    }
    tc_dft16(v, c);
  } else {
    row_compute<N, E, NS, R>(v, tw, t);
  }
}

template <int N, int E, int NS, int OFF, int R, int... Rest>
__device__ __forceinline__ void row_stages_tc(float2 (&v)[E], float2* b, const float2* __restrict__ tw,
                                              int t, TcCtx& c, RL<R, Rest...>) {
  row_compute_tc<N, E, NS, R>(v, tw + OFF, t, c);
  if constexpr (sizeof...(Rest) > 0) {
    row_write<N, E, NS, R>(v, b, t);
    __syncthreads();
    constexpr int R2 = rl_first(RL<Rest...>{});
    row_read<N, E, R2>(v, b, t);
    __syncthreads();
    row_stages_tc<N, E, NS * R, OFF + tw_entries<R>(NS)>(v, b, tw, t, c, RL<Rest...>{});
  }
}

template <int N, int ROWS, int MINB, int... Rs>
__global__ void __launch_bounds__(ROWS*(N / 16), MINB) rowfft_tc_kernel(const PassDesc d) {
  using C = float2;
  constexpr int E = 16;
  constexpr int TH = N / E;
  constexpr int NT = ROWS * TH;
  constexpr int NWG = NT / 128;
  static_assert(NT % 128 == 0, "whole warpgroups");
  constexpr int R0 = rl_first(RL<Rs...>{});
  constexpr int RZ = rl_last(RL<Rs...>{});
  constexpr uint32_t kCols = (32 * NWG <= 32) ? 32 : (32 * NWG <= 64) ? 64 : (32 * NWG <= 128) ? 128 : 256;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t mbar[NWG];
  __shared__ uint32_t tslot;
  // layout: [A hi|lo per warpgroup: 16 KiB each][D hi|lo: 4 KiB][exchange: ROWS * N]
  unsigned char* amem = smem_raw;
  unsigned char* bmem = smem_raw + NWG * 16384;
  C* xbuf = reinterpret_cast<C*>(bmem + 4096);
  const int slot = threadIdx.x / TH;
  const int t = threadIdx.x - slot * TH;
  C* b = xbuf + slot * N;
  const int wg = threadIdx.x >> 7;

  // D_hi / D_lo (32 x 32 f16 each, row-major N x K in global) -> core-matrix layout
  const __half* dm = static_cast<const __half*>(d.tcmat);
  for (int i = threadIdx.x; i < 2 * 1024; i += blockDim.x) {
    const int which = i >> 10, n = (i >> 5) & 31, k = i & 31;
    *reinterpret_cast<__half*>(bmem + which * 2048 + cm_off(n, k)) = dm[i];
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (threadIdx.x == 0) {
    for (int g = 0; g < NWG; ++g) mbar_init(&mbar[g], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tslot)),
                 "r"(kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  TcCtx c;
  c.a_hi = amem + wg * 16384;
  c.a_lo = c.a_hi + 8192;
  c.b_hi = smem_u32(bmem);
  c.b_lo = smem_u32(bmem + 2048);
  c.mbar = &mbar[wg];
  c.phase = 0;
  c.taddr = tslot + uint32_t(32 * wg);
  c.row = threadIdx.x & 127;
  c.wg = wg;
  c.status = d.status;

  const int64_t rows = d.ncols;
  const int64_t nchunks = (rows + ROWS - 1) / ROWS;
  const uint32_t fl = d.flags;
  const float s = float(d.scale);
  const C* __restrict__ tw = static_cast<const C*>(d.tw);
  for (int64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    const int64_t row = ch * ROWS + slot;
    const bool ok = row < rows;
    const C* __restrict__ in = static_cast<const C*>(d.in) + row * d.in_cs;
    C v[E];
#pragma unroll
    for (int q = 0; q < E / R0; ++q)
#pragma unroll
      for (int r = 0; r < R0; ++r) {
        C x = make_float2(0.f, 0.f);
        if (ok) x = in[t + TH * (q + r * (E / R0))];
        if (fl & F_CONJ_IN) x.y = -x.y;
        v[q * R0 + r] = x;
      }
    row_stages_tc<N, E, 1, 0>(v, b, tw, t, c, RL<Rs...>{});
    if (ok) {
      C* __restrict__ out = static_cast<C*>(d.out) + row * d.out_cs;
#pragma unroll
      for (int q = 0; q < E / RZ; ++q)
#pragma unroll
        for (int r = 0; r < RZ; ++r) {
          C x = v[q * RZ + r];
          if (fl & F_SCALE) x = cscale(x, s);
          if (fl & F_CONJ_OUT) x.y = -x.y;
          const int k = t + TH * (q + r * (E / RZ));
          out[k + rot_delta(d, k)] = x;
        }
    }
    __syncthreads();  // the exchange buffer is reused by the next chunk
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (threadIdx.x < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tslot), "r"(kCols) : "memory");
}

template <int N, int ROWS, int MINB, int... Rs>
struct RowTcCfg {
  static constexpr int threads = ROWS * (N / 16);
  static size_t smem() { return size_t(threads / 128) * 16384 + 4096 + size_t(ROWS) * N * 8; }
  static int ctas_per_sm;
  static cudaError_t prepare() {
    cudaError_t e = cudaFuncSetAttribute(rowfft_tc_kernel<N, ROWS, MINB, Rs...>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem()));
    if (e != cudaSuccess) return e;
    int nb = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, rowfft_tc_kernel<N, ROWS, MINB, Rs...>, threads, smem());
    ctas_per_sm = nb > 0 ? nb : 1;
    return e;
  }
  static cudaError_t launch(const PassDesc& d, cudaStream_t s, int sms) {
    const int64_t chunks = (d.ncols + ROWS - 1) / ROWS;
    const int64_t grid = std::min<int64_t>(chunks, int64_t(sms) * ctas_per_sm);
    rowfft_tc_kernel<N, ROWS, MINB, Rs...><<<unsigned(grid), threads, smem(), s>>>(d);
    return cudaGetLastError();
  }
};
template <int N, int ROWS, int MINB, int... Rs>
int RowTcCfg<N, ROWS, MINB, Rs...>::ctas_per_sm = 1;

// lengths with radix-16 stages and whole warpgroups per CTA
// (N, rows per CTA, min CTAs per SM for row_variant 1 / 0, radices).  On
// fft2D 4096^2 the row pass took 151 us at 2 CTAs/SM (128 registers), 177 us
// at 3 (80 registers, spills) and 151 us at 1: the MMA round trip per stage,
// not occupancy, bounds it.
#define GBFFT_ROWTC_TABLE(X)        \
  X(256, 8, 2, 1, 16, 16)           \
  X(512, 4, 2, 1, 16, 16, 2)        \
  X(1024, 2, 2, 1, 16, 16, 4)       \
  X(2048, 1, 2, 3, 16, 16, 8)       \
  X(4096, 1, 2, 3, 16, 16, 16)      \
  X(8192, 1, 1, 1, 16, 16, 16, 2)

template <typename T, int N, int E, int ROWS, int MINB, int... Rs>
struct RowCfg {
  static constexpr int threads = ROWS * (N / E);
  // bulk copies move whole rows: N * 8 bytes must be a multiple of 16
  static constexpr bool tma_capable = sizeof(T) == 4 && N % 2 == 0;
  static size_t smem() { return size_t(2) * ROWS * row_pitch<N>() * sizeof(typename CxT<T>::type); }
  [[maybe_unused]] static int tma_ctas_per_sm;
  static constexpr int MINB1 = (MINB >= 3 && sizeof(T) == 4) ? 4 : MINB;
  static cudaError_t prepare() {
    cudaError_t e = cudaFuncSetAttribute(rowfft_kernel<T, N, E, ROWS, MINB, Rs...>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem()));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(rowfft1_kernel<T, N, E, ROWS, MINB1, Rs...>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem() / 2));
    if constexpr (tma_capable) {
      if (e != cudaSuccess) return e;
      e = cudaFuncSetAttribute(rowfft_tma_kernel<N, E, ROWS, MINB, Rs...>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem()));
      if (e != cudaSuccess) return e;
      int nb = 0;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, rowfft_tma_kernel<N, E, ROWS, MINB, Rs...>,
                                                        threads, smem());
      tma_ctas_per_sm = nb > 0 ? nb : 1;
    }
    return e;
  }
  static cudaError_t launch(const PassDesc& d, cudaStream_t s, int sms) {
    const int64_t chunks = (d.ncols + ROWS - 1) / ROWS;
    if (d.row_variant & 1) {
      rowfft1_kernel<T, N, E, ROWS, MINB1, Rs...><<<unsigned(chunks), threads, smem() / 2, s>>>(d);
      return cudaGetLastError();
    }
    if constexpr (tma_capable) {
      const bool tma_ok = d.in_cs == N && d.out_cs == N &&
                          (reinterpret_cast<uintptr_t>(d.in) & 15) == 0 && d.use_tma;
      if (tma_ok) {
        const int64_t grid = std::min<int64_t>(chunks, int64_t(sms) * tma_ctas_per_sm);
        rowfft_tma_kernel<N, E, ROWS, MINB, Rs...><<<unsigned(grid), threads, smem(), s>>>(d);
        return cudaGetLastError();
      }
    }
    rowfft_kernel<T, N, E, ROWS, MINB, Rs...><<<unsigned(chunks), threads, smem(), s>>>(d);
    return cudaGetLastError();
  }
};
template <typename T, int N, int E, int ROWS, int MINB, int... Rs>
int RowCfg<T, N, E, ROWS, MINB, Rs...>::tma_ctas_per_sm = 1;

// The specialised lengths (type, N, E, rows per CTA, min CTAs per SM,
// radices = factor_device(N)).  Rows per CTA are chosen small and CTAs per
// SM high, so some CTAs load while others compute: measured on GB300 with
// the double-buffered kernel (milliseconds for 512 MiB of rows),
//    32, 64, 128 (64, 32, 16 rows x 5 CTAs; before: the generic tile): 1M rows
//   of 128 1.28 -> 0.31 ms, 2M rows of 64 1.26 -> 0.44 ms, 4M rows of 32
//   1.26 -> 0.82 ms
//   256: 16 rows x 3 CTAs 0.169, 8 x 5 0.161    512: 0.187 -> 0.177
//  1024: 0.201 -> 0.189                        2048: 0.210 -> 0.191
//  1000 (100 threads a row): 4 rows x 2 CTAs 0.251, 2 x 5 (56 registers) 0.203.
#define GBFFT_ROW_TABLE(X)                   \
  X(float, 32, 16, 64, 5, 16, 2)             \
  X(float, 64, 16, 32, 5, 16, 4)             \
  X(float, 128, 16, 16, 5, 16, 8)            \
  X(float, 256, 16, 8, 5, 16, 16)            \
  X(float, 512, 16, 4, 5, 16, 16, 2)         \
  X(float, 1024, 16, 2, 5, 16, 16, 4)        \
  X(float, 2048, 16, 1, 5, 16, 16, 8)        \
  X(float, 4096, 16, 1, 3, 16, 16, 16)       \
  X(float, 8192, 16, 1, 1, 16, 16, 16, 2)    \
  X(float, 1000, 10, 2, 5, 10, 10, 10)       \
  X(double, 256, 16, 16, 2, 16, 16)          \
  X(double, 512, 16, 8, 2, 16, 16, 2)        \
  X(double, 1024, 16, 4, 2, 16, 16, 4)       \
  X(double, 2048, 16, 2, 1, 16, 16, 8)       \
  X(double, 4096, 16, 1, 1, 16, 16, 16)

template <typename T, int N, int E, int ROWS, int MINB, int... Rs>
struct RowBlueCfg {
  static constexpr int threads = ROWS * (N / E);
  static size_t smem() { return size_t(ROWS) * row_pitch<N>() * sizeof(typename CxT<T>::type); }
  static cudaError_t prepare() {
    return cudaFuncSetAttribute(rowblue_kernel<T, N, E, ROWS, MINB, Rs...>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem()));
  }
  static cudaError_t launch(const PassDesc& d, cudaStream_t s) {
    const int64_t chunks = (d.ncols + ROWS - 1) / ROWS;
    rowblue_kernel<T, N, E, ROWS, MINB, Rs...><<<unsigned(chunks), threads, smem(), s>>>(d);
    return cudaGetLastError();
  }
};

// one-pass Bluestein rows: (type, padded length N, E, rows per CTA, min CTAs
// per SM, radices = factor_device(N)).  2048 (rows of 1009): one row per
// CTA and three CTAs per SM ran 16384 rows in 0.187 ms against 0.212 ms
// for two rows and two CTAs.
#define GBFFT_ROWBLUE_TABLE(X)              \
  X(float, 256, 16, 16, 2, 16, 16)          \
  X(float, 512, 16, 8, 2, 16, 16, 2)        \
  X(float, 1024, 16, 4, 2, 16, 16, 4)       \
  X(float, 2048, 16, 1, 3, 16, 16, 8)       \
  X(float, 4096, 16, 1, 2, 16, 16, 16)

int g_sms = 0;

}  // namespace

bool row_kernel_available(int n, bool dbl) {
#define X(T, N, E, ROWS, MINB, ...) \
  if (n == N && dbl == (sizeof(T) == 8)) return true;
  GBFFT_ROW_TABLE(X)
#undef X
  return false;
}

cudaError_t prepare_row_kernels() {
  cudaError_t e = cudaSuccess;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
#define X(T, N, E, ROWS, MINB, ...) \
  if (e == cudaSuccess) e = RowCfg<T, N, E, ROWS, MINB, __VA_ARGS__>::prepare();
  GBFFT_ROW_TABLE(X)
#undef X
#define X(T, N, E, ROWS, MINB, ...) \
  if (e == cudaSuccess) e = RowBlueCfg<T, N, E, ROWS, MINB, __VA_ARGS__>::prepare();
  GBFFT_ROWBLUE_TABLE(X)
#undef X
  return e;
}

bool row_tc_available(int n) {
#define X(N, ROWS, MA, MB, ...) \
  if (n == N) return true;
  GBFFT_ROWTC_TABLE(X)
#undef X
  return false;
}

cudaError_t prepare_row_tc_kernels() {
  cudaError_t e = cudaSuccess;
#define X(N, ROWS, MA, MB, ...)                                          \
  if (e == cudaSuccess) e = RowTcCfg<N, ROWS, MA, __VA_ARGS__>::prepare(); \
  if (e == cudaSuccess && MB != MA) e = RowTcCfg<N, ROWS, MB, __VA_ARGS__>::prepare();
  GBFFT_ROWTC_TABLE(X)
#undef X
  return e;
}

cudaError_t launch_row_tc(const PassDesc& d, cudaStream_t s) {
  const int sms = g_sms > 0 ? g_sms : 1;
#define X(N, ROWS, MA, MB, ...)                                                           \
  if (d.n == N)                                                                           \
    return (d.row_variant & 1) ? RowTcCfg<N, ROWS, MA, __VA_ARGS__>::launch(d, s, sms)   \
                               : RowTcCfg<N, ROWS, MB, __VA_ARGS__>::launch(d, s, sms);
  GBFFT_ROWTC_TABLE(X)
#undef X
  return cudaErrorInvalidValue;
}

bool row_blue_available(int m, bool dbl) {
#define X(T, N, E, ROWS, MINB, ...) \
  if (m == N && dbl == (sizeof(T) == 8)) return true;
  GBFFT_ROWBLUE_TABLE(X)
#undef X
  return false;
}

cudaError_t launch_row(const PassDesc& d, bool dbl, cudaStream_t s) {
  const int sms = g_sms > 0 ? g_sms : 1;
  if (d.flags & F_BLUE) {
#define X(T, N, E, ROWS, MINB, ...) \
  if (d.n == N && dbl == (sizeof(T) == 8)) return RowBlueCfg<T, N, E, ROWS, MINB, __VA_ARGS__>::launch(d, s);
    GBFFT_ROWBLUE_TABLE(X)
#undef X
    return cudaErrorInvalidValue;
  }
#define X(T, N, E, ROWS, MINB, ...) \
  if (d.n == N && dbl == (sizeof(T) == 8)) return RowCfg<T, N, E, ROWS, MINB, __VA_ARGS__>::launch(d, s, sms);
  GBFFT_ROW_TABLE(X)
#undef X
  return cudaErrorInvalidValue;
}

}  // namespace gbfft
