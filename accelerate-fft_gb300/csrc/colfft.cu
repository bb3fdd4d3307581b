// Strided-axis transform of length 4096 (the column pass of fft2D on a
// 4096-row array, or any axis of stride S with S a multiple of 16) in one
// HBM round trip, using an 8-CTA thread-block cluster per 16-column tile.
//
// The 4096-point column DFT is split four-step as 64 x 64 (y = 64a + b,
// k = K + 64k'):
//   phase 1: CTA r owns b in [8r, 8r+8): DFT-64 over a (as 8 x 8, one smem
//            exchange), twiddle W_4096^(b*K); result kept in its smem as
//            [b_local][K][x].
//   cluster barrier
//   phase 2: CTA r owns K in [8r, 8r+8): DFT-64 over b, where b = 8*b1 + bl
//            lives in CTA b1 -- the first radix-8 stage reads one element
//            from each CTA of the cluster through distributed shared memory;
//            output rows K + 64k'.
// Every global access is a 128-byte row segment (16 consecutive columns).
#include <cooperative_groups.h>
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>

#include "butterflies.cuh"
#include "gbfft_internal.h"
#include "tma.cuh"

namespace cg = cooperative_groups;

namespace gbfft {

namespace {

template <typename C>
__device__ __forceinline__ C tw_at(const C* __restrict__ w4096, int t) {
  return __ldg(w4096 + t);
}

// v[k] *= base * W_4096^(m*k), k < 8: the powers come from two table entries
// (W^m, W^4m) with at most two complex multiplications each, applied in
// place so only four twiddles are live at a time.
template <typename C>
__device__ __forceinline__ void apply_powers8(C (&v)[8], const C* __restrict__ w, int m) {
  const C w1 = tw_at(w, m & 4095);
  const C w4 = tw_at(w, (4 * m) & 4095);
  const C w2 = cmul(w1, w1);
  const C w3 = cmul(w2, w1);
  v[1] = cmul(v[1], w1);
  v[2] = cmul(v[2], w2);
  v[3] = cmul(v[3], w3);
  v[4] = cmul(v[4], w4);
  v[5] = cmul(v[5], cmul(w4, w1));
  v[6] = cmul(v[6], cmul(w4, w2));
  v[7] = cmul(v[7], cmul(w4, w3));
}
template <typename C>
__device__ __forceinline__ void apply_powers8(C (&v)[8], const C* __restrict__ w, int m, C base) {
  const C w1 = tw_at(w, m & 4095);
  const C w4 = tw_at(w, (4 * m) & 4095);
  const C w2 = cmul(w1, w1);
  const C w3 = cmul(w2, w1);
  const C b4 = cmul(base, w4);
  v[0] = cmul(v[0], base);
  v[1] = cmul(v[1], cmul(base, w1));
  v[2] = cmul(v[2], cmul(base, w2));
  v[3] = cmul(v[3], cmul(base, w3));
  v[4] = cmul(v[4], b4);
  v[5] = cmul(v[5], cmul(b4, w1));
  v[6] = cmul(v[6], cmul(b4, w2));
  v[7] = cmul(v[7], cmul(b4, w3));
}

// address of the same shared-memory location in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t mapa_u32(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ float2 ld_dsmem(uint32_t addr, float2*) {
  float2 v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ double2 ld_dsmem(uint32_t addr, double2*) {
  double2 v;
  asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "r"(addr) : "memory");
  return v;
}

__device__ __forceinline__ void cluster_arrive_release() {
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait_acquire() {
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Tile of W columns (8 or 16) per cluster; each thread owns U butterflies
// (U = 1 or 2) of every radix-8 stage.  Shared layout [g][row][x] with a pad
// of W elements per g-block (pitch GP) so the half-warps of the W = 8 tile hit
// distinct banks.
template <int W> constexpr int col_gp() { return 64 * W + W; }

template <typename T, int W, int U, int MINB>
__global__ void __cluster_dims__(8, 1, 1) __launch_bounds__(64 * W / U, MINB)
    colfft4096_kernel(const PassDesc d) {
  using C = typename CxT<T>::type;
  constexpr int GP = col_gp<W>();
  constexpr int HS = 8 / U;  // stride between a thread's butterflies
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);
  const int r = int(cg::this_cluster().block_rank());
  const int64_t tile = int64_t(blockIdx.x) >> 3;
  const int64_t tpb = d.ncols / W;  // W-column tiles per batch
  const int64_t bo = tile / tpb;
  const int64_t x0 = (tile - bo * tpb) * W;
  const C* __restrict__ in = static_cast<const C*>(d.in) + bo * d.in_bs + x0;
  C* __restrict__ out = static_cast<C*>(d.out) + bo * d.out_bs + x0;
  const C* __restrict__ w = static_cast<const C*>(d.tw);  // W_4096^t, t < 4096
  const int64_t ies = d.in_es, oes = d.out_es;
  const uint32_t fl = d.flags;

  const int tid = threadIdx.x;
  const int x = tid % W;
  const int g = (tid / W) & 7;
  const int h = tid / (8 * W);  // 0 .. HS-1
  C v[U][8];

  // ---- phase 1, stage A: thread (x, bl = g, a2 in {h + HS*u}) ---------------
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int a2 = h + HS * u;
#pragma unroll
    for (int a1 = 0; a1 < 8; ++a1) {
      const int y = 64 * (8 * a1 + a2) + 8 * r + g;
      C e = in[int64_t(y) * ies + x];
      if (fl & F_CONJ_IN) e.y = -e.y;
      v[u][a1] = e;
    }
  }
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int a2 = h + HS * u;
    dft8(v[u]);
    apply_powers8(v[u], w, 64 * a2);
#pragma unroll
    for (int k1 = 0; k1 < 8; ++k1) sm[g * GP + (a2 * 8 + k1) * W + x] = v[u][k1];
  }
  __syncthreads();
  // ---- stage B: thread (x, bl = g, k1 in {h + HS*u}) -------------------------
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int k1 = h + HS * u;
#pragma unroll
    for (int a2 = 0; a2 < 8; ++a2) v[u][a2] = sm[g * GP + (a2 * 8 + k1) * W + x];
  }
  __syncthreads();
  const int b = 8 * r + g;
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int k1 = h + HS * u;
    dft8(v[u]);
    // W^(b*K) = W^(b*k1) * W^(8*b*k2)
    apply_powers8(v[u], w, 8 * b, tw_at(w, b * k1));
#pragma unroll
    for (int k2 = 0; k2 < 8; ++k2) sm[g * GP + (k1 + 8 * k2) * W + x] = v[u][k2];
  }
  cluster_arrive_release();
  cluster_wait_acquire();

  // ---- phase 2, stage C: thread (x, Kl = g, bl' in {h + HS*u}) ---------------
  const int K = 8 * r + g;
  const uint32_t sm0 = smem_u32(sm);
#pragma unroll
  for (int b1 = 0; b1 < 8; ++b1) {
    const uint32_t rs = mapa_u32(sm0, uint32_t(b1));
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int blp = h + HS * u;
      v[u][b1] = ld_dsmem(rs + uint32_t((blp * GP + K * W + x) * sizeof(C)), (C*)nullptr);
    }
  }
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int blp = h + HS * u;
    dft8(v[u]);
    apply_powers8(v[u], w, 64 * blp);
  }
  // signal that this CTA's reads of the cluster's smem are done (release
  // orders the remote loads before the arrive), and wait until every CTA's
  // are before overwriting local smem
  cluster_arrive_release();
  cluster_wait_acquire();
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int blp = h + HS * u;
#pragma unroll
    for (int kb1 = 0; kb1 < 8; ++kb1) sm[g * GP + (blp * 8 + kb1) * W + x] = v[u][kb1];
  }
  __syncthreads();
  // ---- stage D: thread (x, Kl = g, kb1 in {h + HS*u}) ------------------------
  const T s = T(d.scale);
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int kb1 = h + HS * u;
#pragma unroll
    for (int blp = 0; blp < 8; ++blp) v[u][blp] = sm[g * GP + (blp * 8 + kb1) * W + x];
    dft8(v[u]);
#pragma unroll
    for (int kb2 = 0; kb2 < 8; ++kb2) {
      C e = v[u][kb2];
      if (fl & F_SCALE) e = cscale(e, s);
      if (fl & F_CONJ_OUT) e.y = -e.y;
      const int row = K + 64 * (kb1 + 8 * kb2);
      out[int64_t(row) * oes + x + rot_delta(d, row)] = e;
    }
  }
}

// Push variant: phase-1 results go straight into the owning CTA's receive
// buffer with st.async (distributed shared memory, completing on the
// receiver's mbarrier transaction count), so phase 2 reads only local shared
// memory.  One cluster barrier at the start (before any data is pending)
// makes every receiver's mbarrier initialisation visible; no barrier is
// needed between the phases.  Layout: work buffer 8 x GP (phase-1 exchange
// and phase-2 exchange), receive buffer [b][Kl][x] of 64 * 8 * W elements.
__device__ __forceinline__ void st_async(uint32_t addr, float2 v, uint32_t bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f32 [%0], {%1, %2}, [%3];" ::"r"(addr),
               "f"(v.x), "f"(v.y), "r"(bar)
               : "memory");
}
constexpr uint32_t kColWaitLimit = 1u << 22;

template <typename T, int W, int U, int MINB>
__global__ void __cluster_dims__(8, 1, 1) __launch_bounds__(64 * W / U, MINB)
    colfft4096_push_kernel(const PassDesc d) {
  using C = typename CxT<T>::type;
  constexpr int GP = col_gp<W>();
  constexpr int HS = 8 / U;
  constexpr uint32_t kRecvBytes = 64u * 8u * W * sizeof(C);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);
  C* rv = sm + 8 * GP;  // receive buffer
  __shared__ __align__(8) uint64_t rbar;
  const int r = int(cg::this_cluster().block_rank());
  const int64_t tile = int64_t(blockIdx.x) >> 3;
  const int64_t tpb = d.ncols / W;
  const int64_t bo = tile / tpb;
  const int64_t x0 = (tile - bo * tpb) * W;
  const C* __restrict__ in = static_cast<const C*>(d.in) + bo * d.in_bs + x0;
  C* __restrict__ out = static_cast<C*>(d.out) + bo * d.out_bs + x0;
  const C* __restrict__ w = static_cast<const C*>(d.tw);
  const int64_t ies = d.in_es, oes = d.out_es;
  const uint32_t fl = d.flags;
  const int tid = threadIdx.x;
  const int x = tid % W;
  const int g = (tid / W) & 7;
  const int h = tid / (8 * W);

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&rbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // every receiver's mbarrier is initialised before anyone pushes to it;
  // the wait is deferred until the first push
  cluster_arrive_release();

  C v[U][8];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int a2 = h + HS * u;
#pragma unroll
    for (int a1 = 0; a1 < 8; ++a1) {
      const int y = 64 * (8 * a1 + a2) + 8 * r + g;
      C e = in[int64_t(y) * ies + x];
      if (fl & F_CONJ_IN) e.y = -e.y;
      v[u][a1] = e;
    }
  }
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int a2 = h + HS * u;
    dft8(v[u]);
    apply_powers8(v[u], w, 64 * a2);
#pragma unroll
    for (int k1 = 0; k1 < 8; ++k1) sm[g * GP + (a2 * 8 + k1) * W + x] = v[u][k1];
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int k1 = h + HS * u;
#pragma unroll
    for (int a2 = 0; a2 < 8; ++a2) v[u][a2] = sm[g * GP + (a2 * 8 + k1) * W + x];
  }
  if (tid == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&rbar)),
                 "r"(kRecvBytes)
                 : "memory");
  }
  cluster_wait_acquire();
  const int b = 8 * r + g;
  const uint32_t rv0 = smem_u32(rv), bar0 = smem_u32(&rbar);
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int k1 = h + HS * u;
    dft8(v[u]);
    apply_powers8(v[u], w, 8 * b, tw_at(w, b * k1));
    // K = k1 + 8*k2 lives in CTA k2 at [b][Kl = k1][x]
#pragma unroll
    for (int k2 = 0; k2 < 8; ++k2) {
      const uint32_t dst = mapa_u32(rv0 + uint32_t(((b * 8 + k1) * W + x) * sizeof(C)), uint32_t(k2));
      st_async(dst, v[u][k2], mapa_u32(bar0, uint32_t(k2)));
    }
  }
  // ---- phase 2: wait for all 64 b of this CTA's 8 K values ----------------
  bool ok = false;
  for (uint32_t it = 0; it < kColWaitLimit && !ok; ++it) {
    uint32_t t;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(t)
        : "r"(bar0)
        : "memory");
    ok = t != 0;
  }
  if (!ok && d.status) atomicExch(d.status, GBFFT_ERR_TIMEOUT_DEVICE);
  const int K = 8 * r + g;
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int blp = h + HS * u;
#pragma unroll
    for (int b1 = 0; b1 < 8; ++b1) v[u][b1] = rv[((8 * b1 + blp) * 8 + g) * W + x];
    dft8(v[u]);
    apply_powers8(v[u], w, 64 * blp);
#pragma unroll
    for (int kb1 = 0; kb1 < 8; ++kb1) sm[g * GP + (blp * 8 + kb1) * W + x] = v[u][kb1];
  }
  __syncthreads();
  const T s = T(d.scale);
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int kb1 = h + HS * u;
#pragma unroll
    for (int blp = 0; blp < 8; ++blp) v[u][blp] = sm[g * GP + (blp * 8 + kb1) * W + x];
    dft8(v[u]);
#pragma unroll
    for (int kb2 = 0; kb2 < 8; ++kb2) {
      C e = v[u][kb2];
      if (fl & F_SCALE) e = cscale(e, s);
      if (fl & F_CONJ_OUT) e.y = -e.y;
      out[int64_t(K + 64 * (kb1 + 8 * kb2)) * oes + x + rot_delta(d, K + 64 * (kb1 + 8 * kb2))] = e;
    }
  }
}

template <typename T, int W, int U, int MINB>
struct ColPushCfg {
  static constexpr int threads = 64 * W / U;
  static size_t smem() { return (size_t(8) * col_gp<W>() + size_t(64) * 8 * W) * sizeof(typename CxT<T>::type); }
  static cudaError_t prepare() {
    return cudaFuncSetAttribute(colfft4096_push_kernel<T, W, U, MINB>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem()));
  }
  static cudaError_t launch(const PassDesc& d, cudaStream_t s) {
    const int64_t tiles = (d.ncols / W) * d.nbatch;
    colfft4096_push_kernel<T, W, U, MINB><<<unsigned(tiles * 8), threads, smem(), s>>>(d);
    return cudaGetLastError();
  }
};

// Radix-16 variant: 4096 = 16 x 256 (y = 256a + b, k = K1 + 16k').
//   phase 1: CTA r owns b in [32r, 32r+32): one DFT-16 over a per (b, x)
//            straight from the loaded registers, twiddle W_4096^(b*K1), and
//            K1 is pushed (st.async) to CTA K1/2, receive layout [b][K1 % 2][x].
//   phase 2: CTA r' owns K1 in {2r', 2r'+1}: DFT-256 over b as 16 x 16
//            (b = 16*beta + gamma, k' = kappa + 16*lambda) with one local
//            exchange; output row K1 + 16*kappa + 256*lambda.
// Three radix-16 stages and two twiddle stages per element.
template <typename C>
__device__ __forceinline__ void apply_powers16(C (&v)[16], const C* __restrict__ w, int m) {
  // v[k] *= W_4096^(m*k): W^m, W^4m, W^8m loaded, the rest at most 3 products deep
  const C w1 = tw_at(w, m & 4095), w4 = tw_at(w, (4 * m) & 4095), w8 = tw_at(w, (8 * m) & 4095);
  const C w2 = cmul(w1, w1), w3 = cmul(w2, w1), w12 = cmul(w8, w4);
  v[1] = cmul(v[1], w1);
  v[2] = cmul(v[2], w2);
  v[3] = cmul(v[3], w3);
  v[4] = cmul(v[4], w4);
  v[5] = cmul(v[5], cmul(w4, w1));
  v[6] = cmul(v[6], cmul(w4, w2));
  v[7] = cmul(v[7], cmul(w4, w3));
  v[8] = cmul(v[8], w8);
  v[9] = cmul(v[9], cmul(w8, w1));
  v[10] = cmul(v[10], cmul(w8, w2));
  v[11] = cmul(v[11], cmul(w8, w3));
  v[12] = cmul(v[12], w12);
  v[13] = cmul(v[13], cmul(w12, w1));
  v[14] = cmul(v[14], cmul(w12, w2));
  v[15] = cmul(v[15], cmul(w12, w3));
}

template <typename T, int W, int MINB>
__global__ void __cluster_dims__(8, 1, 1) __launch_bounds__(32 * W, MINB)
    colfft4096_r16_kernel(const PassDesc d) {
  using C = typename CxT<T>::type;
  constexpr uint32_t kRecvBytes = 4096u * W / 8u * sizeof(C);  // 256 b x 2 K1 x W
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* rv = reinterpret_cast<C*>(smem_raw);  // [b][K1l][x], reused for the phase-2 exchange
  __shared__ __align__(8) uint64_t rbar;
  const int r = int(cg::this_cluster().block_rank());
  const int64_t tile = int64_t(blockIdx.x) >> 3;
  const int64_t tpb = d.ncols / W;
  const int64_t bo = tile / tpb;
  const int64_t x0 = (tile - bo * tpb) * W;
  const C* __restrict__ in = static_cast<const C*>(d.in) + bo * d.in_bs + x0;
  C* __restrict__ out = static_cast<C*>(d.out) + bo * d.out_bs + x0;
  const C* __restrict__ w = static_cast<const C*>(d.tw);
  const int64_t ies = d.in_es, oes = d.out_es;
  const uint32_t fl = d.flags;
  const int tid = threadIdx.x;
  const int x = tid % W;
  const int q = tid / W;  // 0..31

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&rbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  cluster_arrive_release();

  // ---- phase 1: thread (x, bl = q): DFT-16 over a of column x, b = 32r + bl
  const int b = 32 * r + q;
  C v[16];
  const bool stream_in = (fl & F_L2_IN_FIRST) != 0;
  const uint64_t ipol = stream_in ? l2_policy_first() : 0;
#pragma unroll
  for (int a = 0; a < 16; ++a) {
    const C* p = in + int64_t(256 * a + b) * ies + x;
    C e = stream_in ? ld_l2hint(p, ipol) : *p;
    if (fl & F_CONJ_IN) e.y = -e.y;
    v[a] = e;
  }
  dft16(v);
  apply_powers16(v, w, b);  // W^(b*K1)
  if (tid == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&rbar)),
                 "r"(kRecvBytes)
                 : "memory");
  }
  cluster_wait_acquire();
  const uint32_t rv0 = smem_u32(rv), bar0 = smem_u32(&rbar);
#pragma unroll
  for (int K1 = 0; K1 < 16; ++K1) {
    const uint32_t dst = mapa_u32(rv0 + uint32_t(((b * 2 + (K1 & 1)) * W + x) * sizeof(C)), uint32_t(K1 >> 1));
    st_async(dst, v[K1], mapa_u32(bar0, uint32_t(K1 >> 1)));
  }
  // ---- phase 2: wait for the 256 b of this CTA's two K1 values ------------
  bool ok = false;
  for (uint32_t it = 0; it < kColWaitLimit && !ok; ++it) {
    uint32_t t;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(t)
        : "r"(bar0)
        : "memory");
    ok = t != 0;
  }
  if (!ok && d.status) atomicExch(d.status, GBFFT_ERR_TIMEOUT_DEVICE);
  // stage 2: thread (x, K1l = q & 1, gamma = q >> 1): DFT-16 over beta
  const int K1l = q & 1;
  const int gamma = q >> 1;
#pragma unroll
  for (int beta = 0; beta < 16; ++beta) v[beta] = rv[((16 * beta + gamma) * 2 + K1l) * W + x];
  dft16(v);
  apply_powers16(v, w, 16 * gamma);  // W_256^(gamma*kappa)
  __syncthreads();  // every stage-2 read of the receive buffer is done
#pragma unroll
  for (int kappa = 0; kappa < 16; ++kappa) rv[((kappa * 16 + gamma) * 2 + K1l) * W + x] = v[kappa];
  __syncthreads();
  // stage 3: thread (x, K1l, kappa = q >> 1): DFT-16 over gamma
  const int kappa = q >> 1;
#pragma unroll
  for (int g = 0; g < 16; ++g) v[g] = rv[((kappa * 16 + g) * 2 + K1l) * W + x];
  dft16(v);
  const int K1 = 2 * r + K1l;
  const T s = T(d.scale);
#pragma unroll
  for (int lambda = 0; lambda < 16; ++lambda) {
    C e = v[lambda];
    if (fl & F_SCALE) e = cscale(e, s);
    if (fl & F_CONJ_OUT) e.y = -e.y;
    out[int64_t(K1 + 16 * kappa + 256 * lambda) * oes + x + rot_delta(d, K1 + 16 * kappa + 256 * lambda)] = e;
  }
}

// Persistent form of the radix-16 kernel: each 8-CTA cluster walks a
// sequence of tiles.  CTA r's 512 input rows (256a + 32r + q, a < 16,
// q < 32) of W columns arrive by ONE tiled tensor copy (box W x 32 x 16 of
// the view [a][b][x]) into a load buffer [a][q][x]; as soon as the tile's
// values are in registers the copy of the cluster's next tile is issued into
// the same buffer, so HBM reads overlap the DFTs, the DSMEM pushes and the
// stores of the current tile.  The receive buffer [b][K1l][x] is reused per
// tile: the per-tile cluster barrier (after every CTA has armed its receive
// mbarrier and finished reading the previous tile) orders the pushes.
// Every wait is bounded; a CTA never leaves the tile loop early, so the
// cluster barriers stay matched.
template <typename T, int W, int MINB>
__global__ void __cluster_dims__(8, 1, 1) __launch_bounds__(32 * W, MINB)
    colfft4096_r16_tma_kernel(const __grid_constant__ CUtensorMap tmap, const PassDesc d) {
  using C = typename CxT<T>::type;
  constexpr int K = int(sizeof(C) / 8);
  constexpr uint32_t kRecvBytes = 4096u * W / 8u * sizeof(C);
  constexpr uint32_t kLoadBytes = 512u * W * sizeof(C);
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  C* lb = reinterpret_cast<C*>(smem_raw + ((128u - (raw & 127u)) & 127u));  // [a][q][x]
  C* rv = lb + 512 * W;                                                       // [b][K1l][x]
  uint64_t* bars = reinterpret_cast<uint64_t*>(rv + 512 * W);                 // load, receive
  // uniform across the cluster (same layout in every CTA): report, copy nothing
  if ((smem_u32(lb) & 127u) != 0 || (reinterpret_cast<uint64_t>(&tmap) & 63u) != 0) {
    if (threadIdx.x == 0 && d.status) atomicExch(d.status, GBFFT_ERR_INTERNAL_DEVICE);
    return;
  }
  const int r = int(cg::this_cluster().block_rank());
  const int64_t tpb = d.ncols / W;
  const int64_t tiles = tpb * d.nbatch;
  const int64_t cid = int64_t(blockIdx.x) >> 3, ncl = int64_t(gridDim.x) >> 3;
  const C* __restrict__ w = static_cast<const C*>(d.tw);
  const int64_t oes = d.out_es;
  const uint32_t fl = d.flags;
  const int tid = threadIdx.x;
  const int x = tid % W;
  const int q = tid / W;  // 0..31
  const int b = 32 * r + q;
  const uint32_t rv0 = smem_u32(rv), rbar = smem_u32(&bars[1]);

  auto issue = [&](int64_t tile) {
    const int64_t bo = tile / tpb;
    const int64_t x0 = (tile - bo * tpb) * W;
    mbar_expect_tx(&bars[0], kLoadBytes);
    tma_load_tile(lb, &tmap, 4, int(x0 * K), 32 * r, 0, int(bo), &bars[0]);
  };
  if (tid == 0) {
    prefetch_tensormap(&tmap);
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if (cid < tiles) issue(cid);
  }
  __syncthreads();
  bool timed_out = false;
  int k = 0;
  for (int64_t tile = cid; tile < tiles; tile += ncl, ++k) {
    const uint32_t par = uint32_t(k) & 1u;
    if (!mbar_wait_bounded(&bars[0], par, d.status)) timed_out = true;
    // ---- phase 1: thread (x, q): DFT-16 over a of column x, b = 32r + q
    C v[16];
#pragma unroll
    for (int a = 0; a < 16; ++a) {
      C e = lb[(a * 32 + q) * W + x];
      if (fl & F_CONJ_IN) e.y = -e.y;
      v[a] = e;
    }
    __syncthreads();  // the load buffer is consumed: fetch the next tile into it
    if (tid == 0 && tile + ncl < tiles) {
      fence_async_smem();
      issue(tile + ncl);
    }
    dft16(v);
    apply_powers16(v, w, b);  // W^(b*K1)
    if (tid == 0) mbar_expect_tx(&bars[1], kRecvBytes);
    cluster_arrive_release();  // receive buffer free (previous tile read) and armed
    cluster_wait_acquire();
#pragma unroll
    for (int K1 = 0; K1 < 16; ++K1) {
      const uint32_t dst = mapa_u32(rv0 + uint32_t(((b * 2 + (K1 & 1)) * W + x) * sizeof(C)), uint32_t(K1 >> 1));
      st_async(dst, v[K1], mapa_u32(rbar, uint32_t(K1 >> 1)));
    }
    if (!mbar_wait_bounded(&bars[1], par, d.status)) timed_out = true;
    // ---- phase 2, stage 2: thread (x, K1l = q & 1, gamma = q >> 1): DFT-16 over beta
    const int K1l = q & 1;
    const int gamma = q >> 1;
#pragma unroll
    for (int beta = 0; beta < 16; ++beta) v[beta] = rv[((16 * beta + gamma) * 2 + K1l) * W + x];
    dft16(v);
    apply_powers16(v, w, 16 * gamma);  // W_256^(gamma*kappa)
    __syncthreads();
#pragma unroll
    for (int kappa = 0; kappa < 16; ++kappa) rv[((kappa * 16 + gamma) * 2 + K1l) * W + x] = v[kappa];
    __syncthreads();
    // stage 3: thread (x, K1l, kappa = q >> 1): DFT-16 over gamma
    const int kappa = q >> 1;
#pragma unroll
    for (int g = 0; g < 16; ++g) v[g] = rv[((kappa * 16 + g) * 2 + K1l) * W + x];
    dft16(v);
    const int64_t bo = tile / tpb;
    const int64_t x0 = (tile - bo * tpb) * W;
    C* __restrict__ out = static_cast<C*>(d.out) + bo * d.out_bs + x0;
    const int K1 = 2 * r + K1l;
    const T s = T(d.scale);
#pragma unroll
    for (int lambda = 0; lambda < 16; ++lambda) {
      C e = v[lambda];
      if (fl & F_SCALE) e = cscale(e, s);
      if (fl & F_CONJ_OUT) e.y = -e.y;
      out[int64_t(K1 + 16 * kappa + 256 * lambda) * oes + x + rot_delta(d, K1 + 16 * kappa + 256 * lambda)] = e;
    }
  }
  // a timed-out wait may leave a copy landing in this CTA's buffers: wait
  // (bounded) for the load barrier's last phase before leaving
  if (timed_out && tid == 0) mbar_wait_bounded(&bars[0], uint32_t(k > 0 ? k - 1 : 0) & 1u, nullptr);
  // no CTA leaves while a sibling may still address its shared memory
  cluster_arrive_release();
  cluster_wait_acquire();
}

template <typename T, int W, int MINB>
struct ColR16Cfg {
  static constexpr int threads = 32 * W;
  static size_t smem() { return size_t(512) * W * sizeof(typename CxT<T>::type); }
  static cudaError_t prepare() {
    return cudaFuncSetAttribute(colfft4096_r16_kernel<T, W, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(smem()));
  }
  static cudaError_t launch(const PassDesc& d, cudaStream_t s) {
    const int64_t tiles = (d.ncols / W) * d.nbatch;
    colfft4096_r16_kernel<T, W, MINB><<<unsigned(tiles * 8), threads, smem(), s>>>(d);
    return cudaGetLastError();
  }
};

// Leaner form of the radix-16 kernel (Complex Float), same split and data
// flow, fewer instructions per element:
//   * twiddles come from two shared-memory tables filled at the start,
//     W_4096^(b*K1) for the CTA's 32 b ([bl][K1]) and W_256^(gamma*kappa)
//     ([gamma][kappa]), read two at a time as 16-byte vectors, instead of
//     being built by products of three table entries;
//   * the two K1 values a thread sends to one CTA go as one 16-byte
//     st.async (receive layout [b][x][K1l]), 8 pushes per thread instead of 16;
//   * the flag handling (conjugation, scaling, output rotation) is hoisted
//     out of the element loops into uniform branches.
__device__ __forceinline__ void st_async2(uint32_t addr, float2 a, float2 b, uint32_t bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(
                   addr),
               "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "r"(bar)
               : "memory");
}

// v[k] *= tab[k], k = 1..15 (tab[0] = 1): eight 16-byte shared loads
__device__ __forceinline__ void apply_table16(float2 (&v)[16], const float2* tab) {
  const float4* t4 = reinterpret_cast<const float4*>(tab);
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float4 p = t4[j];
    if (j > 0) v[2 * j] = cmul(v[2 * j], make_float2(p.x, p.y));
    v[2 * j + 1] = cmul(v[2 * j + 1], make_float2(p.z, p.w));
  }
}

// twiddle table row pitch: 16 entries + one 16-byte pad, so the rows a warp
// reads at once (four of t1, two of t2) start in different banks
constexpr int kTabPitch = 18;

template <int W>
constexpr size_t col_r16b_smem() {
  return size_t(512) * W * sizeof(float2) + size_t(32 + 16) * kTabPitch * sizeof(float2);
}

template <int W, int MINB>
__global__ void __cluster_dims__(8, 1, 1) __launch_bounds__(32 * W, MINB)
    colfft4096_r16b_kernel(const PassDesc d) {
  using C = float2;
  static_assert(W == 8 || W == 16, "whole values of q per warp");
  constexpr uint32_t kRecvBytes = 4096u * W / 8u * sizeof(C);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* rv = reinterpret_cast<C*>(smem_raw);  // [b][x][K1l], reused for the stage-2 exchange
  C* t1 = rv + 512 * W;                     // [bl][K1]: W_4096^((32r + bl) * K1), rows kTabPitch apart
  C* t2 = t1 + 32 * kTabPitch;              // [gamma][kappa]: W_256^(gamma * kappa)
  __shared__ __align__(8) uint64_t rbar;
  const int r = int(cg::this_cluster().block_rank());
  const int64_t tile = int64_t(blockIdx.x) >> 3;
  const int64_t tpb = d.ncols / W;
  const int64_t bo = tile / tpb;
  const int64_t x0 = (tile - bo * tpb) * W;
  const C* __restrict__ w = static_cast<const C*>(d.tw);
  const uint32_t fl = d.flags;
  const int tid = threadIdx.x;
  const int x = tid % W;
  const int q = tid / W;  // 0..31

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&rbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // the mbarrier init is published by its own release fence; the arrive only
  // has to tell the siblings that this CTA runs
  asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");

  // twiddle table entries first (their loads overlap the column loads).
  // Every table row is filled and read by the threads of one warp: row q of
  // t1 by the threads (x, q), row gamma of t2 by the threads with q >> 1 =
  // gamma (a warp holds 32 / W whole values of q, W >= 8), so a warp barrier
  // orders the fills before the reads.
  C e1[16 / W], e2 = make_float2(1.f, 0.f);
#pragma unroll
  for (int i = 0; i < 16 / W; ++i) e1[i] = tw_at(w, ((32 * r + q) * (x + W * i)) & 4095);
  const int k2 = x + W * (q & 1);
  if (k2 < 16) e2 = tw_at(w, (16 * (q >> 1) * k2) & 4095);

  // ---- phase 1: thread (x, bl = q): DFT-16 over a of column x, b = 32r + q
  const int b = 32 * r + q;
  C v[16];
  {
    const C* __restrict__ in = static_cast<const C*>(d.in) + bo * d.in_bs + x0 + int64_t(b) * d.in_es + x;
    const int64_t as = 256 * d.in_es;
    // no evict-first hint on these loads: the other half of each 128-byte
    // line is read by the neighbouring tile's cluster shortly after (with
    // the hint the 4096 x 4096 column pass took 73.7 instead of 71.7 us)
#pragma unroll
    for (int a = 0; a < 16; ++a) v[a] = in[a * as];
  }
#pragma unroll
  for (int i = 0; i < 16 / W; ++i) t1[kTabPitch * q + x + W * i] = e1[i];
  if (k2 < 16) t2[kTabPitch * (q >> 1) + k2] = e2;
  if (fl & F_CONJ_IN) {
#pragma unroll
    for (int a = 0; a < 16; ++a) v[a].y = -v[a].y;
  }
  dft16(v);
  __syncwarp();  // this warp's twiddle table rows
  apply_table16(v, t1 + kTabPitch * q);  // W^(b*K1)
  if (tid == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&rbar)),
                 "r"(kRecvBytes)
                 : "memory");
  }
  cluster_wait_acquire();
  const uint32_t bar0 = smem_u32(&rbar);
  {
    const uint32_t dst = smem_u32(rv) + uint32_t((b * W + x) * 2 * sizeof(C));
#pragma unroll
    for (int j = 0; j < 8; ++j) st_async2(mapa_u32(dst, uint32_t(j)), v[2 * j], v[2 * j + 1], mapa_u32(bar0, uint32_t(j)));
  }
  // ---- phase 2: wait for the 256 b of this CTA's two K1 values ------------
  bool ok = false;
  for (uint32_t it = 0; it < kColWaitLimit && !ok; ++it) {
    uint32_t t;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(t)
        : "r"(bar0)
        : "memory");
    ok = t != 0;
  }
  if (!ok && d.status) atomicExch(d.status, GBFFT_ERR_TIMEOUT_DEVICE);
  // stage 2: thread (x, K1l = q & 1, gamma = q >> 1): DFT-16 over beta
  const int K1l = q & 1;
  const int gamma = q >> 1;
  C* col = rv + 2 * x + K1l;  // element (row, x, K1l) at col[row * 2W]
#pragma unroll
  for (int beta = 0; beta < 16; ++beta) v[beta] = col[(16 * beta + gamma) * 2 * W];
  dft16(v);
  apply_table16(v, t2 + kTabPitch * gamma);  // W_256^(gamma*kappa)
  __syncthreads();  // every stage-2 read of the receive buffer is done
#pragma unroll
  for (int kappa = 0; kappa < 16; ++kappa) col[(kappa * 16 + gamma) * 2 * W] = v[kappa];
  __syncthreads();
  // stage 3: thread (x, K1l, kappa = q >> 1): DFT-16 over gamma
  const int kappa = q >> 1;
#pragma unroll
  for (int g = 0; g < 16; ++g) v[g] = col[(kappa * 16 + g) * 2 * W];
  dft16(v);
  if (fl & (F_SCALE | F_CONJ_OUT)) {
    const float s = (fl & F_SCALE) ? float(d.scale) : 1.0f;
    const float cy = (fl & F_CONJ_OUT) ? -s : s;
#pragma unroll
    for (int lambda = 0; lambda < 16; ++lambda) v[lambda] = make_float2(v[lambda].x * s, v[lambda].y * cy);
  }
  const int K1 = 2 * r + K1l;
  C* __restrict__ out = static_cast<C*>(d.out) + bo * d.out_bs + x0 + x;
  const int64_t oes = d.out_es;
  if (fl & F_ROT_OUT) {
#pragma unroll
    for (int lambda = 0; lambda < 16; ++lambda) {
      const int l = K1 + 16 * kappa + 256 * lambda;
      out[int64_t(l) * oes + rot_delta(d, l)] = v[lambda];
    }
  } else {
    C* o = out + int64_t(K1 + 16 * kappa) * oes;
    const int64_t ls = 256 * oes;
#pragma unroll
    for (int lambda = 0; lambda < 16; ++lambda) o[lambda * ls] = v[lambda];
  }
}

template <int W, int MINB>
struct ColR16bCfg {
  static constexpr int threads = 32 * W;
  static cudaError_t prepare() {
    return cudaFuncSetAttribute(colfft4096_r16b_kernel<W, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(col_r16b_smem<W>()));
  }
  static cudaError_t launch(const PassDesc& d, cudaStream_t s) {
    const int64_t tiles = (d.ncols / W) * d.nbatch;
    colfft4096_r16b_kernel<W, MINB><<<unsigned(tiles * 8), threads, col_r16b_smem<W>(), s>>>(d);
    return cudaGetLastError();
  }
};

template <typename T, int W> size_t col_smem() { return size_t(8) * col_gp<W>() * sizeof(typename CxT<T>::type); }

template <typename T, int W, int U, int MINB>
struct ColCfg {
  static constexpr int threads = 64 * W / U;
  static cudaError_t prepare() {
    return cudaFuncSetAttribute(colfft4096_kernel<T, W, U, MINB>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, int(col_smem<T, W>()));
  }
  static cudaError_t launch(const PassDesc& d, cudaStream_t s) {
    const int64_t tiles = (d.ncols / W) * d.nbatch;
    colfft4096_kernel<T, W, U, MINB><<<unsigned(tiles * 8), threads, col_smem<T, W>(), s>>>(d);
    return cudaGetLastError();
  }
};

// Tensor map of a 4096-point strided pass's input for the persistent
// kernel: (columns in 8-byte words, b, a, batch) with row = 256a + b, box
// W x 32 x 16 x 1.  Returns false when the layout does not fit.
bool col_tensor_map(const PassDesc& d, int W, size_t eb, CUtensorMap* map) {
  if (!d.use_tma || d.in_cs != 1 || (reinterpret_cast<uintptr_t>(d.in) & 15)) return false;
  auto fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(tensor_map_encode_fn());
  if (!fn) return false;
  const uint64_t K = eb / 8;
  const uint64_t es = uint64_t(d.in_es) * eb, bs = uint64_t(d.in_bs) * eb;
  auto fits = [](uint64_t s) { return s > 0 && s % 16 == 0 && s < (uint64_t(1) << 40); };
  if (!fits(es) || !fits(256 * es) || (d.nbatch > 1 && !fits(bs))) return false;
  if (uint64_t(d.ncols) * K > (uint64_t(1) << 31) || d.nbatch > (int64_t(1) << 31)) return false;
  const cuuint64_t dims[4] = {cuuint64_t(d.ncols) * K, 256, 16, cuuint64_t(d.nbatch)};
  const cuuint64_t strides[3] = {es, 256 * es, fits(bs) ? bs : 256 * es};
  const cuuint32_t box[4] = {cuuint32_t(W * K), 32, 16, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 4, const_cast<void*>(d.in), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <typename T, int W, int MINB>
struct ColR16TmaCfg {
  static constexpr int threads = 32 * W;
  static inline int clusters = 0;  // co-resident clusters
  static size_t smem() { return 128 + size_t(1024) * W * sizeof(typename CxT<T>::type) + 2 * sizeof(uint64_t); }
  static cudaError_t prepare() {
    auto k = colfft4096_r16_tma_kernel<T, W, MINB>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem()));
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(8 * 1024, 1, 1);
    cfg.blockDim = dim3(threads, 1, 1);
    cfg.dynamicSmemBytes = smem();
    int n = 0;
    e = cudaOccupancyMaxActiveClusters(&n, (void*)k, &cfg);
    clusters = n > 0 ? n : 1;
    return e;
  }
  static cudaError_t launch(const PassDesc& d, cudaStream_t s) {
    const int64_t tiles = (d.ncols / W) * d.nbatch;
    if (tiles <= 0) return cudaSuccess;
    CUtensorMap map;
    if (!col_tensor_map(d, W, sizeof(typename CxT<T>::type), &map)) return ColR16Cfg<T, W, W == 16 ? 2 : 3>::launch(d, s);
    const int64_t ncl = std::min<int64_t>(tiles, clusters);
    colfft4096_r16_tma_kernel<T, W, MINB><<<unsigned(ncl * 8), threads, smem(), s>>>(map, d);
    return cudaGetLastError();
  }
};

// Variants (selected by PassDesc::col_variant):
//   0: W = 16, U = 2, 512 threads, 2 CTAs/SM
//   1: W = 8,  U = 1, 512 threads, 3 CTAs/SM
//   2: W = 8,  U = 2, 256 threads, 4 CTAs/SM
//   3: W = 16, U = 1, 1024 threads, 1 CTA/SM
#define GBFFT_COL_TABLE(X) \
  X(0, float, 16, 2, 2)    \
  X(1, float, 8, 1, 3)     \
  X(2, float, 8, 2, 4)     \
  X(3, float, 16, 1, 1)

// push variants (st.async into the owner's receive buffer)
#define GBFFT_COLPUSH_TABLE(X) \
  X(4, float, 8, 2, 3)         \
  X(5, float, 8, 1, 3)         \
  X(6, float, 16, 2, 1)        \
  X(7, float, 8, 2, 2)

// radix-16 variants (W, min CTAs per SM)
#define GBFFT_COLR16_TABLE(X) \
  X(8, float, 8, 3)           \
  X(9, float, 16, 2)          \
  X(10, float, 8, 4)          \
  X(11, float, 16, 3)         \
  X(12, float, 32, 1)         \
  X(13, float, 16, 1)

// persistent tensor-fed radix-16 variants (W, min CTAs per SM)
#define GBFFT_COLR16TMA_TABLE(X) \
  X(14, float, 16, 1)            \
  X(15, float, 8, 3)

// lean radix-16 variants, Complex Float only (W, min CTAs per SM); 18 is the
// default: on the 4096 x 4096 column pass 73.7 us against 86.0 us for 9
// (16: 88.1, 19: 75.8-77.8, 17: 86.0, 10: 94.2, 8: 107.9)
#define GBFFT_COLR16B_TABLE(X) \
  X(16, 16, 2)                 \
  X(17, 8, 5)                  \
  X(18, 8, 4)                  \
  X(19, 8, 3)

}  // namespace

cudaError_t prepare_col_kernels() {
  cudaError_t e = cudaSuccess;
#define X(V, T, W, U, MINB) \
  if (e == cudaSuccess) e = ColCfg<T, W, U, MINB>::prepare();
  GBFFT_COL_TABLE(X)
#undef X
#define X(V, T, W, U, MINB) \
  if (e == cudaSuccess) e = ColPushCfg<T, W, U, MINB>::prepare();
  GBFFT_COLPUSH_TABLE(X)
#undef X
#define X(V, T, W, MINB) \
  if (e == cudaSuccess) e = ColR16Cfg<T, W, MINB>::prepare();
  GBFFT_COLR16_TABLE(X)
#undef X
#define X(V, T, W, MINB) \
  if (e == cudaSuccess) e = ColR16TmaCfg<T, W, MINB>::prepare();
  GBFFT_COLR16TMA_TABLE(X)
#undef X
#define X(V, W, MINB) \
  if (e == cudaSuccess) e = ColR16bCfg<W, MINB>::prepare();
  GBFFT_COLR16B_TABLE(X)
#undef X
  if (e == cudaSuccess) e = ColCfg<double, 16, 2, 1>::prepare();
  return e;
}

int col_tile_width(int variant) {
  switch (variant) {
    case 0: case 3: case 6: case 9: case 11: case 13: case 14: case 16: return 16;
    case 12: return 32;
    default: return 8;
  }
}

cudaError_t launch_col4096(const PassDesc& d, bool dbl, cudaStream_t s) {
  if (dbl) return ColCfg<double, 16, 2, 1>::launch(d, s);
#define X(V, T, W, U, MINB) \
  if (d.col_variant == V) return ColCfg<T, W, U, MINB>::launch(d, s);
  GBFFT_COL_TABLE(X)
#undef X
#define X(V, T, W, U, MINB) \
  if (d.col_variant == V) return ColPushCfg<T, W, U, MINB>::launch(d, s);
  GBFFT_COLPUSH_TABLE(X)
#undef X
#define X(V, T, W, MINB) \
  if (d.col_variant == V) return ColR16Cfg<T, W, MINB>::launch(d, s);
  GBFFT_COLR16_TABLE(X)
#undef X
#define X(V, T, W, MINB) \
  if (d.col_variant == V) return ColR16TmaCfg<T, W, MINB>::launch(d, s);
  GBFFT_COLR16TMA_TABLE(X)
#undef X
#define X(V, W, MINB) \
  if (d.col_variant == V) return ColR16bCfg<W, MINB>::launch(d, s);
  GBFFT_COLR16B_TABLE(X)
#undef X
  return cudaErrorInvalidValue;
}

}  // namespace gbfft
