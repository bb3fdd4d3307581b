// One 1024-point Complex Double transform per 8-CTA thread-block cluster,
// one element per thread (8 x 128 threads): the latency path for single
// vectors and small batches (fft1D of one Complex Double vector).  On GB300
// an FP64 transform of this size in one CTA is bound by that SM's FP64 pipe
// and by the few warps a 1024-point transform keeps busy; spread over eight
// SMs every thread does five radix-2 butterflies per half.
//
// 1024 = 32 x 32, input index n = 32a + b, output index k = k1 + 32 k2:
//   phase 1:  warp b (CTA b / 4, warp b % 4), lane a holds x[32a + b]; a
//             radix-2 decimation-in-frequency DFT-32 over the lanes (values
//             exchanged by shuffles) leaves lane l with output k1 =
//             bitrev5(l); it is multiplied by W_1024^(b k1);
//   exchange: each value goes by st.async (16 bytes, completing on the
//             receiver's mbarrier; 2 KiB per CTA) to CTA k1 / 4, slot
//             [k1 % 4][b];
//   phase 2:  warp k1 % 4 of CTA k1 / 4, lane b: DFT-32 over the lanes, lane
//             l holds X[k1 + 32 bitrev5(l)], stored (with the pass's
//             conjugation, scale and output rotation).
// d.tw: W_1024^j, j < 1024 (Complex Double); W_32^m = W_1024^(32 m).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "butterflies.cuh"
#include "gbfft_internal.h"
#include "tma.cuh"

namespace cg = cooperative_groups;

namespace gbfft {
namespace {

constexpr int kVN = 1024;
constexpr int kVThreads = 128;
constexpr uint32_t kVRecvBytes = 128 * sizeof(double2);  // 4 k1 x 32 b
constexpr uint32_t kVWaitLimit = 1u << 22;

__device__ __forceinline__ int bitrev5(int l) { return int(__brev(unsigned(l)) >> 27); }

__device__ __forceinline__ double2 shfl_xor2(double2 v, int m) {
  return make_double2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

// The stage twiddles of one lane: tw[s] = W_{2h}^(lane mod h) for the stage
// of half-size h = 16 >> s (W_{2h}^j = W_32^(j 16/h) = W_1024^(32 j 16/h)),
// loaded once, before any is needed, and used by both DFTs of the lane.
struct LaneTw {
  double2 tw[4];
};
__device__ __forceinline__ LaneTw lane_twiddles(int lane, const double2* __restrict__ w1024) {
  LaneTw t;
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int h = 16 >> s;
    t.tw[s] = __ldg(w1024 + 32 * (lane & (h - 1)) * (16 / h));
  }
  return t;
}

// Radix-2 DIF DFT-32 across the lanes of a warp: lane l holds element l on
// entry and output bitrev5(l) on return.  Stage with half-size h: the lower
// lane of a pair keeps u + v, the upper (u - v) * W_{2h}^(l mod h).
__device__ __forceinline__ double2 dft32_lanes(double2 x, int lane, const LaneTw& t) {
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const int h = 16 >> s;
    const double2 p = shfl_xor2(x, h);
    if (lane & h) {
      const double2 dlt = make_double2(p.x - x.x, p.y - x.y);
      x = (s < 4 && (lane & (h - 1))) ? cmul(dlt, t.tw[s < 4 ? s : 0]) : dlt;
    } else {
      x = make_double2(x.x + p.x, x.y + p.y);
    }
  }
  return x;
}

__global__ void __cluster_dims__(8, 1, 1) __launch_bounds__(kVThreads) vec1024_kernel(const PassDesc d) {
  __shared__ __align__(16) double2 rv[128];  // [k1 % 4][b]
  __shared__ __align__(8) uint64_t rbar;
  const int r = int(cg::this_cluster().block_rank());
  const int64_t col = int64_t(blockIdx.x) >> 3;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const double2* __restrict__ w = static_cast<const double2*>(d.tw);
  const uint32_t fl = d.flags;
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&rbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // the mbarrier init is published by its own release fence
  asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");

  // ---- phase 1: warp b = 4r + warp, lane a -----------------------------------
  const int b = 4 * r + warp;
  const int k1 = bitrev5(lane);
  const double2* __restrict__ in = static_cast<const double2*>(d.in) + col * d.in_cs;
  // every load of the kernel is issued here, before any result is needed
  double2 x = in[32 * lane + b];
  const LaneTw lt = lane_twiddles(lane, w);
  const double2 wb = __ldg(w + ((b * k1) & (kVN - 1)));  // W_1024^(b k1)
  if (fl & F_CONJ_IN) x.y = -x.y;
  x = dft32_lanes(x, lane, lt);
  x = cmul(x, wb);
  if (tid == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&rbar)), "r"(kVRecvBytes)
                 : "memory");
  }
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
  {
    uint32_t dst, bar;
    const uint32_t ldst = smem_u32(&rv[(k1 & 3) * 32 + b]), lbar = smem_u32(&rbar);
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(dst) : "r"(ldst), "r"(uint32_t(k1 >> 2)));
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(bar) : "r"(lbar), "r"(uint32_t(k1 >> 2)));
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f64 [%0], {%1, %2}, [%3];" ::"r"(dst),
                 "d"(x.x), "d"(x.y), "r"(bar)
                 : "memory");
  }
  // ---- phase 2: warp = k1 % 4 of CTA k1 / 4, lane b --------------------------
  bool ok = false;
  for (uint32_t it = 0; it < kVWaitLimit && !ok; ++it) {
    uint32_t t;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(t)
        : "r"(smem_u32(&rbar))
        : "memory");
    ok = t != 0;
  }
  if (!ok && d.status) atomicExch(d.status, GBFFT_ERR_TIMEOUT_DEVICE);
  const int kk1 = 4 * r + warp;
  double2 y = rv[warp * 32 + lane];
  y = dft32_lanes(y, lane, lt);
  const int l = kk1 + 32 * bitrev5(lane);  // output index
  if (fl & F_SCALE) y = make_double2(y.x * d.scale, y.y * d.scale);
  if (fl & F_CONJ_OUT) y.y = -y.y;
  double2* __restrict__ out = static_cast<double2*>(d.out) + col * d.out_cs;
  out[l + rot_delta(d, l)] = y;
}

}  // namespace

bool vec1024_available(int64_t n, bool dbl) { return dbl && n == kVN; }

cudaError_t launch_vec1024(const PassDesc& d, cudaStream_t s) {
  if (d.ncols <= 0) return cudaSuccess;  // vectors d.ncols apart by in_cs / out_cs (nbatch 1)
  vec1024_kernel<<<unsigned(d.ncols * 8), kVThreads, 0, s>>>(d);
  return cudaGetLastError();
}

}  // namespace gbfft
