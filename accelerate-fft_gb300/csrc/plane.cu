// Both axes of a 256 x 256 plane in one HBM round trip: the x and y passes of
// fft3D (and fft2D) on planes of that size, and the plane passes of the
// spectral convolution, fused.
//
// A plane of Complex Float (512 KiB) is split over an 8-CTA thread-block
// cluster, 64 KiB per CTA:
//   row phase:    CTA r loads rows [32r, 32r + 32) and transforms each row
//                 (256 = 16 x 16: DFT-16 over the stride-16 elements, twiddle
//                 W_256^(t*k1), one shared-memory exchange, DFT-16);
//   transpose:    after a cluster barrier (every CTA is done with its row
//                 exchange buffer), each thread pushes its 16 row outputs
//                 straight into the receive buffer [256 rows][32 columns] of
//                 the CTA that owns their column (columns [32r', 32r' + 32)
//                 belong to CTA r'), two columns per 16-byte distributed
//                 shared-memory store; a second cluster barrier publishes them;
//   column phase: CTA r' transforms its 32 columns the same way and writes
//                 them, each warp storing 32 consecutive columns of one row
//                 (256-byte segments).
// Loads are 128-byte row segments, stores 256-byte ones; nothing but the
// plane itself moves through HBM.  No thread waits on anything but the two
// cluster barriers and the CTA barriers.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "butterflies.cuh"
#include "gbfft_internal.h"
#include "tma.cuh"

namespace cg = cooperative_groups;

namespace gbfft {
namespace {

constexpr int kPN = 256;             // plane side
constexpr int kPCta = 8;             // CTAs per plane (the cluster)
constexpr int kPRows = kPN / kPCta;  // rows (and columns) per CTA: 32
constexpr int kPThreads = 512;       // 16 threads per row (column), 16 elements each
constexpr int kPPitch = 264;         // row-phase exchange pitch: the two rows of a warp 16 banks apart
constexpr size_t kPSmem = size_t(kPRows) * kPPitch * sizeof(float2) + size_t(kPN) * sizeof(float2);
static_assert(size_t(kPRows) * kPPitch >= size_t(kPN) * kPRows, "receive buffer fits the exchange region");

__device__ __forceinline__ uint32_t mapa_rank(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ void st_cluster2(uint32_t addr, float2 a, float2 b) {
  asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(a.x), "f"(a.y), "f"(b.x),
               "f"(b.y)
               : "memory");
}
__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// d.in / d.out: planes of 256 x 256 (row stride 256), plane p at p * in_bs /
// p * out_bs; d.ncols planes; d.tw: W_256^j, j < 256.  Flags: F_CONJ_IN on
// load, F_SCALE (by d.scale) and F_CONJ_OUT on store.
__global__ void __cluster_dims__(kPCta, 1, 1) __launch_bounds__(kPThreads, 2) plane256_kernel(const PassDesc d) {
  extern __shared__ __align__(16) float2 psm[];
  float2* ex = psm;                     // row exchange [32][kPPitch], then receive buffer [256][32]
  float2* wt = psm + kPRows * kPPitch;  // [k1][t]: W_256^(t*k1), t, k1 < 16 (t fastest: no bank conflicts)
  const uint32_t r = cg::this_cluster().block_rank();
  const int64_t plane = int64_t(blockIdx.x) / kPCta;
  const float2* __restrict__ in = static_cast<const float2*>(d.in) + plane * d.in_bs;
  float2* __restrict__ out = static_cast<float2*>(d.out) + plane * d.out_bs;
  const float2* __restrict__ tw = static_cast<const float2*>(d.tw);
  const uint32_t fl = d.flags;
  const int tid = threadIdx.x;
  if (tid < kPN) wt[tid] = tw[((tid & 15) * (tid >> 4)) & (kPN - 1)];

  // ---- row phase: thread (lr, t), row 32r + lr, elements t + 16i ---------------
  const int lr = tid >> 4, t = tid & 15;
  float2 v[16];
  {
    const float2* src = in + int64_t(kPRows * r + lr) * kPN + t;
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = src[16 * i];
  }
  if (fl & F_CONJ_IN) {
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i].y = -v[i].y;
  }
  __syncthreads();  // twiddle table
  dft16(v);
#pragma unroll
  for (int k1 = 1; k1 < 16; ++k1) v[k1] = cmul(v[k1], wt[16 * k1 + t]);
  {
    float2* row = ex + lr * kPPitch;
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) row[k1 * 16 + (t ^ k1)] = v[k1];
    __syncthreads();
    // thread t now takes k1 = t: the 16 values of that k1 over the row's t'
#pragma unroll
    for (int tp = 0; tp < 16; ++tp) v[tp] = row[t * 16 + (tp ^ t)];
  }
  dft16(v);  // v[k2] = X[row][t + 16 k2]
  // every CTA of the cluster is done with its exchange buffer
  cluster_barrier();

  // ---- transpose: columns t + 32q and t + 16 + 32q (k2 = 2q, 2q + 1) live in
  // CTA q, whose receive buffer [256 rows][32] keeps column t + 16b of its
  // chunk at slot 2t + b, so the pair goes over as one 16-byte store
  {
    const uint32_t base = smem_u32(ex);
    const int grow = kPRows * int(r) + lr;
    const uint32_t local = base + uint32_t((grow * kPRows + 2 * t) * sizeof(float2));
#pragma unroll
    for (int q = 0; q < 8; ++q) st_cluster2(mapa_rank(local, uint32_t(q)), v[2 * q], v[2 * q + 1]);
  }
  cluster_barrier();  // the receive buffers are complete

  // ---- column phase: thread (c, tc), local column c, rows tc + 16i ---------------
  const int c = tid & 31, tc = tid >> 5;
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = ex[(tc + 16 * i) * kPRows + c];
  __syncthreads();  // every read of the receive buffer is done before the exchange reuses it
  dft16(v);
#pragma unroll
  for (int k1 = 1; k1 < 16; ++k1) v[k1] = cmul(v[k1], wt[16 * k1 + tc]);
#pragma unroll
  for (int k1 = 0; k1 < 16; ++k1) ex[(k1 * 16 + tc) * kPRows + c] = v[k1];
  __syncthreads();
#pragma unroll
  for (int tp = 0; tp < 16; ++tp) v[tp] = ex[(tc * 16 + tp) * kPRows + c];
  dft16(v);  // v[k2] = Y[row tc + 16 k2][column 32r + c]
  const float s = float(d.scale);
  float2* dst = out + int64_t(kPRows) * r + (c >> 1) + 16 * (c & 1);  // slot c holds column (c >> 1) + 16 (c & 1)
#pragma unroll
  for (int k2 = 0; k2 < 16; ++k2) {
    float2 x = v[k2];
    if (fl & F_SCALE) x = cscale(x, s);
    if (fl & F_CONJ_OUT) x.y = -x.y;
    dst[int64_t(tc + 16 * k2) * kPN] = x;
  }
}

}  // namespace

bool plane_available(int64_t h, int64_t w, bool dbl) { return !dbl && h == kPN && w == kPN; }

cudaError_t prepare_plane_kernels() {
  return cudaFuncSetAttribute(plane256_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kPSmem));
}

cudaError_t launch_plane(const PassDesc& d, cudaStream_t s) {
  if (d.ncols <= 0) return cudaSuccess;
  plane256_kernel<<<unsigned(d.ncols * kPCta), kPThreads, kPSmem, s>>>(d);
  return cudaGetLastError();
}

}  // namespace gbfft
