// Bandwidth probe for the access pattern of the strided passes: a copy of a
// rows x cols Complex Float array in tiles of `width` contiguous columns
// (width * 8 bytes per row segment) over all rows.  A column pass that moves
// W-column tiles cannot run faster than this copy at the same W; the copy at
// width = cols is the contiguous (row pass) pattern.  Measurement support
// only: no transform calls it.
#include <cuda_runtime.h>

#include <algorithm>

#include "gbfft.h"
#include "gbfft_internal.h"

namespace gbfft {
namespace {

constexpr int kProbeThreads = 256;
constexpr int kProbeUnroll = 8;

// seg: float4 per row segment (width / 2); rs: rows per tile (64 KiB tiles)
__global__ void __launch_bounds__(kProbeThreads) tile_copy_kernel(const float4* __restrict__ in,
                                                                 float4* __restrict__ out, int64_t rows,
                                                                 int64_t row4, int seg, int rs) {
  const int64_t nsub = (rows + rs - 1) / rs;
  const int64_t ntiles = (row4 / seg) * nsub;
  const int items = seg * rs;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t cb = tile / nsub, sub = tile - cb * nsub;
    const int64_t r0 = sub * rs;
    const int64_t c4 = cb * seg;
    for (int f0 = threadIdx.x; f0 < items; f0 += kProbeThreads * kProbeUnroll) {
      float4 v[kProbeUnroll];
      int64_t off[kProbeUnroll];
#pragma unroll
      for (int u = 0; u < kProbeUnroll; ++u) {
        const int f = f0 + u * kProbeThreads;
        const int r = f / seg, c = f - r * seg;
        off[u] = (f < items && r0 + r < rows) ? (r0 + r) * row4 + c4 + c : -1;
      }
#pragma unroll
      for (int u = 0; u < kProbeUnroll; ++u)
        if (off[u] >= 0) v[u] = in[off[u]];
#pragma unroll
      for (int u = 0; u < kProbeUnroll; ++u)
        if (off[u] >= 0) out[off[u]] = v[u];
    }
  }
}

}  // namespace
}  // namespace gbfft

extern "C" int gbfft_probe_tile_copy(int64_t rows, int64_t cols, int width, const void* in, void* out,
                                     void* stream) {
  using namespace gbfft;
  if (rows < 1 || cols < 2 || width < 2 || width % 2 || cols % width || rows > (int64_t(1) << 40) / cols)
    return GBFFT_ERR_INVALID_ARG;
  if (!in || !out || in == out ||
      ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15))
    return GBFFT_ERR_INVALID_ARG;
  // segments above 8192 columns are copied as contiguous runs of at most
  // 64 KiB (a divisor of the segment), the same access pattern
  int seg = width / 2;
  if (seg > 4096) {
    int best = 1;
    for (int dv = 1; dv <= 4096; ++dv)
      if ((width / 2) % dv == 0) best = dv;
    seg = best;
  }
  const int rs = std::max(1, 4096 / seg);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t ntiles = (cols / 2 / seg) * ((rows + rs - 1) / rs);
  const int64_t grid = std::min<int64_t>(ntiles, int64_t(std::max(sms, 1)) * 8);
  tile_copy_kernel<<<unsigned(grid), kProbeThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const float4*>(in), static_cast<float4*>(out), rows, cols / 2, seg, rs);
  return cudaGetLastError() == cudaSuccess ? GBFFT_OK : GBFFT_ERR_CUDA;
}
