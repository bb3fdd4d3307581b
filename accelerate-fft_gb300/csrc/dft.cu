// Naive DFT with caller-supplied roots of unity, as the reference defines it
// (Data.Array.Accelerate.Math.DFT, DFT.hs:68-111) -- for single bins and tiny
// lengths, where a transform plan does not pay off -- and the centring and
// shifting helpers of Math.DFT.Centre.
//
// dftG roots arr: the reference extends the input with one more axis of
// length shapeSize(arr) and folds along it, so every output element
// (sh_o :. k) is the sum over ALL input elements (sh :. n) of
// arr[sh :. n] * roots[sh :. (k*n) mod l].  For a vector this is the DFT;
// for rank > 1 every output row holds the same values (the transform of the
// rows' sum, each row weighted by its own roots).  dftGS ix roots arr is one
// of those values, k = indexHead ix (foldAll).
//
// GPU form: one CTA per frequency k (grid-stride over k) sums over all
// elements row by row, keeping (k*n) mod l incrementally; a warp-shuffle and
// shared-memory reduction gives the bin, written to the output's first row;
// a second kernel copies that row to the others.  No allocation.
#include <cuda_runtime.h>

#include "butterflies.cuh"
#include "gbfft.h"
#include "gbfft_internal.h"

namespace gbfft {
namespace {

constexpr int kDftThreads = 256;

template <typename C>
__device__ __forceinline__ C warp_sum(C v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_down_sync(0xffffffffu, v.x, o);
    v.y += __shfl_down_sync(0xffffffffu, v.y, o);
  }
  return v;
}

// sum over every element of roots[r*l + (k*n) mod l] * x[r*l + n]
template <typename T>
__device__ typename CxT<T>::type bin_sum(const typename CxT<T>::type* __restrict__ roots,
                                         const typename CxT<T>::type* __restrict__ x, int64_t rows, int64_t l,
                                         int64_t k) {
  using C = typename CxT<T>::type;
  __shared__ C part[kDftThreads / 32];
  C acc = cmake<C>(T(0), T(0));
  const int64_t step = (k * int64_t(blockDim.x)) % l;  // (k*n) mod l advances by this per iteration
  for (int64_t r = 0; r < rows; ++r) {
    const C* xr = x + r * l;
    const C* rr = roots + r * l;
    int64_t m = (k * int64_t(threadIdx.x)) % l;
    for (int64_t n = threadIdx.x; n < l; n += blockDim.x) {
      acc = cadd(acc, cmul(xr[n], rr[m]));
      m += step;
      if (m >= l) m -= l;
    }
  }
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  C tot = cmake<C>(T(0), T(0));
  if (threadIdx.x < 32) {
    tot = threadIdx.x < blockDim.x / 32 ? part[threadIdx.x] : cmake<C>(T(0), T(0));
    tot = warp_sum(tot);
  }
  __syncthreads();  // part is reused by the next bin
  return tot;  // valid in thread 0
}

template <typename T>
__global__ void __launch_bounds__(kDftThreads) dftg_kernel(const typename CxT<T>::type* roots,
                                                           const typename CxT<T>::type* x,
                                                           typename CxT<T>::type* out, int64_t rows, int64_t l) {
  using C = typename CxT<T>::type;
  for (int64_t k = blockIdx.x; k < l; k += gridDim.x) {
    const C s = bin_sum<T>(roots, x, rows, l, k);
    if (threadIdx.x == 0) out[k] = s;
  }
}

template <typename T>
__global__ void dftg_broadcast_kernel(typename CxT<T>::type* out, int64_t rows, int64_t l) {
  const int64_t total = (rows - 1) * l;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x)
    out[l + i] = out[i % l];
}

template <typename T>
__global__ void __launch_bounds__(kDftThreads) dftgs_kernel(int64_t k, const typename CxT<T>::type* roots,
                                                            const typename CxT<T>::type* x,
                                                            typename CxT<T>::type* out, int64_t rows, int64_t l) {
  using C = typename CxT<T>::type;
  const C s = bin_sum<T>(roots, x, rows, l, k);
  if (threadIdx.x == 0) out[0] = s;
}

// Centre.hs (DFT/Centre.hs:36-164) for rank 1..3, dims outermost-first:
//   centre: out(z, y, x) = (-1)^(z + y + x) * in(z, y, x)
//   shift:  out(z, y, x) = in((z + sd) mod d, (y + sh) mod h, (x + sw) mod w)
// with s = n/2 + (n odd) for shift, n/2 for ishift, per axis.  One pass,
// grid-stride over the output, the multi-index from two divisions.
struct Dims3 {
  int64_t d, h, w;
  int64_t sd, sh, sw;
};

template <typename C>
__global__ void centre_kernel(const C* __restrict__ in, C* __restrict__ out, Dims3 g) {
  const int64_t total = g.d * g.h * g.w;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t x = i % g.w, yz = i / g.w, y = yz % g.h, z = yz / g.h;
    C v = in[i];
    if ((x + y + z) & 1) {
      v.x = -v.x;
      v.y = -v.y;
    }
    out[i] = v;
  }
}

template <typename C>
__global__ void shift_kernel(const C* __restrict__ in, C* __restrict__ out, Dims3 g) {
  const int64_t total = g.d * g.h * g.w;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t x = i % g.w, yz = i / g.w, y = yz % g.h, z = yz / g.h;
    int64_t xs = x + g.sw, ys = y + g.sh, zs = z + g.sd;
    if (xs >= g.w) xs -= g.w;
    if (ys >= g.h) ys -= g.h;
    if (zs >= g.d) zs -= g.d;
    out[i] = in[(zs * g.h + ys) * g.w + xs];
  }
}

int dims3(int rank, const int64_t* dims, Dims3& g) {
  if (rank < 1 || rank > 3 || !dims) return GBFFT_ERR_INVALID_ARG;
  int64_t e[3] = {1, 1, 1};
  for (int i = 0; i < rank; ++i) {
    if (dims[i] < 0) return GBFFT_ERR_INVALID_ARG;
    e[3 - rank + i] = dims[i];
  }
  g.d = e[0];
  g.h = e[1];
  g.w = e[2];
  return GBFFT_OK;
}

unsigned grid_for(int64_t total) {
  const int64_t b = (total + 255) / 256;
  return unsigned(b < 8192 ? (b > 0 ? b : 1) : 8192);
}

int shape_rows(int rank, const int64_t* dims, int64_t& rows, int64_t& l) {
  if (rank < 1 || rank > 5 || !dims) return GBFFT_ERR_INVALID_ARG;
  rows = 1;
  for (int i = 0; i < rank - 1; ++i) {
    if (dims[i] < 0) return GBFFT_ERR_INVALID_ARG;
    rows *= dims[i];
  }
  l = dims[rank - 1];
  return l < 0 ? GBFFT_ERR_INVALID_ARG : GBFFT_OK;
}

}  // namespace
}  // namespace gbfft

using namespace gbfft;

extern "C" {

int gbfft_dftG(int rank, const int64_t* dims, int dtype, const void* d_roots, const void* d_in, void* d_out,
               void* stream) {
  int64_t rows = 0, l = 0;
  int st = shape_rows(rank, dims, rows, l);
  if (st != GBFFT_OK) return st;
  if (dtype != GBFFT_C32 && dtype != GBFFT_C64) return GBFFT_ERR_INVALID_ARG;
  if (rows == 0 || l == 0) return GBFFT_OK;
  if (!d_roots || !d_in || !d_out || d_out == d_in || d_out == d_roots) return GBFFT_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const unsigned grid = unsigned(l < 4096 ? l : 4096);
  const int64_t bcast = (rows - 1) * l;  // elements the broadcast writes
  const unsigned bgrid = unsigned(bcast > 0 ? (bcast + 255) / 256 < 4096 ? (bcast + 255) / 256 : 4096 : 1);
  if (dtype == GBFFT_C64) {
    dftg_kernel<double><<<grid, kDftThreads, 0, s>>>(static_cast<const double2*>(d_roots),
                                                     static_cast<const double2*>(d_in), static_cast<double2*>(d_out),
                                                     rows, l);
    if (rows > 1) dftg_broadcast_kernel<double><<<bgrid, 256, 0, s>>>(static_cast<double2*>(d_out), rows, l);
  } else {
    dftg_kernel<float><<<grid, kDftThreads, 0, s>>>(static_cast<const float2*>(d_roots),
                                                    static_cast<const float2*>(d_in), static_cast<float2*>(d_out),
                                                    rows, l);
    if (rows > 1) dftg_broadcast_kernel<float><<<bgrid, 256, 0, s>>>(static_cast<float2*>(d_out), rows, l);
  }
  return cudaGetLastError() == cudaSuccess ? GBFFT_OK : GBFFT_ERR_CUDA;
}

int gbfft_dftGS(int rank, const int64_t* dims, int dtype, int64_t k, const void* d_roots, const void* d_in,
                void* d_out, void* stream) {
  int64_t rows = 0, l = 0;
  int st = shape_rows(rank, dims, rows, l);
  if (st != GBFFT_OK) return st;
  if (dtype != GBFFT_C32 && dtype != GBFFT_C64) return GBFFT_ERR_INVALID_ARG;
  if (!d_out) return GBFFT_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (rows == 0 || l == 0) {
    // the sum over no elements
    return cudaMemsetAsync(d_out, 0, dtype == GBFFT_C64 ? 16 : 8, s) == cudaSuccess ? GBFFT_OK : GBFFT_ERR_CUDA;
  }
  if (k < 0 || !d_roots || !d_in) return GBFFT_ERR_INVALID_ARG;
  k %= l;
  if (dtype == GBFFT_C64)
    dftgs_kernel<double><<<1, kDftThreads, 0, s>>>(k, static_cast<const double2*>(d_roots),
                                                   static_cast<const double2*>(d_in), static_cast<double2*>(d_out),
                                                   rows, l);
  else
    dftgs_kernel<float><<<1, kDftThreads, 0, s>>>(k, static_cast<const float2*>(d_roots),
                                                  static_cast<const float2*>(d_in), static_cast<float2*>(d_out),
                                                  rows, l);
  return cudaGetLastError() == cudaSuccess ? GBFFT_OK : GBFFT_ERR_CUDA;
}

int gbfft_centre(int rank, const int64_t* dims, int dtype, const void* d_in, void* d_out, void* stream) {
  Dims3 g{};
  int st = dims3(rank, dims, g);
  if (st != GBFFT_OK) return st;
  if (dtype != GBFFT_C32 && dtype != GBFFT_C64) return GBFFT_ERR_INVALID_ARG;
  const int64_t total = g.d * g.h * g.w;
  if (total == 0) return GBFFT_OK;
  if (!d_in || !d_out) return GBFFT_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dtype == GBFFT_C64)
    centre_kernel<double2><<<grid_for(total), 256, 0, s>>>(static_cast<const double2*>(d_in),
                                                          static_cast<double2*>(d_out), g);
  else
    centre_kernel<float2><<<grid_for(total), 256, 0, s>>>(static_cast<const float2*>(d_in),
                                                         static_cast<float2*>(d_out), g);
  return cudaGetLastError() == cudaSuccess ? GBFFT_OK : GBFFT_ERR_CUDA;
}

int gbfft_shift(int rank, const int64_t* dims, int dtype, int inverse, const void* d_in, void* d_out,
                void* stream) {
  Dims3 g{};
  int st = dims3(rank, dims, g);
  if (st != GBFFT_OK) return st;
  if (dtype != GBFFT_C32 && dtype != GBFFT_C64) return GBFFT_ERR_INVALID_ARG;
  const int64_t total = g.d * g.h * g.w;
  if (total == 0) return GBFFT_OK;
  if (!d_in || !d_out || d_in == d_out) return GBFFT_ERR_INVALID_ARG;
  auto sft = [&](int64_t n) { return n / 2 + (inverse ? 0 : (n & 1)); };
  g.sd = sft(g.d);
  g.sh = sft(g.h);
  g.sw = sft(g.w);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dtype == GBFFT_C64)
    shift_kernel<double2><<<grid_for(total), 256, 0, s>>>(static_cast<const double2*>(d_in),
                                                         static_cast<double2*>(d_out), g);
  else
    shift_kernel<float2><<<grid_for(total), 256, 0, s>>>(static_cast<const float2*>(d_in),
                                                        static_cast<float2*>(d_out), g);
  return cudaGetLastError() == cudaSuccess ? GBFFT_OK : GBFFT_ERR_CUDA;
}

}  // extern "C"
