// Strided passes: transforms along an axis whose elements are es apart while
// neighbouring columns are adjacent (the y / z axes of fft2D / fft3D, the
// halves of four-step and four-pass Bluestein, the spectral product).
//
// Two kernels share the tile body of strided_tile.cuh:
//  * strfft_kernel: one tile of W columns per CTA, loaded straight from
//    global memory by the threads that transform it.
//  * strfft_tma_kernel: persistent CTAs.  A tile (W columns x N elements,
//    one 128-byte row segment per element index) is fetched into shared
//    memory by tiled tensor copies (cp.async.bulk.tensor, one per 256
//    element indices) completing on an mbarrier, double buffered, so the next tile streams in while the
//    current one is transformed: the plain kernel waits on its own loads
//    with nothing else in flight (long-scoreboard stalls dominated its
//    profile).  The tensor map is encoded on the host for every launch
//    (dims: columns in 8-byte words, element index, batch, outer batch);
//    passes whose layout the map cannot express (unaligned base or
//    strides, per-column offsets, zero-padded Bluestein loads) use the
//    plain kernel.  Waits are bounded and record GBFFT_ERR_TIMEOUT.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>

#include "butterflies.cuh"
#include "gbfft_internal.h"
#include "strided_tile.cuh"
#include "tma.cuh"

namespace gbfft {

namespace {

// Passes with a second in-register transform get more registers per thread.
template <typename T, int N, int W, int MINB, uint32_t OPS, int... Rs>
__global__ void __launch_bounds__(W*(N / 16), ((OPS & (F_SPEC | F_BLUE)) && MINB > 2) ? 2 : MINB)
    strfft_kernel(const PassDesc d) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  str_tile<T, N, W, OPS, Rs...>(d, int64_t(blockIdx.x), smem_raw);
}

// Resident CTAs per SM the tensor-fed kernel can have (shared memory: two
// tile buffers, alignment slack and barriers, of 227 KB), capped by MINB.
template <typename T, int N, int W, int MINB, uint32_t OPS>
constexpr int tma_minb() {
  constexpr int bytes = 128 + 2 * N * W * int(sizeof(T)) * 2 + 16;
  constexpr int fit = (227 * 1024) / bytes;
  constexpr int m = ((OPS & (F_SPEC | F_BLUE)) && MINB > 2) ? 2 : MINB;
  return fit < 1 ? 1 : (fit < m ? fit : m);
}

// rank: 2 (one batch), 3 (batch), 4 (batch and outer batch) -- the
// dimensions of `tmap`, whose box is W columns x N element indices.
template <typename T, int N, int W, int MINB, uint32_t OPS, int... Rs>
__global__ void __launch_bounds__(W*(N / 16), (tma_minb<T, N, W, MINB, OPS>()))
    strfft_tma_kernel(const __grid_constant__ CUtensorMap tmap, const PassDesc d, const int rank) {
  using C = typename CxT<T>::type;
  constexpr int E = 16;
  constexpr int TH = N / E;
  constexpr int TILE = N * W;
  constexpr int K = int(sizeof(C) / 8);  // 8-byte words per element
  constexpr uint32_t kBytes = uint32_t(TILE * sizeof(C));
  constexpr int NBOX = N > 256 ? N / 256 : 1;  // boxes per tile (a box spans <= 256 indices)
  constexpr int BOXN = N / NBOX;
  constexpr int R0 = rl_first(RL<Rs...>{});
  // dynamic shared memory only: [pad to 128 B][tile buffer 0][tile buffer 1]
  // [2 mbarriers]; a tensor copy's shared destination must be 128-byte
  // aligned, which the start of dynamic shared memory does not promise
  extern __shared__ unsigned char smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  C* buf0 = reinterpret_cast<C*>(smem_raw + ((128u - (raw & 127u)) & 127u));
  uint64_t* bars = reinterpret_cast<uint64_t*>(buf0 + 2 * TILE);
  const int64_t tiles = (d.ncols + W - 1) / W;
  const int64_t total = tiles * d.nbatch;
  // alignment self-check (uniform across the CTA): the buffers must be
  // 128-byte aligned and the tensor map 64-byte aligned, else report and
  // issue no copy
  if ((smem_u32(buf0) & 127u) != 0 || (reinterpret_cast<uint64_t>(&tmap) & 63u) != 0) {
    if (threadIdx.x == 0 && d.status) atomicExch(d.status, GBFFT_ERR_INTERNAL_DEVICE);
    return;
  }

  auto issue = [&](int64_t tile, int b) {
    const int64_t bq = tile / tiles;
    const int64_t c0 = (tile - bq * tiles) * W;
    const int64_t b_hi = bq / d.nb_lo;
    const int64_t b_lo = bq - b_hi * d.nb_lo;
    mbar_expect_tx(&bars[b], kBytes);
    // c0 is a multiple of W, so the innermost coordinate is 16-byte aligned
#pragma unroll
    for (int j = 0; j < NBOX; ++j)
      tma_load_tile(buf0 + b * TILE + j * BOXN * W, &tmap, rank, int(c0 * K), j * BOXN, int(b_lo), int(b_hi),
                    &bars[b]);
  };

  if (threadIdx.x == 0) {
    prefetch_tensormap(&tmap);
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < 2; ++k) {
      const int64_t tile = int64_t(blockIdx.x) + int64_t(k) * gridDim.x;
      if (tile < total) issue(tile, k);
    }
  }
  const float csign_in = (d.flags & F_CONJ_IN) ? -1.0f : 1.0f;
  int it = 0;
  for (int64_t tile = blockIdx.x; tile < total; tile += gridDim.x, ++it) {
    const int b = it & 1;
    const uint32_t par = uint32_t(it >> 1) & 1u;
    const bool timed_out = !mbar_wait_bounded(&bars[b], par, d.status);
    if (__syncthreads_or(timed_out)) break;
    const StrCtx c = str_ctx<N, W>(d, tile);
    C* sb = buf0 + b * TILE;
    C v[E];
#pragma unroll
    for (int q = 0; q < E / R0; ++q)
#pragma unroll
      for (int r = 0; r < R0; ++r) {
        const int m = q + r * (E / R0);
        C e = sb[(c.t + TH * m) * W + c.x];
        e.y *= T(csign_in);
        v[q * R0 + r] = e;
      }
    __syncthreads();  // inputs consumed: the tile buffer becomes the exchange buffer
    str_finish<T, N, W, OPS, Rs...>(d, c, v, sb);
    __syncthreads();  // last exchange reads done: the buffer may be refilled
    if (threadIdx.x == 0) {
      const int64_t nt = tile + 2 * int64_t(gridDim.x);
      if (nt < total) {
        fence_async_smem();
        issue(nt, b);
      }
    }
  }
  // drain: do not exit with a tensor copy still targeting this CTA's smem
  if (threadIdx.x == 0) {
    int it2 = it;
    for (int k = 0; k < 2; ++k, ++it2) {
      const int64_t tile = int64_t(blockIdx.x) + int64_t(it2) * gridDim.x;
      if (tile < total) mbar_wait_bounded(&bars[it2 & 1], uint32_t(it2 >> 1) & 1u, d.status);
    }
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(tensor_map_encode_fn());
}

// Rank (2..4) of the tensor map str_tensor_map builds for this pass, or 0
// when the layout does not fit the tensor-copy rules (strides multiples of
// 16 bytes, box <= 256 per dimension, so N > 256 must be a multiple of
// 256); checks the layout alone.
int str_tma_rank(const PassDesc& d, int N, int W, size_t eb) {
  if (!d.use_tma || d.col_in_off || d.in_cs != 1 || (N > 256 && N % 256) || d.ncols < 1) return 0;
  if (d.flags & (F_PAD_IN | F_CHIRP_IN | F_BLUE)) return 0;
  const int64_t K = int64_t(eb / 8);
  if (int64_t(W) * K > 256) return 0;
  const int64_t nb_lo = std::max<int64_t>(d.nb_lo, 1);
  const int64_t nb_hi = (d.nbatch + nb_lo - 1) / nb_lo;
  const int rank = nb_hi > 1 ? 4 : nb_lo > 1 ? 3 : 2;
  const uint64_t es = uint64_t(d.in_es) * eb, bs = uint64_t(d.in_bs) * eb, bs2 = uint64_t(d.in_bs2) * eb;
  auto fits = [](uint64_t s) { return s > 0 && s % 16 == 0 && s < (uint64_t(1) << 40); };
  if (!fits(es)) return 0;
  if (nb_lo > 1 && !fits(bs)) return 0;
  if (rank >= 4 && !fits(bs2)) return 0;
  if (d.ncols * K > (int64_t(1) << 31) || nb_lo > (int64_t(1) << 31) || nb_hi > (int64_t(1) << 31)) return 0;
  return rank;
}

// Tensor map of a strided pass's input as (columns in 8-byte words, element
// index, batch, outer batch) with a box of W columns x N indices; returns its
// rank, or 0 (plain kernel) when the layout or the base address does not fit.
int str_tensor_map(const PassDesc& d, int N, int W, size_t eb, CUtensorMap* map) {
  const int rank = str_tma_rank(d, N, W, eb);
  if (rank == 0 || (reinterpret_cast<uintptr_t>(d.in) & 15)) return 0;
  const int64_t K = int64_t(eb / 8);
  const int64_t nb_lo = std::max<int64_t>(d.nb_lo, 1);
  const int64_t nb_hi = (d.nbatch + nb_lo - 1) / nb_lo;
  const uint64_t es = uint64_t(d.in_es) * eb, bs = uint64_t(d.in_bs) * eb, bs2 = uint64_t(d.in_bs2) * eb;
  auto fits = [](uint64_t s) { return s > 0 && s % 16 == 0 && s < (uint64_t(1) << 40); };
  auto fn = encode_fn();
  if (!fn) return 0;
  const cuuint64_t dims[4] = {cuuint64_t(d.ncols * K), cuuint64_t(N), cuuint64_t(nb_lo), cuuint64_t(nb_hi)};
  // a size-1 batch dimension below a larger one still needs a valid stride
  const cuuint64_t strides[3] = {es, fits(bs) ? bs : es, bs2};
  const cuuint32_t box[4] = {cuuint32_t(W * K), cuuint32_t(std::min(N, 256)), 1, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, cuuint32_t(rank), const_cast<void*>(d.in), dims,
                        strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? rank : 0;
}

int g_str_sms = 0;

// Fused-operation sets the tensor-fed kernel is built for (no zero padding
// or chirp on load).
constexpr int tma_slot(uint32_t ops) {
  return ops == SO_PLAIN ? 0 : ops == SO_TW4 ? 1 : ops == SO_TW4B ? 2 : ops == SO_FILT ? 3 : ops == SO_COUT ? 4
       : ops == SO_SPEC ? 5 : ops == SO_BMID ? 6 : -1;
}

template <typename T, int N, int W, int MINB, bool TMA, int... Rs>
struct StrCfg {
  static constexpr int threads = W * (N / 16);
  static size_t smem() { return size_t(N) * W * sizeof(typename CxT<T>::type); }
  // tensor-fed kernel: alignment slack, two tile buffers, two mbarriers
  static size_t tma_smem() { return 128 + 2 * smem() + 2 * sizeof(uint64_t); }
  [[maybe_unused]] static inline int tma_ctas[7] = {0, 0, 0, 0, 0, 0, 0};  // resident CTAs per SM, tensor-fed
  template <uint32_t OPS>
  static cudaError_t prep1() {
    cudaError_t e = cudaFuncSetAttribute(strfft_kernel<T, N, W, MINB, OPS, Rs...>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem()));
    if constexpr (TMA && tma_slot(OPS) >= 0) {
      auto k = strfft_tma_kernel<T, N, W, MINB, OPS, Rs...>;
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(tma_smem()));
      int nb = 0;
      if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, threads, tma_smem());
      tma_ctas[tma_slot(OPS)] = nb > 0 ? nb : 1;
    }
    return e;
  }
  static cudaError_t prepare() {
    cudaError_t e = prep1<SO_PLAIN>();
    if (e == cudaSuccess) e = prep1<SO_TW4>();
    if (e == cudaSuccess) e = prep1<SO_TW4B>();
    if (e == cudaSuccess) e = prep1<SO_BP1>();
    if (e == cudaSuccess) e = prep1<SO_FILT>();
    if (e == cudaSuccess) e = prep1<SO_COUT>();
    if (e == cudaSuccess) e = prep1<SO_SPEC>();
    if (e == cudaSuccess) e = prep1<SO_BLUE>();
    if (e == cudaSuccess) e = prep1<SO_BMID>();
    return e;
  }
  template <uint32_t OPS>
  static cudaError_t go(const PassDesc& d, cudaStream_t s) {
    const int64_t tiles = (d.ncols + W - 1) / W;
    const int64_t total = tiles * d.nbatch;
    if (total <= 0) return cudaSuccess;
    if constexpr (TMA && tma_slot(OPS) >= 0) {
      CUtensorMap map;
      const int rank = str_tensor_map(d, N, W, sizeof(typename CxT<T>::type), &map);
      if (rank > 0) {
        const int sms = g_str_sms > 0 ? g_str_sms : 1;
        const int64_t grid = std::min<int64_t>(total, int64_t(sms) * tma_ctas[tma_slot(OPS)]);
        strfft_tma_kernel<T, N, W, MINB, OPS, Rs...><<<unsigned(grid), threads, tma_smem(), s>>>(map, d, rank);
        return cudaGetLastError();
      }
    }
    strfft_kernel<T, N, W, MINB, OPS, Rs...><<<unsigned(total), threads, smem(), s>>>(d);
    return cudaGetLastError();
  }
  static cudaError_t launch(const PassDesc& d, cudaStream_t s) {
    switch (d.flags & kStrOpMask) {
      case SO_PLAIN: return go<SO_PLAIN>(d, s);
      case SO_TW4: return go<SO_TW4>(d, s);
      case SO_TW4B: return go<SO_TW4B>(d, s);
      case SO_BP1: return go<SO_BP1>(d, s);
      case SO_FILT: return go<SO_FILT>(d, s);
      case SO_COUT: return go<SO_COUT>(d, s);
      case SO_SPEC: return go<SO_SPEC>(d, s);
      case SO_BLUE: return go<SO_BLUE>(d, s);
      case SO_BMID: return go<SO_BMID>(d, s);
      default: return cudaErrorInvalidValue;
    }
  }
};

// (type, N, W, min CTAs per SM, tensor-fed variant, radices = factor_device(N))
#define GBFFT_STR_TABLE(X)                 \
  X(float, 256, 16, 3, true, 16, 16)       \
  X(float, 512, 16, 2, true, 16, 16, 2)    \
  X(float, 1024, 16, 1, false, 16, 16, 4)  \
  X(float, 128, 16, 6, true, 16, 8)        \
  X(float, 64, 16, 8, true, 16, 4)         \
  X(double, 256, 8, 2, true, 16, 16)       \
  X(double, 512, 8, 1, false, 16, 16, 2)   \
  X(double, 1024, 8, 1, false, 16, 16, 4)

}  // namespace

void* tensor_map_encode_fn() {
  static void* fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return f;
  }();
  return fn;
}

bool str_kernel_available(int n, bool dbl) {
#define X(T, N, W, MINB, TMA, ...) \
  if (n == N && dbl == (sizeof(T) == 8)) return true;
  GBFFT_STR_TABLE(X)
#undef X
  return false;
}

int str_kernel_width(bool dbl) { return dbl ? 8 : 16; }

const char* str_kernel_name(const PassDesc& d, bool dbl) {
#define X(T, N, W, MINB, TMA, ...)                                                       \
  if (d.n == N && dbl == (sizeof(T) == 8) && TMA && tma_slot(d.flags & kStrOpMask) >= 0 && \
      str_tma_rank(d, N, W, sizeof(typename CxT<T>::type)) > 0)                          \
    return "strfft_tma_kernel";
  GBFFT_STR_TABLE(X)
#undef X
  return "strfft_kernel";
}

cudaError_t prepare_str_kernels() {
  cudaError_t e = cudaSuccess;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&g_str_sms, cudaDevAttrMultiProcessorCount, dev);
#define X(T, N, W, MINB, TMA, ...) \
  if (e == cudaSuccess) e = StrCfg<T, N, W, MINB, TMA, __VA_ARGS__>::prepare();
  GBFFT_STR_TABLE(X)
#undef X
  return e;
}

cudaError_t launch_str(const PassDesc& d, bool dbl, cudaStream_t s) {
#define X(T, N, W, MINB, TMA, ...) \
  if (d.n == N && dbl == (sizeof(T) == 8)) return StrCfg<T, N, W, MINB, TMA, __VA_ARGS__>::launch(d, s);
  GBFFT_STR_TABLE(X)
#undef X
  return cudaErrorInvalidValue;
}

}  // namespace gbfft
