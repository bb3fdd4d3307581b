// Generic pencil pass: one CTA transforms a tile of W pencils (strided 1D
// sequences) of length n entirely in shared memory with Stockham
// autosort stages, fusing the pass's pre-operations (conjugate, Bluestein
// chirp, zero padding) into the load and its post-operations (four-step
// twiddle, Bluestein filter / chirp, 1/N scale, conjugate, truncation) into
// the store.  Every transform of the engine -- batched innermost axes,
// strided 2D/3D axes, four-step halves of long axes, Bluestein -- is a
// sequence of these passes.
#include "pencil_tile.cuh"

namespace gbfft {

template <typename T>
__global__ void __launch_bounds__(512) pencil_kernel(const PassDesc d) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pencil_tile<T>(d, int64_t(blockIdx.x), smem_raw);
}

size_t pass_smem_bytes(const PassDesc& d, bool is_double) {
  return size_t(2) * size_t(d.W) * size_t(d.pitch) * (is_double ? 16 : 8);
}

int pass_grid(const PassDesc& d) {
  const int64_t tiles = (d.ncols + d.W - 1) / d.W;
  return int(tiles * d.nbatch);
}

// Applies to the current device; called at every plan creation.
cudaError_t prepare_kernels() {
  cudaError_t e = prepare_row_kernels();
  if (e != cudaSuccess) return e;
  e = prepare_col_kernels();
  if (e != cudaSuccess) return e;
  e = prepare_row_tc_kernels();
  if (e != cudaSuccess) return e;
  e = prepare_str_kernels();
  if (e != cudaSuccess) return e;
  e = prepare_tcdft_kernels();
  if (e != cudaSuccess) return e;
  e = prepare_plane_kernels();
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(pencil_kernel<float>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(pencil_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              227 * 1024);
}

const char* pass_kernel_name(const PassDesc& d, bool dbl) {
  switch (d.kernel) {
    case K_ROW:
      if (d.flags & F_BLUE) return "rowblue_kernel";
      if (d.row_variant & 1) return "rowfft1_kernel";
      return (d.use_tma && d.in_cs == d.n && d.out_cs == d.n) ? "rowfft_tma_kernel" : "rowfft_kernel";
    case K_COL4096:
      return d.col_variant >= 16 ? "colfft4096_r16b_kernel"
           : (d.col_variant >= 14 && d.use_tma && d.in_cs == 1) ? "colfft4096_r16_tma_kernel"
           : d.col_variant >= 8 ? "colfft4096_r16_kernel"
           : d.col_variant >= 4 ? "colfft4096_push_kernel"
                                : "colfft4096_kernel";
    case K_ROW_TC: return "rowfft_tc_kernel";
    case K_TC_FOLD: return "tcdft_fold_kernel";
    case K_TC_DFT: return "tcdft_mma_kernel";
    case K_TC_DFT8: return "tcdft8_kernel";
    case K_PLANE: return "plane256_kernel";
    case K_VEC1024: return "vec1024_kernel";
    case K_STRIDED: return str_kernel_name(d, dbl);
    default: return "pencil_kernel";
  }
}

cudaError_t launch_pass(const PassDesc& d, bool is_double, cudaStream_t stream) {
  if (d.kernel == K_ROW) return launch_row(d, is_double, stream);
  if (d.kernel == K_COL4096) return launch_col4096(d, is_double, stream);
  if (d.kernel == K_ROW_TC) return launch_row_tc(d, stream);
  if (d.kernel == K_STRIDED) return launch_str(d, is_double, stream);
  if (d.kernel == K_TC_FOLD || d.kernel == K_TC_DFT || d.kernel == K_TC_DFT8) return launch_tcdft(d, stream);
  if (d.kernel == K_PLANE) return launch_plane(d, stream);
  if (d.kernel == K_VEC1024) return launch_vec1024(d, stream);
  const int grid = pass_grid(d);
  if (grid <= 0) return cudaSuccess;
  const size_t smem = pass_smem_bytes(d, is_double);
  if (is_double)
    pencil_kernel<double><<<grid, d.threads, smem, stream>>>(d);
  else
    pencil_kernel<float><<<grid, d.threads, smem, stream>>>(d);
  return cudaGetLastError();
}

}  // namespace gbfft
