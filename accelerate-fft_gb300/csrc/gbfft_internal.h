// Internal declarations shared by the host planner and the device kernels.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace gbfft {

constexpr int kMaxStages = 16;

// Value a kernel writes into a plan's device status word when a bounded wait
// gives up (equals GBFFT_ERR_TIMEOUT of the C ABI).
constexpr int GBFFT_ERR_TIMEOUT_DEVICE = 6;
// ... when a kernel's own alignment check fails (GBFFT_ERR_INTERNAL).
constexpr int GBFFT_ERR_INTERNAL_DEVICE = 7;

// Largest transform length one CTA computes in shared memory (two ping-pong
// buffers of one column each); longer axes are split four-step.
constexpr int kCapC32 = 8192;
// Longest row the split-FP16 dense-DFT kernels take (folded length 1025).
constexpr int kTcDftMaxN = 2048;
constexpr int kCapC64 = 4096;

// Pre- and post-operations fused into a pencil pass.
enum PassFlags : uint32_t {
  F_CONJ_IN = 1u << 0,     // conjugate every loaded element (backward via forward)
  F_CONJ_OUT = 1u << 1,    // conjugate every stored element
  F_SCALE = 1u << 2,       // multiply stored elements by `scale` (Inverse 1/N)
  F_TW4 = 1u << 3,         // four-step twiddle W_N^{e*k} on store
  F_TW4_BATCH = 1u << 4,   //   ... exponent multiplier e = batch index (else column)
  F_CHIRP_IN = 1u << 5,    // x[l] * chirp[l] on load (l = logical input index)
  F_PAD_IN = 1u << 6,      // zero for logical input index l >= n_in
  F_BLUE = 1u << 7,        // in-kernel Bluestein: filter, inverse, chirp on store
  F_FILTER_OUT = 1u << 8,  // multiply by filter[l] then conjugate, on store
  F_CHIRP_OUT = 1u << 9,   // conjugate then multiply by chirp[l] on store
  F_TRUNC_OUT = 1u << 10,  // store only logical output index l < n_out
  F_SPEC = 1u << 11,       // in-kernel spectral multiply: DFT, * filter[l], conj, DFT
  F_L2_IN_FIRST = 1u << 12,  // loads: L2 evict_first (input read once)
  F_L2_OUT_LAST = 1u << 13,  // stores: L2 evict_last (a later pass reads them back)
  F_ROT_OUT = 1u << 14,      // stores: output index l along the axis goes to (l - rot_s) mod rot_n
};

// Kernel families a pass can run on.
enum KernelId : int {
  K_PENCIL = 0,   // generic shared-memory pencil kernel (any length <= cap, fused ops)
  K_ROW = 1,      // register-resident contiguous-row kernel (specialised lengths)
  K_COL4096 = 2,  // 8-CTA cluster kernel for stride-S axes of length 4096
  K_ROW_TC = 3,   // contiguous rows, radix-16 stages as split-FP16 tensor-core GEMMs
  K_STRIDED = 4,  // register-resident strided pencils, W adjacent columns per CTA
  K_TC_FOLD = 5,  // split-FP16 dense DFT, step 1: fold rows into hi/lo FP16 operand tiles
  K_TC_DFT = 6,   // split-FP16 dense DFT, step 2: tcgen05 GEMM against cos/sin tiles
  K_TC_DFT8 = 7,  // split-FP16 rows n = 8 * n2: radix-8 on the CUDA cores, dense n2 stage on tcgen05
  K_PLANE = 8,    // both axes of 256 x 256 planes in one pass (8-CTA cluster per plane)
  K_VEC1024 = 9,  // one 1024-point Complex Double vector per 8-CTA cluster, one element per thread
};

struct StageInfo {
  int radix;   // 2, 3, 4, 5, 7, 8 or 16
  int ns;      // product of the radices of earlier stages (Stockham Ns)
  int tw_off;  // offset of this stage's twiddles in the stage table
};

// One pencil pass: for each (batch b, column c) transform the pencil
// i -> base + b_lo*bs + b_hi*bs2 + c*cs + i*es of length n, in shared
// memory, where b = b_hi*nb_lo + b_lo.
struct PassDesc {
  const void* in;
  void* out;
  int64_t in_es, in_cs, in_bs, in_bs2;
  int64_t out_es, out_cs, out_bs, out_bs2;
  int64_t ncols;   // columns per batch
  int64_t nbatch;  // batches (nb_lo * number of b_hi)
  int64_t nb_lo;   // extent of the inner batch index
  int n;           // transform length computed in shared memory
  int W;           // columns per CTA tile
  int pitch;       // shared-memory column pitch (elements, odd)
  int threads;     // CTA size
  int nstages;
  int load_cfast;   // 1: loads map consecutive threads to consecutive columns
  int store_cfast;  // 1: stores map consecutive threads to consecutive columns
  uint32_t flags;
  int kernel;   // KernelId
  int use_tma;  // K_ROW: stream chunks with cp.async.bulk when the layout allows
  int row_variant;  // K_ROW: 0 double-buffered exchanges, 1 single buffer (more CTAs/SM)
  int col_variant;  // K_COL4096: tile width / threads variant (colfft.cu)
  int* status;  // device status word of the plan (0 = ok)
  StageInfo st[kMaxStages];
  const void* tw;  // stage twiddles (element type of the pass)
  double scale;
  // logical index used by chirp / pad / filter / truncation:
  //   l_in = i*lin_es + c*lin_cs,  l_out = k*lout_es + c*lout_cs
  int64_t lin_es, lin_cs, lout_es, lout_cs;
  int64_t n_in, n_out;
  // four-step twiddle W_N^t, t = (e*k) mod N, W = hi[t >> shift] * lo[t & mask]
  int64_t tw4_n;
  int tw4_shift;
  const void* tw4_lo;
  const void* tw4_hi;
  int src_role, dst_role;      // buffer roles (ragged executor)
  const void* tcmat;           // K_ROW_TC: D_hi, D_lo (32 x 32 f16 each, N x K row-major)
  const int64_t* col_in_off;   // optional per-column element offsets (ragged groups)
  const int64_t* col_out_off;
  const void* chirp;   // Bluestein chirp c[l] = exp(-i*pi*l^2/n), l < n
  const void* filter;  // Bluestein filter spectrum DFT(conj chirp)/m, length m
  // F_ROT_OUT (shift / ishift fused into the last pass of an axis): the
  // element with axis index l = k*lout_es + c*lout_cs is stored
  // (rot(l) - l) * rot_stride elements away, rot(l) = (l - rot_s) mod rot_n
  int64_t rot_n, rot_s, rot_stride;
  // K_TC_FOLD / K_TC_DFT: folded length P (= floor(n/2) + 1), K chunks of
  // 32 and output chunks of 128 frequencies covering it
  int tc_p, tc_kc, tc_nc;
};

// Address offset of F_ROT_OUT for axis index l (0 without the flag).
__host__ __device__ inline int64_t rot_delta(const PassDesc& d, int64_t l) {
  if (!(d.flags & F_ROT_OUT)) return 0;
  return (l >= d.rot_s ? -d.rot_s : d.rot_n - d.rot_s) * d.rot_stride;
}

size_t pass_smem_bytes(const PassDesc& d, bool is_double);
int pass_grid(const PassDesc& d);

// cuTensorMapEncodeTiled from the driver (nullptr when unavailable).
void* tensor_map_encode_fn();

// Name of the __global__ function launch_pass runs for d (a 16-byte aligned
// input assumed).
const char* pass_kernel_name(const PassDesc& d, bool is_double);
const char* str_kernel_name(const PassDesc& d, bool is_double);
// Launch one pass on `stream`; returns a cudaError_t.
cudaError_t launch_pass(const PassDesc& d, bool is_double, cudaStream_t stream);

// Prepare kernel attributes (max dynamic shared memory); idempotent.
cudaError_t prepare_kernels();

bool row_kernel_available(int n, bool dbl);
bool row_blue_available(int m, bool dbl);  // one-pass Bluestein rows at padded length m
cudaError_t prepare_row_kernels();
cudaError_t launch_row(const PassDesc& d, bool dbl, cudaStream_t s);
cudaError_t prepare_col_kernels();
bool row_tc_available(int n);
bool str_kernel_available(int n, bool dbl);
int str_kernel_width(bool dbl);
cudaError_t prepare_str_kernels();
cudaError_t launch_str(const PassDesc& d, bool dbl, cudaStream_t s);
cudaError_t prepare_row_tc_kernels();
cudaError_t launch_row_tc(const PassDesc& d, cudaStream_t s);
cudaError_t launch_col4096(const PassDesc& d, bool dbl, cudaStream_t s);
cudaError_t prepare_tcdft_kernels();
bool plane_available(int64_t h, int64_t w, bool dbl);
cudaError_t prepare_plane_kernels();
cudaError_t launch_plane(const PassDesc& d, cudaStream_t s);
bool vec1024_available(int64_t n, bool dbl);
cudaError_t launch_vec1024(const PassDesc& d, cudaStream_t s);
cudaError_t launch_tcdft(const PassDesc& d, cudaStream_t s);
int col_tile_width(int variant);

}  // namespace gbfft
