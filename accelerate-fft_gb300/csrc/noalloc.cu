// Allocation-free batched 1D transform for callers that cannot allocate
// device memory.
//
// Who needs it: a host that owns the device heap itself.  Accelerate's PTX
// backend hands the FFI pre-allocated arrays from its own allocator, keeps
// its own accounting of device memory, and expects a foreign call not to grab
// memory behind its back.  This entry point runs Bluestein's algorithm (four pencil passes: chirp and
// forward four-step half; second half and filter; inverse first half; inverse
// second half and chirp) for any length, and keeps everything the passes need
// beyond the caller's input and output -- twiddle, chirp and filter tables and
// the two padded work sequences -- in one file-scope __device__ array of
// kNoallocBytes.  It calls no cudaMalloc, cudaFree or other device allocator.
//
// Rules of use:
//  * The array exists once per device (once per CUDA context: a context
//    that loads the library gets its own copy) and lives until the process
//    exits.
//  * Every call resolves the array's device address in the context that is
//    current (cudaGetSymbolAddress; host code only holds a stand-in for the
//    symbol), and the first call in a context also sets kernel attributes
//    and uploads the tables; make that first call before any stream capture.
//    The tables held in the array are tracked per context, keyed on the
//    context's never-reused ID, so a caller that switches between contexts
//    (Accelerate's PTX backend creates its own) never reuses the address or
//    the tables of another context.
//  * Every call shares the array and it keeps the last call's contents:
//    tables are rewritten whenever the length changes, nothing relies on
//    the work area starting at zero, and calls that overlap on the GPU (two
//    streams, or two host threads) race on it.
//  * A request whose tables plus 2 * batch * m work elements (m = padded
//    length) do not fit is rejected with GBFFT_ERR_TOO_LARGE.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "gbfft.h"
#include "plan_internal.h"

namespace gbfft {
namespace {

constexpr size_t kNoallocBytes = size_t(16) << 20;  // 16 MiB per device
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

// Per-context state: the array's address in that context and the tables
// currently held at its head.
struct CtxState {
  unsigned char* ptr = nullptr;  // device address of g_noalloc_scratch
  int64_t n = 0, m = 0;
  bool dbl = false;
  size_t tables_bytes = 0;
  std::vector<PassSpec> passes;  // pointing into the array
};

std::mutex g_mu;
std::map<uint64_t, CtxState>& ctx_states() {
  static auto* m = new std::map<uint64_t, CtxState>();
  return *m;
}

// m = m1 * m2 with both factors within one CTA, m1 close to sqrt(m).
bool split_m(int64_t m, int cap, int64_t& m1, int64_t& m2) {
  int64_t best = 0;
  double bd = 1e300;
  for (int64_t a = 2; a <= cap && a < m; ++a) {
    if (m % a || m / a > cap) continue;
    const double d = std::fabs(std::log(double(a)) - std::log(double(m / a)));
    if (d < bd) {
      bd = d;
      best = a;
    }
  }
  if (!best) return false;
  m1 = best;
  m2 = m / best;
  return true;
}

// The four passes for `rows` rows of length n (row stride n), tables in B.
int build_passes(Builder& B, int64_t n, int64_t rows, int64_t m, std::vector<PassSpec>& out) {
  const int cap = B.dbl ? kCapC64 : kCapC32;
  int64_t m1, m2;
  if (!split_m(m, cap, m1, m2)) return GBFFT_ERR_UNSUPPORTED;
  PassSpec p[4];
  for (int i = 0; i < 4; ++i) {
    std::memset(&p[i].d, 0, sizeof(PassDesc));
    p[i].d.scale = 1.0;
    p[i].d.tw4_n = 1;
    if (!B.stages_for(int((i % 2 == 0) ? m1 : m2), p[i])) return GBFFT_ERR_UNSUPPORTED;
    B.blue_for(n, m, p[i]);
    p[i].d.nbatch = p[i].d.nb_lo = rows;
  }
  {  // P1: input -> S1: chirp, zero pad, first half, transposed store
    PassDesc& d = p[0].d;
    B.tw4_for(m, p[0]);
    d.in_bs = n;
    d.out_bs = m;
    d.ncols = m2;
    d.in_cs = 1;
    d.in_es = m2;
    d.out_es = 1;
    d.out_cs = m1;
    d.lin_es = m2;
    d.lin_cs = 1;
    d.n_in = n;
    d.flags = F_PAD_IN | F_CHIRP_IN | F_TW4;
  }
  {  // P2: S1 in place: second half, filter, conjugate
    PassDesc& d = p[1].d;
    d.in_bs = d.out_bs = m;
    d.ncols = m1;
    d.in_cs = d.out_cs = 1;
    d.in_es = d.out_es = m1;
    d.lout_es = m1;
    d.lout_cs = 1;
    d.flags = F_FILTER_OUT;
  }
  {  // P3: S1 -> S2: first half of the inverse
    PassDesc& d = p[2].d;
    B.tw4_for(m, p[2]);
    d.in_bs = d.out_bs = m;
    d.ncols = m2;
    d.in_cs = 1;
    d.in_es = m2;
    d.out_es = 1;
    d.out_cs = m1;
    d.flags = F_TW4;
  }
  {  // P4: S2 -> output: second half, conjugate and chirp, first n outputs
    PassDesc& d = p[3].d;
    d.in_bs = m;
    d.out_bs = n;
    d.ncols = m1;
    d.in_cs = d.out_cs = 1;
    d.in_es = d.out_es = m1;
    d.lout_es = m1;
    d.lout_cs = 1;
    d.n_out = n;
    d.flags = F_CHIRP_OUT | F_TRUNC_OUT;
  }
  const int roles[4][2] = {{R_IN, R_S1}, {R_S1, R_S1}, {R_S1, R_S2}, {R_S2, R_OUT}};
  for (int i = 0; i < 4; ++i) {
    p[i].src = roles[i][0];
    p[i].dst = roles[i][1];
    p[i].d.kernel = K_PENCIL;
    choose_tile(p[i], B.dbl);
    out.push_back(p[i]);
  }
  return GBFFT_OK;
}

}  // namespace
}  // namespace gbfft

using namespace gbfft;

extern "C" int gbfft_fft_noalloc(int mode, int64_t n, int64_t batch, int dtype, const void* d_in,
                                 void* d_out, void* stream) {
  if (mode != GBFFT_FORWARD && mode != GBFFT_REVERSE && mode != GBFFT_INVERSE)
    return GBFFT_ERR_INVALID_ARG;
  if (dtype != GBFFT_C32 && dtype != GBFFT_C64) return GBFFT_ERR_INVALID_ARG;
  if (n < 0 || batch < 0) return GBFFT_ERR_INVALID_ARG;
  if (n == 0 || batch == 0) return GBFFT_OK;
  if (!d_in || !d_out || d_in == d_out) return GBFFT_ERR_INVALID_ARG;
  const bool dbl = dtype == GBFFT_C64;
  const size_t eb = dbl ? 16 : 8;
  if ((reinterpret_cast<uintptr_t>(d_in) | reinterpret_cast<uintptr_t>(d_out)) & (eb - 1))
    return GBFFT_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (n == 1) {
    // the DFT of length 1 is the identity in every mode
    return cudaMemcpyAsync(d_out, d_in, size_t(batch) * eb, cudaMemcpyDeviceToDevice, s) == cudaSuccess
               ? GBFFT_OK
               : GBFFT_ERR_CUDA;
  }
  if (n > (int64_t(1) << 24)) return GBFFT_ERR_TOO_LARGE;
  const int64_t m = bluestein_length(n);
  // the two work sequences alone must fit (checked before any table is built)
  if (2 * double(batch) * double(m) * double(eb) > double(kNoallocBytes)) return GBFFT_ERR_TOO_LARGE;
  // The array's address in the context current on this thread (resolving it
  // also initialises the device's primary context when no context is
  // current, so there is always a context to key the state on).
  void* sym = nullptr;
  if (cudaGetSymbolAddress(&sym, g_noalloc_scratch) != cudaSuccess || !sym) return GBFFT_ERR_CUDA;
  const uint64_t ctx = current_context_id();

  std::lock_guard<std::mutex> lk(g_mu);
  CtxState& st = ctx_states()[ctx];
  if (st.ptr != sym) {
    // set-up, once per context, with that context current
    if (prepare_kernels() != cudaSuccess) {
      ctx_states().erase(ctx);
      return GBFFT_ERR_CUDA;
    }
    st = CtxState();
    st.ptr = static_cast<unsigned char*>(sym);
  }
  if (st.n != n || st.m != m || st.dbl != dbl || st.passes.empty()) {
    // The table upload below copies from host memory that is freed on
    // return; it is not recorded into a stream that is being captured.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) return GBFFT_ERR_CUDA;
    if (cap != cudaStreamCaptureStatusNone) return GBFFT_ERR_UNSUPPORTED;
    Builder B;
    B.dbl = dbl;
    std::vector<PassSpec> passes;
    const int rc = build_passes(B, n, 1, m, passes);
    if (rc != GBFFT_OK) return rc;
    const size_t tb = (B.blob.size() + 255) & ~size_t(255);
    if (tb + 2 * size_t(batch) * size_t(m) * eb > kNoallocBytes) return GBFFT_ERR_TOO_LARGE;
    // the tables go to the head of the array (a copy, not an allocation);
    // the state is marked empty until the copy is enqueued
    st.passes.clear();
    if (cudaMemcpyAsync(st.ptr, B.blob.data(), B.blob.size(), cudaMemcpyHostToDevice, s) != cudaSuccess)
      return GBFFT_ERR_CUDA;
    for (PassSpec& ps : passes) {
      if (ps.tw_off >= 0) ps.d.tw = st.ptr + ps.tw_off;
      if (ps.tw4lo_off >= 0) ps.d.tw4_lo = st.ptr + ps.tw4lo_off;
      if (ps.tw4hi_off >= 0) ps.d.tw4_hi = st.ptr + ps.tw4hi_off;
      if (ps.chirp_off >= 0) ps.d.chirp = st.ptr + ps.chirp_off;
      if (ps.filter_off >= 0) ps.d.filter = st.ptr + ps.filter_off;
    }
    st.passes = passes;
    st.tables_bytes = tb;
    st.n = n;
    st.m = m;
    st.dbl = dbl;
  }
  const size_t work = 2 * size_t(batch) * size_t(m) * eb;
  if (st.tables_bytes + work > kNoallocBytes) return GBFFT_ERR_TOO_LARGE;
  unsigned char* s1 = st.ptr + st.tables_bytes;
  unsigned char* s2 = s1 + size_t(batch) * size_t(m) * eb;
  const size_t last = st.passes.size() - 1;
  for (size_t i = 0; i < st.passes.size(); ++i) {
    PassDesc d = st.passes[i].d;
    d.nbatch = d.nb_lo = batch;
    auto ptr = [&](int role) -> void* {
      switch (role) {
        case R_IN: return const_cast<void*>(d_in);
        case R_OUT: return d_out;
        case R_S1: return s1;
        default: return s2;
      }
    };
    d.in = ptr(st.passes[i].src);
    d.out = ptr(st.passes[i].dst);
    if (mode != GBFFT_FORWARD) {
      if (i == 0) d.flags |= F_CONJ_IN;
      if (i == last) d.flags |= F_CONJ_OUT;
    }
    if (mode == GBFFT_INVERSE && i == last) {
      d.flags |= F_SCALE;
      d.scale = 1.0 / double(n);
    }
    if (launch_pass(d, dbl, s) != cudaSuccess) return GBFFT_ERR_CUDA;
  }
  return GBFFT_OK;
}
