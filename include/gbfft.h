/*
 * gbfft.h -- C ABI of the GB300-native FFT engine that replaces the cuFFT call
 * in accelerate-fft's GPU path.
 *
 * Every function returns an int status (GBFFT_OK == 0) unless stated.  No
 * CUDA or torch types appear in the signatures: device buffers are `void*`,
 * streams are passed as `void*` holding a cudaStream_t (NULL = legacy default
 * stream).  All work is enqueued asynchronously on that stream; no call
 * synchronises the host except plan creation.
 *
 * Element layout: interleaved complex (re, im) pairs -- `Vec2 e` in
 * Accelerate (src/Data/Array/Accelerate/Math/FFT/Type.hs:28-39), i.e.
 * float2 for Complex Float and double2 for Complex Double.  Arrays are
 * row-major with the innermost dimension contiguous, dims given
 * outermost-first exactly as Accelerate's `Z :. d :. h :. w`.
 *
 * Paths below are relative to the accelerate-fft source tree.
 */
#ifndef GBFFT_H
#define GBFFT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  GBFFT_OK = 0,
  GBFFT_ERR_INVALID_ARG = 1,  /* bad rank, dims, mode, kind, dtype, NULL buffer */
  GBFFT_ERR_UNSUPPORTED = 2,  /* valid request this build cannot serve          */
  GBFFT_ERR_ALLOC = 3,        /* device or host allocation failed (or refused)  */
  GBFFT_ERR_CUDA = 4,         /* a CUDA runtime call failed                      */
  GBFFT_ERR_NULL_PLAN = 5,
  GBFFT_ERR_TIMEOUT = 6,      /* a bounded device wait gave up (ragged executor) */
  GBFFT_ERR_INTERNAL = 7,
  GBFFT_ERR_TOO_LARGE = 8     /* request exceeds gbfft_fft_noalloc's fixed work area */
};

/* ---- Mode: src/Data/Array/Accelerate/Math/FFT/Mode.hs:15-26 -------------
 * Forward: sign -1.  Reverse: sign +1, unnormalised.  Inverse: sign +1,
 * normalised inside the kernel (by the innermost length for KIND_MANY and
 * fft1D, by the total size for fft2D/fft3D -- the division FFT.hs:83,110,
 * 141,172 performs after the foreign call today). */
enum { GBFFT_FORWARD = -1, GBFFT_REVERSE = 1, GBFFT_INVERSE = 2 };

/* ---- element type: NumericR (Type.hs:28-30) ---------------------------- */
enum { GBFFT_C32 = 0 /* Complex Float, C2C */, GBFFT_C64 = 1 /* Complex Double, Z2Z */ };

/* ---- transform kind ----------------------------------------------------
 * MANY: batched 1D transforms along the innermost axis of a rank-1..5
 *       array -- PTX.fft (PTX.hs:52-61): "cuda.fft2.many" / "cuda.fft3.many"
 *       (cufftPlanMany [w] batch h or d*h, PTX.hs:158-170).  Ranks 4 and 5,
 *       which the reference sends to its pure transform (FFT.hs:78), run on
 *       the GPU here.
 * FULL: the rank-r transform over every axis -- PTX.fft1D/fft2D/fft3D
 *       (PTX.hs:63-70; cufftPlan1d/2d/3d, PTX.hs:137-156). */
enum { GBFFT_KIND_MANY = 0, GBFFT_KIND_FULL = 1 };

/* ---- precision ---------------------------------------------------------- */
enum { GBFFT_PLAIN = 0, GBFFT_SPLIT_FP16 = 1 };

typedef struct gbfft_plan gbfft_plan;

/* Human-readable text for a status code (static storage, never NULL). */
const char* gbfft_error_string(int status);

/* Library version as 10000*major + 100*minor + patch. */
int gbfft_version(void);

/* Create a plan for the current CUDA device.  Replaces the cufftPlan*
 * constructors the reference caches (PTX.hs:137-170).  Allocates the plan's
 * device workspace (twiddle tables, Bluestein chirp and filter spectrum,
 * scratch for multi-pass transforms) and synchronises the device once.
 * rank 1..3 (1..5 for MANY); dims outermost-first; a zero extent gives a
 * plan whose exec is a no-op. */
int gbfft_plan_create(gbfft_plan** out, int rank, const int64_t* dims, int kind, int dtype,
                      int precision);

/* Free a plan created by gbfft_plan_create (NULL is accepted). */
int gbfft_plan_destroy(gbfft_plan* plan);

/* Execute a plan: out-of-place, d_in preserved (Accelerate arrays are
 * immutable).  Replaces `FFT.setStream h s >> FFT.execC2C/execZ2Z h mode
 * d_in d_out` (PTX.hs:112-124).  The plan holds no per-call mutable state,
 * so concurrent execs of one plan on different streams are safe (the
 * setStream race noted at PTX/Plans.hs:61 does not exist here). */
int gbfft_exec(const gbfft_plan* plan, int mode, const void* d_in, void* d_out, void* stream);

/* Plan-cache lookup: the plan for (current CUDA context, rank, dims, kind,
 * dtype, precision), created on first use.  Replaces `withPlan`
 * (PTX/Plans.hs:66-86), keyed on the full shape rather than on its hash
 * (PTX/Plans.hs:72).  The cache owns the plan; do not destroy it.  Thread
 * safe. */
int gbfft_plan_get(gbfft_plan** out, int rank, const int64_t* dims, int kind, int dtype,
                   int precision);

/* One call doing what PTX.fft' does per node (PTX.hs:84-106): cached plan
 * lookup plus exec.  This is the entry point the Haskell FFI module binds. */
int gbfft_fft(int mode, int rank, const int64_t* dims, int kind, int dtype, const void* d_in,
              void* d_out, void* stream);

/* Drop every cached plan of the current context (the Lifetime finalizer
 * hook of PTX/Plans.hs:79-80). */
int gbfft_cache_clear(void);

/* Device-side status of the plan's earlier execs on `stream`: GBFFT_OK, or
 * GBFFT_ERR_TIMEOUT if a bounded wait inside a kernel gave up (the status is
 * then cleared).  Synchronises the stream. */
int gbfft_exec_status(const gbfft_plan* plan, void* stream);

/* Instrumentation: run passes [first, first+count) of the plan only, with
 * the same buffers and mode handling as gbfft_exec (running every range in
 * order equals one gbfft_exec).  Lets a profiler time each pass. */
int gbfft_exec_range(const gbfft_plan* plan, int mode, int first, int count, const void* d_in,
                     void* d_out, void* stream);

/* Introspection: device bytes held by a plan, and number of kernel launches
 * one exec performs. */
int gbfft_plan_info(const gbfft_plan* plan, size_t* workspace_bytes, int* launches_per_exec);

/* Host-only dry run: describe the passes a plan for these arguments would
 * run, with its table and scratch sizes, without touching the device. */
int gbfft_plan_explain(int rank, const int64_t* dims, int kind, int dtype, int precision, char* buf,
                       size_t cap);

/* Write a one-line description of the plan (passes, radices, tile widths)
 * into buf (NUL-terminated, truncated to cap). */
int gbfft_plan_describe(const gbfft_plan* plan, char* buf, size_t cap);

/* Name of the CUDA kernel that launch `pass` (0-based, in execution order)
 * of one exec runs, e.g. "colfft4096_r16_kernel"; used to match timings to
 * profiler launch lists.  No counterpart in the reference. */
int gbfft_plan_pass_kernel(const gbfft_plan* plan, int pass, char* buf, size_t cap);

/* Bandwidth probe (measurement support, no counterpart in the reference):
 * copies a rows x cols Complex Float array `in` to `out` in tiles of `width`
 * contiguous columns over all rows -- the access pattern of a strided pass
 * with W = width (width = cols: the contiguous pattern of a row pass).
 * width even and dividing cols (widths above 8192 copy runs of at most
 * 8192 columns, contiguous all the same); 16-byte aligned buffers. */
int gbfft_probe_tile_copy(int64_t rows, int64_t cols, int width, const void* in, void* out, void* stream);

/* ---- autotuner: new beyond the reference API ---------------------------
 * The reference takes cuFFT's internal plan choice (PTX.hs:141-169).
 * gbfft_autotune times candidate plans of this transform on the current
 * device (row / column kernel variants, four-step factorisation, tensor-copy
 * strided kernel) on scratch buffers it allocates and frees, on `stream`,
 * and caches the fastest choice per (device, dims, kind, dtype, precision);
 * every later plan creation for that key uses it.  `report` (may be NULL)
 * receives one line per candidate.  GBFFT_AUTOTUNE=1 makes plan creation
 * tune on a cache miss; GBFFT_TUNE_FILE=<path> loads the cache from that
 * file on first use and appends each new result (JSON lines). */
int gbfft_autotune(int rank, const int64_t* dims, int kind, int dtype, int precision, void* stream,
                   char* report, size_t cap);
/* Loads tuned choices from a JSON-lines file; returns the number of entries
 * read (0 if the file is missing), or a negative status.  No device work. */
int gbfft_tune_load(const char* path);
/* Forgets every tuned choice (the file, if any, is re-read on next use). */
int gbfft_tune_clear(void);
/* Number of tuned choices held. */
int gbfft_tune_count(void);

/* ---- naive DFT with caller-supplied roots: DFT.hs:68-111 ---------------
 * gbfft_dftG replaces Math.DFT.dftG (DFT.hs:68-92) for an array of rank
 * 1..5 (dims outermost-first) and roots of the same shape (rootsOfUnity /
 * inverseRootsOfUnity, Roots.hs:26-51, or any others): out(sh_o :. k) =
 * sum over ALL elements (sh :. n) of in(sh :. n) * roots(sh :. (k*n) mod l),
 * l = the innermost extent -- the reference folds over an extended axis of
 * length shapeSize, so for rank > 1 every output row holds the same values.
 * gbfft_dftGS replaces dftGS (DFT.hs:95-111): that single value for bin k,
 * written to d_out[0].  O(size * l) work, no allocation, asynchronous on
 * `stream`. */
int gbfft_dftG(int rank, const int64_t* dims, int dtype, const void* d_roots, const void* d_in, void* d_out,
               void* stream);
int gbfft_dftGS(int rank, const int64_t* dims, int dtype, int64_t k, const void* d_roots, const void* d_in,
                void* d_out, void* stream);

/* ---- fused centring / shifting: Math.DFT.Centre around a full transform --
 * gbfft_exec_ex = gbfft_exec followed or preceded by Centre.hs helpers
 * (DFT/Centre.hs:36-164), for FULL plans of rank 1..3:
 *   GBFFT_OPT_SHIFT_OUT  / GBFFT_OPT_ISHIFT_OUT: shiftND / ishiftND of the
 *     result, fused into the last pass of every axis as an index rotation;
 *   GBFFT_OPT_CENTRE_IN: centreND of the input -- for even extents fused the
 *     same way (centring the input rotates the output by n/2), otherwise one
 *     extra pass before the transform.
 * Axes whose last pass cannot rotate (a strided four-step axis) fall back to
 * one shift pass after the transform (a stream-ordered temporary).  No
 * counterpart in the reference's foreign path. */
enum { GBFFT_OPT_SHIFT_OUT = 1, GBFFT_OPT_ISHIFT_OUT = 2, GBFFT_OPT_CENTRE_IN = 4 };
int gbfft_exec_ex(const gbfft_plan* plan, int mode, const void* d_in, void* d_out, void* stream, int opts);

/* ---- Math.DFT.Centre (DFT/Centre.hs:36-164), rank 1..3 ------------------
 * gbfft_centre: centre1D/2D/3D, out = (-1)^(sum of the indices) * in (d_in
 * may equal d_out).  gbfft_shift: shift1D/2D/3D (inverse = 0, roll by
 * n/2 + (n odd) per axis) or ishift1D/2D/3D (inverse = 1, roll by n/2):
 * out(ix) = in((ix + s) mod n) per axis; out-of-place.  One pass each. */
int gbfft_centre(int rank, const int64_t* dims, int dtype, const void* d_in, void* d_out, void* stream);
int gbfft_shift(int rank, const int64_t* dims, int dtype, int inverse, const void* d_in, void* d_out,
                void* stream);

/* ---- ragged batch: new beyond the reference API -------------------------
 * `count` independent 1D transforms of uneven lengths over one flat buffer,
 * executed by one persistent launch (the reference can only express this as
 * `count` separate fft1D calls, PTX.hs:63-64).  offsets[i] is the element
 * offset of transform i in both d_in and d_out (NULL = packed back to back);
 * modes[i] is GBFFT_FORWARD / REVERSE / INVERSE. */
typedef struct gbfft_ragged_plan gbfft_ragged_plan;
int gbfft_ragged_plan_create(gbfft_ragged_plan** out, int64_t count, const int64_t* lengths,
                             const int64_t* offsets, const int* modes, int dtype);

/* Autotuner for a ragged batch (new): times candidate plans of these
 * lengths and modes (tile budget, Bluestein padded-length weighting,
 * register strided tiles) on scratch buffers on `stream` and caches the
 * fastest per (device, lengths, modes); later gbfft_ragged_plan_create calls
 * for the same batch use it (GBFFT_AUTOTUNE=1 makes plan creation tune on a
 * miss).  `report` (may be NULL) receives one line per candidate. */
int gbfft_ragged_autotune(int64_t count, const int64_t* lengths, const int64_t* offsets, const int* modes,
                          int dtype, void* stream, char* report, size_t cap);
int gbfft_ragged_exec(const gbfft_ragged_plan* plan, const void* d_in, void* d_out, void* stream);
/* The same transforms issued as one launch sequence per transform (the
 * "one launch per transform" comparator). */
int gbfft_ragged_exec_per_transform(const gbfft_ragged_plan* plan, const void* d_in, void* d_out,
                                    void* stream);
int gbfft_ragged_plan_destroy(gbfft_ragged_plan* plan);
/* Device-side status of the last ragged exec on this plan (GBFFT_OK or
 * GBFFT_ERR_TIMEOUT when a bounded wait gave up); synchronises the stream. */
int gbfft_ragged_status(const gbfft_ragged_plan* plan, void* stream);

/* ---- spectral convolution: new beyond the reference API ----------------
 * y_b = fft3D Inverse (fft3D Forward (x_b) * H) for b in [0, batch), x and y
 * batch x d x h x w complex, H d x h x w complex.  The reference composes
 * this from fft3D (FFT.hs:150-173) and zipWith. */
typedef struct gbfft_specconv_plan gbfft_specconv_plan;
int gbfft_specconv_plan_create(gbfft_specconv_plan** out, int64_t batch, int64_t d, int64_t h,
                               int64_t w, int dtype);
int gbfft_specconv_fwd(const gbfft_specconv_plan* plan, const void* d_x, const void* d_H, void* d_y,
                       void* stream);
/* Adjoint: given g_y = dL/dy (conjugate-Wirtinger convention), writes
 * g_x = dL/dx and g_H = dL/dH (g_H summed over the batch).  The forward
 * spectrum of x is recomputed, not stored. */
int gbfft_specconv_bwd(const gbfft_specconv_plan* plan, const void* d_x, const void* d_H,
                       const void* d_gy, void* d_gx, void* d_gH, void* stream);
int gbfft_specconv_plan_destroy(gbfft_specconv_plan* plan);

/* ---- allocation-free transform ------------------------------------------
 * No counterpart in the reference: an addition for callers that cannot
 * allocate device memory, such as a host that owns the device heap itself
 * (Accelerate's PTX backend passes arrays from its own allocator and keeps
 * its own account of device memory).  Transforms `batch` contiguous rows of
 * length n (Bluestein's algorithm, four passes, any n) with Mode semantics
 * as gbfft_exec (Inverse divides by n), reading d_in and writing d_out, and
 * allocates nothing: its tables and padded work sequences live in one fixed
 * 16 MiB __device__ array per device (per CUDA context), kept until the
 * process exits.  Each call resolves the array's address in the context
 * current on the calling thread; the first call in a context also sets the
 * kernels up and uploads the tables (make it before any stream capture).
 * Calls share the array and it keeps the last call's tables, so calls that
 * overlap on the GPU race.  Requests whose tables plus 2 * batch * m
 * elements (m, the padded length, is about 2n to 4n) exceed 16 MiB return
 * GBFFT_ERR_TOO_LARGE. */
int gbfft_fft_noalloc(int mode, int64_t n, int64_t batch, int dtype, const void* d_in, void* d_out,
                      void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GBFFT_H */
