// Host-side planner internals shared by the plan, ragged, spectral-convolution
// and split-precision translation units.
#pragma once

#include <complex>
#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "gbfft_internal.h"

namespace gbfft {

using cd = std::complex<double>;

// Buffer roles of a pass: the user's input / output, or plan scratch.
enum Role { R_IN = 0, R_OUT = 1, R_S1 = 2, R_S2 = 3 };

struct PassSpec {
  PassDesc d;
  int src = R_IN, dst = R_OUT;
  // the last pass of an axis: a fused output shift rotates axis index
  // l = k*lout_es + c*lout_cs, stored rot_stride elements apart; rot_ok is
  // false where the axis index is not of that form (strided four-step)
  bool axis_final = false, rot_ok = false;
  int64_t axis_n = 0, rot_stride = 0;
  // byte offsets into the plan's table blob (-1: none)
  int64_t tw_off = -1, tw4lo_off = -1, tw4hi_off = -1, chirp_off = -1, filter_off = -1;
};

// Accumulates the device tables of a plan (stage twiddles, four-step
// twiddles, Bluestein chirps and filter spectra) in one host blob, with
// per-length caches so repeated lengths share one copy.
struct Builder {
  bool dbl = false;
  std::vector<unsigned char> blob;
  struct StageTable {
    size_t off = 0;
    std::vector<int> offs;
  };
  struct Tw4 {
    size_t lo = 0, hi = 0;
    int shift = 0;
  };
  struct Blue {
    size_t chirp = 0, filter = 0;
  };
  std::map<int64_t, StageTable> stage_cache;
  std::map<int64_t, Tw4> tw4_cache;
  std::map<std::pair<int64_t, int64_t>, Blue> blue_cache;
  std::map<int64_t, size_t> roots_cache;
  // Bluestein tables computed ahead (in parallel) for (n, m): chirp, filter
  std::map<std::pair<int64_t, int64_t>, std::pair<std::vector<cd>, std::vector<cd>>> blue_pre;

  size_t add(const std::vector<cd>& v);
  bool stages_for(int n, PassSpec& ps);
  void tw4_for(int64_t N, PassSpec& ps);
  void blue_for(int64_t n, int64_t m, PassSpec& ps);
  size_t roots_for(int64_t N);  // table of W_N^t, t < N
  // compute the Bluestein chirp / filter of every (n, m) on all host cores
  void precompute_blue(const std::vector<std::pair<int64_t, int64_t>>& nm);
};

// Planner choices the autotuner searches over (defaults: the measured best
// on GB300 for fft2D 4096^2).
struct TuneChoice {
  int row_variant = -1;  // contiguous rows: 1 single-buffered, 0 double-buffered, -1 by kernel
  int row_tma = -1;     //   with row_variant 0: stream rows with cp.async.bulk (-1: by length)
  int col_variant = 18;  // 4096-point strided axes: cluster kernel variant (colfft.cu)
  int split_rank = 0;   // four-step axes: k-th best (n1, n2) factorisation
  int str_tma = 1;      // strided passes: tensor-copy-fed persistent kernel
  int blue_pad = 1;     // Bluestein padding: 1 power of two when cheaper, 0 smallest smooth m,
                        //   -1 the ragged executor's weighting
  int row_kernel = -1;  // contiguous rows: 1 register row kernel, 0 generic tile, -1 by rule
  double blue_weight = 2.0;  // with blue_pad -1: the ragged executor's generic-tile weight
  bool tuned = false;   // set by the autotuner (or its cache)
};

cd unit_root(int64_t t, int64_t L);  // exp(-2*pi*i*t/L), exact reduction
bool factor_device(int64_t n, std::vector<int>& out);
bool is_fast_length(int64_t n);
int64_t bluestein_length(int64_t n);
int64_t bluestein_multipass_length(int64_t n, int cap, bool dbl, double generic);
// Ragged-executor choices the autotuner searches over.
struct RaggedTune {
  int budget = 0;            // elements per tile and single-tile length cap (0: 4096, 2048 for C64)
  double blue_weight = 2.0;  // generic-tile weight when choosing multi-pass Bluestein lengths
                             // (its strided tiles load directly, so the gap to the generic
                             // tile is smaller than in plans, where it is 2.5)
  int strided = 1;           // register strided tiles for power-of-two four-step halves
  bool tuned = false;
};
std::string tune_device_tag();  // "<device name> sm_XY <n>SM" of the current device

void blue_tables(int64_t n, int64_t m, std::vector<cd>& chirp, std::vector<cd>& filter);
void host_fft_fp64(std::vector<cd>& x);
void choose_tile(PassSpec& ps, bool dbl);
bool fault_injected(const char* what);   // GBFFT_FAULT_INJECT=alloc,...
// Never-reused identity of the CUDA context current on this thread (plan.cu).
uint64_t current_context_id();
bool feature_disabled(const char* what);  // GBFFT_DISABLE=tma,row,cluster (A/B checks)
bool feature_enabled(const char* what);   // GBFFT_ENABLE=plane (opt-in variants)

}  // namespace gbfft

// The plan object behind the opaque gbfft_plan handle.
struct gbfft_plan {
  int rank = 0;
  int64_t dims[5] = {0, 0, 0, 0, 0};  // outermost first; rank 4-5 for batched-innermost plans
  int kind = 0, dtype = 0, precision = 0;
  int device = 0;
  bool dbl = false;
  int64_t total = 0;
  double inv_norm = 1.0;
  std::vector<gbfft::PassSpec> passes;
  void* d_tables = nullptr;
  size_t tables_bytes = 0;
  void* d_scratch = nullptr;
  size_t scratch_bytes = 0;
  size_t s2_off = 0;
  int* d_status = nullptr;  // device status word inside d_tables
  void* d_tcmat = nullptr;  // split-FP16 plans: D_hi, D_lo of the DFT-16 (4 KiB)
  gbfft::TuneChoice tune;   // planner choices (defaults, or the autotuner's)
  std::string desc;
  // Plans with scratch: executions on different streams share it, so each
  // one waits for the previous one (an event recorded after it) when the
  // stream changes.  Plans without scratch carry no execution state.
  mutable std::mutex scratch_mu;
  mutable cudaEvent_t scratch_ev = nullptr;
  mutable cudaStream_t scratch_stream = nullptr;
  mutable bool scratch_used = false;
};


namespace gbfft {
struct Axis {
  int64_t n, es, cs, ncols, os, outer;  // element (o, c, i) at o*os + c*cs + i*es
};
int add_axis(Builder& B, std::vector<PassSpec>& passes, const Axis& ax, bool first,
             int64_t& scratch1, int64_t& scratch2, std::string& desc, int cap = 0,
             const TuneChoice* tc = nullptr);  // nullptr: the defaults
int add_bluestein_multipass(Builder& B, std::vector<PassSpec>& passes, const Axis& ax, int src, int64_t m,
                            int cap, int split_rank, int64_t& scratch1, int64_t& scratch2, std::string& desc);
int build_plan(gbfft_plan* p, bool dry);
int build_split_plan(gbfft_plan* p);
int create_plan(gbfft_plan** out, int rank, const int64_t* dims, int kind, int dtype, int precision,
                const TuneChoice* forced);
// Autotuner cache: key of a plan on the current device, lookup / store, and
// the timed search itself (tune.cu).
std::string tune_key(int rank, const int64_t* dims, int kind, int dtype, int precision);
bool tune_lookup(const std::string& key, TuneChoice& out);
void tune_store(const std::string& key, const TuneChoice& c, double ms);
int autotune_plan(int rank, const int64_t* dims, int kind, int dtype, int precision, void* stream,
                  TuneChoice& best, std::string* report);
void* role_ptr(const gbfft_plan* p, int role, const void* in, void* out);
int add_bluestein_multipass(Builder& B, std::vector<PassSpec>& passes, const Axis& ax, int src, int64_t m,
                            int cap, int split_rank, int64_t& scratch1, int64_t& scratch2, std::string& desc);
int build_plan(gbfft_plan* p, bool dry);
int build_split_plan(gbfft_plan* p);
int create_plan(gbfft_plan** out, int rank, const int64_t* dims, int kind, int dtype, int precision,
                const TuneChoice* forced);
int build_split_plan(gbfft_plan* p);
// split-FP16 dense DFT of contiguous rows (tcdft.cu)
bool tcdft_available(int64_t n);
size_t tcdft_scratch_bytes(int64_t n, int64_t rows);
int tcdft_add_passes(Builder& B, int64_t n, int64_t rows, int64_t in_cs, int64_t out_cs, int src, int dst,
                     std::vector<PassSpec>& passes);
bool tcdft8_available(int64_t n);
int tcdft8_add_pass(Builder& B, int64_t n, int64_t rows, int64_t in_cs, int64_t out_cs, int src, int dst,
                    std::vector<PassSpec>& passes);
int exec_passes(const gbfft_plan* p, const std::vector<PassSpec>& passes, int mode, double inv_norm,
                const void* in, void* out, cudaStream_t s, int opts = 0, bool centre_fused = false);
}  // namespace gbfft
