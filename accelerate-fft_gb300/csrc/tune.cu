// Autotuner: times candidate plans of one transform on the current device
// and keeps the fastest choice per (device, shape, kind, type, precision).
//
// Knobs (TuneChoice): the contiguous-row kernel variant (single- or
// double-buffered exchanges, with or without bulk-copy streaming), the
// cluster column kernel variant for 4096-point strided axes, the four-step
// factorisation rank, the tensor-copy-fed strided kernel on or off, and the
// Bluestein padding (power of two or smallest 7-smooth) and the register
// row kernel versus the generic tile for contiguous rows.  The
// search is coordinate descent from the defaults: each knob that applies to
// the plan is swept with the others held at the best so far.  Every
// candidate runs 2 untimed and 5 timed executions (CUDA events on the
// caller's stream, median) on zero-filled scratch buffers of the
// transform's size, allocated for the search and freed after it; a 256 MiB
// write between timed executions evicts L2 (129 MB on GB300), so choices
// hold for data streamed from HBM.
//
// Results live in an in-process cache consulted by every plan creation.
// With GBFFT_TUNE_FILE=<path> the cache is loaded from that file on first
// use and each new result is appended to it as one JSON object per line:
//   {"key": "<device>|<rank>|<dims>|<kind>|<dtype>|<precision>",
//    "row_variant": 1, "row_tma": 1, "col_variant": 9, "split_rank": 0,
//    "str_tma": 1, "blue_pad": 1, "row_kernel": -1, "ms": 0.153}
// With GBFFT_AUTOTUNE=1 a plan creation whose key is not cached runs the
// search first.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "gbfft.h"
#include "plan_internal.h"

namespace gbfft {
namespace {

std::mutex g_mu;
std::map<std::string, std::pair<TuneChoice, double>> g_cache;
bool g_file_loaded = false;

std::string device_tag() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return "nodevice";
  static std::mutex m;
  static std::map<int, std::string> names;
  std::lock_guard<std::mutex> lk(m);
  auto it = names.find(dev);
  if (it != names.end()) return it->second;
  cudaDeviceProp prop;
  std::string tag = "unknown";
  if (cudaGetDeviceProperties(&prop, dev) == cudaSuccess) {
    char b[320];
    std::snprintf(b, sizeof b, "%s sm_%d%d %dSM", prop.name, prop.major, prop.minor, prop.multiProcessorCount);
    tag = b;
    for (char& c : tag)
      if (c == '"' || c == '\\' || c == '|') c = '_';
  }
  names[dev] = tag;
  return tag;
}

bool read_int(const char* line, const char* name, int& v) {
  char pat[64];
  std::snprintf(pat, sizeof pat, "\"%s\":", name);
  const char* q = std::strstr(line, pat);
  if (!q) return false;
  return std::sscanf(q + std::strlen(pat), " %d", &v) == 1;
}

// Parses one JSON line of the tune file; false when it is not one of ours.
bool parse_line(const char* line, std::string& key, TuneChoice& c, double& ms) {
  const char* k = std::strstr(line, "\"key\": \"");
  if (!k) return false;
  k += 8;
  const char* e = std::strchr(k, '"');
  if (!e) return false;
  key.assign(k, e);
  if (!read_int(line, "row_variant", c.row_variant) || !read_int(line, "row_tma", c.row_tma) ||
      !read_int(line, "col_variant", c.col_variant) || !read_int(line, "split_rank", c.split_rank) ||
      !read_int(line, "str_tma", c.str_tma))
    return false;
  if (!read_int(line, "blue_pad", c.blue_pad)) c.blue_pad = 1;
  if (!read_int(line, "row_kernel", c.row_kernel)) c.row_kernel = -1;
  const char* m = std::strstr(line, "\"ms\":");
  ms = 0;
  if (m) std::sscanf(m + 5, " %lf", &ms);
  c.tuned = true;
  return true;
}

int load_file_locked(const char* path) {
  std::FILE* f = std::fopen(path, "r");
  if (!f) return 0;
  int n = 0;
  char line[1024];
  while (std::fgets(line, sizeof line, f)) {
    std::string key;
    TuneChoice c;
    double ms = 0;
    if (parse_line(line, key, c, ms)) {
      g_cache[key] = {c, ms};
      ++n;
    }
  }
  std::fclose(f);
  return n;
}

void ensure_loaded_locked() {
  if (g_file_loaded) return;
  g_file_loaded = true;
  if (const char* f = std::getenv("GBFFT_TUNE_FILE")) load_file_locked(f);
}

bool has_kernel(const gbfft_plan* p, int kernel) {
  for (const PassSpec& ps : p->passes)
    if (ps.d.kernel == kernel) return true;
  return false;
}
bool has_flag(const gbfft_plan* p, uint32_t flag) {
  for (const PassSpec& ps : p->passes)
    if (ps.d.flags & flag) return true;
  return false;
}

}  // namespace

std::string tune_device_tag() { return device_tag(); }

std::string tune_key(int rank, const int64_t* dims, int kind, int dtype, int precision) {
  std::string k = device_tag();
  char b[64];
  std::snprintf(b, sizeof b, "|%d|", rank);
  k += b;
  for (int i = 0; i < rank; ++i) {
    std::snprintf(b, sizeof b, i ? "x%lld" : "%lld", (long long)dims[i]);
    k += b;
  }
  std::snprintf(b, sizeof b, "|%d|%d|%d", kind, dtype, precision);
  k += b;
  return k;
}

bool tune_lookup(const std::string& key, TuneChoice& out) {
  std::lock_guard<std::mutex> lk(g_mu);
  ensure_loaded_locked();
  auto it = g_cache.find(key);
  if (it == g_cache.end()) return false;
  out = it->second.first;
  return true;
}

void tune_store(const std::string& key, const TuneChoice& c, double ms) {
  std::lock_guard<std::mutex> lk(g_mu);
  ensure_loaded_locked();
  g_cache[key] = {c, ms};
  if (const char* path = std::getenv("GBFFT_TUNE_FILE")) {
    if (std::FILE* f = std::fopen(path, "a")) {
      std::fprintf(f,
                   "{\"key\": \"%s\", \"row_variant\": %d, \"row_tma\": %d, \"col_variant\": %d, "
                   "\"split_rank\": %d, \"str_tma\": %d, \"blue_pad\": %d, \"row_kernel\": %d, \"ms\": %.6f}\n",
                   key.c_str(), c.row_variant, c.row_tma, c.col_variant, c.split_rank, c.str_tma, c.blue_pad,
                   c.row_kernel, ms);
      std::fclose(f);
    }
  }
}

int autotune_plan(int rank, const int64_t* dims, int kind, int dtype, int precision, void* stream,
                  TuneChoice& best, std::string* report) {
  const TuneChoice base;
  gbfft_plan* p0 = nullptr;
  int st = create_plan(&p0, rank, dims, kind, dtype, precision, &base);
  if (st != GBFFT_OK) return st;
  std::unique_ptr<gbfft_plan, int (*)(gbfft_plan*)> hold(p0, gbfft_plan_destroy);
  const size_t eb = p0->dbl ? 16 : 8;
  const size_t bytes = size_t(p0->total) * eb;
  best = base;
  if (bytes == 0) return GBFFT_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void *din = nullptr, *dout = nullptr;
  if (cudaMalloc(&din, bytes) != cudaSuccess) return GBFFT_ERR_ALLOC;
  if (cudaMalloc(&dout, bytes) != cudaSuccess) {
    cudaFree(din);
    return GBFFT_ERR_ALLOC;
  }
  constexpr size_t kFlushBytes = size_t(256) << 20;
  void* dflush = nullptr;
  if (cudaMalloc(&dflush, kFlushBytes) != cudaSuccess) {
    dflush = nullptr;  // no flush buffer: time with whatever L2 holds
    cudaGetLastError();
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaMemsetAsync(din, 0, bytes, s);
  auto time_plan = [&](const gbfft_plan* p, double& ms) -> int {
    for (int i = 0; i < 2; ++i) {
      const int r = gbfft_exec(p, GBFFT_FORWARD, din, dout, s);
      if (r != GBFFT_OK) return r;
    }
    std::vector<float> t;
    for (int i = 0; i < 5; ++i) {
      if (dflush) cudaMemsetAsync(dflush, i, kFlushBytes, s);
      cudaEventRecord(e0, s);
      const int r = gbfft_exec(p, GBFFT_FORWARD, din, dout, s);
      if (r != GBFFT_OK) return r;
      cudaEventRecord(e1, s);
      if (cudaEventSynchronize(e1) != cudaSuccess) return GBFFT_ERR_CUDA;
      float x = 0;
      cudaEventElapsedTime(&x, e0, e1);
      t.push_back(x);
    }
    std::sort(t.begin(), t.end());
    ms = t[t.size() / 2];
    return gbfft_exec_status(p, stream);
  };
  auto line = [&](const TuneChoice& c, double ms, const gbfft_plan* p) {
    if (!report) return;
    char b[160];
    std::snprintf(b, sizeof b, "row=%d rowtma=%d col=%d split=%d strtma=%d bluepad=%d rowk=%d: %.4f ms  ",
                  c.row_variant, c.row_tma, c.col_variant, c.split_rank, c.str_tma, c.blue_pad, c.row_kernel, ms);
    *report += b;
    *report += p->desc;
    *report += "\n";
  };
  double best_ms = 0;
  st = time_plan(p0, best_ms);
  if (st == GBFFT_OK) {
    line(base, best_ms, p0);
    struct Knob {
      int TuneChoice::*field;
      std::vector<int> values;
      bool applies;
    };
    const Knob knobs[] = {
        {&TuneChoice::row_variant, {1, 0}, has_kernel(p0, K_ROW) || has_kernel(p0, K_ROW_TC)},
        {&TuneChoice::row_tma, {1, 0}, has_kernel(p0, K_ROW)},
        {&TuneChoice::col_variant, {18, 9, 17, 19, 16, 11, 13, 8, 10, 15, 14}, has_kernel(p0, K_COL4096)},
        {&TuneChoice::split_rank, {0, 1, 2}, has_flag(p0, F_TW4)},
        {&TuneChoice::str_tma, {1, 0}, has_kernel(p0, K_STRIDED)},
        {&TuneChoice::blue_pad, {1, 0}, has_flag(p0, F_CHIRP_IN)},
        {&TuneChoice::row_kernel, {1, 0}, has_kernel(p0, K_ROW) || has_kernel(p0, K_ROW_TC) ||
                                              (p0->dbl && has_kernel(p0, K_PENCIL))},
    };
    for (const Knob& k : knobs) {
      if (!k.applies) continue;
      const TuneChoice start = best;
      for (int v : k.values) {
        if (v == start.*(k.field)) continue;
        TuneChoice c = start;
        c.*(k.field) = v;
        gbfft_plan* pc = nullptr;
        if (create_plan(&pc, rank, dims, kind, dtype, precision, &c) != GBFFT_OK) continue;
        double ms = 0;
        const int r = time_plan(pc, ms);
        if (r == GBFFT_OK) line(c, ms, pc);
        gbfft_plan_destroy(pc);
        if (r != GBFFT_OK) {
          st = r;
          break;
        }
        // a candidate replaces the choice so far only when it is at least 1%
        // faster: differences below that are within the run-to-run spread
        // of these short timings, and the defaults are measured choices
        if (ms < best_ms * 0.99) {
          best_ms = ms;
          best = c;
        }
      }
      if (st != GBFFT_OK) break;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(din);
  cudaFree(dout);
  if (dflush) cudaFree(dflush);
  if (st != GBFFT_OK) return st;
  best.tuned = true;
  tune_store(tune_key(rank, dims, kind, dtype, precision), best, best_ms);
  if (report) {
    char b[96];
    std::snprintf(b, sizeof b, "best: row=%d rowtma=%d col=%d split=%d strtma=%d bluepad=%d rowk=%d %.4f ms\n",
                  best.row_variant, best.row_tma, best.col_variant, best.split_rank, best.str_tma, best.blue_pad,
                  best.row_kernel, best_ms);
    *report += b;
  }
  return GBFFT_OK;
}

}  // namespace gbfft

extern "C" {

int gbfft_tune_load(const char* path) {
  if (!path) return -GBFFT_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(gbfft::g_mu);
  gbfft::g_file_loaded = true;
  return gbfft::load_file_locked(path);
}

int gbfft_tune_clear(void) {
  std::lock_guard<std::mutex> lk(gbfft::g_mu);
  gbfft::g_cache.clear();
  gbfft::g_file_loaded = false;
  return GBFFT_OK;
}

int gbfft_tune_count(void) {
  std::lock_guard<std::mutex> lk(gbfft::g_mu);
  return int(gbfft::g_cache.size());
}

}  // extern "C"
