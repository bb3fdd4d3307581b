// Ragged batch: many independent 1D transforms of uneven lengths and mixed
// modes over one flat buffer, executed by ONE persistent launch.
//
// Planning (host).  Every distinct length gets the pass list of a 1D plan
// (single shared-memory pass, four-step pair, single-kernel Bluestein, or the
// four-pass Bluestein) with tiles capped so three CTAs fit on an SM.  Each
// pass is cut into tasks (one CTA tile each).  Short transforms of the same
// length and mode are grouped into one tile through per-column offsets.
// Tasks are ordered level by level (every transform's first pass before any
// second pass), longest first inside a level, so a task only ever waits on
// tasks handed out before it: the persistent CTAs cannot deadlock.
//
// Execution (device).  CTAs pop task indices from an atomic queue head, copy
// the pass descriptor to shared memory, wait (bounded, with backoff) until
// the transform's previous pass has signalled all its tiles, run the tile
// with the generic pencil body, fence and signal.  A wait that exceeds its
// bound records GBFFT_ERR_TIMEOUT in the plan's status word and stops that
// CTA; nothing spins forever.  The counter reset and the launch form a CUDA
// graph that is instantiated once and relaunched with updated buffers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "gbfft.h"
#include "pencil_tile.cuh"
#include "plan_internal.h"
#include "strided_tile.cuh"

namespace gbfft {

struct RTask {
  int32_t desc;     // pass template
  int32_t member;   // first entry in the member offset lists
  int32_t count;    // columns (transforms) of a grouped tile, else 0
  int32_t tile;     // tile index inside the pass (ungrouped passes)
  int32_t dep;      // counter to wait on (-1: none)
  int32_t need;     // value it must reach
  int32_t signal;   // counter to bump when done (-1: none)
  uint32_t flags;   // mode flags of this transform for this pass
  double scale;
};

struct RaggedArgs {
  const PassDesc* descs;
  const RTask* tasks;
  int64_t ntasks;
  const int64_t* in_off;   // per member: element offset in d_in / d_out
  const int64_t* out_off;
  const int64_t* sc_off;   // per member: element offset of its scratch (S1; S2 follows)
  const int64_t* sc_len;   // per member: scratch length m (S2 = S1 + m)
  const void* in;
  void* out;
  void* scratch;
  int* counters;  // [0] queue head, [1..] per-(transform, pass) tile counters
  int* status;
  uint32_t spin_limit;  // bound of one dependency wait (polls)
};

namespace {

constexpr int kRaggedThreads = 256;
constexpr uint32_t kDepSpinLimit = 1u << 24;  // ~ seconds with the backoff below
// GBFFT_FAULT_INJECT=ragged_dep: the plan's first task waits on a counter no
// task signals, with this short bound (about a millisecond), so the timeout
// path can be exercised without faulting or hanging anything.
constexpr uint32_t kInjectedSpinLimit = 1u << 14;

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Separate (not inlined) bodies per tile kind, so the register allocation of
// one kind does not inflate the others.
template <typename T, int N, int W, int... Rs>
__device__ __noinline__ void ragged_str(const PassDesc& d, int64_t tile, unsigned char* smem) {
  str_tile_dispatch_ragged<T, N, W, Rs...>(d, tile, smem);
}
template <typename T>
__device__ __noinline__ void ragged_pencil(const PassDesc& d, int64_t tile, unsigned char* smem) {
  pencil_tile<T, true>(d, tile, smem);  // offsets within one transform fit in 31 bits
}

template <typename T>
__global__ void __launch_bounds__(kRaggedThreads, sizeof(T) == 4 ? 3 : 2) ragged_kernel(const RaggedArgs a) {
  using C = typename CxT<T>::type;
  extern __shared__ __align__(128) unsigned char smem[];
  constexpr int kDescBytes = (int(sizeof(PassDesc)) + 127) & ~127;
  PassDesc& d = *reinterpret_cast<PassDesc*>(smem);
  unsigned char* bufs = smem + kDescBytes;
  __shared__ int s_task;
  __shared__ int s_timeout;
  for (;;) {
    if (threadIdx.x == 0) s_task = atomicAdd(&a.counters[0], 1);
    __syncthreads();
    const int t = s_task;
    if (t >= a.ntasks) break;
    const RTask task = a.tasks[t];
    {
      const int* src = reinterpret_cast<const int*>(a.descs + task.desc);
      int* dst = reinterpret_cast<int*>(smem);
      for (int i = threadIdx.x; i < int(sizeof(PassDesc) / 4); i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const int64_t m = task.member;
      auto role = [&](int r) -> void* {
        if (r == R_IN) return const_cast<C*>(static_cast<const C*>(a.in)) + (task.count ? 0 : a.in_off[m]);
        if (r == R_OUT) return static_cast<C*>(a.out) + (task.count ? 0 : a.out_off[m]);
        C* base = static_cast<C*>(a.scratch) + a.sc_off[m];
        return r == R_S1 ? base : base + a.sc_len[m];
      };
      d.in = role(d.src_role);
      d.out = role(d.dst_role);
      d.flags |= task.flags;
      if (task.flags & F_SCALE) d.scale = task.scale;
      if (task.count) {
        d.ncols = task.count;
        d.col_in_off = a.in_off + m;
        d.col_out_off = a.out_off + m;
      }
      s_timeout = 0;
      if (task.dep >= 0) {
        uint32_t it = 0;
        while (ld_acquire(&a.counters[task.dep]) < task.need) {
          if (++it > a.spin_limit) {
            s_timeout = 1;
            atomicExch(a.status, GBFFT_ERR_TIMEOUT_DEVICE);
            break;
          }
          __nanosleep(64);
        }
      }
    }
    __syncthreads();
    if (s_timeout) break;
    const int64_t tl = task.count ? 0 : task.tile;
    if (d.kernel == K_STRIDED) {
      // W = 4096 / N keeps every instantiation at kRaggedThreads threads
      switch (d.n) {
        case 64: ragged_str<T, 64, 64, 16, 4>(d, tl, bufs); break;
        case 128: ragged_str<T, 128, 32, 16, 8>(d, tl, bufs); break;
        case 256: ragged_str<T, 256, 16, 16, 16>(d, tl, bufs); break;
        case 512: ragged_str<T, 512, 8, 16, 16, 2>(d, tl, bufs); break;
        case 1024: ragged_str<T, 1024, 4, 16, 16, 4>(d, tl, bufs); break;
        default: break;
      }
    } else {
      ragged_pencil<T>(d, tl, bufs);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0 && task.signal >= 0) atomicAdd(&a.counters[task.signal], 1);
  }
}

}  // namespace

}  // namespace gbfft

using namespace gbfft;

struct gbfft_ragged_plan {
  int64_t count = 0;
  bool dbl = false;
  int device = 0;
  std::vector<int64_t> lengths, offsets;
  std::vector<int> modes;
  // device
  void* d_tables = nullptr;
  PassDesc* d_descs = nullptr;
  RTask* d_tasks = nullptr;
  int64_t* d_members = nullptr;  // in_off | out_off | sc_off | sc_len, 4 * nmembers
  int* d_counters = nullptr;
  int* d_status = nullptr;
  void* d_scratch = nullptr;
  size_t scratch_bytes = 0, tables_bytes = 0;
  int64_t ntasks = 0, nmembers = 0;
  int ncounters = 0;
  int grid = 0;
  size_t smem = 0;
  // graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  cudaGraphNode_t knode = nullptr;
  RaggedArgs args{};
  // per-transform comparator: one ordinary plan per distinct length
  std::map<int64_t, gbfft_plan*> len_plans;
  gbfft::RaggedTune tune;  // the choices the plan was built with
};

namespace gbfft {
int create_ragged(gbfft_ragged_plan** out, int64_t count, const int64_t* lengths, const int64_t* offsets,
                  const int* modes, int dtype, const RaggedTune* forced);
int autotune_ragged(int64_t count, const int64_t* lengths, const int64_t* offsets, const int* modes, int dtype,
                    void* stream, RaggedTune& best, std::string* report);
}  // namespace gbfft

namespace {

// Tile width for a ragged pass: at most `budget` elements per tile.  Strided
// halves whose length has a register kernel use it with W = 4096 / n.
void ragged_tile(PassSpec& ps, bool dbl, int budget, int64_t group, bool strided) {
  PassDesc& d = ps.d;
  const int n = d.n;
  if (strided && group == 0 && d.in_cs == 1 && d.in_es != 1 &&
      (n == 64 || n == 128 || n == 256 || n == 512 || n == 1024) && str_ops_ragged(d.flags & kStrOpMask) &&
      !feature_disabled("strided")) {
    d.kernel = K_STRIDED;
    d.W = 4096 / n;
    d.threads = kRaggedThreads;
    d.pitch = n;
    return;
  }
  d.kernel = K_PENCIL;
  int pitch = n + (n >> 4) + 1;
  if (pitch % 2 == 0) ++pitch;
  d.pitch = pitch;
  int W = std::max(1, budget / n);
  const int64_t cols = group > 0 ? group : d.ncols;
  if (int64_t(W) > cols) W = int(std::max<int64_t>(1, cols));
  d.W = W;
  d.threads = kRaggedThreads;
  d.load_cfast = (d.in_cs == 1 && d.in_es != 1) ? 1 : 0;
  d.store_cfast = (d.out_cs == 1 && d.out_es != 1) ? 1 : 0;
  (void)dbl;
}

double pass_cost(const PassDesc& d, int64_t cols) {
  return double(cols) * double(d.n) * std::log2(double(std::max(2, d.n)));
}

void destroy_ragged(gbfft_ragged_plan* p) {
  if (!p) return;
  if (p->gexec) cudaGraphExecDestroy(p->gexec);
  if (p->graph) cudaGraphDestroy(p->graph);
  for (void* q : {(void*)p->d_tables, (void*)p->d_descs, (void*)p->d_tasks, (void*)p->d_members,
                  (void*)p->d_counters, p->d_scratch})
    if (q) cudaFree(q);
  for (auto& kv : p->len_plans) gbfft_plan_destroy(kv.second);
  delete p;
}

}  // namespace

extern "C" {

int gbfft_ragged_plan_create(gbfft_ragged_plan** out, int64_t count, const int64_t* lengths,
                             const int64_t* offsets, const int* modes, int dtype) {
  return gbfft::create_ragged(out, count, lengths, offsets, modes, dtype, nullptr);
}

int gbfft_ragged_autotune(int64_t count, const int64_t* lengths, const int64_t* offsets, const int* modes,
                          int dtype, void* stream, char* report, size_t cap) {
  gbfft::RaggedTune best;
  std::string rep;
  const int st = gbfft::autotune_ragged(count, lengths, offsets, modes, dtype, stream, best, &rep);
  if (report && cap) std::snprintf(report, cap, "%s", rep.c_str());
  return st;
}

}  // extern "C"

namespace gbfft {

namespace {
std::mutex g_rtune_mu;
std::map<std::string, RaggedTune> g_rtune;

// device + FNV-1a hash of the lengths and modes (the offsets do not change
// the work)
std::string ragged_key(int64_t count, const int64_t* lengths, const int* modes, int dtype) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](uint64_t v) {
    for (int i = 0; i < 8; ++i) {
      h ^= (v >> (8 * i)) & 0xFF;
      h *= 1099511628211ull;
    }
  };
  for (int64_t i = 0; i < count; ++i) {
    mix(uint64_t(lengths[i]));
    mix(uint64_t(uint32_t(modes[i])));
  }
  char b[96];
  std::snprintf(b, sizeof b, "|ragged|%lld|%d|%016llx", (long long)count, dtype, (unsigned long long)h);
  return tune_device_tag() + b;
}
}  // namespace

int create_ragged(gbfft_ragged_plan** out, int64_t count, const int64_t* lengths, const int64_t* offsets,
                  const int* modes, int dtype, const RaggedTune* forced) {
  if (!out) return GBFFT_ERR_INVALID_ARG;
  *out = nullptr;
  if (count < 0 || (count > 0 && (!lengths || !modes))) return GBFFT_ERR_INVALID_ARG;
  if (dtype != GBFFT_C32 && dtype != GBFFT_C64) return GBFFT_ERR_INVALID_ARG;
  if (count >= (int64_t(1) << 28)) return GBFFT_ERR_UNSUPPORTED;
  std::unique_ptr<gbfft_ragged_plan, void (*)(gbfft_ragged_plan*)> p(new gbfft_ragged_plan,
                                                                     destroy_ragged);
  p->count = count;
  p->dbl = dtype == GBFFT_C64;
  p->lengths.assign(lengths, lengths + count);
  p->modes.assign(modes, modes + count);
  p->offsets.resize(size_t(count));
  int64_t run = 0;
  for (int64_t i = 0; i < count; ++i) {
    if (lengths[i] < 0 || lengths[i] > (int64_t(1) << 26)) return GBFFT_ERR_INVALID_ARG;
    const int md = modes[i];
    if (md != GBFFT_FORWARD && md != GBFFT_REVERSE && md != GBFFT_INVERSE) return GBFFT_ERR_INVALID_ARG;
    p->offsets[size_t(i)] = offsets ? offsets[i] : run;
    if (p->offsets[size_t(i)] < 0) return GBFFT_ERR_INVALID_ARG;
    run += lengths[i];
  }
  if (cudaGetDevice(&p->device) != cudaSuccess) return GBFFT_ERR_CUDA;
  if (prepare_kernels() != cudaSuccess) return GBFFT_ERR_CUDA;
  const bool dbl = p->dbl;
  RaggedTune rt;
  if (forced) {
    rt = *forced;
  } else if (count > 0) {
    const std::string key = ragged_key(count, lengths, modes, dtype);
    bool hit = false;
    {
      std::lock_guard<std::mutex> lk(g_rtune_mu);
      auto it = g_rtune.find(key);
      if (it != g_rtune.end()) {
        rt = it->second;
        hit = true;
      }
    }
    if (!hit) {
      if (const char* at = std::getenv("GBFFT_AUTOTUNE"); at && at[0] == '1') {
        RaggedTune best;
        if (autotune_ragged(count, lengths, offsets, modes, dtype, nullptr, best, nullptr) == GBFFT_OK) rt = best;
      }
    }
  }
  p->tune = rt;
  const int budget = rt.budget > 0 ? rt.budget : (dbl ? 2048 : 4096);
  const int cap = budget;  // single-tile lengths; longer ones go four-step
  const bool strided = rt.strided != 0;

  // ---- pass templates per distinct length -------------------------------
  Builder B;
  B.dbl = dbl;
  const size_t status_off = B.add(std::vector<cd>(2, cd(0, 0)));
  struct LenClass {
    std::vector<PassSpec> passes;
    int64_t m = 0;        // scratch length per transform (Bluestein multi-pass)
    int first_desc = 0;   // index of passes[0] in the descriptor array
  };
  std::map<int64_t, LenClass> classes;
  {
    std::vector<std::pair<int64_t, int64_t>> nm;
    for (int64_t i = 0; i < count; ++i) {
      if (lengths[i] <= 1 || is_fast_length(lengths[i])) continue;
      // the padded length add_axis will pick (single tile, or four-pass)
      int64_t m = bluestein_length(lengths[i]);
      if (m > cap) m = bluestein_multipass_length(lengths[i], cap, dbl, rt.blue_weight);
      nm.push_back({lengths[i], m});
    }
    B.precompute_blue(nm);
  }
  for (int64_t i = 0; i < count; ++i) {
    const int64_t n = lengths[i];
    if (n <= 1 || classes.count(n)) continue;
    LenClass lc;
    int64_t s1 = 0, s2 = 0;
    std::string desc;
    const Axis ax{n, 1, n, 1, n, 1};
    TuneChoice rc;
    rc.blue_pad = -1;  // the ragged executor's Bluestein weighting
    rc.blue_weight = rt.blue_weight;
    rc.row_kernel = 0;  // passes run as generic or strided tiles below: no plan-only kernels
                        // (register rows, the single-vector cluster kernel) and their tables
    const int st = add_axis(B, lc.passes, ax, true, s1, s2, desc, cap, &rc);
    if (st != GBFFT_OK) return st;
    lc.m = s2;  // rows (1) * m for the four-pass Bluestein, else 0
    for (PassSpec& ps : lc.passes) {
      ps.d.kernel = K_PENCIL;
      ps.d.src_role = ps.src;
      ps.d.dst_role = ps.dst;
    }
    classes.emplace(n, std::move(lc));
  }
  // descriptors (tiles chosen per use: grouped single passes vs per transform)
  std::vector<PassSpec> descs;
  // group single-pass transforms by (length, mode)
  std::map<std::pair<int64_t, int>, std::vector<int64_t>> groups;
  std::vector<int64_t> multi;  // transforms with more than one pass
  for (int64_t i = 0; i < count; ++i) {
    const int64_t n = lengths[i];
    if (n == 0) continue;
    if (n == 1) {
      groups[{1, modes[i]}].push_back(i);  // identity: handled as a copy group below
      continue;
    }
    if (classes[n].passes.size() == 1) groups[{n, modes[i]}].push_back(i);
    else multi.push_back(i);
  }
  // members: in_off, out_off, sc_off, sc_len
  std::vector<int64_t> m_in, m_out, m_sc, m_len;
  std::vector<RTask> tasks;
  std::vector<std::pair<double, RTask>> level[4];
  int ncounters = 1;
  int64_t scratch_elems = 0;
  std::map<std::pair<int64_t, int>, int> desc_index;  // (length, pass) -> descriptor of grouped use
  auto mode_flags = [&](int md, bool first, bool last) {
    uint32_t f = 0;
    if (md != GBFFT_FORWARD) {
      if (first) f |= F_CONJ_IN;
      if (last) f |= F_CONJ_OUT;
    }
    if (md == GBFFT_INVERSE && last) f |= F_SCALE;
    return f;
  };
  for (auto& kv : groups) {
    const int64_t n = kv.first.first;
    const int md = kv.first.second;
    if (n == 1) continue;  // filled by the copy below
    const PassSpec& base = classes[n].passes[0];
    PassSpec ps = base;
    ragged_tile(ps, dbl, budget, int64_t(kv.second.size()), strided);
    const int W = ps.d.W;
    const int di = int(descs.size());
    descs.push_back(ps);
    for (size_t g0 = 0; g0 < kv.second.size(); g0 += size_t(W)) {
      const int cnt = int(std::min<size_t>(size_t(W), kv.second.size() - g0));
      RTask t{};
      t.desc = di;
      t.member = int32_t(m_in.size());
      t.count = cnt;
      t.dep = -1;
      t.signal = -1;
      t.flags = mode_flags(md, true, true);
      t.scale = 1.0 / double(n);
      for (int c = 0; c < cnt; ++c) {
        const int64_t id = kv.second[g0 + size_t(c)];
        m_in.push_back(p->offsets[size_t(id)]);
        m_out.push_back(p->offsets[size_t(id)]);
        m_sc.push_back(0);
        m_len.push_back(0);
      }
      level[0].push_back({pass_cost(ps.d, cnt), t});
    }
  }
  for (int64_t id : multi) {
    const int64_t n = lengths[size_t(id)];
    LenClass& lc = classes[n];
    const int member = int(m_in.size());
    m_in.push_back(p->offsets[size_t(id)]);
    m_out.push_back(p->offsets[size_t(id)]);
    m_sc.push_back(scratch_elems);
    m_len.push_back(lc.m);
    scratch_elems += 2 * lc.m;
    const int np = int(lc.passes.size());
    int prev_counter = -1, prev_tiles = 0;
    for (int k = 0; k < np; ++k) {
      auto key = std::make_pair(n, k);
      auto it = desc_index.find(key);
      if (it == desc_index.end()) {
        PassSpec ps = lc.passes[size_t(k)];
        ragged_tile(ps, dbl, budget, 0, strided);
        it = desc_index.emplace(key, int(descs.size())).first;
        descs.push_back(ps);
      }
      const PassDesc& d = descs[size_t(it->second)].d;
      const int tiles = pass_grid(d);
      const int counter = (k + 1 < np) ? ncounters++ : -1;
      for (int tl = 0; tl < tiles; ++tl) {
        RTask t{};
        t.desc = it->second;
        t.member = member;
        t.count = 0;
        t.tile = tl;
        t.dep = prev_counter;
        t.need = prev_tiles;
        t.signal = counter;
        t.flags = mode_flags(p->modes[size_t(id)], k == 0, k == np - 1);
        t.scale = 1.0 / double(n);
        level[std::min(k, 3)].push_back({pass_cost(d, d.W), t});
      }
      prev_counter = counter;
      prev_tiles = tiles;
    }
  }
  for (auto& lv : level) {
    std::stable_sort(lv.begin(), lv.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
    for (auto& e : lv) tasks.push_back(e.second);
  }
  // length-1 transforms are the identity for every mode: one grouped copy
  // through a pass-free descriptor is not needed -- they are copied on exec.
  uint32_t spin_limit = kDepSpinLimit;
  if (fault_injected("ragged_dep") && !tasks.empty()) {
    // failure injection: one dependency that nothing ever signals
    tasks[0].dep = ncounters++;
    tasks[0].need = 1;
    spin_limit = kInjectedSpinLimit;
  }
  p->ntasks = int64_t(tasks.size());
  p->nmembers = int64_t(m_in.size());
  p->ncounters = ncounters;

  // ---- device allocations ------------------------------------------------
  if (fault_injected("alloc")) return GBFFT_ERR_ALLOC;
  p->tables_bytes = B.blob.size();
  if (cudaMalloc(&p->d_tables, std::max<size_t>(p->tables_bytes, 256)) != cudaSuccess)
    return GBFFT_ERR_ALLOC;
  if (!B.blob.empty() &&
      cudaMemcpy(p->d_tables, B.blob.data(), B.blob.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return GBFFT_ERR_CUDA;
  unsigned char* tb = static_cast<unsigned char*>(p->d_tables);
  p->d_status = reinterpret_cast<int*>(tb + status_off);
  size_t smem_max = 0;
  std::vector<PassDesc> hdescs;
  for (PassSpec& ps : descs) {
    if (ps.tw_off >= 0) ps.d.tw = tb + ps.tw_off;
    if (ps.tw4lo_off >= 0) ps.d.tw4_lo = tb + ps.tw4lo_off;
    if (ps.tw4hi_off >= 0) ps.d.tw4_hi = tb + ps.tw4hi_off;
    if (ps.chirp_off >= 0) ps.d.chirp = tb + ps.chirp_off;
    if (ps.filter_off >= 0) ps.d.filter = tb + ps.filter_off;
    ps.d.status = p->d_status;
    const size_t sb = ps.d.kernel == K_STRIDED ? size_t(ps.d.n) * ps.d.W * (dbl ? 16 : 8)
                                               : pass_smem_bytes(ps.d, dbl);
    smem_max = std::max(smem_max, sb);
    hdescs.push_back(ps.d);
  }
  const size_t desc_bytes = (sizeof(PassDesc) + 127) & ~size_t(127);
  p->smem = desc_bytes + smem_max;
  auto upload = [](void** dst, const void* src, size_t bytes) {
    if (cudaMalloc(dst, std::max<size_t>(bytes, 16)) != cudaSuccess) return false;
    return bytes == 0 || cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
  };
  std::vector<int64_t> members;
  members.insert(members.end(), m_in.begin(), m_in.end());
  members.insert(members.end(), m_out.begin(), m_out.end());
  members.insert(members.end(), m_sc.begin(), m_sc.end());
  members.insert(members.end(), m_len.begin(), m_len.end());
  if (!upload((void**)&p->d_descs, hdescs.data(), hdescs.size() * sizeof(PassDesc)) ||
      !upload((void**)&p->d_tasks, tasks.data(), tasks.size() * sizeof(RTask)) ||
      !upload((void**)&p->d_members, members.data(), members.size() * sizeof(int64_t)))
    return GBFFT_ERR_ALLOC;
  if (cudaMalloc(&p->d_counters, size_t(ncounters) * sizeof(int)) != cudaSuccess) return GBFFT_ERR_ALLOC;
  p->scratch_bytes = size_t(scratch_elems) * (dbl ? 16 : 8);
  if (p->scratch_bytes && cudaMalloc(&p->d_scratch, p->scratch_bytes) != cudaSuccess)
    return GBFFT_ERR_ALLOC;
  // persistent grid: resident CTAs only
  auto kern = dbl ? (const void*)ragged_kernel<double> : (const void*)ragged_kernel<float>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(p->smem)) != cudaSuccess)
    return GBFFT_ERR_CUDA;
  int per_sm = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kRaggedThreads, p->smem) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess)
    return GBFFT_ERR_CUDA;
  if (per_sm < 1) return GBFFT_ERR_UNSUPPORTED;
  p->grid = int(std::min<int64_t>(int64_t(per_sm) * sms, std::max<int64_t>(1, p->ntasks)));
  RaggedArgs& a = p->args;
  a.descs = p->d_descs;
  a.tasks = p->d_tasks;
  a.ntasks = p->ntasks;
  a.in_off = p->d_members;
  a.out_off = p->d_members + p->nmembers;
  a.sc_off = p->d_members + 2 * p->nmembers;
  a.sc_len = p->d_members + 3 * p->nmembers;
  a.scratch = p->d_scratch;
  a.counters = p->d_counters;
  a.spin_limit = spin_limit;
  a.status = p->d_status;
  if (cudaDeviceSynchronize() != cudaSuccess) return GBFFT_ERR_CUDA;
  *out = p.release();
  return GBFFT_OK;
}

}  // namespace gbfft

extern "C" {

int gbfft_ragged_plan_destroy(gbfft_ragged_plan* plan) {
  destroy_ragged(plan);
  return GBFFT_OK;
}

int gbfft_ragged_exec(const gbfft_ragged_plan* cplan, const void* d_in, void* d_out, void* stream) {
  if (!cplan) return GBFFT_ERR_NULL_PLAN;
  gbfft_ragged_plan* p = const_cast<gbfft_ragged_plan*>(cplan);
  if (p->count == 0) return GBFFT_OK;
  if (!d_in || !d_out || d_in == d_out) return GBFFT_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t eb = p->dbl ? 16 : 8;
  // length-1 transforms are the identity for every mode
  for (int64_t i = 0; i < p->count; ++i)
    if (p->lengths[size_t(i)] == 1) {
      const size_t off = size_t(p->offsets[size_t(i)]) * eb;
      if (cudaMemcpyAsync(static_cast<char*>(d_out) + off, static_cast<const char*>(d_in) + off, eb,
                          cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return GBFFT_ERR_CUDA;
    }
  if (p->ntasks == 0) return GBFFT_OK;
  p->args.in = d_in;
  p->args.out = d_out;
  auto kern = p->dbl ? (void*)ragged_kernel<double> : (void*)ragged_kernel<float>;
  void* kargs[] = {&p->args};
  if (!p->gexec) {
    // counter reset + persistent launch, as a graph instantiated once
    if (cudaGraphCreate(&p->graph, 0) != cudaSuccess) return GBFFT_ERR_CUDA;
    cudaMemsetParams mp{};
    mp.dst = p->d_counters;
    mp.value = 0;
    mp.elementSize = 4;
    mp.width = size_t(p->ncounters);
    mp.height = 1;
    mp.pitch = 0;
    cudaGraphNode_t mnode;
    if (cudaGraphAddMemsetNode(&mnode, p->graph, nullptr, 0, &mp) != cudaSuccess) return GBFFT_ERR_CUDA;
    cudaKernelNodeParams kp{};
    kp.func = kern;
    kp.gridDim = dim3(unsigned(p->grid));
    kp.blockDim = dim3(kRaggedThreads);
    kp.sharedMemBytes = unsigned(p->smem);
    kp.kernelParams = kargs;
    if (cudaGraphAddKernelNode(&p->knode, p->graph, &mnode, 1, &kp) != cudaSuccess) return GBFFT_ERR_CUDA;
    if (cudaGraphInstantiate(&p->gexec, p->graph, 0) != cudaSuccess) return GBFFT_ERR_CUDA;
  } else {
    cudaKernelNodeParams kp{};
    kp.func = kern;
    kp.gridDim = dim3(unsigned(p->grid));
    kp.blockDim = dim3(kRaggedThreads);
    kp.sharedMemBytes = unsigned(p->smem);
    kp.kernelParams = kargs;
    if (cudaGraphExecKernelNodeSetParams(p->gexec, p->knode, &kp) != cudaSuccess) return GBFFT_ERR_CUDA;
  }
  if (cudaGraphLaunch(p->gexec, s) != cudaSuccess) return GBFFT_ERR_CUDA;
  return GBFFT_OK;
}

int gbfft_ragged_exec_per_transform(const gbfft_ragged_plan* p, const void* d_in, void* d_out,
                                    void* stream) {
  if (!p) return GBFFT_ERR_NULL_PLAN;
  if (p->count == 0) return GBFFT_OK;
  if (!d_in || !d_out || d_in == d_out) return GBFFT_ERR_INVALID_ARG;
  const size_t eb = p->dbl ? 16 : 8;
  for (int64_t i = 0; i < p->count; ++i) {
    const int64_t n = p->lengths[size_t(i)];
    if (n == 0) continue;
    const size_t off = size_t(p->offsets[size_t(i)]) * eb;
    const void* in = static_cast<const char*>(d_in) + off;
    void* out = static_cast<char*>(d_out) + off;
    if (n == 1) {
      if (cudaMemcpyAsync(out, in, eb, cudaMemcpyDeviceToDevice, static_cast<cudaStream_t>(stream)) !=
          cudaSuccess)
        return GBFFT_ERR_CUDA;
      continue;
    }
    auto it = p->len_plans.find(n);
    if (it == p->len_plans.end()) {
      // the comparator's ordinary 1D plans are created on first use
      gbfft_plan* lp = nullptr;
      const int st = gbfft_plan_create(&lp, 1, &n, GBFFT_KIND_FULL, p->dbl ? GBFFT_C64 : GBFFT_C32,
                                       GBFFT_PLAIN);
      if (st != GBFFT_OK) return st;
      it = const_cast<gbfft_ragged_plan*>(p)->len_plans.emplace(n, lp).first;
    }
    const int st = gbfft_exec(it->second, p->modes[size_t(i)], in, out, stream);
    if (st != GBFFT_OK) return st;
  }
  return GBFFT_OK;
}

int gbfft_ragged_status(const gbfft_ragged_plan* p, void* stream) {
  if (!p) return GBFFT_ERR_NULL_PLAN;
  if (!p->d_status) return GBFFT_OK;
  int h = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (cudaMemcpyAsync(&h, p->d_status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return GBFFT_ERR_CUDA;
  if (h != 0) cudaMemsetAsync(p->d_status, 0, sizeof(int), s);
  return h;
}

}  // extern "C"

namespace gbfft {

// Times candidate ragged plans (tile budget, Bluestein length weighting,
// register strided tiles) on scratch buffers and keeps the fastest per
// (device, lengths, modes); coordinate descent from the defaults, one
// untimed and three timed launches per candidate (CUDA events, median).
int autotune_ragged(int64_t count, const int64_t* lengths, const int64_t* offsets, const int* modes, int dtype,
                    void* stream, RaggedTune& best, std::string* report) {
  if (count <= 0 || !lengths || !modes) return GBFFT_ERR_INVALID_ARG;
  const bool dbl = dtype == GBFFT_C64;
  const size_t eb = dbl ? 16 : 8;
  int64_t total = 0, run = 0;
  for (int64_t i = 0; i < count; ++i) {
    const int64_t o = offsets ? offsets[i] : run;
    total = std::max(total, o + lengths[i]);
    run += lengths[i];
  }
  best = RaggedTune{};
  if (total == 0) return GBFFT_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void *din = nullptr, *dout = nullptr;
  if (cudaMalloc(&din, size_t(total) * eb) != cudaSuccess) return GBFFT_ERR_ALLOC;
  if (cudaMalloc(&dout, size_t(total) * eb) != cudaSuccess) {
    cudaFree(din);
    return GBFFT_ERR_ALLOC;
  }
  cudaMemsetAsync(din, 0, size_t(total) * eb, s);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto time_one = [&](const RaggedTune& c, double& ms) -> int {
    gbfft_ragged_plan* p = nullptr;
    int st = create_ragged(&p, count, lengths, offsets, modes, dtype, &c);
    if (st != GBFFT_OK) return st;
    std::vector<float> t;
    for (int i = 0; i < 4 && st == GBFFT_OK; ++i) {
      cudaEventRecord(e0, s);
      st = gbfft_ragged_exec(p, din, dout, s);
      cudaEventRecord(e1, s);
      if (cudaEventSynchronize(e1) != cudaSuccess) st = GBFFT_ERR_CUDA;
      float x = 0;
      cudaEventElapsedTime(&x, e0, e1);
      if (i > 0) t.push_back(x);
    }
    if (st == GBFFT_OK) st = gbfft_ragged_status(p, stream);
    gbfft_ragged_plan_destroy(p);
    if (st != GBFFT_OK) return st;
    std::sort(t.begin(), t.end());
    ms = t[t.size() / 2];
    return GBFFT_OK;
  };
  auto line = [&](const RaggedTune& c, double ms) {
    if (!report) return;
    char b[128];
    std::snprintf(b, sizeof b, "budget=%d blue_weight=%.1f strided=%d: %.4f ms\n",
                  c.budget > 0 ? c.budget : (dbl ? 2048 : 4096), c.blue_weight, c.strided, ms);
    *report += b;
  };
  double best_ms = 0;
  int st = time_one(best, best_ms);
  if (st == GBFFT_OK) {
    line(best, best_ms);
    const int b0 = dbl ? 2048 : 4096;
    const std::vector<int> budgets = {b0, b0 / 2};
    const std::vector<double> weights = {2.0, 1.0, 3.0};
    const std::vector<int> strides = {1, 0};
    for (int knob = 0; knob < 3 && st == GBFFT_OK; ++knob) {
      const RaggedTune start = best;
      const size_t nv = knob == 0 ? budgets.size() : knob == 1 ? weights.size() : strides.size();
      for (size_t v = 0; v < nv; ++v) {
        RaggedTune c = start;
        if (knob == 0) {
          if (budgets[v] == (start.budget > 0 ? start.budget : b0)) continue;
          c.budget = budgets[v];
        } else if (knob == 1) {
          if (weights[v] == start.blue_weight) continue;
          c.blue_weight = weights[v];
        } else {
          if (strides[v] == start.strided) continue;
          c.strided = strides[v];
        }
        double ms = 0;
        st = time_one(c, ms);
        if (st != GBFFT_OK) break;
        line(c, ms);
        if (ms < best_ms) {
          best_ms = ms;
          best = c;
        }
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(din);
  cudaFree(dout);
  if (st != GBFFT_OK) return st;
  best.tuned = true;
  {
    std::lock_guard<std::mutex> lk(g_rtune_mu);
    g_rtune[ragged_key(count, lengths, modes, dtype)] = best;
  }
  if (report) {
    char b[128];
    std::snprintf(b, sizeof b, "best: budget=%d blue_weight=%.1f strided=%d %.4f ms\n",
                  best.budget > 0 ? best.budget : (dbl ? 2048 : 4096), best.blue_weight, best.strided, best_ms);
    *report += b;
  }
  return GBFFT_OK;
}

}  // namespace gbfft
