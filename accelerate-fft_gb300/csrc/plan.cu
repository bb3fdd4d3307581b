// Host side of the engine: factoriser, twiddle / Bluestein table builder,
// pass sequencing, the per-context plan cache and the C ABI of gbfft.h.
//
// Replaces, on the accelerate-fft side (paths in the accelerate-fft tree):
//   cufftPlan1d/2d/3d/Many constructors ... src/Data/Array/Accelerate/Math/FFT/LLVM/PTX.hs:137-170
//   withPlan / Plans cache ............... src/Data/Array/Accelerate/Math/FFT/LLVM/PTX/Plans.hs:40-90
//   setStream + execC2C/execZ2Z .......... PTX.hs:112-124
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdio>
#include <functional>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "gbfft.h"
#include "gbfft_internal.h"
#include "plan_internal.h"
#include "strided_tile.cuh"

namespace gbfft {

// ---------------------------------------------------------------------------
// exact unit roots
cd unit_root(int64_t t, int64_t L) {
  t %= L;
  if (t < 0) t += L;
  // angle = 2*pi*t/L = q*pi/2 + (pi/2)*(r/L), q = floor(4t/L)
  const int64_t q = (4 * t) / L;
  const int64_t r = 4 * t - q * L;
  const double hp = 1.57079632679489661923132169163975;
  double c, s;
  if (2 * r <= L) {
    const double x = hp * double(r) / double(L);
    c = std::cos(x);
    s = std::sin(x);
  } else {
    const double x = hp * double(L - r) / double(L);
    c = std::sin(x);
    s = std::cos(x);
  }
  double c2 = c, s2 = s;
  switch (q & 3) {
    case 1: c2 = -s; s2 = c; break;
    case 2: c2 = -c; s2 = -s; break;
    case 3: c2 = s; s2 = -c; break;
    default: break;
  }
  return cd(c2, -s2);  // exp(-i * angle)
}

// Radix list of the device Stockham stages for a 7-smooth n.  Powers of two:
// radix 16 while possible, then 8 / 4 / 2 (the lists the register kernels are
// instantiated with).  Lengths with odd factors: the fewest stages over
// radices up to 16, including the composite radices 6, 9, 10, 12, 14 and 15
// (one shared-memory round trip per stage), larger radices first on ties.
bool factor_device(int64_t n, std::vector<int>& out) {
  out.clear();
  if (n < 1) return false;
  int64_t m = n;
  int a2 = 0, a3 = 0, a5 = 0, a7 = 0;
  while (m % 2 == 0) { m /= 2; ++a2; }
  while (m % 3 == 0) { m /= 3; ++a3; }
  while (m % 5 == 0) { m /= 5; ++a5; }
  while (m % 7 == 0) { m /= 7; ++a7; }
  if (m != 1) return false;
  if (a3 == 0 && a5 == 0 && a7 == 0) {
    while (a2 >= 4) { out.push_back(16); a2 -= 4; }
    if (a2 == 3) out.push_back(8);
    else if (a2 == 2) out.push_back(4);
    else if (a2 == 1) out.push_back(2);
    return true;
  }
  struct Rad { int r, e2, e3, e5, e7; };
  static const Rad rad[] = {{16, 4, 0, 0, 0}, {15, 0, 1, 1, 0}, {14, 1, 0, 0, 1}, {12, 2, 1, 0, 0},
                            {10, 1, 0, 1, 0}, {9, 0, 2, 0, 0},  {8, 3, 0, 0, 0},  {7, 0, 0, 0, 1},
                            {6, 1, 1, 0, 0},  {5, 0, 0, 1, 0},  {4, 2, 0, 0, 0},  {3, 0, 1, 0, 0},
                            {2, 1, 0, 0, 0}};
  // fewest stages for exponents (b2, b3, b5, b7), memoised; -1 = unreachable
  std::map<int64_t, std::pair<int, int>> memo;  // key -> (stages, radix index)
  std::function<int(int, int, int, int)> best = [&](int b2, int b3, int b5, int b7) -> int {
    if (b2 == 0 && b3 == 0 && b5 == 0 && b7 == 0) return 0;
    const int64_t key = ((int64_t(b2) * 64 + b3) * 64 + b5) * 64 + b7;
    auto it = memo.find(key);
    if (it != memo.end()) return it->second.first;
    int bs = -1, bi = -1;
    for (int i = 0; i < int(sizeof(rad) / sizeof(rad[0])); ++i) {
      const Rad& r = rad[i];
      if (r.e2 > b2 || r.e3 > b3 || r.e5 > b5 || r.e7 > b7) continue;
      const int sub = best(b2 - r.e2, b3 - r.e3, b5 - r.e5, b7 - r.e7);
      if (sub >= 0 && (bs < 0 || sub + 1 < bs)) {
        bs = sub + 1;
        bi = i;
      }
    }
    memo[key] = {bs, bi};
    return bs;
  };
  if (best(a2, a3, a5, a7) < 0) return false;
  while (a2 || a3 || a5 || a7) {
    const int64_t key = ((int64_t(a2) * 64 + a3) * 64 + a5) * 64 + a7;
    const Rad& r = rad[memo[key].second];
    out.push_back(r.r);
    a2 -= r.e2;
    a3 -= r.e3;
    a5 -= r.e5;
    a7 -= r.e7;
  }
  return true;
}

bool is_fast_length(int64_t n) {
  if (n < 1) return false;
  for (int p : {2, 3, 5, 7})
    while (n % p == 0) n /= p;
  return n == 1;
}

// FP64 Stockham FFT on the host (forward sign) for 7-smooth lengths; used
// only at plan time for Bluestein filter spectra.
void host_fft_fp64(std::vector<cd>& x) {
  const int64_t n = int64_t(x.size());
  if (n <= 1) return;
  std::vector<int> f;
  {
    int64_t m = n;
    while (m % 4 == 0) { f.push_back(4); m /= 4; }
    while (m % 2 == 0) { f.push_back(2); m /= 2; }
    while (m % 3 == 0) { f.push_back(3); m /= 3; }
    while (m % 5 == 0) { f.push_back(5); m /= 5; }
    while (m % 7 == 0) { f.push_back(7); m /= 7; }
  }
  std::vector<cd> roots(static_cast<size_t>(n));
  for (int64_t t = 0; t < n; ++t) roots[size_t(t)] = unit_root(t, n);
  std::vector<cd> y(static_cast<size_t>(n));
  int64_t Ns = 1;
  for (int R : f) {
    const int64_t nb = n / R, step = n / (Ns * R);
    for (int64_t j = 0; j < nb; ++j) {
      const int64_t p = j % Ns;
      cd v[7];
      for (int r = 0; r < R; ++r) v[r] = x[size_t(j + r * nb)] * roots[size_t((p * r * step) % n)];
      const int64_t base = (j - p) * R + p;
      for (int k = 0; k < R; ++k) {
        cd acc(0, 0);
        for (int r = 0; r < R; ++r) acc += v[r] * roots[size_t(((r * k) % R) * nb)];
        y[size_t(base + k * Ns)] = acc;
      }
    }
    std::swap(x, y);
    Ns *= R;
  }
}

// Bluestein padded length: the 7-smooth m >= 2n-1 with the fewest
// (stages + 1) * m among candidates up to the next power of two.
int64_t bluestein_length(int64_t n) {
  const int64_t lo = 2 * n - 1;
  int64_t p2 = 1;
  while (p2 < lo) p2 *= 2;
  int64_t best = p2;
  std::vector<int> f;
  factor_device(p2, f);
  double best_cost = double(p2) * double(f.size() + 1);
  for (int64_t m = lo; m < p2; ++m) {
    if (!factor_device(m, f)) continue;
    const double cost = double(m) * double(f.size() + 1);
    if (cost < best_cost) {
      best_cost = cost;
      best = m;
    }
  }
  return best;
}

// ---------------------------------------------------------------------------
size_t Builder::add(const std::vector<cd>& v) {
  const size_t eb = dbl ? 16 : 8;
  size_t off = (blob.size() + 255) & ~size_t(255);
  blob.resize(off + v.size() * eb);
  unsigned char* p = blob.data() + off;
  for (size_t i = 0; i < v.size(); ++i) {
    if (dbl) {
      double t[2] = {v[i].real(), v[i].imag()};
      std::memcpy(p + i * 16, t, 16);
    } else {
      float t[2] = {float(v[i].real()), float(v[i].imag())};
      std::memcpy(p + i * 8, t, 8);
    }
  }
  return off;
}

// Stage list + stage twiddle table for a shared-memory transform of length n.
bool Builder::stages_for(int n, PassSpec& ps) {
  std::vector<int> f;
  if (!factor_device(n, f) || int(f.size()) > kMaxStages) return false;
  auto it = stage_cache.find(n);
  std::vector<int> offs(f.size());
  if (it == stage_cache.end()) {
    std::vector<cd> t;
    int64_t Ns = 1;
    // stage (Ns, R): W_{Ns*R}^{p*r}, 0 < r < R, at (r - 1)*Ns + p (p fastest:
    // the butterflies of neighbouring threads read neighbouring entries)
    for (size_t s = 0; s < f.size(); ++s) {
      offs[s] = int(t.size());
      const int R = f[s];
      for (int r = 1; r < R; ++r)
        for (int64_t p = 0; p < Ns; ++p) t.push_back(unit_root(p * r, Ns * R));
      Ns *= R;
    }
    if (t.empty()) t.push_back(cd(1, 0));
    StageTable st;
    st.off = add(t);
    st.offs = offs;
    it = stage_cache.emplace(n, st).first;
  }
  ps.tw_off = int64_t(it->second.off);
  ps.d.n = n;
  ps.d.nstages = int(f.size());
  int Ns = 1;
  for (size_t s = 0; s < f.size(); ++s) {
    ps.d.st[s].radix = f[s];
    ps.d.st[s].ns = Ns;
    ps.d.st[s].tw_off = it->second.offs[s];
    Ns *= f[s];
  }
  return true;
}

// Four-step twiddle tables W_N^t = hi[t >> shift] * lo[t & mask].  N is a
// four-step length n1 * n2 with both halves at most the tile cap (8192),
// so N <= 2^26 and the exponents t < N fit the kernels' 32-bit arithmetic.
void Builder::tw4_for(int64_t N, PassSpec& ps) {
  int shift = 0;
  while ((int64_t(1) << (2 * shift)) < N) ++shift;
  auto it = tw4_cache.find(N);
  if (it == tw4_cache.end()) {
    const int64_t B = int64_t(1) << shift;
    std::vector<cd> lo(static_cast<size_t>(B)), hi(static_cast<size_t>((N + B - 1) / B));
    for (int64_t t = 0; t < B; ++t) lo[size_t(t)] = unit_root(t, N);
    for (int64_t t = 0; t < int64_t(hi.size()); ++t) hi[size_t(t)] = unit_root(t * B, N);
    Tw4 tw;
    tw.lo = add(lo);
    tw.hi = add(hi);
    tw.shift = shift;
    it = tw4_cache.emplace(N, tw).first;
  }
  ps.tw4lo_off = int64_t(it->second.lo);
  ps.tw4hi_off = int64_t(it->second.hi);
  ps.d.tw4_shift = it->second.shift;
  ps.d.tw4_n = N;
}

// chirp c[l] = exp(-i*pi*(l^2 mod 2n)/n), l < n; filter = DFT_m(b)/m with
// b[l] = conj(c[|l|]) on the wrapped indices (-n, n).
void blue_tables(int64_t n, int64_t m, std::vector<cd>& chirp, std::vector<cd>& b) {
  chirp.assign(static_cast<size_t>(n), cd(0, 0));
  b.assign(static_cast<size_t>(m), cd(0, 0));
  for (int64_t l = 0; l < n; ++l) {
    const int64_t q = int64_t((__int128(l) * l) % (2 * n));
    chirp[size_t(l)] = unit_root(q, 2 * n);  // exp(-2*pi*i*q/(2n)) = exp(-i*pi*q/n)
  }
  for (int64_t l = 0; l < n; ++l) {
    b[size_t(l)] = std::conj(chirp[size_t(l)]);
    if (l > 0) b[size_t(m - l)] = std::conj(chirp[size_t(l)]);
  }
  host_fft_fp64(b);
  const double inv = 1.0 / double(m);
  for (auto& v : b) v *= inv;
}

void Builder::precompute_blue(const std::vector<std::pair<int64_t, int64_t>>& nm) {
  std::vector<std::pair<int64_t, int64_t>> todo;
  for (const auto& k : nm)
    if (!blue_cache.count(k) && !blue_pre.count(k)) todo.push_back(k);
  std::sort(todo.begin(), todo.end());
  todo.erase(std::unique(todo.begin(), todo.end()), todo.end());
  if (todo.empty()) return;
  std::vector<std::pair<std::vector<cd>, std::vector<cd>>> res(todo.size());
  std::atomic<size_t> next{0};
  unsigned nt = std::max(1u, std::thread::hardware_concurrency());
  nt = std::min<unsigned>(nt, unsigned(todo.size()));
  std::vector<std::thread> pool;
  for (unsigned t = 0; t < nt; ++t)
    pool.emplace_back([&] {
      for (size_t i; (i = next.fetch_add(1)) < todo.size();)
        blue_tables(todo[i].first, todo[i].second, res[i].first, res[i].second);
    });
  for (auto& th : pool) th.join();
  for (size_t i = 0; i < todo.size(); ++i) blue_pre.emplace(todo[i], std::move(res[i]));
}

void Builder::blue_for(int64_t n, int64_t m, PassSpec& ps) {
  auto key = std::make_pair(n, m);
  auto it = blue_cache.find(key);
  if (it == blue_cache.end()) {
    std::vector<cd> chirp, b;
    auto pre = blue_pre.find(key);
    if (pre != blue_pre.end()) {
      chirp.swap(pre->second.first);
      b.swap(pre->second.second);
      blue_pre.erase(pre);
    } else {
      blue_tables(n, m, chirp, b);
    }
    Blue bl;
    bl.chirp = add(chirp);
    bl.filter = add(b);
    it = blue_cache.emplace(key, bl).first;
  }
  ps.chirp_off = int64_t(it->second.chirp);
  ps.filter_off = int64_t(it->second.filter);
}

size_t Builder::roots_for(int64_t N) {
  auto it = roots_cache.find(N);
  if (it != roots_cache.end()) return it->second;
  std::vector<cd> t(static_cast<size_t>(N));
  for (int64_t i = 0; i < N; ++i) t[size_t(i)] = unit_root(i, N);
  const size_t off = add(t);
  roots_cache.emplace(N, off);
  return off;
}

void choose_tile(PassSpec& ps, bool dbl) {
  PassDesc& d = ps.d;
  const int n = d.n;
  const int eb = dbl ? 16 : 8;
  int pitch = n + (n >> 4) + 1;
  if (pitch % 2 == 0) ++pitch;
  const int64_t smem_cap = 227 * 1024;
  int wmax = int(smem_cap / (int64_t(2) * pitch * eb));
  if (wmax < 1) wmax = 1;
  const bool strided = (d.in_cs == 1 && d.in_es != 1) || (d.out_cs == 1 && d.out_es != 1);
  const int target = dbl ? 2048 : 4096;
  int W = std::max(1, target / n);
  if (strided) W = std::max(W, 16);
  W = std::min(W, wmax);
  if (int64_t(W) > d.ncols) W = int(std::max<int64_t>(1, d.ncols));
  d.W = W;
  d.pitch = pitch;
  d.threads = (int64_t(W) * n >= 8192) ? 512 : 256;
  d.load_cfast = (d.in_cs == 1 && d.in_es != 1) ? 1 : 0;
  d.store_cfast = (d.out_cs == 1 && d.out_es != 1) ? 1 : 0;
}

static PassSpec blank_pass() {
  PassSpec ps;
  std::memset(&ps.d, 0, sizeof(ps.d));
  ps.d.nb_lo = 1;
  ps.d.nbatch = 1;
  ps.d.scale = 1.0;
  ps.d.tw4_n = 1;
  return ps;
}

// Strided halves (consecutive columns adjacent in the source) run on the
// register-resident strided kernel when their length has one.
static void use_strided(PassSpec& ps, bool dbl) {
  PassDesc& d = ps.d;
  if (d.in_cs == 1 && d.in_es != 1 && str_kernel_available(d.n, dbl) && str_ops_supported(d.flags) &&
      !feature_disabled("strided")) {
    d.kernel = K_STRIDED;
    d.W = str_kernel_width(dbl);
  }
}

static int cap_for(bool dbl) { return dbl ? kCapC64 : kCapC32; }

// Split n = n1*n2 (n1 strided first pass, n2 second) with both <= cap,
// n1 as close to sqrt(n) as possible.
// Factorisation n = n1 * n2 of a four-step axis, both halves within one CTA.
// Candidates are ranked by balance, with a bonus for halves that have a
// register-resident strided kernel; `rank` picks the rank-th best (the
// autotuner's knob), clamped to the number of candidates.
static bool split_four_step(int64_t n, int cap, int64_t& n1, int64_t& n2, bool dbl = false, int rank = 0) {
  // divisors of n (n is 7-smooth here): every product of its prime powers
  std::vector<int64_t> divs{1};
  {
    int64_t m = n;
    for (int p : {2, 3, 5, 7}) {
      int e = 0;
      while (m % p == 0) {
        m /= p;
        ++e;
      }
      const size_t k = divs.size();
      int64_t pw = 1;
      for (int i = 0; i < e; ++i) {
        pw *= p;
        for (size_t j = 0; j < k; ++j) divs.push_back(divs[j] * pw);
      }
    }
    if (m != 1) return false;
    std::sort(divs.begin(), divs.end());
  }
  std::vector<std::pair<double, int64_t>> cand;
  for (int64_t a : divs) {
    if (a < 2 || a > cap || a >= n) continue;
    const int64_t b = n / a;
    if (b > cap || b < 2) continue;
    double dd = std::fabs(std::log(double(a)) - std::log(double(b)));
    if (str_kernel_available(int(a), dbl)) dd -= 2.0;
    if (str_kernel_available(int(b), dbl)) dd -= 2.0;
    cand.push_back({dd, a});
  }
  if (cand.empty()) return false;
  std::stable_sort(cand.begin(), cand.end(),
                   [](const std::pair<double, int64_t>& x, const std::pair<double, int64_t>& y) {
                     return x.first < y.first;
                   });
  const size_t k = std::min(cand.size() - 1, size_t(std::max(rank, 0)));
  n1 = cand[k].second;
  n2 = n / n1;
  return true;
}

// "16.16.8": the stage radices of a pass, for plan descriptions.
static std::string radix_list(const PassDesc& d) {
  std::string r;
  for (int i = 0; i < d.nstages; ++i) {
    if (i) r += '.';
    r += std::to_string(d.st[i].radix);
  }
  return r;
}

// Complex Double 1024-point vectors up to this many per axis run one per
// 8-CTA cluster (vec1024.cu); more go to the throughput kernels.
constexpr int64_t kVecMaxCols = 16;

// Appends the passes of one axis.  `first`: this axis reads the user's
// input; later axes work on the output buffer.
int add_axis(Builder& B, std::vector<PassSpec>& passes, const Axis& ax, bool first,
             int64_t& scratch1, int64_t& scratch2, std::string& desc, int cap_in, const TuneChoice* tc) {
  const TuneChoice defaults;
  if (!tc) tc = &defaults;
  const int split_rank = tc->split_rank, blue_pad = tc->blue_pad;
  // register row kernel unless chosen off; by rule, not for Complex Double
  // with fewer rows than 64 (one FP64 row gives it only N/16 threads: the
  // generic tile measured 29 vs 48 us on fft1D 1024)
  const bool use_row = tc->row_kernel >= 0 ? tc->row_kernel != 0 : !(B.dbl && ax.ncols * ax.outer < 64);
  const bool dbl = B.dbl;
  const int cap = cap_in > 0 ? cap_in : cap_for(dbl);
  const int src = first ? R_IN : R_OUT;
  char buf[256];
  if (ax.n <= 1) return GBFFT_OK;

  // A long strided axis (columns of a 2-D array, middle / outer axes of 3-D)
  // with no strided kernel of its own goes four-step above 2048 when a half
  // of the split has a strided kernel: in one generic tile it would hold
  // only one or two columns and read short row segments (fft2D 8192^2: 1.65
  // ms that way, 0.68 ms four-step with both halves on the strided kernels;
  // 6144^2: 1.17 -> 0.98 ms with one).  With two generic halves the split
  // measured slower (3000^2: 0.36 against 0.30 ms), and 2048 (a 32-point
  // generic half) no faster, so those stay one pass.
  const bool own_strided_kernel =
      ax.cs == 1 && ((ax.n == 4096 && ax.ncols % (dbl ? 16 : 8) == 0 && !feature_disabled("cluster")) ||
                     (str_kernel_available(int(ax.n), dbl) && ax.ncols % str_kernel_width(dbl) == 0 &&
                      !feature_disabled("strided")));
  bool long_strided = ax.es != 1 && ax.n > 2048 && ax.cs == 1 && ax.ncols == ax.es && is_fast_length(ax.n) &&
                      !own_strided_kernel && !feature_disabled("longcol");
  if (long_strided) {
    int64_t h1 = 0, h2 = 0;
    long_strided = split_four_step(ax.n, cap, h1, h2, dbl, split_rank) &&
                   (str_kernel_available(int(h1), dbl) || str_kernel_available(int(h2), dbl));
  }

  if (is_fast_length(ax.n) && ax.n <= cap && !long_strided) {
    PassSpec ps = blank_pass();
    if (!B.stages_for(int(ax.n), ps)) return GBFFT_ERR_UNSUPPORTED;
    PassDesc& d = ps.d;
    d.in_es = d.out_es = ax.es;
    d.in_cs = d.out_cs = ax.cs;
    d.in_bs = d.out_bs = ax.os;
    d.ncols = ax.ncols;
    d.nbatch = d.nb_lo = ax.outer;
    choose_tile(ps, dbl);
    const char* kname = "pencil";
    if (ax.es == 1 && ax.outer == 1 && ax.ncols <= kVecMaxCols && vec1024_available(ax.n, dbl) &&
        tc->row_kernel != 0 && !feature_disabled("vec")) {
      // a few Complex Double vectors of 1024: one cluster of 8 CTAs each,
      // one element per thread (latency path)
      d.kernel = K_VEC1024;
      ps.tw_off = int64_t(B.roots_for(1024));
      kname = "vec1024-cluster8";
    } else if (ax.es == 1 && ax.outer == 1 && use_row && row_kernel_available(int(ax.n), dbl) &&
        !feature_disabled("row")) {
      d.kernel = K_ROW;
      kname = "row";
    } else if (ax.n == 4096 && ax.cs == 1 && ax.es != 1 && ax.ncols % (dbl ? 16 : 8) == 0 &&
               !feature_disabled("cluster")) {
      d.kernel = K_COL4096;
      ps.tw_off = int64_t(B.roots_for(4096));
      kname = "col4096-cluster8";
    } else if (ax.cs == 1 && ax.es != 1 && str_kernel_available(int(ax.n), dbl) &&
               ax.ncols % str_kernel_width(dbl) == 0 && !feature_disabled("strided")) {
      d.kernel = K_STRIDED;
      d.W = str_kernel_width(dbl);
      kname = "strided";
    }
    ps.src = src;
    ps.dst = R_OUT;
    ps.d.lout_es = 1;  // axis index = element index k
    ps.d.lout_cs = 0;
    ps.axis_final = ps.rot_ok = true;
    ps.axis_n = ax.n;
    ps.rot_stride = ax.es;
    passes.push_back(ps);
    std::snprintf(buf, sizeof buf, "[n=%lld r=%s es=%lld %s W=%d]", (long long)ax.n, radix_list(ps.d).c_str(),
                  (long long)ax.es, kname, ps.d.W);
    desc += buf;
    return GBFFT_OK;
  }

  if (is_fast_length(ax.n)) {
    int64_t n1, n2;
    if (!split_four_step(ax.n, cap, n1, n2, dbl, split_rank)) return GBFFT_ERR_UNSUPPORTED;
    PassSpec p1 = blank_pass(), p2 = blank_pass();
    if (!B.stages_for(int(n1), p1) || !B.stages_for(int(n2), p2)) return GBFFT_ERR_UNSUPPORTED;
    B.tw4_for(ax.n, p1);
    p1.d.flags |= F_TW4;
    const int mid = first ? R_OUT : R_S1;
    if (!first) scratch1 = std::max(scratch1, ax.n * ax.ncols * ax.outer);
    if (ax.es == 1) {
      // contiguous rows: c indexes rows (stride cs)
      PassDesc& a = p1.d;
      a.nbatch = a.nb_lo = ax.ncols * ax.outer;
      if (ax.outer > 1 && ax.os != ax.ncols * ax.cs) return GBFFT_ERR_UNSUPPORTED;
      a.in_bs = a.out_bs = ax.cs;
      a.ncols = n2;
      a.in_cs = 1;
      a.in_es = n2;
      a.out_es = 1;
      a.out_cs = n1;
      PassDesc& b = p2.d;
      b.nbatch = b.nb_lo = ax.ncols * ax.outer;
      b.in_bs = b.out_bs = ax.cs;
      b.ncols = n1;
      b.in_cs = b.out_cs = 1;
      b.in_es = b.out_es = n1;
    } else {
      // strided axis of stride S = es over cs == 1 columns
      if (ax.cs != 1 || ax.ncols != ax.es) return GBFFT_ERR_UNSUPPORTED;
      const int64_t S = ax.es;
      PassDesc& a = p1.d;
      a.nb_lo = n2;
      a.nbatch = n2 * ax.outer;
      a.in_bs = S;
      a.out_bs = n1 * S;
      a.in_bs2 = a.out_bs2 = ax.os;
      a.ncols = S;
      a.in_cs = a.out_cs = 1;
      a.in_es = n2 * S;
      a.out_es = S;
      a.flags |= F_TW4_BATCH;
      PassDesc& b = p2.d;
      b.nb_lo = n1;
      b.nbatch = n1 * ax.outer;
      b.in_bs = b.out_bs = S;
      b.in_bs2 = b.out_bs2 = ax.os;
      b.ncols = S;
      b.in_cs = b.out_cs = 1;
      b.in_es = b.out_es = n1 * S;
    }
    choose_tile(p1, dbl);
    choose_tile(p2, dbl);
    use_strided(p1, dbl);
    use_strided(p2, dbl);
    p1.src = src;
    p1.dst = mid;
    p2.src = mid;
    p2.dst = R_OUT;
    p2.axis_final = true;
    p2.axis_n = ax.n;
    if (ax.es == 1) {
      // rows: output k = k1 + n1*k2, k2 the element index, k1 the column
      p2.d.lout_es = n1;
      p2.d.lout_cs = 1;
      p2.rot_ok = true;
      p2.rot_stride = 1;
    }
    passes.push_back(p1);
    passes.push_back(p2);
    std::snprintf(buf, sizeof buf, "[n=%lld=%lldx%lld four-step es=%lld W=%d,%d]", (long long)ax.n,
                  (long long)n1, (long long)n2, (long long)ax.es, p1.d.W, p2.d.W);
    desc += buf;
    return GBFFT_OK;
  }

  // Bluestein.  Single pass: the power of two when it is at most 1/8 longer
  // than the cheapest smooth length (radix-16 stages are the fastest per
  // element; 1009 pads to 2048 rather than 2025 = 15 x 15 x 9), unless the
  // autotuner chose the smooth length (blue_pad 0).
  int64_t m = bluestein_length(ax.n);
  if (blue_pad > 0 && m <= cap) {
    int64_t mp = 1;
    while (mp < 2 * ax.n - 1) mp <<= 1;
    if (mp <= cap && 8 * mp <= 9 * m) m = mp;
  }
  if (m <= cap) {
    PassSpec ps = blank_pass();
    if (!B.stages_for(int(m), ps)) return GBFFT_ERR_UNSUPPORTED;
    B.blue_for(ax.n, m, ps);
    PassDesc& d = ps.d;
    d.in_es = d.out_es = ax.es;
    d.in_cs = d.out_cs = ax.cs;
    d.in_bs = d.out_bs = ax.os;
    d.ncols = ax.ncols;
    d.nbatch = d.nb_lo = ax.outer;
    d.flags |= F_PAD_IN | F_CHIRP_IN | F_BLUE | F_TRUNC_OUT;
    d.lin_es = 1;
    d.lin_cs = 0;
    d.lout_es = 1;
    d.lout_cs = 0;
    d.n_in = ax.n;
    d.n_out = ax.n;
    choose_tile(ps, dbl);
    const bool rowk =
        ax.es == 1 && ax.outer == 1 && use_row && row_blue_available(int(m), dbl) && !feature_disabled("row");
    if (rowk) d.kernel = K_ROW;  // register-resident rows
    ps.src = src;
    ps.dst = R_OUT;
    ps.axis_final = ps.rot_ok = true;  // axis index = k (lout_es 1, lout_cs 0)
    ps.axis_n = ax.n;
    ps.rot_stride = ax.es;
    passes.push_back(ps);
    std::snprintf(buf, sizeof buf, "[n=%lld bluestein m=%lld es=%lld %s W=%d]", (long long)ax.n,
                  (long long)m, (long long)ax.es, rowk ? "row" : "pencil", ps.d.W);
    desc += buf;
    return GBFFT_OK;
  }

  // multi-pass Bluestein: contiguous rows only
  if (ax.es != 1) return GBFFT_ERR_UNSUPPORTED;
  if (ax.outer > 1 && ax.os != ax.ncols * ax.cs) return GBFFT_ERR_UNSUPPORTED;
  return add_bluestein_multipass(B, passes, ax, src,
                                 bluestein_multipass_length(ax.n, cap, dbl,
                                                            blue_pad > 0    ? 2.5
                                                            : blue_pad == 0 ? 1.0
                                                                            : tc->blue_weight),
                                 cap, split_rank,
                                 scratch1, scratch2, desc);
}

// Padded length of a multi-pass Bluestein transform: the 7-smooth m in
// [2n - 1, next power of two] with the least m * (c(m1) + c(m2)), where
// m = m1 * m2 is the four-step split and c(h) is 1 for a half with a
// register-resident strided kernel and `generic` otherwise (2.5 for plans:
// the generic tile measured 2.3-3.4x slower per element than the tensor-fed
// strided kernel on 65536 = 256 x 256; the ragged executor passes its own
// weight).  With generic = 1 this is the smallest smooth m.
int64_t bluestein_multipass_length(int64_t n, int cap, bool dbl, double generic) {
  const int64_t lo = 2 * n - 1;
  int64_t hi = 1;
  while (hi < lo) hi <<= 1;
  int64_t best = hi;
  double best_cost = 1e300;
  for (int64_t m = lo; m <= hi; ++m) {
    if (!is_fast_length(m)) continue;
    int64_t a = 0, b = 0;
    if (!split_four_step(m, cap, a, b, dbl)) continue;
    const double ca = str_kernel_available(int(a), dbl) ? 1.0 : generic;
    const double cb = str_kernel_available(int(b), dbl) ? 1.0 : generic;
    const double cost = double(m) * (ca + cb);
    if (cost < best_cost) {
      best_cost = cost;
      best = m;
    }
  }
  return best;
}

// Multi-pass Bluestein over rows of length n padded to m = m1 * m2 (three
// passes).  With j = j1*m2 + j2 and k = k1 + m1*k2 the forward four-step
// gives X[k] in S1 laid out [k2][k1] after its second half; the inverse DFT
// (taken as a forward DFT of the conjugate) is decomposed with output index
// j = j2 + m2*j1, whose first half is a DFT over k2 -- the axis the forward
// transform has just produced in registers.  So the middle pass runs: DFT
// over j2 -> k2, multiply by the filter, conjugate, DFT over k2 -> j2,
// twiddle W_m^(k1*j2), transposed store; the last pass does the DFT over
// k1 -> j1, conjugate, chirp and the first n outputs.
//   P1:  src -> S1[j2][k1]  chirp + zero pad, DFT over j1, twiddle W_m^(j2*k1)
//   P23: S1 -> S2[k1][j2]   DFT over j2, filter, conj, DFT over k2, W_m^(k1*j2)
//   P4:  S2 -> dst          DFT over k1, conj, chirp, y[j2 + m2*j1] for j < n
int add_bluestein_multipass(Builder& B, std::vector<PassSpec>& passes, const Axis& ax, int src, int64_t m,
                            int cap, int split_rank, int64_t& scratch1, int64_t& scratch2, std::string& desc) {
  const bool dbl = B.dbl;
  char buf[256];
  int64_t m1, m2;
  if (!split_four_step(m, cap, m1, m2, dbl, split_rank)) return GBFFT_ERR_UNSUPPORTED;
  const int64_t rows = ax.ncols * ax.outer;
  scratch1 = std::max(scratch1, rows * m);
  scratch2 = std::max(scratch2, rows * m);
  PassSpec p[3] = {blank_pass(), blank_pass(), blank_pass()};
  for (int i = 0; i < 3; ++i) {
    if (!B.stages_for(int(i == 1 ? m2 : m1), p[i])) return GBFFT_ERR_UNSUPPORTED;
    B.blue_for(ax.n, m, p[i]);
    p[i].d.nbatch = p[i].d.nb_lo = rows;
  }
  {  // P1: column j2 < m2 of x[j1*m2 + j2] (j < n, else zero), out S1[j2*m1 + k1]
    PassDesc& d = p[0].d;
    B.tw4_for(m, p[0]);
    d.in_bs = ax.cs;
    d.out_bs = m;
    d.ncols = m2;
    d.in_cs = 1;
    d.in_es = m2;
    d.out_es = 1;
    d.out_cs = m1;
    d.lin_es = m2;
    d.lin_cs = 1;
    d.n_in = ax.n;
    d.flags |= F_PAD_IN | F_CHIRP_IN | F_TW4;
  }
  {  // P23: column k1 < m1 of S1[j2*m1 + k1]; filter index k2*m1 + k1; out S2[k1*m2 + j2]
    PassDesc& d = p[1].d;
    B.tw4_for(m, p[1]);
    d.in_bs = d.out_bs = m;
    d.ncols = m1;
    d.in_cs = 1;
    d.in_es = m1;
    d.out_es = 1;
    d.out_cs = m2;
    d.lout_es = m1;
    d.lout_cs = 1;
    d.flags |= F_SPEC | F_TW4;
  }
  {  // P4: column j2 < m2 of S2[k1*m2 + j2]; out y[j1*m2 + j2] for j < n
    PassDesc& d = p[2].d;
    d.in_bs = m;
    d.out_bs = ax.cs;
    d.ncols = m2;
    d.in_cs = d.out_cs = 1;
    d.in_es = d.out_es = m2;
    d.lout_es = m2;
    d.lout_cs = 1;
    d.n_out = ax.n;
    d.flags |= F_CHIRP_OUT | F_TRUNC_OUT;
  }
  p[0].src = src;
  p[0].dst = R_S1;
  p[1].src = R_S1;
  p[1].dst = R_S2;
  p[2].src = R_S2;
  p[2].dst = R_OUT;
  p[2].axis_final = p[2].rot_ok = true;  // axis index j1*m2 + j2 (lout_es m2, lout_cs 1)
  p[2].axis_n = ax.n;
  p[2].rot_stride = 1;
  for (int i = 0; i < 3; ++i) {
    choose_tile(p[i], dbl);
    use_strided(p[i], dbl);
    passes.push_back(p[i]);
  }
  std::snprintf(buf, sizeof buf, "[n=%lld bluestein m=%lld=%lldx%lld 3-pass]", (long long)ax.n,
                (long long)m, (long long)m1, (long long)m2);
  desc += buf;
  return GBFFT_OK;
}

bool fault_injected(const char* what) {
  const char* e = std::getenv("GBFFT_FAULT_INJECT");
  return e && std::strstr(e, what) != nullptr;
}

bool feature_enabled(const char* what) {
  const char* e = std::getenv("GBFFT_ENABLE");
  return e && std::strstr(e, what) != nullptr;
}

bool feature_disabled(const char* what) {
  const char* e = std::getenv("GBFFT_DISABLE");
  return e && std::strstr(e, what) != nullptr;
}

}  // namespace gbfft

using namespace gbfft;

namespace gbfft {

// Creates a plan.  `forced`: build with these choices (the autotuner's
// candidates); else the autotuner cache's choice for this device and shape,
// else -- with GBFFT_AUTOTUNE=1 -- a fresh search, else the defaults.
int create_plan(gbfft_plan** out, int rank, const int64_t* dims, int kind, int dtype, int precision,
                const TuneChoice* forced) {
  if (!out) return GBFFT_ERR_INVALID_ARG;
  *out = nullptr;
  if (rank < 1 || rank > 5 || !dims) return GBFFT_ERR_INVALID_ARG;
  if (kind != GBFFT_KIND_MANY && kind != GBFFT_KIND_FULL) return GBFFT_ERR_INVALID_ARG;
  // rank 4-5: the innermost-axis transform only (as FFT.hs:63-84); no full 4D/5D
  if (kind == GBFFT_KIND_FULL && rank > 3) return GBFFT_ERR_UNSUPPORTED;
  if (dtype != GBFFT_C32 && dtype != GBFFT_C64) return GBFFT_ERR_INVALID_ARG;
  if (precision != GBFFT_PLAIN && precision != GBFFT_SPLIT_FP16) return GBFFT_ERR_INVALID_ARG;
  int64_t total = 1;
  for (int i = 0; i < rank; ++i) {
    if (dims[i] < 0) return GBFFT_ERR_INVALID_ARG;
    if (dims[i] > 0 && total > (int64_t(1) << 40) / dims[i]) return GBFFT_ERR_UNSUPPORTED;
    total *= dims[i];
  }
  if (precision == GBFFT_SPLIT_FP16 && dtype != GBFFT_C32) return GBFFT_ERR_INVALID_ARG;
  std::unique_ptr<gbfft_plan> p(new gbfft_plan);
  p->rank = rank;
  for (int i = 0; i < rank; ++i) p->dims[i] = dims[i];
  p->kind = kind;
  p->dtype = dtype;
  p->precision = precision;
  p->dbl = dtype == GBFFT_C64;
  p->total = total;
  if (cudaGetDevice(&p->device) != cudaSuccess) return GBFFT_ERR_CUDA;
  if (prepare_kernels() != cudaSuccess) return GBFFT_ERR_CUDA;
  if (forced) {
    p->tune = *forced;
  } else if (total > 0) {
    const std::string key = tune_key(rank, dims, kind, dtype, precision);
    TuneChoice c;
    if (tune_lookup(key, c)) {
      p->tune = c;
    } else if (const char* at = std::getenv("GBFFT_AUTOTUNE"); at && at[0] == '1') {
      if (autotune_plan(rank, dims, kind, dtype, precision, nullptr, c, nullptr) == GBFFT_OK) p->tune = c;
    }
  }
  const int64_t norm = (kind == GBFFT_KIND_FULL) ? total : dims[rank - 1];
  p->inv_norm = norm > 0 ? 1.0 / double(norm) : 1.0;
  if (total > 0) {
    const int st = precision == GBFFT_SPLIT_FP16 ? build_split_plan(p.get()) : build_plan(p.get(), false);
    if (st != GBFFT_OK) {
      gbfft_plan_destroy(p.release());
      return st;
    }
  }
  *out = p.release();
  return GBFFT_OK;
}

int build_plan(gbfft_plan* p, bool dry) {
  Builder B;
  B.dbl = p->dbl;
  const int64_t* dm = p->dims;
  std::vector<Axis> axes;
  const int r = p->rank;
  const int64_t w = dm[r - 1];
  const int64_t rows = p->total / std::max<int64_t>(1, w);
  // innermost axis: contiguous rows
  axes.push_back(Axis{w, 1, w, rows, rows * w, 1});
  if (p->kind == GBFFT_KIND_FULL) {
    if (r == 2) axes.push_back(Axis{dm[0], w, 1, w, dm[0] * w, 1});
    if (r == 3) {
      const int64_t d0 = dm[0], h = dm[1];
      axes.push_back(Axis{h, w, 1, w, h * w, d0});   // y: stride w, outer z
      axes.push_back(Axis{d0, h * w, 1, h * w, d0 * h * w, 1});  // z
    }
  }
  // A four-step axis writes a transposed intermediate and must read the
  // user's input to avoid scratch: put the first such axis first.
  const int cap = cap_for(p->dbl);
  std::stable_sort(axes.begin(), axes.end(), [&](const Axis& a, const Axis& b) {
    const bool fa = is_fast_length(a.n) && a.n > cap;
    const bool fb = is_fast_length(b.n) && b.n > cap;
    return fa && !fb;
  });
  int64_t s1 = 0, s2 = 0;
  char head[128];
  std::snprintf(head, sizeof head, "%s %s rank%d", p->dbl ? "c64" : "c32",
                p->kind == GBFFT_KIND_FULL ? "full" : "many", r);
  p->desc = head;
  bool first = true;
  for (const Axis& ax : axes) {
    if (ax.n <= 1) continue;
    const size_t before = p->passes.size();
    int st = add_axis(B, p->passes, ax, first, s1, s2, p->desc, 0, &p->tune);
    if (st != GBFFT_OK) return st;
    if (p->passes.size() > before) first = false;
  }
  // x and y of 256 x 256 planes (fft2D 256^2, fft3D d x 256 x 256): one
  // cluster pass per plane (plane.cu) instead of two HBM passes
  // Opt-in (GBFFT_ENABLE=plane): measured on GB300 the fused pass takes
  // 99 us for the 256 planes of 256^3 against 48 + 46 us for the two passes
  // it replaces, so the two passes stay the default.  (Split-FP16 plans keep
  // the row pass: it is the one they move to the tensor cores.)
  if (p->kind == GBFFT_KIND_FULL && r >= 2 && plane_available(dm[r - 2], dm[r - 1], p->dbl) &&
      p->precision != GBFFT_SPLIT_FP16 && p->passes.size() >= 2 && feature_enabled("plane")) {
    const PassSpec& px = p->passes[0];
    const PassSpec& py = p->passes[1];
    if (px.axis_final && py.axis_final && px.axis_n == dm[r - 1] && py.axis_n == dm[r - 2] && px.src == R_IN &&
        px.dst == R_OUT && py.src == R_OUT && py.dst == R_OUT) {
      PassSpec f;
      std::memset(&f.d, 0, sizeof(PassDesc));
      f.d.kernel = K_PLANE;
      f.d.n = int(dm[r - 1]);
      f.d.ncols = p->total / (dm[r - 1] * dm[r - 2]);
      f.d.nbatch = f.d.nb_lo = 1;
      f.d.in_bs = f.d.out_bs = dm[r - 1] * dm[r - 2];
      f.d.scale = 1.0;
      f.d.tw4_n = 1;
      f.tw_off = int64_t(B.roots_for(dm[r - 1]));
      f.src = R_IN;
      f.dst = R_OUT;
      f.axis_final = true;  // of both plane axes: no fused rotation offered
      f.rot_ok = false;
      f.axis_n = dm[r - 1];
      p->passes.erase(p->passes.begin(), p->passes.begin() + 2);
      p->passes.insert(p->passes.begin(), f);
      p->desc += " [x+y: 256x256 planes in one cluster pass]";
    }
  }
  // device status word (zero) at the head of the tables
  const size_t status_off = B.add(std::vector<cd>(2, cd(0, 0)));
  // device tables
  const size_t eb = p->dbl ? 16 : 8;
  if (dry) {
    p->tables_bytes = B.blob.size();
    p->scratch_bytes = size_t(s1 + s2) * eb;
    return GBFFT_OK;
  }
  if (!B.blob.empty()) {
    if (fault_injected("alloc")) return GBFFT_ERR_ALLOC;
    p->tables_bytes = B.blob.size();
    if (cudaMalloc(&p->d_tables, p->tables_bytes) != cudaSuccess) return GBFFT_ERR_ALLOC;
    if (cudaMemcpy(p->d_tables, B.blob.data(), p->tables_bytes, cudaMemcpyHostToDevice) != cudaSuccess)
      return GBFFT_ERR_CUDA;
  }
  if (s1 + s2 > 0) {
    if (fault_injected("alloc")) return GBFFT_ERR_ALLOC;
    const size_t b1 = ((size_t(s1) * eb) + 255) & ~size_t(255);
    p->s2_off = b1;
    p->scratch_bytes = b1 + size_t(s2) * eb;
    if (cudaMalloc(&p->d_scratch, p->scratch_bytes) != cudaSuccess) return GBFFT_ERR_ALLOC;
    if (cudaEventCreateWithFlags(&p->scratch_ev, cudaEventDisableTiming) != cudaSuccess) return GBFFT_ERR_CUDA;
  }
  // L2 policy: a pass whose output a later pass reads back stores it with
  // evict_last; every pass after the first streams its input (evict_first)
  if (p->passes.size() > 1 && !feature_disabled("l2hint")) {
    for (size_t i = 0; i < p->passes.size(); ++i) {
      if (i + 1 < p->passes.size()) p->passes[i].d.flags |= F_L2_OUT_LAST;
      p->passes[i].d.flags |= F_L2_IN_FIRST;
    }
  }
  unsigned char* base = static_cast<unsigned char*>(p->d_tables);
  p->d_status = reinterpret_cast<int*>(base + status_off);
  const bool tma = !feature_disabled("tma");
  const gbfft::TuneChoice& tc = p->tune;
  for (PassSpec& ps : p->passes) {
    ps.d.status = p->d_status;
    // tensor / bulk copies per kernel kind as chosen (defaults: measured on
    // GB300); GBFFT_DISABLE=tma turns every one off for A/B checks,
    // GBFFT_ROW_TMA=1 streams register rows by bulk copies
    // untuned: Complex Float rows of 4096 streamed by bulk copies (fft2D 4096^2
    // row pass 51.8 against 53.9 us); other lengths measured faster without
    // (1000: 0.216 against 0.193 ms for 65536 rows; 256: 49.8 against 45.7 us)
    int row_tma = tc.row_tma >= 0 ? tc.row_tma : (ps.d.kernel == K_ROW && ps.d.n == 4096 && !p->dbl) ? 1 : 0;
    if (const char* rt = std::getenv("GBFFT_ROW_TMA")) row_tma = std::atoi(rt) & 1;
    const int want = ps.d.kernel == K_ROW ? row_tma : ps.d.kernel == K_STRIDED ? tc.str_tma : 1;
    ps.d.use_tma = (tma && want) ? 1 : 0;
    // untuned: Complex Float register rows double-buffered (measured faster
    // at every length); Complex Double rows single-buffered (half the shared
    // memory per CTA); tensor-core rows at their lower CTAs-per-SM bound
    ps.d.row_variant = tc.row_variant >= 0 ? tc.row_variant : (ps.d.kernel == K_ROW && !p->dbl) ? 0 : 1;
    ps.d.col_variant = tc.col_variant;
    if (const char* rv = std::getenv("GBFFT_ROW_VARIANT")) ps.d.row_variant = std::atoi(rv) & 1;
    if (const char* cv = std::getenv("GBFFT_COL_VARIANT")) ps.d.col_variant = std::atoi(cv) & 31;
    if (ps.d.col_variant > 19) ps.d.col_variant = 9;
    if (ps.d.kernel == K_COL4096 && ps.d.ncols % col_tile_width(ps.d.col_variant) != 0)
      ps.d.col_variant = 8;  // 8-column tiles
    if (ps.tw_off >= 0) ps.d.tw = base + ps.tw_off;
    if (ps.tw4lo_off >= 0) ps.d.tw4_lo = base + ps.tw4lo_off;
    if (ps.tw4hi_off >= 0) ps.d.tw4_hi = base + ps.tw4hi_off;
    if (ps.chirp_off >= 0) ps.d.chirp = base + ps.chirp_off;
    if (ps.filter_off >= 0) ps.d.filter = base + ps.filter_off;
  }
  for (const PassSpec& ps : p->passes)
    if (ps.d.kernel == K_COL4096) {  // columns per cluster tile of the variant that runs
      char cb[40];
      std::snprintf(cb, sizeof cb, " cluster-columns=%d", p->dbl ? 16 : col_tile_width(ps.d.col_variant));
      p->desc += cb;
      break;
    }
  if (tc.tuned) {
    char tb[96];
    std::snprintf(tb, sizeof tb, " tuned(row=%d%s col=%d split=%d strtma=%d bluepad=%d rowk=%d)", tc.row_variant,
                  tc.row_tma > 0 ? "t" : "", tc.col_variant, tc.split_rank, tc.str_tma, tc.blue_pad, tc.row_kernel);
    p->desc += tb;
  }
  if (std::getenv("GBFFT_PLAN_DUMP")) std::fprintf(stderr, "gbfft plan: %s\n", p->desc.c_str());
  return GBFFT_OK;
}

// Split-FP16 dense rows: the innermost axis of length w (one FP32 pass from
// the input to the output, no plan scratch) becomes the fold pass and the
// tensor-core product pass of tcdft.cu, for lengths without a radix-16
// tensor-core row kernel.  Returns GBFFT_ERR_UNSUPPORTED when the plan does
// not have that shape (the caller then tries the radix-16 form).
static int build_split_dense(gbfft_plan* p) {
  const int64_t w = p->dims[p->rank - 1];
  if (p->passes.empty() || !tcdft_available(w) || row_tc_available(int(w)) || p->d_scratch)
    return GBFFT_ERR_UNSUPPORTED;
  const PassSpec first = p->passes[0];
  if (first.src != R_IN || first.dst != R_OUT || !first.axis_final) return GBFFT_ERR_UNSUPPORTED;
  const int64_t rows = p->total / w;
  Builder B;
  std::vector<PassSpec> tc;
  const bool fused = tcdft8_available(w);  // n = 8 * odd: one pass, no scratch
  int st = fused ? tcdft8_add_pass(B, w, rows, w, w, R_IN, R_OUT, tc)
                 : tcdft_add_passes(B, w, rows, w, w, R_IN, R_OUT, tc);
  if (st != GBFFT_OK) return st;
  if (fault_injected("alloc")) return GBFFT_ERR_ALLOC;
  if (cudaMalloc(&p->d_tcmat, B.blob.size()) != cudaSuccess) return GBFFT_ERR_ALLOC;
  if (cudaMemcpy(p->d_tcmat, B.blob.data(), B.blob.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return GBFFT_ERR_CUDA;
  if (!fused) {
    p->scratch_bytes = tcdft_scratch_bytes(w, rows);
    if (cudaMalloc(&p->d_scratch, p->scratch_bytes) != cudaSuccess) return GBFFT_ERR_ALLOC;
    if (cudaEventCreateWithFlags(&p->scratch_ev, cudaEventDisableTiming) != cudaSuccess) return GBFFT_ERR_CUDA;
  }
  for (PassSpec& ps : tc) {
    ps.d.status = first.d.status;
    if (ps.tw_off >= 0) ps.d.tw = static_cast<unsigned char*>(p->d_tcmat) + ps.tw_off;
  }
  std::vector<PassSpec> passes = tc;
  passes.insert(passes.end(), p->passes.begin() + 1, p->passes.end());
  p->passes = passes;
  const size_t cut = p->desc.find('[');
  const size_t end = p->desc.find(']');
  char buf[160];
  if (fused)
    std::snprintf(buf, sizeof buf, "[n=%lld = 8x%d: radix-8 + tcgen05 split-fp16 dense %d (P=%d)]", (long long)w,
                  tc[0].d.tc_nc, tc[0].d.tc_nc, tc[0].d.tc_p);
  else
    std::snprintf(buf, sizeof buf, "[n=%lld tensor-core dense DFT: fold + tcgen05 split-fp16 (P=%d, %dx%d chunks)]",
                  (long long)w, tc[0].d.tc_p, tc[0].d.tc_kc, tc[0].d.tc_nc);
  if (cut != std::string::npos && end != std::string::npos && end > cut)
    p->desc = p->desc.substr(0, cut) + buf + p->desc.substr(end + 1);
  else
    p->desc += buf;
  p->desc += " split-fp16(tensor-core dense rows)";
  return GBFFT_OK;
}

// Split-FP16 plans: the FP32 plan with its contiguous-row passes moved to the
// tensor cores -- lengths with radix-16 stages to the radix-16 tensor-core
// row kernel, other row lengths up to kTcDftMaxN to the dense DFT
// (build_split_dense).  For the radix-16 kernel D is the 32 x 32 real form of
// the forward DFT-16 (rows: Re y_n then Im y_n; columns: Re x_k then Im x_k),
// split as D_hi + D_lo in FP16.
int build_split_plan(gbfft_plan* p) {
  if (p->dbl) return GBFFT_ERR_INVALID_ARG;
  int st = build_plan(p, false);
  if (st != GBFFT_OK) return st;
  st = build_split_dense(p);
  if (st != GBFFT_ERR_UNSUPPORTED) return st;
  std::vector<__half> dm(2048);
  for (int n = 0; n < 32; ++n)
    for (int k = 0; k < 32; ++k) {
      const int nn = n & 15, kk = k & 15;
      const cd w = unit_root(int64_t(nn) * kk, 16);  // cos - i sin
      const double c = w.real(), sn = -w.imag();
      const double v = (n < 16) ? (k < 16 ? c : sn) : (k < 16 ? -sn : c);
      const __half h = __float2half_rn(float(v));
      dm[size_t(n * 32 + k)] = h;
      dm[size_t(1024 + n * 32 + k)] = __float2half_rn(float(v - double(__half2float(h))));
    }
  // plain row passes only: one-pass Bluestein rows keep their FP32 kernel
  auto tc_row = [](const PassSpec& ps) {
    return ps.d.kernel == K_ROW && !(ps.d.flags & F_BLUE) && row_tc_available(ps.d.n);
  };
  bool any = false;
  for (PassSpec& ps : p->passes)
    if (tc_row(ps)) any = true;
  // A split-FP16 request is served by tensor-core passes or refused: a plan
  // with no pass on the tensor cores would silently be the FP32 plan.
  if (!any) return GBFFT_ERR_UNSUPPORTED;
  if (fault_injected("alloc")) return GBFFT_ERR_ALLOC;
  if (cudaMalloc(&p->d_tcmat, dm.size() * sizeof(__half)) != cudaSuccess) return GBFFT_ERR_ALLOC;
  if (cudaMemcpy(p->d_tcmat, dm.data(), dm.size() * sizeof(__half), cudaMemcpyHostToDevice) != cudaSuccess)
    return GBFFT_ERR_CUDA;
  for (PassSpec& ps : p->passes)
    if (tc_row(ps)) {
      ps.d.kernel = K_ROW_TC;
      ps.d.tcmat = p->d_tcmat;
    }
  p->desc += " split-fp16(tensor-core radix-16 rows)";
  return GBFFT_OK;
}

void* role_ptr(const gbfft_plan* p, int role, const void* in, void* out) {
  switch (role) {
    case R_IN: return const_cast<void*>(in);
    case R_OUT: return out;
    case R_S1: return p->d_scratch;
    case R_S2: return static_cast<unsigned char*>(p->d_scratch) + p->s2_off;
  }
  return nullptr;
}

// Orders executions of a plan with scratch that run on different streams
// (see gbfft_plan::scratch_ev); a no-op for plans without scratch.
class ScratchOrder {
 public:
  ScratchOrder(const gbfft_plan* p, cudaStream_t s) : p_(p), s_(s) {
    if (!p->d_scratch || !p->scratch_ev) return;
    lk_ = std::unique_lock<std::mutex>(p->scratch_mu);
    if (p->scratch_used && p->scratch_stream != s) cudaStreamWaitEvent(s, p->scratch_ev, 0);
  }
  ~ScratchOrder() {
    if (!lk_.owns_lock()) return;
    if (cudaEventRecord(p_->scratch_ev, s_) == cudaSuccess) {
      p_->scratch_stream = s_;
      p_->scratch_used = true;
    }
  }

 private:
  const gbfft_plan* p_;
  cudaStream_t s_;
  std::unique_lock<std::mutex> lk_;
};

// rotation of an axis of length n for the output options (shift, ishift,
// centring of even lengths by the shift theorem)
static int64_t axis_rotation(int64_t n, int opts, bool centre_fused) {
  int64_t s = 0;
  if (opts & GBFFT_OPT_SHIFT_OUT) s += n / 2 + (n & 1);
  if (opts & GBFFT_OPT_ISHIFT_OUT) s += n / 2;
  if (centre_fused) s += n / 2;
  return n > 0 ? s % n : 0;
}

int exec_passes(const gbfft_plan* p, const std::vector<PassSpec>& passes, int mode, double inv_norm,
                const void* in, void* out, cudaStream_t s, int opts, bool centre_fused) {
  const ScratchOrder order(p, s);
  if (passes.empty()) {
    // every axis has length <= 1: the DFT is the identity
    const size_t bytes = size_t(p->total) * (p->dbl ? 16 : 8);
    if (bytes && cudaMemcpyAsync(out, in, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return GBFFT_ERR_CUDA;
    return GBFFT_OK;
  }
  const size_t last = passes.size() - 1;
  for (size_t i = 0; i < passes.size(); ++i) {
    PassDesc d = passes[i].d;
    d.in = role_ptr(p, passes[i].src, in, out);
    d.out = role_ptr(p, passes[i].dst, in, out);
    if (mode != GBFFT_FORWARD) {
      if (i == 0) d.flags |= F_CONJ_IN;
      if (i == last) d.flags |= F_CONJ_OUT;
    }
    if (mode == GBFFT_INVERSE && i == last) {
      d.flags |= F_SCALE;
      d.scale = inv_norm;
    }
    if (passes[i].axis_final && (opts || centre_fused)) {
      const int64_t rot = axis_rotation(passes[i].axis_n, opts, centre_fused);
      if (rot) {
        d.flags |= F_ROT_OUT;
        d.rot_n = passes[i].axis_n;
        d.rot_s = rot;
        d.rot_stride = passes[i].rot_stride;
      }
    }
    if (launch_pass(d, p->dbl, s) != cudaSuccess) return GBFFT_ERR_CUDA;
  }
  return GBFFT_OK;
}

// Identity of the CUDA context current on this thread: cuCtxGetId's ID,
// which the driver never hands out twice in a process (a CUcontext handle of
// a destroyed context can come back for a new one, an ID cannot).  Without a
// current context (cannot happen after cudaFree(nullptr)) the device number
// stands in.
uint64_t current_context_id() {
  static PFN_cuCtxGetCurrent_v4000 get = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f);
  }();
  static PFN_cuCtxGetId_v12000 get_id = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<PFN_cuCtxGetId_v12000>(f);
  }();
  CUcontext c = nullptr;
  if (get) get(&c);
  if (!c) {
    int dev = 0;
    cudaGetDevice(&dev);
    return uint64_t(1) << 63 | uint64_t(dev);
  }
  unsigned long long id = 0;
  if (get_id && get_id(c, &id) == CUDA_SUCCESS) return uint64_t(id);
  return uint64_t(reinterpret_cast<uintptr_t>(c));
}

}  // namespace gbfft

// ---------------------------------------------------------------------------
// C ABI
extern "C" {

const char* gbfft_error_string(int status) {
  switch (status) {
    case GBFFT_OK: return "ok";
    case GBFFT_ERR_INVALID_ARG: return "invalid argument";
    case GBFFT_ERR_UNSUPPORTED: return "unsupported transform for this build";
    case GBFFT_ERR_ALLOC: return "allocation failed";
    case GBFFT_ERR_CUDA: return "CUDA runtime error";
    case GBFFT_ERR_NULL_PLAN: return "null plan";
    case GBFFT_ERR_TIMEOUT: return "bounded device wait timed out";
    case GBFFT_ERR_INTERNAL: return "internal error";
    case GBFFT_ERR_TOO_LARGE: return "request exceeds the fixed work area of gbfft_fft_noalloc";
  }
  return "unknown status";
}

int gbfft_version(void) { return 10000 * 0 + 100 * 1 + 0; }

int gbfft_plan_create(gbfft_plan** out, int rank, const int64_t* dims, int kind, int dtype,
                      int precision) {
  return gbfft::create_plan(out, rank, dims, kind, dtype, precision, nullptr);
}

int gbfft_autotune(int rank, const int64_t* dims, int kind, int dtype, int precision, void* stream,
                   char* report, size_t cap) {
  if (!dims || rank < 1 || rank > 5) return GBFFT_ERR_INVALID_ARG;
  gbfft::TuneChoice best;
  std::string rep;
  const int st = gbfft::autotune_plan(rank, dims, kind, dtype, precision, stream, best, &rep);
  if (report && cap) std::snprintf(report, cap, "%s", rep.c_str());
  return st;
}

int gbfft_plan_explain(int rank, const int64_t* dims, int kind, int dtype, int precision, char* buf,
                       size_t cap) {
  if (!buf || cap == 0 || !dims || rank < 1 || rank > 5) return GBFFT_ERR_INVALID_ARG;
  if (kind != GBFFT_KIND_MANY && kind != GBFFT_KIND_FULL) return GBFFT_ERR_INVALID_ARG;
  if (kind == GBFFT_KIND_FULL && rank > 3) return GBFFT_ERR_UNSUPPORTED;
  if (dtype != GBFFT_C32 && dtype != GBFFT_C64) return GBFFT_ERR_INVALID_ARG;
  gbfft_plan p;
  p.rank = rank;
  p.total = 1;
  for (int i = 0; i < rank; ++i) {
    if (dims[i] < 0) return GBFFT_ERR_INVALID_ARG;
    p.dims[i] = dims[i];
    p.total *= dims[i];
  }
  p.kind = kind;
  p.dtype = dtype;
  p.precision = precision;
  p.dbl = dtype == GBFFT_C64;
  if (precision != GBFFT_PLAIN) return GBFFT_ERR_UNSUPPORTED;
  int st = p.total > 0 ? build_plan(&p, true) : GBFFT_OK;
  if (st != GBFFT_OK) return st;
  std::snprintf(buf, cap, "%s; launches=%d tables=%zu scratch=%zu", p.desc.c_str(),
                int(p.passes.size()), p.tables_bytes, p.scratch_bytes);
  return GBFFT_OK;
}

int gbfft_plan_destroy(gbfft_plan* plan) {
  if (!plan) return GBFFT_OK;
  if (plan->d_tables) cudaFree(plan->d_tables);
  if (plan->d_scratch) cudaFree(plan->d_scratch);
  if (plan->d_tcmat) cudaFree(plan->d_tcmat);
  if (plan->scratch_ev) cudaEventDestroy(plan->scratch_ev);
  delete plan;
  return GBFFT_OK;
}

int gbfft_exec(const gbfft_plan* plan, int mode, const void* d_in, void* d_out, void* stream) {
  if (!plan) return GBFFT_ERR_NULL_PLAN;
  if (mode != GBFFT_FORWARD && mode != GBFFT_REVERSE && mode != GBFFT_INVERSE)
    return GBFFT_ERR_INVALID_ARG;
  if (plan->total == 0) return GBFFT_OK;
  if (!d_in || !d_out || d_in == d_out) return GBFFT_ERR_INVALID_ARG;
  const uintptr_t align = plan->dbl ? 16 : 8;
  if ((reinterpret_cast<uintptr_t>(d_in) | reinterpret_cast<uintptr_t>(d_out)) & (align - 1))
    return GBFFT_ERR_INVALID_ARG;
  return exec_passes(plan, plan->passes, mode, plan->inv_norm, d_in, d_out,
                     static_cast<cudaStream_t>(stream));
}

int gbfft_exec_ex(const gbfft_plan* plan, int mode, const void* d_in, void* d_out, void* stream, int opts) {
  if (!opts) return gbfft_exec(plan, mode, d_in, d_out, stream);
  if (!plan) return GBFFT_ERR_NULL_PLAN;
  if (mode != GBFFT_FORWARD && mode != GBFFT_REVERSE && mode != GBFFT_INVERSE) return GBFFT_ERR_INVALID_ARG;
  const int known = GBFFT_OPT_SHIFT_OUT | GBFFT_OPT_ISHIFT_OUT | GBFFT_OPT_CENTRE_IN;
  if ((opts & ~known) || ((opts & GBFFT_OPT_SHIFT_OUT) && (opts & GBFFT_OPT_ISHIFT_OUT))) return GBFFT_ERR_INVALID_ARG;
  // centre / shift are defined on the whole array (Centre.hs: 1D..3D)
  if (plan->kind != GBFFT_KIND_FULL || plan->rank > 3) return GBFFT_ERR_INVALID_ARG;
  if (plan->total == 0) return GBFFT_OK;
  if (!d_in || !d_out || d_in == d_out) return GBFFT_ERR_INVALID_ARG;
  const uintptr_t align = plan->dbl ? 16 : 8;
  if ((reinterpret_cast<uintptr_t>(d_in) | reinterpret_cast<uintptr_t>(d_out)) & (align - 1))
    return GBFFT_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  bool all_even = true;
  for (int i = 0; i < plan->rank; ++i) all_even = all_even && (plan->dims[i] % 2 == 0);
  const bool centre = (opts & GBFFT_OPT_CENTRE_IN) != 0;
  const bool centre_fused = centre && all_even;  // centring = shifting the output by n/2
  const int out_opts = opts & (GBFFT_OPT_SHIFT_OUT | GBFFT_OPT_ISHIFT_OUT);
  // fused only when every axis of length > 1 ends in exactly one pass that
  // can rotate its store index (the split-FP16 passes mark none)
  int finals = 0, axes = 0;
  bool fuse = true;
  for (int i = 0; i < plan->rank; ++i) axes += plan->dims[i] > 1;
  for (const PassSpec& ps : plan->passes) {
    if (!ps.axis_final) continue;
    ++finals;
    if (axis_rotation(ps.axis_n, out_opts, centre_fused) && !ps.rot_ok) fuse = false;
  }
  if (finals != axes) fuse = false;
  const size_t bytes = size_t(plan->total) * (plan->dbl ? 16 : 8);
  const int dtype = plan->dbl ? GBFFT_C64 : GBFFT_C32;
  const void* src = d_in;
  void* tmp_in = nullptr;
  void* tmp_out = nullptr;
  int st = GBFFT_OK;
  if (centre && !centre_fused) {
    // odd lengths: the sign pattern is not a rotation; one pass before
    if (cudaMallocAsync(&tmp_in, bytes, s) != cudaSuccess) return GBFFT_ERR_ALLOC;
    st = gbfft_centre(plan->rank, plan->dims, dtype, d_in, tmp_in, stream);
    src = tmp_in;
  }
  if (st == GBFFT_OK) {
    if (fuse) {
      st = exec_passes(plan, plan->passes, mode, plan->inv_norm, src, d_out, s, out_opts, centre_fused);
    } else {
      // an axis whose last pass cannot rotate: transform, then one shift pass
      if (cudaMallocAsync(&tmp_out, bytes, s) != cudaSuccess) {
        st = GBFFT_ERR_ALLOC;
      } else {
        st = exec_passes(plan, plan->passes, mode, plan->inv_norm, src, tmp_out, s);
        if (st == GBFFT_OK && centre_fused)
          st = gbfft_shift(plan->rank, plan->dims, dtype, 1, tmp_out, d_out, stream);  // n/2 = ishift for even n
        if (st == GBFFT_OK && out_opts) {
          const void* from = centre_fused ? d_out : tmp_out;
          void* to = centre_fused ? tmp_out : d_out;
          st = gbfft_shift(plan->rank, plan->dims, dtype, (out_opts & GBFFT_OPT_ISHIFT_OUT) ? 1 : 0, from, to, stream);
          if (st == GBFFT_OK && centre_fused &&
              cudaMemcpyAsync(d_out, tmp_out, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            st = GBFFT_ERR_CUDA;
        } else if (st == GBFFT_OK && !centre_fused &&
                   cudaMemcpyAsync(d_out, tmp_out, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
          st = GBFFT_ERR_CUDA;
        }
      }
    }
  }
  if (tmp_in) cudaFreeAsync(tmp_in, s);
  if (tmp_out) cudaFreeAsync(tmp_out, s);
  return st;
}

// ---- plan cache -----------------------------------------------------------
namespace {
using CacheKey = std::tuple<uint64_t, int, int64_t, int64_t, int64_t, int64_t, int64_t, int, int, int>;
std::mutex g_cache_mu;
std::map<CacheKey, gbfft_plan*>& cache() {
  static auto* m = new std::map<CacheKey, gbfft_plan*>();
  return *m;
}

}  // namespace


int gbfft_plan_get(gbfft_plan** out, int rank, const int64_t* dims, int kind, int dtype,
                   int precision) {
  if (!out || !dims || rank < 1 || rank > 5) return GBFFT_ERR_INVALID_ARG;
  // make sure a context exists before keying on it
  cudaFree(nullptr);
  int64_t d[5] = {0, 0, 0, 0, 0};
  for (int i = 0; i < rank; ++i) d[i] = dims[i];
  CacheKey key{current_context_id(), rank, d[0], d[1], d[2], d[3], d[4], kind, dtype, precision};
  std::lock_guard<std::mutex> lk(g_cache_mu);
  auto it = cache().find(key);
  if (it != cache().end()) {
    *out = it->second;
    return GBFFT_OK;
  }
  gbfft_plan* p = nullptr;
  int st = gbfft_plan_create(&p, rank, dims, kind, dtype, precision);
  if (st != GBFFT_OK) return st;
  cache().emplace(key, p);
  *out = p;
  return GBFFT_OK;
}

int gbfft_fft(int mode, int rank, const int64_t* dims, int kind, int dtype, const void* d_in,
              void* d_out, void* stream) {
  gbfft_plan* p = nullptr;
  int st = gbfft_plan_get(&p, rank, dims, kind, dtype, GBFFT_PLAIN);
  if (st != GBFFT_OK) return st;
  return gbfft_exec(p, mode, d_in, d_out, stream);
}

int gbfft_cache_clear(void) {
  cudaFree(nullptr);
  const uint64_t ctx = current_context_id();
  std::lock_guard<std::mutex> lk(g_cache_mu);
  for (auto it = cache().begin(); it != cache().end();) {
    if (std::get<0>(it->first) == ctx) {
      gbfft_plan_destroy(it->second);
      it = cache().erase(it);
    } else {
      ++it;
    }
  }
  return GBFFT_OK;
}

int gbfft_exec_range(const gbfft_plan* plan, int mode, int first, int count, const void* d_in,
                     void* d_out, void* stream) {
  if (!plan) return GBFFT_ERR_NULL_PLAN;
  if (mode != GBFFT_FORWARD && mode != GBFFT_REVERSE && mode != GBFFT_INVERSE)
    return GBFFT_ERR_INVALID_ARG;
  const int np = int(plan->passes.size());
  if (first < 0 || count < 0 || first + count > np) return GBFFT_ERR_INVALID_ARG;
  if (plan->total == 0 || count == 0) return GBFFT_OK;
  if (!d_in || !d_out || d_in == d_out) return GBFFT_ERR_INVALID_ARG;
  const size_t last = plan->passes.size() - 1;
  const ScratchOrder order(plan, static_cast<cudaStream_t>(stream));
  for (int i = first; i < first + count; ++i) {
    const PassSpec& ps = plan->passes[size_t(i)];
    PassDesc d = ps.d;
    d.in = role_ptr(plan, ps.src, d_in, d_out);
    d.out = role_ptr(plan, ps.dst, d_in, d_out);
    if (mode != GBFFT_FORWARD) {
      if (i == 0) d.flags |= F_CONJ_IN;
      if (size_t(i) == last) d.flags |= F_CONJ_OUT;
    }
    if (mode == GBFFT_INVERSE && size_t(i) == last) {
      d.flags |= F_SCALE;
      d.scale = plan->inv_norm;
    }
    if (launch_pass(d, plan->dbl, static_cast<cudaStream_t>(stream)) != cudaSuccess)
      return GBFFT_ERR_CUDA;
  }
  return GBFFT_OK;
}

int gbfft_exec_status(const gbfft_plan* plan, void* stream) {
  if (!plan) return GBFFT_ERR_NULL_PLAN;
  if (!plan->d_status) return GBFFT_OK;
  int h = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (cudaMemcpyAsync(&h, plan->d_status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return GBFFT_ERR_CUDA;
  if (h != 0) cudaMemsetAsync(plan->d_status, 0, sizeof(int), s);
  return h;
}

int gbfft_plan_info(const gbfft_plan* plan, size_t* workspace_bytes, int* launches_per_exec) {
  if (!plan) return GBFFT_ERR_NULL_PLAN;
  if (workspace_bytes) *workspace_bytes = plan->tables_bytes + plan->scratch_bytes;
  if (launches_per_exec) *launches_per_exec = int(plan->passes.size());
  return GBFFT_OK;
}

int gbfft_plan_describe(const gbfft_plan* plan, char* buf, size_t cap) {
  if (!plan) return GBFFT_ERR_NULL_PLAN;
  if (!buf || cap == 0) return GBFFT_ERR_INVALID_ARG;
  std::snprintf(buf, cap, "%s", plan->desc.c_str());
  return GBFFT_OK;
}

int gbfft_plan_pass_kernel(const gbfft_plan* plan, int pass, char* buf, size_t cap) {
  if (!plan) return GBFFT_ERR_NULL_PLAN;
  if (!buf || cap == 0 || pass < 0 || size_t(pass) >= plan->passes.size()) return GBFFT_ERR_INVALID_ARG;
  std::snprintf(buf, cap, "%s", gbfft::pass_kernel_name(plan->passes[size_t(pass)].d, plan->dbl));
  return GBFFT_OK;
}

}  // extern "C"
