// Differentiable spectral convolution over a batch of 3D fields:
//   y_b = fft3D Inverse (fft3D Forward (x_b) * H),  b < batch,
// and its adjoint for L(y) with g_y = dL/dy (conjugate-Wirtinger convention):
//   g_Y,b = (1/N) F(g_y,b)
//   g_H   = sum_b conj(X_b) * g_Y,b          X_b = F(x_b), recomputed
//   g_x,b = F^H(conj(H) * g_Y,b) = conj(F(H * conj(g_Y,b)))
// The reference composes the forward from fft3D (FFT.hs:150-173) and an
// elementwise product, and has no derivative.
//
// Forward, five passes per field instead of six: x, y, then one z kernel that
// does the forward z DFT, the product with H and the first inverse axis (as
// the DFT of the conjugate) in shared memory, then y and x with the final
// conjugate and 1/N.
// Adjoint, seven passes: x, y of x into scratch; x, y of g_y into g_x; one z
// kernel that recomputes X and g_Y along z for every field of the batch,
// accumulates g_H for its columns in shared memory (written once, no
// atomics) and starts the adjoint inverse; then y and x with the conjugate.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "gbfft.h"
#include "pencil_tile.cuh"
#include "plan_internal.h"
#include "strided_tile.cuh"

namespace gbfft {

struct SpecBwdArgs {
  PassDesc z;      // z-axis pass: n = d, column tile of W, pitch, stages, twiddles
  const void* xt;  // batch x N, x after its x and y transforms
  void* g;         // batch x N, g_y after its x and y transforms; z output (in place)
  const void* H;
  void* gH;
  int64_t batch, N, S;  // S = h*w (column count and z stride)
  double invN;
};

namespace {

constexpr int kSpecThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kSpecThreads) specconv_bwd_z_kernel(const SpecBwdArgs a) {
  using C = typename CxT<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const PassDesc& d = a.z;
  const int W = d.W, n = d.n, P = d.pitch;
  C* X0 = reinterpret_cast<C*>(smem_raw);
  C* X1 = X0 + W * P;
  C* G0 = X1 + W * P;
  C* G1 = G0 + W * P;
  C* ACC = G1 + W * P;
  const int64_t c0 = int64_t(blockIdx.x) * W;
  const int total = W * n;
  const C* __restrict__ H = static_cast<const C*>(a.H);
  const T invN = T(a.invN);
  for (int f = threadIdx.x; f < total; f += blockDim.x) {
    const int c = f % W, k = f / W;
    ACC[c * P + spad(k)] = cmake<C>(T(0), T(0));
  }
  for (int64_t b = 0; b < a.batch; ++b) {
    const C* __restrict__ xt = static_cast<const C*>(a.xt) + b * a.N;
    C* __restrict__ g = static_cast<C*>(a.g) + b * a.N;
    for (int f = threadIdx.x; f < total; f += blockDim.x) {
      const int c = f % W, i = f / W;
      const int64_t col = c0 + c;
      C vx = cmake<C>(T(0), T(0)), vg = vx;
      if (col < a.S) {
        vx = xt[int64_t(i) * a.S + col];
        vg = g[int64_t(i) * a.S + col];
      }
      X0[c * P + spad(i)] = vx;
      G0[c * P + spad(i)] = vg;
    }
    __syncthreads();
    const C* rx = run_stages<C>(d, X0, X1);
    C* rg = run_stages<C>(d, G0, G1);
    for (int f = threadIdx.x; f < total; f += blockDim.x) {
      const int c = f % W, k = f / W;
      const int64_t col = c0 + c;
      const int o = c * P + spad(k);
      const C gy = cscale(rg[o], invN);
      C acc = ACC[o];
      acc = cadd(acc, cmul(cconj(rx[o]), gy));
      ACC[o] = acc;
      const C h = (col < a.S) ? H[int64_t(k) * a.S + col] : cmake<C>(T(0), T(0));
      rg[o] = cmul(h, cconj(gy));
    }
    __syncthreads();
    C* other = (rg == G0) ? G1 : G0;
    const C* r2 = run_stages<C>(d, rg, other);
    for (int f = threadIdx.x; f < total; f += blockDim.x) {
      const int c = f % W, k = f / W;
      const int64_t col = c0 + c;
      if (col < a.S) g[int64_t(k) * a.S + col] = r2[c * P + spad(k)];
    }
    __syncthreads();
  }
  C* __restrict__ gH = static_cast<C*>(a.gH);
  for (int f = threadIdx.x; f < total; f += blockDim.x) {
    const int c = f % W, k = f / W;
    const int64_t col = c0 + c;
    if (col < a.S) gH[int64_t(k) * a.S + col] = ACC[c * P + spad(k)];
  }
}

// Register-resident adjoint z stage for z lengths with a strided register
// kernel: W adjacent columns per CTA, thread (x, t) holds elements t + TH*m of
// its column (TH = N/16).  Per field the z DFTs of x~ and g~ run in
// registers with their exchanges in one shared buffer; the thread's own
// (k, x) slots of H (staged once) and of the g_H accumulator live in shared
// memory, so the elementwise step needs no barrier; the first axis of the
// adjoint inverse runs straight from registers and is stored in place.
template <typename T, int N, int W, int... Rs>
__global__ void __launch_bounds__(W*(N / 16), sizeof(T) == 4 ? 2 : 1) specconv_bwd_z_reg(const SpecBwdArgs a) {
  using C = typename CxT<T>::type;
  constexpr int E = 16;
  constexpr int TH = N / E;
  constexpr int R0 = rl_first(RL<Rs...>{});
  constexpr int RZ = rl_last(RL<Rs...>{});
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* xb = reinterpret_cast<C*>(smem_raw);  // exchange buffer [i][x]
  C* hs = xb + N * W;                      // H of the tile [k][x]
  C* acc = hs + N * W;                     // g_H accumulator [k][x]
  const int x = threadIdx.x % W;
  const int t = threadIdx.x / W;
  const int64_t col = int64_t(blockIdx.x) * W + x;
  const bool ok = col < a.S;
  const int64_t S = a.S;
  const C* __restrict__ H = static_cast<const C*>(a.H);
  const C* __restrict__ tw = static_cast<const C*>(a.z.tw);
  const T invN = T(a.invN);
  const C zero = cmake<C>(T(0), T(0));
#pragma unroll
  for (int m = 0; m < E; ++m) {
    const int k = t + TH * m;
    hs[k * W + x] = ok ? H[int64_t(k) * S + col] : zero;
    acc[k * W + x] = zero;
  }
  for (int64_t b = 0; b < a.batch; ++b) {
    const C* __restrict__ xt = static_cast<const C*>(a.xt) + b * a.N;
    C* __restrict__ g = static_cast<C*>(a.g) + b * a.N;
    C vx[E], vg[E];
#pragma unroll
    for (int q = 0; q < E / R0; ++q)
#pragma unroll
      for (int r = 0; r < R0; ++r) {
        const int i = t + TH * (q + r * (E / R0));
        vx[q * R0 + r] = ok ? xt[int64_t(i) * S + col] : zero;
        vg[q * R0 + r] = ok ? g[int64_t(i) * S + col] : zero;
      }
    str_stages<N, E, 1, 0, W>(vx, xb, tw, t, x, RL<Rs...>{});
    str_stages<N, E, 1, 0, W>(vg, xb, tw, t, x, RL<Rs...>{});
    // outputs k = t + TH*m sit in v[q*RZ + r], m = q + r*E/RZ; the third
    // transform's first stage wants element t + TH*m in u[(m % (E/R0))*R0 + m/(E/R0)]
    C u[E];
#pragma unroll
    for (int q = 0; q < E / RZ; ++q)
#pragma unroll
      for (int r = 0; r < RZ; ++r) {
        const int m = q + r * (E / RZ);
        const int o = (t + TH * m) * W + x;
        const C gy = cscale(vg[q * RZ + r], invN);
        acc[o] = cadd(acc[o], cmul(cconj(vx[q * RZ + r]), gy));
        u[(m % (E / R0)) * R0 + m / (E / R0)] = cmul(hs[o], cconj(gy));
      }
    str_stages<N, E, 1, 0, W>(u, xb, tw, t, x, RL<Rs...>{});
    if (ok) {
#pragma unroll
      for (int q = 0; q < E / RZ; ++q)
#pragma unroll
        for (int r = 0; r < RZ; ++r) g[int64_t(t + TH * (q + r * (E / RZ))) * S + col] = u[q * RZ + r];
    }
  }
  if (ok) {
    C* __restrict__ gH = static_cast<C*>(a.gH);
#pragma unroll
    for (int m = 0; m < E; ++m) {
      const int k = t + TH * m;
      gH[int64_t(k) * S + col] = acc[k * W + x];
    }
  }
}

// (type, N, W, radices = factor_device(N)) of the register adjoint kernel
#define GBFFT_SPECBWD_TABLE(X)      \
  X(float, 64, 16, 16, 4)           \
  X(float, 128, 16, 16, 8)          \
  X(float, 256, 16, 16, 16)         \
  X(float, 512, 16, 16, 16, 2)      \
  X(double, 256, 8, 16, 16)

template <typename T, int N, int W, int... Rs>
struct SpecBwdCfg {
  static constexpr int threads = W * (N / 16);
  static size_t smem() { return size_t(3) * N * W * sizeof(typename CxT<T>::type); }
  static cudaError_t prepare() {
    return cudaFuncSetAttribute(specconv_bwd_z_reg<T, N, W, Rs...>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(smem()));
  }
  static cudaError_t launch(const SpecBwdArgs& a, cudaStream_t s) {
    const unsigned grid = unsigned((a.S + W - 1) / W);
    specconv_bwd_z_reg<T, N, W, Rs...><<<grid, threads, smem(), s>>>(a);
    return cudaGetLastError();
  }
};

bool spec_bwd_reg_available(int n, bool dbl) {
#define X(T, N, W, ...) \
  if (n == N && dbl == (sizeof(T) == 8)) return true;
  GBFFT_SPECBWD_TABLE(X)
#undef X
  return false;
}

cudaError_t spec_bwd_reg_prepare() {
  cudaError_t e = cudaSuccess;
#define X(T, N, W, ...) \
  if (e == cudaSuccess) e = SpecBwdCfg<T, N, W, __VA_ARGS__>::prepare();
  GBFFT_SPECBWD_TABLE(X)
#undef X
  return e;
}

cudaError_t spec_bwd_reg_launch(const SpecBwdArgs& a, bool dbl, cudaStream_t s) {
#define X(T, N, W, ...) \
  if (a.z.n == N && dbl == (sizeof(T) == 8)) return SpecBwdCfg<T, N, W, __VA_ARGS__>::launch(a, s);
  GBFFT_SPECBWD_TABLE(X)
#undef X
  return cudaErrorInvalidValue;
}

}  // namespace
}  // namespace gbfft

using namespace gbfft;

struct gbfft_specconv_plan {
  int64_t batch = 0, d = 0, h = 0, w = 0, N = 0;
  bool dbl = false;
  void* d_tables = nullptr;
  void* d_tmp = nullptr;  // batch x N, the adjoint's transformed x
  size_t tables_bytes = 0, tmp_bytes = 0;
  PassSpec px, py, pz;    // x, y passes; z pass with the spectral product
  PassSpec pzb;           // z stages for the adjoint kernel (W, pitch of its tiles)
  PassSpec pxy;           // x and y of each h x w plane in one pass (when has_plane)
  bool has_plane = false;
  size_t bwd_smem = 0;
  bool bwd_reg = false;   // the register-resident adjoint z kernel serves this z length
};

namespace {

void destroy_spec(gbfft_specconv_plan* p) {
  if (!p) return;
  if (p->d_tables) cudaFree(p->d_tables);
  if (p->d_tmp) cudaFree(p->d_tmp);
  delete p;
}

int run(const gbfft_specconv_plan* p, const PassSpec& ps, const void* in, void* out, uint32_t extra,
        double scale, const void* filter, cudaStream_t s) {
  PassDesc d = ps.d;
  d.in = in;
  d.out = out;
  d.flags |= extra;
  if (extra & F_SCALE) d.scale = scale;
  if (filter) d.filter = filter;
  return launch_pass(d, p->dbl, s) == cudaSuccess ? GBFFT_OK : GBFFT_ERR_CUDA;
}

}  // namespace

extern "C" {

int gbfft_specconv_plan_create(gbfft_specconv_plan** out, int64_t batch, int64_t d, int64_t h,
                               int64_t w, int dtype) {
  if (!out) return GBFFT_ERR_INVALID_ARG;
  *out = nullptr;
  if (batch < 1 || d < 1 || h < 1 || w < 1) return GBFFT_ERR_INVALID_ARG;
  if (dtype != GBFFT_C32 && dtype != GBFFT_C64) return GBFFT_ERR_INVALID_ARG;
  std::unique_ptr<gbfft_specconv_plan, void (*)(gbfft_specconv_plan*)> p(new gbfft_specconv_plan,
                                                                         destroy_spec);
  p->batch = batch;
  p->d = d;
  p->h = h;
  p->w = w;
  p->N = d * h * w;
  p->dbl = dtype == GBFFT_C64;
  const bool dbl = p->dbl;
  const int cap = dbl ? kCapC64 : kCapC32;
  for (int64_t e : {d, h, w})
    if (e > cap || !is_fast_length(e) || e < 2) return GBFFT_ERR_UNSUPPORTED;
  if (prepare_kernels() != cudaSuccess) return GBFFT_ERR_CUDA;
  Builder B;
  B.dbl = dbl;
  std::vector<PassSpec> v;
  int64_t s1 = 0, s2 = 0;
  std::string desc;
  const int64_t S = h * w;
  // x: contiguous rows (batch*d*h of them); y: stride w, outer batch*d; z: stride S, outer batch
  int st = add_axis(B, v, Axis{w, 1, w, batch * d * h, batch * p->N, 1}, true, s1, s2, desc);
  if (st == GBFFT_OK) st = add_axis(B, v, Axis{h, w, 1, w, S, batch * d}, false, s1, s2, desc);
  if (st == GBFFT_OK) st = add_axis(B, v, Axis{d, S, 1, S, p->N, batch}, false, s1, s2, desc);
  if (st != GBFFT_OK) return st;
  if (v.size() != 3 || s1 || s2) return GBFFT_ERR_UNSUPPORTED;
  p->px = v[0];
  p->py = v[1];
  p->pz = v[2];
  // the spectral product runs inside the strided register kernel when the
  // z length has one, else inside the generic pencil body
  if (p->pz.d.kernel != K_STRIDED) p->pz.d.kernel = K_PENCIL;
  p->pz.d.flags |= F_SPEC;
  p->pz.d.lout_es = S;
  p->pz.d.lout_cs = 1;
  // adjoint z tiles: five shared-memory regions per tile
  p->pzb = v[2];
  {
    PassDesc& z = p->pzb.d;
    z.kernel = K_PENCIL;
    z.W = dbl ? 4 : 8;
    if (int64_t(z.W) > S) z.W = int(S);
    p->bwd_smem = size_t(5) * z.W * z.pitch * (dbl ? 16 : 8);
    if (p->bwd_smem > 227 * 1024) return GBFFT_ERR_UNSUPPORTED;
  }
  // x and y of each plane in one cluster pass when the planes are 256 x 256;
  // opt-in (GBFFT_ENABLE=plane): measured on 8 x 256^3 it gives forward
  // 2.09 / adjoint 2.94 ms against 2.03 / 2.92 ms for the separate passes
  if (plane_available(h, w, dbl) && feature_enabled("plane")) {
    PassSpec& f = p->pxy;
    std::memset(&f.d, 0, sizeof(PassDesc));
    f.d.kernel = K_PLANE;
    f.d.n = int(w);
    f.d.ncols = batch * d;
    f.d.nbatch = f.d.nb_lo = 1;
    f.d.in_bs = f.d.out_bs = S;
    f.d.scale = 1.0;
    f.d.tw4_n = 1;
    f.tw_off = int64_t(B.roots_for(w));
    p->has_plane = true;
  }
  if (fault_injected("alloc")) return GBFFT_ERR_ALLOC;
  p->tables_bytes = B.blob.size();
  if (cudaMalloc(&p->d_tables, std::max<size_t>(p->tables_bytes, 256)) != cudaSuccess) return GBFFT_ERR_ALLOC;
  if (cudaMemcpy(p->d_tables, B.blob.data(), B.blob.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return GBFFT_ERR_CUDA;
  unsigned char* tb = static_cast<unsigned char*>(p->d_tables);
  for (PassSpec* ps : {&p->px, &p->py, &p->pz, &p->pzb, &p->pxy}) {
    if (ps->tw_off >= 0) ps->d.tw = tb + ps->tw_off;
    ps->d.use_tma = ps->d.kernel == K_ROW ? 0 : 1;  // rows: register kernel, double-buffered
    ps->d.row_variant = dbl ? 1 : 0;
    ps->d.col_variant = 9;
  }
  p->tmp_bytes = size_t(batch) * size_t(p->N) * (dbl ? 16 : 8);
  if (cudaMalloc(&p->d_tmp, p->tmp_bytes) != cudaSuccess) return GBFFT_ERR_ALLOC;
  auto kern = dbl ? (const void*)specconv_bwd_z_kernel<double> : (const void*)specconv_bwd_z_kernel<float>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(p->bwd_smem)) !=
      cudaSuccess)
    return GBFFT_ERR_CUDA;
  if (spec_bwd_reg_prepare() != cudaSuccess) return GBFFT_ERR_CUDA;
  p->bwd_reg = spec_bwd_reg_available(int(d), dbl) && !feature_disabled("strided");
  *out = p.release();
  return GBFFT_OK;
}

int gbfft_specconv_plan_destroy(gbfft_specconv_plan* plan) {
  destroy_spec(plan);
  return GBFFT_OK;
}

int gbfft_specconv_fwd(const gbfft_specconv_plan* p, const void* x, const void* H, void* y, void* stream) {
  if (!p) return GBFFT_ERR_NULL_PLAN;
  if (!x || !H || !y || x == y) return GBFFT_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const double invN = 1.0 / double(p->N);
  if (p->has_plane) {  // three passes: x+y, z with the product, x+y of the conjugate
    int st = run(p, p->pxy, x, y, 0, 1.0, nullptr, s);
    if (st == GBFFT_OK) st = run(p, p->pz, y, y, 0, 1.0, H, s);
    if (st == GBFFT_OK) st = run(p, p->pxy, y, y, F_CONJ_OUT | F_SCALE, invN, nullptr, s);
    return st;
  }
  int st = run(p, p->px, x, y, 0, 1.0, nullptr, s);                 // x: forward
  if (st == GBFFT_OK) st = run(p, p->py, y, y, 0, 1.0, nullptr, s);  // y: forward
  if (st == GBFFT_OK) st = run(p, p->pz, y, y, 0, 1.0, H, s);        // z: fwd, *H, conj, fwd
  if (st == GBFFT_OK) st = run(p, p->py, y, y, 0, 1.0, nullptr, s);  // y of the conjugate
  if (st == GBFFT_OK) st = run(p, p->px, y, y, F_CONJ_OUT | F_SCALE, invN, nullptr, s);
  return st;
}

int gbfft_specconv_bwd(const gbfft_specconv_plan* p, const void* x, const void* H, const void* gy,
                       void* gx, void* gH, void* stream) {
  if (!p) return GBFFT_ERR_NULL_PLAN;
  if (!x || !H || !gy || !gx || !gH || gx == gy || gx == x) return GBFFT_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = GBFFT_OK;
  if (p->has_plane) {
    st = run(p, p->pxy, x, p->d_tmp, 0, 1.0, nullptr, s);
    if (st == GBFFT_OK) st = run(p, p->pxy, gy, gx, 0, 1.0, nullptr, s);
  } else {
    st = run(p, p->px, x, p->d_tmp, 0, 1.0, nullptr, s);
    if (st == GBFFT_OK) st = run(p, p->py, p->d_tmp, p->d_tmp, 0, 1.0, nullptr, s);
    if (st == GBFFT_OK) st = run(p, p->px, gy, gx, 0, 1.0, nullptr, s);
    if (st == GBFFT_OK) st = run(p, p->py, gx, gx, 0, 1.0, nullptr, s);
  }
  if (st != GBFFT_OK) return st;
  SpecBwdArgs a{};
  a.z = p->pzb.d;
  a.xt = p->d_tmp;
  a.g = gx;
  a.H = H;
  a.gH = gH;
  a.batch = p->batch;
  a.N = p->N;
  a.S = p->h * p->w;
  a.invN = 1.0 / double(p->N);
  if (p->bwd_reg) {
    if (spec_bwd_reg_launch(a, p->dbl, s) != cudaSuccess) return GBFFT_ERR_CUDA;
  } else {
    const unsigned grid = unsigned((a.S + a.z.W - 1) / a.z.W);
    if (p->dbl)
      specconv_bwd_z_kernel<double><<<grid, kSpecThreads, p->bwd_smem, s>>>(a);
    else
      specconv_bwd_z_kernel<float><<<grid, kSpecThreads, p->bwd_smem, s>>>(a);
    if (cudaGetLastError() != cudaSuccess) return GBFFT_ERR_CUDA;
  }
  if (p->has_plane) return run(p, p->pxy, gx, gx, F_CONJ_OUT, 1.0, nullptr, s);
  st = run(p, p->py, gx, gx, 0, 1.0, nullptr, s);
  if (st == GBFFT_OK) st = run(p, p->px, gx, gx, F_CONJ_OUT, 1.0, nullptr, s);
  return st;
}

}  // extern "C"
