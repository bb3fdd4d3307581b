// Register-resident Stockham building blocks shared by the row kernels, the
// strided kernel and the persistent ragged executor: compile-time radix
// lists, twiddle loading / derivation, the exchanges of contiguous rows
// (XOR-swizzled) and of interleaved columns, and the strided tile body.
#pragma once

#include "butterflies.cuh"
#include "gbfft_internal.h"

namespace gbfft {

__device__ __forceinline__ int swz(int i) { return i ^ (((i >> 4) & 7) << 1); }

template <int... Rs> struct RL {};
template <int R, int... Rest> constexpr int rl_first(RL<R, Rest...>) { return R; }
template <int R> constexpr int rl_last(RL<R>) { return R; }
template <int R, int R2, int... Rest> constexpr int rl_last(RL<R, R2, Rest...>) {
  return rl_last(RL<R2, Rest...>{});
}
// entries of the stage twiddle table of stage (NS, R)
template <int R> constexpr int tw_entries(int ns) { return (R - 1) * ns; }
// row pitch of the exchange buffers: a multiple of 16 so the swizzle stays
// inside the row and 16-byte stores stay aligned
template <int N> constexpr int row_pitch() { return (N + 15) & ~15; }

// Stage twiddle tables: stage (NS, R) holds W_{NS*R}^{p*r}, 0 < r < R,
// p < NS, at (r - 1) * NS + p -- (R - 1) * NS entries, p fastest, so the
// butterflies of consecutive threads (consecutive p) read consecutive
// entries.  `base` below is the stage table advanced by the butterfly's p.
template <int R, int NS, typename C>
__device__ __forceinline__ void load_tw(C (&w)[R + 1], const C* __restrict__ base) {
#pragma unroll
  for (int r = 1; r < R; ++r) w[r] = __ldg(base + (r - 1) * NS);
}

// Complex Float twiddles derived from a few table entries: W^p, W^4p, W^8p
// are loaded and the other powers formed with at most three complex
// multiplications (a few ulp), three 8-byte loads per butterfly instead of
// R - 1.
template <int R, int NS>
__device__ __forceinline__ void derive_tw(float2 (&w)[R + 1], const float2* __restrict__ base) {
  if constexpr (R == 16) {
    w[1] = __ldg(base);
    w[4] = __ldg(base + 3 * NS);
    w[8] = __ldg(base + 7 * NS);
    w[2] = cmul(w[1], w[1]);
    w[3] = cmul(w[2], w[1]);
    w[5] = cmul(w[4], w[1]);
    w[6] = cmul(w[4], w[2]);
    w[7] = cmul(w[4], w[3]);
    w[9] = cmul(w[8], w[1]);
    w[10] = cmul(w[8], w[2]);
    w[11] = cmul(w[8], w[3]);
    w[12] = cmul(w[8], w[4]);
    w[13] = cmul(w[12], w[1]);
    w[14] = cmul(w[12], w[2]);
    w[15] = cmul(w[12], w[3]);
  } else if constexpr (R == 8) {
    w[1] = __ldg(base);
    w[4] = __ldg(base + 3 * NS);
    w[2] = cmul(w[1], w[1]);
    w[3] = cmul(w[2], w[1]);
    w[5] = cmul(w[4], w[1]);
    w[6] = cmul(w[4], w[2]);
    w[7] = cmul(w[4], w[3]);
  } else {
    load_tw<R, NS>(w, base);
  }
}

template <int N, int E, int NS, int R, typename C>
__device__ __forceinline__ void row_compute(C (&v)[E], const C* __restrict__ tw, int t) {
  constexpr int TH = N / E;
  constexpr int Q = E / R;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    if constexpr (NS > 1) {
      const int j = t + TH * q;
      const int p = j % NS;
      C w[R + 1];
      if constexpr (sizeof(C) == 8)
        derive_tw<R, NS>(w, tw + p);
      else
        load_tw<R, NS>(w, tw + p);
#pragma unroll
      for (int r = 1; r < R; ++r) v[q * R + r] = cmul(v[q * R + r], w[r]);
    }
    dft<R>(&v[q * R]);
  }
}

// After stage (NS, R): outputs go to smem in Stockham order (swizzled).
template <int N, int E, int NS, int R, typename C>
__device__ __forceinline__ void row_write(const C (&v)[E], C* buf, int t) {
  constexpr int TH = N / E;
  constexpr int Q = E / R;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int j = t + TH * q;
    if constexpr (NS == 1 && (R % 2 == 0) && sizeof(C) == 8) {
      // R consecutive outputs j*R + r: store as 16-byte pairs
#pragma unroll
      for (int r = 0; r < R; r += 2) {
        const int i = swz(j * R + r);
        *reinterpret_cast<float4*>(buf + i) =
            make_float4(v[q * R + r].x, v[q * R + r].y, v[q * R + r + 1].x, v[q * R + r + 1].y);
      }
    } else {
      const int p = j % NS;
      const int base = (j - p) * R + p;
#pragma unroll
      for (int r = 0; r < R; ++r) buf[swz(base + r * NS)] = v[q * R + r];
    }
  }
}

// Before a stage of radix R: v[q*R + r] = element j_q + r*N/R.
template <int N, int E, int R, typename C>
__device__ __forceinline__ void row_read(C (&v)[E], const C* buf, int t) {
  constexpr int TH = N / E;
  constexpr int Q = E / R;
#pragma unroll
  for (int q = 0; q < Q; ++q)
#pragma unroll
    for (int r = 0; r < R; ++r) v[q * R + r] = buf[swz(t + TH * q + r * (N / R))];
}


// ---- strided pencils (the y / z axes of fft2D / fft3D, spectral product) -----
// A CTA transforms W adjacent columns of a stride-es axis of length N: thread
// (x, t) holds elements t + TH*m of column x in registers, global accesses are
// W-column row segments, and the exchanges use a column-interleaved layout
// [i][x] (x fastest), which keeps every Stockham access pattern free of bank
// conflicts.  With F_SPEC the kernel multiplies the spectrum by filter[k*S +
// column], conjugates, and runs the same stages again straight from
// registers (the output index set of a transform is the input index set of
// the next), giving the forward z DFT, product and first inverse axis of the
// spectral convolution in one pass.
template <int N, int E, int NS, int R, int W, typename C>
__device__ __forceinline__ void str_write(const C (&v)[E], C* buf, int t, int x) {
  constexpr int TH = N / E;
  constexpr int Q = E / R;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int j = t + TH * q;
    const int p = j % NS;
    const int base = (j - p) * R + p;
#pragma unroll
    for (int r = 0; r < R; ++r) buf[(base + r * NS) * W + x] = v[q * R + r];
  }
}
template <int N, int E, int R, int W, typename C>
__device__ __forceinline__ void str_read(C (&v)[E], const C* buf, int t, int x) {
  constexpr int TH = N / E;
  constexpr int Q = E / R;
#pragma unroll
  for (int q = 0; q < Q; ++q)
#pragma unroll
    for (int r = 0; r < R; ++r) v[q * R + r] = buf[(t + TH * q + r * (N / R)) * W + x];
}
template <int N, int E, int NS, int OFF, int W, typename C, int R, int... Rest>
__device__ __forceinline__ void str_stages(C (&v)[E], C* b, const C* __restrict__ tw, int t, int x,
                                           RL<R, Rest...>) {
  row_compute<N, E, NS, R>(v, tw + OFF, t);
  if constexpr (sizeof...(Rest) > 0) {
    str_write<N, E, NS, R, W>(v, b, t, x);
    __syncthreads();
    constexpr int R2 = rl_first(RL<Rest...>{});
    str_read<N, E, R2, W>(v, b, t, x);
    __syncthreads();
    str_stages<N, E, NS * R, OFF + tw_entries<R>(NS), W>(v, b, tw, t, x, RL<Rest...>{});
  }
}

// Fused-operation sets of a strided pass, fixed at compile time so the
// unrolled load / store loops carry no per-element flag tests.
enum StrOps : uint32_t {
  SO_PLAIN = 0,                                  // conj / scale / L2 hints only
  SO_TW4 = F_TW4,                                // four-step first half
  SO_TW4B = F_TW4 | F_TW4_BATCH,                 //   ... exponent from the batch index
  SO_BP1 = F_PAD_IN | F_CHIRP_IN | F_TW4,        // Bluestein: chirp, pad, first half
  SO_FILT = F_FILTER_OUT,                        // Bluestein: second half, filter
  SO_COUT = F_CHIRP_OUT | F_TRUNC_OUT,           // Bluestein: last half, chirp, first n
  SO_SPEC = F_SPEC,                              // spectral product (second transform)
  SO_BLUE = F_PAD_IN | F_CHIRP_IN | F_BLUE | F_TRUNC_OUT,  // whole Bluestein in one tile
  SO_BMID = F_SPEC | F_TW4,                      // Bluestein middle: filter, inverse first half, twiddle
};
constexpr uint32_t kStrOpMask = F_TW4 | F_TW4_BATCH | F_PAD_IN | F_CHIRP_IN | F_FILTER_OUT | F_CHIRP_OUT |
                                F_TRUNC_OUT | F_SPEC | F_BLUE;

// Position of one thread's column inside a tile of a strided pass.
struct StrCtx {
  int x, t;                  // column within the tile, butterfly row
  int64_t c0, b_lo, b_hi;    // first column of the tile, batch indices
  int64_t col;               // this thread's column
  bool ok;                   // col < ncols
};

template <int N, int W>
__device__ __forceinline__ StrCtx str_ctx(const PassDesc& d, int64_t tile) {
  StrCtx c;
  c.x = threadIdx.x % W;
  c.t = threadIdx.x / W;
  const int64_t tiles = (d.ncols + W - 1) / W;
  const int64_t bq = tile / tiles;
  c.c0 = (tile - bq * tiles) * W;
  c.b_hi = bq / d.nb_lo;
  c.b_lo = bq - c.b_hi * d.nb_lo;
  c.col = c.c0 + c.x;
  c.ok = c.col < d.ncols;
  return c;
}

// Loads of one tile straight from global memory: thread (x, t) reads
// elements t + TH*m of its column, with conjugation, Bluestein chirp and
// zero padding as OPS asks.
template <typename T, int N, int W, uint32_t OPS, int R0>
__device__ __forceinline__ void str_load_global(const PassDesc& d, const StrCtx& c,
                                                typename CxT<T>::type (&v)[16]) {
  using C = typename CxT<T>::type;
  constexpr int E = 16;
  constexpr int TH = N / E;
  const uint32_t fl = d.flags;
  const T csign_in = (fl & F_CONJ_IN) ? T(-1) : T(1);
  const C* __restrict__ chirp = static_cast<const C*>(d.chirp);
  const bool stream_in = (fl & F_L2_IN_FIRST) != 0;
  const uint64_t ipol = stream_in ? l2_policy_first() : 0;
  const int64_t ies = d.in_es;
  const C* __restrict__ in = static_cast<const C*>(d.in) + c.b_lo * d.in_bs + c.b_hi * d.in_bs2 +
                             (c.ok ? (d.col_in_off ? d.col_in_off[c.col] : c.col * d.in_cs) : 0) +
                             int64_t(c.t) * ies;
#pragma unroll
  for (int q = 0; q < E / R0; ++q)
#pragma unroll
    for (int r = 0; r < R0; ++r) {
      const int m = q + r * (E / R0);
      const int i = c.t + TH * m;
      C e = cmake<C>(T(0), T(0));
      bool valid = c.ok;
      int64_t l = 0;
      if constexpr ((OPS & (F_PAD_IN | F_CHIRP_IN)) != 0) {
        l = int64_t(i) * d.lin_es + c.col * d.lin_cs;
        if ((OPS & F_PAD_IN) && l >= d.n_in) valid = false;
      }
      if (valid) {
        const C* a = in + int64_t(TH * m) * ies;
        e = stream_in ? ld_l2hint(a, ipol) : *a;
        e.y *= csign_in;
        if constexpr ((OPS & F_CHIRP_IN) != 0) e = cmul(e, chirp[l]);
      }
      v[q * R0 + r] = e;
    }
}

// Everything of a tile after its loads: the stages, the optional second
// transform (spectral product or in-kernel Bluestein), the store-side
// operations and the stores.  b is the tile's exchange buffer (N*W
// elements); every thread must be done reading its inputs from b, if they
// came from there, before the call.
template <typename T, int N, int W, uint32_t OPS, int... Rs>
__device__ __forceinline__ void str_finish(const PassDesc& d, const StrCtx& c,
                                           typename CxT<T>::type (&v)[16], typename CxT<T>::type* b) {
  using C = typename CxT<T>::type;
  constexpr int E = 16;
  constexpr int TH = N / E;
  constexpr int R0 = rl_first(RL<Rs...>{});
  constexpr int RZ = rl_last(RL<Rs...>{});
  const int x = c.x, t = c.t;
  const int64_t col = c.col, c0 = c.c0;
  const bool ok = c.ok;
  const uint32_t fl = d.flags;
  const C* __restrict__ tw = static_cast<const C*>(d.tw);
  const C* __restrict__ chirp = static_cast<const C*>(d.chirp);
  const C* __restrict__ filt = static_cast<const C*>(d.filter);
  str_stages<N, E, 1, 0, W>(v, b, tw, t, x, RL<Rs...>{});
  if constexpr ((OPS & (F_SPEC | F_BLUE)) != 0) {
    // v[q*RZ + r] holds X[k], k = t + TH*(q + r*E/RZ); the next transform's
    // first stage wants x[t + TH*(q' + r'*E/R0)] in v[q'*R0 + r']
    C u[E];
#pragma unroll
    for (int q = 0; q < E / RZ; ++q)
#pragma unroll
      for (int r = 0; r < RZ; ++r) {
        const int m = q + r * (E / RZ);
        const int k = t + TH * m;
        C h = cmake<C>(T(0), T(0));
        if (ok) {
          if constexpr ((OPS & F_SPEC) != 0)
            h = filt[int64_t(k) * d.lout_es + col * d.lout_cs];
          else
            h = filt[k];
        }
        u[(m % (E / R0)) * R0 + m / (E / R0)] = cconj(cmul(v[q * RZ + r], h));
      }
#pragma unroll
    for (int i = 0; i < E; ++i) v[i] = u[i];
    __syncthreads();
    str_stages<N, E, 1, 0, W>(v, b, tw, t, x, RL<Rs...>{});
  }
  const T s = (fl & F_SCALE) ? T(d.scale) : T(1);
  const T csign_out = (fl & F_CONJ_OUT) ? T(-1) : T(1);
  const bool keep = (fl & F_L2_OUT_LAST) != 0;
  const uint64_t pol = keep ? l2_policy_last() : 0;
  const C* __restrict__ tw4_lo = static_cast<const C*>(d.tw4_lo);
  const C* __restrict__ tw4_hi = static_cast<const C*>(d.tw4_hi);
  const int tw4_shift = d.tw4_shift;
  const int64_t tw4_mask = (int64_t(1) << tw4_shift) - 1;
  const int64_t b_lo = c.b_lo;
  C* __restrict__ out = static_cast<C*>(d.out) + c.b_lo * d.out_bs + c.b_hi * d.out_bs2;
  const int64_t oes = d.out_es;
  // post-operations of output k of column cl; returns false when truncated
  auto post = [&](C& e, int k, int64_t cl) -> bool {
    int64_t l = 0;
    if constexpr ((OPS & (F_FILTER_OUT | F_CHIRP_OUT | F_BLUE | F_TRUNC_OUT)) != 0) {
      l = int64_t(k) * d.lout_es + cl * d.lout_cs;
      if ((OPS & F_TRUNC_OUT) && l >= d.n_out) return false;
    }
    if constexpr ((OPS & F_TW4) != 0) {
      const int64_t tt = ((OPS & F_TW4_BATCH) ? b_lo : cl) * int64_t(k);
      e = cmul(e, cmul(tw4_hi[tt >> tw4_shift], tw4_lo[tt & tw4_mask]));
    }
    if constexpr ((OPS & F_FILTER_OUT) != 0) e = cconj(cmul(e, filt[l]));
    if constexpr ((OPS & (F_BLUE | F_CHIRP_OUT)) != 0) e = cmul(cconj(e), chirp[l]);
    e.x *= s;
    e.y *= s * csign_out;
    return true;
  };
  // the same with 32-bit index arithmetic: the four-step exponent
  // (column or batch) * k below 2^32, the axis index l below 2^31
  auto post32 = [&](C& e, uint32_t k, uint32_t cl) -> bool {
    uint32_t l = 0;
    if constexpr ((OPS & (F_FILTER_OUT | F_CHIRP_OUT | F_BLUE | F_TRUNC_OUT)) != 0) {
      l = k * uint32_t(d.lout_es) + cl * uint32_t(d.lout_cs);
      if ((OPS & F_TRUNC_OUT) && int64_t(l) >= d.n_out) return false;
    }
    if constexpr ((OPS & F_TW4) != 0) {
      const uint32_t tt = ((OPS & F_TW4_BATCH) ? uint32_t(b_lo) : cl) * k;
      e = cmul(e, cmul(tw4_hi[tt >> tw4_shift], tw4_lo[tt & uint32_t(tw4_mask)]));
    }
    if constexpr ((OPS & F_FILTER_OUT) != 0) e = cconj(cmul(e, filt[l]));
    if constexpr ((OPS & (F_BLUE | F_CHIRP_OUT)) != 0) e = cmul(cconj(e), chirp[l]);
    e.x *= s;
    e.y *= s * csign_out;
    return true;
  };
  if (d.out_cs == 1 && !d.col_out_off) {
    if (!ok) return;
    C* o0 = out + col + int64_t(t) * oes;
#pragma unroll
    for (int q = 0; q < E / RZ; ++q)
#pragma unroll
      for (int r = 0; r < RZ; ++r) {
        const int m = q + r * (E / RZ);
        C e = v[q * RZ + r];
        const int k = t + TH * m;
        if (!post(e, k, col)) continue;
        C* o = o0 + int64_t(TH * m) * oes + rot_delta(d, int64_t(k) * d.lout_es + col * d.lout_cs);
        if (keep)
          st_l2hint(o, e, pol);
        else
          *o = e;
      }
  } else {
    // transposed store through shared memory: a warp writes consecutive k.
    // Row k of the staging buffer holds column x at slot x ^ (k mod W) (W is
    // a power of two), so both the row writes and the column reads of
    // consecutive k hit distinct banks.
    static_assert((W & (W - 1)) == 0, "W must be a power of two");
    __syncthreads();
#pragma unroll
    for (int q = 0; q < E / RZ; ++q)
#pragma unroll
      for (int r = 0; r < RZ; ++r) {
        const int k = t + TH * (q + r * (E / RZ));
        b[k * W + (x ^ (k & (W - 1)))] = v[q * RZ + r];
      }
    __syncthreads();
    // 32-bit offsets and exponents when the tile allows (no per-column
    // offsets, no rotation, every product in range): the common case
    const int64_t clast = c0 + W - 1;
    const int64_t lim31 = int64_t(1) << 31;
    const bool small = !d.col_out_off && !(d.flags & F_ROT_OUT) &&
                       int64_t(W - 1) * d.out_cs + int64_t(N - 1) * oes < lim31 &&
                       clast * d.lout_cs + int64_t(N - 1) * d.lout_es < lim31 &&
                       ((OPS & F_TW4) == 0 ||
                        ((OPS & F_TW4_BATCH) ? b_lo : clast) * int64_t(N - 1) < (int64_t(1) << 32)) &&
                       clast < lim31;
    if (small) {
      C* __restrict__ ob = out + c0 * d.out_cs;
      const int ocs = int(d.out_cs), oes32 = int(oes);
      const int cmax = int(d.ncols - c0 < W ? d.ncols - c0 : W);
#pragma unroll 4
      for (int f = threadIdx.x; f < N * W; f += W * TH) {
        const int cc = f / N, k = f % N;
        if (cc >= cmax) continue;
        C e = b[k * W + (cc ^ (k & (W - 1)))];
        if (!post32(e, uint32_t(k), uint32_t(c0 + cc))) continue;
        C* o = ob + (cc * ocs + k * oes32);
        if (keep)
          st_l2hint(o, e, pol);
        else
          *o = e;
      }
      return;
    }
#pragma unroll 4
    for (int f = threadIdx.x; f < N * W; f += W * TH) {
      const int cc = f / N, k = f % N;
      const int64_t cl = c0 + cc;
      if (cl >= d.ncols) continue;
      C e = b[k * W + (cc ^ (k & (W - 1)))];
      if (!post(e, k, cl)) continue;
      const int64_t cb = d.col_out_off ? d.col_out_off[cl] : cl * d.out_cs;
      C* o = out + cb + int64_t(k) * oes + rot_delta(d, int64_t(k) * d.lout_es + cl * d.lout_cs);
      if (keep)
        st_l2hint(o, e, pol);
      else
        *o = e;
    }
  }
}

// One tile (W columns) of a strided pass.  OPS selects the fused operations:
// conjugate, Bluestein chirp and zero padding on load; spectral product or
// in-kernel Bluestein (second transform from registers); four-step twiddle,
// filter, chirp, truncation, scale and conjugate on store.  Stores go
// straight from registers when consecutive columns are adjacent in memory
// (out_cs == 1); otherwise (the transposed store of a four-step first half)
// they go through shared memory so that a warp writes consecutive k.
template <typename T, int N, int W, uint32_t OPS, int... Rs>
__device__ __forceinline__ void str_tile(const PassDesc& d, int64_t tile, unsigned char* smem_raw) {
  using C = typename CxT<T>::type;
  constexpr int R0 = rl_first(RL<Rs...>{});
  const StrCtx c = str_ctx<N, W>(d, tile);
  C v[16];
  str_load_global<T, N, W, OPS, R0>(d, c, v);
  str_finish<T, N, W, OPS, Rs...>(d, c, v, reinterpret_cast<C*>(smem_raw));
}

// Calls the instantiation for the pass's fused-operation set.
template <typename T, int N, int W, int... Rs>
__device__ __forceinline__ bool str_tile_dispatch(const PassDesc& d, int64_t tile, unsigned char* smem) {
  switch (d.flags & kStrOpMask) {
    case SO_PLAIN: str_tile<T, N, W, SO_PLAIN, Rs...>(d, tile, smem); return true;
    case SO_TW4: str_tile<T, N, W, SO_TW4, Rs...>(d, tile, smem); return true;
    case SO_TW4B: str_tile<T, N, W, SO_TW4B, Rs...>(d, tile, smem); return true;
    case SO_BP1: str_tile<T, N, W, SO_BP1, Rs...>(d, tile, smem); return true;
    case SO_FILT: str_tile<T, N, W, SO_FILT, Rs...>(d, tile, smem); return true;
    case SO_COUT: str_tile<T, N, W, SO_COUT, Rs...>(d, tile, smem); return true;
    case SO_SPEC: str_tile<T, N, W, SO_SPEC, Rs...>(d, tile, smem); return true;
    case SO_BLUE: str_tile<T, N, W, SO_BLUE, Rs...>(d, tile, smem); return true;
    case SO_BMID: str_tile<T, N, W, SO_BMID, Rs...>(d, tile, smem); return true;
    default: return false;
  }
}

// The sets the ragged executor generates (four-step halves, multi-pass
// Bluestein): only these are instantiated inside its persistent kernel.
__host__ __device__ constexpr bool str_ops_ragged(uint32_t ops) {
  return ops == SO_PLAIN || ops == SO_TW4 || ops == SO_BP1 || ops == SO_BMID || ops == SO_COUT;
}
template <typename T, int N, int W, int... Rs>
__device__ __forceinline__ bool str_tile_dispatch_ragged(const PassDesc& d, int64_t tile, unsigned char* smem) {
  switch (d.flags & kStrOpMask) {
    case SO_PLAIN: str_tile<T, N, W, SO_PLAIN, Rs...>(d, tile, smem); return true;
    case SO_TW4: str_tile<T, N, W, SO_TW4, Rs...>(d, tile, smem); return true;
    case SO_BP1: str_tile<T, N, W, SO_BP1, Rs...>(d, tile, smem); return true;
    case SO_BMID: str_tile<T, N, W, SO_BMID, Rs...>(d, tile, smem); return true;
    case SO_COUT: str_tile<T, N, W, SO_COUT, Rs...>(d, tile, smem); return true;
    default: return false;
  }
}

// True when a pass's fused operations are one of the strided kernel's sets.
__host__ __device__ inline bool str_ops_supported(uint32_t flags) {
  switch (flags & kStrOpMask) {
    case SO_PLAIN: case SO_TW4: case SO_TW4B: case SO_BP1: case SO_FILT: case SO_COUT: case SO_SPEC:
    case SO_BLUE: case SO_BMID:
      return true;
    default:
      return false;
  }
}

}  // namespace gbfft
