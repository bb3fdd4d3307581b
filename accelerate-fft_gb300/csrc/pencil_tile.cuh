// Device body of the generic pencil pass (shared by the per-pass kernel and
// the persistent ragged-batch executor).
#pragma once

#include "butterflies.cuh"
#include "gbfft_internal.h"

namespace gbfft {

__device__ __forceinline__ int spad(int i) { return i + (i >> 4); }

// Division by a run-time divisor d (1 <= d <= 2^16) of indices x < 2^16 by a
// multiply-high with m = ceil(2^32 / d) (division by invariant integers,
// Granlund and Montgomery 1994): with m = 2^32/d + e, 0 <= e < 1, the error
// x*e/2^32 < 2^-16 <= 1/d never carries floor(x/d) to the next integer.
// Replaces the ~20-instruction integer division in the per-element index
// arithmetic of the tile loops.
struct FDiv {
  uint32_t m, d;
  __device__ __forceinline__ explicit FDiv(uint32_t dd) : m(dd > 1 ? 0xFFFFFFFFu / dd + 1u : 0u), d(dd) {}
  __device__ __forceinline__ uint32_t div(uint32_t x) const { return d > 1 ? __umulhi(x, m) : x; }
};

template <typename C>
__device__ __forceinline__ C ldg_c(const C* p) {
  return __ldg(p);
}

// One Stockham stage of radix R over every pencil of the tile:
// butterfly j reads src[j + r*n/R], twiddles by W_{Ns*R}^{(j mod Ns)*r},
// and writes dst[(j/Ns)*Ns*R + (j mod Ns) + r*Ns].  The stage twiddle table
// holds W_{Ns*R}^{p*r}, 0 < r < R, at (r - 1)*Ns + p.
template <int R, typename C>
__device__ __forceinline__ void stage(const C* __restrict__ src, C* __restrict__ dst,
                                      const C* __restrict__ tw, int n, int Ns, int W, int pitch) {
  const int nb = n / R;
  const int total = W * nb;
  const FDiv div_nb{uint32_t(nb)}, div_ns{uint32_t(Ns)};
  for (int f = threadIdx.x; f < total; f += blockDim.x) {
    const int c = int(div_nb.div(uint32_t(f)));
    const int j = f - c * nb;
    const C* s = src + c * pitch;
    C* o = dst + c * pitch;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = s[spad(j + r * nb)];
    const int p = j - int(div_ns.div(uint32_t(j))) * Ns;
    if (Ns > 1) {
      const C* t = tw + p;
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], ldg_c(t + (r - 1) * Ns));
    }
    dft<R>(v);
    const int base = (j - p) * R + p;
#pragma unroll
    for (int r = 0; r < R; ++r) o[spad(base + r * Ns)] = v[r];
  }
}

// Runs every stage; returns the buffer holding the natural-order result.
template <typename C>
__device__ C* run_stages(const PassDesc& d, C* b0, C* b1) {
  const C* tw = static_cast<const C*>(d.tw);
  C* src = b0;
  C* dst = b1;
  for (int s = 0; s < d.nstages; ++s) {
    const StageInfo si = d.st[s];
    const C* t = tw + si.tw_off;
    switch (si.radix) {
      case 16: stage<16>(src, dst, t, d.n, si.ns, d.W, d.pitch); break;
      case 8: stage<8>(src, dst, t, d.n, si.ns, d.W, d.pitch); break;
      case 4: stage<4>(src, dst, t, d.n, si.ns, d.W, d.pitch); break;
      case 2: stage<2>(src, dst, t, d.n, si.ns, d.W, d.pitch); break;
      case 3: stage<3>(src, dst, t, d.n, si.ns, d.W, d.pitch); break;
      case 5: stage<5>(src, dst, t, d.n, si.ns, d.W, d.pitch); break;
      case 7: stage<7>(src, dst, t, d.n, si.ns, d.W, d.pitch); break;
      case 6: stage<6>(src, dst, t, d.n, si.ns, d.W, d.pitch); break;
      case 9: stage<9>(src, dst, t, d.n, si.ns, d.W, d.pitch); break;
      case 10: stage<10>(src, dst, t, d.n, si.ns, d.W, d.pitch); break;
      case 12: stage<12>(src, dst, t, d.n, si.ns, d.W, d.pitch); break;
      case 14: stage<14>(src, dst, t, d.n, si.ns, d.W, d.pitch); break;
      case 15: stage<15>(src, dst, t, d.n, si.ns, d.W, d.pitch); break;
      default: break;
    }
    __syncthreads();
    C* tmp = src;
    src = dst;
    dst = tmp;
  }
  return src;
}

// Load phase of a generic tile: element i of tile column c goes to
// b0[c*pitch + spad(i)], with conjugation, Bluestein chirp and zero padding.
// KL elements per thread per round: every global load of a round (data, then
// chirp) is issued before any is used.  I is the type of the per-element
// offsets inside the tile (int when they fit in 31 bits: one widening
// multiply-add per address instead of 64-bit products).
template <typename T, typename I, int KL>
__device__ __forceinline__ void pencil_load(const PassDesc& d, const typename CxT<T>::type* __restrict__ in,
                                            typename CxT<T>::type* b0, int64_t c0, const FDiv& div_w,
                                            const FDiv& div_n) {
  using C = typename CxT<T>::type;
  const int W = d.W, n = d.n;
  const int total = W * n;
  const int step = int(blockDim.x);
  const uint32_t fl = d.flags;
  const C* __restrict__ chirp = static_cast<const C*>(d.chirp);
  const I ies = I(d.in_es), ics = I(d.in_cs);
  // the tile's first column (per-column offsets are absolute)
  const C* __restrict__ base = in + (d.col_in_off ? 0 : c0 * d.in_cs);
  for (int f0 = threadIdx.x; f0 < total; f0 += KL * step) {
    int sidx[KL];
    int64_t lidx[KL], cofs[KL];
    I ofs[KL];
    bool inr[KL], ok[KL];
#pragma unroll
    for (int u = 0; u < KL; ++u) {
      const int f = f0 + u * step;
      inr[u] = f < total;
      int c, i;
      if (d.load_cfast) {
        i = int(div_w.div(uint32_t(f)));
        c = f - i * W;
      } else {
        c = int(div_n.div(uint32_t(f)));
        i = f - c * n;
      }
      const int64_t col = c0 + c;
      bool valid = inr[u] && col < d.ncols;
      int64_t l = 0;
      if (fl & (F_PAD_IN | F_CHIRP_IN)) {
        l = int64_t(i) * d.lin_es + col * d.lin_cs;
        if ((fl & F_PAD_IN) && l >= d.n_in) valid = false;
      }
      ok[u] = valid;
      lidx[u] = l;
      sidx[u] = c * d.pitch + spad(i);
      ofs[u] = I(i) * ies + (d.col_in_off ? I(0) : I(c) * ics);
      cofs[u] = (d.col_in_off && valid) ? d.col_in_off[col] : 0;
    }
    C v[KL];
#pragma unroll
    for (int u = 0; u < KL; ++u) v[u] = ok[u] ? base[cofs[u] + ofs[u]] : cmake<C>(T(0), T(0));
    if (fl & F_CHIRP_IN) {
      C ch[KL];
#pragma unroll
      for (int u = 0; u < KL; ++u) ch[u] = ok[u] ? chirp[lidx[u]] : cmake<C>(T(0), T(0));
#pragma unroll
      for (int u = 0; u < KL; ++u) {
        if (fl & F_CONJ_IN) v[u].y = -v[u].y;
        v[u] = cmul(v[u], ch[u]);
      }
    } else if (fl & F_CONJ_IN) {
#pragma unroll
      for (int u = 0; u < KL; ++u) v[u].y = -v[u].y;
    }
#pragma unroll
    for (int u = 0; u < KL; ++u)
      if (inr[u]) b0[sidx[u]] = v[u];
  }
}

// Store phase: output k of tile column c from res[c*pitch + spad(k)], with
// four-step twiddle, filter, chirp, truncation, scale and conjugation.  KU
// outputs per thread per round; the table loads of a round are issued
// together before the arithmetic, and index work a flag does not need is
// skipped.
template <typename T, typename I>
__device__ __forceinline__ void pencil_store(const PassDesc& d, typename CxT<T>::type* __restrict__ out,
                                             const typename CxT<T>::type* res, int64_t c0, int64_t b,
                                             const FDiv& div_w, const FDiv& div_n) {
  using C = typename CxT<T>::type;
  constexpr int KU = 4;
  const int W = d.W, n = d.n;
  const int total = W * n;
  const int step = int(blockDim.x);
  const uint32_t fl = d.flags;
  const C* __restrict__ tw4_lo = static_cast<const C*>(d.tw4_lo);
  const C* __restrict__ tw4_hi = static_cast<const C*>(d.tw4_hi);
  const C* __restrict__ filt = static_cast<const C*>(d.filter);
  const C* __restrict__ chirp = static_cast<const C*>(d.chirp);
  const int64_t tw4_mask = (int64_t(1) << d.tw4_shift) - 1;
  const T sc = (fl & F_SCALE) ? T(d.scale) : T(1);
  const bool need_l = (fl & (F_FILTER_OUT | F_CHIRP_OUT | F_BLUE | F_TRUNC_OUT | F_ROT_OUT)) != 0;
  const I oes = I(d.out_es), ocs = I(d.out_cs);
  C* __restrict__ base = out + (d.col_out_off ? 0 : c0 * d.out_cs);
  for (int f0 = threadIdx.x; f0 < total; f0 += KU * step) {
    C v[KU];
    int64_t lidx[KU], cofs[KU];
    uint32_t tt[KU];  // four-step exponent: column (or batch) * k < n <= 2^26
    I ofs[KU];
    bool ok[KU];
#pragma unroll
    for (int u = 0; u < KU; ++u) {
      const int f = f0 + u * step;
      int c, kk;
      if (d.store_cfast) {
        kk = int(div_w.div(uint32_t(f)));
        c = f - kk * W;
      } else {
        c = int(div_n.div(uint32_t(f)));
        kk = f - c * n;
      }
      const int64_t col = c0 + c;
      bool valid = f < total && col < d.ncols;
      int64_t l = 0;
      if (need_l) {
        l = int64_t(kk) * d.lout_es + col * d.lout_cs;
        if ((fl & F_TRUNC_OUT) && l >= d.n_out) valid = false;
      }
      ok[u] = valid;
      lidx[u] = valid ? l : 0;
      // e < N/n and kk < n, so the four-step exponent stays below N
      tt[u] = (valid && (fl & F_TW4)) ? uint32_t((fl & F_TW4_BATCH) ? b : col) * uint32_t(kk) : 0u;
      v[u] = valid ? res[c * d.pitch + spad(kk)] : cmake<C>(T(0), T(0));
      ofs[u] = I(kk) * oes + (d.col_out_off ? I(0) : I(c) * ocs);
      cofs[u] = (d.col_out_off && valid) ? d.col_out_off[col] : 0;
    }
    if (fl & F_TW4) {
      C wh[KU], wl[KU];
#pragma unroll
      for (int u = 0; u < KU; ++u) {
        wh[u] = tw4_hi[tt[u] >> d.tw4_shift];
        wl[u] = tw4_lo[tt[u] & uint32_t(tw4_mask)];
      }
#pragma unroll
      for (int u = 0; u < KU; ++u) v[u] = cmul(v[u], cmul(wh[u], wl[u]));
    }
    if (fl & F_FILTER_OUT) {
      C h[KU];
#pragma unroll
      for (int u = 0; u < KU; ++u) h[u] = filt[lidx[u]];
#pragma unroll
      for (int u = 0; u < KU; ++u) v[u] = cconj(cmul(v[u], h[u]));
    }
    if (fl & (F_BLUE | F_CHIRP_OUT)) {
      C ch[KU];
#pragma unroll
      for (int u = 0; u < KU; ++u) ch[u] = chirp[lidx[u]];
#pragma unroll
      for (int u = 0; u < KU; ++u) v[u] = cmul(cconj(v[u]), ch[u]);
    }
#pragma unroll
    for (int u = 0; u < KU; ++u) {
      if (!ok[u]) continue;
      C e = v[u];
      if (fl & F_SCALE) e = cscale(e, sc);
      if (fl & F_CONJ_OUT) e.y = -e.y;
      base[cofs[u] + ofs[u] + rot_delta(d, lidx[u])] = e;
    }
  }
}

// True when every per-element offset inside a tile of `d` fits in 31 bits.
__device__ __forceinline__ bool tile_idx32(const PassDesc& d) {
  const int64_t lim = int64_t(1) << 31;
  const int64_t in_span = int64_t(d.n - 1) * d.in_es + (d.col_in_off ? 0 : int64_t(d.W - 1) * d.in_cs);
  const int64_t out_span = int64_t(d.n - 1) * d.out_es + (d.col_out_off ? 0 : int64_t(d.W - 1) * d.out_cs);
  return in_span < lim && out_span < lim && d.in_es < lim && d.out_es < lim && d.in_cs < lim && d.out_cs < lim;
}

// Transforms tile `tile` of pass `d` (tiles enumerate (batch, column block)).
// `smem_raw` holds two buffers of d.W * d.pitch elements.  When
// d.col_in_off / d.col_out_off are set, column c of the tile starts at those
// element offsets instead of c * cs.
// SMALL: the caller guarantees 31-bit offsets inside every tile (the ragged
// executor: strides within one transform), so only that version is built.
template <typename T, bool SMALL = false>
__device__ void pencil_tile(const PassDesc& d, int64_t tile, unsigned char* smem_raw) {
  using C = typename CxT<T>::type;
  C* b0 = reinterpret_cast<C*>(smem_raw);
  C* b1 = b0 + d.W * d.pitch;

  const int64_t tiles = (d.ncols + d.W - 1) / d.W;
  const int64_t bq = tile / tiles;
  const int64_t c0 = (tile - bq * tiles) * d.W;
  const int64_t b_hi = bq / d.nb_lo;
  const int64_t b = bq - b_hi * d.nb_lo;
  const int W = d.W, n = d.n;
  const C* __restrict__ in = static_cast<const C*>(d.in) + b * d.in_bs + b_hi * d.in_bs2;
  const uint32_t fl = d.flags;

  // ---- load (+ conj, chirp, zero padding) ---------------------------------
  const int total = W * n;
  const FDiv div_w{uint32_t(W)}, div_n{uint32_t(n)};
  const bool idx32 = SMALL || tile_idx32(d);
  // the ragged executor's tiles keep eight loads in flight per thread, the
  // per-pass kernel four (its registers bound the resident CTAs)
  constexpr int KL = SMALL ? 8 : 4;
  if (idx32)
    pencil_load<T, int, KL>(d, in, b0, c0, div_w, div_n);
  else if constexpr (!SMALL)
    pencil_load<T, int64_t, KL>(d, in, b0, c0, div_w, div_n);
  __syncthreads();

  C* res = run_stages<C>(d, b0, b1);

  if (fl & F_SPEC) {
    // spectrum * filter[k*lout_es + col*lout_cs], then the next transform of
    // the conjugate (the first axis of an inverse taken as conj(DFT(conj)))
    const C* filt = static_cast<const C*>(d.filter);
    for (int f = threadIdx.x; f < total; f += blockDim.x) {
      int c, kk;
      if (d.store_cfast) {
        kk = int(div_w.div(uint32_t(f)));
        c = f - kk * W;
      } else {
        c = int(div_n.div(uint32_t(f)));
        kk = f - c * n;
      }
      const int64_t col = c0 + c;
      C* p = res + c * d.pitch + spad(kk);
      const C h = (col < d.ncols) ? filt[int64_t(kk) * d.lout_es + col * d.lout_cs] : cmake<C>(T(0), T(0));
      *p = cconj(cmul(*p, h));
    }
    __syncthreads();
    C* other = (res == b0) ? b1 : b0;
    res = run_stages<C>(d, res, other);
  }
  if (fl & F_BLUE) {
    // spectrum * filter, then the inverse DFT as conj(DFT(conj(.)))
    const C* filt = static_cast<const C*>(d.filter);
    for (int f = threadIdx.x; f < total; f += blockDim.x) {
      const int c = int(div_n.div(uint32_t(f))), kk = f - c * n;
      C* p = res + c * d.pitch + spad(kk);
      *p = cconj(cmul(*p, filt[kk]));
    }
    __syncthreads();
    C* other = (res == b0) ? b1 : b0;
    res = run_stages<C>(d, res, other);
  }

  // ---- store (+ twiddle, filter, chirp, scale, conj, truncation) ---------
  C* __restrict__ out = static_cast<C*>(d.out) + b * d.out_bs + b_hi * d.out_bs2;
  if (idx32)
    pencil_store<T, int>(d, out, res, c0, b, div_w, div_n);
  else if constexpr (!SMALL)
    pencil_store<T, int64_t>(d, out, res, c0, b, div_w, div_n);
}


}  // namespace gbfft
