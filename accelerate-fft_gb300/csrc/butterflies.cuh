// Register-level forward DFT kernels of radix 2, 3, 4, 5, 7, 8 and 16 on
// interleaved complex values (float2 / double2).  Only the forward sign
// (exp(-2*pi*i*j*k/R)) exists: backward transforms run as
// conj(forward(conj(x))), folded into the loads and stores of a pass.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace gbfft {

template <typename T> struct CxT;
template <> struct CxT<float> { using type = float2; };
template <> struct CxT<double> { using type = double2; };

template <typename C> __device__ __forceinline__ C cmake(decltype(C::x) x, decltype(C::x) y) {
  C r;
  r.x = x;
  r.y = y;
  return r;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return cmake<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return cmake<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  return cmake<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C> __device__ __forceinline__ C cconj(C a) { return cmake<C>(a.x, -a.y); }
// a * (-i)
template <typename C> __device__ __forceinline__ C cmul_mi(C a) { return cmake<C>(a.y, -a.x); }
template <typename C, typename T> __device__ __forceinline__ C cscale(C a, T s) {
  return cmake<C>(a.x * s, a.y * s);
}
// a * (c + i s) with constant c, s
template <typename C> __device__ __forceinline__ C cmulc(C a, double c, double s) {
  using T = decltype(C::x);
  return cmake<C>(a.x * T(c) - a.y * T(s), a.x * T(s) + a.y * T(c));
}

namespace k {
constexpr double r2 = 0.7071067811865475244008444;
constexpr double c16 = 0.9238795325112867561281832;  // cos(pi/8)
constexpr double s16 = 0.3826834323650897717284600;  // sin(pi/8)
}  // namespace k

// cos(2*pi*idx/R) and sin(2*pi*idx/R) for the odd radices, idx in [1, R).
__host__ __device__ constexpr double odd_cos(int R, int idx) {
  return R == 3 ? -0.5
       : R == 5 ? (idx == 1 || idx == 4 ? 0.3090169943749474241022934 : -0.8090169943749474241022934)
       : (idx == 1 || idx == 6) ? 0.6234898018587335305250049
       : (idx == 2 || idx == 5) ? -0.2225209339563144042889026
                                : -0.9009688679024191262361023;
}
__host__ __device__ constexpr double odd_sin(int R, int idx) {
  return R == 3 ? (idx == 1 ? 0.8660254037844386467637232 : -0.8660254037844386467637232)
       : R == 5 ? (idx == 1 ? 0.9510565162951535721164393
                 : idx == 2 ? 0.5877852522924731291687060
                 : idx == 3 ? -0.5877852522924731291687060
                            : -0.9510565162951535721164393)
       : idx == 1 ? 0.7818314824680298087084445
       : idx == 2 ? 0.9749279121818236070181317
       : idx == 3 ? 0.4338837391175581204757683
       : idx == 4 ? -0.4338837391175581204757683
       : idx == 5 ? -0.9749279121818236070181317
                  : -0.7818314824680298087084445;
}

template <typename C> __device__ __forceinline__ void dft2(C* v) {
  C t = v[0];
  v[0] = cadd(t, v[1]);
  v[1] = csub(t, v[1]);
}

template <typename C> __device__ __forceinline__ void dft4(C& x0, C& x1, C& x2, C& x3) {
  C t0 = cadd(x0, x2), t1 = csub(x0, x2), t2 = cadd(x1, x3), t3 = cmul_mi(csub(x1, x3));
  x0 = cadd(t0, t2);
  x2 = csub(t0, t2);
  x1 = cadd(t1, t3);
  x3 = csub(t1, t3);
}

template <typename C> __device__ __forceinline__ void dft4(C* v) { dft4(v[0], v[1], v[2], v[3]); }

// radix 8 = 2 x 4: even/odd halves, then W8 twiddles.
template <typename C> __device__ __forceinline__ void dft8(C* v) {
  C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  C o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4(e0, e1, e2, e3);
  dft4(o0, o1, o2, o3);
  using T = decltype(C::x);
  o1 = cmake<C>(T(k::r2) * (o1.x + o1.y), T(k::r2) * (o1.y - o1.x));
  o2 = cmul_mi(o2);
  o3 = cmake<C>(T(k::r2) * (o3.y - o3.x), T(-k::r2) * (o3.x + o3.y));
  v[0] = cadd(e0, o0);
  v[4] = csub(e0, o0);
  v[1] = cadd(e1, o1);
  v[5] = csub(e1, o1);
  v[2] = cadd(e2, o2);
  v[6] = csub(e2, o2);
  v[3] = cadd(e3, o3);
  v[7] = csub(e3, o3);
}

// radix 16 = 4 x 4: DFT4 over stride-4 inputs, W16 twiddles, DFT4 across.
template <typename C> __device__ __forceinline__ void dft16(C* v) {
#pragma unroll
  for (int j2 = 0; j2 < 4; ++j2) dft4(v[j2], v[j2 + 4], v[j2 + 8], v[j2 + 12]);
  // v[j2 + 4*k1] *= W16^(j2*k1)
  v[5] = cmulc(v[5], k::c16, -k::s16);    // W^1
  v[6] = cmulc(v[6], k::r2, -k::r2);      // W^2
  v[7] = cmulc(v[7], k::s16, -k::c16);    // W^3
  v[9] = cmulc(v[9], k::r2, -k::r2);      // W^2
  v[10] = cmul_mi(v[10]);                 // W^4
  v[11] = cmulc(v[11], -k::r2, -k::r2);   // W^6
  v[13] = cmulc(v[13], k::s16, -k::c16);  // W^3
  v[14] = cmulc(v[14], -k::r2, -k::r2);   // W^6
  v[15] = cmulc(v[15], -k::c16, k::s16);  // W^9
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) dft4(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
  // X[k1 + 4*k2] = v[4*k1 + k2]: transpose the 4x4 block
  C t[16];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) t[a + 4 * b] = v[4 * a + b];
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = t[i];
}

// Odd radix R in {3, 5, 7}: conjugate-symmetric pairing, y_m = r_m -/+ i s_m.
template <int R, typename C> __device__ __forceinline__ void dft_odd(C* v) {
  using T = decltype(C::x);
  constexpr int H = (R - 1) / 2;
  C a[H], b[H];
#pragma unroll
  for (int q = 1; q <= H; ++q) {
    a[q - 1] = cadd(v[q], v[R - q]);
    b[q - 1] = csub(v[q], v[R - q]);
  }
  C out[R];
  C y0 = v[0];
#pragma unroll
  for (int q = 0; q < H; ++q) y0 = cadd(y0, a[q]);
  out[0] = y0;
#pragma unroll
  for (int m = 1; m <= H; ++m) {
    C r = v[0];
    T sx = T(0), sy = T(0);
#pragma unroll
    for (int q = 1; q <= H; ++q) {
      const int idx = (m * q) % R;
      const T c = T(odd_cos(R, idx)), s = T(odd_sin(R, idx));
      r.x += c * a[q - 1].x;
      r.y += c * a[q - 1].y;
      sx += s * b[q - 1].x;
      sy += s * b[q - 1].y;
    }
    out[m] = cmake<C>(r.x + sy, r.y - sx);
    out[R - m] = cmake<C>(r.x - sy, r.y + sx);
  }
#pragma unroll
  for (int i = 0; i < R; ++i) v[i] = out[i];
}

// cos and sin of 2*pi*a/den at compile time: exact integer reduction to an
// octant (8a = q*den + r) and Taylor series on [0, pi/4] (terms to x^25, well
// below double rounding).  Used for the internal twiddles of the composite
// radices.
namespace cx {
constexpr double kPi4 = 0.78539816339744830961566084581988;  // pi / 4
constexpr double poly_sin(double x) {
  double x2 = x * x, term = x, sum = x;
  for (int k = 1; k <= 12; ++k) {
    term *= -x2 / double((2 * k) * (2 * k + 1));
    sum += term;
  }
  return sum;
}
constexpr double poly_cos(double x) {
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int k = 1; k <= 12; ++k) {
    term *= -x2 / double((2 * k - 1) * (2 * k));
    sum += term;
  }
  return sum;
}
// c = cos(2 pi a / den), s = sin(2 pi a / den)
constexpr void cos_sin(long a, long den, double& c, double& s) {
  a %= den;
  if (a < 0) a += den;
  const long q = (8 * a) / den, r = 8 * a - q * den;
  const double phi = kPi4 * double(r) / double(den);          // angle past the octant start
  const double psi = kPi4 * double(den - r) / double(den);    // pi/4 - phi
  const double sp = poly_sin(phi), cp = poly_cos(phi), sq = poly_sin(psi), cq = poly_cos(psi);
  switch (q) {
    case 0: c = cp; s = sp; break;
    case 1: c = sq; s = cq; break;
    case 2: c = -sp; s = cp; break;
    case 3: c = -cq; s = sq; break;
    case 4: c = -cp; s = -sp; break;
    case 5: c = -sq; s = -cq; break;
    case 6: c = sp; s = -cp; break;
    default: c = cq; s = -sq; break;
  }
}
constexpr double cos2pi(long a, long den) {
  double c = 0, s = 0;
  cos_sin(a, den, c, s);
  return c;
}
constexpr double sin2pi(long a, long den) {
  double c = 0, s = 0;
  cos_sin(a, den, c, s);
  return s;
}
}  // namespace cx

template <int R, typename C> __device__ __forceinline__ void dft(C* v);

// v *= W_R^m = exp(-2 pi i m / R), exact for multiples of a quarter turn
template <int R, int M, typename C> __device__ __forceinline__ C twiddle_const(C a) {
  constexpr int m = M % R;
  if constexpr (m == 0) {
    return a;
  } else if constexpr ((4 * m) % R == 0) {
    constexpr int q = (4 * m) / R;  // quarter turns: W = (-i)^q
    if constexpr (q == 1) return cmul_mi(a);
    else if constexpr (q == 2) return cmake<C>(-a.x, -a.y);
    else return cmake<C>(-a.y, a.x);
  } else {
    return cmulc(a, cx::cos2pi(m, R), -cx::sin2pi(m, R));
  }
}

// Composite radix R = R1 * R2 (Cooley-Tukey inside the registers): inputs
// j = R2*j1 + j2, outputs k = k1 + R1*k2; DFT_R1 over j1 for every j2,
// twiddle W_R^(j2*k1), DFT_R2 over j2 for every k1.
template <int R1, int R2, int J2, int K1, typename C>
__device__ __forceinline__ void comp_tw(const C* t, C* y) {
  if constexpr (K1 < R1) {
    y[K1 * R2 + J2] = twiddle_const<R1 * R2, J2 * K1>(t[K1]);
    comp_tw<R1, R2, J2, K1 + 1>(t, y);
  }
}
template <int R1, int R2, int J2 = 0, typename C>
__device__ __forceinline__ void comp_first(const C* v, C* y) {
  if constexpr (J2 < R2) {
    C t[R1];
#pragma unroll
    for (int j1 = 0; j1 < R1; ++j1) t[j1] = v[R2 * j1 + J2];
    dft<R1>(t);
    y[J2] = t[0];
    comp_tw<R1, R2, J2, 1>(t, y);
    comp_first<R1, R2, J2 + 1>(v, y);
  }
}
template <int R1, int R2, typename C> __device__ __forceinline__ void dft_comp(C* v) {
  C y[R1 * R2];
  comp_first<R1, R2>(v, y);
#pragma unroll
  for (int k1 = 0; k1 < R1; ++k1) {
    C t[R2];
#pragma unroll
    for (int j2 = 0; j2 < R2; ++j2) t[j2] = y[k1 * R2 + j2];
    dft<R2>(t);
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) v[k1 + R1 * k2] = t[k2];
  }
}

template <int R, typename C> __device__ __forceinline__ void dft(C* v) {
  if constexpr (R == 2) dft2(v);
  else if constexpr (R == 4) dft4(v);
  else if constexpr (R == 8) dft8(v);
  else if constexpr (R == 16) dft16(v);
  else if constexpr (R == 6) dft_comp<2, 3>(v);
  else if constexpr (R == 9) dft_comp<3, 3>(v);
  else if constexpr (R == 10) dft_comp<2, 5>(v);
  else if constexpr (R == 12) dft_comp<4, 3>(v);
  else if constexpr (R == 14) dft_comp<2, 7>(v);
  else if constexpr (R == 15) dft_comp<3, 5>(v);
  else dft_odd<R>(v);
}

// L2 eviction-priority hints for streaming loads and for stores a later pass
// reads back.
__device__ __forceinline__ uint64_t l2_policy_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_policy_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ float2 ld_l2hint(const float2* a, uint64_t pol) {
  float2 v;
  asm volatile("ld.global.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ double2 ld_l2hint(const double2* a, uint64_t pol) {
  double2 v;
  asm volatile("ld.global.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(v.x), "=d"(v.y) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ void st_l2hint(float2* a, float2 v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(a), "f"(v.x), "f"(v.y), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void st_l2hint(double2* a, double2 v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v2.f64 [%0], {%1, %2}, %3;" ::"l"(a), "d"(v.x), "d"(v.y), "l"(pol)
               : "memory");
}

}  // namespace gbfft
