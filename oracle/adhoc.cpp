// Oracle: CPU restatement of accelerate-fft's pure-Accelerate transform.
//
// TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
// cpu_baseline / reference legs of bench.py may load this library, and only as
// the checker or the timed CPU baseline.  The product path (libgbfft) never
// links, loads or calls it.
//
// Parity status: UNPINNED for values.  The reference ships no golden vectors
// and cannot be built here (no GHC / Accelerate / FFTW).  This restatement is
// pinned to the reference's property tests (test/Test/FFT.hs:112-236), to
// analytic known answers, and cross-checked against an independent FP64 FFT
// (numpy.fft) and the naive FP64 DFT below.
//
// What is restated (paths relative to the accelerate-fft source tree):
//   Adhoc.fft dispatch ................ src/Data/Array/Accelerate/Math/FFT/Adhoc.hs:37-66
//   ditSplitRadixLoop ................. Adhoc.hs:81-132
//   dit235 (+ twiddles, caches) ....... Adhoc.hs:140-233
//   transformChirp235 / transformChirp  Adhoc.hs:238-286
//   ceiling5Smooth .................... Adhoc.hs:289-313
//   transform2/3/4/5, sumAndConvolve .. Adhoc.hs:440-605
//   sieve/sieveV/twist/merge .......... Adhoc.hs:150-157, 368-406
//   fft / fft1D / fft2D / fft3D ....... src/Data/Array/Accelerate/Math/FFT.hs:63-187
//   signOfMode ........................ src/Data/Array/Accelerate/Math/FFT/Mode.hs:21-26
//   dftG + rootsOfUnity (naive DFT) ... src/Data/Array/Accelerate/Math/DFT.hs:68-92,
//                                       src/Data/Array/Accelerate/Math/DFT/Roots.hs:26-51
//
// Two deliberate departures, both in Bluestein (each is a defect in the
// reference; the restatement computes what the code evidently intends):
//   * Adhoc.hs:292 computes `pow i2 2 * pow i3 3 * pow i5 5`, and `pow x k` is
//     x^k (Adhoc.hs:318-323), so the padded length comes out as
//     i2^2 * i3^3 * i5^5 (0 for n = 1009).  Restated as 2^i2 * 3^i3 * 5^i5.
//   * Adhoc.hs:273 `pad p 0` appends p zeros (Adhoc.hs:325-334) and the
//     following reshape to p columns only lines up for a single row.
//     Restated as zero-padding each row to length p.
//
// Arithmetic follows the reference's expression trees (complex multiply as
// (ac-bd) :+ (ad+bc); angles formed in element precision in the same order of
// operations).  Compile with -ffp-contract=off so no FMA contraction changes
// the rounding.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>

namespace oracle {

template <typename T>
struct Cx {
  T re, im;
};

template <typename T> static inline Cx<T> add(Cx<T> a, Cx<T> b) { return {a.re + b.re, a.im + b.im}; }
template <typename T> static inline Cx<T> sub(Cx<T> a, Cx<T> b) { return {a.re - b.re, a.im - b.im}; }
template <typename T> static inline Cx<T> mul(Cx<T> a, Cx<T> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename T> static inline Cx<T> conj(Cx<T> a) { return {a.re, -a.im}; }

// Haskell's Data.Complex division (scaled), which Accelerate's Complex
// Fractional instance mirrors; used for the Inverse normalisation
// `A.map (/scale)` in FFT.hs:83,110,141,172.
template <typename T> static inline Cx<T> cdiv(Cx<T> z, Cx<T> w) {
  int ex = 0, ey = 0;
  std::frexp(w.re, &ex);
  std::frexp(w.im, &ey);
  if (w.re == T(0)) ex = INT32_MIN / 2;
  if (w.im == T(0)) ey = INT32_MIN / 2;
  int k = -std::max(ex, ey);
  T x2 = std::ldexp(w.re, k), y2 = std::ldexp(w.im, k);
  T d = w.re * x2 + w.im * y2;
  return {(z.re * x2 + z.im * y2) / d, (z.im * x2 - z.re * y2) / d};
}

// ---------------------------------------------------------------------------
// A row-major matrix of complex values: the (sh:.Int:.Int) arrays of Adhoc.hs
// for a single leading index `sh` (every Adhoc operation is independent per
// leading index, so batches are handled by running row by row).
template <typename T>
struct Mat {
  int64_t rows = 0, cols = 0;
  std::vector<Cx<T>> a;
  Mat() = default;
  Mat(int64_t r, int64_t c) : rows(r), cols(c), a(static_cast<size_t>(r * c)) {}
  Cx<T>& at(int64_t r, int64_t c) { return a[size_t(r * cols + c)]; }
  const Cx<T>& at(int64_t r, int64_t c) const { return a[size_t(r * cols + c)]; }
};

// sieve fac start (Adhoc.hs:368-380): every fac-th column from `start`.
template <typename T>
static Mat<T> sieve(int64_t fac, int64_t start, const Mat<T>& x) {
  Mat<T> y(x.rows, x.cols / fac);
  for (int64_t r = 0; r < y.rows; ++r)
    for (int64_t j = 0; j < y.cols; ++j) y.at(r, j) = x.at(r, fac * j + start);
  return y;
}

// sieveV fac start (Adhoc.hs:382-394): every fac-th row from `start`.
template <typename T>
static Mat<T> sieveV(int64_t fac, int64_t start, const Mat<T>& x) {
  Mat<T> y(x.rows / fac, x.cols);
  for (int64_t j = 0; j < y.rows; ++j)
    for (int64_t i = 0; i < y.cols; ++i) y.at(j, i) = x.at(fac * j + start, i);
  return y;
}

// twist fac (Adhoc.hs:396-406): (m, n) -> (fac*m, n/fac),
// new(j, i) = old(j / fac, fac*i + j mod fac).
template <typename T>
static Mat<T> twist(int64_t fac, const Mat<T>& x) {
  Mat<T> y(fac * x.rows, x.cols / fac);
  for (int64_t j = 0; j < y.rows; ++j)
    for (int64_t i = 0; i < y.cols; ++i) y.at(j, i) = x.at(j / fac, fac * i + j % fac);
  return y;
}

// (++^) = concatOn _2: stack rows.
template <typename T>
static Mat<T> vcat(const Mat<T>& x, const Mat<T>& y) {
  int64_t c = std::min(x.cols, y.cols);
  Mat<T> z(x.rows + y.rows, c);
  for (int64_t r = 0; r < x.rows; ++r)
    for (int64_t i = 0; i < c; ++i) z.at(r, i) = x.at(r, i);
  for (int64_t r = 0; r < y.rows; ++r)
    for (int64_t i = 0; i < c; ++i) z.at(x.rows + r, i) = y.at(r, i);
  return z;
}

// Accelerate (++): append along the innermost dimension; the outer extent is
// the intersection.
template <typename T>
static Mat<T> hcat(const Mat<T>& x, const Mat<T>& y) {
  int64_t r = std::min(x.rows, y.rows);
  Mat<T> z(r, x.cols + y.cols);
  for (int64_t j = 0; j < r; ++j) {
    for (int64_t i = 0; i < x.cols; ++i) z.at(j, i) = x.at(j, i);
    for (int64_t i = 0; i < y.cols; ++i) z.at(j, x.cols + i) = y.at(j, i);
  }
  return z;
}

// Accelerate zipWith: elementwise over the intersection of the two shapes.
template <typename T, typename F>
static Mat<T> zipWith(F f, const Mat<T>& x, const Mat<T>& y) {
  Mat<T> z(std::min(x.rows, y.rows), std::min(x.cols, y.cols));
  for (int64_t r = 0; r < z.rows; ++r)
    for (int64_t i = 0; i < z.cols; ++i) z.at(r, i) = f(x.at(r, i), y.at(r, i));
  return z;
}

// dropV n (Adhoc.hs:362-366): drop the first n rows.
template <typename T>
static Mat<T> dropV(int64_t n, const Mat<T>& x) {
  int64_t r = std::max<int64_t>(0, x.rows - n);
  Mat<T> y(r, x.cols);
  std::copy(x.a.begin() + size_t(std::min(n, x.rows) * x.cols), x.a.end(), y.a.begin());
  return y;
}

// transform2 v (Adhoc.hs:440-453).
template <typename T>
static Mat<T> transform2(Cx<T> v, const Mat<T>& x) {
  Mat<T> y(x.rows, 2);
  for (int64_t r = 0; r < x.rows; ++r) {
    Cx<T> x0 = x.at(r, 0), x1 = x.at(r, 1);
    y.at(r, 0) = add(x0, x1);
    y.at(r, 1) = add(x0, mul(v, x1));
  }
  return y;
}

template <typename T> static inline T pi_e() { return T(3.14159265358979323846264338327950288); }

// ---------------------------------------------------------------------------
// ditSplitRadixLoop (Adhoc.hs:81-132), one vector of power-of-two length.
template <typename T>
static std::vector<Cx<T>> split_radix(T sign, const Cx<T>* x, int64_t n) {
  // twiddleSR n4 k j = cos w :+ sign * sin w,  w = pi * k * j / (2*n4)
  auto twiddle = [&](int64_t len4, T k) {
    std::vector<Cx<T>> t(static_cast<size_t>(len4));
    for (int64_t j = 0; j < len4; ++j) {
      T w = ((pi_e<T>() * k) * T(j)) / (T(2) * T(len4));
      t[size_t(j)] = {std::cos(w), sign * std::sin(w)};
    }
    return t;
  };
  // initial: (reshape (sh:.1:.n) arr, fill (sh:.0:.n/2) 0)
  Mat<T> xs(1, n), ys(0, n / 2);
  std::copy(x, x + n, xs.a.begin());
  // reorder loop: while innermost extent of ys > 1
  while (ys.cols > 1) {
    Mat<T> evens = sieve<T>(2, 0, xs), odds = sieve<T>(2, 1, xs);
    Mat<T> nx = vcat(evens, ys);
    ys = twist<T>(2, odds);
    xs = std::move(nx);
  }
  // rebase
  xs = transform2<T>(Cx<T>{T(-1), T(0)}, xs);
  // step loop: while ys has rows
  const Cx<T> im{T(0), sign};
  while (ys.rows > 0) {
    const Mat<T>& us = xs;
    const Mat<T>& zs = ys;
    int64_t k = zs.cols;
    std::vector<Cx<T>> tw1 = twiddle(k, T(1)), tw3 = twiddle(k, T(3));
    Mat<T> ze = sieveV<T>(2, 0, zs), zo = sieveV<T>(2, 1, zs);
    for (int64_t r = 0; r < ze.rows; ++r)
      for (int64_t j = 0; j < k; ++j) ze.at(r, j) = mul(tw1[size_t(j)], ze.at(r, j));
    for (int64_t r = 0; r < zo.rows; ++r)
      for (int64_t j = 0; j < k; ++j) zo.at(r, j) = mul(tw3[size_t(j)], zo.at(r, j));
    Mat<T> zsum = zipWith<T>([](Cx<T> a, Cx<T> b) { return add(a, b); }, ze, zo);
    Mat<T> zdiff = zipWith<T>([&](Cx<T> a, Cx<T> b) { return mul(im, sub(a, b)); }, ze, zo);
    Mat<T> zc = hcat(zsum, zdiff);
    int64_t nrows = zc.rows;
    Mat<T> lo = zipWith<T>([](Cx<T> a, Cx<T> b) { return add(a, b); }, us, zc);
    Mat<T> hi = zipWith<T>([](Cx<T> a, Cx<T> b) { return sub(a, b); }, us, zc);
    Mat<T> nus = hcat(lo, hi);
    Mat<T> nzs = dropV(nrows, us);
    xs = std::move(nus);
    ys = std::move(nzs);
  }
  return std::vector<Cx<T>>(xs.a.begin(), xs.a.begin() + n);
}

// ---------------------------------------------------------------------------
// dit235 (Adhoc.hs:140-233), one vector of 5-smooth length.
template <typename T>
static std::vector<Cx<T>> dit235(T sign, const Cx<T>* x, int64_t n) {
  // cisrat d n = cos w :+ sign * sin w,  w = 2*pi * n / d   (Adhoc.hs:184-187)
  auto cisrat = [&](int64_t d, int64_t m) {
    T w = ((T(2) * pi_e<T>()) * T(m)) / T(d);
    return Cx<T>{std::cos(w), sign * std::sin(w)};
  };
  // caches (Adhoc.hs:192-212)
  const Cx<T> cache2{T(-1), T(0)};
  const T sqrt3d2 = std::sqrt(T(3)) / T(2), mhalf = T(-1) / T(2), u = sign * sqrt3d2;
  const Cx<T> c3a{mhalf, u}, c3b{mhalf, -u};
  const Cx<T> c4a{T(0), sign}, c4b{T(-1), -T(0)}, c4c{T(0), -sign};
  const Cx<T> c5[4] = {cisrat(5, 1), cisrat(5, 2), cisrat(5, 3), cisrat(5, 4)};

  Mat<T> xs(1, n);
  std::copy(x, x + n, xs.a.begin());
  // factor discovery loop (Adhoc.hs:222-232): factors are consed, so they are
  // applied in reverse discovery order.
  std::vector<int64_t> fs;
  while (xs.cols > 1) {
    int64_t len = xs.cols;
    int64_t f = (len % 3 == 0) ? 3 : (len % 4 == 0) ? 4 : (len % 5 == 0) ? 5 : 2;
    xs = twist<T>(f, xs);
    fs.insert(fs.begin(), f);
  }
  for (int64_t fac : fs) {
    // step fac xs (Adhoc.hs:159-170)
    int64_t count = xs.rows, len = xs.cols, groups = count / fac;
    Mat<T> out(groups, fac * len);
    std::vector<Cx<T>> v(static_cast<size_t>(fac)), r(static_cast<size_t>(fac));
    for (int64_t c = 0; c < groups; ++c) {
      for (int64_t i = 0; i < len; ++i) {
        // twiddled (after the transpose): element (c, i, j) = tw(fac*len, j, i) * x(c*fac+j, i)
        for (int64_t j = 0; j < fac; ++j)
          v[size_t(j)] = mul(cisrat(fac * len, (j * i) % (fac * len)), xs.at(c * fac + j, i));
        if (fac == 5) {
          // transform5 (Adhoc.hs:517-539) with sumAndConvolve4 (Adhoc.hs:578-605)
          const Cx<T> x0 = v[0], x1 = v[1], x2 = v[2], x3 = v[3], x4 = v[4];
          const Cx<T> a0 = x1, a1 = x3, a2 = x4, a3 = x2;
          const Cx<T> b0 = c5[0], b1 = c5[1], b2 = c5[3], b3 = c5[2];
          Cx<T> ab0 = mul(a0, b0), ab1 = mul(a1, b1);
          Cx<T> sa01 = add(a0, a1), sb01 = add(b0, b1);
          Cx<T> ab01 = sub(mul(sa01, sb01), add(ab0, ab1));
          Cx<T> ab2 = mul(a2, b2), ab3 = mul(a3, b3);
          Cx<T> sa23 = add(a2, a3), sb23 = add(b2, b3);
          Cx<T> ab23 = sub(mul(sa23, sb23), add(ab2, ab3));
          Cx<T> c0 = sub(add(ab0, ab2), add(ab1, ab3));
          Cx<T> c1 = add(ab01, ab23);
          Cx<T> ab02 = mul(add(a0, a2), add(b0, b2));
          Cx<T> ab13 = mul(add(a1, a3), add(b1, b3));
          Cx<T> sa0123 = add(sa01, sa23), sb0123 = add(sb01, sb23);
          Cx<T> ab0123 = sub(mul(sa0123, sb0123), add(ab02, ab13));
          Cx<T> d0 = add(ab13, c0), d1 = c1, d2 = sub(ab02, c0), d3 = sub(ab0123, c1);
          // ((s,_), (d1,d2,d4,d3)) = sumAndConvolve4 ...
          r[0] = add(x0, sa0123);
          r[1] = add(x0, d0);
          r[2] = add(x0, d1);
          r[3] = add(x0, d3);
          r[4] = add(x0, d2);
        } else if (fac == 4) {
          // transform4 (Adhoc.hs:475-498)
          const Cx<T> x0 = v[0], x1 = v[1], x2 = v[2], x3 = v[3];
          Cx<T> x02a = add(x0, x2), x02b = add(x0, mul(c4b, x2));
          Cx<T> x13a = add(x1, x3), x13b = add(x1, mul(c4b, x3));
          r[0] = add(x02a, x13a);
          r[1] = add(x02b, mul(c4a, x13b));
          r[2] = add(x02a, mul(c4b, x13a));
          r[3] = add(x02b, mul(c4c, x13b));
        } else if (fac == 3) {
          // transform3 (Adhoc.hs:455-473) with sumAndConvolve2 (Adhoc.hs:547-557)
          const Cx<T> x0 = v[0], x1 = v[1], x2 = v[2];
          Cx<T> sa01 = add(x1, x2), sb01 = add(c3a, c3b);
          Cx<T> ab0ab1 = add(mul(x1, c3a), mul(x2, c3b));
          Cx<T> zx2 = sub(mul(sa01, sb01), ab0ab1);
          r[0] = add(x0, sa01);
          r[1] = add(x0, ab0ab1);
          r[2] = add(x0, zx2);
        } else {
          // transform2 cache2 (Adhoc.hs:440-453)
          r[0] = add(v[0], v[1]);
          r[1] = add(v[0], mul(cache2, v[1]));
        }
        // merge (Adhoc.hs:147-157): out(c, q*len + i) = r(q)
        for (int64_t q = 0; q < fac; ++q) out.at(c, q * len + i) = r[size_t(q)];
      }
    }
    xs = std::move(out);
  }
  return std::vector<Cx<T>>(xs.a.begin(), xs.a.begin() + n);
}

// ---------------------------------------------------------------------------
// ceiling5Smooth (Adhoc.hs:289-313): a floating-point search over 3^i3 * 5^i5
// with the power of two from ceiling (logBase 2 (n / p53)).  The exponent
// triple is combined as 2^i2 * 3^i3 * 5^i5 (see the header on Adhoc.hs:292).
static inline double logBase(double b, double x) { return std::log(x) / std::log(b); }

static int64_t ceiling5_smooth(int64_t n_int) {
  const double n = double(n_int);
  const int64_t d3 = int64_t(std::ceil(logBase(3.0, n)));
  const int64_t d5 = int64_t(std::ceil(logBase(5.0, n)));
  double best = 0;
  int64_t bi2 = 0, bi3 = 0, bi5 = 0;
  bool have = false;
  for (int64_t i5 = 0; i5 < d5; ++i5)
    for (int64_t i3 = 0; i3 < d3; ++i3) {
      double p53 = std::pow(5.0, double(i5)) * std::pow(3.0, double(i3));
      int64_t i2 = std::max<int64_t>(0, int64_t(std::ceil(logBase(2.0, n / p53))));
      double v = p53 * std::pow(2.0, double(i2));
      if (!have || v < best) {
        best = v;
        bi2 = i2; bi3 = i3; bi5 = i5;
        have = true;
      }
    }
  if (!have) return 1;
  int64_t p = 1;
  for (int64_t i = 0; i < bi2; ++i) p *= 2;
  for (int64_t i = 0; i < bi3; ++i) p *= 3;
  for (int64_t i = 0; i < bi5; ++i) p *= 5;
  return p;
}

// transformChirp (Adhoc.hs:250-286) with p = ceiling5Smooth (2n).
template <typename T>
static std::vector<Cx<T>> bluestein(T sign, const Cx<T>* x, int64_t n) {
  const int64_t p = ceiling5_smooth(2 * n);
  std::vector<Cx<T>> chirp(static_cast<size_t>(p)), a(size_t(p), Cx<T>{T(0), T(0)}), b(static_cast<size_t>(p));
  for (int64_t k = 0; k < p; ++k) {
    int64_t sk_i = (p > 2 * k) ? k : k - p;
    T sk = T(sk_i);
    T w = ((pi_e<T>() * sk) * sk) / T(n);
    chirp[size_t(k)] = {std::cos(w), sign * std::sin(w)};
  }
  for (int64_t k = 0; k < n; ++k) a[size_t(k)] = mul(chirp[size_t(k)], x[k]);
  for (int64_t k = 0; k < p; ++k) b[size_t(k)] = conj(chirp[size_t(k)]);
  // analysis = dit235 Forward on both rows
  std::vector<Cx<T>> A = dit235<T>(T(-1), a.data(), p);
  std::vector<Cx<T>> B = dit235<T>(T(-1), b.data(), p);
  std::vector<Cx<T>> C(static_cast<size_t>(p));
  for (int64_t k = 0; k < p; ++k) C[size_t(k)] = mul(B[size_t(k)], A[size_t(k)]);
  // synthesis = dit235 Inverse (sign +1, unnormalised)
  std::vector<Cx<T>> D = dit235<T>(T(1), C.data(), p);
  const T s = T(1) / T(p);
  std::vector<Cx<T>> out(static_cast<size_t>(n));
  for (int64_t k = 0; k < n; ++k) {
    Cx<T> e = mul(chirp[size_t(k)], D[size_t(k)]);
    out[size_t(k)] = {s * e.re, s * e.im};
  }
  return out;
}

static inline bool is_pow2(int64_t n) { return n > 0 && (n & (n - 1)) == 0; }

static inline bool is_5smooth(int64_t n) {
  // is2or5smooth (Adhoc.hs:54-61)
  int64_t odd = n / (n & -n);
  while (odd % 3 == 0) odd /= 3;
  while (odd % 5 == 0) odd /= 5;
  return odd == 1;
}

// Adhoc.fft on one vector (Adhoc.hs:37-48).  mode: 0 Forward, 1 Reverse, 2 Inverse.
template <typename T>
static void adhoc_vec(int mode, const Cx<T>* x, Cx<T>* y, int64_t n) {
  const T sign = (mode == 0) ? T(-1) : T(1);  // signOfMode (Mode.hs:21-26)
  if (n <= 1) {
    for (int64_t i = 0; i < n; ++i) y[i] = x[i];
    return;
  }
  std::vector<Cx<T>> r;
  if (is_pow2(n)) r = split_radix<T>(sign, x, n);
  else if (is_5smooth(n)) r = dit235<T>(sign, x, n);
  else r = bluestein<T>(sign, x, n);
  std::copy(r.begin(), r.end(), y);
}

// Innermost-axis transform over `rows` contiguous rows of length n.
template <typename T>
static void adhoc_rows(int mode, const Cx<T>* x, Cx<T>* y, int64_t rows, int64_t n, int threads) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) if (threads > 1)
  for (int64_t r = 0; r < rows; ++r) adhoc_vec<T>(mode, x + r * n, y + r * n, n);
}

template <typename T>
static void scale_inverse(Cx<T>* y, int64_t total, int64_t by, int threads) {
  const Cx<T> s{T(by), T(0)};
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
  for (int64_t i = 0; i < total; ++i) y[i] = cdiv(y[i], s);
}

// A.transpose on a (h, w) matrix.
template <typename T>
static void transpose2(const Cx<T>* x, Cx<T>* y, int64_t h, int64_t w, int threads) {
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
  for (int64_t i = 0; i < w; ++i)
    for (int64_t j = 0; j < h; ++j) y[i * h + j] = x[j * w + i];
}

// rotate3D (FFT.hs:176-187): (z, y, x) -> (y, x, z), new(i0,i1,i2) = old(i2,i0,i1).
template <typename T>
static void rotate3(const Cx<T>* x, Cx<T>* y, int64_t d, int64_t h, int64_t w, int threads) {
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
  for (int64_t i0 = 0; i0 < h; ++i0)
    for (int64_t i1 = 0; i1 < w; ++i1)
      for (int64_t i2 = 0; i2 < d; ++i2) y[(i0 * w + i1) * d + i2] = x[(i2 * h + i0) * w + i1];
}

// kind: 0 = fft (innermost axis, any rank), 1 = fft1D, 2 = fft2D, 3 = fft3D.
template <typename T>
static int run(int mode, int kind, int rank, const int64_t* dims, const Cx<T>* x, Cx<T>* y, int threads) {
  if (rank < 1 || mode < 0 || mode > 2) return 1;
  int64_t total = 1;
  for (int i = 0; i < rank; ++i) {
    if (dims[i] < 0) return 1;
    total *= dims[i];
  }
  if (total == 0) return 0;
  const int64_t n = dims[rank - 1];
  if (kind == 0 || kind == 1) {
    if (kind == 1 && rank != 1) return 1;
    // FFT.hs:63-84 / 92-111: Adhoc on the innermost axis, divide by its length.
    adhoc_rows<T>(mode, x, y, total / n, n, threads);
    if (mode == 2) scale_inverse<T>(y, total, n, threads);
    return 0;
  }
  if (kind == 2) {
    if (rank != 2) return 1;
    // FFT.hs:136-137: A.transpose . Adhoc.fft >-> A.transpose . Adhoc.fft
    const int64_t h = dims[0], w = dims[1];
    std::vector<Cx<T>> t1(static_cast<size_t>(total)), t2(static_cast<size_t>(total));
    adhoc_rows<T>(mode, x, t1.data(), h, w, threads);
    transpose2<T>(t1.data(), t2.data(), h, w, threads);
    adhoc_rows<T>(mode, t2.data(), t1.data(), w, h, threads);
    transpose2<T>(t1.data(), y, w, h, threads);
    if (mode == 2) scale_inverse<T>(y, total, total, threads);
    return 0;
  }
  if (kind == 3) {
    if (rank != 3) return 1;
    // FFT.hs:166-169: (rotate3D . Adhoc.fft) three times.
    int64_t d = dims[0], h = dims[1], w = dims[2];
    std::vector<Cx<T>> t1(static_cast<size_t>(total)), t2(static_cast<size_t>(total));
    std::copy(x, x + total, t2.begin());
    for (int pass = 0; pass < 3; ++pass) {
      adhoc_rows<T>(mode, t2.data(), t1.data(), d * h, w, threads);
      rotate3<T>(t1.data(), t2.data(), d, h, w, threads);
      int64_t nd = h, nh = w, nw = d;  // rotate3D's new shape
      d = nd; h = nh; w = nw;
    }
    std::copy(t2.begin(), t2.end(), y);
    if (mode == 2) scale_inverse<T>(y, total, total, threads);
    return 0;
  }
  return 1;
}

// dftG with rootsOfUnity / inverseRootsOfUnity (DFT.hs:68-92, Roots.hs:26-51):
// out[k] = sum_i in[i] * roots[(k*i) mod n], roots[i] = cos t :+ (sign * sin t),
// t = 2*pi*i/n, summed left to right.
template <typename T>
static void dft_naive(int sign, const Cx<T>* x, Cx<T>* y, int64_t rows, int64_t n, int threads) {
  std::vector<Cx<T>> roots(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i) {
    T t = ((T(2) * pi_e<T>()) * T(i)) / T(n);
    roots[size_t(i)] = {std::cos(t), T(sign) * std::sin(t)};
  }
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) if (threads > 1)
  for (int64_t r = 0; r < rows; ++r) {
    const Cx<T>* xr = x + r * n;
    Cx<T>* yr = y + r * n;
    for (int64_t k = 0; k < n; ++k) {
      Cx<T> acc{T(0), T(0)};
      for (int64_t i = 0; i < n; ++i) acc = add(acc, mul(xr[i], roots[size_t((k * i) % n)]));
      yr[k] = acc;
    }
  }
}

// dftG as written (DFT.hs:68-92): the input is extended with one more axis of
// length shapeSize(base) and folded along it, so every output element
// (sh_o :. k) is the sum over ALL input elements i = (sh_i :. n_i) of
// arr[i] * roots[sh_i :. (k*n_i) mod l] -- for rank > 1 each output row holds
// the transform of the sum of the rows (each row with its own roots); for
// rank 1 it is the ordinary DFT.  Summed left to right in element order.
template <typename T>
static void dft_g(const Cx<T>* roots, const Cx<T>* x, Cx<T>* y, int64_t rows, int64_t l, int threads) {
  const int64_t N = rows * l;
  std::vector<Cx<T>> s(static_cast<size_t>(l));
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
  for (int64_t k = 0; k < l; ++k) {
    Cx<T> acc{T(0), T(0)};
    for (int64_t i = 0; i < N; ++i) {
      const int64_t r = i / l, n = i - r * l;
      acc = add(acc, mul(x[i], roots[r * l + (k * n) % l]));
    }
    s[size_t(k)] = acc;
  }
  for (int64_t r = 0; r < rows; ++r)
    for (int64_t k = 0; k < l; ++k) y[r * l + k] = s[size_t(k)];
}

// dftGS (DFT.hs:95-111): the single value sum over all (sh :. n) of
// arr[sh :. n] * roots[sh :. (k*n) mod l] (foldAll), k = indexHead ix.
template <typename T>
static Cx<T> dft_gs(int64_t k, const Cx<T>* roots, const Cx<T>* x, int64_t rows, int64_t l) {
  Cx<T> acc{T(0), T(0)};
  for (int64_t r = 0; r < rows; ++r)
    for (int64_t n = 0; n < l; ++n) acc = add(acc, mul(x[r * l + n], roots[r * l + (k * n) % l]));
  return acc;
}

}  // namespace oracle

extern "C" {

// dftG / dftGS over `rows` x `l` (rows = product of the outer extents).
int oracle_dftg_f32(int64_t rows, int64_t l, const float* roots, const float* in, float* out, int threads) {
  if (l <= 0 || rows < 0) return 1;
  oracle::dft_g<float>(reinterpret_cast<const oracle::Cx<float>*>(roots),
                       reinterpret_cast<const oracle::Cx<float>*>(in), reinterpret_cast<oracle::Cx<float>*>(out),
                       rows, l, threads);
  return 0;
}
int oracle_dftg_f64(int64_t rows, int64_t l, const double* roots, const double* in, double* out, int threads) {
  if (l <= 0 || rows < 0) return 1;
  oracle::dft_g<double>(reinterpret_cast<const oracle::Cx<double>*>(roots),
                        reinterpret_cast<const oracle::Cx<double>*>(in),
                        reinterpret_cast<oracle::Cx<double>*>(out), rows, l, threads);
  return 0;
}
int oracle_dftgs_f64(int64_t k, int64_t rows, int64_t l, const double* roots, const double* in, double* out) {
  if (l <= 0 || rows < 0 || k < 0) return 1;
  const auto v = oracle::dft_gs<double>(k, reinterpret_cast<const oracle::Cx<double>*>(roots),
                                        reinterpret_cast<const oracle::Cx<double>*>(in), rows, l);
  out[0] = v.re;
  out[1] = v.im;
  return 0;
}

// Status: 0 ok, 1 bad argument.  Buffers hold interleaved (re, im) pairs.
int oracle_fft_f32(int mode, int kind, int rank, const int64_t* dims, const float* in, float* out,
                   int threads) {
  return oracle::run<float>(mode, kind, rank, dims, reinterpret_cast<const oracle::Cx<float>*>(in),
                            reinterpret_cast<oracle::Cx<float>*>(out), threads);
}

int oracle_fft_f64(int mode, int kind, int rank, const int64_t* dims, const double* in, double* out,
                   int threads) {
  return oracle::run<double>(mode, kind, rank, dims, reinterpret_cast<const oracle::Cx<double>*>(in),
                             reinterpret_cast<oracle::Cx<double>*>(out), threads);
}

// Naive O(n^2) DFT along the innermost axis of `rows` rows, in FP64.
// sign: -1 forward roots, +1 inverse roots (unnormalised).
int oracle_dft_naive_f64(int sign, int64_t rows, int64_t n, const double* in, double* out, int threads) {
  if (n <= 0 || rows < 0 || (sign != 1 && sign != -1)) return 1;
  oracle::dft_naive<double>(sign, reinterpret_cast<const oracle::Cx<double>*>(in),
                            reinterpret_cast<oracle::Cx<double>*>(out), rows, n, threads);
  return 0;
}

int64_t oracle_ceiling5_smooth(int64_t n) { return oracle::ceiling5_smooth(n); }

}  // extern "C"
