// Common device types for the GB300 Bloch eigensolver.
//
// Data layout in HBM (all levels, all k-points of a batch):
//   edge block  [K][2][n][n][m]   plane 0 = x-edges, plane 1 = y-edges,
//                                 x-edge (i,j) at row j, column i; the m
//                                 vectors of one block are innermost so a
//                                 warp reads 2 sites x 16 vectors contiguously
//   node block  [K][n][n][m]
//   kappa       [n][n]            one copy per level, shared by all k
// Complex storage: c64 = float2, c128 = double2, cdd = float4 holding a
// float-float ("double-float") number per component: (re.hi, re.lo, im.hi, im.lo).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mx {

// ------------------------------------------------------------------
// float-float arithmetic.  Error-free transformations: Knuth's TwoSum,
// the FMA-based TwoProd, and the double-double add/multiply of Hida, Li and
// Bailey ("Algorithms for quad-double precision floating point arithmetic",
// ARITH 2001), written here for two floats.
// ------------------------------------------------------------------
struct dd {
  float hi, lo;
};

__host__ __device__ __forceinline__ dd dd_make(float h, float l) { dd r; r.hi = h; r.lo = l; return r; }

__device__ __forceinline__ dd two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return dd_make(s, e);
}
__device__ __forceinline__ dd quick_two_sum(float a, float b) {
  float s = a + b;
  float e = b - (s - a);
  return dd_make(s, e);
}
__device__ __forceinline__ dd two_prod(float a, float b) {
  float p = a * b;
  float e = fmaf(a, b, -p);
  return dd_make(p, e);
}
__device__ __forceinline__ dd operator+(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi);
  dd t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dd operator-(dd a) { return dd_make(-a.hi, -a.lo); }
__device__ __forceinline__ dd operator-(dd a, dd b) { return a + (-b); }
__device__ __forceinline__ dd operator*(dd a, dd b) {
  dd p = two_prod(a.hi, b.hi);
  p.lo = fmaf(a.hi, b.lo, p.lo);
  p.lo = fmaf(a.lo, b.hi, p.lo);
  return quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ dd operator*(dd a, float b) {
  dd p = two_prod(a.hi, b);
  p.lo = fmaf(a.lo, b, p.lo);
  return quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ dd operator*(float b, dd a) { return a * b; }
__device__ __forceinline__ dd operator+(dd a, float b) {
  dd s = two_sum(a.hi, b);
  s.lo += a.lo;
  return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dd& operator+=(dd& a, dd b) { a = a + b; return a; }
__device__ __forceinline__ dd& operator-=(dd& a, dd b) { a = a - b; return a; }
__device__ __forceinline__ dd operator/(dd a, dd b) {
  // one Newton correction of the float quotient
  float q1 = a.hi / b.hi;
  dd r = a - b * q1;
  float q2 = r.hi / b.hi;
  return quick_two_sum(q1, q2);
}
__device__ __forceinline__ dd dd_from_double(double d) {
  float h = (float) d;
  float l = (float) (d - (double) h);
  return dd_make(h, l);
}
__host__ __device__ __forceinline__ double dd_to_double(dd a) { return (double) a.hi + (double) a.lo; }

// ------------------------------------------------------------------
// Scalar traits: R is the arithmetic type (float, double or dd).
// ------------------------------------------------------------------
template <typename R> struct Real;
template <> struct Real<float> {
  __device__ static float from_float(float f) { return f; }
  __device__ static float from(double d) { return (float) d; }
  __device__ static double to_double(float f) { return (double) f; }
  __device__ static float zero() { return 0.0f; }
};
template <> struct Real<double> {
  __device__ static double from_float(float f) { return (double) f; }
  __device__ static double from(double d) { return d; }
  __device__ static double to_double(double f) { return f; }
  __device__ static double zero() { return 0.0; }
};
template <> struct Real<dd> {
  __device__ static dd from_float(float f) { return dd_make(f, 0.0f); }
  __device__ static dd from(double d) { return dd_from_double(d); }
  __device__ static double to_double(dd f) { return dd_to_double(f); }
  __device__ static dd zero() { return dd_make(0.0f, 0.0f); }
};

template <typename R> struct cx {
  R re, im;
};
template <typename R> __device__ __forceinline__ cx<R> mkc(R a, R b) { cx<R> r; r.re = a; r.im = b; return r; }
template <typename R> __device__ __forceinline__ cx<R> operator+(cx<R> a, cx<R> b) { return mkc(a.re + b.re, a.im + b.im); }
template <typename R> __device__ __forceinline__ cx<R> operator-(cx<R> a, cx<R> b) { return mkc(a.re - b.re, a.im - b.im); }
template <typename R> __device__ __forceinline__ cx<R> operator-(cx<R> a) { return mkc(-a.re, -a.im); }
template <typename R> __device__ __forceinline__ cx<R> operator*(cx<R> a, cx<R> b) {
  return mkc(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename R, typename S> __device__ __forceinline__ cx<R> scal(S s, cx<R> a) { return mkc(a.re * s, a.im * s); }
template <typename R> __device__ __forceinline__ cx<R>& operator+=(cx<R>& a, cx<R> b) { a = a + b; return a; }
template <typename R> __device__ __forceinline__ cx<R>& operator-=(cx<R>& a, cx<R> b) { a = a - b; return a; }
template <typename R> __device__ __forceinline__ cx<R> conjc(cx<R> a) { return mkc(a.re, -a.im); }
template <typename R> __device__ __forceinline__ cx<R> czero() { return mkc(Real<R>::zero(), Real<R>::zero()); }
template <typename R> __device__ __forceinline__ cx<R> cfrom(double re, double im) {
  return mkc(Real<R>::from(re), Real<R>::from(im));
}
// exactly representable literal constants (no double arithmetic at run time)
template <typename R> __device__ __forceinline__ R rc(float f) { return Real<R>::from_float(f); }

// ------------------------------------------------------------------
// Scalars prepared on the host in all three arithmetics.  GB300 issues FP64
// instructions at a small fraction of its FP32 rate, so the FP32 and
// float-float kernels never compute or convert a constant in double: every
// run-time scalar arrives as (double, float hi, float lo).
// ------------------------------------------------------------------
struct Sc {
  double d;
  float hi, lo;
};
inline Sc make_sc(double d) {
  Sc s;
  s.d = d;
  s.hi = (float) d;
  s.lo = (float) (d - (double) s.hi);
  return s;
}
template <typename R> struct ScGet;
template <> struct ScGet<float> { __device__ static float get(const Sc& s) { return s.hi; } };
template <> struct ScGet<double> { __device__ static double get(const Sc& s) { return s.d; } };
template <> struct ScGet<dd> { __device__ static dd get(const Sc& s) { return dd_make(s.hi, s.lo); } };
template <typename R> __device__ __forceinline__ R sget(const Sc& s) { return ScGet<R>::get(s); }

// a real number stored as a float-float pair (hi, lo) read in arithmetic R
template <typename R> struct PairGet;
template <> struct PairGet<float> { __device__ static float get(const float* p) { return p[0]; } };
template <> struct PairGet<dd> { __device__ static dd get(const float* p) { return dd_make(p[0], p[1]); } };

// ------------------------------------------------------------------
// Storage <-> arithmetic conversions
// ------------------------------------------------------------------
struct cdd {
  float rh, rl, ih, il;
};

template <typename S, typename R> struct Store;
template <> struct Store<float2, float> {
  __device__ static cx<float> ld(const float2* p) { float2 v = *p; return mkc(v.x, v.y); }
  __device__ static void st(float2* p, cx<float> a) { *p = make_float2(a.re, a.im); }
};
template <> struct Store<double2, double> {
  __device__ static cx<double> ld(const double2* p) { double2 v = *p; return mkc(v.x, v.y); }
  __device__ static void st(double2* p, cx<double> a) { *p = make_double2(a.re, a.im); }
};
template <> struct Store<cdd, dd> {
  __device__ static cx<dd> ld(const cdd* p) {
    float4 v = *reinterpret_cast<const float4*>(p);
    return mkc(dd_make(v.x, v.y), dd_make(v.z, v.w));
  }
  __device__ static void st(cdd* p, cx<dd> a) {
    *reinterpret_cast<float4*>(p) = make_float4(a.re.hi, a.re.lo, a.im.hi, a.im.lo);
  }
};
// mixed reads: a c64 value promoted into dd arithmetic, a dd value rounded to float
template <> struct Store<float2, dd> {
  __device__ static cx<dd> ld(const float2* p) { float2 v = *p; return mkc(dd_make(v.x, 0.f), dd_make(v.y, 0.f)); }
  __device__ static void st(float2* p, cx<dd> a) { *p = make_float2(a.re.hi + a.re.lo, a.im.hi + a.im.lo); }
};
template <> struct Store<cdd, float> {
  __device__ static cx<float> ld(const cdd* p) {
    float4 v = *reinterpret_cast<const float4*>(p);
    return mkc(v.x + v.y, v.z + v.w);
  }
  __device__ static void st(cdd* p, cx<float> a) {
    *reinterpret_cast<float4*>(p) = make_float4(a.re, 0.f, a.im, 0.f);
  }
};
template <> struct Store<double2, float> {
  __device__ static cx<float> ld(const double2* p) { double2 v = *p; return mkc((float) v.x, (float) v.y); }
  __device__ static void st(double2* p, cx<float> a) { *p = make_double2(a.re, a.im); }
};
template <> struct Store<double2, dd> {
  __device__ static cx<dd> ld(const double2* p) { double2 v = *p; return mkc(dd_from_double(v.x), dd_from_double(v.y)); }
  __device__ static void st(double2* p, cx<dd> a) { *p = make_double2(dd_to_double(a.re), dd_to_double(a.im)); }
};
template <> struct Store<cdd, double> {
  __device__ static cx<double> ld(const cdd* p) {
    float4 v = *reinterpret_cast<const float4*>(p);
    return mkc((double) v.x + (double) v.y, (double) v.z + (double) v.w);
  }
  __device__ static void st(cdd* p, cx<double> a) {
    dd r = dd_from_double(a.re), i = dd_from_double(a.im);
    *reinterpret_cast<float4*>(p) = make_float4(r.hi, r.lo, i.hi, i.lo);
  }
};
template <> struct Store<float2, double> {
  __device__ static cx<double> ld(const float2* p) { float2 v = *p; return mkc((double) v.x, (double) v.y); }
  __device__ static void st(float2* p, cx<double> a) { *p = make_float2((float) a.re, (float) a.im); }
};

// ------------------------------------------------------------------
// Batched layout and Bloch seams
// ------------------------------------------------------------------
struct Lay {
  int n;   // intervals per side on this level
  int m;   // vectors per k-point
  int K;   // k-points in the batch
  __host__ __device__ size_t edge(int k, int p, int j, int i, int v) const {
    return ((((size_t) k * 2 + p) * n + j) * n + i) * m + v;
  }
  __host__ __device__ size_t node(int k, int j, int i, int v) const {
    return (((size_t) k * n + j) * n + i) * m + v;
  }
  __host__ __device__ size_t edge_len() const { return (size_t) K * 2 * n * n * m; }
  __host__ __device__ size_t node_len() const { return (size_t) K * n * n * m; }
};

// Phase of a site addressed one period outside [0,n)^2: xf^a yf^b with the
// conjugate factor for a = -1 or b = -1 (edge2d.c:1335-1650, node2d.c:516-627).
template <typename R>
struct Seam {
  cx<R> xf, yf;     // e^{i kx}, e^{i ky}
  int n;
  // wrap (i,j) in place; returns the phase to multiply a fetched value by
  __device__ __forceinline__ bool wrap(int& i, int& j, cx<R>& ph) const {
    bool moved = false;
    cx<R> p = mkc(rc<R>(1.0f), Real<R>::zero());
    if (i < 0) { i += n; p = p * conjc(xf); moved = true; }
    else if (i >= n) { i -= n; p = p * xf; moved = true; }
    if (j < 0) { j += n; p = p * conjc(yf); moved = true; }
    else if (j >= n) { j -= n; p = p * yf; moved = true; }
    ph = p;
    return moved;
  }
};

__device__ __forceinline__ int wrapi(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// Phase table of K k-points on the device: 4K doubles (re xf, im xf, re yf,
// im yf of each k) followed by the same 4K numbers as 8K floats, each a
// float-float pair (hi, lo).  FP32 kernels read the hi parts, float-float
// kernels the pairs, FP64 kernels the doubles.
template <typename R> struct SeamLoad {
  __device__ static Seam<R> get(const double* ph, int K, int k, int n) {
    const float* pf = reinterpret_cast<const float*>(ph + 4 * (size_t) K) + 8 * k;
    Seam<R> s;
    s.xf = mkc(PairGet<R>::get(pf + 0), PairGet<R>::get(pf + 2));
    s.yf = mkc(PairGet<R>::get(pf + 4), PairGet<R>::get(pf + 6));
    s.n = n;
    return s;
  }
};
template <> struct SeamLoad<double> {
  __device__ static Seam<double> get(const double* ph, int K, int k, int n) {
    Seam<double> s;
    s.xf = mkc(ph[4 * k + 0], ph[4 * k + 1]);
    s.yf = mkc(ph[4 * k + 2], ph[4 * k + 3]);
    s.n = n;
    return s;
  }
};
template <typename R>
__device__ __forceinline__ Seam<R> seam_load(const double* ph, int K, int k, int n) {
  return SeamLoad<R>::get(ph, K, k, n);
}

// ------------------------------------------------------------------
// Block reductions
// ------------------------------------------------------------------
__device__ __forceinline__ float warp_sum(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ dd warp_sum(dd v) {
  for (int o = 16; o > 0; o >>= 1) {
    dd w;
    w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
    w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
    v = v + w;
  }
  return v;
}

}  // namespace mx

#define MX_CHECK_LAUNCH() do { cudaError_t e_ = cudaGetLastError(); if (e_ != cudaSuccess) return (int) e_; } while (0)
