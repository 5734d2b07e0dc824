// Matrix-free stencils of the Nedelec edge space and the Q1 node space,
// batched over k-points (grid.y / outer index) and block vectors (innermost).
//
// Operators follow the reference (sboerm/Maxwell):
//   edge operator alpha*A + beta*M      edge2d.c:1335-1650 (gather form, the
//                                       kappa of every cell as assembled by
//                                       densematrix_edge2d, edge2d.c:5870-6116)
//   AFW vertex-patch Gauss-Seidel       edge2d.c:2029-3042
//   edge prolongation / restriction     edge2d.c:5583-5705
//   Q1 Laplace, point Gauss-Seidel      node2d.c:516-1138
//   node prolongation / restriction     node2d.c:1140-1273
//   gradient and its adjoint            node2d.c:1275-1350
//   dense coarse matrices               edge2d.c:5870-6116, node2d.c:1429-1602
// On the unit square with h = 1/n: axy = alpha*n^2, mx = my = beta/6.
#include "mx_common.cuh"
#include "mx_internal.h"
#include "maxwell_gb300.h"

#include <atomic>

using namespace mx;

namespace {

constexpr int TPB = 256;

// launch geometry of the site kernels: block (m, 256/m), grid (sites/rows, K)
inline dim3 blk2(int m) { return dim3(m, 256 / m); }
inline dim3 grd2(size_t sites, int m, int K) {
  unsigned rows = 256 / m;
  return dim3((unsigned) ((sites + rows - 1) / rows), K);
}

inline unsigned nblocks(size_t work, int tpb = TPB) {
  size_t b = (work + tpb - 1) / tpb;
  return (unsigned) (b > 0x7fffffff ? 0x7fffffff : b);
}


// kappa of cell (i,j) with periodic wrap, in arithmetic R
template <typename R> struct Kap;
template <> struct Kap<float> {
  const float* p; int n;
  __device__ float at(int c) const { return p[c]; }
  __device__ float operator()(int i, int j) const { return p[wrapi(i, n) + wrapi(j, n) * n]; }
};
template <> struct Kap<double> {
  const double* p; int n;
  __device__ double at(int c) const { return p[c]; }
  __device__ double operator()(int i, int j) const { return p[wrapi(i, n) + wrapi(j, n) * n]; }
};
template <> struct Kap<dd> {
  const float* p; int n;
  __device__ dd at(int c) const {
    float2 v = reinterpret_cast<const float2*>(p)[c];
    return dd_make(v.x, v.y);
  }
  __device__ dd operator()(int i, int j) const { return at(wrapi(i, n) + wrapi(j, n) * n); }
};
// kappa of a cell known to lie inside [0,n)^2: no wrap
template <typename R> struct KapI {
  Kap<R> k;
  __device__ __forceinline__ R operator()(int i, int j) const { return k.at(i + j * k.n); }
};
template <typename R> Kap<R> make_kap(mxk_kappa k, int n);
template <> Kap<float> make_kap<float>(mxk_kappa k, int n) { Kap<float> r; r.p = k.f; r.n = n; return r; }
template <> Kap<double> make_kap<double>(mxk_kappa k, int n) { Kap<double> r; r.p = k.d; r.n = n; return r; }
template <> Kap<dd> make_kap<dd>(mxk_kappa k, int n) { Kap<dd> r; r.p = k.dd; r.n = n; return r; }

// accessor of one (k, v) edge vector: E(p, i, j) with seam phases
template <typename S, typename R>
struct EAcc {
  const S* base;   // points at (k, plane 0, 0, 0, v)
  int n, m;
  Seam<R> seam;
  __device__ __forceinline__ cx<R> operator()(int p, int i, int j) const {
    cx<R> ph;
    bool w = seam.wrap(i, j, ph);
    cx<R> v = Store<S, R>::ld(base + ((size_t) (p * n + j) * n + i) * m);
    return w ? ph * v : v;
  }
};

template <typename S, typename R>
struct NAcc {
  const S* base;
  int n, m;
  Seam<R> seam;
  __device__ __forceinline__ cx<R> operator()(int i, int j) const {
    cx<R> ph;
    bool w = seam.wrap(i, j, ph);
    cx<R> v = Store<S, R>::ld(base + ((size_t) j * n + i) * m);
    return w ? ph * v : v;
  }
};

// The same two accessors for sites whose whole stencil lies inside the unit
// cell: no seam test and 32-bit offsets (2n^2 m < 2^31 for every level).  The
// site kernels take this path for all but the boundary rows and columns.
template <typename S, typename R>
struct EAccI {
  const S* base;
  int n, m;
  __device__ __forceinline__ cx<R> operator()(int p, int i, int j) const {
    return Store<S, R>::ld(base + ((p * n + j) * n + i) * m);
  }
};
template <typename S, typename R>
struct NAccI {
  const S* base;
  int n, m;
  __device__ __forceinline__ cx<R> operator()(int i, int j) const {
    return Store<S, R>::ld(base + (j * n + i) * m);
  }
};


// curl of cell (i,j): bottom - top - left + right
template <typename R, typename A>
__device__ __forceinline__ cx<R> curl(const A& E, int i, int j) {
  return E(0, i, j) - E(0, i, j + 1) - E(1, i, j) + E(1, i + 1, j);
}

// (alpha A + beta M) x at x-edge (i,j) and y-edge (i,j)
template <typename R, typename A, typename KA>
__device__ __forceinline__ cx<R> kx_x(const A& E, const KA& kap, R axy, R mm, int i, int j) {
  cx<R> c0 = E(0, i, j);
  cx<R> mass = scal(mm, scal(rc<R>(4.0f), c0) + E(0, i, j + 1) + E(0, i, j - 1));
  cx<R> cur = scal(kap(i, j), curl<R>(E, i, j)) - scal(kap(i, j - 1), curl<R>(E, i, j - 1));
  return scal(axy, cur) + mass;
}
template <typename R, typename A, typename KA>
__device__ __forceinline__ cx<R> kx_y(const A& E, const KA& kap, R axy, R mm, int i, int j) {
  cx<R> c0 = E(1, i, j);
  cx<R> mass = scal(mm, scal(rc<R>(4.0f), c0) + E(1, i + 1, j) + E(1, i - 1, j));
  cx<R> cur = scal(kap(i - 1, j), curl<R>(E, i - 1, j)) - scal(kap(i, j), curl<R>(E, i, j));
  return scal(axy, cur) + mass;
}
// mass only (no kappa)
template <typename R, typename A>
__device__ __forceinline__ cx<R> mx_x(const A& E, R mm, int i, int j) {
  return scal(mm, scal(rc<R>(4.0f), E(0, i, j)) + E(0, i, j + 1) + E(0, i, j - 1));
}
template <typename R, typename A>
__device__ __forceinline__ cx<R> mx_y(const A& E, R mm, int i, int j) {
  return scal(mm, scal(rc<R>(4.0f), E(1, i, j)) + E(1, i + 1, j) + E(1, i - 1, j));
}


// ------------------------------------------------------------------
// edge operator
// ------------------------------------------------------------------
// y = cy * (yin ? yin : y) + axy*A x + mm*M x; axy = alpha n^2, mm = beta/6
// (per (k, v) from beta_kv when given: that form converts in double and
// serves the shifted operator of the mirror API only)
template <typename SX, typename SY, typename R>
__global__ void k_edge_apply(int n, int m, int K, const double* __restrict__ ph, Kap<R> kap, Sc axy_s,
                             Sc mm_s, const double* __restrict__ beta_kv, Sc cy_s, int has_cy,
                             const SX* __restrict__ x, const SY* yin, SY* y) {
  // block (m, rows): x = vector, y = site; grid.y = k-point
  int k = blockIdx.y, v = threadIdx.x;
  int site = blockIdx.x * blockDim.y + threadIdx.y;
  if (site >= n * n) return;
  int i = site % n, j = site / n;
  Lay L{n, m, K};
  R axy = sget<R>(axy_s);
  R mm = beta_kv ? Real<R>::from(beta_kv[(size_t) k * m + v] / 6.0) : sget<R>(mm_s);
  const SX* xb = x + L.edge(k, 0, 0, 0, v);
  cx<R> ox, oy;
  if (i > 0 && i < n - 1 && j > 0 && j < n - 1) {
    EAccI<SX, R> E{xb, n, m};
    KapI<R> ki{kap};
    ox = kx_x<R>(E, ki, axy, mm, i, j);
    oy = kx_y<R>(E, ki, axy, mm, i, j);
  } else {
    EAcc<SX, R> E{xb, n, m, seam_load<R>(ph, K, k, n)};
    ox = kx_x<R>(E, kap, axy, mm, i, j);
    oy = kx_y<R>(E, kap, axy, mm, i, j);
  }
  size_t ox_at = L.edge(k, 0, j, i, v), oy_at = L.edge(k, 1, j, i, v);
  if (has_cy) {
    const SY* src = yin ? yin : y;
    R c = sget<R>(cy_s);
    ox += scal(c, Store<SY, R>::ld(src + ox_at));
    oy += scal(c, Store<SY, R>::ld(src + oy_at));
  }
  Store<SY, R>::st(y + ox_at, ox);
  Store<SY, R>::st(y + oy_at, oy);
}

// ------------------------------------------------------------------
// AFW vertex-patch line Gauss-Seidel.  One thread owns one (k, row, vector)
// chain and walks its row in the reference's order; rows of one phase touch
// disjoint unknowns (rows j-1..j+1 read, row j of x and rows j-1, j of y
// written), so every row of a phase runs concurrently.
// Local matrix T and its factorisation: see patch_solve in the oracle; the
// reference's starsolve_common (edge2d.c:2029-2183).
// ------------------------------------------------------------------

// One row of one plane of a (k, vector) edge vector: the row index is
// wrapped once (with its seam phase) when the accessor is made, so a load or
// store tests only the column, which is the same for every thread of a warp
// in the row sweeps below.
template <typename S, typename R>
struct RowIO {
  S* row;          // column 0 of the stored row
  int n, m;
  bool rw;         // the addressed row lies one period outside
  cx<R> rph;       // its phase
  cx<R> xf;
  __device__ __forceinline__ cx<R> ld(int i) const {
    cx<R> v;
    if (i < 0) v = conjc(xf) * Store<S, R>::ld(row + (i + n) * m);
    else if (i >= n) v = xf * Store<S, R>::ld(row + (i - n) * m);
    else v = Store<S, R>::ld(row + i * m);
    return rw ? rph * v : v;
  }
  __device__ __forceinline__ void st(int i, cx<R> v) const {
    if (rw) v = conjc(rph) * v;
    if (i < 0) Store<S, R>::st(row + (i + n) * m, xf * v);
    else if (i >= n) Store<S, R>::st(row + (i - n) * m, conjc(xf) * v);
    else Store<S, R>::st(row + i * m, v);
  }
};
template <typename S, typename R>
__device__ __forceinline__ RowIO<S, R> row_io(S* base, int p, int j, int n, int m, const Seam<R>& seam) {
  RowIO<S, R> r;
  r.n = n; r.m = m; r.xf = seam.xf;
  r.rw = j < 0 || j >= n;
  r.rph = j < 0 ? conjc(seam.yf) : seam.yf;
  int jj = j < 0 ? j + n : (j >= n ? j - n : j);
  r.row = base + (p * n + jj) * n * m;
  return r;
}

// Sliding window over a row: the thread holds the patch data of vertex
// (i,j) -- the reference's mxx[2][3], mxy[3][2], meps[2][2], mbx[2], mby[2]
// (edge2d.c:2185-2236) -- and moves it by one column per patch, loading the
// next column only.  Values are written back once no later patch of this row
// changes them (the ones crossing the periodic seam are written at once, so
// that the row's last patches read them back updated, as the reference does).
// The factors of the transformed patch matrix depend on the four cell
// kappas of the vertex and the scalars only, not on the k-point or vector:
// for FP32 sweeps they are tabulated once per level (mxk_afw_factors) as
// (l20, l21, 1/D0, 1/D1) and (1/D2) per vertex, bitwise equal to computing
// them in the sweep.
struct AfwF {
  float l20, l21, i0, i1, i2;
};
template <typename R>
__device__ __forceinline__ void afw_factors(R kLL, R kUL, R kLR, R kUR, R axy, R s8, R& l20, R& l21, R& i0,
                                            R& i1, R& i2) {
  R aLL = axy * kLL, aLR = axy * kLR, aUL = axy * kUL, aUR = axy * kUR;
  R D0 = aUL + aLR + s8;
  l20 = (aUL - aLR) / D0;
  R D1 = aLL + aUR;
  l21 = (aLL - aUR) / D1;
  R D2 = aLL + aUL + aLR + aUR + s8 - l21 * l21 * D1;
  const R one = rc<R>(1.0f);
  i0 = one / D0;
  i1 = one / D1;
  i2 = one / D2;
}

__global__ void k_afw_factors(int n, const float* __restrict__ kap, float axy, float s8, float4* __restrict__ out) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * n) return;
  int i = t % n, j = t / n;
  float kLL = kap[wrapi(i - 1, n) + wrapi(j - 1, n) * n], kUL = kap[wrapi(i - 1, n) + j * n];
  float kLR = kap[i + wrapi(j - 1, n) * n], kUR = kap[i + j * n];
  float l20, l21, i0, i1, i2;
  afw_factors<float>(kLL, kUL, kLR, kUR, axy, s8, l20, l21, i0, i1, i2);
  out[2 * t] = make_float4(l20, l21, i0, i1);
  out[2 * t + 1] = make_float4(i2, 0.0f, 0.0f, 0.0f);
}

template <typename S, typename R>
__global__ void k_edge_gs_rows(int n, int m, int K, const double* __restrict__ ph, Kap<R> kap,
                               const float4* __restrict__ ftab, Sc axy_s, Sc mm_s, Sc s8_s, Sc is8_s, int j0,
                               int jstep, int nrows, int backward, const S* __restrict__ b, S* x) {
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  size_t per_k = (size_t) nrows * m;
  if (t >= per_k * K) return;
  int k = (int) (t / per_k);
  int r = (int) (t - (size_t) k * per_k);
  int v = r % m;
  int j = j0 + (r / m) * jstep;
  Lay L{n, m, K};
  Seam<R> seam = seam_load<R>(ph, K, k, n);
  S* xk = x + L.edge(k, 0, 0, 0, v);
  S* bk = const_cast<S*>(b) + L.edge(k, 0, 0, 0, v);
  const RowIO<S, R> X0m = row_io<S, R>(xk, 0, j - 1, n, m, seam), X0c = row_io<S, R>(xk, 0, j, n, m, seam),
                    X0p = row_io<S, R>(xk, 0, j + 1, n, m, seam), X1m = row_io<S, R>(xk, 1, j - 1, n, m, seam),
                    X1c = row_io<S, R>(xk, 1, j, n, m, seam), B0c = row_io<S, R>(bk, 0, j, n, m, seam),
                    B1m = row_io<S, R>(bk, 1, j - 1, n, m, seam), B1c = row_io<S, R>(bk, 1, j, n, m, seam);
  const R axy = sget<R>(axy_s);
  const R mm = sget<R>(mm_s);
  const R s8 = sget<R>(s8_s);     // 4 (mx + my), mx = my
  const R is8 = sget<R>(is8_s);
  const R four = rc<R>(4.0f), quarter = rc<R>(0.25f);
  const bool tab = ftab != nullptr;
  int i = backward ? n - 1 : 0;
  // x columns i-1 (a) and i (b), rows j-1, j, j+1; y columns i-1 (a), i (b), i+1 (c), rows j-1, j
  cx<R> xa0 = X0m.ld(i - 1), xa1 = X0c.ld(i - 1), xa2 = X0p.ld(i - 1);
  cx<R> xb0 = X0m.ld(i), xb1 = X0c.ld(i), xb2 = X0p.ld(i);
  cx<R> ya0 = X1m.ld(i - 1), ya1 = X1c.ld(i - 1);
  cx<R> yb0 = X1m.ld(i), yb1 = X1c.ld(i);
  cx<R> yc0 = X1m.ld(i + 1), yc1 = X1c.ld(i + 1);
  R kLL = kap(i - 1, j - 1), kUL = kap(i - 1, j), kLR = kap(i, j - 1), kUR = kap(i, j);
  cx<R> bx0 = B0c.ld(i - 1), bx1 = B0c.ld(i), by0 = B1m.ld(i), by1 = B1c.ld(i);
  float4 fa = make_float4(0.0f, 0.0f, 0.0f, 0.0f), fb = fa;
  if (tab) { fa = ftab[2 * ((size_t) j * n + i)]; fb = ftab[2 * ((size_t) j * n + i) + 1]; }
  for (int step = 0; step < n; step++) {
    const bool last = step == n - 1;
    // prefetch the column the next patch adds (never written by this patch)
    cx<R> nx0, nx1, nx2, ny0, ny1, nbx, nby0, nby1;
    R nk0, nk1;
    float4 nfa, nfb;
    if (!last) {
      int ix = backward ? i - 2 : i + 1;    // new x column
      int iy = backward ? i - 2 : i + 2;    // new y column
      int ib = backward ? i - 1 : i + 1;    // new patch column
      nx0 = X0m.ld(ix); nx1 = X0c.ld(ix); nx2 = X0p.ld(ix);
      ny0 = X1m.ld(iy); ny1 = X1c.ld(iy);
      nk0 = kap(ix, j - 1); nk1 = kap(ix, j);
      if (tab) {
        nfa = ftab[2 * ((size_t) j * n + ib)];
        nfb = ftab[2 * ((size_t) j * n + ib) + 1];
      }
      nbx = B0c.ld(backward ? i - 2 : i + 1);
      nby0 = B1m.ld(ib); nby1 = B1c.ld(ib);
    }
    // residual b - (alpha A + beta M) x at the patch unknowns u0..u3 =
    // x(i-1,j), x(i,j), y(i,j-1), y(i,j) from the four cell curls
    cx<R> cLL = xa0 - xa1 - ya0 + yb0;
    cx<R> cUL = xa1 - xa2 - ya1 + yb1;
    cx<R> cLR = xb0 - xb1 - yb0 + yc0;
    cx<R> cUR = xb1 - xb2 - yb1 + yc1;
    cx<R> r0 = bx0 - (scal(axy, scal(kUL, cUL) - scal(kLL, cLL)) + scal(mm, scal(four, xa1) + xa2 + xa0));
    cx<R> r1 = bx1 - (scal(axy, scal(kUR, cUR) - scal(kLR, cLR)) + scal(mm, scal(four, xb1) + xb2 + xb0));
    cx<R> r2 = by0 - (scal(axy, scal(kLL, cLL) - scal(kLR, cLR)) + scal(mm, scal(four, yb0) + yc0 + ya0));
    cx<R> r3 = by1 - (scal(axy, scal(kUL, cUL) - scal(kUR, cUR)) + scal(mm, scal(four, yb1) + yc1 + ya1));
    // transformed local matrix (mx = my: T10 = T32 = 0) and the reference's
    // elimination without the l20 fill of entry (2,2)
    R l20, l21, i0, i1, i2;
    if (tab) {
      l20 = Real<R>::from_float(fa.x); l21 = Real<R>::from_float(fa.y);
      i0 = Real<R>::from_float(fa.z); i1 = Real<R>::from_float(fa.w); i2 = Real<R>::from_float(fb.x);
    } else {
      afw_factors<R>(kLL, kUL, kLR, kUR, axy, s8, l20, l21, i0, i1, i2);
    }
    cx<R> c0 = r0 + r1 + r2 + r3;
    cx<R> c1 = r0 + r1 - r2 - r3;
    cx<R> c2 = r0 - r1 - r2 + r3;
    cx<R> c3 = r0 - r1 + r2 - r3;
    c2 -= scal(l20, c0) + scal(l21, c1);
    c0 = scal(i0, c0);
    c1 = scal(i1, c1);
    c2 = scal(i2, c2);
    c3 = scal(is8, c3);
    c1 -= scal(l21, c2);
    c0 -= scal(l20, c2);
    xa1 += scal(quarter, c0 + c1 + c2 + c3);
    xb1 += scal(quarter, c0 + c1 - c2 - c3);
    yb0 += scal(quarter, c0 - c1 - c2 + c3);
    yb1 += scal(quarter, c0 - c1 + c2 - c3);
    X1m.st(i, yb0);
    X1c.st(i, yb1);
    if (!backward) {
      X0c.st(i - 1, xa1);
      if (last) {
        X0c.st(i, xb1);
        break;
      }
      xa0 = xb0; xa1 = xb1; xa2 = xb2;
      xb0 = nx0; xb1 = nx1; xb2 = nx2;
      ya0 = yb0; ya1 = yb1; yb0 = yc0; yb1 = yc1;
      yc0 = ny0; yc1 = ny1;
      kLL = kLR; kUL = kUR; kLR = nk0; kUR = nk1;
      if (tab) { fa = nfa; fb = nfb; }
      bx0 = bx1; bx1 = nbx; by0 = nby0; by1 = nby1;
      i++;
    } else {
      X0c.st(i, xb1);
      if (last) {
        X0c.st(i - 1, xa1);
        break;
      }
      xb0 = xa0; xb1 = xa1; xb2 = xa2;
      xa0 = nx0; xa1 = nx1; xa2 = nx2;
      yc0 = yb0; yc1 = yb1; yb0 = ya0; yb1 = ya1;
      ya0 = ny0; ya1 = ny1;
      kLR = kLL; kUR = kUL; kLL = nk0; kUL = nk1;
      if (tab) { fa = nfa; fb = nfb; }
      bx1 = bx0; bx0 = nbx; by0 = nby0; by1 = nby1;
      i--;
    }
  }
}

// ------------------------------------------------------------------
// Point Gauss-Seidel of alpha A + beta M, edge by edge, in the reference's
// interleaved row order (gsforward/gsbackward_simple_edge2d with
// SMOOTHER_INTERLEAVED, edge2d.c:3890-5573): forward, row 0, the even rows,
// the odd rows, row n-1, each left to right, x-edge (i,j) then y-edge
// (i,j); backward the exact reverse.  An edge's update is its residual row
// divided by its diagonal, axy (kappa of its two cells) + 4 beta/6.  Row j
// reads rows j-1..j+1 only, so the rows of one parity are independent and
// the sweep is two launches (rows 0, 2, .., n-2 and rows 1, 3, .., n-1),
// one thread per (k, row, vector) walking its row.  The smoother of the
// Hiptmair cycle (hcycle_edge2d).
// ------------------------------------------------------------------
template <typename S, typename R>
__global__ void k_edge_gs_point(int n, int m, int K, const double* __restrict__ ph, Kap<R> kap, Sc axy_s,
                                Sc mm_s, int j0, int jstep, int nrows, int backward, const S* __restrict__ b,
                                S* x) {
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  size_t per_k = (size_t) nrows * m;
  if (t >= per_k * K) return;
  int k = (int) (t / per_k);
  int r = (int) (t - (size_t) k * per_k);
  int v = r % m;
  int j = j0 + (r / m) * jstep;
  Lay L{n, m, K};
  S* xk = x + L.edge(k, 0, 0, 0, v);
  const S* bk = b + L.edge(k, 0, 0, 0, v);
  EAcc<S, R> X{xk, n, m, seam_load<R>(ph, K, k, n)};
  const R axy = sget<R>(axy_s), mm = sget<R>(mm_s), four = rc<R>(4.0f), one = rc<R>(1.0f);
  auto upd_x = [&](int i) {
    size_t o = ((size_t) j * n + i) * m;
    cx<R> res = Store<S, R>::ld(bk + o) - kx_x<R>(X, kap, axy, mm, i, j);
    R diag = axy * (kap(i, j - 1) + kap(i, j)) + four * mm;
    Store<S, R>::st(xk + o, Store<S, R>::ld(xk + o) + scal(one / diag, res));
  };
  auto upd_y = [&](int i) {
    size_t o = ((size_t) (n + j) * n + i) * m;
    cx<R> res = Store<S, R>::ld(bk + o) - kx_y<R>(X, kap, axy, mm, i, j);
    R diag = axy * (kap(i - 1, j) + kap(i, j)) + four * mm;
    Store<S, R>::st(xk + o, Store<S, R>::ld(xk + o) + scal(one / diag, res));
  };
  if (!backward)
    for (int i = 0; i < n; i++) { upd_x(i); upd_y(i); }
  else
    for (int i = n - 1; i >= 0; i--) { upd_y(i); upd_x(i); }
}

// ------------------------------------------------------------------
// AFW vertex-patch smoother in four colours.  The vertices (i, j) split by
// (i mod 2, j mod 2); two patches of one colour share no unknown, and none
// reads an unknown the other writes (a patch writes x(i-1..i, j) and
// y(i, j-1..j) and reads x(i-1..i, j-1..j+1), y(i-1..i+1, j-1..j)), so the
// patches of a colour are solved concurrently, one thread per (patch,
// vector, k-point), the same local solve as the row sweep.  A forward sweep
// takes the colours (0,0), (1,0), (0,1), (1,1), a backward sweep the reverse
// order; the two colours of one vertex-row parity share a launch
// (k_edge_gs_rowpair).  The iterates differ from the reference's row order; both are
// convergent splittings of the same operator, so the eigenpairs the solver
// converges to are the same.
// ------------------------------------------------------------------
template <typename S, typename R>
__device__ __forceinline__ void st_edge(S* base, int n, int m, const Seam<R>& seam, int p, int i, int j, cx<R> v) {
  cx<R> ph;
  if (seam.wrap(i, j, ph)) v = conjc(ph) * v;
  Store<S, R>::st(base + ((p * n + j) * n + i) * m, v);
}

// one patch solve of the colour sweeps: vertex (i, j), k-point k, vector v
template <typename S, typename R>
__device__ __forceinline__ void afw_patch(int n, int m, int K, const double* __restrict__ ph, const Kap<R>& kap,
                                          const float4* __restrict__ ftab, const Sc& axy_s, const Sc& mm_s,
                                          const Sc& s8_s, const Sc& is8_s, int i, int j, int k, int v,
                                          const S* __restrict__ b, S* x) {
  Lay L{n, m, K};
  S* xb = x + L.edge(k, 0, 0, 0, v);
  const S* bb = b + L.edge(k, 0, 0, 0, v);
  const R axy = sget<R>(axy_s), mm = sget<R>(mm_s), s8 = sget<R>(s8_s), is8 = sget<R>(is8_s);
  const R four = rc<R>(4.0f), quarter = rc<R>(0.25f);
  const bool inner = i > 0 && i < n - 1 && j > 0 && j < n - 1;
  cx<R> xa0, xa1, xa2, xb0, xb1, xb2, ya0, ya1, yb0, yb1, yc0, yc1, bx0, bx1, by0, by1;
  R kLL, kUL, kLR, kUR;
  auto gather = [&](const auto& X, const auto& B, const auto& KA) {
    xa0 = X(0, i - 1, j - 1); xa1 = X(0, i - 1, j); xa2 = X(0, i - 1, j + 1);
    xb0 = X(0, i, j - 1); xb1 = X(0, i, j); xb2 = X(0, i, j + 1);
    ya0 = X(1, i - 1, j - 1); ya1 = X(1, i - 1, j);
    yb0 = X(1, i, j - 1); yb1 = X(1, i, j);
    yc0 = X(1, i + 1, j - 1); yc1 = X(1, i + 1, j);
    bx0 = B(0, i - 1, j); bx1 = B(0, i, j); by0 = B(1, i, j - 1); by1 = B(1, i, j);
    kLL = KA(i - 1, j - 1); kUL = KA(i - 1, j); kLR = KA(i, j - 1); kUR = KA(i, j);
  };
  Seam<R> seam;
  if (inner) {
    gather(EAccI<S, R>{xb, n, m}, EAccI<S, R>{bb, n, m}, KapI<R>{kap});
  } else {
    seam = seam_load<R>(ph, K, k, n);
    gather(EAcc<S, R>{xb, n, m, seam}, EAcc<S, R>{bb, n, m, seam}, kap);
  }
  cx<R> cLL = xa0 - xa1 - ya0 + yb0;
  cx<R> cUL = xa1 - xa2 - ya1 + yb1;
  cx<R> cLR = xb0 - xb1 - yb0 + yc0;
  cx<R> cUR = xb1 - xb2 - yb1 + yc1;
  cx<R> r0 = bx0 - (scal(axy, scal(kUL, cUL) - scal(kLL, cLL)) + scal(mm, scal(four, xa1) + xa2 + xa0));
  cx<R> r1 = bx1 - (scal(axy, scal(kUR, cUR) - scal(kLR, cLR)) + scal(mm, scal(four, xb1) + xb2 + xb0));
  cx<R> r2 = by0 - (scal(axy, scal(kLL, cLL) - scal(kLR, cLR)) + scal(mm, scal(four, yb0) + yc0 + ya0));
  cx<R> r3 = by1 - (scal(axy, scal(kUL, cUL) - scal(kUR, cUR)) + scal(mm, scal(four, yb1) + yc1 + ya1));
  R l20, l21, i0, i1, i2;
  if (ftab) {
    float4 fa = ftab[2 * (j * n + i)];
    l20 = Real<R>::from_float(fa.x); l21 = Real<R>::from_float(fa.y);
    i0 = Real<R>::from_float(fa.z); i1 = Real<R>::from_float(fa.w);
    i2 = Real<R>::from_float(ftab[2 * (j * n + i) + 1].x);
  } else {
    afw_factors<R>(kLL, kUL, kLR, kUR, axy, s8, l20, l21, i0, i1, i2);
  }
  cx<R> c0 = r0 + r1 + r2 + r3;
  cx<R> c1 = r0 + r1 - r2 - r3;
  cx<R> c2 = r0 - r1 - r2 + r3;
  cx<R> c3 = r0 - r1 + r2 - r3;
  c2 -= scal(l20, c0) + scal(l21, c1);
  c0 = scal(i0, c0);
  c1 = scal(i1, c1);
  c2 = scal(i2, c2);
  c3 = scal(is8, c3);
  c1 -= scal(l21, c2);
  c0 -= scal(l20, c2);
  xa1 += scal(quarter, c0 + c1 + c2 + c3);
  xb1 += scal(quarter, c0 + c1 - c2 - c3);
  yb0 += scal(quarter, c0 - c1 - c2 + c3);
  yb1 += scal(quarter, c0 - c1 + c2 - c3);
  if (inner) {
    Store<S, R>::st(xb + (j * n + i - 1) * m, xa1);
    Store<S, R>::st(xb + (j * n + i) * m, xb1);
    Store<S, R>::st(xb + ((n + j - 1) * n + i) * m, yb0);
    Store<S, R>::st(xb + ((n + j) * n + i) * m, yb1);
  } else {
    st_edge<S, R>(xb, n, m, seam, 0, i - 1, j, xa1);
    st_edge<S, R>(xb, n, m, seam, 0, i, j, xb1);
    st_edge<S, R>(xb, n, m, seam, 1, i, j - 1, yb0);
    st_edge<S, R>(xb, n, m, seam, 1, i, j, yb1);
  }
}

// The colours (0, cj) and (1, cj) in one launch: a CTA per vertex row j of
// parity cj and k-point.  The first colour is F = rev (even i forward, odd
// i backward), the second G = 1 - F.  A patch interacts (shares unknowns or
// reads another's) only with its left and right neighbours in the row, so
// the CTA walks the row in chunks of P first-colour patches i = 2p + F and,
// after a barrier, solves the second-colour patches i = 2p + F - 1 between
// them and the previous chunk; the wrapped second-colour patch (F - 1 mod n)
// comes last.  Every second-colour patch then runs after both neighbours
// and before nothing that reads it, so the result is that of the two colour
// launches, and a chunk's data are read again while still on chip.  Rows of
// one parity neither share an unknown nor read each other's, so the rows run
// concurrently.  Barriers make a block's global writes visible to the block.
template <typename S, typename R>
__global__ void k_edge_gs_rowpair(int n, int m, int K, const double* __restrict__ ph, Kap<R> kap,
                                  const float4* __restrict__ ftab, Sc axy_s, Sc mm_s, Sc s8_s, Sc is8_s, int cj,
                                  int rev, const S* __restrict__ b, S* x) {
  // block (m, P): x = vector, y = patch lane; grid (rows of the parity, K)
  const int k = blockIdx.y, v = threadIdx.x, P = blockDim.y, h = n / 2;
  const int j = 2 * blockIdx.x + cj, F = rev;
  for (int c = 0; c < h; c += P) {
    const int p = c + threadIdx.y;
    if (p < h) afw_patch<S, R>(n, m, K, ph, kap, ftab, axy_s, mm_s, s8_s, is8_s, 2 * p + F, j, k, v, b, x);
    __syncthreads();
    if (p < h && p >= 1)
      afw_patch<S, R>(n, m, K, ph, kap, ftab, axy_s, mm_s, s8_s, is8_s, 2 * p + F - 1, j, k, v, b, x);
    __syncthreads();
  }
  if (threadIdx.y == 0)
    afw_patch<S, R>(n, m, K, ph, kap, ftab, axy_s, mm_s, s8_s, is8_s, (F + n - 1) % n, j, k, v, b, x);
}

// ------------------------------------------------------------------
// edge transfers (gather form of prolongation_edge2d / restriction_edge2d)
// ------------------------------------------------------------------
template <typename S, typename R>
__global__ void k_edge_prolong(int nc, int m, int K, const double* __restrict__ ph, Sc alpha,
                               const S* __restrict__ c, S* __restrict__ f) {
  int nf = 2 * nc;
  // block (m, rows): x = vector, y = site; grid.y = k-point
  int k = blockIdx.y, v = threadIdx.x;
  int site = blockIdx.x * blockDim.y + threadIdx.y;
  if (site >= nf * nf) return;
  int i = site % nf, j = site / nf;
  Lay Lc{nc, m, K}, Lf{nf, m, K};
  const S* cb = c + Lc.edge(k, 0, 0, 0, v);
  int ci = i >> 1, cj = j >> 1;
  R half = rc<R>(0.5f), quarter = rc<R>(0.25f), a = sget<R>(alpha);
  cx<R> vx, vy;
  auto body = [&](const auto& C) {
    vx = (j & 1) ? scal(quarter, C(0, ci, cj) + C(0, ci, cj + 1)) : scal(half, C(0, ci, cj));
    vy = (i & 1) ? scal(quarter, C(1, ci, cj) + C(1, ci + 1, cj)) : scal(half, C(1, ci, cj));
  };
  if (ci < nc - 1 && cj < nc - 1) body(EAccI<S, R>{cb, nc, m});
  else body(EAcc<S, R>{cb, nc, m, seam_load<R>(ph, K, k, nc)});
  S* px = f + Lf.edge(k, 0, j, i, v);
  S* py = f + Lf.edge(k, 1, j, i, v);
  Store<S, R>::st(px, Store<S, R>::ld(px) + scal(a, vx));
  Store<S, R>::st(py, Store<S, R>::ld(py) + scal(a, vy));
}

template <typename S, typename R>
__global__ void k_edge_restrict(int nc, int m, int K, const double* __restrict__ ph, Sc alpha,
                                const S* __restrict__ f, S* __restrict__ c) {
  int nf = 2 * nc;
  // block (m, rows): x = vector, y = site; grid.y = k-point
  int k = blockIdx.y, v = threadIdx.x;
  int site = blockIdx.x * blockDim.y + threadIdx.y;
  if (site >= nc * nc) return;
  int i = site % nc, j = site / nc;
  Lay Lc{nc, m, K}, Lf{nf, m, K};
  const S* fb = f + Lf.edge(k, 0, 0, 0, v);
  R half = rc<R>(0.5f), quarter = rc<R>(0.25f), a = sget<R>(alpha);
  int fi = 2 * i, fj = 2 * j;
  cx<R> sx, sy;
  auto body = [&](const auto& F) {
    sx = scal(half, F(0, fi, fj) + F(0, fi + 1, fj))
         + scal(quarter, F(0, fi, fj - 1) + F(0, fi + 1, fj - 1) + F(0, fi, fj + 1) + F(0, fi + 1, fj + 1));
    sy = scal(half, F(1, fi, fj) + F(1, fi, fj + 1))
         + scal(quarter, F(1, fi - 1, fj) + F(1, fi - 1, fj + 1) + F(1, fi + 1, fj) + F(1, fi + 1, fj + 1));
  };
  if (i > 0 && j > 0) body(EAccI<S, R>{fb, nf, m});
  else body(EAcc<S, R>{fb, nf, m, seam_load<R>(ph, K, k, nf)});
  S* px = c + Lc.edge(k, 0, j, i, v);
  S* py = c + Lc.edge(k, 1, j, i, v);
  Store<S, R>::st(px, Store<S, R>::ld(px) + scal(a, sx));
  Store<S, R>::st(py, Store<S, R>::ld(py) + scal(a, sy));
}

// ------------------------------------------------------------------
// node space: Q1 Laplace with hx = hy (diagonal 8/3, neighbours -1/3)
// ------------------------------------------------------------------
template <typename R, typename A>
__device__ __forceinline__ cx<R> lap_off(const A& V, int i, int j) {
  return V(i - 1, j) + V(i + 1, j) + V(i, j - 1) + V(i, j + 1) + V(i - 1, j - 1) + V(i + 1, j - 1)
         + V(i - 1, j + 1) + V(i + 1, j + 1);
}

// y = cy yin + alpha L x, a thread per two neighbouring nodes (i, i+1) of a
// row and vector, which share six of their nine stencil values
template <typename S, typename R>
__global__ void k_node_apply(int n, int m, int K, const double* __restrict__ ph, Sc diag, Sc off, Sc cy,
                             int has_cy, const S* __restrict__ x, const S* yin, S* y) {
  // block (m, rows): x = vector, y = node pair; grid.y = k-point
  const int k = blockIdx.y, v = threadIdx.x, hp = (n + 1) / 2;
  const int pair = blockIdx.x * blockDim.y + threadIdx.y;
  if (pair >= hp * n) return;
  const int i = 2 * (pair % hp), j = pair / hp;
  const bool two = i + 1 < n;
  Lay L{n, m, K};
  const S* xb = x + L.node(k, 0, 0, v);
  const R dg = sget<R>(diag), of = sget<R>(off);
  cx<R> o0, o1 = czero<R>();
  auto body = [&](const auto& V) {
    o0 = scal(dg, V(i, j)) + scal(of, lap_off<R>(V, i, j));
    if (two) o1 = scal(dg, V(i + 1, j)) + scal(of, lap_off<R>(V, i + 1, j));
  };
  if (i > 0 && i + 2 < n && j > 0 && j < n - 1) body(NAccI<S, R>{xb, n, m});
  else body(NAcc<S, R>{xb, n, m, seam_load<R>(ph, K, k, n)});
  const size_t at = L.node(k, j, i, v);
  const S* yr = yin ? yin : y;
  if (has_cy) {
    o0 += scal(sget<R>(cy), Store<S, R>::ld(yr + at));
    if (two) o1 += scal(sget<R>(cy), Store<S, R>::ld(yr + at + m));
  }
  Store<S, R>::st(y + at, o0);
  if (two) Store<S, R>::st(y + at + m, o1);
}

// The node residual and its restriction in one pass (the node V-cycle's
// residual + restriction_node2d, node2d.c:1140-1273, 1352-1389):
// c(ci, cj) = sum of d over the 3 x 3 fine nodes around (2ci, 2cj) with
// weights 1, 1/2, 1/4, where d = b - alpha L x is formed from the 5 x 5
// window of x around them; the coarse vector is written, not accumulated.
// Neighbouring threads share their windows through L1, so x and b come from
// DRAM once and d never goes there: 2.25 fine arrays of traffic against
// 4.25 for the two kernels.  Two forms: a thread per (coarse node, vector)
// (k_node_residual_restrict_site), and for large batches a thread per
// (coarse column, strip of RR_CH coarse rows, vector) that walks up its
// strip keeping the fine rows of x and the row of d that the next coarse
// node shares with the last one in registers, so a coarse node costs two
// new rows of x (10 loads), two of b (6) and two rows of d (6 values)
// instead of the whole 5 x 5 window and nine values of d.
template <typename S, typename R>
__global__ void k_node_residual_restrict_site(int nc, int m, int K, const double* __restrict__ ph, Sc diag,
                                              Sc off, const S* __restrict__ x, const S* __restrict__ b,
                                              S* __restrict__ c) {
  const int nf = 2 * nc;
  // block (m, rows): x = vector, y = coarse node; grid.y = k-point
  const int k = blockIdx.y, v = threadIdx.x;
  const int site = blockIdx.x * blockDim.y + threadIdx.y;
  if (site >= nc * nc) return;
  const int ci = site % nc, cj = site / nc, fi = 2 * ci, fj = 2 * cj;
  Lay Lc{nc, m, K}, Lf{nf, m, K};
  const S* xb = x + Lf.node(k, 0, 0, v);
  const S* bb = b + Lf.node(k, 0, 0, v);
  const R dg = sget<R>(diag), of = sget<R>(off), half = rc<R>(0.5f), quarter = rc<R>(0.25f);
  cx<R> sres;
  auto body = [&](const auto& X, const auto& B) {
    cx<R> w[5][5];
#pragma unroll
    for (int q = 0; q < 5; q++)
#pragma unroll
      for (int p = 0; p < 5; p++) w[q][p] = X(fi - 2 + p, fj - 2 + q);
    // d at fine node (fi + a, fj + e), a, e in -1..1
    auto d = [&](int a, int e) {
      const int p = a + 2, q = e + 2;
      const cx<R> nb = w[q][p - 1] + w[q][p + 1] + w[q - 1][p] + w[q + 1][p] + w[q - 1][p - 1] + w[q - 1][p + 1]
                       + w[q + 1][p - 1] + w[q + 1][p + 1];
      return B(fi + a, fj + e) - (scal(dg, w[q][p]) + scal(of, nb));
    };
    sres = d(0, 0) + scal(half, d(-1, 0) + d(1, 0) + d(0, -1) + d(0, 1))
           + scal(quarter, d(-1, -1) + d(1, -1) + d(-1, 1) + d(1, 1));
  };
  if (ci > 0 && cj > 0 && ci < nc - 1 && cj < nc - 1) body(NAccI<S, R>{xb, nf, m}, NAccI<S, R>{bb, nf, m});
  else {
    const Seam<R> seam = seam_load<R>(ph, K, k, nf);
    body(NAcc<S, R>{xb, nf, m, seam}, NAcc<S, R>{bb, nf, m, seam});
  }
  Store<S, R>::st(c + Lc.node(k, cj, ci, v), sres);
}

// coarse rows per strip; the FP32 form is held to 80 registers (3 CTAs per
// SM, a few spilled values) -- at 124 registers it ran 0.906 against 0.741 ms
constexpr int RR_CH = 8;
template <typename S, typename R>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 3 : 1)
    k_node_residual_restrict(int nc, int m, int K, const double* __restrict__ ph, Sc diag, Sc off,
                             const S* __restrict__ x, const S* __restrict__ b, S* __restrict__ c) {
  const int nf = 2 * nc, nst = (nc + RR_CH - 1) / RR_CH;
  // block (m, columns): x = vector, y = (column, strip); grid.y = k-point
  const int k = blockIdx.y, v = threadIdx.x;
  const int s = blockIdx.x * blockDim.y + threadIdx.y;
  if (s >= nc * nst) return;
  const int ci = s % nc, cj0 = (s / nc) * RR_CH, cj1 = min(cj0 + RR_CH, nc), fi = 2 * ci;
  Lay Lc{nc, m, K}, Lf{nf, m, K};
  const S* xb = x + Lf.node(k, 0, 0, v);
  const S* bb = b + Lf.node(k, 0, 0, v);
  const R dg = sget<R>(diag), of = sget<R>(off), half = rc<R>(0.5f), quarter = rc<R>(0.25f);
  auto body = [&](const auto& X, const auto& B) {
    // x at fine columns fi-2..fi+2 of four consecutive fine rows
    cx<R> xa[5], xm[5], xc[5], xd[5], dp[3], d0[3], dn[3];
    auto ldx = [&](cx<R>* w, int fj) {
#pragma unroll
      for (int p = 0; p < 5; p++) w[p] = X(fi - 2 + p, fj);
    };
    // d at fine columns fi-1..fi+1 of row fj, from x rows fj-1 (u), fj (w), fj+1 (l)
    auto drow = [&](const cx<R>* u, const cx<R>* w, const cx<R>* l, int fj, cx<R>* d) {
#pragma unroll
      for (int a = 0; a < 3; a++) {
        const int p = a + 1;
        const cx<R> nb = w[p - 1] + w[p + 1] + u[p] + l[p] + u[p - 1] + u[p + 1] + l[p - 1] + l[p + 1];
        d[a] = B(fi - 1 + a, fj) - (scal(dg, w[p]) + scal(of, nb));
      }
    };
    int fj = 2 * cj0;
    ldx(xc, fj - 2);
    ldx(xa, fj - 1);
    ldx(xm, fj);
    drow(xc, xa, xm, fj - 1, dp);
#pragma unroll 1
    for (int cj = cj0; cj < cj1; cj++, fj += 2) {
      ldx(xc, fj + 1);
      ldx(xd, fj + 2);
      drow(xa, xm, xc, fj, d0);
      drow(xm, xc, xd, fj + 1, dn);
      const cx<R> sres = d0[1] + scal(half, d0[0] + d0[2] + dp[1] + dn[1])
                         + scal(quarter, dp[0] + dp[2] + dn[0] + dn[2]);
      Store<S, R>::st(c + Lc.node(k, cj, ci, v), sres);
#pragma unroll
      for (int p = 0; p < 5; p++) {
        xa[p] = xc[p];
        xm[p] = xd[p];
      }
#pragma unroll
      for (int a = 0; a < 3; a++) dp[a] = dn[a];
    }
  };
  // the strip's x rows run from 2 cj0 - 2 to 2 cj1, its columns from fi-2 to fi+2
  if (ci > 0 && ci < nc - 1 && cj0 > 0 && cj1 < nc) body(NAccI<S, R>{xb, nf, m}, NAccI<S, R>{bb, nf, m});
  else {
    const Seam<R> seam = seam_load<R>(ph, K, k, nf);
    body(NAcc<S, R>{xb, nf, m, seam}, NAcc<S, R>{bb, nf, m, seam});
  }
}

template <typename S, typename R>
struct NIO {
  S* base;
  int n, m;
  Seam<R> seam;
  __device__ __forceinline__ cx<R> ld(int i, int j) const {
    cx<R> ph;
    bool w = seam.wrap(i, j, ph);
    cx<R> v = Store<S, R>::ld(base + ((size_t) j * n + i) * m);
    return w ? ph * v : v;
  }
  __device__ __forceinline__ void st(int i, int j, cx<R> v) const {
    cx<R> ph;
    if (seam.wrap(i, j, ph)) v = conjc(ph) * v;
    Store<S, R>::st(base + ((size_t) j * n + i) * m, v);
  }
};

// Point Gauss-Seidel of one row, solved in parallel.  Along a row the sweep
// is x_i = x_{i-s}/8 + beta_i (s = +1 forward, -1 backward): the coefficient
// of the already updated neighbour is (1/3)*(3/8) = 1/8 for any alpha, and
// beta_i = (3/(8 alpha)) (b_i + (alpha/3) * (old right neighbour + the six
// neighbours in rows j-1, j+1)).  The chain starts at i0 with the old value
// across the seam (folded into beta'_{i0} = beta_{i0} + x_{i0-s}/8) and ends
// with the new x_{i0} across the seam.  Hence
//   x_{i_t} = sum_{d=0}^{min(t,D)} 8^-d beta'_{i_{t-d}},
// truncated where 8^-(D+1) is below the arithmetic's precision.
// A lane takes runs of LR consecutive chain positions.  Pass 1 puts beta'
// of its run into a ring in shared memory, reading old values only: along
// the run the lane keeps the three values of rows j-1 and j+1 that a
// position needs in a sliding window, so a position costs four loads.
// Pass 2 writes the prefix sums of a run into x: the lane starts it with
// the truncated sum over the ring and continues with x_t = x_{t-1}/8 +
// beta'_t (the GS recurrence itself).  Pass 1 of a run reads the row's old
// x at the run's positions and the next one only, so runs whose pass 2
// is done may lie behind it.  The new x_{i0} that the last position needs
// is formed from old values before anything is written.

// the row j of k-point k, vector v, for the sweep; position t sits at
// column i0 + sd t
template <typename S, typename R>
struct GsRow {
  int n, m, j, sd, i0, st;
  Seam<R> seam;
  NAcc<S, R> X;
  const S *bb, *rowm, *rowp, *rowc, *rowb;
  S* xr;
  R inv_ac, third;
  __device__ GsRow(int n_, int m_, int K, int k, int v, int j_, int backward, const double* ph, Sc inv_ac_s,
                   Sc third_s, const S* b, S* x)
      : n(n_), m(m_), j(j_), sd(backward ? -1 : 1), i0(backward ? n_ - 1 : 0), st((backward ? -1 : 1) * m_),
        seam(seam_load<R>(ph, K, k, n_)), X{nullptr, n_, m_, seam}, inv_ac(sget<R>(inv_ac_s)),
        third(sget<R>(third_s)) {
    Lay L{n, m, K};
    const S* xk = x + L.node(k, 0, 0, v);
    X.base = xk;
    bb = b + L.node(k, 0, 0, v);
    xr = x + L.node(k, j, 0, v);
    // rows j-1, j+1 through plain pointers, with the seam phase of the whole
    // row applied to the sums when it lies across the seam
    const int jm = j == 0 ? n - 1 : j - 1, jp = j == n - 1 ? 0 : j + 1;
    rowm = xk + ((size_t) jm * n + i0) * m;
    rowp = xk + ((size_t) jp * n + i0) * m;
    rowc = xk + ((size_t) j * n + i0) * m;
    rowb = bb + ((size_t) j * n + i0) * m;
  }
  __device__ cx<R> beta_at(int ii, cx<R> next) const {
    cx<R> nb = next + X(ii - 1, j - 1) + X(ii, j - 1) + X(ii + 1, j - 1) + X(ii - 1, j + 1) + X(ii, j + 1)
               + X(ii + 1, j + 1);
    return scal(inv_ac, Store<S, R>::ld(bb + ((size_t) j * n + ii) * m) + scal(third, nb));
  }
  // the new x_{i0}, from old values only
  __device__ cx<R> x0() const { return beta_at(i0, X(i0 + sd, j)) + scal(rc<R>(0.125f), X(i0 - sd, j)); }
  // beta' at positions 0 and n-1, whose stencils cross the seam in i
  __device__ cx<R> beta_end(int t, cx<R> x0v) const {
    if (t == 0) return x0v;
    int i = i0 + sd * t, ii = i + sd, jj = j;
    cx<R> phz;
    bool w = seam.wrap(ii, jj, phz);
    return beta_at(i, w ? phz * x0v : x0v);
  }
  // pass 1 of the run [u, ue) (ue <= u + LR): the window loads ...
  template <int LR>
  struct Win {
    cx<R> wm[LR + 2], wp[LR + 2], wc[LR], wb[LR];
  };
  template <int LR>
  __device__ __forceinline__ void load(int u, int ue, Win<LR>& w) const {
    // wm[q], wp[q]: rows j-1, j+1 at position u + q - 1; wc[q], wb[q]: the
    // row's old x at position u + q + 1 and b at u + q
#pragma unroll
    for (int q = 0; q < LR + 2; q++) {
      const int pq = u + q - 1;
      if (pq >= 0 && pq <= ue && pq < n) {
        w.wm[q] = Store<S, R>::ld(rowm + pq * st);
        w.wp[q] = Store<S, R>::ld(rowp + pq * st);
      }
    }
#pragma unroll
    for (int q = 0; q < LR; q++) {
      const int pq = u + q;
      if (pq >= 1 && pq < ue && pq < n - 1) {
        w.wc[q] = Store<S, R>::ld(rowc + (pq + 1) * st);
        w.wb[q] = Store<S, R>::ld(rowb + pq * st);
      }
    }
  }
  // ... and the betas of the run into the ring slots (pos & rmask) * m
  template <int LR>
  __device__ __forceinline__ void betas(int u, int ue, const Win<LR>& w, cx<R>* ring, int rmask,
                                        cx<R> x0v) const {
#pragma unroll
    for (int q = 0; q < LR; q++) {
      const int pq = u + q;
      if (pq < ue) {
        cx<R> be;
        if (pq >= 1 && pq < n - 1) {
          cx<R> sm = w.wm[q] + w.wm[q + 1] + w.wm[q + 2], sp = w.wp[q] + w.wp[q + 1] + w.wp[q + 2];
          if (j == 0) sm = conjc(seam.yf) * sm;
          if (j == n - 1) sp = seam.yf * sp;
          be = scal(inv_ac, w.wb[q] + scal(third, w.wc[q] + sm + sp));
        } else {
          be = beta_end(pq, x0v);
        }
        ring[(pq & rmask) * m] = be;
      }
    }
  }
  // pass 2 over the positions [t, te) in one pass: the truncated sum over
  // the D betas before t, then the recurrence
  template <int D>
  __device__ __forceinline__ void prefix_run(int t, int te, const cx<R>* ring, int rmask) const {
    if (t >= te) return;
    const R eighth = rc<R>(0.125f);
    cx<R> acc = czero<R>();
    const int dmax = t < D ? t : D;
    for (int d = dmax; d >= 1; d--) acc = scal(eighth, acc) + ring[((t - d) & rmask) * m];
    for (int q = t; q < te; q++) {
      acc = scal(eighth, acc) + ring[(q & rmask) * m];
      Store<S, R>::st(xr + (size_t) (i0 + sd * q) * m, acc);
    }
  }
  // pass 2 of the run [t, te) from the ring
  template <int D, int LR>
  __device__ __forceinline__ void prefix(int t, int te, const cx<R>* ring, int rmask) const {
    if (t >= te) return;
    const R eighth = rc<R>(0.125f);
    cx<R> acc = czero<R>();
    const int dmax = t < D ? t : D;
    for (int d = dmax; d >= 1; d--)   // Horner from the farthest term
      acc = scal(eighth, acc) + ring[((t - d) & rmask) * m];
#pragma unroll
    for (int q = 0; q < LR; q++)
      if (t + q < te) {
        acc = scal(eighth, acc) + ring[((t + q) & rmask) * m];
        Store<S, R>::st(xr + (size_t) (i0 + sd * (t + q)) * m, acc);
      }
  }
};

// One CTA per (row, k-point): P position lanes walk the row in segments of
// SEG = P LR positions.  The passes are software-pipelined: a round issues
// the loads of pass 1 for segment s+1, runs pass 2 of segment s while they
// are in flight, stores the betas of s+1 and ends at a barrier.  Pass 2 of
// s reads the ring slots [t0 - D, t1) and pass 1 of s+1 writes the next
// SEG slots, so the ring holds at least 2 SEG + D slots.  Used for the
// single rows 0 and n-1, where one row per k-point leaves the GPU idle
// otherwise.
template <typename S, typename R, int D, int LR>
__global__ void __launch_bounds__(256, 2)
    k_node_gs_row(int n, int m, int K, const double* __restrict__ ph, Sc inv_ac_s, Sc third_s, int j0,
                  int jstep, int backward, int rmask, const S* __restrict__ b, S* x) {
  extern __shared__ float smn[];
  const int k = blockIdx.y, v = threadIdx.x, ty = threadIdx.y, SEG = blockDim.y * LR;
  cx<R>* ring = reinterpret_cast<cx<R>*>(smn) + v;           // (rmask + 1) * m
  cx<R>* x0s = reinterpret_cast<cx<R>*>(smn) + (size_t) (rmask + 1) * m;   // m
  const GsRow<S, R> row(n, m, K, k, v, j0 + blockIdx.x * jstep, backward, ph, inv_ac_s, third_s, b, x);
  using W = typename GsRow<S, R>::template Win<LR>;
  if (ty == 0) x0s[v] = row.x0();
  __syncthreads();
  const cx<R> x0v = x0s[v];
  const int r0 = ty * LR;
  {
    const int u1 = SEG < n ? SEG : n, ue = r0 + LR < u1 ? r0 + LR : u1;
    W w;
    row.template load<LR>(r0, ue, w);
    row.template betas<LR>(r0, ue, w, ring, rmask, x0v);
  }
  __syncthreads();
  for (int t0 = 0; t0 < n; t0 += SEG) {
    const int t1 = t0 + SEG < n ? t0 + SEG : n, u1 = t1 + SEG < n ? t1 + SEG : n;
    const int t = t0 + r0, u = t1 + r0, ue = u + LR < u1 ? u + LR : u1;
    W w;
    row.template load<LR>(u, ue, w);
    row.template prefix<D, LR>(t, t + LR < t1 ? t + LR : t1, ring, rmask);
    row.template betas<LR>(u, ue, w, ring, rmask, x0v);
    __syncthreads();
  }
}

// One warp per (row, k-point), eight rows of a row group per CTA and no
// block barrier: the warp's G = 32/m lane groups take consecutive runs of
// a chunk of G LR positions, the ring of a warp holding a chunk and the D
// positions before it; a chunk's betas and its prefix sums are separated
// by __syncwarp.  Rows of one group read the same neighbour rows, which the
// warps of a CTA then share through L1.
template <typename S, typename R, int D, int LR>
__global__ void __launch_bounds__(256, 2)
    k_node_gs_warp(int n, int m, int K, const double* __restrict__ ph, Sc inv_ac_s, Sc third_s, int j0,
                   int jstep, int nrows, int backward, int rmask, const S* __restrict__ b, S* x) {
  extern __shared__ float smn[];
  const int k = blockIdx.y, wid = threadIdx.x >> 5, lane = threadIdx.x & 31, G = 32 / m;
  const int r = blockIdx.x * 8 + wid;
  if (r >= nrows || lane >= G * m) return;
  const int v = lane % m, g = lane / m, CH = G * LR;
  cx<R>* wbase = reinterpret_cast<cx<R>*>(smn) + (size_t) wid * (rmask + 2) * m;
  cx<R>* ring = wbase + v;                            // (rmask + 1) * m
  cx<R>* x0s = wbase + (size_t) (rmask + 1) * m;      // m
  const GsRow<S, R> row(n, m, K, k, v, j0 + r * jstep, backward, ph, inv_ac_s, third_s, b, x);
  using W = typename GsRow<S, R>::template Win<LR>;
  const unsigned mask = G * m == 32 ? 0xffffffffu : (1u << (G * m)) - 1u;
  if (g == 0) x0s[v] = row.x0();
  __syncwarp(mask);
  const cx<R> x0v = x0s[v];
  for (int c0 = 0; c0 < n; c0 += CH) {
    const int c1 = c0 + CH < n ? c0 + CH : n;
    const int u = c0 + g * LR, ue = u + LR < c1 ? u + LR : c1;
    W w;
    row.template load<LR>(u, ue, w);
    row.template betas<LR>(u, ue, w, ring, rmask, x0v);
    __syncwarp(mask);
    row.template prefix<D, LR>(u, ue, ring, rmask);
    __syncwarp(mask);
  }
}

// One CTA per (row, k-point) with the whole row's betas in shared memory:
// pass 1 for every position of the row (each of the P lanes a contiguous
// stretch of n / P positions, in runs of LR through the sliding window),
// a barrier, then pass 2 with each lane's stretch as one prefix run.  A row
// is two steps deep instead of n / (P LR) rounds, so short rows (the coarser
// levels, the single rows 0 and n-1) stop waiting on one chunk after
// another.  Every old value of the row is read before the barrier and the
// row is written only after it; other rows of the launch never read it.
template <typename S, typename R, int D, int LR>
__global__ void __launch_bounds__(256) k_node_gs_rowpar(int n, int m, int K, const double* __restrict__ ph,
                                                      Sc inv_ac_s, Sc third_s, int j0, int jstep, int backward,
                                                      int rmask, const S* __restrict__ b, S* x) {
  extern __shared__ float smn[];
  const int k = blockIdx.y, v = threadIdx.x, ty = threadIdx.y, P = blockDim.y;
  cx<R>* ring = reinterpret_cast<cx<R>*>(smn) + v;                        // (rmask + 1) * m
  cx<R>* x0s = reinterpret_cast<cx<R>*>(smn) + (size_t) (rmask + 1) * m;   // m
  const GsRow<S, R> row(n, m, K, k, v, j0 + blockIdx.x * jstep, backward, ph, inv_ac_s, third_s, b, x);
  using W = typename GsRow<S, R>::template Win<LR>;
  if (ty == 0) x0s[v] = row.x0();
  __syncthreads();
  const cx<R> x0v = x0s[v];
  const int per = (n + P - 1) / P, p0 = ty * per < n ? ty * per : n, p1 = p0 + per < n ? p0 + per : n;
  for (int u = p0; u < p1; u += LR) {
    const int ue = u + LR < p1 ? u + LR : p1;
    W w;
    row.template load<LR>(u, ue, w);
    row.template betas<LR>(u, ue, w, ring, rmask, x0v);
  }
  __syncthreads();
  row.template prefix_run<D>(p0, p1, ring, rmask);
}

// Bilinear prolongation, one thread per (coarse node, vector): the four
// fine nodes (2ci + oi, 2cj + oj) from the coarse values at the corners of
// cell (ci, cj), weight alpha * (1/2 per odd coordinate), in the order
// c00 (+ c10) (+ c01) (+ c11) for every fine node.
template <typename S, typename R>
__global__ void k_node_prolong(int nc, int m, int K, const double* __restrict__ ph, Sc alpha,
                               const S* __restrict__ c, S* __restrict__ f) {
  const int nf = 2 * nc;
  // block (m, rows): x = vector, y = coarse node; grid.y = k-point
  const int k = blockIdx.y, v = threadIdx.x;
  const int site = blockIdx.x * blockDim.y + threadIdx.y;
  if (site >= nc * nc) return;
  const int ci = site % nc, cj = site / nc;
  Lay Lc{nc, m, K}, Lf{nf, m, K};
  const S* cb = c + Lc.node(k, 0, 0, v);
  cx<R> c00, c10, c01, c11;
  auto body = [&](const auto& C) {
    c00 = C(ci, cj); c10 = C(ci + 1, cj); c01 = C(ci, cj + 1); c11 = C(ci + 1, cj + 1);
  };
  if (ci < nc - 1 && cj < nc - 1) body(NAccI<S, R>{cb, nc, m});
  else body(NAcc<S, R>{cb, nc, m, seam_load<R>(ph, K, k, nc)});
  // weights: exact powers of two
  const R h = rc<R>(0.5f), a = sget<R>(alpha);
  const cx<R> v00 = c00, v10 = scal(h, c00 + c10), v01 = scal(h, c00 + c01);
  const cx<R> v11 = scal(h, scal(h, c00 + c10 + c01 + c11));
  S* p0 = f + Lf.node(k, 2 * cj, 2 * ci, v);
  S* p1 = f + Lf.node(k, 2 * cj + 1, 2 * ci, v);
  const cx<R> f00 = Store<S, R>::ld(p0), f10 = Store<S, R>::ld(p0 + m), f01 = Store<S, R>::ld(p1),
              f11 = Store<S, R>::ld(p1 + m);
  Store<S, R>::st(p0, f00 + scal(a, v00));
  Store<S, R>::st(p0 + m, f10 + scal(a, v10));
  Store<S, R>::st(p1, f01 + scal(a, v01));
  Store<S, R>::st(p1 + m, f11 + scal(a, v11));
}

template <typename S, typename R>
__global__ void k_node_restrict(int nc, int m, int K, const double* __restrict__ ph, Sc alpha,
                                const S* __restrict__ f, S* __restrict__ c) {
  int nf = 2 * nc;
  // block (m, rows): x = vector, y = site; grid.y = k-point
  int k = blockIdx.y, v = threadIdx.x;
  int site = blockIdx.x * blockDim.y + threadIdx.y;
  if (site >= nc * nc) return;
  int i = site % nc, j = site / nc;
  Lay Lc{nc, m, K}, Lf{nf, m, K};
  const S* fb = f + Lf.node(k, 0, 0, v);
  int fi = 2 * i, fj = 2 * j;
  cx<R> s;
  auto body = [&](const auto& F) {
    s = F(fi, fj) + scal(rc<R>(0.5f), F(fi - 1, fj) + F(fi + 1, fj) + F(fi, fj - 1) + F(fi, fj + 1))
        + scal(rc<R>(0.25f), F(fi - 1, fj - 1) + F(fi + 1, fj - 1) + F(fi - 1, fj + 1) + F(fi + 1, fj + 1));
  };
  if (i > 0 && j > 0) body(NAccI<S, R>{fb, nf, m});
  else body(NAcc<S, R>{fb, nf, m, seam_load<R>(ph, K, k, nf)});
  S* p = c + Lc.node(k, j, i, v);
  Store<S, R>::st(p, Store<S, R>::ld(p) + scal(sget<R>(alpha), s));
}

template <typename SV, typename SE, typename R>
__global__ void k_gradient(int n, int m, int K, const double* __restrict__ ph, Sc alpha,
                           const SV* __restrict__ vin, SE* __restrict__ e) {
  // block (m, rows): x = vector, y = site; grid.y = k-point
  int k = blockIdx.y, v = threadIdx.x;
  int site = blockIdx.x * blockDim.y + threadIdx.y;
  if (site >= n * n) return;
  int i = site % n, j = site / n;
  Lay L{n, m, K};
  const SV* vb = vin + L.node(k, 0, 0, v);
  cx<R> gx, gy;
  auto body = [&](const auto& V) {
    cx<R> c = V(i, j);
    gx = V(i + 1, j) - c;
    gy = V(i, j + 1) - c;
  };
  if (i < n - 1 && j < n - 1) body(NAccI<SV, R>{vb, n, m});
  else body(NAcc<SV, R>{vb, n, m, seam_load<R>(ph, K, k, n)});
  R a = sget<R>(alpha);
  SE* px = e + L.edge(k, 0, j, i, v);
  SE* py = e + L.edge(k, 1, j, i, v);
  Store<SE, R>::st(px, Store<SE, R>::ld(px) + scal(a, gx));
  Store<SE, R>::st(py, Store<SE, R>::ld(py) + scal(a, gy));
}

template <typename SE, typename SV, typename R>
__global__ void k_adjgradient(int n, int m, int K, const double* __restrict__ ph, Sc alpha, int mass,
                              Sc sixth, Sc cv, int has_cv, const SE* __restrict__ e, SV* __restrict__ vout) {
  // block (m, rows): x = vector, y = site; grid.y = k-point
  int k = blockIdx.y, v = threadIdx.x;
  int site = blockIdx.x * blockDim.y + threadIdx.y;
  if (site >= n * n) return;
  int i = site % n, j = site / n;
  Lay L{n, m, K};
  const SE* eb = e + L.edge(k, 0, 0, 0, v);
  cx<R> s;
  if (i > 0 && i < n - 1 && j > 0 && j < n - 1) {
    EAccI<SE, R> E{eb, n, m};
    if (mass) {
      R mm = sget<R>(sixth);
      s = mx_x<R>(E, mm, i - 1, j) - mx_x<R>(E, mm, i, j) + mx_y<R>(E, mm, i, j - 1) - mx_y<R>(E, mm, i, j);
    } else {
      s = E(0, i - 1, j) - E(0, i, j) + E(1, i, j - 1) - E(1, i, j);
    }
  } else if (mass) {
    EAcc<SE, R> E{eb, n, m, seam_load<R>(ph, K, k, n)};
    // G^H M e: the mass stencil evaluated at the four edges of the node
    R mm = sget<R>(sixth);
    s = mx_x<R>(E, mm, i - 1, j);
    // the left x-edge value must carry the seam phase of position i-1
    if (i == 0) {
      Seam<R> sm = E.seam;
      cx<R> p = conjc(sm.xf);
      s = p * mx_x<R>(E, mm, n - 1, j);
    }
    cx<R> sy = mx_y<R>(E, mm, i, j - 1);
    if (j == 0) {
      cx<R> p = conjc(E.seam.yf);
      sy = p * mx_y<R>(E, mm, i, n - 1);
    }
    s = s - mx_x<R>(E, mm, i, j) + sy - mx_y<R>(E, mm, i, j);
  } else {
    EAcc<SE, R> E{eb, n, m, seam_load<R>(ph, K, k, n)};
    s = E(0, i - 1, j) - E(0, i, j) + E(1, i, j - 1) - E(1, i, j);
  }
  SV* p = vout + L.node(k, j, i, v);
  cx<R> o = scal(sget<R>(alpha), s);
  if (has_cv) o += scal(sget<R>(cv), Store<SV, R>::ld(p));
  Store<SV, R>::st(p, o);
}

// ------------------------------------------------------------------
// block BLAS-1
// ------------------------------------------------------------------
template <typename SX, typename SY, typename R>
__global__ void k_convert(const SX* __restrict__ x, SY* __restrict__ y, size_t len) {
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (t < len) Store<SY, R>::st(y + t, Store<SX, R>::ld(x + t));
}

template <typename SX, typename SY, typename R>
__global__ void k_axpy(Sc are, Sc aim, const SX* __restrict__ x, SY* __restrict__ y, size_t len) {
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (t < len) {
    cx<R> a = mkc(sget<R>(are), sget<R>(aim));
    Store<SY, R>::st(y + t, Store<SY, R>::ld(y + t) + a * Store<SX, R>::ld(x + t));
  }
}

// mean of each plane of each (k, v), in two passes: partial sums of a chunk
// of sites per block added atomically into acc[(k*2+p)*m+v] (re, im), then
// the subtraction; only k-points whose flag is set are touched
template <typename S> struct CenterAcc { using T = dd; };
template <> struct CenterAcc<double2> { using T = double; };

template <typename S, typename R>
__global__ void k_center_sum(int n, int m, int K, const int* __restrict__ gamma, const S* __restrict__ x,
                             double* acc) {
  int k = blockIdx.y / 2, p = blockIdx.y % 2;
  if (!gamma[k]) return;
  Lay L{n, m, K};
  int v = threadIdx.x, row = threadIdx.y, rows = blockDim.y;
  // float-float sums on the FP32 pipes for c64 and float-float vectors
  // (GB300 adds in FP64 at a small fraction of that rate), FP64 sums for
  // FP64 vectors; FP64 for the block's partial sums
  using A = typename CenterAcc<S>::T;
  A are = Real<A>::zero(), aim = Real<A>::zero();
  for (int s = blockIdx.x * rows + row; s < n * n; s += gridDim.x * rows) {
    cx<A> val = Store<S, A>::ld(x + L.edge(k, p, 0, 0, v) + (size_t) s * m);
    are += val.re;
    aim += val.im;
  }
  __shared__ double sre[256], sim[256];
  int t = threadIdx.y * blockDim.x + threadIdx.x;
  sre[t] = Real<A>::to_double(are);
  sim[t] = Real<A>::to_double(aim);
  __syncthreads();
  if (threadIdx.y == 0) {
    double tr = 0.0, ti = 0.0;
    for (int r = 0; r < rows; r++) { tr += sre[r * blockDim.x + v]; ti += sim[r * blockDim.x + v]; }
    atomicAdd(acc + 2 * ((size_t) (k * 2 + p) * m + v), tr);
    atomicAdd(acc + 2 * ((size_t) (k * 2 + p) * m + v) + 1, ti);
  }
}

template <typename S, typename R>
__global__ void k_center_sub(int n, int m, int K, const int* __restrict__ gamma, const double* __restrict__ acc,
                             S* x) {
  int k = blockIdx.y / 2, p = blockIdx.y % 2;
  if (!gamma[k]) return;
  int v = threadIdx.x;
  int s = blockIdx.x * blockDim.y + threadIdx.y;
  Lay L{n, m, K};
  const double* a = acc + 2 * ((size_t) (k * 2 + p) * m + v);
  // one row of threads forms the block's means (m <= 32), so that the double
  // division and conversion run once per block rather than once per entry
  __shared__ cx<R> mean_s[32];
  if (threadIdx.y == 0) mean_s[v] = cfrom<R>(a[0] / ((double) n * n), a[1] / ((double) n * n));
  __syncthreads();
  if (s >= n * n) return;
  cx<R> mean = mean_s[v];
  S* q = x + L.edge(k, p, 0, 0, v) + (size_t) s * m;
  Store<S, R>::st(q, Store<S, R>::ld(q) - mean);
}

// ------------------------------------------------------------------
// dense coarse matrices: entry (r, c) = row r of the stencil applied to the
// unit vector e_c, which the accessor below presents with its seam phases
// ------------------------------------------------------------------
struct UnitEdge {
  int n, cp, ci, cj;   // plane and site of the unit entry
  Seam<double> seam;
  __device__ cx<double> operator()(int p, int i, int j) const {
    cx<double> ph;
    bool w = seam.wrap(i, j, ph);
    if (p != cp || i != ci || j != cj) return czero<double>();
    return w ? ph : cfrom<double>(1.0, 0.0);
  }
};
struct UnitNode {
  int n, ci, cj;
  Seam<double> seam;
  __device__ cx<double> operator()(int i, int j) const {
    cx<double> ph;
    bool w = seam.wrap(i, j, ph);
    if (i != ci || j != cj) return czero<double>();
    return w ? ph : cfrom<double>(1.0, 0.0);
  }
};

__global__ void k_dense_edge(int n, int K, const double* __restrict__ ph, Kap<double> kap,
                             double alpha, double beta, double* a) {
  int N = 2 * n * n;
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t) N * N * K) return;
  int k = (int) (t / ((size_t) N * N));
  int rc = (int) (t % ((size_t) N * N));
  int row = rc % N, col = rc / N;
  int nn = n * n;
  UnitEdge E{n, col / nn, (col % nn) % n, (col % nn) / n, seam_load<double>(ph, K, k, n)};
  int rp = row / nn, ri = (row % nn) % n, rj = (row % nn) / n;
  double axy = alpha * n * (double) n, mm = beta / 6.0;
  cx<double> val = rp == 0 ? kx_x<double>(E, kap, axy, mm, ri, rj) : kx_y<double>(E, kap, axy, mm, ri, rj);
  double* o = a + 2 * ((size_t) k * N * N + (size_t) col * N + row);
  o[0] = val.re;
  o[1] = val.im;
}

__global__ void k_dense_node(int n, int K, const double* __restrict__ ph, int fixnull, double* a) {
  int N = n * n;
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t) N * N * K) return;
  int k = (int) (t / ((size_t) N * N));
  int rc = (int) (t % ((size_t) N * N));
  int row = rc % N, col = rc / N;
  Seam<double> seam = seam_load<double>(ph, K, k, n);
  UnitNode V{n, col % n, col / n, seam};
  int ri = row % n, rj = row / n;
  cx<double> val = scal(8.0 / 3.0, V(ri, rj)) + scal(-1.0 / 3.0, lap_off<double>(V, ri, rj));
  // node2d.c:1454-1458: at k = 0 every entry gets 0.1/(rows*cols)
  bool gamma = fabs(seam.xf.re - 1.0) + fabs(seam.xf.im) < 1e-8 && fabs(seam.yf.re - 1.0) + fabs(seam.yf.im) < 1e-8;
  if (fixnull && gamma) val.re += 0.1 / ((double) N * N);
  double* o = a + 2 * ((size_t) k * N * N + (size_t) col * N + row);
  o[0] = val.re;
  o[1] = val.im;
}

// per (k, v): out[2*(k*m+v)] += sum_e conj(x) y over `per` entries of the
// [K][per][m] layout (edge: per = 2 n^2, node: per = n^2)
template <typename SX, typename SY, typename R>
__global__ void k_dot(size_t per, int m, const SX* __restrict__ x, const SY* __restrict__ y, double* out) {
  int k = blockIdx.y;
  int v = threadIdx.x % m, row = threadIdx.x / m, rows = blockDim.x / m;
  double re = 0.0, im = 0.0;
  if (row < rows)
    for (size_t e = (size_t) blockIdx.x * rows + row; e < per; e += (size_t) gridDim.x * rows) {
      size_t off = ((size_t) k * per + e) * m + v;
      cx<R> a = Store<SX, R>::ld(x + off), b = Store<SY, R>::ld(y + off);
      cx<R> p = conjc(a) * b;
      re += Real<R>::to_double(p.re);
      im += Real<R>::to_double(p.im);
    }
  __shared__ double sre[256], sim[256];
  sre[threadIdx.x] = re;
  sim[threadIdx.x] = im;
  __syncthreads();
  if (threadIdx.x < m) {
    double tr = 0.0, ti = 0.0;
    for (int r = 0; r < rows; r++) { tr += sre[r * m + threadIdx.x]; ti += sim[r * m + threadIdx.x]; }
    atomicAdd(out + 2 * ((size_t) k * m + threadIdx.x), tr);
    atomicAdd(out + 2 * ((size_t) k * m + threadIdx.x) + 1, ti);
  }
}

}  // namespace

// ------------------------------------------------------------------
// dispatch
// ------------------------------------------------------------------
extern "C" size_t mxk_elem_size(int prec) { return prec == MX_C64 ? 8 : 16; }

// calls F<S, R>(args...) for the storage type of prec with its natural arithmetic
#define MX_BY_PREC(prec, F, ...)                                       \
  ((prec) == MX_C64 ? F<float2, float>(__VA_ARGS__)                    \
   : (prec) == MX_C128 ? F<double2, double>(__VA_ARGS__)               \
   : (prec) == MX_CDD ? F<cdd, dd>(__VA_ARGS__)                        \
   : (int) cudaErrorInvalidValue)

template <typename S, typename R>
static int L_edge_gs_rows(int n, int m, int K, const double* ph, mxk_kappa kap, double alpha,
                          double beta, int j0, int jstep, int nrows, int backward, const void* b,
                          void* x, cudaStream_t st) {
  size_t work = (size_t) nrows * m * K;
  // the tabulated factors serve FP32 sweeps with the scalars they were made for
  const float4* ftab = (sizeof(R) == 4 && kap.afw && kap.afw_alpha == alpha && kap.afw_beta == beta)
                           ? (const float4*) kap.afw : nullptr;
  k_edge_gs_rows<S, R><<<nblocks(work, 64), 64, 0, st>>>(
      n, m, K, ph, make_kap<R>(kap, n), ftab, make_sc(alpha * (double) n * (double) n), make_sc(beta / 6.0),
      make_sc(8.0 * beta / 6.0), make_sc(6.0 / (8.0 * beta)), j0, jstep, nrows, backward, (const S*) b, (S*) x);
  MX_CHECK_LAUNCH();
  return 0;
}
template <typename S, typename R>
static int L_edge_prolong(int nc, int m, int K, const double* ph, double alpha, const void* c, void* f,
                          cudaStream_t st) {
  k_edge_prolong<S, R><<<grd2((size_t) 4 * nc * nc, m, K), blk2(m), 0, st>>>(nc, m, K, ph, make_sc(alpha),
                                                                             (const S*) c, (S*) f);
  MX_CHECK_LAUNCH();
  return 0;
}
template <typename S, typename R>
static int L_edge_restrict(int nc, int m, int K, const double* ph, double alpha, const void* f, void* c,
                           cudaStream_t st) {
  k_edge_restrict<S, R><<<grd2((size_t) nc * nc, m, K), blk2(m), 0, st>>>(nc, m, K, ph, make_sc(alpha),
                                                                          (const S*) f, (S*) c);
  MX_CHECK_LAUNCH();
  return 0;
}
template <typename S, typename R>
static int L_node_apply(int n, int m, int K, const double* ph, double alpha, double cy, const void* x,
                        const void* yin, void* y, cudaStream_t st) {
  k_node_apply<S, R><<<grd2((size_t) ((n + 1) / 2) * n, m, K), blk2(m), 0, st>>>(
      n, m, K, ph, make_sc(alpha * 8.0 / 3.0), make_sc(-alpha / 3.0), make_sc(cy), cy != 0.0, (const S*) x,
      (const S*) yin, (S*) y);
  MX_CHECK_LAUNCH();
  return 0;
}
template <typename S, typename R, int D, int LR>
static int L_node_gs_rows_d(int n, int m, int K, const double* ph, double alpha, int j0, int jstep, int nrows,
                            int backward, const void* b, void* x, cudaStream_t st) {
  const Sc inv_ac = make_sc(3.0 / (8.0 * alpha)), third = make_sc(alpha / 3.0);
  int ring = 1;
  {
    // the single rows 0 and n-1: a CTA per row with the whole row's betas
    // in shared memory, where they fit (the row groups run faster a warp
    // per row: a CTA per row measured 0.96 against 0.87 ms per 512^2 sweep)
    int full = 1;
    while (full < n) full <<= 1;
    const size_t smem = (size_t) (full + 1) * m * sizeof(cx<R>);
    if (m <= 32 && smem <= 96 * 1024 && nrows == 1) {
      if (smem > 48 * 1024)
        cudaFuncSetAttribute(k_node_gs_rowpar<S, R, D, LR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
      k_node_gs_rowpar<S, R, D, LR><<<dim3(nrows, K), blk2(m), smem, st>>>(n, m, K, ph, inv_ac, third, j0, jstep,
                                                                           backward, full - 1, (const S*) b, (S*) x);
      MX_CHECK_LAUNCH();
      return 0;
    }
  }
  if (nrows == 1 || m > 32) {
    // a single row: a CTA of 256 / m position lanes per k-point
    dim3 g(nrows, K), b2 = blk2(m);
    while (ring < 2 * (int) b2.y * LR + D) ring <<= 1;
    size_t smem = (size_t) (ring + 1) * m * sizeof(cx<R>);
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(k_node_gs_row<S, R, D, LR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    k_node_gs_row<S, R, D, LR><<<g, b2, smem, st>>>(n, m, K, ph, inv_ac, third, j0, jstep, backward, ring - 1,
                                                     (const S*) b, (S*) x);
  } else {
    // a row group: a warp per row
    while (ring < (32 / m) * LR + D) ring <<= 1;
    size_t smem = (size_t) 8 * (ring + 1) * m * sizeof(cx<R>);
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(k_node_gs_warp<S, R, D, LR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    k_node_gs_warp<S, R, D, LR><<<dim3((nrows + 7) / 8, K), 256, smem, st>>>(
        n, m, K, ph, inv_ac, third, j0, jstep, nrows, backward, ring - 1, (const S*) b, (S*) x);
  }
  MX_CHECK_LAUNCH();
  return 0;
}
// 8^-(D+1) below the unit roundoff: D = 8 for FP32, 18 for FP64 and float-float
template <typename S, typename R>
static int L_node_gs_rows(int n, int m, int K, const double* ph, double alpha, int j0, int jstep,
                          int nrows, int backward, const void* b, void* x, cudaStream_t st) {
  if constexpr (sizeof(R) == 4)
    return L_node_gs_rows_d<S, R, 8, 7>(n, m, K, ph, alpha, j0, jstep, nrows, backward, b, x, st);
  else
    return L_node_gs_rows_d<S, R, 18, 3>(n, m, K, ph, alpha, j0, jstep, nrows, backward, b, x, st);
}
// The strips pay from 2^25 (coarse node, vector, k-point) triples on
// (the default of g_rr_strips): measured at 32 k-points and 16 vectors,
// 0.757 against 0.813 ms for 256^2 coarse nodes, 0.266 against 0.236 ms for
// 128^2 and several times slower below (a thread's strip is a dependent
// chain; small batches leave too few of them).
static int g_rr_strips = 25;
extern "C" int mxk_node_rr_set_strips(int log2) {
  if (log2 < 0 || log2 > 62) return (int) cudaErrorInvalidValue;
  g_rr_strips = log2;
  return 0;
}
extern "C" int mxk_node_rr_get_strips(void) { return g_rr_strips; }

template <typename S, typename R>
static int L_node_residual_restrict(int nc, int m, int K, const double* ph, double alpha, const void* x,
                                   const void* b, void* c, cudaStream_t st) {
  const Sc diag = make_sc(alpha * 8.0 / 3.0), off = make_sc(-alpha / 3.0);
  if ((size_t) nc * nc * m * K >= ((size_t) 1 << g_rr_strips)) {
    const size_t strips = (size_t) nc * ((nc + RR_CH - 1) / RR_CH);
    k_node_residual_restrict<S, R><<<grd2(strips, m, K), blk2(m), 0, st>>>(nc, m, K, ph, diag, off, (const S*) x,
                                                                         (const S*) b, (S*) c);
  } else {
    k_node_residual_restrict_site<S, R><<<grd2((size_t) nc * nc, m, K), blk2(m), 0, st>>>(
        nc, m, K, ph, diag, off, (const S*) x, (const S*) b, (S*) c);
  }
  MX_CHECK_LAUNCH();
  return 0;
}
template <typename S, typename R>
static int L_node_prolong(int nc, int m, int K, const double* ph, double alpha, const void* c, void* f,
                          cudaStream_t st) {
  k_node_prolong<S, R><<<grd2((size_t) nc * nc, m, K), blk2(m), 0, st>>>(nc, m, K, ph, make_sc(alpha),
                                                                         (const S*) c, (S*) f);
  MX_CHECK_LAUNCH();
  return 0;
}
template <typename S, typename R>
static int L_node_restrict(int nc, int m, int K, const double* ph, double alpha, const void* f, void* c,
                           cudaStream_t st) {
  k_node_restrict<S, R><<<grd2((size_t) nc * nc, m, K), blk2(m), 0, st>>>(nc, m, K, ph, make_sc(alpha),
                                                                          (const S*) f, (S*) c);
  MX_CHECK_LAUNCH();
  return 0;
}
template <typename S, typename R>
static int L_zero(void* x, size_t len, cudaStream_t st) {
  return (int) cudaMemsetAsync(x, 0, len * sizeof(S), st);
}
template <typename S, typename R>
static int L_center(int n, int m, int K, const int* gamma, void* x, double* acc, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(acc, 0, sizeof(double) * 4 * (size_t) K * m, st);
  if (e) return (int) e;
  unsigned chunks = (unsigned) ((n * n + 1023) / 1024);
  k_center_sum<S, R><<<dim3(chunks, 2 * K), blk2(m), 0, st>>>(n, m, K, gamma, (const S*) x, acc);
  MX_CHECK_LAUNCH();
  unsigned rows = 256 / m;
  k_center_sub<S, R><<<dim3((n * n + rows - 1) / rows, 2 * K), blk2(m), 0, st>>>(n, m, K, gamma, acc, (S*) x);
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" size_t mxk_phase_bytes(int K) { return (size_t) K * 4 * sizeof(double) + (size_t) K * 8 * sizeof(float); }

extern "C" void mxk_phase_fill(int K, double* h) {
  float* f = reinterpret_cast<float*>(h + 4 * (size_t) K);
  for (int q = 0; q < 4 * K; q++) {
    Sc c = make_sc(h[q]);
    f[2 * q] = c.hi;
    f[2 * q + 1] = c.lo;
  }
}

extern "C" int mxk_afw_factors(int n, const float* kappa_f, double alpha, double beta, void* out, mx_stream s) {
  size_t nn = (size_t) n * n;
  k_afw_factors<<<nblocks(nn), TPB, 0, (cudaStream_t) s>>>(n, kappa_f, (float) (alpha * (double) n * (double) n),
                                                           (float) (8.0 * beta / 6.0), (float4*) out);
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_edge_apply(int n, int m, int K, const double* ph, mxk_kappa kap, double alpha,
                              double beta, const double* beta_kv, double cy, int px, const void* x,
                              int py, const void* yin, void* y, mx_stream s) {
  dim3 g = grd2((size_t) n * n, m, K), b = blk2(m);
  cudaStream_t st = (cudaStream_t) s;
  Sc axy = make_sc(alpha * (double) n * (double) n), mm = make_sc(beta / 6.0), c = make_sc(cy);
  int has = cy != 0.0;
#define MX_EA(SX, SY, R)                                                                              \
  k_edge_apply<SX, SY, R><<<g, b, 0, st>>>(n, m, K, ph, make_kap<R>(kap, n), axy, mm, beta_kv, c, has, \
                                           (const SX*) x, (const SY*) yin, (SY*) y)
  if (px == MX_C64 && py == MX_C64) MX_EA(float2, float2, float);
  else if (px == MX_C128 && py == MX_C128) MX_EA(double2, double2, double);
  else if (px == MX_CDD && py == MX_CDD) MX_EA(cdd, cdd, dd);
  else if (px == MX_CDD && py == MX_C64) MX_EA(cdd, float2, dd);
  else if (px == MX_C64 && py == MX_CDD) MX_EA(float2, cdd, float);
  else return (int) cudaErrorInvalidValue;
#undef MX_EA
  MX_CHECK_LAUNCH();
  return 0;
}

// The reference's forward order is row 0, even rows 2..n-2, odd rows
// 1..n-3, row n-1 (edge2d.c:2656-2758).  Row 0 commutes with the other even
// rows and row n-1 with the other odd rows (n even), so two phases of
// concurrent rows reproduce it; backward is the exact reverse.
template <typename S, typename R>
static int L_edge_gs_point(int n, int m, int K, const double* ph, mxk_kappa kap, double alpha, double beta,
                           int j0, int backward, const void* b, void* x, cudaStream_t st) {
  size_t work = (size_t) (n / 2) * m * K;
  k_edge_gs_point<S, R><<<nblocks(work, 64), 64, 0, st>>>(n, m, K, ph, make_kap<R>(kap, n),
                                                          make_sc(alpha * (double) n * (double) n),
                                                          make_sc(beta / 6.0), j0, 2, n / 2, backward,
                                                          (const S*) b, (S*) x);
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_edge_gs_point(int n, int m, int K, const double* ph, mxk_kappa kap, double alpha,
                                 double beta, int dir, int prec, const void* b, void* x, mx_stream s) {
  cudaStream_t st = (cudaStream_t) s;
  int e;
  if (n < 2 || (n & 1)) return (int) cudaErrorInvalidValue;
  if (dir == 0 || dir == 2) {
    if ((e = MX_BY_PREC(prec, L_edge_gs_point, n, m, K, ph, kap, alpha, beta, 0, 0, b, x, st))) return e;
    if ((e = MX_BY_PREC(prec, L_edge_gs_point, n, m, K, ph, kap, alpha, beta, 1, 0, b, x, st))) return e;
  }
  if (dir == 1 || dir == 2) {
    if ((e = MX_BY_PREC(prec, L_edge_gs_point, n, m, K, ph, kap, alpha, beta, 1, 1, b, x, st))) return e;
    if ((e = MX_BY_PREC(prec, L_edge_gs_point, n, m, K, ph, kap, alpha, beta, 0, 1, b, x, st))) return e;
  }
  return 0;
}

extern "C" int mxk_edge_gs(int n, int m, int K, const double* ph, mxk_kappa kap, double alpha,
                           double beta, int dir, int prec, const void* b, void* x, mx_stream s) {
  cudaStream_t st = (cudaStream_t) s;
  int e, half = n / 2;
  if (n & 1) return (int) cudaErrorInvalidValue;
  if (dir == 0 || dir == 2) {
    if ((e = MX_BY_PREC(prec, L_edge_gs_rows, n, m, K, ph, kap, alpha, beta, 0, 2, half, 0, b, x, st))) return e;
    if ((e = MX_BY_PREC(prec, L_edge_gs_rows, n, m, K, ph, kap, alpha, beta, 1, 2, half, 0, b, x, st))) return e;
  }
  if (dir == 1 || dir == 2) {
    if ((e = MX_BY_PREC(prec, L_edge_gs_rows, n, m, K, ph, kap, alpha, beta, 1, 2, half, 1, b, x, st))) return e;
    if ((e = MX_BY_PREC(prec, L_edge_gs_rows, n, m, K, ph, kap, alpha, beta, 0, 2, half, 1, b, x, st))) return e;
  }
  return 0;
}

template <typename S, typename R>
static int L_edge_gs_rowpair(int n, int m, int K, const double* ph, mxk_kappa kap, double alpha, double beta,
                             int cj, int rev, const void* b, void* x, cudaStream_t st) {
  const float4* ftab = (sizeof(R) == 4 && kap.afw && kap.afw_alpha == alpha && kap.afw_beta == beta)
                           ? (const float4*) kap.afw : nullptr;
  k_edge_gs_rowpair<S, R><<<dim3(n / 2, K), blk2(m), 0, st>>>(
      n, m, K, ph, make_kap<R>(kap, n), ftab, make_sc(alpha * (double) n * (double) n), make_sc(beta / 6.0),
      make_sc(8.0 * beta / 6.0), make_sc(6.0 / (8.0 * beta)), cj, rev, (const S*) b, (S*) x);
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_edge_gs_colour(int n, int m, int K, const double* ph, mxk_kappa kap, double alpha,
                                  double beta, int dir, int prec, const void* b, void* x, mx_stream s) {
  cudaStream_t st = (cudaStream_t) s;
  int e;
  if (n < 2 || (n & 1) || m < 1 || m > 256) return (int) cudaErrorInvalidValue;
  // forward: colours (0,0), (1,0) in one row-pair launch, then (0,1),
  // (1,1); backward: the four in reverse order
  if (dir == 0 || dir == 2)
    for (int cj = 0; cj < 2; cj++)
      if ((e = MX_BY_PREC(prec, L_edge_gs_rowpair, n, m, K, ph, kap, alpha, beta, cj, 0, b, x, st))) return e;
  if (dir == 1 || dir == 2)
    for (int cj = 1; cj >= 0; cj--)
      if ((e = MX_BY_PREC(prec, L_edge_gs_rowpair, n, m, K, ph, kap, alpha, beta, cj, 1, b, x, st))) return e;
  return 0;
}

extern "C" int mxk_edge_prolong(int nc, int m, int K, const double* ph, double alpha, int prec,
                                const void* c, void* f, mx_stream s) {
  return MX_BY_PREC(prec, L_edge_prolong, nc, m, K, ph, alpha, c, f, (cudaStream_t) s);
}
extern "C" int mxk_edge_restrict(int nc, int m, int K, const double* ph, double alpha, int prec,
                                 const void* f, void* c, mx_stream s) {
  return MX_BY_PREC(prec, L_edge_restrict, nc, m, K, ph, alpha, f, c, (cudaStream_t) s);
}
extern "C" int mxk_node_apply(int n, int m, int K, const double* ph, double alpha, double cy, int prec,
                              const void* x, const void* yin, void* y, mx_stream s) {
  return MX_BY_PREC(prec, L_node_apply, n, m, K, ph, alpha, cy, x, yin, y, (cudaStream_t) s);
}

// Node order (node2d.c:629-1138): forward row 0, odd rows 1..n-3, even rows
// 2..n-2, row n-1, each left to right; backward is the exact reverse.  Rows
// of one group are independent; the four groups run in sequence.
extern "C" int mxk_node_gs(int n, int m, int K, const double* ph, double alpha, int dir, int prec,
                           const void* b, void* x, mx_stream s) {
  cudaStream_t st = (cudaStream_t) s;
  int e;
  if (n < 4 || (n & 1)) return (int) cudaErrorInvalidValue;
  int nodd = (n - 3 - 1) / 2 + 1, neven = (n - 2 - 2) / 2 + 1;
  if (dir == 0 || dir == 2) {
    if ((e = MX_BY_PREC(prec, L_node_gs_rows, n, m, K, ph, alpha, 0, 1, 1, 0, b, x, st))) return e;
    if ((e = MX_BY_PREC(prec, L_node_gs_rows, n, m, K, ph, alpha, 1, 2, nodd, 0, b, x, st))) return e;
    if ((e = MX_BY_PREC(prec, L_node_gs_rows, n, m, K, ph, alpha, 2, 2, neven, 0, b, x, st))) return e;
    if ((e = MX_BY_PREC(prec, L_node_gs_rows, n, m, K, ph, alpha, n - 1, 1, 1, 0, b, x, st))) return e;
  }
  if (dir == 1 || dir == 2) {
    if ((e = MX_BY_PREC(prec, L_node_gs_rows, n, m, K, ph, alpha, n - 1, 1, 1, 1, b, x, st))) return e;
    if ((e = MX_BY_PREC(prec, L_node_gs_rows, n, m, K, ph, alpha, 2, 2, neven, 1, b, x, st))) return e;
    if ((e = MX_BY_PREC(prec, L_node_gs_rows, n, m, K, ph, alpha, 1, 2, nodd, 1, b, x, st))) return e;
    if ((e = MX_BY_PREC(prec, L_node_gs_rows, n, m, K, ph, alpha, 0, 1, 1, 1, b, x, st))) return e;
  }
  return 0;
}

// c = restriction of (b - alpha L x), fine level 2 nc (written, not accumulated)
extern "C" int mxk_node_residual_restrict(int nc, int m, int K, const double* ph, double alpha, int prec,
                                          const void* x, const void* b, void* c, mx_stream s) {
  return MX_BY_PREC(prec, L_node_residual_restrict, nc, m, K, ph, alpha, x, b, c, (cudaStream_t) s);
}

extern "C" int mxk_node_prolong(int nc, int m, int K, const double* ph, double alpha, int prec,
                                const void* c, void* f, mx_stream s) {
  return MX_BY_PREC(prec, L_node_prolong, nc, m, K, ph, alpha, c, f, (cudaStream_t) s);
}
extern "C" int mxk_node_restrict(int nc, int m, int K, const double* ph, double alpha, int prec,
                                 const void* f, void* c, mx_stream s) {
  return MX_BY_PREC(prec, L_node_restrict, nc, m, K, ph, alpha, f, c, (cudaStream_t) s);
}

extern "C" int mxk_gradient(int n, int m, int K, const double* ph, double alpha, int pv, const void* v,
                            int pe, void* e, mx_stream s) {
  dim3 g = grd2((size_t) n * n, m, K), b = blk2(m);
  cudaStream_t st = (cudaStream_t) s;
  Sc a = make_sc(alpha);
#define MX_G(SV, SE, R) k_gradient<SV, SE, R><<<g, b, 0, st>>>(n, m, K, ph, a, (const SV*) v, (SE*) e)
  if (pv == MX_C64 && pe == MX_C64) MX_G(float2, float2, float);
  else if (pv == MX_C128 && pe == MX_C128) MX_G(double2, double2, double);
  else if (pv == MX_C64 && pe == MX_CDD) MX_G(float2, cdd, dd);
  else if (pv == MX_CDD && pe == MX_CDD) MX_G(cdd, cdd, dd);
  else if (pv == MX_C64 && pe == MX_C128) MX_G(float2, double2, double);
  else return (int) cudaErrorInvalidValue;
#undef MX_G
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_adjgradient(int n, int m, int K, const double* ph, double alpha, int mass, double cv,
                               int pe, const void* e, int pv, void* v, mx_stream s) {
  dim3 g = grd2((size_t) n * n, m, K), b = blk2(m);
  cudaStream_t st = (cudaStream_t) s;
  Sc a = make_sc(alpha), sixth = make_sc(1.0 / 6.0), c = make_sc(cv);
  int has = cv != 0.0;
#define MX_AG(SE, SV, R) \
  k_adjgradient<SE, SV, R><<<g, b, 0, st>>>(n, m, K, ph, a, mass, sixth, c, has, (const SE*) e, (SV*) v)
  if (pe == MX_C64 && pv == MX_C64) MX_AG(float2, float2, float);
  else if (pe == MX_C128 && pv == MX_C128) MX_AG(double2, double2, double);
  // G^H M e of a nearly divergence-free eigenvector is a sum with heavy
  // cancellation: it is formed in float-float and only then rounded to c64
  else if (pe == MX_CDD && pv == MX_C64) MX_AG(cdd, float2, dd);
  else if (pe == MX_CDD && pv == MX_CDD) MX_AG(cdd, cdd, dd);
  else if (pe == MX_C128 && pv == MX_C64) MX_AG(double2, float2, double);
  else return (int) cudaErrorInvalidValue;
#undef MX_AG
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_zero(int prec, void* x, size_t len, mx_stream s) {
  return MX_BY_PREC(prec, L_zero, x, len, (cudaStream_t) s);
}

extern "C" int mxk_convert(int px, const void* x, int py, void* y, size_t len, mx_stream s) {
  dim3 g(nblocks(len)), b(TPB);
  cudaStream_t st = (cudaStream_t) s;
  if (px == MX_C128 && py == MX_CDD) k_convert<double2, cdd, dd><<<g, b, 0, st>>>((const double2*) x, (cdd*) y, len);
  else if (px == MX_CDD && py == MX_C128) k_convert<cdd, double2, double><<<g, b, 0, st>>>((const cdd*) x, (double2*) y, len);
  else if (px == MX_C128 && py == MX_C64) k_convert<double2, float2, double><<<g, b, 0, st>>>((const double2*) x, (float2*) y, len);
  else if (px == MX_C64 && py == MX_C128) k_convert<float2, double2, double><<<g, b, 0, st>>>((const float2*) x, (double2*) y, len);
  else if (px == MX_CDD && py == MX_C64) k_convert<cdd, float2, dd><<<g, b, 0, st>>>((const cdd*) x, (float2*) y, len);
  else if (px == MX_C64 && py == MX_CDD) k_convert<float2, cdd, dd><<<g, b, 0, st>>>((const float2*) x, (cdd*) y, len);
  else if (px == py) {
    cudaError_t e = cudaMemcpyAsync(y, x, len * mxk_elem_size(px), cudaMemcpyDeviceToDevice, st);
    return (int) e;
  }
  else return (int) cudaErrorInvalidValue;
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_axpy(double are, double aim, int px, const void* x, int py, void* y, size_t len,
                        mx_stream s) {
  dim3 g(nblocks(len)), b(TPB);
  cudaStream_t st = (cudaStream_t) s;
  Sc ar = make_sc(are), ai = make_sc(aim);
#define MX_AX(SX, SY, R) k_axpy<SX, SY, R><<<g, b, 0, st>>>(ar, ai, (const SX*) x, (SY*) y, len)
  if (px == MX_C64 && py == MX_C64) MX_AX(float2, float2, float);
  else if (px == MX_C128 && py == MX_C128) MX_AX(double2, double2, double);
  else if (px == MX_CDD && py == MX_CDD) MX_AX(cdd, cdd, dd);
  else if (px == MX_C64 && py == MX_CDD) MX_AX(float2, cdd, dd);
  else if (px == MX_C64 && py == MX_C128) MX_AX(float2, double2, double);
  else return (int) cudaErrorInvalidValue;
#undef MX_AX
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_center(int n, int m, int K, const int* gamma, int prec, void* x, double* acc, mx_stream s) {
  if (m > 32) return (int) cudaErrorInvalidValue;
  return MX_BY_PREC(prec, L_center, n, m, K, gamma, x, acc, (cudaStream_t) s);
}

// ------------------------------------------------------------------
// center_edge2d_gpu_noalloc: plane centring for callers that must not
// allocate device memory -- a host application that hands this library a
// fixed memory budget or its own pool, or a loop that cannot afford the
// device-wide synchronisation that cudaMalloc/cudaFree may cause.  The
// kernels are the ones of mxk_center; only their scratch (the plane sums,
// 4 doubles per k-point and vector) lives in the file-scope array below
// instead of device memory allocated per call.  Host code cannot use the
// array's name as a device address, so the first call on each device looks
// the address up with that device current and keeps it.  Every call on a
// device shares the array; L_center clears the sums before accumulating.
// ------------------------------------------------------------------
namespace {
__device__ __align__(256) double g_center_sums[4 * MXG_CENTER_NOALLOC_MAX_KM];
constexpr int kMaxDevices = 64;
std::atomic<double*> g_center_ptr[kMaxDevices];
}  // namespace

extern "C" int center_edge2d_gpu_noalloc(int n, int m, int K, const int* gamma_flag, int prec, void* x,
                                         void* stream) {
  if (n < 2 || m < 1 || m > 32 || K < 1 || (size_t) K * m > MXG_CENTER_NOALLOC_MAX_KM || !gamma_flag || !x
      || (prec != MXG_C64 && prec != MXG_C128 && prec != MXG_CDD))
    return MXG_EINVAL;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int) e;
  if (dev < 0 || dev >= kMaxDevices) return MXG_EINVAL;
  if (stream) {
    // the scratch address below belongs to the current device: a stream of
    // another device is a usage error, not a launch failure
    int sdev = -1;
    e = cudaStreamGetDevice((cudaStream_t) stream, &sdev);
    if (e != cudaSuccess) return (int) e;
    if (sdev != dev) return MXG_EINVAL;
  }
  double* sums = g_center_ptr[dev].load();
  if (!sums) {
    // set-up of this device: the same address whoever gets here first
    e = cudaGetSymbolAddress((void**) &sums, g_center_sums);
    if (e != cudaSuccess) return (int) e;
    g_center_ptr[dev].store(sums);
  }
  return mxk_center(n, m, K, gamma_flag, prec, x, sums, (mx_stream) stream);
}

extern "C" int mxk_dot(size_t per, int m, int K, int px, const void* x, int py, const void* y, double* out,
                       mx_stream s) {
  if (m > 32) return (int) cudaErrorInvalidValue;
  int rows = 256 / m;
  unsigned G = (unsigned) ((per + (size_t) rows * 8 - 1) / ((size_t) rows * 8));
  if (G < 1) G = 1;
  if (G > 2048) G = 2048;
  dim3 g(G, K), b(256);
  cudaStream_t st = (cudaStream_t) s;
  if (px == MX_C64 && py == MX_C64) k_dot<float2, float2, float><<<g, b, 0, st>>>(per, m, (const float2*) x, (const float2*) y, out);
  else if (px == MX_C128 && py == MX_C128) k_dot<double2, double2, double><<<g, b, 0, st>>>(per, m, (const double2*) x, (const double2*) y, out);
  else if (px == MX_CDD && py == MX_CDD) k_dot<cdd, cdd, dd><<<g, b, 0, st>>>(per, m, (const cdd*) x, (const cdd*) y, out);
  else return (int) cudaErrorInvalidValue;
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_dense_edge(int n, int K, const double* ph, mxk_kappa kap, double alpha, double beta,
                              double* a, mx_stream s) {
  size_t N = 2 * (size_t) n * n;
  k_dense_edge<<<nblocks(N * N * K), TPB, 0, (cudaStream_t) s>>>(n, K, ph, make_kap<double>(kap, n), alpha, beta, a);
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_dense_node(int n, int K, const double* ph, int fixnull, double* a, mx_stream s) {
  size_t N = (size_t) n * n;
  k_dense_node<<<nblocks(N * N * K), TPB, 0, (cudaStream_t) s>>>(n, K, ph, fixnull, a);
  MX_CHECK_LAUNCH();
  return 0;
}
