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

using namespace mx;

namespace {

constexpr int TPB = 256;

inline unsigned nblocks(size_t work, int tpb = TPB) {
  size_t b = (work + tpb - 1) / tpb;
  return (unsigned) (b > 0x7fffffff ? 0x7fffffff : b);
}

template <typename R>
__device__ __forceinline__ Seam<R> load_seam(const double* ph, int k, int n) {
  Seam<R> s;
  s.xf = cfrom<R>(ph[4 * k + 0], ph[4 * k + 1]);
  s.yf = cfrom<R>(ph[4 * k + 2], ph[4 * k + 3]);
  s.n = n;
  return s;
}

// kappa of cell (i,j) with periodic wrap, in arithmetic R
template <typename R> struct Kap;
template <> struct Kap<float> {
  const float* p; int n;
  __device__ float operator()(int i, int j) const { return p[wrapi(i, n) + wrapi(j, n) * n]; }
};
template <> struct Kap<double> {
  const double* p; int n;
  __device__ double operator()(int i, int j) const { return p[wrapi(i, n) + wrapi(j, n) * n]; }
};
template <> struct Kap<dd> {
  const float* p; int n;
  __device__ dd operator()(int i, int j) const {
    float2 v = reinterpret_cast<const float2*>(p)[wrapi(i, n) + wrapi(j, n) * n];
    return dd_make(v.x, v.y);
  }
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

template <typename R> __device__ __forceinline__ R rfrom(double d) { return Real<R>::from(d); }

// curl of cell (i,j): bottom - top - left + right
template <typename R, typename A>
__device__ __forceinline__ cx<R> curl(const A& E, int i, int j) {
  return E(0, i, j) - E(0, i, j + 1) - E(1, i, j) + E(1, i + 1, j);
}

// (alpha A + beta M) x at x-edge (i,j) and y-edge (i,j)
template <typename R, typename A>
__device__ __forceinline__ cx<R> kx_x(const A& E, const Kap<R>& kap, R axy, R mm, int i, int j) {
  cx<R> c0 = E(0, i, j);
  cx<R> mass = scal(mm, scal(rfrom<R>(4.0), c0) + E(0, i, j + 1) + E(0, i, j - 1));
  cx<R> cur = scal(kap(i, j), curl<R>(E, i, j)) - scal(kap(i, j - 1), curl<R>(E, i, j - 1));
  return scal(axy, cur) + mass;
}
template <typename R, typename A>
__device__ __forceinline__ cx<R> kx_y(const A& E, const Kap<R>& kap, R axy, R mm, int i, int j) {
  cx<R> c0 = E(1, i, j);
  cx<R> mass = scal(mm, scal(rfrom<R>(4.0), c0) + E(1, i + 1, j) + E(1, i - 1, j));
  cx<R> cur = scal(kap(i - 1, j), curl<R>(E, i - 1, j)) - scal(kap(i, j), curl<R>(E, i, j));
  return scal(axy, cur) + mass;
}
// mass only (no kappa)
template <typename R, typename A>
__device__ __forceinline__ cx<R> mx_x(const A& E, R mm, int i, int j) {
  return scal(mm, scal(rfrom<R>(4.0), E(0, i, j)) + E(0, i, j + 1) + E(0, i, j - 1));
}
template <typename R, typename A>
__device__ __forceinline__ cx<R> mx_y(const A& E, R mm, int i, int j) {
  return scal(mm, scal(rfrom<R>(4.0), E(1, i, j)) + E(1, i + 1, j) + E(1, i - 1, j));
}


// ------------------------------------------------------------------
// edge operator
// ------------------------------------------------------------------
template <typename SX, typename SY, typename R>
__global__ void k_edge_apply(int n, int m, int K, const double* __restrict__ ph, Kap<R> kap,
                             double alpha, double beta, const double* __restrict__ beta_kv,
                             double cy, const SX* __restrict__ x, SY* __restrict__ y) {
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  size_t per_k = (size_t) n * n * m;
  if (t >= per_k * K) return;
  int k = (int) (t / per_k);
  size_t r = t - (size_t) k * per_k;
  int v = (int) (r % m);
  size_t site = r / m;
  int i = (int) (site % n), j = (int) (site / n);
  Lay L{n, m, K};
  EAcc<SX, R> E{x + L.edge(k, 0, 0, 0, v), n, m, load_seam<R>(ph, k, n)};
  R axy = rfrom<R>(alpha * (double) n * (double) n);
  double b = beta_kv ? beta_kv[(size_t) k * m + v] : beta;
  R mm = rfrom<R>(b / 6.0);
  cx<R> ox = kx_x<R>(E, kap, axy, mm, i, j);
  cx<R> oy = kx_y<R>(E, kap, axy, mm, i, j);
  SY* px = y + L.edge(k, 0, j, i, v);
  SY* py = y + L.edge(k, 1, j, i, v);
  if (cy != 0.0) {
    R c = rfrom<R>(cy);
    ox += scal(c, Store<SY, R>::ld(px));
    oy += scal(c, Store<SY, R>::ld(py));
  }
  Store<SY, R>::st(px, ox);
  Store<SY, R>::st(py, oy);
}

// ------------------------------------------------------------------
// AFW vertex-patch line Gauss-Seidel.  One thread owns one (k, row, vector)
// chain and walks its row in the reference's order; rows of one phase touch
// disjoint unknowns (rows j-1..j+1 read, row j of x and rows j-1, j of y
// written), so every row of a phase runs concurrently.
// Local matrix T and its factorisation: see patch_solve in the oracle; the
// reference's starsolve_common (edge2d.c:2029-2183).
// ------------------------------------------------------------------
template <typename S, typename R>
__device__ __forceinline__ void deposit_e(S* base, int n, int m, const Seam<R>& seam, int p, int i,
                                          int j, cx<R> val) {
  cx<R> ph;
  bool w = seam.wrap(i, j, ph);
  if (w) val = conjc(ph) * val;
  S* q = base + ((size_t) (p * n + j) * n + i) * m;
  Store<S, R>::st(q, Store<S, R>::ld(q) + val);
}

template <typename S, typename R>
__global__ void k_edge_gs_rows(int n, int m, int K, const double* __restrict__ ph, Kap<R> kap,
                               double alpha, double beta, int j0, int jstep, int nrows, int backward,
                               const S* __restrict__ b, S* x) {
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  size_t per_k = (size_t) nrows * m;
  if (t >= per_k * K) return;
  int k = (int) (t / per_k);
  int r = (int) (t - (size_t) k * per_k);
  int v = r % m;
  int j = j0 + (r / m) * jstep;
  Lay L{n, m, K};
  Seam<R> seam = load_seam<R>(ph, k, n);
  S* xb = x + L.edge(k, 0, 0, 0, v);
  EAcc<S, R> X{xb, n, m, seam};
  EAcc<S, R> B{b + L.edge(k, 0, 0, 0, v), n, m, seam};
  R axy = rfrom<R>(alpha * (double) n * (double) n);
  R mm = rfrom<R>(beta / 6.0);
  R s8 = rfrom<R>(8.0 * beta / 6.0);   // 4 (mx + my), mx = my
  R quarter = rfrom<R>(0.25);
  for (int step = 0; step < n; step++) {
    int i = backward ? n - 1 - step : step;
    R kLL = axy * kap(i - 1, j - 1), kLR = axy * kap(i, j - 1);
    R kUL = axy * kap(i - 1, j), kUR = axy * kap(i, j);
    // transformed local matrix (mx = my: T10 = T32 = 0)
    R T00 = kUL + kLR + s8, T20 = kUL - kLR;
    R T11 = kLL + kUR, T21 = kLL - kUR;
    R T22 = kLL + kUL + kLR + kUR + s8, T33 = s8;
    // L D L^T with the reference's elimination (no l20 fill in entry (2,2))
    R D0 = T00, l20 = T20 / D0;
    R D1 = T11, l21 = T21 / D1;
    R D2 = T22 - l21 * l21 * D1;
    R D3 = T33;
    cx<R> r0 = B(0, i - 1, j) - kx_x<R>(X, kap, axy, mm, i - 1, j);
    cx<R> r1 = B(0, i, j) - kx_x<R>(X, kap, axy, mm, i, j);
    cx<R> r2 = B(1, i, j - 1) - kx_y<R>(X, kap, axy, mm, i, j - 1);
    cx<R> r3 = B(1, i, j) - kx_y<R>(X, kap, axy, mm, i, j);
    cx<R> c0 = r0 + r1 + r2 + r3;
    cx<R> c1 = r0 + r1 - r2 - r3;
    cx<R> c2 = r0 - r1 - r2 + r3;
    cx<R> c3 = r0 - r1 + r2 - r3;
    c2 -= scal(l20, c0) + scal(l21, c1);
    c0 = scal(rfrom<R>(1.0) / D0, c0);
    c1 = scal(rfrom<R>(1.0) / D1, c1);
    c2 = scal(rfrom<R>(1.0) / D2, c2);
    c3 = scal(rfrom<R>(1.0) / D3, c3);
    c1 -= scal(l21, c2);
    c0 -= scal(l20, c2);
    deposit_e<S, R>(xb, n, m, seam, 0, i - 1, j, scal(quarter, c0 + c1 + c2 + c3));
    deposit_e<S, R>(xb, n, m, seam, 0, i, j, scal(quarter, c0 + c1 - c2 - c3));
    deposit_e<S, R>(xb, n, m, seam, 1, i, j - 1, scal(quarter, c0 - c1 - c2 + c3));
    deposit_e<S, R>(xb, n, m, seam, 1, i, j, scal(quarter, c0 - c1 + c2 - c3));
  }
}

// ------------------------------------------------------------------
// edge transfers (gather form of prolongation_edge2d / restriction_edge2d)
// ------------------------------------------------------------------
template <typename S, typename R>
__global__ void k_edge_prolong(int nc, int m, int K, const double* __restrict__ ph, double alpha,
                               const S* __restrict__ c, S* __restrict__ f) {
  int nf = 2 * nc;
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  size_t per_k = (size_t) nf * nf * m;
  if (t >= per_k * K) return;
  int k = (int) (t / per_k);
  size_t r = t - (size_t) k * per_k;
  int v = (int) (r % m);
  size_t site = r / m;
  int i = (int) (site % nf), j = (int) (site / nf);
  Lay Lc{nc, m, K}, Lf{nf, m, K};
  EAcc<S, R> C{c + Lc.edge(k, 0, 0, 0, v), nc, m, load_seam<R>(ph, k, nc)};
  int ci = i >> 1, cj = j >> 1;
  R half = rfrom<R>(0.5), quarter = rfrom<R>(0.25), a = rfrom<R>(alpha);
  cx<R> vx = (j & 1) ? scal(quarter, C(0, ci, cj) + C(0, ci, cj + 1)) : scal(half, C(0, ci, cj));
  cx<R> vy = (i & 1) ? scal(quarter, C(1, ci, cj) + C(1, ci + 1, cj)) : scal(half, C(1, ci, cj));
  S* px = f + Lf.edge(k, 0, j, i, v);
  S* py = f + Lf.edge(k, 1, j, i, v);
  Store<S, R>::st(px, Store<S, R>::ld(px) + scal(a, vx));
  Store<S, R>::st(py, Store<S, R>::ld(py) + scal(a, vy));
}

template <typename S, typename R>
__global__ void k_edge_restrict(int nc, int m, int K, const double* __restrict__ ph, double alpha,
                                const S* __restrict__ f, S* __restrict__ c) {
  int nf = 2 * nc;
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  size_t per_k = (size_t) nc * nc * m;
  if (t >= per_k * K) return;
  int k = (int) (t / per_k);
  size_t r = t - (size_t) k * per_k;
  int v = (int) (r % m);
  size_t site = r / m;
  int i = (int) (site % nc), j = (int) (site / nc);
  Lay Lc{nc, m, K}, Lf{nf, m, K};
  EAcc<S, R> F{f + Lf.edge(k, 0, 0, 0, v), nf, m, load_seam<R>(ph, k, nf)};
  R half = rfrom<R>(0.5), quarter = rfrom<R>(0.25), a = rfrom<R>(alpha);
  int fi = 2 * i, fj = 2 * j;
  cx<R> sx = scal(half, F(0, fi, fj) + F(0, fi + 1, fj))
             + scal(quarter, F(0, fi, fj - 1) + F(0, fi + 1, fj - 1) + F(0, fi, fj + 1) + F(0, fi + 1, fj + 1));
  cx<R> sy = scal(half, F(1, fi, fj) + F(1, fi, fj + 1))
             + scal(quarter, F(1, fi - 1, fj) + F(1, fi - 1, fj + 1) + F(1, fi + 1, fj) + F(1, fi + 1, fj + 1));
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

template <typename S, typename R>
__global__ void k_node_apply(int n, int m, int K, const double* __restrict__ ph, double alpha,
                             double cy, const S* __restrict__ x, S* __restrict__ y) {
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  size_t per_k = (size_t) n * n * m;
  if (t >= per_k * K) return;
  int k = (int) (t / per_k);
  size_t r = t - (size_t) k * per_k;
  int v = (int) (r % m);
  size_t site = r / m;
  int i = (int) (site % n), j = (int) (site / n);
  Lay L{n, m, K};
  NAcc<S, R> V{x + L.node(k, 0, 0, v), n, m, load_seam<R>(ph, k, n)};
  cx<R> o = scal(rfrom<R>(alpha * 8.0 / 3.0), V(i, j)) + scal(rfrom<R>(-alpha / 3.0), lap_off<R>(V, i, j));
  S* py = y + L.node(k, j, i, v);
  if (cy != 0.0) o += scal(rfrom<R>(cy), Store<S, R>::ld(py));
  Store<S, R>::st(py, o);
}

template <typename S, typename R>
__global__ void k_node_gs_rows(int n, int m, int K, const double* __restrict__ ph, double alpha,
                               int j0, int jstep, int nrows, int backward, const S* __restrict__ b,
                               S* x) {
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  size_t per_k = (size_t) nrows * m;
  if (t >= per_k * K) return;
  int k = (int) (t / per_k);
  int r = (int) (t - (size_t) k * per_k);
  int v = r % m;
  int j = j0 + (r / m) * jstep;
  Lay L{n, m, K};
  S* xb = x + L.node(k, 0, 0, v);
  NAcc<S, R> V{xb, n, m, load_seam<R>(ph, k, n)};
  const S* bb = b + L.node(k, 0, 0, v);
  R inv_ac = rfrom<R>(3.0 / (8.0 * alpha));
  R ao = rfrom<R>(-alpha / 3.0);
  for (int step = 0; step < n; step++) {
    int i = backward ? n - 1 - step : step;
    cx<R> rhs = Store<S, R>::ld(bb + ((size_t) j * n + i) * m) - scal(ao, lap_off<R>(V, i, j));
    Store<S, R>::st(xb + ((size_t) j * n + i) * m, scal(inv_ac, rhs));
  }
}

template <typename S, typename R>
__global__ void k_node_prolong(int nc, int m, int K, const double* __restrict__ ph, double alpha,
                               const S* __restrict__ c, S* __restrict__ f) {
  int nf = 2 * nc;
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  size_t per_k = (size_t) nf * nf * m;
  if (t >= per_k * K) return;
  int k = (int) (t / per_k);
  size_t r = t - (size_t) k * per_k;
  int v = (int) (r % m);
  size_t site = r / m;
  int i = (int) (site % nf), j = (int) (site / nf);
  Lay Lc{nc, m, K}, Lf{nf, m, K};
  NAcc<S, R> C{c + Lc.node(k, 0, 0, v), nc, m, load_seam<R>(ph, k, nc)};
  int ci = i >> 1, cj = j >> 1, oi = i & 1, oj = j & 1;
  cx<R> val = C(ci, cj);
  if (oi) val += C(ci + 1, cj);
  if (oj) val += C(ci, cj + 1);
  if (oi && oj) val += C(ci + 1, cj + 1);
  double w = alpha * (oi ? 0.5 : 1.0) * (oj ? 0.5 : 1.0);
  S* p = f + Lf.node(k, j, i, v);
  Store<S, R>::st(p, Store<S, R>::ld(p) + scal(rfrom<R>(w), val));
}

template <typename S, typename R>
__global__ void k_node_restrict(int nc, int m, int K, const double* __restrict__ ph, double alpha,
                                const S* __restrict__ f, S* __restrict__ c) {
  int nf = 2 * nc;
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  size_t per_k = (size_t) nc * nc * m;
  if (t >= per_k * K) return;
  int k = (int) (t / per_k);
  size_t r = t - (size_t) k * per_k;
  int v = (int) (r % m);
  size_t site = r / m;
  int i = (int) (site % nc), j = (int) (site / nc);
  Lay Lc{nc, m, K}, Lf{nf, m, K};
  NAcc<S, R> F{f + Lf.node(k, 0, 0, v), nf, m, load_seam<R>(ph, k, nf)};
  int fi = 2 * i, fj = 2 * j;
  cx<R> s = F(fi, fj)
            + scal(rfrom<R>(0.5), F(fi - 1, fj) + F(fi + 1, fj) + F(fi, fj - 1) + F(fi, fj + 1))
            + scal(rfrom<R>(0.25), F(fi - 1, fj - 1) + F(fi + 1, fj - 1) + F(fi - 1, fj + 1) + F(fi + 1, fj + 1));
  S* p = c + Lc.node(k, j, i, v);
  Store<S, R>::st(p, Store<S, R>::ld(p) + scal(rfrom<R>(alpha), s));
}

template <typename SV, typename SE, typename R>
__global__ void k_gradient(int n, int m, int K, const double* __restrict__ ph, double alpha,
                           const SV* __restrict__ vin, SE* __restrict__ e) {
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  size_t per_k = (size_t) n * n * m;
  if (t >= per_k * K) return;
  int k = (int) (t / per_k);
  size_t r = t - (size_t) k * per_k;
  int v = (int) (r % m);
  size_t site = r / m;
  int i = (int) (site % n), j = (int) (site / n);
  Lay L{n, m, K};
  NAcc<SV, R> V{vin + L.node(k, 0, 0, v), n, m, load_seam<R>(ph, k, n)};
  cx<R> c = V(i, j);
  R a = rfrom<R>(alpha);
  SE* px = e + L.edge(k, 0, j, i, v);
  SE* py = e + L.edge(k, 1, j, i, v);
  Store<SE, R>::st(px, Store<SE, R>::ld(px) + scal(a, V(i + 1, j) - c));
  Store<SE, R>::st(py, Store<SE, R>::ld(py) + scal(a, V(i, j + 1) - c));
}

template <typename SE, typename SV, typename R>
__global__ void k_adjgradient(int n, int m, int K, const double* __restrict__ ph, double alpha,
                              int mass, double cv, const SE* __restrict__ e, SV* __restrict__ vout) {
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  size_t per_k = (size_t) n * n * m;
  if (t >= per_k * K) return;
  int k = (int) (t / per_k);
  size_t r = t - (size_t) k * per_k;
  int v = (int) (r % m);
  size_t site = r / m;
  int i = (int) (site % n), j = (int) (site / n);
  Lay L{n, m, K};
  EAcc<SE, R> E{e + L.edge(k, 0, 0, 0, v), n, m, load_seam<R>(ph, k, n)};
  cx<R> s;
  if (mass) {
    // G^H M e: the mass stencil evaluated at the four edges of the node
    R mm = rfrom<R>(1.0 / 6.0);
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
    s = E(0, i - 1, j) - E(0, i, j) + E(1, i, j - 1) - E(1, i, j);
  }
  SV* p = vout + L.node(k, j, i, v);
  cx<R> o = scal(rfrom<R>(alpha), s);
  if (cv != 0.0) o += scal(rfrom<R>(cv), Store<SV, R>::ld(p));
  Store<SV, R>::st(p, o);
}

// ------------------------------------------------------------------
// block BLAS-1
// ------------------------------------------------------------------
template <typename S>
__global__ void k_zero(S* x, size_t len) {
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (t < len) memset(x + t, 0, sizeof(S));
}

template <typename SX, typename SY, typename R>
__global__ void k_convert(const SX* __restrict__ x, SY* __restrict__ y, size_t len) {
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (t < len) Store<SY, R>::st(y + t, Store<SX, R>::ld(x + t));
}

template <typename SX, typename SY, typename R>
__global__ void k_axpy(double are, double aim, const SX* __restrict__ x, SY* __restrict__ y, size_t len) {
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (t < len) {
    cx<R> a = cfrom<R>(are, aim);
    Store<SY, R>::st(y + t, Store<SY, R>::ld(y + t) + a * Store<SX, R>::ld(x + t));
  }
}

// mean of each plane of each (k, v): one block per (k, plane), m <= 32 lanes of v
template <typename S, typename R>
__global__ void k_center(int n, int m, int K, const int* __restrict__ gamma, S* x) {
  int k = blockIdx.x / 2, p = blockIdx.x % 2;
  if (!gamma[k]) return;
  Lay L{n, m, K};
  __shared__ double sre[256], sim[256];
  int v = threadIdx.x % m, row = threadIdx.x / m, rows = blockDim.x / m;
  double are = 0.0, aim = 0.0;
  if (row < rows) {
    for (size_t s = row; s < (size_t) n * n; s += rows) {
      cx<R> val = Store<S, R>::ld(x + L.edge(k, p, 0, 0, v) + s * m);
      are += Real<R>::to_double(val.re);
      aim += Real<R>::to_double(val.im);
    }
  }
  sre[threadIdx.x] = are;
  sim[threadIdx.x] = aim;
  __syncthreads();
  if (threadIdx.x < m) {
    double tr = 0.0, ti = 0.0;
    for (int q = threadIdx.x; q < rows * m; q += m) { tr += sre[q]; ti += sim[q]; }
    sre[threadIdx.x] = tr / ((double) n * n);
    sim[threadIdx.x] = ti / ((double) n * n);
  }
  __syncthreads();
  cx<R> mean = cfrom<R>(sre[v], sim[v]);
  if (row < rows)
    for (size_t s = row; s < (size_t) n * n; s += rows) {
      S* q = x + L.edge(k, p, 0, 0, v) + s * m;
      Store<S, R>::st(q, Store<S, R>::ld(q) - mean);
    }
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
  UnitEdge E{n, col / nn, (col % nn) % n, (col % nn) / n, load_seam<double>(ph, k, n)};
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
  Seam<double> seam = load_seam<double>(ph, k, n);
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
  k_edge_gs_rows<S, R><<<nblocks(work, 64), 64, 0, st>>>(n, m, K, ph, make_kap<R>(kap, n), alpha, beta,
                                                         j0, jstep, nrows, backward, (const S*) b, (S*) x);
  MX_CHECK_LAUNCH();
  return 0;
}
template <typename S, typename R>
static int L_edge_prolong(int nc, int m, int K, const double* ph, double alpha, const void* c, void* f,
                          cudaStream_t st) {
  k_edge_prolong<S, R><<<nblocks((size_t) 4 * nc * nc * m * K), TPB, 0, st>>>(nc, m, K, ph, alpha, (const S*) c, (S*) f);
  MX_CHECK_LAUNCH();
  return 0;
}
template <typename S, typename R>
static int L_edge_restrict(int nc, int m, int K, const double* ph, double alpha, const void* f, void* c,
                           cudaStream_t st) {
  k_edge_restrict<S, R><<<nblocks((size_t) nc * nc * m * K), TPB, 0, st>>>(nc, m, K, ph, alpha, (const S*) f, (S*) c);
  MX_CHECK_LAUNCH();
  return 0;
}
template <typename S, typename R>
static int L_node_apply(int n, int m, int K, const double* ph, double alpha, double cy, const void* x,
                        void* y, cudaStream_t st) {
  k_node_apply<S, R><<<nblocks((size_t) n * n * m * K), TPB, 0, st>>>(n, m, K, ph, alpha, cy, (const S*) x, (S*) y);
  MX_CHECK_LAUNCH();
  return 0;
}
template <typename S, typename R>
static int L_node_gs_rows(int n, int m, int K, const double* ph, double alpha, int j0, int jstep,
                          int nrows, int backward, const void* b, void* x, cudaStream_t st) {
  k_node_gs_rows<S, R><<<nblocks((size_t) nrows * m * K, 64), 64, 0, st>>>(n, m, K, ph, alpha, j0, jstep, nrows,
                                                                          backward, (const S*) b, (S*) x);
  MX_CHECK_LAUNCH();
  return 0;
}
template <typename S, typename R>
static int L_node_prolong(int nc, int m, int K, const double* ph, double alpha, const void* c, void* f,
                          cudaStream_t st) {
  k_node_prolong<S, R><<<nblocks((size_t) 4 * nc * nc * m * K), TPB, 0, st>>>(nc, m, K, ph, alpha, (const S*) c, (S*) f);
  MX_CHECK_LAUNCH();
  return 0;
}
template <typename S, typename R>
static int L_node_restrict(int nc, int m, int K, const double* ph, double alpha, const void* f, void* c,
                           cudaStream_t st) {
  k_node_restrict<S, R><<<nblocks((size_t) nc * nc * m * K), TPB, 0, st>>>(nc, m, K, ph, alpha, (const S*) f, (S*) c);
  MX_CHECK_LAUNCH();
  return 0;
}
template <typename S, typename R>
static int L_zero(void* x, size_t len, cudaStream_t st) {
  k_zero<S><<<nblocks(len), TPB, 0, st>>>((S*) x, len);
  MX_CHECK_LAUNCH();
  return 0;
}
template <typename S, typename R>
static int L_center(int n, int m, int K, const int* gamma, void* x, cudaStream_t st) {
  int threads = (256 / m) * m;
  k_center<S, R><<<2 * K, threads, 0, st>>>(n, m, K, gamma, (S*) x);
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_edge_apply(int n, int m, int K, const double* ph, mxk_kappa kap, double alpha,
                              double beta, const double* beta_kv, double cy, int px, const void* x,
                              int py, void* y, mx_stream s) {
  dim3 g(nblocks((size_t) n * n * m * K)), b(TPB);
  cudaStream_t st = (cudaStream_t) s;
  if (px == MX_C64 && py == MX_C64)
    k_edge_apply<float2, float2, float><<<g, b, 0, st>>>(n, m, K, ph, make_kap<float>(kap, n), alpha, beta, beta_kv, cy, (const float2*) x, (float2*) y);
  else if (px == MX_C128 && py == MX_C128)
    k_edge_apply<double2, double2, double><<<g, b, 0, st>>>(n, m, K, ph, make_kap<double>(kap, n), alpha, beta, beta_kv, cy, (const double2*) x, (double2*) y);
  else if (px == MX_CDD && py == MX_CDD)
    k_edge_apply<cdd, cdd, dd><<<g, b, 0, st>>>(n, m, K, ph, make_kap<dd>(kap, n), alpha, beta, beta_kv, cy, (const cdd*) x, (cdd*) y);
  else if (px == MX_CDD && py == MX_C64)
    k_edge_apply<cdd, float2, dd><<<g, b, 0, st>>>(n, m, K, ph, make_kap<dd>(kap, n), alpha, beta, beta_kv, cy, (const cdd*) x, (float2*) y);
  else if (px == MX_C64 && py == MX_CDD)
    k_edge_apply<float2, cdd, float><<<g, b, 0, st>>>(n, m, K, ph, make_kap<float>(kap, n), alpha, beta, beta_kv, cy, (const float2*) x, (cdd*) y);
  else
    return (int) cudaErrorInvalidValue;
  MX_CHECK_LAUNCH();
  return 0;
}

// The reference's forward order is row 0, even rows 2..n-2, odd rows
// 1..n-3, row n-1 (edge2d.c:2656-2758).  Row 0 commutes with the other even
// rows and row n-1 with the other odd rows (n even), so two phases of
// concurrent rows reproduce it; backward is the exact reverse.
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

extern "C" int mxk_edge_prolong(int nc, int m, int K, const double* ph, double alpha, int prec,
                                const void* c, void* f, mx_stream s) {
  return MX_BY_PREC(prec, L_edge_prolong, nc, m, K, ph, alpha, c, f, (cudaStream_t) s);
}
extern "C" int mxk_edge_restrict(int nc, int m, int K, const double* ph, double alpha, int prec,
                                 const void* f, void* c, mx_stream s) {
  return MX_BY_PREC(prec, L_edge_restrict, nc, m, K, ph, alpha, f, c, (cudaStream_t) s);
}
extern "C" int mxk_node_apply(int n, int m, int K, const double* ph, double alpha, double cy, int prec,
                              const void* x, void* y, mx_stream s) {
  return MX_BY_PREC(prec, L_node_apply, n, m, K, ph, alpha, cy, x, y, (cudaStream_t) s);
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
  dim3 g(nblocks((size_t) n * n * m * K)), b(TPB);
  cudaStream_t st = (cudaStream_t) s;
  if (pv == MX_C64 && pe == MX_C64)
    k_gradient<float2, float2, float><<<g, b, 0, st>>>(n, m, K, ph, alpha, (const float2*) v, (float2*) e);
  else if (pv == MX_C128 && pe == MX_C128)
    k_gradient<double2, double2, double><<<g, b, 0, st>>>(n, m, K, ph, alpha, (const double2*) v, (double2*) e);
  else if (pv == MX_C64 && pe == MX_CDD)
    k_gradient<float2, cdd, dd><<<g, b, 0, st>>>(n, m, K, ph, alpha, (const float2*) v, (cdd*) e);
  else if (pv == MX_CDD && pe == MX_CDD)
    k_gradient<cdd, cdd, dd><<<g, b, 0, st>>>(n, m, K, ph, alpha, (const cdd*) v, (cdd*) e);
  else
    return (int) cudaErrorInvalidValue;
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_adjgradient(int n, int m, int K, const double* ph, double alpha, int mass, double cv,
                               int pe, const void* e, int pv, void* v, mx_stream s) {
  dim3 g(nblocks((size_t) n * n * m * K)), b(TPB);
  cudaStream_t st = (cudaStream_t) s;
  if (pe == MX_C64 && pv == MX_C64)
    k_adjgradient<float2, float2, float><<<g, b, 0, st>>>(n, m, K, ph, alpha, mass, cv, (const float2*) e, (float2*) v);
  else if (pe == MX_C128 && pv == MX_C128)
    k_adjgradient<double2, double2, double><<<g, b, 0, st>>>(n, m, K, ph, alpha, mass, cv, (const double2*) e, (double2*) v);
  else if (pe == MX_CDD && pv == MX_C64)
    k_adjgradient<cdd, float2, dd><<<g, b, 0, st>>>(n, m, K, ph, alpha, mass, cv, (const cdd*) e, (float2*) v);
  else if (pe == MX_CDD && pv == MX_CDD)
    k_adjgradient<cdd, cdd, dd><<<g, b, 0, st>>>(n, m, K, ph, alpha, mass, cv, (const cdd*) e, (cdd*) v);
  else
    return (int) cudaErrorInvalidValue;
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
  if (px == MX_C64 && py == MX_C64) k_axpy<float2, float2, float><<<g, b, 0, st>>>(are, aim, (const float2*) x, (float2*) y, len);
  else if (px == MX_C128 && py == MX_C128) k_axpy<double2, double2, double><<<g, b, 0, st>>>(are, aim, (const double2*) x, (double2*) y, len);
  else if (px == MX_CDD && py == MX_CDD) k_axpy<cdd, cdd, dd><<<g, b, 0, st>>>(are, aim, (const cdd*) x, (cdd*) y, len);
  else if (px == MX_C64 && py == MX_CDD) k_axpy<float2, cdd, dd><<<g, b, 0, st>>>(are, aim, (const float2*) x, (cdd*) y, len);
  else if (px == MX_C64 && py == MX_C128) k_axpy<float2, double2, double><<<g, b, 0, st>>>(are, aim, (const float2*) x, (double2*) y, len);
  else return (int) cudaErrorInvalidValue;
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_center(int n, int m, int K, const int* gamma, int prec, void* x, mx_stream s) {
  if (m > 32) return (int) cudaErrorInvalidValue;
  return MX_BY_PREC(prec, L_center, n, m, K, gamma, x, (cudaStream_t) s);
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
