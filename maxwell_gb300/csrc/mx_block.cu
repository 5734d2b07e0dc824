// Eigenvector-block kernels of the Ritz step (exp_bloch2d.c:956-1053,
// test_lobpcg2d.c:217-365) batched over k-points:
//   residual / Rayleigh statistics  (defects of exp_bloch2d.c:1012-1018)
//   Gram matrices S^H (A+M) S, S^H M S   (energyprod/massprod, edge2d.c:1652-2027)
//   block linear combination E = S C     (the add_edge2d loops, exp_bloch2d.c:1006-1010)
//   permittivity sensitivity of eigenvalues
//
// Precision: the eigenvector block E is stored as float-float (cdd) in the
// mixed solver and as c128 in the plain FP64 solver; the search blocks X, P
// are c64 (mixed) or c128 (plain).  Everything that decides eigenvalue
// accuracy (the residual, e^H (A+M) e, e^H M e and the E-E Gram block) is
// computed in float-float or FP64; the Gram entries that involve X or P only
// steer the subspace and are computed in FP32 in the mixed solver.
//
// The Gram uses the cell form of the operator: S^H A S = sum over cells of
// axy*kappa_c * curl_c(S)^H curl_c(S), which avoids the cancellation of
// forming A S first, plus the edge form of the mass matrix.
#include "mx_common.cuh"
#include "mx_internal.h"

using namespace mx;

// ------------------------------------------------------------------
// launch shapes that mxg_autotune chooses (process-wide; the defaults are
// the shapes measured best on the 512^2, 32-k-point, block-16 workload)
// ------------------------------------------------------------------
static mxk_tuning g_tuning = {4, 2, 32};
static int g_sms = 0;

static int sm_count() {
  if (!g_sms) {
    int dev = 0, c = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && c > 0)
      g_sms = c;
    else
      g_sms = 152;
  }
  return g_sms;
}

extern "C" void mxk_get_tuning(mxk_tuning* t) { *t = g_tuning; }
extern "C" int mxk_set_tuning(const mxk_tuning* t) {
  if (t->gram_waves < 1 || t->gram_waves > 64 || t->combine_ctas < 1 || t->combine_ctas > 16 ||
      t->residual_sites < 1 || t->residual_sites > 1024)
    return (int) cudaErrorInvalidValue;
  g_tuning = *t;
  return 0;
}

namespace {


template <typename S, typename R>
struct EA {
  const S* base;
  int n, m;
  Seam<R> seam;
  __device__ __forceinline__ cx<R> operator()(int p, int i, int j) const {
    cx<R> ph;
    bool w = seam.wrap(i, j, ph);
    cx<R> v = Store<S, R>::ld(base + ((size_t) (p * n + j) * n + i) * m);
    return w ? ph * v : v;
  }
};
// the same for stencils inside the unit cell: no seam test, 32-bit offsets
template <typename S, typename R>
struct EAI {
  const S* base;
  int n, m;
  __device__ __forceinline__ cx<R> operator()(int p, int i, int j) const {
    return Store<S, R>::ld(base + ((p * n + j) * n + i) * m);
  }
};


template <typename R> struct KapB;
template <> struct KapB<float> {
  const float* p; int n;
  __device__ float at(int c) const { return p[c]; }
  __device__ float operator()(int i, int j) const { return p[wrapi(i, n) + wrapi(j, n) * n]; }
};
template <> struct KapB<double> {
  const double* p; int n;
  __device__ double at(int c) const { return p[c]; }
  __device__ double operator()(int i, int j) const { return p[wrapi(i, n) + wrapi(j, n) * n]; }
};
template <> struct KapB<dd> {
  const float* p; int n;
  __device__ dd at(int c) const {
    float2 v = reinterpret_cast<const float2*>(p)[c];
    return dd_make(v.x, v.y);
  }
  __device__ dd operator()(int i, int j) const { return at(wrapi(i, n) + wrapi(j, n) * n); }
};
template <typename R> struct KapBI {
  KapB<R> k;
  __device__ __forceinline__ R operator()(int i, int j) const { return k.at(i + j * k.n); }
};
template <typename R> KapB<R> kapb(mxk_kappa k, int n);
template <> KapB<float> kapb<float>(mxk_kappa k, int n) { KapB<float> r; r.p = k.f; r.n = n; return r; }
template <> KapB<double> kapb<double>(mxk_kappa k, int n) { KapB<double> r; r.p = k.d; r.n = n; return r; }
template <> KapB<dd> kapb<dd>(mxk_kappa k, int n) { KapB<dd> r; r.p = k.dd; r.n = n; return r; }

template <typename R, typename A>
__device__ __forceinline__ cx<R> curlc(const A& E, int i, int j) {
  return E(0, i, j) - E(0, i, j + 1) - E(1, i, j) + E(1, i + 1, j);
}

// s + c += a*b for float-float a = (ah, al), b = (bh, bl), dropping al*bl
__device__ __forceinline__ void comp_mac(float& s, float& c, float ah, float al, float bh, float bl) {
  float p = ah * bh;
  float x = fmaf(ah, bl, fmaf(al, bh, fmaf(ah, bh, -p)));
  float t = s + p;
  float bp = t - s;
  c += ((s - (t - bp)) + (p - bp)) + x;
  s = t;
}
// (re, im) += conj(a) * b for float-float complex a, b
__device__ __forceinline__ void comp_cmac(float* acc, const cx<dd>& a, const cx<dd>& b) {
  comp_mac(acc[0], acc[1], a.re.hi, a.re.lo, b.re.hi, b.re.lo);
  comp_mac(acc[0], acc[1], a.im.hi, a.im.lo, b.im.hi, b.im.lo);
  comp_mac(acc[2], acc[3], a.re.hi, a.re.lo, b.im.hi, b.im.lo);
  comp_mac(acc[2], acc[3], -a.im.hi, -a.im.lo, b.re.hi, b.re.lo);
}

// ------------------------------------------------------------------
// residual and Rayleigh statistics
// ------------------------------------------------------------------
constexpr int NSTAT = 5;

template <typename R> struct LoAcc { using T = R; };
template <> struct LoAcc<dd> { using T = float; };
__device__ __forceinline__ cx<float> lo_c(cx<dd> a) { return mkc(a.re.hi, a.im.hi); }
__device__ __forceinline__ cx<float> lo_c(cx<float> a) { return a; }
__device__ __forceinline__ cx<double> lo_c(cx<double> a) { return a; }

template <typename SE, typename SR, typename R>
__global__ void k_block_residual(int n, int m, int K, const double* __restrict__ ph, KapB<R> kap, Sc axy_s,
                                 Sc sixth, const double* __restrict__ mu, const SE* __restrict__ e,
                                 SR* __restrict__ rout, double* __restrict__ stats) {
  // block: m lanes (v) x rows; grid (G, K)
  int k = blockIdx.y;
  int v = threadIdx.x % m, row = threadIdx.x / m, rows = blockDim.x / m;
  Lay L{n, m, K};
  EA<SE, R> E{e + L.edge(k, 0, 0, 0, v), n, m, seam_load<R>(ph, K, k, n)};
  R axy = sget<R>(axy_s), mm = sget<R>(sixth);
  // the shift of each column, converted once per block
  __shared__ R mu_s[32];
  if (threadIdx.x < m) mu_s[threadIdx.x] = Real<R>::from(mu[(size_t) k * m + threadIdx.x]);
  __syncthreads();
  R muv = mu_s[v];
  R four = rc<R>(4.0f);
  // the Rayleigh quotient's sums in R; the norms and the imaginary check
  // need a few digits only and take the leading float of a float-float value
  using RL = typename LoAcc<R>::T;
  R s_ew = Real<R>::zero(), s_ev = Real<R>::zero();
  RL s_r2 = 0, s_v2 = 0, s_ewi = 0;
  size_t nsite = (size_t) n * n;
  if (row < rows) {
    for (int site = blockIdx.x * rows + row; site < (int) nsite; site += gridDim.x * rows) {
      int i = site % n, j = site / n;
      cx<R> x0, y0, vx, vy, wx, wy;
      auto body = [&](const auto& A, const auto& KA) {
        cx<R> cc = curlc<R>(A, i, j);
        cx<R> cb = curlc<R>(A, i, j - 1);
        cx<R> cl = curlc<R>(A, i - 1, j);
        x0 = A(0, i, j);
        y0 = A(1, i, j);
        vx = scal(mm, scal(four, x0) + A(0, i, j + 1) + A(0, i, j - 1));
        vy = scal(mm, scal(four, y0) + A(1, i + 1, j) + A(1, i - 1, j));
        wx = scal(axy, scal(KA(i, j), cc) - scal(KA(i, j - 1), cb)) + vx;
        wy = scal(axy, scal(KA(i - 1, j), cl) - scal(KA(i, j), cc)) + vy;
      };
      if (i > 0 && i < n - 1 && j > 0 && j < n - 1) body(EAI<SE, R>{E.base, n, m}, KapBI<R>{kap});
      else body(E, kap);
      cx<R> rx = wx - scal(muv, vx), ry = wy - scal(muv, vy);
      if (rout) {
        Store<SR, R>::st(rout + L.edge(k, 0, j, i, v), rx);
        Store<SR, R>::st(rout + L.edge(k, 1, j, i, v), ry);
      }
      {
        const cx<RL> lx = lo_c(rx), ly = lo_c(ry), px = lo_c(vx), py = lo_c(vy), ex = lo_c(x0), ey = lo_c(y0),
                     qx = lo_c(wx), qy = lo_c(wy);
        s_r2 += lx.re * lx.re + lx.im * lx.im + ly.re * ly.re + ly.im * ly.im;
        s_v2 += px.re * px.re + px.im * px.im + py.re * py.re + py.im * py.im;
        s_ewi += ex.re * qx.im - ex.im * qx.re + ey.re * qy.im - ey.im * qy.re;
      }
      s_ew += x0.re * wx.re + x0.im * wx.im + y0.re * wy.re + y0.im * wy.im;
      s_ev += x0.re * vx.re + x0.im * vx.im + y0.re * vy.re + y0.im * vy.im;
    }
  }
  __shared__ double sh[NSTAT][256];
  sh[0][threadIdx.x] = (double) s_r2;
  sh[1][threadIdx.x] = (double) s_v2;
  sh[2][threadIdx.x] = Real<R>::to_double(s_ew);
  sh[3][threadIdx.x] = Real<R>::to_double(s_ev);
  sh[4][threadIdx.x] = (double) s_ewi;
  __syncthreads();
  if (threadIdx.x < m * NSTAT) {
    int q = threadIdx.x / m, vv = threadIdx.x % m;
    double t = 0.0;
    for (int r = 0; r < rows; r++) t += sh[q][r * m + vv];
    atomicAdd(stats + ((size_t) k * m + vv) * NSTAT + q, t);
  }
}

// ------------------------------------------------------------------
// Gram matrices.  One CTA handles a chunk of sites of one k.  Per tile of
// TS sites it stages, for every basis column, the cell curl, the x and y
// edge values and the mass stencil at those edges; then every thread
// accumulates its share of the lower-triangle entries.  Partial sums per CTA
// go to scratch and a second kernel adds them in a fixed order.
// Columns of the first block are "high" (float-float or FP64): entries with
// both columns high are accumulated in that arithmetic.
// ------------------------------------------------------------------
constexpr int GT = 256;   // threads
constexpr int TS = 16;    // sites per tile

struct GramArgs {
  int n, m, K, nb, ns;
  int precs[4];
  const void* ptrs[4];
  const double* ph;
  mxk_kappa kap;
  int chunks;              // CTAs per k
  double* partial;         // [K][chunks][nent][4]  (ga re, ga im, gm re, gm im)
  const float2* resid;     // optional c64 residual r_j of the high columns (see below)
  const double* theta;     // their Ritz values
  Sc sixth;
};

// a high-precision value rounded to FP32 (the leading float of a pair)
__device__ __forceinline__ cx<float> to_cf(cx<dd> v) { return mkc(v.re.hi, v.im.hi); }
__device__ __forceinline__ cx<float> to_cf(cx<double> v) { return mkc((float) v.re, (float) v.im); }

template <typename HI> struct KapHi;
template <> struct KapHi<dd> {
  __device__ static dd get(const mxk_kappa& k, size_t c) { return dd_make(k.dd[2 * c], k.dd[2 * c + 1]); }
};
template <> struct KapHi<double> {
  __device__ static double get(const mxk_kappa& k, size_t c) { return k.d[c]; }
};

__device__ __forceinline__ cx<float> ld_any_f(int prec, const void* base, size_t off) {
  if (prec == MX_C64) return Store<float2, float>::ld((const float2*) base + off);
  if (prec == MX_CDD) return Store<cdd, float>::ld((const cdd*) base + off);
  return Store<double2, float>::ld((const double2*) base + off);
}

// HI = dd for the mixed solver (column block 0 is cdd, the other blocks c64),
// double for the plain solver (every block c128, every column high).
template <typename HI>
__global__ void k_block_gram(GramArgs a, int mh, int ebase) {
  int k = blockIdx.y, chunk = blockIdx.x;
  int n = a.n, m = a.m, ns = a.ns;
  int nent = ns * (ns + 1) / 2;
  Lay L{n, m, a.K};
  extern __shared__ double smd[];
  // staging per site and column: curl, x, y, (Mx), (My)
  cx<HI>* hi = reinterpret_cast<cx<HI>*>(smd);                        // TS*mh*5
  cx<float>* lo = reinterpret_cast<cx<float>*>(hi + TS * mh * 5);      // TS*ns*5
  HI* kap_h = reinterpret_cast<HI*>(lo + TS * ns * 5);                // TS
  float* kap_t = reinterpret_cast<float*>(kap_h + TS);                // TS
  cx<float>* rs = reinterpret_cast<cx<float>*>(kap_t + TS);          // TS*mh*2 (x, y of r)
  bool use_r = a.resid != nullptr;
  Seam<float> sf = seam_load<float>(a.ph, a.K, k, n);
  Seam<HI> sh = seam_load<HI>(a.ph, a.K, k, n);
  // a launch accumulates the entries [ebase, ebase + MAXE*GT) of the lower
  // triangle (ns <= 48: one launch; larger blocks take several)
  constexpr int MAXE = 5;
  cx<float> acc_a[MAXE], acc_m[MAXE];
  cx<HI> hacc_a[MAXE], hacc_m[MAXE];
  int ei[MAXE], ej[MAXE];
  for (int t = 0; t < MAXE; t++) {
    acc_a[t] = czero<float>(); acc_m[t] = czero<float>();
    hacc_a[t] = czero<HI>(); hacc_m[t] = czero<HI>();
    int e = ebase + threadIdx.x + t * GT;
    ei[t] = -1; ej[t] = -1;
    if (e < nent) {
      // row-major lower triangle: e = i(i+1)/2 + j, j <= i
      int i = (int) ((sqrtf(8.0f * e + 1.0f) - 1.0f) * 0.5f);
      while (i * (i + 1) / 2 > e) i--;
      while ((i + 1) * (i + 2) / 2 <= e) i++;
      ei[t] = i; ej[t] = e - i * (i + 1) / 2;
    }
  }
  HI mmh = sget<HI>(a.sixth), fourh = rc<HI>(4.0f);
  float mmf = a.sixth.hi;
  size_t nsite = (size_t) n * n;
  size_t per = (nsite + a.chunks - 1) / a.chunks;
  size_t s0 = (size_t) chunk * per, s1 = s0 + per < nsite ? s0 + per : nsite;
  for (size_t base = s0; base < s1; base += TS) {
    __syncthreads();
    for (int w = threadIdx.x; w < TS * ns; w += GT) {
      int ts = w / ns, col = w % ns;
      size_t site = base + ts;
      if (site >= s1) continue;
      int i = (int) site % n, j = (int) site / n;
      int b = col / m, v = col % m;
      int prec = a.precs[b];
      size_t o0 = L.edge(k, 0, 0, 0, v);
      cx<float>* ls = lo + ((size_t) ts * ns + col) * 5;
      if (col < mh) {
        cx<HI> c, x0, y0, mxv, myv;
        if (prec == MX_CDD) {
          EA<cdd, HI> E{(const cdd*) a.ptrs[b] + o0, n, m, sh};
          c = curlc<HI>(E, i, j); x0 = E(0, i, j); y0 = E(1, i, j);
          mxv = scal(mmh, scal(fourh, x0) + E(0, i, j + 1) + E(0, i, j - 1));
          myv = scal(mmh, scal(fourh, y0) + E(1, i + 1, j) + E(1, i - 1, j));
        } else {
          EA<double2, HI> E{(const double2*) a.ptrs[b] + o0, n, m, sh};
          c = curlc<HI>(E, i, j); x0 = E(0, i, j); y0 = E(1, i, j);
          mxv = scal(mmh, scal(fourh, x0) + E(0, i, j + 1) + E(0, i, j - 1));
          myv = scal(mmh, scal(fourh, y0) + E(1, i + 1, j) + E(1, i - 1, j));
        }
        cx<HI>* hs = hi + ((size_t) ts * mh + col) * 5;
        hs[0] = c; hs[1] = x0; hs[2] = y0; hs[3] = mxv; hs[4] = myv;
        ls[0] = to_cf(c); ls[1] = to_cf(x0); ls[2] = to_cf(y0); ls[3] = to_cf(mxv); ls[4] = to_cf(myv);
      } else {
        const void* pb = a.ptrs[b];
        auto X = [&](int p, int ii, int jj) {
          cx<float> phz;
          bool wr = sf.wrap(ii, jj, phz);
          cx<float> val = ld_any_f(prec, pb, o0 + ((size_t) (p * n + jj) * n + ii) * m);
          return wr ? phz * val : val;
        };
        cx<float> x0 = X(0, i, j), y0 = X(1, i, j);
        ls[0] = x0 - X(0, i, j + 1) - y0 + X(1, i + 1, j);
        ls[1] = x0;
        ls[2] = y0;
        ls[3] = scal(mmf, scal(4.0f, x0) + X(0, i, j + 1) + X(0, i, j - 1));
        ls[4] = scal(mmf, scal(4.0f, y0) + X(1, i + 1, j) + X(1, i - 1, j));
      }
    }
    if (use_r)
      for (int w = threadIdx.x; w < TS * mh; w += GT) {
        int ts = w / mh, v = w % mh;
        size_t site = base + ts;
        if (site >= s1) continue;
        int i = (int) site % n, j = (int) site / n;
        float2 rx = a.resid[L.edge(k, 0, j, i, v)], ry = a.resid[L.edge(k, 1, j, i, v)];
        rs[((size_t) ts * mh + v) * 2] = mkc(rx.x, rx.y);
        rs[((size_t) ts * mh + v) * 2 + 1] = mkc(ry.x, ry.y);
      }
    for (int ts = threadIdx.x; ts < TS; ts += GT) {
      size_t site = base + ts;
      if (site < s1) {
        kap_t[ts] = a.kap.f[site];
        kap_h[ts] = KapHi<HI>::get(a.kap, site);
      } else {
        kap_t[ts] = 0.0f;
        kap_h[ts] = Real<HI>::zero();
      }
    }
    __syncthreads();
    int nts = (int) (s1 - base < (size_t) TS ? s1 - base : (size_t) TS);
    for (int t = 0; t < MAXE; t++) {
      int i = ei[t], j = ej[t];
      if (i < 0) continue;
      if (i < mh && j < mh) {
        cx<HI> sa = czero<HI>(), sm2 = czero<HI>();
        for (int ts = 0; ts < nts; ts++) {
          const cx<HI>* hs = hi + (size_t) ts * mh * 5;
          sa += scal(kap_h[ts], conjc(hs[i * 5]) * hs[j * 5]);
          sm2 += conjc(hs[i * 5 + 1]) * hs[j * 5 + 3] + conjc(hs[i * 5 + 2]) * hs[j * 5 + 4];
        }
        hacc_a[t] += sa;
        hacc_m[t] += sm2;
      } else if (use_r && j < mh) {
        // cross entry s_i^H (A+M) e_j = theta_j s_i^H M e_j + s_i^H r_j: only
        // s_i^H r_j is accumulated here, the rest is added at the end
        cx<float> sa = czero<float>(), sm2 = czero<float>();
        for (int ts = 0; ts < nts; ts++) {
          const cx<float>* ls = lo + (size_t) ts * ns * 5;
          const cx<float>* rr = rs + (size_t) ts * mh * 2;
          sa += conjc(ls[i * 5 + 1]) * rr[j * 2] + conjc(ls[i * 5 + 2]) * rr[j * 2 + 1];
          sm2 += conjc(ls[i * 5 + 1]) * ls[j * 5 + 3] + conjc(ls[i * 5 + 2]) * ls[j * 5 + 4];
        }
        acc_a[t] += sa;
        acc_m[t] += sm2;
      } else {
        cx<float> sa = czero<float>(), sm2 = czero<float>();
        for (int ts = 0; ts < nts; ts++) {
          const cx<float>* ls = lo + (size_t) ts * ns * 5;
          sa += scal(kap_t[ts], conjc(ls[i * 5]) * ls[j * 5]);
          sm2 += conjc(ls[i * 5 + 1]) * ls[j * 5 + 3] + conjc(ls[i * 5 + 2]) * ls[j * 5 + 4];
        }
        acc_a[t] += sa;
        acc_m[t] += sm2;
      }
    }
  }
  double axy = (double) n * (double) n;
  double* out = a.partial + (((size_t) k * a.chunks + chunk) * nent) * 4;
  for (int t = 0; t < MAXE; t++) {
    int e = ebase + threadIdx.x + t * GT;
    if (e >= nent) continue;
    double ar = Real<HI>::to_double(hacc_a[t].re) + (double) acc_a[t].re;
    double ai = Real<HI>::to_double(hacc_a[t].im) + (double) acc_a[t].im;
    double mr = Real<HI>::to_double(hacc_m[t].re) + (double) acc_m[t].re;
    double mi = Real<HI>::to_double(hacc_m[t].im) + (double) acc_m[t].im;
    // A + M = axy * (sum over cells of kappa conj(curl_i) curl_j) + M, or
    // for the residual form of the cross entries theta_j * M + s_i^H r_j
    if (use_r && ei[t] >= mh && ej[t] < mh) {
      double th = a.theta[(size_t) k * m + ej[t]];
      out[(size_t) e * 4 + 0] = th * mr + ar;
      out[(size_t) e * 4 + 1] = th * mi + ai;
    } else {
      out[(size_t) e * 4 + 0] = axy * ar + mr;
      out[(size_t) e * 4 + 1] = axy * ai + mi;
    }
    out[(size_t) e * 4 + 2] = mr;
    out[(size_t) e * 4 + 3] = mi;
  }
}

__global__ void k_gram_reduce(int ns, int K, int chunks, const double* __restrict__ partial,
                              double* __restrict__ ga, double* __restrict__ gm) {
  int nent = ns * (ns + 1) / 2;
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t) nent * K) return;
  int k = (int) (t / nent), e = (int) (t % nent);
  int i = (int) ((sqrt(8.0 * e + 1.0) - 1.0) * 0.5);
  while (i * (i + 1) / 2 > e) i--;
  while ((i + 1) * (i + 2) / 2 <= e) i++;
  int j = e - i * (i + 1) / 2;
  double s[4] = {0, 0, 0, 0};
  for (int c = 0; c < chunks; c++) {
    const double* p = partial + (((size_t) k * chunks + c) * nent + e) * 4;
    s[0] += p[0]; s[1] += p[1]; s[2] += p[2]; s[3] += p[3];
  }
  // entry (i,j) = s_i^H K s_j; lower triangle i >= j, upper by symmetry
  double* A = ga + (size_t) k * 2 * ns * ns;
  double* M = gm + (size_t) k * 2 * ns * ns;
  A[2 * ((size_t) j * ns + i) + 0] = s[0];
  A[2 * ((size_t) j * ns + i) + 1] = s[1];
  M[2 * ((size_t) j * ns + i) + 0] = s[2];
  M[2 * ((size_t) j * ns + i) + 1] = s[3];
  A[2 * ((size_t) i * ns + j) + 0] = s[0];
  A[2 * ((size_t) i * ns + j) + 1] = -s[1];
  M[2 * ((size_t) i * ns + j) + 0] = s[2];
  M[2 * ((size_t) i * ns + j) + 1] = -s[3];
}

// ------------------------------------------------------------------
// block combine: out(k, e, j) = sum_i coef[k](row0 + i, j) S_i(k, e)
// ------------------------------------------------------------------
struct CombArgs {
  int n, m, K, nb, ldc, row0;
  int precs[4];
  const void* ptrs[4];
  const double* coef;
  const float4* cpair;     // coef as float-float pairs (re.hi, re.lo, im.hi, im.lo)
};

// coef -> float-float pairs, once per combine, so that the combine kernels
// convert nothing in double
__global__ void k_coef_pairs(const double* __restrict__ coef, float4* __restrict__ out, size_t len) {
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= len) return;
  dd r = dd_from_double(coef[2 * t]), i = dd_from_double(coef[2 * t + 1]);
  out[t] = make_float4(r.hi, r.lo, i.hi, i.lo);
}

template <typename R> struct CoefGet {
  __device__ static cx<R> get(const CombArgs& a, size_t at) {
    float4 c = a.cpair[at];
    return mkc(PairGet<R>::get(&c.x), PairGet<R>::get(&c.z));
  }
};
template <> struct CoefGet<double> {
  __device__ static cx<double> get(const CombArgs& a, size_t at) {
    return mkc(a.coef[2 * at], a.coef[2 * at + 1]);
  }
};

template <typename SO, typename RO>
__global__ void k_block_combine(CombArgs a, SO* __restrict__ out) {
  // block (m, rows): x = output column, y = entry (plane, site); grid.y = k.
  // The coefficients are staged once per block in shared memory in the
  // arithmetic of the block they multiply.
  int k = blockIdx.y;
  int m = a.m;
  int nsrc = a.nb * m;
  extern __shared__ float smc[];
  cx<RO>* chi = reinterpret_cast<cx<RO>*>(smc);                    // nsrc * m
  cx<float>* clo = reinterpret_cast<cx<float>*>(chi + nsrc * m);   // nsrc * m
  size_t cbase = (size_t) k * a.ldc * m;
  int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;
  for (int e = tid; e < nsrc * m; e += nth) {
    int i = e % nsrc, j = e / nsrc;
    size_t at = cbase + (size_t) j * a.ldc + a.row0 + i;
    int b = i / m;
    if (a.precs[b] == MX_C64) {
      float4 c = a.cpair[at];
      clo[j * nsrc + i] = mkc(c.x, c.z);
    } else {
      chi[j * nsrc + i] = CoefGet<RO>::get(a, at);
    }
  }
  __syncthreads();
  size_t per_k = (size_t) 2 * a.n * a.n * m;
  int j = threadIdx.x;
  int ent = blockIdx.x * blockDim.y + threadIdx.y;
  if (ent >= 2 * a.n * a.n) return;
  size_t kbase = (size_t) k * per_k + (size_t) ent * m;
  cx<RO> acc_hi = czero<RO>();
  cx<float> acc_lo = czero<float>();
  for (int b = 0; b < a.nb; b++) {
    int prec = a.precs[b];
    if (prec == MX_C64) {
      const float2* src = (const float2*) a.ptrs[b] + kbase;
      const cx<float>* cc = clo + j * nsrc + b * m;
      for (int i = 0; i < m; i++) {
        float2 v = src[i];
        acc_lo += cc[i] * mkc(v.x, v.y);
      }
    } else {
      const cx<RO>* cc = chi + j * nsrc + b * m;
      for (int i = 0; i < m; i++) {
        cx<RO> v = prec == MX_CDD ? Store<cdd, RO>::ld((const cdd*) a.ptrs[b] + kbase + i)
                                  : Store<double2, RO>::ld((const double2*) a.ptrs[b] + kbase + i);
        acc_hi += cc[i] * v;
      }
    }
  }
  cx<RO> res = acc_hi + mkc(Real<RO>::from_float(acc_lo.re), Real<RO>::from_float(acc_lo.im));
  Store<SO, RO>::st(out + kbase + j, res);
}

// ------------------------------------------------------------------
// Block combination of the mixed solver as a tiled product: a CTA takes
// tiles of CTE entries (site, plane) of one k-point, loads each source
// block's tile (CTE x m contiguous values) and the coefficients into shared
// memory, and every thread forms 4 outputs (entries e0 + 16q, column j).
// Rows of a float-float source (the eigenvector block) are accumulated as
// compensated FP32 sums of exact products, the c64 rows in FP32; the
// float-float output is the normalised sum of both.
// ------------------------------------------------------------------
constexpr int CT = 256;       // threads
constexpr int CTE = 64;       // entries per tile

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned d = (unsigned) __cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// A thread combines a 2x2 tile of outputs: entries ep and ep + 32 of the
// tile, columns cp and cp + 8, so that each source value and coefficient
// it loads from shared memory serves two outputs.  The source tiles (CTE
// entries of each block, contiguous in memory) are copied into shared
// memory by cp.async, double-buffered: the copies of a CTA's next tile are
// in flight while it combines the current one.  Every source block and
// tile starts on a 16-byte boundary (checked at launch).
template <bool DDOUT>
__global__ void __launch_bounds__(CT, 2) k_block_combine_tiled(CombArgs a, void* out) {
  const int k = blockIdx.y, m = a.m, nb = a.nb, nsrc = nb * m;
  extern __shared__ float4 smct[];
  float4* cS = smct;                                             // [48][16] coefficient pairs [row][column]
  float4* tE = cS + 48 * 16;                                     // [2][CTE * 17] float-float source tiles
  float2* tF = reinterpret_cast<float2*>(tE + 2 * CTE * 17);     // [2][2][CTE * 18] c64 source tiles
  const int tid = threadIdx.x;
  // entry strides of the tiles: one float4 / one 16-byte unit past m, so
  // that the four entries a warp reads at once fall on distinct banks (an
  // odd m keeps the c64 tile unpadded: its 16-byte copies would straddle
  // entries)
  const int SE = m + 1, SF = (m & 1) ? m : m + 2;
  for (int q = tid; q < nsrc * m; q += CT) {
    int i = q / m, j = q % m;
    cS[i * 16 + j] = a.cpair[(size_t) k * a.ldc * m + (size_t) j * a.ldc + a.row0 + i];
  }
  const bool dd0 = a.precs[0] == MX_CDD;
  const int cp = tid & 7, ep = tid >> 3;
  const int c0 = cp, c1 = cp + 8 < m ? cp + 8 : cp;
  const bool live = c0 < m, two = cp + 8 < m;
  const size_t per_k = (size_t) 2 * a.n * a.n;           // entries per k-point
  const size_t ntiles = (per_k + CTE - 1) / CTE;
  // copies of tile t into buffer q, one commit group per tile
  auto issue = [&](size_t t, int q) {
    const size_t e_start = t * CTE;
    const int nte = (int) (per_k - e_start < (size_t) CTE ? per_k - e_start : (size_t) CTE);
    const size_t off = ((size_t) k * per_k + e_start) * m;
    const int len = nte * m;   // elements; even, so that c64 tiles are whole 16-byte units
    for (int b = 0; b < nb; b++) {
      if (b == 0 && dd0) {
        const float4* src = (const float4*) a.ptrs[0] + off;
        float4* dst = tE + q * CTE * 17;
        for (int u = tid; u < len; u += CT) {
          const int e = u / m;
          cp_async16(dst + e * SE + (u - e * m), src + u);
        }
      } else {
        const float2* src = (const float2*) a.ptrs[b] + off;
        float2* dst = tF + (q * 2 + (dd0 ? b - 1 : b)) * CTE * 18;
        for (int u = 2 * tid; u < len; u += 2 * CT) {
          const int e = u / m;
          cp_async16(dst + e * SF + (u - e * m), src + u);
        }
      }
    }
  };
  int q = 0;
  if ((size_t) blockIdx.x < ntiles) issue(blockIdx.x, 0);
  cp_async_commit();
  for (size_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, q ^= 1) {
    if (tile + gridDim.x < ntiles) issue(tile + gridDim.x, q ^ 1);
    cp_async_commit();
    cp_async_wait1();
    __syncthreads();
    const size_t e_start = tile * CTE;
    const int nte = (int) (per_k - e_start < (size_t) CTE ? per_k - e_start : (size_t) CTE);
    // the second entry repeats the first past the tile's end (not written)
    const int ea = ep, eb = ep + 32 < nte ? ep + 32 : ep;
    if (live && ea < nte) {
      // output (entry r, column s) at index 2 r + s, r, s in {0, 1}
      float acc[4][4] = {};     // compensated sums re (s, c), im (s, c)
      float fre[4] = {}, fim[4] = {};
      int row = 0;
      if (dd0) {
        const float4* tEq = tE + q * CTE * 17;
#pragma unroll 4
        for (int i = 0; i < m; i++) {
          const float4 c[2] = {cS[i * 16 + c0], cS[i * 16 + c1]};
          const float4 v[2] = {tEq[ea * SE + i], tEq[eb * SE + i]};
#pragma unroll
          for (int r = 0; r < 2; r++)
#pragma unroll
            for (int t = 0; t < 2; t++) {
              float* ac = acc[2 * r + t];
              comp_mac(ac[0], ac[1], c[t].x, c[t].y, v[r].x, v[r].y);
              comp_mac(ac[0], ac[1], -c[t].z, -c[t].w, v[r].z, v[r].w);
              comp_mac(ac[2], ac[3], c[t].x, c[t].y, v[r].z, v[r].w);
              comp_mac(ac[2], ac[3], c[t].z, c[t].w, v[r].x, v[r].y);
            }
        }
        row = m;
      }
      for (int b = dd0 ? 1 : 0; b < nb; b++) {
        const float2* tb = tF + (q * 2 + (dd0 ? b - 1 : b)) * CTE * 18;
#pragma unroll 4
        for (int i = 0; i < m; i++) {
          const float4 c[2] = {cS[(row + i) * 16 + c0], cS[(row + i) * 16 + c1]};
          const float2 v[2] = {tb[ea * SF + i], tb[eb * SF + i]};
#pragma unroll
          for (int r = 0; r < 2; r++)
#pragma unroll
            for (int t = 0; t < 2; t++) {
              fre[2 * r + t] = fmaf(c[t].x, v[r].x, fmaf(-c[t].z, v[r].y, fre[2 * r + t]));
              fim[2 * r + t] = fmaf(c[t].x, v[r].y, fmaf(c[t].z, v[r].x, fim[2 * r + t]));
            }
        }
        row += m;
      }
#pragma unroll
      for (int r = 0; r < 2; r++)
#pragma unroll
        for (int t = 0; t < 2; t++) {
          if ((r && eb == ea) || (t && !two)) continue;
          const int o2 = 2 * r + t;
          const size_t o = ((size_t) k * per_k + e_start + (r ? eb : ea)) * m + (t ? c1 : c0);
          if (DDOUT) {
            dd re = two_sum(acc[o2][0], acc[o2][1] + fre[o2]), im = two_sum(acc[o2][2], acc[o2][3] + fim[o2]);
            reinterpret_cast<float4*>(out)[o] = make_float4(re.hi, re.lo, im.hi, im.lo);
          } else {
            reinterpret_cast<float2*>(out)[o] =
                make_float2(acc[o2][0] + acc[o2][1] + fre[o2], acc[o2][2] + acc[o2][3] + fim[o2]);
          }
        }
    }
    // the buffer is refilled by the next iteration's copies
    __syncthreads();
  }
}

static size_t combine_tiled_smem() {
  return sizeof(float4) * (48 * 16 + 2 * CTE * 17) + sizeof(float2) * 4 * CTE * 18;
}

// ------------------------------------------------------------------
// sensitivity: grad[c] = -n^2 kappa_c^2 sum_{k,v} w_kv |curl_c e_kv|^2
// ------------------------------------------------------------------
template <typename S, typename R>
__global__ void k_eps_sensitivity(int n, int m, int K, const double* __restrict__ ph,
                                  const double* __restrict__ kappa, const double* __restrict__ w,
                                  const S* __restrict__ e, double* __restrict__ grad) {
  size_t c = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (size_t) n * n) return;
  int i = (int) (c % n), j = (int) (c / n);
  Lay L{n, m, K};
  double s = 0.0;
  for (int k = 0; k < K; k++) {
    Seam<R> sm = seam_load<R>(ph, K, k, n);
    for (int v = 0; v < m; v++) {
      double wv = w[(size_t) k * m + v];
      if (wv == 0.0) continue;
      EA<S, R> E{e + L.edge(k, 0, 0, 0, v), n, m, sm};
      cx<R> cu = curlc<R>(E, i, j);
      double re = Real<R>::to_double(cu.re), im = Real<R>::to_double(cu.im);
      s += wv * (re * re + im * im);
    }
  }
  double kc = kappa[c];
  grad[c] = -(double) n * n * kc * kc * s;
}

}  // namespace

extern "C" int mxk_block_residual(int n, int m, int K, const double* ph, mxk_kappa kap, const double* mu,
                                  int pe, const void* e, int pr, void* rout, double* stats, mx_stream s) {
  int rows = 256 / m;
  if (m > 32) return (int) cudaErrorInvalidValue;
  size_t nsite = (size_t) n * n;
  // about residual_sites sites per thread, so that the per-thread double
  // reduction at the end stays small against the sweep
  const size_t per = (size_t) rows * g_tuning.residual_sites;
  unsigned G = (unsigned) ((nsite + per - 1) / per);
  if (G < 1) G = 1;
  if (G > 4096) G = 4096;
  dim3 g(G, K), b(256);
  cudaStream_t st = (cudaStream_t) s;
  Sc axy = make_sc((double) n * (double) n), sixth = make_sc(1.0 / 6.0);
  if (pe == MX_CDD && (pr == MX_C64 || !rout))
    k_block_residual<cdd, float2, dd><<<g, b, 0, st>>>(n, m, K, ph, kapb<dd>(kap, n), axy, sixth, mu, (const cdd*) e, (float2*) rout, stats);
  else if (pe == MX_C128 && (pr == MX_C128 || !rout))
    k_block_residual<double2, double2, double><<<g, b, 0, st>>>(n, m, K, ph, kapb<double>(kap, n), axy, sixth, mu, (const double2*) e, (double2*) rout, stats);
  else if (pe == MX_C128 && pr == MX_C64)
    k_block_residual<double2, float2, double><<<g, b, 0, st>>>(n, m, K, ph, kapb<double>(kap, n), axy, sixth, mu, (const double2*) e, (float2*) rout, stats);
  else if (pe == MX_C64 && (pr == MX_C64 || !rout))
    k_block_residual<float2, float2, float><<<g, b, 0, st>>>(n, m, K, ph, kapb<float>(kap, n), axy, sixth, mu, (const float2*) e, (float2*) rout, stats);
  else
    return (int) cudaErrorInvalidValue;
  MX_CHECK_LAUNCH();
  return 0;
}

__device__ __forceinline__ void tri_index(int e, int& i, int& j) {
  i = (int) ((sqrtf(8.0f * e + 1.0f) - 1.0f) * 0.5f);
  while (i * (i + 1) / 2 > e) i--;
  while ((i + 1) * (i + 2) / 2 <= e) i++;
  j = e - i * (i + 1) / 2;
}

// ------------------------------------------------------------------
// Gram matrices of the mixed solver: column block 0 is the float-float
// eigenvector block E (m <= 16 columns), blocks 1.. are c64, and the
// entries between a c64 column s_i and an E column e_j take the residual
// form theta_j s_i^H M e_j + s_i^H r_j (r_j the float-float residual rounded
// to c64), which keeps the cancellation of s_i^H (A+M) e_j out of FP32.  The
// two kinds of entries are separate CTAs of one launch (grid z = 0: FP32
// entries, z = 1: E-E entries), each staging only what its entries read:
//   FP32 CTAs  every entry with a c64 column: the 4x2 tiles of the block
//              pairs (1,0), (2,0), (2,1) and the lower-triangle tiles of
//              (1,1), (2,2); a tile's two threads take alternate sites of a
//              32-site tile and meet by a shuffle at the end.  Per site a
//              tile loads 4 row and 2 column operands for 8 entries.
//   E-E CTAs   the lower-triangle 2x2 tiles of the E block as compensated
//              FP32 sums of exact products; eight threads per tile take every
//              eighth site and meet by shuffles (in FP64) at the end.
// The E-E sums carry about twice the FP32 precision (TwoProd by FMA, TwoSum;
// the low parts of E enter through the cross products), like float-float
// arithmetic at half its cost.  Partial sums per CTA go to scratch in the
// layout of k_block_gram.
// ------------------------------------------------------------------
constexpr int GS_T = 288;   // threads per CTA
constexpr int GS_S = 32;    // sites per tile
// shared layouts, component-major within a site and a site stride one
// element past a multiple of 32 banks, so that the threads of a warp (tiles
// x neighbouring sites) hit distinct banks:
//   FP32 I (ts, b-1, comp, col) = ts * GS_IS + ((b - 1) * 3 + comp) * 16 + col
//   FP32 J (ts, b, comp, col)   = ts * GS_JS + (b * 4 + comp) * 16 + col
//   E-E  D (ts, comp, col)      = ts * GS_DS + comp * 16 + col
constexpr int GS_IS = 2 * 3 * 16 + 1, GS_JS = 3 * 4 * 16 + 1, GS_DS = 3 * 16 + 1;

// FP32 tiles are 4 rows x 2 columns: 32 per full block pair (1,0), (2,0),
// (2,1) with bi < nb, then 20 per diagonal block (1,1), (2,2) (the tiles with
// an entry on or below the diagonal: 2, 4, 6, 8 column tiles for row tiles 0..3)
__device__ __forceinline__ void gs_tile_f(int q, int nb, int& bi, int& bj, int& ti, int& tj) {
  const int nfull = nb == 3 ? 3 : (nb == 2 ? 1 : 0);
  if (q < 32 * nfull) {
    const int pr = q >> 5, r = q & 31;
    bi = pr == 0 ? 1 : 2;
    bj = pr == 2 ? 1 : 0;
    ti = r >> 3;
    tj = r & 7;
  } else {
    const int r = q - 32 * nfull, rr = r % 20;
    bi = bj = 1 + r / 20;
    ti = rr < 2 ? 0 : (rr < 6 ? 1 : (rr < 12 ? 2 : 3));
    tj = rr - (ti == 0 ? 0 : (ti == 1 ? 2 : (ti == 2 ? 6 : 12)));
  }
}

__global__ void __launch_bounds__(GS_T, 2) k_block_gram_split(GramArgs a) {
  const int n = a.n, m = a.m, ns = a.ns, nb = a.nb;
  // a single block has E-E entries only (grid z = 1)
  const int k = blockIdx.y, chunk = blockIdx.x, role = nb > 1 ? (int) blockIdx.z : 1;
  const int nent = ns * (ns + 1) / 2;
  const int tid = threadIdx.x;
  extern __shared__ float4 sm4[];
  Lay L{n, m, a.K};
  const size_t nsite = (size_t) n * n;
  const size_t per = (nsite + a.chunks - 1) / a.chunks;
  const size_t s0 = (size_t) chunk * per, s1 = s0 + per < nsite ? s0 + per : nsite;
  const double axy = (double) n * (double) n;
  double* out = a.partial + (((size_t) k * a.chunks + chunk) * nent) * 4;
  const bool use_r = a.resid != nullptr;

  if (role == 0) {
    // ---------------- FP32 entries ----------------
    // I[s][b-1][col][3]: curl, x, y of the c64 blocks b = 1, 2
    // J[s][b][col][4]:  b = 0: M x, M y, r x, r y of E; b >= 1: kappa curl, M x, M y
    cx<float>* I = reinterpret_cast<cx<float>*>(sm4);
    cx<float>* J = I + GS_S * GS_IS;
    const int ntile = nb == 3 ? 136 : (nb == 2 ? 52 : 0);
    const int tile = tid >> 1, g = tid & 1;
    const bool live = tile < ntile;
    int bi = 1, bj = 0, ti = 0, tj = 0;
    if (live) gs_tile_f(tile, nb, bi, bj, ti, tj);
    const bool rmode = use_r && bj == 0;
    // rows/columns of the tile inside their blocks, clamped to m - 1 past the block
    int rc_[4], cc_[2];
#pragma unroll
    for (int q = 0; q < 4; q++) rc_[q] = 4 * ti + q < m ? 4 * ti + q : m - 1;
#pragma unroll
    for (int q = 0; q < 2; q++) cc_[q] = 2 * tj + q < m ? 2 * tj + q : m - 1;
    float acc[8][4];   // entry (2 aq + bq): A re, A im, M re, M im
#pragma unroll
    for (int e = 0; e < 8; e++) acc[e][0] = acc[e][1] = acc[e][2] = acc[e][3] = 0.f;
    const float sixth = a.sixth.hi;
    for (size_t base = s0; base < s1; base += GS_S) {
      const int nts = (int) (s1 - base < (size_t) GS_S ? s1 - base : (size_t) GS_S);
      __syncthreads();
      for (int w = tid; w < GS_S * nb * m; w += GS_T) {
        const int ts = w / (nb * m), col = w % (nb * m);
        if (ts >= nts) continue;
        const size_t site = base + ts;
        const int i = (int) (site % n), j = (int) (site / n);
        const int b = col / m, v = col % m;
        const size_t o0 = L.edge(k, 0, 0, 0, v);
        const bool inner = i > 0 && i < n - 1 && j > 0 && j < n - 1;
        cx<float>* Jp = J + (size_t) ts * GS_JS + b * 64 + v;   // component c at Jp[16 c]
        if (b == 0) {
          const cdd* eb = (const cdd*) a.ptrs[0] + o0;
          auto body = [&](const auto& E) {
            const cx<float> x0 = E(0, i, j), y0 = E(1, i, j);
            Jp[0] = scal(sixth, scal(4.0f, x0) + E(0, i, j + 1) + E(0, i, j - 1));
            Jp[16] = scal(sixth, scal(4.0f, y0) + E(1, i + 1, j) + E(1, i - 1, j));
          };
          if (inner) body(EAI<cdd, float>{eb, n, m});
          else body(EA<cdd, float>{eb, n, m, seam_load<float>(a.ph, a.K, k, n)});
          if (use_r) {
            const float2 rx = a.resid[L.edge(k, 0, j, i, v)], ry = a.resid[L.edge(k, 1, j, i, v)];
            Jp[32] = mkc(rx.x, rx.y);
            Jp[48] = mkc(ry.x, ry.y);
          }
        } else {
          const float2* xb = (const float2*) a.ptrs[b] + o0;
          const float kap = a.kap.f[site];
          cx<float>* Ip = I + (size_t) ts * GS_IS + (b - 1) * 48 + v;   // component c at Ip[16 c]
          auto body = [&](const auto& X) {
            const cx<float> x0 = X(0, i, j), t = X(0, i, j + 1), y0 = X(1, i, j), r = X(1, i + 1, j);
            const cx<float> c = x0 - t - y0 + r;
            Ip[0] = c; Ip[16] = x0; Ip[32] = y0;
            Jp[0] = scal(kap, c);
            Jp[16] = scal(sixth, scal(4.0f, x0) + t + X(0, i, j - 1));
            Jp[32] = scal(sixth, scal(4.0f, y0) + r + X(1, i - 1, j));
          };
          if (inner) body(EAI<float2, float>{xb, n, m});
          else body(EA<float2, float>{xb, n, m, seam_load<float>(a.ph, a.K, k, n)});
        }
      }
      __syncthreads();
      if (live) {
        for (int ts = g; ts < nts; ts += 2) {
          const cx<float>* Ib = I + (size_t) ts * GS_IS + (bi - 1) * 48;
          const cx<float>* Jb = J + (size_t) ts * GS_JS + bj * 64;
          cx<float> cr[4], xr[4], yr[4];
#pragma unroll
          for (int q = 0; q < 4; q++) {
            cr[q] = Ib[rc_[q]];
            xr[q] = Ib[16 + rc_[q]];
            yr[q] = Ib[32 + rc_[q]];
          }
#pragma unroll
          for (int bq = 0; bq < 2; bq++) {
            const cx<float>* Jc = Jb + cc_[bq];
            if (rmode) {
              const cx<float> mx = Jc[0], my = Jc[16], rx = Jc[32], ry = Jc[48];
#pragma unroll
              for (int aq = 0; aq < 4; aq++) {
                float* d = acc[2 * aq + bq];
                d[2] = fmaf(xr[aq].re, mx.re, d[2]); d[2] = fmaf(xr[aq].im, mx.im, d[2]);
                d[2] = fmaf(yr[aq].re, my.re, d[2]); d[2] = fmaf(yr[aq].im, my.im, d[2]);
                d[3] = fmaf(xr[aq].re, mx.im, d[3]); d[3] = fmaf(-xr[aq].im, mx.re, d[3]);
                d[3] = fmaf(yr[aq].re, my.im, d[3]); d[3] = fmaf(-yr[aq].im, my.re, d[3]);
                d[0] = fmaf(xr[aq].re, rx.re, d[0]); d[0] = fmaf(xr[aq].im, rx.im, d[0]);
                d[0] = fmaf(yr[aq].re, ry.re, d[0]); d[0] = fmaf(yr[aq].im, ry.im, d[0]);
                d[1] = fmaf(xr[aq].re, rx.im, d[1]); d[1] = fmaf(-xr[aq].im, rx.re, d[1]);
                d[1] = fmaf(yr[aq].re, ry.im, d[1]); d[1] = fmaf(-yr[aq].im, ry.re, d[1]);
              }
            } else {
              const cx<float> kc = Jc[0], mx = Jc[16], my = Jc[32];
#pragma unroll
              for (int aq = 0; aq < 4; aq++) {
                float* d = acc[2 * aq + bq];
                d[2] = fmaf(xr[aq].re, mx.re, d[2]); d[2] = fmaf(xr[aq].im, mx.im, d[2]);
                d[2] = fmaf(yr[aq].re, my.re, d[2]); d[2] = fmaf(yr[aq].im, my.im, d[2]);
                d[3] = fmaf(xr[aq].re, mx.im, d[3]); d[3] = fmaf(-xr[aq].im, mx.re, d[3]);
                d[3] = fmaf(yr[aq].re, my.im, d[3]); d[3] = fmaf(-yr[aq].im, my.re, d[3]);
                d[0] = fmaf(cr[aq].re, kc.re, d[0]); d[0] = fmaf(cr[aq].im, kc.im, d[0]);
                d[1] = fmaf(cr[aq].re, kc.im, d[1]); d[1] = fmaf(-cr[aq].im, kc.re, d[1]);
              }
            }
          }
        }
      }
    }
    // the two threads of a tile meet; the first writes the tile's entries,
    // A from its parts: s^H r + theta s^H M e (residual form) or axy curl + M
#pragma unroll
    for (int e = 0; e < 8; e++) {
      double q[4];
#pragma unroll
      for (int c = 0; c < 4; c++) {
        q[c] = (double) acc[e][c];
        q[c] += __shfl_xor_sync(0xffffffffu, q[c], 1);
      }
      const int rl = 4 * ti + (e >> 1), cl = 2 * tj + (e & 1);
      if (g == 0 && live && rl < m && cl < m && !(bi == bj && rl < cl)) {
        const int r = bi * m + rl, col = bj * m + cl;
        double* o = out + (size_t) (r * (r + 1) / 2 + col) * 4;
        if (rmode) {
          const double th = a.theta[(size_t) k * m + cl];
          o[0] = th * q[2] + q[0];
          o[1] = th * q[3] + q[1];
        } else {
          o[0] = axy * q[0] + q[2];
          o[1] = axy * q[1] + q[3];
        }
        o[2] = q[2];
        o[3] = q[3];
      }
    }
  } else {
    // ---------------- E-E entries ----------------
    // DI[s][col][3]: curl, x, y;  DJ[s][col][3]: kappa curl, M x, M y (float-float)
    cx<dd>* DI = reinterpret_cast<cx<dd>*>(sm4);
    cx<dd>* DJ = DI + GS_S * GS_DS;
    const int tile = tid >> 3, g = tid & 7;
    const bool live = tile < 36;
    int ti = 0, tj = 0;
    if (live) tri_index(tile, ti, tj);
    const int r0 = 2 * ti < m ? 2 * ti : m - 1, r1 = 2 * ti + 1 < m ? 2 * ti + 1 : m - 1;
    const int c0 = 2 * tj < m ? 2 * tj : m - 1, c1 = 2 * tj + 1 < m ? 2 * tj + 1 : m - 1;
    float ea[4][4], em[4][4];   // entry (2a + b): re s, re c, im s, im c
#pragma unroll
    for (int e = 0; e < 4; e++)
#pragma unroll
      for (int c = 0; c < 4; c++) ea[e][c] = em[e][c] = 0.f;
    const dd sixth_d = sget<dd>(a.sixth), four_d = rc<dd>(4.0f);
    for (size_t base = s0; base < s1; base += GS_S) {
      const int nts = (int) (s1 - base < (size_t) GS_S ? s1 - base : (size_t) GS_S);
      __syncthreads();
      for (int w = tid; w < GS_S * m; w += GS_T) {
        const int ts = w / m, v = w % m;
        if (ts >= nts) continue;
        const size_t site = base + ts;
        const int i = (int) (site % n), j = (int) (site / n);
        const size_t o0 = L.edge(k, 0, 0, 0, v);
        const bool inner = i > 0 && i < n - 1 && j > 0 && j < n - 1;
        const cdd* eb = (const cdd*) a.ptrs[0] + o0;
        const dd kap = dd_make(a.kap.dd[2 * site], a.kap.dd[2 * site + 1]);
        cx<dd>* Ip = DI + (size_t) ts * GS_DS + v;   // component c at Ip[16 c]
        cx<dd>* Jp = DJ + (size_t) ts * GS_DS + v;
        auto body = [&](const auto& E) {
          const cx<dd> x0 = E(0, i, j), t = E(0, i, j + 1), y0 = E(1, i, j), r = E(1, i + 1, j);
          const cx<dd> c = x0 - t - y0 + r;
          Ip[0] = c; Ip[16] = x0; Ip[32] = y0;
          Jp[0] = scal(kap, c);
          Jp[16] = scal(sixth_d, scal(four_d, x0) + t + E(0, i, j - 1));
          Jp[32] = scal(sixth_d, scal(four_d, y0) + r + E(1, i - 1, j));
        };
        if (inner) body(EAI<cdd, dd>{eb, n, m});
        else body(EA<cdd, dd>{eb, n, m, seam_load<dd>(a.ph, a.K, k, n)});
      }
      __syncthreads();
      if (live) {
        for (int ts = g; ts < nts; ts += 8) {
          const cx<dd>* Is = DI + (size_t) ts * GS_DS;
          const cx<dd>* Js = DJ + (size_t) ts * GS_DS;
          const cx<dd> Ir[2][3] = {{Is[r0], Is[16 + r0], Is[32 + r0]}, {Is[r1], Is[16 + r1], Is[32 + r1]}};
#pragma unroll
          for (int bq = 0; bq < 2; bq++) {
            const int cq = bq ? c1 : c0;
            const cx<dd> kc = Js[cq], mx = Js[16 + cq], my = Js[32 + cq];
#pragma unroll
            for (int aq = 0; aq < 2; aq++) {
              comp_cmac(ea[2 * aq + bq], Ir[aq][0], kc);
              comp_cmac(em[2 * aq + bq], Ir[aq][1], mx);
              comp_cmac(em[2 * aq + bq], Ir[aq][2], my);
            }
          }
        }
      }
    }
#pragma unroll
    for (int e = 0; e < 4; e++) {
      double q[4] = {(double) ea[e][0] + (double) ea[e][1], (double) ea[e][2] + (double) ea[e][3],
                     (double) em[e][0] + (double) em[e][1], (double) em[e][2] + (double) em[e][3]};
#pragma unroll
      for (int c = 0; c < 4; c++) {
        q[c] += __shfl_xor_sync(0xffffffffu, q[c], 1);
        q[c] += __shfl_xor_sync(0xffffffffu, q[c], 2);
        q[c] += __shfl_xor_sync(0xffffffffu, q[c], 4);
      }
      const int aq = e >> 1, bq = e & 1;
      const int rl = 2 * ti + aq, cl = 2 * tj + bq;
      if (g == 0 && live && rl < m && cl < m && rl >= cl) {
        double* o = out + (size_t) (rl * (rl + 1) / 2 + cl) * 4;
        o[0] = axy * q[0] + q[2];
        o[1] = axy * q[1] + q[3];
        o[2] = q[2];
        o[3] = q[3];
      }
    }
  }
}

static size_t gram_split_smem() {
  const size_t f = sizeof(cx<float>) * GS_S * (GS_IS + GS_JS);
  const size_t d = sizeof(cx<dd>) * GS_S * GS_DS * 2;
  return f > d ? f : d;
}


static int gram_chunks(int K, size_t nsite) {
  int c = (g_tuning.gram_waves * sm_count() + K - 1) / K;
  if (c < 8) c = 8;
  if (c > 256) c = 256;
  size_t maxc = (nsite + TS - 1) / TS;
  if ((size_t) c > maxc) c = (int) maxc;
  return c;
}

extern "C" int mxk_block_gram(int n, int m, int K, const double* ph, mxk_kappa kap, int nb, const int* precs,
                              const void* const* ptrs, const void* resid, const double* theta, double* ga,
                              double* gm, double* scratch, size_t scratch_bytes, mx_stream s) {
  if (nb < 1 || nb > 4 || nb * m > 96) return (int) cudaErrorInvalidValue;
  GramArgs a;
  a.n = n; a.m = m; a.K = K; a.nb = nb; a.ns = nb * m;
  for (int b = 0; b < 4; b++) {
    a.precs[b] = b < nb ? precs[b] : MX_C64;
    a.ptrs[b] = b < nb ? ptrs[b] : nullptr;
  }
  a.ph = ph; a.kap = kap;
  a.resid = (const float2*) resid;
  a.theta = theta;
  a.sixth = make_sc(1.0 / 6.0);
  int nent = a.ns * (a.ns + 1) / 2;
  a.chunks = gram_chunks(K, (size_t) n * n);
  size_t need = (size_t) K * a.chunks * nent * 4 * sizeof(double);
  while (need > scratch_bytes && a.chunks > 1) {
    a.chunks /= 2;
    need = (size_t) K * a.chunks * nent * 4 * sizeof(double);
  }
  if (need > scratch_bytes) return (int) cudaErrorMemoryAllocation;
  a.partial = scratch;
  cudaStream_t st = (cudaStream_t) s;
  dim3 g(a.chunks, K);
  bool all128 = true;
  for (int b = 0; b < nb; b++) all128 = all128 && precs[b] == MX_C128;
  bool hi_dd = precs[0] == MX_CDD;
  int mh = all128 ? a.ns : (precs[0] == MX_C64 ? 0 : m);
  size_t hsz = hi_dd ? sizeof(cx<dd>) : sizeof(cx<double>);
  if (resid && (all128 || mh == 0)) return (int) cudaErrorInvalidValue;
  size_t smem = hsz * TS * mh * 5 + sizeof(cx<float>) * TS * a.ns * 5 + (hsz / 2 + sizeof(float)) * TS
                + sizeof(cx<float>) * TS * mh * 2 + 16;
  bool lo_rest = true;
  for (int q = 1; q < nb; q++) lo_rest = lo_rest && precs[q] == MX_C64;
  if (hi_dd && lo_rest && m <= 16 && nb <= 3 && (nb == 1 || resid)) {
    size_t sm = gram_split_smem();
    cudaFuncSetAttribute(k_block_gram_split, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sm);
    k_block_gram_split<<<dim3(a.chunks, K, nb > 1 ? 2 : 1), GS_T, sm, st>>>(a);
  } else if (hi_dd) {
    cudaFuncSetAttribute(k_block_gram<dd>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    for (int eb = 0; eb < nent; eb += 5 * GT) k_block_gram<dd><<<g, GT, smem, st>>>(a, mh, eb);
  } else {
    cudaFuncSetAttribute(k_block_gram<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    for (int eb = 0; eb < nent; eb += 5 * GT) k_block_gram<double><<<g, GT, smem, st>>>(a, mh, eb);
  }
  MX_CHECK_LAUNCH();
  size_t work = (size_t) nent * K;
  k_gram_reduce<<<(unsigned) ((work + 255) / 256), 256, 0, st>>>(a.ns, K, a.chunks, scratch, ga, gm);
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_block_combine(int n, int m, int K, int nb, const int* precs, const void* const* ptrs,
                                 const double* coef, int ldc, int row0, void* cwork, int pout, void* out,
                                 mx_stream s) {
  if (nb < 1 || nb > 4) return (int) cudaErrorInvalidValue;
  CombArgs a;
  a.n = n; a.m = m; a.K = K; a.nb = nb; a.ldc = ldc; a.row0 = row0; a.coef = coef;
  a.cpair = (const float4*) cwork;
  size_t nc = (size_t) K * ldc * m;
  k_coef_pairs<<<(unsigned) ((nc + 255) / 256), 256, 0, (cudaStream_t) s>>>(coef, (float4*) cwork, nc);
  MX_CHECK_LAUNCH();
  for (int b = 0; b < 4; b++) {
    a.precs[b] = b < nb ? precs[b] : MX_C64;
    a.ptrs[b] = b < nb ? ptrs[b] : nullptr;
  }
  cudaStream_t st = (cudaStream_t) s;
  bool rest64 = true;
  for (int q = 1; q < nb; q++) rest64 = rest64 && precs[q] == MX_C64;
  bool first_ok = precs[0] == MX_CDD || precs[0] == MX_C64;
  int nfloat = precs[0] == MX_CDD ? nb - 1 : nb;
  // the tiles' cp.async copies need 16-byte aligned sources and an even
  // entry count per tile (2 n^2 m entries per k-point: even)
  bool aligned = true;
  for (int q = 0; q < nb; q++) aligned = aligned && ((uintptr_t) ptrs[q] & 15) == 0;
  if (m <= 16 && nfloat <= 2 && first_ok && rest64 && aligned &&
      (pout == MX_CDD || (pout == MX_C64 && precs[0] == MX_C64))) {
    // one wave of CTAs, combine_ctas per SM, each walking tiles of its k-point
    size_t ntiles = (2 * (size_t) n * n + CTE - 1) / CTE;
    size_t want = (size_t) g_tuning.combine_ctas * sm_count() / (size_t) K;
    if (want < 1) want = 1;
    unsigned gx = (unsigned) (ntiles < want ? ntiles : want);
    dim3 g2(gx, K);
    size_t sm = combine_tiled_smem();
    if (pout == MX_CDD) {
      cudaFuncSetAttribute(k_block_combine_tiled<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sm);
      k_block_combine_tiled<true><<<g2, CT, sm, st>>>(a, out);
    } else {
      cudaFuncSetAttribute(k_block_combine_tiled<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sm);
      k_block_combine_tiled<false><<<g2, CT, sm, st>>>(a, out);
    }
    MX_CHECK_LAUNCH();
    return 0;
  }
  if (m > 256) return (int) cudaErrorInvalidValue;
  unsigned rows = 256 / m;
  dim3 g((unsigned) ((2 * (size_t) n * n + rows - 1) / rows), K), b(m, rows);
  size_t ncoef = (size_t) nb * m * m;
  // the coefficients staged per block exceed the default 48 KB for blocks
  // of more than about 24 vectors
  if (pout == MX_CDD) {
    size_t sm = ncoef * (sizeof(cx<dd>) + sizeof(cx<float>));
    cudaFuncSetAttribute(k_block_combine<cdd, dd>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sm);
    k_block_combine<cdd, dd><<<g, b, sm, st>>>(a, (cdd*) out);
  } else if (pout == MX_C128) {
    size_t sm = ncoef * (sizeof(cx<double>) + sizeof(cx<float>));
    cudaFuncSetAttribute(k_block_combine<double2, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sm);
    k_block_combine<double2, double><<<g, b, sm, st>>>(a, (double2*) out);
  } else {
    size_t sm = ncoef * (sizeof(cx<float>) * 2);
    cudaFuncSetAttribute(k_block_combine<float2, float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sm);
    k_block_combine<float2, float><<<g, b, sm, st>>>(a, (float2*) out);
  }
  MX_CHECK_LAUNCH();
  return 0;
}

// ------------------------------------------------------------------
// column selection of the Ritz basis from the residual statistics: column
// i of block j of k-point k stays when j == 0 (the eigenvector block), when
// every column is wanted, or while residual i of k has not met the
// tolerance (soft locking), the residual norm formed as the host forms it
// from the same statistics
// ------------------------------------------------------------------
namespace {
__global__ void k_select_columns(int ns, int m, int K, const double* __restrict__ stats,
                                 const double* __restrict__ mu, double tol, int relative, int all, int* sel) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ns * K) return;
  int k = t / ns, c = t % ns, j = c / m, i = c % m;
  int keep = 1;
  if (j != 0 && !all) {
    const double* st = stats + ((size_t) k * m + i) * 5;
    double r = sqrt(st[0] > 0.0 ? st[0] : 0.0);
    if (relative) r /= fabs(mu[(size_t) k * m + i]) * sqrt(st[1]) + 1e-300;
    keep = !(r <= tol);
  }
  sel[t] = keep;
}
}  // namespace

extern "C" int mxk_select_columns(int ns, int m, int K, const double* stats, const double* mu, double tol,
                                  int relative, int all, int* sel, mx_stream s) {
  k_select_columns<<<(ns * K + 255) / 256, 256, 0, (cudaStream_t) s>>>(ns, m, K, stats, mu, tol, relative, all,
                                                                      sel);
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_eps_sensitivity(int n, int m, int K, const double* ph, const double* kappa, const double* w,
                                   int pe, const void* e, double* grad, mx_stream s) {
  size_t nc = (size_t) n * n;
  dim3 g((unsigned) ((nc + 255) / 256)), b(256);
  cudaStream_t st = (cudaStream_t) s;
  if (pe == MX_CDD) k_eps_sensitivity<cdd, dd><<<g, b, 0, st>>>(n, m, K, ph, kappa, w, (const cdd*) e, grad);
  else if (pe == MX_C128) k_eps_sensitivity<double2, double><<<g, b, 0, st>>>(n, m, K, ph, kappa, w, (const double2*) e, grad);
  else k_eps_sensitivity<float2, float><<<g, b, 0, st>>>(n, m, K, ph, kappa, w, (const float2*) e, grad);
  MX_CHECK_LAUNCH();
  return 0;
}
