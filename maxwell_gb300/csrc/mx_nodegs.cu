// Node Gauss-Seidel sweep (node2d.c:629-1138), out of place and tiled.
//
// The reference sweeps in place: row 0, the odd rows 1..n-3, the even rows
// 2..n-2, row n-1, each row point by point along i.  Inside a row the
// update is x_t = x_{t-1}/8 + beta_t, with beta_t built from old values
// (the right neighbour x_{t+1}, rows j-1 and j+1 at t-1, t, t+1, and b_t);
// unrolled, x_t = sum_{d=0..t} 8^-d beta_{t-d}, truncated after D terms
// (8^-(D+1) below the unit roundoff: D = 8 in FP32).  Position 0 of a row
// starts the recurrence ("cut": x_0 = beta_0 + x_{-1}/8 with the old,
// phase-wrapped x_{n-1}); position n-1 reads the new x_0 of its own row
// through the seam.
//
// This kernel reads the old vector x and writes the new one into y, so
// that every new value is a fixed function of old values and a tile can
// recompute the few new values its neighbours own (halos) instead of
// waiting for them:
//   * launch 1: row 0, from old rows n-1 (seam) and 1;
//   * launch 2: rows 1..n-2 in pairs (odd 2q+1, even 2q+2).  A CTA owns a
//     strip of T positions of a band of pairs of one k-point and VB of the
//     m vectors, walks down the band and keeps its rows in shared memory.
//     An odd row needs old rows only (row 0 is read from y); an even row
//     needs the new odd rows above and below it, so the band recomputes the
//     first odd row of the next band without writing it; the even row n-2
//     reads the old row n-1;
//   * launch 3: row n-1, from the new rows n-2 and 0.
// Along i, an even row's new values at [t0, t0+T) need the new odd values
// at [t0-D-1, t0+T+2), which need old values at [t0-2D-2, t0+T+4): the
// strip stages that window, positions outside [0, n) wrapped with their
// Bloch phase.  The sweep runs in sweep coordinates (t, s): forward
// (t, s) = (i, j), backward (t, s) = (n-1-i, n-1-j) with conjugate phases,
// so one code path serves both directions.
//
// Each step of a CTA stages, by cp.async one step ahead, the two next old
// rows and the two b rows; a step is four phases separated by barriers:
// betas of the odd row (runs of RL positions per thread, a sliding window
// over the neighbour rows), its truncated prefix sums (Horner over the D
// betas before a run, then the recurrence), the betas of the even row, its
// prefix sums.
#include "mx_common.cuh"
#include "mx_internal.h"

using namespace mx;

namespace {

__device__ __forceinline__ void cpa16(void* dst, const void* src) {
  unsigned d = (unsigned) __cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cpa_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cpa_wait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

struct NgsArgs {
  int n, m, K, T, bwd;
  int G;           // vector groups of a k-point (m / VB)
  int qb;          // pairs per band
  int s1;          // the row of a single-row launch (0 or n-1)
  const void* b;
  const void* x;   // old values (read only)
  void* y;         // new values
  const double* ph;
  Sc inv_ac, third;
};

// The CTA's view: strip [t0, t0+T) of k-point k, vectors [v0, v0+VB).
// Shared buffers hold W = T + HL + HR positions x VB vectors, position u
// at slot u - base.
template <typename S, typename R, int D, int VB, int RL>
struct Tile {
  static constexpr int HL = 2 * D + 2, HR = 4;
  static constexpr int CPS = VB * (int) sizeof(S) / 16;   // 16-byte chunks per site
  int n, m, T, W, bwd, t0, base, v0, k;
  cx<R> pl, pr, pb, pa;   // phases of positions u < 0, u >= n, rows s < 0, s >= n
  R inv_ac, third;

  __device__ Tile(const NgsArgs& a, int strip, int g, int k_) {
    n = a.n; m = a.m; T = a.T; W = T + HL + HR; bwd = a.bwd;
    t0 = strip * T; base = t0 - HL; v0 = g * VB; k = k_;
    const Seam<R> sm = seam_load<R>(a.ph, a.K, k, n);
    const cx<R> xs = bwd ? conjc(sm.xf) : sm.xf, ys = bwd ? conjc(sm.yf) : sm.yf;
    pl = conjc(xs); pr = xs; pb = conjc(ys); pa = ys;
    inv_ac = sget<R>(a.inv_ac); third = sget<R>(a.third);
  }
  __device__ __forceinline__ int canon(int u) const { return u < 0 ? u + n : (u >= n ? u - n : u); }
  // element (sweep row s in [-1, n], canonical position c) of a node array
  __device__ __forceinline__ size_t at(int s, int c) const {
    const int sj = s < 0 ? s + n : (s >= n ? s - n : s);
    const int j = bwd ? n - 1 - sj : sj, i = bwd ? n - 1 - c : c;
    return (((size_t) k * n + j) * n + i) * m + v0;
  }
  // stage the window of sweep row s of src into buf (raw values)
  __device__ __forceinline__ void stage(S* buf, const S* src, int s, int tid, int nth) const {
    const int nch = W * CPS;
    for (int q = tid; q < nch; q += nth) {
      const int w = q / CPS, part = q - w * CPS;
      const char* g = reinterpret_cast<const char*>(src + at(s, canon(base + w))) + 16 * part;
      cpa16(reinterpret_cast<char*>(buf + (size_t) w * VB) + 16 * part, g);
    }
  }
  // multiply the wrapped positions of a staged row (and the whole row, if
  // row s lies across the seam) by their phases
  __device__ __forceinline__ void fix(S* buf, int s, int tid, int nth) const {
    const bool rw = s < 0 || s >= n;
    const cx<R> rp = s < 0 ? pb : pa;
    for (int q = tid; q < W * VB; q += nth) {
      const int u = base + q / VB;
      if (!rw && u >= 0 && u < n) continue;
      cx<R> p = u < 0 ? pl : (u >= n ? pr : mkc(rc<R>(1.0f), Real<R>::zero()));
      if (rw) p = p * rp;
      S* e = buf + q;
      Store<S, R>::st(e, p * Store<S, R>::ld(e));
    }
  }
  // the row s of a node array at position 0 of vector v0
  __device__ __forceinline__ size_t row(int s) const {
    const int j = bwd ? n - 1 - s : s;
    return (((size_t) k * n + j) * n) * m + v0;
  }
  __device__ __forceinline__ bool edge() const { return base < 0 || t0 + T + HR > n; }
  __device__ __forceinline__ cx<R> L(const S* buf, int u, int v) const {
    return Store<S, R>::ld(buf + (size_t) (u - base) * VB + v);
  }

  // betas of positions [ua, ub) of a row: below / above are the rows s-1 and
  // s+1 (old or new), own the row's old values, bb its right-hand side
  __device__ void betas(int ua, int ub, const S* below, const S* above, const S* own, const S* bb, S* beta,
                        int tid, int nth) const {
    const R eighth = rc<R>(0.125f);
    const int nrun = (ub - ua + RL - 1) / RL;
    for (int task = tid; task < nrun * VB; task += nth) {
      const int v = task % VB, p0 = ua + (task / VB) * RL, p1 = p0 + RL < ub ? p0 + RL : ub;
      cx<R> cm = L(below, p0 - 1, v) + L(above, p0 - 1, v);
      cx<R> c0 = L(below, p0, v) + L(above, p0, v);
      for (int u = p0; u < p1; u++) {
        const cx<R> cp = L(below, u + 1, v) + L(above, u + 1, v);
        const int c = canon(u);
        cx<R> nxt;
        if (c == n - 1) {
          // the new value at the cut u+1, from old values around it
          const cx<R> cpp = L(below, u + 2, v) + L(above, u + 2, v);
          nxt = scal(inv_ac, L(bb, u + 1, v) + scal(third, L(own, u + 2, v) + ((c0 + cp) + cpp)))
                + scal(eighth, L(own, u, v));
        } else {
          nxt = L(own, u + 1, v);
        }
        cx<R> be = scal(inv_ac, L(bb, u, v) + scal(third, nxt + ((cm + c0) + cp)));
        if (c == 0) be = be + scal(eighth, L(own, u - 1, v));
        Store<S, R>::st(beta + (size_t) (u - base) * VB + v, be);
        cm = c0;
        c0 = cp;
      }
    }
  }
  // new values of positions [ua, ub): into out (shared, may be null) and,
  // for positions in [t0, t0+T), into the row of y at yrow (may be null)
  __device__ void prefix(int ua, int ub, const S* beta, S* out, S* yrow, int tid, int nth) const {
    const R eighth = rc<R>(0.125f);
    const int nrun = (ub - ua + RL - 1) / RL;
    for (int task = tid; task < nrun * VB; task += nth) {
      const int v = task % VB, p0 = ua + (task / VB) * RL, p1 = p0 + RL < ub ? p0 + RL : ub;
      const int c0 = canon(p0), dmax = c0 < D ? c0 : D;
      cx<R> acc = czero<R>();
      for (int d = dmax; d >= 1; d--) acc = scal(eighth, acc) + L(beta, p0 - d, v);
      for (int u = p0; u < p1; u++) {
        const cx<R> be = L(beta, u, v);
        acc = canon(u) == 0 ? be : scal(eighth, acc) + be;
        if (out) Store<S, R>::st(out + (size_t) (u - base) * VB + v, acc);
        if (yrow && u >= t0 && u < t0 + T) Store<S, R>::st(yrow + (size_t) (bwd ? n - 1 - u : u) * m + v, acc);
      }
    }
  }
};

// launch 2: rows 1..n-2, grid (G x strips, bands, K)
template <typename S, typename R, int D, int VB, int RL>
__global__ void __launch_bounds__(128) k_node_gs_tile(NgsArgs a) {
  using TT = Tile<S, R, D, VB, RL>;
  extern __shared__ __align__(16) unsigned char smraw[];
  const TT t(a, blockIdx.x / a.G, blockIdx.x % a.G, blockIdx.z);
  const int tid = threadIdx.x, nth = blockDim.x, n = t.n, t0 = t.t0, T = t.T;
  const int Q = (n - 2) / 2, q0 = blockIdx.y * a.qb, q1 = q0 + a.qb < Q ? q0 + a.qb : Q;
  if (q0 >= Q) return;
  const size_t BS = (size_t) t.W * VB;
  S* sm = reinterpret_cast<S*>(smraw);
  S* old = sm;                 // 5 rows, slot s % 5
  S* bsm = sm + 5 * BS;        // 4 rows: (step & 1) * 2 + {odd, even}
  S* odd = sm + 9 * BS;        // 2 rows: step & 1
  S* beta = sm + 11 * BS;
  const S* X = reinterpret_cast<const S*>(a.x);
  const S* B = reinterpret_cast<const S*>(a.b);
  S* Y = reinterpret_cast<S*>(a.y);
  const bool edge = t.edge();
  const int nsteps = q1 - q0 + 1;

  // prologue: the rows and b of the first odd row (row 0 comes from y)
  {
    const int o = 2 * q0 + 1;
    for (int s = o - 1; s <= o + 1; s++) t.stage(old + (s % 5) * BS, s == 0 ? Y : X, s, tid, nth);
    t.stage(bsm, B, o, tid, nth);
    cpa_commit();
  }
  for (int i = 0; i < nsteps; i++) {
    const int o = 2 * (q0 + i) + 1, e = o - 1;
    // stage step i+1: rows o+2 and o+3, b of its odd and even rows, into
    // slots that step i-1 used last
    if (i + 1 < nsteps) {
      const int o2 = o + 2;
      t.stage(old + (o2 % 5) * BS, X, o2, tid, nth);
      if (o2 + 1 <= n - 1) t.stage(old + ((o2 + 1) % 5) * BS, X, o2 + 1, tid, nth);
      S* bn = bsm + (size_t) ((i + 1) & 1) * 2 * BS;
      if (o2 <= n - 2) t.stage(bn, B, o2, tid, nth);
      t.stage(bn + BS, B, o2 - 1, tid, nth);
    }
    cpa_commit();
    cpa_wait1();
    __syncthreads();
    S* bo = bsm + (size_t) (i & 1) * 2 * BS;
    if (edge) {
      if (i == 0) t.fix(old + ((o - 1) % 5) * BS, o - 1, tid, nth);
      t.fix(old + (o % 5) * BS, o, tid, nth);
      if (o + 1 <= n - 1) t.fix(old + ((o + 1) % 5) * BS, o + 1, tid, nth);
      if (o <= n - 2) t.fix(bo, o, tid, nth);
      if (i > 0) t.fix(bo + BS, e, tid, nth);
      __syncthreads();
    }
    const S* above;
    if (o <= n - 2) {
      S* on = odd + (size_t) (i & 1) * BS;
      t.betas(t0 - 2 * D - 1, t0 + T + 2, old + ((o - 1) % 5) * BS, old + ((o + 1) % 5) * BS, old + (o % 5) * BS,
              bo, beta, tid, nth);
      __syncthreads();
      // the odd row of the next band is recomputed here, not written
      t.prefix(t0 - D - 1, t0 + T + 2, beta, on, i < q1 - q0 ? Y + t.row(o) : nullptr, tid, nth);
      __syncthreads();
      above = on;
    } else {
      above = old + (o % 5) * BS;   // the even row n-2 reads the old row n-1
    }
    if (i > 0) {
      t.betas(t0 - D, t0 + T, odd + (size_t) ((i - 1) & 1) * BS, above, old + (e % 5) * BS, bo + BS, beta, tid,
              nth);
      __syncthreads();
      t.prefix(t0, t0 + T, beta, nullptr, Y + t.row(e), tid, nth);
    }
    __syncthreads();
  }
  cpa_wait0();
}

// launches 1 and 3: the single row s1 (0 or n-1 in sweep order), grid
// (G x strips, 1, K).  Row 0 reads the old rows -1 (the seam) and 1; row
// n-1 reads the new rows n-2 and n (the seam: row 0).
template <typename S, typename R, int D, int VB, int RL>
__global__ void __launch_bounds__(128) k_node_gs_single(NgsArgs a) {
  using TT = Tile<S, R, D, VB, RL>;
  extern __shared__ __align__(16) unsigned char smraw[];
  const TT t(a, blockIdx.x / a.G, blockIdx.x % a.G, blockIdx.z);
  const int tid = threadIdx.x, nth = blockDim.x, t0 = t.t0, T = t.T, s = a.s1;
  const size_t BS = (size_t) t.W * VB;
  S* sm = reinterpret_cast<S*>(smraw);
  const S* X = reinterpret_cast<const S*>(a.x);
  const S* nbr = s == 0 ? X : reinterpret_cast<const S*>(a.y);
  t.stage(sm, nbr, s - 1, tid, nth);
  t.stage(sm + BS, nbr, s + 1, tid, nth);
  t.stage(sm + 2 * BS, X, s, tid, nth);
  t.stage(sm + 3 * BS, reinterpret_cast<const S*>(a.b), s, tid, nth);
  cpa_commit();
  cpa_wait0();
  __syncthreads();
  t.fix(sm, s - 1, tid, nth);
  t.fix(sm + BS, s + 1, tid, nth);
  if (t.edge()) {
    t.fix(sm + 2 * BS, s, tid, nth);
    t.fix(sm + 3 * BS, s, tid, nth);
  }
  __syncthreads();
  t.betas(t0 - D, t0 + T, sm, sm + BS, sm + 2 * BS, sm + 3 * BS, sm + 4 * BS, tid, nth);
  __syncthreads();
  t.prefix(t0, t0 + T, sm + 4 * BS, nullptr, reinterpret_cast<S*>(a.y) + t.row(s), tid, nth);
}

template <typename S, typename R, int D, int VB, int RL>
int run_sweep(int n, int m, int K, const double* ph, double alpha, int bwd, int T, int qb, const void* b,
              const void* x, void* y, cudaStream_t st) {
  using TT = Tile<S, R, D, VB, RL>;
  NgsArgs a;
  a.n = n; a.m = m; a.K = K; a.T = T; a.bwd = bwd; a.G = m / VB; a.qb = qb; a.s1 = 0;
  a.b = b; a.x = x; a.y = y; a.ph = ph;
  a.inv_ac = make_sc(3.0 / (8.0 * alpha));
  a.third = make_sc(alpha / 3.0);
  const int W = T + TT::HL + TT::HR;
  const size_t BS = (size_t) W * VB * sizeof(S);
  int nth = VB * ((T + 2 * D + 3 + RL - 1) / RL);
  nth = (nth + 31) / 32 * 32;
  if (nth > 128) return (int) cudaErrorInvalidConfiguration;
  const unsigned gx = (unsigned) (a.G * (n / T));
  cudaFuncSetAttribute(k_node_gs_tile<S, R, D, VB, RL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int) (12 * BS));
  cudaFuncSetAttribute(k_node_gs_single<S, R, D, VB, RL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int) (5 * BS));
  k_node_gs_single<S, R, D, VB, RL><<<dim3(gx, 1, K), nth, 5 * BS, st>>>(a);
  MX_CHECK_LAUNCH();
  const int Q = (n - 2) / 2;
  k_node_gs_tile<S, R, D, VB, RL><<<dim3(gx, (Q + qb - 1) / qb, K), nth, 12 * BS, st>>>(a);
  MX_CHECK_LAUNCH();
  a.s1 = n - 1;
  k_node_gs_single<S, R, D, VB, RL><<<dim3(gx, 1, K), nth, 5 * BS, st>>>(a);
  MX_CHECK_LAUNCH();
  return 0;
}

// strip 0: the tiled sweep is off and callers use the in-place row kernels
int g_strip = 0, g_band = 16;

}  // namespace

// The strip width for n: the largest of 128 and 64 that divides n and
// leaves the staged window (T + 2D + 6 positions) shorter than a row.
static int strip_for(int n) {
  for (int T = g_strip; T >= 64; T /= 2)   // (no strip when g_strip is 0)
    if (n % T == 0 && T + 2 * 8 + 6 < n) return T;
  return 0;
}

extern "C" int mxk_node_gs_oop_ok(int n, int m, int prec) {
  return prec == MX_C64 && m % 4 == 0 && m >= 4 && (n & 1) == 0 && strip_for(n) > 0;
}

extern "C" int mxk_node_gs_oop_shape(int strip, int band) {
  if ((strip != 0 && strip != 64 && strip != 128) || band < 1 || band > 256) return (int) cudaErrorInvalidValue;
  g_strip = strip;
  g_band = band;
  return 0;
}
extern "C" void mxk_node_gs_oop_get_shape(int* strip, int* band) {
  *strip = g_strip;
  *band = g_band;
}

// One sweep (dir 0 forward, 1 backward) from x into y; b, x and y distinct,
// 16-byte aligned.
extern "C" int mxk_node_gs_oop(int n, int m, int K, const double* ph, double alpha, int dir, int prec,
                               const void* b, const void* x, void* y, mx_stream s) {
  if (!mxk_node_gs_oop_ok(n, m, prec) || (dir != 0 && dir != 1) || x == y || b == y) return (int) cudaErrorInvalidValue;
  if (((uintptr_t) b | (uintptr_t) x | (uintptr_t) y) & 15) return (int) cudaErrorMisalignedAddress;
  return run_sweep<float2, float, 8, 4, 5>(n, m, K, ph, alpha, dir, strip_for(n), g_band, b, x, y,
                                            (cudaStream_t) s);
}
