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
// Each step of a CTA stages, by cp.async P steps ahead, its two next old
// rows and its two b rows; a step is four phases separated by barriers:
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
template <int N>
__device__ __forceinline__ void cpa_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

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
// at slot u - base.  A thread has at most one run of RL positions per
// phase (task = thread); runs away from the row ends and the seam take a
// fast path with fixed shared-memory offsets and no per-position tests,
// and the right-hand side of a fast run is loaded into registers one phase
// before it is used.
template <typename S, typename R, int D, int VB, int RL, int T, int NTH>
struct Tile {
  static constexpr int HL = 2 * D + 2, HR = 4, W = T + HL + HR;
  static constexpr int EPC = 16 / (int) sizeof(S);        // elements per 16-byte chunk
  static constexpr int NCH = W * VB / EPC;                 // chunks per staged row
  static constexpr int NR = (NCH + NTH - 1) / NTH;         // chunks per thread
  int n, m, bwd, t0, base, v0, k;
  cx<R> pl, pr, pb, pa;   // phases of positions u < 0, u >= n, rows s < 0, s >= n
  R inv_ac, third;
  int goff[NR], soff[NR];  // this thread's chunks: element offsets in a row / in a buffer

  __device__ Tile(const NgsArgs& a, int strip, int g, int k_, int tid) {
    n = a.n; m = a.m; bwd = a.bwd;
    t0 = strip * T; base = t0 - HL; v0 = g * VB; k = k_;
    const Seam<R> sm = seam_load<R>(a.ph, a.K, k, n);
    const cx<R> xs = bwd ? conjc(sm.xf) : sm.xf, ys = bwd ? conjc(sm.yf) : sm.yf;
    pl = conjc(xs); pr = xs; pb = conjc(ys); pa = ys;
    inv_ac = sget<R>(a.inv_ac); third = sget<R>(a.third);
#pragma unroll
    for (int r = 0; r < NR; r++) {
      const int q = tid + r * NTH;
      const int w = q * EPC / VB, e = q * EPC - w * VB;
      const int c = canon(base + w);
      goff[r] = (bwd ? n - 1 - c : c) * m + e;
      soff[r] = q < NCH ? w * VB + e : -1;
    }
  }
  __device__ __forceinline__ int canon(int u) const { return u < 0 ? u + n : (u >= n ? u - n : u); }
  __device__ __forceinline__ int col(int u) const { return bwd ? n - 1 - u : u; }   // u in [0, n)
  // the row s (sweep order, -1 and n through the seam) of a node array at i = 0
  __device__ __forceinline__ size_t row(int s) const {
    const int sj = s < 0 ? s + n : (s >= n ? s - n : s);
    const int j = bwd ? n - 1 - sj : sj;
    return (((size_t) k * n + j) * n) * m + v0;
  }
  __device__ __forceinline__ void stage(S* buf, const S* src, int s) const {
    const S* rp = src + row(s);
#pragma unroll
    for (int r = 0; r < NR; r++)
      if (soff[r] >= 0) cpa16(buf + soff[r], rp + goff[r]);
  }
  // multiply the wrapped positions of a staged row (the whole row, if row s
  // lies across the seam) by their phases
  __device__ void fix(S* buf, int s, int tid) const {
    const bool rw = s < 0 || s >= n;
    const cx<R> one = mkc(rc<R>(1.0f), Real<R>::zero());
    const cx<R> rp = rw ? (s < 0 ? pb : pa) : one;
    const int lo = rw ? W : (base < 0 ? -base : 0);            // slots [0, lo) wrap left
    const int hi = rw ? W : (base + W > n ? n - base : W);     // slots [hi, W) wrap right
    for (int q = tid; q < W * VB; q += NTH) {
      const int w = q / VB, u = base + w;
      if (!rw && w >= lo && w < hi) continue;
      const cx<R> p = (u < 0 ? pl : (u >= n ? pr : one)) * rp;
      Store<S, R>::st(buf + q, p * Store<S, R>::ld(buf + q));
    }
  }
  __device__ __forceinline__ bool edge() const { return base < 0 || base + W > n; }
  __device__ __forceinline__ cx<R> L(const S* buf, int u, int v) const {
    return Store<S, R>::ld(buf + (size_t) (u - base) * VB + v);
  }
  // the run [p0, p0+len) of task `task` over [ua, ub); fast: a full run
  // whose betas read canonical positions 1..n-2 only
  __device__ __forceinline__ bool run_of(int task, int ua, int ub, int& v, int& p0, int& len) const {
    v = task % VB;
    p0 = ua + (task / VB) * RL;
    len = ub - p0 < RL ? ub - p0 : RL;
    return len == RL && p0 - 1 >= 1 && p0 + RL + 1 <= n - 2;
  }
  // betas of positions [ua, ub) of a row: below / above are the rows s-1 and
  // s+1 (old or new), own the row's old values, bb its right-hand side
  __device__ void betas(int task, int ua, int ub, const S* below, const S* above, const S* own, const S* bb,
                        S* beta) const {
    int v, p0, len;
    if (task >= ((ub - ua + RL - 1) / RL) * VB) return;
    const R eighth = rc<R>(0.125f);
    if (run_of(task, ua, ub, v, p0, len)) {
      const int o = (p0 - base) * VB + v;
      const S *pb_ = below + o, *pa_ = above + o, *po = own + o, *pr_ = bb + o;
      S* pz = beta + o;
      cx<R> cm = Store<S, R>::ld(pb_ - VB) + Store<S, R>::ld(pa_ - VB);
      cx<R> c0 = Store<S, R>::ld(pb_) + Store<S, R>::ld(pa_);
#pragma unroll
      for (int q = 0; q < RL; q++) {
        const cx<R> cp = Store<S, R>::ld(pb_ + (q + 1) * VB) + Store<S, R>::ld(pa_ + (q + 1) * VB);
        const cx<R> nb = (cm + c0) + cp;
        Store<S, R>::st(pz + q * VB, scal(inv_ac, Store<S, R>::ld(pr_ + q * VB)
                                                      + scal(third, Store<S, R>::ld(po + (q + 1) * VB) + nb)));
        cm = c0;
        c0 = cp;
      }
      return;
    }
    cx<R> cm = L(below, p0 - 1, v) + L(above, p0 - 1, v);
    cx<R> c0 = L(below, p0, v) + L(above, p0, v);
    for (int u = p0; u < p0 + len; u++) {
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
  // new values of positions [ua, ub): into out (shared, may be null) and,
  // for positions in [t0, t0+T), into the row of y at yrow (may be null)
  __device__ void prefix(int task, int ua, int ub, const S* beta, S* out, S* yrow) const {
    int v, p0, len;
    if (task >= ((ub - ua + RL - 1) / RL) * VB) return;
    run_of(task, ua, ub, v, p0, len);
    const R eighth = rc<R>(0.125f);
    // a cut (position 0 mod n) among the D betas before the run or in it
    const int a = p0 - D, b = p0 + len - 1;
    const bool cut = (a <= 0 && b >= 0) || (a <= n && b >= n);
    cx<R> acc = czero<R>();
    if (len == RL && !cut) {
      const int o = (p0 - base) * VB + v;
      const S* pz = beta + o;
#pragma unroll
      for (int d = D; d >= 1; d--) acc = scal(eighth, acc) + Store<S, R>::ld(pz - d * VB);
      const bool in0 = p0 >= t0 && p0 + RL <= t0 + T;
      S* yp = yrow ? yrow + (size_t) (p0 >= 0 && p0 < n ? col(p0) : 0) * m + v : nullptr;
      const int st = bwd ? -m : m;
#pragma unroll
      for (int q = 0; q < RL; q++) {
        acc = scal(eighth, acc) + Store<S, R>::ld(pz + q * VB);
        if (out) Store<S, R>::st(out + o + q * VB, acc);
        if (yp && (in0 || (p0 + q >= t0 && p0 + q < t0 + T))) Store<S, R>::st(yp + q * st, acc);
      }
      return;
    }
    const int c0 = canon(p0), dmax = c0 < D ? c0 : D;
    for (int d = dmax; d >= 1; d--) acc = scal(eighth, acc) + L(beta, p0 - d, v);
    for (int u = p0; u < p0 + len; u++) {
      const cx<R> be = L(beta, u, v);
      acc = canon(u) == 0 ? be : scal(eighth, acc) + be;
      if (out) Store<S, R>::st(out + (size_t) (u - base) * VB + v, acc);
      if (yrow && u >= t0 && u < t0 + T) Store<S, R>::st(yrow + (size_t) col(u) * m + v, acc);
    }
  }
};

// launch 2: rows 1..n-2, grid (G x strips, bands, K).  The copies run P
// steps ahead: rows in a ring of 2P+3 slots (slot s mod 2P+3), the b rows of
// a step's odd and even row in P+1 pairs of slots.
template <typename S, typename R, int D, int VB, int RL, int T, int NTH, int P>
__global__ void __launch_bounds__(NTH) k_node_gs_tile(NgsArgs a) {
  using TT = Tile<S, R, D, VB, RL, T, NTH>;
  constexpr int NO = 2 * P + 3, NB2 = P + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int tid = threadIdx.x;
  const TT t(a, blockIdx.x / a.G, blockIdx.x % a.G, blockIdx.z, tid);
  const int n = t.n, t0 = t.t0;
  const int Q = (n - 2) / 2, q0 = blockIdx.y * a.qb, q1 = q0 + a.qb < Q ? q0 + a.qb : Q;
  if (q0 >= Q) return;
  constexpr int BS = TT::W * VB;
  S* sm = reinterpret_cast<S*>(smraw);
  S* old = sm;                    // NO rows
  S* bsm = sm + NO * BS;          // NB2 pairs (odd, even)
  S* odd = bsm + 2 * NB2 * BS;    // 2 rows: step & 1
  S* beta = odd + 2 * BS;
  const S* X = reinterpret_cast<const S*>(a.x);
  const S* B = reinterpret_cast<const S*>(a.b);
  S* Y = reinterpret_cast<S*>(a.y);
  const bool edge = t.edge();
  const int nsteps = q1 - q0 + 1;
  // the phases' ranges: odd betas, odd new values, even betas / new values
  const int ob0 = t0 - 2 * D - 1, ob1 = t0 + T + 2, on0 = t0 - D - 1, on1 = t0 + T + 2;
  const int eb0 = t0 - D, eb1 = t0 + T;
  // what step j needs beyond the rows of step j-1 (row 0 comes from y)
  auto stage_step = [&](int j) {
    const int o = 2 * (q0 + j) + 1;
    S* bp = bsm + (j % NB2) * 2 * BS;
    if (j == 0) {
      for (int s = o - 1; s <= o + 1; s++) t.stage(old + (s % NO) * BS, s == 0 ? Y : X, s);
    } else {
      t.stage(old + (o % NO) * BS, X, o);
      if (o + 1 <= n - 1) t.stage(old + ((o + 1) % NO) * BS, X, o + 1);
      t.stage(bp + BS, B, o - 1);
    }
    if (o <= n - 2) t.stage(bp, B, o);
  };
#pragma unroll
  for (int j = 0; j < P; j++) {
    if (j < nsteps) stage_step(j);
    cpa_commit();
  }
  for (int i = 0; i < nsteps; i++) {
    const int o = 2 * (q0 + i) + 1, e = o - 1;
    if (i + P < nsteps) stage_step(i + P);   // into slots step i-1 used last
    cpa_commit();
    cpa_wait<P>();
    __syncthreads();
    S* bo = bsm + (i % NB2) * 2 * BS;
    if (edge) {
      if (i == 0) t.fix(old + ((o - 1) % NO) * BS, o - 1, tid);
      t.fix(old + (o % NO) * BS, o, tid);
      if (o + 1 <= n - 1) t.fix(old + ((o + 1) % NO) * BS, o + 1, tid);
      if (o <= n - 2) t.fix(bo, o, tid);
      if (i > 0) t.fix(bo + BS, e, tid);
      __syncthreads();
    }
    const S* above;
    if (o <= n - 2) {
      S* on = odd + (i & 1) * BS;
      t.betas(tid, ob0, ob1, old + ((o - 1) % NO) * BS, old + ((o + 1) % NO) * BS, old + (o % NO) * BS, bo, beta);
      __syncthreads();
      // the odd row of the next band is recomputed here, not written
      t.prefix(tid, on0, on1, beta, on, i < q1 - q0 ? Y + t.row(o) : nullptr);
      __syncthreads();
      above = on;
    } else {
      above = old + (o % NO) * BS;   // the even row n-2 reads the old row n-1
    }
    if (i > 0) {
      t.betas(tid, eb0, eb1, odd + ((i - 1) & 1) * BS, above, old + (e % NO) * BS, bo + BS, beta);
      __syncthreads();
      t.prefix(tid, eb0 + D, eb1, beta, nullptr, Y + t.row(e));
    }
    __syncthreads();
  }
  cpa_wait<0>();
}

// launches 1 and 3: the single row s1 (0 or n-1 in sweep order), grid
// (G x strips, 1, K).  Row 0 reads the old rows -1 (the seam) and 1; row
// n-1 reads the new rows n-2 and n (the seam: row 0).
template <typename S, typename R, int D, int VB, int RL, int T, int NTH>
__global__ void __launch_bounds__(NTH) k_node_gs_single(NgsArgs a) {
  using TT = Tile<S, R, D, VB, RL, T, NTH>;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int tid = threadIdx.x;
  const TT t(a, blockIdx.x / a.G, blockIdx.x % a.G, blockIdx.z, tid);
  const int t0 = t.t0, s = a.s1;
  constexpr int BS = TT::W * VB;
  S* sm = reinterpret_cast<S*>(smraw);
  const S* X = reinterpret_cast<const S*>(a.x);
  const S* nbr = s == 0 ? X : reinterpret_cast<const S*>(a.y);
  t.stage(sm, nbr, s - 1);
  t.stage(sm + BS, nbr, s + 1);
  t.stage(sm + 2 * BS, X, s);
  t.stage(sm + 3 * BS, reinterpret_cast<const S*>(a.b), s);
  cpa_commit();
  cpa_wait<0>();
  __syncthreads();
  t.fix(sm, s - 1, tid);
  t.fix(sm + BS, s + 1, tid);
  if (t.edge()) {
    t.fix(sm + 2 * BS, s, tid);
    t.fix(sm + 3 * BS, s, tid);
  }
  __syncthreads();
  t.betas(tid, t0 - D, t0 + T, sm, sm + BS, sm + 2 * BS, sm + 3 * BS, sm + 4 * BS);
  __syncthreads();
  t.prefix(tid, t0, t0 + T, sm + 4 * BS, nullptr, reinterpret_cast<S*>(a.y) + t.row(s));
}

template <typename S, typename R, int D, int VB, int RL, int T, int P>
int run_sweep(int n, int m, int K, const double* ph, double alpha, int bwd, int qb, const void* b, const void* x,
              void* y, cudaStream_t st) {
  // one run per thread in every phase: the longest phase has T + 2D + 3 positions
  constexpr int NTH = (VB * ((T + 2 * D + 3 + RL - 1) / RL) + 31) / 32 * 32;
  using TT = Tile<S, R, D, VB, RL, T, NTH>;
  NgsArgs a;
  a.n = n; a.m = m; a.K = K; a.T = T; a.bwd = bwd; a.G = m / VB; a.qb = qb; a.s1 = 0;
  a.b = b; a.x = x; a.y = y; a.ph = ph;
  a.inv_ac = make_sc(3.0 / (8.0 * alpha));
  a.third = make_sc(alpha / 3.0);
  const size_t BS = (size_t) TT::W * VB * sizeof(S);
  const unsigned gx = (unsigned) (a.G * (n / T));
  const size_t tile_smem = (size_t) (2 * P + 3 + 2 * (P + 1) + 3) * BS;
  cudaFuncSetAttribute(k_node_gs_tile<S, R, D, VB, RL, T, NTH, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int) tile_smem);
  k_node_gs_single<S, R, D, VB, RL, T, NTH><<<dim3(gx, 1, K), NTH, 5 * BS, st>>>(a);
  MX_CHECK_LAUNCH();
  const int Q = (n - 2) / 2;
  k_node_gs_tile<S, R, D, VB, RL, T, NTH, P><<<dim3(gx, (Q + qb - 1) / qb, K), NTH, tile_smem, st>>>(a);
  MX_CHECK_LAUNCH();
  a.s1 = n - 1;
  k_node_gs_single<S, R, D, VB, RL, T, NTH><<<dim3(gx, 1, K), NTH, 5 * BS, st>>>(a);
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
  if (strip_for(n) == 128)
    return run_sweep<float2, float, 8, 4, 5, 128, 2>(n, m, K, ph, alpha, dir, g_band, b, x, y, (cudaStream_t) s);
  return run_sweep<float2, float, 8, 4, 5, 64, 3>(n, m, K, ph, alpha, dir, g_band, b, x, y, (cudaStream_t) s);
}
