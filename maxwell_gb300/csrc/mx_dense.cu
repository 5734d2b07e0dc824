// Batched small dense complex linear algebra in FP64 (one CTA per k-point).
// These matrices are small (coarse grids of 2*8*8 = 128 edges, Ritz systems
// of at most 3m = 48 columns); the Jacobi sweeps of the Ritz step do most of
// their rotations in FP32 and finish in FP64 (jacobi_mixed).  They replace
// the reference's LAPACK calls (linalg.c:48-317):
//   mxk_hpd_inverse    zpotrf + ztrsm pairs of the coarse-grid solves
//   mxk_heev           zheev (cyclic Jacobi with Brent-Luk parallel ordering)
//   mxk_rayleigh_ritz  zhegv of the Ritz step, as Cholesky-QR of the Gram
//                      matrix with column dropping followed by Jacobi
// Matrices are column-major, complex stored as (re, im) double pairs.
#include "mx_common.cuh"
#include "mx_internal.h"

#include <math.h>

using namespace mx;

namespace {

constexpr int DT = 256;   // threads per CTA

struct Z {
  double re, im;
};
__device__ __forceinline__ Z zmk(double a, double b) { Z z; z.re = a; z.im = b; return z; }
__device__ __forceinline__ Z zadd(Z a, Z b) { return zmk(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ Z zsub(Z a, Z b) { return zmk(a.re - b.re, a.im - b.im); }
__device__ __forceinline__ Z zmul(Z a, Z b) { return zmk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
__device__ __forceinline__ Z zcmul(Z a, Z b) { return zmk(a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re); }  // conj(a) b
__device__ __forceinline__ Z zconj(Z a) { return zmk(a.re, -a.im); }
__device__ __forceinline__ Z zscal(double s, Z a) { return zmk(s * a.re, s * a.im); }
__device__ __forceinline__ double zabs2(Z a) { return a.re * a.re + a.im * a.im; }
__device__ __forceinline__ Z zdiv(Z a, Z b) {
  double d = zabs2(b);
  return zmk((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}

#define AT(M, ld, i, j) (reinterpret_cast<Z*>(M)[(size_t) (j) * (ld) + (i)])

__device__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    t = warp_sum(t);
  }
  __syncthreads();
  if (threadIdx.x == 0) sh[0] = t;
  __syncthreads();
  t = sh[0];
  __syncthreads();
  return t;
}

// ------------------------------------------------------------------
// Gauss-Jordan inverse of a Hermitian positive definite matrix (no
// pivoting is needed for HPD input)
// ------------------------------------------------------------------
__global__ void k_hpd_inverse(int N, double* a, int* info) {
  extern __shared__ double sm[];
  Z* f = reinterpret_cast<Z*>(sm);
  Z* rowp = f + N;
  double* A = a + (size_t) blockIdx.x * 2 * N * N;
  int bad = 0;
  for (int p = 0; p < N; p++) {
    for (int i = threadIdx.x; i < N; i += blockDim.x) f[i] = AT(A, N, i, p);
    __syncthreads();
    Z piv = f[p];
    if (!(piv.re > 0.0)) bad = p + 1;
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
      Z v = j == p ? zmk(1.0, 0.0) : AT(A, N, p, j);
      rowp[j] = zdiv(v, piv);
    }
    __syncthreads();
    for (size_t e = threadIdx.x; e < (size_t) N * N; e += blockDim.x) {
      int i = (int) (e % N), j = (int) (e / N);
      if (i == p) AT(A, N, i, j) = rowp[j];
      else {
        Z v = j == p ? zmk(0.0, 0.0) : AT(A, N, i, j);
        AT(A, N, i, j) = zsub(v, zmul(f[i], rowp[j]));
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0 && info) info[blockIdx.x] = bad;
}

// ------------------------------------------------------------------
// y_k = Ainv_k x_k on a level-0 block: the block of one k-point is a
// row-major N x m matrix (dense row r at offset r*m)
// ------------------------------------------------------------------
// The inverse is read as MS (double2, or its float2 rounding for FP32 solves).
template <typename S, typename R, typename MS>
__global__ void k_coarse_apply(int N, int m, const MS* __restrict__ ainv, const S* __restrict__ x,
                               S* __restrict__ y) {
  int k = blockIdx.y;
  const MS* Ai = ainv + (size_t) k * N * N;
  const S* xk = x + (size_t) k * N * m;
  S* yk = y + (size_t) k * N * m;
  size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t) N * m) return;
  int v = (int) (t % m), r = (int) (t / m);
  cx<R> acc = czero<R>();
  for (int c = 0; c < N; c++)
    acc += Store<MS, R>::ld(Ai + (size_t) c * N + r) * Store<S, R>::ld(xk + (size_t) c * m + v);
  Store<S, R>::st(yk + (size_t) r * m + v, acc);
}

// ------------------------------------------------------------------
// Cyclic Jacobi for a Hermitian N x N matrix in global memory (full storage),
// eigenvectors accumulated in Zm; Brent-Luk round-robin ordering lets the
// N/2 rotations of one round run concurrently.  Rotation: for the pair (p,q)
// with a_pq = g e, g = |a_pq|, tau = (a_qq - a_pp)/(2g),
// t = sgn(tau)/(|tau| + sqrt(1+tau^2)), c = 1/sqrt(1+t^2), s = t c, and
// V = [[c, s e], [-s conj(e), c]] on (p,q); A <- V^H A V, Z <- Z V.
// ------------------------------------------------------------------
__device__ void jacobi_cta(int N, int ld, double* A, double* Zm, double* w, double* shd, int* shi, int max_sweeps,
                           bool init = true) {
  // shd: 4 * (N/2 + 1) doubles of rotation data, plus 32 for reductions
  int Np = N + (N & 1);   // pad to even with a dummy index N
  int half = Np / 2;
  double* cs = shd;             // c
  double* sn = shd + half;      // s
  double* er = shd + 2 * half;  // Re e
  double* ei = shd + 3 * half;  // Im e
  double* red = shd + 4 * half;
  int* pp = shi;
  int* qq = shi + half;
  // with init, Zm starts as the identity and A is completed from its lower
  // triangle; without, A is already full and rotations accumulate onto Zm
  if (init)
    for (size_t e = threadIdx.x; e < (size_t) N * N; e += blockDim.x) {
      int i = (int) (e % N), j = (int) (e / N);
      AT(Zm, ld, i, j) = zmk(i == j ? 1.0 : 0.0, 0.0);
      if (i < j) AT(A, ld, i, j) = zconj(AT(A, ld, j, i));   // complete from the lower triangle
      if (i == j) AT(A, ld, i, i).im = 0.0;
    }
  __syncthreads();
  double fro = 0.0;
  for (size_t e = threadIdx.x; e < (size_t) N * N; e += blockDim.x) fro += zabs2(AT(A, ld, e % N, e / N));
  fro = sqrt(block_sum(fro, red));
  // rotation passes: the (rotation s, row or column i) items e = s N + i
  // are dealt to the threads in strides of blockDim.x, with (s, i) advanced
  // incrementally (no integer division in the loops)
  const int bq = (int) blockDim.x / N, br = (int) blockDim.x % N;
  const int s0 = (int) threadIdx.x / N, i0 = (int) threadIdx.x % N;
  for (int sweep = 0; sweep < max_sweeps; sweep++) {
    // Rutishauser's test: a rotation is skipped when |a_pq| is negligible
    // against sqrt(|a_pp a_qq|) or against the norm of the matrix (a block of
    // equal or zero eigenvalues would otherwise be rotated forever); the
    // iteration stops after a sweep without any rotation
    double rotated = 0.0;
    for (int r = 0; r < Np - 1; r++) {
      for (int s = threadIdx.x; s < half; s += blockDim.x) {
        int a = s == 0 ? 0 : 1 + (s - 1 + r) % (Np - 1);
        int bpos = Np - 1 - s;
        int b = 1 + (bpos - 1 + r) % (Np - 1);
        int p = a < b ? a : b, q = a < b ? b : a;
        double c = 1.0, sv = 0.0, xr = 1.0, xi = 0.0;
        if (q < N) {
          Z apq = AT(A, ld, p, q);
          double g = sqrt(zabs2(apq));
          double scale = sqrt(fabs(AT(A, ld, p, p).re * AT(A, ld, q, q).re));
          if (g > 1e-16 * scale && g > 1e-15 * fro) {
            rotated += 1.0;
            double app = AT(A, ld, p, p).re, aqq = AT(A, ld, q, q).re;
            double tau = (aqq - app) / (2.0 * g);
            double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            sv = t * c;
            xr = apq.re / g;
            xi = apq.im / g;
          }
        }
        pp[s] = p; qq[s] = q; cs[s] = c; sn[s] = sv; er[s] = xr; ei[s] = xi;
      }
      __syncthreads();
      // columns: A <- A V, Z <- Z V
      for (int s = s0, i = i0; s < half;
           s += bq + (i + br >= N), i = i + br >= N ? i + br - N : i + br) {
        int p = pp[s], q = qq[s];
        if (q >= N || sn[s] == 0.0) continue;
        Z ex = zmk(er[s], ei[s]);
        double c = cs[s], sv = sn[s];
        Z ap = AT(A, ld, i, p), aq = AT(A, ld, i, q);
        AT(A, ld, i, p) = zsub(zscal(c, ap), zscal(sv, zmul(zconj(ex), aq)));
        AT(A, ld, i, q) = zadd(zscal(sv, zmul(ex, ap)), zscal(c, aq));
        Z zp = AT(Zm, ld, i, p), zq = AT(Zm, ld, i, q);
        AT(Zm, ld, i, p) = zsub(zscal(c, zp), zscal(sv, zmul(zconj(ex), zq)));
        AT(Zm, ld, i, q) = zadd(zscal(sv, zmul(ex, zp)), zscal(c, zq));
      }
      __syncthreads();
      // rows: A <- V^H A
      for (int s = s0, i = i0; s < half;
           s += bq + (i + br >= N), i = i + br >= N ? i + br - N : i + br) {
        const int j = i;
        int p = pp[s], q = qq[s];
        if (q >= N || sn[s] == 0.0) continue;
        Z ex = zmk(er[s], ei[s]);
        double c = cs[s], sv = sn[s];
        Z ap = AT(A, ld, p, j), aq = AT(A, ld, q, j);
        AT(A, ld, p, j) = zsub(zscal(c, ap), zscal(sv, zmul(ex, aq)));
        AT(A, ld, q, j) = zadd(zscal(sv, zmul(zconj(ex), ap)), zscal(c, aq));
      }
      __syncthreads();
    }
    if (block_sum(rotated, red) == 0.0) break;
  }
  // eigenvalues, then sort ascending (selection sort by one thread on the
  // index permutation; N <= 256)
  if (threadIdx.x == 0) {
    for (int i = 0; i < N; i++) w[i] = AT(A, ld, i, i).re;
    for (int i = 0; i < N; i++) {
      int mi = i;
      for (int j = i + 1; j < N; j++)
        if (w[j] < w[mi]) mi = j;
      if (mi != i) {
        double tw = w[i]; w[i] = w[mi]; w[mi] = tw;
        for (int r = 0; r < N; r++) {
          Z tz = AT(Zm, ld, r, i);
          AT(Zm, ld, r, i) = AT(Zm, ld, r, mi);
          AT(Zm, ld, r, mi) = tz;
        }
      }
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------------
// Mixed-precision Jacobi.  FP64 arithmetic on GB300 runs at a small fraction
// of the FP32 rate and a CTA's Jacobi sweeps are bound by it, so the sweeps
// that do the bulk of the work run in FP32: they bring the off-diagonal
// part down to about 1e-6 of the matrix.  Their accumulated rotations Zf are
// then made unitary to FP64 precision by one Newton-Schulz step
// Q = Z (3I - Z^H Z) / 2, the matrix is transformed exactly in FP64,
// A' = Q^H A Q (same eigenvalues as A), and FP64 sweeps finish A' -- one or
// two, Jacobi converging quadratically -- accumulating into Q.
// ------------------------------------------------------------------
struct Cf {
  float re, im;
};

// one cyclic Jacobi run on the FP32 copy (the same rotation as jacobi_cta)
__device__ void jacobi_f32(int N, int ld, Cf* A, Cf* Zm, float* shf, double* red, int* shi, int max_sweeps) {
  int Np = N + (N & 1);
  int half = Np / 2;
  float* cs = shf;
  float* sn = shf + half;
  float* er = shf + 2 * half;
  float* ei = shf + 3 * half;
  int* pp = shi;
  int* qq = shi + half;
#define AF(M, i, j) (M[(size_t) (j) * ld + (i)])
  double fro = 0.0;
  for (size_t e = threadIdx.x; e < (size_t) N * N; e += blockDim.x) {
    Cf a = AF(A, e % N, e / N);
    fro += (double) a.re * a.re + (double) a.im * a.im;
  }
  float frof = (float) sqrt(block_sum(fro, red));
  // rotation passes: the (rotation s, row or column i) items e = s N + i
  // are dealt to the threads in strides of blockDim.x, with (s, i) advanced
  // incrementally (no integer division in the loops)
  const int bq = (int) blockDim.x / N, br = (int) blockDim.x % N;
  const int s0 = (int) threadIdx.x / N, i0 = (int) threadIdx.x % N;
  for (int sweep = 0; sweep < max_sweeps; sweep++) {
    double rotated = 0.0;
    for (int r = 0; r < Np - 1; r++) {
      for (int s = threadIdx.x; s < half; s += blockDim.x) {
        int a = s == 0 ? 0 : 1 + (s - 1 + r) % (Np - 1);
        int bpos = Np - 1 - s;
        int b = 1 + (bpos - 1 + r) % (Np - 1);
        int p = a < b ? a : b, q = a < b ? b : a;
        float c = 1.0f, sv = 0.0f, xr = 1.0f, xi = 0.0f;
        if (q < N) {
          Cf apq = AF(A, p, q);
          float g = sqrtf(apq.re * apq.re + apq.im * apq.im);
          float scale = sqrtf(fabsf(AF(A, p, p).re * AF(A, q, q).re));
          // stop where FP32 can no longer resolve the coupling
          if (g > 1e-6f * scale && g > 1e-6f * frof) {
            rotated += 1.0;
            float app = AF(A, p, p).re, aqq = AF(A, q, q).re;
            float tau = (aqq - app) / (2.0f * g);
            float t = (tau >= 0.0f ? 1.0f : -1.0f) / (fabsf(tau) + sqrtf(1.0f + tau * tau));
            c = 1.0f / sqrtf(1.0f + t * t);
            sv = t * c;
            xr = apq.re / g;
            xi = apq.im / g;
          }
        }
        pp[s] = p; qq[s] = q; cs[s] = c; sn[s] = sv; er[s] = xr; ei[s] = xi;
      }
      __syncthreads();
      for (int s = s0, i = i0; s < half;
           s += bq + (i + br >= N), i = i + br >= N ? i + br - N : i + br) {
        int p = pp[s], q = qq[s];
        if (q >= N || sn[s] == 0.0f) continue;
        float c = cs[s], sv = sn[s], xr = er[s], xi = ei[s];
        Cf ap = AF(A, i, p), aq = AF(A, i, q);
        // ap' = c ap - s conj(e) aq, aq' = s e ap + c aq
        AF(A, i, p) = Cf{c * ap.re - sv * (xr * aq.re + xi * aq.im), c * ap.im - sv * (xr * aq.im - xi * aq.re)};
        AF(A, i, q) = Cf{sv * (xr * ap.re - xi * ap.im) + c * aq.re, sv * (xr * ap.im + xi * ap.re) + c * aq.im};
        Cf zp = AF(Zm, i, p), zq = AF(Zm, i, q);
        AF(Zm, i, p) = Cf{c * zp.re - sv * (xr * zq.re + xi * zq.im), c * zp.im - sv * (xr * zq.im - xi * zq.re)};
        AF(Zm, i, q) = Cf{sv * (xr * zp.re - xi * zp.im) + c * zq.re, sv * (xr * zp.im + xi * zp.re) + c * zq.im};
      }
      __syncthreads();
      for (int s = s0, i = i0; s < half;
           s += bq + (i + br >= N), i = i + br >= N ? i + br - N : i + br) {
        const int j = i;
        int p = pp[s], q = qq[s];
        if (q >= N || sn[s] == 0.0f) continue;
        float c = cs[s], sv = sn[s], xr = er[s], xi = ei[s];
        Cf ap = AF(A, p, j), aq = AF(A, q, j);
        // ap' = c ap - s e aq, aq' = s conj(e) ap + c aq
        AF(A, p, j) = Cf{c * ap.re - sv * (xr * aq.re - xi * aq.im), c * ap.im - sv * (xr * aq.im + xi * aq.re)};
        AF(A, q, j) = Cf{sv * (xr * ap.re + xi * ap.im) + c * aq.re, sv * (xr * ap.im - xi * ap.re) + c * aq.im};
      }
      __syncthreads();
    }
    if (block_sum(rotated, red) == 0.0) break;
  }
#undef AF
}

// C = op(X) Y for N x N complex FP64 matrices (leading dimension ld), op =
// conjugate transpose when cx
__device__ void zgemm_cta(int N, int ld, double* X, bool cx, double* Y, double* C) {
  for (size_t e = threadIdx.x; e < (size_t) N * N; e += blockDim.x) {
    int i = (int) (e % N), j = (int) (e / N);
    Z s = zmk(0.0, 0.0);
    if (cx)
      for (int l = 0; l < N; l++) s = zadd(s, zcmul(AT(X, ld, l, i), AT(Y, ld, l, j)));
    else
      for (int l = 0; l < N; l++) s = zadd(s, zmul(AT(X, ld, i, l), AT(Y, ld, l, j)));
    AT(C, ld, i, j) = s;
  }
  __syncthreads();
}

// Eigen-decomposition of the Hermitian A (lower triangle used; overwritten)
// into w (ascending) and Zm.  Buffers: F (N*N complex doubles of space: the
// FP32 copies, later Q) and G (N*N complex doubles); all with leading
// dimension ld.
__device__ void jacobi_mixed(int N, int ld, double* A, double* Zm, double* w, double* shd, int* shi, double* F,
                             double* G) {
  int half = (N + (N & 1)) / 2;
  double* red = shd + 4 * (half + 1);
  Cf* Af = reinterpret_cast<Cf*>(F);
  Cf* Zf = Af + (size_t) ld * N;
  for (size_t e = threadIdx.x; e < (size_t) N * N; e += blockDim.x) {
    int i = (int) (e % N), j = (int) (e / N);
    Z a = i >= j ? AT(A, ld, i, j) : zconj(AT(A, ld, j, i));
    if (i == j) a.im = 0.0;
    if (i <= j) AT(A, ld, i, j) = a;   // complete the FP64 matrix as well
    Af[(size_t) j * ld + i] = Cf{(float) a.re, (float) a.im};
    Zf[(size_t) j * ld + i] = Cf{i == j ? 1.0f : 0.0f, 0.0f};
  }
  __syncthreads();
  jacobi_f32(N, ld, Af, Zf, reinterpret_cast<float*>(shd), red, shi, 30);
  for (size_t e = threadIdx.x; e < (size_t) ld * N; e += blockDim.x)
    reinterpret_cast<Z*>(Zm)[e] = zmk((double) Zf[e].re, (double) Zf[e].im);
  __syncthreads();
  // Q = Z (3I - Z^H Z) / 2 into F
  zgemm_cta(N, ld, Zm, true, Zm, G);
  for (size_t e = threadIdx.x; e < (size_t) N * N; e += blockDim.x) {
    int i = (int) (e % N), j = (int) (e / N);
    Z g = AT(G, ld, i, j);
    AT(G, ld, i, j) = zmk((i == j ? 1.5 : 0.0) - 0.5 * g.re, -0.5 * g.im);
  }
  __syncthreads();
  zgemm_cta(N, ld, Zm, false, G, F);
  // A' = Q^H A Q, then the FP64 sweeps accumulate onto Q
  zgemm_cta(N, ld, A, false, F, G);
  zgemm_cta(N, ld, F, true, G, A);
  for (size_t e = threadIdx.x; e < (size_t) ld * N; e += blockDim.x)
    reinterpret_cast<Z*>(Zm)[e] = reinterpret_cast<Z*>(F)[e];
  __syncthreads();
  jacobi_cta(N, ld, A, Zm, w, shd, shi, 20, false);
}

__global__ void k_heev(int N, double* a, double* zwork, double* w, int* info) {
  extern __shared__ double sm[];
  int half = (N + 1) / 2 + 1;
  double* A = a + (size_t) blockIdx.x * 2 * N * N;
  double* Zm = zwork + (size_t) blockIdx.x * 2 * N * N;
  jacobi_cta(N, N, A, Zm, w + (size_t) blockIdx.x * N, sm, reinterpret_cast<int*>(sm + 4 * half + 32), 60);
  for (size_t e = threadIdx.x; e < (size_t) N * N; e += blockDim.x)
    reinterpret_cast<Z*>(A)[e] = reinterpret_cast<Z*>(Zm)[e];
  if (threadIdx.x == 0 && info) info[blockIdx.x] = 0;
}

// odd leading dimension of the Ritz work matrices
__host__ __device__ inline int ritz_ld(int ns) { return ns | 1; }

// ------------------------------------------------------------------
// Rayleigh-Ritz from Gram matrices (see mx_internal.h)
// workspace per k: 5 * ns * ns complex doubles
// ------------------------------------------------------------------
__global__ void k_rayleigh_ritz(int ns, int m, const double* __restrict__ ga, const double* __restrict__ gm,
                                const int* __restrict__ sel, double drop, double theta_min, double* coef,
                                double* theta, int* info, double* work, int in_smem) {
  extern __shared__ double sm[];
  int k = blockIdx.x;
  int half = (ns + 1) / 2 + 1;
  double* shd = sm;                                  // jacobi rotation data: 4*half + 32
  double* d = shd + 4 * half + 32;                   // ns
  double* wv = d + ns;                               // ns
  int* shi = reinterpret_cast<int*>(wv + ns);        // 2*half
  int* idx = shi + 2 * half;                         // ns
  int* kept = idx + ns;                              // ns
  int* cnt = kept + ns;                              // 2
  const double* GA = ga + (size_t) k * 2 * ns * ns;
  const double* GM = gm + (size_t) k * 2 * ns * ns;
  // work matrices: in shared memory for the Ritz systems (ns <= 48), in
  // global memory for the coarse-grid eigenproblem
  // every work matrix has the odd leading dimension ld >= ns: a row of a
  // column-major matrix then falls into distinct shared-memory banks
  const int ld = ritz_ld(ns);
  const size_t msz = (size_t) 2 * ld * ns;           // doubles per work matrix
  double* W0;
  if (in_smem) {
    uintptr_t p0 = reinterpret_cast<uintptr_t>(cnt + 2);
    W0 = reinterpret_cast<double*>((p0 + 15) & ~(uintptr_t) 15);
  } else {
    W0 = work + (size_t) k * 5 * msz;
  }
  double* W1 = W0 + msz;                             // T = D R^-1
  double* W2 = W1 + msz;                             // G_A T, then projected A
  double* W3 = W2 + msz;                             // Jacobi eigenvectors
  double* GS = in_smem ? W3 + msz : nullptr;         // G_A on the selected columns
  // work of the mixed Jacobi: W0 (free once T is formed) and GS, or in global
  // memory a fifth matrix
  double* GB = in_smem ? GS : W3 + msz;
  if (threadIdx.x == 0) {
    int na = 0;
    for (int i = 0; i < ns; i++)
      if (!sel || sel[(size_t) k * ns + i]) idx[na++] = i;
    cnt[0] = na;
  }
  __syncthreads();
  int na = cnt[0];
  for (int i = threadIdx.x; i < na; i += blockDim.x) {
    double g = reinterpret_cast<const Z*>(GM)[(size_t) idx[i] * ns + idx[i]].re;
    d[i] = g > 0.0 ? 1.0 / sqrt(g) : 0.0;
  }
  __syncthreads();
  for (size_t e = threadIdx.x; e < (size_t) na * na; e += blockDim.x) {
    int i = (int) (e % na), j = (int) (e / na);
    Z g = reinterpret_cast<const Z*>(GM)[(size_t) idx[j] * ns + idx[i]];
    AT(W0, ld, i, j) = zscal(d[i] * d[j], g);
  }
  __syncthreads();
  // right-looking Cholesky with column dropping: W0 -> R (upper), kept flags
  for (int j = 0; j < na; j++) {
    double piv = AT(W0, ld, j, j).re;
    bool keep = piv > drop && d[j] > 0.0;
    double rjj = keep ? sqrt(piv) : 0.0;
    __syncthreads();
    if (threadIdx.x == 0) kept[j] = keep;
    for (int l = j + threadIdx.x; l < na; l += blockDim.x) {
      Z v = AT(W0, ld, j, l);
      AT(W0, ld, j, l) = keep ? (l == j ? zmk(rjj, 0.0) : zscal(1.0 / rjj, v)) : zmk(0.0, 0.0);
    }
    __syncthreads();
    if (keep)
      for (size_t e = threadIdx.x; e < (size_t) (na - j - 1) * (na - j - 1); e += blockDim.x) {
        int i = j + 1 + (int) (e % (na - j - 1)), l = j + 1 + (int) (e / (na - j - 1));
        if (i <= l) AT(W0, ld, i, l) = zsub(AT(W0, ld, i, l), zcmul(AT(W0, ld, j, i), AT(W0, ld, j, l)));
      }
    __syncthreads();
  }
  // compact the kept indices
  if (threadIdx.x == 0) {
    int r = 0;
    for (int j = 0; j < na; j++)
      if (kept[j]) kept[r++] = j;
    cnt[1] = r;
  }
  __syncthreads();
  int r = cnt[1];
  if (r < m) {
    if (threadIdx.x == 0) info[k] = -1 - r;
    return;
  }
  // T (na x r): column c solves R[kept,kept] t = e_c, rows scaled by d
  for (int c = threadIdx.x; c < r; c += blockDim.x) {
    for (int i = 0; i < na; i++) AT(W1, ld, i, c) = zmk(0.0, 0.0);
    for (int a = r - 1; a >= 0; a--) {
      int ia = kept[a];
      Z s = zmk(a == c ? 1.0 : 0.0, 0.0);
      for (int b = a + 1; b < r; b++) s = zsub(s, zmul(AT(W0, ld, ia, kept[b]), AT(W1, ld, kept[b], c)));
      AT(W1, ld, ia, c) = zscal(1.0 / AT(W0, ld, ia, ia).re, s);
    }
    for (int i = 0; i < na; i++) AT(W1, ld, i, c) = zscal(d[i], AT(W1, ld, i, c));
  }
  __syncthreads();
  // W3 <- G_A T  (na x r), then W2 <- T^H W3 (r x r)
  if (GS) {
    for (size_t e = threadIdx.x; e < (size_t) na * na; e += blockDim.x) {
      int i = (int) (e % na), l = (int) (e / na);
      AT(GS, ld, i, l) = reinterpret_cast<const Z*>(GA)[(size_t) idx[l] * ns + idx[i]];
    }
    __syncthreads();
  }
  for (size_t e = threadIdx.x; e < (size_t) na * r; e += blockDim.x) {
    int i = (int) (e % na), c = (int) (e / na);
    Z s = zmk(0.0, 0.0);
    if (GS)
      for (int l = 0; l < na; l++) s = zadd(s, zmul(AT(GS, ld, i, l), AT(W1, ld, l, c)));
    else
      for (int l = 0; l < na; l++)
        s = zadd(s, zmul(reinterpret_cast<const Z*>(GA)[(size_t) idx[l] * ns + idx[i]], AT(W1, ld, l, c)));
    AT(W3, ld, i, c) = s;
  }
  __syncthreads();
  for (size_t e = threadIdx.x; e < (size_t) r * r; e += blockDim.x) {
    int a = (int) (e % r), c = (int) (e / r);
    Z s = zmk(0.0, 0.0);
    for (int l = 0; l < na; l++) s = zadd(s, zcmul(AT(W1, ld, l, a), AT(W3, ld, l, c)));
    AT(W2, ld, a, c) = s;
  }
  __syncthreads();
  jacobi_mixed(r, ld, W2, W3, wv, shd, shi, W0, GB);
  // Ritz values at or below theta_min are spurious (null-space) modes and
  // are passed over, as exp_bloch2d.c:546-551 does for its coarse start
  if (threadIdx.x == 0) {
    int f = 0;
    while (f < r && !(wv[f] > theta_min)) f++;
    cnt[0] = f;
  }
  __syncthreads();
  int first = cnt[0];
  if (r - first < m) {
    if (threadIdx.x == 0) info[k] = -1 - (r - first);
    return;
  }
  for (size_t e = threadIdx.x; e < (size_t) ns * m; e += blockDim.x) {
    int i = (int) (e % ns), j = (int) (e / ns);
    reinterpret_cast<Z*>(coef)[(size_t) k * ns * m + (size_t) j * ns + i] = zmk(0.0, 0.0);
  }
  __syncthreads();
  for (size_t e = threadIdx.x; e < (size_t) na * m; e += blockDim.x) {
    int i = (int) (e % na), j = (int) (e / na);
    Z s = zmk(0.0, 0.0);
    for (int l = 0; l < r; l++) s = zadd(s, zmul(AT(W1, ld, i, l), AT(W3, ld, l, first + j)));
    reinterpret_cast<Z*>(coef)[(size_t) k * ns * m + (size_t) j * ns + idx[i]] = s;
  }
  for (int j = threadIdx.x; j < m; j += blockDim.x) theta[(size_t) k * m + j] = wv[first + j];
  if (threadIdx.x == 0) info[k] = r;
}

size_t jacobi_smem(int N) {
  int half = (N + 1) / 2 + 1;
  return sizeof(double) * (4 * half + 32) + sizeof(int) * 2 * half;
}

}  // namespace

extern "C" int mxk_hpd_inverse(int N, int K, double* a, int* info, mx_stream s) {
  k_hpd_inverse<<<K, DT, 2 * N * sizeof(Z), (cudaStream_t) s>>>(N, a, info);
  MX_CHECK_LAUNCH();
  return 0;
}

template <typename S, typename R, typename MS>
static int L_coarse_apply(int N, int m, int K, const void* ainv, const void* x, void* y, cudaStream_t st) {
  dim3 g((unsigned) (((size_t) N * m + 127) / 128), K);
  k_coarse_apply<S, R, MS><<<g, 128, 0, st>>>(N, m, (const MS*) ainv, (const S*) x, (S*) y);
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_coarse_apply(int N, int m, int K, const double* ainv, const void* ainv_c64, int prec,
                                const void* x, void* y, mx_stream s) {
  cudaStream_t st = (cudaStream_t) s;
  if (prec == MX_C64) {
    if (ainv_c64) return L_coarse_apply<float2, float, float2>(N, m, K, ainv_c64, x, y, st);
    return L_coarse_apply<float2, float, double2>(N, m, K, ainv, x, y, st);
  }
  if (prec == MX_C128) return L_coarse_apply<double2, double, double2>(N, m, K, ainv, x, y, st);
  return L_coarse_apply<cdd, dd, double2>(N, m, K, ainv, x, y, st);
}

extern "C" int mxk_heev(int N, int K, double* a, double* zwork, double* w, int* info, mx_stream s) {
  k_heev<<<K, DT, jacobi_smem(N), (cudaStream_t) s>>>(N, a, zwork, w, info);
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" size_t mxk_ritz_work_doubles(int ns) { return (size_t) 10 * ritz_ld(ns) * ns; }

extern "C" int mxk_rayleigh_ritz(int ns, int m, int K, const double* ga, const double* gm, const int* sel,
                                 double drop, double theta_min, double* coef, double* theta, int* info,
                                 double* work, mx_stream s) {
  size_t smem = jacobi_smem(ns) + sizeof(int) * (2 * ns + 4) + sizeof(double) * (2 * ns + 2);
  int in_smem = ns <= 48;
  if (in_smem) {
    smem += 16 + sizeof(double) * 2 * (size_t) ritz_ld(ns) * ns * 5;
    cudaFuncSetAttribute(k_rayleigh_ritz, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  }
  int threads = in_smem ? DT : 1024;
  k_rayleigh_ritz<<<K, threads, smem, (cudaStream_t) s>>>(ns, m, ga, gm, sel, drop, theta_min, coef, theta, info,
                                                         work, in_smem);
  MX_CHECK_LAUNCH();
  return 0;
}

// ------------------------------------------------------------------
// Cholesky-QR coefficients: for the Hermitian positive definite mass Gram
// G = X^H M X of m vectors, G = R^H R with R upper triangular and a positive
// real diagonal, and coef = R^{-1}; X coef is then M-orthonormal and its
// first j columns span the first j columns of X (the function of the
// reference's Householder orthonormalisation, orthonormalize_edge2d,
// edge2d.c:6264-6296).  info[k] = 0, or j+1 if column j is (numerically)
// dependent on the columns before it.
// ------------------------------------------------------------------
namespace {
__global__ void k_chol_qr_coef(int m, const double* __restrict__ gm, double* __restrict__ coef, int* info) {
  extern __shared__ double smc[];
  Z* R = reinterpret_cast<Z*>(smc);          // m x m column-major
  __shared__ int bad;
  const double* G = gm + (size_t) blockIdx.x * 2 * m * m;
  double* C = coef + (size_t) blockIdx.x * 2 * m * m;
  for (int e = threadIdx.x; e < m * m; e += blockDim.x) R[e] = reinterpret_cast<const Z*>(G)[e];
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < m; j++) {
    // row j of R: R_jj = sqrt(G_jj - sum |R_ij|^2), R_jc = (G_jc - sum conj(R_ij) R_ic) / R_jj
    __shared__ double djj;
    if (threadIdx.x == 0) {
      double g = R[j * m + j].re, d = g;
      for (int i = 0; i < j; i++) d -= zabs2(R[j * m + i]);
      // column j counts as dependent when the part of it outside the span
      // of the columns before it has less than 1e-5 of its M-norm
      if (!(d > 1e-10 * g) && !bad) bad = j + 1;
      djj = d > 0.0 ? sqrt(d) : 1.0;
    }
    __syncthreads();
    for (int c = j + 1 + threadIdx.x; c < m; c += blockDim.x) {
      Z s = R[c * m + j];
      for (int i = 0; i < j; i++) s = zsub(s, zcmul(R[j * m + i], R[c * m + i]));
      R[c * m + j] = zscal(1.0 / djj, s);
    }
    __syncthreads();
    if (threadIdx.x == 0) R[j * m + j] = zmk(djj, 0.0);
    __syncthreads();
  }
  // coef = R^{-1}, one column per thread (back substitution)
  for (int c = threadIdx.x; c < m; c += blockDim.x) {
    for (int i = m - 1; i > c; i--) AT(C, m, i, c) = zmk(0.0, 0.0);
    AT(C, m, c, c) = zmk(1.0 / R[c * m + c].re, 0.0);
    for (int i = c - 1; i >= 0; i--) {
      Z s = zmk(0.0, 0.0);
      for (int q = i + 1; q <= c; q++) s = zadd(s, zmul(R[q * m + i], AT(C, m, q, c)));
      AT(C, m, i, c) = zscal(-1.0 / R[i * m + i].re, s);
    }
  }
  if (threadIdx.x == 0 && info) info[blockIdx.x] = bad;
}
}  // namespace

extern "C" int mxk_chol_qr_coef(int m, int K, const double* gm, double* coef, int* info, mx_stream s) {
  if (m < 1 || m > 64) return (int) cudaErrorInvalidValue;
  size_t smem = sizeof(double) * 2 * (size_t) m * m;
  cudaFuncSetAttribute(k_chol_qr_coef, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  k_chol_qr_coef<<<K, 64, smem, (cudaStream_t) s>>>(m, gm, coef, info);
  MX_CHECK_LAUNCH();
  return 0;
}
