// Vector operations of the edge2d / node2d interfaces that the eigensolver's
// own kernels do not cover, batched over k-points and vectors:
//   scale_*         x *= alpha                        (edge2d.c:806-828, node2d.c:385-399)
//   random_*        uniform entries in [-1,1] + i[-1,1] (edge2d.c:161-191, node2d.c:72-90)
//   normmax_*       max |x| per (k, vector)           (edge2d.c:887-920, node2d.c:441-463)
//   plane sums      sum of each plane per (k, vector) (nullprod_edge2d, edge2d.c:1240-1274;
//                   center_node2d, node2d.c:489-514)
//   plane shifts    add a constant per plane          (nulladd_edge2d, edge2d.c:1276-1307)
//   pattern         1/eps per cell from rectangles and circles (setpattern_grid2d,
//                   grid2d.c:171-218)
// The layouts are those of mx_common.cuh: an edge block [K][2][n][n][m] has
// two planes of n*n sites per (k, vector), a node block [K][n][n][m] one.
#include "mx_common.cuh"
#include "mx_internal.h"

using namespace mx;

namespace {

constexpr int VT = 256;

inline unsigned vblocks(size_t work) {
  size_t b = (work + VT - 1) / VT;
  return (unsigned) (b > 0x7fffffffu ? 0x7fffffffu : (b < 1 ? 1 : b));
}

template <typename S, typename R>
__global__ void k_scale(Sc are, Sc aim, size_t len, S* __restrict__ x) {
  for (size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x; t < len; t += (size_t) gridDim.x * blockDim.x) {
    cx<R> a = mkc(sget<R>(are), sget<R>(aim));
    Store<S, R>::st(x + t, a * Store<S, R>::ld(x + t));
  }
}

// SplitMix64 (Steele, Lea and Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014): a counter-based stream, so every entry's value
// depends only on the seed and its position in the batch.
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
// the top 53 bits as a double in [-1, 1)
__device__ __forceinline__ double unit_pm1(unsigned long long r) {
  return (double) (r >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

template <typename S>
__global__ void k_random(unsigned long long seed, S* __restrict__ x, size_t len) {
  for (size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x; t < len; t += (size_t) gridDim.x * blockDim.x) {
    unsigned long long base = seed * 0xd1342543de82ef95ull + 2 * (unsigned long long) t;
    Store<S, double>::st(x + t, mkc(unit_pm1(splitmix64(base)), unit_pm1(splitmix64(base + 1))));
  }
}

// out[k*m+v] = max over `per` entries of |x|; out holds non-negative doubles
// (zeroed by the caller), whose bit patterns order like the values, so the
// maximum is taken with an integer atomic
template <typename S, typename R>
__global__ void k_absmax(size_t per, int m, const S* __restrict__ x, double* out) {
  int k = blockIdx.y;
  int v = threadIdx.x % m, row = threadIdx.x / m, rows = blockDim.x / m;
  double best = 0.0;
  if (row < rows)
    for (size_t e = (size_t) blockIdx.x * rows + row; e < per; e += (size_t) gridDim.x * rows) {
      cx<double> a = Store<S, double>::ld(reinterpret_cast<const S*>(x) + ((size_t) k * per + e) * m + v);
      double r = hypot(a.re, a.im);
      best = r > best ? r : best;
    }
  __shared__ double sm[VT];
  sm[threadIdx.x] = best;
  __syncthreads();
  if (threadIdx.x < m) {
    double b = 0.0;
    for (int r = 0; r < rows; r++) b = sm[r * m + threadIdx.x] > b ? sm[r * m + threadIdx.x] : b;
    atomicMax(reinterpret_cast<unsigned long long*>(out + (size_t) k * m + threadIdx.x),
              (unsigned long long) __double_as_longlong(b));
  }
}

// acc[2*((k*planes+p)*m+v)] += sum over the plane's `nsite` entries (re, im)
template <typename S>
__global__ void k_plane_sums(int nsite, int planes, int m, const S* __restrict__ x, double* acc) {
  int kp = blockIdx.y;
  int v = threadIdx.x % m, row = threadIdx.x / m, rows = blockDim.x / m;
  double re = 0.0, im = 0.0;
  if (row < rows)
    for (int s = blockIdx.x * rows + row; s < nsite; s += gridDim.x * rows) {
      cx<double> a = Store<S, double>::ld(x + ((size_t) kp * nsite + s) * m + v);
      re += a.re;
      im += a.im;
    }
  __shared__ double sre[VT], sim[VT];
  sre[threadIdx.x] = re;
  sim[threadIdx.x] = im;
  __syncthreads();
  if (threadIdx.x < m) {
    double tr = 0.0, ti = 0.0;
    for (int r = 0; r < rows; r++) { tr += sre[r * m + threadIdx.x]; ti += sim[r * m + threadIdx.x]; }
    atomicAdd(acc + 2 * ((size_t) kp * m + threadIdx.x), tr);
    atomicAdd(acc + 2 * ((size_t) kp * m + threadIdx.x) + 1, ti);
  }
  (void) planes;
}

// x[k][p][site][v] += scale * c[2*((k*planes+p)*m+v)] (re, im)
template <typename S, typename R>
__global__ void k_plane_shift(int nsite, int m, size_t len, const double* __restrict__ c, double scale,
                              S* __restrict__ x) {
  for (size_t t = (size_t) blockIdx.x * blockDim.x + threadIdx.x; t < len; t += (size_t) gridDim.x * blockDim.x) {
    size_t kp = t / ((size_t) nsite * m);
    int v = (int) (t % m);
    const double* q = c + 2 * (kp * m + v);
    cx<R> a = cfrom<R>(scale * q[0], scale * q[1]);
    Store<S, R>::st(x + t, Store<S, R>::ld(x + t) + a);
  }
}

// setpattern_grid2d (grid2d.c:171-218): cell (i, j) tested at its lower-left
// corner (i h, j h); later shapes overwrite earlier ones, circles after
// rectangles.  The comparisons use round-to-nearest intrinsics so that no
// fused multiply-add changes a cell on the boundary.
__global__ void k_pattern(int n, double h, const double* __restrict__ rect, int nrect,
                          const double* __restrict__ circ, int ncirc, double eps_base, double* __restrict__ kappa) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * n) return;
  int i = t % n, j = t / n;
  double x = __dmul_rn((double) i, h), y = __dmul_rn((double) j, h);
  double kv = 1.0 / eps_base;
  for (int q = 0; q < nrect; q++) {
    const double* r = rect + 5 * q;
    if (r[1] <= x && x <= __dadd_rn(r[1], r[3]) && r[2] <= y && y <= __dadd_rn(r[2], r[4])) kv = 1.0 / r[0];
  }
  for (int q = 0; q < ncirc; q++) {
    const double* c = circ + 4 * q;
    double dx = __dsub_rn(x, c[1]), dy = __dsub_rn(y, c[2]);
    double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    if (d2 <= __dmul_rn(c[3], c[3])) kv = 1.0 / c[0];
  }
  kappa[t] = kv;
}

#define MX_VEC_BY_PREC(prec, KERNEL, grid, block, st, ...)                                          \
  do {                                                                                             \
    if ((prec) == MX_C64) KERNEL<float2, float><<<grid, block, 0, st>>>(__VA_ARGS__, (float2*) x); \
    else if ((prec) == MX_C128) KERNEL<double2, double><<<grid, block, 0, st>>>(__VA_ARGS__, (double2*) x); \
    else if ((prec) == MX_CDD) KERNEL<cdd, dd><<<grid, block, 0, st>>>(__VA_ARGS__, (cdd*) x);        \
    else return (int) cudaErrorInvalidValue;                                                      \
  } while (0)

}  // namespace

extern "C" int mxk_scale(double are, double aim, int prec, void* x, size_t len, mx_stream s) {
  unsigned g = vblocks(len);
  if (g > 152 * 16) g = 152 * 16;
  MX_VEC_BY_PREC(prec, k_scale, g, VT, (cudaStream_t) s, make_sc(are), make_sc(aim), len);
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_random(unsigned long long seed, int prec, void* x, size_t len, mx_stream s) {
  unsigned g = vblocks(len);
  if (g > 152 * 16) g = 152 * 16;
  cudaStream_t st = (cudaStream_t) s;
  if (prec == MX_C64) k_random<float2><<<g, VT, 0, st>>>(seed, (float2*) x, len);
  else if (prec == MX_C128) k_random<double2><<<g, VT, 0, st>>>(seed, (double2*) x, len);
  else if (prec == MX_CDD) k_random<cdd><<<g, VT, 0, st>>>(seed, (cdd*) x, len);
  else return (int) cudaErrorInvalidValue;
  MX_CHECK_LAUNCH();
  return 0;
}

static dim3 per_vector_grid(size_t per, int m, int K) {
  int rows = VT / m;
  size_t g = (per + (size_t) rows * 8 - 1) / ((size_t) rows * 8);
  if (g < 1) g = 1;
  if (g > 2048) g = 2048;
  return dim3((unsigned) g, (unsigned) K);
}

extern "C" int mxk_absmax(size_t per, int m, int K, int prec, const void* x, double* out, mx_stream s) {
  if (m < 1 || m > 32) return (int) cudaErrorInvalidValue;
  cudaStream_t st = (cudaStream_t) s;
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double) * (size_t) K * m, st);
  if (e != cudaSuccess) return (int) e;
  dim3 g = per_vector_grid(per, m, K);
  if (prec == MX_C64) k_absmax<float2, float><<<g, VT, 0, st>>>(per, m, (const float2*) x, out);
  else if (prec == MX_C128) k_absmax<double2, double><<<g, VT, 0, st>>>(per, m, (const double2*) x, out);
  else if (prec == MX_CDD) k_absmax<cdd, dd><<<g, VT, 0, st>>>(per, m, (const cdd*) x, out);
  else return (int) cudaErrorInvalidValue;
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_plane_sums(int nsite, int planes, int m, int K, int prec, const void* x, double* acc,
                              mx_stream s) {
  if (m < 1 || m > 32 || planes < 1) return (int) cudaErrorInvalidValue;
  cudaStream_t st = (cudaStream_t) s;
  cudaError_t e = cudaMemsetAsync(acc, 0, sizeof(double) * 2 * (size_t) K * planes * m, st);
  if (e != cudaSuccess) return (int) e;
  dim3 g = per_vector_grid((size_t) nsite, m, K * planes);
  if (prec == MX_C64) k_plane_sums<float2><<<g, VT, 0, st>>>(nsite, planes, m, (const float2*) x, acc);
  else if (prec == MX_C128) k_plane_sums<double2><<<g, VT, 0, st>>>(nsite, planes, m, (const double2*) x, acc);
  else if (prec == MX_CDD) k_plane_sums<cdd><<<g, VT, 0, st>>>(nsite, planes, m, (const cdd*) x, acc);
  else return (int) cudaErrorInvalidValue;
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_plane_shift(int nsite, int planes, int m, int K, const double* c, double scale, int prec,
                               void* x, mx_stream s) {
  if (m < 1 || planes < 1) return (int) cudaErrorInvalidValue;
  size_t len = (size_t) K * planes * nsite * m;
  unsigned g = vblocks(len);
  if (g > 152 * 16) g = 152 * 16;
  MX_VEC_BY_PREC(prec, k_plane_shift, g, VT, (cudaStream_t) s, nsite, m, len, c, scale);
  MX_CHECK_LAUNCH();
  return 0;
}

extern "C" int mxk_pattern(int n, const double* rect, int nrect, const double* circ, int ncirc, double eps_base,
                           double* kappa, mx_stream s) {
  if (n < 1) return (int) cudaErrorInvalidValue;
  k_pattern<<<(unsigned) ((n * n + VT - 1) / VT), VT, 0, (cudaStream_t) s>>>(n, 1.0 / n, rect, nrect, circ, ncirc,
                                                                            eps_base, kappa);
  MX_CHECK_LAUNCH();
  return 0;
}
