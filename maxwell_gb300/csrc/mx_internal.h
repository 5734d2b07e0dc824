/* Internal launch interface of libmaxwell_gb300 (C linkage so that the C
 * host driver can call it).  Every function enqueues on `stream` and returns
 * a cudaError_t value (0 on success).  Pointers are device pointers in the
 * batched layout documented in mx_common.cuh. */
#ifndef MX_INTERNAL_H
#define MX_INTERNAL_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *mx_stream;

enum { MX_C64 = 0, MX_C128 = 1, MX_CDD = 2 };

/* launch shapes of the block kernels: Gram CTAs per k-point =
 * gram_waves * SMs / K, tiled-combination CTAs = combine_ctas * SMs, block
 * residual sites per thread (mxg_autotune chooses them) */
typedef struct {
  int gram_waves, combine_ctas, residual_sites;
} mxk_tuning;
void mxk_get_tuning(mxk_tuning *t);
int mxk_set_tuning(const mxk_tuning *t);

/* sizes of one complex entry */
size_t mxk_elem_size(int prec);

/* Phase table of K k-points (the `phases` argument of the kernels below):
 * 4K doubles (re xf, im xf, re yf, im yf per k-point) followed by the same
 * numbers as 8K floats in float-float pairs.  The caller writes the doubles
 * into a host buffer of mxk_phase_bytes(K) bytes, calls mxk_phase_fill to
 * derive the pairs, and copies the whole buffer to the device. */
size_t mxk_phase_bytes(int K);
void mxk_phase_fill(int K, double *host_table);

/* per-level reciprocal permittivity in three precisions */
typedef struct {
  const float *f;        /* n*n */
  const double *d;       /* n*n */
  const float *dd;       /* 2*n*n: (hi, lo) pairs */
  const void *afw;       /* NULL or the AFW patch factors of mxk_afw_factors */
  double afw_alpha, afw_beta;   /* the scalars those factors were made for */
} mxk_kappa;

/* Tabulate the FP32 factors of the AFW patch solves of one level (8 floats
 * per vertex, n*n*32 bytes at out) for the operator alpha*A + beta*M; FP32
 * sweeps with the same scalars read them instead of dividing per patch. */
int mxk_afw_factors(int n, const float *kappa_f, double alpha, double beta, void *out, mx_stream s);

/* ---- edge space ---- */
/* y = cy*(yin ? yin : y) + alpha*A x + beta_kv*M x; beta_kv (K*m doubles)
 * or NULL -> beta; yin (precision prec_y) may be NULL; cy = 0 reads neither */
int mxk_edge_apply(int n, int m, int K, const double *phases, mxk_kappa kap,
                   double alpha, double beta, const double *beta_kv, double cy,
                   int prec_x, const void *x, int prec_y, const void *yin, void *y, mx_stream s);
/* AFW line Gauss-Seidel sweep in the reference's row order; dir 0 forward,
 * 1 backward, 2 symmetric (forward then backward) */
int mxk_edge_gs(int n, int m, int K, const double *phases, mxk_kappa kap,
                double alpha, double beta, int dir, int prec,
                const void *b, void *x, mx_stream s);
/* the same smoother in four vertex colours (each colour one parallel launch):
 * forward (0,0), (1,0), (0,1), (1,1), backward the reverse order */
int mxk_edge_gs_colour(int n, int m, int K, const double *phases, mxk_kappa kap,
                       double alpha, double beta, int dir, int prec,
                       const void *b, void *x, mx_stream s);
/* point Gauss-Seidel of alpha A + beta M in the reference's interleaved row
 * order (gs*_simple_edge2d); dir 0 forward, 1 backward, 2 both */
int mxk_edge_gs_point(int n, int m, int K, const double *phases, mxk_kappa kap,
                      double alpha, double beta, int dir, int prec,
                      const void *b, void *x, mx_stream s);
int mxk_edge_prolong(int nc, int m, int K, const double *phases, double alpha,
                     int prec, const void *c, void *f, mx_stream s);
int mxk_edge_restrict(int nc, int m, int K, const double *phases, double alpha,
                      int prec, const void *f, void *c, mx_stream s);

/* ---- node space ---- */
/* y = cy*(yin ? yin : y) + alpha*L x (Q1 Laplace); cy = 0 reads neither */
int mxk_node_apply(int n, int m, int K, const double *phases, double alpha, double cy,
                   int prec, const void *x, const void *yin, void *y, mx_stream s);
int mxk_node_gs(int n, int m, int K, const double *phases, double alpha, int dir,
                int prec, const void *b, void *x, mx_stream s);
/* c (level nc) = restriction of (b - alpha L x) on level 2 nc, written */
int mxk_node_residual_restrict(int nc, int m, int K, const double *phases, double alpha, int prec,
                               const void *x, const void *b, void *c, mx_stream s);
/* one node GS sweep (dir 0 forward, 1 backward) read from x, written to y
 * (tiled, three launches); for c64 blocks with m % 4 == 0 and n >= 128 */
int mxk_node_gs_oop_ok(int n, int m, int prec);
int mxk_node_gs_oop(int n, int m, int K, const double *phases, double alpha, int dir,
                    int prec, const void *b, const void *x, void *y, mx_stream s);
/* strip width (64 or 128 positions) and band height (pairs of rows) */
int mxk_node_gs_oop_shape(int strip, int band);
void mxk_node_gs_oop_get_shape(int *strip, int *band);
/* the fused node residual + restriction takes strips of coarse rows from
 * 2^log2 (coarse node, vector, k-point) triples on (0 .. 62) */
int mxk_node_rr_set_strips(int log2);
int mxk_node_rr_get_strips(void);
int mxk_node_prolong(int nc, int m, int K, const double *phases, double alpha,
                     int prec, const void *c, void *f, mx_stream s);
int mxk_node_restrict(int nc, int m, int K, const double *phases, double alpha,
                      int prec, const void *f, void *c, mx_stream s);
/* e = ce*e + alpha * G v  (node -> edge) */
int mxk_gradient(int n, int m, int K, const double *phases, double alpha,
                 int prec_v, const void *v, int prec_e, void *e, mx_stream s);
/* v = cv*v + alpha * G^H (mass ? M e : e)  (edge -> node) */
int mxk_adjgradient(int n, int m, int K, const double *phases, double alpha, int mass,
                    double cv, int prec_e, const void *e, int prec_v, void *v, mx_stream s);

/* ---- block BLAS-1 (len complex entries) ---- */
int mxk_zero(int prec, void *x, size_t len, mx_stream s);
int mxk_convert(int prec_x, const void *x, int prec_y, void *y, size_t len, mx_stream s);
/* y += a * x with a complex scalar (re, im) */
int mxk_axpy(double are, double aim, int prec_x, const void *x, int prec_y, void *y,
             size_t len, mx_stream s);
/* out[2*(k*m+v)] += sum conj(x) y over `per` entries per vector (out zeroed by the caller) */
int mxk_dot(size_t per, int m, int K, int prec_x, const void *x, int prec_y, const void *y,
            double *out, mx_stream s);
/* Remove the mean of each plane of every (k, vector) (center_edge2d at k = 0);
 * only applied to k-points whose flag is set.  acc: 4*K*m doubles of scratch. */
int mxk_center(int n, int m, int K, const int *gamma_flag, int prec, void *x, double *acc, mx_stream s);

/* ---- further vector operations (mx_vec.cu) ---- */
/* x *= alpha over len complex entries */
int mxk_scale(double are, double aim, int prec, void *x, size_t len, mx_stream s);
/* uniform re and im in [-1, 1) from a counter-based generator keyed by seed */
int mxk_random(unsigned long long seed, int prec, void *x, size_t len, mx_stream s);
/* out[k*m+v] = max |x| over the `per` entries of each (k, v) */
int mxk_absmax(size_t per, int m, int K, int prec, const void *x, double *out, mx_stream s);
/* acc[2*((k*planes+p)*m+v)] = sum of plane p (nsite entries) of (k, v), (re, im) */
int mxk_plane_sums(int nsite, int planes, int m, int K, int prec, const void *x, double *acc, mx_stream s);
/* plane p of (k, v) += scale * c[2*((k*planes+p)*m+v)] */
int mxk_plane_shift(int nsite, int planes, int m, int K, const double *c, double scale, int prec, void *x,
                    mx_stream s);
/* kappa (n*n device doubles) from rectangles (eps, x0, y0, w, h) and circles
 * (eps, cx, cy, r) in device memory, setpattern_grid2d's rule */
int mxk_pattern(int n, const double *rect, int nrect, const double *circ, int ncirc, double eps_base,
                double *kappa, mx_stream s);

/* ---- coarse dense matrices (one per k, column-major, complex double) ---- */
/* A = alpha*A + beta*M on the 2n^2 edges of level 0 */
int mxk_dense_edge(int n, int K, const double *phases, mxk_kappa kap, double alpha,
                   double beta, double *a, mx_stream s);
/* Q1 Laplace on n^2 nodes; fixnull adds 0.1/N^2 to every entry at k = 0 */
int mxk_dense_node(int n, int K, const double *phases, int fixnull, double *a, mx_stream s);

/* ---- batched small dense linear algebra (complex double, one matrix per k) ---- */
/* in-place inverse of K Hermitian positive definite N x N matrices; info[k] != 0 on breakdown */
int mxk_hpd_inverse(int N, int K, double *a, int *info, mx_stream s);
/* y[k] = A[k] x[k] for K blocks, x,y with m columns in the batched layout of a
 * level-0 edge (N = 2n^2) or node (N = n^2) block; ainv_c64 (may be NULL) is
 * the c64 rounding of ainv that c64 solves read instead */
int mxk_coarse_apply(int N, int m, int K, const double *ainv, const void *ainv_c64, int prec,
                     const void *x, void *y, mx_stream s);
/* Hermitian eigendecomposition by parallel cyclic Jacobi: a (lower triangle
 * used) is overwritten with eigenvectors, w with ascending eigenvalues;
 * zwork: K*N*N complex doubles of scratch */
int mxk_heev(int N, int K, double *a, double *zwork, double *w, int *info, mx_stream s);
/* Rayleigh-Ritz on Gram matrices: reduced basis (sel[k*ns+i] != 0 keeps
 * column i), unit-diagonal scaling, Cholesky with column dropping
 * (pivot^2 <= drop), Jacobi on the projected A.  Outputs the lowest m Ritz
 * values and the ns x m coefficients (zero rows for dropped columns). */
/* Ritz values <= theta_min are skipped (spurious null-space modes);
 * work: mxk_ritz_work_doubles(ns) doubles per k */
size_t mxk_ritz_work_doubles(int ns);
int mxk_rayleigh_ritz(int ns, int m, int K, const double *ga, const double *gm,
                      const int *sel, double drop, double theta_min, double *coef, double *theta,
                      int *info, double *work, mx_stream s);

/* Cholesky-QR coefficients: gm (K Hermitian m x m mass Gram matrices) =
 * R^H R, coef = R^{-1} (upper triangular); info[k] = j+1 at a non-positive pivot */
int mxk_chol_qr_coef(int m, int K, const double *gm, double *coef, int *info, mx_stream s);

/* ---- block (eigenvector) kernels ---- */
/* For every (k,v): W = (A+M) e, V = M e (arithmetic of prec_e);
 * r = W - mu V written to rout (prec_r) when rout != NULL;
 * stats[(k*m+v)*5 + q] += { |r|^2, |V|^2, Re e^H W, Re e^H V, Im e^H W } */
int mxk_block_residual(int n, int m, int K, const double *phases, mxk_kappa kap,
                       const double *mu, int prec_e, const void *e, int prec_r, void *rout,
                       double *stats, mx_stream s);
/* Gram matrices of the basis S = [blocks...]: nb blocks of m vectors each,
 * block b with precision precs[b] at ptrs[b].  ga = S^H (A+M) S, gm = S^H M S,
 * full ns x ns (ns = nb*m) per k, column-major, complex double.
 * With resid (c64, the residuals r_j = (A+M) e_j - theta_j M e_j of the first
 * block, a float-float block) the entries between a low column s_i and e_j
 * are formed as theta_j s_i^H M e_j + s_i^H r_j, which keeps
 * ga - theta gm free of the cancellation that FP32 products would suffer. */
int mxk_block_gram(int n, int m, int K, const double *phases, mxk_kappa kap, int nb,
                   const int *precs, const void *const *ptrs, const void *resid,
                   const double *theta, double *ga, double *gm,
                   double *scratch, size_t scratch_bytes, mx_stream s);
/* out_j = sum_i coef(i,j) S_i for the blocks listed; coef is ldc x m per k,
 * only rows [row0, row0 + nb*m) are used; cwork: K*ldc*m*16 bytes that take
 * the coefficients as float-float pairs */
int mxk_block_combine(int n, int m, int K, int nb, const int *precs, const void *const *ptrs,
                      const double *coef, int ldc, int row0, void *cwork, int prec_out, void *out,
                      mx_stream s);
/* sel[k*ns + j*m + i] = j == 0 || all || residual i of k (from the
 * statistics of mxk_block_residual: absolute, or relative to |mu| ||M e||)
 * above tol: the columns of the Ritz basis under soft locking */
int mxk_select_columns(int ns, int m, int K, const double *stats, const double *mu, double tol,
                       int relative, int all, int *sel, mx_stream s);
/* per-cell eigenvalue sensitivity: grad[c] = -n^2 kappa_c^2 sum_{k,v} w[k*m+v] |curl_c e|^2 */
int mxk_eps_sensitivity(int n, int m, int K, const double *phases, const double *kappa,
                        const double *weights, int prec_e, const void *e, double *grad,
                        mx_stream s);

/* accessors of the public handles (mx_abi.c) */
struct grid2d_gpu;
struct edge2d_gpu;
const double *mxg__grid_phases(const struct grid2d_gpu *g);
void *mxg__edge_data(const struct edge2d_gpu *e);

#ifdef __cplusplus
}
#endif

#endif
