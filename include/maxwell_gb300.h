/* libmaxwell_gb300: C ABI of the GB300 (sm_103a) Bloch eigensolver.
 *
 * Drop-in for the multigrid-preconditioned block eigensolver of sboerm/Maxwell
 * on one GPU.  The names mirror the reference's interfaces with a _gpu
 * suffix; every object lives in device memory and holds a BATCH: K Bloch
 * parameters (k-points) times m vectors.  K = m = 1 gives the reference's
 * single-vector semantics.
 *
 *   reference (file:line)                      this library
 *   grid2d.h:7-78   grid2d, new/del/coarsen    grid2d_gpu, new/del/coarsen_grid2d_gpu
 *   edge2d.h:12-29  edge2d                     edge2d_gpu
 *   edge2d.h:71-291 vector, operator, GS,      *_edge2d_gpu (same argument meaning;
 *                   transfer, V-cycle, dense    scalars per vector come back as arrays)
 *   node2d.h:9-158  node2d + its functions     *_node2d_gpu
 *   linalg.h:7-31   matrix, potrf, potrsv,     matrix_gpu, potrf_matrix_gpu, ...
 *                   syev, sygv
 *   exp_bloch2d.c:556-1053 per-k driver flow   mxg_bloch_solve
 *   (new)                                      mxg_eps_sensitivity
 *
 * Scalar ABI (settings.h:5-17 with FIELD_COMPLEX): real = double,
 * field = double complex.  Host arrays of vectors use the reference's dense
 * order per vector (densefrom_edge2d, edge2d.c:6137-6152): the n*n x-edge
 * coefficients (i + j*n) followed by the n*n y-edge coefficients; batches are
 * [k][vector][entries].
 *
 * Errors: every function returns 0 on success, a negative MXG_E* code for a
 * usage error, or a positive cudaError_t value (the reference's vector
 * functions return void and assert; its LAPACK wrappers return info,
 * linalg.c:54-63,261-317, which potrf/syev/sygv_matrix_gpu return through an
 * info array).  Calls on one grid are stream-ordered; results written to host
 * memory are complete when the call returns.
 *
 * There is no CPU fallback: without a CUDA device every compute call returns
 * a cudaError_t value.
 */
#ifndef MAXWELL_GB300_H
#define MAXWELL_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
typedef struct { double re, im; } mxg_field;
#else
#include <complex.h>
typedef double _Complex mxg_field;
#endif

enum { MXG_C64 = 0, MXG_C128 = 1, MXG_CDD = 2 };   /* storage of a vector batch */

#define MXG_EINVAL (-1)     /* bad argument, shape or precision */
#define MXG_ENOMEM (-2)     /* device allocation failed */
#define MXG_ECONV (-3)      /* Ritz step broke down (rank-deficient basis) */

typedef struct grid2d_gpu grid2d_gpu;
typedef struct edge2d_gpu edge2d_gpu;
typedef struct node2d_gpu node2d_gpu;
typedef struct matrix_gpu matrix_gpu;

/* ---------- grid2d (grid2d.h:36-78) ---------- */
/* new_grid2d (grid2d.c:12-32): nx = ny intervals of the unit square, K Bloch
 * parameters (all factors 1, kappa = 1/eps = 1) */
grid2d_gpu *new_grid2d_gpu(int nx, int ny, double hx, double hy, int K);
void del_grid2d_gpu(grid2d_gpu *gr);
/* coarsen_grid2d (grid2d.c:42-68): kappa averaged over 2x2 children, same factors */
grid2d_gpu *coarsen_grid2d_gpu(const grid2d_gpu *fine);
/* gr->eps (the reciprocal permittivity per cell, grid2d.c:191-214), n*n host doubles */
int setkappa_grid2d_gpu(grid2d_gpu *gr, const double *kappa);
/* gr->xfactor / gr->yfactor for each of the K Bloch parameters */
int setbloch_grid2d_gpu(grid2d_gpu *gr, const mxg_field *xfactor, const mxg_field *yfactor);
int getsize_grid2d_gpu(const grid2d_gpu *gr, int *nx, int *K);
/* the reciprocal permittivity per cell as set on the grid, n*n host doubles */
int getkappa_grid2d_gpu(const grid2d_gpu *gr, double *kappa);
/* epspattern (grid2d.h:40-62): rectangles as (eps, left, bottom, width,
 * height), circles as (eps, centre x, centre y, radius), eps_base around them */
typedef struct {
  double *rectangle;
  int rectangles;
  double *circle;
  int circles;
  double eps_base;
} mxg_epspattern;
/* new_epspattern / del_epspattern (grid2d.c:148-169): zeroed shape arrays */
mxg_epspattern *new_epspattern_gpu(double eps_base, int rectangles, int circles);
void del_epspattern_gpu(mxg_epspattern *pat);
/* setpattern_grid2d (grid2d.c:171-218): 1/eps of every cell from the pattern,
 * each cell tested at its lower-left corner, circles after rectangles; the
 * rasterisation runs on the device.  A NULL pattern leaves the grid as it is. */
int setpattern_grid2d_gpu(const mxg_epspattern *pat, grid2d_gpu *gr);

/* ---------- edge2d (edge2d.h:71-291) ---------- */
edge2d_gpu *new_edge2d_gpu(const grid2d_gpu *gr, int m, int prec);
void del_edge2d_gpu(edge2d_gpu *x);
size_t getdimension_edge2d_gpu(const edge2d_gpu *x);          /* 2 nx ny per vector */
int zero_edge2d_gpu(edge2d_gpu *x);
int copy_edge2d_gpu(const edge2d_gpu *x, edge2d_gpu *y);      /* converts precision */
int add_edge2d_gpu(mxg_field alpha, const edge2d_gpu *x, edge2d_gpu *y);
/* swap_edge2d (edge2d.c:126-159): exchanges the contents of two batches of
 * the same shape and precision (their device storage changes hands) */
int swap_edge2d_gpu(edge2d_gpu *x, edge2d_gpu *y);
/* random_edge2d (edge2d.c:161-191): real and imaginary parts uniform in
 * [-1, 1).  The reference draws from rand(); here a counter-based generator
 * (SplitMix64) keyed by seed gives the same values on every device and
 * for every launch shape. */
int random_edge2d_gpu(edge2d_gpu *x, unsigned long long seed);
/* scale_edge2d (edge2d.c:806-828): x *= alpha */
int scale_edge2d_gpu(mxg_field alpha, edge2d_gpu *x);
/* norms and products per (k, vector): out has K*m entries */
int norm2_edge2d_gpu(const edge2d_gpu *x, double *out);
/* normmax_edge2d (edge2d.c:887-920): max |x_e| per (k, vector) */
int normmax_edge2d_gpu(const edge2d_gpu *x, double *out);
/* dotprod_edge2d (edge2d.c:1207-1238): sum conj(x_e) y_e per (k, vector) */
int dotprod_edge2d_gpu(const edge2d_gpu *x, const edge2d_gpu *y, mxg_field *out);
/* nullprod_edge2d (edge2d.c:1240-1274): L2 products of x with the two
 * constant fields, hy * (sum of the x-edge coefficients) and
 * hx * (sum of the y-edge coefficients), per (k, vector); xprod or yprod may
 * be NULL.  Defined for k = 0 (the reference asserts xfactor = yfactor = 1);
 * computed for every k-point of the batch as given. */
int nullprod_edge2d_gpu(const edge2d_gpu *x, mxg_field *xprod, mxg_field *yprod);
/* nulladd_edge2d (edge2d.c:1276-1307): x-edges += hx xalpha, y-edges +=
 * hy yalpha, one pair of scalars per (k, vector) */
int nulladd_edge2d_gpu(const mxg_field *xalpha, const mxg_field *yalpha, edge2d_gpu *x);
int center_edge2d_gpu(edge2d_gpu *x);
/* No counterpart in the reference.  center_edge2d_gpu for callers that must
 * not allocate device memory (an application that owns a fixed device budget
 * or its own pool, or a loop that cannot take the device synchronisation
 * cudaMalloc/cudaFree may cause).  x: device batch of K k-points x m vectors
 * in the device layout [k][2n^2 entries][vector], precision prec; gamma_flag:
 * K device ints, non-zero for the k-points to centre; stream: a cudaStream_t
 * (NULL = the legacy default stream) on which the work is enqueued.  The call
 * allocates nothing: its scratch (4 doubles per k-point and vector) is a
 * static device array for at most MXG_CENTER_NOALLOC_MAX_KM (k-point, vector)
 * pairs (256 KiB, held by every GPU that loads the library until exit); a
 * larger K*m returns MXG_EINVAL.  The device current for the calling thread
 * must be the one that owns x, gamma_flag and the stream (a stream of another
 * device returns MXG_EINVAL).  The first call on a device looks up the
 * array's address there, so make it before any stream capture.  All calls on
 * a device share the array: calls that overlap on the GPU race. */
#define MXG_CENTER_NOALLOC_MAX_KM 8192
int center_edge2d_gpu_noalloc(int n, int m, int K, const int *gamma_flag, int prec, void *x, void *stream);
/* y += alpha A x + beta M x (edge2d.c:1335-1650) */
int addeval_edge2d_gpu(mxg_field alpha, mxg_field beta, const edge2d_gpu *x, edge2d_gpu *y);
/* the same with one beta per (k, vector): the PINVIT defect with its own shift */
int addeval_shifted_edge2d_gpu(double alpha, const double *beta_per_vector,
                               const edge2d_gpu *x, edge2d_gpu *y);
/* x^H (alpha A + beta M) y and x^H M y per (k, vector) (edge2d.c:1652-2027) */
int energyprod_edge2d_gpu(mxg_field alpha, mxg_field beta, const edge2d_gpu *x,
                          const edge2d_gpu *y, mxg_field *out);
int massprod_edge2d_gpu(const edge2d_gpu *x, const edge2d_gpu *y, mxg_field *out);
/* AFW Gauss-Seidel (edge2d.c:2656-3042) */
int gsforward_edge2d_gpu(mxg_field alpha, mxg_field beta, const edge2d_gpu *b, edge2d_gpu *x);
int gsbackward_edge2d_gpu(mxg_field alpha, mxg_field beta, const edge2d_gpu *b, edge2d_gpu *x);
int gssymm_edge2d_gpu(mxg_field alpha, mxg_field beta, const edge2d_gpu *b, edge2d_gpu *x);
/* No counterpart in the reference: the same vertex-patch solves in four
 * vertex colours, (0,0), (1,0), (0,1), (1,1) by (i mod 2, j mod 2), each colour
 * one parallel pass; dir 0 forward, 1 backward (reverse colour order), 2 both.
 * The solver's default smoother (mxg_solve_opts.smoother = 1). */
int gscolour_edge2d_gpu(mxg_field alpha, mxg_field beta, const edge2d_gpu *b, edge2d_gpu *x, int dir);
/* point Gauss-Seidel, edge by edge, in the reference's interleaved row order
 * (gsforward/gsbackward/gssymm_simple_edge2d, edge2d.c:3890-5581): the
 * smoother of the Hiptmair cycle */
int gsforward_simple_edge2d_gpu(mxg_field alpha, mxg_field beta, const edge2d_gpu *b, edge2d_gpu *x);
int gsbackward_simple_edge2d_gpu(mxg_field alpha, mxg_field beta, const edge2d_gpu *b, edge2d_gpu *x);
int gssymm_simple_edge2d_gpu(mxg_field alpha, mxg_field beta, const edge2d_gpu *b, edge2d_gpu *x);
/* transfers (edge2d.c:5583-5705) */
int prolongation_edge2d_gpu(mxg_field alpha, const edge2d_gpu *c, edge2d_gpu *f);
int restriction_edge2d_gpu(mxg_field alpha, const edge2d_gpu *f, edge2d_gpu *c);
/* vcycle_edge2d (edge2d.c:5707-5754): b, x, d arrays of L+1 levels */
int vcycle_edge2d_gpu(int L, int nu, const matrix_gpu *Ac, edge2d_gpu **b, edge2d_gpu **x,
                      edge2d_gpu **d);
/* hcycle_edge2d (edge2d.c:5756-5823): the Hiptmair cycle for A+M -- point
 * Gauss-Seidel plus a correction in the gradients (nu node Gauss-Seidel
 * sweeps on G^H of the residual) on every level, the coarse dense solve
 * with Ac (or nu symmetric point sweeps); bg, xg: node work vectors of the
 * L+1 levels */
int hcycle_edge2d_gpu(int L, int nu, const matrix_gpu *Ac, edge2d_gpu **b, edge2d_gpu **x, edge2d_gpu **d,
                      node2d_gpu **bg, node2d_gpu **xg);
/* densematrix_edge2d (edge2d.c:5870-6116) for every k of the grid */
int densematrix_edge2d_gpu(mxg_field alpha, mxg_field beta, const grid2d_gpu *gr, matrix_gpu *a);
/* host <-> device in the reference's dense order (denseto/densefrom_edge2d) */
int denseto_edge2d_gpu(const mxg_field *host, edge2d_gpu *y);
int densefrom_edge2d_gpu(const edge2d_gpu *x, mxg_field *host);
/* The Ritz products of exp_bloch2d.c:991-996 for the whole block in one call:
 * a[k] = X^H (A+M) X (energyprod_edge2d(1, 1, .)) and m[k] = X^H M X
 * (massprod_edge2d) for the m vectors of every k-point, full Hermitian
 * m x m matrices, column-major, K of each; a or m may be NULL; m <= 48 */
int gram_edge2d_gpu(const edge2d_gpu *x, mxg_field *a, mxg_field *m);
/* The Ritz combination of exp_bloch2d.c:1006-1010 (e_j = sum_i C_ij u_i,
 * m^2 add_edge2d calls) in one call: y[k][j] = sum_i coef[k](i, j) x[k][i],
 * coef K column-major m x m matrices; x and y distinct, same shape */
int lincomb_edge2d_gpu(const mxg_field *coef, const edge2d_gpu *x, edge2d_gpu *y);
/* orthonormalize_edge2d (edge2d.c:6264-6296): makes the m vectors of every
 * k-point orthonormal in the mass inner product, the first j of them
 * spanning what the first j spanned before.  The reference uses Householder
 * reflections in the M inner product; this is Cholesky-QR: X^H M X = R^H R,
 * X <- X R^-1 (R with a positive real diagonal).  info[k] = 0, or j+1 if
 * column j of k-point k is dependent on the columns before it (the part of
 * it outside their span has less than 1e-5 of its M-norm); then nothing is
 * changed and the call returns MXG_ECONV. */
int orthonormalize_edge2d_gpu(edge2d_gpu *x, int *info);

/* ---------- node2d (node2d.h:28-158) ---------- */
node2d_gpu *new_node2d_gpu(const grid2d_gpu *gr, int m, int prec);
void del_node2d_gpu(node2d_gpu *x);
int zero_node2d_gpu(node2d_gpu *x);
int addeval_node2d_gpu(mxg_field alpha, const node2d_gpu *x, node2d_gpu *y);
int gsforward_node2d_gpu(mxg_field alpha, const node2d_gpu *b, node2d_gpu *x);
int gsbackward_node2d_gpu(mxg_field alpha, const node2d_gpu *b, node2d_gpu *x);
int gssymm_node2d_gpu(mxg_field alpha, const node2d_gpu *b, node2d_gpu *x);
int prolongation_node2d_gpu(mxg_field alpha, const node2d_gpu *c, node2d_gpu *f);
int restriction_node2d_gpu(mxg_field alpha, const node2d_gpu *f, node2d_gpu *c);
/* no reference counterpart: c = restriction of (b - alpha L x), the node
 * V-cycle's residual and restriction (node2d.c:1352-1389) in one pass, c
 * overwritten */
int residual_restriction_node2d_gpu(mxg_field alpha, const node2d_gpu *b, const node2d_gpu *x, node2d_gpu *c);
int gradient_node2d_gpu(mxg_field alpha, const node2d_gpu *x, edge2d_gpu *y);
int adjgradient_node2d_gpu(mxg_field alpha, const edge2d_gpu *x, node2d_gpu *y);
int vcycle_node2d_gpu(int L, int nu, const matrix_gpu *Ac, node2d_gpu **b, node2d_gpu **x,
                      node2d_gpu **d);
int densematrix_node2d_gpu(int fixnull, const grid2d_gpu *gr, matrix_gpu *a);
int denseto_node2d_gpu(const mxg_field *host, node2d_gpu *y);
int densefrom_node2d_gpu(const node2d_gpu *x, mxg_field *host);
/* the vector operations of node2d.h:42-84, as their edge counterparts */
int copy_node2d_gpu(const node2d_gpu *x, node2d_gpu *y);                  /* node2d.c:53-70 */
int random_node2d_gpu(node2d_gpu *x, unsigned long long seed);            /* node2d.c:72-90 */
int scale_node2d_gpu(mxg_field alpha, node2d_gpu *x);                     /* node2d.c:385-399 */
int add_node2d_gpu(mxg_field alpha, const node2d_gpu *x, node2d_gpu *y);  /* node2d.c:401-418 */
int norm2_node2d_gpu(const node2d_gpu *x, double *out);                   /* node2d.c:420-439 */
int normmax_node2d_gpu(const node2d_gpu *x, double *out);                 /* node2d.c:441-463 */
int dotprod_node2d_gpu(const node2d_gpu *x, const node2d_gpu *y, mxg_field *out); /* node2d.c:465-487 */
/* center_node2d (node2d.c:489-514): subtract the mean coefficient */
int center_node2d_gpu(node2d_gpu *x);

/* ---------- linalg (linalg.h:7-31): one square matrix per k ---------- */
matrix_gpu *new_matrix_gpu(int rows, int K);
void del_matrix_gpu(matrix_gpu *a);
int upload_matrix_gpu(matrix_gpu *a, const mxg_field *host);      /* K column-major */
int download_matrix_gpu(const matrix_gpu *a, mxg_field *host);
/* potrf_matrix (linalg.c:54-63) prepares the coarse solve: the factor is kept
 * as the explicit inverse, so potrsv applies one matrix-vector product;
 * info[k] as zpotrf's */
int potrf_matrix_gpu(matrix_gpu *a, int *info);
/* potrsv_matrix (linalg.c:98-113): b <- A^-1 b for every k after
 * potrf_matrix_gpu; b holds K host vectors of `rows` entries */
int potrsv_matrix_gpu(const matrix_gpu *a, mxg_field *b);
/* sygv_matrix (linalg.c:285-317), itype 1: a <- B-orthonormal eigenvectors,
 * lambda (K*rows) ascending, info per k */
int sygv_matrix_gpu(matrix_gpu *a, matrix_gpu *b, double *lambda, int *info);
/* syev_matrix (linalg.c:254-283) */
int syev_matrix_gpu(matrix_gpu *a, double *lambda, int *info);

/* ---------- one PINVIT step (edge2d.h:287-291) ---------- */
/* pinvit_edge2d (edge2d.c:6298-6328) on level l for every (k, vector) of e:
 * defect (A+M) e - lambda M e, prec_steps edge V-cycles with smoother_steps
 * sweeps, e -= update, then the gradient lifting with gradient_steps node
 * V-cycles.  lambda: K*m host doubles (one shift per vector, as the
 * reference is called once per vector with its own Rayleigh quotient). */
int pinvit_edge2d_gpu(int l, int smoother_steps, int prec_steps, int gradient_steps, const double *lambda,
                      edge2d_gpu *e, const matrix_gpu *Ae, edge2d_gpu **b, edge2d_gpu **x, edge2d_gpu **d,
                      const matrix_gpu *An, node2d_gpu **bg, node2d_gpu **xg, node2d_gpu **dg);

/* ---------- the per-k eigensolver (exp_bloch2d.c:556-1053) ---------- */
typedef struct {
  int n0, L;             /* coarse intervals, refinement levels (n = n0 << L) */
  int ieigs, m;          /* wanted pairs, block size (m <= 32) */
  int method;            /* 0 block PINVIT + Ritz (exp_bloch2d), 1 LOBPCG */
  int precision;         /* 0 plain FP64, 1 mixed (FP32 multigrid, float-float eigenvectors),
                          * 2 mixed with FP64 eigenvectors (FP32 multigrid and search
                          * blocks): the float-float block's residual floor, about
                          * ||A|| 2^-48 / lambda relative, grows with n^2 (near 1e-9 at
                          * 1024^2); FP64 lowers it 32-fold */
  int max_nested;        /* block steps per level of the nested iteration */
  int max_steps;         /* block steps at the finest level */
  int prec_steps;        /* edge V-cycles per preconditioner application */
  int gradient_steps;    /* node V-cycles per gradient lifting */
  int smoother_steps;    /* nu */
  int lift_e;            /* LOBPCG: lift the new eigenvector block as well */
  int center;            /* remove the constant fields at k = 0 */
  int wave;              /* k-points per batch; batch w starts from batch w-1 */
  int relative;          /* stopping rule: 0 absolute defect, 1 relative residual */
  double tol;
  int smoother;          /* preconditioner: AFW V-cycle with 0 the reference's row order or
                          * 1 four colours; 2 the Hiptmair cycle (hcycle_edge2d) */
  double drop;           /* Ritz step: columns whose Cholesky-QR pivot^2 falls below this
                          * are dropped; 0 = 1e-6 (mixed) or 1e-12 (plain FP64) */
  int extrapolation;     /* start of every wave after the first, from the same slots of
                          * earlier waves (exp_bloch2d.c:814-895, maxwell_extra):
                          * 'n' or 0 their eigenvectors, '1' Rayleigh-Ritz over the last
                          * two waves, '2' over the last three; 'c' no warm start, every
                          * wave from the nested iteration */
  int refine;            /* 1: after the finest level converges, one more block step with
                          * every search column in the Ritz basis (the refinement sweep
                          * of the 2048^2 configuration), residuals recomputed after it */
  double nested_tol;     /* stopping tolerance of the nested iteration's coarser levels
                          * (the reference's 'r' rule stops them at a defect of 1e-2,
                          * exp_bloch2d.c:296-321, 628); 0 = tol */
} mxg_solve_opts;

typedef struct mxg_solver mxg_solver;
/* Makes CUDA device `device` current for the calling thread (cudaSetDevice):
 * one process per GPU selects its GPU with this before creating objects.
 * A solver lives on the device that was current when it was created and
 * makes that device current again in each of its calls. */
int mxg_set_device(int device);
/* kappa_fine: n*n host doubles */
mxg_solver *mxg_solver_new(const mxg_solve_opts *o, const double *kappa_fine);
void mxg_solver_free(mxg_solver *s);
/* Solve nk k-points (factors e^{i kx}, e^{i ky}); outputs lambda = mu - 1
 * (nk*m), block steps per k (nk), final residual per vector (nk*m).  A
 * k-point within 1e-8 of Gamma (|xf - 1| + |yf - 1| in the 1-norm of the
 * components) gets the constant-field removal when o.center is set. */
int mxg_bloch_solve(mxg_solver *s, int nk, const mxg_field *xfactor, const mxg_field *yfactor,
                    double *lambda, int *steps, double *residual);
/* The full-zone surface of exp_blochsurf (exp_blochsurf.c:25-37, 964-1489):
 * steps x steps k-points k = 2 pi (ix, iy) / (steps - 1) - (pi, pi), solved
 * in waves of o.wave k-points in row order (iy outer); every wave after the
 * first starts from the earlier waves as o.extrapolation says (with o.wave
 * = steps, each k-point from the same column of the rows below it, the
 * reference's extrapolation along y).  Outputs as mxg_bloch_solve, indexed
 * (iy * steps + ix). */
int mxg_bloch_surface(mxg_solver *s, int steps, double *lambda, int *nsteps, double *residual);
/* Eigenvector continuity and Chern partial sums along the k-points of the
 * last mxg_bloch_solve (exp_bloch2d.c:1058-1216), which must have fitted one
 * wave (nk <= o.wave), taken as consecutive points of a curve.  For every
 * point l >= 1, with eold0 / eold1 the adjusted vectors of points l-1 / l-2
 * and the mass products taken with M(k_l):
 *   continuity 'r': for i < ieigs, the vector closest to eold0_i (after a
 *     vertex, vertex[l-1] != 0) or to 2 eold0_i - eold1_i takes place i
 *     (swapping eigenvalues; sign[l] counts the swaps so far), then 's';
 *   continuity 's': every vector is scaled by a unit phase that makes
 *     e_i^H M eold0_i (after a vertex) or e_i^H M (2 eold0_i - eold1_i)
 *     real and positive; 'n' leaves the vectors as they are;
 *   Chern sums, for i < chern_vectors: += (i/2) eold0_i^H M (e_i - eold0_i)
 *     after a vertex, else (i/2) eold0_i^H M (e_i - eold1_i), plus
 *     (i/2) e_i^H M (e_i - eold0_i) when point l is itself a vertex.
 * vertex: nk flags (the curve's corners; the first point counts as one,
 * as exp_bloch2d.c:447 starts); lambda: the nk*m eigenvalues of the solve,
 * reordered in place; chern: nk*chern_vectors partial sums (row 0 zero);
 * sign: nk swap counts or NULL.  The solver's eigenvectors are left
 * adjusted (mxg_solver_eigenvectors returns them so).  Mass products in
 * complex128 on the device; the decisions on the host. */
int mxg_bloch_continuity(mxg_solver *s, int nk, const int *vertex, int continuity, int chern_vectors,
                         double *lambda, mxg_field *chern, int *sign);
/* The protocol file of the reference's Bloch scan (exp_bloch2d.c:416-443
 * header, 754-760 the starting point, 1227-1235 every later point): the
 * header with the settings below, then per point its index, the m
 * eigenvalues, block steps, seconds for the point and accumulated seconds,
 * the real and imaginary part of each Chern partial sum and the swap count,
 * formatted as the reference formats them.  steps, seconds and sign may be
 * NULL (written as 0); chern (nk*chern_vectors) may be NULL when
 * chern_vectors is 0. */
typedef struct {
  const char *pattern;   /* "Permittivity pattern" of the header */
  int n0, L;             /* coarse grid intervals, refinement levels */
  int chern_vectors;
  int extrapolation;     /* 'n', '1', '2', 'c' */
  int stopping;          /* 'r' residual, 'f' fixed steps */
  int continuity;        /* 'n', 's', 'r' */
} mxg_protocol_info;
int mxg_write_protocol(const char *filename, const mxg_protocol_info *info, int nk, int m, const double *lambda,
                       const int *steps, const double *seconds, const mxg_field *chern, const int *sign);
/* eigenvectors of the last solved batch: wave k-points x m vectors in dense order */
int mxg_solver_eigenvectors(const mxg_solver *s, mxg_field *host);
/* device time of the last mxg_bloch_solve in milliseconds, and the number of
 * kernel launches it issued */
int mxg_solver_stats(const mxg_solver *s, double *ms, long *launches);
/* The relative residuals ||(A+M) e - mu M e|| / (mu ||M e||) of the last
 * solved wave (o.wave k-points x m vectors) recomputed in FP64: the
 * eigenvectors converted to complex128 on the device and the residual
 * formed by the complex128 operator kernel in double arithmetic. */
int mxg_solver_check_fp64(mxg_solver *s, double *res);
/* warm-started waves of the last mxg_bloch_solve / mxg_bloch_surface that
 * missed the tolerance and were solved again from a cold start */
int mxg_solver_restarts(const mxg_solver *s);
/* CUDA-event timing, on the solver's stream, of three launch sequences at
 * the finest level: node Gauss-Seidel sweeps of the gradient lifting
 * (MXG_KT_NODE_GS), AFW sweeps of the preconditioner (MXG_KT_AFW) and the
 * Gram matrices of the Ritz step (MXG_KT_GRAM).  With profiling enabled the
 * solver launches the V-cycles directly (no CUDA graph) so that every sweep
 * carries its own events.  kernel_time returns, since profiling was enabled,
 * the summed milliseconds, the number of timed sequences and their summed
 * algorithmic bytes (each array the sequence reads or writes counted once). */
enum { MXG_KT_NODE_GS = 0, MXG_KT_AFW = 1, MXG_KT_GRAM = 2, MXG_KT_N = 3 };
int mxg_solver_profile(mxg_solver *s, int enable);
int mxg_solver_kernel_time(mxg_solver *s, int which, double *ms, long *count, double *bytes);

/* ---------- eigenvalue sensitivity (no counterpart in the reference) ---------- */
/* grad[c] = sum_{k,v} w[k*m+v] d lambda_{k,v} / d eps_c for M-normalised
 * eigenvectors e (host, nk*m*2n^2 in dense order):
 * d lambda / d eps_c = -kappa_c^2 |curl_c e|^2 / (hx hy) */
int mxg_eps_sensitivity(int n, const double *kappa, int nk, const mxg_field *xfactor,
                        const mxg_field *yfactor, int m, const mxg_field *evec,
                        const double *weights, double *grad);

/* ---------- per-kernel timing (no counterpart in the reference) ---------- */
/* Times each hot kernel of one block step at n x n cells, K k-points and
 * block m (<= 16) on synthetic blocks: `reps` calls after one untimed call,
 * CUDA events on the launching stream.  Fills up to maxrows (>= 16) rows with
 * the mean milliseconds per call, the call's algorithmic bytes (each array
 * read or written once) and its kernel launches; returns the number of rows,
 * MXG_EINVAL / MXG_ENOMEM, or -1000 - cudaError_t. */
typedef struct {
  char name[40];
  double ms;
  double bytes;
  int launches;
} mxg_kbench_row;
int mxg_kernel_bench(int n, int K, int m, int reps, mxg_kbench_row *rows, int maxrows);

/* ---------- launch-shape autotuner (no counterpart in the reference) ---------- */
/* Launch shapes, process-wide: the Gram's CTAs per k-point (gram_waves x
 * SMs / K), the tiled combination's CTAs (combine_ctas x SMs), the block
 * residual's sites per thread, the tiled node Gauss-Seidel sweep's strip
 * width (positions) and band height (pairs of rows) per CTA, and from which
 * batch the node V-cycle's residual + restriction walks strips of coarse
 * rows (coarse nodes x vectors x k-points >= 2^restrict_strip_log2) instead
 * of taking a thread per coarse node. */
typedef struct {
  int gram_waves;        /* 1 .. 64 */
  int combine_ctas;      /* 1 .. 16 */
  int residual_sites;    /* 1 .. 1024 */
  int node_strip;        /* 0 (the in-place row kernels), 64 or 128 */
  int node_band;         /* 1 .. 256 */
  int restrict_strip_log2; /* 0 .. 62 (0: always strips, 62: never) */
} mxg_tuning;
int mxg_get_tuning(mxg_tuning *t);
int mxg_set_tuning(const mxg_tuning *t);
/* Times each shape's candidates (`reps` calls after one untimed call, CUDA
 * events) on synthetic blocks of n x n cells, K k-points and block m <= 16,
 * one tunable after the other, keeps the fastest and returns the choice.
 * The block kernels' shapes change launch geometry only (results the same
 * up to the order of floating-point sums); the node sweep's strip width
 * also moves where its truncated prefix sums start, at the 8^-9 level. */
int mxg_autotune(int n, int K, int m, int reps, mxg_tuning *chosen);

int mxg_device_ok(void);

#ifdef __cplusplus
}
#endif

#endif
