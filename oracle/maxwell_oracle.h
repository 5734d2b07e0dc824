/* CPU restatement of the sboerm/Maxwell Bloch eigensolver path.
 *
 * TEST INFRASTRUCTURE: this library is the checker for the CUDA path and the
 * timed CPU baseline.  It is never linked into, called by, or used as a
 * fallback for the product library (libmaxwell_gb300.so).
 *
 * Every array uses the reference's dense order (densefrom_edge2d,
 * edge2d.c:6137-6152; densefrom_node2d, node2d.c:1619-1630):
 *   edge vector  2*n*n complex: x-edge (i,j) at i+j*n, y-edge (i,j) at n*n+i+j*n
 *   node vector  n*n complex:   node (i,j) at i+j*n
 *   kappa        n*n real:      1/eps of cell (i,j) at i+j*n
 * Dense matrices are column-major with leading dimension = rows (linalg.c:8-20).
 * The grid is the unit square with hx = hy = 1/n (grid2d.c:12-32).
 */
#ifndef MAXWELL_ORACLE_H
#define MAXWELL_ORACLE_H

#include <complex.h>

typedef double complex om_cplx;

/* ---- edge space (edge2d.c) ---- */
void om_addeval_edge(int n, const double *kappa, om_cplx xf, om_cplx yf,
                     om_cplx alpha, om_cplx beta, const om_cplx *x, om_cplx *y);
om_cplx om_energyprod_edge(int n, const double *kappa, om_cplx xf, om_cplx yf,
                           om_cplx alpha, om_cplx beta,
                           const om_cplx *x, const om_cplx *y);
om_cplx om_massprod_edge(int n, om_cplx xf, om_cplx yf,
                         const om_cplx *x, const om_cplx *y);
om_cplx om_dot(long len, const om_cplx *x, const om_cplx *y);
double om_norm2(long len, const om_cplx *x);
void om_gs_edge(int n, const double *kappa, om_cplx xf, om_cplx yf,
                om_cplx alpha, om_cplx beta, int dir,
                const om_cplx *b, om_cplx *x);
/* point Gauss-Seidel in the reference's interleaved row order (gs*_simple_edge2d) */
void om_gs_edge_simple(int n, const double *kappa, om_cplx xf, om_cplx yf,
                       om_cplx alpha, om_cplx beta, int dir, const om_cplx *b, om_cplx *x);
/* the same patch solves in four vertex colours (the GPU solver's order) */
void om_gs_edge_colour(int n, const double *kappa, om_cplx xf, om_cplx yf,
                       om_cplx alpha, om_cplx beta, int dir, const om_cplx *b, om_cplx *x);
void om_prolong_edge(int nc, om_cplx xf, om_cplx yf, om_cplx alpha,
                     const om_cplx *c, om_cplx *f);
void om_restrict_edge(int nc, om_cplx xf, om_cplx yf, om_cplx alpha,
                      const om_cplx *f, om_cplx *c);
void om_center_edge(int n, om_cplx *x);
void om_nullprod_edge(int n, const om_cplx *x, om_cplx *xprod, om_cplx *yprod);
void om_nulladd_edge(int n, om_cplx xalpha, om_cplx yalpha, om_cplx *x);
double om_normmax(long len, const om_cplx *x);
void om_dense_edge(int n, const double *kappa, om_cplx xf, om_cplx yf,
                   om_cplx alpha, om_cplx beta, om_cplx *a);

/* ---- node space (node2d.c) ---- */
void om_addeval_node(int n, om_cplx xf, om_cplx yf, om_cplx alpha,
                     const om_cplx *x, om_cplx *y);
void om_gs_node(int n, om_cplx xf, om_cplx yf, om_cplx alpha, int dir,
                const om_cplx *b, om_cplx *x);
void om_prolong_node(int nc, om_cplx xf, om_cplx yf, om_cplx alpha,
                     const om_cplx *c, om_cplx *f);
void om_restrict_node(int nc, om_cplx xf, om_cplx yf, om_cplx alpha,
                      const om_cplx *f, om_cplx *c);
void om_gradient(int n, om_cplx xf, om_cplx yf, om_cplx alpha,
                 const om_cplx *v, om_cplx *e);
void om_adjgradient(int n, om_cplx xf, om_cplx yf, om_cplx alpha,
                    const om_cplx *e, om_cplx *v);
void om_dense_node(int n, om_cplx xf, om_cplx yf, int fixnull, om_cplx *a);
void om_center_node(int n, om_cplx *v);

/* ---- grid (grid2d.c) ---- */
void om_coarsen_kappa(int n, const double *kfine, double *kcoarse);
void om_disc_kappa(int n, int ndiscs, const double *discs /* eps, cx, cy, r */,
                   double eps_base, double *kappa);
void om_pattern_kappa(int n, int nrect, const double *rect, int ncirc, const double *circ,
                      double eps_base, double *kappa);

/* ---- dense linear algebra (linalg.c replacements) ---- */
int om_potrf(int n, om_cplx *a);
void om_potrs(int n, const om_cplx *l, om_cplx *b);
int om_heev(int n, om_cplx *a, double *w);
int om_hegv(int n, om_cplx *a, om_cplx *b, double *w);
int om_rr_svqb(int n, const om_cplx *ga, const om_cplx *gm, int m,
               double drop, om_cplx *c, double *theta);

/* ---- multigrid on one Bloch parameter ---- */
typedef struct om_mg om_mg;
om_mg *om_mg_new(int n0, int L, const double *kappa_fine);
void om_mg_free(om_mg *h);
int om_mg_set_bloch(om_mg *h, om_cplx xf, om_cplx yf);
void om_vcycle_edge(om_mg *h, int l, int nu, int coarse,
                    const om_cplx *b, om_cplx *x);
void om_vcycle_node(om_mg *h, int l, int nu, int coarse,
                    const om_cplx *b, om_cplx *x);
/* the Hiptmair cycle (hcycle_edge2d) with the point smoother */
void om_hcycle_edge(om_mg *h, int l, int nu, int coarse,
                    const om_cplx *b, om_cplx *x);
const double *om_mg_kappa(const om_mg *h, int l);

/* ---- the per-k eigensolver flow ---- */
typedef struct {
  int n0, L;             /* coarse intervals, refinement levels */
  int ieigs, m;          /* wanted pairs, block size (wanted + throw-away) */
  int method;            /* 0 block PINVIT + Ritz, 1 LOBPCG */
  int max_nested;        /* block steps per level of the nested iteration */
  int max_steps;         /* block steps per k-point */
  int prec_steps;        /* edge V-cycles per preconditioner application */
  int gradient_steps;    /* node V-cycles per gradient lifting */
  int smoother_steps;    /* nu, GS sweeps per level */
  int lift_e;            /* LOBPCG: also lift the new eigenvector block */
  int center;            /* remove constant fields at k = 0 */
  int extrapolation;     /* 'n', '1' or '2' */
  int wave;              /* k-points solved together; wave w starts from wave w-1 */
  int relative;          /* 0 absolute defect (reference), 1 relative residual */
  double tol;
  double nested_tol;     /* tolerance of the nested iteration's coarser levels; 0 = tol */
} om_opts;

int om_bloch_solve(const om_opts *o, const double *kappa_fine,
                   int nk, const om_cplx *xfs, const om_cplx *yfs,
                   double *lambda_out, int *steps_out, double *res_out,
                   om_cplx *evec_out);
/* the same, with the wall-clock seconds spent on every k-point (may be NULL) */
int om_bloch_solve_timed(const om_opts *o, const double *kappa_fine,
                         int nk, const om_cplx *xfs, const om_cplx *yfs,
                         double *lambda_out, int *steps_out, double *res_out,
                         om_cplx *evec_out, double *seconds_out);

/* Eigenvector continuity ('n', 's', 'r') and Chern partial sums along nk
 * consecutive k-points (exp_bloch2d.c:1058-1216); vecs and lambda adjusted
 * in place, chern nk*chern_vectors partial sums, sign nk swap counts. */
void om_continuity(int n, int nk, const om_cplx *xfs, const om_cplx *yfs, int m, int ieigs,
                   const int *vertex, int continuity, int chern_vectors, om_cplx *vecs, double *lambda,
                   om_cplx *chern, int *sign);

/* Eigenvalue sensitivity with respect to the permittivity of every cell. */
void om_eps_sensitivity(int n, const double *kappa, om_cplx xf, om_cplx yf,
                        int nvec, const om_cplx *e, const double *weights,
                        double *grad);

int om_max_threads(void);
void om_set_threads(int t);

#endif
