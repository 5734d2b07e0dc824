/* A C driver written against the library's mirror of the reference's
 * edge2d / node2d / grid2d / linalg interfaces, in the order the reference's
 * Bloch driver calls them (exp_bloch2d.c:335-554 set-up, 562-732 nested
 * iteration, 956-1018 block PINVIT + Ritz), for a batch of k-points at once:
 *
 *   new_grid2d / setpattern_grid2d / coarsen_grid2d / Bloch factors
 *   densematrix_edge2d + potrf_matrix, densematrix_node2d + potrf_matrix
 *   densematrix_edge2d (A and M) + sygv_matrix: the coarse eigenproblem,
 *     zero eigenvalues skipped, the lowest m eigenvectors as the start block
 *   per level: prolongation_edge2d, then block steps of
 *     pinvit_edge2d (defect, V-cycles, update, gradient lifting)
 *     energyprod/massprod of all pairs (gram_edge2d) + sygv_matrix
 *     e_j = sum_i C_ij u_i (lincomb_edge2d), defects by addeval + norm2
 *   until the largest absolute defect of the wanted vectors is below tol.
 *
 * Usage: c_driver_pinvit n0 L ieigs m tol max_steps eps r kx ky [kx ky ...]
 * (a disc of permittivity eps and radius r in the centre of the unit cell,
 * eps = 1 around it).  Prints one line per k-point: its block steps and the
 * ieigs eigenvalues lambda = mu - 1.  Exit status 2 on a failed call. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "maxwell_gb300.h"

#define CHECK(x)                                                           \
  do {                                                                     \
    int e_ = (x);                                                          \
    if(e_) {                                                               \
      fprintf(stderr, "%s:%d: %s returned %d\n", __FILE__, __LINE__, #x, e_); \
      exit(2);                                                             \
    }                                                                      \
  } while(0)
#define MAXL 12

static double *re_im(mxg_field *z) { return (double *) z; }

int main(int argc, char **argv)
{
  int n0, L, ieigs, m, max_steps, K, k, l, v, N, nn;
  double tol, eps, r;
  mxg_field *xf, *yf, *host, *ga, *gm, *coef;
  double *lam0, *mu, *defect, *ones;
  int *info;
  grid2d_gpu *gr[MAXL];
  edge2d_gpu *e[MAXL], *u[MAXL], *t[MAXL], *b[MAXL], *x[MAXL], *d[MAXL];
  node2d_gpu *bg[MAXL], *xg[MAXL], *dg[MAXL];
  matrix_gpu *Ae, *An, *A0, *M0, *Ar, *Mr;
  mxg_epspattern *pat;
  int *steps;

  if(argc < 11 || (argc - 9) % 2) {
    fprintf(stderr, "usage: %s n0 L ieigs m tol max_steps eps r kx ky [kx ky ...]\n", argv[0]);
    return 1;
  }
  n0 = atoi(argv[1]); L = atoi(argv[2]); ieigs = atoi(argv[3]); m = atoi(argv[4]);
  tol = atof(argv[5]); max_steps = atoi(argv[6]); eps = atof(argv[7]); r = atof(argv[8]);
  K = (argc - 9) / 2;
  if(L < 1 || L >= MAXL || ieigs > m) return 1;
  CHECK(!mxg_device_ok());
  xf = malloc(sizeof(mxg_field) * K);
  yf = malloc(sizeof(mxg_field) * K);
  for(k = 0; k < K; k++) {
    double kx = atof(argv[9 + 2 * k]), ky = atof(argv[10 + 2 * k]);
    xf[k] = cos(kx) + I * sin(kx);
    yf[k] = cos(ky) + I * sin(ky);
  }

  /* grids: the pattern on the finest level, kappa averaged down
   * (exp_bloch2d.c:335-458), the Bloch factors of every k-point */
  nn = n0 << L;
  gr[L] = new_grid2d_gpu(nn, nn, 1.0 / nn, 1.0 / nn, K);
  CHECK(!gr[L]);
  pat = new_epspattern_gpu(1.0, 0, 1);
  pat->circle[0] = eps; pat->circle[1] = 0.5; pat->circle[2] = 0.5; pat->circle[3] = r;
  CHECK(setpattern_grid2d_gpu(pat, gr[L]));
  del_epspattern_gpu(pat);
  for(l = L; l-- > 0;) {
    gr[l] = coarsen_grid2d_gpu(gr[l + 1]);
    CHECK(!gr[l]);
  }
  for(l = 0; l <= L; l++) {
    CHECK(setbloch_grid2d_gpu(gr[l], xf, yf));
    e[l] = new_edge2d_gpu(gr[l], m, MXG_C128); u[l] = new_edge2d_gpu(gr[l], m, MXG_C128);
    t[l] = new_edge2d_gpu(gr[l], m, MXG_C128);
    b[l] = new_edge2d_gpu(gr[l], m, MXG_C128); x[l] = new_edge2d_gpu(gr[l], m, MXG_C128);
    d[l] = new_edge2d_gpu(gr[l], m, MXG_C128);
    bg[l] = new_node2d_gpu(gr[l], m, MXG_C128); xg[l] = new_node2d_gpu(gr[l], m, MXG_C128);
    dg[l] = new_node2d_gpu(gr[l], m, MXG_C128);
    CHECK(!e[l] || !u[l] || !t[l] || !b[l] || !x[l] || !d[l] || !bg[l] || !xg[l] || !dg[l]);
  }
  info = malloc(sizeof(int) * K);

  /* coarse solvers (exp_bloch2d.c:520-528) */
  N = 2 * n0 * n0;
  Ae = new_matrix_gpu(N, K);
  An = new_matrix_gpu(n0 * n0, K);
  CHECK(densematrix_edge2d_gpu(1.0, 1.0, gr[0], Ae));
  CHECK(potrf_matrix_gpu(Ae, info));
  for(k = 0; k < K; k++) CHECK(info[k]);
  CHECK(densematrix_node2d_gpu(1, gr[0], An));
  CHECK(potrf_matrix_gpu(An, info));
  for(k = 0; k < K; k++) CHECK(info[k]);

  /* coarse generalized eigenproblem, zero eigenvalues skipped
   * (exp_bloch2d.c:530-554) */
  A0 = new_matrix_gpu(N, K);
  M0 = new_matrix_gpu(N, K);
  lam0 = malloc(sizeof(double) * N * K);
  host = malloc(sizeof(mxg_field) * (size_t) N * N * K);
  CHECK(densematrix_edge2d_gpu(1.0, 0.0, gr[0], A0));
  CHECK(densematrix_edge2d_gpu(0.0, 1.0, gr[0], M0));
  CHECK(sygv_matrix_gpu(A0, M0, lam0, info));
  for(k = 0; k < K; k++) CHECK(info[k]);
  CHECK(download_matrix_gpu(A0, host));
  {
    mxg_field *start = malloc(sizeof(mxg_field) * (size_t) K * m * N);
    for(k = 0; k < K; k++) {
      int ev = 0;
      while(ev < N && fabs(lam0[k * N + ev]) < 1e-8) ev++;
      CHECK(ev + m > N);
      for(v = 0; v < m; v++)
        memcpy(start + ((size_t) k * m + v) * N, host + (size_t) k * N * N + (size_t) (ev + v) * N,
               sizeof(mxg_field) * N);
    }
    CHECK(denseto_edge2d_gpu(start, e[0]));
    free(start);
  }

  /* nested iteration, then the finest level (exp_bloch2d.c:562-732, 956-1018) */
  Ar = new_matrix_gpu(m, K);
  Mr = new_matrix_gpu(m, K);
  ga = malloc(sizeof(mxg_field) * m * m * K);
  gm = malloc(sizeof(mxg_field) * m * m * K);
  coef = malloc(sizeof(mxg_field) * m * m * K);
  mu = malloc(sizeof(double) * m * K);
  defect = malloc(sizeof(double) * m * K);
  ones = malloc(sizeof(double) * m * K);
  steps = calloc(K, sizeof(int));
  for(l = 1; l <= L; l++) {
    int step, limit = l < L ? 40 : max_steps;
    double worst = 1e300;
    CHECK(zero_edge2d_gpu(e[l]));
    CHECK(prolongation_edge2d_gpu(1.0, e[l - 1], e[l]));
    for(step = 0; step <= limit; step++) {
      /* Rayleigh quotients and defects of the current block */
      CHECK(gram_edge2d_gpu(e[l], ga, gm));
      for(k = 0; k < K; k++)
        for(v = 0; v < m; v++) {
          size_t q = (size_t) k * m * m + (size_t) v * m + v;
          mu[k * m + v] = re_im(ga + q)[0] / re_im(gm + q)[0];
          ones[k * m + v] = 1.0 - mu[k * m + v];
        }
      CHECK(zero_edge2d_gpu(t[l]));
      CHECK(addeval_shifted_edge2d_gpu(1.0, ones, e[l], t[l]));
      CHECK(norm2_edge2d_gpu(t[l], defect));
      worst = 0.0;
      for(k = 0; k < K; k++)
        for(v = 0; v < ieigs; v++)
          if(defect[k * m + v] > worst) worst = defect[k * m + v];
      if(worst <= tol || step == limit) break;
      /* one block PINVIT step with gradient lifting for every vector */
      CHECK(pinvit_edge2d_gpu(l, 2, 2, 5, mu, e[l], Ae, b, x, d, An, bg, xg, dg));
      /* Ritz step: Gram matrices, generalized eigenproblem, combination */
      CHECK(gram_edge2d_gpu(e[l], ga, gm));
      CHECK(upload_matrix_gpu(Ar, ga));
      CHECK(upload_matrix_gpu(Mr, gm));
      CHECK(sygv_matrix_gpu(Ar, Mr, mu, info));
      for(k = 0; k < K; k++) CHECK(info[k]);
      CHECK(download_matrix_gpu(Ar, coef));
      CHECK(lincomb_edge2d_gpu(coef, e[l], u[l]));
      CHECK(swap_edge2d_gpu(e[l], u[l]));
      if(l == L)
        for(k = 0; k < K; k++) steps[k] = step + 1;
    }
    if(l == L && worst > tol) {
      fprintf(stderr, "not converged: largest defect %.3e after %d steps\n", worst, max_steps);
      return 3;
    }
  }
  for(k = 0; k < K; k++) {
    printf("%d", steps[k]);
    for(v = 0; v < ieigs; v++) printf(" %.17g", mu[k * m + v] - 1.0);
    printf("\n");
  }
  return 0;
}
