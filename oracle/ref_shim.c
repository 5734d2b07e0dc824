/* Flat-array entry points over the UNMODIFIED reference modules
 * (grid2d.c, edge2d.c, node2d.c, linalg.c, basic.c, settings.c of
 * sboerm/Maxwell), compiled from their original location by
 * oracle/Makefile into oracle/_ref/libmaxwell_ref.so.
 *
 * This file is test infrastructure: it is only used in this container to
 * generate the golden vectors under tests/golden/ (tests/golden/gen_golden.py)
 * and to pin the C restatement in oracle/maxwell_oracle.c.
 *
 * Layout of every array passed in or out (the reference's own dense order,
 * densefrom_edge2d / densefrom_node2d, edge2d.c:6137-6152, node2d.c:1619-1630):
 *   edge vector: 2*n*n complex doubles, x-edge (i,j) at i+j*n,
 *                y-edge (i,j) at n*n + i+j*n;
 *   node vector: n*n complex doubles, node (i,j) at i+j*n;
 *   kappa:       n*n doubles, reciprocal permittivity of cell (i,j) at i+j*n.
 */
#include "settings.h"
#include "grid2d.h"
#include "edge2d.h"
#include "node2d.h"
#include "linalg.h"
#include "basic.h"

#include <assert.h>
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

static grid2d *
mkgrid(int n, const double *kappa, field xf, field yf)
{
  grid2d *gr = new_grid2d(n, n, 1.0 / n, 1.0 / n);
  int i;
  if(kappa)
    for(i = 0; i < n * n; i++)
      gr->eps[i] = kappa[i];
  gr->xfactor = xf;
  gr->yfactor = yf;
  return gr;
}

static edge2d *
mkedge(const grid2d *gr, const field *v)
{
  edge2d *e = new_edge2d(gr);
  zero_edge2d(e);
  if(v)
    denseto_edge2d(v, e);
  return e;
}

static node2d *
mknode(const grid2d *gr, const field *v)
{
  node2d *x = new_node2d(gr);
  zero_node2d(x);
  if(v)
    denseto_node2d(v, x);
  return x;
}

void
ref_addeval_edge2d(int n, const double *kappa, field xf, field yf,
                   field alpha, field beta, const field *x, field *y)
{
  grid2d *gr = mkgrid(n, kappa, xf, yf);
  edge2d *ex = mkedge(gr, x), *ey = mkedge(gr, y);
  addeval_edge2d(alpha, beta, ex, ey);
  densefrom_edge2d(ey, y);
  del_edge2d(ex); del_edge2d(ey); del_grid2d(gr);
}

void
ref_products_edge2d(int n, const double *kappa, field xf, field yf,
                    field alpha, field beta, const field *x, const field *y,
                    field *out /* [energyprod, massprod, dotprod] */)
{
  grid2d *gr = mkgrid(n, kappa, xf, yf);
  edge2d *ex = mkedge(gr, x), *ey = mkedge(gr, y);
  out[0] = energyprod_edge2d(alpha, beta, ex, ey);
  out[1] = massprod_edge2d(ex, ey);
  out[2] = dotprod_edge2d(ex, ey);
  del_edge2d(ex); del_edge2d(ey); del_grid2d(gr);
}

/* dir: 0 forward, 1 backward, 2 symmetric */
void
ref_gs_edge2d(int n, const double *kappa, field xf, field yf,
              field alpha, field beta, int dir, const field *b, field *x)
{
  grid2d *gr = mkgrid(n, kappa, xf, yf);
  edge2d *eb = mkedge(gr, b), *ex = mkedge(gr, x);
  if(dir == 0)
    gsforward_edge2d(alpha, beta, eb, ex);
  else if(dir == 1)
    gsbackward_edge2d(alpha, beta, eb, ex);
  else
    gssymm_edge2d(alpha, beta, eb, ex);
  densefrom_edge2d(ex, x);
  del_edge2d(eb); del_edge2d(ex); del_grid2d(gr);
}

/* the point smoother of the Hiptmair cycle: dir 0 forward, 1 backward, 2 symmetric */
void
ref_gs_simple_edge2d(int n, const double *kappa, field xf, field yf,
                     field alpha, field beta, int dir, const field *b, field *x)
{
  grid2d *gr = mkgrid(n, kappa, xf, yf);
  edge2d *eb = mkedge(gr, b), *ex = mkedge(gr, x);
  if(dir == 0)
    gsforward_simple_edge2d(alpha, beta, eb, ex);
  else if(dir == 1)
    gsbackward_simple_edge2d(alpha, beta, eb, ex);
  else
    gssymm_simple_edge2d(alpha, beta, eb, ex);
  densefrom_edge2d(ex, x);
  del_edge2d(eb); del_edge2d(ex); del_grid2d(gr);
}

/* nc: coarse intervals; the fine grid has 2*nc */
void
ref_transfer_edge2d(int nc, field xf, field yf, field alpha, int restrict_,
                    const field *in, field *out)
{
  grid2d *gc = mkgrid(nc, 0, xf, yf), *gf = mkgrid(2 * nc, 0, xf, yf);
  if(restrict_) {
    edge2d *f = mkedge(gf, in), *c = mkedge(gc, out);
    restriction_edge2d(alpha, f, c);
    densefrom_edge2d(c, out);
    del_edge2d(f); del_edge2d(c);
  }
  else {
    edge2d *c = mkedge(gc, in), *f = mkedge(gf, out);
    prolongation_edge2d(alpha, c, f);
    densefrom_edge2d(f, out);
    del_edge2d(f); del_edge2d(c);
  }
  del_grid2d(gc); del_grid2d(gf);
}

void
ref_addeval_node2d(int n, field xf, field yf, field alpha,
                   const field *x, field *y)
{
  grid2d *gr = mkgrid(n, 0, xf, yf);
  node2d *nx_ = mknode(gr, x), *ny_ = mknode(gr, y);
  addeval_node2d(alpha, nx_, ny_);
  densefrom_node2d(ny_, y);
  del_node2d(nx_); del_node2d(ny_); del_grid2d(gr);
}

void
ref_gs_node2d(int n, field xf, field yf, field alpha, int dir,
              const field *b, field *x)
{
  grid2d *gr = mkgrid(n, 0, xf, yf);
  node2d *nb = mknode(gr, b), *nx_ = mknode(gr, x);
  if(dir == 0)
    gsforward_node2d(alpha, nb, nx_);
  else if(dir == 1)
    gsbackward_node2d(alpha, nb, nx_);
  else
    gssymm_node2d(alpha, nb, nx_);
  densefrom_node2d(nx_, x);
  del_node2d(nb); del_node2d(nx_); del_grid2d(gr);
}

void
ref_transfer_node2d(int nc, field xf, field yf, field alpha, int restrict_,
                    const field *in, field *out)
{
  grid2d *gc = mkgrid(nc, 0, xf, yf), *gf = mkgrid(2 * nc, 0, xf, yf);
  if(restrict_) {
    node2d *f = mknode(gf, in), *c = mknode(gc, out);
    restriction_node2d(alpha, f, c);
    densefrom_node2d(c, out);
    del_node2d(f); del_node2d(c);
  }
  else {
    node2d *c = mknode(gc, in), *f = mknode(gf, out);
    prolongation_node2d(alpha, c, f);
    densefrom_node2d(f, out);
    del_node2d(f); del_node2d(c);
  }
  del_grid2d(gc); del_grid2d(gf);
}

/* adjoint_: 0 gradient (node -> edge), 1 adjoint gradient (edge -> node) */
void
ref_gradient_node2d(int n, field xf, field yf, field alpha, int adjoint_,
                    const field *in, field *out)
{
  grid2d *gr = mkgrid(n, 0, xf, yf);
  if(adjoint_) {
    edge2d *e = mkedge(gr, in);
    node2d *v = mknode(gr, out);
    adjgradient_node2d(alpha, e, v);
    densefrom_node2d(v, out);
    del_edge2d(e); del_node2d(v);
  }
  else {
    node2d *v = mknode(gr, in);
    edge2d *e = mkedge(gr, out);
    gradient_node2d(alpha, v, e);
    densefrom_edge2d(e, out);
    del_edge2d(e); del_node2d(v);
  }
  del_grid2d(gr);
}

void
ref_center_edge2d(int n, field *x)
{
  grid2d *gr = mkgrid(n, 0, 1.0, 1.0);
  edge2d *e = mkedge(gr, x);
  center_edge2d(e);
  densefrom_edge2d(e, x);
  del_edge2d(e); del_grid2d(gr);
}

void
ref_densematrix_edge2d(int n, const double *kappa, field xf, field yf,
                       field alpha, field beta, field *a)
{
  grid2d *gr = mkgrid(n, kappa, xf, yf);
  matrix *m = new_matrix(2 * n * n, 2 * n * n);
  densematrix_edge2d(alpha, beta, gr, m);
  memcpy(a, m->a, sizeof(field) * 4 * n * n * n * n);
  del_matrix(m); del_grid2d(gr);
}

void
ref_densematrix_node2d(int n, field xf, field yf, int fixnull, field *a)
{
  grid2d *gr = mkgrid(n, 0, xf, yf);
  matrix *m = new_matrix(n * n, n * n);
  densematrix_node2d(fixnull != 0, gr, m);
  memcpy(a, m->a, sizeof(field) * n * n * n * n);
  del_matrix(m); del_grid2d(gr);
}

/* ------------------------------------------------------------
 * Multigrid hierarchy helpers
 * ------------------------------------------------------------ */

typedef struct {
  int L;
  grid2d **gr;
  edge2d **b, **x, **d;
  node2d **bg, **xg, **dg;
  matrix *Ae, *An;
} hier;

static hier *
mkhier(int n0, int L, const double *kappa_fine, field xf, field yf,
       int coarse_edge, int coarse_node)
{
  hier *h = calloc(1, sizeof(hier));
  int l;
  h->L = L;
  h->gr = malloc(sizeof(grid2d *) * (L + 1));
  h->b = malloc(sizeof(edge2d *) * (L + 1));
  h->x = malloc(sizeof(edge2d *) * (L + 1));
  h->d = malloc(sizeof(edge2d *) * (L + 1));
  h->bg = malloc(sizeof(node2d *) * (L + 1));
  h->xg = malloc(sizeof(node2d *) * (L + 1));
  h->dg = malloc(sizeof(node2d *) * (L + 1));
  h->gr[L] = mkgrid(n0 << L, kappa_fine, xf, yf);
  for(l = L; l-- > 0;)
    h->gr[l] = coarsen_grid2d(h->gr[l + 1]);
  for(l = 0; l <= L; l++) {
    h->b[l] = mkedge(h->gr[l], 0);
    h->x[l] = mkedge(h->gr[l], 0);
    h->d[l] = mkedge(h->gr[l], 0);
    h->bg[l] = mknode(h->gr[l], 0);
    h->xg[l] = mknode(h->gr[l], 0);
    h->dg[l] = mknode(h->gr[l], 0);
  }
  if(coarse_edge) {
    h->Ae = new_matrix(2 * n0 * n0, 2 * n0 * n0);
    densematrix_edge2d(1.0, 1.0, h->gr[0], h->Ae);
    potrf_matrix(h->Ae);
  }
  if(coarse_node) {
    h->An = new_matrix(n0 * n0, n0 * n0);
    densematrix_node2d(true, h->gr[0], h->An);
    potrf_matrix(h->An);
  }
  return h;
}

static void
delhier(hier *h)
{
  int l;
  for(l = 0; l <= h->L; l++) {
    del_edge2d(h->b[l]); del_edge2d(h->x[l]); del_edge2d(h->d[l]);
    del_node2d(h->bg[l]); del_node2d(h->xg[l]); del_node2d(h->dg[l]);
  }
  for(l = 0; l <= h->L; l++)
    del_grid2d(h->gr[l]);
  if(h->Ae) del_matrix(h->Ae);
  if(h->An) del_matrix(h->An);
  free(h->gr); free(h->b); free(h->x); free(h->d);
  free(h->bg); free(h->xg); free(h->dg);
  free(h);
}

/* Coarse kappa of every level, finest first in the output (n_l^2 each). */
void
ref_coarsen_kappa(int n0, int L, const double *kappa_fine, double *out)
{
  hier *h = mkhier(n0, L, kappa_fine, 1.0, 1.0, 0, 0);
  int l;
  size_t off = 0;
  for(l = L; l >= 0; l--) {
    int n = h->gr[l]->nx;
    memcpy(out + off, h->gr[l]->eps, sizeof(double) * n * n);
    off += (size_t) n * n;
  }
  delhier(h);
}

/* `cycles` V-cycles of vcycle_edge2d on the finest level, x updated in place. */
void
ref_vcycle_edge2d(int n0, int L, const double *kappa_fine, field xf, field yf,
                  int nu, int coarse, int cycles, const field *b, field *x)
{
  hier *h = mkhier(n0, L, kappa_fine, xf, yf, coarse, 0);
  int c;
  denseto_edge2d(b, h->b[L]);
  denseto_edge2d(x, h->x[L]);
  for(c = 0; c < cycles; c++)
    vcycle_edge2d(L, nu, coarse ? h->Ae : 0, h->b, h->x, h->d);
  densefrom_edge2d(h->x[L], x);
  delhier(h);
}

/* `cycles` Hiptmair cycles (hcycle_edge2d) on the finest level */
void
ref_hcycle_edge2d(int n0, int L, const double *kappa_fine, field xf, field yf,
                  int nu, int coarse, int cycles, const field *b, field *x)
{
  hier *h = mkhier(n0, L, kappa_fine, xf, yf, coarse, 0);
  int c;
  denseto_edge2d(b, h->b[L]);
  denseto_edge2d(x, h->x[L]);
  for(c = 0; c < cycles; c++)
    hcycle_edge2d(L, nu, coarse ? h->Ae : 0, h->b, h->x, h->d, h->bg, h->xg);
  densefrom_edge2d(h->x[L], x);
  delhier(h);
}

void
ref_vcycle_node2d(int n0, int L, field xf, field yf,
                  int nu, int coarse, int cycles, const field *b, field *x)
{
  hier *h = mkhier(n0, L, 0, xf, yf, 0, coarse);
  int c;
  denseto_node2d(b, h->bg[L]);
  denseto_node2d(x, h->xg[L]);
  for(c = 0; c < cycles; c++)
    vcycle_node2d(L, nu, coarse ? h->An : 0, h->bg, h->xg, h->dg);
  densefrom_node2d(h->xg[L], x);
  delhier(h);
}

/* One pinvit_edge2d call (edge2d.c:6298-6328) on the finest level. */
void
ref_pinvit_edge2d(int n0, int L, const double *kappa_fine, field xf, field yf,
                  int smoother_steps, int prec_steps, int gradient_steps,
                  double lambda, field *e)
{
  hier *h = mkhier(n0, L, kappa_fine, xf, yf, 1, 1);
  edge2d *ev = mkedge(h->gr[L], e);
  pinvit_edge2d(L, smoother_steps, prec_steps, gradient_steps, lambda, ev,
                h->Ae, h->b, h->x, h->d, h->An, h->bg, h->xg, h->dg);
  densefrom_edge2d(ev, e);
  del_edge2d(ev);
  delhier(h);
}

/* ------------------------------------------------------------
 * The exp_bloch2d per-k flow (exp_bloch2d.c:520-1053) over an explicit
 * list of Bloch factors instead of blochcurve(): coarse generalized
 * eigenproblem, nested iteration on k[0], then for k[1..nk-1]
 * refactorisation of the coarse solvers, extrapolation warm start
 * ('n', '1' or '2'), and block PINVIT + Ritz until the largest absolute
 * defect of the first ieigs vectors is <= tol or bloch_steps is reached.
 * With center != 0 the constant fields are removed at k = 0 as in
 * test_block2d.c:219-221, so that only non-zero eigenvalues remain.
 * Outputs mu-1 (the eigenvalues lambda) per k and vector, the number of
 * block steps per k, and the final absolute defects.
 * ------------------------------------------------------------ */

static void
setfactors(hier *h, field xf, field yf)
{
  int l;
  for(l = 0; l <= h->L; l++) {
    h->gr[l]->xfactor = xf;
    h->gr[l]->yfactor = yf;
  }
}

static bool
is_gamma(const grid2d *gr)
{
  return gr->xfactor == 1.0 && gr->yfactor == 1.0;
}

static void
pinvit_block(hier *h, int l, int eigs, edge2d **e, edge2d **u, real *lambda,
             matrix *Ar, matrix *Mr, int prec_steps, int gradient_steps,
             int center, real *norm)
{
  int i, j, info = 0;
  edge2d *aux;

  for(i = 0; i < eigs; i++) {
    zero_edge2d(h->b[l]);
    addeval_edge2d(1.0, 1.0 - lambda[i], e[i], h->b[l]);
    zero_edge2d(h->x[l]);
    for(j = 0; j < prec_steps; j++)
      vcycle_edge2d(l, 2, h->Ae, h->b, h->x, h->d);
    add_edge2d(-1.0, h->x[l], e[i]);
    if(center && is_gamma(h->gr[l]))
      center_edge2d(e[i]);
    zero_edge2d(h->d[l]);
    addeval_edge2d(0.0, 1.0, e[i], h->d[l]);
    zero_node2d(h->bg[l]);
    adjgradient_node2d(1.0, h->d[l], h->bg[l]);
    zero_node2d(h->xg[l]);
    for(j = 0; j < gradient_steps; j++)
      vcycle_node2d(l, 2, h->An, h->bg, h->xg, h->dg);
    gradient_node2d(-1.0, h->xg[l], e[i]);
  }
#pragma omp barrier
#pragma omp single
  for(i = 0; i < eigs; i++) {
    aux = u[i]; u[i] = e[i]; e[i] = aux;
  }
  for(j = 0; j < eigs; j++)
    for(i = j; i < eigs; i++) {
      Ar->a[i + Ar->ld * j] = energyprod_edge2d(1.0, 1.0, u[i], u[j]);
      Mr->a[i + Mr->ld * j] = massprod_edge2d(u[i], u[j]);
    }
#pragma omp single
  {
    info = sygv_matrix(Ar, Mr, lambda);
    assert(info == 0);
  }
  (void) info;
  for(j = 0; j < eigs; j++) {
    zero_edge2d(e[j]);
    for(i = 0; i < eigs; i++)
      add_edge2d(Ar->a[i + Ar->ld * j], u[i], e[j]);
  }
  for(i = 0; i < eigs; i++) {
    zero_edge2d(h->d[l]);
    addeval_edge2d(1.0, 1.0 - lambda[i], e[i], h->d[l]);
    norm[i] = norm2_edge2d(h->d[l]);
  }
}

static real
maxof(const real *v, int k)
{
  real m = v[0];
  int i;
  for(i = 1; i < k; i++)
    if(v[i] > m)
      m = v[i];
  return m;
}

static void
rayleigh_defects(hier *h, int l, int eigs, edge2d **e, real *lambda, real *norm)
{
  int i;
  field p1, p2;
  for(i = 0; i < eigs; i++) {
    zero_edge2d(h->b[l]);
    addeval_edge2d(1.0, 1.0, e[i], h->b[l]);
    zero_edge2d(h->d[l]);
    addeval_edge2d(0.0, 1.0, e[i], h->d[l]);
    p1 = dotprod_edge2d(e[i], h->b[l]);
    p2 = dotprod_edge2d(e[i], h->d[l]);
    lambda[i] = REAL(p1 / p2);
    add_edge2d(-lambda[i], h->d[l], h->b[l]);
    norm[i] = norm2_edge2d(h->b[l]);
  }
}

int
ref_bloch_solve(int n0, int L, const double *kappa_fine, int nk,
                const field *xfs, const field *yfs, int ieigs, int throwaway,
                int pinvit_steps, int bloch_steps, double tol,
                int extrapolation, int prec_steps, int gradient_steps,
                int center, int nthreads,
                double *lambda_out, int *steps_out, double *defect_out,
                field *evec_out /* optional: 2*(n0<<L)^2 * eigs for the last k */)
{
  int eigs = ieigs + throwaway;
  hier *h = mkhier(n0, L, kappa_fine, xfs[0], yfs[0], 1, 1);
  edge2d ***e, ***u, **eold[2];
  matrix *A, *M, *Ar, *Mr, *Ar2, *Ar3;
  real **lambda, *lambda2, *lambda3, *norm;
  field *tau2, *tau3;
  int i, l, ev, kk;
  int n = n0;
  int status = 0;

  e = malloc(sizeof(edge2d **) * (L + 1));
  u = malloc(sizeof(edge2d **) * (L + 1));
  lambda = malloc(sizeof(real *) * (L + 1));
  for(l = 0; l <= L; l++) {
    e[l] = malloc(sizeof(edge2d *) * eigs);
    u[l] = malloc(sizeof(edge2d *) * 3 * eigs);
    for(i = 0; i < eigs; i++)
      e[l][i] = mkedge(h->gr[l], 0);
    for(i = 0; i < 3 * eigs; i++)
      u[l][i] = mkedge(h->gr[l], 0);
    lambda[l] = malloc(sizeof(real) * (l == 0 ? 2 * n * n : 3 * eigs));
  }
  for(kk = 0; kk < 2; kk++) {
    eold[kk] = malloc(sizeof(edge2d *) * eigs);
    for(i = 0; i < eigs; i++)
      eold[kk][i] = mkedge(h->gr[L], 0);
  }
  norm = malloc(sizeof(real) * eigs);
  Ar = new_matrix(eigs, eigs);
  Mr = new_matrix(eigs, eigs);
  Ar2 = new_matrix(2 * ieigs, 2 * ieigs);
  Ar3 = new_matrix(3 * ieigs, 3 * ieigs);
  tau2 = malloc(sizeof(field) * 2 * ieigs);
  tau3 = malloc(sizeof(field) * 3 * ieigs);
  lambda2 = malloc(sizeof(real) * 2 * ieigs);
  lambda3 = malloc(sizeof(real) * 3 * ieigs);

  /* Coarse generalized eigenproblem (exp_bloch2d.c:530-554) */
  A = new_matrix(2 * n * n, 2 * n * n);
  M = new_matrix(2 * n * n, 2 * n * n);
  densematrix_edge2d(1.0, 0.0, h->gr[0], A);
  densematrix_edge2d(0.0, 1.0, h->gr[0], M);
  sygv_matrix(A, M, lambda[0]);
  for(i = 0; i < A->rows && fabs(lambda[0][i]) < 1e-8; i++)
    ;
  ev = i;
  if(ev + eigs > A->rows) {
    status = -1;
    goto done;
  }
  for(i = 0; i < eigs; i++)
    denseto_edge2d(A->a + (ev + i) * A->ld, e[0][i]);

  if(nthreads > 0)
    omp_set_num_threads(nthreads);

#pragma omp parallel private(i, l, kk)
  {
    real maxnorm_l;
    int k;

    /* Nested iteration (exp_bloch2d.c:562-732) */
    for(l = 1; l <= L; l++) {
      for(i = 0; i < eigs; i++) {
        zero_edge2d(e[l][i]);
        prolongation_edge2d(1.0, e[l - 1][i], e[l][i]);
      }
      rayleigh_defects(h, l, eigs, e[l], lambda[l], norm);
      maxnorm_l = maxof(norm, ieigs);
      for(k = 0; k < pinvit_steps && maxnorm_l > tol; k++) {
        pinvit_block(h, l, eigs, e[l], u[l], lambda[l], Ar, Mr,
                     prec_steps, gradient_steps, center, norm);
        maxnorm_l = maxof(norm, ieigs);
      }
#pragma omp single
      if(l == L) {
        for(i = 0; i < eigs; i++) {
          lambda_out[i] = lambda[L][i] - 1.0;
          defect_out[i] = norm[i];
        }
        steps_out[0] = k;
      }
    }

    for(i = 0; i < eigs; i++) {
      zero_edge2d(eold[0][i]);
      zero_edge2d(eold[1][i]);
    }

    /* Bloch scan (exp_bloch2d.c:781-1053) */
    for(kk = 1; kk < nk; kk++) {
      int info;
#pragma omp single
      {
        setfactors(h, xfs[kk], yfs[kk]);
        densematrix_edge2d(1.0, 1.0, h->gr[0], h->Ae);
        potrf_matrix(h->Ae);
        densematrix_node2d(true, h->gr[0], h->An);
        potrf_matrix(h->An);
      }
      if(extrapolation == 'n') {
        for(i = 0; i < eigs; i++) {
          copy_edge2d(eold[0][i], eold[1][i]);
          copy_edge2d(e[L][i], eold[0][i]);
        }
      }
      else if(extrapolation == '1') {
        int j;
        for(i = 0; i < ieigs; i++) {
          copy_edge2d(e[L][i], u[L][i]);
          copy_edge2d(eold[0][i], u[L][i + ieigs]);
        }
        orthonormalize_edge2d(2 * ieigs, u[L], tau2, h->d[L]);
        for(j = 0; j < 2 * ieigs; j++)
          for(i = j; i < 2 * ieigs; i++)
            Ar2->a[i + Ar2->ld * j] = energyprod_edge2d(1.0, 1.0, u[L][i], u[L][j]);
#pragma omp single
        {
          info = syev_matrix(Ar2, lambda2);
          assert(info == 0);
        }
        for(j = 0; j < eigs; j++) {
          copy_edge2d(eold[0][j], eold[1][j]);
          copy_edge2d(e[L][j], eold[0][j]);
          zero_edge2d(e[L][j]);
          for(i = 0; i < 2 * ieigs; i++)
            add_edge2d(Ar2->a[i + Ar2->ld * j], u[L][i], e[L][j]);
        }
      }
      else {
        int j;
        for(i = 0; i < ieigs; i++) {
          copy_edge2d(e[L][i], u[L][i]);
          copy_edge2d(eold[0][i], u[L][i + ieigs]);
          copy_edge2d(eold[1][i], u[L][i + 2 * ieigs]);
        }
        orthonormalize_edge2d(3 * ieigs, u[L], tau3, h->d[L]);
        for(j = 0; j < 3 * ieigs; j++)
          for(i = j; i < 3 * ieigs; i++)
            Ar3->a[i + Ar3->ld * j] = energyprod_edge2d(1.0, 1.0, u[L][i], u[L][j]);
#pragma omp single
        {
          info = syev_matrix(Ar3, lambda3);
          assert(info == 0);
        }
        for(j = 0; j < eigs; j++) {
          copy_edge2d(eold[0][j], eold[1][j]);
          copy_edge2d(e[L][j], eold[0][j]);
          zero_edge2d(e[L][j]);
          for(i = 0; i < 3 * ieigs; i++)
            add_edge2d(Ar3->a[i + Ar3->ld * j], u[L][i], e[L][j]);
        }
      }
      (void) info;
      rayleigh_defects(h, L, eigs, e[L], lambda[L], norm);
      maxnorm_l = maxof(norm, ieigs);
      for(k = 0; k < bloch_steps && maxnorm_l > tol; k++) {
        pinvit_block(h, L, eigs, e[L], u[L], lambda[L], Ar, Mr,
                     prec_steps, gradient_steps, center, norm);
        maxnorm_l = maxof(norm, ieigs);
      }
#pragma omp single
      {
        for(i = 0; i < eigs; i++) {
          lambda_out[kk * eigs + i] = lambda[L][i] - 1.0;
          defect_out[kk * eigs + i] = norm[i];
        }
        steps_out[kk] = k;
      }
    }
  }

  if(evec_out)
    for(i = 0; i < eigs; i++)
      densefrom_edge2d(e[L][i], evec_out + (size_t) i * 2 * (n0 << L) * (n0 << L));

done:
  for(l = 0; l <= L; l++) {
    for(i = 0; i < eigs; i++)
      del_edge2d(e[l][i]);
    for(i = 0; i < 3 * eigs; i++)
      del_edge2d(u[l][i]);
    free(e[l]); free(u[l]); free(lambda[l]);
  }
  for(kk = 0; kk < 2; kk++) {
    for(i = 0; i < eigs; i++)
      del_edge2d(eold[kk][i]);
    free(eold[kk]);
  }
  free(e); free(u); free(lambda); free(norm);
  del_matrix(A); del_matrix(M); del_matrix(Ar); del_matrix(Mr);
  del_matrix(Ar2); del_matrix(Ar3);
  free(tau2); free(tau3); free(lambda2); free(lambda3);
  delhier(h);
  return status;
}
