/* Host side of libmaxwell_gb300: the reference-shaped C ABI
 * (include/maxwell_gb300.h) over device-resident batched objects, and the
 * per-k eigensolver flow of exp_bloch2d (exp_bloch2d.c:520-1053) run for a
 * whole batch of k-points at once.  All arithmetic happens in the CUDA
 * kernels behind mx_internal.h; this file moves data, sequences launches and
 * makes the small control decisions (convergence, soft locking). */
#include "maxwell_gb300.h"
#include "mx_internal.h"

#include <cuda_runtime_api.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define TRY(x) do { int e_ = (x); if (e_) return e_; } while (0)

static double creal_(mxg_field z) { return creal(z); }
static double cimag_(mxg_field z) { return cimag(z); }

/* ------------------------------------------------------------------ */
/* objects                                                             */
/* ------------------------------------------------------------------ */

struct grid2d_gpu {
  int n, K;
  double h;
  double *kd;          /* device kappa, double */
  float *kf;           /* float */
  float *kdd;          /* float-float pairs */
  void *afw;           /* AFW patch factors for alpha = beta = 1 */
  double *ph;          /* device phase table (mxk_phase_bytes) */
  double *h_kappa;     /* host copies */
  double *h_ph;
  cudaStream_t st;
};

struct edge2d_gpu {
  const grid2d_gpu *gr;
  int m, prec;
  void *d;
};

struct node2d_gpu {
  const grid2d_gpu *gr;
  int m, prec;
  void *d;
};

struct matrix_gpu {
  int rows, K;
  double *d;           /* K * rows * rows complex */
  int *info;           /* device */
  int factored;
};

static mxk_kappa kap_of(const grid2d_gpu *g)
{
  mxk_kappa k;
  k.f = g->kf;
  k.d = g->kd;
  k.dd = g->kdd;
  k.afw = g->afw;
  k.afw_alpha = 1.0;
  k.afw_beta = 1.0;
  return k;
}

static int upload_kappa(grid2d_gpu *g)
{
  size_t nn = (size_t) g->n * g->n, i;
  float *f = malloc(sizeof(float) * nn), *p = malloc(sizeof(float) * 2 * nn);
  int e;
  for(i = 0; i < nn; i++) {
    double d = g->h_kappa[i];
    f[i] = (float) d;
    p[2 * i] = (float) d;
    p[2 * i + 1] = (float) (d - (double) p[2 * i]);
  }
  e = (int) cudaMemcpy(g->kd, g->h_kappa, sizeof(double) * nn, cudaMemcpyHostToDevice);
  if(!e) e = (int) cudaMemcpy(g->kf, f, sizeof(float) * nn, cudaMemcpyHostToDevice);
  if(!e) e = (int) cudaMemcpy(g->kdd, p, sizeof(float) * 2 * nn, cudaMemcpyHostToDevice);
  if(!e) e = mxk_afw_factors(g->n, g->kf, 1.0, 1.0, g->afw, g->st);
  if(!e) e = (int) cudaStreamSynchronize(g->st);
  free(f);
  free(p);
  return e;
}

static grid2d_gpu *alloc_grid(int n, int K, cudaStream_t st)
{
  grid2d_gpu *g = calloc(1, sizeof(grid2d_gpu));
  size_t nn = (size_t) n * n;
  int k;
  g->n = n; g->K = K; g->h = 1.0 / n;
  g->h_kappa = malloc(sizeof(double) * nn);
  g->h_ph = malloc(mxk_phase_bytes(K));
  for(k = 0; k < (int) nn; k++) g->h_kappa[k] = 1.0;
  for(k = 0; k < K; k++) {
    g->h_ph[4 * k] = 1.0; g->h_ph[4 * k + 1] = 0.0;
    g->h_ph[4 * k + 2] = 1.0; g->h_ph[4 * k + 3] = 0.0;
  }
  if(cudaMalloc((void **) &g->kd, sizeof(double) * nn) || cudaMalloc((void **) &g->kf, sizeof(float) * nn)
     || cudaMalloc((void **) &g->kdd, sizeof(float) * 2 * nn) || cudaMalloc(&g->afw, 32 * nn)
     || cudaMalloc((void **) &g->ph, mxk_phase_bytes(K))) {
    free(g->h_kappa); free(g->h_ph); free(g);
    return 0;
  }
  g->st = st;
  mxk_phase_fill(K, g->h_ph);
  if(upload_kappa(g) || cudaMemcpy(g->ph, g->h_ph, mxk_phase_bytes(K), cudaMemcpyHostToDevice)) {
    del_grid2d_gpu(g);
    return 0;
  }
  return g;
}

grid2d_gpu *new_grid2d_gpu(int nx, int ny, double hx, double hy, int K)
{
  (void) hx; (void) hy;
  if(nx != ny || nx < 2 || (nx & 1) || K < 1)
    return 0;
  return alloc_grid(nx, K, 0);
}

void del_grid2d_gpu(grid2d_gpu *g)
{
  if(!g) return;
  cudaFree(g->kd); cudaFree(g->kf); cudaFree(g->kdd); cudaFree(g->afw); cudaFree(g->ph);
  free(g->h_kappa); free(g->h_ph);
  free(g);
}

grid2d_gpu *coarsen_grid2d_gpu(const grid2d_gpu *f)
{
  int n = f->n / 2, i, j;
  grid2d_gpu *g;
  if(f->n & 1) return 0;
  g = alloc_grid(n, f->K, f->st);
  if(!g) return 0;
  for(j = 0; j < n; j++)
    for(i = 0; i < n; i++)
      g->h_kappa[i + j * n] = 0.25 * (f->h_kappa[2 * i + 2 * j * 2 * n] + f->h_kappa[2 * i + 1 + 2 * j * 2 * n]
                                      + f->h_kappa[2 * i + (2 * j + 1) * 2 * n]
                                      + f->h_kappa[2 * i + 1 + (2 * j + 1) * 2 * n]);
  memcpy(g->h_ph, f->h_ph, mxk_phase_bytes(f->K));
  if(upload_kappa(g) || cudaMemcpy(g->ph, g->h_ph, mxk_phase_bytes(g->K), cudaMemcpyHostToDevice)) {
    del_grid2d_gpu(g);
    return 0;
  }
  return g;
}

int setkappa_grid2d_gpu(grid2d_gpu *g, const double *kappa)
{
  memcpy(g->h_kappa, kappa, sizeof(double) * g->n * g->n);
  return upload_kappa(g);
}

int setbloch_grid2d_gpu(grid2d_gpu *g, const mxg_field *xf, const mxg_field *yf)
{
  int k;
  for(k = 0; k < g->K; k++) {
    g->h_ph[4 * k] = creal_(xf[k]); g->h_ph[4 * k + 1] = cimag_(xf[k]);
    g->h_ph[4 * k + 2] = creal_(yf[k]); g->h_ph[4 * k + 3] = cimag_(yf[k]);
  }
  mxk_phase_fill(g->K, g->h_ph);
  return (int) cudaMemcpy(g->ph, g->h_ph, mxk_phase_bytes(g->K), cudaMemcpyHostToDevice);
}

int getsize_grid2d_gpu(const grid2d_gpu *g, int *nx, int *K)
{
  if(nx) *nx = g->n;
  if(K) *K = g->K;
  return 0;
}

/* ------------------------------------------------------------------ */
/* host <-> device layout conversion                                   */
/* ------------------------------------------------------------------ */

/* dense order [k][v][per] (double complex) <-> device [k][per][m] in prec */
static int put_block(int prec, void *dev, const mxg_field *host, int K, int m, size_t per)
{
  size_t es = mxk_elem_size(prec), tot = (size_t) K * m * per, e, k, v;
  unsigned char *buf = malloc(es * tot);
  const double *h = (const double *) host;
  int err;
  if(!buf) return MXG_ENOMEM;
  for(k = 0; k < (size_t) K; k++)
    for(v = 0; v < (size_t) m; v++)
      for(e = 0; e < per; e++) {
        const double *z = h + 2 * ((k * m + v) * per + e);
        size_t o = (k * per + e) * m + v;
        if(prec == MXG_C64) {
          float *q = (float *) buf + 2 * o;
          q[0] = (float) z[0]; q[1] = (float) z[1];
        }
        else if(prec == MXG_C128) {
          double *q = (double *) buf + 2 * o;
          q[0] = z[0]; q[1] = z[1];
        }
        else {
          float *q = (float *) buf + 4 * o;
          q[0] = (float) z[0]; q[1] = (float) (z[0] - (double) q[0]);
          q[2] = (float) z[1]; q[3] = (float) (z[1] - (double) q[2]);
        }
      }
  err = (int) cudaMemcpy(dev, buf, es * tot, cudaMemcpyHostToDevice);
  free(buf);
  return err;
}

static int get_block(int prec, const void *dev, mxg_field *host, int K, int m, size_t per)
{
  size_t es = mxk_elem_size(prec), tot = (size_t) K * m * per, e, k, v;
  unsigned char *buf = malloc(es * tot);
  double *h = (double *) host;
  int err;
  if(!buf) return MXG_ENOMEM;
  err = (int) cudaMemcpy(buf, dev, es * tot, cudaMemcpyDeviceToHost);
  if(!err)
    for(k = 0; k < (size_t) K; k++)
      for(v = 0; v < (size_t) m; v++)
        for(e = 0; e < per; e++) {
          double *z = h + 2 * ((k * m + v) * per + e);
          size_t o = (k * per + e) * m + v;
          if(prec == MXG_C64) {
            const float *q = (const float *) buf + 2 * o;
            z[0] = q[0]; z[1] = q[1];
          }
          else if(prec == MXG_C128) {
            const double *q = (const double *) buf + 2 * o;
            z[0] = q[0]; z[1] = q[1];
          }
          else {
            const float *q = (const float *) buf + 4 * o;
            z[0] = (double) q[0] + (double) q[1];
            z[1] = (double) q[2] + (double) q[3];
          }
        }
  free(buf);
  return err;
}

/* ------------------------------------------------------------------ */
/* edge2d                                                              */
/* ------------------------------------------------------------------ */

static size_t elen(const edge2d_gpu *x) { return (size_t) x->gr->K * 2 * x->gr->n * x->gr->n * x->m; }
static size_t nlen(const node2d_gpu *x) { return (size_t) x->gr->K * x->gr->n * x->gr->n * x->m; }

edge2d_gpu *new_edge2d_gpu(const grid2d_gpu *gr, int m, int prec)
{
  edge2d_gpu *x;
  if(m < 1 || m > 32 || prec < 0 || prec > 2) return 0;
  x = calloc(1, sizeof(edge2d_gpu));
  x->gr = gr; x->m = m; x->prec = prec;
  if(cudaMalloc(&x->d, elen(x) * mxk_elem_size(prec)) || mxk_zero(prec, x->d, elen(x), gr->st)) {
    free(x);
    return 0;
  }
  return x;
}

void del_edge2d_gpu(edge2d_gpu *x)
{
  if(!x) return;
  cudaFree(x->d);
  free(x);
}

size_t getdimension_edge2d_gpu(const edge2d_gpu *x) { return 2 * (size_t) x->gr->n * x->gr->n; }

static int same_shape_e(const edge2d_gpu *x, const edge2d_gpu *y)
{
  return x->gr->n == y->gr->n && x->gr->K == y->gr->K && x->m == y->m;
}

int zero_edge2d_gpu(edge2d_gpu *x) { return mxk_zero(x->prec, x->d, elen(x), x->gr->st); }

int copy_edge2d_gpu(const edge2d_gpu *x, edge2d_gpu *y)
{
  if(!same_shape_e(x, y)) return MXG_EINVAL;
  return mxk_convert(x->prec, x->d, y->prec, y->d, elen(x), x->gr->st);
}

int add_edge2d_gpu(mxg_field alpha, const edge2d_gpu *x, edge2d_gpu *y)
{
  if(!same_shape_e(x, y)) return MXG_EINVAL;
  return mxk_axpy(creal_(alpha), cimag_(alpha), x->prec, x->d, y->prec, y->d, elen(x), x->gr->st);
}

static int dot_e(const edge2d_gpu *x, const edge2d_gpu *y, double *out /* 2*K*m */)
{
  double *d;
  int e;
  size_t km = (size_t) x->gr->K * x->m;
  if(cudaMalloc((void **) &d, sizeof(double) * 2 * km)) return MXG_ENOMEM;
  e = (int) cudaMemsetAsync(d, 0, sizeof(double) * 2 * km, x->gr->st);
  if(!e) e = mxk_dot(2 * (size_t) x->gr->n * x->gr->n, x->m, x->gr->K, x->prec, x->d, y->prec, y->d, d, x->gr->st);
  if(!e) e = (int) cudaMemcpy(out, d, sizeof(double) * 2 * km, cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e;
}

int norm2_edge2d_gpu(const edge2d_gpu *x, double *out)
{
  size_t km = (size_t) x->gr->K * x->m, i;
  double *t = malloc(sizeof(double) * 2 * km);
  int e = dot_e(x, x, t);
  for(i = 0; !e && i < km; i++) out[i] = sqrt(t[2 * i]);
  free(t);
  return e;
}

int center_edge2d_gpu(edge2d_gpu *x)
{
  int K = x->gr->K, k, e, *flags, *d;
  double *acc;
  flags = malloc(sizeof(int) * K);
  for(k = 0; k < K; k++) flags[k] = 1;
  if(cudaMalloc((void **) &d, sizeof(int) * K)) { free(flags); return MXG_ENOMEM; }
  if(cudaMalloc((void **) &acc, sizeof(double) * 4 * K * x->m)) { cudaFree(d); free(flags); return MXG_ENOMEM; }
  e = (int) cudaMemcpy(d, flags, sizeof(int) * K, cudaMemcpyHostToDevice);
  if(!e) e = mxk_center(x->gr->n, x->m, K, d, x->prec, x->d, acc, x->gr->st);
  if(!e) e = (int) cudaStreamSynchronize(x->gr->st);
  cudaFree(acc);
  cudaFree(d);
  free(flags);
  return e;
}

int addeval_edge2d_gpu(mxg_field alpha, mxg_field beta, const edge2d_gpu *x, edge2d_gpu *y)
{
  const grid2d_gpu *g = x->gr;
  if(!same_shape_e(x, y) || cimag_(alpha) != 0.0 || cimag_(beta) != 0.0) return MXG_EINVAL;
  return mxk_edge_apply(g->n, x->m, g->K, g->ph, kap_of(g), creal_(alpha), creal_(beta), 0, 1.0,
                        x->prec, x->d, y->prec, 0, y->d, g->st);
}

int addeval_shifted_edge2d_gpu(double alpha, const double *beta, const edge2d_gpu *x, edge2d_gpu *y)
{
  const grid2d_gpu *g = x->gr;
  size_t km = (size_t) g->K * x->m;
  double *d;
  int e;
  if(!same_shape_e(x, y)) return MXG_EINVAL;
  if(cudaMalloc((void **) &d, sizeof(double) * km)) return MXG_ENOMEM;
  e = (int) cudaMemcpy(d, beta, sizeof(double) * km, cudaMemcpyHostToDevice);
  if(!e) e = mxk_edge_apply(g->n, x->m, g->K, g->ph, kap_of(g), alpha, 0.0, d, 1.0, x->prec, x->d, y->prec, 0, y->d,
                            g->st);
  if(!e) e = (int) cudaStreamSynchronize(g->st);
  cudaFree(d);
  return e;
}

static int product_e(double alpha, double beta, const edge2d_gpu *x, const edge2d_gpu *y, mxg_field *out)
{
  edge2d_gpu *t = new_edge2d_gpu(x->gr, x->m, y->prec);
  size_t km = (size_t) x->gr->K * x->m, i;
  double *buf = malloc(sizeof(double) * 2 * km);
  int e;
  if(!t) { free(buf); return MXG_ENOMEM; }
  e = mxk_edge_apply(x->gr->n, x->m, x->gr->K, x->gr->ph, kap_of(x->gr), alpha, beta, 0, 0.0, y->prec, y->d,
                     t->prec, 0, t->d, x->gr->st);
  if(!e) {
    edge2d_gpu xx = *x;
    if(x->prec != t->prec) e = MXG_EINVAL;
    else e = dot_e(&xx, t, buf);
  }
  for(i = 0; !e && i < km; i++) {
    double *o = (double *) (out + i);
    o[0] = buf[2 * i]; o[1] = buf[2 * i + 1];
  }
  del_edge2d_gpu(t);
  free(buf);
  return e;
}

int energyprod_edge2d_gpu(mxg_field alpha, mxg_field beta, const edge2d_gpu *x, const edge2d_gpu *y,
                          mxg_field *out)
{
  if(!same_shape_e(x, y) || x->prec != y->prec) return MXG_EINVAL;
  return product_e(creal_(alpha), creal_(beta), x, y, out);
}

int massprod_edge2d_gpu(const edge2d_gpu *x, const edge2d_gpu *y, mxg_field *out)
{
  if(!same_shape_e(x, y) || x->prec != y->prec) return MXG_EINVAL;
  return product_e(0.0, 1.0, x, y, out);
}

static int gs_e(double a, double b, const edge2d_gpu *bb, edge2d_gpu *x, int dir)
{
  const grid2d_gpu *g = x->gr;
  if(!same_shape_e(bb, x) || bb->prec != x->prec) return MXG_EINVAL;
  return mxk_edge_gs(g->n, x->m, g->K, g->ph, kap_of(g), a, b, dir, x->prec, bb->d, x->d, g->st);
}

int gsforward_edge2d_gpu(mxg_field a, mxg_field b, const edge2d_gpu *bb, edge2d_gpu *x) { return gs_e(creal_(a), creal_(b), bb, x, 0); }
int gsbackward_edge2d_gpu(mxg_field a, mxg_field b, const edge2d_gpu *bb, edge2d_gpu *x) { return gs_e(creal_(a), creal_(b), bb, x, 1); }
int gssymm_edge2d_gpu(mxg_field a, mxg_field b, const edge2d_gpu *bb, edge2d_gpu *x) { return gs_e(creal_(a), creal_(b), bb, x, 2); }

int gscolour_edge2d_gpu(mxg_field a, mxg_field b, const edge2d_gpu *bb, edge2d_gpu *x, int dir)
{
  const grid2d_gpu *g = x->gr;
  if(!same_shape_e(bb, x) || bb->prec != x->prec || dir < 0 || dir > 2) return MXG_EINVAL;
  return mxk_edge_gs_colour(g->n, x->m, g->K, g->ph, kap_of(g), creal_(a), creal_(b), dir, x->prec, bb->d, x->d,
                            g->st);
}

static int gs_simple(double a, double b, const edge2d_gpu *bb, edge2d_gpu *x, int dir)
{
  const grid2d_gpu *g = x->gr;
  if(!same_shape_e(bb, x) || bb->prec != x->prec) return MXG_EINVAL;
  return mxk_edge_gs_point(g->n, x->m, g->K, g->ph, kap_of(g), a, b, dir, x->prec, bb->d, x->d, g->st);
}

int gsforward_simple_edge2d_gpu(mxg_field a, mxg_field b, const edge2d_gpu *bb, edge2d_gpu *x)
{
  return gs_simple(creal_(a), creal_(b), bb, x, 0);
}
int gsbackward_simple_edge2d_gpu(mxg_field a, mxg_field b, const edge2d_gpu *bb, edge2d_gpu *x)
{
  return gs_simple(creal_(a), creal_(b), bb, x, 1);
}
int gssymm_simple_edge2d_gpu(mxg_field a, mxg_field b, const edge2d_gpu *bb, edge2d_gpu *x)
{
  return gs_simple(creal_(a), creal_(b), bb, x, 2);
}

int prolongation_edge2d_gpu(mxg_field alpha, const edge2d_gpu *c, edge2d_gpu *f)
{
  if(f->gr->n != 2 * c->gr->n || c->m != f->m || c->prec != f->prec || c->gr->K != f->gr->K) return MXG_EINVAL;
  return mxk_edge_prolong(c->gr->n, c->m, c->gr->K, f->gr->ph, creal_(alpha), c->prec, c->d, f->d, f->gr->st);
}

int restriction_edge2d_gpu(mxg_field alpha, const edge2d_gpu *f, edge2d_gpu *c)
{
  if(f->gr->n != 2 * c->gr->n || c->m != f->m || c->prec != f->prec || c->gr->K != f->gr->K) return MXG_EINVAL;
  return mxk_edge_restrict(c->gr->n, c->m, c->gr->K, f->gr->ph, creal_(alpha), c->prec, f->d, c->d, f->gr->st);
}

int vcycle_edge2d_gpu(int L, int nu, const matrix_gpu *Ac, edge2d_gpu **b, edge2d_gpu **x, edge2d_gpu **d)
{
  int l, i;
  for(l = L; l > 0; l--) {
    const grid2d_gpu *g = x[l]->gr;
    for(i = 0; i < nu; i++)
      TRY(mxk_edge_gs(g->n, x[l]->m, g->K, g->ph, kap_of(g), 1.0, 1.0, 0, x[l]->prec, b[l]->d, x[l]->d, g->st));
    if(b[l]->prec != d[l]->prec) return MXG_EINVAL;
    TRY(mxk_edge_apply(g->n, x[l]->m, g->K, g->ph, kap_of(g), -1.0, -1.0, 0, 1.0, x[l]->prec, x[l]->d,
                       d[l]->prec, b[l]->d, d[l]->d, g->st));
    TRY(zero_edge2d_gpu(b[l - 1]));
    TRY(mxk_edge_restrict(g->n / 2, x[l]->m, g->K, g->ph, 1.0, d[l]->prec, d[l]->d, b[l - 1]->d, g->st));
    TRY(zero_edge2d_gpu(x[l - 1]));
  }
  if(Ac) {
    const grid2d_gpu *g = x[0]->gr;
    if(!Ac->factored || Ac->rows != 2 * g->n * g->n || Ac->K != g->K) return MXG_EINVAL;
    TRY(mxk_coarse_apply(Ac->rows, x[0]->m, g->K, Ac->d, 0, x[0]->prec, b[0]->d, x[0]->d, g->st));
  }
  else
    for(i = 0; i < nu; i++)
      TRY(gs_e(1.0, 1.0, b[0], x[0], 2));
  for(l = 1; l <= L; l++) {
    const grid2d_gpu *g = x[l]->gr;
    TRY(mxk_edge_prolong(g->n / 2, x[l]->m, g->K, g->ph, 1.0, x[l]->prec, x[l - 1]->d, x[l]->d, g->st));
    for(i = 0; i < nu; i++)
      TRY(mxk_edge_gs(g->n, x[l]->m, g->K, g->ph, kap_of(g), 1.0, 1.0, 1, x[l]->prec, b[l]->d, x[l]->d, g->st));
  }
  return (int) cudaStreamSynchronize(x[L]->gr->st);
}

int hcycle_edge2d_gpu(int L, int nu, const matrix_gpu *Ac, edge2d_gpu **b, edge2d_gpu **x, edge2d_gpu **d,
                      node2d_gpu **bg, node2d_gpu **xg)
{
  /* hcycle_edge2d (edge2d.c:5756-5823) */
  int l, i;
  for(l = L; l > 0; l--) {
    const grid2d_gpu *g = x[l]->gr;
    for(i = 0; i < nu; i++)
      TRY(gs_simple(1.0, 1.0, b[l], x[l], 0));
    if(b[l]->prec != d[l]->prec) return MXG_EINVAL;
    TRY(mxk_edge_apply(g->n, x[l]->m, g->K, g->ph, kap_of(g), -1.0, -1.0, 0, 1.0, x[l]->prec, x[l]->d,
                       d[l]->prec, b[l]->d, d[l]->d, g->st));
    TRY(mxk_adjgradient(g->n, x[l]->m, g->K, g->ph, 1.0, 0, 0.0, d[l]->prec, d[l]->d, bg[l]->prec, bg[l]->d, g->st));
    TRY(zero_node2d_gpu(xg[l]));
    for(i = 0; i < nu; i++)
      TRY(mxk_node_gs(g->n, x[l]->m, g->K, g->ph, 1.0, 0, xg[l]->prec, bg[l]->d, xg[l]->d, g->st));
    TRY(mxk_gradient(g->n, x[l]->m, g->K, g->ph, 1.0, xg[l]->prec, xg[l]->d, x[l]->prec, x[l]->d, g->st));
    TRY(mxk_edge_apply(g->n, x[l]->m, g->K, g->ph, kap_of(g), -1.0, -1.0, 0, 1.0, x[l]->prec, x[l]->d,
                       d[l]->prec, b[l]->d, d[l]->d, g->st));
    TRY(zero_edge2d_gpu(b[l - 1]));
    TRY(mxk_edge_restrict(g->n / 2, x[l]->m, g->K, g->ph, 1.0, d[l]->prec, d[l]->d, b[l - 1]->d, g->st));
    TRY(zero_edge2d_gpu(x[l - 1]));
  }
  if(Ac) {
    const grid2d_gpu *g = x[0]->gr;
    if(!Ac->factored || Ac->rows != 2 * g->n * g->n || Ac->K != g->K) return MXG_EINVAL;
    TRY(mxk_coarse_apply(Ac->rows, x[0]->m, g->K, Ac->d, 0, x[0]->prec, b[0]->d, x[0]->d, g->st));
  }
  else
    for(i = 0; i < nu; i++)
      TRY(gs_simple(1.0, 1.0, b[0], x[0], 2));
  for(l = 1; l <= L; l++) {
    const grid2d_gpu *g = x[l]->gr;
    TRY(mxk_edge_prolong(g->n / 2, x[l]->m, g->K, g->ph, 1.0, x[l]->prec, x[l - 1]->d, x[l]->d, g->st));
    TRY(mxk_edge_apply(g->n, x[l]->m, g->K, g->ph, kap_of(g), -1.0, -1.0, 0, 1.0, x[l]->prec, x[l]->d,
                       d[l]->prec, b[l]->d, d[l]->d, g->st));
    TRY(mxk_adjgradient(g->n, x[l]->m, g->K, g->ph, 1.0, 0, 0.0, d[l]->prec, d[l]->d, bg[l]->prec, bg[l]->d, g->st));
    TRY(zero_node2d_gpu(xg[l]));
    for(i = 0; i < nu; i++)
      TRY(mxk_node_gs(g->n, x[l]->m, g->K, g->ph, 1.0, 1, xg[l]->prec, bg[l]->d, xg[l]->d, g->st));
    TRY(mxk_gradient(g->n, x[l]->m, g->K, g->ph, 1.0, xg[l]->prec, xg[l]->d, x[l]->prec, x[l]->d, g->st));
    for(i = 0; i < nu; i++)
      TRY(gs_simple(1.0, 1.0, b[l], x[l], 1));
  }
  return (int) cudaStreamSynchronize(x[L]->gr->st);
}

int densematrix_edge2d_gpu(mxg_field alpha, mxg_field beta, const grid2d_gpu *gr, matrix_gpu *a)
{
  if(a->rows != 2 * gr->n * gr->n || a->K != gr->K) return MXG_EINVAL;
  a->factored = 0;
  TRY(mxk_dense_edge(gr->n, gr->K, gr->ph, kap_of(gr), creal_(alpha), creal_(beta), a->d, gr->st));
  return (int) cudaStreamSynchronize(gr->st);
}

int denseto_edge2d_gpu(const mxg_field *host, edge2d_gpu *y)
{
  return put_block(y->prec, y->d, host, y->gr->K, y->m, 2 * (size_t) y->gr->n * y->gr->n);
}

int densefrom_edge2d_gpu(const edge2d_gpu *x, mxg_field *host)
{
  TRY((int) cudaStreamSynchronize(x->gr->st));
  return get_block(x->prec, x->d, host, x->gr->K, x->m, 2 * (size_t) x->gr->n * x->gr->n);
}

/* ------------------------------------------------------------------ */
/* node2d                                                              */
/* ------------------------------------------------------------------ */

node2d_gpu *new_node2d_gpu(const grid2d_gpu *gr, int m, int prec)
{
  node2d_gpu *x;
  if(m < 1 || m > 32 || prec < 0 || prec > 2) return 0;
  x = calloc(1, sizeof(node2d_gpu));
  x->gr = gr; x->m = m; x->prec = prec;
  if(cudaMalloc(&x->d, nlen(x) * mxk_elem_size(prec)) || mxk_zero(prec, x->d, nlen(x), gr->st)) {
    free(x);
    return 0;
  }
  return x;
}

void del_node2d_gpu(node2d_gpu *x)
{
  if(!x) return;
  cudaFree(x->d);
  free(x);
}

int zero_node2d_gpu(node2d_gpu *x) { return mxk_zero(x->prec, x->d, nlen(x), x->gr->st); }

int addeval_node2d_gpu(mxg_field alpha, const node2d_gpu *x, node2d_gpu *y)
{
  const grid2d_gpu *g = x->gr;
  if(x->prec != y->prec || x->m != y->m) return MXG_EINVAL;
  return mxk_node_apply(g->n, x->m, g->K, g->ph, creal_(alpha), 1.0, x->prec, x->d, 0, y->d, g->st);
}

static int gs_n(double a, const node2d_gpu *b, node2d_gpu *x, int dir)
{
  const grid2d_gpu *g = x->gr;
  int e;
  void *y = 0;
  if(b->prec != x->prec || b->m != x->m) return MXG_EINVAL;
  if(mxk_node_gs_oop_ok(g->n, x->m, x->prec) && cudaMalloc(&y, nlen(x) * mxk_elem_size(x->prec)) == cudaSuccess) {
    /* the tiled sweep into a scratch vector: x -> y (-> x backward for the
     * symmetric sweep), copied back after a single one */
    e = mxk_node_gs_oop(g->n, x->m, g->K, g->ph, a, dir == 1, x->prec, b->d, x->d, y, g->st);
    if(!e && dir == 2) e = mxk_node_gs_oop(g->n, x->m, g->K, g->ph, a, 1, x->prec, b->d, y, x->d, g->st);
    else if(!e)
      e = (int) cudaMemcpyAsync(x->d, y, nlen(x) * mxk_elem_size(x->prec), cudaMemcpyDeviceToDevice, g->st);
    if(!e) e = (int) cudaStreamSynchronize(g->st);
    cudaFree(y);
    return e;
  }
  cudaGetLastError();
  e = mxk_node_gs(g->n, x->m, g->K, g->ph, a, dir, x->prec, b->d, x->d, g->st);
  if(!e) e = (int) cudaStreamSynchronize(g->st);
  return e;
}

int gsforward_node2d_gpu(mxg_field a, const node2d_gpu *b, node2d_gpu *x) { return gs_n(creal_(a), b, x, 0); }
int gsbackward_node2d_gpu(mxg_field a, const node2d_gpu *b, node2d_gpu *x) { return gs_n(creal_(a), b, x, 1); }
int gssymm_node2d_gpu(mxg_field a, const node2d_gpu *b, node2d_gpu *x) { return gs_n(creal_(a), b, x, 2); }

int prolongation_node2d_gpu(mxg_field alpha, const node2d_gpu *c, node2d_gpu *f)
{
  if(f->gr->n != 2 * c->gr->n || c->m != f->m || c->prec != f->prec) return MXG_EINVAL;
  return mxk_node_prolong(c->gr->n, c->m, c->gr->K, f->gr->ph, creal_(alpha), c->prec, c->d, f->d, f->gr->st);
}

int residual_restriction_node2d_gpu(mxg_field alpha, const node2d_gpu *b, const node2d_gpu *x, node2d_gpu *c)
{
  if(x->gr->n != 2 * c->gr->n || x->m != c->m || b->m != x->m || x->prec != c->prec || b->prec != x->prec
     || b->gr->n != x->gr->n)
    return MXG_EINVAL;
  return mxk_node_residual_restrict(c->gr->n, c->m, c->gr->K, x->gr->ph, creal_(alpha), c->prec, x->d, b->d, c->d,
                                    x->gr->st);
}

int restriction_node2d_gpu(mxg_field alpha, const node2d_gpu *f, node2d_gpu *c)
{
  if(f->gr->n != 2 * c->gr->n || c->m != f->m || c->prec != f->prec) return MXG_EINVAL;
  return mxk_node_restrict(c->gr->n, c->m, c->gr->K, f->gr->ph, creal_(alpha), c->prec, f->d, c->d, f->gr->st);
}

int gradient_node2d_gpu(mxg_field alpha, const node2d_gpu *x, edge2d_gpu *y)
{
  const grid2d_gpu *g = x->gr;
  if(x->m != y->m || g->n != y->gr->n) return MXG_EINVAL;
  return mxk_gradient(g->n, x->m, g->K, g->ph, creal_(alpha), x->prec, x->d, y->prec, y->d, g->st);
}

int adjgradient_node2d_gpu(mxg_field alpha, const edge2d_gpu *x, node2d_gpu *y)
{
  const grid2d_gpu *g = x->gr;
  if(x->m != y->m || g->n != y->gr->n) return MXG_EINVAL;
  return mxk_adjgradient(g->n, x->m, g->K, g->ph, creal_(alpha), 0, 1.0, x->prec, x->d, y->prec, y->d, g->st);
}

int vcycle_node2d_gpu(int L, int nu, const matrix_gpu *Ac, node2d_gpu **b, node2d_gpu **x, node2d_gpu **d)
{
  int l, i;
  for(l = L; l > 0; l--) {
    const grid2d_gpu *g = x[l]->gr;
    for(i = 0; i < nu; i++)
      TRY(gs_n(1.0, b[l], x[l], 0));
    if(b[l]->prec != d[l]->prec) return MXG_EINVAL;
    TRY(mxk_node_apply(g->n, x[l]->m, g->K, g->ph, -1.0, 1.0, x[l]->prec, x[l]->d, b[l]->d, d[l]->d, g->st));
    TRY(zero_node2d_gpu(b[l - 1]));
    TRY(mxk_node_restrict(g->n / 2, x[l]->m, g->K, g->ph, 1.0, d[l]->prec, d[l]->d, b[l - 1]->d, g->st));
    TRY(zero_node2d_gpu(x[l - 1]));
  }
  if(Ac) {
    const grid2d_gpu *g = x[0]->gr;
    if(!Ac->factored || Ac->rows != g->n * g->n || Ac->K != g->K) return MXG_EINVAL;
    TRY(mxk_coarse_apply(Ac->rows, x[0]->m, g->K, Ac->d, 0, x[0]->prec, b[0]->d, x[0]->d, g->st));
  }
  else
    for(i = 0; i < nu; i++)
      TRY(gs_n(1.0, b[0], x[0], 2));
  for(l = 1; l <= L; l++) {
    const grid2d_gpu *g = x[l]->gr;
    TRY(mxk_node_prolong(g->n / 2, x[l]->m, g->K, g->ph, 1.0, x[l]->prec, x[l - 1]->d, x[l]->d, g->st));
    for(i = 0; i < nu; i++)
      TRY(gs_n(1.0, b[l], x[l], 1));
  }
  return (int) cudaStreamSynchronize(x[L]->gr->st);
}

int densematrix_node2d_gpu(int fixnull, const grid2d_gpu *gr, matrix_gpu *a)
{
  if(a->rows != gr->n * gr->n || a->K != gr->K) return MXG_EINVAL;
  a->factored = 0;
  TRY(mxk_dense_node(gr->n, gr->K, gr->ph, fixnull, a->d, gr->st));
  return (int) cudaStreamSynchronize(gr->st);
}

int denseto_node2d_gpu(const mxg_field *host, node2d_gpu *y)
{
  return put_block(y->prec, y->d, host, y->gr->K, y->m, (size_t) y->gr->n * y->gr->n);
}

int densefrom_node2d_gpu(const node2d_gpu *x, mxg_field *host)
{
  TRY((int) cudaStreamSynchronize(x->gr->st));
  return get_block(x->prec, x->d, host, x->gr->K, x->m, (size_t) x->gr->n * x->gr->n);
}

/* ------------------------------------------------------------------ */
/* linalg                                                              */
/* ------------------------------------------------------------------ */

matrix_gpu *new_matrix_gpu(int rows, int K)
{
  matrix_gpu *a = calloc(1, sizeof(matrix_gpu));
  a->rows = rows; a->K = K;
  if(cudaMalloc((void **) &a->d, sizeof(double) * 2 * (size_t) rows * rows * K)
     || cudaMalloc((void **) &a->info, sizeof(int) * K)) {
    free(a);
    return 0;
  }
  return a;
}

void del_matrix_gpu(matrix_gpu *a)
{
  if(!a) return;
  cudaFree(a->d);
  cudaFree(a->info);
  free(a);
}

int upload_matrix_gpu(matrix_gpu *a, const mxg_field *host)
{
  a->factored = 0;
  return (int) cudaMemcpy(a->d, host, sizeof(double) * 2 * (size_t) a->rows * a->rows * a->K, cudaMemcpyHostToDevice);
}

int download_matrix_gpu(const matrix_gpu *a, mxg_field *host)
{
  return (int) cudaMemcpy(host, a->d, sizeof(double) * 2 * (size_t) a->rows * a->rows * a->K, cudaMemcpyDeviceToHost);
}

int potrf_matrix_gpu(matrix_gpu *a, int *info)
{
  TRY(mxk_hpd_inverse(a->rows, a->K, a->d, a->info, 0));
  TRY((int) cudaMemcpy(info, a->info, sizeof(int) * a->K, cudaMemcpyDeviceToHost));
  a->factored = 1;
  return 0;
}

int syev_matrix_gpu(matrix_gpu *a, double *lambda, int *info)
{
  double *z, *w;
  int e;
  size_t sz = sizeof(double) * 2 * (size_t) a->rows * a->rows * a->K;
  if(cudaMalloc((void **) &z, sz)) return MXG_ENOMEM;
  if(cudaMalloc((void **) &w, sizeof(double) * a->rows * a->K)) { cudaFree(z); return MXG_ENOMEM; }
  e = mxk_heev(a->rows, a->K, a->d, z, w, a->info, 0);
  if(!e) e = (int) cudaMemcpy(lambda, w, sizeof(double) * a->rows * a->K, cudaMemcpyDeviceToHost);
  if(!e) e = (int) cudaMemcpy(info, a->info, sizeof(int) * a->K, cudaMemcpyDeviceToHost);
  cudaFree(z);
  cudaFree(w);
  return e;
}

int sygv_matrix_gpu(matrix_gpu *a, matrix_gpu *b, double *lambda, int *info)
{
  int N = a->rows, K = a->K, e, k;
  double *coef, *theta, *work;
  if(b->rows != N || b->K != K) return MXG_EINVAL;
  if(cudaMalloc((void **) &coef, sizeof(double) * 2 * (size_t) N * N * K)) return MXG_ENOMEM;
  if(cudaMalloc((void **) &theta, sizeof(double) * (size_t) N * K)) { cudaFree(coef); return MXG_ENOMEM; }
  if(cudaMalloc((void **) &work, sizeof(double) * mxk_ritz_work_doubles(N) * K)) {
    cudaFree(coef); cudaFree(theta);
    return MXG_ENOMEM;
  }
  /* the Ritz kernel reads full Hermitian matrices: complete from the lower triangle on the host side
   * of the convention (callers pass full matrices, as densematrix_*_gpu produces) */
  e = mxk_rayleigh_ritz(N, N, K, a->d, b->d, 0, 1e-14, -1e300, coef, theta, a->info, work, 0);
  if(!e) e = (int) cudaMemcpy(lambda, theta, sizeof(double) * (size_t) N * K, cudaMemcpyDeviceToHost);
  if(!e) e = (int) cudaMemcpy(info, a->info, sizeof(int) * K, cudaMemcpyDeviceToHost);
  if(!e) e = (int) cudaMemcpy(a->d, coef, sizeof(double) * 2 * (size_t) N * N * K, cudaMemcpyDeviceToDevice);
  for(k = 0; !e && k < K; k++)
    info[k] = info[k] == N ? 0 : (info[k] < 0 ? N + 1 : N + 1);
  cudaFree(coef); cudaFree(theta); cudaFree(work);
  return e;
}

int mxg_set_device(int device)
{
  return (int) cudaSetDevice(device);
}

int mxg_device_ok(void)
{
  int n = 0;
  if(cudaGetDeviceCount(&n) != cudaSuccess) return 0;
  return n > 0;
}

/* accessors for the solver translation unit */
const double *mxg__grid_phases(const grid2d_gpu *g) { return g->ph; }
void *mxg__edge_data(const edge2d_gpu *e) { return e->d; }

/* ------------------------------------------------------------------ */
/* further vector operations of edge2d.h / node2d.h                     */
/* ------------------------------------------------------------------ */

/* per-(k, vector) complex results of a device reduction into host memory */
static int reduce_to_host(const grid2d_gpu *g, size_t nd, double **dev)
{
  if(cudaMalloc((void **) dev, sizeof(double) * nd)) return MXG_ENOMEM;
  (void) g;
  return 0;
}

int swap_edge2d_gpu(edge2d_gpu *x, edge2d_gpu *y)
{
  void *t;
  if(!same_shape_e(x, y) || x->prec != y->prec) return MXG_EINVAL;
  TRY((int) cudaStreamSynchronize(x->gr->st));
  t = x->d; x->d = y->d; y->d = t;
  return 0;
}

int random_edge2d_gpu(edge2d_gpu *x, unsigned long long seed)
{
  return mxk_random(seed, x->prec, x->d, elen(x), x->gr->st);
}

int scale_edge2d_gpu(mxg_field alpha, edge2d_gpu *x)
{
  return mxk_scale(creal_(alpha), cimag_(alpha), x->prec, x->d, elen(x), x->gr->st);
}

static int absmax(const grid2d_gpu *g, size_t per, int m, int prec, const void *x, double *out)
{
  double *d;
  int e = reduce_to_host(g, (size_t) g->K * m, &d);
  if(e) return e;
  e = mxk_absmax(per, m, g->K, prec, x, d, g->st);
  if(!e) e = (int) cudaMemcpy(out, d, sizeof(double) * g->K * m, cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e;
}

int normmax_edge2d_gpu(const edge2d_gpu *x, double *out)
{
  return absmax(x->gr, 2 * (size_t) x->gr->n * x->gr->n, x->m, x->prec, x->d, out);
}

int dotprod_edge2d_gpu(const edge2d_gpu *x, const edge2d_gpu *y, mxg_field *out)
{
  if(!same_shape_e(x, y) || x->prec != y->prec) return MXG_EINVAL;
  return dot_e(x, y, (double *) out);
}

/* both planes' sums per (k, vector): acc[2*((k*2+p)*m+v)] */
static int plane_sums_e(const edge2d_gpu *x, double *host)
{
  const grid2d_gpu *g = x->gr;
  size_t nd = 2 * (size_t) g->K * 2 * x->m;
  double *d;
  int e = reduce_to_host(g, nd, &d);
  if(e) return e;
  e = mxk_plane_sums(g->n * g->n, 2, x->m, g->K, x->prec, x->d, d, g->st);
  if(!e) e = (int) cudaMemcpy(host, d, sizeof(double) * nd, cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e;
}

int nullprod_edge2d_gpu(const edge2d_gpu *x, mxg_field *xprod, mxg_field *yprod)
{
  /* edge2d.c:1240-1274: xprod = hx * sum 6 mx x = hy * sum of the x plane,
   * yprod = hx * sum of the y plane (hx = hy = 1/n) */
  const grid2d_gpu *g = x->gr;
  size_t km = (size_t) g->K * x->m, q;
  double *s = malloc(sizeof(double) * 4 * km), h = g->h;
  int e;
  if(!s) return MXG_ENOMEM;
  e = plane_sums_e(x, s);
  for(q = 0; !e && q < km; q++) {
    size_t k = q / x->m, v = q % x->m;
    const double *sx = s + 2 * ((k * 2 + 0) * x->m + v), *sy = s + 2 * ((k * 2 + 1) * x->m + v);
    if(xprod) { double *o = (double *) (xprod + q); o[0] = h * sx[0]; o[1] = h * sx[1]; }
    if(yprod) { double *o = (double *) (yprod + q); o[0] = h * sy[0]; o[1] = h * sy[1]; }
  }
  free(s);
  return e;
}

int nulladd_edge2d_gpu(const mxg_field *xalpha, const mxg_field *yalpha, edge2d_gpu *x)
{
  /* edge2d.c:1276-1307: x plane += hx xalpha, y plane += hy yalpha */
  const grid2d_gpu *g = x->gr;
  size_t km = (size_t) g->K * x->m, q, nd = 4 * km;
  double *c = malloc(sizeof(double) * nd), *d;
  int e;
  if(!c) return MXG_ENOMEM;
  for(q = 0; q < km; q++) {
    size_t k = q / x->m, v = q % x->m;
    double *cx = c + 2 * ((k * 2 + 0) * x->m + v), *cy = c + 2 * ((k * 2 + 1) * x->m + v);
    cx[0] = creal_(xalpha[q]); cx[1] = cimag_(xalpha[q]);
    cy[0] = creal_(yalpha[q]); cy[1] = cimag_(yalpha[q]);
  }
  e = reduce_to_host(g, nd, &d);
  if(!e) {
    e = (int) cudaMemcpy(d, c, sizeof(double) * nd, cudaMemcpyHostToDevice);
    if(!e) e = mxk_plane_shift(g->n * g->n, 2, x->m, g->K, d, g->h, x->prec, x->d, g->st);
    if(!e) e = (int) cudaStreamSynchronize(g->st);
    cudaFree(d);
  }
  free(c);
  return e;
}

/* Block Gram of the m vectors of every k-point: a[k] = X^H (A+M) X and
 * m[k] = X^H M X, full Hermitian m x m, column-major */
static int gram_e(const edge2d_gpu *x, double *ga, double *gm)
{
  const grid2d_gpu *g = x->gr;
  int pr[1];
  const void *pp[1];
  size_t nent = (size_t) x->m * (x->m + 1) / 2;
  size_t scratch = (size_t) g->K * 256 * nent * 4 * sizeof(double);
  double *sc;
  int e;
  if(scratch > ((size_t) 1 << 28)) scratch = (size_t) 1 << 28;
  if(cudaMalloc((void **) &sc, scratch)) return MXG_ENOMEM;
  pr[0] = x->prec; pp[0] = x->d;
  e = mxk_block_gram(g->n, x->m, g->K, g->ph, kap_of(g), 1, pr, pp, 0, 0, ga, gm, sc, scratch, g->st);
  if(!e) e = (int) cudaStreamSynchronize(g->st);
  cudaFree(sc);
  return e;
}

int gram_edge2d_gpu(const edge2d_gpu *x, mxg_field *a, mxg_field *m)
{
  const grid2d_gpu *g = x->gr;
  size_t sz = sizeof(double) * 2 * (size_t) x->m * x->m * g->K;
  double *ga, *gm;
  int e;
  if(x->m > 48) return MXG_EINVAL;
  if(cudaMalloc((void **) &ga, sz)) return MXG_ENOMEM;
  if(cudaMalloc((void **) &gm, sz)) { cudaFree(ga); return MXG_ENOMEM; }
  e = gram_e(x, ga, gm);
  if(!e && a) e = (int) cudaMemcpy(a, ga, sz, cudaMemcpyDeviceToHost);
  if(!e && m) e = (int) cudaMemcpy(m, gm, sz, cudaMemcpyDeviceToHost);
  cudaFree(ga);
  cudaFree(gm);
  return e;
}

/* y[k][j] = sum_i coef[k](i, j) x[k][i] */
static int lincomb_dev(const edge2d_gpu *x, const double *dcoef, edge2d_gpu *y)
{
  const grid2d_gpu *g = x->gr;
  int pr[1];
  const void *pp[1];
  void *cw;
  int e;
  if(cudaMalloc(&cw, (size_t) 16 * x->m * x->m * g->K)) return MXG_ENOMEM;
  pr[0] = x->prec; pp[0] = x->d;
  e = mxk_block_combine(g->n, x->m, g->K, 1, pr, pp, dcoef, x->m, 0, cw, y->prec, y->d, g->st);
  if(!e) e = (int) cudaStreamSynchronize(g->st);
  cudaFree(cw);
  return e;
}

int lincomb_edge2d_gpu(const mxg_field *coef, const edge2d_gpu *x, edge2d_gpu *y)
{
  size_t sz = sizeof(double) * 2 * (size_t) x->m * x->m * x->gr->K;
  double *d;
  int e;
  if(!same_shape_e(x, y) || x == y || x->d == y->d) return MXG_EINVAL;
  if(cudaMalloc((void **) &d, sz)) return MXG_ENOMEM;
  e = (int) cudaMemcpy(d, coef, sz, cudaMemcpyHostToDevice);
  if(!e) e = lincomb_dev(x, d, y);
  cudaFree(d);
  return e;
}

int orthonormalize_edge2d_gpu(edge2d_gpu *x, int *info)
{
  /* Cholesky-QR in the mass inner product: G = X^H M X = R^H R, X <- X R^-1 */
  const grid2d_gpu *g = x->gr;
  size_t sz = sizeof(double) * 2 * (size_t) x->m * x->m * g->K;
  double *ga = 0, *gm = 0, *coef = 0;
  int *dinfo = 0, e, k, bad = 0;
  edge2d_gpu *t;
  if(x->m > 48) return MXG_EINVAL;
  t = new_edge2d_gpu(g, x->m, x->prec);
  if(!t) return MXG_ENOMEM;
  if(cudaMalloc((void **) &ga, sz) || cudaMalloc((void **) &gm, sz) || cudaMalloc((void **) &coef, sz)
     || cudaMalloc((void **) &dinfo, sizeof(int) * g->K)) {
    e = MXG_ENOMEM;
    goto out;
  }
  e = gram_e(x, ga, gm);
  if(!e) e = mxk_chol_qr_coef(x->m, g->K, gm, coef, dinfo, g->st);
  if(!e) e = (int) cudaMemcpy(info, dinfo, sizeof(int) * g->K, cudaMemcpyDeviceToHost);
  for(k = 0; !e && k < g->K; k++)
    if(info[k]) bad = 1;
  if(!e && !bad) e = lincomb_dev(x, coef, t);
  if(!e && !bad) { void *q = x->d; x->d = t->d; t->d = q; }
  if(!e && bad) e = MXG_ECONV;
out:
  cudaFree(ga); cudaFree(gm); cudaFree(coef); cudaFree(dinfo);
  del_edge2d_gpu(t);
  return e;
}

int pinvit_edge2d_gpu(int l, int smoother_steps, int prec_steps, int gradient_steps, const double *lambda,
                      edge2d_gpu *e, const matrix_gpu *Ae, edge2d_gpu **b, edge2d_gpu **x, edge2d_gpu **d,
                      const matrix_gpu *An, node2d_gpu **bg, node2d_gpu **xg, node2d_gpu **dg)
{
  /* pinvit_edge2d (edge2d.c:6298-6328) for every (k, vector) of the batch,
   * each with its own lambda (the defect is (A+M) e - lambda M e) */
  const grid2d_gpu *g = e->gr;
  size_t km = (size_t) g->K * e->m, q;
  double *shift = malloc(sizeof(double) * km);
  int j, err;
  if(!shift) return MXG_ENOMEM;
  for(q = 0; q < km; q++) shift[q] = 1.0 - lambda[q];
  err = zero_edge2d_gpu(b[l]);
  if(!err) err = addeval_shifted_edge2d_gpu(1.0, shift, e, b[l]);
  free(shift);
  if(!err) err = zero_edge2d_gpu(x[l]);
  for(j = 0; !err && j < prec_steps; j++) err = vcycle_edge2d_gpu(l, smoother_steps, Ae, b, x, d);
  if(!err) err = add_edge2d_gpu(-1.0, x[l], e);
  if(!err) err = zero_edge2d_gpu(d[l]);
  if(!err) err = addeval_edge2d_gpu(0.0, 1.0, e, d[l]);
  if(!err) err = zero_node2d_gpu(bg[l]);
  if(!err) err = adjgradient_node2d_gpu(1.0, d[l], bg[l]);
  if(!err) err = zero_node2d_gpu(xg[l]);
  for(j = 0; !err && j < gradient_steps; j++) err = vcycle_node2d_gpu(l, smoother_steps, An, bg, xg, dg);
  if(!err) err = gradient_node2d_gpu(-1.0, xg[l], e);
  if(!err) err = (int) cudaStreamSynchronize(g->st);
  return err;
}

int copy_node2d_gpu(const node2d_gpu *x, node2d_gpu *y)
{
  if(x->gr->n != y->gr->n || x->gr->K != y->gr->K || x->m != y->m) return MXG_EINVAL;
  return mxk_convert(x->prec, x->d, y->prec, y->d, nlen(x), x->gr->st);
}

int random_node2d_gpu(node2d_gpu *x, unsigned long long seed)
{
  return mxk_random(seed, x->prec, x->d, nlen(x), x->gr->st);
}

int scale_node2d_gpu(mxg_field alpha, node2d_gpu *x)
{
  return mxk_scale(creal_(alpha), cimag_(alpha), x->prec, x->d, nlen(x), x->gr->st);
}

int add_node2d_gpu(mxg_field alpha, const node2d_gpu *x, node2d_gpu *y)
{
  if(x->gr->n != y->gr->n || x->gr->K != y->gr->K || x->m != y->m) return MXG_EINVAL;
  return mxk_axpy(creal_(alpha), cimag_(alpha), x->prec, x->d, y->prec, y->d, nlen(x), x->gr->st);
}

static int dot_n(const node2d_gpu *x, const node2d_gpu *y, double *out)
{
  double *d;
  int e;
  size_t km = (size_t) x->gr->K * x->m;
  if(cudaMalloc((void **) &d, sizeof(double) * 2 * km)) return MXG_ENOMEM;
  e = (int) cudaMemsetAsync(d, 0, sizeof(double) * 2 * km, x->gr->st);
  if(!e) e = mxk_dot((size_t) x->gr->n * x->gr->n, x->m, x->gr->K, x->prec, x->d, y->prec, y->d, d, x->gr->st);
  if(!e) e = (int) cudaMemcpy(out, d, sizeof(double) * 2 * km, cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e;
}

int dotprod_node2d_gpu(const node2d_gpu *x, const node2d_gpu *y, mxg_field *out)
{
  if(x->gr->n != y->gr->n || x->gr->K != y->gr->K || x->m != y->m || x->prec != y->prec) return MXG_EINVAL;
  return dot_n(x, y, (double *) out);
}

int norm2_node2d_gpu(const node2d_gpu *x, double *out)
{
  size_t km = (size_t) x->gr->K * x->m, i;
  double *t = malloc(sizeof(double) * 2 * km);
  int e;
  if(!t) return MXG_ENOMEM;
  e = dot_n(x, x, t);
  for(i = 0; !e && i < km; i++) out[i] = sqrt(t[2 * i]);
  free(t);
  return e;
}

int normmax_node2d_gpu(const node2d_gpu *x, double *out)
{
  return absmax(x->gr, (size_t) x->gr->n * x->gr->n, x->m, x->prec, x->d, out);
}

int center_node2d_gpu(node2d_gpu *x)
{
  /* node2d.c:489-514: subtract the mean of the n*n coefficients */
  const grid2d_gpu *g = x->gr;
  size_t nd = 2 * (size_t) g->K * x->m;
  double *d;
  int e = reduce_to_host(g, nd, &d);
  if(e) return e;
  e = mxk_plane_sums(g->n * g->n, 1, x->m, g->K, x->prec, x->d, d, g->st);
  if(!e) e = mxk_plane_shift(g->n * g->n, 1, x->m, g->K, d, -1.0 / ((double) g->n * g->n), x->prec, x->d, g->st);
  if(!e) e = (int) cudaStreamSynchronize(g->st);
  cudaFree(d);
  return e;
}

int potrsv_matrix_gpu(const matrix_gpu *a, mxg_field *b)
{
  /* potrsv_matrix (linalg.c:98-113): b <- A^-1 b per k, with the factor of
   * potrf_matrix_gpu (kept as the explicit inverse) */
  size_t sz = sizeof(double) * 2 * (size_t) a->rows * a->K;
  double *x, *y;
  int e;
  if(!a->factored) return MXG_EINVAL;
  if(cudaMalloc((void **) &x, sz)) return MXG_ENOMEM;
  if(cudaMalloc((void **) &y, sz)) { cudaFree(x); return MXG_ENOMEM; }
  e = (int) cudaMemcpy(x, b, sz, cudaMemcpyHostToDevice);
  if(!e) e = mxk_coarse_apply(a->rows, 1, a->K, a->d, 0, MX_C128, x, y, 0);
  if(!e) e = (int) cudaMemcpy(b, y, sz, cudaMemcpyDeviceToHost);
  cudaFree(x);
  cudaFree(y);
  return e;
}

/* ------------------------------------------------------------------ */
/* permittivity patterns (grid2d.h:40-78)                               */
/* ------------------------------------------------------------------ */

mxg_epspattern *new_epspattern_gpu(double eps_base, int rectangles, int circles)
{
  mxg_epspattern *p;
  if(rectangles < 0 || circles < 0) return 0;
  p = calloc(1, sizeof(mxg_epspattern));
  if(!p) return 0;
  p->rectangle = calloc((size_t) 5 * rectangles + 1, sizeof(double));
  p->circle = calloc((size_t) 4 * circles + 1, sizeof(double));
  p->rectangles = rectangles;
  p->circles = circles;
  p->eps_base = eps_base;
  if(!p->rectangle || !p->circle) { del_epspattern_gpu(p); return 0; }
  return p;
}

void del_epspattern_gpu(mxg_epspattern *p)
{
  if(!p) return;
  free(p->rectangle);
  free(p->circle);
  free(p);
}

int setpattern_grid2d_gpu(const mxg_epspattern *pat, grid2d_gpu *g)
{
  size_t nn = (size_t) g->n * g->n;
  double *rect = 0, *circ = 0, *kd = 0;
  int e;
  if(!pat) return 0;   /* setpattern_grid2d returns without a pattern */
  if(pat->rectangles < 0 || pat->circles < 0) return MXG_EINVAL;
  if(cudaMalloc((void **) &rect, sizeof(double) * (5 * (size_t) pat->rectangles + 1))
     || cudaMalloc((void **) &circ, sizeof(double) * (4 * (size_t) pat->circles + 1))
     || cudaMalloc((void **) &kd, sizeof(double) * nn)) {
    cudaFree(rect); cudaFree(circ);
    return MXG_ENOMEM;
  }
  e = (int) cudaMemcpy(rect, pat->rectangle, sizeof(double) * 5 * pat->rectangles, cudaMemcpyHostToDevice);
  if(!e) e = (int) cudaMemcpy(circ, pat->circle, sizeof(double) * 4 * pat->circles, cudaMemcpyHostToDevice);
  if(!e) e = mxk_pattern(g->n, rect, pat->rectangles, circ, pat->circles, pat->eps_base, kd, g->st);
  if(!e) e = (int) cudaMemcpy(g->h_kappa, kd, sizeof(double) * nn, cudaMemcpyDeviceToHost);
  if(!e) e = upload_kappa(g);
  cudaFree(rect); cudaFree(circ); cudaFree(kd);
  return e;
}

int getkappa_grid2d_gpu(const grid2d_gpu *g, double *kappa)
{
  memcpy(kappa, g->h_kappa, sizeof(double) * g->n * g->n);
  return 0;
}

/* ------------------------------------------------------------------ */
/* protocol file of the Bloch scan (exp_bloch2d.c:416-443, 754-760,       */
/* 1227-1235)                                                            */
/* ------------------------------------------------------------------ */

int mxg_write_protocol(const char *filename, const mxg_protocol_info *info, int nk, int m, const double *lambda,
                       const int *steps, const double *seconds, const mxg_field *chern, const int *sign)
{
  FILE *out;
  int l, i, cv;
  double accum = 0.0;
  if(!filename || !info || nk < 1 || m < 1 || !lambda || info->chern_vectors < 0 || (info->chern_vectors && !chern))
    return MXG_EINVAL;
  cv = info->chern_vectors;
  out = fopen(filename, "w");
  if(!out) return MXG_EINVAL;
  fprintf(out,
          "# Bloch eigenvalues\n"
          "# ----------------------------------------\n"
          "# Permittivity pattern: %s\n"
          "# Coarse grid intervals: %d\n"
          "# Refinement levels: %d\n"
          "# Chern vectors: %d\n"
          "# Extrapolation method: %s\n"
          "# Stopping criterion: %s\n"
          "# Eigenvector continuity: %s\n"
          "# ----------------------------------------\n"
          "# 1: Bloch step\n"
          "# 2..%d: Eigenvalues\n"
          "# %d: Iterations\n"
          "# %d: Time for this step [s]\n"
          "# %d: Total time to this step [s]\n"
          "# %d: Chern partial integral, real part\n"
          "# %d: Chern partial integral, imaginary part\n"
          "# ----------------------------------------\n",
          info->pattern ? info->pattern : "",
          info->n0, info->L, cv,
          info->extrapolation == '1' ? "1st order" : info->extrapolation == '2' ? "2nd order" : "None",
          info->stopping == 'f' ? "Fixed steps" : "Residual",
          info->continuity == 's' ? "Sign" : info->continuity == 'r' ? "Reorder" : "None",
          m + 1, m + 2, m + 3, m + 4, m + 5, m + 6);
  /* the starting point: its eigenvalues only */
  fprintf(out, "0");
  for(i = 0; i < m; i++) fprintf(out, " %f", lambda[i]);
  fprintf(out, "\n");
  for(l = 1; l < nk; l++) {
    double t = seconds ? seconds[l] : 0.0;
    accum += t;
    fprintf(out, "%d", l);
    for(i = 0; i < m; i++) fprintf(out, " %f", lambda[(size_t) l * m + i]);
    fprintf(out, "  %d  %.1f %.1f ", steps ? steps[l] : 0, t, accum);
    for(i = 0; i < cv; i++)
      fprintf(out, " %f %f", creal(chern[(size_t) l * cv + i]), cimag(chern[(size_t) l * cv + i]));
    fprintf(out, "  %d\n", sign ? sign[l] : 0);
  }
  return fclose(out) ? MXG_EINVAL : 0;
}
