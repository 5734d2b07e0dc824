/* The per-k eigensolver of exp_bloch2d (exp_bloch2d.c:520-1053) for a batch
 * of k-points solved together on one GPU.
 *
 * Flow per batch ("wave") of K k-points:
 *   - coarse dense generalized eigenproblem on level 0 for every k
 *     (exp_bloch2d.c:530-554), skipping the zero eigenvalues, then the nested
 *     iteration over levels 1..L (exp_bloch2d.c:562-732) -- or, for every
 *     wave after the first, a warm start from the converged block of the
 *     k-point one wave earlier (exp_bloch2d.c:814-895, extrapolation 'n');
 *   - block steps until every wanted pair of every k meets the tolerance:
 *       PINVIT + Ritz (exp_bloch2d.c:956-1053): defect, prec_steps edge
 *       V-cycles, update, gradient lifting, Rayleigh-Ritz on the block;
 *       LOBPCG (test_lobpcg2d.c:217-365 with Knyazev's search direction and
 *       soft locking): preconditioned defect X, gradient lifting of X,
 *       Rayleigh-Ritz on [E, X, P] by Cholesky-QR of the Gram matrix.
 * The coarse solvers are refactored per k (exp_bloch2d.c:782-810) as explicit
 * inverses.  Residuals are r_i = (A+M) e_i - mu_i M e_i with, as the
 * stopping rule, either the reference's absolute norm or ||r_i|| / (mu_i ||M e_i||).
 */
#define _POSIX_C_SOURCE 200809L
#include "maxwell_gb300.h"
#include "mx_internal.h"

#include <cuda_profiler_api.h>
#include <cuda_runtime_api.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define MAXL 16
#define NSTAT 5

#include <time.h>
static double now_s(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}
/* GPU time per phase of the block steps at the finest level (CUDA events,
 * read once per step), reported with MXG_TIMING set */
enum { PH_PREC, PH_LIFTX, PH_GRAM, PH_RR, PH_COMB, PH_LIFTE, PH_RESID, PH_N };
static const char *ph_name[PH_N] = {"precondition", "lift X", "gram", "rayleigh-ritz", "combine", "lift E",
                                    "residual"};

struct mxg_solver {
  mxg_solve_opts o;
  int n0, L, m, K, pe, pg;
  cudaStream_t st;
  cudaEvent_t ev0, ev1;
  int n[MAXL];
  double *kd[MAXL];
  float *kf[MAXL], *kdd[MAXL];
  void *kafw[MAXL];                  /* AFW patch factors (alpha = beta = 1) */
  double *ph;                        /* phase table (mxk_phase_bytes) */
  double *ph2;                       /* phase table of a subset of the slots (continuity) */
  int *gamma;                        /* K flags */
  void *b[MAXL], *x[MAXL], *d[MAXL];
  void *bg[MAXL], *xg[MAXL], *dg[MAXL];
  double *ae_inv, *an_inv;
  void *ae_inv_f, *an_inv_f;         /* their c64 roundings (FP32 solves) */
  void *E, *En, *P, *Pn;
  void *Eprev[3];                    /* eigenvectors of the last three waves, newest first */
  void *Eref;                        /* the block before the refinement sweep (refine only) */
  double *ga, *gm, *coef, *theta, *rwork, *gscratch, *mu, *stats;
  size_t gscratch_bytes;
  int *sel, *info;
  double *cacc;                      /* 4*K*m: plane means of center */
  void *combw;                       /* K*ns*m*16: combine coefficients */
  double *cA, *cM, *ccoef, *ctheta, *cwork;   /* coarse eigenproblem */
  int *cinfo;
  /* host */
  double *h_ph, *h_stats, *h_mu, *h_res, *h_rq;
  int *h_sel, *h_info, *h_conv, *h_steps;
  int have_prev, K_prev;              /* waves stored in Eprev (0..3) and their width */
  int last_nk;                        /* k-points of the last mxg_bloch_solve */
  double last_ms;
  long launches;
  /* CUDA-event timing of the finest level's node Gauss-Seidel sweeps, AFW
   * sweeps and Gram launches (mxg_solver_profile): event pairs on the
   * solver's stream, each with its kernel kind and algorithmic bytes */
  int timing;
  cudaEvent_t tev[PH_N + 1];
  double tph[PH_N];
  double cur_tol;       /* stopping tolerance of the level being iterated */
  int wave_gamma;       /* the current wave holds Gamma */
  int prof;
  cudaEvent_t *pev;
  int *ptag;
  double *pbytes;
  int npev, maxpev;
  double prof_ms[MXG_KT_N], prof_bytes[MXG_KT_N];
  long prof_count[MXG_KT_N];
  int prof_step, prof_done;          /* profiler window (MXG_PROFILE_STEP) */
  /* CUDA graphs of the inner multigrid loops, one per level: the edge
   * V-cycles of the preconditioner and the node V-cycles of a lifting */
  cudaGraphExec_t gpre[MAXL], glift[MAXL];
  long gpre_n[MAXL], glift_n[MAXL];   /* kernel launches each graph holds */
  /* the Ritz step (Gram, column selection, Rayleigh-Ritz, combinations) per
   * level, block count and which buffers E and P sit in */
  cudaGraphExec_t gritz[MAXL][3][2][2];
  long gritz_n[MAXL][3][2][2];
  void *E0, *P0;                       /* the first buffers of E and P */
  struct {
    int nb, with_p;
    int pr[3];
    const void *pp[3];
    double drop, theta_min;
  } rb;                                /* arguments of the Ritz step being run */
  int ritz_pending;                    /* a Ritz step's info and Ritz values not yet read */
  int graphs;                          /* 1 capture and replay, 0 launch directly */
  int restarts;                       /* warm-started waves solved again cold */
  int debug;                          /* per-step residual trace on stderr */
  int order;                          /* earlier waves a warm start combines (1, 2 or 3) */
  int all_columns;                    /* Ritz basis with every search column (refinement) */
  int device;                         /* the CUDA device the solver lives on */
};

#define L_(x) do { int e_ = (x); s->launches++; if (e_) return e_; } while (0)
#define TRY(x) do { int e_ = (x); if (e_) return e_; } while (0)

static mxk_kappa kap(const mxg_solver *s, int l)
{
  mxk_kappa k;
  k.f = s->kf[l]; k.d = s->kd[l]; k.dd = s->kdd[l];
  k.afw = s->kafw[l]; k.afw_alpha = 1.0; k.afw_beta = 1.0;
  return k;
}

static size_t elen(const mxg_solver *s, int l) { return (size_t) s->K * 2 * s->n[l] * s->n[l] * s->m; }
static size_t nlen(const mxg_solver *s, int l) { return (size_t) s->K * s->n[l] * s->n[l] * s->m; }

static int dalloc(void **p, size_t bytes)
{
  return cudaMalloc(p, bytes) != cudaSuccess;
}

void mxg_solver_free(mxg_solver *s)
{
  int l;
  if(!s) return;
  for(l = 0; l <= s->L; l++) {
    int a, b, c;
    if(s->gpre[l]) cudaGraphExecDestroy(s->gpre[l]);
    if(s->glift[l]) cudaGraphExecDestroy(s->glift[l]);
    for(a = 0; a < 3; a++)
      for(b = 0; b < 2; b++)
        for(c = 0; c < 2; c++)
          if(s->gritz[l][a][b][c]) cudaGraphExecDestroy(s->gritz[l][a][b][c]);
    cudaFree(s->kd[l]); cudaFree(s->kf[l]); cudaFree(s->kdd[l]); cudaFree(s->kafw[l]);
    cudaFree(s->b[l]); cudaFree(s->x[l]); cudaFree(s->d[l]);
    cudaFree(s->bg[l]); cudaFree(s->xg[l]); cudaFree(s->dg[l]);
  }
  cudaFree(s->ph); cudaFree(s->ph2); cudaFree(s->gamma); cudaFree(s->ae_inv); cudaFree(s->an_inv); cudaFree(s->ae_inv_f); cudaFree(s->an_inv_f);
  cudaFree(s->E); cudaFree(s->En); cudaFree(s->P); cudaFree(s->Pn);
  cudaFree(s->Eprev[0]); cudaFree(s->Eprev[1]); cudaFree(s->Eprev[2]); cudaFree(s->Eref);
  cudaFree(s->ga); cudaFree(s->gm); cudaFree(s->coef); cudaFree(s->theta); cudaFree(s->rwork);
  cudaFree(s->gscratch); cudaFree(s->mu); cudaFree(s->stats); cudaFree(s->sel); cudaFree(s->info);
  cudaFree(s->cA); cudaFree(s->cM); cudaFree(s->ccoef); cudaFree(s->ctheta); cudaFree(s->cwork);
  cudaFree(s->cinfo);
  cudaFree(s->cacc);
  cudaFree(s->combw);
  if(s->pev) {
    int q;
    for(q = 0; q < s->maxpev; q++) cudaEventDestroy(s->pev[q]);
    free(s->pev);
    free(s->ptag);
    free(s->pbytes);
  }
  if(s->st) cudaStreamDestroy(s->st);
  if(s->ev0) cudaEventDestroy(s->ev0);
  if(s->ev1) cudaEventDestroy(s->ev1);
  free(s->h_ph); free(s->h_stats); free(s->h_mu); free(s->h_res); free(s->h_rq);
  free(s->h_sel); free(s->h_info); free(s->h_conv); free(s->h_steps);
  free(s);
}

mxg_solver *mxg_solver_new(const mxg_solve_opts *o, const double *kappa_fine)
{
  mxg_solver *s;
  int l, K, m, ns, N0e, N0n;
  size_t es_g, es_e;
  double *kk[MAXL];
  if(o->L < 0 || o->L >= MAXL - 1 || o->n0 < 4 || (o->n0 & 1) || o->m < 1 || o->m > 32
     || o->ieigs < 1 || o->ieigs > o->m || o->wave < 1 || o->smoother < 0 || o->smoother > 2
     || o->precision < 0 || o->precision > 2
     || (o->extrapolation != 0 && o->extrapolation != 'n' && o->extrapolation != '1' && o->extrapolation != '2'
         && o->extrapolation != 'c'))
    return 0;
  s = calloc(1, sizeof(mxg_solver));
  s->o = *o;
  s->cur_tol = o->tol;
  s->order = o->extrapolation == '2' ? 3 : o->extrapolation == '1' ? 2 : 1;
  if(cudaGetDevice(&s->device) != cudaSuccess) { free(s); return 0; }
  s->n0 = o->n0; s->L = o->L; s->m = m = o->m; s->K = K = o->wave;
  /* precision 0: everything FP64; 1: float-float eigenvector block, FP32
   * multigrid and search blocks; 2: FP64 eigenvector block, FP32 multigrid
   * and search blocks (for residuals below the float-float floor, about
   * ||A|| 2^-48 / lambda relative, which grows with n^2) */
  s->pe = o->precision == 1 ? MX_CDD : MX_C128;
  s->pg = o->precision ? MX_C64 : MX_C128;
  es_g = mxk_elem_size(s->pg);
  es_e = mxk_elem_size(s->pe);
  ns = 3 * m;
  N0e = 2 * o->n0 * o->n0;
  N0n = o->n0 * o->n0;
  if(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) || cudaEventCreate(&s->ev0)
     || cudaEventCreate(&s->ev1))
    goto fail;
  /* kappa hierarchy (coarsen_grid2d, grid2d.c:42-68) */
  for(l = o->L; l >= 0; l--) {
    int n = o->n0 << l, i, j;
    size_t nn = (size_t) n * n, q;
    float *f, *p;
    s->n[l] = n;
    kk[l] = malloc(sizeof(double) * nn);
    if(l == o->L)
      memcpy(kk[l], kappa_fine, sizeof(double) * nn);
    else
      for(j = 0; j < n; j++)
        for(i = 0; i < n; i++)
          kk[l][i + j * n] = 0.25 * (kk[l + 1][2 * i + 2 * j * 2 * n] + kk[l + 1][2 * i + 1 + 2 * j * 2 * n]
                                     + kk[l + 1][2 * i + (2 * j + 1) * 2 * n]
                                     + kk[l + 1][2 * i + 1 + (2 * j + 1) * 2 * n]);
    f = malloc(sizeof(float) * nn);
    p = malloc(sizeof(float) * 2 * nn);
    for(q = 0; q < nn; q++) {
      f[q] = (float) kk[l][q];
      p[2 * q] = (float) kk[l][q];
      p[2 * q + 1] = (float) (kk[l][q] - (double) p[2 * q]);
    }
    if(dalloc((void **) &s->kd[l], sizeof(double) * nn) || dalloc((void **) &s->kf[l], sizeof(float) * nn)
       || dalloc((void **) &s->kdd[l], sizeof(float) * 2 * nn) || dalloc(&s->kafw[l], 32 * nn)
       || cudaMemcpy(s->kd[l], kk[l], sizeof(double) * nn, cudaMemcpyHostToDevice)
       || cudaMemcpy(s->kf[l], f, sizeof(float) * nn, cudaMemcpyHostToDevice)
       || cudaMemcpy(s->kdd[l], p, sizeof(float) * 2 * nn, cudaMemcpyHostToDevice)
       || mxk_afw_factors(n, s->kf[l], 1.0, 1.0, s->kafw[l], s->st) || cudaStreamSynchronize(s->st)) {
      free(f); free(p);
      for(; l <= o->L; l++) free(kk[l]);
      goto fail;
    }
    free(f); free(p);
  }
  for(l = 0; l <= o->L; l++) free(kk[l]);
  for(l = 0; l <= o->L; l++)
    if(dalloc(&s->b[l], elen(s, l) * es_g) || dalloc(&s->x[l], elen(s, l) * es_g) || dalloc(&s->d[l], elen(s, l) * es_g)
       || dalloc(&s->bg[l], nlen(s, l) * es_g) || dalloc(&s->xg[l], nlen(s, l) * es_g)
       || dalloc(&s->dg[l], nlen(s, l) * es_g))
      goto fail;
  if(dalloc((void **) &s->ph, mxk_phase_bytes(K)) || dalloc((void **) &s->ph2, mxk_phase_bytes(K))
     || dalloc((void **) &s->gamma, sizeof(int) * K)
     || dalloc((void **) &s->ae_inv, sizeof(double) * 2 * (size_t) N0e * N0e * K)
     || dalloc((void **) &s->an_inv, sizeof(double) * 2 * (size_t) N0n * N0n * K)
     || dalloc(&s->ae_inv_f, sizeof(float) * 2 * (size_t) N0e * N0e * K)
     || dalloc(&s->an_inv_f, sizeof(float) * 2 * (size_t) N0n * N0n * K)
     || dalloc(&s->E, elen(s, o->L) * es_e) || dalloc(&s->En, elen(s, o->L) * es_e)
     || dalloc(&s->Eprev[0], elen(s, o->L) * es_e)
     || (s->order > 1 && dalloc(&s->Eprev[1], elen(s, o->L) * es_e))
     || (s->order > 2 && dalloc(&s->Eprev[2], elen(s, o->L) * es_e))
     || (o->refine && dalloc(&s->Eref, elen(s, o->L) * es_e))
     || dalloc(&s->P, elen(s, o->L) * es_g) || dalloc(&s->Pn, elen(s, o->L) * es_g)
     || dalloc((void **) &s->ga, sizeof(double) * 2 * ns * ns * K) || dalloc((void **) &s->gm, sizeof(double) * 2 * ns * ns * K)
     || dalloc((void **) &s->coef, sizeof(double) * 2 * ns * m * K) || dalloc((void **) &s->theta, sizeof(double) * m * K)
     || dalloc((void **) &s->rwork, sizeof(double) * mxk_ritz_work_doubles(ns) * K)
     || dalloc((void **) &s->mu, sizeof(double) * m * K) || dalloc((void **) &s->stats, sizeof(double) * NSTAT * m * K)
     || dalloc((void **) &s->sel, sizeof(int) * ns * K) || dalloc((void **) &s->info, sizeof(int) * K)
     || dalloc((void **) &s->cA, sizeof(double) * 2 * (size_t) N0e * N0e * K)
     || dalloc((void **) &s->cM, sizeof(double) * 2 * (size_t) N0e * N0e * K)
     || dalloc((void **) &s->ccoef, sizeof(double) * 2 * (size_t) N0e * N0e * K)
     || dalloc((void **) &s->ctheta, sizeof(double) * (size_t) N0e * K)
     || dalloc((void **) &s->cwork, sizeof(double) * mxk_ritz_work_doubles(N0e) * K)
     || dalloc((void **) &s->cinfo, sizeof(int) * K)
     || dalloc((void **) &s->cacc, sizeof(double) * 4 * K * m)
     || dalloc(&s->combw, (size_t) 16 * ns * m * K))
    goto fail;
  s->E0 = s->E;
  s->P0 = s->P;
  s->gscratch_bytes = (size_t) K * 256 * (ns * (ns + 1) / 2) * 4 * sizeof(double);
  if(s->gscratch_bytes > ((size_t) 1 << 30)) s->gscratch_bytes = (size_t) 1 << 30;
  if(dalloc((void **) &s->gscratch, s->gscratch_bytes)) goto fail;
  s->h_ph = malloc(mxk_phase_bytes(K));
  s->h_stats = malloc(sizeof(double) * NSTAT * m * K);
  s->h_mu = malloc(sizeof(double) * m * K);
  s->h_res = malloc(sizeof(double) * m * K);
  s->h_rq = malloc(sizeof(double) * m * K);
  s->h_sel = malloc(sizeof(int) * ns * K);
  s->h_info = malloc(sizeof(int) * K);
  s->h_conv = malloc(sizeof(int) * K);
  s->h_steps = malloc(sizeof(int) * K);
  /* diagnostics only, read once here: none of them changes a result */
  s->timing = getenv("MXG_TIMING") != 0;
  s->graphs = getenv("MXG_NO_GRAPHS") == 0;
  s->debug = getenv("MXG_DEBUG") != 0;
  /* MXG_PROFILE_STEP=q brackets finest-level block step q of the first wave
   * with cudaProfilerStart/Stop, for a profiler started with profiling off */
  s->prof_step = getenv("MXG_PROFILE_STEP") ? atoi(getenv("MXG_PROFILE_STEP")) : -1;
  if(s->timing) {
    int q;
    for(q = 0; q <= PH_N; q++) cudaEventCreate(&s->tev[q]);
  }
  return s;
fail:
  mxg_solver_free(s);
  return 0;
}

/* ------------------------------------------------------------------ */

/* k = 0 up to rounding: the same rule as the coarse node matrix's fixnull
 * shift (|xf - 1| + |yf - 1| < 1e-8 in the 1-norm of the components) */
static int is_gamma(mxg_field xf, mxg_field yf)
{
  return fabs(creal(xf) - 1.0) + fabs(cimag(xf)) + fabs(creal(yf) - 1.0) + fabs(cimag(yf)) < 1e-8;
}

static int set_bloch(mxg_solver *s, int K, const mxg_field *xf, const mxg_field *yf)
{
  int k, *g = malloc(sizeof(int) * s->K), e;
  for(k = 0; k < s->K; k++) {
    int q = k < K ? k : K - 1;   /* unused slots repeat the last k-point */
    s->h_ph[4 * k] = creal(xf[q]); s->h_ph[4 * k + 1] = cimag(xf[q]);
    s->h_ph[4 * k + 2] = creal(yf[q]); s->h_ph[4 * k + 3] = cimag(yf[q]);
    g[k] = is_gamma(xf[q], yf[q]);
  }
  s->wave_gamma = 0;
  for(k = 0; k < K; k++) s->wave_gamma |= g[k];
  mxk_phase_fill(s->K, s->h_ph);
  e = (int) cudaMemcpyAsync(s->ph, s->h_ph, mxk_phase_bytes(s->K), cudaMemcpyHostToDevice, s->st);
  if(!e) e = (int) cudaMemcpyAsync(s->gamma, g, sizeof(int) * s->K, cudaMemcpyHostToDevice, s->st);
  if(!e) e = (int) cudaStreamSynchronize(s->st);
  free(g);
  return e;
}

/* coarse solvers: explicit inverses of (A+M) on level 0 and of the nodal
 * Laplace with the k = 0 shift (exp_bloch2d.c:520-528, 799-809) */
static int factor_coarse(mxg_solver *s)
{
  int N0e = 2 * s->n0 * s->n0, N0n = s->n0 * s->n0, k;
  L_(mxk_dense_edge(s->n0, s->K, s->ph, kap(s, 0), 1.0, 1.0, s->ae_inv, s->st));
  L_(mxk_hpd_inverse(N0e, s->K, s->ae_inv, s->info, s->st));
  TRY((int) cudaMemcpyAsync(s->h_info, s->info, sizeof(int) * s->K, cudaMemcpyDeviceToHost, s->st));
  TRY((int) cudaStreamSynchronize(s->st));
  for(k = 0; k < s->K; k++)
    if(s->h_info[k]) return MXG_ECONV;
  L_(mxk_dense_node(s->n0, s->K, s->ph, 1, s->an_inv, s->st));
  L_(mxk_hpd_inverse(N0n, s->K, s->an_inv, s->info, s->st));
  TRY((int) cudaMemcpyAsync(s->h_info, s->info, sizeof(int) * s->K, cudaMemcpyDeviceToHost, s->st));
  TRY((int) cudaStreamSynchronize(s->st));
  for(k = 0; k < s->K; k++)
    if(s->h_info[k]) return MXG_ECONV;
  L_(mxk_convert(MX_C128, s->ae_inv, MX_C64, s->ae_inv_f, (size_t) N0e * N0e * s->K, s->st));
  L_(mxk_convert(MX_C128, s->an_inv, MX_C64, s->an_inv_f, (size_t) N0n * N0n * s->K, s->st));
  return 0;
}

static void prof_flush(mxg_solver *s)
{
  int q;
  cudaEventSynchronize(s->pev[s->npev > 0 ? s->npev - 1 : 0]);
  for(q = 0; q + 1 < s->npev; q += 2) {
    float ms = 0.0f;
    int t = s->ptag[q / 2];
    cudaEventElapsedTime(&ms, s->pev[q], s->pev[q + 1]);
    s->prof_ms[t] += ms;
    s->prof_bytes[t] += s->pbytes[q / 2];
    s->prof_count[t]++;
  }
  s->npev = 0;
}

/* brackets one launch sequence of kind `tag` at the finest level with a pair
 * of events when profiling is on; prof_end closes the pair */
static int prof_begin(mxg_solver *s, int l, int tag, double bytes)
{
  if(!s->prof || l != s->L) return 0;
  if(s->npev + 2 > s->maxpev) prof_flush(s);
  s->ptag[s->npev / 2] = tag;
  s->pbytes[s->npev / 2] = bytes;
  cudaEventRecord(s->pev[s->npev++], s->st);
  return 1;
}
static void prof_end(mxg_solver *s, int on)
{
  if(on) cudaEventRecord(s->pev[s->npev++], s->st);
}

/* one AFW sweep: x, b read once, x written once, kappa and the patch
 * factor table read once */
static int edge_gs(mxg_solver *s, int l, int dir)
{
  double nn = (double) s->n[l] * s->n[l];
  int on = prof_begin(s, l, MXG_KT_AFW, (double) elen(s, l) * 3.0 * mxk_elem_size(s->pg) + 36.0 * nn);
  int e;
  if(s->o.smoother)
    e = mxk_edge_gs_colour(s->n[l], s->m, s->K, s->ph, kap(s, l), 1.0, 1.0, dir, s->pg, s->b[l], s->x[l], s->st);
  else
    e = mxk_edge_gs(s->n[l], s->m, s->K, s->ph, kap(s, l), 1.0, 1.0, dir, s->pg, s->b[l], s->x[l], s->st);
  s->launches += 2 * (dir == 2 ? 2 : 1);
  prof_end(s, on);
  return e;
}

/* one node Gauss-Seidel sweep (four row-group launches): x, b read once,
 * x written once */
static int node_gs(mxg_solver *s, int l, int dir)
{
  int on = prof_begin(s, l, MXG_KT_NODE_GS, (double) nlen(s, l) * 3.0 * mxk_elem_size(s->pg));
  int e = mxk_node_gs(s->n[l], s->m, s->K, s->ph, 1.0, dir, s->pg, s->bg[l], s->xg[l], s->st);
  s->launches += 4;
  prof_end(s, on);
  return e;
}

/* nu sweeps of one direction on level l: pairs of out-of-place sweeps
 * xg -> dg -> xg (dg is free while a level smooths), the rest in place */
static int node_smooth(mxg_solver *s, int l, int dir, int nu)
{
  int i = 0;
  if(mxk_node_gs_oop_ok(s->n[l], s->m, s->pg))
    for(; i + 2 <= nu; i += 2) {
      int on = prof_begin(s, l, MXG_KT_NODE_GS, (double) nlen(s, l) * 6.0 * mxk_elem_size(s->pg));
      int e = mxk_node_gs_oop(s->n[l], s->m, s->K, s->ph, 1.0, dir, s->pg, s->bg[l], s->xg[l], s->dg[l], s->st);
      if(!e) e = mxk_node_gs_oop(s->n[l], s->m, s->K, s->ph, 1.0, dir, s->pg, s->bg[l], s->dg[l], s->xg[l], s->st);
      s->launches += 6;
      prof_end(s, on);
      if(e) return e;
    }
  for(; i < nu; i++)
    TRY(node_gs(s, l, dir));
  return 0;
}

/* vcycle_edge2d (edge2d.c:5707-5754) on b[top], x[top] with the coarse inverse */
static int vcycle_e(mxg_solver *s, int top)
{
  int l, i, nu = s->o.smoother_steps, m = s->m, K = s->K, pg = s->pg;
  for(l = top; l > 0; l--) {
    int n = s->n[l];
    for(i = 0; i < nu; i++)
      TRY(edge_gs(s, l, 0));
    L_(mxk_edge_apply(n, m, K, s->ph, kap(s, l), -1.0, -1.0, 0, 1.0, pg, s->x[l], pg, s->b[l], s->d[l], s->st));
    L_(mxk_zero(pg, s->b[l - 1], elen(s, l - 1), s->st));
    L_(mxk_edge_restrict(n / 2, m, K, s->ph, 1.0, pg, s->d[l], s->b[l - 1], s->st));
    L_(mxk_zero(pg, s->x[l - 1], elen(s, l - 1), s->st));
  }
  L_(mxk_coarse_apply(2 * s->n0 * s->n0, m, K, s->ae_inv, s->ae_inv_f, pg, s->b[0], s->x[0], s->st));
  for(l = 1; l <= top; l++) {
    int n = s->n[l];
    L_(mxk_edge_prolong(n / 2, m, K, s->ph, 1.0, pg, s->x[l - 1], s->x[l], s->st));
    for(i = 0; i < nu; i++)
      TRY(edge_gs(s, l, 1));
  }
  return 0;
}

/* vcycle_node2d (node2d.c:1352-1389) on bg[top], xg[top] */
static int vcycle_n(mxg_solver *s, int top)
{
  int l, nu = s->o.smoother_steps, m = s->m, K = s->K, pg = s->pg;
  for(l = top; l > 0; l--) {
    int n = s->n[l];
    TRY(node_smooth(s, l, 0, nu));
    /* the residual and its restriction in one kernel (written, not added) */
    L_(mxk_node_residual_restrict(n / 2, m, K, s->ph, 1.0, pg, s->xg[l], s->bg[l], s->bg[l - 1], s->st));
    L_(mxk_zero(pg, s->xg[l - 1], nlen(s, l - 1), s->st));
  }
  L_(mxk_coarse_apply(s->n0 * s->n0, m, K, s->an_inv, s->an_inv_f, pg, s->bg[0], s->xg[0], s->st));
  for(l = 1; l <= top; l++) {
    int n = s->n[l];
    L_(mxk_node_prolong(n / 2, m, K, s->ph, 1.0, pg, s->xg[l - 1], s->xg[l], s->st));
    TRY(node_smooth(s, l, 1, nu));
  }
  return 0;
}

/* gradient lifting (exp_bloch2d.c:971-978): y -= G L^-1 G^H M y */
/* Runs body(s, l) on the solver's stream through a CUDA graph of level l:
 * captured at the first call, replayed afterwards (every pointer the bodies
 * use is fixed for the solver's lifetime).  With profiling on, or if the
 * capture fails, the body launches directly. */
static int run_graphed(mxg_solver *s, int l, cudaGraphExec_t *exec, long *nlaunch,
                       int (*body)(mxg_solver *, int))
{
  cudaGraph_t g = 0;
  long before;
  int e;
  if(!s->graphs || s->prof) return body(s, l);
  if(!*exec) {
    if(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      s->graphs = 0;
      return body(s, l);
    }
    before = s->launches;
    e = body(s, l);
    if(cudaStreamEndCapture(s->st, &g) != cudaSuccess || e || !g
       || cudaGraphInstantiate(exec, g, 0) != cudaSuccess) {
      if(g) cudaGraphDestroy(g);
      *exec = 0;
      cudaGetLastError();
      s->graphs = 0;
      s->launches = before;
      return body(s, l);
    }
    cudaGraphDestroy(g);
    *nlaunch = s->launches - before;
    s->launches = before;
  }
  s->launches += *nlaunch;
  return (int) cudaGraphLaunch(*exec, s->st);
}

static int lift_body(mxg_solver *s, int l)
{
  int i;
  L_(mxk_zero(s->pg, s->xg[l], nlen(s, l), s->st));
  for(i = 0; i < s->o.gradient_steps; i++)
    TRY(vcycle_n(s, l));
  return 0;
}

static int lift(mxg_solver *s, int l, int py, void *y)
{
  int n = s->n[l];
  if(s->o.gradient_steps <= 0) return 0;
  L_(mxk_adjgradient(n, s->m, s->K, s->ph, 1.0, 1, 0.0, py, y, s->pg, s->bg[l], s->st));
  TRY(run_graphed(s, l, &s->glift[l], &s->glift_n[l], lift_body));
  L_(mxk_gradient(n, s->m, s->K, s->ph, -1.0, s->pg, s->xg[l], py, y, s->st));
  return 0;
}

/* hcycle_edge2d (edge2d.c:5756-5823) on b[top], x[top]: point Gauss-Seidel
 * plus a correction in the gradients on every level (the node vectors of
 * the lifting serve as its work space) */
static int hcycle_e(mxg_solver *s, int top)
{
  int l, i, nu = s->o.smoother_steps, m = s->m, K = s->K, pg = s->pg;
  for(l = top; l >= 1; l--) {
    int n = s->n[l];
    for(i = 0; i < nu; i++)
      L_(mxk_edge_gs_point(n, m, K, s->ph, kap(s, l), 1.0, 1.0, 0, pg, s->b[l], s->x[l], s->st));
    L_(mxk_edge_apply(n, m, K, s->ph, kap(s, l), -1.0, -1.0, 0, 1.0, pg, s->x[l], pg, s->b[l], s->d[l], s->st));
    L_(mxk_adjgradient(n, m, K, s->ph, 1.0, 0, 0.0, pg, s->d[l], pg, s->bg[l], s->st));
    L_(mxk_zero(pg, s->xg[l], nlen(s, l), s->st));
    TRY(node_smooth(s, l, 0, nu));
    L_(mxk_gradient(n, m, K, s->ph, 1.0, pg, s->xg[l], pg, s->x[l], s->st));
    L_(mxk_edge_apply(n, m, K, s->ph, kap(s, l), -1.0, -1.0, 0, 1.0, pg, s->x[l], pg, s->b[l], s->d[l], s->st));
    L_(mxk_zero(pg, s->b[l - 1], elen(s, l - 1), s->st));
    L_(mxk_edge_restrict(n / 2, m, K, s->ph, 1.0, pg, s->d[l], s->b[l - 1], s->st));
    L_(mxk_zero(pg, s->x[l - 1], elen(s, l - 1), s->st));
  }
  L_(mxk_coarse_apply(2 * s->n0 * s->n0, m, K, s->ae_inv, s->ae_inv_f, pg, s->b[0], s->x[0], s->st));
  for(l = 1; l <= top; l++) {
    int n = s->n[l];
    L_(mxk_edge_prolong(n / 2, m, K, s->ph, 1.0, pg, s->x[l - 1], s->x[l], s->st));
    L_(mxk_edge_apply(n, m, K, s->ph, kap(s, l), -1.0, -1.0, 0, 1.0, pg, s->x[l], pg, s->b[l], s->d[l], s->st));
    L_(mxk_adjgradient(n, m, K, s->ph, 1.0, 0, 0.0, pg, s->d[l], pg, s->bg[l], s->st));
    L_(mxk_zero(pg, s->xg[l], nlen(s, l), s->st));
    TRY(node_smooth(s, l, 1, nu));
    L_(mxk_gradient(n, m, K, s->ph, 1.0, pg, s->xg[l], pg, s->x[l], s->st));
    for(i = 0; i < nu; i++)
      L_(mxk_edge_gs_point(n, m, K, s->ph, kap(s, l), 1.0, 1.0, 1, pg, s->b[l], s->x[l], s->st));
  }
  return 0;
}

static int precondition_body(mxg_solver *s, int l)
{
  int i;
  L_(mxk_zero(s->pg, s->x[l], elen(s, l), s->st));
  for(i = 0; i < s->o.prec_steps; i++)
    TRY(s->o.smoother == 2 ? hcycle_e(s, l) : vcycle_e(s, l));
  return 0;
}

/* x[l] = V^prec b[l] from zero */
static int precondition(mxg_solver *s, int l)
{
  return run_graphed(s, l, &s->gpre[l], &s->gpre_n[l], precondition_body);
}

/* residual of E (rhs for the preconditioner into b[l]) and its statistics;
 * host: residual norms, Rayleigh quotients, convergence per k */
static int residual(mxg_solver *s, int l, int write_rhs)
{
  int k, i, m = s->m, K = s->K;
  TRY((int) cudaMemsetAsync(s->stats, 0, sizeof(double) * NSTAT * m * K, s->st));
  L_(mxk_block_residual(s->n[l], m, K, s->ph, kap(s, l), s->mu, s->pe, s->E, s->pg,
                        write_rhs ? s->b[l] : 0, s->stats, s->st));
  TRY((int) cudaMemcpyAsync(s->h_stats, s->stats, sizeof(double) * NSTAT * m * K, cudaMemcpyDeviceToHost, s->st));
  if(s->ritz_pending) {
    /* the Ritz step before this residual: its status and Ritz values (the
     * shifts mu the residual was formed with) come back with the statistics */
    TRY((int) cudaMemcpyAsync(s->h_info, s->info, sizeof(int) * K, cudaMemcpyDeviceToHost, s->st));
    TRY((int) cudaMemcpyAsync(s->h_mu, s->mu, sizeof(double) * m * K, cudaMemcpyDeviceToHost, s->st));
  }
  TRY((int) cudaStreamSynchronize(s->st));
  if(s->ritz_pending) {
    s->ritz_pending = 0;
    for(k = 0; k < K; k++)
      if(s->h_info[k] < m) return MXG_ECONV;
  }
  for(k = 0; k < K; k++)
    for(i = 0; i < m; i++) {
      const double *st = s->h_stats + ((size_t) k * m + i) * NSTAT;
      double mu = s->h_mu[k * m + i];
      double r = sqrt(st[0] > 0.0 ? st[0] : 0.0);
      if(s->o.relative) r /= fabs(mu) * sqrt(st[1]) + 1e-300;
      s->h_res[k * m + i] = r;
      s->h_rq[k * m + i] = st[2] / st[3];
    }
  return 0;
}

static int converged_k(const mxg_solver *s, int k)
{
  int i;
  for(i = 0; i < s->o.ieigs; i++)
    if(!(s->h_res[k * s->m + i] <= s->cur_tol))
      return 0;
  return 1;
}

static int upload_mu(mxg_solver *s)
{
  return (int) cudaMemcpyAsync(s->mu, s->h_mu, sizeof(double) * s->m * s->K, cudaMemcpyHostToDevice, s->st);
}

static void swapp(void **a, void **b)
{
  void *t = *a;
  *a = *b;
  *b = t;
}

/* The launches of one Ritz step on the blocks of s->rb: Gram matrices,
 * column selection from the last residual statistics (soft locking),
 * Rayleigh-Ritz by Cholesky-QR and Jacobi, the Ritz values as the next
 * shifts mu, and the combinations into En (and Pn).  No host decision sits
 * between them, so the sequence is captured as one CUDA graph. */
static int ritz_body(mxg_solver *s, int l)
{
  const int nb = s->rb.nb, m = s->m, K = s->K, ns = nb * m;
  const int *pr = s->rb.pr;
  const void *const *pp = s->rb.pp;
  /* the residual of E sits in b[l] (written by residual()) with the Ritz
   * values mu; the mixed solver forms the E-to-search-block entries from it */
  const void *rr = (s->pg == MX_C64 && nb > 1) ? s->b[l] : 0;
  int tm = s->timing && l == s->L && nb > 1, on, b;
  double gbytes = 12.0 * s->n[l] * s->n[l];   /* kappa as float and float-float pair */
  for(b = 0; b < nb; b++) gbytes += (double) elen(s, l) * mxk_elem_size(pr[b]);
  if(rr) gbytes += (double) elen(s, l) * 8.0;
  on = prof_begin(s, l, MXG_KT_GRAM, gbytes);
  L_(mxk_block_gram(s->n[l], m, K, s->ph, kap(s, l), nb, pr, pp, rr, s->mu, s->ga, s->gm, s->gscratch,
                    s->gscratch_bytes, s->st));
  s->launches++;   /* the reduction of the partial sums */
  prof_end(s, on);
  L_(mxk_select_columns(ns, m, K, s->stats, s->mu, s->cur_tol, s->o.relative, s->all_columns, s->sel, s->st));
  if(tm) cudaEventRecord(s->tev[PH_RR], s->st);
  L_(mxk_rayleigh_ritz(ns, m, K, s->ga, s->gm, s->sel, s->rb.drop, s->rb.theta_min, s->coef, s->theta, s->info,
                       s->rwork, s->st));
  TRY((int) cudaMemcpyAsync(s->mu, s->theta, sizeof(double) * m * K, cudaMemcpyDeviceToDevice, s->st));
  if(tm) cudaEventRecord(s->tev[PH_COMB], s->st);
  if(s->rb.with_p)
    L_(mxk_block_combine(s->n[l], m, K, nb - 1, pr + 1, pp + 1, s->coef, ns, m, s->combw, s->pg, s->Pn, s->st));
  L_(mxk_block_combine(s->n[l], m, K, nb, pr, pp, s->coef, ns, 0, s->combw, s->pe, s->En, s->st));
  return 0;
}

/* Rayleigh-Ritz on the nb blocks (precisions pr, pointers pp) -> coef, theta
 * with soft locking of converged columns; writes the new E (and P).  The
 * step's status (a rank-deficient basis) and its Ritz values reach the host
 * with the next residual(). */
static int ritz(mxg_solver *s, int l, int nb, const int *pr, const void *const *pp, int with_p, double drop,
                double theta_min)
{
  int q;
  s->rb.nb = nb;
  s->rb.with_p = with_p;
  for(q = 0; q < nb; q++) { s->rb.pr[q] = pr[q]; s->rb.pp[q] = pp[q]; }
  s->rb.drop = drop;
  s->rb.theta_min = theta_min;
  if(s->timing || s->all_columns)
    TRY(ritz_body(s, l));
  else {
    int pe = s->E != s->E0, pq = s->P != s->P0;
    TRY(run_graphed(s, l, &s->gritz[l][nb - 1][pe][pq], &s->gritz_n[l][nb - 1][pe][pq], ritz_body));
  }
  s->ritz_pending = 1;
  swapp(&s->E, &s->En);
  if(with_p) swapp(&s->P, &s->Pn);
  return 0;
}

/* pivot^2 below which Cholesky-QR drops a column of the Ritz basis
 * (mxg_solve_opts.drop, or the default of the precision) */
static double drop_tol(const mxg_solver *s)
{
  if(s->o.drop > 0.0) return s->o.drop;
  return s->o.precision ? 1e-6 : 1e-12;
}

/* one block step at level l; on entry b[l] holds the residual of E */
static int block_step(mxg_solver *s, int l, int *have_p)
{
  int m = s->m;
  size_t len = elen(s, l);
  if(s->o.method == 0) {
    /* PINVIT: e -= V(defect); center; lift; Ritz on the block */
    int pr[1];
    const void *pp[1];
    TRY(precondition(s, l));
    L_(mxk_axpy(-1.0, 0.0, s->pg, s->x[l], s->pe, s->E, len, s->st));
    if(s->o.center) L_(mxk_center(s->n[l], m, s->K, s->gamma, s->pe, s->E, s->cacc, s->st));
    TRY(lift(s, l, s->pe, s->E));
    pr[0] = s->pe; pp[0] = s->E;
    return ritz(s, l, 1, pr, pp, 0, 1e-14, -1e300);
  }
  else {
    int pr[3], nb;
    const void *pp[3];
    int tm = s->timing && l == s->L;
    if(tm) cudaEventRecord(s->tev[PH_PREC], s->st);
    TRY(precondition(s, l));
    if(tm) cudaEventRecord(s->tev[PH_LIFTX], s->st);
    if(s->o.center) L_(mxk_center(s->n[l], m, s->K, s->gamma, s->pg, s->x[l], s->cacc, s->st));
    TRY(lift(s, l, s->pg, s->x[l]));
    if(tm) cudaEventRecord(s->tev[PH_GRAM], s->st);
    pr[0] = s->pe; pp[0] = s->E;
    pr[1] = s->pg; pp[1] = s->x[l];
    pr[2] = s->pg; pp[2] = s->P;
    nb = *have_p ? 3 : 2;
    /* mu = 1 + lambda: pairs with lambda <= 1e-7 are gradient (null-space)
     * modes that the search directions' rounding can expose */
    /* the refinement step's basis holds the search columns of converged
     * pairs too, nearly dependent on their eigenvectors: it drops columns
     * more readily */
    TRY(ritz(s, l, nb, pr, pp, 1, s->all_columns && drop_tol(s) < 1e-4 ? 1e-4 : drop_tol(s), 1.0 + 1e-7));
    if(tm) cudaEventRecord(s->tev[PH_LIFTE], s->st);
    *have_p = 1;
    if(s->o.lift_e) {
      if(s->o.center) L_(mxk_center(s->n[l], m, s->K, s->gamma, s->pe, s->E, s->cacc, s->st));
      TRY(lift(s, l, s->pe, s->E));
    }
    if(tm) cudaEventRecord(s->tev[PH_RESID], s->st);
    return 0;
  }
}

/* iterate at level l until all k converge or maxsteps; counts steps per k */
static int iterate(mxg_solver *s, int l, int maxsteps, int K_active)
{
  int step, k, have_p = 0, all;
  /* the tolerance of this level: the nested iteration's own below the
   * finest level (fixed per level, so the level's Ritz graph may keep it) */
  s->cur_tol = l < s->L && s->o.nested_tol > 0.0 ? s->o.nested_tol : s->o.tol;
  for(k = 0; k < s->K; k++) s->h_steps[k] = 0;
  TRY(residual(s, l, 1));
  for(step = 0; step < maxsteps; step++) {
    all = 1;
    for(k = 0; k < K_active; k++) {
      s->h_conv[k] = converged_k(s, k);
      if(!s->h_conv[k]) { all = 0; s->h_steps[k] = step + 1; }
    }
    if(all) break;
    if(l == s->L && step == s->prof_step && !s->prof_done) cudaProfilerStart();
    TRY(block_step(s, l, &have_p));
    TRY(residual(s, l, 1));
    if(l == s->L && step == s->prof_step && !s->prof_done) {
      cudaProfilerStop();
      s->prof_done = 1;
    }
    if(s->timing && l == s->L && s->o.method == 1) {
      int q;
      cudaEventRecord(s->tev[PH_N], s->st);
      cudaEventSynchronize(s->tev[PH_N]);
      for(q = 0; q < PH_N; q++) {
        float ms = 0.0f;
        cudaError_t er = cudaEventElapsedTime(&ms, s->tev[q], s->tev[q + 1]);
        if(er != cudaSuccess) fprintf(stderr, "timing event %d: %s\n", q, cudaGetErrorString(er));
        s->tph[q] += ms;
      }
      cudaGetLastError();
    }
    if(s->debug) {
      int i;
      fprintf(stderr, "level %d step %d rank %d:", l, step, s->h_info[0]);
      for(i = 0; i < s->m; i++) fprintf(stderr, " %.1e", s->h_res[i]);
      fprintf(stderr, "\n");
    }
  }
  for(k = 0; k < K_active; k++)
    if(!converged_k(s, k)) s->h_steps[k] = maxsteps;
  if(l == s->L && s->o.refine) {
    /* the refinement sweep: one more block step with every column of the
     * search blocks in the Ritz basis, then the residuals again.  A k-point
     * whose wanted pairs come out worse keeps its block from before (the
     * sweep is kept per k-point, on the device) */
    double *before = malloc(sizeof(double) * 2 * s->K * s->m);
    int worse = 0, e;
    if(!before) return MXG_ENOMEM;
    memcpy(before, s->h_res, sizeof(double) * s->K * s->m);
    memcpy(before + s->K * s->m, s->h_rq, sizeof(double) * s->K * s->m);
    L_(mxk_convert(s->pe, s->E, s->pe, s->Eref, elen(s, l), s->st));
    s->all_columns = 1;
    TRY(block_step(s, l, &have_p));
    s->all_columns = 0;
    e = residual(s, l, 1);
    if(e && e != MXG_ECONV) { free(before); return e; }
    for(k = 0; k < K_active; k++) {
      double b0 = 0.0, b1 = 0.0;
      int i;
      for(i = 0; i < s->o.ieigs; i++) {
        double r0 = before[k * s->m + i], r1 = s->h_res[k * s->m + i];
        if(r0 > b0) b0 = r0;
        if(!(r1 <= b1)) b1 = r1;   /* NaN counts as worst */
      }
      if(e == MXG_ECONV || !(b1 <= b0)) {
        /* restore the pre-sweep block of this k-point and its statistics */
        const size_t slot = elen(s, l) / s->K * mxk_elem_size(s->pe);
        worse = (int) cudaMemcpyAsync((char *) s->E + k * slot, (const char *) s->Eref + k * slot, slot,
                                      cudaMemcpyDeviceToDevice, s->st);
        memcpy(s->h_res + k * s->m, before + k * s->m, sizeof(double) * s->m);
        memcpy(s->h_rq + k * s->m, before + s->K * s->m + k * s->m, sizeof(double) * s->m);
        if(worse) { free(before); return worse; }
      }
    }
    free(before);
  }
  return 0;
}

/* coarse generalized eigenproblem (exp_bloch2d.c:530-554) and the nested
 * iteration (exp_bloch2d.c:562-732) for every k of the wave */
static int cold_start(mxg_solver *s, int K_active)
{
  int N = 2 * s->n0 * s->n0, m = s->m, K = s->K, k, i, v, l;
  double *th = malloc(sizeof(double) * N * K), *cf = malloc(sizeof(double) * 2 * (size_t) N * N * K);
  double *e0 = malloc(sizeof(double) * 2 * (size_t) K * N * m);
  int e = 0;
  double t0 = now_s();
  L_(mxk_dense_edge(s->n0, K, s->ph, kap(s, 0), 1.0, 0.0, s->cA, s->st));
  L_(mxk_dense_edge(s->n0, K, s->ph, kap(s, 0), 0.0, 1.0, s->cM, s->st));
  L_(mxk_rayleigh_ritz(N, N, K, s->cA, s->cM, 0, 1e-14, -1e300, s->ccoef, s->ctheta, s->cinfo, s->cwork, s->st));
  e = (int) cudaMemcpyAsync(th, s->ctheta, sizeof(double) * N * K, cudaMemcpyDeviceToHost, s->st);
  if(!e) e = (int) cudaMemcpyAsync(cf, s->ccoef, sizeof(double) * 2 * (size_t) N * N * K, cudaMemcpyDeviceToHost, s->st);
  if(!e) e = (int) cudaStreamSynchronize(s->st);
  if(e) { free(th); free(cf); free(e0); return e; }
  if(s->timing) fprintf(stderr, "  coarse eigenproblem %.3f s\n", now_s() - t0);
  /* skip |lambda| < 1e-8 (exp_bloch2d.c:546-551); level-0 block layout of
   * one k is row-major N x m */
  for(k = 0; k < K; k++) {
    int ev;
    for(ev = 0; ev < N && fabs(th[k * N + ev]) < 1e-8; ev++)
      ;
    if(ev + m > N) { free(th); free(cf); free(e0); return MXG_ECONV; }
    for(v = 0; v < m; v++) {
      s->h_mu[k * m + v] = 1.0 + th[k * N + ev + v];
      for(i = 0; i < N; i++) {
        const double *z = cf + 2 * ((size_t) k * N * N + (size_t) (ev + v) * N + i);
        double *q = e0 + 2 * (((size_t) k * N + i) * m + v);
        q[0] = z[0]; q[1] = z[1];
      }
    }
  }
  /* upload as the level-0 E */
  {
    size_t tot = (size_t) K * N * m, o;
    if(s->pe == MX_C128)
      e = (int) cudaMemcpy(s->E, e0, sizeof(double) * 2 * tot, cudaMemcpyHostToDevice);
    else {
      float *f = malloc(sizeof(float) * 4 * tot);
      for(o = 0; o < tot; o++) {
        double re = e0[2 * o], im = e0[2 * o + 1];
        f[4 * o] = (float) re; f[4 * o + 1] = (float) (re - (double) f[4 * o]);
        f[4 * o + 2] = (float) im; f[4 * o + 3] = (float) (im - (double) f[4 * o + 2]);
      }
      e = (int) cudaMemcpy(s->E, f, sizeof(float) * 4 * tot, cudaMemcpyHostToDevice);
      free(f);
    }
  }
  free(th); free(cf); free(e0);
  if(e) return e;
  TRY(upload_mu(s));
  for(l = 1; l <= s->L; l++) {
    L_(mxk_zero(s->pe, s->En, elen(s, l), s->st));
    L_(mxk_edge_prolong(s->n[l - 1], m, K, s->ph, 1.0, s->pe, s->E, s->En, s->st));
    swapp(&s->E, &s->En);
    /* Rayleigh quotients of the prolongated vectors (exp_bloch2d.c:567-583) */
    TRY(residual(s, l, 0));
    for(k = 0; k < K * m; k++) s->h_mu[k] = s->h_rq[k];
    TRY(upload_mu(s));
    t0 = now_s();
    TRY(iterate(s, l, l == s->L ? s->o.max_steps : s->o.max_nested, K_active));
    if(s->timing) {
      cudaStreamSynchronize(s->st);
      fprintf(stderr, "  level %d (n = %d): %.3f s\n", l, s->n[l], now_s() - t0);
    }
  }
  return 0;
}

/* The start block of a warm-started wave.  With np = min(order, stored
 * waves) > 1 it is the Rayleigh-Ritz extrapolation of exp_bloch2d.c:814-895
 * ('1': np = 2, '2': np = 3): Gram matrices of the basis [E_{w-1} .. E_{w-np}]
 * (np*m columns per k-point) under this wave's operators, Cholesky-QR and
 * the Ritz eigenproblem (the reference orthonormalises by Householder and
 * calls zheev), and E = basis * the lowest m Ritz vectors.  Ritz values at
 * or below the null space (lambda <= 1e-7) are skipped; a k-point whose
 * basis cannot supply m Ritz vectors falls back to its previous wave's
 * eigenvectors. */
static int extrapolate(mxg_solver *s)
{
  int np = s->have_prev < s->order ? s->have_prev : s->order, K = s->K, m = s->m, ns, k, j, q, bad = 0;
  int pr[3];
  const void *pp[3];
  if(np <= 1) {
    L_(mxk_convert(s->pe, s->Eprev[0], s->pe, s->E, elen(s, s->L), s->st));
    return 0;
  }
  ns = np * m;
  for(q = 0; q < np; q++) { pr[q] = s->pe; pp[q] = s->Eprev[q]; }
  L_(mxk_block_gram(s->n[s->L], m, K, s->ph, kap(s, s->L), np, pr, pp, 0, 0, s->ga, s->gm, s->gscratch,
                    s->gscratch_bytes, s->st));
  s->launches++;
  for(k = 0; k < K; k++)
    for(j = 0; j < ns; j++) s->h_sel[k * ns + j] = 1;
  TRY((int) cudaMemcpyAsync(s->sel, s->h_sel, sizeof(int) * ns * K, cudaMemcpyHostToDevice, s->st));
  L_(mxk_rayleigh_ritz(ns, m, K, s->ga, s->gm, s->sel, drop_tol(s), 1.0 + 1e-7, s->coef, s->theta, s->info,
                       s->rwork, s->st));
  TRY((int) cudaMemcpyAsync(s->h_info, s->info, sizeof(int) * K, cudaMemcpyDeviceToHost, s->st));
  TRY((int) cudaStreamSynchronize(s->st));
  for(k = 0; k < K; k++)
    if(s->h_info[k] < m) bad = 1;
  if(bad) {
    L_(mxk_convert(s->pe, s->Eprev[0], s->pe, s->E, elen(s, s->L), s->st));
    return 0;
  }
  L_(mxk_block_combine(s->n[s->L], m, K, np, pr, pp, s->coef, ns, 0, s->combw, s->pe, s->E, s->st));
  return 0;
}

int mxg_bloch_solve(mxg_solver *s, int nk, const mxg_field *xf, const mxg_field *yf, double *lambda,
                    int *steps, double *res)
{
  int w, k, i, m = s->m, K = s->K;
  float ms;
  double total = 0.0;
  TRY((int) cudaSetDevice(s->device));
  s->launches = 0;
  s->restarts = 0;
  s->have_prev = 0;   /* every call starts cold; later waves of this call start warm */
  for(w = 0; w * K < nk; w++) {
    int k0 = w * K, Ka = nk - k0 < K ? nk - k0 : K, after_gamma = s->wave_gamma;
    TRY(set_bloch(s, Ka, xf + k0, yf + k0));
    TRY((int) cudaEventRecord(s->ev0, s->st));
    TRY(factor_coarse(s));
    /* a wave after one holding Gamma starts cold: the Gamma block is centred
     * and lacks the two lowest bands of every k != 0 (they tend to the
     * constant fields that centring removes) */
    if(!s->have_prev || s->K_prev != K || s->o.extrapolation == 'c' || after_gamma) {
      double tc = now_s();
      TRY(cold_start(s, Ka));
      if(s->timing) fprintf(stderr, "wave %d: cold start incl. finest-level steps %.3f s\n", w, now_s() - tc);
    }
    else {
      /* warm start from the same slot of the earlier waves
       * (exp_bloch2d.c:814-895): with one stored wave, or extrapolation
       * 'n', its eigenvectors; otherwise the lowest Ritz vectors of this
       * k-point's operator in the span of the stored waves' blocks.  They
       * are divergence-free for their own Bloch phases, not for these, so
       * they are lifted (and centred at Gamma) first */
      TRY(extrapolate(s));
      if(s->o.center) L_(mxk_center(s->n[s->L], m, s->K, s->gamma, s->pe, s->E, s->cacc, s->st));
      TRY(lift(s, s->L, s->pe, s->E));
      TRY(residual(s, s->L, 0));
      for(k = 0; k < K * m; k++) s->h_mu[k] = s->h_rq[k];
      TRY(upload_mu(s));
      TRY(iterate(s, s->L, s->o.max_steps, Ka));
      /* a warm start can fail where the wanted eigenvectors of the previous
       * wave resemble those of these k-points poorly (close to Gamma the
       * direction of k, and with it the splitting into gradient and
       * physical fields, turns quickly): such a wave is solved again from a
       * cold start */
      for(k = 0; k < Ka && converged_k(s, k); k++)
        ;
      if(k < Ka) {
        s->restarts++;
        TRY(cold_start(s, Ka));
      }
    }
    TRY((int) cudaEventRecord(s->ev1, s->st));
    TRY((int) cudaEventSynchronize(s->ev1));
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    total += ms;
    for(k = 0; k < Ka; k++) {
      if(steps) steps[k0 + k] = s->h_steps[k];
      for(i = 0; i < m; i++) {
        if(lambda) lambda[(size_t) (k0 + k) * m + i] = s->h_rq[k * m + i] - 1.0;
        if(res) res[(size_t) (k0 + k) * m + i] = s->h_res[k * m + i];
      }
    }
    {
      /* keep this wave's eigenvectors, the oldest stored wave gives way */
      void *t = s->Eprev[s->order - 1];
      int q;
      for(q = s->order - 1; q > 0; q--) s->Eprev[q] = s->Eprev[q - 1];
      s->Eprev[0] = t;
      L_(mxk_convert(s->pe, s->E, s->pe, s->Eprev[0], elen(s, s->L), s->st));
      if(s->have_prev < s->order) s->have_prev++;
    }
    s->K_prev = K;
  }
  s->last_ms = total;
  s->last_nk = nk;
  if(s->timing) {
    int q;
    if(s->restarts) fprintf(stderr, "%d warm-started wave(s) solved again cold\n", s->restarts);
    fprintf(stderr, "finest-level GPU time per phase:");
    for(q = 0; q < PH_N; q++) {
      fprintf(stderr, " %s %.3f s%s", ph_name[q], s->tph[q] / 1e3, q + 1 < PH_N ? "," : "\n");
      s->tph[q] = 0.0;
    }
  }
  return (int) cudaStreamSynchronize(s->st);
}

/* The full-zone surface of exp_blochsurf (exp_blochsurf.c:25-37, 964-1489):
 * k = (2 pi ix / (steps - 1) - pi, 2 pi iy / (steps - 1) - pi) for
 * ix, iy = 0 .. steps-1, solved in waves of the solver's K k-points taken in
 * row order (iy outer, ix inner).  Wave 0 starts cold; every later wave
 * starts from the same slots of the waves before it (extrapolate), slot i
 * holding the k-point K positions earlier on the grid -- K / steps rows
 * lower when K is a multiple of steps, so that with K = steps every k-point
 * is extrapolated from the same column of the rows below it, as the
 * reference's yext extrapolation (exp_blochsurf.c:332-406, 1066-1489).
 * Outputs are indexed (iy * steps + ix) as in mxg_bloch_solve. */
int mxg_bloch_surface(mxg_solver *s, int steps, double *lambda, int *nsteps, double *residual)
{
  int nk, ix, iy, e;
  mxg_field *xf, *yf;
  if(!s || steps < 2) return MXG_EINVAL;
  nk = steps * steps;
  xf = malloc(sizeof(mxg_field) * nk);
  yf = malloc(sizeof(mxg_field) * nk);
  if(!xf || !yf) { free(xf); free(yf); return MXG_ENOMEM; }
  for(iy = 0; iy < steps; iy++)
    for(ix = 0; ix < steps; ix++) {
      const double pi = 3.14159265358979323846;
      double xk = 2.0 * pi * ix / (steps - 1) - pi, yk = 2.0 * pi * iy / (steps - 1) - pi;
      xf[iy * steps + ix] = cos(xk) + I * sin(xk);
      yf[iy * steps + ix] = cos(yk) + I * sin(yk);
    }
  e = mxg_bloch_solve(s, nk, xf, yf, lambda, nsteps, residual);
  free(xf);
  free(yf);
  return e;
}

int mxg_solver_eigenvectors(const mxg_solver *s, mxg_field *host)
{
  size_t per = 2 * (size_t) s->n[s->L] * s->n[s->L], tot = (size_t) s->K * s->m * per, es = mxk_elem_size(s->pe);
  size_t k, v, e;
  unsigned char *buf = malloc(es * tot);
  double *h = (double *) host;
  int err = (int) cudaSetDevice(s->device);
  if(!err) err = (int) cudaMemcpy(buf, s->E, es * tot, cudaMemcpyDeviceToHost);
  for(k = 0; !err && k < (size_t) s->K; k++)
    for(v = 0; v < (size_t) s->m; v++)
      for(e = 0; e < per; e++) {
        size_t o = (k * per + e) * s->m + v;
        double *z = h + 2 * ((k * s->m + v) * per + e);
        if(s->pe == MX_C128) {
          z[0] = ((double *) buf)[2 * o]; z[1] = ((double *) buf)[2 * o + 1];
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

/* Relative residuals of the last solved wave recomputed in FP64: the
 * eigenvector block converted to complex128 (into the spare block En, of
 * the same size), then the residual statistics of the complex128 kernel --
 * (A+M) e, M e and r = (A+M) e - mu M e in double arithmetic -- with mu the
 * returned eigenvalues + 1 (the final Rayleigh quotients). */
int mxg_solver_check_fp64(mxg_solver *s, double *res)
{
  int k, i, m = s->m, K = s->K, l = s->L;
  TRY((int) cudaSetDevice(s->device));
  L_(mxk_convert(s->pe, s->E, MX_C128, s->En, elen(s, l), s->st));
  TRY((int) cudaMemcpyAsync(s->mu, s->h_rq, sizeof(double) * m * K, cudaMemcpyHostToDevice, s->st));
  TRY((int) cudaMemsetAsync(s->stats, 0, sizeof(double) * NSTAT * m * K, s->st));
  L_(mxk_block_residual(s->n[l], m, K, s->ph, kap(s, l), s->mu, MX_C128, s->En, MX_C128, 0, s->stats, s->st));
  TRY((int) cudaMemcpyAsync(s->h_stats, s->stats, sizeof(double) * NSTAT * m * K, cudaMemcpyDeviceToHost, s->st));
  TRY((int) cudaStreamSynchronize(s->st));
  for(k = 0; k < K; k++)
    for(i = 0; i < m; i++) {
      const double *st = s->h_stats + ((size_t) k * m + i) * NSTAT;
      double mu = s->h_rq[k * m + i];
      res[k * m + i] = sqrt(st[0] > 0.0 ? st[0] : 0.0) / (fabs(mu) * sqrt(st[1]) + 1e-300);
    }
  return upload_mu(s);
}

/* ------------------------------------------------------------------ */
/* eigenvector continuity and Chern partial sums (exp_bloch2d.c:1058-1216) */
/* ------------------------------------------------------------------ */

/* An adjustment of one k-point's block: adjusted vector i = d[i] * raw
 * vector perm[i] (a permutation with unit phases). */
typedef struct {
  int *perm;
  mxg_field *d;
} adjust_t;

/* entry (row a*m + i, column b*m + j) of one k-point's column-major
 * complex Gram matrix of ns columns: (block a, col i)^H M (block b, col j) */
static mxg_field gram_at(const double *g, int ns, int m, int a, int i, int b, int j)
{
  size_t o = 2 * ((size_t) (b * m + j) * ns + (size_t) (a * m + i));
  return g[o] + I * g[o + 1];
}

/* Mass Gram matrices of [E_l, E_{l-1}, E_{l-2}] under M(k_l) for the slots
 * l = l0 .. l0 + cnt - 1 (nb = 3, or 2 when l0 = 1: [E_1, E_0]), from the
 * complex128 copy of the block in En, with a phase table of just those
 * slots; the matrices go to host (cnt * ns * ns complex). */
static int continuity_grams(mxg_solver *s, int l0, int cnt, int nb, double *host)
{
  int m = s->m, ns = nb * m, q, k, pr[3], e;
  const void *pp[3];
  size_t slot = elen(s, s->L) / s->K * mxk_elem_size(MX_C128);
  double *tab = malloc(mxk_phase_bytes(cnt));
  if(!tab) return MXG_ENOMEM;
  for(k = 0; k < cnt; k++)
    memcpy(tab + 4 * k, s->h_ph + 4 * (l0 + k), sizeof(double) * 4);
  mxk_phase_fill(cnt, tab);
  e = (int) cudaMemcpyAsync(s->ph2, tab, mxk_phase_bytes(cnt), cudaMemcpyHostToDevice, s->st);
  for(q = 0; q < nb; q++) {
    pr[q] = MX_C128;
    pp[q] = (const char *) s->En + (size_t) (l0 - q) * slot;
  }
  if(!e) e = mxk_block_gram(s->n[s->L], m, cnt, s->ph2, kap(s, s->L), nb, pr, pp, 0, 0, s->ga, s->gm,
                            s->gscratch, s->gscratch_bytes, s->st);
  s->launches += 2;
  if(!e) e = (int) cudaMemcpyAsync(host, s->gm, sizeof(double) * 2 * (size_t) ns * ns * cnt, cudaMemcpyDeviceToHost,
                                   s->st);
  if(!e) e = (int) cudaStreamSynchronize(s->st);
  free(tab);
  return e;
}

int mxg_bloch_continuity(mxg_solver *s, int nk, const int *vertex, int continuity, int chern_vectors,
                         double *lambda, mxg_field *chern, int *sign)
{
  int m = s->m, K = s->K, ie = s->o.ieigs, l, i, j, swaps = 0, e = 0;
  int ns3 = 3 * m, ns2 = 2 * m;
  double *g1, *g3 = 0, *coef;
  adjust_t *Q;
  mxg_field *ch;
  if(!s || nk < 1 || nk > K || nk != s->last_nk || !vertex || chern_vectors < 0 || chern_vectors > ie
     || (continuity != 'n' && continuity != 's' && continuity != 'r'))
    return MXG_EINVAL;
  TRY((int) cudaSetDevice(s->device));
  g1 = malloc(sizeof(double) * 2 * ns2 * ns2);
  if(nk > 2) g3 = malloc(sizeof(double) * 2 * (size_t) ns3 * ns3 * (nk - 2));
  coef = calloc(2 * (size_t) m * m * K, sizeof(double));
  Q = calloc(nk, sizeof(adjust_t));
  ch = calloc(chern_vectors > 0 ? chern_vectors : 1, sizeof(mxg_field));
  if(!g1 || (nk > 2 && !g3) || !coef || !Q || !ch) { e = MXG_ENOMEM; goto out; }
  for(l = 0; l < nk; l++) {
    Q[l].perm = malloc(sizeof(int) * m);
    Q[l].d = malloc(sizeof(mxg_field) * m);
    if(!Q[l].perm || !Q[l].d) { e = MXG_ENOMEM; goto out; }
    for(i = 0; i < m; i++) { Q[l].perm[i] = i; Q[l].d[i] = 1.0; }
  }
  /* the raw blocks in complex128, and their mass Gram matrices */
  if((e = mxk_convert(s->pe, s->E, MX_C128, s->En, elen(s, s->L), s->st))) goto out;
  if(nk > 1 && (e = continuity_grams(s, 1, 1, 2, g1))) goto out;
  if(nk > 2 && (e = continuity_grams(s, 2, nk - 2, 3, g3))) goto out;
  for(i = 0; i < chern_vectors; i++) chern[i] = 0.0;
  if(sign) sign[0] = 0;
  for(l = 1; l < nk; l++) {
    /* block a of the Gram: 0 this k-point, 1 the one before, 2 the one before that */
    const double *G = l == 1 ? g1 : g3 + 2 * (size_t) ns3 * ns3 * (l - 2);
    int ns = l == 1 ? ns2 : ns3;
    int oldvertex = vertex[l - 1];
    adjust_t *P1 = &Q[l - 1], *P2 = l > 1 ? &Q[l - 2] : 0, *P = &Q[l];
    /* e_j^H M eold0_i for raw e_j: X01[j][perm1[i]] d1[i]; likewise eold1,
     * which is zero at the second point (exp_bloch2d.c:773-777 clears it) */
#define C0(jr, i) (gram_at(G, ns, m, 0, (jr), 1, P1->perm[i]) * P1->d[i])
#define C1(jr, i) (P2 ? gram_at(G, ns, m, 0, (jr), 2, P2->perm[i]) * P2->d[i] : 0.0)
    if(continuity == 'r') {
      /* reorder: greedy, the raw vector closest to the (extrapolated) guess */
      for(i = 0; i < ie; i++) {
        double opt = -1.0;
        int best = i;
        for(j = i; j < ie; j++) {
          int jr = P->perm[j];
          double a = oldvertex ? cabs(C0(jr, i)) : cabs(2.0 * C0(jr, i) - C1(jr, i));
          if(a > opt) { opt = a; best = j; }
        }
        if(best != i) {
          int t = P->perm[i];
          double tl;
          P->perm[i] = P->perm[best];
          P->perm[best] = t;
          tl = lambda[(size_t) l * m + i];
          lambda[(size_t) l * m + i] = lambda[(size_t) l * m + best];
          lambda[(size_t) l * m + best] = tl;
          swaps++;
        }
      }
    }
    if(continuity == 's' || continuity == 'r')
      /* sign (phase): make e_i^H M guess_i real and positive */
      for(i = 0; i < m; i++) {
        int jr = P->perm[i];
        mxg_field p = oldvertex ? C0(jr, i) : 2.0 * C0(jr, i) - C1(jr, i);
        P->d[i] = cabs(p) > 0.0 ? p / cabs(p) : 1.0;
      }
    /* Chern partial sums with the adjusted vectors e'_i = d_i e_perm[i] */
    for(i = 0; i < chern_vectors; i++) {
      mxg_field o0e = conj(P1->d[i]) * gram_at(G, ns, m, 1, P1->perm[i], 0, P->perm[i]) * P->d[i];
      mxg_field chup;
      if(oldvertex) {
        mxg_field o00 = conj(P1->d[i]) * gram_at(G, ns, m, 1, P1->perm[i], 1, P1->perm[i]) * P1->d[i];
        chup = 0.5 * I * (o0e - o00);
      }
      else {
        mxg_field o01 = P2 ? conj(P1->d[i]) * gram_at(G, ns, m, 1, P1->perm[i], 2, P2->perm[i]) * P2->d[i] : 0.0;
        chup = 0.5 * I * (o0e - o01);
        if(vertex[l]) {
          mxg_field ee = conj(P->d[i]) * gram_at(G, ns, m, 0, P->perm[i], 0, P->perm[i]) * P->d[i];
          mxg_field e0 = conj(P->d[i]) * gram_at(G, ns, m, 0, P->perm[i], 1, P1->perm[i]) * P1->d[i];
          chup += 0.5 * I * (ee - e0);
        }
      }
      ch[i] += chup;
      chern[(size_t) l * chern_vectors + i] = ch[i];
    }
    if(sign) sign[l] = swaps;
#undef C0
#undef C1
  }
  /* apply the adjustments to the eigenvectors on the device: column i of
   * k-point l becomes d_i times raw column perm_i */
  for(l = 0; l < K; l++)
    for(i = 0; i < m; i++) {
      double *c;
      int r = l < nk ? Q[l].perm[i] : i;
      mxg_field d = l < nk ? Q[l].d[i] : 1.0;
      c = coef + 2 * ((size_t) l * m * m + (size_t) i * m + r);
      c[0] = creal(d);
      c[1] = cimag(d);
    }
  e = (int) cudaMemcpyAsync(s->coef, coef, sizeof(double) * 2 * (size_t) m * m * K, cudaMemcpyHostToDevice, s->st);
  if(!e) {
    int pr = s->pe;
    const void *pp = s->E;
    e = mxk_block_combine(s->n[s->L], m, K, 1, &pr, &pp, s->coef, m, 0, s->combw, s->pe, s->En, s->st);
    s->launches += 2;
  }
  if(!e) {
    swapp(&s->E, &s->En);
    e = (int) cudaStreamSynchronize(s->st);
  }
  /* the adjusted Rayleigh quotients follow the reordering */
  if(!e)
    for(l = 0; l < nk; l++)
      for(i = 0; i < m; i++)
        s->h_rq[l * m + i] = lambda[(size_t) l * m + i] + 1.0;
out:
  if(Q)
    for(l = 0; l < nk; l++) { free(Q[l].perm); free(Q[l].d); }
  free(Q); free(g1); free(g3); free(coef); free(ch);
  return e;
}

int mxg_solver_restarts(const mxg_solver *s)
{
  return s->restarts;
}

int mxg_solver_stats(const mxg_solver *s, double *ms, long *launches)
{
  if(ms) *ms = s->last_ms;
  if(launches) *launches = s->launches;
  return 0;
}

int mxg_solver_profile(mxg_solver *s, int enable)
{
  int q;
  if(enable && !s->pev) {
    s->maxpev = 4096;
    s->pev = calloc(s->maxpev, sizeof(cudaEvent_t));
    s->ptag = calloc(s->maxpev / 2, sizeof(int));
    s->pbytes = calloc(s->maxpev / 2, sizeof(double));
    if(!s->pev || !s->ptag || !s->pbytes) return MXG_ENOMEM;
    for(q = 0; q < s->maxpev; q++)
      if(cudaEventCreate(&s->pev[q])) return MXG_ENOMEM;
  }
  s->prof = enable;
  s->npev = 0;
  for(q = 0; q < MXG_KT_N; q++) {
    s->prof_ms[q] = 0.0;
    s->prof_bytes[q] = 0.0;
    s->prof_count[q] = 0;
  }
  return 0;
}

int mxg_solver_kernel_time(mxg_solver *s, int which, double *ms, long *count, double *bytes)
{
  if(which < 0 || which >= MXG_KT_N) return MXG_EINVAL;
  if(s->prof && s->npev) prof_flush(s);
  if(ms) *ms = s->prof_ms[which];
  if(count) *count = s->prof_count[which];
  if(bytes) *bytes = s->prof_bytes[which];
  return 0;
}

int mxg_eps_sensitivity(int n, const double *kappa, int nk, const mxg_field *xf, const mxg_field *yf, int m,
                        const mxg_field *evec, const double *weights, double *grad)
{
  grid2d_gpu *g;
  edge2d_gpu *e;
  double *dk, *dw, *dg;
  int err;
  if(m < 1 || m > 32) return MXG_EINVAL;
  g = new_grid2d_gpu(n, n, 1.0 / n, 1.0 / n, nk);
  if(!g) return MXG_ENOMEM;
  err = setkappa_grid2d_gpu(g, kappa);
  if(!err) err = setbloch_grid2d_gpu(g, xf, yf);
  e = err ? 0 : new_edge2d_gpu(g, m, MXG_C128);
  if(!e) { del_grid2d_gpu(g); return err ? err : MXG_ENOMEM; }
  err = denseto_edge2d_gpu(evec, e);
  if(cudaMalloc((void **) &dk, sizeof(double) * n * n)) { del_edge2d_gpu(e); del_grid2d_gpu(g); return MXG_ENOMEM; }
  if(cudaMalloc((void **) &dw, sizeof(double) * nk * m)) { cudaFree(dk); del_edge2d_gpu(e); del_grid2d_gpu(g); return MXG_ENOMEM; }
  if(cudaMalloc((void **) &dg, sizeof(double) * n * n)) { cudaFree(dk); cudaFree(dw); del_edge2d_gpu(e); del_grid2d_gpu(g); return MXG_ENOMEM; }
  if(!err) err = (int) cudaMemcpy(dk, kappa, sizeof(double) * n * n, cudaMemcpyHostToDevice);
  if(!err) err = (int) cudaMemcpy(dw, weights, sizeof(double) * nk * m, cudaMemcpyHostToDevice);
  if(!err) err = mxk_eps_sensitivity(n, m, nk, mxg__grid_phases(g), dk, dw, MX_C128, mxg__edge_data(e), dg, 0);
  if(!err) err = (int) cudaMemcpy(grad, dg, sizeof(double) * n * n, cudaMemcpyDeviceToHost);
  cudaFree(dk); cudaFree(dw); cudaFree(dg);
  del_edge2d_gpu(e);
  del_grid2d_gpu(g);
  return err;
}
