/* Per-kernel timing of the hot kernels of one block step at a given size.
 *
 * Every kernel runs `reps` times on synthetic blocks (seeded values, the disc
 * permittivity of the benchmark, a generic Bloch phase), timed with CUDA
 * events on the launching stream after one untimed launch.  Each row reports
 * the mean time of one call and the call's algorithmic bytes: every array the
 * call must read or write counted once (complex entry sizes 8 for c64, 16 for
 * float-float; kappa 4 bytes per cell, the AFW factor table 32 bytes per
 * vertex).  With K*m*2n^2 entries per block far above the L2 size the
 * repeated calls read from HBM. */
#include "maxwell_gb300.h"
#include "mx_internal.h"

#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define TRY(x) do { int e_ = (x); if(e_) { err = e_; goto done; } } while(0)

static unsigned long long lcg_state;
static float lcg_unit(void)
{
  lcg_state = lcg_state * 6364136223846793005ULL + 1442695040888963407ULL;
  return (float) ((lcg_state >> 40) * (1.0 / 16777216.0)) - 0.5f;
}

/* fill K blocks of `per` entries: one block made on the host, copied K times */
static int fill(void *d, int prec, size_t per, int K)
{
  size_t es = mxk_elem_size(prec), i;
  float *h = malloc(per * es);
  int k, e = 0;
  if(!h) return MXG_ENOMEM;
  for(i = 0; i < per * es / sizeof(float); i++) h[i] = lcg_unit();
  if(prec == MX_CDD)   /* keep the low parts below the high parts' ulp */
    for(i = 0; i < per * 4; i += 2) h[i + 1] = h[i] * 1e-8f;
  for(k = 0; k < K && !e; k++)
    e = (int) cudaMemcpy((char *) d + (size_t) k * per * es, h, per * es, cudaMemcpyHostToDevice);
  free(h);
  return e;
}

static void row(mxg_kbench_row *r, const char *name, float ms, int reps, double bytes, int launches)
{
  strncpy(r->name, name, sizeof(r->name) - 1);
  r->name[sizeof(r->name) - 1] = 0;
  r->ms = ms / reps;
  r->bytes = bytes;
  r->launches = launches;
}

static int run(int n, int K, int m, int reps, mxg_kbench_row *rows, int maxrows, mxg_tuning *tune);

int mxg_kernel_bench(int n, int K, int m, int reps, mxg_kbench_row *rows, int maxrows)
{
  if(!rows || maxrows < 16) return MXG_EINVAL;
  return run(n, K, m, reps, rows, maxrows, 0);
}

int mxg_get_tuning(mxg_tuning *t)
{
  mxk_tuning q;
  mxk_get_tuning(&q);
  t->gram_waves = q.gram_waves;
  t->combine_ctas = q.combine_ctas;
  t->residual_sites = q.residual_sites;
  mxk_node_gs_oop_get_shape(&t->node_strip, &t->node_band);
  t->restrict_strip_log2 = mxk_node_rr_get_strips();
  return 0;
}

int mxg_set_tuning(const mxg_tuning *t)
{
  mxk_tuning q, old;
  int s0, b0;
  q.gram_waves = t->gram_waves;
  q.combine_ctas = t->combine_ctas;
  q.residual_sites = t->residual_sites;
  if(t->restrict_strip_log2 < 0 || t->restrict_strip_log2 > 62) return MXG_EINVAL;
  mxk_get_tuning(&old);
  mxk_node_gs_oop_get_shape(&s0, &b0);
  if(mxk_set_tuning(&q)) return MXG_EINVAL;
  if(mxk_node_gs_oop_shape(t->node_strip, t->node_band)) {
    mxk_set_tuning(&old);
    return MXG_EINVAL;
  }
  return mxk_node_rr_set_strips(t->restrict_strip_log2) ? MXG_EINVAL : 0;
}

int mxg_autotune(int n, int K, int m, int reps, mxg_tuning *chosen)
{
  mxg_tuning t;
  int e;
  if(!chosen) return MXG_EINVAL;
  e = run(n, K, m, reps, 0, 0, &t);
  if(e < 0) return e;
  *chosen = t;
  return mxg_set_tuning(&t);
}

/* the kernel table (rows) or, with tune, the search over launch shapes */
static int run(int n, int K, int m, int reps, mxg_kbench_row *rows, int maxrows, mxg_tuning *tune)
{
  size_t nn = (size_t) n * n, ne = 2 * nn, q;
  size_t E8 = ne * m * K, V8 = nn * m * K;       /* entries per edge / node block */
  int err = 0, nr = 0, k, it;
  const int rr0 = mxk_node_rr_get_strips();
  double *h_ph = 0, *kd = 0, *ph = 0, *theta = 0, *ga = 0, *gm = 0, *coef = 0, *stats = 0, *acc = 0, *gs = 0;
  double *hk = 0, *hmu = 0, *mu = 0;
  float *kf = 0, *kdd = 0, *hkf = 0, *hkdd = 0;
  void *afw = 0, *E = 0, *X = 0, *P = 0, *r = 0, *b = 0, *x = 0, *d = 0, *bc = 0, *nb = 0, *nx = 0, *nd = 0,
       *nbc = 0, *out = 0, *cw = 0;
  int *gamma = 0, *hg = 0, *sel = 0, *info = 0;
  double *rwork = 0;
  cudaStream_t st = 0;
  cudaEvent_t e0 = 0, e1 = 0;
  size_t gbytes;
  float ms;
  mxk_kappa kap;

  if(n < 8 || (n & 1) || K < 1 || m < 1 || m > 16 || reps < 1) return MXG_EINVAL;
  lcg_state = 12345;
  if(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) || cudaEventCreate(&e0) || cudaEventCreate(&e1))
    { err = MXG_ENOMEM; goto done; }
  /* disc of eps = 12, radius 0.3; phases of k = (0.7, 0.3) */
  hk = malloc(sizeof(double) * nn);
  hkf = malloc(sizeof(float) * nn);
  hkdd = malloc(sizeof(float) * 2 * nn);
  h_ph = malloc(mxk_phase_bytes(K));
  hmu = malloc(sizeof(double) * K * m);
  hg = malloc(sizeof(int) * K);
  if(!hk || !hkf || !hkdd || !h_ph || !hmu || !hg) { err = MXG_ENOMEM; goto done; }
  for(q = 0; q < nn; q++) {
    double xx = (double) (q % n) / n - 0.5, yy = (double) (q / n) / n - 0.5;
    hk[q] = xx * xx + yy * yy <= 0.09 ? 1.0 / 12.0 : 1.0;
    hkf[q] = (float) hk[q];
    hkdd[2 * q] = (float) hk[q];
    hkdd[2 * q + 1] = (float) (hk[q] - (double) hkdd[2 * q]);
  }
  for(k = 0; k < K; k++) {
    h_ph[4 * k] = cos(0.7); h_ph[4 * k + 1] = sin(0.7);
    h_ph[4 * k + 2] = cos(0.3); h_ph[4 * k + 3] = sin(0.3);
    hg[k] = 1;
  }
  mxk_phase_fill(K, h_ph);
  for(q = 0; q < (size_t) K * m; q++) hmu[q] = 1.0 + 10.0 * (double) (q % m);
  gbytes = (size_t) K * 256 * ((3 * m) * (3 * m + 1) / 2) * 4 * sizeof(double);
  if(cudaMalloc((void **) &kd, sizeof(double) * nn) || cudaMalloc((void **) &kf, sizeof(float) * nn)
     || cudaMalloc((void **) &kdd, sizeof(float) * 2 * nn) || cudaMalloc(&afw, 32 * nn)
     || cudaMalloc((void **) &ph, mxk_phase_bytes(K)) || cudaMalloc((void **) &mu, sizeof(double) * K * m)
     || cudaMalloc((void **) &gamma, sizeof(int) * K) || cudaMalloc((void **) &theta, sizeof(double) * K * m)
     || cudaMalloc((void **) &ga, sizeof(double) * 2 * 9 * m * m * K)
     || cudaMalloc((void **) &gm, sizeof(double) * 2 * 9 * m * m * K)
     || cudaMalloc((void **) &coef, sizeof(double) * 2 * 3 * m * m * K) || cudaMalloc(&cw, (size_t) 16 * 3 * m * m * K)
     || cudaMalloc((void **) &stats, sizeof(double) * 5 * m * K) || cudaMalloc((void **) &acc, sizeof(double) * 4 * K * m)
     || cudaMalloc((void **) &gs, gbytes)
     || cudaMalloc(&E, E8 * 16) || cudaMalloc(&out, E8 * 16) || cudaMalloc(&X, E8 * 8) || cudaMalloc(&P, E8 * 8)
     || cudaMalloc(&r, E8 * 8) || cudaMalloc(&b, E8 * 8) || cudaMalloc(&x, E8 * 8) || cudaMalloc(&d, E8 * 8)
     || cudaMalloc(&bc, E8 / 4 * 8) || cudaMalloc(&nb, V8 * 8) || cudaMalloc(&nx, V8 * 8) || cudaMalloc(&nd, V8 * 8)
     || cudaMalloc(&nbc, V8 / 4 * 8) || cudaMalloc((void **) &sel, sizeof(int) * 3 * m * K)
     || cudaMalloc((void **) &info, sizeof(int) * K)
     || cudaMalloc((void **) &rwork, sizeof(double) * mxk_ritz_work_doubles(3 * m) * K))
    { err = MXG_ENOMEM; goto done; }
  TRY((int) cudaMemcpy(kd, hk, sizeof(double) * nn, cudaMemcpyHostToDevice));
  TRY((int) cudaMemcpy(kf, hkf, sizeof(float) * nn, cudaMemcpyHostToDevice));
  TRY((int) cudaMemcpy(kdd, hkdd, sizeof(float) * 2 * nn, cudaMemcpyHostToDevice));
  TRY((int) cudaMemcpy(ph, h_ph, mxk_phase_bytes(K), cudaMemcpyHostToDevice));
  TRY((int) cudaMemcpy(mu, hmu, sizeof(double) * K * m, cudaMemcpyHostToDevice));
  TRY((int) cudaMemcpy(theta, hmu, sizeof(double) * K * m, cudaMemcpyHostToDevice));
  TRY((int) cudaMemcpy(gamma, hg, sizeof(int) * K, cudaMemcpyHostToDevice));
  TRY(mxk_afw_factors(n, kf, 1.0, 1.0, afw, st));
  kap.f = kf; kap.d = kd; kap.dd = kdd; kap.afw = afw; kap.afw_alpha = 1.0; kap.afw_beta = 1.0;
  TRY(fill(E, MX_CDD, ne * m, K));
  TRY(fill(X, MX_C64, ne * m, K));
  TRY(fill(P, MX_C64, ne * m, K));
  TRY(fill(r, MX_C64, ne * m, K));
  TRY(fill(b, MX_C64, ne * m, K));
  TRY(fill(x, MX_C64, ne * m, K));
  TRY(fill(nb, MX_C64, nn * m, K));
  TRY(fill(nx, MX_C64, nn * m, K));
  {
    /* coefficients: identity on the first block plus small couplings */
    double *hc = calloc((size_t) 2 * 3 * m * m * K, sizeof(double));
    if(!hc) { err = MXG_ENOMEM; goto done; }
    for(k = 0; k < K; k++)
      for(it = 0; it < m; it++) {
        hc[2 * (((size_t) k * m + it) * 3 * m + it)] = 1.0;
        hc[2 * (((size_t) k * m + it) * 3 * m + m + it)] = 0.01;
        hc[2 * (((size_t) k * m + it) * 3 * m + 2 * m + it)] = 0.001;
      }
    err = (int) cudaMemcpy(coef, hc, sizeof(double) * 2 * 3 * m * m * K, cudaMemcpyHostToDevice);
    free(hc);
    if(err) goto done;
  }
  TRY((int) cudaDeviceSynchronize());

#define TIME(NAME, BYTES, LAUNCHES, CALL)                                          \
  do {                                                                             \
    TRY(CALL);                                                                     \
    TRY((int) cudaEventRecord(e0, st));                                            \
    for(it = 0; it < reps; it++) TRY(CALL);                                        \
    TRY((int) cudaEventRecord(e1, st));                                            \
    TRY((int) cudaEventSynchronize(e1));                                           \
    TRY((int) cudaEventElapsedTime(&ms, e0, e1));                                  \
    if(nr < maxrows) row(rows + nr++, NAME, ms, reps, (double) (BYTES), LAUNCHES); \
  } while(0)

  if(tune) {
    /* each tunable in turn, the others at their current values: the
     * candidate with the least time for `reps` calls wins */
    static const int gw[] = {1, 2, 4, 8, 16}, cc[] = {1, 2, 3, 4}, rs[] = {8, 16, 32, 64, 128};
    int pr3[3] = {MX_CDD, MX_C64, MX_C64};
    const void *pp3[3];
    mxk_tuning base, tr;
    float best;
    int c;
    pp3[0] = E; pp3[1] = X; pp3[2] = P;
    mxk_get_tuning(&base);
#define TUNE(FIELD, LIST, CALL)                                                      \
    do {                                                                             \
      int bestv = base.FIELD;                                                        \
      best = 1e30f;                                                                  \
      for(c = 0; c < (int) (sizeof(LIST) / sizeof(LIST[0])); c++) {                 \
        tr = base;                                                                   \
        tr.FIELD = LIST[c];                                                          \
        TRY(mxk_set_tuning(&tr));                                                    \
        TRY(CALL);                                                                   \
        TRY((int) cudaEventRecord(e0, st));                                          \
        for(it = 0; it < reps; it++) TRY(CALL);                                      \
        TRY((int) cudaEventRecord(e1, st));                                          \
        TRY((int) cudaEventSynchronize(e1));                                         \
        TRY((int) cudaEventElapsedTime(&ms, e0, e1));                                \
        if(ms < best) { best = ms; bestv = LIST[c]; }                                \
      }                                                                              \
      base.FIELD = bestv;                                                            \
      TRY(mxk_set_tuning(&base));                                                    \
    } while(0)
    TUNE(gram_waves, gw,
         mxk_block_gram(n, m, K, ph, kap, 3, pr3, pp3, r, theta, ga, gm, gs, gbytes, st));
    TUNE(combine_ctas, cc,
         mxk_block_combine(n, m, K, 3, pr3, pp3, coef, 3 * m, 0, cw, MX_CDD, out, st));
    TUNE(residual_sites, rs,
         (cudaMemsetAsync(stats, 0, sizeof(double) * 5 * m * K, st),
          mxk_block_residual(n, m, K, ph, kap, mu, MX_CDD, E, MX_C64, r, stats, st)));
#undef TUNE
    tune->gram_waves = base.gram_waves;
    tune->combine_ctas = base.combine_ctas;
    tune->residual_sites = base.residual_sites;
    tune->restrict_strip_log2 = mxk_node_rr_get_strips();
    mxk_node_gs_oop_get_shape(&tune->node_strip, &tune->node_band);
    {
      /* the node sweep: the in-place row kernels (strip 0) against the
       * tiled out-of-place sweep with each strip x band (two sweeps, so
       * that both leave the result where the in-place pair does) */
      static const int strips[] = {0, 64, 128}, bands[] = {4, 8, 16, 32, 64};
      int si, bi, bs = 0, bb = tune->node_band;
      best = 1e30f;
      for(si = 0; si < 3; si++)
        for(bi = 0; bi < (si ? 5 : 1); bi++) {
          int ok;
          TRY(mxk_node_gs_oop_shape(strips[si], si ? bands[bi] : bb));
          ok = mxk_node_gs_oop_ok(n, m, MX_C64);
          if(si && !ok) continue;
#define SWEEP2()                                                                             \
          (ok ? (mxk_node_gs_oop(n, m, K, ph, 1.0, 0, MX_C64, nb, nx, nd, st)                \
                 || mxk_node_gs_oop(n, m, K, ph, 1.0, 0, MX_C64, nb, nd, nx, st))            \
              : (mxk_node_gs(n, m, K, ph, 1.0, 0, MX_C64, nb, nx, st)                        \
                 || mxk_node_gs(n, m, K, ph, 1.0, 0, MX_C64, nb, nx, st)))
          TRY(SWEEP2());
          TRY((int) cudaEventRecord(e0, st));
          for(it = 0; it < reps; it++) TRY(SWEEP2());
#undef SWEEP2
          TRY((int) cudaEventRecord(e1, st));
          TRY((int) cudaEventSynchronize(e1));
          TRY((int) cudaEventElapsedTime(&ms, e0, e1));
          if(ms < best) { best = ms; bs = strips[si]; if(si) bb = bands[bi]; }
        }
      TRY(mxk_node_gs_oop_shape(bs, bb));
      tune->node_strip = bs;
      tune->node_band = bb;
    }
    goto done;
  }
  {
    const double s8 = 8.0, s16 = 16.0;
    const double kb4 = 4.0 * nn;
    int pr3[3] = {MX_CDD, MX_C64, MX_C64}, pr2[2] = {MX_C64, MX_C64};
    const void *pp3[3], *pp2[2];
    pp3[0] = E; pp3[1] = X; pp3[2] = P;
    pp2[0] = X; pp2[1] = P;
    TIME("edge_residual_c64", 3 * E8 * s8 + kb4, 1,
         mxk_edge_apply(n, m, K, ph, kap, -1.0, -1.0, 0, 1.0, MX_C64, x, MX_C64, b, d, st));
    TIME("afw_sweep_forward_c64", 3 * E8 * s8 + kb4 + 32.0 * nn, 2,
         mxk_edge_gs(n, m, K, ph, kap, 1.0, 1.0, 0, MX_C64, b, x, st));
    TIME("afw_colour_forward_c64", 3 * E8 * s8 + kb4 + 32.0 * nn, 2,
         mxk_edge_gs_colour(n, m, K, ph, kap, 1.0, 1.0, 0, MX_C64, b, x, st));
    TIME("edge_restrict_c64", (E8 + 2 * E8 / 4) * s8, 1,
         mxk_edge_restrict(n / 2, m, K, ph, 1.0, MX_C64, d, bc, st));
    TIME("edge_prolong_c64", (E8 / 4 + 2 * E8) * s8, 1,
         mxk_edge_prolong(n / 2, m, K, ph, 1.0, MX_C64, bc, x, st));
    TIME("node_residual_c64", 3 * V8 * s8, 1,
         mxk_node_apply(n, m, K, ph, -1.0, 1.0, MX_C64, nx, nb, nd, st));
    /* both forms of the fused residual + restriction, whatever the current
     * batch threshold (restored at the end): the strips, then a thread per
     * coarse node */
    mxk_node_rr_set_strips(0);
    TIME("node_residual_restrict_c64", (2 * V8 + V8 / 4) * s8, 1,
         mxk_node_residual_restrict(n / 2, m, K, ph, 1.0, MX_C64, nx, nb, nbc, st));
    mxk_node_rr_set_strips(62);
    TIME("node_residual_restrict_site_c64", (2 * V8 + V8 / 4) * s8, 1,
         mxk_node_residual_restrict(n / 2, m, K, ph, 1.0, MX_C64, nx, nb, nbc, st));
    mxk_node_rr_set_strips(rr0);
    TIME("node_gs_forward_c64", 3 * V8 * s8, 4,
         mxk_node_gs(n, m, K, ph, 1.0, 0, MX_C64, nb, nx, st));
    {
      /* the tiled sweep at its default shape, whatever the current one */
      int s0, b0;
      mxk_node_gs_oop_get_shape(&s0, &b0);
      mxk_node_gs_oop_shape(128, 16);
      if(mxk_node_gs_oop_ok(n, m, MX_C64))
        TIME("node_gs_tiled_c64", 3 * V8 * s8, 3,
             mxk_node_gs_oop(n, m, K, ph, 1.0, 0, MX_C64, nb, nx, nd, st));
      mxk_node_gs_oop_shape(64, 16);
      if(mxk_node_gs_oop_ok(n, m, MX_C64))
        TIME("node_gs_tiled64_c64", 3 * V8 * s8, 3,
             mxk_node_gs_oop(n, m, K, ph, 1.0, 0, MX_C64, nb, nx, nd, st));
      mxk_node_gs_oop_shape(s0, b0);
    }
    TIME("node_restrict_c64", (V8 + 2 * V8 / 4) * s8, 1,
         mxk_node_restrict(n / 2, m, K, ph, 1.0, MX_C64, nd, nbc, st));
    TIME("node_prolong_c64", (V8 / 4 + 2 * V8) * s8, 1,
         mxk_node_prolong(n / 2, m, K, ph, 1.0, MX_C64, nbc, nx, st));
    TIME("adjgradient_mass_cdd_to_c64", E8 * s16 + V8 * s8, 1,
         mxk_adjgradient(n, m, K, ph, 1.0, 1, 0.0, MX_CDD, E, MX_C64, nb, st));
    TIME("gradient_c64_to_cdd", V8 * s8 + 2 * E8 * s16, 1,
         mxk_gradient(n, m, K, ph, -1e-3, MX_C64, nx, MX_CDD, E, st));
    TIME("block_residual_cdd", E8 * s16 + E8 * s8 + 8.0 * nn, 1,
         (cudaMemsetAsync(stats, 0, sizeof(double) * 5 * m * K, st),
          mxk_block_residual(n, m, K, ph, kap, mu, MX_CDD, E, MX_C64, r, stats, st)));
    TIME("block_gram_3x16", E8 * (s16 + 3 * s8) + 12.0 * nn, 2,
         mxk_block_gram(n, m, K, ph, kap, 3, pr3, pp3, r, theta, ga, gm, gs, gbytes, st));
    TIME("block_combine_E_cdd", E8 * (s16 + 2 * s8 + s16), 2,
         mxk_block_combine(n, m, K, 3, pr3, pp3, coef, 3 * m, 0, cw, MX_CDD, out, st));
    TIME("block_combine_P_c64", E8 * 3 * s8, 2,
         mxk_block_combine(n, m, K, 2, pr2, pp2, coef, 3 * m, m, cw, MX_C64, r, st));
    TIME("center_cdd_all_k", 3 * E8 * s16, 2,
         mxk_center(n, m, K, gamma, MX_CDD, E, acc, st));
    TIME("axpy_c64_into_cdd", E8 * (s8 + 2 * s16), 1,
         mxk_axpy(-1e-3, 0.0, MX_C64, x, MX_CDD, E, E8, st));
    /* the Ritz step on the Gram matrices of the block_gram row (every
     * column selected); its bytes are the two 48 x 48 matrices per k-point */
    {
      int *hs = malloc(sizeof(int) * 3 * m * K), q;
      if(!hs) { err = MXG_ENOMEM; goto done; }
      for(q = 0; q < 3 * m * K; q++) hs[q] = 1;
      err = (int) cudaMemcpy(sel, hs, sizeof(int) * 3 * m * K, cudaMemcpyHostToDevice);
      free(hs);
      if(err) goto done;
    }
    TIME("rayleigh_ritz_48", 2.0 * 16.0 * 9 * m * m * K, 1,
         mxk_rayleigh_ritz(3 * m, m, K, ga, gm, sel, 1e-6, -1e300, coef, theta, info, rwork, st));
  }
#undef TIME

done:
  mxk_node_rr_set_strips(rr0);
  cudaFree(kd); cudaFree(kf); cudaFree(kdd); cudaFree(afw); cudaFree(ph); cudaFree(mu); cudaFree(gamma);
  cudaFree(theta); cudaFree(ga); cudaFree(gm); cudaFree(coef); cudaFree(cw); cudaFree(stats); cudaFree(acc);
  cudaFree(gs); cudaFree(E); cudaFree(out); cudaFree(X); cudaFree(P); cudaFree(r); cudaFree(b); cudaFree(x);
  cudaFree(d); cudaFree(bc); cudaFree(nb); cudaFree(nx); cudaFree(nd); cudaFree(nbc);
  cudaFree(sel); cudaFree(info); cudaFree(rwork);
  free(hk); free(hkf); free(hkdd); free(h_ph); free(hmu); free(hg);
  if(e0) cudaEventDestroy(e0);
  if(e1) cudaEventDestroy(e1);
  if(st) cudaStreamDestroy(st);
  /* CUDA errors (positive cudaError_t) are returned as -1000 - code */
  return err ? (err > 0 ? -1000 - err : err) : nr;
}
