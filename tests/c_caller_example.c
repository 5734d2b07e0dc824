/* A reference-style C caller: the per-k solve of the reference's driver
 * (exp_bloch2d.c:781-1053) replaced by the library's batched solver
 * (compiled, not run, by tests/test_abi_cpu.py). */
#include <stdlib.h>

#include "maxwell_gb300.h"

/* kappa: n*n doubles (1/eps per cell), xf/yf: nk Bloch factors */
int solve_bloch(int n0, int L, const double *kappa, int nk,
                const mxg_field *xf, const mxg_field *yf, double *lambda, int *steps)
{
  mxg_solve_opts o = {0};
  double *res = malloc(sizeof(double) * nk * 16);
  int e;
  o.n0 = n0; o.L = L; o.ieigs = 12; o.m = 16;
  o.method = 1;               /* LOBPCG; 0 = the reference's block PINVIT + Ritz */
  o.precision = 1;            /* FP32 multigrid, float-float eigenvectors; 2 = FP64
                               * eigenvectors for residuals below the float-float floor
                               * (about 8 n^2 2^-48 / lambda: near 1e-9 at 1024^2) */
  o.max_nested = 20; o.max_steps = 60;
  o.nested_tol = 1e-2;        /* coarser levels of the nested iteration stop at 1e-2
                               * (the driver's default residual rule); 0 = o.tol */
  o.prec_steps = 2; o.gradient_steps = 5; o.smoother_steps = 2;
  o.lift_e = 1; o.center = 1; o.wave = nk; o.relative = 1; o.tol = 1e-8;
  o.smoother = 1;             /* four-colour AFW; 0 = the reference's row order */
  mxg_solver *s = mxg_solver_new(&o, kappa);
  if(!s) { free(res); return MXG_ENOMEM; }
  e = mxg_bloch_solve(s, nk, xf, yf, lambda, steps, res);   /* lambda: nk*16, ascending */
  mxg_solver_free(s);
  free(res);
  return e;
}
