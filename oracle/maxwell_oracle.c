/* CPU restatement of the sboerm/Maxwell Bloch eigensolver path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker for the CUDA path
 * (libmaxwell_gb300.so) and the timed CPU baseline.  Nothing in the product
 * library links to it or falls back to it.
 *
 * It restates, in its own formulation, the reference functions cited in each
 * comment: stencils are written in gather form (one output entry sums the
 * contributions of the cells around it) with a single rule for the Bloch
 * seams: an edge or node addressed one period outside the unit cell holds
 * the stored value times xf^a yf^b, a,b in {-1,0,1}, with the conjugate
 * factor for a = -1 or b = -1 (edge2d.c:1335-1650, node2d.c:516-627).
 * Writes through the seam use the conjugate of that phase.
 * Dense linear algebra replaces LAPACK with a Cholesky factorisation and a
 * cyclic Jacobi eigensolver (linalg.c:48-317).
 */
#include "maxwell_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>

typedef om_cplx cx;

/* ------------------------------------------------------------
 * Seam helpers
 * ------------------------------------------------------------ */

static inline cx
phase(int a, int b, cx xf, cx yf)
{
  cx p = 1.0;
  if(a == 1) p *= xf; else if(a == -1) p *= conj(xf);
  if(b == 1) p *= yf; else if(b == -1) p *= conj(yf);
  return p;
}

/* wrap (i,j) into [0,n)^2, returning the seam crossings in *a,*b */
static inline int
wrap(int n, int *i, int *j)
{
  int a = 0, b = 0;
  if(*i < 0) { *i += n; a = -1; } else if(*i >= n) { *i -= n; a = 1; }
  if(*j < 0) { *j += n; b = -1; } else if(*j >= n) { *j -= n; b = 1; }
  return (a + 1) + 3 * (b + 1);
}

static inline cx
fetch(const cx *v, int n, int i, int j, cx xf, cx yf)
{
  int code = wrap(n, &i, &j);
  cx val = v[i + j * n];
  if(code != 4)
    val *= phase(code % 3 - 1, code / 3 - 1, xf, yf);
  return val;
}

static inline void
deposit(cx *v, int n, int i, int j, cx xf, cx yf, cx val)
{
  int code = wrap(n, &i, &j);
  if(code != 4)
    val *= conj(phase(code % 3 - 1, code / 3 - 1, xf, yf));
  v[i + j * n] += val;
}

static inline double
kap(const double *kappa, int n, int i, int j)
{
  wrap(n, &i, &j);
  return kappa[i + j * n];
}

#define XE(v, i, j) fetch((v), n, (i), (j), xf, yf)
#define YE(v, i, j) fetch((v) + (long) n * n, n, (i), (j), xf, yf)

/* ------------------------------------------------------------
 * Edge operator y += alpha A x + beta M x   (edge2d.c:1335-1650)
 * A: kappa-weighted curl-curl, M: Nedelec mass, axy = alpha/(hx hy),
 * mx = my = beta/6 on the unit square.  kappa == NULL means mass only.
 * Every cell uses its own kappa; this is the operator that
 * densematrix_edge2d (edge2d.c:5870-6116) assembles.  The reference's
 * matrix-free addeval_edge2d and energyprod_edge2d instead take kappa of
 * the upper cell for the lower-cell term of the x-edges in the last column
 * (rows 1..ny-2, edge2d.c:1532) and in the last row (edge2d.c:1564,1597,1627;
 * the same in energyprod_edge2d),
 * which makes them non-Hermitian when kappa varies across those seams; the
 * two agree whenever kappa(i,ny-1) = kappa(i,ny-2) and
 * kappa(nx-1,j) = kappa(nx-1,j-1).
 * ------------------------------------------------------------ */

static inline cx
kx_xedge(int n, const double *kappa, cx xf, cx yf, cx axy, cx mx,
         const cx *x, int i, int j)
{
  cx c0 = XE(x, i, j), up = XE(x, i, j + 1), dn = XE(x, i, j - 1);
  cx curl_above, curl_below;
  if(!kappa)          /* mass only */
    return mx * (4.0 * c0 + up + dn);
  /* cell (i,j): this edge is its bottom edge, curl = b - t - l + r */
  curl_above = c0 - up - YE(x, i, j) + YE(x, i + 1, j);
  /* cell (i,j-1): this edge is its top edge */
  curl_below = dn - c0 - YE(x, i, j - 1) + YE(x, i + 1, j - 1);
  return axy * (kap(kappa, n, i, j) * curl_above - kap(kappa, n, i, j - 1) * curl_below)
         + mx * (4.0 * c0 + up + dn);
}

static inline cx
kx_yedge(int n, const double *kappa, cx xf, cx yf, cx axy, cx my,
         const cx *x, int i, int j)
{
  cx c0 = YE(x, i, j), rt = YE(x, i + 1, j), lt = YE(x, i - 1, j);
  cx curl_right, curl_left;
  if(!kappa)
    return my * (4.0 * c0 + rt + lt);
  /* cell (i,j): this edge is its left edge */
  curl_right = XE(x, i, j) - XE(x, i, j + 1) - c0 + rt;
  /* cell (i-1,j): this edge is its right edge */
  curl_left = XE(x, i - 1, j) - XE(x, i - 1, j + 1) - lt + c0;
  return axy * (kap(kappa, n, i - 1, j) * curl_left - kap(kappa, n, i, j) * curl_right)
         + my * (4.0 * c0 + rt + lt);
}

void
om_addeval_edge(int n, const double *kappa, cx xf, cx yf,
                cx alpha, cx beta, const cx *x, cx *y)
{
  cx axy = alpha * (double) n * (double) n;
  cx mm = beta / 6.0;
  long nn = (long) n * n;
  int i, j;
#pragma omp parallel for private(i) schedule(static)
  for(j = 0; j < n; j++)
    for(i = 0; i < n; i++) {
      y[i + j * n] += kx_xedge(n, kappa, xf, yf, axy, mm, x, i, j);
      y[nn + i + j * n] += kx_yedge(n, kappa, xf, yf, axy, mm, x, i, j);
    }
}

/* Dot products and norms sum fixed chunks of OM_CHUNK entries and combine
 * the chunk sums in chunk order, so that the result does not depend on the
 * thread count or on the order in which threads finish. */
#define OM_CHUNK 4096L

cx
om_dot(long len, const cx *x, const cx *y)
{
  long nc = (len + OM_CHUNK - 1) / OM_CHUNK, c;
  double *part = malloc(sizeof(double) * 2 * (size_t) (nc > 0 ? nc : 1));
  double re = 0.0, im = 0.0;
#pragma omp parallel for schedule(static)
  for(c = 0; c < nc; c++) {
    long k, k1 = (c + 1) * OM_CHUNK < len ? (c + 1) * OM_CHUNK : len;
    double r = 0.0, q = 0.0;
    for(k = c * OM_CHUNK; k < k1; k++) {
      cx p = conj(x[k]) * y[k];
      r += creal(p);
      q += cimag(p);
    }
    part[2 * c] = r;
    part[2 * c + 1] = q;
  }
  for(c = 0; c < nc; c++) {
    re += part[2 * c];
    im += part[2 * c + 1];
  }
  free(part);
  return re + I * im;
}

double
om_norm2(long len, const cx *x)
{
  long nc = (len + OM_CHUNK - 1) / OM_CHUNK, c;
  double *part = malloc(sizeof(double) * (size_t) (nc > 0 ? nc : 1));
  double s = 0.0;
#pragma omp parallel for schedule(static)
  for(c = 0; c < nc; c++) {
    long k, k1 = (c + 1) * OM_CHUNK < len ? (c + 1) * OM_CHUNK : len;
    double r = 0.0;
    for(k = c * OM_CHUNK; k < k1; k++)
      r += creal(x[k]) * creal(x[k]) + cimag(x[k]) * cimag(x[k]);
    part[c] = r;
  }
  for(c = 0; c < nc; c++)
    s += part[c];
  free(part);
  return sqrt(s);
}

/* energyprod_edge2d returns CONJ(sum conj(y) (alpha A + beta M) x),
 * edge2d.c:1652-1959 */
cx
om_energyprod_edge(int n, const double *kappa, cx xf, cx yf,
                   cx alpha, cx beta, const cx *x, const cx *y)
{
  long nn = 2L * n * n;
  cx *t = calloc(nn, sizeof(cx));
  cx s;
  om_addeval_edge(n, kappa, xf, yf, alpha, beta, x, t);
  s = om_dot(nn, y, t);
  free(t);
  return conj(s);
}

/* massprod_edge2d, edge2d.c:1961-2027 */
cx
om_massprod_edge(int n, cx xf, cx yf, const cx *x, const cx *y)
{
  return om_energyprod_edge(n, 0, xf, yf, 0.0, 1.0, x, y);
}

/* center_edge2d, edge2d.c:1309-1333: removes the two constant fields, i.e.
 * subtracts the mean of the x coefficients and of the y coefficients. */
void
om_center_edge(int n, cx *x)
{
  long nn = (long) n * n, k;
  int p;
  for(p = 0; p < 2; p++) {
    cx s = 0.0;
    for(k = 0; k < nn; k++)
      s += x[p * nn + k];
    s /= (double) nn;
    for(k = 0; k < nn; k++)
      x[p * nn + k] -= s;
  }
}

/* nullprod_edge2d, edge2d.c:1240-1274: the L2 products with the constant
 * x and y fields, hx * sum 6 mx x = hy * sum x and hx * sum y (hx = hy = 1/n) */
void
om_nullprod_edge(int n, const cx *x, cx *xprod, cx *yprod)
{
  long nn = (long) n * n, k;
  double h = 1.0 / n;
  cx sx = 0.0, sy = 0.0;
  for(k = 0; k < nn; k++) {
    sx += x[k];
    sy += x[nn + k];
  }
  *xprod = h * sx;
  *yprod = h * sy;
}

/* nulladd_edge2d, edge2d.c:1276-1307: x-edges += hx xalpha, y-edges += hy yalpha */
void
om_nulladd_edge(int n, cx xalpha, cx yalpha, cx *x)
{
  long nn = (long) n * n, k;
  double h = 1.0 / n;
  for(k = 0; k < nn; k++) {
    x[k] += h * xalpha;
    x[nn + k] += h * yalpha;
  }
}

/* normmax_edge2d / normmax_node2d, edge2d.c:887-920, node2d.c:441-463 */
double
om_normmax(long len, const cx *x)
{
  double m = 0.0;
  long k;
  for(k = 0; k < len; k++)
    if(cabs(x[k]) > m) m = cabs(x[k]);
  return m;
}

/* center_node2d, node2d.c:489-514: subtract the mean coefficient */
void
om_center_node(int n, cx *v)
{
  long nn = (long) n * n, k;
  cx s = 0.0;
  for(k = 0; k < nn; k++)
    s += v[k];
  s /= (double) nn;
  for(k = 0; k < nn; k++)
    v[k] -= s;
}

/* ------------------------------------------------------------
 * AFW vertex-patch Gauss-Seidel   (edge2d.c:2029-3042)
 * Patch of vertex (i,j): u = [x(i-1,j), x(i,j), y(i,j-1), y(i,j)], the
 * four edges meeting at the vertex; the cells around it are
 * LL (i-1,j-1), LR (i,j-1), UL (i-1,j), UR (i,j).
 * The update is u += (1/4) Q T^-1 Q^H r with r = b - (alpha A + beta M) x on
 * the patch, Q the 4x4 Hadamard pattern of starsolve_common
 * (edge2d.c:2136-2182) and T the reference's transformed local matrix
 * (edge2d.c:2044-2068) with kXY = axy*kappa_XY, s = 4(mx+my), t = 4(mx-my):
 *   T00 = kUL+kLR+s  T10 = t        T20 = kUL-kLR  T30 = 0
 *   T11 = kLL+kUR    T21 = kLL-kUR  T31 = 0
 *   T22 = kLL+kUL+kLR+kUR+s         T32 = t        T33 = s
 * (T is not (1/4) Q^H K Q of the assembled operator: its mass part differs,
 * and the factorisation below keeps the reference's omission of one fill
 * term; both change only the smoother, not the discrete problem.)
 * ------------------------------------------------------------ */

static void
patch_solve(int n, const double *kappa, cx xf, cx yf, double axy, double mm,
            cx ax_, cx mx_, const cx *b, cx *x, int i, int j)
{
  double kLL = axy * kap(kappa, n, i - 1, j - 1), kLR = axy * kap(kappa, n, i, j - 1);
  double kUL = axy * kap(kappa, n, i - 1, j), kUR = axy * kap(kappa, n, i, j);
  double s = 8.0 * mm, t = 0.0;    /* mx = my = mm on square cells */
  double T00 = kUL + kLR + s, T10 = t, T20 = kUL - kLR;
  double T11 = kLL + kUR, T21 = kLL - kUR;
  double T22 = kLL + kUL + kLR + kUR + s, T32 = t, T33 = s;
  double l10, l20, l21, l32, D0, D1, D2, D3;
  cx r0, r1, r2, r3, c0, c1, c2, c3;
  long nn = (long) n * n;

  /* T = L D L^T, L unit lower with nonzeros l10, l20, l21, l32 */
  D0 = T00;
  l10 = T10 / D0; l20 = T20 / D0;
  D1 = T11 - l10 * l10 * D0;
  l21 = (T21 - l20 * l10 * D0) / D1;
  /* the reference's elimination (edge2d.c:2070-2081) does not subtract the
   * fill l20^2 D0 from entry (2,2), so it factors T + (T20^2/T00) e2 e2^T */
  D2 = T22 - l21 * l21 * D1;
  l32 = T32 / D2;
  D3 = T33 - l32 * l32 * D2;

  r0 = XE(b, i - 1, j) - kx_xedge(n, kappa, xf, yf, ax_, mx_, x, i - 1, j);
  r1 = XE(b, i, j) - kx_xedge(n, kappa, xf, yf, ax_, mx_, x, i, j);
  r2 = YE(b, i, j - 1) - kx_yedge(n, kappa, xf, yf, ax_, mx_, x, i, j - 1);
  r3 = YE(b, i, j) - kx_yedge(n, kappa, xf, yf, ax_, mx_, x, i, j);

  /* c = Q^H r */
  c0 = r0 + r1 + r2 + r3;
  c1 = r0 + r1 - r2 - r3;
  c2 = r0 - r1 - r2 + r3;
  c3 = r0 - r1 + r2 - r3;
  /* T w = c */
  c1 -= l10 * c0;
  c2 -= l20 * c0 + l21 * c1;
  c3 -= l32 * c2;
  c0 /= D0; c1 /= D1; c2 /= D2; c3 /= D3;
  c2 -= l32 * c3;
  c1 -= l21 * c2;
  c0 -= l10 * c1 + l20 * c2;
  /* u = Q w / 4 */
  deposit(x, n, i - 1, j, xf, yf, 0.25 * (c0 + c1 + c2 + c3));
  deposit(x, n, i, j, xf, yf, 0.25 * (c0 + c1 - c2 - c3));
  deposit(x + nn, n, i, j - 1, xf, yf, 0.25 * (c0 - c1 - c2 + c3));
  deposit(x + nn, n, i, j, xf, yf, 0.25 * (c0 - c1 + c2 - c3));
}

/* Rows of one phase touch disjoint unknowns, so they run in parallel; each
 * row is a sequential chain.  Forward order of the reference: row 0, even
 * rows 2..ny-2, odd rows 1..ny-3, row ny-1, each left to right
 * (edge2d.c:2656-2758); backward is the exact reverse (edge2d.c:2760-2861). */
static void
gs_edge_rows(int n, const double *kappa, cx xf, cx yf, double axy, double mm,
             cx ax_, cx mx_, const cx *b, cx *x, int first, int step, int last,
             int backward)
{
  int j;
#pragma omp parallel for schedule(static)
  for(j = first; j <= last; j += step) {
    int i;
    if(!backward)
      for(i = 0; i < n; i++)
        patch_solve(n, kappa, xf, yf, axy, mm, ax_, mx_, b, x, i, j);
    else
      for(i = n - 1; i >= 0; i--)
        patch_solve(n, kappa, xf, yf, axy, mm, ax_, mx_, b, x, i, j);
  }
}

static void
gs_edge_dir(int n, const double *kappa, cx xf, cx yf, cx alpha, cx beta,
            int backward, const cx *b, cx *x)
{
  double axy = creal(alpha) * n * (double) n, mm = creal(beta) / 6.0;
  cx ax_ = alpha * (double) n * (double) n, mx_ = beta / 6.0;
  if(!backward) {
    gs_edge_rows(n, kappa, xf, yf, axy, mm, ax_, mx_, b, x, 0, 1, 0, 0);
    gs_edge_rows(n, kappa, xf, yf, axy, mm, ax_, mx_, b, x, 2, 2, n - 2, 0);
    gs_edge_rows(n, kappa, xf, yf, axy, mm, ax_, mx_, b, x, 1, 2, n - 3, 0);
    gs_edge_rows(n, kappa, xf, yf, axy, mm, ax_, mx_, b, x, n - 1, 1, n - 1, 0);
  }
  else {
    gs_edge_rows(n, kappa, xf, yf, axy, mm, ax_, mx_, b, x, n - 1, 1, n - 1, 1);
    gs_edge_rows(n, kappa, xf, yf, axy, mm, ax_, mx_, b, x, 1, 2, n - 3, 1);
    gs_edge_rows(n, kappa, xf, yf, axy, mm, ax_, mx_, b, x, 2, 2, n - 2, 1);
    gs_edge_rows(n, kappa, xf, yf, axy, mm, ax_, mx_, b, x, 0, 1, 0, 1);
  }
}

void
om_gs_edge(int n, const double *kappa, cx xf, cx yf, cx alpha, cx beta,
           int dir, const cx *b, cx *x)
{
  if(dir == 0 || dir == 2)
    gs_edge_dir(n, kappa, xf, yf, alpha, beta, 0, b, x);
  if(dir == 1 || dir == 2)
    gs_edge_dir(n, kappa, xf, yf, alpha, beta, 1, b, x);
}

/* Point Gauss-Seidel of alpha A + beta M in the reference's interleaved
 * row order (gsforward/gsbackward_simple_edge2d, edge2d.c:3890-5573, the
 * variant compiled with SMOOTHER_INTERLEAVED): forward row 0, rows
 * 2, 4, .., n-2, rows 1, 3, .., n-3, row n-1, each left to right with the
 * x-edge (i,j) before the y-edge (i,j); backward the reverse.  Each edge
 * moves by its residual row over its diagonal axy (kappa of its two cells)
 * + 4 beta/6. */
static void
gs_simple_row(int n, const double *kappa, cx xf, cx yf, cx axy, cx mm, const cx *b, cx *x, int j, int back)
{
  long nn = (long) n * n;
  int s, i;
  for(s = 0; s < n; s++) {
    int q;
    i = back ? n - 1 - s : s;
    for(q = 0; q < 2; q++) {
      int ydir = back ? q == 0 : q == 1;
      if(!ydir) {
        cx r = b[i + j * n] - kx_xedge(n, kappa, xf, yf, axy, mm, x, i, j);
        cx d = axy * (kap(kappa, n, i, j - 1) + kap(kappa, n, i, j)) + 4.0 * mm;
        x[i + j * n] += r / d;
      }
      else {
        cx r = b[nn + i + j * n] - kx_yedge(n, kappa, xf, yf, axy, mm, x, i, j);
        cx d = axy * (kap(kappa, n, i - 1, j) + kap(kappa, n, i, j)) + 4.0 * mm;
        x[nn + i + j * n] += r / d;
      }
    }
  }
}

void
om_gs_edge_simple(int n, const double *kappa, cx xf, cx yf, cx alpha, cx beta, int dir, const cx *b, cx *x)
{
  cx axy = alpha * (double) n * (double) n, mm = beta / 6.0;
  int j;
  if(dir == 0 || dir == 2) {
    gs_simple_row(n, kappa, xf, yf, axy, mm, b, x, 0, 0);
    for(j = 2; j < n - 1; j += 2) gs_simple_row(n, kappa, xf, yf, axy, mm, b, x, j, 0);
    for(j = 1; j < n - 1; j += 2) gs_simple_row(n, kappa, xf, yf, axy, mm, b, x, j, 0);
    gs_simple_row(n, kappa, xf, yf, axy, mm, b, x, n - 1, 0);
  }
  if(dir == 1 || dir == 2) {
    gs_simple_row(n, kappa, xf, yf, axy, mm, b, x, n - 1, 1);
    for(j = 1; j < n - 1; j += 2) gs_simple_row(n, kappa, xf, yf, axy, mm, b, x, j, 1);
    for(j = 2; j < n - 1; j += 2) gs_simple_row(n, kappa, xf, yf, axy, mm, b, x, j, 1);
    gs_simple_row(n, kappa, xf, yf, axy, mm, b, x, 0, 1);
  }
}

/* The four-colour order of the same patch solves (the GPU solver's
 * smoother; it has no counterpart in the reference): vertices split by
 * (i mod 2, j mod 2), forward (0,0), (1,0), (0,1), (1,1), backward the
 * reverse.  Patches of one colour do not read each other's unknowns, so the
 * order inside a colour does not matter. */
static void
gs_edge_colour(int n, const double *kappa, cx xf, cx yf, double axy, double mm, cx ax_, cx mx_,
               const cx *b, cx *x, int ci, int cj)
{
  int j;
#pragma omp parallel for schedule(static)
  for(j = cj; j < n; j += 2) {
    int i;
    for(i = ci; i < n; i += 2)
      patch_solve(n, kappa, xf, yf, axy, mm, ax_, mx_, b, x, i, j);
  }
}

void
om_gs_edge_colour(int n, const double *kappa, cx xf, cx yf, cx alpha, cx beta,
                  int dir, const cx *b, cx *x)
{
  static const int order[4][2] = {{0, 0}, {1, 0}, {0, 1}, {1, 1}};
  double axy = creal(alpha) * n * (double) n, mm = creal(beta) / 6.0;
  cx ax_ = alpha * (double) n * (double) n, mx_ = beta / 6.0;
  int c;
  if(dir == 0 || dir == 2)
    for(c = 0; c < 4; c++)
      gs_edge_colour(n, kappa, xf, yf, axy, mm, ax_, mx_, b, x, order[c][0], order[c][1]);
  if(dir == 1 || dir == 2)
    for(c = 3; c >= 0; c--)
      gs_edge_colour(n, kappa, xf, yf, axy, mm, ax_, mx_, b, x, order[c][0], order[c][1]);
}

/* ------------------------------------------------------------
 * Edge transfers   (edge2d.c:5583-5705)
 * ------------------------------------------------------------ */

void
om_prolong_edge(int nc, cx xf, cx yf, cx alpha, const cx *c, cx *f)
{
  int nf = 2 * nc;
  long fnn = (long) nf * nf;
  int i, j;
#pragma omp parallel for private(i) schedule(static)
  for(j = 0; j < nf; j++)
    for(i = 0; i < nf; i++) {
      int ci = i / 2, cj = j / 2, n = nc;
      cx vx, vy;
      /* x-edge (i,j): on a coarse x-edge row when j is even */
      if(!(j & 1))
        vx = 0.5 * XE(c, ci, cj);
      else
        vx = 0.25 * (XE(c, ci, cj) + XE(c, ci, cj + 1));
      /* y-edge (i,j): on a coarse y-edge column when i is even */
      if(!(i & 1))
        vy = 0.5 * YE(c, ci, cj);
      else
        vy = 0.25 * (YE(c, ci, cj) + YE(c, ci + 1, cj));
      f[i + (long) j * nf] += alpha * vx;
      f[fnn + i + (long) j * nf] += alpha * vy;
    }
}

void
om_restrict_edge(int nc, cx xf, cx yf, cx alpha, const cx *f, cx *c)
{
  int n = 2 * nc;
  long cnn = (long) nc * nc;
  int i, j;
#pragma omp parallel for private(i) schedule(static)
  for(j = 0; j < nc; j++)
    for(i = 0; i < nc; i++) {
      cx sx = 0.5 * (XE(f, 2 * i, 2 * j) + XE(f, 2 * i + 1, 2 * j))
              + 0.25 * (XE(f, 2 * i, 2 * j - 1) + XE(f, 2 * i + 1, 2 * j - 1)
                        + XE(f, 2 * i, 2 * j + 1) + XE(f, 2 * i + 1, 2 * j + 1));
      cx sy = 0.5 * (YE(f, 2 * i, 2 * j) + YE(f, 2 * i, 2 * j + 1))
              + 0.25 * (YE(f, 2 * i - 1, 2 * j) + YE(f, 2 * i - 1, 2 * j + 1)
                        + YE(f, 2 * i + 1, 2 * j) + YE(f, 2 * i + 1, 2 * j + 1));
      c[i + (long) j * nc] += alpha * sx;
      c[cnn + i + (long) j * nc] += alpha * sy;
    }
}

/* ------------------------------------------------------------
 * Node space: Q1 Laplace (node2d.c:516-627), point GS (node2d.c:629-1138),
 * transfers (node2d.c:1140-1273), gradient and adjoint (node2d.c:1275-1350)
 * With hx = hy: diagonal 8/3, all eight neighbours -1/3 (times alpha).
 * ------------------------------------------------------------ */

#define NV(v, i, j) fetch((v), n, (i), (j), xf, yf)

static inline cx
lap_offdiag(int n, cx xf, cx yf, const cx *x, int i, int j)
{
  return NV(x, i - 1, j) + NV(x, i + 1, j) + NV(x, i, j - 1) + NV(x, i, j + 1)
         + NV(x, i - 1, j - 1) + NV(x, i + 1, j - 1)
         + NV(x, i - 1, j + 1) + NV(x, i + 1, j + 1);
}

void
om_addeval_node(int n, cx xf, cx yf, cx alpha, const cx *x, cx *y)
{
  int i, j;
#pragma omp parallel for private(i) schedule(static)
  for(j = 0; j < n; j++)
    for(i = 0; i < n; i++)
      y[i + j * n] += alpha * ((8.0 / 3.0) * x[i + j * n]
                               - (1.0 / 3.0) * lap_offdiag(n, xf, yf, x, i, j));
}

static void
gs_node_rows(int n, cx xf, cx yf, cx alpha, const cx *b, cx *x,
             int first, int step, int last, int backward)
{
  int j;
  cx ac = alpha * (8.0 / 3.0), ao = alpha * (-1.0 / 3.0);
#pragma omp parallel for schedule(static)
  for(j = first; j <= last; j += step) {
    int i, s;
    for(s = 0; s < n; s++) {
      i = backward ? n - 1 - s : s;
      x[i + j * n] = (b[i + j * n] - ao * lap_offdiag(n, xf, yf, x, i, j)) / ac;
    }
  }
}

/* forward: row 0, odd rows 1..ny-3, even rows 2..ny-2, row ny-1 (node2d.c:629-767) */
void
om_gs_node(int n, cx xf, cx yf, cx alpha, int dir, const cx *b, cx *x)
{
  if(dir == 0 || dir == 2) {
    gs_node_rows(n, xf, yf, alpha, b, x, 0, 1, 0, 0);
    gs_node_rows(n, xf, yf, alpha, b, x, 1, 2, n - 3, 0);
    gs_node_rows(n, xf, yf, alpha, b, x, 2, 2, n - 2, 0);
    gs_node_rows(n, xf, yf, alpha, b, x, n - 1, 1, n - 1, 0);
  }
  if(dir == 1 || dir == 2) {
    gs_node_rows(n, xf, yf, alpha, b, x, n - 1, 1, n - 1, 1);
    gs_node_rows(n, xf, yf, alpha, b, x, 2, 2, n - 2, 1);
    gs_node_rows(n, xf, yf, alpha, b, x, 1, 2, n - 3, 1);
    gs_node_rows(n, xf, yf, alpha, b, x, 0, 1, 0, 1);
  }
}

void
om_prolong_node(int nc, cx xf, cx yf, cx alpha, const cx *c, cx *f)
{
  int nf = 2 * nc, n = nc;
  int i, j;
#pragma omp parallel for private(i) schedule(static)
  for(j = 0; j < nf; j++)
    for(i = 0; i < nf; i++) {
      int ci = i / 2, cj = j / 2, oi = i & 1, oj = j & 1;
      cx v = NV(c, ci, cj);
      if(oi) v += NV(c, ci + 1, cj);
      if(oj) v += NV(c, ci, cj + 1);
      if(oi && oj) v += NV(c, ci + 1, cj + 1);
      f[i + (long) j * nf] += alpha * v * (oi ? 0.5 : 1.0) * (oj ? 0.5 : 1.0);
    }
}

void
om_restrict_node(int nc, cx xf, cx yf, cx alpha, const cx *f, cx *c)
{
  int n = 2 * nc;
  int i, j;
#pragma omp parallel for private(i) schedule(static)
  for(j = 0; j < nc; j++)
    for(i = 0; i < nc; i++) {
      int fi = 2 * i, fj = 2 * j;
      cx s = NV(f, fi, fj)
             + 0.5 * (NV(f, fi - 1, fj) + NV(f, fi + 1, fj) + NV(f, fi, fj - 1) + NV(f, fi, fj + 1))
             + 0.25 * (NV(f, fi - 1, fj - 1) + NV(f, fi + 1, fj - 1)
                       + NV(f, fi - 1, fj + 1) + NV(f, fi + 1, fj + 1));
      c[i + (long) j * nc] += alpha * s;
    }
}

void
om_gradient(int n, cx xf, cx yf, cx alpha, const cx *v, cx *e)
{
  long nn = (long) n * n;
  int i, j;
#pragma omp parallel for private(i) schedule(static)
  for(j = 0; j < n; j++)
    for(i = 0; i < n; i++) {
      e[i + j * n] += alpha * (NV(v, i + 1, j) - v[i + j * n]);
      e[nn + i + j * n] += alpha * (NV(v, i, j + 1) - v[i + j * n]);
    }
}

void
om_adjgradient(int n, cx xf, cx yf, cx alpha, const cx *e, cx *v)
{
  long nn = (long) n * n;
  int i, j;
#pragma omp parallel for private(i) schedule(static)
  for(j = 0; j < n; j++)
    for(i = 0; i < n; i++)
      v[i + j * n] += alpha * (XE(e, i - 1, j) - e[i + j * n]
                               + YE(e, i, j - 1) - e[nn + i + j * n]);
}

/* ------------------------------------------------------------
 * Dense coarse matrices (edge2d.c:5870-6152, node2d.c:1429-1602),
 * assembled column by column from the matrix-free operators.
 * ------------------------------------------------------------ */

void
om_dense_edge(int n, const double *kappa, cx xf, cx yf, cx alpha, cx beta, cx *a)
{
  int N = 2 * n * n, c;
  cx *u = calloc(N, sizeof(cx));
  memset(a, 0, sizeof(cx) * (size_t) N * N);
  for(c = 0; c < N; c++) {
    u[c] = 1.0;
    om_addeval_edge(n, kappa, xf, yf, alpha, beta, u, a + (size_t) c * N);
    u[c] = 0.0;
  }
  free(u);
}

/* fixnull: at k = 0 every entry gets +0.1/(rows*cols) (node2d.c:1454-1458) */
void
om_dense_node(int n, cx xf, cx yf, int fixnull, cx *a)
{
  int N = n * n, c;
  size_t k;
  cx *u = calloc(N, sizeof(cx));
  memset(a, 0, sizeof(cx) * (size_t) N * N);
  for(c = 0; c < N; c++) {
    u[c] = 1.0;
    om_addeval_node(n, xf, yf, 1.0, u, a + (size_t) c * N);
    u[c] = 0.0;
  }
  if(fixnull && cabs(xf - 1.0) < 1e-8 && cabs(yf - 1.0) < 1e-8)
    for(k = 0; k < (size_t) N * N; k++)
      a[k] += 0.1 / ((double) N * N);
  free(u);
}

/* ------------------------------------------------------------
 * Grid helpers (grid2d.c)
 * ------------------------------------------------------------ */

/* coarsen_grid2d, grid2d.c:42-68: mean of the four children */
void
om_coarsen_kappa(int n, const double *kf, double *kc)
{
  int nc = n / 2, i, j;
  for(j = 0; j < nc; j++)
    for(i = 0; i < nc; i++)
      kc[i + j * nc] = 0.25 * (kf[2 * i + 2 * j * n] + kf[2 * i + 1 + 2 * j * n]
                               + kf[2 * i + (2 * j + 1) * n] + kf[2 * i + 1 + (2 * j + 1) * n]);
}

/* setpattern_grid2d, grid2d.c:171-218: each cell takes the reciprocal
 * permittivity of the last disc containing its lower-left corner. */
void
om_disc_kappa(int n, int ndiscs, const double *discs, double eps_base,
              double *kappa)
{
  int i, j, k;
  double h = 1.0 / n;
  for(j = 0; j < n; j++)
    for(i = 0; i < n; i++) {
      double x = i * h, y = j * h, kv = 1.0 / eps_base;
      for(k = 0; k < ndiscs; k++) {
        const double *d = discs + 4 * k;
        if((x - d[1]) * (x - d[1]) + (y - d[2]) * (y - d[2]) <= d[3] * d[3])
          kv = 1.0 / d[0];
      }
      kappa[i + j * n] = kv;
    }
}

/* setpattern_grid2d, grid2d.c:171-218: 1/eps_base everywhere, then every
 * rectangle (eps, left, bottom, width, height) and every circle (eps, cx, cy,
 * r) that contains a cell's lower-left corner (i h, j h) sets that cell to
 * 1/eps, later shapes over earlier ones, circles after rectangles. */
void
om_pattern_kappa(int n, int nrect, const double *rect, int ncirc, const double *circ,
                 double eps_base, double *kappa)
{
  int i, j, k;
  double h = 1.0 / n;
  for(j = 0; j < n; j++)
    for(i = 0; i < n; i++)
      kappa[i + j * n] = 1.0 / eps_base;
  for(k = 0; k < nrect; k++) {
    const double *r = rect + 5 * k;
    for(j = 0; j < n; j++)
      for(i = 0; i < n; i++) {
        double x = i * h, y = j * h;
        if(r[1] <= x && x <= r[1] + r[3] && r[2] <= y && y <= r[2] + r[4])
          kappa[i + j * n] = 1.0 / r[0];
      }
  }
  for(k = 0; k < ncirc; k++) {
    const double *c = circ + 4 * k;
    for(j = 0; j < n; j++)
      for(i = 0; i < n; i++) {
        double x = i * h, y = j * h;
        if((x - c[1]) * (x - c[1]) + (y - c[2]) * (y - c[2]) <= c[3] * c[3])
          kappa[i + j * n] = 1.0 / c[0];
      }
  }
}

/* ------------------------------------------------------------
 * Dense Hermitian linear algebra (replaces zpotrf/ztrsm/zheev/zhegv,
 * linalg.c:48-317).  Column-major, leading dimension n.
 * ------------------------------------------------------------ */

#define A_(i, j) a[(i) + (size_t) (j) * n]

int
om_potrf(int n, cx *a)
{
  int i, j, k;
  for(j = 0; j < n; j++) {
    double d = creal(A_(j, j));
    for(k = 0; k < j; k++)
      d -= creal(A_(j, k) * conj(A_(j, k)));
    if(!(d > 0.0))
      return j + 1;
    d = sqrt(d);
    A_(j, j) = d;
    for(i = j + 1; i < n; i++) {
      cx s = A_(i, j);
      for(k = 0; k < j; k++)
        s -= A_(i, k) * conj(A_(j, k));
      A_(i, j) = s / d;
    }
    for(i = 0; i < j; i++)
      A_(i, j) = 0.0;
  }
  return 0;
}

void
om_potrs(int n, const cx *a, cx *b)
{
  int i, k;
  for(i = 0; i < n; i++) {
    cx s = b[i];
    for(k = 0; k < i; k++)
      s -= A_(i, k) * b[k];
    b[i] = s / A_(i, i);
  }
  for(i = n - 1; i >= 0; i--) {
    cx s = b[i];
    for(k = i + 1; k < n; k++)
      s -= conj(A_(k, i)) * b[k];
    b[i] = s / A_(i, i);
  }
}

/* Cyclic Jacobi (Jacobi 1846; rotation formulas as in Rutishauser's
 * handbook algorithm), complex Hermitian.  Input: lower triangle of a.
 * Output: eigenvalues ascending in w, orthonormal eigenvectors in a. */
int
om_heev(int n, cx *a, double *w)
{
  cx *z = calloc((size_t) n * n, sizeof(cx));
  int i, j, p, q, sweep;
  for(j = 0; j < n; j++) {
    A_(j, j) = creal(A_(j, j));
    for(i = j + 1; i < n; i++)
      A_(j, i) = conj(A_(i, j));
    z[j + (size_t) j * n] = 1.0;
  }
  for(sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, diag = 0.0;
    for(j = 0; j < n; j++)
      for(i = 0; i < n; i++) {
        double v = creal(A_(i, j) * conj(A_(i, j)));
        if(i == j) diag += v; else off += v;
      }
    if(off <= 1e-30 * diag || off == 0.0)
      break;
    for(p = 0; p < n - 1; p++)
      for(q = p + 1; q < n; q++) {
        cx apq = A_(p, q);
        double g = cabs(apq), tau, t, c, s;
        cx e;
        if(g == 0.0)
          continue;
        e = apq / g;
        tau = (creal(A_(q, q)) - creal(A_(p, p))) / (2.0 * g);
        t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        c = 1.0 / sqrt(1.0 + t * t);
        s = t * c;
        /* A <- V^H A V, Z <- Z V with the unitary V = [[c, s e], [-s conj(e), c]]
         * on coordinates (p,q); this zeroes A(p,q). */
        for(i = 0; i < n; i++) {
          cx ap = A_(i, p), aq = A_(i, q);
          A_(i, p) = c * ap - s * conj(e) * aq;
          A_(i, q) = s * e * ap + c * aq;
          ap = z[i + (size_t) p * n]; aq = z[i + (size_t) q * n];
          z[i + (size_t) p * n] = c * ap - s * conj(e) * aq;
          z[i + (size_t) q * n] = s * e * ap + c * aq;
        }
        for(i = 0; i < n; i++) {
          cx ap = A_(p, i), aq = A_(q, i);
          A_(p, i) = c * ap - s * e * aq;
          A_(q, i) = s * conj(e) * ap + c * aq;
        }
        A_(p, q) = 0.0;
        A_(q, p) = 0.0;
        A_(p, p) = creal(A_(p, p));
        A_(q, q) = creal(A_(q, q));
      }
  }
  for(i = 0; i < n; i++)
    w[i] = creal(A_(i, i));
  /* sort ascending */
  for(i = 0; i < n; i++) {
    int m = i;
    for(j = i + 1; j < n; j++)
      if(w[j] < w[m])
        m = j;
    if(m != i) {
      double tw = w[i];
      w[i] = w[m]; w[m] = tw;
      for(j = 0; j < n; j++) {
        cx tz = z[j + (size_t) i * n];
        z[j + (size_t) i * n] = z[j + (size_t) m * n];
        z[j + (size_t) m * n] = tz;
      }
    }
  }
  memcpy(a, z, sizeof(cx) * (size_t) n * n);
  free(z);
  return 0;
}

/* A x = w B x, itype 1 (zhegv, linalg.c:285-317): B = L L^H,
 * C = L^-1 A L^-H, x = L^-H y.  Inputs: lower triangles.  Output:
 * eigenvectors in a (B-orthonormal), Cholesky factor in b. */
int
om_hegv(int n, cx *a, cx *b, double *w)
{
  int info, i, j, k;
  cx *c;
  info = om_potrf(n, b);
  if(info)
    return n + info;
  c = calloc((size_t) n * n, sizeof(cx));
  for(j = 0; j < n; j++)
    for(i = j; i < n; i++) {
      c[i + (size_t) j * n] = A_(i, j);
      c[j + (size_t) i * n] = conj(A_(i, j));
    }
  /* C <- L^-1 C */
  for(j = 0; j < n; j++)
    for(i = 0; i < n; i++) {
      cx s = c[i + (size_t) j * n];
      for(k = 0; k < i; k++)
        s -= b[i + (size_t) k * n] * c[k + (size_t) j * n];
      c[i + (size_t) j * n] = s / b[i + (size_t) i * n];
    }
  /* C <- C L^-H : row-wise solve with L^H on the right */
  for(i = 0; i < n; i++)
    for(j = 0; j < n; j++) {
      cx s = c[i + (size_t) j * n];
      for(k = 0; k < j; k++)
        s -= c[i + (size_t) k * n] * conj(b[j + (size_t) k * n]);
      c[i + (size_t) j * n] = s / b[j + (size_t) j * n];
    }
  info = om_heev(n, c, w);
  /* X = L^-H Y */
  for(j = 0; j < n; j++)
    for(i = n - 1; i >= 0; i--) {
      cx s = c[i + (size_t) j * n];
      for(k = i + 1; k < n; k++)
        s -= conj(b[k + (size_t) i * n]) * c[k + (size_t) j * n];
      c[i + (size_t) j * n] = s / b[i + (size_t) i * n];
    }
  memcpy(a, c, sizeof(cx) * (size_t) n * n);
  free(c);
  return info;
}

/* Rayleigh-Ritz on a possibly rank-deficient basis, SVQB style (Stathopoulos
 * and Wu, SIAM J. Sci. Comput. 23 (2002)): scale Gm to unit diagonal,
 * diagonalise it, drop directions whose eigenvalue is below drop*max, and
 * solve the standard problem in the remaining orthonormal basis.
 * ga, gm: full Hermitian n x n.  Returns the number of kept directions
 * (negative if fewer than m), the lowest m Ritz values in theta and the
 * coefficients (n x m, Gm-orthonormal) in c. */
int
om_rr_svqb(int n, const cx *ga, const cx *gm, int m, double drop,
           cx *c, double *theta)
{
  double *d = malloc(sizeof(double) * n), *sig = malloc(sizeof(double) * n);
  double *th = malloc(sizeof(double) * n);
  cx *v = malloc(sizeof(cx) * (size_t) n * n), *t, *at;
  int i, j, k, l, r, keep0;
  double smax;
  for(i = 0; i < n; i++) {
    double g = creal(gm[i + (size_t) i * n]);
    d[i] = g > 0.0 ? 1.0 / sqrt(g) : 0.0;
  }
  for(j = 0; j < n; j++)
    for(i = 0; i < n; i++)
      v[i + (size_t) j * n] = d[i] * gm[i + (size_t) j * n] * d[j];
  om_heev(n, v, sig);
  smax = sig[n - 1];
  for(keep0 = 0; keep0 < n && !(sig[keep0] > drop * smax); keep0++)
    ;
  r = n - keep0;
  if(r < m) {
    free(d); free(sig); free(th); free(v);
    return -r - 1;
  }
  t = malloc(sizeof(cx) * (size_t) n * r);
  at = calloc((size_t) r * r, sizeof(cx));
  for(l = 0; l < r; l++) {
    double sc = 1.0 / sqrt(sig[keep0 + l]);
    for(i = 0; i < n; i++)
      t[i + (size_t) l * n] = d[i] * v[i + (size_t) (keep0 + l) * n] * sc;
  }
  /* at = T^H ga T */
  for(l = 0; l < r; l++)
    for(k = 0; k < r; k++) {
      cx s = 0.0;
      for(j = 0; j < n; j++) {
        cx gt = 0.0;
        for(i = 0; i < n; i++)
          gt += ga[j + (size_t) i * n] * t[i + (size_t) l * n];
        s += conj(t[j + (size_t) k * n]) * gt;
      }
      at[k + (size_t) l * r] = s;
    }
  om_heev(r, at, th);
  for(l = 0; l < m; l++) {
    theta[l] = th[l];
    for(i = 0; i < n; i++) {
      cx s = 0.0;
      for(k = 0; k < r; k++)
        s += t[i + (size_t) k * n] * at[k + (size_t) l * r];
      c[i + (size_t) l * n] = s;
    }
  }
  free(d); free(sig); free(th); free(v); free(t); free(at);
  return r;
}

#undef A_

/* ------------------------------------------------------------
 * Multigrid hierarchy for one Bloch parameter
 * (vcycle_edge2d edge2d.c:5707-5754, vcycle_node2d node2d.c:1352-1389)
 * ------------------------------------------------------------ */

struct om_mg {
  int n0, L;
  double **kappa;             /* per level */
  cx **b, **x, **d;           /* edge work vectors per level */
  cx **bg, **xg, **dg;        /* node work vectors per level */
  cx *Ae, *An;                /* coarse Cholesky factors */
  cx xf, yf;
};

om_mg *
om_mg_new(int n0, int L, const double *kappa_fine)
{
  om_mg *h = calloc(1, sizeof(om_mg));
  int l;
  h->n0 = n0; h->L = L;
  h->kappa = calloc(L + 1, sizeof(double *));
  h->b = calloc(L + 1, sizeof(cx *)); h->x = calloc(L + 1, sizeof(cx *));
  h->d = calloc(L + 1, sizeof(cx *)); h->bg = calloc(L + 1, sizeof(cx *));
  h->xg = calloc(L + 1, sizeof(cx *)); h->dg = calloc(L + 1, sizeof(cx *));
  for(l = L; l >= 0; l--) {
    int n = n0 << l;
    h->kappa[l] = malloc(sizeof(double) * n * n);
    if(l == L)
      memcpy(h->kappa[l], kappa_fine, sizeof(double) * n * n);
    else
      om_coarsen_kappa(2 * n, h->kappa[l + 1], h->kappa[l]);
    h->b[l] = calloc(2L * n * n, sizeof(cx)); h->x[l] = calloc(2L * n * n, sizeof(cx));
    h->d[l] = calloc(2L * n * n, sizeof(cx));
    h->bg[l] = calloc((long) n * n, sizeof(cx)); h->xg[l] = calloc((long) n * n, sizeof(cx));
    h->dg[l] = calloc((long) n * n, sizeof(cx));
  }
  h->Ae = malloc(sizeof(cx) * 4 * (size_t) n0 * n0 * n0 * n0);
  h->An = malloc(sizeof(cx) * (size_t) n0 * n0 * n0 * n0);
  om_mg_set_bloch(h, 1.0, 1.0);
  return h;
}

void
om_mg_free(om_mg *h)
{
  int l;
  for(l = 0; l <= h->L; l++) {
    free(h->kappa[l]); free(h->b[l]); free(h->x[l]); free(h->d[l]);
    free(h->bg[l]); free(h->xg[l]); free(h->dg[l]);
  }
  free(h->kappa); free(h->b); free(h->x); free(h->d);
  free(h->bg); free(h->xg); free(h->dg);
  free(h->Ae); free(h->An);
  free(h);
}

const double *
om_mg_kappa(const om_mg *h, int l)
{
  return h->kappa[l];
}

/* Refactor the coarse solvers for new Bloch factors (exp_bloch2d.c:782-810) */
int
om_mg_set_bloch(om_mg *h, cx xf, cx yf)
{
  int n0 = h->n0, info;
  h->xf = xf; h->yf = yf;
  om_dense_edge(n0, h->kappa[0], xf, yf, 1.0, 1.0, h->Ae);
  info = om_potrf(2 * n0 * n0, h->Ae);
  om_dense_node(n0, xf, yf, 1, h->An);
  info |= om_potrf(n0 * n0, h->An) << 8;
  return info;
}

void
om_vcycle_edge(om_mg *h, int L, int nu, int coarse, const cx *b, cx *x)
{
  int l, s, n;
  long len;
  cx xf = h->xf, yf = h->yf;
  memcpy(h->b[L], b, sizeof(cx) * 2 * (size_t) (h->n0 << L) * (h->n0 << L));
  memcpy(h->x[L], x, sizeof(cx) * 2 * (size_t) (h->n0 << L) * (h->n0 << L));
  for(l = L; l > 0; l--) {
    n = h->n0 << l;
    len = 2L * n * n;
    for(s = 0; s < nu; s++)
      om_gs_edge(n, h->kappa[l], xf, yf, 1.0, 1.0, 0, h->b[l], h->x[l]);
    memcpy(h->d[l], h->b[l], sizeof(cx) * len);
    om_addeval_edge(n, h->kappa[l], xf, yf, -1.0, -1.0, h->x[l], h->d[l]);
    memset(h->b[l - 1], 0, sizeof(cx) * len / 4);
    om_restrict_edge(n / 2, xf, yf, 1.0, h->d[l], h->b[l - 1]);
    memset(h->x[l - 1], 0, sizeof(cx) * len / 4);
  }
  n = h->n0;
  if(coarse) {
    memcpy(h->x[0], h->b[0], sizeof(cx) * 2 * n * n);
    om_potrs(2 * n * n, h->Ae, h->x[0]);
  }
  else
    for(s = 0; s < nu; s++)
      om_gs_edge(n, h->kappa[0], xf, yf, 1.0, 1.0, 2, h->b[0], h->x[0]);
  for(l = 1; l <= L; l++) {
    n = h->n0 << l;
    om_prolong_edge(n / 2, xf, yf, 1.0, h->x[l - 1], h->x[l]);
    for(s = 0; s < nu; s++)
      om_gs_edge(n, h->kappa[l], xf, yf, 1.0, 1.0, 1, h->b[l], h->x[l]);
  }
  memcpy(x, h->x[L], sizeof(cx) * 2 * (size_t) (h->n0 << L) * (h->n0 << L));
}

/* The Hiptmair cycle (hcycle_edge2d, edge2d.c:5756-5823): per level down,
 * nu forward point GS sweeps, then a correction in the gradients (G of nu
 * forward node GS sweeps on G^H of the residual), the residual restricted;
 * the coarse dense solve (or nu symmetric point GS sweeps); per level up,
 * the prolongated correction, a gradient correction with backward node
 * sweeps and nu backward point GS sweeps. */
void
om_hcycle_edge(om_mg *h, int L, int nu, int coarse, const cx *b, cx *x)
{
  int l, s, n;
  long len;
  cx xf = h->xf, yf = h->yf;
  memcpy(h->b[L], b, sizeof(cx) * 2 * (size_t) (h->n0 << L) * (h->n0 << L));
  memcpy(h->x[L], x, sizeof(cx) * 2 * (size_t) (h->n0 << L) * (h->n0 << L));
  for(l = L; l > 0; l--) {
    n = h->n0 << l;
    len = 2L * n * n;
    for(s = 0; s < nu; s++)
      om_gs_edge_simple(n, h->kappa[l], xf, yf, 1.0, 1.0, 0, h->b[l], h->x[l]);
    memcpy(h->d[l], h->b[l], sizeof(cx) * len);
    om_addeval_edge(n, h->kappa[l], xf, yf, -1.0, -1.0, h->x[l], h->d[l]);
    memset(h->bg[l], 0, sizeof(cx) * len / 2);
    om_adjgradient(n, xf, yf, 1.0, h->d[l], h->bg[l]);
    memset(h->xg[l], 0, sizeof(cx) * len / 2);
    for(s = 0; s < nu; s++)
      om_gs_node(n, xf, yf, 1.0, 0, h->bg[l], h->xg[l]);
    om_gradient(n, xf, yf, 1.0, h->xg[l], h->x[l]);
    memcpy(h->d[l], h->b[l], sizeof(cx) * len);
    om_addeval_edge(n, h->kappa[l], xf, yf, -1.0, -1.0, h->x[l], h->d[l]);
    memset(h->b[l - 1], 0, sizeof(cx) * len / 4);
    om_restrict_edge(n / 2, xf, yf, 1.0, h->d[l], h->b[l - 1]);
    memset(h->x[l - 1], 0, sizeof(cx) * len / 4);
  }
  n = h->n0;
  if(coarse) {
    memcpy(h->x[0], h->b[0], sizeof(cx) * 2 * n * n);
    om_potrs(2 * n * n, h->Ae, h->x[0]);
  }
  else
    for(s = 0; s < nu; s++)
      om_gs_edge_simple(n, h->kappa[0], xf, yf, 1.0, 1.0, 2, h->b[0], h->x[0]);
  for(l = 1; l <= L; l++) {
    n = h->n0 << l;
    len = 2L * n * n;
    om_prolong_edge(n / 2, xf, yf, 1.0, h->x[l - 1], h->x[l]);
    memcpy(h->d[l], h->b[l], sizeof(cx) * len);
    om_addeval_edge(n, h->kappa[l], xf, yf, -1.0, -1.0, h->x[l], h->d[l]);
    memset(h->bg[l], 0, sizeof(cx) * len / 2);
    om_adjgradient(n, xf, yf, 1.0, h->d[l], h->bg[l]);
    memset(h->xg[l], 0, sizeof(cx) * len / 2);
    for(s = 0; s < nu; s++)
      om_gs_node(n, xf, yf, 1.0, 1, h->bg[l], h->xg[l]);
    om_gradient(n, xf, yf, 1.0, h->xg[l], h->x[l]);
    for(s = 0; s < nu; s++)
      om_gs_edge_simple(n, h->kappa[l], xf, yf, 1.0, 1.0, 1, h->b[l], h->x[l]);
  }
  memcpy(x, h->x[L], sizeof(cx) * 2 * (size_t) (h->n0 << L) * (h->n0 << L));
}

void
om_vcycle_node(om_mg *h, int L, int nu, int coarse, const cx *b, cx *x)
{
  int l, s, n;
  long len;
  cx xf = h->xf, yf = h->yf;
  memcpy(h->bg[L], b, sizeof(cx) * (size_t) (h->n0 << L) * (h->n0 << L));
  memcpy(h->xg[L], x, sizeof(cx) * (size_t) (h->n0 << L) * (h->n0 << L));
  for(l = L; l > 0; l--) {
    n = h->n0 << l;
    len = (long) n * n;
    for(s = 0; s < nu; s++)
      om_gs_node(n, xf, yf, 1.0, 0, h->bg[l], h->xg[l]);
    memcpy(h->dg[l], h->bg[l], sizeof(cx) * len);
    om_addeval_node(n, xf, yf, -1.0, h->xg[l], h->dg[l]);
    memset(h->bg[l - 1], 0, sizeof(cx) * len / 4);
    om_restrict_node(n / 2, xf, yf, 1.0, h->dg[l], h->bg[l - 1]);
    memset(h->xg[l - 1], 0, sizeof(cx) * len / 4);
  }
  n = h->n0;
  if(coarse) {
    memcpy(h->xg[0], h->bg[0], sizeof(cx) * n * n);
    om_potrs(n * n, h->An, h->xg[0]);
  }
  else
    for(s = 0; s < nu; s++)
      om_gs_node(n, xf, yf, 1.0, 2, h->bg[0], h->xg[0]);
  for(l = 1; l <= L; l++) {
    n = h->n0 << l;
    om_prolong_node(n / 2, xf, yf, 1.0, h->xg[l - 1], h->xg[l]);
    for(s = 0; s < nu; s++)
      om_gs_node(n, xf, yf, 1.0, 1, h->bg[l], h->xg[l]);
  }
  memcpy(x, h->xg[L], sizeof(cx) * (size_t) (h->n0 << L) * (h->n0 << L));
}

/* ------------------------------------------------------------
 * Eigensolver: block PINVIT + Ritz (exp_bloch2d.c:956-1053) and LOBPCG
 * (test_lobpcg2d.c:217-365, with the search direction P of Knyazev's
 * method in place of the previous iterate and SVQB in place of the
 * Householder M-orthonormalisation).
 * ------------------------------------------------------------ */

typedef struct {
  const om_opts *o;
  om_mg *h;
  int l, n;            /* current level and its intervals */
  long len;            /* 2 n^2 */
  cx *t1, *t2, *tn;    /* scratch (edge, edge, node) */
  double tol;          /* stopping tolerance of the current level */
} ctx_t;

/* k = 0 up to rounding (the reference tests xfactor == 1.0 and yfactor ==
 * 1.0 exactly, edge2d.c:1321-1322; a tolerance keeps a k-point computed as
 * exp(i * 1e-17) on the same side as the coarse node matrix's fixnull test) */
static int
is_gamma(cx xf, cx yf)
{
  return fabs(creal(xf) - 1.0) + fabs(cimag(xf)) + fabs(creal(yf) - 1.0) + fabs(cimag(yf)) < 1e-8;
}

/* e -= G L^-1 G^H M e with `steps` node V-cycles from zero */
static void
lift(ctx_t *c, cx *e)
{
  om_mg *h = c->h;
  int n = c->n;
  memset(c->t1, 0, sizeof(cx) * c->len);
  om_addeval_edge(n, 0, h->xf, h->yf, 0.0, 1.0, e, c->t1);
  memset(c->tn, 0, sizeof(cx) * n * n);
  om_adjgradient(n, h->xf, h->yf, 1.0, c->t1, c->tn);
  {
    cx *xg = calloc((size_t) n * n, sizeof(cx));
    int s;
    for(s = 0; s < c->o->gradient_steps; s++)
      om_vcycle_node(h, c->l, c->o->smoother_steps, 1, c->tn, xg);
    om_gradient(n, h->xf, h->yf, -1.0, xg, e);
    free(xg);
  }
}

/* x = V^prec (A+M) e - mu M e, from zero */
static void
precondition(ctx_t *c, const cx *e, double mu, cx *x)
{
  om_mg *h = c->h;
  int s;
  memset(c->t2, 0, sizeof(cx) * c->len);
  om_addeval_edge(c->n, h->kappa[c->l], h->xf, h->yf, 1.0, 1.0 - mu, e, c->t2);
  memset(x, 0, sizeof(cx) * c->len);
  for(s = 0; s < c->o->prec_steps; s++)
    om_vcycle_edge(h, c->l, c->o->smoother_steps, 1, c->t2, x);
}

/* residual norms of M-normalised vectors, absolute or relative */
static double
residual(ctx_t *c, const cx *e, double mu)
{
  om_mg *h = c->h;
  double r, mn;
  memset(c->t1, 0, sizeof(cx) * c->len);
  om_addeval_edge(c->n, h->kappa[c->l], h->xf, h->yf, 1.0, 1.0 - mu, e, c->t1);
  r = om_norm2(c->len, c->t1);
  if(!c->o->relative)
    return r;
  memset(c->t1, 0, sizeof(cx) * c->len);
  om_addeval_edge(c->n, 0, h->xf, h->yf, 0.0, 1.0, e, c->t1);
  mn = om_norm2(c->len, c->t1);
  return r / (mu * mn);
}

static void
gram(ctx_t *c, int ns, cx **s, cx *ga, cx *gm)
{
  om_mg *h = c->h;
  int i, j;
  cx *ka = malloc(sizeof(cx) * c->len * ns), *km = malloc(sizeof(cx) * c->len * ns);
  memset(ka, 0, sizeof(cx) * c->len * ns);
  memset(km, 0, sizeof(cx) * c->len * ns);
  for(j = 0; j < ns; j++) {
    om_addeval_edge(c->n, h->kappa[c->l], h->xf, h->yf, 1.0, 1.0, s[j], ka + j * c->len);
    om_addeval_edge(c->n, 0, h->xf, h->yf, 0.0, 1.0, s[j], km + j * c->len);
  }
  for(j = 0; j < ns; j++)
    for(i = 0; i < ns; i++) {
      ga[i + (size_t) j * ns] = om_dot(c->len, s[i], ka + j * c->len);
      gm[i + (size_t) j * ns] = om_dot(c->len, s[i], km + j * c->len);
    }
  free(ka); free(km);
}

/* combine: out_j = sum_i coef(i,j) in_i, i < ns, j < m (out distinct from in) */
static void
combine(long len, int ns, cx **in, int m, const cx *coef, int ldc, cx **out)
{
  int i, j;
  for(j = 0; j < m; j++) {
    long k;
    memset(out[j], 0, sizeof(cx) * len);
    for(i = 0; i < ns; i++) {
      cx a = coef[i + (size_t) j * ldc];
#pragma omp parallel for schedule(static)
      for(k = 0; k < len; k++)
        out[j][k] += a * in[i][k];
    }
  }
}

typedef struct {
  cx **e, **p, **x, **u, **w;   /* m vectors each */
  double *mu, *res;
  int have_p;
} block_t;

static void
rayleigh(ctx_t *c, block_t *B)
{
  om_mg *h = c->h;
  int i, m = c->o->m;
  for(i = 0; i < m; i++) {
    cx p1 = om_energyprod_edge(c->n, h->kappa[c->l], h->xf, h->yf, 1.0, 1.0, B->e[i], B->e[i]);
    cx p2 = om_massprod_edge(c->n, h->xf, h->yf, B->e[i], B->e[i]);
    B->mu[i] = creal(p1 / p2);
    B->res[i] = residual(c, B->e[i], B->mu[i]);
  }
}

static int
pinvit_step(ctx_t *c, block_t *B)
{
  const om_opts *o = c->o;
  om_mg *h = c->h;
  int m = o->m, i, j, info;
  cx *ga = malloc(sizeof(cx) * m * m), *gm = malloc(sizeof(cx) * m * m);
  for(i = 0; i < m; i++) {
    precondition(c, B->e[i], B->mu[i], B->x[i]);
  }
  for(i = 0; i < m; i++) {
    long k;
    for(k = 0; k < c->len; k++)
      B->e[i][k] -= B->x[i][k];
    if(o->center && is_gamma(h->xf, h->yf))
      om_center_edge(c->n, B->e[i]);
    lift(c, B->e[i]);
  }
  gram(c, m, B->e, ga, gm);
  for(j = 0; j < m; j++)
    for(i = 0; i < j; i++) {
      ga[i + (size_t) j * m] = 0.0;
      gm[i + (size_t) j * m] = 0.0;
    }
  info = om_hegv(m, ga, gm, B->mu);
  if(!info) {
    combine(c->len, m, B->e, m, ga, m, B->u);
    for(i = 0; i < m; i++) {
      cx *t = B->e[i]; B->e[i] = B->u[i]; B->u[i] = t;
      B->res[i] = residual(c, B->e[i], B->mu[i]);
    }
  }
  free(ga); free(gm);
  return info;
}

static double
lobpcg_drop(void)
{
  const char *e = getenv("OM_DROP");
  return e ? atof(e) : 1e-10;
}

/* Soft locking (Knyazev, SIAM J. Sci. Comput. 23 (2001), BLOPEX): a column
 * whose residual is at or below the tolerance keeps its Ritz vector in the
 * basis but contributes no X or P column, so noise-level corrections of
 * converged pairs cannot spoil the small problem. */
static int
lobpcg_step(ctx_t *c, block_t *B)
{
  const om_opts *o = c->o;
  om_mg *h = c->h;
  int m = o->m, ns = B->have_p ? 3 * m : 2 * m, i, j, r, na = 0, nr;
  cx **s = malloc(sizeof(cx *) * ns);
  cx *ga = malloc(sizeof(cx) * ns * ns), *gm = malloc(sizeof(cx) * ns * ns);
  cx *coef = calloc((size_t) ns * m, sizeof(cx));
  int *idx = malloc(sizeof(int) * ns);
  double *theta = malloc(sizeof(double) * m);
  cx *sa, *sm, *sc;
  for(i = 0; i < m; i++) {
    precondition(c, B->e[i], B->mu[i], B->x[i]);
    if(o->center && is_gamma(h->xf, h->yf))
      om_center_edge(c->n, B->x[i]);
    lift(c, B->x[i]);
  }
  for(i = 0; i < m; i++) {
    s[i] = B->e[i];
    s[m + i] = B->x[i];
    if(B->have_p)
      s[2 * m + i] = B->p[i];
  }
  gram(c, ns, s, ga, gm);
  /* reduced basis: all of E, X and P of the unlocked columns */
  for(i = 0; i < m; i++)
    idx[na++] = i;
  for(j = 1; j < ns / m; j++)
    for(i = 0; i < m; i++)
      if(B->res[i] > c->tol)
        idx[na++] = j * m + i;
  sa = malloc(sizeof(cx) * na * na); sm = malloc(sizeof(cx) * na * na);
  sc = malloc(sizeof(cx) * na * m);
  for(j = 0; j < na; j++)
    for(i = 0; i < na; i++) {
      sa[i + (size_t) j * na] = ga[idx[i] + (size_t) idx[j] * ns];
      sm[i + (size_t) j * na] = gm[idx[i] + (size_t) idx[j] * ns];
    }
  nr = om_rr_svqb(na, sa, sm, m, lobpcg_drop(), sc, theta);
  r = nr;
  if(r < 0) {
    free(s); free(ga); free(gm); free(coef); free(theta); free(idx);
    free(sa); free(sm); free(sc);
    return 1;
  }
  for(j = 0; j < m; j++)
    for(i = 0; i < na; i++)
      coef[idx[i] + (size_t) j * ns] = sc[i + (size_t) j * na];
  /* P = [X P] C[m:, :] into u, E = S C into w, then rotate the buffers */
  combine(c->len, ns - m, s + m, m, coef + m, ns, B->u);
  combine(c->len, ns, s, m, coef, ns, B->w);
  for(i = 0; i < m; i++) {
    cx *t = B->p[i];
    B->p[i] = B->u[i];
    B->u[i] = t;
    t = B->e[i];
    B->e[i] = B->w[i];
    B->w[i] = t;
    B->mu[i] = theta[i];
  }
  B->have_p = 1;
  for(i = 0; i < m; i++) {
    if(o->lift_e) {
      if(o->center && is_gamma(h->xf, h->yf))
        om_center_edge(c->n, B->e[i]);
      lift(c, B->e[i]);
    }
    B->res[i] = residual(c, B->e[i], B->mu[i]);
  }
  free(s); free(ga); free(gm); free(coef); free(theta); free(idx);
  free(sa); free(sm); free(sc);
  return 0;
}

static double
maxres(const block_t *B, int ieigs)
{
  double r = 0.0;
  int i;
  for(i = 0; i < ieigs; i++)
    if(B->res[i] > r)
      r = B->res[i];
  return r;
}

static int
iterate(ctx_t *c, block_t *B, int maxsteps)
{
  int k;
  B->have_p = 0;
  c->tol = c->l < c->o->L && c->o->nested_tol > 0.0 ? c->o->nested_tol : c->o->tol;
  for(k = 0; k < maxsteps && maxres(B, c->o->ieigs) > c->tol; k++) {
    int info = c->o->method ? lobpcg_step(c, B) : pinvit_step(c, B);
    if(info)
      return -(k + 1);
    if(getenv("OM_DEBUG")) {
      int i;
      fprintf(stderr, "l=%d step %d:", c->l, k);
      for(i = 0; i < c->o->m; i++)
        fprintf(stderr, " %.1e", B->res[i]);
      fprintf(stderr, "\n");
    }
  }
  return k;
}

static cx **
alloc_block(int m, long len)
{
  cx **b = malloc(sizeof(cx *) * m);
  int i;
  for(i = 0; i < m; i++)
    b[i] = calloc(len, sizeof(cx));
  return b;
}

static void
free_block(cx **b, int m)
{
  int i;
  for(i = 0; i < m; i++)
    free(b[i]);
  free(b);
}

/* Coarse generalized eigenproblem and nested iteration for one k
 * (exp_bloch2d.c:530-732); returns the block steps at the finest level. */
static int
cold_start(ctx_t *c, block_t *B, cx **scratch_levels)
{
  const om_opts *o = c->o;
  om_mg *h = c->h;
  int n0 = o->n0, N = 2 * n0 * n0, m = o->m, i, ev, l, steps = 0;
  cx *A = malloc(sizeof(cx) * (size_t) N * N), *M = malloc(sizeof(cx) * (size_t) N * N);
  double *w = malloc(sizeof(double) * N);
  om_dense_edge(n0, h->kappa[0], h->xf, h->yf, 1.0, 0.0, A);
  om_dense_edge(n0, h->kappa[0], h->xf, h->yf, 0.0, 1.0, M);
  om_hegv(N, A, M, w);
  for(ev = 0; ev < N && fabs(w[ev]) < 1e-8; ev++)
    ;
  if(ev + m > N) {
    free(A); free(M); free(w);
    return -1000;
  }
  for(i = 0; i < m; i++)
    memcpy(scratch_levels[i], A + (size_t) (ev + i) * N, sizeof(cx) * N);
  free(A); free(M); free(w);
  for(l = 1; l <= o->L; l++) {
    int n = n0 << l;
    c->l = l; c->n = n; c->len = 2L * n * n;
    for(i = 0; i < m; i++) {
      memset(B->e[i], 0, sizeof(cx) * c->len);
      om_prolong_edge(n / 2, h->xf, h->yf, 1.0, scratch_levels[i], B->e[i]);
    }
    rayleigh(c, B);
    steps = iterate(c, B, l == o->L ? o->max_steps : o->max_nested);
    if(steps < 0)
      return steps;
    if(l < o->L)
      for(i = 0; i < m; i++)
        memcpy(scratch_levels[i], B->e[i], sizeof(cx) * c->len);
  }
  return steps;
}

/* Rayleigh-Ritz warm start from earlier k-points (exp_bloch2d.c:814-895):
 * basis = the first ieigs vectors of each available earlier block. */
static int
warm_start(ctx_t *c, block_t *B, int nprev, cx ***prev)
{
  const om_opts *o = c->o;
  int m = o->m, ie = o->ieigs, ns = nprev * ie, i, j, r;
  cx **s = malloc(sizeof(cx *) * ns);
  cx *ga = malloc(sizeof(cx) * ns * ns), *gm = malloc(sizeof(cx) * ns * ns);
  cx *coef = malloc(sizeof(cx) * ns * m);
  double *theta = malloc(sizeof(double) * m);
  for(j = 0; j < nprev; j++)
    for(i = 0; i < ie; i++)
      s[j * ie + i] = prev[j][i];
  if(ns < m) {
    /* no room to extrapolate: keep the previous block */
    for(i = 0; i < m; i++)
      memcpy(B->e[i], prev[0][i], sizeof(cx) * c->len);
    free(s); free(ga); free(gm); free(coef); free(theta);
    return 0;
  }
  gram(c, ns, s, ga, gm);
  r = om_rr_svqb(ns, ga, gm, m, 1e-10, coef, theta);
  if(r < 0) {
    for(i = 0; i < m; i++)
      memcpy(B->e[i], prev[0][i], sizeof(cx) * c->len);
  }
  else
    combine(c->len, ns, s, m, coef, ns, B->e);
  free(s); free(ga); free(gm); free(coef); free(theta);
  return 0;
}

int
om_bloch_solve(const om_opts *o, const double *kappa_fine, int nk,
               const cx *xfs, const cx *yfs, double *lambda_out, int *steps_out,
               double *res_out, cx *evec_out)
{
  return om_bloch_solve_timed(o, kappa_fine, nk, xfs, yfs, lambda_out, steps_out, res_out, evec_out, 0);
}

/* The same, with the wall-clock seconds of every k-point (its coarse
 * refactorisation, start block and block steps; the first wave's k-points
 * share their cold start, which is charged to the first of them). */
int
om_bloch_solve_timed(const om_opts *o, const double *kappa_fine, int nk,
                     const cx *xfs, const cx *yfs, double *lambda_out, int *steps_out,
                     double *res_out, cx *evec_out, double *seconds_out)
{
  int m = o->m, W = o->wave > 0 ? o->wave : 1, n = o->n0 << o->L, kk, i;
  long len = 2L * n * n;
  om_mg *h = om_mg_new(o->n0, o->L, kappa_fine);
  ctx_t c;
  block_t B;
  cx ***store = calloc(nk, sizeof(cx **));
  cx **lev = alloc_block(m, len / 4);
  int status = 0;

  c.o = o; c.h = h;
  c.t1 = calloc(len, sizeof(cx)); c.t2 = calloc(len, sizeof(cx));
  c.tn = calloc(len / 2, sizeof(cx));
  B.e = alloc_block(m, len); B.p = alloc_block(m, len);
  B.x = alloc_block(m, len); B.u = alloc_block(m, len); B.w = alloc_block(m, len);
  B.mu = malloc(sizeof(double) * m); B.res = malloc(sizeof(double) * m);

  for(kk = 0; kk < nk && status == 0; kk++) {
    int steps;
    double t0 = omp_get_wtime();
    om_mg_set_bloch(h, xfs[kk], yfs[kk]);
    /* a k-point whose predecessor is Gamma starts cold: the Gamma block is
     * centred and lacks the two lowest bands of every k != 0 (they tend to
     * the constant fields that centring removes), and a warm start without
     * them took 50-60 block steps where a cold start takes 12 */
    if(kk < W || is_gamma(xfs[kk - W], yfs[kk - W])) {
      steps = cold_start(&c, &B, lev);
    }
    else {
      cx **prev[3];
      int np = 0, q;
      int order = o->extrapolation == '2' ? 3 : o->extrapolation == '1' ? 2 : 1;
      c.l = o->L; c.n = n; c.len = len;
      for(q = 1; q <= order && kk - q * W >= 0; q++)
        prev[np++] = store[kk - q * W];
      if(o->extrapolation == 'n' || np == 1) {
        for(i = 0; i < m; i++)
          memcpy(B.e[i], prev[0][i], sizeof(cx) * len);
      }
      else
        warm_start(&c, &B, np, prev);
      rayleigh(&c, &B);
      steps = iterate(&c, &B, o->max_steps);
    }
    if(steps < 0) {
      status = steps;
      break;
    }
    steps_out[kk] = steps;
    if(seconds_out) seconds_out[kk] = omp_get_wtime() - t0;
    for(i = 0; i < m; i++) {
      lambda_out[(size_t) kk * m + i] = B.mu[i] - 1.0;
      res_out[(size_t) kk * m + i] = B.res[i];
    }
    store[kk] = alloc_block(m, len);
    for(i = 0; i < m; i++)
      memcpy(store[kk][i], B.e[i], sizeof(cx) * len);
    if(evec_out)
      for(i = 0; i < m; i++)
        memcpy(evec_out + ((size_t) kk * m + i) * len, B.e[i], sizeof(cx) * len);
    if(kk - 3 * W >= 0 && store[kk - 3 * W]) {
      free_block(store[kk - 3 * W], m);
      store[kk - 3 * W] = 0;
    }
  }
  for(kk = 0; kk < nk; kk++)
    if(store[kk])
      free_block(store[kk], m);
  free(store);
  free_block(lev, m);
  free_block(B.e, m); free_block(B.p, m); free_block(B.x, m); free_block(B.u, m);
  free_block(B.w, m);
  free(B.mu); free(B.res);
  free(c.t1); free(c.t2); free(c.tn);
  om_mg_free(h);
  return status;
}

/* Eigenvector continuity and Chern partial sums along consecutive
 * k-points, as the reference's Bloch scan does them after each point
 * (exp_bloch2d.c:1058-1216): vecs holds nk blocks of m vectors (len each),
 * adjusted in place; eold0 / eold1 are the adjusted blocks of the two points
 * before (eold1 zero at the second point, exp_bloch2d.c:773-777); every mass
 * product is taken with the current point's Bloch factors. */
void
om_continuity(int n, int nk, const cx *xfs, const cx *yfs, int m, int ieigs, const int *vertex,
              int continuity, int chern_vectors, cx *vecs, double *lambda, cx *chern, int *sign)
{
  long len = 2L * n * n, q;
  cx *x = malloc(sizeof(cx) * len), *zero = calloc(len, sizeof(cx));
  cx *chs = calloc(chern_vectors > 0 ? chern_vectors : 1, sizeof(cx));
  int l, i, j, swaps = 0;
  for(i = 0; i < chern_vectors; i++) chern[i] = 0.0;
  if(sign) sign[0] = 0;
  for(l = 1; l < nk; l++) {
    cx *e = vecs + (size_t) l * m * len, *e0 = vecs + (size_t) (l - 1) * m * len;
    cx *e1 = l > 1 ? vecs + (size_t) (l - 2) * m * len : 0;
    int oldvertex = vertex[l - 1];
#define EV(b, i) ((b) ? (b) + (size_t) (i) * len : zero)
#define MP(a, b) om_massprod_edge(n, xfs[l], yfs[l], (a), (b))
    if(continuity == 'r')
      for(i = 0; i < ieigs; i++) {
        double opt, a;
        int k = i;
        if(oldvertex)
          memcpy(x, EV(e0, i), sizeof(cx) * len);
        else {
          for(q = 0; q < len; q++) x[q] = 2.0 * EV(e0, i)[q] - EV(e1, i)[q];
          a = sqrt(creal(MP(x, x)));
          for(q = 0; q < len; q++) x[q] /= a;
        }
        opt = cabs(MP(EV(e, i), x));
        for(j = i + 1; j < ieigs; j++) {
          a = cabs(MP(EV(e, j), x));
          if(a > opt) { k = j; opt = a; }
        }
        if(k != i) {
          double tl;
          for(q = 0; q < len; q++) {
            cx t = EV(e, i)[q];
            EV(e, i)[q] = EV(e, k)[q];
            EV(e, k)[q] = t;
          }
          tl = lambda[(size_t) l * m + i];
          lambda[(size_t) l * m + i] = lambda[(size_t) l * m + k];
          lambda[(size_t) l * m + k] = tl;
          swaps++;
        }
      }
    if(continuity == 's' || continuity == 'r')
      for(i = 0; i < m; i++) {
        cx p;
        if(oldvertex)
          p = MP(EV(e, i), EV(e0, i));
        else {
          for(q = 0; q < len; q++) x[q] = 2.0 * EV(e0, i)[q] - EV(e1, i)[q];
          p = MP(EV(e, i), x);
        }
        p /= cabs(p);
        for(q = 0; q < len; q++) EV(e, i)[q] *= p;
      }
    for(i = 0; i < chern_vectors; i++) {
      cx chup;
      if(oldvertex) {
        for(q = 0; q < len; q++) x[q] = EV(e, i)[q] - EV(e0, i)[q];
        chup = 0.5 * I * MP(EV(e0, i), x);
      }
      else {
        for(q = 0; q < len; q++) x[q] = EV(e, i)[q] - EV(e1, i)[q];
        chup = 0.5 * I * MP(EV(e0, i), x);
        if(vertex[l]) {
          for(q = 0; q < len; q++) x[q] = EV(e, i)[q] - EV(e0, i)[q];
          chup += 0.5 * I * MP(EV(e, i), x);
        }
      }
      chs[i] += chup;
      chern[(size_t) l * chern_vectors + i] = chs[i];
    }
    if(sign) sign[l] = swaps;
#undef EV
#undef MP
  }
  free(x); free(zero); free(chs);
}

/* d lambda_i / d eps_c = -axy kappa_c^2 |curl_c e_i|^2 for M-normalised e_i
 * (from the cell term of the operator, edge2d.c:1504-1514, with kappa =
 * 1/eps); grad_c = sum_i w_i d lambda_i / d eps_c. */
void
om_eps_sensitivity(int n, const double *kappa, cx xf, cx yf, int nvec,
                   const cx *e, const double *weights, double *grad)
{
  double axy = (double) n * n;
  long len = 2L * n * n;
  int i, j;
#pragma omp parallel for private(i) schedule(static)
  for(j = 0; j < n; j++)
    for(i = 0; i < n; i++) {
      double s = 0.0, k = kappa[i + j * n];
      int v;
      for(v = 0; v < nvec; v++) {
        const cx *x = e + (size_t) v * len;
        cx curl = XE(x, i, j) - XE(x, i, j + 1) - YE(x, i, j) + YE(x, i + 1, j);
        s += weights[v] * creal(curl * conj(curl));
      }
      grad[i + j * n] = -axy * k * k * s;
    }
}

int
om_max_threads(void)
{
  return omp_get_max_threads();
}

void
om_set_threads(int t)
{
  omp_set_num_threads(t);
}
