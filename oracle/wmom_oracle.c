/*
 * wmom_oracle.c -- CPU oracle for the thin-wire MoM fill-and-solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this file; only tests/, __graft_entry__.smoke() and the cpu_baseline /
 * reference legs of bench.py use it, and only as the checker.
 *
 * It restates, in plain C, the reference's CPU impedance-matrix fill
 * ("wersja referencyjna/Zmatrix.cpp") and LAPACK's unblocked LU with partial
 * pivoting (zgetf2 + zgetrs semantics, the algorithm behind the reference's
 * LAPACKE_zgetrf / LAPACKE_zgetrs calls in "wersja referencyjna/Wire_MoM.cu"
 * lines 372 and 382).  The blocked, threaded LU used for large sizes is the
 * system LAPACK reached from Python (oracle/oracle.py).
 *
 * Geometry arrays follow the reference layout produced by configwire()
 * (Configuration.cpp:112-520): 0-based storage, 1-based node/segment values,
 * second columns at offset nsmax (ise/ips), ipc signed (junction functions
 * are negative, always used through abs()).
 *
 * Parity is pinned by tests/test_oracle_golden.py: against the Z_in values the
 * reference printed in its run logs, and against the reference's own zmatrix()
 * compiled from its sources (recipe oracle/build.py -> oracle/_ref/).
 *
 * Compile with -ffp-contract=off so that x86-64 and aarch64 builds round the
 * same way (no fused multiply-add contraction).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  double re, im;
} cplx;

static inline cplx c_make(double r, double i) {
  cplx z;
  z.re = r;
  z.im = i;
  return z;
}
static inline cplx c_add(cplx a, cplx b) { return c_make(a.re + b.re, a.im + b.im); }
static inline cplx c_sub(cplx a, cplx b) { return c_make(a.re - b.re, a.im - b.im); }
static inline cplx c_scale(cplx a, double s) { return c_make(a.re * s, a.im * s); }
static inline cplx c_mul(cplx a, cplx b) {
  return c_make(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
/* Complex division by the scaled (Smith-style) formula. */
static inline cplx c_div(cplx a, cplx b) {
  double s = fabs(b.re) + fabs(b.im);
  double inv = 1.0 / s;
  double ar = a.re * inv, ai = a.im * inv, br = b.re * inv, bi = b.im * inv;
  double d = 1.0 / (br * br + bi * bi);
  return c_make((ar * br + ai * bi) * d, (ai * br - ar * bi) * d);
}

/* Geometry view over the reference arrays. */
typedef struct {
  const float *x, *y, *z, *rad;
  const int *ipc, *ips, *ise;
  int nsmax;
  float sgnx, sgny, sgnz, sgnenv;
} geom_t;

/* Gauss-Legendre abscissae/weights on [a-b/2, a+b/2] in the half-width form the
 * reference uses (Zmatrix.cpp:285-296, 332). */
#define GL2_C 0.288675134594812882
#define GL4_C1 0.43056815579702629
#define GL4_W1 0.17392742256872693
#define GL4_C2 0.16999052179242813
#define GL4_W2 0.32607257743127307

/* Complete elliptic integral of the first kind, polynomial-logarithmic
 * approximation with the coefficients of Zmatrix.cpp:731-770 (Hastings form,
 * Abramowitz & Stegun 17.3.34). */
static double ell_k(double bet) {
  const double a0 = 1.38629436112, a1 = 0.09666344259, a2 = 0.03590092383,
               a3 = 0.03742563713, a4 = 0.01451196212;
  const double b0 = 0.5, b1 = 0.12498593597, b2 = 0.06880248576, b3 = 0.03328355346,
               b4 = 0.00441787012;
  double m1 = 1.0 - bet * bet;
  double a = a0 + a1 * m1, b = b0 + b1 * m1;
  double m2 = 0.0, m3 = 0.0, m4;
  if (m1 >= 1.0e-18) {
    m2 = m1 * m1;
    a = a + a2 * m2;
    b = b + b2 * m2;
  }
  if (m1 >= 1.0e-12) {
    m3 = m2 * m1;
    a = a + a3 * m3;
    b = b + b3 * m3;
  }
  if (m1 >= 1.0e-9) {
    m4 = m3 * m1;
    a = a + a4 * m4;
    b = b + b4 * m4;
  }
  return a - b * log(m1);
}

/* Regular reduced kernel exp(-jkR)/R with the current ramp (Zmatrix.cpp:667-692).
 * ifun 1: s/dl, ifun 2: (dl-s)/dl, ifun 3: 1. */
static cplx kern_regular(double s, int ifun, double ka, const double rm[3], const double rn[3],
                         const double dc[3], double an, double dl) {
  double dx = rm[0] - rn[0] - s * dc[0];
  double dy = rm[1] - rn[1] - s * dc[1];
  double dz = rm[2] - rn[2] - s * dc[2];
  double r = sqrt(an * an + dx * dx + dy * dy + dz * dz);
  cplx g = c_make(cos(ka * r) / r, -sin(ka * r) / r);
  if (ifun == 1) return c_scale(g, s / dl);
  if (ifun == 2) return c_scale(g, (dl - s) / dl);
  return g;
}

/* Self (identical-segment) kernel: regularised exp term plus the static
 * thin-wire part through K(beta) (Zmatrix.cpp:695-728). */
static cplx kern_self(double s, int ifun, double ka, double dl, double an) {
  const double pi = acos(-1.0);
  double r = 0.5 * dl - s;
  double rr = sqrt(an * an + r * r);
  cplx e = c_make(cos(ka * rr) - 1.0, -sin(ka * rr));
  e = c_make(e.re / rr, e.im / rr);
  double bet = (an + an) / sqrt(4.0 * an * an + r * r);
  double stat = (bet * ell_k(bet) + log(fabs(r / (8.0 * an)))) / (pi * an);
  cplx v = c_make(e.re + stat, e.im);
  if (ifun == 1) return c_scale(v, s / dl);
  if (ifun == 2) return c_scale(v, (dl - s) / dl);
  return v;
}

/* 4-point Gauss on [lo, hi] of the self kernel. */
static cplx gauss4_self(double lo, double hi, int ifun, double ka, double dl, double an) {
  double a = 0.5 * (lo + hi), b = hi - lo;
  double c = GL4_C1 * b;
  cplx v1 = c_add(kern_self(a + c, ifun, ka, dl, an), kern_self(a - c, ifun, ka, dl, an));
  v1 = c_scale(v1, GL4_W1);
  c = GL4_C2 * b;
  cplx v2 = c_add(kern_self(a + c, ifun, ka, dl, an), kern_self(a - c, ifun, ka, dl, an));
  v2 = c_scale(v2, GL4_W2);
  return c_scale(c_add(v1, v2), b);
}

/*
 * Integral of the kernel over one source half-segment of basis n, seen from the
 * observation point rm on observation segment ms (1-based).
 *   half 1 (cwire1, Zmatrix.cpp:237-339): segment ips[n], from its first node to the
 *          basis centre node |ipc[n]|;
 *   half 2 (cwire2, Zmatrix.cpp:450-555): segment ips[n+nsmax], from the centre node
 *          to the segment's second node.
 * image != 0 mirrors the source through sgnx/sgny/sgnz (cwire1_im / cwire2_im,
 * Zmatrix.cpp:342-446, 559-663); its singular branch also needs the observation
 * segment to lie on z = 0.
 * Writes the unit vector and length of the (possibly mirrored) source segment.
 */
static cplx half_integral(const geom_t *g, int ms, int n, int half, int ifun, const double rm[3],
                          double ka, int image, double dc[3], double *dl_out) {
  const double pi = acos(-1.0);
  const int nsmax = g->nsmax;
  int np = abs(g->ipc[n]);
  int ns = (half == 1) ? g->ips[n] : g->ips[n + nsmax];
  int nl = g->ise[ns - 1], nr = g->ise[ns + nsmax - 1];
  int ml = g->ise[ms - 1], mr = g->ise[ms + nsmax - 1];
  double sx = image ? (double)g->sgnx : 1.0;
  double sy = image ? (double)g->sgny : 1.0;
  double sz = image ? (double)g->sgnz : 1.0;
  int a_node = (half == 1) ? nl : np; /* start of the parametrisation */
  int b_node = (half == 1) ? np : nr; /* end */
  double rs[3], re_[3];
  if (image) {
    rs[0] = sx * (double)g->x[a_node - 1];
    rs[1] = sy * (double)g->y[a_node - 1];
    rs[2] = sz * (double)g->z[a_node - 1];
    re_[0] = sx * (double)g->x[b_node - 1];
    re_[1] = sy * (double)g->y[b_node - 1];
    re_[2] = sz * (double)g->z[b_node - 1];
  } else {
    rs[0] = (double)g->x[a_node - 1];
    rs[1] = (double)g->y[a_node - 1];
    rs[2] = (double)g->z[a_node - 1];
    re_[0] = (double)g->x[b_node - 1];
    re_[1] = (double)g->y[b_node - 1];
    re_[2] = (double)g->z[b_node - 1];
  }
  double an = (double)g->rad[ns - 1];
  double rd0 = re_[0] - rs[0], rd1 = re_[1] - rs[1], rd2 = re_[2] - rs[2];
  double dl = sqrt(rd0 * rd0 + rd1 * rd1 + rd2 * rd2);
  dc[0] = rd0 / dl;
  dc[1] = rd1 / dl;
  dc[2] = rd2 / dl;
  *dl_out = dl;
  int same = ((nl == ml) && (nr == mr)) || ((nl == mr) && (nr == ml));
  if (image) same = same && (g->z[ml - 1] < 1.e-6 && g->z[mr - 1] < 1.e-6);
  if (same) {
    double dlh = 0.5 * dl;
    cplx v = c_add(gauss4_self(0.0, dlh, ifun, ka, dl, an), gauss4_self(dlh, dl, ifun, ka, dl, an));
    double lg = 1.0 + log(16.0 * an / dl);
    double res = (ifun == 3) ? dl * lg / (pi * an) : 0.5 * dl * lg / (pi * an);
    return c_make(v.re + res, v.im);
  }
  double a = 0.5 * dl, b = dl, c = GL2_C * b;
  cplx v = c_add(kern_regular(a + c, ifun, ka, rm, rs, dc, an, dl),
                 kern_regular(a - c, ifun, ka, rm, rs, dc, an, dl));
  return c_scale(v, 0.5 * b);
}

/* One observation half of wim() (Zmatrix.cpp:66-233): the contribution of the
 * observation point on segment ms to Z[m, n]. */
static cplx obs_half(const geom_t *g, int ms, int n, const double rm[3], const double lm[3],
                     double ka, int ienv, int obs_sign) {
  double dc[3], dl;
  double senv = (double)g->sgnenv;
  /* vector potential */
  cplx a1 = half_integral(g, ms, n, 1, 1, rm, ka, 0, dc, &dl);
  cplx av = c_scale(a1, dc[0] * lm[0] + dc[1] * lm[1] + dc[2] * lm[2]);
  if (ienv == 2) {
    cplx ai = half_integral(g, ms, n, 1, 1, rm, ka, 1, dc, &dl);
    av = c_add(av, c_scale(ai, (dc[0] * lm[0] + dc[1] * lm[1] + dc[2] * lm[2]) * senv));
  }
  cplx a2 = half_integral(g, ms, n, 2, 2, rm, ka, 0, dc, &dl);
  av = c_add(av, c_scale(a2, dc[0] * lm[0] + dc[1] * lm[1] + dc[2] * lm[2]));
  if (ienv == 2) {
    cplx ai = half_integral(g, ms, n, 2, 2, rm, ka, 1, dc, &dl);
    av = c_add(av, c_scale(ai, (dc[0] * lm[0] + dc[1] * lm[1] + dc[2] * lm[2]) * senv));
  }
  /* scalar potential */
  cplx p1 = half_integral(g, ms, n, 1, 3, rm, ka, 0, dc, &dl);
  cplx sv = c_make(p1.re / dl, p1.im / dl);
  if (ienv == 2) {
    cplx pi_ = half_integral(g, ms, n, 1, 3, rm, ka, 1, dc, &dl);
    sv = c_add(sv, c_scale(pi_, senv / dl));
  }
  cplx p2 = half_integral(g, ms, n, 2, 3, rm, ka, 0, dc, &dl);
  sv = c_sub(sv, c_make(p2.re / dl, p2.im / dl));
  if (ienv == 2) {
    cplx pi_ = half_integral(g, ms, n, 2, 3, rm, ka, 1, dc, &dl);
    sv = c_sub(sv, c_scale(pi_, senv / dl));
  }
  cplx out = c_scale(av, ka * ka);
  return obs_sign < 0 ? c_sub(out, sv) : c_add(out, sv);
}

/* Z[m, :] for one test function m (Zmatrix.cpp:66-232), scaled by j*eta0/(4*pi*k)
 * (Zmatrix.cpp:35-51).  row_out[n] for n in [0, npls). */
static void fill_row(const geom_t *g, int m, int npls, double ka, int ienv, cplx *row_out,
                     int row_stride) {
  const int nsmax = g->nsmax;
  const double pi = acos(-1.0);
  const double eta0 = 120.0 * pi;
  const double cq = eta0 / (4.0 * pi * ka);
  int mp = abs(g->ipc[m]);
  double rp[3] = {(double)g->x[mp - 1], (double)g->y[mp - 1], (double)g->z[mp - 1]};
  /* observation point on S_m+ */
  int ms1 = g->ips[m];
  int ml = g->ise[ms1 - 1];
  double rl[3] = {(double)g->x[ml - 1], (double)g->y[ml - 1], (double)g->z[ml - 1]};
  double rm1[3], lm1[3];
  for (int k = 0; k < 3; ++k) {
    rm1[k] = 0.5 * (rp[k] + rl[k]);
    lm1[k] = rp[k] - rm1[k];
  }
  /* observation point on S_m- */
  int ms2 = g->ips[m + nsmax];
  int mr = g->ise[ms2 + nsmax - 1];
  double rr[3] = {(double)g->x[mr - 1], (double)g->y[mr - 1], (double)g->z[mr - 1]};
  double rm2[3], lm2[3];
  for (int k = 0; k < 3; ++k) {
    rm2[k] = 0.5 * (rr[k] + rp[k]);
    lm2[k] = rm2[k] - rp[k];
  }
  for (int n = 0; n < npls; ++n) {
    cplx acc = c_make(0.0, 0.0);
    acc = c_add(acc, obs_half(g, ms1, n, rm1, lm1, ka, ienv, -1));
    acc = c_add(acc, obs_half(g, ms2, n, rm2, lm2, ka, ienv, +1));
    /* multiply by j*cq */
    row_out[(size_t)n * row_stride] = c_make(-cq * acc.im, cq * acc.re);
  }
}

/*
 * Fill the npls x npls impedance matrix, column-major (cz[m + n*npls]), as
 * interleaved (re, im) doubles.  nthreads > 1 splits rows across OpenMP threads;
 * every entry is computed by the same sequence of operations either way, so the
 * result does not depend on the thread count.
 */
void oracle_zmatrix(double *cz, const float *x, const float *y, const float *z, const int *ipc,
                    const int *ips, const int *ise, const float *rad, int npls, double ka,
                    int nsmax, int ienv, float sgnx, float sgny, float sgnz, float sgnenv,
                    int nthreads) {
  geom_t g;
  g.x = x;
  g.y = y;
  g.z = z;
  g.rad = rad;
  g.ipc = ipc;
  g.ips = ips;
  g.ise = ise;
  g.nsmax = nsmax;
  g.sgnx = sgnx;
  g.sgny = sgny;
  g.sgnz = sgnz;
  g.sgnenv = sgnenv;
  cplx *out = (cplx *)cz;
#ifdef _OPENMP
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
#endif
  for (int m = 0; m < npls; ++m) fill_row(&g, m, npls, ka, ienv, out + m, npls);
  (void)nthreads;
}

/* Wave number from a float frequency in MHz, as Wire_MoM.cu:338-340 computes it
 * (speed of light 2.99792448e8 m/s). */
double oracle_ka(float freq_mhz) {
  const double c = 2.99792448E+8;
  const double pi = acos(-1.0);
  double lambda = c / freq_mhz * 1E-6;
  return (pi + pi) / lambda;
}

/*
 * Unblocked LU with partial pivoting, LAPACK zgetf2 semantics: the pivot of
 * column j is the first row of maximal |re|+|im| (izamax), rows are swapped
 * across the full width, the column below the pivot is scaled by the
 * reciprocal of the pivot, and a rank-1 update follows.  ipiv is 1-based.
 * Returns 0, or j+1 for the first exactly-zero pivot (the factorisation then
 * continues, as LAPACK does).
 */
int oracle_zgetf2(int n, double *a_, int lda, int *ipiv) {
  cplx *a = (cplx *)a_;
  int info = 0;
  for (int j = 0; j < n; ++j) {
    int p = j;
    double best = -1.0;
    for (int i = j; i < n; ++i) {
      cplx v = a[i + (size_t)j * lda];
      double t = fabs(v.re) + fabs(v.im);
      if (t > best) {
        best = t;
        p = i;
      }
    }
    ipiv[j] = p + 1;
    cplx piv = a[p + (size_t)j * lda];
    if (piv.re != 0.0 || piv.im != 0.0) {
      if (p != j) {
        for (int k = 0; k < n; ++k) {
          cplx t = a[j + (size_t)k * lda];
          a[j + (size_t)k * lda] = a[p + (size_t)k * lda];
          a[p + (size_t)k * lda] = t;
        }
      }
      cplx inv = c_div(c_make(1.0, 0.0), a[j + (size_t)j * lda]);
      for (int i = j + 1; i < n; ++i) a[i + (size_t)j * lda] = c_mul(a[i + (size_t)j * lda], inv);
    } else if (info == 0) {
      info = j + 1;
    }
    for (int k = j + 1; k < n; ++k) {
      cplx u = a[j + (size_t)k * lda];
      if (u.re == 0.0 && u.im == 0.0) continue;
      for (int i = j + 1; i < n; ++i)
        a[i + (size_t)k * lda] = c_sub(a[i + (size_t)k * lda], c_mul(a[i + (size_t)j * lda], u));
    }
  }
  return info;
}

/* zgetrs('N') for one right-hand side: apply the row interchanges, then the unit
 * lower and the upper triangular solves. */
void oracle_zgetrs(int n, const double *a_, int lda, const int *ipiv, double *b_) {
  const cplx *a = (const cplx *)a_;
  cplx *b = (cplx *)b_;
  for (int j = 0; j < n; ++j) {
    int p = ipiv[j] - 1;
    if (p != j) {
      cplx t = b[j];
      b[j] = b[p];
      b[p] = t;
    }
  }
  for (int j = 0; j < n; ++j) {
    cplx bj = b[j];
    if (bj.re == 0.0 && bj.im == 0.0) continue;
    for (int i = j + 1; i < n; ++i) b[i] = c_sub(b[i], c_mul(bj, a[i + (size_t)j * lda]));
  }
  for (int j = n - 1; j >= 0; --j) {
    if (b[j].re == 0.0 && b[j].im == 0.0) continue;
    b[j] = c_div(b[j], a[j + (size_t)j * lda]);
    cplx bj = b[j];
    for (int i = 0; i < j; ++i) b[i] = c_sub(b[i], c_mul(bj, a[i + (size_t)j * lda]));
  }
}
