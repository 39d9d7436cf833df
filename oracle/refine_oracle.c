/*
 * refine_oracle.c -- residuals in about twice double precision, for an
 * extended-precision "truth" of a dense complex solve.  TEST INFRASTRUCTURE ONLY:
 * tests/ and bench.py's accuracy legs use it (through oracle/oracle.py) as the
 * checker; nothing in the product links or loads it.
 *
 * oracle_residual_dd computes r = b - A (xh + xl), A column-major complex128, with
 * every product of A's entries and xh formed exactly (the fma-based two-product) and
 * every sum compensated (Knuth's two-sum), as in Ogita, Rump and Oishi, "Accurate
 * sum and dot product", SIAM J. Sci. Comput. 26 (2005), algorithm Dot2: the result
 * is as accurate as if computed in twice double precision and rounded.  The
 * products with the low part xl are added to the compensation in plain double
 * (their rounding error is below 2^-106 of |A||x|).
 *
 * oracle.refine_truth() iterates x <- x + A^-1 r with an FP64 LU and keeps x as a
 * double-double.  Classical iterative refinement with extra-precise residuals
 * (Wilkinson; Moler, "Iterative refinement in floating point", JACM 14, 1967): for
 * kappa(A) * 2^-53 well below 1 the iteration contracts by about kappa * 2^-53 per
 * step to the solution of the given FP64 matrix, correct to about 2^-106 relative
 * -- which splits the error of any FP64 solver into its own part and the part the
 * conditioning of the matrix imposes on every FP64 solver.
 *
 * Compile with -ffp-contract=off: the two-sums must not be contracted.
 */
#include <math.h>
#include <stddef.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline void two_sum(double a, double b, double* s, double* e) {
  const double t = a + b;
  const double bb = t - a;
  *e = (a - (t - bb)) + (b - bb);
  *s = t;
}

static inline void two_prod(double a, double b, double* p, double* e) {
  const double t = a * b;
  *e = fma(a, b, -t);
  *p = t;
}

/* r_hi + r_lo = b - A (xh + xl) for complex n-vectors stored as interleaved
 * (re, im) doubles; rows are split among `threads` OpenMP threads in blocks of 256,
 * each block sweeping the columns in order (so the result does not depend on the
 * thread count).  r_lo may be NULL. */
void oracle_residual_dd(int n, const double* a, const double* b, const double* xh, const double* xl, double* r_hi,
                        double* r_lo, int threads) {
  enum { RB = 256 };
  const int nblk = (n + RB - 1) / RB;
  if (threads < 1) threads = 1;
#pragma omp parallel for num_threads(threads) schedule(static)
  for (int blk = 0; blk < nblk; ++blk) {
    const int i0 = blk * RB;
    const int i1 = i0 + RB < n ? i0 + RB : n;
    double sre[RB], cre[RB], sim[RB], cim[RB];
    for (int i = i0; i < i1; ++i) {
      sre[i - i0] = b[2 * (size_t)i];
      sim[i - i0] = b[2 * (size_t)i + 1];
      cre[i - i0] = 0.0;
      cim[i - i0] = 0.0;
    }
    for (int j = 0; j < n; ++j) {
      const double xr = xh[2 * (size_t)j], xi = xh[2 * (size_t)j + 1];
      const double lr = xl ? xl[2 * (size_t)j] : 0.0, li = xl ? xl[2 * (size_t)j + 1] : 0.0;
      const double* col = a + 2 * (size_t)j * n;
      for (int i = i0; i < i1; ++i) {
        const double ar = col[2 * (size_t)i], ai = col[2 * (size_t)i + 1];
        const int k = i - i0;
        double p, e, q;
        /* real part: - ar xr + ai xi - ar lr + ai li */
        two_prod(ar, xr, &p, &e);
        two_sum(sre[k], -p, &sre[k], &q);
        cre[k] += q - e;
        two_prod(ai, xi, &p, &e);
        two_sum(sre[k], p, &sre[k], &q);
        cre[k] += q + e;
        cre[k] += ai * li - ar * lr;
        /* imaginary part: - ar xi - ai xr - ar li - ai lr */
        two_prod(ar, xi, &p, &e);
        two_sum(sim[k], -p, &sim[k], &q);
        cim[k] += q - e;
        two_prod(ai, xr, &p, &e);
        two_sum(sim[k], -p, &sim[k], &q);
        cim[k] += q - e;
        cim[k] -= ar * li + ai * lr;
      }
    }
    for (int i = i0; i < i1; ++i) {
      const int k = i - i0;
      double h, l;
      two_sum(sre[k], cre[k], &h, &l);
      r_hi[2 * (size_t)i] = h;
      if (r_lo) r_lo[2 * (size_t)i] = l;
      two_sum(sim[k], cim[k], &h, &l);
      r_hi[2 * (size_t)i + 1] = h;
      if (r_lo) r_lo[2 * (size_t)i + 1] = l;
    }
  }
}
