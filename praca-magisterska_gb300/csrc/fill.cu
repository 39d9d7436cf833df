// fill.cu -- FP64 impedance-matrix fill on the GPU.
//
// Computes Z[m, n] of the reference's thin-wire formulation
// ("wersja referencyjna/Zmatrix.cpp":27-770, the same math as the reference's GPU
// kernels wim_gpu_cknn_* / wim_gpu_ckmn_* in "wersja referencyjna/Wire_MoM.cu":454-4049)
// in ONE kernel launch per batch of frequencies, writing every entry exactly once
// (the reference makes six read-modify-write passes over Z per frequency).
//
// Per entry: two observation points (midpoints of S_m+ and S_m-), two source
// half-segments (S_n+ rising ramp, S_n- falling ramp).  Regular pairs use the
// reference's 2-point Gauss rule of exp(-jkR)/R with R = sqrt(a^2 + |r_m - r'|^2);
// identical segments use its two 4-point rules of the regularised kernel plus the
// analytic log term; both the ramped (vector potential) and the plain (scalar
// potential) integrals come from the same kernel evaluations.  The geometric
// arithmetic is done with explicitly rounded operations in the reference's order,
// so that the float-derived coordinates give the same doubles as the CPU code.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/wmom.h"
#include "stats.h"
#include "wmom_internal.h"

namespace wmom {
namespace {

constexpr double kGl2C = 0.288675134594812882;  // 1/(2*sqrt(3))
constexpr double kGl4C1 = 0.43056815579702629;
constexpr double kGl4W1 = 0.17392742256872693;
constexpr double kGl4C2 = 0.16999052179242813;
constexpr double kGl4W2 = 0.32607257743127307;

struct Cx {
  double re, im;
};

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// ------------------------------------------------------------------------
// sin and cos of the phase k*R of the regular Green's function evaluations.
// Table-driven method (Tang, "Table-driven implementation of the exponential
// function", ACM TOMS 15(2), 1989, applied to sin/cos by angle addition):
//   x = n*h + d,  h = pi/512,  |d| <= h/2 ~ 0.00307,
//   sin x = S_j cos d + C_j sin d,  cos x = C_j cos d - S_j sin d,  j = n mod 1024,
// with (S_j, C_j) = (sin, cos)(j*pi/512) tabulated once per device by sincospi(j/512)
// (an exact argument) and read through the read-only cache, d from a two-constant
// Cody-Waite reduction
// (h_hi = double(pi)/512 exactly, h_lo = (pi - double(pi))/512), and sin d, cos d
// from their Taylor series to d^5 and d^4 (truncation below 2e-17 relative).
// Arguments beyond 1e6 rad take sincos() itself.
// ------------------------------------------------------------------------
constexpr int kSinTab = 1024;
constexpr double kInvH = 162.97466172610082383;      // 512/pi
constexpr double kHHi = 3.141592653589793116 / 512;  // double(pi)/512, exact
constexpr double kHLo = 1.2246467991473532e-16 / 512;  // (pi - double(pi))/512

__device__ double2 g_sin_tab[kSinTab];

__global__ void sin_table_setup_kernel() {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < kSinTab) {
    double sj, cj;
    sincospi(j / 512.0, &sj, &cj);
    g_sin_tab[j] = make_double2(sj, cj);
  }
}

__device__ __forceinline__ void sincos_tab(double x, const double2* tab, double* s, double* c) {
  // |x| < 1e6 (and not NaN), tested on the high word: 1e6 = 0x412E8480'00000000
  if ((__double2hiint(x) & 0x7fffffff) >= 0x412E8480) {
    sincos(x, s, c);
    return;
  }
  // n = x/h rounded to nearest by adding 1.5 * 2^52 (exact for |x/h| < 2^51); the
  // low word of the sum is then n modulo 2^32, whose low bits index the table
  constexpr double kRound = 6755399441055744.0;  // 1.5 * 2^52
  const double tn = fma(x, kInvH, kRound);
  const double n = tn - kRound;
  double d = fma(-n, kHHi, x);
  d = fma(-n, kHLo, d);
  const double2 t = __ldg(&tab[__double2loint(tn) & (kSinTab - 1)]);
  const double d2 = d * d;
  const double sd = fma(d * d2, fma(d2, 1.0 / 120.0, -1.0 / 6.0), d);
  const double cd = fma(d2, fma(d2, 1.0 / 24.0, -0.5), 1.0);
  *s = fma(t.x, cd, t.y * sd);
  *c = fma(t.y, cd, -(t.x * sd));
}


// Complete elliptic integral K, Hastings polynomial-log approximation with the
// reference's coefficients (Zmatrix.cpp:738-747; Abramowitz & Stegun 17.3.34).
__device__ double ell_k(double bet) {
  const double a0 = 1.38629436112, a1 = 0.09666344259, a2 = 0.03590092383,
               a3 = 0.03742563713, a4 = 0.01451196212;
  const double b0 = 0.5, b1 = 0.12498593597, b2 = 0.06880248576, b3 = 0.03328355346,
               b4 = 0.00441787012;
  double m1 = sub(1.0, mul(bet, bet));
  double a = add(a0, mul(a1, m1)), b = add(b0, mul(b1, m1));
  double m2 = 0.0, m3 = 0.0;
  if (m1 >= 1.0e-18) {
    m2 = mul(m1, m1);
    a = add(a, mul(a2, m2));
    b = add(b, mul(b2, m2));
  }
  if (m1 >= 1.0e-12) {
    m3 = mul(m2, m1);
    a = add(a, mul(a3, m3));
    b = add(b, mul(b3, m3));
  }
  if (m1 >= 1.0e-9) {
    double m4 = mul(m3, m1);
    a = add(a, mul(a4, m4));
    b = add(b, mul(b4, m4));
  }
  return sub(a, mul(b, log(m1)));
}

// One regular (observation point, source half) pair, the 2-point rule of the
// reference's cwire1_re/cwire2_re + ckmn (Zmatrix.cpp:237-339, 450-555, 667-692),
// in two parts.  The frequency-independent part gives R and 1/R at the two abscissae
// s[0], s[1] (R^2 = a_n^2 + |ex - s dc|^2, ex = r_m - r_s, one reciprocal square
// root).  The frequency part gives, with g = exp(-j ka R)/R,
//   up = sum s/dl g,  dn = sum (dl - s)/dl g,  pl = sum g,
// from the ramp weights the host precomputed.  Distances and weighted sums are
// FMA-contracted; every fill kernel calls these routines, so all of them produce
// identical matrices.
__device__ __forceinline__ void gauss_geometry(const double ex[3], const double dc[3], double an2, const double s[2],
                                               double r[2], double ri[2]) {
#pragma unroll
  for (int g = 0; g < 2; ++g) {
    const double dx = fma(-s[g], dc[0], ex[0]);
    const double dy = fma(-s[g], dc[1], ex[1]);
    const double dz = fma(-s[g], dc[2], ex[2]);
    const double r2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, an2)));
    ri[g] = rsqrt(r2);
    r[g] = mul(r2, ri[g]);
  }
}

__device__ __forceinline__ void gauss_sums(const double r[2], const double ri[2], const double wu[2],
                                           const double wd[2], double ka, const double2* tab, Cx* up, Cx* dn,
                                           Cx* pl) {
  // the falling ramp is one minus the rising one, so its sum is the plain sum minus
  // the rising sum
  // (wd is kept in the signature for the instances' layout).  The first point starts
  // the sums: the same values as accumulating onto zero, two FP64 additions fewer.
  (void)wd;
  Cx su, sp;
#pragma unroll
  for (int g = 0; g < 2; ++g) {
    double sn, cs;
    sincos_tab(mul(ka, r[g]), tab, &sn, &cs);
    const double gre = mul(cs, ri[g]), gim = -mul(sn, ri[g]);
    if (g == 0) {
      su = Cx{mul(wu[0], gre), mul(wu[0], gim)};
      sp = Cx{gre, gim};
    } else {
      su.re = fma(wu[g], gre, su.re);
      su.im = fma(wu[g], gim, su.im);
      sp.re = add(sp.re, gre);
      sp.im = add(sp.im, gim);
    }
  }
  *up = su;
  *dn = Cx{sub(sp.re, su.re), sub(sp.im, su.im)};
  *pl = sp;
}

__device__ __forceinline__ void regular_sums(const double ex[3], const double dc[3], double an2, const double s[2],
                                             const double wu[2], const double wd[2], double ka, const double2* tab,
                                             Cx* up, Cx* dn, Cx* pl) {
  double r[2], ri[2];
  gauss_geometry(ex, dc, an2, s, r, ri);
  gauss_sums(r, ri, wu, wd, ka, tab, up, dn, pl);
}

// Abscissae and ramp weights of the 2-point rule on a source half of length dl, in
// the host's order of operations (plan.cpp builds the same values for the tiles).
__device__ __forceinline__ void gauss2(double dl, double s[2], double wu[2], double wd[2]) {
  const double a = mul(0.5, dl);
  const double c = mul(kGl2C, dl);
  s[0] = add(a, c);
  s[1] = sub(a, c);
#pragma unroll
  for (int g = 0; g < 2; ++g) {
    wu[g] = __ddiv_rn(s[g], dl);
    wd[g] = __ddiv_rn(sub(dl, s[g]), dl);
  }
}

// One regular source half of the per-entry kernel: the ramped integral times the
// projection t (rising ramp for S_n+, falling for S_n-) and the plain integral over
// dl, i.e. (dl/2) sum g / dl = sum g / 2; the first scaled by kc = k^2 cq, the
// second by cq (hc = cq / 2), as the pair values are.
__device__ void regular_half(const double rm[3], const double rs[3], const double dc[3], double dl, double an,
                             double ka, bool falling, double t, double kc, double hc, const double2* tab, Cx* At,
                             Cx* Pd) {
  double s[2], wu[2], wd[2];
  gauss2(dl, s, wu, wd);
  const double ex[3] = {sub(rm[0], rs[0]), sub(rm[1], rs[1]), sub(rm[2], rs[2])};
  Cx su, sd, sp;
  regular_sums(ex, dc, mul(an, an), s, wu, wd, ka, tab, &su, &sd, &sp);
  const double htk = mul(mul(mul(dl, 0.5), t), kc);
  // the falling ramp's scaled sum as regular_pair_value forms it: plain minus rising
  const Cx wr = {mul(su.re, htk), mul(su.im, htk)};
  *At = falling ? Cx{fma(sp.re, htk, -wr.re), fma(sp.im, htk, -wr.im)} : wr;
  *Pd = Cx{mul(hc, sp.re), mul(hc, sp.im)};
  (void)sd;
}

// Regularised self kernel bracket (Zmatrix.cpp:695-709) at parameter s.
__device__ Cx self_bracket(double s, double ka, double dl, double an) {
  const double pi = 3.141592653589793;  // acos(-1.0)
  const double r = sub(mul(0.5, dl), s);
  const double rr = sqrt(add(mul(an, an), mul(r, r)));
  double sn, cs;
  sincos(mul(ka, rr), &sn, &cs);
  const double ere = __ddiv_rn(sub(cs, 1.0), rr), eim = __ddiv_rn(-sn, rr);
  const double bet = __ddiv_rn(add(an, an), sqrt(add(mul(mul(4.0, an), an), mul(r, r))));
  const double stat =
      __ddiv_rn(add(mul(bet, ell_k(bet)), log(fabs(__ddiv_rn(r, mul(8.0, an))))), mul(pi, an));
  return Cx{add(ere, stat), eim};
}

// Self source half: two 4-point Gauss rules on [0, dl/2] and [dl/2, dl] plus the
// analytic term (Zmatrix.cpp:277-323).
__device__ void self_half(double dl, double an, double ka, bool falling, Cx* A, Cx* P) {
  const double pi = 3.141592653589793;
  const double dlh = mul(0.5, dl);
  Cx ta = {0.0, 0.0}, tp = {0.0, 0.0};
#pragma unroll 1
  for (int part = 0; part < 2; ++part) {
    const double lo = part == 0 ? 0.0 : dlh, hi = part == 0 ? dlh : dl;
    const double a = mul(0.5, add(lo, hi)), b = sub(hi, lo);
    Cx qa[2], qp[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const double c = mul(q == 0 ? kGl4C1 : kGl4C2, b);
      const double s1 = add(a, c), s2 = sub(a, c);
      const Cx v1 = self_bracket(s1, ka, dl, an), v2 = self_bracket(s2, ka, dl, an);
      const double w1 = falling ? __ddiv_rn(sub(dl, s1), dl) : __ddiv_rn(s1, dl);
      const double w2 = falling ? __ddiv_rn(sub(dl, s2), dl) : __ddiv_rn(s2, dl);
      const double wq = q == 0 ? kGl4W1 : kGl4W2;
      qa[q].re = mul(add(mul(w1, v1.re), mul(w2, v2.re)), wq);
      qa[q].im = mul(add(mul(w1, v1.im), mul(w2, v2.im)), wq);
      qp[q].re = mul(add(v1.re, v2.re), wq);
      qp[q].im = mul(add(v1.im, v2.im), wq);
    }
    const double pa_re = mul(add(qa[0].re, qa[1].re), b), pa_im = mul(add(qa[0].im, qa[1].im), b);
    const double pp_re = mul(add(qp[0].re, qp[1].re), b), pp_im = mul(add(qp[0].im, qp[1].im), b);
    ta.re = part == 0 ? pa_re : add(ta.re, pa_re);
    ta.im = part == 0 ? pa_im : add(ta.im, pa_im);
    tp.re = part == 0 ? pp_re : add(tp.re, pp_re);
    tp.im = part == 0 ? pp_im : add(tp.im, pp_im);
  }
  const double lg = add(1.0, log(__ddiv_rn(mul(16.0, an), dl)));
  const double res3 = __ddiv_rn(mul(dl, lg), mul(pi, an));
  const double res12 = __ddiv_rn(mul(mul(0.5, dl), lg), mul(pi, an));
  A->re = add(ta.re, res12);
  A->im = ta.im;
  P->re = add(tp.re, res3);
  P->im = tp.im;
}

__device__ __forceinline__ double dot3(const double a[3], const double b[3]) {
  return add(add(mul(a[0], b[0]), mul(a[1], b[1])), mul(a[2], b[2]));
}


// One thread per entry: blockIdx.x*blockDim.x + threadIdx.x = row m (observation),
// blockIdx.y = column n (source), blockIdx.z = frequency.  Consecutive threads write
// consecutive rows of one column: coalesced 16-byte complex stores.
__global__ void __launch_bounds__(128) fill_entry_kernel(const ObsHalf* __restrict__ obs,
                                                         const SrcHalf* __restrict__ src, int npls,
                                                         const FreqParams* __restrict__ fp,
                                                         double2* __restrict__ Z, long long ldz,
                                                         long long zstride, int ienv,
                                                         float sgnenv) {
  const double2* tab = g_sin_tab;
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = blockIdx.y;
  const int k = blockIdx.z;
  if (m >= npls) return;
  const double ka = fp[k].ka, cq = fp[k].cq, kc = fp[k].kc, hc = fp[k].hc;
  const double senv = (double)sgnenv;
  double acc_re = 0.0, acc_im = 0.0;
#pragma unroll 1
  for (int h = 0; h < 2; ++h) {
    const ObsHalf o = obs[2 * m + h];
    double av_re = 0.0, av_im = 0.0, sv_re = 0.0, sv_im = 0.0;
#pragma unroll 1
    for (int sgm = 0; sgm < 2; ++sgm) {
      const SrcHalf sh = src[2 * n + sgm];
      const bool falling = sgm == 1;
      const bool same = (sh.nl == o.ml && sh.nr == o.mr) || (sh.nl == o.mr && sh.nr == o.ml);
      // At = ramped integral times the projection t, Pd = plain integral / dl
      const double t = dot3(sh.dc, o.lm);
      Cx At, Pd;
      if (same) {
        Cx A, P;
        self_half(sh.dl, sh.an, ka, falling, &A, &P);
        const double tk = mul(t, kc);
        At = Cx{mul(A.re, tk), mul(A.im, tk)};
        Pd = Cx{mul(__ddiv_rn(P.re, sh.dl), cq), mul(__ddiv_rn(P.im, sh.dl), cq)};
      } else {
        regular_half(o.rm, sh.rs, sh.dc, sh.dl, sh.an, ka, falling, t, kc, hc, tab, &At, &Pd);
      }
      // the first term starts the sums (no addition to zero), as in the tile assembly
      av_re = sgm == 0 ? At.re : add(av_re, At.re);
      av_im = sgm == 0 ? At.im : add(av_im, At.im);
      Cx Pid = {0.0, 0.0};
      if (ienv == 2) {
        const double ti = mul(dot3(sh.dc_img, o.lm), senv);
        Cx Ait;
        if (same && o.on_ground) {
          Cx Ai, Pi;
          self_half(sh.dl, sh.an, ka, falling, &Ai, &Pi);
          const double tk = mul(ti, kc);
          Ait = Cx{mul(Ai.re, tk), mul(Ai.im, tk)};
          Pid = Cx{mul(__ddiv_rn(Pi.re, sh.dl), cq), mul(__ddiv_rn(Pi.im, sh.dl), cq)};
        } else {
          regular_half(o.rm, sh.rs_img, sh.dc_img, sh.dl, sh.an, ka, falling, ti, kc, hc, tab, &Ait, &Pid);
        }
        av_re = add(av_re, Ait.re);
        av_im = add(av_im, Ait.im);
      }
      // scalar potential: + P(S_n+)/dl - P(S_n-)/dl
      if (sgm == 0 && ienv != 2) {
        sv_re = Pd.re;
        sv_im = Pd.im;
      } else if (!falling) {
        sv_re = add(sv_re, Pd.re);
        sv_im = add(sv_im, Pd.im);
      } else {
        sv_re = sub(sv_re, Pd.re);
        sv_im = sub(sv_im, Pd.im);
      }
      if (ienv == 2) {
        // image: sgnenv * P_img / dl
        const double qre = mul(Pid.re, senv), qim = mul(Pid.im, senv);
        if (!falling) {
          sv_re = add(sv_re, qre);
          sv_im = add(sv_im, qim);
        } else {
          sv_re = sub(sv_re, qre);
          sv_im = sub(sv_im, qim);
        }
      }
    }
    // k^2 (A+ + A-) -/+ (Phi+ - Phi-), both already scaled by cq
    const double c_re = h == 0 ? sub(av_re, sv_re) : add(av_re, sv_re);
    const double c_im = h == 0 ? sub(av_im, sv_im) : add(av_im, sv_im);
    acc_re = h == 0 ? c_re : add(acc_re, c_re);
    acc_im = h == 0 ? c_im : add(acc_im, c_im);
  }
  // times j (cq is in the terms)
  Z[(size_t)k * zstride + (size_t)n * ldz + m] = make_double2(-acc_im, acc_re);
}

// ------------------------------------------------------------------------
// Pair-tiled fill.  One CTA per 32 x 32 tile of Z (and per frequency): phase A
// evaluates every distinct (observation instance, source instance) pair of the tile
// once -- the rising-ramp, falling-ramp and plain integrals, the first two already
// multiplied by the test-vector projection and the last divided by the segment
// length -- into shared memory; phase B assembles each entry from four pair values
// in the reference's order of operations.  Each pair is the same arithmetic as in
// fill_entry_kernel, so both kernels produce the same matrix.
// ------------------------------------------------------------------------
struct PairVal {
  double2 wu, wd, ph;
};

__device__ void self_pair(double dl, double an, double ka, Cx* Au, Cx* Ad, Cx* P) {
  const double pi = 3.141592653589793;
  const double dlh = mul(0.5, dl);
  Cx tu = {0.0, 0.0}, td = {0.0, 0.0}, tp = {0.0, 0.0};
#pragma unroll 1
  for (int part = 0; part < 2; ++part) {
    const double lo = part == 0 ? 0.0 : dlh, hi = part == 0 ? dlh : dl;
    const double a = mul(0.5, add(lo, hi)), b = sub(hi, lo);
    Cx qu[2], qd[2], qp[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const double c = mul(q == 0 ? kGl4C1 : kGl4C2, b);
      const double s1 = add(a, c), s2 = sub(a, c);
      const Cx v1 = self_bracket(s1, ka, dl, an), v2 = self_bracket(s2, ka, dl, an);
      const double u1 = __ddiv_rn(s1, dl), u2 = __ddiv_rn(s2, dl);
      const double d1 = __ddiv_rn(sub(dl, s1), dl), d2 = __ddiv_rn(sub(dl, s2), dl);
      const double wq = q == 0 ? kGl4W1 : kGl4W2;
      qu[q].re = mul(add(mul(u1, v1.re), mul(u2, v2.re)), wq);
      qu[q].im = mul(add(mul(u1, v1.im), mul(u2, v2.im)), wq);
      qd[q].re = mul(add(mul(d1, v1.re), mul(d2, v2.re)), wq);
      qd[q].im = mul(add(mul(d1, v1.im), mul(d2, v2.im)), wq);
      qp[q].re = mul(add(v1.re, v2.re), wq);
      qp[q].im = mul(add(v1.im, v2.im), wq);
    }
    const Cx pu = {mul(add(qu[0].re, qu[1].re), b), mul(add(qu[0].im, qu[1].im), b)};
    const Cx pd = {mul(add(qd[0].re, qd[1].re), b), mul(add(qd[0].im, qd[1].im), b)};
    const Cx pp = {mul(add(qp[0].re, qp[1].re), b), mul(add(qp[0].im, qp[1].im), b)};
    if (part == 0) {
      tu = pu;
      td = pd;
      tp = pp;
    } else {
      tu = Cx{add(tu.re, pu.re), add(tu.im, pu.im)};
      td = Cx{add(td.re, pd.re), add(td.im, pd.im)};
      tp = Cx{add(tp.re, pp.re), add(tp.im, pp.im)};
    }
  }
  const double lg = add(1.0, log(__ddiv_rn(mul(16.0, an), dl)));
  const double res3 = __ddiv_rn(mul(dl, lg), mul(pi, an));
  const double res12 = __ddiv_rn(mul(mul(0.5, dl), lg), mul(pi, an));
  *Au = Cx{add(tu.re, res12), tu.im};
  *Ad = Cx{add(td.re, res12), td.im};
  *P = Cx{add(tp.re, res3), tp.im};
}

// The tile's index lists (offsets into one int array).
struct TileLists {
  const int* rt_off;
  const int* rt_ids;
  const int* ct_off;
  const int* ct_ids;
  const int* row_local;
  const int* col_local;
};

__device__ __forceinline__ TileLists tile_lists(const int* tiles, int off_rt_ids, int off_ct_off, int off_ct_ids,
                                                int off_row_local, int off_col_local) {
  return TileLists{tiles, tiles + off_rt_ids, tiles + off_ct_off, tiles + off_ct_ids, tiles + off_row_local,
                   tiles + off_col_local};
}

__device__ __forceinline__ bool same_segment(const ObsInst& O, const SrcInst& S) {
  return (S.nl == O.ml && S.nr == O.mr) || (S.nl == O.mr && S.nr == O.ml);
}

// Phase A value of a regular pair from its R, 1/R and ht = (dl/2) t, t the test
// projection (ht does not depend on the frequency).  The ramped integrals carry
// k^2 cq (kc), the plain one cq (hc = cq / 2 with the 1/2 of the 2-point rule), so
// that phase B only adds.
__device__ __forceinline__ PairVal regular_pair_value(const double r[2], const double ri[2], double ht,
                                                      const SrcInst& S, const FreqParams& f, const double2* tab) {
  Cx su, sd, sp;
  gauss_sums(r, ri, S.w_up, S.w_dn, f.ka, tab, &su, &sd, &sp);
  const double htk = mul(ht, f.kc);
  PairVal v;
  v.wu = make_double2(mul(su.re, htk), mul(su.im, htk));
  // falling ramp = plain - rising: (sp - su) htk as sp htk - su htk with one rounding,
  // two FP64 instructions fewer than subtracting first
  v.wd = make_double2(fma(sp.re, htk, -v.wu.x), fma(sp.im, htk, -v.wu.y));
  (void)sd;
  v.ph = make_double2(mul(f.hc, sp.re), mul(f.hc, sp.im));
  return v;
}

// The self integrals of a source instance at one frequency (ramped up, ramped down,
// plain): they depend on the segment's length and radius and on k only.
struct SelfVal {
  double2 au, ad, p;
};

// Self integrals of every source instance for every frequency of a launch, ahead of
// the tile kernels: a self pair costs about thirty regular ones (two 4-point rules,
// sincos, log, divisions), and where they fall into many tiles (junction grids) the
// CTA holding one would otherwise wait on that thread.
__global__ void self_values_kernel(const SrcInst* __restrict__ sinst, int nsrc, const FreqParams* __restrict__ fp,
                                   SelfVal* __restrict__ out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (q >= nsrc) return;
  const SrcInst& S = sinst[q];
  Cx Au, Ad, P;
  self_pair(S.dl, S.an, fp[k].ka, &Au, &Ad, &P);
  out[(size_t)k * nsrc + q] = SelfVal{make_double2(Au.re, Au.im), make_double2(Ad.re, Ad.im), make_double2(P.re, P.im)};
}

// Phase A value of a self pair (identical segments) from its self integrals, scaled
// as above.
__device__ __forceinline__ PairVal self_pair_value(double t, const SrcInst& S, const FreqParams& f,
                                                   const SelfVal& sv) {
  const double tk = mul(t, f.kc);
  PairVal v;
  v.wu = make_double2(mul(sv.au.x, tk), mul(sv.au.y, tk));
  v.wd = make_double2(mul(sv.ad.x, tk), mul(sv.ad.y, tk));
  v.ph = make_double2(mul(__ddiv_rn(sv.p.x, S.dl), f.cq), mul(__ddiv_rn(sv.p.y, S.dl), f.cq));
  return v;
}

// Phase B: the entries of tile (tr, tc) from the pair values, consecutive threads
// on consecutive rows (coalesced 16-byte stores), in the reference's order.
__device__ __forceinline__ void assemble_tile(const PairVal* pt, int nQ, const TileLists& L, int tr, int tc, int npls,
                                              double2* __restrict__ Zk, long long ldz) {
  for (int e = threadIdx.x; e < kPairTile * kPairTile; e += blockDim.x) {
    const int r = e % kPairTile, c = e / kPairTile;
    const int m = tr * kPairTile + r, n = tc * kPairTile + c;
    if (m >= npls || n >= npls) continue;
    const int c0 = L.col_local[2 * n], c1 = L.col_local[2 * n + 1];
    double acc_re = 0.0, acc_im = 0.0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int rl = L.row_local[2 * m + h];
      const int o = rl & 0x3FFFFFFF;
      const PairVal& pu = pt[o * nQ + c0];
      const PairVal& pd = pt[o * nQ + c1];
      double av_re = add(pu.wu.x, pd.wd.x), av_im = add(pu.wu.y, pd.wd.y);
      if (rl >> 30) {
        av_re = -av_re;
        av_im = -av_im;
      }
      const double sv_re = sub(pu.ph.x, pd.ph.x), sv_im = sub(pu.ph.y, pd.ph.y);
      const double c_re = h == 0 ? sub(av_re, sv_re) : add(av_re, sv_re);
      const double c_im = h == 0 ? sub(av_im, sv_im) : add(av_im, sv_im);
      acc_re = h == 0 ? c_re : add(acc_re, c_re);
      acc_im = h == 0 ? c_im : add(acc_im, c_im);
    }
    // times j (cq is in the pair values)
    Zk[(size_t)n * ldz + m] = make_double2(-acc_im, acc_re);
  }
}

// Tile (tr, tc) of one matrix at one frequency: the tile's instances and then its
// pair values are staged in shared memory `sm` (layout from max_o, max_q), and the
// entries are written to Zk.  selfv holds this frequency's self values, indexed by
// source instance.
__device__ __forceinline__ void pair_tile(const ObsInst* __restrict__ oinst, const SrcInst* __restrict__ sinst,
                                          const TileLists& L, int tr, int tc, int npls, int max_o, int max_q,
                                          const FreqParams& f, const SelfVal* __restrict__ selfv,
                                          double2* __restrict__ Zk, long long ldz, unsigned char* sm) {
  const double2* tab = g_sin_tab;
  ObsInst* so = reinterpret_cast<ObsInst*>(sm);
  SrcInst* sq = reinterpret_cast<SrcInst*>(sm + (size_t)max_o * sizeof(ObsInst));
  const size_t pt_off = ((size_t)max_o * sizeof(ObsInst) + (size_t)max_q * sizeof(SrcInst) + 15) & ~(size_t)15;
  PairVal* pt = reinterpret_cast<PairVal*>(sm + pt_off);
  const int tid = threadIdx.x;
  const int o0 = L.rt_off[tr], nO = L.rt_off[tr + 1] - o0;
  const int q0 = L.ct_off[tc], nQ = L.ct_off[tc + 1] - q0;
  for (int i = tid; i < nO; i += blockDim.x) so[i] = oinst[L.rt_ids[o0 + i]];
  for (int i = tid; i < nQ; i += blockDim.x) sq[i] = sinst[L.ct_ids[q0 + i]];
  __syncthreads();

  // phase A: distinct pairs of the tile
  for (int p = tid; p < nO * nQ; p += blockDim.x) {
    const int o = p / nQ, q = p - o * nQ;
    const ObsInst& O = so[o];
    const SrcInst& S = sq[q];
    const double t = dot3(S.dc, O.u);
    if (!same_segment(O, S)) {
      const double ex[3] = {sub(O.rm[0], S.rs[0]), sub(O.rm[1], S.rs[1]), sub(O.rm[2], S.rs[2])};
      double r[2], ri[2];
      gauss_geometry(ex, S.dc, S.an2, S.s, r, ri);
      pt[p] = regular_pair_value(r, ri, mul(S.half, t), S, f, tab);
    } else {
      pt[p] = self_pair_value(t, S, f, selfv[L.ct_ids[q0 + q]]);
    }
  }
  __syncthreads();
  assemble_tile(pt, nQ, L, tr, tc, npls, Zk, ldz);
}

// One CTA per tile and frequency (blockIdx.z).
__global__ void __launch_bounds__(256, 3) fill_pair_kernel(const ObsInst* __restrict__ oinst,
                                                        const SrcInst* __restrict__ sinst,
                                                        const int* __restrict__ tiles, int off_rt_ids,
                                                        int off_ct_off, int off_ct_ids, int off_row_local,
                                                        int off_col_local, int npls, int max_o, int max_q,
                                                        const FreqParams* __restrict__ fp,
                                                        const SelfVal* __restrict__ selfv, int nsrc,
                                                        double2* __restrict__ Z, long long ldz,
                                                        long long zstride) {
  extern __shared__ __align__(16) unsigned char sm[];
  const TileLists L = tile_lists(tiles, off_rt_ids, off_ct_off, off_ct_ids, off_row_local, off_col_local);
  const int k = blockIdx.z;
  pair_tile(oinst, sinst, L, blockIdx.x, blockIdx.y, npls, max_o, max_q, fp[k], selfv + (size_t)k * nsrc,
            Z + (size_t)k * zstride, ldz, sm);
}

// One matrix of a ragged launch over several geometries (one frequency each).
struct FillJob {
  const ObsInst* oi;
  const SrcInst* si;
  const int* tiles;
  int off_rt_ids, off_ct_off, off_ct_ids, off_row_local, off_col_local;
  int npls, n_tiles, max_o, max_q, nsrc;
  long long tile0;  // first block of this matrix in the launch (n_tiles^2 blocks)
  long long self0;  // first of its nsrc self values
  double2* z;
  long long ldz;
  FreqParams f;
};

// The last job whose first index (tile0 or self0) is <= i; jobs are in increasing
// order of both and job 0 starts at 0.
template <bool kSelf>
__device__ __forceinline__ int job_of(const FillJob* __restrict__ jobs, int njobs, long long i) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((kSelf ? jobs[mid].self0 : jobs[mid].tile0) <= i)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// Self values of every job's source instances at its frequency (self_values_kernel
// over a ragged list).
__global__ void self_values_ragged_kernel(const FillJob* __restrict__ jobs, int njobs, long long nself,
                                          SelfVal* __restrict__ out) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= nself) return;
  const FillJob& J = jobs[job_of<true>(jobs, njobs, i)];
  const SrcInst& S = J.si[i - J.self0];
  Cx Au, Ad, P;
  self_pair(S.dl, S.an, J.f.ka, &Au, &Ad, &P);
  out[i] = SelfVal{make_double2(Au.re, Au.im), make_double2(Ad.re, Ad.im), make_double2(P.re, P.im)};
}

// One CTA per tile of every job: the matrices of several geometries of any sizes in
// one launch, each tile computed as fill_pair_kernel computes it.
__global__ void __launch_bounds__(256, 3) fill_pair_ragged_kernel(const FillJob* __restrict__ jobs, int njobs,
                                                               const SelfVal* __restrict__ selfv) {
  extern __shared__ __align__(16) unsigned char sm[];
  const FillJob& J = jobs[job_of<false>(jobs, njobs, blockIdx.x)];
  const int t = (int)(blockIdx.x - J.tile0);
  const TileLists L = tile_lists(J.tiles, J.off_rt_ids, J.off_ct_off, J.off_ct_ids, J.off_row_local, J.off_col_local);
  pair_tile(J.oi, J.si, L, t % J.n_tiles, t / J.n_tiles, J.npls, J.max_o, J.max_q, J.f, selfv + J.self0, J.z, J.ldz,
            sm);
}

// Frequency-independent values of a pair, kept in shared memory across frequencies.
struct PairGeo {
  double r[2], ri[2];
  double tw;  // regular pair: (dl/2) t, frequency-independent; self pair: t
};

constexpr int kMultiThreads = 512;

// One CTA of 16 warps per tile for all nk frequencies: the pairs' geometry (R, 1/R,
// projection) is computed once, then for each frequency phase A (phase and ramps
// only) and phase B.  The arithmetic per pair and entry is fill_pair_kernel's.
__global__ void __launch_bounds__(kMultiThreads, 2) fill_pair_multi_kernel(
    const ObsInst* __restrict__ oinst, const SrcInst* __restrict__ sinst, const int* __restrict__ tiles,
    int off_rt_ids, int off_ct_off, int off_ct_ids, int off_row_local, int off_col_local, int npls, int max_o,
    int max_q, const FreqParams* __restrict__ fp, const SelfVal* __restrict__ selfv, int nsrc, int nk,
    double2* __restrict__ Z, long long ldz, long long zstride) {
  // shared memory holds only the pairs' values and geometry (two CTAs per SM where a
  // tile's pairs allow it); the instances are read through the read-only cache
  extern __shared__ __align__(16) unsigned char sm[];
  const double2* tab = g_sin_tab;
  PairVal* pt = reinterpret_cast<PairVal*>(sm);
  PairGeo* geo = reinterpret_cast<PairGeo*>(sm + (size_t)max_o * max_q * sizeof(PairVal));
  const TileLists L = tile_lists(tiles, off_rt_ids, off_ct_off, off_ct_ids, off_row_local, off_col_local);
  const int tr = blockIdx.x, tc = blockIdx.y;
  const int tid = threadIdx.x;
  const int o0 = L.rt_off[tr], nO = L.rt_off[tr + 1] - o0;
  const int q0 = L.ct_off[tc], nQ = L.ct_off[tc + 1] - q0;
  for (int p = tid; p < nO * nQ; p += blockDim.x) {
    const int o = p / nQ, q = p - o * nQ;
    const ObsInst& O = oinst[L.rt_ids[o0 + o]];
    const SrcInst& S = sinst[L.ct_ids[q0 + q]];
    PairGeo g;
    const double t = dot3(S.dc, O.u);
    if (!same_segment(O, S)) {
      const double ex[3] = {sub(O.rm[0], S.rs[0]), sub(O.rm[1], S.rs[1]), sub(O.rm[2], S.rs[2])};
      gauss_geometry(ex, S.dc, S.an2, S.s, g.r, g.ri);
      g.tw = mul(S.half, t);
    } else {
      g.r[0] = -1.0;  // self pair (a regular pair's R is at least the radius)
      g.tw = t;
    }
    geo[p] = g;
  }
  __syncthreads();
  for (int k = 0; k < nk; ++k) {
    const FreqParams f = fp[k];
    for (int p = tid; p < nO * nQ; p += blockDim.x) {
      const int q = p - (p / nQ) * nQ;
      const int qg = L.ct_ids[q0 + q];
      const SrcInst& S = sinst[qg];
      const PairGeo& g = geo[p];
      pt[p] = g.r[0] < 0.0 ? self_pair_value(g.tw, S, f, selfv[(size_t)k * nsrc + qg])
                           : regular_pair_value(g.r, g.ri, g.tw, S, f, tab);
    }
    __syncthreads();
    assemble_tile(pt, nQ, L, tr, tc, npls, Z + (size_t)k * zstride, ldz);
    __syncthreads();
  }
}

// Diagnostic: the table-driven sin/cos next to CUDA's sincos() on the same inputs.
__global__ void sincos_diag_kernel(const double* __restrict__ x, long long n, double* __restrict__ out) {
  const double2* tab = g_sin_tab;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double s, c, sr, cr;
    sincos_tab(x[i], tab, &s, &c);
    sincos(x[i], &sr, &cr);
    out[4 * i] = s;
    out[4 * i + 1] = c;
    out[4 * i + 2] = sr;
    out[4 * i + 3] = cr;
  }
}

size_t pair_smem_bytes(const PairTiles& t) {
  const size_t head = ((size_t)t.max_o * sizeof(ObsInst) + (size_t)t.max_q * sizeof(SrcInst) + 15) & ~(size_t)15;
  return head + (size_t)t.max_o * t.max_q * sizeof(PairVal);
}

size_t pair_multi_smem_bytes(const PairTiles& t) {
  return (size_t)t.max_o * t.max_q * (sizeof(PairVal) + sizeof(PairGeo));
}

// Builds the sin/cos table of the current device once (on its own stream, waited for,
// so every later launch on any stream sees it).
cudaError_t ensure_sin_table() {
  static std::mutex mu;
  static std::vector<char> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(mu);
  if ((int)done.size() <= dev) done.resize(dev + 1, 0);
  if (done[dev]) return cudaSuccess;
  cudaStream_t s = nullptr;
  e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e != cudaSuccess) return e;
  sin_table_setup_kernel<<<(kSinTab + 255) / 256, 256, 0, s>>>();
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (e == cudaSuccess) done[dev] = 1;
  return e;
}

}  // namespace

FreqParams freq_params(double ka) {
  const double pi = std::acos(-1.0);
  const double eta0 = 120. * pi;
  const double cq = eta0 / (4.0 * pi * ka);
  return FreqParams{ka, ka * ka, cq, (ka * ka) * cq, 0.5 * cq};
}

bool fill_multi_fits(const Plan& p) {
  if (!p.pt.ok) return false;
  const char* single = std::getenv("WMOM_FILL_SINGLE");
  if (single && single[0] == '1') return false;
  int dev = 0, smem_optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return false;
  return pair_multi_smem_bytes(p.pt) + 1024 <= (size_t)smem_optin;
}

cudaError_t launch_fill(const Plan& p, const double* d_fp, int nk, double2* z, long long ldz,
                        long long zstride, cudaStream_t stream) {
  if (nk <= 0 || p.npls <= 0) return cudaSuccess;
  cudaError_t te = ensure_sin_table();
  if (te != cudaSuccess) return te;
  const char* force_entry = std::getenv("WMOM_FILL_ENTRY");
  if (p.pt.ok && p.d_tiles && !(force_entry && force_entry[0] == '1')) {
    const FreqParams* fpd = reinterpret_cast<const FreqParams*>(d_fp);
    const int nsrc = (int)p.pt.src.size();
    SelfVal* selfv = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&selfv), sizeof(SelfVal) * (size_t)nsrc * nk, stream);
    if (e != cudaSuccess) return e;
    stats::Scope sc(stats::kFill, stream, 384.0 * p.npls * (double)p.npls * nk, 2);
    self_values_kernel<<<dim3((nsrc + 127) / 128, nk), 128, 0, stream>>>(p.d_si, nsrc, fpd, selfv);
    // several frequencies: one CTA of 16 warps per tile for all of them, when its
    // shared memory fits (the geometry of the pairs is then computed once per tile)
    const size_t msmem = pair_multi_smem_bytes(p.pt);
    if (nk > 1 && fill_multi_fits(p)) {
      e = allow_dynamic_smem((const void*)fill_pair_multi_kernel, msmem);
      if (e == cudaSuccess) {
        dim3 grid(p.pt.n_tiles, p.pt.n_tiles, 1);
        fill_pair_multi_kernel<<<grid, kMultiThreads, msmem, stream>>>(
            p.d_oi, p.d_si, p.d_tiles, p.off_rt_ids, p.off_ct_off, p.off_ct_ids, p.off_row_local, p.off_col_local,
            p.npls, p.pt.max_o, p.pt.max_q, fpd, selfv, nsrc, nk, z, ldz, zstride);
        e = cudaGetLastError();
      }
    } else {
      const size_t smem = pair_smem_bytes(p.pt);
      e = allow_dynamic_smem((const void*)fill_pair_kernel, smem);
      if (e == cudaSuccess) {
        dim3 grid(p.pt.n_tiles, p.pt.n_tiles, nk);
        fill_pair_kernel<<<grid, 256, smem, stream>>>(p.d_oi, p.d_si, p.d_tiles, p.off_rt_ids, p.off_ct_off,
                                                      p.off_ct_ids, p.off_row_local, p.off_col_local, p.npls,
                                                      p.pt.max_o, p.pt.max_q, fpd, selfv, nsrc, z, ldz, zstride);
        e = cudaGetLastError();
      }
    }
    const cudaError_t fe = cudaFreeAsync(selfv, stream);
    return e != cudaSuccess ? e : fe;
  }
  dim3 block(128);
  dim3 grid((p.npls + 127) / 128, p.npls, nk);
  stats::Scope sc(stats::kFill, stream, 384.0 * p.npls * (double)p.npls * nk);
  fill_entry_kernel<<<grid, block, 0, stream>>>(p.d_obs, p.d_src, p.npls,
                                                reinterpret_cast<const FreqParams*>(d_fp), z, ldz,
                                                zstride, p.ienv, p.sgnenv);
  return cudaGetLastError();
}

cudaError_t launch_fill_geometries(const Plan* const* plans, const double* ka, double2* const* z,
                                   const long long* ldz, int count, cudaStream_t stream) {
  if (count <= 0) return cudaSuccess;
  cudaError_t e = ensure_sin_table();
  if (e != cudaSuccess) return e;
  const char* force_entry = std::getenv("WMOM_FILL_ENTRY");
  const bool entry_only = force_entry && force_entry[0] == '1';
  auto pair_tiled = [&](const Plan& p) { return !entry_only && p.pt.ok && p.d_tiles; };
  std::vector<FillJob> jobs;
  std::vector<FreqParams> fps(count);
  long long ntiles = 0, nself = 0;
  size_t smem = 0;
  double work = 0.0;
  for (int i = 0; i < count; ++i) {
    const Plan& p = *plans[i];
    fps[i] = freq_params(ka[i]);
    if (p.npls <= 0 || !pair_tiled(p)) continue;
    FillJob j{};
    j.oi = p.d_oi;
    j.si = p.d_si;
    j.tiles = p.d_tiles;
    j.off_rt_ids = p.off_rt_ids;
    j.off_ct_off = p.off_ct_off;
    j.off_ct_ids = p.off_ct_ids;
    j.off_row_local = p.off_row_local;
    j.off_col_local = p.off_col_local;
    j.npls = p.npls;
    j.n_tiles = p.pt.n_tiles;
    j.max_o = p.pt.max_o;
    j.max_q = p.pt.max_q;
    j.nsrc = (int)p.pt.src.size();
    j.tile0 = ntiles;
    j.self0 = nself;
    j.z = z[i];
    j.ldz = ldz[i];
    j.f = fps[i];
    ntiles += (long long)j.n_tiles * j.n_tiles;
    nself += j.nsrc;
    smem = std::max(smem, pair_smem_bytes(p.pt));
    work += 384.0 * p.npls * (double)p.npls;
    jobs.push_back(j);
  }
  if (ntiles > 0x7fffffffLL) return cudaErrorInvalidValue;
  // one device block: the jobs, then every matrix's frequency constants
  const size_t jbytes = sizeof(FillJob) * jobs.size();
  const size_t bytes = jbytes + sizeof(FreqParams) * count;
  std::vector<unsigned char> h(bytes);
  if (jbytes) std::memcpy(h.data(), jobs.data(), jbytes);
  std::memcpy(h.data() + jbytes, fps.data(), sizeof(FreqParams) * count);
  unsigned char* d = nullptr;
  e = cudaMallocAsync(reinterpret_cast<void**>(&d), bytes, stream);
  if (e != cudaSuccess) return e;
  SelfVal* selfv = nullptr;
  e = cudaMemcpyAsync(d, h.data(), bytes, cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess && nself > 0) e = cudaMallocAsync(reinterpret_cast<void**>(&selfv), sizeof(SelfVal) * nself, stream);
  if (e == cudaSuccess && !jobs.empty()) {
    stats::Scope sc(stats::kFill, stream, work, 2);
    const FillJob* dj = reinterpret_cast<const FillJob*>(d);
    self_values_ragged_kernel<<<(unsigned)((nself + 127) / 128), 128, 0, stream>>>(dj, (int)jobs.size(), nself, selfv);
    e = allow_dynamic_smem((const void*)fill_pair_ragged_kernel, smem);
    if (e == cudaSuccess) {
      fill_pair_ragged_kernel<<<(unsigned)ntiles, 256, smem, stream>>>(dj, (int)jobs.size(), selfv);
      e = cudaGetLastError();
    }
  }
  // geometries outside the pair-tiled fill (ground plane) take the per-entry kernel
  const FreqParams* dfp = reinterpret_cast<const FreqParams*>(d + jbytes);
  for (int i = 0; i < count && e == cudaSuccess; ++i) {
    const Plan& p = *plans[i];
    if (p.npls > 0 && !pair_tiled(p))
      e = launch_fill(p, reinterpret_cast<const double*>(dfp + i), 1, z[i], ldz[i], 0, stream);
  }
  if (selfv) {
    const cudaError_t fe = cudaFreeAsync(selfv, stream);
    if (e == cudaSuccess) e = fe;
  }
  const cudaError_t fe = cudaFreeAsync(d, stream);
  return e != cudaSuccess ? e : fe;
}

}  // namespace wmom

extern "C" wmom_status wmom_diag_sincos(const double* d_x, long long n, double* d_out, void* stream) {
  if (n < 0 || (n > 0 && (!d_x || !d_out))) return WMOM_ERR_ARG;
  if (n == 0) return WMOM_OK;
  if (wmom::ensure_sin_table() != cudaSuccess) return WMOM_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const long long blocks = (n + 255) / 256;
  wmom::sincos_diag_kernel<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, s>>>(d_x, n, d_out);
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) return WMOM_ERR_CUDA;
  return WMOM_OK;
}
