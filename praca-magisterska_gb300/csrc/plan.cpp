// plan.cpp -- per-geometry source/observation tables (host C++, FP64).
//
// Each basis function n of the reference topology contributes two source halves
// (S_n+ = segment ips[n] from its first node to the centre node |ipc[n]|, rising
// ramp; S_n- = segment ips[n+nsmax] from the centre to its second node, falling
// ramp) and each test function m two observation points (the midpoints of S_m+
// and S_m-).  These are the reference's double-precision expressions of the float
// geometry ("wersja referencyjna/Zmatrix.cpp":69-84, 154-165, 252-276, 466-490),
// evaluated once per geometry here instead of once per entry, with the same
// rounding (this file is compiled without multiply-add contraction).
#include <cmath>
#include <cstdlib>

#include "wmom_internal.h"

namespace wmom {

double ka_from_mhz(float f) {
  const double c = 2.99792448E+8;
  const double pi = std::acos(-1.0);
  double lambda = c / f * 1E-6;
  return (pi + pi) / lambda;
}

int plan_build_tables(Plan* p, const float* x, const float* y, const float* z, const float* rad,
                      const int* ipc, const int* ips, const int* ise) {
  const int npls = p->npls, nsmax = p->nsmax;
  p->h_obs.assign(2 * (size_t)npls, ObsHalf{});
  p->h_src.assign(2 * (size_t)npls, SrcHalf{});
  auto node = [&](int k, double r[3]) {
    r[0] = (double)x[k - 1];
    r[1] = (double)y[k - 1];
    r[2] = (double)z[k - 1];
  };
  auto valid_node = [&](int k) { return k >= 1 && k <= nsmax; };
  auto valid_seg = [&](int s) { return s >= 1 && s <= nsmax; };
  const double sg[3] = {(double)p->sgnx, (double)p->sgny, (double)p->sgnz};
  for (int b = 0; b < npls; ++b) {
    const int np = std::abs(ipc[b]);
    const int s1 = ips[b], s2 = ips[b + nsmax];
    if (!valid_node(np) || !valid_seg(s1) || !valid_seg(s2)) return WMOM_ERR_GEOMETRY;
    const int n1l = ise[s1 - 1], n1r = ise[s1 + nsmax - 1];
    const int n2l = ise[s2 - 1], n2r = ise[s2 + nsmax - 1];
    if (!valid_node(n1l) || !valid_node(n1r) || !valid_node(n2l) || !valid_node(n2r))
      return WMOM_ERR_GEOMETRY;
    double rp[3], r1[3], r2[3];
    node(np, rp);
    node(n1l, r1);  // first node of S+
    node(n2r, r2);  // second node of S-
    // observation halves
    ObsHalf& o0 = p->h_obs[2 * (size_t)b];
    ObsHalf& o1 = p->h_obs[2 * (size_t)b + 1];
    for (int k = 0; k < 3; ++k) {
      o0.rm[k] = 0.5 * (rp[k] + r1[k]);
      o0.lm[k] = rp[k] - o0.rm[k];
      o1.rm[k] = 0.5 * (r2[k] + rp[k]);
      o1.lm[k] = o1.rm[k] - rp[k];
    }
    o0.ml = n1l;
    o0.mr = n1r;
    o1.ml = n2l;
    o1.mr = n2r;
    o0.on_ground = (z[n1l - 1] < 1.e-6 && z[n1r - 1] < 1.e-6) ? 1 : 0;
    o1.on_ground = (z[n2l - 1] < 1.e-6 && z[n2r - 1] < 1.e-6) ? 1 : 0;
    // source halves
    for (int h = 0; h < 2; ++h) {
      SrcHalf& s = p->h_src[2 * (size_t)b + h];
      const int seg = h == 0 ? s1 : s2;
      const double* ra = h == 0 ? r1 : rp;  // start of the parametrisation
      const double* re = h == 0 ? rp : r2;  // end
      double rd[3];
      for (int k = 0; k < 3; ++k) {
        s.rs[k] = ra[k];
        rd[k] = re[k] - ra[k];
      }
      const double dl = std::sqrt(rd[0] * rd[0] + rd[1] * rd[1] + rd[2] * rd[2]);
      if (!(dl > 0.0)) return WMOM_ERR_GEOMETRY;
      s.dl = dl;
      for (int k = 0; k < 3; ++k) s.dc[k] = rd[k] / dl;
      s.an = (double)rad[seg - 1];
      // mirrored source (the reference scales both nodes by sgn and recomputes;
      // with sgn = +-1 that is exactly the mirrored start and unit vector)
      for (int k = 0; k < 3; ++k) {
        s.rs_img[k] = sg[k] * ra[k];
        double rdi = sg[k] * re[k] - sg[k] * ra[k];
        s.dc_img[k] = rdi / dl;
      }
      s.nl = h == 0 ? n1l : n2l;
      s.nr = h == 0 ? n1r : n2r;
    }
  }
  return WMOM_OK;
}

}  // namespace wmom
