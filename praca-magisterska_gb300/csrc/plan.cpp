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
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <utility>
#include <vector>

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
  p->loops = wire_loops(p->h_src, nsmax, z, p->ienv == 2);
  return WMOM_OK;
}

// Independent closed current paths of the structure: the cycle rank E - V + C of the
// graph whose edges are the segments the basis functions use and whose vertices are
// their nodes (over a PEC ground, every node on the ground plane is one vertex: a
// current returns through the plane; the short virtual wires the topology lays in the
// plane to join a grounded wire to its image are then no edges).  Open wires and
// trees have none.  Loops are
// what makes the EFIE's conditioning grow as 1/(ka)^2 towards low frequencies:
// divergence-free loop currents see only the vector potential, which vanishes with k.
int wire_loops(const std::vector<SrcHalf>& src, int nsmax, const float* z, bool ground) {
  std::vector<int> parent(nsmax + 2);
  for (size_t i = 0; i < parent.size(); ++i) parent[i] = (int)i;
  const int gnd = nsmax + 1;
  auto vertex = [&](int k) { return ground && std::fabs(z[k - 1]) < 1.e-6f ? gnd : k; };
  auto find = [&](int a) {
    while (parent[a] != a) a = parent[a] = parent[parent[a]];
    return a;
  };
  std::vector<std::pair<int, int>> seg;
  seg.reserve(src.size());
  for (const SrcHalf& h : src) seg.emplace_back(std::min(h.nl, h.nr), std::max(h.nl, h.nr));
  std::sort(seg.begin(), seg.end());
  seg.erase(std::unique(seg.begin(), seg.end()), seg.end());
  int loops = 0;
  for (const auto& e : seg) {
    if (vertex(e.first) == gnd && vertex(e.second) == gnd) continue;  // lies in the ground plane
    const int a = find(vertex(e.first)), b = find(vertex(e.second));
    if (a == b)
      ++loops;  // this segment closes a path that already joins its nodes
    else
      parent[a] = b;
  }
  return loops;
}

}  // namespace wmom

// ----------------------------------------------------------------------------
// Pair-tiled fill tables.  Neighbouring basis functions share segments, so the
// (observation point, source half-segment) integrals of one tile of 32 x 32 entries
// involve only ~33 x 33 distinct pairs instead of 4 x 32 x 32.  This builds the
// distinct instances and, per tile, the list of them and every half's position in
// that list.  The per-entry values it feeds are the same expressions as above.
// Free space only; the image terms of a PEC ground use the per-entry fill.
// ----------------------------------------------------------------------------
#include <array>
#include <cstring>
#include <map>
#include <unordered_map>
#include <tuple>

namespace wmom {

void plan_build_pair_tiles(Plan* p, const float* x, const float* y, const float* z, const float* rad,
                           const int* ipc, const int* ips, const int* ise) {
  PairTiles& t = p->pt;
  t = PairTiles{};
  if (p->ienv != 1) return;
  const int npls = p->npls, nsmax = p->nsmax;
  const double kGl2C = 0.288675134594812882;
  auto node = [&](int k, double r[3]) {
    r[0] = (double)x[k - 1];
    r[1] = (double)y[k - 1];
    r[2] = (double)z[k - 1];
  };
  // instance ids in first-seen order (hash maps, reserved once: ordered maps made this
  // table build several milliseconds of every N = 8192 plan)
  struct KeyHash {
    size_t operator()(const std::array<uint32_t, 5>& k) const {
      uint64_t h = 0x9E3779B97F4A7C15ull;
      for (uint32_t v : k) h = (h ^ v) * 0xBF58476D1CE4E5B9ull;
      return (size_t)(h ^ (h >> 31));
    }
  };
  std::unordered_map<std::array<uint32_t, 5>, int, KeyHash> okey, qkey;
  okey.reserve(2 * (size_t)npls);
  qkey.reserve(2 * (size_t)npls);
  std::vector<int> obs_of(2 * (size_t)npls), neg_of(2 * (size_t)npls), src_of(2 * (size_t)npls);
  for (int b = 0; b < npls; ++b) {
    const int np = std::abs(ipc[b]);
    const int s1 = ips[b], s2 = ips[b + nsmax];
    for (int h = 0; h < 2; ++h) {
      const int ms = h == 0 ? s1 : s2;
      const int ml = ise[ms - 1], mr = ise[ms + nsmax - 1];
      const int other = h == 0 ? ise[s1 - 1] : ise[s2 + nsmax - 1];
      const int lo = std::min(np, other), hi = std::max(np, other);
      const std::array<uint32_t, 5> key{(uint32_t)ml, (uint32_t)mr, (uint32_t)lo, (uint32_t)hi, 0u};
      auto it = okey.find(key);
      int id;
      const ObsHalf& oh = p->h_obs[2 * (size_t)b + h];
      if (it == okey.end()) {
        ObsInst oi{};
        double rh[3];
        node(hi, rh);
        for (int k = 0; k < 3; ++k) {
          oi.rm[k] = oh.rm[k];
          oi.u[k] = rh[k] - oi.rm[k];
        }
        oi.ml = ml;
        oi.mr = mr;
        oi.on_ground = oh.on_ground;
        id = (int)t.obs.size();
        t.obs.push_back(oi);
        okey.emplace(key, id);
      } else {
        id = it->second;
      }
      const ObsInst& oi = t.obs[id];
      // the observation point and the test vector must be the instance's, bit for bit
      bool pos = true, neg = true;
      for (int k = 0; k < 3; ++k) {
        if (oi.rm[k] != oh.rm[k]) return;
        pos = pos && (oh.lm[k] == oi.u[k]);
        neg = neg && (oh.lm[k] == -oi.u[k]);
      }
      if (!pos && !neg) return;
      obs_of[2 * (size_t)b + h] = id;
      neg_of[2 * (size_t)b + h] = pos ? 0 : 1;
    }
    for (int sg = 0; sg < 2; ++sg) {
      const SrcHalf& sh = p->h_src[2 * (size_t)b + sg];
      const int seg = sg == 0 ? s1 : s2;
      const int a = sg == 0 ? ise[s1 - 1] : np;
      const int e = sg == 0 ? np : ise[s2 + nsmax - 1];
      uint32_t rbits;
      std::memcpy(&rbits, &rad[seg - 1], 4);
      const std::array<uint32_t, 5> key{(uint32_t)a, (uint32_t)e, (uint32_t)sh.nl, (uint32_t)sh.nr, rbits};
      auto it = qkey.find(key);
      int id;
      if (it == qkey.end()) {
        SrcInst si{};
        for (int k = 0; k < 3; ++k) {
          si.rs[k] = sh.rs[k];
          si.dc[k] = sh.dc[k];
        }
        si.dl = sh.dl;
        si.an = sh.an;
        si.an2 = sh.an * sh.an;
        si.half = sh.dl * 0.5;
        const double aa = 0.5 * (0.0 + sh.dl), bb = sh.dl - 0.0, cc = kGl2C * bb;
        si.s[0] = aa + cc;
        si.s[1] = aa - cc;
        for (int g = 0; g < 2; ++g) {
          si.w_up[g] = si.s[g] / sh.dl;
          si.w_dn[g] = (sh.dl - si.s[g]) / sh.dl;
        }
        si.nl = sh.nl;
        si.nr = sh.nr;
        id = (int)t.src.size();
        t.src.push_back(si);
        qkey.emplace(key, id);
      } else {
        id = it->second;
      }
      src_of[2 * (size_t)b + sg] = id;
    }
  }
  const int T = t.tile;
  t.n_tiles = (npls + T - 1) / T;
  t.row_local.assign(2 * (size_t)npls, 0);
  t.col_local.assign(2 * (size_t)npls, 0);
  t.rt_off.assign(t.n_tiles + 1, 0);
  t.ct_off.assign(t.n_tiles + 1, 0);
  // a tile's distinct instances, in first-seen order: at most 2 T of each, so a linear
  // search of the tile's list
  auto local_id = [](std::vector<int>& ids, size_t from, int v) -> int {
    for (size_t i = from; i < ids.size(); ++i)
      if (ids[i] == v) return (int)(i - from);
    ids.push_back(v);
    return (int)(ids.size() - 1 - from);
  };
  for (int tile = 0; tile < t.n_tiles; ++tile) {
    const size_t ro = t.rt_ids.size(), co = t.ct_ids.size();
    const int b0 = tile * T, b1 = std::min(npls, b0 + T);
    for (int b = b0; b < b1; ++b)
      for (int h = 0; h < 2; ++h) {
        const int l = local_id(t.rt_ids, ro, obs_of[2 * (size_t)b + h]);
        t.row_local[2 * (size_t)b + h] = l | (neg_of[2 * (size_t)b + h] ? (1 << 30) : 0);
        t.col_local[2 * (size_t)b + h] = local_id(t.ct_ids, co, src_of[2 * (size_t)b + h]);
      }
    t.rt_off[tile + 1] = (int)t.rt_ids.size();
    t.ct_off[tile + 1] = (int)t.ct_ids.size();
    t.max_o = std::max(t.max_o, (int)(t.rt_ids.size() - ro));
    t.max_q = std::max(t.max_q, (int)(t.ct_ids.size() - co));
  }
  const size_t smem = (size_t)t.max_o * sizeof(ObsInst) + (size_t)t.max_q * sizeof(SrcInst) +
                      (size_t)t.max_o * t.max_q * 48;
  t.ok = smem <= 200 * 1024;
}

}  // namespace wmom
