// topology.cpp -- wire geometry input and basis-function topology (host C++).
//
// Restates the reference's geometry path so that the arrays fed to the fill are
// bit-identical to the reference's:
//   * geo_parse       <- geoinp()     "wersja referencyjna/Configuration.cpp":5-75
//   * build_topology  <- configwire() "wersja referencyjna/Configuration.cpp":112-520
// The node subdivision runs in float32 exactly as the reference does it
// (x = x0 + j*dx with dx = (x1-x0)/ns, all float), because those float nodes
// define every Z entry.  Index conventions are the reference's: arrays are stored
// 0-based but hold 1-based node/segment/basis numbers; the second column of
// ise/isp/ips/iwe lives at offset nsmax; ipc is negative for junction functions.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "wmom_internal.h"

namespace wmom {

int geo_parse(std::istream& in, int nnmax, int nwmax, int ntmax, GeoInput* g, std::string* err) {
  std::string line;
  std::getline(in, line);  // two comment lines
  std::getline(in, line);
  g->nnod = 0;
  g->nw = 0;
  g->nt = 0;
  if (!(in >> g->nnod)) {
    *err = "geo: cannot read the node count";
    return WMOM_ERR_GEOMETRY;
  }
  if (g->nnod > nnmax || g->nnod < 0) {
    *err = "geo: node count exceeds nnmax";
    return WMOM_ERR_GEOMETRY;
  }
  g->xnod.assign(g->nnod + 1, 0.f);
  g->ynod.assign(g->nnod + 1, 0.f);
  g->znod.assign(g->nnod + 1, 0.f);
  for (int i = 1; i <= g->nnod; ++i) {
    if (!(in >> g->xnod[i] >> g->ynod[i] >> g->znod[i])) {
      *err = "geo: truncated node section";
      return WMOM_ERR_GEOMETRY;
    }
  }
  if (!(in >> g->nw)) {
    *err = "geo: cannot read the wire count";
    return WMOM_ERR_GEOMETRY;
  }
  if (g->nw > nwmax || g->nw < 0) {
    *err = "geo: wire count exceeds nwmax";
    return WMOM_ERR_GEOMETRY;
  }
  g->iwn.assign(2 * g->nw + 1, 0);
  g->wrad.assign(g->nw + 1, 0.f);
  g->nsw.assign(g->nw + 1, 0);
  for (int i = 1; i <= g->nw; ++i) {
    if (!(in >> g->iwn[i] >> g->iwn[i + g->nw] >> g->wrad[i] >> g->nsw[i])) {
      *err = "geo: truncated wire section";
      return WMOM_ERR_GEOMETRY;
    }
    if (g->iwn[i] < 1 || g->iwn[i] > g->nnod || g->iwn[i + g->nw] < 1 ||
        g->iwn[i + g->nw] > g->nnod || g->nsw[i] < 1) {
      *err = "geo: wire references a missing node or has no segments";
      return WMOM_ERR_GEOMETRY;
    }
  }
  if (!(in >> g->nt)) g->nt = 0;  // the patch section is optional in practice
  if (g->nt > ntmax || g->nt < 0) {
    *err = "geo: patch count exceeds ntmax";
    return WMOM_ERR_GEOMETRY;
  }
  g->iwt.assign(3 * g->nt, 0);
  for (int i = 0; i < g->nt; ++i) in >> g->iwt[i] >> g->iwt[i + g->nt] >> g->iwt[i + 2 * g->nt];
  return WMOM_OK;
}

namespace {

// Working state of the topology builder, 1-based like the reference.
struct Builder {
  int nsmax, nwmax;
  std::vector<float> x, y, z, rad;
  std::vector<int> ise, isp, ips, ipc, iwe;
  int npnt = 0, np = 0, nseg = 0;
  std::string err;

  Builder(int nsmax_, int nwmax_) : nsmax(nsmax_), nwmax(nwmax_) {
    x.assign(nsmax + 2, 0.f);
    y.assign(nsmax + 2, 0.f);
    z.assign(nsmax + 2, 0.f);
    rad.assign(nsmax + 2, 0.f);
    ipc.assign(nsmax + 2, 0);
    ise.assign(2 * nsmax + 2, 0);
    isp.assign(2 * nsmax + 2, 0);
    ips.assign(2 * nsmax + 2, 0);
    iwe.assign(2 * nsmax + 2, 0);
  }
  bool new_segment() {
    if (++nseg > nsmax) {
      err = "topology: number of segments exceeds nsmax";
      return false;
    }
    return true;
  }
  bool new_basis() {
    if (++np > nsmax - nwmax) {
      err = "topology: number of basis functions on wires exceeds nsmax - nwmax";
      return false;
    }
    return true;
  }
};

}  // namespace

int build_topology(const GeoInput& gin, int nsmax, int nwmax, int ienv, Topology* out,
                   std::string* listing, std::string* err) {
  const int nnod = gin.nnod, nw = gin.nw;
  std::ostringstream lst;
  if (nw == 0) {
    lst << "\n -== NO WIRES IN GEOMETRY ==- \n";
    if (listing) *listing = lst.str();
    out->npnt = out->npls = out->nseg = 0;
    return WMOM_OK;
  }
  if (ienv == 2) {
    for (int i = 1; i <= nnod; ++i)
      if (gin.znod[i] < 0.f) {
        *err = "topology: z-coordinate of a node is negative above a PEC ground";
        return WMOM_ERR_GEOMETRY;
      }
  }
  // Image-side virtual wires (one per grounded node / touching wire) come first,
  // then the real nodes and wires, shifted behind them.
  int ngrounded = 0;
  if (ienv == 2)
    for (int i = 1; i <= nnod; ++i)
      if (std::fabs(gin.znod[i]) < 1.e-6) ++ngrounded;
  const int nvnod = ngrounded + nnod;
  const int nvw = ngrounded + nw;
  std::vector<float> xv(nvnod + 1, 0.f), yv(nvnod + 1, 0.f), zv(nvnod + 1, 0.f),
      wradv(nvw + 1, 0.f);
  std::vector<int> iwnv(2 * nvw + 1, 0), nswv(nvw + 1, 0);
  int ivn = 0, ivw = 0;
  if (ienv == 2) {
    for (int i = 1; i <= nnod; ++i) {
      if (!(std::fabs(gin.znod[i]) < 1.e-6)) continue;
      for (int j = 1; j <= nw; ++j) {
        if (gin.iwn[j] != i && gin.iwn[j + nw] != i) continue;
        ++ivn;
        ++ivw;
        if (ivw > nvw || ivn > nvnod) {
          *err = "topology: a grounded node touches more than one wire";
          return WMOM_ERR_GEOMETRY;
        }
        float dx = gin.xnod[gin.iwn[j + nw]] - gin.xnod[gin.iwn[j]];
        float dy = gin.ynod[gin.iwn[j + nw]] - gin.ynod[gin.iwn[j]];
        float dz = gin.znod[gin.iwn[j + nw]] - gin.znod[gin.iwn[j]];
        float dl = std::sqrt(dx * dx + dy * dy + dz * dz) / (float)gin.nsw[j];
        xv[ivn] = gin.xnod[i] + dl;
        yv[ivn] = gin.ynod[i];
        zv[ivn] = gin.znod[i];
        iwnv[ivw] = i + ngrounded;
        iwnv[ivw + nvw] = ivn;
        wradv[ivw] = gin.wrad[j];
        nswv[ivw] = 1;
      }
    }
  }
  for (int i = 1; i <= nnod; ++i) {
    xv[ivn + i] = gin.xnod[i];
    yv[ivn + i] = gin.ynod[i];
    zv[ivn + i] = gin.znod[i];
  }
  for (int i = 1; i <= nw; ++i) {
    iwnv[ivw + i] = gin.iwn[i] + ngrounded;
    iwnv[ivw + i + nvw] = gin.iwn[i + nw] + ngrounded;
    wradv[ivw + i] = gin.wrad[i];
    nswv[ivw + i] = gin.nsw[i];
  }

  Builder b(nsmax, nwmax);
  auto& ise = b.ise;
  auto& isp = b.isp;
  auto& ips = b.ips;
  auto& ipc = b.ipc;
  auto& iwe = b.iwe;
  int ip = 0;  // point counter
  for (int m = 1; m <= nvw; ++m) {
    const int start = iwnv[m], end = iwnv[m + nvw];
    const int ns = nswv[m];
    float dx = xv[end] - xv[start];
    float dy = yv[end] - yv[start];
    float dz = zv[end] - zv[start];
    if (ns > 1) {
      dx = dx / (float)ns;
      dy = dy / (float)ns;
      dz = dz / (float)ns;
    }
    // Junction at the start of wire m: join the first earlier wire that starts
    // (reversed copy of its first segment) or ends (copy of its last segment) here.
    bool joined = false;
    for (int n = 1; n < m; ++n) {
      int src_seg = 0;
      bool reversed = false;
      if (start == iwnv[n]) {
        src_seg = iwe[n];
        reversed = true;
      } else if (start == iwnv[n + nvw]) {
        src_seg = iwe[n + nsmax];
      } else {
        continue;
      }
      joined = true;
      if (!b.new_segment()) return *err = b.err, WMOM_ERR_GEOMETRY;
      const int s = b.nseg;
      if (reversed) {
        ise[s] = ise[src_seg + nsmax];
        ise[s + nsmax] = ise[src_seg];
      } else {
        ise[s] = ise[src_seg];
        ise[s + nsmax] = ise[src_seg + nsmax];
      }
      b.rad[s] = wradv[n];
      if (!b.new_basis()) return *err = b.err, WMOM_ERR_GEOMETRY;
      ipc[b.np] = -ise[s + nsmax];
      isp[s] = 0;
      isp[s + nsmax] = b.np;
      ips[b.np] = s;
      break;
    }
    if (!joined) {
      ++ip;
      b.x[ip] = xv[start];
      b.y[ip] = yv[start];
      b.z[ip] = zv[start];
    }
    // Interior points and the wire's own segments.
    for (int j = 1; j <= ns; ++j) {
      ++ip;
      if (j == ns) {
        b.x[ip] = xv[end];
        b.y[ip] = yv[end];
        b.z[ip] = zv[end];
      } else {
        const float fj = (float)j;
        b.x[ip] = xv[start] + fj * dx;
        b.y[ip] = yv[start] + fj * dy;
        b.z[ip] = zv[start] + fj * dz;
      }
      if (!b.new_segment()) return *err = b.err, WMOM_ERR_GEOMETRY;
      const int s = b.nseg;
      b.rad[s] = wradv[m];
      if (j == 1) iwe[m] = joined ? s - 1 : s;
      ise[s] = joined ? ise[s - 1 + nsmax] : ip - 1;
      ise[s + nsmax] = ip;
      isp[s] = 0;
      isp[s + nsmax] = 0;
    }
    // Basis functions spanning consecutive segments; with a start junction the
    // junction function (already numbered) takes the wire's first segment as S-.
    const int first = iwe[m];
    int last = first + ns - 2;
    if (joined) {
      ++last;
      --b.np;
    }
    for (int s = first; s <= last; ++s) {
      if (!b.new_basis()) return *err = b.err, WMOM_ERR_GEOMETRY;
      isp[s + nsmax] = b.np;
      isp[s + 1] = b.np;
      ips[b.np] = s;
      ips[b.np + nsmax] = s + 1;
      if (!(joined && s == first)) ipc[b.np] = ise[s + nsmax];
    }
    iwe[m + nsmax] = b.nseg;
    // Junction at the end of wire m: join the first earlier wire that starts
    // (copy of its first segment) or ends (reversed copy of its last segment) here.
    for (int n = 1; n < m; ++n) {
      int src_seg = 0;
      bool reversed = false;
      if (end == iwnv[n]) {
        src_seg = iwe[n];
      } else if (end == iwnv[n + nvw]) {
        src_seg = iwe[n + nsmax];
        reversed = true;
      } else {
        continue;
      }
      if (!b.new_segment()) return *err = b.err, WMOM_ERR_GEOMETRY;
      const int s = b.nseg;
      --ip;  // the wire's end point duplicates the joined node
      if (reversed) {
        ise[s] = ise[src_seg + nsmax];
        ise[s + nsmax] = ise[src_seg];
      } else {
        ise[s] = ise[src_seg];
        ise[s + nsmax] = ise[src_seg + nsmax];
      }
      b.rad[s] = wradv[n];
      if (!b.new_basis()) return *err = b.err, WMOM_ERR_GEOMETRY;
      ipc[b.np] = -ise[s];
      const int lastseg = iwe[m + nsmax];
      isp[lastseg + nsmax] = b.np;
      isp[s] = b.np;
      isp[s + nsmax] = 0;
      ips[b.np] = lastseg;
      ips[b.np + nsmax] = s;
      ise[lastseg + nsmax] = std::abs(ipc[b.np]);
      iwe[m + nsmax] = s;
      break;
    }
  }
  b.npnt = ip;

  // configwire.txt listing (Configuration.cpp:461-481): basis functions of every
  // real wire with the coordinates of their centre nodes.
  lst << "\n Number of wires and basis functions: " << nw << '\t' << b.np << "\n";
  for (int w = 1; w <= nw; ++w) {
    lst << " Drucik nr " << w << "\n";
    const int iw = w + ivw;
    const int nb = isp[iwe[iw] + nsmax];
    const int ne = isp[iwe[iw + nsmax]];
    for (int j = nb; j <= ne; ++j) {
      if (j == 0) {
        lst << " no basis function(s)\n";
      } else {
        const int p = std::abs(ipc[j]);
        lst << j << '\t' << b.x[p] << '\t' << b.y[p] << '\t' << b.z[p] << "\n";
      }
    }
  }
  if (listing) *listing = lst.str();

  // 1-based -> 0-based storage, as the reference leaves its arrays.
  out->npnt = b.npnt;
  out->npls = b.np;
  out->nseg = b.nseg;
  for (int i = 1; i <= nsmax; ++i) {
    out->x[i - 1] = b.x[i];
    out->y[i - 1] = b.y[i];
    out->z[i - 1] = b.z[i];
    out->rad[i - 1] = b.rad[i];
    out->ipc[i - 1] = ipc[i];
  }
  for (int i = 1; i <= nsmax; ++i) {
    out->ise[i - 1] = ise[i];
    out->ise[i - 1 + nsmax] = ise[i + nsmax];
    out->isp[i - 1] = isp[i];
    out->isp[i - 1 + nsmax] = isp[i + nsmax];
    out->ips[i - 1] = ips[i];
    out->ips[i - 1 + nsmax] = ips[i + nsmax];
    out->iwe[i - 1] = iwe[i];
    out->iwe[i - 1 + nsmax] = iwe[i + nsmax];
  }
  // The reference shifts both columns in place in one loop (Configuration.cpp:497-514):
  // its first step overwrites the first column's entry nsmax with the second column's
  // first entry before the last step moves it down, so slot nsmax - 1 of every
  // two-column array ends up holding that entry.  No basis function or segment number
  // reaches that slot; it is kept for drop-in callers that read whole arrays.
  out->ise[nsmax - 1] = ise[nsmax + 1];
  out->isp[nsmax - 1] = isp[nsmax + 1];
  out->ips[nsmax - 1] = ips[nsmax + 1];
  out->iwe[nsmax - 1] = iwe[nsmax + 1];
  return WMOM_OK;
}

}  // namespace wmom

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" wmom_status wmom_topology_from_geo(const char* geo_text, int ienv, int nsmax, int nwmax,
                                              wmom_topology* topo, char* listing,
                                              size_t listing_cap, char* errbuf, size_t errcap) {
  if (!geo_text || !topo || nsmax <= 0 || nwmax < 0 || (ienv != 1 && ienv != 2) || !topo->x ||
      !topo->y || !topo->z || !topo->rad || !topo->ipc || !topo->ips || !topo->ise || !topo->isp ||
      !topo->iwe) {
    if (errbuf && errcap) std::snprintf(errbuf, errcap, "wmom_topology_from_geo: bad argument");
    return WMOM_ERR_ARG;
  }
  std::istringstream in{std::string(geo_text)};
  wmom::GeoInput g;
  std::string err;
  int st = wmom::geo_parse(in, 3000, nwmax, 5000, &g, &err);
  if (st == WMOM_OK) {
    wmom::Topology t;
    t.x = topo->x;
    t.y = topo->y;
    t.z = topo->z;
    t.rad = topo->rad;
    t.ipc = topo->ipc;
    t.ips = topo->ips;
    t.ise = topo->ise;
    t.isp = topo->isp;
    t.iwe = topo->iwe;
    std::string lst;
    st = wmom::build_topology(g, nsmax, nwmax, ienv, &t, &lst, &err);
    if (st == WMOM_OK) {
      topo->nsmax = nsmax;
      topo->npnt = t.npnt;
      topo->npls = t.npls;
      topo->nseg = t.nseg;
      topo->nw = g.nw;
      if (listing && listing_cap) {  // truncated to listing_cap - 1 bytes, no padding
        const size_t len = std::min(lst.size(), listing_cap - 1);
        std::memcpy(listing, lst.data(), len);
        listing[len] = 0;
      }
    }
  }
  if (st != WMOM_OK && errbuf && errcap) std::snprintf(errbuf, errcap, "%s", err.c_str());
  return (wmom_status)st;
}
