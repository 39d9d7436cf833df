// dropin.cpp -- the reference's C++ entry points (see include/wmom_dropin.h)
// implemented on top of libwmom: geometry/topology on the host, the fill on the GPU.
#include "../../include/wmom_dropin.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "wmom_internal.h"

namespace {

[[noreturn]] void fatal(const std::string& msg) {
  std::cout << " " << msg << std::endl;
  std::exit(0);  // the reference's behaviour on bad input (Configuration.cpp:28-34)
}

void fill_to_host(cuDoubleComplex* cz, float* x, float* y, float* z, int* ipc, int* ips, int* ise, float* rad,
                  int npls, double ka, int nsmax, int ienv, float sgnx, float sgny, float sgnz, float sgnenv) {
  wmom_plan plan = nullptr;
  wmom_status st = wmom_plan_create(x, y, z, rad, ipc, ips, ise, nsmax, npls, ienv, sgnx, sgny, sgnz, sgnenv, &plan);
  if (st != WMOM_OK) fatal(std::string("zmatrix: ") + wmom_status_string(st));
  void* dz = nullptr;
  const size_t bytes = sizeof(cuDoubleComplex) * (size_t)npls * npls;
  if (cudaMalloc(&dz, bytes) != cudaSuccess) fatal("zmatrix: out of device memory");
  st = wmom_fill(plan, &ka, 1, dz, npls, (long long)npls * npls, nullptr);
  if (st != WMOM_OK) fatal(std::string("zmatrix: ") + wmom_status_string(st));
  if (cudaMemcpy(cz, dz, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) fatal("zmatrix: copy failed");
  cudaFree(dz);
  wmom_plan_destroy(plan);
}

}  // namespace

void geoinp(int nnmax, int nwmax, int ntmax, int& nnod, float* xnod, float* ynod, float* znod, int& nw, int* iwn,
            float* wrad, int* nsw, int& nt, int* iwt) {
  std::ifstream f("dipol.geo");
  if (!f.good()) fatal("Nie udalo sie otworzyc pliku dipol.geo");
  std::cout << " Nazwa pliku geo: dipol.geo" << std::endl;
  wmom::GeoInput g;
  std::string err;
  if (wmom::geo_parse(f, nnmax, nwmax, ntmax, &g, &err) != WMOM_OK) fatal(err);
  nnod = g.nnod;
  nw = g.nw;
  nt = g.nt;
  for (int i = 1; i <= nnod; ++i) {
    xnod[i] = g.xnod[i];
    ynod[i] = g.ynod[i];
    znod[i] = g.znod[i];
  }
  for (int i = 1; i <= nw; ++i) {
    iwn[i] = g.iwn[i];
    iwn[i + nw] = g.iwn[i + nw];
    wrad[i] = g.wrad[i];
    nsw[i] = g.nsw[i];
  }
  for (int i = 0; i < 3 * nt; ++i) iwt[i] = g.iwt[i];
}

void configwire(int& npnt, int nnod, float* xnod, float* ynod, float* znod, float* x, float* y, float* z, int nw,
                int* iwn, float* wrad, int* nsw, int* ise, int* isp, int* ips, int* ipc, int* iwe, float* rad,
                int& nplsw, int& nseg, int nsmax, int nwmax, int ienv) {
  wmom::GeoInput g;
  g.nnod = nnod;
  g.nw = nw;
  g.xnod.assign(xnod, xnod + nnod + 1);
  g.ynod.assign(ynod, ynod + nnod + 1);
  g.znod.assign(znod, znod + nnod + 1);
  g.iwn.assign(iwn, iwn + 2 * nw + 1);
  g.wrad.assign(wrad, wrad + nw + 1);
  g.nsw.assign(nsw, nsw + nw + 1);
  wmom::Topology t;
  t.x = x;
  t.y = y;
  t.z = z;
  t.rad = rad;
  t.ipc = ipc;
  t.ips = ips;
  t.ise = ise;
  t.isp = isp;
  t.iwe = iwe;
  std::string listing, err;
  if (wmom::build_topology(g, nsmax, nwmax, ienv, &t, &listing, &err) != WMOM_OK) fatal(err);
  std::ofstream wf("configwire.txt");
  wf << listing;
  npnt = t.npnt;
  nplsw = t.npls;
  nseg = t.nseg;
  // geometry input arrays move to 0-based storage as well
  for (int i = 1; i <= nnod; ++i) {
    xnod[i - 1] = g.xnod[i];
    ynod[i - 1] = g.ynod[i];
    znod[i - 1] = g.znod[i];
  }
  for (int i = 1; i <= nw; ++i) {
    iwn[i - 1] = g.iwn[i];
    iwn[i - 1 + nw] = g.iwn[i + nw];
    wrad[i - 1] = g.wrad[i];
    nsw[i - 1] = g.nsw[i];
  }
}

void config(int& npnt, int nnod, float* xnod, float* ynod, float* znod, float* x, float* y, float* z, int nw,
            int* iwn, float* wrad, int* nsw, int* ise, int* isp, int* ips, int* ipc, int* iwe, float* rad,
            int& npls, int& nplsw, int& nseg, int nsmax, int nwmax, int ienv) {
  configwire(npnt, nnod, xnod, ynod, znod, x, y, z, nw, iwn, wrad, nsw, ise, isp, ips, ipc, iwe, rad, nplsw, nseg,
             nsmax, nwmax, ienv);
  npls = nplsw;
  std::cout << "\n Inspect file configwire.txt for a list of current pulses\n"
            << " associated with wires, and coordinates of their nodes\n"
            << std::endl;
}

void zmatrix(cuDoubleComplex* cz, float* x, float* y, float* z, int* ipc, int* ips, int* ise, float* rad, int npls,
             double ka, int nsmax, int ienv, float sgnx, float sgny, float sgnz, float sgnenv) {
  fill_to_host(cz, x, y, z, ipc, ips, ise, rad, npls, ka, nsmax, ienv, sgnx, sgny, sgnz, sgnenv);
}

void zmatrix_gpu(cuDoubleComplex* cz_h, float* x_h, float* y_h, float* z_h, float* rad_h, int* ipc_h, int* ips_h,
                 int* ise_h, int nsmax, double ka, int npls, int ienv, float sgnx, float sgny, float sgnz,
                 float sgnenv) {
  fill_to_host(cz_h, x_h, y_h, z_h, ipc_h, ips_h, ise_h, rad_h, npls, ka, nsmax, ienv, sgnx, sgny, sgnz, sgnenv);
}
