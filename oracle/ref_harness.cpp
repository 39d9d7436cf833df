// ref_harness.cpp -- C entry points around the reference's own CPU code.
//
// TEST INFRASTRUCTURE ONLY.  oracle/build.py compiles this file together with the
// UNMODIFIED reference sources "wersja referencyjna/{Configuration,Zmatrix,Complex}.cpp",
// read in place from the reference checkout, into oracle/_ref/libwmomref.so.  Nothing
// of the reference is copied into this repository; this file only declares extern "C"
// wrappers so that Python tests can call:
//   * geoinp() + config()  (Configuration.cpp:5-108) on a directory that holds a
//     dipol.geo file (geoinp opens that fixed name in the working directory and
//     configwire writes configwire.txt there);
//   * zmatrix()            (Zmatrix.cpp:27-52), the reference's CPU fill.
// The library only exists where the reference sources are present; the GPU machine runs
// the oracle port (oracle/wmom_oracle.c) instead.
#include <unistd.h>

#include <cstring>
#include <iostream>
#include <sstream>

#include "Configuration.h"
#include "Zmatrix.h"

// Array capacities of the reference driver (Wire_MoM.cu:43-44).
static const int kNnmax = 3000, kNtmax = 5000, kNwmax = 10000, kNpwmax = 20480;
static const int kNsmax = kNwmax + kNpwmax;

extern "C" int ref_nsmax() { return kNsmax; }

// Runs geoinp + config in `dir` and copies the topology arrays out.  Every output
// array holds kNsmax (x, y, z, rad, ipc) or 2*kNsmax (ips, ise, isp, iwe) entries.
// counts[0..2] = npnt, npls, nseg.  stdout chatter of the reference is discarded.
// The working arrays handed to config() carry one spare element each: its final
// 1-based -> 0-based shift (Configuration.cpp:499-514) reads one element past nsmax.
extern "C" int ref_load_geometry(const char* dir, int ienv, int* counts, float* x, float* y,
                                 float* z, float* rad, int* ipc, int* ips, int* ise, int* isp,
                                 int* iwe) {
  char cwd[4096];
  if (!getcwd(cwd, sizeof(cwd))) return -1;
  if (chdir(dir) != 0) return -2;
  std::stringstream sink;
  std::streambuf* old = std::cout.rdbuf(sink.rdbuf());

  float* xnod = new float[kNnmax]();
  float* ynod = new float[kNnmax]();
  float* znod = new float[kNnmax]();
  int* iwn = new int[2 * kNwmax]();
  float* wrad = new float[kNwmax]();
  int* nsw = new int[kNwmax]();
  int* iwt = new int[3 * kNtmax]();
  int nnod = 0, nw = 0, nt = 0, npnt = 0, npls = 0, nplsw = 0, nseg = 0;
  geoinp(kNnmax, kNwmax, kNtmax, nnod, xnod, ynod, znod, nw, iwn, wrad, nsw, nt, iwt);

  float* wx = new float[kNsmax + 1]();
  float* wy = new float[kNsmax + 1]();
  float* wz = new float[kNsmax + 1]();
  float* wrd = new float[kNsmax + 1]();
  int* wipc = new int[kNsmax + 1]();
  int* wips = new int[2 * kNsmax + 1]();
  int* wise = new int[2 * kNsmax + 1]();
  int* wisp = new int[2 * kNsmax + 1]();
  int* wiwe = new int[2 * kNsmax + 1]();
  config(npnt, nnod, xnod, ynod, znod, wx, wy, wz, nw, iwn, wrad, nsw, wise, wisp, wips, wipc, wiwe,
         wrd, npls, nplsw, nseg, kNsmax, kNwmax, ienv);
  std::memcpy(x, wx, sizeof(float) * kNsmax);
  std::memcpy(y, wy, sizeof(float) * kNsmax);
  std::memcpy(z, wz, sizeof(float) * kNsmax);
  std::memcpy(rad, wrd, sizeof(float) * kNsmax);
  std::memcpy(ipc, wipc, sizeof(int) * kNsmax);
  std::memcpy(ips, wips, sizeof(int) * 2 * kNsmax);
  std::memcpy(ise, wise, sizeof(int) * 2 * kNsmax);
  std::memcpy(isp, wisp, sizeof(int) * 2 * kNsmax);
  std::memcpy(iwe, wiwe, sizeof(int) * 2 * kNsmax);
  delete[] wx;
  delete[] wy;
  delete[] wz;
  delete[] wrd;
  delete[] wipc;
  delete[] wips;
  delete[] wise;
  delete[] wisp;
  delete[] wiwe;
  counts[0] = npnt;
  counts[1] = npls;
  counts[2] = nseg;

  delete[] xnod;
  delete[] ynod;
  delete[] znod;
  delete[] iwn;
  delete[] wrad;
  delete[] nsw;
  delete[] iwt;
  std::cout.rdbuf(old);
  if (chdir(cwd) != 0) return -3;
  return 0;
}

// The reference fill itself; cz receives npls*npls complex128 values, column-major.
extern "C" void ref_zmatrix(double* cz, float* x, float* y, float* z, int* ipc, int* ips, int* ise,
                            float* rad, int npls, double ka, int nsmax, int ienv, float sgnx,
                            float sgny, float sgnz, float sgnenv) {
  std::stringstream sink;
  std::streambuf* old = std::cout.rdbuf(sink.rdbuf());
  zmatrix(reinterpret_cast<clDoubleComplex*>(cz), x, y, z, ipc, ips, ise, rad, npls, ka, nsmax,
          ienv, sgnx, sgny, sgnz, sgnenv);
  std::cout.rdbuf(old);
}
