// wmom_internal.h -- shared declarations of libwmom's translation units.
#pragma once

#include <cstdint>
#include <istream>
#include <string>
#include <vector>

#include "../../include/wmom.h"

#if defined(__CUDACC__) || defined(WMOM_WITH_CUDA_RUNTIME)
#include <cuda_runtime.h>
#endif

namespace wmom {

// ---------------------------------------------------------------- geometry ----
struct GeoInput {
  int nnod = 0, nw = 0, nt = 0;
  std::vector<float> xnod, ynod, znod;  // 1-based, nnod+1
  std::vector<int> iwn;                 // 1-based: [1..nw] first node, [nw+1..2nw] second
  std::vector<float> wrad;              // 1-based
  std::vector<int> nsw;                 // 1-based segment counts
  std::vector<int> iwt;                 // patch triplets (read and ignored, as the reference)
};

struct Topology {
  int npnt = 0, npls = 0, nseg = 0;
  float *x, *y, *z, *rad;
  int *ipc, *ips, *ise, *isp, *iwe;
};

int geo_parse(std::istream& in, int nnmax, int nwmax, int ntmax, GeoInput* g, std::string* err);
int build_topology(const GeoInput& gin, int nsmax, int nwmax, int ienv, Topology* out,
                   std::string* listing, std::string* err);

// --------------------------------------------------------- fill tables ----
// Observation half of a test function m (h = 0: point on S_m+, h = 1: on S_m-).
// All values are the reference's double expressions of the float geometry
// (Zmatrix.cpp:69-84 and 154-165).
struct ObsHalf {
  double rm[3];  // observation point (segment midpoint)
  double lm[3];  // test vector: h=0 -> r_p - r_m, h=1 -> r_m - r_p
  int ml, mr;    // node numbers of the observation segment (self-term test)
  int on_ground; // both nodes at z < 1e-6 (image self-term test)
  int pad;
};

// Source half of a basis function n (s = 0: S_n+ with rising ramp s/dl from its
// first node to the centre, s = 1: S_n- with falling ramp from the centre).
// (Zmatrix.cpp:252-276 and 466-490.)
struct SrcHalf {
  double rs[3];  // start of the parametrisation
  double dc[3];  // unit vector
  double dl;     // length
  double an;     // wire radius
  double rs_img[3];  // mirrored start (PEC ground image), rs * sgn
  double dc_img[3];  // mirrored unit vector
  int nl, nr;        // node numbers of the source segment
};

// Unique observation point of the pair-tiled fill: the midpoint of one observation
// segment and u = r_hi - r_m (r_hi = the segment node with the larger number);
// every test half-vector l_m of the reference is exactly +u or -u.
struct ObsInst {
  double rm[3];
  double u[3];
  int ml, mr, on_ground, pad;
};

// Unique source half-segment (start node, end node, segment): start, unit vector,
// length, radius, the two Gauss abscissae and both ramps evaluated at them.
struct SrcInst {
  double rs[3];
  double dc[3];
  double dl, an;
  double an2, half;  // an * an and dl * 0.5, as the per-entry kernel computes them
  double s[2];
  double w_up[2];  // s / dl        (rising ramp of S_n+)
  double w_dn[2];  // (dl - s) / dl (falling ramp of S_n-)
  int nl, nr;
};

// Basis-function tiles of the pair-tiled fill: for each tile of kPairTile test
// (source) functions, the list of distinct observation (source) instances its
// halves use, and for every half its index in that list.
constexpr int kPairTile = 32;
struct PairTiles {
  bool ok = false;
  int tile = kPairTile;
  int n_tiles = 0;
  int max_o = 0, max_q = 0;
  std::vector<ObsInst> obs;
  std::vector<SrcInst> src;
  std::vector<int> rt_off, rt_ids, ct_off, ct_ids;
  std::vector<int> row_local;  // 2*npls: local obs index, bit 30 set when l_m = -u
  std::vector<int> col_local;  // 2*npls: local source index
};

// ------------------------------------------------------------------ plan ----
struct Plan {
  int device = 0;
  int npls = 0, nsmax = 0, ienv = 1;
  float sgnx = 1.f, sgny = 1.f, sgnz = 1.f, sgnenv = 1.f;
  std::vector<ObsHalf> h_obs;  // 2*npls
  std::vector<SrcHalf> h_src;  // 2*npls
  ObsHalf* d_obs = nullptr;
  SrcHalf* d_src = nullptr;
  // pair-tiled fill (free space)
  PairTiles pt;
  ObsInst* d_oi = nullptr;
  SrcInst* d_si = nullptr;
  int* d_tiles = nullptr;  // rt_off | rt_ids | ct_off | ct_ids | row_local | col_local
  int off_rt_ids = 0, off_ct_off = 0, off_ct_ids = 0, off_row_local = 0, off_col_local = 0;
  // lumped series loads R + j*2*pi*f[MHz]*L[uH] on diagonal entries (1-based index)
  std::vector<int> load_idx;
  std::vector<double> load_r, load_l_uh;
  int loops = 0;  // independent closed current paths (wire_loops)
};

int wire_loops(const std::vector<SrcHalf>& src, int nsmax, const float* z, bool ground);

int plan_build_tables(Plan* p, const float* x, const float* y, const float* z, const float* rad,
                      const int* ipc, const int* ips, const int* ise);
void plan_build_pair_tiles(Plan* p, const float* x, const float* y, const float* z, const float* rad,
                           const int* ipc, const int* ips, const int* ise);

double ka_from_mhz(float f);

// Per-frequency constants of the fill kernels (host-built, read on the device): k,
// k^2, cq = eta0 / (4 pi k), and the two products the pair values carry so that
// assembling an entry needs additions only: kc = k^2 cq (vector-potential terms) and
// hc = cq / 2 (scalar-potential terms).
struct FreqParams {
  double ka, ka2, cq, kc, hc;
};
FreqParams freq_params(double ka);

}  // namespace wmom

#if defined(__CUDACC__) || defined(WMOM_WITH_CUDA_RUNTIME)
namespace wmom {
// Fill launcher (fill.cu).
cudaError_t launch_fill(const Plan& p, const double* d_ka, int nk, double2* z, long long ldz,
                        long long zstride, cudaStream_t stream);
// Fills count matrices of as many geometries, one wave number each, z[i] with
// leading dimension ldz[i]: every pair-tiled geometry in one launch, the others
// (ground plane) by the per-entry kernel.
cudaError_t launch_fill_geometries(const Plan* const* plans, const double* ka, double2* const* z,
                                   const long long* ldz, int count, cudaStream_t stream);
// True when batches of frequencies are filled with one CTA per tile for all of them.
bool fill_multi_fits(const Plan& p);
// Lets `func` launch with up to `bytes` of dynamic shared memory.  The cap is process-
// wide state of the kernel, so it is only ever raised (to the device's opt-in maximum,
// once per device and kernel): setting it per launch would race with another host
// thread that launches the same kernel with more shared memory.
cudaError_t allow_dynamic_smem(const void* func, size_t bytes);
}  // namespace wmom

#define WMOM_CUDA_TRY(call)                                   \
  do {                                                        \
    cudaError_t _e = (call);                                  \
    if (_e != cudaSuccess) return wmom_fail_cuda(_e, #call);  \
  } while (0)

wmom_status wmom_fail_cuda(cudaError_t e, const char* what);
#endif
