// wmom_dropin.h -- C++ symbols with the reference's own signatures, exported by
// libwmom.so so that the reference's unmodified driver (its main() in
// "wersja referencyjna/Wire_MoM.cu") links against this library instead of its
// CPU/GPU fill and geometry code.  Same names, argument meaning, array layouts
// and side files (reads dipol.geo, writes configwire.txt) as the originals.
#ifndef WMOM_DROPIN_H
#define WMOM_DROPIN_H

#include <cuComplex.h>

// REF/Configuration.h:10-11 (Configuration.cpp:5-75): reads "dipol.geo" from the
// working directory into 1-based arrays; on an over-limit file prints the message
// and exits, as the reference does.
void geoinp(int nnmax, int nwmax, int ntmax, int& nnod, float* xnod, float* ynod, float* znod, int& nw,
            int* iwn, float* wrad, int* nsw, int& nt, int* iwt);

// REF/Configuration.h:13-15 (Configuration.cpp:78-108).
void config(int& npnt, int nnod, float* xnod, float* ynod, float* znod, float* x, float* y, float* z, int nw,
            int* iwn, float* wrad, int* nsw, int* ise, int* isp, int* ips, int* ipc, int* iwe, float* rad,
            int& npls, int& nplsw, int& nseg, int nsmax, int nwmax, int ienv);

// REF/Configuration.h:17-19 (Configuration.cpp:112-520): topology + configwire.txt,
// then the 1-based -> 0-based shift of every array.
void configwire(int& npnt, int nnod, float* xnod, float* ynod, float* znod, float* x, float* y, float* z,
                int nw, int* iwn, float* wrad, int* nsw, int* ise, int* isp, int* ips, int* ipc, int* iwe,
                float* rad, int& nplsw, int& nseg, int nsmax, int nwmax, int ienv);

// REF/Zmatrix.h:7-9 (Zmatrix.cpp:27-52): fills the host matrix cz (npls x npls,
// column-major, j*eta0/(4*pi*k) scale included) -- computed on the GPU.
void zmatrix(cuDoubleComplex* cz, float* x, float* y, float* z, int* ipc, int* ips, int* ise, float* rad,
             int npls, double ka, int nsmax, int ienv, float sgnx, float sgny, float sgnz, float sgnenv);

// REF/Wire_MoM.h:49-51 (Wire_MoM.cu:4052-4197): the same fill, the reference's
// GPU entry point (host in, host out).
void zmatrix_gpu(cuDoubleComplex* cz_h, float* x_h, float* y_h, float* z_h, float* rad_h, int* ipc_h,
                 int* ips_h, int* ise_h, int nsmax, double ka, int npls, int ienv, float sgnx, float sgny,
                 float sgnz, float sgnenv);

#endif  // WMOM_DROPIN_H
