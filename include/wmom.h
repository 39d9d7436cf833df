/*
 * wmom.h -- C ABI of the GB300 thin-wire Method-of-Moments fill-and-solve library
 * (libwmom.so).  Plain pointers and sizes only; every call returns a wmom_status
 * and nothing throws across this boundary.
 *
 * Reference interfaces each entry point replaces (paths inside the reference
 * project; REF = "wersja referencyjna", GPU = "wersja gpu"):
 *
 *   wmom_topology_from_geo   geoinp() + config()/configwire()
 *                            REF/Configuration.h:10-19, REF/Configuration.cpp:5-520
 *   wmom_ka                  wave number from a float MHz frequency, REF/Wire_MoM.cu:338-340
 *   wmom_plan_create/destroy the per-call cudaMalloc + H2D geometry upload of
 *                            zmatrix_gpu(), REF/Wire_MoM.cu:4075-4107 (done once here)
 *   wmom_fill                zmatrix() REF/Zmatrix.h:7-9 and zmatrix_gpu()
 *                            REF/Wire_MoM.h:49-51, into device memory, many
 *                            frequencies per call
 *   wmom_fill_geometries     the same for several geometries of uneven size, one
 *                            frequency each, in one launch
 *   wmom_zgetrf / wmom_zgetrs
 *                            LAPACKE_zgetrf / LAPACKE_zgetrs, REF/Wire_MoM.cu:372,382
 *                            (and cublasZgetrfBatched / cublasZgetrsBatched,
 *                            GPU/Wire_MoM.cu:468,477), on device buffers
 *   wmom_zgesv_like          the LAPACKE_zgetrf + LAPACKE_zgetrs pair on host buffers,
 *                            REF/Wire_MoM.cu:364-389
 *   wmom_excitation          delta-gap excitation vector, REF/Wire_MoM.cu:301-309
 *   wmom_solve_sweep         the per-frequency loop body of main()/CalculateByFreq(),
 *                            REF/Wire_MoM.cu:335-400, GPU/Wire_MoM.cu:331-413,
 *                            batched over frequencies on one GPU
 *
 * Conventions.  Complex numbers are interleaved (re, im) doubles (the layout of
 * cuDoubleComplex / MKL_Complex16).  Matrices are column-major, Z[m + n*ld] with
 * m the observation (test) function and n the source function, as the reference
 * stores them.  Index arrays use the reference's layout: 0-based storage holding
 * 1-based numbers, second columns at offset nsmax.  `stream` arguments are
 * cudaStream_t values passed as void* (NULL = the legacy default stream).
 */
#ifndef WMOM_H
#define WMOM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum wmom_status {
  WMOM_OK = 0,
  WMOM_ERR_ARG = 1,           /* invalid argument: null pointer, size or mode out of range */
  WMOM_ERR_CUDA = 2,          /* a CUDA runtime/driver call failed */
  WMOM_ERR_SINGULAR = 3,      /* exactly zero pivot (LAPACK info > 0) */
  WMOM_ERR_TIMEOUT = 4,       /* a bounded device-side wait gave up */
  WMOM_ERR_NOMEM = 5,         /* device allocation failed or the HBM budget is exceeded */
  WMOM_ERR_NOT_CONVERGED = 6, /* iterative refinement missed its tolerance */
  WMOM_ERR_GEOMETRY = 7,      /* bad .geo input or a topology limit exceeded */
  WMOM_ERR_UNSUPPORTED = 8    /* no device of the required architecture */
} wmom_status;

/* Topology arrays as configwire() leaves them (Configuration.cpp:485-514).  The
 * caller owns every array: x, y, z, rad, ipc hold nsmax entries; ips, ise, isp,
 * iwe hold 2*nsmax. */
typedef struct wmom_topology {
  int nsmax;
  int npnt, npls, nseg, nw; /* out: points, basis functions (unknowns), segments, wires */
  float *x, *y, *z, *rad;
  int *ipc, *ips, *ise, *isp, *iwe;
} wmom_topology;

/* Parses the text of a .geo file and builds the topology.  ienv 1 = free space,
 * 2 = PEC ground at z = 0 (image wires).  `listing` (optional) receives the text
 * the reference writes to configwire.txt; errbuf (optional) a message. */
wmom_status wmom_topology_from_geo(const char* geo_text, int ienv, int nsmax, int nwmax,
                                   wmom_topology* topo, char* listing, size_t listing_cap,
                                   char* errbuf, size_t errcap);

/* k = 2*pi / (c / f * 1e-6) with f in MHz as a float and c = 2.99792448e8. */
double wmom_ka(float freq_mhz);

/* ---------------------------------------------------------------- plans ---- */
/* A plan holds one geometry resident on the current CUDA device: per-basis source
 * and observation tables derived once (in FP64, from the float geometry) and
 * uploaded once.  Plans are independent; distinct plans may be used from
 * different host threads. */
typedef struct wmom_plan_s* wmom_plan;

wmom_status wmom_plan_create(const float* x, const float* y, const float* z, const float* rad,
                             const int* ipc, const int* ips, const int* ise, int nsmax, int npls,
                             int ienv, float sgnx, float sgny, float sgnz, float sgnenv,
                             wmom_plan* out);
wmom_status wmom_plan_destroy(wmom_plan plan);
int wmom_plan_npls(wmom_plan plan);
/* Bytes of per-geometry tables the plan uploaded to the device. */
long long wmom_plan_upload_bytes(wmom_plan plan);
/* 1 when the plan fills with the pair-tiled kernel (free space), 2 when it does and
 * also fills a batch of frequencies with one CTA per tile for all of them, 0 when
 * it fills with the per-entry kernel (PEC ground image terms).  WMOM_FILL_ENTRY=1 in
 * the environment forces the per-entry kernel, WMOM_FILL_SINGLE=1 one CTA per tile
 * and frequency. */
int wmom_plan_fill_variant(wmom_plan plan);
/* Distinct (observation point, source half-segment) pairs the pair-tiled fill
 * evaluates per frequency (each with a 2-point rule), 0 for the per-entry kernel.
 * Divided by npls^2 it is the pairs per entry; the reference evaluates 4. */
long long wmom_plan_fill_pairs(wmom_plan plan);
/* Independent closed current paths of the plan's structure: the cycle rank of the
 * graph of its segments and nodes, with every node on a PEC ground plane taken as one
 * (a current returns through the plane); -1 for a null plan.  Structures with loops
 * are the ones whose conditioning grows as 1/(ka)^2 towards low frequencies (the
 * precision form's second-tier prediction keys on it).  No reference counterpart. */
int wmom_plan_loops(wmom_plan plan);

/* Fills nk impedance matrices, one per wave number ka[i] (host array), in FP64.
 * Matrix i starts at z_dev + i*zstride complex elements; ldz >= npls.  The
 * j*eta0/(4*pi*k) scale of zmatrix() is included. */
wmom_status wmom_fill(wmom_plan plan, const double* ka, int nk, void* z_dev, long long ldz,
                      long long zstride, void* stream);

/* Fills the impedance matrices of `count` geometries of any sizes, one wave number
 * each (host arrays plans[i], ka[i], z_dev[i], ldz[i] >= npls of plans[i]), in one
 * kernel launch for all free-space geometries (ground-plane geometries are filled by
 * their own launch).  Each matrix equals wmom_fill's for the same plan and ka, bit
 * for bit.  The reference fills one geometry per process run (zmatrix_gpu,
 * REF/Wire_MoM.h:49-51); this is its batched form for sets of uneven geometries.
 * Synchronises `stream`. */
wmom_status wmom_fill_geometries(const wmom_plan* plans, int count, const double* ka, void* const* z_dev,
                                 const long long* ldz, void* stream);

/* ------------------------------------------------------------ FP64 LU ---- */
/* In-place LU with partial pivoting of an n x n complex128 device matrix
 * (LAPACK zgetrf semantics: pivot = first row of largest |re|+|im|, ipiv 1-based,
 * L unit lower, U upper).  ipiv_dev: n ints on the device.  *info receives the
 * LAPACK info (0, or the 1-based column of the first exactly-zero pivot, which
 * also returns WMOM_ERR_SINGULAR).  Synchronises `stream`. */
wmom_status wmom_zgetrf(int n, void* a_dev, long long lda, int* ipiv_dev, int* info, void* stream);

/* The same factorisation of an n x n complex64 device matrix, as the precision form
 * runs it: FP32 panels and triangular solves, trailing updates on the tensor cores
 * (3xTF32) where the device has them.  LAPACK cgetrf semantics and results to FP32
 * rounding.  No reference counterpart (the reference factors in FP64 only). */
wmom_status wmom_cgetrf(int n, void* a_dev, long long lda, int* ipiv_dev, int* info, void* stream);

/* Solves A x = b with the factors from wmom_zgetrf for nrhs right-hand sides held
 * column-major in b_dev (ldb >= n); b_dev is overwritten with x. */
wmom_status wmom_zgetrs(int n, int nrhs, const void* a_dev, long long lda, const int* ipiv_dev,
                        void* b_dev, long long ldb, void* stream);

/* FP64 LU that allocates no device memory.  No counterpart in the reference (which
 * allocates per call): for callers that cannot call cudaMalloc -- applications that
 * hand the library device buffers from their own pool and forbid other allocations,
 * or serving processes that must not pay cudaMalloc's device-wide synchronisation
 * once running.  Same arguments and results as wmom_zgetrf; the factorisation's
 * scratch lives in a fixed 576 KiB __device__ array inside the library, held by every
 * GPU that loads the library until exit.  n above WMOM_NOALLOC_MAX_N returns
 * WMOM_ERR_ARG.  Each call looks up the array's device address on the current
 * device (cudaGetSymbolAddress, which allocates nothing), so calls stay valid after
 * a cudaDeviceReset.  The call synchronises `stream` to read the pivot status.  All
 * calls share the array: calls whose work overlaps on the GPU race and must be
 * serialised by the caller. */
#define WMOM_NOALLOC_MAX_N 20480
wmom_status wmom_zgetrf_noalloc(int n, void* a_dev, long long lda, int* ipiv_dev, int* info,
                                void* stream);

/* 1-norm of an n x n complex128 device matrix, max_j sum_i |a_ij| (LAPACK zlange
 * with norm '1'; the moduli are summed in FP32, so the norm is good to about 1e-7,
 * enough for a condition estimate).  Synchronises `stream`.  No reference
 * counterpart (the reference estimates no condition number). */
wmom_status wmom_zlange1(int n, const void* a_dev, long long lda, double* anorm, void* stream);

/* LAPACK zgecon with norm '1' on device factors from wmom_zgetrf: *rcond = 1 /
 * (anorm * est), est an estimate of ||A^-1||_1 by Higham's method (LAPACK zlacn2:
 * solves with A and A^H, at most 5 of each plus one), anorm = ||A||_1 of the matrix
 * before factoring (wmom_zlange1).  *rcond = 0 for anorm = 0.  Synchronises
 * `stream`.  No reference counterpart (the reference only checks zgetrf's info,
 * REF/Wire_MoM.cu:372-377). */
wmom_status wmom_zgecon(int n, const void* a_dev, long long lda, const int* ipiv_dev, double anorm,
                        double* rcond, void* stream);

/* Host-buffer drop-in for LAPACKE_zgetrf + LAPACKE_zgetrs with one right-hand
 * side: z (n*n, overwritten by the factors), v (n), i_out (n), ipiv (n, 1-based). */
wmom_status wmom_zgesv_like(int n, double* z, const double* v, double* i_out, int* ipiv,
                            int* info);

/* The precision form's trailing update on the tensor cores: C -= A * B for complex
 * FP32 (float2) column-major device matrices, C m x n, A m x k, B k x n, computed
 * as 3xTF32 tcgen05 products with FP32 accumulation.  No reference counterpart
 * (the reference never factors in reduced precision); exposed for testing. */
wmom_status wmom_cgemm_sub_tc(int m, int n, int k, const void* a_dev, long long lda, const void* b_dev,
                              long long ldb, void* c_dev, long long ldc, void* stream);

/* The precision form's second-tier trailing update: C -= A * B for complex FP64
 * (double2) column-major device matrices, C m x n, A m x k, B k x n, to FP64-grade
 * accuracy on the bf16 tensor cores.  Each row of A and column of B is split into
 * six 8-bit digit planes under a power-of-two scale (an error-free transformation);
 * digit products of the same weight are summed exactly in FP32 accumulators and
 * the weights are recombined in FP64.  Normwise error about 2^-45 relative to
 * k * max|A| * max|B|.  No reference counterpart; exposed for testing. */
wmom_status wmom_zgemm_sub_emul(int m, int n, int k, const void* a_dev, long long lda, const void* b_dev,
                                long long ldb, void* c_dev, long long ldc, void* stream);

/* The plain FP64 form's trailing update: C -= A * B for complex FP64 (double2)
 * column-major device matrices, C m x n, A m x k, B k x n.  variant 0: SIMT DFMA (the
 * update the plain form uses by default); variant 1: DMMA, warp-level
 * mma.m8n8k4.f64 on the FP64 tensor pipe (selected inside the LU by
 * WMOM_FP64_UPDATE=dmma).  Synchronises `stream`.  No reference counterpart (the
 * reference factors with MKL / cuBLAS); exposed for testing and timing. */
wmom_status wmom_zgemm_sub_fp64(int m, int n, int k, const void* a_dev, long long lda, const void* b_dev,
                                long long ldb, void* c_dev, long long ldc, int variant, void* stream);

/* ----------------------------------------------------------- solver ---- */
typedef enum wmom_mode {
  WMOM_MODE_FP64 = 0, /* plain form: FP64 fill, FP64 LU, FP64 solves */
  WMOM_MODE_MIXED = 1 /* precision form: FP64 fill, complex-FP32 tensor-core LU, FP64
                         iterative refinement, FP64 LU fallback when refinement stalls */
} wmom_mode;

/* OR'd into the mode of wmom_solve_sweep or wmom_factor: every result also carries
 * an estimate of the 1-norm condition number of its matrix (wmom_report.cond1),
 * ||Z||_1 times LAPACK zlacn2's estimate of ||Z^-1||_1 from the factors behind the
 * result (the FP32 factors for tier 1, the FP64-grade ones for tiers 2 and 3).  It
 * costs up to eleven more triangular-solve pairs per matrix. */
#define WMOM_SOLVE_CONDEST 0x100

/* Per-frequency result record. */
typedef struct wmom_report {
  double rel_residual;  /* ||V - Z I||_2 / ||V||_2 of the returned currents (FP64) */
  int iterations;       /* refinement steps taken (0 for WMOM_MODE_FP64) */
  int fell_back;        /* 1 if the FP32 factors were left for FP64-grade ones (tier 2 or 3) */
  int info;             /* LAPACK-style info of the factorisation that produced I */
  int status;           /* wmom_status of this frequency */
  int krylov_steps;     /* GMRES steps of the Krylov refinement (0 when plain refinement
                           converged or for WMOM_MODE_FP64) */
  int tier;             /* factors behind I: 1 FP32 tensor-core LU + FP64 refinement,
                           2 FP64 LU with tensor-core (digit-plane) trailing updates +
                           FP64 refinement, 3 plain FP64 LU; 0 for WMOM_MODE_FP64 */
  double cond1;         /* estimated 1-norm condition number of Z with WMOM_SOLVE_CONDEST,
                           else 0 */
} wmom_report;

/* Lumped series loads for the sweeps of this plan: Z[k-1, k-1] += r_ohm + j*2*pi*f*l_uh
 * with f in MHz (the reference's addloads block, REF/Wire_MoM.cu:346-363, where the
 * indices were hard-wired to one geometry).  idx is 1-based; nloads = 0 clears. */
wmom_status wmom_plan_set_loads(wmom_plan plan, int nloads, const int* idx, const double* r_ohm,
                                const double* l_uh);

/* Delta-gap excitation: V = 0 except V[ngap-1] = ampl*(cos + j sin)(pi*phas/180). */
wmom_status wmom_excitation(int npls, int ngap, float ampl, float phas_deg, double* v);

/* Fills, factors and solves one (geometry, frequency) system per frequency, all
 * frequencies batched on the device.  currents: nfreq*npls complex (host, may be
 * NULL); zin: nfreq complex input impedances V[ngap-1]/I[ngap-1] (host, may be
 * NULL); reports: nfreq records (may be NULL).  tol is the relative residual the
 * mixed mode refines to (<= 0 selects 1e-12). */
wmom_status wmom_solve_sweep(wmom_plan plan, const float* freq_mhz, int nfreq, int ngap,
                             float ampl, float phas_deg, int mode, double tol, double* currents,
                             double* zin, wmom_report* reports, void* stream);

/* --------------------------------------------------- resident factors ---- */
/* Fills and factors one plan's matrices for nfreq frequencies and keeps Z (FP64) and
 * its factors resident on the device, so that new excitations of the same (geometry,
 * frequency) -- another gap, amplitude or phase -- only run the solves.  The
 * reference refills and refactors for every run (REF/Wire_MoM.cu:335-400).  Device
 * memory: nfreq * (16 + 8) * npls^2 bytes (mixed) or nfreq * 32 * npls^2 (FP64). */
typedef struct wmom_factors_s* wmom_factors;

wmom_status wmom_factor(wmom_plan plan, const float* freq_mhz, int nfreq, int mode, wmom_factors* out,
                        void* stream);
/* Solves frequencies [first, first+count) of the set for one excitation; the result
 * arrays are indexed from 0 (= frequency `first`). */
wmom_status wmom_factors_solve(wmom_factors f, int first, int count, int ngap, float ampl, float phas_deg,
                               double tol, double* currents, double* zin, wmom_report* reports, void* stream);
long long wmom_factors_device_bytes(wmom_factors f);
wmom_status wmom_factors_destroy(wmom_factors f);

/* Factor sets for `count` (geometry, frequency) pairs of uneven orders -- plans[i] at
 * freq_mhz[i], the same plan may appear several times -- filled and factored in
 * batched launches instead of one factorisation each.  Each pair's matrix is stored
 * at the padded order of its size class, wmom_padded_order(npls) (four classes per
 * octave, at most 1.25 npls), with an identity block beyond npls; pairs of one class
 * are filled by one ragged launch and factored by one batched launch sequence.  The
 * leading block of the factors, and so every solution, is the geometry's own, and
 * does not depend on the other pairs of the call: a pair's results are the same
 * alone and in any batch, bit for bit.  out[i] receives a one-frequency factor set
 * used like wmom_factor's (wmom_factors_solve returns npls entries per frequency;
 * destroy each set; the sets of a class share one allocation, freed with the last).
 * mode may include WMOM_SOLVE_CONDEST.  The reference solves one geometry per run
 * and factors with a batch of one (cublasZgetrfBatched, GPU/Wire_MoM.cu:468). */
wmom_status wmom_factor_geometries(const wmom_plan* plans, int count, const float* freq_mhz, int mode,
                                   wmom_factors* out, void* stream);
/* The padded order of an npls-unknown geometry in wmom_factor_geometries. */
int wmom_padded_order(int npls);

/* Human-readable name of a status code. */
const char* wmom_status_string(wmom_status s);

/* The CUDA call that last failed on the calling thread and CUDA's message for it
 * ("" if none); valid until that thread's next failing call.  No reference
 * counterpart (the reference printed CUDA errors and exited). */
const char* wmom_last_error(void);

/* ------------------------------------------------------- instrumentation ---- */
/* Launch counters per kernel class are always kept.  With timing enabled every
 * launch is also bracketed by CUDA events on its own stream.  Classes, in order:
 * 0 fill, 1 panel, 2 tensor-core GEMM, 3 SIMT GEMM, 4 triangular solves,
 * 5 row interchanges, 6 FP64 residual, 7 other, 8 FP64-grade tensor-core GEMM
 * (the precision form's second tier), 9 single-right-hand-side triangular solves
 * (solutions and refinement).  wmom_stats_read fills up to n
 * entries of each array (any may be NULL) and returns the number of classes;
 * ms = summed device time, launches = launches issued, timed = launches timed,
 * work = algorithmic flops (bytes for the residual) of the timed launches.  The
 * reference's equivalent is its Timer / "GPU time.dat" (REF/Wire_MoM.cu:8-26,
 * 4085-4175). */
void wmom_stats_enable(int on);
void wmom_stats_reset(void);
int wmom_stats_read(double* ms, long long* launches, long long* timed, double* work, int n);

/* Measures this device's FP64 throughput (TFLOP/s, 2 flop per FMA): the best of
 * short bounded kernels of independent FMA chains and of the plain form's FP64
 * complex GEMM on a compute-bound shape (4096 x 4096 x 256).  It is the denominator
 * of the FP64-bound rooflines (fill, panel, SIMT GEMM).  No reference counterpart. */
wmom_status wmom_probe_fp64_tflops(double* tflops);

/* Diagnostic: for n device doubles x[i] writes d_out[4i..4i+3] = the fill's
 * table-driven (sin, cos)(x[i]) followed by CUDA's sincos() of the same argument,
 * so that tests can bound the difference.  Synchronises `stream`.  No reference
 * counterpart. */
wmom_status wmom_diag_sincos(const double* d_x, long long n, double* d_out, void* stream);

/* The factorisation shape the autotuner chose for order n in `mode` in this process
 * (matrices per batched launch, panels per tensor-core trailing update); returns
 * WMOM_ERR_ARG when no sweep of that order has been tuned yet.  No reference
 * counterpart. */
wmom_status wmom_tuned_config(int n, int mode, int* batch, int* span);
/* The rest of that shape: FP32 columns of the precision form's tensor-core update tile
 * (256 or 128) and its widest FP32 panel (0 = as wide as shared memory allows, else
 * 48 or 32 columns); WMOM_ERR_ARG when order n has not been tuned.  No reference
 * counterpart (the reference's kernels use a fixed BLOCK_SIZE, REF/Wire_MoM.h:21). */
wmom_status wmom_tuned_shape(int n, int mode, int* tile_n, int* panel_w);

/* ---------------------------------------------------------------- testing ---- */
/* Test hook, not for production use: every grid barrier of the plain FP64 LU's
 * cooperative panel kernels waits for `count` arrivals more than its blocks send,
 * so that its bounded wait (2 s) runs out; the factorisation then returns
 * WMOM_ERR_TIMEOUT without a device fault and the next call with count = 0 works.
 * No reference counterpart. */
void wmom_debug_panel_missing_arrivals(int count);

#ifdef __cplusplus
}
#endif

#endif /* WMOM_H */
