/*
 * chflow.h -- C ABI of the GB300 channel-flow time step.
 *
 * Drop-in for the per-step call sequence of poiseuilleflow.f90: the Fortran
 * main loop calls getnonlinear (poiseuilleflow.f90:224) and then the inline
 * per-mode solve (poiseuilleflow.f90:242-394) and the (0,0)-mode solve
 * (poiseuilleflow.f90:401-474).  A driver keeps its module arrays
 * (paraandcons.f90:28-38) on the host and hands them to this library once;
 * the library keeps them resident in device memory, advances them with
 * hand-written sm_103a kernels and hands them back at output/restart steps.
 *
 * Array conventions (identical to the reference, one rank, nproc = 1):
 *   field arrays  real*8 (0:nx,0:ny,0:nz), nx = nnx-1, ny = nny-1, nz = nnz,
 *                 column-major; even x index = real part and odd x index =
 *                 imaginary part of streamwise mode x/2 (poiseuilleflow.f90:8-12);
 *                 Chebyshev coefficients in z for vnp1, omegaynp1, unp1, wnp1,
 *                 omegaxnp1, omegaznp1 after a step; Gauss-Lobatto values for
 *                 the nonlinear histories rhsvn, rhsomegayn (and unp1, wnp1
 *                 between chf_getnonlinear and chf_solve).
 *   mean arrays   real*8 (2,0:nz): clamb1n, clamb1nm1, clamb3n, clamb3nm1,
 *                 au0, w0.
 *
 * Every entry point returns CHF_OK (0) or a negative CHF_E* status and never
 * exits or aborts; chf_last_error() describes the last failure.  A handle is
 * not re-entrant: calls on one handle must not overlap.  Different handles
 * are independent.
 */
#ifndef CHFLOW_H
#define CHFLOW_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CHF_OK 0
#define CHF_E_INVALID (-1)   /* bad argument or configuration */
#define CHF_E_CUDA (-2)      /* CUDA runtime error */
#define CHF_E_NOMEM (-3)     /* device or host allocation failed */
#define CHF_E_STATE (-4)     /* call out of order (e.g. step before upload) */
#define CHF_E_NUMERIC (-5)   /* non-finite values detected */

#define CHF_FP64 0           /* all arithmetic in FP64 */
#define CHF_MIXED 1          /* FP32 x/y transforms and products, exact tensor-core
                                z transforms, FP64 state; the per-mode solve as an
                                FP64 update c + delta whose increment delta is
                                formed by compensated FP32 arithmetic (about
                                2^-38 of its terms), A^-1 r in FP32; the (0,0)
                                mode and the operator factorisations in FP64 */
#define CHF_MIXED_F64SOLVE 2 /* the nonlinear term of CHF_MIXED with the FP64
                                tau solve of CHF_FP64 for every mode */

/* Runtime counterpart of the compile-time parameters of paraandcons.f90:4-25. */
typedef struct chf_config {
  int nnx;        /* streamwise points, paraandcons.f90:5  (multiple of 4) */
  int nny;        /* spanwise points, paraandcons.f90:6    (multiple of 4) */
  int nnz;        /* Chebyshev degree, paraandcons.f90:7   (even, 4..254:
                     the solve holds a column of nnz + 1 values in one warp) */
  double aphi;    /* streamwise box 2*pi*aphi, paraandcons.f90:22 */
  double beta;    /* spanwise box 2*pi*beta, paraandcons.f90:22   */
  double dt;      /* time step, paraandcons.f90:23 */
  double re;      /* Reynolds number (viscosity 1/re), paraandcons.f90:24 */
  double re_p;    /* mean pressure gradient, paraandcons.f90:25 */
  int precision;  /* CHF_FP64, CHF_MIXED or CHF_MIXED_F64SOLVE */
  int zpad;       /* wall-normal intervals of the product grid; 0 = 2*nnz as
                     in getlamb (poiseuilleflow.f90:1647-1648); any value with
                     2*zpad > 3*nnz gives the same (exact) products */
  int device;     /* CUDA device ordinal */
} chf_config;

typedef struct chf_handle chf_handle;

/* Diagnostics of the current state (spectral, Parseval). */
typedef struct chf_diag {
  double energy;        /* 0.5 * sum over the spectral arrays of u^2 + v^2 + w^2 (the sum
                           printed at poiseuilleflow.f90:2322-2336), spanwise Nyquist
                           slot excluded */
  double wall_shear_top;    /* d<u>/dz at z = +1 from au0 */
  double wall_shear_bottom; /* d<u>/dz at z = -1 from au0 */
  double max_abs;       /* max |value| over the six velocity/vorticity fields (no Nyquist slot) */
  int finite;           /* 1 if every value is finite */
} chf_diag;

/* Allocate device state and precompute the implicit operators.  Replaces the
 * set-up of poiseuilleflow.f90:77-214 (allocation, FFT plans, wavenumbers,
 * SCHEB and the zgetrf/zgetri explicit inverses). */
int chf_create(const chf_config* cfg, chf_handle** out);
int chf_destroy(chf_handle* h);

/* Last error message of h, or of the last failed chf_create when h is NULL. */
const char* chf_last_error(const chf_handle* h);

/* Copy the module arrays paraandcons.f90:28-38 host -> device.  Any pointer
 * may be NULL to leave that array unchanged. */
int chf_upload_state(chf_handle* h,
                     const double* vnp1, const double* omegaynp1,
                     const double* unp1, const double* wnp1,
                     const double* omegaxnp1, const double* omegaznp1,
                     const double* rhsvn, const double* rhsomegayn,
                     const double* clamb1n, const double* clamb1nm1,
                     const double* clamb3n, const double* clamb3nm1,
                     const double* au0, const double* w0);

/* Copy the module arrays device -> host (blocking).  NULL pointers skipped. */
int chf_download_state(chf_handle* h,
                       double* vnp1, double* omegaynp1,
                       double* unp1, double* wnp1,
                       double* omegaxnp1, double* omegaznp1,
                       double* rhsvn, double* rhsomegayn,
                       double* clamb1n, double* clamb1nm1,
                       double* clamb3n, double* clamb3nm1,
                       double* au0, double* w0);

/* getnonlinear (poiseuilleflow.f90:1380-1612): Lamb vector by dealiased
 * products, its curl/projection, history swap, coefficients -> GL values. */
int chf_getnonlinear(chf_handle* h);

/* The per-mode solve loop (poiseuilleflow.f90:242-394) followed by the
 * (0,0)-mode solve (poiseuilleflow.f90:401-474). */
int chf_solve(chf_handle* h);

/* nsteps iterations of the main loop body for istep > istepbegin
 * (poiseuilleflow.f90:224 then 242-474).  Asynchronous on the handle's
 * stream; chf_synchronize() waits.  Pairs of steps replay a CUDA graph
 * captured on the first call (one launch per pair instead of one per
 * kernel); the kernels and results are those of chf_getnonlinear +
 * chf_solve.  Steps launch directly instead while per-kernel profiling is
 * on, or when the stream is already under capture by the caller. */
int chf_step(chf_handle* h, int nsteps);

/* nsteps iterations of the main loop body (poiseuilleflow.f90:219-474) on
 * host-resident module arrays, updated in place: the reference driver's
 * step, whose arrays live in host memory.  Blocking.  Equivalent to
 * chf_upload_state + chf_step(nsteps) + chf_download_state on the same
 * arrays (bit-identical results), with the copies overlapped with the
 * computation: the N^{n-1} histories upload during the first nonlinear term,
 * the new histories and (mixed path) vnp1 / omegaynp1 download during the
 * last solve.  Every pointer is required (CHF_E_INVALID otherwise); page-
 * locked host memory gives the full link bandwidth.  Steps launch directly
 * (no CUDA graph). */
int chf_step_host(chf_handle* h, int nsteps,
                  double* vnp1, double* omegaynp1,
                  double* unp1, double* wnp1,
                  double* omegaxnp1, double* omegaznp1,
                  double* rhsvn, double* rhsomegayn,
                  double* clamb1n, double* clamb1nm1,
                  double* clamb3n, double* clamb3nm1,
                  double* au0, double* w0);

int chf_synchronize(chf_handle* h);

/* Diagnostics of the current state (synchronous). */
int chf_diagnostics(chf_handle* h, chf_diag* out);

/* Number of kernels launched per chf_step iteration (for instrumentation). */
int chf_kernels_per_step(const chf_handle* h);

/* Device address of one resident module array (0..7: vnp1, omegaynp1, unp1,
 * wnp1, omegaxnp1, omegaznp1, rhsvn, rhsomegayn), for zero-copy access by
 * device-side callers.  Valid until the next chf_* call on h. */
int chf_device_field(chf_handle* h, int which, void** dptr);

/* Run subsequent work of h on a caller-provided CUDA stream (a cudaStream_t
 * passed as void*), e.g. the stream of a host framework; NULL restores the
 * library's own stream.  The caller keeps the stream alive while h uses it. */
int chf_set_stream(chf_handle* h, void* stream);

/* Test of failure detection, no counterpart in the reference.  The
 * tensor-core GEMMs of the mixed precisions bound every wait of their
 * pipeline (1 s of wall time); on a timeout each role records a code in the
 * handle's device status word, waits (bounded) for its copies and MMAs in
 * flight, frees the tensor memory and returns, and the next
 * chf_synchronize / chf_diagnostics / chf_step_host reports CHF_E_CUDA with
 * the code in chf_last_error, once (the word is cleared; the state of that
 * step is not valid).  This call arms one occurrence: the next GEMM launch
 * on h issues no copies for its first stage, so the waits on that stage run
 * out after wait_us microseconds (1 .. 1000000).  No fault, trap or unbounded
 * wait is involved.  CHF_E_INVALID for CHF_FP64 handles. */
int chf_test_wait_timeout(chf_handle* h, int wait_us);

/* Autotuner, the counterpart of the reference's FFTW_MEASURE planning
 * (poiseuilleflow.f90:100-112): times whole steps of the handle's state
 * (saved first and put back) for the candidate radix orders of the
 * shared-memory FFTs, lines per CTA of the FFT kernels and, for CHF_MIXED,
 * the increment solve's modes per CTA, columns per load batch, rows per
 * thread and block width, and keeps the fastest (each knob in turn; a
 * candidate must be 1% faster; every candidate computes the same results
 * bit for bit).  reps:
 * timed runs per candidate (0: 3).  The choice is cached for the process:
 * later chf_create calls for the same device, grid, product grid and
 * precision start from it.  Synchronous; needs an uploaded state. */
int chf_autotune(chf_handle* h, int reps);
/* The handle's launch shapes and radix orders as text (the measured step
 * times when tuned), NUL-terminated in buf[0..len-1]. */
int chf_tuning(const chf_handle* h, char* buf, int len);
/* Sets one launch shape by name, in place of the rule or the autotuner's
 * choice (every shape but "recover_form" computes the same results, bit for
 * bit):
 *   "inc_modes"    modes per CTA of the CHF_MIXED increment solve: 2 or 4
 *   "inc_columns"  its matrix columns per load batch: 2, 3 or 4
 *   "inc_rows"     its block rows per thread: 1 or 2 (2 with 2 or 3 columns)
 *   "inc_wide"     with one row per thread, every block row in one pass (1,
 *                  up to 416 threads) or 288-thread blocks that loop (0)
 *   "recover_form" arithmetic of the CHF_MIXED recovery of u, w, omega_x,
 *                  omega_z from v and omega_y: 0 FP64, 1 double-float
 *                  (about 2^-44 of the largest term), -1 the rule (double-
 *                  float where the grid has at least 16 x 32 x SMs / 4
 *                  modes).  The one setting whose results differ (in the
 *                  last bits); the autotuner leaves it alone.
 *   "kxb", "xr", "zl_c2v", "zl_curl"  lines per CTA of the shared-memory
 *                  FFT kernels: one of the shapes that fit the grid, or 0
 *                  for the launcher's rule
 * CHF_E_INVALID for an unknown name or a value that the grid or the other
 * shapes rule out (the handle is then unchanged).  Synchronous. */
int chf_set_launch_shape(chf_handle* h, const char* name, int value);

/* Per-kernel timing with CUDA events recorded around every launch on the
 * handle's stream (off by default; the reference's only instrumentation is
 * the mpi_wtime prints at poiseuilleflow.f90:216-229, 481-486). */
int chf_profile_enable(chf_handle* h, int on);
int chf_profile_reset(chf_handle* h);
/* Kernel idx (0-based): its name, launch count and total device time since
 * the last reset (synchronises the stream).  CHF_E_INVALID past the end. */
int chf_profile_read(chf_handle* h, int idx, const char** name, int* launches, double* total_ms);

/* Flow statistics of the current state, as statistics
 * (poiseuilleflow.f90:2666-3198) forms them from the physical
 * nnx x nny x (nz+1) grid, computed here from spectral sums (Parseval) with
 * no in-plane transform.  profiles (NULL or 10 x (nz+1) doubles, row-major):
 * z_k = cos(pi k / nz), <u>, <v>, <w>, <u'u'>, <v'v'>, <w'w'>, <u'v'>, <u'w'>,
 * <v'w'> at the Gauss-Lobatto points (u streamwise, v wall-normal, w
 * spanwise).  The first call allocates a scratch of 3 (nz+1) nnx nny / 2
 * complex doubles kept until chf_destroy.  Synchronous. */
typedef struct chf_stats {
  double u_tau_top, u_tau_bottom;   /* sqrt(|d<u>/dz| / re) at z = +1 and z = -1 */
  double re_tau_top, re_tau_bottom; /* u_tau * re (the "R_t" print) */
  double re_centre;                 /* <u>(z = 0) * re ("R_c") */
  double re_bulk;                   /* 2 U_b re with the reference's half-channel rectangle rule ("R_b") */
  double bulk_velocity;             /* (1/2) int <u> dz, exact from the Chebyshev coefficients of au0 */
  double energy;                    /* 0.5 sum of u^2 + v^2 + w^2 over the physical grid (energy.plt) */
} chf_stats;
int chf_statistics(chf_handle* h, double* profiles, chf_stats* out);

/* Physical space (FP64 for either precision; the first of these calls
 * allocates three field-sized work buffers, kept until chf_destroy; all are
 * synchronous).  The physical grid is the unpadded one of transform:
 * x_i = 2 pi aphi i / nnx, y_j = 2 pi beta j / nny, z_k = cos(pi k / nz),
 * stored as a field array (0:nx,0:ny,0:nz) with x the physical point index.
 *
 * chf_transform: transform (poiseuilleflow.f90:919-1005, with fourtrx_zcomp
 * :774-913) of one host array in place.  isign = 1: spectral (Chebyshev
 * coefficients in z, interleaved (re, im) streamwise modes, spanwise modes)
 * to physical values, spanwise and streamwise Nyquist modes dropped;
 * isign = -1: physical values to the spectral layout (all nny spanwise
 * slots, streamwise modes 0..nnx/2-1, normalised by 1/(nnx nny)). */
int chf_transform(chf_handle* h, int isign, double* u);

/* The CFL numbers printed by statistics (poiseuilleflow.f90:2866-2934), of
 * the current state (call after a solve, where statistics is called):
 * cfl_x = max|u| dt / dx (streamwise), cfl_z = max|w| dt / dz (spanwise,
 * dz = 2 pi beta / nny), cfl_y = max over the interior planes k = 1..nz-1 of
 * max|v| dt / dy(k) (wall-normal; dy(k) the Gauss-Lobatto spacing of
 * statistics, mirrored about the centre).  Maxima over the physical grid;
 * u includes the mean mode au0.  Any pointer may be NULL. */
int chf_cfl(chf_handle* h, double* cfl_x, double* cfl_y, double* cfl_z);

/* The instantaneous physical velocity of the 3Ddata dump of statistics
 * (poiseuilleflow.f90:2745-2764): out (0:nnx-1, 0:nny-1, 0:nz, 3) real*8,
 * Fortran order, component 1 = u + u0(k) (streamwise), 2 = w (spanwise),
 * 3 = v (wall-normal).  u0: base-flow profile (nz + 1 doubles) added to u
 * as the reference adds its u0, or NULL for none. */
int chf_physical_velocity(chf_handle* h, const double* u0, double* out);

/* That dump as statistics writes it: one Fortran unformatted sequential file
 * per rank, <dir>/velocity<istep:8>.<rank:3>.dat (format 212 of
 * poiseuilleflow.f90:2749-2750), one record holding ftmp(0:nx,0:ny,0:nz,1:3)
 * of the rank's streamwise slab of nnx / nproc physical points, framed by
 * 4-byte byte counts; post-processing/post_poiseuilleflow.f90:63-70 reads
 * and joins the slabs.  nproc follows the reference's constraints (nnx a
 * multiple of 2 nproc, nny / 2 a multiple of nproc) and a record must stay
 * below 2 GiB, else CHF_E_INVALID. */
int chf_write_velocity(chf_handle* h, const char* dir, int nproc, int istep, const double* u0);

/* Pressure of the current state (after a solve: velocities and vorticities
 * in the module arrays), as Chebyshev coefficients in the field layout
 * (p_out: (0:nx,0:ny,0:nz) real*8, host).  The reference's pressure routine
 * (instantp, poiseuilleflow.f90:3701-3890) is never called; this is a
 * spectral replacement consistent with the time step: P is the total head
 * p + |u|^2 / 2 of the rotational form u_t = -H - grad P + lap u / re, from
 * (D^2 - k^2) P = -(i alpha H1 + D H2 + i beta H3) with the Neumann walls
 * D P = -H2 + (D^2 - k^2) v / re, collocated at the Gauss-Lobatto points;
 * the (0,0) mode has zero mean over z and excludes the driving gradient
 * re_p.  FP64 for either precision; the first call allocates its work
 * buffers (kept until chf_destroy).  Synchronous. */
int chf_pressure(chf_handle* h, double* p_out);

/* Constant flow rate.  No counterpart in the reference, which drives the
 * flow with the fixed mean pressure gradient re_p (paraandcons.f90:25);
 * required by the 32^3 Poiseuille workload.  With a target bulk velocity
 * U_b > 0 (U_b = (1/2) int u dz over the (0,0) mode), every solve adds to
 * the new mean profile au0 the multiple of the response to a unit mean
 * pressure gradient (same operator and walls as poiseuilleflow.f90:401-474)
 * that restores U_b; that multiple is the step's extra pressure gradient.
 * 0 switches the control off (the default). */
int chf_set_flow_rate(chf_handle* h, double bulk_velocity);
/* The target, the bulk velocity after the last solve and the last extra mean
 * pressure gradient (all 0 while the control is off; synchronous). */
int chf_get_flow_rate(chf_handle* h, double* target, double* bulk_velocity, double* dpdx_correction);

/* Restart files in the reference's layout: one Fortran unformatted
 * sequential file per MPI rank, as output (poiseuilleflow.f90:2460-2504)
 * writes them and initial (poiseuilleflow.f90:1873-1917) reads them.
 * Record 1 holds clamb1n, clamb1nm1, clamb3n, clamb3nm1, au0 and w0.
 * Record 2 holds vnp1, omegaynp1, rhsvn, rhsomegayn, unp1 and wnp1 for the
 * rank's streamwise slab of nnx / nproc slots; records are framed by 4-byte
 * byte counts.  Files are <dir>/data<tag:8>_instant.<rank:3>.dat, or
 * ..._instant.<rank:3>_<istep:8>.dat when istep >= 0 (the reference writes
 * tag 2).  Write where the reference calls output: after chf_getnonlinear.
 * After chf_read_restart the run continues with chf_solve, as the
 * reference's first iteration does.  nproc must satisfy the reference's own
 * constraints (nnx a multiple of 2 nproc, nny / 2 a multiple of nproc), and a
 * rank's record must stay below 2 GiB; else CHF_E_INVALID.  Synchronous. */
int chf_write_restart(chf_handle* h, const char* dir, int nproc, int tag, int istep);
int chf_read_restart(chf_handle* h, const char* dir, int nproc, int tag, int istep);

/* Ensembles.  No counterpart in the reference (one channel per MPI job): a
 * batch holds n independent channels of any sizes, Reynolds numbers and
 * precisions on one device (all cfgs[i].device equal) and advances them
 * together.  Pairs of steps replay one CUDA graph that forks into one branch
 * per channel, so small channels run side by side instead of one launch
 * after another.  chf_batch_handle lends channel i's handle for
 * upload/download/diagnostics/restart calls (do not destroy it; it lives
 * until chf_batch_destroy); each channel's results are bit-identical to
 * stepping it alone.  chf_batch_step is asynchronous and orders itself after
 * work already queued on the channels and before work queued later. */
typedef struct chf_batch chf_batch;
int chf_batch_create(int n, const chf_config* cfgs, chf_batch** out);
int chf_batch_destroy(chf_batch* b);
/* Last error of b, or of the last failed chf_batch_create when b is NULL. */
const char* chf_batch_last_error(const chf_batch* b);
int chf_batch_size(const chf_batch* b);
int chf_batch_handle(chf_batch* b, int i, chf_handle** h);
int chf_batch_step(chf_batch* b, int nsteps);
int chf_batch_synchronize(chf_batch* b);

/* Allocation-free diagnostics.  No counterpart in the reference: an addition
 * for callers that cannot allocate device memory (their device memory is
 * owned by another runtime's pool, or fully committed to the resident state,
 * or their time loop must avoid the synchronisation of cudaMalloc/cudaFree).
 * It computes the energy, max |value| and finiteness of chf_diagnostics
 * (wall shear is reported as 0) on the caller's own device arrays in the
 * field layout above, plus the energy of every wall-normal plane k in
 * energy_profile[k] (k = 0..nnz, may be NULL), with no handle and no
 * allocation: its scratch is a fixed __device__ array inside the library.
 * nnz + 1 must not exceed CHF_STATIC_MAX_PLANES, and the grid must satisfy
 * chf_create's rules (nnx, nny multiples of 4; nnz even, >= 4), else
 * CHF_E_INVALID before any CUDA call.  The call waits for its stream and
 * returns its results in host memory.  The first call on a device looks up
 * the array's address with that device current (cudaGetSymbolAddress), so
 * make that first call before any stream capture.  All calls share the
 * array, so calls that overlap on the GPU race and must be serialised by the
 * caller.  stream: a cudaStream_t or NULL. */
#define CHF_STATIC_MAX_PLANES 1025
int chf_diagnostics_static(int nnx, int nny, int nnz,
                           const double* d_unp1, const double* d_vnp1, const double* d_wnp1,
                           const double* d_omegaxnp1, const double* d_omegaynp1,
                           const double* d_omegaznp1, double* energy_profile, chf_diag* out,
                           void* stream);

#ifdef __cplusplus
}
#endif
#endif /* CHFLOW_H */
