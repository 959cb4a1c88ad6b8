/*
 * chflow_oracle.h -- CPU restatement of the channel-flow time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path
 * is compared against (tests/, __graft_entry__.smoke and the CPU-baseline leg
 * of bench.py).  It is never linked into, called by, or shipped with the
 * product library in channel_flow_gb300/.
 *
 * What it restates: the per-step advance of poiseuilleflow.f90
 * (getnonlinear, poiseuilleflow.f90:1380-1612, followed by the per-mode solve
 * loop and the (0,0)-mode solve, poiseuilleflow.f90:242-474) with nproc = 1,
 * on the reference's own array layout: real*8 (0:nx,0:ny,0:nz), x fastest,
 * even x index = real part and odd = imaginary part of one streamwise mode
 * (poiseuilleflow.f90:8-12).  Third-party arithmetic the reference takes from
 * FFTW 2.1.5 (unnormalised complex DFTs, FFTW_FORWARD = exp(-2 pi i jk/n),
 * fftw_f77.i:8-9) and MKL (zgetrf/zgetri, a partial-pivoting LU inverse) is
 * restated here from the published algorithms: a Stockham mixed-radix DFT and
 * an unblocked LAPACK-style getf2/trtri/getri inverse.
 *
 * Parity status: UNPINNED against the reference itself.  The reference ships
 * no tests, fixtures or golden vectors, and it cannot be built here or on the
 * GPU host (no Fortran compiler, MPI, FFTW 2 or MKL).  The restatement is
 * instead pinned by (a) an independent NumPy restatement (tests/golden), (b)
 * the reference's own A * inv(A) self-check (poiseuilleflow.f90:206-212) and
 * (c) physics known-answer tests (laminar fixed point, divergence, energy).
 */
#ifndef CHFLOW_ORACLE_H
#define CHFLOW_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc orc;

/* Fields of the paraandcons module (paraandcons.f90:28-38), Fortran layout. */
enum {
  ORC_VNP1 = 0, ORC_OMEGAYNP1, ORC_UNP1, ORC_WNP1, ORC_OMEGAXNP1, ORC_OMEGAZNP1,
  ORC_RHSVN, ORC_RHSOMEGAYN, ORC_NFIELDS
};
/* (2,0:nz) mean-mode arrays (paraandcons.f90:33,38). */
enum {
  ORC_CLAMB1N = 0, ORC_CLAMB1NM1, ORC_CLAMB3N, ORC_CLAMB3NM1, ORC_AU0, ORC_W0, ORC_NMEAN
};

orc*    orc_create(int nnx, int nny, int nnz, double aphi, double beta,
                   double dt, double re, double re_p);
void    orc_destroy(orc* o);
void    orc_set_threads(int n);
double* orc_field(orc* o, int which);
double* orc_mean(orc* o, int which);
void    orc_setup(orc* o);                 /* SCHEB + explicit inverses */
void    orc_getnonlinear(orc* o);          /* poiseuilleflow.f90:1380-1612 */
void    orc_solve(orc* o);                 /* poiseuilleflow.f90:242-474   */
void    orc_step(orc* o, int nsteps);      /* nsteps x (getnonlinear + solve) */
void    orc_velocity_all(orc* o);          /* getvelocityandvorticity on every mode */
void    orc_transform(orc* o, int isign, double* u);  /* poiseuilleflow.f90:919-1005 */
/* Unit-test hooks. */
void    orc_fft(int n, int sign, double* data);          /* in-place, interleaved complex */
void    orc_dz(double* v, int n);                        /* poiseuilleflow.f90:570-599 */
void    orc_getlamb(orc* o, const double* u, const double* omega, double* lamb, int with_rep);
void    orc_matrices(orc* o, double kmn, double* av, double* ae, double* xv, double* xe);
void    orc_scheb(orc* o, double* t0, double* t1, double* t2, double* t4);

#ifdef __cplusplus
}
#endif
#endif
