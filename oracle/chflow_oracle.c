/*
 * chflow_oracle.c -- CPU restatement of the channel-flow time step of
 * poiseuilleflow.f90 (nproc = 1).  TEST INFRASTRUCTURE ONLY: the checker for
 * the CUDA path and the timed CPU baseline, never part of the product.
 *
 * Each routine names the Fortran lines it restates.  Where the reference's
 * MPI routines degenerate for one rank they are replaced by the equivalent
 * local index shuffles: transposefft_c_r / transposefft_r_c
 * (poiseuilleflow.f90:1198-1337) become plain transposes and equipment
 * (poiseuilleflow.f90:665-707) becomes the identity.
 *
 * Parity is UNPINNED against the reference itself (no tests, fixtures or
 * buildable toolchain exist for it); see chflow_oracle.h.
 *
 * Build: oracle/build_oracle.py (gcc -O2 -ffp-contract=off -fopenmp), so that x86
 * and Arm hosts round identically (no FMA contraction).
 */
#include "chflow_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Complex DFT: Stockham autosort, radix 4/2/3/5 and a generic odd radix.    */
/* Unnormalised, sign -1 = FFTW_FORWARD, +1 = FFTW_BACKWARD (fftw_f77.i:8-9). */
/* ------------------------------------------------------------------------ */
typedef struct { double re, im; } cx;

#define MAXSTAGE 40
#define MAXRADIX 64

typedef struct {
  int n, nst;
  int R[MAXSTAGE], Ns[MAXSTAGE];
  cx* tw[MAXSTAGE]; /* tw[s][jm*R + r] = exp(-2 pi i r jm / (Ns R)) */
  cx* root;         /* root[k] = exp(-2 pi i k / n) */
} fftplan;

static void plan_init(fftplan* p, int n) {
  memset(p, 0, sizeof(*p));
  p->n = n;
  int m = n;
  while (m > 1) {
    int r;
    if (m % 4 == 0) r = 4;
    else if (m % 2 == 0) r = 2;
    else if (m % 3 == 0) r = 3;
    else if (m % 5 == 0) r = 5;
    else {
      r = 7;
      while (m % r) r += 2;
    }
    p->R[p->nst++] = r;
    m /= r;
  }
  p->root = (cx*)malloc(sizeof(cx) * (size_t)(n > 0 ? n : 1));
  const double twopi = 8.0 * atan(1.0);
  for (int k = 0; k < n; ++k) {
    double a = -twopi * (double)k / (double)n;
    p->root[k].re = cos(a);
    p->root[k].im = sin(a);
  }
  int Ns = 1;
  for (int s = 0; s < p->nst; ++s) {
    int R = p->R[s];
    p->Ns[s] = Ns;
    p->tw[s] = (cx*)malloc(sizeof(cx) * (size_t)Ns * R);
    for (int jm = 0; jm < Ns; ++jm)
      for (int r = 0; r < R; ++r) {
        long idx = ((long)r * jm * (n / (Ns * R))) % n;
        p->tw[s][jm * R + r] = p->root[idx];
      }
    Ns *= R;
  }
}

static void plan_free(fftplan* p) {
  for (int s = 0; s < p->nst; ++s) free(p->tw[s]);
  free(p->root);
}

/* small DFT of length R in place, v[k] = sum_r v[r] exp(sign 2 pi i r k / R) */
static void small_dft(cx* v, int R, int sign, const fftplan* p) {
  if (R == 2) {
    cx a = v[0], b = v[1];
    v[0].re = a.re + b.re; v[0].im = a.im + b.im;
    v[1].re = a.re - b.re; v[1].im = a.im - b.im;
  } else if (R == 4) {
    cx t0 = {v[0].re + v[2].re, v[0].im + v[2].im};
    cx t1 = {v[0].re - v[2].re, v[0].im - v[2].im};
    cx t2 = {v[1].re + v[3].re, v[1].im + v[3].im};
    cx t3 = {v[1].re - v[3].re, v[1].im - v[3].im};
    /* (sign i) * t3 */
    cx st3 = {-(double)sign * t3.im, (double)sign * t3.re};
    v[0].re = t0.re + t2.re; v[0].im = t0.im + t2.im;
    v[2].re = t0.re - t2.re; v[2].im = t0.im - t2.im;
    v[1].re = t1.re + st3.re; v[1].im = t1.im + st3.im;
    v[3].re = t1.re - st3.re; v[3].im = t1.im - st3.im;
  } else if (R == 3) {
    const double c = 0.86602540378443864676; /* sqrt(3)/2 */
    cx s = {v[1].re + v[2].re, v[1].im + v[2].im};
    cx d = {v[1].re - v[2].re, v[1].im - v[2].im};
    cx a = v[0];
    cx m = {a.re - 0.5 * s.re, a.im - 0.5 * s.im};
    /* sign i c d */
    cx e = {-(double)sign * c * d.im, (double)sign * c * d.re};
    v[0].re = a.re + s.re; v[0].im = a.im + s.im;
    v[1].re = m.re + e.re; v[1].im = m.im + e.im;
    v[2].re = m.re - e.re; v[2].im = m.im - e.im;
  } else {
    cx out[MAXRADIX];
    const double twopi = 8.0 * atan(1.0);
    for (int k = 0; k < R; ++k) {
      double sr = 0.0, si = 0.0;
      for (int r = 0; r < R; ++r) {
        double a = (double)sign * twopi * (double)((r * k) % R) / (double)R;
        double cr = cos(a), ci = sin(a);
        sr += v[r].re * cr - v[r].im * ci;
        si += v[r].re * ci + v[r].im * cr;
      }
      out[k].re = sr; out[k].im = si;
    }
    for (int k = 0; k < R; ++k) v[k] = out[k];
  }
  (void)p;
}

/* x: data (n complex), work: scratch (n complex); result in x. */
static void fft_exec(const fftplan* p, cx* x, cx* work, int sign) {
  const int n = p->n;
  cx* a = x;
  cx* b = work;
  for (int s = 0; s < p->nst; ++s) {
    const int R = p->R[s], Ns = p->Ns[s], nr = n / R;
    const cx* tw = p->tw[s];
    for (int j = 0; j < nr; ++j) {
      const int jm = j % Ns;
      cx v[MAXRADIX];
      for (int r = 0; r < R; ++r) {
        cx t = a[j + r * nr];
        cx w = tw[jm * R + r];
        if (sign > 0) w.im = -w.im;
        v[r].re = t.re * w.re - t.im * w.im;
        v[r].im = t.re * w.im + t.im * w.re;
      }
      small_dft(v, R, sign, p);
      const int idxD = (j / Ns) * Ns * R + jm;
      for (int r = 0; r < R; ++r) b[idxD + r * Ns] = v[r];
    }
    cx* t = a; a = b; b = t;
  }
  if (a != x) memcpy(x, a, sizeof(cx) * (size_t)n);
}

/* ------------------------------------------------------------------------ */
/* Solver state                                                              */
/* ------------------------------------------------------------------------ */
struct orc {
  int nnx, nny, nnz;
  int nx, ny, nz, nhx;     /* paraandcons.f90:8-11 with nproc = 1 */
  int X, Y, Z;             /* nx+1, ny+1, nz+1 */
  int PX, PY;              /* 3/2-padded sizes 3*nnx/2, 3*nny/2 */
  double aphi, beta, dt, re, re_p;
  double *iapha, *ibeta;   /* poiseuilleflow.f90:123-134 */
  double *t0, *t1, *t2, *t4; /* (0:nz,0:nz) column-major, SCHEB */
  double* f[ORC_NFIELDS];
  double* mean[ORC_NMEAN]; /* (2,0:nz): [2*k] real part, [2*k+1] imaginary part */
  /* explicit inverses per distinct k^2 (get_coef_* depends only on kmn) */
  int nk2;
  double* k2vals;
  double *xv, *xe;         /* nk2 x (Z*Z), column-major (row i, col j at i + Z*j) */
  int* modek2;             /* (nhx+1)*(ny+1) -> index into k2vals or -1 */
  double *au0mat;          /* A_u0 (Z*Z) column-major */
  fftplan pny, pnnx, ppy, ppx, p2z, p4z;
  double *up, *omegap;     /* PY*PX*Z scratch for getlamb */
  double *lamb1, *lamb2;   /* X*Y*Z scratch for getnonlinear */
  int ready;
};

static int g_threads = 0;
void orc_set_threads(int n) {
  g_threads = n;
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#endif
}

#define IDX(o, i, j, k) ((size_t)(i) + (size_t)(o)->X * ((size_t)(j) + (size_t)(o)->Y * (size_t)(k)))

orc* orc_create(int nnx, int nny, int nnz, double aphi, double beta, double dt, double re,
                double re_p) {
  orc* o = (orc*)calloc(1, sizeof(orc));
  o->nnx = nnx; o->nny = nny; o->nnz = nnz;
  o->nx = nnx - 1; o->ny = nny - 1; o->nz = nnz;
  o->nhx = (o->nx - 1) / 2;
  o->X = o->nx + 1; o->Y = o->ny + 1; o->Z = o->nz + 1;
  o->PX = 3 * nnx / 2; o->PY = 3 * nny / 2;
  o->aphi = aphi; o->beta = beta; o->dt = dt; o->re = re; o->re_p = re_p;
  const size_t nf = (size_t)o->X * o->Y * o->Z;
  for (int w = 0; w < ORC_NFIELDS; ++w) o->f[w] = (double*)calloc(nf, sizeof(double));
  for (int w = 0; w < ORC_NMEAN; ++w) o->mean[w] = (double*)calloc((size_t)2 * o->Z, sizeof(double));
  o->lamb1 = (double*)calloc(nf, sizeof(double));
  o->lamb2 = (double*)calloc(nf, sizeof(double));
  const size_t np = (size_t)o->PX * o->PY * o->Z;
  o->up = (double*)calloc(np, sizeof(double));
  o->omegap = (double*)calloc(np, sizeof(double));
  /* wavenumbers, poiseuilleflow.f90:123-134 (id = 0) */
  o->ibeta = (double*)calloc((size_t)o->Y, sizeof(double));
  o->iapha = (double*)calloc((size_t)o->nhx + 1, sizeof(double));
  for (int j = 0; j <= (o->ny + 1) / 2; ++j) {
    o->ibeta[j] = (double)j / beta;
    if (j <= (o->ny - 1) / 2 - 1) o->ibeta[o->ny - j] = (double)(-j - 1) / beta;
  }
  for (int i = 0; i <= o->nhx; ++i)
    o->iapha[i] = (0.0 * (double)(o->nx + 1) * 0.5 + (double)i) / aphi;
  plan_init(&o->pny, nny);
  plan_init(&o->pnnx, nnx);
  plan_init(&o->ppy, o->PY);
  plan_init(&o->ppx, o->PX);
  plan_init(&o->p2z, 2 * o->nz);
  plan_init(&o->p4z, 4 * o->nz);
  return o;
}

void orc_destroy(orc* o) {
  if (!o) return;
  for (int w = 0; w < ORC_NFIELDS; ++w) free(o->f[w]);
  for (int w = 0; w < ORC_NMEAN; ++w) free(o->mean[w]);
  free(o->lamb1); free(o->lamb2); free(o->up); free(o->omegap);
  free(o->ibeta); free(o->iapha);
  free(o->t0); free(o->t1); free(o->t2); free(o->t4);
  free(o->k2vals); free(o->xv); free(o->xe); free(o->modek2); free(o->au0mat);
  plan_free(&o->pny); plan_free(&o->pnnx); plan_free(&o->ppy); plan_free(&o->ppx);
  plan_free(&o->p2z); plan_free(&o->p4z);
  free(o);
}

double* orc_field(orc* o, int which) { return o->f[which]; }
double* orc_mean(orc* o, int which) { return o->mean[which]; }

/* ------------------------------------------------------------------------ */
/* SCHEB, poiseuilleflow.f90:3272-3342                                       */
/* ------------------------------------------------------------------------ */
static void scheb(int n2, double* t0, double* t1, double* t2, double* t4) {
  const int Z = n2 + 1;
#define T(a, J, L) a[(size_t)(J) + (size_t)Z * (size_t)(L)]
  const double h0 = 4.0 * atan(1.0) / (double)n2;
  for (int L = 0; L <= n2; ++L) {
    double Ld = (double)L;
    double sgnL = (L % 2 == 0) ? 1.0 : -1.0;
    T(t0, 0, L) = 1.0;
    T(t0, n2, L) = sgnL;
    T(t1, 0, L) = Ld * Ld;
    T(t1, n2, L) = -sgnL * Ld * Ld;
    T(t2, 0, L) = Ld * Ld * (Ld * Ld - 1.0) / 3.0;
    T(t2, n2, L) = sgnL * (Ld * Ld) * (Ld * Ld - 1.0) / 3.0;
    T(t4, 0, L) = 0.0;
    T(t4, n2, L) = 0.0;
  }
  for (int J = 1; J <= n2 - 1; ++J) {
    double q = h0 * J;
    double c1 = cos(q), c2 = c1 * c1, s1 = sin(q), s2 = s1 * s1;
    double ds1 = 1.0 / s1, ds3 = ds1 / s2, ds5 = ds3 / s2, ds7 = ds5 / s2;
    (void)ds5;
    for (int L = 0; L <= n2; ++L) {
      double bj = (double)L, qj = q * bj, sj = sin(qj), cj = cos(qj);
      double bs = bj * bj * s2, bc = bj * cj * s1;
      T(t0, J, L) = cj;
      T(t1, J, L) = bj * sj * ds1;
      T(t2, J, L) = bj * (sj * c1 - bc) * ds3;
      T(t4, J, L) = bj * (sj * c1 * (9.0 + 6.0 * (c2 - bs)) - bc * (4.0 + 11.0 * c2 - bs)) * ds7;
    }
  }
#undef T
}

void orc_scheb(orc* o, double* t0, double* t1, double* t2, double* t4) {
  scheb(o->nz, t0, t1, t2, t4);
}

/* ------------------------------------------------------------------------ */
/* Operators, poiseuilleflow.f90:3348-3534 (real: tmpi = 0 throughout)       */
/* ------------------------------------------------------------------------ */
static void get_coef_v(const orc* o, double kmn, double* a) {
  const int n = o->nz, Z = o->Z;
  const double dt = o->dt, re = o->re;
  for (int i = 4; i <= n; ++i)
    for (int j = 0; j <= n; ++j) {
      size_t p = (size_t)(i - 2) + (size_t)Z * j;
      a[i + (size_t)Z * j] = -(o->t4[p] * dt * 0.5 / re) + (1.0 + kmn * dt / re) * o->t2[p] -
                             kmn * (1.0 + kmn * dt * 0.5 / re) * o->t0[p];
    }
  for (int j = 0; j <= n; ++j) {
    double s = (j % 2 == 0) ? 1.0 : -1.0;
    a[0 + (size_t)Z * j] = 1.0;
    a[1 + (size_t)Z * j] = s;
    a[2 + (size_t)Z * j] = (double)j * (double)j;
    a[3 + (size_t)Z * j] = -s * (double)j * (double)j;
  }
}

static void get_coef_omegay(const orc* o, double kmn, double* a) {
  const int n = o->nz, Z = o->Z;
  const double dt = o->dt, re = o->re;
  for (int i = 2; i <= n; ++i)
    for (int j = 0; j <= n; ++j) {
      size_t p = (size_t)(i - 1) + (size_t)Z * j;
      a[i + (size_t)Z * j] = -(o->t2[p] * dt * 0.5 / re) + (1.0 + kmn * dt * 0.5 / re) * o->t0[p];
    }
  for (int j = 0; j <= n; ++j) {
    a[0 + (size_t)Z * j] = 1.0;
    a[1 + (size_t)Z * j] = (j % 2 == 0) ? 1.0 : -1.0;
  }
}

static void get_coef_u0(const orc* o, double* a) {
  const int n = o->nz, Z = o->Z;
  const double dt = o->dt, re = o->re;
  for (int i = 2; i <= n; ++i)
    for (int j = 0; j <= n; ++j) {
      size_t p = (size_t)(i - 1) + (size_t)Z * j;
      a[i + (size_t)Z * j] = -(o->t2[p] * dt * 0.5 / re) + o->t0[p];
    }
  for (int j = 0; j <= n; ++j) {
    a[0 + (size_t)Z * j] = 1.0;
    a[1 + (size_t)Z * j] = (j % 2 == 0) ? 1.0 : -1.0;
  }
}

/* Explicit inverse of a real n x n column-major matrix in place: LU with
 * partial pivoting (first maximal |a|, LAPACK getf2), inv(U) (trtri) and the
 * getri back-substitution with column interchanges.  Restates the
 * zgetrf/zgetri pair at poiseuilleflow.f90:201-204 for matrices whose
 * imaginary parts are zero.  Returns 0 on success. */
static int lu_inverse(double* a, int n, int* ipiv, double* work) {
#define A(i, j) a[(size_t)(i) + (size_t)n * (size_t)(j)]
  for (int j = 0; j < n; ++j) {
    int p = j;
    double amax = fabs(A(j, j));
    for (int i = j + 1; i < n; ++i)
      if (fabs(A(i, j)) > amax) { amax = fabs(A(i, j)); p = i; }
    ipiv[j] = p;
    if (A(p, j) == 0.0) return j + 1;
    if (p != j)
      for (int c = 0; c < n; ++c) { double t = A(j, c); A(j, c) = A(p, c); A(p, c) = t; }
    double r = 1.0 / A(j, j);
    for (int i = j + 1; i < n; ++i) A(i, j) *= r;
    for (int c = j + 1; c < n; ++c) {
      double ujc = A(j, c);
      if (ujc != 0.0)
        for (int i = j + 1; i < n; ++i) A(i, c) -= A(i, j) * ujc;
    }
  }
  /* inv(U), column by column (trti2, upper, non-unit) */
  for (int j = 0; j < n; ++j) {
    A(j, j) = 1.0 / A(j, j);
    double ajj = -A(j, j);
    /* x = triu(A(0:j,0:j)) * A(0:j, j)  (trmv, upper, no-trans) */
    for (int k = 0; k < j; ++k) {
      double t = A(k, j);
      if (t != 0.0) {
        for (int i = 0; i < k; ++i) A(i, j) += t * A(i, k);
        A(k, j) = t * A(k, k);
      }
    }
    for (int i = 0; i < j; ++i) A(i, j) *= ajj;
  }
  /* solve inv(A) * L = inv(U) (getri, unblocked) */
  for (int j = n - 1; j >= 0; --j) {
    for (int i = j + 1; i < n; ++i) { work[i] = A(i, j); A(i, j) = 0.0; }
    if (j < n - 1)
      for (int c = j + 1; c < n; ++c) {
        double w = work[c];
        if (w != 0.0)
          for (int i = 0; i < n; ++i) A(i, j) -= A(i, c) * w;
      }
  }
  for (int j = n - 2; j >= 0; --j) {
    int jp = ipiv[j];
    if (jp != j)
      for (int i = 0; i < n; ++i) { double t = A(i, j); A(i, j) = A(i, jp); A(i, jp) = t; }
  }
  return 0;
#undef A
}

static int cmp_double(const void* a, const void* b) {
  double x = *(const double*)a, y = *(const double*)b;
  return (x > y) - (x < y);
}

/* Setup loop poiseuilleflow.f90:181-214: inverses of A_v and A_omega for every
 * (kx,ky) with kmn != 0.  The operators depend only on kmn, so one inverse per
 * distinct kmn value is computed (bitwise the same matrices). */
void orc_setup(orc* o) {
  const int Z = o->Z;
  free(o->t0); free(o->t1); free(o->t2); free(o->t4);
  o->t0 = (double*)calloc((size_t)Z * Z, sizeof(double));
  o->t1 = (double*)calloc((size_t)Z * Z, sizeof(double));
  o->t2 = (double*)calloc((size_t)Z * Z, sizeof(double));
  o->t4 = (double*)calloc((size_t)Z * Z, sizeof(double));
  scheb(o->nz, o->t0, o->t1, o->t2, o->t4);
  const int nm = (o->nhx + 1) * o->Y;
  double* ks = (double*)malloc(sizeof(double) * (size_t)nm);
  int c = 0;
  for (int i = 0; i <= o->nhx; ++i)
    for (int j = 0; j <= o->ny; ++j) {
      double kmn = o->iapha[i] * o->iapha[i] + o->ibeta[j] * o->ibeta[j];
      if (kmn != 0.0) ks[c++] = kmn;
    }
  qsort(ks, (size_t)c, sizeof(double), cmp_double);
  int u = 0;
  for (int t = 0; t < c; ++t)
    if (u == 0 || ks[t] != ks[u - 1]) ks[u++] = ks[t];
  free(o->k2vals); free(o->xv); free(o->xe); free(o->modek2);
  o->nk2 = u;
  o->k2vals = ks;
  o->xv = (double*)malloc(sizeof(double) * (size_t)u * Z * Z);
  o->xe = (double*)malloc(sizeof(double) * (size_t)u * Z * Z);
  o->modek2 = (int*)malloc(sizeof(int) * (size_t)nm);
  for (int i = 0; i <= o->nhx; ++i)
    for (int j = 0; j <= o->ny; ++j) {
      double kmn = o->iapha[i] * o->iapha[i] + o->ibeta[j] * o->ibeta[j];
      int id = -1;
      if (kmn != 0.0) {
        int lo = 0, hi = u - 1;
        while (lo <= hi) {
          int mid = (lo + hi) / 2;
          if (ks[mid] == kmn) { id = mid; break; }
          if (ks[mid] < kmn) lo = mid + 1; else hi = mid - 1;
        }
      }
      o->modek2[i * o->Y + j] = id;
    }
#pragma omp parallel
  {
    int* ipiv = (int*)malloc(sizeof(int) * (size_t)Z);
    double* work = (double*)malloc(sizeof(double) * (size_t)Z);
#pragma omp for schedule(dynamic)
    for (int t = 0; t < u; ++t) {
      double* xv = o->xv + (size_t)t * Z * Z;
      double* xe = o->xe + (size_t)t * Z * Z;
      get_coef_v(o, ks[t], xv);
      lu_inverse(xv, Z, ipiv, work);
      get_coef_omegay(o, ks[t], xe);
      lu_inverse(xe, Z, ipiv, work);
    }
    free(ipiv); free(work);
  }
  free(o->au0mat);
  o->au0mat = (double*)malloc(sizeof(double) * (size_t)Z * Z);
  get_coef_u0(o, o->au0mat);
  o->ready = 1;
}

static void ensure_scheb(orc* o) {
  if (o->t0) return;
  const int Z = o->Z;
  o->t0 = (double*)calloc((size_t)Z * Z, sizeof(double));
  o->t1 = (double*)calloc((size_t)Z * Z, sizeof(double));
  o->t2 = (double*)calloc((size_t)Z * Z, sizeof(double));
  o->t4 = (double*)calloc((size_t)Z * Z, sizeof(double));
  scheb(o->nz, o->t0, o->t1, o->t2, o->t4);
}

void orc_matrices(orc* o, double kmn, double* av, double* ae, double* xv, double* xe) {
  ensure_scheb(o);
  const int Z = o->Z;
  int* ipiv = (int*)malloc(sizeof(int) * (size_t)Z);
  double* work = (double*)malloc(sizeof(double) * (size_t)Z);
  get_coef_v(o, kmn, av);
  get_coef_omegay(o, kmn, ae);
  memcpy(xv, av, sizeof(double) * (size_t)Z * Z);
  memcpy(xe, ae, sizeof(double) * (size_t)Z * Z);
  lu_inverse(xv, Z, ipiv, work);
  lu_inverse(xe, Z, ipiv, work);
  free(ipiv); free(work);
}

/* ------------------------------------------------------------------------ */
/* dz, poiseuilleflow.f90:570-599: derivative of a Chebyshev series          */
/* ------------------------------------------------------------------------ */
void orc_dz(double* v, int n) {
  double dv[1024];
  double* d = (n + 1 <= 1024) ? dv : (double*)malloc(sizeof(double) * (size_t)(n + 1));
  for (int i = 0; i <= n; ++i) d[i] = 0.0;
  for (int i = 0; i <= n - 1; ++i)
    for (int j = i + 1; j <= n; ++j)
      if ((i + j) % 2 != 0) {
        if (i == 0) d[i] = d[i] + (double)j * v[j];
        else d[i] = d[i] + 2.0 * (double)j * v[j];
      }
  for (int i = 0; i <= n; ++i) v[i] = d[i];
  if (d != dv) free(d);
}

void orc_fft(int n, int sign, double* data) {
  fftplan p;
  plan_init(&p, n);
  cx* w = (cx*)malloc(sizeof(cx) * (size_t)n);
  fft_exec(&p, (cx*)data, w, sign);
  free(w);
  plan_free(&p);
}

/* ------------------------------------------------------------------------ */
/* ftrthreetotwo, poiseuilleflow.f90:1024-1185 (nproc = 1)                   */
/* spectral (X,Y,Z) <-> 3/2-padded physical wpp(0:PY-1, 0:PX-1, 0:nz)        */
/* ------------------------------------------------------------------------ */
static void ftr_to_phys(orc* o, const double* w, double* wpp) {
  const int KX = o->nnx / 2, nny = o->nny, PX = o->PX, PY = o->PY;
#pragma omp parallel
  {
    cx* g = (cx*)malloc(sizeof(cx) * (size_t)KX * PY); /* g[kx*PY + yp] */
    cx* line = (cx*)malloc(sizeof(cx) * (size_t)(PX > PY ? PX : PY));
    cx* work = (cx*)malloc(sizeof(cx) * (size_t)(PX > PY ? PX : PY));
#pragma omp for schedule(static)
    for (int k = 0; k <= o->nz; ++k) {
      /* y direction: expand(1) then backward FFT of length PY (REF:1051-1083) */
      for (int i = 0; i < KX; ++i) {
        cx* in = g + (size_t)i * PY;
        for (int t = 0; t < PY; ++t) { in[t].re = 0.0; in[t].im = 0.0; }
        for (int j = 0; j < nny / 2; ++j) {        /* j = nny/2 is zeroed */
          in[j].re = w[IDX(o, 2 * i, j, k)];
          in[j].im = w[IDX(o, 2 * i + 1, j, k)];
        }
        for (int j = 0; j <= nny / 2 - 2; ++j) {   /* negative modes */
          in[PY - 1 - j].re = w[IDX(o, 2 * i, nny - 1 - j, k)];
          in[PY - 1 - j].im = w[IDX(o, 2 * i + 1, nny - 1 - j, k)];
        }
        fft_exec(&o->ppy, in, work, +1);
      }
      /* transpose + x direction: getall, expand(1), backward FFT of length PX,
       * real part (REF:1089-1124) */
      for (int yp = 0; yp < PY; ++yp) {
        for (int t = 0; t < PX; ++t) { line[t].re = 0.0; line[t].im = 0.0; }
        for (int j = 0; j < KX; ++j) line[j] = g[(size_t)j * PY + yp];
        for (int j = 1; j <= KX - 1; ++j) {
          line[PX - j].re = g[(size_t)j * PY + yp].re;
          line[PX - j].im = -g[(size_t)j * PY + yp].im;
        }
        fft_exec(&o->ppx, line, work, +1);
        for (int xp = 0; xp < PX; ++xp)
          wpp[(size_t)yp + (size_t)PY * ((size_t)xp + (size_t)PX * k)] = line[xp].re;
      }
    }
    free(g); free(line); free(work);
  }
}

static void ftr_to_spec(orc* o, const double* wpp, double* w) {
  const int KX = o->nnx / 2, nny = o->nny, PX = o->PX, PY = o->PY;
  const double norm = (double)(PY * PX);
#pragma omp parallel
  {
    cx* g = (cx*)malloc(sizeof(cx) * (size_t)KX * PY);
    cx* line = (cx*)malloc(sizeof(cx) * (size_t)(PX > PY ? PX : PY));
    cx* work = (cx*)malloc(sizeof(cx) * (size_t)(PX > PY ? PX : PY));
#pragma omp for schedule(static)
    for (int k = 0; k <= o->nz; ++k) {
      /* x direction: forward FFT of the real rows, keep 0..nnx/2-1 (REF:1131-1145) */
      for (int yp = 0; yp < PY; ++yp) {
        for (int xp = 0; xp < PX; ++xp) {
          line[xp].re = wpp[(size_t)yp + (size_t)PY * ((size_t)xp + (size_t)PX * k)];
          line[xp].im = 0.0;
        }
        fft_exec(&o->ppx, line, work, -1);
        for (int j = 0; j < KX; ++j) g[(size_t)j * PY + yp] = line[j];
      }
      /* transpose + y direction: forward FFT of length PY, expand(-1) keeps
       * 0..nny/2 and the negative modes, then 1/(PY*PX) (REF:1152-1181) */
      for (int i = 0; i < KX; ++i) {
        cx* in = g + (size_t)i * PY;
        fft_exec(&o->ppy, in, work, -1);
        for (int j = 0; j <= nny / 2; ++j) {
          w[IDX(o, 2 * i, j, k)] = in[j].re / norm;
          w[IDX(o, 2 * i + 1, j, k)] = in[j].im / norm;
        }
        for (int j = 0; j <= nny / 2 - 2; ++j) {
          w[IDX(o, 2 * i, nny - 1 - j, k)] = in[PY - 1 - j].re / norm;
          w[IDX(o, 2 * i + 1, nny - 1 - j, k)] = in[PY - 1 - j].im / norm;
        }
      }
    }
    free(g); free(line); free(work);
  }
}

/* ------------------------------------------------------------------------ */
/* getlamb / getlamb1, poiseuilleflow.f90:1625-1712 / 1726-1815              */
/* ------------------------------------------------------------------------ */
void orc_getlamb(orc* o, const double* u, const double* omega, double* lamb, int with_rep) {
  const int PX = o->PX, PY = o->PY, mz = o->nz, amz = 2 * mz, mn = 2 * amz;
  ftr_to_phys(o, omega, o->omegap);
  ftr_to_phys(o, u, o->up);
  const size_t plane = (size_t)PX * PY;
  const double re_p = o->re_p;
#pragma omp parallel
  {
    cx* in = (cx*)malloc(sizeof(cx) * (size_t)mn);
    cx* work = (cx*)malloc(sizeof(cx) * (size_t)mn);
    double* tu = (double*)malloc(sizeof(double) * (size_t)(amz + 1));
    double* tw = (double*)malloc(sizeof(double) * (size_t)(amz + 1));
#pragma omp for schedule(static)
    for (long line = 0; line < (long)plane; ++line) {
      for (int k = 0; k <= amz; ++k) {
        if (k <= mz) {
          tu[k] = o->up[(size_t)line + plane * k];
          tw[k] = o->omegap[(size_t)line + plane * k];
        } else {
          tu[k] = 0.0; tw[k] = 0.0;
        }
      }
      for (int i = 0; i <= amz; ++i) {
        in[i].re = tu[i]; in[i].im = tw[i];
        if (i < amz - 1) { in[mn - 1 - i].re = tu[i + 1]; in[mn - 1 - i].im = tw[i + 1]; }
      }
      in[0].re *= 2.0; in[0].im *= 2.0;
      in[amz].re *= 2.0; in[amz].im *= 2.0;
      fft_exec(&o->p4z, in, work, -1);
      for (int i = 0; i <= amz; ++i) tu[i] = in[i].re * in[i].im / 4.0;
      if (with_rep)
        for (int i = 0; i <= amz; ++i) tu[i] = tu[i] - re_p;
      for (int i = 0; i <= amz; ++i) {
        in[i].re = tu[i]; in[i].im = 0.0;
        if (i < amz - 1) { in[mn - 1 - i].re = tu[i + 1]; in[mn - 1 - i].im = 0.0; }
      }
      fft_exec(&o->p4z, in, work, -1);
      for (int i = 0; i <= amz; ++i) tu[i] = in[i].re / (double)amz;
      tu[0] = tu[0] / 2.0;
      tu[amz] = tu[amz] / 2.0;
      for (int k = 0; k <= mz; ++k) o->up[(size_t)line + plane * k] = tu[k];
    }
    free(in); free(work); free(tu); free(tw);
  }
  ftr_to_spec(o, o->up, lamb);
}

/* z: Chebyshev coefficients -> values at z_k = cos(pi k/nz) for a packed pair,
 * with the 2nz FFT (poiseuilleflow.f90:1573-1609). */
static void coef_to_gl_pair(orc* o, double* a, double* b, size_t stride) {
  const int nz = o->nz, amz = 2 * nz;
  cx in[2048], work[2048];
  for (int i = 0; i <= nz; ++i) {
    in[i].re = a[stride * i]; in[i].im = b[stride * i];
    if (i < nz - 1) { in[amz - 1 - i].re = a[stride * (i + 1)]; in[amz - 1 - i].im = b[stride * (i + 1)]; }
  }
  in[0].re *= 2.0; in[0].im *= 2.0;
  in[nz].re *= 2.0; in[nz].im *= 2.0;
  fft_exec(&o->p2z, in, work, -1);
  for (int i = 0; i <= nz; ++i) { a[stride * i] = in[i].re / 2.0; b[stride * i] = in[i].im / 2.0; }
}

/* ------------------------------------------------------------------------ */
/* getnonlinear, poiseuilleflow.f90:1380-1612                                */
/* ------------------------------------------------------------------------ */
void orc_getnonlinear(orc* o) {
  double** f = o->f;
  double *u = f[ORC_UNP1], *v = f[ORC_VNP1], *w = f[ORC_WNP1];
  double *ox = f[ORC_OMEGAXNP1], *oy = f[ORC_OMEGAYNP1], *oz = f[ORC_OMEGAZNP1];
  double *lamb1 = o->lamb1, *lamb2 = o->lamb2;
  const size_t nf = (size_t)o->X * o->Y * o->Z;
  orc_getlamb(o, oy, w, lamb1, 1);            /* REF:1438-1439 */
  orc_getlamb(o, oz, v, lamb2, 0);            /* REF:1440-1441 */
  for (size_t t = 0; t < nf; ++t) lamb1[t] = lamb1[t] - lamb2[t];
  orc_getlamb(o, oz, u, lamb2, 0);            /* REF:1450 */
  orc_getlamb(o, ox, w, oz, 0);               /* REF:1452 */
  for (size_t t = 0; t < nf; ++t) lamb2[t] = lamb2[t] - oz[t];
  orc_getlamb(o, ox, v, oz, 0);               /* REF:1463 */
  orc_getlamb(o, oy, u, ox, 0);               /* REF:1465 */
  for (size_t t = 0; t < nf; ++t) oz[t] = oz[t] - ox[t];
  double* cl1nm1 = o->mean[ORC_CLAMB1NM1];
  double* cl3nm1 = o->mean[ORC_CLAMB3NM1];
  for (int k = 0; k <= o->nz; ++k) {          /* REF:1482-1487 */
    cl1nm1[2 * k] = lamb1[IDX(o, 0, 0, k)];
    cl3nm1[2 * k] = oz[IDX(o, 0, 0, k)];
    cl1nm1[2 * k + 1] = lamb1[IDX(o, 1, 0, k)];
    cl3nm1[2 * k + 1] = oz[IDX(o, 1, 0, k)];
  }
  memcpy(ox, lamb1, sizeof(double) * nf);     /* REF:1489-1496 */
  memcpy(u, lamb2, sizeof(double) * nf);
  /* curl / projection loop, REF:1502-1540 */
  const int nz = o->nz;
#pragma omp parallel for collapse(2) schedule(static)
  for (int i = 0; i <= o->nhx; ++i)
    for (int j = 0; j <= o->ny; ++j) {
      double tvn[1024], tvni[1024];
      const double a = o->iapha[i], b = o->ibeta[j];
      const double kmn = a * a + b * b;
      for (int kk = 0; kk <= nz; ++kk) { tvn[kk] = ox[IDX(o, 2 * i, j, kk)]; tvni[kk] = ox[IDX(o, 2 * i + 1, j, kk)]; }
      orc_dz(tvn, nz); orc_dz(tvni, nz);
      for (int k = 0; k <= nz; ++k) {
        size_t r = IDX(o, 2 * i, j, k), m = IDX(o, 2 * i + 1, j, k);
        u[r] = kmn * u[r] - a * tvni[k];
        u[m] = kmn * u[m] + a * tvn[k];
      }
      for (int kk = 0; kk <= nz; ++kk) { tvn[kk] = oz[IDX(o, 2 * i, j, kk)]; tvni[kk] = oz[IDX(o, 2 * i + 1, j, kk)]; }
      orc_dz(tvn, nz); orc_dz(tvni, nz);
      for (int k = 0; k <= nz; ++k) {
        size_t r = IDX(o, 2 * i, j, k), m = IDX(o, 2 * i + 1, j, k);
        u[r] = u[r] - b * tvni[k];
        u[m] = u[m] + b * tvn[k];
        w[r] = -1.0 * a * oz[m] + b * ox[m];
        w[m] = a * oz[r] - b * ox[r];
      }
    }
  /* history swap, REF:1542-1570 (values exchanged, buffers kept in place) */
  double* rv = f[ORC_RHSVN];
  double* rg = f[ORC_RHSOMEGAYN];
  for (size_t t = 0; t < nf; ++t) {
    double tmp = u[t]; u[t] = rv[t]; rv[t] = tmp;
    tmp = w[t]; w[t] = rg[t]; rg[t] = tmp;
  }
  double* cl1n = o->mean[ORC_CLAMB1N];
  double* cl3n = o->mean[ORC_CLAMB3N];
  for (int k = 0; k < 2 * (nz + 1); ++k) {
    double tmp = cl1nm1[k]; cl1nm1[k] = cl1n[k]; cl1n[k] = tmp;
    tmp = cl3nm1[k]; cl3nm1[k] = cl3n[k]; cl3n[k] = tmp;
  }
  /* coefficients -> Gauss-Lobatto values, REF:1573-1609 */
  const size_t zs = (size_t)o->X * o->Y;
#pragma omp parallel for schedule(static)
  for (long line = 0; line < (long)zs; ++line) coef_to_gl_pair(o, rv + line, rg + line, zs);
  coef_to_gl_pair(o, cl1n, cl3n, 2);
  coef_to_gl_pair(o, cl1n + 1, cl3n + 1, 2);
}

/* ------------------------------------------------------------------------ */
/* getvelocityandvorticity, poiseuilleflow.f90:2347-2407                     */
/* ------------------------------------------------------------------------ */
static void velocity_mode(orc* o, int i, int j) {
  const int nz = o->nz;
  double** f = o->f;
  double *u = f[ORC_UNP1], *v = f[ORC_VNP1], *w = f[ORC_WNP1];
  double *ox = f[ORC_OMEGAXNP1], *oy = f[ORC_OMEGAYNP1], *oz = f[ORC_OMEGAZNP1];
  const double a = o->iapha[i], b = o->ibeta[j], kmn = a * a + b * b;
  double dvr[1024], dvi[1024];
  for (int k = 0; k <= nz; ++k) { dvr[k] = v[IDX(o, 2 * i, j, k)]; dvi[k] = v[IDX(o, 2 * i + 1, j, k)]; }
  orc_dz(dvr, nz); orc_dz(dvi, nz);
  if (kmn == 0.0) return;
  for (int k = 0; k <= nz; ++k) {
    size_t r = IDX(o, 2 * i, j, k), m = IDX(o, 2 * i + 1, j, k);
    u[m] = a * dvr[k] / kmn - b * oy[r] / kmn;
    u[r] = -1.0 * a * dvi[k] / kmn + b * oy[m] / kmn;
    w[m] = b * dvr[k] / kmn + a * oy[r] / kmn;
    w[r] = -1.0 * dvi[k] * b / kmn - 1.0 * oy[m] * a / kmn;
  }
  for (int k = 0; k <= nz; ++k) { dvr[k] = w[IDX(o, 2 * i, j, k)]; dvi[k] = w[IDX(o, 2 * i + 1, j, k)]; }
  orc_dz(dvr, nz); orc_dz(dvi, nz);
  for (int k = 0; k <= nz; ++k) {
    size_t r = IDX(o, 2 * i, j, k), m = IDX(o, 2 * i + 1, j, k);
    ox[r] = dvr[k] + b * v[m];
    ox[m] = dvi[k] - b * v[r];
  }
  for (int k = 0; k <= nz; ++k) { dvr[k] = u[IDX(o, 2 * i, j, k)]; dvi[k] = u[IDX(o, 2 * i + 1, j, k)]; }
  orc_dz(dvr, nz); orc_dz(dvi, nz);
  for (int k = 0; k <= nz; ++k) {
    size_t r = IDX(o, 2 * i, j, k), m = IDX(o, 2 * i + 1, j, k);
    oz[r] = -dvr[k] - a * v[m];
    oz[m] = -dvi[k] + a * v[r];
  }
}

void orc_velocity_all(orc* o) {
#pragma omp parallel for collapse(2) schedule(static)
  for (int i = 0; i <= o->nhx; ++i)
    for (int j = 0; j <= o->ny; ++j) velocity_mode(o, i, j);
}

/* ------------------------------------------------------------------------ */
/* gsij, poiseuilleflow.f90:3540-3618: full-pivot Gauss elimination with a   */
/* real matrix and a complex right-hand side (re, im).  The reference caches */
/* the pivot order after the first call (ka = 1); the matrix is the same on  */
/* every call, so recomputing the pivots selects the same ones and performs  */
/* the same element updates.                                                  */
/* ------------------------------------------------------------------------ */
static void gsij(const double* a_in, double* fr, double* fi, int n1) {
  const int mz = n1 - 1;
  double* aa = (double*)malloc(sizeof(double) * (size_t)n1 * n1);
  double* xr = (double*)malloc(sizeof(double) * (size_t)n1);
  double* xi = (double*)malloc(sizeof(double) * (size_t)n1);
  int* ki = (int*)malloc(sizeof(int) * (size_t)n1);
  int* kj = (int*)malloc(sizeof(int) * (size_t)n1);
  int* ik = (int*)malloc(sizeof(int) * (size_t)n1);
  int* jk = (int*)malloc(sizeof(int) * (size_t)n1);
  memcpy(aa, a_in, sizeof(double) * (size_t)n1 * n1);
#define AA(i, j) aa[(size_t)(i) + (size_t)n1 * (size_t)(j)]
  for (int t = 0; t <= mz; ++t) { ki[t] = 1; kj[t] = 1; }
  int im = 0, jm = 0;
  for (int k = 0; k <= mz; ++k) {
    double dd = 0.0;
    for (int i = 0; i <= mz; ++i)
      if (ki[i] == 1)
        for (int j = 0; j <= mz; ++j) {
          double dq = fabs(AA(i, j));
          if (kj[j] == 1 && dq > dd) { dd = dq; im = i; jm = j; }
        }
    ik[k] = im; jk[k] = jm;
    kj[jm] = 0; ki[im] = 0;
    if (k == mz) break;
    double add = 1.0 / AA(im, jm);
    for (int i = 0; i <= mz; ++i)
      if (ki[i] == 1) {
        double as = AA(i, jm) * add;
        for (int j = 0; j <= mz; ++j)
          if (kj[j] == 1) AA(i, j) = AA(i, j) - as * AA(im, j);
        fr[i] = fr[i] - as * fr[im];
        fi[i] = fi[i] - as * fi[im];
      }
  }
  /* back substitution (REF:3606-3617); the solution is held in xr/xi by column */
  xr[jm] = fr[im] / AA(im, jm);
  xi[jm] = fi[im] / AA(im, jm);
  for (int k = mz - 1; k >= 0; --k) {
    int i = ik[k], j = jk[k];
    double sr = fr[i], si = fi[i];
    for (int lj = k + 1; lj <= mz; ++lj) {
      int jj = jk[lj];
      sr = sr - AA(i, jj) * xr[jj];
      si = si - AA(i, jj) * xi[jj];
    }
    xr[j] = sr / AA(i, j);
    xi[j] = si / AA(i, j);
  }
  for (int j = 0; j <= mz; ++j) { fr[j] = xr[j]; fi[j] = xi[j]; }
#undef AA
  free(aa); free(xr); free(xi); free(ki); free(kj); free(ik); free(jk);
}

/* ------------------------------------------------------------------------ */
/* Per-mode solve loop (REF:242-394) and the (0,0) mode (REF:401-474)        */
/* ------------------------------------------------------------------------ */
static void solve_mode(orc* o, int i, int j) {
  const int nz = o->nz, n = nz, Z = o->Z;
  const double dt = o->dt, re = o->re;
  double** f = o->f;
  double *v = f[ORC_VNP1], *oy = f[ORC_OMEGAYNP1], *u = f[ORC_UNP1], *w = f[ORC_WNP1];
  double *rv = f[ORC_RHSVN], *rg = f[ORC_RHSOMEGAYN];
  const double a = o->iapha[i], b = o->ibeta[j];
  const double kmn = a * a + b * b;
  const int kid = o->modek2[i * o->Y + j];
  double rhsr[1024], rhsi[1024], tvn[1024], tvni[1024], xr[1024], xi[1024];
  /* v equation (REF:253-330) */
  for (int k = 0; k <= nz; ++k) {
    size_t r = IDX(o, 2 * i, j, k), m = IDX(o, 2 * i + 1, j, k);
    rhsr[k] = (3.0 * dt / 2.0 * rv[r] - dt / 2.0 * u[r]) * 1.0;
    rhsi[k] = (3.0 * dt / 2.0 * rv[m] - dt / 2.0 * u[m]) * 1.0;
    tvn[k] = v[r]; tvni[k] = v[m];
  }
  double cr[1024], ci[1024];
  for (int ii = 4; ii <= n; ++ii) {             /* get_coef_rhs REF:3385-3425 */
    double sr = 0.0, si = 0.0;
    for (int jj = 0; jj <= n; ++jj) {
      size_t p = (size_t)(ii - 2) + (size_t)Z * jj;
      double tmpr = (o->t4[p] * dt * 0.5 / re + (1.0 - kmn * dt / re) * o->t2[p] -
                     kmn * (1.0 - kmn * dt * 0.5 / re) * o->t0[p]);
      sr = sr + tmpr * tvn[jj];
      si = si + tmpr * tvni[jj];
    }
    cr[ii] = rhsr[ii - 2] + sr;
    ci[ii] = rhsi[ii - 2] + si;
  }
  cr[0] = cr[1] = cr[2] = cr[3] = 0.0;
  ci[0] = ci[1] = ci[2] = ci[3] = 0.0;
  const double* X = o->xv + (size_t)kid * Z * Z;  /* a_multiply_x REF:4123-4139 */
  for (int ii = 0; ii <= n; ++ii) {
    double sr = 0.0, si = 0.0;
    for (int jj = 0; jj <= n; ++jj) {
      double x = X[(size_t)ii + (size_t)Z * jj];
      sr = sr + x * cr[jj];
      si = si + x * ci[jj];
    }
    xr[ii] = sr; xi[ii] = si;
  }
  for (int k = 0; k <= nz; ++k) {
    v[IDX(o, 2 * i, j, k)] = xr[k];
    v[IDX(o, 2 * i + 1, j, k)] = xi[k];
  }
  /* omega_y equation (REF:333-382) */
  for (int k = 0; k <= nz; ++k) {
    size_t r = IDX(o, 2 * i, j, k), m = IDX(o, 2 * i + 1, j, k);
    rhsr[k] = (3.0 * dt / 2.0 * rg[r] - dt / 2.0 * w[r]) * 1.0;
    rhsi[k] = (3.0 * dt / 2.0 * rg[m] - dt / 2.0 * w[m]) * 1.0;
    tvn[k] = oy[r]; tvni[k] = oy[m];
  }
  for (int ii = 2; ii <= n; ++ii) {             /* get_rhs_omegay REF:3458-3489 */
    double sr = 0.0, si = 0.0;
    for (int jj = 0; jj <= n; ++jj) {
      size_t p = (size_t)(ii - 1) + (size_t)Z * jj;
      double tmpr = o->t2[p] * dt * 0.5 / re + (1.0 - kmn * dt * 0.5 / re) * o->t0[p];
      sr = sr + tmpr * tvn[jj];
      si = si + tmpr * tvni[jj];
    }
    cr[ii] = sr + rhsr[ii - 1];
    ci[ii] = si + rhsi[ii - 1];
  }
  cr[0] = cr[1] = 0.0;
  ci[0] = ci[1] = 0.0;
  X = o->xe + (size_t)kid * Z * Z;
  for (int ii = 0; ii <= n; ++ii) {
    double sr = 0.0, si = 0.0;
    for (int jj = 0; jj <= n; ++jj) {
      double x = X[(size_t)ii + (size_t)Z * jj];
      sr = sr + x * cr[jj];
      si = si + x * ci[jj];
    }
    xr[ii] = sr; xi[ii] = si;
  }
  for (int k = 0; k <= nz; ++k) {
    oy[IDX(o, 2 * i, j, k)] = xr[k];
    oy[IDX(o, 2 * i + 1, j, k)] = xi[k];
  }
  velocity_mode(o, i, j);
}

static void solve_mean_one(orc* o, double* cln, double* clnm1, double* amean, double* vel,
                           double* vort, double vort_sign) {
  const int nz = o->nz, n = nz, Z = o->Z;
  const double dt = o->dt, re = o->re;
  double rhsr[1024], rhsi[1024], cr[1024], ci[1024];
  for (int k = 0; k <= nz; ++k) {
    rhsr[k] = -1.0 * dt / 2.0 * (3.0 * cln[2 * k] - clnm1[2 * k]);
    rhsi[k] = -1.0 * dt / 2.0 * (3.0 * cln[2 * k + 1] - clnm1[2 * k + 1]);
  }
  for (int ii = 2; ii <= n; ++ii) {             /* get_rhs_u0 REF:3515-3534 */
    double sr = 0.0, si = 0.0;
    for (int jj = 0; jj <= n; ++jj) {
      size_t p = (size_t)(ii - 1) + (size_t)Z * jj;
      double tmpr = o->t0[p] + dt * 0.5 / re * o->t2[p];
      sr = sr + tmpr * amean[2 * jj];
      si = si + tmpr * amean[2 * jj + 1];
    }
    cr[ii] = sr + rhsr[ii - 1];
    ci[ii] = si + rhsi[ii - 1];
  }
  cr[0] = cr[1] = 0.0;
  ci[0] = ci[1] = 0.0;
  gsij(o->au0mat, cr, ci, Z);
  for (int k = 0; k <= nz; ++k) {
    amean[2 * k] = cr[k];
    amean[2 * k + 1] = ci[k];
    vel[IDX(o, 0, 0, k)] = cr[k];
    vel[IDX(o, 1, 0, k)] = ci[k];
  }
  orc_dz(cr, nz); orc_dz(ci, nz);
  for (int k = 0; k <= nz; ++k) {
    vort[IDX(o, 0, 0, k)] = vort_sign * cr[k];
    vort[IDX(o, 1, 0, k)] = vort_sign * ci[k];
  }
}

void orc_solve(orc* o) {
  if (!o->ready) orc_setup(o);
#pragma omp parallel for collapse(2) schedule(dynamic, 4)
  for (int i = 0; i <= o->nhx; ++i)
    for (int j = 0; j <= o->ny; ++j) {
      double kmn = o->iapha[i] * o->iapha[i] + o->ibeta[j] * o->ibeta[j];
      if (j == (o->ny + 1) / 2 || kmn == 0.0) continue;
      solve_mode(o, i, j);
    }
  double** f = o->f;
  solve_mean_one(o, o->mean[ORC_CLAMB1N], o->mean[ORC_CLAMB1NM1], o->mean[ORC_AU0],
                 f[ORC_UNP1], f[ORC_OMEGAZNP1], -1.0);
  solve_mean_one(o, o->mean[ORC_CLAMB3N], o->mean[ORC_CLAMB3NM1], o->mean[ORC_W0],
                 f[ORC_WNP1], f[ORC_OMEGAXNP1], 1.0);
}

void orc_step(orc* o, int nsteps) {
  for (int s = 0; s < nsteps; ++s) {
    orc_getnonlinear(o);
    orc_solve(o);
  }
}

/* ------------------------------------------------------------------------ */
/* transform, poiseuilleflow.f90:919-1005, with fourtrx_zcomp (774-913)      */
/* ------------------------------------------------------------------------ */
void orc_transform(orc* o, int isign, double* u) {
  const int nnx = o->nnx, nny = o->nny, KX = nnx / 2, nz = o->nz, mn = 2 * nz;
  const size_t zs = (size_t)o->X * o->Y;
  if (isign == 1) {
    /* fourtrx_zcomp(1): y backward FFT (Nyquist zeroed), x Hermitian fill +
     * backward FFT, real part (REF:782-865) */
#pragma omp parallel
    {
      cx* g = (cx*)malloc(sizeof(cx) * (size_t)KX * nny);
      cx* line = (cx*)malloc(sizeof(cx) * (size_t)(nnx > nny ? nnx : nny));
      cx* work = (cx*)malloc(sizeof(cx) * (size_t)(nnx > nny ? nnx : nny));
#pragma omp for
      for (int k = 0; k <= nz; ++k) {
        for (int i = 0; i < KX; ++i) {
          cx* in = g + (size_t)i * nny;
          for (int j = 0; j < nny; ++j) { in[j].re = u[IDX(o, 2 * i, j, k)]; in[j].im = u[IDX(o, 2 * i + 1, j, k)]; }
          in[nny / 2].re = 0.0; in[nny / 2].im = 0.0;
          fft_exec(&o->pny, in, work, +1);
        }
        for (int y = 0; y < nny; ++y) {
          for (int j = 0; j < KX; ++j) line[j] = g[(size_t)j * nny + y];
          line[KX].re = 0.0; line[KX].im = 0.0;
          for (int j = 1; j <= KX - 1; ++j) { line[nnx - j].re = line[j].re; line[nnx - j].im = -line[j].im; }
          fft_exec(&o->pnnx, line, work, +1);
          for (int x = 0; x < nnx; ++x) u[IDX(o, x, y, k)] = line[x].re;
        }
      }
      free(g); free(line); free(work);
    }
    /* z: coefficients -> values (REF:940-962) */
#pragma omp parallel
    {
      cx* in = (cx*)malloc(sizeof(cx) * (size_t)mn);
      cx* work = (cx*)malloc(sizeof(cx) * (size_t)mn);
#pragma omp for
      for (long line = 0; line < (long)zs; ++line) {
        for (int i = 0; i <= nz; ++i) {
          in[i].re = u[(size_t)line + zs * i]; in[i].im = 0.0;
          if (i < nz - 1) { in[mn - 1 - i].re = u[(size_t)line + zs * (i + 1)]; in[mn - 1 - i].im = 0.0; }
        }
        in[0].re *= 2.0; in[0].im *= 2.0; in[nz].re *= 2.0; in[nz].im *= 2.0;
        fft_exec(&o->p2z, in, work, -1);
        for (int i = 0; i <= nz; ++i) u[(size_t)line + zs * i] = in[i].re / 2.0;
      }
      free(in); free(work);
    }
  } else {
    /* z: values -> coefficients (REF:971-1001) */
#pragma omp parallel
    {
      cx* in = (cx*)malloc(sizeof(cx) * (size_t)mn);
      cx* work = (cx*)malloc(sizeof(cx) * (size_t)mn);
#pragma omp for
      for (long line = 0; line < (long)zs; ++line) {
        for (int i = 0; i <= nz; ++i) {
          in[i].re = u[(size_t)line + zs * i]; in[i].im = 0.0;
          if (i < nz - 1) { in[mn - 1 - i].re = u[(size_t)line + zs * (i + 1)]; in[mn - 1 - i].im = 0.0; }
        }
        fft_exec(&o->p2z, in, work, -1);
        double t[2048];
        for (int i = 0; i <= nz; ++i) t[i] = in[i].re / (double)nz;
        t[0] = t[0] / 2.0; t[nz] = t[nz] / 2.0;
        for (int i = 0; i <= nz; ++i) u[(size_t)line + zs * i] = t[i];
      }
      free(in); free(work);
    }
    /* fourtrx_zcomp(-1): x forward FFT keep 0..nnx/2-1, y forward FFT, then
     * 1/(nnx*nny) (REF:868-911) */
    const double norm = (double)(nnx * nny);
#pragma omp parallel
    {
      cx* g = (cx*)malloc(sizeof(cx) * (size_t)KX * nny);
      cx* line = (cx*)malloc(sizeof(cx) * (size_t)(nnx > nny ? nnx : nny));
      cx* work = (cx*)malloc(sizeof(cx) * (size_t)(nnx > nny ? nnx : nny));
#pragma omp for
      for (int k = 0; k <= nz; ++k) {
        for (int y = 0; y < nny; ++y) {
          for (int x = 0; x < nnx; ++x) { line[x].re = u[IDX(o, x, y, k)]; line[x].im = 0.0; }
          fft_exec(&o->pnnx, line, work, -1);
          for (int j = 0; j < KX; ++j) g[(size_t)j * nny + y] = line[j];
        }
        for (int i = 0; i < KX; ++i) {
          cx* in = g + (size_t)i * nny;
          fft_exec(&o->pny, in, work, -1);
          for (int j = 0; j < nny; ++j) {
            u[IDX(o, 2 * i, j, k)] = in[j].re / norm;
            u[IDX(o, 2 * i + 1, j, k)] = in[j].im / norm;
          }
        }
      }
      free(g); free(line); free(work);
    }
  }
}
