/*
 * icep_oracle.c -- CPU FP64 restatement of the KAPSEL-ICEP per-timestep hot
 * path. TEST INFRASTRUCTURE ONLY: it is the checker for the GPU library (the
 * tests, __graft_entry__.smoke() and bench.py's cpu_baseline leg load it);
 * nothing in the product links or calls it.
 *
 * Parity of this restatement is pinned against the reference's own object
 * code (oracle/ref builds it from the reference sources) through the golden
 * fixtures in tests/golden, generated by tests/golden/make_golden.py.
 *
 * Every function cites the reference function it restates (file:line, paths
 * inside the reference project). Arithmetic is FP64 throughout; loops are
 * written for clarity and OpenMP-parallel over independent grid planes.
 *
 * Data layout: fields are double[NX][NY][NZ_], NZ_ = 2*(NZ/2+1); k-space
 * values are (re,im) pairs, kz = 0..NZ/2 (fft_wrapper.h:681-723).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/icep_types.h"

#define DIM 3
#define SQ(x) ((x) * (x))

/* ------------------------------------------------------------------------ */
/* 1D complex FFT (iterative radix-2, forward kernel exp(-2 pi i jk/n)).     */
/* ------------------------------------------------------------------------ */
typedef struct {
  int n;
  double *tw; /* n/2 complex: exp(-2 pi i k / n) */
  int *rev;
} cplan;

static void cplan_init(cplan *p, int n) {
  p->n = n;
  p->tw = (double *)malloc(sizeof(double) * 2 * (n / 2 > 0 ? n / 2 : 1));
  p->rev = (int *)malloc(sizeof(int) * n);
  for (int k = 0; k < n / 2; k++) {
    double a = -2.0 * M_PI * (double)k / (double)n;
    p->tw[2 * k] = cos(a);
    p->tw[2 * k + 1] = sin(a);
  }
  int lg = 0;
  while ((1 << lg) < n) lg++;
  for (int i = 0; i < n; i++) {
    int r = 0;
    for (int b = 0; b < lg; b++)
      if (i & (1 << b)) r |= 1 << (lg - 1 - b);
    p->rev[i] = r;
  }
}

static void cplan_free(cplan *p) {
  free(p->tw);
  free(p->rev);
}

/* in-place on a[2n] (interleaved). inverse: kernel exp(+...), unnormalised */
static void cfft(const cplan *p, double *a, int inverse) {
  const int n = p->n;
  for (int i = 0; i < n; i++) {
    int r = p->rev[i];
    if (r > i) {
      double t0 = a[2 * i], t1 = a[2 * i + 1];
      a[2 * i] = a[2 * r];
      a[2 * i + 1] = a[2 * r + 1];
      a[2 * r] = t0;
      a[2 * r + 1] = t1;
    }
  }
  const double sgn = inverse ? -1.0 : 1.0;
  for (int len = 2; len <= n; len <<= 1) {
    const int half = len >> 1, step = n / len;
    for (int s = 0; s < n; s += len) {
      for (int k = 0; k < half; k++) {
        double wr = p->tw[2 * k * step], wi = sgn * p->tw[2 * k * step + 1];
        double *x0 = a + 2 * (s + k), *x1 = a + 2 * (s + k + half);
        double tr = x1[0] * wr - x1[1] * wi;
        double ti = x1[0] * wi + x1[1] * wr;
        x1[0] = x0[0] - tr;
        x1[1] = x0[1] - ti;
        x0[0] += tr;
        x0[1] += ti;
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Context                                                                  */
/* ------------------------------------------------------------------------ */
enum {
  F_ZETA0 = 0, F_ZETA1, F_U0, F_U1, F_U2, F_UP0, F_UP1, F_UP2, F_PHI, F_PHI_SUM,
  F_F0, F_F1, F_F2, F_POT, F_EPS, F_GE0, F_GE1, F_GE2, F_C0, F_C1, F_RHO, F_WORK,
  F_SN0, F_SN1, F_SN2, F_NS0_0, F_NS0_1, F_NS1_0, F_NS1_1, F_CRHS0, F_CRHS1,
  F_WV1, F_WV3_0, F_WV3_1, F_WV3_2, F_COUNT
};

typedef struct {
  icep_params P;
  int nx, ny, nz, nzp, hnz;
  int trn[3];
  long nf;  /* NX*NY*NZ_ */
  long nu;  /* NX*NY*NZ  */
  double dx, dx3, wave[3], radius, xi, hxi, sigma, lj_dia, r_cutoff, nu_visc;
  double imass[ICEP_MAX_SPECIES], imoi[ICEP_MAX_SPECIES];
  double valency_e[2], onsager[2];
  int np_domain;
  int *sekibun;
  int np;
  icep_particle *p;
  double *f[F_COUNT];
  double uk_dc[3];
  int ts;
  double time;
  cplan px, py, pz; /* x: NX, y: NY, z: NZ/2 (half-length for the real transform) */
  double *ztw;      /* z post-twiddles exp(-2 pi i k/NZ), k = 0..NZ/2 */
  /* Poisson statistics */
  long last_iters;
  double last_error;
  long matvecs;
  double total_solute[2];
  long pb_iterations; /* relaxation steps of the last Poisson-Boltzmann initialisation */
} ko_ctx;

#define IDX(c, i, j, k) (((long)(i) * (c)->ny + (j)) * (c)->nzp + (k))

static double *zalloc(long n) {
  double *p = (double *)calloc((size_t)n, sizeof(double));
  return p;
}

/* signed wavenumber index: Calc_KX_Ooura etc. (fft_wrapper.h:761-773) */
static inline int kx_of(const ko_ctx *c, int i) { return (i > c->nx / 2) ? i - c->nx : i; }
static inline int ky_of(const ko_ctx *c, int j) { return (j > c->ny / 2) ? j - c->ny : j; }

/* ------------------------------------------------------------------------ */
/* 3D real FFT with the reference's conventions                             */
/* ------------------------------------------------------------------------ */

/* A2a_k (fft_wrapper.h:681-693): forward real DFT, kernel exp(-i k.r),
 * unnormalised, in place on [NX][NY][NZ_]. */
static void fft_r2c(ko_ctx *c, double *a) {
  const int nx = c->nx, ny = c->ny, nz = c->nz, h = nz / 2;
  /* z: real transform of each row via an NZ/2-point complex FFT */
#pragma omp parallel for schedule(static)
  for (int ij = 0; ij < nx * ny; ij++) {
    double *row = a + (long)ij * c->nzp;
    double buf[2 * 2048];
    for (int n = 0; n < h; n++) {
      buf[2 * n] = row[2 * n];
      buf[2 * n + 1] = row[2 * n + 1];
    }
    cfft(&c->pz, buf, 0);
    for (int k = 0; k <= h; k++) {
      int k1 = k % h, k2 = (h - k) % h;
      double zr = buf[2 * k1], zi = buf[2 * k1 + 1];
      double cr = buf[2 * k2], ci = -buf[2 * k2 + 1];
      double er = 0.5 * (zr + cr), ei = 0.5 * (zi + ci);
      double dr = zr - cr, di = zi - ci;
      /* O = d / (2i) */
      double or_ = 0.5 * di, oi = -0.5 * dr;
      double wr = c->ztw[2 * k], wi = c->ztw[2 * k + 1];
      row[2 * k] = er + (wr * or_ - wi * oi);
      row[2 * k + 1] = ei + (wr * oi + wi * or_);
    }
  }
  /* y: complex transform of each (i, kz) column */
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nx; i++) {
    double buf[2 * 2048];
    for (int k = 0; k <= h; k++) {
      for (int j = 0; j < ny; j++) {
        buf[2 * j] = a[IDX(c, i, j, 2 * k)];
        buf[2 * j + 1] = a[IDX(c, i, j, 2 * k + 1)];
      }
      cfft(&c->py, buf, 0);
      for (int j = 0; j < ny; j++) {
        a[IDX(c, i, j, 2 * k)] = buf[2 * j];
        a[IDX(c, i, j, 2 * k + 1)] = buf[2 * j + 1];
      }
    }
  }
  /* x: complex transform of each (j, kz) column */
#pragma omp parallel for schedule(static)
  for (int j = 0; j < ny; j++) {
    double buf[2 * 2048];
    for (int k = 0; k <= h; k++) {
      for (int i = 0; i < nx; i++) {
        buf[2 * i] = a[IDX(c, i, j, 2 * k)];
        buf[2 * i + 1] = a[IDX(c, i, j, 2 * k + 1)];
      }
      cfft(&c->px, buf, 0);
      for (int i = 0; i < nx; i++) {
        a[IDX(c, i, j, 2 * k)] = buf[2 * i];
        a[IDX(c, i, j, 2 * k + 1)] = buf[2 * i + 1];
      }
    }
  }
}

/*
 * The reference's inverse (A_k2a, fft_wrapper.h:704-718: conj, scale 2/N,
 * rdft3dsort(-1), rdft3d(-1)) reads only half of the kz = 0 and kz = NZ/2
 * planes: rdft3dsort (fftsg3d.c:645-667) packs, for kz = 0, the entries with
 * 1 <= j <= NY/2-1 (all i) and with j in {0, NY/2}, i <= NX/2; the kz = NZ/2
 * plane keeps the complementary half (j >= NY/2+1, and j in {0,NY/2} with
 * i > NX/2). At the four self-conjugate points only the real part survives.
 * The dropped half is implied by Hermitian symmetry X(-k) = conj X(k).
 * herm_project rewrites both planes into that Hermitian completion, after
 * which any exact real inverse DFT reproduces the reference.
 */
static int kept_kz0(const ko_ctx *c, int i, int j) {
  if (j >= 1 && j <= c->ny / 2 - 1) return 1;
  if (j == 0 || j == c->ny / 2) return i <= c->nx / 2;
  return 0;
}

static void herm_project(ko_ctx *c, double *a) {
  const int nx = c->nx, ny = c->ny, h = c->nz / 2;
  for (int plane = 0; plane < 2; plane++) {
    int kz = plane ? h : 0;
    for (int i = 0; i < nx; i++) {
      for (int j = 0; j < ny; j++) {
        int mi = (nx - i) % nx, mj = (ny - j) % ny;
        int kept = kept_kz0(c, i, j);
        if (plane) kept = !kept;
        long at = IDX(c, i, j, 2 * kz);
        if (mi == i && mj == j) {
          a[at + 1] = 0.0;
        } else if (!kept) {
          long m = IDX(c, mi, mj, 2 * kz);
          a[at] = a[m];
          a[at + 1] = -a[m + 1];
        }
      }
    }
  }
}

/* A_k2a (fft_wrapper.h:704-718): inverse with 1/N normalisation, in place. */
static void fft_c2r(ko_ctx *c, double *a) {
  const int nx = c->nx, ny = c->ny, nz = c->nz, h = nz / 2;
  herm_project(c, a);
#pragma omp parallel for schedule(static)
  for (int j = 0; j < ny; j++) {
    double buf[2 * 2048];
    for (int k = 0; k <= h; k++) {
      for (int i = 0; i < nx; i++) {
        buf[2 * i] = a[IDX(c, i, j, 2 * k)];
        buf[2 * i + 1] = a[IDX(c, i, j, 2 * k + 1)];
      }
      cfft(&c->px, buf, 1);
      for (int i = 0; i < nx; i++) {
        a[IDX(c, i, j, 2 * k)] = buf[2 * i];
        a[IDX(c, i, j, 2 * k + 1)] = buf[2 * i + 1];
      }
    }
  }
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nx; i++) {
    double buf[2 * 2048];
    for (int k = 0; k <= h; k++) {
      for (int j = 0; j < ny; j++) {
        buf[2 * j] = a[IDX(c, i, j, 2 * k)];
        buf[2 * j + 1] = a[IDX(c, i, j, 2 * k + 1)];
      }
      cfft(&c->py, buf, 1);
      for (int j = 0; j < ny; j++) {
        a[IDX(c, i, j, 2 * k)] = buf[2 * j];
        a[IDX(c, i, j, 2 * k + 1)] = buf[2 * j + 1];
      }
    }
  }
  const double scale = 1.0 / ((double)nx * ny * nz);
#pragma omp parallel for schedule(static)
  for (int ij = 0; ij < nx * ny; ij++) {
    double *row = a + (long)ij * c->nzp;
    double buf[2 * 2048];
    row[1] = 0.0;
    row[2 * h + 1] = 0.0;
    for (int k = 0; k < h; k++) {
      int k2 = h - k;
      double xr = row[2 * k], xi = row[2 * k + 1];
      double cr = row[2 * k2], ci = -row[2 * k2 + 1];
      double sr = xr + cr, si = xi + ci;
      double dr = xr - cr, di = xi - ci;
      /* w = exp(+2 pi i k / NZ) = conj(ztw) */
      double wr = c->ztw[2 * k], wi = -c->ztw[2 * k + 1];
      double tr = wr * dr - wi * di, ti = wr * di + wi * dr;
      /* Z = s + i t */
      buf[2 * k] = sr - ti;
      buf[2 * k + 1] = si + tr;
    }
    cfft(&c->pz, buf, 1);
    for (int n = 0; n < h; n++) {
      row[2 * n] = buf[2 * n] * scale;
      row[2 * n + 1] = buf[2 * n + 1] * scale;
    }
    row[nz] = 0.0;
    row[nz + 1] = 0.0;
  }
}

/* ------------------------------------------------------------------------ */
/* k-space operators                                                        */
/* ------------------------------------------------------------------------ */

/* real wavenumbers of the complex mode (i, j, kz) */
static inline void kvec(const ko_ctx *c, int i, int j, int kz, double *k) {
  k[0] = c->wave[0] * (double)kx_of(c, i);
  k[1] = c->wave[1] * (double)ky_of(c, j);
  k[2] = c->wave[2] * (double)kz;
}
/* K2 and IK2 of Init_K (fft_wrapper.cxx:47-87) */
static inline double k2_of(const ko_ctx *c, int i, int j, int kz) {
  return SQ(c->wave[0] * (double)kx_of(c, i)) + SQ(c->wave[1] * (double)ky_of(c, j)) +
         SQ(c->wave[2] * (double)kz);
}
static inline double ik2_of(const ko_ctx *c, int i, int j, int kz) {
  double k2 = k2_of(c, i, j, kz);
  return (k2 > 0.0) ? 1. / k2 : 0.0;
}

/* Inside the dealiasing region |kx| < TRN_X, |ky| < TRN_Y, kz < TRN_Z: the
 * union of the four 2/3-rule boxes (fft_wrapper.cxx:185-197) and the
 * complement of what Truncate_two_third_rule_ooura zeroes (fft_wrapper.h:797-839). */
static inline int in_two_third(const ko_ctx *c, int i, int j, int kz) {
  int ax = (i <= c->nx / 2) ? i : c->nx - i;
  int ay = (j <= c->ny / 2) ? j : c->ny - j;
  return ax < c->trn[0] && ay < c->trn[1] && kz < c->trn[2];
}

/* Truncate_two_third_rule_ooura (fft_wrapper.h:797-839) */
static void truncate_23(ko_ctx *c, double *a) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int kz = 0; kz < c->hnz; kz++)
        if (!in_two_third(c, i, j, kz)) {
          a[IDX(c, i, j, 2 * kz)] = 0.0;
          a[IDX(c, i, j, 2 * kz + 1)] = 0.0;
        }
}

/* Zeta_k2u_k (fft_wrapper.cxx:614-711): reduced vorticity -> solenoidal
 * velocity in k-space; u(k=0) real part = uk_dc. */
static void zeta_k2u_k(ko_ctx *c, double *const *zeta, const double *uk_dc, double **u) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int kz = 0; kz < c->hnz; kz++) {
        long im = IDX(c, i, j, 2 * kz);
        int KX = kx_of(c, i), KY = ky_of(c, j);
        double kx = c->wave[0] * KX, ky = c->wave[1] * KY, kz_ = c->wave[2] * kz;
        double ik2 = ik2_of(c, i, j, kz);
        double z1r = zeta[0][im], z1i = zeta[0][im + 1];
        double z2r = zeta[1][im], z2i = zeta[1][im + 1];
        double wr[3], wi[3];
        if (KX != 0) {
          wr[0] = -(1. / kx) * (ky * z1r + kz_ * z2r);
          wi[0] = -(1. / kx) * (ky * z1i + kz_ * z2i);
          wr[1] = z1r; wi[1] = z1i;
          wr[2] = z2r; wi[2] = z2i;
        } else if (KY != 0) {
          double r = -(kz_ / ky);
          wr[0] = z2r; wi[0] = z2i;
          wr[1] = r * z1r; wi[1] = r * z1i;
          wr[2] = z1r; wi[2] = z1i;
        } else {
          wr[0] = z1r; wi[0] = z1i;
          wr[1] = z2r; wi[1] = z2i;
          wr[2] = 0.0; wi[2] = 0.0;
        }
        kx *= ik2; ky *= ik2; kz_ *= ik2;
        u[0][im] = -(ky * wi[2] - kz_ * wi[1]);
        u[0][im + 1] = (ky * wr[2] - kz_ * wr[1]);
        u[1][im] = -(kz_ * wi[0] - kx * wi[2]);
        u[1][im + 1] = (kz_ * wr[0] - kx * wr[2]);
        u[2][im] = -(kx * wi[1] - ky * wi[0]);
        u[2][im + 1] = (kx * wr[1] - ky * wr[0]);
      }
  for (int d = 0; d < DIM; d++) u[d][0] = uk_dc[d];
}

/* U_k2zeta_k (fft_wrapper.cxx:428-497) */
static void u_k2zeta_k(ko_ctx *c, double *const *u, double **zeta, double *uk_dc) {
  for (int d = 0; d < DIM; d++) uk_dc[d] = u[d][0];
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int kz = 0; kz < c->hnz; kz++) {
        long im = IDX(c, i, j, 2 * kz);
        double k[3];
        kvec(c, i, j, kz, k);
        double wr[3], wi[3];
        wr[0] = -(k[1] * u[2][im + 1] - k[2] * u[1][im + 1]);
        wi[0] = (k[1] * u[2][im] - k[2] * u[1][im]);
        wr[1] = -(k[2] * u[0][im + 1] - k[0] * u[2][im + 1]);
        wi[1] = (k[2] * u[0][im] - k[0] * u[2][im]);
        wr[2] = -(k[0] * u[1][im + 1] - k[1] * u[0][im + 1]);
        wi[2] = (k[0] * u[1][im] - k[1] * u[0][im]);
        int a, b;
        if (kx_of(c, i) != 0) { a = 1; b = 2; }
        else if (ky_of(c, j) != 0) { a = 2; b = 0; }
        else { a = 0; b = 1; }
        zeta[0][im] = wr[a]; zeta[0][im + 1] = wi[a];
        zeta[1][im] = wr[b]; zeta[1][im + 1] = wi[b];
      }
}

/* U2advection_k (operate_omega.cxx:12-98) followed by Omega_k2zeta_k
 * (fft_wrapper.cxx:248-284). u: real-space velocity on input, scratch on
 * output. adv: reduced advection term (k-space), 2 fields. */
static void u2advection_k(ko_ctx *c, double **u, double **adv) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nz; k++) {
        long im = IDX(c, i, j, k);
        double u1 = u[0][im], u2 = u[1][im], u3 = u[2][im];
        u[0][im] = u2 * u3;
        u[1][im] = u3 * u1;
        u[2][im] = u1 * u2;
        adv[0][im] = (u2 - u3) * (u2 + u3);
        adv[1][im] = (u3 - u1) * (u3 + u1);
      }
  for (int d = 0; d < DIM; d++) fft_r2c(c, u[d]);
  fft_r2c(c, adv[0]);
  fft_r2c(c, adv[1]);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nzp; k++) {
        long im = IDX(c, i, j, k);
        double kv[3];
        kvec(c, i, j, k / 2, kv);
        double k1 = kv[0], k2 = kv[1], k3 = kv[2];
        double u2u3 = u[0][im], u3u1 = u[1][im], u1u2 = u[2][im];
        double u22_u32 = adv[0][im], u32_u12 = adv[1][im];
        double u12_u22 = -u32_u12 - u22_u32;
        double k1k2 = k1 * k2, k2k3 = k2 * k3, k3k1 = k3 * k1;
        double o0 = -(k2k3 * u22_u32 + (k3 - k2) * (k3 + k2) * u2u3 + k3k1 * u1u2 - k1k2 * u3u1);
        double o1 = -(k3k1 * u32_u12 + (k1 - k3) * (k1 + k3) * u3u1 + k1k2 * u2u3 - k2k3 * u1u2);
        double o2 = -(k1k2 * u12_u22 + (k2 - k1) * (k2 + k1) * u1u2 + k2k3 * u3u1 - k3k1 * u2u3);
        u[0][im] = o0; u[1][im] = o1; u[2][im] = o2;
        if (kx_of(c, i) != 0) { adv[0][im] = o1; adv[1][im] = o2; }
        else if (ky_of(c, j) != 0) { adv[0][im] = o2; adv[1][im] = o0; }
        else { adv[0][im] = o0; adv[1][im] = o1; }
      }
}

/* Solenoidal_uk (operate_omega.cxx:187-220) */
static void solenoidal_uk(ko_ctx *c, double **u) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nzp; k++) {
        long im = IDX(c, i, j, k);
        double kv[3];
        kvec(c, i, j, k / 2, kv);
        double r = ik2_of(c, i, j, k / 2) * (u[0][im] * kv[0] + u[1][im] * kv[1] + u[2][im] * kv[2]);
        u[0][im] -= r * kv[0];
        u[1][im] -= r * kv[1];
        u[2][im] -= r * kv[2];
      }
}

/* Solenoidal_u (operate_omega.h:109-116) */
static void solenoidal_u(ko_ctx *c, double **u) {
  for (int d = 0; d < DIM; d++) fft_r2c(c, u[d]);
  for (int d = 0; d < DIM; d++) truncate_23(c, u[d]);
  solenoidal_uk(c, u);
  for (int d = 0; d < DIM; d++) fft_c2r(c, u[d]);
}

/* A_k2dja_k_primitive (fft_wrapper.cxx:214-237): da = i k_d a */
static void a_k2da_k(ko_ctx *c, const double *a, double **da) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int kz = 0; kz < c->hnz; kz++) {
        long im = IDX(c, i, j, 2 * kz);
        double kv[3];
        kvec(c, i, j, kz, kv);
        double re = a[im], imv = a[im + 1];
        for (int d = 0; d < DIM; d++) {
          da[d][im] = -kv[d] * imv;
          da[d][im + 1] = kv[d] * re;
        }
      }
}

/* staggered-grid shift exp(i dx k_d / 2) (Init_K, fft_wrapper.cxx:80-82) */
static inline void shift_of(const ko_ctx *c, double kd, double *sr, double *si) {
  double a = 0.5 * c->dx * kd;
  *sr = cos(a);
  *si = sin(a);
}

/* Shift_vec_fw_imag (fft_wrapper.h:841-858): v_d *= exp(+i dx k_d / 2) */
static void shift_fw(ko_ctx *c, double **v) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int kz = 0; kz < c->hnz; kz++) {
        long im = IDX(c, i, j, 2 * kz);
        double kv[3];
        kvec(c, i, j, kz, kv);
        for (int d = 0; d < DIM; d++) {
          double sr, si;
          shift_of(c, kv[d], &sr, &si);
          double re = v[d][im], imv = v[d][im + 1];
          v[d][im] = re * sr - imv * si;
          v[d][im + 1] = re * si + imv * sr;
        }
      }
}

/* U_k2divergence_k (fft_wrapper.cxx:896-920) */
static void u_k2divergence_k(ko_ctx *c, double *const *u, double *div) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int kz = 0; kz < c->hnz; kz++) {
        long im = IDX(c, i, j, 2 * kz);
        double kv[3];
        kvec(c, i, j, kz, kv);
        double re = -(kv[0] * u[0][im + 1] + kv[1] * u[1][im + 1] + kv[2] * u[2][im + 1]);
        double imv = (kv[0] * u[0][im] + kv[1] * u[1][im] + kv[2] * u[2][im]);
        div[im] = re;
        div[im + 1] = imv;
      }
}

/* U_k2divergence_k_shift (fft_wrapper.h:879-900):
 * div = i sum_d k_d conj(shift_d) u_d */
static void u_k2divergence_k_shift(ko_ctx *c, double *const *u, double *div) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int kz = 0; kz < c->hnz; kz++) {
        long im = IDX(c, i, j, 2 * kz);
        double kv[3];
        kvec(c, i, j, kz, kv);
        double sr_ = 0.0, si_ = 0.0;
        for (int d = 0; d < DIM; d++) {
          double sr, si;
          shift_of(c, kv[d], &sr, &si);
          /* ks = k_d conj(shift) */
          double ksr = kv[d] * sr, ksi = -kv[d] * si;
          double ur = u[d][im], ui = u[d][im + 1];
          sr_ += ur * ksr - ui * ksi;
          si_ += ur * ksi + ui * ksr;
        }
        div[im] = -si_;
        div[im + 1] = sr_;
      }
}

/* ------------------------------------------------------------------------ */
/* Navier-Stokes                                                            */
/* ------------------------------------------------------------------------ */

/* Zeta_k2u (operate_omega.h:138-141) */
static void zeta_k2u(ko_ctx *c, double **zeta, const double *uk_dc, double **u) {
  zeta_k2u_k(c, zeta, uk_dc, u);
  for (int d = 0; d < DIM; d++) fft_c2r(c, u[d]);
}

/* U2zeta_k (operate_omega.h:212-215) */
static void u2zeta_k(ko_ctx *c, double **zeta, double *uk_dc, double **u) {
  for (int d = 0; d < DIM; d++) fft_r2c(c, u[d]);
  u_k2zeta_k(c, u, zeta, uk_dc);
}

/* Zeta_k2advection_k (operate_omega.cxx:100-111) */
static void zeta_k2advection_k(ko_ctx *c, double **zeta, const double *uk_dc, double **adv) {
  double *u[3] = {c->f[F_U0], c->f[F_U1], c->f[F_U2]};
  truncate_23(c, zeta[0]);
  truncate_23(c, zeta[1]);
  zeta_k2u(c, zeta, uk_dc, u);
  u2advection_k(c, u, adv);
}

/* NS_solver_slavedEuler (fluid_solver.cxx:340-366): integrating-factor
 * update over the 2/3 region. */
static void ns_solver_slaved_euler(ko_ctx *c) {
  double *zeta[2] = {c->f[F_ZETA0], c->f[F_ZETA1]};
  double *adv[2] = {c->f[F_NS0_0], c->f[F_NS0_1]};
  zeta_k2advection_k(c, zeta, c->uk_dc, adv);
  const double dmy0 = -c->nu_visc * c->P.dt;
  const double dmy1 = 1. / c->nu_visc;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nzp; k++) {
        if (!in_two_third(c, i, j, k / 2)) continue;
        long im = IDX(c, i, j, k);
        double dmy = exp(dmy0 * k2_of(c, i, j, k / 2)) - 1.;
        double ik2 = ik2_of(c, i, j, k / 2);
        zeta[0][im] += dmy * (zeta[0][im] - dmy1 * ik2 * adv[0][im]);
        zeta[1][im] += dmy * (zeta[1][im] - dmy1 * ik2 * adv[1][im]);
      }
}

/* ------------------------------------------------------------------------ */
/* Smoothed profile and particle <-> grid transfers                         */
/* ------------------------------------------------------------------------ */

static inline int nint(double a) { return (a >= 0.0) ? (int)(a + .5) : (int)(a - .5); }

/* H and Phi (profile.h:29-49) */
static inline double prof_h(const ko_ctx *c, double x) { return x > 0 ? exp(-SQ(c->dx / x)) : 0; }
static inline double prof_phi(const ko_ctx *c, double x, double radius) {
  double a = prof_h(c, radius + c->hxi - x);
  return a / (a + prof_h(c, x - radius + c->hxi));
}
/* Phi_compact_sin (profile.h:139-152) */
static inline double prof_phi_sin(const ko_ctx *c, double x, double radius) {
  double d = radius - x;
  if (fabs(d) <= c->hxi) return 0.5 * sin(M_PI * d / c->xi) + 0.5;
  return (d > c->hxi) ? 1. : 0.;
}

/* DPhi_compact_sin (profile.h:168-181): the surface profile */
static inline double prof_dphi_sin(const ko_ctx *c, double x, double radius) {
  const double hxi = c->xi * .5;
  const double ixi = 1. / c->xi;
  double d = radius - x;
  if (fabs(d) < hxi) return M_PI * .5 * ixi * cos(M_PI * d * ixi);
  return 0.;
}

/* Particle_domain (profile.cxx:25-74): integration stencil offsets, in the
 * reference's loop order. */
static void build_sekibun(ko_ctx *c) {
  int nh = (int)c->P.a + (int)c->P.a_xi + 2;
  double max_r = c->radius + c->hxi + 1.7321 * c->dx;
  int cap = (2 * nh + 1) * (2 * nh + 1) * (2 * nh + 1);
  c->sekibun = (int *)malloc(sizeof(int) * 3 * cap);
  int m = 0;
  for (int i = -nh; i <= nh; i++)
    for (int j = -nh; j <= nh; j++)
      for (int k = -nh; k <= nh; k++) {
        double d = sqrt(SQ(i * c->dx) + SQ(j * c->dx) + SQ(k * c->dx));
        if (d < max_r) {
          c->sekibun[3 * m] = i;
          c->sekibun[3 * m + 1] = j;
          c->sekibun[3 * m + 2] = k;
          m++;
        }
      }
  c->np_domain = m;
}

/* Particle_cell (make_phi.h:114-140) + Relative_coord (make_phi.h:162-179) +
 * Distance (interaction.h:139-147) for one stencil point. */
typedef struct {
  int x_int[3];
  double residue[3];
} pcell;

static inline void particle_cell(const ko_ctx *c, const double *xp, pcell *pc) {
  const double idx = 1. / c->dx;
  for (int d = 0; d < DIM; d++) {
    double v = xp[d] * idx;
    pc->x_int[d] = (int)v;
    pc->residue[d] = (v - (double)pc->x_int[d]) * c->dx;
  }
}

static inline long stencil_point(const ko_ctx *c, const pcell *pc, const double *xp, int m, double *r,
                                 double *dist) {
  const int N[3] = {c->nx, c->ny, c->nz};
  const double Lp[3] = {c->nx * c->dx, c->ny * c->dx, c->nz * c->dx};
  int rm[3];
  double s = 0.0;
  for (int d = 0; d < DIM; d++) {
    int cell = c->sekibun[3 * m + d];
    rm[d] = (pc->x_int[d] + cell + N[d]) % N[d];
    r[d] = (double)cell * c->dx - pc->residue[d];
    double x12 = xp[d] - rm[d] * c->dx;
    x12 -= (double)nint(x12 / Lp[d]) * Lp[d];
    s += SQ(x12);
  }
  *dist = sqrt(s);
  return IDX(c, rm[0], rm[1], rm[2]);
}

/* Angular2v_rot_on/off (make_phi.h:398-417) */
static inline void angular2v(const ko_ctx *c, const double *w, const double *r, double *v) {
  if (c->P.rotation) {
    v[0] = w[1] * r[2] - w[2] * r[1];
    v[1] = w[2] * r[0] - w[0] * r[2];
    v[2] = w[0] * r[1] - w[1] * r[0];
  } else {
    v[0] = v[1] = v[2] = 0.0;
  }
}

static void zero_real(ko_ctx *c, double *a) { memset(a, 0, sizeof(double) * c->nf); }

/* Make_phi_particle_sum (make_phi.cxx:229-275, 519-523): phi_sum = sum of
 * profiles, phi = min(phi_sum, 1). Serial scatter in particle order. */
static void make_phi_particle_sum(ko_ctx *c) {
  double *phi = c->f[F_PHI], *phs = c->f[F_PHI_SUM];
  zero_real(c, phi);
  zero_real(c, phs);
  for (int n = 0; n < c->np; n++) {
    pcell pc;
    particle_cell(c, c->p[n].x, &pc);
    for (int m = 0; m < c->np_domain; m++) {
      double r[3], dist;
      long im = stencil_point(c, &pc, c->p[n].x, m, r, &dist);
      phs[im] += prof_phi(c, dist, c->radius);
    }
  }
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nz; k++) {
        long im = IDX(c, i, j, k);
        phi[im] = (phs[im] < 1.0) ? phs[im] : 1.0;
      }
}

/* Make_phi_particle (make_phi.cxx:506-518 via Make_phi_u_primitive without
 * velocities): the unclipped sum of profiles. */
static void make_phi_particle(ko_ctx *c, double *phi) {
  zero_real(c, phi);
  for (int n = 0; n < c->np; n++) {
    pcell pc;
    particle_cell(c, c->p[n].x, &pc);
    for (int m = 0; m < c->np_domain; m++) {
      double r[3], dist;
      long im = stencil_point(c, &pc, c->p[n].x, m, r, &dist);
      phi[im] += prof_phi(c, dist, c->radius);
    }
  }
}

/* Make_u_particle_sum (make_phi.cxx:329-370, 532-536) into up (zeroed here) */
static void make_u_particle_sum(ko_ctx *c) {
  double *up[3] = {c->f[F_UP0], c->f[F_UP1], c->f[F_UP2]};
  const double *phs = c->f[F_PHI_SUM];
  for (int d = 0; d < DIM; d++) zero_real(c, up[d]);
  for (int n = 0; n < c->np; n++) {
    const icep_particle *p = &c->p[n];
    pcell pc;
    particle_cell(c, p->x, &pc);
    for (int m = 0; m < c->np_domain; m++) {
      double r[3], dist, vr[3];
      long im = stencil_point(c, &pc, p->x, m, r, &dist);
      double w = prof_phi(c, dist, c->radius) / ((phs[im] > 1.0) ? phs[im] : 1.0);
      angular2v(c, p->omega, r, vr);
      for (int d = 0; d < DIM; d++) up[d][im] += (p->v[d] + vr[d]) * w;
    }
  }
}

/* Make_surface_normal (make_phi.cxx:17-61) */
static void make_surface_normal(ko_ctx *c) {
  double *sn[3] = {c->f[F_SN0], c->f[F_SN1], c->f[F_SN2]};
  for (int d = 0; d < DIM; d++) zero_real(c, sn[d]);
  for (int n = 0; n < c->np; n++) {
    pcell pc;
    particle_cell(c, c->p[n].x, &pc);
    for (int m = 0; m < c->np_domain; m++) {
      double r[3], dist;
      long im = stencil_point(c, &pc, c->p[n].x, m, r, &dist);
      double dr = sqrt(SQ(r[0]) + SQ(r[1]) + SQ(r[2]));
      if (fabs(dr - c->radius) < c->hxi) {
        double ir = 1. / dr;
        for (int d = 0; d < DIM; d++) sn[d][im] += r[d] * ir;
      }
    }
  }
}

/* Make_phi_sin_primitive (operate_dielectric.cxx:78-120). With
 * per_particle_eps, eps_w also receives (eps_p - eps_f) * phi_sin per particle
 * (the per-particle permittivity extension). */
static void make_phi_sin(ko_ctx *c, double *phi_sin, double *eps_w) {
  zero_real(c, phi_sin);
  if (eps_w) zero_real(c, eps_w);
  for (int n = 0; n < c->np; n++) {
    pcell pc;
    particle_cell(c, c->p[n].x, &pc);
    double de = c->p[n].eps_p - c->P.eps_fluid;
    for (int m = 0; m < c->np_domain; m++) {
      double r[3], dist;
      long im = stencil_point(c, &pc, c->p[n].x, m, r, &dist);
      double v = prof_phi_sin(c, dist, c->radius);
      phi_sin[im] += v;
      if (eps_w) eps_w[im] += de * v;
    }
  }
}

/* Calc_f_hydro_correct_precision (md_force.cxx:340-449) for spherical particles */
static void calc_f_hydro(ko_ctx *c) {
  const double *u[3] = {c->f[F_U0], c->f[F_U1], c->f[F_U2]};
  const double *phs = c->f[F_PHI_SUM];
  const double dmy = -c->dx3 * c->P.rho / c->P.dt;
#pragma omp parallel for schedule(dynamic)
  for (int n = 0; n < c->np; n++) {
    icep_particle *p = &c->p[n];
    double force[3] = {0, 0, 0}, torque[3] = {0, 0, 0};
    pcell pc;
    particle_cell(c, p->x, &pc);
    for (int m = 0; m < c->np_domain; m++) {
      double r[3], dist, vr[3], fp[3];
      long im = stencil_point(c, &pc, p->x, m, r, &dist);
      angular2v(c, p->omega, r, vr);
      double w = prof_phi(c, dist, c->radius) / ((phs[im] > 1.0) ? phs[im] : 1.0);
      for (int d = 0; d < DIM; d++) {
        fp[d] = ((p->v[d] + vr[d]) - u[d][im]) * w;
        force[d] += fp[d];
      }
      torque[0] += (r[1] * fp[2] - r[2] * fp[1]);
      torque[1] += (r[2] * fp[0] - r[0] * fp[2]);
      torque[2] += (r[0] * fp[1] - r[1] * fp[0]);
    }
    for (int d = 0; d < DIM; d++) p->f_hydro[d] = dmy * force[d];
    if (c->P.rotation)
      for (int d = 0; d < DIM; d++) p->torque_hydro[d] = dmy * torque[d];
  }
}

/* ------------------------------------------------------------------------ */
/* Lennard-Jones and particle integration                                   */
/* ------------------------------------------------------------------------ */

/* Lennard_Jones_f (interaction.h:175-200) */
static double lj_f(const ko_ctx *c, double x, double sigma) {
  double s = sigma / x, t;
  double eps = c->P.lj_epsilon;
  if (c->P.lj_powers == 0) {
    t = SQ(s) * SQ(s) * SQ(s);
    return 24. * eps / SQ(x) * (2.0 * SQ(t) - t);
  } else if (c->P.lj_powers == 1) {
    t = SQ(s) * SQ(s) * SQ(s) * SQ(s) * SQ(s) * SQ(s);
    return 48. * eps / SQ(x) * (2.0 * SQ(t) - t);
  } else {
    t = SQ(s) * SQ(s) * SQ(s) * SQ(s) * SQ(s) * SQ(s) * SQ(s) * SQ(s) * SQ(s);
    return 72. * eps / SQ(x) * (2.0 * SQ(t) - t);
  }
}

/*
 * Calc_f_Lennard_Jones_shear_cap_primitive_lnk (md_force.cxx:16-171) with
 * cap = DBL_MAX: linked cells of edge 16*DX, a 27-cell scan with the
 * reference's wrap rule, pair (i, j) taken when i > j. When a dimension has
 * fewer than three cells the scan visits the same neighbour cell more than
 * once and the pair force is added once per visit (the reference's
 * behaviour, kept). Forces accumulate into fr in the reference's order.
 * If pairs != NULL, every visited pair within the cutoff is recorded as
 * (i, j) into pairs[2*k..] and the count returned (for neighbour-set checks).
 */
static long lj_force(ko_ctx *c, int *pairs, long max_pairs) {
  const int cell_len = 16;
  int lc[3] = {c->nx / cell_len, c->ny / cell_len, c->nz / cell_len};
  double lcr = cell_len * c->dx;
  int lcyz = lc[1] * lc[2], lcxyz = lc[0] * lcyz;
  const double cutoff = c->r_cutoff;
  const double Lp[3] = {c->nx * c->dx, c->ny * c->dx, c->nz * c->dx};
  long npairs = 0;
  if (lcxyz <= 0) return -1;
  int *head = (int *)malloc(sizeof(int) * lcxyz);
  int *lscl = (int *)malloc(sizeof(int) * (c->np > 0 ? c->np : 1));
  for (int q = 0; q < lcxyz; q++) head[q] = -1;
  for (int n = 0; n < c->np; n++) {
    int mc[3];
    for (int d = 0; d < DIM; d++) mc[d] = (int)(c->p[n].x[d] / lcr);
    int cn = mc[0] * lcyz + mc[1] * lc[2] + mc[2];
    lscl[n] = head[cn];
    head[cn] = n;
  }
  int ic[3], icl[3], icls[3];
  for (ic[0] = 0; ic[0] < lc[0]; ic[0]++)
    for (ic[1] = 0; ic[1] < lc[1]; ic[1]++)
      for (ic[2] = 0; ic[2] < lc[2]; ic[2]++) {
        int cn = ic[0] * lcyz + ic[1] * lc[2] + ic[2];
        for (icl[0] = ic[0] - 1; icl[0] <= ic[0] + 1; icl[0]++)
          for (icl[1] = ic[1] - 1; icl[1] <= ic[1] + 1; icl[1]++)
            for (icl[2] = ic[2] - 1; icl[2] <= ic[2] + 1; icl[2]++) {
              for (int d = 0; d < DIM; d++) {
                icls[d] = icl[d];
                if (icls[d] < 0) icls[d] = lc[d] - 1;
                if (icls[d] > lc[d] - 1) icls[d] = 0;
              }
              int cl = icls[0] * lcyz + icls[1] * lc[2] + icls[2];
              for (int i = head[cn]; i != -1; i = lscl[i]) {
                for (int j = head[cl]; j != -1; j = lscl[j]) {
                  if (!(i > j)) continue;
                  double rv[3], s = 0.0;
                  for (int d = 0; d < DIM; d++) {
                    rv[d] = c->p[j].x[d] - c->p[i].x[d];
                    rv[d] -= (double)nint(rv[d] / Lp[d]) * Lp[d];
                    s += SQ(rv[d]);
                  }
                  double rij = sqrt(s);
                  if (rij < cutoff) {
                    double a = DBL_MAX / rij, b = lj_f(c, rij, c->lj_dia);
                    double fr = (a < b) ? a : b;
                    for (int d = 0; d < DIM; d++) {
                      double fi = fr * (-rv[d]);
                      c->p[i].fr[d] += fi;
                      c->p[j].fr[d] -= fi;
                    }
                    if (pairs && npairs < max_pairs) {
                      pairs[2 * npairs] = i;
                      pairs[2 * npairs + 1] = j;
                    }
                    npairs++;
                  }
                }
              }
            }
      }
  free(head);
  free(lscl);
  return npairs;
}

/* Force (particle_solver.h:92-104) for spherical particles */
static void md_force(ko_ctx *c) {
  if (c->P.lj_truncate >= 0) lj_force(c, NULL, 0);
  if (c->P.g != 0.0) {
    double gf = c->P.g * c->P.rho * 4. / 3. * M_PI * SQ(c->radius) * c->radius;
    for (int n = 0; n < c->np; n++)
      c->p[n].fr[c->P.g_direction] -= gf * (c->P.mass_ratio[c->p[n].spec] - 1.0);
  }
}

/* quaternion helpers (quaternion.h:70-291, rigid_body.cxx:10-24,151-165) */
static void qprod(double *q, const double *a, const double *b, double alpha) {
  q[0] = alpha * (a[0] * b[0] - (a[1] * b[1] + a[2] * b[2] + a[3] * b[3]));
  q[1] = alpha * (a[0] * b[1] + b[0] * a[1] + a[2] * b[3] - a[3] * b[2]);
  q[2] = alpha * (a[0] * b[2] + b[0] * a[2] + a[3] * b[1] - a[1] * b[3]);
  q[3] = alpha * (a[0] * b[3] + b[0] * a[3] + a[1] * b[2] - a[2] * b[1]);
}
/* v' = q (0,v) q*  (space from body when conj = 0, body from space when 1) */
static void qrot(double *out, const double *qin, const double *v, int conj) {
  double q[4] = {qin[0], conj ? -qin[1] : qin[1], conj ? -qin[2] : qin[2], conj ? -qin[3] : qin[3]};
  double qs2 = q[0] * q[0] - (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  double qd = q[1] * v[0] + q[2] * v[1] + q[3] * v[2];
  out[0] = qs2 * v[0] + 2.0 * (qd * q[1] + q[0] * (q[2] * v[2] - q[3] * v[1]));
  out[1] = qs2 * v[1] + 2.0 * (qd * q[2] + q[0] * (q[3] * v[0] - q[1] * v[2]));
  out[2] = qs2 * v[2] + 2.0 * (qd * q[3] + q[0] * (q[1] * v[1] - q[2] * v[0]));
}
static void qnormalize(double *q) {
  double n = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  n = 1.0 / n;
  for (int a = 0; a < 4; a++) q[a] *= n;
}

/* PBC (periodic_boundary.h:9-14) */
static void pbc(const ko_ctx *c, double *x) {
  const double Lp[3] = {c->nx * c->dx, c->ny * c->dx, c->nz * c->dx};
  for (int d = 0; d < DIM; d++) x[d] = fmod(x[d] + Lp[d], Lp[d]);
}

/* MD_solver_position_Euler / _AB2 (particle_solver.cxx:39-91) with
 * MD_solver_orientation_Euler / _AB2 (particle_rotation_solver.h:15-39) */
static void md_position(ko_ctx *c, int ab2) {
  const double dt = c->P.dt, hdt = 0.5 * c->P.dt;
  for (int n = 0; n < c->np; n++) {
    icep_particle *p = &c->p[n];
    for (int d = 0; d < DIM; d++) {
      double dx = ab2 ? hdt * (3.0 * p->v[d] - p->v_old[d]) : dt * p->v[d];
      p->x_nopbc[d] += dx;
      p->x[d] += dx;
    }
    pbc(c, p->x);
    if (c->P.rotation) {
      double dq[4], qw[4];
      if (!ab2) {
        memcpy(p->q_old, p->q, sizeof(double) * 4);
        qw[0] = 0.0; qw[1] = p->omega[0]; qw[2] = p->omega[1]; qw[3] = p->omega[2];
        qprod(dq, qw, p->q, 0.5);
        for (int a = 0; a < 4; a++) p->q[a] += dq[a] * dt;
      } else {
        double wb[3], wbo[3];
        qrot(wb, p->q, p->omega, 1);
        qrot(wbo, p->q_old, p->omega_old, 1);
        for (int d = 0; d < DIM; d++) wb[d] = 3.0 * wb[d] - wbo[d];
        memcpy(p->q_old, p->q, sizeof(double) * 4);
        qw[0] = 0.0; qw[1] = wb[0]; qw[2] = wb[1]; qw[3] = wb[2];
        qprod(dq, p->q, qw, 0.5);
        for (int a = 0; a < 4; a++) p->q[a] += dq[a] * hdt;
      }
      qnormalize(p->q);
    }
  }
}

/* reset_Forces (particle_solver.cxx:11-37) */
static void reset_forces(ko_ctx *c) {
  for (int n = 0; n < c->np; n++) {
    icep_particle *p = &c->p[n];
    for (int d = 0; d < DIM; d++) {
      p->fr_previous[d] = p->fr[d];
      p->fr[d] = 0.0;
      p->f_hydro_previous[d] = p->f_hydro[d];
      p->f_hydro[d] = 0.0;
      p->torque_r_previous[d] = p->torque_r[d];
      p->torque_r[d] = 0.0;
      p->torque_hydro_previous[d] = p->torque_hydro[d];
      p->torque_hydro[d] = 0.0;
    }
  }
}

/* MD_solver_velocity_Euler / _AB2_hydro (particle_solver.cxx:109-150, 252-295)
 * with self_propulsion (particle_solver.cxx:94-107). */
static void md_velocity(ko_ctx *c, int ab2) {
  md_force(c);
  int motor_on = 0;
  for (int s = 0; s < c->P.n_species; s++)
    if (c->P.janus_propulsion[s] == ICEP_MOTOR) motor_on = 1;
  for (int n = 0; n < c->np; n++) {
    icep_particle *p = &c->p[n];
    int s = p->spec;
    double sf[3] = {0, 0, 0}, st[3] = {0, 0, 0};
    if (motor_on && c->P.janus_propulsion[s] == ICEP_MOTOR) {
      qrot(sf, p->q, c->P.janus_force[s], 0);
      qrot(st, p->q, c->P.janus_torque[s], 0);
    }
    for (int d = 0; d < DIM; d++) {
      p->v_old[d] = p->v[d];
      p->omega_old[d] = p->omega[d];
      if (!ab2) {
        double a = c->P.dt * c->imass[s], b = c->P.dt * c->imoi[s];
        p->v[d] += a * (p->f_hydro[d] + p->fr[d] + sf[d]);
        p->omega[d] += b * (p->torque_hydro[d] + p->torque_r[d] + st[d]);
      } else {
        double a = 0.5 * c->P.dt * c->imass[s], b = 0.5 * c->P.dt * c->imoi[s];
        p->v[d] += a * (2.0 * (p->f_hydro[d] + sf[d]) + p->fr[d] + p->fr_previous[d]);
        p->omega[d] += b * (2.0 * (p->torque_hydro[d] + st[d]) + p->torque_r[d] + p->torque_r_previous[d]);
      }
    }
  }
  reset_forces(c);
}

/* Make_f_particle_dt_nonsole + Solenoidal_u (f_particle.h:37-78) and
 * Add_f_particle (f_particle.h:79-95) */
static void f_particle_sole_and_add(ko_ctx *c) {
  double *f[3] = {c->f[F_F0], c->f[F_F1], c->f[F_F2]};
  double *u[3] = {c->f[F_U0], c->f[F_U1], c->f[F_U2]};
  double *up[3] = {c->f[F_UP0], c->f[F_UP1], c->f[F_UP2]};
  const double *phi = c->f[F_PHI];
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nz; k++) {
        long im = IDX(c, i, j, k);
        for (int d = 0; d < DIM; d++) f[d][im] = up[d][im] - phi[im] * u[d][im];
      }
  solenoidal_u(c, f);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nz; k++) {
        long im = IDX(c, i, j, k);
        for (int d = 0; d < DIM; d++) u[d][im] += f[d][im];
      }
}

/* ------------------------------------------------------------------------ */
/* Dielectric (ICEP) operator and Poisson solve                             */
/* ------------------------------------------------------------------------ */

static inline long wrap_idx(const ko_ctx *c, int i, int j, int k) {
  /* extract_id (periodic_boundary.h:21-27) */
  i = (i + c->nx) % c->nx;
  j = (j + c->ny) % c->ny;
  k = (k + c->nz) % c->nz;
  return IDX(c, i, j, k);
}

/* Make_janus_normal_dielectric (operate_dielectric.cxx:173-205): the body
 * axis e3 of the species (x, y or z) in the space frame, normalised. */
static void janus_normal(const ko_ctx *c, const icep_particle *p, double *nrm) {
  const int ax = c->P.janus_axis[p->spec];
  const double e3[3] = {ax == ICEP_JANUS_X ? 1.0 : 0.0, ax == ICEP_JANUS_Y ? 1.0 : 0.0, ax == ICEP_JANUS_Z ? 1.0 : 0.0};
  qrot(nrm, p->q, e3, 0);
  const double n = sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
  const double in = 1.0 / n;
  for (int d = 0; d < DIM; d++) nrm[d] *= in;
}

/* Make_dielectric_field, Janus branch (operate_dielectric.cxx:208-292): per
 * particle and stencil point phi = Phi_compact_sin, phi_p += phi,
 * eps += phi (eps_ave + eps_delta tanh(r.n / DX)); then
 * eps += eps_f (1 - phi_p) Dc. */
static void make_janus_eps(ko_ctx *c, double *eps, double *phi_p) {
  const double dc = c->P.dielectric_cst;
  const double eps_ave = 0.5 * (c->P.eps_particle_top + c->P.eps_particle_bottom) * dc;
  const double eps_delta = 0.5 * (c->P.eps_particle_top - c->P.eps_particle_bottom) * dc;
  const double sharp = 1 / c->dx;
  zero_real(c, phi_p);
  zero_real(c, eps);
  for (int n = 0; n < c->np; n++) {
    double nrm[3];
    janus_normal(c, &c->p[n], nrm);
    pcell pc;
    particle_cell(c, c->p[n].x, &pc);
    for (int m = 0; m < c->np_domain; m++) {
      double r[3], dist, jr = 0.0;
      long im = stencil_point(c, &pc, c->p[n].x, m, r, &dist);
      for (int d = 0; d < DIM; d++) jr += r[d] * nrm[d];
      double v = prof_phi_sin(c, dist, c->radius);
      phi_p[im] += v;
      eps[im] += v * (eps_ave + eps_delta * tanh(sharp * jr));
    }
  }
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nz; k++) {
        long im = IDX(c, i, j, k);
        eps[im] += c->P.eps_fluid * (1 - phi_p[im]) * dc;
      }
}

/* Make_dielectric_field, non-Janus branch (operate_dielectric.cxx:270-309):
 * phi_sin into phi_p; eps = eps_f*Dc + (eps_p - eps_f)*Dc*phi_sin. With
 * per_particle_eps the particle term is summed per particle (extension).
 * The field is Janus when particle 0's species has an axis (:276-280). */
static void make_dielectric_field(ko_ctx *c, double *eps, double *phi_p) {
  const double dc = c->P.dielectric_cst, ef = c->P.eps_fluid;
  if (c->np > 0 && c->P.janus_axis[c->p[0].spec] != ICEP_JANUS_NONE) {
    make_janus_eps(c, eps, phi_p);
    return;
  }
  if (!c->P.per_particle_eps) {
    make_phi_sin(c, phi_p, NULL);
    const double de = c->P.eps_particle_top - ef;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < c->nx; i++)
      for (int j = 0; j < c->ny; j++)
        for (int k = 0; k < c->nz; k++) {
          long im = IDX(c, i, j, k);
          eps[im] = ef * dc + de * dc * phi_p[im];
        }
  } else {
    make_phi_sin(c, phi_p, eps);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < c->nx; i++)
      for (int j = 0; j < c->ny; j++)
        for (int k = 0; k < c->nz; k++) {
          long im = IDX(c, i, j, k);
          eps[im] = ef * dc + dc * eps[im];
        }
  }
}

/* Make_phi_qq_particle (operate_electrolyte.cxx:179-243): phi += Phi and
 * surface += Q_e DPhi_compact_sin per particle, then the surface charge
 * rescaled so that its volume integral of |.| is sum_n |Q_e|. */
static void make_phi_qq(ko_ctx *c, double *phi, double *surface) {
  double abs_total = 0.;
  for (int n = 0; n < c->np; n++) {
    const double q = c->P.surface_charge[c->p[n].spec] * c->P.elementary_charge;
    pcell pc;
    particle_cell(c, c->p[n].x, &pc);
    for (int m = 0; m < c->np_domain; m++) {
      double r[3], dist;
      long im = stencil_point(c, &pc, c->p[n].x, m, r, &dist);
      phi[im] += prof_phi(c, dist, c->radius);
      surface[im] += q * prof_dphi_sin(c, dist, c->radius);
    }
    abs_total += fabs(q);
  }
  double dmy = 0.0;
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nz; k++) dmy += fabs(surface[IDX(c, i, j, k)]);
  const double rescale = abs_total / (dmy * c->dx3);
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nz; k++) surface[IDX(c, i, j, k)] *= rescale;
}

/* Conc_k2charge_field_no_surfase_charge (operate_dielectric.cxx:135-160):
 * rho = sum_n z_n e c_n (1 - phi_p); tmp is scratch. With surface charges,
 * Conc_k2charge_field (operate_electrolyte.cxx:45-74): phi_p is rebuilt as
 * the sum of Phi and rho starts from the rescaled surface charge. */
static void conc_k2charge(ko_ctx *c, double *rho, double *phi_p, double *tmp) {
  zero_real(c, rho);
  if (c->P.surface_charge[0] != 0.0) {
    zero_real(c, phi_p);
    make_phi_qq(c, phi_p, rho);
  }
  for (int n = 0; n < 2; n++) {
    memcpy(tmp, c->f[F_C0 + n], sizeof(double) * c->nf);
    fft_c2r(c, tmp);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < c->nx; i++)
      for (int j = 0; j < c->ny; j++)
        for (int k = 0; k < c->nz; k++) {
          long im = IDX(c, i, j, k);
          rho[im] += c->valency_e[n] * tmp[im] * (1. - phi_p[im]);
        }
  }
}

/* Ax (operate_dielectric.cxx:485-522) on unpadded length-N vectors:
 * A x = D^- . (eps_face D^+ x) with spectral staggered derivatives. */
static void apply_A(ko_ctx *c, const double *x, double *y) {
  double *w1 = c->f[F_WV1];
  double *w3[3] = {c->f[F_WV3_0], c->f[F_WV3_1], c->f[F_WV3_2]};
  const double *eps = c->f[F_EPS];
  zero_real(c, w1);
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      memcpy(w1 + IDX(c, i, j, 0), x + ((long)i * c->ny + j) * c->nz, sizeof(double) * c->nz);
  fft_r2c(c, w1);
  a_k2da_k(c, w1, w3);
  shift_fw(c, w3);
  for (int d = 0; d < DIM; d++) fft_c2r(c, w3[d]);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nz; k++) {
        long im = IDX(c, i, j, k);
        double e0 = eps[im];
        w3[0][im] *= 0.5 * (eps[wrap_idx(c, i + 1, j, k)] + e0);
        w3[1][im] *= 0.5 * (eps[wrap_idx(c, i, j + 1, k)] + e0);
        w3[2][im] *= 0.5 * (eps[wrap_idx(c, i, j, k + 1)] + e0);
      }
  for (int d = 0; d < DIM; d++) fft_r2c(c, w3[d]);
  u_k2divergence_k_shift(c, w3, w1);
  fft_c2r(c, w1);
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      memcpy(y + ((long)i * c->ny + j) * c->nz, w1 + IDX(c, i, j, 0), sizeof(double) * c->nz);
  c->matvecs++;
}

/* E_ext at the context's time: times sin(2 pi f t) for an AC field
 * (operate_dielectric.cxx:620-627) */
static void ext_now(const ko_ctx *c, double *E) {
  const double s = c->P.ac ? sin(2.0 * M_PI * c->P.frequency * c->time) : 1.0;
  for (int d = 0; d < DIM; d++) E[d] = c->P.ac ? c->P.e_ext[d] * s : c->P.e_ext[d];
}

/* Build_rhs (operate_dielectric.cxx:524-540) with
 * Interpolate_scalar_on_staggered_grid (operate_dielectric.cxx:57-76):
 * b = D^-.(eps_face E_ext) - rho */
static void build_rhs(ko_ctx *c, double *rhs, const double *rho) {
  double *w3[3] = {c->f[F_WV3_0], c->f[F_WV3_1], c->f[F_WV3_2]};
  const double *eps = c->f[F_EPS];
  double E[3];
  ext_now(c, E);
  zero_real(c, rhs);
  for (int d = 0; d < DIM; d++) zero_real(c, w3[d]);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nz; k++) {
        long im = IDX(c, i, j, k);
        double s0 = 0.5 * eps[im];
        w3[0][im] = (0.5 * eps[wrap_idx(c, i + 1, j, k)] + s0) * E[0];
        w3[1][im] = (0.5 * eps[wrap_idx(c, i, j + 1, k)] + s0) * E[1];
        w3[2][im] = (0.5 * eps[wrap_idx(c, i, j, k + 1)] + s0) * E[2];
      }
  for (int d = 0; d < DIM; d++) fft_r2c(c, w3[d]);
  u_k2divergence_k_shift(c, w3, rhs);
  fft_c2r(c, rhs);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nz; k++) {
        long im = IDX(c, i, j, k);
        rhs[im] -= rho[im];
      }
}

static double vdot(long n, const double *a, const double *b) {
  double s = 0.0;
  for (long i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

/*
 * BiCGSTAB with an identity preconditioner and Eigen's control flow (the
 * solver of Charge_field2potential_dielectric_LO, operate_dielectric.cxx:556-562;
 * Eigen 3.3/3.4 internal::bicgstab, van der Vorst 1992): stop when the
 * recursively updated residual satisfies |r|^2 <= tol^2 |b|^2 or after maxit
 * iterations; restart (r = b - A x, r0 = r) when |rho| < eps^2 |r0|^2, resetting
 * the iteration count on the first restart only; x = 0 if |b| = 0.
 * Returns the iteration count; *err = |r|/|b|.
 */
static long bicgstab(ko_ctx *c, const double *b, double *x, double tol, long maxit, double *err) {
  const long n = c->nu;
  double *r = (double *)malloc(sizeof(double) * n), *r0 = (double *)malloc(sizeof(double) * n);
  double *v = (double *)calloc((size_t)n, sizeof(double)), *p = (double *)calloc((size_t)n, sizeof(double));
  double *s = (double *)malloc(sizeof(double) * n), *t = (double *)malloc(sizeof(double) * n);
  apply_A(c, x, t);
  for (long k = 0; k < n; k++) r[k] = b[k] - t[k];
  memcpy(r0, r, sizeof(double) * n);
  double r0_sq = vdot(n, r0, r0), b_sq = vdot(n, b, b);
  long i = 0;
  if (b_sq == 0) {
    memset(x, 0, sizeof(double) * n);
    *err = 0.0;
    goto done;
  }
  {
    double rho = 1, alpha = 1, w = 1;
    const double tol2 = tol * tol * b_sq, eps2 = DBL_EPSILON * DBL_EPSILON;
    long restarts = 0;
    while (vdot(n, r, r) > tol2 && i < maxit) {
      double rho_old = rho;
      rho = vdot(n, r0, r);
      if (fabs(rho) < eps2 * r0_sq) {
        apply_A(c, x, t);
        for (long k = 0; k < n; k++) r[k] = b[k] - t[k];
        memcpy(r0, r, sizeof(double) * n);
        rho = r0_sq = vdot(n, r, r);
        if (restarts++ == 0) i = 0;
      }
      double beta = (rho / rho_old) * (alpha / w);
      for (long k = 0; k < n; k++) p[k] = r[k] + beta * (p[k] - w * v[k]);
      apply_A(c, p, v);
      alpha = rho / vdot(n, r0, v);
      for (long k = 0; k < n; k++) s[k] = r[k] - alpha * v[k];
      apply_A(c, s, t);
      double tt = vdot(n, t, t);
      w = (tt > 0.0) ? vdot(n, t, s) / tt : 0.0;
      for (long k = 0; k < n; k++) x[k] += alpha * p[k] + w * s[k];
      for (long k = 0; k < n; k++) r[k] = s[k] - w * t[k];
      ++i;
    }
    *err = sqrt(vdot(n, r, r) / b_sq);
  }
done:
  free(r); free(r0); free(v); free(p); free(s); free(t);
  return i;
}

/* Spectral inverse of the constant-permittivity operator, y = M^-1 x:
 * y(k) = -x(k) / (eps_ref |k|^2), y(0) = 0 (preconditioner of the plain
 * GPU method; no counterpart in the reference). */
static void precond_spectral(ko_ctx *c, const double *x, double *y, double eps_ref) {
  double *w = c->f[F_WV1];
  zero_real(c, w);
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      memcpy(w + IDX(c, i, j, 0), x + ((long)i * c->ny + j) * c->nz, sizeof(double) * c->nz);
  fft_r2c(c, w);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int kz = 0; kz < c->hnz; kz++) {
        double k2 = k2_of(c, i, j, kz);
        double f = (k2 > 0.0) ? -1.0 / (eps_ref * k2) : 0.0;
        long im = IDX(c, i, j, 2 * kz);
        w[im] *= f;
        w[im + 1] *= f;
      }
  fft_c2r(c, w);
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      memcpy(y + ((long)i * c->ny + j) * c->nz, w + IDX(c, i, j, 0), sizeof(double) * c->nz);
}

/*
 * The plain method of the GPU path (ICEP_SOLVER_SPECTRAL): BiCGSTAB right-
 * preconditioned by precond_spectral, b projected to mean zero (the range of
 * the singular operator), convergence confirmed on the true residual
 * |b - A x| <= tol |b|. Same loop as bicgstab() otherwise.
 */
static long bicgstab_spectral(ko_ctx *c, double *b, double *x, double tol, long maxit, double *err) {
  const long n = c->nu;
  double mean = 0.0;
  for (long k = 0; k < n; k++) mean += b[k];
  mean /= (double)n;
  for (long k = 0; k < n; k++) b[k] -= mean;
  double eref = 0.0;
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nz; k++) eref += c->f[F_EPS][IDX(c, i, j, k)];
  eref /= (double)n;
  double *r = (double *)malloc(sizeof(double) * n), *r0 = (double *)malloc(sizeof(double) * n);
  const size_t nn = c->nu > 0 ? (size_t)c->nu : 1;
  double *v = (double *)calloc(nn, sizeof(double)), *p = (double *)calloc(nn, sizeof(double));
  double *s = (double *)malloc(sizeof(double) * n), *t = (double *)malloc(sizeof(double) * n);
  double *y = (double *)malloc(sizeof(double) * n), *z = (double *)malloc(sizeof(double) * n);
  apply_A(c, x, t);
  for (long k = 0; k < n; k++) r[k] = b[k] - t[k];
  memcpy(r0, r, sizeof(double) * n);
  double r0_sq = vdot(n, r0, r0), b_sq = vdot(n, b, b);
  long i = 0;
  if (b_sq == 0) {
    memset(x, 0, sizeof(double) * n);
    *err = 0.0;
  } else {
    double rho = 1, alpha = 1, w = 1, rr = r0_sq, rho_new = r0_sq;
    const double tol2 = tol * tol * b_sq, eps2 = DBL_EPSILON * DBL_EPSILON;
    long restarts = 0;
    while (i < maxit) {
      if (!(rr > tol2)) {
        apply_A(c, x, t);
        for (long k = 0; k < n; k++) r[k] = b[k] - t[k];
        rr = vdot(n, r, r);
        if (!(rr > tol2)) break;
        memcpy(r0, r, sizeof(double) * n);
        r0_sq = rho_new = rr;
        memset(v, 0, sizeof(double) * n);
        memset(p, 0, sizeof(double) * n);
        rho = alpha = w = 1;
      }
      double rho_old = rho;
      rho = rho_new;
      if (fabs(rho) < eps2 * r0_sq) {
        apply_A(c, x, t);
        for (long k = 0; k < n; k++) r[k] = b[k] - t[k];
        memcpy(r0, r, sizeof(double) * n);
        rho = r0_sq = vdot(n, r, r);
        if (restarts++ == 0) i = 0;
      }
      double beta = (rho / rho_old) * (alpha / w);
      for (long k = 0; k < n; k++) p[k] = r[k] + beta * (p[k] - w * v[k]);
      precond_spectral(c, p, y, eref);
      apply_A(c, y, v);
      alpha = rho / vdot(n, r0, v);
      for (long k = 0; k < n; k++) s[k] = r[k] - alpha * v[k];
      precond_spectral(c, s, z, eref);
      apply_A(c, z, t);
      double tt = vdot(n, t, t);
      w = (tt > 0.0) ? vdot(n, t, s) / tt : 0.0;
      for (long k = 0; k < n; k++) x[k] += alpha * y[k] + w * z[k];
      for (long k = 0; k < n; k++) r[k] = s[k] - w * t[k];
      rho_new = vdot(n, r0, r);
      rr = vdot(n, r, r);
      ++i;
    }
    *err = sqrt(rr / b_sq);
  }
  free(r); free(r0); free(v); free(p); free(s); free(t); free(y); free(z);
  return i;
}

/* Charge_field2potential_dielectric_LO (operate_dielectric.cxx:542-572) */
static void solve_potential(ko_ctx *c, const double *rho, double *pot, double *rhs_work) {
  const long n = c->nu;
  double *b = (double *)malloc(sizeof(double) * n), *x = (double *)malloc(sizeof(double) * n);
  build_rhs(c, rhs_work, rho);
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++) {
      memcpy(b + ((long)i * c->ny + j) * c->nz, rhs_work + IDX(c, i, j, 0), sizeof(double) * c->nz);
      memcpy(x + ((long)i * c->ny + j) * c->nz, pot + IDX(c, i, j, 0), sizeof(double) * c->nz);
    }
  double err;
  long it;
  if (c->P.solver == ICEP_SOLVER_SPECTRAL) {
    double *b2 = (double *)malloc(sizeof(double) * n);
    memcpy(b2, b, sizeof(double) * n);
    it = bicgstab_spectral(c, b2, x, c->P.potential_tol, c->P.potential_iter, &err);
    if (it == c->P.potential_iter) {
      memset(x, 0, sizeof(double) * n);
      memcpy(b2, b, sizeof(double) * n);
      it = bicgstab_spectral(c, b2, x, c->P.potential_tol, c->P.potential_iter, &err);
    }
    free(b2);
  } else {
    it = bicgstab(c, b, x, c->P.potential_tol, c->P.potential_iter, &err);
    if (it == c->P.potential_iter) {
      memset(x, 0, sizeof(double) * n);
      it = bicgstab(c, b, x, c->P.potential_tol, c->P.potential_iter, &err);
    }
  }
  c->last_iters = it;
  c->last_error = err;
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      memcpy(pot + IDX(c, i, j, 0), x + ((long)i * c->ny + j) * c->nz, sizeof(double) * c->nz);
  free(b);
  free(x);
}

/* Interpolate_vec_on_normal_grid (operate_dielectric.cxx:32-55) */
static void interp_vec_normal(ko_ctx *c, double **v) {
  double *w3[3] = {c->f[F_WV3_0], c->f[F_WV3_1], c->f[F_WV3_2]};
  for (int d = 0; d < DIM; d++) memcpy(w3[d], v[d], sizeof(double) * c->nf);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nz; k++) {
        long im = IDX(c, i, j, k);
        v[0][im] = 0.5 * w3[0][im] + 0.5 * w3[0][wrap_idx(c, i - 1, j, k)];
        v[1][im] = 0.5 * w3[1][im] + 0.5 * w3[1][wrap_idx(c, i, j - 1, k)];
        v[2][im] = 0.5 * w3[2][im] + 0.5 * w3[2][wrap_idx(c, i, j, k - 1)];
      }
}

/* staggered gradient of a real field: R2C, i k, shift, 3 C2R; the field is
 * restored by C2R (the A2a_k/A_k2a round trip of operate_dielectric.cxx:653-667) */
static void staggered_grad(ko_ctx *c, double *a, double **g) {
  fft_r2c(c, a);
  a_k2da_k(c, a, g);
  shift_fw(c, g);
  fft_c2r(c, a);
  for (int d = 0; d < DIM; d++) fft_c2r(c, g[d]);
}

/* Make_Maxwell_force_x_on_fluid (operate_dielectric.cxx:611-764), no surface
 * charge. force: 3 fields (f_particle); rho: free-charge work field. */
static void maxwell_force(ko_ctx *c, double **force, double *rho) {
  double *eps = c->f[F_EPS], *pot = c->f[F_POT];
  double *ge[3] = {c->f[F_GE0], c->f[F_GE1], c->f[F_GE2]};
  double *w1 = c->f[F_WV1];
  double E[3];
  ext_now(c, E);
  const int ext = c->P.external_field;
  make_dielectric_field(c, eps, force[0]);
  conc_k2charge(c, rho, force[0], force[1]);
  solve_potential(c, rho, pot, force[2]);
  staggered_grad(c, eps, ge);
  staggered_grad(c, pot, force);
  zero_real(c, w1);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nz; k++) {
        long im = IDX(c, i, j, k);
        double fw[3] = {-force[0][im], -force[1][im], -force[2][im]};
        double bw[3] = {-force[0][wrap_idx(c, i - 1, j, k)], -force[1][wrap_idx(c, i, j - 1, k)],
                        -force[2][wrap_idx(c, i, j, k - 1)]};
        if (ext)
          for (int d = 0; d < DIM; d++) {
            fw[d] += E[d];
            bw[d] += E[d];
          }
        w1[im] = SQ((fw[0] + bw[0]) / 2.0) + SQ((fw[1] + bw[1]) / 2.0) + SQ((fw[2] + bw[2]) / 2.0);
      }
  for (int d = 0; d < DIM; d++) {
    const int di = (d == 0), dj = (d == 1), dk = (d == 2);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < c->nx; i++)
      for (int j = 0; j < c->ny; j++)
        for (int k = 0; k < c->nz; k++) {
          long im = IDX(c, i, j, k);
          long ip = wrap_idx(c, i + di, j + dj, k + dk);
          double efw = -force[d][im];
          if (ext) efw += E[d];
          double rf = 0.5 * rho[ip] + 0.5 * rho[im];
          double e2 = 0.5 * w1[im] + 0.5 * w1[ip];
          force[d][im] = rf * efw - e2 * ge[d][im] / 2.0;
        }
  }
  interp_vec_normal(c, force);
  for (int d = 0; d < DIM; d++) memcpy(ge[d], force[d], sizeof(double) * c->nf);
}

/* ------------------------------------------------------------------------ */
/* Electrolyte (Nernst-Planck) step                                         */
/* ------------------------------------------------------------------------ */

/*
 * NSsolute_solver_Euler (fluid_solver.cxx:318-338) with
 * Rhs_NS_Nernst_Planck (:246-292, Dielectric branch), Rhs_NS_solute (:184-230),
 * Diffusion_flux_single (solute_rhs.cxx:212-232),
 * Solute_solver_rhs_nonlinear_x_single (:150-189), Solute_impermeability
 * (:42-97), Add_advection_flux (:190-210), Rhs_solvent (fluid_solver.cxx:172-182),
 * Add_zeta_viscous_term (operate_omega.cxx:170-185), Field_solver_Euler
 * (fluid_solver.cxx:121-137) and Add_constant_field_k (:231-244).
 */
static void nssolute_solver_euler(ko_ctx *c) {
  double *zeta[2] = {c->f[F_ZETA0], c->f[F_ZETA1]};
  double *u[3] = {c->f[F_U0], c->f[F_U1], c->f[F_U2]};
  double *flux[3] = {c->f[F_UP0], c->f[F_UP1], c->f[F_UP2]};
  double *gp[3] = {c->f[F_F0], c->f[F_F1], c->f[F_F2]};
  double *sn[3] = {c->f[F_SN0], c->f[F_SN1], c->f[F_SN2]};
  double *rhs_ns[2] = {c->f[F_NS1_0], c->f[F_NS1_1]};
  double *crhs[2] = {c->f[F_CRHS0], c->f[F_CRHS1]};
  double *pot = c->f[F_POT];
  /* grad potential on the staggered grid, minus E_ext at k = 0, to nodes */
  fft_r2c(c, pot);
  a_k2da_k(c, pot, gp);
  shift_fw(c, gp);
  fft_c2r(c, pot);
  if (c->P.external_field) {  /* Add_constant_field_k (fluid_solver.cxx:231-244) */
    double amp = (double)c->nx * c->ny * c->nz;
    if (c->P.ac) amp *= sin(2.0 * M_PI * c->P.frequency * c->time);
    for (int d = 0; d < DIM; d++) gp[d][0] -= c->P.e_ext[d] * amp;
  }
  for (int d = 0; d < DIM; d++) fft_c2r(c, gp[d]);
  interp_vec_normal(c, gp);
  /* Rhs_NS_solute */
  truncate_23(c, zeta[0]);
  truncate_23(c, zeta[1]);
  zeta_k2u(c, zeta, c->uk_dc, u);
  make_surface_normal(c);
  for (int n = 0; n < 2; n++) {
    double *conc = c->f[F_C0 + n];
    truncate_23(c, conc);
    /* Diffusion_flux_single: flux = grad(kBT L c), rhs_ns[0] as scratch */
    double kl = c->P.kbt * c->onsager[n];
    for (long q = 0; q < c->nf; q++) rhs_ns[0][q] = kl * conc[q];
    a_k2da_k(c, rhs_ns[0], flux);
    for (int d = 0; d < DIM; d++) fft_c2r(c, flux[d]);
    memcpy(crhs[n], conc, sizeof(double) * c->nf);
    fft_c2r(c, crhs[n]);
    const double ze = c->valency_e[n], L = c->onsager[n];
#pragma omp parallel for schedule(static)
    for (int i = 0; i < c->nx; i++)
      for (int j = 0; j < c->ny; j++)
        for (int k = 0; k < c->nz; k++) {
          long im = IDX(c, i, j, k);
          double cc = crhs[n][im];
          for (int d = 0; d < DIM; d++) flux[d][im] += cc * (L * (gp[d][im] * ze));
        }
    /* Solute_impermeability: on every point of a particle stencil where the
     * surface normal is nonzero, remove the normal component; applied once
     * per visit, in particle order (a projection: repeated visits change
     * only the rounding) */
    for (int p = 0; p < c->np; p++) {
      pcell pc;
      particle_cell(c, c->p[p].x, &pc);
      for (int m = 0; m < c->np_domain; m++) {
        double r[3], dist;
        long im = stencil_point(c, &pc, c->p[p].x, m, r, &dist);
        double nv[3], n2 = 0.0;
        for (int d = 0; d < DIM; d++) {
          nv[d] = sn[d][im];
          n2 += SQ(nv[d]);
        }
        if (n2 > 0.) {
          double dd = 0.;
          for (int d = 0; d < DIM; d++) dd += flux[d][im] * nv[d];
          dd /= n2;
          for (int d = 0; d < DIM; d++) flux[d][im] -= nv[d] * dd;
        }
      }
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < c->nx; i++)
      for (int j = 0; j < c->ny; j++)
        for (int k = 0; k < c->nz; k++) {
          long im = IDX(c, i, j, k);
          double cc = crhs[n][im];
          for (int d = 0; d < DIM; d++) flux[d][im] += cc * -u[d][im];
        }
    for (int d = 0; d < DIM; d++) fft_r2c(c, flux[d]);
    u_k2divergence_k(c, flux, crhs[n]);
  }
  /* Rhs_solvent + viscous term */
  u2advection_k(c, u, rhs_ns);
  const double nu = c->nu_visc, dt = c->P.dt;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nzp; k++) {
        if (!in_two_third(c, i, j, k / 2)) continue;
        long im = IDX(c, i, j, k);
        double k2 = k2_of(c, i, j, k / 2);
        rhs_ns[0][im] += -(nu * k2 * zeta[0][im]);
        rhs_ns[1][im] += -(nu * k2 * zeta[1][im]);
        zeta[0][im] += dt * rhs_ns[0][im];
        zeta[1][im] += dt * rhs_ns[1][im];
        c->f[F_C0][im] += dt * crhs[0][im];
        c->f[F_C1][im] += dt * crhs[1][im];
      }
}

/* ------------------------------------------------------------------------ */
/* Time step and initialisation                                             */
/* ------------------------------------------------------------------------ */

/* Time_evolution_hydro (sp_3d_ns.cxx:24-186) for spherical particles without
 * slip, thermostat, pinning or shear; Navier_Stokes or Electrolyte with
 * Dielectric_property = ON. */
static void time_evolution_hydro(ko_ctx *c) {
  double *zeta[2] = {c->f[F_ZETA0], c->f[F_ZETA1]};
  double *u[3] = {c->f[F_U0], c->f[F_U1], c->f[F_U2]};
  double *up[3] = {c->f[F_UP0], c->f[F_UP1], c->f[F_UP2]};
  double *f[3] = {c->f[F_F0], c->f[F_F1], c->f[F_F2]};
  const int electrolyte = (c->P.sw_eq == ICEP_ELECTROLYTE);
  if (!electrolyte) ns_solver_slaved_euler(c);
  else nssolute_solver_euler(c);
  for (int d = 0; d < DIM; d++) /* FIX_CELL (sp_3d_ns.cxx:30-36) */
    if ((c->P.fix_cell >> d) & 1) c->uk_dc[d] = 0.0;
  truncate_23(c, zeta[0]);
  truncate_23(c, zeta[1]);
  zeta_k2u(c, zeta, c->uk_dc, u);
  if (!c->P.fixed_particle) md_position(c, c->ts != 0);
  make_phi_particle_sum(c);
  if (electrolyte) {
    for (int d = 0; d < DIM; d++) {
      zero_real(c, up[d]);
      zero_real(c, f[d]);
    }
    calc_f_hydro(c);
    for (int n = 0; n < c->np; n++)
      for (int d = 0; d < DIM; d++) {
        c->p[n].f_hydro1[d] = c->p[n].f_hydro[d];
        c->p[n].torque_hydro1[d] = c->p[n].torque_hydro[d];
      }
    maxwell_force(c, f, up[0]);
    const double dmy = c->P.dt / c->P.rho;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < c->nx; i++)
      for (int j = 0; j < c->ny; j++)
        for (int k = 0; k < c->nz; k++) {
          long im = IDX(c, i, j, k);
          for (int d = 0; d < DIM; d++) u[d][im] += f[d][im] * dmy;
        }
    solenoidal_u(c, u);
  }
  calc_f_hydro(c);
  if (!c->P.fixed_particle) md_velocity(c, c->ts != 0);
  make_u_particle_sum(c);
  f_particle_sole_and_add(c);
  u2zeta_k(c, zeta, c->uk_dc, u);
}

/* Init_rho_ion_dielectric without surface charge (operate_electrolyte.cxx:912-979)
 * with Set_uniform_ion_charge_density_salt_dielectric (:864-910): uniform
 * salt concentrations rho_inf/(z_n (z_+ - z_-)), transformed to k-space. */
/* Salt-free (N_spec = 1): species 0 are the counterions (Valency_counterion,
 * Onsager_coeff_counterion, Init_rho_ion, operate_electrolyte.cxx:755-758);
 * species 1 is absent: zero valency, mobility and concentration, so every
 * sum over species adds exact zeros. */
static void set_salt_free_species(ko_ctx *c) {
  if (!c->P.salt_free) return;
  c->valency_e[0] = c->P.valency_counterion * c->P.elementary_charge;
  c->valency_e[1] = 0.0;
  c->onsager[0] = c->P.onsager_counterion;
  c->onsager[1] = 0.0;
}

/* Count_single_solute (solute_rhs.cxx:130-148): sum (1 - phi) c DX^3 of a
 * real field */
static double count_single_solute(const ko_ctx *c, const double *conc_x, const double *phi) {
  double s = 0.;
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nz; k++) s += (1. - phi[IDX(c, i, j, k)]) * conc_x[IDX(c, i, j, k)];
  return s * c->dx3;
}

/* The Dielectric branch of Calc_free_energy_PB (operate_electrolyte.cxx:
 * 302-421): kBT DX^3 sum (1 - phi) c (log c - 1) over the species plus
 * DX^3 sum rho (Potential/2 - E.r DX) with rho = `charge` + sum z e c (1 - phi).
 * `charge` is the array the reference accumulates into (its up[1]); it is
 * modified here as there. phi is the particle profile. */
static double free_energy_pb(ko_ctx *c, double *charge, const double *phi, double *tmp) {
  double ideal = 0., es = 0.;
  for (int n = 0; n < 2; n++) {
    memcpy(tmp, c->f[F_C0 + n], sizeof(double) * c->nf);
    fft_c2r(c, tmp);
    for (int i = 0; i < c->nx; i++)
      for (int j = 0; j < c->ny; j++)
        for (int k = 0; k < c->nz; k++) {
          const long im = IDX(c, i, j, k);
          const double cc = tmp[im], ph = phi[im];
          ideal += (1. - ph) * cc * (log(cc) - 1.);
          charge[im] += c->valency_e[n] * cc * (1. - ph);
        }
  }
  ideal *= c->P.kbt * c->dx3;
  double ext[DIM];
  for (int d = 0; d < DIM; d++)
    ext[d] = c->P.e_ext[d] * (c->P.ac ? sin(2.0 * M_PI * c->P.frequency * c->time) : 1.0);
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nz; k++) {
        const long im = IDX(c, i, j, k);
        double pot = 0.5 * c->f[F_POT][im];
        if (c->P.external_field) pot -= (ext[0] * (double)i + ext[1] * (double)j + ext[2] * (double)k) * c->dx;
        es += charge[im] * pot;
      }
  return ideal + es * c->dx3;
}

/* Set_steadystate_ion_density (operate_electrolyte.cxx:424-457): the salt
 * densities relaxed by Ion_diffusion_solver_Euler (fluid_solver.cxx:293-316)
 * -- the Nernst-Planck right-hand side of Rhs_NS_Nernst_Planck (:246-292)
 * with the fluid at rest and the potential as it is (zero before the first
 * solve: the external field alone drives the ions), an Euler step of the
 * densities on the 2/3 modes and Rescale_solute (solute_rhs.cxx:99-128) back
 * to the initial totals -- until the free energy changes by less than
 * TOL = 1e-4 (operate_electrolyte.h:22), at most 9999 steps. The free
 * energy's charge array starts as the reference's up[1] (here F_UP1, the
 * particle velocity field) and, inside the loop, as the last species' real
 * density before its rescale (Rescale_solute's working array is up[1]). */
static void steadystate_ions(ko_ctx *c) {
  double *phi = c->f[F_PHI];
  double *gp[3] = {c->f[F_F0], c->f[F_F1], c->f[F_F2]};
  double *flux[3] = {c->f[F_UP0], c->f[F_UP1], c->f[F_UP2]};
  double *sn[3] = {c->f[F_SN0], c->f[F_SN1], c->f[F_SN2]};
  double *crhs[2] = {c->f[F_CRHS0], c->f[F_CRHS1]};
  double *charge = c->f[F_WV3_0], *tmp = c->f[F_WV3_1], *scratch = c->f[F_WV3_2];
  double *pot = c->f[F_POT];
  memcpy(charge, c->f[F_UP1], sizeof(double) * c->nf);
  double f_prev = free_energy_pb(c, charge, phi, tmp);
  c->pb_iterations = 0;
  for (int m = 1; m < 10000; m++) {
    /* grad potential on the staggered grid, minus E_ext at k = 0, to nodes */
    fft_r2c(c, pot);
    a_k2da_k(c, pot, gp);
    shift_fw(c, gp);
    fft_c2r(c, pot);
    if (c->P.external_field) {
      double amp = (double)c->nx * c->ny * c->nz;
      if (c->P.ac) amp *= sin(2.0 * M_PI * c->P.frequency * c->time);
      for (int d = 0; d < DIM; d++) gp[d][0] -= c->P.e_ext[d] * amp;
    }
    for (int d = 0; d < DIM; d++) fft_c2r(c, gp[d]);
    interp_vec_normal(c, gp);
    make_surface_normal(c);
    for (int n = 0; n < 2; n++) {
      double *conc = c->f[F_C0 + n];
      truncate_23(c, conc);
      const double kl = c->P.kbt * c->onsager[n];
      for (long q = 0; q < c->nf; q++) scratch[q] = kl * conc[q];
      a_k2da_k(c, scratch, flux);
      for (int d = 0; d < DIM; d++) fft_c2r(c, flux[d]);
      memcpy(crhs[n], conc, sizeof(double) * c->nf);
      fft_c2r(c, crhs[n]);
      const double ze = c->valency_e[n], L = c->onsager[n];
      for (int i = 0; i < c->nx; i++)
        for (int j = 0; j < c->ny; j++)
          for (int k = 0; k < c->nz; k++) {
            const long im = IDX(c, i, j, k);
            const double cc = crhs[n][im];
            for (int d = 0; d < DIM; d++) flux[d][im] += cc * (L * (gp[d][im] * ze));
          }
      for (int p = 0; p < c->np; p++) {  /* Solute_impermeability, as in nssolute_solver_euler */
        pcell pc;
        particle_cell(c, c->p[p].x, &pc);
        for (int q = 0; q < c->np_domain; q++) {
          double r[3], dist;
          const long im = stencil_point(c, &pc, c->p[p].x, q, r, &dist);
          double nv[3], n2 = 0.0;
          for (int d = 0; d < DIM; d++) {
            nv[d] = sn[d][im];
            n2 += SQ(nv[d]);
          }
          if (n2 > 0.) {
            double dd = 0.;
            for (int d = 0; d < DIM; d++) dd += flux[d][im] * nv[d];
            dd /= n2;
            for (int d = 0; d < DIM; d++) flux[d][im] -= nv[d] * dd;
          }
        }
      }
      /* the fluid is at rest: the advection flux adds -0 */
      for (int d = 0; d < DIM; d++) fft_r2c(c, flux[d]);
      u_k2divergence_k(c, flux, crhs[n]);
    }
    const double dt = c->P.dt;
    for (int i = 0; i < c->nx; i++)
      for (int j = 0; j < c->ny; j++)
        for (int k = 0; k < c->nzp; k++) {
          if (!in_two_third(c, i, j, k / 2)) continue;
          const long im = IDX(c, i, j, k);
          c->f[F_C0][im] += dt * crhs[0][im];
          c->f[F_C1][im] += dt * crhs[1][im];
        }
    /* Rescale_solute: charge ends as the last species' density before its rescale */
    for (int n = 0; n < 2; n++) {
      memcpy(charge, c->f[F_C0 + n], sizeof(double) * c->nf);
      fft_c2r(c, charge);
      const double factor = c->total_solute[n] / count_single_solute(c, charge, phi);
      for (long q = 0; q < c->nf; q++) c->f[F_C0 + n][q] *= factor;
    }
    const double f_now = free_energy_pb(c, charge, phi, tmp);
    c->pb_iterations = m;
    if (fabs(f_now - f_prev) < 1e-4) break;
    f_prev = f_now;
  }
}

static void init_ions(ko_ctx *c) {
  const double z0 = c->P.valency_pos, z1 = c->P.valency_neg;
  c->valency_e[0] = z0 * c->P.elementary_charge;
  c->valency_e[1] = z1 * c->P.elementary_charge;
  c->onsager[0] = c->P.onsager_pos;
  c->onsager[1] = c->P.onsager_neg;
  set_salt_free_species(c);
  make_phi_particle(c, c->f[F_PHI]);
  double rho_inf = c->P.kbt * c->P.dielectric_cst * c->P.eps_fluid /
                   SQ(c->P.elementary_charge * c->P.debye_length * c->radius);
  double cp = rho_inf / (z0 * (z0 - z1));
  double cm = -rho_inf / (z1 * (z0 - z1));
  if (c->P.surface_charge[0] != 0.0) {
    /* Init_rho_ion -> Set_uniform_ion_charge_density_salt
     * (operate_electrolyte.cxx:738-862, 559-620): counterions of the surface
     * charges spread over the fluid volume, plus the salt density
     * kBT Dc eps_f / (e lambda_D)^2 (no radius factor on this branch) */
    double pos = 0., neg = 0.;
    for (int sp = 0; sp < c->P.n_species; sp++) {
      int cnt = 0;
      for (int n = 0; n < c->np; n++) cnt += (c->p[n].spec == sp);
      const double q = c->P.surface_charge[sp], num = (double)cnt;
      if (q < 0.) pos += fabs(q * num / z0);
      else if (q > 0.) neg += fabs(q * num / z1);
    }
    double volume_phi = 0.;
    for (int i = 0; i < c->nx; i++)
      for (int j = 0; j < c->ny; j++)
        for (int k = 0; k < c->nz; k++) volume_phi += (1. - c->f[F_PHI][IDX(c, i, j, k)]);
    rho_inf = c->P.kbt * c->P.dielectric_cst / SQ(c->P.elementary_charge * c->P.debye_length);
    rho_inf *= c->P.eps_fluid;
    cp = pos / (volume_phi * c->dx3) + rho_inf / (z0 * (z0 - z1));
    cm = neg / (volume_phi * c->dx3) + -rho_inf / (z1 * (z0 - z1));
    if (c->P.salt_free) {
      /* N_spec = 1 (Init_rho_ion, operate_electrolyte.cxx:740-787, and
       * Set_uniform_ion_charge_density_nosalt, :459-493): the counterions
       * -sum_i Q_i N_i / z_c spread evenly at Counterion_number over the
       * fluid volume (the reference's OpenMP loop there marks the density
       * private, uninitialised in each thread; this is the serial meaning) */
      double surface_ion_number = 0.;
      for (int sp = 0; sp < c->P.n_species; sp++) {
        int cnt = 0;
        for (int n = 0; n < c->np; n++) cnt += (c->p[n].spec == sp);
        surface_ion_number -= c->P.surface_charge[sp] * cnt;
      }
      const double counterion_number = surface_ion_number / c->P.valency_counterion;
      cp = counterion_number / (volume_phi * c->dx3);
      cm = 0.0;
    }
  }
  for (int n = 0; n < 2; n++) {
    double *cf = c->f[F_C0 + n];
    double val = n ? cm : cp;
    zero_real(c, cf);
    for (int i = 0; i < c->nx; i++)
      for (int j = 0; j < c->ny; j++)
        for (int k = 0; k < c->nz; k++) cf[IDX(c, i, j, k)] = 0.0 + val;
    c->total_solute[n] = count_single_solute(c, cf, c->f[F_PHI]);
    fft_r2c(c, cf);
  }
  /* INIT_profile Poisson_Boltzmann with charged particles in the salt
   * solution, more than one particle (Init_rho_ion, operate_electrolyte.cxx:
   * 834-853) */
  if (c->P.poisson_boltzmann && c->P.surface_charge[0] != 0.0 && !c->P.salt_free && c->np > 1)
    steadystate_ions(c);
}

/* main()'s initialisation after Init_Particle (sp_3d_ns.cxx:425-457) */
static void init_state(ko_ctx *c) {
  double *zeta[2] = {c->f[F_ZETA0], c->f[F_ZETA1]};
  double *u[3] = {c->f[F_U0], c->f[F_U1], c->f[F_U2]};
  for (int n = 0; n < c->np; n++)
    for (int d = 0; d < DIM; d++) c->p[n].x_nopbc[d] = c->p[n].x[d];
  /* Init_zeta_k (init_fluid.cxx:10-26): fluid at rest */
  for (int d = 0; d < DIM; d++) zero_real(c, u[d]);
  for (int d = 0; d < DIM; d++) fft_r2c(c, u[d]);
  solenoidal_uk(c, u);
  u_k2zeta_k(c, u, zeta, c->uk_dc);
  make_phi_particle_sum(c);
  make_u_particle_sum(c);
  zeta_k2u(c, zeta, c->uk_dc, u);
  f_particle_sole_and_add(c);
  u2zeta_k(c, zeta, c->uk_dc, u);
  for (int d = 0; d < DIM; d++) c->uk_dc[d] = 0.0;
  if (c->P.sw_eq == ICEP_ELECTROLYTE && c->P.dielectric) {
    for (int d = 0; d < DIM; d++) zero_real(c, c->f[F_GE0 + d]);
    init_ions(c);
    /* Init_potential_dielectric (operate_dielectric.cxx:574-609) */
    make_dielectric_field(c, c->f[F_EPS], c->f[F_GE2]);
    conc_k2charge(c, c->f[F_GE1], c->f[F_GE2], c->f[F_GE0]);
    solve_potential(c, c->f[F_GE1], c->f[F_POT], c->f[F_GE2]);
  }
}

/* ------------------------------------------------------------------------ */
/* C entry points (ctypes)                                                  */
/* ------------------------------------------------------------------------ */

ko_ctx *ko_create(const icep_params *P, const icep_particle *p, int np) {
  if (np != P->n_particles) return NULL;
  ko_ctx *c = (ko_ctx *)calloc(1, sizeof(ko_ctx));
  c->P = *P;
  c->nx = P->nx; c->ny = P->ny; c->nz = P->nz;
  c->hnz = c->nz / 2 + 1;
  c->nzp = 2 * c->hnz;
  c->nf = (long)c->nx * c->ny * c->nzp;
  c->nu = (long)c->nx * c->ny * c->nz;
  const int N[3] = {c->nx, c->ny, c->nz};
  for (int d = 0; d < DIM; d++) c->trn[d] = (N[d] + 2) / 3;
  c->dx = P->dx;
  c->dx3 = P->dx * P->dx * P->dx;
  for (int d = 0; d < DIM; d++) c->wave[d] = 2.0 * M_PI / (N[d] * P->dx);
  c->radius = P->a * P->dx;
  c->xi = P->a_xi * P->dx;
  c->hxi = 0.5 * c->xi;
  c->sigma = 2.0 * c->radius;
  c->lj_dia = c->sigma;
  double arc;
  if (P->lj_truncate > 0)
    arc = (P->lj_powers == 0) ? pow(2., 1. / 6.) : (P->lj_powers == 1) ? pow(2., 1. / 12.) : pow(2., 1. / 18.);
  else if (P->lj_truncate == 0) {
    int nmin = c->nx < c->ny ? c->nx : c->ny;
    nmin = nmin < c->nz ? nmin : c->nz;
    arc = nmin * c->dx * .5 / c->sigma;
    if (arc > 2.5) arc = 2.5;
  } else
    arc = 0.;
  c->r_cutoff = arc * c->lj_dia;
  c->nu_visc = P->eta / P->rho;
  for (int s = 0; s < ICEP_MAX_SPECIES; s++) {
    double mass = P->mass_ratio[s] * P->rho * 4. / 3. * M_PI * c->radius * c->radius * c->radius;
    c->imass[s] = 1. / mass;
    c->imoi[s] = 1. / (2. / 5. * mass * SQ(c->radius));
  }
  c->valency_e[0] = P->valency_pos * P->elementary_charge;
  c->valency_e[1] = P->valency_neg * P->elementary_charge;
  c->onsager[0] = P->onsager_pos;
  c->onsager[1] = P->onsager_neg;
  set_salt_free_species(c);
  build_sekibun(c);
  c->np = np;
  c->p = (icep_particle *)calloc(np > 0 ? np : 1, sizeof(icep_particle));
  memcpy(c->p, p, sizeof(icep_particle) * np);
  if (!P->per_particle_eps)
    for (int n = 0; n < np; n++) c->p[n].eps_p = P->eps_particle_top;
  for (int q = 0; q < F_COUNT; q++) c->f[q] = zalloc(c->nf);
  cplan_init(&c->px, c->nx);
  cplan_init(&c->py, c->ny);
  cplan_init(&c->pz, c->nz / 2);
  c->ztw = (double *)malloc(sizeof(double) * 2 * (c->nz / 2 + 1));
  for (int k = 0; k <= c->nz / 2; k++) {
    double a = -2.0 * M_PI * (double)k / (double)c->nz;
    c->ztw[2 * k] = cos(a);
    c->ztw[2 * k + 1] = sin(a);
  }
  return c;
}

void ko_destroy(ko_ctx *c) {
  if (!c) return;
  for (int q = 0; q < F_COUNT; q++) free(c->f[q]);
  free(c->p);
  free(c->sekibun);
  cplan_free(&c->px);
  cplan_free(&c->py);
  cplan_free(&c->pz);
  free(c->ztw);
  free(c);
}

int ko_np_domain(const ko_ctx *c) { return c->np_domain; }
void ko_sekibun(const ko_ctx *c, int *cells) { memcpy(cells, c->sekibun, sizeof(int) * 3 * c->np_domain); }
void ko_init_state(ko_ctx *c) { init_state(c); }
void ko_step(ko_ctx *c, int n) {
  for (int s = 0; s < n; s++) {
    time_evolution_hydro(c);
    c->time += c->P.dt;
    c->ts++;
  }
}
void ko_set_ts(ko_ctx *c, int ts, double time) { c->ts = ts; c->time = time; }
void ko_get_particles(const ko_ctx *c, icep_particle *p) { memcpy(p, c->p, sizeof(icep_particle) * c->np); }
void ko_set_particles(ko_ctx *c, const icep_particle *p) { memcpy(c->p, p, sizeof(icep_particle) * c->np); }
int ko_get_field(const ko_ctx *c, int id, double *out) {
  if (id < 0 || id >= F_COUNT) return 1;
  memcpy(out, c->f[id], sizeof(double) * c->nf);
  return 0;
}
int ko_set_field(ko_ctx *c, int id, const double *in) {
  if (id < 0 || id >= F_COUNT) return 1;
  memcpy(c->f[id], in, sizeof(double) * c->nf);
  return 0;
}
void ko_get_uk_dc(const ko_ctx *c, double *o) { memcpy(o, c->uk_dc, sizeof(double) * 3); }
void ko_set_uk_dc(ko_ctx *c, const double *o) { memcpy(c->uk_dc, o, sizeof(double) * 3); }
void ko_a2a_k(ko_ctx *c, double *a) { fft_r2c(c, a); }
void ko_a_k2a(ko_ctx *c, double *a) { fft_c2r(c, a); }
void ko_apply_A(ko_ctx *c, const double *x, double *y) { apply_A(c, x, y); }
long ko_last_iterations(const ko_ctx *c) { return c->last_iters; }
long ko_pb_iterations(const ko_ctx *c) { return c->pb_iterations; }
double ko_last_error(const ko_ctx *c) { return c->last_error; }
long ko_matvec_count(const ko_ctx *c) { return c->matvecs; }
/* MaxIter_potential of later solves (lets a timing harness cap a solve) */
void ko_set_potential_iter(ko_ctx *c, int maxit) { c->P.potential_iter = maxit; }
long ko_lj_pairs(ko_ctx *c, int *pairs, long max_pairs) {
  for (int n = 0; n < c->np; n++)
    for (int d = 0; d < DIM; d++) c->p[n].fr[d] = 0.0;
  return lj_force(c, pairs, max_pairs);
}
int ko_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Isolated calls, numbered like the reference harness's kref_call. */
enum {
  C_ZETA_K2U_K = 1, C_U_K2ZETA_K, C_U2ADVECTION_K, C_SOLENOIDAL_U, C_NS_SLAVED_EULER,
  C_MAKE_PHI_SUM, C_MAKE_U_SUM, C_F_HYDRO, C_LJ, C_POS_EULER, C_POS_AB2, C_VEL_EULER,
  C_VEL_AB2, C_DIELECTRIC_FIELD, C_BUILD_RHS, C_SOLVE_POTENTIAL, C_MAXWELL, C_NSSOLUTE_EULER,
  C_SURFACE_NORMAL, C_F_PARTICLE_SOLE, C_TRUNCATE, C_CHARGE_FIELD, C_INIT_ION, C_ZETA_K2U,
  C_CHARGE_OUTPUT
};

/* The fields of Output_dielectric_charge_field_data (output.cxx:262-320)
 * with vel, phi and charge printed: u = Zeta_k2u(zeta, uk_dc); phi = the
 * unclipped sum of Phi and up0 = the rescaled surface charge times 4 pi a^2
 * (Make_phi_qq_particle; 0/0 = NaN without charged particles);
 * up1 = (sum_n e z_n c_n) (1 - phi); up2 = eps. The concentrations are
 * transformed into scratch, not in place. */
static void charge_output(ko_ctx *c) {
  double *zeta[2] = {c->f[F_ZETA0], c->f[F_ZETA1]};
  double *u[3] = {c->f[F_U0], c->f[F_U1], c->f[F_U2]};
  double *phi = c->f[F_PHI], *up0 = c->f[F_UP0], *up1 = c->f[F_UP1], *up2 = c->f[F_UP2];
  double *c0 = c->f[F_F0], *c1 = c->f[F_F1];
  zeta_k2u(c, zeta, c->uk_dc, u);
  zero_real(c, phi);
  zero_real(c, up0);
  make_phi_qq(c, phi, up0);
  memcpy(c0, c->f[F_C0], sizeof(double) * c->nf);
  memcpy(c1, c->f[F_C1], sizeof(double) * c->nf);
  fft_c2r(c, c0);
  fft_c2r(c, c1);
  const double area = (4. * M_PI) * (c->radius * c->radius);
  for (int i = 0; i < c->nx; i++)
    for (int j = 0; j < c->ny; j++)
      for (int k = 0; k < c->nz; k++) {
        const long im = IDX(c, i, j, k);
        const double q = c->valency_e[0] * c0[im] + c->valency_e[1] * c1[im];
        up0[im] *= area;
        up1[im] = q * (1. - phi[im]);
        up2[im] = c->f[F_EPS][im];
      }
}
int ko_call(ko_ctx *c, int fn) {
  double *zeta[2] = {c->f[F_ZETA0], c->f[F_ZETA1]};
  double *u[3] = {c->f[F_U0], c->f[F_U1], c->f[F_U2]};
  double *f[3] = {c->f[F_F0], c->f[F_F1], c->f[F_F2]};
  double *adv[2] = {c->f[F_NS0_0], c->f[F_NS0_1]};
  switch (fn) {
    case C_ZETA_K2U_K: zeta_k2u_k(c, zeta, c->uk_dc, u); break;
    case C_ZETA_K2U: zeta_k2u(c, zeta, c->uk_dc, u); break;
    case C_U_K2ZETA_K: u_k2zeta_k(c, u, zeta, c->uk_dc); break;
    case C_U2ADVECTION_K: u2advection_k(c, u, adv); break;
    case C_SOLENOIDAL_U: solenoidal_u(c, u); break;
    case C_NS_SLAVED_EULER: ns_solver_slaved_euler(c); break;
    case C_MAKE_PHI_SUM: make_phi_particle_sum(c); break;
    case C_MAKE_U_SUM: make_u_particle_sum(c); break;
    case C_F_HYDRO: calc_f_hydro(c); break;
    case C_LJ:
      for (int n = 0; n < c->np; n++)
        for (int d = 0; d < DIM; d++) c->p[n].fr[d] = 0.0;
      lj_force(c, NULL, 0);
      break;
    case C_POS_EULER: md_position(c, 0); break;
    case C_POS_AB2: md_position(c, 1); break;
    case C_VEL_EULER: md_velocity(c, 0); break;
    case C_VEL_AB2: md_velocity(c, 1); break;
    case C_DIELECTRIC_FIELD: make_dielectric_field(c, c->f[F_EPS], c->f[F_WORK]); break;
    case C_BUILD_RHS: build_rhs(c, c->f[F_WORK], c->f[F_RHO]); break;
    case C_SOLVE_POTENTIAL: solve_potential(c, c->f[F_RHO], c->f[F_POT], c->f[F_WORK]); break;
    case C_MAXWELL: maxwell_force(c, f, c->f[F_RHO]); break;
    case C_NSSOLUTE_EULER: nssolute_solver_euler(c); break;
    case C_SURFACE_NORMAL: make_surface_normal(c); break;
    case C_F_PARTICLE_SOLE: {
      double *ff[3] = {c->f[F_F0], c->f[F_F1], c->f[F_F2]};
      double *up[3] = {c->f[F_UP0], c->f[F_UP1], c->f[F_UP2]};
      for (long q = 0; q < c->nf; q++)
        for (int d = 0; d < DIM; d++) ff[d][q] = up[d][q] - c->f[F_PHI][q] * u[d][q];
      solenoidal_u(c, ff);
      break;
    }
    case C_TRUNCATE: truncate_23(c, zeta[0]); truncate_23(c, zeta[1]); break;
    case C_CHARGE_FIELD: conc_k2charge(c, c->f[F_RHO], c->f[F_WORK], c->f[F_UP0]); break;
    case C_INIT_ION: init_ions(c); break;
    case C_CHARGE_OUTPUT: charge_output(c); break;
    default: return 1;
  }
  return 0;
}
