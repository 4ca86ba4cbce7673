/*
 * CPU oracle for the CCD + (T) hot path.  TEST INFRASTRUCTURE ONLY (see ccd_oracle.h).
 *
 * A plain-C complex<double> restatement of the reference Fortran solver of
 * paolofinelli/Coupled-Cluster-NuclearMatter, directory deltafull-CCMkspace/.
 * Each routine cites the reference lines it follows.  Parity status: UNPINNED
 * (no golden vectors exist in the reference and it cannot be built here).
 *
 * Build: see oracle/Makefile (gcc -O3 -fopenmp -ffp-contract=off).
 */
#include "ccd_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double _Complex zd;

/* constants module, ccm_modules.f90:76-102.  p_mass is a default-real (4-byte)
 * literal in the reference, so its double value is the float-rounded 939.565. */
#define PI 3.14159265358979
#define HBARC 197.326968
#define P_MASS ((double)939.565f)

/* chiral-like synthetic potential constants (the complex SNM workloads) */
#define CL_GA 1.27
#define CL_FPI 92.4
#define CL_MPI 138.0
#define CL_LAMBDA 450.0
#define CL_NREG 3.0
/* nucleon masses of chiral_module_andreas_with_delta.f90:56-57, :131-133 */
#define M_PROTON 9.38272046000000046e+02
#define M_NUCLEON 9.38918267117927371e+02
#define M_NEUTRON 9.39565379000000007e+02

typedef struct {
  int n;
  int *p, *q;
} plist;

struct ocl {
  ocl_params prm;
  /* basis */
  int ns, A, g;
  int *nx, *ny, *nz, *sz, *tz;
  double *kx, *ky, *kz, *e;
  double L, vol, kf, dens;
  int nk[3];          /* max n per axis */
  int tzmin, tzmax;
  int *orbitof;       /* [(nx+nk0)][(ny+nk1)][(nz+nk2)][sz idx][tz idx] */
  /* pair-sum channels, kinds 1..6 */
  int Nmin[3], Nmax[3], Nd[3];
  int *loc[7];
  int nch[7];
  int *qn[7];
  plist *L1[7], *L2[7]; /* side-1 / side-2 pair lists per kind */
  /* pair -> 1-based position maps, ns*ns grids */
  int *hh_hhhh, *hh_hhhp, *hh_hhpp, *hp_hphp, *hp_hhhp, *pp_hhpp, *pp_pppp, *hp_hppp, *pp_hppp;
  /* particle-hole channels, kinds 1 phhp, 2 hphp, 3 hpph */
  int Dmin[3], Dmax[3], Dd[3];
  int *locph[4];
  int nchph[4];
  int *qnph[4];
  plist *P1[4], *P2[4];
  int *ph_ph_phhp, *hp_ph_phhp, *hp_ph_hphp, *hp_ph_hpph, *ph_ph_hpph;
  /* interaction */
  double lec[9];
  zd **V_hhhh, **V_hhhp, **V_hhpp, **V_hphp, **V_pppp, **V_hppp;
  zd *fock;
  zd e0;
  /* amplitudes and intermediates */
  zd **T, **R, **Tph, **Rph;
  zd *d2ij, *d2ab;
  zd *I6, *I7;
  int have_triples_setup;
  /* t3 channels */
  int t3n;
  int *t3qn;
  int *t3hhh_n, *t3ppp_n;
  int **t3hhh, **t3ppp;
  /* diis */
  int subspace, diis_step, nstep;
  int64_t n_diis;
  zd *t2_diis, *t2_diisd;
};

/* ------------------------------------------------------------------ */
/* small helpers                                                        */
/* ------------------------------------------------------------------ */
static void *xcalloc(size_t n, size_t s) {
  void *p = calloc(n ? n : 1, s ? s : 1);
  if (!p) {
    fprintf(stderr, "oracle: out of memory (%zu x %zu)\n", n, s);
    abort();
  }
  return p;
}

int ocl_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* delta(a,b) of ccm_library.f90:70-76 */
static inline double kdelta(int a, int b) { return a == b ? 1.0 : 0.0; }

/* chp_sigma_dot_sigma / chp_tau_dot_tau (chiral_module_andreas_with_delta.f90:2944-3031,
 * :3033-3120): with the j_x, j_y, j_z ladder forms every value is an exact small
 * integer: m1*m2 without flips, 2 for an exchange flip, 0 otherwise. */
static inline double pauli_dot(int m1, int m2, int m3, int m4) {
  if (m1 == m3 && m2 == m4) return (double)(m1 * m2);
  if (m1 == m4 && m2 == m3 && m1 != m2) return 2.0;
  return 0.0;
}

/* 2x2 spinor matrix element <chi_a| (w . sigma) |chi_b>, spin index 0 = up (ms=+1)
 * as nint(1.5-0.5*ms) of chiral_module_andreas_with_delta.f90:3158-3165 */
static inline zd wsigma(int ma, int mb, const double w[3]) {
  int ia = ma > 0 ? 0 : 1, ib = mb > 0 ? 0 : 1;
  if (ia == 0 && ib == 0) return w[2];
  if (ia == 1 && ib == 1) return -w[2];
  if (ia == 0 && ib == 1) return w[0] - I * w[1];
  return w[0] + I * w[1];
}

/* ------------------------------------------------------------------ */
/* Numerical-Recipes style index sort as written at ccm_main.f90:2654-2732
 * (M=7 insertion cut-off, median-of-three quicksort).  Arrays are 1-based. */
static void nr_indexx(int n, const double *arr, int *indx) {
  const int M = 7;
  int istack[256];
  int i, indxt, ir, itemp, j, jstack, k, l;
  double a;
  for (j = 1; j <= n; j++) indx[j] = j;
  jstack = 0;
  l = 1;
  ir = n;
  for (;;) {
    if (ir - l < M) {
      for (j = l + 1; j <= ir; j++) {
        indxt = indx[j];
        a = arr[indxt];
        for (i = j - 1; i >= 1; i--) {
          if (arr[indx[i]] <= a) break;
          indx[i + 1] = indx[i];
        }
        if (i < 1) i = 0;
        indx[i + 1] = indxt;
      }
      if (jstack == 0) return;
      ir = istack[jstack];
      l = istack[jstack - 1];
      jstack -= 2;
    } else {
      k = (l + ir) / 2;
      itemp = indx[k]; indx[k] = indx[l + 1]; indx[l + 1] = itemp;
      if (arr[indx[l + 1]] > arr[indx[ir]]) { itemp = indx[l + 1]; indx[l + 1] = indx[ir]; indx[ir] = itemp; }
      if (arr[indx[l]] > arr[indx[ir]]) { itemp = indx[l]; indx[l] = indx[ir]; indx[ir] = itemp; }
      if (arr[indx[l + 1]] > arr[indx[l]]) { itemp = indx[l + 1]; indx[l + 1] = indx[l]; indx[l] = itemp; }
      i = l + 1;
      j = ir;
      indxt = indx[l];
      a = arr[indxt];
      for (;;) {
        do i++; while (arr[indx[i]] < a);
        do j--; while (arr[indx[j]] > a);
        if (j < i) break;
        itemp = indx[i]; indx[i] = indx[j]; indx[j] = itemp;
      }
      indx[l] = indx[j];
      indx[j] = indxt;
      jstack += 2;
      if (jstack >= 256) { fprintf(stderr, "oracle: index sort stack overflow\n"); abort(); }
      if (ir - i + 1 >= j - l) {
        istack[jstack] = ir;
        istack[jstack - 1] = i;
        ir = j - 1;
      } else {
        istack[jstack] = j - 1;
        istack[jstack - 1] = l;
        l = i;
      }
    }
  }
}

/* ------------------------------------------------------------------ */
/* basis: allocate_sp_data (ccm_main.f90:878-1000) + setup_sp_data (:1003-1197) */
static void build_basis(ocl_t *o) {
  const ocl_params *p = &o->prm;
  int nmax = p->nmax;
  o->A = p->A;
  if (p->snm) {
    o->tzmin = -1; o->tzmax = 1;
    o->dens = p->rho;
    o->kf = pow(3.0 * PI * PI * o->dens / 2.0, 1.0 / 3.0);
  } else {
    o->tzmin = 1; o->tzmax = 1;
    o->dens = p->rho;
    o->kf = pow(3.0 * PI * PI * o->dens, 1.0 / 3.0);
  }
  /* lx = (real(below_ef)/dens)**(1/3) ; volume = lx*ly*lz */
  o->L = pow((double)(float)o->A / o->dens, 1.0 / 3.0);
  o->vol = o->L * o->L * o->L;
  int nkm = 2 * nmax + 1;
  int szmin = -1, szmax = 1;
  o->g = ((szmax - szmin + 2) * (o->tzmax - o->tzmin + 2)) / 4;
  o->ns = o->g * nkm * nkm * nkm;
  double *mesh[3];
  for (int d = 0; d < 3; d++) {
    mesh[d] = (double *)xcalloc(nkm, sizeof(double));
    double th = p->theta[d];
    mesh[d][0] = th / o->L;
    int ii = 0;
    for (int i = 1; i <= nmax; i++) {
      ii++;
      mesh[d][ii] = (2.0 * (double)(-i) * PI + th) / o->L;
      ii++;
      mesh[d][ii] = (2.0 * (double)(i)*PI + th) / o->L;
    }
  }
  int npt = nkm * nkm * nkm;
  double *erg = (double *)xcalloc(npt + 1, sizeof(double));
  int *indx_inv = (int *)xcalloc(npt + 1, sizeof(int));
  int *indx = (int *)xcalloc(npt + 1, sizeof(int));
  int ii = 0;
  for (int i = 0; i < nkm; i++)
    for (int j = 0; j < nkm; j++)
      for (int k = 0; k < nkm; k++) {
        ii++;
        double x = mesh[0][i] * mesh[0][i];
        double y = mesh[1][j] * mesh[1][j];
        double z = mesh[2][k] * mesh[2][k];
        erg[ii] = (x + y) + z;
      }
  nr_indexx(npt, erg, indx_inv);
  for (int i = 1; i <= npt; i++) indx[indx_inv[i]] = i;

  int ns = o->ns;
  o->nx = (int *)xcalloc(ns, sizeof(int));
  o->ny = (int *)xcalloc(ns, sizeof(int));
  o->nz = (int *)xcalloc(ns, sizeof(int));
  o->sz = (int *)xcalloc(ns, sizeof(int));
  o->tz = (int *)xcalloc(ns, sizeof(int));
  o->kx = (double *)xcalloc(ns, sizeof(double));
  o->ky = (double *)xcalloc(ns, sizeof(double));
  o->kz = (double *)xcalloc(ns, sizeof(double));
  o->e = (double *)xcalloc(ns, sizeof(double));
  ii = 0;
  int tzstep = (o->tzmax - o->tzmin + 2) / 2;
  for (int i = 0; i < nkm; i++)
    for (int j = 0; j < nkm; j++)
      for (int k = 0; k < nkm; k++) {
        ii++;
        int jj = indx[ii];
        int is = 0;
        for (int s = szmin; s <= szmax; s += 2) {
          is++;
          int it = 0;
          for (int t = o->tzmin; t <= o->tzmax; t += tzstep) {
            it++;
            int kk = o->g * (jj - 1) + 2 * (it - 1) + is; /* 1-based */
            int c = kk - 1;
            o->kx[c] = mesh[0][i];
            o->ky[c] = mesh[1][j];
            o->kz[c] = mesh[2][k];
            o->nx[c] = (int)lround(((mesh[0][i] * o->L - p->theta[0]) / 2.0) / PI);
            o->ny[c] = (int)lround(((mesh[1][j] * o->L - p->theta[1]) / 2.0) / PI);
            o->nz[c] = (int)lround(((mesh[2][k] * o->L - p->theta[2]) / 2.0) / PI);
            o->sz[c] = s;
            o->tz[c] = t;
            double k2 = (o->kx[c] * o->kx[c] + o->ky[c] * o->ky[c]) + o->kz[c] * o->kz[c];
            o->e[c] = k2 * (HBARC * HBARC) / P_MASS / 2.0;
          }
        }
      }
  for (int d = 0; d < 3; d++) free(mesh[d]);
  free(erg); free(indx_inv); free(indx);

  o->nk[0] = o->nk[1] = o->nk[2] = 0;
  for (int i = 0; i < ns; i++) {
    if (o->nx[i] > o->nk[0]) o->nk[0] = o->nx[i];
    if (o->ny[i] > o->nk[1]) o->nk[1] = o->ny[i];
    if (o->nz[i] > o->nk[2]) o->nk[2] = o->nz[i];
  }
  int dx = 2 * o->nk[0] + 1, dy = 2 * o->nk[1] + 1, dz = 2 * o->nk[2] + 1;
  o->orbitof = (int *)xcalloc((size_t)dx * dy * dz * 2 * 2, sizeof(int));
  for (int i = 0; i < ns; i++) {
    size_t idx = ((((size_t)(o->nx[i] + o->nk[0]) * dy + (o->ny[i] + o->nk[1])) * dz +
                   (o->nz[i] + o->nk[2])) * 2 + (o->sz[i] > 0)) * 2 + (o->tz[i] > 0);
    o->orbitof[idx] = i + 1;
  }
}

/* orbitof(nx,ny,nz,sz,tz): 0-based orbital or -1 (absent) */
static inline int orbitof(const ocl_t *o, int nx, int ny, int nz, int sz, int tz) {
  if (nx < -o->nk[0] || nx > o->nk[0] || ny < -o->nk[1] || ny > o->nk[1] || nz < -o->nk[2] ||
      nz > o->nk[2])
    return -1;
  if (tz < o->tzmin || tz > o->tzmax) return -1;
  int dy = 2 * o->nk[1] + 1, dz = 2 * o->nk[2] + 1;
  size_t idx = ((((size_t)(nx + o->nk[0]) * dy + (ny + o->nk[1])) * dz + (nz + o->nk[2])) * 2 +
                (sz > 0)) * 2 + (tz > 0);
  return o->orbitof[idx] - 1;
}

/* ------------------------------------------------------------------ */
/* potentials                                                           */
/* ------------------------------------------------------------------ */

/* vmom_minnesota, chiral_module_andreas_with_delta.f90:8980-9111 */
static double minnesota(const ocl_t *o, int p, int q, int r, int s) {
  if (o->nx[p] + o->nx[q] != o->nx[r] + o->nx[s]) return 0.0;
  if (o->ny[p] + o->ny[q] != o->ny[r] + o->ny[s]) return 0.0;
  if (o->nz[p] + o->nz[q] != o->nz[r] + o->nz[s]) return 0.0;
  if (o->tz[p] + o->tz[q] != o->tz[r] + o->tz[s]) return 0.0;
  int m1 = o->sz[p], m2 = o->sz[q], m3 = o->sz[r], m4 = o->sz[s];
  int t1 = o->tz[p], t2 = o->tz[q], t3 = o->tz[r], t4 = o->tz[s];
  double k1[3] = {o->kx[p], o->ky[p], o->kz[p]};
  double k2[3] = {o->kx[q], o->ky[q], o->kz[q]};
  double k3[3] = {o->kx[r], o->ky[r], o->kz[r]};
  double k4[3] = {o->kx[s], o->ky[s], o->kz[s]};
  double qt[3];
  for (int d = 0; d < 3; d++) {
    double prel = 0.5 * (k1[d] - k2[d]);
    double pprel = 0.5 * (k3[d] - k4[d]);
    qt[d] = prel - pprel;
  }
  double q2 = (qt[0] * qt[0] + qt[1] * qt[1]) + qt[2] * qt[2];
  double v0r, v0t, v0s, kr, kt, ks;
  if (o->prm.minnesota_f32_literals) {
    v0r = (double)200.0f; v0t = (double)178.0f; v0s = (double)91.85f;
    kr = (double)1.487f; kt = (double)0.639f; ks = (double)0.465f;
  } else {
    v0r = 200.0; v0t = 178.0; v0s = 91.85; kr = 1.487; kt = 0.639; ks = 0.465;
  }
  double pi15 = pow(PI, 1.5);
  double vr = v0r * pi15 * exp(-q2 / (4.0 * kr)) / pow(kr, 1.5);
  double vt = -v0t * pi15 * exp(-q2 / (4.0 * kt)) / pow(kt, 1.5);
  double vs = -v0s * pi15 * exp(-q2 / (4.0 * ks)) / pow(ks, 1.5);
  double dm = kdelta(m1, m3) * kdelta(m2, m4);
  double dt = kdelta(t1, t3) * kdelta(t2, t4);
  double tt = pauli_dot(t1, t2, t3, t4);
  double ss = pauli_dot(m1, m2, m3, m4);
  vr = vr * (3.0 * dm * dt - tt * dm - ss * dt - tt * ss) / 8.0;
  vs = vs * (3.0 * dm * dt + tt * dm - 3.0 * ss * dt - tt * ss) / 16.0;
  vt = vt * (3.0 * dm * dt - 3.0 * tt * dm + ss * dt - tt * ss) / 16.0;
  double vdir = (vs + vr) + vt;
  return vdir / o->vol;
}

/* Chiral-like synthetic kind: the operator structure of chiral_pot
 * (chiral_module_andreas_with_delta.f90:5879-6301) restricted to one-pion exchange
 * (OPE :1110-1121, sigma1.q sigma2.q :3145-3173, tau.tau :3033-3120), the LO contacts
 * CS/CT and the seven NLO contacts (:6123-6156, spin.(q x k) :3235-3264), times the
 * relativity factor and the non-local regulator freg (:3336-3351), and hbarc^3/volume. */
static zd chiral_like(const ocl_t *o, int p, int q, int r, int s) {
  if (o->nx[p] + o->nx[q] != o->nx[r] + o->nx[s]) return 0.0;
  if (o->ny[p] + o->ny[q] != o->ny[r] + o->ny[s]) return 0.0;
  if (o->nz[p] + o->nz[q] != o->nz[r] + o->nz[s]) return 0.0;
  if (o->tz[p] + o->tz[q] != o->tz[r] + o->tz[s]) return 0.0;
  int m1 = o->sz[p], m2 = o->sz[q], m3 = o->sz[r], m4 = o->sz[s];
  int t1 = o->tz[p], t2 = o->tz[q], t3 = o->tz[r], t4 = o->tz[s];
  double k1[3] = {o->kx[p] * HBARC, o->ky[p] * HBARC, o->kz[p] * HBARC};
  double k2[3] = {o->kx[q] * HBARC, o->ky[q] * HBARC, o->kz[q] * HBARC};
  double k3[3] = {o->kx[r] * HBARC, o->ky[r] * HBARC, o->kz[r] * HBARC};
  double k4[3] = {o->kx[s] * HBARC, o->ky[s] * HBARC, o->kz[s] * HBARC};
  double prel[3], pprel[3], km[3], qt[3], qxk[3];
  for (int d = 0; d < 3; d++) {
    prel[d] = 0.5 * (k1[d] - k2[d]);
    pprel[d] = 0.5 * (k3[d] - k4[d]);
    km[d] = 0.5 * (prel[d] + pprel[d]);
    qt[d] = prel[d] - pprel[d];
  }
  double p2 = (prel[0] * prel[0] + prel[1] * prel[1]) + prel[2] * prel[2];
  double pp2 = (pprel[0] * pprel[0] + pprel[1] * pprel[1]) + pprel[2] * pprel[2];
  double km2 = (km[0] * km[0] + km[1] * km[1]) + km[2] * km[2];
  double q2 = (qt[0] * qt[0] + qt[1] * qt[1]) + qt[2] * qt[2];
  qxk[0] = qt[1] * km[2] - qt[2] * km[1];
  qxk[1] = qt[2] * km[0] - qt[0] * km[2];
  qxk[2] = qt[0] * km[1] - qt[1] * km[0];
  int tsum = (t1 + t2) / 2;
  double mn = tsum < 0 ? M_PROTON : (tsum == 0 ? M_NUCLEON : M_NEUTRON);
  double rel = mn / sqrt(sqrt((mn * mn + p2) * (mn * mn + pp2)));
  double dm = kdelta(m1, m3) * kdelta(m2, m4);
  double dt = kdelta(t1, t3) * kdelta(t2, t4);
  double tt = pauli_dot(t1, t2, t3, t4);
  double ss = pauli_dot(m1, m2, m3, m4);
  zd sq = wsigma(m1, m3, qt) * wsigma(m2, m4, qt);
  zd sk = wsigma(m1, m3, km) * wsigma(m2, m4, km);
  zd half_mi = -0.5 * I;
  zd sl = half_mi * wsigma(m1, m3, qxk) * kdelta(m2, m4) + half_mi * wsigma(m2, m4, qxk) * kdelta(m1, m3);
  double c2 = (CL_GA * CL_GA) / (4.0 * CL_FPI * CL_FPI);
  double ope = -1.0 * c2 / (q2 + CL_MPI * CL_MPI);
  zd vlo = ope * sq * tt;
  const double *c = o->lec;
  zd cont_lo = c[0] * dm * dt + c[1] * ss * dt;
  zd cont_nlo = c[2] * q2 * dm * dt + c[3] * km2 * dm * dt + c[4] * q2 * ss * dt +
                c[5] * km2 * ss * dt + c[6] * sl * dt + c[7] * sq * dt + c[8] * sk * dt;
  double l2n = pow(CL_LAMBDA, 2.0 * CL_NREG);
  double freg = exp(-(pow(p2, CL_NREG) / l2n + pow(pp2, CL_NREG) / l2n));
  zd vdir = (vlo + cont_lo + cont_nlo) * rel * freg;
  return (HBARC * HBARC * HBARC) * vdir / o->vol;
}

static inline zd vbare(const ocl_t *o, int p, int q, int r, int s) {
  if (o->prm.potential == OCL_POT_CHIRAL_LIKE) return chiral_like(o, p, q, r, s);
  return minnesota(o, p, q, r, s);
}

/* antisymmetrized element as formed at ccm_iter.f90:854 */
static inline zd vA(const ocl_t *o, int p, int q, int r, int s) {
  return vbare(o, p, q, r, s) - vbare(o, p, q, s, r);
}

/* splitmix64 draw of the contact LECs: centre*(0.5+u), u in [0,1) */
static uint64_t sm64(uint64_t *st) {
  uint64_t z = (*st += 0x9e3779b97f4a7c15ULL);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
static void draw_lecs(ocl_t *o) {
  /* centres in 10^4 GeV^-2 (CS, CT) and 10^4 GeV^-4 (C1..C7), converted to MeV units as
   * at chiral_module_andreas_with_delta.f90:586-596 (x1e-2 MeV^-2, x1e-8 MeV^-4), with the
   * 1/(16 pi) normalisation the reference applies when it forms its operator LECs
   * (CS = (c1s0+3 c3s1)/16/pi, :599-600; cnlo(i) = (...)/(16 pi), :604-614) */
  const double centre[9] = {-0.1, 0.01, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1};
  uint64_t st = o->prm.lec_seed;
  for (int i = 0; i < 9; i++) {
    double u = (double)(sm64(&st) >> 11) * 0x1.0p-53;
    double v = centre[i] * (0.5 + u);
    o->lec[i] = v * (i < 2 ? 1.0e-2 : 1.0e-8) / (16.0 * PI);
  }
}

/* ------------------------------------------------------------------ */
/* channels: setup_channel_structures (ccm_iter.f90:175-812)            */
/* ------------------------------------------------------------------ */
static inline size_t gidx(const int *mn, const int *dd, int tz, int X, int Y, int Z) {
  return (((size_t)(tz + 1) * dd[0] + (X - mn[0])) * dd[1] + (Y - mn[1])) * dd[2] + (Z - mn[2]);
}
static inline int in_range(const int *mn, const int *mx, int X, int Y, int Z) {
  return X >= mn[0] && X <= mx[0] && Y >= mn[1] && Y <= mx[1] && Z >= mn[2] && Z <= mx[2];
}
/* locate_channel(kind, tz, N): 1-based id or 0 */
static inline int locate(const ocl_t *o, int kind, int tz, int X, int Y, int Z) {
  if (!in_range(o->Nmin, o->Nmax, X, Y, Z) || tz < -1 || tz > 1) return 0;
  return o->loc[kind][gidx(o->Nmin, o->Nd, tz, X, Y, Z)];
}
static inline int locate_ph(const ocl_t *o, int kind, int tz, int X, int Y, int Z) {
  if (!in_range(o->Dmin, o->Dmax, X, Y, Z) || tz < -1 || tz > 1) return 0;
  return o->locph[kind][gidx(o->Dmin, o->Dd, tz, X, Y, Z)];
}
#define PIDX(o, a, b) ((size_t)(a) * (o)->ns + (b))

static void plist_push(plist *l, int cap, int p, int q) {
  (void)cap;
  l->p[l->n] = p;
  l->q[l->n] = q;
  l->n++;
}
static plist *plists_alloc(int n, const int *sizes) {
  plist *L = (plist *)xcalloc(n, sizeof(plist));
  for (int i = 0; i < n; i++) {
    L[i].p = (int *)xcalloc(sizes[i], sizeof(int));
    L[i].q = (int *)xcalloc(sizes[i], sizeof(int));
  }
  return L;
}

static void build_channels(ocl_t *o) {
  int ns = o->ns, A = o->A;
  for (int d = 0; d < 3; d++) { o->Nmin[d] = 1000; o->Nmax[d] = -1000; }
  for (int i = 0; i < ns; i++)
    for (int j = 0; j < ns; j++) {
      int s[3] = {o->nx[i] + o->nx[j], o->ny[i] + o->ny[j], o->nz[i] + o->nz[j]};
      for (int d = 0; d < 3; d++) {
        if (s[d] > o->Nmax[d]) o->Nmax[d] = s[d];
        if (s[d] < o->Nmin[d]) o->Nmin[d] = s[d];
      }
    }
  for (int d = 0; d < 3; d++) o->Nd[d] = o->Nmax[d] - o->Nmin[d] + 1;
  size_t gsz = (size_t)3 * o->Nd[0] * o->Nd[1] * o->Nd[2];
  int *num[4];
  for (int k = 1; k <= 3; k++) num[k] = (int *)xcalloc(gsz, sizeof(int));
  for (int k = 1; k <= 6; k++) o->loc[k] = (int *)xcalloc(gsz, sizeof(int));
  for (int a = 0; a < ns; a++)
    for (int b = 0; b < ns; b++) {
      int tz = (o->tz[a] + o->tz[b]) / 2;
      size_t g = gidx(o->Nmin, o->Nd, tz, o->nx[a] + o->nx[b], o->ny[a] + o->ny[b], o->nz[a] + o->nz[b]);
      if (a < A && b < A) num[1][g]++;
      if (a < A && b >= A) num[2][g]++;
      if (a >= A && b >= A) num[3][g]++;
    }
  for (int k = 1; k <= 6; k++) o->nch[k] = 0;
  for (int tz = -1; tz <= 1; tz++)
    for (int X = o->Nmin[0]; X <= o->Nmax[0]; X++)
      for (int Y = o->Nmin[1]; Y <= o->Nmax[1]; Y++)
        for (int Z = o->Nmin[2]; Z <= o->Nmax[2]; Z++) {
          size_t g = gidx(o->Nmin, o->Nd, tz, X, Y, Z);
          if (num[1][g] != 0) o->loc[1][g] = ++o->nch[1];
          if (num[1][g] * num[2][g] != 0) o->loc[2][g] = ++o->nch[2];
          if (num[1][g] * num[3][g] != 0) o->loc[3][g] = ++o->nch[3];
          if (num[2][g] != 0) o->loc[4][g] = ++o->nch[4];
          if (num[1][g] * num[3][g] != 0) o->loc[6][g] = ++o->nch[6];
        }
  for (int k = 1; k <= 6; k++) {
    if (k == 5) continue;
    o->qn[k] = (int *)xcalloc((size_t)4 * (o->nch[k] + 1), sizeof(int));
  }
  for (int tz = -1; tz <= 1; tz++)
    for (int X = o->Nmin[0]; X <= o->Nmax[0]; X++)
      for (int Y = o->Nmin[1]; Y <= o->Nmax[1]; Y++)
        for (int Z = o->Nmin[2]; Z <= o->Nmax[2]; Z++) {
          size_t g = gidx(o->Nmin, o->Nd, tz, X, Y, Z);
          for (int k = 1; k <= 6; k++) {
            if (k == 5 || o->loc[k][g] == 0) continue;
            int *q = o->qn[k] + 4 * (o->loc[k][g] - 1);
            q[0] = tz; q[1] = X; q[2] = Y; q[3] = Z;
          }
        }
  /* per-channel pair counts */
  int *s1[7], *s2[7];
  for (int k = 1; k <= 6; k++) {
    if (k == 5) continue;
    s1[k] = (int *)xcalloc(o->nch[k] + 1, sizeof(int));
    s2[k] = (int *)xcalloc(o->nch[k] + 1, sizeof(int));
  }
  for (int tz = -1; tz <= 1; tz++)
    for (int X = o->Nmin[0]; X <= o->Nmax[0]; X++)
      for (int Y = o->Nmin[1]; Y <= o->Nmax[1]; Y++)
        for (int Z = o->Nmin[2]; Z <= o->Nmax[2]; Z++) {
          size_t g = gidx(o->Nmin, o->Nd, tz, X, Y, Z);
          int c;
          if ((c = o->loc[1][g])) s1[1][c - 1] = num[1][g];
          if ((c = o->loc[2][g])) { s1[2][c - 1] = num[1][g]; s2[2][c - 1] = num[2][g]; }
          if ((c = o->loc[3][g])) { s1[3][c - 1] = num[1][g]; s2[3][c - 1] = num[3][g]; }
          if ((c = o->loc[4][g])) s1[4][c - 1] = num[2][g];
          if ((c = o->loc[6][g])) s1[6][c - 1] = num[3][g];
        }
  o->L1[1] = plists_alloc(o->nch[1], s1[1]);
  o->L1[2] = plists_alloc(o->nch[2], s1[2]);
  o->L2[2] = plists_alloc(o->nch[2], s2[2]);
  o->L1[3] = plists_alloc(o->nch[3], s1[3]);
  o->L2[3] = plists_alloc(o->nch[3], s2[3]);
  o->L1[4] = plists_alloc(o->nch[4], s1[4]);
  o->L1[6] = plists_alloc(o->nch[6], s1[6]);
  for (int k = 1; k <= 6; k++) {
    if (k == 5) continue;
    free(s1[k]); free(s2[k]);
  }
  size_t nn = (size_t)ns * ns;
  o->hh_hhhh = (int *)xcalloc(nn, sizeof(int));
  o->hh_hhhp = (int *)xcalloc(nn, sizeof(int));
  o->hh_hhpp = (int *)xcalloc(nn, sizeof(int));
  o->hp_hphp = (int *)xcalloc(nn, sizeof(int));
  o->hp_hhhp = (int *)xcalloc(nn, sizeof(int));
  o->pp_hhpp = (int *)xcalloc(nn, sizeof(int));
  o->pp_pppp = (int *)xcalloc(nn, sizeof(int));
  /* hh configurations, ccm_iter.f90:415-481 */
  for (int a = 0; a < A; a++)
    for (int b = 0; b < A; b++) {
      int tz = (o->tz[a] + o->tz[b]) / 2;
      int X = o->nx[a] + o->nx[b], Y = o->ny[a] + o->ny[b], Z = o->nz[a] + o->nz[b];
      int c;
      if ((c = locate(o, 1, tz, X, Y, Z))) {
        plist_push(&o->L1[1][c - 1], 0, a, b);
        o->hh_hhhh[PIDX(o, a, b)] = o->L1[1][c - 1].n;
      }
      if ((c = locate(o, 2, tz, X, Y, Z))) {
        plist_push(&o->L1[2][c - 1], 0, a, b);
        o->hh_hhhp[PIDX(o, a, b)] = o->L1[2][c - 1].n;
      }
      if ((c = locate(o, 3, tz, X, Y, Z))) {
        plist_push(&o->L1[3][c - 1], 0, a, b);
        o->hh_hhpp[PIDX(o, a, b)] = o->L1[3][c - 1].n;
      }
    }
  /* hp configurations, ccm_iter.f90:486-550 */
  for (int a = 0; a < A; a++)
    for (int b = A; b < ns; b++) {
      int tz = (o->tz[a] + o->tz[b]) / 2;
      int X = o->nx[a] + o->nx[b], Y = o->ny[a] + o->ny[b], Z = o->nz[a] + o->nz[b];
      int c;
      if ((c = locate(o, 2, tz, X, Y, Z))) {
        plist_push(&o->L2[2][c - 1], 0, a, b);
        o->hp_hhhp[PIDX(o, a, b)] = o->L2[2][c - 1].n;
      }
      if ((c = locate(o, 4, tz, X, Y, Z))) {
        plist_push(&o->L1[4][c - 1], 0, a, b);
        o->hp_hphp[PIDX(o, a, b)] = o->L1[4][c - 1].n;
      }
    }
  /* pp configurations, ccm_iter.f90:556-603 */
  for (int a = A; a < ns; a++)
    for (int b = A; b < ns; b++) {
      int tz = (o->tz[a] + o->tz[b]) / 2;
      int X = o->nx[a] + o->nx[b], Y = o->ny[a] + o->ny[b], Z = o->nz[a] + o->nz[b];
      int c;
      if ((c = locate(o, 3, tz, X, Y, Z))) {
        plist_push(&o->L2[3][c - 1], 0, a, b);
        o->pp_hhpp[PIDX(o, a, b)] = o->L2[3][c - 1].n;
      }
      if ((c = locate(o, 6, tz, X, Y, Z)) && locate(o, 3, tz, X, Y, Z)) {
        plist_push(&o->L1[6][c - 1], 0, a, b);
        o->pp_pppp[PIDX(o, a, b)] = o->L1[6][c - 1].n;
      }
    }
  for (int k = 1; k <= 3; k++) free(num[k]);
}

/* setup_ph_channel_structures, ccm_iter.f90:1816-2105 */
static void build_ph_channels(ocl_t *o) {
  int ns = o->ns, A = o->A;
  for (int d = 0; d < 3; d++) { o->Dmin[d] = 1000; o->Dmax[d] = -1000; }
  for (int i = 0; i < ns; i++)
    for (int j = 0; j < ns; j++) {
      int s[3] = {o->nx[i] - o->nx[j], o->ny[i] - o->ny[j], o->nz[i] - o->nz[j]};
      for (int d = 0; d < 3; d++) {
        if (s[d] > o->Dmax[d]) o->Dmax[d] = s[d];
        if (s[d] < o->Dmin[d]) o->Dmin[d] = s[d];
      }
    }
  for (int d = 0; d < 3; d++) o->Dd[d] = o->Dmax[d] - o->Dmin[d] + 1;
  size_t gsz = (size_t)3 * o->Dd[0] * o->Dd[1] * o->Dd[2];
  int *num1 = (int *)xcalloc(gsz, sizeof(int)), *num2 = (int *)xcalloc(gsz, sizeof(int));
  for (int k = 1; k <= 3; k++) o->locph[k] = (int *)xcalloc(gsz, sizeof(int));
  for (int a = 0; a < ns; a++)
    for (int b = 0; b < ns; b++) {
      int tz = (o->tz[a] - o->tz[b]) / 2;
      size_t g = gidx(o->Dmin, o->Dd, tz, o->nx[a] - o->nx[b], o->ny[a] - o->ny[b], o->nz[a] - o->nz[b]);
      if (a < A && b >= A) num1[g]++;
      if (a >= A && b < A) num2[g]++;
    }
  for (int k = 1; k <= 3; k++) o->nchph[k] = 0;
  for (int tz = -1; tz <= 1; tz++)
    for (int X = o->Dmin[0]; X <= o->Dmax[0]; X++)
      for (int Y = o->Dmin[1]; Y <= o->Dmax[1]; Y++)
        for (int Z = o->Dmin[2]; Z <= o->Dmax[2]; Z++) {
          size_t g = gidx(o->Dmin, o->Dd, tz, X, Y, Z);
          if (num2[g] * num1[g] != 0) o->locph[1][g] = ++o->nchph[1];
          if (num1[g] != 0) o->locph[2][g] = ++o->nchph[2];
          if (num1[g] * num2[g] != 0) o->locph[3][g] = ++o->nchph[3];
        }
  int *s1[4], *s2[4];
  for (int k = 1; k <= 3; k++) {
    o->qnph[k] = (int *)xcalloc((size_t)4 * (o->nchph[k] + 1), sizeof(int));
    s1[k] = (int *)xcalloc(o->nchph[k] + 1, sizeof(int));
    s2[k] = (int *)xcalloc(o->nchph[k] + 1, sizeof(int));
  }
  for (int tz = -1; tz <= 1; tz++)
    for (int X = o->Dmin[0]; X <= o->Dmax[0]; X++)
      for (int Y = o->Dmin[1]; Y <= o->Dmax[1]; Y++)
        for (int Z = o->Dmin[2]; Z <= o->Dmax[2]; Z++) {
          size_t g = gidx(o->Dmin, o->Dd, tz, X, Y, Z);
          for (int k = 1; k <= 3; k++) {
            int c = o->locph[k][g];
            if (!c) continue;
            int *q = o->qnph[k] + 4 * (c - 1);
            q[0] = tz; q[1] = X; q[2] = Y; q[3] = Z;
            if (k == 1) { s1[k][c - 1] = num2[g]; s2[k][c - 1] = num1[g]; }
            if (k == 2) { s1[k][c - 1] = num1[g]; }
            if (k == 3) { s1[k][c - 1] = num1[g]; s2[k][c - 1] = num2[g]; }
          }
        }
  o->P1[1] = plists_alloc(o->nchph[1], s1[1]);
  o->P2[1] = plists_alloc(o->nchph[1], s2[1]);
  o->P1[2] = plists_alloc(o->nchph[2], s1[2]);
  o->P1[3] = plists_alloc(o->nchph[3], s1[3]);
  o->P2[3] = plists_alloc(o->nchph[3], s2[3]);
  for (int k = 1; k <= 3; k++) { free(s1[k]); free(s2[k]); }
  size_t nn = (size_t)ns * ns;
  o->ph_ph_phhp = (int *)xcalloc(nn, sizeof(int));
  o->hp_ph_phhp = (int *)xcalloc(nn, sizeof(int));
  o->hp_ph_hphp = (int *)xcalloc(nn, sizeof(int));
  o->hp_ph_hpph = (int *)xcalloc(nn, sizeof(int));
  o->ph_ph_hpph = (int *)xcalloc(nn, sizeof(int));
  for (int a = 0; a < A; a++)
    for (int b = A; b < ns; b++) {
      int tz = (o->tz[a] - o->tz[b]) / 2;
      int X = o->nx[a] - o->nx[b], Y = o->ny[a] - o->ny[b], Z = o->nz[a] - o->nz[b];
      int c;
      if ((c = locate_ph(o, 1, tz, X, Y, Z))) {
        plist_push(&o->P2[1][c - 1], 0, a, b);
        o->hp_ph_phhp[PIDX(o, a, b)] = o->P2[1][c - 1].n;
      }
      if ((c = locate_ph(o, 2, tz, X, Y, Z))) {
        plist_push(&o->P1[2][c - 1], 0, a, b);
        o->hp_ph_hphp[PIDX(o, a, b)] = o->P1[2][c - 1].n;
      }
      if ((c = locate_ph(o, 3, tz, X, Y, Z))) {
        plist_push(&o->P1[3][c - 1], 0, a, b);
        o->hp_ph_hpph[PIDX(o, a, b)] = o->P1[3][c - 1].n;
      }
    }
  for (int a = A; a < ns; a++)
    for (int b = 0; b < A; b++) {
      int tz = (o->tz[a] - o->tz[b]) / 2;
      int X = o->nx[a] - o->nx[b], Y = o->ny[a] - o->ny[b], Z = o->nz[a] - o->nz[b];
      int c;
      if ((c = locate_ph(o, 1, tz, X, Y, Z))) {
        plist_push(&o->P1[1][c - 1], 0, a, b);
        o->ph_ph_phhp[PIDX(o, a, b)] = o->P1[1][c - 1].n;
      }
      if ((c = locate_ph(o, 3, tz, X, Y, Z))) {
        plist_push(&o->P2[3][c - 1], 0, a, b);
        o->ph_ph_hpph[PIDX(o, a, b)] = o->P2[3][c - 1].n;
      }
    }
  free(num1); free(num2);
}

/* ------------------------------------------------------------------ */
/* interaction blocks, ccm_iter.f90:819-1311; Fock and E0, ccm_main.f90:1586-1684 */
static void build_vblocks(ocl_t *o) {
  int n;
  n = o->nch[1];
  o->V_hhhh = (zd **)xcalloc(n, sizeof(zd *));
  for (int ch = 0; ch < n; ch++) {
    plist *L = &o->L1[1][ch];
    zd *V = o->V_hhhh[ch] = (zd *)xcalloc((size_t)L->n * L->n, sizeof(zd));
    for (int bra = 0; bra < L->n; bra++)
      for (int ket = 0; ket < L->n; ket++)
        V[bra + (size_t)L->n * ket] = vA(o, L->p[bra], L->q[bra], L->p[ket], L->q[ket]);
  }
  n = o->nch[2];
  o->V_hhhp = (zd **)xcalloc(n, sizeof(zd *));
  for (int ch = 0; ch < n; ch++) {
    plist *B = &o->L1[2][ch], *K = &o->L2[2][ch];
    zd *V = o->V_hhhp[ch] = (zd *)xcalloc((size_t)B->n * K->n, sizeof(zd));
    for (int bra = 0; bra < B->n; bra++)
      for (int ket = 0; ket < K->n; ket++)
        V[bra + (size_t)B->n * ket] = vA(o, B->p[bra], B->q[bra], K->p[ket], K->q[ket]);
  }
  n = o->nch[3];
  o->V_hhpp = (zd **)xcalloc(n, sizeof(zd *));
  o->V_pppp = (zd **)xcalloc(n, sizeof(zd *));
  for (int ch = 0; ch < n; ch++) {
    plist *B = &o->L1[3][ch], *K = &o->L2[3][ch];
    zd *V = o->V_hhpp[ch] = (zd *)xcalloc((size_t)B->n * K->n, sizeof(zd));
    for (int ket = 0; ket < K->n; ket++)
      for (int bra = 0; bra < B->n; bra++)
        V[bra + (size_t)B->n * ket] = vA(o, B->p[bra], B->q[bra], K->p[ket], K->q[ket]);
  }
  /* pppp: the pppp channel id equals the hhpp id (same enumeration condition),
   * and its pair list equals the hhpp pp list */
  for (int ch = 0; ch < n; ch++) {
    plist *P = &o->L1[6][ch];
    size_t np = P->n;
    zd *V = o->V_pppp[ch] = (zd *)xcalloc(np * np, sizeof(zd));
#pragma omp parallel for schedule(dynamic, 4)
    for (int bra = 0; bra < (int)np; bra++)
      for (size_t ket = 0; ket < np; ket++)
        V[bra + np * ket] = vA(o, P->p[bra], P->q[bra], P->p[ket], P->q[ket]);
  }
  n = o->nch[4];
  o->V_hphp = (zd **)xcalloc(n, sizeof(zd *));
  for (int ch = 0; ch < n; ch++) {
    plist *L = &o->L1[4][ch];
    zd *V = o->V_hphp[ch] = (zd *)xcalloc((size_t)L->n * L->n, sizeof(zd));
    for (int bra = 0; bra < L->n; bra++)
      for (int ket = 0; ket < L->n; ket++)
        V[bra + (size_t)L->n * ket] = vA(o, L->p[bra], L->q[bra], L->p[ket], L->q[ket]);
  }
  /* normal_ordered_hamiltonian, ccm_main.f90:1586-1684 */
  int ns = o->ns, A = o->A;
  o->fock = (zd *)xcalloc((size_t)ns * ns, sizeof(zd));
  for (int i = 0; i < ns; i++) o->fock[i + (size_t)ns * i] = o->e[i];
  for (int ia = 0; ia < ns; ia++)
    for (int ic = 0; ic < ns; ic++) {
      if (o->nx[ia] != o->nx[ic] || o->ny[ia] != o->ny[ic] || o->nz[ia] != o->nz[ic] || o->tz[ia] != o->tz[ic])
        continue;
      zd acc = o->fock[ia + (size_t)ns * ic];
      for (int h = 0; h < A; h++) {
        zd g;
        if (ia >= A && ic >= A) g = vA(o, h, ia, h, ic);
        else if (ia < A && ic < A) g = vA(o, h, ia, h, ic);
        else if (ia >= A && ic < A) g = vA(o, h, ic, h, ia);
        else g = vA(o, h, ia, h, ic);
        acc += g;
      }
      o->fock[ia + (size_t)ns * ic] = acc;
    }
  zd e0 = 0.0;
  for (int i = 0; i < A; i++) e0 += o->e[i];
  for (int i = 0; i < A; i++)
    for (int j = 0; j < A; j++) {
      int tz = (o->tz[i] + o->tz[j]) / 2;
      int c = locate(o, 1, tz, o->nx[i] + o->nx[j], o->ny[i] + o->ny[j], o->nz[i] + o->nz[j]);
      if (!c) continue;
      int b = o->hh_hhhh[PIDX(o, i, j)];
      if (!b) continue;
      plist *L = &o->L1[1][c - 1];
      e0 += 0.5 * o->V_hhhh[c - 1][(b - 1) + (size_t)L->n * (b - 1)];
    }
  o->e0 = e0;
}

static void alloc_amplitudes(ocl_t *o) {
  int n = o->nch[3];
  o->T = (zd **)xcalloc(n, sizeof(zd *));
  o->R = (zd **)xcalloc(n, sizeof(zd *));
  for (int ch = 0; ch < n; ch++) {
    size_t sz = (size_t)o->L1[3][ch].n * o->L2[3][ch].n;
    o->T[ch] = (zd *)xcalloc(sz, sizeof(zd));
    o->R[ch] = (zd *)xcalloc(sz, sizeof(zd));
  }
  n = o->nchph[1];
  o->Tph = (zd **)xcalloc(n, sizeof(zd *));
  o->Rph = (zd **)xcalloc(n, sizeof(zd *));
  for (int ch = 0; ch < n; ch++) {
    size_t sz = (size_t)o->P1[1][ch].n * o->P2[1][ch].n;
    o->Tph[ch] = (zd *)xcalloc(sz, sizeof(zd));
    o->Rph[ch] = (zd *)xcalloc(sz, sizeof(zd));
  }
  o->d2ij = (zd *)xcalloc(o->A, sizeof(zd));
  o->d2ab = (zd *)xcalloc(o->ns - o->A, sizeof(zd));
  o->I6 = (zd *)xcalloc((size_t)o->ns * o->ns, sizeof(zd));
  o->I7 = (zd *)xcalloc((size_t)o->A * o->A, sizeof(zd));
}

ocl_t *ocl_create(const ocl_params *p) {
  ocl_t *o = (ocl_t *)xcalloc(1, sizeof(ocl_t));
  o->prm = *p;
  draw_lecs(o);
  build_basis(o);
  build_channels(o);
  build_ph_channels(o);
  if (p->layout_only) return o;
  build_vblocks(o);
  alloc_amplitudes(o);
  return o;
}

static void free_plists(plist *L, int n) {
  if (!L) return;
  for (int i = 0; i < n; i++) { free(L[i].p); free(L[i].q); }
  free(L);
}
static void free_blocks(zd **B, int n) {
  if (!B) return;
  for (int i = 0; i < n; i++) free(B[i]);
  free(B);
}

void ocl_destroy(ocl_t *o) {
  if (!o) return;
  free(o->nx); free(o->ny); free(o->nz); free(o->sz); free(o->tz);
  free(o->kx); free(o->ky); free(o->kz); free(o->e); free(o->orbitof);
  for (int k = 1; k <= 6; k++) {
    free(o->loc[k]);
    free(o->qn[k]);
    free_plists(o->L1[k], o->nch[k]);
    free_plists(o->L2[k], o->nch[k]);
  }
  free(o->hh_hhhh); free(o->hh_hhhp); free(o->hh_hhpp); free(o->hp_hphp); free(o->hp_hhhp);
  free(o->pp_hhpp); free(o->pp_pppp); free(o->hp_hppp); free(o->pp_hppp);
  for (int k = 1; k <= 3; k++) {
    free(o->locph[k]); free(o->qnph[k]);
    free_plists(o->P1[k], o->nchph[k]);
    free_plists(o->P2[k], o->nchph[k]);
  }
  free(o->ph_ph_phhp); free(o->hp_ph_phhp); free(o->hp_ph_hphp); free(o->hp_ph_hpph); free(o->ph_ph_hpph);
  free_blocks(o->V_hhhh, o->nch[1]);
  free_blocks(o->V_hhhp, o->nch[2]);
  free_blocks(o->V_hhpp, o->nch[3]);
  free_blocks(o->V_pppp, o->nch[3]);
  free_blocks(o->V_hphp, o->nch[4]);
  free_blocks(o->V_hppp, o->nch[5]);
  free(o->fock);
  free_blocks(o->T, o->nch[3]);
  free_blocks(o->R, o->nch[3]);
  free_blocks(o->Tph, o->nchph[1]);
  free_blocks(o->Rph, o->nchph[1]);
  free(o->d2ij); free(o->d2ab); free(o->I6); free(o->I7);
  if (o->t3qn) {
    for (int c = 0; c < o->t3n; c++) { free(o->t3hhh[c]); free(o->t3ppp[c]); }
    free(o->t3hhh); free(o->t3ppp); free(o->t3hhh_n); free(o->t3ppp_n); free(o->t3qn);
  }
  free(o->t2_diis); free(o->t2_diisd);
  free(o);
}

/* ------------------------------------------------------------------ */
/* layout accessors                                                     */
/* ------------------------------------------------------------------ */
int ocl_n_states(const ocl_t *o) { return o->ns; }
double ocl_box_length(const ocl_t *o) { return o->L; }
double ocl_kf(const ocl_t *o) { return o->kf; }
void ocl_get_orbits(const ocl_t *o, int *nx, int *ny, int *nz, int *sz, int *tz, double *kx,
                    double *ky, double *kz, double *e) {
  size_t n = o->ns;
  if (nx) memcpy(nx, o->nx, n * sizeof(int));
  if (ny) memcpy(ny, o->ny, n * sizeof(int));
  if (nz) memcpy(nz, o->nz, n * sizeof(int));
  if (sz) memcpy(sz, o->sz, n * sizeof(int));
  if (tz) memcpy(tz, o->tz, n * sizeof(int));
  if (kx) memcpy(kx, o->kx, n * sizeof(double));
  if (ky) memcpy(ky, o->ky, n * sizeof(double));
  if (kz) memcpy(kz, o->kz, n * sizeof(double));
  if (e) memcpy(e, o->e, n * sizeof(double));
}
int ocl_n_channels(const ocl_t *o, int kind) {
  if (kind < 1 || kind > 6) return 0;
  return o->nch[kind];
}
void ocl_channel_qn(const ocl_t *o, int kind, int ch, int *qn4) {
  memcpy(qn4, o->qn[kind] + 4 * ch, 4 * sizeof(int));
}
int ocl_channel_pairs(const ocl_t *o, int kind, int side, int ch, int *pairs) {
  plist *L = side == 1 ? o->L1[kind] : o->L2[kind];
  if (!L) return 0;
  plist *l = &L[ch];
  if (pairs)
    for (int i = 0; i < l->n; i++) { pairs[2 * i] = l->p[i]; pairs[2 * i + 1] = l->q[i]; }
  return l->n;
}
int ocl_n_ph_channels(const ocl_t *o, int kind) {
  if (kind < 1 || kind > 3) return 0;
  return o->nchph[kind];
}
void ocl_ph_channel_qn(const ocl_t *o, int kind, int ch, int *qn4) {
  memcpy(qn4, o->qnph[kind] + 4 * ch, 4 * sizeof(int));
}
int ocl_ph_channel_pairs(const ocl_t *o, int kind, int side, int ch, int *pairs) {
  plist *L = side == 1 ? o->P1[kind] : o->P2[kind];
  if (!L) return 0;
  plist *l = &L[ch];
  if (pairs)
    for (int i = 0; i < l->n; i++) { pairs[2 * i] = l->p[i]; pairs[2 * i + 1] = l->q[i]; }
  return l->n;
}

static void put_z(double *out, const zd *in, size_t n) {
  for (size_t i = 0; i < n; i++) { out[2 * i] = creal(in[i]); out[2 * i + 1] = cimag(in[i]); }
}
void ocl_e0(const ocl_t *o, double *re_im) { re_im[0] = creal(o->e0); re_im[1] = cimag(o->e0); }
void ocl_get_fock(const ocl_t *o, double *out) { put_z(out, o->fock, (size_t)o->ns * o->ns); }
void ocl_get_vhhpp(const ocl_t *o, int ch, double *out) {
  put_z(out, o->V_hhpp[ch], (size_t)o->L1[3][ch].n * o->L2[3][ch].n);
}
void ocl_get_vpppp(const ocl_t *o, int ch, double *out) {
  put_z(out, o->V_pppp[ch], (size_t)o->L2[3][ch].n * o->L2[3][ch].n);
}
void ocl_get_vhhhh(const ocl_t *o, int ch, double *out) {
  put_z(out, o->V_hhhh[ch], (size_t)o->L1[1][ch].n * o->L1[1][ch].n);
}
void ocl_get_vhphp(const ocl_t *o, int ch, double *out) {
  put_z(out, o->V_hphp[ch], (size_t)o->L1[4][ch].n * o->L1[4][ch].n);
}
void ocl_get_vhhhp(const ocl_t *o, int ch, double *out) {
  put_z(out, o->V_hhhp[ch], (size_t)o->L1[2][ch].n * o->L2[2][ch].n);
}
void ocl_vmat(const ocl_t *o, int p, int q, int r, int s, double *re_im) {
  zd v = vA(o, p, q, r, s);
  re_im[0] = creal(v);
  re_im[1] = cimag(v);
}
void ocl_lecs(const ocl_t *o, double *out9) { memcpy(out9, o->lec, 9 * sizeof(double)); }

int64_t ocl_n_amps(const ocl_t *o) {
  int64_t n = 0;
  for (int ch = 0; ch < o->nch[3]; ch++) n += (int64_t)o->L1[3][ch].n * o->L2[3][ch].n;
  return n;
}
void ocl_get_t2(const ocl_t *o, int ch, double *out) {
  put_z(out, o->T[ch], (size_t)o->L1[3][ch].n * o->L2[3][ch].n);
}
void ocl_get_r2(const ocl_t *o, int ch, double *out) {
  put_z(out, o->R[ch], (size_t)o->L1[3][ch].n * o->L2[3][ch].n);
}
void ocl_set_t2(ocl_t *o, int ch, const double *in) {
  size_t n = (size_t)o->L1[3][ch].n * o->L2[3][ch].n;
  for (size_t i = 0; i < n; i++) o->T[ch][i] = in[2 * i] + I * in[2 * i + 1];
}
void ocl_get_denoms(const ocl_t *o, double *d2ij, double *d2ab) {
  if (d2ij) put_z(d2ij, o->d2ij, o->A);
  if (d2ab) put_z(d2ab, o->d2ab, o->ns - o->A);
}

/* ------------------------------------------------------------------ */
/* MP2 start, setup_t_amplitudes (ccm_iter.f90:2329-2368)               */
/* ------------------------------------------------------------------ */
#define FOCK(o, p, q) ((o)->fock[(size_t)(p) + (size_t)(o)->ns * (q)])
void ocl_mp2(ocl_t *o) {
  for (int ch = 0; ch < o->nch[3]; ch++) {
    plist *H = &o->L1[3][ch], *P = &o->L2[3][ch];
    zd *T = o->T[ch];
    memset(T, 0, sizeof(zd) * (size_t)H->n * P->n);
    for (int bra = 0; bra < H->n; bra++) {
      int i = H->p[bra], j = H->q[bra];
      for (int ket = 0; ket < P->n; ket++) {
        int a = P->p[ket], b = P->q[ket];
        zd denom = -FOCK(o, a, a) - FOCK(o, b, b) + FOCK(o, i, i) + FOCK(o, j, j);
        if (cabs(denom) == 0.0) continue;
        T[ket + (size_t)P->n * bra] = conj(o->V_hhpp[ch][bra + (size_t)H->n * ket]) / denom;
      }
    }
  }
}

/* One column-major product C(m x n) += alpha A(m x k) B(k x n) of a batch (the
 * per-channel ZGEMM calls of the reference).  The jobs of one batch write disjoint C. */
typedef struct {
  int m, n, k, lda, ldb, ldc;
  zd alpha;
  const zd *A, *B;
  zd *C;
} zjob;

/* Tiles of ZT_MB rows x ZT_NB columns.  Every C element takes its k products in
 * ascending l, one complex multiply-add each -- (tr ar - ti ai) + i (tr ai + ti ar)
 * added to C, products with a zero B entry skipped -- so the result is the one of the
 * plain loop over l and depends neither on the tiling nor on the number of threads.  The
 * tile's C is held split into real and imaginary rows, which the compiler vectorises,
 * and each A column segment is read once for ZT_NB columns. */
#define ZT_MB 128
#define ZT_NB 16
static void ztile(const zjob *g, int i0, int j0) {
  const int ni = g->m - i0 < ZT_MB ? g->m - i0 : ZT_MB, nj = g->n - j0 < ZT_NB ? g->n - j0 : ZT_NB;
  double cr[ZT_NB][ZT_MB], ci[ZT_NB][ZT_MB], ar[ZT_MB], ai[ZT_MB];
  for (int jj = 0; jj < nj; jj++) {
    const zd *c = g->C + (size_t)g->ldc * (j0 + jj) + i0;
    for (int i = 0; i < ni; i++) { cr[jj][i] = creal(c[i]); ci[jj][i] = cimag(c[i]); }
  }
  for (int l = 0; l < g->k; l++) {
    const zd *a = g->A + (size_t)g->lda * l + i0;
    for (int i = 0; i < ni; i++) { ar[i] = creal(a[i]); ai[i] = cimag(a[i]); }
    for (int jj = 0; jj < nj; jj++) {
      const zd t = g->alpha * g->B[l + (size_t)g->ldb * (j0 + jj)];
      if (t == 0.0) continue;
      const double tr = creal(t), ti = cimag(t);
      double *xr = cr[jj], *xi = ci[jj];
      for (int i = 0; i < ni; i++) {
        xr[i] += tr * ar[i] - ti * ai[i];
        xi[i] += tr * ai[i] + ti * ar[i];
      }
    }
  }
  for (int jj = 0; jj < nj; jj++) {
    zd *c = g->C + (size_t)g->ldc * (j0 + jj) + i0;
    for (int i = 0; i < ni; i++) c[i] = CMPLX(cr[jj][i], ci[jj][i]);
  }
}

/* the tiles of all jobs of a batch over the threads */
static void zgemm_batch(const zjob *g, int njobs) {
  long *first = (long *)xcalloc((size_t)njobs + 1, sizeof(long));
  for (int j = 0; j < njobs; j++) {
    long nt = 0;
    if (g[j].m > 0 && g[j].n > 0 && g[j].k > 0)
      nt = (long)((g[j].m + ZT_MB - 1) / ZT_MB) * ((g[j].n + ZT_NB - 1) / ZT_NB);
    first[j + 1] = first[j] + nt;
  }
  const long total = first[njobs];
#pragma omp parallel for schedule(dynamic, 1)
  for (long t = 0; t < total; t++) {
    int lo = 0, hi = njobs;  /* the job with first[j] <= t < first[j + 1] */
    while (hi - lo > 1) {
      const int mid = (lo + hi) / 2;
      if (first[mid] <= t) lo = mid;
      else hi = mid;
    }
    const zjob *q = &g[lo];
    const long u = t - first[lo], nbi = (q->m + ZT_MB - 1) / ZT_MB;
    ztile(q, (int)(u % nbi) * ZT_MB, (int)(u / nbi) * ZT_NB);
  }
  free(first);
}

/* ------------------------------------------------------------------ */
/* t2_intermediate(0), ccm_t2_eqn.f90:4-1304, with setup_I6I7_intermediate :1312-1518 */
/* ------------------------------------------------------------------ */
static inline int pair_channel3(const ocl_t *o, int p, int q) {
  int tz = (o->tz[p] + o->tz[q]) / 2;
  return locate(o, 3, tz, o->nx[p] + o->nx[q], o->ny[p] + o->ny[q], o->nz[p] + o->nz[q]);
}

static void gather_tph(ocl_t *o) {
  /* ccm_t2_eqn.f90:37-62; each channel writes its own block */
#pragma omp parallel for schedule(dynamic, 4)
  for (int ch = 0; ch < o->nchph[1]; ch++) {
    plist *B = &o->P1[1][ch], *K = &o->P2[1][ch];
    zd *Tp = o->Tph[ch];
    memset(Tp, 0, sizeof(zd) * (size_t)B->n * K->n);
    for (int bra = 0; bra < B->n; bra++) {
      int a = B->p[bra], i = B->q[bra];
      for (int ket = 0; ket < K->n; ket++) {
        int j = K->p[ket], b = K->q[ket];
        int c2 = pair_channel3(o, i, j);
        if (!c2) continue;
        int bra2 = o->hh_hhpp[PIDX(o, i, j)], ket2 = o->pp_hhpp[PIDX(o, a, b)];
        if (bra2 * ket2 == 0) continue;
        Tp[bra + (size_t)B->n * ket] = o->T[c2 - 1][(ket2 - 1) + (size_t)o->L2[3][c2 - 1].n * (bra2 - 1)];
      }
    }
  }
}

static void setup_i6i7(ocl_t *o) {
  int ns = o->ns, A = o->A;
  memset(o->I6, 0, sizeof(zd) * (size_t)ns * ns);
  memset(o->I7, 0, sizeof(zd) * (size_t)A * A);
  /* I7(k,i) = 1/2 sum V(kl,cd) T(cd,il), ccm_t2_eqn.f90:1352-1392.  Column i of I7 only
   * takes terms of the bras (i,l); each thread sums whole columns, visiting channels,
   * kets, bras and spins in the order of the reference loop, so every entry sees the
   * same additions in the same order. */
#pragma omp parallel for schedule(dynamic, 1)
  for (int i = 0; i < A; i++) {
    int *mine = (int *)xcalloc((size_t)A, sizeof(int));
    for (int ch = 0; ch < o->nch[3]; ch++) {
      plist *H = &o->L1[3][ch], *P = &o->L2[3][ch];
      int nb = 0;
      for (int bra = 0; bra < H->n; bra++)
        if (H->p[bra] == i) mine[nb++] = bra;
      if (!nb) continue;
      const zd *V = o->V_hhpp[ch], *T = o->T[ch];
      for (int ket = 0; ket < P->n; ket++) {
        for (int x = 0; x < nb; x++) {
          int bra = mine[x], l = H->q[bra];
          for (int szc = -1; szc <= 1; szc += 2) {
            int k = orbitof(o, o->nx[i], o->ny[i], o->nz[i], szc, o->tz[i]);
            if (k < 0 || k >= A) continue;
            int bra2 = o->hh_hhpp[PIDX(o, k, l)];
            if (bra2 == 0) continue;
            zd gmat = V[(bra2 - 1) + (size_t)H->n * ket];
            o->I7[k + (size_t)A * i] += 0.5 * gmat * T[ket + (size_t)P->n * bra];
          }
        }
      }
    }
    free(mine);
  }
  /* I6(a,c) = -1/2 sum V(kl,dc) T(da,kl), ccm_t2_eqn.f90:1399-1441.  Row a of I6 only
   * takes terms of the bras (d,a): those are listed per a, in the reference loop's
   * (channel, bra) order, and each thread sums whole rows in that order. */
  const int np_all = ns - A;
  int64_t *off = (int64_t *)xcalloc((size_t)np_all + 1, sizeof(int64_t));
  for (int ch = 0; ch < o->nch[3]; ch++) {
    plist *P = &o->L2[3][ch];
    for (int bra = 0; bra < P->n; bra++) off[P->q[bra] - A + 1]++;
  }
  for (int a = 0; a < np_all; a++) off[a + 1] += off[a];
  int64_t *fill = (int64_t *)xcalloc((size_t)np_all, sizeof(int64_t));
  int *lch = (int *)xcalloc((size_t)off[np_all], sizeof(int)), *lbra = (int *)xcalloc((size_t)off[np_all], sizeof(int));
  for (int ch = 0; ch < o->nch[3]; ch++) {
    plist *P = &o->L2[3][ch];
    for (int bra = 0; bra < P->n; bra++) {
      int64_t x = off[P->q[bra] - A] + fill[P->q[bra] - A]++;
      lch[x] = ch;
      lbra[x] = bra;
    }
  }
  free(fill);
#pragma omp parallel for schedule(dynamic, 4)
  for (int a = A; a < ns; a++) {
    for (int64_t x = off[a - A]; x < off[a - A + 1]; x++) {
      const int ch = lch[x], bra = lbra[x];
      plist *H = &o->L1[3][ch], *P = &o->L2[3][ch];
      const zd *V = o->V_hhpp[ch], *T = o->T[ch];
      int d = P->p[bra];
      for (int ket = 0; ket < H->n; ket++) {
        zd t2 = T[bra + (size_t)P->n * ket];
        for (int szc = -1; szc <= 1; szc += 2) {
          int c = orbitof(o, o->nx[a], o->ny[a], o->nz[a], szc, o->tz[a]);
          if (c < A) continue;
          int bra2 = o->pp_hhpp[PIDX(o, d, c)];
          if (bra2 == 0) continue;
          zd gmat = V[ket + (size_t)H->n * (bra2 - 1)];
          o->I6[a + (size_t)ns * c] += -0.5 * gmat * t2;
        }
      }
    }
  }
  free(off);
  free(lch);
  free(lbra);
  /* add the Fock blocks, ccm_t2_eqn.f90:1507-1510 */
  for (int i = 0; i < A; i++)
    for (int k = 0; k < A; k++) o->I7[k + (size_t)A * i] += FOCK(o, k, i);
  for (int a = A; a < ns; a++)
    for (int c = A; c < ns; c++) o->I6[a + (size_t)ns * c] += FOCK(o, a, c);
}
#define I6(o, a, c) ((o)->I6[(size_t)(a) + (size_t)(o)->ns * (c)])
#define I7(o, k, i) ((o)->I7[(size_t)(k) + (size_t)(o)->A * (i)])

/* The antisymmetrizing scatter R(ab,ij) += Rph(ai,jb) - Rph(bi,ja) - Rph(aj,ib) +
 * Rph(bj,ia), ccm_t2_eqn.f90:840-892.  The reference pushes every Rph element (loop
 * over ph channels, kets (j,b), bras (a,i)) into its four R entries.  Here every R
 * entry pulls its (up to) four Rph elements and adds them in the order that loop visits
 * them, so each entry sees the same additions in the same order, and the hhpp
 * channels run in parallel. */
typedef struct {
  int64_t key;  /* (ph channel, ket, bra): the push loop's visiting order */
  zd v;
  int sign;
} rph_src;

static inline void rph_pull(const ocl_t *o, int p, int h, int h2, int p2, int sign, rph_src *s, int *n) {
  const int cb = locate_ph(o, 1, (o->tz[p] - o->tz[h]) / 2, o->nx[p] - o->nx[h], o->ny[p] - o->ny[h],
                           o->nz[p] - o->nz[h]);
  if (!cb) return;
  const int ck = locate_ph(o, 1, (o->tz[h2] - o->tz[p2]) / 2, o->nx[h2] - o->nx[p2], o->ny[h2] - o->ny[p2],
                           o->nz[h2] - o->nz[p2]);
  if (ck != cb) return;
  const int ib = o->ph_ph_phhp[PIDX(o, p, h)], ik = o->hp_ph_phhp[PIDX(o, h2, p2)];
  if (!ib || !ik) return;
  rph_src *x = &s[(*n)++];
  x->key = ((int64_t)cb << 42) | ((int64_t)(ik - 1) << 21) | (int64_t)(ib - 1);
  x->v = o->Rph[cb - 1][(ib - 1) + (size_t)o->P1[1][cb - 1].n * (ik - 1)];
  x->sign = sign;
}

static void scatter_rph(ocl_t *o) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int c1 = 0; c1 < o->nch[3]; c1++) {
    plist *H = &o->L1[3][c1], *P = &o->L2[3][c1];
    zd *R = o->R[c1];
    const size_t ld = P->n;
    for (int ket = 0; ket < H->n; ket++) {
      const int i = H->p[ket], j = H->q[ket];
      for (int bra = 0; bra < P->n; bra++) {
        const int a = P->p[bra], b = P->q[bra];
        rph_src s[4];
        int n = 0;
        rph_pull(o, a, i, j, b, +1, s, &n);
        rph_pull(o, b, i, j, a, -1, s, &n);
        rph_pull(o, a, j, i, b, -1, s, &n);
        rph_pull(o, b, j, i, a, +1, s, &n);
        for (int x = 1; x < n; x++)
          for (int y = x; y > 0 && s[y - 1].key > s[y].key; y--) {
            rph_src t = s[y];
            s[y] = s[y - 1];
            s[y - 1] = t;
          }
        zd *r = &R[bra + ld * ket];
        for (int x = 0; x < n; x++) {
          if (s[x].sign > 0) *r += s[x].v;
          else *r -= s[x].v;
        }
      }
    }
  }
}

void ocl_t2_intermediate(ocl_t *o) {
  int A = o->A, ns = o->ns;
  for (int ch = 0; ch < o->nch[3]; ch++)
    memset(o->R[ch], 0, sizeof(zd) * (size_t)o->L1[3][ch].n * o->L2[3][ch].n);
  for (int ch = 0; ch < o->nchph[1]; ch++)
    memset(o->Rph[ch], 0, sizeof(zd) * (size_t)o->P1[1][ch].n * o->P2[1][ch].n);
  gather_tph(o);
  setup_i6i7(o);
  /* dressed denominators, :81-89 */
  for (int i = 0; i < A; i++) { o->d2ij[i] = I7(o, i, i); I7(o, i, i) = 0.0; }
  for (int a = A; a < ns; a++) { o->d2ab[a - A] = I6(o, a, a); I6(o, a, a) = 0.0; }
  /* R = conj(V^T), :106-138 */
#pragma omp parallel for schedule(dynamic, 4)
  for (int ch = 0; ch < o->nch[3]; ch++) {
    plist *H = &o->L1[3][ch], *P = &o->L2[3][ch];
    for (int bra = 0; bra < P->n; bra++)
      for (int ket = 0; ket < H->n; ket++)
        o->R[ch][bra + (size_t)P->n * ket] = conj(o->V_hhpp[ch][ket + (size_t)H->n * bra]);
  }
  /* I6 / I7 one-body terms, :144-211; each channel updates its own block, in the order of
   * the serial loop */
#pragma omp parallel for schedule(dynamic, 4)
  for (int ch = 0; ch < o->nch[3]; ch++) {
    plist *H = &o->L1[3][ch], *P = &o->L2[3][ch];
    zd *R = o->R[ch];
    const zd *T = o->T[ch];
    size_t ld = P->n;
    for (int bra = 0; bra < P->n; bra++) {
      int a = P->p[bra], b = P->q[bra];
      for (int ket = 0; ket < H->n; ket++) {
        int i = H->p[ket], j = H->q[ket];
        zd sum1 = 0.0;
        for (int szc = -1; szc <= 1; szc += 2) {
          int c = orbitof(o, o->nx[b], o->ny[b], o->nz[b], szc, o->tz[b]);
          if (c < A) continue;
          int bra2 = o->pp_hhpp[PIDX(o, a, c)];
          if (bra2 == 0) continue;
          sum1 += I6(o, b, c) * T[(bra2 - 1) + ld * ket];
        }
        R[bra + ld * ket] += sum1;
        int bra3 = o->pp_hhpp[PIDX(o, b, a)];
        R[(bra3 - 1) + ld * ket] -= sum1;
        sum1 = 0.0;
        for (int szk = -1; szk <= 1; szk += 2) {
          int k = orbitof(o, o->nx[j], o->ny[j], o->nz[j], szk, o->tz[j]);
          if (k < 0 || k >= A) continue;
          int ket2 = o->hh_hhpp[PIDX(o, i, k)];
          if (ket2 == 0) continue;
          sum1 -= I7(o, k, j) * T[bra + ld * (ket2 - 1)];
        }
        R[bra + ld * ket] += sum1;
        int ket3 = o->hh_hhpp[PIDX(o, j, i)];
        R[bra + ld * (ket3 - 1)] -= sum1;
      }
    }
  }
  /* I9 = V_hhhh + 1/2 V_hhpp T, :423-560 */
  zd **I9 = (zd **)xcalloc(o->nch[1], sizeof(zd *));
  for (int c1 = 0; c1 < o->nch[1]; c1++) {
    int n = o->L1[1][c1].n;
    I9[c1] = (zd *)xcalloc((size_t)n * n, sizeof(zd));
  }
  /* one job per channel; hhpp and hhhh channels pair one to one, so the jobs write
   * disjoint I9 blocks (and below, disjoint R blocks) */
  zjob *jobs = (zjob *)xcalloc((size_t)o->nch[3] + (size_t)o->nchph[2] + 1, sizeof(zjob));
  int nj = 0;
  for (int ch = 0; ch < o->nch[3]; ch++) {
    int *q = o->qn[3] + 4 * ch;
    int c1 = locate(o, 1, q[0], q[1], q[2], q[3]);
    if (!c1) continue;
    int nh = o->L1[3][ch].n, np = o->L2[3][ch].n;
    jobs[nj++] = (zjob){nh, nh, np, nh, np, nh, 0.5, o->V_hhpp[ch], o->T[ch], I9[c1 - 1]};
  }
  zgemm_batch(jobs, nj);
  for (int c1 = 0; c1 < o->nch[1]; c1++) {
    size_t n = (size_t)o->L1[1][c1].n * o->L1[1][c1].n;
    for (size_t x = 0; x < n; x++) I9[c1][x] += o->V_hhhh[c1][x];
  }
  /* pp-ladder R += 1/2 V_pppp T, :568-606 */
  nj = 0;
  for (int ch = 0; ch < o->nch[3]; ch++) {
    int nh = o->L1[3][ch].n, np = o->L2[3][ch].n;
    jobs[nj++] = (zjob){np, nh, np, np, np, np, 0.5, o->V_pppp[ch], o->T[ch], o->R[ch]};
  }
  zgemm_batch(jobs, nj);
  /* hh-ladder R += 1/2 T I9, :613-645 */
  nj = 0;
  for (int ch = 0; ch < o->nch[3]; ch++) {
    int *q = o->qn[3] + 4 * ch;
    int c1 = locate(o, 1, q[0], q[1], q[2], q[3]);
    if (!c1) continue;
    int nh = o->L1[3][ch].n, np = o->L2[3][ch].n;
    jobs[nj++] = (zjob){np, nh, nh, np, nh, np, 0.5, o->T[ch], I9[c1 - 1], o->R[ch]};
  }
  zgemm_batch(jobs, nj);
  for (int c1 = 0; c1 < o->nch[1]; c1++) free(I9[c1]);
  free(I9);
  /* I4_ph = 1/2 amat T_ph - V_hphp, :654-780 */
  int nhp = o->nchph[2];
  zd **I4 = (zd **)xcalloc(nhp, sizeof(zd *));
  for (int ch = 0; ch < nhp; ch++) {
    int n = o->P1[2][ch].n;
    I4[ch] = (zd *)xcalloc((size_t)n * n, sizeof(zd));
  }
  /* the amat blocks, one per channel, then one job per channel writing its own I4 */
  zd **amats = (zd **)xcalloc(nhp, sizeof(zd *));
#pragma omp parallel for schedule(dynamic, 4)
  for (int ch = 0; ch < nhp; ch++) {
    int *q = o->qnph[2] + 4 * ch;
    int c1 = locate_ph(o, 1, q[0], q[1], q[2], q[3]);
    int c3 = locate_ph(o, 3, q[0], q[1], q[2], q[3]);
    if (c1 * c3 == 0) continue;
    plist *B = &o->P1[3][c3 - 1], *K = &o->P2[3][c3 - 1];
    zd *amat = (zd *)xcalloc((size_t)B->n * K->n, sizeof(zd));
    for (int bra = 0; bra < B->n; bra++) {
      int i = B->p[bra], a = B->q[bra];
      for (int ket = 0; ket < K->n; ket++) {
        int b = K->p[ket], j = K->q[ket];
        int c2 = pair_channel3(o, i, j);
        if (!c2) continue;
        int bra2 = o->hh_hhpp[PIDX(o, i, j)], ket2 = o->pp_hhpp[PIDX(o, a, b)];
        if (bra2 * ket2 == 0) continue;
        amat[bra + (size_t)B->n * ket] = o->V_hhpp[c2 - 1][(bra2 - 1) + (size_t)o->L1[3][c2 - 1].n * (ket2 - 1)];
      }
    }
    amats[ch] = amat;
  }
  nj = 0;
  for (int ch = 0; ch < nhp; ch++) {
    if (!amats[ch]) continue;
    int *q = o->qnph[2] + 4 * ch;
    int c1 = locate_ph(o, 1, q[0], q[1], q[2], q[3]);
    int c3 = locate_ph(o, 3, q[0], q[1], q[2], q[3]);
    int n1 = o->P1[3][c3 - 1].n, n3 = o->P2[3][c3 - 1].n, n2 = o->P2[1][c1 - 1].n;
    jobs[nj++] = (zjob){n1, n2, n3, n1, n3, n1, 0.5, amats[ch], o->Tph[c1 - 1], I4[ch]};
  }
  zgemm_batch(jobs, nj);
  for (int ch = 0; ch < nhp; ch++) free(amats[ch]);
  free(amats);
#pragma omp parallel for schedule(dynamic, 4)
  for (int ch = 0; ch < nhp; ch++) {
    plist *L = &o->P1[2][ch];
    for (int ket = 0; ket < L->n; ket++) {
      int j = L->p[ket], b = L->q[ket];
      for (int bra = 0; bra < L->n; bra++) {
        int i = L->p[bra], a = L->q[bra];
        int tz2 = (o->tz[i] + o->tz[b]) / 2;
        int c2 = locate(o, 4, tz2, o->nx[i] + o->nx[b], o->ny[i] + o->ny[b], o->nz[i] + o->nz[b]);
        if (!c2) continue;
        int ket2 = o->hp_hphp[PIDX(o, i, b)], bra2 = o->hp_hphp[PIDX(o, j, a)];
        if (bra2 * ket2 == 0) continue;
        I4[ch][bra + (size_t)L->n * ket] -= o->V_hphp[c2 - 1][(ket2 - 1) + (size_t)o->L1[4][c2 - 1].n * (bra2 - 1)];
      }
    }
  }
  /* ph-ring R_ph += T_ph I4, :800-829; hp and ph channels pair one to one */
  nj = 0;
  for (int ch = 0; ch < nhp; ch++) {
    int *q = o->qnph[2] + 4 * ch;
    int c2 = locate_ph(o, 1, q[0], q[1], q[2], q[3]);
    if (!c2) continue;
    int n1 = o->P1[1][c2 - 1].n, n3 = o->P2[1][c2 - 1].n, n2 = o->P1[2][ch].n;
    jobs[nj++] = (zjob){n1, n2, n3, n1, n3, n1, 1.0, o->Tph[c2 - 1], I4[ch], o->Rph[c2 - 1]};
  }
  zgemm_batch(jobs, nj);
  free(jobs);
  for (int ch = 0; ch < nhp; ch++) free(I4[ch]);
  free(I4);
  scatter_rph(o);
}

/* ccd_energy_save, ccm_energy.f90:4-71 */
void ocl_ccd_energy(const ocl_t *o, double *re_im) {
  zd sum3 = 0.0;
  for (int ch = 0; ch < o->nch[3]; ch++) {
    plist *H = &o->L1[3][ch], *P = &o->L2[3][ch];
    for (int bra = 0; bra < P->n; bra++)
      for (int ket = 0; ket < H->n; ket++)
        sum3 += 0.25 * o->T[ch][bra + (size_t)P->n * ket] * o->V_hhpp[ch][ket + (size_t)H->n * bra];
  }
  re_im[0] = creal(sum3);
  re_im[1] = cimag(sum3);
}

static inline zd denom_of(const ocl_t *o, int a, int b, int i, int j) {
  return (o->d2ij[i] + o->d2ij[j] - o->d2ab[a - o->A]) - o->d2ab[b - o->A];
}

double ocl_residual_norm(const ocl_t *o) {
  /* per-channel sums in parallel, added in channel order: the same value at any thread
   * count */
  double *part = (double *)xcalloc((size_t)o->nch[3] + 1, sizeof(double));
#pragma omp parallel for schedule(dynamic, 4)
  for (int ch = 0; ch < o->nch[3]; ch++) {
    plist *H = &o->L1[3][ch], *P = &o->L2[3][ch];
    double s = 0.0;
    for (int bra = 0; bra < P->n; bra++)
      for (int ket = 0; ket < H->n; ket++) {
        zd d = denom_of(o, P->p[bra], P->q[bra], H->p[ket], H->q[ket]);
        zd r = o->R[ch][bra + (size_t)P->n * ket] - d * o->T[ch][bra + (size_t)P->n * ket];
        s += creal(r) * creal(r) + cimag(r) * cimag(r);
      }
    part[ch] = s;
  }
  double s = 0.0;
  for (int ch = 0; ch < o->nch[3]; ch++) s += part[ch];
  free(part);
  return sqrt(s);
}

/* ------------------------------------------------------------------ */
/* diis_setup / diis_t1t2, ccm_diis.f90:74-293                          */
/* ------------------------------------------------------------------ */
void ocl_diis_setup(ocl_t *o, int subspace, int diis_step) {
  o->subspace = subspace;
  o->diis_step = diis_step;
  o->nstep = 0;
  o->n_diis = ocl_n_amps(o);
  free(o->t2_diis); free(o->t2_diisd);
  o->t2_diis = (zd *)xcalloc((size_t)o->n_diis * (subspace + 1), sizeof(zd));
  o->t2_diisd = (zd *)xcalloc((size_t)o->n_diis * subspace, sizeof(zd));
}

/* LU solve with partial pivoting on max(|re|+|im|) as ZGESV's izamax does */
static int zsolve(int n, zd *Am, zd *b) {
  int *piv = (int *)xcalloc(n, sizeof(int));
  int info = 0;
  for (int k = 0; k < n; k++) {
    int p = k;
    double best = -1.0;
    for (int i = k; i < n; i++) {
      zd v = Am[i + n * k];
      double m = fabs(creal(v)) + fabs(cimag(v));
      if (m > best) { best = m; p = i; }
    }
    piv[k] = p;
    if (best == 0.0) { info = k + 1; continue; }
    if (p != k)
      for (int j = 0; j < n; j++) { zd t = Am[k + n * j]; Am[k + n * j] = Am[p + n * j]; Am[p + n * j] = t; }
    for (int i = k + 1; i < n; i++) {
      Am[i + n * k] /= Am[k + n * k];
      for (int j = k + 1; j < n; j++) Am[i + n * j] -= Am[i + n * k] * Am[k + n * j];
    }
  }
  if (info) { free(piv); return info; }
  for (int k = 0; k < n; k++)
    if (piv[k] != k) { zd t = b[k]; b[k] = b[piv[k]]; b[piv[k]] = t; }
  for (int i = 0; i < n; i++)
    for (int j = 0; j < i; j++) b[i] -= Am[i + n * j] * b[j];
  for (int i = n - 1; i >= 0; i--) {
    for (int j = i + 1; j < n; j++) b[i] -= Am[i + n * j] * b[j];
    b[i] /= Am[i + n * i];
  }
  free(piv);
  return 0;
}

/* The reference increments nstep in ccd_iter right before each call
 * (ccm_iter.f90:86); this entry point does that increment itself. */
void ocl_diis_t1t2(ocl_t *o, int *count) {
  const double a1 = 0.75, b1 = 0.25;
  if (!o->t2_diis) ocl_diis_setup(o, 6, 6);
  o->nstep++;
  size_t nd = (size_t)o->n_diis;
  if (o->nstep > o->subspace) {
    o->nstep = o->subspace;
    for (int i = 0; i < o->subspace - 1; i++)
      memcpy(o->t2_diis + nd * i, o->t2_diis + nd * (i + 1), nd * sizeof(zd));
  }
  size_t i1 = 0;
  int col = o->nstep - 1;
  for (int ch = 0; ch < o->nch[3]; ch++) {
    plist *H = &o->L1[3][ch], *P = &o->L2[3][ch];
    for (int bra = 0; bra < P->n; bra++) {
      int a = P->p[bra], b = P->q[bra];
      for (int ket = 0; ket < H->n; ket++) {
        int i = H->p[ket], j = H->q[ket];
        zd d = denom_of(o, a, b, i, j);
        zd *t = &o->T[ch][bra + (size_t)P->n * ket];
        *t = a1 * (*t) + b1 * o->R[ch][bra + (size_t)P->n * ket] / d;
        o->t2_diis[i1 + nd * col] = *t;
        i1++;
      }
    }
  }
  if (*count == o->diis_step) {
    *count = 0;
    int ns = o->nstep;
    for (int i = 0; i < ns - 1; i++)
      for (size_t k = 0; k < nd; k++)
        o->t2_diisd[k + nd * i] = o->t2_diis[k + nd * (i + 1)] - o->t2_diis[k + nd * i];
    zd *mat = (zd *)xcalloc((size_t)ns * ns, sizeof(zd));
    zd *sol = (zd *)xcalloc(ns, sizeof(zd));
    for (int i = 0; i < ns - 1; i++)
      for (int j = 0; j < ns - 1; j++) {
        zd s = 0.0;
        for (size_t k = 0; k < nd; k++) s += o->t2_diisd[k + nd * i] * o->t2_diisd[k + nd * j];
        mat[i + ns * j] = s;
      }
    for (int i = 0; i < ns - 1; i++) { mat[i + ns * (ns - 1)] = -1.0; mat[(ns - 1) + ns * i] = -1.0; }
    mat[(ns - 1) + ns * (ns - 1)] = 0.0;
    sol[ns - 1] = -1.0;
    zsolve(ns, mat, sol);
    zd *p = o->t2_diisd; /* column 1 reused as the extrapolated vector */
    for (size_t k = 0; k < nd; k++) p[k] = sol[0] * o->t2_diis[k];
    for (int i = 1; i < ns - 1; i++)
      for (size_t k = 0; k < nd; k++) p[k] += sol[i] * o->t2_diis[k + nd * i];
    i1 = 0;
    for (int ch = 0; ch < o->nch[3]; ch++) {
      size_t n = (size_t)o->L1[3][ch].n * o->L2[3][ch].n;
      plist *H = &o->L1[3][ch], *P = &o->L2[3][ch];
      (void)n;
      for (int bra = 0; bra < P->n; bra++)
        for (int ket = 0; ket < H->n; ket++) {
          o->T[ch][bra + (size_t)P->n * ket] = p[i1];
          i1++;
        }
    }
    free(mat);
    free(sol);
  }
}

/* ------------------------------------------------------------------ */
/* ccd_iter, ccm_iter.f90:1-133 (reference mode), plus a standard mode  */
/* ------------------------------------------------------------------ */
static int standard_solve(int n, double *Bm, double *rhs) {
  /* real Gaussian elimination with partial pivoting */
  for (int k = 0; k < n; k++) {
    int p = k;
    for (int i = k + 1; i < n; i++)
      if (fabs(Bm[i + n * k]) > fabs(Bm[p + n * k])) p = i;
    if (Bm[p + n * k] == 0.0) return 1;
    if (p != k) {
      for (int j = 0; j < n; j++) { double t = Bm[k + n * j]; Bm[k + n * j] = Bm[p + n * j]; Bm[p + n * j] = t; }
      double t = rhs[k]; rhs[k] = rhs[p]; rhs[p] = t;
    }
    for (int i = k + 1; i < n; i++) {
      double f = Bm[i + n * k] / Bm[k + n * k];
      for (int j = k; j < n; j++) Bm[i + n * j] -= f * Bm[k + n * j];
      rhs[i] -= f * rhs[k];
    }
  }
  for (int i = n - 1; i >= 0; i--) {
    for (int j = i + 1; j < n; j++) rhs[i] -= Bm[i + n * j] * rhs[j];
    rhs[i] /= Bm[i + n * i];
  }
  return 0;
}

int ocl_ccd_iter(ocl_t *o, const ocl_iter_opts *opt, ocl_iter_result *res) {
  double e[2];
  memset(res, 0, sizeof(*res));
  ocl_ccd_energy(o, e);
  res->e_mbpt2[0] = e[0];
  res->e_mbpt2[1] = e[1];
  if (opt->mode == OCL_MODE_REFERENCE) {
    ocl_diis_setup(o, 6, 6);
    o->nstep = 0;
    int count = 0;
    zd ener1 = e[0] + I * e[1], ener2 = 0.0, dener = 4.0;
    int it;
    for (it = 1; it <= opt->max_iter; it++) {
      if (!(cabs(dener) > opt->tol)) break;
      ocl_t2_intermediate(o);
      res->res_norm = ocl_residual_norm(o);
      count++;
      ocl_diis_t1t2(o, &count);
      ocl_ccd_energy(o, e);
      ener2 = e[0] + I * e[1];
      dener = ener2 - ener1;
      ener1 = ener2;
      res->iterations = it;
      if (opt->verbose) printf("oracle it %3d dE %.3e E %.12f\n", it, creal(dener), creal(ener2));
    }
    res->converged = !(cabs(dener) > opt->tol);
    res->e_ccd[0] = creal(ener2);
    res->e_ccd[1] = cimag(ener2);
    return 0;
  }
  /* standard mode: Jacobi step + Pulay DIIS over (T_jac, step) pairs */
  int m = opt->diis_dim > 0 ? opt->diis_dim : 8;
  size_t nd = (size_t)ocl_n_amps(o);
  zd *hist_t = (zd *)xcalloc(nd * m, sizeof(zd));
  zd *hist_e = (zd *)xcalloc(nd * m, sizeof(zd));
  int nh = 0, head = 0;
  for (int it = 1; it <= opt->max_iter; it++) {
    ocl_t2_intermediate(o);
    double rn = ocl_residual_norm(o);
    res->res_norm = rn;
    res->iterations = it - 1;
    if (opt->verbose) { ocl_ccd_energy(o, e); printf("oracle it %3d |R| %.3e E %.12f\n", it, rn, e[0]); }
    if (rn < opt->tol) { res->converged = 1; break; }
    size_t k = 0;
    zd *ht = hist_t + nd * head, *he = hist_e + nd * head;
    for (int ch = 0; ch < o->nch[3]; ch++) {
      plist *H = &o->L1[3][ch], *P = &o->L2[3][ch];
      for (int ket = 0; ket < H->n; ket++)
        for (int bra = 0; bra < P->n; bra++) {
          zd d = denom_of(o, P->p[bra], P->q[bra], H->p[ket], H->q[ket]);
          zd t = o->T[ch][bra + (size_t)P->n * ket];
          zd tj = o->R[ch][bra + (size_t)P->n * ket] / d;
          ht[k] = tj;
          he[k] = tj - t;
          k++;
        }
    }
    head = (head + 1) % m;
    if (nh < m) nh++;
    int n1 = nh + 1;
    double *Bm = (double *)xcalloc((size_t)n1 * n1, sizeof(double));
    double *rhs = (double *)xcalloc(n1, sizeof(double));
    for (int i = 0; i < nh; i++)
      for (int j = 0; j <= i; j++) {
        double s = 0.0;
        const zd *ei = hist_e + nd * i, *ej = hist_e + nd * j;
        for (size_t x = 0; x < nd; x++) s += creal(conj(ei[x]) * ej[x]);
        Bm[i + n1 * j] = Bm[j + n1 * i] = s;
      }
    for (int i = 0; i < nh; i++) { Bm[i + n1 * nh] = -1.0; Bm[nh + n1 * i] = -1.0; }
    rhs[nh] = -1.0;
    int bad = nh < 2 ? 1 : standard_solve(n1, Bm, rhs);
    k = 0;
    for (int ch = 0; ch < o->nch[3]; ch++) {
      size_t n = (size_t)o->L1[3][ch].n * o->L2[3][ch].n;
      for (size_t x = 0; x < n; x++, k++) {
        zd v;
        if (bad) v = hist_t[nd * ((head + m - 1) % m) + k];
        else {
          v = 0.0;
          for (int i = 0; i < nh; i++) v += rhs[i] * hist_t[nd * i + k];
        }
        o->T[ch][x] = v;
      }
    }
    free(Bm);
    free(rhs);
    res->iterations = it;
  }
  ocl_ccd_energy(o, e);
  res->e_ccd[0] = e[0];
  res->e_ccd[1] = e[1];
  free(hist_t);
  free(hist_e);
  return 0;
}

/* ------------------------------------------------------------------ */
/* (T): setup_vnn_hppp_block (ccm_iter.f90:1361-1810, NN part),         */
/* setup_t3_channel_structures (ccm_t3full_channels.f90:4-284) and      */
/* pert_triples2 with its helpers (ccm_triples.f90:174-294, 528-735)    */
/* ------------------------------------------------------------------ */
static void setup_triples(ocl_t *o) {
  if (o->have_triples_setup) return;
  int ns = o->ns, A = o->A;
  size_t gsz = (size_t)3 * o->Nd[0] * o->Nd[1] * o->Nd[2];
  int *num2 = (int *)xcalloc(gsz, sizeof(int)), *num3 = (int *)xcalloc(gsz, sizeof(int));
  o->loc[5] = (int *)xcalloc(gsz, sizeof(int));
  for (int a = 0; a < ns; a++)
    for (int b = 0; b < ns; b++) {
      int tz = (o->tz[a] + o->tz[b]) / 2;
      size_t g = gidx(o->Nmin, o->Nd, tz, o->nx[a] + o->nx[b], o->ny[a] + o->ny[b], o->nz[a] + o->nz[b]);
      if (a < A && b >= A) num2[g]++;
      if (a >= A && b >= A) num3[g]++;
    }
  o->nch[5] = 0;
  for (int tz = -1; tz <= 1; tz++)
    for (int X = o->Nmin[0]; X <= o->Nmax[0]; X++)
      for (int Y = o->Nmin[1]; Y <= o->Nmax[1]; Y++)
        for (int Z = o->Nmin[2]; Z <= o->Nmax[2]; Z++) {
          size_t g = gidx(o->Nmin, o->Nd, tz, X, Y, Z);
          if (num2[g] * num3[g] != 0) o->loc[5][g] = ++o->nch[5];
        }
  int n5 = o->nch[5];
  int *s1 = (int *)xcalloc(n5 + 1, sizeof(int)), *s2 = (int *)xcalloc(n5 + 1, sizeof(int));
  o->qn[5] = (int *)xcalloc((size_t)4 * (n5 + 1), sizeof(int));
  for (int tz = -1; tz <= 1; tz++)
    for (int X = o->Nmin[0]; X <= o->Nmax[0]; X++)
      for (int Y = o->Nmin[1]; Y <= o->Nmax[1]; Y++)
        for (int Z = o->Nmin[2]; Z <= o->Nmax[2]; Z++) {
          size_t g = gidx(o->Nmin, o->Nd, tz, X, Y, Z);
          int c = o->loc[5][g];
          if (!c) continue;
          s1[c - 1] = num2[g];
          s2[c - 1] = num3[g];
          int *q = o->qn[5] + 4 * (c - 1);
          q[0] = tz; q[1] = X; q[2] = Y; q[3] = Z;
        }
  o->L1[5] = plists_alloc(n5, s1);
  o->L2[5] = plists_alloc(n5, s2);
  free(s1); free(s2); free(num2); free(num3);
  o->hp_hppp = (int *)xcalloc((size_t)ns * ns, sizeof(int));
  o->pp_hppp = (int *)xcalloc((size_t)ns * ns, sizeof(int));
  for (int a = 0; a < A; a++)
    for (int b = A; b < ns; b++) {
      int tz = (o->tz[a] + o->tz[b]) / 2;
      int c = locate(o, 5, tz, o->nx[a] + o->nx[b], o->ny[a] + o->ny[b], o->nz[a] + o->nz[b]);
      if (!c) continue;
      plist_push(&o->L1[5][c - 1], 0, a, b);
      o->hp_hppp[PIDX(o, a, b)] = o->L1[5][c - 1].n;
    }
  for (int a = A; a < ns; a++)
    for (int b = A; b < ns; b++) {
      int tz = (o->tz[a] + o->tz[b]) / 2;
      int c = locate(o, 5, tz, o->nx[a] + o->nx[b], o->ny[a] + o->ny[b], o->nz[a] + o->nz[b]);
      if (!c) continue;
      plist_push(&o->L2[5][c - 1], 0, a, b);
      o->pp_hppp[PIDX(o, a, b)] = o->L2[5][c - 1].n;
    }
  /* vnn_hppp(bra=(k,l) hp, ket=(i,j) pp) = <ij|V|kl>_A, ccm_iter.f90:1680-1760 */
  o->V_hppp = (zd **)xcalloc(n5, sizeof(zd *));
  for (int ch = 0; ch < n5; ch++) {
    plist *B = &o->L1[5][ch], *K = &o->L2[5][ch];
    zd *V = o->V_hppp[ch] = (zd *)xcalloc((size_t)B->n * K->n, sizeof(zd));
#pragma omp parallel for schedule(dynamic, 8)
    for (int ket = 0; ket < K->n; ket++)
      for (int bra = 0; bra < B->n; bra++)
        V[bra + (size_t)B->n * ket] = vA(o, K->p[ket], K->q[ket], B->p[bra], B->q[bra]);
  }
  /* t3 channels */
  int mn[3] = {1000, 1000, 1000}, mx[3] = {-1000, -1000, -1000}, tmn = 100, tmx = -100;
  for (int i = 0; i < ns; i++)
    for (int j = i + 1; j < ns; j++)
      for (int k = j + 1; k < ns; k++) {
        int s[3] = {o->nx[i] + o->nx[j] + o->nx[k], o->ny[i] + o->ny[j] + o->ny[k], o->nz[i] + o->nz[j] + o->nz[k]};
        for (int d = 0; d < 3; d++) {
          if (s[d] > mx[d]) mx[d] = s[d];
          if (s[d] < mn[d]) mn[d] = s[d];
        }
        int st = o->tz[i] + o->tz[j] + o->tz[k];
        if (st > tmx) tmx = st;
        if (st < tmn) tmn = st;
      }
  int dd[3] = {mx[0] - mn[0] + 1, mx[1] - mn[1] + 1, mx[2] - mn[2] + 1};
  int ntz = tmx - tmn + 1;
  size_t g3 = (size_t)ntz * dd[0] * dd[1] * dd[2];
  int64_t *c1 = (int64_t *)xcalloc(g3, sizeof(int64_t)), *c2 = (int64_t *)xcalloc(g3, sizeof(int64_t));
#define G3(t, X, Y, Z) ((((size_t)((t)-tmn) * dd[0] + ((X)-mn[0])) * dd[1] + ((Y)-mn[1])) * dd[2] + ((Z)-mn[2]))
  for (int a = 0; a < ns; a++)
    for (int b = a + 1; b < ns; b++)
      for (int c = b + 1; c < ns; c++) {
        int allh = a < A && b < A && c < A, allp = a >= A && b >= A && c >= A;
        if (!allh && !allp) continue;
        size_t g = G3(o->tz[a] + o->tz[b] + o->tz[c], o->nx[a] + o->nx[b] + o->nx[c],
                      o->ny[a] + o->ny[b] + o->ny[c], o->nz[a] + o->nz[b] + o->nz[c]);
        if (allh) c1[g]++;
        else c2[g]++;
      }
  int *loc3 = (int *)xcalloc(g3, sizeof(int));
  o->t3n = 0;
  for (int t = tmn; t <= tmx; t += 2)
    for (int X = mn[0]; X <= mx[0]; X++)
      for (int Y = mn[1]; Y <= mx[1]; Y++)
        for (int Z = mn[2]; Z <= mx[2]; Z++) {
          size_t g = G3(t, X, Y, Z);
          if (c1[g] * c2[g] != 0) loc3[g] = ++o->t3n;
        }
  o->t3qn = (int *)xcalloc((size_t)4 * (o->t3n + 1), sizeof(int));
  o->t3hhh_n = (int *)xcalloc(o->t3n + 1, sizeof(int));
  o->t3ppp_n = (int *)xcalloc(o->t3n + 1, sizeof(int));
  o->t3hhh = (int **)xcalloc(o->t3n + 1, sizeof(int *));
  o->t3ppp = (int **)xcalloc(o->t3n + 1, sizeof(int *));
  for (int t = tmn; t <= tmx; t += 2)
    for (int X = mn[0]; X <= mx[0]; X++)
      for (int Y = mn[1]; Y <= mx[1]; Y++)
        for (int Z = mn[2]; Z <= mx[2]; Z++) {
          size_t g = G3(t, X, Y, Z);
          int c = loc3[g];
          if (!c) continue;
          int *q = o->t3qn + 4 * (c - 1);
          q[0] = t; q[1] = X; q[2] = Y; q[3] = Z;
          o->t3hhh[c - 1] = (int *)xcalloc((size_t)3 * c1[g], sizeof(int));
          o->t3ppp[c - 1] = (int *)xcalloc((size_t)3 * c2[g], sizeof(int));
        }
  for (int a = A; a < ns; a++)
    for (int b = a + 1; b < ns; b++)
      for (int c = b + 1; c < ns; c++) {
        int ch = loc3[G3(o->tz[a] + o->tz[b] + o->tz[c], o->nx[a] + o->nx[b] + o->nx[c],
                         o->ny[a] + o->ny[b] + o->ny[c], o->nz[a] + o->nz[b] + o->nz[c])];
        if (!ch) continue;
        int n = o->t3ppp_n[ch - 1]++;
        o->t3ppp[ch - 1][3 * n] = a; o->t3ppp[ch - 1][3 * n + 1] = b; o->t3ppp[ch - 1][3 * n + 2] = c;
      }
  for (int a = 0; a < A; a++)
    for (int b = a + 1; b < A; b++)
      for (int c = b + 1; c < A; c++) {
        int ch = loc3[G3(o->tz[a] + o->tz[b] + o->tz[c], o->nx[a] + o->nx[b] + o->nx[c],
                         o->ny[a] + o->ny[b] + o->ny[c], o->nz[a] + o->nz[b] + o->nz[c])];
        if (!ch) continue;
        int n = o->t3hhh_n[ch - 1]++;
        o->t3hhh[ch - 1][3 * n] = a; o->t3hhh[ch - 1][3 * n + 1] = b; o->t3hhh[ch - 1][3 * n + 2] = c;
      }
#undef G3
  free(c1); free(c2); free(loc3);
  o->have_triples_setup = 1;
}

/* three_body_oneparticle_1, ccm_triples.f90:174-232: sum_d conj(<cb|V|kd>) T(ad,ij) */
static zd tb_oneparticle(const ocl_t *o, int a, int b, int c, int i, int j, int k) {
  zd sum1 = 0.0;
  int A = o->A;
  int nxd = o->nx[i] + o->nx[j] - o->nx[a], nyd = o->ny[i] + o->ny[j] - o->ny[a];
  int nzd = o->nz[i] + o->nz[j] - o->nz[a], tzd = o->tz[i] + o->tz[j] - o->tz[a];
  if (abs(nxd) > o->nk[0] || abs(nyd) > o->nk[1] || abs(nzd) > o->nk[2] || abs(tzd) > 1) return 0.0;
  for (int szd = -1; szd <= 1; szd += 2) {
    int d = orbitof(o, nxd, nyd, nzd, szd, tzd);
    if (d < A) continue;
    int ch2 = pair_channel3(o, i, j);
    if (!ch2) continue;
    int ket2 = o->hh_hhpp[PIDX(o, i, j)], bra2 = o->pp_hhpp[PIDX(o, a, d)];
    if (bra2 * ket2 == 0) continue;
    int tz3 = (o->tz[b] + o->tz[c]) / 2;
    int ch5 = locate(o, 5, tz3, o->nx[b] + o->nx[c], o->ny[b] + o->ny[c], o->nz[b] + o->nz[c]);
    if (!ch5) continue;
    int bra3 = o->hp_hppp[PIDX(o, k, d)], ket3 = o->pp_hppp[PIDX(o, c, b)];
    if (bra3 * ket3 == 0) continue;
    zd v = o->V_hppp[ch5 - 1][(bra3 - 1) + (size_t)o->L1[5][ch5 - 1].n * (ket3 - 1)];
    zd t = o->T[ch2 - 1][(bra2 - 1) + (size_t)o->L2[3][ch2 - 1].n * (ket2 - 1)];
    sum1 += conj(v) * t;
  }
  return sum1;
}

/* three_body_onehole_1, ccm_triples.f90:238-294: sum_l conj(<jk|V|lc>) T(ab,il) */
static zd tb_onehole(const ocl_t *o, int a, int b, int c, int i, int j, int k) {
  zd sum1 = 0.0;
  int A = o->A;
  int nxl = o->nx[k] + o->nx[j] - o->nx[c], nyl = o->ny[k] + o->ny[j] - o->ny[c];
  int nzl = o->nz[k] + o->nz[j] - o->nz[c], tzl = o->tz[k] + o->tz[j] - o->tz[c];
  if (abs(nxl) > o->nk[0] || abs(nyl) > o->nk[1] || abs(nzl) > o->nk[2] || abs(tzl) > 1) return 0.0;
  for (int szl = -1; szl <= 1; szl += 2) {
    int l = orbitof(o, nxl, nyl, nzl, szl, tzl);
    if (l < 0 || l >= A) continue;
    int ch2 = pair_channel3(o, i, l);
    if (!ch2) continue;
    int ket2 = o->hh_hhpp[PIDX(o, i, l)], bra2 = o->pp_hhpp[PIDX(o, a, b)];
    if (bra2 * ket2 == 0) continue;
    int tz3 = (o->tz[l] + o->tz[c]) / 2;
    int ch5 = locate(o, 2, tz3, o->nx[l] + o->nx[c], o->ny[l] + o->ny[c], o->nz[l] + o->nz[c]);
    if (!ch5) continue;
    int bra3 = o->hh_hhhp[PIDX(o, j, k)], ket3 = o->hp_hhhp[PIDX(o, l, c)];
    if (bra3 * ket3 == 0) continue;
    zd v = o->V_hhhp[ch5 - 1][(bra3 - 1) + (size_t)o->L1[2][ch5 - 1].n * (ket3 - 1)];
    zd t = o->T[ch2 - 1][(bra2 - 1) + (size_t)o->L2[3][ch2 - 1].n * (ket2 - 1)];
    sum1 += conj(v) * t;
  }
  return sum1;
}

int ocl_triples_channels(ocl_t *o) {
  setup_triples(o);
  return o->t3n;
}

int64_t ocl_triples_count(ocl_t *o) {
  setup_triples(o);
  int64_t n = 0;
  for (int c = 0; c < o->t3n; c++) n += (int64_t)o->t3hhh_n[c] * o->t3ppp_n[c];
  return n;
}

/* E(T) summed over the (abc) triples k0, k0 + stride, ... of every triple channel (all
 * of them: 0, 1) */
static zd triples_channels(ocl_t *o, int k0, int stride, int64_t *pairs) {
  setup_triples(o);
  zd et = 0.0;
  int64_t np = 0;
  for (int ch = 0; ch < o->t3n; ch++) {
    int nk = o->t3ppp_n[ch], nb = o->t3hhh_n[ch];
    if (nk > k0) np += (int64_t)((nk - k0 + stride - 1) / stride) * nb;
    zd *part = (zd *)xcalloc(nk > 0 ? nk : 1, sizeof(zd));
#pragma omp parallel for schedule(dynamic, 4)
    for (int ket = k0; ket < nk; ket += stride) {
      const int *abc = o->t3ppp[ch] + 3 * ket;
      int a = abc[0], b = abc[1], c = abc[2];
      zd acc = 0.0;
      for (int bra = 0; bra < nb; bra++) {
        const int *ijk = o->t3hhh[ch] + 3 * bra;
        int i = ijk[0], j = ijk[1], k = ijk[2];
        zd spen = FOCK(o, i, i) + FOCK(o, j, j) + FOCK(o, k, k) - FOCK(o, a, a) - FOCK(o, b, b) - FOCK(o, c, c);
        zd s1 = tb_oneparticle(o, a, b, c, i, j, k);
        zd s2 = tb_oneparticle(o, b, a, c, i, j, k);
        zd s3 = tb_oneparticle(o, c, b, a, i, j, k);
        zd s4 = tb_oneparticle(o, a, b, c, k, j, i);
        zd s5 = tb_oneparticle(o, a, b, c, i, k, j);
        zd s6 = tb_oneparticle(o, c, b, a, i, k, j);
        zd s7 = tb_oneparticle(o, c, b, a, k, j, i);
        zd s8 = tb_oneparticle(o, b, a, c, i, k, j);
        zd s9 = tb_oneparticle(o, b, a, c, k, j, i);
        zd tc = (s1 - s2 - s3 - s4 - s5 + s6 + s7 + s8 + s9);
        s1 = tb_onehole(o, a, b, c, i, j, k);
        s2 = tb_onehole(o, a, c, b, i, j, k);
        s3 = tb_onehole(o, c, b, a, i, j, k);
        s4 = tb_onehole(o, a, b, c, k, j, i);
        s5 = tb_onehole(o, a, b, c, j, i, k);
        s6 = tb_onehole(o, c, b, a, j, i, k);
        s7 = tb_onehole(o, c, b, a, k, j, i);
        s8 = tb_onehole(o, a, c, b, j, i, k);
        s9 = tb_onehole(o, a, c, b, k, j, i);
        tc = tc - (s1 - s2 - s3 - s4 - s5 + s6 + s7 + s8 + s9);
        acc += conj(tc) * tc / spen;
      }
      part[ket] = acc;
    }
    for (int ket = 0; ket < nk; ket++) et += part[ket];
    free(part);
  }
  if (pairs) *pairs = np;
  return et;
}

void ocl_pert_triples(ocl_t *o, double *re_im) {
  zd et = triples_channels(o, 0, 1, NULL);
  re_im[0] = creal(et);
  re_im[1] = cimag(et);
}

void ocl_pert_triples_sample(ocl_t *o, int k0, int stride, double *re_im, int64_t *pairs) {
  zd et = triples_channels(o, k0 < 0 ? 0 : k0, stride < 1 ? 1 : stride, pairs);
  re_im[0] = creal(et);
  re_im[1] = cimag(et);
}
