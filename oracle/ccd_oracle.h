/*
 * CPU oracle for the CCD + (T) hot path of paolofinelli/Coupled-Cluster-NuclearMatter.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C, complex<double> restatement of the
 * reference Fortran solver (the .f90 files of deltafull-CCMkspace), loop by loop, used as the
 * checker for the GPU engine.  Only the tests, the smoke check and the CPU-baseline
 * leg of the benchmark may load it.  The product never links or calls it.
 *
 * Parity status: UNPINNED.  The reference ships no golden vectors, tests or
 * fixtures, and it cannot be compiled here (Fortran + MPI + LAPACK are absent), so
 * the restatement is validated by independent checks instead: a dense-tensor
 * textbook CCD (numpy) on small lattices, MP2 closed form, antisymmetry, and
 * thread-count invariance.
 *
 * Conventions: orbitals are 0-based; pair lists hold 0-based orbital indices;
 * per-channel blocks are column-major like the Fortran arrays they restate,
 * e.g. T2 of hhpp channel ch is (n_pp x n_hh), element (ab, ij) at [ab + n_pp*ij].
 */
#ifndef CCD_ORACLE_H
#define CCD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* potential kinds */
#define OCL_POT_MINNESOTA 0   /* vmom_minnesota, chiral_module_andreas_with_delta.f90:8980-9111 */
#define OCL_POT_CHIRAL_LIKE 1 /* OPE + LO/NLO contacts, chiral_pot structure, :5879-6301 */

/* iteration modes */
#define OCL_MODE_REFERENCE 0  /* ccd_iter + diis_t1t2 exactly (ccm_iter.f90:67-96, ccm_diis.f90:74-249) */
#define OCL_MODE_STANDARD  1  /* Jacobi step + Pulay DIIS on the step vectors, residual-norm stop */

typedef struct {
  int nmax;            /* lattice |n_i| <= nmax */
  int A;               /* particle number (holes = first A sorted states) */
  int snm;             /* 0: pure neutron matter, 1: symmetric nuclear matter */
  double rho;          /* density fm^-3 (input_type 'density') */
  double theta[3];     /* twist angles per axis */
  int potential;       /* OCL_POT_* */
  uint64_t lec_seed;   /* seed of the chiral-like contact LEC draw */
  int minnesota_f32_literals; /* 1: reproduce the reference's default-real literals */
  int layout_only;     /* 1: basis and channel tables only (no V blocks, no amplitudes) */
} ocl_params;

typedef struct ocl ocl_t;

ocl_t *ocl_create(const ocl_params *p);
void ocl_destroy(ocl_t *o);
int ocl_num_threads(void);

/* ---- layout ---------------------------------------------------------- */
int ocl_n_states(const ocl_t *o);
/* per-state arrays of length n_states; any pointer may be NULL */
void ocl_get_orbits(const ocl_t *o, int *nx, int *ny, int *nz, int *sz, int *tz,
                    double *kx, double *ky, double *kz, double *e);
double ocl_box_length(const ocl_t *o);
double ocl_kf(const ocl_t *o);
/* kind: 1 hhhh, 2 hhhp, 3 hhpp, 4 hphp, 5 hppp (after triples setup), 6 pppp */
int ocl_n_channels(const ocl_t *o, int kind);
/* quantum numbers of channel ch (0-based) of a kind: tz, Nx, Ny, Nz */
void ocl_channel_qn(const ocl_t *o, int kind, int ch, int *qn4);
/* number of pairs of side (1 or 2) of channel ch; pairs written as p0,q0,p1,q1,... */
int ocl_channel_pairs(const ocl_t *o, int kind, int side, int ch, int *pairs);
/* particle-hole channels: kind 1 phhp, 2 hphp, 3 hpph */
int ocl_n_ph_channels(const ocl_t *o, int kind);
void ocl_ph_channel_qn(const ocl_t *o, int kind, int ch, int *qn4);
int ocl_ph_channel_pairs(const ocl_t *o, int kind, int side, int ch, int *pairs);

/* ---- hamiltonian ----------------------------------------------------- */
void ocl_e0(const ocl_t *o, double *re_im);
/* full Fock matrix (n_states x n_states col-major, interleaved re/im) */
void ocl_get_fock(const ocl_t *o, double *out);
/* V block of hhpp channel ch, (n_hh x n_pp) col-major interleaved complex */
void ocl_get_vhhpp(const ocl_t *o, int ch, double *out);
void ocl_get_vpppp(const ocl_t *o, int ch, double *out);
void ocl_get_vhhhh(const ocl_t *o, int ch, double *out);
void ocl_get_vhphp(const ocl_t *o, int ch, double *out);
void ocl_get_vhhhp(const ocl_t *o, int ch, double *out);
/* the synthetic two-body matrix element (antisymmetrized) <pq|V|rs>_A */
void ocl_vmat(const ocl_t *o, int p, int q, int r, int s, double *re_im);
/* contact LECs of the chiral-like kind: CS, CT, C1..C7 in MeV units */
void ocl_lecs(const ocl_t *o, double *out9);

/* ---- amplitudes ------------------------------------------------------ */
int64_t ocl_n_amps(const ocl_t *o);
void ocl_mp2(ocl_t *o);                          /* setup_t_amplitudes */
void ocl_get_t2(const ocl_t *o, int ch, double *out);
void ocl_set_t2(ocl_t *o, int ch, const double *in);
void ocl_get_r2(const ocl_t *o, int ch, double *out);   /* t2_ccm_eqn after residual */
void ocl_get_denoms(const ocl_t *o, double *d2ij, double *d2ab); /* complex interleaved, len A / ns-A */

/* ---- hot path -------------------------------------------------------- */
void ocl_t2_intermediate(ocl_t *o);              /* t2_intermediate(0) */
void ocl_diis_t1t2(ocl_t *o, int *count);        /* nstep += 1, then diis_t1t2(count) */
void ocl_diis_setup(ocl_t *o, int subspace, int diis_step);
void ocl_ccd_energy(const ocl_t *o, double *re_im);  /* ccd_energy_save */
double ocl_residual_norm(const ocl_t *o);        /* ||R - D T|| over ordered amplitudes */

typedef struct {
  int mode;        /* OCL_MODE_* */
  int max_iter;
  double tol;      /* |dE| (reference mode) or ||R-DT|| (standard mode) */
  int diis_dim;    /* standard mode history length */
  int verbose;
} ocl_iter_opts;

typedef struct {
  int iterations;
  double e_mbpt2[2];   /* correlation energy at MP2 amplitudes */
  double e_ccd[2];     /* correlation energy at the end */
  double res_norm;
  int converged;
} ocl_iter_result;

int ocl_ccd_iter(ocl_t *o, const ocl_iter_opts *opt, ocl_iter_result *res);

/* ---- (T) ------------------------------------------------------------- */
void ocl_pert_triples(ocl_t *o, double *re_im);  /* pert_triples2, NN only */
int64_t ocl_triples_count(ocl_t *o);             /* number of (abc, ijk) pairs */
int ocl_triples_channels(ocl_t *o);              /* number of triple channels */
/* the (T) sum over the (abc) triples k0, k0 + stride, ... of every triple channel only,
 * and the number of (abc, ijk) pairs it covers: a bounded timing sample of pert_triples2 */
void ocl_pert_triples_sample(ocl_t *o, int k0, int stride, double *re_im, int64_t *pairs);

#ifdef __cplusplus
}
#endif
#endif
