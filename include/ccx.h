/*
 * ccx.h -- C ABI of the GB300 CCD + (T) engine.
 *
 * Drop-in boundary for the CCD solver of paolofinelli/Coupled-Cluster-NuclearMatter
 * (directory deltafull-CCMkspace).  The reference has no plugin API: its solver is
 * the set of Fortran subroutines that ccd_iter (ccm_iter.f90:1-170) calls, and they
 * talk through module globals.  Each entry point below names the subroutine or
 * global it replaces.  A Fortran caller binds them with ISO_C_BINDING; complex*16
 * arrays are passed as interleaved (re, im) double pairs, which is the memory
 * layout of complex(c_double_complex).
 *
 * Conventions
 *  - Every function returns 0 on success and a nonzero CCX_E* code on failure; the
 *    message of the last failure on the calling thread is ccx_last_error().  No
 *    entry point exits or stops the process.
 *  - Orbitals are 0-based in pair lists (the Fortran shim adds 1).  Channels are
 *    0-based and numbered in the reference's enumeration order.
 *  - Per-channel blocks use the reference's column-major layout, e.g. the T2 block
 *    of hhpp channel ch is t2_ccm(ch)%val(n_pp, n_hh) with ab fastest.
 *  - One engine drives one GPU through one CUDA stream; calls on one engine are
 *    not thread safe.
 */
#ifndef CCX_H
#define CCX_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CCX_OK 0
#define CCX_EINVAL 1      /* bad argument or malformed input */
#define CCX_ECUDA 2       /* CUDA runtime failure (message holds the CUDA error) */
#define CCX_ENOMEM 3      /* device or host allocation failed / plan too large */
#define CCX_ESTATE 4      /* call out of order (e.g. iterate before amplitudes) */
#define CCX_ENUMERIC 5    /* NaN/Inf detected, or singular DIIS system */
#define CCX_ENOGPU 6      /* no CUDA device available */

typedef struct ccx_layout ccx_layout;
typedef struct ccx_engine ccx_engine;

/* ------------------------------------------------------------------ */
/* Input deck                                                           */
/* ------------------------------------------------------------------ */

/* The nine value lines of ccm_in, read by ccm_main.f90:31-32 and allocate_sp_data
 * (ccm_main.f90:893-900), plus an optional extension block that the reference
 * parser never reads (lines after the ninth value line of the form "key = value"). */
typedef struct {
  int32_t chiral_order;      /* line 1 */
  double lambda;             /* line 1 */
  double cE, cD;             /* line 2 */
  int32_t A;                 /* line 3: number of particles (below_ef) */
  int32_t snm;               /* line 4: 0 pnm, 1 snm */
  int32_t input_is_kfermi;   /* line 4: 0 density, 1 kfermi */
  char bc[16];               /* line 5: PBC / TABC / TABCsp */
  double dens_or_kf;         /* line 6 */
  int32_t ntwist, nmax, my_twists; /* line 6 */
  char cc_approx[16];        /* line 7: CCD / CCD(T) / CCDT1 / mbpt2 */
  int32_t tnf_switch, tnf_approx;  /* line 8 */
  double cutoff_3nf;         /* line 9 */
  int32_t nexp_3nf;          /* line 9 */
  /* extension block (defaults reproduce the reference) */
  int32_t potential;         /* CCX_POT_*; default CCX_POT_MINNESOTA */
  uint64_t lec_seed;         /* default 20261203 */
  int32_t mode;              /* CCX_MODE_*; default CCX_MODE_REFERENCE */
  int32_t diis_dim;          /* standard mode history; default 8 */
  double tol;                /* default 1e-6 (|dE|, reference mode) */
  int32_t max_iter;          /* default 100 */
  int32_t precision;         /* CCX_PREC_*; default CCX_PREC_FP64 */
  double theta[3];           /* twist per axis for PBC runs; default 0 */
} ccx_deck;

/* Parse ccm_in text.  Replaces the read(5,*) sequence of ccm_main.f90:31-32 and
 * allocate_sp_data (ccm_main.f90:893-900). */
int ccx_deck_parse(const char *text, ccx_deck *out);

/* ------------------------------------------------------------------ */
/* Basis and channel layout (host only, no GPU needed)                  */
/* ------------------------------------------------------------------ */

/* Momentum-lattice single-particle basis in the reference's order.  Replaces
 * setup_sp_data (ccm_main.f90:1003-1197): k-mesh order, |k|^2 index sort
 * (ccm_main.f90:2654-2732), spin/isospin inner order, holes = first A states. */
typedef struct {
  int32_t nmax;
  int32_t A;
  int32_t snm;
  double density;            /* fm^-3 */
  double theta[3];           /* twist angles */
} ccx_basis_params;

typedef struct {
  int32_t n_states;          /* all_orbit%total_orbits */
  int32_t n_holes;           /* below_ef */
  const int32_t *nx, *ny, *nz, *sz, *tz;  /* all_orbit%nx ... %itzp */
  const double *kx, *ky, *kz;             /* all_orbit%kx ... (fm^-1) */
  const double *e;           /* all_orbit%e, kinetic energy (MeV) */
  double box_length;         /* lx (fm); volume = lx^3 */
} ccx_orbits;

/* Build the basis; the arrays of *orbits stay owned by the layout. */
int ccx_layout_from_basis(const ccx_basis_params *p, ccx_layout **out);
/* Wrap a caller's basis (e.g. the Fortran all_orbit arrays); arrays are copied.
 * Channel tables are then enumerated exactly as setup_channel_structures
 * (ccm_iter.f90:175-812) and setup_ph_channel_structures (ccm_iter.f90:1816-2105)
 * enumerate them. */
int ccx_layout_from_orbits(const ccx_orbits *orbits, ccx_layout **out);
int ccx_layout_destroy(ccx_layout *l);
int ccx_layout_orbits(const ccx_layout *l, ccx_orbits *out);

/* counts[0..7]: #hhpp (= #pppp), #hhhh, #hhhp, #hphp, #phhp ph channels, #hphp ph
 * channels, #hpph ph channels, #T2 amplitudes (ordered, as t2_ccm stores them) */
int ccx_layout_counts(const ccx_layout *l, int64_t counts[8]);

/* Channel tables.  kind: CCX_CH_* below.  qn = (tz, Nx, Ny, Nz) as in
 * channels%hhpp_quantum_numbers(4*ch-3 .. 4*ch); side 1 is the bra list
 * (lookup_*_configs(1,ch)), side 2 the ket list (lookup_*_configs(2,ch)). */
#define CCX_CH_HHHH 1
#define CCX_CH_HHHP 2
#define CCX_CH_HHPP 3
#define CCX_CH_HPHP 4
#define CCX_CH_HPPP 5   /* setup_vnn_hppp_block channels (ccm_iter.f90:1407-1534), used by (T) */
#define CCX_CH_PH_PHHP 11
#define CCX_CH_PH_HPHP 12
#define CCX_CH_PH_HPPH 13
int ccx_layout_channel(const ccx_layout *l, int32_t kind, int32_t ch, int32_t qn[4],
                       int32_t *n_side1, int32_t *n_side2);
/* pairs written as (p0, q0, p1, q1, ...), 0-based orbitals; NULL to skip a side */
int ccx_layout_pairs(const ccx_layout *l, int32_t kind, int32_t ch, int32_t *side1,
                     int32_t *side2);
/* 64-bit FNV-1a hash over the orbit table and every channel table */
int ccx_layout_hash(const ccx_layout *l, uint64_t *hash);

/* ------------------------------------------------------------------ */
/* Engine                                                               */
/* ------------------------------------------------------------------ */
#define CCX_SCALAR_COMPLEX 0   /* complex*16 arithmetic, as the reference */
#define CCX_SCALAR_REAL 1      /* real arithmetic; V and Fock must be real */

#define CCX_PREC_FP64 0        /* every term in FP64 */
#define CCX_PREC_MIXED 1       /* ladder/ring contractions as BF16 hi/lo split products on the tensor
                                  cores (FP32 accumulate), FP64 defect correction; standard mode; a complex
                                  engine runs each complex product as four real ones */
#define CCX_PREC_MIXED_TF32 2  /* as CCX_PREC_MIXED with TF32 hi/lo split products */

#define CCX_MODE_REFERENCE 0   /* 0.75/0.25 mixing + DIIS every 6 (ccm_diis.f90:74-249), |dE| stop */
#define CCX_MODE_STANDARD 1    /* Jacobi step + Pulay DIIS on steps, ||R - D T|| stop */

typedef struct {
  int32_t device;            /* CUDA device ordinal */
  int32_t scalar;            /* CCX_SCALAR_* */
} ccx_engine_options;

/* Allocate the device image of the layout (T2, R, intermediates, maps). */
int ccx_engine_create(const ccx_layout *l, const ccx_engine_options *opt, ccx_engine **out);
int ccx_engine_destroy(ccx_engine *e);
/* device bytes held by the engine */
int ccx_engine_memory(const ccx_engine *e, int64_t *bytes);

/* ---- interaction input ---------------------------------------------- */
/* Full Fock matrix (n_states x n_states, column-major, complex interleaved);
 * replaces one_body_operators%fock_mtx built by normal_ordered_hamiltonian
 * (ccm_main.f90:1523-1684).  e0 is the reference energy E0. */
int ccx_set_fock(ccx_engine *e, const double *fock, const double e0[2]);

/* One antisymmetrised V block, exactly the array the reference holds:
 *   CCX_CH_HHPP  vnn_hhpp(ch)%val(n_hh, n_pp)      ccm_iter.f90:935-1030
 *   CCX_V_PPPP   vnn_pppp(ch)%val(n_pp, n_pp)      ccm_iter.f90:1203-1305
 *   CCX_CH_HHHH  vnn_hhhh(ch)%val(n_hh, n_hh)      ccm_iter.f90:835-878
 *   CCX_CH_HPHP  vnn_hphp(ch)%val(n_hp, n_hp)      ccm_iter.f90:1070-1150
 *   CCX_CH_HHHP  vnn_hhhp(ch)%val(n_hh, n_hp)      ccm_iter.f90:885-930 (used by (T))
 *   CCX_CH_HPPP  vnn_hppp(ch)%val(n_hp, n_pp)      ccm_iter.f90:1680-1760 (used by (T))
 * col-major, complex interleaved, leading dimension = rows.  The host buffer is
 * only read during the call. */
#define CCX_V_PPPP 6
int ccx_set_vblock(ccx_engine *e, int32_t kind, int32_t ch, const double *v);
/* The same for n blocks of one kind (channels chs[i], buffers v[i]) in one call: the
 * copies are queued back to back and the call returns once all have been read, so a
 * host that hands over every channel of a family pays one synchronisation.  Same
 * reference arrays as ccx_set_vblock.  When every buffer is pinned host memory the
 * device can address (cudaHostAlloc / cudaHostRegister), the packing kernels read the
 * blocks in place, touching only the cache lines of the unique pairs, with no staging
 * copies; ccx_set_vblock does the same for one block. */
int ccx_set_vblocks(ccx_engine *e, int32_t kind, int32_t n, const int32_t *chs, const double *const *v);

/* Generate Fock, E0 and every V block on the device from a synthetic potential
 * (replaces the potential loops of setup_channel_structures, ccm_iter.f90:819-1311,
 * and normal_ordered_hamiltonian, ccm_main.f90:1586-1684). */
#define CCX_POT_MINNESOTA 0    /* vmom_minnesota, chiral_module_andreas_with_delta.f90:8980-9111 */
#define CCX_POT_CHIRAL_LIKE 1  /* OPE + LO/NLO contacts in the operator form of chiral_pot */
typedef struct {
  int32_t kind;              /* CCX_POT_* */
  uint64_t lec_seed;         /* chiral-like contact LEC draw */
  int32_t f32_literals;      /* 1: Minnesota constants rounded to 4-byte reals like the reference */
} ccx_potential;
/* Blocks set with ccx_set_vblock(s) after this call replace the generated ones of their
 * channels; the other channels of every family keep the generated interaction. */
int ccx_generate_interaction(ccx_engine *e, const ccx_potential *pot);
/* E0 = sum_i t_ii + 1/2 sum_ij <ij|V|ij> (ccm_main.f90:1661-1684) of the interaction
 * generated on the device, or the value passed to ccx_set_fock */
int ccx_get_e0(ccx_engine *e, double e0[2]);

/* Export of the interaction in the reference's ordered layout (the inverse of
 * ccx_set_vblock / ccx_set_fock).  For a generated interaction every kind is
 * available (blocks are re-evaluated on the device); for a caller-supplied one, the
 * kinds the engine stores (HHPP, PPPP, HHHH of channels with pp pairs).  The Fock
 * export holds the momentum-diagonal entries the CCD path uses (f(p,p) and the
 * same-momentum spin partners), zeros elsewhere. */
int ccx_get_vblock(ccx_engine *e, int32_t kind, int32_t ch, double *v);
int ccx_get_fock(ccx_engine *e, double *fock);

/* ---- amplitudes ----------------------------------------------------- */
/* MP2 start: setup_t_amplitudes (ccm_iter.f90:2329-2368) */
int ccx_setup_t_amplitudes(ccx_engine *e);
/* t2_ccm(ch)%val in / out, (n_pp x n_hh) col-major complex interleaved */
int ccx_set_t2(ccx_engine *e, int32_t ch, const double *t);
int ccx_get_t2(ccx_engine *e, int32_t ch, double *t);
/* t2_ccm_eqn(ch)%val after ccx_t2_intermediate */
int ccx_get_t2_eqn(ccx_engine *e, int32_t ch, double *r);
/* all channels concatenated in channel order (n_amps complex values); ccx_get_t2_all
 * unpacks straight into pinned device-addressable host memory, one synchronisation */
int ccx_set_t2_all(ccx_engine *e, const double *t);
int ccx_get_t2_all(ccx_engine *e, double *t);
/* T2 checkpoint files (host only, no engine or GPU needed): the ccx_get_t2_all buffer
 * (2 * n_amps doubles) behind a header with the layout hash, a hash of the orbital
 * momenta and box length (the twist), and a checksum of the data.  The write goes to
 * path + ".part" and is renamed into place.  The read checks magic, version, byte
 * order, lattice (layout hash, states, holes, amplitude count), the momenta and box
 * length unless CCX_CKPT_ANY_TWIST is given (a twist that reorders the orbitals changes
 * the layout hash as well), and the checksum; on any error t2 is left untouched and
 * CCX_EINVAL is returned.  Not in the reference (its runs always start from MP2). */
#define CCX_CKPT_ANY_TWIST 1
int ccx_t2_checkpoint_write(const ccx_layout *l, const char *path, const double *t2);
int ccx_t2_checkpoint_read(const ccx_layout *l, const char *path, int32_t flags, double *t2);
/* d2ij(1:A), d2ab(A+1:n) of the last residual, complex interleaved */
int ccx_get_denominators(ccx_engine *e, double *d2ij, double *d2ab);

/* ---- hot path --------------------------------------------------------- */
/* t2_intermediate(0), ccm_t2_eqn.f90:4-1304 (with setup_I6I7_intermediate
 * :1312-1518): the CCD right-hand side R and the dressed denominators from the
 * current T2. */
int ccx_t2_intermediate(ccx_engine *e);
/* diis_t1t2(count), ccm_diis.f90:74-249: T <- 0.75 T + 0.25 R/D, DIIS every
 * diis_step calls; *count is reset to 0 when DIIS runs, as in the reference.
 * The subspace is set by ccx_diis_setup (diis_setup, ccm_diis.f90:257-293). */
int ccx_diis_setup(ccx_engine *e, int32_t subspace, int32_t diis_step);
int ccx_diis_t1t2(ccx_engine *e, int32_t *count);
/* ccd_energy_save(ener), ccm_energy.f90:4-71: 1/4 sum T(ab,ij) V(ij,ab) */
int ccx_ccd_energy(ccx_engine *e, double ener[2]);
/* The same correlation energy on caller-owned device buffers, allocating nothing.
 * No counterpart in the reference.  For callers that cannot allocate device memory:
 * a host that owns every device buffer through its own pool, or code running where
 * an allocation is not allowed.  dims: device array of nch (n_hh, n_pp) pairs;
 * t2 / vhhpp: device, the t2_ccm(ch)%val (n_pp x n_hh) and vnn_hhpp(ch)%val
 * (n_hh x n_pp) blocks concatenated in channel order, complex interleaved; energy:
 * device, 2 doubles.  Asynchronous on stream (NULL: the legacy default stream).
 * Scratch is a static device array of 16384 channel slots (512 KiB) held by each
 * GPU that loads the library until exit; nch > 16384 is rejected.  The first call
 * in a CUDA context looks up that array's address -- make it before any stream
 * capture; the address is cached with the context's id, so after cudaDeviceReset (or
 * in a caller's own context) the next call looks it up again.
 * All calls share the array: calls that overlap on the GPU race. */
int ccx_ccd_energy_noalloc(int32_t nch, const int32_t *dims, const double *t2, const double *vhhpp, double *energy,
                           void *stream);
/* ||R - D T|| over the stored (ordered) amplitudes of the last residual */
int ccx_residual_norm(ccx_engine *e, double *norm);

typedef struct {
  int32_t mode;              /* CCX_MODE_* */
  int32_t precision;         /* CCX_PREC_* */
  int32_t max_iter;          /* reference: 100 (ccm_iter.f90:71) */
  double tol;                /* reference: 1e-6 on |dE| (ccm_iter.f90:74) */
  int32_t diis_dim;          /* standard mode history length */
  int32_t defect_period;     /* mixed precision: FP64 re-base every k iterations; 0 = adaptive
                                (when the mixed residual has dropped 1e4x, stalls or meets tol) */
  int32_t verbose;
  int32_t rebase;            /* mixed precision: CCX_REBASE_* */
  double rebase_drop;        /* mixed precision, adaptive policy: FP64 re-base once the mixed residual
                                has fallen by this factor since the last one (0: the default 1e-4) */
} ccx_iter_opts;
#define CCX_REBASE_FP64 0      /* products of a re-base on the FP64 FMA pipe */
#define CCX_REBASE_DIGITS 1    /* the pp-ladder, I4 and ring products of a re-base as exact 6-bit digit
                                  products on the BF16 tensor cores (Ozaki scheme), FP64-accurate */

typedef struct {
  int32_t iterations;
  int32_t converged;
  double e_mbpt2[2];         /* correlation energy at the start amplitudes */
  double e_ccd[2];           /* final correlation energy (eccsd - e0) */
  double res_norm;           /* ||R - D T|| of the last FP64 residual */
  double seconds;            /* device time of the loop */
  int32_t fp64_sweeps;       /* mixed precision: FP64 residual evaluations (re-bases) */
  int32_t mixed_iterations;  /* mixed precision: tensor-core residual evaluations */
} ccx_iter_result;

/* ccd_iter loop, ccm_iter.f90:67-133 */
int ccx_ccd_iter(ccx_engine *e, const ccx_iter_opts *opt, ccx_iter_result *res);

/* One residual evaluation of the last ccx_ccd_iter (or ccx_ccd_iter_batch) on an engine:
 * the structured form of the per-iteration energy lines the reference writes from
 * ccd_iter (ccm_iter.f90:67-133). */
typedef struct {
  int32_t iteration;         /* 1-based */
  int32_t kind;              /* CCX_ITER_* */
  double energy[2];          /* correlation energy after this iteration's update */
  double de;                 /* Re of the energy change since the previous record (the first: since MP2) */
  double res_norm;           /* ||R - D T|| of this residual (mixed kind: of the mixed residual) */
  double ms;                 /* host wall-clock milliseconds since the previous record; the loop
                                synchronises once an iteration, so this is the iteration's time */
  double term_ms[9];         /* profiling on: device ms of this iteration per residual term, in the
                                slots [0]..[8] of ccx_engine_timers; profiling off: 0 */
} ccx_iter_record;
#define CCX_ITER_REFERENCE 0   /* a step of the reference loop (|dE| test) */
#define CCX_ITER_FP64 1        /* an FP64 residual of the standard loop (or a mixed-precision re-base) */
#define CCX_ITER_MIXED 2       /* a mixed-precision (tensor-core correction) residual */
/* The records of the last solve: *n receives their count, and the first
 * min(*n, capacity) are copied to records (which may be NULL when capacity is 0). */
int ccx_engine_iter_log(const ccx_engine *e, int32_t capacity, ccx_iter_record *records, int32_t *n);
/* The one-time device set-up that the first ccx_ccd_iter with these options would do
 * (tensor-core operand tiles, digit planes of the interaction, DIIS history), without
 * solving, so that a host can keep set-up out of a timed or latency-critical solve.
 * Needs the interaction and amplitudes.  No counterpart in the reference. */
int ccx_engine_prepare(ccx_engine *e, const ccx_iter_opts *opt);
/* n engines on one device (for example the twists of a twist-averaged run,
 * ccm_main.f90:163-279, which the reference solves one after the other) solved
 * together in the standard mode: the iterations run in lockstep, each engine's kernels
 * on its own stream so that the GPU overlaps the engines, with one host
 * synchronisation per step for the whole batch.  res[i] is engine i's result; every
 * res[i].seconds and *seconds hold the wall time of the whole batch. */
int ccx_ccd_iter_batch(ccx_engine *const *engines, int32_t n, const ccx_iter_opts *opt, ccx_iter_result *res,
                       double *seconds);

/* Tile-shape autotuner of the grouped FP64 GEMM (ladder, I4, ring, and the mixed
 * residual's FP64 products).  For each bucket of the problems' column count N (<= 16,
 * <= 32, <= 64, > 64) it times the engine's own problems of that bucket with each tile
 * shape (0: 64 x 64 with 4 x 4 per thread, 1: 128 x 32 with 8 x 2), keeps the faster
 * shape and rebuilds the plans.  shapes[k]: the choice of bucket k; ms[2 k + s]: the
 * time of shape s on bucket k (ms, best of 3).  Needs the interaction and amplitudes;
 * call it between solves. */
int ccx_engine_autotune(ccx_engine *e, int32_t shapes[4], double ms[8]);
/* Launch-form autotuner of the tensor-core correction products of the mixed residual
 * (precision CCX_PREC_MIXED or CCX_PREC_MIXED_TF32): for the pp + hh ladders, dI4 + dX
 * and the ring in turn, it times the engine's own tiles launched once per bucket of the
 * column count (<= 32, <= 64, <= 128, wider; each launch with as many shared-memory
 * stages as its widest tile leaves) and launched all together (stages for the widest
 * tile of all), keeps the faster form and prepares the mixed residual with it.
 * merged[p]: 1 for one launch, 0 for one per bucket; ms[2 p + f]: the time of form f
 * (0 per bucket, 1 one launch; ms, best of 3).  Needs the interaction; call it between
 * solves.  Without it, one launch is used. */
int ccx_engine_autotune_tc(ccx_engine *e, int32_t precision, int32_t merged[3], double ms[6]);

/* ---- (T) -------------------------------------------------------------- */
/* pert_triples2, ccm_triples.f90:528-735 (NN part): E(T) from the current T2 with
 * the V_hppp / V_hhhp blocks of setup_vnn_hppp_block (ccm_iter.f90:1361-1810). */
int ccx_pert_triples(ccx_engine *e, double et[2]);
/* Arithmetic of the 18 gather-contractions W(abc, ijk) of ccx_pert_triples:
 * CCX_TRIPLES_FP32 (the default) runs them in FP32 on FP32 copies of T2, V_hppp and
 * V_hhhp; CCX_TRIPLES_FP64 in FP64.  The sum of |W|^2 / D is FP64 in both.  On the
 * benchmark lattices the FP32 form moves E(T) by about 1e-7 relative (the accuracy
 * bar is 1e-5).  No counterpart in the reference (all FP64). */
#define CCX_TRIPLES_FP64 0
#define CCX_TRIPLES_FP32 1
int ccx_set_triples_precision(ccx_engine *e, int32_t precision);

/* ---- learned warm start ------------------------------------------------------
 * No counterpart in the reference (which always starts from MP2, ccm_iter.f90:2329-2368).
 * A 4-layer MLP (18 features -> 128 -> 128 -> 128 -> 1, SiLU) predicts per packed T2
 * amplitude the difference between the converged CCD amplitude and its MP2 value, from
 * features that transfer across lattices: density, twist, bare denominator / e_F, bare
 * <ij|V|ab> and MP2 amplitude scaled by the volume, momentum transfers and pair momenta
 * / k_F, spin and isospin products, and a prior with its flag: the same difference
 * interpolated from solutions the solver converged at neighbouring densities of the
 * same lattice and twist (ccx_learner_set_prior; 0 and flag 0 without one).  With a
 * prior the network predicts the remainder of the difference beyond the prior, which is
 * added back in FP32 (a skip connection).  Training
 * (FP32, Adam) uses amplitudes the solver converged on other lattices; inference runs in
 * BF16 on the tensor cores.  Real engines only.  The CCD iteration from the warm start
 * is unchanged, so the converged energy is the same as from MP2. */
typedef struct ccx_learner ccx_learner;
#define CCX_ML_FEATURES 18
#define CCX_ML_PARAMS 35585    /* W1[128][18] b1 W2[128][128] b2 W3[128][128] b3 w4[128] b4, FP32 */
int ccx_learner_create(int32_t device, uint64_t seed, ccx_learner **out);
int ccx_learner_destroy(ccx_learner *l);
/* training samples (features, converged - MP2) from the engine's current T2 */
int ccx_learner_add_solution(ccx_learner *l, ccx_engine *e);
/* the same with every stride-th packed amplitude (large lattices, many solutions) */
int ccx_learner_add_solution_sampled(ccx_learner *l, ccx_engine *e, int32_t stride);
/* Prior of later add_solution / ccx_init_learned calls on target: per packed amplitude
 * of target, sum_i weights[i] times the converged-minus-MP2 correction of engines[i]'s
 * current T2 at the same quantum numbers, for example the two neighbouring densities of
 * the same lattice and twist with weights 0.5 and 0.5.  Amplitudes are matched through
 * the orbitals' quantum numbers, not their numbers: the index sort orders the states of a
 * degenerate shell by rounding-level differences of |k|^2, so the orbital numbering
 * differs between densities.  n = 0 clears the prior. */
int ccx_learner_set_prior(ccx_learner *l, ccx_engine *target, int32_t n, ccx_engine *const *engines,
                          const double *weights);
int ccx_learner_clear(ccx_learner *l);
int ccx_learner_samples(const ccx_learner *l, int64_t *n);
/* Adam on shuffled minibatches; *loss = mean loss of the last 10 steps */
int ccx_learner_train(ccx_learner *l, int32_t steps, int32_t batch, double lr, uint64_t seed, double *loss);
/* T2 <- MP2 + predicted correction (needs the interaction; replaces ccx_setup_t_amplitudes) */
int ccx_init_learned(ccx_engine *e, ccx_learner *l);
int ccx_learner_get_params(const ccx_learner *l, float *params);
int ccx_learner_set_params(ccx_learner *l, const float *params);
/* loss and gradient on a host batch (X: n x CCX_ML_FEATURES, y: n) with the training kernels */
int ccx_learner_loss_grad(ccx_learner *l, const float *X, const float *y, int32_t n, double *loss, float *grad);
/* network output on host features: tensor_cores 0 = FP32 training forward, 1 = BF16 kernel */
int ccx_learner_infer(ccx_learner *l, const float *X, int32_t n, float *out, int32_t tensor_cores);

/* ---- host buffers --------------------------------------------------------- */
/* Page-locked host memory that every device can address (cudaHostAlloc, portable and
 * mapped), for hosts that hand over large V families: ccx_set_vblock(s) reads blocks in
 * such memory in place or through the copy engines at the link rate.  No counterpart in
 * the reference (its blocks never leave the host). */
int ccx_host_alloc(int64_t bytes, void **ptr);
int ccx_host_free(void *ptr);

/* ---- diagnostics -------------------------------------------------------- */
const char *ccx_last_error(void);
/* the engine's CUDA stream (cudaStream_t), for callers that order their own work
 * or time with events on it */
int ccx_engine_stream(const ccx_engine *e, void **stream);
/* measured FP64 FMA throughput of the device (TFLOP/s), from a register-only probe */
int ccx_device_fp64_peak(int32_t device, double *tflops);
/* Self-test of the tensor-core split GEMM used by CCX_PREC_MIXED: nprob random
 * problems C += 1/2 A B (M_i x K_i times K_i x N_i, N_i <= 256) through the same
 * operand tiling and tcgen05 kernel, against an FP64 host product.
 * kind 0: BF16 hi/lo split, kind 1: TF32 hi/lo split; use_alo bit 0 clear drops the A_lo
 * term; use_alo bit 1 cuts K into up to three separately tiled products accumulated in one
 * tile with a C0 term (even problems C = C0 + 1/2 A B, odd ones C += C0 + 1/2 A B);
 * kind 2: the FP64-accurate digit-product (Ozaki) GEMM, checked against long double.
 * *max_rel_err = max |C - C_ref| / max |1/2 A B| over the problems; *ms kernel time. */
int ccx_selftest_tc_gemm(int32_t device, int32_t kind, int32_t nprob, const int32_t *M, const int32_t *N,
                         const int32_t *K, int32_t use_alo, uint64_t seed, double *max_rel_err, double *ms);
/* kernel launches issued by this engine since creation */
int ccx_engine_launches(const ccx_engine *e, int64_t *launches);
/* DIIS systems found singular (or with a non-finite solution) since creation; each one
 * kept the plain step instead of the extrapolation.  The reference prints ZGESV's info
 * and goes on with an undefined solution (ccm_diis.f90:173-180). */
int ccx_engine_diis_fallbacks(const ccx_engine *e, int64_t *n);
/* Failure path of the tensor-core kernel's bounded waits: runs the BF16x3 self-test
 * problems with each pipeline wait limited to wait_cycles clock cycles.  A limit too
 * short for the copies and MMAs to land makes the kernel give up: it records an error
 * word (1 load wait, 2 MMA wait, 3 drain wait ran out), waits with the full limit for its
 * own copies and MMAs in flight, frees its tensor memory and returns, and the context
 * stays usable.  *kernel_error receives that word (0: the product completed and was
 * checked against FP64 to the BF16x3 bound, 2e-4 of the largest product). */
int ccx_selftest_tc_wait(int32_t device, int64_t wait_cycles, int32_t *kernel_error);
/* on: ccx_ccd_iter records CUDA events around every residual term and tensor-core
 * launch (about 20 records per iteration, ~5% of a solve) so that ccx_engine_timers and
 * ccx_engine_kernel_timers report the breakdown; off (the default): only the solve's
 * total time is recorded and the breakdown reads zero. */
int ccx_engine_set_profiling(ccx_engine *e, int32_t on);
/* per-term device milliseconds of the last ccx_ccd_iter (profiling on):
 * [0] T_ph gather, [1] I9/I7, [2] I6, [3] I4, [4] ring, [5] R init, [6] ladders,
 * [7] update/energy, [8] DIIS, [9] total */
int ccx_engine_timers(const ccx_engine *e, double ms[10]);
/* device milliseconds and timed brackets of individual kernel launches in the last
 * ccx_ccd_iter with profiling on (CUDA events on the engine stream around each launch or launch group):
 * [0] X = V_hhpp' T' (FP64 split-K GEMM + reduce), [1] I4 (FP64), [2] ring (FP64),
 * [3] fused pp+hh ladder (FP64), [4] V_pppp' T' at a mixed-precision re-base (FP64),
 * [5] hh-ladder of the mixed residual (FP64), [6] pp-ladder and hh-ladder corrections
 * with the cached base terms, one launch (tensor cores), [7] dI4 correction (tensor
 * cores), [8] ring corrections dR_ph, one launch (tensor cores),
 * [9] operand splits, [10] pp-ladder, [11] I4 and [12] ring at a re-base as digit products
 * (tensor cores), [13] I7 of a mixed residual from the X entries it reads (FP64 column
 * dots), [14] X = V_hhpp'^T T' and [15] the hh-ladder base term T' I9' at a re-base as
 * digit products (tensor cores) */
int ccx_engine_kernel_timers(const ccx_engine *e, double ms[16], int64_t launches[16]);

#ifdef __cplusplus
}
#endif
#endif
