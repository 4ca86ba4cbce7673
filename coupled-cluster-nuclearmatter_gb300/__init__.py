"""GB300 CCD + (T) engine for infinite nuclear matter: Python binding of the C ABI.

The engine itself is libccx.so (CUDA, sm_103a) built from csrc/ by build.py; this
module binds include/ccx.h with ctypes.  Nothing here computes on the CPU: when the
library or a GPU is missing every call raises CcxError.

Names follow the reference solver (deltafull-CCMkspace): t2_intermediate,
diis_t1t2, ccd_energy (ccd_energy_save), ccd_iter, pert_triples, and the T2 blocks
t2_ccm(ch)%val as (n_pp, n_hh) column-major complex arrays.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "libccx.so")

CH_HHHH, CH_HHHP, CH_HHPP, CH_HPHP, CH_HPPP = 1, 2, 3, 4, 5
CH_PH_PHHP, CH_PH_HPHP, CH_PH_HPPH = 11, 12, 13
V_PPPP = 6
POT_MINNESOTA, POT_CHIRAL_LIKE = 0, 1
TRIPLES_FP64, TRIPLES_FP32 = 0, 1
MODE_REFERENCE, MODE_STANDARD = 0, 1
PREC_FP64, PREC_MIXED, PREC_MIXED_TF32 = 0, 1, 2
REBASE_FP64, REBASE_DIGITS = 0, 1
CKPT_ANY_TWIST = 1
SCALAR_COMPLEX, SCALAR_REAL = 0, 1


class CcxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ccx error {code}: {msg}")
        self.code = code


class _Deck(C.Structure):
    _fields_ = [
        ("chiral_order", C.c_int32), ("lam", C.c_double), ("cE", C.c_double), ("cD", C.c_double),
        ("A", C.c_int32), ("snm", C.c_int32), ("input_is_kfermi", C.c_int32), ("bc", C.c_char * 16),
        ("dens_or_kf", C.c_double), ("ntwist", C.c_int32), ("nmax", C.c_int32), ("my_twists", C.c_int32),
        ("cc_approx", C.c_char * 16), ("tnf_switch", C.c_int32), ("tnf_approx", C.c_int32),
        ("cutoff_3nf", C.c_double), ("nexp_3nf", C.c_int32),
        ("potential", C.c_int32), ("lec_seed", C.c_uint64), ("mode", C.c_int32), ("diis_dim", C.c_int32),
        ("tol", C.c_double), ("max_iter", C.c_int32), ("precision", C.c_int32), ("theta", C.c_double * 3),
    ]


class _BasisParams(C.Structure):
    _fields_ = [("nmax", C.c_int32), ("A", C.c_int32), ("snm", C.c_int32), ("density", C.c_double),
                ("theta", C.c_double * 3)]


class _Orbits(C.Structure):
    _fields_ = [("n_states", C.c_int32), ("n_holes", C.c_int32),
                ("nx", C.POINTER(C.c_int32)), ("ny", C.POINTER(C.c_int32)), ("nz", C.POINTER(C.c_int32)),
                ("sz", C.POINTER(C.c_int32)), ("tz", C.POINTER(C.c_int32)),
                ("kx", C.POINTER(C.c_double)), ("ky", C.POINTER(C.c_double)), ("kz", C.POINTER(C.c_double)),
                ("e", C.POINTER(C.c_double)), ("box_length", C.c_double)]


class _EngineOptions(C.Structure):
    _fields_ = [("device", C.c_int32), ("scalar", C.c_int32)]


class _Potential(C.Structure):
    _fields_ = [("kind", C.c_int32), ("lec_seed", C.c_uint64), ("f32_literals", C.c_int32)]


class _IterOpts(C.Structure):
    _fields_ = [("mode", C.c_int32), ("precision", C.c_int32), ("max_iter", C.c_int32), ("tol", C.c_double),
                ("diis_dim", C.c_int32), ("defect_period", C.c_int32), ("verbose", C.c_int32), ("rebase", C.c_int32),
                ("rebase_drop", C.c_double)]


class _IterResult(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("converged", C.c_int32), ("e_mbpt2", C.c_double * 2),
                ("e_ccd", C.c_double * 2), ("res_norm", C.c_double), ("seconds", C.c_double),
                ("fp64_sweeps", C.c_int32), ("mixed_iterations", C.c_int32)]


class _IterRecord(C.Structure):
    _fields_ = [("iteration", C.c_int32), ("kind", C.c_int32), ("energy", C.c_double * 2), ("de", C.c_double),
                ("res_norm", C.c_double), ("ms", C.c_double), ("term_ms", C.c_double * 9)]


ITER_KINDS = ("reference", "fp64", "mixed")  # ccx_iter_record.kind
TERM_KEYS = ("tph_gather", "i9_i7", "i6", "i4", "ring", "r_init", "ladders", "update", "diis")

_lib = None
vp = C.c_void_p


def lib():
    """Load libccx.so (raises CcxError if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise CcxError(-1, f"{LIB_PATH} not built; run build.py (or __graft_entry__.build())")
    L = C.CDLL(LIB_PATH)
    i32, i64, dbl = C.c_int32, C.c_int64, C.c_double
    sig = {
        "ccx_last_error": ([], C.c_char_p),
        "ccx_deck_parse": ([C.c_char_p, C.POINTER(_Deck)], C.c_int),
        "ccx_layout_from_basis": ([C.POINTER(_BasisParams), C.POINTER(vp)], C.c_int),
        "ccx_layout_from_orbits": ([C.POINTER(_Orbits), C.POINTER(vp)], C.c_int),
        "ccx_layout_destroy": ([vp], C.c_int),
        "ccx_layout_orbits": ([vp, C.POINTER(_Orbits)], C.c_int),
        "ccx_layout_counts": ([vp, vp], C.c_int),
        "ccx_layout_channel": ([vp, i32, i32, vp, C.POINTER(i32), C.POINTER(i32)], C.c_int),
        "ccx_layout_pairs": ([vp, i32, i32, vp, vp], C.c_int),
        "ccx_layout_hash": ([vp, C.POINTER(C.c_uint64)], C.c_int),
        "ccx_engine_create": ([vp, C.POINTER(_EngineOptions), C.POINTER(vp)], C.c_int),
        "ccx_engine_destroy": ([vp], C.c_int),
        "ccx_engine_memory": ([vp, C.POINTER(i64)], C.c_int),
        "ccx_engine_launches": ([vp, C.POINTER(i64)], C.c_int),
        "ccx_engine_set_profiling": ([vp, i32], C.c_int),
        "ccx_engine_timers": ([vp, vp], C.c_int),
        "ccx_set_fock": ([vp, vp, vp], C.c_int),
        "ccx_set_vblock": ([vp, i32, i32, vp], C.c_int),
        "ccx_generate_interaction": ([vp, C.POINTER(_Potential)], C.c_int),
        "ccx_get_e0": ([vp, vp], C.c_int),
        "ccx_setup_t_amplitudes": ([vp], C.c_int),
        "ccx_set_t2": ([vp, i32, vp], C.c_int),
        "ccx_get_t2": ([vp, i32, vp], C.c_int),
        "ccx_get_t2_eqn": ([vp, i32, vp], C.c_int),
        "ccx_set_t2_all": ([vp, vp], C.c_int),
        "ccx_t2_checkpoint_write": ([vp, C.c_char_p, vp], C.c_int),
        "ccx_t2_checkpoint_read": ([vp, C.c_char_p, i32, vp], C.c_int),
        "ccx_get_t2_all": ([vp, vp], C.c_int),
        "ccx_get_denominators": ([vp, vp, vp], C.c_int),
        "ccx_t2_intermediate": ([vp], C.c_int),
        "ccx_diis_setup": ([vp, i32, i32], C.c_int),
        "ccx_diis_t1t2": ([vp, C.POINTER(i32)], C.c_int),
        "ccx_ccd_energy": ([vp, vp], C.c_int),
        "ccx_residual_norm": ([vp, C.POINTER(dbl)], C.c_int),
        "ccx_ccd_iter": ([vp, C.POINTER(_IterOpts), C.POINTER(_IterResult)], C.c_int),
        "ccx_engine_iter_log": ([vp, i32, vp, C.POINTER(i32)], C.c_int),
        "ccx_pert_triples": ([vp, vp], C.c_int),
        "ccx_get_vblock": ([vp, i32, i32, vp], C.c_int),
        "ccx_get_fock": ([vp, vp], C.c_int),
        "ccx_engine_stream": ([vp, C.POINTER(vp)], C.c_int),
        "ccx_device_fp64_peak": ([i32, C.POINTER(dbl)], C.c_int),
        "ccx_selftest_tc_gemm": ([i32, i32, i32, vp, vp, vp, i32, C.c_uint64, C.POINTER(dbl), C.POINTER(dbl)], C.c_int),
        "ccx_ccd_energy_noalloc": ([i32, vp, vp, vp, vp, vp], C.c_int),
        "ccx_selftest_tc_wait": ([i32, C.c_int64, C.POINTER(i32)], C.c_int),
        "ccx_engine_prepare": ([vp, C.POINTER(_IterOpts)], C.c_int),
        "ccx_host_alloc": ([C.c_int64, C.POINTER(vp)], C.c_int),
        "ccx_host_free": ([vp], C.c_int),
        "ccx_set_triples_precision": ([vp, i32], C.c_int),
        "ccx_engine_diis_fallbacks": ([vp, C.POINTER(C.c_int64)], C.c_int),
        "ccx_engine_kernel_timers": ([vp, vp, vp], C.c_int),
        "ccx_set_vblocks": ([vp, i32, i32, vp, vp], C.c_int),
        "ccx_ccd_iter_batch": ([vp, i32, vp, vp, C.POINTER(C.c_double)], C.c_int),
        "ccx_engine_autotune": ([vp, vp, vp], C.c_int),
        "ccx_engine_autotune_tc": ([vp, C.c_int32, vp, vp], C.c_int),
        "ccx_learner_create": ([i32, C.c_uint64, C.POINTER(vp)], C.c_int),
        "ccx_learner_destroy": ([vp], C.c_int),
        "ccx_learner_add_solution": ([vp, vp], C.c_int),
        "ccx_learner_add_solution_sampled": ([vp, vp, i32], C.c_int),
        "ccx_learner_set_prior": ([vp, vp, i32, vp, vp], C.c_int),
        "ccx_learner_clear": ([vp], C.c_int),
        "ccx_learner_samples": ([vp, vp], C.c_int),
        "ccx_learner_train": ([vp, i32, i32, C.c_double, C.c_uint64, C.POINTER(C.c_double)], C.c_int),
        "ccx_init_learned": ([vp, vp], C.c_int),
        "ccx_learner_get_params": ([vp, vp], C.c_int),
        "ccx_learner_set_params": ([vp, vp], C.c_int),
        "ccx_learner_loss_grad": ([vp, vp, vp, i32, C.POINTER(C.c_double), vp], C.c_int),
        "ccx_learner_infer": ([vp, vp, i32, vp, i32], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _check(rc: int):
    if rc != 0:
        raise CcxError(rc, lib().ccx_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(vp)


def _cplx_fortran(a: np.ndarray) -> np.ndarray:
    """Complex block -> contiguous interleaved doubles in column-major order."""
    z = np.asarray(a, dtype=np.complex128)
    return np.ascontiguousarray(z.reshape(-1, order="F")).view(np.float64)


def device_fp64_peak(device: int = 0) -> float:
    """Measured FP64 FMA throughput of the device in TFLOP/s."""
    x = C.c_double()
    _check(lib().ccx_device_fp64_peak(device, C.byref(x)))
    return x.value


def selftest_tc_gemm(shapes, kind: int = 0, use_alo: bool = True, seed: int = 1, device: int = 0,
                     segments: bool = False):
    """Tensor-core split GEMM against FP64 on random problems [(M, N, K), ...].
    segments: K cut into up to three separately tiled products accumulated into one
    tile plus a C0 term (even problems overwrite C, odd ones accumulate).
    Returns (max relative error, kernel ms)."""
    M = np.array([s[0] for s in shapes], np.int32)
    N = np.array([s[1] for s in shapes], np.int32)
    K = np.array([s[2] for s in shapes], np.int32)
    err, ms = C.c_double(), C.c_double()
    _check(lib().ccx_selftest_tc_gemm(device, kind, len(shapes), _ptr(M), _ptr(N), _ptr(K), int(use_alo) | (2 if segments else 0), seed,
                                      C.byref(err), C.byref(ms)))
    return err.value, ms.value


class HostBuffer:
    """Page-locked, device-addressable host memory (ccx_host_alloc) of n doubles."""

    def __init__(self, ndoubles: int):
        p = vp()
        _check(lib().ccx_host_alloc(8 * max(int(ndoubles), 1), C.byref(p)))
        self.ptr = p.value
        self.n = max(int(ndoubles), 1)

    def array(self) -> np.ndarray:
        return np.ctypeslib.as_array((C.c_double * self.n).from_address(self.ptr))

    def close(self):
        if self.ptr:
            lib().ccx_host_free(C.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def selftest_tc_wait(wait_cycles: int, device: int = 0) -> int:
    """Tensor-core self-test with every pipeline wait limited to wait_cycles; returns the
    kernel's error word (0: completed and checked, else the wait that ran out)."""
    err = C.c_int32()
    _check(lib().ccx_selftest_tc_wait(device, int(wait_cycles), C.byref(err)))
    return err.value


def ccd_energy_noalloc(nch: int, dims_ptr: int, t2_ptr: int, vhhpp_ptr: int, energy_ptr: int, stream: int = 0):
    """ccx_ccd_energy_noalloc on caller-owned device buffers (raw device pointers)."""
    _check(lib().ccx_ccd_energy_noalloc(nch, vp(dims_ptr), vp(t2_ptr), vp(vhhpp_ptr), vp(energy_ptr),
                                        vp(stream) if stream else None))


def ccd_iter_batch(engines, mode=MODE_STANDARD, precision=PREC_FP64, max_iter=200, tol=1e-10, diis_dim=8,
                   defect_period=0, verbose=False, rebase=REBASE_FP64, rebase_drop=0.0):
    """Solve several engines (e.g. twists) together in lockstep; returns (results, seconds)."""
    n = len(engines)
    hs = (vp * n)(*[e._h for e in engines])
    o = _IterOpts(mode, precision, max_iter, tol, diis_dim, defect_period, int(verbose), rebase, rebase_drop)
    rs = (_IterResult * n)()
    sec = C.c_double()
    _check(lib().ccx_ccd_iter_batch(hs, n, C.byref(o), rs, C.byref(sec)))
    out = []
    for r in rs:
        out.append({"iterations": r.iterations, "converged": bool(r.converged),
                    "e_mbpt2": complex(r.e_mbpt2[0], r.e_mbpt2[1]), "e_ccd": complex(r.e_ccd[0], r.e_ccd[1]),
                    "res_norm": r.res_norm, "seconds": r.seconds, "fp64_sweeps": r.fp64_sweeps,
                    "mixed_iterations": r.mixed_iterations})
    return out, sec.value


ML_FEATURES, ML_PARAMS = 18, 35585


class Learner:
    """Learned warm start: MLP predicting converged-minus-MP2 T2 amplitudes."""

    def __init__(self, device: int = 0, seed: int = 20261203):
        h = vp()
        _check(lib().ccx_learner_create(device, seed, C.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            lib().ccx_learner_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_solution(self, engine: "Engine", stride: int = 1):
        """Training samples from the engine's converged T2 (every stride-th amplitude)."""
        if stride == 1:
            _check(lib().ccx_learner_add_solution(self._h, engine._h))
        else:
            _check(lib().ccx_learner_add_solution_sampled(self._h, engine._h, int(stride)))

    def set_prior(self, target: "Engine", engines=(), weights=()):
        """Prior feature for target: sum_i weights[i] x the converged-minus-MP2 correction
        of engines[i] (neighbouring densities of the same lattice), matched by quantum
        numbers; no engines clears it."""
        n = len(engines)
        hs = (vp * max(n, 1))(*[e._h for e in engines])
        ws = (C.c_double * max(n, 1))(*[float(w) for w in weights])
        _check(lib().ccx_learner_set_prior(self._h, target._h, n, hs, ws))

    def clear(self):
        _check(lib().ccx_learner_clear(self._h))

    def samples(self) -> int:
        n = C.c_int64()
        _check(lib().ccx_learner_samples(self._h, C.byref(n)))
        return n.value

    def train(self, steps: int = 2000, batch: int = 8192, lr: float = 1e-3, seed: int = 1) -> float:
        loss = C.c_double()
        _check(lib().ccx_learner_train(self._h, steps, batch, lr, seed, C.byref(loss)))
        return loss.value

    def warm_start(self, engine: "Engine"):
        _check(lib().ccx_init_learned(engine._h, self._h))

    def params(self) -> np.ndarray:
        p = np.zeros(ML_PARAMS, np.float32)
        _check(lib().ccx_learner_get_params(self._h, _ptr(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == ML_PARAMS
        _check(lib().ccx_learner_set_params(self._h, _ptr(p)))

    def loss_grad(self, X, y):
        X = np.ascontiguousarray(X, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        loss = C.c_double()
        g = np.zeros(ML_PARAMS, np.float32)
        _check(lib().ccx_learner_loss_grad(self._h, _ptr(X), _ptr(y), len(y), C.byref(loss), _ptr(g)))
        return loss.value, g

    def infer(self, X, tensor_cores: bool = True) -> np.ndarray:
        X = np.ascontiguousarray(X, np.float32)
        out = np.zeros(len(X), np.float32)
        _check(lib().ccx_learner_infer(self._h, _ptr(X), len(X), _ptr(out), int(tensor_cores)))
        return out


def kfermi(density: float, snm: bool) -> float:
    """Fermi momentum (fm^-1) of a density (fm^-3): rho = g kf^3 / (3 pi^2) with g = 2 for
    symmetric matter, 1 for neutron matter (ccm_main.f90:930-945 converts the other way)."""
    return (3.0 * np.pi ** 2 * density / (2.0 if snm else 1.0)) ** (1.0 / 3.0)


def iteration_records(log, e0: float, A: int) -> list:
    """The structured per-iteration lines of a solve: Engine.iter_log() records as
    JSON-ready dicts with the energy per nucleon (E0 + E_CCD) / A beside the correlation
    energy; term_ms is kept only where the solve was profiled."""
    out = []
    for r in log:
        d = {"record": "iteration", "iteration": r["iteration"], "kind": r["kind"],
             "e_ccd": [r["e_ccd"].real, r["e_ccd"].imag], "e_per_a": (e0 + r["e_ccd"].real) / A,
             "de": r["de"], "res_norm": r["res_norm"], "ms": r["ms"]}
        if any(r["term_ms"].values()):
            d["term_ms"] = dict(r["term_ms"])
        out.append(d)
    return out


def result_record(A: int, density: float, snm: bool, e0: float, e_mbpt2: float, e_ccd: float,
                  e_triples=None, cE: float = 0.0, cD: float = 0.0, iterations=None) -> dict:
    """The final record of a run, the values of the (8f12.5) line ccm_main.f90:338-339
    writes: cE, cD, kf, density and, per nucleon, E0, MBPT2 = E0 + E_MP2, E_CCD = E0 +
    E_CCD(corr) and E_CCD + E(T) (None where (T) was not computed).  Energies are the real
    parts, in MeV; e_mbpt2, e_ccd and e_triples are correlation energies."""
    d = {"record": "result", "cE": cE, "cD": cD, "kf": kfermi(density, snm), "density": density,
         "e0_per_a": e0 / A, "mbpt2_per_a": (e0 + e_mbpt2) / A, "eccd_per_a": (e0 + e_ccd) / A,
         "eccdt_per_a": None if e_triples is None else (e0 + e_ccd + e_triples) / A}
    if iterations is not None:
        d["iterations"] = iterations
    return d


def deck_parse(text: str) -> dict:
    d = _Deck()
    _check(lib().ccx_deck_parse(text.encode(), C.byref(d)))
    out = {k: getattr(d, k) for k, _ in _Deck._fields_}
    out["bc"] = d.bc.decode()
    out["cc_approx"] = d.cc_approx.decode()
    out["theta"] = tuple(d.theta)
    out["lambda"] = out.pop("lam")
    return out


class Layout:
    """Basis and channel tables with the reference's ordering (host only)."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def from_basis(cls, nmax: int, A: int, density: float, snm: bool = False, theta=(0.0, 0.0, 0.0)) -> "Layout":
        p = _BasisParams(nmax, A, int(snm), density, (C.c_double * 3)(*theta))
        h = vp()
        _check(lib().ccx_layout_from_basis(C.byref(p), C.byref(h)))
        return cls(h)

    @classmethod
    def from_orbits(cls, orb: dict, n_holes: int, box_length: float) -> "Layout":
        keep = {k: np.ascontiguousarray(orb[k], dtype=np.int32) for k in ("nx", "ny", "nz", "sz", "tz")}
        keep.update({k: np.ascontiguousarray(orb[k], dtype=np.float64) for k in ("kx", "ky", "kz", "e")})
        o = _Orbits()
        o.n_states = len(keep["nx"])
        o.n_holes = n_holes
        for k in ("nx", "ny", "nz", "sz", "tz"):
            setattr(o, k, keep[k].ctypes.data_as(C.POINTER(C.c_int32)))
        for k in ("kx", "ky", "kz", "e"):
            setattr(o, k, keep[k].ctypes.data_as(C.POINTER(C.c_double)))
        o.box_length = box_length
        h = vp()
        _check(lib().ccx_layout_from_orbits(C.byref(o), C.byref(h)))
        return cls(h)

    def close(self):
        if self._h:
            lib().ccx_layout_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def orbits(self) -> dict:
        o = _Orbits()
        _check(lib().ccx_layout_orbits(self._h, C.byref(o)))
        n = o.n_states
        out = {k: np.ctypeslib.as_array(getattr(o, k), shape=(n,)).copy() for k in ("nx", "ny", "nz", "sz", "tz", "kx", "ky", "kz", "e")}
        out["n_holes"] = o.n_holes
        out["box_length"] = o.box_length
        return out

    def counts(self) -> dict:
        c = np.zeros(8, np.int64)
        _check(lib().ccx_layout_counts(self._h, _ptr(c)))
        keys = ("hhpp", "hhhh", "hhhp", "hphp", "ph_phhp", "ph_hphp", "ph_hpph", "amps")
        return dict(zip(keys, (int(x) for x in c)))

    def channel(self, kind: int, ch: int):
        q = np.zeros(4, np.int32)
        n1, n2 = C.c_int32(), C.c_int32()
        _check(lib().ccx_layout_channel(self._h, kind, ch, _ptr(q), C.byref(n1), C.byref(n2)))
        return q, n1.value, n2.value

    def pairs(self, kind: int, ch: int):
        _, n1, n2 = self.channel(kind, ch)
        a = np.zeros((max(n1, 1), 2), np.int32)
        b = np.zeros((max(n2, 1), 2), np.int32)
        _check(lib().ccx_layout_pairs(self._h, kind, ch, _ptr(a), _ptr(b)))
        return a[:n1], b[:n2]

    def write_t2_checkpoint(self, path: str, t2_all: np.ndarray) -> None:
        """Write amplitudes of this lattice (the t2_all() vector) to a checkpoint file."""
        z = np.ascontiguousarray(np.asarray(t2_all, np.complex128)).view(np.float64)
        if z.size != 2 * self.counts()["amps"]:
            raise CcxError(1, "amplitude vector does not match the lattice")
        _check(lib().ccx_t2_checkpoint_write(self._h, os.fsencode(path), _ptr(z)))

    def read_t2_checkpoint(self, path: str, any_twist: bool = False) -> np.ndarray:
        """Amplitudes of this lattice from a checkpoint file; any_twist accepts the same
        channel structure at another twist or box length."""
        z = np.zeros(2 * self.counts()["amps"])
        _check(lib().ccx_t2_checkpoint_read(self._h, os.fsencode(path), CKPT_ANY_TWIST if any_twist else 0, _ptr(z)))
        return z.view(np.complex128)

    def hash(self) -> int:
        h = C.c_uint64()
        _check(lib().ccx_layout_hash(self._h, C.byref(h)))
        return h.value

    def hhpp_dims(self):
        c = self.counts()["hhpp"]
        return [self.channel(CH_HHPP, i)[1:] for i in range(c)]


class Engine:
    """One CCD problem resident on one GPU."""

    def __init__(self, layout: Layout, device: int = 0, real: bool = True):
        self.layout = layout
        self.real = real
        o = _EngineOptions(device, SCALAR_REAL if real else SCALAR_COMPLEX)
        h = vp()
        _check(lib().ccx_engine_create(layout._h, C.byref(o), C.byref(h)))
        self._h = h
        self._dims = layout.hhpp_dims()  # (n_hh, n_pp) per hhpp channel

    def close(self):
        if getattr(self, "_h", None):
            lib().ccx_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- interaction ------------------------------------------------------
    def generate(self, potential: int = POT_MINNESOTA, lec_seed: int = 20261203, f32_literals: bool = True):
        p = _Potential(potential, lec_seed, int(f32_literals))
        _check(lib().ccx_generate_interaction(self._h, C.byref(p)))

    def set_fock(self, fock: np.ndarray, e0: complex = 0.0):
        f = _cplx_fortran(fock)
        z = np.array([complex(e0).real, complex(e0).imag])
        _check(lib().ccx_set_fock(self._h, _ptr(f), _ptr(z)))

    def set_vblock(self, kind: int, ch: int, block: np.ndarray):
        b = _cplx_fortran(block)
        _check(lib().ccx_set_vblock(self._h, kind, ch, _ptr(b)))

    def set_vblocks(self, kind: int, blocks: dict):
        """Many blocks of one kind in one call: {channel: block}."""
        bs = [_cplx_fortran(b) for b in blocks.values()]
        chs = (C.c_int32 * len(bs))(*blocks.keys())
        ptrs = (vp * len(bs))(*[b.ctypes.data for b in bs])
        _check(lib().ccx_set_vblocks(self._h, kind, len(bs), chs, ptrs))

    def vblock(self, kind: int, ch: int) -> np.ndarray:
        """One V block in the reference's ordered layout (see ccx_get_vblock)."""
        shape = self._vshape(kind, ch)
        z = np.zeros(2 * shape[0] * shape[1])
        _check(lib().ccx_get_vblock(self._h, kind, ch, _ptr(z)))
        return z.view(np.complex128).reshape(shape, order="F")

    def _vshape(self, kind, ch):
        if kind == V_PPPP:
            n = self._dims[ch][1]
            return (n, n)
        _, n1, n2 = self.layout.channel(kind, ch)
        if kind in (CH_HHHH, CH_HPHP):
            return (n1, n1)
        return (n1, n2)

    def fock(self) -> np.ndarray:
        n = len(self.layout.orbits()["nx"])
        z = np.zeros(2 * n * n)
        _check(lib().ccx_get_fock(self._h, _ptr(z)))
        return z.view(np.complex128).reshape(n, n, order="F")

    def stream(self) -> int:
        s = vp()
        _check(lib().ccx_engine_stream(self._h, C.byref(s)))
        return s.value or 0

    def e0(self) -> complex:
        z = np.zeros(2)
        _check(lib().ccx_get_e0(self._h, _ptr(z)))
        return complex(z[0], z[1])

    # ---- amplitudes ---------------------------------------------------------
    def setup_t_amplitudes(self):
        _check(lib().ccx_setup_t_amplitudes(self._h))

    def _get(self, fn, ch):
        nh, npp = self._dims[ch]
        z = np.zeros(2 * nh * npp)
        _check(fn(self._h, ch, _ptr(z)))
        return z.view(np.complex128).reshape(npp, nh, order="F")

    def t2(self, ch: int) -> np.ndarray:
        return self._get(lib().ccx_get_t2, ch)

    def t2_eqn(self, ch: int) -> np.ndarray:
        return self._get(lib().ccx_get_t2_eqn, ch)

    def set_t2(self, ch: int, t: np.ndarray):
        z = _cplx_fortran(t)
        _check(lib().ccx_set_t2(self._h, ch, _ptr(z)))

    def t2_all(self) -> np.ndarray:
        n = self.layout.counts()["amps"]
        z = np.zeros(2 * n)
        _check(lib().ccx_get_t2_all(self._h, _ptr(z)))
        return z.view(np.complex128)

    def set_t2_all(self, flat: np.ndarray):
        z = np.ascontiguousarray(np.asarray(flat, np.complex128)).view(np.float64)
        _check(lib().ccx_set_t2_all(self._h, _ptr(z)))

    def save_t2(self, path: str) -> None:
        """Checkpoint the current amplitudes (resume a solve, or harvest them)."""
        self.layout.write_t2_checkpoint(path, self.t2_all())

    def load_t2(self, path: str, any_twist: bool = False) -> None:
        """Amplitudes from a checkpoint of this lattice (any_twist: of another twist)."""
        self.set_t2_all(self.layout.read_t2_checkpoint(path, any_twist))

    def denominators(self):
        orb = self.layout.orbits()
        A = orb["n_holes"]
        n = len(orb["nx"])
        a = np.zeros(2 * A)
        b = np.zeros(2 * (n - A))
        _check(lib().ccx_get_denominators(self._h, _ptr(a), _ptr(b)))
        return a.view(np.complex128), b.view(np.complex128)

    # ---- hot path -------------------------------------------------------------
    def t2_intermediate(self):
        _check(lib().ccx_t2_intermediate(self._h))

    def diis_setup(self, subspace: int = 6, step: int = 6):
        _check(lib().ccx_diis_setup(self._h, subspace, step))

    def diis_t1t2(self, count: int) -> int:
        c = C.c_int32(count)
        _check(lib().ccx_diis_t1t2(self._h, C.byref(c)))
        return c.value

    def ccd_energy(self) -> complex:
        z = np.zeros(2)
        _check(lib().ccx_ccd_energy(self._h, _ptr(z)))
        return complex(z[0], z[1])

    def residual_norm(self) -> float:
        x = C.c_double()
        _check(lib().ccx_residual_norm(self._h, C.byref(x)))
        return x.value

    def ccd_iter(self, mode=MODE_REFERENCE, precision=PREC_FP64, max_iter=100, tol=1e-6, diis_dim=8,
                 defect_period=0, verbose=False, rebase=REBASE_FP64, rebase_drop=0.0) -> dict:
        o = _IterOpts(mode, precision, max_iter, tol, diis_dim, defect_period, int(verbose), rebase, rebase_drop)
        r = _IterResult()
        _check(lib().ccx_ccd_iter(self._h, C.byref(o), C.byref(r)))
        return {"iterations": r.iterations, "converged": bool(r.converged),
                "e_mbpt2": complex(r.e_mbpt2[0], r.e_mbpt2[1]), "e_ccd": complex(r.e_ccd[0], r.e_ccd[1]),
                "res_norm": r.res_norm, "seconds": r.seconds, "fp64_sweeps": r.fp64_sweeps,
                "mixed_iterations": r.mixed_iterations}

    def iter_log(self) -> list:
        """One record per residual evaluation of the last ccd_iter (or batched solve):
        iteration, kind ("reference", "fp64" or "mixed"), e_ccd after the update, de (the
        change since the previous record), res_norm, ms (host wall-clock of the iteration)
        and term_ms (device ms per residual term; zeros unless profiling is on)."""
        n = C.c_int32()
        _check(lib().ccx_engine_iter_log(self._h, 0, None, C.byref(n)))
        recs = (_IterRecord * max(n.value, 1))()
        _check(lib().ccx_engine_iter_log(self._h, n.value, recs, C.byref(n)))
        return [{"iteration": r.iteration, "kind": ITER_KINDS[r.kind], "e_ccd": complex(r.energy[0], r.energy[1]),
                 "de": r.de, "res_norm": r.res_norm, "ms": r.ms, "term_ms": dict(zip(TERM_KEYS, r.term_ms))}
                for r in recs[:n.value]]

    def prepare(self, mode=MODE_STANDARD, precision=PREC_FP64, diis_dim=8, rebase=REBASE_FP64):
        """The one-time set-up of a solve with these options, without solving."""
        o = _IterOpts(mode, precision, 1, 1e-10, diis_dim, 0, 0, rebase)
        _check(lib().ccx_engine_prepare(self._h, C.byref(o)))

    def set_triples_precision(self, fp32: bool) -> None:
        """(T) contractions in FP32 (default) or FP64; the |W|^2/D sum is FP64 either way."""
        _check(lib().ccx_set_triples_precision(self._h, TRIPLES_FP32 if fp32 else TRIPLES_FP64))

    def pert_triples(self) -> complex:
        z = np.zeros(2)
        _check(lib().ccx_pert_triples(self._h, _ptr(z)))
        return complex(z[0], z[1])

    # ---- diagnostics ----------------------------------------------------------
    def memory(self) -> int:
        x = C.c_int64()
        _check(lib().ccx_engine_memory(self._h, C.byref(x)))
        return x.value

    def launches(self) -> int:
        x = C.c_int64()
        _check(lib().ccx_engine_launches(self._h, C.byref(x)))
        return x.value

    def diis_fallbacks(self) -> int:
        """DIIS systems found singular since creation (each kept the plain step)."""
        x = C.c_int64()
        _check(lib().ccx_engine_diis_fallbacks(self._h, C.byref(x)))
        return x.value

    KERNEL_SLOTS = ("x_fp64", "i4_fp64", "ring_fp64", "ladder_fp64", "pp_rebase_fp64", "hh_fp64",
                    "pp_tc", "i4_tc", "ring_tc", "split", "pp_rebase_digits", "i4_rebase_digits",
                    "ring_rebase_digits", "i7_fp64", "x_rebase_digits", "hh_rebase_digits")

    def autotune(self):
        """Pick the FP64 GEMM tile shape per N bucket by timing; returns (shapes, ms)."""
        s = np.zeros(4, np.int32)
        ms = np.zeros(8)
        _check(lib().ccx_engine_autotune(self._h, _ptr(s), _ptr(ms)))
        return s.tolist(), ms.reshape(4, 2).tolist()

    def autotune_tc(self, precision: int = 1):
        """Pick each tensor-core correction product's launch form (one launch, or one per
        column bucket) by timing; returns (merged flags of pp, I4, ring; ms per form)."""
        m = np.zeros(3, np.int32)
        ms = np.zeros(6)
        _check(lib().ccx_engine_autotune_tc(self._h, int(precision), _ptr(m), _ptr(ms)))
        return m.tolist(), ms.reshape(3, 2).tolist()

    def kernel_timers(self) -> dict:
        """{slot: (total ms, timed brackets)} of individual launches in the last ccd_iter."""
        ms = np.zeros(16)
        n = np.zeros(16, np.int64)
        _check(lib().ccx_engine_kernel_timers(self._h, _ptr(ms), _ptr(n)))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(self.KERNEL_SLOTS)}

    def set_profiling(self, on: bool) -> None:
        """Per-term and per-kernel event timers of ccd_iter (off by default: only the
        total time is recorded; on costs ~20 event records per iteration)."""
        _check(lib().ccx_engine_set_profiling(self._h, int(bool(on))))

    def timers(self) -> dict:
        z = np.zeros(10)
        _check(lib().ccx_engine_timers(self._h, _ptr(z)))
        keys = ("tph_gather", "i9_i7", "i6", "i4", "ring", "r_init", "ladders", "update", "diis", "total")
        return dict(zip(keys, z.tolist()))
