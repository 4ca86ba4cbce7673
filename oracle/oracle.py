"""ctypes binding of the CPU oracle (oracle/ccd_oracle.c).

TEST INFRASTRUCTURE ONLY: the tests, the smoke check and the CPU-baseline leg of
the benchmark load this module as the checker of the GPU engine.  The product
never imports it.  Parity of the oracle with the reference is UNPINNED (the
reference ships no golden vectors and cannot be built here); see the header of
ccd_oracle.h for how it is validated instead.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "libccd_oracle.so")

POT_MINNESOTA = 0
POT_CHIRAL_LIKE = 1
MODE_REFERENCE = 0
MODE_STANDARD = 1


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "ccd_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


class _Params(C.Structure):
    _fields_ = [
        ("nmax", C.c_int),
        ("A", C.c_int),
        ("snm", C.c_int),
        ("rho", C.c_double),
        ("theta", C.c_double * 3),
        ("potential", C.c_int),
        ("lec_seed", C.c_uint64),
        ("minnesota_f32_literals", C.c_int),
        ("layout_only", C.c_int),
    ]


class _IterOpts(C.Structure):
    _fields_ = [
        ("mode", C.c_int),
        ("max_iter", C.c_int),
        ("tol", C.c_double),
        ("diis_dim", C.c_int),
        ("verbose", C.c_int),
    ]


class _IterResult(C.Structure):
    _fields_ = [
        ("iterations", C.c_int),
        ("e_mbpt2", C.c_double * 2),
        ("e_ccd", C.c_double * 2),
        ("res_norm", C.c_double),
        ("converged", C.c_int),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.ocl_create.restype = vp
        L.ocl_create.argtypes = [C.POINTER(_Params)]
        L.ocl_destroy.argtypes = [vp]
        for name in ("ocl_n_states",):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = C.c_int
        L.ocl_box_length.argtypes = [vp]
        L.ocl_box_length.restype = C.c_double
        L.ocl_kf.argtypes = [vp]
        L.ocl_kf.restype = C.c_double
        L.ocl_n_channels.argtypes = [vp, C.c_int]
        L.ocl_n_channels.restype = C.c_int
        L.ocl_n_ph_channels.argtypes = [vp, C.c_int]
        L.ocl_n_ph_channels.restype = C.c_int
        L.ocl_channel_qn.argtypes = [vp, C.c_int, C.c_int, vp]
        L.ocl_ph_channel_qn.argtypes = [vp, C.c_int, C.c_int, vp]
        L.ocl_channel_pairs.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp]
        L.ocl_channel_pairs.restype = C.c_int
        L.ocl_ph_channel_pairs.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp]
        L.ocl_ph_channel_pairs.restype = C.c_int
        L.ocl_get_orbits.argtypes = [vp] * 10
        for name in ("ocl_e0", "ocl_get_fock", "ocl_ccd_energy", "ocl_lecs"):
            getattr(L, name).argtypes = [vp, vp]
        for name in ("ocl_get_vhhpp", "ocl_get_vpppp", "ocl_get_vhhhh", "ocl_get_vhphp",
                     "ocl_get_vhhhp", "ocl_get_t2", "ocl_set_t2", "ocl_get_r2"):
            getattr(L, name).argtypes = [vp, C.c_int, vp]
        L.ocl_vmat.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, vp]
        L.ocl_n_amps.argtypes = [vp]
        L.ocl_n_amps.restype = C.c_int64
        L.ocl_mp2.argtypes = [vp]
        L.ocl_get_denoms.argtypes = [vp, vp, vp]
        L.ocl_t2_intermediate.argtypes = [vp]
        L.ocl_diis_setup.argtypes = [vp, C.c_int, C.c_int]
        L.ocl_diis_t1t2.argtypes = [vp, C.POINTER(C.c_int)]
        L.ocl_residual_norm.argtypes = [vp]
        L.ocl_residual_norm.restype = C.c_double
        L.ocl_ccd_iter.argtypes = [vp, C.POINTER(_IterOpts), C.POINTER(_IterResult)]
        L.ocl_ccd_iter.restype = C.c_int
        L.ocl_pert_triples.argtypes = [vp, vp]
        L.ocl_pert_triples_sample.argtypes = [vp, C.c_int, C.c_int, vp, C.POINTER(C.c_int64)]
        L.ocl_triples_channels.argtypes = [vp]
        L.ocl_triples_channels.restype = C.c_int
        L.ocl_triples_count.argtypes = [vp]
        L.ocl_triples_count.restype = C.c_int64
        L.ocl_num_threads.restype = C.c_int
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


@dataclass
class Config:
    nmax: int = 2
    A: int = 14
    snm: bool = False
    rho: float = 0.08
    theta: tuple = (0.0, 0.0, 0.0)
    potential: int = POT_MINNESOTA
    lec_seed: int = 20261203
    minnesota_f32_literals: bool = True
    layout_only: bool = False  # basis and channel tables only: no V blocks, no amplitudes


class Oracle:
    """One lattice + interaction, with the reference's layout, V blocks and T2 state."""

    def __init__(self, cfg: Config):
        self.cfg = cfg
        p = _Params()
        p.nmax, p.A, p.snm, p.rho = cfg.nmax, cfg.A, int(cfg.snm), cfg.rho
        for d in range(3):
            p.theta[d] = cfg.theta[d]
        p.potential = cfg.potential
        p.lec_seed = cfg.lec_seed
        p.minnesota_f32_literals = int(cfg.minnesota_f32_literals)
        p.layout_only = int(cfg.layout_only)
        self._L = lib()
        self._h = self._L.ocl_create(C.byref(p))
        if not self._h:
            raise RuntimeError("oracle: create failed")

    def close(self):
        if self._h:
            self._L.ocl_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- layout -------------------------------------------------------
    @property
    def n_states(self) -> int:
        return self._L.ocl_n_states(self._h)

    @property
    def box_length(self) -> float:
        return self._L.ocl_box_length(self._h)

    def orbits(self) -> dict:
        n = self.n_states
        ints = {k: np.zeros(n, np.int32) for k in ("nx", "ny", "nz", "sz", "tz")}
        dbl = {k: np.zeros(n, np.float64) for k in ("kx", "ky", "kz", "e")}
        self._L.ocl_get_orbits(self._h, *(_ptr(ints[k]) for k in ("nx", "ny", "nz", "sz", "tz")),
                               *(_ptr(dbl[k]) for k in ("kx", "ky", "kz", "e")))
        return {**ints, **dbl}

    def n_channels(self, kind: int) -> int:
        return self._L.ocl_n_channels(self._h, kind)

    def channel_qn(self, kind: int, ch: int) -> np.ndarray:
        q = np.zeros(4, np.int32)
        self._L.ocl_channel_qn(self._h, kind, ch, _ptr(q))
        return q

    def channel_pairs(self, kind: int, side: int, ch: int) -> np.ndarray:
        n = self._L.ocl_channel_pairs(self._h, kind, side, ch, None)
        out = np.zeros((max(n, 1), 2), np.int32)
        self._L.ocl_channel_pairs(self._h, kind, side, ch, _ptr(out))
        return out[:n]

    def n_ph_channels(self, kind: int) -> int:
        return self._L.ocl_n_ph_channels(self._h, kind)

    def ph_channel_qn(self, kind: int, ch: int) -> np.ndarray:
        q = np.zeros(4, np.int32)
        self._L.ocl_ph_channel_qn(self._h, kind, ch, _ptr(q))
        return q

    def ph_channel_pairs(self, kind: int, side: int, ch: int) -> np.ndarray:
        n = self._L.ocl_ph_channel_pairs(self._h, kind, side, ch, None)
        out = np.zeros((max(n, 1), 2), np.int32)
        self._L.ocl_ph_channel_pairs(self._h, kind, side, ch, _ptr(out))
        return out[:n]

    def hhpp_dims(self) -> list:
        return [(len(self.channel_pairs(3, 1, c)), len(self.channel_pairs(3, 2, c)))
                for c in range(self.n_channels(3))]

    # ---- hamiltonian ---------------------------------------------------
    def e0(self) -> complex:
        z = np.zeros(2)
        self._L.ocl_e0(self._h, _ptr(z))
        return complex(z[0], z[1])

    def fock(self) -> np.ndarray:
        n = self.n_states
        z = np.zeros(2 * n * n)
        self._L.ocl_get_fock(self._h, _ptr(z))
        return z.view(np.complex128).reshape(n, n, order="F")

    def lecs(self) -> np.ndarray:
        z = np.zeros(9)
        self._L.ocl_lecs(self._h, _ptr(z))
        return z

    def vmat(self, p, q, r, s) -> complex:
        z = np.zeros(2)
        self._L.ocl_vmat(self._h, p, q, r, s, _ptr(z))
        return complex(z[0], z[1])

    def _block(self, fn, ch, rows, cols):
        z = np.zeros(2 * rows * cols)
        fn(self._h, ch, _ptr(z))
        return z.view(np.complex128).reshape(rows, cols, order="F")

    def v_hhpp(self, ch):
        nh, npp = self.hhpp_dims()[ch] if not hasattr(self, "_dims") else self._dims[ch]
        return self._block(self._L.ocl_get_vhhpp, ch, nh, npp)

    def v_pppp(self, ch):
        npp = len(self.channel_pairs(3, 2, ch))
        return self._block(self._L.ocl_get_vpppp, ch, npp, npp)

    def v_hhhh(self, ch):
        n = len(self.channel_pairs(1, 1, ch))
        return self._block(self._L.ocl_get_vhhhh, ch, n, n)

    def v_hphp(self, ch):
        n = len(self.channel_pairs(4, 1, ch))
        return self._block(self._L.ocl_get_vhphp, ch, n, n)

    def v_hhhp(self, ch):
        n1 = len(self.channel_pairs(2, 1, ch))
        n2 = len(self.channel_pairs(2, 2, ch))
        return self._block(self._L.ocl_get_vhhhp, ch, n1, n2)

    # ---- amplitudes ----------------------------------------------------
    @property
    def n_amps(self) -> int:
        return self._L.ocl_n_amps(self._h)

    def mp2(self):
        self._L.ocl_mp2(self._h)

    def t2(self, ch) -> np.ndarray:
        nh = len(self.channel_pairs(3, 1, ch))
        npp = len(self.channel_pairs(3, 2, ch))
        return self._block(self._L.ocl_get_t2, ch, npp, nh)

    def r2(self, ch) -> np.ndarray:
        nh = len(self.channel_pairs(3, 1, ch))
        npp = len(self.channel_pairs(3, 2, ch))
        return self._block(self._L.ocl_get_r2, ch, npp, nh)

    def set_t2(self, ch, t: np.ndarray):
        a = np.asfortranarray(t, dtype=np.complex128)
        flat = np.ascontiguousarray(a.reshape(-1, order="F")).view(np.float64)
        self._L.ocl_set_t2(self._h, ch, _ptr(flat))

    def all_t2(self) -> list:
        return [self.t2(c) for c in range(self.n_channels(3))]

    def all_r2(self) -> list:
        return [self.r2(c) for c in range(self.n_channels(3))]

    def denoms(self):
        A = self.cfg.A
        d1 = np.zeros(2 * A)
        d2 = np.zeros(2 * (self.n_states - A))
        self._L.ocl_get_denoms(self._h, _ptr(d1), _ptr(d2))
        return d1.view(np.complex128), d2.view(np.complex128)

    # ---- hot path ------------------------------------------------------
    def t2_intermediate(self):
        self._L.ocl_t2_intermediate(self._h)

    def diis_setup(self, subspace=6, step=6):
        self._L.ocl_diis_setup(self._h, subspace, step)

    def diis_t1t2(self, count: int) -> int:
        c = C.c_int(count)
        self._L.ocl_diis_t1t2(self._h, C.byref(c))
        return c.value

    def energy(self) -> complex:
        z = np.zeros(2)
        self._L.ocl_ccd_energy(self._h, _ptr(z))
        return complex(z[0], z[1])

    def residual_norm(self) -> float:
        return self._L.ocl_residual_norm(self._h)

    def ccd_iter(self, mode=MODE_REFERENCE, max_iter=100, tol=1e-6, diis_dim=8, verbose=False) -> dict:
        o = _IterOpts()
        o.mode, o.max_iter, o.tol, o.diis_dim, o.verbose = mode, max_iter, tol, diis_dim, int(verbose)
        r = _IterResult()
        self._L.ocl_ccd_iter(self._h, C.byref(o), C.byref(r))
        return {
            "iterations": r.iterations,
            "e_mbpt2": complex(r.e_mbpt2[0], r.e_mbpt2[1]),
            "e_ccd": complex(r.e_ccd[0], r.e_ccd[1]),
            "res_norm": r.res_norm,
            "converged": bool(r.converged),
        }

    def triples(self) -> complex:
        z = np.zeros(2)
        self._L.ocl_pert_triples(self._h, _ptr(z))
        return complex(z[0], z[1])

    def triples_sample(self, k0: int, stride: int):
        """(E(T) over the (abc) triples k0, k0 + stride, ... of every triple channel, the
        (abc, ijk) pairs that covers)."""
        z = np.zeros(2)
        n = C.c_int64()
        self._L.ocl_pert_triples_sample(self._h, int(k0), int(stride), _ptr(z), C.byref(n))
        return complex(z[0], z[1]), n.value

    def triples_channels(self) -> int:
        return self._L.ocl_triples_channels(self._h)

    def triples_count(self) -> int:
        return self._L.ocl_triples_count(self._h)


def num_threads() -> int:
    return lib().ocl_num_threads()
