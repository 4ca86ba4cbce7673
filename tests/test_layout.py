"""Host logic of the engine library (no GPU): the basis and channel layout built by
libccx against the oracle's restatement of setup_sp_data / setup_channel_structures /
setup_ph_channel_structures, bit for bit; the ccm_in parser; the exported ABI."""
import os
import re

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

CONFIGS = [
    dict(nmax=2, A=14, snm=False, rho=0.08, theta=(0.0, 0.0, 0.0)),
    dict(nmax=1, A=2, snm=False, rho=0.08, theta=(0.0, 0.0, 0.0)),
    dict(nmax=1, A=4, snm=True, rho=0.16, theta=(0.0, 0.0, 0.0)),
    dict(nmax=2, A=28, snm=True, rho=0.16, theta=(0.0, 0.0, 0.0)),
    dict(nmax=1, A=14, snm=False, rho=0.10, theta=(0.3, -1.1, 2.0)),
    dict(nmax=3, A=66, snm=False, rho=0.16, theta=(0.0, 0.0, 0.0)),
]


# The lattices of the benchmark workloads, where ties in |k|^2 decide the occupied set
# (open shells under a twist): PNM 66 and SNM 132 at nmax=4, SNM 132 at nmax=3 at theta=0
# and at two twists of the 4x4x4 Gauss-Legendre grid on [-pi, pi]^3.
_GL = 0.8611363115940526 * np.pi, 0.3399810435848563 * np.pi
FULL_SIZE = [
    dict(nmax=4, A=66, snm=False, rho=0.16, theta=(0.0, 0.0, 0.0)),
    dict(nmax=3, A=132, snm=True, rho=0.16, theta=(0.0, 0.0, 0.0)),
    dict(nmax=3, A=132, snm=True, rho=0.16, theta=(_GL[0], -_GL[1], _GL[1])),
    dict(nmax=3, A=132, snm=True, rho=0.16, theta=(-_GL[0], -_GL[0], _GL[0])),
    dict(nmax=4, A=132, snm=True, rho=0.16, theta=(0.0, 0.0, 0.0)),
    dict(nmax=4, A=66, snm=False, rho=0.16, theta=(_GL[1], _GL[0], -_GL[1])),
]


def _ids(c):
    tw = "" if not any(c["theta"]) else "tw%+.2f%+.2f%+.2f" % tuple(c["theta"])
    return f"n{c['nmax']}A{c['A']}{'s' if c['snm'] else 'p'}{tw}"


@pytest.mark.parametrize("c", CONFIGS + FULL_SIZE, ids=_ids)
def test_layout_matches_oracle(ccx, O, c):
    o = O.Oracle(O.Config(nmax=c["nmax"], A=c["A"], snm=c["snm"], rho=c["rho"], theta=c["theta"],
                          layout_only=True))
    L = ccx.Layout.from_basis(c["nmax"], c["A"], c["rho"], snm=c["snm"], theta=c["theta"])
    a, b = o.orbits(), L.orbits()
    for k in ("nx", "ny", "nz", "sz", "tz"):
        assert np.array_equal(a[k], b[k]), k
    for k in ("kx", "ky", "kz", "e"):
        assert np.array_equal(a[k], b[k]), k  # bit-exact: same operation order
    assert L.orbits()["box_length"] == o.box_length
    cnt = L.counts()
    assert cnt["hhpp"] == o.n_channels(3) and cnt["hhhh"] == o.n_channels(1)
    assert cnt["hhhp"] == o.n_channels(2) and cnt["hphp"] == o.n_channels(4)
    assert cnt["ph_phhp"] == o.n_ph_channels(1) and cnt["ph_hphp"] == o.n_ph_channels(2)
    assert cnt["ph_hpph"] == o.n_ph_channels(3)
    assert cnt["amps"] == o.n_amps
    for kind in (1, 2, 3, 4):
        for ch in range(o.n_channels(kind)):
            q, n1, n2 = L.channel(kind, ch)
            assert np.array_equal(q, o.channel_qn(kind, ch))
            s1, s2 = L.pairs(kind, ch)
            assert np.array_equal(s1, o.channel_pairs(kind, 1, ch))
            if kind in (2, 3):
                assert np.array_equal(s2, o.channel_pairs(kind, 2, ch))
    for kind in (1, 2, 3):
        for ch in range(o.n_ph_channels(kind)):
            q, n1, n2 = L.channel(10 + kind, ch)
            assert np.array_equal(q, o.ph_channel_qn(kind, ch))
            s1, s2 = L.pairs(10 + kind, ch)
            assert np.array_equal(s1, o.ph_channel_pairs(kind, 1, ch))
            if kind != 2:
                assert np.array_equal(s2, o.ph_channel_pairs(kind, 2, ch))


def test_layout_from_caller_orbits(ccx, O):
    """A Fortran caller hands over all_orbit; the channel tables follow from it."""
    o = O.Oracle(O.Config(nmax=2, A=28, snm=True, rho=0.16))
    orb = o.orbits()
    L1 = ccx.Layout.from_orbits(orb, 28, o.box_length)
    L2 = ccx.Layout.from_basis(2, 28, 0.16, snm=True)
    assert L1.hash() == L2.hash()
    assert L1.counts() == L2.counts()


def test_layout_hash_changes_with_basis(ccx):
    h1 = ccx.Layout.from_basis(2, 14, 0.08).hash()
    h2 = ccx.Layout.from_basis(2, 14, 0.08, theta=(0.1, 0.0, 0.0)).hash()
    h3 = ccx.Layout.from_basis(2, 14, 0.08).hash()
    assert h1 == h3 and h1 != h2


def test_pnm66_nmax4_sizes(ccx):
    """PNM 66 at nmax=4 (1458 states): channel counts and block sizes."""
    L = ccx.Layout.from_basis(4, 66, 0.16)
    c = L.counts()
    assert c["hhpp"] == 185
    dims = L.hhpp_dims()
    nh = sorted(d[0] for d in dims)
    npp = sorted(d[1] for d in dims)
    assert (nh[0], nh[-1]) == (4, 132)
    assert (npp[0], npp[-1]) == (1112, 2784)
    assert c["amps"] == 8067968 == sum(h * p for h, p in dims)
    assert c["ph_phhp"] == 1816


def test_bad_basis_rejected(ccx):
    with pytest.raises(ccx.CcxError):
        ccx.Layout.from_basis(1, 200, 0.16)  # more particles than states
    with pytest.raises(ccx.CcxError):
        ccx.Layout.from_basis(1, 2, -1.0)


DECK = """! chiral order and cutoff
2, 500
! cE and cD
 0.5, -0.25
! number of particles
66
! pnm/snm, density/kfermi
pnm, density
! boundary conditions
PBC
! dens/kf, ntwist, nmax, my_twists
0.16,1,4,1
! cluster approximation
CCD(T)
! tnf switch, approximation
F, 0
! 3nf cutoff, exponent
400, 4
potential = chiral_like
mode = standard
tol = 1e-10
theta = 0.1, 0.2, 0.3
"""


def test_deck_parse(ccx):
    d = ccx.deck_parse(DECK)
    assert d["chiral_order"] == 2 and d["lambda"] == 500.0
    assert d["cE"] == 0.5 and d["cD"] == -0.25
    assert d["A"] == 66 and d["snm"] == 0 and d["input_is_kfermi"] == 0
    assert d["bc"] == "PBC" and d["cc_approx"] == "CCD(T)"
    assert d["dens_or_kf"] == 0.16 and d["ntwist"] == 1 and d["nmax"] == 4 and d["my_twists"] == 1
    assert d["tnf_switch"] == 0 and d["tnf_approx"] == 0
    assert d["cutoff_3nf"] == 400.0 and d["nexp_3nf"] == 4
    assert d["potential"] == ccx.POT_CHIRAL_LIKE and d["mode"] == ccx.MODE_STANDARD
    assert d["tol"] == 1e-10 and d["theta"] == (0.1, 0.2, 0.3)
    base = ccx.deck_parse("\n".join(DECK.splitlines()[:18]))
    assert base["potential"] == ccx.POT_MINNESOTA and base["mode"] == ccx.MODE_REFERENCE
    assert base["tol"] == 1e-6 and base["max_iter"] == 100


@pytest.mark.parametrize("bad", [
    "\n".join(DECK.splitlines()[:10]),                        # truncated deck
    DECK.replace("pnm, density", "xnm, density"),             # bad matter type
    DECK.replace("0.16,1,4,1", "abc,1,4,1"),                  # bad number
    DECK + "unknown_key = 3\n",                               # unknown extension key
])
def test_deck_parse_rejects_malformed(ccx, bad):
    with pytest.raises(ccx.CcxError) as e:
        ccx.deck_parse(bad)
    assert e.value.code == 1


def test_abi_exports_every_declared_symbol(ccx):
    import ctypes
    hdr = open(os.path.join(ROOT, "include", "ccx.h")).read()
    names = sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(ccx_\w+)\s*\(", hdr, re.M)))
    assert len(names) >= 30
    lib = ctypes.CDLL(ccx.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_engine_without_gpu_fails_loudly(ccx):
    """On a machine without a GPU the engine refuses to start (no CPU fallback)."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("GPU present")
    except ImportError:
        pass
    L = ccx.Layout.from_basis(1, 2, 0.08)
    with pytest.raises(ccx.CcxError) as e:
        ccx.Engine(L)
    assert e.value.code in (2, 6)
