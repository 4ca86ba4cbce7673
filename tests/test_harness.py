"""ccx_run, the host program that drives the C ABI as the reference's driver drives its
solver (deck -> layout -> interaction -> MP2 -> ccd_iter loop -> (T)).

CPU: the host part (deck parsing, the kfermi conversion of ccm_main.f90:930-945, the
layout summary against the Python binding), argument errors, and the engine refusing
to start without a GPU.  GPU: the reference loop driven call by call with the
interaction handed over block by block from host arrays, against the library's own
reference-mode loop; the standard-mode mixed solve; a checkpoint resume."""
import math
import os
import re
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
RUN = os.path.join(ROOT, "coupled-cluster-nuclearmatter_gb300", "build", "ccx_run")

DECK = """! chiral order and cutoff
2, 500
! cE and cD
 0.5, -0.25
! number of particles
14
! pnm/snm, density/kfermi
pnm, {input}
! boundary conditions
PBC
! dens/kf, ntwist, nmax, my_twists
{value},1,2,1
! cluster approximation
{approx}
! tnf switch, approximation
F, 0
! 3nf cutoff, exponent
400, 4
"""


def run(*args, check=True):
    r = subprocess.run([RUN, *map(str, args)], capture_output=True, text=True, timeout=600)
    if check and r.returncode != 0:
        raise AssertionError(f"ccx_run {args} -> {r.returncode}\n{r.stdout}\n{r.stderr}")
    return r


def fields(out: str) -> dict:
    d = {}
    for line in out.splitlines():
        parts = line.split()
        if parts:
            d.setdefault(parts[0], parts[1:])
    return d


def layout_line(out: str) -> dict:
    p = fields(out)["layout"]
    return {p[i]: p[i + 1] for i in range(0, len(p), 2)}


@pytest.fixture(scope="module")
def built(ccx):
    assert os.path.exists(RUN), "build() makes coupled-cluster-nuclearmatter_gb300/build/ccx_run"
    return RUN


def test_layout_summary_matches_binding(ccx, built):
    lay = layout_line(run("--nmax", 2, "--A", 14, "--density", 0.08, "--layout-only").stdout)
    L = ccx.Layout.from_basis(2, 14, 0.08)
    c = L.counts()
    assert int(lay["states"]) == 250 and int(lay["holes"]) == 14
    assert int(lay["hhpp"]) == c["hhpp"] and int(lay["hphp"]) == c["hphp"] and int(lay["amps"]) == c["amps"]
    assert int(lay["hash"], 16) == L.hash()
    assert float(lay["box_fm"]) == pytest.approx(L.orbits()["box_length"], rel=1e-9)


def test_deck_kfermi_is_converted_like_the_reference(ccx, built, tmp_path):
    # ccm_main.f90:934: PNM density = kf^3 / (3 pi^2)
    kf = 1.05
    p = tmp_path / "ccm_in"
    p.write_text(DECK.format(input="kfermi", value=kf, approx="CCD"))
    lay = layout_line(run("--deck", p, "--layout-only").stdout)
    rho = kf ** 3 / 3.0 / math.pi ** 2
    L = ccx.Layout.from_basis(2, 14, rho)
    assert int(lay["hash"], 16) == L.hash()
    assert float(lay["box_fm"]) == pytest.approx(L.orbits()["box_length"], rel=1e-9)
    # the same deck with the density given directly
    q = tmp_path / "ccm_in_dens"
    q.write_text(DECK.format(input="density", value=0.08, approx="CCD"))
    lay2 = layout_line(run("--deck", q, "--layout-only").stdout)
    assert int(lay2["hash"], 16) == ccx.Layout.from_basis(2, 14, 0.08).hash()


def test_argument_errors(built, tmp_path):
    assert run("--bogus", check=False).returncode == 2
    assert run("--nmax", 2, check=False).returncode == 2                  # no A / density
    assert run("--nmax", "x", check=False).returncode == 2
    bad = tmp_path / "bad_in"
    bad.write_text("not a deck\n")
    r = run("--deck", bad, "--layout-only", check=False)
    assert r.returncode == 1 and "ccx_deck_parse" in r.stderr


def test_no_gpu_is_refused(ccx, built):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    r = run("--nmax", 1, "--A", 14, "--density", 0.08, check=False)
    assert r.returncode == 6 and "no CUDA device" in r.stderr
    assert "layout states" in r.stdout  # the host part ran first


@pytest.mark.gpu
def test_reference_loop_with_host_blocks_matches_library_loop(ccx, built):
    """The Fortran flow: V handed over block by block from host arrays, then
    t2_intermediate / diis_t1t2 / ccd_energy called per iteration to |dE| < 1e-6,
    against ccx_ccd_iter's reference mode on a generated interaction."""
    out = fields(run("--nmax", 2, "--A", 14, "--density", 0.08, "--blocks", "host", "--loop", "shim").stdout)
    L = ccx.Layout.from_basis(2, 14, 0.08)
    e = ccx.Engine(L, real=True)
    e.generate()
    e.setup_t_amplitudes()
    r = e.ccd_iter(mode=ccx.MODE_REFERENCE)
    assert float(out["e0"][0]) == pytest.approx(e.e0().real, rel=1e-13)
    assert float(out["e_mbpt2"][0]) == pytest.approx(r["e_mbpt2"].real, rel=1e-12)
    # both stop at |dE| < 1e-6 MeV; DIIS of the reference is ill-conditioned (see the
    # step-by-step parity test), so the energies agree at the 1e-6 bar
    assert float(out["e_ccd"][0]) == pytest.approx(r["e_ccd"].real, rel=5e-7)
    assert abs(int(out["iterations"][0]) - r["iterations"]) <= 2


@pytest.mark.gpu
def test_standard_mixed_solve_and_checkpoint_resume(ccx, built, tmp_path):
    ck = str(tmp_path / "c1.t2")
    args = ["--nmax", 2, "--A", 14, "--density", 0.08, "--mode", "standard", "--tol", 1e-10]
    out = fields(run(*args, "--precision", "bf16x3", "--rebase", "digits", "--save", ck).stdout)
    L = ccx.Layout.from_basis(2, 14, 0.08)
    e = ccx.Engine(L, real=True)
    e.generate()
    e.setup_t_amplitudes()
    r = e.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10)
    assert int(out["converged"][0]) == 1
    assert float(out["e_ccd"][0]) == pytest.approx(r["e_ccd"].real, rel=1e-10)
    assert os.path.exists(ck)
    res = fields(run(*args, "--load", ck).stdout)
    assert int(res["converged"][0]) == 1 and int(res["iterations"][0]) <= 1
    assert float(res["e_ccd"][0]) == pytest.approx(r["e_ccd"].real, rel=1e-10)
