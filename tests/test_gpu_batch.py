"""Twist batch: several lattices (twists) solved together in lockstep through
ccx_ccd_iter_batch give exactly the per-engine results of ccx_ccd_iter."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TWISTS = [(0.0, 0.0, 0.0), (0.7, -0.3, 0.2), (-1.1, 0.5, 0.9), (2.0, 1.4, -0.6)]


def engines(ccx, nmax=2, A=14, rho=0.08):
    out = []
    for th in TWISTS:
        L = ccx.Layout.from_basis(nmax, A, rho, theta=th)
        e = ccx.Engine(L, real=True)
        e.generate()
        out.append(e)
    return out


@pytest.mark.parametrize("form", ["fp64", "mixed_digits"])
def test_batch_matches_single_solves(ccx, form):
    prec, rb = (ccx.PREC_FP64, ccx.REBASE_FP64) if form == "fp64" else (ccx.PREC_MIXED, ccx.REBASE_DIGITS)
    es = engines(ccx)
    singles = []
    for e in es:
        e.setup_t_amplitudes()
        singles.append(e.ccd_iter(mode=ccx.MODE_STANDARD, precision=prec, rebase=rb, tol=1e-10, max_iter=200))
    for e in es:
        e.setup_t_amplitudes()
    batch, sec = ccx.ccd_iter_batch(es, precision=prec, rebase=rb, tol=1e-10, max_iter=200)
    assert sec > 0
    for s, b in zip(singles, batch):
        assert s["converged"] and b["converged"]
        assert b["iterations"] == s["iterations"]
        assert b["fp64_sweeps"] == s["fp64_sweeps"]
        # the same kernels in the same order per engine: identical to rounding
        assert abs(b["e_ccd"] - s["e_ccd"]) <= 1e-13 * abs(s["e_ccd"])
    # the twists are different lattices: their total energies differ (with a Minnesota
    # interaction the correlation energy itself depends on the twist only through the
    # occupied set, since V and the denominators depend on momentum differences)
    totals = {round((e.e0() + b["e_ccd"]).real, 6) for e, b in zip(es, batch)}
    assert len(totals) == len(TWISTS)


def test_batch_rejects_reference_mode(ccx):
    es = engines(ccx)[:2]
    for e in es:
        e.setup_t_amplitudes()
    with pytest.raises(ccx.CcxError):
        ccx.ccd_iter_batch(es, mode=ccx.MODE_REFERENCE)
