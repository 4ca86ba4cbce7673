"""Mixed-precision CCD (tensor-core BF16x3 / TF32x3 contractions with FP64 defect
correction) against the FP64 solve of the same engine and the oracle.

Only an FP64 residual can end a mixed solve, so at the same tolerance the converged
E/A agrees with the FP64 one to rounding; the accuracy bar is 1 keV/nucleon."""
import pytest

pytestmark = pytest.mark.gpu


def solve(ccx, nmax, A, rho, precision, tol=1e-10, defect_period=0, snm=False, rebase=0):
    L = ccx.Layout.from_basis(nmax, A, rho, snm=snm)
    e = ccx.Engine(L, real=True)
    e.generate()
    e.setup_t_amplitudes()
    r = e.ccd_iter(mode=ccx.MODE_STANDARD, precision=precision, tol=tol, max_iter=200, defect_period=defect_period,
                   rebase=rebase)
    return e, r


@pytest.mark.parametrize("prec", ["bf16", "tf32"])
def test_mixed_matches_fp64_pnm14(ccx, O, prec):
    p = ccx.PREC_MIXED if prec == "bf16" else ccx.PREC_MIXED_TF32
    e64, r64 = solve(ccx, 2, 14, 0.08, ccx.PREC_FP64)
    em, rm = solve(ccx, 2, 14, 0.08, p)
    assert r64["converged"] and rm["converged"]
    assert rm["res_norm"] < 1e-10
    assert rm["fp64_sweeps"] >= 1 and rm["mixed_iterations"] >= 1
    assert abs(rm["e_ccd"] - r64["e_ccd"]) < 1e-10 * abs(r64["e_ccd"])
    o = O.Oracle(O.Config(nmax=2, A=14, rho=0.08))
    o.mp2()
    ro = o.ccd_iter(mode=O.MODE_STANDARD, tol=1e-10)
    assert abs(rm["e_ccd"] - ro["e_ccd"]) < 1e-10 * abs(ro["e_ccd"])


def test_mixed_fixed_defect_period(ccx):
    _, r64 = solve(ccx, 2, 14, 0.08, ccx.PREC_FP64)
    _, rm = solve(ccx, 2, 14, 0.08, ccx.PREC_MIXED, defect_period=3)
    assert rm["converged"] and abs(rm["e_ccd"] - r64["e_ccd"]) < 1e-10 * abs(r64["e_ccd"])


def test_mixed_snm_minnesota(ccx):
    _, r64 = solve(ccx, 2, 28, 0.16, ccx.PREC_FP64, snm=True)
    _, rm = solve(ccx, 2, 28, 0.16, ccx.PREC_MIXED, snm=True)
    assert rm["converged"] and abs(rm["e_ccd"] - r64["e_ccd"]) < 1e-10 * abs(r64["e_ccd"])


def test_mixed_pnm66_full_size(ccx):
    """PNM 66 at nmax=4 (1458 states): E/A of the mixed solve vs FP64, in keV."""
    e64, r64 = solve(ccx, 4, 66, 0.16, ccx.PREC_FP64)
    em, rm = solve(ccx, 4, 66, 0.16, ccx.PREC_MIXED)
    assert rm["converged"] and rm["res_norm"] < 1e-10
    dea_kev = abs((rm["e_ccd"] - r64["e_ccd"]).real) / 66 * 1e3
    assert dea_kev < 1e-6  # well inside the 1 keV bar
    assert rm["seconds"] < r64["seconds"]


@pytest.mark.parametrize("prec", ["bf16", "tf32"])
def test_digit_rebase_matches_fp64_pnm14(ccx, prec):
    """Re-base products as exact digit products on the tensor cores: same fixed point."""
    p = ccx.PREC_MIXED if prec == "bf16" else ccx.PREC_MIXED_TF32
    _, r64 = solve(ccx, 2, 14, 0.08, ccx.PREC_FP64)
    _, rd = solve(ccx, 2, 14, 0.08, p, rebase=ccx.REBASE_DIGITS)
    assert rd["converged"] and rd["res_norm"] < 1e-10
    assert abs(rd["e_ccd"] - r64["e_ccd"]) < 1e-10 * abs(r64["e_ccd"])


def test_digit_rebase_pnm66_full_size(ccx):
    e64, r64 = solve(ccx, 4, 66, 0.16, ccx.PREC_FP64)
    ed, rd = solve(ccx, 4, 66, 0.16, ccx.PREC_MIXED, rebase=ccx.REBASE_DIGITS)
    assert rd["converged"] and rd["res_norm"] < 1e-10
    assert abs((rd["e_ccd"] - r64["e_ccd"]).real) / 66 * 1e3 < 1e-6
    # the re-base's pp-ladder agrees with the FP64 GEMM: the FP64 and digit re-base
    # solves stop at the same residual level
    _, rf = solve(ccx, 4, 66, 0.16, ccx.PREC_MIXED)
    assert rd["fp64_sweeps"] <= rf["fp64_sweeps"] + 1


@pytest.mark.parametrize("rebase", [0, 1], ids=["fp64_rebase", "digit_rebase"])
def test_mixed_complex_chiral_like_snm(ccx, O, rebase):
    """Complex engine (chiral-like SNM, complex V): each complex product runs as four
    real tensor-core products; the converged energy matches the complex FP64 solve
    and the oracle."""
    L = ccx.Layout.from_basis(1, 4, 0.16, snm=True)
    e64 = ccx.Engine(L, real=False)
    e64.generate(potential=ccx.POT_CHIRAL_LIKE)
    e64.setup_t_amplitudes()
    r64 = e64.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10, max_iter=200)
    em = ccx.Engine(L, real=False)
    em.generate(potential=ccx.POT_CHIRAL_LIKE)
    em.setup_t_amplitudes()
    rm = em.ccd_iter(mode=ccx.MODE_STANDARD, precision=ccx.PREC_MIXED, tol=1e-10, max_iter=200, rebase=rebase)
    assert r64["converged"] and rm["converged"] and rm["res_norm"] < 1e-10
    assert rm["mixed_iterations"] >= 1
    assert abs(rm["e_ccd"] - r64["e_ccd"]) < 1e-10 * abs(r64["e_ccd"])
    o = O.Oracle(O.Config(nmax=1, A=4, rho=0.16, snm=True, potential=O.POT_CHIRAL_LIKE))
    o.mp2()
    ro = o.ccd_iter(mode=O.MODE_STANDARD, tol=1e-10)
    assert abs(rm["e_ccd"] - ro["e_ccd"]) < 1e-9 * abs(ro["e_ccd"])


def test_mixed_complex_matches_real_engine(ccx):
    """The same real problem through a complex engine: identical energies to rounding."""
    L = ccx.Layout.from_basis(2, 14, 0.08)
    er = ccx.Engine(L, real=True)
    ec = ccx.Engine(L, real=False)
    for e in (er, ec):
        e.generate()
        e.setup_t_amplitudes()
    rr = er.ccd_iter(mode=ccx.MODE_STANDARD, precision=ccx.PREC_MIXED, tol=1e-10, max_iter=200,
                     rebase=ccx.REBASE_DIGITS)
    rc = ec.ccd_iter(mode=ccx.MODE_STANDARD, precision=ccx.PREC_MIXED, tol=1e-10, max_iter=200,
                     rebase=ccx.REBASE_DIGITS)
    assert rr["converged"] and rc["converged"]
    assert abs(rc["e_ccd"] - rr["e_ccd"]) < 1e-10 * abs(rr["e_ccd"])


def test_mixed_rejects_unsupported(ccx):
    L = ccx.Layout.from_basis(1, 2, 0.08)
    er = ccx.Engine(L, real=True)
    er.generate()
    er.setup_t_amplitudes()
    with pytest.raises(ccx.CcxError):
        er.ccd_iter(mode=ccx.MODE_REFERENCE, precision=ccx.PREC_MIXED)
    with pytest.raises(ccx.CcxError):
        er.ccd_iter(mode=ccx.MODE_STANDARD, precision=ccx.PREC_MIXED, rebase=7)


def test_mixed_ring_channels_wider_than_256(ccx):
    """A twisted SNM lattice whose ring channels hold more than 256 hole-particle pairs:
    the tensor-core products run as 256-column blocks.  Two iterations from MP2 (a mixed
    one, then a digit-product re-base) stay with the FP64 iteration to the BF16x3 level."""
    th = (-1.068, -1.068, -1.068)
    L = ccx.Layout.from_basis(3, 132, 0.16, snm=True, theta=th)
    nhp = max(L.channel(ccx.CH_PH_PHHP, q)[2] for q in range(L.counts()["ph_phhp"]))
    assert nhp > 256
    out = []
    for prec in (ccx.PREC_FP64, ccx.PREC_MIXED):
        e = ccx.Engine(L, real=True)
        e.generate()
        e.setup_t_amplitudes()
        out.append(e.ccd_iter(mode=ccx.MODE_STANDARD, precision=prec, rebase=ccx.REBASE_DIGITS, max_iter=2,
                              defect_period=1, tol=1e-10))
        del e
    r64, rm = out
    assert rm["mixed_iterations"] == 1 and rm["fp64_sweeps"] == 1
    assert abs(rm["e_ccd"] - r64["e_ccd"]) < 1e-4 * abs(r64["e_ccd"])
    assert abs(rm["res_norm"] - r64["res_norm"]) < 1e-3 * r64["res_norm"]


def test_tensor_core_launch_form_autotune(ccx):
    """The autotuner times each correction product's two launch forms and keeps the
    faster; the mixed solve after it reaches the same energy."""
    L = ccx.Layout.from_basis(2, 28, 0.16, snm=True)
    e = ccx.Engine(L, real=False)
    e.generate(potential=ccx.POT_CHIRAL_LIKE)
    e.setup_t_amplitudes()
    r0 = e.ccd_iter(mode=ccx.MODE_STANDARD, precision=ccx.PREC_MIXED, rebase=ccx.REBASE_DIGITS, tol=1e-10,
                    max_iter=200)
    merged, ms = e.autotune_tc(ccx.PREC_MIXED)
    assert all(m in (0, 1) for m in merged) and len(merged) == 3
    assert all(t[0] > 0 and t[1] > 0 and (t[1] <= t[0]) == bool(m) for t, m in zip(ms, merged))
    e.setup_t_amplitudes()
    r1 = e.ccd_iter(mode=ccx.MODE_STANDARD, precision=ccx.PREC_MIXED, rebase=ccx.REBASE_DIGITS, tol=1e-10,
                    max_iter=200)
    assert r0["converged"] and r1["converged"]
    assert abs(r1["e_ccd"] - r0["e_ccd"]) < 1e-12 * abs(r0["e_ccd"])
