"""GPU engine against the CPU oracle, through the C ABI (libccx.so).

Tolerances: FP64 path vs FP64 oracle.  The engine sums in a different order (packed
a<b, i<j blocks, tiled GEMMs), so element-wise agreement is to ~1e-12 relative to the
block's scale and energies to ~1e-10 relative.  The one exception is the reference's
own DIIS step (see test_reference_iteration_step_by_step).  The accuracy bar (1e-6
relative in E/A, 1e-5 in E(T)) is far looser.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PNM14 = dict(nmax=2, A=14, rho=0.08, snm=False)


def make(ccx, O, nmax, A, rho, snm=False, pot=0, real=True, theta=(0.0, 0.0, 0.0)):
    o = O.Oracle(O.Config(nmax=nmax, A=A, rho=rho, snm=snm, theta=theta, potential=pot))
    L = ccx.Layout.from_basis(nmax, A, rho, snm=snm, theta=theta)
    e = ccx.Engine(L, real=real)
    e.generate(potential=pot)
    return o, L, e


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def check_blocks(o, e, get_o, get_e, tol):
    worst = 0.0
    scale = max(np.abs(get_o(c)).max() for c in range(o.n_channels(3)))
    for c in range(o.n_channels(3)):
        d = np.abs(get_e(c) - get_o(c)).max() / scale
        worst = max(worst, d)
    assert worst < tol, worst
    return worst


def test_e0_and_mp2(ccx, O):
    o, L, e = make(ccx, O, **PNM14)
    assert abs(e.e0() - o.e0()) < 1e-12 * abs(o.e0())
    o.mp2()
    e.setup_t_amplitudes()
    check_blocks(o, e, o.t2, e.t2, 1e-13)
    assert abs(e.ccd_energy() - o.energy()) < 1e-12 * abs(o.energy())


def test_residual_matches_oracle_at_mp2(ccx, O):
    o, L, e = make(ccx, O, **PNM14)
    o.mp2()
    e.setup_t_amplitudes()
    o.t2_intermediate()
    e.t2_intermediate()
    check_blocks(o, e, o.r2, e.t2_eqn, 1e-12)
    d1o, d2o = o.denoms()
    d1e, d2e = e.denominators()
    assert rel(d1e, d1o) < 1e-13 and rel(d2e, d2o) < 1e-13
    assert abs(e.residual_norm() - o.residual_norm()) < 1e-10 * o.residual_norm()


def test_residual_matches_oracle_at_iterated_t(ccx, O):
    """Residual of a non-MP2 amplitude: the oracle's T after 4 reference steps."""
    o, L, e = make(ccx, O, **PNM14)
    o.mp2()
    o.diis_setup()
    cnt = 0
    for _ in range(4):
        o.t2_intermediate()
        cnt = o.diis_t1t2(cnt + 1)
    e.setup_t_amplitudes()
    for c in range(o.n_channels(3)):
        e.set_t2(c, o.t2(c))
    check_blocks(o, e, o.t2, e.t2, 1e-15)
    o.t2_intermediate()
    e.t2_intermediate()
    check_blocks(o, e, o.r2, e.t2_eqn, 1e-12)


def test_reference_iteration_step_by_step(ccx, O):
    """t2_intermediate / diis_t1t2 / ccd_energy called one by one, as ccd_iter does.

    The damped updates agree to rounding.  The reference's DIIS step (every 6th call)
    solves a bordered system of unconjugated dot products of consecutive differences
    (ccm_diis.f90:134-173) whose condition number is ~1e15 here, so a different
    summation order alone moves the extrapolated energy by ~1e-7 relative; after the
    first DIIS step the trajectories are compared at the accuracy bar (1e-6)."""
    o, L, e = make(ccx, O, **PNM14)
    o.mp2()
    e.setup_t_amplitudes()
    o.diis_setup(6, 6)
    e.diis_setup(6, 6)
    co = ce = 0
    for it in range(14):
        o.t2_intermediate()
        e.t2_intermediate()
        co = o.diis_t1t2(co + 1)
        ce = e.diis_t1t2(ce + 1)
        assert co == ce
        eo, ee = o.energy(), e.ccd_energy()
        tol = 1e-11 if it < 5 else 1e-6
        assert abs(ee - eo) < tol * abs(eo), (it, ee, eo)


def test_ccd_iter_reference_mode(ccx, O):
    o, L, e = make(ccx, O, **PNM14)
    o.mp2()
    e.setup_t_amplitudes()
    ro = o.ccd_iter(mode=O.MODE_REFERENCE)
    re_ = e.ccd_iter(mode=ccx.MODE_REFERENCE)
    assert re_["converged"] and abs(re_["iterations"] - ro["iterations"]) <= 2
    # both stop at |dE| < 1e-6 MeV (ccm_iter.f90:74)
    assert abs(re_["e_ccd"] - ro["e_ccd"]) < 5e-7 * abs(ro["e_ccd"])
    assert abs(re_["e_mbpt2"] - ro["e_mbpt2"]) < 1e-12 * abs(ro["e_mbpt2"])


def test_ccd_iter_standard_mode_converges_to_1e10(ccx, O):
    o, L, e = make(ccx, O, **PNM14)
    o.mp2()
    e.setup_t_amplitudes()
    ro = o.ccd_iter(mode=O.MODE_STANDARD, tol=1e-10)
    re_ = e.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10)
    assert re_["converged"] and re_["res_norm"] < 1e-10
    assert abs(re_["e_ccd"] - ro["e_ccd"]) < 1e-11 * abs(ro["e_ccd"])
    # E/A within 1e-6 relative of the oracle (the accuracy bar), here ~1e-12
    ea_o = (o.e0() + ro["e_ccd"]).real / 14
    ea_e = (e.e0() + re_["e_ccd"]).real / 14
    assert abs(ea_e - ea_o) < 1e-6 * abs(ea_o)


def test_complex_engine_matches_real_engine(ccx, O):
    _, L, er = make(ccx, O, **PNM14)
    ec = ccx.Engine(L, real=False)
    ec.generate()
    er.setup_t_amplitudes()
    ec.setup_t_amplitudes()
    rr = er.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10)
    rc = ec.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10)
    assert rr["iterations"] == rc["iterations"]
    assert abs(rr["e_ccd"] - rc["e_ccd"]) < 1e-12 * abs(rr["e_ccd"])


@pytest.mark.parametrize("cfg", [dict(nmax=1, A=4, rho=0.16, snm=True), dict(nmax=2, A=28, rho=0.16, snm=True)],
                         ids=["snm4", "snm28"])
def test_chiral_like_snm_complex(ccx, O, cfg):
    o, L, e = make(ccx, O, pot=1, real=False, **cfg)
    assert abs(e.e0() - o.e0()) < 1e-11 * abs(o.e0())
    o.mp2()
    e.setup_t_amplitudes()
    o.t2_intermediate()
    e.t2_intermediate()
    check_blocks(o, e, o.r2, e.t2_eqn, 1e-11)
    ro = o.ccd_iter(mode=O.MODE_STANDARD, tol=1e-9, max_iter=80)
    o.mp2()
    re_ = e.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-9, max_iter=80)
    assert ro["converged"] and re_["converged"]
    assert abs(re_["e_ccd"] - ro["e_ccd"]) < 1e-9 * abs(ro["e_ccd"])


def test_real_engine_rejects_complex_potential(ccx):
    L = ccx.Layout.from_basis(1, 4, 0.16, snm=True)
    e = ccx.Engine(L, real=True)
    with pytest.raises(ccx.CcxError) as ex:
        e.generate(potential=ccx.POT_CHIRAL_LIKE)
    assert ex.value.code == 1


def test_iterate_before_amplitudes_is_a_state_error(ccx):
    L = ccx.Layout.from_basis(1, 2, 0.08)
    e = ccx.Engine(L, real=True)
    with pytest.raises(ccx.CcxError) as ex:
        e.ccd_iter()
    assert ex.value.code == 4
    e.generate()
    with pytest.raises(ccx.CcxError) as ex:
        e.t2_intermediate()
    assert ex.value.code == 4


def test_triples_matches_oracle(ccx, O):
    o, L, e = make(ccx, O, **PNM14)
    o.mp2()
    e.setup_t_amplitudes()
    o.ccd_iter(mode=O.MODE_STANDARD, tol=1e-10)
    e.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10)
    eo = o.triples()
    ee = e.pert_triples()  # FP32 contractions (the default), FP64 |W|^2 / D sum
    assert abs(ee - eo) < 1e-5 * abs(eo), (ee, eo)
    e.set_triples_precision(fp32=False)
    ee64 = e.pert_triples()
    assert abs(ee64 - eo) < 1e-10 * abs(eo), (ee64, eo)


def test_triples_chiral_like_snm(ccx, O):
    o, L, e = make(ccx, O, nmax=1, A=4, rho=0.16, snm=True, pot=1, real=False)
    o.mp2()
    e.setup_t_amplitudes()
    o.ccd_iter(mode=O.MODE_STANDARD, tol=1e-10)
    e.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10)
    eo, ee = o.triples(), e.pert_triples()
    assert abs(ee - eo) < 1e-5 * abs(eo), (ee, eo)
    e.set_triples_precision(fp32=False)
    ee64 = e.pert_triples()
    assert abs(ee64 - eo) < 1e-9 * abs(eo), (ee64, eo)


def test_caller_supplied_blocks_match_generated(ccx, O):
    """The drop-in path: the Fortran host hands over fock_mtx and the vnn_* blocks."""
    o, L, eg = make(ccx, O, **PNM14)
    e = ccx.Engine(L, real=True)
    e.set_fock(o.fock(), o.e0())
    for c in range(o.n_channels(3)):
        e.set_vblock(ccx.CH_HHPP, c, o.v_hhpp(c))
        e.set_vblock(ccx.V_PPPP, c, o.v_pppp(c))
    for c in range(o.n_channels(1)):
        e.set_vblock(ccx.CH_HHHH, c, o.v_hhhh(c))
    for c in range(o.n_channels(4)):
        e.set_vblock(ccx.CH_HPHP, c, o.v_hphp(c))
    assert abs(e.e0() - o.e0()) == 0.0
    e.setup_t_amplitudes()
    eg.setup_t_amplitudes()
    e.t2_intermediate()
    eg.t2_intermediate()
    for c in range(o.n_channels(3)):
        assert rel(e.t2_eqn(c), eg.t2_eqn(c)) < 1e-12
    e.setup_t_amplitudes()
    eg.setup_t_amplitudes()
    r1 = e.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10)
    r2 = eg.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10)
    o.mp2()
    ro = o.ccd_iter(mode=O.MODE_STANDARD, tol=1e-10)
    assert r1["converged"] and r2["converged"]
    assert abs(r1["e_ccd"] - ro["e_ccd"]) < 1e-11 * abs(ro["e_ccd"])
    assert abs(r1["e_ccd"] - r2["e_ccd"]) < 1e-11 * abs(ro["e_ccd"])


def test_set_vblocks_matches_single_blocks(ccx, O):
    """ccx_set_vblocks (one call per block family) gives the same engine as one call per block."""
    o, L, eg = make(ccx, O, **PNM14)
    e1 = ccx.Engine(L, real=True)
    e2 = ccx.Engine(L, real=True)
    for e in (e1, e2):
        e.set_fock(o.fock(), o.e0())
    for c in range(o.n_channels(3)):
        e1.set_vblock(ccx.CH_HHPP, c, o.v_hhpp(c))
        e1.set_vblock(ccx.V_PPPP, c, o.v_pppp(c))
    for c in range(o.n_channels(1)):
        e1.set_vblock(ccx.CH_HHHH, c, o.v_hhhh(c))
    for c in range(o.n_channels(4)):
        e1.set_vblock(ccx.CH_HPHP, c, o.v_hphp(c))
    e2.set_vblocks(ccx.CH_HHPP, {c: o.v_hhpp(c) for c in range(o.n_channels(3))})
    e2.set_vblocks(ccx.V_PPPP, {c: o.v_pppp(c) for c in range(o.n_channels(3))})
    e2.set_vblocks(ccx.CH_HHHH, {c: o.v_hhhh(c) for c in range(o.n_channels(1))})
    e2.set_vblocks(ccx.CH_HPHP, {c: o.v_hphp(c) for c in range(o.n_channels(4))})
    for e in (e1, e2):
        e.setup_t_amplitudes()
        e.t2_intermediate()
    for c in range(o.n_channels(3)):
        assert np.array_equal(e1.t2_eqn(c), e2.t2_eqn(c))
    with pytest.raises(ccx.CcxError) as ex:
        e2.set_vblocks(ccx.CH_HHPP, {0: o.v_hhpp(0), 1: o.v_hhpp(1) + 1e-3j})
    assert ex.value.code == 1


def test_pinned_host_blocks_are_read_in_place(ccx, O):
    """V blocks and the T2 output in pinned (device-addressable) host memory take the
    in-place path: packing kernels read the host blocks directly and the amplitudes are
    unpacked straight into the host buffer.  The engine must equal one fed from pageable
    memory through staging copies, bit for bit."""
    torch = pytest.importorskip("torch")
    import ctypes as C
    o, L, eg = make(ccx, O, **PNM14)
    e1 = ccx.Engine(L, real=True)
    e2 = ccx.Engine(L, real=True)
    for e in (e1, e2):
        e.set_fock(o.fock(), o.e0())
    fams = {ccx.CH_HHPP: {c: o.v_hhpp(c) for c in range(o.n_channels(3))},
            ccx.V_PPPP: {c: o.v_pppp(c) for c in range(o.n_channels(3))},
            ccx.CH_HHHH: {c: o.v_hhhh(c) for c in range(o.n_channels(1))},
            ccx.CH_HPHP: {c: o.v_hphp(c) for c in range(o.n_channels(4))}}
    keep = []

    def pinned_call(e, kind, blocks):
        bufs = []
        for b in blocks.values():
            f = ccx._cplx_fortran(b)
            t = torch.empty(f.size, dtype=torch.float64, pin_memory=True)
            t.numpy()[:] = f
            bufs.append(t)
        keep.extend(bufs)
        chs = (C.c_int32 * len(bufs))(*blocks.keys())
        ptrs = (C.c_void_p * len(bufs))(*[t.data_ptr() for t in bufs])
        return ccx.lib().ccx_set_vblocks(e._h, kind, len(bufs), chs, ptrs)

    for kind, blocks in fams.items():
        e1.set_vblocks(kind, blocks)
        assert pinned_call(e2, kind, blocks) == 0
    for e in (e1, e2):
        e.setup_t_amplitudes()
        e.t2_intermediate()
    for c in range(o.n_channels(3)):
        assert np.array_equal(e1.t2_eqn(c), e2.t2_eqn(c))
    r1 = e1.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10)
    r2 = e2.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10)
    assert r1["e_ccd"] == r2["e_ccd"]
    n = L.counts()["amps"]
    out = torch.zeros(2 * n, dtype=torch.float64, pin_memory=True)
    ccx._check(ccx.lib().ccx_get_t2_all(e2._h, C.c_void_p(out.data_ptr())))
    assert np.array_equal(out.numpy().view(np.complex128), e1.t2_all())
    # a non-zero imaginary part in pinned memory is rejected like a pageable one
    bad = {0: o.v_hhpp(0), 1: o.v_hhpp(1) + 1e-3j}
    assert pinned_call(e2, ccx.CH_HHPP, bad) == 1


def test_complex_block_into_real_engine_is_rejected(ccx, O):
    o = O.Oracle(O.Config(nmax=1, A=2, rho=0.08))
    L = ccx.Layout.from_basis(1, 2, 0.08)
    e = ccx.Engine(L, real=True)
    v = o.v_hhpp(0) + 1e-3j
    with pytest.raises(ccx.CcxError) as ex:
        e.set_vblock(ccx.CH_HHPP, 0, v)
    assert ex.value.code == 1


def test_twisted_lattice(ccx, O):
    o, L, e = make(ccx, O, nmax=1, A=14, rho=0.10, theta=(0.3, -1.1, 2.0))
    o.mp2()
    e.setup_t_amplitudes()
    ro = o.ccd_iter(mode=O.MODE_STANDARD, tol=1e-10)
    re_ = e.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10)
    assert abs(re_["e_ccd"] - ro["e_ccd"]) < 1e-10 * abs(ro["e_ccd"])


def test_autotune_keeps_results(ccx, O):
    """The GEMM tile-shape autotuner only changes how the products are tiled."""
    o, L, e = make(ccx, O, **PNM14)
    e.setup_t_amplitudes()
    r0 = e.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10)
    shapes, ms = e.autotune()
    assert len(shapes) == 4 and all(s in (0, 1) for s in shapes)
    assert all(t >= 0 for row in ms for t in row)
    e.setup_t_amplitudes()
    r1 = e.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10)
    assert r1["converged"] and abs(r1["e_ccd"] - r0["e_ccd"]) < 1e-12 * abs(r0["e_ccd"])


@pytest.mark.parametrize("prec,rebase", [(0, 0), (1, 0), (1, 1)], ids=["fp64", "mixed-fp64-rebase", "mixed-digits"])
def test_profiling_switch_keeps_results(ccx, O, prec, rebase):
    """Per-term event timers only observe: the solve is the same with them on (launches
    issued one by one) or off (each residual kind replayed as a captured CUDA graph)."""
    o, L, e = make(ccx, O, **PNM14)
    kw = dict(mode=ccx.MODE_STANDARD, tol=1e-10, precision=prec, rebase=rebase)
    for _ in range(2):  # the second solve replays the graphs captured by the first
        e.setup_t_amplitudes()
        r0 = e.ccd_iter(**kw)
    t0, k0 = e.timers(), e.kernel_timers()
    assert t0["total"] > 0 and all(v == 0.0 for k, v in t0.items() if k != "total")
    assert all(n == 0 for _, n in k0.values())
    e.set_profiling(True)
    e.setup_t_amplitudes()
    r1 = e.ccd_iter(**kw)
    t1, k1 = e.timers(), e.kernel_timers()
    e.set_profiling(False)
    assert t1["update"] > 0 and t1["ladders"] > 0 and sum(n for _, n in k1.values()) > 0
    assert r0["converged"] and r1["iterations"] == r0["iterations"]
    assert abs(r1["e_ccd"] - r0["e_ccd"]) <= 1e-13 * abs(r0["e_ccd"])


def test_replayed_residuals_follow_plan_and_interaction_changes(ccx, O):
    """The residual kinds replay captured CUDA graphs.  A tile-shape autotune (new FP64
    plans) and new V blocks between mixed solves must give what a fresh engine gives."""
    o, L, e = make(ccx, O, **PNM14)
    kw = dict(mode=ccx.MODE_STANDARD, tol=1e-10, precision=ccx.PREC_MIXED, rebase=ccx.REBASE_DIGITS)
    e.setup_t_amplitudes()
    r0 = e.ccd_iter(**kw)
    e.autotune()
    e.setup_t_amplitudes()
    r1 = e.ccd_iter(**kw)
    assert r0["converged"] and r1["iterations"] == r0["iterations"]
    assert abs(r1["e_ccd"] - r0["e_ccd"]) < 1e-12 * abs(r0["e_ccd"])
    # a 10% weaker interaction, handed over to the engine that has replayed its graphs
    # and to a fresh one
    s = 0.9
    fresh = ccx.Engine(L, real=True)
    for eng in (e, fresh):
        eng.set_fock(o.fock(), o.e0())
        eng.set_vblocks(ccx.CH_HHPP, {c: s * o.v_hhpp(c) for c in range(o.n_channels(3))})
        eng.set_vblocks(ccx.V_PPPP, {c: s * o.v_pppp(c) for c in range(o.n_channels(3))})
        eng.set_vblocks(ccx.CH_HHHH, {c: s * o.v_hhhh(c) for c in range(o.n_channels(1))})
        eng.set_vblocks(ccx.CH_HPHP, {c: s * o.v_hphp(c) for c in range(o.n_channels(4))})
        eng.setup_t_amplitudes()
    r2 = e.ccd_iter(**kw)
    r3 = fresh.ccd_iter(**kw)
    assert r2["converged"] and r3["converged"]
    assert abs(r2["e_ccd"] - r0["e_ccd"]) > 1e-3 * abs(r0["e_ccd"])  # the new V is in use
    assert abs(r2["e_ccd"] - r3["e_ccd"]) < 1e-11 * abs(r3["e_ccd"])


def test_checkpoint_resumes_a_converged_solve(ccx, O, tmp_path):
    """Amplitudes saved after a converged solve and loaded into a fresh engine of the same
    lattice: the loaded engine is already converged (one FP64 sweep confirms it)."""
    o, L, e = make(ccx, O, **PNM14)
    e.setup_t_amplitudes()
    r0 = e.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10)
    p = str(tmp_path / "c1.t2")
    e.save_t2(p)
    f = ccx.Engine(L, real=True)
    f.generate()
    f.load_t2(p)
    assert np.array_equal(f.t2_all(), e.t2_all())
    r1 = f.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10)
    assert r1["converged"] and r1["iterations"] <= 1
    assert abs(r1["e_ccd"] - r0["e_ccd"]) < 1e-11 * abs(r0["e_ccd"])


@pytest.mark.parametrize("cfg", [dict(nmax=2, A=28, rho=0.16, snm=True, pot=1, real=False, theta=(0.7, -0.4, 1.9)),
                                 dict(nmax=2, A=14, rho=0.08, snm=False, pot=0, real=True, theta=(-0.9, 0.3, 2.2))],
                         ids=["snm28_chiral_twisted", "pnm14_minnesota_twisted"])
def test_generated_interaction_twisted_residual(ccx, O, cfg):
    """The device generator (V_pppp' written on and above the diagonal and mirrored: the
    interaction is Hermitian) against the oracle's interaction at a twist, through the
    residual at the MP2 amplitudes, block by block."""
    o, L, e = make(ccx, O, **cfg)
    try:
        tol = 1e-12 if cfg["real"] else 1e-11
        assert abs(e.e0() - o.e0()) < tol * abs(o.e0())
        o.mp2()
        e.setup_t_amplitudes()
        o.t2_intermediate()
        e.t2_intermediate()
        check_blocks(o, e, o.r2, e.t2_eqn, tol)
    finally:
        e.close()
        o.close()
