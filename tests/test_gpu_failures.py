"""Failure detection through the C ABI, none of which faults the GPU.

- a NaN in a V block handed over by the host is CCX_ENUMERIC, and the engine is usable
  again once the caller hands over a valid block;
- a singular DIIS system keeps the plain step (the reference prints ZGESV's info and
  goes on, ccm_diis.f90:173-180);
- a layout whose resident state does not fit the device is CCX_ENOMEM before the engine
  allocates anything;
- the tensor-core kernel's bounded pipeline waits: with a limit too short for any copy
  to land, the kernel gives up, reports which wait ran out, and the context stays usable.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PNM14 = (2, 14, 0.08)


def _solve(ccx, e, **kw):
    e.setup_t_amplitudes()
    return e.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10, **kw)


@pytest.mark.parametrize("kind", ["hhpp", "pppp"])
def test_nan_vblock_is_numeric_error_and_engine_recovers(ccx, kind):
    L = ccx.Layout.from_basis(*PNM14)
    ref = ccx.Engine(L, real=True)
    ref.generate()
    want = _solve(ccx, ref)["e_ccd"]
    e = ccx.Engine(L, real=True)
    e.generate()
    k = ccx.CH_HHPP if kind == "hhpp" else ccx.V_PPPP
    ch = 3
    good = e.vblock(k, ch)
    bad = good.copy()
    bad[1, 2] = np.nan
    with pytest.raises(ccx.CcxError) as ex:
        e.set_vblock(k, ch, bad)
    assert ex.value.code == 5 and "NaN" in str(ex.value)
    e.set_vblock(k, ch, good)  # the caller hands over a valid block
    got = _solve(ccx, e)["e_ccd"]
    assert abs(got - want) < 1e-12 * abs(want)


def test_nan_in_pinned_block_read_in_place(ccx):
    """The same check on the path that packs pinned host blocks in place."""
    torch = pytest.importorskip("torch")
    L = ccx.Layout.from_basis(*PNM14)
    e = ccx.Engine(L, real=False)
    e.generate()
    good = e.vblock(ccx.V_PPPP, 0)
    host = torch.empty(2 * good.size, dtype=torch.float64, pin_memory=True)
    arr = host.numpy().view(np.complex128).reshape(good.shape, order="F")
    arr[...] = good
    arr[0, 1] = complex(np.inf, 0.0)
    with pytest.raises(ccx.CcxError) as ex:
        e.set_vblocks(ccx.V_PPPP, {0: arr})
    assert ex.value.code == 5
    arr[0, 1] = good[0, 1]
    e.set_vblocks(ccx.V_PPPP, {0: arr})
    e.setup_t_amplitudes()
    assert np.isfinite(e.ccd_iter(mode=ccx.MODE_STANDARD, tol=1e-10)["e_ccd"])


def test_singular_diis_keeps_the_plain_step(ccx):
    """With every V block zero the amplitudes stay zero, the consecutive differences the
    reference DIIS builds its matrix from are all zero, and the system is singular: the
    engine keeps the damped step, counts the fallback and reports no error."""
    L = ccx.Layout.from_basis(*PNM14)
    e = ccx.Engine(L, real=True)
    e.generate()
    c = L.counts()
    for kind, fam, n in ((ccx.CH_HHPP, ccx.CH_HHPP, c["hhpp"]), (ccx.V_PPPP, ccx.CH_HHPP, c["hhpp"]),
                         (ccx.CH_HHHH, ccx.CH_HHHH, c["hhhh"]), (ccx.CH_HPHP, ccx.CH_HPHP, c["hphp"])):
        blocks = {}
        for ch in range(n):
            _, n1, n2 = L.channel(fam, ch)
            shape = {ccx.CH_HHPP: (n1, n2), ccx.V_PPPP: (n2, n2)}.get(kind, (n1, n1))
            blocks[ch] = np.zeros(shape, np.complex128)
        e.set_vblocks(kind, blocks)
    e.setup_t_amplitudes()
    e.diis_setup(6, 6)
    assert e.diis_fallbacks() == 0
    cnt = 0
    for _ in range(6):
        e.t2_intermediate()
        cnt = e.diis_t1t2(cnt + 1)
    assert e.diis_fallbacks() == 1
    assert np.abs(e.t2_all()).max() == 0.0
    assert e.ccd_energy() == 0.0


def test_oversized_layout_is_out_of_memory_before_allocation(ccx):
    """SNM 132 at nmax=7 (13500 states): V_pppp' alone is about 450 GB complex."""
    torch = pytest.importorskip("torch")
    torch.cuda.init()
    L = ccx.Layout.from_basis(7, 132, 0.16, snm=True)
    free0 = torch.cuda.mem_get_info()[0]
    with pytest.raises(ccx.CcxError) as ex:
        ccx.Engine(L, real=False)
    assert ex.value.code == 3 and "device memory" in str(ex.value)
    assert torch.cuda.mem_get_info()[0] == free0


def test_tensor_core_wait_limit_runs_out_and_context_stays_usable(ccx):
    err = ccx.selftest_tc_wait(1)
    assert err in (1, 2, 3), err
    assert ccx.selftest_tc_wait(4_000_000_000) == 0
    L = ccx.Layout.from_basis(*PNM14)
    e = ccx.Engine(L, real=True)
    e.generate()
    r = _solve(ccx, e, precision=ccx.PREC_MIXED)
    assert r["converged"]
