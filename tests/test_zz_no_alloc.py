"""ccx_ccd_energy_noalloc: the correlation energy on caller-owned device buffers.

Some callers cannot allocate device memory (a host that owns every device buffer
through its own pool, or code where an allocation is not allowed); this entry point
works on their buffers with a static scratch array instead.  Its result must match
ccx_ccd_energy on the same amplitudes, for two calls in a row (the second call reuses
the scratch the first one left behind).  The test itself allocates the caller's
buffers with torch; the entry point allocates nothing."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_inputs(ccx, torch, L, e):
    dims = L.hhpp_dims()
    nch = len(dims)
    t2 = e.t2_all()
    v = np.concatenate([e.vblock(ccx.CH_HHPP, c).reshape(-1, order="F") for c in range(nch)])
    d = torch.tensor(np.array(dims, np.int32).reshape(-1), device="cuda")
    t = torch.tensor(np.ascontiguousarray(t2).view(np.float64), device="cuda")
    w = torch.tensor(np.ascontiguousarray(v).view(np.float64), device="cuda")
    return nch, d, t, w


def _two_calls(ccx, torch, L, e):
    """Two calls in a row on different amplitudes, each against ccx_ccd_energy; the
    caller's device memory (torch's allocator and the device's free bytes) must be
    the same before and after each call."""
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    results = []
    for step in range(2):
        if step == 1:  # different amplitudes for the second call
            e.diis_setup(6, 6)
            cnt = 0
            for _ in range(3):
                e.t2_intermediate()
                cnt = e.diis_t1t2(cnt + 1)
        ref = e.ccd_energy()
        nch, d, t, w = _device_inputs(ccx, torch, L, e)
        torch.cuda.synchronize()
        before = (torch.cuda.memory_allocated(), torch.cuda.mem_get_info()[0])
        ccx.ccd_energy_noalloc(nch, d.data_ptr(), t.data_ptr(), w.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        after = (torch.cuda.memory_allocated(), torch.cuda.mem_get_info()[0])
        assert before == after, (step, before, after)
        got = complex(out[0].item(), out[1].item())
        assert abs(got.real - ref.real) < 1e-12 * abs(ref), (step, got, ref)
        assert abs(got.imag - ref.imag) < 1e-12 * abs(ref), (step, got, ref)
        results.append(got)
    assert results[0] != results[1]
    return results


def test_noalloc_energy_matches_ccd_energy(ccx):
    torch = pytest.importorskip("torch")
    L = ccx.Layout.from_basis(2, 14, 0.08)
    e = ccx.Engine(L, real=True)
    e.generate()
    e.setup_t_amplitudes()
    _two_calls(ccx, torch, L, e)


def test_noalloc_energy_matches_complex_engine(ccx):
    """A complex engine (twisted SNM with the chiral-like interaction, whose V is
    complex): the imaginary parts and the complex cross terms of the product are
    checked against ccx_ccd_energy as well."""
    torch = pytest.importorskip("torch")
    L = ccx.Layout.from_basis(1, 4, 0.16, snm=True, theta=(0.3, -0.7, 1.1))
    e = ccx.Engine(L, real=False)
    e.generate(potential=ccx.POT_CHIRAL_LIKE)
    e.setup_t_amplitudes()
    v = np.concatenate([e.vblock(ccx.CH_HHPP, c).ravel() for c in range(len(L.hhpp_dims()))])
    assert np.abs(v.imag).max() > 1e-6 * np.abs(v).max()
    # a global phase on T makes the energy itself complex
    e.set_t2_all(e.t2_all() * np.exp(0.4j))
    res = _two_calls(ccx, torch, L, e)
    assert abs(res[0].imag) > 0.1 * abs(res[0]), res


def test_noalloc_rejects_too_many_channels(ccx):
    torch = pytest.importorskip("torch")
    buf = torch.zeros(4, dtype=torch.float64, device="cuda")
    with pytest.raises(ccx.CcxError) as ex:
        ccx.ccd_energy_noalloc(16385, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), buf.data_ptr())
    assert ex.value.code == 1 and "16384" in str(ex.value)
