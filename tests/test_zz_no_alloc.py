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


def test_noalloc_energy_matches_ccd_energy(ccx):
    torch = pytest.importorskip("torch")
    L = ccx.Layout.from_basis(2, 14, 0.08)
    e = ccx.Engine(L, real=True)
    e.generate()
    e.setup_t_amplitudes()
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
        ccx.ccd_energy_noalloc(nch, d.data_ptr(), t.data_ptr(), w.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        got = complex(out[0].item(), out[1].item())
        assert abs(got - ref) < 1e-12 * abs(ref), (step, got, ref)
        results.append(got)
    assert results[0] != results[1]


def test_noalloc_rejects_too_many_channels(ccx):
    torch = pytest.importorskip("torch")
    buf = torch.zeros(4, dtype=torch.float64, device="cuda")
    with pytest.raises(ccx.CcxError) as ex:
        ccx.ccd_energy_noalloc(16385, buf.data_ptr(), buf.data_ptr(), buf.data_ptr(), buf.data_ptr())
    assert ex.value.code == 1 and "16384" in str(ex.value)
