"""T2 checkpoint files (host only, no GPU): a round trip is bit-exact, and a file of
another lattice, another twist, a corrupted or truncated file, or a missing one is
refused without touching the caller's buffer."""
import os

import numpy as np
import pytest

PNM14_NMAX1 = dict(nmax=1, A=14, density=0.08)


def amps(ccx, L, seed=7):
    n = L.counts()["amps"]
    r = np.random.default_rng(seed)
    return r.standard_normal(n) + 1j * r.standard_normal(n)


def test_round_trip_is_bit_exact(ccx, tmp_path):
    L = ccx.Layout.from_basis(**PNM14_NMAX1)
    t = amps(ccx, L)
    p = str(tmp_path / "t2.ckpt")
    L.write_t2_checkpoint(p, t)
    assert not os.path.exists(p + ".part")
    assert os.path.getsize(p) == 96 + 16 * t.size
    back = L.read_t2_checkpoint(p)
    assert np.array_equal(back.view(np.float64), t.view(np.float64))
    # a second layout object of the same lattice reads it too
    assert np.array_equal(ccx.Layout.from_basis(**PNM14_NMAX1).read_t2_checkpoint(p), t)


def test_other_lattice_is_refused(ccx, tmp_path):
    L = ccx.Layout.from_basis(**PNM14_NMAX1)
    p = str(tmp_path / "t2.ckpt")
    L.write_t2_checkpoint(p, amps(ccx, L))
    other = ccx.Layout.from_basis(nmax=2, A=14, density=0.08)
    with pytest.raises(ccx.CcxError) as ex:
        other.read_t2_checkpoint(p)
    assert ex.value.code == 1 and "another lattice" in str(ex.value)


def test_other_momenta_need_the_flag(ccx, tmp_path):
    # another density: the same orbitals and channel tables, other momenta and box
    L0 = ccx.Layout.from_basis(**PNM14_NMAX1)
    L1 = ccx.Layout.from_basis(nmax=1, A=14, density=0.16)
    assert L0.hash() == L1.hash()
    t = amps(ccx, L0)
    p = str(tmp_path / "t2.ckpt")
    L0.write_t2_checkpoint(p, t)
    with pytest.raises(ccx.CcxError) as ex:
        L1.read_t2_checkpoint(p)
    assert "twist" in str(ex.value)
    assert np.array_equal(L1.read_t2_checkpoint(p, any_twist=True), t)


def test_corrupted_truncated_and_missing_files(ccx, tmp_path):
    L = ccx.Layout.from_basis(**PNM14_NMAX1)
    t = amps(ccx, L)
    p = str(tmp_path / "t2.ckpt")
    L.write_t2_checkpoint(p, t)
    raw = bytearray(open(p, "rb").read())
    cases = {}
    flip = bytearray(raw)
    flip[96 + 8 * 5] ^= 0x10  # one bit of one amplitude
    cases["checksum"] = bytes(flip)
    cases["truncated"] = bytes(raw[:-8])
    cases["trailing"] = bytes(raw) + b"\0"
    cases["not a T2 checkpoint"] = b"XXXXXXXX" + bytes(raw[8:])
    ver = bytearray(raw)
    ver[8] = 9
    cases["version"] = bytes(ver)
    cases["truncated (header)"] = bytes(raw[:40])
    for what, blob in cases.items():
        q = str(tmp_path / "bad.ckpt")
        with open(q, "wb") as f:
            f.write(blob)
        with pytest.raises(ccx.CcxError) as ex:
            L.read_t2_checkpoint(q)
        assert ex.value.code == 1, what
        assert what.split(" (")[0] in str(ex.value), (what, str(ex.value))
    with pytest.raises(ccx.CcxError) as ex:
        L.read_t2_checkpoint(str(tmp_path / "missing.ckpt"))
    assert "cannot open" in str(ex.value)


def test_failed_read_leaves_the_buffer_untouched(ccx, tmp_path):
    import ctypes as C
    L = ccx.Layout.from_basis(**PNM14_NMAX1)
    p = str(tmp_path / "t2.ckpt")
    L.write_t2_checkpoint(p, amps(ccx, L))
    with open(p, "r+b") as f:  # corrupt the last amplitude
        f.seek(-1, os.SEEK_END)
        b = f.read(1)
        f.seek(-1, os.SEEK_END)
        f.write(bytes([b[0] ^ 1]))
    buf = np.full(2 * L.counts()["amps"], 3.5)
    rc = ccx.lib().ccx_t2_checkpoint_read(L._h, os.fsencode(p), 0, buf.ctypes.data_as(C.c_void_p))
    assert rc == 1 and np.all(buf == 3.5)
    rc = ccx.lib().ccx_t2_checkpoint_read(L._h, os.fsencode(p), 2, buf.ctypes.data_as(C.c_void_p))
    assert rc == 1 and "flags" in ccx.lib().ccx_last_error().decode()
