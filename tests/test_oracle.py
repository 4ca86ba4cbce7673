"""The CPU oracle against independent checks (no GPU).

The reference ships no golden vectors and cannot be built here, so the oracle's
restatement of the Fortran solver is checked against a dense-tensor textbook CCD
and (T) written independently in numpy, against the MP2 closed form, antisymmetry,
thread-count invariance, and the regression fixtures under tests/golden.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _dense_t(o, A):
    n = o.n_states
    t = np.zeros((n - A, n - A, A, A), complex)
    for ch in range(o.n_channels(3)):
        hh = o.channel_pairs(3, 1, ch)
        pp = o.channel_pairs(3, 2, ch)
        t[pp[:, 0][:, None] - A, pp[:, 1][:, None] - A, hh[:, 0][None, :], hh[:, 1][None, :]] = o.t2(ch)
    return t


def _residual_vs_dense(O, cfg, tol):
    import dense_ccd as DC
    o = O.Oracle(cfg)
    orb = o.orbits()
    A = cfg.A
    d = DC.DenseCCD(orb, A, DC.minnesota_dense(orb, o.box_length ** 3))
    assert abs(o.e0() - d.e0) < 1e-10 * abs(d.e0)
    o.mp2()
    tm = d.mp2()
    assert abs(o.energy() - d.energy(tm)) < 1e-12 * abs(d.energy(tm))
    o.t2_intermediate()
    d1, d2 = o.denoms()
    rd = d.residual(tm)
    scale = np.abs(rd).max()
    for ch in range(o.n_channels(3)):
        hh = o.channel_pairs(3, 1, ch)
        pp = o.channel_pairs(3, 2, ch)
        D = (d1[hh[:, 0]][None, :] + d1[hh[:, 1]][None, :]) - d2[pp[:, 0] - A][:, None] - d2[pp[:, 1] - A][:, None]
        ro = o.r2(ch) - D * o.t2(ch)
        rdd = rd[pp[:, 0][:, None] - A, pp[:, 1][:, None] - A, hh[:, 0][None, :], hh[:, 1][None, :]]
        assert np.abs(ro - rdd).max() <= tol * scale
    return o, d


def test_oracle_residual_matches_dense_pnm2(O):
    o, d = _residual_vs_dense(O, O.Config(nmax=1, A=2, rho=0.08), 1e-12)
    t, it, rn = d.solve(tol=1e-11)
    o.mp2()
    r = o.ccd_iter(mode=O.MODE_STANDARD, tol=1e-11)
    assert r["converged"]
    assert abs(r["e_ccd"] - d.energy(t)) < 1e-10 * abs(d.energy(t))


def test_oracle_residual_matches_dense_pnm14(O):
    _residual_vs_dense(O, O.Config(nmax=1, A=14, rho=0.08), 1e-12)


def test_oracle_triples_matches_dense(O):
    import dense_ccd as DC
    cfg = O.Config(nmax=1, A=14, rho=0.08)
    o = O.Oracle(cfg)
    orb = o.orbits()
    d = DC.DenseCCD(orb, cfg.A, DC.minnesota_dense(orb, o.box_length ** 3))
    o.mp2()
    o.ccd_iter(mode=O.MODE_STANDARD, tol=1e-11)
    et_dense = DC.triples_dense(d, _dense_t(o, cfg.A))
    et = o.triples()
    assert abs(et - et_dense) < 1e-10 * abs(et_dense)


def test_mp2_closed_form_and_antisymmetry(O):
    o = O.Oracle(O.Config(nmax=2, A=14, rho=0.08))
    o.mp2()
    f = o.fock()
    for ch in range(o.n_channels(3)):
        hh = o.channel_pairs(3, 1, ch)
        pp = o.channel_pairs(3, 2, ch)
        fd = np.real(np.diag(f))
        D = fd[hh[:, 0]][None, :] + fd[hh[:, 1]][None, :] - fd[pp[:, 0]][:, None] - fd[pp[:, 1]][:, None]
        V = o.v_hhpp(ch)
        assert np.allclose(o.t2(ch), np.conj(V.T) / D, rtol=1e-13, atol=0)
    # a few reference iterations keep T antisymmetric in (ab) and (ij)
    o.diis_setup()
    cnt = 0
    for _ in range(3):
        o.t2_intermediate()
        cnt = o.diis_t1t2(cnt + 1)
    for ch in range(o.n_channels(3)):
        hh = [tuple(p) for p in o.channel_pairs(3, 1, ch)]
        pp = [tuple(p) for p in o.channel_pairs(3, 2, ch)]
        hidx = {p: i for i, p in enumerate(hh)}
        pidx = {p: i for i, p in enumerate(pp)}
        t = o.t2(ch)
        for (a, b), r in pidx.items():
            assert abs(t[r, :] + t[pidx[(b, a)], :]).max() <= 1e-13 * max(1.0, abs(t).max())
        for (i, j), c in hidx.items():
            assert abs(t[:, c] + t[:, hidx[(j, i)]]).max() <= 1e-13 * max(1.0, abs(t).max())


def test_thread_count_invariance(O):
    # the PNM 14 reference solve and (T), and every residual block of a complex SNM 28
    # chiral-like lattice (MP2 amplitudes) hashed bit for bit
    code = ("import sys, hashlib; sys.path.insert(0, %r); import oracle as O; import numpy as np; "
            "o = O.Oracle(O.Config(nmax=2, A=14, rho=0.08)); "
            "o.mp2(); r = o.ccd_iter(mode=O.MODE_REFERENCE); print(repr(r['e_ccd'].real), o.triples().real); "
            "s = O.Oracle(O.Config(nmax=2, A=28, rho=0.16, snm=True, potential=O.POT_CHIRAL_LIKE)); "
            "s.mp2(); s.t2_intermediate(); "
            "print(hashlib.sha1(b''.join(np.ascontiguousarray(s.r2(c)).tobytes() "
            "for c in range(s.n_channels(3)))).hexdigest())"
            % os.path.join(os.path.dirname(HERE), "oracle"))
    outs = []
    for nt in ("1", "4"):
        env = dict(os.environ, OMP_NUM_THREADS=nt)
        outs.append(subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                                   check=True).stdout.split())
    assert outs[0][0] == outs[1][0]  # each output element takes its terms in a fixed order
    assert abs(float(outs[0][1]) - float(outs[1][1])) <= 1e-14 * abs(float(outs[0][1]))
    assert outs[0][2] == outs[1][2]


def test_golden_fixtures(O):
    path = os.path.join(HERE, "golden", "oracle_golden.json")
    with open(path) as f:
        gold = json.load(f)
    for case in gold["cases"]:
        c = case["config"]
        cfg = O.Config(nmax=c["nmax"], A=c["A"], snm=c["snm"], rho=c["rho"], theta=tuple(c["theta"]),
                       potential=c["potential"], lec_seed=c["lec_seed"])
        o = O.Oracle(cfg)
        orb = o.orbits()
        assert orb["nx"].tolist()[:len(case["nx_head"])] == case["nx_head"]
        assert [o.n_channels(k) for k in (1, 2, 3, 4)] == case["n_channels"]
        assert o.n_amps == case["n_amps"]
        assert abs(o.e0().real - case["e0"]) <= 1e-12 * abs(case["e0"])
        o.mp2()
        assert abs(o.energy().real - case["e_mp2"]) <= 1e-12 * abs(case["e_mp2"])
        if "e_ccd_reference" in case:
            r = o.ccd_iter(mode=O.MODE_REFERENCE)
            assert r["iterations"] == case["iterations_reference"]
            assert abs(r["e_ccd"].real - case["e_ccd_reference"]) <= 1e-11 * abs(case["e_ccd_reference"])


def test_triples_samples_add_up(O):
    """The strided (T) samples the CPU baseline times (every third (abc) triple of every
    channel): three interleaved samples hold every (abc, ijk) pair once and add up to the
    whole E(T)."""
    o = O.Oracle(O.Config(nmax=2, A=14, rho=0.08))
    o.mp2()
    o.ccd_iter(mode=O.MODE_REFERENCE)
    full = o.triples()
    parts = [o.triples_sample(k, 3) for k in range(3)]
    assert sum(p for _, p in parts) == o.triples_count()
    assert o.triples_channels() >= 3 and all(p > 0 for _, p in parts)
    assert abs(sum(e for e, _ in parts) - full) <= 1e-12 * abs(full)
