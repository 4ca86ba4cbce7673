"""The structured run log: ccx_iter_record and the other ABI structs as the binding lays
them out (against the header, compiled with gcc), the per-iteration and final-result
records (the values of the (8f12.5) line ccm_main.f90:338-339 writes), and ccx_run's
--json flag.  The GPU tests check the engine's log against the solve it records."""
import ctypes as C
import json
import math
import os
import shutil
import subprocess

import pytest

from test_harness import RUN, fields, run

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r"""
#include <stddef.h>
#include <stdio.h>
#include "ccx.h"
#define F(T, m) printf(#T " " #m " %zu\n", offsetof(T, m))
int main(void) {
  printf("ccx_iter_record size %zu\n", sizeof(ccx_iter_record));
  F(ccx_iter_record, kind); F(ccx_iter_record, energy); F(ccx_iter_record, de);
  F(ccx_iter_record, res_norm); F(ccx_iter_record, ms); F(ccx_iter_record, term_ms);
  printf("ccx_iter_opts size %zu\n", sizeof(ccx_iter_opts));
  F(ccx_iter_opts, tol); F(ccx_iter_opts, rebase_drop);
  printf("ccx_iter_result size %zu\n", sizeof(ccx_iter_result));
  F(ccx_iter_result, e_mbpt2); F(ccx_iter_result, fp64_sweeps); F(ccx_iter_result, mixed_iterations);
  printf("ccx_deck size %zu\n", sizeof(ccx_deck));
  F(ccx_deck, cE); F(ccx_deck, lec_seed); F(ccx_deck, theta);
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_binding_structs_match_the_header(ccx, tmp_path):
    src = tmp_path / "probe.c"
    src.write_text(PROBE)
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        t, m, v = line.split()
        got[(t, m)] = int(v)
    py = {"ccx_iter_record": ccx._IterRecord, "ccx_iter_opts": ccx._IterOpts, "ccx_iter_result": ccx._IterResult,
          "ccx_deck": ccx._Deck}
    for (t, m), v in got.items():
        want = C.sizeof(py[t]) if m == "size" else getattr(py[t], m).offset
        assert want == v, (t, m, want, v)


def test_kfermi_inverts_the_deck_conversion(ccx):
    # ccm_main.f90:930-945: rho = kf^3 / (3 pi^2) (PNM), twice that for SNM
    for kf, snm in ((1.05, False), (1.33, True)):
        rho = (2.0 if snm else 1.0) * kf ** 3 / 3.0 / math.pi ** 2
        assert ccx.kfermi(rho, snm) == pytest.approx(kf, rel=1e-14)


def test_result_and_iteration_records(ccx):
    r = ccx.result_record(A=14, density=0.08, snm=False, e0=140.0, e_mbpt2=-7.0, e_ccd=-8.4, cE=0.5, cD=-0.25,
                          iterations=12)
    assert r["e0_per_a"] == pytest.approx(10.0) and r["mbpt2_per_a"] == pytest.approx(9.5)
    assert r["eccd_per_a"] == pytest.approx(9.4) and r["eccdt_per_a"] is None
    assert r["kf"] == pytest.approx((3 * math.pi ** 2 * 0.08) ** (1 / 3))
    assert (r["cE"], r["cD"], r["iterations"]) == (0.5, -0.25, 12)
    rt = ccx.result_record(A=14, density=0.08, snm=False, e0=140.0, e_mbpt2=-7.0, e_ccd=-8.4, e_triples=-1.4)
    assert rt["eccdt_per_a"] == pytest.approx(9.3)
    zero = dict.fromkeys(ccx.TERM_KEYS, 0.0)
    log = [{"iteration": 1, "kind": "fp64", "e_ccd": complex(-8.0, 0.0), "de": -1.0, "res_norm": 1e-2, "ms": 3.0,
            "term_ms": zero},
           {"iteration": 2, "kind": "mixed", "e_ccd": complex(-8.4, 1e-9), "de": -0.4, "res_norm": 1e-4, "ms": 1.0,
            "term_ms": dict(zero, ladders=0.5)}]
    lines = ccx.iteration_records(log, e0=140.0, A=14)
    assert [d["iteration"] for d in lines] == [1, 2]
    assert lines[0]["e_per_a"] == pytest.approx((140.0 - 8.0) / 14)
    assert "term_ms" not in lines[0] and lines[1]["term_ms"]["ladders"] == 0.5
    assert lines[1]["e_ccd"] == [-8.4, 1e-9]
    for d in lines + [r, rt]:
        assert json.loads(json.dumps(d)) == d


def test_run_accepts_json_flag(ccx):
    assert os.path.exists(RUN)
    out = run("--nmax", 2, "--A", 14, "--density", 0.08, "--layout-only", "--json").stdout
    assert "layout" in fields(out)


def json_lines(out: str):
    return [json.loads(line) for line in out.splitlines() if line.startswith("{")]


def check_log(log, r, reference: bool):
    assert log, "no records"
    assert [x["iteration"] for x in log] == list(range(1, len(log) + 1))
    # the reference loop counts every step; the standard loop's count stops before the
    # residual that met the tolerance
    assert len(log) == r["iterations"] + (0 if reference or not r["converged"] else 1)
    assert log[-1]["e_ccd"] == r["e_ccd"]
    prev = r["e_mbpt2"].real
    for x in log:
        assert x["de"] == pytest.approx(x["e_ccd"].real - prev, rel=1e-12, abs=1e-15)
        prev = x["e_ccd"].real
        assert x["ms"] >= 0.0 and x["res_norm"] >= 0.0


@pytest.mark.gpu
def test_engine_log_follows_the_solve(ccx):
    L = ccx.Layout.from_basis(2, 14, 0.08)
    e = ccx.Engine(L, real=True)
    e.generate()
    e.setup_t_amplitudes()
    r = e.ccd_iter(mode=ccx.MODE_REFERENCE)
    log = e.iter_log()
    check_log(log, r, reference=True)
    assert {x["kind"] for x in log} == {"reference"}
    assert all(not any(x["term_ms"].values()) for x in log)  # profiling off
    # mixed precision with profiling: every residual recorded with its kind and term times
    e.setup_t_amplitudes()
    e.set_profiling(True)
    r = e.ccd_iter(mode=ccx.MODE_STANDARD, precision=ccx.PREC_MIXED, tol=1e-10, rebase=ccx.REBASE_DIGITS)
    log = e.iter_log()
    check_log(log, r, reference=False)
    kinds = [x["kind"] for x in log]
    assert kinds.count("fp64") == r["fp64_sweeps"] and kinds.count("mixed") == r["mixed_iterations"]
    assert r["converged"] and kinds[-1] == "fp64"  # only an FP64 residual ends the solve
    assert log[-1]["res_norm"] == r["res_norm"] < 1e-10
    t = e.timers()
    for k in ccx.TERM_KEYS:
        assert sum(x["term_ms"][k] for x in log) == pytest.approx(t[k], rel=1e-9, abs=1e-9), k
    assert sum(x["term_ms"]["ladders"] for x in log) > 0.0


@pytest.mark.gpu
def test_run_json_records(ccx):
    args = ["--nmax", 2, "--A", 14, "--density", 0.08, "--json"]
    out = run(*args, "--mode", "standard", "--tol", 1e-10, "--precision", "bf16x3", "--triples").stdout
    f = fields(out)
    recs = json_lines(out)
    its = [x for x in recs if x["record"] == "iteration"]
    res = [x for x in recs if x["record"] == "result"]
    assert len(res) == 1 and its
    e0, eccd, et = float(f["e0"][0]), float(f["e_ccd"][0]), float(f["e_triples"][0])
    assert its[-1]["e_ccd"][0] == pytest.approx(eccd, rel=1e-15)
    assert its[-1]["kind"] == "fp64" and its[-1]["res_norm"] < 1e-10
    assert res[0]["eccd_per_a"] == pytest.approx((e0 + eccd) / 14, rel=1e-14)
    assert res[0]["eccdt_per_a"] == pytest.approx((e0 + eccd + et) / 14, rel=1e-14)
    assert res[0]["mbpt2_per_a"] == pytest.approx((e0 + float(f["e_mbpt2"][0])) / 14, rel=1e-14)
    assert res[0]["kf"] == pytest.approx(ccx.kfermi(0.08, False), rel=1e-14)
    # the reference loop driven call by call: one record per step, no residual norm
    out = run(*args, "--loop", "shim").stdout
    its = [x for x in json_lines(out) if x["record"] == "iteration"]
    assert len(its) == int(fields(out)["iterations"][0])
    assert all(x["kind"] == "reference" and x["res_norm"] is None for x in its)


def test_iter_log_argument_checks(ccx):
    """No engine is needed to see the entry point refuse bad arguments."""
    L = ccx.lib()
    n = C.c_int32(-1)
    einval = 1  # CCX_EINVAL
    assert L.ccx_engine_iter_log(None, 0, None, C.byref(n)) == einval
    assert "null engine" in L.ccx_last_error().decode()
    fake = C.c_void_p(1)  # never dereferenced: the argument checks come first
    assert L.ccx_engine_iter_log(fake, 0, None, None) == einval
    assert L.ccx_engine_iter_log(fake, -1, None, C.byref(n)) == einval
    assert L.ccx_engine_iter_log(fake, 4, None, C.byref(n)) == einval
    assert "capacity" in L.ccx_last_error().decode() and n.value == -1
