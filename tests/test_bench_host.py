"""Host-side arithmetic of bench.py: the twist grid, the unique-pair work model and the
algorithmic bytes the roofline divides by (no GPU needed)."""
import math
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))
import bench  # noqa: E402


def test_gauss_legendre_twist_grid():
    """64 twists of the 4x4x4 product grid on [-pi, pi]^3; the weights integrate 1 and the
    grid integrates polynomials of each angle up to degree 7 exactly."""
    g = bench.gauss_legendre_twists()
    assert len(g) == 64
    w = np.array([x[1] for x in g])
    th = np.array([x[0] for x in g])
    assert abs(w.sum() - 1.0) < 1e-14
    assert np.all(np.abs(th) < math.pi)
    # mean of theta^2 over [-pi, pi] is pi^2 / 3, of theta^6 pi^6 / 7
    assert abs((w * th[:, 0] ** 2).sum() - math.pi ** 2 / 3) < 1e-12
    assert abs((w * th[:, 1] ** 6).sum() - math.pi ** 6 / 7) < 1e-10
    # the grid is symmetric under theta -> -theta
    s = {tuple(np.round(t, 12)) for t in th}
    assert all(tuple(np.round(-t, 12)) in s for t in th)


def test_flop_model_counts_unique_pairs():
    P, H, ring = [10, 4], [3, 2], [(5, 5), (2, 2)]
    f = bench.flop_model(P, H, ring, real=True)
    assert f["pp_ladder"] == 2 * (10 * 10 * 3 + 4 * 4 * 2)
    assert f["hh_ladder"] == 2 * (10 * 3 * 3 + 4 * 2 * 2)
    assert f["i4"] == 2 * (5 * 5 * 5 + 2 * 2 * 2)
    assert f["total"] == f["ladders"] + f["i9"] + f["i4"] + f["ring"]
    fc = bench.flop_model(P, H, ring, real=False)
    assert fc["total"] == 4 * f["total"]  # a complex multiply-add is four real ones


@pytest.mark.parametrize("real", [True, False])
def test_kernel_work_bytes(real):
    """The roofline's bytes: every operand element of a launch read once and C written
    once, in FP64 (8 bytes) or complex FP64 (16); the digit representation streams 9
    two-byte planes per real component."""
    P, H, ring = [100, 40], [20, 8], [(30, 30), (6, 6)]
    e = 8 if real else 16
    nc = 1 if real else 2
    w = bench.kernel_work(P, H, ring, 1, real=real)
    P2 = sum(p * p for p in P)
    PH = sum(p * h for p, h in zip(P, H))
    kind, alg, rep = w["pp_rebase_digits"]
    assert kind == "byte"
    assert alg == e * (P2 + 2 * PH)
    assert rep == nc * 9 * 2.0 * (P2 + PH) + e * PH
    kind, alg, _ = w["hh_rebase_digits"]
    H2 = sum(h * h for h in H)
    assert kind == "byte" and alg == e * (2 * PH + H2)
    for k, (kind, alg, rep) in w.items():
        assert alg > 0, k
        if kind == "byte":
            assert rep is not None and rep > 0, k


def test_replica_twists_are_distinct():
    th = [bench.replica_theta(r) for r in range(8)]
    assert th[0] == (0.0, 0.0, 0.0)
    assert len({tuple(t) for t in th}) == 8


def test_reference_arm_times_a_whole_solve():
    """The reference arm on the PNM 14 lattice: one whole reference-mode solve of the
    oracle from MP2 (it fits the full-solve budget), reported with the contract's keys."""
    import json
    import subprocess
    out = subprocess.run([sys.executable, os.path.join(os.path.dirname(bench.__file__), "bench.py"), "--impl",
                          "reference", "--workload", "pnm14", "--steps", "1", "--warmup", "3"],
                         capture_output=True, text=True, timeout=600, check=True).stdout
    line = json.loads([x for x in out.splitlines() if x.startswith("{")][-1])
    assert line["impl"] == "reference" and line["unit"] == "s" and line["higher_is_better"] is False
    assert line["config"]["sample_unit"] == "one whole reference-mode solve"
    assert line["config"]["iterations"] == bench.REFERENCE_ITERATIONS["pnm14"]
    assert line["value"] > 0 and line["value"] == line["cpu_baseline"]["value"] == line["e2e"]["value"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


def test_triples_cpu_sample():
    s = bench.triples_cpu_sample(bench.WORKLOADS["pnm14"], 0.5)
    assert s["unit"] == "s" and s["kind"] == "port" and s["value"] > 0 and s["cores"] >= 1
    assert "extrapolated by pairs" in s["sample"]
