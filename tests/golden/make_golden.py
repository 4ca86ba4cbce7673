"""Writes tests/golden/oracle_golden.json: regression fixtures produced by the oracle.

The reference has no golden vectors of its own and cannot be built here, so these
fixtures pin the oracle against itself over time (layout sizes, E0, MP2 and the
reference-mode CCD trajectory end point), after the oracle was checked against the
independent dense-tensor CCD and (T) in tests/test_oracle.py.
Run:  python tests/golden/make_golden.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))
import oracle as O  # noqa: E402

CASES = [
    dict(nmax=2, A=14, snm=False, rho=0.08, theta=[0.0, 0.0, 0.0], potential=0, lec_seed=20261203, ccd=True),
    dict(nmax=1, A=2, snm=False, rho=0.08, theta=[0.0, 0.0, 0.0], potential=0, lec_seed=20261203, ccd=True),
    dict(nmax=1, A=4, snm=True, rho=0.16, theta=[0.0, 0.0, 0.0], potential=0, lec_seed=20261203, ccd=True),
    dict(nmax=1, A=4, snm=True, rho=0.16, theta=[0.0, 0.0, 0.0], potential=1, lec_seed=20261203, ccd=True),
    dict(nmax=1, A=14, snm=False, rho=0.10, theta=[0.3, -1.1, 2.0], potential=0, lec_seed=20261203, ccd=True),
]


def main():
    out = {"generator": "tests/golden/make_golden.py", "cases": []}
    for c in CASES:
        cfg = O.Config(nmax=c["nmax"], A=c["A"], snm=c["snm"], rho=c["rho"], theta=tuple(c["theta"]),
                       potential=c["potential"], lec_seed=c["lec_seed"])
        o = O.Oracle(cfg)
        orb = o.orbits()
        case = {"config": {k: v for k, v in c.items() if k != "ccd"},
                "nx_head": orb["nx"].tolist()[:32],
                "n_channels": [o.n_channels(k) for k in (1, 2, 3, 4)],
                "n_amps": o.n_amps,
                "e0": o.e0().real}
        o.mp2()
        case["e_mp2"] = o.energy().real
        if c["ccd"]:
            r = o.ccd_iter(mode=O.MODE_REFERENCE)
            case["e_ccd_reference"] = r["e_ccd"].real
            case["iterations_reference"] = r["iterations"]
        out["cases"].append(case)
        print(case["config"], case["e0"], case["e_mp2"], case.get("e_ccd_reference"))
    with open(os.path.join(HERE, "oracle_golden.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
