"""Writes tests/golden/fed_tau.json from the reference's own fed.cpp.

Run in a tree where the reference sources are present: oracle/Makefile
target "ref" compiles the reference's src/lib/fed.cpp into
oracle/_ref/libfed_ref.so, and this script records its FED schedules
(fed_tau_by_process_time(T, 1, 0.25, reordering)) for the evolution-time
steps of several level plans and for seeded random stopping times, as
float hex strings.  The test suite checks the oracle and the library's host
plan against these vectors on any machine, with or without the reference.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle_ctypes as oc  # noqa: E402


def plan_steps():
    Ts = []
    for soffset in (1.6, 1.2, 2.0, 0.8):
        for nsub in (2, 3, 4, 5):
            opt = oc.default_options(soffset=soffset, nsublevels=nsub, omax=6)
            o = oc.Oracle(3840, 2160, opt)
            for i in range(1, o.nlevels):
                Ts.append(float(np.float32(o.level(i)["etime"]) - np.float32(o.level(i - 1)["etime"])))
    return Ts


def main():
    oc.build()
    if oc.fed_tau_reference(1.0) is None:
        raise SystemExit("oracle/_ref/libfed_ref.so is missing: the reference sources are needed")
    rng = np.random.default_rng(2024)
    Ts = plan_steps() + [float(np.float32(t)) for t in rng.uniform(0.05, 120.0, 64)]
    cases = []
    for T in Ts:
        for reorder in (True, False):
            tau = oc.fed_tau_reference(T, 1, 0.25, reorder)
            if len(tau) == 1 and reorder:
                continue  # fed.cpp's kappa-cycle with n = 1 reads tauh[-1] (undefined)
            cases.append({"T": float(T).hex(), "reordering": reorder, "tau": [float(x).hex() for x in tau]})
    with open(os.path.join(HERE, "fed_tau.json"), "w") as f:
        json.dump({"source": "reference src/lib/fed.cpp compiled by oracle/Makefile (target ref)",
                   "tau_max": 0.25, "cases": cases}, f, indent=0)
    print(len(cases), "cases")


if __name__ == "__main__":
    main()
