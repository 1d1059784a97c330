"""Writes tests/golden/oracle_h54_bcc_pbe.npz: the oracle's converged SCF and
electronic gradient on the benchmark workload (H54 bcc 3x3x3, rs 1.31,
0.1 Bohr noise with seed 7, gth-dzvp, PBE, 81^3 grid, tol 1e-7).

The reference has no GGA and no forces, and its own form of this workload
would hold a 310 GB rho_pq(G) tensor, so this fixture comes from the oracle
(the NumPy FP64 restatement, itself pinned to the reference's golden vectors
on smaller cases).  It caches a run of several minutes of CPU time so that
the GPU tests can compare the engine with the oracle at full size.

    python tests/golden/make_oracle_h54.py
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from hqc_gb300.workloads import h54_bcc_pbe  # noqa: E402
from oracle.gpw import Solver  # noqa: E402
from oracle.forces import electronic_gradient  # noqa: E402

NAME = "oracle_h54_bcc_pbe"


def main():
    w = h54_bcc_pbe()
    kw = dict(grid_length=w["grid_length"], dft=True, xc="pbe", tol=1e-7, max_cycle=100)
    t0 = time.perf_counter()
    s = Solver(w["n"], w["L"], w["rs"], w["basis"], **kw)
    out = s.solve(w["xp"])
    g = electronic_gradient(s)
    dt = time.perf_counter() - t0
    np.savez(os.path.join(HERE, NAME + ".npz"), xp=w["xp"], L=w["L"], E=out[3], bands=out[2],
             Ki=out[4], Vep=out[5], Vee=out[6], converged=out[8], grad=g)
    man_path = os.path.join(HERE, "manifest.json")
    man = json.load(open(man_path))
    man[NAME] = dict(source="oracle", n=w["n"], rs=w["rs"], basis=w["basis"],
                     kwargs=dict(kw), n_grid=int(s.st.ng), seconds=round(dt, 1))
    json.dump(man, open(man_path, "w"), indent=1, sort_keys=True)
    print(f"{NAME}: E = {out[3]:.10f} Ry, converged = {bool(out[8])}, {dt:.0f} s")


if __name__ == "__main__":
    main()
