"""Command line of fame.interior: the interior eigenpairs of an inclusion
crystal at Gamma (sphere r = 0.25a or regular tetrahedron of edge 0.5a at the
cell origin), 20 pairs closest to 1.05x the 4th band edge, one JSON line.

    python -m fame.interior_cli --shape sphere --gamma 3.46427 --n 60
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from .interior import band_edge, inclusion_plan, interior_modes


def main():
    ap = argparse.ArgumentParser(description="interior eigenpairs of an inclusion crystal at Gamma")
    ap.add_argument("--shape", default="sphere", choices=["sphere", "tetra"])
    ap.add_argument("--gamma", type=float, default=3.46427)
    ap.add_argument("--n", type=int, default=60)
    ap.add_argument("--nev", type=int, default=20)
    ap.add_argument("--factor", type=float, default=1.05, help="sigma = factor * omega_4(Gamma)")
    ap.add_argument("--inner-tol", type=float, default=1e-3)
    ap.add_argument("--tol", type=float, default=1e-8)
    a = ap.parse_args()
    torch.cuda.set_device(0)
    plan = inclusion_plan(a.n, [np.zeros(3)], a.shape, a.gamma)
    t0 = time.perf_counter()
    w4 = band_edge(plan)
    t_edge = time.perf_counter() - t0
    sigma = a.factor * w4
    r = interior_modes(plan, a.nev, sigma, tol=a.tol, inner_tol=a.inner_tol)
    print(json.dumps({"shape": a.shape, "gamma": a.gamma, "n": a.n, "nev": a.nev, "omega4_gamma": w4, "sigma": sigma,
                      "t_band_edge_s": round(t_edge, 3), "t_sira_s": round(r["t_sira"], 3),
                      "t_restore_s": round(r.get("t_restore", 0.0), 3), "status": int(r["status"]),
                      "stats": [int(v) for v in r["stats"]],
                      "omega": [float(v) for v in r["omega"]],
                      "res_nfsep_max": float(np.nanmax(r["res_nfsep"])),
                      "res_orgsep_max": float(np.max(r["res_orgsep"])) if "res_orgsep" in r else None,
                      "max_e_outside": [float(v) for v in r.get("max_e", [])],
                      "max_h_outside": [float(v) for v in r.get("max_h", [])]}))




if __name__ == "__main__":
    main()
