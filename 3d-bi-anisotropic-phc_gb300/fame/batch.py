"""Batched band solves over grids of uneven size.

A workload of k-point instances on several grid sizes (each with its own
chirality and band count) is solved as one plan per grid size: every plan
batches all of its instances in lock-step (fame_band_solve: CG iterations
replayed from CUDA graphs), its fncB launch parameters come from the
autotuner, and the plans run concurrently, each on its own CUDA stream driven
by its own host thread, so the kernels of different grid sizes overlap on the
GPU.  A plan solves its largest requested band count; each instance reports
its own count.  The reference runs one k-point at a time
(band_structure_woodpile_Lanczos_n60_gamma0p2.m:45-93).

    python -m fame.batch            # the 64-instance uneven workload
"""
from __future__ import annotations

import argparse
import json
import threading
import time

import numpy as np

from .handles import woodpile_plan

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


def ibz_kpoints(count, seed=0):
    """`count` wave vectors drawn uniformly from the irreducible wedge of the
    FCC Brillouin zone (a = 1; X along y as in fcc_point):
    0 <= kz <= kx <= ky <= 1 and kx + ky + kz <= 3/2, in units of 2 pi."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < count:
        k = rng.uniform(0.0, 1.0, size=(4 * count, 3))
        ok = (k[:, 2] <= k[:, 0]) & (k[:, 0] <= k[:, 1]) & (k.sum(axis=1) <= 1.5)
        out.extend(k[ok])
    return 2 * np.pi * np.asarray(out[:count])


def uneven_workload(seed=0, sizes=(32, 40, 48, 60), per_size=16, gamma_max=0.5, bands=(8, 16)):
    """Seeded instances: per grid size, `per_size` k-points from the
    irreducible zone, gamma ~ U[0, gamma_max] and a band count ~ U{bands}."""
    rng = np.random.default_rng(seed)
    kv = ibz_kpoints(len(sizes) * per_size, seed=seed)
    groups = []
    for i, n in enumerate(sizes):
        sl = slice(i * per_size, (i + 1) * per_size)
        groups.append(dict(n=int(n), kvecs=kv[sl], gammas=rng.uniform(0.0, gamma_max, per_size),
                           bands=rng.integers(bands[0], bands[1] + 1, per_size)))
    return groups


def prepare_group(g, prec="c64", autotune=True, cache=None):
    """Plan of one grid size and its autotuned fncB launch parameters (timed
    alone on the GPU, before any concurrent work)."""
    t0 = time.perf_counter()
    plan = woodpile_plan(g["n"], g["kvecs"], gammas=g["gammas"])
    tune = None
    if autotune:
        tune = plan.autotune_mixed(cache=cache) if prec == "c64" else plan.autotune(prec=prec, cache=cache)
    torch.cuda.synchronize()
    return plan, tune, time.perf_counter() - t0


def solve_group(plan, g, prec="c64", tol=1e-10, inner_tol=1e-12, stream=None):
    """Batched band solve of one grid size on `stream` (this thread's)."""
    if stream is not None:
        torch.cuda.set_stream(stream)
    t0 = time.perf_counter()
    k = int(np.max(g["bands"]))
    r = plan.band_solve(k, tol=tol, prec=prec, inner_tol=inner_tol, p=max(2 * k, 20))
    torch.cuda.current_stream().synchronize()
    omega = [np.sort(r["omega"][i])[:int(b)] for i, b in enumerate(g["bands"])]
    res = [r["res"][i][np.argsort(r["omega"][i])][:int(b)] for i, b in enumerate(g["bands"])]
    return dict(n=g["n"], omega=omega, res=res, status=int(r["status"]), stats=r["stats"],
                t_solve=time.perf_counter() - t0)


def solve_uneven(groups, prec="c64", tol=1e-10, concurrent=True, autotune=True, cache=None):
    """All groups: plans and autotuning first, then the solves concurrently
    (one stream and host thread per grid size) or one after another.
    Returns (results in group order, wall seconds of the solves)."""
    prep = [prepare_group(g, prec, autotune, cache) for g in groups]
    out = [None] * len(groups)
    errs = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if concurrent:
        streams = [torch.cuda.Stream() for _ in groups]

        def run(i):
            try:
                out[i] = solve_group(prep[i][0], groups[i], prec, tol, stream=streams[i])
            except Exception as e:  # noqa: BLE001 - reported to the caller below
                errs.append(e)

        th = [threading.Thread(target=run, args=(i,)) for i in range(len(groups))]
        for t in th:
            t.start()
        for t in th:
            t.join()
    else:
        for i, g in enumerate(groups):
            out[i] = solve_group(prep[i][0], g, prec, tol)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    for i, (plan, tune, t_setup) in enumerate(prep):
        plan.close()
        if out[i] is not None:
            out[i].update(tune=tune, t_setup=t_setup)
    if errs:
        raise errs[0]
    return out, wall


def main():
    ap = argparse.ArgumentParser(description="uneven-grid batched band solves")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--sizes", default="32,40,48,60")
    ap.add_argument("--per-size", type=int, default=16)
    ap.add_argument("--prec", default="c64", choices=["c64", "c128"])
    ap.add_argument("--sequential", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--cache", default=None, help="autotuner JSON cache")
    a = ap.parse_args()
    torch.cuda.set_device(0)
    groups = uneven_workload(a.seed, tuple(int(s) for s in a.sizes.split(",")), a.per_size)
    res, wall = solve_uneven(groups, a.prec, concurrent=not a.sequential, autotune=not a.no_autotune, cache=a.cache)
    nk = sum(len(g["kvecs"]) for g in groups)
    print(json.dumps({
        "instances": nk, "wall_s": round(wall, 3), "kpoint_solves_per_s": round(nk / wall, 4),
        "concurrent": not a.sequential, "prec": a.prec,
        "groups": [{"n": r["n"], "bands_max": int(np.max(g["bands"])), "status": r["status"],
                    "t_setup_s": round(r["t_setup"], 3), "t_solve_s": round(r["t_solve"], 3),
                    "max_res": float(max(np.max(x) for x in r["res"])), "tune": r["tune"]}
                   for r, g in zip(res, groups)]}))


if __name__ == "__main__":
    main()
