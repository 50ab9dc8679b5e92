"""Woodpile band structure along a k-path, saved in the reference's arrays.

band_structure_woodpile_Lanczos_n60_gamma0p2.m:39-123 loops over the wave
vectors one at a time (set-up, Lanczos, restoration, residuals) and saves
`Freq_mtx` (eigen_wanted x nk frequencies), `iter_records` (Lanczos
iterations per k), `time_minres.compute_eigs` (seconds per k) and the
per-k `res_NFSEP` / `res_ORGSEP` of `result{i}` to a .mat file.  Here the
k-points are solved in lock-step batches (fame_band_solve, one plan per
batch, geometry rasterised on the device), the ORGSEP residuals come from
fame_restore, and the same arrays go to an .npz file:

    python -m fame.band_structure --n 24 --bands 10 --out woodpile_n24.npz

`time_compute_eigs[i]` is the wall time of the batch holding k-point i
divided by the batch size (the k-points of a batch finish together).  With
`concurrent` > 1 that many batches run at once, each on its own CUDA stream
and host thread (the GPU then stays busy while one batch waits on the host);
their times overlap.
"""
from __future__ import annotations

import argparse
import contextlib
import json
import threading
import time

import numpy as np

from .handles import woodpile_plan
from .setup import band_path

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


def band_structure(n=60, wave_vecs=None, bands=8, gamma=0.2, eps_in=13.0, width=0.25, batch=8, prec="c64",
                   tol=1e-10, inner_tol=None, p=None, orgsep=True, autotune=True, out=None, concurrent=1):
    """Solve the `bands` lowest frequencies at every wave vector (rows of
    `wave_vecs`, default the 40-point path G-X-U|K-G-L-W-X) and return a dict
    of the reference's result arrays; with `out` also write them to that .npz
    file.  prec 'c64' is the mixed form (complex64 matvecs, FP64 recurrence
    and refinement), 'c128' the reference's all-FP64 form; `concurrent`
    batches are solved at once on their own streams and host threads."""
    kv = band_path() if wave_vecs is None else np.atleast_2d(np.asarray(wave_vecs, dtype=np.float64))
    nk = kv.shape[0]
    if inner_tol is None:
        inner_tol = 3e-12 if prec == "c64" else 1e-12
    if p is None:
        p = 2 * bands + 4 if prec == "c64" else 2 * bands
    freq = np.zeros((bands, nk))
    res_nfsep = np.zeros((bands, nk))
    res_orgsep = np.full((bands, nk), np.nan)
    iters = np.zeros(nk, dtype=np.int64)
    restarts = np.zeros(nk, dtype=np.int64)
    fncb_calls = np.zeros(nk, dtype=np.int64)
    cg_iters = np.zeros(nk, dtype=np.int64)
    times = np.zeros(nk)
    status = np.zeros(nk, dtype=np.int64)
    tunes = {}  # batch width -> autotuned fncB launch parameters (timed once, on the first plan)
    lock = threading.Lock()

    def solve_batch(idx):
        t0 = time.perf_counter()
        plan = woodpile_plan(n, kv[idx], gamma=gamma, eps_in=eps_in, width=width)
        try:
            if autotune and prec == "c64":
                with lock:
                    t = tunes.get(len(idx))
                    if t is None:
                        tunes[len(idx)] = plan.autotune_mixed(nvec=len(idx))
                    else:
                        plan.set_tune_mixed(len(idx), t)
            r = plan.band_solve(bands, tol=tol, p=p, prec=prec, inner_tol=inner_tol, want_vectors=orgsep)
            if orgsep:
                ev = r["ev"]
                inst = np.repeat(np.arange(len(idx), dtype=np.int32), bands)
                rr = plan.restore(ev.reshape(len(idx) * bands, -1), r["omega"].reshape(-1), inst=inst,
                                  want_fields=False)
                res_orgsep[:, idx] = rr["res_orgsep"].reshape(len(idx), bands).T
                del ev, r["ev"]
            plan.sync()
        finally:
            plan.close()
        dt = time.perf_counter() - t0
        freq[:, idx] = r["omega"].T
        res_nfsep[:, idx] = r["res"].T
        st = r["stats"]
        iters[idx], restarts[idx], fncb_calls[idx], cg_iters[idx] = st[:, 0], st[:, 1], st[:, 2], st[:, 3]
        times[idx] = dt / len(idx)
        status[idx] = r["status"]

    groups = [np.arange(b0, min(nk, b0 + batch)) for b0 in range(0, nk, batch)]
    conc = max(1, int(concurrent))
    if conc == 1:
        for idx in groups:
            solve_batch(idx)
    else:
        cuda = torch is not None and torch.cuda.is_available()
        streams = [torch.cuda.Stream() for _ in range(conc)] if cuda else [None] * conc
        errs = []

        def worker(c):
            try:
                with (torch.cuda.stream(streams[c]) if cuda else contextlib.nullcontext()):
                    for idx in groups[c::conc]:
                        solve_batch(idx)
            except Exception as e:  # noqa: BLE001 - re-raised below
                errs.append(e)

        if autotune and prec == "c64" and groups:
            solve_batch(groups[0])  # tunes once before the threads start
            groups = groups[1:]
        th = [threading.Thread(target=worker, args=(c,)) for c in range(conc)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        if errs:
            raise errs[0]
    result = dict(Freq_mtx=freq, iter_records=iters, restarts=restarts, fncB_calls=fncb_calls, cg_iterations=cg_iters,
                  time_compute_eigs=times, res_NFSEP=res_nfsep, res_ORGSEP=res_orgsep, wave_vec_array=kv.T.copy(),
                  status=status, n=n, gamma=gamma, eps_in=eps_in, width=width, prec=prec, tol=tol)
    if out:
        np.savez(out, **result)
    return result


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--n", type=int, default=60)
    ap.add_argument("--bands", type=int, default=8)
    ap.add_argument("--npts", type=int, default=40, help="samples on the path G-X-U|K-G-L-W-X")
    ap.add_argument("--gamma", type=float, default=0.2)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--prec", choices=("c64", "c128"), default="c64")
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--no-orgsep", action="store_true")
    ap.add_argument("--concurrent", type=int, default=2, help="batches solved at once (own stream and thread)")
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    t0 = time.perf_counter()
    r = band_structure(a.n, band_path(npts=a.npts), a.bands, a.gamma, batch=a.batch, prec=a.prec, tol=a.tol,
                       orgsep=not a.no_orgsep, out=a.out, concurrent=a.concurrent)
    wall = time.perf_counter() - t0
    print(json.dumps(dict(n=a.n, nk=int(r["Freq_mtx"].shape[1]), seconds=round(wall, 3), concurrent=a.concurrent,
                          max_res_NFSEP=float(r["res_NFSEP"].max()),
                          max_res_ORGSEP=float(np.nanmax(r["res_ORGSEP"])) if not a.no_orgsep else None,
                          lowest=[float(x) for x in r["Freq_mtx"][:, 0]])))


if __name__ == "__main__":
    main()
