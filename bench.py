#!/usr/bin/env python3
"""Headline benchmark: k-point band solves per second on one GB300.

Workload: the woodpile photonic crystal of the reference's band-structure
script at n = 60 (FCC, a = 1, rods of width 0.25a, eps = 13, mu = 1,
xi = -zeta = 0.2i inside, vacuum outside), the 40-point band path
Gamma-X-U|K-Gamma-L-W-X, 10 bands per k-point, every eigenpair checked with
FP64 matvecs to the reference's
NFSEP residual ||B x - omega A x|| <= 1e-8 for the B-normalised eigenvector x
(fun_no_inv/EvaluteError_Chiral_no_inv.m:20).  A step solves `--concurrent`
batches of `--batch` k-points of the path, each in one batched band solve
(complex64 matvecs and inner CG, FP64 Lanczos recurrence,
reorthogonalisation, inner-solve residual refinement, a final FP64
refinement sweep of every Ritz pair and the FP64 Ritz check) on its own
stream and host thread; with the defaults (2 batches of 10) two steps cover
the whole path.

Prints one JSON line (rank 0).  `--impl reference` times the reference's
algorithm on the host cores instead (the FP64 CPU restatement; MATLAB is not
available on this machine).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKGDIR = os.path.join(ROOT, "3d-bi-anisotropic-phc_gb300")
for _p in (PKGDIR, ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "k-point band solves/s at n=60, res<=1e-8 (batched mixed complex64/FP64, woodpile, 10 bands)"
UNIT = "k-point solves/s"
N_GRID = 60
BANDS = 10
LANCZOS_TOL = 1e-10        # the reference's Lanczos tolerance (plain FP64 form)
# Mixed form: the Lanczos stops at 1e-8 and the final FP64 refinement sweep
# (FAME_OPT_REFINE) polishes every Ritz pair; the bar is the NFSEP residual
# <= 1e-8 of every pair.  Lanczos tolerance 1e-10 instead takes ~10 % more
# steps and leaves the same worst residual: below ~1e-8 the residual is set by
# the accuracy of the inner solves, not by the Lanczos test.
LANCZOS_TOL_MIXED = 1e-8
INNER_TOL = 1e-12          # B^{-1} of the plain FP64 form (the reference's pcg tolerance)
INNER_TOL_MIXED = 3e-12    # B^{-1} of the mixed form (complex64 CG + FP64 residual refinement;
                           # tightened per k-point by the Ritz-value spread, see solvers.cu).
                           # Measured at n = 60 on the last path batch (X end): 1e-11 leaves
                           # NFSEP residuals up to 7.5e-9, 3e-12 up to 1.8e-9 (most below
                           # 1e-12) for 3.5 % more time; 1e-12 gives the same residuals as
                           # 3e-12 for 24 % more time.
# Lanczos restart size of the mixed form.  The reference uses p = 2k
# (Computational_settings_Lanczos.m:30), which the plain FP64 sample keeps.
# More columns cut the restarts at the batches holding Gamma, whose two
# shifted zero modes occupy part of the Krylov space: 2k + 4 gave +23 % over
# the path at n = 60, 2k + 6 another +3 %.  With the inner tolerance 3e-12
# (relaxed) and the double-single residuals: 2k + 6 -> 2.624 k-point solves/s
# (worst residual 2.95e-9), 2k + 8 -> 2.675 (3.22e-9), 2k + 10 -> 2.687
# (2.60e-9), 2k + 12 -> 2.680 (3.08e-9).
LANCZOS_P_MIXED = 2 * BANDS + 10
RES_TOL = 1e-8
PATH_POINTS = 40
# The FP64 oracle's own Lanczos.m solve of the woodpile at n = 60, X point
# (tests/golden/woodpile_n60_X.npz, made by tests/golden/make_golden.py
# --n60eig): its count of fncB applications turns a timed sample of oracle
# fncB applications into the time of one k-point solve.
N60_EIG_FIXTURE = os.path.join(ROOT, "tests", "golden", "woodpile_n60_X.npz")


def oracle_b_applies_n60():
    """fncB applications of the oracle's FP64 Lanczos solve at n = 60 (counted
    when the fixture was made), or None."""
    try:
        f = np.load(N60_EIG_FIXTURE)
        return float(f["b_applies"][0]) if "b_applies" in f else None
    except OSError:
        return None


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes (read + write) per complex64 fncB vector at n=60 from the
    committed ncu capture (profiles/fncb_c64_n60_traffic.json), with its
    provenance; (None, None) when absent.  It is the capture's figure, not
    measured by this run."""
    p = os.path.join(ROOT, "profiles", "fncb_c64_n60_traffic.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["dram_bytes_per_vector"]), d.get("source")
    except (OSError, KeyError, ValueError):
        return None, None


class Clocks:
    """nvidia-smi sampling of SM clocks, throttle reasons and utilization
    (the share of time a kernel was running) during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,utilization.gpu")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.path = os.path.join("/tmp", f"fame_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, busy, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
            if len(parts) > 9:
                try:
                    busy.append(float(parts[9]))
                except ValueError:
                    pass
        os.remove(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(sm), "reasons": sorted(reasons),
                "gpu_busy_pct": round(statistics.mean(busy), 1) if busy else None}


def workload_config(batch):
    """The benchmark workload, shared by both arms' JSON lines."""
    return {"workload": "woodpile n=60 (FCC a=1, rod width 0.25a, eps=13, xi=-zeta=0.2i), "
                        "40-point path G-X-U|K-G-L-W-X, 10 bands, every NFSEP residual <= 1e-8",
            "n": N_GRID, "bands": BANDS, "kpoints_per_step": batch, "path_kpoints": PATH_POINTS}


def path_batches(batch):
    """The path cut into consecutive batches, except that the Gamma points
    (the path passes Gamma twice) share the first batch: their tighter inner
    solves then overlap in one lock-step batch instead of holding up two.
    Returns (path, batches of wave vectors, batches of path indices)."""
    import fame

    path = fame.band_path(npts=PATH_POINTS)
    nb = max(1, PATH_POINTS // batch)
    order = list(range(nb * batch))
    gam = [i for i in order if not np.any(path[i])]
    slot = batch - 1
    for g in gam[1:]:
        if g < batch:
            continue  # already in the first batch
        while slot > 0 and not np.any(path[order[slot]]):
            slot -= 1  # never displace a Gamma point
        if slot <= 0:
            break
        j = order.index(g)
        order[j], order[slot] = order[slot], g
        slot -= 1
    idx = [np.array(order[i * batch:(i + 1) * batch]) for i in range(nb)]
    return path, [path[ix] for ix in idx], idx


def run_fame(args):
    import torch
    import torch.distributed as dist

    import fame

    from fame.shard import batch_index, max_over_ranks, whole_job_rate

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = fame.load()
    path, batches, bidx_path = path_batches(args.batch)
    nb = len(batches)
    C = max(1, args.concurrent)
    # step s solves batches bidx(s*C) .. bidx(s*C + C - 1), C of them at once
    bidx = lambda s: batch_index(s, rank, world, nb)
    step_batches = lambda s: [bidx(s * C + c) for c in range(C)]
    needed = sorted({b for s in range(args.warmup + args.steps) for b in step_batches(s)})
    plans = {b: fame.woodpile_plan(N_GRID, batches[b]) for b in needed}
    # fncB launch parameters timed once on one plan (fame_autotune) and
    # installed on every plan of the run (fame_set_tune)
    # (complex64 for the inner CG, double-single for the inner solves' residuals,
    # complex128 for the refinement sweep and the NFSEP checks)
    tune = plans[needed[0]].autotune(nvec=args.batch, prec="c64")
    tune128 = plans[needed[0]].autotune(nvec=args.batch, prec="c128")
    tuneds = plans[needed[0]].autotune(nvec=args.batch, prec="c128ds")

    def set_tune(pl):
        for pr, t in ((1, tune), (0, tune128), (2, tuneds)):
            pl.set_tune(pr, args.batch, int(t["chunk"]), int(t["stencil_tpb"]), int(t.get("lanes", -1)))

    for pl in plans.values():
        set_tune(pl)

    def solve(plan):
        return plan.band_solve(BANDS, tol=args.lanczos_tol, prec="c64", inner_tol=INNER_TOL_MIXED, p=args.lanczos_p)

    # C batches at once: each on its own CUDA stream, driven by its own host
    # thread (distinct plans may run concurrently; one plan may not), so the
    # kernels of one batch fill the GPU while the other waits on the host
    # (convergence checks, Gram-Schmidt tests, restarts) or runs its last
    # k-points.  Each stream starts after `start` and the caller's stream
    # waits for all of them.
    side = [torch.cuda.Stream() for _ in range(C)]

    def solve_step(batch_ids, start=None, make_plan=None):
        outs, errs = [None] * len(batch_ids), []

        def work(c, b):
            try:
                with torch.cuda.stream(side[c]):
                    if start is not None:
                        side[c].wait_event(start)
                    outs[c] = make_plan(b) if make_plan else solve(plans[b])
            except Exception as ex:  # noqa: BLE001 - re-raised below
                errs.append(ex)

        if len(batch_ids) == 1:
            work(0, batch_ids[0])
        else:
            th = [threading.Thread(target=work, args=(c, b)) for c, b in enumerate(batch_ids)]
            for t_ in th:
                t_.start()
            for t_ in th:
                t_.join()
        cur = torch.cuda.current_stream()
        for sd in side[:len(batch_ids)]:
            cur.wait_stream(sd)
        if errs:
            raise errs[0]
        return outs

    for s in range(args.warmup):
        solve_step(step_batches(s))
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = Clocks(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = lib.fame_kernel_launches()
    host0 = lib.fame_host_launches()
    clocks.start()
    e0.record(stream)
    results, result_batches = [], []
    for s in range(args.steps):
        ids = step_batches(args.warmup + s)
        results += solve_step(ids, start=e0)
        result_batches += ids
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = lib.fame_kernel_launches() - launches0
    host_launches = lib.fame_host_launches() - host0
    if world > 1:
        dist.barrier()
    t = e0.elapsed_time(e1) / 1000.0
    tmax = max_over_ranks(t, device="cuda")
    value = whole_job_rate(args.batch * C, args.steps, world, tmax)
    res_max = max(float(np.max(r["res"])) for r in results)
    worst = None
    for s, r in enumerate(results):
        i, j = np.unravel_index(int(np.argmax(r["res"])), r["res"].shape)
        if worst is None or r["res"][i, j] > worst["res"]:
            worst = {"path_index": int(bidx_path[result_batches[s]][i]), "band": int(j),
                     "res": float(r["res"][i, j]), "omega": float(r["omega"][i, j])}
    status = [int(r["status"]) for r in results]
    rb = [r["res_before"] for r in results if r.get("res_before") is not None]
    refine_report = None
    if rb:
        refine_report = {"sweeps": "one FP64 Rayleigh-Ritz sweep on [X, B^-1 A X] per k-point",
                         "max_nfsep_before": float(max(np.max(x) for x in rb)),
                         "max_nfsep_after": res_max,
                         "median_nfsep_before": float(np.median(np.concatenate([np.ravel(x) for x in rb]))),
                         "median_nfsep_after": float(np.median(np.concatenate([np.ravel(r["res"]) for r in results])))}
    steps = np.concatenate([r["stats"][:, 0] for r in results])
    cgits = np.concatenate([r["stats"][:, 3] for r in results])

    # ---- end to end through the C ABI with host buffers -------------------

    e2e_steps = max(0, min(args.steps, args.e2e_steps))
    A = fame.fcc_lattice()
    inside = fame.woodpile_inside(fame.vertex_positions(N_GRID, A), 0.25)
    phase_host = torch.from_numpy(inside.astype(np.uint8)).pin_memory().numpy()
    tens = np.stack([fame.covariant_blocks(fame.bi_isotropic(1.0, 0.0), A),
                     fame.covariant_blocks(fame.bi_isotropic(13.0, 0.2), A)])
    h2d = d2h = 0
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    def e2e_batch(b):
        kv = batches[b]
        th = np.stack([fame.bloch_angles(k, A) for k in kv])
        with fame.Plan(N_GRID, th, phase_host, tens) as pl:
            set_tune(pl)
            r = pl.band_solve(BANDS, tol=args.lanczos_tol, prec="c64", inner_tol=INNER_TOL_MIXED, p=args.lanczos_p)
        return r, phase_host.nbytes + th.nbytes + tens.nbytes * len(kv), \
            r["ew"].nbytes + r["res"].nbytes + r["stats"].nbytes

    for s in range(e2e_steps):
        for r, hb, db in solve_step(step_batches(s), make_plan=e2e_batch):
            h2d += hb
            d2h += db
    torch.cuda.synchronize()
    te = max_over_ranks(time.perf_counter() - t0, device="cuda")
    e2e_value = whole_job_rate(args.batch * C, e2e_steps, world, te) if e2e_steps else None

    out = None
    if rank == 0:
        # ---- roofline of the dominant operator: complex64 fncB ------------
        plan = plans[needed[0]]
        L = 4 * N_GRID ** 3
        x = torch.randn(args.batch, L, dtype=torch.complex64, device="cuda")
        for _ in range(3):
            plan.apply_B(x)
        torch.cuda.synchronize()
        r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 20
        r0.record(stream)
        for _ in range(reps):
            plan.apply_B(x)
        r1.record(stream)
        torch.cuda.synchronize()
        t_b = r0.elapsed_time(r1) / 1000.0 / reps
        Nq = N_GRID ** 3
        alg_bytes = args.batch * (32 * Nq * 8 + Nq)
        peak, peak_kind = measured_peak_hbm()
        achieved = alg_bytes / t_b / 1e9
        traffic, traffic_src = profile_traffic()
        roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                    "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                    "traffic": None if traffic is None else round(traffic * args.batch),
                    "traffic_source": traffic_src,
                    "kernel": f"fncB complex64 n=60, {args.batch} vectors per launch sequence",
                    "launch_us": round(t_b * 1e6, 1)}
        # ---- plain FP64 form on a whole batch of the same path ----------------
        # (a batch without the Gamma point, whose shifted zero modes double the
        # count of B applies); the mixed form's eigenvalues of that batch come
        # from the timed steps
        fp64 = None
        if args.fp64_kpoints > 0:
            fb = 1 if nb > 1 else 0
            kv = batches[fb][:args.fp64_kpoints]
            ew_mixed = None
            for s, r in enumerate(results):
                if result_batches[s] == fb:
                    ew_mixed = r["ew"][:args.fp64_kpoints]
            if ew_mixed is None:
                pm = fame.woodpile_plan(N_GRID, kv)
                ew_mixed = pm.band_solve(BANDS, tol=args.lanczos_tol, prec="c64", inner_tol=INNER_TOL_MIXED,
                                         p=args.lanczos_p)["ew"]
                pm.close()

            def fp64_solve(precond, p, inner_tol):
                pl = fame.woodpile_plan(N_GRID, kv)
                pl.set_option("precond", int(precond))
                pl.autotune(nvec=len(kv), prec="c128")
                torch.cuda.synchronize()
                f0 = time.perf_counter()
                r = pl.band_solve(BANDS, tol=LANCZOS_TOL, prec="c128", inner_tol=inner_tol, p=p)
                torch.cuda.synchronize()
                t = time.perf_counter() - f0
                pl.close()
                return r, len(kv) / t

            # the reference's algorithm: unpreconditioned pcg to 1e-12 (fncinvB.m), p = 2k
            r64, v64 = fp64_solve(False, 2 * BANDS, INNER_TOL)
            err = float(np.max(np.abs(ew_mixed - r64["ew"]) / np.abs(r64["ew"])))
            fp64 = {"value": round(v64, 5), "unit": UNIT, "kpoints": int(len(kv)),
                    "form": "FP64 matvecs and CG, unpreconditioned, p = 2k, inner tol 1e-12 (Lanczos.m / fncinvB.m)",
                    "b_applies_per_kpoint": float(np.mean(r64["stats"][:, 2])),
                    "max_res": float(np.max(r64["res"])), "speedup_mixed_vs_fp64": round(value / v64, 2),
                    "max_rel_eig_err_mixed_vs_fp64": err, "eigenvalues_compared": int(r64["ew"].size)}
            if args.fp64_precision_only:
                # the same algorithm as the mixed form (preconditioner, p, inner tolerance) in FP64
                rp, vp = fp64_solve(True, args.lanczos_p, INNER_TOL_MIXED)
                fp64["precision_only"] = {
                    "value": round(vp, 5), "unit": UNIT,
                    "form": f"FP64 matvecs and CG with the mixed form's preconditioner, p = {args.lanczos_p}, "
                            f"inner tol {INNER_TOL_MIXED:g}",
                    "speedup_mixed_vs_fp64": round(value / vp, 2),
                    "max_res": float(np.max(rp["res"])),
                    "max_rel_eig_err_mixed_vs_fp64": float(np.max(np.abs(ew_mixed - rp["ew"]) / np.abs(rp["ew"])))}
        # ---- CPU baseline: the FP64 restatement on the host cores --------------
        cpu = None
        if world == 1 and args.cpu_seconds > 0:
            cpu = cpu_baseline(args.cpu_seconds, fp64["b_applies_per_kpoint"] if fp64 else None)
        out = {
            "metric": METRIC, "value": round(value, 5), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(tmax / args.steps * 1e3, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64/f64", "data": "synthetic (woodpile geometry, "
            "band path generated in-run)",
            "config": dict(workload_config(args.batch * C), batches_at_once=C, kpoints_per_batch=args.batch,
                           lanczos_p=args.lanczos_p, lanczos_tol_mixed=args.lanczos_tol,
                           batching="consecutive path points, the two Gamma points in one batch",
                           fncb_tune={k: int(tune[k]) for k in ("chunk", "stencil_tpb", "lanes")},
                           fncb_tune_c128={k: int(tune128[k]) for k in ("chunk", "stencil_tpb", "lanes")},
                           fncb_tune_c128ds={k: int(tuneds[k]) for k in ("chunk", "stencil_tpb", "lanes")},
                           precision="complex64 fncB + preconditioned CG, FP64 recurrence/reorth, residual "
                                     f"refinement with the double-single fncB (B^-1 to {INNER_TOL_MIXED:g}, tighter near Gamma, relaxed by "
                                     "0.9 / (largest relative Ritz residual) for later Lanczos vectors), FP64 "
                                     "Rayleigh-Ritz refinement sweep of every Ritz pair, FP64 NFSEP check",
                           l2="inputs larger than L2 (Lanczos basis and B*Q of a batch "
                              f"{2 * args.batch * args.lanczos_p * 4 * N_GRID ** 3 * 16 / 1e9:.1f} GB)"),
            "e2e": {"value": None if e2e_value is None else round(e2e_value, 5), "unit": UNIT,
                    "h2d_bytes_per_step": int(h2d / max(1, e2e_steps)),
                    "d2h_bytes_per_step": int(d2h / max(1, e2e_steps)), "steps": e2e_steps,
                    "path": "fame_plan_create (host geometry/material) + fame_band_solve + results to host"},
            "roofline": roofline, "gpu_launches": int(launches),
            "host_launch_calls": int(host_launches),  # direct kernel launches + CUDA graph launches
            "clocks": clk,
            "max_residual": res_max, "res_ok": bool(res_max <= RES_TOL), "worst_pair": worst, "status": status,
            "refinement": refine_report,
            "lanczos_steps_mean": float(np.mean(steps)), "cg_iters_per_kpoint_mean": float(np.mean(cgits)),
            "fp64": fp64, "cpu_baseline": cpu,
        }
    for p in plans.values():
        p.close()
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    if out is not None:
        print(json.dumps(out), flush=True)


def _oracle_problem():
    import oracle as O

    O.fft_workers(os.cpu_count() or 1)
    return O.build_problem(N_GRID, wave_vec=O.fcc_vertex("X"), gamma=0.2)


def cpu_baseline(seconds, b_applies_gpu):
    """Time the oracle's fncB (scipy.sparse + pocketfft, FP64) at n=60 for about
    `seconds` and extrapolate one k-point solve by the oracle's own count of
    fncB applications at n = 60 (its Lanczos.m solve, counted when the
    fixture was made), else by the GPU FP64 form's count."""
    import oracle as O

    threads = O.fft_workers(os.cpu_count() or 1)
    b_applies = oracle_b_applies_n60()
    src = "the oracle's Lanczos.m solve at n=60, X point (fixture count)"
    if b_applies is None:
        b_applies, src = b_applies_gpu, "the GPU FP64 form's count on this path"
    P = _oracle_problem()
    x = np.ones(4 * N_GRID ** 3, dtype=np.complex128)
    P.B(x)
    t0 = time.perf_counter()
    cnt = 0
    while time.perf_counter() - t0 < seconds:
        P.B(x)
        cnt += 1
    tb = (time.perf_counter() - t0) / cnt
    return {"value": round(1.0 / (tb * b_applies), 8), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{cnt} FP64 oracle fncB applications at n=60 (X point), {tb * 1e3:.1f} ms each; one "
                      f"k-point solve extrapolated as {b_applies:.0f} applications ({src})"}


# fncB applications of one FP64 Lanczos solve at n = 60 when the oracle's own
# count is missing from the fixture: the GPU FP64 form's mean on this path
# (its stats at n = 60, 10 bands, p = 2k), labelled as such in the output.
FP64_B_APPLIES_FALLBACK = 11086


def oracle_config1_solve():
    """One full solve of the CPU-sized case on the host cores: the oracle's
    Lanczos.m (FP64, unpreconditioned pcg to 1e-12, p = 2k) on the woodpile at
    n = 24, X point, 10 bands, tol 1e-10.  Returns its wall time and counts."""
    import oracle as O

    P = O.build_problem(24, wave_vec=O.fcc_vertex("X"), gamma=0.2)
    L = 4 * 24 ** 3
    nB = [0]

    def fB(x):
        nB[0] += 1
        return P.B(x)

    t0 = time.perf_counter()
    _, ew, it = O.lanczos(P.A, fB, lambda r: O.fncinvB(r, fB, 1e-12, 10000), L, BANDS, LANCZOS_TOL, 10000,
                          2 * BANDS, np.ones(L, complex))
    t = time.perf_counter() - t0
    return {"workload": "woodpile n=24, X point, 10 bands, tol 1e-10 (FP64 Lanczos.m restated)",
            "seconds": round(t, 2), "kpoint_solves_per_s": round(1.0 / t, 6), "b_applies": int(nB[0]),
            "lanczos_steps": int(it), "omega": [round(float(1.0 / e), 12) for e in ew]}


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return
    import oracle as O
    threads = O.fft_workers(os.cpu_count() or 1)  # FFT threads; the sparse material products run on one
    cfg1 = oracle_config1_solve() if args.ref_config1 else None
    P = _oracle_problem()
    x = np.ones(4 * N_GRID ** 3, dtype=np.complex128)
    for _ in range(args.warmup):
        P.B(x)
    per = max(1, args.ref_applies)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        for _ in range(per):
            P.B(x)
        times.append((time.perf_counter() - t0) / per)
    tb = statistics.median(times)
    nb = oracle_b_applies_n60()
    src = "the oracle's Lanczos.m solve at n=60, X point (fixture count)"
    if nb is None:
        nb, src = FP64_B_APPLIES_FALLBACK, "fallback: the GPU FP64 form's mean count on this path"
    v = 1.0 / (tb * nb)
    sample = (f"{per} FP64 oracle fncB applications per step at n=60 (X point), {tb * 1e3:.1f} ms each; "
              f"one k-point solve = {nb:.0f} applications ({src})")
    cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample}
    if cfg1 is not None:
        cpu["config1_measured"] = cfg1
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(tb * per * 1e3, 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": dict(workload_config(args.batch),
                       lanczos_p=2 * BANDS,
                       precision="FP64 throughout, unpreconditioned pcg to 1e-12 (the reference's algorithm, "
                                 "restated on the CPU; MATLAB unavailable on this box)"),
        "cpu_baseline": cpu,
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def profile_fncb(nvec, prec, tune=None):
    """Three fncB applications to `nvec` vectors at n=60 (first `nvec` path
    k-points): the workload of the committed ncu kernel captures.  `tune`
    (chunk, stencil threads per block) installs fixed launch parameters."""
    import torch

    import fame

    torch.cuda.set_device(0)
    path = fame.band_path(npts=PATH_POINTS)
    plan = fame.woodpile_plan(N_GRID, path[np.arange(nvec) % len(path)])
    if tune is not None:
        plan.set_tune(prec, nvec, tune[0], tune[1], tune[2] if len(tune) > 2 else -1)
    dt = torch.complex64 if prec == "c64" else torch.complex128
    x = torch.randn(nvec, 4 * N_GRID ** 3, dtype=dt, device="cuda")
    if prec == "c128ds":  # complex128 vectors, double-single arithmetic (fame_apply_B, FAME_C128_DS)
        import ctypes
        lib = fame.load()
        y = torch.empty_like(x)
        lib.fame_set_stream(plan.raw, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        for _ in range(3):
            rc = lib.fame_apply_B(plan.raw, 2, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), nvec,
                                  None, 0)
            fame._lib.check(rc, plan.raw, "fame_apply_B")
    else:
        for _ in range(3):
            y = plan.apply_B(x)
    torch.cuda.synchronize()
    print(f"fncB {prec} n={N_GRID} x{nvec}: ok, |y| = {float(torch.linalg.norm(y)):.6e}")
    plan.close()


def profile_cg(nvec):
    """Two preconditioned complex64 CG solves of 4 iterations on `nvec` vectors
    at n=60 (first `nvec` path k-points after Gamma), every kernel launched
    directly (graph replay off): the workload of the committed CG launch list."""
    import torch

    import fame

    torch.cuda.set_device(0)
    path = fame.band_path(npts=PATH_POINTS)
    plan = fame.woodpile_plan(N_GRID, path[8 + np.arange(nvec) % (len(path) - 8)])
    plan.set_option("graph", 0)
    x = torch.randn(nvec, 4 * N_GRID ** 3, dtype=torch.complex64, device="cuda")
    for _ in range(2):
        plan.apply_Binv(x, tol=1e-30, maxit=4)
    torch.cuda.synchronize()
    print(f"CG c64 n={N_GRID} x{nvec}: ok")
    plan.close()


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=10,
                    help="k-points per batched band solve (a step solves --concurrent of them); 10 = the "
                         "40-point path in four batches, whose fncB runs as two sub-batches of 5 vectors "
                         "(fills the last wave of plane-kernel CTAs)")
    ap.add_argument("--impl", choices=["fame", "reference"], default="fame")
    ap.add_argument("--concurrent", type=int, default=2,
                    help="batches solved at once per step, each on its own stream and host thread "
                         "(2: the four path batches in two steps; measured at n = 60 before the relaxed "
                         "inner tolerance: 1 -> 1.90, 2 -> 2.12, 3 -> 2.20, 4 -> 2.19 k-point solves/s, "
                         "GPU busy 97.6 -> 99.5 %%)")
    ap.add_argument("--lanczos-tol", type=float, default=LANCZOS_TOL_MIXED,
                    help="Lanczos tolerance of the mixed form (the FP64 form keeps the reference's 1e-10)")
    ap.add_argument("--lanczos-p", type=int, default=LANCZOS_P_MIXED,
                    help="Lanczos restart size of the mixed form (the reference's p = 2k is kept by the FP64 form)")
    ap.add_argument("--e2e-steps", type=int, default=4,
                    help="end-to-end steps (capped at --steps; the same batches as the timed steps)")
    ap.add_argument("--fp64-kpoints", type=int, default=10,
                    help="k-points of the plain FP64 comparison (one batch of the path without Gamma)")
    ap.add_argument("--fp64-precision-only", type=int, default=1,
                    help="also time FP64 with the mixed form's preconditioner, p and inner tolerance")
    ap.add_argument("--ref-config1", type=int, default=1,
                    help="reference arm: time one full oracle solve of the n=24 X-point case")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-applies", type=int, default=10)
    ap.add_argument("--profile-fncb", type=int, default=0, metavar="NVEC",
                    help="only apply fncB three times to NVEC vectors (for ncu captures) and exit")
    ap.add_argument("--profile-prec", choices=["c64", "c128", "c128ds"], default="c64")
    ap.add_argument("--profile-tune", default=None, metavar="CHUNK,TPB[,LANES]",
                    help="with --profile-fncb: vectors per launch sequence, stencil threads per block and "
                         "threads per FFT pencil of the plane kernels (-1 default, 0 one)")
    ap.add_argument("--profile-cg", type=int, default=0, metavar="NVEC",
                    help="only run two 4-iteration complex64 CG solves on NVEC vectors (for ncu) and exit")
    args = ap.parse_args()
    if args.profile_fncb > 0:
        profile_fncb(args.profile_fncb, args.profile_prec,
                     tuple(int(v) for v in args.profile_tune.split(",")) if args.profile_tune else None)
        return
    if args.profile_cg > 0:
        profile_cg(args.profile_cg)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_fame(args)


if __name__ == "__main__":
    main()
