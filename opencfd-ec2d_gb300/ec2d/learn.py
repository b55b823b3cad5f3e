"""Learned warm start: dataset generation from solved fields, training, and
the comparison of warm-started against freestream-started runs.

The case family is the polar box of the batched configuration -- M ~ U[0.3,
0.8], AoA ~ U[-2, 8] deg, log10 Re ~ U[6, 7], t/c ~ U[0.09, 0.15] -- on a
fixed 257x65 single-block C-grid topology around a symmetric four-digit
airfoil (the geometry follows t/c), Spalart-Allmaras, Roe + MUSCL, LU-SGS.
The family runs on a single grid: with the turbulence equation on the fine
mesh only, the three-level V-cycle loses stability on most of these cases
(the coarse levels carry no eddy viscosity), while the single-grid LU-SGS
iteration converges monotonically.

Every solver call goes through the C-ABI (`gpu.Solver`, `gpu.WarmStartNet`);
cases run in batches of up to 64 per context (one launch per stage for the
whole batch).
"""
from __future__ import annotations

import time
from typing import Dict, List, Sequence, Tuple

import numpy as np

from . import grids
from .inputs import FLUX, SCHEME, TIME_LUSGS, TURB_SA, Params


def warmstart_cases(n: int, seed: int, nx: int = 257, ny: int = 65, num_mesh: int = 1) -> List[Tuple[Params, list, float]]:
    """n cases drawn from the polar box: (params, blocks, t/c); num_mesh 3
    runs them on the 3-level V-cycle."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        M = rng.uniform(0.3, 0.8)
        aoa = rng.uniform(-2.0, 8.0)
        re = 10.0 ** rng.uniform(6.0, 7.0)
        tc = rng.uniform(0.09, 0.15)
        p = Params(Ma=M, AoA=aoa, Re=re, Pr=0.72, If_viscous=1, Iflag_turbulence_model=TURB_SA,
                   Iflag_local_dt=1, CFL=5.0, dtmax=1.0e3, dtmin=1.0e-12, Time_Method=TIME_LUSGS,
                   Iflag_Scheme=SCHEME["MUSCL3"], Iflag_flux=FLUX["ROE"], IFlag_Reconstruction=0,
                   Num_Mesh=num_mesh, Twall=-1.0, vt_inf=3.0, mg_lusgs=1, xaxis=0.25)
        first = 1.0e-6 * 6.5e6 / re * 4.0
        blocks = grids.naca_cgrid(nx, ny, m=0.0, p=0.0, t=tc, radius=20.0, n_wake=(nx - 1) // 8 + 1,
                                  first=first, nblocks=1)
        out.append((p, blocks, tc))
    return out


def _solver(gpu, chunk, bits, mg_amut=False, configure=None):
    s = gpu.Solver([(p, b) for p, b, _ in chunk])
    s.set_lusgs_precision(bits)
    if mg_amut:
        s.mg_eddy_viscosity(1)
    if configure is not None:
        configure(s)
    for c, (_, _, tc) in enumerate(chunk, start=1):
        s.set_case_shape(c, tc)
    return s


def generate(gpu, net, cases, steps: int, batch: int = 64, bits: int = 32, target: float = None,
             check: int = 500, plateau: float = 0.8, max_seconds: float = None, mg_amut: bool = False) -> Dict:
    """Solve the cases in batches from the freestream and add every fine-mesh
    cell of the result to the network's samples.  A batch runs until every
    case's Res_rms(1) dropped below `target` x its first-iteration value, or
    until no case improved its drop by more than the factor `plateau` over
    the last four checks (`check` steps apart), or `steps` steps, or
    `max_seconds` per batch.  Records each field's drop and where it
    stopped.  mg_amut: coarse multigrid levels keep the restricted eddy
    viscosity (ec2d_mg_eddy_viscosity)."""
    t0 = time.perf_counter()
    drops, stopped = [], []
    for k in range(0, len(cases), batch):
        chunk = cases[k:k + batch]
        s = _solver(gpu, chunk, bits, mg_amut)
        s.init_flow()
        s.step(1)
        r0 = np.array([_rms(s, c) for c in range(1, len(chunk) + 1)])
        tb, done, hist, why = time.perf_counter(), 1, [], "steps"
        while done < steps:
            n = min(check, steps - done)
            s.step(n)
            done += n
            r = np.array([_rms(s, c) for c in range(1, len(chunk) + 1)]) / r0
            hist.append(np.where(np.isfinite(r), r, np.inf))
            if target is not None and np.all(hist[-1] <= target):
                why = "target"
                break
            if len(hist) > 4 and np.all(hist[-1] > plateau * hist[-5]):
                why = "plateau"
                break
            if max_seconds is not None and time.perf_counter() - tb > max_seconds:
                why = "time"
                break
        drops.extend(list(hist[-1]) if hist else [1.0] * len(chunk))
        stopped.append({"steps": done, "stop": why})
        net.add_samples(s)
        s.close()
    d = np.array(drops)
    ok = np.isfinite(d)
    return {"cases": len(cases), "steps_cap": steps, "target": target, "batches": stopped,
            "seconds": time.perf_counter() - t0, "samples": net.num_samples(),
            "drop_median": float(np.median(d[ok])) if ok.any() else None,
            "drop_max": float(np.max(d[ok])) if ok.any() else None, "diverged": int((~ok).sum()),
            "drops": [float(x) for x in d]}


def train(net, steps: int, batch: int = 16384, lr: float = 1e-3) -> Dict:
    """Adam with the learning rate cut by 10 for the last 30 % of the steps."""
    t0 = time.perf_counter()
    net.fit_normalization()
    first = net.train(1, batch=batch, lr=lr)
    k1 = int(0.7 * steps)
    mid = net.train(max(k1 - 1, 1), batch=batch, lr=lr)
    last = net.train(max(steps - k1, 1), batch=batch, lr=lr * 0.1)
    return {"steps": steps, "batch": batch, "seconds": time.perf_counter() - t0, "loss_first": first,
            "loss_mid": mid, "loss_last": last}


def _rms(s, c):
    try:
        return s.norms(c)[1][0]
    except Exception:
        return float("nan")


def _move(gpu, s, cases, idx, keep_mask, bits, mg_amut=False, configure=None):
    """The cases of context `s` at positions keep_mask (original indices
    idx[keep_mask]) into a new context: their U, ghosts included, copied
    exactly, so their iteration continues bit for bit."""
    keep = idx[keep_mask]
    Us = [[s.download_U(k + 1, 1, b) for b in range(1, len(cases[c][1]) + 1)]
          for k, c in enumerate(idx) if keep_mask[k]]
    s.close()
    s2 = _solver(gpu, [cases[c] for c in keep], bits, mg_amut, configure)
    s2.init_flow()
    for k, c in enumerate(keep):
        for b, U in enumerate(Us[k], start=1):
            s2.upload_U(k + 1, 1, b, U)
    return s2, keep


def converge(gpu, cases, start: str, bits: int, r0=None, net=None, targets=(1e-4, 1e-6, 1e-8),
             max_steps: int = 30000, check: int = 50, max_seconds: float = None, retire: float = None,
             compact: float = 0.25, fallback_steps: int = 200, fallback_ratio: float = 100.0,
             mg_amut: bool = False, configure=None) -> Dict:
    """Run all cases of `cases` in one context until every case's
    Res_rms(1) <= min(targets) x r0 or max_steps (r0: each case's
    freestream-start first residual, measured here when not given).
    start: 'freestream' or 'warm' (the network's prediction).  Records per
    case and target the first step and wall time at which it was reached.

    retire: a drop at which a case is done.  A done case (or one whose
    residual is no longer finite) has its field read back and its forces
    taken; once at least `compact` of the context's cases are done, the rest
    move into a new, smaller context (their state copied exactly), so the
    time per step follows the cases still iterating.

    A warm start keeps the freestream as the fallback: a case whose residual
    stops being finite, or exceeds fallback_ratio x its freestream-start
    residual, within the first fallback_steps steps restarts from the
    freestream (its state replaced, its status cleared).

    mg_amut: coarse multigrid levels keep the restricted eddy viscosity
    (ec2d_mg_eddy_viscosity) in every context of the run; configure: a
    callable applied to every context the run creates (e.g. the coarse
    levels' flux precision)."""
    ts = time.perf_counter()
    s = _solver(gpu, cases, bits, mg_amut, configure)
    setup_s = time.perf_counter() - ts  # context set-up: grids to the device, geometry
    n = len(cases)
    if r0 is None:
        s.init_flow()
        s.step(1)
        r0 = np.array([_rms(s, c) for c in range(1, n + 1)])
    r0 = np.asarray(r0)
    s.sync()
    t0 = time.perf_counter()
    fallback = 0
    free_U = None
    if start == "warm":
        s.init_flow()
        free_U = [[s.download_U(c, 1, b) for b in range(1, len(cases[c - 1][1]) + 1)] for c in range(1, n + 1)]
        fallback = net.warm_start(s)
    else:
        s.init_flow()
    restarted = 0
    t_start = time.perf_counter() - t0
    first = {t: np.full(n, -1) for t in targets}
    when = {t: np.full(n, np.nan) for t in targets}
    forces = np.full((n, 3), np.nan)
    idx = np.arange(n)  # original index of each case of the current context
    steps, moves, d2h_s = 0, 0, 0.0
    ratio = np.ones(n)
    done = np.zeros(n, bool)

    def finish(k_mask):
        # read the fields of the finishing cases back and take their forces
        nonlocal d2h_s
        tdl = time.perf_counter()
        for k, c in enumerate(idx):
            if k_mask[k]:
                for b in range(1, len(cases[c][1]) + 1):
                    s.download_U(k + 1, 1, b)
                try:
                    forces[c] = s.forces(k + 1)
                except Exception:
                    pass
                done[c] = True
        d2h_s += time.perf_counter() - tdl

    while steps < max_steps:
        s.step(check)
        steps += check
        r = np.array([_rms(s, k) for k in range(1, len(idx) + 1)]) / r0[idx]
        if free_U is not None and steps <= fallback_steps:
            bad = ~np.isfinite(r) | (r > fallback_ratio)
            for k in np.nonzero(bad)[0]:
                for b, U in enumerate(free_U[idx[k]], start=1):
                    s.upload_U(int(k) + 1, 1, b, U)
                s.clear_status(int(k) + 1)
                r[k] = 1.0
                restarted += 1
        ratio[idx] = r
        el = time.perf_counter() - t0
        for t in targets:
            new = (r <= t) & (first[t][idx] < 0)
            first[t][idx[new]] = steps
            when[t][idx[new]] = el
        if np.all((first[min(targets)] >= 0) | ~np.isfinite(ratio)):
            break
        if retire is not None:
            leave = (r <= retire) | ~np.isfinite(r)
            if leave.any() and (leave.all() or leave.sum() >= max(1, compact * len(idx))):
                finish(leave)
                if leave.all():
                    break
                s, idx = _move(gpu, s, cases, idx, ~leave, bits, mg_amut, configure)
                moves += 1
        if max_seconds is not None and el > max_seconds:
            break
    wall = time.perf_counter() - t0
    finish(~done[idx])  # the cases still in the context
    s.close()
    per = {}
    for t in targets:
        ok = first[t] >= 0
        per[f"{t:.0e}"] = {"reached": int(ok.sum()),
                           "steps_median": float(np.median(first[t][ok])) if ok.any() else None,
                           "seconds_all": float(np.max(when[t])) if ok.all() else None,
                           "seconds_p90": float(np.sort(when[t][ok])[int(0.9 * n) - 1]) if ok.sum() >= int(0.9 * n)
                           and int(0.9 * n) >= 1 else None,
                           "steps_per_case": first[t].tolist()}
    return {"start": start, "bits": bits, "cases": n, "steps": steps, "seconds": wall, "start_seconds": t_start,
            "setup_seconds": setup_s, "download_seconds": d2h_s, "context_moves": moves,
            "restarted_from_freestream": restarted,
            "fallback": fallback, "final_drop_max": float(np.nanmax(ratio)), "targets": per,
            "diverged": int(np.sum(~np.isfinite(ratio))),
            "forces": forces, "r0": r0, "first": first, "when": when}


def evaluate(gpu, net, held, targets=(1e-4, 1e-6, 1e-8), max_steps=30000, plain_sample=4) -> Dict:
    """The held-out cases three ways: (1) batched, FP32 LU-SGS, warm start;
    (2) batched, FP32 LU-SGS, freestream; (3) the plain drop-in -- one case
    per context, FP64, freestream -- on the first `plain_sample` cases.  The
    force differences of (1) against (3) on those cases are reported."""
    free = converge(gpu, held, "freestream", 32, targets=targets, max_steps=max_steps)
    warm = converge(gpu, held, "warm", 32, r0=free["r0"], net=net, targets=targets, max_steps=max_steps)
    plain = []
    for k in range(min(plain_sample, len(held))):
        plain.append(converge(gpu, [held[k]], "freestream", 64, r0=free["r0"][k:k + 1], targets=targets,
                              max_steps=max_steps))
    ferr = max(float(np.max(np.abs(warm["forces"][k] - plain[k]["forces"][0]))) for k in range(len(plain)))
    ms_plain = float(np.mean([p["seconds"] / max(p["steps"], 1) for p in plain])) * 1e3
    ms_batch = warm["seconds"] / max(warm["steps"], 1) * 1e3

    def strip(d):
        return {k: v for k, v in d.items() if k not in ("forces", "r0", "first", "when")}

    return {"targets": [f"{t:.0e}" for t in targets], "warm_batched_mixed": strip(warm),
            "freestream_batched_mixed": strip(free), "plain_sample": [strip(p) for p in plain],
            "ms_per_step_plain_one_case_fp64": ms_plain, "ms_per_step_batched_mixed_all_cases": ms_batch,
            "force_error_vs_plain_fp64": ferr}
