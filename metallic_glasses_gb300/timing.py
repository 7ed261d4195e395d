"""Kernel and throughput timing of the STZ step on one GPU.

  python -m metallic_glasses_gb300.timing kernel --grid 128 --which 0 --steps 8
  python -m metallic_glasses_gb300.timing solve --grid 256
  python -m metallic_glasses_gb300.timing batch --replicas 256 --events 32
  python -m metallic_glasses_gb300.timing run --config grf256 --events 20000
  python -m metallic_glasses_gb300.timing ensemble --grid 32 --seeds 8
  python -m metallic_glasses_gb300.timing ensemble --grid 64 --seeds 4 --max-steps 400000 --chunk 20

`kernel` times one per-event kernel of the mixed form launch by launch with
CUDA events (which = 0: the full per-site kernel, 1: its stress-update half
only, 2: a whole event including selection). `solve` times the full re-solve
of the full field (the FFT passes) with the tuned schedule. `batch` advances independent
replicas (grid sizes 32^3..96^3, temperatures and strain rates drawn from the
seed) together in one batch, then the same replicas one at a time, and prints
both aggregate rates (one at a time = each replica in its own
context through stz_run, the single-run path). `run` advances one study
configuration through stz_run and reports its event rate and the stress error
of its periodic re-solves. `ensemble` runs the mixed and the FP64 plain form
on the same seeds through a shear loading at low temperature and compares
their ensemble-mean stress-strain curves (--fp64-incremental: the FP64
side by the incremental update instead of a re-solve per event). These are
the commands the ncu summaries are taken on.
"""
import argparse
import ctypes
import json
import math
import sys
import time

import numpy as np

from . import api, configs


def kernel(grid, which, steps, resolve_period=0):
    eng = api.Engine(configs.mixed128(n=grid, resolve_period=resolve_period))
    ms, n = eng.kernel_time(steps=steps, which=which)
    eng.close()
    return {"grid": grid, "which": which, "launch_ms": ms, "launches": n}


def _profiler(on):
    """Open or close the CUDA profiler's range (cuProfilerStart/Stop of the
    driver), so that `ncu --profile-from-start off` sees only the timed calls."""
    try:
        drv = ctypes.CDLL("libcuda.so.1")
    except OSError:
        return
    (drv.cuProfilerStart if on else drv.cuProfilerStop)()


def solve(grid, reps=5, mixed=True, fp64=False, profile_range=False):
    """Green's-function re-solves of the mixed form's full field at grid^3
    (the FFT passes), in FP32 pairs or (fp64) in FP64, timed with CUDA events.
    alg_bytes: what one solve must move
    through HBM at least, the full re-solve figure 24 N s with s = 8: the
    eigenstrain read and the field written (8 B per component and site) and
    the half spectrum written and read once (16 B per component and wave
    vector)."""
    p = configs.mixed128(n=grid) if mixed else configs.plain128(n=grid)
    p.resolve_fp64 = 1 if fp64 else 0
    eng = api.Engine(p)
    eng.solve()
    eng.sync()
    if profile_range:
        eng.sync()
        _profiler(True)
    eng.timer_start()
    for _ in range(reps):
        eng.solve()
    ms = eng.timer_stop() / reps
    if profile_range:
        _profiler(False)
    sch = eng.fft_schedule()
    eng.close()
    n = grid ** 3
    alg = 6 * n * (8 + 8) + 6 * (grid * grid * (grid // 2 + 1)) * 16 * 2
    return {"grid": grid, "precision": "fp64" if fp64 else "fp32 pairs", "solve_ms": ms, "alg_bytes": alg, "alg_gbs": alg / (ms / 1e3) / 1e9, "schedule": sch}


def batch(replicas, events, alone=None, seed0=0):
    """Aggregate replica-events/s batched vs the same replicas one at a time.

    Every replica advances `events` thermal events in both arms (the warm-up
    of 4 events and the creation are outside the timed regions; a batch run
    returns when every replica has reached its target)."""
    ps = configs.replicas(count=replicas, seed_base=seed0)
    t0 = time.perf_counter()
    b = api.Batch(ps)
    create_s = time.perf_counter() - t0
    b.run(4)
    k0 = sum(r.scalars()["kstep"] for r in b.replicas)
    t0 = time.perf_counter()
    b.run(events)
    dt = time.perf_counter() - t0
    done = sum(r.scalars()["kstep"] for r in b.replicas) - k0
    sites = sum(p.n[0] * p.n[1] * p.n[2] for p in ps)
    b.close()
    # one at a time: every replica of the batch (alone=None) or the first
    # `alone` of them
    n1 = replicas if alone is None else min(alone, replicas)
    t1 = 0.0
    done1 = 0
    for p in ps[:n1]:
        a = api.Engine(p)
        a.run(max_events=4)
        k = a.scalars()["kstep"]
        a.sync()
        t0 = time.perf_counter()
        a.run(max_events=events)
        a.sync()
        t1 += time.perf_counter() - t0
        done1 += a.scalars()["kstep"] - k
        a.close()
    return {"replicas": replicas, "sites": sites, "events_per_replica": events, "create_s": create_s,
            "batched_events_per_s": done / dt, "alone_events_per_s": done1 / t1 if t1 > 0 else None,
            "alone_sample": n1}


RUN_CONFIGS = {"grf256": configs.grf256, "mixed128": configs.mixed128, "plain64": configs.plain128,
               "incr64": configs.incr128,
               # the reference's own 2D model at its shipped grid and input,
               # with the re-solve after every event and with the incremental update
               "ref2d512": lambda: configs.ref2d(512, 512),
               "ref2d512_incremental": lambda: configs.ref2d(512, 512, solver=api.SOLVER_KERNEL)}


def run(config, events, warmup=1000, grid=None):
    """Thermal events per second of one configuration through stz_run.

    Context creation (response table, FFT tuning, the first solve) and
    `warmup` events come before the timed region; the timed region holds
    `events` driver steps and the periodic full re-solves that fall in them,
    timed with CUDA events on the context's stream. stress_err_* are the
    worst differences between the incremental stress and a full re-solve seen
    so far (rms over sites and max, relative to the field's scale)."""
    if grid is None and config == "plain64":
        grid = 64
    p = RUN_CONFIGS[config]() if grid is None else RUN_CONFIGS[config](n=grid)
    t0 = time.perf_counter()
    eng = api.Engine(p)
    eng.sync()
    create_s = time.perf_counter() - t0
    eng.run(max_events=warmup)
    s0 = eng.scalars()
    eng.timer_start()
    eng.run(max_events=events)
    ms = eng.timer_stop()
    s1 = eng.scalars()
    main = rate = None
    if p.precision != api.PREC_MIXED:
        # the FP64 rate kernel of single driver steps (algorithmic bytes: the
        # six FP64 stress components and the FP64 barrier read, 56 B per site)
        kms, kn = eng.kernel_time(steps=16, which=0)
        n_sites = p.n[0] * p.n[1] * p.n[2]
        rate = {"launch_ms": kms, "launches": kn, "alg_bytes": 56 * n_sites,
                "achieved_gbs": 56 * n_sites / (kms / 1e3) / 1e9 if kms > 0 else None}
    if p.precision == api.PREC_MIXED:
        # the per-event pass alone, launch by launch (algorithmic bytes: read
        # and write of 5 FP32 stress coordinates and the FP32 barrier, 44 B
        # per site)
        kms, kn = eng.kernel_time(steps=16, which=0)
        n_sites = p.n[0] * p.n[1] * p.n[2]
        main = {"launch_ms": kms, "launches": kn, "alg_bytes": 44 * n_sites,
                "achieved_gbs": 44 * n_sites / (kms / 1e3) / 1e9 if kms > 0 else None}
    eng.close()
    k = s1["kstep"] - s0["kstep"]
    return {"config": config, "grid": list(p.n), "sites": p.n[0] * p.n[1] * p.n[2], "create_s": create_s,
            "events": k, "athermal_steps": s1["astep"] - s0["astep"], "ms": ms,
            "events_per_s": k / (ms / 1e3), "us_per_event": ms * 1e3 / max(k, 1),
            "resolves": s1["n_resolves"] - s0["n_resolves"],
            "stress_err_rms_worst": s1["stress_err_rms_worst"], "stress_err_max_worst": s1["stress_err_max_worst"],
            "strain": s1["eps_avg"], "stopped": s1["stopped"], "main_pass": main, "rate_pass": rate}


def _ensemble_params(grid, seed, mixed, temperature, eng_rate, eng_end, fp64_incremental=False):
    p = configs.shear64(seed, grid, eng_rate=eng_rate, eng_end=eng_end)
    p.temperature = temperature
    p.t_temp = 1 / (p.trial_frequency * math.exp(-0.37 / (temperature * 1.380658e-23 / 1.60217733e-19)))
    if mixed:
        p.precision = api.PREC_MIXED
        p.solver = api.SOLVER_KERNEL
    elif fp64_incremental:
        p.solver = api.SOLVER_KERNEL
    return p


def ensemble(grid, seeds, max_steps=100000, temperature=250.0, eng_rate=1e-4, eng_end=0.06, chunk=10,
             points=64, fp64_incremental=False, progress=False):
    """Ensemble-mean stress-strain curves of the mixed form and the FP64
    plain form: shear loading at `eng_rate` (engineering) to `eng_end` or
    `max_steps` driver steps, barrier seeds 0..seeds-1 (each seed runs in both
    forms), sigma_xy and eps_xy sampled every `chunk` steps. At 250 K a curve
    has an elastic rise (steps of 1e-4 strain while the total rate times the
    step is below one), thermal yield and strain softening. Every run is
    interpolated onto `points` strains from 0 to the smallest final strain of
    all runs; the curves are the means over seeds. rel_diff_max: the largest
    difference of the two mean curves over the plain curve's largest
    magnitude. fp64_incremental: the FP64 side updates its field by the FP64
    unit-response table instead of re-solving each event (the same events
    within rounding, about twice as fast at 64^3). progress: one line per run
    on stderr."""
    runs = {0: [], 1: []}
    info = {}
    for mixed in (1, 0):
        t0 = time.perf_counter()
        steps = events = ath = 0
        for seed in range(seeds):
            e = api.Engine(_ensemble_params(grid, seed, mixed, temperature, eng_rate, eng_end, fp64_incremental))
            xs, ys = [0.0], [0.0]
            while True:
                e.run(max_steps=chunk)
                s = e.scalars()
                xs.append(s["eps_avg"][5])
                ys.append(s["stress"][5])
                if s["stopped"] or s["step"] >= max_steps:
                    break
            steps += s["step"]
            events += s["kstep"]
            ath += s["astep"]
            e.close()
            runs[mixed].append((np.array(xs), np.array(ys)))
            if progress:
                print("ensemble %s seed %d: %d steps, eps_xy %.5f, %.1f s" % ("mixed" if mixed else "fp64", seed,
                      s["step"], xs[-1], time.perf_counter() - t0), file=sys.stderr, flush=True)
        info["mixed" if mixed else "plain"] = {"steps": steps, "thermal_events": events, "athermal_steps": ath,
                                               "wall_s": time.perf_counter() - t0}
    top = min(x[-1] for r in runs.values() for x, _ in r)
    grid_x = np.linspace(0.0, top, points)
    mean = {k: np.mean([np.interp(grid_x, x, y) for x, y in r], axis=0) for k, r in runs.items()}
    scale = float(np.abs(mean[0]).max())
    diff = np.abs(mean[1] - mean[0])
    return {"grid": grid, "seeds": seeds, "temperature_K": temperature, "eng_rate": eng_rate, "eng_end": eng_end,
            "plain_solver": "fp64 incremental" if fp64_incremental else "fp64 re-solve per event",
            "strain_xy_max": float(top), "rel_diff_max": float(diff.max() / scale) if scale > 0 else None,
            "rel_diff_mean": float(diff.mean() / scale) if scale > 0 else None,
            "peak_stress_plain": scale, "forms": info,
            "curve": {"eps_xy": grid_x[::8].tolist(), "plain": mean[0][::8].tolist(), "mixed": mean[1][::8].tolist()}}


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m metallic_glasses_gb300.timing")
    sub = ap.add_subparsers(dest="cmd", required=True)
    k = sub.add_parser("kernel")
    k.add_argument("--grid", type=int, default=128)
    k.add_argument("--which", type=int, default=0)
    k.add_argument("--steps", type=int, default=8)
    sv = sub.add_parser("solve")
    sv.add_argument("--grid", type=int, default=256)
    sv.add_argument("--reps", type=int, default=5)
    sv.add_argument("--fp64", action="store_true")
    sv.add_argument("--profile-range", action="store_true",
                    help="open the CUDA profiler range around the timed solves only")
    b = sub.add_parser("batch")
    b.add_argument("--replicas", type=int, default=256)
    b.add_argument("--events", type=int, default=32)
    b.add_argument("--alone", type=int, default=None)
    en = sub.add_parser("ensemble")
    en.add_argument("--grid", type=int, default=32)
    en.add_argument("--seeds", type=int, default=8)
    en.add_argument("--max-steps", type=int, default=100000)
    en.add_argument("--temperature", type=float, default=250.0)
    en.add_argument("--chunk", type=int, default=10)
    en.add_argument("--fp64-incremental", action="store_true",
                    help="FP64 side: incremental update by the unit-response table instead of a re-solve per event")
    r = sub.add_parser("run")
    r.add_argument("--config", choices=sorted(RUN_CONFIGS), default="grf256")
    r.add_argument("--events", type=int, default=20000)
    r.add_argument("--warmup", type=int, default=1000)
    r.add_argument("--grid", type=int, default=None)
    a = ap.parse_args(argv)
    if a.cmd == "kernel":
        out = kernel(a.grid, a.which, a.steps)
    elif a.cmd == "solve":
        out = solve(a.grid, a.reps, fp64=a.fp64, profile_range=a.profile_range)
    elif a.cmd == "run":
        out = run(a.config, a.events, a.warmup, a.grid)
    elif a.cmd == "ensemble":
        out = ensemble(a.grid, a.seeds, a.max_steps, a.temperature, chunk=a.chunk,
                       fp64_incremental=a.fp64_incremental, progress=True)
    else:
        out = batch(a.replicas, a.events, a.alone)
    print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
