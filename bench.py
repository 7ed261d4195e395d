"""Benchmark: KMC events/s of the STZ step at 128^3, mixed precision vs FP64 plain.

One step = one batch of `--events-per-step` thermal KMC events of the mixed
form on the 128^3 shear-loaded configuration (synthetic barriers and modes
drawn from seed 0, all state resident in HBM). L2 is flushed between steps
(a 256 MB write). The line also carries the FP64 plain form measured on the
same grid, the stress error of the mixed form against its full re-solves, the
roofline of the per-event kernel, the end-to-end figure through the C ABI
with host-side event and scalar reads, the CPU oracle timed on the host, the
batched replicas against the same replicas one at a time, the 256^3
correlated-barrier run (event rate and stress error), the ensemble-mean
stress-strain curves of the mixed and the plain form on the same seeds, the
FP64 plain form at 64^3 next to the CPU oracle on that grid, and the
reference's own 2D model at its shipped 512 x 512 grid next to the oracle.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun each rank runs its own replica (seed = rank): scaling is weak
and no data-path collective exists.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

GRID = 128
METRIC = "KMC events/s, 128^3 grid: mixed vs FP64 plain, 1 GB300, stress err ≤1e-5"
UNIT = "events/s"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_record(kernel, grid):
    """ncu DRAM bytes per launch recorded under profiles/ (or None)."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            d = json.load(f)
        return d.get("%s@%d" % (kernel, grid))
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            t = [x.strip() for x in line.split(",")]
            if len(t) < 9:
                continue
            try:
                sm.append(float(t[1]))
                smax = float(t[2])
            except ValueError:
                continue
            for n, v in zip(names, t[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.remove(self.path)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(seconds=15.0, grid=GRID, threads=None, params=None, what=None):
    """The CPU oracle (FP64, the reference's full re-solve per event) on all
    host threads (or `threads`), on a bounded sample of the same workload
    (the 3D shear configuration at grid^3, or `params`)."""
    from metallic_glasses_gb300 import configs
    from oracle import pyoracle
    # parameters from the oracle's own derivation: this leg loads no engine code
    p = configs.plain128(n=grid, defaults=pyoracle.default_params) if params is None else params
    m = pyoracle.Model(p)
    all_threads = pyoracle.threads()
    if threads:
        pyoracle.set_threads(threads)
    try:
        m.run(max_events=1)  # first event outside the sample (warm caches)
        t0 = time.perf_counter()
        n = 0
        while time.perf_counter() - t0 < seconds and n < 2000:
            m.run(max_events=1)
            n += 1
        dt = time.perf_counter() - t0
        cores = pyoracle.threads()
    finally:
        pyoracle.set_threads(all_threads)
    what = what or "the %d^3 FP64 shear configuration (seed 0)" % grid
    return {"value": n / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d thermal events of %s after setup, %.1f s" % (n, what, dt)}


def long_checkpoints(eng, events, per=1000):
    """Continue the headline engine for `events` thermal events in steps of
    `per` (one full FP64 re-solve ends each step) and collect the stress error
    of the FP32 field against each re-solve."""
    l2, mx = [], []
    k0 = eng.scalars()["kstep"]
    eng.sync()
    eng.timer_start()
    t0 = time.perf_counter()
    for _ in range(events // per):
        eng.run(max_events=per)
        sc = eng.scalars()
        l2.append(sc["stress_err_rms"])
        mx.append(sc["stress_err_max"])
    ms = eng.timer_stop()
    wall = time.perf_counter() - t0
    sc = eng.scalars()
    done = sc["kstep"] - k0

    def summ(v):
        v = sorted(v)
        q = lambda f: v[min(len(v) - 1, int(f * len(v)))]
        return {"max": v[-1], "p99": q(0.99), "p50": q(0.5), "last": None}

    s2, sm = summ(l2), summ(mx)
    s2["last"], sm["last"] = l2[-1], mx[-1]
    return {"events": done, "checkpoints": len(l2), "resolves_total": sc["n_resolves"],
            "events_per_s": done / (ms / 1e3), "wall_s": wall, "rejections": sc["rejections"],
            "near_ties": sc["near_ties"], "stress_err_rel_l2": s2, "stress_err_rel_max": sm,
            "every_100th_checkpoint_rel_l2": l2[99::100],
            "definition": "per checkpoint (every 1000 events): deviatoric stress of the FP32 incremental "
                          "field against the full FP64 re-solve of the same eigenstrain; relative L2 norm "
                          "and max norm (over the largest value)"}


def reduce_ranks(ms, events, dist=None):
    """Whole-job figures of a weak-scaling run: the slowest rank's time and the
    events of all ranks (host tensors, so gloo serves as well as NCCL)."""
    if dist is None:
        return ms, events
    import torch
    t = torch.tensor([ms], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    e = torch.tensor([events], dtype=torch.float64)
    dist.all_reduce(e)
    return float(t.item()), int(e.item())


DTYPE = ("f32 field/rates/line sums, int64 fixed-point plane/line/site selection, "
         "f64 clock/eigenstrain/mean strain/periodic re-solve")


def headline_config(n, events_per_step, world):
    """The `config` of the headline line (both arms print the same one)."""
    return {"workload": "STZ KMC, mixed form, %d^3 grid, 20 modes, shear strain rate 5e-5/s, T=455 K, "
                        "%d thermal events per step, full FP64 re-solve every 1000 events" % (n, events_per_step),
            "grid": n, "sites": n ** 3, "events_per_step": events_per_step,
            "parallelism": "replicas" if world > 1 else "1 GPU", "l2": "flushed between steps (256 MB write)"}


def run_reference(args, rank, world):
    """The reference's method on the host cores: the CPU oracle (FP64, a full
    re-solve per event; the reference's own FFTW2+MPI+GSL build is not
    buildable here), on the headline configuration, with parameters from the
    oracle's own derivation (no engine code is loaded). Each step is a
    bounded sample of the workload: args.ref_events thermal events."""
    if rank != 0:
        return 0
    from metallic_glasses_gb300 import configs
    from oracle import pyoracle
    m = pyoracle.Model(configs.plain128(n=args.grid, defaults=pyoracle.default_params))
    for _ in range(args.warmup):
        m.run(max_events=args.ref_events)
    k0 = m.scalars()["kstep"]
    t0 = time.perf_counter()
    for _ in range(args.steps):
        m.run(max_events=args.ref_events)
    dt = time.perf_counter() - t0
    events = m.scalars()["kstep"] - k0
    value = events / dt
    cb = {"value": value, "unit": UNIT, "cores": pyoracle.threads(), "kind": "port",
          "sample": "%d steps of %d thermal events of the %d^3 FP64 shear configuration (seed 0), %.1f s"
                    % (args.steps, args.ref_events, args.grid, dt)}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
            "impl": "reference", "dtype": "f64", "data": "synthetic (seeded barriers, modes)", "scaling": "weak",
            "vs_baseline": None, "config": headline_config(args.grid, args.events_per_step, world),
            "implementation": "CPU restatement of the reference's method (oracle/stz_oracle.c, OpenMP, "
                              "FP64, full re-solve per event); the reference's own FFTW2+MPI+GSL build is not "
                              "buildable on this box",
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine")
    ap.add_argument("--events-per-step", type=int, default=1000)
    ap.add_argument("--grid", type=int, default=GRID)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-replicas", type=int, default=256)
    ap.add_argument("--no-grf", action="store_true", help="skip the 256^3 correlated-barrier run")
    ap.add_argument("--grf-events", type=int, default=20000)
    ap.add_argument("--no-ensemble", action="store_true", help="skip the stress-strain ensemble of both forms")
    ap.add_argument("--no-plain64", action="store_true", help="skip the 64^3 FP64 plain run and its CPU oracle")
    ap.add_argument("--no-ref2d", action="store_true", help="skip the reference's 2D model at 512^2")
    ap.add_argument("--no-long", action="store_true", help="skip the 10^6-event run with its checkpoint errors")
    ap.add_argument("--long-events", type=int, default=1000000)
    ap.add_argument("--ref-events", type=int, default=1, help="reference arm: thermal events per step")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        rc = run_reference(args, rank, world)
        if dist:
            dist.destroy_process_group()
        return rc

    from metallic_glasses_gb300 import api, configs
    n = args.grid
    B = args.events_per_step
    p = configs.mixed128(seed=rank, n=n, resolve_period=1000)
    p.resolve_fp64 = 1  # the periodic full re-solve in FP64
    p.device = local
    eng = api.Engine(p)
    # warm-up
    for _ in range(args.warmup):
        eng.flush_l2()
        eng.run(max_events=B)
    eng.sync()

    def barrier():
        if dist:
            dist.barrier()

    barrier()
    eng.sync()
    l0 = eng.launches()
    k0 = eng.scalars()["kstep"]
    with ClockSampler(local) as clk:
        t_wall = time.perf_counter()
        eng.timer_start()
        for _ in range(args.steps):
            eng.flush_l2()
            eng.run(max_events=B)
        ms = eng.timer_stop()
        t_wall = time.perf_counter() - t_wall
    eng.sync()
    barrier()
    sc = eng.scalars()
    events = sc["kstep"] - k0
    launches = eng.launches() - l0
    ms_max, ev_total = reduce_ranks(ms, events, dist)
    value = ev_total / (ms_max / 1e3)

    # e2e through the C ABI: run + copy this step's events and scalars to host
    h0, d0 = eng.transfer_bytes()
    first = sc["n_events_logged"]
    t_e2e = time.perf_counter()
    e2e_events = 0
    for _ in range(args.steps):
        eng.run(max_events=B)
        s2 = eng.scalars()
        evs = eng.events(first=first)
        first += len(evs)
        e2e_events += int((evs["kind"] == api.EV_THERMAL).sum())
    t_e2e = time.perf_counter() - t_e2e
    h1, d1 = eng.transfer_bytes()
    e2e = {"value": e2e_events / t_e2e, "unit": UNIT,
           "h2d_bytes_per_step": int((h1 - h0) / args.steps), "d2h_bytes_per_step": int((d1 - d0) / args.steps),
           "note": "stz_run of %d events + event log and scalars read back to host memory, wall clock" % B}

    # per-event kernel, timed launch by launch with CUDA events
    k_ms, k_n = eng.kernel_time(steps=200)
    N = n ** 3
    alg_bytes = 44 * N  # read+write 5 FP32 deviatoric stress components, read the FP32 barrier
    # the full re-solve method's figure (FFT fwd read + spectrum write + read +
    # stress write of 6 components, FP32): 24 N s bytes per event
    peak, peak_kind = peaks()
    achieved = alg_bytes / (k_ms / 1e3) / 1e9 if k_ms > 0 else None
    tr = traffic_record("k_mixed", n)
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None, "traffic": tr,
            "kernel": "k_mixed<0, 128> (incremental stress update, 20 mode rates, FP32 line sums and the "
                      "athermal vote per line; the plane sums and the selection follow in k_mixed_select)",
            "alg_bytes_per_launch": alg_bytes, "launch_ms": k_ms, "launches_timed": k_n,
            "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
            "alg_bytes_full_resolve_per_event": 24 * N * 4,
            "effective_gbs_full_resolve": 24 * N * 4 * (value / world) / 1e9}
    scf = eng.scalars()
    stress_err = {"rel_l2_worst": scf["stress_err_rms_worst"], "rel_max_worst": scf["stress_err_max_worst"],
                  "resolves": scf["n_resolves"],
                  "definition": "deviatoric stress of the FP32 incremental field vs a full FP64 re-solve of "
                                "the same eigenstrain every 1000 events; relative L2 norm and max norm"}
    long_run = None
    if world == 1 and not args.no_long:
        # the run as configured: 10^6 events on this engine, a full FP64
        # re-solve every 1000 events, the stress error at every checkpoint
        long_run = long_checkpoints(eng, args.long_events)
    eng.close()

    # FP64 plain form on the same grid (full FFT re-solve per event)
    pp = configs.plain128(seed=rank, n=n)
    pp.device = local
    pe = api.Engine(pp)
    pe.run(max_events=3)
    pe.sync()
    plain_events = 30
    pe.flush_l2()
    pe.timer_start()
    pe.run(max_events=plain_events)
    pms = pe.timer_stop()
    plain = plain_events / (pms / 1e3)
    # its FP64 rate pass alone (rates of all sites and modes, sums, selection
    # and commit): an FP64 form with the mixed form's incremental update would
    # still run it once per event, so it bounds such a form's event rate
    rate64_ms, rate64_n = pe.kernel_time(steps=8, which=0)
    pe.close()
    # the FP64 form with the incremental update (the mixed form's method in FP64)
    ip = configs.incr128(seed=rank, n=n)
    ip.device = local
    ie = api.Engine(ip)
    ie.run(max_events=3)
    ie.sync()
    incr_events = 100
    ie.flush_l2()
    ie.timer_start()
    ie.run(max_events=incr_events)
    incr = incr_events / (ie.timer_stop() / 1e3)
    ie.close()
    precision_gain = {
        "fp64_incremental_events_per_s": incr,
        "mixed_over_fp64_incremental": (value / world) / incr,
        "fp64_rate_pass_ms": rate64_ms, "launches_timed": rate64_n,
        "fp64_incremental_events_per_s_at_most": 1e3 / rate64_ms,
        "note": "FP32 against FP64 arithmetic under one method: the FP64 form with the incremental update "
                "(its rate pass alone bounds it from above); mixed_over_plain also compares the incremental "
                "update with the full re-solve per event"}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": DTYPE,
            "data": "synthetic (seeded barriers, modes)",
            "config": headline_config(n, B, world),
            "plain_fp64_events_per_s": plain, "mixed_over_plain": value / world / plain,
            "precision_gain": precision_gain,
            "stress_err": stress_err,
            "roofline": roof, "e2e": e2e, "gpu_launches": launches, "clocks": clk.summary(),
            "wall_s": t_wall}
    if long_run:
        line["long_run"] = long_run
    # the single-GPU studies and the CPU baselines run at N = 1 only: under
    # torchrun the other GPUs would idle while rank 0 runs them
    single = world == 1
    if single and not args.no_batch:
        # independent replicas of uneven sizes advanced together vs one at a time
        from metallic_glasses_gb300 import timing
        bt = timing.batch(args.batch_replicas, events=128)
        bt["workload"] = ("%d replicas, grids uniform over 32^3/48^3/64^3/96^3, T uniform in [325, 585] K, "
                          "strain rate log-uniform in [1e-5, 1e-2] /s, barrier seeds 0..%d, the seed-0 mode set; "
                          "128 thermal events each; one at a time = every replica alone through stz_run"
                          % (args.batch_replicas, args.batch_replicas - 1))
        bt["ratio"] = bt["batched_events_per_s"] / bt["alone_events_per_s"]
        line["batched"] = bt
    if single and not args.no_grf:
        # 256^3 with a correlated barrier field (Gaussian covariance, 4 voxels,
        # sd 0.15 eV), strain rate 5e-4 /s, autotuned FFT schedules
        from metallic_glasses_gb300 import timing
        gr = timing.run("grf256", events=args.grf_events, warmup=1000)
        if gr.get("main_pass") and gr["main_pass"]["achieved_gbs"]:
            # beyond L2 at 256^3: the pass streams its field from HBM
            gr["main_pass"]["peak_gbs"] = peak
            gr["main_pass"]["frac"] = gr["main_pass"]["achieved_gbs"] / peak
        gr["workload"] = ("256^3 mixed form, correlated barriers N(1.2, 0.15) eV with Gaussian covariance of "
                          "length 4 voxels, shear strain rate 5e-4 /s, %d thermal events after 1000 warm-up "
                          "events, full re-solve (FP32 pairs) every 1000 events" % args.grf_events)
        line["grf256"] = gr
    if single and not args.no_ensemble:
        # ensemble-mean stress-strain curves, mixed vs FP64 plain, same seeds
        from metallic_glasses_gb300 import timing
        en = timing.ensemble(n, 4, max_steps=600)
        en["workload"] = ("%d^3, barrier seeds 0..3 in both forms, shear loading at 250 K, first 600 steps "
                          "(the elastic rise to about 0.25 GPa); rel_diff_max = largest difference of the "
                          "two mean curves over the plain curve's peak" % n)
        line["ensemble"] = en
    if single and not args.no_plain64:
        # the FP64 plain form at 64^3 (the reference's method: a full re-solve
        # per event) next to the CPU oracle on the same grid, in the same run
        from metallic_glasses_gb300 import timing
        pl = timing.run("plain64", events=2000, warmup=100)
        rp = pl["rate_pass"]
        pl = {k: pl[k] for k in ("grid", "sites", "events", "athermal_steps", "ms", "events_per_s", "us_per_event")}
        if rp and rp["achieved_gbs"]:
            # the FP64 rate kernel against HBM: far below it, the kernel is
            # bound by the FP64 pipe (ncu: profiles/k_rate64_64.md)
            pl["roofline"] = {"kernel": "k_rate64<1> (FP64 rates of 20 modes, per-block sums, selection and commit "
                                        "in the last block)", "bound": "fp64 pipe (HBM shown for scale)",
                              "achieved": rp["achieved_gbs"], "peak": peak, "unit": "GB/s",
                              "frac": rp["achieved_gbs"] / peak, "alg_bytes_per_launch": rp["alg_bytes"],
                              "launch_ms": rp["launch_ms"], "launches_timed": rp["launches"],
                              "peak_kind": "measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                              else peak_kind}
        if not args.no_cpu:
            pl["cpu_baseline"] = cpu_baseline(seconds=8.0, grid=64)
            pl["gpu_over_cpu"] = pl["events_per_s"] / pl["cpu_baseline"]["value"]
        pl["workload"] = ("64^3 FP64 plain form, shear strain rate 5e-5 /s, T = 455 K, seed 0, 2000 thermal "
                          "events after 100 warm-up events, every event a full FP64 re-solve")
        # the same configuration with the FP64 incremental update
        pi = timing.run("incr64", events=2000, warmup=100, grid=64)
        pl["incremental"] = {"events_per_s": pi["events_per_s"], "us_per_event": pi["us_per_event"],
                             "workload": "the same with the FP64 incremental update in place of the re-solve"}
        line["plain64"] = pl
    if single and not args.no_ref2d:
        # the reference's own 2D model at its shipped 512 x 512 grid and input
        # (FP64 plain form, the reference's method), next to the CPU oracle
        from metallic_glasses_gb300 import configs, timing
        r2 = timing.run("ref2d512", events=2000, warmup=100)
        r2 = {k: r2[k] for k in ("grid", "sites", "events", "athermal_steps", "ms", "events_per_s", "us_per_event")}
        if not args.no_cpu:
            from oracle import pyoracle
            r2["cpu_baseline"] = cpu_baseline(seconds=8.0, params=configs.ref2d(
                512, 512, defaults=pyoracle.default_params, from_input=pyoracle.params_from_input),
                what="the reference's 2D model at 512 x 512 (shipped input)")
            r2["gpu_over_cpu"] = r2["events_per_s"] / r2["cpu_baseline"]["value"]
        r2["workload"] = ("the reference's 2D model (per-site barriers and eigenstrains re-drawn after each "
                          "transformation, softening on) at its shipped 512 x 512 grid and input file, TENSION, "
                          "2000 thermal events after 100 warm-up events, every event a full FP64 re-solve")
        ri = timing.run("ref2d512_incremental", events=2000, warmup=100)
        r2["incremental"] = {"events_per_s": ri["events_per_s"], "us_per_event": ri["us_per_event"],
                             "athermal_steps": ri["athermal_steps"],
                             "workload": "the same with the FP64 incremental update in place of the re-solve"}
        line["ref2d512"] = r2
    if single and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(seconds=15.0, grid=n)
        line["cpu_baseline_1core"] = cpu_baseline(seconds=8.0, grid=n, threads=1)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
