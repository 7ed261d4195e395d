"""Events/s of the reference's own 2D code (a CPU baseline; test infrastructure).

Builds the reference's unmodified sources against the single-rank stand-ins
(build_oracle.build_ref2d, output in oracle/_ref/) at the requested grid and
runs its main on the reference's shipped input values, twice: with a few
events and with more. The difference of the two wall times over the
difference of the events is the per-event cost without the setup. One rank,
one core; the stand-in FFT replaces FFTW 2.

Needs the reference tree (where it is absent the script says so and exits 1).
Usage: python oracle/time_ref2d.py [--nx 512] [--ny 512] [--events 25]
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

from metallic_glasses_gb300 import configs  # noqa: E402
from oracle.build_oracle import build_ref2d, ref_available  # noqa: E402


def run(exe, events):
    d = tempfile.mkdtemp(prefix="stz_ref_time_")
    configs.write_input(os.path.join(d, "input"))
    log = os.path.join(d, "log.txt")
    env = dict(os.environ, STZ_REF_LOG=log, STZ_REF_MAX_EVENTS=str(events))
    t0 = time.perf_counter()
    subprocess.run([exe], cwd=d, env=env, stdout=subprocess.DEVNULL, check=True)
    dt = time.perf_counter() - t0
    thermal = sum(1 for line in open(log) if line.startswith("X") and line.split()[2] == "0")
    return dt, thermal


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=512)
    ap.add_argument("--ny", type=int, default=512)
    ap.add_argument("--events", type=int, default=25)
    a = ap.parse_args(argv)
    if not ref_available():
        print("reference tree not present", file=sys.stderr)
        return 1
    exe = build_ref2d(a.nx, a.ny, "TENSION")
    few = max(1, a.events // 5)
    t1, e1 = run(exe, few)
    t2, e2 = run(exe, a.events)
    print(json.dumps({"grid": [a.nx, a.ny], "events_per_s": (e2 - e1) / (t2 - t1), "cores": 1,
                      "kind": "reference", "sample": "events %d..%d of the reference's main on its shipped "
                      "input, %.1f s" % (e1, e2, t2 - t1)}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
