"""Build-time autotuner of the traversal kernels' compile-time shape.

    python -m ospray_gb300.tune_build [--out tuned.json]

The shared-memory traversal stack depth (B200_STACK_SMEM) and the minimum
resident blocks per SM of the trace kernels (B200_TRACE_MINBLOCKS) and of the
path-tracer shade kernel (B200_SHADE_MINBLOCKS), which bound their registers,
are compile-time constants, so each candidate is a separate build of
libb200.so (into ospray_gb300/_variants/<tag>).

The candidates are timed on a HELD-OUT scene, not on the benchmark's: the
instanced-spheres generator with another seed (other instance transforms and
materials), 40 instances of a 8,192-triangle sphere (levels 5), at 1280x720
and 8 spp (bench.py --scene 7,40,5, 3 warm-up and 5 timed frames).  The
fastest candidate's defines, merged with the fixed ones (FIXED), are written
to tuned.json, which build.py then compiles with; the earlier sweep records
of tuned.json are kept.  The run-time launch shape of batches is tuned
separately (b200_batch_autotune).
"""
import argparse
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

CANDIDATES = [
    {"B200_STACK_SMEM": 12, "B200_TRACE_MINBLOCKS": 8, "B200_SHADE_MINBLOCKS": 3},
    {"B200_STACK_SMEM": 16, "B200_TRACE_MINBLOCKS": 8, "B200_SHADE_MINBLOCKS": 3},
    {"B200_STACK_SMEM": 12, "B200_TRACE_MINBLOCKS": 7, "B200_SHADE_MINBLOCKS": 3},
    {"B200_STACK_SMEM": 12, "B200_TRACE_MINBLOCKS": 6, "B200_SHADE_MINBLOCKS": 3},
    {"B200_STACK_SMEM": 12, "B200_TRACE_MINBLOCKS": 8, "B200_SHADE_MINBLOCKS": 4},
    {"B200_STACK_SMEM": 16, "B200_TRACE_MINBLOCKS": 7, "B200_SHADE_MINBLOCKS": 4},
]
# not swept here (batched trace residency; the refill threshold has its own sweep record)
FIXED = {"B200_BATCH_TRACE_MINBLOCKS": 6, "B200_REFILL_LANES": 8}
HELD_OUT = {"scene": "7,40,5", "size": "1280x720", "spp": 8}


def tag(c):
    return "s%d_b%d_h%d" % (c["B200_STACK_SMEM"], c["B200_TRACE_MINBLOCKS"], c.get("B200_SHADE_MINBLOCKS", 2))


def measure(c, size, spp, scene):
    env = dict(os.environ)
    env["B200_BUILD_DIR"] = os.path.join(HERE, "_variants", tag(c))
    env["B200_DEFINES"] = " ".join("%s=%s" % kv for kv in sorted(dict(FIXED, **c).items()))
    subprocess.run([sys.executable, "-m", "ospray_gb300.build"], cwd=ROOT, env=env, check=True,
                   capture_output=True, text=True)
    r = subprocess.run([sys.executable, "bench.py", "--workload", "pt", "--size", size, "--spp", str(spp),
                        "--scene", scene, "--steps", "5", "--warmup", "3", "--no-cpu-baseline"], cwd=ROOT,
                       env=env, capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        raise RuntimeError("candidate %s failed:\n%s" % (tag(c), r.stderr[-2000:]))
    line = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    return line["value"], line["ms_per_step"]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "tuned.json"))
    ap.add_argument("--size", default=HELD_OUT["size"])
    ap.add_argument("--spp", type=int, default=HELD_OUT["spp"])
    ap.add_argument("--scene", default=HELD_OUT["scene"], help="SEED,INSTANCES,LEVELS of the tuning scene")
    args = ap.parse_args()
    results = []
    for c in CANDIDATES:
        mrays, ms = measure(c, args.size, args.spp, args.scene)
        results.append({"defines": c, "mrays_s": mrays, "ms_per_frame": ms})
        print(json.dumps(results[-1]), flush=True)
    best = max(results, key=lambda r: r["mrays_s"])
    out = {}
    if os.path.exists(args.out):
        with open(args.out) as f:
            out = json.load(f)
    out.update({"defines": dict(FIXED, **best["defines"]),
                "workload": "pt %s %d spp, held-out scene (seed, instances, levels) = %s (bench.py --scene)" %
                            (args.size, args.spp, args.scene),
                "candidates": results})
    with open(args.out, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out["defines"]))


if __name__ == "__main__":
    main()
