"""Writes tests/golden/tuning_gb300.jsonl: exhaustive-tuner timings of seeded
tuning workloads on the GPU this runs on (a GB300 for the committed file).

    python tests/golden/make_tuning_fixture.py [count] [seed]

Each line: the program's IR text, its inputs' shapes, its kind, its points, and
the median time in ms of 5 launches of each of the 48 configurations (L2 flushed
before every timed launch), rounded to four significant digits."""

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "compute.scala_gb300"))

from compute import tuner  # noqa: E402
from compute.runtime import NativeRuntime  # noqa: E402


def main():
    count = int(sys.argv[1]) if len(sys.argv) > 1 else 800
    seed = int(sys.argv[2]) if len(sys.argv) > 2 else 7
    rt = NativeRuntime(0)
    progs = tuner.random_programs(count, seed=seed)
    recs = tuner.collect(rt, progs, reps=5, flush_l2=True)
    with open(os.path.join(HERE, "tuning_gb300.jsonl"), "w") as f:
        for r in recs:
            r = dict(r)
            r["ms"] = [float("%.4g" % v) for v in r["ms"]]
            f.write(json.dumps(r, separators=(",", ":")) + "\n")
    print("wrote %d programs" % len(recs))


if __name__ == "__main__":
    main()
