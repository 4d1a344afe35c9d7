"""The IR parser behind the C ABI rejects malformed input with a typed status
and never crashes the host process (a crash would take down the caller, e.g.
the JVM): seeded random mutations of valid program texts (tokens dropped,
duplicated, replaced by huge, negative or non-numeric values, lines cut)
through cc_codegen, in a child process whose exit status is checked."""

import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys
sys.path.insert(0, %(pkg)r)
sys.path.insert(0, %(root)r)
import numpy as np
from compute import runtime, tuner, _native

r = np.random.RandomState(%(seed)d)
texts = [p["ir"] for p in tuner.random_programs(12, seed=%(seed)d, max_points=1 << 12, max_dim=64)]
ok = bad = 0
for it in range(%(iters)d):
    lines = texts[r.randint(len(texts))].split("\n")
    toks = [l.split(" ") for l in lines]
    for _ in range(r.randint(1, 4)):
        y = r.randint(len(toks))
        if not toks[y] or toks[y] == [""]:
            continue
        x = r.randint(len(toks[y]))
        m = r.randint(6)
        if m == 0:
            del toks[y][x]
        elif m == 1:
            toks[y].insert(x, toks[y][x])
        elif m == 2:
            toks[y][x] = str(r.choice([-1, 0, 2 ** 31, 2 ** 62, -2 ** 40, 17]))
        elif m == 3:
            toks[y][x] = r.choice(["nan", "inf", "x", "", "1e9", "1e308", "-0.5", "ffffffff", "-"])
        elif m == 4:
            del toks[y]
        else:
            toks = toks[:y]
            break
    text = "\n".join(" ".join(t) for t in toks)
    try:
        runtime.codegen(text)
        ok += 1
    except _native.ComputeError:
        bad += 1
print("ok", ok, "rejected", bad)
"""


@pytest.mark.parametrize("seed", [7, 8, 9])
def test_mutated_ir_is_rejected_not_crashing(seed):
    code = CHILD % {"pkg": os.path.join(ROOT, "compute.scala_gb300"), "root": ROOT, "seed": seed, "iters": 10000}
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, (out.returncode, out.stdout[-500:], out.stderr[-2000:])
    words = out.stdout.split()
    ok, rejected = int(words[1]), int(words[3])
    assert ok + rejected == 10000 and rejected > 5000
