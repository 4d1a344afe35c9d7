"""Extracts the expected values of the reference's own tests into reference_goldens.json.

Run with the path of a Compute.scala checkout, as the first argument or in
the COMPUTE_SCALA_REFERENCE environment variable; the JSON it writes is
committed, so the tests never need the reference at run time.  For every test block named below it records, in source
order, each expected value of a ``should be(...)`` assertion: string literals
(joined when the Scala source concatenates them with ``+``), float literals,
and ``Array(...)``/``Seq(...)`` of float or string literals, each with its
file:line.
"""

from __future__ import annotations

import json
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("COMPUTE_SCALA_REFERENCE")
if __name__ == "__main__" and not REF:
    raise SystemExit("usage: make_golden.py <Compute.scala checkout> (or set COMPUTE_SCALA_REFERENCE)")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_goldens.json")

FILES = {
    "TensorsSpec": "Tensors/src/test/scala/com/thoughtworks/compute/TensorsSpec.scala",
    "cpuSpec": "cpu/src/test/scala/com/thoughtworks/compute/cpuSpec.scala",
    "cpu": "cpu/src/main/scala/com/thoughtworks/compute/cpu.scala",
    "NDimensionalAffineTransformSpec":
        "NDimensionalAffineTransform/src/test/scala/com/thoughtworks/compute/NDimensionalAffineTransformSpec.scala",
}

STRING = re.compile(r'"((?:[^"\\]|\\.)*)"')


def _balanced(text: str, start: int) -> int:
    """Index just past the parenthesis that closes the one at text[start]."""
    depth = 0
    i = start
    in_str = False
    while i < len(text):
        c = text[i]
        if in_str:
            if c == "\\":
                i += 2
                continue
            if c == '"':
                in_str = False
        elif c == '"':
            in_str = True
        elif c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
            if depth == 0:
                return i + 1
        i += 1
    raise ValueError("unbalanced")


def _value(expr: str):
    expr = expr.strip()
    strings = STRING.findall(expr)
    if expr.startswith(("Array(", "Seq(")):
        inner = expr[expr.index("(") + 1:-1]
        if strings:
            return {"seq": strings}
        try:
            return {"seq": [float(v.strip().rstrip("f")) for v in inner.split(",") if v.strip()]}
        except ValueError:
            return {"expr": expr}
    if strings:
        return {"string": "".join(strings)}
    m = re.fullmatch(r"(-?[0-9.]+(?:[eE]-?[0-9]+)?)f?", expr)
    if m:
        return {"float": float(m.group(1))}
    return {"expr": expr}


def extract(name: str, rel: str):
    path = os.path.join(REF, rel)
    with open(path) as f:
        text = f.read()
    lines = text.split("\n")
    # test blocks start with "name" in / "name" - ; cpu.scala uses @example blocks
    starts = []
    for i, ln in enumerate(lines):
        m = re.match(r'\s*"([^"]+)"\s+(in|-)\b', ln)
        if m:
            starts.append((i, m.group(1)))
        m = re.match(r"\s*\*\s+@example\s+(.*)", ln)
        if m:
            starts.append((i, "example: " + m.group(1)[:60]))
    cases = []
    offsets = [0]
    for ln in lines:
        offsets.append(offsets[-1] + len(ln) + 1)
    for k, (i, title) in enumerate(starts):
        end_line = starts[k + 1][0] if k + 1 < len(starts) else len(lines)
        block = text[offsets[i]:offsets[end_line]]
        expects = []
        for m in re.finditer(r"should\s+be\s*\(", block):
            a = block.index("(", m.start())
            b = _balanced(block, a)
            expr = re.sub(r"\s*\*\s+", " ", block[a + 1:b - 1]) if title.startswith("example") else block[a + 1:b - 1]
            line_no = i + 1 + block[:m.start()].count("\n")
            v = _value(expr)
            v["at"] = "%s:%d" % (rel, line_no)
            expects.append(v)
        if expects:
            cases.append({"test": title, "at": "%s:%d" % (rel, i + 1), "expect": expects})
    return cases


def main():
    out = {name: extract(name, rel) for name, rel in FILES.items()}
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote", OUT, sum(len(v) for v in out.values()), "test blocks")


if __name__ == "__main__":
    main()
