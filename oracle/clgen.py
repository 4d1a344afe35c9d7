"""ORACLE (test infrastructure only): the reference's OpenCL C kernel text, restated.

``kernel_source(ir_text)`` emits, for an alpha-converted tree, the OpenCL C
program the reference's kernel builder emits for it:

* OpenCLKernelBuilder/src/main/scala/com/thoughtworks/compute/
  OpenCLKernelBuilder.scala: array typedefs (:61-71), the kernel signature and
  ND-range folding for ranks above 3 (:135-221), one ``const float`` per
  operator (:245-326, :516-571), view extraction (:330-456) and tuples
  (:574-655);
* Tensors/src/main/scala/com/thoughtworks/compute/Tensors.scala:1314-1321 for
  the ``jit_kernel`` wrapper and :1346-1375 for the ND-range.

The text is compiled as C by ``cref`` through ``cl_shim.h`` (OpenCL keywords
and work-item functions mapped onto an OpenMP loop nest).  Parameter names are
the alpha-converted ids, as in the reference.  Two deliberate differences: a
float ``%`` becomes ``fmod`` (OpenCL C rejects ``%`` on floats) and infinite
literals are ``INFINITY`` (the reference prints the undefined ``INFINITE``).
"""

from __future__ import annotations

from typing import Dict, List, Tuple

import numpy as np

from .interp import bits_to_f32, decimal_format3, parse

MAX_CL_DIMS = 3


def _java_float_literal(v: np.float32) -> str:
    """``${value}f`` with Scala's Float.toString (OpenCLKernelBuilder.scala:252-262)."""
    if np.isnan(v):
        return "NAN"
    if np.isinf(v):
        return "INFINITY" if v > 0 else "(-INFINITY)"
    import sys
    import os
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "compute.scala_gb300"))
    from compute.javafmt import float_to_string
    return float_to_string(v) + "f"


class _Builder:
    def __init__(self):
        self.seed = 0
        self.global_defs: List[str] = []
        self.local_defs: List[str] = []

    def fresh(self, prefix: str) -> str:
        enc = "".join(c if c.isalnum() else "_" for c in prefix)
        name = ("_%s_%d" % (enc, self.seed)) if (not enc or enc[0].isdigit()) else ("%s_%d" % (enc, self.seed))
        self.seed += 1
        return name


def kernel_source(ir_text: str) -> Tuple[str, Dict]:
    """Returns (OpenCL C source, launch info) for an ``ew`` program without ``v`` nodes."""
    kind, out_shape, nodes, root = parse(ir_text)
    b = _Builder()
    terms: Dict[int, str] = {}
    param_terms: List[Tuple[str, str]] = []  # (type, name) in parameter order
    param_info: Dict[int, Tuple[str, Tuple[int, ...], str]] = {}
    rank = len(out_shape)

    def extract(param_node: int, m, cols) -> str:
        term, pdims, pad_code = param_info[param_node]
        rows = len(pdims)
        if rows == 0:
            t = b.fresh("")
            b.local_defs.append("const float %s = *%s;" % (t, term))
            return t
        indices, bounds = [], []
        for y in range(rows):
            prods = []
            for x in range(cols):
                s = m[y * cols + x]
                if s == 0.0:
                    continue
                if x < cols - 1:
                    prods.append("__global_id_%d" % x if s == 1.0 else "__global_id_%d * %s" % (x, decimal_format3(s)))
                else:
                    prods.append(decimal_format3(s))
            iid = b.fresh("index")
            if not prods:
                b.local_defs.append("const int %s = 0;" % iid)
            else:
                b.local_defs.append("const int %s = (int)(%s);" % (iid, " + ".join(prods)))
                bounds += ["((bool)(%s >= 0))" % iid, "((bool)(%s < %d))" % (iid, pdims[y])]
            indices.append(iid)
        t = b.fresh("")
        deref = "(*%s)%s" % (term, "".join("[%s]" % i for i in indices))
        if bounds:
            b.local_defs.append("const float %s = (%s) ? %s : %s;" % (t, " && ".join(bounds), deref, pad_code))
        else:
            b.local_defs.append("const float %s = %s;" % (t, deref))
        return t

    def gen(i: int) -> str:
        if i in terms:
            return terms[i]
        ln = nodes[i]
        tag = ln[0]
        if tag == "p":
            r = int(ln[1])
            dims = tuple(int(v) for v in ln[2:2 + r])
            pad_code = _java_float_literal(bits_to_f32(ln[2 + r]))
            tname = b.fresh("float_array")
            b.global_defs.append("typedef global const float (* %s)%s;" % (tname, "".join("[%d]" % d for d in dims)))
            pname = b.fresh(str(len(param_terms)))
            param_terms.append((tname, pname))
            param_info[i] = (pname, dims, pad_code)
            terms[i] = pname
            return pname
        if tag == "l":
            out = _java_float_literal(bits_to_f32(ln[1]))
        elif tag == "x":
            gen(int(ln[1]))
            out = extract(int(ln[1]), [float(v) for v in ln[3:]], int(ln[2]))
        elif tag == "u":
            a = gen(int(ln[2]))
            out = b.fresh("")
            f = {"exp": "exp", "log": "log", "tanh": "tanh", "abs": "fabs", "sqrt": "sqrt"}.get(ln[1])
            if ln[1] == "neg":
                b.local_defs.append("const float %s = -%s;" % (out, a))
            else:
                b.local_defs.append("const float %s = %s(%s);" % (out, f, a))
        elif tag == "b":
            a = gen(int(ln[2]))
            c = gen(int(ln[3]))
            out = b.fresh("")
            op = ln[1]
            if op in ("min", "max"):
                b.local_defs.append("const float %s = f%s(%s, %s);" % (out, op, a, c))
            elif op == "mod":
                b.local_defs.append("const float %s = fmod(%s, %s);" % (out, a, c))
            else:
                sym = {"add": "+", "sub": "-", "mul": "*", "div": "/"}[op]
                b.local_defs.append("const float %s = %s %s %s;" % (out, a, sym, c))
        elif tag == "v":
            raise ValueError("the reference's kernels have no inlined views; serialise with fusion off")
        else:
            raise ValueError(tag)
        terms[i] = out
        return out

    rl = nodes[root]
    tuple_len = 1
    if rl[0] == "t":
        tuple_len = int(rl[1])
        elems = [gen(int(v)) for v in rl[2:2 + tuple_len]]
        ttype = b.fresh("float_tuple")
        b.global_defs.append("typedef struct %s { float tuple_data[%d]; } %s;" % (ttype, tuple_len, ttype))
        tv = b.fresh("")
        b.local_defs.append("const %s %s = {{ %s }};" % (ttype, tv, ", ".join(elems)))
        result, out_type = tv, ttype
    else:
        result, out_type = gen(root), "float"

    out_id = b.fresh("output")
    if rank > 0:
        idx = "__global_id_0"
        for d in range(1, rank):
            idx = "(%s * __global_size_%d + __global_id_%d)" % (idx, d, d)
        assign = "%s[%s] = %s;" % (out_id, idx, result)
    else:
        assign = "*%s = %s;" % (out_id, result)
    size_params: List[str] = []
    if rank <= MAX_CL_DIMS:
        dim_defs = "".join("const int __global_size_%d = get_global_size(%d);\nconst int __global_id_%d = get_global_id(%d);\n"
                           % (d, d, d, d) for d in range(rank))
    else:
        pd = rank - MAX_CL_DIMS
        size_params = ["const int __global_size_%d" % d for d in range(1, pd + 1)]
        strides = []
        stride = "1"
        for d in range(pd, -1, -1):
            strides.append("const int __stride_%d = %s;" % (d, stride))
            stride = "__stride_%d * __global_size_%d" % (d, d)
        dim_defs = "\n".join(strides) + "\n"
        dim_defs += "const int __global_size_0 = get_global_size(0) / __stride_0;\n"
        dim_defs += "const int __global_id_0 = get_global_id(0) / __stride_0;\n"
        for d in range(1, pd + 1):
            dim_defs += "const int __global_id_%d = get_global_id(0) / __stride_%d %% __global_size_%d;\n" % (d, d, d)
        for d in range(1, MAX_CL_DIMS):
            dim_defs += "const int __global_size_%d = get_global_size(%d);\nconst int __global_id_%d = get_global_id(%d);\n" % (
                d + pd, d, d + pd, d)
    params = size_params + ["%s const restrict %s" % (t, n) for t, n in param_terms] + \
        ["global %s * const restrict %s" % (out_type, out_id)]
    src = "\n".join(b.global_defs) + "\n" + \
        "kernel void jit_kernel(%s) {\n%s%s\n%s\n}\n" % (", ".join(params), dim_defs, "\n".join(b.local_defs), assign)
    # ND-range of Tensors.scala:1346-1375
    if rank > MAX_CL_DIMS:
        pd = rank - MAX_CL_DIMS
        gws = [int(np.prod(out_shape[:pd + 1]))] + list(out_shape[pd + 1:])
        size_args = list(out_shape[1:pd + 1])
    else:
        gws = list(out_shape)
        size_args = []
    return src, {"global_work_size": gws, "size_args": size_args, "n_params": len(param_terms),
                 "tuple_len": tuple_len, "out_shape": out_shape}
