"""A runtime for the Tensor API that evaluates programs with the numpy oracle.

Test infrastructure only: it lets the CPU test suite drive the real host logic
(tree building, view composition, the fusion planner, IR serialisation) and
check it against the reference's golden vectors without a GPU.  The product's
device object never uses it.
"""

import numpy as np

from oracle import interp, rng


class OracleBuffer:
    def __init__(self, nbytes):
        self.data = np.zeros(max(1, (nbytes + 3) // 4), dtype=np.float32)
        self.nbytes = nbytes
        self.refs = 1

    def retain(self):
        self.refs += 1

    def release(self):
        assert self.refs > 0, "released a dead buffer"
        self.refs -= 1


class OracleRuntime:
    def __init__(self):
        self.launches = []

    def alloc(self, nbytes):
        return OracleBuffer(nbytes)

    def upload(self, buf, array, offset=0):
        a = np.ascontiguousarray(array, dtype=np.float32).ravel()
        buf.data[offset // 4: offset // 4 + a.size] = a

    def download(self, buf, count, dtype=np.float32, offset=0):
        assert buf.refs > 0, "read a released buffer"
        return buf.data[offset // 4: offset // 4 + count].copy()

    def program(self, text):
        return text

    def launch(self, prog, inputs, out):
        for b in inputs:
            assert b.refs > 0, "launched on a released buffer"
        self.launches.append(prog)
        kind = prog.split("\n", 1)[0].split()[2]
        vals = interp.evaluate(prog, [b.data for b in inputs])
        if kind == "sum":
            out.data[0] = np.float32(interp.exact_sum(vals))
        else:
            out.data[:vals.size] = vals

    def random(self, buf, n, seed, normal):
        buf.data[:n] = rng.random_normal(n, seed) if normal else rng.random_uniform(n, seed)
