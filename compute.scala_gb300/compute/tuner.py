"""The tuner and its learned cost model.

The reference has no tuner: it lets the OpenCL runtime choose the local size
(Tensors/src/main/scala/com/thoughtworks/compute/Tensors.scala:1360-1375) and
sizes reduction groups as min(length, CL_KERNEL_WORK_GROUP_SIZE)
(Tensors.scala:700).  Here a program's tunable form runs in 48 launch
configurations (block size x vector width x work items per thread x grid
split, ``config``).  The exhaustive tuner times all of them; the learned tuner
asks a multilayer perceptron (64 features -> 3 x 256 ReLU -> log-runtime),
trained by the library's own CUDA kernels on the exhaustive tuner's timings.

Pieces:
  - ``config`` / ``features``: the configuration table and the model's input;
  - ``TuneSet``: many programs' tunable forms, compiled together and timed;
  - ``random_program``: the seeded generator of tuning workloads (rank 1-4
    outputs, dims 1-4096, at most 64M points, inputs read through random
    views, expression trees as in the batching workload, optional sums);
  - ``collect``: timings of every configuration of every program (the timing
    database, one JSON line per program);
  - ``CostModel``: the network, its training and its choices;
  - ``evaluate``: regret of a choice against the exhaustive best.
"""

from __future__ import annotations

import ctypes
import json
import math
import os
import time
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _native
from ._native import c_handle, call

N_CONFIGS = 48
N_FEATURES = 64
MODEL_DIMS = (64, 256, 256, 256, 1)
# The method without a model: one thread per point, 256 threads per block,
# a grid covering the domain (the reference's ND-range with a typical local size).
DEFAULT_CONFIG = 26
MAX_POINTS = 64 * 1024 * 1024
# The cost model trained on GB300 timings of 18,000 tuning workloads (seed 0).
DEFAULT_MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "costmodel_gb300.npz")


def config(index: int) -> Dict[str, int]:
    """The launch configuration of index ``index`` (cc_tune_config)."""
    v = [ctypes.c_int() for _ in range(4)]
    call("cc_tune_config", int(index), *[ctypes.byref(x) for x in v])
    return {"block": v[0].value, "vec": v[1].value, "ept": v[2].value, "split": v[3].value}


def features(ir_text: str, config_index: int, sm_count: int) -> np.ndarray:
    raw = ir_text.encode()
    out = (ctypes.c_float * N_FEATURES)()
    call("cc_program_features", raw, ctypes.c_size_t(len(raw)), int(config_index), int(sm_count), out)
    return np.frombuffer(out, dtype=np.float32).copy()


def feature_matrix(ir_texts: Sequence[str], sm_count: int) -> np.ndarray:
    """[len(ir_texts) * N_CONFIGS, N_FEATURES]: every configuration of every program, program-major."""
    out = np.empty((len(ir_texts) * N_CONFIGS, N_FEATURES), dtype=np.float32)
    buf = (ctypes.c_float * N_FEATURES)()
    for p, text in enumerate(ir_texts):
        raw = text.encode()
        for c in range(N_CONFIGS):
            call("cc_program_features", raw, ctypes.c_size_t(len(raw)), c, int(sm_count), buf)
            out[p * N_CONFIGS + c] = np.frombuffer(buf, dtype=np.float32)
    return out


def compile_check(ir_texts: Sequence[str], cc=(10, 3)) -> float:
    """NVRTC-compiles the tunable forms (no GPU needed); returns seconds."""
    raws = [t.encode() for t in ir_texts]
    arr = (ctypes.c_char_p * len(raws))(*raws)
    lens = (ctypes.c_size_t * len(raws))(*[len(r) for r in raws])
    secs = ctypes.c_double()
    call("cc_tune_compile_check", arr, lens, len(raws), int(cc[0]), int(cc[1]), ctypes.byref(secs))
    return secs.value


class TuneSet:
    """Tunable forms of many programs (cc_tune_*)."""

    def __init__(self, runtime, ir_texts: Sequence[str]):
        self.rt = runtime
        raws = [t.encode() for t in ir_texts]
        arr = (ctypes.c_char_p * len(raws))(*raws)
        lens = (ctypes.c_size_t * len(raws))(*[len(r) for r in raws])
        h = c_handle()
        call("cc_tune_create", arr, lens, len(raws), ctypes.byref(h))
        self.handle = h.value
        self.n = len(raws)

    def launch(self, program: int, ptrs: Sequence[int], config_index: int):
        arr = (ctypes.c_uint64 * len(ptrs))(*ptrs)
        call("cc_tune_launch", c_handle(self.handle), int(program), arr, ctypes.c_size_t(len(ptrs)),
             int(config_index), ctypes.c_uint64(0))

    def time(self, program: int, ptrs: Sequence[int], configs: Sequence[int] = range(N_CONFIGS), reps: int = 3,
             flush_l2: bool = True) -> np.ndarray:
        arr = (ctypes.c_uint64 * len(ptrs))(*ptrs)
        cfg = (ctypes.c_int * len(configs))(*configs)
        ms = (ctypes.c_float * len(configs))()
        call("cc_tune_time", c_handle(self.handle), int(program), arr, ctypes.c_size_t(len(ptrs)), cfg,
             len(configs), int(reps), 1 if flush_l2 else 0, ms)
        return np.frombuffer(ms, dtype=np.float32).copy()

    def close(self):
        if self.handle:
            call("cc_tune_release", c_handle(self.handle))
            self.handle = 0


# ---------------------------------------------------------------- workloads

def _placeholder(d, shape):
    from .tensors import NonInlineTensor
    return NonInlineTensor(d, tuple(int(s) for s in shape), 0.0, None, kind="input")


def random_program(r: np.random.RandomState, d, max_points: int = MAX_POINTS, max_dim: int = 4096) -> dict:
    """One tuning workload: its IR text, its inputs' shapes and its kind."""
    T = d.Tensor
    rank = int(r.randint(1, 5))
    while True:
        dims = [int(round(math.exp(r.uniform(0.0, math.log(float(max_dim)))))) for _ in range(rank)]
        if int(np.prod(dims)) <= max_points:
            break
    n_in = int(r.randint(1, 5))
    leaves = []
    for _ in range(n_in):
        how = r.choice(["identity", "permute", "broadcast", "translate"], p=[0.4, 0.2, 0.2, 0.2])
        if how == "permute" and rank > 1:
            perm = [int(x) for x in r.permutation(rank)]
            inv = [0] * rank
            for i, p in enumerate(perm):
                inv[p] = i
            p = _placeholder(d, [dims[inv[j]] for j in range(rank)])
            leaves.append(p.permute(perm))
        elif how == "broadcast":
            shape = [1 if r.rand() < 0.5 else s for s in dims]
            leaves.append(_placeholder(d, shape).broadcast(dims))
        elif how == "translate":
            offset = [int(r.randint(-2, 3)) for _ in range(rank)]
            leaves.append(_placeholder(d, dims).translate(offset))
        else:
            leaves.append(_placeholder(d, dims))
    pool = list(leaves)
    for _ in range(int(r.randint(3, 13))):
        op = r.choice(["+", "-", "*", "/", "exp", "log", "tanh", "max"])
        a = pool[-1]
        b = pool[int(r.randint(0, len(pool)))]
        if op == "+":
            t = a + b
        elif op == "-":
            t = a - b
        elif op == "*":
            t = a * b
        elif op == "/":
            t = a / b
        elif op == "max":
            t = T.max(a, b)
        else:
            t = getattr(T, op)(a)
        pool.append(t)
    out = pool[-1]
    u = r.rand()
    if u < 0.2:
        ser = d.serialize(out.closure, out.shape, "sum")
        kind = "sum"
    elif u < 0.35 and rank >= 2 and dims[-1] <= 16:
        seq = out.split(rank - 1)
        s = seq.reduce(lambda x, y: x + y)
        ser = d.serialize(s.closure, s.shape)
        kind = "inner_sum"
    else:
        ser = d.serialize(out.closure, out.shape)
        kind = "ew"
    out_dims = [int(v) for v in ser.text.split("\n")[1].split()[2:]]
    return {"ir": ser.text, "params": [list(t.shape) for t in ser.params], "kind": kind,
            "points": int(np.prod(out_dims)) if out_dims else 1}


def random_programs(count: int, seed: int = 0, max_points: int = MAX_POINTS, max_dim: int = 4096) -> List[dict]:
    from .tensors import Tensors
    d = Tensors(device=0)  # shapes and IR only: no device work
    r = np.random.RandomState(seed)
    return [random_program(r, d, max_points, max_dim) for _ in range(count)]


def time_standard(runtime, ir_text: str, ptrs: Sequence[int], flush, reps: int = 5) -> float:
    """Median device time (ms) of the program's standard generated kernel (the
    runtime's default path), one untimed launch first, each timed launch after
    ``flush`` (a buffer larger than L2) is rewritten."""
    saved = runtime.config_get("tuner")
    if saved:
        runtime.config_set("tuner", 0)
    try:
        prog = runtime.program(ir_text)
    finally:
        if saved:
            runtime.config_set("tuner", saved)
    runtime.launch_ptrs(prog, ptrs[:-1], ptrs[-1])
    times = []
    for r in range(reps):
        if flush is not None:
            runtime.random(flush, flush.nbytes // 4, r, False)
        e0 = runtime.event()
        runtime.launch_ptrs(prog, ptrs[:-1], ptrs[-1])
        e1 = runtime.event()
        runtime.event_wait(e1, 60 * 10 ** 9)
        times.append(runtime.event_elapsed_ms(e0, e1))
        runtime.event_release(e0)
        runtime.event_release(e1)
    return float(sorted(times)[reps // 2])


def collect(runtime, programs: Sequence[dict], reps: int = 5, flush_l2: bool = True, chunk: int = 256,
            log=None, time_budget_s: Optional[float] = None, standard: bool = False) -> List[dict]:
    """Times every configuration of every program; returns one record per program
    ({"ir", "params", "kind", "points", "ms": [48 floats]}), and appends them to
    the file-like ``log`` as JSON lines when given.  With ``standard`` a record
    also holds "std_ms", the time of the program's standard generated kernel.

    Inputs are four shared device buffers of MAX_POINTS floats uniform in
    [0.1, 2] (input i of every program reads buffer i), the output another."""
    from .tensors import Tensors
    d = Tensors(device=0, runtime=runtime)
    p = _placeholder(d, [MAX_POINTS])
    scaled = p * d.Tensor.fill(1.9, [MAX_POINTS]) + d.Tensor.fill(0.1, [MAX_POINTS])
    prog = runtime.program(d.serialize(scaled.closure, scaled.shape).text)
    out = runtime.alloc(MAX_POINTS * 4)
    bufs = []
    for i in range(4):
        b = runtime.alloc(MAX_POINTS * 4)
        runtime.random(out, MAX_POINTS, 0x5eed + i, False)
        runtime.launch(prog, [out], b)  # uniform [0, 1) -> [0.1, 2]
        bufs.append(b)
    ptr_in = [b.device_ptr() for b in bufs]
    ptr_out = out.device_ptr()
    flush = runtime.alloc(256 << 20) if (standard and flush_l2) else None
    records = []
    t0 = time.time()
    firsts = list(range(0, len(programs), chunk))
    # the next chunk compiles (host threads) while this one is timed (GPU)
    from concurrent.futures import ThreadPoolExecutor
    pool = ThreadPoolExecutor(1)
    pending = None
    try:
        pending = pool.submit(TuneSet, runtime, [q["ir"] for q in programs[0:chunk]])
        for i, first in enumerate(firsts):
            ts = pending.result()
            pending = None
            if i + 1 < len(firsts) and not (time_budget_s is not None and time.time() - t0 > time_budget_s):
                nxt = firsts[i + 1]
                pending = pool.submit(TuneSet, runtime, [q["ir"] for q in programs[nxt:nxt + chunk]])
            part = programs[first:first + chunk]
            try:
                for k, q in enumerate(part):
                    ptrs = ptr_in[:len(q["params"])] + [ptr_out]
                    ms = ts.time(k, ptrs, reps=reps, flush_l2=flush_l2)
                    rec = dict(q)
                    rec["ms"] = [float(x) for x in ms]
                    if standard:
                        rec["std_ms"] = time_standard(runtime, q["ir"], ptrs, flush, reps)
                    records.append(rec)
                    if log is not None:
                        log.write(json.dumps(rec) + "\n")
            finally:
                ts.close()
            if pending is None:
                break
    finally:
        if pending is not None:
            try:
                pending.result().close()
            except Exception:
                pass
        pool.shutdown()
        for b in bufs:
            b.release()
        out.release()
        if flush is not None:
            flush.release()
    return records


# ---------------------------------------------------------------- the model

def init_params(dims: Sequence[int], seed: int = 0) -> np.ndarray:
    """He-uniform weights, zero biases, packed per layer as W (inputs x outputs) then b."""
    r = np.random.RandomState(seed)
    parts = []
    for k, n in zip(dims[:-1], dims[1:]):
        lim = math.sqrt(6.0 / k)
        parts.append(r.uniform(-lim, lim, size=(k, n)).astype(np.float32).ravel())
        parts.append(np.zeros(n, dtype=np.float32))
    return np.concatenate(parts)


class Mlp:
    """A network trained and evaluated by the library's CUDA kernels (cc_mlp_*)."""

    def __init__(self, runtime, dims: Sequence[int] = MODEL_DIMS, seed: int = 0):
        self.rt = runtime
        self.dims = tuple(int(x) for x in dims)
        arr = (ctypes.c_int * len(self.dims))(*self.dims)
        h = c_handle()
        call("cc_mlp_create", arr, len(self.dims), ctypes.byref(h))
        self.handle = h.value
        n = ctypes.c_size_t()
        call("cc_mlp_info", c_handle(self.handle), ctypes.byref(n), None)
        self.n_params = n.value
        self.set_params(init_params(self.dims, seed))

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        call("cc_mlp_set_params", c_handle(self.handle), p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
             ctypes.c_size_t(p.size))

    def params(self) -> np.ndarray:
        out = np.empty(self.n_params, dtype=np.float32)
        call("cc_mlp_get_params", c_handle(self.handle), out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
             ctypes.c_size_t(out.size))
        return out

    def gradients(self, x_ptr: int, t_ptr: int, batch: int):
        loss = ctypes.c_float()
        g = np.empty(self.n_params, dtype=np.float32)
        call("cc_mlp_gradients", c_handle(self.handle), ctypes.c_uint64(x_ptr), ctypes.c_uint64(t_ptr), int(batch),
             ctypes.byref(loss), g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        return loss.value, g

    def train_step(self, x_ptr: int, t_ptr: int, batch: int, lr: float, beta1=0.9, beta2=0.999, eps=1e-8,
                   want_loss=False):
        loss = ctypes.c_float()
        call("cc_mlp_train_step", c_handle(self.handle), ctypes.c_uint64(x_ptr), ctypes.c_uint64(t_ptr), int(batch),
             ctypes.c_float(lr), ctypes.c_float(beta1), ctypes.c_float(beta2), ctypes.c_float(eps),
             ctypes.byref(loss) if want_loss else None)
        return loss.value if want_loss else None

    def forward(self, x_ptr: int, batch: int, y_ptr: int):
        call("cc_mlp_forward", c_handle(self.handle), ctypes.c_uint64(x_ptr), int(batch), ctypes.c_uint64(y_ptr),
             ctypes.c_uint64(0))

    def close(self):
        if self.handle:
            call("cc_mlp_release", c_handle(self.handle))
            self.handle = 0


class CostModel:
    """Predicts the log-runtime of (program, configuration) from its features
    (relative to the program's other configurations when trained so)."""

    def __init__(self, runtime, seed: int = 0):
        self.rt = runtime
        self.net = Mlp(runtime, MODEL_DIMS, seed)
        self.mean = np.zeros(N_FEATURES, dtype=np.float32)
        self.inv_std = np.ones(N_FEATURES, dtype=np.float32)
        self.seed = seed

    def _normalise(self, x: np.ndarray) -> np.ndarray:
        return ((x - self.mean) * self.inv_std).astype(np.float32)

    def fit(self, x: np.ndarray, y: np.ndarray, epochs: int = 30, batch: int = 4096, lr: float = 1e-3,
            lr_final: float = 1e-4, log=None) -> List[float]:
        """Adam on the mean squared error of log-runtime; the learning rate
        decays geometrically from lr to lr_final.  Returns the loss per epoch."""
        x = np.asarray(x, dtype=np.float32)
        y = np.asarray(y, dtype=np.float32)
        self.mean = x.mean(axis=0).astype(np.float32)
        std = x.std(axis=0)
        self.inv_std = np.where(std > 1e-6, 1.0 / np.maximum(std, 1e-6), 0.0).astype(np.float32)
        xn = self._normalise(x)
        n = xn.shape[0]
        r = np.random.RandomState(self.seed + 1)
        xb = self.rt.alloc(xn.nbytes)
        tb = self.rt.alloc(y.nbytes)
        losses = []
        try:
            xp, tp = xb.device_ptr(), tb.device_ptr()
            steps_per_epoch = max(1, n // batch)
            total = epochs * steps_per_epoch
            step = 0
            for ep in range(epochs):
                perm = r.permutation(n)
                self.rt.upload(xb, xn[perm])
                self.rt.upload(tb, y[perm])
                ep_loss = 0.0
                for s in range(steps_per_epoch):
                    rate = lr * (lr_final / lr) ** (step / max(1, total - 1))
                    last = s == steps_per_epoch - 1
                    b = batch if s < steps_per_epoch - 1 else n - s * batch
                    loss = self.net.train_step(xp + 4 * N_FEATURES * s * batch, tp + 4 * s * batch, b, rate,
                                               want_loss=last)
                    step += 1
                    if last:
                        ep_loss = loss
                losses.append(ep_loss)
                if log:
                    log("epoch %d loss %.4f" % (ep, ep_loss))
        finally:
            xb.release()
            tb.release()
        return losses

    def predict(self, x: np.ndarray, batch: int = 65536) -> np.ndarray:
        xn = self._normalise(np.asarray(x, dtype=np.float32))
        out = np.empty(xn.shape[0], dtype=np.float32)
        xb = self.rt.alloc(max(1, min(batch, xn.shape[0])) * N_FEATURES * 4)
        yb = self.rt.alloc(max(1, min(batch, xn.shape[0])) * 4)
        try:
            for i in range(0, xn.shape[0], batch):
                part = xn[i:i + batch]
                self.rt.upload(xb, part)
                self.net.forward(xb.device_ptr(), part.shape[0], yb.device_ptr())
                out[i:i + part.shape[0]] = self.rt.download(yb, part.shape[0])
        finally:
            xb.release()
            yb.release()
        return out

    def choose(self, x_program: np.ndarray) -> int:
        """Configuration with the least predicted runtime, from a [N_CONFIGS, N_FEATURES] block."""
        return int(np.argmin(self.predict(x_program)))

    def install(self):
        """Makes this model the learned tuner's (the "tuner" knob at 2)."""
        call("cc_tuner_set_model", c_handle(self.net.handle), self.mean.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
             self.inv_std.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))

    def save(self, path: str):
        np.savez(path, params=self.net.params(), mean=self.mean, inv_std=self.inv_std, dims=np.array(MODEL_DIMS))

    def load(self, path: str):
        z = np.load(path)
        if tuple(int(v) for v in z["dims"]) != MODEL_DIMS:
            raise ValueError("model file has other layer widths")
        self.net.set_params(z["params"])
        self.mean = z["mean"].astype(np.float32)
        self.inv_std = z["inv_std"].astype(np.float32)

    def close(self):
        self.net.close()


# ---------------------------------------------------------------- evaluation

def training_arrays(records: Sequence[dict], sm_count: int, relative: bool = True):
    """Features and targets of every (program, configuration) that ran.

    The target is log(ms); with ``relative`` it is taken relative to the mean
    log(ms) of the program's configurations, so the network spends its capacity
    on how the configurations of one program differ (all a choice needs)
    rather than on each program's overall scale."""
    x = feature_matrix([r["ir"] for r in records], sm_count)
    ms = np.array([r["ms"] for r in records], dtype=np.float64)
    ok = ms > 0
    lg = np.log(np.where(ok, ms, 1.0))
    if relative:
        mean = (lg * ok).sum(axis=1, keepdims=True) / np.maximum(ok.sum(axis=1, keepdims=True), 1)
        lg = lg - mean
    ok = ok.reshape(-1)
    return x[ok], lg.reshape(-1)[ok].astype(np.float32)


def regret(records: Sequence[dict], picks: Sequence[int]) -> np.ndarray:
    """t(pick) / t(exhaustive best) - 1 per program (configurations that did not run count as missing)."""
    out = []
    for rec, p in zip(records, picks):
        ms = np.array(rec["ms"], dtype=np.float64)
        ok = ms > 0
        best = ms[ok].min()
        t = ms[p] if ms[p] > 0 else np.inf
        out.append(t / best - 1.0)
    return np.array(out)


def best_fixed_config(records: Sequence[dict]) -> int:
    """The one configuration with the least total time over the records."""
    ms = np.array([r["ms"] for r in records], dtype=np.float64)
    ms = np.where(ms > 0, ms, np.inf)
    return int(np.argmin(ms.sum(axis=0)))


def evaluate(model: CostModel, records: Sequence[dict], sm_count: int, fixed: Optional[int] = None) -> dict:
    """Regret (mean, geometric-mean slowdown, median) of the learned pick, the
    default configuration and, when given, another fixed configuration; the
    summed runtime of each choice against the summed exhaustive best."""
    x = feature_matrix([r["ir"] for r in records], sm_count)
    pred = model.predict(x).reshape(len(records), N_CONFIGS)
    ms = np.array([r["ms"] for r in records], dtype=np.float64)
    pred = np.where(ms > 0, pred, np.inf)
    learned = [int(np.argmin(p)) for p in pred]
    best_total = float(np.where(ms > 0, ms, np.inf).min(axis=1).sum())

    def summary(picks):
        g = regret(records, picks)
        total = float(sum(ms[i, p] if ms[i, p] > 0 else np.inf for i, p in enumerate(picks)))
        return {"mean_regret": float(np.mean(g)), "geomean_slowdown": float(np.exp(np.mean(np.log1p(g)))) - 1.0,
                "median_regret": float(np.median(g)), "total_time_regret": total / best_total - 1.0}

    out = {"learned": summary(learned), "default": summary([DEFAULT_CONFIG] * len(records)),
           "programs": len(records)}
    if fixed is not None:
        out["best_fixed"] = summary([fixed] * len(records))
        out["best_fixed"]["config"] = fixed
    if all("std_ms" in r for r in records):
        # the runtime's tuner also times the standard generated kernel (the product's
        # default) and keeps the faster: learned = min(model's first choice, standard)
        std = np.array([r["std_ms"] for r in records], dtype=np.float64)
        pick = np.array([ms[i, p] if ms[i, p] > 0 else np.inf for i, p in enumerate(learned)])
        tuned = np.minimum(pick, std)
        best49 = np.minimum(np.where(ms > 0, ms, np.inf).min(axis=1), std)
        out["vs_standard_kernel"] = {
            "learned_speedup_geomean": float(np.exp(np.mean(np.log(std / tuned)))),
            "learned_speedup_total": float(std.sum() / tuned.sum()),
            "exhaustive_speedup_geomean": float(np.exp(np.mean(np.log(std / best49)))),
            "exhaustive_speedup_total": float(std.sum() / best49.sum()),
            "learned_regret_vs_exhaustive_geomean": float(np.exp(np.mean(np.log(tuned / best49)))) - 1.0,
            "standard_wins": int((std <= pick).sum()),
            "note": "standard = the runtime's default generated kernel; learned = the faster of the model's "
                    "first choice and the standard kernel (what the learned tuner keeps); exhaustive = the "
                    "fastest of the 48 configurations and the standard kernel"}
    return out


def use_learned_tuner(runtime, path: str = DEFAULT_MODEL) -> CostModel:
    """Loads a cost model (by default the one shipped with the library),
    installs it, and turns the learned tuner on: programs obtained from now on
    compile in their tunable form and launch in the configuration the model
    ranks fastest.  Keep the returned model alive while the tuner uses it."""
    model = CostModel(runtime)
    model.load(path)
    model.install()
    runtime.config_set("tuner", 2)
    return model
