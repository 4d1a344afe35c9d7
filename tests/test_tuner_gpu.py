"""The tuner on the GPU: every launch configuration of a program's tunable
form computes what the program computes; the network's kernels give the FP64
oracle's gradients and Adam steps; a network trained on GB300 timings picks
faster configurations than the fixed default; the runtime's tuner modes."""

import json
import os

import numpy as np
import pytest

from compute import tuner
from oracle import interp, mlp as omlp

pytestmark = pytest.mark.gpu


def _inputs(rt, program, seed):
    r = np.random.RandomState(seed)
    arrays, bufs = [], []
    for shape in program["params"]:
        a = r.uniform(0.1, 2.0, size=int(np.prod(shape))).astype(np.float32)
        b = rt.alloc(max(1, a.size) * 4)
        rt.upload(b, a)
        arrays.append(a)
        bufs.append(b)
    return arrays, bufs


def _same(a, b):
    nan = np.isnan(a)
    return np.array_equal(nan, np.isnan(b)) and np.array_equal(a[~nan].view(np.int32), b[~nan].view(np.int32))


def test_every_configuration_computes_the_program(cuda_device):
    rt = cuda_device.runtime
    progs = tuner.random_programs(24, seed=21, max_points=1 << 18, max_dim=700)
    ts = tuner.TuneSet(rt, [p["ir"] for p in progs])
    try:
        for k, p in enumerate(progs):
            arrays, bufs = _inputs(rt, p, k)
            n_out = 1 if p["kind"] == "sum" else p["points"]
            std = rt.alloc(max(1, n_out) * 4)
            rt.launch(rt.program(p["ir"]), bufs, std)
            want = rt.download(std, n_out)
            values = interp.evaluate(p["ir"], arrays)
            if p["kind"] != "sum" and not any(f"u {op}" in p["ir"] for op in ("exp", "log", "tanh")):
                assert _same(want, values), k  # without transcendentals the kernel is the oracle's bits
            out = rt.alloc(max(1, n_out) * 4)
            ptrs = [b.device_ptr() for b in bufs] + [out.device_ptr()]
            for c in range(tuner.N_CONFIGS):
                rt.upload(out, np.full(max(1, n_out), np.nan, np.float32))
                ts.launch(k, ptrs, c)
                got = rt.download(out, n_out)
                if p["kind"] == "sum":
                    exact = interp.exact_sum(values.astype(np.float64))
                    if np.isfinite(exact):
                        tol = 4 * np.sqrt(values.size) * 2.0 ** -24 * max(np.abs(values).sum(), 1e-30)
                        assert abs(float(got[0]) - exact) <= tol, (k, c)
                else:
                    assert _same(got, want), (k, c)
            for b in bufs + [std, out]:
                b.release()
    finally:
        ts.close()


def test_timing_reports_every_configuration(cuda_device):
    rt = cuda_device.runtime
    progs = tuner.random_programs(3, seed=5, max_points=1 << 20)
    ts = tuner.TuneSet(rt, [p["ir"] for p in progs])
    try:
        for k, p in enumerate(progs):
            _, bufs = _inputs(rt, p, k)
            out = rt.alloc(max(1, p["points"]) * 4)
            ms = ts.time(k, [b.device_ptr() for b in bufs] + [out.device_ptr()], reps=3)
            assert ms.shape == (48,) and np.all(ms > 0) and np.all(ms < 1000)
            for b in bufs + [out]:
                b.release()
    finally:
        ts.close()


def test_network_gradients_match_the_fp64_oracle(cuda_device):
    rt = cuda_device.runtime
    dims = (64, 256, 256, 256, 1)
    net = tuner.Mlp(rt, dims, seed=3)
    r = np.random.RandomState(0)
    p = net.params().astype(np.float64)
    p += r.uniform(0.01, 0.05, p.size) * r.choice([-1, 1], p.size)  # nonzero biases
    net.set_params(p.astype(np.float32))
    p = net.params().astype(np.float64)
    batch = 300  # not a multiple of the 64-row tile
    x = r.normal(size=(batch, 64)).astype(np.float32)
    t = r.normal(size=batch).astype(np.float32)
    xb, tb = rt.alloc(x.nbytes), rt.alloc(t.nbytes)
    rt.upload(xb, x)
    rt.upload(tb, t)
    loss, g = net.gradients(xb.device_ptr(), tb.device_ptr(), batch)
    want_loss, want = omlp.loss_and_gradients(p, dims, x.astype(np.float64), t.astype(np.float64))
    assert abs(loss - want_loss) <= 1e-5 * abs(want_loss)
    off = 0
    for k, n in zip(dims[:-1], dims[1:]):
        for size in (k * n, n):
            a, b = g[off:off + size].astype(np.float64), want[off:off + size]
            assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b), (k, n, size)
            off += size
    # forward alone gives the oracle's outputs
    yb = rt.alloc(batch * 4)
    net.forward(xb.device_ptr(), batch, yb.device_ptr())
    y = rt.download(yb, batch)
    want_y, _ = omlp.forward(p, dims, x.astype(np.float64))
    assert np.max(np.abs(y - want_y)) <= 1e-4 * max(1.0, np.max(np.abs(want_y)))
    # two Adam steps match the oracle's
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    q = p.copy()
    for step in (1, 2):
        _, gq = omlp.loss_and_gradients(q, dims, x.astype(np.float64), t.astype(np.float64))
        q, m, v = omlp.adam_step(q, gq, m, v, step, 1e-3)
        net.train_step(xb.device_ptr(), tb.device_ptr(), batch, 1e-3)
    got = net.params().astype(np.float64)
    assert np.linalg.norm(got - q) <= 1e-3 * np.linalg.norm(q - p)
    for b in (xb, tb, yb):
        b.release()
    net.close()


def _fixture():
    path = os.path.join(os.path.dirname(__file__), "golden", "tuning_gb300.jsonl")
    if not os.path.exists(path):
        pytest.skip("no timing fixture")
    return [json.loads(line) for line in open(path)]


def test_learned_tuner_beats_the_default_on_held_out_programs(cuda_device):
    recs = _fixture()
    split = int(len(recs) * 0.8)
    train, test = recs[:split], recs[split:]
    sm = cuda_device.runtime.device_info()["sm_count"]
    x, y = tuner.training_arrays(train, sm)
    model = tuner.CostModel(cuda_device.runtime, seed=0)
    losses = model.fit(x, y, epochs=40, batch=2048, lr=2e-3, lr_final=1e-4)
    assert losses[-1] < losses[0]
    res = tuner.evaluate(model, test, sm, fixed=tuner.best_fixed_config(train))
    print(json.dumps(res))
    assert res["learned"]["total_time_regret"] < res["default"]["total_time_regret"]
    assert res["learned"]["geomean_slowdown"] < res["default"]["geomean_slowdown"]
    model.close()


def test_runtime_tuner_modes(cuda_device):
    rt = cuda_device.runtime
    progs = tuner.random_programs(4, seed=8, max_points=1 << 20)
    model = tuner.CostModel(rt, seed=0)
    recs = _fixture() if os.path.exists(os.path.join(os.path.dirname(__file__), "golden", "tuning_gb300.jsonl")) else None
    if recs:
        x, y = tuner.training_arrays(recs[:200], rt.device_info()["sm_count"])
        model.fit(x, y, epochs=5, batch=2048)
    try:
        for k, p in enumerate(progs):
            arrays, bufs = _inputs(rt, p, k)
            n_out = 1 if p["kind"] == "sum" else p["points"]
            ref = rt.alloc(max(1, n_out) * 4)
            rt.launch(rt.program(p["ir"]), bufs, ref)
            want = rt.download(ref, n_out)
            for mode in (1, 2):
                rt.config_set("tuner", mode)
                if mode == 2:
                    model.install()
                prog = rt.program(p["ir"])
                out = rt.alloc(max(1, n_out) * 4)
                rt.launch(prog, bufs, out)
                got = rt.download(out, n_out)
                choice = rt.tuner_choice(prog)
                assert 0 <= choice <= 48  # 48: the standard generated kernel won
                if p["kind"] == "sum":
                    assert np.allclose(got, want, rtol=1e-5, equal_nan=True)
                else:
                    assert _same(got, want), (k, mode)
                out.release()
            rt.config_set("tuner", 0)
            for b in bufs + [ref]:
                b.release()
    finally:
        rt.config_set("tuner", 0)
        model.close()


def test_shipped_model_drives_the_learned_tuner(cuda_device):
    if not os.path.exists(tuner.DEFAULT_MODEL):
        pytest.skip("no shipped cost model")
    rt = cuda_device.runtime
    model = tuner.use_learned_tuner(rt)
    try:
        progs = tuner.random_programs(3, seed=17, max_points=1 << 20)
        for k, p in enumerate(progs):
            _, bufs = _inputs(rt, p, k)
            n_out = 1 if p["kind"] == "sum" else p["points"]
            out = rt.alloc(max(1, n_out) * 4)
            prog = rt.program(p["ir"])
            rt.launch(prog, bufs, out)
            assert 0 <= rt.tuner_choice(prog) <= 48
            rt.config_set("tuner", 0)
            ref = rt.alloc(max(1, n_out) * 4)
            rt.launch(rt.program(p["ir"]), bufs, ref)
            got, want = rt.download(out, n_out), rt.download(ref, n_out)
            if p["kind"] == "sum":
                assert np.allclose(got, want, rtol=1e-5, equal_nan=True)
            else:
                assert _same(got, want)
            rt.config_set("tuner", 2)
            for b in bufs + [out, ref]:
                b.release()
    finally:
        rt.config_set("tuner", 0)
        model.close()


def test_the_tuned_choice_is_never_slower_than_the_standard_kernel(cuda_device):
    """The tuner times the standard generated kernel beside the tunable form's
    configurations (exhaustive: all 48; learned: the model's first choice), so
    the kernel a tuned program runs is at most as slow as the standard one, up
    to timing noise."""
    rt = cuda_device.runtime
    progs = tuner.random_programs(6, seed=23, max_points=1 << 22)
    try:
        for k, p in enumerate(progs):
            _, bufs = _inputs(rt, p, k)
            n_out = 1 if p["kind"] == "sum" else p["points"]
            out = rt.alloc(max(1, n_out) * 4)
            std = rt.program(p["ir"])
            rt.config_set("tuner", 1)
            tuned = rt.program(p["ir"])
            rt.launch(tuned, bufs, out)
            choice = rt.tuner_choice(tuned)
            rt.config_set("tuner", 0)
            assert 0 <= choice <= 48

            def median_ms(prog):
                times = []
                for _ in range(7):
                    rt.synchronize()
                    e0 = rt.event()
                    rt.launch(prog, bufs, out)
                    e1 = rt.event()
                    rt.event_wait(e1)
                    times.append(rt.event_elapsed_ms(e0, e1))
                    rt.event_release(e0)
                    rt.event_release(e1)
                return sorted(times)[3]

            t_std, t_tuned = median_ms(std), median_ms(tuned)
            assert t_tuned <= 1.25 * t_std + 0.003, (k, choice, t_tuned, t_std)
            for b in bufs + [out]:
                b.release()
    finally:
        rt.config_set("tuner", 0)
