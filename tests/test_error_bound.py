"""The oracle's error bound for programs with exp/log/tanh (test infrastructure).

``oracle.interp.evaluate_with_bound`` gives, per point, how far a device whose
exp/log/tanh are within 2 ulp of correctly rounded may be from the oracle.  The
batched-program GPU test relies on it, so it is checked here against a model of
such a device: the same evaluation with every transcendental result moved by a
random number of ulps in [-2, 2].  Programs are the batched workload's
generator (3-12-node trees over {+,-,*,/,exp,log,tanh,max}, 1-4 inputs uniform
in [0.1, 2]) at small lengths.
"""

import numpy as np

from oracle import interp


def _programs():
    import bench
    from compute import Tensors
    from oracle_runtime import OracleRuntime
    d = Tensors(runtime=OracleRuntime())
    progs = bench.c4_programs(d.Tensor, seed=7, count=300, lo=256, hi=2048)
    for t, inputs in progs:
        ser = d.serialize(t.closure, t.shape)
        yield ser.text, [p.flatArray() for p in ser.params]


def test_bound_covers_a_device_within_two_ulp():
    rs = np.random.RandomState(0)
    with_transcendentals = 0
    for text, ins in _programs():
        want, bound = interp.evaluate_with_bound(text, ins)
        assert np.array_equal(np.nan_to_num(want), np.nan_to_num(interp.evaluate(text, ins)))
        if not bound.any():
            continue
        with_transcendentals += 1
        for _ in range(3):
            dev, _ = interp.evaluate_with_bound(text, ins, perturb=rs)
            nan = np.isnan(want)
            fin = ~nan & np.isfinite(want) & np.isfinite(bound) & np.isfinite(dev)
            assert np.all(np.abs(dev[fin].astype(np.float64) - want[fin]) <= bound[fin]), text
    assert with_transcendentals > 100


def test_bound_is_zero_without_transcendentals():
    text = "ccir 1 ew\no 1 4\np 1 4 00000000\nx 0 2 1 0\nb mul 1 1\nb div 2 1\nr 3\n"
    x = np.array([0.5, 1.0, 1.5, 2.0], np.float32)
    want, bound = interp.evaluate_with_bound(text, [x])
    assert not bound.any()
    assert np.array_equal(want, interp.evaluate(text, [x]))


def test_window_of_a_contiguous_program():
    text = "ccir 1 ew\no 1 6\np 1 6 00000000\nx 0 2 1 0\nu exp 1\nr 2\n"
    x = np.linspace(0.1, 2, 6).astype(np.float32)
    full = interp.evaluate(text, [x])
    part = interp.evaluate(interp.window_text(text, 3), [x[2:5]])
    assert np.array_equal(part, full[2:5])
