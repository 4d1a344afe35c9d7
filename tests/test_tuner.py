"""Tuner host logic, the tuning-workload generator, the tunable forms' NVRTC
compile, and the FP64 network oracle (no GPU needed)."""

import json
import os

import numpy as np
import pytest

from compute import tuner
from oracle import mlp as omlp


def test_config_table():
    seen = set()
    for i in range(tuner.N_CONFIGS):
        c = tuner.config(i)
        assert c["block"] == (64, 128, 256, 512)[i % 4]
        assert c["vec"] == (1, 4)[(i // 4) % 2]
        assert c["ept"] == (1, 2, 4)[(i // 8) % 3]
        assert c["split"] == (1, 2)[(i // 24) % 2]
        seen.add(tuple(sorted(c.items())))
    assert len(seen) == 48
    assert tuner.config(tuner.DEFAULT_CONFIG) == {"block": 256, "vec": 1, "ept": 1, "split": 2}
    with pytest.raises(tuner._native.InvalidValue):
        tuner.config(48)


def test_generator_is_seeded_and_in_range():
    a = tuner.random_programs(40, seed=3)
    b = tuner.random_programs(40, seed=3)
    assert [p["ir"] for p in a] == [p["ir"] for p in b]
    assert [p["ir"] for p in a] != [p["ir"] for p in tuner.random_programs(40, seed=4)]
    kinds = set()
    for p in a:
        head = p["ir"].split("\n")
        out_dims = [int(v) for v in head[1].split()[2:]]
        assert len(out_dims) <= 4
        assert all(1 <= d <= 4096 for d in out_dims)
        assert p["points"] <= tuner.MAX_POINTS
        assert 1 <= len(p["params"]) <= 4
        for shape in p["params"]:
            assert int(np.prod(shape)) <= tuner.MAX_POINTS
        kinds.add(p["kind"])
    assert "ew" in kinds and "sum" in kinds


def test_features():
    progs = tuner.random_programs(6, seed=5)
    for p in progs:
        rows = np.stack([tuner.features(p["ir"], c, 152) for c in range(tuner.N_CONFIGS)])
        assert rows.shape == (48, 64) and np.all(np.isfinite(rows))
        # the program part is the same for every configuration; the configuration part differs
        assert np.all(rows[:, :44] == rows[0, :44])
        assert len({tuple(r[44:]) for r in rows}) == 48
        for c in range(48):
            cfg = tuner.config(c)
            assert rows[c, 44 + c % 4] == 1 and rows[c, 44:48].sum() == 1
            assert rows[c, 48 + (cfg["vec"] == 4)] == 1
            assert rows[c, 53 + (cfg["split"] == 2)] == 1
        assert rows[0, 0] == (1.0 if p["kind"] == "sum" else 0.0)
    m = tuner.feature_matrix([p["ir"] for p in progs], 152)
    assert m.shape == (6 * 48, 64)
    assert np.array_equal(m[48 * 2 + 7], tuner.features(progs[2]["ir"], 7, 152))


def test_tunable_forms_compile_for_sm103a():
    progs = tuner.random_programs(8, seed=11)
    secs = tuner.compile_check([p["ir"] for p in progs])
    assert secs > 0


def test_regret_helpers():
    recs = [{"ms": [2.0, 1.0, 4.0] + [5.0] * 45}, {"ms": [1.0, -1.0, 3.0] + [5.0] * 45}]
    g = tuner.regret(recs, [0, 0])
    assert np.allclose(g, [1.0, 0.0])
    g = tuner.regret(recs, [1, 1])
    assert g[0] == 0.0 and np.isinf(g[1])  # a configuration that did not run
    assert tuner.best_fixed_config(recs) == 0


def test_oracle_gradients_match_finite_differences():
    dims = (5, 7, 6, 1)
    r = np.random.RandomState(0)
    # every parameter nonzero: with zero biases a sample whose first-layer units
    # are all off puts the next pre-activation exactly on ReLU's kink
    p = tuner.init_params(dims, seed=1).astype(np.float64) + r.uniform(0.05, 0.3, size=97) * r.choice([-1, 1], 97)
    x = r.normal(size=(9, 5))
    t = r.normal(size=9)
    _, g = omlp.loss_and_gradients(p, dims, x, t)
    h = 1e-6
    for i in r.choice(p.size, 40, replace=False):
        q = p.copy()
        q[i] += h
        lp, _ = omlp.loss_and_gradients(q, dims, x, t)
        q[i] -= 2 * h
        lm, _ = omlp.loss_and_gradients(q, dims, x, t)
        assert abs((lp - lm) / (2 * h) - g[i]) <= 1e-6 * max(1.0, abs(g[i]))


def test_oracle_adam_first_step_moves_by_lr():
    p = np.zeros(4)
    g = np.array([1.0, -2.0, 0.5, 1e-3])
    q, m, v = omlp.adam_step(p, g, np.zeros(4), np.zeros(4), 1, 0.01)
    # with bias correction the first step is lr * sign(g) (up to eps)
    assert np.allclose(q, -0.01 * np.sign(g), rtol=1e-4)


def test_tuning_fixture_is_well_formed():
    path = os.path.join(os.path.dirname(__file__), "golden", "tuning_gb300.jsonl")
    if not os.path.exists(path):
        pytest.skip("no timing fixture")
    recs = [json.loads(line) for line in open(path)]
    assert len(recs) >= 200
    for r in recs:
        assert len(r["ms"]) == 48
        assert any(v > 0 for v in r["ms"])


def test_shipped_cost_model_file():
    if not os.path.exists(tuner.DEFAULT_MODEL):
        pytest.skip("no shipped cost model")
    z = np.load(tuner.DEFAULT_MODEL)
    assert tuple(int(v) for v in z["dims"]) == tuner.MODEL_DIMS
    n = sum(k * m + m for k, m in zip(tuner.MODEL_DIMS[:-1], tuner.MODEL_DIMS[1:]))
    assert z["params"].shape == (n,) and np.all(np.isfinite(z["params"]))
    assert z["mean"].shape == (64,) and z["inv_std"].shape == (64,)


def test_evaluation_against_the_standard_kernel():
    """With the standard generated kernel's time in each record, the learned
    tuner's result is the faster of the model's first choice and that kernel
    (what the runtime keeps), compared with the standard kernel and with the
    fastest of the 48 configurations and the standard kernel."""
    progs = tuner.random_programs(4, seed=9)
    recs = []
    for k, p in enumerate(progs):
        rec = dict(p)
        ms = np.full(48, 2.0)
        ms[5] = 1.0           # the fastest configuration
        rec["ms"] = list(ms)
        rec["std_ms"] = [1.5, 0.5, 2.0, 4.0][k]  # the standard kernel: slower, faster, equal, slower
        recs.append(rec)

    class PicksConfigZero:
        def predict(self, x):
            out = np.ones(x.shape[0], dtype=np.float32)
            out[::48] = 0.0  # configuration 0 of every program (2.0 ms)
            return out

    res = tuner.evaluate(PicksConfigZero(), recs, 152)
    v = res["vs_standard_kernel"]
    tuned = np.array([1.5, 0.5, 2.0, 2.0])
    std = np.array([1.5, 0.5, 2.0, 4.0])
    best = np.array([1.0, 0.5, 1.0, 1.0])
    assert v["learned_speedup_total"] == pytest.approx(std.sum() / tuned.sum())
    assert v["learned_speedup_geomean"] == pytest.approx(np.exp(np.mean(np.log(std / tuned))))
    assert v["exhaustive_speedup_total"] == pytest.approx(std.sum() / best.sum())
    assert v["learned_regret_vs_exhaustive_geomean"] == pytest.approx(np.exp(np.mean(np.log(tuned / best))) - 1)
    assert v["standard_wins"] == 3
