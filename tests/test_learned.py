"""The learned cost model: its CUDA gradients against the FP64 oracle, its
training, and the work-unit packing it proposes for the staged kernel."""
import numpy as np
import pytest

import btc_gpu as bg
import mlp_oracle

pytestmark = pytest.mark.gpu


def test_mlp_gradient_matches_oracle():
    rng = np.random.default_rng(0)
    m = bg.MLP(10, seed=7)
    x = rng.normal(0, 1, (3000, 10)).astype(np.float32)
    y = rng.normal(0, 1, 3000).astype(np.float32)
    g, loss = m.gradient(x, y)
    want, wloss = mlp_oracle.gradient(m.params(), x, y)
    assert loss == pytest.approx(wloss, rel=1e-4)
    assert np.linalg.norm(g - want) <= 1e-3 * np.linalg.norm(want)
    assert np.abs(g - want).max() <= 1e-3 * np.abs(want).max()


def test_mlp_learns_a_smooth_cost():
    rng = np.random.default_rng(1)
    x = rng.uniform(0, 1, (4000, 10)).astype(np.float32)
    y = (1.5 + 2.0 * x[:, 0] + np.log1p(5 * x[:, 1]) - x[:, 2] * x[:, 3]).astype(np.float32)
    m = bg.MLP(10, seed=3)
    loss = m.train(x, y, steps=600, lr=3e-3)
    assert loss < 0.05 * y.var()
    pred = m.predict(x)
    assert np.abs(pred - y).mean() < 0.15


def test_learned_work_units_are_kept_only_if_faster():
    tx, tv, sx, sv = bg.gen_tensor(20000, 20000, 5000, 600000, zipf=(1.2, 1.2, 1.2), gt_rank=8, seed=5)
    tx, tv = bg.shuffle(tx, tv)
    cfg = bg.config(I=20000, J=20000, K=5000, rank=32, lr=0.005, reg=0.02, block_s=2048, mode=bg.STAGED)
    s = bg.Schedule(cfg, tx)
    ctx = bg.Context(cfg, s, tx, tv, sx, sv)
    ctx.init_factors(1, 0.0, 0.1)
    ctx.train_epochs(2)
    model = bg.MLP()
    r = ctx.learn_work_units(model, train_steps=300, trial_epochs=3)
    assert r.samples > 100 and r.units > 0
    assert r.model_r2 > 0.3
    assert r.kept == (1 if r.learned_ms < r.plain_ms else 0)
    # training goes on with whichever packing was kept
    before = ctx.eval(bg.TEST).rmse
    ctx.train_epochs(2)
    assert np.isfinite(ctx.eval(bg.TEST).rmse) and abs(ctx.eval(bg.TEST).rmse - before) < 0.05 * before
    print("learned units: plain %.3f ms, learned %.3f ms, kept %d, R2 %.3f, units %d" %
          (r.plain_ms, r.learned_ms, r.kept, r.model_r2, r.units))
