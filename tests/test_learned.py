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


@pytest.mark.parametrize("dtype", [bg.F32, bg.BF16])
def test_autotuner_picks_a_valid_shape_and_keeps_the_results(dtype):
    """The autotuner times lane shapes (lanes per entry x vectors per lane)
    and CTAs per SM on the context's own tiles and keeps the fastest; the
    chosen shape must cover the rank, and an epoch after tuning must still
    move the factors as the serial FP64 oracle's epoch does."""
    import oracle
    from factor_check import check_bf16, check_fp

    I, J, K, R = 20000, 20000, 5000, 32
    tx, tv, sx, sv = bg.gen_tensor(I, J, K, 600000, zipf=(1.2, 1.2, 1.2), gt_rank=8, seed=5)
    tx, tv = bg.shuffle(tx, tv)
    cfg = bg.config(I=I, J=J, K=K, rank=R, lr=0.01, reg=0.01, block_s=2048, mode=bg.STAGED, dtype=dtype,
                    resident_blocks=-1)
    s = bg.Schedule(cfg, tx)
    ctx = bg.Context(cfg, s, tx, tv, sx, sv)
    ctx.init_factors(1, 0.0, 0.1)
    r = ctx.autotune(1)
    assert r.candidates >= 2 and r.lanes_per_entry in (1, 2, 4, 8, 16, 32) and r.vectors_per_lane >= 1
    assert r.lanes_per_entry * r.vectors_per_lane * 4 >= R and r.ctas_per_sm >= 2
    assert 0 < r.best_ms <= r.default_ms
    start = [ctx.get_factors(m) for m in range(3)]
    ref = [m.copy() for m in start]
    osched = oracle.Schedule(tx, I, J, K, 2048, 8)
    osched.sgd_epoch(tv, R, 0.01, 0.01, *ref)
    assert ctx.train_epoch().device_status == 0
    got = [ctx.get_factors(m) for m in range(3)]
    ok, why = (check_bf16 if dtype == bg.BF16 else check_fp)(got, ref, start)
    assert ok, why
    ctx.close()


def test_trained_model_gains_over_the_learned_blocking_without_it():
    """The learned blocking with its split axes chosen by the block cost model
    (trained on block timings the context records) against the same builder
    with the axes taken in turn: both schedule every train entry once, and
    the model's blocking runs an epoch faster (measured on the GB300: 11.2
    vs 13.5 ms on the 45M-entry skewed C2 tensor, 6.1 vs 7.5 ms on a
    20M-entry C3-shaped one)."""
    I, J, K, R = 100000, 100000, 10000, 32
    tx, tv, sx, sv = bg.gen_tensor(I, J, K, 10_000_000, zipf=(1.2, 1.2, 1.2), gt_rank=16, noise_std=0.05,
                                   train_frac=0.9, seed=21)
    tx, tv = bg.shuffle(tx, tv)
    cfg = bg.config(I=I, J=J, K=K, rank=R, lr=0.005, reg=0.02, block_s=2048, parallel_sequence_size=8,
                    mode=bg.STAGED, dtype=bg.BF16)
    ref = bg.Context(cfg, bg.Schedule(cfg, tx), tx, tv, sx, sv)
    ref.init_factors(1, 0.0, 0.1)
    ref.train_epochs(2)
    f, y = ref.block_profile()
    ref.close()
    assert len(y) > 1000 and np.isfinite(f).all() and np.isfinite(y).all()
    model = bg.MLP(n_in=bg.BLOCK_FEATURES, seed=7)
    loss = model.train(f, y, 400)
    assert 1.0 - loss / float(np.var(y)) > 0.8  # the model explains most of the block-time variance
    times = {}
    for name, m in (("model", model), ("turns", None)):
        s = bg.Schedule(cfg, tx, learned=True, model=m)
        assert s.summary.scheduled_updates == len(tv)
        ctx = bg.Context(cfg, s, tx, tv, sx, sv)
        ctx.init_factors(1, 0.0, 0.1)
        ctx.train_epochs(2)
        times[name] = min(ctx.train_epochs(1).kernel_ms for _ in range(5))
        assert np.isfinite(ctx.eval(bg.TEST).rmse)
        ctx.close()
    model.close()
    assert times["model"] < times["turns"], times
