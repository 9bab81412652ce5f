"""GPU parity: the CUDA path through the C ABI against the FP64 oracle.

* FP64 deterministic mode equals the serial FP64 replay of the reference
  update rule (sgd_Kernel.cu:336-351) bit for bit, epoch after epoch.
* FP32 deterministic mode: per-epoch RMSE within 1e-5 relative and factors
  within 1e-4 max relative error after one epoch (spec gates).
* Hogwild (the reference's own execution model: concurrent entries of a slot
  read rows while others add to them) agrees within a looser tolerance.
* Metrics (compute_metrics_gpu) agree with the oracle's FP64 sums.
* The timed kernels (Hogwild, staged FP32/FP64/BF16) move the factors as the
  oracle does: after one epoch their factor change matches the oracle's
  change (deviation and slope), while a no-op epoch or one at half the
  learning rate fails the same check (the check can fail).
"""
import numpy as np
import pytest

import btc_gpu as bg
import goldens
import oracle
from factor_check import check_bf16, check_fp

pytestmark = pytest.mark.gpu

LR, REG = 0.01, 0.01


def _setup(case_name, R, seed=3):
    c = goldens.Case(case_name)
    I, J, K = c.dims
    xyz = c.shuffled
    val = c.shuffled_values()
    rng = np.random.default_rng(seed)
    init = [rng.uniform(0.0, 0.1, (n, R)) for n in (I, J, K)]
    sched = oracle.Schedule(xyz, I, J, K, c.meta["block_s"], c.meta["parallel_sequence_size"])
    return c, xyz, val, init, sched


def _ctx(c, xyz, val, R, dtype, mode, test_xyz=None, test_val=None):
    I, J, K = c.dims
    cfg = bg.config(I=I, J=J, K=K, rank=R, lr=LR, reg=REG, block_s=c.meta["block_s"],
                    parallel_sequence_size=c.meta["parallel_sequence_size"], dtype=dtype, mode=mode,
                    resident_blocks=-1)
    s = bg.Schedule(cfg, xyz)
    tx = xyz if test_xyz is None else test_xyz
    tv = val if test_val is None else test_val
    return bg.Context(cfg, s, xyz, val, tx, tv)


@pytest.mark.parametrize("case_name,R", [("uniform_3k", 16), ("zipf13_6k", 16), ("zipf_bs4_dup", 8),
                                         ("cube1000_20k", 32), ("uniform_pss3", 5), ("bigdim", 100)])
def test_f64_deterministic_bit_exact(case_name, R):
    c, xyz, val, init, sched = _setup(case_name, R)
    ref = [m.copy() for m in init]
    ctx = _ctx(c, xyz, val, R, bg.F64, bg.DETERMINISTIC)
    for m in range(3):
        ctx.set_factors(m, init[m])
    for epoch in range(3):
        upd = sched.sgd_epoch(val, R, LR, REG, *ref)
        st = ctx.train_epoch()
        assert st.updates == upd
        for m in range(3):
            got = ctx.get_factors(m)
            assert np.array_equal(got, ref[m]), (epoch, m, np.abs(got - ref[m]).max())
        mt = ctx.eval(bg.TEST)
        sse, sae, r2 = oracle.metrics(xyz, val, R, *ref)
        assert mt.count == len(val)
        assert mt.sse == pytest.approx(sse, rel=1e-12)
        assert mt.sae == pytest.approx(sae, rel=1e-12)
        assert mt.ref2 == pytest.approx(r2, rel=1e-12)


@pytest.mark.parametrize("case_name,R", [("cube1000_20k", 16), ("zipf13_6k", 32), ("uniform_3k", 64)])
def test_f32_deterministic_gates(case_name, R):
    c, xyz, val, init, sched = _setup(case_name, R)
    ref = [m.copy() for m in init]
    ctx = _ctx(c, xyz, val, R, bg.F32, bg.DETERMINISTIC)
    for m in range(3):
        ctx.set_factors(m, init[m])
    for epoch in range(5):
        sched.sgd_epoch(val, R, LR, REG, *ref)
        ctx.train_epoch()
        if epoch == 0:
            for m in range(3):
                got = ctx.get_factors(m)
                rel = np.abs(got - ref[m]).max() / np.abs(ref[m]).max()
                assert rel <= 1e-4, (m, rel)
        rmse = ctx.eval(bg.TEST).rmse
        want = oracle.rmse_mae_er(xyz, val, R, *ref)[0]
        assert abs(rmse - want) / want <= 1e-5, (epoch, rmse, want)


@pytest.mark.parametrize("mode", [bg.HOGWILD, bg.STAGED])
@pytest.mark.parametrize("dtype", [bg.F32, bg.F64])
@pytest.mark.parametrize("case_name,R", [("cube1000_20k", 16), ("zipf13_6k", 32), ("zipf15_auto", 8),
                                         ("bigdim", 100)])
def test_parallel_modes_close_to_serial(case_name, R, dtype, mode):
    """Hogwild and staged runs read rows while other entries of the same
    slot update them, as the reference kernel does; they track the serial
    replay closely but not bit for bit."""
    c, xyz, val, init, sched = _setup(case_name, R)
    ref = [m.copy() for m in init]
    ctx = _ctx(c, xyz, val, R, dtype, mode)
    for m in range(3):
        ctx.set_factors(m, init[m])
    for epoch in range(5):
        sched.sgd_epoch(val, R, LR, REG, *ref)
        ctx.train_epoch()
        rmse = ctx.eval(bg.TEST).rmse
        want = oracle.rmse_mae_er(xyz, val, R, *ref)[0]
        assert abs(rmse - want) / want <= 2e-3, (epoch, rmse, want)


def test_empty_test_split_gives_nan():
    c, xyz, val, init, sched = _setup("uniform_3k", 16)
    ctx = _ctx(c, xyz, val, 16, bg.F32, bg.HOGWILD, test_xyz=np.zeros((0, 3), np.int32),
               test_val=np.zeros(0))
    m = ctx.eval(bg.TEST)
    assert m.count == 0 and np.isnan(m.rmse) and np.isnan(m.mae) and np.isnan(m.er)


@pytest.mark.parametrize("R", [1, 128])
@pytest.mark.parametrize("dtype,mode,tol", [(bg.F32, bg.HOGWILD, 2e-3), (bg.F32, bg.STAGED, 2e-3),
                                            (bg.BF16, bg.STAGED, 2e-2)])
def test_rank_extremes_close_to_serial(R, dtype, mode, tol):
    """The smallest and the largest rank the library accepts (1 and 128)
    take the same kernels' padded and widest lane shapes."""
    c, xyz, val, init, sched = _setup("zipf13_6k", R)
    ref = [m.copy() for m in init]
    ctx = _ctx(c, xyz, val, R, dtype, mode)
    for m in range(3):
        ctx.set_factors(m, init[m])
    for epoch in range(3):
        sched.sgd_epoch(val, R, LR, REG, *ref)
        st = ctx.train_epoch()
        assert st.device_status == 0
        rmse = ctx.eval(bg.TEST).rmse
        want = oracle.rmse_mae_er(xyz, val, R, *ref)[0]
        assert abs(rmse - want) / want <= tol, (epoch, rmse, want)


@pytest.mark.parametrize("dtype,mode", [(bg.F32, bg.HOGWILD), (bg.F64, bg.DETERMINISTIC), (bg.F32, bg.STAGED),
                                        (bg.BF16, bg.STAGED)])
def test_empty_train_split_epochs_are_no_ops(dtype, mode):
    """No training entries: the schedule is empty, an epoch executes no update
    and leaves the factors as they were, and the test split still evaluates."""
    c, xyz, val, init, sched = _setup("uniform_3k", 8)
    I, J, K = c.dims
    cfg = bg.config(I=I, J=J, K=K, rank=8, lr=LR, reg=REG, block_s=c.meta["block_s"], dtype=dtype, mode=mode)
    empty = np.zeros((0, 3), np.int32)
    s = bg.Schedule(cfg, empty)
    assert s.summary.num_slots == 0 and s.summary.scheduled_updates == 0
    ctx = bg.Context(cfg, s, empty, np.zeros(0), xyz, val)
    for m in range(3):
        ctx.set_factors(m, init[m])
    before = [ctx.get_factors(m) for m in range(3)]
    st = ctx.train_epochs(2)
    assert st.updates == 0 and st.device_status == 0
    for m in range(3):
        assert np.array_equal(ctx.get_factors(m), before[m])
    mt = ctx.eval(bg.TEST)
    assert mt.count == len(val) and np.isfinite(mt.rmse)
    ctx.close()


def test_factor_roundtrip_and_init():
    c, xyz, val, init, sched = _setup("uniform_3k", 24)
    for dtype in (bg.F32, bg.F64):
        ctx = _ctx(c, xyz, val, 24, dtype, bg.HOGWILD)
        for m in range(3):
            ctx.set_factors(m, init[m])
            got = ctx.get_factors(m)
            if dtype == bg.F64:
                assert np.array_equal(got, init[m])
            else:
                assert np.array_equal(got, init[m].astype(np.float32).astype(np.float64))
        ctx.init_factors(99, 0.0, 0.1)
        a1 = ctx.get_factors(0)
        ctx.init_factors(99, 0.0, 0.1)
        assert np.array_equal(a1, ctx.get_factors(0))
        assert a1.min() >= 0.0 and a1.max() < 0.1 and abs(a1.mean() - 0.05) < 0.005


@pytest.mark.parametrize("case_name,R", [("cube1000_20k", 16), ("zipf13_6k", 32), ("bigdim", 100)])
def test_bf16_staged_close_to_fp32(case_name, R):
    """BF16 storage (FP32 math, stochastic rounding, FP32 masters of the
    hottest rows) stays within 1% of the FP32 run's test RMSE."""
    c, xyz, val, init, sched = _setup(case_name, R)
    ctx32 = _ctx(c, xyz, val, R, bg.F32, bg.STAGED)
    ctx16 = _ctx(c, xyz, val, R, bg.BF16, bg.STAGED)
    for m in range(3):
        ctx32.set_factors(m, init[m])
        ctx16.set_factors(m, init[m])
    for epoch in range(5):
        st = ctx16.train_epoch()
        assert st.device_status == 0
        ctx32.train_epoch()
        r16, r32 = ctx16.eval(bg.TEST).rmse, ctx32.eval(bg.TEST).rmse
        assert abs(r16 - r32) / r32 <= 1e-2, (epoch, r16, r32)


def test_bf16_stochastic_rounding_is_unbiased():
    """Updates far below one BF16 ulp still move the rows on average: the mean
    BF16 change matches the FP32 change (round-to-nearest would lose it)."""
    R = 16
    c, xyz, val, init, sched = _setup("cube1000_20k", R)
    I, J, K = c.dims
    cfg = dict(I=I, J=J, K=K, rank=R, lr=2e-3, reg=0.0, block_s=c.meta["block_s"],
               parallel_sequence_size=c.meta["parallel_sequence_size"], mode=bg.STAGED, resident_blocks=-1)
    s = bg.Schedule(bg.config(**cfg), xyz)
    val = np.ones(len(val))  # every update pushes the same way, about 0.3 ulp per row in total
    base = [np.full((n, R), 0.0625) for n in (I, J, K)]  # exactly representable in BF16
    out = {}
    for dt in (bg.F32, bg.BF16):
        ctx = bg.Context(bg.config(dtype=dt, **cfg), s, xyz, val, xyz, val)
        for m in range(3):
            ctx.set_factors(m, base[m])
        ctx.train_epoch()
        out[dt] = [ctx.get_factors(m) - base[m] for m in range(3)]
        ctx.close()
    d32 = np.concatenate([d.ravel() for d in out[bg.F32]])
    d16 = np.concatenate([d.ravel() for d in out[bg.BF16]])
    ulp = 0.0625 * 2.0 ** -7
    assert 0 < d32.mean() < 0.5 * ulp  # the whole epoch moves a row by less than one ulp ...
    assert abs(d16.mean() - d32.mean()) <= 0.05 * d32.mean()  # ... and the BF16 rows move as much on average


def test_bf16_stochastic_rounding_per_element():
    """Every stochastic rounding draws fresh random bits, so each element's
    BF16 change follows its own FP32 change, not only the mean over elements.

    A uniform 500^3 tensor of 250k entries gives every row ~500 entries per
    epoch spread over many tiles, and padding runs some blocks in several
    slots.  Each element takes many sub-ulp increments (about 1.1 ulp in
    total).  Independent roundings leave it a Poisson-like number of ulps
    from the FP32 result: RMS about 1 ulp, and above 10 ulp with probability
    below 1e-3 over all 24k elements.  Bits shared across the updates of an
    epoch (one draw per element, or one per tile for a block visited from
    several slots) round an element the same way every time; on this tensor
    that put elements 20-40 ulp away."""
    n, R = 500, 16
    tx, _, _, _ = bg.gen_tensor(n, n, n, 250_000, gt_rank=4, train_frac=1.0, seed=7)
    val = np.ones(len(tx))  # every update pushes the same way
    cfg = dict(I=n, J=n, K=n, rank=R, lr=2e-4, reg=0.0, mode=bg.STAGED, resident_blocks=-1)
    s = bg.Schedule(bg.config(**cfg), tx)
    base = [np.full((n, R), 0.0625) for _ in range(3)]  # exactly representable in BF16
    ulp = 0.0625 * 2.0 ** -7
    out = {}
    for dt in (bg.F32, bg.BF16):
        ctx = bg.Context(bg.config(dtype=dt, **cfg), s, tx, val, tx, val)
        for m in range(3):
            ctx.set_factors(m, base[m])
        assert ctx.train_epoch().device_status == 0
        out[dt] = np.stack([ctx.get_factors(m) - base[m] for m in range(3)]) / ulp
        ctx.close()
    d32, d16 = out[bg.F32], out[bg.BF16]
    assert 0.5 < d32.mean() < 2.0 and d32.max() < 4.0  # many sub-ulp increments, about one ulp in all
    err = d16 - d32
    assert abs(d16.mean() - d32.mean()) <= 0.05 * d32.mean()
    assert np.sqrt((err ** 2).mean()) <= 1.6, np.sqrt((err ** 2).mean())
    assert np.abs(err).max() <= 10.0, np.abs(err).max()


def test_staged_stable_under_strong_regularisation_on_hot_rows():
    """Rows that decay fast relative to a tile's share of the epoch (here the
    Zipf(1.5) heads: one row holds ~38 % of mode 1's entries and sits in
    almost every stratum) take their regularisation from the row's value at
    write time.  With the tile-start snapshot, the many concurrent tiles
    stepping such a row formed delayed negative feedback that diverged to NaN
    within one epoch at lambda 0.05 on this shape (50M entries).  At lambda
    0.05 BF16 and FP32 staged follow the plain Hogwild path (the reference's
    execution model).  Stronger settings (lambda 0.2 at lr 0.01) make Hogwild
    itself diverge and are not held to any path."""
    I, J, K, R = 200_000, 2_000, 1_000_000, 32
    tx, tv, sx, sv = bg.gen_tensor(I, J, K, 10_000_000, zipf=(1.5, 0.0, 1.5), gt_rank=0, noise_std=0.0,
                                   train_frac=0.9, seed=20261207)
    bg.shuffle(tx, tv)
    rng = np.random.default_rng(5)
    init = [rng.uniform(0.0, 0.1, (n, R)) for n in (I, J, K)]
    sched = None
    out = {}
    for name, dt, md in (("bf16", bg.BF16, bg.STAGED), ("f32", bg.F32, bg.STAGED), ("plain", bg.F32, bg.HOGWILD)):
        cfg = bg.config(I=I, J=J, K=K, rank=R, lr=0.01, reg=0.05, block_s=2048, parallel_sequence_size=8,
                        dtype=dt, mode=md)
        sched = sched or bg.Schedule(cfg, tx)
        ctx = bg.Context(cfg, sched, tx, tv, sx, sv)
        for m in range(3):
            ctx.set_factors(m, init[m])
        r = []
        for _ in range(3):
            ctx.train_epoch()
            r.append(ctx.eval(bg.TEST).rmse)
        assert np.isfinite(ctx.get_factors(0)).all() and np.isfinite(ctx.get_factors(2)).all(), name
        out[name] = r
        ctx.close()
    for name in ("bf16", "f32"):
        assert np.isfinite(out[name]).all(), (name, out[name])
        assert abs(out[name][-1] - out["plain"][-1]) <= 1e-3 * out["plain"][-1], out


FACTOR_CASES = [("cube1000_20k", 16), ("zipf13_6k", 32), ("zipf15_auto", 8), ("bigdim", 100), ("uniform_3k", 16)]


def _one_epoch_vs_oracle(case_name, R, dtype, mode):
    """One GPU epoch and the serial FP64 oracle epoch (sgd_Kernel.cu:336-351)
    from the same initial factors (as the device stores them), plus the two
    controls: no update at all, and an oracle epoch at half the rate."""
    c, xyz, val, init, sched = _setup(case_name, R)
    ctx = _ctx(c, xyz, val, R, dtype, mode)
    for m in range(3):
        ctx.set_factors(m, init[m])
    start = [ctx.get_factors(m) for m in range(3)]
    ref = [m.copy() for m in start]
    half = [m.copy() for m in start]
    upd = sched.sgd_epoch(val, R, LR, REG, *ref)
    sched.sgd_epoch(val, R, LR / 2, REG, *half)
    st = ctx.train_epoch()
    assert st.updates == upd and st.device_status == 0
    got = [ctx.get_factors(m) for m in range(3)]
    ctx.close()
    return got, ref, start, half


@pytest.mark.parametrize("dtype,mode", [(bg.F32, bg.HOGWILD), (bg.F64, bg.HOGWILD), (bg.F32, bg.STAGED),
                                        (bg.F64, bg.STAGED)])
@pytest.mark.parametrize("case_name,R", FACTOR_CASES)
def test_timed_kernels_move_factors_like_the_oracle(case_name, R, dtype, mode):
    """Per mode, after one epoch: ||F - F_oracle|| <= 0.1 ||F_oracle - F_0||
    and the slope of F - F_0 on F_oracle - F_0 within 0.08 of 1.  Hogwild and
    staged runs let entries of a slot (staged: of a tile) read rows before
    other entries' updates land, as the reference kernel does, so they are
    not bit-exact; measured deviations are <= 0.044 and slopes 1.002-1.039."""
    got, ref, start, half = _one_epoch_vs_oracle(case_name, R, dtype, mode)
    ok, why = check_fp(got, ref, start)
    assert ok, why
    assert not check_fp(start, ref, start)[0]  # control: nothing moved
    assert not check_fp(half, ref, start)[0]  # control: half the step


@pytest.mark.parametrize("case_name,R", FACTOR_CASES)
def test_bf16_staged_moves_factors_like_the_oracle(case_name, R):
    """BF16 storage: each element carries about one ulp of stochastic-rounding
    noise, comparable to one epoch's movement at this rate, so the deviation
    ratio says little.  The slope of the BF16 change on the oracle's change
    is insensitive to zero-mean noise (no-op: 0, half rate: 0.5) and must lie
    within 0.15 of 1; the residual after the oracle's change must stay within
    a few ulps RMS of the oracle's values."""
    got, ref, start, half = _one_epoch_vs_oracle(case_name, R, bg.BF16, bg.STAGED)
    ok, why = check_bf16(got, ref, start)
    assert ok, why
    assert not check_bf16(start, ref, start)[0]
    assert not check_bf16(half, ref, start)[0]


@pytest.mark.parametrize("case_name,R", [("uniform_3k", 16), ("zipf13_6k", 16), ("zipf_bs4_dup", 8), ("bigdim", 100)])
def test_lockfree_f64_equals_the_serial_lockfree_rule(case_name, R):
    """The lock-free variant (tensor_LF): every block of the conflict-free
    strata once, in-place A-then-B-then-C updates without coe weights; FP64
    epochs equal the oracle's serial replay of that rule bit for bit."""
    c, xyz, val, init, sched = _setup(case_name, R)
    ref = [m.copy() for m in init]
    ctx = _ctx(c, xyz, val, R, bg.F64, bg.LOCKFREE)
    for m in range(3):
        ctx.set_factors(m, init[m])
    for epoch in range(3):
        upd = sched.lf_epoch(val, R, LR, REG, *ref)
        st = ctx.train_epoch()
        # every block once; the duplicating re-split (Q4) can leave an entry
        # in two blocks, so an epoch can hold more updates than entries
        assert st.updates == upd >= len(val) and st.device_status == 0
        for m in range(3):
            got = ctx.get_factors(m)
            assert np.array_equal(got, ref[m]), (epoch, m, np.abs(got - ref[m]).max())


@pytest.mark.parametrize("case_name,R", [("cube1000_20k", 16), ("zipf13_6k", 32)])
def test_lockfree_f32_moves_factors_like_the_oracle(case_name, R):
    c, xyz, val, init, sched = _setup(case_name, R)
    ctx = _ctx(c, xyz, val, R, bg.F32, bg.LOCKFREE)
    for m in range(3):
        ctx.set_factors(m, init[m])
    start = [ctx.get_factors(m) for m in range(3)]
    ref = [m.copy() for m in start]
    half = [m.copy() for m in start]
    sched.lf_epoch(val, R, LR, REG, *ref)
    sched.lf_epoch(val, R, LR / 2, REG, *half)
    ctx.train_epoch()
    got = [ctx.get_factors(m) for m in range(3)]
    ok, why = check_fp(got, ref, start, dev_tol=1e-3, slope_tol=1e-3)
    assert ok, why
    assert not check_fp(half, ref, start)[0]


def test_lockfree_has_no_bf16_form():
    c, xyz, val, init, sched = _setup("uniform_3k", 8)
    with pytest.raises(bg.BtcError) as e:
        _ctx(c, xyz, val, 8, bg.BF16, bg.LOCKFREE)
    assert e.value.status == 7  # BTC_ERR_UNSUPPORTED


@pytest.mark.parametrize("dtype", [bg.F32, bg.BF16])
def test_staged_stays_stable_where_the_factors_grow(dtype):
    """No regularisation and lr 0.02 on a skewed tensor: the factors grow from
    U(0, 0.1) to the data's scale within a few epochs.  Tiles that let a hot
    row take hundreds of snapshot updates diverged here; with the row bound
    (16 per tile at this rate) the staged paths stay finite and learn, as
    the plain Hogwild path does."""
    I, J, K, R = 100000, 100000, 10000, 32
    tx, tv, sx, sv = bg.gen_tensor(I, J, K, 5_000_000, zipf=(1.2, 1.2, 1.2), gt_rank=16, noise_std=0.05,
                                   train_frac=0.9, seed=23)
    tx, tv = bg.shuffle(tx, tv)
    out = {}
    for name, dt, md in (("staged", dtype, bg.STAGED), ("plain", bg.F32, bg.HOGWILD)):
        cfg = bg.config(I=I, J=J, K=K, rank=R, lr=0.02, reg=0.0, block_s=2048, parallel_sequence_size=8,
                        dtype=dt, mode=md)
        ctx = bg.Context(cfg, bg.Schedule(cfg, tx), tx, tv, sx, sv)
        ctx.init_factors(3, 0.0, 0.1)
        r0 = ctx.eval(bg.TEST).rmse
        rs = []
        for _ in range(15):
            assert ctx.train_epoch().device_status == 0
            rs.append(ctx.eval(bg.TEST).rmse)
        ctx.close()
        out[name] = (r0, rs)
        assert np.isfinite(rs).all(), (name, rs)
    r0, rs = out["staged"]
    assert rs[-1] < 0.6 * r0, out  # it learned
    assert rs[-1] < 2.0 * out["plain"][1][-1], out
