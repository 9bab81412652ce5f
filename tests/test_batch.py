"""Many tensors in one persistent launch (btc_batch_*), with and without the
epoch captured as a CUDA graph: after one batched epoch every tensor's
factors have moved as the serial FP64 oracle moves them (the factor check of
factor_check.py: deviation and slope against the oracle's change, with a
no-op and a half-rate epoch failing the same check)."""
import numpy as np
import pytest

import btc_gpu as bg
import oracle
from factor_check import check_bf16, check_fp

pytestmark = pytest.mark.gpu

LR, REG = 0.01, 0.01
SPECS = [(800, 600, 500, 60000, 8), (2000, 300, 900, 150000, 16), (500, 500, 500, 40000, 32),
         (3000, 1000, 200, 90000, 16), (1200, 1200, 1200, 120000, 8)]


def _tensor(i, spec, dtype):
    I, J, K, nnz, R = spec
    tx, tv, sx, sv = bg.gen_tensor(I, J, K, nnz, zipf=(1.1, 1.1, 1.1), gt_rank=8, noise_std=0.01, seed=100 + i)
    tx, tv = bg.shuffle(tx, tv)
    cfg = bg.config(I=I, J=J, K=K, rank=R, lr=LR, reg=REG, block_s=1024, mode=bg.STAGED, dtype=dtype,
                    resident_blocks=-1)
    s = bg.Schedule(cfg, tx)
    rng = np.random.default_rng(i)
    init = [rng.uniform(0.0, 0.1, (n, R)) for n in (I, J, K)]
    return cfg, s, (tx, tv, sx, sv), init


@pytest.mark.parametrize("dtype", [bg.F32, bg.BF16])
@pytest.mark.parametrize("graph", [False, True])
def test_batch_moves_every_tensor_like_the_oracle(dtype, graph):
    tensors = [_tensor(i, sp, dtype) for i, sp in enumerate(SPECS)]
    ctxs = []
    for cfg, s, data, init in tensors:
        c = bg.Context(cfg, s, *data)
        for m in range(3):
            c.set_factors(m, init[m])
        ctxs.append(c)
    start = [[c.get_factors(m) for m in range(3)] for c in ctxs]
    b = bg.Batch(ctxs)
    st = b.train_epochs(1, graph=graph)
    assert st.device_status == 0
    assert st.updates == sum(t[1].summary.scheduled_updates for t in tensors) and st.launches >= 1
    check = check_bf16 if dtype == bg.BF16 else check_fp
    for (cfg, s, data, init), c, f0 in zip(tensors, ctxs, start):
        osched = oracle.Schedule(data[0], cfg.I, cfg.J, cfg.K, 1024, 8)
        R = cfg.rank
        ref = [m.copy() for m in f0]
        half = [m.copy() for m in f0]
        osched.sgd_epoch(data[1], R, LR, REG, *ref)
        osched.sgd_epoch(data[1], R, LR / 2, REG, *half)
        got = [c.get_factors(m) for m in range(3)]
        ok, why = check(got, ref, f0)
        assert ok, (R, why)
        assert not check(f0, ref, f0)[0] and not check(half, ref, f0)[0]
    b.close()
    for c in ctxs:
        c.close()
