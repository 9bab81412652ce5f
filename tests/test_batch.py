"""Many tensors in one persistent launch (btc_batch_*), with and without the
epoch captured as a CUDA graph: each tensor's test RMSE tracks the same
tensor trained on its own."""
import numpy as np
import pytest

import btc_gpu as bg

pytestmark = pytest.mark.gpu

SPECS = [(800, 600, 500, 60000, 8), (2000, 300, 900, 150000, 16), (500, 500, 500, 40000, 32),
         (3000, 1000, 200, 90000, 16), (1200, 1200, 1200, 120000, 8)]


def _tensor(i, spec, dtype):
    I, J, K, nnz, R = spec
    tx, tv, sx, sv = bg.gen_tensor(I, J, K, nnz, zipf=(1.1, 1.1, 1.1), gt_rank=8, noise_std=0.01, seed=100 + i)
    tx, tv = bg.shuffle(tx, tv)
    cfg = bg.config(I=I, J=J, K=K, rank=R, lr=0.01, reg=0.01, block_s=1024, mode=bg.STAGED, dtype=dtype,
                    resident_blocks=-1)
    s = bg.Schedule(cfg, tx)
    rng = np.random.default_rng(i)
    init = [rng.uniform(0.0, 0.1, (n, R)) for n in (I, J, K)]
    return cfg, s, (tx, tv, sx, sv), init


@pytest.mark.parametrize("dtype", [bg.F32, bg.BF16])
@pytest.mark.parametrize("graph", [False, True])
def test_batch_tracks_single_tensor_runs(dtype, graph):
    tensors = [_tensor(i, sp, dtype) for i, sp in enumerate(SPECS)]
    alone, batched = [], []
    for cfg, s, data, init in tensors:
        for lst in (alone, batched):
            c = bg.Context(cfg, s, *data)
            for m in range(3):
                c.set_factors(m, init[m])
            lst.append(c)
    for c in alone:
        c.train_epochs(3)
    b = bg.Batch(batched)
    st = b.train_epochs(3, graph=graph)
    assert st.device_status == 0
    assert st.updates > 0 and st.launches >= 3
    for ca, cb in zip(alone, batched):
        ra, rb = ca.eval(bg.TEST).rmse, cb.eval(bg.TEST).rmse
        assert abs(ra - rb) / ra <= 2e-3, (ra, rb)
    b.close()
