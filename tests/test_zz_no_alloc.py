"""The allocation-free error sums agree with the context's own evaluation.

Callers that cannot call cudaMalloc -- hosts whose framework owns every
device allocation, allocation-free real-time loops -- use btc_eval_sums_noalloc,
whose only scratch is a static device array inside the library.  The inputs
and outputs here are device buffers the test allocates itself (with torch);
the entry point allocates nothing.  Two calls in a row share that scratch
array, so both are checked.  This file is collected last so that a failure
here leaves every other test already run.
"""
import numpy as np
import pytest

import btc_gpu as bg

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

ERR_RANGE = 8


def _context(dtype, R):
    I, J, K = 300, 200, 100
    tx, tv, sx, sv = bg.gen_tensor(I, J, K, 40000, zipf=(1.1, 1.1, 1.1), gt_rank=4, seed=11)
    tx, tv = bg.shuffle(tx, tv)
    cfg = bg.config(I=I, J=J, K=K, rank=R, lr=0.01, reg=0.01, block_s=256, dtype=dtype, mode=bg.HOGWILD,
                    resident_blocks=-1)
    sched = bg.Schedule(cfg, tx)
    ctx = bg.Context(cfg, sched, tx, tv, sx, sv)
    rng = np.random.default_rng(5)
    for m, n in enumerate((I, J, K)):
        ctx.set_factors(m, rng.uniform(0.0, 0.1, (n, R)))
    ctx.train_epoch()
    return ctx, sx, sv, [ctx.get_factors(m) for m in range(3)]


@pytest.mark.parametrize("dtype,R,rel", [(bg.F64, 16, 1e-12), (bg.F32, 32, 1e-6), (bg.F32, 5, 1e-6)])
def test_noalloc_sums_match_eval(dtype, R, rel):
    ctx, sx, sv, F = _context(dtype, R)
    want = ctx.eval(bg.TEST)
    dev = torch.device("cuda", 0)
    tdt = torch.float64 if dtype == bg.F64 else torch.float32
    xyz = torch.from_numpy(np.ascontiguousarray(sx, np.int32)).to(dev)
    val = torch.from_numpy(np.ascontiguousarray(sv, np.float64)).to(dev)
    fac = [torch.from_numpy(np.ascontiguousarray(f)).to(device=dev, dtype=tdt).contiguous() for f in F]
    sums = torch.zeros(3, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    fn = bg.lib().btc_eval_sums_noalloc
    for call in range(2):
        sums.fill_(-1.0)
        st = fn(xyz.data_ptr(), val.data_ptr(), len(sv), fac[0].data_ptr(), fac[1].data_ptr(),
                fac[2].data_ptr(), dtype, R, R, sums.data_ptr(), stream.cuda_stream)
        assert st == 0, (call, st)
        torch.cuda.synchronize(dev)
        got = sums.cpu().numpy()
        assert got[0] == pytest.approx(want.sse, rel=rel), call
        assert got[1] == pytest.approx(want.sae, rel=rel), call
        assert got[2] == pytest.approx(want.ref2, rel=1e-12), call
    ctx.close()


def test_noalloc_rejects_sizes_beyond_scratch():
    dev = torch.device("cuda", 0)
    xyz = torch.zeros((1, 3), dtype=torch.int32, device=dev)
    val = torch.zeros(1, dtype=torch.float64, device=dev)
    fac = torch.zeros((1, 4), dtype=torch.float32, device=dev)
    sums = torch.full((3,), 7.0, dtype=torch.float64, device=dev)
    st = bg.lib().btc_eval_sums_noalloc(xyz.data_ptr(), val.data_ptr(), bg.NOALLOC_MAX_ENTRIES + 1,
                                        fac.data_ptr(), fac.data_ptr(), fac.data_ptr(), bg.F32, 4, 4,
                                        sums.data_ptr(), None)
    assert st == ERR_RANGE
    torch.cuda.synchronize(dev)
    assert sums.cpu().tolist() == [7.0, 7.0, 7.0]  # nothing was launched


def test_noalloc_padded_rows_and_empty_input():
    """Rows stored with a stride above the rank (padding columns that must not
    enter the dot products), and n = 0, which writes three zeros."""
    R, stride = 12, 16
    ctx, sx, sv, F = _context(bg.F32, R)
    want = ctx.eval(bg.TEST)
    dev = torch.device("cuda", 0)
    xyz = torch.from_numpy(np.ascontiguousarray(sx, np.int32)).to(dev)
    val = torch.from_numpy(np.ascontiguousarray(sv, np.float64)).to(dev)
    fac = []
    for f in F:
        p = np.full((f.shape[0], stride), 1e3, np.float32)  # padding that would spoil any dot it entered
        p[:, :R] = f
        fac.append(torch.from_numpy(p).to(dev))
    sums = torch.full((3,), -1.0, dtype=torch.float64, device=dev)
    fn = bg.lib().btc_eval_sums_noalloc
    st = fn(xyz.data_ptr(), val.data_ptr(), len(sv), fac[0].data_ptr(), fac[1].data_ptr(), fac[2].data_ptr(),
            bg.F32, R, stride, sums.data_ptr(), None)
    assert st == 0
    torch.cuda.synchronize(dev)
    got = sums.cpu().numpy()
    assert got[0] == pytest.approx(want.sse, rel=1e-6)
    assert got[1] == pytest.approx(want.sae, rel=1e-6)
    sums.fill_(-1.0)
    st = fn(xyz.data_ptr(), val.data_ptr(), 0, fac[0].data_ptr(), fac[1].data_ptr(), fac[2].data_ptr(),
            bg.F32, R, stride, sums.data_ptr(), None)
    assert st == 0
    torch.cuda.synchronize(dev)
    assert sums.cpu().tolist() == [0.0, 0.0, 0.0]
    ctx.close()
