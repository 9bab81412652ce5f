"""The factor check the GPU parity tests apply (factor_check.py), exercised on
the CPU with the oracle alone: an epoch agrees with itself, a no-op epoch and
an epoch at half the rate (or one that drops a mode's updates) are rejected,
and stochastically rounded BF16 copies of the oracle's result pass the BF16
form of the check while their unrounded movement is lost in a no-op."""
import numpy as np

import goldens
import oracle
from factor_check import agreement, bf16_ulp_residual, check_bf16, check_fp


def _epochs(case="zipf13_6k", R=16, lr=0.01, reg=0.01):
    c = goldens.Case(case)
    I, J, K = c.dims
    xyz, val = c.shuffled, c.shuffled_values()
    rng = np.random.default_rng(3)
    f0 = [rng.uniform(0.0, 0.1, (n, R)) for n in (I, J, K)]
    s = oracle.Schedule(xyz, I, J, K, c.meta["block_s"], c.meta["parallel_sequence_size"])
    ref = [m.copy() for m in f0]
    half = [m.copy() for m in f0]
    s.sgd_epoch(val, R, lr, reg, *ref)
    s.sgd_epoch(val, R, lr / 2, reg, *half)
    return f0, ref, half


def test_check_accepts_the_oracle_and_rejects_the_controls():
    f0, ref, half = _epochs()
    assert check_fp(ref, ref, f0)[0]
    ag = agreement(ref, ref, f0)
    assert all(d == 0.0 and abs(s - 1.0) < 1e-12 for d, s in ag)
    assert not check_fp(f0, ref, f0)[0]
    assert not check_fp(half, ref, f0)[0]
    dropped = [ref[0], ref[1], f0[2]]  # mode C never updated
    assert not check_fp(dropped, ref, f0)[0]
    assert not check_bf16(f0, ref, f0)[0] and not check_bf16(half, ref, f0)[0]
    slopes = [s for _, s in agreement(half, ref, f0)]
    assert all(0.4 < s < 0.6 for s in slopes), slopes


def test_bf16_form_accepts_stochastically_rounded_results():
    f0, ref, half = _epochs()
    rng = np.random.default_rng(9)

    def sr_bf16(x):
        b = x.astype(np.float32).view(np.uint32).astype(np.uint64)
        b = (b + rng.integers(0, 1 << 16, size=b.shape, dtype=np.uint64)) & 0xFFFF0000
        return b.astype(np.uint32).view(np.float32).astype(np.float64)

    q0 = [sr_bf16(m) for m in f0]
    got = [sr_bf16(m) for m in ref]
    # the starting point as the device would store it, the oracle from there
    ok, why = check_bf16(got, ref, f0)
    assert ok, why
    assert bf16_ulp_residual(got, ref) < 1.0
    assert not check_bf16(q0, ref, f0)[0]
