"""The oracle restates the reference's blocking and schedule bit-exactly.

Pinned against fixtures produced by the reference's own block.cu
(tests/golden/make_golden.py): block ids, levels, nnz, stratum/group
membership and order, coe weights and per-slot entry order.
"""
import numpy as np
import pytest

import goldens
import oracle

CASES = goldens.cases()


@pytest.fixture(scope="module", params=CASES)
def case(request):
    c = goldens.Case(request.param)
    s = oracle.Schedule(c.shuffled, *c.dims, c.meta["block_s"], c.meta["parallel_sequence_size"])
    return c, s


def test_blocks_match_reference(case):
    c, s = case
    assert c.header["num_block_total"] == s.nblocks
    nonempty = [b for b in range(s.nblocks) if s.block_nnz[b] > 0]
    assert len(nonempty) == len(c.blocks)
    for b, rb in zip(nonempty, c.blocks):
        assert rb["id"] == b
        assert rb["nnz"] == int(s.block_nnz[b])
        assert rb["levels"] == tuple(int(v) for v in s.block_levels[b])
        assert rb["ids"] == tuple(s.id_string(b, a) for a in range(3))


def test_strata_and_groups_match_reference(case):
    c, s = case
    assert c.header["conflict_free_sequence_count"] == s.nstrata
    assert c.header["conflict_free_max_parallel_blocks"] == s.max_parallel_cf
    assert c.header["target_gpu_blocks"] == s.target
    assert [q["ids"] for q in c.seqs] == s.groups
    assert c.schedule["num_parallel"] == s.ngroups + 1
    assert c.schedule["max_parallel"] == s.max_parallel
    assert c.schedule["num_bs"] == [len(g) for g in s.groups]


def test_slots_match_reference(case):
    c, s = case
    slots = c.schedule["slots"]
    assert len(slots) == s.nslots
    for k, sl in enumerate(slots):
        b = int(s.slot_ids[k])
        assert sl["id"] == b
        assert sl["coe"] == tuple(float(v) for v in s.slot_coe[k])  # bit-exact
        mine = [tuple(int(v) for v in c.shuffled[e]) for e in s.block_entries[b]]
        assert mine == sl["xyz"]


def test_fixtures_cover_quirks():
    """The fixture set exercises the reference quirks the builder must keep."""
    seen = dict(dup=False, empty=False, q3=False, multi_pad=False)
    for name in CASES:
        c = goldens.Case(name)
        s = oracle.Schedule(c.shuffled, *c.dims, c.meta["block_s"], c.meta["parallel_sequence_size"])
        seen["dup"] |= s.counters["duplicating"] > 0
        seen["empty"] |= s.counters["empty_resplit"] > 0
        seen["multi_pad"] |= s.nslots > len(set(s.slot_ids.tolist()))
        # Q3: entries outside their block's prefix range (split on the global-level bit)
        for b in range(s.nblocks):
            if s.block_nnz[b] == 0:
                continue
            L = int(s.block_levels[b, 0])
            g = s.global_levels[0]
            code = int(s.block_codes[b, 0])
            for e in s.block_entries[b][:64]:
                n2 = oracle.hx(c.dims[0], g, int(c.shuffled[e, 0]))
                pre = (n2 >> (g - L)) & ((1 << (L - 1)) - 1) if L > 1 else 0
                if pre != code:
                    seen["q3"] = True
                    break
    assert all(seen.values()), seen


def test_flat_schedule_sample_is_a_prefix(case):
    """The CPU legs of the bench replay a bounded leading sample of large
    schedules: that sample is the full schedule's first groups, and replaying
    it gives exactly the factors of replaying those groups of the full one."""
    c, s = case
    full = oracle.FlatSchedule(s.group_off, s.slot_ids, s.slot_coe, lambda b: s.block_entries[b])
    if full.nslots < 2:
        pytest.skip("single-slot schedule")
    cap = int(full.soff[full.nslots // 2])
    part = oracle.FlatSchedule(s.group_off, s.slot_ids, s.slot_coe, lambda b: s.block_entries[b],
                               max_updates=cap)
    assert 0 < part.ngroups <= full.ngroups and part.soff[-1] >= cap
    assert np.array_equal(part.goff, full.goff[: part.ngroups + 1])
    assert np.array_equal(part.soff, full.soff[: part.nslots + 1])
    assert np.array_equal(part.ent, full.ent[: len(part.ent)])
    R = 4
    rng = np.random.default_rng(1)
    F1 = [rng.uniform(0, 0.1, (n, R)) for n in c.dims]
    F2 = [f.copy() for f in F1]
    val = c.shuffled_values()
    u1 = full.replay(c.shuffled, val, R, 0.01, 0.01, *F1, 0, part.nslots)
    u2 = part.replay(c.shuffled, val, R, 0.01, 0.01, *F2)
    assert u1 == u2 and all(np.array_equal(a, b) for a, b in zip(F1, F2))


def test_hx_float_rounding():
    """hx divides in float: near the top of a 5M axis the bucket differs from
    the exact integer quotient (block.cu:41-42)."""
    I = 4999999
    diffs = 0
    for num in range(I - 4000, I):
        for level in (20, 22, 23):
            exact = (num * (1 << (level - 1))) // (I + 1)
            if oracle.hx(I, level, num) != exact:
                diffs += 1
    assert diffs > 0


@pytest.mark.parametrize("spec", [dict(I=500, J=400, K=300, nnz=20000, zipf=(1.2, 1.2, 1.2), gt_rank=4, seed=3),
                                  dict(I=2000, J=300, K=90000, nnz=100000, zipf=(1.5, 0.0, 1.5), gt_rank=0,
                                       noise_std=0.0, seed=4),
                                  dict(I=100000, J=100000, K=10000, nnz=200000, zipf=(1.3, 1.3, 1.3), gt_rank=32,
                                       noise_std=0.05, train_frac=0.95, seed=20261208)])
def test_oracle_generator_and_shuffle_equal_the_library(spec):
    """The reference arm draws its sample with the oracle's generator and
    shuffles it with the oracle's std::mt19937 shuffle, never loading the
    product library; both must give exactly the library's entries, and a
    draw of fewer cells must be a prefix of a larger draw."""
    import btc_gpu as bg

    got = oracle.gen_tensor(**spec)
    want = bg.gen_tensor(**spec)
    for a, b in zip(got, want):
        assert a.dtype == b.dtype and np.array_equal(a, b)
    small = oracle.gen_tensor(**dict(spec, nnz=spec["nnz"] // 2))
    if spec.get("gt_rank", 8) > 0:  # log-normal values are rescaled by each draw's own maximum
        for a, b in ((small[0], got[0]), (small[1], got[1])):
            assert np.array_equal(a, b[: len(a)])
    tx, tv = oracle.shuffle(got[0].copy(), got[1].copy())
    ux, uv = bg.shuffle(want[0].copy(), want[1].copy())
    assert np.array_equal(tx, ux) and np.array_equal(tv, uv)
