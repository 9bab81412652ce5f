"""Host logic of the product library (no GPU): schedule builder, report,
shuffle, text reader and the C ABI's exported symbols.

The builder is compared with the golden fixtures produced by the reference's
own block.cu (tests/golden/make_golden.py): same blocks, groups, coe weights
and per-slot entry order, and a byte-identical block_parallel.txt.
"""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import btc_gpu as bg
import goldens

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = goldens.cases()


def _cfg(c, **kw):
    return bg.config(I=c.meta["I"], J=c.meta["J"], K=c.meta["K"], block_s=c.meta["block_s"],
                     parallel_sequence_size=c.meta["parallel_sequence_size"], resident_blocks=-1, **kw)


@pytest.fixture(scope="module", params=CASES)
def built(request):
    c = goldens.Case(request.param)
    xyz, val = bg.shuffle(c.input_xyz.copy(), c.input_val.copy())
    return c, xyz, val, bg.Schedule(_cfg(c), xyz)


def test_shuffle_matches_reference(built):
    c, xyz, val, s = built
    assert np.array_equal(xyz, c.shuffled)


def test_blocks_match_reference(built):
    c, xyz, val, s = built
    meta, codes = s.blocks()
    assert c.header["num_block_total"] == s.summary.num_blocks
    nonempty = [b for b in range(s.summary.num_blocks) if meta[b, 0] > 0]
    assert [rb["id"] for rb in c.blocks] == nonempty
    for b, rb in zip(nonempty, c.blocks):
        assert rb["nnz"] == int(meta[b, 0])
        assert rb["levels"] == tuple(int(v) for v in meta[b, 1:])
        for a in range(3):
            L = int(meta[b, 1 + a])
            bits = "0" + (format(int(codes[b, a]), "0%db" % (L - 1)) if L > 1 else "")
            assert rb["ids"][a] == bits


def test_groups_slots_coe_match_reference(built):
    c, xyz, val, s = built
    off, ids, coe = s.groups()
    assert [ids[off[i]:off[i + 1]].tolist() for i in range(len(off) - 1)] == [q["ids"] for q in c.seqs]
    assert s.summary.max_parallel == c.schedule["max_parallel"]
    assert s.summary.num_groups + 1 == c.schedule["num_parallel"]
    for k, sl in enumerate(c.schedule["slots"]):
        assert tuple(float(v) for v in coe[k]) == sl["coe"]
        ent = s.block_entries(int(ids[k]))
        assert [tuple(v) for v in xyz[ent].tolist()] == sl["xyz"]


@pytest.mark.parametrize("seed,dims,nnz,zipf,block_s", [
    (11, (3000, 3000, 3000), 200_000, (0.0, 0.0, 0.0), 256),
    (12, (20000, 20000, 5000), 300_000, (1.2, 1.2, 1.2), 512),
    (13, (50000, 500, 200000), 300_000, (1.5, 0.0, 1.5), 512),
    (14, (100000, 100000, 10000), 400_000, (1.3, 1.3, 1.3), 2048),
    (15, (2000, 2000, 2000), 100_000, (1.5, 1.5, 1.5), 64),
])
def test_strata_and_groups_match_oracle_on_skewed_inputs(seed, dims, nnz, zipf, block_s):
    """The product builder (threaded first-fit strata, threaded padding) gives
    the oracle's strata, groups and coe weights on larger skewed inputs than
    the fixtures: hot rows make long chains of mutually conflicting blocks."""
    import oracle

    I, J, K = dims
    tx, _, _, _ = bg.gen_tensor(I, J, K, nnz, zipf=zipf, train_frac=1.0, seed=seed)
    o = oracle.Schedule(tx, I, J, K, block_s, 8)
    s = bg.Schedule(bg.config(I=I, J=J, K=K, block_s=block_s, parallel_sequence_size=8, resident_blocks=-1), tx)
    assert s.summary.num_strata == o.nstrata
    assert s.strata() == o.strata
    off, ids, coe = s.groups()
    assert np.array_equal(off, o.group_off) and np.array_equal(ids, o.slot_ids)
    assert np.array_equal(coe, o.slot_coe)


def test_threaded_builder_equals_serial_builder():
    """With thousands of open strata the first-fit scan is split over host
    threads (and padding runs per group on threads); the schedule must not
    depend on the thread count.  This input has ~9,400 strata."""
    I, J, K = 50000, 500, 200000
    tx, _, _, _ = bg.gen_tensor(I, J, K, 2_000_000, zipf=(1.5, 0.0, 1.5), train_frac=1.0, seed=3)
    out = []
    for threads in (1, 4):
        s = bg.Schedule(bg.config(I=I, J=J, K=K, block_s=256, parallel_sequence_size=8, host_threads=threads), tx)
        assert s.summary.num_strata > 4096
        out.append((s.strata(), s.groups()))
    assert out[0][0] == out[1][0]
    for x, y in zip(out[0][1], out[1][1]):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("dims,nnz,zipf,block_s", [((20000, 20000, 5000), 300_000, (1.2, 1.2, 1.2), 16),
                                                   ((50000, 500, 200000), 400_000, (1.5, 0.0, 1.5), 256),
                                                   ((1000, 1000, 1000), 300_000, (1.3, 1.3, 1.3), 32),
                                                   ((300, 200, 100), 200_000, (1.1, 1.1, 1.1), 8)])
def test_chunked_blocking_equals_serial_blocking(dims, nnz, zipf, block_s):
    """With several host threads the blocking runs in chunks: entries grouped
    by the leaf they reach in a snapshot of the tree, each group replayed into
    its own subtree on a thread, a chunk cut short where a split would raise a
    global level.  Blocks (ids, levels, codes, entry order), strata and slots
    must equal the one-thread insertion loop's.  Small block_s gives tens of
    thousands of splits and many global-level changes."""
    I, J, K = dims
    tx, _, _, _ = bg.gen_tensor(I, J, K, nnz, zipf=zipf, gt_rank=2, train_frac=1.0, seed=nnz + block_s)
    tx, _ = bg.shuffle(tx, np.zeros(len(tx)))
    out = []
    for threads in (1, 6):
        s = bg.Schedule(bg.config(I=I, J=J, K=K, block_s=block_s, parallel_sequence_size=8, host_threads=threads,
                                  resident_blocks=-1), tx)
        meta, codes = s.blocks()
        out.append((s, meta, codes))
    (a, ma, ca), (b, mb, cb) = out
    assert np.array_equal(ma, mb) and np.array_equal(ca, cb)
    assert a.summary.num_blocks > 1000
    for i in range(len(ma)):
        assert np.array_equal(a.block_entries(i), b.block_entries(i)), i
    assert a.strata() == b.strata()
    for x, y in zip(a.groups(), b.groups()):
        assert np.array_equal(x, y)


def test_report_byte_identical(built, tmp_path):
    c, xyz, val, s = built
    p = tmp_path / "block_parallel.txt"
    s.write_report(str(p))
    with open(os.path.join(c.dir, "block_parallel.txt"), "rb") as f:
        assert p.read_bytes() == f.read()


def test_reader_skips_like_the_reference(tmp_path):
    p = tmp_path / "t.train"
    p.write_text("# comment\n% also\n\n1 2 3 0.5\n4 5 6 7e-1 extra fields\n1.5 2 3 4\nbad line\n"
                 "  7 8 9   -2.25\n1 2\n3 3 3 inf\n2 2 2 1e\n2 2 2 1e999\n5 5 5 1e-999\n")
    xyz, val = bg.read_entries(str(p), 1, 10, 10, 10)
    # the same lines libstdc++'s stream extraction accepts (main.cpp:47-63)
    assert xyz.tolist() == [[0, 1, 2], [3, 4, 5], [6, 7, 8], [4, 4, 4]]
    assert val.tolist() == [0.5, 0.7, -2.25, 0.0]


_TRICKY = ("# comment\n% also\n\n1 2 3 0.5\n4 5 6 7e-1 extra fields\n1.5 2 3 4\nbad line\n"
           "  7 8 9   -2.25\n1 2\n3 3 3 inf\n2 2 2 1e\n2 2 2 1e999\n5 5 5 1e-999\n")


def test_reader_large_file_parses_like_small_ones(tmp_path):
    """Files of 64 MB and more are parsed in newline-aligned chunks on host
    threads: the entries, their order and the skipped lines are the same as
    for the small file repeated."""
    reps = (64 << 20) // len(_TRICKY) + 1000
    p = tmp_path / "big.train"
    p.write_text(_TRICKY * reps)
    xyz, val = bg.read_entries(str(p), 1, 10, 10, 10)
    one_xyz = np.array([[0, 1, 2], [3, 4, 5], [6, 7, 8], [4, 4, 4]], np.int32)
    one_val = np.array([0.5, 0.7, -2.25, 0.0])
    assert xyz.shape == (4 * reps, 3)
    assert np.array_equal(xyz, np.tile(one_xyz, (reps, 1))) and np.array_equal(val, np.tile(one_val, reps))


def test_reader_large_file_reports_the_first_bad_line(tmp_path):
    """An out-of-range line late in a chunked file is reported by its line
    number in the whole file, the first such line winning."""
    reps = (64 << 20) // len(_TRICKY) + 1000
    lines_per = _TRICKY.count("\n")
    k1, k2 = reps * 3 // 4, reps - 5
    text = _TRICKY * k1 + "11 1 1 1.0\n" + _TRICKY * (k2 - k1) + "1 11 1 1.0\n" + _TRICKY * (reps - k2)
    p = tmp_path / "bad.train"
    p.write_text(text)
    with pytest.raises(bg.BtcError) as e:
        bg.read_entries(str(p), 1, 10, 10, 10)
    assert e.value.status == 8 and e.value.line == k1 * lines_per + 1


def test_binary_cache_round_trip_and_invalidation(tmp_path):
    p = tmp_path / "t.train"
    p.write_text(_TRICKY)
    cache = str(tmp_path / "t.train.btcbin")
    want = bg.read_entries(str(p), 1, 10, 10, 10)
    got = bg.read_entries(str(p), 1, 10, 10, 10, cache=cache)  # parses, writes the cache
    assert not bg.read_entries.from_cache and os.path.exists(cache)
    again = bg.read_entries(str(p), 1, 10, 10, 10, cache=cache)
    assert bg.read_entries.from_cache
    for a, b, c in zip(want, got, again):
        assert np.array_equal(a, b) and np.array_equal(a, c) and a.dtype == c.dtype
    # another base or shape is not served from this cache (and rewrites it)
    bg.read_entries(str(p), 0, 11, 11, 11, cache=cache)
    assert not bg.read_entries.from_cache
    bg.read_entries(str(p), 1, 10, 10, 10, cache=cache)
    assert not bg.read_entries.from_cache
    # an edited source is parsed again
    p.write_text(_TRICKY + "9 9 9 1.25\n")
    x2, v2 = bg.read_entries(str(p), 1, 10, 10, 10, cache=cache)
    assert not bg.read_entries.from_cache and v2[-1] == 1.25 and len(v2) == len(want[1]) + 1
    # a truncated cache falls back to the text
    with open(cache, "r+b") as f:
        f.truncate(60)
    x3, v3 = bg.read_entries(str(p), 1, 10, 10, 10, cache=cache)
    assert not bg.read_entries.from_cache and np.array_equal(v3, v2)
    # an unwritable cache location is no error
    x4, v4 = bg.read_entries(str(p), 1, 10, 10, 10, cache=str(tmp_path / "missing" / "c.btcbin"))
    assert np.array_equal(v4, v2)


def test_binary_cache_with_out_of_range_payload_is_parsed_again(tmp_path):
    """A cache whose header matches but whose coordinates break the shape
    (a damaged file, a stamp collision) is not trusted: the text is parsed."""
    p = tmp_path / "t.train"
    p.write_text(_TRICKY)
    cache = str(tmp_path / "t.train.btcbin")
    want = bg.read_entries(str(p), 1, 10, 10, 10, cache=cache)
    assert os.path.exists(cache)
    with open(cache, "r+b") as f:
        f.seek(48)  # first coordinate after the 48-byte header
        f.write(np.array([10], np.int32).tobytes())  # x = I: out of range
    st = os.stat(str(p))
    got = bg.read_entries(str(p), 1, 10, 10, 10, cache=cache)
    assert not bg.read_entries.from_cache
    assert os.stat(str(p)).st_mtime_ns == st.st_mtime_ns
    for a, b in zip(want, got):
        assert np.array_equal(a, b)


def test_context_rejects_out_of_range_coordinates_before_the_device():
    """Train or test coordinates outside the shape fail with BTC_ERR_RANGE
    before any device work, so no kernel can index past a factor."""
    I, J, K = 6, 5, 4
    tx = np.array([[0, 0, 0], [5, 4, 3], [1, 2, 3]], np.int32)
    tv = np.ones(3)
    cfg = bg.config(I=I, J=J, K=K, rank=4, block_s=2, resident_blocks=-1)
    sched = bg.Schedule(cfg, tx)
    for bad_test in (np.array([[0, 0, 4]], np.int32), np.array([[-1, 0, 0]], np.int32),
                     np.array([[6, 0, 0]], np.int32)):
        with pytest.raises(bg.BtcError) as e:
            bg.Context(cfg, sched, tx, tv, bad_test, np.ones(1))
        assert e.value.status == 8
    # a train array other than the one the schedule was built from, with a
    # coordinate out of range
    with pytest.raises(bg.BtcError) as e:
        bg.Context(cfg, sched, np.array([[0, 0, 0], [5, 5, 3], [1, 2, 3]], np.int32), tv, tx, tv)
    assert e.value.status == 8


def test_reader_rejects_out_of_range(tmp_path):
    p = tmp_path / "t.train"
    p.write_text("1 1 1 1.0\n0 1 1 2.0\n")
    with pytest.raises(bg.BtcError) as e:
        bg.read_entries(str(p), 1, 5, 5, 5)
    assert e.value.status == 8 and e.value.line == 2


def test_builder_rejects_out_of_range_coordinates():
    cfg = bg.config(I=4, J=4, K=4, resident_blocks=-1)
    with pytest.raises(bg.BtcError):
        bg.Schedule(cfg, np.array([[0, 0, 4]], np.int32))


def test_config_validation():
    assert bg.validate(bg.config()) == 0
    for kw in (dict(rank=0), dict(rank=129), dict(lr=0.0), dict(reg=-1.0), dict(block_s=0),
               dict(thread_size=1025), dict(parallel_sequence_size=-1), dict(epochs=0), dict(dtype=7)):
        assert bg.validate(bg.config(**kw)) != 0, kw


def test_abi_exports_every_declared_symbol():
    with open(os.path.join(ROOT, "include", "btc_gpu.h")) as f:
        hdr = f.read()
    declared = set(re.findall(r"\b(btc_[a-z0-9_]+)\s*\(", hdr))
    declared -= {"btc_status"}
    lib = bg.lib()
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(bg.SIGNATURES) == declared


def test_generator_is_deterministic_and_deduplicated():
    a = bg.gen_tensor(500, 400, 300, 20000, zipf=(1.2, 1.2, 1.2), gt_rank=4, seed=3)
    b = bg.gen_tensor(500, 400, 300, 20000, zipf=(1.2, 1.2, 1.2), gt_rank=4, seed=3)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    allx = np.concatenate([a[0], a[2]])
    assert len(allx) == 20000
    assert len(np.unique(allx, axis=0)) == 20000
    assert 0.85 < len(a[1]) / 20000 < 0.95


def test_cli_arguments_like_the_reference():
    cli = bg.CLI_PATH
    r = subprocess.run([cli, "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "Usage:" in r.stderr
    r = subprocess.run([cli, "ds", "1", "2"], capture_output=True, text=True)
    assert r.returncode == 1
    r = subprocess.run([cli, "ds", "10", "10", "10", "/tmp", "0", "/tmp", "--rank", "101"],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "rank r must be in [1, 100]" in r.stderr
    r = subprocess.run([cli, "ds", "10", "10", "10", "--bogus=1"], capture_output=True, text=True)
    assert r.returncode == 1 and "Unknown option: --bogus" in r.stderr
    r = subprocess.run([cli, "ds", "10", "10", "10", "/tmp", "2"], capture_output=True, text=True)
    assert r.returncode == 1 and "coord_base must be 0 or 1." in r.stderr
    # this library's own options are accepted next to the reference's
    r = subprocess.run([cli, "ds", "10", "10", "10", "/tmp", "0", "/tmp", "--rank", "101", "--bin-cache", "/tmp",
                        "--precision", "bf16", "--mode", "staged"], capture_output=True, text=True)
    assert r.returncode == 1 and "Unknown option" not in r.stderr and "rank r must be in [1, 100]" in r.stderr


@pytest.mark.parametrize("dims,nnz,zipf,block_s", [((20000, 20000, 5000), 300_000, (1.2, 1.2, 1.2), 256),
                                                   ((50000, 500, 200000), 400_000, (1.5, 0.0, 1.5), 1024),
                                                   ((300, 200, 100), 50_000, (0.0, 0.0, 0.0), 64)])
def test_learned_blocking_schedules_every_entry_once_in_conflict_free_groups(dims, nnz, zipf, block_s):
    """The learned blocking (no model: split axes in turn) is a partition of
    the train entries into boxes of at most block_s entries, each block once
    per epoch (no padding), grouped so that no two blocks of a group share a
    row of any mode; every coe weight is 1."""
    I, J, K = dims
    tx, _, _, _ = bg.gen_tensor(I, J, K, nnz, zipf=zipf, gt_rank=2, train_frac=1.0, seed=11)
    tx, _ = bg.shuffle(tx, np.zeros(len(tx)))
    cfg = bg.config(I=I, J=J, K=K, block_s=block_s, parallel_sequence_size=8, resident_blocks=-1)
    s = bg.Schedule(cfg, tx, learned=True)
    sm = s.summary
    assert sm.scheduled_updates == len(tx) and sm.num_slots == sm.num_blocks
    boxes = s.boxes()
    seen = np.zeros(len(tx), np.int64)
    for b in range(sm.num_blocks):
        e = s.block_entries(b)
        assert 0 < len(e) <= block_s
        assert np.all(np.diff(e) > 0)  # input order kept inside a block
        seen[e] += 1
        c = tx[e]
        assert (c >= boxes[b, :, 0]).all() and (c < boxes[b, :, 1]).all()
    assert (seen == 1).all()
    off, ids, coe = s.groups()
    assert np.all(coe == 1.0) and sorted(ids.tolist()) == list(range(sm.num_blocks))
    for g in range(len(off) - 1):
        bl = ids[off[g]:off[g + 1]]
        assert 1 <= len(bl) <= 8
        lo, hi = boxes[bl, :, 0], boxes[bl, :, 1]
        overlap = (lo[:, None, :] < hi[None, :, :]) & (lo[None, :, :] < hi[:, None, :])
        np.fill_diagonal(overlap[:, :, 0], False)
        np.fill_diagonal(overlap[:, :, 1], False)
        np.fill_diagonal(overlap[:, :, 2], False)
        assert not overlap.any()
    # deterministic for any thread count
    s1 = bg.Schedule(bg.config(I=I, J=J, K=K, block_s=block_s, parallel_sequence_size=8, resident_blocks=-1,
                               host_threads=1), tx, learned=True)
    assert np.array_equal(s1.boxes(), boxes)
    for x, y in zip(s1.groups(), s.groups()):
        assert np.array_equal(x, y)


def test_config1_blocking_equals_the_pinned_reference_schedule(tmp_path):
    """The 1M-entry config-1 input (900k train entries): the product builder's
    schedule -- groups, slots, coe weights, every slot's entries in order --
    and its block_parallel.txt hash to the digests of the reference's own
    block.cu output committed by tests/golden/make_c1_pin.py."""
    import hashlib
    import json

    import make_c1_pin as pin_mod

    with open(os.path.join(ROOT, "tests", "golden", "c1_pin.json")) as f:
        pin = json.load(f)
    spec = dict(pin["spec"])
    I, J, K, nnz = spec.pop("I"), spec.pop("J"), spec.pop("K"), spec.pop("nnz")
    tx, tv, _, _ = bg.gen_tensor(I, J, K, nnz, **spec)
    tx, tv = bg.shuffle(tx, tv)
    assert len(tv) == pin["train_nnz"]
    cfg = bg.config(I=I, J=J, K=K, block_s=pin["block_s"], parallel_sequence_size=pin["parallel_sequence_size"],
                    resident_blocks=-1)
    s = bg.Schedule(cfg, tx)
    off, ids, coe = s.groups()
    assert len(ids) == pin["slots"] and len(off) - 1 == pin["groups"]
    slots = []
    for k in range(len(ids)):
        e = s.block_entries(int(ids[k]))
        slots.append(dict(id=int(ids[k]), nnz=len(e), coe=tuple(coe[k]), xyz=tx[e].tolist()))
    num_bs = [int(off[g + 1] - off[g]) for g in range(len(off) - 1)]
    assert pin_mod.digest(pin_mod.canonical(num_bs, slots)) == pin["schedule_sha256"]
    rep = tmp_path / "block_parallel.txt"
    s.write_report(str(rep))
    assert hashlib.sha256(rep.read_bytes()).hexdigest() == pin["report_sha256"]
