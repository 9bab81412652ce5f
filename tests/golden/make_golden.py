"""Generate the golden blocking/schedule fixtures from the reference itself.

Runs the reference's own block.cu (built by `make -C oracle ref` from the
reference source tree into oracle/_ref/) on small seeded inputs and stores,
per case:

  input.txt.gz        0-based "x y z value" lines (value printed %.12g, the
                      writer format of the reference's dataset scripts)
  shuffled.txt.gz     the train order after std::shuffle(mt19937(42))
  block_parallel.txt  the reference's schedule report
  schedule.txt.gz     the schedule block_problem hands to sgd_train
  meta.json           dims, block_s, parallel_sequence_size, train_rate

Only this generator needs the reference sources; the fixtures it writes are
committed and the tests read them anywhere.

    python tests/golden/make_golden.py [REF_DIR]
"""
import gzip
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def zipf_idx(rng, n, s, size):
    w = 1.0 / np.arange(1, n + 1, dtype=np.float64) ** s
    c = np.cumsum(w)
    c /= c[-1]
    return np.minimum(np.searchsorted(c, rng.random(size)), n - 1).astype(np.int64)


def uniform(rng, dims, n):
    return np.column_stack([rng.integers(0, d, n) for d in dims])


def zipf(rng, dims, s, n):
    return np.column_stack([zipf_idx(rng, d, s, n) for d in dims])


def dedup(xyz):
    # unique coordinates in first-seen order (the writer never repeats a cell)
    _, first = np.unique(xyz, axis=0, return_index=True)
    return xyz[np.sort(first)]


CASES = {
    # name: (dims, generator, block_s, pss)
    "uniform_3k": ((200, 300, 150), lambda r: uniform(r, (200, 300, 150), 3000), 64, 8),
    "zipf13_6k": ((2000, 2000, 500), lambda r: zipf(r, (2000, 2000, 500), 1.3, 6000), 64, 8),
    "zipf15_auto": ((800, 900, 700), lambda r: zipf(r, (800, 900, 700), 1.5, 3000), 16, 0),
    "zipf_bs4_dup": ((1500, 400, 900), lambda r: zipf(r, (1500, 400, 900), 1.6, 1200), 4, 50),
    "uniform_pss3": ((64, 64, 64), lambda r: uniform(r, (64, 64, 64), 2000), 32, 3),
    "pss_clamp": ((100, 100, 100), lambda r: uniform(r, (100, 100, 100), 500), 200, 50),
    "single": ((10, 10, 10), lambda r: np.array([[3, 4, 5]]), 8, 8),
    "bigdim": ((4999999, 17, 3), lambda r: np.column_stack([
        np.concatenate([r.integers(0, 4999999, 1500), 4999999 - 1 - r.integers(0, 64, 300),
                        r.integers(0, 64, 200)]),
        r.integers(0, 17, 2000), r.integers(0, 3, 2000)]), 32, 8),
    "cube1000_20k": ((1000, 1000, 1000), lambda r: uniform(r, (1000, 1000, 1000), 20000), 512, 8),
}


def make_case(name, ref_bin, seed):
    dims, gen, block_s, pss = CASES[name]
    rng = np.random.default_rng(seed)
    xyz = dedup(np.asarray(gen(rng), dtype=np.int64))
    val = rng.normal(0.0, 0.5, len(xyz))
    out = os.path.join(HERE, name)
    os.makedirs(out, exist_ok=True)
    lines = "".join("%d %d %d %.12g\n" % (a, b, c, v) for (a, b, c), v in zip(xyz, val))
    with gzip.open(os.path.join(out, "input.txt.gz"), "wt") as f:
        f.write(lines)
    tmp = tempfile.mkdtemp()
    try:
        inp = os.path.join(tmp, "in.txt")
        with open(inp, "w") as f:
            f.write(lines)
        rate = "0.9"
        subprocess.check_call([ref_bin, inp, str(dims[0]), str(dims[1]), str(dims[2]),
                               str(block_s), str(pss), tmp, "golden", rate],
                              stdout=subprocess.DEVNULL)
        shutil.copy(os.path.join(tmp, "golden_" + rate, "block_parallel.txt"),
                    os.path.join(out, "block_parallel.txt"))
        for src, dst in (("shuffled.txt", "shuffled.txt.gz"), ("schedule.txt", "schedule.txt.gz")):
            with open(os.path.join(tmp, src)) as fi, gzip.open(os.path.join(out, dst), "wt") as fo:
                fo.write(fi.read())
    finally:
        shutil.rmtree(tmp)
    with open(os.path.join(out, "meta.json"), "w") as f:
        json.dump(dict(I=dims[0], J=dims[1], K=dims[2], block_s=block_s,
                       parallel_sequence_size=pss, train_rate=float(rate), nnz=int(len(xyz)),
                       seed=seed), f, indent=1)
    print("%-14s nnz=%d" % (name, len(xyz)))


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("BTC_REFERENCE_SRC", "/root/reference")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "REF=" + ref])
    ref_bin = os.path.join(ROOT, "oracle", "_ref", "ref_block")
    for i, name in enumerate(sorted(CASES)):
        make_case(name, ref_bin, 20261203 + i)


if __name__ == "__main__":
    main()
