"""Pin the reference's blocking on the 1M-entry config-1 input.

The config-1 workload (I = J = K = 1000, 1M cells with uniform indices, 90/10
split; the benchmark's "c1" draw, seed 20261204) has ~900k train entries: too
many to commit as a fixture, few enough that the reference's own block.cu
(built by `make -C oracle ref` into oracle/_ref/) schedules them in seconds.
This script writes the train entries in the benchmark's order, runs the
reference (which shuffles them with std::mt19937(42) and calls block_problem
with block_s 2048 and 8 blocks per sequence), and commits SHA-256 digests of
its block_parallel.txt and of a canonical text of the schedule it hands to
sgd_train (per group its size; per slot block id, nnz, coe weights as hex and
the entries' coordinates in order), with the counts, to c1_pin.json.

    python tests/golden/make_c1_pin.py [REF_DIR]
"""
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [HERE, os.path.join(ROOT, "oracle")]

import oracle  # noqa: E402
import refdump  # noqa: E402

SPEC = dict(I=1000, J=1000, K=1000, nnz=1_000_000, zipf=(0.0, 0.0, 0.0), gt_rank=8, gt_std=0.5, noise_std=0.01,
            train_frac=0.9, seed=20261204)
BLOCK_S, PSS = 2048, 8


def canonical(num_bs, slots):
    """The schedule as one text: group sizes, then per slot its block id, nnz,
    coe weights (hex) and entries' coordinates."""
    out = ["num_bs " + " ".join(str(v) for v in num_bs)]
    for s in slots:
        out.append("%d %d %s %s %s" % (s["id"], s["nnz"], *(float(c).hex() for c in s["coe"])))
        out.extend("%d %d %d" % tuple(p) for p in s["xyz"])
    return "\n".join(out) + "\n"


def digest(text):
    return hashlib.sha256(text.encode() if isinstance(text, str) else text).hexdigest()


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("BTC_REFERENCE_SRC", "/root/reference")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "REF=" + ref])
    ref_bin = os.path.join(ROOT, "oracle", "_ref", "ref_block")
    spec = dict(SPEC)
    tx, tv, _, _ = oracle.gen_tensor(spec.pop("I"), spec.pop("J"), spec.pop("K"), spec.pop("nnz"), **spec)
    tmp = tempfile.mkdtemp()
    inp = os.path.join(tmp, "in.txt")
    with open(inp, "w") as f:
        f.writelines("%d %d %d %.17g\n" % (a, b, c, v) for (a, b, c), v in zip(tx.tolist(), tv.tolist()))
    subprocess.check_call([ref_bin, inp, "1000", "1000", "1000", str(BLOCK_S), str(PSS), tmp, "c1", "0.9"],
                          stdout=subprocess.DEVNULL)
    try:
        sched = refdump.parse_schedule(os.path.join(tmp, "schedule.txt"))
        with open(os.path.join(tmp, "c1_0.9", "block_parallel.txt"), "rb") as f:
            report = f.read()
    finally:
        shutil.rmtree(tmp)
    pin = dict(spec=SPEC, block_s=BLOCK_S, parallel_sequence_size=PSS, train_nnz=int(len(tv)),
               slots=len(sched["slots"]), groups=len(sched["num_bs"]), max_parallel=sched["max_parallel"],
               schedule_sha256=digest(canonical(sched["num_bs"], sched["slots"])),
               report_sha256=digest(report))
    with open(os.path.join(HERE, "c1_pin.json"), "w") as f:
        json.dump(pin, f, indent=1)
    print(json.dumps(pin))


if __name__ == "__main__":
    main()
