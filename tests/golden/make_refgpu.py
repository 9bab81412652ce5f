"""Parity fixture from the reference binary itself, run on a GB300.

Runs the reference (built by `make -C oracle refgpu REF=<reference sources>`:
its own main.cpp, block.cu and sgd_Kernel.cu, with tensor_SGD replaced by
oracle/ref_seam/ref_tensor_sgd.cpp so the factor init is injected and the
final factors are dumped) and this repo's CLI on the same files and the same
initial factors, and writes one JSON summary:

  * reference per-epoch test RMSE for several runs (its Hogwild kernel is
    run-to-run nondeterministic, so the spread is recorded) and its epoch
    times (kernel_time.txt);
  * this repo's per-epoch test RMSE for each precision/mode;
  * max relative factor error after one epoch of every path against the
    reference and against the serial FP64 replay (the oracle).

Workload: I = J = K = 1000, 1M unique uniform entries, values from a rank-8
ground-truth CP (N(0, 0.5) factors) + N(0, 0.01) noise, 90/10 split, rank 16,
lr 0.01, lambda 0.01, 10 epochs, factors U(0, 0.1) from a seed, coord_base 0.

    python tests/golden/make_refgpu.py <tensor_sgd_ref> <out_dir> [runs]
"""
import glob
import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "btc-gpu_gb300", "python"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

N, R, LR, REG, EPOCHS, SEED = 1000, 16, 0.01, 0.01, 10, 20261203


def read_error(path):
    rm = []
    with open(path) as f:
        next(f)
        for line in f:
            p = line.split()
            rm.append(float(p[1]))
    return rm


def read_times(path):
    with open(path) as f:
        return [float(l) for l in f if l.strip()]


def main():
    ref_bin, out = sys.argv[1], sys.argv[2]
    runs = int(sys.argv[3]) if len(sys.argv) > 3 else 5
    import btc_gpu as bg
    import oracle

    os.makedirs(out, exist_ok=True)
    data = os.path.join(out, "data")
    os.makedirs(data, exist_ok=True)
    tx, tv, sx, sv = bg.gen_tensor(N, N, N, 1_000_000, gt_rank=8, gt_std=0.5, noise_std=0.01, train_frac=0.9,
                                   seed=SEED)
    for name, x, v in (("c1.train", tx, tv), ("c1.test", sx, sv)):
        with open(os.path.join(data, name), "w") as f:
            f.write("".join("%d %d %d %.17g\n" % (a, b, c, w) for (a, b, c), w in zip(x.tolist(), v.tolist())))
    rng = np.random.default_rng(SEED)
    init = [rng.uniform(0.0, 0.1, (N, R)) for _ in range(3)]
    init_path = os.path.join(out, "init.bin")
    with open(init_path, "wb") as f:
        for m in init:
            f.write(m.astype(np.float64).tobytes())
    common = ["c1", str(N), str(N), str(N), data, "0"]
    opts = ["--epochs", str(EPOCHS), "--rank", str(R), "--lr", str(LR), "--reg", str(REG), "--gpus", "1"]
    summary = dict(workload="1000^3, 1M uniform, R=16, lr 0.01, lambda 0.01, 10 epochs",
                   train=int(len(tv)), test=int(len(sv)))

    # the reference binary
    env = dict(os.environ, BTC_REF_INIT=init_path)
    ref_rmse, ref_times = [], []
    for k in range(runs):
        od = os.path.join(out, "ref_%d" % k)
        t = time.time()
        subprocess.check_call([ref_bin] + common + [od] + opts, env=env, stdout=subprocess.DEVNULL)
        d = glob.glob(os.path.join(od, "c1_*"))[0]
        ref_rmse.append(read_error(os.path.join(d, "error.txt")))
        ref_times.append(read_times(os.path.join(d, "kernel_time.txt")))
        print("reference run %d: %.1fs, final rmse %.10g" % (k, time.time() - t, ref_rmse[-1][-1]), flush=True)
    opts1 = [o if o != str(EPOCHS) else "1" for o in opts]
    ref_e1s = []
    for k in range(runs):
        env1 = dict(env, BTC_REF_DUMP=os.path.join(out, "ref_e1_%d.bin" % k))
        subprocess.check_call([ref_bin] + common + [os.path.join(out, "ref_e1_%d" % k)] + opts1, env=env1,
                              stdout=subprocess.DEVNULL)
        raw = np.fromfile(os.path.join(out, "ref_e1_%d.bin" % k), np.float64).reshape(3, N, R)
        ref_e1s.append([raw[m] for m in range(3)])
    ref_e1 = ref_e1s[0]
    np.savez_compressed(os.path.join(out, "reference_epoch1_factors.npz"),
                        A=ref_e1[0].astype(np.float32), B=ref_e1[1].astype(np.float32),
                        C=ref_e1[2].astype(np.float32))

    # the serial FP64 replay of the same schedule
    cfg = bg.config(I=N, J=N, K=N, rank=R, lr=LR, reg=REG)
    sx_, sv_ = bg.shuffle(tx.copy(), tv.copy())
    sched = bg.Schedule(cfg, sx_)
    off, ids, coe = sched.groups()
    flat = oracle.FlatSchedule(off, ids, coe, sched.block_entries)
    F = [m.copy() for m in init]
    orc_rmse, orc_e1 = [], None
    prev = None
    for e in range(EPOCHS):
        flat.replay(sx_, sv_, R, LR, REG, *F)
        if e == 0:
            orc_e1 = [m.copy() for m in F]
        cur = oracle.rmse_mae_er(sx, sv, R, *F)[0]
        orc_rmse.append(cur)
        if prev is not None and prev - cur < 1e-8:
            break
        prev = cur

    def maxrel(a, b):
        return float(max(np.abs(x - y).max() for x, y in zip(a, b)) / max(np.abs(y).max() for y in b))

    ours = {}
    for prec, mode in (("f32", "staged"), ("f32", "hogwild"), ("f32", "deterministic"), ("f64", "hogwild"),
                       ("f64", "deterministic"), ("f64", "staged")):
        key = "%s_%s" % (prec, mode)
        od = os.path.join(out, "ours_" + key)
        subprocess.check_call([bg.CLI_PATH] + common + [od] + opts +
                              ["--precision", prec, "--mode", mode, "--init-file", init_path],
                              stdout=subprocess.DEVNULL)
        rm = read_error(os.path.join(glob.glob(os.path.join(od, "c1_*"))[0], "error.txt"))
        od1 = os.path.join(out, "ours1_" + key)
        subprocess.check_call([bg.CLI_PATH] + common + [od1] + opts1 +
                              ["--precision", prec, "--mode", mode, "--init-file", init_path, "--dump-factors",
                               os.path.join(od1, "f")], stdout=subprocess.DEVNULL)
        e1 = [np.loadtxt(os.path.join(od1, "f", n)) for n in ("A.txt", "B.txt", "C.txt")]
        ours[key] = dict(rmse=rm, factor_maxrel_vs_reference_e1=maxrel(e1, ref_e1),
                         factor_maxrel_vs_oracle_e1=maxrel(e1, orc_e1))
        print(key, rm[-1], ours[key]["factor_maxrel_vs_reference_e1"], flush=True)

    ref_arr = np.array([r[:min(map(len, ref_rmse))] for r in ref_rmse])
    mean = ref_arr.mean(0)
    summary["reference"] = dict(rmse=ref_rmse, kernel_s=ref_times,
                                spread_rel=[float(v) for v in (ref_arr.max(0) - ref_arr.min(0)) / mean],
                                factor_maxrel_vs_oracle_e1=maxrel(ref_e1, orc_e1),
                                factor_spread_e1=[maxrel(r, ref_e1) for r in ref_e1s[1:]],
                                updates_per_epoch=int(sched.summary.scheduled_updates))
    summary["oracle"] = dict(rmse=orc_rmse)
    for key, d in ours.items():
        n = min(len(d["rmse"]), len(mean))
        d["rel_vs_reference_mean"] = [float(abs(a - b) / b) for a, b in zip(d["rmse"][:n], mean[:n])]
        d["rel_vs_oracle"] = [float(abs(a - b) / b) for a, b in zip(d["rmse"], orc_rmse)]
    summary["ours"] = ours
    with open(os.path.join(out, "summary.json"), "w") as f:
        json.dump(summary, f, indent=1)
    print(json.dumps({k: (v["rel_vs_reference_mean"][-1], v["factor_maxrel_vs_reference_e1"])
                      for k, v in ours.items()}))
    print("reference spread", summary["reference"]["spread_rel"])
    print("reference factor spread e1", summary["reference"]["factor_spread_e1"],
          "vs oracle", summary["reference"]["factor_maxrel_vs_oracle_e1"])


if __name__ == "__main__":
    main()
