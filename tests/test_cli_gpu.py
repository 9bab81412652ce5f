"""The drop-in CLI end to end on a GPU: same files and stdout lines as the
reference binary, and the schedule report byte-identical to the one the
reference's own block.cu wrote for the same train file."""
import glob
import os
import subprocess

import numpy as np
import pytest

import btc_gpu as bg
import goldens

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("extra", [[], ["--precision", "bf16", "--mode", "staged"],
                                   ["--precision", "f64", "--mode", "deterministic"]])
def test_cli_runs_like_the_reference(tmp_path, extra):
    c = goldens.Case("uniform_3k")
    data = tmp_path / "data"
    data.mkdir()
    with open(data / "ds.train", "w") as f:
        for (x, y, z), v in zip(c.input_xyz.tolist(), c.input_val.tolist()):
            f.write("%d %d %d %.12g\n" % (x + 1, y + 1, z + 1, v))  # 1-based, the reference's default
    with open(data / "ds.test", "w") as f:
        f.write("# test split\n")
        for (x, y, z), v in list(zip(c.input_xyz.tolist(), c.input_val.tolist()))[:100]:
            f.write("%d %d %d %.12g\n" % (x + 1, y + 1, z + 1, v))
    out = tmp_path / "out"
    I, J, K = c.dims
    r = subprocess.run([bg.CLI_PATH, "ds", str(I), str(J), str(K), str(data), "1", str(out), "--epochs", "3",
                        "--block", str(c.meta["block_s"]), "--parallel-sequence-size",
                        str(c.meta["parallel_sequence_size"]), "--seed", "5", "--dump-factors",
                        str(tmp_path / "f")] + extra, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    so = r.stdout
    for needle in ("Loaded 3000 train entries", "Loaded 100 test entries",
                   "Shuffled train entries with seed=42 before block construction.", "Train rate=",
                   "max_parallel=", "GPU:", "Epoch:0 test_RMSE=", "Final test RMSE=", "first train entry: ("):
        assert needle in so, needle
    d = glob.glob(str(out / "ds_*"))
    assert len(d) == 1
    d = d[0]
    with open(os.path.join(d, "block_parallel.txt"), "rb") as f, \
            open(os.path.join(c.dir, "block_parallel.txt"), "rb") as g:
        assert f.read() == g.read()
    lines = open(os.path.join(d, "error.txt")).read().splitlines()
    assert lines[0] == "epoch test_RMSE test_MAE test_ER test_count"
    assert len(lines) >= 2 and lines[1].split()[0] == "0" and lines[1].split()[-1] == "100"
    for name in ("time.txt", "kernel_time.txt", "sync_time.txt"):
        assert os.path.getsize(os.path.join(d, name)) > 0
    A = np.loadtxt(tmp_path / "f" / "A.txt")
    assert A.shape == (I, 16) and np.isfinite(A).all()


def test_cli_early_stop_and_literal_output_directory(tmp_path):
    """The epoch loop stops once test RMSE improves by less than 1e-8 over the
    previous epoch (sgd_Kernel.cu:1308-1317): with a learning rate too small
    to move it, epochs 0 and 1 run and the loop ends.  The output and dump
    directories are created as named, shell metacharacters included."""
    c = goldens.Case("uniform_3k")
    data = tmp_path / "data"
    data.mkdir()
    with open(data / "ds.train", "w") as f:
        for (x, y, z), v in zip(c.input_xyz.tolist(), c.input_val.tolist()):
            f.write("%d %d %d %.12g\n" % (x, y, z, v))
    with open(data / "ds.test", "w") as f:
        for (x, y, z), v in list(zip(c.input_xyz.tolist(), c.input_val.tolist()))[:200]:
            f.write("%d %d %d %.12g\n" % (x, y, z, v))
    marker = tmp_path / "ran"
    out = tmp_path / ('o "q" $(touch %s)' % marker)
    dump = tmp_path / "d;touch x"
    I, J, K = c.dims
    r = subprocess.run([bg.CLI_PATH, "ds", str(I), str(J), str(K), str(data), "0", str(out), "--epochs", "50",
                        "--lr", "1e-12", "--seed", "5", "--dump-factors", str(dump)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert not marker.exists()
    d = glob.glob(os.path.join(glob.escape(str(out)), "ds_*"))
    assert len(d) == 1 and os.path.isdir(d[0])
    lines = open(os.path.join(d[0], "error.txt")).read().splitlines()
    assert [ln.split()[0] for ln in lines[1:]] == ["0", "1"]
    assert "Epoch:1 test_RMSE=" in r.stdout and "Epoch:2 " not in r.stdout
    assert (dump / "A.txt").is_file()
