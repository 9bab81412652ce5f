"""The N>1 path on host cores (no GPU): bench.py runs one replica per rank,
times every rank between barriers and reports the maximum over ranks; the
reference arm runs on rank 0 alone while the other ranks exit without work.
Ranks talk over gloo on 127.0.0.1."""
import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


class _Stats:
    def __init__(self, ms):
        self.kernel_ms = ms


class _FakeContext:
    """Stands in for a device context: its epochs take a rank-dependent time."""

    def __init__(self, ms):
        self.ms = ms

    def train_epochs(self, n):
        return _Stats(self.ms * n)


def _rank_main(rank, world, port, queue):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench

    st, ms = bench._timed(_FakeContext(10.0 * (rank + 1)), 3, dist)
    e2e = bench._max_over_ranks(0.5 + rank, dist)
    queue.put((rank, ms, e2e, st.kernel_ms))
    dist.barrier()
    dist.destroy_process_group()


def test_timing_takes_the_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(queue.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [60.0, 60.0]  # both ranks report the slower rank's 3 epochs
    assert [o[2] for o in out] == [1.5, 1.5]
    assert [o[3] for o in out] == [30.0, 60.0]  # each rank's own stats are untouched


def test_reference_arm_runs_on_rank_zero_only_under_torchrun():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "small", "--gpus", "2",
           "--steps", "1", "--warmup", "1", "--ref-seconds", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-3000:]
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


def test_reference_arm_does_not_load_the_product_library():
    """The reference arm draws, shuffles and blocks its sample with oracle
    code and replays it with the oracle: the process never maps the product
    library."""
    code = ("import sys; sys.path[:0] = [%r, %r]; import bench; "
            "w, m, tx, tv, sched, flat = bench.reference_sample('small'); "
            "u, t, g = bench.cpu_sample(flat, tx, tv, w, 0.5, 2); "
            "maps = open('/proc/self/maps').read(); "
            "print('LOADED', 'libbtcgpu' in maps, 'ORACLE', 'libbtc_oracle' in maps, 'UPDATES', u)"
            % (ROOT, os.path.join(ROOT, "oracle")))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    out = r.stdout.split()
    assert out[out.index("LOADED") + 1] == "False"
    assert out[out.index("ORACLE") + 1] == "True"
    assert int(out[out.index("UPDATES") + 1]) > 0
