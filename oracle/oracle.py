"""ctypes view of the C oracle (btc_oracle.c).

Test infrastructure only: the tests, the smoke entry and the bench's
CPU-baseline leg use it as the checker.  The product library never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libbtc_oracle.so")
_lib = None


def build():
    """Compile the oracle library (gcc only; no GPU, no reference sources)."""
    subprocess.check_call(["make", "-s", "-C", _HERE, "oracle"])


def _load():
    global _lib
    if _lib is not None:
        return _lib
    srcs = ("btc_oracle.c", "gen.c", "shuffle.cpp")
    if not os.path.exists(_LIB_PATH) or any(
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, f)) for f in srcs
    ):
        build()
    lib = ctypes.CDLL(_LIB_PATH)
    P = ctypes.c_void_p
    lib.orc_build.argtypes = [P, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                              ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(P)]
    lib.orc_build.restype = ctypes.c_int
    lib.orc_free.argtypes = [P]
    for name in ("orc_num_blocks", "orc_num_strata", "orc_num_groups", "orc_num_slots"):
        getattr(lib, name).argtypes = [P]
        getattr(lib, name).restype = ctypes.c_int
    lib.orc_info.argtypes = [P, P, P, P]
    lib.orc_blocks.argtypes = [P, P, P]
    lib.orc_block_entries.argtypes = [P, ctypes.c_int, P]
    lib.orc_block_entries.restype = ctypes.c_int
    lib.orc_strata_arrays.argtypes = [P, P, P]
    lib.orc_groups.argtypes = [P, P, P, P]
    lib.orc_sgd_epoch.argtypes = [P, P, P, ctypes.c_int, ctypes.c_double, ctypes.c_double, P, P, P]
    lib.orc_sgd_epoch.restype = ctypes.c_int64
    lib.orc_lf_epoch.argtypes = [P, P, P, ctypes.c_int, ctypes.c_double, ctypes.c_double, P, P, P]
    lib.orc_lf_epoch.restype = ctypes.c_int64
    lib.orc_metrics.argtypes = [P, P, ctypes.c_int64, ctypes.c_int, P, P, P, P]
    lib.orc_sgd_replay.argtypes = [ctypes.c_int64, ctypes.c_int64, P, P, P, P, P, ctypes.c_int,
                                   ctypes.c_double, ctypes.c_double, P, P, P]
    lib.orc_sgd_replay.restype = ctypes.c_int64
    lib.orc_sgd_replay_mt.argtypes = [ctypes.c_int64, ctypes.c_int64, P, P, P, P, P, P, ctypes.c_int,
                                      ctypes.c_double, ctypes.c_double, P, P, P, ctypes.c_int]
    lib.orc_sgd_replay_mt.restype = ctypes.c_int64
    lib.orc_hx_public.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P]
    lib.orc_hx_public.restype = ctypes.c_int
    PP = ctypes.POINTER(ctypes.c_void_p)
    I64P = ctypes.POINTER(ctypes.c_int64)
    lib.orc_gen_tensor.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int64, P, ctypes.c_int,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                   PP, PP, I64P, PP, PP, I64P]
    lib.orc_gen_tensor.restype = ctypes.c_int
    lib.orc_gen_free.argtypes = [P]
    lib.orc_shuffle.argtypes = [P, P, ctypes.c_int64, ctypes.c_uint32]
    lib.orc_shuffle.restype = ctypes.c_int
    _lib = lib
    return lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Schedule:
    """Blocking + strata + balanced GPU schedule of one input, as the
    reference's block_problem would produce it (block.cu:1233-1287)."""

    def __init__(self, xyz, I, J, K, block_s, pss=8, resident=0):
        lib = _load()
        self.xyz = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
        h = ctypes.c_void_p()
        rc = lib.orc_build(_ptr(self.xyz), self.xyz.shape[0], I, J, K, block_s, pss, resident,
                           ctypes.byref(h))
        if rc != 0:
            raise RuntimeError("oracle build failed with status %d" % rc)
        self._h = h
        info = np.zeros(8, np.int32)
        cnt = np.zeros(4, np.int64)
        gmax = np.zeros(3, np.int32)
        lib.orc_info(h, _ptr(info), _ptr(cnt), _ptr(gmax))
        (self.nblocks, self.nstrata, self.max_parallel_cf, self.target, self.ngroups,
         self.nslots, self.max_parallel, _) = [int(v) for v in info]
        self.counters = dict(splits=int(cnt[0]), flag0=int(cnt[1]), duplicating=int(cnt[2]),
                             empty_resplit=int(cnt[3]))
        self.global_levels = [int(v) for v in gmax]
        meta = np.zeros((self.nblocks, 4), np.int32)
        codes = np.zeros((self.nblocks, 3), np.uint64)
        lib.orc_blocks(h, _ptr(meta), _ptr(codes))
        self.block_nnz = meta[:, 0].copy()
        self.block_levels = meta[:, 1:4].copy()
        self.block_codes = codes
        self.block_entries = []
        buf = np.zeros(max(block_s, 1), np.int32)
        for b in range(self.nblocks):
            n = lib.orc_block_entries(h, b, _ptr(buf))
            self.block_entries.append(buf[:n].copy())
        soff = np.zeros(self.nstrata + 1, np.int32)
        sids = np.zeros(max(int(self.block_nnz.astype(bool).sum()), 1), np.int32)
        lib.orc_strata_arrays(h, _ptr(soff), _ptr(sids))
        self.strata = [sids[soff[i]:soff[i + 1]].tolist() for i in range(self.nstrata)]
        goff = np.zeros(self.ngroups + 1, np.int32)
        gids = np.zeros(max(self.nslots, 1), np.int32)
        coe = np.zeros((max(self.nslots, 1), 3), np.float64)
        lib.orc_groups(h, _ptr(goff), _ptr(gids), _ptr(coe))
        self.group_off = goff
        self.slot_ids = gids[: self.nslots]
        self.slot_coe = coe[: self.nslots]
        self.groups = [gids[goff[i]:goff[i + 1]].tolist() for i in range(self.ngroups)]

    def id_string(self, b, axis):
        """Bit string of a block id on one axis, as the reference prints it."""
        L = int(self.block_levels[b, axis])
        code = int(self.block_codes[b, axis])
        bits = "0" + (format(code, "0%db" % (L - 1)) if L > 1 else "")
        return bits

    def sgd_epoch(self, val, R, lr, reg, A, B, C):
        """One serial FP64 epoch in place on A, B, C; returns executed updates."""
        lib = _load()
        val = np.ascontiguousarray(val, dtype=np.float64)
        for M in (A, B, C):
            assert M.dtype == np.float64 and M.flags.c_contiguous
        return lib.orc_sgd_epoch(self._h, _ptr(self.xyz), _ptr(val), R, lr, reg, _ptr(A),
                                 _ptr(B), _ptr(C))

    def lf_epoch(self, val, R, lr, reg, A, B, C):
        """One serial FP64 epoch of the lock-free variant in place on A, B, C."""
        lib = _load()
        val = np.ascontiguousarray(val, dtype=np.float64)
        for M in (A, B, C):
            assert M.dtype == np.float64 and M.flags.c_contiguous
        return lib.orc_lf_epoch(self._h, _ptr(self.xyz), _ptr(val), R, lr, reg, _ptr(A), _ptr(B), _ptr(C))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib is not None:
            _lib.orc_free(h)
            self._h = None


def metrics(xyz, val, R, A, B, C):
    """(SSE, SAE, sum ref^2) in FP64, serial order."""
    lib = _load()
    xyz = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
    val = np.ascontiguousarray(val, dtype=np.float64)
    out = np.zeros(3, np.float64)
    lib.orc_metrics(_ptr(xyz), _ptr(val), xyz.shape[0], R, _ptr(A), _ptr(B), _ptr(C), _ptr(out))
    return out


def rmse_mae_er(xyz, val, R, A, B, C):
    """compute_metrics_gpu's outputs (sgd_Kernel.cu:136-201)."""
    n = len(val)
    if n == 0:
        return float("nan"), float("nan"), float("nan")
    sse, sae, r2 = metrics(xyz, val, R, A, B, C)
    return float(np.sqrt(sse / n)), float(sae / n), float(sse / r2) if r2 > 0 else float("nan")


def hx(end, level, num):
    lib = _load()
    out = np.zeros(1, np.int64)
    rc = lib.orc_hx_public(end, level, num, _ptr(out))
    if rc:
        raise OverflowError("hx out of range")
    return int(out[0])


class FlatSchedule:
    """A schedule given as flat arrays (groups -> slots -> entry indices), for
    replaying the reference update rule on host cores (the CPU baseline)."""

    def __init__(self, group_off, slot_blocks, slot_coe, block_entries, max_updates=None):
        """max_updates: keep only the leading groups, up to the first group
        boundary at or past this many updates (a bounded sample of a large
        schedule); None keeps them all."""
        goff = np.asarray(group_off, np.int64)
        cache = {}
        parts = []
        total = 0
        ngroups = len(goff) - 1
        for g in range(ngroups):
            if max_updates is not None and total >= max_updates:
                ngroups = g
                break
            for k in range(int(goff[g]), int(goff[g + 1])):
                b = int(slot_blocks[k])
                if b not in cache:
                    cache[b] = np.asarray(block_entries(b), np.int32)
                parts.append(cache[b])
                total += len(cache[b])
        self.goff = np.ascontiguousarray(goff[: ngroups + 1])
        nslots = int(self.goff[-1]) if ngroups > 0 else 0
        self.soff = np.zeros(nslots + 1, np.int64)
        np.cumsum([len(p) for p in parts[:nslots]], out=self.soff[1:])
        self.ent = np.ascontiguousarray(np.concatenate(parts[:nslots]) if nslots else np.zeros(0, np.int32))
        self.coe = np.ascontiguousarray(np.asarray(slot_coe, np.float64).reshape(-1)[: 3 * nslots])
        self.nslots = nslots
        self.ngroups = ngroups

    def replay(self, xyz, val, R, lr, reg, A, B, C, s0=0, s1=None):
        lib = _load()
        s1 = self.nslots if s1 is None else s1
        xyz = np.ascontiguousarray(xyz, np.int32)
        val = np.ascontiguousarray(val, np.float64)
        return lib.orc_sgd_replay(s0, s1, _ptr(self.soff), _ptr(self.ent), _ptr(self.coe), _ptr(xyz),
                                  _ptr(val), R, lr, reg, _ptr(A), _ptr(B), _ptr(C))

    def replay_mt(self, xyz, val, R, lr, reg, A, B, C, threads, g0=0, g1=None):
        lib = _load()
        g1 = self.ngroups if g1 is None else g1
        xyz = np.ascontiguousarray(xyz, np.int32)
        val = np.ascontiguousarray(val, np.float64)
        return lib.orc_sgd_replay_mt(g0, g1, _ptr(self.goff), _ptr(self.soff), _ptr(self.ent),
                                     _ptr(self.coe), _ptr(xyz), _ptr(val), R, lr, reg, _ptr(A), _ptr(B),
                                     _ptr(C), threads)


def gen_tensor(I, J, K, nnz, zipf=(0.0, 0.0, 0.0), gt_rank=8, gt_std=0.5, noise_std=0.01, train_frac=0.9,
               seed=1):
    """The benchmark's synthetic tensor drawn by the oracle's restatement of
    the generator (gen.c): (train xyz, train values, test xyz, test values).
    A draw of nnz = M cells is the first M cells of a larger draw."""
    lib = _load()
    zs = np.ascontiguousarray(zipf, dtype=np.float64)
    ptrs = [ctypes.c_void_p() for _ in range(4)]
    ntr, nte = ctypes.c_int64(), ctypes.c_int64()
    rc = lib.orc_gen_tensor(I, J, K, nnz, _ptr(zs), gt_rank, gt_std, noise_std, train_frac, seed,
                            ctypes.byref(ptrs[0]), ctypes.byref(ptrs[1]), ctypes.byref(ntr),
                            ctypes.byref(ptrs[2]), ctypes.byref(ptrs[3]), ctypes.byref(nte))
    if rc != 0:
        raise RuntimeError("oracle generator failed with status %d" % rc)

    def take(p, n, dt, width):
        out = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(dt)), shape=(max(n * width, 1),))[: n * width].copy()
        lib.orc_gen_free(p)
        return out.reshape(n, width) if width > 1 else out

    tx = take(ptrs[0], ntr.value, ctypes.c_int32, 3)
    tv = take(ptrs[1], ntr.value, ctypes.c_double, 1)
    sx = take(ptrs[2], nte.value, ctypes.c_int32, 3)
    sv = take(ptrs[3], nte.value, ctypes.c_double, 1)
    return tx, tv, sx, sv


def shuffle(xyz, val, seed=42):
    """main.cpp:303-306: std::shuffle with std::mt19937(seed), in place."""
    lib = _load()
    assert xyz.dtype == np.int32 and xyz.flags.c_contiguous and val.dtype == np.float64 and val.flags.c_contiguous
    lib.orc_shuffle(_ptr(xyz), _ptr(val), len(val), seed)
    return xyz, val
