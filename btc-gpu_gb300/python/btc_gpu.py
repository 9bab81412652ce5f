"""ctypes binding of the C ABI in include/btc_gpu.h.

This is how the tests, the bench and the smoke entry drive the library; it is
also the template for the ctypes stub a Python caller of the reference would
add.  Every call goes through lib/libbtcgpu.so: there is no Python or CPU
fallback, and a missing library is an error.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "lib", "libbtcgpu.so")
CLI_PATH = os.path.join(PKG, "bin", "tensor_sgd")

F32, F64, BF16 = 0, 1, 2
NOALLOC_MAX_ENTRIES = 67108864
BLOCK_FEATURES = 10
TILE_FEATURES = 10
HOGWILD, DETERMINISTIC, STAGED, LOCKFREE = 0, 1, 2, 3
TRAIN, TEST = 0, 1


class BtcError(RuntimeError):
    def __init__(self, status, what):
        super().__init__("%s failed: %s (status %d)" % (what, _lib().btc_status_string(status).decode(), status))
        self.status = status


class Config(ctypes.Structure):
    _fields_ = [
        ("I", ctypes.c_int32), ("J", ctypes.c_int32), ("K", ctypes.c_int32),
        ("epochs", ctypes.c_int32), ("rank", ctypes.c_int32),
        ("lr", ctypes.c_double), ("reg", ctypes.c_double),
        ("block_s", ctypes.c_int32), ("thread_size", ctypes.c_int32),
        ("parallel_sequence_size", ctypes.c_int32), ("requested_gpu_count", ctypes.c_int32),
        ("dtype", ctypes.c_int32), ("mode", ctypes.c_int32), ("device", ctypes.c_int32),
        ("resident_blocks", ctypes.c_int32), ("chunk", ctypes.c_int32),
        ("host_threads", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32),
        ("row_repeat", ctypes.c_int32), ("reserved", ctypes.c_int32 * 5),
    ]


class ScheduleSummary(ctypes.Structure):
    _fields_ = [
        ("num_blocks", ctypes.c_int32), ("nonempty_blocks", ctypes.c_int32),
        ("num_strata", ctypes.c_int32), ("max_parallel_cf", ctypes.c_int32),
        ("target_gpu_blocks", ctypes.c_int32), ("num_groups", ctypes.c_int32),
        ("num_slots", ctypes.c_int32), ("max_parallel", ctypes.c_int32),
        ("scheduled_updates", ctypes.c_int64), ("train_nnz", ctypes.c_int64),
        ("global_levels", ctypes.c_int32 * 3), ("reserved", ctypes.c_int32),
        ("build_seconds", ctypes.c_double * 3),
    ]


class Metrics(ctypes.Structure):
    _fields_ = [("rmse", ctypes.c_double), ("mae", ctypes.c_double), ("er", ctypes.c_double),
                ("sse", ctypes.c_double), ("sae", ctypes.c_double), ("ref2", ctypes.c_double),
                ("count", ctypes.c_int64)]


class EpochStats(ctypes.Structure):
    _fields_ = [("kernel_ms", ctypes.c_double), ("updates", ctypes.c_int64),
                ("launches", ctypes.c_int32), ("device_status", ctypes.c_int32)]


class GenSpec(ctypes.Structure):
    _fields_ = [("I", ctypes.c_int32), ("J", ctypes.c_int32), ("K", ctypes.c_int32),
                ("nnz", ctypes.c_int64), ("zipf_s", ctypes.c_double * 3),
                ("gt_rank", ctypes.c_int32), ("gt_std", ctypes.c_double),
                ("noise_std", ctypes.c_double), ("train_frac", ctypes.c_double),
                ("seed", ctypes.c_uint64), ("threads", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 3)]


# every symbol the header declares, with its argument types
P = ctypes.c_void_p
I32, I64, U32, U64, D = ctypes.c_int32, ctypes.c_int64, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_double
SIGNATURES = {
    "btc_status_string": ([ctypes.c_int], ctypes.c_char_p),
    "btc_abi_version": ([], I32),
    "btc_config_default": ([P], ctypes.c_int),
    "btc_config_validate": ([P], ctypes.c_int),
    "btc_read_entries": ([ctypes.c_char_p, I32, I32, I32, I32, P, P, P, P], ctypes.c_int),
    "btc_read_entries_cached": ([ctypes.c_char_p, ctypes.c_char_p, I32, I32, I32, I32, P, P, P, P, P],
                                ctypes.c_int),
    "btc_free": ([P], None),
    "btc_shuffle_entries": ([P, P, I64, U32], ctypes.c_int),
    "btc_schedule_build": ([P, P, I64, P], ctypes.c_int),
    "btc_schedule_build_learned": ([P, P, I64, P, P], ctypes.c_int),
    "btc_schedule_block_boxes": ([P, P], ctypes.c_int),
    "btc_ctx_block_profile": ([P, P, P, ctypes.POINTER(I64)], ctypes.c_int),
    "btc_mlp_inputs": ([P], I32),
    "btc_ctx_set_rates": ([P, ctypes.c_double, ctypes.c_double], ctypes.c_int),
    "btc_schedule_summarize": ([P, P], ctypes.c_int),
    "btc_schedule_blocks": ([P, P, P], ctypes.c_int),
    "btc_schedule_block_entries": ([P, I32, P, P], ctypes.c_int),
    "btc_schedule_strata": ([P, P, P], ctypes.c_int),
    "btc_schedule_groups": ([P, P, P, P], ctypes.c_int),
    "btc_schedule_write_report": ([P, P, ctypes.c_char_p], ctypes.c_int),
    "btc_schedule_free": ([P], None),
    "btc_ctx_create": ([P, P, P, P, I64, P, P, I64, P], ctypes.c_int),
    "btc_ctx_set_factors": ([P, I32, P], ctypes.c_int),
    "btc_ctx_get_factors": ([P, I32, P], ctypes.c_int),
    "btc_ctx_init_factors": ([P, U64, D, D], ctypes.c_int),
    "btc_train_epoch": ([P, P], ctypes.c_int),
    "btc_train_epochs": ([P, I32, P], ctypes.c_int),
    "btc_eval": ([P, I32, P], ctypes.c_int),
    "btc_host_alloc": ([P, I64], ctypes.c_int),
    "btc_device_count": ([P], ctypes.c_int),
    "btc_ctx_tile_count": ([P, P], ctypes.c_int),
    "btc_mlp_create": ([I32, I32, U64, I32, P], ctypes.c_int),
    "btc_mlp_destroy": ([P], ctypes.c_int),
    "btc_mlp_param_count": ([P, P], ctypes.c_int),
    "btc_mlp_get_params": ([P, P], ctypes.c_int),
    "btc_mlp_set_params": ([P, P], ctypes.c_int),
    "btc_mlp_gradient": ([P, P, P, I64, P, P], ctypes.c_int),
    "btc_mlp_train": ([P, P, P, I64, I32, ctypes.c_float, P], ctypes.c_int),
    "btc_mlp_predict": ([P, P, I64, P], ctypes.c_int),
    "btc_ctx_learn_work_units": ([P, P, I32, I32, P], ctypes.c_int),
    "btc_ctx_autotune": ([P, I32, P], ctypes.c_int),
    "btc_batch_create": ([P, I32, P], ctypes.c_int),
    "btc_batch_train_epochs": ([P, I32, I32, P], ctypes.c_int),
    "btc_batch_destroy": ([P], ctypes.c_int),
    "btc_ctx_slot_tiles": ([P, P, P], ctypes.c_int),
    "btc_ctx_set_work_units": ([P, P, I32], ctypes.c_int),
    "btc_ctx_tile_features": ([P, P], ctypes.c_int),
    "btc_train_epoch_profiled": ([P, P, P], ctypes.c_int),
    "btc_eval_sums_noalloc": ([P, P, I64, P, P, P, I32, I32, I64, P, P], ctypes.c_int),
    "btc_device_info": ([I32, ctypes.c_char_p, P, P], ctypes.c_int),
    "btc_host_free": ([P], None),
    "btc_ctx_stream": ([P], P),
    "btc_ctx_destroy": ([P], ctypes.c_int),
    "btc_train_epoch_host": ([P, P, P, P, P, P], ctypes.c_int),
    "btc_gen_tensor": ([P, P, P, P, P, P, P], ctypes.c_int),
}

_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libbtcgpu.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
        lib = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = lib
    return _LIB


def lib():
    return _lib()


def _ck(status, what):
    if status != 0:
        raise BtcError(status, what)


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def config(**kw):
    c = Config()
    _ck(_lib().btc_config_default(ctypes.byref(c)), "btc_config_default")
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def validate(cfg):
    return _lib().btc_config_validate(ctypes.byref(cfg))


def shuffle(xyz, val, seed=42):
    """Permute (xyz, val) in place exactly as the reference's main does."""
    xyz = np.ascontiguousarray(xyz, dtype=np.int32)
    val = np.ascontiguousarray(val, dtype=np.float64)
    _ck(_lib().btc_shuffle_entries(_p(xyz), _p(val), len(val), seed), "btc_shuffle_entries")
    return xyz, val


def read_entries(path, coord_base, I, J, K, cache=None):
    """Entries of a text file as (xyz int32 [n, 3], val float64 [n]).  With
    `cache`, through btc_read_entries_cached; the returned arrays are the same
    and `read_entries.from_cache` tells whether the cache was used."""
    L = _lib()
    px, pv = ctypes.c_void_p(), ctypes.c_void_p()
    n, line = ctypes.c_int64(), ctypes.c_int64()
    if cache is None:
        st = L.btc_read_entries(path.encode(), coord_base, I, J, K, ctypes.byref(px), ctypes.byref(pv),
                                ctypes.byref(n), ctypes.byref(line))
        read_entries.from_cache = False
    else:
        fc = ctypes.c_int32()
        st = L.btc_read_entries_cached(path.encode(), cache.encode(), coord_base, I, J, K, ctypes.byref(px),
                                       ctypes.byref(pv), ctypes.byref(n), ctypes.byref(line), ctypes.byref(fc))
        read_entries.from_cache = bool(fc.value)
    if st != 0:
        err = BtcError(st, "btc_read_entries")
        err.line = line.value
        raise err
    try:
        xyz = np.ctypeslib.as_array(ctypes.cast(px, ctypes.POINTER(ctypes.c_int32)), (max(n.value, 1) * 3,))
        val = np.ctypeslib.as_array(ctypes.cast(pv, ctypes.POINTER(ctypes.c_double)), (max(n.value, 1),))
        return xyz[: 3 * n.value].reshape(-1, 3).copy(), val[: n.value].copy()
    finally:
        L.btc_free(px)
        L.btc_free(pv)


def gen_tensor(I, J, K, nnz, zipf=(0.0, 0.0, 0.0), gt_rank=8, gt_std=0.5, noise_std=0.01,
               train_frac=0.9, seed=20261203, threads=0):
    """Synthetic tensor: returns (train_xyz, train_val, test_xyz, test_val)."""
    L = _lib()
    sp = GenSpec()
    sp.I, sp.J, sp.K, sp.nnz = I, J, K, nnz
    for a in range(3):
        sp.zipf_s[a] = zipf[a]
    sp.gt_rank, sp.gt_std, sp.noise_std, sp.train_frac = gt_rank, gt_std, noise_std, train_frac
    sp.seed, sp.threads = seed, threads
    ptrs = [ctypes.c_void_p() for _ in range(4)]
    ntr, nte = ctypes.c_int64(), ctypes.c_int64()
    _ck(L.btc_gen_tensor(ctypes.byref(sp), ctypes.byref(ptrs[0]), ctypes.byref(ptrs[1]),
                         ctypes.byref(ntr), ctypes.byref(ptrs[2]), ctypes.byref(ptrs[3]),
                         ctypes.byref(nte)), "btc_gen_tensor")
    out = []
    try:
        for k, (n, cols) in enumerate(((ntr.value, 3), (ntr.value, 1), (nte.value, 3), (nte.value, 1))):
            ct = ctypes.c_int32 if cols == 3 else ctypes.c_double
            a = np.ctypeslib.as_array(ctypes.cast(ptrs[k], ctypes.POINTER(ct)), (max(n, 1) * cols,))
            a = a[: n * cols].copy()
            out.append(a.reshape(-1, 3) if cols == 3 else a)
    finally:
        for p in ptrs:
            L.btc_free(p)
    return tuple(out)


class LearnReport(ctypes.Structure):
    _fields_ = [("plain_ms", ctypes.c_double), ("learned_ms", ctypes.c_double),
                ("model_loss", ctypes.c_double), ("model_r2", ctypes.c_double),
                ("samples", ctypes.c_int64), ("units", ctypes.c_int32), ("kept", ctypes.c_int32)]


class AutotuneReport(ctypes.Structure):
    _fields_ = [("lanes_per_entry", ctypes.c_int32), ("vectors_per_lane", ctypes.c_int32),
                ("ctas_per_sm", ctypes.c_int32), ("candidates", ctypes.c_int32),
                ("best_ms", ctypes.c_double), ("default_ms", ctypes.c_double)]


class MLP:
    """The cost model: n_in -> 32 -> 32 -> 1 (tanh), trained on the GPU."""

    def __init__(self, n_in=None, hidden=32, seed=1, device=0):
        n_in = TILE_FEATURES if n_in is None else n_in
        h = ctypes.c_void_p()
        _ck(_lib().btc_mlp_create(n_in, hidden, seed, device, ctypes.byref(h)), "btc_mlp_create")
        self._h = h
        self.n_in = n_in
        n = ctypes.c_int64()
        _ck(_lib().btc_mlp_param_count(h, ctypes.byref(n)), "btc_mlp_param_count")
        self.nparam = n.value

    @property
    def handle(self):
        return self._h

    def params(self):
        p = np.zeros(self.nparam, np.float32)
        _ck(_lib().btc_mlp_get_params(self._h, _p(p)), "btc_mlp_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        _ck(_lib().btc_mlp_set_params(self._h, _p(p)), "btc_mlp_set_params")

    def gradient(self, x, y):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        g = np.zeros(self.nparam, np.float32)
        loss = ctypes.c_double()
        _ck(_lib().btc_mlp_gradient(self._h, _p(x), _p(y), len(y), _p(g), ctypes.byref(loss)), "btc_mlp_gradient")
        return g, loss.value

    def train(self, x, y, steps, lr=3e-3):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        loss = ctypes.c_double()
        _ck(_lib().btc_mlp_train(self._h, _p(x), _p(y), len(y), steps, lr, ctypes.byref(loss)), "btc_mlp_train")
        return loss.value

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros(len(x), np.float32)
        _ck(_lib().btc_mlp_predict(self._h, _p(x), len(x), _p(y)), "btc_mlp_predict")
        return y

    def close(self):
        if getattr(self, "_h", None):
            _lib().btc_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Several staged contexts trained as one persistent launch per epoch."""

    def __init__(self, contexts):
        self.contexts = list(contexts)
        arr = (ctypes.c_void_p * len(self.contexts))(*[c.handle.value for c in self.contexts])
        h = ctypes.c_void_p()
        _ck(_lib().btc_batch_create(arr, len(self.contexts), ctypes.byref(h)), "btc_batch_create")
        self._h = h

    def train_epochs(self, n, graph=True):
        st = EpochStats()
        _ck(_lib().btc_batch_train_epochs(self._h, n, 1 if graph else 0, ctypes.byref(st)), "btc_batch_train_epochs")
        return st

    def close(self):
        if getattr(self, "_h", None):
            _lib().btc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PinnedArray:
    """float64 array in page-locked host memory (btc_host_alloc)."""

    def __init__(self, shape):
        n = int(np.prod(shape))
        self._p = ctypes.c_void_p()
        _ck(_lib().btc_host_alloc(ctypes.byref(self._p), max(n, 1) * 8), "btc_host_alloc")
        buf = (ctypes.c_double * max(n, 1)).from_address(self._p.value)
        self.array = np.frombuffer(buf, np.float64)[:n].reshape(shape)

    def free(self):
        if self._p:
            self.array = None
            _lib().btc_host_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Schedule:
    """Host schedule: block_problem's blocking, strata and balancing; with
    learned=True the learned blocking (btc_schedule_build_learned) instead,
    its split axes chosen by `model` (an MLP over BLOCK_FEATURES, or None for
    the axes in turn)."""

    def __init__(self, cfg, xyz, learned=False, model=None):
        self.cfg = cfg
        self.learned = learned
        self.xyz = np.ascontiguousarray(xyz, dtype=np.int32).reshape(-1, 3)
        h = ctypes.c_void_p()
        if learned:
            _ck(_lib().btc_schedule_build_learned(ctypes.byref(cfg), _p(self.xyz), self.xyz.shape[0],
                                                  model.handle if model is not None else None, ctypes.byref(h)),
                "btc_schedule_build_learned")
        else:
            _ck(_lib().btc_schedule_build(ctypes.byref(cfg), _p(self.xyz), self.xyz.shape[0], ctypes.byref(h)),
                "btc_schedule_build")
        self._h = h
        s = ScheduleSummary()
        _ck(_lib().btc_schedule_summarize(h, ctypes.byref(s)), "btc_schedule_summarize")
        self.summary = s

    @property
    def handle(self):
        return self._h

    def blocks(self):
        n = self.summary.num_blocks
        meta = np.zeros((n, 4), np.int32)
        codes = np.zeros((n, 3), np.uint64)
        _ck(_lib().btc_schedule_blocks(self._h, _p(meta), _p(codes)), "btc_schedule_blocks")
        return meta, codes

    def boxes(self):
        """[lo, hi) per axis of every block of a learned schedule, (blocks, 3, 2)."""
        out = np.zeros((self.summary.num_blocks, 3, 2), np.int32)
        _ck(_lib().btc_schedule_block_boxes(self._h, _p(out)), "btc_schedule_block_boxes")
        return out

    def block_entries(self, b):
        cap = ctypes.c_int32(self.cfg.block_s)
        out = np.zeros(max(self.cfg.block_s, 1), np.int32)
        _ck(_lib().btc_schedule_block_entries(self._h, b, _p(out), ctypes.byref(cap)), "btc_schedule_block_entries")
        return out[: cap.value].copy()

    def strata(self):
        s = self.summary
        off = np.zeros(s.num_strata + 1, np.int32)
        ids = np.zeros(max(s.nonempty_blocks, 1), np.int32)
        _ck(_lib().btc_schedule_strata(self._h, _p(off), _p(ids)), "btc_schedule_strata")
        return [ids[off[i]:off[i + 1]].tolist() for i in range(s.num_strata)]

    def groups(self):
        s = self.summary
        off = np.zeros(s.num_groups + 1, np.int32)
        ids = np.zeros(max(s.num_slots, 1), np.int32)
        coe = np.zeros((max(s.num_slots, 1), 3), np.float64)
        _ck(_lib().btc_schedule_groups(self._h, _p(off), _p(ids), _p(coe)), "btc_schedule_groups")
        return off, ids[: s.num_slots], coe[: s.num_slots]

    def write_report(self, path):
        _ck(_lib().btc_schedule_write_report(self._h, ctypes.byref(self.cfg), path.encode()),
            "btc_schedule_write_report")

    def close(self):
        if getattr(self, "_h", None):
            _lib().btc_schedule_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """Device state of one training run (sgd_train's allocations)."""

    def __init__(self, cfg, schedule, train_xyz, train_val, test_xyz, test_val):
        self.cfg = cfg
        self._keep = [np.ascontiguousarray(a) for a in (train_xyz, train_val, test_xyz, test_val)]
        tx = np.ascontiguousarray(train_xyz, np.int32)
        tv = np.ascontiguousarray(train_val, np.float64)
        sx = np.ascontiguousarray(test_xyz, np.int32)
        sv = np.ascontiguousarray(test_val, np.float64)
        h = ctypes.c_void_p()
        _ck(_lib().btc_ctx_create(ctypes.byref(cfg), schedule.handle, _p(tx), _p(tv), len(tv), _p(sx),
                                  _p(sv), len(sv), ctypes.byref(h)), "btc_ctx_create")
        self._h = h
        self.rows = (cfg.I, cfg.J, cfg.K)

    @property
    def handle(self):
        return self._h

    def set_factors(self, mode, arr):
        arr = np.ascontiguousarray(arr, np.float64)
        assert arr.shape == (self.rows[mode], self.cfg.rank)
        _ck(_lib().btc_ctx_set_factors(self._h, mode, _p(arr)), "btc_ctx_set_factors")

    def get_factors(self, mode):
        out = np.zeros((self.rows[mode], self.cfg.rank), np.float64)
        _ck(_lib().btc_ctx_get_factors(self._h, mode, _p(out)), "btc_ctx_get_factors")
        return out

    def init_factors(self, seed, lo=0.0, hi=0.1):
        _ck(_lib().btc_ctx_init_factors(self._h, seed, lo, hi), "btc_ctx_init_factors")

    def train_epoch(self):
        st = EpochStats()
        _ck(_lib().btc_train_epoch(self._h, ctypes.byref(st)), "btc_train_epoch")
        return st

    def train_epochs(self, n):
        st = EpochStats()
        _ck(_lib().btc_train_epochs(self._h, n, ctypes.byref(st)), "btc_train_epochs")
        return st

    def tile_features(self):
        n = ctypes.c_int64()
        _ck(_lib().btc_ctx_tile_count(self._h, ctypes.byref(n)), "btc_ctx_tile_count")
        f = np.zeros((n.value, TILE_FEATURES), np.float32)
        _ck(_lib().btc_ctx_tile_features(self._h, _p(f)), "btc_ctx_tile_features")
        return f

    def slot_tiles(self, nslots):
        t0 = np.zeros(max(nslots, 1), np.int32)
        tn = np.zeros(max(nslots, 1), np.int32)
        _ck(_lib().btc_ctx_slot_tiles(self._h, _p(t0), _p(tn)), "btc_ctx_slot_tiles")
        return t0[:nslots], tn[:nslots]

    def set_work_units(self, unit_off):
        u = np.ascontiguousarray(unit_off, np.int32)
        _ck(_lib().btc_ctx_set_work_units(self._h, _p(u), len(u) - 1), "btc_ctx_set_work_units")

    def learn_work_units(self, model, train_steps=300, trial_epochs=3):
        r = LearnReport()
        _ck(_lib().btc_ctx_learn_work_units(self._h, model.handle, train_steps, trial_epochs, ctypes.byref(r)),
            "btc_ctx_learn_work_units")
        return r

    def autotune(self, epochs_per_candidate=2):
        r = AutotuneReport()
        _ck(_lib().btc_ctx_autotune(self._h, epochs_per_candidate, ctypes.byref(r)), "btc_ctx_autotune")
        return r

    def set_rates(self, lr, reg):
        _ck(_lib().btc_ctx_set_rates(self._h, lr, reg), "btc_ctx_set_rates")

    def block_profile(self):
        """(features, log microseconds) of every scheduled block, from one
        profiled training epoch (the block cost model's training samples)."""
        n = ctypes.c_int64(0)
        _lib().btc_ctx_block_profile(self._h, None, None, ctypes.byref(n))
        f = np.zeros((max(n.value, 1), BLOCK_FEATURES), np.float32)
        y = np.zeros(max(n.value, 1), np.float32)
        _ck(_lib().btc_ctx_block_profile(self._h, _p(f), _p(y), ctypes.byref(n)), "btc_ctx_block_profile")
        return f[: n.value], y[: n.value]

    def train_epoch_profiled(self):
        n = ctypes.c_int64()
        _ck(_lib().btc_ctx_tile_count(self._h, ctypes.byref(n)), "btc_ctx_tile_count")
        ns = np.zeros(max(n.value, 1), np.uint32)
        st = EpochStats()
        _ck(_lib().btc_train_epoch_profiled(self._h, _p(ns), ctypes.byref(st)), "btc_train_epoch_profiled")
        return st, ns[: n.value]

    def eval(self, split=TEST):
        m = Metrics()
        _ck(_lib().btc_eval(self._h, split, ctypes.byref(m)), "btc_eval")
        return m

    def train_epoch_host(self, A, B, C, test=True):
        st, m = EpochStats(), Metrics()
        _ck(_lib().btc_train_epoch_host(self._h, _p(A), _p(B), _p(C), ctypes.byref(st),
                                        ctypes.byref(m) if test else None), "btc_train_epoch_host")
        return st, m

    @property
    def stream(self):
        return _lib().btc_ctx_stream(self._h)

    def close(self):
        if getattr(self, "_h", None):
            _lib().btc_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
