"""ctypes binding of libgpx (include/gpx.h).

The library is the product: every exploration here runs the CUDA kernels in
``_lib/libgpx.so``.  Loading fails loudly when the library has not been built;
there is no fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Dict, List, Optional, Sequence

import numpy as np

from .build import LIB

GPX_OK = 0
GPX_ERR_UNSUPPORTED = 7
STATUS = ["ok", "parse", "no_gpu", "cuda", "table_full", "timeout", "invalid", "unsupported", "store_full", "nomem"]
PROP_NONE, PROP_DEADLOCK, PROP_SAFETY, PROP_LIVENESS = 0, 1, 2, 3
PROPERTIES = {"none": PROP_NONE, "deadlock": PROP_DEADLOCK, "safety": PROP_SAFETY, "liveness": PROP_LIVENESS}
VERDICTS = {v: k for k, v in PROPERTIES.items()}
STOPS = ["done", "violation", "budget", "error"]

EXPORTS = [
    "gpx_status_string", "gpx_abi_version", "gpx_device_info_get", "gpx_options_init", "gpx_model_load",
    "gpx_model_load_file", "gpx_model_from_words", "gpx_model_info_get", "gpx_model_free", "gpx_explore",
    "gpx_explorer_create", "gpx_explorer_run", "gpx_explorer_set_model", "gpx_explorer_destroy",
    "gpx_result_free", "gpx_explorer_dump", "gpx_explore_noalloc", "gpx_random_gather_probe", "gpx_random_insert_probe",
    "gpx_selftest_bounded_wait", "gpx_batch_options_init", "gpx_batch_job_init", "gpx_batch_explore",
    "gpx_explorer_set_por_model", "gpx_explorer_set_por_log", "gpx_explorer_get_por_log",
    "gpx_train_options_init", "gpx_por_train", "gpx_por_grad",
]

POR_F, POR_H = 40, 64


class PorModel(C.Structure):
    """gpx_por_model: int8 w1[64][40], s1[64], b1[64], int8 w2[64], s2, b2."""
    _fields_ = [("w1", (C.c_int8 * POR_F) * POR_H), ("s1", C.c_float * POR_H), ("b1", C.c_float * POR_H),
                ("w2", C.c_int8 * POR_H), ("s2", C.c_float), ("b2", C.c_float)]

    def to_bytes(self) -> bytes:
        return bytes(memoryview(self))

    @classmethod
    def from_bytes(cls, b: bytes) -> "PorModel":
        m = cls()
        C.memmove(C.addressof(m), b, C.sizeof(cls))
        return m


class PorLogRow(C.Structure):
    _fields_ = [("x", C.c_uint8 * POR_F), ("succ", C.c_uint32), ("new_succ", C.c_uint32), ("state_tag", C.c_uint32),
                ("popc", C.c_uint8), ("cample_choice", C.c_uint8), ("pad", C.c_uint8 * 2)]


POR_LOG_DTYPE = np.dtype([("x", np.uint8, (POR_F,)), ("succ", np.uint32), ("new_succ", np.uint32),
                          ("state_tag", np.uint32), ("popc", np.uint8), ("cample_choice", np.uint8),
                          ("pad", np.uint8, (2,))])


class TrainOptions(C.Structure):
    _fields_ = [("struct_size", C.c_uint32), ("device", C.c_int32), ("epochs", C.c_uint32), ("batch", C.c_uint32),
                ("lr", C.c_float), ("weight_decay", C.c_float), ("seed", C.c_uint64)]


class Options(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32), ("blocks", C.c_int32), ("threads", C.c_int32),
        ("kernel_iters", C.c_int32), ("verbosity", C.c_int32), ("q_words", C.c_uint64),
        ("por", C.c_int32), ("cycle_proviso", C.c_int32), ("property", C.c_int32), ("device", C.c_int32),
        ("seed", C.c_uint64), ("max_states", C.c_uint64), ("store_states", C.c_uint64),
        ("collect_states", C.c_int32), ("bucket_bytes", C.c_int32),
        ("launch_graph", C.c_int32), ("prune_commuting", C.c_int32), ("set_hash", C.c_int32),
    ]


class Result(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32), ("status", C.c_int32), ("stopped", C.c_int32), ("verdict", C.c_int32),
        ("states", C.c_uint64), ("nlevels", C.c_uint32), ("level_counts", C.POINTER(C.c_uint64)),
        ("transitions", C.c_uint64), ("probes", C.c_uint64), ("launches", C.c_uint64),
        ("explore_ms", C.c_double), ("setup_ms", C.c_double), ("set_hash", C.c_uint64),
        ("key_words", C.c_uint32), ("table_count", C.c_uint64), ("lookups", C.c_uint64),
        ("expanded", C.c_uint64), ("kernel_ms", C.c_double), ("states_buf", C.POINTER(C.c_uint32)),
        ("table_slots", C.c_uint64), ("slot_bytes", C.c_uint32), ("blocks", C.c_uint32), ("threads", C.c_uint32),
        ("inserts", C.c_uint64), ("evictions", C.c_uint64),
        ("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64), ("live_states", C.c_uint64), ("live_ms", C.c_double),
        ("live_rounds", C.c_uint64), ("table_generation", C.c_uint32), ("table_cleared", C.c_int32),
        ("pruned", C.c_uint64), ("overflowed", C.c_uint64), ("evict_ms", C.c_double),
    ]


class BatchJob(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32), ("property", C.c_int32), ("por", C.c_int32), ("cycle_proviso", C.c_int32),
        ("max_states", C.c_uint64), ("capacity", C.c_uint64),
    ]


class BatchItem(C.Structure):
    _fields_ = [
        ("status", C.c_int32), ("stopped", C.c_int32), ("verdict", C.c_int32), ("nlevels", C.c_uint32),
        ("states", C.c_uint64), ("set_hash", C.c_uint64), ("capacity", C.c_uint64),
        ("completion_ms", C.c_double), ("admissions", C.c_uint32), ("slot_bytes", C.c_uint32),
    ]


class BatchOptions(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32), ("device", C.c_int32), ("blocks", C.c_int32), ("threads", C.c_int32),
        ("claim", C.c_int32), ("kernel_iters", C.c_int32), ("autotune", C.c_int32), ("max_admissions", C.c_int32),
        ("load_factor", C.c_double), ("seed", C.c_uint64), ("por_model", C.c_void_p),
        ("latency_sms", C.c_int32), ("prune_commuting", C.c_int32), ("narrow_slots", C.c_int32),
    ]


class BatchStats(C.Structure):
    _fields_ = [
        ("device_ms", C.c_double), ("states", C.c_uint64), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
        ("launches", C.c_uint32), ("claim", C.c_int32), ("threads", C.c_int32), ("blocks", C.c_int32),
        ("load_factor", C.c_double), ("tune_ms", C.c_double), ("kernel_iters", C.c_int32),
        ("instances_by_slot", C.c_uint32 * 3), ("narrow_slots", C.c_int32),
    ]


class ModelInfo(C.Structure):
    _fields_ = [
        ("liveness", C.c_uint32), ("nr_procs", C.c_uint32), ("bits_act", C.c_uint32),
        ("proc_nrstates", C.c_uint32), ("bits_statevector", C.c_uint32), ("nbits_offset", C.c_uint32),
        ("max_buf_ints", C.c_uint32), ("nr_trans", C.c_uint32), ("state_bits", C.c_uint32),
        ("key_words", C.c_uint32), ("firstbit", C.c_uint32 * 33), ("bits_state", C.c_uint32 * 32),
    ]


class DeviceInfo(C.Structure):
    _fields_ = [
        ("total_global_mem", C.c_uint64), ("shared_mem_per_block", C.c_int32), ("shared_mem_per_sm", C.c_int32),
        ("max_threads_per_block", C.c_int32), ("max_grid_size", C.c_int32), ("sm_count", C.c_int32),
        ("name", C.c_char * 256),
    ]


_lib: Optional[C.CDLL] = None
ABI_VERSION = 4


def load(path: str = LIB) -> C.CDLL:
    """Load libgpx.so (build it first with gpuexplore_gb300.build.build_all)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libgpx is not built ({path} missing): run __graft_entry__.build()")
    lib = C.CDLL(path)
    vp, i, u32p = C.c_void_p, C.c_int, C.POINTER(C.c_uint32)
    lib.gpx_status_string.restype = C.c_char_p
    lib.gpx_status_string.argtypes = [i]
    lib.gpx_abi_version.restype = i
    if lib.gpx_abi_version() != ABI_VERSION:  # the structures below mirror this version of gpx.h
        raise RuntimeError(f"libgpx ABI {lib.gpx_abi_version()} != {ABI_VERSION}: rebuild it")
    lib.gpx_device_info_get.argtypes = [i, C.POINTER(DeviceInfo)]
    lib.gpx_options_init.argtypes = [C.POINTER(Options)]
    lib.gpx_options_init.restype = None
    lib.gpx_model_load.argtypes = [C.c_char_p, C.POINTER(vp)]
    lib.gpx_model_load_file.argtypes = [C.c_char_p, C.POINTER(vp)]
    lib.gpx_model_from_words.argtypes = [u32p, C.c_size_t, C.POINTER(vp)]
    lib.gpx_model_info_get.argtypes = [vp, C.POINTER(ModelInfo)]
    lib.gpx_model_free.argtypes = [vp]
    lib.gpx_model_free.restype = None
    lib.gpx_explore.argtypes = [vp, C.POINTER(Options), C.POINTER(Result)]
    lib.gpx_explorer_create.argtypes = [vp, C.POINTER(Options), C.POINTER(vp)]
    lib.gpx_explorer_run.argtypes = [vp, C.POINTER(Result)]
    lib.gpx_explorer_set_model.argtypes = [vp, vp]
    lib.gpx_explorer_destroy.argtypes = [vp]
    lib.gpx_explorer_destroy.restype = None
    lib.gpx_result_free.argtypes = [C.POINTER(Result)]
    lib.gpx_result_free.restype = None
    lib.gpx_explorer_dump.argtypes = [vp, C.c_char_p]
    lib.gpx_explore_noalloc.argtypes = [vp, C.POINTER(Options), C.POINTER(C.c_uint64), C.c_uint32,
                                        C.POINTER(Result)]
    lib.gpx_random_gather_probe.argtypes = [i, C.c_uint64, C.POINTER(C.c_double)]
    lib.gpx_random_insert_probe.argtypes = [i, C.c_uint64, C.POINTER(C.c_double)]
    lib.gpx_selftest_bounded_wait.argtypes = [i, C.c_uint64, C.POINTER(C.c_uint64)]
    lib.gpx_explorer_set_por_model.argtypes = [vp, C.POINTER(PorModel)]
    lib.gpx_explorer_set_por_log.argtypes = [vp, C.c_uint64, C.c_uint32]
    lib.gpx_explorer_get_por_log.argtypes = [vp, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]
    lib.gpx_train_options_init.argtypes = [C.POINTER(TrainOptions)]
    lib.gpx_train_options_init.restype = None
    lib.gpx_por_train.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.POINTER(TrainOptions), C.POINTER(PorModel),
                                  C.POINTER(C.c_float)]
    fp = C.POINTER(C.c_float)
    lib.gpx_por_grad.argtypes = [i, fp, fp, fp, C.c_float, C.c_void_p, fp, C.c_uint32, fp, fp, fp, fp, fp]
    lib.gpx_batch_options_init.argtypes = [C.POINTER(BatchOptions)]
    lib.gpx_batch_options_init.restype = None
    lib.gpx_batch_job_init.argtypes = [C.POINTER(BatchJob)]
    lib.gpx_batch_job_init.restype = None
    lib.gpx_batch_explore.argtypes = [C.POINTER(vp), C.POINTER(BatchJob), C.c_uint32, C.POINTER(BatchOptions),
                                      C.POINTER(BatchItem), C.POINTER(C.c_uint64), C.c_uint32,
                                      C.POINTER(BatchStats)]
    _lib = lib
    return lib


class GpxError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        name = STATUS[status] if 0 <= status < len(STATUS) else str(status)
        super().__init__(f"{what}: gpx status {status} ({name})")


# Fields set on every options() call after gpx_options_init and before the
# call's own keyword arguments (e.g. {"set_hash": 1} to get the visited-set
# hash from every run of a process that compares runs).
DEFAULT_OPTIONS: Dict[str, int] = {}


def options(**kw) -> Options:
    """Options with the library defaults, then DEFAULT_OPTIONS, then the given
    fields (property may be a name)."""
    lib = load()
    o = Options()
    lib.gpx_options_init(C.byref(o))
    for k, v in list(DEFAULT_OPTIONS.items()) + list(kw.items()):
        if k == "property" and isinstance(v, str):
            v = PROPERTIES[v]
        setattr(o, k, int(v))
    return o


class Model:
    """A loaded gpf network (owned handle)."""

    def __init__(self, handle: int):
        self.handle = C.c_void_p(handle)

    @classmethod
    def from_file(cls, path: str) -> "Model":
        lib = load()
        h = C.c_void_p()
        rc = lib.gpx_model_load_file(path.encode(), C.byref(h))
        if rc != GPX_OK:
            raise GpxError(rc, f"loading {path}")
        return cls(h.value)

    @classmethod
    def from_words(cls, words: Sequence[int]) -> "Model":
        lib = load()
        if isinstance(words, np.ndarray) and words.dtype == np.uint32:
            arr = np.ascontiguousarray(words)  # a host buffer of gpf words, used in place
        else:
            arr = np.ascontiguousarray(np.asarray(words, dtype=np.uint64).astype(np.uint32))
        h = C.c_void_p()
        rc = lib.gpx_model_from_words(arr.ctypes.data_as(C.POINTER(C.c_uint32)), arr.size, C.byref(h))
        if rc != GPX_OK:
            raise GpxError(rc, "parsing gpf words")
        return cls(h.value)

    def info(self) -> ModelInfo:
        inf = ModelInfo()
        rc = load().gpx_model_info_get(self.handle, C.byref(inf))
        if rc != GPX_OK:
            raise GpxError(rc, "model info")
        return inf

    def close(self) -> None:
        if self.handle:
            load().gpx_model_free(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _result_dict(r: Result) -> Dict:
    levels = [int(r.level_counts[i]) for i in range(r.nlevels)] if r.level_counts else []
    d = {
        "status": int(r.status), "stopped": STOPS[r.stopped] if 0 <= r.stopped < 4 else str(r.stopped),
        "verdict": VERDICTS.get(int(r.verdict), str(r.verdict)), "states": int(r.states), "levels": levels,
        "transitions": int(r.transitions), "probes": int(r.probes), "lookups": int(r.lookups),
        "inserts": int(r.inserts), "evictions": int(r.evictions),
        "h2d_bytes": int(r.h2d_bytes), "d2h_bytes": int(r.d2h_bytes), "live_states": int(r.live_states),
        "live_ms": float(r.live_ms), "live_rounds": int(r.live_rounds),
        "table_generation": int(r.table_generation), "table_cleared": int(r.table_cleared),
        "pruned": int(r.pruned), "overflowed": int(r.overflowed), "evict_ms": float(r.evict_ms),
        "expanded": int(r.expanded), "launches": int(r.launches), "explore_ms": float(r.explore_ms),
        "kernel_ms": float(r.kernel_ms), "setup_ms": float(r.setup_ms), "set_hash": f"{r.set_hash:016x}",
        "key_words": int(r.key_words), "table_count": int(r.table_count), "table_slots": int(r.table_slots),
        "slot_bytes": int(r.slot_bytes), "blocks": int(r.blocks), "threads": int(r.threads),
    }
    if r.states_buf:
        n = r.states * r.key_words
        buf = np.ctypeslib.as_array(r.states_buf, shape=(n,)).copy() if n else np.zeros(0, np.uint32)
        d["states_words"] = buf.reshape(-1, r.key_words) if r.key_words else buf
    return d


class Explorer:
    """A reusable explorer: device memory is allocated once; each run() resets it."""

    def __init__(self, model: Model, opts: Options):
        lib = load()
        self.model = model
        h = C.c_void_p()
        rc = lib.gpx_explorer_create(model.handle, C.byref(opts), C.byref(h))
        if rc != GPX_OK:
            raise GpxError(rc, "creating explorer")
        self.handle = h

    def run(self, check: bool = True) -> Dict:
        lib = load()
        r = Result()
        rc = lib.gpx_explorer_run(self.handle, C.byref(r))
        try:
            d = _result_dict(r)
        finally:
            lib.gpx_result_free(C.byref(r))
        if check and rc != GPX_OK:
            raise GpxError(rc, "exploring")
        d["rc"] = rc
        return d

    def set_model(self, model: Model) -> None:
        rc = load().gpx_explorer_set_model(self.handle, model.handle)
        if rc != GPX_OK:
            raise GpxError(rc, "replacing model")
        self.model = model

    def set_por_model(self, model: Optional["PorModel"]) -> None:
        rc = load().gpx_explorer_set_por_model(self.handle, C.byref(model) if model is not None else None)
        if rc != GPX_OK:
            raise GpxError(rc, "setting the POR model")

    def set_por_log(self, capacity: int, sample_every: int) -> None:
        rc = load().gpx_explorer_set_por_log(self.handle, capacity, sample_every)
        if rc != GPX_OK:
            raise GpxError(rc, "setting the POR log")

    def get_por_log(self) -> np.ndarray:
        L = load()
        n = C.c_uint64()
        rc = L.gpx_explorer_get_por_log(self.handle, None, 0, C.byref(n))
        if rc != GPX_OK:
            raise GpxError(rc, "reading the POR log")
        out = np.zeros(n.value, dtype=POR_LOG_DTYPE)
        if n.value:
            rc = L.gpx_explorer_get_por_log(self.handle, out.ctypes.data, n.value, C.byref(n))
            if rc != GPX_OK:
                raise GpxError(rc, "reading the POR log")
        return out

    def dump(self, path: str) -> None:
        rc = load().gpx_explorer_dump(self.handle, path.encode())
        if rc != GPX_OK:
            raise GpxError(rc, "dumping")

    def close(self) -> None:
        if self.handle:
            load().gpx_explorer_destroy(self.handle)
            self.handle = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def explore(path_or_model, check: bool = True, **kw) -> Dict:
    """One-shot exploration of a gpf file (or Model) through gpx_explore."""
    lib = load()
    model = path_or_model if isinstance(path_or_model, Model) else Model.from_file(path_or_model)
    o = options(**kw)
    r = Result()
    rc = lib.gpx_explore(model.handle, C.byref(o), C.byref(r))
    try:
        d = _result_dict(r)
    finally:
        lib.gpx_result_free(C.byref(r))
    if check and rc != GPX_OK:
        raise GpxError(rc, "exploring")
    d["rc"] = rc
    return d


def explore_noalloc(model: Model, level_capacity: int = 1 << 16, check: bool = True, **kw) -> Dict:
    """gpx_explore_noalloc: the exploration with all device scratch in the library's
    static array (no allocation by the library).  The level counts land in a
    caller-owned array; the result is not passed to gpx_result_free.  `levels`
    holds the first min(nlevels, level_capacity) counts and `nlevels` the full
    count the library reported, so a truncated list is visible."""
    lib = load()
    o = options(**kw)
    levels = (C.c_uint64 * max(1, level_capacity))()
    r = Result()
    rc = lib.gpx_explore_noalloc(model.handle, C.byref(o), levels, level_capacity, C.byref(r))
    nlevels = int(r.nlevels)
    r.nlevels = min(r.nlevels, level_capacity)
    d = _result_dict(r) if rc == GPX_OK or r.level_counts else {"status": rc}
    d["nlevels"] = nlevels
    if check and rc != GPX_OK:
        raise GpxError(rc, "exploring without allocation")
    d["rc"] = rc
    return d


def random_gather_rate(device: int = 0, nbytes: int = 20 << 30) -> float:
    """Sustained random 32-byte gathers per second over an `nbytes` buffer (the
    random-access ceiling of the hash-table probes)."""
    v = C.c_double()
    rc = load().gpx_random_gather_probe(device, nbytes, C.byref(v))
    if rc != GPX_OK:
        raise GpxError(rc, "random gather probe")
    return v.value


def random_insert_rate(device: int = 0, nbytes: int = 20 << 30) -> float:
    """Sustained insert-like accesses per second (read a random 32-byte bucket,
    CAS its first slot) over an `nbytes` buffer: the ceiling of table inserts."""
    v = C.c_double()
    rc = load().gpx_random_insert_probe(device, nbytes, C.byref(v))
    if rc != GPX_OK:
        raise GpxError(rc, "random insert probe")
    return v.value


def selftest_bounded_wait(timeout_ns: int, device: int = 0):
    """Run the device-side bounded wait on a flag nothing sets; returns (status, waited_ns)."""
    w = C.c_uint64()
    rc = load().gpx_selftest_bounded_wait(device, timeout_ns, C.byref(w))
    return rc, w.value


def batch_explore(models: Sequence[Model], jobs: Sequence[Dict], level_capacity: int = 256,
                  check: bool = True, **opts):
    """gpx_batch_explore over `models` with one job dict per model (keys: property,
    por, cycle_proviso, max_states, capacity).  Returns (items, stats)."""
    lib = load()
    n = len(models)
    hs = (C.c_void_p * n)(*[m.handle.value for m in models])
    js = (BatchJob * n)()
    for k, j in enumerate(jobs):
        lib.gpx_batch_job_init(C.byref(js[k]))
        for key, v in j.items():
            if key == "property" and isinstance(v, str):
                v = PROPERTIES[v]
            setattr(js[k], key, int(v))
    o = BatchOptions()
    lib.gpx_batch_options_init(C.byref(o))
    keep = None
    for key, v in opts.items():
        if key == "por_model":
            keep = v
            o.por_model = C.cast(C.pointer(v), C.c_void_p) if v is not None else None
            continue
        setattr(o, key, float(v) if key == "load_factor" else int(v))
    items = (BatchItem * n)()
    levels = (C.c_uint64 * (n * level_capacity))()
    st = BatchStats()
    rc = lib.gpx_batch_explore(hs, js, n, C.byref(o), items, levels, level_capacity, C.byref(st))
    if check and rc != GPX_OK:
        raise GpxError(rc, "batch exploration")
    out = []
    for k in range(n):
        it = items[k]
        nl = min(it.nlevels, level_capacity)
        out.append({"status": it.status, "stopped": STOPS[it.stopped] if 0 <= it.stopped < 4 else str(it.stopped),
                    "verdict": VERDICTS.get(it.verdict, str(it.verdict)), "states": it.states,
                    "levels": [int(levels[k * level_capacity + l]) for l in range(nl)], "nlevels": it.nlevels,
                    "set_hash": f"{it.set_hash:016x}", "capacity": it.capacity,
                    "completion_ms": it.completion_ms, "admissions": it.admissions,
                    "slot_bytes": it.slot_bytes})
    stats = {f: getattr(st, f) for f, _ in BatchStats._fields_}
    stats["instances_by_slot"] = list(st.instances_by_slot)
    stats["rc"] = rc
    del keep
    return out, stats


def por_train(x: np.ndarray, y: np.ndarray, **kw):
    """gpx_por_train: returns (PorModel, final loss)."""
    L = load()
    x = np.ascontiguousarray(x, dtype=np.uint8)
    y = np.ascontiguousarray(y, dtype=np.float32)
    o = TrainOptions()
    L.gpx_train_options_init(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, float(v) if k in ("lr", "weight_decay") else int(v))
    m = PorModel()
    loss = C.c_float()
    rc = L.gpx_por_train(x.ctypes.data, y.ctypes.data, x.shape[0], C.byref(o), C.byref(m), C.byref(loss))
    if rc != GPX_OK:
        raise GpxError(rc, "training the POR model")
    return m, float(loss.value)


def por_grad(w1, b1, w2, b2, x, y, device: int = 0):
    """gpx_por_grad: (loss, gw1, gb1, gw2, gb2) of one forward/backward pass."""
    L = load()
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
    w1, b1, w2, y = f(w1), f(b1), f(w2), f(y)
    x = np.ascontiguousarray(x, dtype=np.uint8)
    gw1, gb1, gw2 = np.zeros_like(w1), np.zeros_like(b1), np.zeros_like(w2)
    gb2, loss = C.c_float(), C.c_float()
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    rc = L.gpx_por_grad(device, fp(w1), fp(b1), fp(w2), float(b2), x.ctypes.data, fp(y), x.shape[0], fp(gw1),
                        fp(gb1), fp(gw2), C.byref(gb2), C.byref(loss))
    if rc != GPX_OK:
        raise GpxError(rc, "POR gradient")
    return float(loss.value), gw1, gb1, gw2, float(gb2.value)


def device_info(device: int = 0) -> Optional[DeviceInfo]:
    inf = DeviceInfo()
    rc = load().gpx_device_info_get(device, C.byref(inf))
    return inf if rc == GPX_OK else None


def states_set_hash(words: np.ndarray) -> str:
    """Order-independent set hash of state-vector rows (same formula as the oracle and libgpx)."""
    words = np.asarray(words, dtype=np.uint64)
    if words.ndim == 1:
        words = words[:, None]
    M = np.uint64(0xFFFFFFFFFFFFFFFF)
    with np.errstate(over="ignore"):
        h = np.full(words.shape[0], 0x9E3779B97F4A7C15, dtype=np.uint64)
        for j in range(0, words.shape[1], 2):
            c = words[:, j].copy()
            if j + 1 < words.shape[1]:
                c |= words[:, j + 1] << np.uint64(32)
            z = (h ^ c) + np.uint64(0x9E3779B97F4A7C15)
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            h = z ^ (z >> np.uint64(31))
        total = int(h.sum(dtype=np.uint64)) & int(M)
    return f"{total:016x}"


def exported_symbols(path: str = LIB) -> List[str]:
    lib = C.CDLL(path)
    return [s for s in EXPORTS if hasattr(lib, s)]
