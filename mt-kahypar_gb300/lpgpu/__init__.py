"""lpgpu: GB300-native label-propagation (km1) refinement behind a C ABI.

This module is a thin ctypes binding of ``liblpgpu.so`` (declared in
``include/lpgpu.h``). It loads the in-tree library and raises if it is
missing: there is no CPU fallback anywhere in the product path.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblpgpu.so")

I64P = ctypes.POINTER(ctypes.c_int64)
I32P = ctypes.POINTER(ctypes.c_int32)
U32P = ctypes.POINTER(ctypes.c_uint32)
U8P = ctypes.POINTER(ctypes.c_uint8)

OK, ERR_INVALID_ARG, ERR_OOM, ERR_ADMISSION, ERR_TIMEOUT, ERR_CUDA, ERR_NO_DEVICE, ERR_STATE = range(8)
MAX_K = 1024
FLAG_NO_GRAPH = 1
FLAG_PERSISTENT = 2
FLAG_MULTI_LAUNCH = 4
PERSISTENT_MAX_K = 64
MODE_MULTI_LAUNCH, MODE_PERSISTENT = 0, 1
# tuning table written by lpgpu.autotune on a GB300 (loaded with the library)
TUNING_PATH = os.path.join(HERE, "tuning_gb300.json")


class Tuning(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int32), ("ctas_per_sm", ctypes.c_int32), ("unroll", ctypes.c_int32),
                ("order", ctypes.c_int32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class TuningEntry(ctypes.Structure):
    _fields_ = [("max_mean_pins", ctypes.c_int64), ("min_instances", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("tuning", Tuning)]


class Config(ctypes.Structure):
    _fields_ = [("rounds", ctypes.c_int32), ("activation_threshold", ctypes.c_int32),
                ("rebalancing", ctypes.c_int32), ("subrounds", ctypes.c_int32),
                ("revert", ctypes.c_int32), ("rollback", ctypes.c_int32),
                ("flags", ctypes.c_int32), ("reserved1", ctypes.c_int32)]


class InstanceDesc(ctypes.Structure):
    """lpgpu_instance: one batch instance in its own ids."""
    _fields_ = [("num_vertices", ctypes.c_int64), ("num_nets", ctypes.c_int64),
                ("net_offsets", I64P), ("pins", I32P), ("vertex_weights", I32P), ("net_weights", I32P)]


class Result(ctypes.Structure):
    _fields_ = [("km1_before", ctypes.c_int64), ("km1_after", ctypes.c_int64),
                ("delta", ctypes.c_int64), ("moves", ctypes.c_int64),
                ("pins_processed", ctypes.c_int64), ("rounds", ctypes.c_int32),
                ("improved", ctypes.c_int32), ("imbalance", ctypes.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class RoundStats(ctypes.Structure):
    _fields_ = [("active", ctypes.c_int64), ("pins", ctypes.c_int64),
                ("candidates", ctypes.c_int64), ("moved", ctypes.c_int64),
                ("reverted", ctypes.c_int64), ("delta", ctypes.c_int64),
                ("moved_pins", ctypes.c_int64), ("toggles", ctypes.c_int64)]


class PhaseTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 24), ("launches", ctypes.c_int64), ("ms", ctypes.c_double)]


class LpgpuError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"lpgpu status {status}: {msg}")
        self.status = status


_lib = None

# exported C symbols (every declaration of include/lpgpu.h)
SYMBOLS = [
    "lpgpu_config_default", "lpgpu_status_string", "lpgpu_last_error", "lpgpu_refine_km1",
    "lpgpu_session_create", "lpgpu_session_destroy", "lpgpu_session_upload",
    "lpgpu_session_set_partition", "lpgpu_session_refine", "lpgpu_session_round_stats",
    "lpgpu_session_get_partition", "lpgpu_session_metrics", "lpgpu_session_get_block_weights",
    "lpgpu_session_get_pin_counts", "lpgpu_session_get_connectivity",
    "lpgpu_session_get_incidence", "lpgpu_session_best_moves", "lpgpu_session_gain_cache",
    "lpgpu_session_apply_moves", "lpgpu_session_footprint", "lpgpu_estimate_footprint",
    "lpgpu_session_enable_timing", "lpgpu_session_phase_times", "lpgpu_session_save_partition",
    "lpgpu_session_restore_partition", "lpgpu_kernel_launches", "lpgpu_host_alloc",
    "lpgpu_host_free", "lpgpu_session_event_record", "lpgpu_session_event_elapsed",
    "lpgpu_session_synchronize", "lpgpu_session_upload_batch", "lpgpu_session_set_partition_batch",
    "lpgpu_session_instance_km1", "lpgpu_partition_metrics_noalloc", "lpgpu_session_upload_instances",
    "lpgpu_session_set_partition_instances", "lpgpu_session_get_partition_instances", "lpgpu_read_hgr",
    "lpgpu_free", "lpgpu_read_partition", "lpgpu_write_partition", "lpgpu_session_init_gain_cache",
    "lpgpu_session_drop_gain_cache", "lpgpu_session_project_partition", "lpgpu_session_rebalance",
    "lpgpu_session_repair_empty_blocks", "lpgpu_set_tuning_table", "lpgpu_session_set_tuning",
    "lpgpu_session_tuning", "lpgpu_stepper_create", "lpgpu_stepper_destroy", "lpgpu_session_begin_rounds",
    "lpgpu_stepper_launch", "lpgpu_stepper_wait", "lpgpu_session_end_rounds",
]


def lib():
    """Loads liblpgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run build() first (no CPU fallback exists)")
        L = ctypes.CDLL(LIB_PATH)
        L.lpgpu_last_error.restype = ctypes.c_char_p
        L.lpgpu_status_string.restype = ctypes.c_char_p
        L.lpgpu_estimate_footprint.restype = ctypes.c_int64
        L.lpgpu_estimate_footprint.argtypes = [ctypes.c_int64] * 3 + [ctypes.c_int32] * 2
        L.lpgpu_kernel_launches.restype = ctypes.c_int64
        L.lpgpu_host_alloc.restype = ctypes.c_void_p
        L.lpgpu_host_alloc.argtypes = [ctypes.c_size_t]
        L.lpgpu_host_free.argtypes = [ctypes.c_void_p]
        _lib = L
        if os.path.exists(TUNING_PATH):
            load_tuning(TUNING_PATH)
    return _lib


def set_tuning_table(rows):
    """Process-wide tuning table (lpgpu_set_tuning_table): rows of dicts with
    max_mean_pins, min_instances, mode, ctas_per_sm, unroll, order."""
    arr = (TuningEntry * max(1, len(rows)))()
    for i, r in enumerate(rows):
        arr[i].max_mean_pins = int(r["max_mean_pins"])
        arr[i].min_instances = int(r["min_instances"])
        arr[i].tuning = Tuning(int(r["mode"]), int(r["ctas_per_sm"]), int(r["unroll"]), int(r["order"]))
    _check(lib().lpgpu_set_tuning_table(arr, ctypes.c_int32(len(rows))))


def load_tuning(path=TUNING_PATH):
    """Loads an autotuner table (JSON with an "entries" list) into the library."""
    import json
    with open(path) as f:
        set_tuning_table(json.load(f)["entries"])


def _check(status):
    if status != OK:
        msg = lib().lpgpu_last_error().decode(errors="replace")
        raise LpgpuError(status, msg)


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


# lpgpu_instance as a numpy record (same layout as InstanceDesc on 64-bit
# hosts): descriptors of many instances are filled column by column.
_INSTANCE_DTYPE = np.dtype([("num_vertices", "<i8"), ("num_nets", "<i8"), ("net_offsets", "<u8"),
                            ("pins", "<u8"), ("vertex_weights", "<u8"), ("net_weights", "<u8")])
assert _INSTANCE_DTYPE.itemsize == ctypes.sizeof(InstanceDesc)


def _addr(a):
    """Address of a contiguous array's first element (0 for None). Through the
    buffer protocol where the array is writable (a third of the cost of
    building __array_interface__, which a batch of thousands of instances
    pays per array), else through the interface."""
    if a is None:
        return 0
    try:
        return ctypes.addressof(ctypes.c_char.from_buffer(a))
    except (TypeError, ValueError):  # read-only or empty
        return a.__array_interface__["data"][0]


def _addresses(arrays):
    """uintptr_t array of the arrays' addresses (a C array of pointers)."""
    return np.fromiter((_addr(a) for a in arrays), np.uintp, len(arrays))


def default_config(**over) -> Config:
    c = Config()
    lib().lpgpu_config_default(ctypes.byref(c))
    for k, v in over.items():
        setattr(c, k, int(v))
    return c


class Session:
    """Device-resident hypergraph + partition state (one CUDA stream)."""

    def __init__(self, device: int = 0):
        self._h = ctypes.c_void_p()
        _check(lib().lpgpu_session_create(ctypes.c_int32(device), ctypes.byref(self._h)))
        self.n = self.m = self.k = self.num_blocks = 0

    def close(self):
        if self._h:
            lib().lpgpu_session_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, hg):
        self.n, self.m = int(hg.n), int(hg.m)
        self._keep = (np.ascontiguousarray(hg.net_off, np.int64), np.ascontiguousarray(hg.pins, np.int32),
                      np.ascontiguousarray(hg.w_v, np.int32), np.ascontiguousarray(hg.w_e, np.int32))
        no, pi, wv, we = self._keep
        _check(lib().lpgpu_session_upload(self._h, ctypes.c_int64(self.n), ctypes.c_int64(self.m),
                                          _p(no, I64P), _p(pi, I32P), _p(wv, I32P), _p(we, I32P)))
        self._keep = None
        return self

    def upload_batch(self, hgs):
        """Uploads a list of hypergraphs as one batched union (instance order kept)."""
        nv = np.array([0] + [h.n for h in hgs], np.int64).cumsum()
        ne = np.array([0] + [h.m for h in hgs], np.int64).cumsum()
        pin_base = np.array([0] + [h.num_pins for h in hgs], np.int64).cumsum()
        net_off = np.concatenate([hgs[0].net_off[:1]] + [h.net_off[1:] + pin_base[i] for i, h in enumerate(hgs)])
        pins = np.concatenate([h.pins.astype(np.int64) + nv[i] for i, h in enumerate(hgs)]).astype(np.int32)
        w_v = np.concatenate([h.w_v for h in hgs]).astype(np.int32)
        w_e = np.concatenate([h.w_e for h in hgs]).astype(np.int32)
        self.n, self.m = int(nv[-1]), int(ne[-1])
        self.inst_voff, self.inst_noff = nv, ne
        self.num_inst = len(hgs)
        _check(lib().lpgpu_session_upload_batch(self._h, ctypes.c_int32(len(hgs)), _p(nv, I64P), _p(ne, I64P),
                                                _p(np.ascontiguousarray(net_off, np.int64), I64P),
                                                _p(pins, I32P), _p(w_v, I32P), _p(w_e, I32P)))
        return self

    def upload_instances(self, hgs):
        """Uploads a list of hypergraphs as one batch from their own buffers
        (lpgpu_session_upload_instances: no union is built on the host)."""
        def arr(a, dt):
            return None if a is None else np.ascontiguousarray(a, dt)
        offs = [arr(h.net_off, np.int64) for h in hgs]
        pins = [arr(h.pins, np.int32) for h in hgs]
        wvs = [arr(h.w_v, np.int32) for h in hgs]
        wes = [arr(h.w_e, np.int32) for h in hgs]
        descs = np.zeros(len(hgs), _INSTANCE_DTYPE)
        descs["num_vertices"] = [h.n for h in hgs]
        descs["num_nets"] = [h.m for h in hgs]
        descs["net_offsets"] = _addresses(offs)
        descs["pins"] = _addresses(pins)
        descs["vertex_weights"] = _addresses(wvs)
        descs["net_weights"] = _addresses(wes)
        nv = np.concatenate([[0], np.cumsum(descs["num_vertices"])]).astype(np.int64)
        ne = np.concatenate([[0], np.cumsum(descs["num_nets"])]).astype(np.int64)
        _check(lib().lpgpu_session_upload_instances(self._h, ctypes.c_int32(len(hgs)),
                                                    ctypes.c_void_p(descs.ctypes.data)))
        self.n, self.m = int(nv[-1]), int(ne[-1])
        self.inst_voff, self.inst_noff = nv, ne
        self.num_inst = len(hgs)
        return self

    def set_partition_instances(self, ks, parts, eps=0.03):
        """Per-instance k and one instance-local partition array per instance."""
        ks = np.ascontiguousarray(ks, np.int32)
        ep = np.ascontiguousarray(np.broadcast_to(np.asarray(eps, np.float64), ks.shape), np.float64)
        arrs = [np.ascontiguousarray(p, np.int32) for p in parts]
        ptrs = _addresses(arrs)
        self.k = int(ks.max())
        self.num_blocks = int(ks.sum())
        _check(lib().lpgpu_session_set_partition_instances(self._h, _p(ks, I32P),
                                                           ep.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                           ctypes.c_void_p(ptrs.ctypes.data)))
        return self

    def partition_instances(self, out=None):
        """Instance-local partitions, one array per instance (into `out` if given)."""
        off = self.inst_voff
        outs = out if out is not None else [np.empty(int(off[i + 1] - off[i]), np.int32)
                                            for i in range(self.num_inst)]
        if any(not a.flags.c_contiguous or a.dtype != np.int32 for a in outs):
            raise ValueError("outputs must be contiguous int32 arrays")
        ptrs = _addresses(outs)
        _check(lib().lpgpu_session_get_partition_instances(self._h, ctypes.c_void_p(ptrs.ctypes.data)))
        return outs

    def set_partition_batch(self, ks, parts, eps=0.03):
        """Per-instance k and instance-local partitions (list of arrays)."""
        ks = np.ascontiguousarray(ks, np.int32)
        ep = np.ascontiguousarray(np.broadcast_to(np.asarray(eps, np.float64), ks.shape), np.float64)
        part = np.ascontiguousarray(np.concatenate(parts), np.int32)
        self.k = int(ks.max())          # Φ row width (largest instance k)
        self.num_blocks = int(ks.sum())  # global blocks: block weights come one per block
        _check(lib().lpgpu_session_set_partition_batch(self._h, _p(ks, I32P),
                                                       ep.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                       _p(part, I32P)))
        return self

    def instance_km1(self):
        out = np.empty(getattr(self, "num_inst", 1), np.int64)
        _check(lib().lpgpu_session_instance_km1(self._h, _p(out, I64P)))
        return out

    def set_partition(self, k, part, eps=0.03, lmax=None, perfect=None):
        self.k = int(k)
        self.num_blocks = int(k)
        p = np.ascontiguousarray(part, np.int32)
        lm = None if lmax is None else np.ascontiguousarray(lmax, np.int64)
        pf = None if perfect is None else np.ascontiguousarray(perfect, np.int64)
        _check(lib().lpgpu_session_set_partition(self._h, ctypes.c_int32(k), ctypes.c_double(eps),
                                                 _p(p, I32P), _p(lm, I64P), _p(pf, I64P)))
        return self

    def refine(self, cfg: Config = None, nodes=None) -> Result:
        r = Result()
        nd = None if nodes is None else np.ascontiguousarray(nodes, np.int32)
        _check(lib().lpgpu_session_refine(self._h, None if cfg is None else ctypes.byref(cfg),
                                          _p(nd, I32P), ctypes.c_int64(0 if nd is None else len(nd)),
                                          ctypes.byref(r)))
        return r

    def round_stats(self):
        buf = (RoundStats * 256)()
        cnt = ctypes.c_int32()
        _check(lib().lpgpu_session_round_stats(self._h, buf, 256, ctypes.byref(cnt)))
        return [{f: getattr(buf[i], f) for f, _ in RoundStats._fields_} for i in range(min(256, cnt.value))]

    def partition(self):
        out = np.empty(self.n, np.int32)
        _check(lib().lpgpu_session_get_partition(self._h, _p(out, I32P)))
        return out

    def metrics(self):
        km1, cut, imb = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_double()
        _check(lib().lpgpu_session_metrics(self._h, ctypes.byref(km1), ctypes.byref(cut), ctypes.byref(imb)))
        return km1.value, cut.value, imb.value

    def block_weights(self):
        out = np.empty(self.num_blocks, np.int64)
        _check(lib().lpgpu_session_get_block_weights(self._h, _p(out, I64P)))
        return out

    def pin_counts(self):
        out = np.empty(self.m * self.k, np.int32)
        _check(lib().lpgpu_session_get_pin_counts(self._h, _p(out, I32P)))
        return out.reshape(self.m, self.k)

    def connectivity(self):
        W = (self.k + 31) // 32
        out = np.empty(self.m * W, np.uint32)
        _check(lib().lpgpu_session_get_connectivity(self._h, _p(out, U32P)))
        return out.reshape(self.m, W)

    def incidence(self, num_pins):
        vo = np.empty(self.n + 1, np.int64)
        ie = np.empty(num_pins, np.int32)
        _check(lib().lpgpu_session_get_incidence(self._h, _p(vo, I64P), _p(ie, I32P)))
        return vo, ie

    def best_moves(self):
        to = np.empty(self.n, np.int32)
        gain = np.empty(self.n, np.int32)
        border = np.empty(self.n, np.uint8)
        _check(lib().lpgpu_session_best_moves(self._h, _p(to, I32P), _p(gain, I32P), _p(border, U8P)))
        return to, gain, border.astype(bool)

    def gain_cache(self):
        b = np.empty(self.n, np.int32)
        p = np.empty(self.n * self.k, np.int32)
        _check(lib().lpgpu_session_gain_cache(self._h, _p(b, I32P), _p(p, I32P)))
        return b, p.reshape(self.n, self.k)

    def rebalance(self, max_rounds=16) -> Result:
        """Deterministic rebalancer (lpgpu_session_rebalance)."""
        r = Result()
        _check(lib().lpgpu_session_rebalance(self._h, ctypes.c_int32(max_rounds), ctypes.byref(r)))
        return r

    def set_tuning(self, mode=None, ctas_per_sm=1, unroll=4, order=0):
        """Per-session tuning (lpgpu_session_set_tuning); mode None: back to the table."""
        if mode is None:
            _check(lib().lpgpu_session_set_tuning(self._h, None))
        else:
            t = Tuning(int(mode), int(ctas_per_sm), int(unroll), int(order))
            _check(lib().lpgpu_session_set_tuning(self._h, ctypes.byref(t)))
        return self

    def tuning(self):
        """The tuning the next refine uses (lpgpu_session_tuning)."""
        t = Tuning()
        _check(lib().lpgpu_session_tuning(self._h, ctypes.byref(t)))
        return t.as_dict()

    def begin_rounds(self, cfg: Config = None):
        """Starts a stepped refinement (lpgpu_session_begin_rounds)."""
        _check(lib().lpgpu_session_begin_rounds(self._h, None if cfg is None else ctypes.byref(cfg)))
        return self

    def end_rounds(self) -> Result:
        """Result of a stepped refinement (lpgpu_session_end_rounds)."""
        r = Result()
        _check(lib().lpgpu_session_end_rounds(self._h, ctypes.byref(r)))
        return r

    def repair_empty_blocks(self):
        """Moves of repairEmptyBlocks (lpgpu_session_repair_empty_blocks), not applied:
        a list of (vertex, from, to, gain) in empty-block order."""
        k = max(1, self.k)
        out = [np.zeros(k, np.int32) for _ in range(4)]
        cnt = ctypes.c_int32()
        _check(lib().lpgpu_session_repair_empty_blocks(self._h, *[_p(a, I32P) for a in out], ctypes.byref(cnt)))
        return [tuple(int(a[i]) for a in out) for i in range(cnt.value)]

    def project_partition(self, coarse, fine_to_coarse):
        """This (fine) session's partition from `coarse`'s through the vertex map."""
        m = np.ascontiguousarray(fine_to_coarse, np.int32)
        _check(lib().lpgpu_session_project_partition(self._h, coarse._h, _p(m, I32P)))
        self.k = coarse.k
        self.num_blocks = coarse.k
        return self

    def init_gain_cache(self):
        """Keeps a device gain cache that apply_moves maintains."""
        _check(lib().lpgpu_session_init_gain_cache(self._h))
        return self

    def drop_gain_cache(self):
        _check(lib().lpgpu_session_drop_gain_cache(self._h))
        return self

    def apply_moves(self, vertices, from_, to):
        v = np.ascontiguousarray(vertices, np.int32)
        f = np.ascontiguousarray(from_, np.int32)
        t = np.ascontiguousarray(to, np.int32)
        d = ctypes.c_int64()
        _check(lib().lpgpu_session_apply_moves(self._h, ctypes.c_int64(len(v)), _p(v, I32P), _p(f, I32P),
                                               _p(t, I32P), ctypes.byref(d)))
        return d.value

    def save_partition(self):
        _check(lib().lpgpu_session_save_partition(self._h))

    def restore_partition(self):
        _check(lib().lpgpu_session_restore_partition(self._h))

    def record(self, slot):
        _check(lib().lpgpu_session_event_record(self._h, ctypes.c_int32(slot)))

    def elapsed_ms(self, a, b):
        ms = ctypes.c_double()
        _check(lib().lpgpu_session_event_elapsed(self._h, ctypes.c_int32(a), ctypes.c_int32(b),
                                                 ctypes.byref(ms)))
        return ms.value

    def synchronize(self):
        _check(lib().lpgpu_session_synchronize(self._h))

    def footprint(self):
        b = ctypes.c_int64()
        _check(lib().lpgpu_session_footprint(self._h, ctypes.byref(b)))
        return b.value

    def enable_timing(self, on=True):
        _check(lib().lpgpu_session_enable_timing(self._h, ctypes.c_int32(1 if on else 0)))

    def phase_times(self):
        buf = (PhaseTime * 64)()
        cnt = ctypes.c_int32()
        _check(lib().lpgpu_session_phase_times(self._h, buf, 64, ctypes.byref(cnt)))
        return {buf[i].name.decode(): (buf[i].launches, buf[i].ms) for i in range(min(64, cnt.value))}


class Stepper:
    """Runs one LP round of many sessions per persistent launch (lpgpu_stepper_*)."""

    def __init__(self, device: int = 0):
        self._h = ctypes.c_void_p()
        _check(lib().lpgpu_stepper_create(ctypes.c_int32(device), ctypes.byref(self._h)))

    def close(self):
        if self._h:
            lib().lpgpu_stepper_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def launch(self, sessions):
        """Enqueues the next round of every session in the list (no wait)."""
        self._n = len(sessions)
        arr = (ctypes.c_void_p * max(1, self._n))(*[x._h.value for x in sessions])
        _check(lib().lpgpu_stepper_launch(self._h, arr, ctypes.c_int32(self._n)))

    def wait(self):
        """Waits for the launched round; one bool per session: its refinement is done."""
        done = np.zeros(max(1, self._n), np.int32)
        _check(lib().lpgpu_stepper_wait(self._h, _p(done, I32P)))
        return done[:self._n].astype(bool)

    def round(self, sessions):
        self.launch(sessions)
        return self.wait()


def refine_km1(hg, k, part, eps=0.03, cfg: Config = None):
    """One-shot lpgpu_refine_km1 on host buffers; returns (new partition, Result)."""
    p = np.array(part, np.int32, copy=True)
    r = Result()
    no = np.ascontiguousarray(hg.net_off, np.int64)
    pi = np.ascontiguousarray(hg.pins, np.int32)
    wv = np.ascontiguousarray(hg.w_v, np.int32)
    we = np.ascontiguousarray(hg.w_e, np.int32)
    _check(lib().lpgpu_refine_km1(ctypes.c_int64(hg.n), ctypes.c_int64(hg.m), _p(no, I64P), _p(pi, I32P),
                                  _p(wv, I32P), _p(we, I32P), ctypes.c_int32(k), ctypes.c_double(eps),
                                  _p(p, I32P), None if cfg is None else ctypes.byref(cfg), ctypes.byref(r)))
    return p, r


class PinnedArray:
    """A numpy array over page-locked host memory (lpgpu_host_alloc)."""

    def __init__(self, shape, dtype):
        dtype = np.dtype(dtype)
        nbytes = max(1, int(np.prod(shape)) * dtype.itemsize)
        self._ptr = lib().lpgpu_host_alloc(nbytes)
        if not self._ptr:
            raise LpgpuError(ERR_OOM, "cudaHostAlloc failed")
        buf = (ctypes.c_char * nbytes).from_address(self._ptr)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def __del__(self):
        try:
            if self._ptr:
                lib().lpgpu_host_free(self._ptr)
                self._ptr = None
        except Exception:
            pass


def pinned_copy(a):
    p = PinnedArray(a.shape, a.dtype)
    p.array[...] = a
    return p


def read_hgr(path):
    """Reads an hMetis .hgr file (lpgpu_read_hgr: the reference reader's rules,
    single-pin nets dropped). Returns (Hypergraph, number of dropped nets)."""
    from .gen import Hypergraph
    L = lib()
    n, m, removed = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    off, pins, vw, ew = I64P(), I32P(), I32P(), I32P()
    _check(L.lpgpu_read_hgr(os.fsencode(path), ctypes.byref(n), ctypes.byref(m), ctypes.byref(off),
                            ctypes.byref(pins), ctypes.byref(vw), ctypes.byref(ew), ctypes.byref(removed)))
    try:
        nn, mm = n.value, m.value
        P = off[mm] if mm > 0 else 0
        hg = Hypergraph(nn, mm, np.ctypeslib.as_array(off, (mm + 1,)).copy(),
                        np.ctypeslib.as_array(pins, (max(P, 1),))[:P].copy(),
                        np.ctypeslib.as_array(vw, (max(nn, 1),))[:nn].copy(),
                        np.ctypeslib.as_array(ew, (max(mm, 1),))[:mm].copy())
    finally:
        for ptr in (off, pins, vw, ew):
            L.lpgpu_free(ptr)
    return hg, removed.value


def read_partition(path, n):
    out = np.empty(n, np.int32)
    _check(lib().lpgpu_read_partition(os.fsencode(path), ctypes.c_int64(n), _p(out, I32P)))
    return out


def write_partition(path, part):
    p = np.ascontiguousarray(part, np.int32)
    _check(lib().lpgpu_write_partition(os.fsencode(path), ctypes.c_int64(len(p)), _p(p, I32P)))


def kernel_launches():
    return int(lib().lpgpu_kernel_launches())


def estimate_footprint(n, m, pins, k, subrounds=16):
    return int(lib().lpgpu_estimate_footprint(n, m, pins, k, subrounds))


def build(force=False):
    """Compiles liblpgpu.so in-tree (see mt-kahypar_gb300/build.py)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_lpgpu_build", os.path.join(os.path.dirname(HERE), "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)
