"""ctypes binding of libfastoverlap_gb300.so (C ABI in include/fastoverlap_gb300.h).

The library is the only compute path: if it cannot be loaded (not built, no
CUDA device) every call raises; there is no CPU fallback.
"""
import atexit
import ctypes
import os
import threading
import weakref

import numpy as np

from . import build as _build

FO_OK = 0
FO_PREC_FP64 = 0
FO_PREC_MIXED = 1

_STATUS = {0: "ok", 1: "bad arguments", 2: "no peaks found", 3: "assignment failed",
           4: "timeout", 5: "HBM budget exceeded", 6: "CUDA error", 7: "unimplemented",
           8: "queue full", 9: "not ready"}


class FoError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = status
        super().__init__("fastoverlap_gb300: %s (%d)%s" % (_STATUS.get(status, "?"), status,
                                                          (": " + msg) if msg else ""))


class FoOpts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("precision", ctypes.c_int),
                ("hbm_budget_bytes", ctypes.c_size_t), ("cutoff", ctypes.c_int),
                ("profile", ctypes.c_int)]


class FoClusterPair(ctypes.Structure):
    _fields_ = [("natoms", ctypes.c_int), ("ngroups", ctypes.c_int), ("jmax", ctypes.c_int),
                ("nrot", ctypes.c_int), ("invert", ctypes.c_int), ("reserved", ctypes.c_int),
                ("sigma", ctypes.c_double), ("coord_off", ctypes.c_int64),
                ("perm_off", ctypes.c_int64), ("group_off", ctypes.c_int64)]


class FoBulkPair(ctypes.Structure):
    _fields_ = [("natoms", ctypes.c_int), ("ngroups", ctypes.c_int), ("nwave", ctypes.c_int),
                ("nfspace", ctypes.c_int), ("ndisps", ctypes.c_int), ("ohcell", ctypes.c_int),
                ("sigma", ctypes.c_double), ("box", ctypes.c_double * 3),
                ("coord_off", ctypes.c_int64), ("perm_off", ctypes.c_int64),
                ("group_off", ctypes.c_int64)]


class FoPairResult(ctypes.Structure):
    _fields_ = [("dist", ctypes.c_double), ("rmat", ctypes.c_double * 9),
                ("disp", ctypes.c_double * 3), ("overlap_max", ctypes.c_double),
                ("sigma", ctypes.c_double), ("inverted", ctypes.c_int), ("ncand", ctypes.c_int),
                ("status", ctypes.c_int), ("niter", ctypes.c_int)]


class FoRequest(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("natoms", ctypes.c_int), ("ngroups", ctypes.c_int),
                ("jmax", ctypes.c_int), ("nrot", ctypes.c_int), ("invert", ctypes.c_int),
                ("nwave", ctypes.c_int), ("nfspace", ctypes.c_int), ("sigma", ctypes.c_double),
                ("box", ctypes.c_double * 3), ("pos1", ctypes.POINTER(ctypes.c_double)),
                ("pos2", ctypes.POINTER(ctypes.c_double)), ("perm", ctypes.POINTER(ctypes.c_int)),
                ("group_sizes", ctypes.POINTER(ctypes.c_int))]


class FoServerOpts(ctypes.Structure):
    _fields_ = [("max_batch", ctypes.c_int), ("max_queue", ctypes.c_int),
                ("max_wait_ms", ctypes.c_double), ("workers", ctypes.c_int),
                ("reserved", ctypes.c_int)]


class FoServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64),
                ("failed", ctypes.c_int64), ("batches", ctypes.c_int64),
                ("latency_p50_ms", ctypes.c_double), ("latency_p99_ms", ctypes.c_double),
                ("latency_max_ms", ctypes.c_double), ("mean_batch", ctypes.c_double),
                ("busy_ms", ctypes.c_double)]


RESULT_DTYPE = np.dtype([("dist", "f8"), ("rmat", "f8", (9,)), ("disp", "f8", (3,)),
                         ("overlap_max", "f8"), ("sigma", "f8"), ("inverted", "i4"),
                         ("ncand", "i4"), ("status", "i4"), ("niter", "i4")])
assert RESULT_DTYPE.itemsize == ctypes.sizeof(FoPairResult)

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p

# Every exported symbol of include/fastoverlap_gb300.h with its ctypes signature.
EXPORTS = {
    "fo_ctx_create": (ctypes.c_int, [ctypes.POINTER(FoOpts), ctypes.POINTER(_vp)]),
    "fo_ctx_destroy": (None, [_vp]),
    "fo_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "fo_last_error": (ctypes.c_char_p, [_vp]),
    "fo_set_precision": (ctypes.c_int, [_vp, ctypes.c_int]),
    "fo_set_tensor_cores": (ctypes.c_int, [_vp, ctypes.c_int]),
    "fo_set_autotune": (ctypes.c_int, [_vp, ctypes.c_int]),
    "fo_host_register": (ctypes.c_int, [_vp, _vp, ctypes.c_size_t]),
    "fo_host_unregister": (ctypes.c_int, [_vp, _vp]),
    "fo_plan_tile_shape": (ctypes.c_int, [_vp, _ip, _ip]),
    "fo_cluster_align_batch": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _dp, _dp, _ip, _ip,
                                              ctypes.c_int, _dp, _ip, _vp]),
    "fo_bulk_align_batch": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _dp, _dp, _ip, _ip,
                                           ctypes.c_int, _dp, _ip, _vp]),
    "fo_cluster_plan_create": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _dp, _dp, _ip, _ip,
                                              ctypes.c_int, ctypes.POINTER(_vp)]),
    "fo_plan_set_graph": (ctypes.c_int, [_vp, ctypes.c_int]),
    "fo_bnb_cluster": (ctypes.c_int, [_vp, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_longlong,
                                      ctypes.c_double, ctypes.c_double, _dp, _dp,
                                      ctypes.POINTER(ctypes.c_longlong)]),
    "fo_bnb_cluster_batch": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _dp, _dp, ctypes.c_int, ctypes.c_longlong,
                                            ctypes.c_double, ctypes.c_double, _dp, _dp,
                                            ctypes.POINTER(ctypes.c_longlong)]),
    "fo_bulk_plan_create": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _dp, _dp, _ip, _ip,
                                           ctypes.c_int, ctypes.POINTER(_vp)]),
    "fo_plan_run": (ctypes.c_int, [_vp]),
    "fo_plan_wait": (ctypes.c_int, [_vp]),
    "fo_plan_results": (ctypes.c_int, [_vp, _dp, _ip, _vp]),
    "fo_plan_device_bytes": (ctypes.c_size_t, [_vp]),
    "fo_plan_launches": (ctypes.c_int, [_vp]),
    "fo_plan_destroy": (None, [_vp]),
    "fo_setperm": (ctypes.c_int, [_vp, ctypes.c_int, _ip, _ip, ctypes.c_int]),
    "fo_get_bestperm": (ctypes.c_int, [_vp, _ip]),
    "fo_set_ohcell": (ctypes.c_int, [_vp, ctypes.c_int]),
    "fo_cluster_align": (ctypes.c_int, [_vp, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        _dp, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]),
    "fo_bulk_align": (ctypes.c_int, [_vp, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp]),
    "fo_cluster_align_harm": (ctypes.c_int, [_vp, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_double, ctypes.c_double, _dp, _dp, _dp,
                                             ctypes.c_int, ctypes.c_int]),
    "fo_calc_overlap_matrices": (ctypes.c_int, [_vp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_double, ctypes.c_double, _dp, _dp]),
    "fo_cluster_harm_align_batch": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _dp, _dp, _ip, _ip, ctypes.c_int,
                                                   ctypes.c_int, ctypes.c_double, _dp, _ip, _vp]),
    "fo_cluster_harm_plan_create": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _dp, _dp, _ip, _ip, ctypes.c_int,
                                                   ctypes.c_int, ctypes.c_double, ctypes.POINTER(_vp)]),
    "fo_bulk_align_group": (ctypes.c_int, [_vp, _dp, ctypes.c_int, _dp, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_int]),
    "fo_bulk_calcdefaults": (ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double, _dp, _ip, _ip]),
    "fo_profile_kernels": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_char_p), _dp, _ip,
                                          ctypes.c_int]),
    "fo_profile_reset": (None, [_vp]),
    "fo_cluster_overlap": (ctypes.c_int, [_vp, _vp, _dp, _dp, _ip, _ip, ctypes.c_int, _dp, _dp]),
    "fo_bulk_overlap": (ctypes.c_int, [_vp, _vp, _dp, _dp, _ip, _ip, ctypes.c_int, _dp]),
    "fo_findpeaks": (ctypes.c_int, [_vp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp, _ip]),
    "fo_bulk_overlap_noalloc": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _ip, ctypes.c_int,
                                                ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                                ctypes.c_double, ctypes.c_int, ctypes.c_int, _vp,
                                                _vp]),
    "fo_bulk_overlap_noalloc_scratch_bytes": (ctypes.c_size_t, []),
    "fo_ctx_record": (ctypes.c_int, [_vp, ctypes.c_int]),
    "fo_ctx_elapsed_ms": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_float)]),
    "fo_ctx_flush_l2": (ctypes.c_int, [_vp, ctypes.c_size_t]),
    "fo_ctx_synchronize": (ctypes.c_int, [_vp]),
    "fo_server_create": (ctypes.c_int, [_vp, ctypes.POINTER(FoServerOpts), ctypes.POINTER(_vp)]),
    "fo_server_submit": (ctypes.c_int, [_vp, ctypes.POINTER(FoRequest),
                                        ctypes.POINTER(ctypes.c_int64)]),
    "fo_server_poll": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.POINTER(FoPairResult), _dp, _ip]),
    "fo_server_wait": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_double,
                                      ctypes.POINTER(FoPairResult), _dp, _ip]),
    "fo_server_stats_get": (ctypes.c_int, [_vp, ctypes.POINTER(FoServerStats)]),
    "fo_server_destroy": (None, [_vp]),
}

_LIB = None
_LOCK = threading.Lock()

# Library objects still open at interpreter exit are closed here, servers
# first, then plans, then contexts, while the interpreter is intact: calling
# into the library from __del__ during interpreter teardown is not safe.
_LIVE = {"servers": weakref.WeakSet(), "plans": weakref.WeakSet(), "contexts": weakref.WeakSet()}


def track(kind, obj):
    _LIVE[kind].add(obj)


@atexit.register
def _close_all():
    for kind in ("servers", "plans", "contexts"):
        for obj in list(_LIVE[kind]):
            try:
                obj.close()
            except Exception:
                pass


def load(build_if_missing=True):
    """Load the CUDA library (building it in place with nvcc if needed)."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = _build.LIB
        if build_if_missing and (not os.path.exists(path) or _build._stale()):
            _build.build()
        if not os.path.exists(path):
            raise ImportError("libfastoverlap_gb300.so is missing; run fastoverlap_gb300.build.build()")
        lib = ctypes.CDLL(path)
        for name, (res, args) in EXPORTS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
        return lib


def d(a):
    return a.ctypes.data_as(_dp)


def i(a):
    return a.ctypes.data_as(_ip)


def vp(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


class Context(object):
    """Owns one fo_ctx (CUDA stream, Wigner-table cache) on one device."""

    def __init__(self, device=0, precision="fp64", cutoff=True, hbm_budget_bytes=0, profile=False,
                 tensor_cores=True):
        self.lib = load()
        opts = FoOpts(device=device, precision=_prec(precision),
                      hbm_budget_bytes=int(hbm_budget_bytes), cutoff=int(bool(cutoff)),
                      profile=int(bool(profile)))
        h = ctypes.c_void_p()
        st = self.lib.fo_ctx_create(ctypes.byref(opts), ctypes.byref(h))
        if st != FO_OK:
            raise FoError(st, "fo_ctx_create (is a CUDA device visible?)")
        track("contexts", self)
        self.h = h
        self.precision = precision
        if not tensor_cores:
            self.set_tensor_cores(False)

    def close(self):
        if getattr(self, "h", None):
            self.lib.fo_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st, what=""):
        if st != FO_OK:
            msg = self.lib.fo_last_error(self.h)
            raise FoError(st, (what + ": " if what else "") + (msg.decode() if msg else ""))

    def set_precision(self, precision):
        self.check(self.lib.fo_set_precision(self.h, _prec(precision)))
        self.precision = precision

    def set_autotune(self, on):
        """Mixed form: time the tensor-core tile shapes of new plan shapes (default) or not."""
        self.check(self.lib.fo_set_autotune(self.h, int(bool(on))))

    def set_tensor_cores(self, on):
        """Mixed form: the coefficient and Wigner-d contractions on the tcgen05
        tensor cores (default) or on the FP32 CUDA cores."""
        self.check(self.lib.fo_set_tensor_cores(self.h, int(bool(on))))

    def profile(self):
        cap = 32
        names = (ctypes.c_char_p * cap)()
        ms = np.zeros(cap)
        n = np.zeros(cap, np.int32)
        k = self.lib.fo_profile_kernels(self.h, names, d(ms), i(n), cap)
        return {names[j].decode(): (float(ms[j]), int(n[j])) for j in range(k)}

    def profile_reset(self):
        self.lib.fo_profile_reset(self.h)

    def record(self, slot):
        self.check(self.lib.fo_ctx_record(self.h, slot), "record")

    def elapsed_ms(self, a, b):
        ms = ctypes.c_float()
        self.check(self.lib.fo_ctx_elapsed_ms(self.h, a, b, ctypes.byref(ms)), "elapsed")
        return float(ms.value)

    def flush_l2(self, nbytes=256 << 20):
        self.check(self.lib.fo_ctx_flush_l2(self.h, nbytes), "flush_l2")

    def synchronize(self):
        self.check(self.lib.fo_ctx_synchronize(self.h), "synchronize")


def _prec(p):
    if p in (FO_PREC_FP64, "fp64", "plain", None):
        return FO_PREC_FP64
    if p in (FO_PREC_MIXED, "mixed", "fp32", "tf32", "bf16x3"):
        return FO_PREC_MIXED
    raise ValueError("unknown precision %r" % (p,))


_DEFAULT = {}


def default_context(precision="fp64", device=0, cutoff=True):
    key = (device, _prec(precision), bool(cutoff))
    with _LOCK:
        ctx = _DEFAULT.get(key)
    if ctx is None:
        ctx = Context(device=device, precision=precision, cutoff=cutoff)
        with _LOCK:
            _DEFAULT[key] = ctx
    return ctx
