"""ctypes binding of the C ABI in include/mtgp_gpu.h.

Loads the in-tree mtgp_gb300/lib/libmtgp_gb300.so.  There is no fallback:
if the library is missing or fails to load, `lib()` raises.
"""
import ctypes
import os

from .params import MTGP32Params, MTGP64Params

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libmtgp_gb300.so")

MTGP_OK = 0
ERRORS = {-1: "ALLOC", -2: "INVALID", -3: "UNSUPPORTED", -4: "BAD_JUMP", -5: "CUDA",
          -6: "TIMEOUT", -7: "BUDGET", -8: "BUSY"}

c_int, c_size_t, c_u32, c_u64 = ctypes.c_int, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_uint64
vp = ctypes.c_void_p
cp = ctypes.c_char_p
P32 = ctypes.POINTER(MTGP32Params)
P64 = ctypes.POINTER(MTGP64Params)
pp = ctypes.POINTER(ctypes.c_void_p)


class WorkItem(ctypes.Structure):
    """mtgp_work_item_t."""
    _fields_ = [("stream", c_u32), ("kind", ctypes.c_int32), ("count", c_u64),
                ("out_offset", c_u64), ("skip", c_u64)]


assert ctypes.sizeof(WorkItem) == 32


class Request(ctypes.Structure):
    """mtgp_request_t (one request of a serving trace)."""
    _fields_ = [("pool", ctypes.c_int32), ("stream", c_u32), ("kind", ctypes.c_int32),
                ("pad_", ctypes.c_int32), ("skip", c_u64), ("count", c_u64), ("dst", vp)]


assert ctypes.sizeof(Request) == 40

# name -> (restype, argtypes)
SIGS = {
    "mtgp_gpu_last_error": (cp, []),
    "mtgp_gpu_version": (cp, []),
    "mtgp_gpu_plan_launch": (c_int, [vp, vp, vp]),
    "mtgp_gpu_plan_graph_launch": (c_int, [vp, vp, vp]),
    "mtgp_gpu_plan_output_bytes": (c_u64, [vp]),
    "mtgp_gpu_plan_free": (None, [vp]),
    "mtgp_gpu_plan_info": (c_int, [vp, vp, vp]),
    "mtgp_gpu_plan_describe": (c_int, [vp, vp, c_int]),
    "mtgp_gpu_set_tuning": (c_int, [cp, ctypes.c_int64]),
    "mtgp32_gpu_batch_noalloc": (c_int, [P32, c_int, vp, vp, c_int, vp, c_int, vp, vp]),
    "mtgp_server_create": (c_int, [pp, vp, vp, c_u64, c_int, c_int]),
    "mtgp_server_submit": (c_int, [vp, c_int, c_u32, c_int, c_u64, c_u64, vp, vp]),
    "mtgp_server_cancel": (c_int, [vp, c_u64]),
    "mtgp_server_result": (c_int, [vp, c_u64, vp, vp]),
    "mtgp_server_release": (c_int, [vp, c_u64]),
    "mtgp_server_wait": (c_int, [vp, c_u64, ctypes.c_double, vp]),
    "mtgp_server_drain": (c_int, [vp, ctypes.c_double]),
    "mtgp_server_results": (c_int, [vp, vp, vp, c_u64, vp]),
    "mtgp_server_stats": (c_int, [vp, vp, vp, vp]),
    "mtgp_server_profile": (c_int, [vp, vp, c_int]),
    "mtgp_server_replay": (c_int, [vp, vp, vp, c_int, vp]),
    "mtgp_server_destroy": (None, [vp]),
}
for B, P, W in ((32, P32, c_u32), (64, P64, c_u64)):
    pre = "mtgp%d_gpu_" % B
    SIGS.update({
        pre + "init": (c_int, [pp, P, W]),
        pre + "gen_set_tuning": (c_int, [vp, cp, ctypes.c_int64]),
        pre + "pool_set_tuning": (c_int, [vp, cp, ctypes.c_int64]),
        pre + "init_by_array": (c_int, [pp, P, vp, c_int]),
        pre + "init_by_str": (c_int, [pp, P, cp]),
        pre + "free": (None, [vp]),
        pre + "fill": (c_int, [vp, c_int, vp, c_size_t, vp]),
        pre + "skip": (c_int, [vp, c_u64, vp]),
        pre + "fast_jump": (c_int, [vp, cp, vp]),
        pre + "jump_array": (c_int, [vp, vp, c_int, vp]),
        pre + "jump_steps": (c_int, [vp, c_u64, c_u64, vp]),
        pre + "export": (c_int, [vp, vp]),
        pre + "import": (c_int, [vp, vp]),
        pre + "get_window_host": (c_int, [vp, vp, c_int]),
        pre + "set_window_host": (c_int, [vp, vp, c_int]),
        pre + "pool_create": (c_int, [pp, P, c_int, vp, vp, c_int]),
        pre + "pool_create_substreams": (c_int, [pp, P, W, c_int, vp, c_int, c_int, vp]),
        pre + "pool_create_by_array": (c_int, [pp, P, c_int, vp, vp, vp, c_int]),
        pre + "pool_create_by_str": (c_int, [pp, P, c_int, vp, vp, c_int]),
        pre + "pool_free": (None, [vp]),
        pre + "pool_size": (c_int, [vp]),
        pre + "pool_fill": (c_int, [vp, c_int, vp, c_size_t, vp]),
        pre + "pool_fill_stream": (c_int, [vp, c_int, c_int, vp, c_size_t, vp]),
        pre + "pool_submit": (c_int, [vp, vp, c_int, vp, vp]),
        pre + "pool_plan": (c_int, [vp, vp, c_int, pp]),
        pre + "pool_replan": (c_int, [vp, vp, c_int, vp]),
        pre + "pool_jump_array": (c_int, [vp, c_int, vp, c_int, vp]),
        pre + "pool_jump_polys": (c_int, [vp, c_int, vp, c_int, vp, vp]),
        pre + "pool_get_windows_host": (c_int, [vp, vp, c_size_t]),
        pre + "pool_set_windows_host": (c_int, [vp, vp, c_size_t]),
        pre + "pool_export": (c_int, [vp, c_int, vp]),
        pre + "pool_autotune": (c_int, [vp, vp, c_int, vp, vp, c_int, pp, ctypes.c_char_p, c_int]),
    })
    kinds = ("uint%d" % B, "close1_open2", "close_open", "open_close", "open_open")
    for k in kinds:
        SIGS[pre + "fill_" + k] = (c_int, [vp, vp, c_size_t, vp])

_lib = None


class MTGPError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code


def lib():
    """The loaded library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libmtgp_gb300.so is not built (%s); run "
                               "`python -m mtgp_gb300.build`" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc):
    if rc != MTGP_OK:
        raise MTGPError(rc, lib().mtgp_gpu_last_error().decode(errors="replace"))
    return rc
