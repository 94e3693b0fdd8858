"""Python mirror of the reference C API, on the GPU.

Names and argument meanings follow the reference (mtgp32-fast.h:108-130,
mtgp64-fast.h:107-129, mtgp32-fast-jump.h:25): a generator is created from a
parameter set and a seed (or a seed array / string), fills return the same
values as successive genrand_* calls, and fast_jump takes the reference's
hex jump string.  Device memory and streams come from PyTorch; everything
else goes through the C ABI of libmtgp_gb300.so.
"""
import ctypes

import numpy as np
import torch

from ._lib import WorkItem, check, lib
from .params import MTGP32Params, MTGP64Params

KIND_UINT, KIND_CLOSE1_OPEN2, KIND_CLOSE_OPEN, KIND_OPEN_CLOSE, KIND_OPEN_OPEN = range(5)
KINDS = {"uint": 0, "close1_open2": 1, "close_open": 2, "open_close": 3, "open_open": 4}


def _stream(stream):
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def _dtype(bits, kind):
    if bits == 32:
        return torch.int32 if kind == 0 else torch.float32
    return torch.int64 if kind == 0 else torch.float64


class _Gen:
    bits = 32

    def __init__(self, params, seed=None, array=None, string=None):
        L = lib()
        self._L = L
        self.pre = "mtgp%d_gpu_" % self.bits
        self.params = params
        h = ctypes.c_void_p()
        if string is not None:
            if isinstance(string, str):
                string = string.encode("latin-1")
            check(getattr(L, self.pre + "init_by_str")(ctypes.byref(h), ctypes.byref(params), string))
        elif array is not None:
            a = np.ascontiguousarray(array, dtype=np.uint32 if self.bits == 32 else np.uint64)
            check(getattr(L, self.pre + "init_by_array")(
                ctypes.byref(h), ctypes.byref(params), a.ctypes.data_as(ctypes.c_void_p), len(a)))
        else:
            check(getattr(L, self.pre + "init")(ctypes.byref(h), ctypes.byref(params),
                                                0 if seed is None else seed))
        self.h = h
        self.size = params.mexp // self.bits + 1

    def close(self):
        if self.h:
            getattr(self._L, self.pre + "free")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def fill_into(self, kind, out, n=None, stream=None):
        """Write n values of `kind` into the CUDA tensor `out` (in order)."""
        n = out.numel() if n is None else n
        assert out.is_cuda and out.is_contiguous() and out.element_size() * 8 == self.bits
        check(getattr(self._L, self.pre + "fill")(self.h, kind, ctypes.c_void_p(out.data_ptr()),
                                                  n, _stream(stream)))
        return out

    def fill(self, kind, n, device="cuda", stream=None):
        out = torch.empty(n, dtype=_dtype(self.bits, kind), device=device)
        return self.fill_into(kind, out, n, stream)

    def set_tuning(self, key, value):
        """This generator's tuning knob (the keys of set_tuning)."""
        check(getattr(self._L, self.pre + "gen_set_tuning")(self.h, key.encode(), int(value)))

    def skip(self, n, stream=None):
        check(getattr(self._L, self.pre + "skip")(self.h, n, _stream(stream)))

    def fast_jump(self, jump_string, stream=None):
        check(getattr(self._L, self.pre + "fast_jump")(self.h, jump_string.encode(), _stream(stream)))

    def jump_array(self, words, stream=None):
        w = np.ascontiguousarray(words, dtype=np.uint32)
        check(getattr(self._L, self.pre + "jump_array")(self.h, w.ctypes.data_as(ctypes.c_void_p),
                                                        len(w), _stream(stream)))

    def jump_steps(self, steps, stream=None):
        if not 0 <= steps < 2 ** 128:
            raise ValueError("steps must be in [0, 2^128)")
        check(getattr(self._L, self.pre + "jump_steps")(self.h, steps & (2**64 - 1), steps >> 64,
                                                        _stream(stream)))

    def window(self):
        w = np.empty(self.size, dtype=np.uint32 if self.bits == 32 else np.uint64)
        check(getattr(self._L, self.pre + "get_window_host")(self.h, w.ctypes.data_as(ctypes.c_void_p),
                                                             self.size))
        return w

    def set_window(self, win):
        w = np.ascontiguousarray(win, dtype=np.uint32 if self.bits == 32 else np.uint64)
        check(getattr(self._L, self.pre + "set_window_host")(self.h, w.ctypes.data_as(ctypes.c_void_p),
                                                             len(w)))


class MTGP32(_Gen):
    """GPU twin of mtgp32_fast_t (mtgp32-fast.h:86-89)."""
    bits = 32

    def fill_uint32(self, n, **kw):
        return self.fill(0, n, **kw)

    def fill_close1_open2(self, n, **kw):
        return self.fill(1, n, **kw)

    def fill_close_open(self, n, **kw):
        return self.fill(2, n, **kw)

    def fill_open_close(self, n, **kw):
        return self.fill(3, n, **kw)

    def fill_open_open(self, n, **kw):
        return self.fill(4, n, **kw)


class MTGP64(_Gen):
    """GPU twin of mtgp64_fast_t (mtgp64-fast.h:85-88)."""
    bits = 64

    def fill_uint64(self, n, **kw):
        return self.fill(0, n, **kw)

    def fill_close1_open2(self, n, **kw):
        return self.fill(1, n, **kw)

    def fill_close_open(self, n, **kw):
        return self.fill(2, n, **kw)

    def fill_open_close(self, n, **kw):
        return self.fill(3, n, **kw)

    def fill_open_open(self, n, **kw):
        return self.fill(4, n, **kw)


class Plan:
    """A prepared batch (mtgp_gpu_plan_t)."""

    def __init__(self, handle, pool):
        self.h = handle
        self.pool = pool  # keep the pool alive

    @property
    def output_bytes(self):
        return lib().mtgp_gpu_plan_output_bytes(self.h)

    def info(self):
        """(tasks after splitting, chunk length used for splitting or 0)."""
        t, c = ctypes.c_int64(), ctypes.c_int64()
        check(lib().mtgp_gpu_plan_info(self.h, ctypes.byref(t), ctypes.byref(c)))
        return t.value, c.value

    def describe(self):
        """Configuration: tasks, split chunk, core, grid, kernels per launch,
        in-kernel jumps, tasks from windows jumped ahead of the launch, and
        whether those run beside the others (see mtgp_gpu_plan_describe)."""
        v = np.zeros(8, dtype=np.int64)
        check(lib().mtgp_gpu_plan_describe(self.h, v.ctypes.data_as(ctypes.c_void_p), 8))
        return {"tasks": int(v[0]), "split_chunk": int(v[1]), "core": int(v[2]),
                "grid": int(v[3]), "kernels_per_launch": int(v[4]), "jumps": bool(v[5]),
                "prejumps": int(v[6]), "overlap": int(v[7])}

    def launch(self, out, stream=None):
        check(lib().mtgp_gpu_plan_launch(self.h, ctypes.c_void_p(out.data_ptr()), _stream(stream)))

    def graph_launch(self, out, stream=None):
        check(lib().mtgp_gpu_plan_graph_launch(self.h, ctypes.c_void_p(out.data_ptr()),
                                               _stream(stream)))

    def close(self):
        if self.h:
            lib().mtgp_gpu_plan_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_tuning(key, value):
    """Process-wide default knobs, taken by pools and generators created
    afterwards (existing ones keep theirs; Pool.set_tuning and
    MTGP32.set_tuning change one handle's): "split_chunk" (0 auto, <0 never,
    >0 chunk length), "batch_grid" (0 auto, >0 CTAs), "core" (1, 2, 4),
    "poly_window" (0, 2, 4), "single_chunk" (0 auto), "jump_parts" (0 auto,
    -1 in-kernel)."""
    check(lib().mtgp_gpu_set_tuning(key.encode(), int(value)))


def work_items(streams, kinds, counts, offsets, skips=None):
    n = len(streams)
    arr = (WorkItem * n)()
    for k in range(n):
        arr[k].stream = int(streams[k])
        arr[k].kind = int(kinds[k])
        arr[k].count = int(counts[k])
        arr[k].out_offset = int(offsets[k])
        arr[k].skip = 0 if skips is None else int(skips[k])
    return arr


class Pool:
    """Many device-resident streams (mtgp32_gpu_pool_t / mtgp64_gpu_pool_t)."""

    def __init__(self, bits, handle, mexp):
        self.bits = bits
        self.pre = "mtgp%d_gpu_pool_" % bits
        self.h = handle
        self.mexp = mexp
        self.size = mexp // bits + 1  # words of a window
        self.count = getattr(lib(), self.pre + "size")(handle)

    @classmethod
    def create(cls, params_list, seeds, param_idx=None):
        bits = 32 if isinstance(params_list[0], MTGP32Params) else 64
        P = MTGP32Params if bits == 32 else MTGP64Params
        arr = (P * len(params_list))(*params_list)
        sd = np.ascontiguousarray(seeds, dtype=np.uint32 if bits == 32 else np.uint64)
        pidx = None if param_idx is None else np.ascontiguousarray(param_idx, dtype=np.int32)
        h = ctypes.c_void_p()
        check(getattr(lib(), "mtgp%d_gpu_pool_create" % bits)(
            ctypes.byref(h), arr, len(params_list),
            None if pidx is None else pidx.ctypes.data_as(ctypes.c_void_p),
            sd.ctypes.data_as(ctypes.c_void_p), len(sd)))
        return cls(bits, h, params_list[0].mexp)

    @classmethod
    def create_by_array(cls, params_list, keys, param_idx=None):
        """Stream i = init_by_array(params_list[param_idx[i]], keys[i]),
        seeded on the device."""
        bits = 32 if isinstance(params_list[0], MTGP32Params) else 64
        P = MTGP32Params if bits == 32 else MTGP64Params
        arr = (P * len(params_list))(*params_list)
        dt = np.uint32 if bits == 32 else np.uint64
        off = np.zeros(len(keys) + 1, dtype=np.uint64)
        off[1:] = np.cumsum([len(k) for k in keys])
        flat = np.ascontiguousarray(np.concatenate([np.asarray(k, dtype=dt) for k in keys])
                                    if int(off[-1]) else np.zeros(1, dt))
        pidx = None if param_idx is None else np.ascontiguousarray(param_idx, dtype=np.int32)
        h = ctypes.c_void_p()
        check(getattr(lib(), "mtgp%d_gpu_pool_create_by_array" % bits)(
            ctypes.byref(h), arr, len(params_list),
            None if pidx is None else pidx.ctypes.data_as(ctypes.c_void_p),
            flat.ctypes.data_as(ctypes.c_void_p), off.ctypes.data_as(ctypes.c_void_p), len(keys)))
        return cls(bits, h, params_list[0].mexp)

    @classmethod
    def create_by_str(cls, params_list, strings, param_idx=None):
        """Stream i = init_by_str(params_list[param_idx[i]], strings[i]) (bytes),
        seeded on the device."""
        bits = 32 if isinstance(params_list[0], MTGP32Params) else 64
        P = MTGP32Params if bits == 32 else MTGP64Params
        arr = (P * len(params_list))(*params_list)
        strs = (ctypes.c_char_p * len(strings))(*[bytes(x) for x in strings])
        pidx = None if param_idx is None else np.ascontiguousarray(param_idx, dtype=np.int32)
        h = ctypes.c_void_p()
        check(getattr(lib(), "mtgp%d_gpu_pool_create_by_str" % bits)(
            ctypes.byref(h), arr, len(params_list),
            None if pidx is None else pidx.ctypes.data_as(ctypes.c_void_p),
            ctypes.cast(strs, ctypes.c_void_p), len(strings)))
        return cls(bits, h, params_list[0].mexp)

    @classmethod
    def substreams(cls, params, seed, count, table, stream=None):
        bits = 32 if isinstance(params, MTGP32Params) else 64
        t = np.ascontiguousarray(table, dtype=np.uint32)
        h = ctypes.c_void_p()
        check(getattr(lib(), "mtgp%d_gpu_pool_create_substreams" % bits)(
            ctypes.byref(h), ctypes.byref(params), seed, count,
            t.ctypes.data_as(ctypes.c_void_p), t.shape[0], t.shape[1], _stream(stream)))
        return cls(bits, h, params.mexp)

    def close(self):
        if self.h:
            getattr(lib(), self.pre + "free")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def fill(self, kind, out, n_per_stream, stream=None):
        check(getattr(lib(), self.pre + "fill")(self.h, kind, ctypes.c_void_p(out.data_ptr()),
                                                n_per_stream, _stream(stream)))

    def fill_stream(self, s, kind, out, n, stream=None, byte_offset=0):
        check(getattr(lib(), self.pre + "fill_stream")(
            self.h, s, kind, ctypes.c_void_p(out.data_ptr() + byte_offset), n, _stream(stream)))

    def set_tuning(self, key, value):
        """This pool's tuning knob for the plans and fills it makes afterwards
        (the keys of set_tuning)."""
        check(getattr(lib(), self.pre + "set_tuning")(self.h, key.encode(), int(value)))

    def plan(self, items):
        ph = ctypes.c_void_p()
        check(getattr(lib(), self.pre + "plan")(self.h, items, len(items), ctypes.byref(ph)))
        return Plan(ph, self)

    def replan(self, items, plan):
        """Refill `plan` (made by this pool, idle on the GPU) with new items."""
        check(getattr(lib(), self.pre + "replan")(self.h, items, len(items), plan.h))
        return plan

    def autotune(self, items, out, stream=None, reps=3):
        """Fastest plan for these items on this output buffer (the pool's
        windows are left unchanged); returns (plan, report text)."""
        ph = ctypes.c_void_p()
        buf = ctypes.create_string_buffer(1 << 17)
        check(getattr(lib(), self.pre + "autotune")(
            self.h, items, len(items), ctypes.c_void_p(out.data_ptr()), _stream(stream), reps,
            ctypes.byref(ph), buf, len(buf)))
        return Plan(ph, self), buf.value.decode()

    def submit(self, items, out, stream=None):
        check(getattr(lib(), self.pre + "submit")(self.h, items, len(items),
                                                  ctypes.c_void_p(out.data_ptr()), _stream(stream)))

    def jump_polys(self, param_set, steps, stream=None):
        """X^steps[j] mod chi of a parameter set, computed on the GPU: a
        (len(steps), mexp/32 + 1) CUDA tensor of uint32 words (as int32)."""
        st = np.ascontiguousarray(steps, dtype=np.uint64)
        out = torch.empty((len(st), self.mexp // 32 + 1), dtype=torch.int32, device="cuda")
        check(getattr(lib(), self.pre + "jump_polys")(
            self.h, int(param_set), st.ctypes.data_as(ctypes.c_void_p), len(st),
            ctypes.c_void_p(out.data_ptr()), _stream(stream)))
        return out

    def jump_array(self, s, words, stream=None):
        w = np.ascontiguousarray(words, dtype=np.uint32)
        check(getattr(lib(), self.pre + "jump_array")(self.h, s, w.ctypes.data_as(ctypes.c_void_p),
                                                      len(w), _stream(stream)))

    def windows(self):
        w = np.empty(self.count * self.size, dtype=np.uint32 if self.bits == 32 else np.uint64)
        check(getattr(lib(), self.pre + "get_windows_host")(self.h, w.ctypes.data_as(ctypes.c_void_p),
                                                            w.size))
        return w.reshape(self.count, self.size)

    def set_windows(self, win):
        w = np.ascontiguousarray(win, dtype=np.uint32 if self.bits == 32 else np.uint64).ravel()
        check(getattr(lib(), self.pre + "set_windows_host")(self.h, w.ctypes.data_as(ctypes.c_void_p),
                                                            w.size))


# mtgp_request_t as a numpy record (traces of many requests are built with
# numpy and handed to the library without per-request Python work)
REQUEST_DTYPE = np.dtype([("pool", "<i4"), ("stream", "<u4"), ("kind", "<i4"), ("pad_", "<i4"),
                          ("skip", "<u8"), ("count", "<u8"), ("dst", "<u8")])
assert REQUEST_DTYPE.itemsize == 40


def requests(pools, streams, kinds, counts, skips=None):
    """A trace of requests (no destinations) as a REQUEST_DTYPE array."""
    r = np.zeros(len(streams), dtype=REQUEST_DTYPE)
    r["pool"], r["stream"], r["kind"], r["count"] = pools, streams, kinds, counts
    if skips is not None:
        r["skip"] = skips
    return r


class Server:
    """Continuous-batching request loop over resident pools (mtgp_server_t).

    `submit` queues a request and returns its ticket; the values land in
    `dst` (a CUDA or CPU tensor of the pool's word size) once `wait(ticket)`
    returns.  Without `dst` the result stays in the server's device arena:
    `result(ticket)` is a zero-copy view of it until `release(ticket)`."""

    def __init__(self, pool32=None, pool64=None, budget_bytes=1 << 30, slots=4, max_batch=4096):
        self.pools = (pool32, pool64)  # keep the pools alive
        h = ctypes.c_void_p()
        check(lib().mtgp_server_create(ctypes.byref(h), pool32.h if pool32 else None,
                                       pool64.h if pool64 else None, budget_bytes, slots,
                                       max_batch))
        self.h = h
        self._keep = {}

    def submit(self, pool, stream, kind, count, dst=None, skip=0):
        t = ctypes.c_uint64()
        ptr = None if dst is None else ctypes.c_void_p(dst.data_ptr())
        check(lib().mtgp_server_submit(self.h, pool, stream, kind, skip, count, ptr,
                                       ctypes.byref(t)))
        if dst is not None:
            self._keep[t.value] = dst
        return t.value

    def wait(self, ticket, timeout=60.0):
        """Status of the finished request (0 = done)."""
        st = ctypes.c_int()
        check(lib().mtgp_server_wait(self.h, ticket, timeout, ctypes.byref(st)))
        self._keep.pop(ticket, None)
        return st.value

    def cancel(self, ticket):
        check(lib().mtgp_server_cancel(self.h, ticket))

    def result(self, ticket, dtype=torch.int32):
        """Zero-copy view (CUDA tensor) of a finished request submitted
        without destination; valid until release(ticket)."""
        ptr, nbytes = ctypes.c_void_p(), ctypes.c_uint64()
        check(lib().mtgp_server_result(self.h, ticket, ctypes.byref(ptr), ctypes.byref(nbytes)))
        esz = torch.tensor([], dtype=dtype).element_size()
        typestr = {torch.int32: "<i4", torch.float32: "<f4", torch.int64: "<i8",
                   torch.float64: "<f8"}[dtype]

        class _View:
            __cuda_array_interface__ = {"shape": (nbytes.value // esz,), "typestr": typestr,
                                        "data": (ptr.value or 0, False), "version": 3,
                                        "strides": None}
        return torch.as_tensor(_View(), device="cuda")

    def release(self, ticket):
        check(lib().mtgp_server_release(self.h, ticket))

    def drain(self, timeout=600.0):
        check(lib().mtgp_server_drain(self.h, timeout))
        self._keep.clear()

    def results(self):
        """(latency seconds, status) arrays by ticket - 1."""
        n = ctypes.c_uint64()
        check(lib().mtgp_server_results(self.h, None, None, 0, ctypes.byref(n)))
        lat = np.empty(n.value, dtype=np.float64)
        st = np.empty(n.value, dtype=np.int32)
        check(lib().mtgp_server_results(self.h, lat.ctypes.data_as(ctypes.c_void_p),
                                        st.ctypes.data_as(ctypes.c_void_p), n.value,
                                        ctypes.byref(n)))
        return lat, st

    def stats(self):
        """(completed requests, bytes produced, batches launched)."""
        c, b, k = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        check(lib().mtgp_server_stats(self.h, ctypes.byref(c), ctypes.byref(b), ctypes.byref(k)))
        return c.value, b.value, k.value

    def profile(self):
        """Host seconds: admitting, planning + launching (of which planning),
        retiring (summed over the slot workers), scheduler idle."""
        out = np.zeros(5, dtype=np.float64)
        check(lib().mtgp_server_profile(self.h, out.ctypes.data_as(ctypes.c_void_p), 5))
        return {"admit_s": out[0], "launch_s": out[1], "plan_s": out[4], "retire_s": out[2],
                "idle_s": out[3]}

    def replay(self, requests, arrivals):
        """Submit `requests` (a REQUEST_DTYPE array) at `arrivals` (seconds
        from now) and drain; returns the wall time in seconds.  Results of
        requests without destination are discarded at completion."""
        req = np.ascontiguousarray(requests, dtype=REQUEST_DTYPE)
        arr = np.ascontiguousarray(arrivals, dtype=np.float64)
        assert len(req) == len(arr)
        wall = ctypes.c_double()
        check(lib().mtgp_server_replay(self.h, req.ctypes.data_as(ctypes.c_void_p),
                                       arr.ctypes.data_as(ctypes.c_void_p), len(arr),
                                       ctypes.byref(wall)))
        return wall.value

    def close(self):
        if self.h:
            lib().mtgp_server_destroy(self.h)
            self.h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
