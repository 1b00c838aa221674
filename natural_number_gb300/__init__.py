"""GB300-native big-number multiply path (Natural_Number's three-prime NTT
multiply, base case, Newton division) — Python access to the C ABI.

The compute lives in libnatural_gb300.so (sm_103a CUDA kernels + C++ host
orchestration, include/natural_gb300.h).  This module is a thin ctypes layer
for tests, benchmarks and Python callers; it has no CPU fallback: if the
library or a CUDA device is missing, calls raise.

Host-pointer calls take and return numpy uint64 arrays (little-endian limbs,
like basic_natural).  Device calls take torch uint64 CUDA tensors and are
ordered on the context's stream (set to torch's current stream by default).
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "_build", "libnatural_gb300.so")
HEADER = os.path.join(ROOT, "include", "natural_gb300.h")

NN_OK, NN_ERR_INVALID, NN_ERR_OOM, NN_ERR_CUDA, NN_ERR_TIMEOUT, NN_ERR_BUDGET, NN_ERR_NO_DEVICE = range(7)

_u64p = C.POINTER(C.c_uint64)
_vp = C.c_void_p
_lib = None


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("out_n", C.c_uint64), ("r_n", C.c_uint64), ("t_submit", C.c_double),
                ("t_admit", C.c_double), ("t_done", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("in_flight_bytes", C.c_uint64), ("peak_bytes", C.c_uint64), ("waiting", C.c_uint64),
                ("batches", C.c_uint64), ("max_concurrent_batches", C.c_uint64), ("max_batch_jobs", C.c_uint64)]


class MulJob(C.Structure):
    """nn_mul_job: one product of a batch (device pointers)."""
    _fields_ = [("d_a", C.c_void_p), ("n_a", C.c_uint64), ("d_b", C.c_void_p), ("n_b", C.c_uint64),
                ("d_out", C.c_void_p)]


def _trim(x: np.ndarray) -> np.ndarray:
    """Drops leading zero limbs, keeping at least one (natural::std)."""
    nz = np.flatnonzero(x)
    return x[: (int(nz[-1]) + 1) if nz.size else 1]


class NNError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


def header_functions() -> list[str]:
    """Names of every function declared in include/natural_gb300.h."""
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(nn_\w+)\s*\(", txt, flags=re.M)))


def lib() -> C.CDLL:
    """Loads the extension (building it first when nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _b
        _b.build()
    L = C.CDLL(LIB_PATH)
    sig = {
        "nn_context_create": (C.c_int, [C.c_int, C.c_uint64, C.POINTER(_vp)]),
        "nn_context_destroy": (C.c_int, [_vp]),
        "nn_context_set_stream": (C.c_int, [_vp, _vp]),
        "nn_context_use_own_stream": (C.c_int, [_vp]),
        "nn_context_stream": (_vp, [_vp]),
        "nn_context_synchronize": (C.c_int, [_vp]),
        "nn_context_probe_wait": (C.c_int, [_vp, C.c_int]),
        "nn_status_string": (C.c_char_p, [C.c_int]),
        "nn_last_error": (C.c_char_p, [_vp]),
        "nn_context_device_bytes": (C.c_uint64, [_vp]),
        "nn_transform_create": (C.c_int, [_vp, C.POINTER(_vp)]),
        "nn_transform_destroy": (C.c_int, [_vp, _vp]),
        "nn_transform_scale": (C.c_int, [_vp]),
        "nn_transform_set_scale": (None, [_vp, C.c_int]),
        "nn_transform_forward": (C.c_int, [_vp, _vp, _vp, C.c_uint64, C.c_int]),
        "nn_transform_pointwise": (C.c_int, [_vp, _vp, _vp, _vp]),
        "nn_transform_inverse_save": (C.c_int, [_vp, _vp, _vp, C.c_uint64, _u64p]),
        "nn_transform_residues": (C.c_int, [_vp, _vp, _vp]),
        "nn_mul": (C.c_int, [_vp, _vp, _vp, C.c_uint64, _vp, C.c_uint64]),
        "nn_sqr": (C.c_int, [_vp, _vp, _vp, C.c_uint64]),
        "nn_ntt_mul": (C.c_int, [_vp, _vp, _vp, C.c_uint64, _vp, C.c_uint64, C.c_int, C.c_uint64, _u64p]),
        "nn_mul_base": (C.c_int, [_vp, _vp, _vp, C.c_uint64, _vp, C.c_uint64]),
        "nn_batch_create": (C.c_int, [_vp, _u64p, _u64p, C.POINTER(C.c_int), C.c_uint64, C.POINTER(_vp)]),
        "nn_batch_run": (C.c_int, [_vp, _vp, C.POINTER(MulJob)]),
        "nn_batch_destroy": (C.c_int, [_vp, _vp]),
        "nn_batch_items": (C.c_uint64, [_vp]),
        "nn_batch_mul": (C.c_int, [_vp, C.POINTER(MulJob), C.c_uint64]),
        "nn_mul_each": (C.c_int, [_vp, C.POINTER(MulJob), C.c_uint64]),
        "nn_context_set_tunable": (C.c_int, [_vp, C.c_char_p, C.c_int64]),
        "nn_context_get_tunable": (C.c_int64, [_vp, C.c_char_p]),
        "nn_mul_base_noalloc": (C.c_int, [_vp, C.c_uint64, _vp, C.c_uint64, _vp, _vp]),
        "nn_batch_launch": (C.c_int, [_vp, _vp, C.POINTER(MulJob)]),
        "nn_server_create": (C.c_int, [C.c_int, C.c_uint64, C.c_int, C.c_int, C.POINTER(_vp)]),
        "nn_server_submit_mul": (C.c_int, [_vp, _u64p, C.c_uint64, _u64p, C.c_uint64, _u64p, _u64p]),
        "nn_server_submit_div": (C.c_int, [_vp, _u64p, C.c_uint64, _u64p, C.c_uint64, _u64p, _u64p, _u64p]),
        "nn_server_wait": (C.c_int, [_vp, C.c_uint64, C.c_double, C.POINTER(RequestInfo)]),
        "nn_server_get_stats": (C.c_int, [_vp, C.POINTER(ServerStats)]),
        "nn_server_clock": (C.c_double, [_vp]),
        "nn_server_destroy": (C.c_int, [_vp]),
        "nn_pi_dec_levels": (C.c_int, [_vp, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64, C.POINTER(_vp), _u64p,
                                       C.POINTER(C.c_double)]),
        "nn_e_dec_levels": (C.c_int, [_vp, C.c_uint64, C.c_uint64, C.c_uint64, C.POINTER(_vp), _u64p,
                                      C.POINTER(C.c_double)]),
        "nn_to_dec_levels": (C.c_int, [_vp, _u64p, C.c_uint64, C.c_uint64, C.POINTER(_vp), _u64p]),
        "nn_launch_count": (C.c_uint64, []),
        "nn_profile_enable": (None, [C.c_int]),
        "nn_profile_report": (C.c_uint64, [C.c_char_p, C.c_uint64]),
        "nn_free": (None, [_vp]),
        "nn_div_host": (C.c_int, [_vp, _u64p, C.c_uint64, _u64p, C.c_uint64, C.POINTER(_u64p), _u64p,
                                  C.POINTER(_u64p), _u64p]),
        "nn_pow_host": (C.c_int, [_vp, _u64p, C.c_uint64, C.c_uint64, C.POINTER(_u64p), _u64p]),
        "nn_div": (C.c_int, [_vp, _vp, _vp, _vp, C.c_uint64, _vp, C.c_uint64]),
        "nn_divmod_host": (C.c_int, [_vp, _u64p, _u64p, _u64p, C.c_uint64, _u64p, C.c_uint64]),
        "nn_reciprocal_host": (C.c_int, [_vp, _u64p, C.c_uint64, C.c_uint64, C.c_int, C.POINTER(_u64p), _u64p]),
        "nn_to_dec_host": (C.c_int, [_vp, _u64p, C.c_uint64, C.POINTER(_vp), _u64p]),
        "nn_pi_dec_host": (C.c_int, [_vp, C.c_uint64, C.c_uint64, C.c_uint64, C.POINTER(_vp), _u64p]),
        "nn_e_dec_host": (C.c_int, [_vp, C.c_uint64, C.c_uint64, C.POINTER(_vp), _u64p]),
        "nn_mul_base_host": (C.c_int, [_vp, _u64p, _u64p, C.c_uint64, _u64p, C.c_uint64]),
        "nn_default_context": (_vp, []),
        "nn_transform_forward_host": (C.c_int, [_vp, _vp, _u64p, C.c_uint64, C.c_int]),
        "nn_transform_inverse_save_host": (C.c_int, [_vp, _vp, _u64p, C.c_uint64, _u64p]),
        "nn_mul_host": (C.c_int, [_vp, _u64p, _u64p, _u64p, C.c_uint64, _u64p, C.c_uint64]),
        "nn_sqr_host": (C.c_int, [_vp, _u64p, _u64p, _u64p, C.c_uint64]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _np(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.uint64))


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_u64p)


def _dptr(t) -> int:
    """Device pointer of a torch CUDA tensor (uint64 limbs)."""
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    return t.data_ptr()


class Context:
    """nn_context: one CUDA device, one stream, twiddle tables and scratch."""

    def __init__(self, device: int = 0, hbm_budget: int = 0, use_torch_stream: bool = True):
        L = lib()
        h = _vp()
        st = L.nn_context_create(device, hbm_budget, C.byref(h))
        if st != NN_OK:
            raise NNError(st, "nn_context_create: " + L.nn_status_string(st).decode())
        self.h = h
        self.device = device
        from .autotune import apply as _apply_tuning
        self.tuning = _apply_tuning(self)
        if use_torch_stream:
            try:
                import torch
                if torch.cuda.is_available():
                    self.set_stream(torch.cuda.current_stream(device).cuda_stream)
            except ImportError:
                pass

    # -- plumbing -------------------------------------------------------------
    def _check(self, st: int, what: str) -> None:
        if st != NN_OK:
            msg = lib().nn_last_error(self.h).decode()
            raise NNError(st, f"{what}: {lib().nn_status_string(st).decode()}: {msg}")

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().nn_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr: int | None) -> None:
        """Order work on a cudaStream_t handle (0 = the legacy default stream);
        None returns to the context's own stream."""
        if stream_ptr is None:
            self._check(lib().nn_context_use_own_stream(self.h), "use_own_stream")
        else:
            self._check(lib().nn_context_set_stream(self.h, _vp(stream_ptr)), "set_stream")

    def synchronize(self) -> None:
        self._check(lib().nn_context_synchronize(self.h), "synchronize")

    def probe_wait(self, spin_limit: int = 1000) -> int:
        """Runs the carry lookback's bounded wait on a status word nothing
        sets; returns the status (NN_ERR_TIMEOUT when the wait gave up)."""
        return lib().nn_context_probe_wait(self.h, spin_limit)

    def device_bytes(self) -> int:
        return lib().nn_context_device_bytes(self.h)

    # -- host-pointer API (natural.h operator surface) ------------------------
    def mul(self, a, b, out: np.ndarray | None = None) -> np.ndarray:
        """natural operator* on host arrays; `out` (n_a + n_b limbs, e.g. pinned) is reused if given."""
        a, b = _np(a), _np(b)
        if out is None:
            out = np.empty(a.size + b.size, dtype=np.uint64)
        elif out.dtype != np.uint64 or out.size < a.size + b.size or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous uint64 array of n_a + n_b limbs")
        n = C.c_uint64()
        self._check(lib().nn_mul_host(self.h, _ptr(out), C.byref(n), _ptr(a), a.size, _ptr(b), b.size), "mul")
        return out[: n.value]

    def sqr(self, a, out: np.ndarray | None = None) -> np.ndarray:
        a = _np(a)
        if out is None:
            out = np.empty(2 * a.size, dtype=np.uint64)
        elif out.dtype != np.uint64 or out.size < 2 * a.size or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous uint64 array of 2 n limbs")
        n = C.c_uint64()
        self._check(lib().nn_sqr_host(self.h, _ptr(out), C.byref(n), _ptr(a), a.size), "sqr")
        return out[: n.value]

    def _take(self, p, n) -> np.ndarray:
        out = np.ctypeslib.as_array(p, shape=(max(n, 1),))[:n].copy()
        lib().nn_free(C.cast(p, _vp))
        return out

    def _take_str(self, p, n) -> str:
        s = C.string_at(p, n).decode()
        lib().nn_free(p)
        return s

    def mul_base(self, a, b) -> np.ndarray:
        """Schoolbook product on the GPU (n_a + n_b limbs, not normalised)."""
        a, b = _np(a), _np(b)
        out = np.empty(a.size + b.size, dtype=np.uint64)
        self._check(lib().nn_mul_base_host(self.h, _ptr(out), _ptr(a), a.size, _ptr(b), b.size), "mul_base")
        return out

    def div(self, a, b) -> tuple[np.ndarray, np.ndarray]:
        """natural::_div: (quotient, remainder) with the reference's sizes."""
        a, b = _np(a), _np(b)
        q, r, qn, rn = _u64p(), _u64p(), C.c_uint64(), C.c_uint64()
        self._check(lib().nn_div_host(self.h, _ptr(a), a.size, _ptr(b), b.size, C.byref(q), C.byref(qn),
                                      C.byref(r), C.byref(rn)), "div")
        return self._take(q, qn.value), self._take(r, rn.value)

    def divmod(self, a, b) -> tuple[np.ndarray, np.ndarray]:
        """Quotient and remainder by the division with every step on the GPU
        (nn_divmod_host), normalised; the divisor's top limb must be nonzero."""
        a, b = _np(a), _np(b)
        q = np.zeros(a.size - b.size + 1, dtype=np.uint64)
        r = np.zeros(b.size, dtype=np.uint64)
        self._check(lib().nn_divmod_host(self.h, _ptr(q), _ptr(r), _ptr(a), a.size, _ptr(b), b.size), "divmod")
        return _trim(q), _trim(r)

    def pow(self, b, e: int) -> np.ndarray:
        b = _np(b)
        p, n = _u64p(), C.c_uint64()
        self._check(lib().nn_pow_host(self.h, _ptr(b), b.size, e, C.byref(p), C.byref(n)), "pow")
        return self._take(p, n.value)

    def reciprocal(self, d, divd_size: int, variant: int = 2) -> np.ndarray:
        d = _np(d)
        p, n = _u64p(), C.c_uint64()
        self._check(lib().nn_reciprocal_host(self.h, _ptr(d), d.size, divd_size, variant, C.byref(p), C.byref(n)),
                    "reciprocal")
        return self._take(p, n.value)

    def to_dec(self, a) -> str:
        a = _np(a)
        p, n = _vp(), C.c_uint64()
        self._check(lib().nn_to_dec_host(self.h, _ptr(a), a.size, C.byref(p), C.byref(n)), "to_dec")
        return self._take_str(p, n.value)

    def pi_dec(self, terms: int, acc: int, digits: int) -> str:
        p, n = _vp(), C.c_uint64()
        self._check(lib().nn_pi_dec_host(self.h, terms, acc, digits, C.byref(p), C.byref(n)), "pi_dec")
        return self._take_str(p, n.value)

    def e_dec(self, terms: int, digits: int) -> str:
        p, n = _vp(), C.c_uint64()
        self._check(lib().nn_e_dec_host(self.h, terms, digits, C.byref(p), C.byref(n)), "e_dec")
        return self._take_str(p, n.value)

    _TIMING = ("total_s", "tree_s", "division_s", "decimal_s", "gpu_batch_s", "host_product_s", "gpu_products",
               "host_products")

    def pi_dec_levels(self, terms: int, acc: int, digits: int, host_below: int = 128):
        """pi digits with level-by-level batched trees; returns (digits, timing dict).
        host_below 128 balances the host subtrees against the device levels on
        a GB300 with 16 host cores (pi to 10^8 digits: 0.46 s, 0.59 s at 256)."""
        p, n, t = _vp(), C.c_uint64(), (C.c_double * 8)()
        self._check(lib().nn_pi_dec_levels(self.h, terms, acc, digits, host_below, C.byref(p), C.byref(n), t),
                    "pi_dec_levels")
        return self._take_str(p, n.value), dict(zip(self._TIMING, list(t)))

    def e_dec_levels(self, terms: int, digits: int, host_below: int = 256):
        p, n, t = _vp(), C.c_uint64(), (C.c_double * 8)()
        self._check(lib().nn_e_dec_levels(self.h, terms, digits, host_below, C.byref(p), C.byref(n), t),
                    "e_dec_levels")
        return self._take_str(p, n.value), dict(zip(self._TIMING, list(t)))

    def to_dec_levels(self, a, host_below: int = 256) -> str:
        a = _np(a)
        p, n = _vp(), C.c_uint64()
        self._check(lib().nn_to_dec_levels(self.h, _ptr(a), a.size, host_below, C.byref(p), C.byref(n)),
                    "to_dec_levels")
        return self._take_str(p, n.value)

    # -- device-pointer API ---------------------------------------------------
    def mul_device(self, out, a, b, na: int | None = None, nb: int | None = None) -> None:
        na = a.numel() if na is None else na
        nb = b.numel() if nb is None else nb
        self._check(lib().nn_mul(self.h, _vp(_dptr(out)), _vp(_dptr(a)), na, _vp(_dptr(b)), nb), "nn_mul")

    def sqr_device(self, out, a, n: int | None = None) -> None:
        n = a.numel() if n is None else n
        self._check(lib().nn_sqr(self.h, _vp(_dptr(out)), _vp(_dptr(a)), n), "nn_sqr")

    def div_device(self, q, r, a, b) -> None:
        """nn_div on device tensors: q (n_a - n_b + 1 limbs) and r (n_b limbs)."""
        self._check(lib().nn_div(self.h, _vp(_dptr(q)), _vp(_dptr(r)), _vp(_dptr(a)), a.numel(), _vp(_dptr(b)),
                                 b.numel()), "nn_div")

    def mul_base_device(self, out, a, b) -> None:
        self._check(lib().nn_mul_base(self.h, _vp(_dptr(out)), _vp(_dptr(a)), a.numel(), _vp(_dptr(b)), b.numel()),
                    "nn_mul_base")

    def ntt_mul_device(self, out, a, b, scale: int, size: int) -> int:
        w = C.c_uint64()
        self._check(lib().nn_ntt_mul(self.h, _vp(_dptr(out)), _vp(_dptr(a)), a.numel(), _vp(_dptr(b)), b.numel(),
                                     scale, size, C.byref(w)), "nn_ntt_mul")
        return w.value

    def transform(self) -> "Transform":
        return Transform(self)

    def set_tunable(self, name: str, value: int) -> None:
        self._check(lib().nn_context_set_tunable(self.h, name.encode(), int(value)), "set_tunable " + name)

    def get_tunable(self, name: str) -> int:
        return int(lib().nn_context_get_tunable(self.h, name.encode()))

    def mul_each(self, jobs) -> None:
        """Products one nn_mul at a time from a MulJob array (unbatched path)."""
        self._check(lib().nn_mul_each(self.h, jobs, len(jobs)), "mul_each")

    def batch(self, sizes_a, sizes_b, square=None) -> "Batch":
        return Batch(self, sizes_a, sizes_b, square)

    def batch_mul_device(self, pairs, outs) -> None:
        """One-shot batch: pairs of torch tensors (a, b), outputs of n_a + n_b limbs."""
        arr = (MulJob * len(pairs))()
        for k, ((a, b), o) in enumerate(zip(pairs, outs)):
            arr[k] = MulJob(_dptr(a), a.numel(), _dptr(b), b.numel(), _dptr(o))
        self._check(lib().nn_batch_mul(self.h, arr, len(pairs)), "batch_mul")


class Batch:
    """nn_batch: a planned batch of products (one persistent launch per run,
    replayed from a CUDA graph)."""

    def __init__(self, ctx: Context, sizes_a, sizes_b, square=None):
        self.ctx = ctx
        na = np.ascontiguousarray(sizes_a, dtype=np.uint64)
        nb = np.ascontiguousarray(sizes_b, dtype=np.uint64)
        self.count = na.size
        sq = None
        if square is not None:
            self._sq = np.ascontiguousarray(square, dtype=np.int32)
            sq = self._sq.ctypes.data_as(C.POINTER(C.c_int))
        h = _vp()
        ctx._check(lib().nn_batch_create(ctx.h, _ptr(na), _ptr(nb), sq, na.size, C.byref(h)), "batch_create")
        self.h = h
        self._jobs = (MulJob * self.count)()

    @property
    def items(self) -> int:
        return int(lib().nn_batch_items(self.h))

    def run(self, pairs, outs) -> None:
        for k, ((a, b), o) in enumerate(zip(pairs, outs)):
            self._jobs[k] = MulJob(_dptr(a), a.numel(), _dptr(b), b.numel(), _dptr(o))
        self.ctx._check(lib().nn_batch_run(self.ctx.h, self.h, self._jobs), "batch_run")

    def run_jobs(self, jobs) -> None:
        """Runs on a prepared MulJob array (no per-job Python work)."""
        self.ctx._check(lib().nn_batch_run(self.ctx.h, self.h, jobs), "batch_run")

    def close(self) -> None:
        if getattr(self, "h", None) and self.ctx.h:
            lib().nn_batch_destroy(self.ctx.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Transform:
    """nn_transform — the device-resident NTT_info (ntt_info.h:10-67)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        h = _vp()
        ctx._check(lib().nn_transform_create(ctx.h, C.byref(h)), "transform_create")
        self.h = h

    @property
    def scale(self) -> int:
        return lib().nn_transform_scale(self.h)

    def forward(self, limbs, scale: int, n: int | None = None) -> "Transform":
        n = limbs.numel() if n is None else n
        self.ctx._check(lib().nn_transform_forward(self.ctx.h, self.h, _vp(_dptr(limbs)), n, scale), "forward")
        return self

    def pointwise(self, a: "Transform", b: "Transform") -> "Transform":
        self.ctx._check(lib().nn_transform_pointwise(self.ctx.h, self.h, a.h, b.h), "pointwise")
        return self

    def inverse_save(self, out, size: int) -> int:
        w = C.c_uint64()
        self.ctx._check(lib().nn_transform_inverse_save(self.ctx.h, self.h, _vp(_dptr(out)), size, C.byref(w)),
                        "inverse_save")
        return w.value

    def residues(self, out) -> None:
        self.ctx._check(lib().nn_transform_residues(self.ctx.h, self.h, _vp(_dptr(out))), "residues")

    def close(self) -> None:
        if getattr(self, "h", None) and self.ctx.h:
            lib().nn_transform_destroy(self.ctx.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def launch_count() -> int:
    """Kernels launched by the library so far (process-wide)."""
    return int(lib().nn_launch_count())


def profile_enable(on: bool) -> None:
    lib().nn_profile_enable(int(bool(on)))


def profile_report() -> dict:
    """{kernel: (launches, total_ms)} for launches recorded since the last report."""
    buf = C.create_string_buffer(1 << 20)  # the report consumes the records: read once
    lib().nn_profile_report(buf, len(buf))
    out = {}
    for line in buf.value.decode().splitlines():
        name, cnt, ms = line.split()
        out[name] = (int(cnt), float(ms))
    return out


class Server:
    """nn_server: continuous batching of multiply/divide requests (host arrays)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0, streams: int = 3, div_workers: int = 2):
        h = _vp()
        st = lib().nn_server_create(device, hbm_budget, streams, div_workers, C.byref(h))
        if st != NN_OK:
            raise NNError(st, "nn_server_create: " + lib().nn_status_string(st).decode())
        self.h = h
        self._keep = {}

    def clock(self) -> float:
        return lib().nn_server_clock(self.h)

    def submit_mul(self, a, b) -> int:
        a, b = _np(a), _np(b)
        out = np.empty(a.size + b.size, dtype=np.uint64)
        t = C.c_uint64()
        st = lib().nn_server_submit_mul(self.h, _ptr(a), a.size, _ptr(b), b.size, _ptr(out), C.byref(t))
        if st != NN_OK:
            raise NNError(st, "submit_mul: " + lib().nn_status_string(st).decode())
        self._keep[t.value] = ("mul", a, b, out, None)
        return t.value

    def submit_div(self, a, b) -> int:
        a, b = _np(a), _np(b)
        q = np.empty(a.size + 1, dtype=np.uint64)
        r = np.empty(max(a.size, b.size) + 1, dtype=np.uint64)
        t = C.c_uint64()
        st = lib().nn_server_submit_div(self.h, _ptr(a), a.size, _ptr(b), b.size, _ptr(q), _ptr(r), C.byref(t))
        if st != NN_OK:
            raise NNError(st, "submit_div: " + lib().nn_status_string(st).decode())
        self._keep[t.value] = ("div", a, b, q, r)
        return t.value

    def wait(self, ticket: int, timeout: float = 30.0):
        """Returns (result, info): the product, or (quotient, remainder).

        Raises NNError with NN_ERR_TIMEOUT if the request has not finished
        within `timeout` seconds; the request stays queued or in flight, its
        host buffers stay referenced here, and the ticket can be waited on
        again."""
        info = RequestInfo()
        st = lib().nn_server_wait(self.h, ticket, timeout, C.byref(info))
        if st == NN_ERR_TIMEOUT:
            raise NNError(st, "request %d not finished within %.1f s" % (ticket, timeout))
        kind, _, _, out, r = self._keep.pop(ticket)
        if st != NN_OK:
            raise NNError(st, "request failed: " + lib().nn_status_string(st).decode())
        meta = {"submit": info.t_submit, "admit": info.t_admit, "done": info.t_done}
        if kind == "mul":
            return out[: info.out_n], meta
        return (out[: info.out_n], r[: info.r_n]), meta

    def stats(self) -> dict:
        s = ServerStats()
        lib().nn_server_get_stats(self.h, C.byref(s))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().nn_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
