"""TEST INFRASTRUCTURE ONLY — Python access to the oracle.

`Oracle("port")` loads the CPU restatement (oracle/_build/liboracle.so, built by
`build_oracle()`); `Oracle("ref")` loads the reference compiled from its own
sources (oracle/_ref/libref.so, x86-64 hosts only, built by oracle/build_ref.sh).
Both export the same entry points, so tests and fixture generation can drive
either.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
may import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")

_u64p = C.POINTER(C.c_uint64)


def build_oracle(force: bool = False) -> str:
    """Compile the CPU restatement with g++ (portable C++20, no intrinsics)."""
    src = [os.path.join(HERE, f) for f in ("oracle_capi.cpp", "nn_oracle.hpp")]
    if not force and os.path.exists(PORT_SO) and all(
            os.path.getmtime(PORT_SO) >= os.path.getmtime(s) for s in src):
        return PORT_SO
    os.makedirs(os.path.dirname(PORT_SO), exist_ok=True)
    subprocess.check_call(["g++", "-O2", "-std=c++20", "-fPIC", "-shared",
                           src[0], "-o", PORT_SO + ".tmp"])
    os.replace(PORT_SO + ".tmp", PORT_SO)
    return PORT_SO


def build_reference() -> str | None:
    """Compile the reference itself (x86-64 with the reference present)."""
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")])
    return REF_SO if os.path.exists(REF_SO) else None


def _arr(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.uint64))


class Oracle:
    def __init__(self, kind: str = "port"):
        self.kind = kind
        if kind == "port":
            path, self.pre = build_oracle(), "nno_"
        elif kind == "ref":
            path, self.pre = REF_SO, "ref_"
            if not os.path.exists(path):
                raise FileNotFoundError("reference library not built: " + path)
        else:
            raise ValueError(kind)
        self.lib = C.CDLL(path)
        L = self.lib
        f = self._f
        for name in ("mul", "mul_base"):
            f(name).argtypes = [_u64p, C.c_uint64, _u64p, C.c_uint64, _u64p]
            f(name).restype = _u64p
        f("sqr").argtypes = [_u64p, C.c_uint64, _u64p]
        f("sqr").restype = _u64p
        f("ntt_mul_raw").argtypes = [_u64p, C.c_uint64, _u64p, C.c_uint64, C.c_int, C.c_uint64, _u64p]
        f("ntt_mul_raw").restype = _u64p
        f("ntt_sqr_raw").argtypes = [_u64p, C.c_uint64, C.c_int, C.c_uint64, _u64p]
        f("ntt_sqr_raw").restype = _u64p
        f("ntt_forward").argtypes = [_u64p, C.c_uint64, C.c_int, _u64p]
        f("ntt_forward").restype = None
        f("root_table").argtypes = [C.c_int, C.c_int, C.c_int, _u64p]
        f("root_table").restype = None
        f("div").argtypes = [_u64p, C.c_uint64, _u64p, C.c_uint64, _u64p, C.POINTER(_u64p), _u64p]
        f("div").restype = _u64p
        f("pow").argtypes = [_u64p, C.c_uint64, C.c_uint64, _u64p]
        f("pow").restype = _u64p
        for name in ("reciprocal2", "reciprocal3"):
            f(name).argtypes = [_u64p, C.c_uint64, C.c_uint64, _u64p]
            f(name).restype = _u64p
        f("to_dec").argtypes = [_u64p, C.c_uint64, _u64p]
        f("to_dec").restype = C.c_void_p
        f("pi_dec").argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, _u64p]
        f("pi_dec").restype = C.c_void_p
        f("e_dec").argtypes = [C.c_uint64, C.c_uint64, _u64p]
        f("e_dec").restype = C.c_void_p
        f("time_mul").argtypes = [_u64p, C.c_uint64, _u64p, C.c_uint64, C.c_int]
        f("time_mul").restype = C.c_double
        f("time_sqr").argtypes = [_u64p, C.c_uint64, C.c_int]
        f("time_sqr").restype = C.c_double
        f("free").argtypes = [C.c_void_p]
        f("free").restype = None

    def _f(self, name):
        return getattr(self.lib, self.pre + name)

    # -- helpers --------------------------------------------------------------
    @staticmethod
    def _p(a: np.ndarray):
        return a.ctypes.data_as(_u64p)

    def _take(self, ptr, n: int) -> np.ndarray:
        out = np.ctypeslib.as_array(ptr, shape=(max(n, 1),))[:n].copy()
        self._f("free")(C.cast(ptr, C.c_void_p))
        return out

    def _take_str(self, ptr, n: int) -> str:
        s = C.string_at(ptr, n).decode()
        self._f("free")(ptr)
        return s

    # -- entry points ---------------------------------------------------------
    def mul(self, a, b) -> np.ndarray:
        a, b = _arr(a), _arr(b)
        n = C.c_uint64()
        return self._take(self._f("mul")(self._p(a), a.size, self._p(b), b.size, C.byref(n)), n.value)

    def mul_base(self, a, b) -> np.ndarray:
        a, b = _arr(a), _arr(b)
        n = C.c_uint64()
        return self._take(self._f("mul_base")(self._p(a), a.size, self._p(b), b.size, C.byref(n)), n.value)

    def sqr(self, a) -> np.ndarray:
        a = _arr(a)
        n = C.c_uint64()
        return self._take(self._f("sqr")(self._p(a), a.size, C.byref(n)), n.value)

    def ntt_mul_raw(self, a, b, scale: int, size: int) -> np.ndarray:
        a, b = _arr(a), _arr(b)
        n = C.c_uint64()
        return self._take(self._f("ntt_mul_raw")(self._p(a), a.size, self._p(b), b.size, scale, size,
                                                  C.byref(n)), n.value)

    def ntt_sqr_raw(self, a, scale: int, size: int) -> np.ndarray:
        a = _arr(a)
        n = C.c_uint64()
        return self._take(self._f("ntt_sqr_raw")(self._p(a), a.size, scale, size, C.byref(n)), n.value)

    def ntt_forward(self, a, scale: int) -> np.ndarray:
        a = _arr(a)
        out = np.zeros(3 << scale, dtype=np.uint64)
        self._f("ntt_forward")(self._p(a), a.size, scale, self._p(out))
        return out.reshape(3, 1 << scale)

    def root_table(self, scale: int, prime: int, inverse: bool) -> np.ndarray:
        out = np.zeros(1 << (scale - 1), dtype=np.uint64)
        self._f("root_table")(scale, prime, int(inverse), self._p(out))
        return out

    def div(self, a, b):
        a, b = _arr(a), _arr(b)
        qn, rn, rp = C.c_uint64(), C.c_uint64(), _u64p()
        q = self._f("div")(self._p(a), a.size, self._p(b), b.size, C.byref(qn), C.byref(rp), C.byref(rn))
        return self._take(q, qn.value), self._take(rp, rn.value)

    def pow(self, b, e: int) -> np.ndarray:
        b = _arr(b)
        n = C.c_uint64()
        return self._take(self._f("pow")(self._p(b), b.size, e, C.byref(n)), n.value)

    def reciprocal2(self, d, divd_size: int) -> np.ndarray:
        d = _arr(d)
        n = C.c_uint64()
        return self._take(self._f("reciprocal2")(self._p(d), d.size, divd_size, C.byref(n)), n.value)

    def reciprocal3(self, d, divd_size: int) -> np.ndarray:
        d = _arr(d)
        n = C.c_uint64()
        return self._take(self._f("reciprocal3")(self._p(d), d.size, divd_size, C.byref(n)), n.value)

    def to_dec(self, a) -> str:
        a = _arr(a)
        n = C.c_uint64()
        return self._take_str(self._f("to_dec")(self._p(a), a.size, C.byref(n)), n.value)

    def pi_dec(self, terms: int, acc: int, digits: int) -> str:
        n = C.c_uint64()
        return self._take_str(self._f("pi_dec")(terms, acc, digits, C.byref(n)), n.value)

    def e_dec(self, terms: int, digits: int) -> str:
        n = C.c_uint64()
        return self._take_str(self._f("e_dec")(terms, digits, C.byref(n)), n.value)

    def time_mul(self, a, b, reps: int) -> float:
        a, b = _arr(a), _arr(b)
        return self._f("time_mul")(self._p(a), a.size, self._p(b), b.size, reps)

    def time_sqr(self, a, reps: int) -> float:
        a = _arr(a)
        return self._f("time_sqr")(self._p(a), a.size, reps)


def to_int(limbs) -> int:
    """Little-endian u64 limbs -> Python int."""
    a = _arr(limbs)
    return int.from_bytes(a.astype("<u8").tobytes(), "little")


def from_int(x: int) -> np.ndarray:
    n = max(1, (x.bit_length() + 63) // 64)
    return np.frombuffer(x.to_bytes(8 * n, "little"), dtype="<u8").astype(np.uint64)
