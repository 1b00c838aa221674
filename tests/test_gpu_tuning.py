"""Contexts created through the C ABI (the drop-in header's, the request
server's) apply the tuning file themselves: $NN_TUNING, or the package's
tuning.json; "off" keeps the defaults; unknown keys are skipped."""
import ctypes as C
import json

import pytest

pytestmark = pytest.mark.gpu


def _lib():
    import natural_number_gb300 as nn
    L = nn.lib()
    L.nn_context_create.restype = C.c_int
    L.nn_context_create.argtypes = [C.c_int, C.c_uint64, C.POINTER(C.c_void_p)]
    L.nn_context_get_tunable.restype = C.c_int64
    L.nn_context_get_tunable.argtypes = [C.c_void_p, C.c_char_p]
    L.nn_context_destroy.restype = C.c_int
    L.nn_context_destroy.argtypes = [C.c_void_p]
    return L


def _tunable(L, name):
    ctx = C.c_void_p()
    assert L.nn_context_create(0, 0, C.byref(ctx)) == 0
    try:
        return L.nn_context_get_tunable(ctx, name.encode())
    finally:
        L.nn_context_destroy(ctx)


def test_c_contexts_read_the_tuning_file(tmp_path, monkeypatch):
    L = _lib()
    p = tmp_path / "tuning.json"
    p.write_text(json.dumps({"tunables": {"no_such_tunable": 3, "batch_ntt_min": 77, "batch_r_last@14": 6},
                             "device": "test"}))
    monkeypatch.setenv("NN_TUNING", str(p))
    assert _tunable(L, "batch_ntt_min") == 77
    assert _tunable(L, "batch_r_last@14") == 6
    monkeypatch.setenv("NN_TUNING", "off")
    assert _tunable(L, "batch_ntt_min") == 384
    monkeypatch.delenv("NN_TUNING")
    with open(__import__("natural_number_gb300.autotune", fromlist=["TUNING"]).TUNING) as f:
        packaged = json.load(f)["tunables"]
    assert _tunable(L, "batch_ntt_min") == packaged["batch_ntt_min"]
