"""CPU checks of the C-ABI library: it builds for sm_103a, loads, exports every
function include/natural_gb300.h declares, and fails cleanly without a GPU."""
import ctypes as C

import pytest

import natural_number_gb300 as nn


def test_library_exports_every_declared_symbol():
    L = nn.lib()
    names = nn.header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_status_strings():
    L = nn.lib()
    for s in range(7):
        assert L.nn_status_string(s)


def test_context_without_gpu_reports_no_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = nn.lib()
    h = C.c_void_p()
    st = L.nn_context_create(0, 0, C.byref(h))
    assert st == nn.NN_ERR_NO_DEVICE
    assert not h.value


def test_null_arguments_are_rejected():
    L = nn.lib()
    assert L.nn_context_destroy(None) == nn.NN_ERR_INVALID
    assert L.nn_mul(None, None, None, 1, None, 1) == nn.NN_ERR_INVALID
    assert L.nn_context_synchronize(None) == nn.NN_ERR_INVALID
