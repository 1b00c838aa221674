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


def test_library_exports_nothing_else_with_c_linkage():
    """Every unmangled function the library exports is one the header
    declares: internal helpers keep internal linkage."""
    import shutil
    import subprocess
    if not shutil.which("nm"):
        pytest.skip("nm is not installed")
    nn.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", nn.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = {f[2] for f in (line.split() for line in out.splitlines())
                if len(f) == 3 and f[1] == "T" and not f[2].startswith("_Z")}
    extra = sorted(exported - set(nn.header_functions()))
    assert not extra, extra


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
