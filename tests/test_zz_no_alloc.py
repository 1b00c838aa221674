"""The allocation-free schoolbook product (nn_mul_base_noalloc) against the
regular one (nn_mul_base), through the C ABI.

nn_mul_base_noalloc exists for callers that must not allocate device memory
where they multiply (code under another framework's memory pool, or
latency-sensitive loops where cudaMalloc/cudaFree would stall the device).
It keeps its scratch in a fixed device array shared by every call, so this
test makes two calls in a row and checks that the second is not disturbed by
what the first left behind.  The file is named to be collected last."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_mul_base_on_consecutive_calls():
    import torch

    import natural_number_gb300 as nn
    from natural_number_gb300.synth import limbs

    L = nn.lib()
    ctx = nn.Context(0)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    cases = [(5000, 4000, 1), (300, 70000, 2)]  # second call: more tiles, different shape
    for na, nb, seed in cases:
        a = torch.from_numpy(limbs(seed, na)).cuda()
        b = torch.from_numpy(limbs(seed + 10, nb)).cuda()
        want = torch.zeros(na + nb, dtype=torch.uint64, device="cuda")
        got = torch.full((na + nb,), 0x5A5A5A5A5A5A5A5A, dtype=torch.uint64, device="cuda")
        ctx.mul_base_device(want, a, b)
        st = L.nn_mul_base_noalloc(C.c_void_p(a.data_ptr()), na, C.c_void_p(b.data_ptr()), nb,
                                   C.c_void_p(got.data_ptr()), stream)
        assert st == nn.NN_OK
        torch.cuda.synchronize()
        ctx.synchronize()
        assert torch.equal(got, want), (na, nb)
    ctx.close()


def test_noalloc_rejects_products_beyond_its_scratch():
    import torch

    import natural_number_gb300 as nn
    L = nn.lib()
    a = torch.zeros(1, dtype=torch.uint64, device="cuda")
    st = L.nn_mul_base_noalloc(C.c_void_p(a.data_ptr()), (1 << 22), C.c_void_p(a.data_ptr()), 1,
                               C.c_void_p(a.data_ptr()), None)
    assert st == nn.NN_ERR_INVALID
    # sizes whose sum wraps around 2^64 are refused too, not taken as small
    st = L.nn_mul_base_noalloc(C.c_void_p(a.data_ptr()), 2**64 - 1, C.c_void_p(a.data_ptr()), 1,
                               C.c_void_p(a.data_ptr()), None)
    assert st == nn.NN_ERR_INVALID


def test_noalloc_reports_a_carry_wait_that_gave_up_then_recovers(monkeypatch):
    """With the library's test hook one scan tile is left out, so a carry
    wait polls a status word that nothing sets until it gives up: the call
    returns NN_ERR_TIMEOUT instead of a silent wrong product.  The next call,
    without the hook, clears the error word and gives the right product."""
    import torch

    import natural_number_gb300 as nn
    from natural_number_gb300.synth import limbs

    L = nn.lib()
    ctx = nn.Context(0)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    na, nb = 2500, 1500  # two scan tiles
    a = torch.from_numpy(limbs(31, na)).cuda()
    b = torch.from_numpy(limbs(32, nb)).cuda()
    want = torch.zeros(na + nb, dtype=torch.uint64, device="cuda")
    ctx.mul_base_device(want, a, b)
    got = torch.zeros(na + nb, dtype=torch.uint64, device="cuda")

    def call():
        return L.nn_mul_base_noalloc(C.c_void_p(a.data_ptr()), na, C.c_void_p(b.data_ptr()), nb,
                                     C.c_void_p(got.data_ptr()), stream)

    monkeypatch.setenv("NN_NOALLOC_SKIP_FIRST_TILE", "1")
    assert call() == nn.NN_ERR_TIMEOUT
    monkeypatch.delenv("NN_NOALLOC_SKIP_FIRST_TILE")
    got.fill_(0x5A5A5A5A5A5A5A5A)
    assert call() == nn.NN_OK
    ctx.synchronize()
    assert torch.equal(got, want)
    ctx.close()
