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
