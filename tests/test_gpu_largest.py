"""The largest product the benchmark does not reach: 2^28 x 2^28 limbs
(2 GiB operands, transform length 2^29: 12 GiB of residues per transform),
and its square, checked by size-independent identities: the value mod
2^64 - 1 and mod 2^64 + 1 of the product against those of the operands."""
import numpy as np
import pytest

from gpu_util import mod_checks

pytestmark = pytest.mark.gpu


def test_product_and_square_at_transform_length_2p29():
    import torch

    import natural_number_gb300 as nn
    n = 1 << 28
    g = torch.Generator(device="cuda")
    g.manual_seed(29)
    a = torch.randint(-(2**63), 2**63 - 1, (n,), dtype=torch.int64, device="cuda", generator=g).view(torch.uint64)
    b = torch.randint(-(2**63), 2**63 - 1, (n,), dtype=torch.int64, device="cuda", generator=g).view(torch.uint64)
    a[-1] = 1
    b[-1] = 3
    ctx = nn.Context(0)
    try:
        out = torch.empty(2 * n, dtype=torch.uint64, device="cuda")
        ctx.mul_device(out, a, b)
        ctx.synchronize()
        ma, mb = mod_checks(a.cpu().numpy()), mod_checks(b.cpu().numpy())
        mp = mod_checks(out.cpu().numpy())
        assert mp[0] == ma[0] * mb[0] % (2**64 - 1)
        assert mp[1] == ma[1] * mb[1] % (2**64 + 1)
        ctx.sqr_device(out, a)
        ctx.synchronize()
        ms = mod_checks(out.cpu().numpy())
        assert ms[0] == ma[0] * ma[0] % (2**64 - 1)
        assert ms[1] == ma[1] * ma[1] % (2**64 + 1)
    finally:
        ctx.close()
