"""GPU test of msot_interp_transpose_noalloc, the adjoint entry point that
allocates no device memory (for callers that are not allowed to, e.g. a host
application whose device memory belongs to another allocator, or one that
runs under a fixed memory budget).  It must give the result of
msot_interp_transpose, which uses the plan's scratch, up to FP32 summation
order, on two calls in a row (the second call reuses the library's fixed
array), and the second call must not change the device's free memory.

The file name sorts last so that a `-x` run reaches it only after every
other test; it also passes when run alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(L, plan, raw, out, W):
    import torch
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return L.msot_interp_transpose_noalloc(plan, C.c_void_p(raw.data_ptr()),
                                           C.c_void_p(out.data_ptr()), W, st)


def test_noalloc_adjoint_matches_plan_scratch_adjoint(cuda):
    torch = cuda
    from msot_gb300 import _lib
    from pairs import make_pair, rel
    L = _lib.load()
    pm, _ = make_pair(n=96, n_det=128, n_samples=1600, radius=0.03, fov_half=0.0095,
                      norm=1.0, max_batch=4)
    W = 4
    g = torch.Generator(device="cuda").manual_seed(11)
    raw = torch.randn((W, 128, 1600), device="cuda", generator=g)
    ref = pm.interp_transpose(raw).cpu().numpy()
    out = torch.empty((W, 96 * 96), device="cuda")
    free = []
    for _ in range(2):
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        _lib.check(_noalloc(L, pm.plan, raw, out, W))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel(got, ref) < 1e-6
    # the first call may load the library's module (and with it the array)
    # under lazy loading; the second call allocates nothing
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free[1]


# (64 px, batch 1024): batch x pixels = 4 Mi exactly, the whole array up to
# its last element is used; (128 px, batch 130): the detector-group count the
# GPU's size asks for (2) is cut to the one group the array holds
@pytest.mark.parametrize("n,W,chunk", [(64, 1024, 128), (128, 130, 65)])
def test_noalloc_adjoint_at_the_array_limit(cuda, n, W, chunk):
    torch = cuda
    from msot_gb300 import _lib
    from pairs import make_pair, rel
    L = _lib.load()
    D, T = 64, 1200
    pm, _ = make_pair(n=n, n_det=D, n_samples=T, radius=0.02, fov_half=0.0063, norm=1.0,
                      max_batch=chunk)
    g = torch.Generator(device="cuda").manual_seed(12)
    raw = torch.randn((W, D, T), device="cuda", generator=g)
    ref = torch.cat([pm.interp_transpose(raw[i:i + chunk]) for i in range(0, W, chunk)])
    out = torch.full((W, n * n), float("nan"), device="cuda")
    for _ in range(2):
        _lib.check(_noalloc(L, pm.plan, raw, out, W))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel(got, ref.cpu().numpy()) < 1e-6


def test_noalloc_adjoint_rejects_oversized_batch(cuda):
    torch = cuda
    from msot_gb300 import _lib
    from pairs import make_pair
    L = _lib.load()
    pm, _ = make_pair(n=64, n_det=64, n_samples=1200, radius=0.02, fov_half=0.0063,
                      norm=1.0, max_batch=1)
    too_many = (4 << 20) // (64 * 64) + 1  # one instance over the fixed limit
    # real (small) device buffers: the call must fail on the size check
    # before anything is launched
    raw = torch.zeros(16, device="cuda")
    out = torch.zeros(16, device="cuda")
    rc = _noalloc(L, pm.plan, raw, out, too_many)
    assert rc == -2
    assert b"fixed scratch" in L.msot_last_error()
    torch.cuda.synchronize()
    assert torch.all(out == 0)
