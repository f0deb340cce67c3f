"""GPU test of msot_interp_transpose_noalloc, the adjoint entry point that
allocates no device memory (for callers that are not allowed to, e.g. a host
application whose device memory belongs to another allocator).  It must give
the same result as msot_interp_transpose, which uses the plan's scratch, on
two calls in a row (the second call reuses the library's fixed array).

The file name sorts last so that a `-x` run reaches it only after every
other test; it also passes when run alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


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
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(2):
        out.fill_(float("nan"))
        _lib.check(L.msot_interp_transpose_noalloc(pm.plan, C.c_void_p(raw.data_ptr()),
                                                   C.c_void_p(out.data_ptr()), W, st))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel(got, ref) < 1e-6


def test_noalloc_adjoint_rejects_oversized_batch(cuda):
    from msot_gb300 import _lib
    from pairs import make_pair
    L = _lib.load()
    pm, _ = make_pair(n=64, n_det=64, n_samples=1200, radius=0.02, fov_half=0.0063,
                      norm=1.0, max_batch=1)
    too_many = (4 << 20) // (64 * 64) + 1  # one instance over the fixed limit
    rc = L.msot_interp_transpose_noalloc(pm.plan, C.c_void_p(1), C.c_void_p(1), too_many, None)
    assert rc == -2
    assert b"fixed scratch" in L.msot_last_error()
