"""dm_diagnostics_noalloc: the diagnostics for callers that can't allocate
device memory (their own memory pool or budget, or no cudaMalloc-induced
device synchronisation allowed).  Its partial sums live in a fixed
file-scope device array instead of a buffer allocated per call.

Checked through the C ABI against dm_cloud_diagnostics (the existing
entry point) on two calls in a row, since every call reuses -- and must
fully overwrite -- the same shared scratch.  This file sorts last so a
run that stops at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from demon_simulation_code_gb300 import Context, DeviceCloud, _lib, workloads as W

pytestmark = pytest.mark.gpu


def _cloud(n, seed):
    c0 = W.disk_cloud(n, 2e-3 * np.sqrt(n / 2000.0), seed)
    rng = np.random.default_rng(seed + 1)
    c0.vx = rng.normal(0, 1e-3, n)
    c0.vy = rng.normal(0, 1e-3, n)
    return c0


def test_noalloc_diagnostics_matches_cloud_diagnostics_twice():
    import torch

    lib = _lib.load()
    ctx = Context(0)
    stream = torch.cuda.current_stream().cuda_stream
    # two different clouds in a row: the second call must not see the first's partials
    for n, seed in ((3000, 5), (1111, 9)):
        c0 = _cloud(n, seed)
        ref = DeviceCloud.from_cloud(ctx, c0).diagnostics()
        dev = [torch.tensor(a, dtype=torch.float64, device="cuda")
               for a in (c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m)]
        out = torch.full((5,), float("nan"), dtype=torch.float64, device="cuda")
        p = _lib.force_params(**c0.params())
        rc = lib.dm_diagnostics_noalloc(n, *(t.data_ptr() for t in dev), ctypes.byref(p),
                                        out.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got, ref, rtol=1e-11, atol=1e-30)


def _call(lib, c0, params, stream):
    import torch

    dev = [torch.tensor(a, dtype=torch.float64, device="cuda")
           for a in (c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m)]
    out = torch.full((5,), float("nan"), dtype=torch.float64, device="cuda")
    p = _lib.force_params(**params)
    rc = lib.dm_diagnostics_noalloc(c0.n, *(t.data_ptr() for t in dev), ctypes.byref(p),
                                    out.data_ptr(), stream)
    assert rc == 0
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_diagnostics_match_the_oracle_including_the_size_limit():
    """The device reduction itself (per-block partials in the fixed scratch,
    then one block's strided sums) against the oracle's FP64 diagnostics:
    a small cloud, then n = 524,288, the most the scratch holds (4096
    blocks, each of the finishing block's 256 threads summing 16 rows) --
    with the pair term off so that the large call stays short."""
    import torch

    import oracle

    lib = _lib.load()
    o = oracle.Oracle()
    stream = torch.cuda.current_stream().cuda_stream
    small = _cloud(2048, 3)
    big = _cloud(524288, 4)
    for c0, flags in ((small, None), (big, 3)):
        params = c0.params() if flags is None else {**c0.params(), "flags": flags}
        got = _call(lib, c0, params, stream)
        ref = o.diagnostics(c0.x, c0.y, c0.vx, c0.vy, c0.q, c0.m, oracle.make_params(**params))
        scale = np.abs(ref).max()
        np.testing.assert_allclose(got, ref, rtol=1e-11, atol=1e-11 * scale)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch

    lib = _lib.load()
    dummy = torch.zeros(4, dtype=torch.float64, device="cuda")
    out = torch.zeros(5, dtype=torch.float64, device="cuda")
    p = _lib.force_params(flags=7, shielding=2e4, confine=1e8, gamma=3.0)
    ptrs = [dummy.data_ptr()] * 6
    for n in (0, 524288 + 1):
        rc = lib.dm_diagnostics_noalloc(n, *ptrs, ctypes.byref(p), out.data_ptr(), None)
        assert rc == _lib.DM_ERR_ARG
