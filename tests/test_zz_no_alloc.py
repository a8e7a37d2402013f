"""genpk_power_noalloc through the C ABI: binning without any allocation.

Callers that run under an allocator owning the whole GPU, or inside a loop that
cannot pay for an allocation, cannot create a context (which allocates grids,
plans and scratch).  genpk_power_noalloc bins a spectrum they already hold on
the GPU into their own output buffer, using a fixed static scratch array.
This checks it against the context path (genpk_load_spectrum + genpk_power) on
the same spectrum, within the 1e-5 per-bin tolerance of the parity tests, on
two calls in a row (the second reuses the array the first left behind).

The file name sorts last, so a run that stops at the first failure has run
every other test before this one.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

P_RTOL = 1e-5


def _call(lib, native, a, b, dims, nrbins, ma, mb, out):
    count = np.zeros(nrbins, dtype=np.int32)
    keffs = np.zeros(nrbins)
    rc = lib.genpk_power_noalloc(ctypes.c_void_p(a.data_ptr()),
                                 ctypes.c_void_p(b.data_ptr()) if b is not None else None,
                                 dims, nrbins, ma, mb, ctypes.c_void_p(out.data_ptr()),
                                 count.ctypes.data_as(native.c_i32p),
                                 keffs.ctypes.data_as(native.c_f64p), None)
    return rc, count, keffs


def test_noalloc_power_matches_context_power(native_lib):
    import torch

    from genpk_gb300 import Context, native
    assert torch.cuda.is_available()
    lib = native.load()
    dims, nrbins = 64, 32
    gen = torch.Generator(device="cuda").manual_seed(5)
    rho_a = torch.rand((dims, dims, dims), generator=gen, device="cuda")
    rho_b = rho_a + 0.3 * torch.rand((dims, dims, dims), generator=gen, device="cuda")
    spec_a = torch.fft.rfftn(rho_a).contiguous()  # in-place r2c layout, complex64
    spec_b = torch.fft.rfftn(rho_b).contiguous()
    ma, mb = float(rho_a.double().sum()), float(rho_b.double().sum())
    with Context(dims, nrbins, nfields=2) as ctx:
        ctx.load_spectrum(0, spec_a.cpu().numpy())
        ctx.load_spectrum(1, spec_b.cpu().numpy())
        ref_auto, ref_count, ref_keffs = ctx.power(0, 0, ma, ma)
        ref_cross, _, _ = ctx.power(0, 1, ma, mb)
    out = torch.empty(nrbins, dtype=torch.float64, device="cuda")
    for _ in range(2):
        out.fill_(float("nan"))
        rc, count, keffs = _call(lib, native, spec_a, None, dims, nrbins, ma, ma, out)
        torch.cuda.synchronize()
        assert rc == 0
        got = out.cpu().numpy()
        ok = ref_count > 0
        np.testing.assert_allclose(got[ok], ref_auto[ok], rtol=P_RTOL)
        assert np.all(got[~ok] == 0)
        assert np.array_equal(count, ref_count)
        np.testing.assert_allclose(keffs, ref_keffs, rtol=1e-12)
    for _ in range(2):
        out.fill_(float("nan"))
        rc, _, _ = _call(lib, native, spec_a, spec_b, dims, nrbins, ma, mb, out)
        torch.cuda.synchronize()
        assert rc == 0
        got = out.cpu().numpy()
        ok = ref_count > 0
        np.testing.assert_allclose(got[ok], ref_cross[ok], rtol=P_RTOL,
                                   atol=P_RTOL * np.abs(ref_cross[ok]).max())


def test_noalloc_rejects_sizes_beyond_its_limit(native_lib):
    import torch

    from genpk_gb300 import native
    lib = native.load()
    spec = torch.zeros(8, dtype=torch.complex64, device="cuda")
    out = torch.zeros(8, dtype=torch.float64, device="cuda")
    big = lib.genpk_power_noalloc(ctypes.c_void_p(spec.data_ptr()), None, 2048, 8, 1.0, 1.0,
                                  ctypes.c_void_p(out.data_ptr()), None, None, None)
    many = lib.genpk_power_noalloc(ctypes.c_void_p(spec.data_ptr()), None, 64, 4096, 1.0, 1.0,
                                   ctypes.c_void_p(out.data_ptr()), None, None, None)
    assert big == 7 and many == 7  # GENPK_ERR_UNSUPPORTED
