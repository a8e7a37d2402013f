"""genpk_power_noalloc through the C ABI: binning without any allocation.

Callers that run under an allocator owning the whole GPU, or inside a loop that
cannot pay for an allocation, cannot create a context (which allocates grids,
plans and scratch).  genpk_power_noalloc bins a spectrum they already hold on
the GPU into their own output buffer, using a fixed static scratch array.
This checks it against the context path (genpk_load_spectrum + genpk_power) on
the same spectrum, within the 1e-5 per-bin tolerance of the parity tests, on
two calls in a row (the second reuses the array the first left behind), then
after a call at another grid and bin count.

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


def _case(dims, nrbins, seed):
    """Two correlated densities on a dims^3 grid, their spectra (in-place r2c
    layout, complex64) and masses, and the context path's auto, second auto and
    cross spectra of them (genpk_load_spectrum + genpk_power)."""
    import torch

    from genpk_gb300 import Context
    gen = torch.Generator(device="cuda").manual_seed(seed)
    rho_a = torch.rand((dims, dims, dims), generator=gen, device="cuda")
    rho_b = rho_a + 0.3 * torch.rand((dims, dims, dims), generator=gen, device="cuda")
    spec_a = torch.fft.rfftn(rho_a).contiguous()
    spec_b = torch.fft.rfftn(rho_b).contiguous()
    ma, mb = float(rho_a.double().sum()), float(rho_b.double().sum())
    with Context(dims, nrbins, nfields=2) as ctx:
        ctx.load_spectrum(0, spec_a.cpu().numpy())
        ctx.load_spectrum(1, spec_b.cpu().numpy())
        ref_aa, ref_count, ref_keffs = ctx.power(0, 0, ma, ma)
        ref_bb, _, _ = ctx.power(1, 1, mb, mb)
        ref_ab, _, _ = ctx.power(0, 1, ma, mb)
    return dict(dims=dims, nrbins=nrbins, a=spec_a, b=spec_b, ma=ma, mb=mb, aa=ref_aa,
                bb=ref_bb, ab=ref_ab, count=ref_count, keffs=ref_keffs)


def _check(lib, native, c, out):
    """Auto then cross spectrum of case c through the allocation-free call,
    each bin within P_RTOL of the context path's (cross bins relative to
    sqrt(P_aa P_bb), the scale of a cross spectrum that may cross zero)."""
    import torch
    ok = c["count"] > 0
    out.fill_(float("nan"))
    rc, count, keffs = _call(lib, native, c["a"], None, c["dims"], c["nrbins"], c["ma"], c["ma"],
                             out)
    torch.cuda.synchronize()
    assert rc == 0
    got = out[:c["nrbins"]].cpu().numpy()
    np.testing.assert_allclose(got[ok], c["aa"][ok], rtol=P_RTOL)
    assert np.all(got[~ok] == 0)
    assert np.array_equal(count, c["count"])
    np.testing.assert_allclose(keffs, c["keffs"], rtol=1e-12)
    out.fill_(float("nan"))
    rc, _, _ = _call(lib, native, c["a"], c["b"], c["dims"], c["nrbins"], c["ma"], c["mb"], out)
    torch.cuda.synchronize()
    assert rc == 0
    got = out[:c["nrbins"]].cpu().numpy()
    scale = np.sqrt(np.abs(c["aa"] * c["bb"]))
    rel = np.abs(got[ok] - c["ab"][ok]) / np.maximum(np.abs(c["ab"][ok]), scale[ok])
    assert rel.max() <= P_RTOL, rel.max()


def test_noalloc_power_matches_context_power(native_lib):
    """Two calls in a row at one size, one at another size (the bin tables are
    rebuilt and uploaded again), then the first size again."""
    import torch

    from genpk_gb300 import native
    assert torch.cuda.is_available()
    lib = native.load()
    first = _case(64, 32, seed=5)
    other = _case(32, 16, seed=6)
    out = torch.empty(64, dtype=torch.float64, device="cuda")
    for c in (first, first, other, first):
        _check(lib, native, c, out)


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
