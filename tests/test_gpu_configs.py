"""The benchmark configurations at their stated sizes, through the C ABI,
against the FP64 oracle.

  * 1024^3 Zel'dovich particles on a 1024^3 grid (L = 500000 kpc/h): the
    forward spectrum, then forward + adjoint with the density recomputed;
  * three species on a 512^3 grid (DM 256^3, gas 256^3, 1.2e7 lognormal
    stars with lognormal masses): 3 auto + 3 cross spectra in one call;
  * 256^3 Zel'dovich particles (L = 50000 kpc/h), 64 bins, the relative loss
    against a second realisation's spectrum: central finite differences (step
    1e-3 cell) on 256 random particles.

Tolerances: every P(k) bin within 1e-5 relative of the FP64 oracle (cross
spectra relative to sqrt(P_aa P_bb), their scale where they cross zero),
mode counts bit-exact; gradients within 1e-4 relative (norm-wise, and per
element of the largest element) of the FP64 reference gradient and of the
finite differences.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

P_RTOL = 1e-5
G_RTOL = 1e-4
WORKERS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def gp(native_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    import genpk_gb300
    return genpk_gb300


def host_available_bytes():
    with open("/proc/meminfo") as f:
        for line in f:
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) * 1024
    return 0


def bins_close(p, pr, cr, rtol=P_RTOL):
    ok = cr > 0
    rel = np.abs(p[ok] - pr[ok]) / np.abs(pr[ok])
    assert rel.max() <= rtol, f"max per-bin rel err {rel.max():.3e} at bin {np.argmax(rel)}"
    assert np.all(p[~ok] == 0)
    return rel.max()


def grad_close(g, ref, rtol=G_RTOL):
    g = np.asarray(g, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    norm = np.linalg.norm(g - ref) / np.linalg.norm(ref)
    elem = np.abs(g - ref).max() / np.abs(ref).max()
    assert norm <= rtol and elem <= rtol, (norm, elem)
    return norm


def test_large_box_1024_forward_and_recompute_adjoint(gp):
    """1024^3 = 1,073,741,824 particles (Zel'dovich lattice, equal masses, float32
    positions) on a 1024^3 FP32 grid, 64 bins.  Forward: every bin within 1e-5
    of the FP64 oracle, counts bit-exact.  Then forward + adjoint with the
    density grid recomputed rather than stored (recompute=True) for dL/dP_b =
    linspace(1, -1) / P_b: the gradients of 4096 sampled particles within 1e-4
    of the FP64 reference gradient (FP64 deposit, r2c, mode gradient and c2r of
    all particles, gathered at the sample).
    Memory: device about 45 GB (positions 12.9 GB, grid 4.3, 64-bit
    accumulator 8.6, cuFFT work area, gradients 12.9); host about 60 GB
    (positions 12.9 GB, the FP64 grid and spectrum 8.6 GB each, the FFT's
    temporaries and the c2r output 8.6 GB)."""
    import torch
    from genpk_gb300 import synth
    free, _ = torch.cuda.mem_get_info()
    if free < 64e9 or host_available_bytes() < 100e9:
        pytest.skip("needs 64 GB of free device memory and 100 GB of host memory")
    dims, box, nrbins = 1024, 500000.0, 64
    n = dims ** 3
    dpos = synth.zeldovich(dims, box, seed=1, device="cuda")
    m = O.total_mass(n, None, 1.0)
    with gp.Context(dims, nrbins) as ctx:
        ctx.deposit(0, box, dpos, None, 1.0)
        p, c, k = ctx.power(0, 0, m, m)
        g = np.linspace(1.0, -1.0, nrbins) / np.maximum(np.abs(p), 1e-30)
        gpos = torch.empty_like(dpos)
        ctx.adjoint(0, box, dpos, g, m, mass=1.0, grad_pos=gpos, recompute=True)
        torch.cuda.synchronize()
    sample = np.sort(np.random.default_rng(5).choice(n, 4096, replace=False))
    got = gpos[torch.from_numpy(sample).cuda()].cpu().numpy()
    del gpos
    pos = dpos.cpu().numpy()
    del dpos
    torch.cuda.empty_cache()
    pr, cr, kr, rpos, _, _ = O.reference_gradient_sampled(pos, box, dims, nrbins, g, sample,
                                                          None, 1.0, m_norm=m, workers=WORKERS)
    assert np.array_equal(c, cr)
    np.testing.assert_allclose(k, kr, rtol=1e-12)
    bins_close(p, pr, cr)
    grad_close(got, rpos)


def test_multispecies_512_three_auto_three_cross(gp):
    """DM: 256^3 Zel'dovich particles, mass 1.0; gas: the same field at 0.7
    displacement amplitude, mass 0.19; stars: 1.2e7 particles drawn from a
    lognormal density field (sigma_ln 1.5) with lognormal masses (mu -5,
    sigma 0.8).  One 512^3 grid per species, L = 100000 kpc/h, 64 bins; the 3
    auto and 3 cross spectra from one genpk_power_multi call."""
    import torch
    from genpk_gb300 import synth
    n, nrbins, box = 512, 64, 100000.0
    dm = synth.zeldovich(256, box, seed=11, device="cuda")
    gas = synth.zeldovich(256, box, seed=11, amplitude=0.7, device="cuda")
    spos, smass = synth.lognormal(12_000_000, box, 256, sigma=1.5, seed=12, mass_mu=-5.0,
                                  mass_sigma=0.8)
    species = [(dm, None, 1.0), (gas, None, 0.19), (spos, smass, 0.0)]
    ms = [O.total_mass(len(dm), None, 1.0), O.total_mass(len(gas), None, 0.19),
          O.total_mass(len(spos), smass)]
    pairs = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
    pm = [(ms[a], ms[b]) for a, b in pairs]
    with gp.Context(n, nrbins, nfields=3) as ctx:
        for f, (pos, masses, mass) in enumerate(species):
            ctx.deposit(f, box, pos if f < 2 else torch.from_numpy(pos).cuda(),
                        None if masses is None else torch.from_numpy(masses).cuda(), mass)
        p, c, k = ctx.power_multi(pairs, pm)
    port = O.port()
    spec = []
    for pos, masses, mass in species:
        hp = pos.cpu().numpy() if hasattr(pos, "cpu") else pos
        spec.append(O.rfft_padded(O.deposit(hp, box, n, masses, mass), WORKERS))
    ref = [port.powerspectrum(n, spec[a], spec[b], nrbins, ma, mb)
           for (a, b), (ma, mb) in zip(pairs, pm)]
    auto = {a: ref[i][0] for i, (a, b) in enumerate(pairs) if a == b}
    for i, (a, b) in enumerate(pairs):
        pr, cr, kr = ref[i]
        assert np.array_equal(c, cr)
        ok = cr > 0
        scale = np.maximum(np.abs(pr), np.sqrt(np.abs(auto[a] * auto[b])))
        rel = np.abs(p[i][ok] - pr[ok]) / scale[ok]
        assert rel.max() <= P_RTOL, (a, b, rel.max())
        assert np.all(p[i][~ok] == 0)


def _fd_central(F, bins, wmode, P, T, w, cnt, pos, masses, idx, axes, box, dims, h_cells):
    """Central differences of the FP64 oracle loss L = sum_b w_b (P_b - T_b)^2
    / T_b^2 for moving particle idx[q] by +-h along axes[q], evaluated exactly
    through the linearity of the DFT: the particle's CIC density is a tensor
    product of its per-axis weights, so moving it changes the spectrum by
    dF = m (X' - X) (x) Y (x) Z (the axis moved, primed, at the new
    position), and P_b(+-) = P_b + sum_{m in b} c V (2 Re(F conj dF) + |dF|^2)
    / (C_b M^2).  wmode = c V / (C_b M^2) per mode (0 for the k = 0 mode, whose
    bin index is mapped to 0), F the FP64 spectrum.
    The per-mode arithmetic runs in FP64 with torch on the device (no product
    kernel involved).  Returns dL/dpos (box units) per sampled particle."""
    import torch
    dev = "cuda"
    half = dims // 2
    units = dims / box
    k_full = torch.arange(dims, device=dev, dtype=torch.float64)
    k_half = torch.arange(half + 1, device=dev, dtype=torch.float64)
    ok = torch.from_numpy(cnt > 0).to(dev)
    Pt = torch.from_numpy(P).to(dev)
    Tt = torch.from_numpy(T).to(dev)
    wt = torch.from_numpy(w).to(dev)
    A = Pt - Tt

    def axis_vec(x, kv):
        f = np.floor(x)
        d = x - f
        lo = int(f) % dims
        hi = (lo + 1) % dims
        ph = -2.0 * np.pi / dims
        e_lo = torch.polar(torch.ones_like(kv), ph * kv * lo)
        e_hi = torch.polar(torch.ones_like(kv), ph * kv * hi)
        return (1.0 - d) * e_lo + d * e_hi

    out = np.zeros(len(idx))
    for q, (i, a) in enumerate(zip(idx, axes)):
        x = pos[i].astype(np.float64) * units
        m = float(masses[i]) if masses is not None else 1.0
        kvs = [k_full, k_full, k_half]
        base = [axis_vec(x[e], kvs[e]) for e in range(3)]
        dP = []
        for sgn in (1.0, -1.0):
            vec = list(base)
            vec[a] = axis_vec(x[a] + sgn * h_cells, kvs[a]) - base[a]
            dF = m * vec[0][:, None, None] * vec[1][None, :, None] * vec[2][None, None, :]
            term = wmode * (2.0 * (F * dF.conj()).real + dF.abs() ** 2)
            dP.append(torch.zeros(len(P), dtype=torch.float64, device=dev).index_add_(
                0, bins.reshape(-1), term.reshape(-1)))
        dp, dm = dP
        # L(+) - L(-) = sum_b w_b (dp - dm)(2 A + dp + dm) / T_b^2, bins with count > 0
        diff = torch.where(ok, wt * (dp - dm) * (2.0 * A + dp + dm) / (Tt * Tt), 0.0).sum()
        out[q] = float(diff) / (2.0 * h_cells / units)
    return out


def test_differentiable_pk_256_central_finite_differences(gp):
    """256^3 Zel'dovich particles (L = 50000 kpc/h, float32 positions, masses
    1 + 0.1 N(0, 1)), 64 bins, loss sum_b (P_b - T_b)^2 / T_b^2 against the
    spectrum T of a second seed.  The GPU adjoint, given the FP64 loss's
    dL/dP_b, against central differences (step 1e-3 cell) of that FP64 oracle
    loss for the position gradients of 256 random particles.  The differences
    are first checked against the FP64 reference gradient (to 1e-6), which
    pins the difference machinery itself.  Particles
    within one step of a cell face along the differenced axis are left out:
    the CIC density has a kink there, where a difference is not a derivative."""
    import torch
    from genpk_gb300 import synth
    dims, box, nrbins = 256, 50000.0, 64
    pos = synth.zeldovich(dims, box, seed=1)
    tgt = synth.zeldovich(dims, box, seed=2)
    rng = np.random.default_rng(7)
    masses = (1.0 + 0.1 * rng.standard_normal(len(pos))).astype(np.float32)
    m = O.total_mass(len(pos), masses)
    mt = O.total_mass(len(tgt), None, 1.0)
    T, cnt_t, _ = O.pk(tgt, box, dims, nrbins, None, 1.0, m_norm=mt, workers=WORKERS)
    T = np.where(cnt_t > 0, T, 1.0)
    w = np.ones(nrbins)
    # FP64 oracle forward (its spectrum is kept for the differences)
    f = O.rfft_padded(O.deposit(pos, box, dims, masses, 0.0), WORKERS)
    P, cnt, _ = O.port().powerspectrum(dims, f, f, nrbins, m, m)
    g64 = np.where(cnt > 0, 2.0 * w * (P - T) / T ** 2, 0.0)  # dL/dP_b of the FP64 loss
    with gp.Context(dims, nrbins) as ctx:
        ctx.deposit(0, box, pos, masses)
        p, c, _ = ctx.power(0, 0, m, m)
        assert np.array_equal(c, cnt)
        bins_close(p, P, cnt)
        gpos, _, _ = ctx.adjoint(0, box, pos, g64, m, masses=masses)
    # the sample: 256 particles and axes away from cell faces along the axis
    h_cells = 1e-3
    units = dims / box
    frac = pos.astype(np.float64) * units
    frac -= np.floor(frac)
    idx, axes = [], []
    while len(idx) < 256:
        i, a = int(rng.integers(len(pos))), int(rng.integers(3))
        if 2 * h_cells < frac[i, a] < 1 - 2 * h_cells and i not in idx:
            idx.append(i)
            axes.append(a)
    idx, axes = np.array(idx), np.array(axes)
    # the FP64 reference gradient at the sample
    _, _, _, rpos, _, _ = O.reference_gradient_sampled(pos, box, dims, nrbins, g64, idx, masses,
                                                       0.0, m_norm=m, workers=WORKERS)
    bins, cm, v = O.mode_tables(dims, nrbins)
    cb = np.where(cnt > 0, cnt, 1).astype(np.float64)
    wmode = np.where(bins >= 0, cm * v / (cb[np.maximum(bins, 0)] * m * m), 0.0)
    dev = "cuda"
    Ft = torch.from_numpy(f).to(dev)
    bt = torch.from_numpy(np.maximum(bins, 0)).to(dev)
    wt = torch.from_numpy(wmode).to(dev)
    fd = _fd_central(Ft, bt, wt, P, T, w, cnt, pos, masses, idx, axes, box, dims, h_cells)
    ref = rpos[np.arange(len(idx)), axes]
    assert np.linalg.norm(fd - ref) / np.linalg.norm(ref) <= 1e-6
    got = gpos[idx, axes].astype(np.float64)
    grad_close(got, fd)


def test_kz_major_transform_1024(gp):
    """The N = 1024 transform: a field pending in the accumulator goes through
    the kz-major z pass, one batched 2-D C2C over the kz planes and the
    kz-major binning (which clears the accumulator).  256^3 lattice particles
    on the 1024^3 grid: its auto spectrum, binning the kept spectrum again, the
    kz-major adjoint from the kept spectrum (mode gradient, inverse 2-D C2C,
    inverse z pass), and a cross spectrum with a second field (which reads the
    spectrum back in the in-place r2c layout), against the FP64 oracle.  The 3-D
    cuFFT R2C path on the same particles agrees to 5e-5 (its lowest bin is
    1.8e-5 from the oracle on this sparse field, 1/64 particle per cell;
    the kz-major transform stays within 1e-5)."""
    import torch
    from genpk_gb300 import synth
    dims, box, nrbins = 1024, 500000.0, 64
    pos = torch.from_numpy(synth.zeldovich(256, box, seed=7)).cuda()
    other = torch.from_numpy(synth.zeldovich(256, box, seed=8)).cuda()
    n = pos.shape[0]
    m = O.total_mass(n, None, 1.0)
    g = np.linspace(1.0, -1.0, nrbins) * 1e3
    res = {}
    for mode in (gp.api.FFT_AUTO, gp.api.FFT_CUFFT3D):
        with gp.Context(dims, nrbins, nfields=2, timing=True) as ctx:
            ctx.set_engine(gp.api.ENGINE_STREAM)
            ctx.set_fft_mode(mode)
            ctx.deposit(0, box, pos, None, 1.0)
            ctx.timing_reset()
            p, c, k = ctx.power(0, 0, m, m)
            st = ctx.stage_times()
            again, _, _ = ctx.power(0, 0, m, m)
            ctx.timing_reset()
            gpos = ctx.adjoint(0, box, pos, g, m, mass=1.0)[0].cpu().numpy()  # kept spectrum
            sta = ctx.stage_times()
            ctx.zero(0)
            ctx.deposit(0, box, pos, None, 1.0)
            ctx.power(0, 0, m, m)
            ctx.deposit(1, box, other, None, 1.0)
            cross, _, _ = ctx.power(0, 1, m, m)
            auto_after, _, _ = ctx.power(0, 0, m, m)
            if mode == gp.api.FFT_AUTO:
                # the same particles from host memory in two chunks: staged,
                # deposited as one pass, and transformed kz-major as well
                hp = pos.cpu().numpy()
                ctx.zero(0)
                ctx.deposit(0, box, hp[: n // 2], None, 1.0)
                ctx.deposit(0, box, hp[n // 2:], None, 1.0)
                ctx.timing_reset()
                p_host, _, _ = ctx.power(0, 0, m, m)
                assert "zfft_kz" in ctx.stage_times()
                assert np.array_equal(p_host, p)
            res[mode] = (p, c, again, cross, auto_after, gpos, st, sta)
    pk, ck, again, cross, auto_after, gk, st, sta = res[gp.api.FFT_AUTO]
    p3, c3, _, _, _, g3, st3, _ = res[gp.api.FFT_CUFFT3D]
    assert "zfft_kz" in st and "fft2d_kz" in st and "bin_kz" in st, st
    assert "adj_modes_kz" in sta and "adj_fft2d_kz" in sta and "kz_to_rows" not in sta, sta
    assert "win_convert" not in st and "zfft_kz" not in st3
    assert np.array_equal(ck, c3)
    hp, ho = pos.cpu().numpy(), other.cpu().numpy()
    fa = O.rfft_padded(O.deposit(hp, box, dims, None, 1.0), WORKERS)
    fb = O.rfft_padded(O.deposit(ho, box, dims, None, 1.0), WORKERS)
    pr, cr, kr = O.cross_pk(fa, fa, dims, nrbins, m, m)
    pb, _, _ = O.cross_pk(fb, fb, dims, nrbins, m, m)
    px, _, _ = O.cross_pk(fa, fb, dims, nrbins, m, m)
    del fa, fb
    assert np.array_equal(ck, cr)
    bins_close(pk, pr, cr)
    bins_close(p3, pr, cr, rtol=5e-5)
    np.testing.assert_allclose(again, pk, rtol=1e-12)      # the same kernel on the kept spectrum
    bins_close(auto_after, pr, cr)                         # binned from the r2c layout
    ok = cr > 0
    scale = np.maximum(np.abs(px), np.sqrt(np.abs(pr * pb)))
    rel = np.abs(cross[ok] - px[ok]) / scale[ok]
    assert rel.max() <= P_RTOL, rel.max()
    sample = np.sort(np.random.default_rng(3).choice(n, 2048, replace=False))
    _, _, _, rpos, _, _ = O.reference_gradient_sampled(hp, box, dims, nrbins, g, sample, None, 1.0,
                                                       m_norm=m, workers=WORKERS)
    grad_close(gk[sample], rpos)
    grad_close(g3[sample], rpos)
