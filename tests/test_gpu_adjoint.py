"""GPU adjoint (gradient of a P(k) loss w.r.t. positions and masses) against the
FP64 reference gradient (oracle.reference_gradient) and central finite
differences of the FP64 oracle forward.

Tolerances: gradients within 1e-4 relative of the FP64 reference gradient,
norm-wise, and per element within 1e-4 of the largest element.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

G_RTOL = 1e-4


@pytest.fixture(scope="module")
def gp(native_lib):
    import torch
    assert torch.cuda.is_available()
    import genpk_gb300
    return genpk_gb300


def loss_grad(p, target, count):
    ok = count > 0
    d = np.where(ok, (p - target) / target, 0.0)
    return float(np.sum(d * d)), np.where(ok, 2.0 * (p - target) / target ** 2, 0.0)


def grad_close(g, ref, rtol=G_RTOL):
    g = np.asarray(g, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    norm = np.linalg.norm(g - ref) / np.linalg.norm(ref)
    elem = np.abs(g - ref).max() / np.abs(ref).max()
    assert norm <= rtol and elem <= rtol, (norm, elem)
    return norm


def make_case(kind, dims, box, seed, nrbins, var):
    from genpk_gb300 import synth
    if kind == "uniform":
        pos = synth.uniform(dims ** 3, box, seed=seed)
    else:
        pos = synth.zeldovich(dims, box, seed=seed)
    rng = np.random.default_rng(seed + 100)
    masses = (rng.random(len(pos)) + 0.5).astype(np.float32) if var else None
    return pos, masses


@pytest.mark.parametrize("kind,dims,var", [("uniform", 32, False), ("zeldovich", 32, True),
                                           ("zeldovich", 64, False), ("uniform", 48, True),
                                           ("uniform", 64, True), ("zeldovich", 128, True)])
def test_adjoint_matches_fp64_reference_gradient(gp, kind, dims, var):
    """Grids of 64 to 512 cells (powers of two) take the fused inverse x pass
    + 2-D C2R; the others the mode-gradient kernel + 3-D C2R."""
    box, nrbins, mass = 1000.0, 24, 1.0
    pos, masses = make_case(kind, dims, box, 3, nrbins, var)
    tgt_pos, _ = make_case(kind, dims, box, 4, nrbins, False)
    m = O.total_mass(len(pos), masses, 0.0 if var else mass)
    target, cnt, _ = O.pk(tgt_pos, box, dims, nrbins, None, 1.0)
    target = np.where(cnt > 0, target, 1.0)
    with gp.Context(dims, nrbins) as ctx:
        ctx.deposit(0, box, pos, masses, mass)
        p, c, _ = ctx.power(0, 0, m, m)
        _, g = loss_grad(p, target, c)
        gpos, gmass, dldm = ctx.adjoint(0, box, pos, g, m, masses=masses, mass=mass)
    rpos, rmass, rdldm = O.reference_gradient(pos, box, dims, nrbins, g, masses, mass, m_norm=m)
    grad_close(gpos, rpos)
    if var:
        grad_close(gmass, rmass)
    assert abs(dldm - rdldm) <= G_RTOL * abs(rdldm) + 1e-300


def test_adjoint_many_bins(gp):
    """More bins than the fused forward binning takes (300 > 256): the forward
    spectrum is binned by the separate kernel, the adjoint's fused inverse x
    pass still holds its 300 thresholds and coefficients in shared memory."""
    dims, box, nrbins = 64, 1000.0, 300
    pos, _ = make_case("zeldovich", dims, box, 11, nrbins, False)
    tgt, _ = make_case("zeldovich", dims, box, 12, nrbins, False)
    m = O.total_mass(len(pos), None, 1.0)
    target, cnt, _ = O.pk(tgt, box, dims, nrbins, None, 1.0)
    target = np.where(cnt > 0, target, 1.0)
    with gp.Context(dims, nrbins) as ctx:
        ctx.deposit(0, box, pos, None, 1.0)
        p, c, _ = ctx.power(0, 0, m, m)
        _, g = loss_grad(p, target, c)
        gpos, _, dldm = ctx.adjoint(0, box, pos, g, m, mass=1.0)
    rpos, _, rdldm = O.reference_gradient(pos, box, dims, nrbins, g, None, 1.0, m_norm=m)
    grad_close(gpos, rpos)
    assert abs(dldm - rdldm) <= G_RTOL * abs(rdldm) + 1e-300


def test_adjoint_paths_agree_at_512(gp):
    """At N = 512 the mode-gradient kernel (3-D cuFFT mode) walks each row in
    two chunks of kz (257 modes > 256); the default path applies the mode
    gradient inside the inverse x pass.  The two gradients agree to FP32
    transform rounding."""
    import torch
    from genpk_gb300 import synth
    dims, box, nrbins = 512, 1000.0, 24
    pos = torch.from_numpy(synth.uniform(200_000, box, seed=21)).cuda()
    m = O.total_mass(200_000, None, 1.0)
    g = np.linspace(1.0, -1.0, nrbins) * 1e3
    out = {}
    with gp.Context(dims, nrbins) as ctx:
        for mode in (gp.api.FFT_AUTO, gp.api.FFT_CUFFT3D):
            ctx.set_fft_mode(mode)
            ctx.zero(0)
            ctx.deposit(0, box, pos, None, 1.0)
            ctx.power(0, 0, m, m)
            out[mode] = ctx.adjoint(0, box, pos, g, m, mass=1.0)[0].cpu().numpy()
    a, b = out[gp.api.FFT_AUTO], out[gp.api.FFT_CUFFT3D]
    assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 1e-5


def test_adjoint_recompute_equals_stored_spectrum(gp):
    dims, box, nrbins = 32, 100.0, 16
    pos, masses = make_case("zeldovich", dims, box, 9, nrbins, True)
    m = O.total_mass(len(pos), masses)
    g = np.linspace(-1.0, 1.0, nrbins) * 1e3
    with gp.Context(dims, nrbins) as ctx:
        ctx.deposit(0, box, pos, masses)
        ctx.power(0, 0, m, m)
        a = ctx.adjoint(0, box, pos, g, m, masses=masses)
        b = ctx.adjoint(0, box, pos, g, m, masses=masses, recompute=True)
        ctx.zero(0)
        c = ctx.adjoint(0, box, pos, g, m, masses=masses)  # nothing stored: recomputes
    for x, y in ((a, b), (a, c)):
        np.testing.assert_allclose(x[0], y[0], rtol=1e-5, atol=1e-6 * np.abs(a[0]).max())
        np.testing.assert_allclose(x[1], y[1], rtol=1e-5, atol=1e-6 * np.abs(a[1]).max())


def test_adjoint_device_pointers(gp):
    import torch
    dims, box, nrbins = 32, 100.0, 16
    pos, masses = make_case("uniform", dims, box, 5, nrbins, True)
    m = O.total_mass(len(pos), masses)
    g = np.ones(nrbins)
    with gp.Context(dims, nrbins) as ctx:
        ctx.deposit(0, box, pos, masses)
        ctx.power(0, 0, m, m)
        h = ctx.adjoint(0, box, pos, g, m, masses=masses, recompute=True)
        d = ctx.adjoint(0, box, torch.from_numpy(pos).cuda(), g, m,
                        masses=torch.from_numpy(masses).cuda(), recompute=True)
    # the deposit is bit-reproducible, so host and device inputs give identical gradients
    assert np.array_equal(d[0].cpu().numpy(), h[0])
    assert np.array_equal(d[1].cpu().numpy(), h[1])


def test_adjoint_ragged_tile_and_unaligned_arrays(gp):
    """A ragged particle count (not a multiple of 4, 256 or 1024) through
    aligned device arrays (the gather's four-particles-per-thread path) and
    through device arrays that start 12 bytes past a 16-byte boundary (one
    particle per thread): the same gradients bit for bit, and the FP64
    reference gradient.  Non-finite positions, one among the first particles
    and one among the last n % 4, get zero gradients and leave the others
    unchanged."""
    import torch
    dims, box, nrbins, n = 32, 1000.0, 16, 3003
    pos, masses = make_case("uniform", dims, box, 7, nrbins, True)
    pos, masses = pos[:n].copy(), masses[:n].copy()
    m = O.total_mass(n, masses)
    g = np.linspace(-1.0, 1.0, nrbins) * 1e3
    al = torch.from_numpy(pos).cuda()
    am = torch.from_numpy(masses).cuda()
    bp = torch.empty(3 * n + 3, dtype=torch.float32, device="cuda")
    bp[3:] = al.reshape(-1)
    bm = torch.empty(n + 3, dtype=torch.float32, device="cuda")
    bm[3:] = am
    gb = torch.empty(3 * n + 3, dtype=torch.float32, device="cuda")
    gmb = torch.empty(n + 3, dtype=torch.float32, device="cuda")
    with gp.Context(dims, nrbins) as ctx:
        ctx.deposit(0, box, pos, masses)
        ctx.power(0, 0, m, m)
        a = ctx.adjoint(0, box, al, g, m, masses=am, recompute=True)
        b = ctx.adjoint(0, box, bp[3:], g, m, masses=bm[3:], recompute=True,
                        grad_pos=gb[3:], grad_mass=gmb[3:])
        ctx.zero(0)
        ctx.deposit(0, box, pos, masses)
        ctx.power(0, 0, m, m)
        bad = al.clone()
        bad[5, 1] = float("nan")
        bad[n - 1, 2] = float("inf")
        c = ctx.adjoint(0, box, bad, g, m, masses=am)  # from the kept spectrum
    assert bp[3:].data_ptr() % 16 == 12
    assert np.array_equal(a[0].cpu().numpy(), gb[3:].reshape(n, 3).cpu().numpy())
    assert np.array_equal(a[1].cpu().numpy(), gmb[3:].cpu().numpy())
    keep = np.ones(n, dtype=bool)
    keep[[5, n - 1]] = False
    cp, cm = c[0].cpu().numpy(), c[1].cpu().numpy()
    assert np.all(cp[~keep] == 0.0) and np.all(cm[~keep] == 0.0)
    assert np.array_equal(cp[keep], a[0].cpu().numpy()[keep])
    assert np.array_equal(cm[keep], a[1].cpu().numpy()[keep])
    rpos, rmass, _ = O.reference_gradient(pos, box, dims, nrbins, g, masses, 0.0, m_norm=m)
    grad_close(a[0].cpu().numpy(), rpos)
    grad_close(a[1].cpu().numpy(), rmass)


def test_adjoint_central_finite_differences_256_particles(gp):
    """Central differences (step 1e-3 cell) of the FP64 oracle loss on 256
    random particles against the GPU gradient."""
    dims, box, nrbins = 32, 3200.0, 16
    pos, masses = make_case("zeldovich", dims, box, 11, nrbins, True)
    tgt, _ = make_case("zeldovich", dims, box, 12, nrbins, False)
    target, cnt, _ = O.pk(tgt, box, dims, nrbins, None, 1.0)
    target = np.where(cnt > 0, target, 1.0)

    def oracle_loss(p64, m32):
        mm = O.total_mass(len(p64), m32)
        pw, c, _ = O.pk(p64.astype(np.float32), box, dims, nrbins, m32, 0.0, m_norm=mm)
        return loss_grad(pw, target, c)[0]

    m = O.total_mass(len(pos), masses)
    with gp.Context(dims, nrbins) as ctx:
        ctx.deposit(0, box, pos, masses)
        p, c, _ = ctx.power(0, 0, m, m)
        _, g = loss_grad(p, target, c)
        gpos, gmass, _ = ctx.adjoint(0, box, pos, g, m, masses=masses)
    rng = np.random.default_rng(0)
    idx = rng.choice(len(pos), 256, replace=False)
    axes = rng.integers(0, 3, 256)
    h = 1e-3 * box / dims
    p64 = pos.astype(np.float64)
    fd = np.empty(256)
    for q, (i, a) in enumerate(zip(idx, axes)):
        pp, pm = p64.copy(), p64.copy()
        pp[i, a] += h
        pm[i, a] -= h
        fd[q] = (oracle_loss(pp, masses) - oracle_loss(pm, masses)) / (2 * h)
    got = gpos[idx, axes].astype(np.float64)
    scale = np.abs(fd).max()
    err = np.abs(got - fd)
    # CIC is piecewise linear: a step that crosses a cell face has an O(h) kink
    # error, so allow a handful of outliers and bound the rest tightly.
    assert np.mean(err <= 2e-3 * scale) >= 0.97, np.sort(err / scale)[-10:]
    assert np.linalg.norm(got - fd) / np.linalg.norm(fd) <= 2e-2


def test_autograd_binding(gp):
    import torch
    from genpk_gb300 import autograd as ag
    dims, box, nrbins = 32, 100.0, 16
    pos, masses = make_case("zeldovich", dims, box, 21, nrbins, True)
    tgt, _ = make_case("zeldovich", dims, box, 22, nrbins, False)
    target, cnt, _ = O.pk(tgt, box, dims, nrbins, None, 1.0)
    target = np.where(cnt > 0, target, 1.0)
    tp = torch.from_numpy(pos).cuda().requires_grad_(True)
    tm = torch.from_numpy(masses).cuda().requires_grad_(True)
    with gp.Context(dims, nrbins) as ctx:
        p = ag.power_spectrum(tp, tm, ctx, box)
        loss = ag.relative_loss(p, target, cnt)
        loss.backward()
    m = O.total_mass(len(pos), masses)
    _, g = loss_grad(p.detach().cpu().numpy(), target, cnt)
    rpos, rmass, _ = O.reference_gradient(pos, box, dims, nrbins, g, masses, 0.0, m_norm=m)
    grad_close(tp.grad.cpu().numpy(), rpos)
    grad_close(tm.grad.cpu().numpy(), rmass)


def test_adjoint_differentiable_pk_256(gp):
    """256^3 Zel'dovich particles on a 256^3 grid (L = 50000 kpc/h), 64 bins,
    loss against the spectrum of a second seed: GPU gradient vs the FP64
    reference gradient."""
    from genpk_gb300 import synth
    dims, box, nrbins = 256, 50000.0, 64
    pos = synth.zeldovich(dims, box, seed=1)
    tgt = synth.zeldovich(dims, box, seed=2)
    rng = np.random.default_rng(7)
    masses = (1.0 + 0.1 * rng.standard_normal(len(pos))).astype(np.float32)
    m = O.total_mass(len(pos), masses)
    with gp.Context(dims, nrbins) as ctx:
        ctx.deposit(0, box, tgt, None, 1.0)
        target, cnt, _ = ctx.power(0, 0, O.total_mass(len(tgt), None, 1.0),
                                   O.total_mass(len(tgt), None, 1.0))
        target = np.where(cnt > 0, target, 1.0)
        ctx.zero(0)
        ctx.deposit(0, box, pos, masses)
        p, c, _ = ctx.power(0, 0, m, m)
        _, g = loss_grad(p, target, c)
        gpos, gmass, _ = ctx.adjoint(0, box, pos, g, m, masses=masses)
    rpos, rmass, _ = O.reference_gradient(pos, box, dims, nrbins, g, masses, 0.0, m_norm=m)
    grad_close(gpos, rpos)
    grad_close(gmass, rmass)
