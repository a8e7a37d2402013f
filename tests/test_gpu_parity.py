"""GPU parity: the CUDA path through the C ABI against the FP64 oracle and the
reference's golden fixtures.

Tolerances:
  * mode counts: bit-exact; keffs: 1e-12 relative (pure geometry, FP64).
  * P(k): every bin within 1e-5 relative of the FP64 oracle (the stated bar
    for the FP32 deposit + FP32 FFT path).
  * deposited grid: |gpu - oracle| <= 2e-6 * max|oracle| per cell (FP32 CIC
    weights and FP32 accumulation against FP64).
"""
import numpy as np
import pytest

from conftest import cases
from oracle import oracle as O

pytestmark = pytest.mark.gpu

P_RTOL = 1e-5


@pytest.fixture(scope="module")
def gp(native_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    import genpk_gb300
    return genpk_gb300


def grid_close(gpu, ref, tol=2e-6):
    scale = max(np.abs(ref).max(), 1e-30)
    err = np.abs(gpu - ref).max() / scale
    assert err <= tol, f"grid max rel err {err:.3e}"


def bins_close(p_gpu, p_ref, cnt, rtol=P_RTOL):
    ok = cnt > 0
    rel = np.abs(p_gpu[ok] - p_ref[ok]) / np.maximum(np.abs(p_ref[ok]), 1e-300)
    assert rel.max() <= rtol, f"max per-bin rel err {rel.max():.3e} at bin {np.argmax(rel)}"
    assert np.all(p_gpu[~ok] == 0)
    return rel.max()


# ---------------------------------------------------------------------------
# The reference's own known answers (test.cpp) through reference-named calls
# ---------------------------------------------------------------------------

def test_check_fieldize_known_answer(gp):
    """test.cpp:31-50 through the fieldize() drop-in."""
    dims = 5
    field = np.zeros(2 * dims * dims * (dims // 2 + 1))
    pos = (np.arange(30) / 3.0).astype(np.float32)
    masses = np.full(30, 10.0, dtype=np.float32)
    assert gp.fieldize(10, dims, field, pos, masses[:10], 10.0, 1) == 0
    assert abs(field[0] - 8.61111) <= 8.61111e-5
    assert field[3] == 0 and field[20] == 0 and field[125] == 0
    assert abs(field[124] - 1.66666) <= 1.66666e-5


def test_check_powerspectrum_known_answer(gp):
    """test.cpp:59-86 through the powerspectrum() drop-in (FFT by the caller)."""
    field = np.zeros(2 * 4 * 4 * 3)
    for i in range(32):
        field[6 * (i // 4) + i % 4] = 1
    field[0] = 2
    f = O.rfft_padded(field.reshape(4, 4, 6))
    p, c, k = gp.powerspectrum(4, f, f, 10, 64.0, 64.0)
    assert abs(k[2] - np.sqrt(2)) <= np.sqrt(2) * 1e-5
    assert (c[0], c[1], c[2]) == (6, 0, 12)
    assert abs(p[0] - 0.0677526) <= 0.0677526e-5
    assert p[1] == 0
    assert abs(p[2] - 0.000565561) <= 0.000565561e-5
    assert abs(p[9] - 0.0550908) <= 0.0550908e-5


def test_check_powerspectrum_known_answer_gpu_fft(gp):
    """Same field, FFT on the GPU: load it as a density and bin."""
    field = np.zeros((4, 4, 6))
    flat = field.reshape(-1)
    for i in range(32):
        flat[6 * (i // 4) + i % 4] = 1
    flat[0] = 2
    f = O.rfft_padded(field)
    with gp.Context(4, 10) as ctx:
        ctx.load_spectrum(0, f)
        p, c, k = ctx.power(0, 0, 64.0, 64.0)
    assert (c[0], c[1], c[2]) == (6, 0, 12)
    assert abs(p[9] - 0.0550908) <= 0.0550908e-5


# ---------------------------------------------------------------------------
# Golden fixtures from the reference build
# ---------------------------------------------------------------------------

def test_deposit_matches_reference_golden_grids(gp, golden):
    for name, c in cases(golden["fieldize"]).items():
        dims, box, n, extra, mass = c["meta"]
        dims, extra = int(dims), int(extra)
        pos, masses = c["pos"], c.get("masses")
        if extra == 1:
            with gp.Context(dims, 1) as ctx:
                ctx.deposit(0, box, pos, masses, mass)
                g = ctx.read_field(0).reshape(-1)
        else:
            g = np.zeros_like(c["grid"])
            gp.fieldize(box, dims, g, pos, masses, mass, extra)
        grid_close(g, c["grid"])


def test_power_matches_reference_golden(gp, golden):
    for name, c in cases(golden["power"]).items():
        dims, box, n, mass, nrbins, m = c["meta"]
        dims, nrbins = int(dims), int(nrbins)
        with gp.Context(dims, nrbins) as ctx:
            ctx.deposit(0, box, c["pos"], c.get("masses"), mass)
            p, cnt, k = ctx.power(0, 0, m, m)
        assert np.array_equal(cnt, c["count"]), name
        np.testing.assert_allclose(k, c["keffs"], rtol=1e-12, err_msg=name)
        bins_close(p, c["power"], cnt)


# ---------------------------------------------------------------------------
# Oracle comparisons at larger sizes
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("kind,dims,nrbins", [("uniform", 64, 64), ("uniform", 128, 64),
                                              ("zeldovich", 64, 64), ("zeldovich", 128, 128)])
def test_power_matches_oracle(gp, kind, dims, nrbins):
    from genpk_gb300 import synth
    box = 25000.0
    if kind == "uniform":
        pos = synth.uniform(dims ** 3, box, seed=dims)
    else:
        pos = synth.zeldovich(dims, box, seed=dims)
    mass = 1.0e-2
    m = O.total_mass(len(pos), None, mass)
    pr, cr, kr = O.pk(pos, box, dims, nrbins, None, mass, m_norm=m)
    with gp.Context(dims, nrbins) as ctx:
        ctx.deposit(0, box, pos, None, mass)
        p, c, k = ctx.power(0, 0, m, m)
    assert np.array_equal(c, cr)
    assert c.astype(np.int64).sum() == dims ** 3 - 1
    np.testing.assert_allclose(k, kr, rtol=1e-12)
    bins_close(p, pr, c)


def test_variable_masses_lognormal(gp):
    from genpk_gb300 import synth
    dims, box, nrbins = 64, 1000.0, 32
    pos, masses = synth.lognormal(150000, box, 64, sigma=1.5, seed=4, mass_mu=-5, mass_sigma=0.8)
    m = O.total_mass(len(pos), masses)
    pr, cr, _ = O.pk(pos, box, dims, nrbins, masses, 0.0, m_norm=m)
    with gp.Context(dims, nrbins) as ctx:
        ctx.deposit(0, box, pos, masses)
        g = ctx.read_field(0)
        p, c, _ = ctx.power(0, 0, m, m)
    grid_close(g, O.deposit(pos, box, dims, masses, 0.0))
    bins_close(p, pr, c)


@pytest.mark.parametrize("dims", [2, 3, 5, 7, 9, 17, 33, 48])
def test_small_and_odd_grids(gp, dims):
    rng = np.random.default_rng(dims)
    box = 7.0
    pos = (rng.random((3000, 3)) * 9.0 - 1.0).astype(np.float32)  # wraps both ways
    masses = (rng.random(3000) + 0.1).astype(np.float32)
    nrbins = max(3, dims)
    m = O.total_mass(len(pos), masses)
    ref_grid = O.deposit(pos, box, dims, masses, 0.0)
    pr, cr, kr = O.pk(pos, box, dims, nrbins, masses, 0.0, m_norm=m)
    with gp.Context(dims, nrbins) as ctx:
        ctx.deposit(0, box, pos, masses)
        grid_close(ctx.read_field(0), ref_grid)
        p, c, k = ctx.power(0, 0, m, m)
    assert np.array_equal(c, cr)
    bins_close(p, pr, c)  # 1e-5; the largest seen is 2.8e-7


def test_deposit_is_bit_reproducible_across_tiles_and_pointer_kinds(gp):
    """64-bit fixed-point accumulation: the grid does not depend on summation
    order, tile shape or where the particles came from."""
    import torch
    from genpk_gb300 import synth
    dims, box = 96, 1000.0
    pos = synth.uniform(200000, box, seed=7)
    masses = np.linspace(0.2, 3.0, len(pos)).astype(np.float32)
    ref = O.deposit(pos, box, dims, masses, 0.0)
    grids = []
    for tile in [(8, 8, 8), (16, 16, 8), (16, 16, 16)]:
        with gp.Context(dims, 16) as ctx:
            ctx.set_engine(gp.api.ENGINE_SORTED)
            ctx.set_tile(*tile)
            ctx.deposit(0, box, pos, masses)
            grids.append(ctx.read_field(0))
            ctx.zero(0)
            ctx.deposit(0, box, torch.from_numpy(pos).cuda(), torch.from_numpy(masses).cuda())
            grids.append(ctx.read_field(0))
    grid_close(grids[0], ref)
    for g in grids[1:]:
        assert np.array_equal(g, grids[0])


CHUNKED = {"window": 2, "stream": 3}  # api.ENGINE_WINDOW, api.ENGINE_STREAM


@pytest.mark.parametrize("engine", ["window", "stream"])
@pytest.mark.parametrize("var", [False, True])
def test_window_engine_matches_oracle(gp, var, engine):
    """Lattice-ordered particles through the window engine (shared windows
    per chunk, no sort) and its stream mode (neighbour-merged reductions)."""
    from genpk_gb300 import synth
    dims, box, nrbins = 128, 25000.0, 64
    pos = synth.zeldovich(128, box, seed=3)
    masses = np.linspace(0.5, 1.5, len(pos)).astype(np.float32) if var else None
    mass = 0.0 if var else 1.0e-2
    m = O.total_mass(len(pos), masses, mass)
    ref = O.deposit(pos, box, dims, masses, mass)
    pr, cr, _ = O.pk(pos, box, dims, nrbins, masses, mass, m_norm=m)
    with gp.Context(dims, nrbins) as ctx:
        ctx.set_engine(CHUNKED[engine])
        ctx.deposit(0, box, pos, masses, mass)
        ctx.sync()
        assert ctx.last_engine == CHUNKED[engine]
        grid_close(ctx.read_field(0), ref, tol=1e-6)
        p, c, _ = ctx.power(0, 0, m, m)
    assert np.array_equal(c, cr)
    bins_close(p, pr, c)


@pytest.mark.parametrize("engine", ["window", "stream"])
@pytest.mark.parametrize("case", ["unaligned_tail", "dense_carry", "negative_mass_carry",
                                  "tiny_grid", "grid_8"])
def test_window_engine_edge_cases(gp, case, engine):
    """Window-engine paths the lattice case does not reach: an input pointer
    that is not 16-byte aligned (chunks copied by threads, not bulk copies) with
    a partial last chunk; window cells whose 32-bit fixed-point sum overflows
    (carried to the grid), for positive and negative masses; grids so small
    that every axis is taken whole with the wrapped extra layer."""
    import torch
    from genpk_gb300 import synth
    rng = np.random.default_rng(11)
    masses, mass = None, 1.0
    if case == "unaligned_tail":
        dims, box = 64, 1000.0
        full = synth.zeldovich(64, box, seed=12)[: 3 * 4096 + 1235]
        pos = full[1:]
        dev = torch.from_numpy(full).cuda()[1:]
        assert dev.data_ptr() % 16 != 0
    elif case in ("dense_carry", "negative_mass_carry"):
        dims, box = 16, 16.0
        lat = synth.zeldovich(16, box, seed=13)
        clump = (np.array([3.0, 4.0, 5.0]) + rng.random((9000, 3)) * 0.5).astype(np.float32)
        pos = np.concatenate([lat, clump, lat]).astype(np.float32)
        if case == "negative_mass_carry":
            masses = rng.uniform(-1.0, 1.0, len(pos)).astype(np.float32)
            masses[len(lat): len(lat) + 9000] = -rng.uniform(0.5, 1.0, 9000)
            mass = 0.0
        dev = torch.from_numpy(pos).cuda()
    else:
        dims = 6 if case == "tiny_grid" else 8
        box = 3.0
        pos = (rng.random((50000, 3)) * box).astype(np.float32)
        pos = pos[np.lexsort((pos[:, 2], pos[:, 1], pos[:, 0]))]
        dev = torch.from_numpy(pos).cuda()
    ref = O.deposit(pos, box, dims, masses, mass)
    with gp.Context(dims, 8) as ctx:
        ctx.set_engine(CHUNKED[engine])
        ctx.deposit(0, box, dev, None if masses is None else torch.from_numpy(masses).cuda(), mass)
        ctx.sync()
        assert ctx.last_engine == CHUNKED[engine]
        grid_close(ctx.read_field(0), ref, tol=1e-6)


@pytest.mark.parametrize("var", [False, True])
def test_pinned_host_input_read_in_place(gp, var):
    """Large pinned host arrays are read in place by the window engine (no
    staging copy); the sorted engine gets them copied once.  Same grids as
    from device memory."""
    import torch
    from genpk_gb300 import synth
    dims, box = 128, 1000.0
    pos = synth.zeldovich(128, box, seed=15)
    hpos = torch.from_numpy(pos).pin_memory()
    masses = hmass = None
    mass = 1.0
    if var:
        masses = np.linspace(0.5, 1.5, len(pos)).astype(np.float32)
        hmass = torch.from_numpy(masses).pin_memory()
        mass = 0.0
    dpos = hpos.cuda()
    dmass = hmass.cuda() if var else None
    with gp.Context(dims, 16) as ctx:
        out = {}
        for eng in (gp.api.ENGINE_WINDOW, gp.api.ENGINE_STREAM, gp.api.ENGINE_SORTED):
            ctx.set_engine(eng)
            for name, p_, m_ in (("dev", dpos, dmass), ("pinned", hpos, hmass)):
                ctx.zero(0)
                ctx.deposit(0, box, p_, m_, mass)
                ctx.sync()
                assert ctx.last_engine == eng
                out[(eng, name)] = ctx.read_field(0)
    for eng in (gp.api.ENGINE_WINDOW, gp.api.ENGINE_STREAM, gp.api.ENGINE_SORTED):
        assert np.array_equal(out[(eng, "pinned")], out[(eng, "dev")])
        assert np.array_equal(out[(eng, "pinned")], out[(gp.api.ENGINE_SORTED, "dev")])
    grid_close(out[(gp.api.ENGINE_WINDOW, "pinned")], O.deposit(pos, box, dims, masses, mass),
               tol=1e-6)


@pytest.mark.parametrize("engine", ["window", "stream"])
def test_window_engine_reports_non_finite(gp, engine):
    from genpk_gb300 import synth
    dims, box = 32, 100.0
    pos = synth.zeldovich(32, box, seed=14)
    bad = pos.copy()
    bad[5, 2] = np.nan
    bad[9000, 0] = -np.inf
    keep = np.ones(len(pos), bool)
    keep[[5, 9000]] = False
    with gp.Context(dims, 8) as ctx:
        ctx.set_engine(CHUNKED[engine])
        ctx.deposit(0, box, bad, None, 1.0)
        with pytest.raises(gp.GenPKError) as e:
            ctx.sync()
        assert e.value.status == 5
        g = ctx.read_field(0)
    grid_close(g, O.deposit(pos[keep], box, dims, None, 1.0), tol=1e-6)


@pytest.mark.parametrize("engine", ["window", "stream"])
def test_window_engine_direct_fallback_on_random_order(gp, engine):
    """Randomly ordered particles: no chunk fits a window (every corner takes a
    global reduction), no neighbours merge.  Still correct."""
    from genpk_gb300 import synth
    dims, box, nrbins = 64, 1000.0, 32
    pos = synth.uniform(300000, box, seed=4)
    m = O.total_mass(len(pos), None, 1.0)
    pr, cr, _ = O.pk(pos, box, dims, nrbins, None, 1.0, m_norm=m)
    with gp.Context(dims, nrbins) as ctx:
        ctx.set_engine(CHUNKED[engine])
        ctx.deposit(0, box, pos, None, 1.0)
        grid_close(ctx.read_field(0), O.deposit(pos, box, dims, None, 1.0), tol=1e-6)
        p, c, _ = ctx.power(0, 0, m, m)
    bins_close(p, pr, c)


def test_auto_engine_choice(gp):
    """A lattice at one particle per cell (consecutive particles one z cell
    apart): stream mode; at eight per cell: windows; random order: the
    autotuner's faster of the sorted and the stream engine; a pass too small
    to judge or tune: sorted."""
    from genpk_gb300 import synth
    box = 1000.0
    lattice = synth.zeldovich(128, box, seed=5)              # 2^21 particles, coherent
    rand = synth.uniform(len(lattice), box, seed=6)           # same count, random order
    with gp.Context(128, 16) as ctx:
        ctx.deposit(0, box, lattice, None, 1.0)
        ctx.sync()
        assert ctx.last_engine == gp.api.ENGINE_STREAM
    with gp.Context(64, 16) as ctx:
        ctx.deposit(0, box, lattice, None, 1.0)
        ctx.sync()
        assert ctx.last_engine == gp.api.ENGINE_WINDOW
    with gp.Context(128, 16) as ctx:
        ctx.zero(0)
        ctx.deposit(0, box, rand, None, 1.0)
        ctx.sync()
        best = min(ctx.deposit_trials(), key=lambda r: r[2])
        assert ctx.last_engine == (gp.api.ENGINE_STREAM if best[0] == (0, 0, 0)
                                   else gp.api.ENGINE_SORTED)
        ctx.zero(0)
        ctx.deposit(0, box, lattice[:1000], None, 1.0)       # small pass: sorted
        ctx.sync()
        assert ctx.last_engine == gp.api.ENGINE_SORTED


def test_engine_choice_is_kept_for_the_same_arrays(gp):
    """Device arrays deposited again take their previous automatic choice (no
    probe, no host round trip; a few arrays are remembered, one per species of
    a multi-species loop); new arrays are probed."""
    import torch
    from genpk_gb300 import synth
    box = 1000.0
    lattice = torch.from_numpy(synth.zeldovich(128, box, seed=5)).cuda()
    rand = torch.from_numpy(synth.uniform(len(lattice), box, seed=6)).cuda()
    with gp.Context(128, 16, timing=True) as ctx:
        got = []
        for src in (lattice, rand, rand, lattice):
            ctx.timing_reset()
            ctx.zero(0)
            ctx.deposit(0, box, src, None, 1.0)
            ctx.sync()
            got.append((ctx.last_engine, "probe" in ctx.stage_times()))
        best = min(ctx.deposit_trials(), key=lambda r: r[2])  # random order: tuned
    S = gp.api.ENGINE_STREAM
    R = S if best[0] == (0, 0, 0) else gp.api.ENGINE_SORTED
    assert got == [(S, True), (R, True), (R, False), (S, False)]


def test_sparse_lattice_picks_a_shorter_window_chunk(gp):
    """128^3 lattice particles on a 256^3 grid (two cells per lattice
    spacing): a 4096-particle chunk's window does not fit, a 1024-particle
    chunk's does, so the automatic choice is still the window engine."""
    from genpk_gb300 import synth
    dims, box = 256, 1000.0
    pos = synth.zeldovich(128, box, seed=17)
    with gp.Context(dims, 16) as ctx:
        ctx.deposit(0, box, pos, None, 1.0)
        ctx.sync()
        assert ctx.last_engine == gp.api.ENGINE_WINDOW
        grid_close(ctx.read_field(0), O.deposit(pos, box, dims, None, 1.0), tol=1e-6)


@pytest.mark.parametrize("var", [False, True])
def test_window_and_sorted_engines_agree_bit_for_bit(gp, var):
    """All engines add the same integer CIC weights (28-bit fractions from the
    exact split) exactly and round each cell once: identical grids, also when
    a grid accumulates two passes."""
    import torch
    from genpk_gb300 import synth
    dims, box = 96, 1000.0
    pos = torch.from_numpy(synth.zeldovich(96, box, seed=7)).cuda()
    masses = (torch.linspace(0.3, 2.0, len(pos)) if var else torch.ones(len(pos))).cuda()
    with gp.Context(dims, 16) as ctx:
        grids = []
        for eng in (gp.api.ENGINE_SORTED, gp.api.ENGINE_WINDOW, gp.api.ENGINE_STREAM):
            ctx.set_engine(eng)
            ctx.zero(0)
            if var:
                ctx.deposit(0, box, pos[:400000], masses[:400000])
                ctx.deposit(0, box, pos[400000:], masses[400000:])
            else:
                ctx.deposit(0, box, pos[:400000], None, 1.0)
                ctx.deposit(0, box, pos[400000:], None, 1.0)
            ctx.sync()
            assert ctx.last_engine == eng
            grids.append(ctx.read_field(0))
    assert np.array_equal(grids[0], grids[1])
    assert np.array_equal(grids[0], grids[2])


_WIDE_CHECK = """
import sys, numpy as np, torch
sys.path.insert(0, {root!r})
import genpk_gb300 as gp
from genpk_gb300 import synth
box = 1000.0
pos = torch.from_numpy(synth.zeldovich(64, box, seed=21)).cuda()
masses = torch.linspace(-0.5, 1.5, len(pos)).cuda()
grids = []
with gp.Context(64, 8) as ctx:
    for eng, m in ((gp.api.ENGINE_SORTED, None), (gp.api.ENGINE_STREAM, None),
                   (gp.api.ENGINE_SORTED, masses), (gp.api.ENGINE_STREAM, masses)):
        ctx.set_engine(eng)
        ctx.zero(0)
        ctx.deposit(0, box, pos, m, 1.0)
        ctx.sync()
        grids.append(ctx.read_field(0))
assert np.array_equal(grids[0], grids[1]) and np.array_equal(grids[2], grids[3])
print("wide ok")
"""


def test_stream_mode_64bit_indices(gp):
    """The stream kernel's 64-bit element-index variant (chosen for grids of 2^32 or more
    elements, N >= 1626) forced on a 64^3 grid through the GENPK_WIDE_INDEX=1 hook, in a
    child process (the hook is read once): the same grids as the sorted engine, uniform and
    signed variable masses."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _WIDE_CHECK.format(root=root)],
                       env={**os.environ, "GENPK_WIDE_INDEX": "1"}, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0 and "wide ok" in r.stdout, r.stdout + r.stderr


@pytest.mark.parametrize("engine", ["sorted", "window", "stream"])
def test_faint_high_k_bins_of_a_smooth_lattice(gp, engine):
    """128^3 Zel'dovich lattice (the GPU generator, L = 25000, 64 bins): the
    highest-k bins hold ~1e-10 of the peak power and are sensitive to the
    fraction precision (28-bit fractions from the exact split) and to any
    rounding of partial cell sums; every bin within 1e-5 of the FP64 oracle."""
    from genpk_gb300 import synth
    n, box, nrb = 128, 25000.0, 64
    dpos = synth.zeldovich(n, box, seed=1, device="cuda")
    pos = dpos.cpu().numpy()
    m = O.total_mass(len(pos), None, 1.0)
    pr, cr, _ = O.pk(pos, box, n, nrb, None, 1.0, m_norm=m)
    with gp.Context(n, nrb) as ctx:
        ctx.set_engine({"sorted": 1, "window": 2, "stream": 3}[engine])
        ctx.deposit(0, box, dpos, None, 1.0)
        p, c, _ = ctx.power(0, 0, m, m)
    assert np.array_equal(c, cr)
    bins_close(p, pr, c)


def test_global_counter_sort_mode(gp):
    """More tiles than a shared histogram holds (8^3 tiles on 288^3: 46656
    tiles) switches the sort to warp-aggregated global counters."""
    from genpk_gb300 import synth
    dims, box, nrbins = 288, 1000.0, 32
    pos = synth.uniform(400000, box, seed=8)
    ref = O.deposit(pos, box, dims, None, 1.0)
    m = O.total_mass(len(pos), None, 1.0)
    with gp.Context(dims, nrbins) as ctx:
        ctx.set_engine(gp.api.ENGINE_SORTED)
        ctx.set_tile(8, 8, 8)
        ctx.deposit(0, box, pos, None, 1.0)
        g8 = ctx.read_field(0)
        ctx.zero(0)
        ctx.set_tile(16, 16, 16)
        ctx.deposit(0, box, pos, None, 1.0)
        g16 = ctx.read_field(0)
        p, c, _ = ctx.power(0, 0, m, m)
    grid_close(g8, ref)
    assert np.array_equal(g8, g16)
    pr, cr, _ = O.pk(pos, box, dims, nrbins, None, 1.0, m_norm=m)
    bins_close(p, pr, c)


def test_dense_cells_accumulate_exactly(gp):
    """Thousands of particles per cell: 64-bit integer sums lose nothing."""
    rng = np.random.default_rng(3)
    dims, box = 4, 4.0
    pos = (rng.random((200000, 3)) * box).astype(np.float32)
    ref = O.deposit(pos, box, dims, None, 1.0)
    with gp.Context(dims, 4) as ctx:
        ctx.deposit(0, box, pos, None, 1.0)
        g = ctx.read_field(0)
    grid_close(g, ref, tol=1e-7)


# ---------------------------------------------------------------------------
# Accumulation semantics, pointer kinds, cross spectra
# ---------------------------------------------------------------------------

def test_chunked_host_and_device_deposits_accumulate(gp):
    import torch
    from genpk_gb300 import synth
    dims, box = 64, 500.0
    pos = synth.uniform(300000, box, seed=9)
    masses = np.linspace(0.5, 1.5, len(pos)).astype(np.float32)
    ref = O.deposit(pos, box, dims, masses, 0.0)
    with gp.Context(dims, 8) as ctx:
        # host chunks like read_fieldize's <= 2^26 loop (read_fieldize.cpp:45-93)
        for a in range(0, len(pos), 70000):
            ctx.deposit(0, box, pos[a:a + 70000], masses[a:a + 70000])
        grid_close(ctx.read_field(0), ref)
        ctx.zero(0)
        dpos = torch.from_numpy(pos).cuda()
        dm = torch.from_numpy(masses).cuda()
        ctx.deposit(0, box, dpos[:100000], dm[:100000])
        ctx.deposit(0, box, pos[100000:200000], masses[100000:200000])  # host
        ctx.deposit(0, box, dpos[200000:], masses[200000:])             # mixed kinds
        grid_close(ctx.read_field(0), ref)


def test_uniform_and_variable_mass_chunks_into_one_grid(gp):
    """Gas + stars into one grid (gen-pk.cpp:215-230 with -s 1)."""
    from genpk_gb300 import synth
    dims, box = 32, 100.0
    gas = synth.uniform(20000, box, seed=1)
    stars = synth.uniform(3000, box, seed=2)
    sm = np.full(3000, 0.37, dtype=np.float32)
    ref = O.deposit(gas, box, dims, None, 0.19)
    O.port().fieldize(box, dims, ref, stars, sm, 0.0, 1)
    with gp.Context(dims, 8) as ctx:
        ctx.deposit(0, box, gas, None, 0.19)
        ctx.deposit(0, box, stars, sm)
        grid_close(ctx.read_field(0), ref)


@pytest.mark.parametrize("dims", [64, 128, 256, 512])
def test_fft_paths_agree(gp, dims):
    """The fused path (2-D cuFFT over x-planes, own x-axis pass binning the
    auto spectrum in the same read) against 3-D cuFFT + the binning kernel:
    the same spectrum is left in the grid (a cross spectrum of two copies
    binned from it equals the fused auto spectrum) and the bins agree."""
    from genpk_gb300 import synth
    box, nrbins = 1000.0, 48
    pos = synth.zeldovich(min(dims, 128), box, seed=21)
    m = O.total_mass(len(pos), None, 1.0)
    out = {}
    with gp.Context(dims, nrbins, nfields=2) as ctx:
        for mode in (gp.api.FFT_AUTO, gp.api.FFT_CUFFT3D):
            ctx.set_fft_mode(mode)
            for f in (0, 1):
                ctx.zero(f)
                ctx.set_engine(gp.api.ENGINE_SORTED)
                ctx.deposit(f, box, pos, None, 1.0)
            p, c, _ = ctx.power(0, 0, m, m)      # fused when mode is AUTO
            x, _, _ = ctx.power(0, 1, m, m)      # from the stored spectra
            out[mode] = (p, c, x)
    pa, ca, xa = out[gp.api.FFT_AUTO]
    p3, c3, x3 = out[gp.api.FFT_CUFFT3D]
    assert np.array_equal(ca, c3)
    # two FP32 transforms: their difference is FP32 rounding, well inside the
    # 1e-5 bar each meets against the FP64 oracle
    bins_close(pa, p3, ca, rtol=1e-5)
    bins_close(xa, pa, ca, rtol=2e-6)
    bins_close(x3, p3, ca, rtol=1e-6)
    if dims <= 256:
        pr, cr, _ = O.pk(pos, box, dims, nrbins, None, 1.0, m_norm=m)
        bins_close(pa, pr, cr)


@pytest.mark.parametrize("engine", ["window", "stream"])
def test_accumulator_cleared_by_the_transform(gp, engine):
    """The own x pass clears the window engine's 64-bit accumulator once its
    pass has been used (read by the z pass, or converted), and the next window
    pass skips its own clear.  Spectra through one reused context equal those
    of fresh contexts bit for bit: single-field steps, two fields per step (one
    converted and batched through the 2-D transform), and a += pass whose
    accumulator was cleared by the x pass of another field's spectrum."""
    from genpk_gb300 import synth
    dims, box, nrbins = 128, 1000.0, 32
    eng = {"window": gp.api.ENGINE_WINDOW, "stream": gp.api.ENGINE_STREAM}[engine]
    boxes = [synth.zeldovich(128, box, seed=s) for s in (31, 32, 33)]
    m = O.total_mass(len(boxes[0]), None, 1.0)
    pairs, pm = [(0, 0), (1, 1), (0, 1)], [(m, m)] * 3

    def fresh(steps):
        with gp.Context(dims, nrbins, nfields=2) as c:
            c.set_engine(eng)
            return steps(c)

    def single(pos):
        def steps(c):
            c.zero(0)
            c.deposit(0, box, pos, None, 1.0)
            return c.power(0, 0, m, m)
        return steps

    def double(pa, pb):
        def steps(c):
            c.zero(0)
            c.zero(1)
            c.deposit(0, box, pa, None, 1.0)
            c.deposit(1, box, pb, None, 1.0)
            return c.power_multi(pairs, pm)
        return steps

    def same(a, b):
        for x, y in zip(a, b):
            assert np.array_equal(np.asarray(x), np.asarray(y))

    with gp.Context(dims, nrbins, nfields=2) as ctx:
        ctx.set_engine(eng)
        for pos in boxes:
            same(single(pos)(ctx), fresh(single(pos)))
        for pa, pb in ((boxes[0], boxes[1]), (boxes[2], boxes[0])):
            same(double(pa, pb)(ctx), fresh(double(pa, pb)))
        same(single(boxes[1])(ctx), fresh(single(boxes[1])))
        # field 0 pending, field 1's spectrum converts it and clears the
        # accumulator; the += pass into field 0 then starts from that clear
        ctx.zero(0)
        ctx.zero(1)
        ctx.deposit(1, box, boxes[2], None, 1.0)
        ctx.deposit(0, box, boxes[0], None, 1.0)
        ctx.power(1, 1, m, m)
        ctx.deposit(0, box, boxes[1], None, 1.0)
        got = ctx.power(0, 0, 2 * m, 2 * m)

    def twice(c):
        # two passes, as above (without the sync the two staged host deposits
        # would merge into one pass, rounded to FP32 once instead of twice)
        c.zero(0)
        c.deposit(0, box, boxes[0], None, 1.0)
        c.sync()
        c.deposit(0, box, boxes[1], None, 1.0)
        return c.power(0, 0, 2 * m, 2 * m)
    same(got, fresh(twice))
    pr, cr, _ = O.pk(np.concatenate([boxes[0], boxes[1]]), box, dims, nrbins, None, 1.0,
                     m_norm=2 * m)
    bins_close(got[0], pr, cr)


def test_sorted_engine_autotuner(gp):
    """The sorted engine's first clean pass of a density band tries every
    tile and sort-CTA candidate, keeps the fastest, and the grid equals the
    one a fixed tile gives, bit for bit; the next pass of that band reuses the
    choice (no new trials); fixing a tile turns the tuner off."""
    from genpk_gb300 import synth
    dims, box = 128, 1000.0
    pos = synth.uniform(2_000_000, box, seed=31)
    with gp.Context(dims, 16) as ctx:
        ctx.set_engine(gp.api.ENGINE_SORTED)
        ctx.deposit(0, box, pos, None, 1.0)
        tuned = ctx.read_field(0)
        trials = ctx.deposit_trials()
        assert len(trials) >= 3 and all(ms > 0 for _, _, ms in trials)
        assert {t for t, _, _ in trials} == {(8, 8, 8), (16, 16, 8), (16, 16, 16)}
        best = min(trials, key=lambda r: r[2])
        cfg = ctx.deposit_config()
        assert cfg["tile"] == best[0] and cfg["sort_ctas"] == best[1]
        ctx.zero(0)
        ctx.deposit(0, box, pos[:1_900_000], None, 1.0)  # the same band: no new tuning
        ctx.read_field(0)
        assert ctx.deposit_trials() == trials
        for tile in ((16, 16, 16), (8, 8, 8)):
            ctx.set_tile(*tile)
            ctx.zero(0)
            ctx.deposit(0, box, pos, None, 1.0)
            assert np.array_equal(ctx.read_field(0), tuned)
            assert ctx.deposit_config()["tile"] == tile
    grid_close(tuned, O.deposit(pos, box, dims, None, 1.0))


def test_autotuner_chooses_between_sorted_and_stream_engines(gp):
    """Uniform random particles (no spatial coherence) with the automatic
    engine: the first clean pass of a density band also times the stream
    engine (reported as tile 0x0x0), the faster engine is kept for the band,
    and the grid equals the sorted engine's bit for bit whichever won."""
    from genpk_gb300 import synth
    dims, box = 128, 1000.0
    pos = synth.uniform(1_000_000, box, seed=33)
    with gp.Context(dims, 16) as ctx:
        ctx.deposit(0, box, pos, None, 1.0)
        auto_grid = ctx.read_field(0)
        trials = ctx.deposit_trials()
        assert ((0, 0, 0), 0) in [(t, c) for t, c, _ in trials]
        best = min(trials, key=lambda r: r[2])
        want = gp.api.ENGINE_STREAM if best[0] == (0, 0, 0) else gp.api.ENGINE_SORTED
        assert ctx.last_engine == want
        ctx.zero(0)
        ctx.deposit(0, box, pos[:950_000], None, 1.0)  # the same band: the kept choice
        ctx.read_field(0)
        assert ctx.last_engine == want and ctx.deposit_trials() == trials
    with gp.Context(dims, 16) as ctx:
        ctx.set_engine(gp.api.ENGINE_SORTED)
        ctx.deposit(0, box, pos, None, 1.0)
        assert np.array_equal(ctx.read_field(0), auto_grid)


@pytest.mark.parametrize("engine", ["sorted", "window", "stream"])
def test_deposit_conserves_mass(gp, engine):
    """The grid's real cells sum to the deposited mass in every engine
    (variable masses, two passes into one field, positions outside the box)."""
    from genpk_gb300 import synth
    rng = np.random.default_rng(12)
    box, dims = 1000.0, 128
    lat = synth.zeldovich(128, box, seed=12)
    out = rng.uniform(-2 * box, 3 * box, (len(lat), 3)).astype(np.float32)
    m1 = rng.lognormal(0.0, 0.5, len(lat)).astype(np.float32)
    m2 = rng.lognormal(-1.0, 0.5, len(lat)).astype(np.float32)
    eng = {"sorted": gp.api.ENGINE_SORTED, "window": gp.api.ENGINE_WINDOW,
           "stream": gp.api.ENGINE_STREAM}[engine]
    with gp.Context(dims, 16) as ctx:
        ctx.set_engine(eng)
        ctx.deposit(0, box, lat, m1)
        ctx.sync()
        ctx.deposit(0, box, out, m2)
        g = ctx.read_field(0)
    total = m1.astype(np.float64).sum() + m2.astype(np.float64).sum()
    assert abs(g[:, :, :dims].sum() - total) <= 1e-6 * total


def test_contexts_on_concurrent_host_threads(gp):
    """Contexts used from several host threads at once (one stream each), with
    different grid sizes, so that kernels with size-dependent shared memory
    launch concurrently: every spectrum equals the same context's result run
    alone, bit for bit."""
    import threading
    import torch
    from genpk_gb300 import synth
    box, nrbins = 1000.0, 24
    jobs = [(64, torch.from_numpy(synth.uniform(300_000, box, seed=40)).cuda()),
            (128, torch.from_numpy(synth.uniform(1_500_000, box, seed=41)).cuda()),
            (128, torch.from_numpy(synth.zeldovich(128, box, seed=42)).cuda()),
            (256, torch.from_numpy(synth.zeldovich(128, box, seed=43)).cuda()),
            (64, torch.from_numpy(synth.zeldovich(64, box, seed=44)).cuda()),
            (256, torch.from_numpy(synth.uniform(2_000_000, box, seed=45)).cuda())]

    def run(ctx, pos, reps, out, i):
        m = O.total_mass(len(pos), None, 1.0)
        for _ in range(reps):
            ctx.zero(0)
            ctx.deposit(0, box, pos, None, 1.0)
            out[i] = ctx.power(0, 0, m, m)

    ctxs = [gp.Context(n, nrbins) for n, _ in jobs]
    try:
        alone = [None] * len(jobs)
        for i, (c, (_, pos)) in enumerate(zip(ctxs, jobs)):
            run(c, pos, 1, alone, i)
        together = [None] * len(jobs)
        ths = [threading.Thread(target=run, args=(c, pos, 5, together, i))
               for i, (c, (_, pos)) in enumerate(zip(ctxs, jobs))]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
    finally:
        for c in ctxs:
            c.close()
    for a, b in zip(alone, together):
        assert b is not None
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_cross_and_multi_spectra(gp):
    from genpk_gb300 import synth
    dims, box, nrbins = 64, 1000.0, 24
    a = synth.zeldovich(64, box, seed=1)
    b = synth.zeldovich(64, box, seed=1, amplitude=0.7)
    c = synth.uniform(100000, box, seed=3)
    cm = np.linspace(0.1, 2.0, len(c)).astype(np.float32)
    ma, mb, mc = O.total_mass(len(a), None, 1.0), O.total_mass(len(b), None, 0.19), O.total_mass(len(c), cm)
    fa = O.rfft_padded(O.deposit(a, box, dims, None, 1.0))
    fb = O.rfft_padded(O.deposit(b, box, dims, None, 0.19))
    fc = O.rfft_padded(O.deposit(c, box, dims, cm, 0.0))
    port = O.port()
    refs = {(0, 0): port.powerspectrum(dims, fa, fa, nrbins, ma, ma),
            (1, 1): port.powerspectrum(dims, fb, fb, nrbins, mb, mb),
            (2, 2): port.powerspectrum(dims, fc, fc, nrbins, mc, mc),
            (0, 1): port.powerspectrum(dims, fa, fb, nrbins, ma, mb),
            (0, 2): port.powerspectrum(dims, fa, fc, nrbins, ma, mc),
            (1, 2): port.powerspectrum(dims, fb, fc, nrbins, mb, mc)}
    mass = {0: ma, 1: mb, 2: mc}
    with gp.Context(dims, nrbins, nfields=3) as ctx:
        ctx.deposit(0, box, a, None, 1.0)
        ctx.deposit(1, box, b, None, 0.19)
        ctx.deposit(2, box, c, cm)
        pairs = list(refs)
        p, cnt, _ = ctx.power_multi(pairs, [(mass[i], mass[j]) for i, j in pairs])
        for q, pr in enumerate(pairs):
            ok = cnt > 0
            ref = refs[pr][0]
            auto = pr[0] == pr[1]
            rel = np.abs(p[q][ok] - ref[ok]) / np.abs(ref[ok]).max()
            # cross spectra can cross zero: compare relative to the bin scale
            assert rel.max() <= (P_RTOL if auto else 1e-5), (pr, rel.max())
        # a single cross call after the FFTs are done re-bins without new FFTs; the
        # launch shape differs, so FP32 partial sums group differently (~1e-8)
        p01, _, _ = ctx.power(0, 1, ma, mb)
        np.testing.assert_allclose(p01, p[pairs.index((0, 1))], rtol=1e-6)


def test_compat_bound_fields_route_to_device(gp):
    """The fieldize/powerspectrum drop-ins on a bound host field: the reader's
    chunked fieldize calls and the driver's powerspectrum call, unchanged,
    reach the device grid of the context the field is bound to."""
    from genpk_gb300 import native, synth
    compat = native.load_compat()
    dims, box, nrbins = 32, 100.0, 16
    pos = synth.uniform(30000, box, seed=5)
    host_field = np.zeros(2 * dims * dims * (dims // 2 + 1))
    with gp.Context(dims, nrbins) as ctx:
        assert compat.genpk_compat_bind(ctx.h, 0, host_field.ctypes.data) == 0
        for a in range(0, len(pos), 10000):
            chunk = np.ascontiguousarray(pos[a:a + 10000])
            rc = compat.fieldize(box, dims, host_field.ctypes.data_as(native.c_f64p), len(chunk),
                                 chunk.ctypes.data_as(native.c_f32p), None, 1.0, 1)
            assert rc == 0
        assert not host_field.any()  # host array untouched: the grid lives on the GPU
        m = O.total_mass(len(pos), None, 1.0)
        p = np.zeros(nrbins)
        c = np.zeros(nrbins, dtype=np.int32)
        k = np.zeros(nrbins)
        fp = host_field.ctypes.data_as(native.c_f64p)
        rc = compat.powerspectrum(dims, fp, fp, nrbins, p.ctypes.data_as(native.c_f64p),
                                  c.ctypes.data_as(native.c_i32p), k.ctypes.data_as(native.c_f64p),
                                  m, m)
        assert rc == 0
        assert compat.genpk_compat_unbind(host_field.ctypes.data) == 0
    pr, cr, _ = O.pk(pos, box, dims, nrbins, None, 1.0, m_norm=m)
    assert np.array_equal(c, cr)
    bins_close(p, pr, c)


# ---------------------------------------------------------------------------
# Errors are statuses, never aborts
# ---------------------------------------------------------------------------

def test_non_finite_particles_are_reported_and_skipped(gp):
    dims, box = 16, 10.0
    rng = np.random.default_rng(1)
    pos = (rng.random((1000, 3)) * box).astype(np.float32)
    bad = pos.copy()
    bad[10, 1] = np.nan
    bad[20, 0] = np.inf
    with gp.Context(dims, 4) as ctx:
        ctx.deposit(0, box, bad, None, 1.0)
        with pytest.raises(gp.GenPKError) as e:
            ctx.read_field(0)
        assert e.value.status == 5
        ctx.zero(0)
        ctx.deposit(0, box, bad, None, 1.0)
        with pytest.raises(gp.GenPKError):
            ctx.sync()
        g = ctx.read_field(0)  # status was cleared; skipped particles are absent
    keep = np.ones(1000, bool)
    keep[[10, 20]] = False
    grid_close(g, O.deposit(pos[keep], box, dims, None, 1.0))


def test_state_and_argument_errors(gp):
    with gp.Context(8, 4, nfields=2) as ctx:
        pos = np.zeros((10, 3), np.float32)
        with pytest.raises(gp.GenPKError) as e:
            ctx.deposit(5, 1.0, pos)
        assert e.value.status == 1
        with pytest.raises(gp.GenPKError):
            ctx.deposit(0, -1.0, pos)
        ctx.deposit(0, 1.0, pos, None, 1.0)
        ctx.power(0, 0, 11.0, 11.0)
        with pytest.raises(gp.GenPKError) as e:
            ctx.deposit(0, 1.0, pos, None, 1.0)  # grid holds a spectrum now
        assert e.value.status == 6
        with pytest.raises(gp.GenPKError):
            ctx.read_field(0)
        ctx.zero(0)
        ctx.deposit(0, 1.0, pos, None, 1.0)
        p, c, _ = ctx.power(1, 1, 1.0, 1.0)  # never-deposited grid: all zero
        assert not p.any()
        with pytest.raises(gp.GenPKError):
            ctx.set_tile(7, 7, 7)


def test_empty_inputs(gp):
    """Empty particle arrays (host and device): a grid that receives none has
    a zero spectrum with the full mode counts; a batch with an empty box gives
    zeros for it and the other box's spectrum unchanged, through the eager,
    captured and replayed calls; a species step with an empty species gives
    zero auto and cross spectra for it."""
    import torch
    from genpk_gb300 import synth
    box, nrbins, n = 1000.0, 16, 100_000
    empty_h = np.zeros((0, 3), np.float32)
    empty_d = torch.zeros((0, 3), dtype=torch.float32, device="cuda")
    hp = synth.uniform(n, box, seed=5)
    full = torch.from_numpy(hp).cuda()
    m = O.total_mass(n, None, 1.0)
    pr, cr, _ = O.pk(hp, box, 32, nrbins, None, 1.0, m_norm=m)
    with gp.Context(32, nrbins) as ctx:
        ctx.deposit(0, box, empty_h, None, 1.0)
        ctx.deposit(0, box, empty_d, None, 1.0)
        p, c, _ = ctx.power(0, 0, 1.0, 1.0)
    assert not p.any() and np.array_equal(c, cr)
    with gp.Context(32, nrbins) as ctx:
        ctx.deposit(0, box, full, None, 1.0)
        alone, _, _ = ctx.power(0, 0, m, m)
    with gp.Batch([32, 32], nrbins) as b:
        for _ in range(3):  # eager, captured and replayed, replayed
            pw, cw, _ = b.power(box, [empty_d, full], [1.0, m], mass=1.0)
            assert not pw[0].any() and np.array_equal(pw[1], alone)
            assert np.array_equal(cw[0], cr) and np.array_equal(cw[1], cr)
    with gp.Context(32, nrbins, nfields=2) as ctx:
        ps, cs, _ = ctx.power_step(box, [full, empty_d], [(0, 0), (1, 1), (0, 1)],
                                   [(m, m), (1.0, 1.0), (m, 1.0)], mass=[1.0, 1.0])
    assert not ps[1].any() and not ps[2].any() and np.array_equal(cs, cr)
    bins_close(ps[0], pr, cr)


def test_negative_uniform_mass_every_engine(gp):
    """A negative uniform mass (no mass array) through the sorted engine, the
    windowed mode and the stream mode: the oracle's grid, and the same grid bit
    for bit from each."""
    import torch
    from genpk_gb300 import synth
    dims, box, mass = 32, 500.0, -0.7
    pos = synth.zeldovich(32, box, seed=81)
    dev = torch.from_numpy(pos).cuda()
    ref = O.deposit(pos, box, dims, None, mass)
    grids = []
    with gp.Context(dims, 8) as ctx:
        for eng in (gp.api.ENGINE_SORTED, gp.api.ENGINE_WINDOW, gp.api.ENGINE_STREAM):
            ctx.set_engine(eng)
            ctx.zero(0)
            ctx.deposit(0, box, dev, None, mass)
            ctx.sync()
            assert ctx.last_engine == eng
            g = ctx.read_field(0)
            grid_close(g, ref, tol=1e-6)
            grids.append(g)
    for g in grids[1:]:
        assert np.array_equal(g, grids[0])
