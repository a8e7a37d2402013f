"""The CPU oracle (oracle/genpk_oracle.c) pinned to the reference.

Known answers are the reference's own tests (test.cpp:31-86); golden fixtures
come from the reference's fieldize.cpp / powerspectrum.c compiled in
oracle/_ref (tests/golden/make_golden.py).  Tolerance of the known answers is
the reference's FLOATS_NEAR_TO: |x-y| <= max(|x|,|y|)/1e5 (test.cpp:25-26).
"""
import numpy as np
import pytest

from conftest import cases
from oracle import oracle as O


def near(x, y, rel=1e-5):
    return abs(x - y) <= max(abs(x), abs(y)) * rel


def impls():
    out = [("port", O.port())]
    r = O.ref()
    if r is not None:
        out.append(("ref", r))
    return out


@pytest.mark.parametrize("name,impl", impls())
def test_check_fieldize_known_answer(name, impl):
    """test.cpp:31-50."""
    dims = 5
    field = np.zeros(2 * dims * dims * (dims // 2 + 1))
    pos = (np.arange(30) / 3.0).astype(np.float32).reshape(10, 3)
    masses = np.full(30, 10.0, dtype=np.float32)
    impl.fieldize(10, dims, field, pos, masses[:10], 10.0, 1)
    assert near(field[0], 8.61111)
    assert field[3] == 0 and field[20] == 0 and field[125] == 0
    assert near(field[124], 1.66666)


@pytest.mark.parametrize("name,impl", impls())
def test_check_invwindow_known_answer(name, impl):
    """test.cpp:52-57."""
    assert near(impl.invwindow(0, 3, 4, 5), 71.8177719)
    assert near(impl.invwindow(4, 4, 4, 5), 6111.20801)
    assert impl.invwindow(1, 1, 1, 0) == 0


def _testcpp_power_field():
    field = np.zeros(2 * 4 * 4 * 3)
    for i in range(32):
        ii = i // 4
        field[6 * ii + i % 4] = 1
    field[0] = 2
    return field.reshape(4, 4, 6)


@pytest.mark.parametrize("name,impl", impls())
def test_check_powerspectrum_known_answer(name, impl):
    """test.cpp:59-86 with pocketfft FP64 in place of FFTW."""
    f = O.rfft_padded(_testcpp_power_field())
    p, c, k = impl.powerspectrum(4, f, f, 10, 64.0, 64.0)
    assert near(k[2], np.sqrt(2))
    assert (c[0], c[1], c[2]) == (6, 0, 12)
    assert near(p[0], 0.0677526)
    assert p[1] == 0
    assert near(p[2], 0.000565561)
    assert near(p[9], 0.0550908)
    assert c.sum() == 4 ** 3 - 1


def test_port_fieldize_matches_golden(golden, oracle_port):
    for name, c in cases(golden["fieldize"]).items():
        dims, box, n, extra, mass = c["meta"]
        dims, n, extra = int(dims), int(n), int(extra)
        grid = np.zeros_like(c["grid"])
        oracle_port.fieldize(box, dims, grid, c["pos"], c.get("masses"), mass, extra)
        np.testing.assert_allclose(grid, c["grid"], rtol=1e-12, atol=1e-12 * abs(c["grid"]).max(),
                                   err_msg=name)


def test_port_powerspectrum_matches_golden(golden, oracle_port):
    for name, c in cases(golden["power"]).items():
        dims, box, n, mass, nrbins, m = c["meta"]
        dims, nrbins = int(dims), int(nrbins)
        p, cnt, k = O.pk(c["pos"], box, dims, nrbins, c.get("masses"), mass, m_norm=m,
                         impl=oracle_port)
        assert np.array_equal(cnt, c["count"]), name
        np.testing.assert_allclose(p, c["power"], rtol=1e-10, atol=1e-300, err_msg=name)
        np.testing.assert_allclose(k, c["keffs"], rtol=1e-12, err_msg=name)


def test_port_counts_match_golden(golden, oracle_port):
    for key, c in cases(golden["counts"]).items():
        dims, nrbins = map(int, key.split("_"))
        zero = np.zeros((dims, dims, dims // 2 + 1), dtype=np.complex128)
        _, cnt, k = oracle_port.powerspectrum(dims, zero, zero, nrbins, 1.0, 1.0)
        assert np.array_equal(cnt, c["count"]), key
        np.testing.assert_allclose(k, c["keffs"], rtol=1e-12, err_msg=key)


@pytest.mark.skipif(O.ref() is None, reason="reference sources not present")
def test_port_matches_reference_build_random():
    rng = np.random.default_rng(5)
    ref, port = O.ref(), O.port()
    for dims in (6, 7, 20):
        pos = (rng.random((3000, 3)) * 7.0 - 1.0).astype(np.float32)  # includes wrap-around
        m = rng.random(3000).astype(np.float32)
        a, b = O.zeros_grid(dims), O.zeros_grid(dims)
        ref.fieldize(5.0, dims, a, pos, m, 0.0, 1)
        port.fieldize(5.0, dims, b, pos, m, 0.0, 1)
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-13)
        f = O.rfft_padded(a)
        g = O.rfft_padded(O.zeros_grid(dims) + 0.5 * a)
        for nr in (3, dims, 64):
            pr = ref.powerspectrum(dims, f, g, nr, 2.0, 3.0)
            pp = port.powerspectrum(dims, f, g, nr, 2.0, 3.0)
            assert np.array_equal(pr[1], pp[1])
            np.testing.assert_allclose(pr[0], pp[0], rtol=1e-11)


def test_port_deposit_conserves_mass(oracle_port):
    """Sum of the FP64 grid equals the deposited mass (CIC weights of each
    particle sum to one), including positions outside the box (wrapped)."""
    from genpk_gb300 import synth
    rng = np.random.default_rng(8)
    pos = np.concatenate([synth.uniform(20000, 100.0, seed=8),
                          rng.uniform(-250.0, 350.0, (5000, 3)).astype(np.float32)])
    masses = rng.lognormal(0.0, 1.0, len(pos)).astype(np.float32)
    for dims in (16, 17, 32):
        g = O.zeros_grid(dims)
        oracle_port.fieldize(100.0, dims, g, pos, masses, 0.0, 1)
        assert abs(g.sum() - masses.astype(np.float64).sum()) <= 1e-9 * masses.sum()


def test_port_bin_of_is_monotone_and_in_range():
    port = O.port()
    for dims, nr in ((64, 64), (128, 17), (256, 256)):
        kmax = 3 * (dims // 2) ** 2
        prev = -1
        for kk2 in range(1, kmax + 1, max(1, kmax // 5000)):
            b = port.bin_of(kk2, dims, nr)
            assert 0 <= b < nr and b >= prev
            prev = b


def test_reference_gradient_matches_finite_differences():
    """The FP64 adjoint restatement against central differences (small case)."""
    rng = np.random.default_rng(3)
    dims, box, nr = 8, 8.0, 6
    pos = (rng.random((200, 3)) * box).astype(np.float64)
    masses = (rng.random(200) + 0.5).astype(np.float32)
    target = np.abs(rng.standard_normal(nr)) + 0.1

    def loss(p, m):
        pw, cnt, _ = O.pk(p.astype(np.float32), box, dims, nr, m, 0.0)
        ok = cnt > 0
        return float(np.sum(((pw - target) ** 2 / target ** 2)[ok])), pw, cnt

    l0, pw, cnt = loss(pos, masses)
    g = np.where(cnt > 0, 2 * (pw - target) / target ** 2, 0.0)
    gpos, gmass, _ = O.reference_gradient(pos.astype(np.float32), box, dims, nr, g, masses, 0.0)
    h = 1e-3
    for idx in [(0, 0), (5, 1), (17, 2), (100, 0)]:
        pp, pm = pos.copy(), pos.copy()
        pp[idx] += h
        pm[idx] -= h
        fd = (loss(pp, masses)[0] - loss(pm, masses)[0]) / (2 * h)
        assert abs(fd - gpos[idx]) <= 2e-3 * max(abs(fd), 1e-6) + 1e-9, (idx, fd, gpos[idx])
    for i in (3, 42):
        mp, mm = masses.astype(np.float64).copy(), masses.astype(np.float64).copy()
        mp[i] += h
        mm[i] -= h
        fd = (loss(pos, mp.astype(np.float32))[0] - loss(pos, mm.astype(np.float32))[0]) / (2 * h)
        assert abs(fd - gmass[i]) <= 2e-2 * abs(fd) + 1e-6, (i, fd, gmass[i])


def test_sampled_reference_gradient_matches_the_full_one():
    """The plane-by-plane, sampled FP64 gradient (used where the full one's
    temporaries would not fit) equals reference_gradient at the sampled
    particles, with the same forward; even and odd grids, both mass kinds."""
    from genpk_gb300 import synth
    for dims, var in ((32, True), (24, False), (15, True)):
        box, nrbins = 1000.0, 12
        pos = synth.zeldovich(dims, box, seed=dims)
        masses = (np.random.default_rng(dims).random(len(pos)) + 0.5).astype(np.float32) \
            if var else None
        g = np.linspace(1.0, -2.0, nrbins) * 1e3
        m = O.total_mass(len(pos), masses, 0.0 if var else 1.0)
        rpos, rmass, rdm = O.reference_gradient(pos, box, dims, nrbins, g, masses,
                                                0.0 if var else 1.0, m_norm=m)
        pr, cr, kr = O.pk(pos, box, dims, nrbins, masses, 0.0 if var else 1.0, m_norm=m)
        idx = np.random.default_rng(1).choice(len(pos), 200, replace=False)
        p, c, k, gpos, gmass, dm = O.reference_gradient_sampled(
            pos, box, dims, nrbins, g, idx, masses, 0.0 if var else 1.0, m_norm=m, workers=2)
        assert np.array_equal(c, cr)
        np.testing.assert_allclose(p, pr, rtol=1e-12, atol=0)
        np.testing.assert_allclose(gpos, rpos[idx], rtol=1e-9, atol=1e-12 * np.abs(rpos).max())
        if var:
            np.testing.assert_allclose(gmass, rmass[idx], rtol=1e-9,
                                       atol=1e-12 * np.abs(rmass).max())
        assert dm == pytest.approx(rdm, rel=1e-12)
