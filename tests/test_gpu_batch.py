"""Many boxes in one call (genpk_batch_power): uneven particle counts and grid
sizes, host and device arrays, uniform and per-particle masses.  Every box's
spectrum against the same box computed through a context of its own and
against the FP64 oracle; mode counts bit-exact."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

P_RTOL = 1e-5


@pytest.fixture(scope="module")
def gp(native_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    import genpk_gb300
    return genpk_gb300


def boxes():
    import torch
    from genpk_gb300 import synth
    box = 1000.0
    rng = np.random.default_rng(3)
    lmass = rng.lognormal(0.0, 0.5, 300_000).astype(np.float32)
    # (dims, positions, masses or None, uniform mass, on the device?)
    return box, [
        (32, synth.uniform(20_000, box, seed=1), None, 1.0, False),
        (64, synth.zeldovich(64, box, seed=2), None, 0.5, True),
        (96, synth.uniform(1_000_000, box, seed=3), None, 2.0, True),
        (128, synth.uniform(2_000_000, box, seed=4), None, 1.0, False),
        (128, synth.zeldovich(128, box, seed=5), None, 1.0, True),
        (64, synth.uniform(300_000, box, seed=6), lmass, 0.0, True),
    ]


def test_batch_matches_contexts_and_oracle(gp):
    import torch
    box, spec = boxes()
    nrbins = 24
    dims = [d for d, _, _, _, _ in spec]
    pos = [torch.from_numpy(p).cuda() if dev else p for _, p, _, _, dev in spec]
    masses = [None if m is None else (torch.from_numpy(m).cuda() if dev else m)
              for _, _, m, _, dev in spec]
    mass = [mu for _, _, _, mu, _ in spec]
    norm = [O.total_mass(len(p), m, mu) for _, p, m, mu, _ in spec]
    with gp.Batch(dims, nrbins) as b:
        first = b.power(box, pos, norm, masses_list=masses, mass=mass)
        again = b.power(box, pos, norm, masses_list=masses, mass=mass)  # choices kept
        assert b.launches > 0
    for i, (d, p, m, mu, _) in enumerate(spec):
        with gp.Context(d, nrbins) as ctx:
            ctx.deposit(0, box, pos[i], masses[i], mu)
            pc, cc, kc = ctx.power(0, 0, norm[i], norm[i])
        pr, cr, kr = O.pk(p, box, d, nrbins, m, mu, m_norm=norm[i])
        for pb, cb, kb in (first, again):
            assert np.array_equal(cb[i], cr) and np.array_equal(cb[i], cc)
            np.testing.assert_allclose(kb[i], kr, rtol=1e-12)
            ok = cr > 0
            rel = np.abs(pb[i][ok] - pr[ok]) / np.abs(pr[ok])
            assert rel.max() <= P_RTOL, (i, rel.max())
            # the same box alone: equal up to which FFT path its engine took
            np.testing.assert_allclose(pb[i], pc, rtol=1e-6, atol=0)


def test_batch_reports_a_failing_box_and_stays_usable(gp):
    """A box with a non-finite position reports GENPK_ERR_BAD_INPUT naming
    that box; every other box is still computed and the batch is usable."""
    import torch
    from genpk_gb300 import synth
    box, nrbins = 1000.0, 16
    good = torch.from_numpy(synth.uniform(100_000, box, seed=8)).cuda()
    bad = synth.uniform(100_000, box, seed=9)
    bad[123, 1] = np.nan
    badd = torch.from_numpy(bad).cuda()
    m = O.total_mass(100_000, None, 1.0)
    with gp.Batch([32, 32], nrbins) as b:
        with pytest.raises(gp.GenPKError) as e:
            b.power(box, [good, badd], m, mass=1.0)
        assert e.value.status == 5 and "box 1" in str(e.value)
        p, c, _ = b.power(box, [good, good], m, mass=1.0)
    assert np.array_equal(p[0], p[1])
