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


def test_batch_graph_replay_matches_eager_calls(gp):
    """Repeated identical calls: the second is captured as one CUDA graph and
    later ones replay it.  Every replay gives the eager path's spectra bit for
    bit, also after the positions change in place (a replay reads the arrays'
    current contents), after a new array (eager again, then a new capture) and
    after a box's context is used on its own (the graph is dropped)."""
    import torch
    from genpk_gb300 import synth
    box, nrbins = 1000.0, 20
    dims = [64, 32, 128, 64]
    pos = [torch.from_numpy(synth.zeldovich(64, box, seed=31)).cuda(),
           torch.from_numpy(synth.uniform(50_000, box, seed=32)).cuda(),
           torch.from_numpy(synth.uniform(3_000_000, box, seed=33)).cuda(),
           torch.from_numpy(synth.uniform(400_000, box, seed=34)).cuda()]
    masses = [None, None, None,
              torch.from_numpy(np.random.default_rng(35).lognormal(0.0, 0.4, 400_000)
                               .astype(np.float32)).cuda()]
    mass = [1.0, 0.5, 2.0, 0.0]

    def norms():
        return [O.total_mass(len(p), None if m is None else m.cpu().numpy(), mu)
                for p, m, mu in zip(pos, masses, mass)]

    def same(a, b):
        return all(np.array_equal(x, y) for x, y in zip(a, b))

    with gp.Batch(dims, nrbins) as g, gp.Batch(dims, nrbins) as e:
        g.set_mode("per_box")
        e.set_mode("per_box")
        e.use_graph(False)
        ref = e.power(box, pos, norms(), masses_list=masses, mass=mass)
        outs = [g.power(box, pos, norms(), masses_list=masses, mass=mass) for _ in range(2)]
        l0 = g.launches  # (the first call's tuning trials and probes are not steady state)
        outs += [g.power(box, pos, norms(), masses_list=masses, mass=mass) for _ in range(3)]
        r5 = g.graph_replays
        assert r5 == 4, r5  # call 2 is captured and replayed, calls 3-5 replay
        assert e.graph_replays == 0
        assert all(same(o, ref) for o in outs)
        per_call = (g.launches - l0) / 3
        le = e.launches
        e.power(box, pos, norms(), masses_list=masses, mass=mass)
        assert per_call == e.launches - le  # a replay counts the kernels it launches

        # new contents, same arrays (and the same normalising masses, which are
        # arguments): replayed, equal to the eager path
        nm = norms()
        with torch.no_grad():
            pos[2].mul_(0.5)
            masses[3].mul_(1.5)
        r = g.power(box, pos, nm, masses_list=masses, mass=mass)
        assert g.graph_replays == r5 + 1
        assert same(r, e.power(box, pos, nm, masses_list=masses, mass=mass))

        # a new array for box 1: eager, then captured again on the next repeat
        pos[1] = torch.from_numpy(synth.uniform(60_000, box, seed=36)).cuda()
        refn = e.power(box, pos, norms(), masses_list=masses, mass=mass)
        for k in range(3):
            assert same(g.power(box, pos, norms(), masses_list=masses, mass=mass), refn)
        assert g.graph_replays == r5 + 3  # eager, captured + replayed, replayed

        # a non-finite position written into box 2's array after the capture:
        # the replay reports it for that box, and the batch stays usable
        with torch.no_grad():
            keep = pos[2][7, 0].item()
            pos[2][7, 0] = float("nan")
        r0 = g.graph_replays
        with pytest.raises(gp.api.GenPKError) as err:
            g.power(box, pos, norms(), masses_list=masses, mass=mass)
        assert err.value.status == 5 and "box 2" in err.value.message
        assert g.graph_replays == r0 + 1
        with torch.no_grad():
            pos[2][7, 0] = keep
        assert same(g.power(box, pos, norms(), masses_list=masses, mass=mass), refn)
        assert g.graph_replays == r0 + 2

        # box 0's context used on its own: the graph is dropped, the call eager
        lib = g.lib
        assert lib.genpk_zero(lib.genpk_batch_box(g.h, 0), 0) == 0
        assert same(g.power(box, pos, norms(), masses_list=masses, mass=mass), refn)
        assert g.graph_replays == r0 + 2
        assert same(g.power(box, pos, norms(), masses_list=masses, mass=mass), refn)
        assert g.graph_replays == r0 + 3


def test_batch_grouped_matches_per_box_and_oracle(gp):
    """Grouped mode: the boxes of each grid size share one grouped
    sorted-engine pass, one batched transform and the binning launches.
    Every box (uneven counts, uniform and per-particle masses, an empty box)
    against the per-box path and the FP64 oracle; counts bit-exact.  Repeated
    calls replay one graph with the eager grouped results bit for bit; a
    non-finite position is reported for its box; switching back gives the
    per-box path."""
    import torch
    from genpk_gb300 import synth
    box, nrbins = 1000.0, 24
    rng = np.random.default_rng(41)
    lm = rng.lognormal(0.0, 0.5, 250_000).astype(np.float32)
    spec = [  # dims, positions, masses or None, uniform mass, normalising mass
        (64, synth.uniform(200_000, box, seed=42), None, 1.0),
        (128, synth.uniform(1_500_000, box, seed=43), None, 0.5),
        (64, synth.zeldovich(64, box, seed=44), None, 2.0),
        (128, synth.uniform(40_000, box, seed=45), None, 1.0),
        (32, synth.uniform(30_000, box, seed=46), None, 1.0),
        (64, synth.uniform(250_000, box, seed=47), lm, 0.0),
        (128, np.zeros((0, 3), np.float32), None, 1.0),
    ]
    dims = [d for d, _, _, _ in spec]
    pos = [torch.from_numpy(p).cuda() for _, p, _, _ in spec]
    masses = [None if m is None else torch.from_numpy(m).cuda() for _, _, m, _ in spec]
    mass = [mu for _, _, _, mu in spec]
    norm = [O.total_mass(len(p), m, mu) if len(p) else 1.0 for _, p, m, mu in spec]
    with gp.Batch(dims, nrbins) as g, gp.Batch(dims, nrbins) as e, \
            gp.Batch(dims, nrbins) as pb:
        g.set_mode(True)
        e.set_mode(True)
        e.use_graph(False)
        pb.set_mode(False)
        per_box = pb.power(box, pos, norm, masses_list=masses, mass=mass)
        assert pb.last_mode == "per_box"
        ref = e.power(box, pos, norm, masses_list=masses, mass=mass)
        assert e.last_mode == "grouped"
        groups = e.groups()
        assert sorted(x["dims"] for x in groups) == [32, 64, 128]
        assert sorted(i for x in groups for i in x["boxes"]) == list(range(len(spec)))
        for x in groups:
            assert all(dims[i] == x["dims"] for i in x["boxes"])
            assert x["trials"] and x["config"]["sort_ctas"] > 0
        outs = [g.power(box, pos, norm, masses_list=masses, mass=mass) for _ in range(2)]
        l0 = g.launches
        outs += [g.power(box, pos, norm, masses_list=masses, mass=mass) for _ in range(2)]
        assert g.graph_replays == 3
        for o in outs:
            assert all(np.array_equal(a, b) for a, b in zip(o, ref))
        # one grouped pass per grid size: far fewer kernels than box by box
        l1 = pb.launches
        pb.power(box, pos, norm, masses_list=masses, mass=mass)
        assert (g.launches - l0) / 2 < pb.launches - l1, (g.launches - l0, pb.launches - l1)

        for i, (d, p, m, mu) in enumerate(spec):
            pg, cg, kg = ref[0][i], ref[1][i], ref[2][i]
            assert np.array_equal(cg, per_box[1][i])
            np.testing.assert_allclose(kg, per_box[2][i], rtol=1e-12)
            if len(p) == 0:
                assert not pg.any() and not per_box[0][i].any()
                continue
            pr, cr, kr = O.pk(p, box, d, nrbins, m, mu, m_norm=norm[i])
            assert np.array_equal(cg, cr)
            ok = cr > 0
            rel = np.abs(pg[ok] - pr[ok]) / np.abs(pr[ok])
            assert rel.max() <= P_RTOL, (i, rel.max())
            np.testing.assert_allclose(pg, per_box[0][i], rtol=1e-6, atol=0)

        # a non-finite position in box 3 (a 128^3 box grouped with others):
        # reported for that box; the replayed graph and the batch stay usable
        with torch.no_grad():
            keep = pos[3][11, 2].item()
            pos[3][11, 2] = float("inf")
        with pytest.raises(gp.api.GenPKError) as err:
            g.power(box, pos, norm, masses_list=masses, mass=mass)
        assert err.value.status == 5 and "box 3" in err.value.message
        with torch.no_grad():
            pos[3][11, 2] = keep
        r = g.power(box, pos, norm, masses_list=masses, mass=mass)
        assert all(np.array_equal(a, b) for a, b in zip(r, ref))

        # back to per-box issue
        g.set_mode(False)
        r = g.power(box, pos, norm, masses_list=masses, mass=mass)
        for a, b in zip(r, per_box):
            np.testing.assert_allclose(a, b, rtol=1e-6, atol=0)


def test_batch_grouped_splits_large_groups_and_falls_back(gp):
    """33 boxes of one grid size make two groups (at most 32 boxes each); host
    arrays are not grouped (the call runs box by box) and give the same
    spectra as device arrays."""
    import torch
    from genpk_gb300 import synth
    box, nrbins, nb = 500.0, 12, 33
    pos = [synth.uniform(5_000 + 300 * i, box, seed=100 + i) for i in range(nb)]
    norm = [O.total_mass(len(p), None, 1.0) for p in pos]
    dpos = [torch.from_numpy(p).cuda() for p in pos]
    with gp.Batch([32] * nb, nrbins) as b:
        b.set_mode(True)
        ph, ch, _ = b.power(box, pos, norm, mass=1.0)  # host arrays: per box
        assert b.groups() == []
        pd, cd, _ = b.power(box, dpos, norm, mass=1.0)
        sizes = sorted(len(x["boxes"]) for x in b.groups())
        assert sizes == [1, 32], sizes
    assert np.array_equal(ch, cd)
    np.testing.assert_allclose(pd, ph, rtol=1e-6, atol=0)
    for i in (0, 17, 32):
        pr, cr, _ = O.pk(pos[i], box, 32, nrbins, None, 1.0, m_norm=norm[i])
        assert np.array_equal(cd[i], cr)
        ok = cr > 0
        assert (np.abs(pd[i][ok] - pr[ok]) / np.abs(pr[ok])).max() <= P_RTOL


def test_batch_auto_mode_times_both_ways_then_keeps_the_faster(gp):
    """The default mode: the first four calls of one shape run per box,
    grouped, per box, grouped (eager; the last two timed), later calls the
    faster way, captured and replayed.  Every call agrees with the oracle; a
    call of another shape starts the trials again; host arrays run per box."""
    import torch
    from genpk_gb300 import synth
    box, nrbins = 1000.0, 16
    dims = [64, 64, 32]
    host = [synth.uniform(150_000, box, seed=61), synth.uniform(60_000, box, seed=62),
            synth.uniform(20_000, box, seed=63)]
    pos = [torch.from_numpy(p).cuda() for p in host]
    norm = [O.total_mass(len(p), None, 1.0) for p in host]
    refs = [O.pk(p, box, d, nrbins, None, 1.0, m_norm=m) for p, d, m in zip(host, dims, norm)]

    def check(out):
        for i, (pr, cr, _) in enumerate(refs):
            assert np.array_equal(out[1][i], cr)
            ok = cr > 0
            assert (np.abs(out[0][i][ok] - pr[ok]) / np.abs(pr[ok])).max() <= P_RTOL

    with gp.Batch(dims, nrbins) as b:
        modes = []
        for k in range(7):
            check(b.power(box, pos, norm, mass=1.0))
            modes.append(b.last_mode)
            if k < 3:
                assert b.auto_times()["choice"] is None
        t = b.auto_times()
        assert modes[:4] == ["per_box", "grouped", "per_box", "grouped"], modes
        assert t["choice"] in ("per_box", "grouped") and t["per_box_ms"] > 0 and t["grouped_ms"] > 0
        assert modes[4:] == [t["choice"]] * 3
        assert b.graph_replays == 3  # call 5 captured and replayed, 6 and 7 replayed
        # another shape: the trials again
        pos2 = [pos[0], pos[1][:50_000], pos[2]]
        b.power(box, pos2, norm, mass=1.0)
        assert b.last_mode == "per_box" and b.auto_times()["choice"] is None
        # host arrays are never grouped
        out = b.power(box, host, norm, mass=1.0)
        assert b.last_mode == "per_box"
        check(out)


def test_batch_grouped_odd_grids_and_negative_masses(gp):
    """Grouped boxes on odd and non-power-of-two grids (3-D cuFFT and the
    binning kernel; no corner mode), with a negative uniform mass and signed
    per-particle masses: the per-box path's spectra and the FP64 oracle's."""
    import torch
    from genpk_gb300 import synth
    box, nrbins = 700.0, 12
    rng = np.random.default_rng(71)
    sm = rng.normal(0.0, 1.0, 80_000).astype(np.float32)
    spec = [(33, synth.uniform(90_000, box, seed=72), None, -0.5),
            (33, synth.uniform(80_000, box, seed=73), sm, 0.0),
            (48, synth.uniform(120_000, box, seed=74), None, 2.0),
            (33, synth.zeldovich(33, box, seed=75), None, 1.0)]
    dims = [d for d, _, _, _ in spec]
    pos = [torch.from_numpy(p).cuda() for _, p, _, _ in spec]
    masses = [None if m is None else torch.from_numpy(m).cuda() for _, _, m, _ in spec]
    mass = [mu for _, _, _, mu in spec]
    norm = [O.total_mass(len(p), m, mu) for _, p, m, mu in spec]
    with gp.Batch(dims, nrbins) as g, gp.Batch(dims, nrbins) as pb:
        g.set_mode("grouped")
        pb.set_mode("per_box")
        out = g.power(box, pos, norm, masses_list=masses, mass=mass)
        assert g.last_mode == "grouped"
        assert sorted(len(x["boxes"]) for x in g.groups()) == [1, 3]
        ref = pb.power(box, pos, norm, masses_list=masses, mass=mass)
    for i, (d, p, m, mu) in enumerate(spec):
        pr, cr, _ = O.pk(p, box, d, nrbins, m, mu, m_norm=norm[i])
        assert np.array_equal(out[1][i], cr) and np.array_equal(ref[1][i], cr)
        ok = cr > 0
        for got in (out, ref):
            rel = np.abs(got[0][i][ok] - pr[ok]) / np.abs(pr[ok])
            assert rel.max() <= P_RTOL, (i, rel.max())
        np.testing.assert_allclose(out[0][i], ref[0][i], rtol=1e-6, atol=0)
