"""One step of the per-species loop (genpk_power_step): three species on one
grid, three auto and three cross spectra, against the same step issued call by
call (deposit per species + genpk_power_multi) and against the FP64 oracle.
Repeated identical steps replay a captured CUDA graph of the whole step."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

P_RTOL = 1e-5
PAIRS = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]


@pytest.fixture(scope="module")
def gp(native_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    import genpk_gb300
    return genpk_gb300


def species():
    import torch
    from genpk_gb300 import synth
    box = 20000.0
    dm = torch.from_numpy(synth.zeldovich(64, box, seed=41)).cuda()
    gas = torch.from_numpy(synth.zeldovich(64, box, seed=41, amplitude=0.7)).cuda()
    spos, smass = synth.lognormal(300_000, box, 64, sigma=1.2, seed=42, mass_mu=-3.0,
                                  mass_sigma=0.6)
    stars = torch.from_numpy(spos).cuda()
    sm = torch.from_numpy(smass).cuda()
    return box, [dm, gas, stars], [None, None, sm], [1.0, 0.19, 0.0]


def step_by_calls(gp, dims, nrbins, box, pos, masses, mass, pm):
    with gp.Context(dims, nrbins, nfields=3) as ctx:
        for f in range(3):
            ctx.deposit(f, box, pos[f], masses[f], mass[f])
        return ctx.power_multi(PAIRS, pm)


def test_power_step_graph_replays_match_calls_and_oracle(gp):
    import torch
    dims, nrbins = 64, 32
    box, pos, masses, mass = species()

    def norms():
        ms = [O.total_mass(len(p), None if m is None else m.cpu().numpy(), mu)
              for p, m, mu in zip(pos, masses, mass)]
        return [(ms[a], ms[b]) for a, b in PAIRS]

    ref = step_by_calls(gp, dims, nrbins, box, pos, masses, mass, norms())
    with gp.Context(dims, nrbins, nfields=3) as ctx:
        outs = [ctx.power_step(box, pos, PAIRS, norms(), masses_list=masses, mass=mass)
                for _ in range(5)]
        assert ctx.step_replays == 4, ctx.step_replays
        for o in outs:
            for x, y in zip(o, ref):
                assert np.array_equal(x, y)
        # new contents in the same arrays (the normalising masses, which are
        # arguments, kept): replayed, equal to the calls
        nm = norms()
        with torch.no_grad():
            pos[2].mul_(0.75)
            masses[2].mul_(2.0)
        r = ctx.power_step(box, pos, PAIRS, nm, masses_list=masses, mass=mass)
        assert ctx.step_replays == 5
        ref2 = step_by_calls(gp, dims, nrbins, box, pos, masses, mass, nm)
        for x, y in zip(r, ref2):
            assert np.array_equal(x, y)
        # the context used otherwise: the graph is dropped, the next step eager
        ctx.zero(1)
        r = ctx.power_step(box, pos, PAIRS, nm, masses_list=masses, mass=mass)
        assert ctx.step_replays == 5
        for x, y in zip(r, ref2):
            assert np.array_equal(x, y)
        # graphs off: eager steps, the same results
        ctx.step_use_graph(False)
        for _ in range(3):
            r = ctx.power_step(box, pos, PAIRS, nm, masses_list=masses, mass=mass)
        assert ctx.step_replays == 5
        for x, y in zip(r, ref2):
            assert np.array_equal(x, y)
    # the oracle: every auto bin within 1e-5, cross bins relative to sqrt(P_aa P_bb)
    p, c, k = ref2
    ms = nm
    spec = [O.rfft_padded(O.deposit(q.cpu().numpy(), box, dims,
                                    None if m is None else m.cpu().numpy(), mu))
            for q, m, mu in zip(pos, masses, mass)]
    port = O.port()
    refs = [port.powerspectrum(dims, spec[a], spec[b], nrbins, ma, mb)
            for (a, b), (ma, mb) in zip(PAIRS, ms)]
    auto = {a: refs[i][0] for i, (a, b) in enumerate(PAIRS) if a == b}
    for i, (a, b) in enumerate(PAIRS):
        pr, cr, kr = refs[i]
        assert np.array_equal(c, cr)
        ok = cr > 0
        scale = np.abs(pr) if a == b else np.maximum(np.abs(pr), np.sqrt(np.abs(auto[a] * auto[b])))
        rel = np.abs(p[i][ok] - pr[ok]) / scale[ok]
        assert rel.max() <= P_RTOL, (a, b, rel.max())


def test_power_step_host_arrays_run_eagerly(gp):
    """Host (numpy) particle arrays: every step eager (their staging copies
    are host work a replay would not repeat), results equal to the calls."""
    box, pos, masses, mass = species()
    hpos = [p.cpu().numpy() for p in pos]
    hm = [None if m is None else m.cpu().numpy() for m in masses]
    ms = [O.total_mass(len(p), m, mu) for p, m, mu in zip(hpos, hm, mass)]
    pm = [(ms[a], ms[b]) for a, b in PAIRS]
    ref = step_by_calls(gp, 64, 16, box, hpos, hm, mass, pm)
    with gp.Context(64, 16, nfields=3) as ctx:
        for _ in range(3):
            r = ctx.power_step(box, hpos, PAIRS, pm, masses_list=hm, mass=mass)
        assert ctx.step_replays == 0
    for x, y in zip(r, ref):
        assert np.array_equal(x, y)
