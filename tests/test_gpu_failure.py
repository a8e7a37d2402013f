"""Failure detection on the GPU without a fault: a bounded device wait made to
run out on purpose.

The window engine's kernels (windowed and stream mode) wait for each chunk's
bulk copy on an mbarrier, with a bounded spin (about a second).
genpk_inject_copy_timeout makes the next pass leave one chunk's copy unissued
and gives that one wait a short limit, so it gives up with nothing in flight:
nothing faults or hangs.  Checked here:
  * the status reaches the caller as GENPK_ERR_TIMEOUT (8) at the next sync
    point, with the one wait counted;
  * the pass still deposits every particle (the CTA loads that chunk and its
    later ones with plain loads): its grid equals an undisturbed pass's bit for
    bit;
  * the context stays usable: the next pass on it is exact and its spectrum
    matches the FP64 oracle.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TIMEOUT = 8


@pytest.fixture(scope="module")
def gp(native_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    import genpk_gb300
    return genpk_gb300


def _grid(gp, dims, nrbins, engine, box, dpos, inject=None):
    """One deposit pass; returns (grid, status of the sync after it)."""
    with gp.Context(dims, nrbins) as ctx:
        ctx.set_engine(engine)
        if inject is not None:
            ctx.inject_copy_timeout(inject, 1 << 14)
        ctx.deposit(0, box, dpos, None, 1.0)
        status, msg = 0, ""
        try:
            ctx.sync()
        except gp.GenPKError as e:
            status, msg = e.status, str(e)
        assert ctx.last_engine == engine
        return ctx.read_field(0), status, msg


@pytest.mark.parametrize("engine_name,dims,chunk", [
    ("stream", 128, 3),     # the first chunk of a CTA (issued before its loop)
    ("stream", 128, 157),   # a prefetched chunk (a CTA's second on 152 SMs)
    ("window", 64, 3),
    ("window", 64, 157),
])
def test_copy_wait_timeout_is_reported_and_the_pass_completes(gp, engine_name, dims, chunk):
    import torch
    from genpk_gb300 import api, synth
    engine = {"stream": api.ENGINE_STREAM, "window": api.ENGINE_WINDOW}[engine_name]
    box, nrbins = 1000.0, 32
    pos = synth.zeldovich(128, box, seed=31)  # 2^21 particles: 512 chunks of 4096
    dpos = torch.from_numpy(pos).cuda()
    clean, st0, _ = _grid(gp, dims, nrbins, engine, box, dpos)
    assert st0 == 0
    got, st, msg = _grid(gp, dims, nrbins, engine, box, dpos, inject=chunk)
    assert st == TIMEOUT, (st, msg)
    assert "1 bounded device wait(s) gave up" in msg, msg
    assert np.array_equal(got, clean), "the pass that timed out lost particles"


def test_context_stays_usable_after_a_timeout(gp):
    import torch
    from genpk_gb300 import api, synth
    box, dims, nrbins = 1000.0, 128, 32
    pos = synth.zeldovich(128, box, seed=32)
    dpos = torch.from_numpy(pos).cuda()
    m = O.total_mass(len(pos), None, 1.0)
    pr, cr, _ = O.pk(pos, box, dims, nrbins, None, 1.0, m_norm=m)
    with gp.Context(dims, nrbins) as ctx:
        ctx.set_engine(api.ENGINE_STREAM)
        ctx.inject_copy_timeout(200, 1 << 14)
        ctx.deposit(0, box, dpos, None, 1.0)
        with pytest.raises(gp.GenPKError) as e:
            ctx.power(0, 0, m, m)
        assert e.value.status == TIMEOUT
        # the status was reported once; the next pass runs undisturbed
        ctx.zero(0)
        ctx.deposit(0, box, dpos, None, 1.0)
        p, c, _ = ctx.power(0, 0, m, m)
    assert np.array_equal(c, cr)
    ok = cr > 0
    rel = np.abs(p[ok] - pr[ok]) / np.abs(pr[ok])
    assert rel.max() <= 1e-5, rel.max()
