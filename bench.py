#!/usr/bin/env python
"""Benchmark of the GB300 power-spectrum hot path.

Workload (default): 512^3 particles on a lattice displaced by the Zel'dovich
approximation (P(k) ~ k^-2 exp(-(k/k_c)^2), k_c = k_Nyq/2, RMS displacement 0.3
lattice spacings), L = 100000 kpc/h, equal masses 1.0, FP32 512^3 grid, 64
log-k bins.  One step = one spectrum: zero the grid, CIC-deposit all
particles, r2c FFT, fused deconvolution + binning, read the 64 bins back.

  value      particles/s with the particles resident in HBM (Np / device time
             of one step, CUDA events on the library's stream), summed over
             ranks (each rank an independent box: replicas, weak scaling).
  e2e        the same through the C ABI from pinned host buffers: the H2D copy
             of the positions and the D2H of the bins are inside each step.
  e2e_pageable  the same from pageable host memory in chunks of 2^26 particles,
             the way the reference's reader hands them to fieldize.
  roofline   HBM roofline of the deposit pass (the dominant stage): algorithmic
             bytes Np*12 + 4*N^2*2(N/2+1) over its device time; also the
             binning kernel and deposit+binning together.
  cpu_baseline  the FP64 oracle port (OpenMP, all host cores) on the same
             particles: deposit + FP64 r2c (pocketfft) + binning.

``--impl reference`` times the CPU implementation of the reference's algorithm
(the oracle port: the reference sources are not available on the GPU host) on
the same config, the whole workload every step, and prints one line with
"impl": "reference".
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = ("particles/s + ms/spectrum at 512^3 grid vs FP64 oracle; "
          "fwd+adjoint/fwd time ratio")
PEAKS_FALLBACK = {"hbm_gbs": 6800.0}
# dram__bytes_read.sum + dram__bytes_write.sum of one deposit-kernel launch,
# from ncu captures of Zel'dovich lattices in lattice order (uniform mass),
# keyed by (kernel, particles per side, grid): the positions and the 64-bit
# accumulator's lines read, the accumulator written.  Reported only for those
# workloads.
NCU_TRAFFIC = {("k_stream_deposit", 512, 512): 2.691e9 + 1.036e9,
               ("k_window_deposit", 512, 512): 2.692e9 + 1.052e9,
               ("k_stream_deposit", 256, 256): 337.3e6 + 92.7e6}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--nside", type=int, default=512, help="particles per lattice side")
    ap.add_argument("--grid", type=int, default=512)
    ap.add_argument("--nrbins", type=int, default=64)
    ap.add_argument("--box", type=float, default=100000.0)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU oracle leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--engine", choices=["auto", "sorted", "window", "stream"], default="auto",
                    help="deposit engine (default: the library's automatic choice)")
    ap.add_argument("--fft", choices=["auto", "cufft3d"], default="auto",
                    help="forward FFT path (default: the library's choice)")
    ap.add_argument("--workload", choices=["zeldovich", "uniform", "multispecies", "boxes"],
                    default="zeldovich",
                    help="zeldovich: one species (sizes from --nside/--grid/--box); "
                         "multispecies: DM 256^3 + gas 256^3 + 1.2e7 lognormal stars on a "
                         "512^3 grid, 3 auto + 3 cross spectra per step; boxes: 16 boxes of "
                         "uniform particles, counts log-uniform in [1e5, 3e7], grids 128^3 or "
                         "256^3, one auto spectrum each per step")
    ap.add_argument("--order", choices=["lattice", "morton", "random"], default="lattice",
                    help="particle order of the Zel'dovich workload: lattice (x slowest), "
                         "morton (a space-filling curve, as snapshots are often written) or "
                         "random (shuffled)")
    ap.add_argument("--batch-mode", choices=["auto", "per_box", "grouped"], default="auto",
                    help="boxes workload: how the timed batch calls run (auto: the library's "
                         "default, per box or grouped by its own timed trials)")
    ap.add_argument("--profile-timed", action="store_true",
                    help="open the CUDA profiler range (cudaProfilerStart/Stop) around the timed "
                         "steps only, for `ncu --profile-from-start off`: set-up, tuning and "
                         "warm-up launches stay out of a launch list")
    return ap.parse_args()


class ProfiledRange:
    """cudaProfilerStart/Stop around a block when enabled (no effect otherwise)."""

    def __init__(self, on):
        self.on = on

    def __enter__(self):
        if self.on:
            import torch
            torch.cuda.synchronize()
            torch.cuda.profiler.start()

    def __exit__(self, *exc):
        if self.on:
            import torch
            torch.cuda.synchronize()
            torch.cuda.profiler.stop()


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return PEAKS_FALLBACK, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.dev), "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                    power.append(float(parts[3]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(smax),
                "power_w_max": max(power), "samples": len(sm), "reasons": sorted(reasons)}


def dist_setup(backend):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend=backend)
    return world, rank, local


def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """The largest x over all ranks: the whole job's step time is the slowest
    rank's (each rank deposits and transforms its own box)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: int, world: int, ms_slowest: float) -> float:
    """Whole-job units per second: every rank's units over the slowest rank's
    time (weak scaling: each rank holds the same work)."""
    return units_per_rank * world / (ms_slowest * 1e-3)


def algorithmic_bytes(np_, n, var_masses=False):
    cells = 4 * n * n * 2 * (n // 2 + 1)
    dep = np_ * (12 + (4 if var_masses else 0)) + cells
    binb = 8 * n * n * (n // 2 + 1)
    return dep, binb


# ---------------------------------------------------------------------------
# CPU leg (oracle port): used for cpu_baseline and for the reference arm
# ---------------------------------------------------------------------------

def cpu_pipeline(pos_host, box, n, nrbins, mass):
    """FP64 deposit + FFT + binning of all the particles on the host cores.
    Returns (power, count, timings dict, particles deposited)."""
    from oracle import oracle as O
    import scipy.fft as sfft
    port = O.port()
    cores = port.num_threads()
    sub = pos_host
    grid = O.zeros_grid(n)
    t0 = time.perf_counter()
    port.fieldize(box, n, grid, sub, None, mass, 1)
    t1 = time.perf_counter()
    f = sfft.rfftn(grid[:, :, :n], workers=cores)
    t2 = time.perf_counter()
    m = O.total_mass(len(pos_host), None, mass)
    p, c, k = port.powerspectrum(n, f, f, nrbins, m, m)
    t3 = time.perf_counter()
    return p, c, {"deposit": t1 - t0, "fft": t2 - t1, "bin": t3 - t2, "cores": cores}, len(sub)


def reference_arm(args):
    world, rank, _ = dist_setup("gloo")
    if rank != 0:
        return
    n, nside = args.grid, args.nside
    npart = nside ** 3
    pos = positions(args, seed=1)
    times, stages = [], {"deposit": 0.0, "fft": 0.0, "bin": 0.0}
    cores = 1
    for it in range(args.warmup + args.steps):
        _, _, t, ndep = cpu_pipeline(pos, args.box, n, args.nrbins, particle_mass(args))
        assert ndep == npart
        cores = t["cores"]
        if it >= args.warmup:
            times.append(t["deposit"] + t["fft"] + t["bin"])
            for k in stages:
                stages[k] += t[k] / args.steps
    tstep = float(np.mean(times))
    value = npart / tstep
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "particles/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": tstep * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": f"synthetic (seeded, {'uniform random' if args.workload == 'uniform' else 'Zeldovich lattice'})",
        "config": config_dict(args, npart),
        "cpu_baseline": {"value": value, "unit": "particles/s", "cores": cores, "kind": "port",
                         "sample": f"each step the whole workload: deposit of all {npart} "
                                   f"particles, {n}^3 FP64 r2c and binning"},
        "stages_s": {k: round(v, 4) for k, v in stages.items()},
        "e2e": {"value": value, "unit": "particles/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def morton_order(nside, device):
    """Permutation of an nside^3 lattice (x slowest) into Morton (Z-curve) order
    of the lattice cells: blocks of 2^k cells stay together, as in snapshots
    written in a space-filling-curve order."""
    import torch
    i = torch.arange(nside ** 3, device=device, dtype=torch.int64)
    x, y, z = i // (nside * nside), (i // nside) % nside, i % nside
    code = torch.zeros_like(i)
    for b in range(max(1, (nside - 1).bit_length())):
        code |= ((x >> b) & 1) << (3 * b + 2)
        code |= ((y >> b) & 1) << (3 * b + 1)
        code |= ((z >> b) & 1) << (3 * b)
    return torch.argsort(code)


def positions(args, seed, device="cpu"):
    """nside^3 particles: a Zel'dovich lattice (lattice order, or reordered by
    --order), or i.i.d. uniform positions in [0, box) (the 128^3
    Gadget-snapshot configuration)."""
    from genpk_gb300 import synth
    if args.workload == "uniform":
        return synth.uniform(args.nside ** 3, args.box, seed=seed, device=device)
    pos = synth.zeldovich(args.nside, args.box, seed=seed, device=device)
    if args.order == "lattice":
        return pos
    import torch
    t = pos if isinstance(pos, torch.Tensor) else torch.from_numpy(pos)
    if args.order == "morton":
        perm = morton_order(args.nside, t.device)
    else:
        g = torch.Generator(device="cpu").manual_seed(seed)
        perm = torch.randperm(args.nside ** 3, generator=g).to(t.device)
    out = t[perm].contiguous()
    return out if isinstance(pos, torch.Tensor) else out.numpy()


def particle_mass(args):
    return 1.0e-2 if args.workload == "uniform" else 1.0


L2_BYTES = 129 * 2 ** 20  # GB300 L2 (queried on the device where torch reports it)


def l2_bytes():
    try:
        import torch
        return int(getattr(torch.cuda.get_device_properties(0), "L2_cache_size", L2_BYTES))
    except Exception:
        return L2_BYTES


def needs_l2_flush(npart):
    """Positions smaller than twice the L2 would be served from it on the next
    step: such runs write a buffer larger than the L2 between steps."""
    return npart * 12 < 2 * l2_bytes()


def config_dict(args, npart):
    kind = ("uniform random particles (mass 1e-2)" if args.workload == "uniform"
            else "Zel'dovich lattice particles" + ("" if args.order == "lattice"
                                                   else f" in {args.order} order"))
    l2 = (f"L2 flushed between steps (a {2 * l2_bytes() / 1e6:.0f} MB buffer written outside "
          f"the stage events; {npart * 12 / 1e9:.3f} GB of positions per step)"
          if needs_l2_flush(npart)
          else f"inputs larger than L2 ({npart * 12 / 1e9:.2f} GB of positions per step)")
    return {"workload": (f"{kind}, {args.nside}^3 particles, L={args.box:g} kpc/h, "
                         f"FP32 {args.grid}^3 grid, {args.nrbins} log-k bins, auto spectrum"),
            "particles": npart, "grid": args.grid, "nrbins": args.nrbins, "boxsize": args.box,
            "l2": l2, "parallelism": "replicas (one independent box per GPU)"}


def tuning_record(cfg, trials, engine):
    """The deposit engine a context used and, for the sorted engine, its tile,
    sort CTAs and the autotuner's timed trials."""
    label = lambda t: "stream" if t == (0, 0, 0) else "x".join(str(v) for v in t)
    rec = {"engine": engine}
    if engine == "sorted":
        rec["tile"] = label(cfg["tile"])
        rec["sort_ctas"] = cfg["sort_ctas"]
    if trials:
        rec["trials_ms"] = [[label(t) + ("" if t == (0, 0, 0) else f"/{c}"), round(float(ms), 4)]
                            for t, c, ms in trials]
    return rec


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def multispecies(args):
    """Three species on one 512^3 grid per step: DM (256^3 Zel'dovich, mass
    1.0), gas (the same field at 0.7 displacement amplitude, mass 0.19) and
    1.2e7 stars Poisson-sampled from a lognormal field (sigma_ln 1.5) with
    lognormal masses (mu -5, sigma 0.8); 3 auto and 3 cross spectra."""
    import torch
    import genpk_gb300 as gp
    from genpk_gb300 import synth
    from oracle import oracle as O
    n, nrbins, box = 512, args.nrbins, args.box
    dm = synth.zeldovich(256, box, seed=11, device="cuda")
    gas = synth.zeldovich(256, box, seed=11, amplitude=0.7, device="cuda")
    spos, smass = synth.lognormal(12_000_000, box, 256, sigma=1.5, seed=12, mass_mu=-5.0,
                                  mass_sigma=0.8)
    stars = torch.from_numpy(spos).cuda()
    smass_d = torch.from_numpy(smass).cuda()
    torch.cuda.synchronize()
    m_dm = O.total_mass(len(dm), None, 1.0)
    m_gas = O.total_mass(len(gas), None, 0.19)
    m_st = O.total_mass(len(spos), smass)
    ms = [m_dm, m_gas, m_st]
    pairs = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
    pm = [(ms[a], ms[b]) for a, b in pairs]
    ctx = gp.Context(n, nrbins, nfields=3, timing=True)
    ctx.set_fft_mode({"auto": 0, "cufft3d": 1}[args.fft])

    def step():
        ctx.timing_reset()
        for f in range(3):
            ctx.zero(f)
        ctx.deposit(0, box, dm, None, 1.0)
        ctx.deposit(1, box, gas, None, 0.19)
        ctx.deposit(2, box, stars, smass_d, 0.0)
        p, c, k = ctx.power_multi(pairs, pm)
        return p, c, ctx.stage_times()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    dev_ms, stages = [], {}
    t0 = time.perf_counter()
    with ProfiledRange(args.profile_timed):
        for _ in range(args.steps):
            p, c, st = step()
            dev_ms.append(sum(st.values()))
            for key, v in st.items():
                stages[key] = stages.get(key, 0.0) + v
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ms_step = float(np.mean(dev_ms))
    npart = len(dm) + len(gas) + len(spos)
    line = {"metric": "particles/s + ms per step (3 species, 3 auto + 3 cross spectra)",
            "value": npart / (ms_step * 1e-3), "unit": "particles/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: Zel'dovich DM and gas on the GPU, lognormal stars (numpy)",
            "config": {"workload": "DM 256^3 + gas 256^3 + 1.2e7 stars, 512^3 grid, "
                                   f"{nrbins} bins, 3 auto + 3 cross spectra",
                       "particles": npart, "grid": n, "nrbins": nrbins, "boxsize": box,
                       "l2": f"inputs larger than L2 ({npart * 12 / 1e9:.2f} GB of positions and "
                             "three 1.08 GB grids per step)"},
            "wall_ms_per_step": wall / args.steps * 1e3,
            "stages_ms": {k: round(v / args.steps, 5) for k, v in stages.items()},
            "deposit_engines": "per species, automatic"}
    ctx.close()
    # The same step through genpk_power_step on a context without stage events:
    # repeated identical steps replay one captured CUDA graph of the whole step.
    # Wall clock per step (each call returns with the spectra on the host).
    gctx = gp.Context(n, nrbins, nfields=3)
    gctx.set_fft_mode({"auto": 0, "cufft3d": 1}[args.fft])
    spec_pos, spec_m, spec_mu = [dm, gas, stars], [None, None, smass_d], [1.0, 0.19, 0.0]
    for _ in range(max(args.warmup, 3)):
        gctx.power_step(box, spec_pos, pairs, pm, masses_list=spec_m, mass=spec_mu)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        pg, cg, _ = gctx.power_step(box, spec_pos, pairs, pm, masses_list=spec_m, mass=spec_mu)
    g_ms = (time.perf_counter() - t0) / args.steps * 1e3
    line["graph_step"] = {"api": "genpk_power_step (one call per step)",
                          "wall_ms_per_step": g_ms, "graph_replays": gctx.step_replays,
                          "same_as_calls": bool(np.array_equal(pg, p) and np.array_equal(cg, c))}
    gctx.close()
    if not args.no_cpu:
        # every bin of the 6 spectra against the FP64 oracle (deposit, r2c, binning)
        import scipy.fft as sfft
        port = O.port()
        cores = port.num_threads()
        t0 = time.perf_counter()
        spec = []
        for sp, sm, mass in ((dm, None, 1.0), (gas, None, 0.19), (spos, smass, 0.0)):
            g = O.zeros_grid(n)
            hp = sp.cpu().numpy() if hasattr(sp, "cpu") else sp
            port.fieldize(box, n, g, hp, sm, mass, 1)
            spec.append(sfft.rfftn(g[:, :, :n], workers=cores))
            del g
        ref = [port.powerspectrum(n, spec[a], spec[b], nrbins, ma, mb)
               for (a, b), (ma, mb) in zip(pairs, pm)]
        auto = {a: ref[i][0] for i, (a, b) in enumerate(pairs) if a == b}
        worst, exact = 0.0, True
        for i, (a, b) in enumerate(pairs):
            pr, cr, _ = ref[i]
            ok = cr > 0
            # cross spectra change sign: relative to the bin's auto-power scale
            scale = np.maximum(np.abs(pr), np.sqrt(np.abs(auto[a] * auto[b])))
            worst = max(worst, float(np.max(np.abs(p[i][ok] - pr[ok]) / scale[ok])))
            exact = exact and bool(np.array_equal(c, cr))
        line["parity"] = {"max_bin_rel_err": worst, "counts_bit_exact": exact,
                          "oracle": "FP64 CIC (oracle port) + FP64 r2c (scipy) + binning, "
                                    "3 auto + 3 cross spectra; cross bins relative to "
                                    "max(|P_ab|, sqrt(P_aa P_bb))",
                          "oracle_s": time.perf_counter() - t0}
    print(json.dumps(line), flush=True)


def box_batch(seed=21, nboxes=16, box=25000.0):
    """The batch of independent boxes: counts log-uniform in [1e5, 3e7], grid
    128^3 or 256^3 per box (seeded), uniform random positions in [0, box)."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(np.log(1e5), np.log(3e7), nboxes)).astype(np.int64)
    grids = rng.choice([128, 256], nboxes)
    return [(int(c), int(g), seed + 1 + i) for i, (c, g) in enumerate(zip(counts, grids))], box


def boxes(args):
    """16 independent boxes per step, each one CIC deposit + r2c + binned auto
    spectrum on its own grid, through one genpk_batch_power call from one host
    thread: every box's work is issued on its own stream (largest first) and
    the call waits once per box for the results.  Timed by wall clock with the
    device synchronised on both sides: at these sizes the launches and the
    result read-backs are part of the cost."""
    import torch
    import genpk_gb300 as gp
    from genpk_gb300 import synth
    from oracle import oracle as O
    batch, box = box_batch()
    mass = 1.0e-2
    nrbins = args.nrbins
    pos = [synth.uniform(c, box, seed=sd, device="cuda") for c, g, sd in batch]
    torch.cuda.synchronize()
    norms = [O.total_mass(c, None, mass) for c, _, _ in batch]
    b = gp.Batch([g for _, g, _ in batch], nrbins)
    b.set_mode(args.batch_mode)

    def step(src):
        return b.power(box, src, norms, mass=mass)

    def timed(src, steps):
        ts = []
        for _ in range(steps):
            torch.cuda.synchronize()
            t = time.perf_counter()
            step(src)
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t)
        return float(np.mean(ts))

    # (the default mode times one call each way after one untuned call each
    # way, then keeps the faster: six calls reach its replayed graph)
    for _ in range(max(args.warmup, 6)):
        res = step(pos)
    launches0 = b.launches
    with ProfiledRange(args.profile_timed):
        t_dev = timed(pos, args.steps)
    launches = (b.launches - launches0) / args.steps
    npart = sum(c for c, _, _ in batch)
    line = {"metric": "particles/s + ms per batch (16 boxes, one auto spectrum each)",
            "value": npart / t_dev, "unit": "particles/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_dev * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded uniform random particles generated on the GPU",
            "config": {"workload": f"16 boxes of uniform random particles, counts log-uniform "
                                   f"in [1e5, 3e7], grid 128^3 or 256^3 per box, L={box:g} "
                                   f"kpc/h, mass {mass:g}, {nrbins} bins",
                       "boxes": [{"particles": c, "grid": g} for c, g, _ in batch],
                       "particles": npart, "host_threads": 1,
                       "l2": f"inputs larger than L2 ({npart * 12 / 1e9:.2f} GB of positions "
                             f"per batch, every box read once per step)",
                       "api": "genpk_batch_power (one call per batch, default mode: per box "
                              "or grouped, whichever its timed trial calls found faster; then "
                              "one replay of a captured CUDA graph per call)",
                       "timing": "wall clock per batch, device synchronised on both sides"},
            "gpu_launches": launches,
            "batch_mode": b.last_mode, "batch_mode_set": args.batch_mode,
            "auto_trials": b.auto_times(),
            "graph_replays": b.graph_replays}
    # the host's launches per timed call: one graph launch once the call is replayed
    line["host_launches_per_step"] = 1 if b.graph_replays >= args.steps else launches

    def leg(mode, graph=True):
        b.set_mode(mode)
        b.use_graph(graph)
        for _ in range(3):
            out = step(pos)
        l0, r0 = b.launches, b.graph_replays
        t = timed(pos, args.steps)
        diff = max(float(np.max(np.abs(out[0][i] - res[0][i]) /
                                np.maximum(np.abs(res[0][i]), 1e-300)))
                   for i in range(len(batch)))
        rec = {"ms_per_step": t * 1e3, "value": npart / t, "unit": "particles/s",
               "gpu_launches": (b.launches - l0) / args.steps,
               "graph_replays": b.graph_replays - r0,
               "max_bin_rel_diff_vs_main": diff,
               "counts_equal_main": bool(np.array_equal(out[1], res[1]))}
        b.use_graph(True)
        return rec

    # Per box: every box its own deposit pass (engine and tile tuned per box),
    # transform and binning, on its own stream.
    line["per_box"] = leg("per_box")
    line["per_box"]["engines"] = [("sorted", "window", "stream")[b.engine(i) - 1]
                                  for i in range(len(batch))]
    line["per_box"]["deposit_tuning"] = [
        tuning_record(b.deposit_config(i), b.deposit_trials(i), line["per_box"]["engines"][i])
        for i in range(len(batch))]
    line["per_box"]["eager_ms_per_step"] = leg("per_box", graph=False)["ms_per_step"]
    # Grouped: the boxes of each grid size share every kernel launch of one
    # grouped sorted-engine pass, one batched transform and one binning x pass.
    line["grouped"] = leg("grouped")
    line["grouped"]["groups"] = [
        {"grid": x["dims"], "boxes": len(x["boxes"]), "tile": list(x["config"]["tile"]),
         "sort_ctas": x["config"]["sort_ctas"],
         "trials": [{"tile": list(t), "sort_ctas": c, "ms": round(ms, 4)}
                    for t, c, ms in x["trials"]]} for x in b.groups()]
    line["grouped"]["eager_ms_per_step"] = leg("grouped", graph=False)["ms_per_step"]
    b.set_mode("auto")
    for _ in range(6):
        step(pos)
    if not args.no_e2e:
        hpos = [p.cpu().pin_memory() for p in pos]
        step(hpos)
        t_e2e = timed(hpos, max(3, min(args.steps, 10)))
        line["e2e"] = {"value": npart / t_e2e, "unit": "particles/s",
                       "h2d_bytes_per_step": npart * 12, "d2h_bytes_per_step": 16 * nrbins * 8,
                       "ms_per_step": t_e2e * 1e3}
        del hpos
    if not args.no_cpu:
        worst, exact = 0.0, True
        pw, cnt, _ = res
        for i, ((c, g, _), p) in enumerate(zip(batch, pos)):
            pr, cr, _, _ = cpu_pipeline(p.cpu().numpy(), box, g, nrbins, mass)
            ok = cr > 0
            worst = max(worst, float(np.max(np.abs(pw[i][ok] - pr[ok]) / np.abs(pr[ok]))))
            exact = exact and bool(np.array_equal(cnt[i], cr))
        line["parity"] = {"max_bin_rel_err": worst, "counts_bit_exact": exact,
                          "oracle": "FP64 CIC (oracle port) + FP64 pocketfft r2c + binning, "
                                    "every box"}
    b.close()
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
        return
    if args.workload == "multispecies":
        multispecies(args)
        return
    if args.workload == "boxes":
        boxes(args)
        return
    import torch
    world, rank, local = dist_setup("nccl")
    torch.cuda.set_device(local)
    import genpk_gb300 as gp
    from oracle import oracle as O

    n, nrbins, box, nside = args.grid, args.nrbins, args.box, args.nside
    npart = nside ** 3
    mass = particle_mass(args)
    m_norm = O.total_mass(npart, None, mass)
    dpos = positions(args, seed=1 + rank, device="cuda")
    torch.cuda.synchronize()
    ctx = gp.Context(n, nrbins, timing=True)
    ctx.set_engine({"auto": 0, "sorted": 1, "window": 2, "stream": 3}[args.engine])
    ctx.set_fft_mode({"auto": 0, "cufft3d": 1}[args.fft])

    flush = (torch.empty(2 * l2_bytes(), dtype=torch.uint8, device="cuda")
             if needs_l2_flush(npart) else None)

    def step(src, flush_l2=True):
        if flush is not None and flush_l2:  # (host input is read over the link anyway)
            flush.fill_(1)
            torch.cuda.synchronize()  # the library's stream does not wait for torch's
        ctx.timing_reset()
        ctx.zero(0)
        ctx.deposit(0, box, src, None, mass)
        p, c, k = ctx.power(0, 0, m_norm, m_norm)
        return p, c, ctx.stage_times()

    for _ in range(args.warmup):
        step(dpos)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier()
    launches0 = ctx.launches
    t0 = time.perf_counter()
    dev_ms, stages = [], {}
    with ProfiledRange(args.profile_timed):
        for _ in range(args.steps):
            p, c, st = step(dpos)
            dev_ms.append(sum(st.values()))
            for key, v in st.items():
                stages[key] = stages.get(key, 0.0) + v
    barrier()
    wall = time.perf_counter() - t0
    launches = ctx.launches - launches0
    clk = clocks.stop()
    ms_step = max_over_ranks(float(np.mean(dev_ms)), world)
    stages = {k: v / args.steps for k, v in stages.items()}
    value = job_throughput(npart, world, ms_step)

    # roofline: the dominant kernel (k_stream_deposit / k_window_deposit, or
    # the sorted engine's whole pass), the deposit pass, and deposit + binning
    pk_, pk_src = peaks()
    peak = float(pk_["hbm_gbs"])
    b_dep, b_bin = algorithmic_bytes(npart, n)
    engine = {1: "sorted", 2: "window", 3: "stream"}.get(ctx.last_engine, "?")
    t_pass = sum(v for k, v in stages.items() if k.startswith(("dep_", "win_", "stream_"))) * 1e-3
    # binning time: the fused x-axis FFT + binning kernel when it ran (it also
    # does the last FFT pass, so this overstates the binning time), else k_bin
    t_bin = (stages.get("xfft_bin", 0.0) + stages.get("bin_kz", 0.0) + stages.get("bin", 0.0)) * 1e-3
    if engine in ("window", "stream"):
        stage = "win_deposit" if engine == "window" else "stream_deposit"
        t_k = stages.get(stage, 0.0) * 1e-3
        kname = "k_window_deposit" if engine == "window" else "k_stream_deposit"
        lattice = args.workload == "zeldovich" and args.order == "lattice"
        traffic = NCU_TRAFFIC.get((kname, nside, n)) if lattice else None
    else:
        t_k = t_pass
        kname = "deposit pass (sorted engine: all its kernels)"
        traffic = None
    ach = b_dep / t_k / 1e9
    ach_bin = b_bin / t_bin / 1e9 if t_bin > 0 else None
    roofline = {"kernel": kname, "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                "frac": ach / peak, "peak_source": pk_src, "traffic": traffic,
                "algorithmic_bytes": b_dep,
                "note": "achieved = algorithmic bytes (particles read once + grid written once) "
                        "/ mean CUDA-event time of the kernel; peak = measured copy bandwidth",
                "deposit_pass": {"ms": t_pass * 1e3, "frac": b_dep / t_pass / 1e9 / peak},
                "bin": {"kernel": "k_xfft (x-axis FFT pass + binning)" if "xfft_bin" in stages
                        else "k_bin_kz (kz-major binning)" if "bin_kz" in stages
                        else "k_bin", "achieved": ach_bin,
                        "frac": (ach_bin / peak) if ach_bin else None, "algorithmic_bytes": b_bin},
                "deposit_plus_bin_frac": (b_dep + b_bin) / (t_pass + t_bin) / 1e9 / peak}

    line = {"metric": METRIC, "value": value, "unit": "particles/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": ("synthetic: seeded uniform random positions generated on the GPU"
                     if args.workload == "uniform"
                     else "synthetic: seeded Zel'dovich lattice generated on the GPU"),
            "config": config_dict(args, npart), "ms_per_spectrum": ms_step,
            "wall_ms_per_step": wall / args.steps * 1e3,
            "stages_ms": {k: round(v, 5) for k, v in stages.items()},
            "roofline": roofline, "gpu_launches": launches, "clocks": clk,
            "deposit_engine": engine,
            "deposit_tuning": tuning_record(ctx.deposit_config(), ctx.deposit_trials(), engine)}

    # end to end through the C ABI from pinned host memory (before the adjoint
    # section: after it, the host-link reads of a newly pinned buffer were
    # sometimes slower, 14-23 ms against 9.0 ms per step)
    if not args.no_e2e:
        hpos = dpos.cpu().pin_memory()
        for _ in range(2):
            step(hpos, flush_l2=False)
        torch.cuda.synchronize()
        e2e_t = []
        for _ in range(max(3, min(args.steps, 20))):
            t1 = time.perf_counter()
            step(hpos, flush_l2=False)
            e2e_t.append(time.perf_counter() - t1)
        e_ms = max_over_ranks(float(np.mean(e2e_t)) * 1e3, world)
        line["e2e"] = {"value": job_throughput(npart, world, e_ms), "unit": "particles/s",
                       "h2d_bytes_per_step": npart * 12, "d2h_bytes_per_step": nrbins * 8,
                       "ms_per_step": e_ms, "ms_min": min(e2e_t) * 1e3,
                       "ms_max": max(e2e_t) * 1e3}
        del hpos
        # the same from pageable host memory handed over in chunks of at most 2^26
        # particles, as the reference's reader calls fieldize (read_fieldize.cpp:45-93)
        hp = dpos.cpu().numpy()
        chunk = 1 << 26

        def step_pageable():
            ctx.timing_reset()
            ctx.zero(0)
            for a in range(0, npart, chunk):
                ctx.deposit(0, box, hp[a:a + chunk], None, mass)
            ctx.power(0, 0, m_norm, m_norm)

        for _ in range(2):
            step_pageable()
        pg_t = []
        for _ in range(max(3, min(args.steps, 10))):
            t1 = time.perf_counter()
            step_pageable()
            pg_t.append(time.perf_counter() - t1)
        p_ms = max_over_ranks(float(np.mean(pg_t)) * 1e3, world)
        line["e2e_pageable"] = {"value": job_throughput(npart, world, p_ms), "unit": "particles/s",
                                "h2d_bytes_per_step": npart * 12,
                                "d2h_bytes_per_step": nrbins * 8, "ms_per_step": p_ms,
                                "chunk_particles": chunk,
                                "vs_pinned": p_ms / e_ms}
        del hp

    # forward + adjoint / forward
    if not args.no_adjoint:
        g = np.linspace(1.0, -1.0, nrbins) / np.maximum(np.abs(p), 1e-30)
        gpos = torch.empty((npart, 3), device="cuda", dtype=torch.float32)
        fwd, adj, adj_rc = [], [], []
        adj_st, rc_st = {}, {}
        for it in range(4):
            _, _, st = step(dpos)
            ctx.timing_reset()
            ctx.adjoint(0, box, dpos, g, m_norm, mass=mass, grad_pos=gpos)
            sa = ctx.stage_times()
            ctx.timing_reset()
            ctx.adjoint(0, box, dpos, g, m_norm, mass=mass, grad_pos=gpos, recompute=True)
            sr = ctx.stage_times()
            if it:
                fwd.append(sum(st.values()))
                adj.append(sum(sa.values()))
                adj_rc.append(sum(sr.values()))
                for key, v in sa.items():
                    adj_st[key] = adj_st.get(key, 0.0) + v / 3
                for key, v in sr.items():
                    rc_st[key] = rc_st.get(key, 0.0) + v / 3
        f_ms = float(np.mean(fwd))
        line["fwd_adj_ratio"] = (f_ms + float(np.mean(adj))) / f_ms
        line["fwd_adj_recompute_ratio"] = (f_ms + float(np.mean(adj_rc))) / f_ms
        line["adjoint_ms"] = float(np.mean(adj))
        line["adjoint_stages_ms"] = {k: round(v, 5) for k, v in adj_st.items()}
        line["adjoint_recompute_stages_ms"] = {k: round(v, 5) for k, v in rc_st.items()}
        del gpos

    # FP64 oracle on the same particles (rank 0): parity at full size + CPU baseline
    if rank == 0 and not args.no_cpu:
        hp = dpos.cpu().numpy()
        # twice, timing the second: the first pays the host threads' start and
        # first touches, as the reference arm's warm-up step does
        cpu_pipeline(hp, box, n, nrbins, mass)
        pr, cr, t, nd = cpu_pipeline(hp, box, n, nrbins, mass)
        ok = cr > 0
        rel = np.abs(p[ok] - pr[ok]) / np.abs(pr[ok])
        line["parity"] = {"max_bin_rel_err": float(rel.max()),
                          "counts_bit_exact": bool(np.array_equal(c, cr)),
                          "oracle": "FP64 CIC (oracle port) + FP64 pocketfft r2c + binning"}
        tcpu = t["deposit"] + t["fft"] + t["bin"]
        line["cpu_baseline"] = {"value": npart / tcpu, "unit": "particles/s",
                                "cores": t["cores"], "kind": "port",
                                "sample": f"the full workload ({nd} particles), the second of "
                                          f"two runs: deposit "
                                          f"{t['deposit']:.2f} s, FP64 r2c {t['fft']:.2f} s, "
                                          f"binning {t['bin']:.2f} s"}
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
