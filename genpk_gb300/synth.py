"""Seeded synthetic particle sets for tests and benchmarks.

The reference names no public dataset; these generators produce inputs with
the shapes, sizes and value distributions of the benchmark workloads:

* ``uniform``    i.i.d. uniform float32 positions in [0, box).
* ``zeldovich``  a regular lattice displaced by the Zel'dovich approximation
                 from a Gaussian random field with P(k) = A k^-2 exp(-(k/k_c)^2),
                 k_c = kc_frac * k_Nyquist, scaled so the RMS 3-D displacement
                 is ``rms`` lattice spacings, wrapped periodically, stored as
                 float32 in lattice order (x slowest).
* ``lognormal``  particles Poisson-sampled from a lognormal density
                 exp(sigma g - sigma^2/2) of a Gaussian field g, jittered
                 uniformly inside their cell; optional lognormal masses.

numpy implementations run anywhere; ``device="cuda"`` builds the same
construction with torch on the GPU (used for the large benchmark sets).
"""
from __future__ import annotations

import numpy as np


def uniform(n: int, box: float, seed: int = 1, device: str = "cpu"):
    if device != "cpu":
        import torch
        g = torch.Generator(device=device).manual_seed(seed)
        return (torch.rand((n, 3), generator=g, device=device, dtype=torch.float32) * box).clamp_(
            max=np.nextafter(np.float32(box), np.float32(0)))
    rng = np.random.default_rng(seed)
    pos = (rng.random((n, 3)) * box).astype(np.float32)
    pos[pos >= np.float32(box)] = np.nextafter(np.float32(box), np.float32(0))
    return pos


def _kgrid_np(n):
    k = np.fft.fftfreq(n) * n
    kz = np.arange(n // 2 + 1, dtype=np.float64)
    return k, kz


def zeldovich(nside: int, box: float, seed: int = 1, rms: float = 0.3, kc_frac: float = 0.5,
              amplitude: float = 1.0, device: str = "cpu"):
    """nside^3 particles, lattice + Zel'dovich displacement (see module doc)."""
    if device != "cpu":
        return _zeldovich_torch(nside, box, seed, rms, kc_frac, amplitude, device)
    rng = np.random.default_rng(seed)
    n = nside
    white = rng.standard_normal((n, n, n))
    wk = np.fft.rfftn(white)
    k, kz = _kgrid_np(n)
    kx, ky, kzz = np.meshgrid(k, k, kz, indexing="ij")
    k2 = kx * kx + ky * ky + kzz * kzz
    kc = kc_frac * (n / 2)
    with np.errstate(divide="ignore", invalid="ignore"):
        amp = np.where(k2 > 0, np.sqrt(k2 ** -1.0 * np.exp(-k2 / kc ** 2)), 0.0)
        dk = wk * amp
        # psi_k = i k / k^2 delta_k
        inv = np.where(k2 > 0, 1.0 / k2, 0.0)
    psi = [np.fft.irfftn(1j * kk * inv * dk, s=(n, n, n), axes=(0, 1, 2)) for kk in (kx, ky, kzz)]
    cur = np.sqrt(np.mean(psi[0] ** 2 + psi[1] ** 2 + psi[2] ** 2))
    spacing = box / n
    scale = amplitude * rms * spacing / cur
    idx = np.arange(n, dtype=np.float64) * spacing
    lx, ly, lz = np.meshgrid(idx, idx, idx, indexing="ij")
    pos = np.stack([lx + scale * psi[0], ly + scale * psi[1], lz + scale * psi[2]], axis=-1)
    pos = np.mod(pos, box).reshape(-1, 3).astype(np.float32)
    pos[pos >= np.float32(box)] = 0.0
    return pos


def _zeldovich_torch(nside, box, seed, rms, kc_frac, amplitude, device):
    import torch
    n = nside
    g = torch.Generator(device=device).manual_seed(seed)
    white = torch.randn((n, n, n), generator=g, device=device, dtype=torch.float32)
    wk = torch.fft.rfftn(white)
    del white
    k = torch.fft.fftfreq(n, device=device, dtype=torch.float32) * n
    kz = torch.arange(n // 2 + 1, device=device, dtype=torch.float32)
    kc = kc_frac * (n / 2)
    spacing = box / n
    out = torch.empty((n, n, n, 3), device=device, dtype=torch.float32)
    k2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + kz[None, None, :] ** 2
    amp = torch.where(k2 > 0, torch.rsqrt(k2.clamp(min=1e-30)) * torch.exp(-0.5 * k2 / kc ** 2),
                      torch.zeros((), device=device))
    inv = torch.where(k2 > 0, 1.0 / k2.clamp(min=1e-30), torch.zeros((), device=device))
    dk = wk * (amp * inv)
    del wk, amp, inv, k2
    sumsq = 0.0
    comps = []
    for axis in range(3):
        if axis == 0:
            kk = k[:, None, None]
        elif axis == 1:
            kk = k[None, :, None]
        else:
            kk = kz[None, None, :]
        psi = torch.fft.irfftn(1j * kk * dk, s=(n, n, n))
        sumsq += float((psi.double() ** 2).mean())
        comps.append(psi)
    scale = amplitude * rms * spacing / np.sqrt(sumsq)
    idx = torch.arange(n, device=device, dtype=torch.float64) * spacing
    lat = [idx[:, None, None], idx[None, :, None], idx[None, None, :]]
    for axis in range(3):
        p = (lat[axis] + scale * comps[axis].double()).remainder(box)
        out[..., axis] = p.float()
    comps.clear()
    out[out >= box] = 0.0
    return out.reshape(-1, 3)


def lognormal(n_mean: int, box: float, ngrid: int, sigma: float = 1.5, seed: int = 1,
              mass_mu=None, mass_sigma=None):
    """~n_mean particles from a lognormal field on an ngrid^3 mesh (numpy).
    Returns (pos float32 [n,3], masses float32 [n] or None)."""
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((ngrid,) * 3)
    gk = np.fft.rfftn(g)
    k, kz = _kgrid_np(ngrid)
    k2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + kz[None, None, :] ** 2
    kc = 0.25 * ngrid
    gk *= np.exp(-0.5 * k2 / kc ** 2)
    g = np.fft.irfftn(gk, s=(ngrid,) * 3, axes=(0, 1, 2))
    g /= g.std()
    rho = np.exp(sigma * g - 0.5 * sigma ** 2)
    lam = rho * (n_mean / rho.sum())
    counts = rng.poisson(lam).reshape(-1)
    cells = np.repeat(np.arange(counts.size), counts)
    ix, iy, iz = np.unravel_index(cells, (ngrid,) * 3)
    cell = box / ngrid
    pos = np.stack([ix, iy, iz], axis=-1) + rng.random((cells.size, 3))
    pos = (pos * cell).astype(np.float32)
    pos[pos >= np.float32(box)] = 0.0
    masses = None
    if mass_mu is not None:
        masses = rng.lognormal(mass_mu, mass_sigma, cells.size).astype(np.float32)
    return pos, masses


def write_gadget2(base: str, pos_by_type: dict, masses_by_type: dict, box: float,
                  nfiles: int = 1, time: float = 1.0, redshift: float = 0.0,
                  hubble: float = 0.7, omega0: float = 0.3, extra_blocks: bool = True):
    """Write a Gadget-2 format-II snapshot: `base` (nfiles = 1) or base.0 ...
    base.(nfiles-1), each type's particles split into contiguous parts.

    pos_by_type: {type: float32 [n, 3]}.  masses_by_type: {type: float (the
    header mass table) or float32 [n] (the MASS block; header mass 0)}.
    Each block is a label record (int32 8, name, int32 size + 8, int32 8) and
    a data record (int32 size, data, int32 size); HEAD is the 256-byte
    io_header.  extra_blocks adds VEL and ID blocks, which readers skip."""
    import struct

    ntypes = 6
    counts = [len(pos_by_type.get(t, ())) for t in range(ntypes)]
    table = [0.0 if not np.isscalar(masses_by_type.get(t, 0.0)) else float(masses_by_type.get(t, 0.0))
             for t in range(ntypes)]
    paths = [base] if nfiles == 1 else [f"{base}.{i}" for i in range(nfiles)]

    def split(n, i):
        edges = [n * k // nfiles for k in range(nfiles + 1)]
        return edges[i], edges[i + 1]

    def block(f, name, data: bytes):
        f.write(struct.pack("<i4sii", 8, name.encode(), len(data) + 8, 8))
        f.write(struct.pack("<i", len(data)))
        f.write(data)
        f.write(struct.pack("<i", len(data)))

    for i, path in enumerate(paths):
        npart = []
        pos_parts, mass_parts, vel_parts = [], [], []
        for t in range(ntypes):
            lo, hi = split(counts[t], i)
            npart.append(hi - lo)
            if hi > lo:
                p = np.ascontiguousarray(pos_by_type[t][lo:hi], dtype=np.float32)
                pos_parts.append(p)
                vel_parts.append(np.zeros_like(p))
                if table[t] == 0.0:
                    mass_parts.append(np.asarray(masses_by_type[t][lo:hi], dtype=np.float32))
        head = struct.pack("<6I6dddii6Iiiddddii6I", *npart, *table, time, redshift, 0, 0,
                           *[c & 0xFFFFFFFF for c in counts], 0, nfiles, box, omega0,
                           1.0 - omega0, hubble, 0, 0, *[c >> 32 for c in counts])
        head = head + b"\0" * (256 - len(head))
        with open(path, "wb") as f:
            block(f, "HEAD", head)
            block(f, "POS ", b"".join(p.tobytes() for p in pos_parts))
            if extra_blocks:
                block(f, "VEL ", b"".join(v.tobytes() for v in vel_parts))
                ids = np.arange(sum(npart), dtype=np.uint32)
                block(f, "ID  ", ids.tobytes())
            if mass_parts:
                block(f, "MASS", b"".join(m.tobytes() for m in mass_parts))
    return paths


def write_bigfile(root: str, pos_by_type: dict, masses_by_type: dict, box: float,
                  time: float = 1.0, hubble: float = 0.7, omega0: float = 0.3,
                  nfiles: int = 2, pos_dtype: str = "<f8", mass_dtype: str = "<f4"):
    """Write a BigFile snapshot directory (the layout MP-Gadget writes): a
    "Header" block whose attr-v2 file holds TotNumPart, MassTable, Time,
    HubbleParam, Omega0 and BoxSize, and per type the columns
    "<type>/Position" (pos_dtype x 3) and, where masses_by_type[type] is an
    array (MassTable 0), "<type>/Mass" (mass_dtype), each split over nfiles
    data files named 000000, 000001, ...

    pos_by_type: {type: float32 [n, 3]}.  masses_by_type: {type: float (the
    MassTable entry) or float32 [n]}."""
    import os

    def attr_line(name, dtype, values):
        arr = np.asarray(values, dtype=np.dtype(dtype))
        human = " ".join(repr(v) for v in arr.tolist())
        return f"{name} {dtype} {arr.size} {arr.tobytes().hex().upper()} #HUMANE [ {human} ]\n"

    def column(name, data, dtype, nmemb):
        d = os.path.join(root, name)
        os.makedirs(d, exist_ok=True)
        arr = np.ascontiguousarray(np.asarray(data).reshape(-1, nmemb).astype(np.dtype(dtype)))
        n = len(arr)
        edges = [n * k // nfiles for k in range(nfiles + 1)]
        lines = [f"DTYPE: {dtype}\n", f"NMEMB: {nmemb}\n", f"NFILE: {nfiles}\n"]
        for f in range(nfiles):
            part = arr[edges[f]:edges[f + 1]]
            with open(os.path.join(d, f"{f:06X}"), "wb") as fh:
                fh.write(part.tobytes())
            lines.append(f"{f:06X}: {len(part)} : 0 : 0\n")
        with open(os.path.join(d, "header"), "w") as fh:
            fh.writelines(lines)
        with open(os.path.join(d, "attr-v2"), "w") as fh:
            fh.write("")

    ntypes = 6
    counts = [len(pos_by_type.get(t, ())) for t in range(ntypes)]
    table = [0.0 if not np.isscalar(masses_by_type.get(t, 0.0)) else float(masses_by_type.get(t, 0.0))
             for t in range(ntypes)]
    hdir = os.path.join(root, "Header")
    os.makedirs(hdir, exist_ok=True)
    with open(os.path.join(hdir, "header"), "w") as fh:
        fh.write("DTYPE: <f8\nNMEMB: 1\nNFILE: 0\n")
    with open(os.path.join(hdir, "attr-v2"), "w") as fh:
        fh.write(attr_line("TotNumPart", "<u8", counts))
        fh.write(attr_line("MassTable", "<f8", table))
        fh.write(attr_line("Time", "<f8", [time]))
        fh.write(attr_line("HubbleParam", "<f8", [hubble]))
        fh.write(attr_line("Omega0", "<f8", [omega0]))
        fh.write(attr_line("BoxSize", "<f8", [box]))
    for t in range(ntypes):
        if counts[t] == 0:
            continue
        column(f"{t}/Position", pos_by_type[t], pos_dtype, 3)
        if table[t] == 0.0:
            column(f"{t}/Mass", masses_by_type[t], mass_dtype, 1)
    return root
