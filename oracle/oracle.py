"""FP64 CPU oracle for GenPK's power-spectrum hot path.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and
bench.py (cpu_baseline leg and the ``--impl reference`` arm) as the checker;
the product package (genpk_gb300) never imports it.

Two CPU implementations live behind this module:

* ``port``  -- genpk_oracle.c, this repository's restatement of
  fieldize.cpp:46-133 and powerspectrum.c:35-111, built by ``make port``.
* ``ref``   -- the reference's own fieldize.cpp + powerspectrum.c compiled from
  the reference tree with shim headers (``make ref``).  It only exists where
  the reference sources do; tests use it to pin the port.

The FFT between deposit and binning is numpy's FP64 pocketfft ``rfftn``,
which follows FFTW's r2c convention (unnormalised forward transform, e^{-ikx},
N x N x (N/2+1) output).  FFTW itself (gen-pk.cpp:186-193,233) is not installed.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libgenpk_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libgenpk_ref.so")
# The reference source tree that oracle/_ref was compiled from: written by
# build(ref_dir=...) beside the library, or named by GENPK_REFERENCE_DIR.  No
# default: where neither exists, the reference build and its fixtures are skipped.
REF_DIR_RECORD = os.path.join(HERE, "_ref", "source_dir")

_f64p = ctypes.POINTER(ctypes.c_double)
_f32p = ctypes.POINTER(ctypes.c_float)
_i32p = ctypes.POINTER(ctypes.c_int)


def reference_tree():
    """The reference source tree (GENPK_REFERENCE_DIR, else the one the
    reference build was made from), or None."""
    d = os.environ.get("GENPK_REFERENCE_DIR")
    if not d and os.path.exists(REF_DIR_RECORD):
        with open(REF_DIR_RECORD) as f:
            d = f.read().strip()
    if d and os.path.exists(os.path.join(d, "fieldize.cpp")):
        return d
    return None


def build(ref_dir=None) -> None:
    """Compile the port (always) and, given the reference's source tree
    (ref_dir, or GENPK_REFERENCE_DIR), the reference build from it."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    d = ref_dir or os.environ.get("GENPK_REFERENCE_DIR")
    if d and os.path.exists(os.path.join(d, "fieldize.cpp")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFDIR={d}"], check=True)
        with open(REF_DIR_RECORD, "w") as f:
            f.write(os.path.abspath(d) + "\n")


def _bind(lib, name, restype, argtypes):
    fn = getattr(lib, name)
    fn.restype = restype
    fn.argtypes = argtypes
    return fn


class _Impl:
    """ctypes view of one CPU implementation (port or reference build)."""

    def __init__(self, path: str, fieldize_sym: str, power_sym: str, invwin_sym: str):
        self.path = path
        lib = ctypes.CDLL(path)
        self.lib = lib
        self._fieldize = _bind(lib, fieldize_sym, ctypes.c_int,
                               [ctypes.c_double, ctypes.c_int, _f64p, ctypes.c_int64,
                                _f32p, _f32p, ctypes.c_double, ctypes.c_int])
        self._power = _bind(lib, power_sym, ctypes.c_int,
                            [ctypes.c_int64, _f64p, _f64p, ctypes.c_int, _f64p, _i32p,
                             _f64p, ctypes.c_double, ctypes.c_double])
        self._invwindow = _bind(lib, invwin_sym, ctypes.c_double,
                                [ctypes.c_int64] * 4)

    def fieldize(self, boxsize, dims, out, pos, masses=None, mass=0.0, extra=1):
        """+= CIC deposit into ``out`` (float64, padded layout), like fieldize.cpp:46."""
        assert out.dtype == np.float64 and out.flags.c_contiguous
        pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
        mp = None
        if masses is not None:
            masses = np.ascontiguousarray(masses, dtype=np.float32)
            mp = masses.ctypes.data_as(_f32p)
        rc = self._fieldize(float(boxsize), int(dims), out.ctypes.data_as(_f64p),
                            pos.shape[0], pos.ctypes.data_as(_f32p), mp, float(mass), int(extra))
        assert rc == 0
        return out

    def invwindow(self, kx, ky, kz, n):
        return self._invwindow(int(kx), int(ky), int(kz), int(n))

    def powerspectrum(self, dims, f1, f2, nrbins, m1, m2):
        """Bin the half-complex spectra f1, f2 (complex128) like powerspectrum.c:35."""
        f1 = np.ascontiguousarray(f1, dtype=np.complex128)
        f2 = f1 if f2 is None else np.ascontiguousarray(f2, dtype=np.complex128)
        power = np.zeros(nrbins)
        count = np.zeros(nrbins, dtype=np.int32)
        keffs = np.zeros(nrbins)
        rc = self._power(int(dims), f1.ctypes.data_as(_f64p), f2.ctypes.data_as(_f64p),
                         int(nrbins), power.ctypes.data_as(_f64p), count.ctypes.data_as(_i32p),
                         keffs.ctypes.data_as(_f64p), float(m1), float(m2))
        assert rc == 0
        return power, count, keffs


_PORT = None
_REF = None


def port() -> _Impl:
    """The C restatement (always available once built)."""
    global _PORT
    if _PORT is None:
        if not os.path.exists(PORT_LIB):
            build()
        _PORT = _Impl(PORT_LIB, "oracle_fieldize", "oracle_powerspectrum", "oracle_invwindow")
        lib = _PORT.lib
        _PORT.gather = _bind(lib, "oracle_cic_gather", ctypes.c_int,
                             [ctypes.c_double, ctypes.c_int, _f64p, ctypes.c_int64, _f32p,
                              _f32p, ctypes.c_double, _f64p, _f64p])
        _PORT.bin_of = _bind(lib, "oracle_bin_of", ctypes.c_int64,
                             [ctypes.c_int64, ctypes.c_int64, ctypes.c_int])
        _PORT.num_threads = _bind(lib, "oracle_num_threads", ctypes.c_int, [])
        _PORT.onedinvwindow = _bind(lib, "oracle_onedinvwindow", ctypes.c_double,
                                    [ctypes.c_int64, ctypes.c_int64])
    return _PORT


def ref():
    """The reference's own code compiled here, or None where it cannot be built."""
    global _REF
    if _REF is None:
        if not os.path.exists(REF_LIB):
            tree = reference_tree()
            if tree is None:
                return None
            build(ref_dir=tree)
        _REF = _Impl(REF_LIB, "ref_fieldize", "powerspectrum", "invwindow")
    return _REF


# ---------------------------------------------------------------------------
# Grid helpers and the full FP64 pipeline
# ---------------------------------------------------------------------------

def padded_len(dims: int) -> int:
    """Row length of the in-place r2c grid: 2*(dims/2+1) (gen-pk.cpp:176)."""
    return 2 * (dims // 2 + 1)


def zeros_grid(dims: int) -> np.ndarray:
    return np.zeros((dims, dims, padded_len(dims)), dtype=np.float64)


def rfft_padded(grid: np.ndarray, workers=None) -> np.ndarray:
    """FP64 r2c of the real part of a padded grid -> (dims, dims, dims/2+1) complex128.
    workers: threads for scipy's pocketfft (large grids); None: numpy's."""
    dims = grid.shape[0]
    if workers:
        import scipy.fft as sfft
        return sfft.rfftn(grid[:, :, :dims], axes=(0, 1, 2), workers=workers)
    return np.fft.rfftn(grid[:, :, :dims], axes=(0, 1, 2))


def irfft_unnormalised(h: np.ndarray, dims: int) -> np.ndarray:
    """Unnormalised c2r (e^{+ikx}) of a half-complex array -> real (dims,)*3."""
    return np.fft.irfftn(h, s=(dims, dims, dims), axes=(0, 1, 2)) * float(dims) ** 3


def total_mass(n: int, masses=None, mass: float = 0.0, quirk: float = 1.0) -> float:
    """Mass normalisation as gen-pk computes it: sum of masses plus the +1 that
    read_fieldize adds per call (read_fieldize.cpp:79-94)."""
    m = float(np.sum(masses, dtype=np.float64)) if masses is not None else mass * n
    return m + quirk


def deposit(pos, boxsize, dims, masses=None, mass=1.0, impl=None) -> np.ndarray:
    impl = impl or port()
    g = zeros_grid(dims)
    impl.fieldize(boxsize, dims, g, pos, masses, mass, 1)
    return g


def pk(pos, boxsize, dims, nrbins, masses=None, mass=1.0, m_norm=None, impl=None,
       workers=None):
    """Deposit + FP64 r2c + binning: the P(k) gen-pk writes for one species."""
    impl = impl or port()
    g = deposit(pos, boxsize, dims, masses, mass, impl)
    f = rfft_padded(g, workers)
    del g
    if m_norm is None:
        m_norm = total_mass(len(pos), masses, mass)
    return impl.powerspectrum(dims, f, f, nrbins, m_norm, m_norm)


def cross_pk(fa, fb, dims, nrbins, ma, mb, impl=None):
    impl = impl or port()
    return impl.powerspectrum(dims, fa, fb, nrbins, ma, mb)


# ---------------------------------------------------------------------------
# FP64 reference gradient of a P(k) loss (no reference counterpart)
# ---------------------------------------------------------------------------

def kval(dims: int) -> np.ndarray:
    i = np.arange(dims)
    return np.where(i <= dims // 2, i, i - dims)


def mode_tables(dims: int, nrbins: int):
    """Per-mode bin index, reference weight c_m and invwindow^2 V_m on the
    half-complex grid, evaluated with the oracle's own expressions."""
    impl = port()
    half = dims // 2
    kv = kval(dims)
    kz = np.arange(half + 1)
    kk2 = (kv[:, None, None] ** 2 + kv[None, :, None] ** 2 + kz[None, None, :] ** 2)
    bins = bin_lut(dims, nrbins)[kk2]
    c = np.full(kk2.shape, 2.0)
    c[:, :, 0] = 1.0
    c[:, :, half] = 1.0
    c[0, 0, 0] = 0.0
    bins[0, 0, 0] = -1
    iw1 = np.array([impl.onedinvwindow(int(k), dims) for k in kv], dtype=np.float32)
    prod = (iw1[:, None, None] * iw1[None, :, None]).astype(np.float32) * iw1[None, None, :half + 1]
    v = prod.astype(np.float32).astype(np.float64) ** 4
    return bins, c, v


def reference_gradient(pos, boxsize, dims, nrbins, gbin, masses=None, mass=1.0,
                       m_norm=None, quirk=1.0):
    """FP64 gradient of L with respect to positions and masses, given
    gbin = dL/dP_b for the auto spectrum of one species.

    Forward: P_b = S_b / (M^2 C_b), S_b = sum_{m in b} c_m |F_m|^2 V_m,
    F = r2c(rho), M = sum(masses) + quirk.
    dL/drho(x) = sum_m (2 g_b c_m V_m / (M^2 C_b)) Re(F_m e^{ikx}), evaluated as
    an unnormalised c2r of H_m = 2 g_b V_m F_m c_m / (M^2 C_b mult_m) where
    mult_m is the c2r multiplicity of the mode (1 on self-conjugate planes).
    Returns (gpos [n,3], gmass [n] or None, dL/dM)."""
    impl = port()
    n = len(pos)
    if m_norm is None:
        m_norm = total_mass(n, masses, mass, quirk)
    g = deposit(pos, boxsize, dims, masses, mass, impl)
    f = rfft_padded(g)
    power, count, _ = impl.powerspectrum(dims, f, f, nrbins, m_norm, m_norm)
    bins, c, v = mode_tables(dims, nrbins)
    half = dims // 2
    mult = np.full(c.shape, 2.0)
    mult[:, :, 0] = 1.0
    if dims % 2 == 0:
        mult[:, :, half] = 1.0
    cb = count.astype(np.float64)
    gb = np.asarray(gbin, dtype=np.float64)
    scale = np.zeros(bins.shape)
    ok = bins >= 0
    scale[ok] = 2.0 * gb[bins[ok]] * v[ok] * c[ok] / (m_norm ** 2 * cb[bins[ok]] * mult[ok])
    h = scale * f
    drho = irfft_unnormalised(h, dims)
    gpad = zeros_grid(dims)
    gpad[:, :, :dims] = drho
    gpos = np.zeros((n, 3))
    gw = np.zeros(n)
    pos32 = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
    mp = None
    if masses is not None:
        masses = np.ascontiguousarray(masses, dtype=np.float32)
        mp = masses.ctypes.data_as(_f32p)
    impl.gather(float(boxsize), int(dims), gpad.ctypes.data_as(_f64p), n,
                pos32.ctypes.data_as(_f32p), mp, float(mass),
                gpos.ctypes.data_as(_f64p), gw.ctypes.data_as(_f64p))
    dl_dm = float(np.sum(gb * (-2.0 * power / m_norm)))
    gmass = gw + dl_dm if masses is not None else None
    return gpos, gmass, dl_dm


def bin_lut(dims: int, nrbins: int) -> np.ndarray:
    """Bin of every integer |k|^2 from 0 to 3 (dims/2)^2 (-1 for 0), from the
    port's restatement of the reference's bin expression (powerspectrum.c:38,66)."""
    impl = port()
    half = dims // 2
    top = 3 * half * half
    lut = np.array([impl.bin_of(v, dims, nrbins) for v in range(1, top + 1)], dtype=np.int64)
    return np.concatenate([[-1], lut])


def cic_gather_sample(drho, pos, boxsize, masses=None, mass=1.0):
    """oracle_cic_gather for a few particles, in numpy: the CIC-weighted value
    of the real grid drho [dims]^3 at each particle (the mass gradient before
    dL/dM) and its position derivative m * units * sum (+-1) prod_{e!=a} w_e."""
    dims = drho.shape[0]
    units = dims / boxsize
    x = np.asarray(pos, dtype=np.float32).reshape(-1, 3).astype(np.float64) * units
    f = np.floor(x)
    d = x - f
    t = 1.0 - d
    lo = np.mod(f.astype(np.int64), dims)
    hi = np.mod(f.astype(np.int64) + 1, dims)
    m = (np.asarray(masses, dtype=np.float32).astype(np.float64) if masses is not None
         else np.full(len(x), float(mass)))
    sw = np.zeros(len(x))
    dg = np.zeros((len(x), 3))
    for c in range(8):
        b = [(c >> a) & 1 for a in range(3)]
        w = [d[:, a] if b[a] else t[:, a] for a in range(3)]
        idx = [hi[:, a] if b[a] else lo[:, a] for a in range(3)]
        gv = drho[idx[0], idx[1], idx[2]]
        sw += w[0] * w[1] * w[2] * gv
        for a in range(3):
            sgn = 1.0 if b[a] else -1.0
            other = np.ones(len(x))
            for e in range(3):
                if e != a:
                    other = other * w[e]
            dg[:, a] += sgn * other * gv
    return dg * (m * units)[:, None], sw


def reference_gradient_sampled(pos, boxsize, dims, nrbins, gbin, sample, masses=None,
                               mass=1.0, m_norm=None, quirk=1.0, workers=None):
    """reference_gradient's mathematics for grids too large for its
    full-size temporaries: the FP64 deposit and r2c of all particles, the
    mode gradient applied one x-plane at a time, the unnormalised c2r, and
    the CIC gather at the particles `sample` only.  Also returns the FP64
    forward of the same run.
    Returns (power, count, keffs, gpos [len(sample), 3], gmass or None, dL/dM)."""
    impl = port()
    n = len(pos)
    if m_norm is None:
        m_norm = total_mass(n, masses, mass, quirk)
    f = rfft_padded(deposit(pos, boxsize, dims, masses, mass, impl), workers)
    power, count, keffs = impl.powerspectrum(dims, f, f, nrbins, m_norm, m_norm)
    half = dims // 2
    kv = kval(dims)
    kz = np.arange(half + 1)
    lut = bin_lut(dims, nrbins)
    iw1 = np.array([impl.onedinvwindow(int(k), dims) for k in kv], dtype=np.float32)
    c = np.full((dims, half + 1), 2.0)
    c[:, 0] = 1.0
    c[:, half] = 1.0
    mult = np.full((dims, half + 1), 2.0)
    mult[:, 0] = 1.0
    if dims % 2 == 0:
        mult[:, half] = 1.0
    cb = count.astype(np.float64)
    gb = np.asarray(gbin, dtype=np.float64)
    coef = np.zeros(nrbins)
    okb = cb > 0
    coef[okb] = 2.0 * gb[okb] / (m_norm ** 2 * cb[okb])
    for i in range(dims):
        kk2 = kv[i] ** 2 + kv[:, None] ** 2 + kz[None, :] ** 2
        bins = lut[kk2]
        ci = c.copy()
        if i == 0:
            ci[0, 0] = 0.0
        prod = (iw1[i] * iw1[:, None]).astype(np.float32) * iw1[None, :half + 1]
        v = prod.astype(np.float32).astype(np.float64) ** 4
        scale = np.where(bins >= 0, coef[np.maximum(bins, 0)], 0.0) * v * ci / mult
        f[i] *= scale
    import scipy.fft as sfft
    drho = sfft.irfftn(f, s=(dims, dims, dims), axes=(0, 1, 2), workers=workers or 1)
    drho *= float(dims) ** 3
    del f
    sp = np.asarray(pos, dtype=np.float32).reshape(-1, 3)[sample]
    sm = np.asarray(masses, dtype=np.float32)[sample] if masses is not None else None
    gpos, gw = cic_gather_sample(drho, sp, boxsize, sm, mass)
    dl_dm = float(np.sum(gb * (-2.0 * power / m_norm)))
    gmass = gw + dl_dm if masses is not None else None
    return power, count, keffs, gpos, gmass, dl_dm
