"""Python mirror of GenPK's hot-path interface, running on the GB300 library.

Module-level functions keep the reference's names, argument meaning and
return conventions:

  fieldize(boxsize, dims, out, pos, masses, mass, extra)   fieldize.cpp:46
  invwindow(kx, ky, kz, n)                                  fieldize.cpp:125
  powerspectrum(dims, outfield, outfield2, nrbins, M1, M2)  powerspectrum.c:35

``Context`` is the device-resident interface the C ABI exposes (grids stay in
HBM; the FFT and binning run on the GPU).  Arrays may be numpy arrays or torch
tensors (host or CUDA); torch is only used as a container for device memory.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import native

GENPK_FLAG_TIMING = 0x1
ENGINE_AUTO, ENGINE_SORTED, ENGINE_WINDOW, ENGINE_STREAM = 0, 1, 2, 3
FFT_AUTO, FFT_CUFFT3D = 0, 1
GENPK_BATCH_PER_BOX, GENPK_BATCH_GROUPED, GENPK_BATCH_AUTO = 0, 1, 2
_BATCH_MODES = {False: GENPK_BATCH_PER_BOX, "per_box": GENPK_BATCH_PER_BOX,
                True: GENPK_BATCH_GROUPED, "grouped": GENPK_BATCH_GROUPED,
                "auto": GENPK_BATCH_AUTO}


class GenPKError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"genpk status {status}: {message}")
        self.status = status
        self.message = message


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _arg(x, np_dtype, torch_dtype_name):
    """(address, keep-alive object, is_device) for a numpy array or torch tensor."""
    if x is None:
        return None, None, False
    if _is_torch(x):
        import torch
        t = x.detach()
        want = getattr(torch, torch_dtype_name)
        if t.dtype != want:
            t = t.to(want)
        t = t.contiguous()
        return t.data_ptr(), t, t.is_cuda
    a = np.ascontiguousarray(x, dtype=np_dtype)
    return a.ctypes.data, a, False


def _check(lib, ctx, rc):
    if rc != 0:
        msg = lib.genpk_last_error(ctx).decode() if ctx else ""
        if not msg:
            msg = lib.genpk_status_string(rc).decode()
        raise GenPKError(rc, msg)


class Context:
    """Device-resident grids for one grid size (replaces fftw_malloc + plan)."""

    def __init__(self, dims: int, nrbins: int, nfields: int = 1, timing: bool = False):
        self.lib = native.load()
        self.dims = int(dims)
        self.nrbins = int(nrbins)
        self.nfields = int(nfields)
        self.row = 2 * (self.dims // 2 + 1)
        h = ctypes.c_void_p()
        rc = self.lib.genpk_ctx_create(self.dims, self.nrbins, self.nfields,
                                       GENPK_FLAG_TIMING if timing else 0, ctypes.byref(h))
        if rc != 0:
            msg = self.lib.genpk_last_error(h).decode() if h.value else ""
            if h.value:
                self.lib.genpk_ctx_destroy(h)
            raise GenPKError(rc, msg or self.lib.genpk_status_string(rc).decode())
        self.h = h

    # -- life cycle ---------------------------------------------------------
    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.genpk_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _chk(self, rc):
        _check(self.lib, self.h, rc)

    # -- grids ----------------------------------------------------------------
    def zero(self, field: int = 0):
        self._chk(self.lib.genpk_zero(self.h, field))

    def deposit(self, field, boxsize, pos, masses=None, mass=0.0):
        """+= CIC deposit of particles (fieldize semantics)."""
        pp, pk, _ = _arg(pos, np.float32, "float32")
        n = (pk.numel() if _is_torch(pk) else pk.size) // 3
        mp, mk, _ = _arg(masses, np.float32, "float32")
        self._chk(self.lib.genpk_deposit(self.h, field, float(boxsize), pp, mp, float(mass), n))
        return self

    def sync(self):
        self._chk(self.lib.genpk_sync(self.h))

    def read_field(self, field: int = 0) -> np.ndarray:
        out = np.empty((self.dims, self.dims, self.row), dtype=np.float64)
        self._chk(self.lib.genpk_read_field(self.h, field,
                                            out.ctypes.data_as(native.c_f64p)))
        return out

    def load_spectrum(self, field, spec):
        spec = np.ascontiguousarray(spec, dtype=np.complex128)
        self._chk(self.lib.genpk_load_spectrum(self.h, field,
                                               spec.ctypes.data_as(native.c_f64p)))

    # -- spectra --------------------------------------------------------------
    def power(self, field_a=0, field_b=None, mass_a=1.0, mass_b=None):
        """(power, count, keffs) like powerspectrum(); FFTs the grids if needed."""
        field_b = field_a if field_b is None else field_b
        mass_b = mass_a if mass_b is None else mass_b
        p = np.zeros(self.nrbins)
        c = np.zeros(self.nrbins, dtype=np.int32)
        k = np.zeros(self.nrbins)
        self._chk(self.lib.genpk_power(self.h, field_a, field_b, float(mass_a), float(mass_b),
                                       p.ctypes.data_as(native.c_f64p),
                                       c.ctypes.data_as(native.c_i32p),
                                       k.ctypes.data_as(native.c_f64p)))
        return p, c, k

    def power_multi(self, pairs, pair_masses):
        pairs = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
        pm = np.ascontiguousarray(np.asarray(pair_masses, dtype=np.float64).reshape(-1, 2))
        npair = pairs.shape[0]
        p = np.zeros((npair, self.nrbins))
        c = np.zeros(self.nrbins, dtype=np.int32)
        k = np.zeros(self.nrbins)
        self._chk(self.lib.genpk_power_multi(self.h, npair, pairs.ctypes.data_as(native.c_i32p),
                                             pm.ctypes.data_as(native.c_f64p),
                                             p.ctypes.data_as(native.c_f64p),
                                             c.ctypes.data_as(native.c_i32p),
                                             k.ctypes.data_as(native.c_f64p)))
        return p, c, k

    def power_step(self, boxsize, pos_list, pairs, pair_masses, masses_list=None, mass=0.0):
        """One step of the per-species loop (genpk_power_step): species s is
        deposited into cleared field s, then the spectra of `pairs` as
        power_multi returns them.  Repeated identical calls on device arrays
        replay a captured CUDA graph of the whole step."""
        ns = len(pos_list)
        keep, pp, mp, n = [], [], [], []
        for s in range(ns):
            a, k, _ = _arg(pos_list[s], np.float32, "float32")
            pp.append(a)
            keep.append(k)
            n.append((k.numel() if _is_torch(k) else k.size) // 3)
            m = masses_list[s] if masses_list is not None else None
            b, km, _ = _arg(m, np.float32, "float32")
            mp.append(b)
            keep.append(km)
        ms = np.ascontiguousarray(np.broadcast_to(np.asarray(mass, dtype=np.float64), (ns,)))
        nn = np.ascontiguousarray(np.asarray(n, dtype=np.int64))
        pairs = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
        pm = np.ascontiguousarray(np.asarray(pair_masses, dtype=np.float64).reshape(-1, 2))
        npair = pairs.shape[0]
        pos_arr = (ctypes.c_void_p * ns)(*pp)
        mass_arr = (ctypes.c_void_p * ns)(*mp) if masses_list is not None else None
        p = np.zeros((npair, self.nrbins))
        c = np.zeros(self.nrbins, dtype=np.int32)
        k = np.zeros(self.nrbins)
        rc = self.lib.genpk_power_step(self.h, ns, float(boxsize), pos_arr, mass_arr,
                                       ms.ctypes.data_as(native.c_f64p),
                                       nn.ctypes.data_as(native.c_i64p), npair,
                                       pairs.ctypes.data_as(native.c_i32p),
                                       pm.ctypes.data_as(native.c_f64p),
                                       p.ctypes.data_as(native.c_f64p),
                                       c.ctypes.data_as(native.c_i32p),
                                       k.ctypes.data_as(native.c_f64p))
        del keep
        self._chk(rc)
        return p, c, k

    def step_use_graph(self, on: bool = True):
        self._chk(self.lib.genpk_power_step_use_graph(self.h, 1 if on else 0))

    @property
    def step_replays(self) -> int:
        return int(self.lib.genpk_power_step_replays(self.h))

    # -- adjoint --------------------------------------------------------------
    def adjoint(self, field, boxsize, pos, dl_dp, mass_norm, masses=None, mass=0.0,
                recompute=False, grad_pos=None, grad_mass=None):
        """dL/dpos [n,3], dL/dmass [n] (or None) and dL/dM for the auto spectrum of
        `field`; outputs live where `pos` lives (host numpy or CUDA tensor)."""
        pp, pk, dev = _arg(pos, np.float32, "float32")
        n = (pk.numel() if _is_torch(pk) else pk.size) // 3
        mp, mk, _ = _arg(masses, np.float32, "float32")
        if dev:
            import torch
            gp = grad_pos if grad_pos is not None else torch.empty((n, 3), dtype=torch.float32,
                                                                     device=pk.device)
            gm = None
            if masses is not None:
                gm = grad_mass if grad_mass is not None else torch.empty(
                    n, dtype=torch.float32, device=pk.device)
            gpp, gmp = gp.data_ptr(), (gm.data_ptr() if gm is not None else None)
        else:
            gp = np.empty((n, 3), dtype=np.float32)
            gm = np.empty(n, dtype=np.float32) if masses is not None else None
            gpp, gmp = gp.ctypes.data, (gm.ctypes.data if gm is not None else None)
        g = np.ascontiguousarray(dl_dp, dtype=np.float64)
        dldm = ctypes.c_double(0.0)
        self._chk(self.lib.genpk_adjoint(self.h, field, float(boxsize), pp, mp, float(mass), n,
                                         float(mass_norm), g.ctypes.data_as(native.c_f64p),
                                         gpp, gmp, ctypes.byref(dldm), 1 if recompute else 0))
        return gp, gm, dldm.value

    # -- introspection --------------------------------------------------------
    def timing_reset(self):
        self._chk(self.lib.genpk_timing_reset(self.h))

    def stage_times(self) -> dict:
        """{kernel/stage name: ms} since the last timing_reset (CUDA events)."""
        names = (ctypes.c_char_p * 64)()
        ms = (ctypes.c_float * 64)()
        k = self.lib.genpk_stage_times(self.h, names, ms, 64)
        out = {}
        for i in range(k):
            key = names[i].decode() if names[i] else f"stage{i}"
            out[key] = out.get(key, 0.0) + ms[i]
        return out

    def deposit_config(self) -> dict:
        """The sorted engine's tile and sort CTAs of the latest pass."""
        return _deposit_config(self.lib, self.h, self._chk)

    def set_engine(self, engine: int):
        """Deposit engine: ENGINE_AUTO, ENGINE_SORTED, ENGINE_WINDOW or
        ENGINE_STREAM (identical grids; they differ in speed by particle order
        and density)."""
        self._chk(self.lib.genpk_set_deposit_engine(self.h, int(engine)))

    def set_fft_mode(self, mode: int):
        """Forward-FFT path: FFT_AUTO (2-D cuFFT + fused x-pass/binning where
        supported) or FFT_CUFFT3D (3-D cuFFT + binning kernel)."""
        self._chk(self.lib.genpk_set_fft_mode(self.h, int(mode)))

    @property
    def last_engine(self) -> int:
        return int(self.lib.genpk_last_deposit_engine(self.h))

    def set_tile(self, tx: int, ty: int, tz: int):
        """Fix the sorted engine's tile (turns its autotuner off); (0, 0, 0):
        automatic again."""
        self._chk(self.lib.genpk_set_deposit_tile(self.h, tx, ty, tz))

    def deposit_trials(self) -> list:
        """The sorted engine's latest tuning: [(tile, sort CTAs, ms), ...]
        (tile (0, 0, 0): the stream mode's trial)."""
        return _deposit_trials(self.lib, self.h)

    @property
    def launches(self) -> int:
        return int(self.lib.genpk_kernel_launches(self.h))

    def bin_of(self, kk2: int) -> int:
        return int(self.lib.genpk_bin_of(self.h, int(kk2)))

    def inject_copy_timeout(self, chunk: int, wait_clocks: int = 1 << 16):
        """Testing aid: the next window/stream-engine pass leaves chunk
        `chunk` without its bulk copy, so its bounded wait gives up
        (genpk_inject_copy_timeout)."""
        self._chk(self.lib.genpk_inject_copy_timeout(self.h, int(chunk), int(wait_clocks)))


class Batch:
    """Many independent boxes (grids of any sizes, one bin count) whose auto
    spectra one call computes: genpk_batch_power issues every box's deposit,
    transform and binning from this thread, each box on its own stream, and
    waits once for all of them."""

    def __init__(self, dims_list, nrbins: int, timing: bool = False):
        self.lib = native.load()
        self.dims = [int(d) for d in dims_list]
        self.nboxes = len(self.dims)
        self.nrbins = int(nrbins)
        arr = (ctypes.c_int64 * self.nboxes)(*self.dims)
        h = ctypes.c_void_p()
        rc = self.lib.genpk_batch_create(self.nboxes, arr, self.nrbins,
                                         GENPK_FLAG_TIMING if timing else 0, ctypes.byref(h))
        if rc != 0:
            msg = self.lib.genpk_batch_last_error(h).decode() if h.value else ""
            if h.value:
                self.lib.genpk_batch_destroy(h)
            raise GenPKError(rc, msg or self.lib.genpk_status_string(rc).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.genpk_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def power(self, boxsize, pos_list, mass_norm, masses_list=None, mass=0.0):
        """(power, count, keffs), each [nboxes][nrbins].  boxsize, mass and
        mass_norm: a number for every box or one per box."""
        nb = self.nboxes

        def per_box(v):
            return [float(x) for x in v] if np.ndim(v) else [float(v)] * nb

        keep, pp, mp, n = [], [], [], []
        for i in range(nb):
            a, k, _ = _arg(pos_list[i], np.float32, "float32")
            pp.append(a)
            keep.append(k)
            n.append((k.numel() if _is_torch(k) else k.size) // 3)
            m = masses_list[i] if masses_list is not None else None
            b, km, _ = _arg(m, np.float32, "float32")
            mp.append(b)
            keep.append(km)
        bs = (ctypes.c_double * nb)(*per_box(boxsize))
        ms = (ctypes.c_double * nb)(*per_box(mass))
        mn = (ctypes.c_double * nb)(*per_box(mass_norm))
        nn = (ctypes.c_int64 * nb)(*n)
        pos_arr = (ctypes.c_void_p * nb)(*pp)
        mass_arr = (ctypes.c_void_p * nb)(*mp) if masses_list is not None else None
        p = np.zeros((nb, self.nrbins))
        c = np.zeros((nb, self.nrbins), dtype=np.int32)
        kf = np.zeros((nb, self.nrbins))
        rc = self.lib.genpk_batch_power(self.h, bs, pos_arr, mass_arr, ms, nn, mn,
                                        p.ctypes.data_as(native.c_f64p),
                                        c.ctypes.data_as(native.c_i32p),
                                        kf.ctypes.data_as(native.c_f64p))
        del keep
        if rc != 0:
            raise GenPKError(rc, self.lib.genpk_batch_last_error(self.h).decode())
        return p, c, kf

    def engine(self, i: int) -> int:
        """Deposit engine box i's latest pass used."""
        return int(self.lib.genpk_last_deposit_engine(self.lib.genpk_batch_box(self.h, i)))

    def deposit_config(self, i: int) -> dict:
        """Box i's sorted-engine tile and sort CTAs of its latest pass."""
        box = self.lib.genpk_batch_box(self.h, i)

        def chk(rc):
            if rc != 0:
                raise GenPKError(rc, "genpk_deposit_config")
        return _deposit_config(self.lib, box, chk)

    def deposit_trials(self, i: int) -> list:
        """Box i's latest sorted-engine tuning, as Context.deposit_trials."""
        return _deposit_trials(self.lib, self.lib.genpk_batch_box(self.h, i))

    @property
    def launches(self) -> int:
        return int(self.lib.genpk_batch_launches(self.h))

    def use_graph(self, on: bool = True):
        """Capture repeated identical calls in a CUDA graph and replay it (on by
        default); False: every call issues its kernels one by one."""
        rc = self.lib.genpk_batch_use_graph(self.h, 1 if on else 0)
        if rc != 0:
            raise GenPKError(rc, "genpk_batch_use_graph")

    @property
    def graph_replays(self) -> int:
        """Calls served by a replay of the captured graph."""
        return int(self.lib.genpk_batch_graph_replays(self.h))

    def set_mode(self, mode):
        """True or "grouped": boxes of one grid size share each kernel launch of
        a grouped sorted-engine pass, one batched transform and one binning x
        pass (GENPK_BATCH_GROUPED); False or "per_box": every box has its own
        passes; "auto" (the default): the faster of the two, from timed trial
        calls."""
        rc = self.lib.genpk_batch_set_mode(self.h, _BATCH_MODES[mode])
        if rc != 0:
            raise GenPKError(rc, "genpk_batch_set_mode")

    @property
    def last_mode(self) -> str:
        """How the latest call ran: "per_box" or "grouped" (None before a call)."""
        m = int(self.lib.genpk_batch_last_mode(self.h))
        return {GENPK_BATCH_PER_BOX: "per_box", GENPK_BATCH_GROUPED: "grouped"}.get(m)

    def auto_times(self) -> dict:
        """The auto mode's timed trial calls (ms) and its choice (None while the
        trials run)."""
        a, g = ctypes.c_double(), ctypes.c_double()
        c = int(self.lib.genpk_batch_auto_times(self.h, ctypes.byref(a), ctypes.byref(g)))
        return {"per_box_ms": a.value, "grouped_ms": g.value,
                "choice": {GENPK_BATCH_PER_BOX: "per_box",
                           GENPK_BATCH_GROUPED: "grouped"}.get(c)}

    def groups(self) -> list:
        """The groups of the latest grouped call: for each, its boxes, grid size,
        tuned tile and sort CTAs, tuning trials and kernel launches."""
        out = []
        for g in range(max(int(self.lib.genpk_batch_groups(self.h)), 0)):
            nb = ctypes.c_int()
            boxes = (ctypes.c_int * 32)()
            h = self.lib.genpk_batch_group(self.h, g, ctypes.byref(nb),
                                           ctypes.cast(boxes, native.c_i32p))

            def chk(rc):
                if rc != 0:
                    raise GenPKError(rc, "genpk_deposit_config")
            out.append({"boxes": [boxes[i] for i in range(nb.value)],
                        "dims": self.dims[boxes[0]],
                        "config": _deposit_config(self.lib, h, chk),
                        "trials": _deposit_trials(self.lib, h),
                        "launches": int(self.lib.genpk_kernel_launches(h))})
        return out


def _deposit_config(lib, h, chk) -> dict:
    v = [ctypes.c_int() for _ in range(4)]
    chk(lib.genpk_deposit_config(h, *[ctypes.byref(x) for x in v]))
    return {"tile": (v[0].value, v[1].value, v[2].value), "sort_ctas": v[3].value}


def _deposit_trials(lib, h) -> list:
    from . import native
    cap = 10
    tx = (ctypes.c_int * cap)()
    ty = (ctypes.c_int * cap)()
    tz = (ctypes.c_int * cap)()
    sc = (ctypes.c_int * cap)()
    ms = (ctypes.c_float * cap)()
    k = lib.genpk_deposit_trials(h, ctypes.cast(tx, native.c_i32p), ctypes.cast(ty, native.c_i32p),
                                 ctypes.cast(tz, native.c_i32p), ctypes.cast(sc, native.c_i32p),
                                 ctypes.cast(ms, native.c_f32p), cap)
    return [((tx[i], ty[i], tz[i]), sc[i], ms[i]) for i in range(max(k, 0))]


# ---------------------------------------------------------------------------
# Reference-named functions
# ---------------------------------------------------------------------------

def invwindow(kx, ky, kz, n) -> float:
    """fieldize.cpp:125-133."""
    return native.load().genpk_invwindow(int(kx), int(ky), int(kz), int(n))


def geometry(dims, nrbins):
    """Weighted mode counts and mean |k| per bin (host only, no GPU)."""
    lib = native.load()
    c = np.zeros(nrbins, dtype=np.int32)
    k = np.zeros(nrbins)
    _check(lib, None, lib.genpk_geometry(int(dims), int(nrbins), c.ctypes.data_as(native.c_i32p),
                                         k.ctypes.data_as(native.c_f64p)))
    return c, k


def fieldize(boxsize, dims, out, pos, masses=None, mass=0.0, extra=1) -> int:
    """fieldize.cpp:46: += CIC deposit into the float64 host array `out`
    (size dims*dims*2*(dims/2+extra)), computed on the GPU.  Returns 0."""
    lib = native.load_compat()
    assert out.dtype == np.float64 and out.flags.c_contiguous
    pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1)
    mp = None
    if masses is not None:
        masses = np.ascontiguousarray(masses, dtype=np.float32)
        mp = masses.ctypes.data_as(native.c_f32p)
    rc = lib.fieldize(float(boxsize), int(dims), out.ctypes.data_as(native.c_f64p),
                      pos.size // 3, pos.ctypes.data_as(native.c_f32p), mp, float(mass),
                      int(extra))
    _check(native.load(), None, rc)
    return rc


def powerspectrum(dims, outfield, outfield2, nrbins, total_mass, total_mass2):
    """powerspectrum.c:35 on the caller's half-complex spectra (complex128,
    dims x dims x dims/2+1), binned on the GPU.  Returns (power, count, keffs)."""
    lib = native.load_compat()
    f1 = np.ascontiguousarray(outfield, dtype=np.complex128)
    f2 = f1 if outfield2 is None or outfield2 is outfield else np.ascontiguousarray(
        outfield2, dtype=np.complex128)
    p = np.zeros(nrbins)
    c = np.zeros(nrbins, dtype=np.int32)
    k = np.zeros(nrbins)
    rc = lib.powerspectrum(int(dims), f1.ctypes.data_as(native.c_f64p),
                           f2.ctypes.data_as(native.c_f64p), int(nrbins),
                           p.ctypes.data_as(native.c_f64p), c.ctypes.data_as(native.c_i32p),
                           k.ctypes.data_as(native.c_f64p), float(total_mass),
                           float(total_mass2))
    _check(native.load(), None, rc)
    return p, c, k
