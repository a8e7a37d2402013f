"""The gen-pk command line (genpk_gb300/cli): format-II reading, the grid and
bin rule, and the per-type, -s, -c and -j outputs against the FP64 oracle.

The CPU tests run the reader alone (-d prints the header and needs no GPU);
the GPU tests run whole snapshots through the C ABI and compare every written
file with the oracle's deposit + FP64 FFT + binning of the same particles,
normalised as the reference does (sum of masses + 1 per type read,
read_fieldize.cpp:94)."""
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

CLI = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "genpk_gb300",
                   "_lib", "gen-pk-gb300")


def run_cli(*args):
    return subprocess.run([CLI, *args], capture_output=True, text=True, timeout=600)


def species(seed=5):
    """Gas (per-particle masses), dark matter (header mass) and stars
    (per-particle masses), as a hydrodynamic snapshot holds them."""
    from genpk_gb300 import synth
    rng = np.random.default_rng(seed)
    box = 1000.0
    dm = synth.zeldovich(16, box, seed=seed)
    gas = synth.zeldovich(16, box, seed=seed + 1)[:3000]
    stars = synth.uniform(700, box, seed=seed + 2)
    pos = {0: gas, 1: dm, 4: stars}
    masses = {0: rng.uniform(0.1, 0.3, len(gas)).astype(np.float32), 1: 0.5,
              4: rng.lognormal(-1.0, 0.5, len(stars)).astype(np.float32)}
    return box, pos, masses


def write(tmp_path, name="snap", nfiles=2, seed=5):
    from genpk_gb300 import synth
    box, pos, masses = species(seed)
    base = str(tmp_path / name)
    synth.write_gadget2(base, pos, masses, box, nfiles=nfiles, time=0.25, redshift=3.0)
    return base, box, pos, masses


def read_pk(path):
    rows = np.loadtxt(path, ndmin=2)
    return rows[:, 0], rows[:, 1], rows[:, 2].astype(np.int64)


def expect(pos, masses, t, box, dims, nrbins):
    """(power, count, keffs, M) of the oracle for type t (non-empty bins only)."""
    m = masses[t]
    arr = None if np.isscalar(m) else m
    mass = float(m) if np.isscalar(m) else 0.0
    M = O.total_mass(len(pos[t]), arr, mass)
    p, c, k = O.pk(pos[t], box, dims, nrbins, arr, mass, m_norm=M)
    return p, c, k, M


def close(a, b, tol):
    return np.all(np.abs(a - b) <= tol * np.maximum(np.abs(b), 1e-300))


def test_cli_reads_the_header(native_lib, tmp_path):
    base, box, pos, masses = write(tmp_path)
    r = run_cli("-i", base, "-d")
    assert r.returncode == 0, r.stderr
    out = r.stdout
    assert "files=2" in out and "Boxsize=1000" in out
    assert f"type 0 (by): npart={len(pos[0])} mass=0\n" in out
    assert f"type 1 (DM): npart={len(pos[1])} mass=0.5\n" in out
    assert f"type 4 (st): npart={len(pos[4])} mass=0\n" in out
    assert "type 2 (nu): npart=0" in out


def test_cli_reads_the_reference_snapshot_fixture(native_lib):
    """The reference's own two-file format-II fixture (written by Gadget), where
    its source tree is present: particle counts, box and scale factor."""
    tree = O.reference_tree()
    if tree is None or not os.path.exists(os.path.join(tree, "test_g2_snap.0")):
        pytest.skip("reference tree not present")
    base = os.path.join(tree, "test_g2_snap")
    r = run_cli("-i", base, "-d")
    assert r.returncode == 0, r.stderr
    assert "files=2" in r.stdout and "Boxsize=3000" in r.stdout
    for line in ("type 0 (by): npart=4039 ", "type 1 (DM): npart=4096 ", "type 4 (st): npart=57 "):
        assert line in r.stdout
    t = float(r.stdout.split("time=")[1].split()[0])
    assert abs(t - 0.2778) < 1e-3


def test_cli_rejects_what_is_not_a_snapshot(native_lib, tmp_path):
    bad = tmp_path / "junk"
    bad.write_bytes(b"\x10\x00\x00\x00not a snapshot at all")
    r = run_cli("-i", str(bad), "-d")
    assert r.returncode == 1 and "not a format-II snapshot" in r.stderr
    r = run_cli("-i", str(tmp_path / "missing"), "-d")
    assert r.returncode == 1 and "no such snapshot" in r.stderr


@pytest.mark.gpu
def test_cli_per_type_spectra(native_lib, tmp_path):
    """Default mode with the grid and bins overridden: one PK file per type,
    every bin within 1e-5 of the oracle (printed to 7 digits), counts exact."""
    base, box, pos, masses = write(tmp_path)
    out = tmp_path / "out"
    out.mkdir()
    r = run_cli("-i", base, "-o", str(out), "-g", "32", "-b", "12")
    assert r.returncode == 0, r.stdout + r.stderr
    for t, name in ((0, "by"), (1, "DM"), (4, "st")):
        k, p, c = read_pk(out / f"PK-{name}-snap")
        pe, ce, ke, M = expect(pos, masses, t, box, 32, 12)
        ok = ce > 0
        assert np.array_equal(c, ce[ok])
        assert close(p, pe[ok], 1e-5) and close(k, ke[ok], 1e-6)
        assert f"total_mass in type {t} = {M:g}" in r.stdout
    assert not (out / "PK-nu-snap").exists()


@pytest.mark.gpu
def test_cli_uniform_128_snapshot(native_lib, tmp_path):
    """The 128^3 snapshot configuration: one format-II file holding only
    type 1, 128^3 = 2,097,152 particles with float32 positions i.i.d. uniform
    in [0, 25000) kpc/h and the header mass 1.0e-2 (box 25000, a = 1,
    h = 0.7), run as gen-pk -g 128 -b 64.  The PK-DM file against the oracle
    normalised with the reader's +1 (read_fieldize.cpp:94): every bin within
    1e-5 (printed to 7 digits), counts bit-exact."""
    from genpk_gb300 import synth
    box, n = 25000.0, 128 ** 3
    pos = synth.uniform(n, box, seed=1)
    base = str(tmp_path / "snap_128")
    synth.write_gadget2(base, {1: pos}, {1: 1.0e-2}, box, nfiles=1, time=1.0, redshift=0.0,
                        hubble=0.7)
    out = tmp_path / "out"
    out.mkdir()
    r = run_cli("-i", base, "-o", str(out), "-g", "128", "-b", "64")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FFT grid dimension: 128" in r.stdout
    M = O.total_mass(n, None, 1.0e-2)
    assert f"total_mass in type 1 = {M:g}" in r.stdout
    pe, ce, ke = O.pk(pos, box, 128, 64, None, 1.0e-2, m_norm=M)
    k, p, c = read_pk(out / "PK-DM-snap_128")
    ok = ce > 0
    assert np.array_equal(c, ce[ok])
    assert close(p, pe[ok], 1e-5) and close(k, ke[ok], 1e-6)
    assert sorted(os.listdir(out)) == ["PK-DM-snap_128"]


@pytest.mark.gpu
def test_cli_default_grid_rule_and_stars_in_baryons(native_lib, tmp_path):
    """No -g / -b: grid = max over types of 2*nexttwo(cbrt(npart)) = 32 for
    16^3 dark-matter particles, nrbins = grid.  -s 1 adds the stars to the
    baryon field with their own +1 in the normalising mass."""
    base, box, pos, masses = write(tmp_path, nfiles=1)
    out = tmp_path / "out"
    out.mkdir()
    r = run_cli("-i", base, "-o", str(out), "-s", "1")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FFT grid dimension: 32" in r.stdout
    allpos = np.concatenate([pos[0], pos[4]])
    allm = np.concatenate([masses[0], masses[4]])
    M = O.total_mass(len(pos[0]), masses[0]) + O.total_mass(len(pos[4]), masses[4])
    pe, ce, ke = O.pk(allpos, box, 32, 32, allm, 0.0, m_norm=M)
    k, p, c = read_pk(out / "PK-by-snap")
    ok = ce > 0
    assert np.array_equal(c, ce[ok]) and close(p, pe[ok], 1e-5)


@pytest.mark.gpu
def test_cli_cross_spectra(native_lib, tmp_path):
    """-c 4: dark matter x stars in one snapshot; -j: each type of one snapshot
    against the same type of a second snapshot."""
    base, box, pos, masses = write(tmp_path)
    base2, _, pos2, masses2 = write(tmp_path, name="other", seed=9)
    out = tmp_path / "out"
    out.mkdir()
    dims, nrb = 32, 12

    def field(p, m):
        arr = None if np.isscalar(m) else m
        mass = float(m) if np.isscalar(m) else 0.0
        return O.rfft_padded(O.deposit(p, box, dims, arr, mass)), O.total_mass(len(p), arr, mass)

    r = run_cli("-i", base, "-o", str(out), "-g", str(dims), "-b", str(nrb), "-c", "4")
    assert r.returncode == 0, r.stdout + r.stderr
    (fa, ma), (fb, mb) = field(pos[1], masses[1]), field(pos[4], masses[4])
    pe, ce, ke = O.cross_pk(fa, fb, dims, nrb, ma, mb)
    k, p, c = read_pk(out / "PK-DMxst-snap")
    ok = ce > 0
    assert np.array_equal(c, ce[ok]) and close(p, pe[ok], 1e-5)

    r = run_cli("-i", base, "-j", base2, "-o", str(out), "-g", str(dims), "-b", str(nrb))
    assert r.returncode == 0, r.stdout + r.stderr
    for t, name in ((0, "by"), (1, "DM"), (4, "st")):
        (fa, ma), (fb, mb) = field(pos[t], masses[t]), field(pos2[t], masses2[t])
        pe, ce, ke = O.cross_pk(fa, fb, dims, nrb, ma, mb)
        k, p, c = read_pk(out / f"PX-{name}-snap")
        ok = ce > 0
        assert np.array_equal(c, ce[ok])
        # cross spectra change sign; compare against the bin's auto-power scale
        scale = np.sqrt(np.abs(O.cross_pk(fa, fa, dims, nrb, ma, ma)[0] *
                               O.cross_pk(fb, fb, dims, nrb, mb, mb)[0]))[ok]
        assert np.all(np.abs(p - pe[ok]) <= 1e-5 * np.maximum(np.abs(pe[ok]), scale))

    r = run_cli("-i", base, "-o", str(out), "-c", "2")
    assert r.returncode == 1 and "Can't cross-correlate" in r.stderr


# ---------------------------------------------------------------------------
# BigFile snapshots (read_fieldize_bigfile.cpp): positions stored as f8 and
# narrowed to float, masses as f4, no +1 in the normalising mass
# ---------------------------------------------------------------------------

def write_bf(tmp_path, name="bfsnap", nfiles=3, pos_dtype="<f8", seed=5):
    from genpk_gb300 import synth
    box, pos, masses = species(seed)
    # positions stored in double precision, as MP-Gadget writes them
    pos64 = {t: p.astype(np.float64) + 1e-9 for t, p in pos.items()}
    root = str(tmp_path / name)
    synth.write_bigfile(root, pos64, masses, box, time=0.5, hubble=0.7, nfiles=nfiles,
                        pos_dtype=pos_dtype)
    pos32 = {t: p.astype(np.float32) for t, p in pos64.items()}
    return root, box, pos32, masses


def bf_mass(masses, t, n):
    """The BigFile path's normalising mass: the float masses summed in double
    plus MassTable * n, with no +1 (read_fieldize_bigfile.cpp:97-117)."""
    m = masses[t]
    if np.isscalar(m):
        return float(m) * n
    return float(np.sum(m.astype(np.float64)))


def test_cli_reads_a_bigfile_header(native_lib, tmp_path):
    root, box, pos, masses = write_bf(tmp_path)
    r = run_cli("-i", root, "-d")
    assert r.returncode == 0, r.stderr
    assert "format=bigfile" in r.stdout and "Boxsize=1000" in r.stdout
    assert "time=0.5" in r.stdout and "redshift=1," in r.stdout
    assert f"type 0 (by): npart={len(pos[0])} mass=0\n" in r.stdout
    assert f"type 1 (DM): npart={len(pos[1])} mass=0.5\n" in r.stdout
    assert "type 3 (xx): npart=0" in r.stdout


def test_cli_refuses_broken_bigfile_and_hdf5(native_lib, tmp_path):
    root, _, _, _ = write_bf(tmp_path)
    # a Header block without its BoxSize attribute
    attrs = tmp_path / "bfsnap" / "Header" / "attr-v2"
    attrs.write_text("".join(l for l in attrs.read_text().splitlines(True)
                             if not l.startswith("BoxSize")))
    r = run_cli("-i", root, "-d")
    assert r.returncode == 1 and "BoxSize" in r.stderr
    h5 = tmp_path / "snap.hdf5"
    h5.write_bytes(b"\x89HDF\r\n\x1a\n" + b"\0" * 64)
    r = run_cli("-i", str(h5), "-d")
    assert r.returncode == 1 and "HDF5" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("pos_dtype", ["<f8", "<f4"])
def test_cli_bigfile_per_type_spectra(native_lib, tmp_path, pos_dtype):
    """Every type of a BigFile snapshot (columns split over three data files)
    against the oracle on the narrowed float positions, normalised by the
    masses alone: every bin within 1e-5, counts bit-exact."""
    root, box, pos, masses = write_bf(tmp_path, pos_dtype=pos_dtype)
    out = tmp_path / "out"
    out.mkdir()
    r = run_cli("-i", root, "-o", str(out), "-g", "32", "-b", "12")
    assert r.returncode == 0, r.stdout + r.stderr
    for t, name in ((0, "by"), (1, "DM"), (4, "st")):
        M = bf_mass(masses, t, len(pos[t]))
        assert f"total_mass in type {t} = {M:g}" in r.stdout
        arr = None if np.isscalar(masses[t]) else masses[t]
        mass = float(masses[t]) if np.isscalar(masses[t]) else 0.0
        pe, ce, ke = O.pk(pos[t], box, 32, 12, arr, mass, m_norm=M)
        k, p, c = read_pk(out / f"PK-{name}-bfsnap")
        ok = ce > 0
        assert np.array_equal(c, ce[ok])
        assert close(p, pe[ok], 1e-5) and close(k, ke[ok], 1e-6)
