"""The grid cache contract of the reference (test_framework_energy_grid_cache.cc),
ported case by case.

* Round trip (:80-122): a grid from loadOrBuild's second call comes from the
  file the first call wrote, and interpolates bit-identically (GPU).
* Mutating any single key field is a real cache miss (:124-201): each field
  the key holds (atom x, y, z, species, lattice, epsilon, sigma, cutoff,
  truncation, guest set, spacing) changes the content-addressed name, so a
  lookup under the mutated inputs finds no file (host only).
* A file whose stored key does not match the requested key is a hard error,
  never a silent reuse (:203-240): the baseline file copied to another key's
  path makes cacheHit and loadFromCache raise (host only: the key is read and
  compared before any device work). The energy cap, which no input sets,
  is covered by a file whose stored cap was changed in place.
* A format version mismatch is a hard error (:242-): both calls raise.
* The tables may come in any order: the reference writes them in its hash
  map's iteration order, which is a property of one standard library (GPU).

The baseline file is the reference's own cache file for the 424-atom cubic
cell (tests/golden/grid_cubic.npz, written by the reference build)."""
import shutil
import struct

import numpy as np
import pytest

from conftest import golden
from test_oracle_golden import _cache_tables


@pytest.fixture(scope="module")
def A():
    import aleator_gb300 as A
    from aleator_gb300.build import LIB, build

    if not LIB.exists():
        build()
    A.load_library()
    return A


def _inputs(A, g, **mut):
    x, y, z = g["x"].copy(), g["y"].copy(), g["z"].copy()
    species = g["species"].copy()
    lat = g["lattice"].copy()
    eps, sigma = g["eps"].copy(), g["sigma"].copy()
    cutoff = float(g["cutoff"])
    trunc = A.SHIFTED
    guests = [int(v) for v in g["guests"]]
    spacing = float(g["spacing"])
    if "x" in mut:
        x[0] += 0.5
    if "y" in mut:
        y[1] -= 0.3
    if "z" in mut:
        z[2] += 1.1
    if "species" in mut:
        species[0] = 1 if species[0] == 0 else 0
    if "lattice" in mut:
        lat[0, 0] += 0.2
    if "eps" in mut:
        eps[0] *= 1.01
    if "sigma" in mut:
        sigma[0] *= 1.01
    if "cutoff" in mut:
        cutoff += mut["cutoff"]
    if "truncation" in mut:
        trunc = A.TRUNCATED
    if "guests" in mut:
        guests = guests + [99]
    if "spacing" in mut:
        spacing += 0.25
    ff = A.LennardJones(eps, sigma, cutoff, trunc)
    p = A.ParticleData(x, y, z, g["charge"], species)
    return ff, p, lat, guests, spacing


def _baseline_dir(A, g, tmp_path):
    ff, p, lat, guests, spacing = _inputs(A, g)
    name = A.FrameworkEnergyGrid.cache_file_name(ff, p, lat, guests, spacing)
    assert name == str(g["cache_name"])
    (tmp_path / name).write_bytes(g["cache_file"].tobytes())
    return tmp_path / name


FIELDS = ["x", "y", "z", "species", "lattice", "eps", "sigma", "cutoff", "truncation", "guests",
          "spacing"]


def test_mutating_any_single_key_field_is_a_miss(A, tmp_path):
    g = golden("grid_cubic")
    base = _baseline_dir(A, g, tmp_path)
    ff, p, lat, guests, spacing = _inputs(A, g)
    assert A.FrameworkEnergyGrid.cache_hit(tmp_path, ff, p, lat, guests, spacing)
    names = {base.name}
    for field in FIELDS:
        ff, p, lat, guests, spacing = _inputs(A, g, **{field: 0.5})
        name = A.FrameworkEnergyGrid.cache_file_name(ff, p, lat, guests, spacing)
        assert name not in names, field  # the hash moved
        names.add(name)
        assert not A.FrameworkEnergyGrid.cache_hit(tmp_path, ff, p, lat, guests, spacing), field
        assert A.FrameworkEnergyGrid.load_from_cache(tmp_path, ff, p, lat, guests, spacing) is None
    # the guest set is a set: order and repeats do not change the key
    ff, p, lat, guests, spacing = _inputs(A, g)
    assert A.FrameworkEnergyGrid.cache_file_name(ff, p, lat, guests[::-1] + guests[:1],
                                                 spacing) == base.name


def test_stored_key_mismatch_is_a_hard_error(A, tmp_path):
    g = golden("grid_cubic")
    base = _baseline_dir(A, g, tmp_path)
    ff, p, lat, guests, spacing = _inputs(A, g, cutoff=1.0)
    other = tmp_path / A.FrameworkEnergyGrid.cache_file_name(ff, p, lat, guests, spacing)
    assert other != base
    shutil.copyfile(base, other)
    with pytest.raises(RuntimeError, match="stored key does not exactly match"):
        A.FrameworkEnergyGrid.cache_hit(tmp_path, ff, p, lat, guests, spacing)
    with pytest.raises(RuntimeError, match="stored key does not exactly match"):
        A.FrameworkEnergyGrid.load_from_cache(tmp_path, ff, p, lat, guests, spacing)


def _cap_offset(b: bytes) -> int:
    """Byte offset of the stored key's energy cap (the last key field)."""
    off = 4
    for _ in range(3):
        n, = struct.unpack_from("<Q", b, off)
        off += 8 + 8 * n
    n, = struct.unpack_from("<Q", b, off)
    off += 8 + 4 * n + 72
    ns, = struct.unpack_from("<Q", b, off)
    off += 8 + 16 * ns + 8 + 1
    n, = struct.unpack_from("<Q", b, off)
    return off + 8 + 4 * n + 8


def test_stored_energy_cap_mismatch_is_a_hard_error(A, tmp_path):
    g = golden("grid_cubic")
    base = _baseline_dir(A, g, tmp_path)
    b = bytearray(base.read_bytes())
    off = _cap_offset(bytes(b))
    assert struct.unpack_from("<d", b, off)[0] == 1e5
    struct.pack_into("<d", b, off, 2e5)
    base.write_bytes(bytes(b))
    ff, p, lat, guests, spacing = _inputs(A, g)
    for call in (A.FrameworkEnergyGrid.cache_hit, A.FrameworkEnergyGrid.load_from_cache):
        with pytest.raises(RuntimeError, match="stored key does not exactly match"):
            call(tmp_path, ff, p, lat, guests, spacing)


def test_version_mismatch_is_a_hard_error(A, tmp_path):
    g = golden("grid_cubic")
    base = _baseline_dir(A, g, tmp_path)
    b = bytearray(base.read_bytes())
    b[0] = 2
    base.write_bytes(bytes(b))
    ff, p, lat, guests, spacing = _inputs(A, g)
    for call in (A.FrameworkEnergyGrid.cache_hit, A.FrameworkEnergyGrid.load_from_cache):
        with pytest.raises(RuntimeError, match="format version 2, this build expects 1"):
            call(tmp_path, ff, p, lat, guests, spacing)


def test_missing_directory_is_a_miss(A, tmp_path):
    g = golden("grid_cubic")
    ff, p, lat, guests, spacing = _inputs(A, g)
    assert not A.FrameworkEnergyGrid.cache_hit(tmp_path / "none", ff, p, lat, guests, spacing)


def _reorder_tables(b: bytes, order) -> bytes:
    """The same file with its tables written in another order."""
    counts, tables = _cache_tables(np.frombuffer(b, dtype=np.uint8))
    head_len = len(b) - sum(12 + 8 * len(t) for t in tables.values())
    out = bytearray(b[:head_len])
    for sid in order:
        out += struct.pack("<IQ", sid, len(tables[sid])) + tables[sid].tobytes()
    return bytes(out)


@pytest.mark.gpu
def test_tables_in_any_order_load_the_same(A, tmp_path):
    g = golden("grid_cubic")
    base = _baseline_dir(A, g, tmp_path)
    ff, p, lat, guests, spacing = _inputs(A, g)
    counts, tables = _cache_tables(g["cache_file"])
    assert list(tables) == sorted(tables, reverse=True)  # the reference's order on this host
    for order in (sorted(tables), [5, 4, 6], [6, 4, 5]):
        base.write_bytes(_reorder_tables(g["cache_file"].tobytes(), order))
        grid = A.FrameworkEnergyGrid.load_from_cache(tmp_path, ff, p, lat, guests, spacing)
        assert grid.species() == sorted(tables)
        for sid, t in tables.items():
            assert np.array_equal(grid.table(sid), t)
        for i, sid in enumerate(g["guests"]):
            assert np.array_equal(grid.interpolate(int(sid), g["points"]), g["interp"][i])


@pytest.mark.gpu
def test_load_or_build_round_trip_is_bit_identical(A, tmp_path):
    from aleator_gb300 import workloads as W

    fw = W.cubic_framework(seed=11)
    ff = A.LennardJones(fw.eps, fw.sigma, 6.0, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    sid = fw.guest_species["CH4"]
    first, hit1 = A.FrameworkEnergyGrid.load_or_build(tmp_path, ff, p, fw.lattice, [sid], 1.0)
    assert not hit1  # nothing cached yet
    second, hit2 = A.FrameworkEnergyGrid.load_or_build(tmp_path, ff, p, fw.lattice, [sid], 1.0)
    assert hit2      # from the file just written, not a rebuild
    pts = np.array([[1.0 + i * 0.27, 2.0 + i * 0.19, 3.0 + i * 0.11] for i in range(50)])
    assert np.array_equal(first.interpolate(sid, pts), second.interpolate(sid, pts))
    assert np.array_equal(first.table(sid), second.table(sid))
