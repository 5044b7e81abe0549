"""Restart and forcing files (nsdg_restart_* in include/nsdg.h,
nextsimdg_gb300/restart.py): ParaGridIO's read and write sides without
netCDF or HDF5.

Pinned on the reference's own input file core/test/ParaGridIO_input_test.nc
(written by netCDF4-python through core/test/ParaGridIO_input_test.py; read
by the reference test "Test array ordering", core/test/ParaGrid_test.cpp:
478-519, which asserts index2d(3, 5) == 35).  The file's contents follow from
the generating script: on a 9 x 11 grid, index2d = 10 x + y, longitude = x,
latitude = y, one time record at 0 s, the "structure" type
"parametric_rectangular" and the metadata time "1970-01-01T00:00:00Z".  Its
HDF5 checksums (superblock, object headers, continuation chunks) are all
verified on the way, which also pins the lookup3 checksum; lookup3 itself is
checked against the published test values of Jenkins' lookup3.c driver.
Damaged files (truncated, flipped bytes, bad checksums) must give an error
status, never a crash: checked by mutating the fixture in child processes.
The writer (dumpModelState) is checked by reading its files back: no
netCDF-C or HDF5 library exists on either machine to read them
independently."""
import os
import shutil
import subprocess
import sys
import textwrap
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
def _fixture() -> Path:
    """The reference's ParaGridIO test input, core/test/ParaGridIO_input_test.nc,
    in the reference source tree ($NSDG_REFERENCE, else the location the
    oracle build recipe uses); read where that tree is present."""
    from oracle import pyref
    root = pyref.reference_root()
    return (root if root else Path("/nonexistent")) / "core" / "test" / "ParaGridIO_input_test.nc"


FIXTURE = _fixture()
needs_fixture = pytest.mark.skipif(not FIXTURE.exists(), reason="the reference's test input is not on this machine")


@pytest.fixture(scope="module")
def lib_built():
    from nextsimdg_gb300 import build
    build.build()


def test_lookup3_known_answers(tmp_path):
    src = tmp_path / "l3.cpp"
    src.write_text(textwrap.dedent("""
        #include "nsdg_restart.hpp"
        #include <cstdio>
        int main() {
            const char* s = "Four score and seven years ago";
            const uint8_t* e = reinterpret_cast<const uint8_t*>("");
            const uint8_t* f = reinterpret_cast<const uint8_t*>(s);
            std::printf("%08x %08x %08x %08x\\n", nsdg_nc::lookup3(e, 0, 0), nsdg_nc::lookup3(e, 0, 0xdeadbeef),
                nsdg_nc::lookup3(f, 30, 0), nsdg_nc::lookup3(f, 30, 1));
        }"""))
    exe = tmp_path / "l3"
    csrc = ROOT / "nextsimdg_gb300" / "csrc"
    subprocess.run([shutil.which("g++") or "g++", "-std=c++17", "-O2", "-I", str(csrc), str(src),
                    str(csrc / "nsdg_restart.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert out == ["deadbeef", "bd5b7dde", "17770551", "cd628161"]


@needs_fixture
def test_reference_input_file(lib_built):
    from nextsimdg_gb300.restart import ParaGridFile
    with ParaGridFile(FIXTURE) as f:
        assert f.structure_type() == "parametric_rectangular"
        assert f.text("metadata", "type") == "parametric_rectangular"
        assert f.metadata_time() == (0.0, "1970-01-01T00:00:00Z")
        assert f.text("metadata/time/formatted") == "1970-01-01T00:00:00Z"
        assert f.text("metadata/time/formatted", "format") == "%Y-%m-%dT%H:%M:%SZ"
        assert f.text("metadata/time/time", "units") == "seconds since 1970-01-01T00:00:00Z"
        vs = {v.name: v for v in f.variables("data")}
        assert list(vs) == ["longitude", "latitude", "time", "index2d"]
        assert vs["index2d"].dim_names == ("time", "y", "x")
        assert (vs["index2d"].model_type, vs["index2d"].n_records, vs["index2d"].n_values) == ("H", 1, 99)
        assert vs["longitude"].dim_names == ("y", "x") and vs["longitude"].model_type == "H"
        assert vs["time"].dim_names == ("time",) and vs["time"].model_type is None
        x, y = np.meshgrid(np.arange(9), np.arange(11))
        idx = f.read("data/index2d")
        np.testing.assert_array_equal(idx, (10 * x + y).ravel())
        # ModelArray index i + nx j: the reference's index2d(3, 5) == 35
        assert idx[3 + 9 * 5] == 35
        np.testing.assert_array_equal(f.read("data/longitude"), x.ravel())
        np.testing.assert_array_equal(f.read("data/latitude"), y.ravel())
        np.testing.assert_array_equal(f.read("data/time"), [0.0])


@needs_fixture
def test_read_forcing_time_static_and_get_model_state(lib_built):
    from nextsimdg_gb300.restart import ParaGridFile
    with ParaGridFile(FIXTURE) as f:
        for t in (-3600.0, 0.0, 86400.0):  # before, at and after the only record
            st = f.read_forcing_time_static({"index2d", "not_in_file"}, t)
            assert set(st) == {"index2d"}
            assert st["index2d"][3 + 9 * 5] == 35
        # the data group's "time" variable has no ModelArray type: the
        # reference's getModelState throws std::out_of_range for it
        with pytest.raises(KeyError, match="dimensional key time"):
            f.get_model_state()


@needs_fixture
def test_errors_are_statuses(lib_built, tmp_path):
    from nextsimdg_gb300._lib import NsdgError
    from nextsimdg_gb300.restart import ParaGridFile
    with pytest.raises(FileNotFoundError):
        ParaGridFile(tmp_path / "a44f5cc1f7934a8ae8dd03a95308745d.nc")
    (tmp_path / "text.nc").write_text("netcdf not really\n" * 8)
    with pytest.raises(NsdgError):
        ParaGridFile(tmp_path / "text.nc")
    b = bytearray(FIXTURE.read_bytes())
    b[0x40] ^= 0x01  # inside the root object header: its checksum no longer holds
    (tmp_path / "flip.nc").write_bytes(bytes(b))
    with pytest.raises(NsdgError, match="checksum"):
        ParaGridFile(tmp_path / "flip.nc")
    (tmp_path / "cut.nc").write_bytes(FIXTURE.read_bytes()[:0x800])
    with pytest.raises(NsdgError):
        with ParaGridFile(tmp_path / "cut.nc") as f:
            f.read("data/index2d")
    with ParaGridFile(FIXTURE) as f:
        with pytest.raises(KeyError):
            f.read("data/hice")
        with pytest.raises(KeyError):
            f.variables("nodata")


_PROBE = """
import sys
from nextsimdg_gb300.restart import ParaGridFile
from nextsimdg_gb300._lib import NsdgError
for p in sys.argv[1:]:
    try:
        with ParaGridFile(p) as f:
            for g in ("data", "metadata/time"):
                for v in f.variables(g):
                    try:
                        f.read(g + "/" + v.name) if v.n_values < 10**7 else None
                    except (NsdgError, KeyError):
                        pass
            f.structure_type()
    except (NsdgError, KeyError, FileNotFoundError, UnicodeDecodeError):
        pass
print("survived")
"""


@needs_fixture
def test_damaged_files_never_crash(lib_built, tmp_path):
    rng = np.random.default_rng(11)
    src = FIXTURE.read_bytes()
    paths = []
    for i in range(120):
        b = bytearray(src)
        for pos in rng.integers(0, len(b), rng.integers(1, 9)):
            b[pos] = int(rng.integers(0, 256))
        if i % 5 == 0:
            b = b[: int(rng.integers(48, len(b)))]
        p = tmp_path / f"m{i}.nc"
        p.write_bytes(bytes(b))
        paths.append(str(p))
    env = dict(os.environ, PYTHONPATH=str(ROOT))
    r = subprocess.run([sys.executable, "-c", _PROBE, *paths], capture_output=True, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0 and "survived" in r.stdout, r.stderr[-2000:]


def test_dump_model_state_round_trip(lib_built, tmp_path):
    """The writer (ParaGridIO::dumpModelState) and the reader agree bit for
    bit on every ModelArray type; only the reference's restart fields are
    written; dimension names and sizes follow the reference's
    definedDimensions; CG fields come back untyped because the reference's
    read key for them ("ycgxcg") does not match the names it writes
    ("y_cg", "x_cg"), kept as in the reference."""
    from nextsimdg_gb300.restart import ParaGridFile, dump_model_state
    nx, ny, nz = 13, 9, 3
    rng = np.random.default_rng(3)
    state = {
        "hice": ("DG", rng.random(nx * ny * 6)),
        "cice": ("DG", rng.random(nx * ny * 6)),
        "damage": ("DG", rng.random(nx * ny * 6)),
        "mask": ("H", (rng.random(nx * ny) > 0.2).astype(float)),
        "u": ("H", rng.standard_normal(nx * ny)),
        "coords": ("VERTEX", rng.random((nx + 1) * (ny + 1) * 2) * 1e6),
        "tice": ("Z", -rng.random(nx * ny * nz) * 10),
        "grid_azimuth": ("CG", rng.random((2 * nx + 1) * (2 * ny + 1))),
        "uwind": ("H", rng.random(nx * ny)),      # not a restart field
        "stress": ("DGSTRESS", rng.random(nx * ny * 8)),  # not a restart field
    }
    path = tmp_path / "restart.nc"
    written = dump_model_state(path, state, nx, ny, nz=nz, time_seconds=86400 * 3,
                               time_formatted="1970-01-04T00:00:00Z")
    assert written == ["cice", "coords", "damage", "grid_azimuth", "hice", "mask", "tice", "u"]
    with ParaGridFile(path) as f:
        assert f.structure_type() == "parametric_rectangular"
        assert f.metadata_time() == (259200.0, "1970-01-04T00:00:00Z")
        assert f.text("metadata/time/time", "units") == "seconds since 1970-01-01T00:00:00Z"
        assert f.variables("metadata/configuration") == []
        vs = {v.name: v for v in f.variables("data")}
        assert list(vs) == written  # dimension-only scales are not variables
        assert vs["hice"].dim_names == ("ydim", "xdim", "dg_comp") and vs["hice"].model_type == "DG"
        assert vs["hice"].n_components == 6
        assert vs["coords"].dim_names == ("yvertex", "xvertex", "ncoords") and vs["coords"].model_type == "VERTEX"
        assert vs["tice"].dim_names == ("zdim", "ydim", "xdim") and vs["tice"].model_type == "Z"
        assert vs["grid_azimuth"].dim_names == ("y_cg", "x_cg") and vs["grid_azimuth"].model_type is None
        for name in written:
            np.testing.assert_array_equal(f.read(f"data/{name}"), state[name][1])
        with pytest.raises(KeyError, match="y_cgx_cg"):
            f.get_model_state()
    # without the CG field, getModelState returns the state as written
    del state["grid_azimuth"]
    dump_model_state(path, state, nx, ny, nz=nz)
    with ParaGridFile(path) as f:
        got = f.get_model_state()
    assert set(got) == {"cice", "coords", "damage", "hice", "mask", "tice", "u"}
    for name, (mtype, arr) in got.items():
        expect = "H" if name in ("mask", "u") else state[name][0]
        assert mtype == expect
        np.testing.assert_array_equal(arr, state[name][1])


def test_writer_rejects_bad_sizes(lib_built, tmp_path):
    from nextsimdg_gb300._lib import NsdgError
    from nextsimdg_gb300.restart import dump_model_state
    with pytest.raises(NsdgError):
        dump_model_state(tmp_path / "bad.nc", {"hice": ("DG", np.zeros(10))}, 4, 4)
    with pytest.raises(NsdgError):
        dump_model_state(tmp_path / "no_such_dir" / "x.nc", {"hice": ("H", np.zeros(16))}, 4, 4)


def test_diagnostic_file_records(lib_built, tmp_path):
    """writeDiagnosticTime: one record per call along an unlimited time axis
    (chunked, one chunk per record; 70 records need a two-level chunk
    B-tree), mask and VERTEX written once (the mask with the (xdim, ydim)
    dimension order of the reference, which no dimension key maps to a
    type), a field left out of a record holds the fill value, a field new
    after the first record is refused, and readForcingTimeStatic picks the
    record at or before the requested time."""
    from nextsimdg_gb300.restart import DiagnosticFile, ParaGridFile
    nx, ny = 6, 4
    rng = np.random.default_rng(8)
    recs = []
    path = tmp_path / "diagnostic.nc"
    with DiagnosticFile(path, nx, ny) as d:
        for r in range(70):
            st = {"hice": ("DG", rng.random(nx * ny * 6)), "cice": ("H", rng.random(nx * ny)),
                  "mask": ("H", (rng.random(nx * ny) > 0.5).astype(float)),
                  "coords": ("VERTEX", rng.random((nx + 1) * (ny + 1) * 2))}
            if r == 5:
                del st["cice"]
            recs.append(st)
            d.write(st, 1800.0 * r)
        with pytest.raises(KeyError):
            d.write({"damage": ("DG", np.zeros(nx * ny * 6))}, 1e9)
    with ParaGridFile(path) as f:
        vs = {v.name: v for v in f.variables("data")}
        assert list(vs) == ["time", "cice", "coords", "hice", "mask"]
        assert vs["hice"].dim_names == ("time", "ydim", "xdim", "dg_comp")
        assert (vs["hice"].model_type, vs["hice"].n_records, vs["hice"].n_values) == ("DG", 70, nx * ny * 6)
        assert vs["mask"].dim_names == ("xdim", "ydim") and vs["mask"].model_type is None
        assert vs["coords"].dim_names == ("yvertex", "xvertex", "ncoords") and vs["coords"].n_records == 1
        np.testing.assert_array_equal(f.read("data/time"), 1800.0 * np.arange(70))
        for r in range(70):
            np.testing.assert_array_equal(f.read("data/hice", r), recs[r]["hice"][1])
            expect = np.full(nx * ny, 9.9692099683868690e+36) if r == 5 else recs[r]["cice"][1]
            np.testing.assert_array_equal(f.read("data/cice", r), expect)
        np.testing.assert_array_equal(f.read("data/mask"), recs[0]["mask"][1])
        np.testing.assert_array_equal(f.read("data/coords"), recs[0]["coords"][1])
        got = f.read_forcing_time_static({"hice", "cice"}, 1800.0 * 64 + 900.0)
        np.testing.assert_array_equal(got["hice"], recs[64]["hice"][1])
        got = f.read_forcing_time_static({"hice"}, 1e12)
        np.testing.assert_array_equal(got["hice"], recs[69]["hice"][1])


_PROBE_RECORDS = """
import sys
from nextsimdg_gb300.restart import ParaGridFile
from nextsimdg_gb300._lib import NsdgError
for p in sys.argv[1:]:
    try:
        with ParaGridFile(p) as f:
            for v in f.variables("data"):
                for rec in {0, v.n_records // 2, v.n_records - 1}:
                    try:
                        f.read("data/" + v.name, rec) if v.n_values < 10**7 else None
                    except (NsdgError, KeyError):
                        pass
            f.metadata_time()
    except (NsdgError, KeyError, FileNotFoundError, UnicodeDecodeError):
        pass
print("survived")
"""


def test_damaged_written_files_never_crash(lib_built, tmp_path):
    """The same robustness on the writer's own files, which hold the
    structures the reference's fixture lacks (a two-level chunk B-tree, many
    global heap references): damaged copies give statuses, never a crash."""
    from nextsimdg_gb300.restart import DiagnosticFile
    nx, ny = 5, 3
    rng = np.random.default_rng(21)
    src = tmp_path / "d.nc"
    with DiagnosticFile(src, nx, ny) as d:
        for r in range(70):
            d.write({"hice": ("DG", rng.random(nx * ny * 6)), "cice": ("H", rng.random(nx * ny))}, 60.0 * r)
    data = src.read_bytes()
    paths = []
    for i in range(100):
        b = bytearray(data)
        for pos in rng.integers(0, len(b), rng.integers(1, 9)):
            b[pos] = int(rng.integers(0, 256))
        if i % 5 == 0:
            b = b[: int(rng.integers(48, len(b)))]
        p = tmp_path / f"w{i}.nc"
        p.write_bytes(bytes(b))
        paths.append(str(p))
    env = dict(os.environ, PYTHONPATH=str(ROOT))
    r = subprocess.run([sys.executable, "-c", _PROBE_RECORDS, *paths], capture_output=True, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0 and "survived" in r.stdout, r.stderr[-2000:]


def test_restart_entry_points_from_c(lib_built, tmp_path):
    """tests/cpp/restart_capi_test.c: the nsdg_restart_* and
    nsdg_diagnostic_writer_* entry points compiled as C99 against
    include/nsdg.h and linked to the library, run without a GPU."""
    exe = tmp_path / "restart_capi_test"
    lib_dir = ROOT / "nextsimdg_gb300"
    subprocess.run([shutil.which("gcc") or "gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I",
                    str(ROOT / "include"), str(ROOT / "tests" / "cpp" / "restart_capi_test.c"), "-L", str(lib_dir),
                    "-lnsdg_gb300", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), str(tmp_path / "r.nc"), str(tmp_path / "d.nc")], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr


def test_paragrid_io_cpp_wrapper(lib_built, tmp_path):
    """tests/cpp/paragrid_io_test.cpp: include/nsdg_paragrid_io.hpp
    (Nextsim::GB300::ParaGridIO) compiled as C++17 and run without a GPU."""
    exe = tmp_path / "paragrid_io_test"
    lib_dir = ROOT / "nextsimdg_gb300"
    subprocess.run([shutil.which("g++") or "g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I",
                    str(ROOT / "include"), str(ROOT / "tests" / "cpp" / "paragrid_io_test.cpp"), "-L", str(lib_dir),
                    "-lnsdg_gb300", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr


_PROBE_OVERSIZED = """
import sys
from ctypes import c_void_p
import numpy as np
from nextsimdg_gb300.restart import ParaGridFile
n = int(sys.argv[2])
errors = 0
with ParaGridFile(sys.argv[1]) as f:
    buf = np.zeros(n)
    for name in ("u", "mask"):
        for rec in range(3):
            # a caller's buffer of the undamaged size, straight through the C ABI
            st = f._lib.nsdg_restart_read(f._h, ("data/" + name).encode(), rec, buf.ctypes.data_as(c_void_p), n)
            errors += st != 0
print("errors", errors)
"""


def _lookup3(data: bytes, initval: int = 0) -> int:
    """Bob Jenkins' lookup3 hashlittle (public domain), the HDF5 checksum."""
    M = 0xFFFFFFFF

    def rot(x, k):
        return ((x << k) | (x >> (32 - k))) & M

    n = len(data)
    a = b = c = (0xDEADBEEF + n + initval) & M
    i = 0
    while n - i > 12:
        a = (a + int.from_bytes(data[i:i + 4], "little")) & M
        b = (b + int.from_bytes(data[i + 4:i + 8], "little")) & M
        c = (c + int.from_bytes(data[i + 8:i + 12], "little")) & M
        a = ((a - c) & M) ^ rot(c, 4); c = (c + b) & M
        b = ((b - a) & M) ^ rot(a, 6); a = (a + c) & M
        c = ((c - b) & M) ^ rot(b, 8); b = (b + a) & M
        a = ((a - c) & M) ^ rot(c, 16); c = (c + b) & M
        b = ((b - a) & M) ^ rot(a, 19); a = (a + c) & M
        c = ((c - b) & M) ^ rot(b, 4); b = (b + a) & M
        i += 12
    if n - i == 0:
        return c
    tail = data[i:] + bytes(12 - (n - i))
    a = (a + int.from_bytes(tail[0:4], "little")) & M
    b = (b + int.from_bytes(tail[4:8], "little")) & M
    c = (c + int.from_bytes(tail[8:12], "little")) & M
    c ^= b; c = (c - rot(b, 14)) & M
    a ^= c; a = (a - rot(c, 11)) & M
    b ^= a; b = (b - rot(a, 25)) & M
    c ^= b; c = (c - rot(b, 16)) & M
    a ^= c; a = (a - rot(c, 4)) & M
    b ^= a; b = (b - rot(a, 14)) & M
    c ^= b; c = (c - rot(b, 24)) & M
    return c


def _reseal(b: bytearray, pos: int) -> None:
    """Recomputes the checksum of the version 2 object header ("OHDR", chunk
    0) that contains byte `pos`."""
    start = b.rfind(b"OHDR", 0, pos)
    assert start >= 0
    flags = b[start + 5]
    o = start + 6 + (16 if flags & 0x20 else 0) + (4 if flags & 0x10 else 0)
    w = 1 << (flags & 3)
    end = o + w + int.from_bytes(b[o:o + w], "little")
    assert start < pos < end
    b[end:end + 4] = _lookup3(bytes(b[start:end])).to_bytes(4, "little")


def test_oversized_dataspace_is_an_error(lib_built, tmp_path):
    """A damaged dataspace whose element count times the element size
    overflows 64 bits (dims [2^61 + 3, 13] of 8-byte values, the object
    header's checksum recomputed so that the damage is not caught there)
    must give an error status, never a read past the mapped file."""
    assert [_lookup3(b""), _lookup3(b"", 0xDEADBEEF), _lookup3(b"Four score and seven years ago"),
            _lookup3(b"Four score and seven years ago", 1)] == [0xDEADBEEF, 0xBD5B7DDE, 0x17770551, 0xCD628161]
    import struct
    from nextsimdg_gb300.restart import dump_model_state
    nx, ny = 13, 9
    rng = np.random.default_rng(4)
    path = tmp_path / "r.nc"
    dump_model_state(path, {"u": ("H", rng.standard_normal(nx * ny)), "mask": ("H", np.ones(nx * ny))}, nx, ny)
    data = path.read_bytes()
    pattern = struct.pack("<QQ", ny, nx)
    hits = [i for i in range(len(data) - 15) if data[i:i + 16] == pattern]
    assert hits, "no dataspace with the grid's dimensions found"
    env = dict(os.environ, PYTHONPATH=str(ROOT))
    for k, pos in enumerate(hits):
        b = bytearray(data)
        b[pos:pos + 8] = struct.pack("<Q", (1 << 61) + 3)
        _reseal(b, pos)
        p = tmp_path / f"o{k}.nc"
        p.write_bytes(bytes(b))
        r = subprocess.run([sys.executable, "-c", _PROBE_OVERSIZED, str(p), str(nx * ny)], capture_output=True,
                           text=True, env=env, timeout=120)
        assert r.returncode == 0 and "errors" in r.stdout, r.stderr[-2000:]
        assert int(r.stdout.split()[-1]) >= 1  # the damaged variable is refused
