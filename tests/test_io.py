"""The .ini parameters and HDF5 snapshot layout (include/fv2d_io.h), no GPU.

* .ini: inih line rules, the Reader's float rounding, map-valued errors; and,
  where the reference's sources are staged, every settings/*.ini read by this
  library equals the reference's own readInifile result (all parameters) and
  the echoed parameter file is byte-identical to Reader::outputValues.
* HDF5: snapshots written by the library are read back by its own reader and
  by an independent Python reader (tests/h5lite.py); both readers also parse
  a file written by libhdf5 itself (scipy's MATLAB v7.3 test file).
"""
import ctypes as C
import glob
import os

import numpy as np
import pytest

import fv2d_gb300 as fv
from fv2d_gb300._abi import Params
from fv2d_testlib import ref_available, ref_lib
from h5lite import H5

# the reference's sources as staged for the cross-check build (oracle/ref_check/stage.sh)
REF_DIR = os.environ.get("REF_DIR",
                         os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "baseline", "_ref"))


class RunConfig(C.Structure):
    _fields_ = [("problem", C.c_char * 64), ("output_filename", C.c_char * 256), ("output_path", C.c_char * 512),
                ("restart_file", C.c_char * 512), ("multiple_outputs", C.c_int32), ("problem_id", C.c_int32)]


def io_lib():
    L = fv.lib()
    L.fv2d_read_ini.argtypes = [C.c_char_p, C.POINTER(Params), C.POINTER(RunConfig), C.c_char_p, C.c_int]
    L.fv2d_write_ini_echo.argtypes = [C.c_char_p, C.c_char_p]
    L.fv2d_snapshot_write.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.POINTER(Params), C.c_char_p,
                                      C.c_int, C.c_double, C.POINTER(C.c_double), C.c_char_p, C.c_int]
    L.fv2d_snapshot_read.argtypes = [C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                     C.POINTER(C.c_int), C.c_char_p, C.c_int]
    L.fv2d_h5_read_doubles.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_double), C.c_int64,
                                       C.POINTER(C.c_int64)]
    L.fv2d_h5_read_attr.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(C.c_double)]
    return L


@pytest.fixture(scope="module")
def L():
    from fv2d_gb300 import build as b
    b.build()
    return io_lib()


def read_ini(L, path):
    p, r = Params(), RunConfig()
    err = C.create_string_buffer(1024)
    rc = L.fv2d_read_ini(path.encode(), C.byref(p), C.byref(r), err, 1024)
    return rc, p, r, err.value.decode(errors="replace")


def test_ini_rules(L, tmp_path):
    f = tmp_path / "a.ini"
    f.write_text("""; comment
# other comment
[MESH]
nx = 48
Ny : 24   ; inline comment
xmax=2.0
[solvers]
CFL=0.45
riemann_solver = hll
reconstruction=plm
[physics]
gamma0 = 1.4
problem = sod_x
[gravity]
mode=constant
gy = -0.1
[run]
boundaries_x = periodic
tend = 0.3
""")
    rc, p, r, err = read_ini(L, str(f))
    assert rc == 0, err
    assert (p.Nx, p.Ny) == (48, 24)
    assert p.xmax == 2.0
    assert p.CFL == float(np.float32(0.45))  # GetFloat goes through strtof
    assert p.gamma0 == float(np.float32(1.4))
    assert p.gy == float(np.float32(-0.1))
    assert p.riemann_solver == fv.HLL and p.reconstruction == fv.PLM and p.gravity_mode == fv.GRAV_CONSTANT
    assert p.boundary_x == fv.BC_PERIODIC and p.boundary_y == fv.BC_REFLECTING
    assert r.problem == b"sod_x" and r.problem_id == 0
    assert p.epsilon == float(np.float32(1e-6))  # default, also float


def test_ini_bad_map_value(L, tmp_path):
    f = tmp_path / "b.ini"
    f.write_text("[solvers]\nriemann_solver=roe\n")
    rc, _, _, err = read_ini(L, str(f))
    assert rc == fv._abi.ERR_INVALID
    assert err.startswith("bad parameter for riemann_solver") and "allowed values: fslp, hll, hllc" in err


def test_ini_string_too_long_for_its_field_is_refused(L, tmp_path):
    f = tmp_path / "long.ini"
    f.write_text("[run]\noutput_path=" + "d" * 511 + "\n")
    rc, _, r, _ = read_ini(L, str(f))
    assert rc == 0 and r.output_path == b"d" * 511  # the longest that fits
    f.write_text("[run]\noutput_path=" + "d" * 512 + "\n")
    rc, _, _, err = read_ini(L, str(f))
    assert rc == fv._abi.ERR_SIZE and err == "[run] output_path is longer than 511 bytes"
    f.write_text("[run]\nrestart_file=" + "r" * 600 + "\n")
    rc, _, _, err = read_ini(L, str(f))
    assert rc == fv._abi.ERR_SIZE and "restart_file" in err


REF_DUMP = ["Nx", "Ny", "Nghosts", "xmin", "xmax", "ymin", "ymax", "CFL", "boundary_x", "boundary_y",
            "reconstruction", "riemann_solver", "time_stepping", "tend", "save_freq", "gamma0", "epsilon",
            "epsilon_reset_negative", "well_balanced_flux_at_y_bc", "fslp_K", "seed", "log_frequency", "gravity_mode",
            "analytical_gravity_mode", "gx", "gy", "hot_bubble_g0", "thermal_conductivity_active",
            "thermal_conductivity_mode", "kappa", "bctc_ymin", "bctc_ymax", "bctc_ymin_value", "bctc_ymax_value",
            "viscosity_active", "viscosity_mode", "mu", "m1", "theta1", "m2", "theta2", "h84_pert", "c91_pert",
            "kh_a", "kh_amp", "kh_P0", "kh_rho_fac", "kh_sigma", "kh_uflow", "kh_y1", "kh_y2", "gresho_density",
            "gresho_Mach"]


@pytest.mark.skipif(not ref_available() or not os.path.isdir(os.path.join(REF_DIR, "settings")),
                    reason="reference checkout / cross-check build not present")
def test_ini_matches_reference_reader(L, tmp_path):
    R = ref_lib()
    R.fv2d_ref_echo.argtypes = [C.c_void_p, C.c_char_p]
    R.fv2d_ref_dump.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_int]
    files = sorted(glob.glob(os.path.join(REF_DIR, "settings", "*.ini")))
    assert len(files) >= 9
    for path in files:
        rc, p, r, err = read_ini(L, path)
        assert rc == 0, (path, err)
        h = R.fv2d_ref_create(path.encode())
        assert h
        vals = (C.c_double * 64)()
        n = R.fv2d_ref_dump(h, vals, 64)
        assert n == len(REF_DUMP)
        for k, name in enumerate(REF_DUMP):
            assert float(getattr(p, name)) == vals[k], (os.path.basename(path), name, getattr(p, name), vals[k])
        mine, theirs = tmp_path / "mine.ini", tmp_path / "ref.ini"
        assert L.fv2d_write_ini_echo(path.encode(), str(mine).encode()) == 0
        assert R.fv2d_ref_echo(h, str(theirs).encode()) == 0
        assert mine.read_text() == theirs.read_text(), os.path.basename(path)
        R.fv2d_ref_destroy(h)


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def write(L, d, name, multiple, trunc, p, problem, it, t, q):
    err = C.create_string_buffer(512)
    rc = L.fv2d_snapshot_write(str(d).encode(), name.encode(), multiple, trunc, C.byref(p), problem.encode(), it, t,
                               _dp(q), err, 512)
    assert rc == 0, err.value


def read(L, file, nx, ny):
    q = np.empty((ny, nx, 4))
    t, it = C.c_double(), C.c_int()
    err = C.create_string_buffer(512)
    rc = L.fv2d_snapshot_read(file.encode(), nx, ny, _dp(q), C.byref(t), C.byref(it), err, 512)
    return rc, q, t.value, it.value, err.value.decode()


def test_unique_file_roundtrip(L, tmp_path):
    nx, ny = 12, 7
    p = fv.default_params(Nx=nx, Ny=ny, xmin=-0.5, xmax=0.7, ymin=0.1, ymax=0.45)
    rng = np.random.default_rng(3)
    qs = [rng.uniform(0.1, 2.0, (ny, nx, 4)) for _ in range(3)]
    times = [0.0, 0.0125, 0.25]
    for k in range(3):
        write(L, tmp_path, "run", 0, 1 if k == 0 else 0, p, "blast", k, times[k], qs[k])
    f = str(tmp_path / "run.h5")
    # this library's reader: the latest group, then each group by name
    rc, q, t, it, err = read(L, f, nx, ny)
    assert rc == 0, err
    assert it == 2 and t == 0.25 and np.array_equal(q, qs[2])
    for k in range(3):
        rc, q, t, it, _ = read(L, f + ":/ite_%04d" % k, nx, ny)
        assert rc == 0 and it == k and t == times[k] and np.array_equal(q, qs[k])
    rc, _, _, _, err = read(L, f, nx + 1, ny)
    assert rc != 0 and "different resolution" in err
    # independent reader
    h = H5(f)
    assert sorted(h.links(h.root)) == ["ite_0000", "ite_0001", "ite_0002", "x", "y"]
    ra = h.attrs("/")
    assert (ra["Ntx"], ra["Nty"], ra["Nx"], ra["Ny"], ra["ibeg"], ra["iend"], ra["jbeg"], ra["jend"]) == \
        (nx + 4, ny + 4, nx, ny, 2, nx + 2, 2, ny + 2)
    assert ra["problem"].split(b"\0")[0] == b"blast"
    x, y = h.dataset("/x"), h.dataset("/y")
    assert x.shape == ((nx + 1) * (ny + 1),)
    dx = (0.7 - -0.5) / nx
    assert x[1] == 1 * dx + -0.5 and y[nx + 1] == 1 * ((0.45 - 0.1) / ny) + 0.1
    for k in range(3):
        g = "/ite_%04d/" % k
        a = h.attrs(g)
        assert a["time"] == times[k] and a["iteration"] == k
        for f_, name in enumerate(["rho", "u", "v", "prs"]):
            assert np.array_equal(h.dataset(g + name), qs[k][..., f_].ravel())
    assert h.eof == os.path.getsize(f)
    xmf = (tmp_path / "run.xmf").read_text()
    assert xmf.count("<Grid Name=\"ite_") == 3 and xmf.rstrip().endswith("</Xdmf>")
    assert "&file;/ite_0002/rho" in xmf


def test_multiple_output_files(L, tmp_path):
    nx, ny = 5, 9
    p = fv.default_params(Nx=nx, Ny=ny)
    q = np.random.default_rng(4).uniform(0.5, 1.5, (ny, nx, 4))
    write(L, tmp_path, "snap", 1, 1, p, "sod_x", 7, 0.5, q)
    f = str(tmp_path / "snap_0007.h5")
    rc, q2, t, it, err = read(L, f, nx, ny)
    assert rc == 0, err
    assert t == 0.5 and it == 7 and np.array_equal(q, q2)
    h = H5(f)
    assert sorted(h.links(h.root)) == ["prs", "rho", "u", "v", "x", "y"]
    assert h.attrs("/")["iteration"] == 7
    assert (tmp_path / "snap_0007.xmf").exists()


def _matlab_file():
    try:
        import scipy
    except ImportError:
        return None
    f = os.path.join(os.path.dirname(scipy.__file__), "io", "matlab", "tests", "data", "testhdf5_7.4_GLNX86.mat")
    return f if os.path.exists(f) else None


@pytest.mark.skipif(_matlab_file() is None, reason="no libhdf5-written file available")
def test_readers_parse_a_libhdf5_file(L):
    """A file written by libhdf5 (512-byte user block, superblock v0,
    symbol-table groups): both readers recover the same dataset."""
    f = _matlab_file()
    h = H5(f)
    ref = h.dataset("/testdouble").ravel()
    assert np.allclose(ref, np.linspace(0, 2 * np.pi, 9))
    n = C.c_int64()
    out = np.empty(64)
    assert L.fv2d_h5_read_doubles(f.encode(), b"/testdouble", _dp(out), 64, C.byref(n)) == 0
    assert n.value == 9 and np.array_equal(out[:9], ref)


def test_damaged_snapshot_files_are_reported_not_read(L, tmp_path):
    """A restart from a truncated, overwritten or non-HDF5 file returns an
    error code and a message; it never reads past the file or crashes."""
    nx, ny = 12, 7
    p = fv.default_params(Nx=nx, Ny=ny)
    q = np.random.default_rng(5).uniform(0.1, 2.0, (ny, nx, 4))
    write(L, tmp_path, "run", 0, 1, p, "blast", 0, 0.0, q)
    good = tmp_path / "run.h5"
    data = good.read_bytes()
    cases = {
        "empty.h5": b"",
        "text.h5": b"not an hdf5 file\n" * 40,
        "sig_only.h5": data[:8],
    }
    for frac in (0.1, 0.3, 0.5, 0.8, 0.95):
        cases[f"cut{int(frac * 100)}.h5"] = data[:int(len(data) * frac)]
    rng = np.random.default_rng(9)
    for k in range(4):  # random bytes overwritten after the superblock
        b = bytearray(data)
        pos = rng.integers(64, len(b), 32)
        for i in pos:
            b[i] = int(rng.integers(0, 256))
        cases[f"noise{k}.h5"] = bytes(b)
    for name, blob in cases.items():
        f = tmp_path / name
        f.write_bytes(blob)
        rc, _, _, _, err = read(L, str(f) + ":/ite_0000", nx, ny)
        if name.startswith("noise") and rc == 0:
            continue  # the overwritten bytes may have missed every structure that is read
        assert rc != 0 and err, name
    rc, q2, t, it, err = read(L, str(good) + ":/ite_0000", nx, ny)
    assert rc == 0 and np.array_equal(q2, q), err


FUZZ_SCRIPT = r"""
import sys, ctypes as C
import numpy as np
sys.path[:0] = [{repo!r}, {tests!r}]
from test_io import io_lib, read
L = io_lib()
good, path, nx, ny = {good!r}, {path!r}, {nx}, {ny}
data = open(good, "rb").read()
rng = np.random.default_rng(23)
cases = [data[:cut] for cut in range(0, len(data), max(1, len(data) // 300))]
for k in range(800):  # a few random bytes anywhere
    b = bytearray(data)
    for i in rng.integers(0, len(b), int(rng.integers(1, 9))):
        b[i] = int(rng.integers(0, 256))
    cases.append(bytes(b))
for k in range(400):  # an aligned 8-byte field set to an extreme or self-referring value
    b = bytearray(data)
    off = int(rng.integers(0, len(b) - 8)) & ~7
    vals = [2**63, 2**64 - 1, 2**32, 2**16 - 1, len(data), off, off - 16 if off >= 16 else 0, 0]
    v = vals[int(rng.integers(0, len(vals)))]
    b[off:off + 8] = v.to_bytes(8, "little")
    cases.append(bytes(b))
for k in range(400):  # a 2-byte field (message sizes, counts) set to an extreme value
    b = bytearray(data)
    off = int(rng.integers(0, len(b) - 2)) & ~1
    vals = [0, 1, 0xFFFF, 0x8000, 8, 16]
    b[off:off + 2] = vals[int(rng.integers(0, len(vals)))].to_bytes(2, "little")
    cases.append(bytes(b))
for v in (0, 1, 3, 5, 16, 255):  # superblock offset / length sizes
    for pos in (13, 14):
        b = bytearray(data)
        b[pos] = v
        cases.append(bytes(b))
out = (C.c_double * (4 * nx * ny))()
n = C.c_int64()
import os
import fv2d_gb300 as fv
prm = fv.default_params(Nx=nx, Ny=ny)
q = np.ones((ny, nx, 4))
qp = q.ctypes.data_as(C.POINTER(C.c_double))
err = C.create_string_buffer(256)
xmf = open(good[:-3] + ".xmf", "rb").read()
read_ok = append_ok = 0
for k, blob in enumerate(cases):
    open(path, "wb").write(blob)
    rc = read(L, path + ":/ite_0000", nx, ny)[0]
    read_ok += rc == 0
    for ds in (b"/ite_0000/rho", b"/x", b"/ite_0000"):
        L.fv2d_h5_read_doubles(path.encode(), ds, out, 4 * nx * ny, C.byref(n))
    if k % 4 == 0:  # appending a snapshot parses the existing root group
        open(path[:-3] + ".xmf", "wb").write(xmf)
        rc = L.fv2d_snapshot_write(os.path.dirname(path).encode(), b"fuzz", 0, 0, C.byref(prm), b"blast", 1, 0.5,
                                   qp, err, 256)
        append_ok += rc == 0
print("done", len(cases), read_ok, append_ok, flush=True)
"""


def test_snapshot_reader_survives_malformed_files(L, tmp_path):
    """Some 2000 malformed variants of a snapshot (truncations; random bytes;
    offsets, lengths and counts set to extreme or self-referring values;
    unsupported offset sizes) are read -- and a quarter of them appended to --
    in a child process: every call returns, with an error or a result, and
    the process neither crashes nor loops (the reader bounds every read by
    the file and every walk)."""
    import subprocess
    import sys
    nx, ny = 12, 7
    p = fv.default_params(Nx=nx, Ny=ny)
    q = np.random.default_rng(5).uniform(0.1, 2.0, (ny, nx, 4))
    write(L, tmp_path, "run", 0, 1, p, "blast", 0, 0.0, q)
    here = os.path.dirname(os.path.abspath(__file__))
    script = FUZZ_SCRIPT.format(repo=os.path.dirname(here), tests=here, good=str(tmp_path / "run.h5"),
                                path=str(tmp_path / "fuzz.h5"), nx=nx, ny=ny)
    r = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout[-500:], r.stderr[-2000:])
    assert r.stdout.startswith("done"), r.stdout


INI_FUZZ_SCRIPT = r"""
import sys, ctypes as C
import numpy as np
sys.path[:0] = [{repo!r}, {tests!r}]
from test_io import io_lib, read_ini
L = io_lib()
base = open({base!r}, "rb").read()
path, echo = {path!r}, {echo!r}
rng = np.random.default_rng(31)
lines = base.split(b"\n")
cases = [base[:cut] for cut in range(0, len(base), 7)]
for k in range(600):  # random bytes anywhere (NULs, high bytes, brackets, separators)
    b = bytearray(base)
    for i in rng.integers(0, len(b), int(rng.integers(1, 12))):
        b[i] = int(rng.choice([0, 10, 13, 32, 59, 35, 61, 58, 91, 93, 255, int(rng.integers(0, 256))]))
    cases.append(bytes(b))
for k in range(300):  # lines dropped, repeated, indented (continuations) or made very long
    out = []
    for ln in lines:
        r = rng.random()
        if r < 0.1:
            continue
        if r < 0.2:
            out += [ln, ln]
        elif r < 0.3:
            out.append(b"   " + ln)
        elif r < 0.35:
            out.append(ln + b"9" * int(rng.integers(100, 5000)))
        else:
            out.append(ln)
    cases.append(b"\n".join(out))
for v in (b"1e999", b"-1e999", b"nan", b"0x7fffffffffffffff", b"-", b"", b"2147483648", b"-2147483649"):
    for key in (b"Nx", b"CFL", b"tend", b"seed", b"log_frequency"):
        cases.append(base.replace(b"Nx=64", key + b"=" + v))
codes = set()
for data in cases:
    open(path, "wb").write(data)
    rc = read_ini(L, path)[0]
    codes.add(rc)
    L.fv2d_write_ini_echo(path.encode(), echo.encode())
assert codes <= {{0, 1, 7}}, codes
print("done", len(cases), sorted(codes))
"""


def test_ini_reader_survives_malformed_files(L, tmp_path):
    """About 1000 malformed variants of an .ini file (truncations; random bytes
    including NULs and separators; lines dropped, repeated, indented or made
    thousands of characters long; extreme and non-numeric values) are read
    and echoed in a child process: every call returns FV2D_OK,
    FV2D_ERR_INVALID or FV2D_ERR_SIZE, and the process does not crash."""
    import subprocess
    import sys
    base = tmp_path / "base.ini"
    base.write_text("[mesh]\nNx=64\nNy=8\nxmin=0.0\nxmax=1.0\n\n[run]\ntend=0.05\nsave_freq=0.01\n"
                    "boundaries_x=absorbing\nboundaries_y=periodic\noutput_path=out\noutput_filename=run\n"
                    "restart_file=\n\n[solvers]\nriemann_solver=hllc\nreconstruction=plm\nCFL=0.8\n\n"
                    "[physics]\ngamma0=1.4\nproblem=sod_x\n\n[misc]\nlog_frequency=3\nseed=12345\n")
    here = os.path.dirname(os.path.abspath(__file__))
    script = INI_FUZZ_SCRIPT.format(repo=os.path.dirname(here), tests=here, base=str(base),
                                    path=str(tmp_path / "fuzz.ini"), echo=str(tmp_path / "echo.ini"))
    r = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, errors="replace",
                       timeout=300)  # the warnings quote the malformed keys
    assert r.returncode == 0, (r.returncode, r.stdout[-500:], r.stderr[-2000:])
    assert r.stdout.startswith("done"), r.stdout
    assert int(r.stdout.split()[1]) >= 900


def _reference_xdmf_strings():
    """The XDMF format strings of the reference's IOManager.h (raw-string literals)."""
    import re
    path = os.path.join(REF_DIR, "IOManager.h")
    if not os.path.exists(path):
        return None
    text = open(path).read()
    out = {}
    for m in re.finditer(r'char (str_xdmf_\w+)\[\] =\s*R"xml\((.*?)\)xml";', text, flags=re.S):
        out[m.group(1)] = m.group(2)
    return out


@pytest.mark.skipif(_reference_xdmf_strings() is None, reason="reference checkout not present")
def test_xdmf_sidecars_are_byte_identical_to_the_references(L, tmp_path):
    """The XDMF files that saveSolutionUnique / saveSolutionMultiple
    (IOManager.h:107-279) write -- their printf formats applied in the same
    order, including the unique mode's rewind of sizeof(footer) bytes before
    each new grid -- against the library's files for the same snapshots."""
    S = _reference_xdmf_strings()
    c = lambda s: s.replace("%lf", "%f")  # noqa: E731  (C's %lf is %f)

    def fields(group):
        return (c(S["str_xdmf_scalar_field"]) % ("rho", group, "rho") +
                c(S["str_xdmf_vector_field"]) % ("velocity", group, "u", group, "v") +
                c(S["str_xdmf_scalar_field"]) % ("prs", group, "prs") + S["str_xdmf_ite_footer"])

    d = tmp_path
    nx, ny = 12, 7
    p = fv.default_params(Nx=nx, Ny=ny)
    q = np.ones((ny, nx, 4))
    times = [0.0, 0.0125, 1.0 / 3.0]
    footer = S["str_xdmf_footer"]
    # unique file: header + footer, then per snapshot a rewind of sizeof(footer) = len + 1 bytes
    ref = bytearray((c(S["str_xdmf_header"]) % ("run.h5", ny, nx, ny + 1, nx + 1) + footer).encode())
    for k, t in enumerate(times):
        write(L, d, "run", 0, 1 if k == 0 else 0, p, "blast", k, t, q)
        name = "ite_%04d" % k
        del ref[len(ref) - (len(footer) + 1):]
        ref += (c(S["str_xdmf_ite_header"]) % (name, t) + fields(name + "/") + footer).encode()
    assert (d / "run.xmf").read_bytes() == bytes(ref)
    # one file per snapshot
    write(L, d, "snap", 1, 1, p, "sod_x", 7, 0.5, q)
    ref = (c(S["str_xdmf_header"]) % ("snap_0007.h5", ny, nx, ny + 1, nx + 1) +
           c(S["str_xdmf_ite_header"]) % ("snap_0007", 0.5) + fields("") + footer)
    assert (d / "snap_0007.xmf").read_bytes() == ref.encode()
