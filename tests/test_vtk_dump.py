"""VTK / LAMMPS dump files of the phafd_gpu interpreter, byte for byte against
a Python restatement of the reference writer (src/dump.cpp).

A small C++ driver (tests/vtk_dump_driver.cpp) writes every dump kind from
fixed synthetic beads and fields through phafd_gb300/host/vtk_dump.hpp; the
expected bytes below follow dump.cpp's stream output.  C++ ostream formatting
of a double is printf %g by default (precision 6), %.Nf under std::fixed with
setprecision(N), %.Ne under std::scientific (N = 6 unless set)."""
import os
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
XML = '<?xml version="1.0"?>\n'


def vtkfile(kind):
    return '<VTKFile type="%s"  version="1.0" byte_order="LittleEndian">\n' % kind


@pytest.fixture(scope="module")
def written(tmp_path_factory):
    d = tmp_path_factory.mktemp("dump")
    exe = str(d / "driver")
    try:
        subprocess.check_call(["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "phafd_gb300", "host"), "-o",
                               exe, os.path.join(ROOT, "tests", "vtk_dump_driver.cpp")])
    except (OSError, subprocess.CalledProcessError) as e:  # pragma: no cover
        pytest.skip("cannot compile the dump driver: %s" % e)
    (d / "sub").mkdir()
    subprocess.check_call([exe, str(d)])
    return d


def scene():
    """The driver's synthetic data (tests/vtk_dump_driver.cpp)."""
    n = 5
    i = np.arange(3 * n)
    x = -3.25 + 1.0 / 3.0 * i
    ux = 100.0 * x + 1e-7 * i
    f = np.where(i % 2 == 1, -1.0, 1.0) * 1.2345678901e-5 * (i + 1)
    j = np.arange(n)
    ints = dict(ix=512 * 512 * (j % 3) + j, ID=j + 1, molID=j // 3, type=j % 2, label=np.zeros(n, int))
    nx, ny, nz = 3, 4, 5
    k = np.arange(nx * ny * nz)
    fields = dict(phi=0.5 + 0.01 * k, chempot=-1.0 / (k + 1))
    box = [(-16.0, 16.0), (-16.0, 17.0), (-16.0, 18.0)]
    return dict(n=n, x=x, ux=ux, F=f, ints=ints, nx=nx, ny=ny, nz=nz, fields=fields, box=box,
                origin=(-1.5, -2.0, -2.5), spacing=(1.0, 1.0, 1.0))


def num(v, precision=-1, fmt="lf"):
    """One double through the stream settings of dump.cpp:362-368."""
    if precision > 0 and fmt == "lf":
        return "%.*f" % (precision, v)
    if precision > 0 and fmt == "e":
        return "%.*e" % (precision, v)
    if fmt == "e":
        return "%e" % v
    return "%g" % v


def data_array3(name, a, n, p, fmt):  # dump.cpp:1010-1048
    body = "".join("%s %s %s " % (num(a[3 * i], p, fmt), num(a[3 * i + 1], p, fmt), num(a[3 * i + 2], p, fmt))
                   for i in range(n))
    return ('<DataArray Name="%s" type="Float64" NumberOfComponents="3" format="ascii">\n' % name + body +
            "\n</DataArray>\n")


def data_array1(name, a):  # dump.cpp:1053-1090
    return ('<DataArray Name="%s" type="Int64" NumberOfComponents="1" format="ascii">\n' % name +
            "".join("%d " % v for v in a) + "\n</DataArray>\n")


def pdata_array(name, three):
    if three:
        return '<PDataArray Name="%s" type="Float64" NumberOfComponents="3" format="ascii"/>\n' % name
    return '<PDataArray Name="%s" type="Int64" NumberOfComponents="1" format="ascii"/>\n' % name


def expect_vtp(s, attrs, p, fmt):  # write_atom_timestep, dump.cpp:343-408
    out = XML + vtkfile("PolyData") + "<PolyData>\n" + '<Piece NumberOfPoints="%d" NumberOfLines="1">\n' % s["n"]
    out += "<Points>\n" + data_array3("x", s["x"], s["n"], p, fmt) + "</Points>\n<PointData>\n"
    for w in attrs:
        if w in ("F", "ux"):
            out += data_array3(w, s[w], s["n"], p, fmt)
        elif w != "x":
            out += data_array1(w, s["ints"][w])
    return out + "</PointData>\n</Piece>\n</PolyData>\n</VTKFile>\n"


def expect_pvtp(attrs, source):  # write_atom_timestep_pvtp, dump.cpp:411-480
    out = XML + vtkfile("PPolyData") + '<PPolyData GhostLevel="0">\n<PPoints>\n' + pdata_array("x", True)
    out += "</PPoints>\n<PPointData>\n"
    for w in attrs:
        if w != "x":
            out += pdata_array(w, w in ("F", "ux"))
    return out + '</PPointData>\n<Piece Source="%s"/>\n</PPolyData>\n</VTKFile>\n' % source


def expect_pvd(base, steps, dt, ext):  # dump.cpp:235-309
    out = XML + vtkfile("Collection") + "<Collection>\n"
    for t in steps:
        out += '<DataSet timestep="%s" group="" part="0" file="%s_%d.p%s"/>\n' % (num(t * dt), base, t, ext)
    return out + "</Collection>\n</VTKFile>"


def expect_lammps(s, attrs, steps, p, fmt):  # write_lammps_dump, dump.cpp:484-668
    out = ""
    names = {"x": "x y z ", "F": "Fx Fy Fz ", "ux": "ux uy uz "}
    for t in steps:
        out += "ITEM: TIMESTEP\n%d\nITEM: NUMBER OF ATOMS\n%d\nITEM: BOX BOUNDS pp pp pp\n" % (t, s["n"])
        for lo, hi in s["box"]:
            out += "%s %s\n" % (num(lo, p, fmt), num(hi, p, fmt))
        out += "ITEM: ATOMS " + "".join(names.get(w, w + " ") for w in attrs) + "\n"
        for i in range(s["n"]):
            for w in attrs:
                if w in ("x", "F", "ux"):
                    out += "%s %s %s " % tuple(num(s[w][3 * i + c], p, fmt) for c in range(3))
                else:
                    out += "%d " % s["ints"][w][i]
            out += "\n"
    return out


def expect_vti(s, attrs):
    """write_grid_timestep (dump.cpp:681-783) for one domain holding all Nz
    planes: extent 0 .. Nz-1, Nx*Ny*Nz doubles after each UInt32 length."""
    nx, ny, nz = s["nx"], s["ny"], s["nz"]
    o, h = s["origin"], s["spacing"]
    nbytes = nx * ny * nz * 8
    head = XML + vtkfile("ImageData")
    head += '<ImageData WholeExtent="0 %d 0 %d 0  %d" Origin="%s %s %s " Spacing="%s %s %s ">\n' % (
        nx - 1, ny - 1, nz - 1, *map(num, o), *map(num, h))
    head += '<Piece Extent="0 %d 0 %d 0 %d">\n<PointData Scalars="scalars">\n' % (nx - 1, ny - 1, nz - 1)
    for c, w in enumerate(attrs):
        head += '<DataArray Name="%s" type="Float64" format="appended" offset="%d"/>\n' % (w, c * (nbytes + 4))
    head += '</PointData>\n</Piece>\n</ImageData>\n<AppendedData encoding="raw">\n_'
    raw = b"".join(struct.pack("<I", nbytes) + np.asarray(s["fields"][w], "<f8").tobytes() for w in attrs)
    return head.encode() + raw + b"\n</AppendedData>\n</VTKFile>\n"


def expect_pvti(s, attrs, source):  # write_grid_timestep_pvti, dump.cpp:786-867
    nx, ny, nz = s["nx"], s["ny"], s["nz"]
    o, h = s["origin"], s["spacing"]
    out = XML + vtkfile("PImageData")
    out += '<PImageData WholeExtent="0 %d 0 %d  0 %d" Origin="%s %s %s " Spacing="%s %s %s" GhostLevel="1">\n' % (
        nx - 1, ny - 1, nz - 1, *map(num, o), *map(num, h))
    out += '<PPointData Scalars="scalars">\n'
    out += "".join('<PDataArray Name="%s" type="Float64"/>\n' % w for w in attrs)
    out += '</PPointData>\n<Piece Extent="0 %d 0 %d 0 %d" Source="%s"/>\n' % (nx, ny, nz - 1, source)
    return out + "\n</PImageData>\n</VTKFile>\n"


ATOM_CASES = [  # base (under the output directory), attributes, decimalplaces, fmt
    ("sub/atoms", ["x", "ux", "F", "ix", "ID", "molID", "type", "label"], -1, "lf"),
    ("atoms2", ["x", "F"], 4, "e"),
    ("atoms3", ["x"], 3, "lf"),
    ("atoms4", ["x"], -1, "e"),
]


@pytest.mark.parametrize("base,attrs,p,fmt", ATOM_CASES)
def test_atom_dumps_match_reference_format(written, base, attrs, p, fmt):
    s = scene()
    nopath = base.split("/")[-1]
    assert (written / (base + ".pvd")).read_text() == expect_pvd(nopath, [0, 10], 1e-3, "vtp")
    for t in (0, 10):
        assert (written / ("%s_p0_%d.vtp" % (base, t))).read_text() == expect_vtp(s, attrs, p, fmt)
        assert (written / ("%s_%d.pvtp" % (base, t))).read_text() == expect_pvtp(
            attrs, "%s_p0_%d.vtp" % (nopath, t))


def test_grid_dump_matches_reference_format(written):
    s = scene()
    attrs = ["phi", "chempot"]
    assert (written / "grid.pvd").read_text() == expect_pvd("grid", [0, 10], 1e-3, "vti")
    for t in (0, 10):
        got = (written / ("grid_p0_%d.vti" % t)).read_bytes()
        assert got == expect_vti(s, attrs)
        assert (written / ("grid_%d.pvti" % t)).read_text() == expect_pvti(s, attrs, "grid_p0_%d.vti" % t)


def test_grid_dump_appended_arrays_read_back(written):
    """The raw appended block holds each field in [z][y][x] order after its
    UInt32 byte count, at the offsets the DataArray headers name."""
    s = scene()
    got = (written / "grid_p0_0.vti").read_bytes()
    start = got.index(b'<AppendedData encoding="raw">\n_') + len(b'<AppendedData encoding="raw">\n_')
    n = s["nx"] * s["ny"] * s["nz"]
    for c, w in enumerate(["phi", "chempot"]):
        at = start + c * (8 * n + 4)
        assert struct.unpack_from("<I", got, at)[0] == 8 * n
        np.testing.assert_array_equal(np.frombuffer(got, "<f8", n, at + 4), s["fields"][w])


def test_lammps_dump_matches_reference_format(written):
    s = scene()
    assert not (written / "lmp.pvd").exists()
    assert (written / "lmp_p0.lmmpstrj").read_text() == expect_lammps(s, ["ID", "type", "x", "F"], [0, 10], -1,
                                                                       "lf")


def test_ftgrid_dump_matches_reference_format(written):
    """dump ftgrid of a per_ftgrid compute (dump.cpp:681-867 with the ftgrid
    branch): dimensions of the transposed half spectrum, spacing dq, origin 0."""
    sk = 1.0 / (np.arange(4 * 5 * 4) + 3)
    s = dict(nx=4, ny=5, nz=4, origin=(0.0, 0.0, 0.0),
             spacing=(2 * 3.141592 / 12.0, 2 * 3.141592 / 10.0, 2 * 3.141592 / 8.0), fields={"c_sk": sk})
    assert (written / "spec.pvd").read_text() == expect_pvd("spec", [5], 1e-3, "vti")
    assert (written / "spec_p0_5.vti").read_bytes() == expect_vti(s, ["c_sk"])
    assert (written / "spec_5.pvti").read_text() == expect_pvti(s, ["c_sk"], "spec_p0_5.vti")
