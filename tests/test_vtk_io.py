"""The reference's file formats on the host (no GPU): frame files written
byte-identical to the reference's _writeData_, frame payloads read as its
_load3dDataArrayVTK_ reads them, centre files parsed as its _readData_
parses them (tests/golden/vtk_io.npz, made by the reference itself)."""
import os

import numpy as np
import pytest

from conftest import load_golden

VTK_HEADER = ("# vtk DataFile Version 3.0\nmovingBalls test frame\nBINARY\nDATASET STRUCTURED_POINTS\n"
              "DIMENSIONS {nx} {ny} {nz}\nORIGIN 0 0 0\nSPACING 0.5 0.25 1\nPOINT_DATA {n}\n"
              "SCALARS scalars unsigned_char\nLOOKUP_TABLE default\n")


def test_written_frames_match_reference(ss4d, tmp_path):
    d = load_golden("vtk_io.npz")
    nx, ny, nz, nt = (int(v) for v in d["dims"])
    org, sp = d["origin_spacing"][:3], d["origin_spacing"][3:]
    u = d["u_written"]
    for l in range(1, nt + 1):
        # the reference's conversion (unsigned char)(255 v + 0.5) for v in [0, 1]
        b = np.floor(255.0 * u[l, 1:-1, 1:-1, 1:-1] + 0.5).astype(np.uint8)
        path = str(tmp_path / f"f{l}.vtk")
        ss4d.vtk_write_frame(path, b, origin=org, spacing=sp)
        with open(path, "rb") as fh:
            assert np.array_equal(np.frombuffer(fh.read(), dtype=np.uint8), d["written"][l - 1]), f"frame {l}"


def test_read_frames_and_centres_match_reference(ss4d, tmp_path):
    d = load_golden("vtk_io.npz")
    nx, ny, nz, nt = (int(v) for v in d["dims"])
    sp = tuple(d["origin_spacing"][3:])
    cen = [tuple(c) for c in d["centres"]]
    for l in range(1, nt + 1):
        path = str(tmp_path / f"frame{l}.vtk")
        with open(path, "wb") as fh:
            fh.write(VTK_HEADER.format(nx=nx, ny=ny, nz=nz, n=nx * ny * nz).encode() + d["payloads"][l - 1].tobytes())
        b = ss4d.vtk_read_frame(path, nx, ny, nz)
        assert np.array_equal(b.reshape(-1), d["payloads"][l - 1])
        # the reference read the same bytes into i0 as byte / 255.
        assert np.array_equal(b / 255.0, d["i0_read"][l, 1:-1, 1:-1, 1:-1])
        cpath = str(tmp_path / f"centres{l}.vtk")
        with open(cpath, "w") as fh:
            fh.write(str(d["centre_texts"][l - 1]))
        got = ss4d.vtk_read_centers(cpath, sp)
        assert got == [c[1:] for c in cen if int(c[0]) == l], f"frame {l}"


def test_bad_files_are_refused(ss4d, tmp_path):
    path = str(tmp_path / "short.vtk")
    with open(path, "wb") as fh:
        fh.write(VTK_HEADER.format(nx=4, ny=4, nz=4, n=64).encode() + bytes(10))
    with pytest.raises(ss4d.SS4DError):
        ss4d.vtk_read_frame(path, 4, 4, 4)
    with pytest.raises(ss4d.SS4DError):
        ss4d.vtk_read_frame(str(tmp_path / "missing.vtk"), 4, 4, 4)
    cpath = str(tmp_path / "c.vtk")
    with open(cpath, "w") as fh:
        fh.write("# c\nx\nASCII\nDATASET POLYDATA\nPOINTS 3 float\n1 2 3\n4 5 6\n7 8 9\n")
    with pytest.raises(ss4d.SS4DError):
        ss4d.vtk_read_centers(cpath, max_points=2)
    assert ss4d.vtk_read_centers(cpath) == [(1.0, 2.0, 3.0), (4.0, 5.0, 6.0), (7.0, 8.0, 9.0)]
