"""Frame files through the GPU: bytes -> frame (byte / 255.) and frame ->
bytes ((unsigned char)(255 v + 0.5), and the v >= 0.5 mask) on the device,
and the reference-named _readData_ / _writeData_ / _load3dDataArrayVTK_
against the reference's own results (tests/golden/vtk_io.npz)."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import load_golden
from test_vtk_io import VTK_HEADER

pytestmark = pytest.mark.gpu


def test_frame_byte_conversions_match_reference(ss4d, cuda):
    torch = cuda
    d = load_golden("vtk_io.npz")
    nx, ny, nz, nt = (int(v) for v in d["dims"])
    shape = d["i0_read"].shape
    img = torch.full(shape, -1.0, dtype=torch.float64, device="cuda")
    u = torch.from_numpy(d["u_written"]).cuda()
    with ss4d.Solver(*shape[::-1]) as S:
        for l in range(1, nt + 1):
            S.frame_from_bytes(img, l, torch.from_numpy(d["payloads"][l - 1]).cuda())
        for l in range(1, nt + 1):
            b = torch.zeros(nx * ny * nz, dtype=torch.uint8, device="cuda")
            S.frame_to_bytes(u, l, b, mode=0)
            m = torch.zeros_like(b)
            S.frame_to_bytes(u, l, m, mode=1)
            S.synchronize()
            assert np.array_equal(b.cpu().numpy(), d["written"][l - 1][-nx * ny * nz:]), f"frame {l}"
            want_m = (d["u_written"][l, 1:-1, 1:-1, 1:-1] >= 0.5).astype(np.uint8).reshape(-1)
            assert np.array_equal(m.cpu().numpy(), want_m)
        with pytest.raises(ss4d.SS4DError):
            S.frame_to_bytes(u, 0, torch.zeros(8, dtype=torch.uint8, device="cuda"))
    assert np.array_equal(img.cpu().numpy(), d["i0_read"])  # ghosts untouched (-1)


def test_reference_named_file_functions(ss4d, cuda, tmp_path):
    d = load_golden("vtk_io.npz")
    nx, ny, nz, nt = (int(v) for v in d["dims"])
    shape = d["i0_read"].shape
    lM, kM, jM, iM = shape
    for l in range(1, nt + 1):
        with open(tmp_path / ("movingBalls_457_at_time_%03d.vtk" % l), "wb") as fh:
            fh.write(VTK_HEADER.format(nx=nx, ny=ny, nz=nz, n=nx * ny * nz).encode() + d["payloads"][l - 1].tobytes())
        with open(tmp_path / ("movingBalls_457_centers_at_timestep_%03d.vtk" % l), "w") as fh:
            fh.write(str(d["centre_texts"][l - 1]))
    L = C.CDLL(ss4d.SEG_PATH, mode=os.RTLD_LOCAL)
    for nm, v in (("iMax", iM), ("jMax", jM), ("kMax", kM), ("lMax", lM)):
        C.c_int.in_dll(L, nm).value = v
    org, sp = d["origin_spacing"][:3], d["origin_spacing"][3:]
    for nm, v in zip(("origin_x", "origin_y", "origin_z", "spacing_x", "spacing_y", "spacing_z"), list(org) + list(sp)):
        C.c_double.in_dll(L, nm).value = float(v)
    noc = (C.c_int * lM)()
    for c in d["centres"]:
        noc[int(c[0])] += 1
    C.c_void_p.in_dll(L, "no_of_centers").value = C.addressof(noc)
    for fn in ("_allocateMem_", "_deallocateMem_", "_writeData_", "_load3dDataArrayVTK_"):
        getattr(L, fn).restype = C.c_bool
    L._readData_.restype = None
    assert L._allocateMem_()
    try:
        n = int(np.prod(shape))
        i0 = np.ctypeslib.as_array((C.c_double * n).from_address(C.c_void_p.in_dll(L, "i0").value)).reshape(shape)
        i0[...] = -1.0
        L._readData_(C.c_void_p(i0.ctypes.data), C.c_char_p(str(tmp_path).encode()))
        assert np.array_equal(i0, d["i0_read"])
        pp = C.POINTER(C.POINTER(C.c_double))
        cx, cy, cz = (pp.in_dll(L, nm) for nm in ("center_x", "center_y", "center_z"))
        seen = [0] * lM
        for c in d["centres"]:
            l = int(c[0])
            assert (cx[l][seen[l]], cy[l][seen[l]], cz[l][seen[l]]) == tuple(c[1:])
            seen[l] += 1
        # one frame again through _load3dDataArrayVTK_: the other frames stay
        i0[2, 1:-1, 1:-1, 1:-1] = 7.0
        assert L._load3dDataArrayVTK_(C.c_void_p(i0.ctypes.data), 2,
                                      C.c_char_p(str(tmp_path / "movingBalls_457_at_time_002.vtk").encode()))
        assert np.array_equal(i0, d["i0_read"])
        u = np.ctypeslib.as_array((C.c_double * n).from_address(C.c_void_p.in_dll(L, "u").value)).reshape(shape)
        u[...] = d["u_written"]
        assert L._writeData_(C.c_void_p(u.ctypes.data), C.c_char_p(str(tmp_path / "out").encode()))
        for l in range(1, nt + 1):
            with open(tmp_path / ("out_at_time_%03d.vtk" % l), "rb") as fh:
                assert np.array_equal(np.frombuffer(fh.read(), dtype=np.uint8), d["written"][l - 1]), f"frame {l}"
    finally:
        L._deallocateMem_()
