"""The C ABI boundary without a GPU: the libraries load, export every symbol
the headers declare, validate arguments on the host, and fail loudly (never
fall back to a CPU path) when no device is visible."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, PKG


def _declared(header: str) -> list[str]:
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b((?:ss4d|_)[A-Za-z0-9_]*)\s*\(", text)) - {"__attribute__"})


def _exports(so: str) -> set[str]:
    import subprocess
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True, check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if ln.strip()}


def test_native_library_exports_header(ss4d):
    syms = _exports(ss4d.LIB_PATH)
    names = [n for n in _declared("ss4d.h") if n.startswith("ss4d_")]
    assert len(names) >= 30
    missing = [n for n in names if n not in syms]
    assert not missing, missing
    assert ss4d.lib().ss4d_abi_version() == ss4d.ABI_VERSION == 3


def test_reference_named_libraries_export_reference_interface(ss4d):
    seg = _exports(ss4d.SEG_PATH)
    mcf = _exports(ss4d.MCF_PATH)
    decl = _declared("ss4d_compat.h")
    seg_names = [n for n in decl if n.startswith("_") and not n.endswith("mcf") and n != "_mcfTimeStep"]
    mcf_names = [n for n in decl if n.endswith("_mcf") or n == "_mcfTimeStep"]
    for n in seg_names + ["ijkl", "ss4d_compat_sync_host", "ss4d_compat_last_stats"]:
        assert n in seg, n
    for n in mcf_names + ["ijkl", "ss4d_compat_sync_host", "ss4d_compat_last_stats"]:
        assert n in mcf, n
    # the reference's globals, same names (segmentation4D.c:14-58, mcf_4D.c:12-34)
    for g in ("iMax", "jMax", "kMax", "lMax", "u", "prev_u", "i0", "Mmask", "e", "w", "n", "s", "t", "b", "fw", "bw",
              "g_e", "g_w", "g_n", "g_s", "g_t", "g_b", "g_fw", "g_bw", "K", "eps2", "tau", "h", "omega_c", "gsTol",
              "maxNoGSIteration", "sigma", "omega_sigma", "maxNoGSIteration_sigma", "theta_img", "rho_thr",
              "no_of_centers", "center_x", "center_y", "center_z", "ballRadius", "numberOfTimeStep"):
        assert g in seg, g
    for g in ("iMax", "u", "prev_u", "exact_u", "e", "bw", "tau", "h", "eps2", "omega_c", "gsTol", "mcfTol",
              "maxNoGSIteration", "numberOfTimeStep"):
        assert g in mcf, g


def test_compat_scalar_helpers_match_reference_formulas(ss4d):
    L = C.CDLL(ss4d.SEG_PATH)
    for nm, v in (("iMax", 7), ("jMax", 6), ("kMax", 5), ("lMax", 4)):
        C.c_int.in_dll(L, nm).value = v
    L.ijkl.restype = C.c_int
    assert L.ijkl(3, 2, 1, 2) == ((2 * 5 + 1) * 6 + 2) * 7 + 3  # segmentation4D.c:61-65
    L._gFunction_.restype = C.c_double
    L._gFunction_.argtypes = [C.c_double, C.c_double]
    assert L._gFunction_(0.25, 1000.0) == 1.0 / (1 + 1000.0 * 0.25)  # segmentation4D.c:67-70


def test_host_side_validation_needs_no_device(ss4d):
    L = ss4d.lib()
    out = C.c_void_p()
    bad = ss4d.Dims(2, 5, 5, 5)  # an extent below 3
    assert L.ss4d_solver_create(C.byref(bad), 1, None, C.byref(out)) == 1
    assert b"extent" in L.ss4d_last_error()
    huge = ss4d.Dims(2000, 2000, 1000, 10)  # more than 2^31 voxels
    assert L.ss4d_solver_create(C.byref(huge), 1, None, C.byref(out)) == 1
    ok = ss4d.Dims(6, 6, 6, 6)
    assert L.ss4d_solver_create(C.byref(ok), 9, None, C.byref(out)) == 1  # unknown arithmetic
    assert L.ss4d_solver_create(C.byref(ok), 1, None, None) == 1


def test_no_device_fails_loudly(ss4d):
    if ss4d.device_count() > 0:
        pytest.skip("a CUDA device is visible")
    with pytest.raises(ss4d.SS4DError) as ei:
        ss4d.Solver(6, 6, 6, 6)
    assert ei.value.status == 7  # SS4D_ERR_NO_DEVICE: no CPU fallback


def test_scene_generator_is_seeded_and_thread_independent(ss4d):
    a_i0, a_u0 = ss4d.scene(1, 16, 12, 10, 4, seed=3, threads=1)
    b_i0, b_u0 = ss4d.scene(1, 16, 12, 10, 4, seed=3, threads=4)
    c_i0, _ = ss4d.scene(1, 16, 12, 10, 4, seed=4, threads=1)
    assert np.array_equal(a_i0, b_i0) and np.array_equal(a_u0, b_u0)
    assert not np.array_equal(a_i0, c_i0)
    # intensities are bytes/255 like the reference loader; ghosts are zero
    q = a_i0 * 255
    assert np.allclose(q, np.round(q))
    assert a_i0[0].max() == 0 and a_i0[:, :, :, 0].max() == 0
    # u0 = 1/(|x-s|+1) on every voxel, ghosts included
    assert a_u0.min() > 0 and a_u0.max() <= 1.0
    for kind in (2, 3):
        i0, u0 = ss4d.scene(kind, 20, 18, 16, 5, seed=5)
        assert np.isfinite(i0).all() and np.isfinite(u0).all()
        assert i0[1:-1, 1:-1, 1:-1, 1:-1].max() > 0.5  # objects brighter than the background


def test_noalloc_wrapper_rejects_arrays_it_cannot_check(ss4d):
    """The allocation-free rescale takes no handle, so nothing on the C side
    knows the array behind the pointer: the Python wrapper refuses host
    arrays, other dtypes, non-contiguous views and shapes that differ from
    dims before the call is made."""
    torch = pytest.importorskip("torch")
    p = ss4d.scene_params()
    dims = (6, 5, 4, 3)
    with pytest.raises(ValueError, match="CUDA"):
        ss4d.rescale_to_zero_one_noalloc(dims, p, np.zeros((3, 4, 5, 6)))
    with pytest.raises(ValueError, match="CUDA"):
        ss4d.rescale_to_zero_one_noalloc(dims, p, torch.zeros((3, 4, 5, 6), dtype=torch.float64))

    class FakeCuda:
        """stands in for a device tensor: only the attributes the checks read"""

        def __init__(self, shape, dtype="torch.float64", contiguous=True):
            self.shape, self.dtype, self._c, self.is_cuda = shape, dtype, contiguous, True

        def is_contiguous(self):
            return self._c

    with pytest.raises(ValueError, match="float64"):
        ss4d.rescale_to_zero_one_noalloc(dims, p, FakeCuda((3, 4, 5, 6), dtype="torch.float32"))
    with pytest.raises(ValueError, match="contiguous"):
        ss4d.rescale_to_zero_one_noalloc(dims, p, FakeCuda((3, 4, 5, 6), contiguous=False))
    with pytest.raises(ValueError, match="shape"):
        ss4d.rescale_to_zero_one_noalloc(dims, p, FakeCuda((3, 4, 6, 5)))
    with pytest.raises(ValueError, match="mmask"):
        ss4d.rescale_to_zero_one_noalloc(dims, p, FakeCuda((3, 4, 5, 6)), np.ones((3, 4, 5, 6)))
