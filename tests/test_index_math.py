"""The kernels' index arithmetic on the CPU: FastDiv (division by a fixed
divisor for numerators below 2^31) and the float-float assembly's
plane-frame block order (PlaneOrder, plane_frame) from
csrc/ss4d_common.cuh, compiled by nvcc as host code and checked against
plain integer division.  Needs nvcc, no GPU."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "4d-image-segmentation-algorithm_gb300", "csrc")

PROGRAM = r"""
#include "ss4d_common.cuh"
#include <cstdio>

using namespace ss4d;

static unsigned state = 12345u;
static unsigned next_u31() { state = state * 1664525u + 1013904223u; return state & 0x7FFFFFFFu; }

// the division form of the block order (what PlaneOrder replaces)
static void plane_frame_div(int z, int P, int F, int kb, int &pk, int &fl)
{
    if (kb <= 0 || kb >= P) { pk = z % P; fl = z / P; return; }
    const int full = P / kb, blk = kb * F, b = z / blk;
    if (b < full) { const int r = z - b * blk; fl = r / kb; pk = b * kb + r % kb; }
    else { const int rest = P - full * kb, r = z - full * blk; fl = r / rest; pk = full * kb + r % rest; }
}

int main()
{
    long long checks = 0;
    const unsigned top = 0x7FFFFFFFu;
    for (unsigned d = 1; d <= (1u << 17); ++d) {
        const FastDiv f = make_fastdiv(d);
        const unsigned edge[] = {0u, 1u, d - 1, d, d + 1, 2 * d - 1, 2 * d, top, top - 1, (top / d) * d,
                                 (top / d) * d - 1};
        for (unsigned n : edge) {
            if (n > top) continue;
            if (fdiv(n, f) != n / d) { std::printf("fdiv %u / %u\n", n, d); return 1; }
            ++checks;
        }
        for (int r = 0; r < 48; ++r) {
            const unsigned n = next_u31();
            if (fdiv(n, f) != n / d) { std::printf("fdiv %u / %u\n", n, d); return 1; }
            ++checks;
        }
    }
    const unsigned ds[] = {3u, 7u, 22u, 130u, 258u, 65535u, 1000003u};
    for (unsigned d : ds) {
        const FastDiv f = make_fastdiv(d);
        for (unsigned n = 0; n < (1u << 24); ++n) {
            if (fdiv(n, f) != n / d) { std::printf("fdiv %u / %u\n", n, d); return 1; }
            ++checks;
        }
    }
    const int Ps[] = {1, 2, 3, 4, 5, 6, 7, 8, 9, 15, 16, 17, 31, 33, 64, 65, 128, 129, 257};
    const int Fs[] = {1, 2, 3, 5, 8, 13, 20, 22, 50};
    const int kbs[] = {0, 1, 2, 3, 4, 5, 7, 8, 16, 32, 64, 1000};
    for (int P : Ps)
        for (int F : Fs)
            for (int kb : kbs) {
                const PlaneOrder o = make_plane_order(P, F, kb);
                for (int z = 0; z < P * F; ++z) {
                    int pk, fl, pk0, fl0;
                    plane_frame((unsigned)z, o, pk, fl);
                    plane_frame_div(z, P, F, kb, pk0, fl0);
                    if (pk != pk0 || fl != fl0) { std::printf("plane_frame %d %d %d %d\n", P, F, kb, z); return 1; }
                    ++checks;
                }
            }
    std::printf("ok %lld\n", checks);
    return 0;
}
"""


def test_fastdiv_and_plane_order_match_integer_division(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not found")
    src = tmp_path / "index_math.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "index_math"
    subprocess.run([nvcc, "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", f"-I{CSRC}",
                    str(src), "-o", str(exe)], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok"), out.stdout
