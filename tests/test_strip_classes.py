"""The host/device helpers that decide which sweep kernel walks a strip and how wide a DST tile
is, compiled from the library's headers as a host program and checked over every basin up to
300 x 300 (no GPU needed).

A strip filed as interior (class 0) is walked without any bounds predicate, so every row and
column it reads (x0 - 2 .. x0 + 61, jb - 2 .. band end + 1) must lie strictly inside the member;
an edge-in-x strip (class 3) must have its rows inside and an edge-in-y strip (class 4) its
columns.  Row bands must tile the rows, start on multiples of 16 (the walk's unrolled ring slots)
and hold at most 64 rows (the wind profile a strip keeps in two registers per lane).  A DST output
tile must be a multiple of 16 wide, no wider than the plan's tile, and the member's last tile
must cover the columns left."""

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

HARNESS = r"""
#include <cstdio>
#include "qg_tc.cuh"
using namespace qg;
int main() {
    long bad = 0, n = 0;
    const int Rs[3] = {16, 32, 64};
    for (int Ny = 3; Ny <= 300; ++Ny)
        for (int Nx = 3; Nx <= 300; ++Nx)
            for (int R : Rs) {
                const int nb = lsweep_bands(Ny, R);
                int prev = 0;
                for (int sy = 0; sy < nb; ++sy) {
                    const int jb = sy * R, je = lsweep_band_end(Ny, sy, R);
                    if (jb != prev || je <= jb || je - jb > 64 || jb % 16) ++bad;
                    prev = je;
                    for (int sx = 0; sx * kLSweepOut < Nx; ++sx) {
                        const int c = lsweep_item_class(Ny, Nx, false, sx, sy, R);
                        const int x0 = sx * kLSweepOut;
                        const bool xin = x0 - 2 >= 1 && x0 + 61 <= Nx - 2;
                        const bool yin = jb - 2 >= 1 && je + 1 <= Ny - 2;
                        if ((c == 0 && !(xin && yin)) || (c == 3 && !yin) || (c == 4 && !xin) || c < 0 || c > 4 ||
                            c == 2)
                            ++bad;
                        if (lsweep_item_class(Ny, Nx, true, sx, sy, R) != 2) ++bad;
                        ++n;
                    }
                }
                if (prev != Ny) ++bad;
            }
    const int bns[5] = {144, 80, 48, 32, 16};
    for (int Nn = 1; Nn <= 1100; ++Nn)
        for (int bn : bns) {
            const int nt = (Nn + bn - 1) / bn;
            for (int t = 0; t < nt; ++t) {
                const int w = tc_tile_width(Nn, t, bn);
                const int left = Nn - t * bn;
                if (w % 16 || w > bn || w > TC_BN || w > TC_TMEM_BUF || w < (left < bn ? left : bn)) ++bad;
                if (left >= bn && w != bn) ++bad;
                ++n;
            }
        }
    printf("%ld %ld\n", n, bad);
    return bad != 0;
}
"""


def test_strip_classes_and_tile_widths(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if Path("/usr/local/cuda/bin/nvcc").exists() else None)
    if nvcc is None:
        pytest.skip("nvcc not found")
    src = tmp_path / "strips.cu"
    src.write_text(HARNESS)
    exe = tmp_path / "strips"
    r = subprocess.run([nvcc, "-std=c++17", "-I", str(ROOT / "somax_gb300" / "csrc"), "-I", str(ROOT / "include"),
                        "-o", str(exe), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    checked, bad = (int(x) for x in out.stdout.split())
    assert checked > 4_000_000 and bad == 0 and out.returncode == 0
