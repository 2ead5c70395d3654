"""Host-side pieces of the generated modules' shared header, run on the CPU: a
small program compiled by nvcc against ``xgrid_gen.cuh`` (no device code runs).

* The mixed-precision work area: the byte size that ``mixed.aux_bytes`` allocates
  is what ``xg_mx_layout`` needs, and the error word sits where
  ``mixed.aux_error_offset`` says, for square, odd and 3-D shapes.
* Launch-invariant divisors and scales: ``xg_make_scale`` marks exactly the
  powers of two (with their exponent), ``xg_make_divisor`` keeps RN(1/d) and the
  correction term and enables the fast path for normal divisors."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from xgrid_gb300 import build, mixed

HARNESS = r"""
#include "xgrid_gen.cuh"
#include <cstdio>
int main(int argc, char** argv) {
  const long long shapes[][3] = {{1, 257, 257}, {1, 4097, 4097}, {1, 203, 333}, {5, 7, 45}, {1, 1, 1}};
  for (const auto& s : shapes) {
    xg_grid g;
    memset(&g, 0, sizeof g);
    g.ndim = s[0] == 1 ? 2 : 3;
    if (g.ndim == 2) { g.shape[0] = s[1]; g.shape[1] = s[2]; }
    else { g.shape[0] = s[0]; g.shape[1] = s[1]; g.shape[2] = s[2]; }
    static unsigned char dummy[16];
    g.aux = dummy;
    xg_mx_aux a;
    // the smallest size xg_mx_layout accepts
    long long lo = 0, hi = 1LL << 40;
    while (lo < hi) {
      const long long mid = (lo + hi) / 2;
      g.aux_bytes = mid;
      if (xg_mx_layout(&g, &a) == 0) hi = mid; else lo = mid + 1;
    }
    g.aux_bytes = lo;
    xg_mx_layout(&g, &a);
    printf("layout %lld %lld %lld %lld %lld %lld\n", s[0], s[1], s[2], lo,
           (long long)((unsigned char*)a.err - (unsigned char*)g.aux), (long long)a.XP);
  }
  const double ds[] = {0.5, 2.0, 0.25, 1024.0, 3.0, 0.1, 2.0 / 1024, 1e-5, -4.0, 6.103515625e-05, 1e300, 5e-324};
  for (double d : ds) {
    const xg_scale k = xg_make_scale(d);
    const xg_divisor v = xg_make_divisor(d);
    printf("scale %.17g %d %d %u\n", d, k.p2, k.s, k.sg);
    printf("divisor %.17g %d %.17g %.17g %d\n", d, v.ok, v.zh, v.zl, v.rz.p2);
  }
  return 0;
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    d = tmp_path_factory.mktemp("layout")
    src = d / "h.cu"
    src.write_text(HARNESS)
    exe = d / "h"
    subprocess.run([nvcc, *build.ARCH, "-std=c++17", "-w", "-I", build.INCLUDE, "-I", build.CSRC, str(src),
                    "-L", build.LIBDIR, "-lxgrid_gb300", "-Xlinker", f"-rpath,{build.LIBDIR}", "-o", str(exe)],
                   check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return [l.split() for l in out.splitlines()]


def test_work_area_size_and_error_word_match(harness):
    rows = [r for r in harness if r[0] == "layout"]
    assert len(rows) == 5
    for _, z, y, x, need, err, xp in rows:
        z, y, x = int(z), int(y), int(x)
        shape = (y, x) if z == 1 else (z, y, x)
        assert mixed.aux_bytes(shape) == int(need), shape
        assert mixed.aux_error_offset(shape) == int(err), shape
        assert int(xp) % mixed.AUX_PITCH == 0 and int(xp) >= x


def test_scales_and_divisors(harness):
    for r in harness:
        if r[0] == "scale":
            d, p2, s, sg = float(r[1]), int(r[2]), int(r[3]), int(r[4])
            m, e = np.frexp(abs(d))
            is_p2 = np.isfinite(d) and d != 0 and abs(m) == 0.5 and abs(d) >= np.finfo(float).tiny
            assert p2 == int(is_p2), d
            if p2:
                assert 2.0 ** s == abs(d) and (sg != 0) == (d < 0)
        elif r[0] == "divisor":
            d, ok, zh, zl, rz = float(r[1]), int(r[2]), float(r[3]), float(r[4]), int(r[5])
            normal = np.isfinite(d) and abs(d) >= np.finfo(float).tiny and np.isfinite(1.0 / d) \
                and abs(1.0 / d) >= np.finfo(float).tiny
            if normal:
                assert zh == 1.0 / d and ok == 1, d
                # zl: the rounding error of zh, divided by d (|zl| far below |zh|)
                assert abs(zl) <= abs(zh) * 2.0 ** -52
                m, _ = np.frexp(abs(1.0 / d))
                assert rz == int(abs(m) == 0.5), d
            else:
                assert ok == 0, d
