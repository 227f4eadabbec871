"""The smoothers divide by 3 with two FMAs instead of a division (see
div3 in flowlab_gb300/csrc/fl_multigrid.cu): q0 = RN(s * RN(1/3)),
r = s - 3 q0, q = RN(q0 + r * RN(1/3)), zero and infinities taking q0. This
checks the formula against IEEE float division on the host, on every 97th
bit pattern of the 2^32 floats plus the special values (CPU; the full
space was checked exhaustively when the formula was adopted)."""
import os
import shutil
import subprocess
import tempfile

import pytest

SRC = r"""
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
static int check(uint32_t b) {
  float a; memcpy(&a, &b, 4);
  const float y = 1.0f / 3.0f;
  float ref = a / 3.0f;
  float q0 = a * y;
  float r = fmaf(-3.0f, q0, a);
  float q1 = fmaf(r, y, q0);
  float q = (a == 0.0f || isinf(a)) ? q0 : q1;
  uint32_t rb, qb; memcpy(&rb, &ref, 4); memcpy(&qb, &q, 4);
  if (isnan(ref) && isnan(q)) return 0;
  return rb != qb;
}
int main(void) {
  unsigned long long bad = 0, n = 0;
  const uint32_t special[] = {0u, 0x80000000u, 1u, 0x80000001u, 0x007fffffu, 0x00800000u, 0x7f7fffffu,
                              0xff7fffffu, 0x7f800000u, 0xff800000u, 0x7fc00000u, 0x3f800000u, 0x40400000u};
  for (unsigned k = 0; k < sizeof special / sizeof special[0]; k++) { bad += check(special[k]); n++; }
  for (uint64_t u = 0; u < 0x100000000ull; u += 97) { bad += check((uint32_t)u); n++; }
  printf("%llu %llu\n", n, bad);
  return 0;
}
"""


def test_fma_division_by_three_is_correctly_rounded():
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "div3.c")
        exe = os.path.join(d, "div3")
        with open(src, "w") as fh:
            fh.write(SRC)
        subprocess.run([cc, "-O2", "-ffp-contract=off", src, "-o", exe, "-lm"], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    n, bad = int(out[0]), int(out[1])
    assert n > 4e7 and bad == 0
