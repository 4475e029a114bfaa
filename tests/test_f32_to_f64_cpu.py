"""The integer-pipe FP32 -> FP64 widening used by the FP32 quartet kernels
before their FP64 atomics (csrc/f32_to_f64.h), checked on the CPU over every
one of the 2^32 float bit patterns against the compiler's conversion: equal
bits for every normal value, zero and infinity, a NaN for every NaN, and a
signed zero for the FP32 subnormals."""
import os
import subprocess
import sys

import pytest

HDR = os.path.join(os.path.dirname(__file__), '..', 'gpu4pyscf_gb300', 'csrc')

SRC = r'''
#include <cmath>
#include <cstdio>
#include <cstring>
#include "f32_to_f64.h"
int main() {
    unsigned long long bad = 0, sub = 0;
    uint32_t u = 0;
    do {
        float f; memcpy(&f, &u, 4);
        double got = f32_to_f64_exact(f), want = (double)f;
        uint64_t gb, wb; memcpy(&gb, &got, 8); memcpy(&wb, &want, 8);
        const uint32_t e = (u >> 23) & 0xffu;
        if (e == 0u && (u & 0x7fffffu)) {
            ++sub;
            if (got != 0.0 || std::signbit(got) != std::signbit(want)) ++bad;
        } else if (std::isnan(want)) {
            if (!std::isnan(got)) ++bad;
        } else if (gb != wb) {
            ++bad;
        }
    } while (++u != 0u);
    printf("%llu %llu\n", bad, sub);
    return bad != 0;
}
'''


@pytest.mark.timeout(300)
def test_every_float(tmp_path):
    src = tmp_path / 'f2d.cpp'
    exe = tmp_path / 'f2d'
    src.write_text(SRC)
    subprocess.check_call(['g++', '-O2', '-std=c++17', '-I', HDR, str(src), '-o', str(exe)])
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=280)
    bad, sub = map(int, out.stdout.split())
    assert bad == 0
    assert sub == 2 * (2 ** 23 - 1)
