"""Known-answer vectors of Philox4x32-10 (Salmon, Moraes, Dror and Shaw,
"Parallel Random Numbers: As Easy as 1, 2, 3", SC'11; the published
known-answer vectors of its Random123 distribution) against the project's
Philox in oracle/philox.h, the generator that replaces the reference's
glibc rand() sampler (src/sampler/samplerstd.cpp:7-10).

The GPU kernels (nuray_gb300/csrc/nr_device.cuh, philox10) draw the same
stream: the per-sample parity tests compare GPU and oracle radiance on
identical (pixel, sample) streams, so this pin carries over to them.
"""
import os
import subprocess

import pytest

from conftest import ROOT

KAT = [  # (counter, key) -> output, all 32-bit words
    ((0x00000000, 0x00000000, 0x00000000, 0x00000000), (0x00000000, 0x00000000),
     (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF), (0xFFFFFFFF, 0xFFFFFFFF),
     (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]

PROBE = r"""
#include <stdio.h>
#include <stdlib.h>
#include "philox.h"
int main(int argc, char** argv) {
    uint32_t c[4], k[2], o[4];
    for (int i = 0; i < 4; ++i) c[i] = (uint32_t)strtoul(argv[1 + i], 0, 16);
    for (int i = 0; i < 2; ++i) k[i] = (uint32_t)strtoul(argv[5 + i], 0, 16);
    nr_philox4x32_10(c, k, o);
    printf("%08x %08x %08x %08x\n", o[0], o[1], o[2], o[3]);
    return 0;
}
"""


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    d = tmp_path_factory.mktemp("philox")
    src, exe = d / "kat.c", d / "kat"
    src.write_text(PROBE)
    subprocess.run(["gcc", "-O2", "-I", os.path.join(ROOT, "oracle"), str(src), "-o", str(exe)], check=True)
    return str(exe)


@pytest.mark.parametrize("ctr,key,want", KAT)
def test_philox4x32_10_known_answers(probe, ctr, key, want):
    out = subprocess.run([probe] + [f"{x:08x}" for x in ctr + key], capture_output=True, text=True, check=True)
    got = tuple(int(w, 16) for w in out.stdout.split())
    assert got == want, [f"{x:08x}" for x in got]


def test_uniforms_from_the_stream(probe):
    """The stream's uniform is the top 24 bits of a word times 2^-24: every
    value lies in [0, 1) and 1 - 2^-24 is reachable."""
    import numpy as np
    x = np.array([0x00000000, 0x000000FF, 0x00000100, 0xFFFFFFFF], np.uint64)
    u = (x >> 8).astype(np.float32) * np.float32(1.0 / 16777216.0)
    assert u[0] == 0 and u[1] == 0 and u[2] == np.float32(2.0 ** -24) and u[3] == np.float32(1 - 2.0 ** -24)
