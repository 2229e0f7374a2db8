"""The X320 exact accumulator's conversion to double is the correctly rounded value
(ties to even) of the 320-bit integer times 2^-149, and the 32-bit digit split used
for grid-wide atomics round-trips.  Compiles tests/native/x320_check.cu for the host
with nvcc; no GPU needed."""

import random
import shutil
import subprocess
from fractions import Fraction

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = tmp_path_factory.mktemp("x320") / "x320_check"
    subprocess.run([nvcc, "-O2", "-std=c++17", "-o", str(out), str(ROOT / "tests" / "native" / "x320_check.cu")],
                   check=True, capture_output=True)
    return out


def cases():
    rnd = random.Random(1)
    vals = [0, 1, -1, 1 << 309, -(1 << 309)]
    for i in range(4000):
        kind = i % 5
        if kind == 0:
            v = rnd.getrandbits(rnd.randint(1, 318))
        elif kind == 1:
            v = -rnd.getrandbits(rnd.randint(1, 318))
        elif kind == 2:
            v = rnd.getrandbits(53) << rnd.randint(0, 250)
        elif kind == 3:  # sticky bit far below the guard bit
            v = (rnd.getrandbits(53) << rnd.randint(60, 250)) + (1 << rnd.randint(0, 59))
        else:  # exact halfway cases
            b = rnd.randint(54, 300)
            v = ((rnd.getrandbits(52) | (1 << 52)) << (b - 52)) + (1 << (b - 53))
        vals.append(v)
    return vals


def test_x320_to_double_correctly_rounded(checker):
    vals = cases()
    lines = []
    for v in vals:
        u = v % (1 << 320)
        lines.append(" ".join("%x" % ((u >> (64 * k)) & ((1 << 64) - 1)) for k in range(5)))
    out = subprocess.run([str(checker)], input="\n".join(lines) + "\n", capture_output=True, text=True,
                         check=True).stdout
    assert "MISMATCH" not in out
    got = [float.fromhex(x) for x in out.split()]
    assert len(got) == len(vals)
    for v, g in zip(vals, got):
        assert g == float(Fraction(v, 1 << 149)), v
