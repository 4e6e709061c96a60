"""The checkpoint checksum of alps-looper_gb300/csrc/lg_host.cpp (what lg_save stores and lg_load
checks) against the Python restatement in looper_gb300.checkpoint_checksum, without a GPU: both
over the same bytes, one, two and three 1 MiB blocks and ragged tails."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

import looper_gb300 as lg

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#include <cstdarg>
#include <cstdio>
#include <vector>
#include "lg_host.h"
int lg_fail(int code, const char*, ...) { return code; }
int main(int argc, char** argv) {
  std::FILE* f = std::fopen(argv[1], "rb");
  std::vector<uint8_t> b;
  int c;
  while ((c = std::fgetc(f)) != EOF) b.push_back((uint8_t)c);
  std::fclose(f);
  std::printf("%llu\n", (unsigned long long)checkpoint_checksum(b.data(), b.size()));
  return 0;
}
"""


@pytest.fixture(scope="module")
def exe():
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    d = tempfile.mkdtemp()
    src = os.path.join(d, "sum.cpp")
    with open(src, "w") as fh:
        fh.write(SRC)
    out = os.path.join(d, "sum")
    cmd = [cxx, "-std=c++17", "-O2", "-I" + os.path.join(REPO, "include"),
           "-I" + os.path.join(REPO, "alps-looper_gb300", "csrc"),
           os.path.join(REPO, "alps-looper_gb300", "csrc", "lg_host.cpp"), src, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    yield out, d
    shutil.rmtree(d, ignore_errors=True)


@pytest.mark.parametrize("size", [8, 9, 40, 1 << 20, (1 << 20) + 8, (1 << 20) + 13,
                                  (5 << 19) + 3, 3 << 20])
def test_checksum_matches_the_library(exe, size):
    out, d = exe
    data = np.random.default_rng(size).integers(0, 256, size=size, dtype=np.uint8).tobytes()
    path = os.path.join(d, "blob")
    with open(path, "wb") as fh:
        fh.write(data)
    r = subprocess.run([out, path], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert int(r.stdout) == lg.checkpoint_checksum(data)
