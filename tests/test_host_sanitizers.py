"""The host side of the C ABI under gcc's sanitizers (CPU only).

tests/host_fuzz.cpp is compiled together with alps-looper_gb300/csrc/lg_host.cpp with the
address, undefined-behaviour and float-cast-overflow sanitizers, every report fatal, and fuzzes
the parameter parser, the model setup, the record accumulators and the checkpoint decoder (see
the harness for the cases).  Skipped where the compiler cannot build sanitized programs.
"""
import os
import shutil
import subprocess
import tempfile

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SAN = ["-fsanitize=address,undefined,float-cast-overflow", "-fno-sanitize-recover=all"]


def test_host_code_is_clean_under_sanitizers():
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "host_fuzz")
        cmd = [cxx, "-std=c++17", "-O1", "-g"] + SAN + [
            "-I" + os.path.join(REPO, "include"),
            "-I" + os.path.join(REPO, "alps-looper_gb300", "csrc"),
            os.path.join(REPO, "alps-looper_gb300", "csrc", "lg_host.cpp"),
            os.path.join(REPO, "tests", "host_fuzz.cpp"), "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
        if r.returncode != 0:
            if "sanitize" in r.stderr or "asan" in r.stderr.lower():
                pytest.skip("sanitizer runtime unavailable: " + r.stderr[-300:])
            raise AssertionError(r.stderr[-3000:])
        env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1", UBSAN_OPTIONS="print_stacktrace=1")
        r = subprocess.run([exe], capture_output=True, text=True, timeout=600, env=env)
        assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-3000:])
        assert r.stdout.startswith("ok:"), r.stdout
