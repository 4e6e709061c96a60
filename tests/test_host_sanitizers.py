"""Host code under gcc's sanitizers (CPU only): address, undefined behaviour and float-cast
overflow, every report fatal.  Skipped where the compiler cannot build sanitized programs.

* the host side of the C ABI: tests/host_fuzz.cpp with alps-looper_gb300/csrc/lg_host.cpp fuzzes
  the parameter parser, the model setup, the record accumulators and the checkpoint decoder;
* the CPU oracle the parity tests rest on: tests/oracle_sanitized.cpp with
  oracle/looper_oracle.cpp runs every model family and the standalone mode.
"""
import os
import shutil
import subprocess
import tempfile

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SAN = ["-fsanitize=address,undefined,float-cast-overflow", "-fno-sanitize-recover=all"]


def _build_and_run(sources, includes=()):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "sanitized")
        cmd = [cxx, "-std=c++17", "-O1", "-g"] + SAN + ["-I" + i for i in includes] + \
            list(sources) + ["-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
        if r.returncode != 0:
            if "sanitize" in r.stderr or "asan" in r.stderr.lower():
                pytest.skip("sanitizer runtime unavailable: " + r.stderr[-300:])
            raise AssertionError(r.stderr[-3000:])
        env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1", UBSAN_OPTIONS="print_stacktrace=1")
        r = subprocess.run([exe], capture_output=True, text=True, timeout=600, env=env)
        assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-3000:])
        return r.stdout


def test_host_code_is_clean_under_sanitizers():
    out = _build_and_run(
        [os.path.join(REPO, "alps-looper_gb300", "csrc", "lg_host.cpp"),
         os.path.join(REPO, "tests", "host_fuzz.cpp")],
        [os.path.join(REPO, "include"), os.path.join(REPO, "alps-looper_gb300", "csrc")])
    assert out.startswith("ok:"), out


def test_oracle_is_clean_under_sanitizers():
    out = _build_and_run([os.path.join(REPO, "oracle", "looper_oracle.cpp"),
                          os.path.join(REPO, "tests", "oracle_sanitized.cpp")])
    assert out.strip() == "ok", out
