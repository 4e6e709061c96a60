"""loop_gpu: looper's standalone loop program (standalone/loop.C with standalone/options.h) on the
GB300 engine, a C++ program over the C ABI.

* CPU: the standalone program's option handling: -h prints the option list on stdout, an odd
  length prints "invalid parameter" and the list on stderr, an unknown option the list; each
  exits with status 255 (options.h:42-88, loop.C:42).
* GPU: the standalone program's golden run (standalone/loop.op: L = 8, T = 0.2, 65536 + 8192
  sweeps): the parameter lines digit for digit, and every result within 4 combined standard
  errors of the golden one (the engine's random streams are its own).
"""
import json
import math
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def exe():
    import build as b
    b.build()
    assert os.path.exists(b.EXE)
    return b.EXE


def _run(exe, *args, timeout=600):
    return subprocess.run([exe, *args], capture_output=True, text=True, timeout=timeout)


def test_options_like_the_standalone_program(exe):
    r = _run(exe, "-h")
    assert r.returncode == 255 and "-l int     System Length" in r.stdout
    r = _run(exe, "-l", "7")
    assert r.returncode == 255 and r.stderr.startswith("invalid parameter")
    assert "-n int     MCS for Measurement" in r.stderr and r.stdout == ""
    r = _run(exe, "-t", "0")
    assert r.returncode == 255 and r.stderr.startswith("invalid parameter")
    r = _run(exe, "-x")
    assert r.returncode == 255 and "[command line options]" in r.stderr


def _value(line):
    name, rest = line.split("=", 1)
    mean, err = rest.split("+-")
    return name.strip(), float(mean), float(err)


@pytest.mark.gpu
def test_golden_run_of_the_standalone_program(exe):
    with open(os.path.join(HERE, "golden", "standalone_loop_op.json")) as f:
        g = json.load(f)
    r = _run(exe, "-l", str(g["L"]), "-t", str(g["T"]), "-n", str(g["sweeps"]))
    assert r.returncode == 0, r.stderr
    assert "Speed = " in r.stderr
    out = r.stdout.strip().splitlines()
    assert out[:4] == g["lines"][:4]
    assert len(out) == len(g["lines"]) == 9
    for got, ref in zip(out[4:], g["lines"][4:]):
        name, m, e = _value(got)
        rname, rm, re_ = _value(ref)
        assert name == rname
        assert e > 0
        assert abs(m - rm) <= 4.0 * math.hypot(e, re_), (name, m, e, rm, re_)
