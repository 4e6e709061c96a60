"""The parapack worker plug-in of INTEGRATION.md, compiled from the document itself.

Its source (the C++ block of section 1) is extracted, compiled against include/looper_gpu.h with
stand-in ALPS and Boost headers (tests/plugin_stub) and driven by tests/plugin_main.cpp the way
parapack drives a worker: init_observables, then run() until progress() reaches 1.
* CPU: the plug-in compiles and links against the library.
* GPU: the means of the values it pushes equal the library's own observables for the same
  parameters, and a save / load in the middle of the run resumes with exactly the same values.
"""
import os
import re
import shutil
import subprocess
import tempfile

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(REPO, "alps-looper_gb300", "lib")

PARAMS = {"LATTICE": "square lattice", "L": "8", "T": "0.5", "J": "1", "SWEEPS": "600",
          "THERMALIZATION": "100", "SEED": "77", "WORKER_SEED": "77"}


def _plugin_source():
    with open(os.path.join(REPO, "INTEGRATION.md")) as f:
        text = f.read()
    m = re.search(r"```cpp\n(// gpu_path_integral\.C.*?)```", text, re.S)
    assert m, "the plug-in block of INTEGRATION.md"
    return m.group(1)


def _build(link):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    d = tempfile.mkdtemp()
    with open(os.path.join(d, "gpu_path_integral.C"), "w") as f:
        f.write(_plugin_source())
    out = os.path.join(d, "plugin_main")
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", "-Wno-unused-local-typedefs",
           '-DGPU_PLUGIN_SOURCE="gpu_path_integral.C"', "-I" + d,
           "-I" + os.path.join(REPO, "tests", "plugin_stub"), "-I" + os.path.join(REPO, "include"),
           os.path.join(REPO, "tests", "plugin_main.cpp")]
    if link:
        cmd += ["-o", out, "-L" + LIBDIR, "-llooper_gb300", "-Wl,-rpath," + LIBDIR]
    else:
        cmd += ["-c", "-o", out + ".o"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-4000:]
    return d, out


def test_plugin_compiles():
    d, _ = _build(link=False)
    shutil.rmtree(d, ignore_errors=True)


@pytest.mark.gpu
def test_plugin_pushes_the_library_observables():
    import build as b
    b.build()
    import looper_gb300 as lg
    d, exe = _build(link=True)
    args = ["%s=%s" % kv for kv in PARAMS.items()]
    r = subprocess.run([exe] + args + ["--save-at", "250"], capture_output=True, text=True,
                       timeout=600)
    shutil.rmtree(d, ignore_errors=True)
    assert r.returncode == 0, r.stdout + r.stderr
    pushed = {}
    for line in r.stdout.splitlines():
        f = line.split("\t")
        if len(f) == 3:
            pushed[f[0]] = (int(f[1]), float(f[2]))
    assert "resumed identical" in r.stdout
    text = "".join("%s = %s\n" % (k, v if k != "LATTICE" else '"%s"' % v)
                   for k, v in PARAMS.items() if k != "WORKER_SEED")
    w = lg.LoopWorker(lg.parse_params(text))
    w.run(int(PARAMS["SWEEPS"]) + int(PARAMS["THERMALIZATION"]))
    obs = w.observables()
    common = [k for k in pushed if k in obs]
    assert {"Energy", "Energy Density", "Staggered Magnetization^2", "Susceptibility"} <= set(common)
    for k in common:
        count, mean = pushed[k]
        assert count == int(PARAMS["SWEEPS"]), k
        assert mean == pytest.approx(obs[k][0], rel=1e-12, abs=1e-12), k
    w.close()
