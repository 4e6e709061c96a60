"""The product's host measurement code against exact diagonalization, without a GPU.

tests/measure_check.cpp feeds the CPU oracle's per-sweep records (bit-identical to the GPU's, by
the record parity tests) through record_values and ChainAcc of alps-looper_gb300/csrc/lg_host.cpp,
the code lg_observables reports from.  Its observables, with their binning or jackknife errors,
must lie within 3.5 sigma of ED:
* the improved estimators and, with DISABLE_IMPROVED_ESTIMATOR, the normal ones (the reference's
  check/chain-6 case);
* a field (normal estimators, path_integral.C:217), the square and cubic lattices, spin 1.
"""
import os
import shutil
import subprocess
import tempfile

import pytest

import oracle_lib as orc

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def exe():
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    d = tempfile.mkdtemp()
    out = os.path.join(d, "measure_check")
    cmd = [cxx, "-std=c++17", "-O2", "-I" + os.path.join(REPO, "include"),
           "-I" + os.path.join(REPO, "alps-looper_gb300", "csrc"),
           os.path.join(REPO, "alps-looper_gb300", "csrc", "lg_host.cpp"),
           os.path.join(REPO, "oracle", "looper_oracle.cpp"),
           os.path.join(REPO, "tests", "measure_check.cpp"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    yield out
    shutil.rmtree(d, ignore_errors=True)


def _observables(exe, dim, L, beta, jxy, jz, h, spin2, disable, therm, sweeps, seed):
    args = [str(x) for x in (dim, L, beta, jxy, jz, h, spin2, disable, therm, sweeps, seed)]
    r = subprocess.run([exe] + args, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    out = {}
    for ln in r.stdout.splitlines():
        name, m, e = ln.split("\t")
        out[name] = (float(m), float(e))
    return out


CASES = {
    # dim, L, beta, jxy, jz, h, spin2, disable_improved
    "chain_heisenberg_normal": (1, 8, 2.0, 1.0, 1.0, 0.0, 1, 1),
    "chain_heisenberg_improved": (1, 8, 2.0, 1.0, 1.0, 0.0, 1, 0),
    "square_xxz_field": (2, 2, 2.0, 1.0, 0.5, 0.3, 1, 0),
    "cubic_xxz_normal": (3, 2, 2.0, 1.0, 0.5, 0.0, 1, 1),
    "chain_spin1_normal": (1, 4, 2.0, 1.0, 1.0, 0.0, 2, 1),
}
KEYS = ["Energy", "Energy Density", "Specific Heat", "Magnetization^2", "Susceptibility",
        "Staggered Magnetization^2", "Staggered Susceptibility"]


@pytest.mark.parametrize("name", sorted(CASES))
def test_host_measurement_of_oracle_records_vs_ed(exe, name):
    dim, L, beta, jxy, jz, h, spin2, disable = CASES[name]
    got = _observables(exe, dim, L, beta, jxy, jz, h, spin2, disable, 1000, 40000,
                       100 + len(name))
    ref = orc.ed.thermal(dim, L, 1.0 / beta, jxy=jxy, jz=jz, h=h, spin2=spin2)
    for k in KEYS:
        m, e = got[k]
        assert e > 0, k
        assert abs(m - ref[k]) <= 3.5 * e + 1e-12, (name, k, m, e, ref[k])
