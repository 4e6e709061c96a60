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
        f = ln.split("\t")
        if f[0] == "V":
            out["V:" + f[1]] = float(f[2])
        else:
            out[f[0]] = (float(f[1]), float(f[2]))
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


# Values a worker plug-in pushes per sweep (lg_fetch_values) whose plain mean is, by the
# reference's own definitions, the mean lg_observables reports under the same name.
SAME = ["Energy", "Energy Density", "Energy^2", "Magnetization", "|Magnetization|",
        "Magnetization^2", "Magnetization^4", "Susceptibility", "Staggered Magnetization^2",
        "Staggered Magnetization^4", "Staggered Susceptibility", "Generalized Magnetization^2",
        "Generalized Susceptibility", "Number of Clusters", "Stiffness"]


@pytest.mark.parametrize("name", sorted(CASES))
def test_per_sweep_values_reproduce_observables(exe, name):
    """The per-sweep values a parapack plug-in pushes into its ObservableSet average to the
    means lg_observables reports (path_integral.C:827-862 pushes; the engine's binned view)."""
    dim, L, beta, jxy, jz, h, spin2, disable = CASES[name]
    got = _observables(exe, dim, L, beta, jxy, jz, h, spin2, disable, 50, 3000, 7 + len(name))
    improved = not disable and h == 0.0
    checked = 0
    for k in SAME:
        if ("V:" + k) not in got:
            assert k.startswith("Generalized") and not improved, k
            continue
        m = got[k][0]
        assert got["V:" + k] == pytest.approx(m, rel=1e-12, abs=1e-300), (name, k)
        checked += 1
    assert checked >= 12
    # constant entries and the reference's fixed zeros of the improved estimator
    assert got["V:Inverse Temperature"] == beta
    assert got["V:Temperature"] == pytest.approx(1.0 / beta, rel=1e-15)
    assert got["V:Volume"] == L ** dim and got["V:Number of Sites"] == L ** dim
    if improved:
        assert got["V:Magnetization"] == 0.0 and got["V:Staggered Magnetization"] == 0.0
        assert "V:Generalized Staggered Susceptibility" in got
    else:
        assert "V:Generalized Magnetization^2" not in got
    assert got["V:Energy Density"] == pytest.approx(got["V:Energy"] / L ** dim, rel=1e-12)
