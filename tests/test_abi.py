"""The C-ABI library builds, loads and exports every entry point of include/looper_gpu.h.

No device work here: only host-side entry points (parameter defaults/parsing, names) are called.
"""
import ctypes
import math
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lg():
    sys.path.insert(0, os.path.join(REPO, "alps-looper_gb300"))
    import build as b
    b.build()
    import looper_gb300 as m
    return m


def test_exports_every_declared_symbol(lg):
    names = lg.exported_symbols()
    assert len(names) >= 25
    L = ctypes.CDLL(lg.LIB_PATH)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_nm_dynamic_symbols(lg):
    out = subprocess.run(["nm", "-D", "--defined-only", lg.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    syms = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    for n in lg.exported_symbols():
        assert n in syms, n


def test_params_defaults_follow_reference(lg):
    p = lg.make_params()
    assert p.lattice == lg.CHAIN and p.L == 8 and p.sweeps == 65536
    assert p.thermalization == -1  # SWEEPS/8 (montecarlo.h:41-45)
    assert math.isnan(p.Jz) and math.isnan(p.Jxy)


def test_params_parse_alps_keys(lg):
    p = lg.parse_params('LATTICE = "square lattice"; L = 128\nT = 1/64 # comment\nJ = 1;\n'
                        'SWEEPS = 8192; THERMALIZATION = 1024; SEED = 7\nh = 0.3\nJz = 0.5\n'
                        'INITIAL_SPINS = random')
    assert p.lattice == lg.SQUARE and p.L == 128
    assert p.T == pytest.approx(1 / 64)
    assert p.sweeps == 8192 and p.thermalization == 1024 and p.seed == 7
    assert p.h == 0.3 and p.Jz == 0.5 and math.isnan(p.Jxy) and p.init_spins == 1


def test_params_parse_correlation_switches(lg):
    p = lg.make_params()
    assert p.measure_correlations == 0 and p.measure_structure_factor == 0 and p.initial_site == -1
    p = lg.parse_params("MEASURE[Correlations] = true; MEASURE[Structure Factor] = 1;\n"
                        "INITIAL_SITE = 3")
    assert p.measure_correlations == 1 and p.measure_structure_factor == 1 and p.initial_site == 3
    with pytest.raises(lg.LoopError):
        lg.parse_params("MEASURE[Correlations] = maybe")


def test_params_parse_local_spin(lg):
    assert lg.make_params().spin2 == 1
    assert lg.parse_params("local_S = 1").spin2 == 2
    assert lg.parse_params("local_S = 3/2").spin2 == 3
    assert lg.make_params(local_S=1.5).spin2 == 3
    with pytest.raises(lg.LoopError):
        lg.parse_params("local_S = 0.3")


def test_params_parse_rejects_bad_values(lg):
    with pytest.raises(lg.LoopError) as e:
        lg.parse_params("L = abc")
    assert e.value.code == -1
    with pytest.raises(lg.LoopError) as e:
        lg.parse_params('LATTICE = "triangular lattice"')
    assert e.value.code == -4


def test_params_parse_rejects_out_of_range_integers(lg):
    # integer keys take finite values within their type's range, truncated toward zero
    for text in ("L = 1e300", "L = nan", "L = inf", "L = -3e9", "SWEEPS = -5", "SWEEPS = 1e30",
                 "SEED = nan", "SEED = -1", "SEED = 2e19", "THERMALIZATION = 1e300",
                 "INITIAL_SITE = 3e9", "local_S = 1e300", "local_S = inf"):
        with pytest.raises(lg.LoopError) as e:
            lg.parse_params(text)
        assert e.value.code == -1, text
    p = lg.parse_params("L = 8.9; SWEEPS = 1e4; THERMALIZATION = -1; INITIAL_SITE = -1; "
                        "SEED = 18446744073709549568")
    assert (p.L, p.sweeps, p.thermalization, p.initial_site) == (8, 10000, -1, -1)
    assert p.seed == 18446744073709549568


def test_params_parse_survives_random_text(lg):
    # random texts and random edits of a valid parameter file: the parser answers OK, LG_EINVAL
    # or LG_EUNSUPPORTED (an unknown LATTICE) and nothing else; a memory fault would end the run
    import numpy as np
    rng = np.random.default_rng(11)
    base = ('LATTICE = "square lattice"; L = 16\nT = 1/4 # comment\nJz = 0.5; Jxy = 1; h = 0.2\n'
            'SWEEPS = 1024; THERMALIZATION = 128; SEED = 3; local_S = 1/2\n'
            'MEASURE[Correlations] = true; INITIAL_SITE = 2; INITIAL_SPINS = random\n')
    alphabet = list('=;#"[]/ \n\t.-+eE0123456789abcdfinLTJhSWEPNAMRCU_xyz') + ["nan", "inf"]
    codes = set()
    for i in range(4000):
        if i % 4 == 0:
            text = "".join(rng.choice(alphabet, size=int(rng.integers(0, 240))))
        else:
            t = list(base)
            for _ in range(int(rng.integers(1, 8))):
                k = int(rng.integers(0, len(t) + 1))
                op = int(rng.integers(0, 3))
                if op == 0 and k < len(t):
                    del t[k]
                elif op == 1:
                    t.insert(k, str(rng.choice(alphabet)))
                elif k < len(t):
                    t[k] = str(rng.choice(alphabet))
            text = "".join(t)
        p = lg.Params()
        lg.lib().lg_params_default(ctypes.byref(p))
        rc = lg.lib().lg_params_parse(text.encode(), ctypes.byref(p))
        assert rc in (0, -1, -4), (rc, text)
        codes.add(rc)
    assert {0, -1} <= codes


def test_obs_names_match_reference_keys(lg):
    names = lg.obs_names()
    for key in ("Energy", "Energy Density", "Specific Heat", "Susceptibility",
                "Staggered Magnetization^2", "Staggered Susceptibility", "Number of Clusters"):
        assert key in names


def test_request_bytes_estimate(lg):
    small = lg.request_bytes(lg.make_params(LATTICE="square", L=8, T=1.0))
    big = lg.request_bytes(lg.make_params(LATTICE="square", L=64, T=1.0))
    cold = lg.request_bytes(lg.make_params(LATTICE="square", L=64, T=0.02))
    assert 0 < small < big < cold
    # about 1e7 operators at beta = 64 on 128x128 needs a few hundred MB, not GB
    b = lg.request_bytes(lg.make_params(LATTICE="square", L=128, BETA=64.0))
    assert 1e8 < b < 2e9
    assert lg.request_bytes(lg.make_params(LATTICE="square", L=7, T=1.0)) < 0  # sign problem


def test_host_allocation_failure_is_a_status_not_an_exception(lg):
    # lg_batch_create sizes its host-side chain table before reading any parameters: a count of
    # 2^31 - 1 chains (over 150 GB of table) fails to allocate, which the ABI must report as
    # LG_ENOMEM instead of letting std::bad_alloc through (that would end this process).  Only
    # where the kernel refuses an allocation larger than the machine's memory.
    try:
        mode = open("/proc/sys/vm/overcommit_memory").read().strip()
        mem = {}
        for ln in open("/proc/meminfo"):
            k, v = ln.split(":")
            mem[k] = int(v.split()[0]) * 1024
    except OSError:
        pytest.skip("no /proc to check the overcommit policy")
    n = 2 ** 31 - 1
    if mode == "1" or mem.get("MemTotal", 0) + mem.get("SwapTotal", 0) >= n * 72:
        pytest.skip("the kernel might grant the allocation")
    p = lg.Params()
    lg.lib().lg_params_default(ctypes.byref(p))
    out = ctypes.c_void_p()
    rc = lg.lib().lg_batch_create(n, ctypes.byref(p), ctypes.byref(out))
    assert rc == -2, (rc, lg.last_error())
    assert "allocation" in lg.last_error()


def test_invalid_models_are_rejected_before_device_work(lg):
    # lg_create validates the parameters (ChainSpec::init) before touching the GPU, so each of
    # these returns its status code on a machine without one
    cases = [
        (dict(LATTICE="chain", L=1), -1),                                 # LG_EINVAL
        (dict(LATTICE="chain", L=8, T=-1.0), -1),
        (dict(LATTICE="chain", L=8, T=float("nan")), -1),
        (dict(LATTICE="chain", L=8, BETA=float("inf")), -1),
        (dict(LATTICE="chain", L=8, T=1.0, Jz=float("inf")), -1),
        (dict(LATTICE="chain", L=8, T=1.0, h=float("nan")), -1),
        (dict(LATTICE="chain", L=8, T=1.0, FORCE_SCATTER=float("nan")), -1),
        (dict(LATTICE="cubic", L=162, T=1.0), -6),                        # > 2^22 sites: EBUDGET
        (dict(LATTICE="square", L=7, T=1.0), -4),                         # sign problem
        (dict(LATTICE="cubic", L=4, T=1.0, local_S=2.5), -4),             # 30 virtual neighbours
        (dict(LATTICE="chain", L=8, T=1.0, local_S=4.5), -4),             # 2S > 8 virtual sites
        (dict(LATTICE="chain", L=8, T=1.0, local_S=1, MEASURE_CORRELATIONS=True), -4),
        (dict(LATTICE="chain", L=8, T=1.0, MEASURE_CORRELATIONS=True, INITIAL_SITE=8), -1),
    ]
    for kw, code in cases:
        with pytest.raises(lg.LoopError) as e:
            lg.LoopWorker(lg.make_params(**kw))
        assert e.value.code == code, (kw, e.value)
