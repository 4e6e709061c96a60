"""The host packing of lg_load / lg_set_state (alps-looper_gb300/csrc/lg_pack.h) against a plain
restatement, without a GPU: endpoint lists per site in (time, bond) order, sites one after
another; invalid operators and odd sites reported.  Random operators on periodic chains and
square lattices, in order (the multi-threaded bucketed path) and shuffled (the sort path), from a
handful to a million operators."""
import os
import shutil
import subprocess
import tempfile

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>
#include "lg_pack.h"
using namespace lg;
int main(int argc, char** argv) {
  const int dim = std::atoi(argv[1]), L = std::atoi(argv[2]);
  const long long n = std::atoll(argv[3]);
  // 0 ordered, 1 shuffled, 2 one bad bond, 3 one bad time, 4 ordered with odd sites
  const int mode = std::atoi(argv[4]);
  const int threads = std::atoi(argv[5]);
  const unsigned seed = (unsigned)std::atoi(argv[6]);
  const int N = dim == 1 ? L : L * L, NB = dim * N;
  std::vector<int> s0(NB), s1(NB);
  std::vector<uint8_t> d0(NB), d1(NB);
  for (int i = 0; i < N; ++i)
    for (int a = 0; a < dim; ++a) {
      const int b = i * dim + a;
      const int x = i % L, y = i / L;
      s0[b] = i;
      s1[b] = a == 0 ? (x + 1) % L + y * L : x + ((y + 1) % L) * L;
      d0[b] = (uint8_t)(2 * a);
      d1[b] = (uint8_t)(2 * a + 1);
    }
  std::mt19937_64 g(seed);
  std::vector<int> bond(n);
  std::vector<double> tm(n);
  // operators in pairs on one bond, so that every site has an even count (a world line), except
  // in mode 4, where the last operator has no partner
  for (long long i = 0; i < n; ++i) {
    bond[i] = (i & 1) && !(mode == 4 && i == n - 1) ? bond[i - 1] : (int)(g() % NB);
    tm[i] = (double)(g() >> 11) * 0x1.0p-53;
  }
  // (time, bond) order, then per mode
  std::vector<long long> idx(n);
  for (long long i = 0; i < n; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](long long a, long long b) {
    return tm[a] < tm[b] || (tm[a] == tm[b] && bond[a] < bond[b]);
  });
  std::vector<int> ob(n);
  std::vector<double> ot(n);
  for (long long i = 0; i < n; ++i) { ob[i] = bond[idx[i]]; ot[i] = tm[idx[i]]; }
  if (mode == 1) {
    for (long long i = n - 1; i > 0; --i) {
      const long long j = (long long)(g() % (unsigned long long)(i + 1));
      std::swap(ob[i], ob[j]);
      std::swap(ot[i], ot[j]);
    }
  }
  const long long badi = n / 3;
  if (mode == 2) ob[badi] = NB;
  if (mode == 3) ot[badi] = 1.0;
  PackTables P;
  P.N = N; P.NB = NB; P.s0 = s0.data(); P.s1 = s1.data(); P.dir0 = d0.data(); P.dir1 = d1.data();
  P.check_parity = true;
  std::vector<uint64_t> t(2 * n + 1);
  std::vector<uint8_t> d(2 * n + 1);
  std::vector<PackRec> scratch(2 * n + 1);
  PackResult R;
  pack_site_lists(P, n, [&](long long i, int* b, uint64_t* tb) { *b = ob[i]; std::memcpy(tb, &ot[i], 8); },
                  t.data(), d.data(), scratch.data(), R, threads);
  if (mode == 2 || mode == 3) {
    std::printf("%s\n", R.bad == badi ? "ok" : "bad index not reported");
    return 0;
  }
  // the restatement: endpoints by site, (time bits, bond) order within a site
  std::vector<std::vector<std::pair<std::pair<uint64_t, int>, uint8_t>>> ref(N);
  for (long long i = 0; i < n; ++i) {
    uint64_t tb;
    std::memcpy(&tb, &ot[i], 8);
    ref[s0[ob[i]]].push_back({{tb, ob[i]}, d0[ob[i]]});
    ref[s1[ob[i]]].push_back({{tb, ob[i]}, d1[ob[i]]});
  }
  int odd = -1;
  for (int i = 0; i < N; ++i)
    if ((ref[i].size() & 1) && odd < 0) odd = i;
  if (R.ordered != (mode != 1) && n > 1) { std::printf("ordered flag %d\n", (int)R.ordered); return 0; }
  if (R.odd_site != odd) { std::printf("odd site %d, expected %d\n", R.odd_site, odd); return 0; }
  if (odd >= 0) { std::printf("ok\n"); return 0; }
  long long k = 0;
  for (int i = 0; i < N; ++i) {
    std::sort(ref[i].begin(), ref[i].end());
    if (R.oc[i] != (int)ref[i].size()) { std::printf("count of site %d\n", i); return 0; }
    for (auto& e : ref[i]) {
      if (t[k] != e.first.first || d[k] != e.second) { std::printf("entry %lld of site %d\n", k, i); return 0; }
      ++k;
    }
  }
  std::printf("ok\n");
  return 0;
}
"""


@pytest.fixture(scope="module")
def exe():
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    d = tempfile.mkdtemp()
    src = os.path.join(d, "pack.cpp")
    with open(src, "w") as fh:
        fh.write(SRC)
    out = os.path.join(d, "pack")
    cmd = [cxx, "-std=c++17", "-O2", "-pthread",
           "-I" + os.path.join(REPO, "alps-looper_gb300", "csrc"), src, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    yield out
    shutil.rmtree(d, ignore_errors=True)


def _run(exe, *args):
    r = subprocess.run([exe] + [str(a) for a in args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout.strip()


@pytest.mark.parametrize("dim,L,n,threads", [(1, 8, 8, 1), (1, 64, 5000, 4), (2, 16, 200000, 8),
                                             (2, 128, 1000000, 8), (1, 4096, 300002, 3)])
@pytest.mark.parametrize("mode", [0, 1, 4])
def test_packing_matches_the_restatement(exe, dim, L, n, threads, mode):
    for seed in (1, 2):
        assert _run(exe, dim, L, n, mode, threads, seed) == "ok"


@pytest.mark.parametrize("mode", [2, 3])
@pytest.mark.parametrize("threads", [1, 8])
def test_first_invalid_operator_is_reported(exe, mode, threads):
    assert _run(exe, 2, 32, 300000, mode, threads, 5) == "ok"
