"""Generate the golden fixtures under tests/golden/ (run in the build container only).

Sources:
  * standalone/loop.op            -> standalone_loop_op.json   (deterministic standalone run)
  * test/union_find.op            -> union_find_op.json        (100 unions + full listing)
  * loop.op (diag, PI, SSE)      -> loop_op.json              (known answers, L=4 chains,
                                                                  with the correlation vectors)
  * oracle (philox mode) configs  -> uf_labels.json            (cluster-construction configs)
  * oracle/ed.py (momentum ED)    -> ed_chain16.json           (exact L=16 chain at T=0.1)
    labelled by the reference's own looper/union_find.h, compiled in place by oracle/Makefile
    (oracle/_ref/uf_deterministic, oracle/_ref/uf_weighted).

Usage:  make -C oracle all ref REFERENCE=<ref> && python tests/golden/make_golden.py <ref>
        (<ref>: a checkout of the reference; required)
"""
from __future__ import annotations

import ctypes
import json
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "tests"))

from oracle_lib import Oracle  # noqa: E402


def standalone(ref):
    text = open(os.path.join(ref, "standalone", "loop.op")).read().splitlines()
    out = {"L": 8, "T": 0.2, "therm": 8192, "sweeps": 65536, "lines": text[:9]}
    return out


def union_find(ref):
    lines = open(os.path.join(ref, "test", "union_find.op")).read().splitlines()
    pairs = []
    for ln in lines:
        m = re.match(r"connecting node (\d+) to node (\d+)", ln)
        if m:
            pairs.append([int(m.group(1)), int(m.group(2))])
    i = lines.index("[results]")
    return {"n": 100, "pairs": pairs, "listing": lines[i + 1:]}


def _block(lines, start, keys):
    vals = {}
    for ln in lines[start:]:
        if ln.startswith("[input parameters]") and vals:
            break
        for k in keys:
            if ln.startswith(k + ":"):
                m = re.match(re.escape(k) + r": (\S+) \+/- (\S+)", ln)
                vals[k] = [float(m.group(1)), m.group(2).rstrip(";")]
    return vals


VECTORS = ["Spin Correlations", "Staggered Spin Correlations", "Spin Structure Factor"]


def _vectors(lines, start):
    """Vector observables of the block starting at `start`: name -> [[label, mean, error]...]
    from the "Entry[label]: mean +/- error" lines after the name line."""
    out = {}
    cur = None
    for ln in lines[start:]:
        if ln.startswith("[input parameters]"):
            break
        if ln in VECTORS:
            cur = out.setdefault(ln, [])
            continue
        m = re.match(r"Entry\[(.*)\]: (\S+) \+/- (\S+);", ln)
        if m and cur is not None:
            cur.append([m.group(1), float(m.group(2)), float(m.group(3))])
        elif not ln.startswith("Entry[") and not ln.startswith("    bin"):
            cur = None
    return out


def loop_op(ref):
    lines = open(os.path.join(ref, "loop.op")).read().splitlines()
    keys = ["Energy", "Specific Heat", "Magnetization^2", "Susceptibility",
            "Staggered Magnetization^2", "Staggered Susceptibility", "Number of Clusters"]
    # block start lines (0-based) located by their parameter headers
    blocks = []
    for i, ln in enumerate(lines):
        if ln.startswith("ALGORITHM = "):
            hdr = lines[max(0, i - 12):i + 1]
            blocks.append((i, hdr))
    out = []
    for i, hdr in blocks:
        h = "\n".join(hdr)
        alg = lines[i].split("=", 1)[1].strip().rstrip(";").strip('"')
        if alg not in ("diagonalization", "loop; path integral", "loop; sse"):
            continue
        lat = re.findall(r'LATTICE = "?([^";]+)"?;', h)
        if not lat or lat[-1] != "chain lattice":
            continue
        # spin-1 blocks are kept when they have no single-ion anisotropy D
        spin = re.findall(r"local_S = ([^;]+);", h)
        spin2 = round(2 * eval(spin[-1].replace("/", "/ "))) if spin else 1
        D = re.findall(r"\nD = ([^;]+);", "\n" + h)
        if D and float(D[-1]) != 0.0:
            continue
        L = int(re.findall(r"\nL = ([^;]+);", "\n" + h)[-1])
        T = re.findall(r"\nT = ([^;]+);", "\n" + h)
        Tv = T[-1].replace("L", str(L))
        Tf = float(eval(Tv))
        jz = re.findall(r"Jz = ([^;]+);", h)
        jxy = re.findall(r"Jxy = ([^;]+);", h)
        vals = _block(lines, i + 1, keys)
        entry = {"algorithm": alg, "L": L, "T": Tf,
                 "jz": float(jz[-1]) if jz else 1.0, "jxy": float(jxy[-1]) if jxy else 1.0,
                 "values": vals}
        if spin2 != 1:
            entry["spin2"] = spin2
        vec = _vectors(lines, i + 1)
        if vec:
            entry["vectors"] = vec
        out.append(entry)
    return out


def _ref_ids(binary, nsites, seq):
    text = "%d %d\n%s\nids\n" % (nsites, len(seq), "\n".join(seq))
    res = subprocess.run([binary], input=text, capture_output=True, text=True, check=True)
    nums = [int(x) for x in res.stdout.split()]
    return nums[0], nums[1:]


def _reconnect_sequence(N, s0, s1, bonds, graphs):
    cur = list(range(N))
    seq = []
    nfrag = N
    for b, g in zip(bonds, graphs):
        a, c = s0[b], s1[b]
        c0, c1 = cur[a], cur[c]
        if g & 2:
            seq.append("u %d %d" % (c0, c1))
            cur[a] = cur[c] = c0
        elif g == 0:
            seq.append("a")
            f = nfrag
            nfrag += 1
            seq.append("u %d %d" % (c0, c1))
            cur[a] = cur[c] = f
        else:
            cur[a], cur[c] = c1, c0
    for s in range(N):
        seq.append("u %d %d" % (s, cur[s]))
    return seq


def uf_labels():
    cases = [
        dict(name="chain16_heisenberg_b10", dim=1, L=16, beta=10.0, jxy=1.0, jz=1.0, h=0.0, sweeps=40),
        dict(name="chain64_heisenberg_b10", dim=1, L=64, beta=10.0, jxy=1.0, jz=1.0, h=0.0, sweeps=20),
        dict(name="square8_heisenberg_b4", dim=2, L=8, beta=4.0, jxy=1.0, jz=1.0, h=0.0, sweeps=20),
        dict(name="square6_xxz_jz05_b3", dim=2, L=6, beta=3.0, jxy=1.0, jz=0.5, h=0.0, sweeps=20),
        dict(name="cubic4_xxz_jz15_h02_b2", dim=3, L=4, beta=2.0, jxy=1.0, jz=1.5, h=0.2, sweeps=20),
        dict(name="chain12_ferro_b5", dim=1, L=12, beta=5.0, jxy=-1.0, jz=-1.0, h=0.0, sweeps=20),
        dict(name="chain10_ising_b2", dim=1, L=10, beta=2.0, jxy=0.0, jz=1.0, h=0.0, sweeps=20),
    ]
    out = []
    ubin_d = os.path.join(REPO, "oracle", "_ref", "uf_deterministic")
    ubin_w = os.path.join(REPO, "oracle", "_ref", "uf_weighted")
    for c in cases:
        o = Oracle(c["dim"], c["L"], c["beta"], c["jxy"], c["jz"], c["h"], seed=12345)
        o.sweep(c["sweeps"])
        cfg = o.last_config()
        s0, s1 = o.bonds()
        seq = _reconnect_sequence(o.N, s0, s1, cfg["bonds"], cfg["graphs"])
        nc_d, ids_d = _ref_ids(ubin_d, o.N, seq)
        nc_w, ids_w = _ref_ids(ubin_w, o.N, seq)
        assert nc_d == nc_w
        out.append(dict(c, seed=12345, N=o.N, spins=cfg["spins"], bonds=cfg["bonds"],
                        graphs=cfg["graphs"], offdiag=cfg["offdiag"],
                        times=[float.hex(t) for t in cfg["times"]],
                        nc=nc_d, labels_deterministic=ids_d, labels_weighted=ids_w))
        o.close()
    return out


def ed_chain16():
    """Exact values for the S=1/2 Heisenberg chain L=16, J=1, T=0.1 (the CPU-runnable chain
    workload's correctness point), from the momentum-sector restatement of diag.C in
    oracle/ed.py (about 20 s of CPU, hence stored)."""
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "..", "oracle"))
    import ed
    r = ed.chain_translation(16, 0.1, 1.0, 1.0, 0.0)
    return {"L": 16, "T": 0.1, "jxy": 1.0, "jz": 1.0, "h": 0.0,
            "values": {k: (list(map(float, v)) if hasattr(v, "__len__") else float(v))
                       for k, v in r.items()}}


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference checkout>")
    ref = sys.argv[1]
    data = {
        "standalone_loop_op.json": standalone(ref),
        "union_find_op.json": union_find(ref),
        "loop_op.json": loop_op(ref),
        "uf_labels.json": uf_labels(),
        "ed_chain16.json": ed_chain16(),
    }
    for name, obj in data.items():
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(obj, f, indent=None, separators=(",", ":"))
            f.write("\n")
        print("wrote", name)


if __name__ == "__main__":
    main()
