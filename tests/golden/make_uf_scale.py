"""Cluster labels at scale from the reference's own union-find (run in the build container only).

Two cluster-construction configurations of the 2D Heisenberg antiferromagnet, made by the CPU
oracle (Philox mode, so they can be made again anywhere from the seed):
  * 32x32, beta = 16, seed 2101, 24 sweeps: about 2e4 vertices.  Stored whole (bonds, graphs)
    with the reference's deterministic labels, compressed: uf_scale_32.npz.
  * 128x128, beta = 64, seed 2102, 12 sweeps (the operator count is settled by then): about
    1.2e6 vertices, the bench workload's size.  Too large to store, so uf_scale.json keeps the
    SHA-256 of the configuration (bonds and graphs as little-endian int32) and of the reference's
    labels, and the cluster count; the GPU test makes the configuration again with the oracle,
    checks its hash and compares the labels' hash.
The labels come from oracle/_ref/uf_deterministic (looper/union_find.h compiled in place with
-DLOOPER_USE_DETERMINISTIC_UNIFY, union_find.h:231-233) fed with the reference's fragment
sequence (graph_impl.h:280-295, path_integral.C:482,584-589: sites first, a new fragment per
graph-0 vertex in time order, then the temporal closure), and are checked against the partition
of oracle/_ref/uf_weighted (the default unify).

Usage:  make -C oracle all ref REFERENCE=<ref> && python tests/golden/make_uf_scale.py
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "tests"))

from oracle_lib import Oracle  # noqa: E402

CASES = {
    "square32_b16": dict(dim=2, L=32, beta=16.0, seed=2101, sweeps=24),
    "square128_b64": dict(dim=2, L=128, beta=64.0, seed=2102, sweeps=12),
}


def config(c):
    """The oracle's last cluster-construction configuration after c["sweeps"] sweeps."""
    o = Oracle(c["dim"], c["L"], c["beta"], 1.0, 1.0, 0.0, seed=c["seed"])
    o.sweep(c["sweeps"])
    cfg = o.last_config()
    s0, s1 = o.bonds()
    o.close()
    return (np.asarray(cfg["bonds"], dtype=np.int32), np.asarray(cfg["graphs"], dtype=np.int32),
            np.asarray(s0), np.asarray(s1))


def config_sha(bonds, graphs):
    return hashlib.sha256(bonds.astype("<i4").tobytes() + graphs.astype("<i4").tobytes()).hexdigest()


def labels_sha(labels):
    return hashlib.sha256(np.asarray(labels, dtype="<i4").tobytes()).hexdigest()


def _sequence(N, s0, s1, bonds, graphs):
    cur = list(range(N))
    out = []
    nfrag = N
    for b, g in zip(bonds.tolist(), graphs.tolist()):
        a, c = int(s0[b]), int(s1[b])
        c0, c1 = cur[a], cur[c]
        if g & 2:
            out.append("u %d %d" % (c0, c1))
            cur[a] = cur[c] = c0
        elif g == 0:
            out.append("a")
            out.append("u %d %d" % (c0, c1))
            cur[a] = cur[c] = nfrag
            nfrag += 1
        else:
            cur[a], cur[c] = c1, c0
    for s in range(N):
        out.append("u %d %d" % (s, cur[s]))
    return out


def _ref_ids(binary, N, seq):
    text = "%d %d\n%s\nids\n" % (N, len(seq), "\n".join(seq))
    r = subprocess.run([binary], input=text, capture_output=True, text=True, check=True)
    nums = np.array(r.stdout.split(), dtype=np.int64)
    return int(nums[0]), nums[1:].astype(np.int32)


def _canon(lab):
    _, first = np.unique(lab, return_index=True)
    order = np.argsort(first)
    remap = np.empty(order.size, dtype=np.int64)
    remap[order] = np.arange(order.size)
    return remap[np.searchsorted(np.unique(lab), lab)]


def main():
    det = os.path.join(REPO, "oracle", "_ref", "uf_deterministic")
    wei = os.path.join(REPO, "oracle", "_ref", "uf_weighted")
    meta = {}
    for name, c in CASES.items():
        bonds, graphs, s0, s1 = config(c)
        N = c["L"] ** c["dim"]
        seq = _sequence(N, s0, s1, bonds, graphs)
        nc, ids = _ref_ids(det, N, seq)
        ncw, idw = _ref_ids(wei, N, seq)
        assert nc == ncw and np.array_equal(_canon(ids), _canon(idw))
        meta[name] = dict(c, N=N, nops=int(bonds.size), nfrag=int(ids.size), nc=nc,
                          config_sha256=config_sha(bonds, graphs), labels_sha256=labels_sha(ids))
        if name == "square32_b16":
            np.savez_compressed(os.path.join(HERE, "uf_scale_32.npz"), bonds=bonds.astype(np.int16),
                                graphs=graphs.astype(np.int8), labels=ids)
        print(name, "vertices", bonds.size, "fragments", ids.size, "clusters", nc)
    with open(os.path.join(HERE, "uf_scale.json"), "w") as f:
        json.dump(meta, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
