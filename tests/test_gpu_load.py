"""lg_load's checks and packing on the GPU (a single chain on the grid path): a loaded checkpoint
continues exactly like the chain it came from; a checkpoint with an out-of-range operator or a
site that is not periodic in imaginary time is refused (re-signed, so that the checksum passes)
and leaves the chain as it was; operators out of order take the host packing and give the same
state as the ordered blob."""
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HEAD = 32


@pytest.fixture(scope="module")
def lg():
    import build as b
    b.build()
    import looper_gb300 as m
    return m


def _params(lg, seed=11):
    return lg.make_params(LATTICE="square", L=16, BETA=4.0, J=1.0, SEED=seed, SWEEPS=4096,
                          THERMALIZATION=0, INITIAL_SPINS="random")


def _split(blob, nsites):
    n = struct.unpack_from("<Q", blob, 24)[0]
    rec = np.frombuffer(blob, dtype=np.dtype([("b", "<i4"), ("t", "<f8")]), count=n,
                        offset=HEAD + nsites).copy()
    return bytearray(blob[:HEAD + nsites]), rec


def _join(lg, head, rec):
    out = bytearray(head)
    struct.pack_into("<Q", out, 24, len(rec))
    out += rec.tobytes() + b"\0" * 8
    struct.pack_into("<Q", out, len(out) - 8, lg.checkpoint_checksum(out))
    return bytes(out)


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a.state(), b.state()))


def test_load_continues_like_the_source(lg):
    src = lg.LoopWorker(_params(lg))
    src.run(40)
    blob = src.save()
    dst = lg.LoopWorker(_params(lg))  # the seed is a parameter, not part of the checkpoint
    dst.load(blob)
    assert _same(src, dst)
    src.run(15)
    dst.run(15)
    assert _same(src, dst)
    src.close()
    dst.close()


def test_rejected_checkpoints_leave_the_chain(lg):
    src = lg.LoopWorker(_params(lg))
    src.run(30)
    blob = src.save()
    n_sites = 16 * 16
    head, rec = _split(blob, n_sites)
    assert len(rec) > 10
    w = lg.LoopWorker(_params(lg, seed=5))
    w.run(7)
    before = w.state()
    # an operator on a bond that does not exist
    bad = rec.copy()
    bad["b"][len(bad) // 2] = 2 * n_sites
    with pytest.raises(lg.LoopError) as e:
        w.load(_join(lg, head, bad))
    assert e.value.code == -7 and "out of range" in str(e.value)
    # a time outside [0, 1)
    bad = rec.copy()
    bad["t"][3] = 1.0
    with pytest.raises(lg.LoopError) as e:
        w.load(_join(lg, head, bad))
    assert e.value.code == -7
    # one operator fewer: its two sites flip an odd number of times
    with pytest.raises(lg.LoopError) as e:
        w.load(_join(lg, head, rec[1:]))
    assert e.value.code == -1 and "periodic" in str(e.value)
    for x, y in zip(before, w.state()):
        assert np.array_equal(x, y)
    # the chain still runs, and a good checkpoint still loads
    w.run(3)
    w.load(blob)
    assert _same(src, w)
    src.close()
    w.close()


def test_unordered_operators_pack_on_the_host(lg):
    src = lg.LoopWorker(_params(lg))
    src.run(25)
    blob = src.save()
    head, rec = _split(blob, 16 * 16)
    shuffled = rec[np.random.default_rng(3).permutation(len(rec))]
    a = lg.LoopWorker(_params(lg))
    a.load(_join(lg, head, shuffled))
    assert _same(src, a)
    src.run(10)
    a.run(10)
    assert _same(src, a)
    src.close()
    a.close()
