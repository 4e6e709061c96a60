"""The allocation-free labelling entry point (lg_uf_label_static) against lg_uf_label.

lg_uf_label_static serves callers that cannot allocate device memory (a plug-in under a framework
that owns every device allocation, or a path that cannot take cudaFree's device-wide
synchronisation): it takes device buffers owned by the caller and keeps its intermediates in a
fixed static device array.  Its labels must equal those of the allocating entry point exactly
(labels are integers), on consecutive calls that share that static array, up to the advertised
size limits; it must leave the rest of the caller's output buffer alone and take no device memory.
This file is collected last on purpose.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_OPS = 1 << 18


@pytest.fixture(scope="module")
def lg():
    import build as b
    b.build()
    import looper_gb300 as m
    return m


def _static_labels(lg, torch, dim, L, bonds, graphs):
    bonds = torch.tensor(np.asarray(bonds, dtype=np.int32), device="cuda")
    graphs = torch.tensor(np.asarray(graphs, dtype=np.int32), device="cuda")
    nfrag_max = L ** dim + len(bonds) + 1
    out = torch.full((nfrag_max,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    nf, nc = lg.uf_label_static(dim, L, len(bonds), bonds.data_ptr(), graphs.data_ptr(),
                                out.data_ptr(), 0)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    lab = out.cpu().numpy()
    assert np.all(lab[nf:] == -7), "wrote past the fragments"
    return lab[:nf], nc, free1 - free0


def test_static_labels_equal_allocating_labels_on_consecutive_calls(lg, golden):
    torch = pytest.importorskip("torch")
    cases = golden("uf_labels.json")
    # calls in a row on different configurations share the static scratch
    for i, c in enumerate((cases[2], cases[4], cases[2])):
        ref, rnc = lg.uf_label(c["dim"], c["L"], c["bonds"], c["graphs"])
        lab, nc, dfree = _static_labels(lg, torch, c["dim"], c["L"], c["bonds"], c["graphs"])
        assert nc == rnc
        assert lab.tolist() == ref.tolist()
        assert lab.tolist() == c["labels_deterministic"]
        if i > 0:  # after the first call's one-time set-up: no device memory taken
            assert dfree == 0


def test_static_labels_near_the_size_limits(lg):
    """A 128x128 configuration of about 2x10^5 vertices (the oracle's, beta = 10) and a two-site
    chain carrying the full 2^18 vertices on its two bonds: labels equal lg_uf_label's."""
    torch = pytest.importorskip("torch")
    import oracle_lib as orc
    o = orc.Oracle(2, 128, 10.0, 1.0, 1.0, 0.0, seed=77)
    o.sweep(5)
    cfg = o.last_config()
    o.close()
    assert 1 << 17 < len(cfg["bonds"]) <= MAX_OPS
    rng = np.random.default_rng(5)
    two = (rng.integers(0, 2, MAX_OPS).astype(np.int32), rng.integers(0, 2, MAX_OPS).astype(np.int32))
    for dim, L, bonds, graphs in ((2, 128, cfg["bonds"], cfg["graphs"]), (1, 2) + two):
        ref, rnc = lg.uf_label(dim, L, bonds, graphs)
        for k in range(2):
            lab, nc, dfree = _static_labels(lg, torch, dim, L, bonds, graphs)
            assert nc == rnc and np.array_equal(lab, ref)
            if k > 0:  # the first call in a fresh process may do the one-time set-up
                assert dfree == 0


def test_static_rejects_sizes_beyond_its_limit(lg):
    torch = pytest.importorskip("torch")
    dummy = torch.zeros(4, dtype=torch.int32, device="cuda")
    with pytest.raises(lg.LoopError) as e:
        lg.uf_label_static(2, 256, 4, dummy.data_ptr(), dummy.data_ptr(), dummy.data_ptr(), 0)
    assert e.value.code == -6 and "static limit" in str(e.value)
    with pytest.raises(lg.LoopError) as e:
        lg.uf_label_static(1, 64, MAX_OPS + 1, dummy.data_ptr(), dummy.data_ptr(),
                           dummy.data_ptr(), 0)
    assert e.value.code == -6
