"""The allocation-free labelling entry point (lg_uf_label_static) against lg_uf_label.

lg_uf_label_static serves callers that cannot allocate device memory: it takes device buffers
owned by the caller and keeps its intermediates in a fixed static device array.  Its labels must
equal those of the allocating entry point exactly (labels are integers), on consecutive calls
that share that static array.  This file is collected last on purpose.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lg():
    import build as b
    b.build()
    import looper_gb300 as m
    return m


def _static_labels(lg, torch, c):
    bonds = torch.tensor(c["bonds"], dtype=torch.int32, device="cuda")
    graphs = torch.tensor(c["graphs"], dtype=torch.int32, device="cuda")
    nfrag_max = c["N"] + len(c["bonds"]) + 1
    out = torch.full((nfrag_max,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    nf, nc = lg.uf_label_static(c["dim"], c["L"], len(c["bonds"]), bonds.data_ptr(),
                                graphs.data_ptr(), out.data_ptr(), 0)
    torch.cuda.synchronize()
    return out[:nf].cpu().numpy(), nc


def test_static_labels_equal_allocating_labels_on_consecutive_calls(lg, golden):
    torch = pytest.importorskip("torch")
    cases = golden("uf_labels.json")
    # two calls in a row on different configurations share the static scratch
    for c in (cases[2], cases[4], cases[2]):
        ref, rnc = lg.uf_label(c["dim"], c["L"], c["bonds"], c["graphs"])
        lab, nc = _static_labels(lg, torch, c)
        assert nc == rnc
        assert lab.tolist() == ref.tolist()
        assert lab.tolist() == c["labels_deterministic"]


def test_static_rejects_sizes_beyond_its_limit(lg):
    torch = pytest.importorskip("torch")
    dummy = torch.zeros(4, dtype=torch.int32, device="cuda")
    with pytest.raises(lg.LoopError) as e:
        lg.uf_label_static(2, 256, 4, dummy.data_ptr(), dummy.data_ptr(), dummy.data_ptr(), 0)
    assert e.value.code == -6 and "static limit" in str(e.value)
    with pytest.raises(lg.LoopError) as e:
        lg.uf_label_static(1, 64, (1 << 18) + 1, dummy.data_ptr(), dummy.data_ptr(),
                           dummy.data_ptr(), 0)
    assert e.value.code == -6
