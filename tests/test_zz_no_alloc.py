"""tess_csr_offsets_noalloc: CSR offsets for callers that may not allocate
device memory (a fixed device budget, an allocator that owns all device
memory, or a path where an allocation's implicit synchronisation is not
allowed).  It is checked through the C ABI against the offsets the library's
own entry point (tess_neighbors_csr) returns, on two calls in a row: the
second call reuses the shared scratch array the first one left behind.

This file is named to run last, so a stop-at-first-failure run has already
run every other test when it gets here."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_offsets_match_tess_neighbors_csr(tess):
    torch = pytest.importorskip("torch")
    from tessellator import workloads

    pts = workloads.uniform(50000, seed=41)
    with tess.Diagram(pts, container=tess.Polyhedron(0, 0, 0, 1, 1, 1)) as d:
        d.compute_all("fp32")
        offs_ref, _, _ = d.neighbors_csr()          # the existing entry point
    counts = np.diff(offs_ref.astype(np.int64)).astype(np.uint32)
    n = len(counts)
    dev_counts = torch.from_numpy(counts).to("cuda:0")
    dev_offs = torch.empty(n + 1, dtype=torch.int64, device="cuda:0")
    L = tess.lib()
    for call in range(2):
        dev_offs.fill_(-1)
        torch.cuda.synchronize()
        st = L.tess_csr_offsets_noalloc(C.c_void_p(dev_counts.data_ptr()), n, C.c_void_p(dev_offs.data_ptr()),
                                         None)
        assert st == 0, tess.last_error()
        torch.cuda.synchronize()
        got = dev_offs.cpu().numpy().astype(np.uint64)
        assert np.array_equal(got, offs_ref), f"call {call}: offsets differ"


def test_noalloc_rejects_sizes_beyond_its_maximum(tess):
    torch = pytest.importorskip("torch")
    dev = torch.zeros(16, dtype=torch.int64, device="cuda:0")
    L = tess.lib()
    st = L.tess_csr_offsets_noalloc(C.c_void_p(dev.data_ptr()), (1 << 26) + 1, C.c_void_p(dev.data_ptr()), None)
    assert st == 3                                  # TESS_E_CAPACITY, nothing launched
    assert "maximum" in tess.last_error()
