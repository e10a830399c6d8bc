"""mbe_enumerate_static: enumeration that allocates no device memory.

It exists for callers that may not allocate device memory while they run
(hosts that own the device through their own pool allocator, serving loops
that cannot afford the synchronisation of cudaMalloc/cudaFree, plugin
runtimes without an allocation budget).  The test allocates the graph and
result buffers itself (with torch), calls the entry point through the C ABI
twice in a row, and checks count and canonical hash bit-exactly against
mbe_enumerate and the CPU oracle on the same graph.  Collected last so that a failure here
stops a -x run only after every other test has run.
"""
import numpy as np
import pytest

import cumbe_gb300 as cm
import oracle
from conftest import random_csr

pytestmark = pytest.mark.gpu


def _device_csr(nr, nc, rp, ci):
    import torch
    rp = np.asarray(rp, dtype=np.int64)
    ci = np.asarray(ci, dtype=np.int64)
    rows = np.repeat(np.arange(nr), np.diff(rp))
    order = np.lexsort((rows, ci))  # transpose: by col, then row
    cp = np.zeros(nc + 1, np.int64)
    np.add.at(cp, ci + 1, 1)
    cp = np.cumsum(cp)
    dev = "cuda:0"
    as_u32 = lambda a: torch.tensor(np.asarray(a, dtype=np.int32), dtype=torch.int32, device=dev)
    return [as_u32(rp), as_u32(ci if ci.size else [0]), as_u32(cp), as_u32(rows[order] if ci.size else [0])]


def _call_static(nr, nc, bufs, variant="cuMBE"):
    import torch
    out = torch.zeros(2, dtype=torch.int64, device="cuda:0")
    st = cm.lib().mbe_enumerate_static(nr, nc, bufs[0].data_ptr(), bufs[1].data_ptr(), bufs[2].data_ptr(),
                                       bufs[3].data_ptr(), cm.VARIANTS[variant], out.data_ptr(), None)
    torch.cuda.synchronize()
    assert st == 0, cm.lib().mbe_last_error().decode()
    c, h = (int(x) & 0xFFFFFFFFFFFFFFFF for x in out.cpu().tolist())
    return c, h


@pytest.mark.parametrize("case", ["random_60x40", "power_law_2000x1000", "wide_40x300"])
def test_static_matches_enumerate_twice(engine, case):
    rng = np.random.default_rng(21)
    if case == "random_60x40":
        g = random_csr(rng, 60, 40, 0.15)
    elif case == "wide_40x300":
        g = random_csr(rng, 40, 300, 0.05)
    else:
        g = cm.Graph.generate(2000, 1000, 10000, 2.1, 2.1, 0, 1).csr()
    nr, nc, rp, ci = g
    want = engine.enumerate(cm.Graph.from_csr(nr, nc, rp, ci))
    ref = oracle.ref_enumerate(nr, nc, rp, ci, threads=4)
    assert (want.count, want.hash) == (ref.count, ref.hash)
    bufs = _device_csr(nr, nc, rp, ci)
    for _ in range(2):  # the second call reuses the array the first one left behind
        assert _call_static(nr, nc, bufs) == (want.count, want.hash)


def _wide_row_csr(rng, nr=100, nc=3000, wide_deg=2600, p=0.05):
    """Row 0 meets wide_deg of the nc cols (a root whose degree needs more
    than the 4,096 u32 of shared histogram: 2 x degree > 4096); the other
    rows are uniform at density p, so row 0's root has candidates of higher
    id (a non-empty P side) and of lower id (none: it is row 0) alike."""
    M = rng.random((nr, nc)) < p
    M[0, :] = False
    M[0, rng.choice(nc, wide_deg, replace=False)] = True
    rp = np.zeros(nr + 1, np.uint64)
    rp[1:] = np.cumsum(M.sum(1))
    return nr, nc, rp, np.nonzero(M)[1].astype(np.uint32)


@pytest.mark.parametrize("wide_row", [0, 57])
def test_static_row_wider_than_shared_histogram(engine, wide_row):
    """A row of degree 2,600 of 3,000 cols: its root expansion keeps the
    count histogram in the per-block global scratch, which must be sized
    for the widest row.  Count and hash bit-exact against the oracle and
    against mbe_enumerate, on two calls in a row."""
    rng = np.random.default_rng(5 + wide_row)
    nr, nc, rp, ci = _wide_row_csr(rng)
    if wide_row:
        # move the wide row to position wide_row: its root then has both a Q
        # (rows below it) and a P (rows above it) side
        order = np.r_[np.arange(1, wide_row + 1), 0, np.arange(wide_row + 1, nr)]
        deg = np.diff(rp.astype(np.int64))
        rows = [ci[rp[r]:rp[r + 1]] for r in range(nr)]
        rows = [rows[r] for r in order]
        rp = np.zeros(nr + 1, np.uint64)
        rp[1:] = np.cumsum([len(x) for x in rows])
        ci = np.concatenate(rows).astype(np.uint32)
        assert deg.max() == 2600
    want = oracle.ref_enumerate(nr, nc, rp, ci, threads=4)
    got = engine.enumerate(cm.Graph.from_csr(nr, nc, rp, ci))
    assert (got.count, got.hash) == (want.count, want.hash)
    bufs = _device_csr(nr, nc, rp, ci)
    for _ in range(2):
        assert _call_static(nr, nc, bufs) == (want.count, want.hash)


def test_static_rejects_oversized_graphs(engine):
    import torch
    dummy = torch.zeros(8, dtype=torch.int32, device="cuda:0")
    out = torch.zeros(2, dtype=torch.int64, device="cuda:0")
    st = cm.lib().mbe_enumerate_static(5000, 10, dummy.data_ptr(), dummy.data_ptr(), dummy.data_ptr(),
                                       dummy.data_ptr(), 0, out.data_ptr(), None)
    assert st == 7  # MBE_ERR_CAPACITY
    assert "at most 4096" in cm.lib().mbe_last_error().decode()
