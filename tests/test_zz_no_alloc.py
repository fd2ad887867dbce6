"""The allocation-free cell-range entry point (xd_reorder_and_find_cell_start_noalloc).

It exists for callers that may not allocate device memory while they run (an
application that hands out all device memory from its own pool at start-up,
or a process held to a fixed memory budget): its sort scratch is a fixed
device array inside libxdem.  The test calls it through the C ABI twice in a
row, on different inputs, and checks each result bit for bit against the
ordinary entry point (integer results, so the tolerance is zero); then it
checks the size limit, and that a later call leaves the device's free memory
unchanged (under lazy module loading the first call on a device is the one
that brings in the fixed array).  This file is collected last so that a run stopping at
the first failure has already run every other test; it also passes alone.
"""
import numpy as np
import pytest
import torch

from metakonga_gb300 import dem
from metakonga_gb300._lib import XdemError, call, lib, ptr
from metakonga_gb300.layouts import make_params

pytestmark = pytest.mark.gpu

MAX_ENTRIES = 1 << 20


def _hashes(n, seed, ncell):
    """Cell hashes of random positions, computed by the library's own hash call."""
    rng = np.random.Generator(np.random.MT19937(seed))
    pos = np.empty((n, 4))
    pos[:, :3] = rng.uniform(-1.0, 0.02, size=(n, 3))
    pos[:, 3] = 0.004
    side = round(ncell ** (1 / 3))
    prm = make_params(np_=n, ncell=ncell, grid=(side, side, side), dt=1e-5, cell_size=0.008,
                      world_origin=(-1.0, -1.0, -1.0), gravity=(0, 0, -9.81))
    dem.set_symbolic_parameter(prm)
    h = torch.zeros(n, dtype=torch.int32, device="cuda")
    ix = torch.zeros(n, dtype=torch.int32, device="cuda")
    dpos = dem.to_dev(pos)
    call("xd_calculate_hash_and_index", ptr(h), ptr(ix), ptr(dpos), n, dem.stream_handle())
    torch.cuda.synchronize()
    return h, ix


def _run(entry, h, ix, ncell):
    n = h.numel()
    hh, ii = h.clone(), ix.clone()
    cs = torch.full((ncell,), 123, dtype=torch.int32, device="cuda")
    ce = torch.full((ncell,), 456, dtype=torch.int32, device="cuda")
    so = torch.zeros(n, dtype=torch.int32, device="cuda")
    call(entry, ptr(hh), ptr(ii), ptr(cs), ptr(ce), ptr(so), n, ncell, dem.stream_handle())
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in (hh, ii, cs, ce, so)]


@pytest.mark.parametrize("calls", [[(700_001, 1), (MAX_ENTRIES, 2)]])
def test_noalloc_matches_allocating_entry_point(calls):
    assert torch.cuda.is_available()
    assert lib().xd_reorder_and_find_cell_start_noalloc is not None
    ncell = 128 ** 3
    for n, seed in calls:          # two calls in a row share the fixed scratch
        h, ix = _hashes(n, seed, ncell)
        got = _run("xd_reorder_and_find_cell_start_noalloc", h, ix, ncell)
        want = _run("xd_reorder_and_find_cell_start", h, ix, ncell)
        for name, a, b in zip(("hash", "index", "cstart", "cend", "sorted"), got, want):
            assert np.array_equal(a, b), f"{name} differs for n={n}"
        assert (got[2] != -1).sum() > 1000          # many occupied cells


def test_noalloc_rejects_more_than_the_maximum():
    n = MAX_ENTRIES + 1
    ncell = 64 ** 3
    h = torch.zeros(n, dtype=torch.int32, device="cuda")
    ix = torch.arange(n, dtype=torch.int32, device="cuda")
    cs = torch.zeros(ncell, dtype=torch.int32, device="cuda")
    ce = torch.zeros(ncell, dtype=torch.int32, device="cuda")
    so = torch.zeros(n, dtype=torch.int32, device="cuda")
    with pytest.raises(XdemError) as ei:
        call("xd_reorder_and_find_cell_start_noalloc", ptr(h), ptr(ix), ptr(cs), ptr(ce), ptr(so), n,
             ncell, dem.stream_handle())
    assert ei.value.status == 4 and "maximum" in str(ei.value)


def test_noalloc_later_call_takes_no_device_memory():
    """After a set-up call with n = 0, a full-size call changes nothing in the
    device's free memory: the scratch is the fixed array, not an allocation."""
    n, ncell = 500_000, 128 ** 3
    h, ix = _hashes(n, 3, ncell)
    cs = torch.zeros(ncell, dtype=torch.int32, device="cuda")
    ce = torch.zeros(ncell, dtype=torch.int32, device="cuda")
    so = torch.zeros(n, dtype=torch.int32, device="cuda")
    # the set-up call: no entries, only the cell arrays are cleared
    call("xd_reorder_and_find_cell_start_noalloc", None, None, ptr(cs), ptr(ce), None, 0, ncell,
         dem.stream_handle())
    torch.cuda.synchronize()
    assert int((cs == -1).sum()) == ncell and int(ce.abs().sum()) == 0
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        call("xd_reorder_and_find_cell_start_noalloc", ptr(h), ptr(ix), ptr(cs), ptr(ce), ptr(so), n,
             ncell, dem.stream_handle())
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert free1 == free0, (free0, free1)
    # sorted_index is a permutation of the entries' indices
    assert torch.equal(torch.sort(so).values, torch.arange(n, device="cuda", dtype=torch.int32))
