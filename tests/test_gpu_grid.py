"""Cell grid on the GPU against the oracle: hash, stable sort, cell ranges.
Integer results must be bit-exact."""
import numpy as np
import pytest
import torch

from metakonga_gb300 import dem, scenes
from metakonga_gb300._lib import call, ptr
from metakonga_gb300.layouts import make_params

from .cases import packed_scene, random_positions

pytestmark = pytest.mark.gpu


def _gpu_detection(prm, pos, sphere=None):
    dem.set_symbolic_parameter(prm)
    g = dem.NeighborhoodCell()
    g.setGridSize(prm["grid"])
    npt = pos.shape[0]
    nt = 0 if sphere is None else sphere.shape[0]
    g.initialize(npt + nt)
    dpos = dem.to_dev(pos)
    dsph = dem.to_dev(sphere) if nt else None
    g.detection(dpos, dsph, npt, nt)
    torch.cuda.synchronize()
    u = lambda t, n: t[:n].cpu().numpy().view(np.uint32)
    n = npt + nt
    return (u(g.cellID(), n), u(g.bodyID(), n), u(g.cellStart(), g.ng), u(g.cellEnd(), g.ng),
            u(g.sortedID(), n))


def _check_same(gpu, ref):
    names = ("hash", "index", "cstart", "cend", "sorted")
    for name, a, b in zip(names, gpu, ref):
        assert a.shape == b.shape, name
        bad = np.flatnonzero(a != b)
        assert bad.size == 0, f"{name}: {bad.size} mismatches, first at {bad[:5]}"


def test_grid_settle_box(cuda, oracle):
    sc = scenes.settle_box()
    _check_same(_gpu_detection(sc.params, sc.pos), oracle.detection(sc.params, sc.pos))


def test_grid_packed_and_wrapped(cuda, oracle):
    """Negative coordinates and positions beyond 128 cells exercise the & wrap."""
    pos = random_positions(50_000, (-1.7, -1.2, -0.9), (1.9, 0.6, 2.5), 0.002, 0.004, seed=11)
    prm = make_params(np_=pos.shape[0], ncell=128 ** 3, grid=(128, 128, 128), dt=1e-5,
                      cell_size=0.008, world_origin=(-1.0, -1.0, -1.0), gravity=(0, 0, -9.81))
    _check_same(_gpu_detection(prm, pos), oracle.detection(prm, pos))


def test_grid_exact_cell_faces(cuda, oracle):
    """Particles exactly on cell boundaries (and one ulp either side)."""
    cs = 0.01
    k = np.arange(-40, 40)
    base = -1.0 + k * cs
    vals = np.concatenate([base, np.nextafter(base, -np.inf), np.nextafter(base, np.inf)])
    rng = np.random.Generator(np.random.MT19937(4))
    pos = np.empty((vals.size * 3, 4))
    for a in range(3):
        pos[:, a] = rng.permutation(np.tile(vals, 3))
    pos[:, 3] = 0.004
    prm = make_params(np_=pos.shape[0], ncell=64 * 64 * 64, grid=(64, 64, 64), dt=1e-5, cell_size=cs,
                      world_origin=(-1.0, -1.0, -1.0), gravity=(0, 0, -9.81))
    _check_same(_gpu_detection(prm, pos), oracle.detection(prm, pos))


def test_grid_all_in_one_cell_and_single(cuda, oracle):
    prm = make_params(np_=1, ncell=8 ** 3, grid=(8, 8, 8), dt=1e-5, cell_size=0.1,
                      world_origin=(0.0, 0.0, 0.0), gravity=(0, 0, -9.81))
    one = np.array([[0.05, 0.05, 0.05, 0.01]])
    _check_same(_gpu_detection(prm, one), oracle.detection(prm, one))
    same = np.tile(one, (5000, 1))
    _check_same(_gpu_detection(prm, same), oracle.detection(prm, same))


def test_grid_with_triangle_spheres(cuda, oracle):
    sc = packed_scene(n_side=8)
    rng = np.random.Generator(np.random.MT19937(9))
    sph = np.empty((3000, 4))
    sph[:, :3] = rng.uniform(sc.pos[:, :3].min(0), sc.pos[:, :3].max(0), size=(3000, 3))
    sph[:, 3] = 0.003
    _check_same(_gpu_detection(sc.params, sc.pos, sph), oracle.detection(sc.params, sc.pos, sph))


def test_grid_empty(cuda):
    prm = make_params(np_=0, ncell=4 ** 3, grid=(4, 4, 4), dt=1e-5, cell_size=0.1,
                      world_origin=(0.0, 0.0, 0.0), gravity=(0, 0, -9.81))
    dem.set_symbolic_parameter(prm)
    g = dem.NeighborhoodCell()
    g.setGridSize((4, 4, 4))
    g.initialize(0)
    g.d_cell_start.fill_(7)
    g.d_cell_end.fill_(7)
    g.detection(dem.to_dev(np.zeros((1, 4))), None, 0, 0)
    torch.cuda.synchronize()
    assert (g.cellStart().cpu().numpy().view(np.uint32) == 0xFFFFFFFF).all()
    assert (g.cellEnd().cpu().numpy() == 0).all()


@pytest.mark.parametrize("n,bits", [(1, 21), (4097, 21), (1_000_003, 21), (300_000, 32), (77_777, 9)])
def test_radix_sort_stable(cuda, n, bits):
    rng = np.random.Generator(np.random.MT19937(n + bits))
    hi = (1 << bits) if bits < 32 else (1 << 32)
    keys = rng.integers(0, min(hi, 1 << 32), size=n, dtype=np.uint64).astype(np.uint32)
    if n > 10:
        keys[: n // 3] = keys[n // 3]          # many ties
    vals = np.arange(n, dtype=np.uint32)
    dk = torch.from_numpy(keys.view(np.int32).copy()).cuda()
    dv = torch.from_numpy(vals.view(np.int32).copy()).cuda()
    call("xd_radix_sort_pairs", ptr(dk), ptr(dv), n, bits, dem.stream_handle())
    torch.cuda.synchronize()
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(dk.cpu().numpy().view(np.uint32), keys[order])
    assert np.array_equal(dv.cpu().numpy().view(np.uint32), vals[order])


def test_hash_out_of_range_is_an_error(cuda):
    """A hash value >= ncell (a caller whose ncell is smaller than the grid) is
    reported as XD_ERR_INVALID instead of writing past cstart/cend."""
    from metakonga_gb300._lib import XdemError
    n = 100
    keys = torch.full((n,), 70, dtype=torch.int32, device="cuda")
    idx = torch.arange(n, dtype=torch.int32, device="cuda")
    cs = torch.zeros(64, dtype=torch.int32, device="cuda")
    ce = torch.zeros(64, dtype=torch.int32, device="cuda")
    so = torch.zeros(n, dtype=torch.int32, device="cuda")
    with pytest.raises(XdemError):
        call("xd_reorder_and_find_cell_start", ptr(keys), ptr(idx), ptr(cs), ptr(ce), ptr(so), n, 64,
             dem.stream_handle())
