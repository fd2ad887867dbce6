"""Result and restart files in the reference's byte layouts (no GPU)."""
import struct

import numpy as np

from metakonga_gb300 import results


def test_part_file_layout_and_round_trip(tmp_path):
    rng = np.random.Generator(np.random.MT19937(5))
    pos = rng.normal(size=(7, 4))
    path = results.part_name(str(tmp_path), 12)
    assert path.endswith("part0012.bin")
    results.write_part(path, 0.125, pos)
    raw = open(path, "rb").read()
    # double ct, uint np, double pos[np][4] (dem_simulation.cpp:491-519)
    assert len(raw) == 8 + 4 + 7 * 4 * 8
    assert struct.unpack("<dI", raw[:12]) == (0.125, 7)
    assert np.array_equal(np.frombuffer(raw[12:], "<f8").reshape(7, 4), pos)
    ct, back = results.read_part(path)
    assert ct == 0.125 and np.array_equal(back, pos)
    # single-precision model: float positions
    results.write_part(path, 1.0, pos, precision=1)
    assert len(open(path, "rb").read()) == 12 + 7 * 4 * 4
    ct, back = results.read_part(path, precision=1)
    assert np.array_equal(back, pos.astype(np.float32))


def test_final_file_layout_and_round_trip(tmp_path):
    rng = np.random.Generator(np.random.MT19937(6))
    n = 9
    pos, vel, avel = rng.normal(size=(n, 4)), rng.normal(size=(n, 3)), rng.normal(size=(n, 3))
    path = str(tmp_path / "model_final.bfr")
    results.write_final(path, 2.5, pos, vel, avel)
    raw = open(path, "rb").read()
    # double ct, int precision = 2, int flag = 1, pos, vel, avel (xDynamicsSolver.cpp:111-130,
    # dem_simulation.cpp:551-566)
    assert struct.unpack("<dii", raw[:16]) == (2.5, 2, 1)
    assert len(raw) == 16 + n * 10 * 8
    ct, prec, p, v, a = results.read_final(path, n)
    assert (ct, prec) == (2.5, 2)
    assert np.array_equal(p, pos) and np.array_equal(v, vel) and np.array_equal(a, avel)
    results.write_final(path, 2.5, pos, vel, avel, precision=1)
    ct, prec, p, v, a = results.read_final(path, n)
    assert prec == 1 and p.dtype == np.float32 and np.array_equal(v, vel.astype(np.float32))
    # a file without particle data (flag != 1) gives no arrays
    with open(path, "wb") as f:
        f.write(struct.pack("<dii", 3.0, 2, 0))
    assert results.read_final(path, n)[2:] == (None, None, None)


def test_checkpoint_round_trip(tmp_path):
    rng = np.random.Generator(np.random.MT19937(7))
    n = 11
    st = {"pos": rng.normal(size=(n, 4))}
    for k in ("vel", "acc", "omega", "alpha", "force", "moment"):
        st[k] = rng.normal(size=(n, 3))
    m, inertia = rng.uniform(1, 2, n), rng.uniform(1, 2, n)
    path = str(tmp_path / "c.ckpt")
    results.write_checkpoint(path, 0.75, st, m, inertia)
    ct, back = results.read_checkpoint(path)
    assert ct == 0.75
    for k in st:
        assert np.array_equal(back[k], st[k]), k
    assert np.array_equal(back["mass"], m) and np.array_equal(back["inertia"], inertia)
