"""Long runs of the 8,000-sphere settle judged by ensemble statistics.

Granular flow is chaotic: a rounding-level difference in one force grows
until two runs differ sphere by sphere after a few thousand steps.  So the
mixed form is compared with the FP64 form over 30,000 steps (0.3 s, from the
lattice through the collapse into a bed) by the statistics of the state, each
within a stated band:

* the kinetic-energy decay curve, sampled every 1,000 steps: within 0.3
  decades (a factor of two) wherever either run's energy is above 1e-3 of the
  peak;
* the packing fraction of the bed's interior (ensemble.bed_box): within 0.01;
* the mean coordination number (particle-particle contacts per sphere):
  within 0.25.

The same bands hold between the FP64 form and itself started 1e-12 m away
(every sphere displaced at random by that much): the natural spread of the
statistics, which the bands must exceed to mean anything.
"""
import numpy as np
import pytest

from metakonga_gb300 import engine, ensemble, scenes

pytestmark = pytest.mark.gpu

STEPS, EVERY = 30_000, 1_000
KE_DECADES, PHI_BAND, Z_BAND = 0.3, 0.01, 0.25


def _run(sc, mode, oracle):
    ds = engine.DeviceScene(sc, mode=mode)
    ke = []
    for _ in range(STEPS // EVERY):
        ds.step(EVERY, check=True)
        st = ds.download()
        ke.append(ensemble.kinetic_energy(st["vel"], st["omega"], sc.mass, sc.inertia))
    if mode == engine.MODE_MIXED:
        pairs = ds.pair_list(cap=32)
    else:
        p = sc.params.copy()
        p["np"] = sc.np_
        pos = np.ascontiguousarray(st["pos"])
        _, _, cs, ce, so = oracle.detection(p, pos)
        pairs = oracle.pair_list(p, pos, so, cs, ce)
    ds.close()
    lo, hi = ensemble.bed_box(st["pos"], (-0.15, -0.15, 0.0), (0.15, 0.15, 0.5))
    return {"ke": np.array(ke), "phi": ensemble.packing_fraction(st["pos"], lo, hi),
            "z": ensemble.coordination(pairs, sc.np_), "zmin": float(st["pos"][:, 2].min())}


def _bands(a, b):
    floor = 1e-3 * max(a["ke"].max(), b["ke"].max())
    return (ensemble.log_band(a["ke"], b["ke"], floor), abs(a["phi"] - b["phi"]), abs(a["z"] - b["z"]))


def test_settle_8000_mixed_within_ensemble_bands_of_fp64(cuda, oracle):
    sc = scenes.settle_box()
    ref = _run(sc, engine.MODE_FP64, oracle)
    mix = _run(sc, engine.MODE_MIXED, oracle)
    pert = sc.copy()
    rng = np.random.Generator(np.random.MT19937(99))
    pert.pos[:, :3] += rng.choice([-1e-12, 1e-12], size=(sc.np_, 3))
    nat = _run(pert, engine.MODE_FP64, oracle)
    # the run reaches a bed: energy down from its peak, contacts everywhere
    assert ref["ke"][-1] < 0.05 * ref["ke"].max() and ref["z"] > 3.5 and ref["phi"] > 0.5, ref
    for name, (dke, dphi, dz) in (("mixed", _bands(mix, ref)), ("fp64 perturbed", _bands(nat, ref))):
        assert dke <= KE_DECADES, (name, dke)
        assert dphi <= PHI_BAND, (name, dphi, mix["phi"], nat["phi"], ref["phi"])
        assert dz <= Z_BAND, (name, dz, mix["z"], nat["z"], ref["z"])
    assert mix["zmin"] > -0.001
