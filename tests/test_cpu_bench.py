"""bench.py's host-side figures, without a GPU: the DRAM traffic per unit it
reads from the committed ncu summaries, the measured peaks, the rank
environment, and the summaries' commands (each one a bench.py run, with the
GPU clocks left alone)."""
import json
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture
def bench(monkeypatch):
    # bench sets CUDA_DEVICE_MAX_CONNECTIONS on import: keep that to this test
    monkeypatch.setenv("CUDA_DEVICE_MAX_CONNECTIONS", os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS", "32"))
    monkeypatch.syspath_prepend(ROOT)
    import bench as b
    return b


def test_traffic_figures_come_from_the_profiles(bench):
    adv = bench._traffic_from_profiles("advance_batch_hopper.md", "traffic_bytes_per_particle")
    con = bench._traffic_from_profiles("contact_mixed_hopper_settled.md", "traffic_bytes_per_listed_sphere")
    assert adv == pytest.approx(323.7) and con == pytest.approx(275.8)
    # DRAM bytes near the algorithmic figures: no wholesale re-reads
    assert 0.8 * bench.B_ADVANCE <= adv <= 1.2 * bench.B_ADVANCE
    assert bench.B_LISTED <= con <= 2 * bench.B_LISTED
    for name in ("advance_mixed_polydisperse_box.md", "contact_mixed_polydisperse_box.md",
                 "p2p_fp64_polydisperse_box.md"):
        assert bench._traffic_from_profiles(name) > 0
    assert bench._traffic_from_profiles("no_such_profile.md") is None
    assert bench._traffic_from_profiles("advance_batch_hopper.md", "no_such_key") is None


def test_peaks_are_the_measured_ones(bench):
    peak, kind = bench._peaks()
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            assert kind == "measured" and peak == float(json.load(f)["hbm_gbs"])
    else:
        assert kind == "fallback" and peak == 6800.0


def test_rank_environment(bench, monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert bench._dist() == (1, 0, 0)
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert bench._dist() == (2, 1, 1)


def test_profiles_give_bench_commands_with_clocks_left_alone():
    d = os.path.join(ROOT, "profiles")
    names = sorted(os.listdir(d))
    assert names
    for f in names:
        assert f.endswith((".md", ".txt")), f
        text = open(os.path.join(d, f)).read()
        # a command may continue over lines ending in a backslash
        cmd = re.sub(r"\\\n\s*", " ", text)
        lines = [ln for ln in cmd.splitlines() if re.search(r"(^|\s)ncu\s", ln) and ln.startswith("    ")]
        assert lines, f
        for ln in lines:
            assert "--clock-control none" in ln, (f, ln)
            assert "python bench.py" in ln, (f, ln)
