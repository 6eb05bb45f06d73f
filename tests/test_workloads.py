"""Host-side logic of the batched and served forms (no GPU): the seeded ensemble and request
generators against the distributions they state, and the tile autotuner's choices."""
import ctypes as C
import math

import numpy as np
import pytest

from kestrel_gb300 import abi, autotune, workloads


@pytest.fixture
def flat_terrain(monkeypatch):
    """The draws do not depend on the terrain: skip the spectral synthesis."""
    monkeypatch.setattr(workloads, "fractal_terrain", lambda nx, ny, dx, seed, **kw: np.zeros((ny, nx)))


def test_ensemble_draws(flat_terrain):
    """Sides log-uniform in [128, 1024] (multiples of 64), volumes log-uniform in [1e3, 1e6]
    m^3, drag from Chezy / Voellmy / Manning, morphodynamics and cap-or-flux about half
    each, every member a valid run whose tile side divides the grid with an interior."""
    import _oracle
    O = _oracle.load()
    members = workloads.ensemble(96, seed=2024)
    sides = np.array([d["side"] for _, _, d in members])
    vols = np.array([d["volume"] for _, _, d in members])
    assert sides.min() >= 128 and sides.max() <= 1024 and (sides % 64 == 0).all()
    assert len(set(sides)) >= 6
    assert vols.min() >= 1e3 and vols.max() <= 1e6
    # log-uniform: log10 V uniform on [3, 6] (mean 4.5, sd 0.87); log2 side uniform on [7, 10]
    logv, logs = np.log10(vols), np.log2(sides)
    assert abs(logv.mean() - 4.5) < 0.3 and 0.65 < logv.std() < 1.05
    assert abs(logs.mean() - 8.5) < 0.3 and 0.65 < logs.std() < 1.05
    assert {d["drag"] for _, _, d in members} == set(workloads.DRAGS)
    assert 0.3 <= np.mean([d["morpho"] for _, _, d in members]) <= 0.7
    assert 0.3 <= np.mean([d["source"][0] == "cap" for _, _, d in members]) <= 0.7
    for p, b0, d in members:
        t = d["tile"]
        assert d["side"] % t == 0 and d["side"] // t >= 4
        assert b0.shape == (d["side"] + 1, d["side"] + 1)
        assert p.MorphodynamicsOn == int(d["morpho"]) and p.bcs == abi.BCS["sponge"]
        assert 60.0 <= p.tend <= 600.0
        h = C.c_void_p()
        assert O.ko_create(C.byref(p), C.byref(h)) == abi.KG_OK, O.ko_last_error(None)
        O.ko_destroy(h)


def test_ensemble_is_reproducible(flat_terrain):
    a = workloads.ensemble(8, seed=7)
    b = workloads.ensemble(8, seed=7)
    for (pa, _, da), (pb, _, db) in zip(a, b):
        assert da == db and bytes(pa) == bytes(pb)


def test_request_stream(flat_terrain):
    """Poisson arrivals at the stated rate, sides from the stated set, end times in range."""
    reqs = workloads.serve_requests(200, rate=20.0, seed=77, sides=(256, 512))
    t = np.array([r[0] for r in reqs])
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert (gaps > 0).all()
    assert abs(1.0 / gaps.mean() - 20.0) < 4.0                       # rate within ~3 standard errors
    assert abs(gaps.std() / gaps.mean() - 1.0) < 0.25                # exponential: cv ~ 1
    assert {r[3]["side"] for r in reqs} == {256, 512}
    assert all(60.0 <= r[1].tend <= 600.0 for r in reqs)


def test_autotune_candidates_and_mapping(tmp_path):
    assert autotune.candidates(128) == [16, 32]
    assert autotune.candidates(1024) == [16, 32, 64]
    assert autotune.candidates(192) == [16, 32]          # 192 / 64 = 3 tiles: no interior
    assert autotune.candidates(48) == []
    tuned = {128: 16, 512: 32, 2048: 64}
    assert autotune.tile_for(128, tuned) == 16
    assert autotune.tile_for(576, tuned) == 32           # nearest class in log size: 512
    assert autotune.tile_for(1024, tuned) in (32, 64)
    assert autotune.tile_for(192, {2048: 64}) == 32      # the tuned 64 leaves no interior here
    assert autotune.tile_for(512, {}) == 64              # untuned: the largest candidate
    cache = tmp_path / "tiles.json"
    cache.write_text('{"256": 32, "1024": 64}')
    assert autotune.tune(cache=str(cache)) == {256: 32, 1024: 64}  # read back without trials
    assert math.isfinite(autotune.tile_for(300, autotune.tune(cache=str(cache))))


def test_autotune_choice_is_stable_within_the_noise():
    """Candidates within 5% of the fastest resolve to the largest of them; a smaller tile
    wins only when it is faster by more than that."""
    assert autotune.choose({16: 1.00, 32: 0.97, 64: 1.00}) == 64
    assert autotune.choose({16: 1.00, 32: 0.90, 64: 1.00}) == 32
    assert autotune.choose({32: 2.0, 64: 2.08}) == 64
    assert autotune.choose({32: 2.0, 64: 2.2}) == 32
