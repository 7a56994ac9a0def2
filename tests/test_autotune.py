"""The autotuner's host logic without a GPU: the workload key, the JSON
cache (store, reload, a corrupt file), the defaults for an unknown key, and
that every candidate geometry is one the plan accepts (period cap^2 <= 8 x
threads per CTA, the accumulator bound of the tiled kernels)."""
import json

from rc_gb300 import autotune as AT


def test_signature_buckets_the_workload():
    sup, counts = [8, 16, 32], [1000, 500, 100]
    a = AT.signature(sup, counts, kept=1600, tiles_occupied=40, grid_edge=2048)
    assert a == AT.signature(sup, counts, kept=1600, tiles_occupied=40, grid_edge=2048)
    assert a.startswith("smax32-")
    # 8x denser or a 4x larger grid change the key; a few percent do not
    assert AT.signature(sup, counts, 12800, 40, 2048) != a
    assert AT.signature(sup, counts, 1600, 40, 8192) != a
    assert AT.signature(sup, counts, 1650, 40, 2048) == a


def test_cache_round_trip_and_defaults(tmp_path, monkeypatch):
    monkeypatch.setenv("RC_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    assert AT.best("unknown") == AT.DEFAULT
    params = {"tile": 16, "threads": 512, "period_cap": 32, "bundles_per_cta": 8}
    AT._store({"k1": {"params": params, "ms": 1.0}})
    assert AT.best("k1") == params
    assert json.load(open(tmp_path / "tune.json"))["k1"]["params"] == params
    (tmp_path / "tune.json").write_text("{not json")
    assert AT._load() == {}
    assert AT.best("k1") == AT.DEFAULT


def test_every_candidate_is_a_valid_geometry():
    assert AT.DEFAULT in AT.CANDIDATES
    for c in AT.CANDIDATES:
        assert c["period_cap"] ** 2 <= 8 * c["threads"]
        assert c["tile"] > 0 and c["bundles_per_cta"] > 0
    assert len({tuple(sorted(c.items())) for c in AT.CANDIDATES}) == len(AT.CANDIDATES) == 54
