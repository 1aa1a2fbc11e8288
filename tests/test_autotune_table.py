"""The serving autotuner's bucketing and table (CPU)."""
import os

from sisi4s_gb300 import autotune


def test_buckets_cover_the_request_stream():
    seen = set()
    for No in range(4, 17):
        for Nv in range(20, 161):
            seen.add(autotune.bucket_of(No, Nv))
    assert seen == {(i, j) for i in range(3) for j in range(3)}
    # outside the tuned ranges: the nearest bucket
    assert autotune.bucket_of(2, 10) == (0, 0)
    assert autotune.bucket_of(40, 400) == (2, 2)


def test_lookup_without_a_table_changes_nothing():
    assert autotune.lookup(None, "emu", 8, 50) == {}
    assert autotune.lookup({"emu": []}, "emu", 8, 50) == {}


def test_committed_table_is_complete():
    assert os.path.exists(autotune.TABLE)
    t = autotune.load()
    keys = {"emu": {"emu_min_flops", "f64_split_blocks", "emu_max_ksplit"},
            "fp64": {"f64_split_blocks"}}
    for prec, want in keys.items():
        rows = t[prec]
        assert sorted(tuple(r["bucket"]) for r in rows) == [(i, j) for i in range(3)
                                                            for j in range(3)]
        for r in rows:
            assert set(r["setting"]) == want
            assert r["setting"] in autotune.candidates(prec)
            # the kept setting is the cheapest one measured
            assert r["cost_ms"] == min(x["cost_ms"] for x in r["tried"])
            assert r["cost_ms"] <= r["default_cost_ms"]
        assert autotune.lookup(t, prec, 10, 100) == rows[[tuple(r["bucket"])
                                                          for r in rows].index((1, 2))]["setting"]
