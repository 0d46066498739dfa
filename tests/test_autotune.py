"""The autotuner's bookkeeping on the CPU: size buckets, the settings it
skips as equivalent, and the per-bucket table's round trip through JSON.
(The timed search itself runs in the benchmark on a GPU.)"""
import json


class FakeEngine:
    def __init__(self, n, scenes=0):
        self.n = n
        self.n_scenes = scenes


def test_buckets():
    from stardust_gb300 import autotune
    assert autotune.bucket_of(FakeEngine(100)) == "scene:2^12"
    assert autotune.bucket_of(FakeEngine(4096)) == "scene:2^12"
    assert autotune.bucket_of(FakeEngine(1 << 20)) == "scene:2^18"
    assert autotune.bucket_of(FakeEngine(2_097_151)) == "scene:2^18"
    assert autotune.bucket_of(FakeEngine(2_097_152)) == "scene:2^21"
    assert autotune.bucket_of(FakeEngine(3_000_000, 512)) == "batch:2^21"
    assert autotune.bucket_of(FakeEngine(3_000_000, 1)) == "scene:2^21"


def test_equivalent_settings_are_skipped():
    from stardust_gb300 import autotune
    r = autotune._redundant
    assert r({"contact_mode": 1, "skin_um": 50})
    assert r({"contact_mode": 1, "skin_um": 0, "contact_block": 128})
    assert not r({"contact_mode": 1, "skin_um": 0, "listed_blocks": 5, "contact_block": 256})
    assert r({"skin_um": 0, "listed_blocks": 4})
    assert not r({"skin_um": 20, "listed_blocks": 4})
    assert r({"resort_max": 0, "skin_um": 20})
    # every knob value the searches try is accepted by the library
    from stardust_gb300 import _abi
    for space in (autotune.SCENE_KNOBS, autotune.BATCH_KNOBS):
        for k, values in space.items():
            old = _abi.tune_get(k)
            try:
                for v in values:
                    _abi.tune_set(k, v)
                    assert _abi.tune_get(k) == v
            finally:
                _abi.tune_set(k, old)


def test_table_round_trip(tmp_path, sdlib):
    from stardust_gb300 import _abi, autotune
    autotune._TABLE.clear()
    autotune._TABLE["scene:2^12"] = {"skin_um": 20, "contact_block": 128}
    f = tmp_path / "tune.json"
    autotune.save(f)
    assert json.loads(f.read_text()) == {"scene:2^12": {"contact_block": 128, "skin_um": 20}}
    autotune._TABLE.clear()
    assert autotune.load(f) == {"scene:2^12": {"skin_um": 20, "contact_block": 128}}
    old = {k: _abi.tune_get(k) for k in ("skin_um", "contact_block")}
    try:
        assert autotune.apply(FakeEngine(1000)) == {"skin_um": 20, "contact_block": 128}
        assert _abi.tune_get("skin_um") == 20 and _abi.tune_get("contact_block") == 128
        assert autotune.apply(FakeEngine(1 << 20)) is None
    finally:
        for k, v in old.items():
            _abi.tune_set(k, v)
        autotune._TABLE.clear()


def test_coordinate_descent_finds_the_best_setting(sdlib):
    """The search on a stand-in timer (a cost of the current knobs): it
    reaches the best combination, skips equivalent settings, records every
    timed setting under the statistic's name, sets the choice and keeps it
    for the bucket or label."""
    from stardust_gb300 import _abi, autotune

    class Eng(FakeEngine):
        def step(self, dt, k):
            pass

        def sync(self):
            pass

    knobs = {"skin_um": (0, 20, 50, 100), "listed_blocks": (4, 5, 6)}
    best = {"skin_um": 50, "listed_blocks": 6}

    def cost():
        c = {k: _abi.tune_get(k) for k in knobs}
        return 1.0 + sum(abs(c[k] - best[k]) for k in knobs) / 100.0

    old = {k: _abi.tune_get(k) for k in knobs}
    try:
        r = autotune.tune_engine(Eng(1 << 20), 1e-5, knobs=knobs, label="test:cost", stat="mean", timer=cost)
        assert r["choice"] == best and r["ms"] == 1.0
        assert {k: _abi.tune_get(k) for k in knobs} == best
        assert autotune.table()["test:cost"] == best
        assert all("ms_mean" in t for t in r["table"])
        # skin 0 takes no list kernel: its register budget is not timed apart
        assert not any(t["knobs"]["skin_um"] == 0 and t["knobs"]["listed_blocks"] != 5 for t in r["table"])
    finally:
        for k, v in old.items():
            _abi.tune_set(k, v)
        autotune._TABLE.pop("test:cost", None)
