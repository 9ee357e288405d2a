"""The column-tile autotuner's selection and caching logic (CPU, fake timer).

The timings are injected, so no GPU is needed: the tuner must pick the
fastest shape, measure a shape only once, keep the choice across instances
through its JSON cache, key by device, mesh, scheme, grids and particle-count
bucket, and not measure a mesh size that has a single shape.
"""
import json

from gbpowspec.tune import Tuner

SHAPES = {64: [(4, 4), (8, 4)], 256: [(8, 4), (4, 4), (8, 8)], 1024: [(4, 4)]}


class FakeTimer:
    def __init__(self, ms):
        self.ms, self.calls = ms, []

    def __call__(self, N, mas, interlace, n, tiles, device):
        self.calls.append((N, mas, interlace, n, tiles))
        return self.ms[(N, tiles)] / 1e3


def _tuner(path, timer, dev="GB300"):
    return Tuner(path=str(path), timer=timer, variants=lambda N: SHAPES[N], device_name=lambda d: dev)


def test_picks_the_fastest_and_caches(tmp_path):
    cache = tmp_path / "tiles.json"
    t = FakeTimer({(256, (8, 4)): 1.0, (256, (4, 4)): 0.7, (256, (8, 8)): 0.9})
    tu = _tuner(cache, t)
    assert tu.best(256, "tsc", True, n=2_000_000) == (4, 4)
    assert len(t.calls) == 3 and tu.timings == 1
    assert tu.best(256, "tsc", True, n=2_100_000) == (4, 4)          # same bucket: no new timing
    assert len(t.calls) == 3
    rec = json.loads(cache.read_text())
    (key, val), = rec.items()
    assert key.startswith("GB300|N256|tsc|G2|n2^")
    assert val["tiles"] == [4, 4] and set(val["ms"]) == {"8x4", "4x4", "8x8"}
    # another process (a new instance) reads the choice back without timing
    t2 = FakeTimer({})
    assert _tuner(cache, t2).best(256, "tsc", True, n=2_000_000) == (4, 4)
    assert t2.calls == []


def test_keys_separate_shapes_and_devices(tmp_path):
    cache = tmp_path / "tiles.json"
    t = FakeTimer({(64, (4, 4)): 2.0, (64, (8, 4)): 1.0, (256, (8, 4)): 1.0, (256, (4, 4)): 2.0,
                   (256, (8, 8)): 3.0})
    tu = _tuner(cache, t)
    assert tu.best(64, "cic", True, n=100_000) == (8, 4)
    assert tu.best(64, "cic", False, n=100_000) == (8, 4)            # other grid count: timed again
    assert tu.best(64, "tsc", True, n=100_000) == (8, 4)             # other scheme
    assert tu.best(64, "cic", True, n=1_000_000) == (8, 4)           # other particle bucket
    assert tu.best(256, "cic", True, n=100_000) == (8, 4)
    assert tu.timings == 5
    other = FakeTimer({(64, (4, 4)): 1.0, (64, (8, 4)): 2.0})
    assert _tuner(cache, other, dev="other GPU").best(64, "cic", True, n=100_000) == (4, 4)
    assert len(other.calls) == 2


def test_single_shape_is_not_timed_and_ties_keep_library_order(tmp_path):
    t = FakeTimer({(64, (4, 4)): 1.0, (64, (8, 4)): 1.0})
    tu = _tuner(tmp_path / "c.json", t)
    assert tu.best(1024, "pcs", True, n=16_000_000) == (4, 4)
    assert t.calls == []
    assert tu.best(64, "ngp", False, n=10) == (4, 4)                 # a tie: the default (listed first)


def test_unwritable_cache_keeps_choices_in_memory(tmp_path):
    blocker = tmp_path / "file"
    blocker.write_text("x")
    t = FakeTimer({(64, (4, 4)): 2.0, (64, (8, 4)): 1.0})
    tu = _tuner(blocker / "sub" / "tiles.json", t)                   # a path under a regular file
    assert tu.best(64, "cic", True, n=5000) == (8, 4)
    assert tu.best(64, "cic", True, n=5000) == (8, 4)
    assert len(t.calls) == 2


def test_library_lists_tile_shapes():
    from gbpowspec import _native
    assert _native.tile_variants(512)[0] == (8, 4)
    assert (4, 4) in _native.tile_variants(512)
    assert _native.tile_variants(1024) == [(4, 4)]
    assert _native.tile_variants(96) == []
