"""Host logic of the decomposition tuner and the serving loop (no GPU)."""
import json

import numpy as np
import torch

from his_gb300 import autotune as A
from his_gb300 import workloads as W
from his_gb300.serving import estimate_bytes


def test_candidates_are_distinct_decompositions():
    shapes = [(81, 100)] * 4 + [(325, 400)]
    cands = A.candidates(shapes)
    assert (58, 16) in cands and len(cands) == len(set(cands))
    sigs = set()
    for tx, ty in cands:
        sig = []
        for ny, nx in sorted(set(shapes)):
            ns, nch = -(-nx // tx), -(-ny // ty)
            sig.append((-(-nx // ns), -(-ny // nch), A.strip_threads(tx)))
        sigs.add(tuple(sig))
    assert len(sigs) == len(cands)
    # a chunk height above every grid's row count collapses to one candidate per CTA width
    tall = A.candidates([(10, 30)])
    assert len(tall) == 4
    assert [A.strip_threads(tx) for tx in (58, 59, 122, 123, 218, 219, 346)] == [64, 128, 128, 224, 224, 352, 352]


def test_tune_cache_round_trip(tmp_path, monkeypatch):
    monkeypatch.setenv("HIS_GB300_TUNE_CACHE", str(tmp_path / "tiles.json"))
    A._store_file("dev|prec1|o2|81x100*4", (58, 24), {"58x24": 0.1, "58x48": 0.2})
    data = json.loads((tmp_path / "tiles.json").read_text())
    assert data["dev|prec1|o2|81x100*4"]["tile"] == [58, 24]
    assert A._load_file()["dev|prec1|o2|81x100*4"]["ms"]["58x48"] == 0.2


def test_footprint_estimate_covers_the_state():
    s = W.uneven_member("fp/0", 2, 3600.0)
    b32 = estimate_bytes(s, torch.float32)
    b64 = estimate_bytes(s, torch.float64)
    assert b32 >= 16 * s.cells * 4
    assert b64 > 1.9 * b32 - 1e6
    assert estimate_bytes(s, torch.float32, track_peaks=False) < b32


def test_request_stream_is_seeded():
    a = W.served_requests(2.0, 30.0, key="srv-test")
    b = W.served_requests(2.0, 30.0, key="srv-test")
    assert a == b and len(a) > 20
    t = np.array([x[0] for x in a])
    assert np.all(np.diff(t) > 0) and t[-1] <= 30.0
    assert {x[1] for x in a} <= {0, 1, 2}


def test_chain_split_matches_the_engine_rule():
    """Tiles per member follow his_grid_create's split (77 strip-chunks of a 400 x 325
    grid at 58 x 32), and chain bounds give every chain at least one member at the
    nearest tile shares."""
    from his_gb300.autotune import chain_bounds, tiles_per_member
    assert tiles_per_member([(325, 400)], (58, 32)) == [77]
    assert tiles_per_member([(81, 100), (163, 200)], (58, 48)) == [4, 16]
    counts = [77] * 64
    assert chain_bounds(counts, 8) == [0, 8, 16, 24, 32, 40, 48, 56, 64]
    assert chain_bounds(counts, 1) == [0, 64]
    uneven = [4] * 16 + [16] * 16 + [56] * 16
    b = chain_bounds(uneven, 4)
    assert b[0] == 0 and b[-1] == 48 and all(x < y for x, y in zip(b[:-1], b[1:]))
    tot = sum(uneven)
    shares = [sum(uneven[x:y]) for x, y in zip(b[:-1], b[1:])]
    assert max(shares) <= tot / 4 + 56
    assert chain_bounds([5, 1, 1], 3) == [0, 1, 2, 3]


def test_default_chain_rule_of_the_library():
    """his_engine_default_chains (called here without a GPU): one chain per 256
    strip-chunk tiles, at least 1, at most 8 and at most one per member."""
    from his_gb300 import _lib
    lib = _lib.load()
    rule = lib.his_engine_default_chains
    assert rule(64, 3136) == 8            # 64 x 400x325 in 58 x 48 tiles
    assert rule(64, 2368) == 8
    assert rule(6, 300) == 1              # a small served batch
    assert rule(2, 10000) == 2
    assert rule(100, 1000) == 3
    assert rule(1, 0) == 1
