"""Host-side logic of the trajectory autotuner (no GPU): the candidate set,
workload signatures and the result cache."""
import json

from qsim_gb300 import autotune as AT


def test_candidates_cover_every_mode():
    c = AT.candidates(24)
    assert {x["max_fused_size"] for x in c} == {3, 4}
    assert {x["tc_from"] for x in c} == {0, 20, 22, 24}
    assert not any(x["tc_from"] for x in AT.candidates(24, forms=((4, False),)))
    assert any(x["split"] == 0 for x in c)          # stream path only
    assert any(x["split"] == 24 for x in c)         # all in the packed kernel
    assert any(0 < x["split"] < 24 for x in c)      # split, both at once
    for x in c:
        if x["split"]:
            assert x["ctas_per_sm"] >= 1 and x["tile_kib"] in (32, 64, 96)
    # Splits at or above the largest circuit collapse into "all packed".
    assert all(x["split"] in (0, 14) for x in AT.candidates(14))


def test_runners_follow_the_split():
    made = {}

    def make(f, tensor):
        return made.setdefault((f, tensor), [(f, tensor, i) for i in range(4)])
    cfg = dict(max_fused_size=3, tensor=False, tc_from=22, split=16,
               ctas_per_sm=1, tile_kib=32)
    rs = AT.runners_for(make, [12, 16, 20, 24], cfg)
    assert rs == [(4, False, 0), (4, False, 1), (3, False, 2), (6, True, 3)]


def test_signature_depends_on_workload_only():
    a = AT.signature([12, 13, 24], 32, "noise")
    assert a == AT.signature([24, 12, 13], 32, "noise")
    assert a != AT.signature([12, 13, 24], 16, "noise")
    assert a != AT.signature([12, 13, 24], 32, "other")


def test_cache_round_trip(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("QSG_AUTOTUNE_CACHE", str(path))
    assert AT._load() == {}
    AT._store({"k": {"best": {"split": 0}, "table": []}})
    assert json.loads(path.read_text())["k"]["best"] == {"split": 0}
    assert AT._load()["k"]["table"] == []
