"""Autotuner table and its use by the batched path (host logic, no GPU)."""
import json

from tapkee_gb300 import autotune, batch


def test_search_space_is_the_full_product():
    cands = list(autotune.candidates())
    keys = {json.dumps(c, sort_keys=True) for c in cands}
    n = 1
    for v in autotune.SPACE.values():
        n *= len(v)
    assert len(cands) == len(keys) == n
    for c in cands:
        assert c["screen_qt"][0] in autotune.SPACE["screen_qt0"] and c["screen_qt"][1] == 1
        assert c["lle_warps"] in autotune.SPACE["lle_warps"]
        assert c["wide_lists"] in autotune.SPACE["wide_lists"]


def test_committed_table_names_its_best_candidate():
    with open(batch.TUNING_PATH) as f:
        table = json.load(f)
    best = table["best"]
    assert json.dumps(best, sort_keys=True) in {json.dumps(c, sort_keys=True) for c in autotune.candidates()}
    # the best entry is the one with the smallest median time, and every candidate was timed
    assert len(table["results"]) == len(list(autotune.candidates()))
    fastest = min(table["results"], key=lambda r: r["ms_median"])
    assert fastest["tuning"] == best and abs(fastest["ms_median"] - table["best_ms"]) < 1e-9


def test_default_tuning_reads_the_table(tmp_path, monkeypatch):
    from tapkee_gb300 import build as tkbuild
    tkbuild.build()
    with open(batch.TUNING_PATH) as f:
        best = json.load(f)["best"]
    assert batch.default_tuning() == best
    # without a table (or with an unreadable one) the library defaults apply
    monkeypatch.setattr(batch, "TUNING_PATH", str(tmp_path / "missing.json"))
    lib_default = batch.default_tuning()
    assert lib_default == {"screen_qt": [2, 1], "lle_warps": 8, "wide_lists": 0}
    bad = tmp_path / "bad.json"
    bad.write_text("{not json")
    monkeypatch.setattr(batch, "TUNING_PATH", str(bad))
    assert batch.default_tuning() == lib_default
    # unknown keys in a table are ignored
    extra = tmp_path / "extra.json"
    extra.write_text(json.dumps({"best": {"lle_warps": 4, "bogus": 1}}))
    monkeypatch.setattr(batch, "TUNING_PATH", str(extra))
    assert batch.default_tuning() == dict(lib_default, lle_warps=4)
    # the ctypes struct carries every field
    s = batch._tuning_struct(best)
    assert [s.screen_qt[0], s.screen_qt[1], s.lle_warps, s.wide_lists] == \
        [best["screen_qt"][0], best["screen_qt"][1], best["lle_warps"], best["wide_lists"]]
