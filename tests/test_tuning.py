"""The autotuner cache (ec2d/tuning.py) without a GPU: a stand-in solver with
the binding's launch_signature / launch_config / set_launch_config /
autotune methods, whose setter takes the ranges ec2d_set_launch_config takes.
A stored signature is applied without timing; any other signature, a
refresh, an unreadable file or an entry the setter rejects runs the
autotuner and stores its result."""
import json
import os

import pytest

from ec2d import tuning

KEYS = ("lusgs_cs", "rows", "lanes", "concurrent", "tile_residual")
DEFAULT = {"lusgs_cs": 0, "rows": 12, "lanes": 0, "concurrent": 1, "tile_residual": 0}


class StandIn:
    def __init__(self, sig, tuned, ms=0.9):
        self.sig, self.tuned, self.ms = sig, dict(tuned), ms
        self.cfg = dict(DEFAULT)
        self.autotune_calls = 0

    def launch_signature(self):
        return self.sig

    def launch_config(self):
        return dict(self.cfg)

    def set_launch_config(self, cfg):
        v = {k: int(cfg[k]) for k in KEYS}
        if not (0 <= v["lusgs_cs"] <= 8 and 4 <= v["rows"] <= 32 and v["lanes"] in (0, 4, 8)
                and v["concurrent"] in (0, 1) and v["tile_residual"] in (0, 1)):
            raise RuntimeError("ec2d_set_launch_config: invalid argument or call order")
        self.cfg = v

    def autotune(self, trial_steps=5):
        self.autotune_calls += 1
        self.cfg = dict(self.tuned)
        return self.cfg["lusgs_cs"], self.cfg["rows"], self.cfg["concurrent"], self.ms


SIG_A = "ec2d-launch-1 lib=10000 build=0123 dev=GB300 sm=103 sms=152 L1:nv4,96x96*2"
SIG_B = SIG_A.replace("96x96*2", "128x128*4")
TUNED = {"lusgs_cs": 0, "rows": 8, "lanes": 8, "concurrent": 0, "tile_residual": 1}


def test_miss_tunes_and_stores_then_hit_applies(tmp_path):
    path = str(tmp_path / "cache.json")
    a = StandIn(SIG_A, TUNED, ms=0.87)
    r = tuning.autotune_cached(a, path, trial_steps=3)
    assert r["source"] == "autotune" and r["config"] == TUNED and a.autotune_calls == 1
    doc = json.load(open(path))
    assert doc["format"] == tuning.FORMAT
    (e,) = doc["entries"].values()
    assert e["signature"] == SIG_A and e["config"] == TUNED and e["trial_steps"] == 3 and e["ms_per_step"] == 0.87
    b = StandIn(SIG_A, {"lusgs_cs": 1, "rows": 32, "lanes": 0, "concurrent": 1, "tile_residual": 0})
    r = tuning.autotune_cached(b, path)
    assert r["source"] == "cache" and b.autotune_calls == 0
    assert b.launch_config() == TUNED and r["ms_per_step"] == 0.87


def test_other_signature_refresh_and_env(tmp_path, monkeypatch):
    path = str(tmp_path / "sub" / "cache.json")
    tuning.autotune_cached(StandIn(SIG_A, TUNED), path)
    c = StandIn(SIG_B, DEFAULT)
    assert tuning.autotune_cached(c, path)["source"] == "autotune" and c.autotune_calls == 1
    assert len(json.load(open(path))["entries"]) == 2
    d = StandIn(SIG_A, DEFAULT)
    assert tuning.autotune_cached(d, path, refresh=True)["source"] == "autotune" and d.autotune_calls == 1
    assert tuning.lookup(path, SIG_A)["config"] == DEFAULT
    monkeypatch.setenv(tuning.ENV, path)
    e = StandIn(SIG_B, TUNED)
    assert tuning.autotune_cached(e)["source"] == "cache" and e.autotune_calls == 0


def test_no_path_tunes_and_writes_nothing(tmp_path, monkeypatch):
    monkeypatch.delenv(tuning.ENV, raising=False)
    monkeypatch.chdir(tmp_path)
    a = StandIn(SIG_A, TUNED)
    assert tuning.autotune_cached(a)["source"] == "autotune" and a.autotune_calls == 1
    assert os.listdir(tmp_path) == []


def test_unreadable_or_foreign_file_is_replaced(tmp_path):
    path = str(tmp_path / "cache.json")
    for text in ("{not json", json.dumps({"format": "something-else", "entries": {}})):
        with open(path, "w") as fh:
            fh.write(text)
        a = StandIn(SIG_A, TUNED)
        with pytest.warns(UserWarning):
            assert tuning.autotune_cached(a, path)["source"] == "autotune"
        assert tuning.lookup(path, SIG_A)["config"] == TUNED
    assert [f for f in os.listdir(tmp_path) if f != "cache.json"] == []  # no temporary file left


def test_rejected_entry_falls_back_to_the_autotuner(tmp_path):
    path = str(tmp_path / "cache.json")
    tuning.store(path, SIG_A, dict(TUNED, rows=99), 1.0, 5)
    a = StandIn(SIG_A, TUNED)
    with pytest.warns(UserWarning):
        r = tuning.autotune_cached(a, path)
    assert r["source"] == "autotune" and a.cfg == TUNED
    assert tuning.lookup(path, SIG_A)["config"] == TUNED


def test_key_collision_is_not_a_hit(tmp_path):
    """An entry is used only for its own signature, not for another that
    happened to land on the same key."""
    path = str(tmp_path / "cache.json")
    tuning.store(path, SIG_A, TUNED, 1.0, 5)
    doc = json.load(open(path))
    doc["entries"][tuning.signature_key(SIG_B)] = doc["entries"].pop(tuning.signature_key(SIG_A))
    json.dump(doc, open(path, "w"))
    assert tuning.lookup(path, SIG_B) is None
