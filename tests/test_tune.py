"""The tuning table (rawspec_gb300_tune_lookup, tune.c) and the tuner's
table writer, on the host: no CUDA call is made."""
import os
import sys
from pathlib import Path

import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))

from rawspec_gb300 import api, tune  # noqa: E402

TABLE = """# tuning table
1024 8 1 dft=cuda ctas=8   # trailing comment
1048576 8 1 lag=3 ring=6
1048576 8 1 lag=4 ring=9
256 8 4 dft=tc
65536 16 1 ctas=2
this is not an entry
8 8 1 lag=3 ring=2
8 8 1 ctas=0
8 8 1 speed=fast
"""


@pytest.fixture
def table(tmp_path, monkeypatch):
    p = tmp_path / "t.tune"
    p.write_text(TABLE)
    monkeypatch.setenv("RAWSPEC_GB300_TUNE_FILE", str(p))
    return p


def test_entries_are_found_and_the_last_one_wins(table):
    r, t = api.tune_lookup(1024, 8, 1)
    assert r == 1 and (t.dft, t.ctas, t.lag, t.ring) == (0, 8, 0, 0)
    r, t = api.tune_lookup(1048576, 8, 1)
    assert r == 1 and (t.dft, t.ctas, t.lag, t.ring) == (-1, 0, 4, 9)
    r, t = api.tune_lookup(256, 8, 4)
    assert r == 1 and t.dft == 1
    r, t = api.tune_lookup(65536, 16, 1)
    assert r == 1 and t.ctas == 2


def test_keys_are_exact(table):
    for key in [(1024, 8, 4), (1024, 16, 1), (2048, 8, 1), (65536, 8, 1)]:
        r, t = api.tune_lookup(*key)
        assert r == 0 and (t.dft, t.ctas, t.lag, t.ring) == (-1, 0, 0, 0)


def test_malformed_entries_are_skipped(table, capfd):
    # a ring not longer than the lag, a zero CTA count and an unknown key
    r, t = api.tune_lookup(8, 8, 1)
    assert r == 0 and (t.dft, t.ctas, t.lag, t.ring) == (-1, 0, 0, 0)
    err = capfd.readouterr().err
    assert err.count("malformed entry skipped") == 4


def test_no_table_and_unreadable_table(tmp_path, monkeypatch):
    monkeypatch.delenv("RAWSPEC_GB300_TUNE_FILE", raising=False)
    assert api.tune_lookup(1024, 8, 1)[0] == 0
    monkeypatch.setenv("RAWSPEC_GB300_TUNE_FILE", str(tmp_path / "missing.tune"))
    assert api.tune_lookup(1024, 8, 1)[0] == -1


def test_tuner_writes_what_the_library_reads(tmp_path, monkeypatch):
    p = tmp_path / "out.tune"
    entries = {(1048576, 8, 1): {"lag": 5, "ring": 10}, (8, 8, 1): {"dft": "cuda", "ctas": 16},
               (1024, 8, 1): {}}
    tune.write_table(str(p), entries, ["a comment"])
    text = p.read_text()
    assert text.startswith("# a comment\n") and "1024 8 1" not in text
    monkeypatch.setenv("RAWSPEC_GB300_TUNE_FILE", str(p))
    r, t = api.tune_lookup(1048576, 8, 1)
    assert r == 1 and (t.lag, t.ring) == (5, 10)
    r, t = api.tune_lookup(8, 8, 1)
    assert r == 1 and (t.dft, t.ctas) == (0, 16)


def test_candidates_follow_the_kernel():
    assert {"dft": "tc"} in tune.candidates("small") and {"dft": "cuda", "ctas": 4} in tune.candidates("tc")
    assert all(c["ring"] > c["lag"] for c in tune.candidates("large_fused"))
    assert all(set(c) == {"ctas"} for c in tune.candidates("large_a"))


class FakeCase:
    """Stands in for the GPU: the time of a buffer is a function of the table."""

    def __init__(self, prods, keys, kinds, cost):
        self.prods, self.keys, self.kinds, self.cost = prods, keys, kinds, cost
        self.calls = 0

    def run(self, table, path):
        self.calls += 1
        kinds = list(self.kinds)
        for i, key in enumerate(self.keys):
            if table.get(key, {}).get("dft") == "cuda":
                kinds[i] = "small"
            elif table.get(key, {}).get("dft") == "tc" and self.kinds[i] == "tc":
                kinds[i] = "tc"
        return self.cost(table), kinds


class Args:
    passes, rounds, min_gain = 1, 2, 0.02


def test_tuner_keeps_a_candidate_only_past_the_threshold():
    keys = [(1048576, 8, 1), (1024, 8, 1)]

    def cost(table):
        t = 1.0
        t += {2: 0.3, 3: 0.05, 4: 0.0, 5: -0.05, 6: -0.01}.get(table.get(keys[0], {}).get("lag", 4), 0.0)
        c = table.get(keys[1], {})
        t += 0.05 if c.get("dft") == "cuda" else 0.0
        t -= 0.01 if c.get("ctas") == 16 else 0.0   # 1 %: below the 2 % threshold
        return t

    case = FakeCase([(1048576, 51, 1), (1024, 3072, 1)], keys, ["large_fused", "tc"], cost)
    table, notes = tune.tune(Args(), log=lambda m: None, case=case)
    assert table == {keys[0]: {"lag": 5, "ring": 10}}
    assert notes[0].startswith("library defaults") and notes[-1].startswith("tuned:")
    # every setting twice (the current one included), plus the first and last runs
    assert case.calls == 2 + 2 * (1 + 5) + 2 * (1 + 6)


def test_tuner_skips_tensor_cores_where_the_library_has_none():
    keys = [(512, 8, -4)]
    case = FakeCase([(512, 64, -4)], keys, ["small"], lambda table: 0.9 if table.get(keys[0], {}).get("dft") == "tc"
                    else 1.0)
    table, notes = tune.tune(Args(), log=lambda m: None, case=case)
    assert table == {} and not any("dft=tc" in n for n in notes)
