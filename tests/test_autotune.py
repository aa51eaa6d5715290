"""The autotuner on the CPU with a fake measurement: the fastest candidate wins,
failing candidates (forced errors) are skipped, all-failing raises, the cache is used."""
import pytest

from orbkit_gb300 import autotune


def test_picks_fastest_and_caches(tmp_path):
    path = str(tmp_path / "tune.json")
    cands = [{"n": 32, "g": 1}, {"n": 64, "g": 1}, {"n": 64, "g": 4}]
    calls = []

    def measure(c):
        calls.append(c)
        return {32: 5.0, 64: 3.0}[c["n"]] + 0.1 * c["g"]

    best, rep = autotune.tune("k", cands, measure, repeats=2, path=path)
    assert best == {"n": 64, "g": 1} and len(calls) == 6
    best2, rep2 = autotune.tune("k", cands, lambda c: 1 / 0, path=path)
    assert best2 == best and rep2[0][2] == "cached"


def test_failing_candidates_are_skipped(tmp_path):
    def measure(c):
        if c["n"] == 64:
            raise RuntimeError("forced failure: shape rejected")
        return 2.0

    best, rep = autotune.tune("k2", [{"n": 64}, {"n": 32}], measure, path=str(tmp_path / "t.json"))
    assert best == {"n": 32}
    assert any(err and "forced failure" in err for _, _, err in rep)


def test_all_failing_raises(tmp_path):
    with pytest.raises(autotune.TuneError):
        autotune.tune("k3", [{"n": 1}, {"n": 2}], lambda c: float("nan"), path=str(tmp_path / "t.json"))


def test_bucket_keys():
    assert autotune.bucket(nmol=256, pts=2 ** 27) == autotune.bucket(pts=2 ** 27 + 5, nmol=300)
    assert autotune.bucket(nmol=1) != autotune.bucket(nmol=2)
