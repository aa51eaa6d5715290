"""A small measuring autotuner.

``tune(key, candidates, measure)`` times every candidate configuration with the
caller's ``measure(candidate) -> milliseconds`` (best of ``repeats``), skips
candidates whose measurement raises (a kernel that rejects a shape, a failed
launch), keeps the fastest and caches the choice in a JSON file under a key
built from size buckets (``bucket(...)``), so later runs with similar shapes
reuse it without measuring.
"""
import json
import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_CACHE = os.path.join(HERE, "_build", "autotune.json")


def cache_path():
    return os.environ.get("ORBKIT_GB300_TUNE_CACHE", DEFAULT_CACHE)


def bucket(**dims):
    """Key from power-of-two buckets of each (non-negative integer) dimension."""
    parts = []
    for k in sorted(dims):
        v = int(dims[k])
        parts.append("%s%d" % (k, 0 if v <= 0 else int(math.log2(v))))
    return "-".join(parts)


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, data):
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    tmp = path + ".tmp%d" % os.getpid()
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


class TuneError(RuntimeError):
    pass


def tune(key, candidates, measure, repeats=2, use_cache=True, path=None):
    """Returns (best candidate, report).  report: list of (candidate, ms or None, error)."""
    path = path or cache_path()
    candidates = [dict(c) for c in candidates]
    if not candidates:
        raise TuneError("autotune: no candidates for %s" % key)
    if use_cache:
        hit = _load(path).get(key)
        if hit is not None and hit in candidates:
            return hit, [(hit, None, "cached")]
    report = []
    for c in candidates:
        try:
            ms = min(float(measure(c)) for _ in range(max(1, repeats)))
            if not math.isfinite(ms) or ms <= 0:
                raise ValueError("non-positive time %r" % ms)
            report.append((c, ms, None))
        except Exception as e:  # a rejected or failed candidate is skipped
            report.append((c, None, "%s: %s" % (type(e).__name__, e)))
    ok = [(ms, i) for i, (c, ms, err) in enumerate(report) if ms is not None]
    if not ok:
        raise TuneError("autotune: every candidate failed for %s: %s" % (key, [r[2] for r in report]))
    best = report[min(ok)[1]][0]
    if use_cache:
        data = _load(path)
        data[key] = best
        _store(path, data)
    return best, report
