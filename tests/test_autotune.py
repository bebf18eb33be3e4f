"""The autotuner picks the fastest candidate, skips failing ones, and
returns a cached choice for a known workload signature without trials."""
import pytest

from gpufs_gb300 import autotune


def test_picks_fastest_and_skips_failures(tmp_path):
    calls = []

    def trial(cfg):
        calls.append(cfg["page"])
        if cfg["page"] == 19:
            raise RuntimeError("out of frames")
        return {16: 0.5, 18: 0.2, 19: 0.0, 21: 0.3}[cfg["page"]]

    cands = [{"page": p} for p in (16, 18, 19, 21)]
    best, res = autotune.tune(cands, trial)
    assert best == {"page": 18}
    assert [c["page"] for c, _ in res] == [16, 18, 19, 21]
    assert dict((c["page"], t) for c, t in res)[19] is None


def test_cache_by_signature(tmp_path):
    path = str(tmp_path / "tune.json")
    key = autotune.signature(files=4096, op="grep+xxh64", device="GB300")
    n = [0]

    def trial(cfg):
        n[0] += 1
        return 1.0 / cfg["page"]

    cands = [{"page": p} for p in (18, 20, 21)]
    best, res = autotune.tune(cands, trial, key=key, cache_path=path)
    assert best == {"page": 21} and n[0] == 3 and len(res) == 3
    best2, res2 = autotune.tune(cands, trial, key=key, cache_path=path)
    assert best2 == best and res2 == [] and n[0] == 3
    # another workload is tuned afresh
    best3, _ = autotune.tune(cands, trial, key=autotune.signature(files=1), cache_path=path)
    assert n[0] == 6 and best3 == best


def test_all_failing_raises():
    with pytest.raises(RuntimeError):
        autotune.tune([{"a": 1}], lambda c: (_ for _ in ()).throw(OSError("x")))
