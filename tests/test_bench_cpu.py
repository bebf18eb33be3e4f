"""Host logic of the benchmark (CPU only): the served workload's request
trace has the stated op mix, popularity skew and offsets (reads and greps
at any byte, writes 16-byte aligned), writes go to
disjoint regions of the output files, the byte accounting clamps at end of
file, the max-over-ranks helper is the identity on one rank, the reference
arm (a CPU path) prints the contract's JSON line, and the nvidia-smi clock
samples reduce to the median SM clock, the maximum and the active throttle
reasons."""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402
import gpufs_gb300 as g  # noqa: E402


def _trace(n_files=2000, n_req=20000, n_out=8, seed=1):
    rng = np.random.default_rng(seed)
    sizes = [int(x) for x in rng.integers(4096, 4 << 20, n_files)]
    return sizes, bench._served_trace(sizes, n_req, n_out, np.random.default_rng(seed + 1))


def test_served_trace_op_mix_and_alignment():
    sizes, reqs = _trace()
    ops = reqs["op"]
    mix = [float(np.mean(ops == op)) for op in (g.SV_READ, g.SV_GREP, g.SV_WRITE)]
    assert abs(mix[0] - 0.80) < 0.02 and abs(mix[1] - 0.15) < 0.02 and abs(mix[2] - 0.05) < 0.01
    rd = reqs[ops != g.SV_WRITE]
    sz = np.asarray(sizes, dtype=np.uint64)
    assert np.all(rd["offset"] <= sz[rd["file"]])
    # offsets fall on any byte: every residue mod 16 appears, most are unaligned
    assert len(np.unique(rd["offset"] % 16)) == 16
    assert float(np.mean(rd["offset"] % 4096 == 0)) < 0.01
    lengths = reqs["length"].astype(np.float64)
    assert lengths.min() >= 4096 and lengths.max() <= 16 << 20
    # log-uniform lengths: the median sits near the geometric mean of the range
    assert abs(np.log(np.median(lengths)) - 0.5 * (np.log(4096) + np.log(16 << 20))) < 0.2


def test_served_trace_popularity_is_skewed():
    sizes, reqs = _trace()
    rd = reqs[reqs["op"] != g.SV_WRITE]
    counts = np.sort(np.bincount(rd["file"], minlength=len(sizes)))[::-1]
    # Zipf(0.9) over 2000 files: the top 1 % of files draw a large share
    assert counts[:20].sum() > 0.15 * counts.sum()
    assert counts[0] > 10 * max(1, int(np.median(counts)))


def test_served_writes_are_disjoint_and_aligned():
    _, reqs = _trace()
    wr = reqs[reqs["op"] == g.SV_WRITE]
    assert np.all(wr["offset"] % 16 == 0)
    for f in np.unique(wr["file"]):
        w = np.sort(wr[wr["file"] == f], order="offset")
        ends = w["offset"] + w["length"]
        assert np.all(ends[:-1] <= w["offset"][1:])


def test_served_bytes_clamp_at_end_of_file():
    sizes = [10000, 5000]
    reqs = np.zeros(4, dtype=g.SERVE_REQ)
    reqs[0] = (g.SV_READ, 0, 8192, 100000, 0)   # clamps to 1808
    reqs[1] = (g.SV_GREP, 1, 0, 1000, 0)       # 1000
    reqs[2] = (g.SV_READ, 1, 8192, 4096, 0)    # past the end: 0
    reqs[3] = (g.SV_WRITE, 0, 0, 777, 0)       # writes count their length
    assert bench._served_bytes(reqs, sizes) == 1808 + 1000 + 0 + 777


def test_allmax_single_rank():
    assert bench.allmax(None, 3.5) == 3.5


def test_reference_arm_prints_the_contract_line(built, tmp_path, monkeypatch, capsys):
    from gpufs_gb300 import datagen

    def small_corpus(d, total=None):
        return datagen.grep_corpus(str(tmp_path / "c"), bench.N_FILES, bench.N_FILES * (40 << 10), n_vocab=2000,
                                   n_dict=300, seed=9)

    monkeypatch.setattr(bench, "make_data", small_corpus)

    class Args:
        steps, warmup, gpus = 2, 3, 1

    bench.run_reference(Args(), 0, 1, None, str(tmp_path))
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e", "gpu_launches"):
        assert k in line, k
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == "GB/s"
    assert line["value"] > 0 and line["steps"] == 2 and line["warmup"] == 3 and line["higher_is_better"] is True
    assert line["config"]["sample_bytes"] == bench.N_FILES * (32 << 10)
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert line["gpu_launches"] == 0



class _DoneProc:
    def poll(self):
        return 0

    def terminate(self):
        pass

    def kill(self):
        pass

    def wait(self, timeout=None):
        return 0


def test_clock_samples_give_median_max_and_active_reasons():
    c = bench.Clocks(0)
    c.f.write("0, 2070, 2070, 812.1, 0x0, Not Active, Not Active, Not Active, Not Active\n"
              "0, 1965, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active\n"
              "0, 2025, 2070, 1210.7, 0x0, Not Active, Not Active, Not Active, Not Active\n"
              "0, [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A]\n"
              "garbage line\n")
    c.p = _DoneProc()
    got = c.stop()
    assert got == {"sm_mhz": 2025.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 4}
    assert not os.path.exists(c.f.name)


def test_clock_reasons_name_thermal_and_hw_slowdowns():
    c = bench.Clocks(0)
    c.f.write("0, 1500, 2070, 900, 0x48, Active, Not Active, Active, Not Active\n")
    c.p = _DoneProc()
    assert c.stop()["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]


def test_hist_quantiles_take_bucket_upper_edges():
    h = np.zeros(64, dtype=np.uint64)
    h[10] = 50   # [1024, 2048) ns
    h[20] = 49   # [~1.05 ms, ~2.1 ms)
    h[30] = 1
    q = bench._hist_quantiles(h, (50, 99, 99.9))
    assert q["p50"] == 2048 / 1e3
    assert q["p99"] == 2 ** 21 / 1e3
    assert q["p99.9"] == 2 ** 31 / 1e3
    assert bench._hist_quantiles(np.zeros(64, dtype=np.uint64), (50,)) is None
