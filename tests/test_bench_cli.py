"""bench.py's command line and helpers (CPU): the options of the report
modes and the LES mode's learning-rate schedule."""
import importlib.util
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_cli", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_options(monkeypatch):
    b = load_bench()
    monkeypatch.setattr(sys, "argv", ["bench.py", "--shape", "3", "0", "--les-seeds", "3", "--lr-schedule", "step",
                                      "--workload", "les", "--train-iters", "20000"])
    a = b.parse()
    assert a.shape == [3, 0] and a.les_seeds == 3 and a.lr_schedule == "step" and a.workload == "les"
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = b.parse()
    assert a.shape is None and a.les_seeds == 1 and a.lr_schedule == "const" and a.N == 512


def test_lr_chunks():
    b = load_bench()
    assert b.lr_chunks(2000, "const") == [(2000, 1e-3)]
    ch = b.lr_chunks(20000, "step")
    assert ch == [(10000, 1e-3), (6000, 3e-4), (4000, 1e-4)]
    for n in (1, 7, 10, 101, 999):
        assert sum(it for it, _ in b.lr_chunks(n, "step")) == n
        assert all(it > 0 for it, _ in b.lr_chunks(n, "step"))


def test_traffic_table():
    """The committed ncu summary holds the dominant kernel's measured DRAM bytes per launch at
    the bench's sizes; the 512^3 figure lies between the kernel's written and its read+written
    compulsory bytes (3 and 9 fields of 512^2 x 176 stored kz rows, FP32 complex)."""
    b = load_bench()
    t512 = b.read_traffic("k_zline", 512, "fp32")
    assert t512 is not None and b.read_traffic("k_zline", 256, "fp32") is not None
    row = 512 * 512 * 176 * 8
    assert 3 * row < t512 <= 9 * row
    assert b.read_traffic("k_zline", 333, "fp32") is None
