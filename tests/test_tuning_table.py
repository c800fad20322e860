"""CPU tests of the autotuner's table (ns3d_tuning_set / get / save / load / clear
and NS3D_TUNING_FILE): host logic only, no GPU. The GPU tests in test_autotune.py
time the shapes and check that engines built afterwards use the chosen one."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def shape(ns3d, N):
    t = ns3d.tuning(N)
    return None if t is None else (t["variant"], t["zform"])


def test_set_save_clear_load_round_trip(ns3d, tmp_path):
    ns3d.tuning_clear()
    assert ns3d.tuning(512) is None
    ns3d.tuning_set(512, 3, 0)
    ns3d.tuning_set(256, 6, 1)
    assert shape(ns3d, 512) == (3, 0) and shape(ns3d, 256) == (6, 1)
    assert ns3d.tuning(512, "fp64") is None   # keyed by (N, precision)
    f = tmp_path / "table.txt"
    ns3d.tuning_save(f)
    ns3d.tuning_clear()
    assert ns3d.tuning(512) is None and ns3d.tuning(256) is None
    ns3d.tuning_load(f)
    assert shape(ns3d, 512) == (3, 0) and shape(ns3d, 256) == (6, 1)
    ns3d.tuning_clear()


def test_rejects_unknown_shapes(ns3d, tmp_path):
    ns3d.tuning_clear()
    with pytest.raises(ns3d.NS3DError):
        ns3d.tuning_set(64, 99, 0)     # no such tile variant
    with pytest.raises(ns3d.NS3DError):
        ns3d.tuning_set(64, 0, 3)      # no such z-pass form
    ns3d.tuning_set(64, 0, 2)          # the tensor-core z pass
    assert shape(ns3d, 64) == (0, 2)
    ns3d.tuning_clear()
    f = tmp_path / "mixed.txt"
    f.write_text("# N precision variant zform ms\n64 1 2 0 0.5\n96 1 42 0 0.5\n128 1 1 7 0.1\nnot a line\n")
    with pytest.raises(ns3d.NS3DError):
        ns3d.tuning_load(f)            # the invalid lines are reported ...
    assert shape(ns3d, 64) == (2, 0)   # ... and the valid ones kept
    assert ns3d.tuning(96) is None and ns3d.tuning(128) is None
    ns3d.tuning_clear()


def test_shipped_table_through_the_environment():
    """NS3D_TUNING_FILE names a table loaded before the first lookup of a process;
    the shipped GB300 table parses and holds the 512^3 and 1024^3 choices."""
    path = os.path.join(ROOT, "3d_navier_stokes_gb300", "tuning", "gb300.txt")
    code = ("import importlib, sys; sys.path.insert(0, %r); "
            "m = importlib.import_module('3d_navier_stokes_gb300'); "
            "print(*[m.tuning(n)['variant'] for n in (256, 512, 1024)])" % ROOT)
    r = subprocess.run([sys.executable, "-c", code], env=dict(os.environ, NS3D_TUNING_FILE=path),
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.split() == ["6", "3", "3"]
