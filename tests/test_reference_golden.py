"""The oracle against fixtures made by the reference's own code
(tests/golden/ref_N16.npz, written by tests/golden/make_ref_golden.py from
Solver/src/solver.c compiled unchanged against oracle/ref_shim). These run
where the reference sources are absent; tests/test_reference_parity.py calls
the reference directly where they are present. Bar: 1e-12 relative L2."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_N16.npz")
TOL = 1e-12


def rel(a, b):
    n = np.linalg.norm(np.ravel(b))
    return float(np.linalg.norm(np.ravel(a - b)) / (n if n > 0 else 1.0))


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def test_rhs_matches_reference(oracle, gold):
    o = oracle.Oracle(16, nu=0.01, bugcompat_dealias=True)
    assert rel(o.rhs(gold["uh"]), gold["rhs"]) <= TOL


@pytest.mark.parametrize("key,visc_pow", [("rk4cn3", 1), ("rk4cn3_hyper", 2)])
def test_rk4step_matches_reference(oracle, gold, key, visc_pow):
    o = oracle.Oracle(16, nu=0.02, dt=2e-3, integrator=oracle.RK4CN, visc_pow=visc_pow, bugcompat_dealias=True)
    o.set_state(gold["uh"])
    o.step(3)
    assert rel(o.get_state(), gold[key]) <= TOL


def test_measurables_match_reference(oracle, gold):
    ob = oracle.Oracle(16, nu=0.01, bugcompat_measures=True)
    of = oracle.Oracle(16, nu=0.01)
    ob.set_state(gold["uh"])
    of.set_state(gold["uh"])
    assert rel(ob.measurables()[0], gold["tot"]) <= TOL
    tf, Ek, Ok = of.measurables()
    assert rel(Ek, gold["Ek"]) <= TOL and rel(Ok, gold["Ok"]) <= TOL
    assert abs(tf[0] - gold["Ek"].sum()) <= TOL * tf[0]
    oh = oracle.Oracle(16, nu=0.01, visc_pow=2, bugcompat_measures=True)
    oh.set_state(gold["uh"])
    assert rel(oh.measurables()[0], gold["tot_hyper"]) <= TOL


def test_random_ic_matches_reference(oracle, gold):
    o = oracle.Oracle(16, nu=0.01, bugcompat_dealias=True)
    o.ic("RANDOM")
    assert rel(o.get_state(), gold["random_ic"]) <= TOL
