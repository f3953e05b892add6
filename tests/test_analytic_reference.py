"""uw.function.analytic against the reference's own solution code (CPU).

Every solution, at its defaults and at one other parameter set
(tests/golden/analytic_cases.py), is compared field by field with

* the committed fixture tests/golden/analytic_fields.npz, made by
  tests/golden/make_analytic_golden.py from the reference's C and C++ solution
  classes compiled from the reference tree (L/Underworld/Function/src/
  AnalyticSol*.hpp, L/Underworld/SysTest/AnalyticPlugins/Velic_sol*/sol*.c);
* the same compiled code live, at fresh points, where the reference tree is
  present (oracle/ref_analytic.py), skipped elsewhere.

The solutions here are derived independently (module _analytic_series: a
layered mode solve; closed forms for SolM, SolNL, SolDB2d, SolDB3d); the
tolerance is 1e-11 of each field's largest magnitude.
"""
import os
import sys

import numpy as np
import pytest

from underworld2_gb300 import function as fn

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
from analytic_cases import CASES, FIELDS  # noqa: E402

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "analytic_fields.npz"))
RTOL = 1e-11

_objs = {}


def _sol(i):
    if i not in _objs:
        name, _, kw, _ = CASES[i]
        _objs[i] = getattr(fn.analytic, name)(**kw)
    return _objs[i]


def _check(sol, x, ref, label):
    for f in FIELDS:
        mine = getattr(sol, "fn_" + f).evaluate(x)
        scale = max(np.abs(ref[f]).max(), 1e-300)
        err = np.abs(mine - ref[f]).max() / scale
        assert err < RTOL, "%s %s: %.3e" % (label, f, err)


@pytest.mark.parametrize("i", range(len(CASES)), ids=["%s-%d" % (c[0], i) for i, c in enumerate(CASES)])
def test_matches_reference_fixture(i):
    x = GOLD["%d/points" % i]
    _check(_sol(i), x, {f: GOLD["%d/%s" % (i, f)] for f in FIELDS}, CASES[i][0])


@pytest.mark.parametrize("i", range(len(CASES)), ids=["%s-%d" % (c[0], i) for i, c in enumerate(CASES)])
def test_matches_reference_live(i):
    from oracle import ref_analytic
    if not ref_analytic.available():
        pytest.skip("reference tree not present")
    name, prm, _, dim = CASES[i]
    x = np.random.default_rng(i).uniform(0.0, 1.0, (200 if dim == 2 else 40, dim))
    _check(_sol(i), x, ref_analytic.evaluate(name, prm, x), name)


def test_solution_discovery():
    """The reference's convergence notebook finds the solutions as the
    subclasses of fn.analytic._SolBase."""
    found = sorted(n for n in dir(fn.analytic) if not n.startswith("_")
                   and isinstance(getattr(fn.analytic, n), type)
                   and issubclass(getattr(fn.analytic, n), fn.analytic._SolBase))
    assert found == sorted({c[0] for c in CASES})
    assert fn.analytic.SolNL().nonlinear and not fn.analytic.SolCx().nonlinear


def test_parameter_checks():
    """The reference's argument checks (P/function/analytic.py)."""
    with pytest.raises(TypeError):
        fn.analytic.SolA(n_x=2.5)
    with pytest.raises(TypeError):
        fn.analytic.SolB(n_x=2, n_z=2.)
    with pytest.raises(TypeError):
        fn.analytic.SolCx(eta_B=10)
    with pytest.raises(TypeError):
        fn.analytic.SolKz(sigma_0=2.)
    with pytest.raises(TypeError):
        fn.analytic.SolM(n_z=4, m_x=4.)
    with pytest.raises(ValueError):
        fn.analytic.SolCx(x_c=1.5)
