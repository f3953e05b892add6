"""uw.utils.Integral and mesh.integrate (P/utils/_utils.py:38-206,
P/mesh/_mesh.py:1200-1226): the reference's docstring answers and exact
integrals of polynomials the Gauss rules integrate exactly."""
import numpy as np
import pytest

import underworld2_gb300 as uw

fn = uw.function


def test_docstring_volume_and_surface():
    mesh = uw.mesh.FeMesh_Cartesian(minCoord=(0.0, 0.0), maxCoord=(1.0, 1.0))
    assert np.allclose(1.0, uw.utils.Integral(fn=1.0, mesh=mesh).evaluate(), rtol=1e-8)
    s = uw.utils.Integral(fn=1.0, mesh=mesh, integrationType="surface",
                          surfaceIndexSet=mesh.specialSets["AllWalls_VertexSet"])
    assert np.allclose(4.0, s.evaluate(), rtol=1e-8)


@pytest.mark.parametrize("et,res", [("Q1/dQ0", (5, 3)), ("Q2/dPc1", (2, 4)), ("Q1/dQ0", (2, 3, 2)),
                                    ("Q2/dPc1", (2, 1, 3))])
def test_exact_polynomial_integrals(et, res):
    dim = len(res)
    lo, hi = (-1.0, 0.5, 0.0)[:dim], (2.0, 1.5, 0.75)[:dim]
    m = uw.mesh.FeMesh_Cartesian(et, res, lo, hi)
    x = fn.coord()
    vol = np.prod([h - l for l, h in zip(lo, hi)])
    # x^2 y (degree 2 in x, 1 in y): exact on 3 and 5 points
    f = x[0] * x[0] * x[1]
    exact = (hi[0] ** 3 - lo[0] ** 3) / 3 * (hi[1] ** 2 - lo[1] ** 2) / 2 * (vol / ((hi[0] - lo[0]) * (hi[1] - lo[1])))
    assert abs(m.integrate(f)[0] - exact) < 1e-12 * abs(exact)
    # a vector function: one value per component
    v = uw.utils.Integral((1.0, x[0]) + ((x[2],) if dim == 3 else ()), mesh=m).evaluate()
    assert v.shape == (dim,)
    assert abs(v[0] - vol) < 1e-12 * vol
    assert abs(v[1] - vol * (lo[0] + hi[0]) / 2) < 1e-12 * vol
    # top wall: integral of x over y = max
    s = uw.utils.Integral(x[0], mesh=m, integrationType="surface",
                          surfaceIndexSet=m.specialSets["MaxJ_VertexSet"]).evaluate()
    area = vol / (hi[1] - lo[1])
    assert abs(s[0] - area * (lo[0] + hi[0]) / 2) < 1e-12 * area


def test_integral_argument_checks():
    m = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (4, 4), (0.0, 0.0), (1.0, 1.0))
    with pytest.raises(ValueError):
        uw.utils.Integral(1.0, mesh=None)
    with pytest.raises(ValueError):
        uw.utils.Integral(1.0, mesh=m, integrationType="line")
    with pytest.raises(RuntimeError):
        uw.utils.Integral(1.0, mesh=m, integrationType="surface")
    inner = uw.mesh.IndexSet(m.nodesGlobal, [12])
    with pytest.raises(ValueError):
        uw.utils.Integral(1.0, mesh=m, integrationType="surface", surfaceIndexSet=inner)


def test_gauss_integration_swarm():
    """uw.swarm.GaussIntegrationSwarm (P/swarm/_integration_swarm.py:155-200): 3 points
    per axis by default, 5 on Q2, 1..5 allowed; as an Integral's integrationSwarm
    (with integrationType=None, as the reference's convergence notebook uses it)
    its n-point rule integrates x^(2n-1) exactly and x^(2n) not."""
    import pytest
    m1 = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (3, 2), (0.0, 0.0), (1.0, 1.0))
    m2 = uw.mesh.FeMesh_Cartesian("Q2/dPc1", (3, 2), (0.0, 0.0), (1.0, 1.0))
    assert uw.swarm.GaussIntegrationSwarm(m1).particleCount == 3
    assert uw.swarm.GaussIntegrationSwarm(m2).particleCount == 5
    assert uw.swarm.GaussIntegrationSwarm(m1, 2).particleLocalCount == 6 * 4
    with pytest.raises(ValueError):
        uw.swarm.GaussIntegrationSwarm(m1, 6)
    with pytest.raises(ValueError):
        uw.swarm.GaussIntegrationSwarm(m1, 2.0)
    x = uw.function.input()[0]
    for n in (1, 2, 3, 4, 5):
        sw = uw.swarm.GaussIntegrationSwarm(m1, n)
        odd = uw.utils.Integral(x ** (2 * n - 1), m1, integrationSwarm=sw, integrationType=None).evaluate()[0]
        assert abs(odd - 1.0 / (2 * n)) < 1e-14
        even = uw.utils.Integral(x ** (2 * n), m1, integrationSwarm=sw, integrationType=None).evaluate()[0]
        assert abs(even - 1.0 / (2 * n + 1)) > 1e-13
    with pytest.raises(RuntimeError):
        uw.utils.Integral(1.0, m1, integrationSwarm=uw.swarm.GaussIntegrationSwarm(m1))
