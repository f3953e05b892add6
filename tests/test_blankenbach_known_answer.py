"""Known answers of the reference's Blankenbach convection benchmark notebook
(docs/examples/03_BlankenbachBenchmark.ipynb, case "a", Ra = 1e4), from the
steady-state temperature field the reference ships as an HDF5 file written by
h5py/libhdf5 (docs/examples/input/03_BlankenbachBenchmark/tempfield_inp_64_Ra1e4.h5).

The file is read by the package's own HDF5 reader through MeshVariable.load (a
64 x 64 Q1 field; the root group holds the dataset as a hard link and the mesh
file as an external link).  As the notebook does, the field is interpolated
onto a 128 x 128 Q1/dQ0 mesh, then: Stokes with unit viscosity and buoyancy
Ra T z on free-slip walls, one SUPG step at get_max_dt(), Stokes again (Nu and
v_rms), a second SUPG step (q1, q2), and the topography of the top surface
from the last Stokes solution (sigma_zz = 2 dw/dz - p minus its mean, scaled by
eta0 kappa / h^2 / (rho g)).  Discretisation and solves are the oracle's
(tests/oracle_system.py, oracle/advdiff.py); the notebook's tolerances apply:
1e-2 for Nu, v_rms, q1, q2 and 1e-3 for the topography at both top corners and
the x position of its zero.  Both SUPG steps are also held to the reference's
own run as the notebook's saved output prints it (Nu before the loop to 6
decimals, v_rms to 3, the relative Nu change of the first step to 4
significant digits, q1 and q2 after the second step to 3 decimals).  The test reads the reference tree and is skipped where
it is absent.
"""
import os

import numpy as np
import pytest

import oracle
from oracle.ref_analytic import REFERENCE_TREE
from oracle import advdiff
from tests import analytic_convergence as ac
from tests import oracle_system as osys
import underworld2_gb300 as uw

INPUT = os.path.join(REFERENCE_TREE, "docs", "examples", "input",
                     "03_BlankenbachBenchmark")

pytestmark = pytest.mark.skipif(not os.path.isdir(INPUT), reason="reference tree not present")


def _bilinear(t64, res):
    """Values of the 64 x 64 Q1 field [65, 65] (z rows, x columns) at the nodes of a res x res mesh."""
    x = np.linspace(0.0, 1.0, res + 1) * 64
    i0 = np.minimum(x.astype(int), 63)
    a = x - i0
    rows = (1 - a)[:, None] * t64[i0] + a[:, None] * t64[i0 + 1]           # interpolate in z
    return (1 - a)[None, :] * rows[:, i0] + a[None, :] * rows[:, i0 + 1]   # then in x


@pytest.mark.parametrize("case", ["1e4", "1e5", "1e6"])
def test_reference_files_load(case):
    """All three shipped fields read: 65 x 65 nodal values, 1 on the bottom, 0 on the top."""
    mesh = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (64, 64), (0.0, 0.0), (1.0, 1.0))
    T = mesh.add_variable(1)
    T.load(os.path.join(INPUT, "tempfield_inp_64_Ra%s.h5" % case))
    t = T.data[:, 0].reshape(65, 65)
    assert np.all(t[0] == 1.0) and np.all(t[-1] == 0.0)
    assert t.min() >= 0.0 and t.max() <= 1.0 and 0.3 < t.mean() < 0.7
    f = uw.h5.File(os.path.join(INPUT, "tempfield_inp_64_Ra%s.h5" % case))
    assert f.links["mesh"][0].endswith(".h5")


def test_blankenbach_case_a():
    res, Ra = 128, 1.0e4
    mesh64 = uw.mesh.FeMesh_Cartesian("Q1/dQ0", (64, 64), (0.0, 0.0), (1.0, 1.0))
    T64 = mesh64.add_variable(1)
    T64.load(os.path.join(INPUT, "tempfield_inp_64_Ra1e4.h5"))
    T = _bilinear(T64.data[:, 0].reshape(65, 65), res)
    T[0, :], T[-1, :] = 1.0, 0.0
    T = T.ravel()

    m = oracle.Mesh(2, 1, (res, res), (0.0, 0.0), (1.0, 1.0))
    rule = ac._Rule(m, 2)
    nq = len(rule.w)
    X = m.node_coords()[:, :2]
    mask = np.zeros(m.n_nodes * 2, np.uint8)
    for d in range(2):
        mask[np.flatnonzero(np.isclose(X[:, d], 0.0) | np.isclose(X[:, d], 1.0)) * 2 + d] = 1
    zero = np.zeros(m.n_nodes * 2)
    pts = [(e * nq + np.arange(nq), rule.xi, rule.w) for e in range(m.n_el)]
    tbc = np.isclose(X[:, 1], 0.0) | np.isclose(X[:, 1], 1.0)
    kq = np.ones((m.n_el, 9))

    def stokes(Tn):
        body = np.zeros((m.n_el * nq, 2))
        body[:, 1] = Ra * np.einsum("qn,en->eq", rule.N, Tn[rule.nodes]).ravel()
        sysd = osys.assemble(m, pts, np.ones(m.n_el * nq), body, mask, zero)
        return osys.solve(sysd, m.n_nodes * 2)

    Tdot = np.zeros(m.n_nodes)                         # the notebook's temperatureDotField, kept across steps

    def supg(u, Tn):
        nonlocal Tdot
        U = u.reshape(-1, 2)
        dt = advdiff.max_dt(m, U, kq)
        Tn2, Tdot = advdiff.step(m, dt, U, kq, None, tbc, Tn.copy(), None, Tn.copy(), Tdot)
        return Tn2

    h = 1.0 / res
    rule3 = ac._Rule(m, 3)

    def nusselt(Tn):
        Tg = Tn.reshape(res + 1, res + 1)
        dTdz = (Tg[-1] - Tg[-2]) / h                  # top row: linear in x along each element
        return -np.sum(0.5 * (dTdz[1:] + dTdz[:-1]) * h) / np.sum(0.5 * (Tg[0, 1:] + Tg[0, :-1]) * h)

    def v_rms(u):
        uq = np.einsum("qn,eni->eqi", rule3.N, u.reshape(-1, 2)[rule3.nodes]).reshape(-1, 2)
        return np.sqrt(np.tile(rule3.w * rule3.det, m.n_el) @ (uq ** 2).sum(1))

    nu0 = nusselt(T)
    u, p = stokes(T)
    vrms0 = v_rms(u)
    T = supg(u, T)
    u, p = stokes(T)
    nu, vrms = nusselt(T), v_rms(u)
    # the notebook's asserted values (the published benchmark), at its tolerances
    assert np.isclose(nu, 4.884, rtol=1e-2), nu
    assert np.isclose(vrms, 42.865, rtol=1e-2), vrms
    # the reference's own run, as the notebook's saved output prints it:
    # "Nusselt number = 4.856902" before the loop, then v_rms = 42.869 at steps
    # 0 and 1 and a relative Nu change of 1.416e-03 over the first SUPG step
    assert abs(nu0 - 4.856902) <= 5e-7, nu0
    assert round(vrms0, 3) == 42.869 and round(vrms, 3) == 42.869, (vrms0, vrms)
    assert abs(abs(nu - nu0) / nu - 1.416e-3) <= 5e-7, (nu - nu0) / nu

    Tg = supg(u, T).reshape(res + 1, res + 1)
    dTdz = (Tg[-1] - Tg[-2]) / h
    assert np.isclose(-dTdz[0], 8.020, rtol=1e-2), -dTdz[0]
    assert np.isclose(-dTdz[-1], 0.589, rtol=1e-2), -dTdz[-1]
    # the saved output of the reference's run: "q1 = 8.021; q2 = 0.589"
    assert round(-dTdz[0], 3) == 8.021 and round(-dTdz[-1], 3) == 0.589, (-dTdz[0], -dTdz[-1])

    W = u.reshape(res + 1, res + 1, 2)[..., 1]
    dwdz = (W[-1] - W[-2]) / h                        # at the top nodes, per top element linear in x
    ptop = p.reshape(res, res)[-1]
    mean = -np.sum((dwdz[1:] + dwdz[:-1]) * h - ptop * h)          # int of -sigma_zz over the top
    sig = np.array([2.0 * dwdz[i] - ptop[min(i, res - 1)] for i in range(res + 1)])   # owning element: floor(x / h)
    topo = (-sig - mean) * (1e23 * 1e-6 / 1e12) / (4e3 * 10.0)
    x0 = np.linspace(0.0, 1.0, res + 1)[np.argmin(np.abs(topo))]
    assert np.isclose(topo[0], 2254.02, rtol=1e-3), topo[0]
    assert np.isclose(topo[-1], -2903.23, rtol=1e-3), topo[-1]
    assert np.isclose(x0, 0.539372, rtol=1e-3), x0
