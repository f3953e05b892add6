"""Dirichlet and Neumann conditions (``uw.conditions``, P/conditions/_conditions.py:18-170)."""
import numpy as np


class SystemCondition:
    """A condition on the dofs of a MeshVariable: one IndexSet (or None) of
    nodes per dof (P/conditions/_conditions.py:18-60)."""

    def __init__(self, variable, indexSetsPerDof):
        from .container import IndexSet
        from .mesh import MeshVariable
        if not isinstance(variable, MeshVariable):
            raise TypeError("Provided variable must be of class 'MeshVariable'.")
        self._variable = variable
        if isinstance(indexSetsPerDof, IndexSet):
            sets = (indexSetsPerDof,)
        elif isinstance(indexSetsPerDof, (list, tuple)):
            sets = tuple(indexSetsPerDof)
        else:
            raise TypeError("You must provide the required 'indexSetsPerDof' item\n"
                            "as a list or tuple of 'IndexSet' items.")
        for s in sets:
            if not isinstance(s, (IndexSet, type(None))):
                raise TypeError("Provided list must only contain objects of 'NoneType' or type 'IndexSet'.")
        if variable.nodeDofCount != len(sets):
            raise ValueError("Provided variable has a nodeDofCount of {}, however you have ".format(variable.nodeDofCount)
                             + "provided {} index set(s). You must provide an index set for each degree ".format(len(sets))
                             + "of freedom of your variable, but no more.")
        self._indexSets = sets

    @property
    def indexSetsPerDof(self):
        return self._indexSets

    @property
    def variable(self):
        return self._variable

    def mask(self):
        """[n_nodes, dofs] uint8: 1 where a dof is in its set."""
        n, k = self.variable.data.shape
        m = np.zeros((n, k), np.uint8)
        for d, s in enumerate(self._indexSets):
            if s is not None:
                m[s.data.astype(np.int64), d] = 1
        return m


class DirichletCondition(SystemCondition):
    """Fix the dofs of ``variable`` on the node sets given per dof; the fixed
    values are the variable's current ``data`` at those nodes (as
    FeVariable_SetBC reads them) (P/conditions/_conditions.py:63-101)."""

    def __init__(self, variable, indexSetsPerDof):
        super().__init__(variable, indexSetsPerDof)


class NeumannCondition(SystemCondition):
    """A flux (traction, for a velocity field) ``fn_flux`` on the nodes given
    per dof of ``variable`` (P/conditions/_conditions.py:104-170).  The systems
    add its surface integral to their right-hand side: Gauss points on the
    element faces whose nodes all lie in the sets, weight times surface
    Jacobian times flux times the shape function of each flagged dof."""

    def __init__(self, variable, indexSetsPerDof=None, fn_flux=None):
        super().__init__(variable, indexSetsPerDof)
        from . import function as _fn
        f = _fn.Function.convert(fn_flux)
        if not isinstance(f, _fn.Function):
            raise TypeError("Provided 'fn_flux' must be of or convertible to 'Function' class.")
        self._fn_flux = f

    @property
    def fn_flux(self):
        """The Function that gives the flux."""
        return self._fn_flux

    @fn_flux.setter
    def fn_flux(self, fn):
        from . import function as _fn
        f = _fn.Function.convert(fn)
        if not isinstance(f, _fn.Function):
            raise ValueError("Provided '_fn' must be of or convertible to 'Function' class.")
        self._fn_flux = f
