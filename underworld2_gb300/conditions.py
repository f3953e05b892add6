"""Dirichlet and Neumann conditions (``uw.conditions`` subset, P/conditions/_conditions.py:63-170)."""
import numpy as np


class SystemCondition:
    pass


class DirichletCondition(SystemCondition):
    """Fix the dofs of ``variable`` on the node sets given per dof; the fixed
    values are the variable's current ``data`` at those nodes (as
    FeVariable_SetBC reads them)."""

    def __init__(self, variable, indexSetsPerDof):
        self.variable = variable
        if not isinstance(indexSetsPerDof, (list, tuple)):
            indexSetsPerDof = (indexSetsPerDof,)
        if len(indexSetsPerDof) != variable.nodeDofCount:
            raise ValueError("indexSetsPerDof needs one entry (or None) per dof of the variable")
        self.indexSetsPerDof = tuple(indexSetsPerDof)

    def mask(self):
        n, k = variable_shape = self.variable.data.shape
        m = np.zeros((n, k), np.uint8)
        for d, s in enumerate(self.indexSetsPerDof):
            if s is None:
                continue
            idx = s.data if hasattr(s, "data") else np.asarray(list(s), np.int64)
            m[idx, d] = 1
        return m


class NeumannCondition(SystemCondition):
    """A flux (traction, for a velocity field) ``fn_flux`` on the nodes given
    per dof of ``variable`` (P/conditions/_conditions.py:109-170).  The systems
    add its surface integral to their right-hand side: Gauss points on the
    element faces whose nodes all lie in the sets, weight times surface
    Jacobian times flux times the shape function of each flagged dof."""

    def __init__(self, variable, indexSetsPerDof=None, fn_flux=None):
        from . import function as _fn
        from .mesh import MeshVariable
        if not isinstance(variable, MeshVariable):
            raise TypeError("Provided 'variable' must be of 'MeshVariable' class.")
        self.variable = variable
        if indexSetsPerDof is None:
            raise ValueError("'indexSetsPerDof' must be provided")
        if not isinstance(indexSetsPerDof, (list, tuple)):
            indexSetsPerDof = (indexSetsPerDof,)
        if len(indexSetsPerDof) != variable.nodeDofCount:
            raise ValueError("indexSetsPerDof needs one entry (or None) per dof of the variable")
        self.indexSetsPerDof = tuple(indexSetsPerDof)
        f = _fn.Function.convert(fn_flux)
        if not isinstance(f, _fn.Function):
            raise ValueError("Provided 'fn_flux' must be of or convertible to 'Function' class.")
        self.fn_flux = f

    def mask(self):
        return DirichletCondition.mask(self)
