"""Dirichlet conditions (``uw.conditions`` subset, P/conditions/_conditions.py:63)."""
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
    def __init__(self, *args, **kwargs):
        raise NotImplementedError("Neumann conditions are not part of the GPU PIC Stokes path")
