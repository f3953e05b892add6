"""CPU restatement of the reference's Neumann (flux / traction) surface term
(TEST INFRASTRUCTURE: the checker of the package's surface integral, never the
product).

VectorSurfaceAssemblyTerm_NA__Fn__ni (L/Underworld/Utils/src/
VectorSurfaceAssemblyTerm_NA__Fn__ni.cpp:163-236) on a GaussBorderIntegrationSwarm
(L/StgDomain/Swarm/src/GaussBorderParticleLayout.c:186-320): for every element
with a condition dof, for every Gauss point on each of its 2*dim faces (faces
0, 1 at y = -1, +1; 2, 3 at x = -1, +1; 4, 5 at z = -1, +1), the flux function
masked by the interpolated node indicator (> 0.999,
P/systems/sle/_assemblyterm.py:129-144) times the point weight times the
surface Jacobian (ElementType.c:566-606) is added to N_A times each flagged dof
(A, d) of the element.  Plain Python loops over a regular mesh.
"""
import itertools

import numpy as np

_FACE_AXIS = (1, 1, 0, 0, 2, 2)


def _basis(order, s):
    if order == 1:
        return [(1 - s) / 2, (1 + s) / 2]
    return [0.5 * s * (s - 1), 1 - s * s, 0.5 * s * (s + 1)]


def surface_term(axes, order, cond_mask, flux, n_gauss):
    """axes: per-axis node coordinates (length res*order+1); cond_mask[n_nodes,
    ndof] (bool); flux(x) -> sequence of ndof values at a global point.
    Returns the term as [n_nodes * ndof]."""
    dim = len(axes)
    nn = [len(a) for a in axes]
    res = [(n - 1) // order for n in nn]
    ndof = cond_mask.shape[1]
    out = np.zeros(int(np.prod(nn)) * ndof)
    node_on = cond_mask.any(1)
    x1, w1 = np.polynomial.legendre.leggauss(n_gauss)
    k = order + 1
    for e_idx in itertools.product(*[range(r) for r in reversed(res)]):
        e_idx = e_idx[::-1]                      # x fastest
        nodes, coords = [], []
        for loc in itertools.product(*[range(k)] * dim):
            loc = loc[::-1]
            g = [e_idx[d] * order + loc[d] for d in range(dim)]
            n = g[0] + nn[0] * g[1] + (nn[0] * nn[1] * g[2] if dim == 3 else 0)
            nodes.append(n)
            coords.append([axes[d][g[d]] for d in range(dim)])
        if not any(node_on[n] for n in nodes):
            continue
        h = [axes[d][(e_idx[d] + 1) * order] - axes[d][e_idx[d] * order] for d in range(dim)]
        for f in range(2 * dim):
            kax = _FACE_AXIS[f]
            others = [a for a in range(dim) if a != kax]
            for gi in itertools.product(range(n_gauss), repeat=dim - 1):
                xi = [0.0] * dim
                xi[kax] = -1.0 if f % 2 == 0 else 1.0
                w = 1.0
                for a, i in zip(others, gi):
                    xi[a] = x1[i]
                    w *= w1[i]
                jac = 1.0
                for a in others:
                    jac *= h[a] / 2.0
                B = [_basis(order, xi[d]) for d in range(dim)]
                N = []
                for loc in itertools.product(*[range(k)] * dim):
                    loc = loc[::-1]
                    v = 1.0
                    for d in range(dim):
                        v *= B[d][loc[d]]
                    N.append(v)
                delta = sum(N[a] * (1.0 if node_on[nodes[a]] else 0.0) for a in range(len(nodes)))
                if not delta > 0.999:
                    continue
                x = [sum(N[a] * coords[a][d] for a in range(len(nodes))) for d in range(dim)]
                q = flux(np.array(x))
                for a in range(len(nodes)):
                    for d in range(ndof):
                        if cond_mask[nodes[a], d]:
                            out[nodes[a] * ndof + d] += w * jac * q[d] * N[a]
    return out
