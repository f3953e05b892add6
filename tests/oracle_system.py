"""Oracle-side global assembly and direct solve (test helper, CPU only).

Builds the reduced Stokes system the reference assembles -- BC dofs removed,
equations node-major and dof-minor (L/StgFEM/Discretisation/src/
FeEquationNumber.c:807-1091), element matrices scattered as in
__StiffnessMatrix_NewAssemble (L/StgFEM/SLE/SystemSetup/src/StiffnessMatrix.c:552-744)
-- from the oracle's element terms, and solves it with a sparse direct method.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def pic_points_by_element(tbl, cnt, ip_xi, ip_w):
    """Integration points per element in cell-table order."""
    out = []
    for e in range(len(cnt)):
        ps = tbl[e, : cnt[e]]
        out.append((ps, ip_xi[ps], ip_w[ps]))
    return out


def assemble(mesh, pts, eta_p, body_p, bc_mask, bc_val):
    """Full-dof K, G, f, h plus reduced-system index maps.

    pts: list per element of (particle ids, xi, w).  bc_mask/bc_val: [n_nodes*dim]."""
    dim, nen, npn = mesh.dim, mesh.nen, mesh.npn
    nv = mesh.n_nodes * dim
    ne = mesh.n_el
    Kr, Kc, Kv = [], [], []
    Gr, Gc, Gv = [], [], []
    f = np.zeros(nv)
    gxi, gw = mesh.gauss_points()
    Shat = np.zeros(ne) if npn == 1 else np.zeros((ne, npn, npn))
    for e in range(ne):
        nodes = mesh.element_nodes(e)
        dofs = (nodes[:, None] * dim + np.arange(dim)[None, :]).ravel()
        ps, xi, w = pts[e]
        Ke = mesh.element_K(e, xi, w, eta_p[ps])
        fe = mesh.element_f(e, xi, w, body_p[ps])
        Ge = mesh.element_G(e, gxi, gw)
        Se = mesh.element_S(Ke, Ge)
        if npn == 1:
            Shat[e] = Se[0, 0]
        else:
            Shat[e] = Se
        Kr.append(np.repeat(dofs, len(dofs))); Kc.append(np.tile(dofs, len(dofs))); Kv.append(Ke.ravel())
        Gr.append(np.repeat(dofs, npn)); Gc.append(np.tile(e * npn + np.arange(npn), len(dofs))); Gv.append(Ge.ravel())
        f[dofs] += fe
    K = sp.csr_matrix((np.concatenate(Kv), (np.concatenate(Kr), np.concatenate(Kc))), shape=(nv, nv))
    G = sp.csr_matrix((np.concatenate(Gv), (np.concatenate(Gr), np.concatenate(Gc))), shape=(nv, ne * npn))
    free = np.where(bc_mask == 0)[0]
    bcd = np.where(bc_mask != 0)[0]
    g = bc_val[bcd]
    f_l = f[free] - K[free][:, bcd] @ g
    h_l = -(G[bcd].T @ g)
    return dict(K=K, G=G, f=f, free=free, bcd=bcd, f_lift=f_l, h_lift=np.asarray(h_l).ravel(),
                Kff=K[free][:, free].tocsc(), Gf=G[free].tocsc(), Shat=Shat)


def solve(sysd, nv):
    """Direct solve of [[Kff, Gf], [Gf^T, 0]] with the pressure mean pinned.

    Returns full velocity (Dirichlet values filled by the caller) and pressure
    with zero mean."""
    Kff, Gf = sysd["Kff"], sysd["Gf"]
    nf, npr = Kff.shape[0], Gf.shape[1]
    ones = sp.csr_matrix(np.ones((1, npr)))
    A = sp.bmat([[Kff, Gf, None], [Gf.T, None, ones.T], [None, ones, None]], format="csc")
    rhs = np.concatenate([sysd["f_lift"], sysd["h_lift"], [0.0]])
    x = spla.spsolve(A, rhs)
    u = np.zeros(nv)
    u[sysd["free"]] = x[:nf]
    return u, x[nf: nf + npr]
