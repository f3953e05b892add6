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


def assemble(mesh, pts, eta_p, body_p, bc_mask, bc_val, lam_p=None, src_p=None):
    """Full-dof K, G, f, h plus reduced-system index maps.

    pts: list per element of (particle ids, xi, w).  bc_mask/bc_val: [n_nodes*dim].
    lam_p: per-particle 1/lambda; the pressure block C = M(-1/lambda)
    (MatrixAssemblyTerm_NA__NB__Fn with fn = -fn_one_on_lambda, P/systems/_stokes.py:147-151,298-307).
    src_p: per-particle continuity source, added to h (P/systems/_stokes.py:284-288)."""
    dim, nen, npn = mesh.dim, mesh.nen, mesh.npn
    nv = mesh.n_nodes * dim
    ne = mesh.n_el
    Kr, Kc, Kv = [], [], []
    Gr, Gc, Gv = [], [], []
    Cr, Cc, Cv = [], [], []
    f = np.zeros(nv)
    h = np.zeros(ne * npn)
    gxi, gw = mesh.gauss_points()
    Shat = np.zeros(ne) if npn == 1 else np.zeros((ne, npn, npn))
    for e in range(ne):
        nodes = mesh.element_nodes(e)
        dofs = (nodes[:, None] * dim + np.arange(dim)[None, :]).ravel()
        pd = e * npn + np.arange(npn)
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
        Gr.append(np.repeat(dofs, npn)); Gc.append(np.tile(pd, len(dofs))); Gv.append(Ge.ravel())
        f[dofs] += fe
        if lam_p is not None:
            Me = mesh.element_M(e, xi, w, -lam_p[ps])
            Cr.append(np.repeat(pd, npn)); Cc.append(np.tile(pd, npn)); Cv.append(Me.ravel())
        if src_p is not None:
            h[pd] += mesh.element_h(e, xi, w, src_p[ps])
    K = sp.csr_matrix((np.concatenate(Kv), (np.concatenate(Kr), np.concatenate(Kc))), shape=(nv, nv))
    G = sp.csr_matrix((np.concatenate(Gv), (np.concatenate(Gr), np.concatenate(Gc))), shape=(nv, ne * npn))
    C = None
    if lam_p is not None:
        C = sp.csr_matrix((np.concatenate(Cv), (np.concatenate(Cr), np.concatenate(Cc))), shape=(ne * npn, ne * npn))
    free = np.where(bc_mask == 0)[0]
    bcd = np.where(bc_mask != 0)[0]
    g = bc_val[bcd]
    f_l = f[free] - K[free][:, bcd] @ g
    h_l = h - (G[bcd].T @ g)
    return dict(K=K, G=G, C=C, f=f, free=free, bcd=bcd, f_lift=f_l, h_lift=np.asarray(h_l).ravel(),
                Kff=K[free][:, free].tocsc(), Gf=G[free].tocsc(), Shat=Shat)


def checkerboard_vectors(res, npn=1):
    """Indicator vectors of the even cells (i+j+k even) and of the odd cells
    (KSPBuildPressure_CB_Nullspace_BSSCR, ksp_pressure_nullspace.c:28-80)."""
    idx = np.indices(tuple(res[::-1])).sum(axis=0).ravel()   # cells numbered x fastest
    even = (idx % 2 == 0).astype(float)
    return [np.repeat(even, npn), np.repeat(1.0 - even, npn)]


def solve(sysd, nv, null_vectors=None):
    """Direct solve of [[Kff, Gf], [Gf^T, C]].

    Incompressible (C is None): the components of h along each null vector are
    projected out, as KSPRemovePressureNullspace_BSSCR does for h^ (default null
    vector: the constant).  One pressure dof per null vector is pinned to zero
    (a dense constraint row would fill the LU factors), and the null vectors
    (mutually orthogonal) are projected out of the solution afterwards.  Sparse
    LU (COLAMD ordering) plus two steps of iterative refinement.  Returns full
    velocity (Dirichlet values filled by the caller) and pressure."""
    Kff, Gf = sysd["Kff"], sysd["Gf"]
    nf, npr = Kff.shape[0], Gf.shape[1]
    h = sysd["h_lift"].copy()
    keep = np.arange(npr)
    if sysd.get("C") is not None:
        A = sp.bmat([[Kff, Gf], [Gf.T, sysd["C"]]], format="csc")
    else:
        if null_vectors is None:
            null_vectors = [np.ones(npr)]
        pinned = []
        for t in null_vectors:
            h -= (t @ h) / (t @ t) * t
            pinned.append(next(i for i in np.flatnonzero(t) if i not in pinned))
        keep = np.setdiff1d(keep, pinned)
        Gk = Gf[:, keep]
        A = sp.bmat([[Kff, Gk], [Gk.T, None]], format="csc")
    rhs = np.concatenate([sysd["f_lift"], h[keep]])
    lu = spla.splu(A, permc_spec="COLAMD")
    x = lu.solve(rhs)
    for _ in range(2):
        x += lu.solve(rhs - A @ x)
    u = np.zeros(nv)
    u[sysd["free"]] = x[:nf]
    p = np.zeros(npr)
    p[keep] = x[nf:]
    for t in (null_vectors if sysd.get("C") is None else []):
        p -= (t @ p) / (t @ t) * t
    return u, p
