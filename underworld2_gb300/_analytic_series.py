"""Free-slip analytic Stokes solutions of the reference's ``uw.function.analytic``
(P/function/analytic.py:113-565), derived here from their problem statements.

Each solution is a box [0, 1]^d with free-slip walls, a viscosity that varies in
one coordinate s only (constant, exponential, or piecewise constant) and a body
force that is a single Fourier mode, or a cosine series, in the other
coordinates t.  For one mode with wavenumber k the fields separate as

    v_s = a(s) cos(k t),   v_t = b(s) sin(k t),   p = P(s) cos(k t),
    sigma_ss = S(s) cos(k t),   sigma_st = T(s) sin(k t),

and the Stokes equations (-div(2 eta e) + grad p = f, div v = 0) become the
first-order system

    a' = -k b,             b' = k a + T/eta,
    S' = -k T - F_s,       T' = k S + 4 eta k^2 b - F_t,

with f_s = F_s(s) cos(k t) and f_t = F_t(s) sin(k t).  For eta = eta_0 exp(2 B s)
(B = 0 on a constant layer) the scaled tractions S/eta, T/eta make it constant-
coefficient, and a(s) satisfies

    a'''' + 4B a''' + (4B^2 - 2k^2) a'' - 4Bk^2 a' + k^2 (k^2 + 4B^2) a
        = k (G_t' + 2B G_t + k G_s),   G = F/eta.

Homogeneous solutions are exp(lambda s) (s exp(lambda s) for the double roots
+-k when B = 0), each anchored at the end of its layer where it is largest so
that no basis function exceeds one in magnitude; forcing terms C exp(nu s) give
particular solutions by undetermined coefficients.  Free slip (a = T = 0) at
s = 0 and s = 1, and continuity of a, b, S, T across each viscosity interface,
fix the four coefficients per layer (a complex linear solve at construction).
Evaluation runs in torch on the points' device, chunked over points.
"""
import numpy as np
import torch

from .function import Function, _SolBase, constant, input, math as _fmath, branching as _branching

_PI = np.pi


# ---------------------------------------------------------------------------
# one Fourier mode in a layered box
# ---------------------------------------------------------------------------
def _roots(k, B):
    """Characteristic roots and multiplicity indices (1 marks s exp(lambda s))."""
    if B == 0.0:
        return np.array([k, k, -k, -k], dtype=complex), np.array([0, 1, 0, 1])
    c = [1.0, 4.0 * B, 4.0 * B * B - 2.0 * k * k, -4.0 * B * k * k, k * k * (k * k + 4.0 * B * B)]
    r = np.roots(c).astype(complex)
    r = r[np.argsort(r.real)]
    sep = min(abs(r[i] - r[j]) for i in range(4) for j in range(i + 1, 4))
    if sep < 1e-7 * (abs(k) + abs(B)):
        raise ValueError("viscosity parameter too close to zero for the exponential-viscosity solution")
    return r, np.zeros(4, dtype=int)


def _charpoly(lam, k, B):
    return lam ** 4 + 4 * B * lam ** 3 + (4 * B * B - 2 * k * k) * lam ** 2 - 4 * B * k * k * lam \
        + k * k * (k * k + 4 * B * B)


def _derivs(lam, m, sig, e):
    """d^i/ds^i of sig^m exp(lam sig), i = 0..3, given e = exp(lam sig)."""
    return [e * (lam ** i * sig ** m + m * i * lam ** max(i - 1, 0)) for i in range(4)]


def _state(d, k, B, eta, gt):
    """(a, b, S, T) from the derivatives of a (S, T unscaled tractions)."""
    a = d[0]
    b = -d[1] / k
    Tt = -d[2] / k - k * d[0]
    Ttp = -d[3] / k - k * d[1]
    St = (Ttp + 2.0 * B * Tt - 4.0 * k * k * b + gt) / k
    return a, b, eta * St, eta * Tt


class _Mode:
    """Coefficients of one mode: k, layers (lo, hi, eta0, B), forcing terms
    F_s = sum Cs exp(nu s), F_t = sum Ct exp(nu s) as lists of (C, nu)."""

    def __init__(self, k, layers, fs_terms=(), ft_terms=()):
        self.k = float(k)
        self.layers = [tuple(float(v) for v in L) for L in layers]
        nl = len(self.layers)
        self.lam, self.mult, self.s0 = [], [], []
        self.part = []         # per layer: list of (A, g_t, rho) with a_p = A e^{rho s}, G_t = g_t e^{rho s}
        for lo, hi, eta0, B in self.layers:
            lam, mult = _roots(self.k, B)
            self.lam.append(lam)
            self.mult.append(mult)
            self.s0.append(np.where(lam.real > 0, hi, lo))
            terms = []
            for C, nu in fs_terms:
                rho = complex(nu) - 2.0 * B
                P = _charpoly(rho, self.k, B)
                if abs(P) < 1e-12 * max(1.0, abs(rho)) ** 4:
                    raise ValueError("body-force wavenumber resonates with the flow mode")
                terms.append((self.k * self.k * C / eta0 / P, 0.0, rho))
            for C, nu in ft_terms:
                rho = complex(nu) - 2.0 * B
                P = _charpoly(rho, self.k, B)
                if abs(P) < 1e-12 * max(1.0, abs(rho)) ** 4:
                    raise ValueError("body-force wavenumber resonates with the flow mode")
                g = C / eta0
                terms.append((self.k * (rho + 2.0 * B) * g / P, g, rho))
            self.part.append(terms)
        # boundary and interface conditions
        M = np.zeros((4 * nl, 4 * nl), dtype=complex)
        rhs = np.zeros(4 * nl, dtype=complex)

        def quantities(L, s):
            lo, hi, eta0, B = self.layers[L]
            eta = eta0 * np.exp(2.0 * B * s)
            hom = []
            for j in range(4):
                sig = s - self.s0[L][j]
                e = np.exp(self.lam[L][j] * sig)
                hom.append(_state(_derivs(self.lam[L][j], self.mult[L][j], sig, e), self.k, B, eta, 0.0))
            pa = [0.0, 0.0, 0.0, 0.0]
            for A, g, rho in self.part[L]:
                e = np.exp(rho * s)
                st = _state([A * rho ** i * e for i in range(4)], self.k, B, eta, g * e)
                pa = [x + y for x, y in zip(pa, st)]
            return np.array(hom).T, np.array(pa)     # [4 quantities, 4 basis], [4]

        row = 0
        H, p = quantities(0, self.layers[0][0])
        for q in (0, 3):
            M[row, 0:4] = H[q]
            rhs[row] = -p[q]
            row += 1
        for L in range(nl - 1):
            s = self.layers[L][1]
            H1, p1 = quantities(L, s)
            H2, p2 = quantities(L + 1, s)
            for q in range(4):
                M[row, 4 * L:4 * L + 4] = H1[q]
                M[row, 4 * L + 4:4 * L + 8] = -H2[q]
                rhs[row] = p2[q] - p1[q]
                row += 1
        H, p = quantities(nl - 1, self.layers[-1][1])
        for q in (0, 3):
            M[row, 4 * nl - 4:] = H[q]
            rhs[row] = -p[q]
            row += 1
        self.coef = np.linalg.solve(M, rhs).reshape(nl, 4)


class _ModeSet:
    """A sum of modes sharing the layering: weights w_n, wavenumbers k_n and,
    for 3D, horizontal wavevectors.  Packs the coefficients as tensors."""

    def __init__(self, modes, weights, kvec=None):
        self.modes = modes
        self.nl = len(modes[0].layers)
        self.layers = modes[0].layers
        self.w = np.asarray(weights, dtype=np.float64)
        self.k = np.array([m.k for m in modes])
        self.kvec = None if kvec is None else np.asarray(kvec, dtype=np.float64)
        nq = max(len(m.part[L]) for m in modes for L in range(self.nl))
        nm = len(modes)
        self.lam = np.zeros((self.nl, nm, 4), dtype=complex)
        self.mult = np.zeros((self.nl, nm, 4))
        self.s0 = np.zeros((self.nl, nm, 4))
        self.coef = np.zeros((self.nl, nm, 4), dtype=complex)
        self.pA = np.zeros((self.nl, nm, max(nq, 1)), dtype=complex)
        self.pg = np.zeros((self.nl, nm, max(nq, 1)), dtype=complex)
        self.prho = np.zeros((self.nl, nm, max(nq, 1)), dtype=complex)
        for i, m in enumerate(modes):
            for L in range(self.nl):
                self.lam[L, i] = m.lam[L]
                self.mult[L, i] = m.mult[L]
                self.s0[L, i] = m.s0[L]
                self.coef[L, i] = m.coef[L]
                for q, (A, g, rho) in enumerate(m.part[L]):
                    self.pA[L, i, q], self.pg[L, i, q], self.prho[L, i, q] = A, g, rho
        self._dev = {}

    def _t(self, dev):
        if dev not in self._dev:
            c = lambda a: torch.as_tensor(a, device=dev)
            self._dev[dev] = dict(lam=c(self.lam), mult=c(self.mult), s0=c(self.s0), coef=c(self.coef),
                                  pA=c(self.pA), pg=c(self.pg), prho=c(self.prho), k=c(self.k), w=c(self.w))
        return self._dev[dev]

    def profiles(self, s):
        """(a, b, S/eta, T/eta, eta) per point and mode: [n, nmodes] each."""
        T = self._t(s.device)
        n, nm = s.shape[0], self.k.shape[0]
        chunk = max(64, (1 << 19) // nm)
        out = [torch.zeros((n, nm), dtype=torch.float64, device=s.device) for _ in range(4)]
        eta = torch.zeros(n, dtype=torch.float64, device=s.device)
        k = T["k"][None, :]
        for L, (lo, hi, eta0, B) in enumerate(self.layers):
            sel = s >= lo if L > 0 else torch.ones_like(s, dtype=torch.bool)
            if L < self.nl - 1:
                sel = sel & (s < hi)
            idx = torch.nonzero(sel).flatten()
            if idx.numel() == 0:
                continue
            eta[idx] = eta0 * torch.exp(2.0 * B * s[idx])
            for c0 in range(0, idx.numel(), chunk):
                ii = idx[c0:c0 + chunk]
                sc = s[ii].to(torch.complex128)[:, None, None]
                lam, mult = T["lam"][L][None], T["mult"][L][None]
                sig = sc - T["s0"][L][None]
                e = torch.exp(lam * sig) * T["coef"][L][None]
                sigm = torch.where(mult > 0, sig, torch.ones_like(sig))
                d = [(e * (lam ** i * sigm + mult * i * lam ** max(i - 1, 0))).sum(-1) for i in range(4)]
                rho = T["prho"][L][None]
                ep = torch.exp(rho * sc)
                for i in range(4):
                    d[i] = d[i] + (T["pA"][L][None] * rho ** i * ep).sum(-1)
                gt = (T["pg"][L][None] * ep).sum(-1)
                d = [x.real for x in d]
                gt = gt.real
                a = d[0]
                b = -d[1] / k
                Tt = -d[2] / k - k * d[0]
                Ttp = -d[3] / k - k * d[1]
                St = (Ttp + 2.0 * B * Tt - 4.0 * k * k * b + gt) / k
                for o, v in zip(out, (a, b, St, Tt)):
                    o[ii] = v
        return out + [eta]


# ---------------------------------------------------------------------------
# Function nodes over a mode set
# ---------------------------------------------------------------------------
class _SeriesField(Function):
    """One field of a layered series solution at the evaluation points."""

    def __init__(self, sol, what):
        self.sol, self.what = sol, what
        if what in ("stress", "strainRate"):
            self._kind = "symtensor"

    def _eval(self, ctx):
        return self.sol._field(ctx.coords, self.what)

    def depends_on(self, kinds):
        return "coord" in kinds


class _SeriesSolution(_SolBase):
    """Shared machinery: ``_s``/``_t`` axis of the layering and of the Fourier
    dependence (2D), a _ModeSet, an optional uniform (k = 0) body-force part
    F0 along s, and the stress convention (total stress here)."""

    dim = 2
    nonlinear = False
    _zz_unit_viscosity = False     # the reference's SolA forms sigma_zz with viscosity 1
    _F0 = 0.0          # uniform part of the body force along s (k = 0 mode)
    _p0 = 0.0          # pressure constant of the k = 0 mode: p0(s) = F0 (s - _p0)

    def _fields_2d(self, x):
        s, t = x[:, self._s], x[:, self._t]
        a, b, St, Tt, eta = self.modes.profiles(s)
        T = self.modes._t(x.device)
        k, w = T["k"][None, :], T["w"][None, :]
        ck, sk = torch.cos(k * t[:, None]), torch.sin(k * t[:, None])
        e1 = eta[:, None]
        vs = (w * a * ck).sum(1)
        vt = (w * b * sk).sum(1)
        P = -e1 * St - 2.0 * e1 * k * b
        p = (w * P * ck).sum(1) + self._F0 * (s - self._p0)
        e_ss = (w * (-k * b) * ck).sum(1)
        e_tt = -e_ss
        e_st = (w * 0.5 * Tt * sk).sum(1)
        return vs, vt, p, e_ss, e_tt, e_st, eta

    def _field(self, x, what):
        x = x.to(torch.float64)
        if self.dim == 3:
            return self._field_3d(x, what)
        vs, vt, p, e_ss, e_tt, e_st, eta = self._fields_2d(x)
        if self._s == 0:
            vx, vz, exx, ezz = vs, vt, e_ss, e_tt
        else:
            vx, vz, exx, ezz = vt, vs, e_tt, e_ss
        if what == "velocity":
            return torch.stack([vx, vz], 1)
        if what == "pressure":
            return p[:, None]
        if what == "strainRate":
            return torch.stack([exx, ezz, e_st], 1)
        if what == "stress":
            eta_zz = torch.ones_like(eta) if self._zz_unit_viscosity else eta
            return torch.stack([-p + 2.0 * eta * exx, -p + 2.0 * eta_zz * ezz, 2.0 * eta * e_st], 1)
        raise ValueError(what)

    def _finish(self):
        for what in ("velocity", "pressure", "stress", "strainRate"):
            setattr(self, "fn_" + what, _SeriesField(self, what))

    def get_bcs(self, velVar):
        """Free slip on every wall: each wall's normal velocity component fixed
        (P/function/analytic.py:80-110).  Returns the DirichletCondition."""
        from . import conditions as _cond
        ss = velVar.mesh.specialSets
        names = "IJK"[: self.dim]
        return _cond.DirichletCondition(
            velVar, tuple(ss["Min%s_VertexSet" % c] + ss["Max%s_VertexSet" % c] for c in names))


def _sin_terms(amp, k):
    """amp sin(k s) as exponential terms."""
    return [(amp / 2j, 1j * k), (-amp / 2j, -1j * k)]


def _cos_terms(amp, k):
    return [(amp / 2.0, 1j * k), (amp / 2.0, -1j * k)]


def _check_positive(name, v):
    if v <= 0:
        raise TypeError("'%s' parameter must be positive." % name)


class SolA(_SeriesSolution):
    """Isoviscous flow driven by f = (0, sigma_0 cos(n_x pi x) sin(n_z pi z))
    (P/function/analytic.py:113-144).  fn_stress is the total stress; its zz
    component is -p + 2 e_zz, without eta_0, as the reference's solution
    computes it (L/Underworld/SysTest/AnalyticPlugins/Velic_solA/solA.c:193);
    the two agree at the default eta_0 = 1."""
    eqn_bodyforce = "(0,-\\sigma_0 \\cos(n_x \\pi x) \\sin(n_z \\pi z))"
    eqn_viscosity = "\\eta_0"
    _s, _t = 1, 0
    _zz_unit_viscosity = True

    def __init__(self, sigma_0=1., n_x=3, n_z=2., eta_0=1., *args, **kwargs):
        _check_positive("eta_0", eta_0)
        _check_positive("sigma_0", sigma_0)
        if not isinstance(n_x, int):
            raise TypeError("'n_x' parameter must be of 'int' type.")
        self.sigma_0, self.n_x, self.n_z, self.eta_0 = float(sigma_0), n_x, float(n_z), float(eta_0)
        kx, kz = n_x * _PI, self.n_z * _PI
        self.modes = _ModeSet([_Mode(kx, [(0.0, 1.0, self.eta_0, 0.0)], fs_terms=_sin_terms(self.sigma_0, kz))], [1.0])
        x, z = input()[0], input()[1]
        self.fn_viscosity = constant(float(self.eta_0))
        self.fn_bodyforce = Function.convert((0.0, self.sigma_0 * _fmath.cos(kx * x) * _fmath.sin(kz * z)))
        self._finish()


class SolB(_SeriesSolution):
    """Isoviscous flow driven by f = (0, sigma_0 cos(n_x pi x) sinh(n_z pi z))
    (P/function/analytic.py:146-175)."""
    eqn_bodyforce = "(0,-\\sigma_0 \\cos(n_x \\pi x) \\sinh(n_z \\pi z))"
    eqn_viscosity = "\\eta_0"
    _s, _t = 1, 0

    def __init__(self, sigma_0=1., n_x=3, n_z=2., eta_0=1., *args, **kwargs):
        _check_positive("eta_0", eta_0)
        _check_positive("sigma_0", sigma_0)
        if not isinstance(n_x, int):
            raise TypeError("'n_x' parameter must be of 'int' type.")
        if abs(float(n_x) - float(n_z)) < 1e-5:
            raise TypeError("'n_z' must be different than 'n_x'.")
        self.sigma_0, self.n_x, self.n_z, self.eta_0 = float(sigma_0), n_x, float(n_z), float(eta_0)
        kx, kz = n_x * _PI, self.n_z * _PI
        fs = [(self.sigma_0 / 2.0, kz), (-self.sigma_0 / 2.0, -kz)]
        self.modes = _ModeSet([_Mode(kx, [(0.0, 1.0, self.eta_0, 0.0)], fs_terms=fs)], [1.0])
        x, z = input()[0], input()[1]
        self.fn_viscosity = constant(float(self.eta_0))
        self.fn_bodyforce = Function.convert((0.0, self.sigma_0 * _fmath.cos(kx * x) * _fmath.sinh(kz * z)))
        self._finish()


class SolCx(_SeriesSolution):
    """Viscosity eta_A for x < x_c and eta_B beyond, f = (0, cos(pi x) sin(n_z pi z))
    (P/function/analytic.py:211-240)."""
    eqn_bodyforce = "(0,-\\cos(\\pi x) \\sin(n_z \\pi z))"
    eqn_viscosity = "\\operatorname{step}(\\eta_A,\\eta_B,x_c; x)"
    _s, _t = 0, 1

    def __init__(self, n_z=3, eta_A=1., eta_B=1.e8, x_c=0.75, *args, **kwargs):
        if not isinstance(eta_A, float) or eta_A <= 0:
            raise TypeError("'eta_A' must be a positive float.")
        if not isinstance(eta_B, float) or eta_B <= 0:
            raise TypeError("'eta_B' must be a positive float.")
        if not isinstance(x_c, float):
            raise TypeError("'x_c' parameter must be of type 'float'.")
        if not isinstance(n_z, int):
            raise TypeError("'n_z' parameter must be of type 'int'.")
        if x_c < 0.0 or x_c > 1.0:
            raise ValueError("Valid range of xc values is [0,1]. Provided value was %r" % x_c)
        self.n_z, self.eta_A, self.eta_B, self.x_c = n_z, eta_A, eta_B, x_c
        kz = n_z * _PI
        layers = [L for L in ((0.0, x_c, eta_A, 0.0), (x_c, 1.0, eta_B, 0.0)) if L[1] > L[0]]
        self.modes = _ModeSet([_Mode(kz, layers, ft_terms=_cos_terms(1.0, _PI))], [1.0])
        x, z = input()[0], input()[1]
        self.fn_viscosity = _branching.conditional(((x < x_c, eta_A), (True, eta_B)))
        self.fn_bodyforce = Function.convert((0.0, _fmath.cos(_PI * x) * _fmath.sin(kz * z)))
        self._finish()


class SolKx(_SeriesSolution):
    """Viscosity exp(2 B x), f = (0, sigma_0 cos(n_x pi x) sin(n_z pi z))
    (P/function/analytic.py:382-412); n_z is taken as an integer, as the
    reference's solution class stores it."""
    eqn_bodyforce = "(0,-\\sigma_0 \\cos(n_x \\pi x) \\sin(n_z \\pi z))"
    eqn_viscosity = "\\exp(2Bx)"
    _s, _t = 0, 1

    def __init__(self, sigma_0=1., n_x=3, n_z=2., B=2.302585092994046, *args, **kwargs):
        if not isinstance(sigma_0, float):
            raise TypeError("'sigma_0' must be a float.")
        if not isinstance(n_x, int):
            raise TypeError("'n_x' must be an int.")
        if not isinstance(n_z, (int, float)):
            raise TypeError("'n_z' parameter must be of type 'float'.")
        if not isinstance(B, float):
            raise TypeError("'B' parameter must be of type 'float'.")
        self.sigma_0, self.n_x, self.n_z, self.B = sigma_0, n_x, int(n_z), B
        kx, kz = n_x * _PI, self.n_z * _PI
        self.modes = _ModeSet([_Mode(kz, [(0.0, 1.0, 1.0, B)], ft_terms=_cos_terms(sigma_0, kx))], [1.0])
        x, z = input()[0], input()[1]
        self.fn_viscosity = _fmath.exp(2.0 * B * x)
        self.fn_bodyforce = Function.convert((0.0, sigma_0 * _fmath.cos(kx * x) * _fmath.sin(kz * z)))
        self._finish()


class SolKz(_SeriesSolution):
    """Viscosity exp(2 B z), f = (0, sigma_0 cos(n_x pi x) sin(n_z pi z))
    (P/function/analytic.py:415-446); sigma_0 must be 1, as in the reference."""
    eqn_bodyforce = "(0,-\\sigma_0 \\cos(n_x \\pi x) \\sin(n_z \\pi z))"
    eqn_viscosity = "\\exp(2Bz)"
    _s, _t = 1, 0

    def __init__(self, sigma_0=1., n_x=3, n_z=2., B=2.302585092994046, *args, **kwargs):
        if not isinstance(sigma_0, float) or sigma_0 != 1.:
            raise TypeError("'sigma_0' can be any float as long as it's 1.")
        if not isinstance(n_x, int):
            raise TypeError("'n_x' must be an int.")
        if not isinstance(n_z, (int, float)):
            raise TypeError("'n_z' parameter must be of type 'float'.")
        if not isinstance(B, float):
            raise TypeError("'B' parameter must be of type 'float'.")
        self.sigma_0, self.n_x, self.n_z, self.B = sigma_0, n_x, float(n_z), B
        kx, kz = n_x * _PI, self.n_z * _PI
        self.modes = _ModeSet([_Mode(kx, [(0.0, 1.0, 1.0, B)], fs_terms=_sin_terms(sigma_0, kz))], [1.0])
        x, z = input()[0], input()[1]
        self.fn_viscosity = _fmath.exp(2.0 * B * z)
        self.fn_bodyforce = Function.convert((0.0, sigma_0 * _fmath.cos(kx * x) * _fmath.sin(kz * z)))
        self._finish()


class SolC(_SeriesSolution):
    """Isoviscous flow driven by f = (0, -sigma_0) for x < x_c, 0 beyond, as the
    cosine series of the step in x truncated to modes 1 .. nmodes-1
    (P/function/analytic.py:177-209)."""
    eqn_bodyforce = "(0,-\\sigma_0 \\operatorname{step}(1,0,x_c; x))"
    eqn_viscosity = "\\eta_0"
    _s, _t = 1, 0

    def __init__(self, sigma_0=1., x_c=0.5, eta_0=1., nmodes=200, *args, **kwargs):
        if not isinstance(eta_0, float) or eta_0 <= 0:
            raise TypeError("'eta_0' must be a positive float.")
        if not isinstance(x_c, float):
            raise TypeError("'x_c' parameter must be of type 'float'.")
        self.sigma_0, self.x_c, self.eta_0, self.nmodes = float(sigma_0), x_c, eta_0, int(nmodes)
        n = np.arange(1, self.nmodes)
        kn = n * _PI
        wn = -2.0 * self.sigma_0 * np.sin(kn * x_c) / kn
        self.modes = _ModeSet([_Mode(k, [(0.0, 1.0, eta_0, 0.0)], fs_terms=[(1.0, 0.0)]) for k in kn], wn)
        self._F0 = -self.sigma_0 * x_c
        self._p0 = 0.5
        x = input()[0]
        self.fn_viscosity = constant(float(eta_0))
        self.fn_bodyforce = Function.convert((0.0, _branching.conditional(((x < x_c, -self.sigma_0), (True, 0.0)))))
        self._finish()


class SolDA(_SeriesSolution):
    """Viscosity eta_A for z < z_c and eta_B above, f = (0, -sigma_0) in the column
    |x - x_c| <= x_w/2, 0 outside, as the cosine series truncated to modes
    1 .. nmodes-1 (P/function/analytic.py:242-284)."""
    eqn_bodyforce = "(0, -\\sigma_0 \\operatorname{rect}(x_c,x_w; x) )"
    eqn_viscosity = "\\operatorname{step}(\\eta_A,\\eta_B,z_c; z)"
    _s, _t = 1, 0

    def __init__(self, sigma_0=1., x_c=0.375, x_w=0.25, eta_A=1., eta_B=10., z_c=0.75, nmodes=200,
                 *args, **kwargs):
        if not isinstance(sigma_0, float):
            raise TypeError("'sigma_0' must be a float.")
        if not isinstance(eta_A, float) or eta_A <= 0:
            raise TypeError("'eta_A' must be a positive float.")
        if not isinstance(eta_B, float) or eta_B <= 0:
            raise TypeError("'eta_B' must be a positive float.")
        for nm, v in (("x_c", x_c), ("x_w", x_w), ("z_c", z_c)):
            if not isinstance(v, float):
                raise TypeError("'%s' parameter must be of type 'float'." % nm)
        if not isinstance(nmodes, int) or nmodes <= 0:
            raise TypeError("'nmodes' parameter must be a positive int.")
        lo, hi = x_c - 0.5 * x_w, x_c + 0.5 * x_w
        if lo < 0.0 or hi > 1.0:
            raise ValueError("The column must lie inside the unit square.")
        self.sigma_0, self.x_c, self.x_w, self.eta_A, self.eta_B, self.z_c, self.nmodes = \
            sigma_0, x_c, x_w, eta_A, eta_B, z_c, nmodes
        n = np.arange(1, nmodes)
        kn = n * _PI
        wn = -2.0 * sigma_0 * (np.sin(kn * hi) - np.sin(kn * lo)) / kn
        layers = [L for L in ((0.0, z_c, eta_A, 0.0), (z_c, 1.0, eta_B, 0.0)) if L[1] > L[0]]
        self.modes = _ModeSet([_Mode(k, layers, fs_terms=[(1.0, 0.0)]) for k in kn], wn)
        self._F0 = -sigma_0 * x_w
        self._p0 = z_c
        x, z = input()[0], input()[1]
        self.fn_viscosity = _branching.conditional(((z < z_c, eta_A), (True, eta_B)))
        self.fn_bodyforce = Function.convert(
            (0.0, _branching.conditional((((x >= lo) & (x <= hi), -sigma_0), (True, 0.0)))))
        self._finish()


class SolH(_SeriesSolution):
    """3D isoviscous flow driven by f = (0, 0, -sigma_0) where x <= x_c and
    y <= y_c, 0 elsewhere (P/function/analytic.py:286-329).  The double cosine
    series of the force, truncated to mode numbers 0 .. nmodes-1 in x and in y,
    is solved mode by mode: for the horizontal wavevector (k_x, k_y), k = |k_h|,
    the poloidal flow v_z = a(z) cos cos, v_h = b(z) k_h/k (sin cos, cos sin)
    satisfies the 2D system above with wavenumber k."""
    eqn_bodyforce = "(0, 0, -\\sigma_0 \\operatorname{step}(1, 0, x_c; x) \\operatorname{step}(1, 0, y_c; y) )"
    eqn_viscosity = "\\eta_0"
    dim = 3

    def __init__(self, sigma_0=1000., x_c=0.5, y_c=0.5, eta_0=1., nmodes=30, *args, **kwargs):
        if not isinstance(sigma_0, float):
            raise TypeError("'sigma_0' must be a float.")
        if not isinstance(eta_0, float) or eta_0 <= 0:
            raise TypeError("'eta_0' must be a positive float.")
        if not isinstance(x_c, float):
            raise TypeError("'x_c' parameter must be of type 'float'.")
        if not isinstance(y_c, float):
            raise TypeError("'y_c' parameter must be of type 'float'.")
        if not isinstance(nmodes, int) or nmodes <= 0:
            raise TypeError("'nmodes' parameter must be a positive int.")
        self.sigma_0, self.x_c, self.y_c, self.eta_0, self.nmodes = sigma_0, x_c, y_c, eta_0, nmodes
        n = np.arange(nmodes)
        cx = np.where(n == 0, x_c, 2.0 * np.sin(n * _PI * x_c) / np.maximum(n, 1) / _PI)
        cy = np.where(n == 0, y_c, 2.0 * np.sin(n * _PI * y_c) / np.maximum(n, 1) / _PI)
        modes, w, kv = [], [], []
        for i in range(nmodes):
            for j in range(nmodes):
                if i == 0 and j == 0:
                    continue
                kx, ky = i * _PI, j * _PI
                modes.append(_Mode(np.hypot(kx, ky), [(0.0, 1.0, eta_0, 0.0)], fs_terms=[(1.0, 0.0)]))
                w.append(-sigma_0 * cx[i] * cy[j])
                kv.append((kx, ky))
        self.modes = _ModeSet(modes, w, kv)
        self._F0 = -sigma_0 * x_c * y_c
        self._p0 = 0.5
        x, y = input()[0], input()[1]
        self.fn_viscosity = constant(float(eta_0))
        self.fn_bodyforce = Function.convert(
            (0.0, 0.0, _branching.conditional((((x <= x_c) & (y <= y_c), -sigma_0), (True, 0.0)))))
        self._finish()

    def _field_3d(self, x, what):
        a, b, St, Tt, eta = self.modes.profiles(x[:, 2])
        T = self.modes._t(x.device)
        if "kv" not in T:
            T["kv"] = torch.as_tensor(self.modes.kvec, device=x.device)
        kx, ky = T["kv"][None, :, 0], T["kv"][None, :, 1]
        k, w = T["k"][None, :], T["w"][None, :]
        cx, sx = torch.cos(kx * x[:, 0:1]), torch.sin(kx * x[:, 0:1])
        cy, sy = torch.cos(ky * x[:, 1:2]), torch.sin(ky * x[:, 1:2])
        cc = cx * cy
        e1 = eta[:, None]
        if what == "velocity":
            return torch.stack([(w * b * kx / k * sx * cy).sum(1), (w * b * ky / k * cx * sy).sum(1),
                                (w * a * cc).sum(1)], 1)
        P = -e1 * St - 2.0 * e1 * k * b
        p = (w * P * cc).sum(1) + self._F0 * (x[:, 2] - self._p0)
        if what == "pressure":
            return p[:, None]
        e = [(w * b * kx * kx / k * cc).sum(1), (w * b * ky * ky / k * cc).sum(1), (w * (-k * b) * cc).sum(1),
             (w * (-b * kx * ky / k) * sx * sy).sum(1), (w * 0.5 * kx / k * Tt * sx * cy).sum(1),
             (w * 0.5 * ky / k * Tt * cx * sy).sum(1)]
        if what == "strainRate":
            return torch.stack(e, 1)
        if what == "stress":
            return torch.stack([2.0 * eta * c - (p if i < 3 else 0.0) for i, c in enumerate(e)], 1)
        raise ValueError(what)


class SolM(_SeriesSolution):
    """Viscosity 1 + eta_0 (1 + cos(m_x pi x)) with the prescribed flow
    v = (-sin(n_x pi x) n_z pi cos(n_z pi z), cos(n_x pi x) n_x pi sin(n_z pi z))
    (P/function/analytic.py:448-479).  The pressure is the antiderivative in x
    of the x-momentum balance (no body force along x) and the body force along
    z closes the z balance.  fn_stress is 2 eta_0 (1 + cos(m_x pi x)) times the
    strain rate: the viscosity without its background 1, as the reference's
    solution class defines it (L/Underworld/Function/src/AnalyticSolM.hpp,
    SolM::stress)."""
    eqn_bodyforce = None
    eqn_viscosity = "1 + \\eta_0(1+\\cos(m_x \\pi x))"

    def __init__(self, eta_0=1., n_x=3, n_z=2, m_x=4., *args, **kwargs):
        if not isinstance(eta_0, float) or eta_0 <= 0.:
            raise TypeError("'eta_0' can be any positive float.")
        if not isinstance(n_x, int):
            raise TypeError("'n_x' must be an int.")
        if not isinstance(n_z, int):
            raise TypeError("'n_z' must be an int.")
        if not isinstance(m_x, float):
            raise TypeError("'m_x' parameter must be a 'float' and != 'n_z'.")
        if abs(float(n_z) - m_x) < 1e-5:
            raise TypeError("'m_x' must be different than 'n_z'.")
        self.eta_0, self.n_x, self.n_z, self.m_x = eta_0, n_x, n_z, m_x
        km, kn, kr = n_x * _PI, n_z * _PI, m_x * _PI
        x, z = input()[0], input()[1]
        Cm, Sm = _fmath.cos(km * x), _fmath.sin(km * x)
        Cn, Sn = _fmath.cos(kn * z), _fmath.sin(kn * z)
        Cr, Sr = _fmath.cos(kr * x), _fmath.sin(kr * x)
        eta = 1.0 + eta_0 * (1.0 + Cr)
        deta = -eta_0 * kr * Sr
        d = kn * kn - km * km
        # int eta sin(km x) dx
        I = -(1.0 + eta_0) / km * Cm - eta_0 * (km * Cm * Cr + kr * Sm * Sr) / (km * km - kr * kr)
        self.fn_velocity = Function.convert((-kn * Sm * Cn, km * Cm * Sn))
        exx = -km * kn * Cm * Cn
        exz = 0.5 * d * Sm * Sn
        self.fn_strainRate = Function.convert((exx, -exx, exz))
        eta_s = eta_0 * (1.0 + Cr)
        self.fn_stress = Function.convert((2.0 * eta_s * exx, -2.0 * eta_s * exx, 2.0 * eta_s * exz))
        self.fn_viscosity = eta
        self.fn_pressure = kn * Cn * (-2.0 * km * eta * Cm + d * I)
        self.fn_bodyforce = Function.convert(
            (0.0, Sn * (4.0 * km * kn * kn * eta * Cm - kn * kn * d * I - d * (deta * Sm + km * eta * Cm))))


class SolNL(_SolBase):
    """Power-law flow (P/function/analytic.py:481-565): v = (-e^x cos(n_z pi z) n_z pi,
    e^x sin(n_z pi z)) with viscosity 2 eta_0 (e_xx^2 + e_xz^2)^(1/r - 1).  With
    E = e^x, c, s = cos, sin(n_z pi z), q = c^2 k^2 + s^2 (k^2+1)^2/4, the strain
    rate invariant is E^2 q; the pressure is the antiderivative in x of the
    x-momentum balance, p = E^(1+2 alpha) Pi(z), and the body force along z
    closes the z balance.  ``fn_viscosity`` is the analytic viscosity (a
    function of position); ``get_viscosity_nl`` the same law of a numerical
    velocity.  Stress is 2 eta times the strain rate."""
    eqn_bodyforce = None
    eqn_viscosity = "\\eta_0 ( \\dot{\\eta}_{ij} \\dot{\\eta}_{ij} )^{(1/r - 1)}"
    dim = 2

    def __init__(self, eta_0=1., n_z=1, r=1.5, *args, **kwargs):
        if not isinstance(eta_0, float) or eta_0 <= 0.:
            raise TypeError("'eta_0' can be any positive float.")
        if not isinstance(n_z, int):
            raise TypeError("'n_z' must be an int.")
        if not isinstance(r, float):
            raise TypeError("'r' parameter must be a 'float'.")
        self.eta_0, self.n_z, self.r = eta_0, n_z, r
        self.nonlinear = True
        k = n_z * _PI
        al = 1.0 / r - 1.0
        x, z = input()[0], input()[1]
        E = _fmath.exp(x)
        c, s = _fmath.cos(k * z), _fmath.sin(k * z)
        k2p = k * k + 1.0
        q = c * c * (k * k) + 0.25 * k2p * k2p * s * s
        D = 0.5 * k2p * k2p - 2.0 * k * k
        qa = _fmath.pow(q, al)
        qa1 = _fmath.pow(q, al - 1.0)
        qa2 = _fmath.pow(q, al - 2.0)
        Ea = _fmath.pow(E, 1.0 + 2.0 * al)
        self.fn_velocity = Function.convert((-k * E * c, E * s))
        exx = -k * E * c
        exz = 0.5 * k2p * E * s
        eta = 2.0 * eta_0 * _fmath.pow(exx * exx + exz * exz, al)
        self.fn_viscosity = eta
        self.fn_strainRate = Function.convert((exx, -exx, exz))
        self.fn_stress = Function.convert((2.0 * eta * exx, -2.0 * eta * exx, 2.0 * eta * exz))
        h = q + al * s * s * D
        dqac = k * s * qa1 * (al * c * c * D - q)                       # (q^a c)'
        dqas = k * c * qa1 * h                                          # (q^a s)'
        d2qas = k * k * s * qa2 * (-q * h + (al - 1.0) * c * c * D * h + (1.0 + 2.0 * al) * c * c * D * q)
        self.fn_pressure = Ea * (-4.0 * eta_0 * k * qa * c + 2.0 * eta_0 * k2p * dqas / (1.0 + 2.0 * al))
        self.fn_bodyforce = Function.convert(
            (0.0, Ea * (-8.0 * eta_0 * k * dqac + 2.0 * eta_0 * k2p * d2qas / (1.0 + 2.0 * al)
                        - (1.0 + 2.0 * al) * 2.0 * eta_0 * k2p * qa * s)))

    def get_bcs(self, velVar):
        """Analytic velocity on every wall; x velocity fixed on the vertical walls,
        z velocity on all walls (P/function/analytic.py:512-544)."""
        from . import conditions as _cond
        mesh = velVar.mesh
        ss = mesh.specialSets
        walls = ss["AllWalls_VertexSet"]
        velVar.data[walls.data] = self.fn_velocity.evaluate(mesh.data[walls.data])
        iw = ss["MinI_VertexSet"] + ss["MaxI_VertexSet"]
        jw = ss["MinJ_VertexSet"] + ss["MaxJ_VertexSet"]
        return _cond.DirichletCondition(velVar, (iw, iw + jw))

    def get_viscosity_nl(self, velocity, pressure):
        """2 eta_0 (second invariant of the deviatoric strain rate of `velocity`)
        ^ (2/r - 2) (P/function/analytic.py:546-565)."""
        from .function import tensor as _tensor
        inv2 = _tensor.second_invariant(_tensor.deviatoric(_tensor.symmetric(velocity.fn_gradient)))
        return 2.0 * self.eta_0 * _fmath.pow(inv2, 2.0 / self.r - 2.0)
