"""Parameter sets of the analytic-solution fixtures: (name, constructor
parameters of the reference's C++ solution class in the Python interface's
order, keyword arguments of uw.function.analytic.<name>, dim).  Each solution
at its defaults and at one other set."""
LN10 = 2.302585092994046

CASES = [
    ("SolA", (1., 1., 3, 2.), {}, 2),
    ("SolA", (2., 3., 2, 1.5), dict(sigma_0=2., n_x=2, n_z=1.5, eta_0=3.), 2),
    ("SolB", (1., 1., 3, 2.), {}, 2),
    ("SolB", (2., 3., 2, 1.5), dict(sigma_0=2., n_x=2, n_z=1.5, eta_0=3.), 2),
    ("SolC", (1., 1., 0.5, 200), {}, 2),
    ("SolC", (2., 3., 0.3, 50), dict(sigma_0=2., eta_0=3., x_c=0.3, nmodes=50), 2),
    ("SolCx", (1., 1e8, 0.75, 3), {}, 2),
    ("SolCx", (1., 10., 0.4, 2), dict(n_z=2, eta_B=10., x_c=0.4), 2),
    ("SolDA", (1., 0.375, 0.25, 1., 10., 0.75, 200), {}, 2),
    ("SolDA", (2., 0.5, 0.3, 3., 1., 0.4, 100),
     dict(sigma_0=2., x_c=0.5, x_w=0.3, eta_A=3., eta_B=1., z_c=0.4, nmodes=100), 2),
    ("SolH", (1000., 0.5, 0.5, 1., 30), {}, 3),
    ("SolH", (10., 0.3, 0.6, 2., 12), dict(sigma_0=10., x_c=0.3, y_c=0.6, eta_0=2., nmodes=12), 3),
    ("SolKx", (1., 3, 2., LN10), {}, 2),
    ("SolKx", (1.5, 2, 3., 1.1), dict(sigma_0=1.5, n_x=2, n_z=3., B=1.1), 2),
    ("SolKz", (1., 3, 2., LN10), {}, 2),
    ("SolKz", (1., 2, 1.5, 0.7), dict(n_x=2, n_z=1.5, B=0.7), 2),
    ("SolM", (1., 3, 2, 4.), {}, 2),
    ("SolM", (2., 2, 3, 1.5), dict(eta_0=2., n_x=2, n_z=3, m_x=1.5), 2),
    ("SolNL", (1., 1, 1.5), {}, 2),
    ("SolNL", (2., 2, 2.5), dict(eta_0=2., n_z=2, r=2.5), 2),
    ("SolDB2d", (), {}, 2),
    ("SolDB3d", (4.,), {}, 3),
    ("SolDB3d", (1.5,), dict(Beta=1.5), 3),
]

FIELDS = ("velocity", "pressure", "stress", "strainRate", "viscosity", "bodyforce")
