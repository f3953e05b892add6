// TEST INFRASTRUCTURE: a C entry point over the reference's own analytic Stokes
// solutions, compiled from the reference tree by oracle/ref_analytic.py into
// oracle/_ref/ (never shipped, never linked by the package).  The solution
// classes are the reference's (underworld/libUnderworld/Underworld/Function/src/
// AnalyticSol*.hpp over SysTest/AnalyticPlugins/Velic_sol*/sol*.c); this file only
// constructs them with the parameters of the Python interface
// (src/underworld/function/analytic.py:142-656) and calls their member functions.
#include <cstring>
#include <stdexcept>

#include "AnalyticSolA.hpp"
#include "AnalyticSolB.hpp"
#include "AnalyticSolC.hpp"
#include "AnalyticSolCx.hpp"
#include "AnalyticSolDA.hpp"
#include "AnalyticSolDB2d.hpp"
#include "AnalyticSolDB3d.hpp"
#include "AnalyticSolH.hpp"
#include "AnalyticSolKx.hpp"
#include "AnalyticSolKz.hpp"
#include "AnalyticSolM.hpp"
#include "AnalyticSolNL.hpp"

// Per point, `out` receives dim velocity components, the pressure, the stress and
// the strain rate (3 or 6 symmetric-tensor components each), the viscosity and dim
// body-force components: 2*dim + 8 values in 2D, 2*dim + 14 in 3D.
template <class S>
static void eval_points(S& s, int dim, const double* pos, long n, double* out)
{
    const int ns = dim == 2 ? 3 : 6;
    const int stride = 2 * dim + 2 + 2 * ns;
    for (long i = 0; i < n; i++) {
        const double* x = pos + i * dim;
        double* o = out + i * stride;
        s.velocity(x, o);
        s.pressure(x, o + dim);
        s.stress(x, o + dim + 1);
        s.strainrate(x, o + dim + 1 + ns);
        s.viscosity(x, o + dim + 1 + 2 * ns);
        s.bodyforce(x, o + dim + 2 + 2 * ns);
    }
}

extern "C" int uwref_analytic(const char* name, const double* p, const double* pos, long n, double* out)
{
    try {
        if (!strcmp(name, "SolA")) { Fn::SolA s(p[0], p[1], (unsigned)p[2], p[3]); eval_points(s, 2, pos, n, out); }
        else if (!strcmp(name, "SolB")) { Fn::SolB s(p[0], p[1], (unsigned)p[2], p[3]); eval_points(s, 2, pos, n, out); }
        else if (!strcmp(name, "SolC")) { Fn::SolC s(p[0], p[1], p[2], (int)p[3]); eval_points(s, 2, pos, n, out); }
        else if (!strcmp(name, "SolCx")) { Fn::SolCx s(p[0], p[1], p[2], (unsigned)p[3]); eval_points(s, 2, pos, n, out); }
        else if (!strcmp(name, "SolDA")) { Fn::SolDA s(p[0], p[1], p[2], p[3], p[4], p[5], (int)p[6]); eval_points(s, 2, pos, n, out); }
        else if (!strcmp(name, "SolH")) { Fn::SolH s(p[0], p[1], p[2], p[3], (int)p[4]); eval_points(s, 3, pos, n, out); }
        else if (!strcmp(name, "SolKx")) { Fn::SolKx s(p[0], p[1], p[2], p[3]); eval_points(s, 2, pos, n, out); }
        else if (!strcmp(name, "SolKz")) { Fn::SolKz s(p[0], (unsigned)p[1], p[2], p[3]); eval_points(s, 2, pos, n, out); }
        else if (!strcmp(name, "SolM")) { Fn::SolM s(p[0], (unsigned)p[1], (unsigned)p[2], p[3]); eval_points(s, 2, pos, n, out); }
        else if (!strcmp(name, "SolNL")) { Fn::SolNL s(p[0], (unsigned)p[1], p[2]); eval_points(s, 2, pos, n, out); }
        else if (!strcmp(name, "SolDB2d")) { Fn::SolDB2d s; eval_points(s, 2, pos, n, out); }
        else if (!strcmp(name, "SolDB3d")) { Fn::SolDB3d s(p[0]); eval_points(s, 3, pos, n, out); }
        else return -1;
    } catch (const std::exception&) {
        return -2;
    }
    return 0;
}
