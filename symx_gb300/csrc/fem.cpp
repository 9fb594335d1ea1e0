#include "fem.h"

#include <cmath>
#include <stdexcept>

namespace symx {

std::string get_name(const FEM_Element& e)
{
    switch (e) {
        case FEM_Element::Tet4: return "Tet4";
        case FEM_Element::Tet10: return "Tet10";
        case FEM_Element::Hex8: return "Hex8";
        default: return "Hex27";
    }
}

int get_stride(const FEM_Element& e)
{
    switch (e) {
        case FEM_Element::Tet4: return 4;
        case FEM_Element::Tet10: return 10;
        case FEM_Element::Hex8: return 8;
        default: return 27;
    }
}

std::vector<std::array<double, 4>> get_integration_rule(const FEM_Element& e)
{
    if (e == FEM_Element::Tet4) return {{1.0 / 6.0, 0.25, 0.25, 0.25}};
    if (e == FEM_Element::Hex8) {
        const double p = 1.0 / std::sqrt(3.0);
        return {{1.0, -p, -p, -p}, {1.0, p, -p, -p}, {1.0, p, p, -p}, {1.0, -p, p, -p},
                {1.0, -p, -p, p},  {1.0, p, -p, p},  {1.0, p, p, p},  {1.0, -p, p, p}};
    }
    if (e == FEM_Element::Tet10) {
        // 4-point rule with the reference's rounded weights and points
        // (symx/src/solver/fem_integrators.cpp:60-68), kept identical so energies match
        const double w = 0.041666667, a = 0.58541020, b = 0.13819660;
        return {{w, a, b, b}, {w, b, a, b}, {w, b, b, a}, {w, b, b, b}};
    }
    if (e == FEM_Element::Hex27) {
        // 3x3x3 Gauss-Legendre, products of the 1-D weights 5/9 and 8/9 at -p, 0, p with
        // p = sqrt(3/5): corners, edge, face and centre points in the reference's order and
        // with its rounded values (symx/src/solver/fem_integrators.cpp:83-113)
        const double p = 0.7745966692;
        const double wc = 0.1714677641, we = 0.2743484225, wf = 0.4389574760, w0 = 0.7023319616;
        return {{wc, -p, -p, -p}, {wc, p, -p, -p}, {wc, -p, p, -p}, {wc, p, p, -p},
                {wc, -p, -p, p},  {wc, p, -p, p},  {wc, -p, p, p},  {wc, p, p, p},
                {we, 0.0, -p, -p}, {we, -p, 0.0, -p}, {we, p, 0.0, -p}, {we, 0.0, p, -p},
                {we, -p, -p, 0.0}, {we, p, -p, 0.0}, {we, -p, p, 0.0}, {we, p, p, 0.0},
                {we, 0.0, -p, p},  {we, -p, 0.0, p},  {we, p, 0.0, p},  {we, 0.0, p, p},
                {wf, 0.0, 0.0, -p}, {wf, 0.0, -p, 0.0}, {wf, -p, 0.0, 0.0},
                {wf, p, 0.0, 0.0},  {wf, 0.0, p, 0.0},  {wf, 0.0, 0.0, p},
                {w0, 0.0, 0.0, 0.0}};
    }
    throw std::runtime_error("symx_gb300: unknown element type");
}

Vector fem_interpolation(const FEM_Element& e, const std::vector<Vector>& vh, const Vector& xi)
{
    std::vector<Scalar> N;
    if (e == FEM_Element::Tet4) {
        if (vh.size() != 4) throw std::runtime_error("symx: Tet4 interpolation needs 4 nodes");
        N = {1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]};
    } else if (e == FEM_Element::Hex8) {
        if (vh.size() != 8) throw std::runtime_error("symx: Hex8 interpolation needs 8 nodes");
        const Scalar xm = 0.5 * (1.0 - xi[0]), xp = 0.5 * (1.0 + xi[0]);
        const Scalar ym = 0.5 * (1.0 - xi[1]), yp = 0.5 * (1.0 + xi[1]);
        const Scalar zm = 0.5 * (1.0 - xi[2]), zp = 0.5 * (1.0 + xi[2]);
        N = {xm * ym * zm, xp * ym * zm, xp * yp * zm, xm * yp * zm,
             xm * ym * zp, xp * ym * zp, xp * yp * zp, xm * yp * zp};
    } else if (e == FEM_Element::Tet10) {
        if (vh.size() != 10) throw std::runtime_error("symx: Tet10 interpolation needs 10 nodes");
        const Scalar n0 = 1.0 - xi[0] - xi[1] - xi[2], n1 = xi[0], n2 = xi[1], n3 = xi[2];
        N = {n0 * (2.0 * n0 - 1.0), n1 * (2.0 * n1 - 1.0), n2 * (2.0 * n2 - 1.0), n3 * (2.0 * n3 - 1.0),
             4.0 * n0 * n1,         4.0 * n1 * n2,         4.0 * n2 * n0,         4.0 * n0 * n3,
             4.0 * n1 * n3,         4.0 * n2 * n3};
    } else if (e == FEM_Element::Hex27) {
        // triquadratic Lagrange: per axis L-(t) = t(t-1)/2, L+(t) = t(t+1)/2, L0(t) = 1-t^2,
        // nodes ordered corners, mid-edges (z = -1 ring, z = +1 ring, vertical), faces
        // (x-, x+, y+, y-, z-, z+), centre, as the reference's Hex27 mesh and shape functions
        if (vh.size() != 27) throw std::runtime_error("symx: Hex27 interpolation needs 27 nodes");
        std::array<std::array<Scalar, 3>, 3> L{};  // L[axis][0: -1, 1: 0, 2: +1]
        for (int k = 0; k < 3; ++k) {
            const Scalar& t = xi[k];
            L[k][0] = 0.5 * t * (t - 1.0);
            L[k][1] = 1.0 - t * t;
            L[k][2] = 0.5 * t * (t + 1.0);
        }
        static const int at[27][3] = {{0, 0, 0}, {2, 0, 0}, {2, 2, 0}, {0, 2, 0}, {0, 0, 2}, {2, 0, 2}, {2, 2, 2},
                                      {0, 2, 2}, {1, 0, 0}, {2, 1, 0}, {1, 2, 0}, {0, 1, 0}, {1, 0, 2}, {2, 1, 2},
                                      {1, 2, 2}, {0, 1, 2}, {0, 0, 1}, {2, 0, 1}, {2, 2, 1}, {0, 2, 1}, {0, 1, 1},
                                      {2, 1, 1}, {1, 2, 1}, {1, 0, 1}, {1, 1, 0}, {1, 1, 2}, {1, 1, 1}};
        for (const auto& a : at) N.push_back(L[0][a[0]] * L[1][a[1]] * L[2][a[2]]);
    } else {
        throw std::runtime_error("symx_gb300: unknown element type");
    }
    Vector x = vh[0] * N[0];
    for (size_t a = 1; a < vh.size(); ++a) x = x + vh[a] * N[a];
    return x;
}

Matrix fem_jacobian(const FEM_Element& e, const std::vector<Vector>& xh, const Vector& xi)
{
    const Vector x = fem_interpolation(e, xh, xi);
    std::vector<Scalar> v;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) v.push_back(diff(x[i], xi[j]));
    return Matrix(v, {3, 3});
}

Scalar fem_integrator(MappedWorkspace<double>& mws, const FEM_Element& e,
                      std::function<Scalar(Scalar& w, Vector& xi)> summand)
{
    const std::vector<std::array<double, 4>> rule = get_integration_rule(e);
    return mws.add_for_each(rule, [&](Vector& ip) {
        Scalar w = ip[0];
        Vector xi({ip[1], ip[2], ip[3]});
        return summand(w, xi);
    });
}

}  // namespace symx
