// FEM helpers for potential definitions (reference: symx/src/solver/fem_integrators.{h,cpp}).
// Shape functions and quadrature rules for Tet4 (1 point, weight 1/6), Tet10 (4 points),
// Hex8 (2x2x2 Gauss, weight 1, +-1/sqrt(3)) and Hex27 (3x3x3 Gauss, triquadratic
// Lagrange); fem_integrator registers the rule as a
// summation, so the element kernel runs the summand once per quadrature point.
#pragma once

#include <array>
#include <functional>
#include <string>
#include <vector>

#include "mapped_workspace.h"

namespace symx {

enum class FEM_Element { Tet4, Tet10, Hex8, Hex27 };

std::string get_name(const FEM_Element& element);
int get_stride(const FEM_Element& element);
// Rows {weight, xi0, xi1, xi2}.
std::vector<std::array<double, 4>> get_integration_rule(const FEM_Element& element);
Vector fem_interpolation(const FEM_Element& element, const std::vector<Vector>& vh, const Vector& xi);
// J = d(sum_a N_a(xi) x_a) / d xi, by symbolic differentiation with respect to xi.
Matrix fem_jacobian(const FEM_Element& element, const std::vector<Vector>& xh, const Vector& xi);
Scalar fem_integrator(MappedWorkspace<double>& mws, const FEM_Element& element,
                      std::function<Scalar(Scalar& w, Vector& xi)> summand);

}  // namespace symx
