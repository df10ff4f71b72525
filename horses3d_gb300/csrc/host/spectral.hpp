// Spectral operators of one polynomial order: nodes, weights, derivative and boundary matrices.
// Follows NodalStorageClass.f90:170-338 (ConstructNodalStorage), LegendreAlgorithms.f90:137-361,
// InterpolationAndDerivatives.f90:109-255,413-458,799-828 and InterpolationMatrices.f90:42-113.
//
// Matrices are stored row-major: M[i*(cols)+j] = M(i,j) with the reference's 0-based indices.
#pragma once
#include <vector>

namespace h3d {

constexpr double kPi = 3.141592653589793238462643;

struct NodalStorage {
    int N = 0;
    int nodes = 0;                  // 0 Gauss, 1 Gauss-Lobatto
    std::vector<double> x, w, wb;   // nodes, quadrature weights, barycentric weights
    std::vector<double> D;          // D(i,j) = l_j'(x_i)
    std::vector<double> hatD;       // hatD(i,j) = D(j,i) w_j / w_i
    std::vector<double> sharpD;     // Gauss-Lobatto only: 2D with corner corrections
    std::vector<double> vL, vR;     // l_j(-1), l_j(+1)
    std::vector<double> bL, bR;     // v / w
    std::vector<double> xCGL, wbCGL, DCGL;
    std::vector<double> TCheb2Gauss;  // (0:N,0:N): CGL -> solution nodes
};

// Cached per (nodes, N); valid for the lifetime of the process.
const NodalStorage& nodal_storage(int nodes, int N);

// Tset(Norigin, Ndest)%T (0:Ndest, 0:Norigin), row-major [Ndest+1][Norigin+1].
std::vector<double> interpolation_matrix(int nodes, int Norigin, int Ndest);

bool almost_equal(double a, double b);
void barycentric_weights(int N, const double* x, double* w);
void interpolating_polynomial_vector(double x, int N, const double* nodes, const double* wb, double* p);
void polynomial_derivative_matrix(int N, const double* nodes, double* D);
void polynomial_interpolation_matrix(int N, int M, const double* oldNodes, const double* wb,
                                     const double* newNodes, double* T);

}  // namespace h3d
