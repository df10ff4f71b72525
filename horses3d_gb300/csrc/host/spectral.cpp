// Spectral operators: see spectral.hpp for the reference routines each function follows.
#include "spectral.hpp"

#include <cfloat>
#include <cmath>
#include <map>
#include <mutex>
#include <utility>

namespace h3d {

// Utilities.f90:110-139 (AlmostEqual with its default tolerance 2*epsilon).
bool almost_equal(double a, double b) {
    const double tol = 2.0 * DBL_EPSILON;
    if (a == 0.0 || b == 0.0) return std::fabs(a - b) <= tol;
    return std::fabs(b - a) <= tol * std::fmax(std::fabs(a), std::fabs(b));
}

// LegendreAlgorithms.f90 LegendrePolyAndDerivative: three-term recursion.
static void legendre_and_derivative(int N, double x, double& L, double& Lp) {
    if (N == 0) { L = 1.0; Lp = 0.0; return; }
    if (N == 1) { L = x; Lp = 1.0; return; }
    double Lm2 = 1.0, Lpm2 = 0.0, Lm1 = x, Lpm1 = 1.0;
    for (int k = 2; k <= N; ++k) {
        L = ((2 * k - 1) * x * Lm1 - (k - 1) * Lm2) / k;
        Lp = Lpm2 + (2 * k - 1) * Lm1;
        Lm2 = Lm1; Lm1 = L; Lpm2 = Lpm1; Lpm1 = Lp;
    }
}

// LegendreAlgorithms.f90:137 GaussLegendreNodesAndWeights (Newton on P_{N+1}).
static void gauss_nodes(int N, double* x, double* w) {
    const double tol = 4.0 * DBL_EPSILON;
    double L, Lp;
    if (N == 0) { x[0] = 0.0; w[0] = 2.0; return; }
    if (N == 1) {
        x[0] = -std::sqrt(1.0 / 3.0); w[0] = 1.0; x[1] = -x[0]; w[1] = w[0];
    } else {
        const int half = (N + 1) / 2;
        for (int j = 0; j < half; ++j) {
            double xj = -std::cos((2 * j + 1) * kPi / (2 * N + 2));
            for (int k = 0; k <= 10; ++k) {
                legendre_and_derivative(N + 1, xj, L, Lp);
                const double delta = -L / Lp;
                xj = xj + delta;
                if (std::fabs(delta) <= tol * std::fabs(xj)) break;
            }
            legendre_and_derivative(N + 1, xj, L, Lp);
            x[j] = xj;
            w[j] = 2.0 / ((1.0 - xj * xj) * (Lp * Lp));
            x[N - j] = -xj;
            w[N - j] = w[j];
        }
    }
    if (N % 2 == 0) {
        legendre_and_derivative(N + 1, 0.0, L, Lp);
        x[N / 2] = 0.0;
        w[N / 2] = 2.0 / (Lp * Lp);
    }
}

// LegendreAlgorithms.f90 qAndLEvaluation: q = L_{N+1} - L_{N-1} and its derivative.
static void q_and_l(int N, double x, double& q, double& qp, double& LN) {
    double Lm2 = 1.0, Lpm2 = 0.0, Lm1 = x, Lpm1 = 1.0, Lk = 0.0, Lpk = 0.0;
    for (int k = 2; k <= N; ++k) {
        Lk = ((2 * k - 1) * x * Lm1 - (k - 1) * Lm2) / k;
        Lpk = Lpm2 + (2 * k - 1) * Lm1;
        Lm2 = Lm1; Lm1 = Lk; Lpm2 = Lpm1; Lpm1 = Lpk;
    }
    const int k = N + 1;
    Lk = ((2 * k - 1) * x * Lm1 - (k - 1) * Lm2) / k;
    Lpk = Lpm2 + (2 * k - 1) * Lm1;
    q = Lk - Lm2;
    qp = Lpk - Lpm2;
    LN = Lm1;
}

// LegendreAlgorithms.f90:275 LegendreLobattoNodesAndWeights.
static void lobatto_nodes(int N, double* x, double* w) {
    const double tol = 4.0 * DBL_EPSILON;
    if (N == 0) { x[0] = 0.0; w[0] = 2.0; return; }  // NodalStorage special case for N=0
    if (N == 1) {
        x[0] = -1.0; w[0] = 1.0; x[1] = 1.0; w[1] = 1.0;
    } else {
        x[0] = -1.0; w[0] = 2.0 / (N * (N + 1)); x[N] = 1.0; w[N] = w[0];
        const int half = (N + 1) / 2;
        for (int j = 1; j <= half - 1; ++j) {
            double xj = -std::cos((j + 0.25) * kPi / N - 3.0 / (8 * N * kPi * (j + 0.25)));
            double q, qp, LN;
            for (int k = 0; k <= 10; ++k) {
                q_and_l(N, xj, q, qp, LN);
                const double delta = -q / qp;
                xj = xj + delta;
                if (std::fabs(delta) <= tol * std::fabs(xj)) break;
            }
            q_and_l(N, xj, q, qp, LN);
            x[j] = xj;
            w[j] = 2.0 / (N * (N + 1) * (LN * LN));
            x[N - j] = -xj;
            w[N - j] = w[j];
        }
    }
    if (N % 2 == 0) {
        double LN, Lp;
        legendre_and_derivative(N, 0.0, LN, Lp);
        x[N / 2] = 0.0;
        w[N / 2] = 2.0 / (N * (N + 1) * (LN * LN));
    }
}

// InterpolationAndDerivatives.f90:230-255.
void barycentric_weights(int N, const double* x, double* w) {
    for (int j = 0; j <= N; ++j) w[j] = 1.0;
    for (int j = 1; j <= N; ++j)
        for (int k = 0; k <= j - 1; ++k) {
            w[k] = w[k] * (x[k] - x[j]);
            w[j] = w[j] * (x[j] - x[k]);
        }
    for (int j = 0; j <= N; ++j) w[j] = 1.0 / w[j];
}

// InterpolationAndDerivatives.f90:109-159 (barycentric Lagrange basis at x).
void interpolating_polynomial_vector(double x, int N, const double* nodes, const double* wb, double* p) {
    bool match = false;
    for (int j = 0; j <= N; ++j) {
        p[j] = 0.0;
        if (almost_equal(x, nodes[j])) { p[j] = 1.0; match = true; }
    }
    if (match) return;
    double d = 0.0;
    for (int j = 0; j <= N; ++j) {
        const double t = wb[j] / (x - nodes[j]);
        p[j] = t;
        d = d + t;
    }
    for (int j = 0; j <= N; ++j) p[j] = p[j] / d;
}

// InterpolationAndDerivatives.f90:799-828.
void polynomial_derivative_matrix(int N, const double* nodes, double* D) {
    std::vector<double> bw(N + 1);
    barycentric_weights(N, nodes, bw.data());
    const int n1 = N + 1;
    for (int i = 0; i <= N; ++i) {
        D[i * n1 + i] = 0.0;
        for (int j = 0; j <= N; ++j) {
            if (j == i) continue;
            D[i * n1 + j] = bw[j] / (bw[i] * (nodes[i] - nodes[j]));
            D[i * n1 + i] = D[i * n1 + i] - D[i * n1 + j];
        }
    }
}

// InterpolationAndDerivatives.f90:413-458: T(0:M,0:N) row-major.
void polynomial_interpolation_matrix(int N, int M, const double* oldNodes, const double* wb,
                                     const double* newNodes, double* T) {
    const int n1 = N + 1;
    for (int k = 0; k <= M; ++k) {
        bool match = false;
        for (int j = 0; j <= N; ++j) {
            T[k * n1 + j] = 0.0;
            if (almost_equal(newNodes[k], oldNodes[j])) { match = true; T[k * n1 + j] = 1.0; }
        }
        if (!match) {
            double s = 0.0;
            for (int j = 0; j <= N; ++j) {
                const double tmp = wb[j] / (newNodes[k] - oldNodes[j]);
                T[k * n1 + j] = tmp;
                s = s + tmp;
            }
            for (int j = 0; j <= N; ++j) T[k * n1 + j] = T[k * n1 + j] / s;
        }
    }
}

static NodalStorage build_nodal_storage(int nodes, int N) {
    NodalStorage s;
    s.N = N;
    s.nodes = nodes;
    const int n1 = N + 1;
    s.x.assign(n1, 0.0); s.w.assign(n1, 0.0); s.wb.assign(n1, 0.0);
    if (nodes == 0) gauss_nodes(N, s.x.data(), s.w.data());
    else lobatto_nodes(N, s.x.data(), s.w.data());

    s.D.assign(n1 * n1, 0.0);
    s.hatD.assign(n1 * n1, 0.0);
    polynomial_derivative_matrix(N, s.x.data(), s.D.data());
    for (int j = 0; j <= N; ++j)
        for (int i = 0; i <= N; ++i) {
            const double DT = s.D[j * n1 + i];  // DT(i,j) = D(j,i)
            s.hatD[i * n1 + j] = DT * s.w[j] / s.w[i];
        }
    if (nodes == 1) {
        s.sharpD.assign(n1 * n1, 0.0);
        if (N != 0) {
            for (int k = 0; k < n1 * n1; ++k) s.sharpD[k] = 2.0 * s.D[k];
            s.sharpD[0] = 2.0 * s.D[0] + 1.0 / s.w[0];
            s.sharpD[N * n1 + N] = 2.0 * s.D[N * n1 + N] - 1.0 / s.w[N];
        }
    }
    barycentric_weights(N, s.x.data(), s.wb.data());
    s.vL.assign(n1, 0.0); s.vR.assign(n1, 0.0);
    interpolating_polynomial_vector(1.0, N, s.x.data(), s.wb.data(), s.vR.data());
    interpolating_polynomial_vector(-1.0, N, s.x.data(), s.wb.data(), s.vL.data());
    s.bL.resize(n1); s.bR.resize(n1);
    for (int i = 0; i <= N; ++i) { s.bL[i] = s.vL[i] / s.w[i]; s.bR[i] = s.vR[i] / s.w[i]; }

    s.xCGL.assign(n1, 0.0); s.wbCGL.assign(n1, 0.0); s.DCGL.assign(n1 * n1, 0.0);
    s.TCheb2Gauss.assign(n1 * n1, 0.0);
    if (N != 0)
        for (int i = 0; i <= N; ++i) s.xCGL[i] = -std::cos(1.0 * i * kPi / N);
    barycentric_weights(N, s.xCGL.data(), s.wbCGL.data());
    polynomial_derivative_matrix(N, s.xCGL.data(), s.DCGL.data());
    polynomial_interpolation_matrix(N, N, s.xCGL.data(), s.wbCGL.data(), s.x.data(), s.TCheb2Gauss.data());
    return s;
}

const NodalStorage& nodal_storage(int nodes, int N) {
    static std::mutex mu;
    static std::map<std::pair<int, int>, NodalStorage> cache;
    std::lock_guard<std::mutex> lock(mu);
    auto key = std::make_pair(nodes, N);
    auto it = cache.find(key);
    if (it == cache.end()) it = cache.emplace(key, build_nodal_storage(nodes, N)).first;
    return it->second;
}

// InterpolationMatrices.f90:42-113: prolongation (interpolation) when Norigin < Ndest, otherwise
// the transposed interpolation scaled by w_origin/w_dest (an L2 projection).
std::vector<double> interpolation_matrix(int nodes, int Norigin, int Ndest) {
    const NodalStorage& o = nodal_storage(nodes, Norigin);
    const NodalStorage& d = nodal_storage(nodes, Ndest);
    std::vector<double> T((Ndest + 1) * (Norigin + 1), 0.0);
    if (Norigin < Ndest) {
        polynomial_interpolation_matrix(Norigin, Ndest, o.x.data(), o.wb.data(), d.x.data(), T.data());
    } else {
        std::vector<double> Tt((Norigin + 1) * (Ndest + 1));
        polynomial_interpolation_matrix(Ndest, Norigin, d.x.data(), d.wb.data(), o.x.data(), Tt.data());
        for (int j = 0; j <= Norigin; ++j)
            for (int i = 0; i <= Ndest; ++i)
                T[i * (Norigin + 1) + j] = Tt[j * (Ndest + 1) + i] * o.w[j] / d.w[i];
    }
    return T;
}

}  // namespace h3d
