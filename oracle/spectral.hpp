// ORACLE -- test infrastructure only (see dg_oracle.cpp). The oracle's own spectral operators and
// index maps, shared by the right-hand side (dg_oracle.cpp) and the mesh geometry (geometry.cpp).
#pragma once
#include <cfloat>
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

namespace orc {

constexpr double PI = 3.141592653589793238462643;
enum { EFRONT = 1, EBACK, EBOTTOM, ERIGHT, ETOP, ELEFT };

// ---------------------------------------------------------------- spectral (own copy) ------
static inline bool almost_equal(double a, double b) {
    const double tol = 2.0 * DBL_EPSILON;
    if (a == 0.0 || b == 0.0) return std::fabs(a - b) <= tol;
    return std::fabs(b - a) <= tol * std::fmax(std::fabs(a), std::fabs(b));
}
static inline void legendre(int N, double x, double& L, double& Lp) {
    if (N == 0) { L = 1.0; Lp = 0.0; return; }
    if (N == 1) { L = x; Lp = 1.0; return; }
    double a = 1.0, ap = 0.0, b = x, bp = 1.0;
    for (int k = 2; k <= N; ++k) {
        L = ((2 * k - 1) * x * b - (k - 1) * a) / k;
        Lp = ap + (2 * k - 1) * b;
        a = b; b = L; ap = bp; bp = Lp;
    }
}
static inline void gauss(int N, double* x, double* w) {  // LegendreAlgorithms.f90:137
    double L, Lp;
    if (N == 0) { x[0] = 0; w[0] = 2; return; }
    if (N == 1) { x[0] = -std::sqrt(1.0 / 3.0); w[0] = 1; x[1] = -x[0]; w[1] = 1; }
    else {
        for (int j = 0; j < (N + 1) / 2; ++j) {
            double xj = -std::cos((2 * j + 1) * PI / (2 * N + 2));
            for (int k = 0; k <= 10; ++k) {
                legendre(N + 1, xj, L, Lp);
                const double d = -L / Lp;
                xj += d;
                if (std::fabs(d) <= 4.0 * DBL_EPSILON * std::fabs(xj)) break;
            }
            legendre(N + 1, xj, L, Lp);
            x[j] = xj; w[j] = 2.0 / ((1.0 - xj * xj) * (Lp * Lp));
            x[N - j] = -xj; w[N - j] = w[j];
        }
    }
    if (N % 2 == 0) { legendre(N + 1, 0.0, L, Lp); x[N / 2] = 0.0; w[N / 2] = 2.0 / (Lp * Lp); }
}
static inline void lobatto(int N, double* x, double* w) {  // LegendreAlgorithms.f90:275
    if (N == 0) { x[0] = 0; w[0] = 2; return; }
    if (N == 1) { x[0] = -1; w[0] = 1; x[1] = 1; w[1] = 1; }
    else {
        x[0] = -1; w[0] = 2.0 / (N * (N + 1)); x[N] = 1; w[N] = w[0];
        for (int j = 1; j <= (N + 1) / 2 - 1; ++j) {
            double xj = -std::cos((j + 0.25) * PI / N - 3.0 / (8 * N * PI * (j + 0.25)));
            double q = 0, qp = 0, LN = 0;
            auto qandl = [&](double xx) {
                double a = 1.0, ap = 0.0, b = xx, bp = 1.0, Lk = 0, Lpk = 0;
                for (int k = 2; k <= N; ++k) {
                    Lk = ((2 * k - 1) * xx * b - (k - 1) * a) / k; Lpk = ap + (2 * k - 1) * b;
                    a = b; b = Lk; ap = bp; bp = Lpk;
                }
                const int k = N + 1;
                Lk = ((2 * k - 1) * xx * b - (k - 1) * a) / k; Lpk = ap + (2 * k - 1) * b;
                q = Lk - a; qp = Lpk - ap; LN = b;
            };
            for (int k = 0; k <= 10; ++k) {
                qandl(xj);
                const double d = -q / qp;
                xj += d;
                if (std::fabs(d) <= 4.0 * DBL_EPSILON * std::fabs(xj)) break;
            }
            qandl(xj);
            x[j] = xj; w[j] = 2.0 / (N * (N + 1) * (LN * LN));
            x[N - j] = -xj; w[N - j] = w[j];
        }
    }
    if (N % 2 == 0) { double L, Lp; legendre(N, 0.0, L, Lp); x[N / 2] = 0; w[N / 2] = 2.0 / (N * (N + 1) * (L * L)); }
}
static inline void bary(int N, const double* x, double* w) {
    for (int j = 0; j <= N; ++j) w[j] = 1.0;
    for (int j = 1; j <= N; ++j)
        for (int k = 0; k < j; ++k) { w[k] *= (x[k] - x[j]); w[j] *= (x[j] - x[k]); }
    for (int j = 0; j <= N; ++j) w[j] = 1.0 / w[j];
}
static inline void lagrange_at(double x, int N, const double* nodes, const double* wb, double* p) {
    bool match = false;
    for (int j = 0; j <= N; ++j) { p[j] = 0.0; if (almost_equal(x, nodes[j])) { p[j] = 1.0; match = true; } }
    if (match) return;
    double d = 0.0;
    for (int j = 0; j <= N; ++j) { const double t = wb[j] / (x - nodes[j]); p[j] = t; d += t; }
    for (int j = 0; j <= N; ++j) p[j] /= d;
}
static inline void interp_matrix(int N, int M, const double* on, const double* wb, const double* nn, double* T) {
    for (int k = 0; k <= M; ++k) {
        bool match = false;
        for (int j = 0; j <= N; ++j) { T[k * (N + 1) + j] = 0.0; if (almost_equal(nn[k], on[j])) { match = true; T[k * (N + 1) + j] = 1.0; } }
        if (!match) {
            double s = 0.0;
            for (int j = 0; j <= N; ++j) { const double t = wb[j] / (nn[k] - on[j]); T[k * (N + 1) + j] = t; s += t; }
            for (int j = 0; j <= N; ++j) T[k * (N + 1) + j] /= s;
        }
    }
}

// PolynomialDerivativeMatrix (InterpolationAndDerivatives.f90:799-828): D(i,j) row-major.
static inline void derivative_matrix(int N, const double* x, double* D) {
    std::vector<double> wb(N + 1);
    bary(N, x, wb.data());
    const int n1 = N + 1;
    for (int i = 0; i <= N; ++i) {
        D[i * n1 + i] = 0.0;
        for (int j = 0; j <= N; ++j)
            if (j != i) {
                D[i * n1 + j] = wb[j] / (wb[i] * (x[i] - x[j]));
                D[i * n1 + i] -= D[i * n1 + j];
            }
    }
}

struct Nodal {  // NodalStorageClass.f90:170-338 (the parts the right-hand side and the geometry use)
    int N;
    std::vector<double> x, w, D, hatD, sharpD, vL, vR, bL, bR;
    std::vector<double> xCGL, DCGL, TCheb2Gauss;  // Chebyshev-Gauss-Lobatto framework (:294-308)
};
// Cached per (nodes, N). Called from OpenMP regions: the lookup is serialised (map nodes are stable,
// so the returned reference stays valid); orc_create fills the cache before any parallel region.
static inline const Nodal& nodal(int nodes, int N) {
    static std::map<std::pair<int, int>, Nodal> cache;
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    auto key = std::make_pair(nodes, N);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    Nodal s;
    s.N = N;
    const int n1 = N + 1;
    s.x.resize(n1); s.w.resize(n1);
    if (nodes == 0) gauss(N, s.x.data(), s.w.data()); else lobatto(N, s.x.data(), s.w.data());
    std::vector<double> wb(n1);
    bary(N, s.x.data(), wb.data());
    s.D.assign(n1 * n1, 0.0);
    for (int i = 0; i <= N; ++i) {  // InterpolationAndDerivatives.f90:799-828
        s.D[i * n1 + i] = 0.0;
        for (int j = 0; j <= N; ++j)
            if (j != i) {
                s.D[i * n1 + j] = wb[j] / (wb[i] * (s.x[i] - s.x[j]));
                s.D[i * n1 + i] -= s.D[i * n1 + j];
            }
    }
    s.hatD.resize(n1 * n1);
    for (int j = 0; j <= N; ++j)
        for (int i = 0; i <= N; ++i) s.hatD[i * n1 + j] = s.D[j * n1 + i] * s.w[j] / s.w[i];
    if (nodes == 1) {
        s.sharpD.resize(n1 * n1);
        for (int k = 0; k < n1 * n1; ++k) s.sharpD[k] = 2.0 * s.D[k];
        s.sharpD[0] = 2.0 * s.D[0] + 1.0 / s.w[0];
        s.sharpD[N * n1 + N] = 2.0 * s.D[N * n1 + N] - 1.0 / s.w[N];
    }
    s.vL.resize(n1); s.vR.resize(n1); s.bL.resize(n1); s.bR.resize(n1);
    lagrange_at(1.0, N, s.x.data(), wb.data(), s.vR.data());
    lagrange_at(-1.0, N, s.x.data(), wb.data(), s.vL.data());
    for (int i = 0; i <= N; ++i) { s.bL[i] = s.vL[i] / s.w[i]; s.bR[i] = s.vR[i] / s.w[i]; }
    s.xCGL.resize(n1);
    for (int i = 0; i <= N; ++i) s.xCGL[i] = N != 0 ? -std::cos(1.0 * i * PI / N) : 0.0;
    s.DCGL.assign(n1 * n1, 0.0);
    derivative_matrix(N, s.xCGL.data(), s.DCGL.data());
    std::vector<double> wbc(n1);
    bary(N, s.xCGL.data(), wbc.data());
    s.TCheb2Gauss.assign(n1 * n1, 0.0);
    interp_matrix(N, N, s.xCGL.data(), wbc.data(), s.x.data(), s.TCheb2Gauss.data());
    return cache.emplace(key, s).first->second;
}
// InterpolationMatrices.f90:42-113: T(0:Nd,0:No) row-major.
static inline std::vector<double> tset(int nodes, int No, int Nd) {
    const Nodal& o = nodal(nodes, No);
    const Nodal& d = nodal(nodes, Nd);
    std::vector<double> T((Nd + 1) * (No + 1));
    std::vector<double> wbo(No + 1), wbd(Nd + 1);
    bary(No, o.x.data(), wbo.data());
    bary(Nd, d.x.data(), wbd.data());
    if (No < Nd) interp_matrix(No, Nd, o.x.data(), wbo.data(), d.x.data(), T.data());
    else {
        std::vector<double> Tt((No + 1) * (Nd + 1));
        interp_matrix(Nd, No, d.x.data(), wbd.data(), o.x.data(), Tt.data());
        for (int j = 0; j <= No; ++j)
            for (int i = 0; i <= Nd; ++i) T[i * (No + 1) + j] = Tt[j * (Nd + 1) + i] * o.w[j] / d.w[i];
    }
    return T;
}

// MeshTypes.f90:70-107 leftIndexes2Right.
static inline void l2r(int i, int j, int Nx, int Ny, int rot, int& ii, int& jj) {
    switch (rot) {
        case 0: ii = i; jj = j; break;
        case 1: ii = Ny - j; jj = i; break;
        case 2: ii = Nx - i; jj = Ny - j; break;
        case 3: ii = j; jj = Nx - i; break;
        case 4: ii = j; jj = i; break;
        case 5: ii = Nx - i; jj = j; break;
        case 6: ii = Ny - j; jj = Nx - i; break;
        default: ii = i; jj = Ny - j; break;
    }
}

}  // namespace orc
