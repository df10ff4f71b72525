// Host mesh construction. Each routine names the reference routine whose behaviour it follows.
#include "mesh.hpp"

#include <algorithm>
#include <cctype>
#include <cfloat>
#include <cmath>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>

#include "spectral.hpp"

namespace h3d {

namespace {

// localFaceNode(4,6) (HexElementConnectivityDefinitions.f90:69-77), 0-based node numbers.
const int kLocalFaceNode[6][4] = {
    {0, 1, 5, 4},  // FRONT
    {3, 2, 6, 7},  // BACK
    {0, 1, 2, 3},  // BOTTOM
    {1, 2, 6, 5},  // RIGHT
    {4, 5, 6, 7},  // TOP
    {0, 3, 7, 4},  // LEFT
};
// axisMap(2,6): element directions spanned by each side (1-based directions).
const int kAxisMap[6][2] = {{1, 3}, {1, 3}, {1, 2}, {2, 3}, {1, 2}, {2, 3}};

std::string lower(std::string s) {
    for (auto& c : s) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
    return s;
}

inline void vcross(const double u[3], const double v[3], double r[3]) {
    r[0] = u[1] * v[2] - v[1] * u[2];
    r[1] = u[2] * v[0] - v[2] * u[0];
    r[2] = u[0] * v[1] - v[0] * u[1];
}

inline double vnorm(const double v[3]) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

// HexMesh.f90:490-515 faceRotation.
int face_rotation(const int master[4], const int slave[4]) {
    static const int next[4] = {1, 2, 3, 0};
    int j = 0;
    for (j = 0; j < 4; ++j)
        if (master[0] == slave[j]) break;
    if (j == 4) j = 3;  // unreachable for matched faces; mirrors the loop exit value
    if (master[1] == slave[next[j]]) return j;
    return j + 4;
}

// HexMesh.f90:740-800 CompareTwoNodes, called with a fixed coordinate "coord" to skip.
bool compare_two_nodes(const double* x1, const double* x2, int coord) {
    int counter = 0;
    for (int i = 0; i < 3; ++i)
        if (i != coord && almost_equal(x1[i], x2[i])) ++counter;
    return counter >= 2;
}

}  // namespace

// ----------------------------------------------------------------------------- FacePatch --
void FacePatch::construct(const std::vector<double>& u, const std::vector<double>& v,
                          const std::vector<double>& points) {
    nu = static_cast<int>(u.size());
    nv = static_cast<int>(v.size());
    if (nu > kMaxKnots || nv > kMaxKnots) throw std::invalid_argument("face patch order above 31");
    uk = u; vk = v;
    wbu.assign(nu, 0.0); wbv.assign(nv, 0.0);
    Du.assign(nu * nu, 0.0); Dv.assign(nv * nv, 0.0);
    barycentric_weights(nu - 1, uk.data(), wbu.data());
    barycentric_weights(nv - 1, vk.data(), wbv.data());
    polynomial_derivative_matrix(nu - 1, uk.data(), Du.data());
    polynomial_derivative_matrix(nv - 1, vk.data(), Dv.data());
    pts = points;
}

// FacePatchClass.f90:189-268 ComputeFacePoint / ComputePoly2D.
void FacePatch::point(double u1, double u2, double p[3]) const {
    if (is_quad()) {
        for (int j = 0; j < 3; ++j) {
            p[j] = pts[3 * 0 + j] * (1.0 - u1) * (1.0 - u2) + pts[3 * 1 + j] * (1.0 + u1) * (1.0 - u2) +
                   pts[3 * 3 + j] * (1.0 + u1) * (1.0 + u2) + pts[3 * 2 + j] * (1.0 - u1) * (1.0 + u2);
            p[j] = 0.25 * p[j];
        }
        return;
    }
    double li[kMaxKnots], lj[kMaxKnots];
    interpolating_polynomial_vector(u1, nu - 1, uk.data(), wbu.data(), li);
    interpolating_polynomial_vector(u2, nv - 1, vk.data(), wbv.data(), lj);
    p[0] = p[1] = p[2] = 0.0;
    for (int j = 0; j < nv; ++j)
        for (int i = 0; i < nu; ++i)
            for (int c = 0; c < 3; ++c) p[c] = p[c] + pts[3 * (i + nu * j) + c] * li[i] * lj[j];
}

// FacePatchClass.f90:312-418 ComputeFaceDerivative / Compute2DPolyDeriv.
void FacePatch::deriv(double u1, double u2, double g[3][2]) const {
    if (is_quad()) {
        for (int j = 0; j < 3; ++j) {
            g[j][0] = -pts[3 * 0 + j] * (1.0 - u2) + pts[3 * 1 + j] * (1.0 - u2) + pts[3 * 3 + j] * (1.0 + u2) -
                      pts[3 * 2 + j] * (1.0 + u2);
            g[j][1] = -pts[3 * 0 + j] * (1.0 - u1) - pts[3 * 1 + j] * (1.0 + u1) + pts[3 * 3 + j] * (1.0 + u1) +
                      pts[3 * 2 + j] * (1.0 - u1);
            g[j][0] = 0.25 * g[j][0];
            g[j][1] = 0.25 * g[j][1];
        }
        return;
    }
    double li[kMaxKnots], lj[kMaxKnots], dli[kMaxKnots] = {}, dlj[kMaxKnots] = {};
    interpolating_polynomial_vector(u1, nu - 1, uk.data(), wbu.data(), li);
    interpolating_polynomial_vector(u2, nv - 1, vk.data(), wbv.data(), lj);
    for (int i = 0; i < nu; ++i)
        for (int j = 0; j < nu; ++j) dli[i] = dli[i] + Du[j * nu + i] * li[j];
    for (int i = 0; i < nv; ++i)
        for (int j = 0; j < nv; ++j) dlj[i] = dlj[i] + Dv[j * nv + i] * lj[j];
    for (int c = 0; c < 3; ++c) g[c][0] = g[c][1] = 0.0;
    for (int j = 0; j < nv; ++j)
        for (int i = 0; i < nu; ++i)
            for (int c = 0; c < 3; ++c) {
                g[c][0] = g[c][0] + pts[3 * (i + nu * j) + c] * dli[i] * lj[j];
                g[c][1] = g[c][1] + pts[3 * (i + nu * j) + c] * li[i] * dlj[j];
            }
}

// ------------------------------------------------------------------------------- HexMap --
// TransfiniteMaps3D.f90:80-119 constructWithFaces.
void HexMap::set_faces() {
    hex8 = false;
    const double pm[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
    for (int c = 0; c < 4; ++c) {
        faces[2].point(pm[c][0], pm[c][1], corners[c]);
        faces[4].point(pm[c][0], pm[c][1], corners[4 + c]);
    }
}

void HexMap::map_at(const double u[3], double x[3]) const {
    const double xi[3] = {0.5 * (u[0] + 1.0), 0.5 * (u[1] + 1.0), 0.5 * (u[2] + 1.0)};
    if (hex8) {  // TransfiniteMaps3D.f90:186-212 Hex8TransfiniteMap
        for (int j = 0; j < 3; ++j)
            x[j] = corners[0][j] * (1.0 - xi[0]) * (1.0 - xi[1]) * (1.0 - xi[2]) +
                   corners[1][j] * xi[0] * (1.0 - xi[1]) * (1.0 - xi[2]) +
                   corners[2][j] * xi[0] * xi[1] * (1.0 - xi[2]) +
                   corners[3][j] * (1.0 - xi[0]) * xi[1] * (1.0 - xi[2]) +
                   corners[4][j] * (1.0 - xi[0]) * (1.0 - xi[1]) * xi[2] +
                   corners[5][j] * xi[0] * (1.0 - xi[1]) * xi[2] +
                   corners[6][j] * xi[0] * xi[1] * xi[2] +
                   corners[7][j] * (1.0 - xi[0]) * xi[1] * xi[2];
        return;
    }
    // TransfiniteMaps3D.f90:300-448 GeneralHexTransfiniteMap / ComputeHexTransfiniteMap
    double e[12][3], f[6][3];
    faces[0].point(u[0], -1.0, e[0]);
    faces[0].point(1.0, u[2], e[1]);
    faces[0].point(u[0], 1.0, e[2]);
    faces[0].point(-1.0, u[2], e[3]);
    faces[1].point(u[0], -1.0, e[4]);
    faces[1].point(1.0, u[2], e[5]);
    faces[1].point(u[0], 1.0, e[6]);
    faces[1].point(-1.0, u[2], e[7]);
    faces[3].point(u[1], -1.0, e[9]);
    faces[5].point(u[1], -1.0, e[8]);
    faces[3].point(u[1], 1.0, e[10]);
    faces[5].point(u[1], 1.0, e[11]);
    faces[0].point(u[0], u[2], f[0]);
    faces[1].point(u[0], u[2], f[1]);
    faces[2].point(u[0], u[1], f[2]);
    faces[3].point(u[1], u[2], f[3]);
    faces[4].point(u[0], u[1], f[4]);
    faces[5].point(u[1], u[2], f[5]);
    const double* c[8];
    for (int k = 0; k < 8; ++k) c[k] = corners[k];
    for (int j = 0; j < 3; ++j) {
        x[j] = f[5][j] * (1.0 - xi[0]) + f[3][j] * xi[0] + f[0][j] * (1.0 - xi[1]) + f[1][j] * xi[1] +
               f[2][j] * (1.0 - xi[2]) + f[4][j] * xi[2];
        x[j] = x[j] - e[0][j] * (1.0 - xi[1]) * (1.0 - xi[2]) - e[2][j] * (1.0 - xi[1]) * xi[2] -
               e[4][j] * xi[1] * (1.0 - xi[2]) - e[6][j] * xi[1] * xi[2] -
               e[8][j] * (1.0 - xi[0]) * (1.0 - xi[2]) - e[11][j] * (1.0 - xi[0]) * xi[2] -
               e[9][j] * (1.0 - xi[2]) * xi[0] - e[10][j] * xi[0] * xi[2] -
               e[3][j] * (1.0 - xi[0]) * (1.0 - xi[1]) - e[7][j] * (1.0 - xi[0]) * xi[1] -
               e[1][j] * xi[0] * (1.0 - xi[1]) - e[5][j] * xi[0] * xi[1];
        x[j] = x[j] + c[0][j] * (1.0 - xi[0]) * (1.0 - xi[1]) * (1.0 - xi[2]) +
               c[4][j] * (1.0 - xi[0]) * (1.0 - xi[1]) * xi[2] + c[3][j] * (1.0 - xi[0]) * xi[1] * (1.0 - xi[2]) +
               c[7][j] * (1.0 - xi[0]) * xi[1] * xi[2] + c[1][j] * xi[0] * (1.0 - xi[1]) * (1.0 - xi[2]) +
               c[5][j] * xi[0] * (1.0 - xi[1]) * xi[2] + c[2][j] * xi[0] * xi[1] * (1.0 - xi[2]) +
               c[6][j] * xi[0] * xi[1] * xi[2];
    }
}

void HexMap::grad_at(const double u[3], double g[3][3]) const {
    const double xi[3] = {0.5 * (u[0] + 1.0), 0.5 * (u[1] + 1.0), 0.5 * (u[2] + 1.0)};
    if (hex8) {  // TransfiniteMaps3D.f90:230-281 GradHex8TransfiniteMap
        for (int i = 0; i < 3; ++i) {
            const double c1 = corners[0][i], c2 = corners[1][i], c3 = corners[2][i], c4 = corners[3][i];
            const double c5 = corners[4][i], c6 = corners[5][i], c7 = corners[6][i], c8 = corners[7][i];
            g[i][0] = -c1 * (1.0 - xi[1]) * (1.0 - xi[2]) + c2 * (1.0 - xi[1]) * (1.0 - xi[2]) +
                      c3 * xi[1] * (1.0 - xi[2]) - c4 * xi[1] * (1.0 - xi[2]) - c5 * (1.0 - xi[1]) * xi[2] +
                      c6 * (1.0 - xi[1]) * xi[2] + c7 * xi[1] * xi[2] - c8 * xi[1] * xi[2];
            g[i][1] = -c1 * (1.0 - xi[0]) * (1.0 - xi[2]) - c2 * xi[0] * (1.0 - xi[2]) +
                      c3 * xi[0] * (1.0 - xi[2]) + c4 * (1.0 - xi[0]) * (1.0 - xi[2]) -
                      c5 * (1.0 - xi[0]) * xi[2] - c6 * xi[0] * xi[2] + c7 * xi[0] * xi[2] +
                      c8 * (1.0 - xi[0]) * xi[2];
            g[i][2] = -c1 * (1.0 - xi[0]) * (1.0 - xi[1]) - c2 * xi[0] * (1.0 - xi[1]) - c3 * xi[0] * xi[1] -
                      c4 * (1.0 - xi[0]) * xi[1] + c5 * (1.0 - xi[0]) * (1.0 - xi[1]) +
                      c6 * xi[0] * (1.0 - xi[1]) + c7 * xi[0] * xi[1] + c8 * (1.0 - xi[0]) * xi[1];
        }
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) g[i][j] = 0.5 * g[i][j];
        return;
    }
    // TransfiniteMaps3D.f90:468-739 GradGeneralHexTransfiniteMap / ComputeGradHexTransfiniteMap
    double e[12][3], ed[12][3], f[6][3], fd[6][3][2], g2[3][2];
    faces[0].point(u[0], -1.0, e[0]);
    faces[0].point(1.0, u[2], e[1]);
    faces[0].point(u[0], 1.0, e[2]);
    faces[0].point(-1.0, u[2], e[3]);
    faces[1].point(u[0], -1.0, e[4]);
    faces[1].point(1.0, u[2], e[5]);
    faces[1].point(u[0], 1.0, e[6]);
    faces[1].point(-1.0, u[2], e[7]);
    faces[3].point(u[1], -1.0, e[9]);
    faces[5].point(u[1], -1.0, e[8]);
    faces[3].point(u[1], 1.0, e[10]);
    faces[5].point(u[1], 1.0, e[11]);
    faces[0].point(u[0], u[2], f[0]);
    faces[1].point(u[0], u[2], f[1]);
    faces[2].point(u[0], u[1], f[2]);
    faces[3].point(u[1], u[2], f[3]);
    faces[4].point(u[0], u[1], f[4]);
    faces[5].point(u[1], u[2], f[5]);
    auto edge_der = [&](int face, double a, double b, int comp, int idx) {
        faces[face].deriv(a, b, g2);
        for (int c = 0; c < 3; ++c) ed[idx][c] = g2[c][comp];
    };
    edge_der(0, u[0], -1.0, 0, 0);
    edge_der(0, 1.0, u[2], 1, 1);
    edge_der(0, u[0], 1.0, 0, 2);
    edge_der(0, -1.0, u[2], 1, 3);
    edge_der(1, u[0], -1.0, 0, 4);
    edge_der(1, 1.0, u[2], 1, 5);
    edge_der(1, u[0], 1.0, 0, 6);
    edge_der(1, -1.0, u[2], 1, 7);
    edge_der(5, u[1], -1.0, 0, 8);
    edge_der(3, u[1], -1.0, 0, 9);
    edge_der(3, u[1], 1.0, 0, 10);
    edge_der(5, u[1], 1.0, 0, 11);
    const double fu[6][2] = {{u[0], u[2]}, {u[0], u[2]}, {u[0], u[1]}, {u[1], u[2]}, {u[0], u[1]}, {u[1], u[2]}};
    for (int k = 0; k < 6; ++k) {
        faces[k].deriv(fu[k][0], fu[k][1], g2);
        for (int c = 0; c < 3; ++c) { fd[k][c][0] = 2.0 * g2[c][0]; fd[k][c][1] = 2.0 * g2[c][1]; }
    }
    for (int k = 0; k < 12; ++k)
        for (int c = 0; c < 3; ++c) ed[k][c] = 2.0 * ed[k][c];
    const double* c[8];
    for (int k = 0; k < 8; ++k) c[k] = corners[k];
    for (int j = 0; j < 3; ++j) {
        double a = -f[5][j] + f[3][j] + fd[0][j][0] * (1.0 - xi[1]) + fd[1][j][0] * xi[1] +
                   fd[2][j][0] * (1.0 - xi[2]) + fd[4][j][0] * xi[2];
        a = a - ed[0][j] * (1.0 - xi[1]) * (1.0 - xi[2]) - ed[2][j] * (1.0 - xi[1]) * xi[2] -
            ed[4][j] * xi[1] * (1.0 - xi[2]) - ed[6][j] * xi[1] * xi[2] + e[8][j] * (1.0 - xi[2]) +
            e[11][j] * xi[2] - e[9][j] * (1.0 - xi[2]) - e[10][j] * xi[2] + e[3][j] * (1.0 - xi[1]) +
            e[7][j] * xi[1] - e[1][j] * (1.0 - xi[1]) - e[5][j] * xi[1];
        a = a - c[0][j] * (1.0 - xi[1]) * (1.0 - xi[2]) - c[4][j] * (1.0 - xi[1]) * xi[2] -
            c[3][j] * xi[1] * (1.0 - xi[2]) - c[7][j] * xi[1] * xi[2] + c[1][j] * (1.0 - xi[1]) * (1.0 - xi[2]) +
            c[5][j] * (1.0 - xi[1]) * xi[2] + c[2][j] * xi[1] * (1.0 - xi[2]) + c[6][j] * xi[1] * xi[2];
        g[j][0] = a;

        double b = fd[5][j][0] * (1.0 - xi[0]) + fd[3][j][0] * xi[0] - f[0][j] + f[1][j] +
                   fd[2][j][1] * (1.0 - xi[2]) + fd[4][j][1] * xi[2];
        b = b + e[0][j] * (1.0 - xi[2]) + e[2][j] * xi[2] - e[4][j] * (1.0 - xi[2]) - e[6][j] * xi[2] -
            ed[8][j] * (1.0 - xi[0]) * (1.0 - xi[2]) - ed[11][j] * (1.0 - xi[0]) * xi[2] -
            ed[9][j] * (1.0 - xi[2]) * xi[0] - ed[10][j] * xi[0] * xi[2] + e[3][j] * (1.0 - xi[0]) -
            e[7][j] * (1.0 - xi[0]) + e[1][j] * xi[0] - e[5][j] * xi[0];
        b = b - c[0][j] * (1.0 - xi[0]) * (1.0 - xi[2]) - c[4][j] * (1.0 - xi[0]) * xi[2] +
            c[3][j] * (1.0 - xi[0]) * (1.0 - xi[2]) + c[7][j] * (1.0 - xi[0]) * xi[2] -
            c[1][j] * xi[0] * (1.0 - xi[2]) - c[5][j] * xi[0] * xi[2] + c[2][j] * xi[0] * (1.0 - xi[2]) +
            c[6][j] * xi[0] * xi[2];
        g[j][1] = b;

        double d = fd[5][j][1] * (1.0 - xi[0]) + fd[3][j][1] * xi[0] + fd[0][j][1] * (1.0 - xi[1]) +
                   fd[1][j][1] * xi[1] - f[2][j] + f[4][j];
        d = d + e[0][j] * (1.0 - xi[1]) - e[2][j] * (1.0 - xi[1]) + e[4][j] * xi[1] - e[6][j] * xi[1] +
            e[8][j] * (1.0 - xi[0]) - e[11][j] * (1.0 - xi[0]) + e[9][j] * xi[0] - e[10][j] * xi[0] -
            ed[3][j] * (1.0 - xi[0]) * (1.0 - xi[1]) - ed[7][j] * (1.0 - xi[0]) * xi[1] -
            ed[1][j] * xi[0] * (1.0 - xi[1]) - ed[5][j] * xi[0] * xi[1];
        d = d - c[0][j] * (1.0 - xi[0]) * (1.0 - xi[1]) + c[4][j] * (1.0 - xi[0]) * (1.0 - xi[1]) -
            c[3][j] * (1.0 - xi[0]) * xi[1] + c[7][j] * (1.0 - xi[0]) * xi[1] - c[1][j] * xi[0] * (1.0 - xi[1]) +
            c[5][j] * xi[0] * (1.0 - xi[1]) - c[2][j] * xi[0] * xi[1] + c[6][j] * xi[0] * xi[1];
        g[j][2] = d;
    }
    const double eps = 100.0 * DBL_EPSILON;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            g[i][j] = 0.5 * g[i][j];
            if (std::fabs(g[i][j]) <= eps) g[i][j] = 0.0;
        }
}

// ----------------------------------------------------------------------------- sources --
std::vector<std::pair<std::string, std::string>> parse_periodic(const std::string& spec) {
    std::vector<std::pair<std::string, std::string>> out;
    std::stringstream ss(spec);
    std::string item;
    while (std::getline(ss, item, ',')) {
        const auto pos = item.find(':');
        if (pos == std::string::npos) continue;
        auto trim = [](std::string s) {
            s.erase(0, s.find_first_not_of(" \t"));
            s.erase(s.find_last_not_of(" \t") + 1);
            return s;
        };
        out.emplace_back(lower(trim(item.substr(0, pos))), lower(trim(item.substr(pos + 1))));
    }
    return out;
}

static FacePatch flat_patch(const double* p1, const double* p2, const double* p3, const double* p4) {
    // valuesFlat(:,1,1)=p1, (:,2,1)=p2, (:,2,2)=p3, (:,1,2)=p4 (Read_SpecMesh.f90:176-221)
    std::vector<double> pts(12);
    for (int c = 0; c < 3; ++c) {
        pts[3 * 0 + c] = p1[c];
        pts[3 * 1 + c] = p2[c];
        pts[3 * 3 + c] = p3[c];
        pts[3 * 2 + c] = p4[c];
    }
    FacePatch f;
    f.construct({-1.0, 1.0}, {-1.0, 1.0}, pts);
    return f;
}

// Fortran list-directed input as the SpecMesh reader uses it: every READ statement starts at a new
// record (line), takes its values from as many records as it needs and skips the rest of its last
// record (so element records with more face flags than the six read are accepted).
template <typename T>
static bool read_record(std::istream& in, T* v, int n) {
    int got = 0;
    std::string line;
    while (got < n) {
        if (!std::getline(in, line)) return false;
        std::istringstream ls(line);
        while (got < n && (ls >> v[got])) ++got;
    }
    return true;
}

// Read_SpecMesh.f90:36-342 (serial path): header, nodes, element records with optional curved
// face patches given at Chebyshev-Lobatto knots, boundary names.
bool read_specmesh(const std::string& path, MeshSource& src, std::string& err) {
    std::ifstream in(path);
    if (!in) { err = "cannot open mesh file " + path; return false; }
    int head[3] = {0, 0, 0};
    if (!read_record(in, head, 3)) { err = "bad SpecMesh header"; return false; }
    const int nNodes = head[0], nElem = head[1], bOrder = head[2];
    if (nNodes < 8 || nElem < 1 || bOrder < 1) { err = "bad SpecMesh header"; return false; }
    src.bface_order = bOrder;
    const int nb = bOrder + 1;
    std::vector<double> knots(nb);
    for (int i = 0; i < nb; ++i) knots[i] = -std::cos((i * 1.0) * kPi / (nb - 1.0));
    src.nodes.resize(3 * static_cast<size_t>(nNodes));
    for (int j = 0; j < nNodes; ++j)
        if (!read_record(in, &src.nodes[3 * j], 3)) { err = "bad node record"; return false; }
    src.elem_nodes.resize(8 * static_cast<size_t>(nElem));
    src.maps.assign(nElem, HexMap());
    src.bnames.assign(6 * static_cast<size_t>(nElem), "---");
    for (int l = 0; l < nElem; ++l) {
        int ids[8], flags[6];
        if (!read_record(in, ids, 8) || !read_record(in, flags, 6)) { err = "bad element record"; return false; }
        for (int k = 0; k < 8; ++k) {
            if (ids[k] < 1 || ids[k] > nNodes) { err = "element node id out of range"; return false; }
            src.elem_nodes[8 * l + k] = ids[k] - 1;
        }
        HexMap& m = src.maps[l];
        const int maxflag = *std::max_element(flags, flags + 6);
        if (maxflag == 0) {
            m.hex8 = true;
            for (int k = 0; k < 8; ++k)
                for (int c = 0; c < 3; ++c) m.corners[k][c] = src.nodes[3 * src.elem_nodes[8 * l + k] + c];
        } else {
            for (int k = 0; k < 6; ++k) {
                if (flags[k] == 0) {
                    const double* p[4];
                    for (int q = 0; q < 4; ++q) p[q] = &src.nodes[3 * src.elem_nodes[8 * l + kLocalFaceNode[k][q]]];
                    m.faces[k] = flat_patch(p[0], p[1], p[2], p[3]);
                } else {
                    std::vector<double> pts(3 * nb * nb);
                    for (int j = 0; j < nb; ++j)
                        for (int i = 0; i < nb; ++i)
                            if (!read_record(in, &pts[3 * (i + nb * j)], 3)) {
                                err = "bad face patch record"; return false;
                            }
                    m.faces[k].construct(knots, knots, pts);
                }
            }
            m.set_faces();
        }
        std::string names[6];
        if (!read_record(in, names, 6)) { err = "truncated SpecMesh file"; return false; }
        for (int k = 0; k < 6; ++k) src.bnames[6 * l + k] = lower(names[k]);
    }
    return true;
}

// Structured periodic box; node (i,j,k) has id i + (nx+1)*(j + (ny+1)*k). Elements are numbered
// with i fastest. Side names: front/back (y), bottom/top (z), left/right (x).
void box_source(int nx, int ny, int nz, const double lo[3], const double hi[3], double warp,
                int patch_order, MeshSource& src) {
    const int n[3] = {nx, ny, nz};
    auto coord = [&](int d, int i) { return (i == n[d]) ? hi[d] : lo[d] + (hi[d] - lo[d]) * i / n[d]; };
    // sin() of a coordinate, exactly zero on the box planes so that periodic partners coincide.
    auto s = [&](int d, double v) { return (v == lo[d] || v == hi[d]) ? 0.0 : std::sin(v); };
    auto warp_point = [&](const double in[3], double out[3]) {
        const double w = warp * s(0, in[0]) * s(1, in[1]) * s(2, in[2]);
        for (int c = 0; c < 3; ++c) out[c] = in[c] + w;
    };
    const int nn = (nx + 1) * (ny + 1) * (nz + 1);
    src.nodes.resize(3 * static_cast<size_t>(nn));
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i <= nx; ++i) {
                const double p[3] = {coord(0, i), coord(1, j), coord(2, k)};
                warp_point(p, &src.nodes[3 * (i + (nx + 1) * (j + (ny + 1) * k))]);
            }
    const int K = nx * ny * nz;
    src.elem_nodes.resize(8 * static_cast<size_t>(K));
    src.maps.assign(K, HexMap());
    src.bnames.assign(6 * static_cast<size_t>(K), "---");
    const bool curved = patch_order >= 2;
    src.bface_order = curved ? patch_order : 1;
    std::vector<double> knots;
    if (curved) {
        knots.resize(patch_order + 1);
        for (int i = 0; i <= patch_order; ++i) knots[i] = -std::cos((i * 1.0) * kPi / patch_order);
    }
    auto nid = [&](int i, int j, int k) { return i + (nx + 1) * (j + (ny + 1) * k); };
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int e = i + nx * (j + ny * k);
                const int ids[8] = {nid(i, j, k),         nid(i + 1, j, k),         nid(i + 1, j + 1, k),
                                    nid(i, j + 1, k),     nid(i, j, k + 1),         nid(i + 1, j, k + 1),
                                    nid(i + 1, j + 1, k + 1), nid(i, j + 1, k + 1)};
                for (int q = 0; q < 8; ++q) src.elem_nodes[8 * e + q] = ids[q];
                if (j == 0) src.bnames[6 * e + 0] = "front";
                if (j == ny - 1) src.bnames[6 * e + 1] = "back";
                if (k == 0) src.bnames[6 * e + 2] = "bottom";
                if (i == nx - 1) src.bnames[6 * e + 3] = "right";
                if (k == nz - 1) src.bnames[6 * e + 4] = "top";
                if (i == 0) src.bnames[6 * e + 5] = "left";
                HexMap& m = src.maps[e];
                if (!curved) {
                    m.hex8 = true;
                    for (int q = 0; q < 8; ++q)
                        for (int c = 0; c < 3; ++c) m.corners[q][c] = src.nodes[3 * ids[q] + c];
                    continue;
                }
                // Undeformed element box, then warped patch points at the CGL knots.
                const double x0[3] = {coord(0, i), coord(1, j), coord(2, k)};
                const double x1[3] = {coord(0, i + 1), coord(1, j + 1), coord(2, k + 1)};
                auto ref_to_phys = [&](double a, double b, double c, double out[3]) {
                    const double r[3] = {a, b, c};
                    double p[3];
                    for (int d = 0; d < 3; ++d) {
                        if (r[d] == -1.0) p[d] = x0[d];
                        else if (r[d] == 1.0) p[d] = x1[d];
                        else p[d] = x0[d] + 0.5 * (r[d] + 1.0) * (x1[d] - x0[d]);
                    }
                    warp_point(p, out);
                };
                const int nb = patch_order + 1;
                for (int f = 0; f < 6; ++f) {
                    std::vector<double> pts(3 * nb * nb);
                    for (int jj = 0; jj < nb; ++jj)
                        for (int ii = 0; ii < nb; ++ii) {
                            const double a = knots[ii], b = knots[jj];
                            double* out = &pts[3 * (ii + nb * jj)];
                            switch (f) {
                                case 0: ref_to_phys(a, -1.0, b, out); break;
                                case 1: ref_to_phys(a, 1.0, b, out); break;
                                case 2: ref_to_phys(a, b, -1.0, out); break;
                                case 3: ref_to_phys(1.0, a, b, out); break;
                                case 4: ref_to_phys(a, b, 1.0, out); break;
                                default: ref_to_phys(-1.0, a, b, out); break;
                            }
                        }
                    m.faces[f].construct(knots, knots, pts);
                }
                m.set_faces();
            }
}

// --------------------------------------------------------------------------- geometry ----
namespace {

// MappedGeometry.f90:174-386 computeMetricTermsConservativeForm, element e of orders (Nx,Ny,Nz).
void element_geometry(const HexMap& map, int nodes, int Nx, int Ny, int Nz, double* x, double* jaXi,
                      double* jaEta, double* jaZeta, double* jac, double* invJac) {
    const NodalStorage& sx = nodal_storage(nodes, Nx);
    const NodalStorage& sy = nodal_storage(nodes, Ny);
    const NodalStorage& sz = nodal_storage(nodes, Nz);
    const int px = Nx + 1, py = Ny + 1, pz = Nz + 1, np = px * py * pz;
    auto id = [&](int i, int j, int k) { return i + px * (j + py * k); };
    for (int k = 0; k < pz; ++k)
        for (int j = 0; j < py; ++j)
            for (int i = 0; i < px; ++i) {
                const double u[3] = {sx.x[i], sy.x[j], sz.x[k]};
                map.map_at(u, &x[3 * id(i, j, k)]);
            }
    std::vector<double> xc(3 * np), gx(9 * np);  // gx[9*n + 3*r + c] = grad_x(r+1, c+1)
    for (int k = 0; k < pz; ++k)
        for (int j = 0; j < py; ++j)
            for (int i = 0; i < px; ++i) {
                const double u[3] = {sx.xCGL[i], sy.xCGL[j], sz.xCGL[k]};
                const int n = id(i, j, k);
                map.map_at(u, &xc[3 * n]);
                double g[3][3];
                map.grad_at(u, g);
                for (int r = 0; r < 3; ++r)
                    for (int c = 0; c < 3; ++c) gx[9 * n + 3 * r + c] = g[r][c];
            }
    std::vector<double> cp(3 * np), aux(9 * np), Ja[3];  // aux[9n + 3*d + m] = auxgrad(m, d)
    for (int a = 0; a < 3; ++a) Ja[a].assign(3 * np, 0.0);
    // The three passes build the x-, y- and z-components of Ja^1, Ja^2, Ja^3.
    const int l1[3] = {2, 0, 1}, l2[3] = {1, 2, 0};
    for (int comp = 0; comp < 3; ++comp) {
        for (int n = 0; n < np; ++n)
            for (int m = 0; m < 3; ++m)
                cp[3 * n + m] = xc[3 * n + l1[comp]] * gx[9 * n + 3 * l2[comp] + m] -
                                xc[3 * n + l2[comp]] * gx[9 * n + 3 * l1[comp] + m];
        std::fill(aux.begin(), aux.end(), 0.0);
        for (int k = 0; k < pz; ++k)
            for (int j = 0; j < py; ++j)
                for (int i = 0; i < px; ++i) {
                    double* A = &aux[9 * id(i, j, k)];
                    for (int l = 0; l < px; ++l)
                        for (int m = 0; m < 3; ++m) A[0 * 3 + m] = A[0 * 3 + m] + cp[3 * id(l, j, k) + m] * sx.DCGL[i * px + l];
                    for (int l = 0; l < py; ++l)
                        for (int m = 0; m < 3; ++m) A[1 * 3 + m] = A[1 * 3 + m] + cp[3 * id(i, l, k) + m] * sy.DCGL[j * py + l];
                    for (int l = 0; l < pz; ++l)
                        for (int m = 0; m < 3; ++m) A[2 * 3 + m] = A[2 * 3 + m] + cp[3 * id(i, j, l) + m] * sz.DCGL[k * pz + l];
                }
        for (int n = 0; n < np; ++n) {
            const double* A = &aux[9 * n];
            auto ag = [&](int m, int d) { return A[3 * (d - 1) + (m - 1)]; };  // auxgrad(m,d)
            const double J1 = ag(3, 2) - ag(2, 3);
            const double J2 = ag(1, 3) - ag(3, 1);
            const double J3 = ag(2, 1) - ag(1, 2);
            Ja[0][3 * n + comp] = -0.5 * J1;
            Ja[1][3 * n + comp] = -0.5 * J2;
            Ja[2][3 * n + comp] = -0.5 * J3;
        }
    }
    std::vector<double> jc(np);
    for (int n = 0; n < np; ++n) {
        const double a1[3] = {gx[9 * n + 0], gx[9 * n + 3], gx[9 * n + 6]};
        const double a2[3] = {gx[9 * n + 1], gx[9 * n + 4], gx[9 * n + 7]};
        const double a3[3] = {gx[9 * n + 2], gx[9 * n + 5], gx[9 * n + 8]};
        double v[3];
        vcross(a2, a3, v);
        jc[n] = a1[0] * v[0] + a1[1] * v[1] + a1[2] * v[2];
    }
    double* out[3] = {jaXi, jaEta, jaZeta};
    for (int k = 0; k < pz; ++k)
        for (int j = 0; j < py; ++j)
            for (int i = 0; i < px; ++i) {
                const int t = id(i, j, k);
                for (int a = 0; a < 3; ++a)
                    for (int c = 0; c < 3; ++c) out[a][3 * t + c] = 0.0;
                jac[t] = 0.0;
                for (int nn = 0; nn < pz; ++nn)
                    for (int mm = 0; mm < py; ++mm)
                        for (int ll = 0; ll < px; ++ll) {
                            const int s = id(ll, mm, nn);
                            const double tx = sx.TCheb2Gauss[i * px + ll], ty = sy.TCheb2Gauss[j * py + mm],
                                         tz = sz.TCheb2Gauss[k * pz + nn];
                            for (int a = 0; a < 3; ++a)
                                for (int c = 0; c < 3; ++c)
                                    out[a][3 * t + c] = out[a][3 * t + c] + Ja[a][3 * s + c] * tx * ty * tz;
                            jac[t] = jac[t] + jc[s] * tx * ty * tz;
                        }
            }
    for (int n = 0; n < np; ++n) invJac[n] = 1.0 / jac[n];
}

}  // namespace

// ------------------------------------------------------------------------ build_mesh ----
bool build_mesh(const MeshSource& src, int node_type, const std::vector<int32_t>& orders,
                const std::vector<std::pair<std::string, std::string>>& periodic, Mesh& out,
                std::string& err) {
    const int K = static_cast<int>(src.elem_nodes.size() / 8);
    if (static_cast<int>(orders.size()) != 3 * K) { err = "orders must hold 3 entries per element"; return false; }
    for (int v : orders)
        if (v < 1 || v > 12) { err = "polynomial orders must lie in 1..12"; return false; }
    out = Mesh();
    out.K = K;
    out.node_type = node_type;
    out.order = orders;

    // ---- faces (HexMesh.f90:356-432 ConstructFaces) ------------------------------------
    struct F {
        int nodes[4];
        int elem[2] = {-1, -1}, side[2] = {0, 0};
        int rot = 0;
        bool interior = false, deleted = false;
        std::string bname;
    };
    std::vector<F> faces;
    std::map<std::array<int, 4>, int> table;
    for (int e = 0; e < K; ++e)
        for (int s = 0; s < 6; ++s) {
            int fn[4];
            for (int q = 0; q < 4; ++q) fn[q] = src.elem_nodes[8 * e + kLocalFaceNode[s][q]];
            std::array<int, 4> key = {fn[0], fn[1], fn[2], fn[3]};
            std::sort(key.begin(), key.end());
            auto it = table.find(key);
            if (it != table.end()) {
                F& f = faces[it->second];
                f.elem[1] = e;
                f.side[1] = s + 1;
                f.interior = true;
                f.rot = face_rotation(f.nodes, fn);
            } else {
                F f;
                for (int q = 0; q < 4; ++q) f.nodes[q] = fn[q];
                f.elem[0] = e;
                f.side[0] = s + 1;
                f.bname = src.bnames[6 * e + s];
                table.emplace(key, static_cast<int>(faces.size()));
                faces.push_back(f);
            }
        }

    // ---- periodic faces (HexMesh.f90:519-736 ConstructPeriodicFaces) -------------------
    const double* X = src.nodes.data();
    for (const auto& pr : periodic) {
        int coord = -1;
        std::vector<int> plus, minus;
        for (int i = 0; i < static_cast<int>(faces.size()); ++i) {
            if (faces[i].interior) continue;
            if (faces[i].bname == pr.first) plus.push_back(i);
            else if (faces[i].bname == pr.second) minus.push_back(i);
        }
        for (int i : plus) {
            if (faces[i].interior) continue;
            bool found = false;
            for (int j : minus) {
                if (faces[j].interior || faces[j].deleted) continue;
                bool mm[4] = {false, false, false, false};
                int use_coord = coord;
                auto try_coord = [&](int cc) {
                    bool sm[4] = {false, false, false, false};
                    for (int q = 0; q < 4; ++q) mm[q] = false;
                    for (int k = 0; k < 4; ++k) {
                        for (int l = 0; l < 4; ++l) {
                            if (sm[l]) continue;
                            if (compare_two_nodes(X + 3 * faces[i].nodes[k], X + 3 * faces[j].nodes[l], cc)) {
                                mm[k] = true; sm[l] = true; break;
                            }
                        }
                        if (!mm[k]) return false;
                    }
                    return true;
                };
                bool ok = false;
                if (coord < 0) {
                    for (int cc = 0; cc < 3 && !ok; ++cc)
                        if (try_coord(cc)) { ok = true; use_coord = cc; }
                } else {
                    ok = try_coord(coord);
                }
                if (!ok) continue;
                coord = use_coord;
                F& f = faces[i];
                f.elem[1] = faces[j].elem[0];
                f.side[1] = faces[j].side[0];
                f.interior = true;
                f.bname = "---";
                int slave[4] = {-1, -1, -1, -1};
                for (int k = 0; k < 4; ++k)
                    for (int l = 0; l < 4; ++l)
                        if (compare_two_nodes(X + 3 * f.nodes[k], X + 3 * faces[j].nodes[l], coord))
                            slave[l] = f.nodes[k];
                f.rot = face_rotation(f.nodes, slave);
                faces[j].deleted = true;
                found = true;
                break;
            }
            if (!found) {
                err = "periodic face of zone '" + pr.first + "' found no partner in '" + pr.second + "'";
                return false;
            }
        }
    }

    // ---- compact, element -> face tables (DeletePeriodicMinusFaces, GetElementsFaceIDs) ----
    // Faces left without a partner are boundary faces of their zone (HexMesh.f90:433-480,
    // ConstructZones): one element, normal pointing out of the domain.
    std::vector<F> kept;
    for (auto& f : faces)
        if (!f.deleted) kept.push_back(f);
    out.F = static_cast<int>(kept.size());
    out.face_elem.resize(2 * out.F);
    out.face_side.resize(2 * out.F);
    out.face_rot.resize(out.F);
    out.face_nf.resize(2 * out.F);
    out.face_zone.assign(out.F, -1);
    out.elem_face.assign(6 * K, -1);
    out.elem_face_side.assign(6 * K, 0);
    out.n_boundary_faces = 0;
    for (int f = 0; f < out.F; ++f) {
        for (int s = 0; s < 2; ++s) {
            out.face_elem[2 * f + s] = kept[f].elem[s];
            out.face_side[2 * f + s] = kept[f].side[s];
            if (kept[f].elem[s] < 0) continue;
            out.elem_face[6 * kept[f].elem[s] + kept[f].side[s] - 1] = f;
            out.elem_face_side[6 * kept[f].elem[s] + kept[f].side[s] - 1] = s + 1;
        }
        out.face_rot[f] = kept[f].rot;
        if (!kept[f].interior) {
            const std::string& name = kept[f].bname;
            if (name.empty() || name == "---") {
                err = "a boundary face of element " + std::to_string(kept[f].elem[0] + 1) + " has no zone name";
                return false;
            }
            int z = 0;
            while (z < static_cast<int>(out.zone_names.size()) && out.zone_names[z] != name) ++z;
            if (z == static_cast<int>(out.zone_names.size())) out.zone_names.push_back(name);
            out.face_zone[f] = z;
            ++out.n_boundary_faces;
        }
    }

    // ---- face orders (HexMesh.f90:2420-2480, FaceClass.f90:187-276 Face_LinkWithElements) ----
    std::vector<int> NfLeft(2 * out.F), NfRight(2 * out.F);
    for (int f = 0; f < out.F; ++f) {
        const int eL = out.face_elem[2 * f], eR = out.face_elem[2 * f + 1];
        const int sL = out.face_side[2 * f] - 1, sR = out.face_side[2 * f + 1] - 1;
        int NelL[2], NelR[2];
        for (int a = 0; a < 2; ++a) {
            NelL[a] = orders[3 * eL + kAxisMap[sL][a] - 1];
            NelR[a] = eR >= 0 ? orders[3 * eR + kAxisMap[sR][a] - 1] : NelL[a];
        }
        NfLeft[2 * f] = NelL[0]; NfLeft[2 * f + 1] = NelL[1];
        if (eR < 0) {  // boundary faces keep their element's face orders
            NfRight[2 * f] = NelL[0]; NfRight[2 * f + 1] = NelL[1];
            out.face_nf[2 * f] = NelL[0];
            out.face_nf[2 * f + 1] = NelL[1];
            continue;
        }
        switch (out.face_rot[f]) {
            case 0: case 2: case 5: case 7:
                NfRight[2 * f] = NelR[0]; NfRight[2 * f + 1] = NelR[1]; break;
            default:
                NfRight[2 * f] = NelR[1]; NfRight[2 * f + 1] = NelR[0]; break;
        }
        out.face_nf[2 * f] = std::max(NfLeft[2 * f], NfRight[2 * f]);
        out.face_nf[2 * f + 1] = std::max(NfLeft[2 * f + 1], NfRight[2 * f + 1]);
    }

    // ---- curved face patch adaptation (HexMesh.f90:2800-2870), interior faces ----------
    std::vector<HexMap> maps = src.maps;
    auto adapt = [&](HexMap& m, int side, int c1, int c2) {
        FacePatch& p = m.faces[side];
        if (c1 >= p.nu - 1 && c2 >= p.nv - 1) return;
        if (!(c1 < p.nu - 1 || c2 < p.nv - 1)) return;
        const NodalStorage& n1 = nodal_storage(node_type, c1);
        const NodalStorage& n2 = nodal_storage(node_type, c2);
        std::vector<double> pts(3 * (c1 + 1) * (c2 + 1));
        for (int j = 0; j <= c2; ++j)
            for (int i = 0; i <= c1; ++i) p.point(n1.xCGL[i], n2.xCGL[j], &pts[3 * (i + (c1 + 1) * j)]);
        FacePatch q;
        q.construct(n1.xCGL, n2.xCGL, pts);
        p = q;
    };
    for (int f = 0; f < out.F; ++f) {
        const int eL = out.face_elem[2 * f], eR = out.face_elem[2 * f + 1];
        const int sL = out.face_side[2 * f] - 1, sR = out.face_side[2 * f + 1] - 1;
        if (eR < 0) {  // boundary face: the patch is adapted to the element's face orders
            HexMap& m = maps[eL];
            if (m.hex8) continue;
            const int nL[2] = {m.faces[sL].nu - 1, m.faces[sL].nv - 1};
            if (nL[0] == 1 && nL[1] == 1) continue;
            const int CLN[2] = {NfLeft[2 * f], NfLeft[2 * f + 1]};
            if (CLN[0] < nL[0] || CLN[1] < nL[1]) adapt(m, sL, CLN[0], CLN[1]);
            continue;
        }
        HexMap& mL = maps[eL];
        HexMap& mR = maps[eR];
        if (mL.hex8 && mR.hex8) continue;
        const int nL[2] = {mL.hex8 ? 1 : mL.faces[sL].nu - 1, mL.hex8 ? 1 : mL.faces[sL].nv - 1};
        const int nR[2] = {mR.hex8 ? 1 : mR.faces[sR].nu - 1, mR.hex8 ? 1 : mR.faces[sR].nv - 1};
        if (mL.hex8 && nR[0] == 1 && nR[1] == 1) continue;
        if (mR.hex8 && nL[0] == 1 && nL[1] == 1) continue;
        if (nL[0] == 1 && nL[1] == 1 && nR[0] == 1 && nR[1] == 1) continue;
        int CLN[2] = {std::min(NfLeft[2 * f], NfRight[2 * f]), std::min(NfLeft[2 * f + 1], NfRight[2 * f + 1])};
        if (!mL.hex8 && (CLN[0] < nL[0] || CLN[1] < nL[1])) adapt(mL, sL, CLN[0], CLN[1]);
        switch (out.face_rot[f]) {
            case 1: case 3: case 4: case 6: std::swap(CLN[0], CLN[1]); break;
            default: break;
        }
        if (!mR.hex8 && (CLN[0] < nR[0] || CLN[1] < nR[1])) adapt(mR, sR, CLN[0], CLN[1]);
    }
    for (auto& m : maps)
        if (!m.hex8) m.set_faces();

    // ---- element geometry -----------------------------------------------------------------
    out.elem_offset.resize(K + 1);
    out.elem_offset[0] = 0;
    for (int e = 0; e < K; ++e)
        out.elem_offset[e + 1] =
            out.elem_offset[e] + static_cast<int64_t>(orders[3 * e] + 1) * (orders[3 * e + 1] + 1) * (orders[3 * e + 2] + 1);
    const int64_t ndof = out.elem_offset[K];
    out.x.resize(3 * ndof); out.ja_xi.resize(3 * ndof); out.ja_eta.resize(3 * ndof); out.ja_zeta.resize(3 * ndof);
    out.jac.resize(ndof); out.inv_jac.resize(ndof);
#pragma omp parallel for schedule(dynamic)
    for (int e = 0; e < K; ++e) {
        const int64_t o = out.elem_offset[e];
        element_geometry(maps[e], node_type, orders[3 * e], orders[3 * e + 1], orders[3 * e + 2], &out.x[3 * o],
                         &out.ja_xi[3 * o], &out.ja_eta[3 * o], &out.ja_zeta[3 * o], &out.jac[o], &out.inv_jac[o]);
    }
    out.volume = 0.0;
    for (int e = 0; e < K; ++e) {
        const NodalStorage& sx = nodal_storage(node_type, orders[3 * e]);
        const NodalStorage& sy = nodal_storage(node_type, orders[3 * e + 1]);
        const NodalStorage& sz = nodal_storage(node_type, orders[3 * e + 2]);
        const int px = orders[3 * e] + 1, py = orders[3 * e + 1] + 1, pz = orders[3 * e + 2] + 1;
        for (int k = 0; k < pz; ++k)
            for (int j = 0; j < py; ++j)
                for (int i = 0; i < px; ++i)
                    out.volume += sx.w[i] * sy.w[j] * sz.w[k] * out.jac[out.elem_offset[e] + i + px * (j + py * k)];
    }

    // ---- face geometry (MappedGeometry.f90:482-760, left element, eSide=1, rot=0) ----------
    out.face_offset.resize(out.F + 1);
    out.face_offset[0] = 0;
    for (int f = 0; f < out.F; ++f)
        out.face_offset[f + 1] = out.face_offset[f] + static_cast<int64_t>(out.face_nf[2 * f] + 1) * (out.face_nf[2 * f + 1] + 1);
    const int64_t nfp = out.face_offset[out.F];
    out.face_normal.resize(3 * nfp); out.face_t1.resize(3 * nfp); out.face_t2.resize(3 * nfp);
    out.face_jac.resize(nfp); out.face_x.resize(3 * nfp);
#pragma omp parallel for schedule(dynamic)
    for (int f = 0; f < out.F; ++f) {
        const int e = out.face_elem[2 * f];
        const int side = out.face_side[2 * f];
        const int Nf[2] = {out.face_nf[2 * f], out.face_nf[2 * f + 1]};
        const int Nelf[2] = {NfLeft[2 * f], NfLeft[2 * f + 1]};
        const int N3[3] = {orders[3 * e], orders[3 * e + 1], orders[3 * e + 2]};
        const int p3[3] = {N3[0] + 1, N3[1] + 1, N3[2] + 1};
        const int64_t eo = out.elem_offset[e];
        const NodalStorage& f1 = nodal_storage(node_type, Nf[0]);
        const NodalStorage& f2 = nodal_storage(node_type, Nf[1]);
        const HexMap& map = maps[e];
        const int64_t fo = out.face_offset[f];
        const int q1 = Nf[0] + 1, q2 = Nf[1] + 1;
        // face coordinates
        for (int j = 0; j < q2; ++j)
            for (int i = 0; i < q1; ++i) {
                const double a = f1.x[i], b = f2.x[j];
                double u[3];
                switch (side) {
                    case ELEFT: u[0] = -1.0; u[1] = a; u[2] = b; break;
                    case ERIGHT: u[0] = 1.0; u[1] = a; u[2] = b; break;
                    case EBOTTOM: u[0] = a; u[1] = b; u[2] = -1.0; break;
                    case ETOP: u[0] = a; u[1] = b; u[2] = 1.0; break;
                    case EFRONT: u[0] = a; u[1] = -1.0; u[2] = b; break;
                    default: u[0] = a; u[1] = 1.0; u[2] = b; break;
                }
                map.map_at(u, &out.face_x[3 * (fo + i + q1 * j)]);
            }
        // dS on the element face grid (0:Nel(1),0:Nel(2))
        const int n1 = Nelf[0] + 1, n2 = Nelf[1] + 1;
        std::vector<double> dS(3 * n1 * n2, 0.0);
        auto nid = [&](int i, int j, int k) { return eo + i + p3[0] * (j + p3[1] * k); };
        for (int k = 0; k < p3[2]; ++k)
            for (int j = 0; j < p3[1]; ++j)
                for (int i = 0; i < p3[0]; ++i) {
                    const int64_t n = nid(i, j, k);
                    double* d = nullptr;
                    const double* ja = nullptr;
                    double v = 0.0;
                    switch (side) {
                        case ELEFT: d = &dS[3 * (j + n1 * k)]; ja = &out.ja_xi[3 * n]; v = nodal_storage(node_type, N3[0]).vL[i]; break;
                        case ERIGHT: d = &dS[3 * (j + n1 * k)]; ja = &out.ja_xi[3 * n]; v = nodal_storage(node_type, N3[0]).vR[i]; break;
                        case EBOTTOM: d = &dS[3 * (i + n1 * j)]; ja = &out.ja_zeta[3 * n]; v = nodal_storage(node_type, N3[2]).vL[k]; break;
                        case ETOP: d = &dS[3 * (i + n1 * j)]; ja = &out.ja_zeta[3 * n]; v = nodal_storage(node_type, N3[2]).vR[k]; break;
                        case EFRONT: d = &dS[3 * (i + n1 * k)]; ja = &out.ja_eta[3 * n]; v = nodal_storage(node_type, N3[1]).vL[j]; break;
                        default: d = &dS[3 * (i + n1 * k)]; ja = &out.ja_eta[3 * n]; v = nodal_storage(node_type, N3[1]).vR[j]; break;
                    }
                    for (int c = 0; c < 3; ++c) d[c] = d[c] + ja[c] * v;
                }
        if (side == ELEFT || side == EBOTTOM || side == EFRONT)
            for (auto& v : dS) v = -v;
        // projection to the face order (projectionType(1))
        double* nrm = &out.face_normal[3 * fo];
        const bool px = Nelf[0] != Nf[0], py = Nelf[1] != Nf[1];
        if (!px && !py) {
            for (int q = 0; q < 3 * q1 * q2; ++q) nrm[q] = dS[q];
        } else {
            const std::vector<double> T1 = interpolation_matrix(node_type, Nelf[0], Nf[0]);
            const std::vector<double> T2 = interpolation_matrix(node_type, Nelf[1], Nf[1]);
            for (int q = 0; q < 3 * q1 * q2; ++q) nrm[q] = 0.0;
            if (px && !py) {
                for (int j = 0; j < q2; ++j)
                    for (int l = 0; l < n1; ++l)
                        for (int i = 0; i < q1; ++i)
                            for (int c = 0; c < 3; ++c)
                                nrm[3 * (i + q1 * j) + c] += T1[i * n1 + l] * dS[3 * (l + n1 * j) + c];
            } else if (!px && py) {
                for (int l = 0; l < n2; ++l)
                    for (int j = 0; j < q2; ++j)
                        for (int i = 0; i < q1; ++i)
                            for (int c = 0; c < 3; ++c)
                                nrm[3 * (i + q1 * j) + c] += T2[j * n2 + l] * dS[3 * (i + n1 * l) + c];
            } else {
                for (int l = 0; l < n2; ++l)
                    for (int j = 0; j < q2; ++j)
                        for (int m = 0; m < n1; ++m)
                            for (int i = 0; i < q1; ++i)
                                for (int c = 0; c < 3; ++c)
                                    nrm[3 * (i + q1 * j) + c] += T1[i * n1 + m] * T2[j * n2 + l] * dS[3 * (m + n1 * l) + c];
            }
        }
        for (int p = 0; p < q1 * q2; ++p) {
            double* nn = &nrm[3 * p];
            const double J = vnorm(nn);
            out.face_jac[fo + p] = J;
            for (int c = 0; c < 3; ++c) nn[c] = nn[c] / J;
        }
        // tangents: t1 = D x along the first face direction, made orthogonal to n; t2 = n x t1
        double* t1 = &out.face_t1[3 * fo];
        double* t2 = &out.face_t2[3 * fo];
        for (int q = 0; q < 3 * q1 * q2; ++q) t1[q] = 0.0;
        const double* fx = &out.face_x[3 * fo];
        for (int j = 0; j < q2; ++j)
            for (int l = 0; l < q1; ++l)
                for (int i = 0; i < q1; ++i)
                    for (int c = 0; c < 3; ++c)
                        t1[3 * (i + q1 * j) + c] = t1[3 * (i + q1 * j) + c] + f1.D[i * q1 + l] * fx[3 * (l + q1 * j) + c];
        for (int p = 0; p < q1 * q2; ++p) {
            double* a = &t1[3 * p];
            const double* n = &nrm[3 * p];
            const double dot = a[0] * n[0] + a[1] * n[1] + a[2] * n[2];
            for (int c = 0; c < 3; ++c) a[c] = a[c] - dot * n[c];
            const double an = vnorm(a);
            for (int c = 0; c < 3; ++c) a[c] = a[c] / an;
            vcross(n, a, &t2[3 * p]);
        }
    }
    return true;
}

}  // namespace h3d
