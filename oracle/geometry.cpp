// ORACLE -- test infrastructure only. Nothing in the product links or calls this file.
//
// The oracle's own construction of a periodic hexahedral box mesh and its one-time FP64 geometry,
// restated from the reference so that the product's mesh builder can be checked against an
// independent computation, and so that the CPU reference timing can build its workload without the
// product library:
//   FacePatch evaluation          FacePatchClass.f90:69-110 (construct), :189-268 (ComputeFacePoint,
//                                 ComputePoly2D), :312-418 (ComputeFaceDerivative, Compute2DPolyDeriv)
//   transfinite hexahedral map    TransfiniteMaps3D.f90:38-60 (constructWithFaces), :145-215
//                                 (Hex8TransfiniteMap, GradHex8TransfiniteMap), :240-335
//                                 (GeneralHexTransfiniteMap, ComputeHexTransfiniteMap), :460-640
//                                 (GradGeneralHexTransfiniteMap, ComputeGradHexTransfiniteMap)
//   element metric terms          MappedGeometry.f90:64-135 (ConstructMappedGeometry),
//                                 :174-386 (computeMetricTermsConservativeForm)
//   face geometry                 MappedGeometry.f90:482-760 (ConstructMappedGeometryFace, the left
//                                 element's side, eSide = 1, projection type 0)
//   face list and rotations       HexMesh.f90:356-432 (ConstructFaces: a face is created by the first
//                                 element that reaches it), :490-515 (faceRotation), :519-736
//                                 (ConstructPeriodicFaces: the plus zone's face keeps its place and
//                                 takes the minus zone's element; the minus face is deleted)
//
// The box itself is the benchmark workload's definition: [lo,hi] split into nx*ny*nz hexahedra,
// elements numbered with i fastest, nodes warped by x_c += warp*s(x)s(y)s(z) where s(v) = sin(v)
// except exactly 0 on the box planes, curved faces given as Lagrange patches through the warped
// points at the Chebyshev-Gauss-Lobatto knots of order patch_order (patch_order < 2: straight hex8
// elements from the warped corners). Periodic in all three directions. Uniform order N; patch_order
// must not exceed N (the reference would first re-interpolate the patches to the face order,
// HexMesh.f90:2800-2870, which this builder does not restate).
#include <cmath>
#include <cstdint>
#include <vector>

#include "horses3d_gb300.h"
#include "spectral.hpp"

namespace orc {
namespace {

// FacePatchClass.f90: a Lagrange surface patch through points on a tensor grid of knots.
struct Patch {
    int nu = 0, nv = 0;
    std::vector<double> uk, vk, wbu, wbv, Du, Dv, pts;  // pts[3*(i + nu*j) + c]
    void construct(const std::vector<double>& u, const std::vector<double>& v, const std::vector<double>& points) {
        nu = static_cast<int>(u.size());
        nv = static_cast<int>(v.size());
        uk = u;
        vk = v;
        wbu.resize(nu);
        wbv.resize(nv);
        bary(nu - 1, uk.data(), wbu.data());
        bary(nv - 1, vk.data(), wbv.data());
        Du.resize(nu * nu);
        Dv.resize(nv * nv);
        derivative_matrix(nu - 1, uk.data(), Du.data());
        derivative_matrix(nv - 1, vk.data(), Dv.data());
        pts = points;
    }
    const double* P(int i, int j) const { return &pts[3 * (i + nu * j)]; }
    bool quad() const { return nu == 2 && nv == 2; }  // FaceIs4CorneredQuad
    // ComputeFacePoint
    void point(double u1, double u2, double p[3]) const {
        if (quad()) {
            for (int c = 0; c < 3; ++c)
                p[c] = 0.25 * (P(0, 0)[c] * (1.0 - u1) * (1.0 - u2) + P(1, 0)[c] * (1.0 + u1) * (1.0 - u2) +
                               P(1, 1)[c] * (1.0 + u1) * (1.0 + u2) + P(0, 1)[c] * (1.0 - u1) * (1.0 + u2));
            return;
        }
        std::vector<double> li(nu), lj(nv);
        lagrange_at(u1, nu - 1, uk.data(), wbu.data(), li.data());
        lagrange_at(u2, nv - 1, vk.data(), wbv.data(), lj.data());
        p[0] = p[1] = p[2] = 0.0;
        for (int j = 0; j < nv; ++j)
            for (int i = 0; i < nu; ++i)
                for (int c = 0; c < 3; ++c) p[c] = p[c] + P(i, j)[c] * li[i] * lj[j];
    }
    // ComputeFaceDerivative: g[c][0] = dp_c/du1, g[c][1] = dp_c/du2
    void deriv(double u1, double u2, double g[3][2]) const {
        if (quad()) {
            for (int c = 0; c < 3; ++c) {
                g[c][0] = 0.25 * (-P(0, 0)[c] * (1.0 - u2) + P(1, 0)[c] * (1.0 - u2) + P(1, 1)[c] * (1.0 + u2) -
                                  P(0, 1)[c] * (1.0 + u2));
                g[c][1] = 0.25 * (-P(0, 0)[c] * (1.0 - u1) - P(1, 0)[c] * (1.0 + u1) + P(1, 1)[c] * (1.0 + u1) +
                                  P(0, 1)[c] * (1.0 - u1));
            }
            return;
        }
        std::vector<double> li(nu), lj(nv), dli(nu, 0.0), dlj(nv, 0.0);
        lagrange_at(u1, nu - 1, uk.data(), wbu.data(), li.data());
        lagrange_at(u2, nv - 1, vk.data(), wbv.data(), lj.data());
        for (int i = 0; i < nu; ++i)
            for (int j = 0; j < nu; ++j) dli[i] = dli[i] + Du[j * nu + i] * li[j];
        for (int i = 0; i < nv; ++i)
            for (int j = 0; j < nv; ++j) dlj[i] = dlj[i] + Dv[j * nv + i] * lj[j];
        for (int c = 0; c < 3; ++c) g[c][0] = g[c][1] = 0.0;
        for (int j = 0; j < nv; ++j)
            for (int i = 0; i < nu; ++i)
                for (int c = 0; c < 3; ++c) {
                    g[c][0] = g[c][0] + P(i, j)[c] * dli[i] * lj[j];
                    g[c][1] = g[c][1] + P(i, j)[c] * li[i] * dlj[j];
                }
    }
};

// TransfiniteHexMap: corners (standard FE order) and, for curved elements, six face patches.
struct HexMap {
    bool hex8 = true;
    double corner[8][3] = {};
    Patch face[6];

    // constructWithFaces: the corners are the patches of faces 3 and 5 at their four corners
    void set_corners_from_faces() {
        const double uv[4][2] = {{-1.0, -1.0}, {1.0, -1.0}, {1.0, 1.0}, {-1.0, 1.0}};
        for (int q = 0; q < 4; ++q) {
            face[2].point(uv[q][0], uv[q][1], corner[q]);
            face[4].point(uv[q][0], uv[q][1], corner[4 + q]);
        }
        hex8 = false;
    }

    void map_at(const double u[3], double x[3]) const {
        const double xi[3] = {0.5 * (u[0] + 1.0), 0.5 * (u[1] + 1.0), 0.5 * (u[2] + 1.0)};
        const double a = xi[0], b = xi[1], c = xi[2];
        const double* C[8] = {corner[0], corner[1], corner[2], corner[3], corner[4], corner[5], corner[6], corner[7]};
        if (hex8) {  // Hex8TransfiniteMap
            for (int j = 0; j < 3; ++j)
                x[j] = C[0][j] * (1.0 - a) * (1.0 - b) * (1.0 - c) + C[1][j] * a * (1.0 - b) * (1.0 - c) +
                       C[2][j] * a * b * (1.0 - c) + C[3][j] * (1.0 - a) * b * (1.0 - c) +
                       C[4][j] * (1.0 - a) * (1.0 - b) * c + C[5][j] * a * (1.0 - b) * c + C[6][j] * a * b * c +
                       C[7][j] * (1.0 - a) * b * c;
            return;
        }
        double E[12][3], F[6][3];  // GeneralHexTransfiniteMap: edges, then faces
        edges_and_faces(u, E, F);
        for (int j = 0; j < 3; ++j) {  // ComputeHexTransfiniteMap
            x[j] = F[5][j] * (1.0 - a) + F[3][j] * a + F[0][j] * (1.0 - b) + F[1][j] * b + F[2][j] * (1.0 - c) +
                   F[4][j] * c;
            x[j] = x[j] - E[0][j] * (1.0 - b) * (1.0 - c) - E[2][j] * (1.0 - b) * c - E[4][j] * b * (1.0 - c) -
                   E[6][j] * b * c - E[8][j] * (1.0 - a) * (1.0 - c) - E[11][j] * (1.0 - a) * c -
                   E[9][j] * (1.0 - c) * a - E[10][j] * a * c - E[3][j] * (1.0 - a) * (1.0 - b) -
                   E[7][j] * (1.0 - a) * b - E[1][j] * a * (1.0 - b) - E[5][j] * a * b;
            x[j] = x[j] + C[0][j] * (1.0 - a) * (1.0 - b) * (1.0 - c) + C[4][j] * (1.0 - a) * (1.0 - b) * c +
                   C[3][j] * (1.0 - a) * b * (1.0 - c) + C[7][j] * (1.0 - a) * b * c +
                   C[1][j] * a * (1.0 - b) * (1.0 - c) + C[5][j] * a * (1.0 - b) * c + C[2][j] * a * b * (1.0 - c) +
                   C[6][j] * a * b * c;
        }
    }

    // g[i][j] = d x_i / d u_j
    void grad_at(const double u[3], double g[3][3]) const {
        const double xi[3] = {0.5 * (u[0] + 1.0), 0.5 * (u[1] + 1.0), 0.5 * (u[2] + 1.0)};
        const double a = xi[0], b = xi[1], c = xi[2];
        const double* C[8] = {corner[0], corner[1], corner[2], corner[3], corner[4], corner[5], corner[6], corner[7]};
        if (hex8) {  // GradHex8TransfiniteMap
            for (int i = 0; i < 3; ++i) {
                g[i][0] = -C[0][i] * (1.0 - b) * (1.0 - c) + C[1][i] * (1.0 - b) * (1.0 - c) + C[2][i] * b * (1.0 - c) -
                          C[3][i] * b * (1.0 - c) - C[4][i] * (1.0 - b) * c + C[5][i] * (1.0 - b) * c +
                          C[6][i] * b * c - C[7][i] * b * c;
                g[i][1] = -C[0][i] * (1.0 - a) * (1.0 - c) - C[1][i] * a * (1.0 - c) + C[2][i] * a * (1.0 - c) +
                          C[3][i] * (1.0 - a) * (1.0 - c) - C[4][i] * (1.0 - a) * c - C[5][i] * a * c +
                          C[6][i] * a * c + C[7][i] * (1.0 - a) * c;
                g[i][2] = -C[0][i] * (1.0 - a) * (1.0 - b) - C[1][i] * a * (1.0 - b) - C[2][i] * a * b -
                          C[3][i] * (1.0 - a) * b + C[4][i] * (1.0 - a) * (1.0 - b) + C[5][i] * a * (1.0 - b) +
                          C[6][i] * a * b + C[7][i] * (1.0 - a) * b;
            }
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) g[i][j] = 0.5 * g[i][j];
            return;
        }
        // GradGeneralHexTransfiniteMap: edges, faces, and their derivatives (scaled by 2 before use)
        double E[12][3], F[6][3], ED[12][3], FD[6][3][2], t[3][2];
        edges_and_faces(u, E, F);
        face[0].deriv(u[0], -1.0, t); for (int q = 0; q < 3; ++q) ED[0][q] = t[q][0];
        face[0].deriv(1.0, u[2], t);  for (int q = 0; q < 3; ++q) ED[1][q] = t[q][1];
        face[0].deriv(u[0], 1.0, t);  for (int q = 0; q < 3; ++q) ED[2][q] = t[q][0];
        face[0].deriv(-1.0, u[2], t); for (int q = 0; q < 3; ++q) ED[3][q] = t[q][1];
        face[1].deriv(u[0], -1.0, t); for (int q = 0; q < 3; ++q) ED[4][q] = t[q][0];
        face[1].deriv(1.0, u[2], t);  for (int q = 0; q < 3; ++q) ED[5][q] = t[q][1];
        face[1].deriv(u[0], 1.0, t);  for (int q = 0; q < 3; ++q) ED[6][q] = t[q][0];
        face[1].deriv(-1.0, u[2], t); for (int q = 0; q < 3; ++q) ED[7][q] = t[q][1];
        face[5].deriv(u[1], -1.0, t); for (int q = 0; q < 3; ++q) ED[8][q] = t[q][0];
        face[3].deriv(u[1], -1.0, t); for (int q = 0; q < 3; ++q) ED[9][q] = t[q][0];
        face[3].deriv(u[1], 1.0, t);  for (int q = 0; q < 3; ++q) ED[10][q] = t[q][0];
        face[5].deriv(u[1], 1.0, t);  for (int q = 0; q < 3; ++q) ED[11][q] = t[q][0];
        face[0].deriv(u[0], u[2], FD[0]);
        face[1].deriv(u[0], u[2], FD[1]);
        face[2].deriv(u[0], u[1], FD[2]);
        face[3].deriv(u[1], u[2], FD[3]);
        face[4].deriv(u[0], u[1], FD[4]);
        face[5].deriv(u[1], u[2], FD[5]);
        for (int e = 0; e < 12; ++e)
            for (int q = 0; q < 3; ++q) ED[e][q] = 2.0 * ED[e][q];
        for (int f = 0; f < 6; ++f)
            for (int q = 0; q < 3; ++q)
                for (int d = 0; d < 2; ++d) FD[f][q][d] = 2.0 * FD[f][q][d];
        for (int j = 0; j < 3; ++j) {  // ComputeGradHexTransfiniteMap
            double gx = -F[5][j] + F[3][j] + FD[0][j][0] * (1.0 - b) + FD[1][j][0] * b + FD[2][j][0] * (1.0 - c) +
                        FD[4][j][0] * c;
            gx = gx - ED[0][j] * (1.0 - b) * (1.0 - c) - ED[2][j] * (1.0 - b) * c - ED[4][j] * b * (1.0 - c) -
                 ED[6][j] * b * c + E[8][j] * (1.0 - c) + E[11][j] * c - E[9][j] * (1.0 - c) - E[10][j] * c +
                 E[3][j] * (1.0 - b) + E[7][j] * b - E[1][j] * (1.0 - b) - E[5][j] * b;
            gx = gx - C[0][j] * (1.0 - b) * (1.0 - c) - C[4][j] * (1.0 - b) * c - C[3][j] * b * (1.0 - c) -
                 C[7][j] * b * c + C[1][j] * (1.0 - b) * (1.0 - c) + C[5][j] * (1.0 - b) * c +
                 C[2][j] * b * (1.0 - c) + C[6][j] * b * c;
            double gy = FD[5][j][0] * (1.0 - a) + FD[3][j][0] * a - F[0][j] + F[1][j] + FD[2][j][1] * (1.0 - c) +
                        FD[4][j][1] * c;
            gy = gy + E[0][j] * (1.0 - c) + E[2][j] * c - E[4][j] * (1.0 - c) - E[6][j] * c -
                 ED[8][j] * (1.0 - a) * (1.0 - c) - ED[11][j] * (1.0 - a) * c - ED[9][j] * (1.0 - c) * a -
                 ED[10][j] * a * c + E[3][j] * (1.0 - a) - E[7][j] * (1.0 - a) + E[1][j] * a - E[5][j] * a;
            gy = gy - C[0][j] * (1.0 - a) * (1.0 - c) - C[4][j] * (1.0 - a) * c + C[3][j] * (1.0 - a) * (1.0 - c) +
                 C[7][j] * (1.0 - a) * c - C[1][j] * a * (1.0 - c) - C[5][j] * a * c + C[2][j] * a * (1.0 - c) +
                 C[6][j] * a * c;
            double gz = FD[5][j][1] * (1.0 - a) + FD[3][j][1] * a + FD[0][j][1] * (1.0 - b) + FD[1][j][1] * b -
                        F[2][j] + F[4][j];
            gz = gz + E[0][j] * (1.0 - b) - E[2][j] * (1.0 - b) + E[4][j] * b - E[6][j] * b + E[8][j] * (1.0 - a) -
                 E[11][j] * (1.0 - a) + E[9][j] * a - E[10][j] * a - ED[3][j] * (1.0 - a) * (1.0 - b) -
                 ED[7][j] * (1.0 - a) * b - ED[1][j] * a * (1.0 - b) - ED[5][j] * a * b;
            gz = gz - C[0][j] * (1.0 - a) * (1.0 - b) + C[4][j] * (1.0 - a) * (1.0 - b) - C[3][j] * (1.0 - a) * b +
                 C[7][j] * (1.0 - a) * b - C[1][j] * a * (1.0 - b) + C[5][j] * a * (1.0 - b) - C[2][j] * a * b +
                 C[6][j] * a * b;
            g[j][0] = 0.5 * gx;
            g[j][1] = 0.5 * gy;
            g[j][2] = 0.5 * gz;
        }
        const double eps = 100.0 * DBL_EPSILON;  // zero out rounded quantities
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                if (std::fabs(g[i][j]) <= eps) g[i][j] = 0.0;
    }

    // The edge and face points of GeneralHexTransfiniteMap at u.
    void edges_and_faces(const double u[3], double E[12][3], double F[6][3]) const {
        face[0].point(u[0], -1.0, E[0]);
        face[0].point(1.0, u[2], E[1]);
        face[0].point(u[0], 1.0, E[2]);
        face[0].point(-1.0, u[2], E[3]);
        face[1].point(u[0], -1.0, E[4]);
        face[1].point(1.0, u[2], E[5]);
        face[1].point(u[0], 1.0, E[6]);
        face[1].point(-1.0, u[2], E[7]);
        face[3].point(u[1], -1.0, E[9]);
        face[5].point(u[1], -1.0, E[8]);
        face[3].point(u[1], 1.0, E[10]);
        face[5].point(u[1], 1.0, E[11]);
        face[0].point(u[0], u[2], F[0]);
        face[1].point(u[0], u[2], F[1]);
        face[2].point(u[0], u[1], F[2]);
        face[3].point(u[1], u[2], F[3]);
        face[4].point(u[0], u[1], F[4]);
        face[5].point(u[1], u[2], F[5]);
    }
};

// computeMetricTermsConservativeForm and the node coordinates of ConstructMappedGeometry for one
// element of uniform order N.
void element_geometry(const HexMap& map, int nodes, int N, double* x, double* ja[3], double* jac, double* ijac) {
    const Nodal& s = nodal(nodes, N);
    const int p = N + 1, np = p * p * p;
    auto id = [p](int i, int j, int k) { return i + p * (j + p * k); };
    for (int k = 0; k < p; ++k)
        for (int j = 0; j < p; ++j)
            for (int i = 0; i < p; ++i) {
                const double u[3] = {s.x[i], s.x[j], s.x[k]};
                map.map_at(u, &x[3 * id(i, j, k)]);
            }
    // the mapping and its gradient at the Chebyshev-Gauss-Lobatto points
    std::vector<double> xc(3 * np), gr(9 * np);  // gr[9n + 3r + c] = grad_x(r, c)
    for (int k = 0; k < p; ++k)
        for (int j = 0; j < p; ++j)
            for (int i = 0; i < p; ++i) {
                const double u[3] = {s.xCGL[i], s.xCGL[j], s.xCGL[k]};
                const int n = id(i, j, k);
                map.map_at(u, &xc[3 * n]);
                double g[3][3];
                map.grad_at(u, g);
                for (int r = 0; r < 3; ++r)
                    for (int c = 0; c < 3; ++c) gr[9 * n + 3 * r + c] = g[r][c];
            }
    // Ja^i_n = -1/2 curl(X_l grad X_m - X_m grad X_l), one Cartesian component n per pass
    std::vector<double> prod(3 * np), aux(9 * np), JaC[3];  // aux[9n + 3d + m] = auxgrad(m, d)
    for (auto& v : JaC) v.assign(3 * np, 0.0);
    const int lA[3] = {2, 0, 1}, mA[3] = {1, 2, 0};  // (x: z grad y - y grad z), (y: x grad z - z grad x), ...
    for (int comp = 0; comp < 3; ++comp) {
        for (int n = 0; n < np; ++n)
            for (int m = 0; m < 3; ++m)
                prod[3 * n + m] = xc[3 * n + lA[comp]] * gr[9 * n + 3 * mA[comp] + m] -
                                  xc[3 * n + mA[comp]] * gr[9 * n + 3 * lA[comp] + m];
        for (auto& v : aux) v = 0.0;
        for (int k = 0; k < p; ++k)
            for (int j = 0; j < p; ++j)
                for (int i = 0; i < p; ++i) {
                    double* A = &aux[9 * id(i, j, k)];
                    for (int l = 0; l < p; ++l)
                        for (int m = 0; m < 3; ++m) A[m] = A[m] + prod[3 * id(l, j, k) + m] * s.DCGL[i * p + l];
                    for (int l = 0; l < p; ++l)
                        for (int m = 0; m < 3; ++m) A[3 + m] = A[3 + m] + prod[3 * id(i, l, k) + m] * s.DCGL[j * p + l];
                    for (int l = 0; l < p; ++l)
                        for (int m = 0; m < 3; ++m) A[6 + m] = A[6 + m] + prod[3 * id(i, j, l) + m] * s.DCGL[k * p + l];
                }
        for (int n = 0; n < np; ++n) {
            const double* A = &aux[9 * n];
            // curl: Jai(1) = auxgrad(3,2) - auxgrad(2,3), Jai(2) = auxgrad(1,3) - auxgrad(3,1), ...
            const double c1 = A[3 + 2] - A[6 + 1];
            const double c2 = A[6 + 0] - A[0 + 2];
            const double c3 = A[0 + 1] - A[3 + 0];
            JaC[0][3 * n + comp] = -0.5 * c1;
            JaC[1][3 * n + comp] = -0.5 * c2;
            JaC[2][3 * n + comp] = -0.5 * c3;
        }
    }
    std::vector<double> jc(np);  // jacobian3D(a1, a2, a3) = a1 . (a2 x a3), a_d = column d of grad_x
    for (int n = 0; n < np; ++n) {
        const double* g = &gr[9 * n];
        const double a1[3] = {g[0], g[3], g[6]}, a2[3] = {g[1], g[4], g[7]}, a3[3] = {g[2], g[5], g[8]};
        const double v[3] = {a2[1] * a3[2] - a3[1] * a2[2], a2[2] * a3[0] - a3[2] * a2[0], a2[0] * a3[1] - a3[0] * a2[1]};
        jc[n] = a1[0] * v[0] + a1[1] * v[1] + a1[2] * v[2];
    }
    // return to the solution nodes
    for (int k = 0; k < p; ++k)
        for (int j = 0; j < p; ++j)
            for (int i = 0; i < p; ++i) {
                const int t = id(i, j, k);
                for (int a = 0; a < 3; ++a)
                    for (int c = 0; c < 3; ++c) ja[a][3 * t + c] = 0.0;
                jac[t] = 0.0;
                for (int nn = 0; nn < p; ++nn)
                    for (int mm = 0; mm < p; ++mm)
                        for (int ll = 0; ll < p; ++ll) {
                            const int q = id(ll, mm, nn);
                            const double tx = s.TCheb2Gauss[i * p + ll], ty = s.TCheb2Gauss[j * p + mm],
                                         tz = s.TCheb2Gauss[k * p + nn];
                            for (int a = 0; a < 3; ++a)
                                for (int c = 0; c < 3; ++c) ja[a][3 * t + c] = ja[a][3 * t + c] + JaC[a][3 * q + c] * tx * ty * tz;
                            jac[t] = jac[t] + jc[q] * tx * ty * tz;
                        }
            }
    for (int n = 0; n < np; ++n) ijac[n] = 1.0 / jac[n];
}

const int kLocalFaceNode[6][4] = {{0, 1, 5, 4}, {3, 2, 6, 7}, {0, 1, 2, 3}, {1, 2, 6, 5}, {4, 5, 6, 7}, {0, 3, 7, 4}};

// faceRotation (HexMesh.f90:490-515) of two lists of matching corner ids.
int face_rotation(const int master[4], const int slave[4]) {
    const int next[4] = {1, 2, 3, 0};
    int j = 0;
    while (j < 3 && master[0] != slave[j]) ++j;
    return master[1] == slave[next[j]] ? j : j + 4;
}

struct BoxMesh {
    int K = 0, N = 0, nodes = 0, F = 0;
    std::vector<int32_t> order, face_elem, face_side, face_rot, face_nf;
    std::vector<double> x, ja[3], jac, ijac, fn, ft1, ft2, fj;
};

}  // namespace
}  // namespace orc

using orc::BoxMesh;

extern "C" {

// Builds the box mesh (see the file header). Returns NULL on invalid arguments.
void* orc_box_mesh_create(int nx, int ny, int nz, const double* lo, const double* hi, double warp, int patch_order,
                          int node_type, int N) {
    using namespace orc;
    if (nx < 2 || ny < 2 || nz < 2 || N < 1 || N > 12 || (patch_order >= 2 && patch_order > N)) return nullptr;
    const int n[3] = {nx, ny, nz};
    auto coord = [&](int d, int i) { return (i == n[d]) ? hi[d] : lo[d] + (hi[d] - lo[d]) * i / n[d]; };
    auto s = [&](int d, double v) { return (v == lo[d] || v == hi[d]) ? 0.0 : std::sin(v); };
    auto warp_point = [&](const double in[3], double out[3]) {
        const double w = warp * s(0, in[0]) * s(1, in[1]) * s(2, in[2]);
        for (int c = 0; c < 3; ++c) out[c] = in[c] + w;
    };
    auto nid = [&](int i, int j, int k) { return i + (nx + 1) * (j + (ny + 1) * k); };
    std::vector<double> X(3 * static_cast<size_t>((nx + 1) * (ny + 1) * (nz + 1)));
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i <= nx; ++i) {
                const double p[3] = {coord(0, i), coord(1, j), coord(2, k)};
                warp_point(p, &X[3 * nid(i, j, k)]);
            }
    auto* m = new BoxMesh;
    m->K = nx * ny * nz;
    m->N = N;
    m->nodes = node_type;
    const int K = m->K, P = N + 1, P3 = P * P * P, P2 = P * P;
    m->order.assign(3 * static_cast<size_t>(K), N);
    const bool curved = patch_order >= 2;
    std::vector<double> knots(curved ? patch_order + 1 : 0);
    for (int i = 0; curved && i <= patch_order; ++i) knots[i] = -std::cos((i * 1.0) * PI / patch_order);
    std::vector<HexMap> maps(K);
    std::vector<int> corners(8 * static_cast<size_t>(K));
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int e = i + nx * (j + ny * k);
                const int ids[8] = {nid(i, j, k),         nid(i + 1, j, k),         nid(i + 1, j + 1, k),
                                    nid(i, j + 1, k),     nid(i, j, k + 1),         nid(i + 1, j, k + 1),
                                    nid(i + 1, j + 1, k + 1), nid(i, j + 1, k + 1)};
                for (int q = 0; q < 8; ++q) corners[8 * e + q] = ids[q];
                HexMap& hm = maps[e];
                if (!curved) {
                    for (int q = 0; q < 8; ++q)
                        for (int c = 0; c < 3; ++c) hm.corner[q][c] = X[3 * ids[q] + c];
                    continue;
                }
                const double x0[3] = {coord(0, i), coord(1, j), coord(2, k)};
                const double x1[3] = {coord(0, i + 1), coord(1, j + 1), coord(2, k + 1)};
                auto ref_to_phys = [&](double a, double b, double c, double out[3]) {
                    const double r[3] = {a, b, c};
                    double p[3];
                    for (int d = 0; d < 3; ++d)
                        p[d] = r[d] == -1.0 ? x0[d] : (r[d] == 1.0 ? x1[d] : x0[d] + 0.5 * (r[d] + 1.0) * (x1[d] - x0[d]));
                    warp_point(p, out);
                };
                const int nb = patch_order + 1;
                for (int f = 0; f < 6; ++f) {  // face parameters as GeneralHexTransfiniteMap evaluates them
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
                    hm.face[f].construct(knots, knots, pts);
                }
                hm.set_corners_from_faces();
            }
    // element geometry
    const int64_t ndof = static_cast<int64_t>(K) * P3;
    m->x.resize(3 * ndof);
    for (auto& v : m->ja) v.resize(3 * ndof);
    m->jac.resize(ndof);
    m->ijac.resize(ndof);
    nodal(node_type, N);  // fill the operator cache before the parallel region
#pragma omp parallel for schedule(dynamic)
    for (int e = 0; e < K; ++e) {
        const int64_t o = static_cast<int64_t>(e) * P3;
        double* ja[3] = {&m->ja[0][3 * o], &m->ja[1][3 * o], &m->ja[2][3 * o]};
        element_geometry(maps[e], node_type, N, &m->x[3 * o], ja, &m->jac[o], &m->ijac[o]);
    }
    // faces in creation order (ConstructFaces + ConstructPeriodicFaces); the minus sides of the
    // periodic pairs (back, top and right at the box planes) are the deleted faces
    auto neighbour = [&](int e, int side, int& en, int& sn, bool& plus, bool& minus) {
        int c[3] = {e % nx, (e / nx) % ny, e / (nx * ny)};
        const int axis = (side == 1 || side == 2) ? 1 : (side == 3 || side == 5) ? 2 : 0;
        const bool up = side == 2 || side == 5 || side == 4;
        plus = !up && c[axis] == 0;
        minus = up && c[axis] == n[axis] - 1;
        c[axis] = (c[axis] + (up ? 1 : n[axis] - 1)) % n[axis];
        en = c[0] + nx * (c[1] + ny * c[2]);
        sn = side == 1 ? 2 : side == 2 ? 1 : side == 3 ? 5 : side == 5 ? 3 : side == 4 ? 6 : 4;
    };
    for (int e = 0; e < K; ++e)
        for (int side = 1; side <= 6; ++side) {
            int en, sn;
            bool plus, minus;
            neighbour(e, side, en, sn, plus, minus);
            if (minus) continue;                // deleted periodic minus face
            if (!plus && en < e) continue;      // created earlier by the neighbour
            int mst[4], slv[4];
            for (int q = 0; q < 4; ++q) {
                mst[q] = corners[8 * e + kLocalFaceNode[side - 1][q]];
                slv[q] = corners[8 * en + kLocalFaceNode[sn - 1][q]];
            }
            if (plus) {  // periodic partner: the matching corner is the one across the box
                const int axis = (side == 1) ? 1 : (side == 3) ? 2 : 0;
                const int stride = axis == 0 ? 1 : axis == 1 ? (nx + 1) : (nx + 1) * (ny + 1);
                for (int q = 0; q < 4; ++q) slv[q] -= n[axis] * stride;
            }
            m->face_elem.push_back(e);
            m->face_elem.push_back(en);
            m->face_side.push_back(side);
            m->face_side.push_back(sn);
            m->face_rot.push_back(face_rotation(mst, slv));
            m->face_nf.push_back(N);
            m->face_nf.push_back(N);
        }
    m->F = static_cast<int>(m->face_rot.size());
    // face geometry from the left element (eSide = 1), projection type 0 (uniform order)
    const int64_t nfp = static_cast<int64_t>(m->F) * P2;
    m->fn.resize(3 * nfp);
    m->ft1.resize(3 * nfp);
    m->ft2.resize(3 * nfp);
    m->fj.resize(nfp);
    const Nodal& sp = nodal(node_type, N);
#pragma omp parallel for schedule(dynamic)
    for (int f = 0; f < m->F; ++f) {
        const int e = m->face_elem[2 * f], side = m->face_side[2 * f];
        const int64_t eo = static_cast<int64_t>(e) * P3, fo = static_cast<int64_t>(f) * P2;
        std::vector<double> fx(3 * P2), dS(3 * P2, 0.0);
        for (int j = 0; j < P; ++j)
            for (int i = 0; i < P; ++i) {
                const double a = sp.x[i], b = sp.x[j];
                double u[3];
                switch (side) {
                    case ELEFT: u[0] = -1.0; u[1] = a; u[2] = b; break;
                    case ERIGHT: u[0] = 1.0; u[1] = a; u[2] = b; break;
                    case EBOTTOM: u[0] = a; u[1] = b; u[2] = -1.0; break;
                    case ETOP: u[0] = a; u[1] = b; u[2] = 1.0; break;
                    case EFRONT: u[0] = a; u[1] = -1.0; u[2] = b; break;
                    default: u[0] = a; u[1] = 1.0; u[2] = b; break;
                }
                maps[e].map_at(u, &fx[3 * (i + P * j)]);
            }
        for (int k = 0; k < P; ++k)
            for (int j = 0; j < P; ++j)
                for (int i = 0; i < P; ++i) {
                    const int64_t nn = eo + i + P * (j + P * k);
                    int t;
                    const double* jv;
                    double v;
                    switch (side) {
                        case ELEFT: t = j + P * k; jv = &m->ja[0][3 * nn]; v = sp.vL[i]; break;
                        case ERIGHT: t = j + P * k; jv = &m->ja[0][3 * nn]; v = sp.vR[i]; break;
                        case EBOTTOM: t = i + P * j; jv = &m->ja[2][3 * nn]; v = sp.vL[k]; break;
                        case ETOP: t = i + P * j; jv = &m->ja[2][3 * nn]; v = sp.vR[k]; break;
                        case EFRONT: t = i + P * k; jv = &m->ja[1][3 * nn]; v = sp.vL[j]; break;
                        default: t = i + P * k; jv = &m->ja[1][3 * nn]; v = sp.vR[j]; break;
                    }
                    for (int c = 0; c < 3; ++c) dS[3 * t + c] = dS[3 * t + c] + jv[c] * v;
                }
        if (side == ELEFT || side == EBOTTOM || side == EFRONT)
            for (auto& v : dS) v = -v;
        for (int q = 0; q < P2; ++q) {
            double* nrm = &m->fn[3 * (fo + q)];
            const double J = std::sqrt(dS[3 * q] * dS[3 * q] + dS[3 * q + 1] * dS[3 * q + 1] + dS[3 * q + 2] * dS[3 * q + 2]);
            m->fj[fo + q] = J;
            for (int c = 0; c < 3; ++c) nrm[c] = dS[3 * q + c] / J;
        }
        // tangents: t1 = derivative of the face points along the first face direction, made
        // orthogonal to n and normalised; t2 = n x t1
        for (int j = 0; j < P; ++j)
            for (int i = 0; i < P; ++i) {
                double t1[3] = {0.0, 0.0, 0.0};
                for (int l = 0; l < P; ++l)
                    for (int c = 0; c < 3; ++c) t1[c] = t1[c] + sp.D[i * P + l] * fx[3 * (l + P * j) + c];
                const double* nrm = &m->fn[3 * (fo + i + P * j)];
                const double dot = t1[0] * nrm[0] + t1[1] * nrm[1] + t1[2] * nrm[2];
                for (int c = 0; c < 3; ++c) t1[c] = t1[c] - dot * nrm[c];
                const double tn = std::sqrt(t1[0] * t1[0] + t1[1] * t1[1] + t1[2] * t1[2]);
                double* o1 = &m->ft1[3 * (fo + i + P * j)];
                double* o2 = &m->ft2[3 * (fo + i + P * j)];
                for (int c = 0; c < 3; ++c) o1[c] = t1[c] / tn;
                o2[0] = nrm[1] * o1[2] - o1[1] * nrm[2];
                o2[1] = nrm[2] * o1[0] - o1[2] * nrm[0];
                o2[2] = nrm[0] * o1[1] - o1[0] * nrm[1];
            }
    }
    return m;
}

// Fills a dg_mesh_desc with the mesh's arrays (valid while the mesh lives).
int orc_box_mesh_describe(void* h, dg_mesh_desc* d) {
    auto* m = static_cast<BoxMesh*>(h);
    if (!m || !d) return DG_ERR_INVALID;
    *d = dg_mesh_desc{};
    d->n_elements = m->K;
    d->node_type = m->nodes;
    d->order = m->order.data();
    d->x = m->x.data();
    d->ja_xi = m->ja[0].data();
    d->ja_eta = m->ja[1].data();
    d->ja_zeta = m->ja[2].data();
    d->jacobian = m->jac.data();
    d->inv_jacobian = m->ijac.data();
    d->n_faces = m->F;
    d->face_elem = m->face_elem.data();
    d->face_side = m->face_side.data();
    d->face_rotation = m->face_rot.data();
    d->face_nf = m->face_nf.data();
    d->face_normal = m->fn.data();
    d->face_t1 = m->ft1.data();
    d->face_t2 = m->ft2.data();
    d->face_jacobian = m->fj.data();
    d->face_boundary = nullptr;
    d->n_boundaries = 0;
    d->boundaries = nullptr;
    return DG_OK;
}

void orc_box_mesh_free(void* h) { delete static_cast<BoxMesh*>(h); }

}  // extern "C"
