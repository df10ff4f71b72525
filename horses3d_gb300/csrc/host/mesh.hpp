// Host-side hexahedral mesh: SpecMesh input, connectivity (faces, rotations, periodic pairs)
// and the one-time FP64 geometry (node coordinates, conservative metric terms, face normals).
// This is the data HexMesh holds after ConstructMesh_FromSpecMeshFile_ (Read_SpecMesh.f90:36-342)
// and HexMesh_ConstructGeometry (HexMesh.f90:2677-2990).
#pragma once
#include <array>
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

namespace h3d {

// Element sides as numbered by the reference (HexElementConnectivityDefinitions.f90:69-77).
enum Side { EFRONT = 1, EBACK = 2, EBOTTOM = 3, ERIGHT = 4, ETOP = 5, ELEFT = 6 };

// Lagrange surface patch through points given on a tensor grid of knots (FacePatchClass.f90).
constexpr int kMaxKnots = 32;
struct FacePatch {
    int nu = 0, nv = 0;
    std::vector<double> uk, vk, wbu, wbv, Du, Dv;
    std::vector<double> pts;  // pts[3*(i + nu*j) + c]
    void construct(const std::vector<double>& u, const std::vector<double>& v, const std::vector<double>& points);
    bool is_quad() const { return nu == 2 && nv == 2; }
    void point(double u1, double u2, double p[3]) const;
    void deriv(double u1, double u2, double g[3][2]) const;
};

// Transfinite hexahedral map from 8 corners (hex8) or from 6 face patches (TransfiniteMaps3D.f90).
struct HexMap {
    bool hex8 = true;
    double corners[8][3] = {};
    FacePatch faces[6];
    void set_faces();  // computes corners from faces 3 and 5 (constructWithFaces)
    void map_at(const double u[3], double x[3]) const;
    void grad_at(const double u[3], double g[3][3]) const;  // g[i][j] = dx_i / du_j
};

// What a SpecMesh file (or a generator) provides before connectivity and geometry.
struct MeshSource {
    std::vector<double> nodes;          // 3 per node
    std::vector<int> elem_nodes;        // 8 per element, 0-based, standard FE ordering
    std::vector<HexMap> maps;           // per element
    std::vector<std::string> bnames;    // 6 per element, lower case, "---" for none
    int bface_order = 1;
};

struct Mesh {
    int K = 0;
    int node_type = 0;
    std::vector<int32_t> order;                 // 3 per element
    std::vector<int64_t> elem_offset;           // node offset of each element (K+1 entries)
    std::vector<double> x, ja_xi, ja_eta, ja_zeta, jac, inv_jac;
    int F = 0;
    std::vector<int32_t> face_elem, face_side, face_rot, face_nf;
    std::vector<int64_t> face_offset;           // face point offset (F+1 entries)
    std::vector<double> face_normal, face_t1, face_t2, face_jac, face_x;
    std::vector<int32_t> elem_face, elem_face_side;  // 6 per element (face id, 1 or 2)
    int n_boundary_faces = 0;
    std::vector<std::string> zone_names;        // non-periodic boundary zones
    std::vector<int32_t> face_zone;             // [F] zone of a boundary face, -1 for interior faces
    double volume = 0.0;
};

// Parses "a:b,c:d" into lower-case pairs.
std::vector<std::pair<std::string, std::string>> parse_periodic(const std::string& spec);

bool read_specmesh(const std::string& path, MeshSource& src, std::string& err);
void box_source(int nx, int ny, int nz, const double lo[3], const double hi[3], double warp,
                int patch_order, MeshSource& src);

// orders: 3 per element. Builds faces, periodic connections, face orders and geometry.
bool build_mesh(const MeshSource& src, int node_type, const std::vector<int32_t>& orders,
                const std::vector<std::pair<std::string, std::string>>& periodic, Mesh& out,
                std::string& err);

}  // namespace h3d
