// extern "C" mesh builder entry points declared in include/horses3d_gb300.h.
#include <cstring>
#include <new>
#include <string>

#include "horses3d_gb300.h"
#include "mesh.hpp"
#include "spectral.hpp"
#include "status.hpp"

struct h3d_mesh {
    h3d::Mesh m;
};

namespace {

int finish(const h3d::MeshSource& src, int node_type, int uniform_n, const int32_t* orders,
           const std::string& periodic, h3d_mesh** out) {
    const int K = static_cast<int>(src.elem_nodes.size() / 8);
    std::vector<int32_t> ord(3 * static_cast<size_t>(K));
    for (int e = 0; e < K; ++e)
        for (int d = 0; d < 3; ++d) ord[3 * e + d] = orders ? orders[3 * e + d] : uniform_n;
    auto* mesh = new (std::nothrow) h3d_mesh();
    if (!mesh) return h3d::fail(DG_ERR_NOMEM, "host allocation failed");
    std::string err;
    if (!h3d::build_mesh(src, node_type, ord, h3d::parse_periodic(periodic), mesh->m, err)) {
        delete mesh;
        return h3d::fail(DG_ERR_INVALID, err);
    }
    *out = mesh;
    return DG_OK;
}

}  // namespace

extern "C" {

int h3d_mesh_read_specmesh(const char* path, int node_type, int uniform_n, const int32_t* orders,
                           const char* periodic, h3d_mesh** out) {
    if (!path || !out) return h3d::fail(DG_ERR_INVALID, "null argument");
    if (node_type != DG_NODES_GAUSS && node_type != DG_NODES_GAUSS_LOBATTO)
        return h3d::fail(DG_ERR_INVALID, "unknown node type");
    h3d::MeshSource src;
    std::string err;
    if (!h3d::read_specmesh(path, src, err)) return h3d::fail(DG_ERR_IO, err);
    return finish(src, node_type, uniform_n, orders, periodic ? periodic : "", out);
}

int h3d_mesh_box(int nx, int ny, int nz, const double lo[3], const double hi[3], double warp,
                 int patch_order, int node_type, int uniform_n, const int32_t* orders, h3d_mesh** out) {
    if (!lo || !hi || !out || nx < 1 || ny < 1 || nz < 1) return h3d::fail(DG_ERR_INVALID, "bad box arguments");
    if (node_type != DG_NODES_GAUSS && node_type != DG_NODES_GAUSS_LOBATTO)
        return h3d::fail(DG_ERR_INVALID, "unknown node type");
    if (warp != 0.0 && patch_order < 2)
        return h3d::fail(DG_ERR_INVALID, "a warped box needs curved face patches (patch_order >= 2)");
    h3d::MeshSource src;
    h3d::box_source(nx, ny, nz, lo, hi, warp, patch_order, src);
    return finish(src, node_type, uniform_n, orders, "front:back,bottom:top,left:right", out);
}

int h3d_mesh_box_zones(int nx, int ny, int nz, const double lo[3], const double hi[3], double warp,
                       int patch_order, int node_type, int uniform_n, const int32_t* orders,
                       const char* periodic, h3d_mesh** out) {
    if (!lo || !hi || !out || nx < 1 || ny < 1 || nz < 1) return h3d::fail(DG_ERR_INVALID, "bad box arguments");
    if (node_type != DG_NODES_GAUSS && node_type != DG_NODES_GAUSS_LOBATTO)
        return h3d::fail(DG_ERR_INVALID, "unknown node type");
    if (warp != 0.0 && patch_order < 2)
        return h3d::fail(DG_ERR_INVALID, "a warped box needs curved face patches (patch_order >= 2)");
    h3d::MeshSource src;
    h3d::box_source(nx, ny, nz, lo, hi, warp, patch_order, src);
    return finish(src, node_type, uniform_n, orders, periodic ? periodic : "", out);
}

int h3d_mesh_describe(const h3d_mesh* mesh, dg_mesh_desc* d) {
    if (!mesh || !d) return h3d::fail(DG_ERR_INVALID, "null argument");
    const h3d::Mesh& m = mesh->m;
    std::memset(d, 0, sizeof(*d));
    d->n_elements = m.K;
    d->node_type = m.node_type;
    d->order = m.order.data();
    d->x = m.x.data();
    d->ja_xi = m.ja_xi.data();
    d->ja_eta = m.ja_eta.data();
    d->ja_zeta = m.ja_zeta.data();
    d->jacobian = m.jac.data();
    d->inv_jacobian = m.inv_jac.data();
    d->n_faces = m.F;
    d->face_elem = m.face_elem.data();
    d->face_side = m.face_side.data();
    d->face_rotation = m.face_rot.data();
    d->face_nf = m.face_nf.data();
    d->face_normal = m.face_normal.data();
    d->face_t1 = m.face_t1.data();
    d->face_t2 = m.face_t2.data();
    d->face_jacobian = m.face_jac.data();
    d->face_boundary = m.n_boundary_faces > 0 ? m.face_zone.data() : nullptr;
    d->n_boundaries = static_cast<int32_t>(m.zone_names.size());
    d->boundaries = nullptr;
    return DG_OK;
}

int h3d_mesh_zone_count(const h3d_mesh* mesh) { return mesh ? static_cast<int>(mesh->m.zone_names.size()) : 0; }

const char* h3d_mesh_zone_name(const h3d_mesh* mesh, int zone) {
    if (!mesh || zone < 0 || zone >= static_cast<int>(mesh->m.zone_names.size())) return nullptr;
    return mesh->m.zone_names[zone].c_str();
}

double h3d_mesh_volume(const h3d_mesh* mesh) { return mesh ? mesh->m.volume : 0.0; }

void h3d_mesh_free(h3d_mesh* mesh) { delete mesh; }

int h3d_nodal_storage(int node_type, int n, double* x, double* w, double* d) {
    if (n < 0 || n > 16) return h3d::fail(DG_ERR_INVALID, "order out of range");
    if (node_type != DG_NODES_GAUSS && node_type != DG_NODES_GAUSS_LOBATTO)
        return h3d::fail(DG_ERR_INVALID, "unknown node type");
    const h3d::NodalStorage& s = h3d::nodal_storage(node_type, n);
    const int n1 = n + 1;
    if (x) std::memcpy(x, s.x.data(), sizeof(double) * n1);
    if (w) std::memcpy(w, s.w.data(), sizeof(double) * n1);
    if (d) std::memcpy(d, s.D.data(), sizeof(double) * n1 * n1);
    return DG_OK;
}

}  // extern "C"
