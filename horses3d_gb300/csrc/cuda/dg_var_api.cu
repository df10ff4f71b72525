// Variable-order (p-anisotropic) and multi-case contexts: host set-up of the work items, slot and
// face tables, operator and Tset tables, and the per-case reductions. The public entry points of
// dg_api.cu dispatch here when a context holds anisotropic orders or several cases.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../host/spectral.hpp"
#include "dg_context.cuh"

using h3dctx::cuda_fail;

namespace {

constexpr int kItemNodes = 256;  // nodes per work item (one element when it holds more)

int side_count(int side, const int32_t* ord) {
    const int px = ord[0] + 1, py = ord[1] + 1, pz = ord[2] + 1;
    switch (side) {
        case 1: case 2: return px * pz;
        case 3: case 5: return px * py;
        default: return py * pz;
    }
}

void side_orders(int side, const int32_t* ord, int& n1, int& n2) {
    switch (side) {
        case 1: case 2: n1 = ord[0]; n2 = ord[2]; break;
        case 3: case 5: n1 = ord[0]; n2 = ord[1]; break;
        default: n1 = ord[1]; n2 = ord[2]; break;
    }
}

int validate_case(const dg_mesh_desc* m, const dg_physics* ph, int c) {
    const std::string tag = "case " + std::to_string(c) + ": ";
    if (m->n_elements < 1 || m->n_faces < 1) return h3d::fail(DG_ERR_INVALID, tag + "empty mesh");
    if (!m->order || !m->x || !m->ja_xi || !m->ja_eta || !m->ja_zeta || !m->jacobian || !m->inv_jacobian ||
        !m->face_elem || !m->face_side || !m->face_rotation || !m->face_nf || !m->face_normal || !m->face_t1 ||
        !m->face_t2 || !m->face_jacobian)
        return h3d::fail(DG_ERR_INVALID, tag + "mesh description has a null array");
    if (m->node_type != DG_NODES_GAUSS && m->node_type != DG_NODES_GAUSS_LOBATTO)
        return h3d::fail(DG_ERR_INVALID, tag + "unknown node type");
    for (int e = 0; e < m->n_elements; ++e)
        for (int d = 0; d < 3; ++d)
            if (m->order[3 * e + d] < 1 || m->order[3 * e + d] + 1 > dg::kMaxP)
                return h3d::fail(DG_ERR_UNSUPPORTED, tag + "polynomial order outside 1..7");
    int64_t sides = 0;
    for (int f = 0; f < m->n_faces; ++f) {
        if (m->face_rotation[f] < 0 || m->face_rotation[f] > 7)
            return h3d::fail(DG_ERR_INVALID, tag + "face rotation outside 0..7");
        int dims[2][2];
        if (m->face_elem[2 * f + 1] < 0) {  // boundary face: one side, face orders its own
            int rc = h3dctx::validate_boundary_face(m, f);
            if (rc) return rc;
            const int e = m->face_elem[2 * f], side = m->face_side[2 * f];
            if (e < 0 || e >= m->n_elements || side < 1 || side > 6)
                return h3d::fail(DG_ERR_INVALID, tag + "face connectivity out of range");
            side_orders(side, m->order + 3 * e, dims[0][0], dims[0][1]);
            if (m->face_nf[2 * f] != dims[0][0] || m->face_nf[2 * f + 1] != dims[0][1])
                return h3d::fail(DG_ERR_INVALID, tag + "a boundary face's orders are not its element side's");
            ++sides;
            continue;
        }
        sides += 2;
        for (int s = 0; s < 2; ++s) {
            const int e = m->face_elem[2 * f + s], side = m->face_side[2 * f + s];
            if (e < 0 || e >= m->n_elements || side < 1 || side > 6)
                return h3d::fail(DG_ERR_INVALID, tag + "face connectivity out of range");
            side_orders(side, m->order + 3 * e, dims[s][0], dims[s][1]);
        }
        const int r = m->face_rotation[f];
        if (!(r == 0 || r == 2 || r == 5 || r == 7)) std::swap(dims[1][0], dims[1][1]);
        for (int a = 0; a < 2; ++a)
            if (m->face_nf[2 * f + a] != std::max(dims[0][a], dims[1][a]))
                return h3d::fail(DG_ERR_INVALID, tag + "face order is not the larger of its two sides' orders");
    }
    if (sides != 6 * static_cast<int64_t>(m->n_elements))
        return h3d::fail(DG_ERR_INVALID, tag + "the faces do not cover every element side once");
    if (ph->mach <= 0.0) return h3d::fail(DG_ERR_INVALID, tag + "Mach number must be positive");
    if (ph->navier_stokes && ph->reynolds <= 0.0) return h3d::fail(DG_ERR_INVALID, tag + "Reynolds number must be positive");
    return DG_OK;
}

dg::PhysConst phys_const(const dg_physics* ph, const dg_options* op) {
    // PhysicsStorage_NS.f90:186-290,413-429 (air, Sutherland defaults)
    dg::PhysConst pc{};
    pc.gamma = 1.4;
    pc.gm1 = 1.4 - 1.0;
    pc.gammaM2 = pc.gamma * (ph->mach * ph->mach);
    pc.ns = ph->navier_stokes ? 1 : 0;
    if (pc.ns) {
        pc.mu = 1.0 / ph->reynolds;
        pc.kappa = 1.0 / (pc.gm1 * (ph->mach * ph->mach) * ph->reynolds * ph->prandtl);
        pc.mu_to_kappa = 1.0 / (pc.gm1 * (ph->mach * ph->mach) * ph->prandtl);
    }
    const double TRef = 520.0 * 5.0 / 9.0;
    pc.S_div_TRef = (198.6 * 5.0 / 9.0) / TRef;
    pc.TReNorm = TRef / TRef;
    pc.lambda_stab = op->riemann == DG_RIEMANN_CENTRAL ? 0.0 : op->lambda_stab;  // SetRiemannSolver
    pc.vns_kappa = 1.0 / (3.0 / 4.0 * pc.gm1 * (ph->mach * ph->mach));              // FluidData_NS.f90:173-181
    pc.riemann = op->riemann;
    pc.averaging = op->averaging;
    pc.inviscid = op->inviscid;
    pc.source = op->source;
    pc.grad_vars = pc.ns ? op->gradient_variables : 0;
    return pc;
}

template <typename R>
cudaError_t upload_as(h3dctx::DevBuf<R>& dst, const std::vector<double>& src, cudaStream_t s) {
    std::vector<R> tmp(src.size());
    for (size_t i = 0; i < src.size(); ++i) tmp[i] = static_cast<R>(src[i]);
    return dst.upload(tmp.data(), tmp.size(), s);
}

// Host copies of the concatenated case data, kept only during set-up.
struct Gathered {
    std::vector<double> ja_xi, ja_eta, ja_zeta, jac, inv_jac, x, fn, ft1, ft2, fj;
    int64_t slot_points = 0;
};

template <typename R>
int setup_vstore(dg_ctx* c, h3dctx::VStore<R>& st, const Gathered& h) {
    cudaStream_t s = c->stream;
    const size_t nd = static_cast<size_t>(c->ndof);
    const size_t sp = static_cast<size_t>(h.slot_points);
    CK(upload_as(st.ja_xi, h.ja_xi, s));
    CK(upload_as(st.ja_eta, h.ja_eta, s));
    CK(upload_as(st.ja_zeta, h.ja_zeta, s));
    CK(upload_as(st.jac, h.jac, s));
    CK(upload_as(st.inv_jac, h.inv_jac, s));
    CK(upload_as(st.fn, h.fn, s));
    CK(upload_as(st.ft1, h.ft1, s));
    CK(upload_as(st.ft2, h.ft2, s));
    CK(upload_as(st.fj, h.fj, s));
    // operators per node count and Tset per (origin, destination) order
    std::vector<dg::OpsP<R>> ops(dg::kMaxP + 1);
    std::memset(ops.data(), 0, sizeof(dg::OpsP<R>) * ops.size());
    for (int P = 2; P <= dg::kMaxP; ++P) {
        const h3d::NodalStorage& ns = h3d::nodal_storage(c->nodes, P - 1);
        for (int i = 0; i < P; ++i) {
            for (int l = 0; l < P; ++l) {
                ops[P].D[i * dg::kMaxP + l] = static_cast<R>(ns.D[i * P + l]);
                ops[P].hatD[i * dg::kMaxP + l] = static_cast<R>(ns.hatD[i * P + l]);
                if (c->nodes == DG_NODES_GAUSS_LOBATTO) ops[P].sharpD[i * dg::kMaxP + l] = static_cast<R>(ns.sharpD[i * P + l]);
            }
            ops[P].vL[i] = static_cast<R>(ns.vL[i]);
            ops[P].vR[i] = static_cast<R>(ns.vR[i]);
            ops[P].bL[i] = static_cast<R>(ns.bL[i]);
            ops[P].bR[i] = static_cast<R>(ns.bR[i]);
        }
    }
    CK(st.ops.upload(ops.data(), ops.size(), s));
    std::vector<double> ts(static_cast<size_t>(dg::kMaxP) * dg::kMaxP * dg::kTsetStride, 0.0);
    for (int No = 1; No < dg::kMaxP; ++No)
        for (int Nd = 1; Nd < dg::kMaxP; ++Nd) {
            const std::vector<double> T = h3d::interpolation_matrix(c->nodes, No, Nd);
            double* o = ts.data() + (No * dg::kMaxP + Nd) * dg::kTsetStride;
            for (int i = 0; i <= Nd; ++i)
                for (int j = 0; j <= No; ++j) o[i * dg::kMaxP + j] = T[i * (No + 1) + j];
        }
    CK(upload_as(st.tset, ts, s));
    std::vector<dg::PhysR<R>> ph(c->n_cases);
    for (int k = 0; k < c->n_cases; ++k) ph[k] = dg::make_phys<R>(c->case_pc[k]);
    CK(st.ph.upload(ph.data(), ph.size(), s));
    {  // boundary conditions of all cases in this precision
        std::vector<dg::BoundaryR<R>> b(c->bcs.size());
        for (size_t i = 0; i < c->bcs.size(); ++i) b[i] = dg::make_boundary<R>(c->bcs[i], c->case_pc[c->bc_case[i]]);
        CK(st.bcs.upload(b.data(), b.size(), s));
    }
    const bool ns = c->pc.ns != 0;
    CK(st.QDot.alloc(5 * nd));
    CK(cudaMemsetAsync(st.QDot.p, 0, sizeof(R) * 5 * nd, s));
    CK(st.Ux.alloc(ns ? 5 * nd : 0));
    CK(st.Uy.alloc(ns ? 5 * nd : 0));
    CK(st.Uz.alloc(ns ? 5 * nd : 0));
    CK(st.QF.alloc(5 * sp));
    CK(st.GF.alloc(ns ? 15 * sp : 0));
    CK(st.UJ.alloc(ns ? 15 * sp : 0));
    CK(st.FS.alloc(5 * sp));

    dg::VArgs<R>& a = st.args;
    std::memset(&a, 0, sizeof(a));
    a.n_items = c->n_items;
    a.n_faces = c->F;
    a.item0 = 0;
    a.n_nc = static_cast<int>(c->h_nc.size());
    a.nc_faces = c->nc_faces.p;
    a.n_groups = c->n_groups;
    a.direct_faces = c->direct_faces.p;
    for (int g = 0; g <= c->n_groups; ++g) {
        a.gf0[g] = c->gf0[g];
        a.gp0[g] = c->gp0[g];
    }
    for (int g = 0; g < c->n_groups; ++g) {
        a.gq1[g] = c->gq1[g];
        a.gq2[g] = c->gq2[g];
    }
    for (int q = 0; q <= dg::kItemClasses; ++q) a.cls[q] = c->cls[q];
    for (int q = 0; q < dg::kItemClasses; ++q) a.ccap[q] = c->ccap[q];
    a.ns = c->pc.ns;
    a.source = c->opt.source;
    a.riemann = c->pc.riemann;
    a.averaging = c->pc.averaging;
    a.grad_vars = c->pc.grad_vars;
    a.split = c->opt.inviscid == DG_INVISCID_SPLIT ? 1 : 0;
    a.items = c->items.p;
    a.item_elems = c->item_elems.p;
    a.eord = c->eord.p;
    a.eoff = c->eoff.p;
    a.soff = c->soff.p;
    a.faces = c->faces4.p;
    a.foff = c->foff.p;
    a.ops = st.ops.p;
    a.tset = st.tset.p;
    a.bc = st.bcs.p;
    a.ph = st.ph.p;
    a.cc = c->cc.p;
    a.time = c->scal.p;
    a.dt = c->scal.p + c->n_cases;
    a.ja_xi = st.ja_xi.p; a.ja_eta = st.ja_eta.p; a.ja_zeta = st.ja_zeta.p;
    a.jac = st.jac.p; a.inv_jac = st.inv_jac.p;
    a.x = c->x.p;
    a.fn = st.fn.p; a.ft1 = st.ft1.p; a.ft2 = st.ft2.p; a.fj = st.fj.p;
    a.Q = c->Q.p; a.G = c->G.p; a.QDot = st.QDot.p;
    a.Ux = st.Ux.p; a.Uy = st.Uy.p; a.Uz = st.Uz.p;
    a.QF = st.QF.p; a.GF = st.GF.p; a.UJ = st.UJ.p; a.FS = st.FS.p;
    return DG_OK;
}

// ------------------------------------------------------------------------------------------------
// Work items and their autotuned size
// ------------------------------------------------------------------------------------------------
// Elements per item for each order triple, chosen by dg_autotune and kept for the process (and, with
// HORSES3D_GB300_TUNE_FILE set, in that file): key (px, py, pz, FP32?, NS?, node type) -> nodes per item.
struct TuneKey {
    int ord, mixed, ns, nodes;
    bool operator<(const TuneKey& o) const {
        return std::tie(ord, mixed, ns, nodes) < std::tie(o.ord, o.mixed, o.ns, o.nodes);
    }
};
std::mutex g_tune_mutex;
std::map<TuneKey, int> g_tune;
bool g_tune_loaded = false;

const char* tune_file() { return std::getenv("HORSES3D_GB300_TUNE_FILE"); }

void load_tune_file_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char* path = tune_file();
    if (!path) return;
    std::FILE* f = std::fopen(path, "r");
    if (!f) return;
    int px, py, pz, mx, ns, nd, cap;
    while (std::fscanf(f, "%d %d %d %d %d %d %d", &px, &py, &pz, &mx, &ns, &nd, &cap) == 7)
        if (px >= 2 && py >= 2 && pz >= 2 && px <= dg::kMaxP && py <= dg::kMaxP && pz <= dg::kMaxP && cap > 0)
            g_tune[TuneKey{px | (py << 8) | (pz << 16), mx, ns, nd}] = cap;
    std::fclose(f);
}

void save_tune_file_locked() {
    const char* path = tune_file();
    if (!path) return;
    std::FILE* f = std::fopen(path, "w");
    if (!f) return;
    for (const auto& kv : g_tune)
        std::fprintf(f, "%d %d %d %d %d %d %d\n", kv.first.ord & 255, (kv.first.ord >> 8) & 255, (kv.first.ord >> 16) & 255,
                     kv.first.mixed, kv.first.ns, kv.first.nodes, kv.second);
    std::fclose(f);
}

int tuned_item_nodes(int ord, bool mixed, bool ns, int nodes) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    load_tune_file_locked();
    auto it = g_tune.find(TuneKey{ord, mixed ? 1 : 0, ns ? 1 : 0, nodes});
    return it == g_tune.end() ? kItemNodes : it->second;
}

struct ItemTable {
    std::vector<int4> items;
    std::vector<int> elems;
    int cls[dg::kItemClasses + 1];
    int ccap[dg::kItemClasses] = {};  // largest item (nodes) per class
    int cap = 0;                      // largest item overall
};

// Elements bucketed by (item class, case, order triple), heaviest buckets first within a class;
// class 0 = anisotropic triples, class P = the isotropic triple (P,P,P). An item holds up to
// item_nodes nodes of one bucket (at least one element). only_cls >= 0 keeps that item class alone
// (autotuning); item_nodes_override > 0 replaces the tuned size.
int isotropic_class(int ord) {
    const int px = ord & 255, py = (ord >> 8) & 255, pz = (ord >> 16) & 255;
    return (px == py && py == pz) ? px : 0;
}

// An isotropic order gets its own class (its own launch with compile-time P) only when it has enough
// nodes to fill the GPU twice over (152 SMs x 2 CTAs x 256 nodes); smaller ones join class 0, whose
// launch would otherwise be followed by a nearly empty one.
constexpr int64_t kClassMinNodes = 152LL * 2 * 256;

std::vector<int> class_of_orders(const std::vector<int>& eord) {
    std::map<int, int64_t> nodes_of;  // isotropic P -> nodes
    for (int o : eord) {
        const int p = isotropic_class(o);
        if (p) nodes_of[p] += static_cast<int64_t>(p) * p * p;
    }
    std::vector<int> cls_of_p(dg::kItemClasses, 0);
    for (const auto& kv : nodes_of)
        if (kv.second >= kClassMinNodes) cls_of_p[kv.first] = kv.first;
    return cls_of_p;
}

int item_class(int ord, const std::vector<int>& cls_of_p) { return cls_of_p[isotropic_class(ord)]; }

ItemTable build_items(const std::vector<int>& eord, const std::vector<int>& ecase, int only_cls, bool mixed, bool ns,
                      int nodes, int item_nodes_override = 0) {
    std::map<std::tuple<int, int, int, int>, std::vector<int>> buckets;  // (class, -np, case, ord) -> elements
    const std::vector<int> cls_of_p = class_of_orders(eord);
    for (size_t e = 0; e < eord.size(); ++e) {
        const int o = eord[e];
        const int cls = item_class(o, cls_of_p);
        if (only_cls >= 0 && cls != only_cls) continue;
        const int px = o & 255, py = (o >> 8) & 255, pz = (o >> 16) & 255;
        buckets[std::make_tuple(cls, -px * py * pz, ecase[e], o)].push_back(static_cast<int>(e));
    }
    ItemTable t;
    int start[dg::kItemClasses + 1];
    for (int q = 0; q <= dg::kItemClasses; ++q) start[q] = -1;
    for (const auto& b : buckets) {
        const int cls = std::get<0>(b.first);
        if (start[cls] < 0) start[cls] = static_cast<int>(t.items.size());
        const int np = -std::get<1>(b.first);
        const int ord = std::get<3>(b.first);
        const int nodes_per_item = item_nodes_override > 0 ? item_nodes_override : tuned_item_nodes(ord, mixed, ns, nodes);
        const int per = std::max(1, nodes_per_item / np);
        const std::vector<int>& els = b.second;
        for (size_t i0 = 0; i0 < els.size(); i0 += per) {
            const int cnt = static_cast<int>(std::min<size_t>(per, els.size() - i0));
            int4 it;
            it.x = static_cast<int>(t.elems.size());
            it.y = cnt;
            it.z = ord;
            it.w = std::get<2>(b.first);
            t.items.push_back(it);
            for (int q = 0; q < cnt; ++q) t.elems.push_back(els[i0 + q]);
            t.cap = std::max(t.cap, cnt * np);
            t.ccap[cls] = std::max(t.ccap[cls], cnt * np);
        }
    }
    // class ranges: an empty class starts where the next non-empty one does
    t.cls[dg::kItemClasses] = static_cast<int>(t.items.size());
    for (int q = dg::kItemClasses - 1; q >= 0; --q) t.cls[q] = start[q] >= 0 ? start[q] : t.cls[q + 1];
    return t;
}

// The reference's discretisation is not free-stream preserving where curved faces join elements of
// different orders: the two sides' metric terms, interpolated to the face points with Tset, do not
// match, and a fluid at rest at pressure p gets the momentum residual p G(x). The mixed form leaves
// the constant p_ref out of its FP32 momentum fluxes (exact where G = 0), so it adds p_ref G back in
// the update. G is the FP64 right-hand side of the state at rest with unit pressure (no source),
// computed once here with the FP64 kernels and FP64 item sizes; where its largest value is round-off
// (straight or conforming meshes, below 1e-8) nothing is added.
int static_pressure_residual(dg_ctx* c, const Gathered& h) {
    cudaStream_t s = c->stream;
    const size_t nd = static_cast<size_t>(c->ndof);
    const ItemTable t = build_items(c->h_eord, c->h_ecase, -1, false, c->pc.ns != 0, c->nodes);
    h3dctx::DevBuf<int4> items;
    h3dctx::DevBuf<int> elems;
    h3dctx::VStore<double> st;
    auto done = [&](int rc) {
        st.free();
        items.free();
        elems.free();
        return rc;
    };
    cudaError_t e;
    if ((e = items.upload(t.items.data(), t.items.size(), s)) || (e = elems.upload(t.elems.data(), t.elems.size(), s)))
        return done(cuda_fail(e, "static pressure items"));
    int rc = setup_vstore(c, st, h);
    if (rc) return done(rc);
    {  // every boundary as an adiabatic free-slip wall: its external state is the state at rest itself,
       // so the residual below is that of a constant pressure (the part the mixed fluxes leave out)
        std::vector<dg::BoundaryR<double>> b(c->bcs.size());
        for (size_t i = 0; i < c->bcs.size(); ++i) {
            dg_boundary w{};
            w.type = DG_BC_FREE_SLIP_WALL;
            w.wall_temperature = 1.0;
            b[i] = dg::make_boundary<double>(w, c->case_pc[c->bc_case[i]]);
        }
        if (!b.empty() &&
            (e = cudaMemcpyAsync(st.bcs.p, b.data(), sizeof(b[0]) * b.size(), cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return done(cuda_fail(e, "static pressure boundaries"));
    }
    dg::VArgs<double>& a = st.args;
    a.items = items.p;
    a.item_elems = elems.p;
    a.n_items = static_cast<int>(t.items.size());
    a.cap = t.cap;
    for (int q = 0; q <= dg::kItemClasses; ++q) a.cls[q] = t.cls[q];
    for (int q = 0; q < dg::kItemClasses; ++q) a.ccap[q] = t.ccap[q];
    a.source = DG_SOURCE_NONE;
    const dg::VStageFn<double> fn = dg::vstage_fn_fp64();
    std::vector<double> q(5 * nd);
    for (size_t g = 0; g < nd; ++g) {
        q[5 * g] = 1.0;
        q[5 * g + 1] = q[5 * g + 2] = q[5 * g + 3] = 0.0;
        q[5 * g + 4] = 1.0 / c->pc.gm1;
    }
    if ((e = cudaMemcpyAsync(c->Q.p, q.data(), sizeof(double) * q.size(), cudaMemcpyHostToDevice, s)) ||
        (e = fn(a, dg::kPrepare, 0.0, 0, s, nullptr)) || (e = fn(a, dg::kTraces, 0.0, 0, s, nullptr)) ||
        (e = fn(a, -1, 0.0, dg::kWriteQDot, s, nullptr)) ||
        (e = cudaMemcpyAsync(q.data(), st.QDot.p, sizeof(double) * q.size(), cudaMemcpyDeviceToHost, s)) ||
        (e = cudaMemsetAsync(c->Q.p, 0, sizeof(double) * q.size(), s)) || (e = cudaStreamSynchronize(s)))
        return done(cuda_fail(e, "static pressure residual"));
    std::vector<double> g3(3 * nd);
    double mx = 0.0;
    for (size_t g = 0; g < nd; ++g)
        for (int d = 0; d < 3; ++d) {
            g3[3 * g + d] = q[5 * g + 1 + d];
            mx = std::max(mx, std::fabs(g3[3 * g + d]));
        }
    if (mx > 1e-8) {  // round-off of straight or conforming meshes stays far below; curved p-nonconforming ~0.1
        if ((e = c->pstat.upload(g3.data(), g3.size(), s)) != cudaSuccess)
            return done(cuda_fail(e, "static pressure upload"));
    }
    return done(DG_OK);
}

}  // namespace

namespace h3dvar {

bool needs_variable_path(const dg_mesh_desc* m) {
    if (!m || !m->order || m->n_elements < 1) return false;
    const int N = m->order[0];
    for (int e = 0; e < m->n_elements; ++e)
        for (int d = 0; d < 3; ++d)
            if (m->order[3 * e + d] != N) return true;
    return false;
}

int create(int n_cases, const dg_mesh_desc* meshes, const dg_physics* phys, const dg_options* op, dg_ctx** out) {
    if (!out) return h3d::fail(DG_ERR_INVALID, "null output pointer");
    *out = nullptr;
    if (n_cases < 1 || !meshes || !phys || !op) return h3d::fail(DG_ERR_INVALID, "null argument or no case");
    if (op->inviscid != DG_INVISCID_STANDARD && op->inviscid != DG_INVISCID_SPLIT)
        return h3d::fail(DG_ERR_UNSUPPORTED, "inviscid discretization");
    if (op->riemann < DG_RIEMANN_ROE || op->riemann > DG_RIEMANN_U_DISS) return h3d::fail(DG_ERR_UNSUPPORTED, "riemann solver");
    if (op->averaging < DG_AVG_STANDARD || op->averaging > DG_AVG_CHANDRASEKAR)
        return h3d::fail(DG_ERR_UNSUPPORTED, "averaging");
    if (op->precision != DG_PRECISION_FP64 && op->precision != DG_PRECISION_MIXED)
        return h3d::fail(DG_ERR_UNSUPPORTED, "precision");
    if (op->source < DG_SOURCE_NONE || op->source > DG_SOURCE_MMS_LAMB_VECTOR)
        return h3d::fail(DG_ERR_UNSUPPORTED, "source");
    if (op->gradient_variables < DG_GRADVARS_STATE || op->gradient_variables > DG_GRADVARS_ENERGY)
        return h3d::fail(DG_ERR_UNSUPPORTED, "gradient variables");
    for (int k = 0; k < n_cases; ++k) {
        int rc = validate_case(&meshes[k], &phys[k], k);
        if (rc) return rc;
        if (meshes[k].node_type != meshes[0].node_type)
            return h3d::fail(DG_ERR_UNSUPPORTED, "all cases of a batch need the same node type");
        if (op->inviscid == DG_INVISCID_SPLIT && meshes[k].node_type != DG_NODES_GAUSS_LOBATTO)
            return h3d::fail(DG_ERR_INVALID, "the split form needs Gauss-Lobatto nodes");
        if ((phys[k].navier_stokes != 0) != (phys[0].navier_stokes != 0))
            return h3d::fail(DG_ERR_UNSUPPORTED, "all cases of a batch need the same equations (Euler or NS)");
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return h3d::fail(DG_ERR_NODEVICE, "no CUDA device visible");

    auto* c = new dg_ctx();
    auto bail = [&](int code) {
        dg_destroy(c);
        return code;
    };
    c->var = true;
    c->n_cases = n_cases;
    c->phys = phys[0];
    c->opt = *op;
    c->nodes = meshes[0].node_type;
    c->mixed = op->precision == DG_PRECISION_MIXED;
    c->pc = phys_const(&phys[0], op);
    c->case_pc.resize(n_cases);
    c->case_const.resize(n_cases);
    for (int k = 0; k < n_cases; ++k) {
        c->case_pc[k] = phys_const(&phys[k], op);
        const dg::PhysConst& pc = c->case_pc[k];
        c->case_const[k] = dg::CaseConst{0.0, pc.gm1, pc.gammaM2, 0.0, 0.0};
        dg::source_constants(op->source, phys[k].mach, phys[k].reynolds, phys[k].prandtl, pc.ns,
                             &c->case_const[k].mu, &c->case_const[k].kappa);
    }

    // element, slot and face tables of the concatenated cases
    std::vector<int> eord;
    std::vector<long long> eoff, soff, foff;
    std::vector<int4> faces;
    std::vector<int> ecase;
    Gathered h;
    c->case_ndof_off.assign(n_cases + 1, 0);
    c->case_elem_off.assign(n_cases + 1, 0);
    c->case_mach.resize(n_cases);
    for (int k = 0; k < n_cases; ++k) c->case_mach[k] = phys[k].mach;
    int64_t nodes = 0, spts = 0, fpts = 0;
    int kbase = 0;
    for (int k = 0; k < n_cases; ++k) {
        const dg_mesh_desc& m = meshes[k];
        int64_t case_nodes = 0;
        for (int e = 0; e < m.n_elements; ++e) {
            const int32_t* o = m.order + 3 * e;
            eord.push_back((o[0] + 1) | ((o[1] + 1) << 8) | ((o[2] + 1) << 16));
            eoff.push_back(nodes + case_nodes);
            ecase.push_back(k);
            case_nodes += static_cast<int64_t>(o[0] + 1) * (o[1] + 1) * (o[2] + 1);
            for (int side = 1; side <= 6; ++side) {
                soff.push_back(spts);
                spts += side_count(side, o);
            }
        }
        auto append = [](std::vector<double>& dst, const double* src, int64_t n) { dst.insert(dst.end(), src, src + n); };
        append(h.ja_xi, m.ja_xi, 3 * case_nodes);
        append(h.ja_eta, m.ja_eta, 3 * case_nodes);
        append(h.ja_zeta, m.ja_zeta, 3 * case_nodes);
        append(h.jac, m.jacobian, case_nodes);
        append(h.inv_jac, m.inv_jacobian, case_nodes);
        append(h.x, m.x, 3 * case_nodes);
        int64_t case_fpts = 0;
        std::vector<int> seen(6 * static_cast<size_t>(m.n_elements), 0);
        const int bc_base = static_cast<int>(c->bcs.size());
        if (m.n_boundaries > 0 && m.boundaries)
            for (int b = 0; b < m.n_boundaries; ++b) {
                c->bcs.push_back(m.boundaries[b]);
                c->bc_case.push_back(k);
            }
        if (c->bcs.size() >= (1u << 11)) return bail(h3d::fail(DG_ERR_UNSUPPORTED, "more than 2047 boundary conditions"));
        for (int f = 0; f < m.n_faces; ++f) {
            const int q1 = m.face_nf[2 * f] + 1, q2 = m.face_nf[2 * f + 1] + 1;
            const bool boundary = m.face_elem[2 * f + 1] < 0;
            for (int s = 0; s < (boundary ? 1 : 2); ++s) {
                int& mark = seen[6 * static_cast<size_t>(m.face_elem[2 * f + s]) + m.face_side[2 * f + s] - 1];
                if (mark) return bail(h3d::fail(DG_ERR_INVALID, "an element side belongs to two faces"));
                mark = 1;
            }
            int4 fd;
            fd.x = kbase + m.face_elem[2 * f];
            fd.y = boundary ? -1 : kbase + m.face_elem[2 * f + 1];
            fd.z = m.face_side[2 * f] | ((boundary ? 0 : m.face_side[2 * f + 1]) << 4) | (m.face_rotation[f] << 8) |
                   (q1 << 12) | (q2 << 16) | (boundary ? (bc_base + m.face_boundary[f]) << 20 : 0);
            fd.w = k;
            faces.push_back(fd);
            foff.push_back(fpts + case_fpts);
            case_fpts += static_cast<int64_t>(q1) * q2;
        }
        append(h.fn, m.face_normal, 3 * case_fpts);
        append(h.ft1, m.face_t1, 3 * case_fpts);
        append(h.ft2, m.face_t2, 3 * case_fpts);
        append(h.fj, m.face_jacobian, case_fpts);
        nodes += case_nodes;
        fpts += case_fpts;
        kbase += m.n_elements;
        c->case_elem_off[k + 1] = kbase;
        c->case_ndof_off[k + 1] = nodes;
    }
    c->K = kbase;
    c->F = static_cast<int>(faces.size());
    c->ndof = nodes;
    h.slot_points = spts;

    // faces whose sides already carry the face's point counts need no Tset interpolation and go to
    // the one-thread-per-point kernel, grouped by point counts; the others keep the staged kernel
    {
        std::map<std::pair<int, int>, std::vector<int>> groups;
        std::vector<int> nc;
        for (int f = 0; f < c->F; ++f) {
            const int4& fd = faces[f];
            const int q1 = (fd.z >> 12) & 15, q2 = (fd.z >> 16) & 15;
            if (fd.y < 0) {  // boundary faces carry their element side's orders
                groups[{q1, q2}].push_back(f);
                continue;
            }
            const int oL = eord[fd.x], oR = eord[fd.y];
            const int32_t ordL[3] = {(oL & 255) - 1, ((oL >> 8) & 255) - 1, ((oL >> 16) & 255) - 1};
            const int32_t ordR[3] = {(oR & 255) - 1, ((oR >> 8) & 255) - 1, ((oR >> 16) & 255) - 1};
            int l1, l2, r1, r2;
            side_orders(fd.z & 15, ordL, l1, l2);
            side_orders((fd.z >> 4) & 15, ordR, r1, r2);
            const int rot = (fd.z >> 8) & 15;
            if (!(rot == 0 || rot == 2 || rot == 5 || rot == 7)) std::swap(r1, r2);
            if (l1 + 1 == q1 && l2 + 1 == q2 && r1 + 1 == q1 && r2 + 1 == q2) groups[{q1, q2}].push_back(f);
            else nc.push_back(f);
        }
        c->h_nc = nc;
        c->h_direct.clear();
        c->n_groups = 0;
        c->gf0[0] = 0;
        c->gp0[0] = 0;
        for (const auto& kv : groups) {
            const int g = c->n_groups++;
            c->gq1[g] = static_cast<unsigned char>(kv.first.first);
            c->gq2[g] = static_cast<unsigned char>(kv.first.second);
            c->h_direct.insert(c->h_direct.end(), kv.second.begin(), kv.second.end());
            c->gf0[g + 1] = static_cast<int>(c->h_direct.size());
            c->gp0[g + 1] = c->gp0[g] + static_cast<int>(kv.second.size()) * kv.first.first * kv.first.second;
        }
    }

    c->h_eord = eord;
    c->h_ecase = ecase;
    ItemTable tab = build_items(c->h_eord, c->h_ecase, -1, c->mixed, c->pc.ns != 0, c->nodes);
    const std::vector<int4>& items = tab.items;
    const std::vector<int>& item_elems = tab.elems;
    const int cap = tab.cap;
    c->n_items = static_cast<int>(items.size());
    for (int q = 0; q <= dg::kItemClasses; ++q) c->cls[q] = tab.cls[q];
    for (int q = 0; q < dg::kItemClasses; ++q) c->ccap[q] = tab.ccap[q];

    cudaError_t e;
    if ((e = cudaGetDevice(&c->device)) != cudaSuccess) return bail(cuda_fail(e, "cudaGetDevice"));
    if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return bail(cuda_fail(e, "cudaStreamCreate"));
    if ((e = dg::create_lanes(c->lanes)) != cudaSuccess) return bail(cuda_fail(e, "side streams"));
    if ((e = cudaMallocHost(reinterpret_cast<void**>(&c->h_scal), sizeof(double) * (4 * n_cases + 8))) != cudaSuccess)
        return bail(cuda_fail(e, "cudaMallocHost"));
    cudaStream_t s = c->stream;
    const size_t nd = static_cast<size_t>(c->ndof);
    if ((e = c->Q.alloc(5 * nd)) || (e = c->G.alloc(5 * nd)) || (e = c->scal.alloc(2 * n_cases)) ||
        (e = c->red.alloc(8 * n_cases)) || (e = c->vnan.alloc(n_cases)) || (e = c->nan_flag.alloc(1)))
        return bail(cuda_fail(e, "alloc state"));
    if ((e = cudaMemsetAsync(c->Q.p, 0, sizeof(double) * 5 * nd, s)) ||
        (e = cudaMemsetAsync(c->G.p, 0, sizeof(double) * 5 * nd, s)) ||
        (e = cudaMemsetAsync(c->scal.p, 0, sizeof(double) * 2 * n_cases, s)))
        return bail(cuda_fail(e, "clear state"));
    {
        std::vector<unsigned long long> init(8 * static_cast<size_t>(n_cases), 0ull);
        const double big = 1.0e300;
        unsigned long long bb;
        std::memcpy(&bb, &big, 8);
        for (int k = 0; k < n_cases; ++k) {
            init[8 * k] = init[8 * k + 1] = bb;
            init[8 * k + 7] = dg::kDtEstimateInit;
        }
        if ((e = c->red.upload(init.data(), init.size(), s)) != cudaSuccess) return bail(cuda_fail(e, "init reductions"));
    }
    if ((e = c->x.upload(h.x.data(), h.x.size(), s)) || (e = c->items.upload(items.data(), items.size(), s)) ||
        (e = c->item_elems.upload(item_elems.data(), item_elems.size(), s)) ||
        (e = c->eord.upload(eord.data(), eord.size(), s)) || (e = c->eoff.upload(eoff.data(), eoff.size(), s)) ||
        (e = c->soff.upload(soff.data(), soff.size(), s)) || (e = c->faces4.upload(faces.data(), faces.size(), s)) ||
        (e = c->foff.upload(foff.data(), foff.size(), s)) ||
        (e = c->nc_faces.upload(c->h_nc.data(), c->h_nc.size(), s)) ||
        (e = c->direct_faces.upload(c->h_direct.data(), c->h_direct.size(), s)) ||
        (e = c->cc.upload(c->case_const.data(), c->case_const.size(), s)))
        return bail(cuda_fail(e, "upload tables"));
    {
        std::vector<double> dxi(dg::kMaxP + 1, 0.0), gm2(n_cases);
        for (int P = 2; P <= dg::kMaxP; ++P) {
            const h3d::NodalStorage& ns = h3d::nodal_storage(c->nodes, P - 1);
            dxi[P] = 1.0 / std::fabs(ns.x[1] - ns.x[0]);
        }
        for (int k = 0; k < n_cases; ++k) gm2[k] = c->case_pc[k].gammaM2;
        if ((e = c->dxi_table.upload(dxi.data(), dxi.size(), s)) || (e = c->gamma_M2.upload(gm2.data(), gm2.size(), s)))
            return bail(cuda_fail(e, "upload dt tables"));
    }
    int rc;
    if (c->mixed) {
        if ((rc = static_pressure_residual(c, h))) return bail(rc);
        if ((rc = setup_vstore(c, c->v32, h))) return bail(rc);
        c->v32.args.pstat = c->pstat.p;
        c->v32.args.cap = cap;
        c->v32.stage = dg::vstage_fn_fp32();
        c->v32.times = dg::vtimes_fn_fp32();
        c->v32.tune = dg::vtune_fn_fp32();
    } else {
        if ((rc = setup_vstore(c, c->v64, h))) return bail(rc);
        c->v64.args.cap = cap;
        c->v64.stage = dg::vstage_fn_fp64();
        c->v64.times = dg::vtimes_fn_fp64();
        c->v64.tune = dg::vtune_fn_fp64();
    }
    if ((e = stage(c, dg::kPrepare, 0.0, 0)) != cudaSuccess) return bail(cuda_fail(e, "kernel attributes"));
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return bail(cuda_fail(e, "set-up"));
    *out = c;
    return DG_OK;
}

void release(dg_ctx* c) {
    dg::destroy_lanes(c->lanes);
    c->v64.free();
    c->v32.free();
    for (auto* b : {&c->items, &c->faces4}) b->free();
    for (auto* b : {&c->item_elems, &c->eord, &c->vnan, &c->nc_faces, &c->direct_faces}) b->free();
    for (auto* b : {&c->eoff, &c->soff, &c->foff}) b->free();
    c->cc.free();
    c->pstat.free();
    c->esum.free();
    c->dxi_table.free();
    c->gamma_M2.free();
}

int upload(dg_ctx* c, const double* q) {
    bool changed = false;
    CK(cudaMemcpyAsync(c->Q.p, q, sizeof(double) * 5 * c->ndof, cudaMemcpyHostToDevice, c->stream));
    if (c->mixed) {  // energy reference of every case: the mean energy of its uploaded state
        for (int k = 0; k < c->n_cases; ++k) {
            const int64_t g0 = c->case_ndof_off[k], g1 = c->case_ndof_off[k + 1];
            double e_ref = 0.0;
            int rc = h3dctx::device_mean_energy(c, g0, g1, &e_ref);
            if (rc) return rc;
            if (!std::isfinite(e_ref)) return h3d::fail(DG_ERR_NAN, "NaN or Inf in the uploaded state");
            if (e_ref != c->case_const[k].e_ref) {
                c->case_const[k].e_ref = e_ref;
                changed = true;
            }
        }
        if (changed) {
            std::vector<dg::PhysR<float>> ph(c->n_cases);
            for (int k = 0; k < c->n_cases; ++k) {
                ph[k] = dg::make_phys<float>(c->case_pc[k]);
                dg::set_reference_energy(ph[k], c->case_pc[k].gm1, c->case_const[k].e_ref);
            }
            CK(cudaMemcpyAsync(c->v32.ph.p, ph.data(), sizeof(ph[0]) * ph.size(), cudaMemcpyHostToDevice, c->stream));
            CK(cudaMemcpyAsync(c->cc.p, c->case_const.data(), sizeof(dg::CaseConst) * c->n_cases, cudaMemcpyHostToDevice,
                               c->stream));
            CK(cudaStreamSynchronize(c->stream));
        }
    }
    CK(cudaMemsetAsync(c->G.p, 0, sizeof(double) * 5 * c->ndof, c->stream));
    CK(stage(c, dg::kTraces, 0.0, 0));
    CK(cudaStreamSynchronize(c->stream));
    return DG_OK;
}

cudaError_t stage(dg_ctx* c, int st, double tshift, int flags) {
    if (c->mixed) return c->v32.stage(c->v32.args, st, tshift, flags, c->stream, &c->lanes);
    return c->v64.stage(c->v64.args, st, tshift, flags, c->stream, &c->lanes);
}

cudaError_t enqueue_max_dt(dg_ctx* c, double cfl, double dcfl) {
    dg::VDtArgs d;
    d.items = c->items.p;
    d.item_elems = c->item_elems.p;
    d.eoff = c->eoff.p;
    d.Q = c->Q.p;
    d.dxi = c->dxi_table.p;
    d.gamma_M2 = c->gamma_M2.p;
    d.cfl = cfl;
    d.dcfl = dcfl;
    d.gamma = c->pc.gamma;
    d.gm1 = c->pc.gm1;
    d.S_div_TRef = c->pc.S_div_TRef;
    d.TReNorm = c->pc.TReNorm;
    d.ns = c->pc.ns;
    d.red = c->red.p;
    for (int pass = 0; pass < 2; ++pass) {
        if (c->mixed)
            dg::kv_dt_pass<float><<<c->n_items, 256, 0, c->stream>>>(d, c->v32.ja_xi.p, c->v32.ja_eta.p,
                                                                      c->v32.ja_zeta.p, c->v32.jac.p, pass);
        else
            dg::kv_dt_pass<double><<<c->n_items, 256, 0, c->stream>>>(d, c->v64.ja_xi.p, c->v64.ja_eta.p,
                                                                       c->v64.ja_zeta.p, c->v64.jac.p, pass);
    }
    dg::kv_dt_final<<<1, 256, 0, c->stream>>>(c->red.p, c->scal.p + c->n_cases, c->n_cases);
    return cudaGetLastError();
}

cudaError_t enqueue_advance_time(dg_ctx* c) {
    dg::kv_advance_time<<<1, 256, 0, c->stream>>>(c->scal.p, c->scal.p + c->n_cases, c->n_cases);
    return cudaGetLastError();
}

cudaError_t enqueue_residuals(dg_ctx* c) {
    cudaError_t e;
    for (int k = 0; k < c->n_cases; ++k)
        if ((e = cudaMemsetAsync(c->red.p + 8 * k + 2, 0, 5 * sizeof(unsigned long long), c->stream)) != cudaSuccess)
            return e;
    if ((e = cudaMemsetAsync(c->vnan.p, 0, sizeof(int) * c->n_cases, c->stream)) != cudaSuccess) return e;
    if (c->mixed)
        dg::kv_residuals<float><<<c->n_items, 256, 0, c->stream>>>(c->items.p, c->item_elems.p, c->eoff.p,
                                                                    c->v32.QDot.p, c->Q.p, c->red.p, c->vnan.p);
    else
        dg::kv_residuals<double><<<c->n_items, 256, 0, c->stream>>>(c->items.p, c->item_elems.p, c->eoff.p,
                                                                     c->v64.QDot.p, c->Q.p, c->red.p, c->vnan.p);
    return cudaGetLastError();
}

int residuals(dg_ctx* c, double* maxres, int* nan_case) {
    CK(enqueue_residuals(c));
    std::vector<unsigned long long> bits(8 * static_cast<size_t>(c->n_cases));
    std::vector<int> flags(c->n_cases);
    CK(cudaMemcpyAsync(bits.data(), c->red.p, sizeof(unsigned long long) * bits.size(), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(flags.data(), c->vnan.p, sizeof(int) * flags.size(), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    int any = 0;
    for (int k = 0; k < c->n_cases; ++k) {
        for (int v = 0; v < 5; ++v) std::memcpy(&maxres[5 * k + v], &bits[8 * k + 2 + v], sizeof(double));
        if (nan_case) nan_case[k] = flags[k];
        any |= flags[k];
    }
    return any ? h3d::fail(DG_ERR_NAN, "NaN or Inf in Q") : DG_OK;
}

int kernel_times(dg_ctx* c, int reps, double* ms) {
    if (c->mixed) CK(c->v32.times(c->v32.args, reps, c->stream, ms));
    else CK(c->v64.times(c->v64.args, reps, c->stream, ms));
    return DG_OK;
}

namespace {

// Installs an item table in the context: device copies, launch arguments, kernel attributes for
// its largest item; drops the captured graph (its launches used the old table).
template <typename R>
int apply_items(dg_ctx* c, h3dctx::VStore<R>& st, const ItemTable& t) {
    c->items.free();
    c->item_elems.free();
    CK(c->items.upload(t.items.data(), t.items.size(), c->stream));
    CK(c->item_elems.upload(t.elems.data(), t.elems.size(), c->stream));
    c->n_items = static_cast<int>(t.items.size());
    for (int q = 0; q <= dg::kItemClasses; ++q) c->cls[q] = t.cls[q];
    for (int q = 0; q < dg::kItemClasses; ++q) c->ccap[q] = t.ccap[q];
    dg::VArgs<R>& a = st.args;
    a.items = c->items.p;
    a.item_elems = c->item_elems.p;
    a.n_items = c->n_items;
    a.cap = t.cap;
    for (int q = 0; q <= dg::kItemClasses; ++q) a.cls[q] = t.cls[q];
    for (int q = 0; q < dg::kItemClasses; ++q) a.ccap[q] = t.ccap[q];
    CK(st.stage(a, dg::kPrepare, 0.0, 0, c->stream, nullptr));
    h3dctx::drop_graphs(c);
    return DG_OK;
}

// For every item class of the context (the anisotropic triples together; each isotropic order on its
// own) times the volume and update kernels over that class with each candidate item size; the class
// is one launch in a stage, so its time alone is the time it takes in the step. The fastest size is
// recorded for every order triple of the class.
template <typename R>
int autotune_store(dg_ctx* c, h3dctx::VStore<R>& st, int reps) {
    cudaStream_t s = c->stream;
    const size_t n5 = 5 * static_cast<size_t>(c->ndof);
    h3dctx::DevBuf<double> q0, g0;
    h3dctx::DevBuf<R> d0;
    int rc = DG_OK;
    CK(q0.alloc(n5));
    CK(g0.alloc(n5));
    CK(d0.alloc(n5));
    CK(cudaMemcpyAsync(q0.p, c->Q.p, sizeof(double) * n5, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(g0.p, c->G.p, sizeof(double) * n5, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(d0.p, st.QDot.p, sizeof(R) * n5, cudaMemcpyDeviceToDevice, s));
    {
        dg::VArgs<R> big = st.args;
        big.cap = 2 * kItemNodes;  // kernel attributes for the largest candidate
        CK(st.stage(big, dg::kPrepare, 0.0, 0, s, nullptr));
    }
    const int candidates[] = {kItemNodes / 4, kItemNodes / 2, kItemNodes, 2 * kItemNodes};
    std::map<int, std::vector<int>> class_ords;  // class -> its order triples
    const std::vector<int> cls_of_p = class_of_orders(c->h_eord);
    for (int o : c->h_eord) {
        std::vector<int>& v = class_ords[item_class(o, cls_of_p)];
        if (std::find(v.begin(), v.end(), o) == v.end()) v.push_back(o);
    }
    h3dctx::DevBuf<int4> titems;
    h3dctx::DevBuf<int> telems;
    std::map<TuneKey, int> chosen;
    for (const auto& co : class_ords) {
        const int cls = co.first;
        double best_ms = 1e300;
        int best = kItemNodes;
        std::vector<int> seen_caps;
        for (int cand : candidates) {
            const ItemTable t = build_items(c->h_eord, c->h_ecase, cls, c->mixed, c->pc.ns != 0, c->nodes, cand);
            if (std::find(seen_caps.begin(), seen_caps.end(), static_cast<int>(t.items.size())) != seen_caps.end())
                continue;  // same grouping as a smaller candidate
            seen_caps.push_back(static_cast<int>(t.items.size()));
            titems.free();
            telems.free();
            CK(titems.upload(t.items.data(), t.items.size(), s));
            CK(telems.upload(t.elems.data(), t.elems.size(), s));
            dg::VArgs<R> b = st.args;
            b.items = titems.p;
            b.item_elems = telems.p;
            b.n_items = static_cast<int>(t.items.size());
            b.cap = t.cap;
            for (int q = 0; q <= dg::kItemClasses; ++q) b.cls[q] = t.cls[q];
            for (int q = 0; q < dg::kItemClasses; ++q) b.ccap[q] = t.ccap[q];
            double ms_min = 1e300;
            for (int trial = 0; trial < 3; ++trial) {
                float ms = 0.f;
                CK(st.tune(b, reps, s, &ms));
                ms_min = std::min(ms_min, static_cast<double>(ms));
            }
            if (ms_min < best_ms) {
                best_ms = ms_min;
                best = cand;
            }
        }
        for (int o : co.second) chosen[TuneKey{o, c->mixed ? 1 : 0, c->pc.ns ? 1 : 0, c->nodes}] = best;
    }
    titems.free();
    telems.free();
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        load_tune_file_locked();
        for (const auto& kv : chosen) g_tune[kv.first] = kv.second;
        save_tune_file_locked();
    }
    CK(cudaMemcpyAsync(c->Q.p, q0.p, sizeof(double) * n5, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(c->G.p, g0.p, sizeof(double) * n5, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(st.QDot.p, d0.p, sizeof(R) * n5, cudaMemcpyDeviceToDevice, s));
    CK(cudaStreamSynchronize(s));
    q0.free();
    g0.free();
    d0.free();
    const ItemTable t = build_items(c->h_eord, c->h_ecase, -1, c->mixed, c->pc.ns != 0, c->nodes);
    if ((rc = apply_items(c, st, t))) return rc;
    CK(stage(c, dg::kTraces, 0.0, 0));  // Q traces of the restored state
    CK(cudaStreamSynchronize(s));
    return DG_OK;
}

}  // namespace

int autotune(dg_ctx* c, int reps) {
    if (reps < 1) return h3d::fail(DG_ERR_INVALID, "reps must be positive");
    return c->mixed ? autotune_store(c, c->v32, reps) : autotune_store(c, c->v64, reps);
}

}  // namespace h3dvar
