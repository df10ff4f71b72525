// C ABI of the GB300 DGSEM right-hand side (include/horses3d_gb300.h): context set-up, state
// transfer, the RK3 driver, CUDA-graph replay of whole steps and the device reductions.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../host/spectral.hpp"
#include "../host/status.hpp"
#include "dg_context.cuh"

using dg::Args;

using h3dctx::cuda_fail;
using h3dctx::DevBuf;
using h3dctx::Store;

namespace {

// The face point (i, j) whose leftIndexes2Right image is (ii, jj) (MeshTypes.f90:70-107 inverted).
void right_to_left(int ii, int jj, int N, int rot, int& i, int& j) {
    switch (rot) {
        case 0: i = ii; j = jj; break;
        case 1: i = jj; j = N - ii; break;
        case 2: i = N - ii; j = N - jj; break;
        case 3: i = N - jj; j = ii; break;
        case 4: i = jj; j = ii; break;
        case 5: i = N - ii; j = jj; break;
        case 6: i = N - jj; j = N - ii; break;
        default: i = ii; j = N - jj; break;
    }
}

}  // namespace

namespace {

template <typename R>
int upload_convert(DevBuf<R>& dst, const double* src, size_t n, cudaStream_t s) {
    CK(dst.alloc(n));
    if (sizeof(R) == sizeof(double)) {
        CK(cudaMemcpyAsync(dst.p, src, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    } else {
        std::vector<R> tmp(n);
        for (size_t i = 0; i < n; ++i) tmp[i] = static_cast<R>(src[i]);
        CK(cudaMemcpyAsync(dst.p, tmp.data(), sizeof(R) * n, cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));
    }
    return DG_OK;
}

template <typename R>
int setup_store(dg_ctx* c, Store<R>& st, const dg_mesh_desc* m) {
    const size_t nd = static_cast<size_t>(c->ndof);
    const size_t nfp = static_cast<size_t>(c->F) * c->P * c->P;
    const size_t nslot = c->n_slots();
    int rc;
    if ((rc = upload_convert(st.ja_xi, m->ja_xi, 3 * nd, c->stream))) return rc;
    if ((rc = upload_convert(st.ja_eta, m->ja_eta, 3 * nd, c->stream))) return rc;
    if ((rc = upload_convert(st.ja_zeta, m->ja_zeta, 3 * nd, c->stream))) return rc;
    if ((rc = upload_convert(st.jac, m->jacobian, nd, c->stream))) return rc;
    if ((rc = upload_convert(st.inv_jac, m->inv_jacobian, nd, c->stream))) return rc;
    // face geometry in face order, one component after the other (coalesced per component)
    {
        std::vector<double> soa(3 * nfp);
        const double* src[3] = {m->face_normal, m->face_t1, m->face_t2};
        DevBuf<R>* dst[3] = {&st.fn, &st.ft1, &st.ft2};
        for (int a = 0; a < 3; ++a) {
            for (size_t fp = 0; fp < nfp; ++fp)
                for (int c3 = 0; c3 < 3; ++c3) soa[c3 * nfp + fp] = src[a][3 * fp + c3];
            if ((rc = upload_convert(*dst[a], soa.data(), 3 * nfp, c->stream))) return rc;
            CK(cudaStreamSynchronize(c->stream));
        }
    }
    if ((rc = upload_convert(st.fj, m->face_jacobian, nfp, c->stream))) return rc;
    // per-slot geometry (n, Jf) in each side's own face coordinates
    {
        const int P = c->P, P2 = P * P;
        std::vector<double> sg(4 * nslot * P2);
        for (int f = 0; f < c->F; ++f)
            for (int side = 0; side < 2; ++side) {
                if (m->face_elem[2 * f + side] < 0) continue;  // boundary face: one side
                const size_t sl = 6 * static_cast<size_t>(m->face_elem[2 * f + side]) + (m->face_side[2 * f + side] - 1);
                for (int cb = 0; cb < P; ++cb)
                    for (int ca = 0; ca < P; ++ca) {
                        int i = ca, j = cb;
                        if (side == 1) right_to_left(ca, cb, P - 1, m->face_rotation[f], i, j);
                        const size_t fp = static_cast<size_t>(f) * P2 + i + P * j;
                        const int p = ca + P * cb;
                        for (int c3 = 0; c3 < 3; ++c3) sg[(sl * 4 + c3) * P2 + p] = m->face_normal[3 * fp + c3];
                        sg[(sl * 4 + 3) * P2 + p] = m->face_jacobian[fp];
                    }
            }
        if ((rc = upload_convert(st.sgeo, sg.data(), 4 * nslot * P2, c->stream))) return rc;
        CK(cudaStreamSynchronize(c->stream));
    }
    {  // boundary conditions in this precision
        std::vector<dg::BoundaryR<R>> b(c->bcs.size());
        for (size_t k = 0; k < c->bcs.size(); ++k) b[k] = dg::make_boundary<R>(c->bcs[k], c->pc);
        CK(st.bcs.upload(b.data(), b.size(), c->stream));
    }
    CK(st.QDot.alloc(5 * nd));
    CK(cudaMemsetAsync(st.QDot.p, 0, sizeof(R) * 5 * nd, c->stream));
    const bool ns = c->phys.navier_stokes != 0;
    CK(st.Ux.alloc(ns ? 5 * nd : 0));
    CK(st.Uy.alloc(ns ? 5 * nd : 0));
    CK(st.Uz.alloc(ns ? 5 * nd : 0));
    const size_t P2s = static_cast<size_t>(c->P) * c->P;
    CK(st.QF.alloc(5 * nslot * P2s));
    CK(st.FV.alloc(ns ? 5 * nslot * P2s : 0));
    CK(st.FS.alloc(5 * nslot * P2s));

    Args<R>& a = st.args;
    std::memset(&a, 0, sizeof(a));
    a.K = c->K;
    a.F = c->F;
    a.ph = dg::make_phys<R>(c->pc);
    const h3d::NodalStorage& ns_ = h3d::nodal_storage(c->nodes, c->P - 1);
    for (int i = 0; i < c->P; ++i) {
        for (int l = 0; l < c->P; ++l) {
            a.ops.D[i * dg::kMaxP + l] = static_cast<R>(ns_.D[i * c->P + l]);
            a.ops.hatD[i * dg::kMaxP + l] = static_cast<R>(ns_.hatD[i * c->P + l]);
            a.ops.sharpD[i * dg::kMaxP + l] = c->nodes == 1 ? static_cast<R>(ns_.sharpD[i * c->P + l]) : R(0);
        }
        a.ops.vL[i] = static_cast<R>(ns_.vL[i]);
        a.ops.vR[i] = static_cast<R>(ns_.vR[i]);
        a.ops.bL[i] = static_cast<R>(ns_.bL[i]);
        a.ops.bR[i] = static_cast<R>(ns_.bR[i]);
    }
    a.inviscid = c->opt.inviscid;
    a.source = c->opt.source;
    a.ja_xi = st.ja_xi.p; a.ja_eta = st.ja_eta.p; a.ja_zeta = st.ja_zeta.p;
    a.jac = st.jac.p; a.inv_jac = st.inv_jac.p;
    a.x = c->x.p;
    a.face_elem = c->face_elem.p; a.face_side = c->face_side.p; a.face_rot = c->face_rot.p;
    a.fn = st.fn.p; a.ft1 = st.ft1.p; a.ft2 = st.ft2.p; a.fj = st.fj.p;
    a.nb_slot = c->nb_slot.p; a.nb_map = c->nb_map.p; a.sgeo = st.sgeo.p;
    a.Q = c->Q.p; a.G = c->G.p; a.QDot = st.QDot.p;
    a.Ux = st.Ux.p; a.Uy = st.Uy.p; a.Uz = st.Uz.p;
    a.QF = st.QF.p; a.FV = st.FV.p; a.FS = st.FS.p;
    a.nsp = static_cast<int64_t>(nslot) * c->P * c->P;
    a.time = c->scal.p;
    a.dt = c->scal.p + 1;
    a.src_gm1 = c->pc.gm1;
    a.src_gM2 = c->pc.gammaM2;
    dg::source_constants(c->opt.source, c->phys.mach, c->phys.reynolds, c->phys.prandtl, c->pc.ns, &a.src_mu,
                         &a.src_kappa);
    a.err = c->err_flag.p;
    a.bc = st.bcs.p;
    return DG_OK;
}

cudaError_t run_stage(dg_ctx* c, int stage, double tshift, int flags) {
    if (c->var) return h3dvar::stage(c, stage, tshift, flags);
    if (c->mixed) return c->s32.stage(c->s32.args, stage, tshift, flags, c->stream);
    return c->s64.stage(c->s64.args, stage, tshift, flags, c->stream);
}

// Queue one RK3 step (time and dt are read from device memory). The last stage keeps its QDot for
// the residuals, as TakeRK3Step leaves the third stage's QDot in storage.
// fuse_monitor: the last stage's update writes the elements' residual records; with fused_dt (CFL
// steps) the first stage's volume kernel writes the time-step estimates and the step's dt is formed
// between the first stage's volume and flux kernels (enqueue_max_dt_fused).
cudaError_t enqueue_max_dt_fused(dg_ctx* c, double cfl, double dcfl);
cudaError_t enqueue_step(dg_ctx* c, bool fuse_monitor = false, bool fused_dt = false, double cfl = 0.0,
                         double dcfl = 0.0) {
    static const double b[3] = {0.0, 1.0 / 3.0, 3.0 / 4.0};
    for (int k = 0; k < 3; ++k) {
        const int last = dg::kWriteQDot | (c->keep_grad ? dg::kStoreGrad : 0) | (fuse_monitor ? dg::kFuseMonitor : 0);
        cudaError_t e;
        if (k == 0 && fused_dt) {
            e = run_stage(c, 0, b[0], dg::kVolumeOnly | dg::kEstimateDt);
            if (e == cudaSuccess) e = enqueue_max_dt_fused(c, cfl, dcfl);
            if (e == cudaSuccess) e = run_stage(c, 0, b[0], dg::kSurfaceOnly);
        } else {
            e = run_stage(c, k, b[k], k == 2 ? last : 0);
        }
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// The monitored time loop takes its residuals and NaN test from the last stage's update and its
// MaxTimeStep estimate from the first stage's volume kernel (uniform orders with the one-element
// kernels, whole meshes, the CUDA-core volume form).
bool fused_monitor(const dg_ctx* c) {
    if (c->var || c->n_ghost != 0) return false;
    if (c->mixed && c->s32.args.tc) return false;
    return c->mixed ? c->s32.mon.dt != nullptr : c->s64.mon.dt != nullptr;
}

dg::DtArgs dt_args(dg_ctx* c, double cfl, double dcfl) {
    dg::DtArgs d;
    d.ndof = c->ndof;
    d.cfl = cfl;
    d.dcfl = dcfl;
    for (int r = 0; r < 3; ++r) { d.dxi[r] = c->dxi[r]; d.dxi2[r] = c->dxi[r] * c->dxi[r]; }
    d.ns = c->pc.ns;
    d.gamma = c->pc.gamma; d.gm1 = c->pc.gm1; d.gammaM2 = c->pc.gammaM2;
    d.S_div_TRef = c->pc.S_div_TRef; d.TReNorm = c->pc.TReNorm;
    d.Q = c->Q.p;
    d.red = c->red.p;
    return d;
}

// Points the kernel arguments at the monitor records and the time-step constants of (cfl, dcfl).
int setup_fused_monitor(dg_ctx* c, double cfl, double dcfl) {
    if (!c->mon_part.p) CK(c->mon_part.alloc(8 * static_cast<size_t>(c->K)));
    const dg::DtConst32 c32 = dg::dt_const32(cfl, dcfl, c->dxi, c->pc.gamma, c->pc.gm1, c->pc.gammaM2, c->pc.S_div_TRef,
                                             c->pc.TReNorm, c->pc.ns);
    c->s32.args.mon = c->mon_part.p;
    c->s32.args.dtc = c32;
    c->s64.args.mon = c->mon_part.p;
    c->s64.args.dtc = c32;
    return DG_OK;
}

cudaError_t enqueue_max_dt_fused(dg_ctx* c, double cfl, double dcfl) {
    const dg::DtArgs d = dt_args(c, cfl, dcfl);
    cudaError_t e = c->mixed ? c->s32.mon.dt(c->s32.args, d, c->stream) : c->s64.mon.dt(c->s64.args, d, c->stream);
    if (e != cudaSuccess) return e;
    dg::k_dt_final<<<1, 1, 0, c->stream>>>(c->red.p, c->scal.p + 1);
    return cudaGetLastError();
}

cudaError_t enqueue_max_dt(dg_ctx* c, double cfl, double dcfl) {
    if (c->var) return h3dvar::enqueue_max_dt(c, cfl, dcfl);
    const dg::DtArgs d = dt_args(c, cfl, dcfl);
    const dg::DtConst32 c32 = dg::dt_const32(cfl, dcfl, c->dxi, d.gamma, d.gm1, d.gammaM2, d.S_div_TRef, d.TReNorm, d.ns);
    const int blocks = dg::kDtBlocks;
    if (c->mixed) {
        const Store<float>& st = c->s32;
        dg::k_dt_estimate<float><<<blocks, 256, 0, c->stream>>>(c32, c->ndof, c->Q.p, st.ja_xi.p, st.ja_eta.p,
                                                                 st.ja_zeta.p, st.jac.p, c->red.p, c->dt_bmin.p);
        dg::k_dt_exact<float><<<blocks, 256, 0, c->stream>>>(d, c32, st.ja_xi.p, st.ja_eta.p, st.ja_zeta.p, st.jac.p,
                                                             c->dt_bmin.p);
    } else {
        const Store<double>& st = c->s64;
        dg::k_dt_estimate<double><<<blocks, 256, 0, c->stream>>>(c32, c->ndof, c->Q.p, st.ja_xi.p, st.ja_eta.p,
                                                                  st.ja_zeta.p, st.jac.p, c->red.p, c->dt_bmin.p);
        dg::k_dt_exact<double><<<blocks, 256, 0, c->stream>>>(d, c32, st.ja_xi.p, st.ja_eta.p, st.ja_zeta.p, st.jac.p,
                                                              c->dt_bmin.p);
    }
    dg::k_dt_final<<<1, 1, 0, c->stream>>>(c->red.p, c->scal.p + 1);
    return cudaGetLastError();
}

// Every case's step start time and dt (one case unless the context is a batch).
// Reads and clears the device flag a kernel sets when a bounded wait gave up (after a synchronise).
int check_device_error(dg_ctx* c) {
    if (!c->err_flag.p) return DG_OK;
    int flag = 0;
    CK(cudaMemcpy(&flag, c->err_flag.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (!flag) return DG_OK;
    CK(cudaMemset(c->err_flag.p, 0, sizeof(int)));
    return h3d::fail(DG_ERR_TIMEOUT, "a kernel's bounded wait for a bulk copy gave up; the step is incomplete");
}

int set_scalars(dg_ctx* c, double t, double dt) {
    const int n = c->n_cases;
    for (int k = 0; k < n; ++k) {
        c->h_scal[k] = t;
        c->h_scal[n + k] = dt;
    }
    CK(cudaMemcpyAsync(c->scal.p, c->h_scal, 2 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    return DG_OK;
}

}  // namespace

namespace h3dctx {

// A boundary face (face_elem[2f+1] == -1) of a mesh description: one element side, a valid
// condition index and a supported condition type.
int validate_boundary_face(const dg_mesh_desc* m, int f) {
    if (!m->face_boundary || !m->boundaries)
        return h3d::fail(DG_ERR_INVALID, "a boundary face needs face_boundary and the boundaries table");
    const int b = m->face_boundary[f];
    if (b < 0 || b >= m->n_boundaries) return h3d::fail(DG_ERR_INVALID, "face_boundary outside 0..n_boundaries-1");
    const int t = m->boundaries[b].type;
    if (t < DG_BC_NO_SLIP_WALL || t > DG_BC_OUTFLOW) return h3d::fail(DG_ERR_UNSUPPORTED, "boundary condition type");
    if (m->face_rotation[f] != 0) return h3d::fail(DG_ERR_INVALID, "a boundary face has rotation 0");
    return DG_OK;
}

}  // namespace h3dctx

namespace {

using h3dctx::validate_boundary_face;

int validate(const dg_mesh_desc* m, const dg_physics* ph, const dg_options* op, int n_ghost) {
    if (!m || !ph || !op) return h3d::fail(DG_ERR_INVALID, "null argument");
    if (m->n_elements < 1 || m->n_faces < 1) return h3d::fail(DG_ERR_INVALID, "empty mesh");
    if (!m->order || !m->x || !m->ja_xi || !m->ja_eta || !m->ja_zeta || !m->jacobian || !m->inv_jacobian ||
        !m->face_elem || !m->face_side || !m->face_rotation || !m->face_nf || !m->face_normal || !m->face_t1 ||
        !m->face_t2 || !m->face_jacobian)
        return h3d::fail(DG_ERR_INVALID, "mesh description has a null array");
    if (m->node_type != DG_NODES_GAUSS && m->node_type != DG_NODES_GAUSS_LOBATTO)
        return h3d::fail(DG_ERR_INVALID, "unknown node type");
    const int N = m->order[0];
    for (int e = 0; e < m->n_elements + n_ghost; ++e)
        for (int d = 0; d < 3; ++d)
            if (m->order[3 * e + d] != N)
                return h3d::fail(DG_ERR_UNSUPPORTED, "the GPU path needs one isotropic order on every element");
    if (N + 1 < 2 || N + 1 > dg::kMaxP) return h3d::fail(DG_ERR_UNSUPPORTED, "polynomial order outside 1..7");
    int64_t sides = 0;
    for (int f = 0; f < m->n_faces; ++f) {
        if (m->face_nf[2 * f] != N || m->face_nf[2 * f + 1] != N)
            return h3d::fail(DG_ERR_INVALID, "face order differs from the element order");
        if (m->face_rotation[f] < 0 || m->face_rotation[f] > 7) return h3d::fail(DG_ERR_INVALID, "face rotation outside 0..7");
        const bool boundary = m->face_elem[2 * f + 1] < 0;
        if (boundary) {
            int rc = validate_boundary_face(m, f);
            if (rc) return rc;
        }
        int ghosts = 0;
        for (int s = 0; s < (boundary ? 1 : 2); ++s) {
            const int e = m->face_elem[2 * f + s], side = m->face_side[2 * f + s];
            if (e < 0 || e >= m->n_elements + n_ghost || side < 1 || side > 6)
                return h3d::fail(DG_ERR_INVALID, "face connectivity out of range");
            if (e < m->n_elements) ++sides;
            else ++ghosts;
        }
        if (ghosts > (boundary ? 0 : 1))
            return h3d::fail(DG_ERR_INVALID, "a face of a partition must have one of its own elements");
    }
    if (sides != 6 * static_cast<int64_t>(m->n_elements))
        return h3d::fail(DG_ERR_INVALID, "the faces do not cover every element side once");
    if (ph->mach <= 0.0) return h3d::fail(DG_ERR_INVALID, "Mach number must be positive");
    if (ph->navier_stokes && ph->reynolds <= 0.0) return h3d::fail(DG_ERR_INVALID, "Reynolds number must be positive");
    if (op->inviscid != DG_INVISCID_STANDARD && op->inviscid != DG_INVISCID_SPLIT)
        return h3d::fail(DG_ERR_UNSUPPORTED, "inviscid discretization");
    if (op->inviscid == DG_INVISCID_SPLIT && m->node_type != DG_NODES_GAUSS_LOBATTO)
        return h3d::fail(DG_ERR_INVALID, "the split form needs Gauss-Lobatto nodes");
    if (op->riemann < DG_RIEMANN_ROE || op->riemann > DG_RIEMANN_U_DISS) return h3d::fail(DG_ERR_UNSUPPORTED, "riemann solver");
    if (op->averaging < DG_AVG_STANDARD || op->averaging > DG_AVG_CHANDRASEKAR)
        return h3d::fail(DG_ERR_UNSUPPORTED, "averaging");
    if (op->precision != DG_PRECISION_FP64 && op->precision != DG_PRECISION_MIXED &&
        op->precision != DG_PRECISION_MIXED_TC)
        return h3d::fail(DG_ERR_UNSUPPORTED, "precision");
    if (op->precision == DG_PRECISION_MIXED_TC &&
        (N != 5 || m->node_type != DG_NODES_GAUSS || op->inviscid != DG_INVISCID_STANDARD ||
         (ph->navier_stokes && op->gradient_variables != DG_GRADVARS_STATE)))
        return h3d::fail(DG_ERR_UNSUPPORTED,
                         "the tensor-core form needs N = 5 Gauss nodes, the standard volume form and state gradients");
    if (op->source < DG_SOURCE_NONE || op->source > DG_SOURCE_MMS_LAMB_VECTOR)
        return h3d::fail(DG_ERR_UNSUPPORTED, "source");
    if (op->gradient_variables < DG_GRADVARS_STATE || op->gradient_variables > DG_GRADVARS_ENERGY)
        return h3d::fail(DG_ERR_UNSUPPORTED, "gradient variables");
    return DG_OK;
}

}  // namespace

extern "C" {

int dg_device_count(int* count) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (count) *count = (e == cudaSuccess) ? n : 0;
    if (e != cudaSuccess) return h3d::fail(DG_ERR_NODEVICE, cudaGetErrorString(e));
    return DG_OK;
}

namespace {

int create_uniform(const dg_mesh_desc* m, int n_ghost, const dg_physics* ph, const dg_options* op, dg_ctx** out);

}  // namespace

int dg_create(const dg_mesh_desc* m, const dg_physics* ph, const dg_options* op, dg_ctx** out) {
    if (!out) return h3d::fail(DG_ERR_INVALID, "null output pointer");
    *out = nullptr;
    if (m && ph && op && h3dvar::needs_variable_path(m)) return h3dvar::create(1, m, ph, op, out);
    return create_uniform(m, 0, ph, op, out);
}

int dg_create_partition(const dg_mesh_desc* m, int32_t n_ghost, const dg_physics* ph, const dg_options* op,
                        dg_ctx** out) {
    if (!out) return h3d::fail(DG_ERR_INVALID, "null output pointer");
    *out = nullptr;
    if (n_ghost < 0) return h3d::fail(DG_ERR_INVALID, "negative ghost element count");
    if (m && m->n_elements > 0 && m->order) {
        const int N = m->order[0];
        for (int64_t q = 0; q < 3 * (static_cast<int64_t>(m->n_elements) + n_ghost); ++q)
            if (m->order[q] != N)
                return h3d::fail(DG_ERR_UNSUPPORTED, "element partitions need one isotropic order on every element");
    }
    return create_uniform(m, n_ghost, ph, op, out);
}

}  // extern "C"

namespace {

int create_uniform(const dg_mesh_desc* m, int n_ghost, const dg_physics* ph, const dg_options* op, dg_ctx** out) {
    int rc = validate(m, ph, op, n_ghost);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return h3d::fail(DG_ERR_NODEVICE, "no CUDA device visible");
    auto* c = new dg_ctx();
    c->phys = *ph;
    c->opt = *op;
    if (m->n_boundaries > 0 && m->boundaries) c->bcs.assign(m->boundaries, m->boundaries + m->n_boundaries);
    c->K = m->n_elements;
    c->n_ghost = n_ghost;
    c->F = m->n_faces;
    c->P = m->order[0] + 1;
    c->nodes = m->node_type;
    c->ndof = static_cast<int64_t>(c->K) * c->P * c->P * c->P;
    c->mixed = op->precision == DG_PRECISION_MIXED || op->precision == DG_PRECISION_MIXED_TC;
    // PhysicsStorage_NS.f90:186-290,413-429 (air, Sutherland defaults)
    dg::PhysConst& pc = c->pc;
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
    const h3d::NodalStorage& nsx = h3d::nodal_storage(c->nodes, c->P - 1);
    for (int d = 0; d < 3; ++d) c->dxi[d] = 1.0 / std::fabs(nsx.x[1] - nsx.x[0]);

    auto bail = [&](int code) {
        dg_destroy(c);
        return code;
    };
    cudaError_t e;
    if ((e = cudaGetDevice(&c->device)) != cudaSuccess) return bail(cuda_fail(e, "cudaGetDevice"));
    if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return bail(cuda_fail(e, "cudaStreamCreate"));
    if ((e = cudaMallocHost(reinterpret_cast<void**>(&c->h_scal), 8 * sizeof(double))) != cudaSuccess)
        return bail(cuda_fail(e, "cudaMallocHost"));
    const size_t nd = static_cast<size_t>(c->ndof);
    if ((e = c->Q.alloc(5 * nd)) != cudaSuccess) return bail(cuda_fail(e, "alloc Q"));
    if ((e = c->G.alloc(5 * nd)) != cudaSuccess) return bail(cuda_fail(e, "alloc G"));
    if ((e = c->scal.alloc(4)) != cudaSuccess) return bail(cuda_fail(e, "alloc scalars"));
    if ((e = c->red.alloc(8)) != cudaSuccess) return bail(cuda_fail(e, "alloc reductions"));
    if ((e = c->nan_flag.alloc(1)) != cudaSuccess) return bail(cuda_fail(e, "alloc flag"));
    if ((e = c->err_flag.alloc(1)) != cudaSuccess || (e = cudaMemset(c->err_flag.p, 0, sizeof(int))) != cudaSuccess)
        return bail(cuda_fail(e, "alloc error flag"));
    if ((e = c->x.alloc(3 * nd)) != cudaSuccess) return bail(cuda_fail(e, "alloc x"));
    if ((e = cudaMemcpyAsync(c->x.p, m->x, sizeof(double) * 3 * nd, cudaMemcpyHostToDevice, c->stream)) != cudaSuccess)
        return bail(cuda_fail(e, "copy x"));
    if ((e = cudaMemsetAsync(c->G.p, 0, sizeof(double) * 5 * nd, c->stream)) != cudaSuccess) return bail(cuda_fail(e, "memset G"));
    if ((e = cudaMemsetAsync(c->Q.p, 0, sizeof(double) * 5 * nd, c->stream)) != cudaSuccess) return bail(cuda_fail(e, "memset Q"));
    // reduction slots start at "+infinity" for the dt minimum
    {
        unsigned long long init[8];
        const double big = 1.0e300;
        unsigned long long bb;
        std::memcpy(&bb, &big, 8);
        for (int i = 0; i < 8; ++i) init[i] = i < 2 ? bb : 0ull;
        init[7] = dg::kDtEstimateInit;
        if ((e = cudaMemcpy(c->red.p, init, sizeof(init), cudaMemcpyHostToDevice)) != cudaSuccess)
            return bail(cuda_fail(e, "init reductions"));
    }
    if ((e = c->dt_bmin.alloc(2 * dg::kDtBlocks)) != cudaSuccess) return bail(cuda_fail(e, "alloc dt chunks"));
    if ((e = c->face_elem.alloc(2 * c->F)) != cudaSuccess) return bail(cuda_fail(e, "alloc faces"));
    if ((e = c->face_side.alloc(2 * c->F)) != cudaSuccess) return bail(cuda_fail(e, "alloc faces"));
    if ((e = c->face_rot.alloc(c->F)) != cudaSuccess) return bail(cuda_fail(e, "alloc faces"));
    std::vector<int> fside(m->face_side, m->face_side + 2 * c->F);
    for (int f = 0; f < c->F; ++f)  // a boundary face's second entry holds its condition index on the device
        if (m->face_elem[2 * f + 1] < 0) fside[2 * f + 1] = m->face_boundary[f];
    if ((e = cudaMemcpyAsync(c->face_elem.p, m->face_elem, sizeof(int) * 2 * c->F, cudaMemcpyHostToDevice, c->stream)) ||
        (e = cudaMemcpyAsync(c->face_side.p, fside.data(), sizeof(int) * 2 * c->F, cudaMemcpyHostToDevice, c->stream)) ||
        (e = cudaMemcpyAsync(c->face_rot.p, m->face_rotation, sizeof(int) * c->F, cudaMemcpyHostToDevice, c->stream)) ||
        (e = cudaStreamSynchronize(c->stream)))
        return bail(cuda_fail(e, "copy faces"));
    {  // slot neighbour tables: the other side's slot and (rotation | own side << 3)
        const size_t nslot = c->n_slots();
        std::vector<int> nbs(nslot, -1), nbm(nslot, 0);
        std::vector<char> seen(nslot, 0);
        for (int f = 0; f < c->F; ++f)
            for (int side = 0; side < 2; ++side) {
                if (m->face_elem[2 * f + side] < 0) continue;
                const size_t sl = 6 * static_cast<size_t>(m->face_elem[2 * f + side]) + (m->face_side[2 * f + side] - 1);
                if (seen[sl]) return bail(h3d::fail(DG_ERR_INVALID, "an element side belongs to two faces"));
                seen[sl] = 1;
                if (m->face_elem[2 * f + 1] < 0) {  // boundary: -1 - condition index, own side 1
                    nbs[sl] = -1 - m->face_boundary[f];
                    nbm[sl] = 1 << 3;
                    continue;
                }
                const size_t so = 6 * static_cast<size_t>(m->face_elem[2 * f + 1 - side]) + (m->face_side[2 * f + 1 - side] - 1);
                nbs[sl] = static_cast<int>(so);
                nbm[sl] = m->face_rotation[f] | ((side + 1) << 3);
            }
        for (size_t sl = 0; sl < 6 * static_cast<size_t>(c->K); ++sl)  // every side of the own elements
            if (!seen[sl]) return bail(h3d::fail(DG_ERR_INVALID, "an element side has no face"));
        if ((e = c->nb_slot.alloc(nslot)) != cudaSuccess || (e = c->nb_map.alloc(nslot)) != cudaSuccess)
            return bail(cuda_fail(e, "alloc slot tables"));
        if ((e = cudaMemcpy(c->nb_slot.p, nbs.data(), sizeof(int) * nslot, cudaMemcpyHostToDevice)) != cudaSuccess ||
            (e = cudaMemcpy(c->nb_map.p, nbm.data(), sizeof(int) * nslot, cudaMemcpyHostToDevice)) != cudaSuccess)
            return bail(cuda_fail(e, "copy slot tables"));
    }
    if (c->mixed) {
        if ((rc = setup_store(c, c->s32, m))) return bail(rc);
        c->s32.args.tc = op->precision == DG_PRECISION_MIXED_TC ? 1 : 0;
        c->s32.mon = dg::monitor_fns_fp32(c->P, c->nodes == DG_NODES_GAUSS_LOBATTO);
        c->s32.stage = dg::stage_fn_fp32(c->P, c->nodes == DG_NODES_GAUSS_LOBATTO);
        c->s32.times = dg::times_fn_fp32(c->P, c->nodes == DG_NODES_GAUSS_LOBATTO);
    } else {
        if ((rc = setup_store(c, c->s64, m))) return bail(rc);
        c->s64.mon = dg::monitor_fns_fp64(c->P, c->nodes == DG_NODES_GAUSS_LOBATTO);
        c->s64.stage = dg::stage_fn_fp64(c->P, c->nodes == DG_NODES_GAUSS_LOBATTO);
        c->s64.times = dg::times_fn_fp64(c->P, c->nodes == DG_NODES_GAUSS_LOBATTO);
    }
    if ((e = run_stage(c, dg::kPrepare, 0.0, 0)) != cudaSuccess) return bail(cuda_fail(e, "kernel attributes"));
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) return bail(cuda_fail(e, "set-up"));
    *out = c;
    return DG_OK;
}

}  // namespace

extern "C" {

void dg_destroy(dg_ctx* c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    h3dctx::drop_graphs(c);
    if (c->var) h3dvar::release(c);
    c->s64.free();
    c->s32.free();
    c->Q.free(); c->G.free(); c->x.free(); c->scal.free(); c->red.free(); c->nan_flag.free(); c->err_flag.free();
    c->face_elem.free(); c->face_side.free(); c->face_rot.free(); c->nb_slot.free(); c->nb_map.free();
    c->mon.free(); c->mon_count.free(); c->esum.free(); c->dt_bmin.free();
    c->halo_send.free(); c->halo_recv.free(); c->mon_part.free();
    if (c->h_scal) cudaFreeHost(c->h_scal);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int64_t dg_ndof(const dg_ctx* c) { return c ? c->ndof : 0; }

int dg_upload_state(dg_ctx* c, const double* q) {
    if (!c || !q) return h3d::fail(DG_ERR_INVALID, "null argument");
    if (c->var) return h3dvar::upload(c, q);  // per-case constants live in device memory: graphs stay valid
    CK(cudaMemcpyAsync(c->Q.p, q, sizeof(double) * 5 * c->ndof, cudaMemcpyHostToDevice, c->stream));
    if (c->mixed) {
        // energy reference of the mixed form: the mean energy of the uploaded state (device sum)
        double e_ref = 0.0;
        int rc = h3dctx::device_mean_energy(c, 0, c->ndof, &e_ref);
        if (rc) return rc;
        if (!std::isfinite(e_ref)) return h3d::fail(DG_ERR_NAN, "NaN or Inf in the uploaded state");
        if (e_ref != c->s32.args.e_ref) {
            c->s32.args.e_ref = e_ref;
            dg::set_reference_energy(c->s32.args.ph, c->pc.gm1, e_ref);
            h3dctx::drop_graphs(c);  // kernel arguments changed
        }
    }
    CK(cudaMemsetAsync(c->G.p, 0, sizeof(double) * 5 * c->ndof, c->stream));
    CK(run_stage(c, dg::kTraces, 0.0, 0));  // face traces of the new state
    CK(cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int dg_set_energy_reference(dg_ctx* c, double e_ref) {
    if (!c) return h3d::fail(DG_ERR_INVALID, "null context");
    if (!std::isfinite(e_ref)) return h3d::fail(DG_ERR_INVALID, "the energy reference must be finite");
    if (c->var) return h3d::fail(DG_ERR_UNSUPPORTED, "energy reference of a uniform-order context only");
    if (!c->mixed) return DG_OK;
    if (e_ref != c->s32.args.e_ref) {
        c->s32.args.e_ref = e_ref;
        dg::set_reference_energy(c->s32.args.ph, c->pc.gm1, e_ref);
        h3dctx::drop_graphs(c);  // kernel arguments changed
    }
    CK(run_stage(c, dg::kTraces, 0.0, 0));  // the traces carry the energy relative to the reference
    CK(cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int dg_download(dg_ctx* c, int field, double* dst) {
    if (!c || !dst) return h3d::fail(DG_ERR_INVALID, "null argument");
    const size_t n = 5 * static_cast<size_t>(c->ndof);
    const void* src = nullptr;
    bool is_real = false;
    switch (field) {
        case DG_FIELD_Q: src = c->Q.p; break;
        case DG_FIELD_G: src = c->G.p; break;
        case DG_FIELD_QDOT:
            src = c->var ? (c->mixed ? static_cast<const void*>(c->v32.QDot.p) : c->v64.QDot.p)
                         : (c->mixed ? static_cast<const void*>(c->s32.QDot.p) : c->s64.QDot.p);
            is_real = true;
            break;
        case DG_FIELD_UX:
            src = c->var ? (c->mixed ? static_cast<const void*>(c->v32.Ux.p) : c->v64.Ux.p)
                         : (c->mixed ? static_cast<const void*>(c->s32.Ux.p) : c->s64.Ux.p);
            is_real = true;
            break;
        case DG_FIELD_UY:
            src = c->var ? (c->mixed ? static_cast<const void*>(c->v32.Uy.p) : c->v64.Uy.p)
                         : (c->mixed ? static_cast<const void*>(c->s32.Uy.p) : c->s64.Uy.p);
            is_real = true;
            break;
        case DG_FIELD_UZ:
            src = c->var ? (c->mixed ? static_cast<const void*>(c->v32.Uz.p) : c->v64.Uz.p)
                         : (c->mixed ? static_cast<const void*>(c->s32.Uz.p) : c->s64.Uz.p);
            is_real = true;
            break;
        default: return h3d::fail(DG_ERR_INVALID, "unknown field");
    }
    if (field >= DG_FIELD_UX && !c->phys.navier_stokes) return h3d::fail(DG_ERR_INVALID, "no gradients in Euler mode");
    if (is_real && c->mixed) {
        std::vector<float> tmp(n);
        CK(cudaMemcpyAsync(tmp.data(), src, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        for (size_t i = 0; i < n; ++i) dst[i] = tmp[i];
    } else {
        CK(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    return DG_OK;
}

int dg_rhs(dg_ctx* c, double t) {
    if (!c) return h3d::fail(DG_ERR_INVALID, "null context");
    int rc = set_scalars(c, t, 0.0);
    if (rc) return rc;
    CK(run_stage(c, -1, 0.0, dg::kStoreGrad | dg::kWriteQDot));
    CK(cudaStreamSynchronize(c->stream));
    return check_device_error(c);
}

int dg_partition_stage(dg_ctx* c, int stage, int phase, double t, double dt) {
    static const double b[3] = {0.0, 1.0 / 3.0, 3.0 / 4.0};
    if (!c) return h3d::fail(DG_ERR_INVALID, "null context");
    if (c->var) return h3d::fail(DG_ERR_UNSUPPORTED, "partition stages need a uniform-order context");
    if (stage < -1 || stage > 2 || phase < 0 || phase > 1) return h3d::fail(DG_ERR_INVALID, "stage or phase out of range");
    if (stage >= 0 && (!(dt > 0.0) || !std::isfinite(dt))) return h3d::fail(DG_ERR_INVALID, "dt must be positive and finite");
    CK(cudaStreamSynchronize(c->stream));  // the pinned scalar staging is free again
    int rc = set_scalars(c, t, stage >= 0 ? dt : 0.0);
    if (rc) return rc;
    const int part = phase == 0 ? dg::kVolumeOnly : dg::kSurfaceOnly;
    const int keep = stage < 0 ? (dg::kStoreGrad | dg::kWriteQDot) : (stage == 2 ? dg::kWriteQDot : 0);
    CK(run_stage(c, stage, stage >= 0 ? b[stage] : 0.0, part | keep));
    CK(cudaStreamSynchronize(c->stream));
    return check_device_error(c);
}

int dg_keep_gradients(dg_ctx* c, int on) {
    if (!c) return h3d::fail(DG_ERR_INVALID, "null context");
    if (c->var) return h3d::fail(DG_ERR_UNSUPPORTED, "keeping the step gradients needs a uniform-order context");
    if (!c->pc.ns) return h3d::fail(DG_ERR_INVALID, "an Euler context has no gradients");
    if ((on != 0) != c->keep_grad) {
        c->keep_grad = on != 0;
        h3dctx::drop_graphs(c);  // the captured steps change
    }
    return DG_OK;
}

int dg_rk3_step(dg_ctx* c, double t, double dt) {
    if (!c) return h3d::fail(DG_ERR_INVALID, "null context");
    if (!(dt > 0.0) || !std::isfinite(dt)) return h3d::fail(DG_ERR_INVALID, "dt must be positive and finite");
    int rc = set_scalars(c, t, dt);
    if (rc) return rc;
    dg::failed_launch()[0] = 0;
    {
        const cudaError_t e = enqueue_step(c);
        if (e != cudaSuccess)
            return h3d::fail(DG_ERR_CUDA, std::string("enqueue_step: ") + cudaGetErrorString(e) + " " + dg::failed_launch());
    }
    CK(cudaStreamSynchronize(c->stream));
    return check_device_error(c);
}

}  // extern "C"

namespace {

// Captures one whole RK3 step (optionally preceded by the device CFL dt) in a CUDA graph, once per
// (mode, cfl, dcfl).
int prepare_graph(dg_ctx* c, int mode, double cfl, double dcfl) {
    const bool stale = !c->graph || c->graph_mode != mode || c->graph_key[1] != cfl || c->graph_key[2] != dcfl;
    if (!stale) return DG_OK;
    if (c->graph) cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    if (mode == 1) e = enqueue_max_dt(c, cfl, dcfl);
    if (e == cudaSuccess) e = enqueue_step(c);
    if (e == cudaSuccess) {
        if (c->var) {
            e = h3dvar::enqueue_advance_time(c);
        } else {
            dg::k_advance_time<<<1, 1, 0, c->stream>>>(c->scal.p, c->scal.p + 1);
            e = cudaGetLastError();
        }
    }
    cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
    if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return cuda_fail(e, "capture RK3 step");
    }
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&c->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    c->graph_mode = mode;
    c->graph_key[1] = cfl;
    c->graph_key[2] = dcfl;
    return DG_OK;
}

// The step graph of dg_integrate: prepare_graph's step followed by ComputeMaxResiduals / checkForNan
// into the history row of the step (captured once per mode, cfl, dcfl and history buffer).
int prepare_monitor_graph(dg_ctx* c, int mode, double cfl, double dcfl) {
    const bool stale = !c->mgraph || c->mgraph_mode != mode || c->mgraph_key[1] != cfl || c->mgraph_key[2] != dcfl;
    if (!stale) return DG_OK;
    if (c->mgraph) cudaGraphExecDestroy(c->mgraph);
    c->mgraph = nullptr;
    cudaGraph_t g = nullptr;
    const bool fused = fused_monitor(c);
    if (fused) {
        int rc = setup_fused_monitor(c, cfl, dcfl);
        if (rc) return rc;
    }
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    if (mode == 1 && !fused) e = enqueue_max_dt(c, cfl, dcfl);
    if (e == cudaSuccess) e = enqueue_step(c, fused, fused && mode == 1, cfl, dcfl);
    if (e == cudaSuccess) {
        if (c->var) {
            e = h3dvar::enqueue_advance_time(c);
        } else {
            dg::k_advance_time<<<1, 1, 0, c->stream>>>(c->scal.p, c->scal.p + 1);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) {
        if (c->var) {
            e = h3dvar::enqueue_residuals(c);
            if (e == cudaSuccess) {
                dg::k_record_monitor<<<1, 1, 0, c->stream>>>(c->red.p, 8, c->vnan.p, c->n_cases, c->mon.p,
                                                             c->mon_count.p, c->mon_rows);
                e = cudaGetLastError();
            }
        } else {
            e = cudaMemsetAsync(c->red.p + 2, 0, 5 * sizeof(unsigned long long), c->stream);
            if (e == cudaSuccess) e = cudaMemsetAsync(c->nan_flag.p, 0, sizeof(int), c->stream);
            if (e == cudaSuccess && fused) {
                dg::k_monitor_fold<<<dg::kFoldBlocks, 256, 0, c->stream>>>(c->mon_part.p, c->K, c->red.p, c->nan_flag.p);
                dg::k_record_monitor<<<1, 1, 0, c->stream>>>(c->red.p, 0, c->nan_flag.p, 1, c->mon.p, c->mon_count.p,
                                                             c->mon_rows);
                e = cudaGetLastError();
            } else if (e == cudaSuccess) {
                if (c->mixed)
                    dg::k_residuals<float><<<152 * 4, 256, 0, c->stream>>>(c->ndof, c->s32.QDot.p, c->Q.p, c->red.p + 2,
                                                                           c->nan_flag.p);
                else
                    dg::k_residuals<double><<<152 * 4, 256, 0, c->stream>>>(c->ndof, c->s64.QDot.p, c->Q.p,
                                                                            c->red.p + 2, c->nan_flag.p);
                dg::k_record_monitor<<<1, 1, 0, c->stream>>>(c->red.p, 0, c->nan_flag.p, 1, c->mon.p, c->mon_count.p,
                                                             c->mon_rows);
                e = cudaGetLastError();
            }
        }
    }
    cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
    if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return cuda_fail(e, "capture monitored RK3 step");
    }
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&c->mgraph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    c->mgraph_mode = mode;
    c->mgraph_key[1] = cfl;
    c->mgraph_key[2] = dcfl;
    return DG_OK;
}

// n graph launches of one RK3 step (mode 0: the dt on the device; mode 1: MaxTimeStep first).
int run_graph(dg_ctx* c, int n, int mode, double cfl, double dcfl, double* ms) {
    int rc = prepare_graph(c, mode, cfl, dcfl);
    if (rc) return rc;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (ms) {
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        CK(cudaEventRecord(e0, c->stream));
    }
    for (int s = 0; s < n; ++s) CK(cudaGraphLaunch(c->graph, c->stream));
    if (ms) {
        CK(cudaEventRecord(e1, c->stream));
        CK(cudaEventSynchronize(e1));
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, e0, e1));
        *ms = t;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return check_device_error(c);
    }
    return DG_OK;
}

int steps_common(dg_ctx* c, int n, double t0, double dt, double cfl, double dcfl, double* t_end, double* ms) {
    if (!c || n < 0) return h3d::fail(DG_ERR_INVALID, "bad arguments");
    const int mode = dt > 0.0 ? 0 : 1;
    if (mode == 1 && !(cfl > 0.0)) return h3d::fail(DG_ERR_INVALID, "CFL stepping needs cfl > 0");
    int rc = set_scalars(c, t0, mode == 0 ? dt : 0.0);
    if (rc) return rc;
    if ((rc = run_graph(c, n, mode, cfl, dcfl, ms))) return rc;
    if (t_end) {
        CK(cudaMemcpyAsync(c->h_scal, c->scal.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        *t_end = c->h_scal[0];
        return check_device_error(c);
    }
    return DG_OK;
}

}  // namespace

extern "C" {

int dg_run_steps(dg_ctx* c, int n, double t0, double dt, double cfl, double dcfl, double* t_end) {
    return steps_common(c, n, t0, dt, cfl, dcfl, t_end, nullptr);
}

}  // extern "C"

namespace {

// dg_integrate / dg_batch_integrate from the current device clock (mode 0: each case's dt, mode 1:
// MaxTimeStep each step). t_end receives case 0's final time.
int integrate_core(dg_ctx* c, int n, int mode, double cfl, double dcfl, double* t_end, double* residuals,
                   int* nan_step) {
    if (nan_step) *nan_step = 0;
    if (n == 0) return DG_OK;
    const int nc = c->n_cases;
    if (n > c->mon_rows) {  // grow the history; the captured graph points at the old buffer
        c->mon.free();
        c->mon_rows = 0;
        CK(c->mon.alloc(static_cast<size_t>(n) * 6 * nc));
        if (!c->mon_count.p) CK(c->mon_count.alloc(1));
        c->mon_rows = n;
        if (c->mgraph) cudaGraphExecDestroy(c->mgraph);
        c->mgraph = nullptr;
    }
    int rc = prepare_monitor_graph(c, mode, cfl, dcfl);
    if (rc) return rc;
    CK(cudaMemsetAsync(c->mon_count.p, 0, sizeof(int), c->stream));
    for (int s = 0; s < n; ++s) CK(cudaGraphLaunch(c->mgraph, c->stream));
    std::vector<double> rows(static_cast<size_t>(n) * 6 * nc);
    CK(cudaMemcpyAsync(rows.data(), c->mon.p, sizeof(double) * rows.size(), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(c->h_scal, c->scal.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (t_end) *t_end = c->h_scal[0];
    rc = check_device_error(c);
    if (rc) return rc;
    int first = 0;
    for (int s = 0; s < n && !first; ++s)
        for (int k = 0; k < nc; ++k)
            if (rows[(static_cast<size_t>(s) * nc + k) * 6 + 5] != 0.0) first = s + 1;
    if (residuals)
        for (int s = 0; s < n; ++s)
            for (int k = 0; k < nc; ++k)
                for (int v = 0; v < 5; ++v)
                    residuals[(static_cast<size_t>(s) * nc + k) * 5 + v] = rows[(static_cast<size_t>(s) * nc + k) * 6 + v];
    if (nan_step) *nan_step = first;
    return first ? h3d::fail(DG_ERR_NAN, "NaN or Inf in Q after step " + std::to_string(first)) : DG_OK;
}

}  // namespace

extern "C" {

int dg_integrate(dg_ctx* c, int n, double t0, double dt, double cfl, double dcfl, double* t_end,
                 double* residuals, int* nan_step) {
    if (!c || n < 0) return h3d::fail(DG_ERR_INVALID, "bad arguments");
    const int mode = dt > 0.0 ? 0 : 1;
    if (mode == 1 && !(cfl > 0.0)) return h3d::fail(DG_ERR_INVALID, "CFL stepping needs cfl > 0");
    if (n == 0 && t_end) *t_end = t0;
    int rc = set_scalars(c, t0, mode == 0 ? dt : 0.0);
    if (rc) return rc;
    return integrate_core(c, n, mode, cfl, dcfl, t_end, residuals, nan_step);
}

int dg_time_steps(dg_ctx* c, int n, double t0, double dt, double cfl, double dcfl, double* ms) {
    if (!ms) return h3d::fail(DG_ERR_INVALID, "null argument");
    return steps_common(c, n, t0, dt, cfl, dcfl, nullptr, ms);
}

int dg_kernel_times(dg_ctx* c, int reps, double t0, double dt, double ms[5]) {
    if (!c || !ms || reps < 1) return h3d::fail(DG_ERR_INVALID, "bad arguments");
    int rc = set_scalars(c, t0, dt);
    if (rc) return rc;
    for (int kk = 0; kk < 5; ++kk) ms[kk] = 0.0;
    if (c->var) return h3dvar::kernel_times(c, reps, ms);
    if (c->mixed) CK(c->s32.times(c->s32.args, reps, c->stream, ms));
    else CK(c->s64.times(c->s64.args, reps, c->stream, ms));
    return DG_OK;
}

int dg_max_dt(dg_ctx* c, double cfl, double dcfl, double* dt) {
    if (!c || !dt) return h3d::fail(DG_ERR_INVALID, "null argument");
    CK(enqueue_max_dt(c, cfl, dcfl));
    const int n = c->n_cases;
    CK(cudaMemcpyAsync(c->h_scal + 2 * n, c->scal.p + n, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    double m = c->h_scal[2 * n];
    for (int k = 1; k < n; ++k) m = std::fmin(m, c->h_scal[2 * n + k]);
    *dt = m;  // a batch reports the smallest case dt; every case keeps its own on the device
    return DG_OK;
}

int dg_residuals(dg_ctx* c, double maxres[5], int* nan_found) {
    if (!c || !maxres) return h3d::fail(DG_ERR_INVALID, "null argument");
    if (c->var) {  // the maximum over the cases of a batch
        std::vector<double> r(5 * static_cast<size_t>(c->n_cases));
        std::vector<int> nan(c->n_cases);
        const int rc = h3dvar::residuals(c, r.data(), nan.data());
        if (rc != DG_OK && rc != DG_ERR_NAN) return rc;
        int any = 0;
        for (int v = 0; v < 5; ++v) maxres[v] = 0.0;
        for (int k = 0; k < c->n_cases; ++k) {
            for (int v = 0; v < 5; ++v) maxres[v] = std::fmax(maxres[v], r[5 * k + v]);
            any |= nan[k];
        }
        if (nan_found) *nan_found = any;
        return rc;
    }
    CK(cudaMemsetAsync(c->red.p + 2, 0, 5 * sizeof(unsigned long long), c->stream));
    CK(cudaMemsetAsync(c->nan_flag.p, 0, sizeof(int), c->stream));
    const int blocks = 152 * 4;
    if (c->mixed) dg::k_residuals<float><<<blocks, 256, 0, c->stream>>>(c->ndof, c->s32.QDot.p, c->Q.p, c->red.p + 2, c->nan_flag.p);
    else dg::k_residuals<double><<<blocks, 256, 0, c->stream>>>(c->ndof, c->s64.QDot.p, c->Q.p, c->red.p + 2, c->nan_flag.p);
    CK(cudaGetLastError());
    unsigned long long bits[5];
    int flag = 0;
    CK(cudaMemcpyAsync(bits, c->red.p + 2, sizeof(bits), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&flag, c->nan_flag.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int v = 0; v < 5; ++v) std::memcpy(&maxres[v], &bits[v], sizeof(double));
    if (nan_found) *nan_found = flag;
    return flag ? h3d::fail(DG_ERR_NAN, "NaN or Inf in Q") : DG_OK;
}

int dg_synchronize(dg_ctx* c) {
    if (!c) return h3d::fail(DG_ERR_INVALID, "null context");
    CK(cudaStreamSynchronize(c->stream));
    return DG_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ batches of cases ----------
extern "C" {

int dg_create_batch(int n_cases, const dg_mesh_desc* meshes, const dg_physics* phys, const dg_options* opts,
                    dg_ctx** out) {
    return h3dvar::create(n_cases, meshes, phys, opts, out);
}

int dg_batch_size(const dg_ctx* c) { return c ? c->n_cases : 0; }

int64_t dg_case_offset(const dg_ctx* c, int k) {
    if (!c || k < 0 || k > c->n_cases) return -1;
    if (!c->var) return k == 0 ? 0 : c->ndof;
    return c->case_ndof_off[k];
}

int dg_batch_set_clock(dg_ctx* c, const double* t, const double* dt) {
    if (!c || !t || !dt) return h3d::fail(DG_ERR_INVALID, "null argument");
    const int n = c->n_cases;
    for (int k = 0; k < n; ++k) {
        if (!std::isfinite(t[k]) || !(dt[k] >= 0.0) || !std::isfinite(dt[k]))
            return h3d::fail(DG_ERR_INVALID, "case times must be finite and dt non-negative");
        c->h_scal[k] = t[k];
        c->h_scal[n + k] = dt[k];
    }
    CK(cudaMemcpyAsync(c->scal.p, c->h_scal, 2 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int dg_batch_get_clock(dg_ctx* c, double* t, double* dt) {
    if (!c || !t || !dt) return h3d::fail(DG_ERR_INVALID, "null argument");
    const int n = c->n_cases;
    CK(cudaMemcpyAsync(c->h_scal, c->scal.p, 2 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (int k = 0; k < n; ++k) {
        t[k] = c->h_scal[k];
        dt[k] = c->h_scal[n + k];
    }
    return DG_OK;
}

int dg_batch_max_dt(dg_ctx* c, double cfl, double dcfl, double* dt) {
    if (!c || !dt) return h3d::fail(DG_ERR_INVALID, "null argument");
    CK(enqueue_max_dt(c, cfl, dcfl));
    const int n = c->n_cases;
    CK(cudaMemcpyAsync(dt, c->scal.p + n, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int dg_batch_residuals(dg_ctx* c, double* maxres, int* nan_found) {
    if (!c || !maxres) return h3d::fail(DG_ERR_INVALID, "null argument");
    if (!c->var) return dg_residuals(c, maxres, nan_found);
    return h3dvar::residuals(c, maxres, nan_found);
}

int dg_inject_fault(dg_ctx* c, int kind) {
    if (!c) return h3d::fail(DG_ERR_INVALID, "null context");
    if (kind != DG_FAULT_NONE && kind != DG_FAULT_TMA_WAIT) return h3d::fail(DG_ERR_INVALID, "unknown fault kind");
    if (c->var) return h3d::fail(DG_ERR_UNSUPPORTED, "the variable-order kernels have no bulk-copy waits");
    const uint32_t extra = kind == DG_FAULT_TMA_WAIT ? 16u : 0u;
    c->s32.args.extra_tx = extra;
    c->s64.args.extra_tx = extra;
    h3dctx::drop_graphs(c);  // the captured launches carry the old arguments
    return DG_OK;
}

int dg_autotune(dg_ctx* c, int reps) {
    if (!c) return h3d::fail(DG_ERR_INVALID, "null context");
    if (!c->var) return DG_OK;  // the uniform-order kernels have one fixed shape per order
    return h3dvar::autotune(c, reps);
}

int dg_batch_run_steps(dg_ctx* c, int n, double cfl, double dcfl, double* ms) {
    if (!c || n < 0) return h3d::fail(DG_ERR_INVALID, "bad arguments");
    return run_graph(c, n, cfl > 0.0 ? 1 : 0, cfl, dcfl, ms);
}

int dg_batch_integrate(dg_ctx* c, int n, double cfl, double dcfl, double* residuals, int* nan_step) {
    if (!c || n < 0) return h3d::fail(DG_ERR_INVALID, "bad arguments");
    return integrate_core(c, n, cfl > 0.0 ? 1 : 0, cfl, dcfl, nullptr, residuals, nan_step);
}

}  // extern "C"

// ------------------------------------------------------------------ solution files ------------
namespace {

// Element range, node range and orders of case k of a context.
struct CaseView {
    int e0 = 0, e1 = 0;
    int64_t g0 = 0, g1 = 0;
    std::vector<int32_t> orders;
    double mach = 0.0;
};

int case_view(const dg_ctx* c, int k, CaseView& v) {
    if (k < 0 || k >= c->n_cases) return h3d::fail(DG_ERR_INVALID, "case index out of range");
    if (!c->var) {
        v.e0 = 0;
        v.e1 = c->K;
        v.g0 = 0;
        v.g1 = c->ndof;
        v.orders.assign(3 * static_cast<size_t>(c->K), c->P - 1);
        v.mach = c->phys.mach;
        return DG_OK;
    }
    v.e0 = c->case_elem_off[k];
    v.e1 = c->case_elem_off[k + 1];
    v.g0 = c->case_ndof_off[k];
    v.g1 = c->case_ndof_off[k + 1];
    v.orders.resize(3 * static_cast<size_t>(v.e1 - v.e0));
    for (int e = v.e0; e < v.e1; ++e) {
        const int o = c->h_eord[e];
        v.orders[3 * (e - v.e0)] = (o & 255) - 1;
        v.orders[3 * (e - v.e0) + 1] = ((o >> 8) & 255) - 1;
        v.orders[3 * (e - v.e0) + 2] = ((o >> 16) & 255) - 1;
    }
    v.mach = c->case_mach[k];
    return DG_OK;
}

}  // namespace

extern "C" {

int dg_save_solution(dg_ctx* c, int k, const char* path, int iteration, double time, int with_gradients) {
    if (!c || !path) return h3d::fail(DG_ERR_INVALID, "null argument");
    CaseView v;
    int rc = case_view(c, k, v);
    if (rc) return rc;
    if (with_gradients && !c->phys.navier_stokes) return h3d::fail(DG_ERR_INVALID, "no gradients in Euler mode");
    const size_t n5 = 5 * static_cast<size_t>(c->ndof);
    std::vector<double> q(n5);
    if ((rc = dg_download(c, DG_FIELD_Q, q.data()))) return rc;
    std::vector<double> grad;
    if (with_gradients) {
        if ((rc = dg_rhs(c, time))) return rc;
        std::vector<double> ux(n5), uy(n5), uz(n5);
        if ((rc = dg_download(c, DG_FIELD_UX, ux.data())) || (rc = dg_download(c, DG_FIELD_UY, uy.data())) ||
            (rc = dg_download(c, DG_FIELD_UZ, uz.data())))
            return rc;
        grad.resize(3 * 5 * static_cast<size_t>(v.g1 - v.g0));
        int64_t off = v.g0;
        for (int e = 0; e < v.e1 - v.e0; ++e) {
            const int64_t np = static_cast<int64_t>(v.orders[3 * e] + 1) * (v.orders[3 * e + 1] + 1) * (v.orders[3 * e + 2] + 1);
            const std::vector<double>* src[3] = {&ux, &uy, &uz};
            for (int d = 0; d < 3; ++d)
                std::memcpy(grad.data() + 15 * (off - v.g0) + 5 * np * d, src[d]->data() + 5 * off, sizeof(double) * 5 * np);
            off += np;
        }
    }
    h3d_solution_header h;
    std::memset(&h, 0, sizeof(h));
    std::strncpy(h.name, path, sizeof(h.name));
    h.file_type = with_gradients ? 3 : 2;
    h.node_type = c->nodes == DG_NODES_GAUSS ? 1 : 2;
    h.n_elements = v.e1 - v.e0;
    h.iteration = iteration;
    h.time = time;
    // PhysicsStorage_NS.f90:290-310 reference values (air defaults)
    const double R = 287.15, T = 520.0 * 5.0 / 9.0;
    h.refs[0] = 1.4;
    h.refs[1] = R;
    h.refs[2] = v.mach * std::sqrt(1.4 * R * T);
    h.refs[3] = 101325.0 / (R * T);
    h.refs[4] = T;
    h.refs[5] = v.mach;
    return h3d_write_solution(path, &h, v.orders.data(), q.data() + 5 * v.g0, with_gradients ? grad.data() : nullptr);
}

int dg_load_solution(dg_ctx* c, int k, const char* path, int* iteration, double* time) {
    if (!c || !path) return h3d::fail(DG_ERR_INVALID, "null argument");
    CaseView v;
    int rc = case_view(c, k, v);
    if (rc) return rc;
    h3d_solution_header h;
    if ((rc = h3d_read_solution_header(path, &h))) return rc;
    if (h.file_type != 2 && h.file_type != 3)
        return h3d::fail(DG_ERR_UNSUPPORTED, std::string(path) + ": only solution files (types 2 and 3) are read");
    if (h.node_type != (c->nodes == DG_NODES_GAUSS ? 1 : 2))
        return h3d::fail(DG_ERR_INVALID, std::string(path) + ": the file was written for the other node type");
    std::vector<double> q(5 * static_cast<size_t>(c->ndof));
    if ((rc = dg_download(c, DG_FIELD_Q, q.data()))) return rc;
    if ((rc = h3d_read_solution(path, v.e1 - v.e0, v.orders.data(), q.data() + 5 * v.g0, nullptr))) return rc;
    if ((rc = dg_upload_state(c, q.data()))) return rc;
    if (iteration) *iteration = h.iteration;
    if (time) *time = h.time;
    return DG_OK;
}

}  // extern "C"
