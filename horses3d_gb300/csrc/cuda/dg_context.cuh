// Internal: the context behind the opaque dg_ctx handle of the C ABI, shared by the uniform-order
// path (dg_api.cu) and the variable-order / multi-case path (dg_var_api.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../host/status.hpp"
#include "dg_var.cuh"
#include "horses3d_gb300.h"

namespace h3dctx {

inline int cuda_fail(cudaError_t e, const char* where) {
    return h3d::fail(e == cudaErrorMemoryAllocation ? DG_ERR_NOMEM : DG_ERR_CUDA,
                     std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                                       \
    do {                                                               \
        cudaError_t e_ = (call);                                       \
        if (e_ != cudaSuccess) return h3dctx::cuda_fail(e_, #call);    \
    } while (0)

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t alloc(size_t count) {
        n = count;
        return cudaMalloc(reinterpret_cast<void**>(&p), sizeof(T) * (count ? count : 1));
    }
    cudaError_t upload(const T* src, size_t count, cudaStream_t s) {
        cudaError_t e = alloc(count);
        if (e != cudaSuccess) return e;
        if (count == 0) return cudaSuccess;
        e = cudaMemcpyAsync(p, src, sizeof(T) * count, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return e;
        return cudaStreamSynchronize(s);
    }
    void free() {
        if (p) cudaFree(p);
        p = nullptr;
    }
};

// Uniform-order path: everything one precision needs on the device.
template <typename R>
struct Store {
    DevBuf<R> ja_xi, ja_eta, ja_zeta, jac, inv_jac, fn, ft1, ft2, fj, sgeo;
    DevBuf<R> QDot, Ux, Uy, Uz, QF, FV, FS;
    DevBuf<dg::BoundaryR<R>> bcs;
    dg::Args<R> args;
    dg::StageFn<R> stage = nullptr;
    dg::KernelTimesFn<R> times = nullptr;
    dg::MonitorFns<R> mon{nullptr};  // fused time-loop monitor (the one-element-per-CTA orders)
    void free() {
        for (DevBuf<R>* b : {&ja_xi, &ja_eta, &ja_zeta, &jac, &inv_jac, &fn, &ft1, &ft2, &fj, &sgeo, &QDot, &Ux, &Uy,
                             &Uz, &QF, &FV, &FS})
            b->free();
        bcs.free();
    }
};

// Variable-order path: per-precision buffers.
template <typename R>
struct VStore {
    DevBuf<R> ja_xi, ja_eta, ja_zeta, jac, inv_jac, fn, ft1, ft2, fj, tset;
    DevBuf<R> QDot, Ux, Uy, Uz, QF, GF, UJ, FS;
    DevBuf<dg::OpsP<R>> ops;
    DevBuf<dg::PhysR<R>> ph;
    DevBuf<dg::BoundaryR<R>> bcs;
    dg::VArgs<R> args;
    dg::VStageFn<R> stage = nullptr;
    dg::VTimesFn<R> times = nullptr;
    dg::VTuneFn<R> tune = nullptr;
    void free() {
        for (DevBuf<R>* b : {&ja_xi, &ja_eta, &ja_zeta, &jac, &inv_jac, &fn, &ft1, &ft2, &fj, &tset, &QDot, &Ux, &Uy,
                             &Uz, &QF, &GF, &UJ, &FS})
            b->free();
        ops.free();
        ph.free();
        bcs.free();
    }
};

}  // namespace h3dctx

struct dg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int K = 0, F = 0, P = 0, nodes = 0;
    int64_t ndof = 0;
    // element partition: remote neighbours as ghost elements K .. K + n_ghost - 1, which own face
    // slots (filled by the halo exchange) but no nodes; 0 for a whole mesh
    int n_ghost = 0;
    size_t n_slots() const { return 6 * (static_cast<size_t>(K) + static_cast<size_t>(n_ghost)); }
    h3dctx::DevBuf<int> halo_send, halo_recv;  // slots packed for the neighbours / ghost slots filled
    int n_halo_send = 0, n_halo_recv = 0;
    dg_physics phys{};
    dg_options opt{};
    std::vector<dg_boundary> bcs;  // boundary conditions (variable-order path: of all cases, appended)
    std::vector<int> bc_case;      // variable-order path: the case of each boundary condition
    dg::PhysConst pc{};
    bool mixed = false;
    double dxi[3] = {0, 0, 0};
    h3dctx::DevBuf<double> Q, G, x, scal;    // scal: time[n_cases], then dt[n_cases]
    h3dctx::DevBuf<unsigned long long> red;  // uniform: [0..1] dt, [2..6] residuals; variable: 8 per case
    h3dctx::DevBuf<int> face_elem, face_side, face_rot, nan_flag, nb_slot, nb_map;
    h3dctx::DevBuf<int> err_flag;  // set by kernels whose bounded waits gave up
    h3dctx::DevBuf<double> esum;   // energy sums of the mixed form's reference (partials, then per case)
    h3dctx::DevBuf<float> dt_bmin;  // per-chunk minima of the MaxTimeStep estimate pass
    h3dctx::Store<double> s64;
    h3dctx::Store<float> s32;
    double* h_scal = nullptr;  // pinned staging for the per-case scalars (4 * n_cases doubles)
    cudaGraphExec_t graph = nullptr;
    double graph_key[3] = {0, 0, 0};  // (mode, cfl, dcfl) the graph was captured for
    int graph_mode = -1;
    // IntegrateInTime on the device (dg_integrate): the step graph with residual monitoring, and the
    // per-step history rows (per case: 5 residuals and a NaN flag) with their device row counter
    cudaGraphExec_t mgraph = nullptr;
    double mgraph_key[3] = {0, 0, 0};
    int mgraph_mode = -1;
    h3dctx::DevBuf<double> mon;
    h3dctx::DevBuf<int> mon_count;
    int mon_rows = 0;
    bool keep_grad = false;  // the last stage of every step stores the lifted gradients
    h3dctx::DevBuf<unsigned long long> mon_part;  // fused time-loop monitor: 8 words per element

    // variable-order / multi-case path
    bool var = false;
    int n_cases = 1;
    std::vector<int64_t> case_ndof_off;  // [n_cases + 1] node offsets of the cases
    std::vector<int> case_elem_off;      // [n_cases + 1] element offsets of the cases
    std::vector<double> case_mach;
    std::vector<dg::CaseConst> case_const;
    std::vector<dg::PhysConst> case_pc;
    h3dctx::DevBuf<int4> items, faces4;
    h3dctx::DevBuf<int> item_elems, eord, vnan;
    h3dctx::DevBuf<long long> eoff, soff, foff;
    h3dctx::DevBuf<dg::CaseConst> cc;
    h3dctx::DevBuf<double> dxi_table, gamma_M2;
    h3dctx::DevBuf<double> pstat;  // mixed form: momentum residual of the state at rest per unit pressure
    h3dctx::VStore<double> v64;
    h3dctx::VStore<float> v32;
    dg::Lanes lanes;  // side streams of the stage phases
    int n_items = 0;
    int cls[dg::kItemClasses + 1] = {};  // item class ranges (see dg::VArgs::cls)
    int ccap[dg::kItemClasses] = {};     // largest item per class
    std::vector<int> h_eord, h_ecase;    // per element: packed orders, case (to rebuild the items)
    // face lists: staged (Tset) faces and per-point faces grouped by point counts (see dg::VArgs)
    std::vector<int> h_nc, h_direct;
    h3dctx::DevBuf<int> nc_faces, direct_faces;
    int n_groups = 0;
    int gf0[dg::kMaxP * dg::kMaxP + 1] = {};
    int gp0[dg::kMaxP * dg::kMaxP + 1] = {};
    unsigned char gq1[dg::kMaxP * dg::kMaxP] = {};
    unsigned char gq2[dg::kMaxP * dg::kMaxP] = {};
};

namespace h3dctx {
// Mean of Q[5g+4] over [g0, g1) of the device state, summed in a fixed order (same bits for the same
// state), into *mean on the host.
inline int device_mean_energy(dg_ctx* c, int64_t g0, int64_t g1, double* mean) {
    if (!c->esum.p) CK(c->esum.alloc(dg::kSumBlocks + 1));
    dg::k_energy_partial<<<dg::kSumBlocks, 256, 0, c->stream>>>(g0, g1, c->Q.p, c->esum.p);
    dg::k_energy_final<<<1, 256, 0, c->stream>>>(c->esum.p, c->esum.p + dg::kSumBlocks);
    CK(cudaGetLastError());
    double sum = 0.0;
    CK(cudaMemcpyAsync(&sum, c->esum.p + dg::kSumBlocks, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *mean = sum / static_cast<double>(g1 - g0);
    return DG_OK;
}

// Drops the captured step graphs (their kernel arguments or buffers changed).
inline void drop_graphs(dg_ctx* c) {
    if (c->graph) cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
    if (c->mgraph) cudaGraphExecDestroy(c->mgraph);
    c->mgraph = nullptr;
}

int validate_boundary_face(const dg_mesh_desc* m, int f);  // dg_api.cu
}  // namespace h3dctx

// Variable-order / multi-case path (dg_var_api.cu).

namespace h3dvar {
bool needs_variable_path(const dg_mesh_desc* m);
int create(int n_cases, const dg_mesh_desc* meshes, const dg_physics* phys, const dg_options* opt, dg_ctx** out);
void release(dg_ctx* c);
int upload(dg_ctx* c, const double* q);
cudaError_t stage(dg_ctx* c, int stage, double tshift, int flags);
cudaError_t enqueue_max_dt(dg_ctx* c, double cfl, double dcfl);
cudaError_t enqueue_advance_time(dg_ctx* c);
int residuals(dg_ctx* c, double* maxres, int* nan_case);  // maxres [5*n_cases], nan_case [n_cases]
cudaError_t enqueue_residuals(dg_ctx* c);                  // into red[8k+2..6] and vnan[k], no sync
int kernel_times(dg_ctx* c, int reps, double* ms);
int autotune(dg_ctx* c, int reps);
}  // namespace h3dvar
