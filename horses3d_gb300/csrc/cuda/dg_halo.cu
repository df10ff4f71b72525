// Halo exchange of element partitions: gathers the face-slot data a partition sends to its
// neighbours into one contiguous buffer, and scatters received data into its ghost slots.
//
// The reference exchanges, per MPI face, the face's Q and then its gradients (MPI_Face_SendQ and the
// gradient sends, MPI_Face.f90:203-383; HexMesh_UpdateMPIFacesSolution / ...Gradients,
// HexMesh.f90:1199-1730). This path keeps data in element-face slots (the side's own face
// coordinates), so a slot's P^2 points x 5 values move as they are: the Q traces before the volume
// kernel (the BR1 jump reads the neighbour's trace), and the viscous normal fluxes Fv(Q, grad U).n
// before the face-flux kernel (which averages both sides'). Payload layout: slot after slot in the
// registered order, point after point, 5 values per point, in the working precision.
#include <cuda_runtime.h>

#include <string>

#include "dg_context.cuh"

namespace {

using h3dctx::DevBuf;

template <typename R>
__global__ void k_halo_pack(const R* __restrict__ buf, int64_t nsp, int P2, const int* __restrict__ slots, int n,
                            R* __restrict__ out) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= static_cast<int64_t>(n) * P2) return;
    const int i = static_cast<int>(t / P2), p = static_cast<int>(t - static_cast<int64_t>(i) * P2);
    const int64_t idx = static_cast<int64_t>(slots[i]) * P2 + p;
    R* o = out + 5 * t;
#pragma unroll
    for (int v = 0; v < 4; ++v) o[v] = buf[4 * idx + v];
    o[4] = buf[4 * nsp + idx];
}

template <typename R>
__global__ void k_halo_unpack(R* __restrict__ buf, int64_t nsp, int P2, const int* __restrict__ slots, int n,
                              const R* __restrict__ in) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= static_cast<int64_t>(n) * P2) return;
    const int i = static_cast<int>(t / P2), p = static_cast<int>(t - static_cast<int64_t>(i) * P2);
    const int64_t idx = static_cast<int64_t>(slots[i]) * P2 + p;
    const R* s = in + 5 * t;
#pragma unroll
    for (int v = 0; v < 4; ++v) buf[4 * idx + v] = s[v];
    buf[4 * nsp + idx] = s[4];
}

template <typename R>
int halo_move(dg_ctx* c, const h3dctx::Store<R>& st, int field, bool pack, void* data) {
    const R* src = field == DG_HALO_Q_TRACES ? st.QF.p : st.FV.p;
    if (field == DG_HALO_VISCOUS_FLUX && !c->pc.ns)
        return h3d::fail(DG_ERR_INVALID, "viscous normal fluxes exist for Navier-Stokes contexts only");
    const int P2 = c->P * c->P;
    const int n = pack ? c->n_halo_send : c->n_halo_recv;
    if (n == 0) return DG_OK;
    const int64_t threads = static_cast<int64_t>(n) * P2;
    const int blocks = static_cast<int>((threads + 255) / 256);
    const int64_t nsp = st.args.nsp;
    if (pack)
        k_halo_pack<R><<<blocks, 256, 0, c->stream>>>(src, nsp, P2, c->halo_send.p, n, static_cast<R*>(data));
    else
        k_halo_unpack<R><<<blocks, 256, 0, c->stream>>>(const_cast<R*>(src), nsp, P2, c->halo_recv.p, n,
                                                        static_cast<const R*>(data));
    CK(cudaGetLastError());
    // complete when the call returns: the packed buffer is ready for any stream or library, and a
    // received buffer may be released or reused at once
    CK(cudaStreamSynchronize(c->stream));
    return DG_OK;
}

int halo_common(dg_ctx* c, int field, bool pack, void* data) {
    if (!c || !data) return h3d::fail(DG_ERR_INVALID, "null argument");
    if (c->var) return h3d::fail(DG_ERR_UNSUPPORTED, "halo exchange needs a uniform-order partition context");
    if (field != DG_HALO_Q_TRACES && field != DG_HALO_VISCOUS_FLUX) return h3d::fail(DG_ERR_INVALID, "unknown halo field");
    return c->mixed ? halo_move(c, c->s32, field, pack, data) : halo_move(c, c->s64, field, pack, data);
}

int upload_slots(dg_ctx* c, DevBuf<int>& dst, int n, const int32_t* slots, size_t lo, size_t hi, const char* what) {
    for (int i = 0; i < n; ++i)
        if (slots[i] < 0 || static_cast<size_t>(slots[i]) < lo || static_cast<size_t>(slots[i]) >= hi)
            return h3d::fail(DG_ERR_INVALID, std::string(what) + " slot outside its range");
    dst.free();
    CK(dst.upload(slots, static_cast<size_t>(n), c->stream));
    return DG_OK;
}

}  // namespace

extern "C" {

int dg_halo_set_slots(dg_ctx* c, int32_t n_send, const int32_t* send_slots, int32_t n_recv, const int32_t* recv_slots) {
    if (!c || n_send < 0 || n_recv < 0 || (n_send && !send_slots) || (n_recv && !recv_slots))
        return h3d::fail(DG_ERR_INVALID, "bad halo slot lists");
    if (c->var) return h3d::fail(DG_ERR_UNSUPPORTED, "halo exchange needs a uniform-order partition context");
    const size_t own = 6 * static_cast<size_t>(c->K);
    int rc = upload_slots(c, c->halo_send, n_send, send_slots, 0, own, "send");
    if (rc) return rc;
    rc = upload_slots(c, c->halo_recv, n_recv, recv_slots, own, c->n_slots(), "receive");
    if (rc) return rc;
    c->n_halo_send = n_send;
    c->n_halo_recv = n_recv;
    return DG_OK;
}

int64_t dg_halo_slot_bytes(const dg_ctx* c) {
    if (!c || c->var) return 0;
    return static_cast<int64_t>(c->P) * c->P * 5 * (c->mixed ? sizeof(float) : sizeof(double));
}

int dg_halo_pack(dg_ctx* c, int field, void* dst) { return halo_common(c, field, true, dst); }

int dg_halo_unpack(dg_ctx* c, int field, const void* src) { return halo_common(c, field, false, const_cast<void*>(src)); }

}  // extern "C"
