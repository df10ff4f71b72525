// DGSEM right-hand-side kernels for uniform-order hexahedral meshes, templated on the number of
// nodes per direction P = N+1, the node family (GL = Gauss-Lobatto) and the arithmetic type R
// (double: plain form, float: mixed form; the state Q and the RK register G are FP64 in both).
//
// One RK stage is three kernels; the fourth runs once after an upload:
//   k_volume    element: local BR1 gradient (HexElementClass.f90:427-531); BR1 interface jump
//               1/2 (U_R - U_L) Jf n from the own and the neighbour's Q traces
//               (EllipticBR1.f90:571-627, FaceClass.f90:865-963); lifting (EllipticBR1.f90:531-569);
//               gradient traces (HexElementClass.f90:304-372) turned into each side's viscous
//               normal flux Fv(Q, grad U) . n (EllipticBR1.f90:816-868); viscosity, contravariant
//               fluxes and the weak or split-form volume integral
//               (SpatialDiscretization.f90:1602-1682, DGIntegrals.f90:56-129) -> QDot
//   k_flux      face:    Roe/LxF flux minus the averaged viscous normal flux, times Jf; side 1 gets
//               f*, side 2 gets -f* (SpatialDiscretization.f90:1710-1799, FaceClass.f90:597-703)
//   k_update    element: surface integral, 1/J, source (DGIntegrals.f90:214-273,
//               SpatialDiscretization.f90:483-494,564-639), the Williamson RK3 update
//               (ExplicitMethods.f90:748-779) and the Q face traces of the updated state for the next
//               stage (HexElementClass.f90:233-302)
//   k_traces    element: Q face traces of the current state (after an upload)
//
// Face data live in element-face "slots" (slot = 6e + side-1, sides numbered as the reference), in
// the element's own face coordinates (the FaceStorage(side) arrays), one 5-vector per slot point
// idx = slot*P^2 + p, p = a + P*b: values 0..3 at [4*idx], the fifth at [4*nsp + idx].
#pragma once
#include <cstdint>

#include "dg_convert.cuh"
#include "dg_dt.cuh"
#include "dg_physics.cuh"
#include "dg_tc.cuh"
#include "dg_tma.cuh"

namespace dg {

constexpr int kMaxP = 8;

template <typename R>
struct Ops {  // NodalStorage of the mesh order (NodalStorageClass.f90:170-338), row-major (i,l)
    R D[kMaxP * kMaxP], hatD[kMaxP * kMaxP], sharpD[kMaxP * kMaxP];
    R vL[kMaxP], vR[kMaxP], bL[kMaxP], bR[kMaxP];
};

template <typename R>
struct Args {
    int K, F;
    PhysR<R> ph;
    Ops<R> ops;
    int inviscid, source;
    int tc;  // volume kernel with the tensor-core gradient contractions (DG_PRECISION_MIXED_TC)
    // geometry per node
    const R* ja_xi;
    const R* ja_eta;
    const R* ja_zeta;
    const R* jac;
    const R* inv_jac;
    const double* x;
    // faces: connectivity and geometry in face order (SoA: component c at [c*nfp + fp])
    const int* face_elem;
    const int* face_side;
    const int* face_rot;
    const R* fn;
    const R* ft1;
    const R* ft2;
    const R* fj;
    // slots: neighbour slot, (rotation | own side << 3), geometry (n_x,n_y,n_z,Jf) in own coordinates
    const int* nb_slot;
    const int* nb_map;
    const R* sgeo;  // [6K][4][P^2]
    // state
    double* Q;
    double* G;
    R* QDot;
    R* Ux;  // lifted gradient, written only when store_grad is set
    R* Uy;
    R* Uz;
    // slot arrays, one 5-vector per slot point idx = slot*P^2 + p (see gld5): Q traces, viscous
    // normal fluxes of each side, surface fluxes
    R* QF;
    R* FV;
    R* FS;
    int64_t nsp;  // slot points, 6 K P^2
    const double* time;  // device scalars: step start time and dt
    const double* dt;
    double e_ref;        // energy reference of the mixed form (0 for the plain form)
    const BoundaryR<R>* bc;  // boundary conditions (a boundary slot has nb_slot = -1 - its index)
    int* err;            // set by a kernel whose bounded wait on a bulk copy gave up
    // device time loop with the residual monitor and the MaxTimeStep estimate fused into the last
    // stage's update: per element 8 words (max |QDot| per variable as FP64 bit images, a NaN/Inf
    // flag, the FP32 convective and viscous estimates of the new state as bit images)
    unsigned long long* mon;
    DtConst32 dtc;
    uint32_t extra_tx;   // bytes the update kernel's mbarrier expects beyond its copies (fault injection; 0)
    // manufactured-solution source constants
    double src_gm1, src_gM2, src_mu, src_kappa;
};

template <int P>
struct Geo {
    static constexpr int P2 = P * P, P3 = P * P * P;
    static constexpr int EPB = (P3 >= 128) ? 1 : (256 / P3);  // elements per block
    static constexpr int THREADS = EPB * P3;
};

// Minimum resident blocks per SM requested from the register allocator: the kernels are latency
// bound at one element per block, so occupancy is bought with a register budget per thread. The
// FP32 volume budgets are measured: 64 registers (4 blocks) for P = 5 (the split-form workload,
// +6 %), 72 elsewhere (P = 6: 64 spills; P = 4: 64 measured 8 % slower).
template <int P, typename R>
struct Occupancy {
    static constexpr int blocks(int regs) {
        return (65536 / (Geo<P>::THREADS * regs)) > 0 ? (65536 / (Geo<P>::THREADS * regs)) : 1;
    }
    static constexpr int volume = blocks(sizeof(R) == 4 ? (P == 5 ? 64 : 72) : 168);
    static constexpr int update = blocks(sizeof(R) == 4 ? 64 : 96);
};

__device__ __forceinline__ int64_t slot(int e, int side) { return 6 * static_cast<int64_t>(e) + (side - 1); }

// The FP64 state of node g in the working precision; the energy relative to e_ref (FP64 difference).
// INT selects the integer-pipe conversion (kernels whose FP64 pipe is their bottleneck) over the
// hardware one (issue-bound kernels, where the extra integer instructions cost more).
template <bool INT = false, typename R>
__device__ __forceinline__ void load_state(const Args<R>& a, int64_t g, R* q) {
    if (INT) {
#pragma unroll
        for (int v = 0; v < 4; ++v) q[v] = from_f64<R>(a.Q[5 * g + v]);
        q[4] = from_f64<R>(a.Q[5 * g + 4] - a.e_ref);
    } else {
#pragma unroll
        for (int v = 0; v < 4; ++v) q[v] = R(a.Q[5 * g + v]);
        q[4] = R(a.Q[5 * g + 4] - a.e_ref);
    }
}

// Node of line position l through face point (ca, cb) of a side.
template <int P>
__device__ __forceinline__ int line_node(int side, int ca, int cb, int l) {
    switch (side) {
        case 1: case 2: return ca + P * (l + P * cb);   // FRONT/BACK: (i, k)
        case 3: case 5: return ca + P * (cb + P * l);   // BOTTOM/TOP: (i, j)
        default: return l + P * (ca + P * cb);          // RIGHT/LEFT: (j, k)
    }
}
__device__ __forceinline__ bool right_end(int side) { return side == 2 || side == 4 || side == 5; }

// Neighbour point of own face point (ca,cb): leftIndexes2Right from side 1, its inverse from side 2.
template <int P>
__device__ __forceinline__ int neighbour_point(int map, int ca, int cb) {
    const int rot = map & 7, side = map >> 3;
    constexpr int N = P - 1;
    int ii, jj;
    if (side == 1) {
        left2right(ca, cb, N, N, rot, ii, jj);
    } else {
        switch (rot) {  // the (i, j) with left2right(i, j) = (ca, cb)
            case 0: ii = ca; jj = cb; break;
            case 1: ii = cb; jj = N - ca; break;
            case 2: ii = N - ca; jj = N - cb; break;
            case 3: ii = N - cb; jj = ca; break;
            case 4: ii = cb; jj = ca; break;
            case 5: ii = N - ca; jj = cb; break;
            case 6: ii = N - cb; jj = N - ca; break;
            default: ii = ca; jj = N - cb; break;
        }
    }
    return ii + P * jj;
}

// Shared-memory operands of k_volume are 5-vectors (the five conserved variables, or the five
// components of one direction of a gradient or flux) stored as a 16-byte part holding values 0..3 at
// v4[4*i4] and the fifth value at v1[i1]: a 5-vector costs one 128-bit and one 32-bit load (two
// 128-bit and one 64-bit for double) instead of five scalar loads, and nodes 16 or 48 bytes apart
// keep the 128-bit load phases free of bank conflicts.
template <typename R>
__device__ __forceinline__ void ld5(const R* v4, int i4, const R* v1, int i1, R* o);
template <>
__device__ __forceinline__ void ld5<float>(const float* v4, int i4, const float* v1, int i1, float* o) {
    const float4 t = *reinterpret_cast<const float4*>(v4 + 4 * i4);
    o[0] = t.x;
    o[1] = t.y;
    o[2] = t.z;
    o[3] = t.w;
    o[4] = v1[i1];
}
template <>
__device__ __forceinline__ void ld5<double>(const double* v4, int i4, const double* v1, int i1, double* o) {
    const double2 x = *reinterpret_cast<const double2*>(v4 + 4 * i4);
    const double2 y = *reinterpret_cast<const double2*>(v4 + 4 * i4 + 2);
    o[0] = x.x;
    o[1] = x.y;
    o[2] = y.x;
    o[3] = y.y;
    o[4] = v1[i1];
}
template <typename R>
__device__ __forceinline__ void st5(R* v4, int i4, R* v1, int i1, const R* x);
template <>
__device__ __forceinline__ void st5<float>(float* v4, int i4, float* v1, int i1, const float* x) {
    *reinterpret_cast<float4*>(v4 + 4 * i4) = make_float4(x[0], x[1], x[2], x[3]);
    v1[i1] = x[4];
}
template <>
__device__ __forceinline__ void st5<double>(double* v4, int i4, double* v1, int i1, const double* x) {
    *reinterpret_cast<double2*>(v4 + 4 * i4) = make_double2(x[0], x[1]);
    *reinterpret_cast<double2*>(v4 + 4 * i4 + 2) = make_double2(x[2], x[3]);
    v1[i1] = x[4];
}

// A 3-vector padded to four values at v[4*i] (one 128-bit access for float, two for double).
template <typename R>
__device__ __forceinline__ void st4(R* v, int i, R x0, R x1, R x2) {
    if constexpr (sizeof(R) == 4) {
        *reinterpret_cast<float4*>(v + 4 * i) = make_float4(x0, x1, x2, 0.f);
    } else {
        *reinterpret_cast<double2*>(v + 4 * i) = make_double2(x0, x1);
        *reinterpret_cast<double2*>(v + 4 * i + 2) = make_double2(x2, 0.0);
    }
}
template <typename R>
__device__ __forceinline__ void ld4(const R* v, int i, R* o) {
    if constexpr (sizeof(R) == 4) {
        const float4 t = *reinterpret_cast<const float4*>(v + 4 * i);
        o[0] = t.x;
        o[1] = t.y;
        o[2] = t.z;
        o[3] = t.w;
    } else {
        const double2 x = *reinterpret_cast<const double2*>(v + 4 * i);
        const double2 y = *reinterpret_cast<const double2*>(v + 4 * i + 2);
        o[0] = x.x;
        o[1] = x.y;
        o[2] = y.x;
        o[3] = y.y;
    }
}

// Slot arrays in global memory use the same split: the 16-byte parts of all slot points first, then
// the fifth values; the threads of a face read consecutive 16-byte parts (coalesced 128-bit loads).
template <typename R>
__device__ __forceinline__ void gld5(const R* base, int64_t nsp, int64_t idx, R* o) {
    ld5(base + 4 * idx, 0, base + 4 * nsp + idx, 0, o);
}
template <typename R>
__device__ __forceinline__ void gst5(R* base, int64_t nsp, int64_t idx, const R* x) {
    st5(base + 4 * idx, 0, base + 4 * nsp + idx, 0, x);
}

// Offsets (values of R) of one element's k_volume workspace; every region starts on 16 bytes.
//   Q4/Q1  state, 5-vector per node
//   G4/G1  lifted gradient, 3 directions per node (later the contravariant or viscous fluxes)
//   M      metric vectors per node (split form only; empty otherwise)
//   U4/U1  BR1 jumps per face point of the six sides: FP32, uStar (5-vectors) with the unit normals
//          in NN (4 values each, the fourth unused), the lifting forming uStar n_d in registers;
//          FP64, uStar n_d for the 3 directions (the FP64 pipe binds that form: the products are
//          formed once per face point, not once per node and side)
//   T4/T1  own Q traces per face point of the six sides
//   F4/F1  split form: the two-point fluxes of one direction, D = P/2 pairs per node, staged over
//          U, T and beyond once the gradient phases are done
template <int P, typename R>
struct VolLayout {
    static constexpr int P2 = P * P, P3 = P * P * P, A = 16 / static_cast<int>(sizeof(R));
    static constexpr int D = P / 2;
    __host__ __device__ static constexpr int up(int x) { return (x + A - 1) / A * A; }
    static constexpr int Q4 = 0, Q1 = Q4 + up(4 * P3);
    static constexpr int G4 = Q1 + up(P3), G1 = G4 + up(12 * P3);
    static constexpr int M = G1 + up(3 * P3);
    __host__ __device__ static constexpr int U4(bool split) { return M + (split ? up(9 * P3) : 0); }
    static constexpr bool JN = sizeof(R) == 4;  // jumps and normals apart
    __host__ __device__ static constexpr int U1(bool split) { return U4(split) + up((JN ? 24 : 72) * P2); }
    __host__ __device__ static constexpr int NN(bool split) { return U1(split) + up((JN ? 6 : 18) * P2); }
    __host__ __device__ static constexpr int T4(bool split) { return NN(split) + (JN ? up(24 * P2) : 0); }
    __host__ __device__ static constexpr int T1(bool split) { return T4(split) + up(24 * P2); }
    __host__ __device__ static constexpr int end_faces(bool split) { return T1(split) + up(6 * P2); }
    static constexpr int F4 = M + up(9 * P3), F1 = F4 + up(4 * P3 * D), F_END = F1 + up(P3 * D);
    __host__ __device__ static constexpr int values(bool split) {
        return split ? (end_faces(true) > F_END ? end_faces(true) : F_END) : end_faces(false);
    }
};

template <int P, typename R>
__host__ __device__ constexpr int volume_smem_values(bool split) {
    return VolLayout<P, R>::values(split);
}

// Tensor-core gradient of k_volume (one element per CTA): the A operand of one direction, rows
// (variable v, line) = v P^2 + line with K = the node's position on the line (hi and lo TF32 parts,
// 2 x 128-row blocks), and the B operand [D; vL; vR] (16 rows, hi and lo), after the FP32 workspace
// at a 128-byte boundary.
struct TcLayout {
    static constexpr uint32_t kARows = 256, kBRows = 16;
    static constexpr uint32_t A_HI = 0, A_LO = tc::operand_bytes(kARows), B_HI = 2 * tc::operand_bytes(kARows),
                              B_LO = B_HI + tc::operand_bytes(kBRows), BYTES = B_LO + tc::operand_bytes(kBRows);
    static constexpr uint32_t kCols = 32;  // TMEM columns: 2 blocks of N = 16
};
template <int P, typename R>
__host__ __device__ constexpr size_t volume_tc_offset() {
    return (static_cast<size_t>(VolLayout<P, R>::values(false)) * sizeof(R) + 127) / 128 * 128;
}

// Work item tt of the 6 P^2 face points of an element -> (side, point). For Gauss nodes the two ends
// of a line are adjacent items (lanes 2q and 2q+1): their traces read the same shared-memory words in
// the same instructions, which the hardware serves as one broadcast; Gauss-Lobatto traces read one
// end node only and keep the side-major order.
template <int P, bool GL>
__device__ __forceinline__ void face_point_of(int tt, int& side, int& p) {
    constexpr int P2 = P * P;
    if (GL) {
        side = 1 + tt / P2;
        p = tt - (side - 1) * P2;
        return;
    }
    const int q = tt >> 1, axis = q / P2;
    p = q - axis * P2;
    const bool hi = (tt & 1) != 0;
    side = axis == 0 ? (hi ? 2 : 1) : axis == 1 ? (hi ? 5 : 3) : (hi ? 4 : 6);
}

// Trace at face point (ca,cb) of a side of D 5-vectors per entry (entry m, direction d at
// v4[(m*D+d)*4], v1[d*n+m]): sum_l v(l) s(line node l) in line order (HexElementClass.f90:233-372);
// the Gauss-Lobatto end weights are unit vectors, so the end node is picked.
template <int P, bool GL, int D, typename R>
__device__ __forceinline__ void trace5(const Ops<R>& ops, const R* v4, const R* v1, int n, int side, int ca, int cb,
                                       R out[D][5]) {
    if (GL) {
        const int m = line_node<P>(side, ca, cb, right_end(side) ? P - 1 : 0);
#pragma unroll
        for (int d = 0; d < D; ++d) ld5(v4, m * D + d, v1, d * n + m, out[d]);
        return;
    }
    const R* w = right_end(side) ? ops.vR : ops.vL;
#pragma unroll
    for (int d = 0; d < D; ++d)
#pragma unroll
        for (int v = 0; v < 5; ++v) out[d][v] = R(0);
#pragma unroll
    for (int l = 0; l < P; ++l) {
        const int m = line_node<P>(side, ca, cb, l);
        const R wl = w[l];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            R x[5];
            ld5(v4, m * D + d, v1, d * n + m, x);
#pragma unroll
            for (int v = 0; v < 5; ++v) out[d][v] = out[d][v] + x[v] * wl;
        }
    }
}

// ------------------------------------------------------------------------------------------------
// k_traces: Q face traces of the current state.
// ------------------------------------------------------------------------------------------------
template <int P, bool GL, typename R>
__global__ void __launch_bounds__(Geo<P>::THREADS) k_traces(Args<R> a) {
    constexpr int P2 = Geo<P>::P2, P3 = Geo<P>::P3, EPB = Geo<P>::EPB;
    __shared__ __align__(16) R sQ4[EPB][4 * P3];
    __shared__ R sQ1[EPB][P3];
    const int le = threadIdx.x / P3, n = threadIdx.x - le * P3;
    const int e = blockIdx.x * EPB + le;
    const bool active = e < a.K;
    if (active) {
        R q[5];
        load_state<true>(a, static_cast<int64_t>(e) * P3 + n, q);
        st5(sQ4[le], n, sQ1[le], n, q);
    }
    __syncthreads();
    if (!active) return;
    for (int t = n; t < 6 * P2; t += P3) {
        const int side = 1 + t / P2, p = t - (side - 1) * P2;
        R tq[1][5];
        trace5<P, GL, 1>(a.ops, sQ4[le], sQ1[le], P3, side, p % P, p / P, tq);
        gst5(a.QF, a.nsp, slot(e, side) * P2 + p, tq[0]);
    }
}

// ------------------------------------------------------------------------------------------------
// k_volume: gradient, BR1 lifting, viscous normal fluxes on the faces, volume integral -> QDot.
// ------------------------------------------------------------------------------------------------
// EST (the first stage of a step of the monitored time loop): the FP32 MaxTimeStep estimate of the
// step's initial state at every node, its element minima into the element's monitor record
// (a.mon[8e + 6], [8e + 7]), from the state and metric terms the kernel loads anyway.
template <int P, bool GL, typename R, bool TC = false, bool EST = false>
__global__ void __launch_bounds__(Geo<P>::THREADS, (Occupancy<P, R>::volume)) k_volume(Args<R> a, int store_grad) {
    using L = VolLayout<P, R>;
    constexpr int P2 = Geo<P>::P2, P3 = Geo<P>::P3, F6 = 6 * P2;
    static_assert(!TC || (Geo<P>::EPB == 1 && 5 * P2 <= 192 && P + 2 <= 16), "tensor-core gradient: one element per CTA");
    static_assert(!EST || (Geo<P>::EPB == 1 && !TC), "time-step estimate: one element per CTA");
    __shared__ uint2 est_part[EST ? (P3 + 31) / 32 : 1];
    const bool split = a.inviscid != 0;
    const bool ns = a.ph.ns;
    extern __shared__ __align__(16) unsigned char dsm[];
    const int le = threadIdx.x / P3, n = threadIdx.x - le * P3;
    R* base = reinterpret_cast<R*>(dsm) + le * L::values(split);
    R* Q4 = base + L::Q4;
    R* Q1 = base + L::Q1;
    R* G4 = base + L::G4;  // lifted gradient, then the fluxes (same layout)
    R* G1 = base + L::G1;
    R* U4 = base + L::U4(split);
    R* U1 = base + L::U1(split);
    R* NN = base + L::NN(split);
    R* T4 = base + L::T4(split);
    R* T1 = base + L::T1(split);
    R* sM = base + L::M;
    const int e = blockIdx.x * Geo<P>::EPB + le;
    const bool active = e < a.K;
    const int i = n % P, j = (n / P) % P, k = n / P2;
    const int64_t g = static_cast<int64_t>(e) * P3 + n;

    R q[5];
    R jxs[3], jes[3], jzs[3];
    __shared__ __align__(8) uint64_t tc_bar;
    __shared__ uint32_t tc_slot;
    unsigned char* tcm = dsm + volume_tc_offset<P, R>();
    if constexpr (TC) {
        // TMEM for the accumulators, zero A operands (the padding rows and K = P..7 stay zero), the
        // B operand [D; vL; vR] split into TF32 hi and lo parts, the MMA completion barrier
        if (threadIdx.x < 32) {
            tc::tmem_alloc(&tc_slot, TcLayout::kCols);
            tc::fence_before_sync();
        }
        for (int w = threadIdx.x; w < static_cast<int>(TcLayout::B_HI / 16); w += blockDim.x)
            reinterpret_cast<float4*>(tcm)[w] = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int w = threadIdx.x; w < static_cast<int>(TcLayout::kBRows) * 8; w += blockDim.x) {
            const int nr = w >> 3, kk = w & 7;
            float x = 0.f;
            if (kk < P) x = nr < P ? float(a.ops.D[nr * kMaxP + kk]) : nr == P ? float(a.ops.vL[kk])
                                                                     : nr == P + 1 ? float(a.ops.vR[kk]) : 0.f;
            const float hi = tc::tf32_hi(x);
            *reinterpret_cast<float*>(tcm + TcLayout::B_HI + tc::operand_offset(nr, kk)) = hi;
            *reinterpret_cast<float*>(tcm + TcLayout::B_LO + tc::operand_offset(nr, kk)) = x - hi;
        }
        if (threadIdx.x == 0) {
            mbar_init(&tc_bar, 1);
            mbar_init_fence();
        }
    }
    if (active) {
        load_state(a, g, q);
        st5(Q4, n, Q1, n, q);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            jxs[c] = a.ja_xi[3 * g + c];
            jes[c] = a.ja_eta[3 * g + c];
            jzs[c] = a.ja_zeta[3 * g + c];
        }
    }
    if constexpr (EST) {
        // the FP32 inputs of the estimate: the state rounded to FP32 (the mixed form's q already is,
        // except the energy, which it holds relative to e_ref)
        float cv, vs;
        const float E = sizeof(R) == 4 ? to_f32(a.Q[5 * g + 4]) : as_f32(q[4]);
        dt_estimate_f(a.dtc, as_f32(q[0]), as_f32(q[1]), as_f32(q[2]), as_f32(q[3]), E, jxs, jes, jzs, a.jac[g], cv, vs);
        const int w = n >> 5, cnt = P3 - 32 * w < 32 ? P3 - 32 * w : 32;
        const unsigned mask = cnt == 32 ? 0xffffffffu : (1u << cnt) - 1u;
        // minima of non-negative floats (and NaN, which loses to every number) by their bit patterns
        const unsigned c = __reduce_min_sync(mask, __float_as_uint(cv));
        const unsigned v = __reduce_min_sync(mask, __float_as_uint(vs));
        if ((n & 31) == 0) est_part[w] = make_uint2(c, v);
    }
    __syncthreads();
    if constexpr (EST) {
        if (n < 32) {
            constexpr int NW = (P3 + 31) / 32;
            const uint2 p = n < NW ? est_part[n] : make_uint2(0xffffffffu, 0xffffffffu);
            const unsigned c = __reduce_min_sync(0xffffffffu, p.x);
            const unsigned v = __reduce_min_sync(0xffffffffu, p.y);
            if (n == 0) {
                a.mon[8 * static_cast<int64_t>(e) + 6] = c;
                a.mon[8 * static_cast<int64_t>(e) + 7] = v;
            }
        }
    }
    if constexpr (TC) {
        // Gradient contractions on the tensor cores (HexElement_ComputeLocalGradient,
        // HexElementClass.f90:427-531, and the Q traces of ProlongSolutionToFaces): per direction,
        // C = X [D; vL; vR]^T with X the lines of Q as TF32 split products, the derivatives at the
        // line's nodes in columns 0..P-1 and its two end values in columns P, P+1. The derivatives
        // go to the G workspace as [direction][variable][node], the end values to the own-trace
        // workspace T. One direction at a time through one A buffer and 32 TMEM columns.
        tc::fence_after_sync();
        const uint32_t tbase = tc_slot;
        bool ok = true;
        if (ns) {
            R* Gs = G4;  // the lifted gradient's space, free until the lifting writes it
            const int w = threadIdx.x >> 5;
            for (int d = 0; d < 3; ++d) {
                const int self = d == 0 ? i : (d == 1 ? j : k);
                const int line = d == 0 ? (j + P * k) : (d == 1 ? (i + P * k) : (i + P * j));
                if (active) {
#pragma unroll
                    for (int v = 0; v < 5; ++v) {
                        const float x = float(q[v]), hi = tc::tf32_hi(x);
                        const uint32_t off = tc::operand_offset(v * P2 + line, self);
                        *reinterpret_cast<float*>(tcm + TcLayout::A_HI + off) = hi;
                        *reinterpret_cast<float*>(tcm + TcLayout::A_LO + off) = x - hi;
                    }
                }
                fence_proxy_async_smem();  // the operand stores before the tensor core reads them
                tc::fence_before_sync();
                __syncthreads();
                tc::fence_after_sync();
                if (threadIdx.x == 0) {
                    constexpr uint32_t id = tc::idesc_tf32(128, 16);
                    const uint64_t bh = tc::smem_desc(tcm + TcLayout::B_HI), bl = tc::smem_desc(tcm + TcLayout::B_LO);
#pragma unroll
                    for (int b = 0; b < 2; ++b) {
                        const uint32_t ta = tbase + 16u * b;
                        const uint32_t ob = b * tc::operand_bytes(128);
                        tc::mma_tf32(ta, tc::smem_desc(tcm + TcLayout::A_HI + ob), bh, id, false);
                        tc::mma_tf32(ta, tc::smem_desc(tcm + TcLayout::A_HI + ob), bl, id, true);
                        tc::mma_tf32(ta, tc::smem_desc(tcm + TcLayout::A_LO + ob), bh, id, true);
                    }
                    tc::commit(&tc_bar);
                }
                const bool done = mbar_wait(&tc_bar, d & 1);
                if (__syncthreads_or(!done)) {  // block-uniform
                    ok = false;
                    if (threadIdx.x == 0) {
                        atomicOr(a.err, 1);
                        mbar_wait(&tc_bar, d & 1, kWaitNs / 4);  // bounded: let a late MMA land before TMEM is freed
                    }
                    __syncthreads();
                    break;
                }
                tc::fence_after_sync();
                if (w < 6) {  // full warps: warps 0-3 read block 0, warps 4-5 lanes 0-63 of block 1
                    const int b = w >> 2;
                    const int row = 128 * b + 32 * (w & 3) + (threadIdx.x & 31);
                    float val[16];
                    tc::ld_32x32b_x16(tbase + 16u * b + ((32u * (w & 3)) << 16), val);
                    if (row < 5 * P2) {
                        const int v = row / P2, ln = row - v * P2;
#pragma unroll
                        for (int l = 0; l < P; ++l) {
                            const int node = d == 0 ? (l + P * ln) : (d == 1 ? ((ln % P) + P * l + P2 * (ln / P)) : (ln + P2 * l));
                            Gs[(d * 5 + v) * P3 + node] = R(val[l]);
                        }
                        // own Q traces at the two end faces of the line, in the sides' face
                        // coordinates: LEFT (6) / RIGHT (4), FRONT (1) / BACK (2), BOTTOM (3) / TOP (5)
                        const int tl = ((d == 0 ? 6 : (d == 1 ? 1 : 3)) - 1) * P2 + ln;
                        const int tr = ((d == 0 ? 4 : (d == 1 ? 2 : 5)) - 1) * P2 + ln;
                        if (v < 4) {
                            T4[4 * tl + v] = R(val[P]);
                            T4[4 * tr + v] = R(val[P + 1]);
                        } else {
                            T1[tl] = R(val[P]);
                            T1[tr] = R(val[P + 1]);
                        }
                    }
                }
                tc::fence_before_sync();
                __syncthreads();  // the next direction reuses the A buffer and the accumulators
            }
        }
        tc::fence_after_sync();
        if (threadIdx.x < 32) tc::tmem_dealloc(tbase, TcLayout::kCols);
        if (!ok) return;
    }

    R U[3][5];
    // gradient variables other than the state are formed per node into the (still unused) gradient
    // space, read with the stride of its 3-direction layout
    const bool gv = ns && a.ph.grad_vars != 0;
    if (gv) {
        if (active) {
            R u[5];
            gradient_variables(a.ph, q, u);
            st5(G4, n * 3, G1, n, u);
        }
        __syncthreads();
    }
    const R* X4 = gv ? G4 : Q4;
    const R* X1 = gv ? G1 : Q1;
    const int xs = gv ? 3 : 1;
    if (ns) {
        if (active) {
            // local gradient: U_x = (U_xi Ja^xi_x + U_eta Ja^eta_x + U_zeta Ja^zeta_x) / J
            R uxi[5] = {0, 0, 0, 0, 0}, ueta[5] = {0, 0, 0, 0, 0}, uzeta[5] = {0, 0, 0, 0, 0};
            if constexpr (TC) {
#pragma unroll
                for (int v = 0; v < 5; ++v) {
                    uxi[v] = G4[(0 * 5 + v) * P3 + n];
                    ueta[v] = G4[(1 * 5 + v) * P3 + n];
                    uzeta[v] = G4[(2 * 5 + v) * P3 + n];
                }
            } else {
#pragma unroll
            for (int l = 0; l < P; ++l) {
                const R w = a.ops.D[i * kMaxP + l];
                const int m = l + P * (j + P * k);
                R x[5];
                ld5(X4, m * xs, X1, m, x);
#pragma unroll
                for (int v = 0; v < 5; ++v) uxi[v] = uxi[v] + x[v] * w;
            }
#pragma unroll
            for (int l = 0; l < P; ++l) {
                const R w = a.ops.D[j * kMaxP + l];
                const int m = i + P * (l + P * k);
                R x[5];
                ld5(X4, m * xs, X1, m, x);
#pragma unroll
                for (int v = 0; v < 5; ++v) ueta[v] = ueta[v] + x[v] * w;
            }
#pragma unroll
            for (int l = 0; l < P; ++l) {
                const R w = a.ops.D[k * kMaxP + l];
                const int m = i + P * (j + P * l);
                R x[5];
                ld5(X4, m * xs, X1, m, x);
#pragma unroll
                for (int v = 0; v < 5; ++v) uzeta[v] = uzeta[v] + x[v] * w;
            }
            }
            const R ij = a.inv_jac[g];
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                U[0][v] = (uxi[v] * jxs[0] + ueta[v] * jes[0] + uzeta[v] * jzs[0]) * ij;
                U[1][v] = (uxi[v] * jxs[1] + ueta[v] * jes[1] + uzeta[v] * jzs[1]) * ij;
                U[2][v] = (uxi[v] * jxs[2] + ueta[v] * jes[2] + uzeta[v] * jzs[2]) * ij;
            }
            // BR1 jumps at the six sides: 1/2 (U_R - U_L) Jf n in the face's orientation (left -> right)
            for (int tt = n; tt < F6; tt += P3) {
                int side, p;
                face_point_of<P, GL>(tt, side, p);
                const int t = (side - 1) * P2 + p;
                const int ca = p % P, cb = p / P;
                const int64_t s = slot(e, side);
                R own[1][5], nbr[5];
                if constexpr (TC) {
                    ld5(T4, t, T1, t, own[0]);  // from the tensor-core contraction
                } else {
                    trace5<P, GL, 1>(a.ops, Q4, Q1, P3, side, ca, cb, own);
                    st5(T4, t, T1, t, own[0]);
                }
                const int map = a.nb_map[s];
                const int nb = a.nb_slot[s];
                const R* sg = a.sgeo + s * 4 * P2 + p;
                const R nn[3] = {sg[0], sg[P2], sg[2 * P2]};
                const R J = sg[3 * P2];
                R uo[5], u[5];
                gradient_variables(a.ph, own[0], uo);
                if (nb < 0) {  // boundary: (U* - U) Jf n (EllipticBR1.f90:686-736)
                    R us[5];
                    bc_gradvars(a.ph, a.bc[-1 - nb], nn, own[0], uo, us);
#pragma unroll
                    for (int v = 0; v < 5; ++v) u[v] = (us[v] - uo[v]) * J;
                } else {
                    const int pn = neighbour_point<P>(map, ca, cb);
                    gld5(a.QF, a.nsp, static_cast<int64_t>(nb) * P2 + pn, nbr);
                    const bool left = (map >> 3) == 1;
                    R un[5];
                    gradient_variables(a.ph, nbr, un);
#pragma unroll
                    for (int v = 0; v < 5; ++v) u[v] = R(0.5) * (left ? (un[v] - uo[v]) : (uo[v] - un[v])) * J;
                }
                if constexpr (L::JN) {  // the jump and the normal; the lifting forms uStar n_d
                    st5(U4, t, U1, t, u);
                    st4(NN, t, nn[0], nn[1], nn[2]);
                } else {
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        R x[5];
#pragma unroll
                        for (int v = 0; v < 5; ++v) x[v] = u[v] * nn[d];
                        st5(U4, t * 3 + d, U1, d * F6 + t, x);
                    }
                }
            }
        }
        __syncthreads();
        if (active) {
            // lifting: U += (sum over sides of b (x) uStar n) / J in VectorWeakIntegrals_StdFace order
            // (left, right, front, back, bottom, top)
            const R ij = a.inv_jac[g];
            const int pt[6] = {(5 * P2) + (j + P * k), (3 * P2) + (j + P * k), (0 * P2) + (i + P * k),
                               (1 * P2) + (i + P * k), (2 * P2) + (i + P * j), (4 * P2) + (i + P * j)};
            R bw[6];
            bool use[6];
            if (GL) {  // b(:,LEFT/RIGHT) vanish away from the end nodes
                const R bl = a.ops.bL[0], br = a.ops.bR[P - 1];
                use[0] = i == 0; use[1] = i == P - 1; use[2] = j == 0; use[3] = j == P - 1; use[4] = k == 0;
                use[5] = k == P - 1;
                bw[0] = bl; bw[1] = br; bw[2] = bl; bw[3] = br; bw[4] = bl; bw[5] = br;
            } else {
                bw[0] = a.ops.bL[i]; bw[1] = a.ops.bR[i]; bw[2] = a.ops.bL[j]; bw[3] = a.ops.bR[j];
                bw[4] = a.ops.bL[k]; bw[5] = a.ops.bR[k];
#pragma unroll
                for (int sd = 0; sd < 6; ++sd) use[sd] = true;
            }
            if constexpr (!L::JN) {
                if (!GL || use[0] || use[1] || use[2] || use[3] || use[4] || use[5]) {
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        R fi[5] = {0, 0, 0, 0, 0};
                        bool first = true;
#pragma unroll
                        for (int sd = 0; sd < 6; ++sd) {
                            if (!use[sd]) continue;
                            R h[5];
                            ld5(U4, pt[sd] * 3 + d, U1, d * F6 + pt[sd], h);
#pragma unroll
                            for (int v = 0; v < 5; ++v) fi[v] = first ? h[v] * bw[sd] : fi[v] + h[v] * bw[sd];
                            first = false;
                        }
#pragma unroll
                        for (int v = 0; v < 5; ++v) U[d][v] = U[d][v] + fi[v] * ij;
                    }
                }
            } else if (!GL || use[0] || use[1] || use[2] || use[3] || use[4] || use[5]) {
                // per side one jump and one normal from shared memory, the three directions'
                // products uStar n_d in registers (each rounded as a stored product would be)
                R fi[3][5];
                bool first = true;
#pragma unroll
                for (int sd = 0; sd < 6; ++sd) {
                    if (!use[sd]) continue;
                    R u[5], nv[4];
                    ld5(U4, pt[sd], U1, pt[sd], u);
                    ld4(NN, pt[sd], nv);
#pragma unroll
                    for (int d = 0; d < 3; ++d)
#pragma unroll
                        for (int v = 0; v < 5; ++v) {
                            const R h = u[v] * nv[d];
                            fi[d][v] = first ? h * bw[sd] : fi[d][v] + h * bw[sd];
                        }
                    first = false;
                }
#pragma unroll
                for (int d = 0; d < 3; ++d)
#pragma unroll
                    for (int v = 0; v < 5; ++v) U[d][v] = U[d][v] + fi[d][v] * ij;
            }
#pragma unroll
            for (int d = 0; d < 3; ++d) st5(G4, n * 3 + d, G1, d * P3 + n, U[d]);
            if (store_grad) {
#pragma unroll
                for (int v = 0; v < 5; ++v) {
                    a.Ux[5 * g + v] = U[0][v];
                    a.Uy[5 * g + v] = U[1][v];
                    a.Uz[5 * g + v] = U[2][v];
                }
            }
        }
        __syncthreads();
        if (active) {
            // viscous normal flux of this side at its face points: Fv(Q, grad U, mu(Q)) . n
            for (int tt = n; tt < F6; tt += P3) {
                int side, p;
                face_point_of<P, GL>(tt, side, p);
                const int t = (side - 1) * P2 + p;
                const int ca = p % P, cb = p / P;
                const int64_t s = slot(e, side);
                R tq[5], tg[3][5];
                ld5(T4, t, T1, t, tq);
                trace5<P, GL, 3>(a.ops, G4, G1, P3, side, ca, cb, tg);
                R mu, kap;
                mu_kappa(a.ph, tq, mu, kap);
                R C[3][5];
                viscous_flux(a.ph, tq, tg[0], tg[1], tg[2], mu, kap, C);
                const R* sg = a.sgeo + s * 4 * P2 + p;
                const R n0 = sg[0], n1 = sg[P2], n2 = sg[2 * P2];
                R fv[5];
#pragma unroll
                for (int v = 0; v < 5; ++v) fv[v] = C[0][v] * n0 + C[1][v] * n1 + C[2][v] * n2;
                gst5(a.FV, a.nsp, s * P2 + p, fv);
            }
        }
    }

    __syncthreads();  // the gradient is read above and its space reused for the fluxes below
    // contravariant fluxes (HyperbolicDiscretizationClass.f90:132-149, EllipticBR1.f90:794-812);
    // the lifted gradient is read back from this node's own entries
    R Fi[3][5], Fv[3][5];
    if (active) {
        euler_contravariant(a.ph, q, jxs, jes, jzs, Fi);
        if (ns) {
            R Ug[3][5];
#pragma unroll
            for (int d = 0; d < 3; ++d) ld5(G4, n * 3 + d, G1, d * P3 + n, Ug[d]);
            R mu, kappa;
            mu_kappa(a.ph, q, mu, kappa);
            R C[3][5];
            viscous_flux(a.ph, q, Ug[0], Ug[1], Ug[2], mu, kappa, C);
            const R* ja[3] = {jxs, jes, jzs};
#pragma unroll
            for (int d = 0; d < 3; ++d)
#pragma unroll
                for (int v = 0; v < 5; ++v) Fv[d][v] = C[0][v] * ja[d][0] + C[1][v] * ja[d][1] + C[2][v] * ja[d][2];
        } else {
#pragma unroll
            for (int d = 0; d < 3; ++d)
#pragma unroll
                for (int v = 0; v < 5; ++v) Fv[d][v] = R(0);
        }
    }
    if (!split) {
        // ScalarWeakIntegrals_StdVolumeGreen on F = Finv - Fvisc
        if (active) {
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                R x[5];
#pragma unroll
                for (int v = 0; v < 5; ++v) x[v] = Fi[d][v] - Fv[d][v];
                st5(G4, n * 3 + d, G1, d * P3 + n, x);
            }
        }
        __syncthreads();
        if (!active) return;
        R acc[5] = {0, 0, 0, 0, 0};
#pragma unroll
        for (int l = 0; l < P; ++l) {
            const R h = a.ops.hatD[i * kMaxP + l];
            const int m = l + P * (j + P * k);
            R x[5];
            ld5(G4, m * 3 + 0, G1, 0 * P3 + m, x);
#pragma unroll
            for (int v = 0; v < 5; ++v) acc[v] = acc[v] + h * x[v];
        }
#pragma unroll
        for (int l = 0; l < P; ++l) {
            const R h = a.ops.hatD[j * kMaxP + l];
            const int m = i + P * (l + P * k);
            R x[5];
            ld5(G4, m * 3 + 1, G1, 1 * P3 + m, x);
#pragma unroll
            for (int v = 0; v < 5; ++v) acc[v] = acc[v] + h * x[v];
        }
#pragma unroll
        for (int l = 0; l < P; ++l) {
            const R h = a.ops.hatD[k * kMaxP + l];
            const int m = i + P * (j + P * l);
            R x[5];
            ld5(G4, m * 3 + 2, G1, 2 * P3 + m, x);
#pragma unroll
            for (int v = 0; v < 5; ++v) acc[v] = acc[v] + h * x[v];
        }
#pragma unroll
        for (int v = 0; v < 5; ++v) a.QDot[5 * g + v] = acc[v];
    } else {
        // Split form (Gauss-Lobatto, HyperbolicSplitForm.f90:64-116): the two-point flux f#(a,b) of
        // a pair of nodes on a line is symmetric, and the reference evaluates it once per pair (for
        // l > i, copied to f#(l,i)). Here node s of a line evaluates the pairs (s, s + delta mod P),
        // delta = 1..D with D = P/2, which covers every pair once for odd P; for even P the pairs at
        // distance P/2 belong to the nodes s < P/2. The lower line index is "left" as in the
        // reference. One direction at a time, the fluxes are staged per (line, s, delta) in shared
        // memory, then every node sums its line in line order:
        // volInt += sharpD(i,l) f#(i,l) + hatD(i,l) Fv(l), QDot = -volInt (DGIntegrals.f90:92-129).
        constexpr int D = L::D;
        R* F4 = base + L::F4;
        R* F1 = base + L::F1;
        if (active) {
#pragma unroll
            for (int d = 0; d < 3; ++d) st5(G4, n * 3 + d, G1, d * P3 + n, Fv[d]);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                sM[c * P3 + n] = jxs[c];
                sM[(3 + c) * P3 + n] = jes[c];
                sM[(6 + c) * P3 + n] = jzs[c];
            }
        }
        __syncthreads();
        R acc[5] = {0, 0, 0, 0, 0};
        const R* myJ[3] = {jxs, jes, jzs};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int self = d == 0 ? i : (d == 1 ? j : k);
            const int line = d == 0 ? (j + P * k) : (d == 1 ? (i + P * k) : (i + P * j));
            const int stride = d == 0 ? 1 : (d == 1 ? P : P2);
            const int first = n - self * stride;  // node of line position 0
            if (active) {
#pragma unroll
                for (int dl = 1; dl <= D; ++dl) {
                    if ((P % 2) == 0 && dl == D && self >= D) continue;
                    const int l = (self + dl) % P;
                    const int m = first + l * stride;
                    R qo[5], jo[3], fs[5];
                    ld5(Q4, m, Q1, m, qo);
#pragma unroll
                    for (int c = 0; c < 3; ++c) jo[c] = sM[(3 * d + c) * P3 + m];
                    if (self < l) two_point_flux(a.ph, q, qo, myJ[d], jo, fs);
                    else two_point_flux(a.ph, qo, q, jo, myJ[d], fs);
                    const int idx = (line * P + self) * D + (dl - 1);
                    st5(F4, idx, F1, idx, fs);
                }
            }
            __syncthreads();
            if (active) {
#pragma unroll
                for (int l = 0; l < P; ++l) {
                    const int m = first + l * stride;
                    R fs[5];
                    if (l == self) {
#pragma unroll
                        for (int v = 0; v < 5; ++v) fs[v] = Fi[d][v];
                    } else {
                        const int dl = (l - self + P) % P;
                        const bool mine = dl < D || (dl == D && ((P % 2) == 1 || self < D));
                        const int idx = mine ? (line * P + self) * D + (dl - 1) : (line * P + l) * D + (P - dl - 1);
                        ld5(F4, idx, F1, idx, fs);
                    }
                    const R sh = a.ops.sharpD[self * kMaxP + l];
                    const R h = a.ops.hatD[self * kMaxP + l];
                    R fv[5];
                    ld5(G4, m * 3 + d, G1, d * P3 + m, fv);
#pragma unroll
                    for (int v = 0; v < 5; ++v) acc[v] = acc[v] + sh * fs[v] + h * fv[v];
                }
            }
            __syncthreads();  // the next direction overwrites the staged fluxes
        }
        if (active) {
#pragma unroll
            for (int v = 0; v < 5; ++v) a.QDot[5 * g + v] = -acc[v];
        }
    }
}

// ------------------------------------------------------------------------------------------------
// k_flux: f* = (F_inv(QL,QR) - 1/2 (Fv_L.n + Fv_R.n)) Jf; side 1 gets f*, side 2 gets -f*.
// ------------------------------------------------------------------------------------------------
template <int P, typename R, bool GEN>
__global__ void __launch_bounds__(128) k_flux(Args<R> a) {
    constexpr int P2 = P * P;
    const int64_t nfp = static_cast<int64_t>(a.F) * P2;
    const int64_t gid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (gid >= nfp) return;
    const int f = static_cast<int>(gid / P2), p = static_cast<int>(gid - static_cast<int64_t>(f) * P2);
    int ii, jj;
    left2right(p % P, p / P, P - 1, P - 1, a.face_rot[f], ii, jj);
    const int pr = ii + P * jj;
    const int eR = a.face_elem[2 * f + 1];
    const bool boundary = eR < 0;  // a boundary face: its condition's ghost state is the right side
    const int64_t iL = slot(a.face_elem[2 * f], a.face_side[2 * f]) * P2 + p;
    const int64_t iR = boundary ? iL : slot(eR, a.face_side[2 * f + 1]) * P2 + pr;
    const R n[3] = {a.fn[gid], a.fn[nfp + gid], a.fn[2 * nfp + gid]};
    const R J = a.fj[gid];
    R QL[5], QR[5];
    gld5(a.QF, a.nsp, iL, QL);
    if (boundary) {
#pragma unroll
        for (int v = 0; v < 5; ++v) QR[v] = QL[v];
        bc_state(a.ph, a.bc[a.face_side[2 * f + 1]], n, QR);
    } else {
        gld5(a.QF, a.nsp, iR, QR);
    }
    R inv[5];
    if (GEN) {  // standard Roe, Roe-Pike, low-dissipation Roe, matrix dissipation, viscous NS
        const R t1[3] = {a.ft1[gid], a.ft1[nfp + gid], a.ft1[2 * nfp + gid]};
        const R t2[3] = {a.ft2[gid], a.ft2[nfp + gid], a.ft2[2 * nfp + gid]};
        riemann_flux(a.ph, QL, QR, n, t1, t2, inv);
    } else if (a.ph.riemann == 0) {
        roe_flux(a.ph, QL, QR, n, inv);
    } else if (a.ph.riemann == 3) {
        rusanov_flux(a.ph, QL, QR, n, inv);
    } else {  // LxF, central, u-diss
        const R t1[3] = {a.ft1[gid], a.ft1[nfp + gid], a.ft1[2 * nfp + gid]};
        const R t2[3] = {a.ft2[gid], a.ft2[nfp + gid], a.ft2[2 * nfp + gid]};
        lxf_flux<R, false>(a.ph, QL, QR, n, t1, t2, inv);
    }
    R vL[5] = {0, 0, 0, 0, 0}, vR[5] = {0, 0, 0, 0, 0};
    if (a.ph.ns) {
        gld5(a.FV, a.nsp, iL, vL);
        if (boundary) {  // the interior viscous flux through the condition's Neumann rule
            bc_neumann(a.bc[a.face_side[2 * f + 1]], QL, vL);
#pragma unroll
            for (int v = 0; v < 5; ++v) vR[v] = vL[v];
        } else {
            gld5(a.FV, a.nsp, iR, vR);
        }
    }
    R fl[5], fr[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        const R visc = a.ph.ns ? R(0.5) * (vL[v] + vR[v]) : R(0);
        fl[v] = (inv[v] - visc) * J;
        fr[v] = -fl[v];
    }
    gst5(a.FS, a.nsp, iL, fl);
    if (!boundary) gst5(a.FS, a.nsp, iR, fr);
}

// Surface integral in the reference's order (left, right, front, back, bottom, top), division by J
// and the manufactured source at time t_src: qd = (qd - sum b f*)/J + S.
template <int P, bool GL, bool SRC, typename R>
__device__ __forceinline__ void surface_integral(const Args<R>& a, int i, int j, int k, int64_t g,
                                                 const bool use[6], const R fs[6][5], R J, double t_src, R qd[5]) {
    if (GL) {
        const R bl = a.ops.bL[0], br = a.ops.bR[P - 1];
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            R fi = R(0);
            if (use[5]) fi = fs[5][v] * bl;
            if (use[3]) fi = fi + fs[3][v] * br;
            if (use[0]) fi = fi + fs[0][v] * bl;
            if (use[1]) fi = fi + fs[1][v] * br;
            if (use[2]) fi = fi + fs[2][v] * bl;
            if (use[4]) fi = fi + fs[4][v] * br;
            qd[v] = (qd[v] - fi) / J;
        }
    } else {
        const R bxl = a.ops.bL[i], bxr = a.ops.bR[i], byl = a.ops.bL[j], byr = a.ops.bR[j];
        const R bzl = a.ops.bL[k], bzr = a.ops.bR[k];
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            R fi = fs[5][v] * bxl;
            fi = fi + fs[3][v] * bxr;
            fi = fi + fs[0][v] * byl;
            fi = fi + fs[1][v] * byr;
            fi = fi + fs[2][v] * bzl;
            fi = fi + fs[4][v] * bzr;
            qd[v] = (qd[v] - fi) / J;
        }
    }
    if (SRC) {
        double S[5];
        manufactured_source(a.source, a.x[3 * g], a.x[3 * g + 1], a.x[3 * g + 2], t_src, a.src_gm1, a.src_gM2,
                            a.src_mu, a.src_kappa, S);
#pragma unroll
        for (int v = 0; v < 5; ++v) qd[v] = R(double(qd[v]) + S[v]);
    }
}

// Williamson low-storage RK3 stage in FP64 (ExplicitMethods.f90:748-779): G = a_k G + QDot,
// Q = Q + c_k dt G.
template <typename R>
__device__ __forceinline__ void rk3_stage(int stage, double dt, const R qd[5], double gq[5], double qq[5]) {
    const double ak = stage == 0 ? 0.0 : (stage == 1 ? -5.0 / 9.0 : -153.0 / 128.0);
    const double ck = stage == 0 ? 1.0 / 3.0 : (stage == 1 ? 15.0 / 16.0 : 8.0 / 15.0);
    const double cdt = ck * dt;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        gq[v] = ak * gq[v] + widen(qd[v]);
        qq[v] = qq[v] + cdt * gq[v];
    }
}

// The six surface fluxes of node (i,j,k) of element e (Gauss-Lobatto: only the sides the node
// touches); use[] marks the loaded ones.
template <int P, bool GL, typename R>
__device__ __forceinline__ void load_surface_fluxes(const Args<R>& a, int e, int i, int j, int k, bool use[6],
                                                    R fs[6][5]) {
    constexpr int P2 = P * P;
    const int64_t s1 = slot(e, 1) * P2;  // the six slots of e are contiguous
    const int pL = j + P * k, pF = i + P * k, pO = i + P * j;
    const bool u[6] = {GL ? j == 0 : true, GL ? j == P - 1 : true, GL ? k == 0 : true,
                       GL ? i == P - 1 : true, GL ? k == P - 1 : true, GL ? i == 0 : true};
    const int pt[6] = {pF, pF, pO, pL, pO, pL};
#pragma unroll
    for (int sd = 0; sd < 6; ++sd) {
        use[sd] = u[sd];
        if (u[sd]) {
            gld5(a.FS, a.nsp, s1 + sd * P2 + pt[sd], fs[sd]);
        } else {
#pragma unroll
            for (int v = 0; v < 5; ++v) fs[sd][v] = R(0);
        }
    }
}

// ------------------------------------------------------------------------------------------------
// k_update: QDot = (QDot - surface integral)/J + S; stage >= 0 adds the low-storage update
// G = a_k G + QDot, Q = Q + c_k dt G in FP64 and writes the Q traces of the new state.
// write_qdot stores the final QDot (residuals, downloads).
// ------------------------------------------------------------------------------------------------
template <int P, bool GL, bool SRC, typename R>
__global__ void __launch_bounds__(Geo<P>::THREADS, (Occupancy<P, R>::update))
    k_update(Args<R> a, int stage, double tshift, int write_qdot) {
    constexpr int P2 = Geo<P>::P2, P3 = Geo<P>::P3, EPB = Geo<P>::EPB;
    __shared__ __align__(16) R sQ4[EPB][4 * P3];
    __shared__ R sQ1[EPB][P3];
    const int le = threadIdx.x / P3, n = threadIdx.x - le * P3;
    const int e = blockIdx.x * EPB + le;
    const bool active = e < a.K;
    const int i = n % P, j = (n / P) % P, k = n / P2;
    const int64_t g = static_cast<int64_t>(e) * P3 + n;
    if (active) {
        // every load of the node up front (QDot, J, the six surface fluxes, G and Q), then the math
        R qd[5], fs[6][5];
        bool use[6];
        double gq[5], qq[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) qd[v] = a.QDot[5 * g + v];
        const R J = a.jac[g];
        load_surface_fluxes<P, GL>(a, e, i, j, k, use, fs);
        if (stage >= 0) {
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                gq[v] = a.G[5 * g + v];
                qq[v] = a.Q[5 * g + v];
            }
        }
        const double dt = *a.dt;
        surface_integral<P, GL, SRC>(a, i, j, k, g, use, fs, J, *a.time + tshift * dt, qd);
        if (write_qdot) {
#pragma unroll
            for (int v = 0; v < 5; ++v) a.QDot[5 * g + v] = qd[v];
        }
        if (stage >= 0) {
            rk3_stage(stage, dt, qd, gq, qq);
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                a.G[5 * g + v] = gq[v];
                a.Q[5 * g + v] = qq[v];
            }
            const R qn[5] = {from_f64<R>(qq[0]), from_f64<R>(qq[1]), from_f64<R>(qq[2]), from_f64<R>(qq[3]),
                             from_f64<R>(qq[4] - a.e_ref)};
            st5(sQ4[le], n, sQ1[le], n, qn);
        }
    }
    if (stage < 0) return;
    __syncthreads();
    if (!active) return;
    for (int t = n; t < 6 * P2; t += P3) {  // Q traces of the updated state
        const int side = 1 + t / P2, p = t - (side - 1) * P2;
        R tq[1][5];
        trace5<P, GL, 1>(a.ops, sQ4[le], sQ1[le], P3, side, p % P, p / P, tq);
        gst5(a.QF, a.nsp, slot(e, side) * P2 + p, tq[0]);
    }
}

// The residual record of one element (one CTA of NT threads) in the monitored time loop: max |QDot|
// per variable (FP64 bit images) and a NaN/Inf flag, words 0..5 of the element's 8-word record (the
// volume kernel of the step's first stage writes the time-step estimates into words 6 and 7). Each
// warp reduces its lanes (the CTA may end in a partial warp, whose missing lanes are left out) into
// shared memory before a CTA barrier; after it warp 0 folds the warp partials.
struct MonitorPart {
    unsigned long long m[5];
    int b;
};

template <int NT>
struct MonitorScratch {
    static constexpr int NW = (NT + 31) / 32;
    MonitorPart w[NW];
};

// Shuffle-down maximum over the first `cnt` lanes of a warp (mask: exactly those lanes).
__device__ __forceinline__ void monitor_warp(MonitorPart& p, unsigned mask, int cnt) {
    const int lane = threadIdx.x & 31;
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long q[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) q[v] = __shfl_down_sync(mask, p.m[v], o);
        const int qb = __shfl_down_sync(mask, p.b, o);
        if (lane + o < cnt) {
#pragma unroll
            for (int v = 0; v < 5; ++v) p.m[v] = q[v] > p.m[v] ? q[v] : p.m[v];
            p.b |= qb;
        }
    }
}

__device__ __forceinline__ unsigned warp_lanes_mask(int nt, int w, int& cnt) {
    cnt = nt - 32 * w < 32 ? nt - 32 * w : 32;
    return cnt == 32 ? 0xffffffffu : (1u << cnt) - 1u;
}

// First half, FP64 patterns (63 bits): shuffles.
template <int NT>
__device__ __forceinline__ void monitor_partial(const unsigned long long m[5], int bad, MonitorScratch<NT>& sp) {
    static_assert(NT >= 32, "warp 0 is full");
    const int t = threadIdx.x, w = t >> 5;
    MonitorPart p;
#pragma unroll
    for (int v = 0; v < 5; ++v) p.m[v] = m[v];
    p.b = bad;
    int cnt;
    const unsigned mask = warp_lanes_mask(NT, w, cnt);
    monitor_warp(p, mask, cnt);
    if ((t & 31) == 0) sp.w[w] = p;
}

// The FP32 form keeps 32-bit patterns (|QDot| as 31-bit FP32 images, the flag) through both halves
// and reduces them with single-instruction warp reductions; thread 0 widens the maxima to the FP64
// images at the end.
template <int NT>
struct MonitorScratch32 {
    static constexpr int NW = (NT + 31) / 32;
    unsigned w[6][NW];
};

template <int NT>
__device__ __forceinline__ void monitor_partial32(const unsigned m[5], int bad, MonitorScratch32<NT>& sp) {
    static_assert(NT >= 32, "warp 0 is full");
    const int t = threadIdx.x, w = t >> 5;
    int cnt;
    const unsigned mask = warp_lanes_mask(NT, w, cnt);
    unsigned mm[6];
#pragma unroll
    for (int v = 0; v < 5; ++v) mm[v] = __reduce_max_sync(mask, m[v]);
    mm[5] = __reduce_or_sync(mask, bad ? 1u : 0u);
    if ((t & 31) == 0) {
#pragma unroll
        for (int v = 0; v < 6; ++v) sp.w[v][w] = mm[v];
    }
}

template <int NT>
__device__ __forceinline__ void monitor_finish32(const MonitorScratch32<NT>& sp, unsigned long long* out) {
    constexpr int NW = MonitorScratch32<NT>::NW;
    const int t = threadIdx.x;
    if (t >= 32) return;
    unsigned mm[6];
#pragma unroll
    for (int v = 0; v < 6; ++v) mm[v] = __reduce_max_sync(0xffffffffu, t < NW ? sp.w[v][t] : 0u);
    if (t == 0) {
#pragma unroll
        for (int v = 0; v < 5; ++v) out[v] = abs_bits_as_double(mm[v], static_cast<const float*>(nullptr));
        out[5] = mm[5] ? 1ull : 0ull;
    }
}

// Second half (after the barrier, warp 0): the warp partials folded, words 0..5 written by thread 0.
template <int NT>
__device__ __forceinline__ void monitor_finish(const MonitorScratch<NT>& sp, unsigned long long* out) {
    constexpr int NW = MonitorScratch<NT>::NW;
    const int t = threadIdx.x;
    if (t >= 32) return;
    MonitorPart p;
    if (t < NW) {
        p = sp.w[t];
    } else {
#pragma unroll
        for (int v = 0; v < 5; ++v) p.m[v] = 0;
        p.b = 0;
    }
    monitor_warp(p, 0xffffffffu, NW);
    if (t == 0) {
#pragma unroll
        for (int v = 0; v < 5; ++v) out[v] = p.m[v];
        out[5] = p.b ? 1ull : 0ull;
    }
}

// ------------------------------------------------------------------------------------------------
// k_update_tma: k_update for one element per CTA whose Q, G (FP64), QDot and J blocks are 16-byte
// aligned (P = 6): the four element blocks arrive in shared memory as TMA bulk copies on an
// mbarrier while the threads fetch their surface fluxes; the updated Q and G leave as bulk stores.
// A copy that does not complete within the bounded wait sets *a.err and the CTA returns.
// ------------------------------------------------------------------------------------------------
// FUSE (the last stage of a monitored time-loop step): the element's residual/NaN record goes to
// a.mon[8e .. 8e + 5].
template <int P, bool GL, bool SRC, typename R, bool FUSE = false>
__global__ void __launch_bounds__(Geo<P>::THREADS, (Occupancy<P, R>::update))
    k_update_tma(Args<R> a, int stage, double tshift, int write_qdot) {
    static_assert(Geo<P>::EPB == 1, "one element per CTA");
    constexpr int P2 = Geo<P>::P2, P3 = Geo<P>::P3;
    constexpr uint32_t BQ = 5 * P3 * sizeof(double), BD = 5 * P3 * sizeof(R), BJ = P3 * sizeof(R);
    static_assert(BQ % 16 == 0 && BD % 16 == 0 && BJ % 16 == 0, "bulk copies move multiples of 16 bytes");
    __shared__ __align__(128) double sQd[5 * P3];
    __shared__ __align__(128) double sGd[5 * P3];
    __shared__ __align__(128) R sDot[5 * P3];
    __shared__ __align__(128) R sJ[P3];
    __shared__ __align__(16) R sQ4[4 * P3];
    __shared__ R sQ1[P3];
    // FUSE: the warp partials of the monitor record
    __shared__ MonitorScratch<(FUSE && sizeof(R) == 8) ? P3 : 32> smon;
    __shared__ MonitorScratch32<(FUSE && sizeof(R) == 4) ? P3 : 32> smon32;
    __shared__ __align__(8) uint64_t bar;
    const int n = threadIdx.x;
    const int e = blockIdx.x;
    const int i = n % P, j = (n / P) % P, k = n / P2;
    const int64_t g0 = static_cast<int64_t>(e) * P3, g = g0 + n;
    if (n == 0) {
        mbar_init(&bar, 1);
        mbar_init_fence();
    }
    __syncthreads();
    if (n == 0) {
        mbar_arrive_expect_tx(&bar, (stage >= 0 ? 2 * BQ : 0) + BD + BJ + a.extra_tx);
        if (stage >= 0) {
            bulk_load(sQd, a.Q + 5 * g0, BQ, &bar);
            bulk_load(sGd, a.G + 5 * g0, BQ, &bar);
        }
        bulk_load(sDot, a.QDot + 5 * g0, BD, &bar);
        bulk_load(sJ, a.jac + g0, BJ, &bar);
    }
    R fs[6][5];
    bool use[6];
    load_surface_fluxes<P, GL>(a, e, i, j, k, use, fs);
    const bool arrived = mbar_wait(&bar, 0);
    if (__syncthreads_or(!arrived)) {  // block-uniform: every thread leaves
        if (n == 0) {
            atomicOr(a.err, 1);
            mbar_wait(&bar, 0, kWaitNs / 4);  // bounded: let a late copy land before the CTA's memory is reused
        }
        return;
    }
    R qd[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) qd[v] = sDot[5 * n + v];
    const double dt = *a.dt;
    surface_integral<P, GL, SRC>(a, i, j, k, g, use, fs, sJ[n], *a.time + tshift * dt, qd);
    if (write_qdot) {
#pragma unroll
        for (int v = 0; v < 5; ++v) a.QDot[5 * g + v] = qd[v];
    }
    if (stage < 0) return;
    double gq[5], qq[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        gq[v] = sGd[5 * n + v];
        qq[v] = sQd[5 * n + v];
    }
    rk3_stage(stage, dt, qd, gq, qq);
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        sGd[5 * n + v] = gq[v];
        sQd[5 * n + v] = qq[v];
    }
    const R qn[5] = {from_f64<R>(qq[0]), from_f64<R>(qq[1]), from_f64<R>(qq[2]), from_f64<R>(qq[3]),
                     from_f64<R>(qq[4] - a.e_ref)};
    st5(sQ4, n, sQ1, n, qn);
    if constexpr (FUSE) {
        // ComputeMaxResiduals (max |QDot| of this stage) and checkForNan (the new Q) of the element,
        // and the FP32 time-step estimates of the new state (the first pass of MaxTimeStep)
        // NaN/Inf: all exponent bits set, tested on the high words
        unsigned hx = 0;
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            const unsigned h = static_cast<unsigned>(__double2hiint(qq[v])) & 0x7ff00000u;
            hx |= h == 0x7ff00000u ? 1u : 0u;
        }
        const int bad = static_cast<int>(hx);
        if constexpr (sizeof(R) == 4) {
            unsigned m[5];
#pragma unroll
            for (int v = 0; v < 5; ++v) m[v] = static_cast<unsigned>(abs_bits(qd[v]));
            monitor_partial32<P3>(m, bad, smon32);
        } else {
            unsigned long long m[5];
#pragma unroll
            for (int v = 0; v < 5; ++v) m[v] = abs_bits(qd[v]);
            monitor_partial<P3>(m, bad, smon);
        }
    }
    fence_proxy_async_smem();  // this thread's Q, G writes before the bulk stores read them
    __syncthreads();
    if (n == 0) {
        bulk_store(a.Q + 5 * g0, sQd, BQ);
        bulk_store(a.G + 5 * g0, sGd, BQ);
        bulk_commit();
    }
    if constexpr (FUSE) {
        if constexpr (sizeof(R) == 4) monitor_finish32<P3>(smon32, a.mon + 8 * static_cast<int64_t>(e));
        else monitor_finish<P3>(smon, a.mon + 8 * static_cast<int64_t>(e));
    }
    for (int t = n; t < 6 * P2; t += P3) {  // Q traces of the updated state
        const int side = 1 + t / P2, p = t - (side - 1) * P2;
        R tq[1][5];
        trace5<P, GL, 1>(a.ops, sQ4, sQ1, P3, side, p % P, p / P, tq);
        gst5(a.QF, a.nsp, slot(e, side) * P2 + p, tq[0]);
    }
    if (n == 0) bulk_wait_all();
}

}  // namespace dg
