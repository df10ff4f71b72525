// DGSEM right-hand-side kernels for uniform-order hexahedral meshes, templated on the number of
// nodes per direction P = N+1, the node family (GL = Gauss-Lobatto) and the arithmetic type R.
//
// One RK stage runs five kernels (the two face kernels have one thread per face point, the three
// element kernels one thread per node and one element per P^3 threads):
//   k_prolong_grad  element: BR1 local gradient (HexElementClass.f90:427-531) and Q face traces
//                   (HexElementClass.f90:233-302)
//   k_br1_face      face:    BR1 interface jump 1/2 (UR-UL) Jf n to both sides
//                   (EllipticBR1.f90:571-627, FaceClass.f90:865-963)
//   k_lift_volume   element: BR1 lifting (EllipticBR1.f90:531-569), gradient traces
//                   (HexElementClass.f90:304-372), viscosity, contravariant fluxes and the weak or
//                   split-form volume integral (SpatialDiscretization.f90:1602-1682, DGIntegrals.f90:56-129)
//   k_flux_face     face:    Roe/LxF + BR1 averaged viscous flux times Jf, minus on side 2
//                   (SpatialDiscretization.f90:1710-1799, FaceClass.f90:597-703)
//   k_surface_rk    element: surface integral, 1/J, source, Williamson RK3 update
//                   (DGIntegrals.f90:214-273, SpatialDiscretization.f90:483-494, ExplicitMethods.f90:748-779)
//
// Face data live in element-face "slots": slot = 6*e + side-1 (sides numbered as the reference),
// point index a + P*b in the element's own face coordinates (the FaceStorage(side) arrays).
#pragma once
#include <cstdint>

#include "dg_physics.cuh"

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
    // geometry (per node / per face point)
    const R* ja_xi;
    const R* ja_eta;
    const R* ja_zeta;
    const R* jac;
    const R* inv_jac;
    const double* x;
    const int* face_elem;
    const int* face_side;
    const int* face_rot;
    const R* fn;
    const R* ft1;
    const R* ft2;
    const R* fj;
    // state
    double* Q;
    double* G;
    R* QDot;
    R* Ux;
    R* Uy;
    R* Uz;
    R* QF;   // [6K][P^2][5]
    R* UN;   // [6K][P^2][15]
    R* GF;   // [6K][P^2][15]
    R* FS;   // [6K][P^2][5]
    const double* time;  // device scalars: step start time and dt
    const double* dt;
    double e_ref;        // energy reference of the mixed form (0 for the plain form)
    // MMS source constants
    double src_gm1, src_gM2, src_mu, src_kappa;
};

template <int P>
struct Geo {
    static constexpr int P2 = P * P, P3 = P * P * P;
    static constexpr int EPB = (P3 >= 128) ? 1 : (256 / P3);  // elements per block
    static constexpr int THREADS = EPB * P3;
};

// Element-face slot index of side s (1..6) and the face coordinates (a,b) of node (i,j,k).
__device__ __forceinline__ int64_t slot(int e, int side) { return 6 * static_cast<int64_t>(e) + (side - 1); }

// The FP64 state of node g in the working precision; the energy relative to e_ref (FP64 difference).
template <typename R>
__device__ __forceinline__ void load_state(const Args<R>& a, int64_t g, R* q) {
#pragma unroll
    for (int v = 0; v < 4; ++v) q[v] = R(a.Q[5 * g + v]);
    q[4] = R(a.Q[5 * g + 4] - a.e_ref);
}

// ------------------------------------------------------------------------------------------------
// k_prolong_grad: local gradient U_x,U_y,U_z (state gradient variables U = Q) and Q face traces.
// ------------------------------------------------------------------------------------------------
template <int P, bool GL, typename R>
__global__ void __launch_bounds__(Geo<P>::THREADS) k_prolong_grad(Args<R> a) {
    constexpr int P2 = Geo<P>::P2, P3 = Geo<P>::P3, EPB = Geo<P>::EPB;
    __shared__ R sQ[EPB][5][P3];
    const int le = threadIdx.x / P3, n = threadIdx.x - le * P3;
    const int e = blockIdx.x * EPB + le;
    const bool active = e < a.K;
    const int i = n % P, j = (n / P) % P, k = n / P2;
    const int64_t g = static_cast<int64_t>(e) * P3 + n;
    R q[5];
    if (active) {
        load_state(a, g, q);
#pragma unroll
        for (int v = 0; v < 5; ++v) sQ[le][v][n] = q[v];
    }
    __syncthreads();
    if (!active) return;
    const bool ns = a.ph.ns;
    if (ns) {
        R uxi[5] = {0, 0, 0, 0, 0}, ueta[5] = {0, 0, 0, 0, 0}, uzeta[5] = {0, 0, 0, 0, 0};
#pragma unroll
        for (int l = 0; l < P; ++l) {
            const R dx = a.ops.D[i * kMaxP + l], dy = a.ops.D[j * kMaxP + l], dz = a.ops.D[k * kMaxP + l];
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                uxi[v] = uxi[v] + sQ[le][v][l + P * (j + P * k)] * dx;
                ueta[v] = ueta[v] + sQ[le][v][i + P * (l + P * k)] * dy;
                uzeta[v] = uzeta[v] + sQ[le][v][i + P * (j + P * l)] * dz;
            }
        }
        const R* jx = a.ja_xi + 3 * g;
        const R* je = a.ja_eta + 3 * g;
        const R* jz = a.ja_zeta + 3 * g;
        const R ij = a.inv_jac[g];
        const R jx0 = jx[0], jx1 = jx[1], jx2 = jx[2], je0 = je[0], je1 = je[1], je2 = je[2];
        const R jz0 = jz[0], jz1 = jz[1], jz2 = jz[2];
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            a.Ux[5 * g + v] = (uxi[v] * jx0 + ueta[v] * je0 + uzeta[v] * jz0) * ij;
            a.Uy[5 * g + v] = (uxi[v] * jx1 + ueta[v] * je1 + uzeta[v] * jz1) * ij;
            a.Uz[5 * g + v] = (uxi[v] * jx2 + ueta[v] * je2 + uzeta[v] * jz2) * ij;
        }
    }
    // Q face traces, written in each side's own coordinates.
    if (GL) {
        auto put = [&](int side, int p) {
            R* d = a.QF + (slot(e, side) * P2 + p) * 5;
#pragma unroll
            for (int v = 0; v < 5; ++v) d[v] = q[v];
        };
        if (i == 0) put(6, j + P * k);
        if (i == P - 1) put(4, j + P * k);
        if (j == 0) put(1, i + P * k);
        if (j == P - 1) put(2, i + P * k);
        if (k == 0) put(3, i + P * j);
        if (k == P - 1) put(5, i + P * j);
    } else {
        for (int t = n; t < 6 * P2; t += P3) {
            const int side = 1 + t / P2, p = t - (side - 1) * P2;
            const int ca = p % P, cb = p / P;
            R acc[5] = {0, 0, 0, 0, 0};
#pragma unroll
            for (int l = 0; l < P; ++l) {
                int idx;
                R w;
                switch (side) {
                    case 1: idx = ca + P * (l + P * cb); w = a.ops.vL[l]; break;   // FRONT (i,k)
                    case 2: idx = ca + P * (l + P * cb); w = a.ops.vR[l]; break;   // BACK
                    case 3: idx = ca + P * (cb + P * l); w = a.ops.vL[l]; break;   // BOTTOM (i,j)
                    case 4: idx = l + P * (ca + P * cb); w = a.ops.vR[l]; break;   // RIGHT (j,k)
                    case 5: idx = ca + P * (cb + P * l); w = a.ops.vR[l]; break;   // TOP
                    default: idx = l + P * (ca + P * cb); w = a.ops.vL[l]; break;  // LEFT
                }
#pragma unroll
                for (int v = 0; v < 5; ++v) acc[v] = acc[v] + sQ[le][v][idx] * w;
            }
            R* d = a.QF + (slot(e, side) * P2 + p) * 5;
#pragma unroll
            for (int v = 0; v < 5; ++v) d[v] = acc[v];
        }
    }
}

// ------------------------------------------------------------------------------------------------
// k_br1_face: uStar_n = 1/2 (UR - UL) Jf n, the same value on both sides (factor +1).
// ------------------------------------------------------------------------------------------------
template <int P, typename R>
__global__ void __launch_bounds__(128) k_br1_face(Args<R> a) {
    constexpr int P2 = P * P;
    const int64_t gid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (gid >= static_cast<int64_t>(a.F) * P2) return;
    const int f = static_cast<int>(gid / P2), p = static_cast<int>(gid - static_cast<int64_t>(f) * P2);
    const int i = p % P, j = p / P;
    int ii, jj;
    left2right(i, j, P - 1, P - 1, a.face_rot[f], ii, jj);
    const int pr = ii + P * jj;
    const int eL = a.face_elem[2 * f], eR = a.face_elem[2 * f + 1];
    const int64_t sL = slot(eL, a.face_side[2 * f]) * P2 + p;
    const int64_t sR = slot(eR, a.face_side[2 * f + 1]) * P2 + pr;
    const R* QL = a.QF + 5 * sL;
    const R* QR = a.QF + 5 * sR;
    const int64_t fp = gid;
    const R J = a.fj[fp];
    const R n0 = a.fn[3 * fp], n1 = a.fn[3 * fp + 1], n2 = a.fn[3 * fp + 2];
    R* dL = a.UN + 15 * sL;
    R* dR = a.UN + 15 * sR;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        const R u = R(0.5) * (QR[v] - QL[v]) * J;
        const R x = u * n0, y = u * n1, z = u * n2;
        dL[v] = x; dL[5 + v] = y; dL[10 + v] = z;
        dR[v] = x; dR[5 + v] = y; dR[10 + v] = z;
    }
}

// ------------------------------------------------------------------------------------------------
// k_lift_volume: BR1 lifting, gradient traces, viscosity, fluxes and the volume integral -> QDot.
// store_grad writes the lifted gradient back to Ux/Uy/Uz.
// ------------------------------------------------------------------------------------------------
template <int P, bool GL, typename R>
__global__ void __launch_bounds__(Geo<P>::THREADS) k_lift_volume(Args<R> a, int store_grad) {
    constexpr int P2 = Geo<P>::P2, P3 = Geo<P>::P3, EPB = Geo<P>::EPB;
    // Dynamic shared memory, per element: standard form 15*P3 values (gradient for the Gauss traces,
    // then the contravariant flux); split form 29*P3 values (Q, viscous flux, metric vectors).
    extern __shared__ __align__(16) unsigned char dsm[];
    const int stride = (a.inviscid == 0 ? 15 : 29) * P3;
    const int le = threadIdx.x / P3, n = threadIdx.x - le * P3;
    R* sF = reinterpret_cast<R*>(dsm) + le * stride;
    const int e = blockIdx.x * EPB + le;
    const bool active = e < a.K;
    const int i = n % P, j = (n / P) % P, k = n / P2;
    const int64_t g = static_cast<int64_t>(e) * P3 + n;
    const bool ns = a.ph.ns;
    R U[3][5];
    R q[5];
    if (active) load_state(a, g, q);
    if (ns && active) {
#pragma unroll
        for (int v = 0; v < 5; ++v) { U[0][v] = a.Ux[5 * g + v]; U[1][v] = a.Uy[5 * g + v]; U[2][v] = a.Uz[5 * g + v]; }
        // lifting: faceInt = sum over sides of b (x) unStar (VectorWeakIntegrals_StdFace)
        const R ij = a.inv_jac[g];
        const R* HL = a.UN + (slot(e, 6) * P2 + (j + P * k)) * 15;
        const R* HR = a.UN + (slot(e, 4) * P2 + (j + P * k)) * 15;
        const R* HF = a.UN + (slot(e, 1) * P2 + (i + P * k)) * 15;
        const R* HB = a.UN + (slot(e, 2) * P2 + (i + P * k)) * 15;
        const R* HO = a.UN + (slot(e, 3) * P2 + (i + P * j)) * 15;
        const R* HT = a.UN + (slot(e, 5) * P2 + (i + P * j)) * 15;
        if (GL) {
            // b(:,LEFT) and b(:,RIGHT) vanish away from the end nodes: only boundary nodes lift.
            const R bL = a.ops.bL[0], bR = a.ops.bR[P - 1];
            const bool iL = i == 0, iR = i == P - 1, jL = j == 0, jR = j == P - 1, kL = k == 0, kR = k == P - 1;
            if (iL || iR || jL || jR || kL || kR) {
#pragma unroll
                for (int d = 0; d < 3; ++d)
#pragma unroll
                    for (int v = 0; v < 5; ++v) {
                        const int c = v + 5 * d;
                        R fi = R(0);
                        if (iL) fi = HL[c] * bL;
                        if (iR) fi = fi + HR[c] * bR;
                        if (jL) fi = fi + HF[c] * bL;
                        if (jR) fi = fi + HB[c] * bR;
                        if (kL) fi = fi + HO[c] * bL;
                        if (kR) fi = fi + HT[c] * bR;
                        U[d][v] = U[d][v] + fi * ij;
                    }
            }
        } else {
            const R bxl = a.ops.bL[i], bxr = a.ops.bR[i], byl = a.ops.bL[j], byr = a.ops.bR[j];
            const R bzl = a.ops.bL[k], bzr = a.ops.bR[k];
#pragma unroll
            for (int d = 0; d < 3; ++d)
#pragma unroll
                for (int v = 0; v < 5; ++v) {
                    const int c = v + 5 * d;
                    R fi = HL[c] * bxl;
                    fi = fi + HR[c] * bxr;
                    fi = fi + HF[c] * byl;
                    fi = fi + HB[c] * byr;
                    fi = fi + HO[c] * bzl;
                    fi = fi + HT[c] * bzr;
                    U[d][v] = U[d][v] + fi * ij;
                }
        }
        if (store_grad) {
#pragma unroll
            for (int v = 0; v < 5; ++v) { a.Ux[5 * g + v] = U[0][v]; a.Uy[5 * g + v] = U[1][v]; a.Uz[5 * g + v] = U[2][v]; }
        }
        if (GL) {  // gradient face traces: end nodes copy
            auto put = [&](int side, int p) {
                R* d = a.GF + (slot(e, side) * P2 + p) * 15;
#pragma unroll
                for (int dd = 0; dd < 3; ++dd)
#pragma unroll
                    for (int v = 0; v < 5; ++v) d[v + 5 * dd] = U[dd][v];
            };
            if (i == 0) put(6, j + P * k);
            if (i == P - 1) put(4, j + P * k);
            if (j == 0) put(1, i + P * k);
            if (j == P - 1) put(2, i + P * k);
            if (k == 0) put(3, i + P * j);
            if (k == P - 1) put(5, i + P * j);
        }
    }
    if (ns && !GL) {  // gradient face traces: contraction with v(:,LEFT/RIGHT)
        if (active) {
#pragma unroll
            for (int d = 0; d < 3; ++d)
#pragma unroll
                for (int v = 0; v < 5; ++v) sF[(v + 5 * d) * P3 + n] = U[d][v];
        }
        __syncthreads();
        if (active) {
            for (int t = n; t < 6 * P2; t += P3) {
                const int side = 1 + t / P2, p = t - (side - 1) * P2;
                const int ca = p % P, cb = p / P;
                R acc[15];
#pragma unroll
                for (int c = 0; c < 15; ++c) acc[c] = R(0);
#pragma unroll
                for (int l = 0; l < P; ++l) {
                    int idx;
                    R w;
                    switch (side) {
                        case 1: idx = ca + P * (l + P * cb); w = a.ops.vL[l]; break;
                        case 2: idx = ca + P * (l + P * cb); w = a.ops.vR[l]; break;
                        case 3: idx = ca + P * (cb + P * l); w = a.ops.vL[l]; break;
                        case 4: idx = l + P * (ca + P * cb); w = a.ops.vR[l]; break;
                        case 5: idx = ca + P * (cb + P * l); w = a.ops.vR[l]; break;
                        default: idx = l + P * (ca + P * cb); w = a.ops.vL[l]; break;
                    }
#pragma unroll
                    for (int c = 0; c < 15; ++c) acc[c] = acc[c] + sF[c * P3 + idx] * w;
                }
                R* d = a.GF + (slot(e, side) * P2 + p) * 15;
#pragma unroll
                for (int c = 0; c < 15; ++c) d[c] = acc[c];
            }
        }
        __syncthreads();
    }
    // contravariant fluxes (HyperbolicDiscretizationClass.f90:132-149, EllipticBR1.f90:794-812)
    R Fi[3][5], Fv[3][5];
    R jxs[3], jes[3], jzs[3];
    if (active) {
        const R* jx = a.ja_xi + 3 * g;
        const R* je = a.ja_eta + 3 * g;
        const R* jz = a.ja_zeta + 3 * g;
#pragma unroll
        for (int c = 0; c < 3; ++c) { jxs[c] = jx[c]; jes[c] = je[c]; jzs[c] = jz[c]; }
        euler_contravariant(a.ph, q, jxs, jes, jzs, Fi);
        if (ns) {
            R mu, kappa;
            mu_kappa(a.ph, q, mu, kappa);
            R C[3][5];
            viscous_flux(a.ph, q, U[0], U[1], U[2], mu, kappa, C);
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
    if (a.inviscid == 0) {
        // ScalarWeakIntegrals_StdVolumeGreen on F = Finv - Fvisc
        if (active) {
#pragma unroll
            for (int d = 0; d < 3; ++d)
#pragma unroll
                for (int v = 0; v < 5; ++v) sF[(v + 5 * d) * P3 + n] = Fi[d][v] - Fv[d][v];
        }
        __syncthreads();
        if (!active) return;
        R acc[5] = {0, 0, 0, 0, 0};
#pragma unroll
        for (int l = 0; l < P; ++l) {
            const R h = a.ops.hatD[i * kMaxP + l];
#pragma unroll
            for (int v = 0; v < 5; ++v) acc[v] = acc[v] + h * sF[v * P3 + l + P * (j + P * k)];
        }
#pragma unroll
        for (int l = 0; l < P; ++l) {
            const R h = a.ops.hatD[j * kMaxP + l];
#pragma unroll
            for (int v = 0; v < 5; ++v) acc[v] = acc[v] + h * sF[(5 + v) * P3 + i + P * (l + P * k)];
        }
#pragma unroll
        for (int l = 0; l < P; ++l) {
            const R h = a.ops.hatD[k * kMaxP + l];
#pragma unroll
            for (int v = 0; v < 5; ++v) acc[v] = acc[v] + h * sF[(10 + v) * P3 + i + P * (j + P * l)];
        }
#pragma unroll
        for (int v = 0; v < 5; ++v) a.QDot[5 * g + v] = acc[v];
    } else {
        // Split form (Gauss-Lobatto only): the two-point flux of each node with every node of its
        // xi/eta/zeta line (HyperbolicSplitForm.f90:64-116), accumulated as
        // volInt += sharpD(i,l) f#(l,i) + hatD(i,l) Fv(l) line by line (DGIntegrals.f90:92-129).
        R* sQ = sF;               // 5*P3
        R* sV = sF + 5 * P3;      // 15*P3
        R* sM = sF + 20 * P3;     // 9*P3: Ja^d_c at [(3d+c)*P3]
        if (active) {
#pragma unroll
            for (int v = 0; v < 5; ++v) sQ[v * P3 + n] = q[v];
#pragma unroll
            for (int d = 0; d < 3; ++d)
#pragma unroll
                for (int v = 0; v < 5; ++v) sV[(v + 5 * d) * P3 + n] = Fv[d][v];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                sM[c * P3 + n] = jxs[c];
                sM[(3 + c) * P3 + n] = jes[c];
                sM[(6 + c) * P3 + n] = jzs[c];
            }
        }
        __syncthreads();
        if (!active) return;
        R acc[5] = {0, 0, 0, 0, 0};
        const R* myJ[3] = {jxs, jes, jzs};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int self = d == 0 ? i : (d == 1 ? j : k);
#pragma unroll
            for (int l = 0; l < P; ++l) {
                const int m = d == 0 ? (l + P * (j + P * k)) : (d == 1 ? (i + P * (l + P * k)) : (i + P * (j + P * l)));
                R fs[5];
                if (l == self) {
#pragma unroll
                    for (int v = 0; v < 5; ++v) fs[v] = Fi[d][v];
                } else {
                    R qo[5], jo[3];
#pragma unroll
                    for (int v = 0; v < 5; ++v) qo[v] = sQ[v * P3 + m];
#pragma unroll
                    for (int c = 0; c < 3; ++c) jo[c] = sM[(3 * d + c) * P3 + m];
                    // the reference evaluates each pair once with the lower index as "left"
                    if (self < l) two_point_flux(a.ph, q, qo, myJ[d], jo, fs);
                    else two_point_flux(a.ph, qo, q, jo, myJ[d], fs);
                }
                const R s = a.ops.sharpD[self * kMaxP + l];
                const R h = a.ops.hatD[self * kMaxP + l];
#pragma unroll
                for (int v = 0; v < 5; ++v) acc[v] = acc[v] + s * fs[v] + h * sV[(v + 5 * d) * P3 + m];
            }
        }
#pragma unroll
        for (int v = 0; v < 5; ++v) a.QDot[5 * g + v] = -acc[v];
    }
}

// ------------------------------------------------------------------------------------------------
// k_flux_face: f* = (F_inv(QL,QR) - 1/2 (Fv_L + Fv_R).n) Jf; side 1 gets f*, side 2 gets -f*.
// ------------------------------------------------------------------------------------------------
template <int P, typename R>
__global__ void __launch_bounds__(128) k_flux_face(Args<R> a) {
    constexpr int P2 = P * P;
    const int64_t gid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (gid >= static_cast<int64_t>(a.F) * P2) return;
    const int f = static_cast<int>(gid / P2), p = static_cast<int>(gid - static_cast<int64_t>(f) * P2);
    const int i = p % P, j = p / P;
    int ii, jj;
    left2right(i, j, P - 1, P - 1, a.face_rot[f], ii, jj);
    const int eL = a.face_elem[2 * f], eR = a.face_elem[2 * f + 1];
    const int64_t sL = slot(eL, a.face_side[2 * f]) * P2 + p;
    const int64_t sR = slot(eR, a.face_side[2 * f + 1]) * P2 + ii + P * jj;
    R QL[5], QR[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) { QL[v] = a.QF[5 * sL + v]; QR[v] = a.QF[5 * sR + v]; }
    const R n[3] = {a.fn[3 * gid], a.fn[3 * gid + 1], a.fn[3 * gid + 2]};
    const R J = a.fj[gid];
    R visc[5] = {0, 0, 0, 0, 0};
    if (a.ph.ns) {
        R gl[15], gr[15];
#pragma unroll
        for (int c = 0; c < 15; ++c) { gl[c] = a.GF[15 * sL + c]; gr[c] = a.GF[15 * sR + c]; }
        R muL, kL, muR, kR;
        mu_kappa(a.ph, QL, muL, kL);
        mu_kappa(a.ph, QR, muR, kR);
        R fL[3][5], fR[3][5];
        viscous_flux(a.ph, QL, gl, gl + 5, gl + 10, muL, kL, fL);
        viscous_flux(a.ph, QR, gr, gr + 5, gr + 10, muR, kR, fR);
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            const R x = R(0.5) * (fL[0][v] + fR[0][v]), y = R(0.5) * (fL[1][v] + fR[1][v]), z = R(0.5) * (fL[2][v] + fR[2][v]);
            visc[v] = x * n[0] + y * n[1] + z * n[2];
        }
    }
    R inv[5];
    if (a.ph.riemann == 0) {
        roe_flux(a.ph, QL, QR, n, inv);
    } else {
        const R t1[3] = {a.ft1[3 * gid], a.ft1[3 * gid + 1], a.ft1[3 * gid + 2]};
        const R t2[3] = {a.ft2[3 * gid], a.ft2[3 * gid + 1], a.ft2[3 * gid + 2]};
        lxf_flux(a.ph, QL, QR, n, t1, t2, inv);
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        const R fl = (inv[v] - visc[v]) * J;
        a.FS[5 * sL + v] = fl;
        a.FS[5 * sR + v] = -fl;
    }
}

// ------------------------------------------------------------------------------------------------
// k_surface_rk: QDot = (QDot - surface integral)/J + S; then (stage >= 0) the low-storage update
// G = a_k G + QDot, Q = Q + c_k dt G in FP64.
// ------------------------------------------------------------------------------------------------
template <int P, bool GL, typename R>
__global__ void __launch_bounds__(Geo<P>::THREADS) k_surface_rk(Args<R> a, int stage, double tshift) {
    constexpr int P2 = Geo<P>::P2, P3 = Geo<P>::P3, EPB = Geo<P>::EPB;
    const int le = threadIdx.x / P3, n = threadIdx.x - le * P3;
    const int e = blockIdx.x * EPB + le;
    if (e >= a.K) return;
    const int i = n % P, j = (n / P) % P, k = n / P2;
    const int64_t g = static_cast<int64_t>(e) * P3 + n;
    const R* FL = a.FS + (slot(e, 6) * P2 + (j + P * k)) * 5;
    const R* FR = a.FS + (slot(e, 4) * P2 + (j + P * k)) * 5;
    const R* FF = a.FS + (slot(e, 1) * P2 + (i + P * k)) * 5;
    const R* FB = a.FS + (slot(e, 2) * P2 + (i + P * k)) * 5;
    const R* FO = a.FS + (slot(e, 3) * P2 + (i + P * j)) * 5;
    const R* FT = a.FS + (slot(e, 5) * P2 + (i + P * j)) * 5;
    const R J = a.jac[g];
    R qd[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) qd[v] = a.QDot[5 * g + v];
    if (GL) {
        const R bL = a.ops.bL[0], bR = a.ops.bR[P - 1];
        const bool iL = i == 0, iR = i == P - 1, jL = j == 0, jR = j == P - 1, kL = k == 0, kR = k == P - 1;
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            R fi = R(0);
            if (iL) fi = FL[v] * bL;
            if (iR) fi = fi + FR[v] * bR;
            if (jL) fi = fi + FF[v] * bL;
            if (jR) fi = fi + FB[v] * bR;
            if (kL) fi = fi + FO[v] * bL;
            if (kR) fi = fi + FT[v] * bR;
            qd[v] = (qd[v] - fi) / J;
        }
    } else {
        const R bxl = a.ops.bL[i], bxr = a.ops.bR[i], byl = a.ops.bL[j], byr = a.ops.bR[j];
        const R bzl = a.ops.bL[k], bzr = a.ops.bR[k];
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            R fi = FL[v] * bxl;
            fi = fi + FR[v] * bxr;
            fi = fi + FF[v] * byl;
            fi = fi + FB[v] * byr;
            fi = fi + FO[v] * bzl;
            fi = fi + FT[v] * bzr;
            qd[v] = (qd[v] - fi) / J;
        }
    }
    const double dt = *a.dt;
    if (a.source == 1) {
        double S[5];
        const double t = *a.time + tshift * dt;
        mms_source(a.x[3 * g], a.x[3 * g + 1], a.x[3 * g + 2], t, a.src_gm1, a.src_gM2, a.src_mu, a.src_kappa, S);
#pragma unroll
        for (int v = 0; v < 5; ++v) qd[v] = R(double(qd[v]) + S[v]);
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) a.QDot[5 * g + v] = qd[v];
    if (stage < 0) return;
    const double ak = stage == 0 ? 0.0 : (stage == 1 ? -5.0 / 9.0 : -153.0 / 128.0);
    const double ck = stage == 0 ? 1.0 / 3.0 : (stage == 1 ? 15.0 / 16.0 : 8.0 / 15.0);
    const double cdt = ck * dt;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        const double gn = ak * a.G[5 * g + v] + double(qd[v]);
        a.G[5 * g + v] = gn;
        a.Q[5 * g + v] = a.Q[5 * g + v] + cdt * gn;
    }
}

}  // namespace dg
