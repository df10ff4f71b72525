// DGSEM right-hand side for p-anisotropic elements and for batches of independent cases: every
// element has its own orders (Nx,Ny,Nz) and belongs to one case, each case with its own physics
// constants, time and dt. The arithmetic type R is double (plain form) or float (mixed form); Q and
// the RK register G are FP64 in both.
//
// Work is cut into items: one CTA processes `count` consecutive elements of one order triple and one
// case (the elements are bucketed by order triple on the host), so the per-element loops of a CTA
// have one trip count and the operators of the three directions sit in shared memory. Threads loop
// over the item's nodes, so an item may hold more nodes than the CTA has threads.
//
// Faces follow the reference's conforming treatment (FaceClass.f90:281-470, 597-703, 865-963): each
// face has its own order (Nf1,Nf2) = max of its two sides; the element traces are interpolated to the
// face points with Tset (InterpolationMatrices.f90:42-113), the face quantity is formed there and
// projected back to each side's order with the transposed, weight-scaled Tset. A CTA processes
// FPB faces with one 64-thread group each (a face has at most 8 x 8 points).
//
// Kernels of one RK stage (Navier-Stokes; Euler skips kv_face<JUMP>):
//   kv_face<kJump>   BR1 interface jump 1/2 (U_R - U_L) Jf n at the face points, projected to both sides
//                    (EllipticBR1.f90:571-627)
//   kv_volume        local gradient, lifting, gradient traces, contravariant fluxes and the weak
//                    volume integral -> QDot (HexElementClass.f90:304-531, EllipticBR1.f90:531-569,
//                    SpatialDiscretization.f90:1602-1682, DGIntegrals.f90:56-87)
//   kv_face<kFlux*>  Roe/LxF flux minus the averaged viscous normal flux, times Jf, projected to both
//                    sides, side 2 negated (SpatialDiscretization.f90:1710-1799, EllipticBR1.f90:816-868)
//   kv_update        surface integral, 1/J, source, Williamson RK3 update, Q traces of the new state
//
// Slot data (slot = 6e + side - 1) are stored per slot and variable: value(slot, v, p) at
// [soff[slot]*NV + v*n_slot + p], n_slot the side's point count at the element's own orders.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cstdio>

#include "dg_launch.cuh"

namespace dg {

// Operators of one node count P (NodalStorageClass.f90:170-338), row stride kMaxP.
template <typename R>
struct OpsP {
    R D[kMaxP * kMaxP], hatD[kMaxP * kMaxP];
    R sharpD[kMaxP * kMaxP];  // split form (Gauss-Lobatto nodes); zero otherwise
    R vL[kMaxP], vR[kMaxP], bL[kMaxP], bR[kMaxP];
};

constexpr int kTsetStride = kMaxP * kMaxP;  // Tset(No -> Nd) at tset[(No * kMaxP + Nd) * kTsetStride]

// Per-case FP64 constants: energy reference of the mixed form and the manufactured-source constants.
struct CaseConst {
    double e_ref, gm1, gM2, mu, kappa;
};

// Item classes: 0 holds the items of anisotropic order triples (runtime loop bounds), class P
// (2..kMaxP) the items of the isotropic triple (P,P,P), whose kernels have P as a compile-time
// constant. The items of a class are contiguous.
constexpr int kItemClasses = kMaxP + 1;

template <typename R>
struct VArgs {
    int n_items, n_faces, cap;  // cap: largest node count of an item
    int ns, source;
    int riemann, averaging, grad_vars;  // the host's copies of the solver, average and gradient variables
    int split;                          // split-form volume integral (Gauss-Lobatto nodes)
    int item0;                     // first item of the launch (the grid covers one class)
    int cls[kItemClasses + 1];     // class c holds items [cls[c], cls[c+1])
    int ccap[kItemClasses];        // largest node count of an item of class c (its shared memory)
    // faces whose two sides need a Tset interpolation (kv_face, one 64-thread group per face)
    int n_nc;
    const int* nc_faces;
    // faces whose sides already have the face's point counts (kv_face_direct, one thread per point),
    // grouped by point counts (q1, q2): group g holds face-list entries [gf0[g], gf0[g+1]) and
    // points [gp0[g], gp0[g+1])
    int n_groups;
    const int* direct_faces;
    int gf0[kMaxP * kMaxP + 1];
    int gp0[kMaxP * kMaxP + 1];
    unsigned char gq1[kMaxP * kMaxP];
    unsigned char gq2[kMaxP * kMaxP];
    const int4* items;          // x: first index into item_elems, y: count, z: px|py<<8|pz<<16, w: case
    const int* item_elems;
    const int* eord;            // px|py<<8|pz<<16 per element
    const long long* eoff;      // first node of each element
    const long long* soff;      // first point of each slot
    const int4* faces;          // x: left elem, y: right elem, z: sideL|sideR<<4|rot<<8|q1<<12|q2<<16, w: case
    const long long* foff;      // first face point of each face
    const OpsP<R>* ops;         // [kMaxP + 1], indexed by P
    const R* tset;
    const PhysR<R>* ph;         // per case
    const CaseConst* cc;        // per case
    const double* time;         // per case: step start time
    const double* dt;           // per case
    const R* ja_xi;
    const R* ja_eta;
    const R* ja_zeta;
    const R* jac;
    const R* inv_jac;
    const double* x;
    // Mixed form on geometries that are not free-stream preserving: per node, the momentum residual
    // of the state at rest with unit pressure (3 values), added times p_ref in the update; null when
    // the geometry preserves a uniform state to round-off.
    const double* pstat;
    const BoundaryR<R>* bc;  // boundary conditions of all cases (a boundary face's record holds its index)
    const R* fn;                // face points, 3 per point
    const R* ft1;
    const R* ft2;
    const R* fj;
    double* Q;
    double* G;
    R* QDot;
    R* Ux;
    R* Uy;
    R* Uz;
    R* QF;  // Q traces        (5 per slot point)
    R* GF;  // gradient traces (15 per slot point)
    R* UJ;  // BR1 jumps       (15 per slot point)
    R* FS;  // surface fluxes  (5 per slot point)
};

struct ItemDims {
    int first, count, px, py, pz, kase, np, ntot;
};

// PC > 0: the item belongs to the isotropic class P = PC and its orders are compile-time constants.
template <int PC = 0>
__device__ __forceinline__ ItemDims item_dims(const int4 it) {
    ItemDims d;
    d.first = it.x;
    d.count = it.y;
    d.px = PC ? PC : (it.z & 255);
    d.py = PC ? PC : ((it.z >> 8) & 255);
    d.pz = PC ? PC : ((it.z >> 16) & 255);
    d.kase = it.w;
    d.np = d.px * d.py * d.pz;
    d.ntot = d.count * d.np;
    return d;
}

// Quotient of a small non-negative integer by a runtime divisor through the FP32 reciprocal:
// trunc((n + 1/2) rn(1/d)). (n + 1/2)/d lies at least 1/(2d) from an integer, and the two roundings
// move the product by at most (n + 1/2)/d * 1.5 * 2^-23, which stays below 1/(2d) for n < 2^21; the
// item and face indices decoded here are far below that. Five instructions instead of the integer
// division's twenty.
struct Div {
    int d;
    float r;
};
__device__ __forceinline__ Div make_div(int d) { return {d, __frcp_rn(static_cast<float>(d))}; }
__device__ __forceinline__ int quot(int n, const Div& v) {
    return __float2int_rz((static_cast<float>(n) + 0.5f) * v.r);
}

// Item node t -> (local element le, node n, indices i, j, k); compile-time orders keep the constant
// divisions.
template <int PC>
struct NodeDecoder {
    int np, px, py;
    Div dnp, dpx, dpxy;
    __device__ __forceinline__ explicit NodeDecoder(const ItemDims& d) : np(d.np), px(d.px), py(d.py) {
        if constexpr (PC == 0) {
            dnp = make_div(np);
            dpx = make_div(px);
            dpxy = make_div(px * py);
        }
    }
    __device__ __forceinline__ void elem(int t, int& le, int& n) const {
        if constexpr (PC > 0) le = t / (PC * PC * PC);
        else le = quot(t, dnp);
        n = t - le * np;
    }
    __device__ __forceinline__ void ijk(int n, int& i, int& j, int& k) const {
        if constexpr (PC > 0) {
            i = n % PC;
            j = (n / PC) % PC;
            k = n / (PC * PC);
        } else {
            const int a = quot(n, dpx);
            k = quot(n, dpxy);
            i = n - a * px;
            j = a - k * py;
        }
    }
};

// Face point counts of a side (first, second face direction), sides numbered as the reference.
__device__ __forceinline__ void side_dims(int side, int ord, int& d1, int& d2) {
    const int px = ord & 255, py = (ord >> 8) & 255, pz = (ord >> 16) & 255;
    switch (side) {
        case 1: case 2: d1 = px; d2 = pz; break;
        case 3: case 5: d1 = px; d2 = py; break;
        default: d1 = py; d2 = pz; break;
    }
}

// Node at line position l through face point (ca, cb) of a side.
__device__ __forceinline__ int vline_node(int side, int ca, int cb, int l, int px, int py) {
    switch (side) {
        case 1: case 2: return ca + px * (l + py * cb);
        case 3: case 5: return ca + px * (cb + py * l);
        default: return l + px * (ca + py * cb);
    }
}

// Trace task r of an element (tasks ordered side 1..6, point p within the side).
__device__ __forceinline__ int side_of_task(int r, int A, int B, int C, int& p) {
    if (r < A) { p = r; return 1; }
    r -= A;
    if (r < A) { p = r; return 2; }
    r -= A;
    if (r < B) { p = r; return 3; }
    r -= B;
    if (r < C) { p = r; return 4; }
    r -= C;
    if (r < B) { p = r; return 5; }
    p = r - B;
    return 6;
}

// The three directions' operators of an item into shared memory.
template <typename R>
__device__ __forceinline__ void load_ops(const OpsP<R>* ops, OpsP<R>* s, int px, int py, int pz) {
    constexpr int W = static_cast<int>(sizeof(OpsP<R>) / sizeof(R));
    for (int t = threadIdx.x; t < 3 * W; t += blockDim.x) {
        const int d = t / W, w = t - d * W;
        const int P = d == 0 ? px : (d == 1 ? py : pz);
        reinterpret_cast<R*>(s)[t] = reinterpret_cast<const R*>(ops + P)[w];
    }
}

// NV traces of the item's nodes held in s (value v of item node m at s[v*ntot + m]) into the slots.
template <typename R, int NV, int PC>
__device__ __forceinline__ void write_traces(const VArgs<R>& a, const ItemDims& d, const OpsP<R>* sO, const R* s,
                                             R* dst) {
    const int A = d.px * d.pz, B = d.px * d.py, C = d.py * d.pz, Te = 2 * (A + B + C);
    const Div dte = make_div(Te), dx = make_div(d.px), dy = make_div(d.py);
    for (int t = threadIdx.x; t < d.count * Te; t += blockDim.x) {
        const int le = PC ? t / (6 * PC * PC) : quot(t, dte);
        int p;
        const int side = side_of_task(t - le * Te, A, B, C, p);
        const int ns = side <= 2 ? A : ((side == 3 || side == 5) ? B : C);
        const int d1 = side <= 2 ? d.px : ((side == 3 || side == 5) ? d.px : d.py);
        const int cb = PC ? p / PC : quot(p, side == 4 || side == 6 ? dy : dx), ca = p - cb * d1;
        const int dir = side <= 2 ? 1 : ((side == 3 || side == 5) ? 2 : 0);
        const int L = dir == 0 ? d.px : (dir == 1 ? d.py : d.pz);
        const R* v = (side == 2 || side == 4 || side == 5) ? sO[dir].vR : sO[dir].vL;
        const R* base = s + le * d.np;
        R acc[NV];
#pragma unroll
        for (int c = 0; c < NV; ++c) acc[c] = R(0);
        #pragma unroll
        for (int l = 0; l < L; ++l) {
            const R w = v[l];
            const int m = vline_node(side, ca, cb, l, d.px, d.py);
#pragma unroll
            for (int c = 0; c < NV; ++c) acc[c] = acc[c] + base[c * d.ntot + m] * w;
        }
        const int e = a.item_elems[d.first + le];
        R* o = dst + a.soff[6LL * e + side - 1] * NV + p;
#pragma unroll
        for (int c = 0; c < NV; ++c) o[c * ns] = acc[c];
    }
}

// ------------------------------------------------------------------------------------------------
// kv_traces: Q traces of the current state (after an upload).
// ------------------------------------------------------------------------------------------------
template <typename R, int PC>
__global__ void __launch_bounds__(256) kv_traces(VArgs<R> a) {
    extern __shared__ __align__(16) unsigned char vsm[];
    const ItemDims d = item_dims<PC>(a.items[a.item0 + blockIdx.x]);
    OpsP<R>* sO = reinterpret_cast<OpsP<R>*>(vsm);
    R* sQ = reinterpret_cast<R*>(sO + 3);
    load_ops(a.ops, sO, d.px, d.py, d.pz);
    const double eref = a.cc[d.kase].e_ref;
    const NodeDecoder<PC> nd(d);
    for (int t = threadIdx.x; t < d.ntot; t += blockDim.x) {
        int le, n;
        nd.elem(t, le, n);
        const long long g = a.eoff[a.item_elems[d.first + le]] + n;
#pragma unroll
        for (int v = 0; v < 4; ++v) sQ[v * d.ntot + t] = R(a.Q[5 * g + v]);
        sQ[4 * d.ntot + t] = R(a.Q[5 * g + 4] - eref);
    }
    __syncthreads();
    write_traces<R, 5, PC>(a, d, sO, sQ, a.QF);
}

// ------------------------------------------------------------------------------------------------
// kv_volume: gradient + lifting + gradient traces (Navier-Stokes), fluxes, weak volume integral.
// ------------------------------------------------------------------------------------------------
template <typename R, int PC>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 4 : 0) kv_volume(VArgs<R> a, int store_grad) {
    extern __shared__ __align__(16) unsigned char vsm[];
    const ItemDims d = item_dims<PC>(a.items[a.item0 + blockIdx.x]);
    const int px = d.px, py = d.py, pz = d.pz, np = d.np, ntot = d.ntot;
    OpsP<R>* sO = reinterpret_cast<OpsP<R>*>(vsm);  // xi, eta, zeta operators
    R* sQ = reinterpret_cast<R*>(sO + 3);            // 5*ntot: state
    R* sG = sQ + 5 * ntot;                           // 15*ntot: lifted gradient, then the fluxes
    R* sM = sG + 15 * ntot;                          // split form: 9*ntot metric terms
    load_ops(a.ops, sO, px, py, pz);
    const PhysR<R> ph = a.ph[d.kase];
    const double eref = a.cc[d.kase].e_ref;
    // sQ holds the gradient variables while the gradient is formed: the state itself, or U(Q) for
    // the entropy and energy variables (then the fluxes below read the state from global memory)
    const bool gv = a.ns && ph.grad_vars != 0;
    const NodeDecoder<PC> nd(d);
    for (int t = threadIdx.x; t < ntot; t += blockDim.x) {
        int le, n;
        nd.elem(t, le, n);
        const long long g = a.eoff[a.item_elems[d.first + le]] + n;
        R x[5];
#pragma unroll
        for (int v = 0; v < 4; ++v) x[v] = R(a.Q[5 * g + v]);
        x[4] = R(a.Q[5 * g + 4] - eref);
        if (gv) {
            R u[5];
            gradient_variables(ph, x, u);
#pragma unroll
            for (int v = 0; v < 5; ++v) sQ[v * ntot + t] = u[v];
        } else {
#pragma unroll
            for (int v = 0; v < 5; ++v) sQ[v * ntot + t] = x[v];
        }
    }
    __syncthreads();
    if (a.ns) {
        const int A = px * pz, B = px * py, C = py * pz;
        for (int t = threadIdx.x; t < ntot; t += blockDim.x) {
            int le, n, i, j, k;
            nd.elem(t, le, n);
            nd.ijk(n, i, j, k);
            const int e = a.item_elems[d.first + le];
            const long long g = a.eoff[e] + n;
            const R* q0 = sQ + le * np;
            R uxi[5] = {0, 0, 0, 0, 0}, ueta[5] = {0, 0, 0, 0, 0}, uzeta[5] = {0, 0, 0, 0, 0};
            #pragma unroll
            for (int l = 0; l < px; ++l) {
                const R w = sO[0].D[i * kMaxP + l];
#pragma unroll
                for (int v = 0; v < 5; ++v) uxi[v] = uxi[v] + q0[v * ntot + l + px * (j + py * k)] * w;
            }
            #pragma unroll
            for (int l = 0; l < py; ++l) {
                const R w = sO[1].D[j * kMaxP + l];
#pragma unroll
                for (int v = 0; v < 5; ++v) ueta[v] = ueta[v] + q0[v * ntot + i + px * (l + py * k)] * w;
            }
            #pragma unroll
            for (int l = 0; l < pz; ++l) {
                const R w = sO[2].D[k * kMaxP + l];
#pragma unroll
                for (int v = 0; v < 5; ++v) uzeta[v] = uzeta[v] + q0[v * ntot + i + px * (j + py * l)] * w;
            }
            R jx[3], je[3], jz[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                jx[c] = a.ja_xi[3 * g + c];
                je[c] = a.ja_eta[3 * g + c];
                jz[c] = a.ja_zeta[3 * g + c];
            }
            const R ij = a.inv_jac[g];
            R U[3][5];
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                U[0][v] = (uxi[v] * jx[0] + ueta[v] * je[0] + uzeta[v] * jz[0]) * ij;
                U[1][v] = (uxi[v] * jx[1] + ueta[v] * je[1] + uzeta[v] * jz[1]) * ij;
                U[2][v] = (uxi[v] * jx[2] + ueta[v] * je[2] + uzeta[v] * jz[2]) * ij;
            }
            // lifting (VectorWeakIntegrals_StdFace order: left, right, front, back, bottom, top)
            const long long s0 = 6LL * e;
            const R* HF = a.UJ + a.soff[s0 + 0] * 15 + (i + px * k);
            const R* HB = a.UJ + a.soff[s0 + 1] * 15 + (i + px * k);
            const R* HO = a.UJ + a.soff[s0 + 2] * 15 + (i + px * j);
            const R* HR = a.UJ + a.soff[s0 + 3] * 15 + (j + py * k);
            const R* HT = a.UJ + a.soff[s0 + 4] * 15 + (i + px * j);
            const R* HL = a.UJ + a.soff[s0 + 5] * 15 + (j + py * k);
            const R bxl = sO[0].bL[i], bxr = sO[0].bR[i], byl = sO[1].bL[j], byr = sO[1].bR[j];
            const R bzl = sO[2].bL[k], bzr = sO[2].bR[k];
#pragma unroll
            for (int dd = 0; dd < 3; ++dd)
#pragma unroll
                for (int v = 0; v < 5; ++v) {
                    const int c = v + 5 * dd;
                    R fi = HL[c * C] * bxl;
                    fi = fi + HR[c * C] * bxr;
                    fi = fi + HF[c * A] * byl;
                    fi = fi + HB[c * A] * byr;
                    fi = fi + HO[c * B] * bzl;
                    fi = fi + HT[c * B] * bzr;
                    U[dd][v] = U[dd][v] + fi * ij;
                }
#pragma unroll
            for (int dd = 0; dd < 3; ++dd)
#pragma unroll
                for (int v = 0; v < 5; ++v) sG[(v + 5 * dd) * ntot + t] = U[dd][v];
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
        write_traces<R, 15, PC>(a, d, sO, sG, a.GF);
        __syncthreads();
    }
    // contravariant fluxes F = Finv - Fvisc at each node, over the node's own gradient column
    for (int t = threadIdx.x; t < ntot; t += blockDim.x) {
        int le, n;
        nd.elem(t, le, n);
        const long long g = a.eoff[a.item_elems[d.first + le]] + n;
        R q[5], jx[3], je[3], jz[3];
        if (gv) {
#pragma unroll
            for (int v = 0; v < 4; ++v) q[v] = R(a.Q[5 * g + v]);
            q[4] = R(a.Q[5 * g + 4] - eref);
        } else {
#pragma unroll
            for (int v = 0; v < 5; ++v) q[v] = sQ[v * ntot + t];
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            jx[c] = a.ja_xi[3 * g + c];
            je[c] = a.ja_eta[3 * g + c];
            jz[c] = a.ja_zeta[3 * g + c];
        }
        R F[3][5];
        if (a.split) {
            // split form: the viscous contravariant fluxes here; the two-point fluxes below read
            // every node's state and metric terms from shared memory
#pragma unroll
            for (int dd = 0; dd < 3; ++dd)
#pragma unroll
                for (int v = 0; v < 5; ++v) F[dd][v] = R(0);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                sM[c * ntot + t] = jx[c];
                sM[(3 + c) * ntot + t] = je[c];
                sM[(6 + c) * ntot + t] = jz[c];
            }
        } else {
            euler_contravariant(ph, q, jx, je, jz, F);
        }
        if (a.ns) {
            R Ug[15];
#pragma unroll
            for (int c = 0; c < 15; ++c) Ug[c] = sG[c * ntot + t];
            R mu, kap;
            mu_kappa(ph, q, mu, kap);
            R Cv[3][5];
            viscous_flux(ph, q, Ug, Ug + 5, Ug + 10, mu, kap, Cv);
            const R* ja[3] = {jx, je, jz};
            const R sgn = a.split ? R(1) : R(-1);  // split: Fv; standard: Finv - Fv
#pragma unroll
            for (int dd = 0; dd < 3; ++dd)
#pragma unroll
                for (int v = 0; v < 5; ++v)
                    F[dd][v] = F[dd][v] + sgn * (Cv[0][v] * ja[dd][0] + Cv[1][v] * ja[dd][1] + Cv[2][v] * ja[dd][2]);
        }
#pragma unroll
        for (int dd = 0; dd < 3; ++dd)
#pragma unroll
            for (int v = 0; v < 5; ++v) sG[(v + 5 * dd) * ntot + t] = F[dd][v];
        if (a.split && gv) {  // the state in place of the gradient variables
#pragma unroll
            for (int v = 0; v < 5; ++v) sQ[v * ntot + t] = q[v];
        }
    }
    __syncthreads();
    if (a.split) {
        // Split form with per-direction orders (HyperbolicSplitForm.f90:64-116, DGIntegrals.f90:92-129):
        // along each direction's line, volInt += sharpD(i,l) f#(l,i) + hatD(i,l) Fv(l), with the
        // two-point flux of each pair evaluated with the lower line index as "left" and the node's
        // own contravariant Euler flux at l = i; QDot = -volInt.
        for (int t = threadIdx.x; t < ntot; t += blockDim.x) {
            int le, n, i, j, k;
            nd.elem(t, le, n);
            nd.ijk(n, i, j, k);
            const long long g = a.eoff[a.item_elems[d.first + le]] + n;
            const int b0 = le * np;
            R q[5], jm[3][3];
#pragma unroll
            for (int v = 0; v < 5; ++v) q[v] = sQ[v * ntot + t];
#pragma unroll
            for (int dd = 0; dd < 3; ++dd)
#pragma unroll
                for (int c = 0; c < 3; ++c) jm[dd][c] = sM[(3 * dd + c) * ntot + t];
            R Fi[3][5];
            euler_contravariant(ph, q, jm[0], jm[1], jm[2], Fi);
            R acc[5] = {0, 0, 0, 0, 0};
#pragma unroll
            for (int dd = 0; dd < 3; ++dd) {
                const int len = dd == 0 ? px : (dd == 1 ? py : pz);
                const int self = dd == 0 ? i : (dd == 1 ? j : k);
                const int stride = dd == 0 ? 1 : (dd == 1 ? px : px * py);
                const int first = n - self * stride;
                for (int l = 0; l < len; ++l) {
                    const int m = b0 + first + l * stride;
                    R fs[5];
                    if (l == self) {
#pragma unroll
                        for (int v = 0; v < 5; ++v) fs[v] = Fi[dd][v];
                    } else {
                        R qo[5], jo[3];
#pragma unroll
                        for (int v = 0; v < 5; ++v) qo[v] = sQ[v * ntot + m];
#pragma unroll
                        for (int c = 0; c < 3; ++c) jo[c] = sM[(3 * dd + c) * ntot + m];
                        if (self < l) two_point_flux(ph, q, qo, jm[dd], jo, fs);
                        else two_point_flux(ph, qo, q, jo, jm[dd], fs);
                    }
                    const R sh = sO[dd].sharpD[self * kMaxP + l];
                    const R h = sO[dd].hatD[self * kMaxP + l];
#pragma unroll
                    for (int v = 0; v < 5; ++v) acc[v] = acc[v] + sh * fs[v] + h * sG[(v + 5 * dd) * ntot + m];
                }
            }
#pragma unroll
            for (int v = 0; v < 5; ++v) a.QDot[5 * g + v] = -acc[v];
        }
        return;
    }
    // ScalarWeakIntegrals_StdVolumeGreen
    for (int t = threadIdx.x; t < ntot; t += blockDim.x) {
        int le, n, i, j, k;
        nd.elem(t, le, n);
        nd.ijk(n, i, j, k);
        const long long g = a.eoff[a.item_elems[d.first + le]] + n;
        const R* F0 = sG + le * np;
        R acc[5] = {0, 0, 0, 0, 0};
        #pragma unroll
        for (int l = 0; l < px; ++l) {
            const R h = sO[0].hatD[i * kMaxP + l];
#pragma unroll
            for (int v = 0; v < 5; ++v) acc[v] = acc[v] + h * F0[v * ntot + l + px * (j + py * k)];
        }
        #pragma unroll
        for (int l = 0; l < py; ++l) {
            const R h = sO[1].hatD[j * kMaxP + l];
#pragma unroll
            for (int v = 0; v < 5; ++v) acc[v] = acc[v] + h * F0[(5 + v) * ntot + i + px * (l + py * k)];
        }
        #pragma unroll
        for (int l = 0; l < pz; ++l) {
            const R h = sO[2].hatD[k * kMaxP + l];
#pragma unroll
            for (int v = 0; v < 5; ++v) acc[v] = acc[v] + h * F0[(10 + v) * ntot + i + px * (j + py * l)];
        }
#pragma unroll
        for (int v = 0; v < 5; ++v) a.QDot[5 * g + v] = acc[v];
    }
}

// ------------------------------------------------------------------------------------------------
// kv_face: BR1 jump (kJump) or interface flux (kFluxEuler / kFluxNS) at the face points.
// ------------------------------------------------------------------------------------------------
constexpr int kJump = 0;
constexpr int kFluxEuler = 1;
constexpr int kFluxNS = 2;
constexpr int kFacePts = kMaxP * kMaxP;  // threads per face group

template <typename R, int MODE>
struct FaceCfg {
    static constexpr int NVIN = MODE == kFluxNS ? 20 : 5;
    static constexpr int NVOUT = MODE == kJump ? 15 : 5;
    static constexpr int NVB = NVIN > NVOUT ? NVIN : NVOUT;
    static constexpr int FPB = (sizeof(R) == 8 && NVB > 5) ? 2 : 4;  // faces per CTA
    static constexpr int THREADS = FPB * kFacePts;
    static constexpr size_t SMEM = static_cast<size_t>(FPB) * 4 * NVB * kFacePts * sizeof(R);
};

// Interpolation of NV values from (s1 x s2) points in S to the face's (q1 x q2) points, one of the
// two passes (first: along the first face direction, S -> A; second: along the second, cur -> nxt).
template <typename R, int NV>
__device__ __forceinline__ void face_pass1(const R* tset, const R* S, R* A, int s1, int s2, int q1, const Div& dq1,
                                           int lane) {
    const R* T = tset + ((s1 - 1) * kMaxP + (q1 - 1)) * kTsetStride;
    for (int p = lane; p < q1 * s2; p += kFacePts) {  // A(i, l) = sum_m T1(i, m) S(m, l)
        const int l = quot(p, dq1), i = p - l * q1;
        R acc[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[v] = R(0);
        for (int m = 0; m < s1; ++m) {
            const R w = T[i * kMaxP + m];
#pragma unroll
            for (int v = 0; v < NV; ++v) acc[v] = acc[v] + w * S[v * kFacePts + m + s1 * l];
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) A[v * kFacePts + p] = acc[v];
    }
}
template <typename R, int NV>
__device__ __forceinline__ void face_pass2(const R* tset, const R* cur, R* nxt, int s2, int q1, int q2, const Div& dq1,
                                           int lane) {
    const R* T = tset + ((s2 - 1) * kMaxP + (q2 - 1)) * kTsetStride;
    for (int p = lane; p < q1 * q2; p += kFacePts) {  // nxt(i, j) = sum_l T2(j, l) cur(i, l)
        const int j = quot(p, dq1), i = p - j * q1;
        R acc[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[v] = R(0);
        for (int l = 0; l < s2; ++l) {
            const R w = T[j * kMaxP + l];
#pragma unroll
            for (int v = 0; v < NV; ++v) acc[v] = acc[v] + w * cur[v * kFacePts + i + q1 * l];
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) nxt[v * kFacePts + p] = acc[v];
    }
}

// Both sides' traces to the face points: the left side's (l1 x l2) points in SL (work buffer AL) and
// the right side's (s1R x s2R) points in SR (AR), each pass of the two sides between the same two
// CTA barriers. XL, XR receive the buffers that hold the results. Every thread of the CTA must call it.
template <typename R, int NV>
__device__ __forceinline__ void both_to_face_points(const R* tset, R* SL, R* AL, int l1, int l2, R* SR, R* AR, int s1R,
                                                    int s2R, int q1, int q2, int lane, bool active, const R*& XL,
                                                    const R*& XR) {
    const Div dq1 = make_div(q1);
    const bool a1 = active && l1 != q1, a2 = active && l2 != q2;
    const bool b1 = active && s1R != q1, b2 = active && s2R != q2;
    if (a1) face_pass1<R, NV>(tset, SL, AL, l1, l2, q1, dq1, lane);
    if (b1) face_pass1<R, NV>(tset, SR, AR, s1R, s2R, q1, dq1, lane);
    __syncthreads();
    R* curL = a1 ? AL : SL;
    R* nxtL = a1 ? SL : AL;
    R* curR = b1 ? AR : SR;
    R* nxtR = b1 ? SR : AR;
    if (a2) face_pass2<R, NV>(tset, curL, nxtL, l2, q1, q2, dq1, lane);
    if (b2) face_pass2<R, NV>(tset, curR, nxtR, s2R, q1, q2, dq1, lane);
    __syncthreads();
    XL = a2 ? nxtL : curL;
    XR = b2 ? nxtR : curR;
}

// V selects the compiled variant: for kJump, gradient variables other than the state (V = 1); for
// the flux modes, the Riemann solvers beyond Roe / LxF / central / Rusanov / u-diss or the
// logarithmic-mean averages (V = 1). The common variants (V = 0) keep the short code and register
// footprint.
template <typename R, int MODE, int V>
__global__ void __launch_bounds__(FaceCfg<R, MODE>::THREADS, (sizeof(R) == 4 && MODE == kFluxEuler && V == 0) ? 5 : 0)
    kv_face(VArgs<R> a) {
    using Cfg = FaceCfg<R, MODE>;
    constexpr int NVIN = Cfg::NVIN, NVOUT = Cfg::NVOUT, NVB = Cfg::NVB, NP = kFacePts;
    extern __shared__ __align__(16) unsigned char fsm[];
    const int grp = threadIdx.x / NP, lane = threadIdx.x - grp * NP;
    R* SL = reinterpret_cast<R*>(fsm) + grp * 4 * NVB * NP;
    R* AL = SL + NVB * NP;
    R* SR = AL + NVB * NP;
    R* AR = SR + NVB * NP;
    const int fi = blockIdx.x * Cfg::FPB + grp;
    const bool active = fi < a.n_nc;
    const int f = active ? a.nc_faces[fi] : 0;
    int eL = 0, eR = 0, rot = 0, q1 = 1, q2 = 1, kase = 0;
    int l1 = 1, l2 = 1, r1 = 1, r2 = 1, s1R = 1, s2R = 1;
    long long offL = 0, offR = 0, fo = 0;
    if (active) {
        const int4 fd = a.faces[f];
        eL = fd.x;
        eR = fd.y;
        const int sL = fd.z & 15, sR = (fd.z >> 4) & 15;
        rot = (fd.z >> 8) & 15;
        q1 = (fd.z >> 12) & 15;
        q2 = (fd.z >> 16) & 15;
        kase = fd.w;
        side_dims(sL, a.eord[eL], l1, l2);
        side_dims(sR, a.eord[eR], r1, r2);
        const bool swap = !(rot == 0 || rot == 2 || rot == 5 || rot == 7);
        s1R = swap ? r2 : r1;
        s2R = swap ? r1 : r2;
        offL = a.soff[6LL * eL + sL - 1];
        offR = a.soff[6LL * eR + sR - 1];
        fo = a.foff[f];
    }
    const int nL = l1 * l2, nR = r1 * r2;
    if (active) {
        for (int p = lane; p < nL; p += NP) {
#pragma unroll
            for (int v = 0; v < 5; ++v) SL[v * NP + p] = a.QF[offL * 5 + v * nL + p];
            if (MODE == kFluxNS) {
#pragma unroll
                for (int c = 0; c < 15; ++c) SL[(5 + c) * NP + p] = a.GF[offL * 15 + c * nL + p];
            }
        }
        const Div ds1R = make_div(s1R);
        for (int p = lane; p < nR; p += NP) {  // right trace in the left side's orientation
            const int j = quot(p, ds1R), i = p - j * s1R;
            int ii, jj;
            left2right(i, j, s1R - 1, s2R - 1, rot, ii, jj);
            const int src = ii + r1 * jj;
#pragma unroll
            for (int v = 0; v < 5; ++v) SR[v * NP + p] = a.QF[offR * 5 + v * nR + src];
            if (MODE == kFluxNS) {
#pragma unroll
                for (int c = 0; c < 15; ++c) SR[(5 + c) * NP + p] = a.GF[offR * 15 + c * nR + src];
            }
        }
    }
    __syncthreads();
    const R *XL, *XR;
    both_to_face_points<R, NVIN>(a.tset, SL, AL, l1, l2, SR, AR, s1R, s2R, q1, q2, lane, active, XL, XR);
    R out[NVOUT];
    const bool point = active && lane < q1 * q2;
    if (point) {
        const long long gp = fo + lane;
        const R n[3] = {a.fn[3 * gp], a.fn[3 * gp + 1], a.fn[3 * gp + 2]};
        const R J = a.fj[gp];
        if (MODE == kJump) {
            const PhysR<R> ph = a.ph[kase];
            R QL[5], QR[5], UL[5], UR[5];
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                QL[v] = XL[v * NP + lane];
                QR[v] = XR[v * NP + lane];
            }
            if (V) {
                gradient_variables(ph, QL, UL);
                gradient_variables(ph, QR, UR);
            } else {
#pragma unroll
                for (int v = 0; v < 5; ++v) {
                    UL[v] = QL[v];
                    UR[v] = QR[v];
                }
            }
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                const R u = R(0.5) * (UR[v] - UL[v]) * J;
                out[v] = u * n[0];
                out[5 + v] = u * n[1];
                out[10 + v] = u * n[2];
            }
        } else {
            const PhysR<R> ph = a.ph[kase];
            R QL[5], QR[5], inv[5];
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                QL[v] = XL[v * NP + lane];
                QR[v] = XR[v * NP + lane];
            }
            if (V) {
                const R t1[3] = {a.ft1[3 * gp], a.ft1[3 * gp + 1], a.ft1[3 * gp + 2]};
                const R t2[3] = {a.ft2[3 * gp], a.ft2[3 * gp + 1], a.ft2[3 * gp + 2]};
                riemann_flux(ph, QL, QR, n, t1, t2, inv);
            } else if (ph.riemann == 0) {
                roe_flux(ph, QL, QR, n, inv);
            } else if (ph.riemann == 3) {
                rusanov_flux(ph, QL, QR, n, inv);
            } else {  // LxF, central, u-diss
                const R t1[3] = {a.ft1[3 * gp], a.ft1[3 * gp + 1], a.ft1[3 * gp + 2]};
                const R t2[3] = {a.ft2[3 * gp], a.ft2[3 * gp + 1], a.ft2[3 * gp + 2]};
                lxf_flux<R, false>(ph, QL, QR, n, t1, t2, inv);
            }
            R visc[5] = {0, 0, 0, 0, 0};
            if (MODE == kFluxNS) {
                R gl[15], gr[15];
#pragma unroll
                for (int c = 0; c < 15; ++c) {
                    gl[c] = XL[(5 + c) * NP + lane];
                    gr[c] = XR[(5 + c) * NP + lane];
                }
                R mu, kap, FL[3][5], FR[3][5];
                mu_kappa(ph, QL, mu, kap);
                viscous_flux(ph, QL, gl, gl + 5, gl + 10, mu, kap, FL);
                mu_kappa(ph, QR, mu, kap);
                viscous_flux(ph, QR, gr, gr + 5, gr + 10, mu, kap, FR);
#pragma unroll
                for (int v = 0; v < 5; ++v)
                    visc[v] = R(0.5) * (FL[0][v] + FR[0][v]) * n[0] + R(0.5) * (FL[1][v] + FR[1][v]) * n[1] +
                              R(0.5) * (FL[2][v] + FR[2][v]) * n[2];
            }
#pragma unroll
            for (int v = 0; v < 5; ++v) out[v] = (inv[v] - visc[v]) * J;
        }
    }
    __syncthreads();  // the traces are consumed: SL holds the face values from here on
    if (point) {
#pragma unroll
        for (int v = 0; v < NVOUT; ++v) SL[v * NP + lane] = out[v];
    }
    __syncthreads();
    // projection to each side's order (transposed Tset), first direction into AL / AR
    const bool pL1 = active && l1 != q1, pL2 = active && l2 != q2;
    const bool pR1 = active && s1R != q1, pR2 = active && s2R != q2;
    const Div dl1 = make_div(l1), dsR = make_div(s1R);
    if (pL1) {
        const R* T = a.tset + ((q1 - 1) * kMaxP + (l1 - 1)) * kTsetStride;
        for (int p = lane; p < l1 * q2; p += NP) {
            const int l = quot(p, dl1), i = p - l * l1;
#pragma unroll
            for (int v = 0; v < NVOUT; ++v) {
                R acc = R(0);
                for (int m = 0; m < q1; ++m) acc = acc + T[i * kMaxP + m] * SL[v * NP + m + q1 * l];
                AL[v * NP + p] = acc;
            }
        }
    }
    if (pR1) {
        const R* T = a.tset + ((q1 - 1) * kMaxP + (s1R - 1)) * kTsetStride;
        for (int p = lane; p < s1R * q2; p += NP) {
            const int l = quot(p, dsR), i = p - l * s1R;
#pragma unroll
            for (int v = 0; v < NVOUT; ++v) {
                R acc = R(0);
                for (int m = 0; m < q1; ++m) acc = acc + T[i * kMaxP + m] * SL[v * NP + m + q1 * l];
                AR[v * NP + p] = acc;
            }
        }
    }
    __syncthreads();
    if (!active) return;
    R* dstL = MODE == kJump ? a.UJ + offL * 15 : a.FS + offL * 5;
    R* dstR = MODE == kJump ? a.UJ + offR * 15 : a.FS + offR * 5;
    const R sign2 = MODE == kJump ? R(1) : R(-1);
    {
        const R* src = pL1 ? AL : SL;  // (l1 x q2) points
        const R* T = a.tset + ((q2 - 1) * kMaxP + (l2 - 1)) * kTsetStride;
        for (int p = lane; p < nL; p += NP) {
            const int j = quot(p, dl1), i = p - j * l1;
#pragma unroll
            for (int v = 0; v < NVOUT; ++v) {
                R val;
                if (pL2) {
                    val = R(0);
                    for (int l = 0; l < q2; ++l) val = val + T[j * kMaxP + l] * src[v * NP + i + l1 * l];
                } else {
                    val = src[v * NP + i + l1 * j];
                }
                dstL[v * nL + p] = val;
            }
        }
    }
    {
        const R* src = pR1 ? AR : SL;  // (s1R x q2) points
        const R* T = a.tset + ((q2 - 1) * kMaxP + (s2R - 1)) * kTsetStride;
        for (int p = lane; p < nR; p += NP) {
            const int j = quot(p, dsR), i = p - j * s1R;
            int ii, jj;
            left2right(i, j, s1R - 1, s2R - 1, rot, ii, jj);
            const int o = ii + r1 * jj;
#pragma unroll
            for (int v = 0; v < NVOUT; ++v) {
                R val;
                if (pR2) {
                    val = R(0);
                    for (int l = 0; l < q2; ++l) val = val + T[j * kMaxP + l] * src[v * NP + i + s1R * l];
                } else {
                    val = src[v * NP + i + s1R * j];
                }
                dstR[v * nR + o] = sign2 * val;
            }
        }
    }
}

// ------------------------------------------------------------------------------------------------
// kv_face_direct: the same face quantities for faces whose sides already have the face's point
// counts (the Tset interpolation is the identity there, FaceClass.f90:281-382 projection type 0):
// one thread per face point reads both sides' traces in place, the right side re-indexed by
// leftIndexes2Right, and writes both sides' results.
// ------------------------------------------------------------------------------------------------
template <typename R, int MODE, int V>
__global__ void __launch_bounds__(128) kv_face_direct(VArgs<R> a) {
    using Cfg = FaceCfg<R, MODE>;
    constexpr int NVOUT = Cfg::NVOUT;
    const int gp = blockIdx.x * blockDim.x + threadIdx.x;
    if (gp >= a.gp0[a.n_groups]) return;
    int g = 0;
    while (gp >= a.gp0[g + 1]) ++g;
    const int q1 = a.gq1[g], q2 = a.gq2[g], np = q1 * q2;
    const int local = gp - a.gp0[g];
    const int f = a.direct_faces[a.gf0[g] + local / np];
    const int p = local % np;
    const int i = p % q1, j = p / q1;
    const int4 fd = a.faces[f];
    const int eL = fd.x, eR = fd.y, sL = fd.z & 15, sR = (fd.z >> 4) & 15, rot = (fd.z >> 8) & 15;
    const bool boundary = eR < 0;  // one element side; the condition index sits in bits 20.. of z
    int r1 = q1, r2 = q2;
    if (!boundary) side_dims(sR, a.eord[eR], r1, r2);
    int ii = i, jj = j;
    if (!boundary) left2right(i, j, q1 - 1, q2 - 1, rot, ii, jj);
    const int pr = ii + r1 * jj;
    const long long offL = a.soff[6LL * eL + sL - 1];
    const long long offR = boundary ? offL : a.soff[6LL * eR + sR - 1];
    const long long gpt = a.foff[f] + p;
    const R n[3] = {a.fn[3 * gpt], a.fn[3 * gpt + 1], a.fn[3 * gpt + 2]};
    const R J = a.fj[gpt];
    R QL[5], QR[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        QL[v] = a.QF[offL * 5 + v * np + p];
        QR[v] = a.QF[offR * 5 + v * np + pr];
    }
    R out[NVOUT];
    if (MODE == kJump && boundary) {  // (U* - U) Jf n (EllipticBR1.f90:686-736)
        const PhysR<R> ph = a.ph[fd.w];
        R UL[5], us[5];
        gradient_variables(ph, QL, UL);
        bc_gradvars(ph, a.bc[static_cast<unsigned>(fd.z) >> 20], n, QL, UL, us);
        R* dL = a.UJ + offL * 15 + p;
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            const R u = (us[v] - UL[v]) * J;
            dL[v * np] = u * n[0];
            dL[(5 + v) * np] = u * n[1];
            dL[(10 + v) * np] = u * n[2];
        }
        return;
    }
    if (MODE != kJump && boundary) {  // the condition's external state (computeBoundaryFlux)
#pragma unroll
        for (int v = 0; v < 5; ++v) QR[v] = QL[v];
        bc_state(a.ph[fd.w], a.bc[static_cast<unsigned>(fd.z) >> 20], n, QR);
    }
    if (MODE == kJump) {
        R UL[5], UR[5];
        if (V) {
            gradient_variables(a.ph[fd.w], QL, UL);
            gradient_variables(a.ph[fd.w], QR, UR);
        } else {
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                UL[v] = QL[v];
                UR[v] = QR[v];
            }
        }
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            const R u = R(0.5) * (UR[v] - UL[v]) * J;
            out[v] = u * n[0];
            out[5 + v] = u * n[1];
            out[10 + v] = u * n[2];
        }
        R* dL = a.UJ + offL * 15 + p;
        R* dR = a.UJ + offR * 15 + pr;
#pragma unroll
        for (int c = 0; c < 15; ++c) {
            dL[c * np] = out[c];
            dR[c * np] = out[c];
        }
        return;
    }
    const PhysR<R> ph = a.ph[fd.w];
    R inv[5];
    if (V) {
        const R t1[3] = {a.ft1[3 * gpt], a.ft1[3 * gpt + 1], a.ft1[3 * gpt + 2]};
        const R t2[3] = {a.ft2[3 * gpt], a.ft2[3 * gpt + 1], a.ft2[3 * gpt + 2]};
        riemann_flux(ph, QL, QR, n, t1, t2, inv);
    } else if (ph.riemann == 0) {
        roe_flux(ph, QL, QR, n, inv);
    } else if (ph.riemann == 3) {
        rusanov_flux(ph, QL, QR, n, inv);
    } else {  // LxF, central, u-diss
        const R t1[3] = {a.ft1[3 * gpt], a.ft1[3 * gpt + 1], a.ft1[3 * gpt + 2]};
        const R t2[3] = {a.ft2[3 * gpt], a.ft2[3 * gpt + 1], a.ft2[3 * gpt + 2]};
        lxf_flux<R, false>(ph, QL, QR, n, t1, t2, inv);
    }
    R visc[5] = {0, 0, 0, 0, 0};
    if (MODE == kFluxNS && boundary) {  // the interior viscous flux through the Neumann rule
        R gl[15];
#pragma unroll
        for (int c = 0; c < 15; ++c) gl[c] = a.GF[offL * 15 + c * np + p];
        R mu, kap, FL[3][5];
        mu_kappa(ph, QL, mu, kap);
        viscous_flux(ph, QL, gl, gl + 5, gl + 10, mu, kap, FL);
#pragma unroll
        for (int v = 0; v < 5; ++v) visc[v] = FL[0][v] * n[0] + FL[1][v] * n[1] + FL[2][v] * n[2];
        bc_neumann(a.bc[static_cast<unsigned>(fd.z) >> 20], QL, visc);
    } else if (MODE == kFluxNS) {
        R gl[15], gr[15];
#pragma unroll
        for (int c = 0; c < 15; ++c) {
            gl[c] = a.GF[offL * 15 + c * np + p];
            gr[c] = a.GF[offR * 15 + c * np + pr];
        }
        R mu, kap, FL[3][5], FR[3][5];
        mu_kappa(ph, QL, mu, kap);
        viscous_flux(ph, QL, gl, gl + 5, gl + 10, mu, kap, FL);
        mu_kappa(ph, QR, mu, kap);
        viscous_flux(ph, QR, gr, gr + 5, gr + 10, mu, kap, FR);
#pragma unroll
        for (int v = 0; v < 5; ++v)
            visc[v] = R(0.5) * (FL[0][v] + FR[0][v]) * n[0] + R(0.5) * (FL[1][v] + FR[1][v]) * n[1] +
                      R(0.5) * (FL[2][v] + FR[2][v]) * n[2];
    }
    R* dL = a.FS + offL * 5 + p;
    R* dR = a.FS + offR * 5 + pr;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
        const R fl = (inv[v] - visc[v]) * J;
        dL[v * np] = fl;
        if (!boundary) dR[v * np] = -fl;
    }
}

// Shared memory of kv_update: the operators, sQ (5 R per node: the new Q for the traces) and, for
// items of up to kStageNodes nodes, the updated G and Q (5 doubles per node each, stored back as flat
// arrays) and the elements' value offsets. Larger items store G and Q per node: their staging space
// would cut the resident blocks below the six that the kernel's 40 registers allow, and the kernel
// is bound by the latency of its loads.
constexpr int kStageNodes = 256;
__host__ __device__ constexpr bool vupdate_staged(int cap) { return cap <= kStageNodes; }
template <typename R>
__host__ __device__ constexpr size_t vupdate_stage_offset(int cap) {
    return (3 * sizeof(OpsP<R>) + static_cast<size_t>(5) * cap * sizeof(R) + 15) / 16 * 16;
}

// Elements of an item: each has at least 8 nodes (P >= 2 per direction), so at most cap/8 + 1.
__host__ __device__ constexpr int vupdate_max_elems(int cap) { return cap / 8 + 1; }

template <typename R>
size_t vupdate_smem(int cap) {
    if (!vupdate_staged(cap)) return 3 * sizeof(OpsP<R>) + static_cast<size_t>(5) * cap * sizeof(R);
    return vupdate_stage_offset<R>(cap) + static_cast<size_t>(10) * cap * sizeof(double) +
           static_cast<size_t>(vupdate_max_elems(cap)) * sizeof(long long);
}

// Flat store of the item's element blocks (W values per element, element le's block at global value
// index base[le]) from shared memory: consecutive lanes write consecutive values. inv_w = 1/W as a
// float gives the exact element of every index (f + 0.5 stays at least 0.5/W from a multiple of W).
__device__ __forceinline__ void vupdate_store(const double* shared, double* global, const long long* base, int W, int n,
                                              float inv_w) {
    for (int f = threadIdx.x; f < n; f += blockDim.x) {
        const int le = static_cast<int>((static_cast<float>(f) + 0.5f) * inv_w);
        global[base[le] + (f - le * W)] = shared[f];
    }
}

// ------------------------------------------------------------------------------------------------
// kv_update: surface integral, 1/J, source, RK3 stage update (per-case dt), traces of the new Q.
// SRC adds the manufactured source, PST the static-pressure residual of the mixed form; both are
// compile-time so that the common kernel carries neither (40 registers instead of 48). FP32 <-> FP64
// conversions use the integer pipe (bit-exact with the hardware conversion, which runs on the FP64
// pipe beside the update's FP64 multiply-adds).
// ------------------------------------------------------------------------------------------------
template <typename R, int PC, bool SRC, bool PST>
__global__ void __launch_bounds__(256, sizeof(R) == 4 && !SRC && !PST ? 6 : 0)
    kv_update(VArgs<R> a, int stage, double tshift, int write_qdot, int cap) {
    extern __shared__ __align__(16) unsigned char vsm[];
    const ItemDims d = item_dims<PC>(a.items[a.item0 + blockIdx.x]);
    const int px = d.px, py = d.py, np = d.np, ntot = d.ntot;
    OpsP<R>* sO = reinterpret_cast<OpsP<R>*>(vsm);
    R* sQ = reinterpret_cast<R*>(sO + 3);
    const bool staged = vupdate_staged(cap);
    double* sG = reinterpret_cast<double*>(vsm + vupdate_stage_offset<R>(cap));
    double* sQd = sG + 5 * cap;
    long long* sE = reinterpret_cast<long long*>(sQd + 5 * cap);
    // the operators in shared memory serve the traces at the end (after the barrier there); the
    // surface integral reads its six weights through the cache, so no barrier precedes the node loads
    load_ops(a.ops, sO, px, py, d.pz);
    const CaseConst cc = a.cc[d.kase];
    const double dt = stage >= 0 ? a.dt[d.kase] : 0.0;
    const double ak = stage == 0 ? 0.0 : (stage == 1 ? -5.0 / 9.0 : -153.0 / 128.0);
    const double ck = stage == 0 ? 1.0 / 3.0 : (stage == 1 ? 15.0 / 16.0 : 8.0 / 15.0);
    const int A = px * d.pz, B = px * py, C = py * d.pz;
    const NodeDecoder<PC> nd(d);
    for (int t = threadIdx.x; t < ntot; t += blockDim.x) {
        int le, n, i, j, k;
        nd.elem(t, le, n);
        nd.ijk(n, i, j, k);
        const int e = a.item_elems[d.first + le];
        const long long g = a.eoff[e] + n;
        const long long s0 = 6LL * e;
        const R* FF = a.FS + a.soff[s0 + 0] * 5 + (i + px * k);
        const R* FB = a.FS + a.soff[s0 + 1] * 5 + (i + px * k);
        const R* FO = a.FS + a.soff[s0 + 2] * 5 + (i + px * j);
        const R* FR = a.FS + a.soff[s0 + 3] * 5 + (j + py * k);
        const R* FT = a.FS + a.soff[s0 + 4] * 5 + (i + px * j);
        const R* FL = a.FS + a.soff[s0 + 5] * 5 + (j + py * k);
        const R bxl = __ldg(&a.ops[px].bL[i]), bxr = __ldg(&a.ops[px].bR[i]);
        const R byl = __ldg(&a.ops[py].bL[j]), byr = __ldg(&a.ops[py].bR[j]);
        const R bzl = __ldg(&a.ops[d.pz].bL[k]), bzr = __ldg(&a.ops[d.pz].bR[k]);
        const R J = a.jac[g];
        R qd[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            R fi = FL[v * C] * bxl;
            fi = fi + FR[v * C] * bxr;
            fi = fi + FF[v * A] * byl;
            fi = fi + FB[v * A] * byr;
            fi = fi + FO[v * B] * bzl;
            fi = fi + FT[v * B] * bzr;
            qd[v] = (a.QDot[5 * g + v] - fi) / J;
        }
        if (SRC) {
            double S[5];
            const double tt = a.time[d.kase] + tshift * dt;
            manufactured_source(a.source, a.x[3 * g], a.x[3 * g + 1], a.x[3 * g + 2], tt, cc.gm1, cc.gM2, cc.mu,
                                cc.kappa, S);
#pragma unroll
            for (int v = 0; v < 5; ++v) qd[v] = from_f64<R>(widen(qd[v]) + S[v]);
        }
        if (PST) {
            const double pr = cc.gm1 * cc.e_ref;  // the pressure the momentum fluxes leave out
#pragma unroll
            for (int c = 0; c < 3; ++c) qd[1 + c] = from_f64<R>(widen(qd[1 + c]) + pr * a.pstat[3 * g + c]);
        }
        if (write_qdot) {
#pragma unroll
            for (int v = 0; v < 5; ++v) a.QDot[5 * g + v] = qd[v];
        }
        if (stage >= 0) {
            const double cdt = ck * dt;
            double qq[5];
#pragma unroll
            for (int v = 0; v < 5; ++v) {
                const double gq = ak * a.G[5 * g + v] + widen(qd[v]);
                qq[v] = a.Q[5 * g + v] + cdt * gq;
                if (staged) {
                    sG[5 * t + v] = gq;
                    sQd[5 * t + v] = qq[v];
                } else {
                    a.G[5 * g + v] = gq;
                    a.Q[5 * g + v] = qq[v];
                }
            }
            if (staged && n == 0) sE[le] = 5 * g;
#pragma unroll
            for (int v = 0; v < 4; ++v) sQ[v * ntot + t] = from_f64<R>(qq[v]);
            sQ[4 * ntot + t] = from_f64<R>(qq[4] - cc.e_ref);
        }
    }
    if (stage < 0) return;
    __syncthreads();
    if (staged) {
        const int W = 5 * np;
        const float inv_w = 1.0f / static_cast<float>(W);
        vupdate_store(sG, a.G, sE, W, 5 * ntot, inv_w);
        vupdate_store(sQd, a.Q, sE, W, 5 * ntot, inv_w);
    }
    write_traces<R, 5, PC>(a, d, sO, sQ, a.QF);
}

// ------------------------------------------------------------------------------------------------
// Per-case reductions: CFL time step (MaxTimeStep with per-direction node spacing, DGSEMClass.f90:
// 870-1038) and residuals (ComputeMaxResiduals / checkForNan). red holds 8 words per case:
// [0] convective dt, [1] viscous dt, [2..6] max |QDot| per variable (bit images).
// ------------------------------------------------------------------------------------------------
struct VDtArgs {
    const int4* items;
    const int* item_elems;
    const long long* eoff;
    const double* Q;
    const double* dxi;       // [kMaxP + 1]: 1/|x_1 - x_0| of the node set with P nodes
    const double* gamma_M2;  // per case: gamma M^2
    double cfl, dcfl, gamma, gm1, S_div_TRef, TReNorm;
    int ns;
    unsigned long long* red;
};

// Two-pass MaxTimeStep per case (the FP32 filter and exact FP64 pass of k_dt_estimate/k_dt_exact),
// with the node spacing of each item's own orders. exact = 0: FP32 estimates into red[8c+7];
// exact = 1: exact FP64 limits of the nodes inside the window into red[8c], red[8c+1].
template <typename R>
__global__ void __launch_bounds__(256) kv_dt_pass(VDtArgs v, const R* ja_xi, const R* ja_eta, const R* ja_zeta,
                                                  const R* jac, int exact) {
    const ItemDims it = item_dims(v.items[blockIdx.x]);
    const double dx[3] = {v.dxi[it.px], v.dxi[it.py], v.dxi[it.pz]};
    const double dx2[3] = {dx[0] * dx[0], dx[1] * dx[1], dx[2] * dx[2]};
    const double gM2 = v.gamma_M2[it.kase];
    const DtConst32 c = dt_const32(v.cfl, v.dcfl, dx, v.gamma, v.gm1, gM2, v.S_div_TRef, v.TReNorm, v.ns);
    unsigned long long* red = v.red + 8 * it.kase;
    if (!exact) {
        float conv = 3.0e38f, visc = 3.0e38f;
        for (int t = threadIdx.x; t < it.ntot; t += blockDim.x) {
            const int le = t / it.np, n = t - le * it.np;
            const long long g = v.eoff[v.item_elems[it.first + le]] + n;
            float cv, vs;
            dt_estimate(c, v.Q + 5 * g, ja_xi + 3 * g, ja_eta + 3 * g, ja_zeta + 3 * g, jac[g], cv, vs);
            conv = fminf(conv, cv);
            visc = fminf(visc, vs);
        }
        float bc, bv;
        block_min2(conv, visc, &bc, &bv);
        if (threadIdx.x == 0) {
            unsigned int* s32 = reinterpret_cast<unsigned int*>(red + 7);
            atomicMin(&s32[0], fbits(bc));
            atomicMin(&s32[1], fbits(bv));
        }
        return;
    }
    DtArgs d;
    d.cfl = v.cfl;
    d.dcfl = v.dcfl;
    d.gamma = v.gamma;
    d.gm1 = v.gm1;
    d.S_div_TRef = v.S_div_TRef;
    d.TReNorm = v.TReNorm;
    d.ns = v.ns;
    const unsigned int* s32 = reinterpret_cast<const unsigned int*>(red + 7);
    const float thr_c = __uint_as_float(s32[0]) * (1.0f + kDtWindow);
    const float thr_v = __uint_as_float(s32[1]) * (1.0f + kDtWindow);
    double conv = 1.0e300, visc = 1.0e300;
    for (int t = threadIdx.x; t < it.ntot; t += blockDim.x) {
        const int le = t / it.np, n = t - le * it.np;
        const long long g = v.eoff[v.item_elems[it.first + le]] + n;
        const double* Q = v.Q + 5 * g;
        float cv, vs;
        dt_estimate(c, Q, ja_xi + 3 * g, ja_eta + 3 * g, ja_zeta + 3 * g, jac[g], cv, vs);
        const bool wc = !(cv > thr_c), wv = v.ns && !(vs > thr_v);
        if (wc || wv) {
            double ec = 1.0e300, ev = 1.0e300;
            dt_exact(d, dx, dx2, Q, ja_xi + 3 * g, ja_eta + 3 * g, ja_zeta + 3 * g, jac[g], gM2, wc, wv, ec, ev);
            conv = fmin(conv, ec);
            visc = fmin(visc, ev);
        }
    }
    double bc, bv;
    block_min2(conv, visc, &bc, &bv);
    if (threadIdx.x == 0) {
        atomicMin(&red[0], dbits(bc));
        atomicMin(&red[1], dbits(bv));
    }
}

// dt of every case = min(convective, viscous); resets the dt slots.
static __global__ void kv_dt_final(unsigned long long* red, double* dt, int n_cases) {
    for (int c = threadIdx.x; c < n_cases; c += blockDim.x) {
        const double conv = __longlong_as_double(static_cast<long long>(red[8 * c]));
        const double visc = __longlong_as_double(static_cast<long long>(red[8 * c + 1]));
        dt[c] = conv < visc ? conv : visc;
        red[8 * c] = dbits(1.0e300);
        red[8 * c + 1] = dbits(1.0e300);
        red[8 * c + 7] = kDtEstimateInit;
    }
}

static __global__ void kv_advance_time(double* t, const double* dt, int n_cases) {
    for (int c = threadIdx.x; c < n_cases; c += blockDim.x) t[c] = t[c] + dt[c];
}

template <typename R>
__global__ void __launch_bounds__(256) kv_residuals(const int4* items, const int* item_elems, const long long* eoff,
                                                    const R* qdot, const double* Q, unsigned long long* red,
                                                    int* nan_flag) {
    const ItemDims it = item_dims(items[blockIdx.x]);
    unsigned long long m[5] = {0, 0, 0, 0, 0};  // bit patterns, as k_residuals
    int bad = 0;
    for (int t = threadIdx.x; t < it.ntot; t += blockDim.x) {
        const int le = t / it.np, n = t - le * it.np;
        const long long g = eoff[item_elems[it.first + le]] + n;
#pragma unroll
        for (int v = 0; v < 5; ++v) {
            const unsigned long long a = abs_bits(qdot[5 * g + v]);
            m[v] = a > m[v] ? a : m[v];
            bad |= nonfinite(Q[5 * g + v]);
        }
    }
#pragma unroll
    for (int v = 0; v < 5; ++v)
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long x = __shfl_down_sync(0xffffffffu, m[v], o);
            m[v] = x > m[v] ? x : m[v];
        }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int v = 0; v < 5; ++v) atomicMax(&red[8 * it.kase + 2 + v], abs_bits_as_double(m[v], qdot));
    }
    if (bad) atomicOr(&nan_flag[it.kase], 1);
}

// ------------------------------------------------------------------------------------------------
// Launch wrappers
// ------------------------------------------------------------------------------------------------
template <typename R>
size_t vitem_smem(int cap, int nv) {
    return 3 * sizeof(OpsP<R>) + static_cast<size_t>(nv) * cap * sizeof(R);
}

struct Lanes;
template <typename R>
using VStageFn = cudaError_t (*)(const VArgs<R>& a, int stage, double tshift, int flags, cudaStream_t s,
                                  const Lanes* lanes);

template <typename R>
using VTimesFn = cudaError_t (*)(const VArgs<R>& a, int reps, cudaStream_t s, double* ms);

// Side streams for the independent launches of one phase (the item classes of a kernel, the two
// face lists, and for the Euler equations the face fluxes beside the volume kernels), so that their
// tails and latency-bound stretches overlap. A Fork records an event on the stage's stream when it
// opens; a side stream joins at its first launch by waiting on that event, and join() makes the
// stage's stream wait for every side stream used. Inside a stream capture the side streams become
// branches of the graph. Without lanes every launch goes to the stage's stream in order.
constexpr int kLanes = 3;
struct Lanes {
    int n = 0;
    cudaStream_t side[kLanes] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t done[kLanes] = {};
};

class Fork {
  public:
    Fork(const Lanes* l, cudaStream_t s) : l_(l && l->n > 0 ? l : nullptr), s_(s) {
        if (l_) note(cudaEventRecord(l_->fork, s_));
    }
    explicit Fork(cudaStream_t s) : l_(nullptr), s_(s) {}
    // The stream of the next independent launch (round robin over the stage's stream and the lanes).
    cudaStream_t next() {
        if (!l_) return s_;
        const int k = turn_++ % (l_->n + 1);
        if (k == 0) return s_;
        if (!(used_ & (1u << k))) {
            note(cudaStreamWaitEvent(l_->side[k - 1], l_->fork, 0));
            used_ |= 1u << k;
        }
        return l_->side[k - 1];
    }
    // The stage's stream waits for the lanes used since the fork; the first error of the fork.
    cudaError_t join() {
        if (l_) {
            for (int k = 1; k <= l_->n; ++k) {
                if (!(used_ & (1u << k))) continue;
                note(cudaEventRecord(l_->done[k - 1], l_->side[k - 1]));
                note(cudaStreamWaitEvent(s_, l_->done[k - 1], 0));
            }
            used_ = 0;
        }
        return err_;
    }
    void note(cudaError_t e) {
        if (err_ == cudaSuccess) err_ = e;
    }
    cudaError_t error() const { return err_; }

  private:
    const Lanes* l_;
    cudaStream_t s_;
    int turn_ = 0;
    unsigned used_ = 0;
    cudaError_t err_ = cudaSuccess;
};

// Lanes of a context: kLanes non-blocking side streams and their events (n = 0 if any creation failed).
inline cudaError_t create_lanes(Lanes& l) {
    cudaError_t e = cudaEventCreateWithFlags(&l.fork, cudaEventDisableTiming);
    for (int k = 0; k < kLanes && e == cudaSuccess; ++k) {
        e = cudaStreamCreateWithFlags(&l.side[k], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&l.done[k], cudaEventDisableTiming);
    }
    l.n = e == cudaSuccess ? kLanes : 0;
    return e;
}
inline void destroy_lanes(Lanes& l) {
    for (int k = 0; k < kLanes; ++k) {
        if (l.side[k]) cudaStreamDestroy(l.side[k]);
        if (l.done[k]) cudaEventDestroy(l.done[k]);
        l.side[k] = nullptr;
        l.done[k] = nullptr;
    }
    if (l.fork) cudaEventDestroy(l.fork);
    l.fork = nullptr;
    l.n = 0;
}

template <typename R, int MODE, int V>
cudaError_t launch_face_variant(const VArgs<R>& a, Fork& f) {
    using Cfg = FaceCfg<R, MODE>;
    if (a.n_nc > 0) {
        const int blocks = (a.n_nc + Cfg::FPB - 1) / Cfg::FPB;
        kv_face<R, MODE, V><<<blocks, Cfg::THREADS, Cfg::SMEM, f.next()>>>(a);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    const int npts = a.gp0[a.n_groups];
    if (npts > 0) {
        kv_face_direct<R, MODE, V><<<(npts + 127) / 128, 128, 0, f.next()>>>(a);
        return cudaGetLastError();
    }
    return cudaSuccess;
}

template <typename R, int MODE>
cudaError_t launch_face(const VArgs<R>& a, Fork& f) {
    const bool v = MODE == kJump ? a.grad_vars != 0 : ((a.riemann >= 4 && a.riemann <= 8) || a.averaging >= 5);
    return v ? launch_face_variant<R, MODE, 1>(a, f) : launch_face_variant<R, MODE, 0>(a, f);
}
template <typename R, int MODE>
cudaError_t launch_face(const VArgs<R>& a, cudaStream_t s) {
    Fork f(s);
    return launch_face<R, MODE>(a, f);
}

// Item kernels of one class: 0 traces, 1 volume, 2 update, 3 update with the manufactured source.
// Description of the last item launch that failed (kernel, class, grid, shared memory), for the
// error text of the entry point.
inline char* failed_launch() {
    static thread_local char buf[160] = "";
    return buf;
}

template <typename R, int PC>
cudaError_t launch_item_class(const VArgs<R>& a, int which, int n, size_t smem, cudaStream_t s, int store_grad,
                              int stage, double tshift, int wq, int cap) {
    switch (which) {
        case 0: kv_traces<R, PC><<<n, 256, smem, s>>>(a); break;
        case 1: kv_volume<R, PC><<<n, 256, smem, s>>>(a, store_grad); break;
        // the update kernel is bound by its memory traffic; compile-time orders only lengthen it
        case 2:
            if (a.pstat) kv_update<R, 0, false, true><<<n, 256, smem, s>>>(a, stage, tshift, wq, cap);
            else kv_update<R, 0, false, false><<<n, 256, smem, s>>>(a, stage, tshift, wq, cap);
            break;
        default:
            if (a.pstat) kv_update<R, 0, true, true><<<n, 256, smem, s>>>(a, stage, tshift, wq, cap);
            else kv_update<R, 0, true, false><<<n, 256, smem, s>>>(a, stage, tshift, wq, cap);
            break;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        cudaFuncAttributes fa{};
        const void* fn = which == 0 ? reinterpret_cast<const void*>(kv_traces<R, PC>)
                         : which == 1 ? reinterpret_cast<const void*>(kv_volume<R, PC>)
                         : which == 2 ? (a.pstat ? reinterpret_cast<const void*>(kv_update<R, 0, false, true>)
                                                 : reinterpret_cast<const void*>(kv_update<R, 0, false, false>))
                         : (a.pstat ? reinterpret_cast<const void*>(kv_update<R, 0, true, true>)
                                    : reinterpret_cast<const void*>(kv_update<R, 0, true, false>));
        cudaFuncGetAttributes(&fa, fn);
        snprintf(failed_launch(), 160, "item kernel %d class %d grid %d smem %zu (limit %d, static %zu, regs %d)", which,
                 PC, n, smem, fa.maxDynamicSharedSizeBytes, fa.sharedSizeBytes, fa.numRegs);
    }
    return e;
}

// One launch per non-empty item class (anisotropic items with runtime orders, isotropic items with
// compile-time P), each with the shared memory of its own largest item. which: 0 traces, 1 volume,
// 2 update, 3 update with the manufactured source.
template <typename R>
cudaError_t launch_items(const VArgs<R>& a0, int which, Fork& f, int store_grad = 0, int stage = 0,
                         double tshift = 0.0, int wq = 0) {
    for (int c = 0; c < kItemClasses; ++c) {
        const int n = a0.cls[c + 1] - a0.cls[c];
        if (n <= 0) continue;
        const cudaStream_t s = f.next();
        VArgs<R> a = a0;
        a.item0 = a0.cls[c];
        const int cap = a0.ccap[c];
        const size_t smem = which >= 2 ? vupdate_smem<R>(cap) : vitem_smem<R>(cap, which == 1 ? (a0.split ? 29 : 20) : 5);
        cudaError_t e;
        switch (c) {
            case 0: e = launch_item_class<R, 0>(a, which, n, smem, s, store_grad, stage, tshift, wq, cap); break;
            case 2: e = launch_item_class<R, 2>(a, which, n, smem, s, store_grad, stage, tshift, wq, cap); break;
            case 3: e = launch_item_class<R, 3>(a, which, n, smem, s, store_grad, stage, tshift, wq, cap); break;
            case 4: e = launch_item_class<R, 4>(a, which, n, smem, s, store_grad, stage, tshift, wq, cap); break;
            case 5: e = launch_item_class<R, 5>(a, which, n, smem, s, store_grad, stage, tshift, wq, cap); break;
            case 6: e = launch_item_class<R, 6>(a, which, n, smem, s, store_grad, stage, tshift, wq, cap); break;
            case 7: e = launch_item_class<R, 7>(a, which, n, smem, s, store_grad, stage, tshift, wq, cap); break;
            case 8: e = launch_item_class<R, 8>(a, which, n, smem, s, store_grad, stage, tshift, wq, cap); break;
            default: e = cudaErrorInvalidValue; break;  // no item has a single node per direction
        }
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

template <typename R>
cudaError_t launch_items(const VArgs<R>& a0, int which, cudaStream_t s, int store_grad = 0, int stage = 0,
                         double tshift = 0.0, int wq = 0) {
    Fork f(s);
    return launch_items(a0, which, f, store_grad, stage, tshift, wq);
}

template <typename R, int PC>
cudaError_t set_item_attributes(size_t vol, size_t upd, size_t trc) {
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(kv_volume<R, PC>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(vol))) ||
        (e = cudaFuncSetAttribute(kv_update<R, 0, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(upd))) ||
        (e = cudaFuncSetAttribute(kv_update<R, 0, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(upd))) ||
        (e = cudaFuncSetAttribute(kv_update<R, 0, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(upd))) ||
        (e = cudaFuncSetAttribute(kv_update<R, 0, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  static_cast<int>(upd))) ||
        (e = cudaFuncSetAttribute(kv_traces<R, PC>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(trc))))
        return e;
    return cudaSuccess;
}

// The update of a stage: one launch per item class (the manufactured-source variant where a case has
// a source).
template <typename R>
cudaError_t launch_update(const VArgs<R>& a, Fork& f, int stage, double tshift, int wq) {
    return launch_items(a, a.source ? 3 : 2, f, 0, stage, tshift, wq);
}

template <typename R>
cudaError_t vrun_stage(const VArgs<R>& a, int stage, double tshift, int flags, cudaStream_t s, const Lanes* lanes) {
    const size_t vol = vitem_smem<R>(a.cap, a.split ? 29 : 20), trc = vitem_smem<R>(a.cap, 5);
    const size_t upd = std::max(vupdate_smem<R>(a.cap), vupdate_smem<R>(std::min(a.cap, kStageNodes)));
    if (stage == kPrepare) {
        cudaError_t e;
        if ((e = set_item_attributes<R, 0>(vol, upd, trc)) || (e = set_item_attributes<R, 2>(vol, upd, trc)) ||
            (e = set_item_attributes<R, 3>(vol, upd, trc)) || (e = set_item_attributes<R, 4>(vol, upd, trc)) ||
            (e = set_item_attributes<R, 5>(vol, upd, trc)) || (e = set_item_attributes<R, 6>(vol, upd, trc)) ||
            (e = set_item_attributes<R, 7>(vol, upd, trc)) || (e = set_item_attributes<R, 8>(vol, upd, trc)) ||
            (e = cudaFuncSetAttribute(kv_face<R, kJump, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(FaceCfg<R, kJump>::SMEM))) ||
            (e = cudaFuncSetAttribute(kv_face<R, kJump, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(FaceCfg<R, kJump>::SMEM))) ||
            (e = cudaFuncSetAttribute(kv_face<R, kFluxEuler, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(FaceCfg<R, kFluxEuler>::SMEM))) ||
            (e = cudaFuncSetAttribute(kv_face<R, kFluxEuler, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(FaceCfg<R, kFluxEuler>::SMEM))) ||
            (e = cudaFuncSetAttribute(kv_face<R, kFluxNS, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(FaceCfg<R, kFluxNS>::SMEM))) ||
            (e = cudaFuncSetAttribute(kv_face<R, kFluxNS, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      static_cast<int>(FaceCfg<R, kFluxNS>::SMEM))))
            return e;
        return cudaSuccess;
    }
    // each phase forks and joins; a failed launch still joins its lanes before the error returns
    auto phase = [&](auto&& launches) -> cudaError_t {
        Fork f(lanes, s);
        f.note(launches(f));
        return f.join();
    };
    if (stage == kTraces) return phase([&](Fork& f) { return launch_items(a, 0, f); });
    cudaError_t e;
    if (a.ns) {
        // jumps -> volume (gradient traces) -> fluxes: three phases
        if ((e = phase([&](Fork& f) { return launch_face<R, kJump>(a, f); })) != cudaSuccess) return e;
        if ((e = phase([&](Fork& f) { return launch_items(a, 1, f, flags & kStoreGrad); })) != cudaSuccess) return e;
        if ((e = phase([&](Fork& f) { return launch_face<R, kFluxNS>(a, f); })) != cudaSuccess) return e;
    } else {
        // Euler: the face fluxes read only the Q traces, so they run beside the volume kernels
        e = phase([&](Fork& f) {
            const cudaError_t ef = launch_face<R, kFluxEuler>(a, f);
            return ef != cudaSuccess ? ef : launch_items(a, 1, f, flags & kStoreGrad);
        });
        if (e != cudaSuccess) return e;
    }
    const int wq = (flags & kWriteQDot) ? 1 : 0;
    return phase([&](Fork& f) { return launch_update(a, f, stage, tshift, wq); });
}

// Average device time of each kernel alone: ms[0] volume, [1] face flux, [2] update (stage 1),
// [3] traces, [4] BR1 jump faces.
template <typename R>
cudaError_t vkernel_times(const VArgs<R>& a, int reps, cudaStream_t s, double* ms) {
    cudaEvent_t e0, e1;
    cudaError_t err = cudaEventCreate(&e0);
    if (err != cudaSuccess) return err;
    if ((err = cudaEventCreate(&e1)) != cudaSuccess) {
        cudaEventDestroy(e0);
        return err;
    }
    for (int kk = 0; kk < 5; ++kk) {
        if (kk == 4 && !a.ns) {
            ms[kk] = 0.0;
            continue;
        }
        cudaEventRecord(e0, s);
        for (int r = 0; r < reps; ++r) {
            switch (kk) {
                case 0: launch_items(a, 1, s, 0); break;
                case 1: a.ns ? launch_face<R, kFluxNS>(a, s) : launch_face<R, kFluxEuler>(a, s); break;
                case 2: {
                    Fork f(s);
                    launch_update(a, f, 1, 1.0 / 3.0, 0);
                    break;
                }
                case 3: launch_items(a, 0, s); break;
                default: launch_face<R, kJump>(a, s); break;
            }
        }
        cudaEventRecord(e1, s);
        if ((err = cudaEventSynchronize(e1)) != cudaSuccess) break;
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        ms[kk] = reps > 0 ? t / reps : 0.0;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err != cudaSuccess) return err;
    return cudaGetLastError();
}

// Autotuner timing: reps launches of the volume and update (stage 1) kernels over the items of b;
// *ms receives the elapsed device time.
template <typename R>
cudaError_t vtime_items(const VArgs<R>& b, int reps, cudaStream_t s, float* ms) {
    cudaEvent_t e0, e1;
    cudaError_t err = cudaEventCreate(&e0);
    if (err != cudaSuccess) return err;
    if ((err = cudaEventCreate(&e1)) != cudaSuccess) {
        cudaEventDestroy(e0);
        return err;
    }
    cudaEventRecord(e0, s);
    for (int r = 0; r < reps && err == cudaSuccess; ++r) {
        err = launch_items(b, 1, s, 0);
        if (err == cudaSuccess) err = launch_items(b, 2, s, 0, 1, 1.0 / 3.0, 0);
    }
    cudaEventRecord(e1, s);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    if (err == cudaSuccess) err = cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return err;
}

template <typename R>
using VTuneFn = cudaError_t (*)(const VArgs<R>& b, int reps, cudaStream_t s, float* ms);

// Resolved in the instantiation translation units. The item and face kernels are launched only
// from there: a __global__ template instantiated in two translation units (without relocatable
// device code) registers two device functions under one host stub, so an attribute set through one
// would not reach the copy the other launches.
VTuneFn<double> vtune_fn_fp64();
VTuneFn<float> vtune_fn_fp32();
VStageFn<double> vstage_fn_fp64();
VStageFn<float> vstage_fn_fp32();
VTimesFn<double> vtimes_fn_fp64();
VTimesFn<float> vtimes_fn_fp32();

}  // namespace dg
