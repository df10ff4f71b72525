// Point-wise physics on the device: Euler and BR1 viscous fluxes, Sutherland viscosity, Roe and
// Lax-Friedrichs Riemann solvers, split-form two-point fluxes and the manufactured-solution source.
// Templated on the arithmetic type R (double for the plain form, float for the mixed form).
#pragma once
#include <cuda_runtime.h>

#include "horses3d_gb300.h"

namespace dg {

// Derived physics constants (PhysicsStorage_NS.f90:186-429), host-filled.
struct PhysConst {
    double gamma, gm1, gammaM2, mu, kappa, mu_to_kappa, S_div_TRef, TReNorm;
    double vns_kappa;  // conductivity of the viscous-NS Riemann solver, 1 / (3/4 (gamma-1) M^2)
    double lambda_stab;
    int ns, riemann, averaging, inviscid, source, grad_vars;
};

// The mixed form stores the energy relative to a constant reference E_ref (Q5' = E - E_ref, formed in
// FP64 before the conversion to FP32). Pressures are then p' = p - p_ref with p_ref = (gamma-1) E_ref,
// and total enthalpies add h_ref = E_ref + p_ref back. The constant p_ref is left out of the momentum
// fluxes: a constant flux has zero DG divergence on these metrics (free-stream preservation), while
// carrying it in FP32 would bury the O(1) pressure gradient under the O(1/(gamma M^2)) background.
// The plain FP64 form uses E_ref = p_ref = h_ref = 0, i.e. the reference's formulas unchanged.
template <typename R>
struct PhysR {
    R gamma, gm1, gammaM2, mu, kappa, mu_to_kappa, S_div_TRef, TReNorm, lambda_stab;
    R g_over_gm1, gp1_over_4, gm1_gammaM2;
    R gp1_over_2, gm1_over_2, inv_gamma, inv_gm1, gm1_over_2g, vns_kappa;
    R e_ref, p_ref, h_ref;
    int ns, riemann, averaging, grad_vars;
};

template <typename R>
PhysR<R> make_phys(const PhysConst& c) {
    PhysR<R> p;
    p.gamma = R(c.gamma); p.gm1 = R(c.gm1); p.gammaM2 = R(c.gammaM2); p.mu = R(c.mu); p.kappa = R(c.kappa);
    p.mu_to_kappa = R(c.mu_to_kappa); p.S_div_TRef = R(c.S_div_TRef); p.TReNorm = R(c.TReNorm);
    p.lambda_stab = R(c.lambda_stab);
    p.g_over_gm1 = R(c.gamma / (c.gamma - 1.0));
    p.gp1_over_4 = R((c.gamma + 1.0) / 4.0);
    p.gm1_gammaM2 = R(c.gm1 * c.gammaM2);
    // PhysicsStorage_NS.f90:115-133 (gammaPlus1Div2, gammaMinus1Div2, InvGamma, InvGammaMinus1,
    // gammaMinus1Div2g)
    p.gp1_over_2 = R((c.gamma + 1.0) / 2.0);
    p.gm1_over_2 = R(c.gm1 / 2.0);
    p.inv_gamma = R(1.0 / c.gamma);
    p.inv_gm1 = R(1.0 / c.gm1);
    p.gm1_over_2g = R(c.gm1 / (2.0 * c.gamma));
    p.vns_kappa = R(c.vns_kappa);
    p.e_ref = R(0); p.p_ref = R(0); p.h_ref = R(0);
    p.ns = c.ns; p.riemann = c.riemann; p.averaging = c.averaging; p.grad_vars = c.grad_vars;
    return p;
}

template <typename R>
void set_reference_energy(PhysR<R>& p, double gm1, double e_ref) {
    p.e_ref = R(e_ref);
    p.p_ref = R(gm1 * e_ref);
    p.h_ref = R(e_ref + gm1 * e_ref);
}

template <typename R> __device__ __forceinline__ R dsqrt(R x);
template <> __device__ __forceinline__ double dsqrt<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float dsqrt<float>(float x) { return sqrtf(x); }
template <typename R> __device__ __forceinline__ R dlog(R x);
template <> __device__ __forceinline__ double dlog<double>(double x) { return log(x); }
template <> __device__ __forceinline__ float dlog<float>(float x) { return logf(x); }

// Utilities.f90:269-301 logarithmicMean (Ismail and Roe): (aL - aR) / (ln aL - ln aR), with a
// series in ((xi - 1) / (xi + 1))^2 near xi = aL / aR = 1.
template <typename R>
__device__ __forceinline__ R log_mean(R aL, R aR) {
    const R xi = aL / aR;
    const R f = (xi - R(1)) / (xi + R(1));
    const R u = f * f;
    R FF;
    if (u < R(0.01)) FF = R(1) + (R(1) / R(3)) * u + (R(1) / R(5)) * (u * u) + (R(1) / R(7)) * ((u * u) * u);
    else FF = dlog(xi) / (R(2) * f);
    return R(0.5) * (aL + aR) / FF;
}

// VariableConversion_NS.f90:44-57,147-186: pressure, temperature, Sutherland's law.
template <typename R>
__device__ __forceinline__ void mu_kappa(const PhysR<R>& p, const R* Q, R& mu, R& kappa) {
    const R pr = p.gm1 * (Q[4] - R(0.5) * (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]) / Q[0]) + p.p_ref;
    const R T = p.gammaM2 * pr / Q[0];
    const R t = T * p.TReNorm;
    const R s = (R(1) + p.S_div_TRef) / (t + p.S_div_TRef) * t * dsqrt(t);
    mu = p.mu * s;
    kappa = mu * p.mu_to_kappa;
}

// Physics_NS.f90:51-103 EulerFlux contracted with the three metric vectors:
// F[d][v] = sum_c f_c(Q)[v] Ja^d_c (HyperbolicDiscretizationClass.f90:132-149).
template <typename R>
__device__ __forceinline__ void euler_contravariant(const PhysR<R>& p, const R* Q, const R* ja0, const R* ja1,
                                                    const R* ja2, R F[3][5]) {
    const R u = Q[1] / Q[0], v = Q[2] / Q[0], w = Q[3] / Q[0];
    const R pr = p.gm1 * (Q[4] - R(0.5) * (Q[1] * u + Q[2] * v + Q[3] * w));
    const R H = Q[4] + pr + p.h_ref;  // rho * total enthalpy
    const R f[5] = {Q[1], Q[1] * u + pr, Q[1] * v, Q[1] * w, H * u};
    const R g[5] = {Q[2], f[2], Q[2] * v + pr, Q[2] * w, H * v};
    const R h[5] = {Q[3], f[3], g[3], Q[3] * w + pr, H * w};
    const R* ja[3] = {ja0, ja1, ja2};
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int q = 0; q < 5; ++q) F[d][q] = f[q] * ja[d][0] + g[q] * ja[d][1] + h[q] * ja[d][2];
}

// BR1's gradient variables U(Q) (VariableConversion_NS.f90:196-262): the state itself, the entropy
// variables or (rho, u, v, w, T). The entropy and energy variables take the absolute pressure.
template <typename R>
__device__ __forceinline__ void gradient_variables(const PhysR<R>& p, const R* Q, R* U) {
    if (p.grad_vars == 0) {
#pragma unroll
        for (int v = 0; v < 5; ++v) U[v] = Q[v];
        return;
    }
    const R irho = R(1) / Q[0];
    const R rV2 = (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]) * irho;
    const R pr = p.gm1 * (Q[4] - R(0.5) * rV2) + p.p_ref;
    if (p.grad_vars == 1) {
        const R ip = R(1) / pr;
        U[0] = (p.gamma - (dlog(pr) - p.gamma * dlog(Q[0]))) * p.inv_gm1 - R(0.5) * rV2 * ip;
        U[1] = Q[1] * ip;
        U[2] = Q[2] * ip;
        U[3] = Q[3] * ip;
        U[4] = -Q[0] * ip;
    } else {
        U[0] = Q[0];
        U[1] = Q[1] * irho;
        U[2] = Q[2] * irho;
        U[3] = Q[3] * irho;
        U[4] = p.gammaM2 * pr * irho;
    }
}

// Physics_NS.f90:246-414 ViscousFlux_STATE / _ENTROPY / _ENERGY (beta = 0): F[c][v] cartesian
// component c, from the gradients Ux, Uy, Uz of the gradient variables.
template <typename R>
__device__ __forceinline__ void viscous_flux(const PhysR<R>& p, const R* Q, const R* Ux, const R* Uy, const R* Uz,
                                             R mu, R kappa, R F[3][5]) {
    const R invRho = R(1) / Q[0];
    const R u = Q[1] * invRho, v = Q[2] * invRho, w = Q[3] * invRho;
    R ux[3], uy[3], uz[3];
    R nTx, nTy, nTz;
    if (p.grad_vars == 0) {
        const R ud[3] = {u * invRho, v * invRho, w * invRho};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            ux[c] = invRho * Ux[1 + c] - ud[c] * Ux[0];
            uy[c] = invRho * Uy[1 + c] - ud[c] * Uy[0];
            uz[c] = invRho * Uz[1 + c] - ud[c] * Uz[0];
        }
        const R g = p.gm1_gammaM2;
        const R e2 = (Q[4] + p.e_ref) * invRho * invRho;
        nTx = g * (invRho * Ux[4] - e2 * Ux[0] - u * ux[0] - v * ux[1] - w * ux[2]);
        nTy = g * (invRho * Uy[4] - e2 * Uy[0] - u * uy[0] - v * uy[1] - w * uy[2]);
        nTz = g * (invRho * Uz[4] - e2 * Uz[0] - u * uz[0] - v * uz[1] - w * uz[2]);
    } else if (p.grad_vars == 1) {
        const R pdr = p.gm1 * invRho * (Q[4] - R(0.5) * (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]) * invRho) +
                      p.p_ref * invRho;
        const R um[3] = {u, v, w};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            ux[c] = pdr * (Ux[1 + c] + um[c] * Ux[4]);
            uy[c] = pdr * (Uy[1 + c] + um[c] * Uy[4]);
            uz[c] = pdr * (Uz[1 + c] + um[c] * Uz[4]);
        }
        const R g = p.gammaM2 * (pdr * pdr);
        nTx = g * Ux[4];
        nTy = g * Uy[4];
        nTz = g * Uz[4];
    } else {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            ux[c] = Ux[1 + c];
            uy[c] = Uy[1 + c];
            uz[c] = Uz[1 + c];
        }
        nTx = Ux[4];
        nTy = Uy[4];
        nTz = Uz[4];
    }
    const R divV = ux[0] + uy[1] + uz[2];
    const R tt = R(2) / R(3) * divV;
    const R txx = mu * (R(2) * ux[0] - tt);
    const R txy = mu * (ux[1] + uy[0]);
    const R txz = mu * (ux[2] + uz[0]);
    const R tyy = mu * (R(2) * uy[1] - tt);
    const R tyz = mu * (uy[2] + uz[1]);
    const R tzz = mu * (R(2) * uz[2] - tt);
    F[0][0] = R(0); F[0][1] = txx; F[0][2] = txy; F[0][3] = txz;
    F[0][4] = txx * u + txy * v + txz * w + kappa * nTx;
    F[1][0] = R(0); F[1][1] = txy; F[1][2] = tyy; F[1][3] = tyz;
    F[1][4] = txy * u + tyy * v + tyz * w + kappa * nTy;
    F[2][0] = R(0); F[2][1] = txz; F[2][2] = tyz; F[2][3] = tzz;
    F[2][4] = txz * u + tyz * v + tzz * w + kappa * nTz;
}

// RiemannSolvers_NS.f90:1541-1655 RoeRiemannSolver (with its entropy fix): the upwind side's flux
// plus the one acoustic wave that can change sign, evaluated at the Roe-averaged state.
template <typename R>
__device__ __forceinline__ void roe_flux(const PhysR<R>& p, const R* QL, const R* QR, const R* n, R* flux) {
    const R gm1 = p.gamma - R(1);
    const R rL = QL[0], rR = QR[0];
    const R uL = QL[1] / rL, vL = QL[2] / rL, wL = QL[3] / rL;
    const R prL = gm1 * (QL[4] - R(0.5) / rL * (QL[1] * QL[1] + QL[2] * QL[2] + QL[3] * QL[3]));
    const R uR = QR[1] / rR, vR = QR[2] / rR, wR = QR[3] / rR;
    const R prR = gm1 * (QR[4] - R(0.5) / rR * (QR[1] * QR[1] + QR[2] * QR[2] + QR[3] * QR[3]));
    const R vnL = n[0] * uL + n[1] * vL + n[2] * wL;  // normal velocities
    const R vnR = n[0] * uR + n[1] * vR + n[2] * wR;
    const R HL = R(0.5) * (uL * uL + vL * vL + wL * wL) + p.g_over_gm1 * (prL + p.p_ref) / rL;  // total enthalpies
    const R HR = R(0.5) * (uR * uR + vR * vR + wR * wR) + p.g_over_gm1 * (prR + p.p_ref) / rR;
    // Roe average: weights sqrt(rho) / (sqrt(rhoL) + sqrt(rhoR)) in the form rhoL / (rhoL + sqrt(rhoL rhoR))
    const R r_avg = dsqrt(rL * rR);
    const R wgtL = rL / (rL + r_avg), wgtR = R(1) - wgtL;
    const R ua = wgtL * uL + wgtR * uR, va = wgtL * vL + wgtR * vR, wa = wgtL * wL + wgtR * wR;
    const R Ha = wgtL * HL + wgtR * HR;
    const R ca2 = gm1 * (Ha - R(0.5) * (ua * ua + va * va + wa * wa));
    const R ca = dsqrt(ca2);
    const R vna = ua * n[0] + va * n[1] + wa * n[2];
    if (vna >= R(0)) {  // left state upwind; the u - c wave
        const R amp = R(0.5) * ((prR - prL) / ca2 - (vnR - vnL) * r_avg / ca);
        const R lam = vna - ca;
        const R lam_neg = lam < R(0) ? lam : R(0);
        const R spread = (p.gp1_over_4 * ca / r_avg) * amp;  // entropy fix: the wave speeds' jump
        const R fix0 = -fabs(lam) - spread;
        const R fix = fix0 > R(0) ? fix0 : R(0);
        const R wave = amp * (lam_neg - R(0.5) * fix);
        const R mflux = rL * vnL;
        flux[0] = mflux + wave;
        flux[1] = mflux * uL + prL * n[0] + wave * (ua - ca * n[0]);
        flux[2] = mflux * vL + prL * n[1] + wave * (va - ca * n[1]);
        flux[3] = mflux * wL + prL * n[2] + wave * (wa - ca * n[2]);
        flux[4] = mflux * HL + wave * (Ha - vna * ca);
    } else {  // right state upwind; the u + c wave
        const R amp = R(0.5) * ((prR - prL) / ca2 + (vnR - vnL) * r_avg / ca);
        const R lam = vna + ca;
        const R lam_pos = lam > R(0) ? lam : R(0);
        const R spread = (p.gp1_over_4 * ca / r_avg) * amp;
        const R fix0 = -fabs(lam) + spread;
        const R fix = fix0 > R(0) ? fix0 : R(0);
        const R wave = amp * (lam_pos + R(0.5) * fix);
        const R mflux = rR * vnR;
        flux[0] = mflux - wave;
        flux[1] = mflux * uR + prR * n[0] - wave * (ua + ca * n[0]);
        flux[2] = mflux * vR + prR * n[1] - wave * (va + ca * n[1]);
        flux[3] = mflux * wR + prR * n[2] - wave * (wa + ca * n[2]);
        flux[4] = mflux * HR - wave * (Ha + vna * ca);
    }
}

// The Ismail-Roe (entropy conserving) and Chandrasekar mean states of two states: density,
// velocity, ABSOLUTE pressure and total enthalpy. The pressures pL, pR given are the absolute ones.
// EntropyConservingAverage (RiemannSolvers_NS.f90:1964-2026, z-sums; the two-point flux :2439-2558
// uses z-means, so `half` selects 1/2 zSum), ChandrasekarAverage (:2028-2077, :2560-2641).
template <typename R>
__device__ __forceinline__ void log_mean_state(const PhysR<R>& p, bool entropy_conserving, R rhoL, R rhoR, R uL, R uR,
                                               R vL, R vR, R wL, R wR, R pL, R pR, R& rho, R& u, R& v, R& w,
                                               R& pm, R& h, bool zmean) {
    if (entropy_conserving) {
        const R z5L = dsqrt(rhoL * pL), z5R = dsqrt(rhoR * pR);
        const R z1L = rhoL / z5L, z1R = rhoR / z5R;
        R s1, s2, s3, s4, s5;
        if (zmean) {
            s1 = R(0.5) * (z1L + z1R); s2 = R(0.5) * (z1L * uL + z1R * uR); s3 = R(0.5) * (z1L * vL + z1R * vR);
            s4 = R(0.5) * (z1L * wL + z1R * wR); s5 = R(0.5) * (z5L + z5R);
        } else {
            s1 = z1L + z1R; s2 = z1L * uL + z1R * uR; s3 = z1L * vL + z1R * vR; s4 = z1L * wL + z1R * wR;
            s5 = z5L + z5R;
        }
        const R inv1 = R(1) / s1;
        const R z1Log = log_mean(z1L, z1R), z5Log = log_mean(z5L, z5R);
        rho = zmean ? s1 * z5Log : R(0.5) * s1 * z5Log;
        u = s2 * inv1; v = s3 * inv1; w = s4 * inv1; pm = s5 * inv1;
        const R p2 = (p.gp1_over_2 * z5Log / z1Log + p.gm1_over_2 * pm) * p.inv_gamma;
        h = p.g_over_gm1 * p2 / rho + R(0.5) * (u * u + v * v + w * w);
    } else {
        const R betaL = R(0.5) * rhoL / pL, betaR = R(0.5) * rhoR / pR;
        const R betaLog = log_mean(betaL, betaR);
        rho = log_mean(rhoL, rhoR);
        u = R(0.5) * (uL + uR); v = R(0.5) * (vL + vR); w = R(0.5) * (wL + wR);
        pm = R(0.5) * (rhoL + rhoR) / (betaL + betaR);
        h = R(0.5) / (betaLog * p.gm1) - R(0.5) * (R(0.5) * ((uL * uL + vL * vL + wL * wL) + (uR * uR + vR * vR + wR * wR))) +
            pm / rho + u * u + v * v + w * w;
    }
}

// Averaged states of the face-normal frame (L, R = rho, rho u_n, rho u_t1, rho u_t2, E with the mixed
// form's E'): StandardAverage (RiemannSolvers_NS.f90:1784-1819), DucrosAverage (:1821-1848),
// MorinishiAverage (:1850-1886), KennedyGruberAverage (:1888-1925), PirozzoliAverage (:1927-1962),
// EntropyConservingAverage (:1964-2026), ChandrasekarAverage (:2028-2077).
// Absolute energies and pressures are E' + e_ref, p' + p_ref; momentum fluxes carry p' only.
// LM = false compiles the averages without the logarithmic means (callers that never see averages
// 5 and 6 keep a smaller register footprint).
template <typename R, bool LM = true>
__device__ __forceinline__ void averaged_states(const PhysR<R>& p, const R* L, const R* Rt, R pL, R pR, R iL, R iR,
                                                R* f) {
    const R uL = iL * L[1], uR = iR * Rt[1], vL = iL * L[2], vR = iR * Rt[2], wL = iL * L[3], wR = iR * Rt[3];
    switch (LM ? p.averaging : (p.averaging >= 5 ? 0 : p.averaging)) {
        case 5:
        case 6: {  // entropy conserving, Chandrasekar
            R rho, u, v, w, pm, h;
            log_mean_state(p, p.averaging == 5, L[0], Rt[0], uL, uR, vL, vR, wL, wR, pL + p.p_ref, pR + p.p_ref, rho,
                           u, v, w, pm, h, false);
            f[0] = rho * u;
            f[1] = rho * u * u + (pm - p.p_ref);
            f[2] = rho * u * v;
            f[3] = rho * u * w;
            f[4] = rho * u * h;
            break;
        }
        case 0: {  // standard
            f[0] = R(0.5) * (L[1] + Rt[1]);
            f[1] = R(0.5) * (L[1] * uL + Rt[1] * uR + pL + pR);
            f[2] = R(0.5) * (L[1] * vL + Rt[1] * vR);
            f[3] = R(0.5) * (L[1] * wL + Rt[1] * wR);
            f[4] = R(0.5) * (uL * (L[4] + pL + p.h_ref) + uR * (Rt[4] + pR + p.h_ref));
            break;
        }
        case 2: {  // Ducros
            const R su = uL + uR;
            f[0] = R(0.25) * (L[0] + Rt[0]) * su;
            f[1] = R(0.25) * (L[1] + Rt[1]) * su + R(0.5) * (pL + pR);
            f[2] = R(0.25) * (L[2] + Rt[2]) * su;
            f[3] = R(0.25) * (L[3] + Rt[3]) * su;
            f[4] = R(0.25) * (L[4] + pL + Rt[4] + pR + R(2) * p.h_ref) * su;
            break;
        }
        case 3: {  // Morinishi: the enthalpy without kinetic energy, cp p
            const R hL = p.g_over_gm1 * (pL + p.p_ref), hR = p.g_over_gm1 * (pR + p.p_ref);
            const R m = L[1] + Rt[1];
            f[0] = R(0.5) * m;
            f[1] = R(0.25) * m * (uL + uR) + R(0.5) * (pL + pR);
            f[2] = R(0.25) * m * (vL + vR);
            f[3] = R(0.25) * m * (wL + wR);
            f[4] = R(0.5) * (uL * hL + uR * hR) + R(0.25) * (L[1] * uL + Rt[1] * uR) * (uL + uR) +
                   R(0.25) * (L[1] * vL + Rt[1] * vR) * (vL + vR) + R(0.25) * (L[1] * wL + Rt[1] * wR) * (wL + wR) -
                   R(0.25) * (L[1] * uL * uL + Rt[1] * uR * uR) - R(0.25) * (L[1] * vL * vL + Rt[1] * vR * vR) -
                   R(0.25) * (L[1] * wL * wL + Rt[1] * wR * wR);
            break;
        }
        case 4: {  // Kennedy-Gruber
            const R rho = R(0.5) * (L[0] + Rt[0]), u = R(0.5) * (uL + uR), v = R(0.5) * (vL + vR);
            const R w = R(0.5) * (wL + wR), pp = R(0.5) * (pL + pR);
            const R e = R(0.5) * ((L[4] + p.e_ref) * iL + (Rt[4] + p.e_ref) * iR);
            f[0] = rho * u;
            f[1] = rho * u * u + pp;
            f[2] = rho * u * v;
            f[3] = rho * u * w;
            f[4] = rho * u * e + (pp + p.p_ref) * u;
            break;
        }
        default: {  // Pirozzoli
            const R rho = R(0.5) * (L[0] + Rt[0]), u = R(0.5) * (uL + uR), v = R(0.5) * (vL + vR);
            const R w = R(0.5) * (wL + wR), pp = R(0.5) * (pL + pR);
            const R h = R(0.5) * ((L[4] + pL + p.h_ref) * iL + (Rt[4] + pR + p.h_ref) * iR);
            f[0] = rho * u; f[1] = rho * u * u + pp; f[2] = rho * u * v; f[3] = rho * u * w; f[4] = rho * u * h;
            break;
        }
    }
}

// RiemannSolvers_NS.f90:1251-1334 LxFRiemannSolver (the averaging of the control file) and :375-428
// CentralRiemannSolver, which is the same average with lambda_stab = 0 (SetRiemannSolver, :224).
template <typename R, bool LM = true>
__device__ __forceinline__ void lxf_flux(const PhysR<R>& p, const R* QL, const R* QR, const R* n, const R* t1,
                                         const R* t2, R* flux) {
    const R iL = R(1) / QL[0], iR = R(1) / QR[0];
    const R ruL = QL[1] * n[0] + QL[2] * n[1] + QL[3] * n[2];
    const R ruR = QR[1] * n[0] + QR[2] * n[1] + QR[3] * n[2];
    const R rvL = QL[1] * t1[0] + QL[2] * t1[1] + QL[3] * t1[2];
    const R rvR = QR[1] * t1[0] + QR[2] * t1[1] + QR[3] * t1[2];
    const R rwL = QL[1] * t2[0] + QL[2] * t2[1] + QL[3] * t2[2];
    const R rwR = QR[1] * t2[0] + QR[2] * t2[1] + QR[3] * t2[2];
    const R pL = p.gm1 * (QL[4] - R(0.5) * ((ruL * ruL + rvL * rvL + rwL * rwL) * iL));
    const R pR = p.gm1 * (QR[4] - R(0.5) * ((ruR * ruR + rvR * rvR + rwR * rwR) * iR));
    const R Lr[5] = {QL[0], ruL, rvL, rwL, QL[4]};
    const R Rr[5] = {QR[0], ruR, rvR, rwR, QR[4]};
    R f[5];
    averaged_states<R, LM>(p, Lr, Rr, pL, pR, iL, iR, f);
    if (p.riemann != 2) {  // central fluxes carry no dissipation
        // u-diss (RiemannSolvers_NS.f90:1336-1425) drops the sound speeds
        const R aL = p.riemann == 9 ? R(0) : dsqrt(p.gamma * (pL + p.p_ref) * iL);
        const R aR = p.riemann == 9 ? R(0) : dsqrt(p.gamma * (pR + p.p_ref) * iR);
        const R lL = fabs(ruL * iL) + aL, lR = fabs(ruR * iR) + aR;
        const R lambda = lL > lR ? lL : lR;
        const R ls = p.lambda_stab * (R(0.5) * lambda);
        f[0] = f[0] - ls * (QR[0] - QL[0]);
        f[1] = f[1] - ls * (ruR - ruL);
        f[2] = f[2] - ls * (rvR - rvL);
        f[3] = f[3] - ls * (rwR - rwL);
        f[4] = f[4] - ls * (QR[4] - QL[4]);
    }
    flux[0] = f[0];
#pragma unroll
    for (int c = 0; c < 3; ++c) flux[1 + c] = n[c] * f[1] + t1[c] * f[2] + t2[c] * f[3];
    flux[4] = f[4];
}

// RiemannSolvers_NS.f90:1661-1762 RusanovRiemannSolver: the mean of the two normal fluxes minus
// max(|q| + a) times the jump, over two.
template <typename R>
__device__ __forceinline__ void rusanov_flux(const PhysR<R>& p, const R* QL, const R* QR, const R* n, R* flux) {
    const R gm1 = p.gamma - R(1);
    const R rL = QL[0], rR = QR[0];
    const R uL = QL[1] / rL, vL = QL[2] / rL, wL = QL[3] / rL;
    const R prL = gm1 * (QL[4] - R(0.5) / rL * (QL[1] * QL[1] + QL[2] * QL[2] + QL[3] * QL[3]));
    const R uR = QR[1] / rR, vR = QR[2] / rR, wR = QR[3] / rR;
    const R prR = gm1 * (QR[4] - R(0.5) / rR * (QR[1] * QR[1] + QR[2] * QR[2] + QR[3] * QR[3]));
    const R vnL = n[0] * uL + n[1] * vL + n[2] * wL;
    const R vnR = n[0] * uR + n[1] * vR + n[2] * wR;
    const R keL = R(0.5) * (uL * uL + vL * vL + wL * wL), keR = R(0.5) * (uR * uR + vR * vR + wR * wR);
    const R HL = keL + p.g_over_gm1 * (prL + p.p_ref) / rL;
    const R HR = keR + p.g_over_gm1 * (prR + p.p_ref) / rR;
    const R cR = dsqrt(gm1 * (HR - keR)), cL = dsqrt(gm1 * (HL - keL));
    const R mL = rL * vnL, mR = rR * vnR;  // normal mass fluxes
    R f[5];
    f[0] = mL + mR;
    f[1] = mL * uL + prL * n[0] + mR * uR + prR * n[0];
    f[2] = mL * vL + prL * n[1] + mR * vR + prR * n[1];
    f[3] = mL * wL + prL * n[2] + mR * wR + prR * n[2];
    f[4] = mL * HL + mR * HR;
    const R sR = cR + fabs(vnR), sL = cL + fabs(vnL);
    const R smax = sR > sL ? sR : sL;
#pragma unroll
    for (int v = 0; v < 5; ++v) flux[v] = (f[v] - smax * (QR[v] - QL[v])) / R(2);
}

template <typename R>
__device__ __forceinline__ void to_face_frame(const R* Q, const R* n, const R* t1, const R* t2, R* r) {
    r[0] = Q[0];
    r[1] = Q[1] * n[0] + Q[2] * n[1] + Q[3] * n[2];
    r[2] = Q[1] * t1[0] + Q[2] * t1[1] + Q[3] * t1[2];
    r[3] = Q[1] * t2[0] + Q[2] * t2[1] + Q[3] * t2[2];
    r[4] = Q[4];
}
template <typename R>
__device__ __forceinline__ void from_face_frame(const R* f, const R* n, const R* t1, const R* t2, R* flux) {
    flux[0] = f[0];
#pragma unroll
    for (int c = 0; c < 3; ++c) flux[1 + c] = n[c] * f[1] + t1[c] * f[2] + t2[c] * f[3];
    flux[4] = f[4];
}

// Van Leer's modification of Harten's entropy fix of an acoustic wave speed (RiemannSolvers_NS.f90:
// 507-530): sL, sR are the one-sided speeds u -/+ a.
template <typename R>
__device__ __forceinline__ R entropy_fix(R lambda, R sL, R sR) {
    const R d = sR - sL;
    const R dl = d > R(0) ? d : R(0);
    const R al = fabs(lambda);
    if (al >= R(2) * dl) return al;
    return lambda * lambda / (R(4) * dl) + dl;
}

// average - lambda_stab sum_i 1/2 alpha_i |lambda_i| K_i with the Roe eigenvectors K of (u, v, w, H, a)
// in the face frame; the Pirozzoli and Kennedy-Gruber averages take lambda_1 = lambda_5 (Winters et
// al., as the reference does).
template <typename R>
__device__ __forceinline__ void roe_stabilised(const PhysR<R>& p, const R* L, const R* Rt, R pL, R pR, R iL, R iR, R u,
                                               R v, R w, R V2, R H, R a, const R* alpha, R* lambda, R* f) {
    averaged_states(p, L, Rt, pL, pR, iL, iR, f);
    if (p.averaging == 1 || p.averaging == 4) lambda[0] = lambda[4];
    const R K[5][5] = {{R(1), u - a, v, w, H - u * a},
                       {R(1), u, v, w, R(0.5) * V2},
                       {R(0), R(0), R(1), R(0), v},
                       {R(0), R(0), R(0), R(1), w},
                       {R(1), u + a, v, w, H + u * a}};
    R stab[5] = {R(0), R(0), R(0), R(0), R(0)};
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const R c = R(0.5) * alpha[i] * fabs(lambda[i]);
#pragma unroll
        for (int q = 0; q < 5; ++q) stab[q] = stab[q] + c * K[i][q];
    }
#pragma unroll
    for (int q = 0; q < 5; ++q) f[q] = f[q] - p.lambda_stab * stab[q];
}

// StdRoeRiemannSolver (RiemannSolvers_NS.f90:430-576) and RoePikeRiemannSolver (:721-861): the chosen
// average plus the Roe dissipation with getRoeVariables' averages (VariableConversion_NS.f90:323-365);
// the wave strengths are the projections of the jump (standard) or of the primitive jumps (Roe-Pike).
template <typename R>
__device__ __forceinline__ void std_roe_flux(const PhysR<R>& p, bool pike, const R* QL, const R* QR, const R* n,
                                             const R* t1, const R* t2, R* flux) {
    R L[5], Rt[5];
    to_face_frame(QL, n, t1, t2, L);
    to_face_frame(QR, n, t1, t2, Rt);
    // getPrimitiveVariables (VariableConversion_NS.f90:266-294)
    const R iL = R(1) / L[0], iR = R(1) / Rt[0];
    const R uL = L[1] * iL, vL = L[2] * iL, wL = L[3] * iL, uR = Rt[1] * iR, vR = Rt[2] * iR, wR = Rt[3] * iR;
    const R pL = p.gm1 * (L[4] - R(0.5) * (uL * L[1] + vL * L[2] + wL * L[3]));
    const R pR = p.gm1 * (Rt[4] - R(0.5) * (uR * Rt[1] + vR * Rt[2] + wR * Rt[3]));
    const R aL = dsqrt(p.gamma * (pL + p.p_ref) * iL), aR = dsqrt(p.gamma * (pR + p.p_ref) * iR);
    const R sL = dsqrt(L[0]), sR = dsqrt(Rt[0]);
    const R inv = R(1) / (sL + sR);
    const R HL = (pL + L[4] + p.h_ref) * iL, HR = (pR + Rt[4] + p.h_ref) * iR;
    const R rho = sL * sR;
    const R u = (sL * uL + sR * uR) * inv, v = (sL * vL + sR * vR) * inv, w = (sL * wL + sR * wR) * inv;
    const R H = (sL * HL + sR * HR) * inv;
    const R V2 = u * u + v * v + w * w;
    const R a = dsqrt(p.gm1 * (H - R(0.5) * V2));
    R lambda[5] = {u - a, u, u, u, u + a};
    R alpha[5];
    if (!pike) {
        R dQ[5];
#pragma unroll
        for (int q = 0; q < 5; ++q) dQ[q] = Rt[q] - L[q];
        alpha[2] = dQ[2] - v * dQ[0];
        alpha[3] = dQ[3] - w * dQ[0];
        dQ[4] = dQ[4] - alpha[2] * v - alpha[3] * w;
        alpha[1] = p.gm1 * (dQ[0] * (H - u * u) + u * dQ[1] - dQ[4]) / (a * a);
        alpha[0] = R(0.5) * (dQ[0] * lambda[4] - dQ[1] - a * alpha[1]) / a;
        alpha[4] = dQ[0] - alpha[0] - alpha[1];
    } else {
        const R dp = pR - pL, du = uR - uL;
        alpha[0] = (dp - rho * a * du) / (R(2) * a * a);
        alpha[1] = (Rt[0] - L[0]) - dp / (a * a);
        alpha[2] = rho * (vR - vL);
        alpha[3] = rho * (wR - wL);
        alpha[4] = (dp + rho * a * du) / (R(2) * a * a);
    }
    lambda[0] = entropy_fix(lambda[0], uL - aL, uR - aR);
    lambda[4] = entropy_fix(lambda[4], uL + aL, uR + aR);
    R f[5];
    roe_stabilised(p, L, Rt, pL, pR, iL, iR, u, v, w, V2, H, a, alpha, lambda, f);
    from_face_frame(f, n, t1, t2, flux);
}

// Face-frame states and Roe-Pike averages written with 1/sqrt(rho), as LowDissipationRoeRiemannSolver
// (:863-1058) and ViscousNSRiemannSolver (:1060-1247) form them.
template <typename R>
struct RoePike {
    R L[5], Rt[5], iL, iR, uL, vL, wL, uR, vR, wR, pL, pR, aL, aR, rho, u, v, w, H, V2, a;
};
template <typename R>
__device__ __forceinline__ void roe_pike_state(const PhysR<R>& p, const R* QL, const R* QR, const R* n, const R* t1,
                                               const R* t2, RoePike<R>& s) {
    to_face_frame(QL, n, t1, t2, s.L);
    to_face_frame(QR, n, t1, t2, s.Rt);
    s.iL = R(1) / s.L[0]; s.iR = R(1) / s.Rt[0];
    const R sL = dsqrt(s.L[0]), sR = dsqrt(s.Rt[0]);
    const R isL = R(1) / sL, isR = R(1) / sR;
    const R inv = R(1) / (sL + sR);
    s.uL = s.L[1] * s.iL; s.uR = s.Rt[1] * s.iR;
    s.vL = s.L[2] * s.iL; s.vR = s.Rt[2] * s.iR;
    s.wL = s.L[3] * s.iL; s.wR = s.Rt[3] * s.iR;
    const R rV2L = (s.uL * s.uL + s.vL * s.vL + s.wL * s.wL) * s.L[0];
    const R rV2R = (s.uR * s.uR + s.vR * s.vR + s.wR * s.wR) * s.Rt[0];
    const R rHL = p.gamma * s.L[4] - R(0.5) * p.gm1 * rV2L + p.h_ref;
    const R rHR = p.gamma * s.Rt[4] - R(0.5) * p.gm1 * rV2R + p.h_ref;
    s.pL = p.gm1 * (s.L[4] - R(0.5) * rV2L);
    s.pR = p.gm1 * (s.Rt[4] - R(0.5) * rV2R);
    s.aL = dsqrt(p.gamma * (s.pL + p.p_ref) * s.iL);
    s.aR = dsqrt(p.gamma * (s.pR + p.p_ref) * s.iR);
    s.rho = sL * sR;
    s.u = (isL * s.L[1] + isR * s.Rt[1]) * inv;
    s.v = (isL * s.L[2] + isR * s.Rt[2]) * inv;
    s.w = (isL * s.L[3] + isR * s.Rt[3]) * inv;
    s.H = (isL * rHL + isR * rHR) * inv;
    s.V2 = s.u * s.u + s.v * s.v + s.w * s.w;
    s.a = dsqrt(p.gm1 * (s.H - R(0.5) * s.V2));
}

// LowDissipationRoeRiemannSolver (:863-1058): Roe-Pike wave strengths with the velocity jumps scaled
// by z = min(1, max(M_L, M_R)) (L2Roe).
template <typename R>
__device__ __forceinline__ void low_diss_roe_flux(const PhysR<R>& p, const R* QL, const R* QR, const R* n, const R* t1,
                                                  const R* t2, R* flux) {
    RoePike<R> s;
    roe_pike_state(p, QL, QR, n, t1, t2, s);
    const R u = s.u, a = s.a, rho = s.rho;
    R lambda[5] = {u - a, u, u, u, u + a};
    const R ML = fabs(s.uL) / s.aL, MR = fabs(s.uR) / s.aR;
    const R mx = ML > MR ? ML : MR;
    const R z = mx < R(1) ? mx : R(1);
    const R du = z * (s.uR - s.uL), dv = z * (s.vR - s.vL), dw = z * (s.wR - s.wL), dp = s.pR - s.pL;
    R alpha[5];
    alpha[0] = (dp - rho * a * du) / (R(2) * a * a);
    alpha[1] = (s.Rt[0] - s.L[0]) - dp / (a * a);
    alpha[2] = rho * dv;
    alpha[3] = rho * dw;
    alpha[4] = (dp + rho * a * du) / (R(2) * a * a);
    lambda[0] = entropy_fix(lambda[0], s.uL - s.aL, s.uR - s.aR);
    lambda[4] = entropy_fix(lambda[4], s.uL + s.aL, s.uR + s.aR);
    R f[5];
    roe_stabilised(p, s.L, s.Rt, s.pL, s.pR, s.iL, s.iR, s.u, s.v, s.w, s.V2, s.H, a, alpha, lambda, f);
    from_face_frame(f, n, t1, t2, flux);
}

// ViscousNSRiemannSolver (:1060-1247): the average plus a dissipation shaped like the NS viscous
// terms of the velocity and temperature jumps, times the largest wave speed, added in the
// Cartesian frame (conductivity with Pr = 3/4, FluidData_NS.f90:173-181).
template <typename R>
__device__ __forceinline__ void viscous_ns_flux(const PhysR<R>& p, const R* QL, const R* QR, const R* n, const R* t1,
                                                const R* t2, R* flux) {
    RoePike<R> s;
    roe_pike_state(p, QL, QR, n, t1, t2, s);
    R lambda[5] = {s.u - s.a, s.u, s.u, s.u, s.u + s.a};
    lambda[0] = entropy_fix(lambda[0], s.uL - s.aL, s.uR - s.aR);
    lambda[4] = entropy_fix(lambda[4], s.uL + s.aL, s.uR + s.aR);
    R f[5];
    averaged_states(p, s.L, s.Rt, s.pL, s.pR, s.iL, s.iR, f);
    if (p.averaging == 1 || p.averaging == 4) lambda[0] = lambda[4];
    const R uL = QL[1] / QL[0], uR = QR[1] / QR[0];
    const R vL = QL[2] / QL[0], vR = QR[2] / QR[0];
    const R wL = QL[3] / QL[0], wR = QR[3] / QR[0];
    const R u = R(0.5) * (uL + uR), v = R(0.5) * (vL + vR), w = R(0.5) * (wL + wR);
    const R du = uR - uL, dv = vR - vL, dw = wR - wL;
    const R divV = du * n[0] + dv * n[1] + dw * n[2];
    const R third = R(1) / R(3);
    const R t11 = R(2) * du * n[0] - third * divV;
    const R t22 = R(2) * dv * n[1] - third * divV;
    const R t33 = R(2) * dw * n[2] - third * divV;
    const R t12 = du * n[1] + dv * n[0];
    const R t13 = du * n[2] + dw * n[0];
    const R t23 = dv * n[2] + dw * n[1];
    const R TL = (s.pL + p.p_ref) * p.gammaM2 / s.L[0], TR = (s.pR + p.p_ref) * p.gammaM2 / s.Rt[0];
    R lmax = R(0);
#pragma unroll
    for (int i = 0; i < 5; ++i) lmax = fabs(lambda[i]) > lmax ? fabs(lambda[i]) : lmax;
    from_face_frame(f, n, t1, t2, flux);
    R stab[5];
    stab[0] = R(0);
    stab[1] = lmax * (t11 * n[0] + t12 * n[1] + t13 * n[2]);
    stab[2] = lmax * (t12 * n[0] + t22 * n[1] + t23 * n[2]);
    stab[3] = lmax * (t13 * n[0] + t23 * n[1] + t33 * n[2]);
    stab[4] = lmax * ((u * t11 + v * t12 + w * t13) * n[0] + (u * t12 + v * t22 + w * t23) * n[1] +
                      (u * t13 + v * t23 + w * t33) * n[2] + p.vns_kappa * (TR - TL));
#pragma unroll
    for (int q = 0; q < 5; ++q) flux[q] = flux[q] - p.lambda_stab * stab[q];
}

// NSGradientVariables_ENTROPY (VariableConversion_NS.f90:211-237) with the absolute pressure.
template <typename R>
__device__ __forceinline__ void entropy_variables(const PhysR<R>& p, const R* Q, R* U) {
    const R irho = R(1) / Q[0];
    const R rV2 = (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]) * irho;
    const R pr = p.gm1 * (Q[4] - R(0.5) * rV2) + p.p_ref;
    const R ip = R(1) / pr;
    U[0] = (p.gamma - (dlog(pr) - p.gamma * dlog(Q[0]))) * p.inv_gm1 - R(0.5) * rV2 * ip;
    U[1] = Q[1] * ip;
    U[2] = Q[2] * ip;
    U[3] = Q[3] * ip;
    U[4] = -Q[0] * ip;
}

// MatrixDissipationRiemannSolver (:578-719): the average minus the entropy-variable jump times
// R |Lambda| T R^T / 2 of the logarithmic-mean states.
template <typename R>
__device__ __forceinline__ void matrix_diss_flux(const PhysR<R>& p, const R* QL, const R* QR, const R* n, const R* t1,
                                                 const R* t2, R* flux) {
    R L[5], Rt[5], EVL[5], EVR[5];
    to_face_frame(QL, n, t1, t2, L);
    to_face_frame(QR, n, t1, t2, Rt);
    entropy_variables(p, L, EVL);
    entropy_variables(p, Rt, EVR);
    const R iL = R(1) / L[0], iR = R(1) / Rt[0];
    const R uL = L[1] * iL, uR = Rt[1] * iR, vL = L[2] * iL, vR = Rt[2] * iR, wL = L[3] * iL, wR = Rt[3] * iR;
    const R vtL = uL * uL + vL * vL + wL * wL, vtR = uR * uR + vR * vR + wR * wR;
    const R pL = p.gm1 * (L[4] - R(0.5) * L[0] * vtL), pR = p.gm1 * (Rt[4] - R(0.5) * Rt[0] * vtR);
    const R betaL = R(-0.5) * EVL[4], betaR = R(-0.5) * EVR[4];
    const R betaLog = log_mean(betaL, betaR), rhoLog = log_mean(L[0], Rt[0]);
    const R pMean = R(0.5) * (L[0] + Rt[0]) / (betaL + betaR);
    const R a = dsqrt(p.gamma * pMean / rhoLog);
    const R u = R(0.5) * (uL + uR), v = R(0.5) * (vL + vR), w = R(0.5) * (wL + wR);
    const R V2 = R(2) * (u * u + v * v + w * w) - R(0.5) * (vtL + vtR);
    const R h = R(0.5) * (p.g_over_gm1 / betaLog + V2);
    R lambda[5] = {fabs(u - a), fabs(u), fabs(u), fabs(u), fabs(u + a)};
    const R Rm[5][5] = {{R(1), u - a, v, w, h - u * a},
                        {R(1), u, v, w, R(0.5) * V2},
                        {R(0), R(0), R(1), R(0), v},
                        {R(0), R(0), R(0), R(1), w},
                        {R(1), u + a, v, w, h + u * a}};  // Rm[j][i] = R1(i, j)
    const R T1 = R(0.5) * rhoLog * p.inv_gamma;
    const R T[5] = {T1, R(2) * p.gm1_over_2g * rhoLog, pMean, pMean, T1};
    R f[5];
    averaged_states(p, L, Rt, pL, pR, iL, iR, f);
    if (p.averaging == 1 || p.averaging == 4) lambda[0] = lambda[4];
    R dEV[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) dEV[k] = EVR[k] - EVL[k];
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        R st = R(0);
#pragma unroll
        for (int j = 0; j < 5; ++j)
#pragma unroll
            for (int k = 0; k < 5; ++k) st = st + R(0.5) * Rm[j][i] * lambda[j] * T[j] * Rm[j][k] * dEV[k];
        f[i] = f[i] - p.lambda_stab * st;
    }
    from_face_frame(f, n, t1, t2, flux);
}

// The interface flux of the chosen solver: Roe (0), LxF (1), central (2), Rusanov (3), standard Roe
// (4), Roe-Pike (5), low-dissipation Roe (6), matrix dissipation (7), viscous NS (8), u-diss (9).
template <typename R>
__device__ __forceinline__ void riemann_flux(const PhysR<R>& p, const R* QL, const R* QR, const R* n, const R* t1,
                                             const R* t2, R* flux) {
    switch (p.riemann) {
        case 0: roe_flux(p, QL, QR, n, flux); break;
        case 3: rusanov_flux(p, QL, QR, n, flux); break;
        case 4: std_roe_flux(p, false, QL, QR, n, t1, t2, flux); break;
        case 5: std_roe_flux(p, true, QL, QR, n, t1, t2, flux); break;
        case 6: low_diss_roe_flux(p, QL, QR, n, t1, t2, flux); break;
        case 7: matrix_diss_flux(p, QL, QR, n, t1, t2, flux); break;
        case 8: viscous_ns_flux(p, QL, QR, n, t1, t2, flux); break;
        default: lxf_flux(p, QL, QR, n, t1, t2, flux); break;
    }
}

// Two-point fluxes of the split form, contracted with the averaged metric vector:
// StandardDG_TwoPointFlux (RiemannSolvers_NS.f90:2085-2145), Morinishi_TwoPointFlux (:2147-2229),
// Ducros_TwoPointFlux (:2231-2294), KennedyGruber_TwoPointFlux (:2296-2367), Pirozzoli_TwoPointFlux
// (:2369-2437), EntropyConserving_TwoPointFlux (:2439-2558), Chandrasekar_TwoPointFlux (:2560-2641).
template <typename R>
__device__ __forceinline__ void two_point_flux(const PhysR<R>& p, const R* QL, const R* QR, const R* JaL, const R* JaR,
                                               R* fs) {
    const R iL = R(1) / QL[0], iR = R(1) / QR[0];
    const R uL = iL * QL[1], uR = iR * QR[1], vL = iL * QL[2], vR = iR * QR[2], wL = iL * QL[3], wR = iR * QR[3];
    const R pL = p.gm1 * (QL[4] - R(0.5) * (QL[1] * uL + QL[2] * vL + QL[3] * wL));
    const R pR = p.gm1 * (QR[4] - R(0.5) * (QR[1] * uR + QR[2] * vR + QR[3] * wR));
    if (p.averaging == 0) {
        const R J0 = JaL[0] + JaR[0], J1 = JaL[1] + JaR[1], J2 = JaL[2] + JaR[2];
        const R HL = QL[4] + pL + p.h_ref, HR = QR[4] + pR + p.h_ref;
        const R f[5] = {QL[1] + QR[1], QL[1] * uL + QR[1] * uR + pL + pR, QL[1] * vL + QR[1] * vR, QL[1] * wL + QR[1] * wR,
                        uL * HL + uR * HR};
        const R g[5] = {QL[2] + QR[2], QL[2] * uL + QR[2] * uR, QL[2] * vL + QR[2] * vR + pL + pR, QL[2] * wL + QR[2] * wR,
                        vL * HL + vR * HR};
        const R h[5] = {QL[3] + QR[3], QL[3] * uL + QR[3] * uR, QL[3] * vL + QR[3] * vR, QL[3] * wL + QR[3] * wR + pL + pR,
                        wL * HL + wR * HR};
#pragma unroll
        for (int q = 0; q < 5; ++q) fs[q] = R(0.25) * (f[q] * J0 + g[q] * J1 + h[q] * J2);
        return;
    }
    const R J0 = R(0.5) * (JaL[0] + JaR[0]), J1 = R(0.5) * (JaL[1] + JaR[1]), J2 = R(0.5) * (JaL[2] + JaR[2]);
    const R vel[2][3] = {{uL, vL, wL}, {uR, vR, wR}};
    R F[3][5];
    if (p.averaging == 2) {  // Ducros
        const R pp = R(0.5) * (pL + pR);
        const R HL = QL[4] + pL + p.h_ref, HR = QR[4] + pR + p.h_ref;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const R su = vel[0][d] + vel[1][d];
            F[d][0] = R(0.25) * (QL[0] + QR[0]) * su;
            F[d][1] = R(0.25) * (QL[1] + QR[1]) * su + (d == 0 ? pp : R(0));
            F[d][2] = R(0.25) * (QL[2] + QR[2]) * su + (d == 1 ? pp : R(0));
            F[d][3] = R(0.25) * (QL[3] + QR[3]) * su + (d == 2 ? pp : R(0));
            F[d][4] = R(0.25) * (HL + HR) * su;
        }
    } else if (p.averaging == 3) {  // Morinishi
        const R pp = R(0.5) * (pL + pR);
        const R hL = p.g_over_gm1 * (pL + p.p_ref), hR = p.g_over_gm1 * (pR + p.p_ref);
        const R kL2 = uL * uL + vL * vL + wL * wL, kR2 = uR * uR + vR * vR + wR * wR;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const R mL = QL[1 + d], mR = QR[1 + d], m = mL + mR;
            F[d][0] = R(0.5) * m;
            F[d][1] = R(0.25) * m * (uL + uR) + (d == 0 ? pp : R(0));
            F[d][2] = R(0.25) * m * (vL + vR) + (d == 1 ? pp : R(0));
            F[d][3] = R(0.25) * m * (wL + wR) + (d == 2 ? pp : R(0));
            F[d][4] = R(0.5) * (vel[0][d] * hL + vel[1][d] * hR) + R(0.25) * (mL * uL + mR * uR) * (uL + uR) +
                      R(0.25) * (mL * vL + mR * vR) * (vL + vR) + R(0.25) * (mL * wL + mR * wR) * (wL + wR) -
                      R(0.25) * (mL * kL2 + mR * kR2);
        }
    } else if (p.averaging == 4) {  // Kennedy-Gruber
        const R rho = R(0.5) * (QL[0] + QR[0]), u = R(0.5) * (uL + uR), v = R(0.5) * (vL + vR);
        const R w = R(0.5) * (wL + wR), pp = R(0.5) * (pL + pR);
        const R e = R(0.5) * ((QL[4] + p.e_ref) * iL + (QR[4] + p.e_ref) * iR);
        const R pa = pp + p.p_ref;
        const R um[3] = {u, v, w};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const R ru = rho * um[d];
            F[d][0] = ru;
            F[d][1] = ru * u + (d == 0 ? pp : R(0));
            F[d][2] = ru * v + (d == 1 ? pp : R(0));
            F[d][3] = ru * w + (d == 2 ? pp : R(0));
            F[d][4] = ru * e + pa * um[d];
        }
    } else if (p.averaging == 5 || p.averaging == 6) {  // entropy conserving, Chandrasekar
        R rho, u, v, w, pm, h;
        log_mean_state(p, p.averaging == 5, QL[0], QR[0], uL, uR, vL, vR, wL, wR, pL + p.p_ref, pR + p.p_ref, rho, u, v,
                       w, pm, h, true);
        const R pp = pm - p.p_ref;
        const R ru = rho * u, rv = rho * v, rw = rho * w;
        fs[0] = ru * J0 + rv * J1 + rw * J2;
        fs[1] = (ru * u + pp) * J0 + (rv * u) * J1 + (rw * u) * J2;
        fs[2] = (ru * v) * J0 + (rv * v + pp) * J1 + (rw * v) * J2;
        fs[3] = (ru * w) * J0 + (rv * w) * J1 + (rw * w + pp) * J2;
        fs[4] = (ru * h) * J0 + (rv * h) * J1 + (rw * h) * J2;
        return;
    } else {  // Pirozzoli
        const R rho = R(0.5) * (QL[0] + QR[0]), u = R(0.5) * (uL + uR), v = R(0.5) * (vL + vR), w = R(0.5) * (wL + wR);
        const R pp = R(0.5) * (pL + pR);
        const R h = R(0.5) * ((QL[4] + pL + p.h_ref) * iL + (QR[4] + pR + p.h_ref) * iR);
        const R ru = rho * u, rv = rho * v, rw = rho * w;
        fs[0] = ru * J0 + rv * J1 + rw * J2;
        fs[1] = (ru * u + pp) * J0 + (rv * u) * J1 + (rw * u) * J2;
        fs[2] = (ru * v) * J0 + (rv * v + pp) * J1 + (rw * v) * J2;
        fs[3] = (ru * w) * J0 + (rv * w) * J1 + (rw * w + pp) * J2;
        fs[4] = (ru * h) * J0 + (rv * h) * J1 + (rw * h) * J2;
        return;
    }
#pragma unroll
    for (int q = 0; q < 5; ++q) fs[q] = F[0][q] * J0 + F[1][q] * J1 + F[2][q] * J2;
}

// Convergence/SETUP/ProblemFile.f90:31-133 state_source_in_point: the source term S(x,t).
__device__ __forceinline__ void mms_source(double x, double y, double z, double t, double gm1, double gMa2, double mu,
                                           double kap, double* S) {
    const double c_u = 1.0, c_v = 2.0, c_w = -c_u - c_v;
    const double Ssu = 0.381923076923077;
    const double PI = 3.141592653589793238462643;
    const double arg = PI * (x + y + z - 2.0 * t);
    double sa, ca;
    sincos(arg, &sa, &ca);
    const double rho = 2.0 + 0.1 * sa;
    const double u = c_u * rho - 1.0, v = c_v * rho - 4.0, w = c_w * rho + 5.0, e = rho;
    const double vtot = u * u + v * v + w * w;
    const double p = gm1 * (rho * e - 0.5 * rho * vtot);
    const double Temp = gMa2 * gm1 * (e - 0.5 * vtot);
    const double suther = (1.0 + Ssu) / (Temp + Ssu) * Temp * sqrt(Temp);
    const double dsdT = 1.5 * suther / Temp - suther / (Ssu + Temp);
    const double rho_t = 0.1 * (-2.0 * PI) * ca;
    const double u_t = c_u * rho_t, v_t = c_v * rho_t, w_t = c_w * rho_t, e_t = rho_t;
    const double rx = 0.1 * PI * ca;  // every component of grad(rho)
    const double ux = c_u * rx, vx = c_v * rx, wx = c_w * rx, ex = rx;
    const double px = gm1 * rx * (e - 0.5 * vtot) + gm1 * rho * (ex - u * ux - v * vx - w * wx);
    const double Tx = gMa2 * gm1 * (ex - u * ux - v * vx - w * wx);
    const double div_v = ux + vx + wx;
    // grad_u(i,j) = d(vel_j)/dx_i is the same for every i: rows (ux, vx, wx)
    const double gj[3] = {ux, vx, wx};
    double tau[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) tau[i][j] = mu * suther * (gj[j] + gj[i] - 2.0 * div_v * (i == j ? 1.0 : 0.0) / 3.0);
    const double rxx = -0.1 * (PI * PI) * sa;
    const double uxx = c_u * rxx, vxx = c_v * rxx, wxx = c_w * rxx, exx = rxx;
    double Txx_tr = 0.0;
    for (int i = 0; i < 3; ++i)
        Txx_tr += gMa2 * gm1 * (exx - ux * ux - vx * vx - wx * wx - u * uxx - v * vxx - w * wxx);
    double dtau[3];
    for (int j = 0; j < 3; ++j) {
        const double tr[3] = {3.0 * uxx, 3.0 * vxx, 3.0 * wxx};
        dtau[j] = uxx + vxx + wxx + tr[j] - (2.0 / 3.0) * (uxx + vxx + wxx);
        dtau[j] = mu * suther * dtau[j];
        const double mt = tau[j][0] * Tx + tau[j][1] * Tx + tau[j][2] * Tx;
        dtau[j] = dtau[j] + (dsdT / suther) * mt;
    }
    double sgt = 0.0;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) sgt += gj[j] * tau[i][j];
    const double vw = sgt + u * dtau[0] + v * dtau[1] + w * dtau[2];
    const double heat = kap * dsdT * (3.0 * Tx * Tx) + kap * suther * Txx_tr;
    S[0] = rho_t + u * rx + v * rx + w * rx + rho * div_v;
    S[1] = u * S[0] + rho * u_t + rho * u * ux + rho * v * ux + rho * w * ux + px - dtau[0];
    S[2] = v * S[0] + rho * v_t + rho * u * vx + rho * v * vx + rho * w * vx + px - dtau[1];
    S[3] = w * S[0] + rho * w_t + rho * u * wx + rho * v * wx + rho * w * wx + px - dtau[2];
    S[4] = e * S[0] + rho * e_t + rho * (u * ex + v * ex + w * ex) + p * div_v + u * px + v * px + w * px - vw - heat;
}

// LambVector/SETUP/ProblemFile.f90:377-423 UserDefinedSourceTermNS for the state of :8-27,
//   rho = 3 + sin(phi) e^t, (u, v, w) = (cos phi, sin phi, cos phi) e^-t, E = rho |u|^2 / 2 + 1,
// phi = x + y + z: the residual dQ/dt + div(F_inviscid - F_viscous / Re) of the dimensionless NS
// equations for that state, with the constant viscosity mu and conductivity kappa the source term
// is defined with (the solver's own fluxes keep Sutherland's law). Every field depends on phi
// only, so d/dx = d/dy = d/dz = d/dphi; primes below are d/dphi. mu_re = mu / Re and
// kap_re = kappa / Re.
__host__ __device__ inline void lamb_vector_source(double x, double y, double z, double t, double gm1, double gMa2,
                                                   double mu_re, double kap_re, double* S) {
    const double ph = x + y + z;
    const double a = sin(ph), b = cos(ph), ep = exp(t), em = exp(-t);
    const double r = 3.0 + a * ep, r1 = b * ep, r2 = -a * ep, rt = a * ep;
    const double U[3] = {b * em, a * em, b * em};     // dU/dt = -U
    const double U1[3] = {-a * em, b * em, -a * em};
    const double U2[3] = {-b * em, -a * em, -b * em};
    double s = 0.0, D = 0.0, D1 = 0.0, k = 0.0, k1 = 0.0, k2 = 0.0, uu2 = 0.0, g1 = 0.0;
    for (int i = 0; i < 3; ++i) {
        s += U[i];              // u + v + w
        D += U1[i];             // div u
        D1 += U2[i];
        k += 0.5 * U[i] * U[i];  // |u|^2 / 2
        k1 += U[i] * U1[i];
        uu2 += U[i] * U2[i];
        g1 += U1[i] * U1[i];
    }
    k2 = g1 + uu2;
    const double kt = -2.0 * k;
    const double E = r * k + 1.0, E1 = r1 * k + r * k1, E2 = r2 * k + 2.0 * r1 * k1 + r * k2, Et = rt * k + r * kt;
    const double ei = E - k, ei1 = E1 - k1, ei2 = E2 - k2;  // internal energy
    const double p = gm1 * r * ei, p1 = gm1 * (r1 * ei + r * ei1);
    const double T2 = gMa2 * gm1 * ei2;  // T = gamma M^2 (gamma - 1) e
    S[0] = rt + r1 * s + r * D;
    for (int j = 0; j < 3; ++j)
        S[1 + j] = rt * U[j] - r * U[j] + (r1 * U[j] + r * U1[j]) * s + r * U[j] * D + p1 -
                   mu_re * (3.0 * U2[j] + D1 / 3.0);
    S[4] = rt * E + r * Et + (r1 * E + r * E1 + p1) * s + (r * E + p) * D -
           mu_re * (D1 * s / 3.0 + 3.0 * uu2 + D * D / 3.0 + 3.0 * g1) - 3.0 * kap_re * T2;
}

// The source of the given DG_SOURCE_* kind (1 Convergence, 2 LambVector) with its constants.
__device__ __forceinline__ void manufactured_source(int kind, double x, double y, double z, double t, double gm1,
                                                    double gMa2, double mu, double kap, double* S) {
    if (kind == 2) lamb_vector_source(x, y, z, t, gm1, gMa2, mu, kap, S);
    else mms_source(x, y, z, t, gm1, gMa2, mu, kap, S);
}

// Viscosity and conductivity the sources are evaluated with, (mu, kappa) as the source functions
// take them. Convergence: the dimensionless 1/Re and 1/((gamma-1) M^2 Re Pr). LambVector: the
// dimensional reference viscosity refValues%mu = rho_ref V_ref L_ref / Re (PhysicsStorage_NS.f90:
// 292-309; T_ref = 520*5/9 K, p_ref = 101325 Pa, R = 287.15 J/(kg K), L_ref = 1 m) and
// kappa = mu * mu_to_kappa, both divided by Re; zero for the Euler equations.
inline void source_constants(int kind, double mach, double reynolds, double prandtl, int ns, double* mu,
                             double* kap) {
    const double gamma = 1.4, gm1 = 1.4 - 1.0;
    *mu = 0.0;
    *kap = 0.0;
    if (!ns) return;
    if (kind == 2) {
        const double R = 287.15, T = 520.0 * 5.0 / 9.0;
        const double rho_ref = 101325.0 / (R * T), V_ref = mach * sqrt(gamma * R * T);
        const double mu_ref = rho_ref * V_ref * 1.0 * (1.0 / reynolds);
        *mu = mu_ref / reynolds;
        *kap = mu_ref * (1.0 / (gm1 * (mach * mach) * prandtl)) / reynolds;
    } else {
        *mu = 1.0 / reynolds;
        *kap = 1.0 / (gm1 * (mach * mach) * reynolds * prandtl);
    }
}

// ---- boundary conditions (physics/common/*BC.f90, NAVIERSTOKES parts) ----------------------------
// The energies of the state vectors are the stored ones (E' = E - e_ref in the mixed form); the
// formulas are arranged so that the reference energy cancels where it does in exact arithmetic.
template <typename R>
struct BoundaryR {
    int type;
    R wt;          // 1 isothermal, 0 adiabatic (wallType)
    R ewall;       // T_w/T_ref / ((gamma-1) gamma M^2): wall internal energy
    R pwall;       // T_w/T_ref / (gamma M^2): wall pressure per unit density
    R vw[3];       // no-slip wall velocity
    R rho, u, v, w, E;  // inflow state (absolute total energy)
    R pext;        // outflow pressure
};

template <typename R>
BoundaryR<R> make_boundary(const dg_boundary& b, const PhysConst& c) {
    BoundaryR<R> r;
    r.type = b.type;
    r.wt = R(b.isothermal ? 1.0 : 0.0);
    r.ewall = R(b.wall_temperature / (c.gammaM2 * c.gm1));
    r.pwall = R(b.wall_temperature / c.gammaM2);
    for (int k = 0; k < 3; ++k) r.vw[k] = R(b.wall_velocity[k]);
    r.rho = R(b.rho); r.u = R(b.u); r.v = R(b.v); r.w = R(b.w);
    r.E = R(b.p / (c.gamma - 1.0) + 0.5 * b.rho * (b.u * b.u + b.v * b.v + b.w * b.w));
    r.pext = R(b.pressure);
    return r;
}

// FlowState: the external state of the Riemann problem (NoSlipWallBC.f90:265-296,
// FreeSlipWallBC.f90:249-286, InflowBC.f90:363-406, OutflowBC.f90:226-288).
template <typename R>
__device__ __forceinline__ void bc_state(const PhysR<R>& p, const BoundaryR<R>& b, const R* n, R* Q) {
    if (b.type == 1) {
#pragma unroll
        for (int c = 0; c < 3; ++c) Q[1 + c] = R(2) * Q[0] * b.vw[c] - Q[1 + c];
        Q[4] = Q[4] + b.wt * (Q[0] * b.ewall - p.e_ref - Q[4]);
    } else if (b.type == 2) {
        const R qn = n[0] * Q[1] + n[1] * Q[2] + n[2] * Q[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) Q[1 + c] = Q[1 + c] - R(2) * qn * n[c];
        const R pa = Q[0] * b.pwall;
        Q[4] = Q[4] + b.wt * (pa / p.gm1 + R(0.5) * (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]) / Q[0] - p.e_ref - Q[4]);
    } else if (b.type == 3) {
        Q[0] = b.rho;
        Q[1] = b.rho * b.u;
        Q[2] = b.rho * b.v;
        Q[3] = b.rho * b.w;
        Q[4] = b.E - p.e_ref;
    } else {
        R qn = (n[0] * Q[1] + n[1] * Q[2] + n[2] * Q[3]) / Q[0];
        const R tx = Q[1] / Q[0] - qn * n[0], ty = Q[2] / Q[0] - qn * n[1], tz = Q[3] / Q[0] - qn * n[2];
        const R pr = p.gm1 * (Q[4] - R(0.5) * (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]) / Q[0]) + p.p_ref;
        const R a2 = p.gamma * pr / Q[0];
        R a = dsqrt(a2);
        if (fabs(qn / a) <= R(1)) {
            const R rPlus = qn + R(2) * a / p.gm1;
            const R ent = pr - a2 * Q[0];
            const R rho = -(ent - b.pext) / a2;
            a = dsqrt(p.gamma * b.pext / rho);
            qn = rPlus - R(2) * a / p.gm1;
            const R u = tx + qn * n[0], v = ty + qn * n[1], w = tz + qn * n[2];
            Q[0] = rho;
            Q[1] = rho * u;
            Q[2] = rho * v;
            Q[3] = rho * w;
            Q[4] = b.pext / p.gm1 + R(0.5) * rho * (u * u + v * v + w * w) - p.e_ref;
        }
    }
}

// FlowGradVars: U* at the boundary from the interior state Q and its gradient variables U
// (NoSlipWallBC.f90:298-337, FreeSlipWallBC.f90:288-318, GenericBC_FlowGradVars for in/outflow).
template <typename R>
__device__ __forceinline__ void bc_gradvars(const PhysR<R>& p, const BoundaryR<R>& b, const R* n, const R* Q,
                                            const R* U, R* Us) {
    R Qa[5];
    if (b.type == 1) {
        const R m2 = (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]) / Q[0];
        const R kw = R(0.5) * Q[0] * (b.vw[0] * b.vw[0] + b.vw[1] * b.vw[1] + b.vw[2] * b.vw[2]);
        Qa[0] = Q[0];
#pragma unroll
        for (int c = 0; c < 3; ++c) Qa[1 + c] = Q[0] * b.vw[c];
        // rho ((1 - wt) e_int + wt e_wall + |v_w|^2 / 2), relative to e_ref
        Qa[4] = (R(1) - b.wt) * (Q[4] - R(0.5) * m2) + b.wt * (Q[0] * b.ewall - p.e_ref) + kw;
        gradient_variables(p, Qa, Us);
        Us[0] = U[0];
    } else if (b.type == 2) {
#pragma unroll
        for (int c = 0; c < 4; ++c) Qa[c] = Q[c];
        Qa[4] = Q[4] + b.wt * (Q[0] * b.ewall + R(0.5) * (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]) / Q[0] - p.e_ref - Q[4]);
        gradient_variables(p, Qa, Us);
    } else {
#pragma unroll
        for (int c = 0; c < 5; ++c) Qa[c] = Q[c];
        bc_state(p, b, n, Qa);
        R Ua[5];
        gradient_variables(p, Qa, Ua);
#pragma unroll
        for (int c = 0; c < 5; ++c) Us[c] = R(0.5) * (Ua[c] + U[c]);
    }
}

// FlowNeumann: the boundary's viscous normal flux from the interior one (NoSlipWallBC.f90:339-372,
// FreeSlipWallBC.f90:320-351; inflow and outflow cancel it).
template <typename R>
__device__ __forceinline__ void bc_neumann(const BoundaryR<R>& b, const R* Q, R* f) {
    if (b.type == 1) {
        const R ir = R(1) / Q[0];
        const R work = (ir * Q[1]) * f[1] + (ir * Q[2]) * f[2] + (ir * Q[3]) * f[3];
        const R heat = f[4] - work;
        f[0] = R(0);
        f[4] = (b.vw[0] * f[1] + b.vw[1] * f[2] + b.vw[2] * f[3]) + b.wt * heat;
    } else if (b.type == 2) {
        const R work = (f[1] * Q[1] + f[2] * Q[2] + f[3] * Q[3]) / Q[0];
        const R heat = f[4] - work;
        f[0] = f[1] = f[2] = f[3] = R(0);
        f[4] = b.wt * heat;
    } else {
#pragma unroll
        for (int c = 0; c < 5; ++c) f[c] = R(0);
    }
}

// MeshTypes.f90:70-107 leftIndexes2Right.
__device__ __forceinline__ void left2right(int i, int j, int Nx, int Ny, int rot, int& ii, int& jj) {
    switch (rot) {
        case 0: ii = i; jj = j; break;
        case 1: ii = Ny - j; jj = i; break;
        case 2: ii = Nx - i; jj = Ny - j; break;
        case 3: ii = j; jj = Nx - i; break;
        case 4: ii = j; jj = i; break;
        case 5: ii = Nx - i; jj = j; break;
        case 6: ii = Ny - j; jj = Nx - i; break;
        default: ii = i; jj = Ny - j; break;
    }
}

}  // namespace dg
