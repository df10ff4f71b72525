// ORACLE -- test infrastructure only. Nothing in the product links or calls this file; it is the
// CPU FP64 checker that tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use.
//
// A loop-for-loop C++ restatement of HORSES3D's compressible Navier-Stokes right-hand side and
// Williamson RK3 step. Element arrays keep the reference layout Q(1:NEQ,0:Nx,0:Ny,0:Nz); face arrays
// keep the per-side FaceStorage layout. Each routine cites the reference routine it follows.
// It consumes the same dg_mesh_desc as the GPU library (the geometry is an input to both), and it
// computes its own spectral operators so that a fault in the product's operators cannot hide.
//
// Parity: pinned by tests/test_oracle_golden.py against the goldens of
// Solver/test/NavierStokes/Convergence/SETUP/ProblemFile.f90:617-635 (tol 1e-11, :711-790).
// Build: oracle/Makefile (g++ -O2 -ffp-contract=off -fopenmp).
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include <omp.h>

#include "horses3d_gb300.h"
#include "spectral.hpp"

namespace orc {

enum { IRHO = 0, IRHOU, IRHOV, IRHOW, IRHOE };

// ---------------------------------------------------------------- physics --------------------
struct Phys {
    double gamma = 1.4, gm1 = 1.4 - 1.0, Mach, Re, Pr, mu, kappa, mu_to_kappa, gammaM2;  // PhysicsStorage_NS.f90:115-133
    double S_div_TRef, TReNorm;
    bool ns;
    int grad_vars = DG_GRADVARS_STATE;
};

static inline double pressure(const Phys& p, const double* Q) {  // VariableConversion_NS.f90:44-57
    return p.gm1 * (Q[4] - 0.5 * (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]) / Q[0]);
}
static inline double sutherland(const Phys& p, double T) {  // VariableConversion_NS.f90:170-186
    const double t = T * p.TReNorm;
    return (1.0 + p.S_div_TRef) / (t + p.S_div_TRef) * t * std::sqrt(t);
}
static inline void mu_kappa(const Phys& p, const double* Q, double& mu, double& kappa) {  // :147-164
    const double T = p.gammaM2 * pressure(p, Q) / Q[0];
    const double s = sutherland(p, T);
    mu = p.mu * s;
    kappa = mu * p.mu_to_kappa;
}

// Physics_NS.f90:51-103 EulerFlux: F(1:5,1:3) stored F[v + 5*d].
static void euler_flux(const Phys& p, const double* Q, double* F) {
    const double u = Q[1] / Q[0], v = Q[2] / Q[0], w = Q[3] / Q[0];
    const double pr = p.gm1 * (Q[4] - 0.5 * (Q[1] * u + Q[2] * v + Q[3] * w));
    F[0] = Q[1]; F[1] = Q[1] * u + pr; F[2] = Q[1] * v; F[3] = Q[1] * w; F[4] = (Q[4] + pr) * u;
    F[5] = Q[2]; F[6] = F[2]; F[7] = Q[2] * v + pr; F[8] = Q[2] * w; F[9] = (Q[4] + pr) * v;
    F[10] = Q[3]; F[11] = F[3]; F[12] = F[8]; F[13] = Q[3] * w + pr; F[14] = (Q[4] + pr) * w;
}

// VariableConversion_NS.f90:196-262 NSGradientVariables_STATE / _ENTROPY / _ENERGY.
static void gradient_variables(const Phys& p, const double* Q, double* U) {
    if (p.grad_vars == DG_GRADVARS_STATE) {
        for (int v = 0; v < 5; ++v) U[v] = Q[v];
        return;
    }
    const double invRho = 1.0 / Q[0];
    const double rhoV2 = (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]) * invRho;
    const double pr = p.gm1 * (Q[4] - 0.5 * rhoV2);
    if (p.grad_vars == DG_GRADVARS_ENTROPY) {
        const double invP = 1.0 / pr;
        U[0] = (p.gamma - (std::log(pr) - p.gamma * std::log(Q[0]))) * (1.0 / (1.4 - 1.0)) - 0.5 * rhoV2 * invP;
        U[1] = Q[1] * invP;
        U[2] = Q[2] * invP;
        U[3] = Q[3] * invP;
        U[4] = -Q[0] * invP;
    } else {
        U[0] = Q[0];
        U[1] = Q[1] * invRho;
        U[2] = Q[2] * invRho;
        U[3] = Q[3] * invRho;
        U[4] = p.gammaM2 * pr * invRho;
    }
}

// Physics_NS.f90:246-414 ViscousFlux_STATE, ViscousFlux_ENTROPY, ViscousFlux_ENERGY.
static void viscous_flux(const Phys& p, const double* Q, const double* Ux, const double* Uy, const double* Uz,
                         double mu, double beta, double kappa, double* F) {
    const double invRho = 1.0 / Q[0];
    const double u = Q[1] * invRho, v = Q[2] * invRho, w = Q[3] * invRho;
    double ux[3], uy[3], uz[3], nTx, nTy, nTz;
    if (p.grad_vars == DG_GRADVARS_STATE) {
        const double ud[3] = {u * invRho, v * invRho, w * invRho};
        for (int c = 0; c < 3; ++c) {
            ux[c] = invRho * Ux[1 + c] - ud[c] * Ux[0];
            uy[c] = invRho * Uy[1 + c] - ud[c] * Uy[0];
            uz[c] = invRho * Uz[1 + c] - ud[c] * Uz[0];
        }
        const double g = p.gm1 * p.gammaM2;
        nTx = g * (invRho * Ux[4] - Q[4] * invRho * invRho * Ux[0] - u * ux[0] - v * ux[1] - w * ux[2]);
        nTy = g * (invRho * Uy[4] - Q[4] * invRho * invRho * Uy[0] - u * uy[0] - v * uy[1] - w * uy[2]);
        nTz = g * (invRho * Uz[4] - Q[4] * invRho * invRho * Uz[0] - u * uz[0] - v * uz[1] - w * uz[2]);
    } else if (p.grad_vars == DG_GRADVARS_ENTROPY) {
        const double pdr = p.gm1 * invRho * (Q[4] - 0.5 * (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]) * invRho);
        const double um[3] = {u, v, w};
        for (int c = 0; c < 3; ++c) {
            ux[c] = pdr * (Ux[1 + c] + um[c] * Ux[4]);
            uy[c] = pdr * (Uy[1 + c] + um[c] * Uy[4]);
            uz[c] = pdr * (Uz[1 + c] + um[c] * Uz[4]);
        }
        nTx = p.gammaM2 * (pdr * pdr) * Ux[4];
        nTy = p.gammaM2 * (pdr * pdr) * Uy[4];
        nTz = p.gammaM2 * (pdr * pdr) * Uz[4];
    } else {
        for (int c = 0; c < 3; ++c) {
            ux[c] = Ux[1 + c];
            uy[c] = Uy[1 + c];
            uz[c] = Uz[1 + c];
        }
        nTx = Ux[4];
        nTy = Uy[4];
        nTz = Uz[4];
    }
    const double divV = ux[0] + uy[1] + uz[2];
    F[0] = 0.0;
    F[1] = mu * (2.0 * ux[0] - 2.0 / 3.0 * divV) + beta * divV;
    F[2] = mu * (ux[1] + uy[0]);
    F[3] = mu * (ux[2] + uz[0]);
    F[4] = F[1] * u + F[2] * v + F[3] * w + kappa * nTx;
    F[5] = 0.0;
    F[6] = F[2];
    F[7] = mu * (2.0 * uy[1] - 2.0 / 3.0 * divV) + beta * divV;
    F[8] = mu * (uy[2] + uz[1]);
    F[9] = F[6] * u + F[7] * v + F[8] * w + kappa * nTy;
    F[10] = 0.0;
    F[11] = F[3];
    F[12] = F[8];
    F[13] = mu * (2.0 * uz[2] - 2.0 / 3.0 * divV) + beta * divV;
    F[14] = F[11] * u + F[12] * v + F[13] * w + kappa * nTz;
}

// RiemannSolvers_NS.f90:1541-1655 RoeRiemannSolver.
static void roe(const Phys& p, const double* QL, const double* QR, const double* n, double* flux) {
    const double g = p.gamma;
    const double rho = QL[0], rhou = QL[1], rhov = QL[2], rhow = QL[3], rhoe = QL[4];
    const double rhon = QR[0], rhoun = QR[1], rhovn = QR[2], rhown = QR[3], rhoen = QR[4];
    const double ul = rhou / rho, vl = rhov / rho, wl = rhow / rho;
    const double pleft = (g - 1.0) * (rhoe - 0.5 / rho * (rhou * rhou + rhov * rhov + rhow * rhow));
    const double ur = rhoun / rhon, vr = rhovn / rhon, wr = rhown / rhon;
    const double pright = (g - 1.0) * (rhoen - 0.5 / rhon * (rhoun * rhoun + rhovn * rhovn + rhown * rhown));
    const double ql = n[0] * ul + n[1] * vl + n[2] * wl;
    const double qr = n[0] * ur + n[1] * vr + n[2] * wr;
    const double hl = 0.5 * (ul * ul + vl * vl + wl * wl) + g / (g - 1.0) * pleft / rho;
    const double hr = 0.5 * (ur * ur + vr * vr + wr * wr) + g / (g - 1.0) * pright / rhon;
    const double rtd = std::sqrt(rho * rhon);
    const double betal = rho / (rho + rtd), betar = 1.0 - betal;
    const double utd = betal * ul + betar * ur, vtd = betal * vl + betar * vr, wtd = betal * wl + betar * wr;
    const double htd = betal * hl + betar * hr;
    const double atd2 = (g - 1.0) * (htd - 0.5 * (utd * utd + vtd * vtd + wtd * wtd));
    const double atd = std::sqrt(atd2);
    const double qtd = utd * n[0] + vtd * n[1] + wtd * n[2];
    if (qtd >= 0.0) {
        const double dw1 = 0.5 * ((pright - pleft) / atd2 - (qr - ql) * rtd / atd);
        const double sp1 = qtd - atd;
        const double sp1m = std::fmin(sp1, 0.0);
        const double hd1m = ((g + 1.0) / 4.0 * atd / rtd) * dw1;
        const double eta1 = std::fmax(-std::fabs(sp1) - hd1m, 0.0);
        const double udw1 = dw1 * (sp1m - 0.5 * eta1);
        const double rql = rho * ql;
        flux[0] = 1.0 * (rql + udw1);
        flux[1] = 1.0 * (rql * ul + pleft * n[0] + udw1 * (utd - atd * n[0]));
        flux[2] = 1.0 * (rql * vl + pleft * n[1] + udw1 * (vtd - atd * n[1]));
        flux[3] = 1.0 * (rql * wl + pleft * n[2] + udw1 * (wtd - atd * n[2]));
        flux[4] = 1.0 * (rql * hl + udw1 * (htd - qtd * atd));
    } else {
        const double dw4 = 0.5 * ((pright - pleft) / atd2 + (qr - ql) * rtd / atd);
        const double sp4 = qtd + atd;
        const double sp4p = std::fmax(sp4, 0.0);
        const double hd4 = ((g + 1.0) / 4.0 * atd / rtd) * dw4;
        const double eta4 = std::fmax(-std::fabs(sp4) + hd4, 0.0);
        const double udw4 = dw4 * (sp4p + 0.5 * eta4);
        const double rqr = rhon * qr;
        flux[0] = 1.0 * (rqr - udw4);
        flux[1] = 1.0 * (rqr * ur + pright * n[0] - udw4 * (utd + atd * n[0]));
        flux[2] = 1.0 * (rqr * vr + pright * n[1] - udw4 * (vtd + atd * n[1]));
        flux[3] = 1.0 * (rqr * wr + pright * n[2] - udw4 * (wtd + atd * n[2]));
        flux[4] = 1.0 * (rqr * hr - udw4 * (htd + qtd * atd));
    }
}

// Averaged states of the rotated (normal, t1, t2) frame: RiemannSolvers_NS.f90:1784-1819 StandardAverage,
// :1821-1848 DucrosAverage, :1850-1886 MorinishiAverage, :1888-1925 KennedyGruberAverage,
// :1927-1962 PirozzoliAverage.
// Utilities.f90:269-301 logarithmicMean (Ismail and Roe).
static double log_mean(double aL, double aR) {
    const double xi = aL / aR;
    const double f = (xi - 1.0) / (xi + 1.0);
    const double u = f * f;
    double FF;
    if (u < 0.01) FF = 1.0 + (1.0 / 3.0) * u + (1.0 / 5.0) * (u * u) + (1.0 / 7.0) * ((u * u) * u);
    else FF = std::log(xi) / (2.0 * f);
    return 0.5 * (aL + aR) / FF;
}

static void average(const Phys& ph, int avg, const double* L, const double* R, double pL, double pR, double iL,
                    double iR, double* f) {
    const double uL = iL * L[1], uR = iR * R[1], vL = iL * L[2], vR = iR * R[2], wL = iL * L[3], wR = iR * R[3];
    if (avg == DG_AVG_ENTROPY_CONSERVING) {  // :1964-2026 EntropyConservingAverage (Ismail and Roe)
        const double rhoL = L[0], rhoR = R[0];
        double zL[5], zR[5], zS[5];
        zL[4] = std::sqrt(rhoL * pL); zR[4] = std::sqrt(rhoR * pR);
        zL[0] = rhoL / zL[4]; zR[0] = rhoR / zR[4];
        zL[1] = zL[0] * uL; zR[1] = zR[0] * uR;
        zL[2] = zL[0] * vL; zR[2] = zR[0] * vR;
        zL[3] = zL[0] * wL; zR[3] = zR[0] * wR;
        for (int q = 0; q < 5; ++q) zS[q] = zL[q] + zR[q];
        const double inv1 = 1.0 / zS[0];
        const double z1Log = log_mean(zL[0], zR[0]), z5Log = log_mean(zL[4], zR[4]);
        const double rho = 0.5 * zS[0] * z5Log;
        const double u = zS[1] * inv1, v = zS[2] * inv1, w = zS[3] * inv1, p = zS[4] * inv1;
        const double p2 = ((ph.gamma + 1.0) / 2.0 * z5Log / z1Log + (ph.gamma - 1.0) / 2.0 * p) * (1.0 / ph.gamma);
        const double h = ph.gamma / ph.gm1 * p2 / rho + 0.5 * (u * u + v * v + w * w);
        f[0] = rho * u; f[1] = rho * u * u + p; f[2] = rho * u * v; f[3] = rho * u * w; f[4] = rho * u * h;
        return;
    }
    if (avg == DG_AVG_CHANDRASEKAR) {  // :2028-2077 ChandrasekarAverage
        const double rhoL = L[0], rhoR = R[0];
        const double betaL = 0.5 * rhoL / pL, betaR = 0.5 * rhoR / pR;
        const double betaLog = log_mean(betaL, betaR);
        const double rho = log_mean(rhoL, rhoR);
        const double u = 0.5 * (uL + uR), v = 0.5 * (vL + vR), w = 0.5 * (wL + wR);
        const double p = 0.5 * (rhoL + rhoR) / (betaL + betaR);
        const double h = 0.5 / (betaLog * ph.gm1) -
                         0.5 * (0.5 * ((uL * uL + vL * vL + wL * wL) + (uR * uR + vR * vR + wR * wR))) + p / rho +
                         u * u + v * v + w * w;
        f[0] = rho * u; f[1] = rho * u * u + p; f[2] = rho * u * v; f[3] = rho * u * w; f[4] = rho * u * h;
        return;
    }
    if (avg == DG_AVG_STANDARD) {
        f[0] = 0.5 * (L[1] + R[1]);
        f[1] = 0.5 * (L[1] * uL + R[1] * uR + pL + pR);
        f[2] = 0.5 * (L[1] * vL + R[1] * vR);
        f[3] = 0.5 * (L[1] * wL + R[1] * wR);
        f[4] = 0.5 * (uL * (L[4] + pL) + uR * (R[4] + pR));
    } else if (avg == DG_AVG_DUCROS) {
        f[0] = 0.25 * (L[0] + R[0]) * (uL + uR);
        f[1] = 0.25 * (L[1] + R[1]) * (uL + uR) + 0.5 * (pL + pR);
        f[2] = 0.25 * (L[2] + R[2]) * (uL + uR);
        f[3] = 0.25 * (L[3] + R[3]) * (uL + uR);
        f[4] = 0.25 * (L[4] + pL + R[4] + pR) * (uL + uR);
    } else if (avg == DG_AVG_MORINISHI) {
        const double cp = ph.gamma / ph.gm1;
        const double hL = cp * pL, hR = cp * pR;
        f[0] = 0.5 * (L[1] + R[1]);
        f[1] = 0.25 * (L[1] + R[1]) * (uL + uR) + 0.5 * (pL + pR);
        f[2] = 0.25 * (L[1] + R[1]) * (vL + vR);
        f[3] = 0.25 * (L[1] + R[1]) * (wL + wR);
        f[4] = 0.5 * (uL * hL + uR * hR) + 0.25 * (L[1] * uL + R[1] * uR) * (uL + uR) +
               0.25 * (L[1] * vL + R[1] * vR) * (vL + vR) + 0.25 * (L[1] * wL + R[1] * wR) * (wL + wR) -
               0.25 * (L[1] * uL * uL + R[1] * uR * uR) - 0.25 * (L[1] * vL * vL + R[1] * vR * vR) -
               0.25 * (L[1] * wL * wL + R[1] * wR * wR);
    } else if (avg == DG_AVG_KENNEDY_GRUBER) {
        const double rho = 0.5 * (L[0] + R[0]), u = 0.5 * (uL + uR), v = 0.5 * (vL + vR), w = 0.5 * (wL + wR);
        const double p = 0.5 * (pL + pR), e = 0.5 * (L[4] * iL + R[4] * iR);
        f[0] = rho * u; f[1] = rho * u * u + p; f[2] = rho * u * v; f[3] = rho * u * w; f[4] = rho * u * e + p * u;
    } else {
        const double rho = 0.5 * (L[0] + R[0]), u = 0.5 * (uL + uR), v = 0.5 * (vL + vR), w = 0.5 * (wL + wR);
        const double p = 0.5 * (pL + pR);
        const double h = 0.5 * ((L[4] + pL) * iL + (R[4] + pR) * iR);
        f[0] = rho * u; f[1] = rho * u * u + p; f[2] = rho * u * v; f[3] = rho * u * w; f[4] = rho * u * h;
    }
}

// RiemannSolvers_NS.f90:1251-1334 LxFRiemannSolver.
static void lxf(const Phys& p, int avg, double lambdaStab, const double* QL, const double* QR, const double* n,
                const double* t1, const double* t2, double* flux) {
    const double rhoL = QL[0], rhoR = QR[0];
    const double iL = 1.0 / rhoL, iR = 1.0 / rhoR;
    const double rhouL = QL[1] * n[0] + QL[2] * n[1] + QL[3] * n[2];
    const double rhouR = QR[1] * n[0] + QR[2] * n[1] + QR[3] * n[2];
    const double rhovL = QL[1] * t1[0] + QL[2] * t1[1] + QL[3] * t1[2];
    const double rhovR = QR[1] * t1[0] + QR[2] * t1[1] + QR[3] * t1[2];
    const double rhowL = QL[1] * t2[0] + QL[2] * t2[1] + QL[3] * t2[2];
    const double rhowR = QR[1] * t2[0] + QR[2] * t2[1] + QR[3] * t2[2];
    const double V2L = (rhouL * rhouL + rhovL * rhovL + rhowL * rhowL) * iL;
    const double V2R = (rhouR * rhouR + rhovR * rhovR + rhowR * rhowR) * iR;
    const double pL = p.gm1 * (QL[4] - 0.5 * V2L), pR = p.gm1 * (QR[4] - 0.5 * V2R);
    const double aL = std::sqrt(p.gamma * pL * iL), aR = std::sqrt(p.gamma * pR * iR);
    const double lambda = std::fmax(std::fabs(rhouL * iL) + aL, std::fabs(rhouR * iR) + aR);
    const double Lr[5] = {rhoL, rhouL, rhovL, rhowL, QL[4]};
    const double Rr[5] = {rhoR, rhouR, rhovR, rhowR, QR[4]};
    double f[5];
    average(p, avg, Lr, Rr, pL, pR, iL, iR, f);
    for (int v = 0; v < 5; ++v) f[v] = f[v] - lambdaStab * (0.5 * lambda * (Rr[v] - Lr[v]));
    flux[0] = f[0];
    for (int c = 0; c < 3; ++c) flux[1 + c] = n[c] * f[1] + t1[c] * f[2] + t2[c] * f[3];
    flux[4] = f[4];
}

// RiemannSolvers_NS.f90:1661-1762 RusanovRiemannSolver.
static void rusanov(const Phys& p, const double* QL, const double* QR, const double* n, double* flux) {
    const double g = p.gamma;
    const double rho = QL[0], rhou = QL[1], rhov = QL[2], rhow = QL[3], rhoe = QL[4];
    const double rhon = QR[0], rhoun = QR[1], rhovn = QR[2], rhown = QR[3], rhoen = QR[4];
    const double ul = rhou / rho, vl = rhov / rho, wl = rhow / rho;
    const double pleft = (g - 1.0) * (rhoe - 0.5 / rho * (rhou * rhou + rhov * rhov + rhow * rhow));
    const double ur = rhoun / rhon, vr = rhovn / rhon, wr = rhown / rhon;
    const double pright = (g - 1.0) * (rhoen - 0.5 / rhon * (rhoun * rhoun + rhovn * rhovn + rhown * rhown));
    const double ql = n[0] * ul + n[1] * vl + n[2] * wl;
    const double qr = n[0] * ur + n[1] * vr + n[2] * wr;
    const double hl = 0.5 * (ul * ul + vl * vl + wl * wl) + g / (g - 1.0) * pleft / rho;
    const double hr = 0.5 * (ur * ur + vr * vr + wr * wr) + g / (g - 1.0) * pright / rhon;
    const double ar = std::sqrt((g - 1.0) * (hr - 0.5 * (ur * ur + vr * vr + wr * wr)));
    const double al = std::sqrt((g - 1.0) * (hl - 0.5 * (ul * ul + vl * vl + wl * wl)));
    const double rql = rho * ql, rqr = rhon * qr;
    double f[5];
    f[0] = rql + rqr;
    f[1] = rql * ul + pleft * n[0] + rqr * ur + pright * n[0];
    f[2] = rql * vl + pleft * n[1] + rqr * vr + pright * n[1];
    f[3] = rql * wl + pleft * n[2] + rqr * wr + pright * n[2];
    f[4] = rql * hl + rqr * hr;
    const double smax = std::fmax(ar + std::fabs(qr), al + std::fabs(ql));
    for (int v = 0; v < 5; ++v) flux[v] = (f[v] - smax * (QR[v] - QL[v])) / 2.0;
}

// ---- the Roe family, matrix dissipation, viscous-NS and u-diss solvers (RiemannSolvers_NS.f90) ----
static void rotate_in(const double* Q, const double* n, const double* t1, const double* t2, double* r) {
    r[0] = Q[0];
    r[1] = Q[1] * n[0] + Q[2] * n[1] + Q[3] * n[2];
    r[2] = Q[1] * t1[0] + Q[2] * t1[1] + Q[3] * t1[2];
    r[3] = Q[1] * t2[0] + Q[2] * t2[1] + Q[3] * t2[2];
    r[4] = Q[4];
}
static void rotate_out(const double* f, const double* n, const double* t1, const double* t2, double* flux) {
    flux[0] = f[0];
    for (int c = 0; c < 3; ++c) flux[1 + c] = n[c] * f[1] + t1[c] * f[2] + t2[c] * f[3];
    flux[4] = f[4];
}

// VariableConversion_NS.f90:266-294 getPrimitiveVariables: [1/rho, u, v, w, p, T, a^2].
struct Prim {
    double irho, u, v, w, p, T, a2;
};
static Prim primitive(const Phys& ph, const double* U) {
    Prim V;
    V.irho = 1.0 / U[0];
    V.u = U[1] * V.irho; V.v = U[2] * V.irho; V.w = U[3] * V.irho;
    V.p = ph.gm1 * (U[4] - 0.5 * (V.u * U[1] + V.v * U[2] + V.w * U[3]));
    V.T = V.p * ph.gammaM2 * V.irho;
    V.a2 = ph.gamma * V.p * V.irho;
    return V;
}

// Van Leer's modification of Harten's entropy fix of the acoustic waves (RiemannSolvers_NS.f90:507-530).
static double entropy_fix(double lambda, double sL, double sR) {
    const double dl = std::fmax(sR - sL, 0.0);
    if (std::fabs(lambda) >= 2.0 * dl) return std::fabs(lambda);
    return lambda * lambda / (4.0 * dl) + dl;
}

// stab = sum_i 1/2 alpha_i |lambda_i| K_i with the Roe eigenvectors of (u, v, w, H, a), then
// flux = average - lambdaStab * stab in the face frame.
static void roe_stabilised(const Phys& ph, int avg, double lambdaStab, const double* L, const double* R, double pL,
                           double pR, double iL, double iR, double u, double v, double w, double V2, double H,
                           double a, const double* alpha, double* lambda, double* f) {
    (void)ph;
    const double K[5][5] = {{1.0, u - a, v, w, H - u * a},
                            {1.0, u, v, w, 0.5 * V2},
                            {0.0, 0.0, 1.0, 0.0, v},
                            {0.0, 0.0, 0.0, 1.0, w},
                            {1.0, u + a, v, w, H + u * a}};
    average(ph, avg, L, R, pL, pR, iL, iR, f);
    if (avg == DG_AVG_PIROZZOLI || avg == DG_AVG_KENNEDY_GRUBER) lambda[0] = lambda[4];
    double stab[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < 5; ++i)
        for (int c = 0; c < 5; ++c) stab[c] = stab[c] + 0.5 * alpha[i] * std::fabs(lambda[i]) * K[i][c];
    for (int c = 0; c < 5; ++c) f[c] = f[c] - lambdaStab * stab[c];
}

// :430-576 StdRoeRiemannSolver and :721-861 RoePikeRiemannSolver (Roe averages of getRoeVariables,
// VariableConversion_NS.f90:323-365; the projections differ).
static void std_roe(const Phys& ph, int avg, double lambdaStab, bool pike, const double* QL, const double* QR,
                    const double* n, const double* t1, const double* t2, double* flux) {
    double L[5], R[5];
    rotate_in(QL, n, t1, t2, L);
    rotate_in(QR, n, t1, t2, R);
    const Prim VL = primitive(ph, L), VR = primitive(ph, R);
    const double aL = std::sqrt(VL.a2), aR = std::sqrt(VR.a2);
    const double sL = std::sqrt(L[0]), sR = std::sqrt(R[0]);
    const double inv = 1.0 / (sL + sR);
    const double HL = (VL.p + L[4]) * VL.irho, HR = (VR.p + R[4]) * VR.irho;
    const double rho = sL * sR;
    const double u = (sL * VL.u + sR * VR.u) * inv, v = (sL * VL.v + sR * VR.v) * inv, w = (sL * VL.w + sR * VR.w) * inv;
    const double H = (sL * HL + sR * HR) * inv;
    const double V2 = u * u + v * v + w * w;
    const double a = std::sqrt(ph.gm1 * (H - 0.5 * V2));
    double lambda[5] = {u - a, u, u, u, u + a};
    double alpha[5];
    if (!pike) {
        double dQ[5];
        for (int q = 0; q < 5; ++q) dQ[q] = R[q] - L[q];
        alpha[2] = dQ[2] - v * dQ[0];
        alpha[3] = dQ[3] - w * dQ[0];
        dQ[4] = dQ[4] - alpha[2] * v - alpha[3] * w;
        alpha[1] = ph.gm1 * (dQ[0] * (H - u * u) + u * dQ[1] - dQ[4]) / (a * a);
        alpha[0] = 0.5 * (dQ[0] * lambda[4] - dQ[1] - a * alpha[1]) / a;
        alpha[4] = dQ[0] - alpha[0] - alpha[1];
    } else {
        const double dp = VR.p - VL.p, du = VR.u - VL.u;
        alpha[0] = (dp - rho * a * du) / (2.0 * a * a);
        alpha[1] = (QR[0] - QL[0]) - dp / (a * a);
        alpha[2] = rho * (VR.v - VL.v);
        alpha[3] = rho * (VR.w - VL.w);
        alpha[4] = (dp + rho * a * du) / (2.0 * a * a);
    }
    lambda[0] = entropy_fix(lambda[0], VL.u - aL, VR.u - aR);
    lambda[4] = entropy_fix(lambda[4], VL.u + aL, VR.u + aR);
    double f[5];
    roe_stabilised(ph, avg, lambdaStab, L, R, VL.p, VR.p, VL.irho, VR.irho, u, v, w, V2, H, a, alpha, lambda, f);
    rotate_out(f, n, t1, t2, flux);
}

// Face-frame states and Roe-Pike averages written with 1/sqrt(rho) (the form of :863-1058 and
// :1060-1247).
struct RoePikeState {
    double L[5], R[5], iL, iR, uL, vL, wL, uR, vR, wR, pL, pR, aL, aR, rho, u, v, w, H, V2, a;
};
static RoePikeState roe_pike_state(const Phys& ph, const double* QL, const double* QR, const double* n,
                                   const double* t1, const double* t2) {
    RoePikeState s;
    rotate_in(QL, n, t1, t2, s.L);
    rotate_in(QR, n, t1, t2, s.R);
    const double rhoL = s.L[0], rhoR = s.R[0];
    s.iL = 1.0 / rhoL; s.iR = 1.0 / rhoR;
    const double sL = std::sqrt(rhoL), sR = std::sqrt(rhoR);
    const double isL = 1.0 / sL, isR = 1.0 / sR;
    const double inv = 1.0 / (sL + sR);
    s.uL = s.L[1] * s.iL; s.uR = s.R[1] * s.iR;
    s.vL = s.L[2] * s.iL; s.vR = s.R[2] * s.iR;
    s.wL = s.L[3] * s.iL; s.wR = s.R[3] * s.iR;
    const double rV2L = (s.uL * s.uL + s.vL * s.vL + s.wL * s.wL) * rhoL;
    const double rV2R = (s.uR * s.uR + s.vR * s.vR + s.wR * s.wR) * rhoR;
    const double rHL = ph.gamma * s.L[4] - 0.5 * ph.gm1 * rV2L, rHR = ph.gamma * s.R[4] - 0.5 * ph.gm1 * rV2R;
    s.pL = ph.gm1 * (s.L[4] - 0.5 * rV2L);
    s.pR = ph.gm1 * (s.R[4] - 0.5 * rV2R);
    s.aL = std::sqrt(ph.gamma * s.pL * s.iL);
    s.aR = std::sqrt(ph.gamma * s.pR * s.iR);
    s.rho = sL * sR;
    s.u = (isL * s.L[1] + isR * s.R[1]) * inv;
    s.v = (isL * s.L[2] + isR * s.R[2]) * inv;
    s.w = (isL * s.L[3] + isR * s.R[3]) * inv;
    s.H = (isL * rHL + isR * rHR) * inv;
    s.V2 = s.u * s.u + s.v * s.v + s.w * s.w;
    s.a = std::sqrt(ph.gm1 * (s.H - 0.5 * s.V2));
    return s;
}

// :863-1058 LowDissipationRoeRiemannSolver (L2Roe: velocity jumps scaled by min(1, max(ML, MR))).
static void low_diss_roe(const Phys& ph, int avg, double lambdaStab, const double* QL, const double* QR,
                         const double* n, const double* t1, const double* t2, double* flux) {
    const RoePikeState s = roe_pike_state(ph, QL, QR, n, t1, t2);
    const double u = s.u, a = s.a, rho = s.rho;
    double lambda[5] = {u - a, u, u, u, u + a};
    const double ML = std::fabs(s.uL) / s.aL, MR = std::fabs(s.uR) / s.aR;
    const double z = std::fmin(1.0, std::fmax(ML, MR));
    const double du = z * (s.uR - s.uL), dv = z * (s.vR - s.vL), dw = z * (s.wR - s.wL), dp = s.pR - s.pL;
    double alpha[5];
    alpha[0] = (dp - rho * a * du) / (2.0 * a * a);
    alpha[1] = (s.R[0] - s.L[0]) - dp / (a * a);
    alpha[2] = rho * dv;
    alpha[3] = rho * dw;
    alpha[4] = (dp + rho * a * du) / (2.0 * a * a);
    lambda[0] = entropy_fix(lambda[0], s.uL - s.aL, s.uR - s.aR);
    lambda[4] = entropy_fix(lambda[4], s.uL + s.aL, s.uR + s.aR);
    double f[5];
    roe_stabilised(ph, avg, lambdaStab, s.L, s.R, s.pL, s.pR, s.iL, s.iR, s.u, s.v, s.w, s.V2, s.H, a, alpha, lambda,
                   f);
    rotate_out(f, n, t1, t2, flux);
}

// :1060-1247 ViscousNSRiemannSolver: the average plus a dissipation shaped like the NS viscous terms
// of the velocity and temperature jumps, scaled by the largest wave speed (added in the Cartesian frame).
static void viscous_ns(const Phys& ph, int avg, double lambdaStab, const double* QL, const double* QR, const double* n,
                       const double* t1, const double* t2, double* flux) {
    const RoePikeState s = roe_pike_state(ph, QL, QR, n, t1, t2);
    double lambda[5] = {s.u - s.a, s.u, s.u, s.u, s.u + s.a};
    lambda[0] = entropy_fix(lambda[0], s.uL - s.aL, s.uR - s.aR);
    lambda[4] = entropy_fix(lambda[4], s.uL + s.aL, s.uR + s.aR);
    double f[5];
    average(ph, avg, s.L, s.R, s.pL, s.pR, s.iL, s.iR, f);
    if (avg == DG_AVG_PIROZZOLI || avg == DG_AVG_KENNEDY_GRUBER) lambda[0] = lambda[4];
    const double uL = QL[1] / QL[0], uR = QR[1] / QR[0];
    const double vL = QL[2] / QL[0], vR = QR[2] / QR[0];
    const double wL = QL[3] / QL[0], wR = QR[3] / QR[0];
    const double u = 0.5 * (uL + uR), v = 0.5 * (vL + vR), w = 0.5 * (wL + wR);
    const double divV = (uR - uL) * n[0] + (vR - vL) * n[1] + (wR - wL) * n[2];
    double tau[3][3];
    tau[0][0] = 2.0 * (uR - uL) * n[0] - (1.0 / 3.0) * divV;
    tau[1][1] = 2.0 * (vR - vL) * n[1] - (1.0 / 3.0) * divV;
    tau[2][2] = 2.0 * (wR - wL) * n[2] - (1.0 / 3.0) * divV;
    tau[0][1] = (uR - uL) * n[1] + (vR - vL) * n[0];
    tau[0][2] = (uR - uL) * n[2] + (wR - wL) * n[0];
    tau[1][2] = (vR - vL) * n[2] + (wR - wL) * n[1];
    tau[1][0] = tau[0][1]; tau[2][0] = tau[0][2]; tau[2][1] = tau[1][2];
    const double kappa = 1.0 / (3.0 / 4.0 * ph.gm1 * (ph.Mach * ph.Mach));  // FluidData_NS.f90:173-181, Pr = 3/4
    const double TL = s.pL * ph.gammaM2 / s.L[0], TR = s.pR * ph.gammaM2 / s.R[0];  // :156-164
    double lmax = 0.0;
    for (int i = 0; i < 5; ++i) lmax = std::fmax(lmax, std::fabs(lambda[i]));
    double stab[5];
    stab[0] = 0.0;
    for (int r = 0; r < 3; ++r) stab[1 + r] = lmax * (tau[r][0] * n[0] + tau[r][1] * n[1] + tau[r][2] * n[2]);
    stab[4] = lmax * ((u * tau[0][0] + v * tau[0][1] + w * tau[0][2]) * n[0] +
                      (u * tau[1][0] + v * tau[1][1] + w * tau[1][2]) * n[1] +
                      (u * tau[2][0] + v * tau[2][1] + w * tau[2][2]) * n[2] + kappa * (TR - TL));
    rotate_out(f, n, t1, t2, flux);
    for (int c = 0; c < 5; ++c) flux[c] = flux[c] - lambdaStab * stab[c];
}

// VariableConversion_NS.f90:211-237 NSGradientVariables_ENTROPY.
static void entropy_variables(const Phys& ph, const double* Q, double* U) {
    const double irho = 1.0 / Q[0];
    const double rV2 = (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]) * irho;
    const double p = ph.gm1 * (Q[4] - 0.5 * rV2);
    const double ip = 1.0 / p;
    U[0] = (ph.gamma - (std::log(p) - ph.gamma * std::log(Q[0]))) * (1.0 / (1.4 - 1.0)) - 0.5 * rV2 * ip;
    U[1] = Q[1] * ip;
    U[2] = Q[2] * ip;
    U[3] = Q[3] * ip;
    U[4] = -Q[0] * ip;
}

// :578-719 MatrixDissipationRiemannSolver: dissipation of the entropy-variable jump with the
// eigenvectors and scalings of the logarithmic-mean states.
static void matrix_diss(const Phys& ph, int avg, double lambdaStab, const double* QL, const double* QR,
                        const double* n, const double* t1, const double* t2, double* flux) {
    double L[5], R[5], EVL[5], EVR[5];
    rotate_in(QL, n, t1, t2, L);
    rotate_in(QR, n, t1, t2, R);
    entropy_variables(ph, L, EVL);
    entropy_variables(ph, R, EVR);
    const double iL = 1.0 / L[0], iR = 1.0 / R[0];
    const double uL = L[1] * iL, uR = R[1] * iR, vL = L[2] * iL, vR = R[2] * iR, wL = L[3] * iL, wR = R[3] * iR;
    const double vtL = uL * uL + vL * vL + wL * wL, vtR = uR * uR + vR * vR + wR * wR;
    const double pL = ph.gm1 * (L[4] - 0.5 * L[0] * vtL), pR = ph.gm1 * (R[4] - 0.5 * R[0] * vtR);
    const double betaL = -0.5 * EVL[4], betaR = -0.5 * EVR[4];
    const double betaLog = log_mean(betaL, betaR), rhoLog = log_mean(L[0], R[0]);
    const double pMean = 0.5 * (L[0] + R[0]) / (betaL + betaR);
    const double a = std::sqrt(ph.gamma * pMean / rhoLog);
    const double u = 0.5 * (uL + uR), v = 0.5 * (vL + vR), w = 0.5 * (wL + wR);
    const double V2 = 2.0 * (u * u + v * v + w * w) - 0.5 * (vtL + vtR);
    const double h = 0.5 * (ph.gamma / ph.gm1 / betaLog + V2);
    double lambda[5] = {std::fabs(u - a), std::fabs(u), std::fabs(u), std::fabs(u), std::fabs(u + a)};
    const double Rm[5][5] = {{1.0, u - a, v, w, h - u * a},
                             {1.0, u, v, w, 0.5 * V2},
                             {0.0, 0.0, 1.0, 0.0, v},
                             {0.0, 0.0, 0.0, 1.0, w},
                             {1.0, u + a, v, w, h + u * a}};  // Rm[j][i] = R1(i, j)
    const double T1 = 0.5 * rhoLog * (1.0 / ph.gamma);
    const double T[5] = {T1, 2.0 * ((1.4 - 1.0) / (2.0 * 1.4)) * rhoLog, pMean, pMean, T1};
    double f[5];
    average(ph, avg, L, R, pL, pR, iL, iR, f);
    if (avg == DG_AVG_PIROZZOLI || avg == DG_AVG_KENNEDY_GRUBER) lambda[0] = lambda[4];
    double stab[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j)
            for (int k = 0; k < 5; ++k)
                stab[i] = stab[i] + 0.5 * Rm[j][i] * lambda[j] * T[j] * Rm[j][k] * (EVR[k] - EVL[k]);
    for (int c = 0; c < 5; ++c) f[c] = f[c] - lambdaStab * stab[c];
    rotate_out(f, n, t1, t2, flux);
}

// :1336-1425 u_dissRiemannSolver: the LxF form with lambda = max(|u_L|, |u_R|) (no sound speed).
static void u_diss(const Phys& p, int avg, double lambdaStab, const double* QL, const double* QR, const double* n,
                   const double* t1, const double* t2, double* flux) {
    double L[5], R[5];
    rotate_in(QL, n, t1, t2, L);
    rotate_in(QR, n, t1, t2, R);
    const double iL = 1.0 / L[0], iR = 1.0 / R[0];
    const double V2L = (L[1] * L[1] + L[2] * L[2] + L[3] * L[3]) * iL;
    const double V2R = (R[1] * R[1] + R[2] * R[2] + R[3] * R[3]) * iR;
    const double pL = p.gm1 * (L[4] - 0.5 * V2L), pR = p.gm1 * (R[4] - 0.5 * V2R);
    const double lambda = std::fmax(std::fabs(L[1] * iL), std::fabs(R[1] * iR));
    double f[5];
    average(p, avg, L, R, pL, pR, iL, iR, f);
    for (int v = 0; v < 5; ++v) f[v] = f[v] - lambdaStab * (0.5 * lambda * (R[v] - L[v]));
    rotate_out(f, n, t1, t2, flux);
}

// RiemannSolvers_NS.f90:2085-2145 StandardDG_TwoPointFlux and :2369-2437 Pirozzoli_TwoPointFlux.
static void two_point(const Phys& p, int avg, const double* QL, const double* QR, const double* JaL, const double* JaR,
                      double* fs) {
    const double iL = 1.0 / QL[0], iR = 1.0 / QR[0];
    const double uL = iL * QL[1], uR = iR * QR[1], vL = iL * QL[2], vR = iR * QR[2], wL = iL * QL[3], wR = iR * QR[3];
    const double pL = p.gm1 * (QL[4] - 0.5 * (QL[1] * uL + QL[2] * vL + QL[3] * wL));
    const double pR = p.gm1 * (QR[4] - 0.5 * (QR[1] * uR + QR[2] * vR + QR[3] * wR));
    double f[5], g[5], h[5];
    if (avg == DG_AVG_STANDARD) {
        const double Ja[3] = {JaL[0] + JaR[0], JaL[1] + JaR[1], JaL[2] + JaR[2]};
        f[0] = QL[1] + QR[1]; f[1] = QL[1] * uL + QR[1] * uR + pL + pR; f[2] = QL[1] * vL + QR[1] * vR;
        f[3] = QL[1] * wL + QR[1] * wR; f[4] = uL * (QL[4] + pL) + uR * (QR[4] + pR);
        g[0] = QL[2] + QR[2]; g[1] = QL[2] * uL + QR[2] * uR; g[2] = QL[2] * vL + QR[2] * vR + pL + pR;
        g[3] = QL[2] * wL + QR[2] * wR; g[4] = vL * (QL[4] + pL) + vR * (QR[4] + pR);
        h[0] = QL[3] + QR[3]; h[1] = QL[3] * uL + QR[3] * uR; h[2] = QL[3] * vL + QR[3] * vR;
        h[3] = QL[3] * wL + QR[3] * wR + pL + pR; h[4] = wL * (QL[4] + pL) + wR * (QR[4] + pR);
        for (int v = 0; v < 5; ++v) fs[v] = 0.25 * (f[v] * Ja[0] + g[v] * Ja[1] + h[v] * Ja[2]);
        return;
    }
    const double Ja[3] = {0.5 * (JaL[0] + JaR[0]), 0.5 * (JaL[1] + JaR[1]), 0.5 * (JaL[2] + JaR[2])};
    if (avg == DG_AVG_DUCROS) {  // :2231-2294
        const double su[3] = {uL + uR, vL + vR, wL + wR};
        double* F[3] = {f, g, h};
        for (int d = 0; d < 3; ++d) {
            F[d][0] = 0.25 * (QL[0] + QR[0]) * su[d];
            F[d][1] = 0.25 * (QL[1] + QR[1]) * su[d];
            F[d][2] = 0.25 * (QL[2] + QR[2]) * su[d];
            F[d][3] = 0.25 * (QL[3] + QR[3]) * su[d];
            F[d][1 + d] += 0.5 * (pL + pR);
            F[d][4] = 0.25 * (QL[4] + pL + QR[4] + pR) * su[d];
        }
    } else if (avg == DG_AVG_MORINISHI) {  // :2147-2229
        const double hL = p.gamma / p.gm1 * pL, hR = p.gamma / p.gm1 * pR;
        const double velL[3] = {uL, vL, wL}, velR[3] = {uR, vR, wR};
        double* F[3] = {f, g, h};
        for (int d = 0; d < 3; ++d) {
            const double mL = QL[1 + d], mR = QR[1 + d];
            F[d][0] = 0.5 * (mL + mR);
            F[d][1] = 0.25 * (mL + mR) * (uL + uR);
            F[d][2] = 0.25 * (mL + mR) * (vL + vR);
            F[d][3] = 0.25 * (mL + mR) * (wL + wR);
            F[d][1 + d] += 0.5 * (pL + pR);
            F[d][4] = 0.5 * (velL[d] * hL + velR[d] * hR) + 0.25 * (mL * uL + mR * uR) * (uL + uR) +
                      0.25 * (mL * vL + mR * vR) * (vL + vR) + 0.25 * (mL * wL + mR * wR) * (wL + wR) -
                      0.25 * (mL * uL * uL + mR * uR * uR) - 0.25 * (mL * vL * vL + mR * vR * vR) -
                      0.25 * (mL * wL * wL + mR * wR * wR);
        }
    } else if (avg == DG_AVG_KENNEDY_GRUBER) {  // :2296-2367
        const double rho = 0.5 * (QL[0] + QR[0]), u = 0.5 * (uL + uR), v = 0.5 * (vL + vR), w = 0.5 * (wL + wR);
        const double pp = 0.5 * (pL + pR), e = 0.5 * (QL[4] * iL + QR[4] * iR);
        const double um[3] = {u, v, w};
        double* F[3] = {f, g, h};
        for (int d = 0; d < 3; ++d) {
            F[d][0] = rho * um[d];
            F[d][1] = rho * um[d] * u;
            F[d][2] = rho * um[d] * v;
            F[d][3] = rho * um[d] * w;
            F[d][1 + d] += pp;
            F[d][4] = rho * um[d] * e + pp * um[d];
        }
    } else if (avg == DG_AVG_ENTROPY_CONSERVING || avg == DG_AVG_CHANDRASEKAR) {
        // :2439-2558 EntropyConserving_TwoPointFlux, :2560-2641 Chandrasekar_TwoPointFlux: the averaged
        // states of the two-point average, fluxes in all three directions.
        double rho, u, v, w, pp, hh;
        if (avg == DG_AVG_ENTROPY_CONSERVING) {
            double zL[5], zR[5], zA[5];
            zL[4] = std::sqrt(QL[0] * pL); zR[4] = std::sqrt(QR[0] * pR);
            zL[0] = QL[0] / zL[4]; zR[0] = QR[0] / zR[4];
            zL[1] = zL[0] * uL; zR[1] = zR[0] * uR;
            zL[2] = zL[0] * vL; zR[2] = zR[0] * vR;
            zL[3] = zL[0] * wL; zR[3] = zR[0] * wR;
            for (int q = 0; q < 5; ++q) zA[q] = 0.5 * (zL[q] + zR[q]);
            const double inv1 = 1.0 / zA[0];
            const double z1Log = log_mean(zL[0], zR[0]), z5Log = log_mean(zL[4], zR[4]);
            rho = zA[0] * z5Log;
            u = zA[1] * inv1; v = zA[2] * inv1; w = zA[3] * inv1; pp = zA[4] * inv1;
            const double p2 = ((p.gamma + 1.0) / 2.0 * z5Log / z1Log + (p.gamma - 1.0) / 2.0 * pp) * (1.0 / p.gamma);
            hh = p.gamma / p.gm1 * p2 / rho + 0.5 * (u * u + v * v + w * w);
        } else {
            const double betaL = 0.5 * QL[0] / pL, betaR = 0.5 * QR[0] / pR;
            const double betaLog = log_mean(betaL, betaR);
            rho = log_mean(QL[0], QR[0]);
            u = 0.5 * (uL + uR); v = 0.5 * (vL + vR); w = 0.5 * (wL + wR);
            pp = 0.5 * (QL[0] + QR[0]) / (betaL + betaR);
            hh = 0.5 / (betaLog * p.gm1) - 0.5 * (0.5 * ((uL * uL + vL * vL + wL * wL) + (uR * uR + vR * vR + wR * wR))) +
                 pp / rho + u * u + v * v + w * w;
        }
        const double ff[5] = {rho * u, rho * u * u + pp, rho * u * v, rho * u * w, rho * u * hh};
        const double gg[5] = {rho * v, rho * v * u, rho * v * v + pp, rho * v * w, rho * v * hh};
        const double hhh[5] = {rho * w, rho * w * u, rho * w * v, rho * w * w + pp, rho * w * hh};
        for (int q = 0; q < 5; ++q) fs[q] = ff[q] * Ja[0] + gg[q] * Ja[1] + hhh[q] * Ja[2];
        return;
    } else {  // Pirozzoli, :2369-2437
        const double rho = 0.5 * (QL[0] + QR[0]), u = 0.5 * (uL + uR), v = 0.5 * (vL + vR), w = 0.5 * (wL + wR);
        const double pp = 0.5 * (pL + pR);
        const double hh = 0.5 * ((QL[4] + pL) * iL + (QR[4] + pR) * iR);
        const double ff[5] = {rho * u, rho * u * u + pp, rho * u * v, rho * u * w, rho * u * hh};
        const double gg[5] = {rho * v, rho * v * u, rho * v * v + pp, rho * v * w, rho * v * hh};
        const double hhh[5] = {rho * w, rho * w * u, rho * w * v, rho * w * w + pp, rho * w * hh};
        for (int q = 0; q < 5; ++q) fs[q] = ff[q] * Ja[0] + gg[q] * Ja[1] + hhh[q] * Ja[2];
        return;
    }
    for (int q = 0; q < 5; ++q) fs[q] = f[q] * Ja[0] + g[q] * Ja[1] + h[q] * Ja[2];
}

// Convergence/SETUP/ProblemFile.f90:31-133 state_source_in_point (manufactured solution).
static void mms_point(double x, double y, double z, double t, double gm1, double gMa2, double mu, double kap,
                      double* Q, double* S, double* QDot) {
    const double c_u = 1.0, c_v = 2.0, c_w = -c_u - c_v;
    const double Ssu = 0.381923076923077;
    const double arg = PI * (x + y + z - 2.0 * t), dargdx = PI, dargdt = -2.0 * PI;
    const double rho = 2.0 + 0.1 * std::sin(arg);
    const double u = c_u * rho - 1.0, v = c_v * rho - 4.0, w = c_w * rho + 5.0, e = rho;
    const double vtot = u * u + v * v + w * w;
    const double p = gm1 * (rho * e - 0.5 * rho * vtot);
    const double Temp = gMa2 * gm1 * (e - 0.5 * vtot);
    const double suther = (1.0 + Ssu) / (Temp + Ssu) * Temp * std::sqrt(Temp);
    const double dsutherdT = 1.5 * suther / Temp - suther / (Ssu + Temp);
    Q[0] = rho; Q[1] = rho * u; Q[2] = rho * v; Q[3] = rho * w; Q[4] = rho * e;
    const double rho_t = 0.1 * dargdt * std::cos(arg);
    const double u_t = c_u * rho_t, v_t = c_v * rho_t, w_t = c_w * rho_t, e_t = rho_t;
    QDot[0] = rho_t; QDot[1] = rho_t * u + rho * u_t; QDot[2] = rho_t * v + rho * v_t;
    QDot[3] = rho_t * w + rho * w_t; QDot[4] = rho_t * e + rho * e_t;
    double rho_x[3], u_x[3], v_x[3], w_x[3], e_x[3], p_x[3], T_x[3];
    for (int i = 0; i < 3; ++i) {
        rho_x[i] = 0.1 * dargdx * std::cos(arg);
        u_x[i] = c_u * rho_x[i]; v_x[i] = c_v * rho_x[i]; w_x[i] = c_w * rho_x[i]; e_x[i] = rho_x[i];
    }
    for (int i = 0; i < 3; ++i) {
        p_x[i] = gm1 * rho_x[i] * (e - 0.5 * vtot) + gm1 * rho * (e_x[i] - u * u_x[i] - v * v_x[i] - w * w_x[i]);
        T_x[i] = gMa2 * gm1 * (e_x[i] - u * u_x[i] - v * v_x[i] - w * w_x[i]);
    }
    const double div_v = u_x[0] + v_x[1] + w_x[2];
    double gu[3][3], tau[3][3];  // gu[i][j] = grad_u(i,j)
    for (int i = 0; i < 3; ++i) { gu[i][0] = u_x[i]; gu[i][1] = v_x[i]; gu[i][2] = w_x[i]; }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            tau[i][j] = mu * suther * (gu[i][j] + gu[j][i] - 2.0 * div_v * (i == j ? 1.0 : 0.0) / 3.0);
    double rxx[3][3], uxx[3][3], vxx[3][3], wxx[3][3], exx[3][3], Txx[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            rxx[i][j] = -0.1 * (dargdx * dargdx) * std::sin(arg);
            uxx[i][j] = c_u * rxx[i][j]; vxx[i][j] = c_v * rxx[i][j]; wxx[i][j] = c_w * rxx[i][j]; exx[i][j] = rxx[i][j];
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            Txx[i][j] = gMa2 * gm1 * (exx[i][j] - u_x[i] * u_x[j] - v_x[i] * v_x[j] - w_x[i] * w_x[j] - u * uxx[i][j] -
                                      v * vxx[i][j] - w * wxx[i][j]);
    double dt[3];
    const double tr[3] = {uxx[0][0] + uxx[1][1] + uxx[2][2], vxx[0][0] + vxx[1][1] + vxx[2][2], wxx[0][0] + wxx[1][1] + wxx[2][2]};
    const double gd[3] = {uxx[0][0] + vxx[1][0] + wxx[2][0], uxx[1][0] + vxx[1][1] + wxx[1][2], uxx[0][2] + vxx[1][2] + wxx[2][2]};
    for (int j = 0; j < 3; ++j) dt[j] = uxx[0][j] + vxx[1][j] + wxx[2][j] + tr[j] - (2.0 / 3.0) * gd[j];
    for (int j = 0; j < 3; ++j) dt[j] = mu * suther * dt[j];
    for (int i = 0; i < 3; ++i) {
        double mt = 0.0;
        for (int j = 0; j < 3; ++j) mt += tau[i][j] * T_x[j];
        dt[i] = dt[i] + (dsutherdT / suther) * mt;
    }
    double sgt = 0.0;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) sgt += gu[i][j] * tau[i][j];
    const double visc_work = sgt + u * dt[0] + v * dt[1] + w * dt[2];
    const double heat = kap * dsutherdT * (T_x[0] * T_x[0] + T_x[1] * T_x[1] + T_x[2] * T_x[2]) +
                        kap * suther * (Txx[0][0] + Txx[1][1] + Txx[2][2]);
    S[0] = rho_t + u * rho_x[0] + v * rho_x[1] + w * rho_x[2] + rho * div_v;
    S[1] = u * S[0] + rho * u_t + rho * u * u_x[0] + rho * v * u_x[1] + rho * w * u_x[2] + p_x[0] - dt[0];
    S[2] = v * S[0] + rho * v_t + rho * u * v_x[0] + rho * v * v_x[1] + rho * w * v_x[2] + p_x[1] - dt[1];
    S[3] = w * S[0] + rho * w_t + rho * u * w_x[0] + rho * v * w_x[1] + rho * w * w_x[2] + p_x[2] - dt[2];
    S[4] = e * S[0] + rho * e_t + rho * (u * e_x[0] + v * e_x[1] + w * e_x[2]) + p * div_v + u * p_x[0] + v * p_x[1] +
           w * p_x[2] - visc_work - heat;
}

// LambVector/SETUP/ProblemFile.f90:377-423 UserDefinedSourceTermNS, for the manufactured state of
// :8-27 (rho = 3 + sin(phi) e^t, u = w = cos(phi) e^-t, v = sin(phi) e^-t, E = rho |u|^2/2 + 1,
// phi = x + y + z). The source is dQ/dt + div(F_inviscid) - div(F_viscous)/Re with the constant
// viscosity mu = refValues%mu and kappa = mu * mu_to_kappa it is defined with. Written here in
// tensor form, term by term (d_i of every flux column by the product rule); every field depends
// on phi only, so d_i f = f' and d_i d_l f = f'' for all i, l.
static void lamb_point(double x, double y, double z, double t, double gm1, double gMa2, double mu_ref,
                       double kap_ref, double Re, double* S) {
    const double phi = x + y + z;
    const double sn = std::sin(phi), cs = std::cos(phi), et = std::exp(t), emt = std::exp(-t);
    const double rho = 3.0 + sn * et, rho_t = sn * et, rho_d = cs * et, rho_dd = -sn * et;
    const double V[3] = {cs * emt, sn * emt, cs * emt};
    const double V_t[3] = {-cs * emt, -sn * emt, -cs * emt};
    const double V_d[3] = {-sn * emt, cs * emt, -sn * emt};
    const double V_dd[3] = {-cs * emt, -sn * emt, -cs * emt};
    const double q2 = V[0] * V[0] + V[1] * V[1] + V[2] * V[2];
    const double q2_t = 2.0 * (V[0] * V_t[0] + V[1] * V_t[1] + V[2] * V_t[2]);
    const double q2_d = 2.0 * (V[0] * V_d[0] + V[1] * V_d[1] + V[2] * V_d[2]);
    const double q2_dd = 2.0 * (V_d[0] * V_d[0] + V_d[1] * V_d[1] + V_d[2] * V_d[2] + V[0] * V_dd[0] +
                                V[1] * V_dd[1] + V[2] * V_dd[2]);
    const double E = rho * q2 / 2.0 + 1.0;
    const double E_t = rho_t * q2 / 2.0 + rho * q2_t / 2.0;
    const double E_d = rho_d * q2 / 2.0 + rho * q2_d / 2.0;
    const double E_dd = rho_dd * q2 / 2.0 + rho_d * q2_d + rho * q2_dd / 2.0;
    const double p = gm1 * (rho * E - 0.5 * rho * q2);
    const double p_d = gm1 * (rho_d * E + rho * E_d - 0.5 * (rho_d * q2 + rho * q2_d));
    const double T_dd = gm1 * gMa2 * (E_dd - 0.5 * q2_dd);
    // d_i(u_i): the divergence and its derivative
    const double div = V_d[0] + V_d[1] + V_d[2], div_d = V_dd[0] + V_dd[1] + V_dd[2];
    // time derivatives of Q
    double dQ[5] = {rho_t, rho_t * V[0] + rho * V_t[0], rho_t * V[1] + rho * V_t[1], rho_t * V[2] + rho * V_t[2],
                    rho_t * E + rho * E_t};
    // inviscid divergence
    double dF[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < 3; ++i) {
        dF[0] += rho_d * V[i] + rho * V_d[i];
        for (int j = 0; j < 3; ++j)
            dF[1 + j] += rho_d * V[j] * V[i] + rho * V_d[j] * V[i] + rho * V[j] * V_d[i] + (i == j ? p_d : 0.0);
        dF[4] += (rho_d * E + rho * E_d + p_d) * V[i] + (rho * E + p) * V_d[i];
    }
    // viscous divergence: tau_ji = mu (d_i u_j + d_j u_i - 2/3 delta_ij div u)
    double dG[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) {
            const double tau = mu_ref * (V_d[j] + V_d[i] - (i == j ? 2.0 / 3.0 * div : 0.0));
            const double tau_d = mu_ref * (V_dd[j] + V_dd[i] - (i == j ? 2.0 / 3.0 * div_d : 0.0));
            dG[1 + j] += tau_d;
            dG[4] += tau_d * V[j] + tau * V_d[j];
        }
        dG[4] += kap_ref * T_dd;
    }
    for (int q = 0; q < 5; ++q) S[q] = dQ[q] + dF[q] - dG[q] / Re;
}

// ---------------------------------------------------------------- boundary conditions --------
// physics/common/{NoSlipWallBC,FreeSlipWallBC,InflowBC,OutflowBC}.f90 (NAVIERSTOKES parts) and
// GenericBoundaryConditionClass.f90:243-291 (the default gradient variables and Neumann flux).
static double wall_type(const dg_boundary& b) { return b.isothermal ? 1.0 : 0.0; }

// FlowState: the external state of the Riemann problem at a boundary point.
static void bc_state(const Phys& p, const dg_boundary& b, const double* n, double* Q) {
    switch (b.type) {
        case DG_BC_NO_SLIP_WALL: {  // NoSlipWallBC.f90:265-296
            for (int c = 0; c < 3; ++c) Q[1 + c] = 2.0 * Q[0] * b.wall_velocity[c] - Q[1 + c];
            Q[4] = Q[4] + wall_type(b) * (Q[0] * b.wall_temperature / (p.gammaM2 * p.gm1) - Q[4]);
            break;
        }
        case DG_BC_FREE_SLIP_WALL: {  // FreeSlipWallBC.f90:249-286
            const double qn = n[0] * Q[1] + n[1] * Q[2] + n[2] * Q[3];
            for (int c = 0; c < 3; ++c) Q[1 + c] = Q[1 + c] - 2.0 * qn * n[c];
            const double pa = Q[0] * b.wall_temperature / p.gammaM2;
            Q[4] = Q[4] + wall_type(b) * (pa / p.gm1 + 0.5 * (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]) / Q[0] - Q[4]);
            break;
        }
        case DG_BC_INFLOW: {  // InflowBC.f90:363-406 (no turbulence intensity)
            Q[0] = b.rho;
            Q[1] = Q[0] * b.u;
            Q[2] = Q[0] * b.v;
            Q[3] = Q[0] * b.w;
            Q[4] = b.p / (p.gamma - 1.0) + 0.5 * Q[0] * (b.u * b.u + b.v * b.v + b.w * b.w);
            break;
        }
        default: {  // OutflowBC.f90:226-288
            double qn = (n[0] * Q[1] + n[1] * Q[2] + n[2] * Q[3]) / Q[0];
            const double tx = Q[1] / Q[0] - qn * n[0], ty = Q[2] / Q[0] - qn * n[1], tz = Q[3] / Q[0] - qn * n[2];
            const double pr = p.gm1 * (Q[4] - 0.5 * (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]) / Q[0]);
            const double a2 = p.gamma * pr / Q[0];
            double a = std::sqrt(a2);
            if (std::fabs(qn / a) <= 1.0) {
                const double rPlus = qn + 2.0 * a / p.gm1;
                const double ent = pr - a2 * Q[0];
                const double rho = -(ent - b.pressure) / a2;
                a = std::sqrt(p.gamma * b.pressure / rho);
                qn = rPlus - 2.0 * a / p.gm1;
                const double u = tx + qn * n[0], v = ty + qn * n[1], w = tz + qn * n[2];
                Q[0] = rho;
                Q[1] = rho * u;
                Q[2] = rho * v;
                Q[3] = rho * w;
                Q[4] = b.pressure / p.gm1 + 0.5 * rho * (u * u + v * v + w * w);
            }
            break;
        }
    }
}

// FlowGradVars: U (in: the interior gradient variables, out: U* at the boundary).
static void bc_gradvars(const Phys& p, const dg_boundary& b, const double* n, const double* Q, double* U) {
    double Qa[5];
    switch (b.type) {
        case DG_BC_NO_SLIP_WALL: {  // NoSlipWallBC.f90:298-337
            const double invRho = 1.0 / Q[0];
            const double e_int = invRho * (Q[4] - 0.5 * invRho * (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]));
            const double ewall = b.wall_temperature / (p.gm1 * p.gammaM2);
            const double wt = wall_type(b);
            const double* vw = b.wall_velocity;
            Qa[0] = Q[0];
            for (int c = 0; c < 3; ++c) Qa[1 + c] = Q[0] * vw[c];
            Qa[4] = Q[0] * ((1.0 - wt) * e_int + wt * ewall + 0.5 * (vw[0] * vw[0] + vw[1] * vw[1] + vw[2] * vw[2]));
            const double U1 = U[0];
            gradient_variables(p, Qa, U);
            U[0] = U1;
            return;
        }
        case DG_BC_FREE_SLIP_WALL: {  // FreeSlipWallBC.f90:288-318
            const double ewall = b.wall_temperature / (p.gm1 * p.gammaM2);
            for (int c = 0; c < 4; ++c) Qa[c] = Q[c];
            Qa[4] = Q[4] + wall_type(b) * (Q[0] * ewall + 0.5 * (Q[1] * Q[1] + Q[2] * Q[2] + Q[3] * Q[3]) / Q[0] - Q[4]);
            gradient_variables(p, Qa, U);
            return;
        }
        default: {  // GenericBC_FlowGradVars: U* = (U(FlowState(Q)) + U) / 2
            for (int c = 0; c < 5; ++c) Qa[c] = Q[c];
            bc_state(p, b, n, Qa);
            double Ua[5];
            gradient_variables(p, Qa, Ua);
            for (int c = 0; c < 5; ++c) U[c] = 0.5 * (Ua[c] + U[c]);
            return;
        }
    }
}

// FlowNeumann: the boundary's viscous normal flux from the interior one.
static void bc_neumann(const dg_boundary& b, const double* Q, double* f) {
    switch (b.type) {
        case DG_BC_NO_SLIP_WALL: {  // NoSlipWallBC.f90:339-372
            const double invRho = 1.0 / Q[0];
            const double u = invRho * Q[1], v = invRho * Q[2], w = invRho * Q[3];
            const double work = u * f[1] + v * f[2] + w * f[3];
            const double heat = f[4] - work;
            f[0] = 0.0;
            f[4] = (b.wall_velocity[0] * f[1] + b.wall_velocity[1] * f[2] + b.wall_velocity[2] * f[3]) +
                   wall_type(b) * heat;
            return;
        }
        case DG_BC_FREE_SLIP_WALL: {  // FreeSlipWallBC.f90:320-351
            const double work = (f[1] * Q[1] + f[2] * Q[2] + f[3] * Q[3]) / Q[0];
            const double heat = f[4] - work;
            f[0] = f[1] = f[2] = f[3] = 0.0;
            f[4] = wall_type(b) * heat;
            return;
        }
        default:  // InflowBC.f90:408-414, OutflowBC.f90:290-304
            for (int c = 0; c < 5; ++c) f[c] = 0.0;
            return;
    }
}

// ---------------------------------------------------------------- solver state ---------------
struct Elem {
    int N[3];
    int P[3];
    int64_t off;
    int face[6], fside[6];
};
struct Face {
    int elem[2], side[2], rot;
    int bc = -1;  // boundary condition of a boundary face (elem[1] == -1)
    int Nf[2], NelL[2], NelR[2], NfL[2], NfR[2], proj[2];
    int64_t off;  // face point offset in the geometry arrays
    std::vector<double> Q[2], Ux[2], Uy[2], Uz[2], mu[2];  // at Nf
    std::vector<double> unStar[2];                         // (5,3, element-face dims)
    std::vector<double> fStar[2];                          // (5, element-face dims)
};

struct Solver {
    Phys ph;
    std::vector<dg_boundary> bcs;
    dg_options opt;
    int nodes;
    int K;
    std::vector<Elem> el;
    std::vector<Face> fa;
    std::vector<double> x, jaXi, jaEta, jaZeta, jac, invJac;
    std::vector<double> fn, ft1, ft2, fj;
    std::vector<double> Q, QDot, G, Ux, Uy, Uz, mu2;  // element storage, reference layout
    int64_t ndof;
};

static int axis_of(int side, int a) {
    static const int m[6][2] = {{0, 2}, {0, 2}, {0, 1}, {1, 2}, {0, 1}, {1, 2}};
    return m[side - 1][a];
}

// Element-face trace (nv values per point at element-face dims n1 x n2) -> face storage at Nf
// (FaceClass.f90:281-382 Face_AdaptSolutionToFace, :384-470 Face_AdaptGradientsToFace).
static void adapt_to_face(const Face& f, int side, int nv, const std::vector<double>& e, int n1, int n2,
                          std::vector<double>& out, int nodes) {
    std::vector<double> rot;
    const std::vector<double>* src = &e;
    int s1 = n1, s2 = n2;
    if (side == 1) {
        s1 = f.NfL[0] + 1; s2 = f.NfL[1] + 1;
    } else {
        s1 = f.NfR[0] + 1; s2 = f.NfR[1] + 1;
        rot.assign(nv * s1 * s2, 0.0);
        for (int j = 0; j < s2; ++j)
            for (int i = 0; i < s1; ++i) {
                int ii, jj;
                l2r(i, j, f.NfR[0], f.NfR[1], f.rot, ii, jj);
                for (int v = 0; v < nv; ++v) rot[v + nv * (i + s1 * j)] = e[v + nv * (ii + n1 * jj)];
            }
        src = &rot;
    }
    const int q1 = f.Nf[0] + 1, q2 = f.Nf[1] + 1;
    out.assign(nv * q1 * q2, 0.0);
    const int pt = f.proj[side - 1];
    const int* Ns = side == 1 ? f.NfL : f.NfR;
    const std::vector<double>& S = *src;
    if (pt == 0) { out = S; return; }
    const std::vector<double> T1 = tset(nodes, Ns[0], f.Nf[0]);
    const std::vector<double> T2 = tset(nodes, Ns[1], f.Nf[1]);
    if (pt == 1) {
        for (int j = 0; j < q2; ++j)
            for (int l = 0; l < s1; ++l)
                for (int i = 0; i < q1; ++i)
                    for (int v = 0; v < nv; ++v) out[v + nv * (i + q1 * j)] += T1[i * s1 + l] * S[v + nv * (l + s1 * j)];
    } else if (pt == 2) {
        for (int l = 0; l < s2; ++l)
            for (int j = 0; j < q2; ++j)
                for (int i = 0; i < q1; ++i)
                    for (int v = 0; v < nv; ++v) out[v + nv * (i + q1 * j)] += T2[j * s2 + l] * S[v + nv * (i + s1 * l)];
    } else {
        for (int l = 0; l < s2; ++l)
            for (int j = 0; j < q2; ++j)
                for (int m = 0; m < s1; ++m)
                    for (int i = 0; i < q1; ++i)
                        for (int v = 0; v < nv; ++v)
                            out[v + nv * (i + q1 * j)] += T1[i * s1 + m] * T2[j * s2 + l] * S[v + nv * (m + s1 * l)];
    }
}

// Face flux at Nf -> element-face storage of side (FaceClass.f90:597-703 / 865-963); sign applies
// to side 2 (-1 for the Riemann flux, +1 for the BR1 jump).
static void project_to_side(const Face& f, int side, int nv, const std::vector<double>& flux, std::vector<double>& out,
                            double sign2, int nodes) {
    const int q1 = f.Nf[0] + 1, q2 = f.Nf[1] + 1;
    const int* Ns = side == 1 ? f.NfL : f.NfR;
    const int s1 = Ns[0] + 1, s2 = Ns[1] + 1;
    std::vector<double> aux(nv * s1 * s2, 0.0);
    const int pt = f.proj[side - 1];
    if (pt == 0) aux = flux;
    else {
        const std::vector<double> T1 = tset(nodes, f.Nf[0], Ns[0]);
        const std::vector<double> T2 = tset(nodes, f.Nf[1], Ns[1]);
        if (pt == 1) {
            for (int j = 0; j < s2; ++j)
                for (int l = 0; l < q1; ++l)
                    for (int i = 0; i < s1; ++i)
                        for (int v = 0; v < nv; ++v) aux[v + nv * (i + s1 * j)] += T1[i * q1 + l] * flux[v + nv * (l + q1 * j)];
        } else if (pt == 2) {
            for (int l = 0; l < q2; ++l)
                for (int j = 0; j < s2; ++j)
                    for (int i = 0; i < s1; ++i)
                        for (int v = 0; v < nv; ++v) aux[v + nv * (i + s1 * j)] += T2[j * q2 + l] * flux[v + nv * (i + q1 * l)];
        } else {
            for (int l = 0; l < q2; ++l)
                for (int j = 0; j < s2; ++j)
                    for (int m = 0; m < q1; ++m)
                        for (int i = 0; i < s1; ++i)
                            for (int v = 0; v < nv; ++v)
                                aux[v + nv * (i + s1 * j)] += T1[i * q1 + m] * T2[j * q2 + l] * flux[v + nv * (m + q1 * l)];
        }
    }
    if (side == 1) { out = aux; return; }
    // Right element: element-face dims are the unrotated NelR.
    const int r1 = f.NelR[0] + 1, r2 = f.NelR[1] + 1;
    out.assign(nv * r1 * r2, 0.0);
    for (int j = 0; j < s2; ++j)
        for (int i = 0; i < s1; ++i) {
            int ii, jj;
            l2r(i, j, f.NfR[0], f.NfR[1], f.rot, ii, jj);
            for (int v = 0; v < nv; ++v) out[v + nv * (ii + r1 * jj)] = aux[v + nv * (i + s1 * j)];
        }
    for (auto& v : out) v = sign2 * v;
}

// Per-element face traces of an element array (HexElementClass.f90:233-372).
static void prolong(const Solver& s, const Elem& e, int nv, const double* A, std::vector<double> tr[6]) {
    const Nodal& sx = nodal(s.nodes, e.N[0]);
    const Nodal& sy = nodal(s.nodes, e.N[1]);
    const Nodal& sz = nodal(s.nodes, e.N[2]);
    const int px = e.P[0], py = e.P[1], pz = e.P[2];
    tr[ELEFT - 1].assign(nv * py * pz, 0.0);
    tr[ERIGHT - 1].assign(nv * py * pz, 0.0);
    tr[EFRONT - 1].assign(nv * px * pz, 0.0);
    tr[EBACK - 1].assign(nv * px * pz, 0.0);
    tr[EBOTTOM - 1].assign(nv * px * py, 0.0);
    tr[ETOP - 1].assign(nv * px * py, 0.0);
    for (int k = 0; k < pz; ++k)
        for (int j = 0; j < py; ++j)
            for (int i = 0; i < px; ++i) {
                const double* a = A + nv * (i + px * (j + py * k));
                for (int v = 0; v < nv; ++v) {
                    tr[ELEFT - 1][v + nv * (j + py * k)] += a[v] * sx.vL[i];
                    tr[ERIGHT - 1][v + nv * (j + py * k)] += a[v] * sx.vR[i];
                    tr[EFRONT - 1][v + nv * (i + px * k)] += a[v] * sy.vL[j];
                    tr[EBACK - 1][v + nv * (i + px * k)] += a[v] * sy.vR[j];
                    tr[EBOTTOM - 1][v + nv * (i + px * j)] += a[v] * sz.vL[k];
                    tr[ETOP - 1][v + nv * (i + px * j)] += a[v] * sz.vR[k];
                }
            }
}

static int face_dims(const Elem& e, int side, int a) { return e.P[axis_of(side, a)]; }

// ---------------------------------------------------------------- right-hand side ----------
// phase < 0: the whole right-hand side. An element partition runs it in three phases with the
// reference's face exchanges between them (HexMesh_UpdateMPIFacesSolution before phase 1,
// HexMesh_UpdateMPIFacesGradients before phase 2; HexMesh.f90:1199-1730, MPI_Face.f90:203-383):
// phase 0 prolongs Q to the faces, phase 1 forms the BR1 gradients and their face traces, phase 2
// the time derivative.
static void compute_rhs(Solver& s, double t, int phase = -1) {
    const int K = s.K;
    const bool ns = s.ph.ns;
    // 1) prolong Q to faces (HexMesh.f90:948-1036)
    if (phase < 0 || phase == 0) {
#pragma omp parallel for schedule(static)
        for (int id = 0; id < K; ++id) {
            const Elem& e = s.el[id];
            std::vector<double> tr[6];
            prolong(s, e, 5, &s.Q[5 * e.off], tr);
            for (int side = 1; side <= 6; ++side) {
                Face& f = s.fa[e.face[side - 1]];
                const int fs = e.fside[side - 1];
                adapt_to_face(f, fs, 5, tr[side - 1], face_dims(e, side, 0), face_dims(e, side, 1), f.Q[fs - 1], s.nodes);
            }
        }
    }
    // 2) BR1 gradients (EllipticBR1.f90:71-159, 168-397)
    if (ns && (phase < 0 || phase == 1)) {
#pragma omp parallel for schedule(static)
        for (int id = 0; id < K; ++id) {  // HexElement_ComputeLocalGradient (HexElementClass.f90:427-531)
            const Elem& e = s.el[id];
            const Nodal& sx = nodal(s.nodes, e.N[0]);
            const Nodal& sy = nodal(s.nodes, e.N[1]);
            const Nodal& sz = nodal(s.nodes, e.N[2]);
            const int px = e.P[0], py = e.P[1], pz = e.P[2], np = px * py * pz;
            std::vector<double> Uv(5 * np);  // GetGradients at the nodes (HexElementClass.f90:463-470)
            for (int q = 0; q < np; ++q) gradient_variables(s.ph, &s.Q[5 * (e.off + q)], &Uv[5 * q]);
            const double* U = Uv.data();
            std::vector<double> Uxi(5 * np, 0.0), Ueta(5 * np, 0.0), Uzeta(5 * np, 0.0);
            auto n = [&](int i, int j, int k) { return i + px * (j + py * k); };
            for (int k = 0; k < pz; ++k) for (int j = 0; j < py; ++j) for (int l = 0; l < px; ++l) for (int i = 0; i < px; ++i)
                for (int v = 0; v < 5; ++v) Uxi[5 * n(i, j, k) + v] += U[5 * n(l, j, k) + v] * sx.D[i * px + l];
            for (int k = 0; k < pz; ++k) for (int l = 0; l < py; ++l) for (int j = 0; j < py; ++j) for (int i = 0; i < px; ++i)
                for (int v = 0; v < 5; ++v) Ueta[5 * n(i, j, k) + v] += U[5 * n(i, l, k) + v] * sy.D[j * py + l];
            for (int l = 0; l < pz; ++l) for (int k = 0; k < pz; ++k) for (int j = 0; j < py; ++j) for (int i = 0; i < px; ++i)
                for (int v = 0; v < 5; ++v) Uzeta[5 * n(i, j, k) + v] += U[5 * n(i, j, l) + v] * sz.D[k * pz + l];
            for (int q = 0; q < np; ++q) {
                const int64_t g = e.off + q;
                const double* a = &s.jaXi[3 * g];
                const double* b = &s.jaEta[3 * g];
                const double* c = &s.jaZeta[3 * g];
                for (int v = 0; v < 5; ++v) {
                    s.Ux[5 * g + v] = (Uxi[5 * q + v] * a[0] + Ueta[5 * q + v] * b[0] + Uzeta[5 * q + v] * c[0]) * s.invJac[g];
                    s.Uy[5 * g + v] = (Uxi[5 * q + v] * a[1] + Ueta[5 * q + v] * b[1] + Uzeta[5 * q + v] * c[1]) * s.invJac[g];
                    s.Uz[5 * g + v] = (Uxi[5 * q + v] * a[2] + Ueta[5 * q + v] * b[2] + Uzeta[5 * q + v] * c[2]) * s.invJac[g];
                }
            }
        }
        // BR1_ComputeElementInterfaceAverage (EllipticBR1.f90:571-627)
#pragma omp parallel for schedule(static)
        for (int fid = 0; fid < static_cast<int>(s.fa.size()); ++fid) {
            Face& f = s.fa[fid];
            const int q1 = f.Nf[0] + 1, q2 = f.Nf[1] + 1;
            std::vector<double> us(15 * q1 * q2);
            const bool boundary = f.elem[1] < 0;
            for (int j = 0; j < q2; ++j)
                for (int i = 0; i < q1; ++i) {
                    const int p = i + q1 * j;
                    const double J = s.fj[f.off + p];
                    const double* n = &s.fn[3 * (f.off + p)];
                    double UL[5], UR[5];
                    gradient_variables(s.ph, &f.Q[0][5 * p], UL);
                    if (boundary) {  // BR1_ComputeBoundaryFlux (EllipticBR1.f90:686-736): (U* - U) Jf n
                        double Us[5];
                        for (int v = 0; v < 5; ++v) Us[v] = UL[v];
                        bc_gradvars(s.ph, s.bcs[f.bc], n, &f.Q[0][5 * p], Us);
                        for (int v = 0; v < 5; ++v) {
                            const double u = (Us[v] - UL[v]) * J;
                            us[15 * p + v] = u * n[0];
                            us[15 * p + 5 + v] = u * n[1];
                            us[15 * p + 10 + v] = u * n[2];
                        }
                        continue;
                    }
                    gradient_variables(s.ph, &f.Q[1][5 * p], UR);
                    for (int v = 0; v < 5; ++v) {
                        const double u = 0.5 * (UR[v] - UL[v]) * J;
                        us[15 * p + v] = u * n[0];
                        us[15 * p + 5 + v] = u * n[1];
                        us[15 * p + 10 + v] = u * n[2];
                    }
                }
            project_to_side(f, 1, 15, us, f.unStar[0], 1.0, s.nodes);
            if (!boundary) project_to_side(f, 2, 15, us, f.unStar[1], 1.0, s.nodes);
        }
        // BR1_GradientFaceLoop + ProlongGradientsToFaces (EllipticBR1.f90:531-569; DGIntegrals.f90:365-443)
#pragma omp parallel for schedule(static)
        for (int id = 0; id < K; ++id) {
            const Elem& e = s.el[id];
            const Nodal& sx = nodal(s.nodes, e.N[0]);
            const Nodal& sy = nodal(s.nodes, e.N[1]);
            const Nodal& sz = nodal(s.nodes, e.N[2]);
            const int px = e.P[0], py = e.P[1], pz = e.P[2];
            auto H = [&](int side) -> const std::vector<double>& {
                return s.fa[e.face[side - 1]].unStar[e.fside[side - 1] - 1];
            };
            const std::vector<double>&HF = H(EFRONT), &HBK = H(EBACK), &HBO = H(EBOTTOM), &HR = H(ERIGHT),
                                    &HT = H(ETOP), &HL = H(ELEFT);
            for (int k = 0; k < pz; ++k)
                for (int j = 0; j < py; ++j)
                    for (int i = 0; i < px; ++i) {
                        const int64_t g = e.off + i + px * (j + py * k);
                        for (int d = 0; d < 3; ++d) {
                            double* Ud = d == 0 ? &s.Ux[5 * g] : (d == 1 ? &s.Uy[5 * g] : &s.Uz[5 * g]);
                            for (int v = 0; v < 5; ++v) {
                                double fi = HL[v + 5 * d + 15 * (j + py * k)] * sx.bL[i];
                                fi = fi + HR[v + 5 * d + 15 * (j + py * k)] * sx.bR[i];
                                fi = fi + HF[v + 5 * d + 15 * (i + px * k)] * sy.bL[j];
                                fi = fi + HBK[v + 5 * d + 15 * (i + px * k)] * sy.bR[j];
                                fi = fi + HBO[v + 5 * d + 15 * (i + px * j)] * sz.bL[k];
                                fi = fi + HT[v + 5 * d + 15 * (i + px * j)] * sz.bR[k];
                                Ud[v] = Ud[v] + fi * s.invJac[g];
                            }
                        }
                    }
            std::vector<double> tx[6], ty[6], tz[6];
            prolong(s, e, 5, &s.Ux[5 * e.off], tx);
            prolong(s, e, 5, &s.Uy[5 * e.off], ty);
            prolong(s, e, 5, &s.Uz[5 * e.off], tz);
            for (int side = 1; side <= 6; ++side) {
                Face& f = s.fa[e.face[side - 1]];
                const int fs = e.fside[side - 1];
                const int d1 = face_dims(e, side, 0), d2 = face_dims(e, side, 1);
                adapt_to_face(f, fs, 5, tx[side - 1], d1, d2, f.Ux[fs - 1], s.nodes);
                adapt_to_face(f, fs, 5, ty[side - 1], d1, d2, f.Uy[fs - 1], s.nodes);
                adapt_to_face(f, fs, 5, tz[side - 1], d1, d2, f.Uz[fs - 1], s.nodes);
            }
        }
    }
    // 3) TimeDerivative_ComputeQDot (SpatialDiscretization.f90:379-685)
    if (phase >= 0 && phase != 2) return;
    if (ns) {
#pragma omp parallel for schedule(static)
        for (int64_t g = 0; g < s.ndof; ++g) mu_kappa(s.ph, &s.Q[5 * g], s.mu2[2 * g], s.mu2[2 * g + 1]);
#pragma omp parallel for schedule(static)
        for (int fid = 0; fid < static_cast<int>(s.fa.size()); ++fid) {
            Face& f = s.fa[fid];
            const int np = (f.Nf[0] + 1) * (f.Nf[1] + 1);
            for (int side = 0; side < 2; ++side) {
                if (f.elem[side] < 0) continue;
                f.mu[side].resize(2 * np);
                for (int p = 0; p < np; ++p) mu_kappa(s.ph, &f.Q[side][5 * p], f.mu[side][2 * p], f.mu[side][2 * p + 1]);
            }
        }
    }
    // Volume integrals (SpatialDiscretization.f90:1602-1682)
#pragma omp parallel for schedule(static)
    for (int id = 0; id < K; ++id) {
        const Elem& e = s.el[id];
        const Nodal& sx = nodal(s.nodes, e.N[0]);
        const Nodal& sy = nodal(s.nodes, e.N[1]);
        const Nodal& sz = nodal(s.nodes, e.N[2]);
        const int px = e.P[0], py = e.P[1], pz = e.P[2], np = px * py * pz;
        std::vector<double> Fi(15 * np), Fv(15 * np, 0.0);  // contravariant: F[v + 5*(n) + 5*np*d]
        auto n = [&](int i, int j, int k) { return i + px * (j + py * k); };
        for (int q = 0; q < np; ++q) {
            const int64_t g = e.off + q;
            double cf[15];
            euler_flux(s.ph, &s.Q[5 * g], cf);
            const double* ja[3] = {&s.jaXi[3 * g], &s.jaEta[3 * g], &s.jaZeta[3 * g]};
            for (int d = 0; d < 3; ++d)
                for (int v = 0; v < 5; ++v)
                    Fi[v + 5 * q + 5 * np * d] = cf[v] * ja[d][0] + cf[v + 5] * ja[d][1] + cf[v + 10] * ja[d][2];
            if (ns) {
                viscous_flux(s.ph, &s.Q[5 * g], &s.Ux[5 * g], &s.Uy[5 * g], &s.Uz[5 * g], s.mu2[2 * g], 0.0, s.mu2[2 * g + 1], cf);
                for (int d = 0; d < 3; ++d)
                    for (int v = 0; v < 5; ++v)
                        Fv[v + 5 * q + 5 * np * d] = cf[v] * ja[d][0] + cf[v + 5] * ja[d][1] + cf[v + 10] * ja[d][2];
            }
        }
        double* qd = &s.QDot[5 * e.off];
        for (int q = 0; q < 5 * np; ++q) qd[q] = 0.0;
        if (s.opt.inviscid == DG_INVISCID_STANDARD) {
            std::vector<double> Fc(15 * np);
            for (int q = 0; q < 15 * np; ++q) Fc[q] = Fi[q] - Fv[q];
            // ScalarWeakIntegrals_StdVolumeGreen (DGIntegrals.f90:56-87)
            for (int k = 0; k < pz; ++k) for (int j = 0; j < py; ++j) for (int l = 0; l < px; ++l) for (int i = 0; i < px; ++i)
                for (int v = 0; v < 5; ++v) qd[5 * n(i, j, k) + v] += sx.hatD[i * px + l] * Fc[v + 5 * n(l, j, k)];
            for (int k = 0; k < pz; ++k) for (int l = 0; l < py; ++l) for (int j = 0; j < py; ++j) for (int i = 0; i < px; ++i)
                for (int v = 0; v < 5; ++v) qd[5 * n(i, j, k) + v] += sy.hatD[j * py + l] * Fc[v + 5 * n(i, l, k) + 5 * np];
            for (int l = 0; l < pz; ++l) for (int k = 0; k < pz; ++k) for (int j = 0; j < py; ++j) for (int i = 0; i < px; ++i)
                for (int v = 0; v < 5; ++v) qd[5 * n(i, j, k) + v] += sz.hatD[k * pz + l] * Fc[v + 5 * n(i, j, l) + 10 * np];
        } else {
            // SplitDG_ComputeSplitFormFluxes (HyperbolicSplitForm.f90:64-116) and
            // ScalarWeakIntegrals_SplitVolumeDivergence (DGIntegrals.f90:92-129), negated.
            std::vector<double> fS(5 * px * np), gS(5 * py * np), hS(5 * pz * np);
            auto fi = [&](int l, int q) { return 5 * (l + px * q); };
            auto gi = [&](int l, int q) { return 5 * (l + py * q); };
            auto hi = [&](int l, int q) { return 5 * (l + pz * q); };
            for (int k = 0; k < pz; ++k) for (int j = 0; j < py; ++j) for (int i = 0; i < px; ++i)
                for (int v = 0; v < 5; ++v) {
                    fS[fi(i, n(i, j, k)) + v] = Fi[v + 5 * n(i, j, k)];
                    gS[gi(j, n(i, j, k)) + v] = Fi[v + 5 * n(i, j, k) + 5 * np];
                    hS[hi(k, n(i, j, k)) + v] = Fi[v + 5 * n(i, j, k) + 10 * np];
                }
            const double* Q = &s.Q[5 * e.off];
            const double* jx = &s.jaXi[3 * e.off];
            const double* je = &s.jaEta[3 * e.off];
            const double* jz = &s.jaZeta[3 * e.off];
            for (int k = 0; k < pz; ++k) for (int j = 0; j < py; ++j) for (int i = 0; i < px; ++i)
                for (int l = i + 1; l < px; ++l) {
                    double* o = &fS[fi(l, n(i, j, k))];
                    two_point(s.ph, s.opt.averaging, Q + 5 * n(i, j, k), Q + 5 * n(l, j, k), jx + 3 * n(i, j, k), jx + 3 * n(l, j, k), o);
                    for (int v = 0; v < 5; ++v) fS[fi(i, n(l, j, k)) + v] = o[v];
                }
            for (int k = 0; k < pz; ++k) for (int j = 0; j < py; ++j) for (int i = 0; i < px; ++i)
                for (int l = j + 1; l < py; ++l) {
                    double* o = &gS[gi(l, n(i, j, k))];
                    two_point(s.ph, s.opt.averaging, Q + 5 * n(i, j, k), Q + 5 * n(i, l, k), je + 3 * n(i, j, k), je + 3 * n(i, l, k), o);
                    for (int v = 0; v < 5; ++v) gS[gi(j, n(i, l, k)) + v] = o[v];
                }
            for (int k = 0; k < pz; ++k) for (int j = 0; j < py; ++j) for (int i = 0; i < px; ++i)
                for (int l = k + 1; l < pz; ++l) {
                    double* o = &hS[hi(l, n(i, j, k))];
                    two_point(s.ph, s.opt.averaging, Q + 5 * n(i, j, k), Q + 5 * n(i, j, l), jz + 3 * n(i, j, k), jz + 3 * n(i, j, l), o);
                    for (int v = 0; v < 5; ++v) hS[hi(k, n(i, j, l)) + v] = o[v];
                }
            std::vector<double> vi(5 * np, 0.0);
            for (int k = 0; k < pz; ++k) for (int j = 0; j < py; ++j) for (int l = 0; l < px; ++l) for (int i = 0; i < px; ++i)
                for (int v = 0; v < 5; ++v)
                    vi[5 * n(i, j, k) + v] = vi[5 * n(i, j, k) + v] + sx.sharpD[i * px + l] * fS[fi(l, n(i, j, k)) + v] +
                                             sx.hatD[i * px + l] * Fv[v + 5 * n(l, j, k)];
            for (int k = 0; k < pz; ++k) for (int l = 0; l < py; ++l) for (int j = 0; j < py; ++j) for (int i = 0; i < px; ++i)
                for (int v = 0; v < 5; ++v)
                    vi[5 * n(i, j, k) + v] = vi[5 * n(i, j, k) + v] + sy.sharpD[j * py + l] * gS[gi(l, n(i, j, k)) + v] +
                                             sy.hatD[j * py + l] * Fv[v + 5 * n(i, l, k) + 5 * np];
            for (int l = 0; l < pz; ++l) for (int k = 0; k < pz; ++k) for (int j = 0; j < py; ++j) for (int i = 0; i < px; ++i)
                for (int v = 0; v < 5; ++v)
                    vi[5 * n(i, j, k) + v] = vi[5 * n(i, j, k) + v] + sz.sharpD[k * pz + l] * hS[hi(l, n(i, j, k)) + v] +
                                             sz.hatD[k * pz + l] * Fv[v + 5 * n(i, j, l) + 10 * np];
            for (int q = 0; q < 5 * np; ++q) qd[q] = -vi[q];
        }
    }
    // Interface fluxes (SpatialDiscretization.f90:1710-1799)
#pragma omp parallel for schedule(static)
    for (int fid = 0; fid < static_cast<int>(s.fa.size()); ++fid) {
        Face& f = s.fa[fid];
        const int q1 = f.Nf[0] + 1, q2 = f.Nf[1] + 1, np = q1 * q2;
        std::vector<double> flux(5 * np);
        const bool boundary = f.elem[1] < 0;
        for (int p = 0; p < np; ++p) {
            double visc[5] = {0, 0, 0, 0, 0};
            const double* n = &s.fn[3 * (f.off + p)];
            double Qb[5];
            if (boundary) {  // computeBoundaryFlux (SpatialDiscretization.f90:1896-2028)
                const dg_boundary& b = s.bcs[f.bc];
                for (int v = 0; v < 5; ++v) Qb[v] = f.Q[0][5 * p + v];
                bc_state(s.ph, b, n, Qb);
                if (ns) {
                    double fL[15];
                    viscous_flux(s.ph, &f.Q[0][5 * p], &f.Ux[0][5 * p], &f.Uy[0][5 * p], &f.Uz[0][5 * p],
                                 f.mu[0][2 * p], 0.0, f.mu[0][2 * p + 1], fL);
                    for (int v = 0; v < 5; ++v) visc[v] = fL[v] * n[0] + fL[v + 5] * n[1] + fL[v + 10] * n[2];
                    bc_neumann(b, &f.Q[0][5 * p], visc);
                }
            } else if (ns) {  // BR1_RiemannSolver (EllipticBR1.f90:816-868)
                double fL[15], fR[15];
                viscous_flux(s.ph, &f.Q[0][5 * p], &f.Ux[0][5 * p], &f.Uy[0][5 * p], &f.Uz[0][5 * p], f.mu[0][2 * p], 0.0,
                             f.mu[0][2 * p + 1], fL);
                viscous_flux(s.ph, &f.Q[1][5 * p], &f.Ux[1][5 * p], &f.Uy[1][5 * p], &f.Uz[1][5 * p], f.mu[1][2 * p], 0.0,
                             f.mu[1][2 * p + 1], fR);
                for (int v = 0; v < 5; ++v) {
                    const double a = 0.5 * (fL[v] + fR[v]), b = 0.5 * (fL[v + 5] + fR[v + 5]), c = 0.5 * (fL[v + 10] + fR[v + 10]);
                    visc[v] = a * n[0] + b * n[1] + c * n[2];
                }
            }
            double inv[5];
            const double* QL = &f.Q[0][5 * p];
            const double* QR = boundary ? Qb : &f.Q[1][5 * p];
            const double* t1 = &s.ft1[3 * (f.off + p)];
            const double* t2 = &s.ft2[3 * (f.off + p)];
            const int avg = s.opt.averaging;
            const double ls = s.opt.lambda_stab;
            switch (s.opt.riemann) {
                case DG_RIEMANN_ROE: roe(s.ph, QL, QR, n, inv); break;
                case DG_RIEMANN_RUSANOV: rusanov(s.ph, QL, QR, n, inv); break;
                case DG_RIEMANN_STD_ROE: std_roe(s.ph, avg, ls, false, QL, QR, n, t1, t2, inv); break;
                case DG_RIEMANN_ROE_PIKE: std_roe(s.ph, avg, ls, true, QL, QR, n, t1, t2, inv); break;
                case DG_RIEMANN_LOW_DISS_ROE: low_diss_roe(s.ph, avg, ls, QL, QR, n, t1, t2, inv); break;
                case DG_RIEMANN_MATRIX_DISS: matrix_diss(s.ph, avg, ls, QL, QR, n, t1, t2, inv); break;
                case DG_RIEMANN_VISCOUS_NS: viscous_ns(s.ph, avg, ls, QL, QR, n, t1, t2, inv); break;
                case DG_RIEMANN_U_DISS: u_diss(s.ph, avg, ls, QL, QR, n, t1, t2, inv); break;
                default:  // LxF, or central = LxF with lambdaStab = 0 (RiemannSolvers_NS.f90:224)
                    lxf(s.ph, avg, s.opt.riemann == DG_RIEMANN_CENTRAL ? 0.0 : ls, QL, QR, n, t1, t2, inv);
                    break;
            }
            for (int v = 0; v < 5; ++v) flux[5 * p + v] = (inv[v] - visc[v]) * s.fj[f.off + p];
        }
        project_to_side(f, 1, 5, flux, f.fStar[0], -1.0, s.nodes);
        if (!boundary) project_to_side(f, 2, 5, flux, f.fStar[1], -1.0, s.nodes);
    }
    // Surface integrals, 1/J, source (SpatialDiscretization.f90:483-494, 1686-1701, 564-639)
    const double mms_mu = s.ph.mu, mms_kap = s.ph.kappa;
    // LambVector's source viscosity: refValues%mu = rho_ref V_ref L_ref mu (PhysicsStorage_NS.f90:292-309),
    // with T_ref = 520*5/9 K, p_ref = 101325 Pa, R = 287.15 J/(kg K), L_ref = 1; zero for Euler.
    const double T_ref = 520.0 * 5.0 / 9.0, R_gas = 287.15;
    const double lamb_mu = s.ph.ns ? (101325.0 / (R_gas * T_ref)) * (s.ph.Mach * std::sqrt(s.ph.gamma * R_gas * T_ref)) *
                                         1.0 * s.ph.mu
                                   : 0.0;
    const double lamb_kap = lamb_mu * s.ph.mu_to_kappa;
#pragma omp parallel for schedule(static)
    for (int id = 0; id < K; ++id) {
        const Elem& e = s.el[id];
        const Nodal& sx = nodal(s.nodes, e.N[0]);
        const Nodal& sy = nodal(s.nodes, e.N[1]);
        const Nodal& sz = nodal(s.nodes, e.N[2]);
        const int px = e.P[0], py = e.P[1], pz = e.P[2];
        auto Fs = [&](int side) -> const std::vector<double>& { return s.fa[e.face[side - 1]].fStar[e.fside[side - 1] - 1]; };
        const std::vector<double>&FFR = Fs(EFRONT), &FBK = Fs(EBACK), &FBO = Fs(EBOTTOM), &FR = Fs(ERIGHT), &FT = Fs(ETOP),
                                &FL = Fs(ELEFT);
        for (int k = 0; k < pz; ++k)
            for (int j = 0; j < py; ++j)
                for (int i = 0; i < px; ++i) {
                    const int64_t g = e.off + i + px * (j + py * k);
                    for (int v = 0; v < 5; ++v) {
                        double fi = FL[v + 5 * (j + py * k)] * sx.bL[i];
                        fi = fi + FR[v + 5 * (j + py * k)] * sx.bR[i];
                        fi = fi + FFR[v + 5 * (i + px * k)] * sy.bL[j];
                        fi = fi + FBK[v + 5 * (i + px * k)] * sy.bR[j];
                        fi = fi + FBO[v + 5 * (i + px * j)] * sz.bL[k];
                        fi = fi + FT[v + 5 * (i + px * j)] * sz.bR[k];
                        s.QDot[5 * g + v] = s.QDot[5 * g + v] - fi;
                        s.QDot[5 * g + v] = s.QDot[5 * g + v] / s.jac[g];
                    }
                    if (s.opt.source == DG_SOURCE_MMS_LAMB_VECTOR) {
                        double S[5];
                        const double* xx = &s.x[3 * g];
                        lamb_point(xx[0], xx[1], xx[2], t, s.ph.gm1, s.ph.gammaM2, lamb_mu, lamb_kap, s.ph.Re, S);
                        for (int v = 0; v < 5; ++v) s.QDot[5 * g + v] = s.QDot[5 * g + v] + S[v];
                    }
                    if (s.opt.source == DG_SOURCE_MMS_CONVERGENCE) {
                        double Qe[5], S[5], Qd[5];
                        const double* xx = &s.x[3 * g];
                        mms_point(xx[0], xx[1], xx[2], t, s.ph.gm1, s.ph.gammaM2, mms_mu, mms_kap, Qe, S, Qd);
                        for (int v = 0; v < 5; ++v) s.QDot[5 * g + v] = s.QDot[5 * g + v] + S[v];
                    }
                }
    }
}

// DGSEMClass.f90:870-1038 MaxTimeStep.
static double max_dt(const Solver& s, double cfl, double dcfl) {
    double conv = HUGE_VAL, visc = HUGE_VAL;
#pragma omp parallel for schedule(static) reduction(min : conv, visc)
    for (int id = 0; id < s.K; ++id) {
        const Elem& e = s.el[id];
        double dd[3], dd2[3];
        for (int d = 0; d < 3; ++d) {
            const Nodal& sp = nodal(s.nodes, e.N[d]);
            dd[d] = e.N[d] != 0 ? 1.0 / std::fabs(sp.x[1] - sp.x[0]) : 0.0;
            dd2[d] = dd[d] * dd[d];
        }
        const int np = e.P[0] * e.P[1] * e.P[2];
        for (int q = 0; q < np; ++q) {
            const int64_t g = e.off + q;
            const double* Q = &s.Q[5 * g];
            const double a = std::sqrt(s.ph.gamma * pressure(s.ph, Q) / Q[0]);
            const double ev[3] = {std::fabs(Q[1] / Q[0]) + a, std::fabs(Q[2] / Q[0]) + a, std::fabs(Q[3] / Q[0]) + a};
            const double* ja[3] = {&s.jaXi[3 * g], &s.jaEta[3 * g], &s.jaZeta[3 * g]};
            double lam[3];
            for (int d = 0; d < 3; ++d) lam[d] = std::fabs(ja[d][0] * ev[0] + ja[d][1] * ev[1] + ja[d][2] * ev[2]) * dd[d];
            conv = std::fmin(conv, cfl * std::fabs(s.jac[g]) / (lam[0] + lam[1] + lam[2]));
            if (s.ph.ns) {
                const double T = s.ph.gammaM2 * pressure(s.ph, Q) / Q[0];
                const double mu = sutherland(s.ph, T);
                double lv[3];
                for (int d = 0; d < 3; ++d) lv[d] = mu * dd2[d] * std::fabs(ja[d][0] + ja[d][1] + ja[d][2]);
                visc = std::fmin(visc, dcfl * std::fabs(s.jac[g]) / (lv[0] + lv[1] + lv[2]));
            }
        }
    }
    return conv < visc ? conv : visc;
}

}  // namespace orc

// ---------------------------------------------------------------- C API ----------------------
using orc::Solver;

// n_ghost > 0: an element partition. Faces may name the remote elements n_elements ..
// n_elements + n_ghost - 1 (the order array holds their orders too); those elements have no
// storage here, and their face sides are filled by orc_face_trace (the MPI faces of the reference).
static Solver* create(const dg_mesh_desc* m, int n_ghost, const dg_physics* ph, const dg_options* op);

extern "C" {

void* orc_create(const dg_mesh_desc* m, const dg_physics* ph, const dg_options* op) { return create(m, 0, ph, op); }
void* orc_create_partition(const dg_mesh_desc* m, int n_ghost, const dg_physics* ph, const dg_options* op) {
    return n_ghost >= 0 ? create(m, n_ghost, ph, op) : nullptr;
}

}  // extern "C"

static Solver* create(const dg_mesh_desc* m, int n_ghost, const dg_physics* ph, const dg_options* op) {
    auto* s = new Solver();
    s->opt = *op;
    s->nodes = m->node_type;
    s->K = m->n_elements;
    s->ph.Mach = ph->mach;
    s->ph.Re = ph->reynolds;
    s->ph.Pr = ph->prandtl;
    s->ph.ns = ph->navier_stokes != 0;
    s->ph.grad_vars = s->ph.ns ? op->gradient_variables : DG_GRADVARS_STATE;
    // PhysicsStorage_NS.f90:186-290,413-429
    s->ph.gammaM2 = s->ph.gamma * (ph->mach * ph->mach);
    if (s->ph.ns) {
        s->ph.mu = 1.0 / ph->reynolds;
        s->ph.kappa = 1.0 / (s->ph.gm1 * (ph->mach * ph->mach) * ph->reynolds * ph->prandtl);
        s->ph.mu_to_kappa = 1.0 / (s->ph.gm1 * (ph->mach * ph->mach) * ph->prandtl);
    } else {
        s->ph.mu = s->ph.kappa = s->ph.mu_to_kappa = 0.0;
    }
    const double TRef = 520.0 * 5.0 / 9.0;
    s->ph.S_div_TRef = (198.6 * 5.0 / 9.0) / TRef;
    s->ph.TReNorm = TRef / TRef;
    s->el.resize(s->K + n_ghost);
    int64_t off = 0;
    for (int e = 0; e < s->K + n_ghost; ++e) {
        auto& E = s->el[e];
        for (int d = 0; d < 3; ++d) { E.N[d] = m->order[3 * e + d]; E.P[d] = E.N[d] + 1; }
        E.off = e < s->K ? off : -1;
        if (e < s->K) off += static_cast<int64_t>(E.P[0]) * E.P[1] * E.P[2];
    }
    s->ndof = off;
    auto cp = [&](const double* src, int64_t n) { return std::vector<double>(src, src + n); };
    s->x = cp(m->x, 3 * off);
    s->jaXi = cp(m->ja_xi, 3 * off); s->jaEta = cp(m->ja_eta, 3 * off); s->jaZeta = cp(m->ja_zeta, 3 * off);
    s->jac = cp(m->jacobian, off); s->invJac = cp(m->inv_jacobian, off);
    s->fa.resize(m->n_faces);
    int64_t foff = 0;
    if (m->n_boundaries > 0 && m->boundaries) s->bcs.assign(m->boundaries, m->boundaries + m->n_boundaries);
    for (int f = 0; f < m->n_faces; ++f) {
        auto& F = s->fa[f];
        for (int q = 0; q < 2; ++q) {
            F.elem[q] = m->face_elem[2 * f + q];
            F.side[q] = m->face_side[2 * f + q];
            F.Nf[q] = m->face_nf[2 * f + q];
            if (F.elem[q] < 0) continue;  // boundary face: no second element
            s->el[F.elem[q]].face[F.side[q] - 1] = f;
            s->el[F.elem[q]].fside[F.side[q] - 1] = q + 1;
        }
        F.rot = m->face_rotation[f];
        const bool boundary = F.elem[1] < 0;
        if (boundary) F.bc = m->face_boundary ? m->face_boundary[f] : -1;
        for (int a = 0; a < 2; ++a) {
            F.NelL[a] = s->el[F.elem[0]].N[orc::axis_of(F.side[0], a)];
            F.NelR[a] = boundary ? F.NelL[a] : s->el[F.elem[1]].N[orc::axis_of(F.side[1], a)];
            F.NfL[a] = F.NelL[a];
        }
        switch (F.rot) {
            case 0: case 2: case 5: case 7: F.NfR[0] = F.NelR[0]; F.NfR[1] = F.NelR[1]; break;
            default: F.NfR[0] = F.NelR[1]; F.NfR[1] = F.NelR[0]; break;
        }
        auto ptype = [&](const int* Ns) {
            const bool a = Ns[0] != F.Nf[0], b = Ns[1] != F.Nf[1];
            return (!a && !b) ? 0 : (a && !b) ? 1 : (!a && b) ? 2 : 3;
        };
        F.proj[0] = ptype(F.NfL);
        F.proj[1] = ptype(F.NfR);
        F.off = foff;
        foff += static_cast<int64_t>(F.Nf[0] + 1) * (F.Nf[1] + 1);
    }
    for (const auto& E : s->el)
        for (int d = 0; d < 3; ++d) orc::nodal(s->nodes, E.N[d]);
    for (const auto& F : s->fa)
        for (int d = 0; d < 2; ++d) orc::nodal(s->nodes, F.Nf[d]);
    s->fn = cp(m->face_normal, 3 * foff); s->ft1 = cp(m->face_t1, 3 * foff); s->ft2 = cp(m->face_t2, 3 * foff);
    s->fj = cp(m->face_jacobian, foff);
    s->Q.assign(5 * off, 0.0); s->QDot.assign(5 * off, 0.0); s->G.assign(5 * off, 0.0);
    s->Ux.assign(5 * off, 0.0); s->Uy.assign(5 * off, 0.0); s->Uz.assign(5 * off, 0.0);
    s->mu2.assign(2 * off, 0.0);
    return s;
}

extern "C" {

void orc_destroy(void* h) { delete static_cast<Solver*>(h); }
// OpenMP threads of the following parallel regions (the checker's own sizing; all cores by default).
void orc_set_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
}
int64_t orc_ndof(void* h) { return static_cast<Solver*>(h)->ndof; }

void orc_set_state(void* h, const double* q) {
    auto* s = static_cast<Solver*>(h);
    std::memcpy(s->Q.data(), q, sizeof(double) * 5 * s->ndof);
    std::fill(s->G.begin(), s->G.end(), 0.0);
}

// field: 0 Q, 1 QDot, 2 G, 3/4/5 U_x/U_y/U_z
void orc_get(void* h, int field, double* out) {
    auto* s = static_cast<Solver*>(h);
    const std::vector<double>* v[] = {&s->Q, &s->QDot, &s->G, &s->Ux, &s->Uy, &s->Uz};
    std::memcpy(out, v[field]->data(), sizeof(double) * 5 * s->ndof);
}

void orc_rhs(void* h, double t) { orc::compute_rhs(*static_cast<Solver*>(h), t); }

// One phase (0, 1, 2) of the right-hand side at time t; see compute_rhs.
void orc_rhs_phase(void* h, double t, int phase) { orc::compute_rhs(*static_cast<Solver*>(h), t, phase); }

// The data an MPI face moves (MPI_Face_SendQ / the gradient sends, MPI_Face.f90:203-383): one side
// (1 or 2) of face f at its face points in the face's frame, Q (what 0, 5 per point) or the gradient
// traces U_x, U_y, U_z (what 1, three blocks of 5 per point). set = 0 copies out, 1 copies in.
// Returns the number of values, or -1 for bad arguments.
int64_t orc_face_trace(void* h, int f, int side, int what, double* buf, int set) {
    auto* s = static_cast<Solver*>(h);
    if (f < 0 || f >= static_cast<int>(s->fa.size()) || side < 1 || side > 2 || what < 0 || what > 1) return -1;
    orc::Face& F = s->fa[f];
    const int64_t np = static_cast<int64_t>(F.Nf[0] + 1) * (F.Nf[1] + 1);
    std::vector<double>* blocks[3] = {&F.Q[side - 1], nullptr, nullptr};
    int nb = 1;
    if (what == 1) {
        blocks[0] = &F.Ux[side - 1];
        blocks[1] = &F.Uy[side - 1];
        blocks[2] = &F.Uz[side - 1];
        nb = 3;
    }
    for (int b = 0; b < nb; ++b) {
        std::vector<double>& v = *blocks[b];
        if (set) {
            v.assign(buf + 5 * np * b, buf + 5 * np * (b + 1));
        } else {
            if (static_cast<int64_t>(v.size()) != 5 * np) return -1;
            std::memcpy(buf + 5 * np * b, v.data(), sizeof(double) * 5 * np);
        }
    }
    return 5 * np * nb;
}

// Stage k (0..2) of the low-storage update after the stage's right-hand side (ExplicitMethods.f90:748-779).
void orc_rk3_update(void* h, int k, double dt) {
    auto* s = static_cast<Solver*>(h);
    const double a[3] = {0.0, -5.0 / 9.0, -153.0 / 128.0};
    const double c[3] = {1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0};
    const int64_t n = 5 * s->ndof;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        s->G[i] = a[k] * s->G[i] + s->QDot[i];
        s->Q[i] = s->Q[i] + c[k] * dt * s->G[i];
    }
}

// ExplicitMethods.f90:748-779 (the dt_vec-free branch).
void orc_rk3_step(void* h, double t, double dt) {
    auto* s = static_cast<Solver*>(h);
    const double a[3] = {0.0, -5.0 / 9.0, -153.0 / 128.0};
    const double b[3] = {0.0, 1.0 / 3.0, 3.0 / 4.0};
    const double c[3] = {1.0 / 3.0, 15.0 / 16.0, 8.0 / 15.0};
    for (int k = 0; k < 3; ++k) {
        orc::compute_rhs(*s, t + b[k] * dt);
        const int64_t n = 5 * s->ndof;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            s->G[i] = a[k] * s->G[i] + s->QDot[i];
            s->Q[i] = s->Q[i] + c[k] * dt * s->G[i];
        }
    }
}

double orc_max_dt(void* h, double cfl, double dcfl) { return orc::max_dt(*static_cast<Solver*>(h), cfl, dcfl); }

// DGSEMClass.f90:770-868 ComputeMaxResiduals; returns 1 if Q holds a NaN (checkForNan).
int orc_residuals(void* h, double* res) {
    auto* s = static_cast<Solver*>(h);
    for (int v = 0; v < 5; ++v) res[v] = 0.0;
    int nan = 0;
    for (int64_t g = 0; g < s->ndof; ++g)
        for (int v = 0; v < 5; ++v) {
            res[v] = std::fmax(res[v], std::fabs(s->QDot[5 * g + v]));
            if (std::isnan(s->Q[5 * g + v])) nan = 1;
        }
    return nan;
}

// Manufactured solution of the Convergence case at the nodes: writes Q (and QDot) at time t.
void orc_mms_state(void* h, double t, double* q, double* qdot) {
    auto* s = static_cast<Solver*>(h);
    for (int64_t g = 0; g < s->ndof; ++g) {
        double S[5];
        orc::mms_point(s->x[3 * g], s->x[3 * g + 1], s->x[3 * g + 2], t, s->ph.gm1, s->ph.gammaM2, s->ph.mu, s->ph.kappa,
                       q + 5 * g, S, qdot ? qdot + 5 * g : S);
    }
}

}  // extern "C"
