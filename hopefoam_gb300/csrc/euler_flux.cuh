// euler_flux.cuh -- point-wise Euler fluxes (device), templated on the
// arithmetic type (double for the FP64 path, float for the split path).
#pragma once

namespace dgk {

// physical flux at a point; p = (gamma-1)(E - rho |U|^2 / 2) as gther_p of
// tutorials/DG/2D/isentropicVortex/dgEulerFoam/dgEulerFoam.C:81-82
template <typename T>
__device__ __forceinline__ void euler_phys_flux(T gamma, const T q[4], T fx[4], T fy[4]) {
    const T rho = q[0];
    const T u = q[1] / rho, v = q[2] / rho;
    const T p = (gamma - T(1)) * (q[3] - T(0.5) * (rho * (u * u + v * v)));
    fx[0] = q[1];
    fx[1] = u * q[1] + p;
    fx[2] = u * q[2];
    fx[3] = u * (q[3] + p);
    fy[0] = q[2];
    fy[1] = v * q[1];
    fy[2] = v * q[2] + p;
    fy[3] = v * (q[3] + p);
}

// outward unit normal and sJ/J of local face f of an affine triangle from its
// metrics (face 0: s = -1, face 1: r + s = 0, face 2: r = -1); equals the
// reference's faceNx / fscale (gaussTriangleIntegration.C:153-192,
// triangleBaseFunction.C:393-419) for straight edges.
__device__ __forceinline__ void face_normal(int f, double rx, double sx, double ry, double sy, double& nx, double& ny,
                                            double& fsc) {
    double gx, gy;
    if (f == 0) { gx = -sx; gy = -sy; }
    else if (f == 1) { gx = rx + sx; gy = ry + sy; }
    else { gx = -rx; gy = -ry; }
    fsc = sqrt(gx * gx + gy * gy);
    nx = gx / fsc;
    ny = gy / fsc;
}

template <typename T>
__device__ __forceinline__ T wave_speed(T gamma, T nx, T ny, const T q[4]) {
    const T rho = q[0], u = q[1] / rho, v = q[2] / rho;
    const T p = (gamma - T(1)) * (q[3] - T(0.5) * rho * (u * u + v * v));
    const T c = sqrt(fabs(gamma * p / rho));
    return fabs(u * nx + v * ny) + c;
}

// Euler Lax-Friedrichs (Rusanov): n.F* = 1/2 (F- + F+).n + 1/2 lam (q- - q+)
template <typename T>
__device__ __forceinline__ void lf_flux(T gamma, T nx, T ny, T lam, const T qm[4], const T qp[4], T F[4]) {
    T fxa[4], fya[4], fxb[4], fyb[4];
    euler_phys_flux(gamma, qm, fxa, fya);
    euler_phys_flux(gamma, qp, fxb, fyb);
#pragma unroll
    for (int v = 0; v < 4; v++)
        F[v] = T(0.5) * ((fxa[v] + fxb[v]) * nx + (fya[v] + fyb[v]) * ny) + T(0.5) * lam * (qm[v] - qp[v]);
}

// Roe flux in the face-normal frame, entropy fix 0
// (DG/godunovFlux/fluxSchemes/scheme/RoeFlux/RoeFlux.C:129-178).
template <typename T>
__device__ __forceinline__ void roe_flux(T gamma, T nx, T ny, const T qO[4], const T qN[4], T F[4]) {
    const T QP2 = nx * qN[1] + ny * qN[2], QM2 = nx * qO[1] + ny * qO[2];
    const T QP3 = nx * qN[2] - ny * qN[1], QM3 = nx * qO[2] - ny * qO[1];
    const T rhoP = qN[0], rhoM = qO[0];
    const T uM = QM2 / rhoM, uP = QP2 / rhoP, vM = QM3 / rhoM, vP = QP3 / rhoP;
    const T pM = (gamma - T(1)) * (qO[3] - T(0.5) * (QM2 * uM + QM3 * vM));
    const T pP = (gamma - T(1)) * (qN[3] - T(0.5) * (QP2 * uP + QP3 * vP));
    const T HM = (qO[3] + pM) / rhoM, HP = (qN[3] + pP) / rhoP;
    T fr = (QM2 + QP2) / T(2);
    T fu = (QM2 * uM + pM + QP2 * uP + pP) / T(2);
    T fv = (QM3 * uM + QP3 * uP) / T(2);
    T fe = (uM * (qO[3] + pM) + uP * (qN[3] + pP)) / T(2);
    const T rhoMs = sqrt(rhoM), rhoPs = sqrt(rhoP);
    const T rhob = rhoMs * rhoPs;
    const T u = (rhoMs * uM + rhoPs * uP) / (rhoMs + rhoPs);
    const T v = (rhoMs * vM + rhoPs * vP) / (rhoMs + rhoPs);
    const T H = (rhoMs * HM + rhoPs * HP) / (rhoMs + rhoPs);
    const T c2 = (gamma - T(1)) * (H - T(0.5) * (u * u + v * v));
    const T c = sqrt(fabs(c2));
    const T dw1 = (T(-0.5) * rhob * (uP - uM) / c + T(0.5) * (pP - pM) / c2) * fabs(u - c);
    const T dw2 = ((rhoP - rhoM) - (pP - pM) / c2) * fabs(u);
    const T dw3 = (rhob * (vP - vM)) * fabs(u);
    const T dw4 = (T(0.5) * rhob * (uP - uM) / c + T(0.5) * (pP - pM) / c2) * fabs(u + c);
    fr -= (dw1 + dw2 + dw4) / T(2);
    fu -= (dw1 * (u - c) + dw2 * u + dw4 * (u + c)) / T(2);
    fv -= (dw1 * v + dw2 * v + dw3 + dw4 * v) / T(2);
    fe -= (dw1 * (H - u * c) + dw2 * (u * u + v * v) / T(2) + dw3 * v + dw4 * (H + u * c)) / T(2);
    F[0] = fr;
    F[1] = nx * fu - ny * fv;
    F[2] = ny * fu + nx * fv;
    F[3] = fe;
}

}  // namespace dgk
