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
__host__ __device__ __forceinline__ void face_normal(int f, double rx, double sx, double ry, double sy, double& nx,
                                                     double& ny, double& fsc) {
    double gx, gy;
    if (f == 0) { gx = -sx; gy = -sy; }
    else if (f == 1) { gx = rx + sx; gy = ry + sy; }
    else { gx = -rx; gy = -ry; }
    fsc = sqrt(gx * gx + gy * gy);
    nx = gx / fsc;
    ny = gy / fsc;
}

// FP32 version for the split path (GB300 runs FP64 sqrt/divide as long DFMA
// sequences at 1/70 of the FP32 rate)
__device__ __forceinline__ void face_normal_f(int f, float rx, float sx, float ry, float sy, float& nx, float& ny,
                                              float& fsc) {
    float gx, gy;
    if (f == 0) { gx = -sx; gy = -sy; }
    else if (f == 1) { gx = rx + sx; gy = ry + sy; }
    else { gx = -rx; gy = -ry; }
    fsc = sqrtf(gx * gx + gy * gy);
    const float inv = 1.f / fsc;
    nx = gx * inv;
    ny = gy * inv;
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

// ---------------------------------------------------------------------------
// Delta (product-rule) forms used by the split-precision path (FP32; the
// divisions use the fast approximate form: their results carry FP32-level
// relative error, inside the path's error budget).  With a
// per-element reference state qb and q = qb + dq, the weak right-hand side
// satisfies R(F) = R(F - F(qb)) exactly (the discrete divergence of a
// constant flux cancels against its own surface term), so the kernels feed the
// contractions with dF = F(qb + dq) - F(qb).  Written as below, dF carries
// FP32 round-off relative to |dq| instead of |q|: no cancellation.

struct RefState {
    float rho, m, n, E, u, v, p, H;  // H = E + p
};

__device__ __forceinline__ RefState make_ref(float gamma, const float qb[4]) {
    RefState b;
    b.rho = qb[0];
    b.m = qb[1];
    b.n = qb[2];
    b.E = qb[3];
    const float ir = __fdividef(1.f, b.rho);
    b.u = b.m * ir;
    b.v = b.n * ir;
    b.p = (gamma - 1.f) * (b.E - 0.5f * (b.m * b.u + b.n * b.v));
    b.H = b.E + b.p;
    return b;
}

// full velocities and pressure delta of q = qb + dq (helpers shared by the fluxes)
struct DeltaPrim {
    float rho, u, v, du, dv, dp, E;
};

__device__ __forceinline__ DeltaPrim delta_prim(float gamma, const RefState& b, const float dq[4]) {
    DeltaPrim d;
    d.rho = b.rho + dq[0];
    const float m = b.m + dq[1], n = b.n + dq[2];
    const float ir = __fdividef(1.f, d.rho);
    d.du = (dq[1] - b.u * dq[0]) * ir;
    d.dv = (dq[2] - b.v * dq[0]) * ir;
    d.u = b.u + d.du;
    d.v = b.v + d.dv;
    const float dK = 0.5f * (dq[1] * b.u + m * d.du + dq[2] * b.v + n * d.dv);
    d.dp = (gamma - 1.f) * (dq[3] - dK);
    d.E = b.E + dq[3];
    return d;
}

__device__ __forceinline__ void flux_delta(const RefState& b, const float dq[4], const DeltaPrim& d, float dFx[4],
                                           float dFy[4]) {
    const float m = b.m + dq[1], n = b.n + dq[2];
    const float dH = dq[3] + d.dp;
    dFx[0] = dq[1];
    dFx[1] = dq[1] * b.u + m * d.du + d.dp;
    dFx[2] = dq[2] * b.u + n * d.du;
    dFx[3] = d.du * b.H + d.u * dH;
    dFy[0] = dq[2];
    dFy[1] = dq[1] * b.v + m * d.dv;
    dFy[2] = dq[2] * b.v + n * d.dv + d.dp;
    dFy[3] = d.dv * b.H + d.v * dH;
}

__device__ __forceinline__ float wave_speed_delta(float gamma, float nx, float ny, const RefState& b, const DeltaPrim& d) {
    const float p = b.p + d.dp;
    return fabsf(d.u * nx + d.v * ny) + sqrtf(fabsf(__fdividef(gamma * p, d.rho)));
}

// n.F*(q-, q+) - n.F(qb), Lax-Friedrichs
__device__ __forceinline__ void lf_flux_delta(float nx, float ny, float lam, const RefState& b, const float dm[4],
                                              const DeltaPrim& pm, const float dpq[4], const DeltaPrim& pp, float F[4]) {
    float fxm[4], fym[4], fxp[4], fyp[4];
    flux_delta(b, dm, pm, fxm, fym);
    flux_delta(b, dpq, pp, fxp, fyp);
#pragma unroll
    for (int v = 0; v < 4; v++)
        F[v] = 0.5f * ((fxm[v] + fxp[v]) * nx + (fym[v] + fyp[v]) * ny) + 0.5f * lam * (dm[v] - dpq[v]);
}

// n.F*(q-, q+) - n.F(qb), Roe (RoeFlux.C:129-178 rearranged: central part in
// delta form, wave strengths from side-to-side jumps of the deltas)
__device__ __forceinline__ void roe_flux_delta(float gamma, float nx, float ny, const RefState& b, const float dm[4],
                                               const DeltaPrim& pm, const float dpq[4], const DeltaPrim& pp,
                                               float F[4]) {
    float fxm[4], fym[4], fxp[4], fyp[4];
    flux_delta(b, dm, pm, fxm, fym);
    flux_delta(b, dpq, pp, fxp, fyp);
    const float unM = nx * pm.u + ny * pm.v, unP = nx * pp.u + ny * pp.v;
    const float utM = nx * pm.v - ny * pm.u, utP = nx * pp.v - ny * pp.u;
    const float pM = b.p + pm.dp, pP = b.p + pp.dp;
    const float HM = (pm.E + pM) / pm.rho, HP = (pp.E + pP) / pp.rho;
    const float sM = sqrtf(pm.rho), sP = sqrtf(pp.rho);
    const float rhob = sM * sP;
    const float inv = 1.f / (sM + sP);
    const float u = (sM * unM + sP * unP) * inv;
    const float v = (sM * utM + sP * utP) * inv;
    const float H = (sM * HM + sP * HP) * inv;
    const float c2 = (gamma - 1.f) * (H - 0.5f * (u * u + v * v));
    const float c = sqrtf(fabsf(c2));
    const float jr = dpq[0] - dm[0];
    const float jdu = pp.du - pm.du, jdv = pp.dv - pm.dv;
    const float jun = nx * jdu + ny * jdv, jut = nx * jdv - ny * jdu;
    const float jp = pp.dp - pm.dp;
    const float dw1 = (-0.5f * rhob * jun / c + 0.5f * jp / c2) * fabsf(u - c);
    const float dw2 = (jr - jp / c2) * fabsf(u);
    const float dw3 = (rhob * jut) * fabsf(u);
    const float dw4 = (0.5f * rhob * jun / c + 0.5f * jp / c2) * fabsf(u + c);
    const float dr = dw1 + dw2 + dw4;
    const float du = dw1 * (u - c) + dw2 * u + dw4 * (u + c);
    const float dv = dr * v + dw3;
    const float de = dw1 * (H - u * c) + dw2 * (u * u + v * v) * 0.5f + dw3 * v + dw4 * (H + u * c);
    F[0] = 0.5f * ((fxm[0] + fxp[0]) * nx + (fym[0] + fyp[0]) * ny) - 0.5f * dr;
    F[1] = 0.5f * ((fxm[1] + fxp[1]) * nx + (fym[1] + fyp[1]) * ny) - 0.5f * (nx * du - ny * dv);
    F[2] = 0.5f * ((fxm[2] + fxp[2]) * nx + (fym[2] + fyp[2]) * ny) - 0.5f * (ny * du + nx * dv);
    F[3] = 0.5f * ((fxm[3] + fxp[3]) * nx + (fym[3] + fyp[3]) * ny) - 0.5f * de;
}

}  // namespace dgk
