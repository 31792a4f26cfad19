// omx_emitter.cuh -- few-level density-matrix emitter arithmetic shared by the emitter kernels.
#pragma once

namespace omx {

// ---- few-level density-matrix emitters (new model behind TQ_sys_base%td_propagate) --------
// State (FP64): 2-level [p_e, Re rho_eg, Im rho_eg]; 3-level (V system)
// [p1, p2, Re r10, Im r10, Re r20, Im r20, Re r21, Im r21].  d rho/dt = -i[H0 - E_u V, rho]
// + T1 population decay to the ground state + T2 coherence decay, RK4 with E_u held over dt;
// the rates 1/T1, 1/T2 are formed once per step (FP64 division is expensive on this part).
__device__ __forceinline__ void rhs2(const double *pr, double E_u, double g1, double g2, const double *rho, double *d)
{
    const double w0 = pr[0], mu = pr[1];
    const double pe = rho[0], a = rho[1], b = rho[2];
    const double pg = 1.0 - pe;
    const double muE = mu * E_u;
    d[0] = 2.0 * muE * b - pe * g1;
    d[1] = w0 * b - a * g2;
    d[2] = -(w0 * a) + muE * (pg - pe) - b * g2;
}

__device__ __forceinline__ void rhs3(const double *pr, double E_u, double g1r, double g2r, const double *rho, double *d)
{
    const double e1 = pr[0], e2 = pr[1], mu1 = pr[2], mu2 = pr[3];
    const double p1 = rho[0], p2 = rho[1];
    const double a10 = rho[2], b10 = rho[3], a20 = rho[4], b20 = rho[5], a21 = rho[6], b21 = rho[7];
    const double p0 = 1.0 - p1 - p2;
    const double g1 = mu1 * E_u, g2 = mu2 * E_u;
    d[0] = 2.0 * g1 * b10 - p1 * g1r;
    d[1] = 2.0 * g2 * b20 - p2 * g1r;
    d[2] = e1 * b10 - g2 * b21 - a10 * g2r;
    d[3] = -(e1 * a10) + g1 * (p0 - p1) - g2 * a21 - b10 * g2r;
    d[4] = e2 * b20 + g1 * b21 - a20 * g2r;
    d[5] = -(e2 * a20) + g2 * (p0 - p2) - g1 * a21 - b20 * g2r;
    const double de = e2 - e1;
    d[6] = de * b21 + g2 * b10 + g1 * b20 - a21 * g2r;
    d[7] = -(de * a21) + g2 * a10 - g1 * a20 - b21 * g2r;
}

// One RK4 step with the decay rates g1 = 1/T1, g2 = 1/T2 and the step fractions h2 = dt/2,
// h6 = dt/6 supplied by the caller (formed once, not per emitter and step).
template <int NST>
__device__ __forceinline__ void rk4r(int model, const double *pr, double *rho, double E_u, double dt, double h2,
                                     double h6, double g1, double g2)
{
    double k1[NST], k2[NST], k3[NST], k4[NST], t[NST];
    if (model == 1) rhs2(pr, E_u, g1, g2, rho, k1); else rhs3(pr, E_u, g1, g2, rho, k1);
#pragma unroll
    for (int q = 0; q < NST; ++q) t[q] = rho[q] + h2 * k1[q];
    if (model == 1) rhs2(pr, E_u, g1, g2, t, k2); else rhs3(pr, E_u, g1, g2, t, k2);
#pragma unroll
    for (int q = 0; q < NST; ++q) t[q] = rho[q] + h2 * k2[q];
    if (model == 1) rhs2(pr, E_u, g1, g2, t, k3); else rhs3(pr, E_u, g1, g2, t, k3);
#pragma unroll
    for (int q = 0; q < NST; ++q) t[q] = rho[q] + dt * k3[q];
    if (model == 1) rhs2(pr, E_u, g1, g2, t, k4); else rhs3(pr, E_u, g1, g2, t, k4);
#pragma unroll
    for (int q = 0; q < NST; ++q) rho[q] = rho[q] + h6 * (k1[q] + 2.0 * k2[q] + 2.0 * k3[q] + k4[q]);
}

// Same step forming the rates and fractions itself.
template <int NST>
__device__ __forceinline__ void rk4(int model, const double *pr, double *rho, double E_u, double dt)
{
    const double g1 = 1.0 / pr[model == 1 ? 2 : 4], g2 = 1.0 / pr[model == 1 ? 3 : 5];
    rk4r<NST>(model, pr, rho, E_u, dt, 0.5 * dt, dt / 6.0, g1, g2);
}

}  // namespace omx
