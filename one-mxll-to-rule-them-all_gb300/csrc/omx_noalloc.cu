// omx_noalloc.cu -- an emitter step that allocates nothing.
//
// Some callers cannot call cudaMalloc: hosts that own all device memory through their own pool
// or through Fortran/OpenACC device arrays, and that forbid allocation in their time loop
// because cudaMalloc / cudaFree synchronise the whole device and would stall every stream the
// host keeps busy.  For them this file provides one entry point that advances a batch of
// few-level emitters and updates the emitter current arrays entirely in caller-provided device
// memory.  The only extra memory it needs -- the dP/dt of every emitter, produced by the
// density-matrix step and consumed by the current scatter -- lives in a fixed file-scope
// device array below.
//
// Compiled without FMA contraction, like every FP64 kernel of the library: the results equal
// the context API's (omx_qgroup_step) bit for bit for the same inputs.
#include <cuda_runtime.h>

#include <atomic>
#include <string>

#include "../../include/omx_gpu.h"
#include "omx_emitter.cuh"

namespace omx {
void set_global_error(const std::string &msg);
}

namespace {

// dP/dt scratch: 3 doubles per emitter, for at most OMX_NOALLOC_MAX_EMITTERS emitters.  Every
// GPU that loads the library holds it until the process exits.  All calls share it.
__device__ __align__(256) double g_noalloc_dpdt[3 * OMX_NOALLOC_MAX_EMITTERS];

// Address of g_noalloc_dpdt on each device, looked up once per device (host code cannot use the
// symbol's name as a device address: on the host it names a stand-in, not device memory).  Two
// host threads making their first call on a device at the same time may both look it up; they
// store the same value, and the atomic makes that store well defined.  The address belongs to
// the device's primary context: after cudaDeviceReset the library's state on that device,
// this cache included, is no longer valid, and the process must not call into it again.
constexpr int kMaxDevices = 64;
std::atomic<double *> g_scratch_addr[kMaxDevices] = {};

// td_propagate for every emitter from caller-provided E samples (the gathered E of
// send_E_to_J_ranks): RK4 density-matrix step, dipole, dP/dt into the scratch.
__global__ void k_emit_samples(int n, int model, int npar, int nst, const double *E, const double *par, double *rho,
                               double *dipole, double dt, double *dpdt)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const double *pr = par + (long long)e * npar;
    const double *u = pr + (npar - 3);
    const double Ex = E[3 * e], Ey = E[3 * e + 1], Ez = E[3 * e + 2];
    const double E_u = u[0] * Ex + u[1] * Ey + u[2] * Ez;
    double st[8];
    double *s = rho + (long long)e * nst;
    double d;
    if (model == OMX_EMITTER_TWO_LEVEL) {
#pragma unroll
        for (int q = 0; q < 3; ++q) st[q] = s[q];
        omx::rk4<3>(1, pr, st, E_u, dt);
#pragma unroll
        for (int q = 0; q < 3; ++q) s[q] = st[q];
        d = 2.0 * pr[1] * st[1];
    } else {
#pragma unroll
        for (int q = 0; q < 8; ++q) st[q] = s[q];
        omx::rk4<8>(2, pr, st, E_u, dt);
#pragma unroll
        for (int q = 0; q < 8; ++q) s[q] = st[q];
        d = 2.0 * pr[2] * st[2] + 2.0 * pr[3] * st[4];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double old = dipole[3 * e + a];
        const double nw = d * u[a];
        dipole[3 * e + a] = nw;
        dpdt[3 * e + a] = (nw - old) / dt;
    }
}

// send_J_to_E_ranks: J_old = J; J = wk * dP/dt of the winning emitter; dJ = (J - J_old)/dt.
__global__ void k_scatter_samples(int np, int n, int c0, int c1, const int *win, const double *wk, const double *dpdt,
                                  double *J, double *J_old, double *dJ, double dt)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const int w = win[p];
    const bool own = w >= 0 && w < n;   // indices outside this call's emitters do not write
    for (int c = c0; c <= c1; ++c) {
        const long long o = (long long)c * np + p;
        const double jo = J[o];
        const double jn = own ? wk[p] * dpdt[3 * w + c] : jo;
        J_old[o] = jo;
        J[o] = jn;
        dJ[o] = (jn - jo) / dt;
    }
}

int fail(int code, const char *msg)
{
    omx::set_global_error(msg);   // read back with omx_last_error(NULL)
    return code;
}

}  // namespace

extern "C" int omx_emitter_step_noalloc(int model, int n_emitters, const double *E, const double *params,
                                        double *rho, double *dipole, int n_points, const int *winner,
                                        const double *wk, double *J, double *J_old, double *dJ, int comp_first,
                                        int comp_last, double dt, void *stream)
{
    if (model != OMX_EMITTER_TWO_LEVEL && model != OMX_EMITTER_THREE_LEVEL)
        return fail(OMX_ERR_ARG, "omx_emitter_step_noalloc: unknown emitter model");
    if (n_emitters < 0 || n_emitters > OMX_NOALLOC_MAX_EMITTERS)
        return fail(OMX_ERR_ARG, "omx_emitter_step_noalloc: n_emitters exceeds OMX_NOALLOC_MAX_EMITTERS");
    if (n_points < 0 || comp_first < 0 || comp_last > 2 || comp_first > comp_last || !(dt > 0))
        return fail(OMX_ERR_ARG, "omx_emitter_step_noalloc: bad n_points, component range or dt");
    if ((n_emitters > 0 && (!E || !params || !rho || !dipole)) ||
        (n_points > 0 && (!winner || !wk || !J || !J_old || !dJ)))
        return fail(OMX_ERR_ARG, "omx_emitter_step_noalloc: null device pointer");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return fail(OMX_ERR_NODEV, "omx_emitter_step_noalloc: no usable CUDA device");
    }
    // first call on this device, with the device current: look the scratch address up (no
    // allocation); make this first call before any stream capture
    double *dpdt = g_scratch_addr[dev].load(std::memory_order_acquire);
    if (!dpdt) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_dpdt);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return fail(OMX_ERR_CUDA, "omx_emitter_step_noalloc: cudaGetSymbolAddress failed");
        }
        dpdt = static_cast<double *>(p);
        g_scratch_addr[dev].store(dpdt, std::memory_order_release);
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int npar = model == OMX_EMITTER_TWO_LEVEL ? 7 : 9;
    const int nst = model == OMX_EMITTER_TWO_LEVEL ? 3 : 8;
    if (n_emitters > 0)
        k_emit_samples<<<(n_emitters + 63) / 64, 64, 0, s>>>(n_emitters, model, npar, nst, E, params, rho, dipole, dt,
                                                             dpdt);
    if (n_points > 0)
        k_scatter_samples<<<(n_points + 127) / 128, 128, 0, s>>>(n_points, n_emitters, comp_first, comp_last, winner,
                                                                 wk, dpdt, J, J_old, dJ, dt);
    const cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess) return fail(OMX_ERR_CUDA, cudaGetErrorString(e));
    return OMX_OK;
}
