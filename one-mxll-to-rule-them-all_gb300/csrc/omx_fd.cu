// omx_fd.cu -- the frequency-domain operator of the reference's inverse-design program on the GPU
// (src/freq_domain_inverse_design/operator_mod.f90: apply_operator_1D :293-361, _2D :364-514,
// _3D :518-710) and its BiCGStab(L) solver (bicgstab_mod.f90:76-243).
//
// Vectors are complex components (Riemann-Silberstein pl_x, pl_y, pl_z, mi_x, mi_y, mi_z; in 1D
// pl_x, pl_y, mi_x, mi_y), each an array over [1-g, n+g] along every active axis (g = n_der
// ghost cells), x fastest, FP64 as in the reference.
// The operator kernel keeps the reference's operand order with FMA contraction off (this file is
// compiled with -fmad=false), so A f equals the FP64 oracle bit for bit.  The solver's scalar
// recursion runs on the host exactly as the oracle's; its dot products are reduced on the device
// per block and summed on the host in block order (deterministic, not the oracle's order).
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "../../include/omx_gpu.h"

namespace omx {
void set_global_error(const std::string &msg);
}

namespace {

struct cplx {
    double re, im;
};
__host__ __device__ inline cplx cadd(cplx a, cplx b) { return {a.re + b.re, a.im + b.im}; }
__host__ __device__ inline cplx csub(cplx a, cplx b) { return {a.re - b.re, a.im - b.im}; }
__host__ __device__ inline cplx cmul(cplx a, cplx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__host__ __device__ inline cplx cscale(cplx a, double s) { return {a.re * s, a.im * s}; }
// complex division by Smith's method (R. L. Smith, CACM 5:435, 1962), the range-reduced form
// gfortran uses for complex(dp) division under its default Fortran rules
inline cplx cdiv(cplx a, cplx b)
{
    if (std::fabs(b.re) < std::fabs(b.im)) {
        const double t = b.re / b.im, d = b.re * t + b.im;
        return {(a.re * t + a.im) / d, (a.im * t - a.re) / d};
    }
    const double t = b.im / b.re, d = b.im * t + b.re;
    return {(a.im * t + a.re) / d, (a.im - a.re * t) / d};
}

struct FdGeom {
    int dims, ncomp, nx, ny, nz, g, gy, gz, n_der;   // ny = nz = 1 in 1D, nz = 1 in 2D
    long long px, pxy, len;   // padded row and plane pitch, elements per component
    int per[3];
    double coef[9];
    double w0, sign;
};

__device__ inline long long fd_at(const FdGeom &G, int i, int j, int k)   // 1-based interior indices
{
    return (long long)(i - 1 + G.g) + G.px * (j - 1 + G.gy) + G.pxy * (k - 1 + G.gz);
}

// periodic ghost copies (1D operator_mod.f90:316-329, 2D :389-452, 3D :549-621): axis 0 over
// interior y, z; axis 1 over interior x, z (in 3D with mi_x only into the low ghosts and mi_y only
// into the high ones); axis 2 over interior x, y.  One thread per (component, ghost cell pair).
__global__ void k_fd_ghosts(cplx *f, FdGeom G, int axis)
{
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int na = axis == 0 ? G.nx : (axis == 1 ? G.ny : G.nz);
    const int n1 = axis == 0 ? G.ny : G.nx, n2 = axis == 2 ? G.ny : G.nz;
    const long long per_c = (long long)G.g * n1 * n2;
    if (q >= G.ncomp * per_c) return;
    const int c = (int)(q / per_c);
    long long r = q % per_c;
    const int t = 1 + (int)(r % G.g);
    r /= G.g;
    const int a1 = 1 + (int)(r % n1), a2 = 1 + (int)(r / n1);
    cplx *v = f + c * G.len;
    auto at = [&](int s) {
        if (axis == 0) return fd_at(G, s, a1, a2);
        if (axis == 1) return fd_at(G, a1, s, a2);
        return fd_at(G, a1, a2, s);
    };
    const bool quirk = axis == 1 && G.dims == 3;
    const bool lo = !(quirk && c == 4), hi = !(quirk && c == 3);
    if (lo) v[at(1 - t)] = v[at(na + 1 - t)];
    if (hi) v[at(na + t)] = v[at(t)];
}

// apply_operator_3D: one thread per interior cell
__global__ void __launch_bounds__(128) k_fd_apply(const cplx *__restrict__ f, cplx *__restrict__ Af, FdGeom G,
                                                  const cplx *__restrict__ sx, const cplx *__restrict__ sy,
                                                  const cplx *__restrict__ sz, const cplx *__restrict__ eps)
{
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x, j = 1 + blockIdx.y, k = 1 + blockIdx.z;
    if (i > G.nx) return;
    const long long p = fd_at(G, i, j, k);
    const cplx *plx = f, *ply = f + G.len, *plz = f + 2 * G.len, *mix = f + 3 * G.len, *miy = f + 4 * G.len,
               *miz = f + 5 * G.len;
    const int n = G.n_der;
    cplx dpydx = {0, 0}, dpzdx = {0, 0}, dmydx = {0, 0}, dmzdx = {0, 0};
    cplx dpxdy = {0, 0}, dpzdy = {0, 0}, dmxdy = {0, 0}, dmzdy = {0, 0};
    cplx dpxdz = {0, 0}, dpydz = {0, 0}, dmxdz = {0, 0}, dmydz = {0, 0};
    for (int q = -n; q <= n; ++q) {
        const double a = G.coef[n + q];
        dpydx = cadd(dpydx, cscale(ply[p + q], a));
        dpzdx = cadd(dpzdx, cscale(plz[p + q], a));
        dmydx = cadd(dmydx, cscale(miy[p + q], a));
        dmzdx = cadd(dmzdx, cscale(miz[p + q], a));
    }
    for (int q = -n; q <= n; ++q) {
        const double a = G.coef[n + q];
        const long long o = p + q * G.px;
        dpxdy = cadd(dpxdy, cscale(plx[o], a));
        dpzdy = cadd(dpzdy, cscale(plz[o], a));
        dmxdy = cadd(dmxdy, cscale(mix[o], a));
        dmzdy = cadd(dmzdy, cscale(miz[o], a));
    }
    for (int q = -n; q <= n; ++q) {
        const double a = G.coef[n + q];
        const long long o = p + q * G.pxy;
        dpxdz = cadd(dpxdz, cscale(plx[o], a));
        dpydz = cadd(dpydz, cscale(ply[o], a));
        dmxdz = cadd(dmxdz, cscale(mix[o], a));
        dmydz = cadd(dmydz, cscale(miy[o], a));
    }
    const cplx Ex = cadd(plx[p], mix[p]), Ey = cadd(ply[p], miy[p]), Ez = cadd(plz[p], miz[p]);
    const cplx sxi = sx[i - 1], syj = sy[j - 1], szk = sz[k - 1];
    dpxdy = cmul(dpxdy, syj);
    dpxdz = cmul(dpxdz, szk);
    dpydx = cmul(dpydx, sxi);
    dpydz = cmul(dpydz, szk);
    dpzdx = cmul(dpzdx, sxi);
    dpzdy = cmul(dpzdy, syj);
    dmxdy = cmul(dmxdy, syj);
    dmxdz = cmul(dmxdz, szk);
    dmydz = cmul(dmydz, szk);
    dmydx = cmul(dmydx, sxi);
    dmzdx = cmul(dmzdx, sxi);
    dmzdy = cmul(dmzdy, syj);
    // C1 = sign c0 i, C2 = -w0 i, C3 = -w0 i / (2 eps0), C4 = eps0 (c0 = eps0 = 1)
    const cplx C1 = {0.0, G.sign}, mC1 = {-0.0, -G.sign}, C2 = {0.0, -G.w0}, C3 = {0.0, -G.w0 / 2.0}, C4 = {1.0, 0.0};
    const cplx e = eps[(long long)(i - 1) + (long long)G.nx * ((j - 1) + (long long)G.ny * (k - 1))];
    const cplx m3 = cmul(C3, csub(e, C4));
    Af[p] = cadd(cadd(cmul(C1, csub(dpzdy, dpydz)), cmul(C2, plx[p])), cmul(m3, Ex));
    Af[p + G.len] = cadd(cadd(cmul(C1, csub(dpxdz, dpzdx)), cmul(C2, ply[p])), cmul(m3, Ey));
    Af[p + 2 * G.len] = cadd(cadd(cmul(C1, csub(dpydx, dpxdy)), cmul(C2, plz[p])), cmul(m3, Ez));
    Af[p + 3 * G.len] = cadd(cadd(cmul(mC1, csub(dmzdy, dmydz)), cmul(C2, mix[p])), cmul(m3, Ex));
    Af[p + 4 * G.len] = cadd(cadd(cmul(mC1, csub(dmxdz, dmzdx)), cmul(C2, miy[p])), cmul(m3, Ey));
    Af[p + 5 * G.len] = cadd(cadd(cmul(mC1, csub(dmydx, dmxdy)), cmul(C2, miz[p])), cmul(m3, Ez));
}

// apply_operator_1D: one thread per cell; the products keep the reference's order C1 * d * s_inv,
// and the y components carry no medium term (as written in the reference)
__global__ void __launch_bounds__(128) k_fd_apply1(const cplx *__restrict__ f, cplx *__restrict__ Af, FdGeom G,
                                                   const cplx *__restrict__ sx, const cplx *__restrict__ eps)
{
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i > G.nx) return;
    const long long p = fd_at(G, i, 1, 1);
    const cplx *plx = f, *ply = f + G.len, *mix = f + 2 * G.len, *miy = f + 3 * G.len;
    const int n = G.n_der;
    cplx dpxdz = {0, 0}, dpydz = {0, 0}, dmxdz = {0, 0}, dmydz = {0, 0};
    for (int q = -n; q <= n; ++q) {
        const double a = G.coef[n + q];
        dpxdz = cadd(dpxdz, cscale(plx[p + q], a));
        dpydz = cadd(dpydz, cscale(ply[p + q], a));
        dmxdz = cadd(dmxdz, cscale(mix[p + q], a));
        dmydz = cadd(dmydz, cscale(miy[p + q], a));
    }
    const cplx C1 = {0.0, G.sign}, mC1 = {-0.0, -G.sign}, C2 = {0.0, -G.w0}, C3 = {0.0, -G.w0 / 2.0}, C4 = {1.0, 0.0};
    const cplx Ex = cadd(plx[p], mix[p]);
    const cplx s = sx[i - 1], e = eps[i - 1];
    const cplx m3 = cmul(C3, csub(e, C4));
    Af[p] = cadd(cadd(cmul(cmul(mC1, dpydz), s), cmul(C2, plx[p])), cmul(m3, Ex));
    Af[p + G.len] = cadd(cmul(cmul(C1, dpxdz), s), cmul(C2, ply[p]));
    Af[p + 2 * G.len] = cadd(cadd(cmul(cmul(C1, dmydz), s), cmul(C2, mix[p])), cmul(m3, Ex));
    Af[p + 3 * G.len] = cadd(cmul(cmul(mC1, dmxdz), s), cmul(C2, miy[p]));
}

// apply_operator_2D: one thread per cell; the curl terms carry the opposite sign of the 3D
// operator's (as written in the reference)
__global__ void __launch_bounds__(128) k_fd_apply2(const cplx *__restrict__ f, cplx *__restrict__ Af, FdGeom G,
                                                   const cplx *__restrict__ sx, const cplx *__restrict__ sy,
                                                   const cplx *__restrict__ eps)
{
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x, j = 1 + blockIdx.y;
    if (i > G.nx) return;
    const long long p = fd_at(G, i, j, 1);
    const cplx *plx = f, *ply = f + G.len, *plz = f + 2 * G.len, *mix = f + 3 * G.len, *miy = f + 4 * G.len,
               *miz = f + 5 * G.len;
    const int n = G.n_der;
    cplx dpxdy = {0, 0}, dpydx = {0, 0}, dpzdx = {0, 0}, dpzdy = {0, 0};
    cplx dmxdy = {0, 0}, dmydx = {0, 0}, dmzdx = {0, 0}, dmzdy = {0, 0};
    for (int q = -n; q <= n; ++q) {
        const double a = G.coef[n + q];
        dpydx = cadd(dpydx, cscale(ply[p + q], a));
        dpzdx = cadd(dpzdx, cscale(plz[p + q], a));
        dmydx = cadd(dmydx, cscale(miy[p + q], a));
        dmzdx = cadd(dmzdx, cscale(miz[p + q], a));
    }
    for (int q = -n; q <= n; ++q) {
        const double a = G.coef[n + q];
        const long long o = p + q * G.px;
        dpxdy = cadd(dpxdy, cscale(plx[o], a));
        dpzdy = cadd(dpzdy, cscale(plz[o], a));
        dmxdy = cadd(dmxdy, cscale(mix[o], a));
        dmzdy = cadd(dmzdy, cscale(miz[o], a));
    }
    const cplx Ex = cadd(plx[p], mix[p]), Ey = cadd(ply[p], miy[p]), Ez = cadd(plz[p], miz[p]);
    const cplx sxi = sx[i - 1], syj = sy[j - 1];
    dpxdy = cmul(dpxdy, syj);
    dpydx = cmul(dpydx, sxi);
    dpzdx = cmul(dpzdx, sxi);
    dpzdy = cmul(dpzdy, syj);
    dmxdy = cmul(dmxdy, syj);
    dmydx = cmul(dmydx, sxi);
    dmzdx = cmul(dmzdx, sxi);
    dmzdy = cmul(dmzdy, syj);
    const cplx C1 = {0.0, G.sign}, mC1 = {-0.0, -G.sign}, C2 = {0.0, -G.w0}, C3 = {0.0, -G.w0 / 2.0}, C4 = {1.0, 0.0};
    const cplx e = eps[(long long)(i - 1) + (long long)G.nx * (j - 1)];
    const cplx m3 = cmul(C3, csub(e, C4));
    Af[p] = cadd(cadd(cmul(mC1, dpzdy), cmul(C2, plx[p])), cmul(m3, Ex));
    Af[p + G.len] = cadd(cadd(cmul(C1, dpzdx), cmul(C2, ply[p])), cmul(m3, Ey));
    Af[p + 2 * G.len] = cadd(cadd(cmul(mC1, csub(dpydx, dpxdy)), cmul(C2, plz[p])), cmul(m3, Ez));
    Af[p + 3 * G.len] = cadd(cadd(cmul(C1, dmzdy), cmul(C2, mix[p])), cmul(m3, Ex));
    Af[p + 4 * G.len] = cadd(cadd(cmul(mC1, dmzdx), cmul(C2, miy[p])), cmul(m3, Ey));
    Af[p + 5 * G.len] = cadd(cadd(cmul(C1, csub(dmydx, dmxdy)), cmul(C2, miz[p])), cmul(m3, Ez));
}

// vector operations over the interior of every component (rs_operations_subs_mod.f90)
// mode 0: v1 = v1 + a v2;  mode 1: v1 = a v1 + v2;  mode 2: v1 = a v1
__global__ void k_fd_lin(cplx *v1, const cplx *v2, cplx a, FdGeom G, int mode)
{
    const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x, j = 1 + blockIdx.y, k = 1 + blockIdx.z;
    if (i > G.nx) return;
    const long long p = fd_at(G, i, j, k);
    for (int c = 0; c < G.ncomp; ++c) {
        const long long q = p + c * G.len;
        const cplx x = v1[q];
        if (mode == 0) v1[q] = cadd(x, cmul(a, v2[q]));
        else if (mode == 1) v1[q] = cadd(cmul(a, x), v2[q]);
        else v1[q] = cmul(a, x);
    }
}

// per-block partial sums of conj(v1) v2 over the interior (one block per (j, k) row)
__global__ void k_fd_dot(const cplx *v1, const cplx *v2, FdGeom G, cplx *part)
{
    __shared__ cplx sh[128];
    const int j = 1 + blockIdx.x, k = 1 + blockIdx.y;
    cplx s = {0, 0};
    for (int c = 0; c < G.ncomp; ++c)
        for (int i = 1 + threadIdx.x; i <= G.nx; i += blockDim.x) {
            const long long q = fd_at(G, i, j, k) + c * G.len;
            const cplx a = {v1[q].re, -v1[q].im};
            s = cadd(s, cmul(a, v2[q]));
        }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] = cadd(sh[threadIdx.x], sh[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x + (long long)gridDim.x * blockIdx.y] = sh[0];
}

}  // namespace

struct omx_fdop {
    FdGeom G{};
    cudaStream_t s = nullptr;
    cplx *sx = nullptr, *sy = nullptr, *sz = nullptr, *eps = nullptr;
    cplx *part = nullptr, *hpart = nullptr;
    std::vector<cplx *> vecs;   // solver work vectors
    ~omx_fdop()
    {
        cudaFree(sx);
        cudaFree(sy);
        cudaFree(sz);
        cudaFree(eps);
        cudaFree(part);
        if (hpart) cudaFreeHost(hpart);
        for (auto *v : vecs) cudaFree(v);
        if (s) cudaStreamDestroy(s);
    }
};

namespace {

int fd_fail(int code, const std::string &m)
{
    omx::set_global_error("omx_fd: " + m);
    return code;
}

struct FdErr {
    int code;
    std::string msg;
};
void fck(cudaError_t e, const char *w)
{
    if (e != cudaSuccess) throw FdErr{OMX_ERR_CUDA, std::string(w) + ": " + cudaGetErrorString(e)};
}

dim3 cell_grid(const FdGeom &G) { return dim3((G.nx + 127) / 128, G.ny, G.nz); }

void fd_apply_dev(omx_fdop *op, cplx *f, cplx *Af)
{
    const FdGeom &G = op->G;
    for (int a = 0; a < G.dims; ++a) {
        if (!G.per[a]) continue;
        const int n1 = a == 0 ? G.ny : G.nx, n2 = a == 2 ? G.ny : G.nz;
        const long long cnt = (long long)G.ncomp * G.g * n1 * n2;
        k_fd_ghosts<<<(unsigned)((cnt + 255) / 256), 256, 0, op->s>>>(f, G, a);
    }
    if (G.dims == 1) k_fd_apply1<<<cell_grid(G), 128, 0, op->s>>>(f, Af, G, op->sx, op->eps);
    else if (G.dims == 2) k_fd_apply2<<<cell_grid(G), 128, 0, op->s>>>(f, Af, G, op->sx, op->sy, op->eps);
    else k_fd_apply<<<cell_grid(G), 128, 0, op->s>>>(f, Af, G, op->sx, op->sy, op->sz, op->eps);
}

void fd_lin(omx_fdop *op, cplx *v1, const cplx *v2, cplx a, int mode)
{
    k_fd_lin<<<cell_grid(op->G), 128, 0, op->s>>>(v1, v2, a, op->G, mode);
}

cplx fd_dot(omx_fdop *op, const cplx *v1, const cplx *v2)
{
    const FdGeom &G = op->G;
    k_fd_dot<<<dim3(G.ny, G.nz), 128, 0, op->s>>>(v1, v2, G, op->part);
    const size_t nb = (size_t)G.ny * G.nz;
    fck(cudaMemcpyAsync(op->hpart, op->part, nb * sizeof(cplx), cudaMemcpyDeviceToHost, op->s), "dot");
    fck(cudaStreamSynchronize(op->s), "dot");
    cplx s = {0, 0};
    for (size_t b = 0; b < nb; ++b) s = cadd(s, op->hpart[b]);
    return s;
}

}  // namespace

extern "C" {

int omx_fd_create(int dimensions, const int grid_Ndims[3], int n_pml, int n_der, const int boundaries[3], double dr,
                  double w0, const double *eps_r, omx_fdop **out)
{
    if (!grid_Ndims || !boundaries || !eps_r || !out || n_der < 1 || n_der > 4 || !(dr > 0) || !(w0 > 0) ||
        dimensions < 1 || dimensions > 3)
        return fd_fail(OMX_ERR_ARG, "bad argument (dimensions 1..3, n_der 1..4)");
    for (int a = 0; a < dimensions; ++a) {
        if (grid_Ndims[a] < 1) return fd_fail(OMX_ERR_ARG, "grid sizes must be >= 1");
        if (boundaries[a] < 1 || boundaries[a] > 3) return fd_fail(OMX_ERR_ARG, "boundaries: 1 close, 2 periodic, 3 PML");
        if (boundaries[a] == 3 && grid_Ndims[a] < 2 * n_pml) return fd_fail(OMX_ERR_ARG, "PML slabs do not fit");
        if (boundaries[a] == 2 && grid_Ndims[a] < n_der) return fd_fail(OMX_ERR_ARG, "periodic axis shorter than the stencil");
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fd_fail(OMX_ERR_NODEV, "no CUDA device");
    }
    *out = nullptr;
    omx_fdop *op = new omx_fdop;
    try {
        FdGeom &G = op->G;
        G.dims = dimensions;
        G.ncomp = dimensions == 1 ? 4 : 6;
        G.nx = grid_Ndims[0];
        G.ny = dimensions >= 2 ? grid_Ndims[1] : 1;
        G.nz = dimensions == 3 ? grid_Ndims[2] : 1;
        G.g = n_der;
        G.gy = dimensions >= 2 ? n_der : 0;
        G.gz = dimensions == 3 ? n_der : 0;
        G.n_der = n_der;
        G.px = G.nx + 2 * G.g;
        G.pxy = G.px * (G.ny + 2 * G.gy);
        G.len = G.pxy * (G.nz + 2 * G.gz);
        for (int a = 0; a < 3; ++a) G.per[a] = a < dimensions && boundaries[a] == 2;
        G.w0 = w0;
        // operator_mod.f90:97-140: central-difference coefficients of order 2 n_der, / dr
        static const double C[4][9] = {{-0.5, 0.0, 0.5},
                                       {1.0 / 12.0, -2.0 / 3.0, 0.0, 2.0 / 3.0, -1.0 / 12.0},
                                       {-1.0 / 60.0, 3.0 / 20.0, -3.0 / 4.0, 0.0, 3.0 / 4.0, -3.0 / 20.0, 1.0 / 60.0},
                                       {1.0 / 280.0, -4.0 / 105.0, 1.0 / 5.0, -4.0 / 5.0, 0.0, 4.0 / 5.0, -1.0 / 5.0,
                                        4.0 / 105.0, -1.0 / 280.0}};
        for (int q = 0; q <= 2 * n_der; ++q) G.coef[q] = C[n_der - 1][q] / dr;
        // :185-232: s_inv = 1 / (kappa + sig / (i w0 eps0)) on the PML faces, 1 elsewhere
        const int n[3] = {G.nx, G.ny, G.nz};
        std::vector<cplx> s[3];
        const double m = 3.0, kmax = 5.0, sig_max = 0.8 * (m + 1.0) / (dr * std::sqrt(1.0 / 1.0));
        for (int a = 0; a < 3; ++a) {
            s[a].assign(n[a], cplx{1.0, 0.0});
            if (a >= dimensions || boundaries[a] != 3) continue;
            for (int i = 1; i <= n_pml; ++i) {
                const double r = (double)(n_pml - i + 1) / (double)n_pml;
                const double sig = sig_max * std::pow(r, m);
                const double kap = 1.0 + (kmax - 1.0) * std::pow(r, m);
                const cplx si = {kap, -(sig / w0)};
                s[a][i - 1] = cdiv(cplx{1.0, 0.0}, si);
                s[a][n[a] - n_pml + (n_pml - i)] = cdiv(cplx{1.0, 0.0}, si);
            }
        }
        fck(cudaStreamCreateWithFlags(&op->s, cudaStreamNonBlocking), "stream");
        cplx **dst[3] = {&op->sx, &op->sy, &op->sz};
        for (int a = 0; a < 3; ++a) {
            fck(cudaMalloc(dst[a], sizeof(cplx) * n[a]), "alloc");
            fck(cudaMemcpy(*dst[a], s[a].data(), sizeof(cplx) * n[a], cudaMemcpyHostToDevice), "upload");
            fck(cudaStreamSynchronize(0), "upload");   // pageable copies may return before their DMA ends
        }
        const size_t ncell = (size_t)G.nx * G.ny * G.nz;
        fck(cudaMalloc(&op->eps, sizeof(cplx) * ncell), "alloc");
        fck(cudaMemcpy(op->eps, eps_r, sizeof(cplx) * ncell, cudaMemcpyHostToDevice), "upload");
        fck(cudaStreamSynchronize(0), "upload");   // pageable copies may return before their DMA ends
        fck(cudaMalloc(&op->part, sizeof(cplx) * (size_t)G.ny * G.nz), "alloc");
        fck(cudaMallocHost(&op->hpart, sizeof(cplx) * (size_t)G.ny * G.nz), "alloc");
    } catch (const FdErr &e) {
        delete op;
        return fd_fail(e.code, e.msg);
    }
    *out = op;
    return OMX_OK;
}

int omx_fd_set_eps(omx_fdop *op, const double *eps_r)
{
    if (!op || !eps_r) return fd_fail(OMX_ERR_ARG, "null argument");
    try {
        const size_t ncell = (size_t)op->G.nx * op->G.ny * op->G.nz;
        fck(cudaMemcpyAsync(op->eps, eps_r, sizeof(cplx) * ncell, cudaMemcpyHostToDevice, op->s), "upload");
        fck(cudaStreamSynchronize(op->s), "upload");
    } catch (const FdErr &e) {
        return fd_fail(e.code, e.msg);
    }
    return OMX_OK;
}

int omx_fd_destroy(omx_fdop *op)
{
    if (op) {
        cudaStreamSynchronize(op->s);
        delete op;
    }
    return OMX_OK;
}

long long omx_fd_vector_length(const omx_fdop *op) { return op ? (long long)op->G.ncomp * op->G.len : 0; }

int omx_fd_apply(omx_fdop *op, const double *f, double *Af, int transpose)
{
    if (!op || !f || !Af) return fd_fail(OMX_ERR_ARG, "null argument");
    cplx *df = nullptr, *dAf = nullptr;
    try {
        op->G.sign = transpose ? -1.0 : 1.0;
        const size_t bytes = sizeof(cplx) * op->G.ncomp * op->G.len;
        fck(cudaMalloc(&df, bytes), "alloc");
        fck(cudaMalloc(&dAf, bytes), "alloc");
        fck(cudaMemcpy(df, f, bytes, cudaMemcpyHostToDevice), "upload");
        fck(cudaStreamSynchronize(0), "upload");   // pageable copies may return before their DMA ends
        fck(cudaMemsetAsync(dAf, 0, bytes, op->s), "memset");
        fd_apply_dev(op, df, dAf);
        fck(cudaStreamSynchronize(op->s), "apply");
        fck(cudaMemcpy(Af, dAf, bytes, cudaMemcpyDeviceToHost), "download");
    } catch (const FdErr &e) {
        cudaFree(df);
        cudaFree(dAf);
        return fd_fail(e.code, e.msg);
    }
    cudaFree(df);
    cudaFree(dAf);
    return OMX_OK;
}

// Mean time of `reps` operator applications on device-resident vectors (random interior values),
// CUDA events on the operator's stream.
int omx_fd_time_apply(omx_fdop *op, int reps, double *ms_per_apply)
{
    if (!op || reps < 1 || !ms_per_apply) return fd_fail(OMX_ERR_ARG, "bad argument");
    cplx *df = nullptr, *dAf = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    try {
        op->G.sign = 1.0;
        const size_t n = (size_t)op->G.ncomp * op->G.len;
        std::vector<cplx> h(n);
        unsigned long long x = 88172645463325252ull;
        for (auto &v : h) {
            x ^= x << 13;
            x ^= x >> 7;
            x ^= x << 17;
            v = {(double)(x >> 11) * (1.0 / 9007199254740992.0) - 0.5, (double)(x & 0xffff) / 65536.0 - 0.5};
        }
        fck(cudaMalloc(&df, n * sizeof(cplx)), "alloc");
        fck(cudaMalloc(&dAf, n * sizeof(cplx)), "alloc");
        fck(cudaMemcpy(df, h.data(), n * sizeof(cplx), cudaMemcpyHostToDevice), "upload");
        fck(cudaStreamSynchronize(0), "upload");   // pageable copies may return before their DMA ends
        fck(cudaEventCreate(&e0), "event");
        fck(cudaEventCreate(&e1), "event");
        for (int r = 0; r < 2; ++r) fd_apply_dev(op, df, dAf);
        fck(cudaEventRecord(e0, op->s), "event");
        for (int r = 0; r < reps; ++r) fd_apply_dev(op, df, dAf);
        fck(cudaEventRecord(e1, op->s), "event");
        fck(cudaEventSynchronize(e1), "apply");
        float ms = 0.f;
        fck(cudaEventElapsedTime(&ms, e0, e1), "event");
        *ms_per_apply = ms / reps;
    } catch (const FdErr &e) {
        cudaFree(df);
        cudaFree(dAf);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        return fd_fail(e.code, e.msg);
    }
    cudaFree(df);
    cudaFree(dAf);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return OMX_OK;
}

// BICGStab_L (bicgstab_mod.f90:76-243), the oracle's scalar recursion on the host
int omx_fd_solve(omx_fdop *op, const double *j_vec, double *f_io, int transpose, double tol, int n_max, int L,
                 int *converged, double *abs_err, int *iterations)
{
    if (!op || !j_vec || !f_io || L < 1 || L > 8 || n_max < 0 || !(tol > 0)) return fd_fail(OMX_ERR_ARG, "bad argument");
    try {
        FdGeom &G = op->G;
        G.sign = transpose ? -1.0 : 1.0;
        const size_t bytes = sizeof(cplx) * G.ncomp * G.len;
        const size_t need = 5 + 2 * (size_t)(L + 1);
        while (op->vecs.size() < need) {
            cplx *v = nullptr;
            fck(cudaMalloc(&v, bytes), "alloc");
            op->vecs.push_back(v);
        }
        cplx *r0 = op->vecs[0], *f = op->vecs[1], *Af = op->vecs[2], *jv = op->vecs[3], *f_out = op->vecs[4];
        cplx *r[9], *u[9];
        for (int l = 0; l <= L; ++l) {
            r[l] = op->vecs[5 + l];
            u[l] = op->vecs[5 + L + 1 + l];
        }
        for (size_t q = 0; q < need; ++q) fck(cudaMemsetAsync(op->vecs[q], 0, bytes, op->s), "memset");
        fck(cudaMemcpyAsync(f, f_io, bytes, cudaMemcpyHostToDevice, op->s), "upload");
        fck(cudaMemcpyAsync(jv, j_vec, bytes, cudaMemcpyHostToDevice, op->s), "upload");
        fck(cudaMemcpyAsync(f_out, f_io, bytes, cudaMemcpyHostToDevice, op->s), "upload");
        cplx tau[9][9] = {}, gam[9] = {}, gam_p[9] = {}, gam_pp[9] = {}, sig[9] = {};
        cplx rho0 = {1, 0}, rho1 = {1, 0}, alpha = {1, 0}, omega = {1, 0}, beta, dot;
        fd_apply_dev(op, f, Af);
        fck(cudaMemcpyAsync(r0, jv, bytes, cudaMemcpyDeviceToDevice, op->s), "copy");
        fd_lin(op, r0, Af, cplx{-1.0, 0.0}, 0);                 // r0 = j - A f
        fck(cudaMemcpyAsync(r[0], r0, bytes, cudaMemcpyDeviceToDevice, op->s), "copy");
        dot = fd_dot(op, r0, r0);
        double norm_t = std::sqrt(dot.re);
        fd_lin(op, r0, nullptr, cplx{1.0 / norm_t, 0.0}, 2);    // r0 = r0 / |r0|
        dot = fd_dot(op, jv, jv);
        norm_t = std::sqrt(dot.re);
        double err_r = 1.0;
        int n = 0, conv = 0;
        while (n <= n_max && !conv) {
            rho0 = cmul(cscale(omega, -1.0), rho0);
            for (int l = 0; l <= L - 1; ++l) {
                dot = fd_dot(op, r0, r[l]);
                rho1 = dot;
                beta = cdiv(cmul(alpha, rho1), rho0);
                rho0 = rho1;
                for (int i = 0; i <= l; ++i) fd_lin(op, u[i], r[i], cscale(beta, -1.0), 1);
                fd_apply_dev(op, u[l], u[l + 1]);
                dot = fd_dot(op, r0, u[l + 1]);
                alpha = cdiv(rho0, dot);
                for (int i = 0; i <= l; ++i) fd_lin(op, r[i], u[i + 1], cscale(alpha, -1.0), 0);
                fd_apply_dev(op, r[l], r[l + 1]);
                fd_lin(op, f_out, u[0], alpha, 0);
            }
            for (int l = 1; l <= L; ++l) {
                for (int i = 1; i <= l - 1; ++i) {
                    dot = fd_dot(op, r[i], r[l]);
                    tau[i][l] = cdiv(dot, sig[i]);
                    fd_lin(op, r[l], r[i], cscale(tau[i][l], -1.0), 0);
                }
                sig[l] = fd_dot(op, r[l], r[l]);
                dot = fd_dot(op, r[l], r[0]);
                gam_p[l] = cdiv(dot, sig[l]);
            }
            gam[L] = gam_p[L];
            omega = gam[L];
            for (int l = L - 1; l >= 1; --l) {
                gam[l] = gam_p[l];
                for (int i = l + 1; i <= L; ++i) gam[l] = csub(gam[l], cmul(tau[l][i], gam[i]));
            }
            for (int l = 1; l <= L - 1; ++l) {
                gam_pp[l] = gam[l + 1];
                for (int i = l + 1; i <= L - 1; ++i) gam_pp[l] = cadd(gam_pp[l], cmul(tau[l][i], gam[i + 1]));
            }
            fd_lin(op, f_out, r[0], gam[1], 0);
            fd_lin(op, r[0], r[L], cscale(gam_p[L], -1.0), 0);
            fd_lin(op, u[0], u[L], cscale(gam[L], -1.0), 0);
            for (int l = 1; l <= L - 1; ++l) {
                fd_lin(op, u[0], u[l], cscale(gam[l], -1.0), 0);
                fd_lin(op, f_out, r[l], gam_pp[l], 0);
                fd_lin(op, r[0], r[l], cscale(gam_p[l], -1.0), 0);
            }
            dot = fd_dot(op, r[0], r[0]);
            err_r = std::sqrt(dot.re);
            n = n + 1;
            if (err_r <= tol * norm_t) conv = 1;
        }
        fck(cudaMemcpyAsync(f_io, f_out, bytes, cudaMemcpyDeviceToHost, op->s), "download");
        fck(cudaStreamSynchronize(op->s), "solve");
        if (converged) *converged = conv;
        if (abs_err) *abs_err = err_r / norm_t;
        if (iterations) *iterations = n;
    } catch (const FdErr &e) {
        return fd_fail(e.code, e.msg);
    }
    return OMX_OK;
}

}  // extern "C"
