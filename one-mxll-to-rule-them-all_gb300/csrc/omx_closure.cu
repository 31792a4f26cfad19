// omx_closure.cu -- learned emitter closure: BF16 tensor-core GEMM (tcgen05, TMA, TMEM) and
// the launch helpers built on it.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/omx_gpu.h"
#include "omx_gemm_tc.cuh"
#include "omx_internal.h"

namespace omx {
void set_global_error(const std::string &msg);

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime (no link to libcuda)
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// 2D BF16 tensor [rows x cols] (row stride ld elements) read in boxes of 64 columns x box_rows rows
// with the 128-byte swizzle; reads outside the tensor return zero.
static bool tmap_bf16(CUtensorMap *m, const void *base, unsigned long long rows, unsigned long long cols,
                      unsigned long long ld, unsigned box_rows)
{
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {ld * 2};
    const cuuint32_t box[2] = {64, box_rows};
    const cuuint32_t es[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

constexpr int GEMM_MAX_DEV = 64;

// Ring depth: 4 slots for long K, 2 for short K (the closure's K = 128..256).  Grid: per K split,
// enough persistent CTAs for two per SM over the tiles; with many row tiles each CTA takes whole
// rows of tiles (measured on the 1e6-row gate GEMM: 0.84 against 0.93 ms), else the flat order
// (small training GEMMs keep every SM busy).  A CTA holds two
// accumulators of TMEM_COLS columns; its shared memory is padded so that no more CTAs share an SM
// than its 512 TMEM columns hold (an allocation beyond them would wait for a CTA to finish).
template <int BN, int STAGES>
static cudaError_t gemm_launch_s(const CUtensorMap &ta, const CUtensorMap &tb, int K, const GemmEpi &E, cudaStream_t s)
{
    using S = GemmSmem<BN, STAGES>;
    static int attr[GEMM_MAX_DEV] = {};
    static int sms[GEMM_MAX_DEV] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    const int di = dev < GEMM_MAX_DEV ? dev : 0;
    const int per_sm = 512 / (2 * (int)S::TMEM_COLS);
    const int bytes = std::max(S::BYTES, 233472 / (per_sm + 1) + 1024);
    if (!attr[di]) {
        cudaError_t e = cudaFuncSetAttribute(k_gemm_tc<BN, STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms[di], cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        attr[di] = 1;
    }
    const int nk = (K + 63) / 64;
    const int splits = E.kpz > 0 ? (nk + E.kpz - 1) / E.kpz : 1;
    const int mt = (E.M + 127) / 128, tiles = mt * ((E.N + BN - 1) / BN);
    const int cap = std::max(1, 2 * sms[di] / std::max(1, splits));
    GemmEpi Ep = E;
    Ep.row_major_tiles = mt >= 2 * cap ? 1 : 0;
    const int px = Ep.row_major_tiles ? cap : std::min(tiles, cap);
    const dim3 grid((unsigned)px, 1, (unsigned)splits);
    k_gemm_tc<BN, STAGES><<<grid, GEMM_THREADS, bytes, s>>>(ta, tb, K, Ep);
    return cudaGetLastError();
}
template <int BN>
static cudaError_t gemm_launch(const CUtensorMap &ta, const CUtensorMap &tb, int K, const GemmEpi &E, cudaStream_t s)
{
    const int nk = (E.kpz > 0 ? E.kpz : (K + 63) / 64);
    return nk <= 4 ? gemm_launch_s<BN, 2>(ta, tb, K, E, s) : gemm_launch_s<BN, 4>(ta, tb, K, E, s);
}

// D = act(alpha * A * B^T + bias) on device buffers; A [M x K] (lda), B [N x K] (ldb) in BF16.
// lda, ldb multiples of 8 (16-byte rows), buffers 16-byte aligned.
bool gemm_bf16(const uint16_t *A, int lda, const uint16_t *B, int ldb, int K, const GemmEpi &E, cudaStream_t s,
               std::string &err)
{
    if (E.M <= 0 || E.N <= 0 || K <= 0) return true;
    if (E.kpz > 0 && ((K + 63) / 64 + E.kpz - 1) / E.kpz > 1 && (E.d_bf16 || E.act || E.dtanh || E.bias)) {
        err = "gemm: split-K writes plain partial sums only";
        return false;
    }
    if (lda % 8 || ldb % 8 || (reinterpret_cast<uintptr_t>(A) & 15) || (reinterpret_cast<uintptr_t>(B) & 15)) {
        err = "gemm: rows must be 16-byte aligned";
        return false;
    }
    const int BN = E.N <= 16 ? 16 : (E.N <= 64 ? 64 : 128);
    CUtensorMap ta, tb;
    if (!tmap_bf16(&ta, A, (unsigned long long)E.M, (unsigned long long)K, (unsigned long long)lda, 128) ||
        !tmap_bf16(&tb, B, (unsigned long long)E.N, (unsigned long long)K, (unsigned long long)ldb, (unsigned)BN)) {
        err = "gemm: tensor map encoding failed";
        return false;
    }
    cudaError_t e;
    if (BN == 16) e = gemm_launch<16>(ta, tb, K, E, s);
    else if (BN == 64) e = gemm_launch<64>(ta, tb, K, E, s);
    else e = gemm_launch<128>(ta, tb, K, E, s);
    if (e != cudaSuccess) {
        err = std::string("gemm launch: ") + cudaGetErrorString(e);
        return false;
    }
    return true;
}

}  // namespace omx

// ---- C-ABI: the GEMM on host arrays, for validation --------------------------------------------
extern "C" int omx_tc_gemm_bf16(const uint16_t *A, const uint16_t *B, const float *bias, float *D, int M, int N, int K,
                                float alpha, int act)
{
    using namespace omx;
    auto fail = [](int code, const std::string &m) {
        set_global_error("omx_tc_gemm_bf16: " + m);
        return code;
    };
    if (!A || !B || !D || M <= 0 || N <= 0 || K <= 0 || K % 8 || act < 0 || act > 3)
        return fail(OMX_ERR_ARG, "bad argument (K must be a multiple of 8)");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(OMX_ERR_NODEV, "no CUDA device");
    }
    uint16_t *dA = nullptr, *dB = nullptr;
    float *dD = nullptr, *dbias = nullptr;
    int *derr = nullptr;
    int herr = 0;
    std::string err;
    bool ok = cudaMalloc(&dA, sizeof(uint16_t) * M * (size_t)K) == cudaSuccess &&
              cudaMalloc(&dB, sizeof(uint16_t) * N * (size_t)K) == cudaSuccess &&
              cudaMalloc(&dD, sizeof(float) * M * (size_t)N) == cudaSuccess &&
              cudaMalloc(&derr, sizeof(int)) == cudaSuccess && (!bias || cudaMalloc(&dbias, sizeof(float) * N) == cudaSuccess);
    if (ok) {
        cudaMemcpy(dA, A, sizeof(uint16_t) * M * (size_t)K, cudaMemcpyHostToDevice);
        cudaMemcpy(dB, B, sizeof(uint16_t) * N * (size_t)K, cudaMemcpyHostToDevice);
        if (bias) cudaMemcpy(dbias, bias, sizeof(float) * N, cudaMemcpyHostToDevice);
        cudaMemset(derr, 0, sizeof(int));
        cudaStreamSynchronize(0);   // the legacy stream does not order non-blocking streams, and pageable
                                    // copies may return before their DMA ends
        GemmEpi E{};
        E.d_f32 = dD;
        E.ld_f32 = N;
        E.bias = dbias;
        E.act = act;
        E.alpha = alpha;
        E.M = M;
        E.N = N;
        E.err = derr;
        ok = gemm_bf16(dA, K, dB, K, K, E, 0, err);
        if (ok) {
            const cudaError_t e = cudaDeviceSynchronize();
            if (e != cudaSuccess) {
                ok = false;
                err = std::string("gemm: ") + cudaGetErrorString(e);
            }
        }
        if (ok) {
            cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost);
            if (herr) {
                ok = false;
                err = "gemm: a pipeline wait ran out";
            } else {
                cudaMemcpy(D, dD, sizeof(float) * M * (size_t)N, cudaMemcpyDeviceToHost);
            }
        }
    } else {
        err = "device allocation failed";
    }
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dD);
    cudaFree(dbias);
    cudaFree(derr);
    return ok ? OMX_OK : fail(OMX_ERR_CUDA, err);
}

// =====================================================================================================
// The closure network: per emitter and quantum step, a GRU (hidden 128) over windows of the last 32
// field samples on the emitter's dipole axis, then a tanh MLP (3 x 256) and a linear read-out of
// the (scaled) dipole on that axis.  GEMMs run on the tensor cores in BF16 with FP32 accumulation;
// elementwise work and the state are FP32; the FP32 master weights are updated by Adam.
// Parameter layout (flat FP32): Wg [512 x 160], bg [512], W1 [256 x 128], b1, W2 [256 x 256], b2,
// W3 [256 x 256], b3, w4 [256], b4 [1].  Wg's rows: r | z | nx | nh gates (128 each); the nx rows
// see only the 32 window columns, the nh rows only the 128 hidden columns (mask).
// =====================================================================================================
namespace omx {

constexpr int CL_W = 32, CL_H = 128, CL_F = 256, CL_XH = CL_W + CL_H, CL_G = 4 * CL_H, CL_OUT = 16;
constexpr long long CL_OFF_WG = 0, CL_OFF_BG = CL_OFF_WG + (long long)CL_G * CL_XH, CL_OFF_W1 = CL_OFF_BG + CL_G,
                    CL_OFF_B1 = CL_OFF_W1 + (long long)CL_F * CL_H, CL_OFF_W2 = CL_OFF_B1 + CL_F,
                    CL_OFF_B2 = CL_OFF_W2 + (long long)CL_F * CL_F, CL_OFF_W3 = CL_OFF_B2 + CL_F,
                    CL_OFF_B3 = CL_OFF_W3 + (long long)CL_F * CL_F, CL_OFF_W4 = CL_OFF_B3 + CL_F,
                    CL_OFF_B4 = CL_OFF_W4 + CL_F, CL_NPARAM = CL_OFF_B4 + 1;

__device__ __forceinline__ bool cl_wg_masked(int row, int col)
{
    return (row >= 2 * CL_H && row < 3 * CL_H && col >= CL_W) || (row >= 3 * CL_H && col < CL_W);
}
__device__ __forceinline__ float cl_sigmoid(float x) { return 1.0f / (1.0f + expf(-x)); }

// FP32 master -> BF16 weights (row-major and transposed), masked Wg, padded read-out row
// row of the gate weights in the deployment order: tile b of 128 rows holds hidden units
// 32b .. 32b+31, four consecutive rows per unit in gate order r, z, nx, nh (the fused GRU epilogue)
__device__ __forceinline__ int cl_gate_perm(int r)
{
    const int gate = r / CL_H, j = r % CL_H;
    return 128 * (j / 32) + 4 * (j % 32) + gate;
}

__global__ void k_cl_refresh(const float *__restrict__ p, uint16_t *wg, uint16_t *wgT, uint16_t *w1, uint16_t *w1T,
                             uint16_t *w2, uint16_t *w2T, uint16_t *w3, uint16_t *w3T, uint16_t *w4, uint16_t *w4T,
                             float *b4pad, uint16_t *wgp, float *bgp)
{
    const long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (n < (long long)CL_G * CL_XH) {
        const int r = (int)(n / CL_XH), c = (int)(n % CL_XH);
        const uint16_t v = cl_wg_masked(r, c) ? (uint16_t)0 : f32_to_bf16_rn(p[CL_OFF_WG + n]);
        wg[n] = v;
        wgT[(long long)c * CL_G + r] = v;
        wgp[(long long)cl_gate_perm(r) * CL_XH + c] = v;
    }
    if (n < CL_G) bgp[cl_gate_perm((int)n)] = p[CL_OFF_BG + n];
    if (n < (long long)CL_F * CL_H) {
        const int r = (int)(n / CL_H), c = (int)(n % CL_H);
        const uint16_t v = f32_to_bf16_rn(p[CL_OFF_W1 + n]);
        w1[n] = v;
        w1T[(long long)c * CL_F + r] = v;
    }
    if (n < (long long)CL_F * CL_F) {
        const int r = (int)(n / CL_F), c = (int)(n % CL_F);
        const uint16_t v2 = f32_to_bf16_rn(p[CL_OFF_W2 + n]), v3 = f32_to_bf16_rn(p[CL_OFF_W3 + n]);
        w2[n] = v2;
        w2T[(long long)c * CL_F + r] = v2;
        w3[n] = v3;
        w3T[(long long)c * CL_F + r] = v3;
    }
    if (n < (long long)CL_OUT * CL_F) {
        const int r = (int)(n / CL_F), c = (int)(n % CL_F);
        const uint16_t v = r == 0 ? f32_to_bf16_rn(p[CL_OFF_W4 + c]) : (uint16_t)0;
        w4[n] = v;
        w4T[(long long)c * CL_OUT + r] = v;
    }
    if (n < CL_OUT) b4pad[n] = n == 0 ? p[CL_OFF_B4] : 0.f;
}

// XH row of step t: window e[b, t .. t+W-1] (row stride lde) and the previous hidden state
__global__ void k_cl_build_xh(const float *__restrict__ e, long long lde, int t, const float *__restrict__ hprev,
                              uint16_t *__restrict__ xh, int B)
{
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= (long long)B * CL_XH) return;
    const int b = (int)(q / CL_XH), c = (int)(q % CL_XH);
    const float v = c < CL_W ? e[b * lde + t + c] : (hprev ? hprev[(long long)b * CL_H + (c - CL_W)] : 0.f);
    xh[q] = f32_to_bf16_rn(v);
}

// GRU cell: gates G [B x 512] (pre-activations, biases included) -> h_t (FP32 and BF16); the
// activations r, z, n and the nh pre-activation are kept for the backward pass when cache != null
__global__ void k_cl_gru_fwd(const float *__restrict__ G, const float *hprev, float *h, uint16_t *__restrict__ hb,
                             float *__restrict__ cache, int B, const int *skip)
{
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= (long long)B * CL_H || (skip && *skip)) return;
    const int b = (int)(q / CL_H), j = (int)(q % CL_H);
    const float *g = G + (long long)b * CL_G;
    const float r = cl_sigmoid(g[j]), z = cl_sigmoid(g[CL_H + j]);
    const float nh = g[3 * CL_H + j];
    const float n = tanhf(g[2 * CL_H + j] + r * nh);
    const float hp = hprev ? hprev[q] : 0.f;
    const float hn = (1.0f - z) * n + z * hp;
    h[q] = hn;
    hb[q] = f32_to_bf16_rn(hn);
    if (cache) {
        float *c = cache + (long long)b * 4 * CL_H;
        c[j] = r;
        c[CL_H + j] = z;
        c[2 * CL_H + j] = n;
        c[3 * CL_H + j] = nh;
    }
}

// loss and its gradient: y = Y[:, 0] (rows t*B + b), target [T][B]; steps t < skip do not count
__global__ void k_cl_loss(const float *__restrict__ Y, const float *__restrict__ target, int B, int T, int skip,
                          uint16_t *__restrict__ dY, double *loss)
{
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long rows = (long long)B * T;
    double part = 0.0;
    if (q < rows) {
        const int t = (int)(q / B);
        const float d = Y[q * CL_OUT] - target[q];
        const double cnt = (double)(T - skip) * B;
        const float g = t >= skip ? (float)(2.0 * d / cnt) : 0.f;
        if (t >= skip) part = (double)d * d / cnt;
#pragma unroll
        for (int c = 0; c < CL_OUT; ++c) dY[q * CL_OUT + c] = c == 0 ? f32_to_bf16_rn(g) : (uint16_t)0;
    }
    for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0 && part != 0.0) atomicAdd(loss, part);
}

// GRU backward of step t: dh = dHm_t + dh_next -> dG_t (BF16, gate pre-activation gradients)
// and the direct part of dh_prev (dh * z)
__global__ void k_cl_gru_bwd(const float *__restrict__ dHm, const float *__restrict__ dh_next,
                             const float *__restrict__ cache, const float *__restrict__ hprev,
                             uint16_t *__restrict__ dG, float *__restrict__ dh_direct, int B)
{
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= (long long)B * CL_H) return;
    const int b = (int)(q / CL_H), j = (int)(q % CL_H);
    const float *c = cache + (long long)b * 4 * CL_H;
    const float r = c[j], z = c[CL_H + j], n = c[2 * CL_H + j], nh = c[3 * CL_H + j];
    const float hp = hprev ? hprev[q] : 0.f;
    const float dh = dHm[q] + (dh_next ? dh_next[q] : 0.f);
    const float dn = dh * (1.0f - z);
    const float dz = dh * (hp - n) * z * (1.0f - z);
    const float dpn = dn * (1.0f - n * n);
    const float dr = dpn * nh * r * (1.0f - r);
    uint16_t *g = dG + (long long)b * CL_G;
    g[j] = f32_to_bf16_rn(dr);
    g[CL_H + j] = f32_to_bf16_rn(dz);
    g[2 * CL_H + j] = f32_to_bf16_rn(dpn);
    g[3 * CL_H + j] = f32_to_bf16_rn(dpn * r);
    dh_direct[q] = dh * z;
}

// dh_prev = dXH[:, W:] + dh_direct
__global__ void k_cl_dh_prev(const float *__restrict__ dXH, const float *__restrict__ dh_direct, float *__restrict__ out,
                             int B)
{
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= (long long)B * CL_H) return;
    const int b = (int)(q / CL_H), j = (int)(q % CL_H);
    out[q] = dXH[(long long)b * CL_XH + CL_W + j] + dh_direct[q];
}

// BF16 transpose [R x C] -> [C x R] (32 x 32 tiles through shared memory)
__global__ void k_cl_transpose(const uint16_t *__restrict__ src, int R, int C, int lds, uint16_t *__restrict__ dst,
                               int ldd)
{
    __shared__ uint16_t tile[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int r = r0 + k, c = c0 + threadIdx.x;
        tile[k][threadIdx.x] = (r < R && c < C) ? src[(long long)r * lds + c] : (uint16_t)0;
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int c = c0 + k, r = r0 + threadIdx.x;
        if (c < C && r < R) dst[(long long)c * ldd + r] = tile[threadIdx.x][k];
    }
}

// out[i] = sum over the row i of a BF16 [rows x n] matrix (one warp per row, fixed order)
__global__ void k_cl_rowsum(const uint16_t *__restrict__ src, int rows, long long n, long long ld, float *__restrict__ out)
{
    const int row = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
    if (row >= rows) return;
    float s = 0.f;
    for (long long k = lane; k < n; k += 32) s += __bfloat162float(__ushort_as_bfloat16(src[row * ld + k]));
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) out[row] = s;
}

// out = sum of `splits` partial [n] arrays (fixed order), optionally masked like Wg
__global__ void k_cl_reduce(const float *__restrict__ part, int splits, long long n, float *__restrict__ out, int wg_mask,
                            int row_len)
{
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= n) return;
    float s = 0.f;
    for (int z = 0; z < splits; ++z) s += part[z * n + q];
    if (wg_mask && cl_wg_masked((int)(q / row_len), (int)(q % row_len))) s = 0.f;
    out[q] = s;
}

__global__ void k_cl_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                          long long n, float lr, float c1, float c2)
{
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= n) return;
    const float gq = g[q];
    const float mq = 0.9f * m[q] + 0.1f * gq, vq = 0.999f * v[q] + 0.001f * gq * gq;
    m[q] = mq;
    v[q] = vq;
    p[q] -= lr * (mq / c1) / (sqrtf(vq / c2) + 1e-8f);
}

// y[b] = Y[b, 0] (strided read-out of the padded output)
__global__ void k_cl_take_y(const float *__restrict__ Y, long long rows, float *__restrict__ y)
{
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q < rows) y[q] = Y[q * CL_OUT];
}

static inline unsigned cl_blocks(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

template <class T> struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    ~DBuf() { cudaFree(p); }
    bool ensure(size_t count)
    {
        if (count <= n) return true;
        cudaFree(p);
        p = nullptr;
        n = 0;
        if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) return false;
        n = count;
        return true;
    }
};

}  // namespace omx

struct omx_closure {
    cudaStream_t stream = nullptr;
    long long adam_step = 0;
    double e_scale = 1.0, d_scale = 1.0;   // field and dipole scales of the training data
    omx::DBuf<float> p, g, m, v, b4pad, bgp;
    omx::DBuf<uint16_t> wg, wgT, w1, w1T, w2, w2T, w3, w3T, w4, w4T, wgp;   // wgp, bgp: deployment gate order
    // training / batch work buffers (grown on demand)
    omx::DBuf<float> e, tgt, G, H, cache, A1, A2, A3, Y, dHm, dXH, dh, dhd, part;
    omx::DBuf<uint16_t> XH, Hb, A1b, A2b, A3b, dY, dZ1, dZ2, dZ3, dG, T1, T2;
    omx::DBuf<double> loss;
    omx::DBuf<int> err;
};

namespace omx {

#define CL_CK(x)                                                                    \
    do {                                                                            \
        cudaError_t e_ = (x);                                                       \
        if (e_ != cudaSuccess) {                                                    \
            err = std::string(#x) + ": " + cudaGetErrorString(e_);                  \
            return false;                                                           \
        }                                                                           \
    } while (0)
#define CL_NEED(buf, cnt)                                                           \
    do {                                                                            \
        if (!(buf).ensure(cnt)) {                                                   \
            err = "closure: device allocation failed";                              \
            return false;                                                           \
        }                                                                           \
    } while (0)

static bool cl_refresh(omx_closure *c, std::string &err)
{
    k_cl_refresh<<<cl_blocks((long long)CL_F * CL_F > (long long)CL_G * CL_XH ? (long long)CL_F * CL_F
                                                                            : (long long)CL_G * CL_XH),
                   256, 0, c->stream>>>(c->p.p, c->wg.p, c->wgT.p, c->w1.p, c->w1T.p, c->w2.p, c->w2T.p, c->w3.p,
                                        c->w3T.p, c->w4.p, c->w4T.p, c->b4pad.p, c->wgp.p, c->bgp.p);
    CL_CK(cudaGetLastError());
    return true;
}

static GemmEpi cl_epi(omx_closure *c, int M, int N)
{
    GemmEpi E{};
    E.alpha = 1.0f;
    E.M = M;
    E.N = N;
    E.err = c->err.p;
    return E;
}

// Forward over T steps for B sequences: e [B][T + W - 1] scaled field samples.  Leaves the
// per-step activations in the work buffers (rows t*B + b) and Y [T*B][16].
static bool cl_forward(omx_closure *c, int B, int T, bool keep, std::string &err)
{
    const long long TB = (long long)T * B;
    CL_NEED(c->XH, (size_t)TB * CL_XH);
    CL_NEED(c->G, (size_t)B * CL_G);
    CL_NEED(c->H, (size_t)TB * CL_H);
    CL_NEED(c->Hb, (size_t)TB * CL_H);
    CL_NEED(c->cache, (size_t)(keep ? TB : B) * 4 * CL_H);
    CL_NEED(c->A1, (size_t)TB * CL_F);
    CL_NEED(c->A2, (size_t)TB * CL_F);
    CL_NEED(c->A3, (size_t)TB * CL_F);
    CL_NEED(c->A1b, (size_t)TB * CL_F);
    CL_NEED(c->A2b, (size_t)TB * CL_F);
    CL_NEED(c->A3b, (size_t)TB * CL_F);
    CL_NEED(c->Y, (size_t)TB * CL_OUT);
    const long long lde = T + CL_W - 1;
    for (int t = 0; t < T; ++t) {
        const float *hprev = t > 0 ? c->H.p + (long long)(t - 1) * B * CL_H : nullptr;
        uint16_t *xh = c->XH.p + (long long)t * B * CL_XH;
        k_cl_build_xh<<<cl_blocks((long long)B * CL_XH), 256, 0, c->stream>>>(c->e.p, lde, t, hprev, xh, B);
        GemmEpi E = cl_epi(c, B, CL_G);
        E.d_f32 = c->G.p;
        E.ld_f32 = CL_G;
        E.bias = c->p.p + CL_OFF_BG;
        if (!gemm_bf16(xh, CL_XH, c->wg.p, CL_XH, CL_XH, E, c->stream, err)) return false;
        k_cl_gru_fwd<<<cl_blocks((long long)B * CL_H), 256, 0, c->stream>>>(
            c->G.p, hprev, c->H.p + (long long)t * B * CL_H, c->Hb.p + (long long)t * B * CL_H,
            c->cache.p + (keep ? (long long)t * B * 4 * CL_H : 0), B, nullptr);
    }
    // MLP on all T*B rows at once
    struct Layer {
        const uint16_t *in;
        int k;
        const uint16_t *w;
        long long boff;
        float *out;
        uint16_t *outb;
    } L[3] = {{c->Hb.p, CL_H, c->w1.p, CL_OFF_B1, c->A1.p, c->A1b.p},
              {c->A1b.p, CL_F, c->w2.p, CL_OFF_B2, c->A2.p, c->A2b.p},
              {c->A2b.p, CL_F, c->w3.p, CL_OFF_B3, c->A3.p, c->A3b.p}};
    for (auto &l : L) {
        GemmEpi E = cl_epi(c, (int)TB, CL_F);
        E.d_f32 = l.out;
        E.ld_f32 = CL_F;
        E.d_bf16 = l.outb;
        E.ld_bf16 = CL_F;
        E.bias = c->p.p + l.boff;
        E.act = 1;
        if (!gemm_bf16(l.in, l.k, l.w, l.k, l.k, E, c->stream, err)) return false;
    }
    GemmEpi E = cl_epi(c, (int)TB, CL_OUT);
    E.d_f32 = c->Y.p;
    E.ld_f32 = CL_OUT;
    E.bias = c->b4pad.p;
    if (!gemm_bf16(c->A3b.p, CL_F, c->w4.p, CL_F, CL_F, E, c->stream, err)) return false;
    CL_CK(cudaGetLastError());
    return true;
}

// dW [N x K] = sum over rows of dZ[:, n] * X[:, k]: one long-K GEMM over the T*B rows (both
// operands transposed first), split over K and reduced in a fixed order
static bool cl_weight_grad(omx_closure *c, const uint16_t *dZ, int N, const uint16_t *X, int K, long long TB, float *out,
                           int wg_mask, std::string &err)
{
    const int ldT = (int)((TB + 7) / 8 * 8);
    CL_NEED(c->T1, (size_t)N * ldT);
    CL_NEED(c->T2, (size_t)K * ldT);
    const dim3 tb(32, 8);
    k_cl_transpose<<<dim3((N + 31) / 32, (unsigned)((TB + 31) / 32)), tb, 0, c->stream>>>(dZ, (int)TB, N, N, c->T1.p, ldT);
    k_cl_transpose<<<dim3((K + 31) / 32, (unsigned)((TB + 31) / 32)), tb, 0, c->stream>>>(X, (int)TB, K, K, c->T2.p, ldT);
    const int nk = (int)((TB + 63) / 64);
    const int kpz = nk < 32 ? nk : (nk + 31) / 32;      // about 32 splits
    const int splits = (nk + kpz - 1) / kpz;
    CL_NEED(c->part, (size_t)splits * N * K);
    GemmEpi E = cl_epi(c, N, K);
    E.d_f32 = c->part.p;
    E.ld_f32 = K;
    E.kpz = kpz;
    E.split_stride = (long long)N * K;
    if (!gemm_bf16(c->T1.p, ldT, c->T2.p, ldT, (int)TB, E, c->stream, err)) return false;
    k_cl_reduce<<<cl_blocks((long long)N * K), 256, 0, c->stream>>>(c->part.p, splits, (long long)N * K, out, wg_mask,
                                                                   K);
    CL_CK(cudaGetLastError());
    return true;
}

// bias gradient: sums of the first N columns of a BF16 [TB x ld] matrix (through its
// transpose, one warp per column, fixed order)
static bool cl_bias_grad(omx_closure *c, const uint16_t *dZ, int N, int ld, long long TB, float *out, std::string &err)
{
    const int ldT = (int)((TB + 7) / 8 * 8);
    CL_NEED(c->T1, (size_t)N * ldT);
    k_cl_transpose<<<dim3((N + 31) / 32, (unsigned)((TB + 31) / 32)), dim3(32, 8), 0, c->stream>>>(dZ, (int)TB, N, ld,
                                                                                                 c->T1.p, ldT);
    k_cl_rowsum<<<(N + 7) / 8, 256, 0, c->stream>>>(c->T1.p, N, TB, ldT, out);
    CL_CK(cudaGetLastError());
    return true;
}

// loss and full gradient (into c->g) for e [B][T+W-1], target [T][B]; forward included
static bool cl_gradient(omx_closure *c, int B, int T, int skip, std::string &err)
{
    if (!cl_forward(c, B, T, true, err)) return false;
    const long long TB = (long long)T * B;
    CL_NEED(c->dY, (size_t)TB * CL_OUT);
    CL_NEED(c->dZ1, (size_t)TB * CL_F);
    CL_NEED(c->dZ2, (size_t)TB * CL_F);
    CL_NEED(c->dZ3, (size_t)TB * CL_F);
    CL_NEED(c->dHm, (size_t)TB * CL_H);
    CL_NEED(c->dG, (size_t)TB * CL_G);
    CL_NEED(c->dXH, (size_t)B * CL_XH);
    CL_NEED(c->dh, (size_t)B * CL_H);
    CL_NEED(c->dhd, (size_t)B * CL_H);
    CL_CK(cudaMemsetAsync(c->loss.p, 0, sizeof(double), c->stream));
    k_cl_loss<<<cl_blocks(TB), 256, 0, c->stream>>>(c->Y.p, c->tgt.p, B, T, skip, c->dY.p, c->loss.p);
    // MLP backward on all rows: dZ3 = (dY W4) (1 - a3^2), dZ2, dZ1, dHm = dZ1 W1
    struct Back {
        const uint16_t *in;
        int k;
        const uint16_t *wT;
        int n;
        const float *a;
        uint16_t *outb;
        float *outf;
    } Bk[4] = {{c->dY.p, CL_OUT, c->w4T.p, CL_F, c->A3.p, c->dZ3.p, nullptr},
               {c->dZ3.p, CL_F, c->w3T.p, CL_F, c->A2.p, c->dZ2.p, nullptr},
               {c->dZ2.p, CL_F, c->w2T.p, CL_F, c->A1.p, c->dZ1.p, nullptr},
               {c->dZ1.p, CL_F, c->w1T.p, CL_H, nullptr, nullptr, c->dHm.p}};
    for (auto &b : Bk) {
        GemmEpi E = cl_epi(c, (int)TB, b.n);
        E.d_bf16 = b.outb;
        E.ld_bf16 = b.n;
        E.d_f32 = b.outf;
        E.ld_f32 = b.n;
        E.dtanh = b.a;
        E.ld_dtanh = b.n;
        if (!gemm_bf16(b.in, b.k, b.wT, b.k, b.k, E, c->stream, err)) return false;
    }
    // weight and bias gradients of the MLP
    CL_NEED(c->part, (size_t)CL_OUT * CL_F);
    float *g = c->g.p;
    if (!cl_weight_grad(c, c->dZ3.p, CL_F, c->A2b.p, CL_F, TB, g + CL_OFF_W3, 0, err)) return false;
    if (!cl_weight_grad(c, c->dZ2.p, CL_F, c->A1b.p, CL_F, TB, g + CL_OFF_W2, 0, err)) return false;
    if (!cl_weight_grad(c, c->dZ1.p, CL_F, c->Hb.p, CL_H, TB, g + CL_OFF_W1, 0, err)) return false;
    if (!cl_bias_grad(c, c->dZ3.p, CL_F, CL_F, TB, g + CL_OFF_B3, err)) return false;
    if (!cl_bias_grad(c, c->dZ2.p, CL_F, CL_F, TB, g + CL_OFF_B2, err)) return false;
    if (!cl_bias_grad(c, c->dZ1.p, CL_F, CL_F, TB, g + CL_OFF_B1, err)) return false;
    // read-out row: dw4 = dY[:, 0]^T A3, db4 = sum dY[:, 0] (via a 16 x 256 product and row 0)
    CL_NEED(c->G, (size_t)B * CL_G > (size_t)CL_OUT * CL_F ? (size_t)B * CL_G : (size_t)CL_OUT * CL_F);
    if (!cl_weight_grad(c, c->dY.p, CL_OUT, c->A3b.p, CL_F, TB, c->G.p, 0, err)) return false;
    CL_CK(cudaMemcpyAsync(g + CL_OFF_W4, c->G.p, sizeof(float) * CL_F, cudaMemcpyDeviceToDevice, c->stream));
    if (!cl_bias_grad(c, c->dY.p, 1, CL_OUT, TB, g + CL_OFF_B4, err)) return false;
    // GRU, backward through time
    for (int t = T - 1; t >= 0; --t) {
        const float *hprev = t > 0 ? c->H.p + (long long)(t - 1) * B * CL_H : nullptr;
        k_cl_gru_bwd<<<cl_blocks((long long)B * CL_H), 256, 0, c->stream>>>(
            c->dHm.p + (long long)t * B * CL_H, t < T - 1 ? c->dh.p : nullptr, c->cache.p + (long long)t * B * 4 * CL_H,
            hprev, c->dG.p + (long long)t * B * CL_G, c->dhd.p, B);
        if (t > 0) {
            GemmEpi E = cl_epi(c, B, CL_XH);
            E.d_f32 = c->dXH.p;
            E.ld_f32 = CL_XH;
            if (!gemm_bf16(c->dG.p + (long long)t * B * CL_G, CL_G, c->wgT.p, CL_G, CL_G, E, c->stream, err))
                return false;
            k_cl_dh_prev<<<cl_blocks((long long)B * CL_H), 256, 0, c->stream>>>(c->dXH.p, c->dhd.p, c->dh.p, B);
        }
    }
    if (!cl_weight_grad(c, c->dG.p, CL_G, c->XH.p, CL_XH, TB, g + CL_OFF_WG, 1, err)) return false;
    if (!cl_bias_grad(c, c->dG.p, CL_G, CL_G, TB, g + CL_OFF_BG, err)) return false;
    CL_CK(cudaGetLastError());
    return true;
}

static bool cl_upload_batch(omx_closure *c, const float *e, const float *target, int B, int T, std::string &err)
{
    const size_t ne = (size_t)B * (T + CL_W - 1);
    CL_NEED(c->e, ne);
    CL_CK(cudaMemcpyAsync(c->e.p, e, ne * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    if (target) {
        CL_NEED(c->tgt, (size_t)B * T);
        CL_CK(cudaMemcpyAsync(c->tgt.p, target, (size_t)B * T * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    }
    return true;
}

static bool cl_finish(omx_closure *c, std::string &err)
{
    CL_CK(cudaStreamSynchronize(c->stream));
    int h = 0;
    CL_CK(cudaMemcpy(&h, c->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) {
        cudaMemsetAsync(c->err.p, 0, sizeof(int), c->stream);
        err = "closure: a tensor-core pipeline wait ran out";
        return false;
    }
    return true;
}

}  // namespace omx

namespace omx {

// network input of a deployed group: the window (oldest sample first; the newest was written at
// the ring head cl_step % W) and the GRU state
__global__ void k_cl_dep_xh(ClDeploy D)
{
    const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (q >= (long long)D.n * CL_XH || D.st->skip_nn) return;
    const int n = (int)(q / CL_XH), c = (int)(q % CL_XH);
    const int head = D.st->cl_step % CL_WIN;
    const float v = c < CL_W ? D.win[(long long)n * CL_WIN + (head + 1 + c) % CL_WIN] : D.hst[(long long)n * CL_H + c - CL_W];
    D.xh[q] = f32_to_bf16_rn(v);
}

// dipole = y * d_scale along the emitter axis, dP/dt against the previous dipole; then the ring
// advances (one thread, after every reader of this step's head)
__global__ void k_cl_dep_dipole(const float *__restrict__ Y, EmitArgs A, ClDeploy D)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (D.st->skip_nn) return;
    if (n < A.n) {
        const double *u = A.par + (long long)n * A.npar + (A.npar - 3);
        const double d = (double)Y[(long long)n * CL_OUT] * D.d_scale;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const double old = A.dipole[3 * n + a];
            const double nw = d * u[a];
            A.dipole[3 * n + a] = nw;
            A.dPdt[3 * n + a] = (nw - old) / A.dt;
        }
    }
}
__global__ void k_cl_dep_advance(ClDeploy D)
{
    if (!D.st->skip_nn) D.st->cl_step += 1;
}

// One network step of a deployed group (after k_cl_gather, before the spot-check kernels).
bool closure_infer(omx_closure *c, const ClDeploy &D, const EmitArgs &A, cudaStream_t s, std::string &err)
{
    // every buffer belongs to the deployment (allocated when it was attached): nothing is
    // allocated here, so the step can be captured in a graph
    const int n = D.n;
    const int *skip = &D.st->skip_nn;
    k_cl_dep_xh<<<cl_blocks((long long)n * CL_XH), 256, 0, s>>>(D);
    // gates and GRU cell in one launch: the epilogue turns the permuted gate columns into h
    GemmEpi E = cl_epi(c, n, CL_G);
    E.bias = c->bgp.p;
    E.gru_h = D.hst;
    E.gru_hb = D.hb;
    E.skip = skip;
    E.err = D.err;
    if (!gemm_bf16(D.xh, CL_XH, c->wgp.p, CL_XH, CL_XH, E, s, err)) return false;
    const uint16_t *in[3] = {D.hb, D.a1, D.a2};
    uint16_t *out[3] = {D.a1, D.a2, D.a3};
    const uint16_t *w[3] = {c->w1.p, c->w2.p, c->w3.p};
    const long long bo[3] = {CL_OFF_B1, CL_OFF_B2, CL_OFF_B3};
    const int k[3] = {CL_H, CL_F, CL_F};
    for (int l = 0; l < 3; ++l) {
        GemmEpi El = cl_epi(c, n, CL_F);
        El.d_bf16 = out[l];
        El.ld_bf16 = CL_F;
        El.bias = c->p.p + bo[l];
        El.act = 1;
        El.skip = skip;
        El.err = D.err;
        if (!gemm_bf16(in[l], k[l], w[l], k[l], k[l], El, s, err)) return false;
    }
    GemmEpi Eo = cl_epi(c, n, CL_OUT);
    Eo.d_f32 = D.Y;
    Eo.ld_f32 = CL_OUT;
    Eo.bias = c->b4pad.p;
    Eo.skip = skip;
    Eo.err = D.err;
    if (!gemm_bf16(D.a3, CL_F, c->w4.p, CL_F, CL_F, Eo, s, err)) return false;
    k_cl_dep_dipole<<<(n + 127) / 128, 128, 0, s>>>(D.Y, A, D);
    k_cl_dep_advance<<<1, 1, 0, s>>>(D);
    CL_CK(cudaGetLastError());
    return true;
}

double closure_e_scale(const omx_closure *c) { return c->e_scale; }
double closure_d_scale(const omx_closure *c) { return c->d_scale; }
int *closure_err_word(omx_closure *c) { return c->err.p; }

}  // namespace omx

// ---- C-ABI of the closure ----------------------------------------------------------------------
namespace {
int cl_fail(int code, const std::string &m)
{
    omx::set_global_error("closure: " + m);
    return code;
}
bool cl_shape_ok(int B, int T) { return B >= 8 && B % 8 == 0 && T >= 1; }
}  // namespace

extern "C" {

int omx_closure_create(omx_closure **out)
{
    using namespace omx;
    if (!out) return cl_fail(OMX_ERR_ARG, "null argument");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return cl_fail(OMX_ERR_NODEV, "no CUDA device");
    }
    omx_closure *c = new omx_closure;
    bool ok = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) == cudaSuccess && c->p.ensure(CL_NPARAM) &&
              c->g.ensure(CL_NPARAM) && c->m.ensure(CL_NPARAM) && c->v.ensure(CL_NPARAM) && c->b4pad.ensure(CL_OUT) &&
              c->wg.ensure((size_t)CL_G * CL_XH) && c->wgT.ensure((size_t)CL_G * CL_XH) &&
              c->w1.ensure((size_t)CL_F * CL_H) && c->w1T.ensure((size_t)CL_F * CL_H) &&
              c->w2.ensure((size_t)CL_F * CL_F) && c->w2T.ensure((size_t)CL_F * CL_F) &&
              c->w3.ensure((size_t)CL_F * CL_F) && c->w3T.ensure((size_t)CL_F * CL_F) &&
              c->w4.ensure((size_t)CL_OUT * CL_F) && c->w4T.ensure((size_t)CL_OUT * CL_F) &&
              c->wgp.ensure((size_t)CL_G * CL_XH) && c->bgp.ensure(CL_G) && c->loss.ensure(1) &&
              c->err.ensure(1);
    if (ok) ok = cudaMemset(c->p.p, 0, sizeof(float) * CL_NPARAM) == cudaSuccess &&
                 cudaMemset(c->m.p, 0, sizeof(float) * CL_NPARAM) == cudaSuccess &&
                 cudaMemset(c->v.p, 0, sizeof(float) * CL_NPARAM) == cudaSuccess &&
                 cudaMemset(c->err.p, 0, sizeof(int)) == cudaSuccess &&
                 cudaStreamSynchronize(0) == cudaSuccess;   // before the closure's own stream runs
    if (!ok) {
        if (c->stream) cudaStreamDestroy(c->stream);
        delete c;
        return cl_fail(OMX_ERR_NOMEM, "device allocation failed");
    }
    *out = c;
    return OMX_OK;
}

int omx_closure_destroy(omx_closure *c)
{
    if (!c) return OMX_OK;
    cudaStreamSynchronize(c->stream);
    cudaStream_t s = c->stream;
    delete c;
    cudaStreamDestroy(s);
    return OMX_OK;
}

long long omx_closure_n_params(void) { return omx::CL_NPARAM; }

int omx_closure_set_params(omx_closure *c, const float *params, double e_scale, double d_scale)
{
    using namespace omx;
    if (!c || !params || !(e_scale > 0) || !(d_scale > 0)) return cl_fail(OMX_ERR_ARG, "bad argument");
    std::string err;
    c->e_scale = e_scale;
    c->d_scale = d_scale;
    c->adam_step = 0;
    if (cudaMemcpyAsync(c->p.p, params, sizeof(float) * CL_NPARAM, cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
        cudaMemsetAsync(c->m.p, 0, sizeof(float) * CL_NPARAM, c->stream) != cudaSuccess ||
        cudaMemsetAsync(c->v.p, 0, sizeof(float) * CL_NPARAM, c->stream) != cudaSuccess || !cl_refresh(c, err) ||
        !cl_finish(c, err))
        return cl_fail(OMX_ERR_CUDA, err.empty() ? "upload failed" : err);
    return OMX_OK;
}

int omx_closure_get_params(omx_closure *c, float *params, double *e_scale, double *d_scale)
{
    using namespace omx;
    if (!c || !params) return cl_fail(OMX_ERR_ARG, "bad argument");
    std::string err;
    if (!cl_finish(c, err) ||
        cudaMemcpy(params, c->p.p, sizeof(float) * CL_NPARAM, cudaMemcpyDeviceToHost) != cudaSuccess)
        return cl_fail(OMX_ERR_CUDA, err.empty() ? "download failed" : err);
    if (e_scale) *e_scale = c->e_scale;
    if (d_scale) *d_scale = c->d_scale;
    return OMX_OK;
}

int omx_closure_forward(omx_closure *c, const float *e, int B, int T, float *y)
{
    using namespace omx;
    if (!c || !e || !y || !cl_shape_ok(B, T)) return cl_fail(OMX_ERR_ARG, "bad argument (B a multiple of 8)");
    std::string err;
    const long long TB = (long long)T * B;
    DBuf<float> yd;
    if (!yd.ensure((size_t)TB)) return cl_fail(OMX_ERR_NOMEM, "device allocation failed");
    if (!cl_upload_batch(c, e, nullptr, B, T, err) || !cl_forward(c, B, T, false, err))
        return cl_fail(OMX_ERR_CUDA, err);
    k_cl_take_y<<<cl_blocks(TB), 256, 0, c->stream>>>(c->Y.p, TB, yd.p);
    if (cudaMemcpyAsync(y, yd.p, sizeof(float) * TB, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        !cl_finish(c, err))
        return cl_fail(OMX_ERR_CUDA, err.empty() ? "forward failed" : err);
    return OMX_OK;
}

int omx_closure_gradient(omx_closure *c, const float *e, const float *target, int B, int T, int skip, float *grad,
                         double *loss)
{
    using namespace omx;
    if (!c || !e || !target || !cl_shape_ok(B, T) || skip < 0 || skip >= T)
        return cl_fail(OMX_ERR_ARG, "bad argument (B a multiple of 8, 0 <= skip < T)");
    std::string err;
    if (!cl_upload_batch(c, e, target, B, T, err) || !cl_gradient(c, B, T, skip, err)) return cl_fail(OMX_ERR_CUDA, err);
    double l = 0.0;
    if ((grad && cudaMemcpyAsync(grad, c->g.p, sizeof(float) * CL_NPARAM, cudaMemcpyDeviceToHost, c->stream) !=
                     cudaSuccess) ||
        cudaMemcpyAsync(&l, c->loss.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        !cl_finish(c, err))
        return cl_fail(OMX_ERR_CUDA, err.empty() ? "gradient failed" : err);
    if (loss) *loss = l;
    return OMX_OK;
}

int omx_closure_train_step(omx_closure *c, const float *e, const float *target, int B, int T, int skip, float lr,
                           double *loss)
{
    using namespace omx;
    if (!c || !e || !target || !cl_shape_ok(B, T) || skip < 0 || skip >= T || !(lr > 0))
        return cl_fail(OMX_ERR_ARG, "bad argument");
    std::string err;
    if (!cl_upload_batch(c, e, target, B, T, err) || !cl_gradient(c, B, T, skip, err)) return cl_fail(OMX_ERR_CUDA, err);
    c->adam_step += 1;
    const float c1 = (float)(1.0 - std::pow(0.9, (double)c->adam_step));
    const float c2 = (float)(1.0 - std::pow(0.999, (double)c->adam_step));
    k_cl_adam<<<cl_blocks(CL_NPARAM), 256, 0, c->stream>>>(c->p.p, c->g.p, c->m.p, c->v.p, CL_NPARAM, lr, c1, c2);
    double l = 0.0;
    if (!cl_refresh(c, err) ||
        cudaMemcpyAsync(&l, c->loss.p, sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        !cl_finish(c, err))
        return cl_fail(OMX_ERR_CUDA, err.empty() ? "train step failed" : err);
    if (loss) *loss = l;
    return OMX_OK;
}

int omx_closure_trajectories(int model, int n, int T, int K, double dt, const double *params, const double *drive,
                             double e_scale, double d_scale, float *e, float *d)
{
    using namespace omx;
    if ((model != OMX_EMITTER_TWO_LEVEL && model != OMX_EMITTER_THREE_LEVEL) || n <= 0 || T <= 0 || K <= 0 ||
        !(dt > 0) || !params || !drive || !e || !d || !(e_scale > 0) || !(d_scale > 0))
        return cl_fail(OMX_ERR_ARG, "bad argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return cl_fail(OMX_ERR_NODEV, "no CUDA device");
    }
    const int npar = model == OMX_EMITTER_TWO_LEVEL ? 7 : 9;
    DBuf<double> dp, dd;
    DBuf<float> de, ddip;
    if (!dp.ensure((size_t)n * npar) || !dd.ensure((size_t)n * (1 + 3 * K)) || !de.ensure((size_t)n * T) ||
        !ddip.ensure((size_t)n * T))
        return cl_fail(OMX_ERR_NOMEM, "device allocation failed");
    cudaMemcpy(dp.p, params, sizeof(double) * n * npar, cudaMemcpyHostToDevice);
    cudaMemcpy(dd.p, drive, sizeof(double) * n * (1 + 3 * K), cudaMemcpyHostToDevice);
    cudaStreamSynchronize(0);   // pageable copies may return before their DMA ends
    ClTrajArgs A{};
    A.n = n;
    A.T = T;
    A.K = K;
    A.model = model;
    A.npar = npar;
    A.dt = dt;
    A.e_scale = e_scale;
    A.d_scale = d_scale;
    A.params = dp.p;
    A.drive = dd.p;
    A.e = de.p;
    A.d = ddip.p;
    launch_cl_trajectories(A, 0);
    const cudaError_t err = cudaDeviceSynchronize();
    if (err != cudaSuccess) return cl_fail(OMX_ERR_CUDA, std::string("trajectories: ") + cudaGetErrorString(err));
    cudaMemcpy(e, de.p, sizeof(float) * n * (size_t)T, cudaMemcpyDeviceToHost);
    cudaMemcpy(d, ddip.p, sizeof(float) * n * (size_t)T, cudaMemcpyDeviceToHost);
    return OMX_OK;
}

}  // extern "C"
