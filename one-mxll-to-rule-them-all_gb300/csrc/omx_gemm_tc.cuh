// omx_gemm_tc.cuh -- BF16 GEMM on the 5th-generation tensor cores (tcgen05), FP32 accumulation
// in tensor memory, for the learned emitter closure.
//
//   D[M x N] = act(alpha * A[M x K] * B[N x K]^T + bias[N])      (A, B row-major, K contiguous)
//
// Optional epilogue factor (1 - a^2) from an FP32 array a of the same shape (the derivative of a
// tanh layer, for back-propagation).  Split-K: blockIdx.z takes K blocks [z*kpz, (z+1)*kpz) and
// writes its partial sums at d_f32 + z * split_stride (reduced afterwards in a fixed order).
//
// A persistent CTA computes a sequence of 128 x BN tiles (see k_gemm_tc): TMA loads of 128 x 64
// A and BN x 64 B tiles into a STAGES-deep ring (128-byte swizzle, out-of-range rows and columns
// read as zero), MMAs of K = 16 into one of two TMEM accumulators, the epilogue of one tile under
// the MMAs of the next.  Every wait is bounded; a wait that runs out sets bit 1 of *err.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include "omx_tc.cuh"

namespace omx {

constexpr long long TC_WAIT_CYCLES = 2000000000LL;

struct GemmEpi {
    float *d_f32;          // optional FP32 output (row stride ld_f32)
    uint16_t *d_bf16;      // optional BF16 output (row stride ld_bf16)
    const float *bias;     // optional, per output column
    const float *dtanh;    // optional: multiply by (1 - a^2), a = dtanh[row * ld_dtanh + col]
    int ld_f32, ld_bf16, ld_dtanh;
    int kpz;               // K blocks (of 64) per split (gridDim.z splits)
    const int *skip;       // optional: the whole launch does nothing while *skip != 0
    // GRU epilogue (gate rows permuted so that the 16 columns of a chunk hold r, z, nx, nh of
    // four hidden units: column 4u + gate of chunk c in column tile b is unit 32b + 4c + u):
    // h = (1 - z) tanh(nx + r nh) + z h, written in place to gru_h (row stride 128) and as BF16
    float *gru_h;
    uint16_t *gru_hb;
    long long split_stride;
    int act;               // 0 none, 1 tanh, 2 sigmoid, 3 relu
    float alpha;
    int M, N;
    int *err;
    int row_major_tiles;   // set by the launcher: each persistent CTA takes every column tile of its row tiles
};

__device__ __forceinline__ uint16_t f32_to_bf16_rn(float f)
{
    return __bfloat16_as_ushort(__float2bfloat16_rn(f));
}

__device__ __forceinline__ float epi_act(float v, int act)
{
    if (act == 1) return tanhf(v);
    if (act == 2) return 1.0f / (1.0f + expf(-v));
    if (act == 3) return v > 0.f ? v : 0.f;
    return v;
}

// Shared memory of the persistent GEMM: the STAGES-deep ring of A / B tiles, then the barriers.
template <int BN, int STAGES> struct GemmSmem {
    static constexpr int A_BYTES = 128 * 128;          // 128 rows x 64 BF16
    static constexpr int B_BYTES = BN * 128;           // BN rows x 64 BF16
    static constexpr int STAGE = A_BYTES + B_BYTES;
    static constexpr int BARS = STAGES * STAGE;        // offset of the barriers
    static constexpr int BYTES = BARS + (2 * STAGES + 4) * 8 + 16 + 1024;   // + alignment slack
    // one accumulator (power of two >= 32 columns); the kernel allocates two
    static constexpr uint32_t TMEM_COLS = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));
};

// Epilogue of one tile for the 32 accumulator rows of one warp and its columns cb0 .. cb1 - 1 (a
// multiple of 16 apart): tacc is the TMEM address of those rows at the accumulator's first
// column, row the output row of this thread, n0 the tile's first column, z the split.
__device__ __forceinline__ void gemm_epi_tile(const GemmEpi &E, uint32_t tacc, int row, int n0, int z, int cb0,
                                              int cb1)
{
    float *const dout = E.d_f32 ? E.d_f32 + (long long)z * E.split_stride : nullptr;
    if (E.gru_h) {
#pragma unroll 1
        for (int c0 = cb0; c0 < cb1; c0 += 16) {
            float v[16];
            __syncwarp();              // tcgen05.ld is warp-collective: reconverge first
            tmem_ld16(tacc + (uint32_t)c0, v);
            if (row < E.M) {
                const long long h0 = (long long)row * 128 + (n0 >> 2) + (c0 >> 2);   // 4 units, 16-byte aligned
                const float4 hp = *reinterpret_cast<const float4 *>(E.gru_h + h0);
                const float hpv[4] = {hp.x, hp.y, hp.z, hp.w};
                float hn[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int col = n0 + c0 + 4 * u;
                    const float gr = v[4 * u] + E.bias[col], gz = v[4 * u + 1] + E.bias[col + 1];
                    const float gx = v[4 * u + 2] + E.bias[col + 2], gh = v[4 * u + 3] + E.bias[col + 3];
                    const float r = 1.0f / (1.0f + expf(-gr)), zz = 1.0f / (1.0f + expf(-gz));
                    const float nn = tanhf(gx + r * gh);
                    hn[u] = (1.0f - zz) * nn + zz * hpv[u];
                }
                *reinterpret_cast<float4 *>(E.gru_h + h0) = make_float4(hn[0], hn[1], hn[2], hn[3]);
                const uint32_t lo = (uint32_t)f32_to_bf16_rn(hn[0]) | ((uint32_t)f32_to_bf16_rn(hn[1]) << 16);
                const uint32_t hi = (uint32_t)f32_to_bf16_rn(hn[2]) | ((uint32_t)f32_to_bf16_rn(hn[3]) << 16);
                *reinterpret_cast<uint2 *>(E.gru_hb + h0) = make_uint2(lo, hi);
            }
        }
        return;
    }
#pragma unroll 1
    for (int c0 = cb0; c0 < cb1; c0 += 16) {
        float v[16];
        __syncwarp();                  // tcgen05.ld is warp-collective: reconverge first
        tmem_ld16(tacc + (uint32_t)c0, v);
        const int cb = n0 + c0;
        // whole chunk inside the matrix with 16-byte aligned rows: vector stores
        const bool vec = row < E.M && cb + 16 <= E.N && !E.dtanh && (!dout || (E.ld_f32 % 4) == 0) &&
                         (!E.d_bf16 || (E.ld_bf16 % 8) == 0);
        if (vec) {
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                float x = E.alpha * v[q];
                if (E.bias) x += E.bias[cb + q];
                v[q] = epi_act(x, E.act);
            }
            if (dout) {
                float4 *o = reinterpret_cast<float4 *>(dout + (long long)row * E.ld_f32 + cb);
#pragma unroll
                for (int q = 0; q < 4; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            }
            if (E.d_bf16) {
                uint32_t w[8];
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    w[q] = (uint32_t)f32_to_bf16_rn(v[2 * q]) | ((uint32_t)f32_to_bf16_rn(v[2 * q + 1]) << 16);
                uint4 *o = reinterpret_cast<uint4 *>(E.d_bf16 + (long long)row * E.ld_bf16 + cb);
                o[0] = make_uint4(w[0], w[1], w[2], w[3]);
                o[1] = make_uint4(w[4], w[5], w[6], w[7]);
            }
            continue;
        }
        if (row < E.M) {
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const int col = n0 + c0 + q;
                if (col >= E.N) break;
                float x = E.alpha * v[q];
                if (E.bias) x += E.bias[col];
                x = epi_act(x, E.act);
                if (E.dtanh) {
                    const float a = E.dtanh[(long long)row * E.ld_dtanh + col];
                    x *= 1.0f - a * a;
                }
                if (dout) dout[(long long)row * E.ld_f32 + col] = x;
                if (E.d_bf16) E.d_bf16[(long long)row * E.ld_bf16 + col] = f32_to_bf16_rn(x);
            }
        }
    }
}

// Persistent form: CTA (x, 0, z) computes 128 x BN tiles of split z: with E.row_major_tiles, the
// row tiles m = x, x + gridDim.x, ... and every column tile of each in turn (the second and later
// read the A tile from L2); otherwise the tiles q = x, x + gridDim.x, ... of the flat order
// (m, n) = (q / ny, q % ny), for few row tiles (the CTAs that take the column tiles of one m run at
// the same time).  Ten warps: warp 0 (one lane) streams the A / B tiles of every tile's K blocks
// through the ring; warp 1 (one lane) issues the MMAs of tile t into accumulator t & 1 (two in
// TMEM) and commits it to tfull[t & 1]; warps 2..9 read accumulator t & 1 (warp w the TMEM lanes
// 32 (w % 4) .. 32 (w % 4) + 31, the rows it may access, and half of the columns) and apply the
// epilogue while the MMAs of tile t + 1 run, then release it on tempty[t & 1].  Every wait is
// bounded; a wait that runs out sets bit 1 of *err and every role leaves its loop.
constexpr int GEMM_THREADS = 320;
template <int BN, int STAGES>
__global__ void __launch_bounds__(GEMM_THREADS, 1) k_gemm_tc(const __grid_constant__ CUtensorMap tmA,
                                                    const __grid_constant__ CUtensorMap tmB, int K, GemmEpi E)
{
    using S = GemmSmem<BN, STAGES>;
    if (E.skip && *E.skip) return;   // uniform for the launch; before any barrier or TMEM use
    extern __shared__ unsigned char gemm_smem_raw[];
    unsigned char *sm = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(gemm_smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(sm + S::BARS);
    uint64_t *empty = full + STAGES;
    uint64_t *tfull = empty + STAGES;     // [2]
    uint64_t *tempty = tfull + 2;         // [2]
    uint32_t *tslot = reinterpret_cast<uint32_t *>(tempty + 2);
    __shared__ int s_fail;
    volatile int *fail = &s_fail;         // set by whichever role's wait runs out; read by all
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ny = (E.N + BN - 1) / BN, mt = (E.M + 127) / 128;
    const int x = (int)blockIdx.x, P = (int)gridDim.x, rm = E.row_major_tiles;
    const int units = rm ? mt : mt * ny;   // row tiles, or tiles of the flat order
    const int ntile = (units > x ? (units - 1 - x) / P + 1 : 0) * (rm ? ny : 1);
    auto tile_m0 = [&](int t) { return (rm ? x + (t / ny) * P : (x + t * P) / ny) * 128; };
    auto tile_n0 = [&](int t) { return (rm ? t % ny : (x + t * P) % ny) * BN; };
    const int nk_all = (K + 63) / 64;
    const int kb0 = gridDim.z > 1 ? (int)blockIdx.z * E.kpz : 0;
    const int nk = gridDim.z > 1 ? min(E.kpz, nk_all - kb0) : nk_all;
    if (threadIdx.x == 0) {
        s_fail = 0;
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(&tfull[a], 1);
            mbar_init(&tempty[a], 8);     // one arrival per epilogue warp
        }
        mbar_fence_init();
    }
    if (warp == 0) tmem_alloc(tslot, 2 * S::TMEM_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = *tslot;

    if (warp == 0) {
        if (lane == 0) {
            // ---- TMA producer: K block g of the CTA's sequence goes to slot g % STAGES
            long long g = 0;
            for (int t = 0; t < ntile && !*fail; ++t) {
                const int m0 = tile_m0(t), n0 = tile_n0(t);
                for (int kb = 0; kb < nk; ++kb, ++g) {
                    const int s = (int)(g % STAGES);
                    if (g >= STAGES &&
                        !mbar_wait_bounded(&empty[s], (uint32_t)(((g / STAGES) - 1) & 1), TC_WAIT_CYCLES)) {
                        atomicExch(&s_fail, 1);
                        break;
                    }
                    unsigned char *a = sm + s * S::STAGE;
                    mbar_arrive_expect_tx(&full[s], (uint32_t)S::STAGE);
                    tma_load_2d(a, &tmA, (kb0 + kb) * 64, m0, &full[s]);
                    tma_load_2d(a + S::A_BYTES, &tmB, (kb0 + kb) * 64, n0, &full[s]);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer
            constexpr uint32_t idesc = tc_idesc_bf16(BN);
            long long g = 0;
            for (int t = 0; t < ntile && !*fail; ++t) {
                const int acc = t & 1;
                if (t >= 2 && !mbar_wait_bounded(&tempty[acc], (uint32_t)(((t >> 1) - 1) & 1), TC_WAIT_CYCLES)) {
                    atomicExch(&s_fail, 1);
                    break;
                }
                tc_fence_after();
                const uint32_t tacc = taddr + (uint32_t)(acc * S::TMEM_COLS);
                bool ok = true;
                for (int kb = 0; kb < nk; ++kb, ++g) {
                    const int s = (int)(g % STAGES);
                    if (!mbar_wait_bounded(&full[s], (uint32_t)((g / STAGES) & 1), TC_WAIT_CYCLES)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t a = smem_u32(sm + s * S::STAGE);
                    const uint32_t b = a + S::A_BYTES;
#pragma unroll
                    for (int k16 = 0; k16 < 4; ++k16)
                        tc_mma_bf16(tacc, tc_smem_desc_sw128(a + 32 * k16), tc_smem_desc_sw128(b + 32 * k16), idesc,
                                    (kb | k16) != 0 ? 1u : 0u);
                    tc_commit(&empty[s]);      // the stage is free once these MMAs have read it
                }
                if (!ok) {
                    atomicExch(&s_fail, 1);
                    break;
                }
                tc_commit(&tfull[acc]);        // the tile's MMAs are complete
            }
        }
    } else {
        // ---- epilogue warps 2..9: TMEM lanes 32 (warp % 4) .., columns of half (warp - 2) / 4 (a
        // tile narrower than 32 columns is left to the first half)
        const int ew = warp & 3, half = (warp - 2) >> 2;
        const int cb0 = BN >= 32 ? half * (BN / 2) : (half ? BN : 0);
        const int cb1 = BN >= 32 ? cb0 + BN / 2 : (half ? BN : BN);
        for (int t = 0; t < ntile; ++t) {
            const int acc = t & 1;
            const bool ok = mbar_wait_bounded(&tfull[acc], (uint32_t)((t >> 1) & 1), TC_WAIT_CYCLES);
            if (!ok) atomicExch(&s_fail, 1);
            __syncwarp();
            if (__any_sync(0xffffffffu, !ok || *fail)) break;
            tc_fence_after();
            gemm_epi_tile(E, taddr + (uint32_t)(acc * S::TMEM_COLS) + ((uint32_t)(ew * 32) << 16),
                          tile_m0(t) + ew * 32 + lane, tile_n0(t), (int)blockIdx.z, cb0, cb1);
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[acc]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (*fail && threadIdx.x == 0) atomicOr(E.err, 2);
    if (warp == 0) tmem_dealloc(taddr, 2 * S::TMEM_COLS);
}

}  // namespace omx
