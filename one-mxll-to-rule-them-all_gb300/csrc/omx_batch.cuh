// omx_batch.cuh -- batched multi-grid launches.  Several independent 3D grids advance together:
// each pass (H, bulk E) is ONE persistent launch whose blocks walk a tile list that concatenates
// every grid's 32 x 4 x kch tiles (grid-major), and the point sources and detectors of all grids
// go in one launch each (k_src_batch / k_sample_batch).  A block copies the arguments of the grid it is working on into shared
// memory when it moves to another grid; the tile arithmetic is the single-grid kernels' own
// (h3_tile / e3_tile, src_point, sample_point), so every grid's result equals its solo run.
#pragma once
#include "omx_stencil.cuh"

namespace omx {

template <class R, bool EXACT, int PASS>
__global__ void __launch_bounds__(128, 5) k_batch3(const BatchGrid<R> *__restrict__ grids, int n, long long total, int kch)
{
    __shared__ __align__(16) unsigned char raw[sizeof(BatchGrid<R>)];
    const BatchGrid<R> &sg = *reinterpret_cast<const BatchGrid<R> *>(raw);
    const int tid = threadIdx.x + 32 * threadIdx.y;
    int cur = -1;
    for (long long t = blockIdx.x; t < total; t += gridDim.x) {
        int g = cur < 0 ? 0 : cur;
        while (g + 1 < n && grids[g + 1].tile0 <= t) ++g;          // tiles only move forward
        if (g != cur) {
            __syncthreads();                                       // done with the previous grid
            const int *src = reinterpret_cast<const int *>(&grids[g]);
            int *dst = reinterpret_cast<int *>(raw);
            for (int w = tid; w < (int)(sizeof(BatchGrid<R>) / 4); w += 128) dst[w] = src[w];
            __syncthreads();
            cur = g;
        }
        const long long lt = t - sg.tile0;
        const int bx = (int)(lt % sg.tx);
        const int by = (int)((lt / sg.tx) % sg.ty);
        const int bz = (int)(lt / ((long long)sg.tx * sg.ty));
        if (PASS == 0) h3_tile<R, EXACT>(sg.F, sg.G, kch, bx, by, bz);
        else e3_tile<R, EXACT>(sg.F, sg.G, kch, bx, by, bz);
    }
}

template <class R, bool EXACT>
void launch_batch3_impl(int pass, const BatchGrid<R> *grids, int n, long long total, int kch, int blocks, void *s)
{
    if (n <= 0 || total <= 0) return;
    const int g = (int)(total < blocks ? total : blocks);
    const dim3 b(32, 4, 1);
    if (pass == 0) k_batch3<R, EXACT, 0><<<g, b, 0, (cudaStream_t)s>>>(grids, n, total, kch);
    else k_batch3<R, EXACT, 1><<<g, b, 0, (cudaStream_t)s>>>(grids, n, total, kch);
}

template <class R, bool EXACT> int batch3_blocks_impl()
{
    int dev = 0, sms = 0, a = 0, b = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_batch3<R, EXACT, 0>, 128, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_batch3<R, EXACT, 1>, 128, 0);
    const int per = a < b ? a : b;
    return (sms > 0 ? sms : 152) * (per > 0 ? per : 1);
}

}  // namespace omx
