// Fused sequential trace, float-float form (bt_trace_ff.cuh): one thread
// carries one ray through every stage, in registers, as in trace.cu.
#include <cuda_runtime.h>
#include <stdlib.h>
#include "bt_internal.h"
#include "bt_device.cuh"
#include "bt_stage_smem.cuh"
#include "bt_trace_core.cuh"
#define BT_FF_INLINE_NEWTON 1
#include "bt_trace_ff.cuh"

#define TRACE_FF_THREADS 256
#define TRACE_FF_MINB 2

// Reads and clears this translation unit's device status word.
cudaError_t bt_read_trace_ff_device_status(int* status, cudaStream_t stream) {
    int zero = 0;
    cudaError_t e = cudaMemcpyFromSymbolAsync(status, bt_dev_status, sizeof(int), 0,
                                              cudaMemcpyDeviceToHost, stream);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return e;
    if (*status != 0) {
        e = cudaMemcpyToSymbolAsync(bt_dev_status, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, stream);
        if (e != cudaSuccess) return e;
        e = cudaStreamSynchronize(stream);
    }
    return e;
}

// Stage-synchronous like k_trace: a barrier after every stage keeps one
// stage's code live per block.  Register budget for 2 resident blocks per
// SM (128 registers, 16 warps per SM); 3 blocks (80 registers, 24 warps)
// measured 18 % slower (spills).
__global__ void __launch_bounds__(TRACE_FF_THREADS, TRACE_FF_MINB)
k_trace_ff(const unsigned char* __restrict__ gblob, int blob_bytes, RV in, RV out,
           const __grid_constant__ SnapSet snaps, int nsnaps, int niter) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar;
    if (!bt_stage_blob(smem, gblob, blob_bytes, &bar)) return;
    // a per-thread copy (on the stack, as the out-of-line helpers take it by
    // reference): measured 1.5 % faster than one shared copy per block
    const Prog P = prog_from_blob(smem);
    const int T = blockDim.x;
    const long long stride = (long long)gridDim.x * T;
    for (long long base = (long long)blockIdx.x * T; base < in.n; base += stride) {
        const long long i = base + threadIdx.x;
        const bool act = i < in.n;
        RayState r;
        if (act) {
            r.x = in.x[i];
            r.y = in.y[i];
            r.z = in.z[i];
            r.vx = in.vx[i];
            r.vy = in.vy[i];
            r.vz = in.vz[i];
            r.t = in.t[i];
            r.w = in.w[i];
            r.f = in.f[i];
            r.vig = in.vig[i] != 0;
            r.fail = in.fail[i] != 0;
        }
        MediumCacheF mc;
        mc.idx = -1;
        RayCacheF fc;
        fc.ok = false;
        for (int s = 0; s < P.nstages; s++) {
            if (act) {
                run_stage_ff(P, P.stages[s], r, niter, mc, fc);
                if (s < nsnaps) store_ray(snaps.s[s], i, r);
            }
            __syncthreads();
        }
        if (act && nsnaps == 0) store_ray(out, i, r);
    }
}

// Rays one launch of the persistent grid takes per round.
long long bt_trace_ff_round_rays() { return (long long)bt_sm_count() * TRACE_FF_MINB * TRACE_FF_THREADS; }

cudaError_t bt_launch_trace_ff(const unsigned char* d_blob, int blob_bytes, const RV& in, const RV& out,
                               const SnapSet* snaps, int nsnaps, int niter, cudaStream_t stream) {
    if (in.n <= 0) return cudaSuccess;
    static SnapSet empty;
    const SnapSet& ss = snaps ? *snaps : empty;
    if (blob_bytes > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_trace_ff, cudaFuncAttributeMaxDynamicSharedMemorySize, blob_bytes);
        if (e != cudaSuccess) return e;
    }
    const int grid = bt_grid_for(in.n, TRACE_FF_THREADS, TRACE_FF_MINB);
    k_trace_ff<<<grid, TRACE_FF_THREADS, blob_bytes, stream>>>(d_blob, blob_bytes, in, out, ss, nsnaps, niter);
    return cudaGetLastError();
}
