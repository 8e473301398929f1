// Fused sequential trace: one thread carries one ray through every stage of
// an optic, in registers.  Replaces the per-surface OpenMP passes of the
// reference (src/batoid.cpp:151-506) driven by CompoundOptic.trace
// (batoid/optic.py:1013-1083): instead of reading and writing all 74 bytes
// per ray once per surface, each ray is loaded once and stored once.
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>
#include "bt_internal.h"
#include "bt_device.cuh"
#include "bt_stage_smem.cuh"
#include "bt_trace_core.cuh"

cudaError_t bt_read_device_status(int* status, cudaStream_t stream) {
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

#define TRACE_THREADS 256
#define BT_TRACE_MINB 2

// MINB = resident blocks per SM the register budget is sized for: 2 gives
// 128 registers (16 warps per SM).  (1, the compiler's choice of registers
// and 8 warps per SM, measured slower.)
//
// Stage-synchronous: the block's rays advance one stage at a time with a
// barrier between stages, so all warps of the block run the same stage's
// code together.  The code for all stage and surface kinds is far larger
// than the instruction cache; warps spread over different stages missed in
// it most of the time (ncu: instruction-cache hit rate 67 % and
// "no instruction" the second stall reason), and the barrier keeps the
// working set to one stage's code.  Rays of a stage differ only in Newton
// iteration counts, so the barrier wait is short.
template <int MINB>
__global__ void __launch_bounds__(TRACE_THREADS, MINB)
k_trace(const unsigned char* __restrict__ gblob, int blob_bytes, RV in, RV out,
        const __grid_constant__ SnapSet snaps, int nsnaps, int niter) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar;
    if (!bt_stage_blob(smem, gblob, blob_bytes, &bar)) return;
    const Prog P = prog_from_blob(smem);
    const int T = blockDim.x;
    const long long stride = (long long)gridDim.x * T;
    // block-uniform trip counts: every thread reaches every barrier
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
        int cached_medium = -1;
        double cached_n = 0.0, cached_inv_n = 0.0;
        for (int s = 0; s < P.nstages; s++) {
            if (act) {
                run_stage(P, P.stages[s], r, niter, cached_medium, cached_n, cached_inv_n);
                if (s < nsnaps) store_ray(snaps.s[s], i, r);
            }
            __syncthreads();
        }
        if (act && nsnaps == 0) store_ray(out, i, r);
    }
}

static int g_sm_count = 0;

// The library's short-lived scratch comes from the device's default memory
// pool (cudaMallocAsync).  By default the pool returns freed memory to the
// driver at every synchronisation, so each call would map its scratch anew;
// keeping up to 256 MiB cached makes repeated calls reuse it.  A property of
// this process's pool, set once.
void bt_keep_pool() {
    static bool done = false;
    if (done) return;
    done = true;
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    uint64_t keep = 256ull << 20;
    if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) cudaGetLastError();
}

int bt_sm_count() {
    if (g_sm_count == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev);
        if (g_sm_count <= 0) g_sm_count = 1;
    }
    return g_sm_count;
}

int bt_grid_for(long long n, int threads, int per_sm) {
    long long need = (n + threads - 1) / threads;
    long long cap = (long long)bt_sm_count() * per_sm;
    if (need > cap) need = cap;
    if (need < 1) need = 1;
    return (int)need;
}

cudaError_t bt_launch_trace(const unsigned char* d_blob, int blob_bytes, const RV& in, const RV& out,
                            const SnapSet* snaps, int nsnaps, int niter, cudaStream_t stream) {
    if (in.n <= 0) return cudaSuccess;
    // The float-float form (trace_ff.cu) unless Newton is capped below 3
    // iterations (its float-float iterations then cannot stand for the
    // reference's FP64 ones) or BATOID_GB300_TRACE_FORM=fp64 asks for the
    // FP64 form (a diagnostic: both forms meet the same tolerances).
    static int form = -1;
    if (form < 0) {
        const char* env = getenv("BATOID_GB300_TRACE_FORM");
        form = (env && strcmp(env, "fp64") == 0) ? 0 : 1;
    }
    if (form == 1 && niter >= 3) return bt_launch_trace_ff(d_blob, blob_bytes, in, out, snaps, nsnaps, niter, stream);
    static SnapSet empty;
    const SnapSet& ss = snaps ? *snaps : empty;
    auto kern = k_trace<BT_TRACE_MINB>;
    if (blob_bytes > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, blob_bytes);
        if (e != cudaSuccess) return e;
    }
    // Persistent grid (2 blocks per SM): the blob is staged once per block
    // and amortised over the grid-stride loop.
    const int grid = bt_grid_for(in.n, TRACE_THREADS, 2);
    kern<<<grid, TRACE_THREADS, blob_bytes, stream>>>(d_blob, blob_bytes, in, out, ss, nsnaps, niter);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Surface sag / normal, medium index and obscuration evaluated on arrays.
// Each takes a one-surface / one-medium / one-obscuration program.
// ---------------------------------------------------------------------------

__global__ void k_surface_eval(const unsigned char* __restrict__ gblob, int blob_bytes, const double* x,
                               const double* y, double* sag, double* normal, long long n) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar;
    if (!bt_stage_blob(smem, gblob, blob_bytes, &bar)) return;
    const Prog P = prog_from_blob(smem);
    const int si = P.stages[0].surf;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double xx = x[i], yy = y[i];
        if (sag) {
            double s, ux, uy;
            bt_surf_eval(P, si, xx, yy, true, false, &s, &ux, &uy);
            sag[i] = s;
        }
        if (normal) {
            double nx, ny, nz;
            bt_surf_normal(P, si, xx, yy, &nx, &ny, &nz);
            normal[i] = nx;
            normal[i + n] = ny;
            normal[i + 2 * n] = nz;
        }
    }
}

cudaError_t bt_launch_surface_eval(const unsigned char* d_blob, int blob_bytes, const double* x,
                                   const double* y, double* sag, double* normal, long long n,
                                   cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    if (blob_bytes > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_surface_eval, cudaFuncAttributeMaxDynamicSharedMemorySize, blob_bytes);
        if (e != cudaSuccess) return e;
    }
    k_surface_eval<<<bt_grid_for(n, 256, 8), 256, blob_bytes, stream>>>(d_blob, blob_bytes, x, y, sag, normal, n);
    return cudaGetLastError();
}

__global__ void k_getN(const unsigned char* __restrict__ gblob, int blob_bytes, const double* w, double* out,
                       long long n) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar;
    if (!bt_stage_blob(smem, gblob, blob_bytes, &bar)) return;
    const Prog P = prog_from_blob(smem);
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = bt_getN(P, 0, w[i]);
}

cudaError_t bt_launch_getN(const unsigned char* d_blob, int blob_bytes, const double* w, double* out,
                           long long n, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    k_getN<<<bt_grid_for(n, 256, 8), 256, blob_bytes, stream>>>(d_blob, blob_bytes, w, out, n);
    return cudaGetLastError();
}

// Either fills out[i] = contains(x[i], y[i]) or, given a ray bundle, applies
// vignetted |= contains(x, y) (src/batoid.cpp:151-172).
__global__ void k_obsc(const unsigned char* __restrict__ gblob, int blob_bytes, const double* x, const double* y,
                       uint8_t* out, RV rv, int use_rv, long long n) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar;
    if (!bt_stage_blob(smem, gblob, blob_bytes, &bar)) return;
    const Prog P = prog_from_blob(smem);
    const bt_stage& st = P.stages[0];
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        if (use_rv) {
            if (bt_obsc_run(P, st.obsc_begin, st.obsc_end, rv.x[i], rv.y[i])) rv.vig[i] = 1;
        } else {
            out[i] = bt_obsc_run(P, st.obsc_begin, st.obsc_end, x[i], y[i]) ? 1 : 0;
        }
    }
}

cudaError_t bt_launch_obsc(const unsigned char* d_blob, int blob_bytes, const double* x, const double* y,
                           uint8_t* out, const RV* rv, long long n, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    RV dummy = {};
    k_obsc<<<bt_grid_for(n, 256, 8), 256, blob_bytes, stream>>>(d_blob, blob_bytes, x, y, out, rv ? *rv : dummy,
                                                             rv ? 1 : 0, n);
    return cudaGetLastError();
}
