// Ray splitting at one surface (rSplit of the reference): its own
// translation unit so that it compiles in parallel with the fused trace.
#include <cuda_runtime.h>
#include "bt_internal.h"
#include "bt_device.cuh"
#include "bt_stage_smem.cuh"

#define TRACE_THREADS 256

// Reads and clears this translation unit's device status word.
cudaError_t bt_read_split_device_status(int* status, cudaStream_t stream) {
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

// ---------------------------------------------------------------------------
// Split at one surface (src/batoid.cpp:509-674): the refracted ray replaces
// the input ray, the reflected ray goes to `sp` (which holds a copy of the
// input on entry); fluxes take the coating's transmit / reflect factors.
// Stage 0 of the program: the surface, its transform, the outgoing medium
// and the coating factors.
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(TRACE_THREADS)
k_rsplit(const unsigned char* __restrict__ gblob, int blob_bytes, RV rv, RV sp, int niter) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar;
    if (!bt_stage_blob(smem, gblob, blob_bytes, &bar)) return;
    const Prog P = prog_from_blob(smem);
    const bt_stage& st = P.stages[0];
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < rv.n; i += stride) {
        if (rv.fail[i]) continue;
        const double dx = rv.x[i] - st.dr[0], dy = rv.y[i] - st.dr[1], dz = rv.z[i] - st.dr[2];
        double x = dx * st.drot[0] + dy * st.drot[3] + dz * st.drot[6];
        double y = dx * st.drot[1] + dy * st.drot[4] + dz * st.drot[7];
        double z = dx * st.drot[2] + dy * st.drot[5] + dz * st.drot[8];
        const double vx = rv.vx[i] * st.drot[0] + rv.vy[i] * st.drot[3] + rv.vz[i] * st.drot[6];
        const double vy = rv.vx[i] * st.drot[1] + rv.vy[i] * st.drot[4] + rv.vz[i] * st.drot[7];
        const double vz = rv.vx[i] * st.drot[2] + rv.vy[i] * st.drot[5] + rv.vz[i] * st.drot[8];
        double dt = 0.0;
        if (!bt_surf_tti_fast(P, st.surf, x, y, z, vx, vy, vz, dt, niter)) {
            rv.vig[i] = 1;
            rv.fail[i] = 1;
            sp.vig[i] = 1;
            sp.fail[i] = 1;
            continue;
        }
        x += vx * dt;
        y += vy * dt;
        z += vz * dt;
        const double t = rv.t[i] + dt;
        const double n1 = 1.0 / sqrt(vx * vx + vy * vy + vz * vz);
        const double nvx = vx * n1, nvy = vy * n1, nvz = vz * n1;
        double nx, ny, nz;
        bt_normal_precise(P, st.surf, x, y, &nx, &ny, &nz);
        double alpha = nvx * nx + nvy * ny + nvz * nz;
        if (alpha > 0.) {
            nx = -nx; ny = -ny; nz = -nz;
            alpha = -alpha;
        }
        const double w = rv.w[i];
        const double f = rv.f[i];
        // reflection
        sp.x[i] = x;
        sp.y[i] = y;
        sp.z[i] = z;
        sp.vx[i] = vx - 2 * alpha * nx / n1;
        sp.vy[i] = vy - 2 * alpha * ny / n1;
        sp.vz[i] = vz - 2 * alpha * nz / n1;
        sp.t[i] = t;
        sp.w[i] = w;
        sp.f[i] = f * st.coat_r;
        sp.vig[i] = rv.vig[i];
        sp.fail[i] = 0;
        // refraction
        const double n2 = bt_getN(P, st.medium, w);
        const double eta = n1 / n2;
        const double sinsqr = eta * eta * (1 - alpha * alpha);
        rv.x[i] = x;
        rv.y[i] = y;
        rv.z[i] = z;
        rv.t[i] = t;
        if (sinsqr > 1.0) {
            rv.vx[i] = NAN;
            rv.vy[i] = NAN;
            rv.vz[i] = NAN;
            rv.fail[i] = 1;
            rv.vig[i] = 1;
        } else {
            const double nfactor = eta * alpha + sqrt(1 - sinsqr);
            rv.vx[i] = (eta * nvx - nfactor * nx) / n2;
            rv.vy[i] = (eta * nvy - nfactor * ny) / n2;
            rv.vz[i] = (eta * nvz - nfactor * nz) / n2;
        }
        rv.f[i] = f * st.coat_t;
    }
}

cudaError_t bt_launch_rsplit(const unsigned char* d_blob, int blob_bytes, const RV& rv, const RV& sp, int niter,
                             cudaStream_t stream) {
    if (rv.n <= 0) return cudaSuccess;
    if (blob_bytes > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_rsplit, cudaFuncAttributeMaxDynamicSharedMemorySize, blob_bytes);
        if (e != cudaSuccess) return e;
    }
    k_rsplit<<<bt_grid_for(rv.n, TRACE_THREADS, 16), TRACE_THREADS, blob_bytes, stream>>>(d_blob, blob_bytes, rv, sp,
                                                                                       niter);
    return cudaGetLastError();
}

