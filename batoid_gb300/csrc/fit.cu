// Normal equations of the Zernike wavefront fit (batoid/analysis.py:563-573:
// basis construction + least squares).  One block per fit: the block
// evaluates the Cartesian-polynomial basis at a tile of points into shared
// memory and accumulates the upper triangle of B^T B and B^T v in FP64.
// Many fits (e.g. every (state, field) of a batched wavefront run) go in one
// launch, one block each, with no inter-block communication.
#include <cuda_runtime.h>
#include <stdint.h>
#include "bt_internal.h"

#define FIT_THREADS 256
#define FIT_TILE 32
#define FIT_MAX_J 64
#define FIT_MAX_SIDE 12
#define FIT_MAX_ACC 10  // ceil((FIT_MAX_J*(FIT_MAX_J+1)/2 + FIT_MAX_J) / FIT_THREADS)

__global__ void __launch_bounds__(FIT_THREADS)
k_zk_normal(const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ v,
            const long long* __restrict__ offsets, const double* __restrict__ basis, int jmax, int side,
            double* G, double* b) {
    extern __shared__ double sm[];
    double* sbasis = sm;                            // jmax * side * side
    double* sval = sbasis + jmax * side * side;     // FIT_TILE * (jmax + 1)
    const int fit = blockIdx.x;
    const long long p0 = offsets[fit], p1 = offsets[fit + 1];
    const int nb = jmax * side * side;
    for (int i = threadIdx.x; i < nb; i += FIT_THREADS) sbasis[i] = basis[i];
    const int npairs = jmax * (jmax + 1) / 2;
    const int ntot = npairs + jmax;
    double acc[FIT_MAX_ACC];
#pragma unroll
    for (int q = 0; q < FIT_MAX_ACC; q++) acc[q] = 0.0;
    __syncthreads();
    const int stride = jmax + 1;
    for (long long base = p0; base < p1; base += FIT_TILE) {
        const int cnt = (int)((p1 - base) < FIT_TILE ? (p1 - base) : FIT_TILE);
        // basis values: thread -> (point, basis function) pairs
        for (int e = threadIdx.x; e < cnt * jmax; e += FIT_THREADS) {
            const int pt = e / jmax, j = e % jmax;
            const double xx = x[base + pt], yy = y[base + pt];
            const double* c = sbasis + j * side * side;
            // sum_a sum_b c[a][b] x^a y^b by 2-D Horner
            double r = 0.0;
            for (int a = side - 1; a >= 0; a--) {
                double row = 0.0;
                for (int bb = side - 1; bb >= 0; bb--) row = row * yy + c[a * side + bb];
                r = r * xx + row;
            }
            sval[pt * stride + j] = r;
        }
        for (int pt = threadIdx.x; pt < cnt; pt += FIT_THREADS) sval[pt * stride + jmax] = v[base + pt];
        __syncthreads();
        int q = 0;
        for (int p = threadIdx.x; p < ntot; p += FIT_THREADS, q++) {
            int j, k;
            if (p < npairs) {
                // p -> (j, k), j <= k, row-major over the upper triangle
                j = 0;
                int rem = p;
                while (rem >= jmax - j) { rem -= jmax - j; j++; }
                k = j + rem;
            } else {
                j = p - npairs;
                k = jmax;  // right-hand side column
            }
            double s = 0.0;
            for (int pt = 0; pt < cnt; pt++) s += sval[pt * stride + j] * sval[pt * stride + k];
            acc[q] += s;
        }
        __syncthreads();
    }
    int q = 0;
    for (int p = threadIdx.x; p < ntot; p += FIT_THREADS, q++) {
        if (p < npairs) {
            int j = 0, rem = p;
            while (rem >= jmax - j) { rem -= jmax - j; j++; }
            const int k = j + rem;
            G[(long long)fit * jmax * jmax + j * jmax + k] = acc[q];
            G[(long long)fit * jmax * jmax + k * jmax + j] = acc[q];
        } else {
            b[(long long)fit * jmax + (p - npairs)] = acc[q];
        }
    }
}

cudaError_t bt_launch_zk_normal(const double* x, const double* y, const double* v, const long long* offsets,
                                int nfits, const double* basis, int jmax, int side, double* G, double* b,
                                cudaStream_t stream) {
    if (nfits <= 0) return cudaSuccess;
    if (jmax < 1 || jmax > FIT_MAX_J || side < 1 || side > FIT_MAX_SIDE) return cudaErrorInvalidValue;
    const size_t smem = sizeof(double) * ((size_t)jmax * side * side + (size_t)FIT_TILE * (jmax + 1));
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_zk_normal, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k_zk_normal<<<nfits, FIT_THREADS, smem, stream>>>(x, y, v, offsets, basis, jmax, side, G, b);
    return cudaGetLastError();
}
