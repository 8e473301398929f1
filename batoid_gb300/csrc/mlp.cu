// BF16 GEMMs of the wavefront surrogate MLP on the 5th-generation tensor
// cores (tcgen05), FP32 accumulation in tensor memory, with fused epilogues.
//
//   C[M x N] = A[M x K] . B[N x K]^T      (both operands K-major, bf16)
//
// Tiles of 128 x BN (BN = 128 or 256) over a K range; one persistent CTA
// per SM (384 threads) walks the tile list:
//   * warp 0 / lane 0 streams 128 x 64 and BN x 64 operand tiles from global
//     memory with TMA (cp.async.bulk.tensor, 128-byte swizzle) into a
//     4-stage shared-memory ring (full / empty mbarriers);
//   * warp 1 / lane 0 issues tcgen05.mma (M 128, N BN, K 16) from shared
//     memory descriptors into one of two TMEM accumulators of BN columns,
//     releases each stage with tcgen05.commit and hands the finished
//     accumulator to the epilogue;
//   * warps 4..11 read it back with tcgen05.ld (warp w owns TMEM lanes
//     32(w%4)..32(w%4)+31 = tile rows, and half (w-4)/4 of the columns) and
//     run the epilogue while the next tile accumulates in the other buffer;
//     outputs go through a per-warp 4 KB staging tile in shared memory
//     (32 rows x 64 bf16 or 32 FP32 columns, 128-byte swizzle) and leave by
//     TMA store, whole lines at a time.
// Every wait is bounded: on expiry the CTA records BT_ERR_TIMEOUT in the
// device status word, stops issuing, waits (bounded) for the copies and
// MMAs it started, frees its TMEM and returns.
//
// Epilogues (per element (m, n) of the tile):
//   F32      out32[kz][m][n] = acc                       (split-K partials)
//   BIAS     out32[m][n]     = acc + bias[n]             (output layer)
//   GELU     z = acc + bias[n]; zs[m][n] = z;  h = gelu(z) (tanh form);
//            h16[m][n] = h16T[n][m] = bf16(h)             (hidden layers)
//   DGELU    g = acc * gelu'(zs[m][n]);
//            h16[m][n] = h16T[n][m] = bf16(g)             (backward)
#include <cuda_runtime.h>
#include <cuda.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <string.h>
#include <stdlib.h>
#include "bt_internal.h"
#include "bt_stage_smem.cuh"
#include "bt_mlp.h"

#define MLP_BM 128
#define MLP_BK 64
#define MLP_STAGES 4
#define MLP_THREADS 384
#define MLP_EPI_WARP0 4
#define MLP_NEPI 8
#define MLP_STG_BYTES (32 * 64 * 2)  // per epilogue warp: 32 rows x 64 bf16 columns

cudaError_t bt_read_mlp_device_status(int* status, cudaStream_t stream) {
    int zero = 0;
    cudaError_t e = cudaMemcpyFromSymbolAsync(status, bt_dev_status, sizeof(int), 0, cudaMemcpyDeviceToHost, stream);
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
// PTX wrappers
// ---------------------------------------------------------------------------

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bt_smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bt_smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// Bounded parity wait; false when the limit expired or another role aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort) {
    for (uint32_t i = 0; i < BT_WAIT_LIMIT; i++) {
        if (bt_mbar_try_wait(bar, parity)) return true;
        if ((i & 1023u) == 1023u && *abort) return false;
    }
    *abort = 1;
    atomicExch(&bt_dev_status, 5 /* BT_ERR_TIMEOUT */);
    return false;
}

__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, const void* src, int x, int y) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];"
                 ::"l"((uint64_t)map), "r"(x), "r"(y), "r"(bt_smem_addr(src))
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(bt_smem_addr(dst)), "l"((uint64_t)map), "r"(x), "r"(y), "r"(bt_smem_addr(bar))
        : "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, rows of
// 128 bytes in 8-row (1024-byte) atoms.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);   // start address
    d |= (uint64_t)1 << 16;                      // leading byte offset (unused here)
    d |= (uint64_t)(1024 >> 4) << 32;            // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1 << 46;                      // descriptor version
    d |= (uint64_t)2 << 61;                      // 128-byte swizzle
    return d;
}

// Instruction descriptor of kind::f16: D f32, A and B bf16, both K-major.
__device__ __forceinline__ uint32_t mma_idesc(int bn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(bn >> 3) << 17) | ((uint32_t)(MLP_BM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(tmem), "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 ::"r"(bt_smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// GELU, tanh form: 0.5 z (1 + tanh(s (z + 0.044715 z^3))), s = sqrt(2/pi),
// with the hardware tanh approximation (one MUFU op); and its derivative.
__device__ __forceinline__ float tanh_fast(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float gelu_f(float z) {
    const float u = 0.7978845608028654f * fmaf(0.044715f * z, z * z, z);
    return 0.5f * z * (1.0f + tanh_fast(u));
}
__device__ __forceinline__ float dgelu_f(float z) {
    const float z2 = z * z;
    const float t = tanh_fast(0.7978845608028654f * fmaf(0.044715f * z, z2, z));
    return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * 0.7978845608028654f * fmaf(0.134145f, z2, 1.0f);
}

// ---------------------------------------------------------------------------
// The GEMM kernel
// ---------------------------------------------------------------------------

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bt_smem_addr(bar)) : "memory");
}

// Persistent: one CTA per SM walks the tile list (N fastest, so the CTAs
// running together cover whole row blocks of A: A streams from DRAM once and
// the small weight operand stays in L2).  Warp 0 lane 0 streams operands
// into the ring; warp 1 lane 0 issues the MMAs of tile i into TMEM
// accumulator buffer i % 2; warps 4..11 drain the other buffer (epilogue)
// meanwhile.  Barriers: full/empty per ring stage, acc_full/acc_empty per
// accumulator buffer; the first use of each "empty" barrier waits on the
// phase before the barrier's first, which counts as completed.
__global__ void __launch_bounds__(MLP_THREADS, 1)
k_mlp_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
           const __grid_constant__ CUtensorMap tmH, MlpGemmArgs g) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full[MLP_STAGES];
    __shared__ __align__(8) uint64_t empty[MLP_STAGES];
    __shared__ __align__(8) uint64_t acc_full[2];
    __shared__ __align__(8) uint64_t acc_empty[2];
    __shared__ __align__(8) uint64_t done;
    __shared__ uint32_t s_tmem;
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int BN = g.bn;
    const int NS = g.stages;
    const uint32_t raw = bt_smem_addr(smem_raw);
    unsigned char* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    const uint32_t a_bytes = MLP_BM * MLP_BK * 2, b_bytes = (uint32_t)BN * MLP_BK * 2;
    unsigned char* sA = base;
    unsigned char* sB = base + NS * a_bytes;
    unsigned char* sStg = base + NS * (a_bytes + b_bytes);  // epilogue staging, MLP_STG_BYTES per warp
    const int tiles_m = g.M / MLP_BM, tiles_n = g.N / BN;
    const int nk = g.kchunk / MLP_BK;
    volatile int* abort = &s_abort;
    const int nwork = tiles_m * tiles_n * (g.K / g.kchunk);
    const int w0 = blockIdx.x, wstep = gridDim.x;

    if (tid == 0) {
        for (int s = 0; s < NS; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], MLP_NEPI);
        }
        mbar_init(&done, 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(bt_smem_addr(&s_tmem)), "r"((uint32_t)(2 * BN)) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;

    if (warp == 0 && lane == 0) {
        // producer
        int gk = 0;
        for (int t = w0; t < nwork && !*abort; t += wstep) {
            const int kz = t / (tiles_m * tiles_n), r = t - kz * tiles_m * tiles_n;
            const int m0 = (r / tiles_n) * MLP_BM, n0 = (r % tiles_n) * BN;
            const int kbeg = kz * g.kchunk;
            for (int kb = 0; kb < nk; kb++, gk++) {
                const int s = gk % NS;
                if (!mbar_wait(&empty[s], ((gk / NS) & 1) ^ 1, abort)) break;
                mbar_expect_tx(&full[s], a_bytes + b_bytes);
                tma_load_2d(sA + s * a_bytes, &tmA, kbeg + kb * MLP_BK, m0, &full[s]);
                tma_load_2d(sB + s * b_bytes, &tmB, kbeg + kb * MLP_BK, n0, &full[s]);
            }
        }
        // copies still in flight complete before the CTA may exit
        for (int k = (gk > NS ? gk - NS : 0); k < gk; k++) {
            for (uint32_t i = 0; i < BT_WAIT_LIMIT; i++)
                if (bt_mbar_try_wait(&full[k % NS], (k / NS) & 1)) break;
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        const uint32_t idesc = mma_idesc(BN);
        int gk = 0, it = 0;
        for (int t = w0; t < nwork && !*abort; t += wstep, it++) {
            const int b = it & 1;
            if (!mbar_wait(&acc_empty[b], ((it >> 1) & 1) ^ 1, abort)) break;
            tc_fence_after();
            const uint32_t d = tmem + (uint32_t)(b * BN);
            bool ok = true;
            for (int kb = 0; kb < nk; kb++, gk++) {
                const int s = gk % NS;
                if (!mbar_wait(&full[s], (gk / NS) & 1, abort)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t a0 = bt_smem_addr(sA + s * a_bytes), b0 = bt_smem_addr(sB + s * b_bytes);
#pragma unroll
                for (int k = 0; k < MLP_BK / 16; k++)
                    mma_bf16(d, sw128_desc(a0 + k * 32), sw128_desc(b0 + k * 32), idesc, (kb > 0 || k > 0) ? 1u : 0u);
                mma_commit(&empty[s]);
            }
            if (!ok) break;
            mma_commit(&acc_full[b]);
        }
        // completes once every MMA issued above has finished
        mma_commit(&done);
    } else if (warp >= MLP_EPI_WARP0) {
        // epilogue: warp w reads TMEM lanes 32 (w % 4).. and half (w - 4) / 4 of the columns
        const int q = warp & 3, half = (warp - MLP_EPI_WARP0) >> 2;
        unsigned char* stg = sStg + (warp - MLP_EPI_WARP0) * MLP_STG_BYTES;
        int it = 0;
        for (int t = w0; t < nwork; t += wstep, it++) {
            const int b = it & 1;
            if (!mbar_wait(&acc_full[b], (it >> 1) & 1, abort)) break;
            tc_fence_after();
            const int kz = t / (tiles_m * tiles_n), r = t - kz * tiles_m * tiles_n;
            const int m0 = (r / tiles_n) * MLP_BM, n0 = (r % tiles_n) * BN;
            const int m = m0 + q * 32 + lane;
            const uint32_t trow = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * BN);
            const int c0 = half * (BN / 2);
            for (int c = c0; c < c0 + BN / 2; c += 32) {
                const int nb = n0 + c;
                // this chunk's bias (or pre-activations) are requested before
                // the TMEM load so that both latencies overlap
                float4 pre[8];
                if (g.mode == MLP_EPI_BIAS || g.mode == MLP_EPI_GELU) {
                    const float4* b4 = reinterpret_cast<const float4*>(g.bias + nb);
#pragma unroll
                    for (int k = 0; k < 8; k++) pre[k] = __ldg(b4 + k);
                } else if (g.mode == MLP_EPI_DGELU) {
                    const float4* z4 = reinterpret_cast<const float4*>(g.zs + (size_t)m * g.N + nb);
#pragma unroll
                    for (int k = 0; k < 8; k++) pre[k] = z4[k];
                }
                float v[32];
                tmem_ld32(trow + (uint32_t)c, v);
                if (g.mode == MLP_EPI_F32 || g.mode == MLP_EPI_BIAS) {
                    // row `lane` of a 32 x 32 FP32 staging tile (128-byte
                    // rows, chunk j at j ^ (row % 8)), stored by TMA
                    if (g.mode == MLP_EPI_BIAS) {
#pragma unroll
                        for (int i = 0; i < 32; i += 4) {
                            const float4 bb = pre[i / 4];
                            v[i] += bb.x;
                            v[i + 1] += bb.y;
                            v[i + 2] += bb.z;
                            v[i + 3] += bb.w;
                        }
                    }
                    if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                    __syncwarp();
#pragma unroll
                    for (int j = 0; j < 8; j++)
                        *reinterpret_cast<float4*>(stg + lane * 128 + ((j ^ (lane & 7)) << 4)) =
                            make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) tma_store_2d(&tmH, stg, nb, kz * g.M + m0 + q * 32);
                } else {
                    float h[32];
                    if (g.mode == MLP_EPI_GELU) {
#pragma unroll
                        for (int i = 0; i < 32; i += 4) {
                            const float4 bb = pre[i / 4];
                            v[i] += bb.x;
                            v[i + 1] += bb.y;
                            v[i + 2] += bb.z;
                            v[i + 3] += bb.w;
                        }
#pragma unroll
                        for (int i = 0; i < 32; i++) h[i] = gelu_f(v[i]);
                        if (g.zs) {
                            float* zs = g.zs + (size_t)m * g.N + nb;
#pragma unroll
                            for (int i = 0; i < 32; i += 4) *reinterpret_cast<float4*>(zs + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
                        }
                    } else {  // MLP_EPI_DGELU
#pragma unroll
                        for (int i = 0; i < 32; i += 4) {
                            const float4 zz = pre[i / 4];
                            h[i] = v[i] * dgelu_f(zz.x);
                            h[i + 1] = v[i + 1] * dgelu_f(zz.y);
                            h[i + 2] = v[i + 2] * dgelu_f(zz.z);
                            h[i + 3] = v[i + 3] * dgelu_f(zz.w);
                        }
                    }
                    // row `lane` of the 32 x 64 staging tile; 16-byte chunk j of
                    // the row sits at chunk j ^ (row % 8) (128-byte swizzle)
                    const int hh = ((c - c0) >> 5) & 1;
                    if (hh == 0) {
                        // the previous store from this tile has finished reading it
                        if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                        __syncwarp();
                    }
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        __align__(16) __nv_bfloat162 p[4];
#pragma unroll
                        for (int e = 0; e < 4; e++) p[e] = __floats2bfloat162_rn(h[8 * k + 2 * e], h[8 * k + 2 * e + 1]);
                        const int j = hh * 4 + k;
                        *reinterpret_cast<uint4*>(stg + lane * 128 + ((j ^ (lane & 7)) << 4)) = *reinterpret_cast<uint4*>(p);
                    }
                    if (hh == 1) {
                        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                        __syncwarp();
                        if (lane == 0) tma_store_2d(&tmH, stg, nb - 32, m0 + q * 32);
                    }
                    if (g.h16t) {
#pragma unroll
                        for (int i = 0; i < 32; i++) g.h16t[(size_t)(nb + i) * g.M + m] = __float2bfloat16_rn(h[i]);
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[b]);
        }
        // tiles stored by TMA are complete before the CTA exits
        if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    }
    __syncwarp();
    mbar_wait(&done, 0, abort);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)(2 * BN)) : "memory");
    }
}

// ---------------------------------------------------------------------------
// Host side: tensor maps and launch
// ---------------------------------------------------------------------------

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// Row-major bf16 matrix [rows][cols] viewed as (cols, rows) with a box of
// 64 x box_rows elements and 128-byte swizzle.
static bool make_map(CUtensorMap* map, const void* ptr, int rows, int cols, int box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
    cuuint32_t box[2] = {MLP_BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Row-major FP32 matrix [rows][cols] viewed as (cols, rows) with a box of
// 32 x 32 elements (128-byte rows) and 128-byte swizzle: the epilogue's
// FP32 staging tile.
static bool make_map_f32(CUtensorMap* map, const void* ptr, long long rows, int cols) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * 4};
    cuuint32_t box[2] = {32, 32};
    cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(ptr), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static int mlp_stages(int bn) { return MLP_STAGES; }

size_t bt_mlp_gemm_smem(int bn) {
    return 1024 + (size_t)mlp_stages(bn) * (MLP_BM * MLP_BK * 2 + (size_t)bn * MLP_BK * 2) +
           (size_t)MLP_NEPI * MLP_STG_BYTES;
}

cudaError_t bt_launch_mlp_gemm(const __nv_bfloat16* A, const __nv_bfloat16* B, const MlpGemmArgs& a, int splitk,
                               cudaStream_t stream) {
    if (a.M % MLP_BM || (a.bn != 128 && a.bn != 256) || a.N % a.bn || splitk < 1 || a.K % (splitk * MLP_BK))
        return cudaErrorInvalidValue;
    if (splitk > 1 && a.mode != MLP_EPI_F32) return cudaErrorInvalidValue;  // only partials are split
    if (((uintptr_t)A & 15) || ((uintptr_t)B & 15)) return cudaErrorInvalidValue;
    const long long ntiles = (long long)(a.M / MLP_BM) * (a.N / a.bn) * splitk;
    const int sms = bt_sm_count();
    CUtensorMap ta, tb, th;
    if (!make_map(&ta, A, a.M, a.K, MLP_BM) || !make_map(&tb, B, a.N, a.K, a.bn))
        return cudaErrorInvalidValue;
    memset(&th, 0, sizeof(th));
    if (a.mode == MLP_EPI_GELU || a.mode == MLP_EPI_DGELU) {
        // bf16 output [M][N], stored in boxes of 64 columns x 32 rows
        if (!a.h16 || ((uintptr_t)a.h16 & 15) || !make_map(&th, a.h16, a.M, a.N, 32)) return cudaErrorInvalidValue;
    } else {
        // FP32 output [splitk x M][N] (split-K partials stacked) or [M][N],
        // stored in boxes of 32 columns x 32 rows
        const long long rows = (long long)a.M * (a.mode == MLP_EPI_F32 ? splitk : 1);
        if (!a.out32 || ((uintptr_t)a.out32 & 15) || !make_map_f32(&th, a.out32, rows, a.N))
            return cudaErrorInvalidValue;
    }
    if ((a.mode == MLP_EPI_BIAS || a.mode == MLP_EPI_GELU) && (!a.bias || ((uintptr_t)a.bias & 15)))
        return cudaErrorInvalidValue;
    if (a.mode == MLP_EPI_DGELU && (!a.zs || ((uintptr_t)a.zs & 15))) return cudaErrorInvalidValue;
    MlpGemmArgs g = a;
    g.kchunk = a.K / splitk;
    g.stages = mlp_stages(a.bn);
    const size_t smem = bt_mlp_gemm_smem(a.bn);
    static int attr_set = 0;
    if (!attr_set) {
        const int lim = (int)(bt_mlp_gemm_smem(256) > bt_mlp_gemm_smem(128) ? bt_mlp_gemm_smem(256)
                                                                              : bt_mlp_gemm_smem(128));
        cudaError_t e = cudaFuncSetAttribute(k_mlp_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        if (e != cudaSuccess) return e;
        attr_set = 1;
    }
    const int grid = (int)(ntiles < sms ? ntiles : sms);
    k_mlp_gemm<<<grid, MLP_THREADS, smem, stream>>>(ta, tb, th, g);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Training and inference helpers
// ---------------------------------------------------------------------------

// FP32 features [rows][cols] -> bf16 [rows_out][ld_out] and its transpose,
// zero-padded.
__global__ void k_mlp_pack(const float* __restrict__ x, int rows, int cols, int ld_out, int rows_out,
                           __nv_bfloat16* __restrict__ out, __nv_bfloat16* __restrict__ out_t) {
    const long long n = (long long)rows_out * ld_out;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(e / ld_out), c = (int)(e - (long long)r * ld_out);
        const float v = (r < rows && c < cols) ? x[(size_t)r * cols + c] : 0.f;
        const __nv_bfloat16 b = __float2bfloat16_rn(v);
        out[e] = b;
        if (out_t) out_t[(size_t)c * rows_out + r] = b;
    }
}

// Both forms through a shared 32 x 32 tile (threads 32 columns x 8 rows):
// rows of out and of out_t leave as 64-byte runs.
__global__ void __launch_bounds__(256) k_mlp_pack_t(const float* __restrict__ x, int rows, int cols, int ld_out,
                                                    int rows_out, __nv_bfloat16* __restrict__ out,
                                                    __nv_bfloat16* __restrict__ out_t) {
    __shared__ __nv_bfloat16 tile[32][34];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int tilesc = (ld_out + 31) / 32;
    const int r0 = (blockIdx.x / tilesc) * 32, c0 = (blockIdx.x % tilesc) * 32;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int r = r0 + ty + 8 * k, c = c0 + tx;
        if (r < rows_out && c < ld_out) {
            const float v = (r < rows && c < cols) ? x[(size_t)r * cols + c] : 0.f;
            const __nv_bfloat16 b = __float2bfloat16_rn(v);
            out[(size_t)r * ld_out + c] = b;
            tile[ty + 8 * k][tx] = b;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int c = c0 + ty + 8 * k, r = r0 + tx;
        if (r < rows_out && c < ld_out) out_t[(size_t)c * rows_out + r] = tile[tx][ty + 8 * k];
    }
}

// Row-major form only (no transposed copy), 8 columns per thread and one
// 16-byte store; needs ld_out % 8 == 0, a 16-byte aligned `out` and
// rows_out * ld_out / 8 < 2^31.
__global__ void k_mlp_pack8(const float* __restrict__ x, int rows, int cols, int cpr, int nchunk,
                            __nv_bfloat16* __restrict__ out) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nchunk; e += gridDim.x * blockDim.x) {
        const int r = e / cpr, c0 = (e - r * cpr) * 8;
        __align__(16) __nv_bfloat162 b[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int c = c0 + 2 * k;
            const float v0 = (r < rows && c < cols) ? x[(size_t)r * cols + c] : 0.f;
            const float v1 = (r < rows && c + 1 < cols) ? x[(size_t)r * cols + c + 1] : 0.f;
            b[k] = __floats2bfloat162_rn(v0, v1);
        }
        *reinterpret_cast<uint4*>(out + (size_t)e * 8) = *reinterpret_cast<const uint4*>(b);
    }
}

// Gradient of the weighted mean-squared error of columns [0, ncols) and of
// the error head (column err_col, which predicts the log of the row's
// residual norm sqrt(sum_j r_j^2), a detached target).  A block takes 32
// rows: each warp 4 rows with lanes over the columns (coalesced dz rows),
// the gradients staged in shared memory so that the transposed copy dzt
// leaves as 64-byte runs of 32 consecutive rows.  Needs ld_out <= 128.
#define MLP_LOSS_ROWS 32
__global__ void __launch_bounds__(256) k_mlp_loss(const float* __restrict__ y, int ldy, const float* __restrict__ t,
                                                  const float* __restrict__ wt, int rows, int rows_valid, int ncols,
                                                  int err_col, float err_weight, int ld_out,
                                                  __nv_bfloat16* __restrict__ dz, __nv_bfloat16* __restrict__ dzt,
                                                  float* loss) {
    __shared__ float g_s[MLP_LOSS_ROWS][129];
    __shared__ float s_main[8], s_err[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int m0 = blockIdx.x * MLP_LOSS_ROWS;
    const float scale = 2.0f / (float)rows_valid;
    float lm = 0.f, le = 0.f;
    for (int q = 0; q < MLP_LOSS_ROWS / 8; q++) {
        const int rr = warp * (MLP_LOSS_ROWS / 8) + q, m = m0 + rr;
        if (m >= rows) break;
        const bool valid = m < rows_valid;
        float ss = 0.f;
        for (int j = lane; j < ld_out; j += 32) {
            float g = 0.f;
            if (valid && j < ncols) {
                const float r = y[(size_t)m * ldy + j] - t[(size_t)m * ncols + j];
                const float w = wt ? wt[j] : 1.0f;
                ss += r * r;
                lm += w * r * r;
                g = scale * w * r;
            }
            g_s[rr][j] = g;
        }
        __syncwarp();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
        if (err_col >= 0 && lane == 0) {
            float g = 0.f;
            if (valid) {
                const float target = 0.5f * __logf(ss + 1e-12f);
                const float r = y[(size_t)m * ldy + err_col] - target;
                le += r * r;
                g = scale * err_weight * r;
            }
            g_s[rr][err_col] = g;
        }
        __syncwarp();
        for (int j = lane; j < ld_out; j += 32) dz[(size_t)m * ld_out + j] = __float2bfloat16_rn(g_s[rr][j]);
    }
    __syncthreads();
    // transposed copy: thread (j, r) with r fastest
    for (int e = threadIdx.x; e < ld_out * MLP_LOSS_ROWS; e += blockDim.x) {
        const int j = e / MLP_LOSS_ROWS, rr = e - j * MLP_LOSS_ROWS, m = m0 + rr;
        if (m < rows) dzt[(size_t)j * rows + m] = __float2bfloat16_rn(g_s[rr][j]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lm += __shfl_xor_sync(0xffffffffu, lm, o);
        le += __shfl_xor_sync(0xffffffffu, le, o);
    }
    if (lane == 0) {
        s_main[warp] = lm;
        s_err[warp] = le;
    }
    __syncthreads();
    if (threadIdx.x == 0 && loss) {
        float a = 0.f, b = 0.f;
        for (int w = 0; w < 8; w++) {
            a += s_main[w];
            b += s_err[w];
        }
        atomicAdd(loss, a / (float)rows_valid);
        atomicAdd(loss + 1, b / (float)rows_valid);
    }
}

// out[r] = sum_c xt[r][c]: one block per row; 16-byte loads (8 values)
// when the row is 16-byte aligned and cols % 8 == 0, then warp shuffles.
__global__ void __launch_bounds__(256) k_mlp_colsum(const __nv_bfloat16* __restrict__ xt, int cols,
                                                    float* __restrict__ out) {
    __shared__ float s[8];
    const __nv_bfloat16* row = xt + (size_t)blockIdx.x * cols;
    float acc = 0.f;
    if ((cols & 7) == 0 && (((uintptr_t)row) & 15) == 0) {
        const uint4* r4 = reinterpret_cast<const uint4*>(row);
        for (int c = threadIdx.x; c < cols / 8; c += blockDim.x) {
            const uint4 u = __ldg(r4 + c);
            const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const float2 f = __bfloat1622float2(h[k]);
                acc += f.x + f.y;
            }
        }
    } else {
        for (int c = threadIdx.x; c < cols; c += blockDim.x) acc += __bfloat162float(row[c]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) a += s[w];
        out[blockIdx.x] = a;
    }
}

// Adam step on FP32 master weights from the sum of split-K partial gradients
// (or a direct gradient), then the bf16 copies used by the GEMMs:
// w16 [rows][cols] and, if given, w16t [cols][rows].
// hyper (may be null): {lr, bc1, bc2} read from device memory instead of
// the arguments, so that a captured training step follows a schedule
// computed on the device.
__global__ void k_mlp_adam(const float* __restrict__ partials, int nsplit, const float* __restrict__ gdir,
                           long long n, float* __restrict__ w, float* __restrict__ m, float* __restrict__ v, float lr,
                           float b1, float b2, float eps, float bc1, float bc2, int rows, int cols,
                           __nv_bfloat16* __restrict__ w16, __nv_bfloat16* __restrict__ w16t,
                           const float* __restrict__ hyper) {
    if (hyper) {
        lr = hyper[0];
        bc1 = hyper[1];
        bc2 = hyper[2];
    }
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float g = gdir ? gdir[i] : 0.f;
        for (int s = 0; s < nsplit; s++) g += partials[(size_t)s * n + i];
        const float mi = b1 * m[i] + (1.f - b1) * g;
        const float vi = b2 * v[i] + (1.f - b2) * g * g;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
        w[i] = wi;
        if (w16) {
            const __nv_bfloat16 b = __float2bfloat16_rn(wi);
            w16[i] = b;
            if (w16t) {
                const int r = (int)(i / cols), c = (int)(i - (long long)r * cols);
                w16t[(size_t)c * rows + r] = b;
            }
        }
    }
}

// The same update for a weight matrix with both bf16 copies: a block takes
// 8 rows x 128 columns, each thread 4 consecutive columns of a row with
// 16-byte loads and stores (the split-K partials are the bulk of the
// traffic); the transposed copy goes through a shared tile so that w16t
// rows leave as 32-byte runs.  Needs cols % 4 == 0 and 16-byte aligned
// arrays; each weight's arithmetic is the one of k_mlp_adam.
__global__ void __launch_bounds__(256) k_mlp_adam_t(const float* __restrict__ partials, int nsplit,
                                                    const float* __restrict__ gdir, float* __restrict__ w,
                                                    float* __restrict__ m, float* __restrict__ v, float lr, float b1,
                                                    float b2, float eps, float bc1, float bc2, int rows, int cols,
                                                    __nv_bfloat16* __restrict__ w16, __nv_bfloat16* __restrict__ w16t,
                                                    const float* __restrict__ hyper) {
    __shared__ __nv_bfloat16 tile[8][130];
    if (hyper) {
        lr = hyper[0];
        bc1 = hyper[1];
        bc2 = hyper[2];
    }
    const long long n = (long long)rows * cols;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 4 columns, 8 rows
    const int tilesc = (cols + 127) / 128;
    const int r0 = (blockIdx.x / tilesc) * 8, c0 = (blockIdx.x % tilesc) * 128;
    {
        const int rr = ty, r = r0 + rr, c = c0 + 4 * tx;
        if (r < rows && c < cols) {
            const long long i = (long long)r * cols + c;
            float4 g = gdir ? *reinterpret_cast<const float4*>(gdir + i) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
            for (int s = 0; s < nsplit; s++) {
                const float4 p = __ldcs(reinterpret_cast<const float4*>(partials + (size_t)s * n + i));
                g.x += p.x;
                g.y += p.y;
                g.z += p.z;
                g.w += p.w;
            }
            float4 mv = *reinterpret_cast<float4*>(m + i), vv = *reinterpret_cast<float4*>(v + i),
                   wv = *reinterpret_cast<float4*>(w + i);
            float* gp = &g.x;
            float* mp = &mv.x;
            float* vp = &vv.x;
            float* wp = &wv.x;
            __align__(8) __nv_bfloat16 b[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float mi = b1 * mp[q] + (1.f - b1) * gp[q];
                const float vi = b2 * vp[q] + (1.f - b2) * gp[q] * gp[q];
                mp[q] = mi;
                vp[q] = vi;
                wp[q] = wp[q] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
                b[q] = __float2bfloat16_rn(wp[q]);
                tile[rr][4 * tx + q] = b[q];
            }
            *reinterpret_cast<float4*>(m + i) = mv;
            *reinterpret_cast<float4*>(v + i) = vv;
            *reinterpret_cast<float4*>(w + i) = wv;
            *reinterpret_cast<uint2*>(w16 + i) = *reinterpret_cast<const uint2*>(b);
        }
    }
    __syncthreads();
    // transposed copy: 128 columns x 8 rows, thread c < 128 writes column c's
    // 8 rows, one 16-byte store when they are whole and aligned
    const bool vec = (rows % 8 == 0) && ((((uintptr_t)w16t) & 15) == 0);
    for (int cc = threadIdx.x; cc < 128; cc += blockDim.x) {
        const int c = c0 + cc;
        if (c >= cols) continue;
        if (vec && r0 + 8 <= rows) {
            __align__(16) __nv_bfloat16 b[8];
#pragma unroll
            for (int q = 0; q < 8; q++) b[q] = tile[q][cc];
            *reinterpret_cast<uint4*>(w16t + (size_t)c * rows + r0) = *reinterpret_cast<const uint4*>(b);
        } else {
            for (int q = 0; q < 8; q++) {
                const int r = r0 + q;
                if (r < rows) w16t[(size_t)c * rows + r] = tile[q][cc];
            }
        }
    }
}

// Start of a captured training step: rows perm[k * batch + b] of x_all and
// t_all gathered into the step's minibatch (k = *k_in_epoch).
__global__ void k_mlp_gather(const long long* __restrict__ perm, const long long* __restrict__ k_in_epoch,
                             const float* __restrict__ x_all, int nxc, const float* __restrict__ t_all, int ntc,
                             int batch, float* __restrict__ xb, float* __restrict__ tb) {
    const long long k = *k_in_epoch;
    const int w = nxc + ntc;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)batch * w;
         e += (long long)gridDim.x * blockDim.x) {
        const int b = (int)(e / w), c = (int)(e - (long long)b * w);
        const long long src = perm[k * batch + b];
        if (c < nxc) xb[(size_t)b * nxc + c] = x_all[(size_t)src * nxc + c];
        else tb[(size_t)b * ntc + (c - nxc)] = t_all[(size_t)src * ntc + (c - nxc)];
    }
}

// hyper = table[step] ({lr, bc1, bc2} of the step, computed on the host),
// then both step counters advance.  One thread.
__global__ void k_mlp_schedule(long long* __restrict__ k_in_epoch, long long* __restrict__ step,
                               const float* __restrict__ table, long long total, float* __restrict__ hyper) {
    long long g = *step;
    if (g >= total) g = total - 1;
    hyper[0] = table[3 * g];
    hyper[1] = table[3 * g + 1];
    hyper[2] = table[3 * g + 2];
    *step += 1;
    *k_in_epoch += 1;
}

static int mlp_grid(long long n) {
    long long b = (n + 255) / 256;
    long long cap = (long long)bt_sm_count() * 8;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

cudaError_t bt_launch_mlp_pack(const float* x, int rows, int cols, int ld_out, int rows_out, __nv_bfloat16* out,
                               __nv_bfloat16* out_t, cudaStream_t stream) {
    const long long nchunk = (long long)rows_out * ld_out / 8;
    if (!out_t && ld_out % 8 == 0 && ((uintptr_t)out & 15) == 0 && nchunk < (1LL << 31)) {
        k_mlp_pack8<<<mlp_grid(nchunk), 256, 0, stream>>>(x, rows, cols, ld_out / 8, (int)nchunk, out);
        return cudaGetLastError();
    }
    if (out_t) {
        const long long tiles = (long long)((rows_out + 31) / 32) * ((ld_out + 31) / 32);
        if (tiles < (1LL << 31)) {
            k_mlp_pack_t<<<(unsigned)tiles, 256, 0, stream>>>(x, rows, cols, ld_out, rows_out, out, out_t);
            return cudaGetLastError();
        }
    }
    k_mlp_pack<<<mlp_grid((long long)rows_out * ld_out), 256, 0, stream>>>(x, rows, cols, ld_out, rows_out, out, out_t);
    return cudaGetLastError();
}

cudaError_t bt_launch_mlp_loss(const float* y, int ldy, const float* t, const float* wt, int rows, int rows_valid,
                               int ncols, int err_col, float err_weight, int ld_out, __nv_bfloat16* dz,
                               __nv_bfloat16* dzt, float* loss, cudaStream_t stream) {
    if (ld_out > 128 || err_col >= ld_out) return cudaErrorInvalidValue;
    k_mlp_loss<<<(rows + MLP_LOSS_ROWS - 1) / MLP_LOSS_ROWS, 256, 0, stream>>>(y, ldy, t, wt, rows, rows_valid, ncols,
                                                                             err_col, err_weight, ld_out, dz, dzt,
                                                                             loss);
    return cudaGetLastError();
}

cudaError_t bt_launch_mlp_gather(const long long* perm, const long long* k_in_epoch, const float* x_all, int nxc,
                                 const float* t_all, int ntc, int batch, float* xb, float* tb, cudaStream_t stream) {
    if (batch <= 0) return cudaSuccess;
    k_mlp_gather<<<mlp_grid((long long)batch * (nxc + ntc)), 256, 0, stream>>>(perm, k_in_epoch, x_all, nxc, t_all, ntc,
                                                                              batch, xb, tb);
    return cudaGetLastError();
}

cudaError_t bt_launch_mlp_schedule(long long* k_in_epoch, long long* step, const float* table, long long total,
                                   float* hyper, cudaStream_t stream) {
    k_mlp_schedule<<<1, 1, 0, stream>>>(k_in_epoch, step, table, total, hyper);
    return cudaGetLastError();
}

cudaError_t bt_launch_mlp_colsum(const __nv_bfloat16* xt, int rows, int cols, float* out, cudaStream_t stream) {
    k_mlp_colsum<<<rows, 256, 0, stream>>>(xt, cols, out);
    return cudaGetLastError();
}

cudaError_t bt_launch_mlp_adam(const float* partials, int nsplit, const float* grad_direct, long long n, float* w,
                               float* m, float* v, float lr, float b1, float b2, float eps, float bc1, float bc2,
                               int rows, int cols, __nv_bfloat16* w16, __nv_bfloat16* w16t, const float* hyper,
                               cudaStream_t stream) {
    const bool aligned = ((((uintptr_t)partials | (uintptr_t)grad_direct | (uintptr_t)w | (uintptr_t)m |
                            (uintptr_t)v) & 15) == 0) && ((((uintptr_t)w16) & 7) == 0);
    if (w16 && w16t && (long long)rows * cols == n && cols % 4 == 0 && aligned) {
        const long long tiles = (long long)((rows + 7) / 8) * ((cols + 127) / 128);
        k_mlp_adam_t<<<(unsigned)tiles, 256, 0, stream>>>(partials, nsplit, grad_direct, w, m, v, lr, b1, b2, eps, bc1,
                                                         bc2, rows, cols, w16, w16t, hyper);
        return cudaGetLastError();
    }
    k_mlp_adam<<<mlp_grid(n), 256, 0, stream>>>(partials, nsplit, grad_direct, n, w, m, v, lr, b1, b2, eps, bc1, bc2,
                                                rows, cols, w16, w16t, hyper);
    return cudaGetLastError();
}

// Surrogate output: per sample n (group g = grp[n]),
//   lin_j = theta[g][0][j] + sum_k theta[g][1 + k][j] * feat[n][k]   (k < nlin)
//   out[n][0] = 0, out[n][1 + j] = lin_j + y[n][j] * scale / (wl[n] * 1e9)   (waves)
//   err_nm[n] = scale * exp(y[n][err_col])
// FP64 for the linear part, which carries most of the signal.
// Everything on the FP32 pipe: the linear model in float-float (theta as
// hi/lo float pairs; each term's product error recovered with an FMA, the
// sum compensated: ~48-bit accuracy, far below the model's own error), the
// network's residual (a bf16 network's output) converted to waves in FP32
// and added into the float-float sum.  Only the final conversion of each
// coefficient to double uses the FP64 pipe.
__global__ void k_surrogate_combine(const float* __restrict__ feat, int nfeat, int nlin, const int* __restrict__ grp,
                                    const float2* __restrict__ theta, const float* __restrict__ y, int ldy,
                                    const double* __restrict__ wl, float scale, int J, int err_col,
                                    double* __restrict__ out, float* __restrict__ err_nm, int n) {
    const long long total = (long long)n * J;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int s = (int)(e / J), j = (int)(e - (long long)s * J);
        const float2* th = theta + (size_t)grp[s] * (nlin + 1) * J + j;
        float hi = th[0].x, lo = th[0].y;
        const float* f = feat + (size_t)s * nfeat;
        for (int k = 0; k < nlin; k++) {
            const float2 t = th[(size_t)(k + 1) * J];
            const float fk = f[k];
            const float p = t.x * fk;
            const float pe = fmaf(t.y, fk, fmaf(t.x, fk, -p));
            const float sum = hi + p;
            const float bb = sum - hi;
            lo += ((hi - (sum - bb)) + (p - bb)) + pe;
            hi = sum;
        }
        const float r = y[(size_t)s * ldy + j] * (scale / ((float)wl[s] * 1e9f));
        const float sum = hi + r;
        const float bb = sum - hi;
        lo += (hi - (sum - bb)) + (r - bb);
        out[(size_t)s * (J + 1) + 1 + j] = (double)sum + (double)lo;
        if (j == 0) {
            out[(size_t)s * (J + 1)] = 0.0;
            if (err_nm) err_nm[s] = scale * expf(y[(size_t)s * ldy + err_col]);
        }
    }
}

// Vignetting guard: one warp per sample, lanes over the group's kept
// aperture margins k (K a multiple of 32, padding m0 = 3e38).  Predicted
// margin m = m0[g][k] + sum_d jac[g][d][k] z[d] (z: the sample's normalised
// dofs, the first ndof feature columns); the sample is flagged when any m
// has the opposite sign of m0 or |m| < band_abs + band_rel |m - m0|, or
// when some |z[d]| exceeds reach[d] (outside the box the margins were
// chosen for).
__global__ void k_surrogate_guard(const float* __restrict__ feat, int nfeat, int ndof, const int* __restrict__ grp,
                                  const float* __restrict__ m0, const float* __restrict__ jac,
                                  const float* __restrict__ reach, int K, float band_abs, float band_rel,
                                  int* __restrict__ flag, int n) {
    const int lane = threadIdx.x & 31;
    const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long s = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5); s < n; s += nw) {
        const int g = grp[s];
        const float* f = feat + (size_t)s * nfeat;
        bool hit = false;
        if (reach)
            for (int d = lane; d < ndof; d += 32) hit |= !(fabsf(f[d]) <= reach[d]);
        for (int k = lane; k < K; k += 32) {
            const float a = m0[(size_t)g * K + k];
            if (!(a < 1e38f)) continue;
            float m = a;
            const float* j = jac + (size_t)g * ndof * K + k;
            for (int d = 0; d < ndof; d++) m = fmaf(j[(size_t)d * K], f[d], m);
            const float side = (a >= 0.f) ? m : -m;
            hit |= side < band_abs + band_rel * fabsf(m - a);
        }
        const unsigned any = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) flag[s] = any != 0u;
    }
}

cudaError_t bt_launch_surrogate_guard(const float* feat, int nfeat, int ndof, const int* grp, const float* m0,
                                      const float* jac, const float* reach, int K, float band_abs, float band_rel,
                                      int* flag, int n, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    const long long need = ((long long)n + 7) / 8;  // 8 warps (samples) per block
    const int blocks = (int)(need < 152 * 16 ? need : 152 * 16);
    k_surrogate_guard<<<blocks, 256, 0, stream>>>(feat, nfeat, ndof, grp, m0, jac, reach, K, band_abs, band_rel, flag,
                                                  n);
    return cudaGetLastError();
}

cudaError_t bt_launch_surrogate_combine(const float* feat, int nfeat, int nlin, const int* grp, const float* theta,
                                        const float* y, int ldy, const double* wl, double scale, int J, int err_col,
                                        double* out, float* err_nm, int n, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    k_surrogate_combine<<<mlp_grid((long long)n * J), 256, 0, stream>>>(feat, nfeat, nlin, grp,
                                                                         reinterpret_cast<const float2*>(theta), y, ldy, wl,
                                                                         (float)scale, J, err_col, out, err_nm, n);
    return cudaGetLastError();
}
