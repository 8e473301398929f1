// Internal interface of the surrogate MLP kernels (mlp.cu).
#pragma once
#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>

enum {
    MLP_EPI_F32 = 0,    // out32[kz][m][n] = acc (split-K partials)
    MLP_EPI_BIAS = 1,   // out32[m][n] = acc + bias[n]
    MLP_EPI_GELU = 2,   // zs = acc + bias, h16 = h16t^T = bf16(gelu(zs))
    MLP_EPI_DGELU = 3   // h16 = h16t^T = bf16(acc * gelu'(zs))
};

struct MlpGemmArgs {
    int M, N, K;        // C[M x N] = A[M x K] . B[N x K]^T
    int bn;             // tile width, 128 or 256
    int kchunk;         // K per split (set by the launcher)
    int stages;         // operand ring depth (set by the launcher)
    int mode;
    const float* bias;  // [N]
    float* out32;       // F32: [splitk][M][N]; BIAS: [M][N]
    float* zs;          // GELU: written [M][N] (may be null); DGELU: read
    __nv_bfloat16* h16;   // [M][N]
    __nv_bfloat16* h16t;  // [N][M] (may be null)
};

size_t bt_mlp_gemm_smem(int bn);
cudaError_t bt_launch_mlp_gemm(const __nv_bfloat16* A, const __nv_bfloat16* B, const MlpGemmArgs& a, int splitk,
                               cudaStream_t stream);
cudaError_t bt_launch_mlp_pack(const float* x, int rows, int cols, int ld_out, int rows_out, __nv_bfloat16* out,
                               __nv_bfloat16* out_t, cudaStream_t stream);
cudaError_t bt_launch_mlp_loss(const float* y, int ldy, const float* t, const float* wt, int rows, int rows_valid,
                               int ncols, int err_col, float err_weight, int ld_out, __nv_bfloat16* dz,
                               __nv_bfloat16* dzt, float* loss, cudaStream_t stream);
cudaError_t bt_launch_mlp_colsum(const __nv_bfloat16* xt, int rows, int cols, float* out, cudaStream_t stream);
cudaError_t bt_launch_mlp_adam(const float* partials, int nsplit, const float* grad_direct, long long n, float* w,
                               float* m, float* v, float lr, float b1, float b2, float eps, float bc1, float bc2,
                               int rows, int cols, __nv_bfloat16* w16, __nv_bfloat16* w16t, const float* hyper,
                               cudaStream_t stream);
cudaError_t bt_launch_surrogate_combine(const float* feat, int nfeat, int nlin, const int* grp, const float* theta,
                                        const float* y, int ldy, const double* wl, double scale, int J, int err_col,
                                        double* out, float* err_nm, int n, cudaStream_t stream);
cudaError_t bt_launch_mlp_gather(const long long* perm, const long long* k_in_epoch, const float* x_all, int nxc,
                                 const float* t_all, int ntc, int batch, float* xb, float* tb, cudaStream_t stream);
cudaError_t bt_launch_mlp_schedule(long long* k_in_epoch, long long* step, const float* table, long long total,
                                   float* hyper, cudaStream_t stream);
cudaError_t bt_launch_surrogate_guard(const float* feat, int nfeat, int ndof, const int* grp, const float* m0,
                                      const float* jac, const float* reach, int K, float band_abs, float band_rel,
                                      int* flag, int n, cudaStream_t stream);
cudaError_t bt_read_mlp_device_status(int* status, cudaStream_t stream);
