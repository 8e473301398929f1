// Internal declarations shared by the C-ABI translation unit and the kernel
// translation units.  Not part of the public interface.
#pragma once
#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime.h>
#include "bt_desc.h"

#define BT_MAX_STAGES 64

// Device view of a ray bundle (same fields as bt_rayvector).
struct RV {
    double* x;
    double* y;
    double* z;
    double* vx;
    double* vy;
    double* vz;
    double* t;
    double* w;
    double* f;
    uint8_t* vig;
    uint8_t* fail;
    long long n;
};

struct SnapSet {
    RV s[BT_MAX_STAGES];
};

// Status word written by kernels whose bounded waits expire (0 = fine).
// Read and cleared by bt_check_device_status().
cudaError_t bt_read_device_status(int* status, cudaStream_t stream);
cudaError_t bt_read_split_device_status(int* status, cudaStream_t stream);
cudaError_t bt_read_trace_ff_device_status(int* status, cudaStream_t stream);
long long bt_trace_ff_round_rays();

// trace_ff.cu: the float-float form of the fused trace
cudaError_t bt_launch_trace_ff(const unsigned char* d_blob, int blob_bytes, const RV& in, const RV& out,
                               const SnapSet* snaps, int nsnaps, int niter, cudaStream_t stream);

// trace.cu
cudaError_t bt_launch_trace(const unsigned char* d_blob, int blob_bytes, const RV& in, const RV& out,
                            const SnapSet* snaps, int nsnaps, int niter, cudaStream_t stream);
cudaError_t bt_launch_surface_eval(const unsigned char* d_blob, int blob_bytes, const double* x,
                                   const double* y, double* sag, double* normal, long long n,
                                   cudaStream_t stream);
cudaError_t bt_launch_getN(const unsigned char* d_blob, int blob_bytes, const double* w, double* out,
                           long long n, cudaStream_t stream);
cudaError_t bt_launch_rsplit(const unsigned char* d_blob, int blob_bytes, const RV& rv, const RV& sp, int niter,
                             cudaStream_t stream);
cudaError_t bt_launch_obsc(const unsigned char* d_blob, int blob_bytes, const double* x, const double* y,
                           uint8_t* out, const RV* rv, long long n, cudaStream_t stream);

// rayvec.cu
cudaError_t bt_launch_transform_rv(const double dr[3], const double drot[9], const RV& rv, bool forward,
                                   cudaStream_t stream);
cudaError_t bt_launch_transform_arrays(const double dr[3], const double drot[9], double* x, double* y,
                                       double* z, long long n, bool forward, cudaStream_t stream);
cudaError_t bt_launch_finish_parallel(const double dr[3], const double drot[9], const double vv[3],
                                      double* x, double* y, double* z, long long n, cudaStream_t stream);
cudaError_t bt_launch_stop_grid(int nx, int ny, double valx, double valy, const double lx[2], const double ly[2],
                                double* x, double* y, cudaStream_t stream);
cudaError_t bt_launch_stop_rings(int nring, const double* r, const double* step, const long long* off, long long n,
                                 double* x, double* y, cudaStream_t stream);
cudaError_t bt_launch_stop_spokes(const double* rings, int nr, const double* spokes, int ns, double* x, double* y,
                                  cudaStream_t stream);
cudaError_t bt_launch_position_at_time(const RV& rv, double t, double* xo, double* yo, double* zo,
                                       cudaStream_t stream);
cudaError_t bt_launch_propagate(const RV& rv, double t, cudaStream_t stream);
cudaError_t bt_launch_phase(const RV& rv, double x, double y, double z, double t, double* out,
                            bool amplitude, cudaStream_t stream);
cudaError_t bt_launch_sum_amplitude(const RV& rv, double x, double y, double z, double t, bool ignore_vig,
                                    double* d_out2, cudaStream_t stream);
cudaError_t bt_launch_rv_equal(const RV& a, const RV& b, int* d_flag, cudaStream_t stream);
cudaError_t bt_launch_dfma_probe(int iters, double* sink, float* ms, double* flops, cudaStream_t stream);
cudaError_t bt_launch_ffma_probe(int iters, double* sink, float* ms, double* flops, cudaStream_t stream);

// huygens.cu
cudaError_t bt_launch_huygens(const RV& rv, double px, double py, double pz, const double lat[4], int na,
                              int nb, double t0, bool ignore_vig, double* out_re, double* out_im,
                              cudaStream_t stream);

cudaError_t bt_launch_huygens_fields(const RV& rv, long long per_field, int nfields, const double* px,
                                     const double* py, const double* pz, const double* lat, const double* t0,
                                     int ps, int na, int nb, bool ignore_vig, double* out_re, double* out_im,
                                     cudaStream_t stream);
// huygens.cu, allocation-free variant (file-scope device scratch)
cudaError_t bt_launch_huygens_noalloc(const RV& rv, double px, double py, double pz, const double lat[4], int na,
                                      int nb, double t0, bool ignore_vig, double* out_re, double* out_im,
                                      cudaStream_t stream, size_t* needed);

// fit.cu
cudaError_t bt_launch_zk_normal(const double* x, const double* y, const double* v, const long long* offsets,
                                int nfits, const double* basis, int jmax, int side, double* G, double* b,
                                cudaStream_t stream);

int bt_sm_count();
int bt_grid_for(long long n, int threads, int per_sm);  // ceil(n / threads), at most per_sm per SM
void bt_keep_pool();  // keep the default pool's freed scratch cached (once per process)
