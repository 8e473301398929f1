// Internal interface of the batched wavefront / Zernike-fit kernel (batch.cu).
#pragma once
#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime.h>

#define BT_BATCH_MAX_THREADS 256
// resident blocks per SM the register budget is sized for (128 registers)
#define BT_BATCH_MIN_BLOCKS 2
#define BT_BATCH_MAX_J 32
#define BT_BATCH_MAX_VAR 8
#define BT_BATCH_MAX_NX 512
#define BT_BATCH_MAX_SMEM (227 * 1024)
// most resident blocks per SM the OPD scratch is sized for
#define BT_BATCH_MAX_CTAS_PER_SM 8
// A Cholesky pivot at or below this fraction of the largest diagonal entry
// of B^T B marks the fit rank-deficient.
#define BT_BATCH_PIVOT_TOL 1e-12
// per-job status values (-1: not processed)
#define BT_BATCH_BAD_NX 1  // BT_ERR_ARG: no fit tables for this grid size
#define BT_BATCH_RANK 4    // BT_ERR_RANK

struct BatchArgs {
    // per state s
    const double* xf;     // [S][nvar][12]: dr(3), drot(9) of each varying stage
    const double* det;    // [S][12]: origin(3), rot(9, row-major) of the last stage's frame
    const double* amps;   // [S][nmodes]
    const int* nxs;       // [S] pupil grid size
    const double* wl;     // [S] wavelength
    // per field f: back-propagation frame dr(3), rot(9); local and global velocity
    const double* field;  // [F][18]
    // fit tables
    const double* basis;          // per grid size: [jmax][nx*nx]
    const long long* basis_off;   // [nx_cap + 1], -1 where absent
    const double* gref;           // [nx_cap + 1][jmax][jmax]
    // schedule and outputs
    double* scratch;        // OPD of every ray of a job: one row per block, or per queue entry when split
    long long scratch_stride;  // doubles per row (>= the largest nx * nx)
    const int* order;   // [njobs] job ids (s * nfields + f) in scheduling order
    int* counter;       // queue head (work items), zeroed before each launch
    int* jobcnt;        // [nqueue] finished chunks per job when split, zeroed before each launch
    int nchunk;         // blocks sharing one job's rays (1: a job per block)
    double* coefs;      // [njobs][jmax + 1]
    int* status;        // [njobs]
    int njobs;          // nstates * nfields (status / coefs extent)
    int nqueue;         // entries of order to run
    int nfields;
    int nx_cap;
    // plan
    int nvar;
    int var_stage[BT_BATCH_MAX_VAR];
    int ntrace;         // optic stages; stage ntrace is the reference-sphere stage
    int modal_surf;     // MODAL surface record, -1 for none
    int nmodes;
    double stop_dr[3];  // transform from the (flat) stop surface's frame to the optic's
    double stop_drot[9];
    double sphere_R;
    double pupil;
    double r_in2;
    double r_out2;
    int jmax;
    int niter;
};

struct BatchSmem {
    size_t mc, gcorr, zv, G, bv, mcf, mcell, total;
};

__host__ __device__ inline BatchSmem bt_batch_smem_layout(int blob_bytes, int T, int J) {
    BatchSmem L;
    size_t off = ((size_t)blob_bytes + 127) & ~(size_t)127;
    // the MODAL corner cache (ray phase) and the per-warp Gram corrections
    // (fit phase) share one region
    L.mc = off;
    L.gcorr = off;
    {
        const size_t a = (size_t)16 * T * sizeof(double), b = (size_t)(T / 32) * (J * (J + 1) / 2) * sizeof(double);
        off += a > b ? a : b;
    }
    L.zv = off;
    off += (size_t)(T / 32) * 32 * sizeof(double);
    L.G = off;
    off += (size_t)J * J * sizeof(double);
    L.bv = off;
    off += 32 * sizeof(double);
    L.mcf = off;
    off += (size_t)16 * T * sizeof(float);
    L.mcell = off;
    off += (size_t)T * sizeof(int);
    L.total = (off + 15) & ~(size_t)15;
    return L;
}

cudaError_t bt_batch_set_smem_limit();
int bt_batch_smem_max();
cudaError_t bt_launch_batch_zernike(const unsigned char* d_blob, int blob_bytes, const BatchArgs& a, int threads,
                                    int ctas_per_sm, cudaStream_t stream);
cudaError_t bt_launch_batch_tables(int nx, double pupil, const double* cart, int jmax, int side, double* out,
                                   cudaStream_t stream);
cudaError_t bt_launch_batch_gref(const int* d_nx_list, int n, double pupil, double r_in2, double r_out2,
                                 const double* basis, const long long* basis_off, int jmax, double* gref,
                                 cudaStream_t stream);
cudaError_t bt_read_batch_device_status(int* status, cudaStream_t stream);
