// Batched wavefronts and annular-Zernike fits of many perturbed states of one
// telescope, in one persistent launch.
//
// A job is one (state, field) pair and reproduces, for that state's optic,
// batoid.zernike (batoid/analysis.py:479-573) built on batoid.wavefront
// (batoid/analysis.py:308-388):
//   * rays on the square pupil grid of RayVector.asGrid
//     (batoid/rayVector.py:220-444, _finish 817-858, finishParallel
//     src/batoid.cpp:40-69), generated in registers from the grid index;
//   * the sequential trace through the state's optic (the fused stage loop
//     shared with the plain trace kernel);
//   * reference = 'chief': the grid's centre ray fixes the reference point;
//     every ray moves into the frame shifted by point + (0, 0, R) and is
//     intersected with Sphere(-R); OPD = (t_chief - t) / wavelength;
//   * the least-squares fit of the annular Zernike basis to the OPD of the
//     non-vignetted rays, solved here by Cholesky of the normal equations.
//
// Per-job state lives in the block's shared memory: the staged program is
// patched with the state's stage transforms and bending amplitudes before
// the job's rays run.  Blocks pull jobs from an atomic queue (longest jobs
// first when the host orders them so), so uneven pupil grids balance.
//
// Normal equations: the Gram matrix over the non-vignetted grid points is
// G = G_ref(nx) + sum over points valid but outside the reference annulus
// - sum over points inside it but vignetted, with G_ref(nx) the Gram matrix
// of all grid points inside the fit annulus (built once per grid size).  Only
// the (few) rays whose vignetting differs from the annulus test update G;
// every valid ray adds its OPD times its basis row to B^T v.
#include <cuda_runtime.h>
#include "bt_internal.h"
#include "bt_device.cuh"
#include "bt_stage_smem.cuh"
#include "bt_trace_core.cuh"
#include "bt_trace_ff.cuh"
#include "bt_batch.h"

cudaError_t bt_read_batch_device_status(int* status, cudaStream_t stream) {
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

// Grid point i of an nx x nx pupil grid of side `pupil`:
// fftshift(fftfreq(nx, d)) with d = (nx-2)/nx (even) or (nx-1)/nx (odd),
// scaled by the pupil size (batoid/rayVector.py:404-437).  Unfused products
// keep the values identical to the host construction.
__device__ __forceinline__ void bt_grid_point(int nx, int i, double pupil, double* x, double* y) {
    const int iy = i / nx, ix = i - iy * nx;
    const double d = (nx <= 2) ? 1.0 : (double)(nx - ((nx % 2 == 0) ? 2 : 1)) / (double)nx;
    const double val = 1.0 / ((double)nx * d);
    const int h = nx / 2;
    *x = __dmul_rn(pupil, __dmul_rn((double)(ix - h), val));
    *y = __dmul_rn(pupil, __dmul_rn((double)(iy - h), val));
}

__device__ __forceinline__ bool bt_in_annulus(double x, double y, double r_in2, double r_out2) {
    const double r2 = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
    return r2 >= r_in2 && r2 <= r_out2;
}

// Ray i of a job: point of the (flat) stop surface, transform into the
// optic's frame, back-propagation onto the plane through the field frame's
// origin (batoid/rayVector.py:817-846; src/batoid.cpp:8-69).
__device__ __forceinline__ void bt_batch_ray(const BatchArgs& A, const double* F, int nx, int i, double wl,
                                             RayState& r, double* gx, double* gy) {
    double x, y;
    bt_grid_point(nx, i, A.pupil, &x, &y);
    *gx = x;
    *gy = y;
    double z = 0.0;
    {
        const double* dr = A.stop_dr;
        const double* m = A.stop_drot;
        const double dx = x - dr[0], dy = y - dr[1], dz = z - dr[2];
        x = dx * m[0] + dy * m[3] + dz * m[6];
        y = dx * m[1] + dy * m[4] + dz * m[7];
        z = dx * m[2] + dy * m[5] + dz * m[8];
    }
    {
        // F: dr(3) rot(9) v_local(3) v(3)
        const double* f = F + 3;
        const double dx = x - F[0], dy = y - F[1], dz = z - F[2];
        double lx = dx * f[0] + dy * f[3] + dz * f[6];
        double ly = dx * f[1] + dy * f[4] + dz * f[7];
        double lz = dx * f[2] + dy * f[5] + dz * f[8];
        const double dt = -lz / F[14];
        lx += dt * F[12];
        ly += dt * F[13];
        lz += dt * F[14];
        r.x = lx * f[0] + ly * f[1] + lz * f[2] + F[0];
        r.y = lx * f[3] + ly * f[4] + lz * f[5] + F[1];
        r.z = lx * f[6] + ly * f[7] + lz * f[8] + F[2];
    }
    r.vx = F[15];
    r.vy = F[16];
    r.vz = F[17];
    r.t = 0.0;
    r.w = wl;
    r.f = 1.0;
    r.vig = false;
    r.fail = false;
}

// Reference-sphere frame of a job from its traced chief ray: the state's
// detector frame shifted locally by point + (0, 0, R) (CoordSys.shiftLocal,
// batoid/coordSys.py), expressed as the transform from the detector frame
// (CoordTransform: dr = R^T (o' - o), drot = R^T R).
__device__ __noinline__ void bt_batch_target(const BatchArgs& A, int s, const RayState& r, bt_stage& sph) {
    const double* D = A.det + (size_t)s * 12;
    const double* R = D + 3;  // row-major
    const double qv[3] = {r.x, r.y, r.z + A.sphere_R};
    double d[3];
    for (int i = 0; i < 3; i++) {
        const double o2 = D[i] + (R[3 * i] * qv[0] + R[3 * i + 1] * qv[1] + R[3 * i + 2] * qv[2]);
        d[i] = o2 - D[i];
    }
    for (int i = 0; i < 3; i++) {
        sph.dr[i] = R[i] * d[0] + R[3 + i] * d[1] + R[6 + i] * d[2];
        for (int j = 0; j < 3; j++) sph.drot[3 * i + j] = R[i] * R[j] + R[3 + i] * R[3 + j] + R[6 + i] * R[6 + j];
    }
    sph.identity = 0;
}

// The reference-sphere stage: transform into the sphere's frame, intersect
// the Sphere(-R) surface (src/sphere.cpp root choice), propagate; a miss
// fails and vignettes the ray (src/batoid.cpp:175-270 with a sphere).
__device__ __forceinline__ void bt_sphere_stage(const Prog& P, const bt_stage& st, RayState& r) {
    if (r.fail) return;
    const double dx = r.x - st.dr[0], dy = r.y - st.dr[1], dz = r.z - st.dr[2];
    double x = dx * st.drot[0] + dy * st.drot[3] + dz * st.drot[6];
    double y = dx * st.drot[1] + dy * st.drot[4] + dz * st.drot[7];
    double z = dx * st.drot[2] + dy * st.drot[5] + dz * st.drot[8];
    const double vx = r.vx * st.drot[0] + r.vy * st.drot[3] + r.vz * st.drot[6];
    const double vy = r.vx * st.drot[1] + r.vy * st.drot[4] + r.vz * st.drot[7];
    const double vz = r.vx * st.drot[2] + r.vy * st.drot[5] + r.vz * st.drot[8];
    const bt_surf& sp = P.surfs[st.surf];
    const double R = sp.p[0];
    const double z0 = z - R;
    const double a = vz * vz + (vx * vx + vy * vy);
    const double b = 2 * vz * z0 + 2 * (vx * x + vy * y);
    const double c = z0 * z0 - sp.p[1] + (x * x + y * y);
    const bool want_max = (vz * R < 0);
    double dt;
    if (!bt_one_root(a, b, c, want_max == (a > 0), &dt)) {
        r.fail = true;
        r.vig = true;
        return;
    }
    r.x = x + vx * dt;
    r.y = y + vy * dt;
    r.z = z + vz * dt;
    r.vx = vx;
    r.vy = vy;
    r.vz = vz;
    r.t += dt;
}

__device__ __forceinline__ double bt_warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// (a, b), b <= a, of packed lower-triangle index e = a (a + 1) / 2 + b.
__device__ __forceinline__ void bt_tri_index(int e, int* a, int* b) {
    int aa = 0, bb = e;
    while (bb > aa) {
        bb -= aa + 1;
        aa++;
    }
    *a = aa;
    *b = bb;
}

// gw += sign * z z^T on the packed lower triangle, lanes striding over the
// entries (one vignetting mismatch; out of line, it is rare).
__device__ __noinline__ void bt_gram_update(double* gw, const double* zv, double sign, int lane, int NT) {
    int a, b;
    bt_tri_index(lane, &a, &b);
    for (int e = lane; e < NT; e += 32) {
        gw[e] += sign * (zv[a] * zv[b]);
        b += 32;
        while (b > a) {
            b -= a + 1;
            a++;
        }
    }
}

// Cholesky G = L L^T in place (lower triangle; lanes = rows) and the two
// triangular solves of G c = bv by one warp.  Writes out[0] = 0 and
// out[1..J], or NaN and the rank status when a pivot falls below
// BT_BATCH_PIVOT_TOL of the largest diagonal entry.
__device__ __noinline__ void bt_chol_solve(double* G, const double* bv, int J, int lane, double* out, int* status) {
    double maxd = 0.0;
    for (int j = 0; j < J; j++) maxd = fmax(maxd, G[j * J + j]);
    const double tol = maxd * BT_BATCH_PIVOT_TOL;
    bool ok = true;
    for (int k = 0; k < J; k++) {
        __syncwarp();
        const double dkk = G[k * J + k];
        if (!(dkk > tol)) {
            ok = false;
            break;
        }
        const double l = sqrt(dkk);
        __syncwarp();
        if (lane > k && lane < J) G[lane * J + k] /= l;
        __syncwarp();
        if (lane == k) G[k * J + k] = l;
        if (lane > k && lane < J) {
            const double lik = G[lane * J + k];
            for (int j = k + 1; j <= lane; j++) G[lane * J + j] -= lik * G[j * J + k];
        }
    }
    __syncwarp();
    if (ok) {
        double x = (lane < J) ? bv[lane] : 0.0;
        for (int k = 0; k < J; k++) {
            const double yk = __shfl_sync(0xffffffffu, x, k) / G[k * J + k];
            if (lane == k) x = yk;
            else if (lane > k && lane < J) x -= G[lane * J + k] * yk;
        }
        for (int k = J - 1; k >= 0; k--) {
            const double ck = __shfl_sync(0xffffffffu, x, k) / G[k * J + k];
            if (lane == k) x = ck;
            else if (lane < k) x -= G[k * J + lane] * ck;
        }
        if (lane < J) out[1 + lane] = x;
        if (lane == 0) {
            out[0] = 0.0;
            *status = 0;
        }
    } else {
        for (int j = lane; j <= J; j += 32) out[j] = NAN;
        if (lane == 0) *status = BT_BATCH_RANK;
    }
}

// The FP64 form of a stage (Newton capped below 3 iterations), out of line.
static __device__ __noinline__ void bt_batch_stage_fp64(const Prog& P, const bt_stage& st, RayState& r, int niter,
                                                        int& cm, double& cn, double& cin) {
    run_stage<true>(P, st, r, niter, cm, cn, cin);
}

__global__ void __launch_bounds__(BT_BATCH_MAX_THREADS, BT_BATCH_MIN_BLOCKS)
k_batch_zernike(const unsigned char* __restrict__ gblob, int blob_bytes, const __grid_constant__ BatchArgs A) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ int s_q;
    __shared__ double s_t0;
    if (!bt_stage_blob(smem, gblob, blob_bytes, &bar)) return;
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = T >> 5;
    const int J = A.jmax, NT = J * (J + 1) / 2;
    const bt_prog_header* hdr = reinterpret_cast<const bt_prog_header*>(smem);
    bt_stage* stages = reinterpret_cast<bt_stage*>(smem + hdr->off_stages);
    double* pool = reinterpret_cast<double*>(smem + hdr->off_pool);
    BatchSmem L = bt_batch_smem_layout(blob_bytes, T, J);
    double* mc = reinterpret_cast<double*>(smem + L.mc);
    __shared__ int s_last;
    const int nchunk = A.nchunk;
    double* gcorr = reinterpret_cast<double*>(smem + L.gcorr);
    double* zv = reinterpret_cast<double*>(smem + L.zv) + warp * 32;
    double* G = reinterpret_cast<double*>(smem + L.G);
    double* bv = reinterpret_cast<double*>(smem + L.bv);
    float* mcf = reinterpret_cast<float*>(smem + L.mcf);
    int* mcell = reinterpret_cast<int*>(smem + L.mcell);
    // one copy of the program's pointers per block (the out-of-line
    // helpers take it by reference: no per-thread stack copy)
    __shared__ Prog sP;
    if (tid == 0) {
        sP = prog_from_blob(smem);
        sP.mc = mc;
        sP.mcf = mcf;
        sP.mcell = mcell;
        sP.mstride = T;
    }
    __syncthreads();
    const Prog& P = sP;
    bt_stage& sph = stages[A.ntrace];
    const int modal_off = (A.modal_surf >= 0) ? P.surfs[A.modal_surf].off : 0;
    double* gw = gcorr + warp * NT;

    // work items: (queue entry q, chunk c of its rays); nchunk = 1 gives a
    // whole job per item
    for (;;) {
        if (tid == 0) s_q = atomicAdd(A.counter, 1);
        __syncthreads();
        const int item = s_q;
        if (item >= A.nqueue * nchunk) break;
        const int q = item / nchunk, chunk = item - q * nchunk;
        const int job = A.order[q];
        const int s = job / A.nfields, f = job - s * A.nfields;
        const int nx = A.nxs[s];
        const double wl = A.wl[s];
        const long long boff = (nx >= 1 && nx <= A.nx_cap) ? A.basis_off[nx] : -1;
        if (boff < 0) {
            // grid size without prepared fit tables (reported by chunk 0)
            if (chunk == 0) {
                if (tid == 0) A.status[job] = BT_BATCH_BAD_NX;
                for (int j = tid; j <= J; j += T) A.coefs[(size_t)job * (J + 1) + j] = NAN;
            }
            __syncthreads();
            continue;
        }
        // state's stage transforms and bending amplitudes into the program
        for (int k = tid; k < A.nvar * 12; k += T) {
            const double v = A.xf[(size_t)s * A.nvar * 12 + k];
            bt_stage& st = stages[A.var_stage[k / 12]];
            const int c = k % 12;
            if (c < 3) st.dr[c] = v;
            else st.drot[c - 3] = v;
        }
        if (A.modal_surf >= 0) {
            ff* amp = reinterpret_cast<ff*>(pool + modal_off);
            for (int m = tid; m < A.nmodes; m += T) {
                const double a = A.amps[(size_t)s * A.nmodes + m];
                const float h = __double2float_rn(a);
                amp[m] = ff{h, __double2float_rn(a - (double)h)};
            }
        }
        mcell[tid] = -1;  // the corner cache shares its space with the fit's gcorr
        __syncthreads();

        const double* F = A.field + (size_t)f * 18;
        const int nray = nx * nx;
        const double* Z = A.basis + boff;
        // this job's per-ray OPD (NaN: vignetted): the block's own row, or
        // the queue entry's row shared by the job's chunks
        double* opdbuf = A.scratch + (size_t)(nchunk > 1 ? q : blockIdx.x) * A.scratch_stride;
        // this chunk's rays [r0, r1), whole rounds of T
        const int per = ((nray + nchunk - 1) / nchunk + T - 1) / T * T;
        const int r0 = chunk * per < nray ? chunk * per : nray;
        const int r1 = r0 + per < nray ? r0 + per : nray;
        // chief ray: the grid's centre point (batoid/analysis.py:340-343),
        // traced by thread 0 in a first pass of its own
        const int cridx = (nx % 2 == 0) ? (nx / 2) * nx + nx / 2 : (nx * nx - 1) / 2;
        // (a chunk without rays only counts itself)
        for (int base = (r0 < r1 ? r0 - T : r1); base < r1; base += T) {
            const bool chief = base < r0;
            const int i = chief ? cridx : base + tid;
            const bool active = chief ? (tid == 0) : (i < r1);
            RayState r;
            double gx = 0.0, gy = 0.0;
            int cm = -1;
            double cn = 0.0, cin = 0.0;
            MediumCacheF mcf_;
            mcf_.idx = -1;
            RayCacheF fcache;
            fcache.ok = false;
            if (active) bt_batch_ray(A, F, nx, i, wl, r, &gx, &gy);
            // stage-synchronous: all warps of the block run the same stage's
            // code together (instruction-cache working set of one stage).
            // The float-float form of the stages (as the fused trace) unless
            // Newton is capped below 3 iterations.
            for (int k = 0; k < A.ntrace; k++) {
                if (active) {
                    if (A.niter >= 3) run_stage_ff(P, stages[k], r, A.niter, mcf_, fcache);
                    else bt_batch_stage_fp64(P, stages[k], r, A.niter, cm, cn, cin);
                }
                __syncthreads();
            }
            if (active) {
                if (chief) bt_batch_target(A, s, r, sph);
                bt_sphere_stage(P, sph, r);
            }
            if (chief) {
                if (tid == 0) s_t0 = r.t;
                __syncthreads();  // reference frame and t0 visible to all
                continue;
            }
            if (active) opdbuf[i] = r.vig ? (double)NAN : (s_t0 - r.t) / wl;
        }
        __syncthreads();
        if (nchunk > 1) {
            // the block finishing a job's last chunk fits it: every chunk's
            // OPDs are visible device-wide before its count is
            __threadfence();
            if (tid == 0) s_last = (atomicAdd(A.jobcnt + q, 1) == nchunk - 1);
            __syncthreads();
            if (!s_last) continue;
            __threadfence();
        }
        for (int e = lane; e < NT; e += 32) gw[e] = 0.0;
        // B^T v: warp w sums rows j = w, w + nwarps, ... of Z^T opd, every
        // lane over points i = lane, lane + 32, ... (independent accumulators)
        {
            const int nj = (J - warp + nwarps - 1) / nwarps;  // rows of this warp
            for (int q0 = 0; q0 < nj; q0 += 8) {
                double acc[8];
#pragma unroll
                for (int q = 0; q < 8; q++) acc[q] = 0.0;
                for (int i = lane; i < nray; i += 32) {
                    const double o = __ldcg(opdbuf + i);
                    if (o == o) {
#pragma unroll
                        for (int q = 0; q < 8; q++)
                            if (q0 + q < nj) acc[q] += __ldg(Z + (size_t)(warp + (q0 + q) * nwarps) * nray + i) * o;
                    }
                }
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    if (q0 + q < nj) {
                        const double v = bt_warp_sum(acc[q]);
                        if (lane == 0) bv[warp + (q0 + q) * nwarps] = v;
                    }
                }
            }
        }
        // vignetting that disagrees with the fit annulus corrects G_ref
        for (int base = 0; base < nray; base += T) {
            const int i = base + tid;
            bool valid = false, inref = false;
            if (i < nray) {
                double gx, gy;
                bt_grid_point(nx, i, A.pupil, &gx, &gy);
                const double o = __ldcg(opdbuf + i);
                valid = (o == o);
                inref = bt_in_annulus(gx, gy, A.r_in2, A.r_out2);
            }
            unsigned mm = __ballot_sync(0xffffffffu, valid != inref);
            while (mm) {
                const int src = __ffs(mm) - 1;
                mm &= mm - 1;
                const int pi = __shfl_sync(0xffffffffu, i, src);
                const double sign = __shfl_sync(0xffffffffu, valid ? 1.0 : -1.0, src);
                __syncwarp();
                if (lane < J) zv[lane] = __ldg(Z + (size_t)lane * nray + pi);
                __syncwarp();
                bt_gram_update(gw, zv, sign, lane, NT);
            }
        }
        __syncthreads();
        // B^T B
        const double* GR = A.gref + (size_t)nx * J * J;
        for (int e = tid; e < NT; e += T) {
            int a, b;
            bt_tri_index(e, &a, &b);
            double v = GR[a * J + b];
            for (int w = 0; w < nwarps; w++) v += gcorr[w * NT + e];
            G[a * J + b] = v;
            G[b * J + a] = v;
        }
        __syncthreads();
        if (warp == 0) bt_chol_solve(G, bv, J, lane, A.coefs + (size_t)job * (J + 1), A.status + job);
    }
}

// Basis table of one grid size: Z[j][i] = Z_{j+1}(grid point i), from the
// Cartesian coefficient arrays c[j][a][b] (x^a y^b) by 2-D Horner.
__global__ void k_batch_basis(int nx, double pupil, const double* __restrict__ cart, int jmax, int side,
                              double* __restrict__ out) {
    const int nray = nx * nx;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nray * jmax; e += gridDim.x * blockDim.x) {
        const int j = e / nray, i = e - j * nray;
        double x, y;
        bt_grid_point(nx, i, pupil, &x, &y);
        const double* c = cart + (size_t)j * side * side;
        double r = 0.0;
        for (int a = side - 1; a >= 0; a--) {
            double row = 0.0;
            for (int b = side - 1; b >= 0; b--) row = row * y + c[a * side + b];
            r = r * x + row;
        }
        out[e] = r;
    }
}

// G_ref(nx) = sum over grid points inside the fit annulus of Z Z^T; one block
// per grid size, one thread per packed entry, points in order.
__global__ void k_batch_gref(const int* __restrict__ nx_list, double pupil, double r_in2, double r_out2,
                             const double* __restrict__ basis, const long long* __restrict__ basis_off, int jmax,
                             double* __restrict__ gref) {
    const int nx = nx_list[blockIdx.x];
    const int nray = nx * nx;
    const double* Z = basis + basis_off[nx];
    const int NT = jmax * (jmax + 1) / 2;
    for (int e = threadIdx.x; e < NT; e += blockDim.x) {
        int a, b;
        bt_tri_index(e, &a, &b);
        double acc = 0.0;
        for (int i = 0; i < nray; i++) {
            double x, y;
            bt_grid_point(nx, i, pupil, &x, &y);
            if (bt_in_annulus(x, y, r_in2, r_out2)) acc += Z[(size_t)a * nray + i] * Z[(size_t)b * nray + i];
        }
        gref[(size_t)nx * jmax * jmax + a * jmax + b] = acc;
        gref[(size_t)nx * jmax * jmax + b * jmax + a] = acc;
    }
}

static int g_batch_smem_max = 0;

// Largest dynamic shared memory the kernel can take on this device: the
// per-block opt-in maximum less the kernel's static shared memory.
cudaError_t bt_batch_set_smem_limit() {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_batch_zernike);
    if (e != cudaSuccess) return e;
    int lim = optin - (int)fa.sharedSizeBytes;
    if (lim > BT_BATCH_MAX_SMEM) lim = BT_BATCH_MAX_SMEM;
    e = cudaFuncSetAttribute(k_batch_zernike, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    if (e == cudaSuccess) g_batch_smem_max = lim;
    return e;
}

int bt_batch_smem_max() { return g_batch_smem_max; }

cudaError_t bt_launch_batch_zernike(const unsigned char* d_blob, int blob_bytes, const BatchArgs& a, int threads,
                                    int ctas_per_sm, cudaStream_t stream) {
    if (a.nqueue <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(a.counter, 0, sizeof(int), stream);
    if (e != cudaSuccess) return e;
    if (a.nchunk > 1) {
        e = cudaMemsetAsync(a.jobcnt, 0, sizeof(int) * (size_t)a.nqueue, stream);
        if (e != cudaSuccess) return e;
    }
    e = cudaMemsetAsync(a.status, 0xff, sizeof(int) * (size_t)a.njobs, stream);
    if (e != cudaSuccess) return e;
    const size_t smem = bt_batch_smem_layout(blob_bytes, threads, a.jmax).total;
    long long grid = (long long)bt_sm_count() * ctas_per_sm;
    if (grid > (long long)a.nqueue * a.nchunk) grid = (long long)a.nqueue * a.nchunk;
    if (grid < 1) grid = 1;
    k_batch_zernike<<<(int)grid, threads, smem, stream>>>(d_blob, blob_bytes, a);
    return cudaGetLastError();
}

cudaError_t bt_launch_batch_tables(int nx, double pupil, const double* cart, int jmax, int side, double* out,
                                   cudaStream_t stream) {
    const long long n = (long long)nx * nx * jmax;
    long long blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_batch_basis<<<(int)blocks, 256, 0, stream>>>(nx, pupil, cart, jmax, side, out);
    return cudaGetLastError();
}

cudaError_t bt_launch_batch_gref(const int* d_nx_list, int n, double pupil, double r_in2, double r_out2,
                                 const double* basis, const long long* basis_off, int jmax, double* gref,
                                 cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    k_batch_gref<<<n, 512, 0, stream>>>(d_nx_list, pupil, r_in2, r_out2, basis, basis_off, jmax, gref);
    return cudaGetLastError();
}
