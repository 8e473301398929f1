// Huygens phasor sum over a pixel lattice (replaces the per-pixel Python loop
// of huygensPSF calling RayVector.sumAmplitude, batoid/analysis.py:296-304 and
// src/rayVector.cpp:169-222).
//
// The phase of ray r at lattice point P(a, b) = P0 + b'*p0 + a'*p1
// (a' = a - na/2, b' = b - nb/2) is linear in (a', b'):
//     phi = 2 pi [ phi0_r + b' alpha_r + a' beta_r ]        (in turns)
// phi0, alpha, beta are formed once per ray in FP64 and reduced modulo one
// turn into 32-bit fixed point, so phi(a, b) = th + b' A + a' B is evaluated
// exactly modulo 2^32 with integer wrap-around.  Per ray-pixel pair the
// kernel then needs one integer FMA, a fast FP32 sincos (or a complex
// rotation by exp(2 pi i A) for neighbouring pixels) and one complex FMA.
// Each thread owns HUY_PX consecutive pixels of one lattice row; sums over a
// shared-memory tile of rays are plain FP32 and folded into Kahan-compensated
// FP32 running sums.  Rays are split across blocks; the per-split partial
// sums (device scratch) are reduced in FP64 in a fixed order.
#include <cuda_runtime.h>
#include <stdint.h>
#include "bt_internal.h"

#define HUY_THREADS 256
#define HUY_PX 4
#define HUY_TILE 256

struct __align__(16) HuyRec {
    uint32_t th;   // phase at P0, turns * 2^32
    uint32_t A;    // phase step per b, turns * 2^32
    uint32_t B;    // phase step per a, turns * 2^32
    float f;       // flux (0 for excluded rays)
    float ca;      // cos(2 pi A / 2^32)
    float sa;      // sin(2 pi A / 2^32)
    float pad0, pad1;
};

__device__ __forceinline__ uint32_t turns_to_fix32(double turns) {
    double fr = turns - floor(turns);           // [0, 1]
    double s = rint(fr * 4294967296.0);         // [0, 2^32]
    unsigned long long u = (unsigned long long)s;
    return (uint32_t)(u & 0xffffffffull);
}

// Lattice and reference point of one field: amplitudes at
// P(a, b) = (px, py, pz) + (b - nb/2) (l0, l1, 0) + (a - na/2) (l2, l3, 0).
struct HuyField {
    double px, py, pz, l0, l1, l2, l3, t0;
};

#define HUY_MAX_FIELDS 64

// Up to HUY_MAX_FIELDS fields per launch set, passed by value (4 KB).
struct HuyFields {
    HuyField f[HUY_MAX_FIELDS];
};

// Rays [f * per_field, (f + 1) * per_field) belong to field f.
__global__ void k_huy_prep(RV rv, long long per_field, const __grid_constant__ HuyFields F, int ignore_vig,
                           HuyRec* rec) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < rv.n;
         i += (long long)gridDim.x * blockDim.x) {
        const HuyField& fd = F.f[i / per_field];
        HuyRec r;
        r.pad0 = 0.f;
        r.pad1 = 0.f;
        const bool use = !rv.fail[i] && !(ignore_vig && rv.vig[i]);
        if (use) {
            const double vx = rv.vx[i], vy = rv.vy[i], vz = rv.vz[i];
            const double v2 = vx * vx + vy * vy + vz * vz;
            const double w = rv.w[i];
            // same ordering as src/rayVector.cpp:208-214, in turns
            double ph = (fd.px - rv.x[i]) * vx;
            ph += (fd.py - rv.y[i]) * vy;
            ph += (fd.pz - rv.z[i]) * vz;
            ph /= v2;
            ph -= fd.t0 - rv.t[i];
            ph /= w;
            const double al = (fd.l0 * vx + fd.l1 * vy) / v2 / w;
            const double be = (fd.l2 * vx + fd.l3 * vy) / v2 / w;
            r.th = turns_to_fix32(ph);
            r.A = turns_to_fix32(al);
            r.B = turns_to_fix32(be);
            r.f = (float)rv.f[i];
            double sd, cd;
            sincospi((double)(int32_t)r.A * (2.0 / 4294967296.0), &sd, &cd);
            r.ca = (float)cd;
            r.sa = (float)sd;
            if (!(ph == ph) || !(al == al) || !(be == be)) {
                // non-finite phase: contributes NaN, as in the reference
                r.f = __int_as_float(0x7fc00000);
            }
        } else {
            r.th = 0u; r.A = 0u; r.B = 0u;
            r.f = 0.f; r.ca = 1.f; r.sa = 0.f;
        }
        rec[i] = r;
    }
}

__device__ __forceinline__ void kahan_add(float& sum, float& comp, float v) {
    const float y = v - comp;
    const float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

// grid: (tiles, nsplit, fields).  rec: per_field records per field;
// part_* : [fields][nsplit][na*nb] doubles.
__global__ void __launch_bounds__(HUY_THREADS)
k_huy_main(const HuyRec* __restrict__ rec, long long per_field, int na, int nb, int ngroups_b,
           long long rays_per_split, double* part_re, double* part_im) {
    rec += (long long)blockIdx.z * per_field;
    const long long nrays = per_field;
    __shared__ HuyRec tile[HUY_TILE];
    const long long g = (long long)blockIdx.x * HUY_THREADS + threadIdx.x;  // pixel group
    const long long ngroups = (long long)na * ngroups_b;
    const bool active = g < ngroups;
    const int a = active ? (int)(g / ngroups_b) : 0;
    const int b0 = active ? (int)(g % ngroups_b) * HUY_PX : 0;
    const int ap = a - na / 2;
    const int bp = b0 - nb / 2;

    float sre[HUY_PX], cre[HUY_PX], sim[HUY_PX], cim[HUY_PX];
#pragma unroll
    for (int k = 0; k < HUY_PX; k++) { sre[k] = 0.f; cre[k] = 0.f; sim[k] = 0.f; cim[k] = 0.f; }

    const long long r0 = (long long)blockIdx.y * rays_per_split;
    long long r1 = r0 + rays_per_split;
    if (r1 > nrays) r1 = nrays;
    const float two_pi_over_2_32 = 1.4629180792671596e-09f;  // 2 pi / 2^32

    for (long long base = r0; base < r1; base += HUY_TILE) {
        const int cnt = (int)((r1 - base) < HUY_TILE ? (r1 - base) : HUY_TILE);
        __syncthreads();
        if (threadIdx.x < cnt) tile[threadIdx.x] = rec[base + threadIdx.x];
        __syncthreads();
        if (!active) continue;
        float tre[HUY_PX], tim[HUY_PX];
#pragma unroll
        for (int k = 0; k < HUY_PX; k++) { tre[k] = 0.f; tim[k] = 0.f; }
        for (int j = 0; j < cnt; j++) {
            const HuyRec r = tile[j];
            const uint32_t th = r.th + (uint32_t)bp * r.A + (uint32_t)ap * r.B;
            float s, c;
            __sincosf((float)(int32_t)th * two_pi_over_2_32, &s, &c);
            tre[0] = fmaf(r.f, c, tre[0]);
            tim[0] = fmaf(r.f, s, tim[0]);
#pragma unroll
            for (int k = 1; k < HUY_PX; k++) {
                const float c2 = c * r.ca - s * r.sa;
                const float s2 = s * r.ca + c * r.sa;
                c = c2;
                s = s2;
                tre[k] = fmaf(r.f, c, tre[k]);
                tim[k] = fmaf(r.f, s, tim[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < HUY_PX; k++) {
            kahan_add(sre[k], cre[k], tre[k]);
            kahan_add(sim[k], cim[k], tim[k]);
        }
    }
    if (!active) return;
    const long long npix = (long long)na * nb;
    const long long part = (long long)blockIdx.z * gridDim.y + blockIdx.y;
    double* pr = part_re + part * npix;
    double* pi = part_im + part * npix;
#pragma unroll
    for (int k = 0; k < HUY_PX; k++) {
        const int b = b0 + k;
        if (b < nb) {
            pr[(long long)a * nb + b] = (double)sre[k] - (double)cre[k];
            pi[(long long)a * nb + b] = (double)sim[k] - (double)cim[k];
        }
    }
}

// out_*: [fields][npix]; the splits of a pixel are added in a fixed order.
__global__ void k_huy_reduce(const double* part_re, const double* part_im, int nsplit, long long npix, int nfields,
                             double* out_re, double* out_im) {
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < npix * nfields;
         p += (long long)gridDim.x * blockDim.x) {
        const long long f = p / npix, q = p - f * npix;
        const double* pr = part_re + f * nsplit * npix + q;
        const double* pi = part_im + f * nsplit * npix + q;
        double re = 0.0, im = 0.0;
        for (int s = 0; s < nsplit; s++) {
            re += pr[(long long)s * npix];
            im += pi[(long long)s * npix];
        }
        out_re[p] = re;
        out_im[p] = im;
    }
}

// Ray splits per field: enough blocks for ~4 per SM over all fields, each
// split a multiple of the ray tile.
static void huy_split(long long per_field, long long tiles, int nfields, long long max_split_mem, long long* nsplit,
                      long long* per) {
    const int sms = bt_sm_count();
    long long ns = (4LL * sms + tiles * nfields - 1) / (tiles * nfields);
    const long long max_split = (per_field + HUY_TILE - 1) / HUY_TILE;
    if (ns > max_split) ns = max_split;
    if (ns > max_split_mem) ns = max_split_mem;
    if (ns > 65535) ns = 65535;
    if (ns < 1) ns = 1;
    long long pr = (per_field + ns - 1) / ns;
    pr = ((pr + HUY_TILE - 1) / HUY_TILE) * HUY_TILE;
    *per = pr;
    *nsplit = (per_field + pr - 1) / pr;
}

// prep + main + reduce for nfields (<= HUY_MAX_FIELDS) fields whose rays
// are consecutive blocks of per_field rays; scratch holds the records
// (rec_bytes, 256-aligned) and then the partial sums.
static cudaError_t huy_run(const RV& rv, long long per_field, const HuyFields& F, int nfields, int na, int nb,
                           bool ignore_vig, long long nsplit, long long per, char* scratch, size_t rec_bytes,
                           double* out_re, double* out_im, cudaStream_t stream) {
    const long long npix = (long long)na * nb;
    const int ngroups_b = (nb + HUY_PX - 1) / HUY_PX;
    const long long tiles = ((long long)na * ngroups_b + HUY_THREADS - 1) / HUY_THREADS;
    const int sms = bt_sm_count();
    HuyRec* rec = reinterpret_cast<HuyRec*>(scratch);
    double* pre = reinterpret_cast<double*>(scratch + rec_bytes);
    double* pim = pre + (size_t)nfields * nsplit * npix;
    long long pg = (rv.n + 255) / 256;
    if (pg > (long long)sms * 16) pg = (long long)sms * 16;
    k_huy_prep<<<(int)pg, 256, 0, stream>>>(rv, per_field, F, ignore_vig ? 1 : 0, rec);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)tiles, (unsigned)nsplit, (unsigned)nfields);
    k_huy_main<<<grid, HUY_THREADS, 0, stream>>>(rec, per_field, na, nb, ngroups_b, per, pre, pim);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    long long rg = (npix * nfields + 255) / 256;
    if (rg > (long long)sms * 8) rg = (long long)sms * 8;
    k_huy_reduce<<<(int)rg, 256, 0, stream>>>(pre, pim, (int)nsplit, npix, nfields, out_re, out_im);
    return cudaGetLastError();
}

static HuyField huy_field(double px, double py, double pz, const double lat[4], double t0) {
    HuyField f;
    f.px = px; f.py = py; f.pz = pz;
    f.l0 = lat[0]; f.l1 = lat[1]; f.l2 = lat[2]; f.l3 = lat[3];
    f.t0 = t0;
    return f;
}

cudaError_t bt_launch_huygens(const RV& rv, double px, double py, double pz, const double lat[4], int na,
                              int nb, double t0, bool ignore_vig, double* out_re, double* out_im,
                              cudaStream_t stream) {
    return bt_launch_huygens_fields(rv, rv.n, 1, &px, &py, &pz, lat, &t0, 1, na, nb, ignore_vig, out_re, out_im,
                                    stream);
}

// Many fields: field f's rays are rows [f * per_field, (f + 1) * per_field)
// of rv, its point (px[f*ps], py[f*ps], pz[f*ps]) (ps = point stride), its
// lattice lat[4f .. 4f+3] and reference time t0[f]; outputs [nfields][na*nb].
// One launch set (prep, main, reduce) per HUY_MAX_FIELDS fields.
cudaError_t bt_launch_huygens_fields(const RV& rv, long long per_field, int nfields, const double* px,
                                     const double* py, const double* pz, const double* lat, const double* t0,
                                     int ps, int na, int nb, bool ignore_vig, double* out_re, double* out_im,
                                     cudaStream_t stream) {
    const long long npix = (long long)na * nb;
    if (npix <= 0 || nfields <= 0) return cudaSuccess;
    if (per_field <= 0) {
        cudaError_t e = cudaMemsetAsync(out_re, 0, npix * nfields * sizeof(double), stream);
        if (e != cudaSuccess) return e;
        return cudaMemsetAsync(out_im, 0, npix * nfields * sizeof(double), stream);
    }
    const int ngroups_b = (nb + HUY_PX - 1) / HUY_PX;
    const long long tiles = ((long long)na * ngroups_b + HUY_THREADS - 1) / HUY_THREADS;
    const int chunk = nfields < HUY_MAX_FIELDS ? nfields : HUY_MAX_FIELDS;
    // each field is split as a single-field call splits it, so that every
    // field's amplitudes are bit-identical to that call's
    long long nsplit, per;
    huy_split(per_field, tiles, 1, 1LL << 40, &nsplit, &per);
    // scratch: ray records and per-split partial sums of one chunk of fields
    const size_t rec_bytes = (((size_t)per_field * chunk * sizeof(HuyRec)) + 255) & ~(size_t)255;
    const size_t part_bytes = (size_t)chunk * nsplit * npix * sizeof(double);
    char* scratch = nullptr;
    bt_keep_pool();
    cudaError_t e = cudaMallocAsync((void**)&scratch, rec_bytes + 2 * part_bytes, stream);
    if (e != cudaSuccess) return e;
    HuyFields F;
    for (int f0 = 0; f0 < nfields && e == cudaSuccess; f0 += HUY_MAX_FIELDS) {
        const int nf = (nfields - f0) < HUY_MAX_FIELDS ? (nfields - f0) : HUY_MAX_FIELDS;
        for (int k = 0; k < nf; k++) {
            const int f = f0 + k;
            F.f[k] = huy_field(px[(size_t)f * ps], py[(size_t)f * ps], pz[(size_t)f * ps], lat + 4 * (size_t)f, t0[f]);
        }
        RV sub = rv;
        sub.n = per_field * nf;
        const long long off = per_field * f0;
        sub.x += off; sub.y += off; sub.z += off; sub.vx += off; sub.vy += off; sub.vz += off;
        sub.t += off; sub.w += off; sub.f += off; sub.vig += off; sub.fail += off;
        e = huy_run(sub, per_field, F, nf, na, nb, ignore_vig, nsplit, per, scratch, rec_bytes,
                    out_re + (size_t)f0 * npix, out_im + (size_t)f0 * npix, stream);
    }
    cudaError_t e2 = cudaFreeAsync(scratch, stream);
    return e != cudaSuccess ? e : e2;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the Huygens amplitudes.
//
// Some callers cannot let this library allocate device memory: a host
// framework that owns every byte of device memory under a fixed budget, code
// that must not trigger the implicit synchronisation or allocator traffic of
// cudaMalloc inside a latency-critical loop, or an embedding that only hands
// over pre-allocated input and output buffers.  For them the scratch this
// kernel needs (32 bytes per ray for the phase records plus 16 bytes per
// pixel per ray split for partial sums) lives in a fixed file-scope device
// array of HUY_NOALLOC_BYTES, which every GPU that loads the library holds
// until the process exits.
//
// Set-up: the first call on a device (with that device current) looks up the
// array's device address with cudaGetSymbolAddress and caches it per device;
// make that first call before any stream capture.  The cached address is not
// looked up again: after cudaDeviceReset (or anything else that destroys the
// device's primary context) it is stale, so a process that resets a device
// must not call this entry point on that device again.  All calls share the one
// array and it keeps the last call's contents: nothing in it has to start at
// zero (every record and partial sum is written before it is read within a
// call), but calls whose kernels overlap on the GPU -- on different streams
// without ordering, or from several host threads -- race on it.
// ---------------------------------------------------------------------------

#include <mutex>

#define HUY_NOALLOC_BYTES (8u << 20)
#define HUY_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_huy_noalloc_scratch[HUY_NOALLOC_BYTES];

static std::mutex g_huy_noalloc_mu;
static void* g_huy_noalloc_ptr[HUY_MAX_DEVICES];

static cudaError_t huy_noalloc_scratch(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= HUY_MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_huy_noalloc_mu);
    if (!g_huy_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_huy_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_huy_noalloc_ptr[dev] = p;
    }
    *out = g_huy_noalloc_ptr[dev];
    return cudaSuccess;
}

// Returns cudaErrorInvalidValue when the problem does not fit the scratch
// array (the C-ABI wrapper turns that into a size message).
cudaError_t bt_launch_huygens_noalloc(const RV& rv, double px, double py, double pz, const double lat[4], int na,
                                      int nb, double t0, bool ignore_vig, double* out_re, double* out_im,
                                      cudaStream_t stream, size_t* needed) {
    const long long npix = (long long)na * nb;
    *needed = 0;
    if (npix <= 0) return cudaSuccess;
    if (rv.n <= 0) {
        cudaError_t e = cudaMemsetAsync(out_re, 0, npix * sizeof(double), stream);
        if (e != cudaSuccess) return e;
        return cudaMemsetAsync(out_im, 0, npix * sizeof(double), stream);
    }
    const size_t rec_bytes = ((size_t)rv.n * sizeof(HuyRec) + 255) & ~(size_t)255;
    const size_t split_bytes = 2 * (size_t)npix * sizeof(double);
    *needed = rec_bytes + split_bytes;
    if (rec_bytes + split_bytes > HUY_NOALLOC_BYTES) return cudaErrorInvalidValue;
    const long long max_split_mem = (long long)((HUY_NOALLOC_BYTES - rec_bytes) / split_bytes);
    const int ngroups_b = (nb + HUY_PX - 1) / HUY_PX;
    const long long tiles = ((long long)na * ngroups_b + HUY_THREADS - 1) / HUY_THREADS;
    long long nsplit, per;
    huy_split(rv.n, tiles, 1, max_split_mem, &nsplit, &per);

    void* base = nullptr;
    cudaError_t e = huy_noalloc_scratch(&base);
    if (e != cudaSuccess) return e;
    HuyFields F;
    F.f[0] = huy_field(px, py, pz, lat, t0);
    return huy_run(rv, rv.n, F, 1, na, nb, ignore_vig, nsplit, per, static_cast<char*>(base), rec_bytes, out_re,
                   out_im, stream);
}
