// Per-ray stage logic shared by the fused trace kernel and the batched
// wavefront kernel.
#pragma once
#include "bt_internal.h"
#include "bt_device.cuh"

struct RayState {
    double x, y, z, vx, vy, vz, t, w, f;
    bool vig, fail;
};

__device__ __forceinline__ void store_ray(const RV& o, long long i, const RayState& r) {
    o.x[i] = r.x;
    o.y[i] = r.y;
    o.z[i] = r.z;
    o.vx[i] = r.vx;
    o.vy[i] = r.vy;
    o.vz[i] = r.vz;
    o.t[i] = r.t;
    o.w[i] = r.w;
    o.f[i] = r.f;
    o.vig[i] = r.vig;
    o.fail[i] = r.fail;
}

// Phase screen (src/batoid.cpp:677-810): the direction cosines relative to
// an orthonormal basis around the surface normal change by the screen's
// gradient; the screen's sag adds to the time.  Out of line: only OPDScreen
// stages reach it.
static __device__ __noinline__ void bt_screen_deflect(const Prog P, int surf, int screen, double x, double y,
                                                      double* vx, double* vy, double* vz, double* t) {
    const double norm = sqrt(*vx * *vx + *vy * *vy + *vz * *vz);
    const double norm_inv = 1 / norm;
    double e3x, e3y, e3z;
    bt_normal_precise(P, surf, x, y, &e3x, &e3y, &e3z);
    const double e1norm = sqrt(e3z * e3z + e3x * e3x);
    const double e1x = e3z / e1norm, e1y = 0, e1z = -e3x / e1norm;
    const double e2x = e3y * e1z - e3z * e1y;
    const double e2y = e3z * e1x - e3x * e1z;
    const double e2z = e3x * e1y - e3y * e1x;
    double cos1 = *vx * norm_inv * e1x + *vy * norm_inv * e1y + *vz * norm_inv * e1z;
    double cos2 = *vx * norm_inv * e2x + *vy * norm_inv * e2y + *vz * norm_inv * e2z;
    double cos3 = *vx * norm_inv * e3x + *vy * norm_inv * e3y + *vz * norm_inv * e3z;
    double sag, ux, uy;
    bt_surf_eval(P, screen, x, y, true, true, &sag, &ux, &uy);
    const double dPdx = -ux, dPdy = -uy;
    const double dPd1 = dPdx * e1x + dPdy * e1y;
    const double dPd2 = dPdx * e2x + dPdy * e2y;
    if (cos3 < 0) {
        cos1 += dPd1;
        cos2 += dPd2;
        cos3 = -sqrt(1 - cos1 * cos1 - cos2 * cos2);
    } else {
        cos1 -= dPd1;
        cos2 -= dPd2;
        cos3 = sqrt(1 - cos1 * cos1 - cos2 * cos2);
    }
    *vx = cos1 * norm * e1x + cos2 * norm * e2x + cos3 * norm * e3x;
    *vy = cos1 * norm * e1y + cos2 * norm * e2y + cos3 * norm * e3y;
    *vz = cos1 * norm * e1z + cos2 * norm * e2z + cos3 * norm * e3z;
    *t += sag;
}

// One stage of the trace for one ray.  Semantics of src/batoid.cpp:175-506:
// failed rays are skipped and keep their coordinates in the previous frame;
// a ray that misses the surface is flagged failed+vignetted and likewise
// keeps its previous coordinates; TIR writes the position, NaN velocity.
// A medium's index and its reciprocal depend only on the ray's wavelength,
// so they are computed once per ray per medium.
template <bool PRESTEP = false>
__device__ __forceinline__ void run_stage(const Prog& P, const bt_stage& st, RayState& r, int niter,
                                          int& cached_medium, double& cached_n, double& cached_inv_n) {
    if (st.kind != BT_ST_OBSCURE && !r.fail) {
        double x, y, z, vx, vy, vz;
        if (st.identity == 1) {
            x = r.x; y = r.y; z = r.z; vx = r.vx; vy = r.vy; vz = r.vz;
        } else if (st.identity == 2) {
            // rotation is the identity: dx*1 + dy*0 + dz*0 == dx exactly
            x = r.x - st.dr[0]; y = r.y - st.dr[1]; z = r.z - st.dr[2];
            vx = r.vx; vy = r.vy; vz = r.vz;
        } else {
            const double dx = r.x - st.dr[0], dy = r.y - st.dr[1], dz = r.z - st.dr[2];
            x = dx * st.drot[0] + dy * st.drot[3] + dz * st.drot[6];
            y = dx * st.drot[1] + dy * st.drot[4] + dz * st.drot[7];
            z = dx * st.drot[2] + dy * st.drot[5] + dz * st.drot[8];
            vx = r.vx * st.drot[0] + r.vy * st.drot[3] + r.vz * st.drot[6];
            vy = r.vx * st.drot[1] + r.vy * st.drot[4] + r.vz * st.drot[7];
            vz = r.vx * st.drot[2] + r.vy * st.drot[5] + r.vz * st.drot[8];
        }
        double dt = 0.0;
        const bool ok = bt_surf_tti_fast<PRESTEP>(P, st.surf, x, y, z, vx, vy, vz, dt, niter);
        if (ok) {
            x += vx * dt;
            y += vy * dt;
            z += vz * dt;
            double t = r.t + dt;
            if (st.kind == BT_ST_INTERSECT) {
                if (st.coated) r.f *= st.coat_t;
            } else if (st.kind == BT_ST_SCREEN) {
                bt_screen_deflect(P, st.surf, st.screen, x, y, &vx, &vy, &vz, &t);
            } else {
                double nx, ny, nz;
                bt_normal_precise(P, st.surf, x, y, &nx, &ny, &nz);
                if (st.kind == BT_ST_REFLECT) {
                    // src/batoid.cpp:343-353
                    const double alpha = vx * nx + vy * ny + vz * nz;
                    vx -= 2 * alpha * nx;
                    vy -= 2 * alpha * ny;
                    vz -= 2 * alpha * nz;
                    if (st.coated) r.f *= st.coat_r;
                } else {
                    // src/batoid.cpp:453-499
                    const double n1 = rsqrt(vx * vx + vy * vy + vz * vz);
                    const double nvx = vx * n1, nvy = vy * n1, nvz = vz * n1;
                    double alpha = nvx * nx + nvy * ny + nvz * nz;
                    if (alpha > 0.) {
                        nx = -nx; ny = -ny; nz = -nz;
                        alpha = -alpha;
                    }
                    double n2, inv_n2;
                    const int mi = st.medium;
                    if (P.media[mi].kind == BT_M_CONST) {
                        n2 = P.media[mi].p[0];
                        inv_n2 = P.media[mi].p[1];
                    } else if (mi == cached_medium) {
                        n2 = cached_n;   // same medium, same wavelength: same value
                        inv_n2 = cached_inv_n;
                    } else {
                        n2 = bt_getN(P, mi, r.w);
                        inv_n2 = 1.0 / n2;
                        if (P.media[mi].kind != BT_M_CONST) {
                            cached_medium = mi;
                            cached_n = n2;
                            cached_inv_n = inv_n2;
                        }
                    }
                    const double eta = n1 * inv_n2;
                    const double sinsqr = eta * eta * (1 - alpha * alpha);
                    if (sinsqr > 1.0) {
                        vx = NAN; vy = NAN; vz = NAN;
                        r.fail = true;
                        r.vig = true;
                    } else {
                        double cosr, rs;
                        bt_sqrt_rsqrt(1 - sinsqr, &cosr, &rs);
                        const double nfactor = eta * alpha + cosr;
                        vx = (eta * nvx - nfactor * nx) * inv_n2;
                        vy = (eta * nvy - nfactor * ny) * inv_n2;
                        vz = (eta * nvz - nfactor * nz) * inv_n2;
                    }
                    if (st.coated) r.f *= st.coat_t;
                }
            }
            r.x = x; r.y = y; r.z = z;
            r.vx = vx; r.vy = vy; r.vz = vz;
            r.t = t;
        } else {
            r.fail = true;
            r.vig = true;
        }
    }
    if (st.obsc_end > st.obsc_begin) {
        // src/batoid.cpp:169-171: vignetted |= contains(x, y), for every ray
        if (bt_obsc_run(P, st.obsc_begin, st.obsc_end, r.x, r.y)) r.vig = true;
    }
}

