/*
 * batoid_gb300 — C-ABI of the GB300-native sequential ray tracer.
 *
 * This header is the drop-in boundary that replaces the reference's pybind11
 * module `batoid._batoid` (pysrc/batoid.cpp:31-154 of jmeyers314/batoid).  Each
 * entry point below names the reference interface it replaces.
 *
 * Conventions
 *  - Every function returns an int status: BT_OK (0) or one of BT_ERR_*;
 *    bt_last_error() returns a message for the last failure in this thread.
 *  - Ray arrays and output arrays are DEVICE pointers (CUDA global memory of
 *    the current device) unless a function says "host".  The library never
 *    takes ownership of them (the reference's DualView also wraps caller
 *    memory: src/dualView.cpp:5-10).
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *    stream).  Launches are stream-ordered and asynchronous; functions that
 *    return a host value synchronise the stream first.
 *  - `max_threads` is accepted for signature compatibility with the
 *    reference and ignored; `niter` is the Newton iteration cap
 *    (batoid/global_vars.py:9).
 *  - Per-ray failures are data, as in the reference: the `failed` and
 *    `vignetted` flags and NaN directions (src/batoid.cpp:264-267, 482-487).
 *  - Rotation matrices `drot` are 9 doubles, column-major, exactly as the
 *    reference passes `CoordTransform.drot.ravel()` (include/batoid.h:13).
 */
#ifndef BATOID_GB300_H
#define BATOID_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BT_OK 0
#define BT_ERR_ARG 1          /* invalid argument */
#define BT_ERR_CUDA 2         /* CUDA runtime error */
#define BT_ERR_UNSUPPORTED 3  /* valid but unsupported configuration */
#define BT_ERR_RANK 4         /* rank-deficient least-squares system */
#define BT_ERR_TIMEOUT 5      /* a bounded device wait expired */
#define BT_ERR_ALLOC 6        /* device allocation failed */

/* Structure-of-arrays ray bundle, 74 bytes per ray.
 * Replaces CPPRayVector(x, y, z, vx, vy, vz, t, wavelength, flux, vignetted,
 * failed, N) (pysrc/rayVector.cpp:32-62; include/rayVector.h:8-39).
 * Flags are one byte each (C/C++ bool). */
typedef struct bt_rayvector {
    double* x;
    double* y;
    double* z;
    double* vx;
    double* vy;
    double* vz;
    double* t;
    double* wavelength;
    double* flux;
    uint8_t* vignetted;
    uint8_t* failed;
    size_t size;
} bt_rayvector;

typedef struct bt_surface bt_surface;
typedef struct bt_table bt_table;
typedef struct bt_medium_h bt_medium_h;
typedef struct bt_obscuration bt_obscuration;
typedef struct bt_coating bt_coating;
typedef struct bt_optic bt_optic;

/* ---- library ----------------------------------------------------------- */
const char* bt_last_error(void);
int bt_version(void);
/* Number of SMs of the current device (used to size persistent grids). */
int bt_device_sm_count(int* out);

/* ---- surfaces (pysrc/{plane,tilted,sphere,paraboloid,quadric,asphere,
 *      polynomialSurface,table,bicubic,sum}.cpp) ----------------------------- */
int bt_plane_create(bt_surface** out);                                /* CPPPlane()            pysrc/plane.cpp */
int bt_tilted_create(double tanx, double tany, bt_surface** out);     /* CPPTilted(tanx, tany) pysrc/tilted.cpp */
int bt_sphere_create(double R, bt_surface** out);                     /* CPPSphere(R)          pysrc/sphere.cpp */
int bt_paraboloid_create(double R, bt_surface** out);                 /* CPPParaboloid(R)      pysrc/paraboloid.cpp */
int bt_quadric_create(double R, double conic, bt_surface** out);      /* CPPQuadric(R, conic)  pysrc/quadric.cpp */
/* CPPAsphere(R, conic, coef_ptr, n) (pysrc/asphere.cpp:11-24); coefs are the
 * padded host array whose entry i multiplies r^(2i+2). */
int bt_asphere_create(double R, double conic, const double* coefs, size_t n, bt_surface** out);
/* CPPPolynomialSurface(coefs, gradx, grady, xorigin, yorigin, xsize, ysize)
 * (pysrc/polynomialSurface.cpp:10-28); host arrays, coefs [ysize][xsize],
 * gradients [(ysize-1)][(xsize-1)]. */
int bt_polynomial_create(const double* coefs, const double* gradx, const double* grady,
                         double xorigin, double yorigin, size_t xsize, size_t ysize,
                         bt_surface** out);
/* CPPTable(x0, y0, dx, dy, z, dzdx, dzdy, d2zdxdy, nx, ny, use_nan)
 * (pysrc/table.cpp:10-33); host arrays [ny][nx], copied to device memory
 * owned by the table. */
int bt_table_create(double x0, double y0, double dx, double dy,
                    const double* z, const double* dzdx, const double* dzdy, const double* d2zdxdy,
                    size_t nx, size_t ny, int use_nan, bt_table** out);
void bt_table_destroy(bt_table* table);
/* CPPBicubic(table) (pysrc/bicubic.cpp); the table must outlive the surface. */
int bt_bicubic_create(const bt_table* table, bt_surface** out);
/* CPPSum(list) (pysrc/sum.cpp:11-19); children are copied by value, so they
 * may be destroyed afterwards.  Children may not themselves be Sums. */
int bt_sum_create(const bt_surface* const* surfaces, size_t n, bt_surface** out);
void bt_surface_destroy(bt_surface* s);
/* Surface.sag (pysrc/surface.cpp:10; py::vectorize(&Surface::sag)): device arrays. */
int bt_surface_sag(const bt_surface* s, const double* x, const double* y, double* out, size_t n, void* stream);
/* Surface.normal (pysrc/surface.cpp:11-21): out holds nx[0..n), ny[0..n), nz[0..n). */
int bt_surface_normal(const bt_surface* s, const double* x, const double* y, double* out, size_t n, void* stream);

/* ---- media (pysrc/medium.cpp; src/medium.cpp) ---------------------------- */
int bt_const_medium_create(double n, bt_medium_h** out);                                   /* CPPConstMedium */
int bt_table_medium_create(const double* wavelengths, const double* ns, size_t n, bt_medium_h** out); /* CPPTableMedium */
int bt_sellmeier_medium_create(double B1, double B2, double B3, double C1, double C2, double C3,
                               bt_medium_h** out);                                         /* CPPSellmeierMedium */
int bt_sumita_medium_create(double A0, double A1, double A2, double A3, double A4, double A5,
                            bt_medium_h** out);                                            /* CPPSumitaMedium */
int bt_air_create(double pressure, double temperature, double h2o_pressure, bt_medium_h** out); /* CPPAir */
void bt_medium_destroy(bt_medium_h* m);
/* Medium.getN over a device array of wavelengths. */
int bt_medium_getN(const bt_medium_h* m, const double* wavelength, double* out, size_t n, void* stream);

/* ---- obscurations (pysrc/obscuration.cpp; src/obscuration.cpp) ---------- */
int bt_obsc_circle_create(double radius, double x0, double y0, bt_obscuration** out);
int bt_obsc_annulus_create(double inner, double outer, double x0, double y0, bt_obscuration** out);
int bt_obsc_rectangle_create(double width, double height, double x0, double y0, double theta, bt_obscuration** out);
int bt_obsc_ray_create(double width, double theta, double x0, double y0, bt_obscuration** out);
int bt_obsc_polygon_create(const double* xs, const double* ys, size_t n, bt_obscuration** out);
int bt_obsc_negation_create(const bt_obscuration* original, bt_obscuration** out);
int bt_obsc_union_create(const bt_obscuration* const* items, size_t n, bt_obscuration** out);
int bt_obsc_intersection_create(const bt_obscuration* const* items, size_t n, bt_obscuration** out);
void bt_obsc_destroy(bt_obscuration* o);
/* Obscuration.contains over device arrays; out is one byte per point. */
int bt_obsc_contains(const bt_obscuration* o, const double* x, const double* y, uint8_t* out, size_t n, void* stream);

/* ---- coatings (pysrc/coating.cpp) ---------------------------------------- */
int bt_simple_coating_create(double reflectivity, double transmissivity, bt_coating** out);
void bt_coating_destroy(bt_coating* c);

/* ---- per-surface trace operations (include/batoid.h:15-42;
 *      src/batoid.cpp:8-506) -------------------------------------------------- */
int bt_apply_forward_transform(const double dr[3], const double drot[9], const bt_rayvector* rv,
                               int max_threads, void* stream);           /* src/batoid.cpp:71-108 */
int bt_apply_reverse_transform(const double dr[3], const double drot[9], const bt_rayvector* rv,
                               int max_threads, void* stream);           /* src/batoid.cpp:111-148 */
int bt_apply_forward_transform_arrays(const double dr[3], const double drot[9],
                                      double* x, double* y, double* z, size_t n,
                                      int max_threads, void* stream);    /* src/batoid.cpp:8-22 */
int bt_apply_reverse_transform_arrays(const double dr[3], const double drot[9],
                                      double* x, double* y, double* z, size_t n,
                                      int max_threads, void* stream);    /* src/batoid.cpp:24-38 */
int bt_finish_parallel(const double dr[3], const double drot[9], const double vv[3],
                       double* x, double* y, double* z, size_t n, void* stream); /* src/batoid.cpp:40-69 */
/* Stop-surface sample points of the ray factories, generated on the device
 * (replaces the numpy point generation of RayVector.asGrid / asPolar /
 * asSpokes, batoid/rayVector.py:411-444, batoid/utils.py:512-535,
 * batoid/rayVector.py:786-814; the reference builds these arrays on the host
 * and copies them).  x, y: device arrays of nx*ny, n, nr*ns points.
 *   grid:   point i = (i % nx, i / nx): u = (i%nx - nx/2) valx,
 *           w = (i/nx - ny/2) valy (valx = 1/(nx dx), numpy fftfreq),
 *           x = lx[0] u + lx[1] w, y = ly[0] u + ly[1] w;
 *   rings:  ring k holds points off[k]..off[k+1]-1 at radius r[k], azimuth
 *           j step[k] (r, step, off: device arrays of nring, nring, nring+1);
 *   spokes: point i at radius rings[i % nr], azimuth spokes[i / nr] (device). */
int bt_stop_points_grid(int nx, int ny, double valx, double valy, const double lx[2], const double ly[2],
                        double* x, double* y, void* stream);
int bt_stop_points_rings(int nring, const double* r, const double* step, const long long* off, long long n,
                         double* x, double* y, void* stream);
int bt_stop_points_spokes(const double* rings, int nr, const double* spokes, int ns, double* x, double* y,
                          void* stream);
/* refractScreen(surface, dr, drot, screen, rv, max_threads, niter)
 * (src/batoid.cpp:677-810; batoid/trace.py:139-153): intersect, then deflect
 * the direction cosines by the gradient of the screen surface's sag and add
 * the sag to the time. */
int bt_refract_screen(const bt_surface* s, const double dr[3], const double drot[9], const bt_surface* screen,
                      const bt_rayvector* rv, int max_threads, int niter, void* stream);
/* rSplit(surface, dr, drot, m1, m2, coating, rv, rvSplit, max_threads, niter)
 * (src/batoid.cpp:509-674; pysrc/batoid.cpp): intersect, then the refracted
 * ray replaces rv's ray and the reflected ray is written to rv_split, which
 * must hold a copy of rv on entry (batoid/trace.py:125); fluxes are scaled
 * by the coating's transmissivity / reflectivity. */
int bt_rsplit(const bt_surface* s, const double dr[3], const double drot[9], const bt_medium_h* m1,
              const bt_medium_h* m2, const bt_coating* coating, const bt_rayvector* rv, const bt_rayvector* rv_split,
              int max_threads, int niter, void* stream);
int bt_obscure(const bt_obscuration* o, const bt_rayvector* rv, int max_threads, void* stream); /* src/batoid.cpp:151-172 */
int bt_intersect(const bt_surface* s, const double dr[3], const double drot[9], const bt_rayvector* rv,
                 const bt_coating* coating, int max_threads, int niter, void* stream); /* src/batoid.cpp:175-270 */
int bt_reflect(const bt_surface* s, const double dr[3], const double drot[9], const bt_rayvector* rv,
               const bt_coating* coating, int max_threads, int niter, void* stream);   /* src/batoid.cpp:273-378 */
int bt_refract(const bt_surface* s, const double dr[3], const double drot[9],
               const bt_medium_h* m1, const bt_medium_h* m2, const bt_rayvector* rv,
               const bt_coating* coating, int max_threads, int niter, void* stream);   /* src/batoid.cpp:381-506 */

/* ---- RayVector methods (include/rayVector.h:10-25; src/rayVector.cpp) ---- */
int bt_rv_position_at_time(const bt_rayvector* rv, double t, double* xout, double* yout, double* zout,
                           int max_threads, void* stream);   /* src/rayVector.cpp:26-54 */
int bt_rv_propagate_in_place(const bt_rayvector* rv, double t, int max_threads, void* stream); /* :56-82 */
int bt_rv_phase(const bt_rayvector* rv, double x, double y, double z, double t, double* out,
                int max_threads, void* stream);              /* :84-122 */
/* out: interleaved (re, im) doubles, 2n entries (std::complex<double> layout). */
int bt_rv_amplitude(const bt_rayvector* rv, double x, double y, double z, double t, double* out,
                    int max_threads, void* stream);          /* :124-166 */
/* Synchronous; host out[2] = (re, im).  src/rayVector.cpp:169-222 */
int bt_rv_sum_amplitude(const bt_rayvector* rv, double x, double y, double z, double t,
                        int ignore_vignetted, int max_threads, double* out, void* stream);
/* Synchronous; host *out = 1 if every field of every ray is bitwise equal (:224-238). */
int bt_rv_equal(const bt_rayvector* a, const bt_rayvector* b, int* out, void* stream);

/* ---- fused optic trace (replaces the per-surface Python loop of
 *      CompoundOptic.trace/traceFull, batoid/optic.py:1013-1182) ------------ */
#define BT_STAGE_INTERSECT 0   /* Detector, Baffle, Interface (batoid/optic.py:541-546) */
#define BT_STAGE_REFLECT 1     /* Mirror (batoid/optic.py:814-816) */
#define BT_STAGE_REFRACT 2     /* RefractiveInterface (batoid/optic.py:776-781) */
#define BT_STAGE_SCREEN 4      /* OPDScreen (batoid/optic.py:912-918) */
/* Packs nstages interfaces, in trace order, into a device-resident program.
 * Per stage: kind, surface, transform from the previous stage's frame
 * (dr 3 doubles, drot 9 doubles column-major), outgoing medium (REFRACT
 * only, else NULL), obscuration (nullable) and coating (nullable). */
int bt_optic_create(size_t nstages, const int* kinds, const bt_surface* const* surfaces,
                    const double* dr, const double* drot,
                    const bt_medium_h* const* media, const bt_obscuration* const* obscurations,
                    const bt_coating* const* coatings, bt_optic** out);
/* Same, with screens[k] the OPD surface of each BT_STAGE_SCREEN stage
 * (screens may be NULL when no stage is a screen). */
int bt_optic_create_ex(size_t nstages, const int* kinds, const bt_surface* const* surfaces,
                       const double* dr, const double* drot,
                       const bt_medium_h* const* media, const bt_obscuration* const* obscurations,
                       const bt_coating* const* coatings, const bt_surface* const* screens, bt_optic** out);
void bt_optic_destroy(bt_optic* o);
int bt_optic_nstages(const bt_optic* o, int* out);
/* In-place trace of all stages in one launch (CompoundOptic.trace). */
int bt_optic_trace(const bt_optic* o, const bt_rayvector* rv, int niter, void* stream);
/* Out-of-place trace: reads `in`, writes the traced rays to `out` (same
 * size; may not partially overlap `in`).  Equivalent to copying then
 * tracing in place (CompoundOptic.trace on rv.copy()). */
int bt_optic_trace_into(const bt_optic* o, const bt_rayvector* in, const bt_rayvector* out, int niter,
                        void* stream);
/* traceFull: rv is read only; snaps[k] receives the rays after stage k
 * (CompoundOptic.traceFull's per-interface 'out' copies). */
int bt_optic_trace_full(const bt_optic* o, const bt_rayvector* rv, const bt_rayvector* snaps,
                        int niter, void* stream);
/* End-to-end trace of HOST arrays (pinned for overlap): copies in, traces
 * and copies out, pipelined in chunks of about `chunk` rays (0: 4M) over
 * device scratch buffers that the library allocates; a chunk of at least
 * 8 rounds of the trace kernel's persistent grid is rounded to a whole
 * number of 8 rounds.  Synchronous. */
int bt_optic_trace_host(const bt_optic* o, const bt_rayvector* host_rv, int niter, size_t chunk,
                        void* stream);

/* ---- Huygens PSF (replaces the per-pixel sumAmplitude loop of huygensPSF,
 *      batoid/analysis.py:296-304) --------------------------------------------
 * Amplitude at lattice points P(a, b) = (px, py, pz) + (b - nb/2)*p0 + (a - na/2)*p1
 * (integer division; p0 = (lat[0], lat[1], 0), p1 = (lat[2], lat[3], 0)),
 * a in [0, na), b in [0, nb), as the reference's transposed Lattice coords.
 * Phases are reduced modulo 2*pi in FP64 per ray; the per-pixel phasor
 * sum runs in FP32 with compensated summation.  Outputs: device arrays of
 * na*nb doubles (re, im), row-major [a][b]. */
int bt_huygens_amplitudes(const bt_rayvector* rv, double px, double py, double pz,
                          const double lat[4], int na, int nb, double t0, int ignore_vignetted,
                          double* out_re, double* out_im, void* stream);

/* bt_huygens_amplitudes for many fields in one launch set (what huygensPSF
 * computes per field, batoid/analysis.py:181-305, for a list of fields).
 * Field f's rays are rows [f*n/nfields, (f+1)*n/nfields) of rv (n must be a
 * multiple of nfields); its point is points[3f..3f+2], its lattice
 * lat[4f..4f+3] and its reference time t0[f] (host arrays).  Outputs:
 * device arrays of nfields*na*nb doubles, [f][a][b]. */
int bt_huygens_amplitudes_fields(const bt_rayvector* rv, int nfields, const double* points, const double* lat,
                                 const double* t0, int na, int nb, int ignore_vignetted, double* out_re,
                                 double* out_im, void* stream);

/* Allocation-free bt_huygens_amplitudes (no counterpart in the reference).
 * For callers that may not allocate device memory -- e.g. a host framework
 * that owns all device memory under a fixed budget, or a latency-critical
 * loop that must not trigger cudaMalloc/cudaFree: the scratch lives in a
 * fixed 8 MiB device array inside the library, held by every GPU that loads
 * the library until exit.  Limit: 32 bytes per ray + 16 bytes per pixel must
 * fit in 8 MiB (e.g. 245,760 rays with a 128x128 lattice); larger problems
 * return BT_ERR_ARG with the size needed.  The first call on a device sets
 * up the scratch address (make it before any stream capture); that address
 * is cached and not refreshed after cudaDeviceReset, so do not call this
 * again on a device that was reset.  All calls share the array: calls that
 * overlap on the GPU race. */
int bt_huygens_amplitudes_noalloc(const bt_rayvector* rv, double px, double py, double pz,
                                  const double lat[4], int na, int nb, double t0, int ignore_vignetted,
                                  double* out_re, double* out_im, void* stream);

/* ---- Zernike wavefront fit (batoid/analysis.py:563-573) ------------------
 * Normal equations of nfits independent least-squares fits, one CUDA block
 * per fit.  Fit f uses points [offsets[f], offsets[f+1]) of x, y (pupil
 * coordinates) and v (wavefront values).  basis: jmax polynomials, each a
 * side x side array C[a][b] of x^a y^b coefficients (Z_1..Z_jmax).
 * Outputs G (nfits x jmax x jmax, symmetric) and b (nfits x jmax).  All
 * pointers are device pointers; offsets are int64.  jmax <= 64, side <= 12. */
int bt_zernike_normal_equations(const double* x, const double* y, const double* v, const long long* offsets,
                                int nfits, const double* basis, int jmax, int side, double* G, double* b,
                                void* stream);

/* ---- Batched wavefronts and Zernike fits of perturbed states --------------
 * No single counterpart in the reference.  One call computes, for every
 * (state, field) job of nstates x nfields, what batoid.zernike
 * (batoid/analysis.py:479-573; reference='chief', include_vignetted=False)
 * computes for one optic on top of batoid.wavefront (batoid/analysis.py:
 * 308-388): an nx x nx RayVector.asGrid pupil grid (batoid/rayVector.py:
 * 220-444) traced through the state's optic, moved to the reference sphere
 * of radius sphere_radius around the chief ray's image, OPD in waves, and the
 * least-squares fit of jmax annular Zernike terms to the non-vignetted OPD.
 * All jobs run in one persistent kernel launch.
 *
 * A state differs from the nominal optic in (a) the transforms of the stages
 * listed in var_stages (rigid-body motions: the per-state table replaces
 * them) and (b) an optional bending term sum_m a_m * table_m added to the
 * surface of stage modal_stage, the tables being nmodes bicubic tables on
 * one grid (FP32 device data, layout [iy][ix][q][mode], q = z, dz/dx,
 * dz/dy, d2z/dxdy, nmodes a multiple of 4; the caller keeps it alive).     */
typedef struct bt_batch bt_batch;

typedef struct bt_batch_desc {
    /* nominal optic: the arrays of bt_optic_create (no coatings) */
    size_t nstages;
    const int* kinds;
    const bt_surface* const* surfaces;
    const double* dr;
    const double* drot;
    const bt_medium_h* const* media;
    const bt_obscuration* const* obscurations;
    /* stages whose transform is given per state (at most 8) */
    int nvar;
    const int* var_stages;
    /* bending term (modal_stage = -1: none) */
    int modal_stage;
    double modal_grid[4]; /* x0, y0, dx, dy */
    int modal_nx;
    int modal_ny;
    int nmodes;
    const float* modes;   /* device */
    int modal_use_nan;
    /* flat stop surface: transform from its frame to the rays' input frame */
    double stop_dr[3];
    double stop_drot[9];
    /* reference sphere: a Sphere(-sphere_radius) surface */
    const bt_surface* sphere;
    double sphere_radius;
    /* fit: pupil grid side, annulus of the fit, basis (host array of jmax
     * side x side Cartesian coefficient arrays, as for the normal equations) */
    double pupil_size;
    double r_inner;
    double r_outer;
    int jmax;             /* <= 32 */
    const double* basis;
    int side;
} bt_batch_desc;

int bt_batch_create(const bt_batch_desc* desc, bt_batch** out);
void bt_batch_destroy(bt_batch* b);
/* Builds the fit tables of the given grid sizes (2 <= nx <= 512; host
 * array).  Synchronous; call before bt_batch_zernike uses those sizes. */
int bt_batch_prepare(bt_batch* b, int n, const int* nx_values, void* stream);
/* Device arrays, per state s: xf[s][nvar][12] (dr(3), drot(9) of each varying
 * stage), det[s][12] (origin(3), rot(9) row-major of the last stage's
 * frame), amps[s][nmodes], nx[s], wavelength[s]; per field f: fields[f][18]
 * (back-propagation frame dr(3), rot(9), local velocity(3), velocity(3) as
 * batoid's finishParallel takes them); order[nqueue] = the job ids
 * s*nfields+f to run, in scheduling order (nqueue <= 0: all nstates*nfields
 * jobs, order holding each once).  Outputs coefs[job][jmax+1] (waves, entry
 * 0 = 0) and status[job] (0, BT_ERR_ARG for a grid size not prepared,
 * BT_ERR_RANK, -1 if not run).  threads: 32..256, a multiple of 32;
 * ctas_per_sm 1..8.  With fewer jobs than thread blocks (SMs x
 * ctas_per_sm) each job's rays are split over several blocks; results are
 * the same.  Stream-ordered. */
int bt_batch_zernike(bt_batch* b, int nstates, const double* xf, const double* det, const double* amps,
                     const int* nx, const double* wavelength, int nfields, const double* fields,
                     const int* order, int nqueue, double* coefs, int* status, int threads, int ctas_per_sm,
                     int niter, void* stream);
/* Same, replayed from a CUDA graph captured on the first call with these
 * arguments (recaptured when they change).  stream must not be the legacy
 * default stream. */
int bt_batch_zernike_graph(bt_batch* b, int nstates, const double* xf, const double* det, const double* amps,
                           const int* nx, const double* wavelength, int nfields, const double* fields,
                           const int* order, int nqueue, double* coefs, int* status, int threads,
                           int ctas_per_sm, int niter, void* stream);

/* ---- Wavefront surrogate MLP (BF16 tensor cores) -------------------------
 * No counterpart in the reference.  Building blocks of the training and
 * inference of the surrogate network that maps perturbation dofs, field
 * and wavelength to Zernike coefficients; all pointers are device pointers,
 * bf16 arrays are 16-byte aligned row-major, all calls stream-ordered.
 *
 * C[M x N] = A[M x K] . B[N x K]^T with A, B bf16 (K contiguous), FP32
 * accumulation in tensor memory (tcgen05.mma), fused epilogue `mode`:
 *   0: out32[kz][m][n] = partial sum of K-split kz (splitk splits)
 *   1: out32[m][n] = acc + bias[n]
 *   2: zs[m][n] = acc + bias[n] (zs may be null); h16[m][n] = h16t[n][m] =
 *      bf16(gelu(zs)) (h16t may be null)
 *   3: h16[m][n] = h16t[n][m] = bf16(acc * gelu'(zs[m][n]))
 * M a multiple of 128; bn 128 or 256 dividing N; K a multiple of 64*splitk. */
int bt_mlp_gemm(const void* A, const void* B, int M, int N, int K, int bn, int splitk, int mode, const float* bias,
                float* out32, float* zs, void* h16, void* h16t, void* stream);
/* FP32 features x[rows][cols] -> bf16 out[rows_out][ld_out] (zero padded)
 * and its transpose out_t[ld_out][rows_out] (may be null). */
int bt_mlp_pack(const float* x, int rows, int cols, int ld_out, int rows_out, void* out, void* out_t, void* stream);
/* Gradient of the mean (over rows_valid rows) of sum_j wt[j] (y - t)^2 over
 * columns j < ncols, and of the squared error of column err_col (if >= 0)
 * against the detached target log sqrt(sum_j (y - t)^2), weighted by
 * err_weight; written as bf16 dz[rows][ld_out] and dzt[ld_out][rows].
 * loss[0], loss[1] (may be null) accumulate the two terms. */
int bt_mlp_loss(const float* y, int ldy, const float* t, const float* wt, int rows, int rows_valid, int ncols,
                int err_col, float err_weight, int ld_out, void* dz, void* dzt, float* loss, void* stream);
/* out[r] = sum_c xt[r][c] of a bf16 [rows][cols] array (bias gradients). */
int bt_mlp_colsum(const void* xt, int rows, int cols, float* out, void* stream);
/* One Adam step of n FP32 parameters w (moments m, v; bias corrections
 * bc1 = 1 - b1^t, bc2 = 1 - b2^t) with gradient grad (may be null) plus the
 * sum of nsplit partial gradients (partials, [nsplit][n], may be null);
 * refreshes the bf16 copies w16 [rows][cols] and w16t [cols][rows] (either
 * may be null). */
int bt_mlp_adam(const float* partials, int nsplit, const float* grad, long long n, float* w, float* m, float* v,
                float lr, float b1, float b2, float eps, float bc1, float bc2, int rows, int cols, void* w16,
                void* w16t, void* stream);
/* bt_mlp_adam with {lr, bc1, bc2} read from the device array hyper[3] when
 * the kernel runs, so that a training step captured in a CUDA graph follows
 * a learning-rate schedule and bias corrections computed on the device. */
int bt_mlp_adam_dev(const float* partials, int nsplit, const float* grad, long long n, float* w, float* m, float* v,
                    const float* hyper, float b1, float b2, float eps, int rows, int cols, void* w16, void* w16t,
                    void* stream);

/* Surrogate output assembly: for sample s in group grp[s], Zernike
 * coefficients out[s][0..J] (waves; entry 0 = 0) = linear model
 * theta[grp][0][j] + sum_k theta[grp][1+k][j] feat[s][k] (k < nlin; theta
 * is [groups][nlin+1][J] float-float pairs (hi, lo), 8-byte aligned, with
 * hi + lo the FP64 coefficient; evaluated to ~48 bits on the FP32 pipe)
 * plus the network's residual y[s][j] (nm
 * divided by `scale`) converted to waves at wl[s]; err_nm[s] (may be null)
 * = scale * exp(y[s][err_col]), the predicted residual norm in nm. */
int bt_surrogate_combine(const float* feat, int nfeat, int nlin, const int* grp, const float* theta, const float* y,
                         int ldy, const double* wl, double scale, int J, int err_col, double* out, float* err_nm,
                         int n, void* stream);

/* Start of a training step captured in a CUDA graph (no reference
 * counterpart): rows perm[k * batch + b] (k = *k_in_epoch, read on the
 * device) of x_all [.][nxc] and t_all [.][ntc] into xb [batch][nxc] and
 * tb [batch][ntc]. */
int bt_mlp_gather(const long long* perm, const long long* k_in_epoch, const float* x_all, int nxc,
                  const float* t_all, int ntc, int batch, float* xb, float* tb, void* stream);

/* Copies hyper[0..3) = table[3 g .. 3 g + 3) for step g = *step (clamped
 * to total - 1): the {learning rate, Adam bias corrections} of each step,
 * tabulated on the host, into the array bt_mlp_adam_dev reads; then
 * advances *step and *k_in_epoch by one. */
int bt_mlp_schedule(long long* k_in_epoch, long long* step, const float* table, long long total, float* hyper,
                    void* stream);

/* Vignetting guard of the surrogate (no reference counterpart): for sample s
 * in group grp[s], with z = feat[s][0..ndof) (normalised dofs), the kept
 * aperture margins of its group m = m0[g][k] + sum_d jac[g][d][k] z[d]
 * (m0: [groups][K], K a multiple of 32, entries >= 1e38 unused; jac:
 * [groups][ndof][K]); flag[s] = 1 when any m has the opposite sign of m0[g][k]
 * or |m| < band_abs + band_rel * |m - m0[g][k]|, or when reach (may be null;
 * [ndof]) is given and some |z[d]| > reach[d]; else 0. */
int bt_surrogate_guard(const float* feat, int nfeat, int ndof, const int* grp, const float* m0, const float* jac,
                       const float* reach, int K, double band_abs, double band_rel, int* flag, int n, void* stream);

/* Measures the device's FP64 FMA throughput (TFLOP/s, 2 flops per FMA)
 * with independent DFMA chains; `iters` FMAs per chain (e.g. 1 << 14).
 * The denominator of the tracer's FP64 roofline.  Synchronous. */
int bt_measure_fp64_peak(int iters, double* tflops, void* stream);

/* The same for the FP32 pipe (independent FFMA chains, 2 flops per FMA):
 * the denominator of the Huygens phasor sums' roofline.  Synchronous. */
int bt_measure_fp32_peak(int iters, double* tflops, void* stream);

/* Reads and clears the device status word of the blob-staging kernels:
 * BT_ERR_TIMEOUT if a kernel's bounded wait for its descriptor copy expired
 * (that kernel then left every ray untouched).  Synchronous. */
int bt_check_device_status(void* stream);

#ifdef __cplusplus
}
#endif
#endif /* BATOID_GB300_H */
