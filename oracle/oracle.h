/*
 * ORACLE — test infrastructure only.  Plain-C CPU restatement of the
 * reference's per-ray trace algorithm (jmeyers314/batoid, src/ C++ files), used
 * by the tests as the checker of the CUDA path and by bench.py as the timed
 * CPU baseline ("port").  Nothing in the product links or calls it.
 *
 * Each function cites the reference file:line it restates.  Data structures
 * are plain tagged structs (no virtual dispatch); the arithmetic and its
 * order follow the reference expressions.
 */
#ifndef BT_ORACLE_H
#define BT_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORA_PLANE = 0, ORA_TILTED, ORA_SPHERE, ORA_PARABOLOID, ORA_QUADRIC, ORA_ASPHERE, ORA_POLY,
       ORA_BICUBIC, ORA_SUM };

typedef struct ora_surface {
    int kind;
    /* PLANE: -; TILTED: tanx tany; SPHERE/PARABOLOID: R; QUADRIC: R conic;
       ASPHERE: R conic + coefs[ncoef]; POLY: xorigin yorigin + coefs
       [ny][nx], gradx/grady [(ny-1)][(nx-1)]; BICUBIC: x0 y0 dx dy use_nan +
       z/dzdx/dzdy/d2zdxdy [ny][nx]; SUM: children[nchild] */
    double a, b, c, d, e;
    int n, m;
    const double* p0;
    const double* p1;
    const double* p2;
    const double* p3;
    const struct ora_surface* const* children;
    int nchild;
} ora_surface;

enum { ORA_M_CONST = 0, ORA_M_TABLE, ORA_M_SELLMEIER, ORA_M_SUMITA, ORA_M_AIR };
typedef struct ora_medium {
    int kind;
    double p[6];
    const double* args;
    const double* vals;
    int n;
} ora_medium;

enum { ORA_O_CIRCLE = 0, ORA_O_ANNULUS, ORA_O_RECT, ORA_O_RAY, ORA_O_POLYGON, ORA_O_NEG, ORA_O_UNION,
       ORA_O_INTERSECT };
typedef struct ora_obsc {
    int kind;
    double p[6]; /* circle: r x0 y0; annulus: in out x0 y0; rect: w h x0 y0 theta; ray: w theta x0 y0 */
    const double* xs;
    const double* ys;
    int n;
    const struct ora_obsc* const* items;  /* NEG: items[0]; UNION/INTERSECT: items[n] */
} ora_obsc;

typedef struct ora_rv {
    double *x, *y, *z, *vx, *vy, *vz, *t, *w, *f;
    uint8_t *vig, *fail;
    size_t n;
} ora_rv;

double ora_sag(const ora_surface* s, double x, double y);
void ora_normal(const ora_surface* s, double x, double y, double* nx, double* ny, double* nz);
double ora_getN(const ora_medium* m, double w);
int ora_contains(const ora_obsc* o, double x, double y);

void ora_intersect(const ora_surface* s, const double* dr, const double* drot, ora_rv* rv, const double* coatRT,
                   int threads, int niter);
void ora_reflect(const ora_surface* s, const double* dr, const double* drot, ora_rv* rv, const double* coatRT,
                 int threads, int niter);
void ora_refract(const ora_surface* s, const double* dr, const double* drot, const ora_medium* m2, ora_rv* rv,
                 const double* coatRT, int threads, int niter);
void ora_obscure(const ora_obsc* o, ora_rv* rv, int threads);
void ora_forward_transform(const double* dr, const double* drot, ora_rv* rv, int threads);
void ora_reverse_transform(const double* dr, const double* drot, ora_rv* rv, int threads);
void ora_position_at_time(const ora_rv* rv, double t, double* xo, double* yo, double* zo, int threads);
void ora_propagate(ora_rv* rv, double t, int threads);
void ora_phase(const ora_rv* rv, double x, double y, double z, double t, double* out, int threads);
void ora_sum_amplitude(const ora_rv* rv, double x, double y, double z, double t, int ignore_vig, int threads,
                       double* out2);
void ora_finish_parallel(const double* dr, const double* drot, const double* vv, double* x, double* y, double* z,
                         size_t n);
void ora_sag_array(const ora_surface* s, const double* x, const double* y, double* out, size_t n);
void ora_normal_array(const ora_surface* s, const double* x, const double* y, double* out, size_t n);
int ora_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
