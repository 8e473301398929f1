/*
 * ORACLE — test infrastructure only (see oracle.h).  CPU restatement of the
 * reference's per-ray algorithm; every function names the reference
 * file:line it follows.  OpenMP over rays, as the reference.
 */
#include "oracle.h"

#include <math.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int ora_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---- polynomial helpers: src/polynomialSurface.cpp:50-66 ---------------- */
static double horner(double x, const double* c, int n) {
    double r = 0.0;
    for (int i = n - 1; i >= 0; i--) {
        r *= x;
        r += c[i];
    }
    return r;
}

static double horner2d(double x, double y, const double* c, int nx, int ny) {
    double r = 0.0;
    for (int i = ny - 1; i >= 0; i--) {
        r *= x;
        r += horner(y, c + i * nx, nx);
    }
    return r;
}

/* ---- table: src/table.cpp:42-158 ------------------------------------------ */
static double spline1(double x, double v0, double v1, double d0, double d1) {
    double a = 2 * (v0 - v1) + d0 + d1;
    double b = 3 * (v1 - v0) - 2 * d0 - d1;
    double c = d0;
    double d = v0;
    return d + x * (c + x * (b + x * a));
}

static double grad1(double x, double v0, double v1, double d0, double d1) {
    double a = 2 * (v0 - v1) + d0 + d1;
    double b = 3 * (v1 - v0) - 2 * d0 - d1;
    double c = d0;
    return c + x * (2 * b + x * 3 * a);
}

/* cell index as the reference computes int(floor(...)); NaN / huge -> outside */
static int cell(double v, double v0, double dv, int nmax, int* idx) {
    double f = floor((v - v0) / dv);
    if (!(f >= 0.0) || f >= (double)(nmax - 1)) return 0;
    *idx = (int)f;
    return 1;
}

static double table_eval(const ora_surface* s, double x, double y) {
    const double x0 = s->a, y0 = s->b, dx = s->c, dy = s->d;
    const int nx = s->n, ny = s->m;
    int ix, iy;
    if (!cell(x, x0, dx, nx, &ix) || !cell(y, y0, dy, ny, &iy)) return s->e != 0.0 ? NAN : 0.0;
    const double *Z = s->p0, *ZX = s->p1, *ZY = s->p2, *ZXY = s->p3;
    double xgrid = x0 + ix * dx;
    double ygrid = y0 + iy * dy;
    double xfrac = (x - xgrid) / dx;
    double yfrac = (y - ygrid) / dy;
    double val0 = spline1(xfrac, Z[nx * iy + ix], Z[nx * iy + ix + 1], ZX[nx * iy + ix] * dx,
                          ZX[nx * iy + ix + 1] * dx);
    double val1 = spline1(xfrac, Z[nx * (iy + 1) + ix], Z[nx * (iy + 1) + ix + 1], ZX[nx * (iy + 1) + ix] * dx,
                          ZX[nx * (iy + 1) + ix + 1] * dx);
    double der0 = spline1(xfrac, ZY[nx * iy + ix], ZY[nx * iy + ix + 1], ZXY[nx * iy + ix] * dx,
                          ZXY[nx * iy + ix + 1] * dx);
    double der1 = spline1(xfrac, ZY[nx * (iy + 1) + ix], ZY[nx * (iy + 1) + ix + 1], ZXY[nx * (iy + 1) + ix] * dx,
                          ZXY[nx * (iy + 1) + ix + 1] * dx);
    return spline1(yfrac, val0, val1, der0 * dy, der1 * dy);
}

static void table_grad(const ora_surface* s, double x, double y, double* dzdx, double* dzdy) {
    const double x0 = s->a, y0 = s->b, dx = s->c, dy = s->d;
    const int nx = s->n, ny = s->m;
    int ix, iy;
    if (!cell(x, x0, dx, nx, &ix) || !cell(y, y0, dy, ny, &iy)) {
        double f = s->e != 0.0 ? NAN : 0.0;
        *dzdx = f;
        *dzdy = f;
        return;
    }
    const double *Z = s->p0, *ZX = s->p1, *ZY = s->p2, *ZXY = s->p3;
    double xfrac = (x - (x0 + ix * dx)) / dx;
    double yfrac = (y - (y0 + iy * dy)) / dy;
    int i00 = nx * iy + ix, i01 = i00 + 1, i10 = i00 + nx, i11 = i10 + 1;
    double val0 = grad1(xfrac, Z[i00], Z[i01], ZX[i00] * dx, ZX[i01] * dx);
    double val1 = grad1(xfrac, Z[i10], Z[i11], ZX[i10] * dx, ZX[i11] * dx);
    double der0 = grad1(xfrac, ZY[i00], ZY[i01], ZXY[i00] * dx, ZXY[i01] * dx);
    double der1 = grad1(xfrac, ZY[i10], ZY[i11], ZXY[i10] * dx, ZXY[i11] * dx);
    *dzdx = spline1(yfrac, val0, val1, der0 * dy, der1 * dy) / dx;
    val0 = grad1(yfrac, Z[i00], Z[i10], ZY[i00] * dy, ZY[i10] * dy);
    val1 = grad1(yfrac, Z[i01], Z[i11], ZY[i01] * dy, ZY[i11] * dy);
    der0 = grad1(yfrac, ZX[i00], ZX[i10], ZXY[i00] * dy, ZXY[i10] * dy);
    der1 = grad1(yfrac, ZX[i01], ZX[i11], ZXY[i01] * dy, ZXY[i11] * dy);
    *dzdy = spline1(xfrac, val0, val1, der0 * dx, der1 * dx) / dy;
}

/* ---- sag: src/{plane,tilted,sphere,paraboloid,quadric,asphere,
 *      polynomialSurface,bicubic,sum}.cpp -------------------------------------- */
static double quadric_sag(double R, double conic, double x, double y) {
    /* src/quadric.cpp:18-26 with the constructor's constants (:9-14) */
    double cp1 = conic + 1;
    double cp1RR = cp1 / R / R;
    double r2 = x * x + y * y;
    if (R != 0) return r2 / (R * (1. + sqrt(1. - r2 * cp1RR)));
    return 0.0;
}

static double quadric_dzdr(double R, double conic, double r) {
    /* src/quadric.cpp:73-77 */
    double cp1RR = (conic + 1) / R / R;
    if (R != 0.0) return r / (R * sqrt(1 - r * r * cp1RR));
    return 0.0;
}

double ora_sag(const ora_surface* s, double x, double y) {
    switch (s->kind) {
    case ORA_PLANE:
        return 0.0; /* src/plane.cpp:17-19 */
    case ORA_TILTED:
        return x * s->a + y * s->b; /* src/tilted.cpp:14-16 */
    case ORA_SPHERE: {
        /* src/sphere.cpp:15-19 */
        double R = s->a;
        if (R != 0) return R * (1 - sqrt(1 - (x * x + y * y) * (1. / R / R)));
        return 0.0;
    }
    case ORA_PARABOLOID: {
        /* src/paraboloid.cpp:15-21 */
        double R = s->a;
        if (R != 0) return (x * x + y * y) * (1. / 2 / R);
        return 0.0;
    }
    case ORA_QUADRIC:
        return quadric_sag(s->a, s->b, x, y);
    case ORA_ASPHERE: {
        /* src/asphere.cpp:37-46 */
        double r2 = x * x + y * y;
        double rr = 1.0;
        double result = quadric_sag(s->a, s->b, x, y);
        for (int i = 0; i < s->n; i++) {
            rr *= r2;
            result += s->p0[i] * rr;
        }
        return result;
    }
    case ORA_POLY:
        /* src/polynomialSurface.cpp:35-37 */
        return horner2d(x - s->a, y - s->b, s->p0, s->n, s->m);
    case ORA_BICUBIC:
        return table_eval(s, x, y); /* src/bicubic.cpp:19-21 */
    case ORA_SUM: {
        /* src/sum.cpp:23-28 */
        double r = 0.0;
        for (int i = 0; i < s->nchild; i++) r += ora_sag(s->children[i], x, y);
        return r;
    }
    }
    return NAN;
}

void ora_normal(const ora_surface* s, double x, double y, double* nx, double* ny, double* nz) {
    switch (s->kind) {
    case ORA_PLANE:
        *nx = 0.0; *ny = 0.0; *nz = 1.0; /* src/plane.cpp:21-25 */
        return;
    case ORA_TILTED:
        /* src/tilted.cpp:18-27 */
        *nx = -s->a;
        *ny = -s->b;
        *nz = sqrt(1 - s->a * s->a - s->b * s->b);
        return;
    case ORA_SPHERE: {
        /* src/sphere.cpp:21-34, 69-72 */
        double R = s->a;
        double rsqr = x * x + y * y;
        if (R == 0.0 || rsqr == 0.0) {
            *nx = 0.0; *ny = 0.0; *nz = 1.0;
        } else {
            double r = sqrt(rsqr);
            double rat = r * (1. / R);
            double dzdr = rat / sqrt(1 - rat * rat);
            *nz = 1 / sqrt(1 + dzdr * dzdr);
            *nx = -x / r * dzdr * *nz;
            *ny = -y / r * dzdr * *nz;
        }
        return;
    }
    case ORA_PARABOLOID: {
        /* src/paraboloid.cpp:23-36 */
        double R = s->a;
        if (R == 0) {
            *nx = 0.0; *ny = 0.0; *nz = 1.0;
        } else {
            double Rinv = 1. / R;
            *nz = 1 / sqrt(1 + (x * x + y * y) * Rinv * Rinv);
            *nx = -x * Rinv * *nz;
            *ny = -y * Rinv * *nz;
        }
        return;
    }
    case ORA_QUADRIC:
    case ORA_ASPHERE: {
        /* src/quadric.cpp:28-39, src/asphere.cpp:48-74 */
        double r = sqrt(x * x + y * y);
        if (r == 0.0) {
            *nx = 0.0; *ny = 0.0; *nz = 1.0;
            return;
        }
        double dzdr = quadric_dzdr(s->a, s->b, r);
        if (s->kind == ORA_ASPHERE) {
            double rr = r * r;
            double rrr = r;
            for (int i = 0; i < s->n; i++) {
                dzdr += s->p0[i] * (2 * (i + 1)) * rrr;
                rrr *= rr;
            }
        }
        *nz = 1 / sqrt(1 + dzdr * dzdr);
        *nx = -x / r * dzdr * *nz;
        *ny = -y / r * dzdr * *nz;
        return;
    }
    case ORA_POLY: {
        /* src/polynomialSurface.cpp:39-48 */
        double gx = -horner2d(x - s->a, y - s->b, s->p1, s->n - 1, s->m - 1);
        double gy = -horner2d(x - s->a, y - s->b, s->p2, s->n - 1, s->m - 1);
        *nz = 1. / sqrt(gx * gx + gy * gy + 1);
        *nx = gx * *nz;
        *ny = gy * *nz;
        return;
    }
    case ORA_BICUBIC: {
        /* src/bicubic.cpp:23-40 */
        double dx, dy;
        table_grad(s, x, y, &dx, &dy);
        if (isnan(dx)) {
            *nx = NAN; *ny = NAN; *nz = NAN;
            return;
        }
        *nz = 1 / sqrt(1 + dx * dx + dy * dy);
        *nx = -dx * *nz;
        *ny = -dy * *nz;
        return;
    }
    case ORA_SUM: {
        /* src/sum.cpp:30-45 */
        double sx = 0.0, sy = 0.0;
        for (int i = 0; i < s->nchild; i++) {
            double tx, ty, tz;
            ora_normal(s->children[i], x, y, &tx, &ty, &tz);
            sx += tx / tz;
            sy += ty / tz;
        }
        *nz = 1. / sqrt(sx * sx + sy * sy + 1);
        *nx = sx * *nz;
        *ny = sy * *nz;
        return;
    }
    }
    *nx = NAN; *ny = NAN; *nz = NAN;
}

/* ---- intersections --------------------------------------------------------- */
/* Newton iteration, src/surface.cpp:22-49 */
static int newton(const ora_surface* s, double x, double y, double z, double vx, double vy, double vz, double* dt,
                  int niter) {
    double rPx = x + vx * *dt;
    double rPy = y + vy * *dt;
    double rPz = z + vz * *dt;
    double sz = ora_sag(s, rPx, rPy);
    for (int iter = 0; iter < niter; iter++) {
        double nx, ny, nz;
        ora_normal(s, rPx, rPy, &nx, &ny, &nz);
        *dt = (rPx - x) * nx + (rPy - y) * ny + (sz - z) * nz;
        *dt /= (nx * vx + ny * vy + nz * vz);
        rPx = x + vx * *dt;
        rPy = y + vy * *dt;
        rPz = z + vz * *dt;
        sz = ora_sag(s, rPx, rPy);
    }
    return fabs(sz - rPz) < 1e-12;
}

static int roots(double a, double b, double c, double* dt1, double* dt2) {
    double disc = b * b - 4 * a * c;
    if (disc < 0) return 0;
    if (b > 0)
        *dt1 = (-b - sqrt(disc)) / (2 * a);
    else
        *dt1 = 2 * c / (-b + sqrt(disc));
    *dt2 = c / (a * *dt1);
    return 1;
}

static int tti(const ora_surface* s, double x, double y, double z, double vx, double vy, double vz, double* dt,
               int niter) {
    switch (s->kind) {
    case ORA_PLANE:
        /* src/plane.cpp:27-33 */
        if (vz == 0) return 0;
        *dt = -z / vz;
        return 1;
    case ORA_TILTED: {
        /* src/tilted.cpp:29-37 */
        double num = z - x * s->a - y * s->b;
        double den = vx * s->a + vy * s->b - vz;
        if (den == 0) return 0;
        *dt = num / den;
        return 1;
    }
    case ORA_SPHERE: {
        /* src/sphere.cpp:36-67 */
        double R = s->a;
        double vr2 = vx * vx + vy * vy;
        double vz2 = vz * vz;
        double vrr0 = vx * x + vy * y;
        double r02 = x * x + y * y;
        double z0term = z - R;
        double a = vz2 + vr2;
        double b = 2 * vz * z0term + 2 * vrr0;
        double c = z0term * z0term - R * R + r02;
        double t1, t2;
        if (!roots(a, b, c, &t1, &t2)) return 0;
        *dt = (vz * R < 0) ? fmax(t1, t2) : fmin(t1, t2);
        return 1;
    }
    case ORA_PARABOLOID: {
        /* src/paraboloid.cpp:38-71 */
        double R = s->a;
        double Rinv = 1. / R, tRinv = 1. / 2 / R;
        double a = (vx * vx + vy * vy) * tRinv;
        double b = (x * vx + y * vy) * Rinv - vz;
        double c = (x * x + y * y) * tRinv - z;
        if (a == 0) {
            *dt = -c / b;
            return 1;
        }
        double t1, t2;
        if (!roots(a, b, c, &t1, &t2)) return 0;
        *dt = (vz * R < 0) ? fmax(t1, t2) : fmin(t1, t2);
        return 1;
    }
    case ORA_QUADRIC:
    case ORA_ASPHERE: {
        /* src/quadric.cpp:41-71 */
        double R = s->a, cp1 = s->b + 1;
        double cp1inv = 1. / cp1, Rcp1 = R / cp1, RRcp1cp1 = R * R / cp1 / cp1;
        double z0term = z - Rcp1;
        double vrr0 = vx * x + vy * y;
        double a = vz * vz + (vx * vx + vy * vy) * cp1inv;
        double b = 2 * (vz * z0term + vrr0 * cp1inv);
        double c = z0term * z0term - RRcp1cp1 + (x * x + y * y) * cp1inv;
        double t1, t2;
        if (!roots(a, b, c, &t1, &t2)) return 0;
        double z1 = z + vz * t1;
        double z2 = z + vz * t2;
        *dt = (fabs(z1) < fabs(z2)) ? t1 : t2;
        if (s->kind == ORA_QUADRIC) return 1;
        /* src/asphere.cpp:76-85 */
        return newton(s, x, y, z, vx, vy, vz, dt, niter);
    }
    case ORA_SUM:
        /* src/sum.cpp:47-56 */
        if (!tti(s->children[0], x, y, z, vx, vy, vz, dt, niter)) return 0;
        return newton(s, x, y, z, vx, vy, vz, dt, niter);
    default:
        return newton(s, x, y, z, vx, vy, vz, dt, niter);
    }
}

/* ---- media: src/medium.cpp ------------------------------------------------- */
double ora_getN(const ora_medium* m, double w) {
    switch (m->kind) {
    case ORA_M_CONST:
        return m->p[0]; /* :30-32 */
    case ORA_M_TABLE: {
        /* :89-105 */
        if (w < m->args[0]) return NAN;
        if (w > m->args[m->n - 1]) return NAN;
        if (m->n < 2) return m->vals[0];
        int u;
        for (u = 1; u < m->n; u++)
            if (w < m->args[u]) break;
        if (u >= m->n) u = m->n - 1;
        double out = (w - m->args[u - 1]);
        out *= (m->vals[u] - m->vals[u - 1]);
        out /= (m->args[u] - m->args[u - 1]);
        out += m->vals[u - 1];
        return out;
    }
    case ORA_M_SELLMEIER: {
        /* :145-149 */
        double x = w * w * 1e12;
        return sqrt(1.0 + m->p[0] * x / (x - m->p[3]) + m->p[1] * x / (x - m->p[4]) + m->p[2] * x / (x - m->p[5]));
    }
    case ORA_M_SUMITA: {
        /* :186-191 */
        double x = w * w * 1e12;
        double y = 1. / x;
        return sqrt(m->p[0] + m->p[1] * x + y * (m->p[2] + y * (m->p[3] + y * (m->p[4] + y * m->p[5]))));
    }
    case ORA_M_AIR: {
        /* :230-245; p = (pressure kPa, temperature K, h2o kPa) */
        double P = m->p[0] * 7.50061683, T = m->p[1] - 273.15, W = m->p[2] * 7.50061683;
        double s2 = 1e-12 / (w * w);
        double nm1 = (64.328 + (29498.1 / (146.0 - s2)) + (255.4 / (41.0 - s2))) * 1.e-6;
        nm1 *= P * (1.0 + (1.049 - 0.0157 * T) * 1.e-6 * P) / (720.883 * (1.0 + 0.003661 * T));
        nm1 -= (0.0624 - 0.000680 * s2) / (1.0 + 0.003661 * T) * W * 1.e-6;
        return 1 + nm1;
    }
    }
    return NAN;
}

/* ---- obscurations: src/obscuration.cpp ------------------------------------- */
int ora_contains(const ora_obsc* o, double x, double y) {
    switch (o->kind) {
    case ORA_O_CIRCLE:
        return hypot(x - o->p[1], y - o->p[2]) < o->p[0]; /* :32-34 */
    case ORA_O_ANNULUS: {
        double h = hypot(x - o->p[2], y - o->p[3]); /* :80-83 */
        return (o->p[0] <= h) && (h < o->p[1]);
    }
    case ORA_O_RECT: {
        /* :117-121 */
        double sth = sin(o->p[4]), cth = cos(o->p[4]);
        double xp = (x - o->p[2]) * cth + (y - o->p[3]) * sth;
        double yp = -(x - o->p[2]) * sth + (y - o->p[3]) * cth;
        return (xp > -o->p[0] / 2 && xp < o->p[0] / 2 && yp > -o->p[1] / 2 && yp < o->p[1] / 2);
    }
    case ORA_O_RAY: {
        /* :155-159 */
        double sth = sin(o->p[1]), cth = cos(o->p[1]);
        double xp = (x - o->p[2]) * cth + (y - o->p[3]) * sth;
        double yp = -(x - o->p[2]) * sth + (y - o->p[3]) * cth;
        return (xp > 0.0 && yp > -o->p[0] / 2 && yp < o->p[0] / 2);
    }
    case ORA_O_POLYGON: {
        /* :201-225 */
        double x1 = o->xs[0], y1 = o->ys[0];
        double xinters = 0.0;
        int inside = 0;
        for (int i = 1; i <= o->n; i++) {
            double x2 = o->xs[i % o->n], y2 = o->ys[i % o->n];
            if (y > fmin(y1, y2)) {
                if (y <= fmax(y1, y2)) {
                    if (x <= fmax(x1, x2)) {
                        if (y1 != y2) xinters = (y - y1) * (x2 - x1) / (y2 - y1) + x1;
                        if (x1 == x2 || x <= xinters) inside = !inside;
                    }
                }
            }
            x1 = x2;
            y1 = y2;
        }
        return inside;
    }
    case ORA_O_NEG:
        return !ora_contains(o->items[0], x, y); /* :320-322 */
    case ORA_O_UNION: {
        int r = 0; /* :364-370 */
        for (int i = 0; i < o->n; i++) r |= ora_contains(o->items[i], x, y);
        return r;
    }
    case ORA_O_INTERSECT: {
        int r = 1; /* :415-421 */
        for (int i = 0; i < o->n; i++) r &= ora_contains(o->items[i], x, y);
        return r;
    }
    }
    return 0;
}

/* ---- trace loops: src/batoid.cpp:151-506 ----------------------------------- */
#define XFORM()                                                     \
    double dx = rv->x[i] - dr[0];                                   \
    double dy = rv->y[i] - dr[1];                                   \
    double dz = rv->z[i] - dr[2];                                   \
    double x = dx * drot[0] + dy * drot[3] + dz * drot[6];          \
    double y = dx * drot[1] + dy * drot[4] + dz * drot[7];          \
    double z = dx * drot[2] + dy * drot[5] + dz * drot[8];          \
    double vx = rv->vx[i] * drot[0] + rv->vy[i] * drot[3] + rv->vz[i] * drot[6]; \
    double vy = rv->vx[i] * drot[1] + rv->vy[i] * drot[4] + rv->vz[i] * drot[7]; \
    double vz = rv->vx[i] * drot[2] + rv->vy[i] * drot[5] + rv->vz[i] * drot[8]; \
    double t = rv->t[i];

void ora_intersect(const ora_surface* s, const double* dr, const double* drot, ora_rv* rv, const double* coatRT,
                   int threads, int niter) {
    /* src/batoid.cpp:175-270 */
    long long n = (long long)rv->n;
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long i = 0; i < n; i++) {
        XFORM();
        if (!rv->fail[i]) {
            double dt = 0.0;
            if (tti(s, x, y, z, vx, vy, vz, &dt, niter)) {
                x += vx * dt;
                y += vy * dt;
                z += vz * dt;
                t += dt;
                rv->x[i] = x; rv->y[i] = y; rv->z[i] = z;
                rv->vx[i] = vx; rv->vy[i] = vy; rv->vz[i] = vz;
                rv->t[i] = t;
                if (coatRT) rv->f[i] *= coatRT[1];
            } else {
                rv->fail[i] = 1;
                rv->vig[i] = 1;
            }
        }
    }
}

void ora_reflect(const ora_surface* s, const double* dr, const double* drot, ora_rv* rv, const double* coatRT,
                 int threads, int niter) {
    /* src/batoid.cpp:273-378 */
    long long n = (long long)rv->n;
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long i = 0; i < n; i++) {
        XFORM();
        if (!rv->fail[i]) {
            double dt = 0.0;
            if (tti(s, x, y, z, vx, vy, vz, &dt, niter)) {
                x += vx * dt;
                y += vy * dt;
                z += vz * dt;
                t += dt;
                double nx, ny, nz;
                ora_normal(s, x, y, &nx, &ny, &nz);
                double alpha = vx * nx;
                alpha += vy * ny;
                alpha += vz * nz;
                vx -= 2 * alpha * nx;
                vy -= 2 * alpha * ny;
                vz -= 2 * alpha * nz;
                rv->x[i] = x; rv->y[i] = y; rv->z[i] = z;
                rv->vx[i] = vx; rv->vy[i] = vy; rv->vz[i] = vz;
                rv->t[i] = t;
                if (coatRT) rv->f[i] *= coatRT[0];
            } else {
                rv->fail[i] = 1;
                rv->vig[i] = 1;
            }
        }
    }
}

void ora_refract(const ora_surface* s, const double* dr, const double* drot, const ora_medium* m2, ora_rv* rv,
                 const double* coatRT, int threads, int niter) {
    /* src/batoid.cpp:381-506 */
    long long n = (long long)rv->n;
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long i = 0; i < n; i++) {
        XFORM();
        if (!rv->fail[i]) {
            double dt = 0.0;
            if (tti(s, x, y, z, vx, vy, vz, &dt, niter)) {
                x += vx * dt;
                y += vy * dt;
                z += vz * dt;
                t += dt;
                double n1 = vx * vx;
                n1 += vy * vy;
                n1 += vz * vz;
                n1 = 1 / sqrt(n1);
                double nvx = vx * n1, nvy = vy * n1, nvz = vz * n1;
                double nx, ny, nz;
                ora_normal(s, x, y, &nx, &ny, &nz);
                double alpha = nvx * nx;
                alpha += nvy * ny;
                alpha += nvz * nz;
                if (alpha > 0.) {
                    nx *= -1; ny *= -1; nz *= -1;
                    alpha *= -1;
                }
                double n2 = ora_getN(m2, rv->w[i]);
                double eta = n1 / n2;
                double sinsqr = eta * eta * (1 - alpha * alpha);
                rv->x[i] = x; rv->y[i] = y; rv->z[i] = z;
                rv->t[i] = t;
                if (sinsqr > 1.0) {
                    rv->vx[i] = NAN; rv->vy[i] = NAN; rv->vz[i] = NAN;
                    rv->fail[i] = 1;
                    rv->vig[i] = 1;
                } else {
                    double nfactor = eta * alpha + sqrt(1 - sinsqr);
                    rv->vx[i] = eta * nvx - nfactor * nx;
                    rv->vy[i] = eta * nvy - nfactor * ny;
                    rv->vz[i] = eta * nvz - nfactor * nz;
                    rv->vx[i] /= n2;
                    rv->vy[i] /= n2;
                    rv->vz[i] /= n2;
                }
                if (coatRT) rv->f[i] *= coatRT[1];
            } else {
                rv->fail[i] = 1;
                rv->vig[i] = 1;
            }
        }
    }
}

void ora_obscure(const ora_obsc* o, ora_rv* rv, int threads) {
    /* src/batoid.cpp:151-172 */
    long long n = (long long)rv->n;
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long i = 0; i < n; i++) rv->vig[i] |= (uint8_t)ora_contains(o, rv->x[i], rv->y[i]);
}

void ora_forward_transform(const double* dr, const double* drot, ora_rv* rv, int threads) {
    /* src/batoid.cpp:71-108 */
    long long n = (long long)rv->n;
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long i = 0; i < n; i++) {
        double dx = rv->x[i] - dr[0], dy = rv->y[i] - dr[1], dz = rv->z[i] - dr[2];
        rv->x[i] = dx * drot[0] + dy * drot[3] + dz * drot[6];
        rv->y[i] = dx * drot[1] + dy * drot[4] + dz * drot[7];
        rv->z[i] = dx * drot[2] + dy * drot[5] + dz * drot[8];
        double vx = rv->vx[i] * drot[0] + rv->vy[i] * drot[3] + rv->vz[i] * drot[6];
        double vy = rv->vx[i] * drot[1] + rv->vy[i] * drot[4] + rv->vz[i] * drot[7];
        double vz = rv->vx[i] * drot[2] + rv->vy[i] * drot[5] + rv->vz[i] * drot[8];
        rv->vx[i] = vx; rv->vy[i] = vy; rv->vz[i] = vz;
    }
}

void ora_reverse_transform(const double* dr, const double* drot, ora_rv* rv, int threads) {
    /* src/batoid.cpp:111-148 */
    long long n = (long long)rv->n;
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long i = 0; i < n; i++) {
        double x = rv->x[i] * drot[0] + rv->y[i] * drot[1] + rv->z[i] * drot[2] + dr[0];
        double y = rv->x[i] * drot[3] + rv->y[i] * drot[4] + rv->z[i] * drot[5] + dr[1];
        double z = rv->x[i] * drot[6] + rv->y[i] * drot[7] + rv->z[i] * drot[8] + dr[2];
        rv->x[i] = x; rv->y[i] = y; rv->z[i] = z;
        double vx = rv->vx[i] * drot[0] + rv->vy[i] * drot[1] + rv->vz[i] * drot[2];
        double vy = rv->vx[i] * drot[3] + rv->vy[i] * drot[4] + rv->vz[i] * drot[5];
        double vz = rv->vx[i] * drot[6] + rv->vy[i] * drot[7] + rv->vz[i] * drot[8];
        rv->vx[i] = vx; rv->vy[i] = vy; rv->vz[i] = vz;
    }
}

void ora_position_at_time(const ora_rv* rv, double t, double* xo, double* yo, double* zo, int threads) {
    /* src/rayVector.cpp:26-54 */
    long long n = (long long)rv->n;
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long i = 0; i < n; i++) {
        xo[i] = rv->x[i] + rv->vx[i] * (t - rv->t[i]);
        yo[i] = rv->y[i] + rv->vy[i] * (t - rv->t[i]);
        zo[i] = rv->z[i] + rv->vz[i] * (t - rv->t[i]);
    }
}

void ora_propagate(ora_rv* rv, double t, int threads) {
    /* src/rayVector.cpp:56-82 */
    long long n = (long long)rv->n;
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long i = 0; i < n; i++) {
        rv->x[i] += rv->vx[i] * (t - rv->t[i]);
        rv->y[i] += rv->vy[i] * (t - rv->t[i]);
        rv->z[i] += rv->vz[i] * (t - rv->t[i]);
        rv->t[i] = t;
    }
}

static double phase_of(const ora_rv* rv, long long i, double x, double y, double z, double t) {
    /* src/rayVector.cpp:110-121 */
    const double PI = 3.14159265358979323846;
    double v2 = rv->vx[i] * rv->vx[i] + rv->vy[i] * rv->vy[i] + rv->vz[i] * rv->vz[i];
    double out = (x - rv->x[i]) * rv->vx[i];
    out += (y - rv->y[i]) * rv->vy[i];
    out += (z - rv->z[i]) * rv->vz[i];
    out /= v2;
    out -= t - rv->t[i];
    out *= 2 * PI / rv->w[i];
    return out;
}

void ora_phase(const ora_rv* rv, double x, double y, double z, double t, double* out, int threads) {
    long long n = (long long)rv->n;
#pragma omp parallel for num_threads(threads) schedule(static)
    for (long long i = 0; i < n; i++) out[i] = phase_of(rv, i, x, y, z, t);
}

void ora_sum_amplitude(const ora_rv* rv, double x, double y, double z, double t, int ignore_vig, int threads,
                       double* out2) {
    /* src/rayVector.cpp:169-222 */
    long long n = (long long)rv->n;
    double re = 0, im = 0;
#pragma omp parallel for reduction(+ : re, im) num_threads(threads) schedule(static)
    for (long long i = 0; i < n; i++) {
        double ph = phase_of(rv, i, x, y, z, t);
        if (!rv->fail[i] && !(ignore_vig && rv->vig[i])) {
            re += cos(ph) * rv->f[i];
            im += sin(ph) * rv->f[i];
        }
    }
    out2[0] = re;
    out2[1] = im;
}

void ora_finish_parallel(const double* dr, const double* drot, const double* vv, double* X, double* Y, double* Z,
                         size_t n) {
    /* src/batoid.cpp:40-69 */
    double vxl = -vv[0] * drot[0] - vv[1] * drot[3] - vv[2] * drot[6];
    double vyl = -vv[0] * drot[1] - vv[1] * drot[4] - vv[2] * drot[7];
    double vzl = -vv[0] * drot[2] - vv[1] * drot[5] - vv[2] * drot[8];
    for (size_t i = 0; i < n; i++) {
        double dx = X[i] - dr[0], dy = Y[i] - dr[1], dz = Z[i] - dr[2];
        double x = dx * drot[0] + dy * drot[3] + dz * drot[6];
        double y = dx * drot[1] + dy * drot[4] + dz * drot[7];
        double z = dx * drot[2] + dy * drot[5] + dz * drot[8];
        double dt = -z / vzl;
        x += dt * vxl;
        y += dt * vyl;
        z += dt * vzl;
        X[i] = x * drot[0] + y * drot[1] + z * drot[2] + dr[0];
        Y[i] = x * drot[3] + y * drot[4] + z * drot[5] + dr[1];
        Z[i] = x * drot[6] + y * drot[7] + z * drot[8] + dr[2];
    }
}

void ora_sag_array(const ora_surface* s, const double* x, const double* y, double* out, size_t n) {
    for (size_t i = 0; i < n; i++) out[i] = ora_sag(s, x[i], y[i]);
}

void ora_normal_array(const ora_surface* s, const double* x, const double* y, double* out, size_t n) {
    for (size_t i = 0; i < n; i++) ora_normal(s, x[i], y[i], out + i, out + i + n, out + i + 2 * n);
}
