// C-ABI entry points (include/batoid_gb300.h): host-side objects for
// surfaces, media, obscurations and coatings, the packer that flattens them
// into a program blob (bt_desc.h), and the launch wrappers.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>
#include <string>
#include <vector>
#include <mutex>
#include <algorithm>
#include "../../include/batoid_gb300.h"
#include "bt_internal.h"
#include "bt_batch.h"
#include "bt_mlp.h"

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------

static thread_local std::string g_err;

static int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

static int cuda_fail(cudaError_t e, const char* where) {
    return fail(BT_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CUDA_TRY(expr, where)                     \
    do {                                          \
        cudaError_t _e = (expr);                  \
        if (_e != cudaSuccess) return cuda_fail(_e, where); \
    } while (0)

extern "C" const char* bt_last_error(void) { return g_err.c_str(); }
extern "C" int bt_version(void) { return 1; }

extern "C" int bt_device_sm_count(int* out) {
    if (!out) return fail(BT_ERR_ARG, "null out");
    *out = bt_sm_count();
    return BT_OK;
}

// ---------------------------------------------------------------------------
// host objects
// ---------------------------------------------------------------------------

// A bicubic table keeps its host copy and is uploaded to device memory on
// first use by a kernel (so surfaces can be built without touching the GPU).
struct bt_table {
    double x0, y0, dx, dy;
    size_t nx, ny;
    int use_nan;
    std::vector<double> host;  // 4*nx*ny doubles: z, dzdx, dzdy, d2zdxdy
    double* d_tab = nullptr;
    std::mutex mu;
};

// A surface is a small list of descriptors: recs[0] is the root; a Sum's
// children follow it (root.m is the index of the first child, relative).
// pool offsets are relative to `pool`.  tables[i] is the bicubic table of
// recs[i] (nullptr otherwise); tables are shared, not owned.
// Chunk buffers (and streams) of the host-buffer trace pipeline: copies in
// of one chunk, the trace of another and copies out of a third overlap.
#define BT_HOST_PIPE 3

struct bt_surface {
    std::vector<bt_surf> recs;
    std::vector<double> pool;
    std::vector<bt_table*> tables;
};

static cudaError_t table_device(bt_table* t, const double** out) {
    std::lock_guard<std::mutex> lock(t->mu);
    if (!t->d_tab) {
        cudaError_t e = cudaMalloc((void**)&t->d_tab, t->host.size() * sizeof(double));
        if (e != cudaSuccess) { t->d_tab = nullptr; return e; }
        e = cudaMemcpy(t->d_tab, t->host.data(), t->host.size() * sizeof(double), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) { cudaFree(t->d_tab); t->d_tab = nullptr; return e; }
    }
    *out = t->d_tab;
    return cudaSuccess;
}

struct bt_medium_h {
    bt_medium rec;
    std::vector<double> pool;
};

// Postfix obscuration program.
struct bt_obscuration {
    std::vector<bt_obsc> ops;
    std::vector<double> pool;
};

struct bt_coating {
    double R, T;
};

static bt_surf blank_surf(int kind) {
    bt_surf s;
    memset(&s, 0, sizeof(s));
    s.kind = kind;
    s.ffc = -1;
    return s;
}

// A double's float-float split (hi, lo) stored in one double slot.
static double ff_slot(double v) {
    float pair[2];
    pair[0] = (float)v;
    pair[1] = (float)(v - (double)pair[0]);
    double out;
    memcpy(&out, pair, sizeof(out));
    return out;
}

static void append_ff(std::vector<double>& pool, size_t begin, size_t n) {
    for (size_t i = 0; i < n; i++) pool.push_back(ff_slot(pool[begin + i]));
}

// Appends the float-float constants of a record to its surface's pool and
// points the record's ffc at them.
static void push_ffc(bt_surface* s, bt_surf& r, std::initializer_list<double> vals) {
    r.ffc = (int32_t)s->pool.size();
    for (double v : vals) s->pool.push_back(ff_slot(v));
}

static void push_rec(bt_surface* s, const bt_surf& r, bt_table* t = nullptr) {
    s->recs.push_back(r);
    s->tables.push_back(t);
}

template <class T>
static int make_out(T** out, T* obj) {
    if (!out) {
        delete obj;
        return fail(BT_ERR_ARG, "null output handle");
    }
    *out = obj;
    return BT_OK;
}

extern "C" int bt_plane_create(bt_surface** out) {
    bt_surface* s = new bt_surface;
    push_rec(s, blank_surf(BT_S_PLANE));
    return make_out(out, s);
}

extern "C" int bt_tilted_create(double tanx, double tany, bt_surface** out) {
    bt_surface* s = new bt_surface;
    bt_surf r = blank_surf(BT_S_TILTED);
    r.p[0] = tanx;
    r.p[1] = tany;
    r.p[2] = sqrt(1 - tanx * tanx - tany * tany);
    push_rec(s, r);
    return make_out(out, s);
}

extern "C" int bt_sphere_create(double R, bt_surface** out) {
    bt_surface* s = new bt_surface;
    bt_surf r = blank_surf(BT_S_SPHERE);
    // src/sphere.cpp:10-13
    r.p[0] = R;
    r.p[1] = R * R;
    r.p[2] = 1. / R;
    r.p[3] = 1. / R / R;
    push_ffc(s, r, {R, R * R, 1. / R, 1. / R / R});
    push_rec(s, r);
    return make_out(out, s);
}

extern "C" int bt_paraboloid_create(double R, bt_surface** out) {
    bt_surface* s = new bt_surface;
    bt_surf r = blank_surf(BT_S_PARABOLOID);
    // src/paraboloid.cpp:10-12
    r.p[0] = R;
    r.p[1] = 1. / R;
    r.p[2] = 1. / 2 / R;
    push_ffc(s, r, {R, 1. / R, 1. / 2 / R});
    push_rec(s, r);
    return make_out(out, s);
}


static void fill_quadric(bt_surf& r, double R, double conic) {
    // src/quadric.cpp:9-14
    const double cp1 = conic + 1;
    r.p[0] = R;
    r.p[1] = conic;
    r.p[2] = R * R;
    r.p[3] = 1. / R / R;
    r.p[4] = cp1;
    r.p[5] = 1. / cp1;
    r.p[6] = R / cp1;
    r.p[7] = R * R / cp1 / cp1;
    r.p[8] = cp1 / R / R;
    r.p[9] = (R != 0.0) ? 1. / R : 0.0;
    // (1 - q) * R/(1+k) replaces r^2 / (R (1 + q)) when R/(1+k) is moderate:
    // its absolute rounding error is ~|R/(1+k)| ulp(1)
    const double rc = R / cp1;
    r.p[10] = (R != 0.0 && cp1 != 0.0 && isfinite(rc) && fabs(rc) <= 100.0) ? 1.0 : 0.0;
    // FP32 copies of (1+k)/R^2 and 1/R, packed in p[11], for the trace
    // kernel's FP32 Newton pre-step on aspheres
    const float f2[2] = {(float)r.p[8], (float)r.p[9]};
    memcpy(&r.p[11], f2, sizeof(f2));
}

extern "C" int bt_quadric_create(double R, double conic, bt_surface** out) {
    bt_surface* s = new bt_surface;
    bt_surf r = blank_surf(BT_S_QUADRIC);
    fill_quadric(r, R, conic);
    push_ffc(s, r, {r.p[0], r.p[5], r.p[6], r.p[7], r.p[8], r.p[9]});
    push_rec(s, r);
    return make_out(out, s);
}

extern "C" int bt_asphere_create(double R, double conic, const double* coefs, size_t n, bt_surface** out) {
    if (n > 0 && !coefs) return fail(BT_ERR_ARG, "asphere: null coefs");
    bt_surface* s = new bt_surface;
    bt_surf r = blank_surf(BT_S_ASPHERE);
    fill_quadric(r, R, conic);
    r.n = (int32_t)n;
    r.off = 0;
    s->pool.assign(coefs, coefs + n);
    // dz/dr coefficients: entry j multiplies r^(2j+1) with factor 2(j+1)
    // (src/asphere.cpp:10-16)
    for (size_t j = 0; j < n; j++) s->pool.push_back(coefs[j] * (double)(2 * (j + 1)));
    append_ff(s->pool, 0, 2 * n);
    push_ffc(s, r, {r.p[0], r.p[5], r.p[6], r.p[7], r.p[8], r.p[9]});
    push_rec(s, r);
    return make_out(out, s);
}

extern "C" int bt_polynomial_create(const double* coefs, const double* gradx, const double* grady,
                                    double xorigin, double yorigin, size_t xsize, size_t ysize,
                                    bt_surface** out) {
    if (xsize < 1 || ysize < 1 || !coefs) return fail(BT_ERR_ARG, "polynomial: bad coefficient array");
    const size_t gsz = (xsize - 1) * (ysize - 1);
    if (gsz > 0 && (!gradx || !grady)) return fail(BT_ERR_ARG, "polynomial: null gradient arrays");
    bt_surface* s = new bt_surface;
    bt_surf r = blank_surf(BT_S_POLY);
    r.p[0] = xorigin;
    r.p[1] = yorigin;
    r.n = (int32_t)xsize;
    r.m = (int32_t)ysize;
    r.off = 0;
    s->pool.assign(coefs, coefs + xsize * ysize);
    if (gsz > 0) {
        s->pool.insert(s->pool.end(), gradx, gradx + gsz);
        s->pool.insert(s->pool.end(), grady, grady + gsz);
    }
    append_ff(s->pool, 0, xsize * ysize + 2 * gsz);
    push_ffc(s, r, {xorigin, yorigin});
    // p2 = 1: square arrays whose coefficients with i + j >= K are zero (the
    // Cartesian form of a Zernike sum); the trace then skips those terms
    bool tri = xsize == ysize && xsize >= 2;
    for (size_t i = 0; tri && i < ysize; i++)
        for (size_t j = 0; j < xsize; j++) {
            if (i + j >= xsize && coefs[i * xsize + j] != 0.0) tri = false;
            if (i < ysize - 1 && j < xsize - 1 && i + j >= xsize - 1 &&
                (gradx[i * (xsize - 1) + j] != 0.0 || grady[i * (xsize - 1) + j] != 0.0))
                tri = false;
        }
    r.p[2] = tri ? 1.0 : 0.0;
    push_rec(s, r);
    return make_out(out, s);
}

extern "C" int bt_table_create(double x0, double y0, double dx, double dy, const double* z, const double* dzdx,
                               const double* dzdy, const double* d2zdxdy, size_t nx, size_t ny, int use_nan,
                               bt_table** out) {
    if (!z || !dzdx || !dzdy || !d2zdxdy || nx < 2 || ny < 2) return fail(BT_ERR_ARG, "table: bad arrays");
    bt_table* t = new bt_table;
    t->x0 = x0; t->y0 = y0; t->dx = dx; t->dy = dy;
    t->nx = nx; t->ny = ny; t->use_nan = use_nan ? 1 : 0;
    const size_t plane = nx * ny;
    const double* src[4] = {z, dzdx, dzdy, d2zdxdy};
    t->host.reserve(4 * plane);
    for (int k = 0; k < 4; k++) t->host.insert(t->host.end(), src[k], src[k] + plane);
    return make_out(out, t);
}

extern "C" void bt_table_destroy(bt_table* t) {
    if (!t) return;
    if (t->d_tab) cudaFree(t->d_tab);
    delete t;
}

extern "C" int bt_bicubic_create(const bt_table* t, bt_surface** out) {
    if (!t) return fail(BT_ERR_ARG, "bicubic: null table");
    bt_surface* s = new bt_surface;
    bt_surf r = blank_surf(BT_S_BICUBIC);
    r.p[0] = t->x0; r.p[1] = t->y0; r.p[2] = t->dx; r.p[3] = t->dy;
    r.p[4] = t->use_nan ? 1.0 : 0.0;
    r.n = (int32_t)t->nx;
    r.m = (int32_t)t->ny;
    r.tab = nullptr;  // resolved to the device copy when packed into a program
    push_rec(s, r, const_cast<bt_table*>(t));
    return make_out(out, s);
}

extern "C" int bt_sum_create(const bt_surface* const* surfaces, size_t n, bt_surface** out) {
    if (!surfaces || n < 1) return fail(BT_ERR_ARG, "sum: no surfaces");
    if (n > BT_MAX_SUM_CHILDREN) return fail(BT_ERR_UNSUPPORTED, "sum: too many surfaces");
    for (size_t i = 0; i < n; i++) {
        if (!surfaces[i]) return fail(BT_ERR_ARG, "sum: null surface");
        if (surfaces[i]->recs[0].kind == BT_S_SUM)
            return fail(BT_ERR_UNSUPPORTED, "sum: nested Sum surfaces are not supported");
    }
    bt_surface* s = new bt_surface;
    bt_surf root = blank_surf(BT_S_SUM);
    root.n = (int32_t)n;
    root.m = 1;
    push_rec(s, root);
    for (size_t i = 0; i < n; i++) {
        bt_surf c = surfaces[i]->recs[0];
        if (c.ffc >= 0) c.ffc += (int32_t)s->pool.size();
        c.off += (int32_t)s->pool.size();
        s->pool.insert(s->pool.end(), surfaces[i]->pool.begin(), surfaces[i]->pool.end());
        push_rec(s, c, surfaces[i]->tables[0]);
    }
    return make_out(out, s);
}

extern "C" void bt_surface_destroy(bt_surface* s) { delete s; }

// media ---------------------------------------------------------------------

static bt_medium_h* new_medium(int kind) {
    bt_medium_h* m = new bt_medium_h;
    memset(&m->rec, 0, sizeof(m->rec));
    m->rec.kind = kind;
    return m;
}

extern "C" int bt_const_medium_create(double n, bt_medium_h** out) {
    bt_medium_h* m = new_medium(BT_M_CONST);
    m->rec.p[0] = n;
    m->rec.p[1] = 1.0 / n;  // reciprocal used by the refraction kernels
    m->rec.p[2] = ff_slot(n);
    m->rec.p[3] = ff_slot(1.0 / n);
    return make_out(out, m);
}

extern "C" int bt_table_medium_create(const double* w, const double* ns, size_t n, bt_medium_h** out) {
    if (!w || !ns || n < 1) return fail(BT_ERR_ARG, "table medium: bad arrays");
    bt_medium_h* m = new_medium(BT_M_TABLE);
    m->rec.n = (int32_t)n;
    m->pool.assign(w, w + n);
    m->pool.insert(m->pool.end(), ns, ns + n);
    return make_out(out, m);
}

extern "C" int bt_sellmeier_medium_create(double B1, double B2, double B3, double C1, double C2, double C3,
                                          bt_medium_h** out) {
    bt_medium_h* m = new_medium(BT_M_SELLMEIER);
    double p[6] = {B1, B2, B3, C1, C2, C3};
    memcpy(m->rec.p, p, sizeof(p));
    for (double v : p) m->pool.push_back(ff_slot(v));  // float-float copies at pool[off]
    return make_out(out, m);
}

extern "C" int bt_sumita_medium_create(double A0, double A1, double A2, double A3, double A4, double A5,
                                       bt_medium_h** out) {
    bt_medium_h* m = new_medium(BT_M_SUMITA);
    double p[6] = {A0, A1, A2, A3, A4, A5};
    memcpy(m->rec.p, p, sizeof(p));
    return make_out(out, m);
}

extern "C" int bt_air_create(double pressure, double temperature, double h2o_pressure, bt_medium_h** out) {
    bt_medium_h* m = new_medium(BT_M_AIR);
    // SI inputs converted as src/medium.cpp:230-233
    m->rec.p[0] = pressure * 7.50061683;
    m->rec.p[1] = temperature - 273.15;
    m->rec.p[2] = h2o_pressure * 7.50061683;
    return make_out(out, m);
}

extern "C" void bt_medium_destroy(bt_medium_h* m) { delete m; }

// obscurations --------------------------------------------------------------

static bt_obsc blank_op(int op) {
    bt_obsc o;
    memset(&o, 0, sizeof(o));
    o.op = op;
    return o;
}

static bt_obscuration* leaf_obsc(const bt_obsc& o) {
    bt_obscuration* r = new bt_obscuration;
    r->ops.push_back(o);
    return r;
}

extern "C" int bt_obsc_circle_create(double radius, double x0, double y0, bt_obscuration** out) {
    bt_obsc o = blank_op(BT_O_CIRCLE);
    o.p[0] = radius; o.p[1] = x0; o.p[2] = y0;
    o.p[3] = ff_slot(radius); o.p[4] = ff_slot(x0); o.p[5] = ff_slot(y0);  // float-float copies
    return make_out(out, leaf_obsc(o));
}

extern "C" int bt_obsc_annulus_create(double inner, double outer, double x0, double y0, bt_obscuration** out) {
    bt_obsc o = blank_op(BT_O_ANNULUS);
    o.p[0] = inner; o.p[1] = outer; o.p[2] = x0; o.p[3] = y0;
    o.p[4] = ff_slot(inner); o.p[5] = ff_slot(outer);  // float-float copies
    return make_out(out, leaf_obsc(o));
}

extern "C" int bt_obsc_rectangle_create(double width, double height, double x0, double y0, double theta,
                                        bt_obscuration** out) {
    bt_obsc o = blank_op(BT_O_RECT);
    o.p[0] = width; o.p[1] = height; o.p[2] = x0; o.p[3] = y0;
    o.p[4] = sin(theta); o.p[5] = cos(theta);  // src/obscuration.cpp:110-113
    return make_out(out, leaf_obsc(o));
}

extern "C" int bt_obsc_ray_create(double width, double theta, double x0, double y0, bt_obscuration** out) {
    bt_obsc o = blank_op(BT_O_RAY);
    o.p[0] = width; o.p[1] = x0; o.p[2] = y0;
    o.p[3] = sin(theta); o.p[4] = cos(theta);  // src/obscuration.cpp:148-151
    return make_out(out, leaf_obsc(o));
}

extern "C" int bt_obsc_polygon_create(const double* xs, const double* ys, size_t n, bt_obscuration** out) {
    if (!xs || !ys || n < 1) return fail(BT_ERR_ARG, "polygon: bad vertex arrays");
    bt_obsc o = blank_op(BT_O_POLYGON);
    o.n = (int32_t)n;
    o.off = 0;
    bt_obscuration* r = leaf_obsc(o);
    r->pool.assign(xs, xs + n);
    r->pool.insert(r->pool.end(), ys, ys + n);
    return make_out(out, r);
}

static void append_obsc(bt_obscuration* dst, const bt_obscuration* src) {
    const int32_t base = (int32_t)dst->pool.size();
    for (bt_obsc o : src->ops) {
        if (o.op == BT_O_POLYGON) o.off += base;
        dst->ops.push_back(o);
    }
    dst->pool.insert(dst->pool.end(), src->pool.begin(), src->pool.end());
}

// Maximum operand-stack depth of a postfix program.
static int obsc_depth(const bt_obscuration* o) {
    int sp = 0, mx = 0;
    for (const bt_obsc& op : o->ops) {
        if (op.op == BT_O_NEGATION) sp -= 1;
        else if (op.op == BT_O_UNION || op.op == BT_O_INTERSECTION) sp -= op.n;
        sp += 1;
        if (sp > mx) mx = sp;
    }
    return mx;
}

extern "C" int bt_obsc_negation_create(const bt_obscuration* original, bt_obscuration** out) {
    if (!original) return fail(BT_ERR_ARG, "negation: null original");
    bt_obscuration* r = new bt_obscuration;
    append_obsc(r, original);
    r->ops.push_back(blank_op(BT_O_NEGATION));
    return make_out(out, r);
}

static int compound_obsc(int op, const bt_obscuration* const* items, size_t n, bt_obscuration** out) {
    if (!items || n < 1) return fail(BT_ERR_ARG, "compound obscuration: no items");
    bt_obscuration* r = new bt_obscuration;
    for (size_t i = 0; i < n; i++) {
        if (!items[i]) { delete r; return fail(BT_ERR_ARG, "compound obscuration: null item"); }
        append_obsc(r, items[i]);
    }
    bt_obsc o = blank_op(op);
    o.n = (int32_t)n;
    r->ops.push_back(o);
    if (obsc_depth(r) > BT_MAX_OBSC_STACK) {
        delete r;
        return fail(BT_ERR_UNSUPPORTED, "obscuration expression too deep");
    }
    return make_out(out, r);
}

extern "C" int bt_obsc_union_create(const bt_obscuration* const* items, size_t n, bt_obscuration** out) {
    return compound_obsc(BT_O_UNION, items, n, out);
}

extern "C" int bt_obsc_intersection_create(const bt_obscuration* const* items, size_t n, bt_obscuration** out) {
    return compound_obsc(BT_O_INTERSECTION, items, n, out);
}

extern "C" void bt_obsc_destroy(bt_obscuration* o) { delete o; }

extern "C" int bt_simple_coating_create(double reflectivity, double transmissivity, bt_coating** out) {
    bt_coating* c = new bt_coating;
    c->R = reflectivity;
    c->T = transmissivity;
    return make_out(out, c);
}

extern "C" void bt_coating_destroy(bt_coating* c) { delete c; }

// ---------------------------------------------------------------------------
// program packing
// ---------------------------------------------------------------------------

struct ProgBuilder {
    std::vector<bt_stage> stages;
    std::vector<bt_surf> surfs;
    std::vector<bt_medium> media;
    std::vector<const bt_medium_h*> media_src;
    std::vector<bt_obsc> obsc;
    std::vector<double> pool;

    // Appends a surface's descriptors; returns the root index or -1 (error
    // message set) when a bicubic table cannot be placed in device memory.
    int add_surface(const bt_surface* s) {
        const int32_t base_rec = (int32_t)surfs.size();
        const int32_t base_pool = (int32_t)pool.size();
        for (size_t i = 0; i < s->recs.size(); i++) {
            bt_surf r = s->recs[i];
            r.off += base_pool;
            if (r.ffc >= 0) r.ffc += base_pool;
            if (r.kind == BT_S_SUM) r.m += base_rec;
            if (r.kind == BT_S_BICUBIC) {
                cudaError_t e = table_device(s->tables[i], &r.tab);
                if (e != cudaSuccess) {
                    cuda_fail(e, "bicubic table upload");
                    return -1;
                }
            }
            surfs.push_back(r);
        }
        pool.insert(pool.end(), s->pool.begin(), s->pool.end());
        return base_rec;
    }

    int add_medium(const bt_medium_h* m) {
        for (size_t i = 0; i < media_src.size(); i++)
            if (media_src[i] == m) return (int)i;
        bt_medium r = m->rec;
        r.off = (int32_t)pool.size();
        pool.insert(pool.end(), m->pool.begin(), m->pool.end());
        media.push_back(r);
        media_src.push_back(m);
        return (int)media.size() - 1;
    }

    void add_obsc(const bt_obscuration* o, int32_t* b, int32_t* e) {
        *b = (int32_t)obsc.size();
        const int32_t base = (int32_t)pool.size();
        for (bt_obsc op : o->ops) {
            if (op.op == BT_O_POLYGON) op.off += base;
            obsc.push_back(op);
        }
        pool.insert(pool.end(), o->pool.begin(), o->pool.end());
        *e = (int32_t)obsc.size();
    }

    static size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

    std::vector<unsigned char> blob() const {
        bt_prog_header h;
        memset(&h, 0, sizeof(h));
        h.nstages = (int32_t)stages.size();
        h.nsurf = (int32_t)surfs.size();
        h.nmedia = (int32_t)media.size();
        h.nobsc = (int32_t)obsc.size();
        h.npool = (int32_t)pool.size();
        size_t off = align16(sizeof(h));
        h.off_stages = (int32_t)off;
        off = align16(off + stages.size() * sizeof(bt_stage));
        h.off_surfs = (int32_t)off;
        off = align16(off + surfs.size() * sizeof(bt_surf));
        h.off_media = (int32_t)off;
        off = align16(off + media.size() * sizeof(bt_medium));
        h.off_obsc = (int32_t)off;
        off = align16(off + obsc.size() * sizeof(bt_obsc));
        h.off_pool = (int32_t)off;
        off = align16(off + pool.size() * sizeof(double));
        h.total_bytes = (int32_t)off;
        std::vector<unsigned char> b(off, 0);
        memcpy(b.data(), &h, sizeof(h));
        if (!stages.empty()) memcpy(b.data() + h.off_stages, stages.data(), stages.size() * sizeof(bt_stage));
        if (!surfs.empty()) memcpy(b.data() + h.off_surfs, surfs.data(), surfs.size() * sizeof(bt_surf));
        if (!media.empty()) memcpy(b.data() + h.off_media, media.data(), media.size() * sizeof(bt_medium));
        if (!obsc.empty()) memcpy(b.data() + h.off_obsc, obsc.data(), obsc.size() * sizeof(bt_obsc));
        if (!pool.empty()) memcpy(b.data() + h.off_pool, pool.data(), pool.size() * sizeof(double));
        return b;
    }
};

static const size_t kMaxBlobBytes = 200 * 1024;

static bt_stage blank_stage(int kind) {
    bt_stage st;
    memset(&st, 0, sizeof(st));
    st.kind = kind;
    st.surf = -1;
    st.medium = -1;
    st.screen = -1;
    st.obsc_begin = 0;
    st.obsc_end = 0;
    st.identity = 1;
    st.drot[0] = st.drot[4] = st.drot[8] = 1.0;
    return st;
}

static void set_transform(bt_stage& st, const double* dr, const double* drot) {
    if (!dr || !drot) return;
    bool zero_shift = true, unit_rot = true;
    for (int i = 0; i < 3; i++) {
        st.dr[i] = dr[i];
        if (dr[i] != 0.0) zero_shift = false;
    }
    for (int i = 0; i < 9; i++) {
        st.drot[i] = drot[i];
        const double want = (i % 4 == 0) ? 1.0 : 0.0;
        if (drot[i] != want) unit_rot = false;
    }
    st.identity = unit_rot ? (zero_shift ? 1 : 2) : 0;
}

// A temporary device copy of a blob, freed stream-ordered.
struct TempBlob {
    unsigned char* d = nullptr;
    int bytes = 0;
    cudaStream_t stream = 0;
    cudaError_t upload(const std::vector<unsigned char>& b, cudaStream_t s) {
        stream = s;
        bytes = (int)b.size();
        bt_keep_pool();
        cudaError_t e = cudaMallocAsync((void**)&d, b.size(), s);
        if (e != cudaSuccess) { d = nullptr; return e; }
        return cudaMemcpyAsync(d, b.data(), b.size(), cudaMemcpyHostToDevice, s);
    }
    ~TempBlob() {
        if (d) cudaFreeAsync(d, stream);
    }
};

static RV to_rv(const bt_rayvector* r) {
    RV v;
    v.x = r->x; v.y = r->y; v.z = r->z;
    v.vx = r->vx; v.vy = r->vy; v.vz = r->vz;
    v.t = r->t; v.w = r->wavelength; v.f = r->flux;
    v.vig = r->vignetted; v.fail = r->failed;
    v.n = (long long)r->size;
    return v;
}

static int check_rv(const bt_rayvector* rv) {
    if (!rv) return fail(BT_ERR_ARG, "null ray vector");
    if (rv->size == 0) return BT_OK;
    if (!rv->x || !rv->y || !rv->z || !rv->vx || !rv->vy || !rv->vz || !rv->t || !rv->wavelength || !rv->flux ||
        !rv->vignetted || !rv->failed)
        return fail(BT_ERR_ARG, "ray vector has a null array");
    return BT_OK;
}

static int run_single(const ProgBuilder& pb, const bt_rayvector* rv, int niter, cudaStream_t stream,
                      const char* what) {
    std::vector<unsigned char> b = pb.blob();
    if (b.size() > kMaxBlobBytes) return fail(BT_ERR_UNSUPPORTED, std::string(what) + ": descriptor too large");
    TempBlob tb;
    CUDA_TRY(tb.upload(b, stream), what);
    RV v = to_rv(rv);
    CUDA_TRY(bt_launch_trace(tb.d, tb.bytes, v, v, nullptr, 0, niter, stream), what);
    return BT_OK;
}

static int surface_op(int kind, const bt_surface* s, const double* dr, const double* drot, const bt_medium_h* m2,
                      const bt_rayvector* rv, const bt_coating* coating, int niter, void* stream, const char* what,
                      const bt_surface* screen = nullptr) {
    if (!s) return fail(BT_ERR_ARG, std::string(what) + ": null surface");
    int rc = check_rv(rv);
    if (rc != BT_OK) return rc;
    if (!dr || !drot) return fail(BT_ERR_ARG, std::string(what) + ": null transform");
    if (niter < 0) return fail(BT_ERR_ARG, std::string(what) + ": negative niter");
    if (rv->size == 0) return BT_OK;
    ProgBuilder pb;
    bt_stage st = blank_stage(kind);
    set_transform(st, dr, drot);
    st.surf = pb.add_surface(s);
    if (st.surf < 0) return BT_ERR_CUDA;
    if (kind == BT_ST_REFRACT) {
        if (!m2) return fail(BT_ERR_ARG, "refract: null medium");
        st.medium = pb.add_medium(m2);
    }
    if (kind == BT_ST_SCREEN) {
        if (!screen) return fail(BT_ERR_ARG, "refractScreen: null screen");
        st.screen = pb.add_surface(screen);
        if (st.screen < 0) return BT_ERR_CUDA;
    }
    if (coating) {
        st.coated = 1;
        st.coat_r = coating->R;
        st.coat_t = coating->T;
    }
    pb.stages.push_back(st);
    return run_single(pb, rv, niter, (cudaStream_t)stream, what);
}

extern "C" int bt_intersect(const bt_surface* s, const double dr[3], const double drot[9], const bt_rayvector* rv,
                            const bt_coating* coating, int max_threads, int niter, void* stream) {
    (void)max_threads;
    return surface_op(BT_ST_INTERSECT, s, dr, drot, nullptr, rv, coating, niter, stream, "intersect");
}

extern "C" int bt_reflect(const bt_surface* s, const double dr[3], const double drot[9], const bt_rayvector* rv,
                          const bt_coating* coating, int max_threads, int niter, void* stream) {
    (void)max_threads;
    return surface_op(BT_ST_REFLECT, s, dr, drot, nullptr, rv, coating, niter, stream, "reflect");
}

extern "C" int bt_refract(const bt_surface* s, const double dr[3], const double drot[9], const bt_medium_h* m1,
                          const bt_medium_h* m2, const bt_rayvector* rv, const bt_coating* coating, int max_threads,
                          int niter, void* stream) {
    (void)max_threads;
    (void)m1;  // n1 comes from |v| (src/batoid.cpp:454-458)
    return surface_op(BT_ST_REFRACT, s, dr, drot, m2, rv, coating, niter, stream, "refract");
}

extern "C" int bt_refract_screen(const bt_surface* s, const double dr[3], const double drot[9],
                                 const bt_surface* screen, const bt_rayvector* rv, int max_threads, int niter,
                                 void* stream) {
    (void)max_threads;
    return surface_op(BT_ST_SCREEN, s, dr, drot, nullptr, rv, nullptr, niter, stream, "refractScreen", screen);
}

extern "C" int bt_rsplit(const bt_surface* s, const double dr[3], const double drot[9], const bt_medium_h* m1,
                         const bt_medium_h* m2, const bt_coating* coating, const bt_rayvector* rv,
                         const bt_rayvector* rv_split, int max_threads, int niter, void* stream) {
    (void)max_threads;
    (void)m1;  // n1 comes from |v| (src/batoid.cpp:599-603)
    if (!s || !m2 || !coating) return fail(BT_ERR_ARG, "rsplit: null surface, medium or coating");
    int rc = check_rv(rv);
    if (rc != BT_OK) return rc;
    rc = check_rv(rv_split);
    if (rc != BT_OK) return rc;
    if (rv_split->size != rv->size) return fail(BT_ERR_ARG, "rsplit: ray vectors differ in size");
    if (!dr || !drot) return fail(BT_ERR_ARG, "rsplit: null transform");
    if (niter < 0) return fail(BT_ERR_ARG, "rsplit: negative niter");
    if (rv->size == 0) return BT_OK;
    ProgBuilder pb;
    bt_stage st = blank_stage(BT_ST_REFRACT);
    set_transform(st, dr, drot);
    st.surf = pb.add_surface(s);
    if (st.surf < 0) return BT_ERR_CUDA;
    st.medium = pb.add_medium(m2);
    st.coated = 1;
    st.coat_r = coating->R;
    st.coat_t = coating->T;
    pb.stages.push_back(st);
    std::vector<unsigned char> b = pb.blob();
    TempBlob tb;
    CUDA_TRY(tb.upload(b, (cudaStream_t)stream), "rsplit");
    RV v = to_rv(rv), w = to_rv(rv_split);
    CUDA_TRY(bt_launch_rsplit(tb.d, tb.bytes, v, w, niter, (cudaStream_t)stream), "rsplit");
    return BT_OK;
}

extern "C" int bt_obscure(const bt_obscuration* o, const bt_rayvector* rv, int max_threads, void* stream) {
    (void)max_threads;
    if (!o) return fail(BT_ERR_ARG, "obscure: null obscuration");
    int rc = check_rv(rv);
    if (rc != BT_OK || rv->size == 0) return rc;
    ProgBuilder pb;
    bt_stage st = blank_stage(BT_ST_OBSCURE);
    pb.add_obsc(o, &st.obsc_begin, &st.obsc_end);
    pb.stages.push_back(st);
    std::vector<unsigned char> b = pb.blob();
    TempBlob tb;
    CUDA_TRY(tb.upload(b, (cudaStream_t)stream), "obscure");
    RV v = to_rv(rv);
    CUDA_TRY(bt_launch_obsc(tb.d, tb.bytes, nullptr, nullptr, nullptr, &v, v.n, (cudaStream_t)stream), "obscure");
    return BT_OK;
}

extern "C" int bt_obsc_contains(const bt_obscuration* o, const double* x, const double* y, uint8_t* out, size_t n,
                                void* stream) {
    if (!o) return fail(BT_ERR_ARG, "contains: null obscuration");
    if (n == 0) return BT_OK;
    if (!x || !y || !out) return fail(BT_ERR_ARG, "contains: null array");
    ProgBuilder pb;
    bt_stage st = blank_stage(BT_ST_OBSCURE);
    pb.add_obsc(o, &st.obsc_begin, &st.obsc_end);
    pb.stages.push_back(st);
    std::vector<unsigned char> b = pb.blob();
    TempBlob tb;
    CUDA_TRY(tb.upload(b, (cudaStream_t)stream), "contains");
    CUDA_TRY(bt_launch_obsc(tb.d, tb.bytes, x, y, out, nullptr, (long long)n, (cudaStream_t)stream), "contains");
    return BT_OK;
}

extern "C" int bt_surface_sag(const bt_surface* s, const double* x, const double* y, double* out, size_t n,
                              void* stream) {
    if (!s) return fail(BT_ERR_ARG, "sag: null surface");
    if (n == 0) return BT_OK;
    if (!x || !y || !out) return fail(BT_ERR_ARG, "sag: null array");
    ProgBuilder pb;
    bt_stage st = blank_stage(BT_ST_INTERSECT);
    st.surf = pb.add_surface(s);
    if (st.surf < 0) return BT_ERR_CUDA;
    pb.stages.push_back(st);
    TempBlob tb;
    CUDA_TRY(tb.upload(pb.blob(), (cudaStream_t)stream), "sag");
    CUDA_TRY(bt_launch_surface_eval(tb.d, tb.bytes, x, y, out, nullptr, (long long)n, (cudaStream_t)stream), "sag");
    return BT_OK;
}

extern "C" int bt_surface_normal(const bt_surface* s, const double* x, const double* y, double* out, size_t n,
                                 void* stream) {
    if (!s) return fail(BT_ERR_ARG, "normal: null surface");
    if (n == 0) return BT_OK;
    if (!x || !y || !out) return fail(BT_ERR_ARG, "normal: null array");
    ProgBuilder pb;
    bt_stage st = blank_stage(BT_ST_INTERSECT);
    st.surf = pb.add_surface(s);
    if (st.surf < 0) return BT_ERR_CUDA;
    pb.stages.push_back(st);
    TempBlob tb;
    CUDA_TRY(tb.upload(pb.blob(), (cudaStream_t)stream), "normal");
    CUDA_TRY(bt_launch_surface_eval(tb.d, tb.bytes, x, y, nullptr, out, (long long)n, (cudaStream_t)stream),
             "normal");
    return BT_OK;
}

extern "C" int bt_medium_getN(const bt_medium_h* m, const double* w, double* out, size_t n, void* stream) {
    if (!m) return fail(BT_ERR_ARG, "getN: null medium");
    if (n == 0) return BT_OK;
    if (!w || !out) return fail(BT_ERR_ARG, "getN: null array");
    ProgBuilder pb;
    pb.add_medium(m);
    pb.stages.push_back(blank_stage(BT_ST_OBSCURE));
    TempBlob tb;
    CUDA_TRY(tb.upload(pb.blob(), (cudaStream_t)stream), "getN");
    CUDA_TRY(bt_launch_getN(tb.d, tb.bytes, w, out, (long long)n, (cudaStream_t)stream), "getN");
    return BT_OK;
}

// ---------------------------------------------------------------------------
// transforms and RayVector methods
// ---------------------------------------------------------------------------

extern "C" int bt_apply_forward_transform(const double dr[3], const double drot[9], const bt_rayvector* rv,
                                          int max_threads, void* stream) {
    (void)max_threads;
    int rc = check_rv(rv);
    if (rc != BT_OK) return rc;
    if (!dr || !drot) return fail(BT_ERR_ARG, "transform: null transform");
    CUDA_TRY(bt_launch_transform_rv(dr, drot, to_rv(rv), true, (cudaStream_t)stream), "applyForwardTransform");
    return BT_OK;
}

extern "C" int bt_apply_reverse_transform(const double dr[3], const double drot[9], const bt_rayvector* rv,
                                          int max_threads, void* stream) {
    (void)max_threads;
    int rc = check_rv(rv);
    if (rc != BT_OK) return rc;
    if (!dr || !drot) return fail(BT_ERR_ARG, "transform: null transform");
    CUDA_TRY(bt_launch_transform_rv(dr, drot, to_rv(rv), false, (cudaStream_t)stream), "applyReverseTransform");
    return BT_OK;
}

extern "C" int bt_apply_forward_transform_arrays(const double dr[3], const double drot[9], double* x, double* y,
                                                 double* z, size_t n, int max_threads, void* stream) {
    (void)max_threads;
    if (n == 0) return BT_OK;
    if (!dr || !drot || !x || !y || !z) return fail(BT_ERR_ARG, "transform arrays: null argument");
    CUDA_TRY(bt_launch_transform_arrays(dr, drot, x, y, z, (long long)n, true, (cudaStream_t)stream),
             "applyForwardTransformArrays");
    return BT_OK;
}

extern "C" int bt_apply_reverse_transform_arrays(const double dr[3], const double drot[9], double* x, double* y,
                                                 double* z, size_t n, int max_threads, void* stream) {
    (void)max_threads;
    if (n == 0) return BT_OK;
    if (!dr || !drot || !x || !y || !z) return fail(BT_ERR_ARG, "transform arrays: null argument");
    CUDA_TRY(bt_launch_transform_arrays(dr, drot, x, y, z, (long long)n, false, (cudaStream_t)stream),
             "applyReverseTransformArrays");
    return BT_OK;
}

extern "C" int bt_finish_parallel(const double dr[3], const double drot[9], const double vv[3], double* x,
                                  double* y, double* z, size_t n, void* stream) {
    if (n == 0) return BT_OK;
    if (!dr || !drot || !vv || !x || !y || !z) return fail(BT_ERR_ARG, "finishParallel: null argument");
    CUDA_TRY(bt_launch_finish_parallel(dr, drot, vv, x, y, z, (long long)n, (cudaStream_t)stream), "finishParallel");
    return BT_OK;
}

extern "C" int bt_stop_points_grid(int nx, int ny, double valx, double valy, const double lx[2], const double ly[2],
                                   double* x, double* y, void* stream) {
    if (nx < 1 || ny < 1) return fail(BT_ERR_ARG, "stop points (grid): nx and ny must be positive");
    if (!lx || !ly || !x || !y) return fail(BT_ERR_ARG, "stop points (grid): null argument");
    CUDA_TRY(bt_launch_stop_grid(nx, ny, valx, valy, lx, ly, x, y, (cudaStream_t)stream), "stop points (grid)");
    return BT_OK;
}

extern "C" int bt_stop_points_rings(int nring, const double* r, const double* step, const long long* off,
                                    long long n, double* x, double* y, void* stream) {
    if (n == 0) return BT_OK;
    if (nring < 1 || n < 0) return fail(BT_ERR_ARG, "stop points (rings): bad ring count or size");
    if (!r || !step || !off || !x || !y) return fail(BT_ERR_ARG, "stop points (rings): null argument");
    CUDA_TRY(bt_launch_stop_rings(nring, r, step, off, n, x, y, (cudaStream_t)stream), "stop points (rings)");
    return BT_OK;
}

extern "C" int bt_stop_points_spokes(const double* rings, int nr, const double* spokes, int ns, double* x, double* y,
                                     void* stream) {
    if (nr == 0 || ns == 0) return BT_OK;
    if (nr < 0 || ns < 0) return fail(BT_ERR_ARG, "stop points (spokes): negative size");
    if (!rings || !spokes || !x || !y) return fail(BT_ERR_ARG, "stop points (spokes): null argument");
    CUDA_TRY(bt_launch_stop_spokes(rings, nr, spokes, ns, x, y, (cudaStream_t)stream), "stop points (spokes)");
    return BT_OK;
}

extern "C" int bt_rv_position_at_time(const bt_rayvector* rv, double t, double* xo, double* yo, double* zo,
                                      int max_threads, void* stream) {
    (void)max_threads;
    int rc = check_rv(rv);
    if (rc != BT_OK || rv->size == 0) return rc;
    if (!xo || !yo || !zo) return fail(BT_ERR_ARG, "positionAtTime: null output");
    CUDA_TRY(bt_launch_position_at_time(to_rv(rv), t, xo, yo, zo, (cudaStream_t)stream), "positionAtTime");
    return BT_OK;
}

extern "C" int bt_rv_propagate_in_place(const bt_rayvector* rv, double t, int max_threads, void* stream) {
    (void)max_threads;
    int rc = check_rv(rv);
    if (rc != BT_OK || rv->size == 0) return rc;
    CUDA_TRY(bt_launch_propagate(to_rv(rv), t, (cudaStream_t)stream), "propagateInPlace");
    return BT_OK;
}

extern "C" int bt_rv_phase(const bt_rayvector* rv, double x, double y, double z, double t, double* out,
                           int max_threads, void* stream) {
    (void)max_threads;
    int rc = check_rv(rv);
    if (rc != BT_OK || rv->size == 0) return rc;
    if (!out) return fail(BT_ERR_ARG, "phase: null output");
    CUDA_TRY(bt_launch_phase(to_rv(rv), x, y, z, t, out, false, (cudaStream_t)stream), "phase");
    return BT_OK;
}

extern "C" int bt_rv_amplitude(const bt_rayvector* rv, double x, double y, double z, double t, double* out,
                               int max_threads, void* stream) {
    (void)max_threads;
    int rc = check_rv(rv);
    if (rc != BT_OK || rv->size == 0) return rc;
    if (!out) return fail(BT_ERR_ARG, "amplitude: null output");
    CUDA_TRY(bt_launch_phase(to_rv(rv), x, y, z, t, out, true, (cudaStream_t)stream), "amplitude");
    return BT_OK;
}

extern "C" int bt_rv_sum_amplitude(const bt_rayvector* rv, double x, double y, double z, double t,
                                   int ignore_vignetted, int max_threads, double* out, void* stream) {
    (void)max_threads;
    int rc = check_rv(rv);
    if (rc != BT_OK) return rc;
    if (!out) return fail(BT_ERR_ARG, "sumAmplitude: null output");
    out[0] = 0.0;
    out[1] = 0.0;
    if (rv->size == 0) return BT_OK;
    cudaStream_t s = (cudaStream_t)stream;
    double* d = nullptr;
    bt_keep_pool();
    CUDA_TRY(cudaMallocAsync((void**)&d, 2 * sizeof(double), s), "sumAmplitude");
    cudaError_t e = bt_launch_sum_amplitude(to_rv(rv), x, y, z, t, ignore_vignetted != 0, d, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(d, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "sumAmplitude");
    return BT_OK;
}

extern "C" int bt_rv_equal(const bt_rayvector* a, const bt_rayvector* b, int* out, void* stream) {
    int rc = check_rv(a);
    if (rc != BT_OK) return rc;
    rc = check_rv(b);
    if (rc != BT_OK) return rc;
    if (!out) return fail(BT_ERR_ARG, "equal: null output");
    if (a->size != b->size) { *out = 0; return BT_OK; }
    if (a->size == 0) { *out = 1; return BT_OK; }
    cudaStream_t s = (cudaStream_t)stream;
    int* d = nullptr;
    int one = 1;
    bt_keep_pool();
    CUDA_TRY(cudaMallocAsync((void**)&d, sizeof(int), s), "equal");
    cudaError_t e = cudaMemcpyAsync(d, &one, sizeof(int), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = bt_launch_rv_equal(to_rv(a), to_rv(b), d, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(d, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "equal");
    return BT_OK;
}

// ---------------------------------------------------------------------------
// fused optic
// ---------------------------------------------------------------------------

struct bt_optic {
    int nstages;
    int blob_bytes;
    unsigned char* d_blob;
    // host pipeline scratch for bt_optic_trace_host
    std::mutex mu;
    size_t host_chunk = 0;
    // host-buffer pipeline: BT_HOST_PIPE chunk buffers, one stream each
    unsigned char* d_chunk[BT_HOST_PIPE] = {nullptr, nullptr, nullptr};
    cudaStream_t streams[BT_HOST_PIPE] = {nullptr, nullptr, nullptr};
    cudaEvent_t done[BT_HOST_PIPE] = {nullptr, nullptr, nullptr};
};

extern "C" int bt_optic_create_ex(size_t nstages, const int* kinds, const bt_surface* const* surfaces,
                                  const double* dr, const double* drot, const bt_medium_h* const* media,
                                  const bt_obscuration* const* obscurations, const bt_coating* const* coatings,
                                  const bt_surface* const* screens, bt_optic** out);

extern "C" int bt_optic_create(size_t nstages, const int* kinds, const bt_surface* const* surfaces, const double* dr,
                               const double* drot, const bt_medium_h* const* media,
                               const bt_obscuration* const* obscurations, const bt_coating* const* coatings,
                               bt_optic** out) {
    return bt_optic_create_ex(nstages, kinds, surfaces, dr, drot, media, obscurations, coatings, nullptr, out);
}

extern "C" int bt_optic_create_ex(size_t nstages, const int* kinds, const bt_surface* const* surfaces,
                                  const double* dr, const double* drot, const bt_medium_h* const* media,
                                  const bt_obscuration* const* obscurations, const bt_coating* const* coatings,
                                  const bt_surface* const* screens, bt_optic** out) {
    if (!out) return fail(BT_ERR_ARG, "optic: null output");
    if (nstages > BT_MAX_STAGES) return fail(BT_ERR_UNSUPPORTED, "optic: too many stages");
    if (nstages > 0 && (!kinds || !surfaces || !dr || !drot)) return fail(BT_ERR_ARG, "optic: null stage arrays");
    ProgBuilder pb;
    for (size_t k = 0; k < nstages; k++) {
        const int kind = kinds[k];
        if (kind != BT_ST_INTERSECT && kind != BT_ST_REFLECT && kind != BT_ST_REFRACT && kind != BT_ST_SCREEN)
            return fail(BT_ERR_ARG, "optic: bad stage kind");
        if (!surfaces[k]) return fail(BT_ERR_ARG, "optic: null surface");
        bt_stage st = blank_stage(kind);
        set_transform(st, dr + 3 * k, drot + 9 * k);
        st.surf = pb.add_surface(surfaces[k]);
        if (st.surf < 0) return BT_ERR_CUDA;
        if (kind == BT_ST_SCREEN) {
            if (!screens || !screens[k]) return fail(BT_ERR_ARG, "optic: screen stage without a screen surface");
            st.screen = pb.add_surface(screens[k]);
            if (st.screen < 0) return BT_ERR_CUDA;
        }
        if (kind == BT_ST_REFRACT) {
            if (!media || !media[k]) return fail(BT_ERR_ARG, "optic: refracting stage without a medium");
            st.medium = pb.add_medium(media[k]);
        }
        if (obscurations && obscurations[k]) pb.add_obsc(obscurations[k], &st.obsc_begin, &st.obsc_end);
        if (coatings && coatings[k]) {
            st.coated = 1;
            st.coat_r = coatings[k]->R;
            st.coat_t = coatings[k]->T;
        }
        pb.stages.push_back(st);
    }
    std::vector<unsigned char> b = pb.blob();
    if (b.size() > kMaxBlobBytes) return fail(BT_ERR_UNSUPPORTED, "optic: descriptor too large");
    bt_optic* o = new bt_optic;
    o->nstages = (int)nstages;
    o->blob_bytes = (int)b.size();
    cudaError_t e = cudaMalloc((void**)&o->d_blob, b.size());
    if (e != cudaSuccess) { delete o; return cuda_fail(e, "optic alloc"); }
    e = cudaMemcpy(o->d_blob, b.data(), b.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { cudaFree(o->d_blob); delete o; return cuda_fail(e, "optic upload"); }
    *out = o;
    return BT_OK;
}

static void release_host_pipeline(bt_optic* o) {
    for (int k = 0; k < BT_HOST_PIPE; k++) {
        if (o->d_chunk[k]) cudaFree(o->d_chunk[k]);
        if (o->streams[k]) cudaStreamDestroy(o->streams[k]);
        if (o->done[k]) cudaEventDestroy(o->done[k]);
        o->d_chunk[k] = nullptr;
        o->streams[k] = nullptr;
        o->done[k] = nullptr;
    }
    o->host_chunk = 0;
}

extern "C" void bt_optic_destroy(bt_optic* o) {
    if (!o) return;
    release_host_pipeline(o);
    if (o->d_blob) cudaFree(o->d_blob);
    delete o;
}

extern "C" int bt_optic_nstages(const bt_optic* o, int* out) {
    if (!o || !out) return fail(BT_ERR_ARG, "null argument");
    *out = o->nstages;
    return BT_OK;
}

extern "C" int bt_optic_trace(const bt_optic* o, const bt_rayvector* rv, int niter, void* stream) {
    if (!o) return fail(BT_ERR_ARG, "trace: null optic");
    int rc = check_rv(rv);
    if (rc != BT_OK || rv->size == 0) return rc;
    if (niter < 0) return fail(BT_ERR_ARG, "trace: negative niter");
    RV v = to_rv(rv);
    CUDA_TRY(bt_launch_trace(o->d_blob, o->blob_bytes, v, v, nullptr, 0, niter, (cudaStream_t)stream), "trace");
    return BT_OK;
}

extern "C" int bt_optic_trace_into(const bt_optic* o, const bt_rayvector* in, const bt_rayvector* out, int niter,
                                   void* stream) {
    if (!o) return fail(BT_ERR_ARG, "trace: null optic");
    int rc = check_rv(in);
    if (rc != BT_OK) return rc;
    rc = check_rv(out);
    if (rc != BT_OK) return rc;
    if (in->size != out->size) return fail(BT_ERR_ARG, "trace: input and output sizes differ");
    if (in->size == 0) return BT_OK;
    if (niter < 0) return fail(BT_ERR_ARG, "trace: negative niter");
    CUDA_TRY(bt_launch_trace(o->d_blob, o->blob_bytes, to_rv(in), to_rv(out), nullptr, 0, niter,
                             (cudaStream_t)stream),
             "trace");
    return BT_OK;
}

extern "C" int bt_optic_trace_full(const bt_optic* o, const bt_rayvector* rv, const bt_rayvector* snaps, int niter,
                                   void* stream) {
    if (!o) return fail(BT_ERR_ARG, "traceFull: null optic");
    int rc = check_rv(rv);
    if (rc != BT_OK) return rc;
    if (!snaps && o->nstages > 0) return fail(BT_ERR_ARG, "traceFull: null snapshots");
    if (rv->size == 0 || o->nstages == 0) return BT_OK;
    SnapSet ss;
    memset(&ss, 0, sizeof(ss));
    for (int k = 0; k < o->nstages; k++) {
        rc = check_rv(&snaps[k]);
        if (rc != BT_OK) return rc;
        if (snaps[k].size != rv->size) return fail(BT_ERR_ARG, "traceFull: snapshot size mismatch");
        ss.s[k] = to_rv(&snaps[k]);
    }
    RV v = to_rv(rv);
    CUDA_TRY(bt_launch_trace(o->d_blob, o->blob_bytes, v, v, &ss, o->nstages, niter, (cudaStream_t)stream),
             "traceFull");
    return BT_OK;
}

// Device chunk layout: 9 double arrays then 2 byte arrays, each `chunk` long.
static RV chunk_rv(unsigned char* base, size_t chunk, long long n) {
    RV v;
    double* d = reinterpret_cast<double*>(base);
    v.x = d; v.y = d + chunk; v.z = d + 2 * chunk;
    v.vx = d + 3 * chunk; v.vy = d + 4 * chunk; v.vz = d + 5 * chunk;
    v.t = d + 6 * chunk; v.w = d + 7 * chunk; v.f = d + 8 * chunk;
    v.vig = base + 9 * chunk * sizeof(double);
    v.fail = v.vig + chunk;
    v.n = n;
    return v;
}

extern "C" int bt_optic_trace_host(const bt_optic* oc, const bt_rayvector* h, int niter, size_t chunk,
                                   void* stream) {
    bt_optic* o = const_cast<bt_optic*>(oc);
    if (!o) return fail(BT_ERR_ARG, "traceHost: null optic");
    int rc = check_rv(h);
    if (rc != BT_OK || h->size == 0) return rc;
    if (chunk == 0) chunk = (size_t)1 << 22;
    {
        // whole rounds of the persistent grid per chunk (and per eighth of
        // one, the pieces the first and last buffers are filled in)
        const size_t round8 = (size_t)bt_trace_ff_round_rays() * 8;
        if (round8 > 0 && chunk >= round8) chunk = (chunk + round8 / 2) / round8 * round8;
    }
    if (chunk > h->size) chunk = h->size;
    std::lock_guard<std::mutex> lock(o->mu);
    const size_t bytes = chunk * (9 * sizeof(double) + 2);
    if (o->host_chunk != chunk) {
        release_host_pipeline(o);
        for (int k = 0; k < BT_HOST_PIPE; k++) {
            cudaError_t e = cudaMalloc((void**)&o->d_chunk[k], bytes);
            if (e != cudaSuccess) { release_host_pipeline(o); return fail(BT_ERR_ALLOC, "traceHost: device scratch"); }
            CUDA_TRY(cudaStreamCreateWithFlags(&o->streams[k], cudaStreamNonBlocking), "traceHost streams");
            CUDA_TRY(cudaEventCreateWithFlags(&o->done[k], cudaEventDisableTiming), "traceHost events");
        }
        o->host_chunk = chunk;
    }
    // Order the pipeline after prior work on the caller's stream.
    cudaStream_t user = (cudaStream_t)stream;
    cudaEvent_t start;
    CUDA_TRY(cudaEventCreateWithFlags(&start, cudaEventDisableTiming), "traceHost");
    CUDA_TRY(cudaEventRecord(start, user), "traceHost");
    for (int k = 0; k < BT_HOST_PIPE; k++) CUDA_TRY(cudaStreamWaitEvent(o->streams[k], start, 0), "traceHost");
    cudaEventDestroy(start);
    const size_t n = h->size;
    // Chunk boundaries.  On long inputs the first and last chunk buffers
    // are filled in steps of chunk/8, /8, /4, /2: the copy in before the
    // first trace and the copy out after the last one are what the
    // pipeline cannot overlap, so they are made small.
    std::vector<size_t> cut{0};
    {
        auto push = [&](size_t m) { cut.push_back(cut.back() + m); };
        const size_t e = chunk / 8;
        if (e > 0 && n >= 4 * chunk) {
            push(e);
            push(e);
            push(chunk / 4);
            push(chunk / 2);
            const size_t ramp = e + e + chunk / 4 + chunk / 2;  // the head's (and tail's) total
            while (n - cut.back() >= ramp + chunk + chunk) push(chunk);
            const size_t mid = n - cut.back() - ramp;  // in [chunk, 2 chunk)
            push(mid / 2);
            push(mid - mid / 2);
            push(chunk / 2);
            push(chunk / 4);
            push(e);
            push(n - cut.back());
        } else {
            while (cut.back() < n) push((n - cut.back()) < chunk ? (n - cut.back()) : chunk);
        }
    }
    const size_t nchunks = cut.size() - 1;
    for (size_t c = 0; c < nchunks; c++) {
        const int k = (int)(c % BT_HOST_PIPE);
        cudaStream_t s = o->streams[k];
        const size_t i0 = cut[c];
        const size_t m = cut[c + 1] - i0;
        RV d = chunk_rv(o->d_chunk[k], chunk, (long long)m);
        double* hd[9] = {h->x, h->y, h->z, h->vx, h->vy, h->vz, h->t, h->wavelength, h->flux};
        double* dd[9] = {d.x, d.y, d.z, d.vx, d.vy, d.vz, d.t, d.w, d.f};
        for (int a = 0; a < 9; a++)
            CUDA_TRY(cudaMemcpyAsync(dd[a], hd[a] + i0, m * sizeof(double), cudaMemcpyHostToDevice, s), "traceHost H2D");
        CUDA_TRY(cudaMemcpyAsync(d.vig, h->vignetted + i0, m, cudaMemcpyHostToDevice, s), "traceHost H2D");
        CUDA_TRY(cudaMemcpyAsync(d.fail, h->failed + i0, m, cudaMemcpyHostToDevice, s), "traceHost H2D");
        CUDA_TRY(bt_launch_trace(o->d_blob, o->blob_bytes, d, d, nullptr, 0, niter, s), "traceHost trace");
        // wavelength is never modified by a trace: no copy back
        double* ho[8] = {h->x, h->y, h->z, h->vx, h->vy, h->vz, h->t, h->flux};
        double* dout[8] = {d.x, d.y, d.z, d.vx, d.vy, d.vz, d.t, d.f};
        for (int a = 0; a < 8; a++)
            CUDA_TRY(cudaMemcpyAsync(ho[a] + i0, dout[a], m * sizeof(double), cudaMemcpyDeviceToHost, s), "traceHost D2H");
        CUDA_TRY(cudaMemcpyAsync(h->vignetted + i0, d.vig, m, cudaMemcpyDeviceToHost, s), "traceHost D2H");
        CUDA_TRY(cudaMemcpyAsync(h->failed + i0, d.fail, m, cudaMemcpyDeviceToHost, s), "traceHost D2H");
    }
    for (int k = 0; k < BT_HOST_PIPE; k++) {
        CUDA_TRY(cudaEventRecord(o->done[k], o->streams[k]), "traceHost");
        CUDA_TRY(cudaStreamWaitEvent(user, o->done[k], 0), "traceHost");
    }
    CUDA_TRY(cudaStreamSynchronize(user), "traceHost sync");
    return BT_OK;
}

// ---------------------------------------------------------------------------
// Huygens
// ---------------------------------------------------------------------------

extern "C" int bt_huygens_amplitudes(const bt_rayvector* rv, double px, double py, double pz, const double lat[4],
                                     int na, int nb, double t0, int ignore_vignetted, double* out_re,
                                     double* out_im, void* stream) {
    int rc = check_rv(rv);
    if (rc != BT_OK) return rc;
    if (!lat || na < 0 || nb < 0) return fail(BT_ERR_ARG, "huygens: bad lattice");
    if ((long long)na * nb == 0) return BT_OK;
    if (!out_re || !out_im) return fail(BT_ERR_ARG, "huygens: null output");
    CUDA_TRY(bt_launch_huygens(to_rv(rv), px, py, pz, lat, na, nb, t0, ignore_vignetted != 0, out_re, out_im,
                               (cudaStream_t)stream),
             "huygens");
    return BT_OK;
}

// All fields of huygensPSFs in one launch set: field f's rays are the f-th
// block of rv->n / nfields rays; points [nfields][3], lat [nfields][4] and
// t0 [nfields] are host arrays; outputs [nfields][na*nb] on the device.
extern "C" int bt_huygens_amplitudes_fields(const bt_rayvector* rv, int nfields, const double* points,
                                            const double* lat, const double* t0, int na, int nb,
                                            int ignore_vignetted, double* out_re, double* out_im, void* stream) {
    int rc = check_rv(rv);
    if (rc != BT_OK) return rc;
    if (nfields < 1 || !points || !lat || !t0) return fail(BT_ERR_ARG, "huygens fields: bad field arrays");
    if (na < 0 || nb < 0) return fail(BT_ERR_ARG, "huygens fields: bad lattice");
    if (rv->size % nfields != 0) return fail(BT_ERR_ARG, "huygens fields: rays are not nfields equal blocks");
    if ((long long)na * nb == 0) return BT_OK;
    if (!out_re || !out_im) return fail(BT_ERR_ARG, "huygens fields: null output");
    CUDA_TRY(bt_launch_huygens_fields(to_rv(rv), (long long)rv->size / nfields, nfields, points, points + 1, points + 2, lat, t0,
                                      3, na, nb, ignore_vignetted != 0, out_re, out_im, (cudaStream_t)stream),
             "huygens fields");
    return BT_OK;
}

// Same result as bt_huygens_amplitudes, but allocates no device memory: the
// scratch is a fixed 8 MiB array inside the library (see huygens.cu).
extern "C" int bt_huygens_amplitudes_noalloc(const bt_rayvector* rv, double px, double py, double pz,
                                             const double lat[4], int na, int nb, double t0, int ignore_vignetted,
                                             double* out_re, double* out_im, void* stream) {
    int rc = check_rv(rv);
    if (rc != BT_OK) return rc;
    if (!lat || na < 0 || nb < 0) return fail(BT_ERR_ARG, "huygens (no-alloc): bad lattice");
    if ((long long)na * nb == 0) return BT_OK;
    if (!out_re || !out_im) return fail(BT_ERR_ARG, "huygens (no-alloc): null output");
    size_t needed = 0;
    cudaError_t e = bt_launch_huygens_noalloc(to_rv(rv), px, py, pz, lat, na, nb, t0, ignore_vignetted != 0, out_re,
                                              out_im, (cudaStream_t)stream, &needed);
    if (e == cudaErrorInvalidValue && needed > (8u << 20))
        return fail(BT_ERR_ARG, "huygens (no-alloc): problem needs " + std::to_string(needed) +
                                    " bytes of scratch (32 per ray + 16 per pixel), limit is 8388608");
    if (e != cudaSuccess) return cuda_fail(e, "huygens (no-alloc)");
    return BT_OK;
}

extern "C" int bt_zernike_normal_equations(const double* x, const double* y, const double* v,
                                           const long long* offsets, int nfits, const double* basis, int jmax,
                                           int side, double* G, double* b, void* stream) {
    if (nfits < 0 || jmax < 1 || side < 1) return fail(BT_ERR_ARG, "zernike fit: bad sizes");
    if (jmax > 64 || side > 12) return fail(BT_ERR_UNSUPPORTED, "zernike fit: jmax <= 64 and order <= 11 supported");
    if (nfits == 0) return BT_OK;
    if (!x || !y || !v || !offsets || !basis || !G || !b) return fail(BT_ERR_ARG, "zernike fit: null array");
    CUDA_TRY(bt_launch_zk_normal(x, y, v, offsets, nfits, basis, jmax, side, G, b, (cudaStream_t)stream),
             "zernike fit");
    return BT_OK;
}

extern "C" int bt_measure_fp64_peak(int iters, double* tflops, void* stream) {
    if (!tflops || iters < 8) return fail(BT_ERR_ARG, "fp64 probe: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    double* sink = nullptr;
    bt_keep_pool();
    CUDA_TRY(cudaMallocAsync((void**)&sink, sizeof(double), s), "fp64 probe");
    float ms = 0.f;
    double flops = 0.0;
    cudaError_t e = bt_launch_dfma_probe(iters, sink, &ms, &flops, s);
    cudaFreeAsync(sink, s);
    cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "fp64 probe");
    *tflops = flops / (ms * 1e-3) / 1e12;
    return BT_OK;
}

extern "C" int bt_measure_fp32_peak(int iters, double* tflops, void* stream) {
    if (!tflops || iters < 8) return fail(BT_ERR_ARG, "fp32 probe: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    double* sink = nullptr;
    bt_keep_pool();
    CUDA_TRY(cudaMallocAsync((void**)&sink, sizeof(double), s), "fp32 probe");
    float ms = 0.f;
    double flops = 0.0;
    cudaError_t e = bt_launch_ffma_probe(iters, sink, &ms, &flops, s);
    cudaFreeAsync(sink, s);
    cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "fp32 probe");
    *tflops = flops / (ms * 1e-3) / 1e12;
    return BT_OK;
}

// Test hook: reads and clears the device status word of the trace kernels
// (BT_ERR_TIMEOUT if a bounded wait expired).  Synchronous.
extern "C" int bt_check_device_status(void* stream) {
    int st = 0, sb = 0, sm = 0, ss = 0;
    CUDA_TRY(bt_read_device_status(&st, (cudaStream_t)stream), "device status");
    CUDA_TRY(bt_read_split_device_status(&ss, (cudaStream_t)stream), "device status");
    if (st == 0) st = ss;
    CUDA_TRY(bt_read_trace_ff_device_status(&ss, (cudaStream_t)stream), "device status");
    if (st == 0) st = ss;
    CUDA_TRY(bt_read_batch_device_status(&sb, (cudaStream_t)stream), "device status");
    CUDA_TRY(bt_read_mlp_device_status(&sm, (cudaStream_t)stream), "device status");
    const int any = st ? st : (sb ? sb : sm);
    if (any != 0) return fail(any, "a kernel's bounded wait expired");
    return BT_OK;
}

// ---------------------------------------------------------------------------
// Surrogate MLP building blocks
// ---------------------------------------------------------------------------

extern "C" int bt_mlp_gemm(const void* A, const void* B, int M, int N, int K, int bn, int splitk, int mode,
                           const float* bias, float* out32, float* zs, void* h16, void* h16t, void* stream) {
    if (!A || !B) return fail(BT_ERR_ARG, "mlp gemm: null operand");
    if (M <= 0 || N <= 0 || K <= 0 || M % 128 || (bn != 128 && bn != 256) || N % bn || splitk < 1 ||
        K % (64 * splitk))
        return fail(BT_ERR_ARG, "mlp gemm: M % 128, N % bn (128 or 256) and K % (64 * splitk) must be 0");
    if (((uintptr_t)A & 15) || ((uintptr_t)B & 15)) return fail(BT_ERR_ARG, "mlp gemm: operands must be 16-byte aligned");
    switch (mode) {
    case MLP_EPI_F32:
        if (!out32) return fail(BT_ERR_ARG, "mlp gemm: mode 0 needs out32");
        break;
    case MLP_EPI_BIAS:
        if (!out32 || !bias || splitk != 1) return fail(BT_ERR_ARG, "mlp gemm: mode 1 needs out32, bias, splitk 1");
        break;
    case MLP_EPI_GELU:
        if (!h16 || !bias || splitk != 1) return fail(BT_ERR_ARG, "mlp gemm: mode 2 needs h16, bias, splitk 1");
        break;
    case MLP_EPI_DGELU:
        if (!h16 || !zs || splitk != 1) return fail(BT_ERR_ARG, "mlp gemm: mode 3 needs h16, zs, splitk 1");
        break;
    default:
        return fail(BT_ERR_ARG, "mlp gemm: bad mode");
    }
    MlpGemmArgs a;
    memset(&a, 0, sizeof(a));
    a.M = M;
    a.N = N;
    a.K = K;
    a.bn = bn;
    a.mode = mode;
    a.bias = bias;
    a.out32 = out32;
    a.zs = zs;
    a.h16 = (__nv_bfloat16*)h16;
    a.h16t = (__nv_bfloat16*)h16t;
    CUDA_TRY(bt_launch_mlp_gemm((const __nv_bfloat16*)A, (const __nv_bfloat16*)B, a, splitk, (cudaStream_t)stream),
             "mlp gemm");
    return BT_OK;
}

extern "C" int bt_mlp_pack(const float* x, int rows, int cols, int ld_out, int rows_out, void* out, void* out_t,
                           void* stream) {
    if (!x || !out || rows < 0 || cols < 0 || rows_out < rows || ld_out < cols)
        return fail(BT_ERR_ARG, "mlp pack: bad arguments");
    if (rows_out == 0) return BT_OK;
    CUDA_TRY(bt_launch_mlp_pack(x, rows, cols, ld_out, rows_out, (__nv_bfloat16*)out, (__nv_bfloat16*)out_t,
                                (cudaStream_t)stream), "mlp pack");
    return BT_OK;
}

extern "C" int bt_mlp_loss(const float* y, int ldy, const float* t, const float* wt, int rows, int rows_valid,
                           int ncols, int err_col, float err_weight, int ld_out, void* dz, void* dzt, float* loss,
                           void* stream) {
    if (!y || !t || !dz || !dzt || rows_valid < 1 || rows_valid > rows || ncols > ld_out || ncols > ldy ||
        err_col >= ld_out || err_col >= ldy)
        return fail(BT_ERR_ARG, "mlp loss: bad arguments");
    CUDA_TRY(bt_launch_mlp_loss(y, ldy, t, wt, rows, rows_valid, ncols, err_col, err_weight, ld_out,
                                (__nv_bfloat16*)dz, (__nv_bfloat16*)dzt, loss, (cudaStream_t)stream), "mlp loss");
    return BT_OK;
}

extern "C" int bt_mlp_colsum(const void* xt, int rows, int cols, float* out, void* stream) {
    if (!xt || !out || rows < 1 || cols < 1) return fail(BT_ERR_ARG, "mlp colsum: bad arguments");
    CUDA_TRY(bt_launch_mlp_colsum((const __nv_bfloat16*)xt, rows, cols, out, (cudaStream_t)stream), "mlp colsum");
    return BT_OK;
}

extern "C" int bt_surrogate_combine(const float* feat, int nfeat, int nlin, const int* grp, const float* theta,
                                    const float* y, int ldy, const double* wl, double scale, int J, int err_col,
                                    double* out, float* err_nm, int n, void* stream) {
    if (n < 0 || (n > 0 && (!feat || !grp || !theta || !y || !wl || !out)) || nlin > nfeat || J < 1 || J > ldy ||
        err_col >= ldy || ((uintptr_t)theta & 7))
        return fail(BT_ERR_ARG, "surrogate combine: bad arguments");
    CUDA_TRY(bt_launch_surrogate_combine(feat, nfeat, nlin, grp, theta, y, ldy, wl, scale, J, err_col, out, err_nm, n,
                                         (cudaStream_t)stream), "surrogate combine");
    return BT_OK;
}

extern "C" int bt_mlp_gather(const long long* perm, const long long* k_in_epoch, const float* x_all, int nxc,
                             const float* t_all, int ntc, int batch, float* xb, float* tb, void* stream) {
    if (batch < 0 || (batch > 0 && (!perm || !k_in_epoch || !x_all || !t_all || !xb || !tb)) || nxc < 1 || ntc < 1)
        return fail(BT_ERR_ARG, "mlp gather: bad arguments");
    CUDA_TRY(bt_launch_mlp_gather(perm, k_in_epoch, x_all, nxc, t_all, ntc, batch, xb, tb, (cudaStream_t)stream),
             "mlp gather");
    return BT_OK;
}

extern "C" int bt_mlp_schedule(long long* k_in_epoch, long long* step, const float* table, long long total,
                               float* hyper, void* stream) {
    if (!k_in_epoch || !step || !table || !hyper || total < 1) return fail(BT_ERR_ARG, "mlp schedule: bad arguments");
    CUDA_TRY(bt_launch_mlp_schedule(k_in_epoch, step, table, total, hyper, (cudaStream_t)stream), "mlp schedule");
    return BT_OK;
}

extern "C" int bt_surrogate_guard(const float* feat, int nfeat, int ndof, const int* grp, const float* m0,
                                  const float* jac, const float* reach, int K, double band_abs, double band_rel,
                                  int* flag, int n, void* stream) {
    if (n < 0 || (n > 0 && (!feat || !grp || !m0 || !jac || !flag)) || ndof < 0 || ndof > nfeat || K < 32 ||
        (K % 32) != 0 || !(band_abs >= 0.0) || !(band_rel >= 0.0))
        return fail(BT_ERR_ARG, "surrogate guard: bad arguments");
    CUDA_TRY(bt_launch_surrogate_guard(feat, nfeat, ndof, grp, m0, jac, reach, K, (float)band_abs, (float)band_rel,
                                       flag, n, (cudaStream_t)stream), "surrogate guard");
    return BT_OK;
}

extern "C" int bt_mlp_adam(const float* partials, int nsplit, const float* grad, long long n, float* w, float* m,
                           float* v, float lr, float b1, float b2, float eps, float bc1, float bc2, int rows, int cols,
                           void* w16, void* w16t, void* stream) {
    if (!w || !m || !v || n < 1 || (nsplit > 0 && !partials) || (long long)rows * cols != n || !(bc1 > 0.f) ||
        !(bc2 > 0.f))
        return fail(BT_ERR_ARG, "mlp adam: bad arguments");
    CUDA_TRY(bt_launch_mlp_adam(partials, nsplit, grad, n, w, m, v, lr, b1, b2, eps, bc1, bc2, rows, cols,
                                (__nv_bfloat16*)w16, (__nv_bfloat16*)w16t, nullptr, (cudaStream_t)stream), "mlp adam");
    return BT_OK;
}

extern "C" int bt_mlp_adam_dev(const float* partials, int nsplit, const float* grad, long long n, float* w, float* m,
                               float* v, const float* hyper, float b1, float b2, float eps, int rows, int cols,
                               void* w16, void* w16t, void* stream) {
    if (!w || !m || !v || !hyper || n < 1 || (nsplit > 0 && !partials) || (long long)rows * cols != n)
        return fail(BT_ERR_ARG, "mlp adam (device schedule): bad arguments");
    CUDA_TRY(bt_launch_mlp_adam(partials, nsplit, grad, n, w, m, v, 0.f, b1, b2, eps, 1.f, 1.f, rows, cols,
                                (__nv_bfloat16*)w16, (__nv_bfloat16*)w16t, hyper, (cudaStream_t)stream),
             "mlp adam (device schedule)");
    return BT_OK;
}

// ---------------------------------------------------------------------------
// Batched wavefronts / Zernike fits
// ---------------------------------------------------------------------------

struct bt_batch {
    unsigned char* d_blob = nullptr;
    int blob_bytes = 0;
    int ntrace = 0;
    int nvar = 0;
    int var_stage[BT_BATCH_MAX_VAR] = {0};
    int modal_surf = -1;
    int nmodes = 0;
    double stop_dr[3] = {0, 0, 0};
    double stop_drot[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    double sphere_R = 0.0;
    double pupil = 0.0;
    double r_in2 = 0.0, r_out2 = 0.0;
    int jmax = 0;
    int side = 0;
    double* d_cart = nullptr;
    std::vector<long long> off;  // per grid size, -1 where absent
    long long* d_off = nullptr;
    double* d_basis = nullptr;
    double* d_gref = nullptr;
    int* d_counter = nullptr;
    int* d_jobcnt = nullptr;  // finished chunks per queue entry (split jobs)
    double* d_scratch = nullptr;  // per block: OPD of each ray of its job
    long long scratch_stride = 0;
    std::mutex mu;
    cudaGraphExec_t gexec = nullptr;
    std::vector<unsigned char> gkey;
};

static void batch_free(bt_batch* b) {
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->d_blob) cudaFree(b->d_blob);
    if (b->d_cart) cudaFree(b->d_cart);
    if (b->d_off) cudaFree(b->d_off);
    if (b->d_basis) cudaFree(b->d_basis);
    if (b->d_gref) cudaFree(b->d_gref);
    if (b->d_counter) cudaFree(b->d_counter);
    if (b->d_jobcnt) cudaFree(b->d_jobcnt);
    if (b->d_scratch) cudaFree(b->d_scratch);
    delete b;
}

extern "C" void bt_batch_destroy(bt_batch* b) {
    if (b) batch_free(b);
}

extern "C" int bt_batch_create(const bt_batch_desc* d, bt_batch** out) {
    if (!d || !out) return fail(BT_ERR_ARG, "batch: null argument");
    if (d->nstages < 1 || d->nstages + 1 > BT_MAX_STAGES) return fail(BT_ERR_UNSUPPORTED, "batch: stage count");
    if (!d->kinds || !d->surfaces || !d->dr || !d->drot) return fail(BT_ERR_ARG, "batch: null stage arrays");
    if (d->nvar < 0 || d->nvar > BT_BATCH_MAX_VAR || (d->nvar > 0 && !d->var_stages))
        return fail(BT_ERR_ARG, "batch: at most 8 varying stages");
    if (d->jmax < 1 || d->jmax > BT_BATCH_MAX_J) return fail(BT_ERR_UNSUPPORTED, "batch: jmax must be 1..32");
    if (d->side < 1 || !d->basis) return fail(BT_ERR_ARG, "batch: missing fit basis");
    if (!d->sphere) return fail(BT_ERR_ARG, "batch: missing reference sphere");
    if (!(d->pupil_size > 0.0) || !(d->r_outer >= d->r_inner)) return fail(BT_ERR_ARG, "batch: pupil / annulus");
    const bool modal = d->modal_stage >= 0;
    if (modal) {
        if ((size_t)d->modal_stage >= d->nstages) return fail(BT_ERR_ARG, "batch: modal stage out of range");
        if (d->nmodes < 4 || d->nmodes % 4 != 0 || !d->modes || d->modal_nx < 2 || d->modal_ny < 2 ||
            !(d->modal_grid[2] > 0.0) || !(d->modal_grid[3] > 0.0))
            return fail(BT_ERR_ARG, "batch: modal tables (nmodes a positive multiple of 4, grid >= 2x2)");
        if (((uintptr_t)d->modes & 15) != 0) return fail(BT_ERR_ARG, "batch: mode data must be 16-byte aligned");
    }
    bt_batch* b = new bt_batch;
    ProgBuilder pb;
    for (size_t k = 0; k < d->nstages; k++) {
        const int kind = d->kinds[k];
        if (kind != BT_ST_INTERSECT && kind != BT_ST_REFLECT && kind != BT_ST_REFRACT) {
            batch_free(b);
            return fail(BT_ERR_ARG, "batch: bad stage kind");
        }
        if (!d->surfaces[k]) {
            batch_free(b);
            return fail(BT_ERR_ARG, "batch: null surface");
        }
        bt_stage st = blank_stage(kind);
        set_transform(st, d->dr + 3 * k, d->drot + 9 * k);
        st.surf = pb.add_surface(d->surfaces[k]);
        if (st.surf < 0) {
            batch_free(b);
            return BT_ERR_CUDA;
        }
        if (modal && (int)k == d->modal_stage) {
            bt_surf m = blank_surf(BT_S_MODAL);
            m.n = d->modal_nx;
            m.m = d->modal_ny;
            for (int i = 0; i < 4; i++) m.p[i] = d->modal_grid[i];
            m.p[4] = d->modal_use_nan ? 1.0 : 0.0;
            m.p[5] = (double)d->nmodes;
            m.p[6] = 1.0 / d->modal_grid[2];
            m.p[7] = 1.0 / d->modal_grid[3];
            m.off = (int32_t)pb.pool.size();
            m.tab = reinterpret_cast<const double*>(d->modes);
            pb.pool.insert(pb.pool.end(), (size_t)d->nmodes, 0.0);  // amplitudes, per job
            const int root = st.surf;
            const int nrec = (int)pb.surfs.size();
            if (pb.surfs[root].kind == BT_S_SUM && pb.surfs[root].m + pb.surfs[root].n == nrec &&
                pb.surfs[root].n < BT_MAX_SUM_CHILDREN) {
                pb.surfs.push_back(m);
                pb.surfs[root].n += 1;
                b->modal_surf = nrec;
            } else if (pb.surfs[root].kind != BT_S_SUM && root == nrec - 1) {
                pb.surfs.push_back(m);
                bt_surf sum;
                memset(&sum, 0, sizeof(sum));
                sum.kind = BT_S_SUM;
                sum.n = 2;
                sum.m = root;
                pb.surfs.push_back(sum);
                st.surf = nrec + 1;
                b->modal_surf = nrec;
            } else {
                batch_free(b);
                return fail(BT_ERR_UNSUPPORTED, "batch: cannot add the bending term to this surface");
            }
        }
        if (kind == BT_ST_REFRACT) {
            if (!d->media || !d->media[k]) {
                batch_free(b);
                return fail(BT_ERR_ARG, "batch: refracting stage without a medium");
            }
            st.medium = pb.add_medium(d->media[k]);
        }
        if (d->obscurations && d->obscurations[k]) pb.add_obsc(d->obscurations[k], &st.obsc_begin, &st.obsc_end);
        pb.stages.push_back(st);
    }
    for (int v = 0; v < d->nvar; v++) {
        const int k = d->var_stages[v];
        if (k < 0 || (size_t)k >= d->nstages) {
            batch_free(b);
            return fail(BT_ERR_ARG, "batch: varying stage out of range");
        }
        pb.stages[k].identity = 0;
        b->var_stage[v] = k;
    }
    bt_stage sph = blank_stage(BT_ST_INTERSECT);
    sph.identity = 0;
    sph.surf = pb.add_surface(d->sphere);
    if (sph.surf < 0) {
        batch_free(b);
        return BT_ERR_CUDA;
    }
    pb.stages.push_back(sph);
    std::vector<unsigned char> blob = pb.blob();
    if (blob.size() > kMaxBlobBytes) {
        batch_free(b);
        return fail(BT_ERR_UNSUPPORTED, "batch: descriptor too large");
    }
    b->blob_bytes = (int)blob.size();
    b->ntrace = (int)d->nstages;
    b->nvar = d->nvar;
    b->nmodes = modal ? d->nmodes : 0;
    for (int i = 0; i < 3; i++) b->stop_dr[i] = d->stop_dr[i];
    for (int i = 0; i < 9; i++) b->stop_drot[i] = d->stop_drot[i];
    b->sphere_R = d->sphere_radius;
    b->pupil = d->pupil_size;
    b->r_in2 = d->r_inner * d->r_inner;
    b->r_out2 = d->r_outer * d->r_outer;
    b->jmax = d->jmax;
    b->side = d->side;
    b->off.assign(BT_BATCH_MAX_NX + 1, -1);
    const size_t ncart = (size_t)d->jmax * d->side * d->side;
    const size_t ngref = (size_t)(BT_BATCH_MAX_NX + 1) * d->jmax * d->jmax;
    cudaError_t e = cudaMalloc((void**)&b->d_blob, blob.size());
    if (e == cudaSuccess) e = cudaMemcpy(b->d_blob, blob.data(), blob.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_cart, ncart * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(b->d_cart, d->basis, ncart * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_off, b->off.size() * sizeof(long long));
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_off, b->off.data(), b->off.size() * sizeof(long long), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_gref, ngref * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(b->d_gref, 0, ngref * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_counter, sizeof(int));
    if (e == cudaSuccess)
        e = cudaMalloc((void**)&b->d_jobcnt, sizeof(int) * (size_t)bt_sm_count() * BT_BATCH_MAX_CTAS_PER_SM);
    if (e == cudaSuccess) e = bt_batch_set_smem_limit();
    if (e != cudaSuccess) {
        cudaGetLastError();  // leave no error behind for the next launch check
        batch_free(b);
        return cuda_fail(e, "batch: set-up");
    }
    *out = b;
    return BT_OK;
}

extern "C" int bt_batch_prepare(bt_batch* b, int n, const int* nx_values, void* stream) {
    if (!b || (n > 0 && !nx_values)) return fail(BT_ERR_ARG, "batch prepare: null argument");
    std::lock_guard<std::mutex> lock(b->mu);
    std::vector<char> want(BT_BATCH_MAX_NX + 1, 0);
    bool fresh = false;
    for (int i = 0; i < n; i++) {
        const int nx = nx_values[i];
        if (nx < 2 || nx > BT_BATCH_MAX_NX) return fail(BT_ERR_ARG, "batch prepare: grid size must be 2..512");
        want[nx] = 1;
        if (b->off[nx] < 0) fresh = true;
    }
    if (!fresh) return BT_OK;
    for (int nx = 0; nx <= BT_BATCH_MAX_NX; nx++)
        if (b->off[nx] >= 0) want[nx] = 1;
    std::vector<long long> off(BT_BATCH_MAX_NX + 1, -1);
    std::vector<int> list;
    long long total = 0;
    for (int nx = 2; nx <= BT_BATCH_MAX_NX; nx++) {
        if (!want[nx]) continue;
        off[nx] = total;
        total += (long long)nx * nx * b->jmax;
        list.push_back(nx);
    }
    cudaStream_t s = (cudaStream_t)stream;
    double* basis = nullptr;
    int* d_list = nullptr;
    cudaError_t e = cudaMalloc((void**)&basis, (size_t)total * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&d_list, list.size() * sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_list, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->d_off, off.data(), off.size() * sizeof(long long), cudaMemcpyHostToDevice, s);
    for (size_t i = 0; e == cudaSuccess && i < list.size(); i++)
        e = bt_launch_batch_tables(list[i], b->pupil, b->d_cart, b->jmax, b->side, basis + off[list[i]], s);
    if (e == cudaSuccess)
        e = bt_launch_batch_gref(d_list, (int)list.size(), b->pupil, b->r_in2, b->r_out2, basis, b->d_off, b->jmax,
                                 b->d_gref, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (d_list) cudaFree(d_list);
    if (e != cudaSuccess) {
        if (basis) cudaFree(basis);
        // device offsets may already name the new tables: mark all absent
        std::vector<long long> none(BT_BATCH_MAX_NX + 1, -1);
        cudaMemcpy(b->d_off, none.data(), none.size() * sizeof(long long), cudaMemcpyHostToDevice);
        b->off = none;
        if (b->d_basis) cudaFree(b->d_basis);
        b->d_basis = nullptr;
        return cuda_fail(e, "batch prepare");
    }
    // OPD scratch for the largest grid, one slot per block the launch may run
    long long maxray = 0;
    for (int nx : list) maxray = std::max(maxray, (long long)nx * nx);
    if (maxray > b->scratch_stride) {
        double* sc = nullptr;
        e = cudaMalloc((void**)&sc, sizeof(double) * (size_t)maxray * bt_sm_count() * BT_BATCH_MAX_CTAS_PER_SM);
        if (e != cudaSuccess) {
            cudaFree(basis);
            return cuda_fail(e, "batch prepare: scratch");
        }
        if (b->d_scratch) cudaFree(b->d_scratch);
        b->d_scratch = sc;
        b->scratch_stride = maxray;
    }
    if (b->d_basis) cudaFree(b->d_basis);
    b->d_basis = basis;
    b->off = off;
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
        b->gkey.clear();
    }
    return BT_OK;
}

static int batch_args(bt_batch* b, int nstates, const double* xf, const double* det, const double* amps,
                      const int* nx, const double* wavelength, int nfields, const double* fields, const int* order,
                      int nqueue, double* coefs, int* status, int threads, int ctas_per_sm, int niter,
                      BatchArgs* a) {
    if (!b) return fail(BT_ERR_ARG, "batch: null plan");
    if (nstates < 0 || nfields < 0) return fail(BT_ERR_ARG, "batch: negative sizes");
    if ((long long)nstates * nfields > 0x7fffffffLL) return fail(BT_ERR_UNSUPPORTED, "batch: too many jobs");
    if (threads < 32 || threads > BT_BATCH_MAX_THREADS || threads % 32 != 0)
        return fail(BT_ERR_ARG, "batch: threads must be 32.." + std::to_string(BT_BATCH_MAX_THREADS) +
                                    ", a multiple of 32");
    if (ctas_per_sm < 1 || ctas_per_sm > BT_BATCH_MAX_CTAS_PER_SM)
        return fail(BT_ERR_ARG, "batch: ctas_per_sm must be 1..8");
    if (niter < 0) return fail(BT_ERR_ARG, "batch: negative niter");
    if (bt_batch_smem_layout(b->blob_bytes, threads, b->jmax).total > (size_t)bt_batch_smem_max())
        return fail(BT_ERR_UNSUPPORTED, "batch: shared memory exceeds the limit for this block size");
    const int njobs = nstates * nfields;
    if (njobs > 0 && (!nx || !wavelength || !fields || !order || !coefs || !status || !det ||
                      (b->nvar > 0 && !xf) || (b->nmodes > 0 && !amps)))
        return fail(BT_ERR_ARG, "batch: null array");
    if (!b->d_basis && njobs > 0) return fail(BT_ERR_ARG, "batch: no grid size prepared");
    memset(a, 0, sizeof(*a));
    a->xf = xf;
    a->det = det;
    a->amps = amps;
    a->nxs = nx;
    a->wl = wavelength;
    a->field = fields;
    a->basis = b->d_basis;
    a->basis_off = b->d_off;
    a->gref = b->d_gref;
    a->order = order;
    a->counter = b->d_counter;
    a->scratch = b->d_scratch;
    a->scratch_stride = b->scratch_stride;
    a->coefs = coefs;
    a->status = status;
    a->njobs = njobs;
    a->nqueue = (nqueue <= 0 || nqueue > njobs) ? njobs : nqueue;
    a->jobcnt = b->d_jobcnt;
    // fewer jobs than blocks: each job's rays are split over several blocks
    // (scratch rows and chunk counters per queue entry, both sized for
    // SMs x BT_BATCH_MAX_CTAS_PER_SM entries)
    const long long blocks = (long long)bt_sm_count() * ctas_per_sm;
    a->nchunk = 1;
    if (a->nqueue > 0 && a->nqueue < blocks) {
        const long long c = (blocks + a->nqueue - 1) / a->nqueue;
        a->nchunk = (int)(c < 32 ? c : 32);
    }
    a->nfields = nfields;
    a->nx_cap = BT_BATCH_MAX_NX;
    a->nvar = b->nvar;
    for (int i = 0; i < BT_BATCH_MAX_VAR; i++) a->var_stage[i] = b->var_stage[i];
    a->ntrace = b->ntrace;
    a->modal_surf = b->modal_surf;
    a->nmodes = b->nmodes;
    for (int i = 0; i < 3; i++) a->stop_dr[i] = b->stop_dr[i];
    for (int i = 0; i < 9; i++) a->stop_drot[i] = b->stop_drot[i];
    a->sphere_R = b->sphere_R;
    a->pupil = b->pupil;
    a->r_in2 = b->r_in2;
    a->r_out2 = b->r_out2;
    a->jmax = b->jmax;
    a->niter = niter;
    return BT_OK;
}

extern "C" int bt_batch_zernike(bt_batch* b, int nstates, const double* xf, const double* det, const double* amps,
                                const int* nx, const double* wavelength, int nfields, const double* fields,
                                const int* order, int nqueue, double* coefs, int* status, int threads,
                                int ctas_per_sm, int niter, void* stream) {
    BatchArgs a;
    int rc = batch_args(b, nstates, xf, det, amps, nx, wavelength, nfields, fields, order, nqueue, coefs, status,
                        threads, ctas_per_sm, niter, &a);
    if (rc != BT_OK) return rc;
    std::lock_guard<std::mutex> lock(b->mu);
    CUDA_TRY(bt_launch_batch_zernike(b->d_blob, b->blob_bytes, a, threads, ctas_per_sm, (cudaStream_t)stream),
             "batch zernike");
    return BT_OK;
}

extern "C" int bt_batch_zernike_graph(bt_batch* b, int nstates, const double* xf, const double* det,
                                      const double* amps, const int* nx, const double* wavelength, int nfields,
                                      const double* fields, const int* order, int nqueue, double* coefs,
                                      int* status, int threads, int ctas_per_sm, int niter, void* stream) {
    if (!stream) return fail(BT_ERR_ARG, "batch graph: the legacy default stream cannot be captured");
    BatchArgs a;
    int rc = batch_args(b, nstates, xf, det, amps, nx, wavelength, nfields, fields, order, nqueue, coefs, status,
                        threads, ctas_per_sm, niter, &a);
    if (rc != BT_OK) return rc;
    if (a.njobs == 0) return BT_OK;
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<unsigned char> key(sizeof(a) + 3 * sizeof(int) + sizeof(void*));
    memcpy(key.data(), &a, sizeof(a));
    const int extra[3] = {threads, ctas_per_sm, niter};
    memcpy(key.data() + sizeof(a), extra, sizeof(extra));
    memcpy(key.data() + sizeof(a) + sizeof(extra), &stream, sizeof(void*));
    std::lock_guard<std::mutex> lock(b->mu);
    if (!b->gexec || b->gkey != key) {
        if (b->gexec) {
            cudaGraphExecDestroy(b->gexec);
            b->gexec = nullptr;
        }
        cudaGraph_t g = nullptr;
        CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "batch graph capture");
        cudaError_t le = bt_launch_batch_zernike(b->d_blob, b->blob_bytes, a, threads, ctas_per_sm, s);
        cudaError_t ce = cudaStreamEndCapture(s, &g);
        if (le != cudaSuccess || ce != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return cuda_fail(le != cudaSuccess ? le : ce, "batch graph capture");
        }
        cudaError_t ie = cudaGraphInstantiate(&b->gexec, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            b->gexec = nullptr;
            return cuda_fail(ie, "batch graph instantiate");
        }
        b->gkey = key;
    }
    CUDA_TRY(cudaGraphLaunch(b->gexec, s), "batch graph launch");
    return BT_OK;
}
