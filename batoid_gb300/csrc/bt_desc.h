// Flat, pointer-free (except bicubic tables) description of an optic, packed
// on the host and staged into shared memory by the trace kernels.
//
// A "program" is a byte blob:
//   [bt_prog_header][bt_stage x nstages][bt_surf x nsurf][bt_medium x nmedia]
//   [bt_obsc x nobsc][double pool x npool]
// every section 16-byte aligned, the whole blob padded to 16 bytes so that it
// can be moved with one cp.async.bulk copy.
//
// One stage is one Interface of the reference optic tree (batoid/optic.py:391-424):
// coordinate transform into the surface frame, intersection, interaction
// (reflect / refract / pass through) and the interface's obscuration.
#pragma once
#include <stdint.h>

#define BT_MAX_SUM_CHILDREN 16
#define BT_MAX_OBSC_STACK   30

enum bt_surf_kind {
    BT_S_PLANE = 0,
    BT_S_TILTED = 1,
    BT_S_SPHERE = 2,
    BT_S_PARABOLOID = 3,
    BT_S_QUADRIC = 4,
    BT_S_ASPHERE = 5,
    BT_S_POLY = 6,
    BT_S_BICUBIC = 7,
    BT_S_SUM = 8,
    BT_S_MODAL = 9
};

// Surface parameter slots (p[]):
//  TILTED:     p0=tanx p1=tany p2=sqrt(1-tanx^2-tany^2)
//  SPHERE:     p0=R p1=R*R p2=1/R p3=1/R/R
//  PARABOLOID: p0=R p1=1/R p2=1/2/R
//  QUADRIC/ASPHERE: p0=R p1=conic p2=R*R p3=1/R/R p4=conic+1 p5=1/(conic+1)
//              p6=R/(conic+1) p7=R*R/(conic+1)/(conic+1) p8=(conic+1)/R/R
//              p9=1/R (0 if R == 0) p10=1 if the sag may use (1-q)*R/(conic+1)
//              ASPHERE: n coefs at pool[off], n dz/dr coefs at pool[off+n],
//              then both again as float-float pairs (one double slot each)
//  POLY:       p0=xorigin p1=yorigin p2=1 if triangular (square, coefficients
//              with i + j >= size zero, also in the gradient arrays);
//              n=xsize m=ysize;
//              coefs pool[off .. off+n*m), gradx then grady ((n-1)*(m-1) each),
//              then the three arrays again as float-float pairs
//  BICUBIC:    p0=x0 p1=y0 p2=dx p3=dy p4=use_nan; n=nx m=ny; tab = 4 arrays
//              (z, dzdx, dzdy, d2zdxdy), each nx*ny, row-major [iy][ix]
//  SUM:        n=#children m=index of first child (children are contiguous)
//  MODAL:      sum_m a_m * table_m of nmodes bicubic tables on one grid, the
//              amplitudes a_m supplied per job by the batched kernel:
//              p0=x0 p1=y0 p2=dx p3=dy p4=use_nan p5=nmodes (multiple of 4)
//              p6=1/dx p7=1/dy;
//              n=nx m=ny; off = pool index of the nmodes amplitudes, stored
//              as float-float pairs; tab = FP32 mode data laid out
//              [iy][ix][q][mode] with q = z, dz/dx, dz/dy, d2z/dxdy.
//              Only the batched wavefront kernel evaluates it.
typedef struct bt_surf {
    int32_t kind;
    int32_t n;
    int32_t m;
    int32_t off;
    double p[12];
    const double* tab;
    int32_t ffc;   // pool index of the float-float constants (see below), -1 if none
    int32_t pad_;
} bt_surf;  // 128 bytes

// Float-float constants (one (hi, lo) float pair per double slot of the
// pool, at index ffc) used by the trace kernel's float-float path:
//  SPHERE:     R, R^2, 1/R, 1/R^2
//  PARABOLOID: R, 1/R, 1/(2R)
//  QUADRIC/ASPHERE: R, 1/(1+k), R/(1+k), R^2/(1+k)^2, (1+k)/R^2, 1/R
//  POLY:       xorigin, yorigin

enum bt_medium_kind {
    BT_M_CONST = 0,
    BT_M_TABLE = 1,
    BT_M_SELLMEIER = 2,
    BT_M_SUMITA = 3,
    BT_M_AIR = 4
};

// CONST: p0=n p1=1/n p2=(n as a float-float pair) p3=(1/n as a pair).
// TABLE: n entries, args at pool[off], vals at pool[off+n].
// SELLMEIER: B1 B2 B3 C1 C2 C3 (and as float-float pairs at pool[off]).
// SUMITA: A0..A5.
// AIR: p0=P(mmHg) p1=T(C) p2=W(mmHg)
typedef struct bt_medium {
    int32_t kind;
    int32_t n;
    int32_t off;
    int32_t pad_;
    double p[6];
} bt_medium;  // 64 bytes

enum bt_obsc_op {
    BT_O_CIRCLE = 0,     // p0=r p1=x0 p2=y0; p3..p5 the same as float-float pairs
    BT_O_ANNULUS = 1,    // p0=inner p1=outer p2=x0 p3=y0; p4, p5 inner, outer as pairs
    BT_O_RECT = 2,       // p0=w p1=h p2=x0 p3=y0 p4=sin(th) p5=cos(th)
    BT_O_RAY = 3,        // p0=w p1=x0 p2=y0 p3=sin(th) p4=cos(th)
    BT_O_POLYGON = 4,    // n vertices, xs at pool[off], ys at pool[off+n]
    BT_O_NEGATION = 5,   // pops 1, pushes !v
    BT_O_UNION = 6,      // pops n, pushes OR
    BT_O_INTERSECTION = 7 // pops n, pushes AND
};

typedef struct bt_obsc {
    int32_t op;
    int32_t n;
    int32_t off;
    int32_t pad_;
    double p[6];
} bt_obsc;  // 64 bytes, one postfix instruction

enum bt_stage_kind {
    BT_ST_INTERSECT = 0,  // Detector / Baffle / plain Interface
    BT_ST_REFLECT = 1,    // Mirror
    BT_ST_REFRACT = 2,    // RefractiveInterface
    BT_ST_OBSCURE = 3,    // obscuration only (no transform, no surface)
    BT_ST_SCREEN = 4      // OPDScreen: intersect, deflect by the screen's gradient
};

typedef struct bt_stage {
    int32_t kind;
    int32_t surf;        // index of the surface's root descriptor
    int32_t medium;      // refract: outgoing medium index; else -1
    int32_t obsc_begin;  // postfix program [obsc_begin, obsc_end), empty = none
    int32_t obsc_end;
    int32_t identity;    // 1: dr == 0 and drot == I; 2: drot == I (translation); 0: general
    int32_t coated;      // 1: multiply flux by coat_r (reflect) / coat_t
    int32_t screen;      // screen: root descriptor of the OPD surface, else -1
    double dr[3];
    double drot[9];      // column-major, as the reference passes it
    double coat_r;
    double coat_t;
} bt_stage;  // 144 bytes

typedef struct bt_prog_header {
    int32_t nstages;
    int32_t nsurf;
    int32_t nmedia;
    int32_t nobsc;
    int32_t npool;
    int32_t total_bytes;  // multiple of 16
    int32_t off_stages;   // byte offsets from the blob start
    int32_t off_surfs;
    int32_t off_media;
    int32_t off_obsc;
    int32_t off_pool;
    int32_t pad_[5];
} bt_prog_header;  // 64 bytes

#ifdef __cplusplus
static_assert(sizeof(bt_surf) == 128, "bt_surf layout");
static_assert(sizeof(bt_medium) == 64, "bt_medium layout");
static_assert(sizeof(bt_obsc) == 64, "bt_obsc layout");
static_assert(sizeof(bt_stage) == 144, "bt_stage layout");
static_assert(sizeof(bt_prog_header) == 64, "bt_prog_header layout");
#endif
