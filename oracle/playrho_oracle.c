/*
 * playrho_oracle.c -- CPU restatement of the PlayRho 2.0.0 regular-phase world
 * step (TEST INFRASTRUCTURE ONLY; see playrho_oracle.h).
 *
 * Every routine names the reference function it follows (paths are inside the
 * PlayRho project, Library/...).  The order of floating-point operations follows
 * the reference so that, compiled with -ffp-contract=off, the FP32 build gives
 * the reference's FP32 numbers.  Compile with -DOR_DOUBLE for the FP64 oracle.
 *
 * Scope: disks, convex polygons and edges (one child per shape), revolute
 * joints, contact persistence with fattened/displaced proxy AABBs, island
 * discovery by depth-first search, sequential-impulse Gauss-Seidel velocity
 * solve with the 2-point block solver, NGS position solve, sleep, and the TOI
 * phase (StepConf::doToi): GJK distance, conservative advancement by separating
 * axes, and the sequential sub-stepping of time-of-impact events.
 */
#include "playrho_oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef or_real real;

#ifdef OR_DOUBLE
#define RSQRT sqrt
#define RCOS cos
#define RSIN sin
#define RHYPOT hypot
#define RNEXT nextafter
#define RMIN_NORMAL DBL_MIN
#define RMAXV DBL_MAX
#else
#define RSQRT sqrtf
#define RCOS cosf
#define RSIN sinf
#define RHYPOT hypotf
#define RNEXT nextafterf
#define RMIN_NORMAL FLT_MIN
#define RMAXV FLT_MAX
#endif
#define R(x) ((real)(x))
#define RINF ((real)INFINITY)

/* ------------------------------------------------------------------------- */
/* Small value types: Vector2, UnitVec, Transformation, Position/Velocity.    */
/* ------------------------------------------------------------------------- */
typedef struct { real x, y; } v2;
typedef struct { v2 p; v2 q; } xf_t;       /* q = (cos, sin) as UnitVec */
typedef struct { v2 lin; real ang; } pos_t; /* Position and Velocity */

static inline v2 V(real x, real y) { v2 r = {x, y}; return r; }
static inline v2 vadd(v2 a, v2 b) { return V(a.x + b.x, a.y + b.y); }
static inline v2 vsub(v2 a, v2 b) { return V(a.x - b.x, a.y - b.y); }
static inline v2 vneg(v2 a) { return V(-a.x, -a.y); }
/* Vector * scalar (Vector.hpp:497-504): a[i] * s. */
static inline v2 vmul(v2 a, real s) { return V(a.x * s, a.y * s); }
/* Vector / scalar (Vector.hpp:511-519): a[i] * (1 / s). */
static inline v2 vdiv(v2 a, real s) { const real inv = R(1) / s; return V(a.x * inv, a.y * inv); }
/* Dot (Math.hpp:320-333): accumulates from zero. */
static inline real dot(v2 a, v2 b) { real r = R(0); r += a.x * b.x; r += a.y * b.y; return r; }
/* Cross (Math.hpp:365-386). */
static inline real cross(v2 a, v2 b) { const real m = a.x * b.y; const real s = a.y * b.x; return m - s; }
/* GetMagnitudeSquared (Math.hpp:274-283). */
static inline real mag2(v2 a) { real r = R(0); r += a.x * a.x; r += a.y * a.y; return r; }
/* GetRevPerpendicular (-y, x) and GetFwdPerpendicular (y, -x) (UnitVec.hpp:364-378). */
static inline v2 revperp(v2 a) { return V(-a.y, a.x); }
static inline v2 fwdperp(v2 a) { return V(a.y, -a.x); }
/* Rotate / InverseRotate (d2/Math.hpp, Rotate and InverseRotate templates). */
static inline v2 rotate(v2 v, v2 q) {
    const real nx = (q.x * v.x) - (q.y * v.y);
    const real ny = (q.y * v.x) + (q.x * v.y);
    return V(nx, ny);
}
static inline v2 invrotate(v2 v, v2 q) {
    const real nx = (q.x * v.x) + (q.y * v.y);
    const real ny = (q.x * v.y) - (q.y * v.x);
    return V(nx, ny);
}
/* UnitVec::Rotate (UnitVec.hpp:353-358). */
static inline v2 urotate(v2 u, v2 amount) {
    return V(u.x * amount.x - u.y * amount.y, u.y * amount.x + u.x * amount.y);
}
/* Transform / InverseTransform (d2/Math.hpp). */
static inline v2 xform(v2 v, xf_t t) { return vadd(rotate(v, t.q), t.p); }
static inline v2 invxform(v2 v, xf_t t) { return invrotate(vsub(v, t.p), t.q); }
/* MulT(A, B) (d2/Math.hpp): {InverseRotate(B.p - A.p, A.q), B.q.Rotate(A.q.FlipY())}. */
static inline xf_t mult(xf_t A, xf_t B) {
    xf_t r;
    r.p = invrotate(vsub(B.p, A.p), A.q);
    r.q = urotate(B.q, V(A.q.x, -A.q.y));
    return r;
}
/* UnitVec::Get(angle) (UnitVec.cpp:27-30). */
static inline v2 unit_from_angle(real a) { return V(RCOS(a), RSIN(a)); }
/* UnitVec::Get(x, y, fallback) (UnitVec.hpp:175-235). */
static inline v2 unit_vector(v2 v, v2 fallback) {
    const real m2 = v.x * v.x + v.y * v.y;
    if (isnormal(m2)) {
        const real m = RSQRT(m2);
        const real inv = R(1) / m;
        return V(v.x * inv, v.y * inv);
    }
    const real m = RHYPOT(v.x, v.y);
    if (!isnormal(m)) {
        return fallback;
    }
    return V(v.x / m, v.y / m);
}
/* GetTransformation(pos, localCenter) (d2/Math.hpp). */
static inline xf_t get_xf(pos_t pos, v2 lc) {
    xf_t t;
    t.q = unit_from_angle(pos.ang);
    t.p = vsub(pos.lin, rotate(lc, t.q));
    return t;
}
/* AlmostZero / AlmostEqual (Math.hpp:177-194). */
static inline int almost_zero(real v) { return fabs(v) < RMIN_NORMAL; }
static inline int almost_equal(real a, real b) {
    int ulp = 4;
    for (; (a != b) && (ulp > 0); --ulp) {
        a = RNEXT(a, b);
    }
    return a == b;
}
static inline real clampr(real v, real lo, real hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }
static inline real maxr(real a, real b) { return (a < b) ? b : a; }
static inline real minr(real a, real b) { return (b < a) ? b : a; }

/* ------------------------------------------------------------------------- */
/* Growable integer vectors.                                                  */
/* ------------------------------------------------------------------------- */
typedef struct { int64_t* a; int n, cap; } ivec;
static void iv_push(ivec* v, int64_t x) {
    if (v->n == v->cap) {
        v->cap = v->cap ? v->cap * 2 : 8;
        v->a = (int64_t*)realloc(v->a, (size_t)v->cap * sizeof(int64_t));
    }
    v->a[v->n++] = x;
}
static void iv_erase_at(ivec* v, int i) {
    memmove(v->a + i, v->a + i + 1, (size_t)(v->n - i - 1) * sizeof(int64_t));
    --v->n;
}
static void iv_free(ivec* v) { free(v->a); v->a = NULL; v->n = v->cap = 0; }

/* ------------------------------------------------------------------------- */
/* Entities.                                                                  */
/* ------------------------------------------------------------------------- */
typedef struct {
    v2 lp;
    unsigned char tA, iA, tB, iB;
    real ni, ti;
} mpt;
enum { M_UNSET = 0, M_CIRCLES = 1, M_FACEA = 2, M_FACEB = 3 };
typedef struct { int type; v2 ln; v2 lp; int count; mpt p[2]; } manifold;

typedef struct { int count; v2 v[OR_MAXV]; v2 n[OR_MAXV]; real r; } dproxy;

enum { BF_AWAKE = 1u, BF_ALLOW_SLEEP = 2u, BF_FIXED_ROT = 4u, BF_ENABLED = 8u, BF_BULLET = 16u };
typedef struct {
    int type;
    unsigned flags;
    pos_t pos0, pos1;
    v2 lc;
    xf_t xf;
    pos_t vel;
    v2 la;
    real aa, ldamp, adamp, invM, invI, uat;
    real alpha0;  /* Sweep::alpha0: only non-zero inside the TOI phase */
    int islanded; /* m_islanded.bodies entry of the TOI phase */
    ivec shapes, proxies;
    ivec ckeys, cids; /* body contact list: (key, contactID), insertion order */
    ivec jids, jother; /* body joint list: (jointID, other body) */
} body_t;

typedef struct {
    int kind;
    dproxy dp;
    real density, friction, restitution;
    unsigned cat, mask;
    int group, sensor;
    /* a child of a multi-child shape (ChainShapeConf: edges, MultiShapeConf: convex
     * hulls): the index of the shape's first child and the kind (1 chain, 2 multi);
     * owner -1 for a shape of one child */
    int owner, okind;
} shape_t;

typedef struct {
    int bA, bB;
    v2 laA, laB;
    real refAngle, lower, upper, motorSpeed, maxMotorTorque;
    int enableLimit, enableMotor, collideConnected;
    /* solver state */
    v2 rA, rB;
    real mass[3][3];
    real angularMass, motorImpulse;
    real imp[3];
    int limitState;
    /* the other joint types: kind, parameters (OR_JOINT_* layouts) and solver state */
    int type;
    real extra[8];
    v2 u, linErr;
    real jmass, invGamma, bias, length, angErr;
    real lm[2][2];
    /* prismatic (axis perp a1 a2 s1 s2), wheel (ax=axis ay=perp sAx=a1 sBx=a2
     * sAy=s1 sBy=s2), pulley (uA=u uB=u2) and target (C=linErr) state */
    v2 axis, perp, u2;
    real a1, a2, s1, s2, springMass, gamma, springImp, angImp;
    /* gear joint (GearJointConf.hpp): bodies C and D, the kind of each coupled
     * joint (0 revolute, 1 prismatic) with its data, ratio, constant, solver state */
    int bC, bD, gAC, gBD;
    real gRefAC, gRefBD, ratio, constant;
    v2 gLaAC, gLbAC, gAxAC, gLaBD, gLbBD, gAxBD;
    v2 JvAC, JvBD;
    real JwA, JwB, JwC, JwD, gmass, gimp;
} joint_t;
enum { LS_INACTIVE = 0, LS_LOWER = 1, LS_UPPER = 2, LS_EQUAL = 3 };

typedef struct {
    int body, shape, child;
    real aabb[4]; /* minx miny maxx maxy -- the tree (fat) AABB */
} proxy_t;

typedef struct {
    int alive;
    uint64_t key;
    int pA, pB; /* proxy ids (min, max) */
    int bA, sA, cA, bB, sB, cB;
    int touching, sensor, needsUpdate, impenetrable;
    real friction, restitution, tangentSpeed;
    manifold m;
    real toi;                      /* Contact::m_toi, valid when toiValid (e_toiFlag) */
    int toiValid, toiCount, islanded;
} contact_t;

struct or_world {
    body_t* b; int nb, capb;
    shape_t* s; int ns, caps;
    joint_t* j; int nj, capj;
    proxy_t* p; int np, capp;
    contact_t* c; int nc, capc;
    ivec cfree;
    ivec wkeys, wcids;      /* m_contacts: (key, contactID) in insertion order */
    ivec fixturesForProxies; /* pairs (body << 32 | shape) */
    ivec bodiesForSync;
    ivec proxiesForContacts;
    real inv_dt0;
    int sub_stepping;       /* SetSubStepping: the TOI phase stops after one event */
    int step_incomplete;    /* !IsStepComplete: the next Step skips the regular phase */
    ivec events;            /* the last step's contact listener calls: (kind, shape, shape) */
    ivec solve_calls;       /* the last step's preSolve / postSolve calls, 9 words each */
    /* or_set_solve_order: ranks of contacts (by shape pair) and joints for the
     * next step's island solves; empty: the reference's order */
    ivec order_ckeys;       /* (shape min << 32 | shape max), sorted */
    ivec order_crank;       /* rank of order_ckeys[i] */
    ivec order_jrank;       /* rank of joint j, or -1 */
};

/* A BeginContact (1) or EndContact (2) listener call, with the contact's shapes
 * in ascending order (AabbTreeWorld.cpp:2249-2253, 2703-2714). */
static void record_event(or_world* w, int kind, const contact_t* c) {
    iv_push(&w->events, kind);
    iv_push(&w->events, c->sA < c->sB ? c->sA : c->sB);
    iv_push(&w->events, c->sA < c->sB ? c->sB : c->sA);
}

/* A PreSolveContact (kind 3: the manifold before the update, AabbTreeWorld.cpp:
 * 2716-2720) or PostSolveContact (kind 4: the velocity constraint's impulses,
 * GetContactImpulses, ContactImpulsesList.cpp:28-38, and the iteration argument,
 * AabbTreeWorld.cpp:196-205) listener call: kind, shapes in ascending order,
 * point count, iteration, then the two points' normal and tangent impulses as
 * the bits of doubles. */
static void record_solve_call(or_world* w, int kind, const contact_t* c, int count, int iter, const real* ni,
                              const real* ti) {
    iv_push(&w->solve_calls, kind);
    iv_push(&w->solve_calls, c->sA < c->sB ? c->sA : c->sB);
    iv_push(&w->solve_calls, c->sA < c->sB ? c->sB : c->sA);
    iv_push(&w->solve_calls, count);
    iv_push(&w->solve_calls, iter);
    for (int k = 0; k < 2; ++k) {
        const double v[2] = {k < count ? (double)ni[k] : 0.0, k < count ? (double)ti[k] : 0.0};
        for (int q = 0; q < 2; ++q) {
            int64_t bits;
            memcpy(&bits, &v[q], sizeof bits);
            iv_push(&w->solve_calls, bits);
        }
    }
}

#define GROW(ptr, n, cap, T)                                                   \
    do {                                                                       \
        if ((n) == (cap)) {                                                    \
            (cap) = (cap) ? (cap) * 2 : 16;                                    \
            (ptr) = (T*)realloc((ptr), (size_t)(cap) * sizeof(T));             \
        }                                                                      \
    } while (0)

static inline uint64_t make_key(int a, int b) {
    const uint32_t lo = (uint32_t)(a < b ? a : b), hi = (uint32_t)(a < b ? b : a);
    return ((uint64_t)lo << 32) | hi;
}

static inline int is_speedable(const body_t* b) { return b->type != OR_STATIC; }
static inline int is_accelerable(const body_t* b) { return b->type == OR_DYNAMIC; }
/* Body::GetFlags (Body.cpp:32-66): static and kinematic bodies, and bullets. */
static inline int is_impenetrable(const body_t* b) { return b->type != OR_DYNAMIC || (b->flags & BF_BULLET); }

/* Body::SetAwake (Body.cpp:161-169). */
static void body_set_awake(body_t* b) {
    if (is_speedable(b)) { b->flags |= BF_AWAKE; b->uat = R(0); }
}
/* Body::UnsetAwake via Unawaken (Body.hpp:1203-1210, Body.cpp:171-180). */
static int body_unawaken(body_t* b) {
    if ((b->flags & BF_AWAKE) && (b->flags & BF_ALLOW_SLEEP)) {
        b->flags &= ~BF_AWAKE;
        b->uat = R(0);
        b->vel.lin = V(R(0), R(0));
        b->vel.ang = R(0);
        return 1;
    }
    return 0;
}
/* Body::SetPosition1 keeps m_xf = GetTransform1(sweep) (Body.hpp:701-714). */
static void body_set_pos1(body_t* b, pos_t p) { b->pos1 = p; b->xf = get_xf(p, b->lc); }

/* ------------------------------------------------------------------------- */
/* World construction.                                                        */
/* ------------------------------------------------------------------------- */
or_world* or_world_create(void) {
    or_world* w = (or_world*)calloc(1, sizeof(or_world));
    return w;
}

void or_world_destroy(or_world* w) {
    if (!w) return;
    for (int i = 0; i < w->nb; ++i) {
        body_t* b = &w->b[i];
        iv_free(&b->shapes); iv_free(&b->proxies); iv_free(&b->ckeys); iv_free(&b->cids);
        iv_free(&b->jids); iv_free(&b->jother);
    }
    free(w->b); free(w->s); free(w->j); free(w->p); free(w->c);
    iv_free(&w->cfree); iv_free(&w->wkeys); iv_free(&w->wcids);
    iv_free(&w->fixturesForProxies); iv_free(&w->bodiesForSync); iv_free(&w->proxiesForContacts);
    iv_free(&w->events);
    iv_free(&w->solve_calls);
    iv_free(&w->order_ckeys); iv_free(&w->order_crank); iv_free(&w->order_jrank);
    free(w);
}

/* Body(BodyConf) (Body.cpp:88-109) + flags from Body::GetFlags. */
int or_add_body(or_world* w, int type, real px, real py, real angle, real vx, real vy,
                real av, real ax, real ay, real aa, real linDamp, real angDamp, unsigned flags) {
    GROW(w->b, w->nb, w->capb, body_t);
    body_t* b = &w->b[w->nb];
    memset(b, 0, sizeof(*b));
    b->type = type;
    b->flags = 0;
    if (flags & OR_BF_ALLOW_SLEEP) b->flags |= BF_ALLOW_SLEEP;
    if (flags & OR_BF_FIXED_ROTATION) b->flags |= BF_FIXED_ROT;
    if (flags & OR_BF_ENABLED) b->flags |= BF_ENABLED;
    if (flags & OR_BF_BULLET) b->flags |= BF_BULLET;
    if ((flags & OR_BF_AWAKE) && type != OR_STATIC) b->flags |= BF_AWAKE;
    b->lc = V(R(0), R(0));
    b->pos0.lin = V(px, py); b->pos0.ang = angle;
    body_set_pos1(b, b->pos0);
    if (type == OR_STATIC) {
        b->vel.lin = V(R(0), R(0)); b->vel.ang = R(0);
    } else {
        b->vel.lin = V(vx, vy); b->vel.ang = av;
    }
    if (type == OR_DYNAMIC) { b->la = V(ax, ay); b->aa = aa; }
    b->ldamp = linDamp; b->adamp = angDamp;
    /* default inverse mass data (Body.cpp: dynamic bodies start with 1 kg). */
    b->invM = (type == OR_DYNAMIC) ? R(1) : R(0);
    b->invI = R(0);
    b->uat = R(0);
    return w->nb++;
}

/* GetFwdNormalsVector (d2/Math.cpp) -- polygon / edge normals. */
static void make_normals(dproxy* dp) {
    if (dp->count > 1) {
        for (int i = 0; i < dp->count; ++i) {
            const int nx = (i + 1) % dp->count;
            const v2 e = vsub(dp->v[nx], dp->v[i]);
            dp->n[i] = unit_vector(fwdperp(e), V(R(0), R(0)));
        }
    } else if (dp->count == 1) {
        dp->n[0] = V(R(0), R(0));
    }
}

int or_add_shape(or_world* w, int body, int kind, int nverts, const real* xy, real radius,
                 real density, real friction, real restitution, unsigned categoryBits,
                 unsigned maskBits, int groupIndex, int sensor) {
    GROW(w->s, w->ns, w->caps, shape_t);
    shape_t* s = &w->s[w->ns];
    memset(s, 0, sizeof(*s));
    s->kind = kind;
    s->dp.count = nverts > OR_MAXV ? OR_MAXV : nverts;
    for (int i = 0; i < s->dp.count; ++i) s->dp.v[i] = V(xy[2 * i], xy[2 * i + 1]);
    s->dp.r = radius;
#ifdef OR_DOUBLE
    /* Scenes carry float32 values; a 0.01f polygon/edge skin is just under the
     * Real = double world's minimum vertex radius (0.01 m), which CreateShape
     * enforces (AabbTreeWorld.cpp:1239-1249), so it is raised to that minimum. */
    if (kind != OR_SHAPE_DISK && s->dp.r < R(0.01)) s->dp.r = R(0.01);
#endif
    make_normals(&s->dp);
    s->density = density; s->friction = friction; s->restitution = restitution;
    s->cat = categoryBits; s->mask = maskBits; s->group = groupIndex; s->sensor = sensor;
    s->owner = -1; s->okind = 0;
    const int sid = w->ns++;
    /* CreateBody / Attach queue the fixture for proxy creation in the next Step,
     * for an enabled body only (AabbTreeWorld.cpp:1040-1041, :1302). */
    iv_push(&w->b[body].shapes, sid);
    if (w->b[body].flags & BF_ENABLED) iv_push(&w->fixturesForProxies, ((int64_t)body << 32) | (int64_t)sid);
    return sid;
}

/* GetMassData for disk / edge / polygon (MassData.cpp). */
static void shape_mass(const shape_t* s, real* mass, v2* center, real* I) {
    const real Pi = R(3.14159265358979323846264338327950288L);
    const real density = s->density;
    const dproxy* dp = &s->dp;
    if (dp->count == 1) {
        const real r = dp->r;
        const real r2 = r * r;
        const real area = r2 * Pi;
        *mass = density * area;
        const real Iz = area * ((r2 / R(2)) + mag2(dp->v[0]));
        *I = Iz * density;
        *center = dp->v[0];
        return;
    }
    if (dp->count == 2) {
        const real r = dp->r;
        const real r2 = r * r;
        const real circle_area = r2 * Pi;
        const real circle_mass = density * circle_area;
        const v2 v0 = dp->v[0], v1 = dp->v[1];
        const v2 d = vsub(v1, v0);
        const v2 offset = vmul(revperp(unit_vector(d, V(R(0), R(0)))), r);
        const real b = RSQRT(mag2(d));
        const real h = r * R(2);
        const real rect_mass = density * b * h;
        *mass = circle_mass + rect_mass;
        *center = vdiv(vadd(v0, v1), R(2));
        const real halfCircleArea = circle_area / R(2);
        const real halfRSquared = r2 / R(2);
        v2 q[4] = {vadd(v0, offset), vsub(v0, offset), vsub(v1, offset), vadd(v1, offset)};
        /* GetPolarMoment (Math.cpp:243-275) */
        real sum_x = R(0), sum_y = R(0);
        for (int i = 0; i < 4; ++i) {
            const v2 tv = q[i];
            const v2 nv = q[(i + 1) % 4];
            const real fact_b = cross(tv, nv);
            sum_x += ((tv.y * tv.y) + tv.y * nv.y + (nv.y * nv.y)) * fact_b;
            sum_y += ((tv.x * tv.x) + tv.x * nv.x + (nv.x * nv.x)) * fact_b;
        }
        const real RealInverseOfTwelve = R(1) / R(12);
        const real Iz = (sum_x + sum_y) * RealInverseOfTwelve;
        const real I0 = halfCircleArea * (halfRSquared + mag2(v0));
        const real I1 = halfCircleArea * (halfRSquared + mag2(v1));
        *I = (I0 + I1 + Iz) * density;
        return;
    }
    /* Polygon (MassData.cpp, GetMassData(vertexRadius, density, vertices)). */
    const int count = dp->count;
    v2 ctr = V(R(0), R(0));
    real area = R(0);
    real II = R(0);
    v2 s0 = V(R(0), R(0));
    for (int i = 0; i < count; ++i) s0 = vadd(s0, dp->v[i]);
    s0 = vdiv(s0, (real)count); /* Average(vertices) */
    for (int i = 0; i < count; ++i) {
        const v2 e1 = vsub(dp->v[i], s0);
        const v2 e2 = vsub(dp->v[(i + 1) % count], s0);
        const real D = cross(e1, e2);
        const real RealReciprocalOfTwo = R(1) / R(2);
        const real triangleArea = D * RealReciprocalOfTwo;
        area += triangleArea;
        const real RealReciprocalOfThree = R(1) / R(3);
        ctr = vadd(ctr, vmul(vmul(vadd(e1, e2), triangleArea), RealReciprocalOfThree));
        const real intx2 = (e1.x * e1.x) + e2.x * e1.x + (e2.x * e2.x);
        const real inty2 = (e1.y * e1.y) + e2.y * e1.y + (e2.y * e2.y);
        const real RealReciprocalOfTwelve = R(1) / R(3 * 4);
        const real triangleI = D * (intx2 + inty2) * RealReciprocalOfTwelve;
        II += triangleI;
    }
    const real m = density * area;
    ctr = ((area > R(0)) && !almost_zero(area)) ? vdiv(ctr, area) : V(R(0), R(0));
    const v2 massDataCenter = vadd(ctr, s0);
    const real massCenterOffset = mag2(massDataCenter);
    const real centerOffset = mag2(ctr);
    const real inertialLever = massCenterOffset - centerOffset;
    *mass = m;
    *center = massDataCenter;
    *I = ((density * II) + (m * inertialLever));
}

/* ResetMassData -> ComputeMassData (WorldShape.cpp:160-176) -> SetMassData
 * (WorldBody.cpp:365-400). */
void or_set_shape_owner(or_world* w, int shape, int owner, int kind) {
    w->s[shape].owner = owner;
    w->s[shape].okind = kind;
}

/* GetMassData of a multi-child shape from its children first..first+n-1:
 * ChainShapeConf::GetMassData (ChainShapeConf.cpp:113-147: the segments' masses,
 * inertias and mass-weighted centres summed, the centre divided by the summed
 * segment areas) or GetMassData(MultiShapeConf) (MultiShapeConf.cpp:35-57: the
 * hulls' masses, inertias and mass-weighted centres summed, the centre divided
 * by the mass). */
static void group_mass(const or_world* w, int first, int n, int kind, real* mass, v2* center, real* I) {
    const real Pi = R(3.14159265358979323846264338327950288L);
    real m = R(0), Iz = R(0), area = R(0);
    v2 c = V(R(0), R(0));
    for (int k = 0; k < n; ++k) {
        const shape_t* s = &w->s[first + k];
        real mk, ik;
        v2 ck;
        shape_mass(s, &mk, &ck, &ik);
        m += mk;
        Iz += ik;
        if (kind == 1) {
            c = vadd(c, vmul(ck, mk));
            const v2 d = vsub(s->dp.v[1], s->dp.v[0]);
            const real bl = RSQRT(mag2(d));
            const real h = s->dp.r * R(2);
            area += bl * h + (s->dp.r * s->dp.r) * Pi;
        } else {
            c = vadd(c, vmul(ck, mk));
        }
    }
    if (kind == 1) c = vdiv(c, area);
    else c = (m > R(0)) ? vdiv(c, m) : V(R(0), R(0));
    *mass = m; *center = c; *I = Iz;
}

void or_reset_mass(or_world* w, int body) {
    body_t* b = &w->b[body];
    real mass = R(0), I = R(0);
    v2 wc = V(R(0), R(0));
    for (int k = 0; k < b->shapes.n; ++k) {
        const int sid = (int)b->shapes.a[k];
        const shape_t* s = &w->s[sid];
        if (s->owner >= 0 && s->owner != sid) continue;  /* a later child: counted with the first */
        if (s->density > R(0)) {
            real m, i;
            v2 c;
            if (s->owner == sid) {
                int n = 1;
                while (k + n < b->shapes.n && w->s[b->shapes.a[k + n]].owner == sid) ++n;
                group_mass(w, sid, n, s->okind, &m, &c, &i);
            } else {
                shape_mass(s, &m, &c, &i);
            }
            mass += m;
            wc = vadd(wc, vmul(c, m));
            I += i;
        }
    }
    const v2 center = (mass > R(0)) ? vdiv(wc, mass) : V(R(0), R(0));
    if (!is_accelerable(b)) {
        b->invM = R(0); b->invI = R(0);
        if (!is_speedable(b)) {
            /* SetSweep(Sweep{Position{location, angle}}) with zero local center. */
            const v2 loc = b->xf.p;
            const real ang = b->pos1.ang;
            b->lc = V(R(0), R(0));
            b->pos0.lin = loc; b->pos0.ang = ang;
            body_set_pos1(b, b->pos0);
        }
        return;
    }
    const real m = (mass > R(0)) ? mass : R(1);
    const real invMass = R(1) / m;
    real invRotI = R(0);
    if ((I > R(0)) && !(b->flags & BF_FIXED_ROT)) {
        const real lengthSquared = mag2(center);
        const real Ic = I - (m * lengthSquared);
        invRotI = R(1) / Ic;
    }
    b->invM = invMass; b->invI = invRotI;
    const v2 oldCenter = b->pos1.lin;
    const pos_t np = {xform(center, b->xf), b->pos1.ang};
    b->lc = center;
    b->pos0 = np;
    body_set_pos1(b, np);
    const v2 newCenter = b->pos1.lin;
    const v2 dc = vsub(newCenter, oldCenter);
    b->vel.lin = vadd(b->vel.lin, vmul(revperp(dc), b->vel.ang));
}

static v2 unit_len(v2 v, real* len);

/* CreateJoint of the other joint types: anchors, collideConnected and the
 * type's parameters (the OR_JOINT_* layouts in playrho_oracle.h). */
int or_add_joint(or_world* w, int type, int bodyA, int bodyB, real lax, real lay, real lbx, real lby,
                 int collideConnected, const real* extra8) {
    const int jid = or_add_revolute(w, bodyA, bodyB, lax, lay, lbx, lby, R(0), 0, R(0), R(0), 0, R(0), R(0),
                                    collideConnected);
    joint_t* j = &w->j[jid];
    j->type = type;
    for (int k = 0; k < 8; ++k) j->extra[k] = extra8 ? extra8[k] : R(0);
    if (type == OR_JOINT_PRISMATIC || type == OR_JOINT_WHEEL) {
        /* localXAxisA is the UnitVec::Get of the given axis (UnitVec.hpp:175-235) */
        real len;
        const v2 ax = unit_len(V(j->extra[0], j->extra[1]), &len);
        j->extra[0] = ax.x; j->extra[1] = ax.y;
    }
    return jid;
}

/* enableLimit / enableMotor of a prismatic (both) or wheel (enableMotor) joint. */
/* GetGearJointConf(world, id1, id2, ratio) (GearJointConf.cpp:66-160): body A/B
 * are the second bodies of the two joints, C/D their first bodies; the constant
 * is the joints' coordinates now, so that the gear holds the current pose. */
int or_add_gear(or_world* w, int joint1, int joint2, real ratio) {
    const joint_t j1 = w->j[joint1], j2 = w->j[joint2];
    const int A = j1.bB, B = j2.bB, C = j1.bA, D = j2.bA;
    const int jid = or_add_revolute(w, A, B, R(0), R(0), R(0), R(0), R(0), 0, R(0), R(0), 0, R(0), R(0), 0);
    joint_t* j = &w->j[jid];
    j->type = OR_JOINT_GEAR;
    j->bC = C; j->bD = D;
    real scalar1 = R(0), scalar2 = R(0);
    if (j1.type == OR_JOINT_PRISMATIC) {
        j->gAC = 1;
        j->gLaAC = j1.laA; j->gLbAC = j1.laB; j->gAxAC = V(j1.extra[0], j1.extra[1]);
        const xf_t xfA = w->b[A].xf, xfC = w->b[C].xf;
        const v2 pC = j1.laA;
        const v2 pA = invrotate(vadd(rotate(j1.laB, xfA.q), vsub(xfA.p, xfC.p)), xfC.q);
        scalar1 = dot(vsub(pA, pC), j->gAxAC);
    } else {
        j->gAC = 0;
        j->gRefAC = j1.refAngle;
        scalar1 = (w->b[A].pos1.ang - w->b[C].pos1.ang) - j1.refAngle;
    }
    if (j2.type == OR_JOINT_PRISMATIC) {
        j->gBD = 1;
        j->gLaBD = j2.laA; j->gLbBD = j2.laB; j->gAxBD = V(j2.extra[0], j2.extra[1]);
        const xf_t xfB = w->b[B].xf, xfD = w->b[D].xf;
        const v2 pD = j2.laA;
        const v2 pB = invrotate(vadd(rotate(j2.laB, xfB.q), vsub(xfB.p, xfD.p)), xfD.q);
        scalar2 = dot(vsub(pB, pD), j->gAxBD);
    } else {
        j->gBD = 0;
        j->gRefBD = j2.refAngle;
        scalar2 = (w->b[B].pos1.ang - w->b[D].pos1.ang) - j2.refAngle;
    }
    j->ratio = ratio;
    j->constant = scalar1 + ratio * scalar2;
    return jid;
}

void or_joint_enable(or_world* w, int jid, int enableLimit, int enableMotor) {
    w->j[jid].enableLimit = enableLimit;
    w->j[jid].enableMotor = enableMotor;
}

int or_add_revolute(or_world* w, int bodyA, int bodyB, real lax, real lay, real lbx, real lby,
                    real refAngle, int enableLimit, real lower, real upper, int enableMotor,
                    real motorSpeed, real maxMotorTorque, int collideConnected) {
    GROW(w->j, w->nj, w->capj, joint_t);
    joint_t* j = &w->j[w->nj];
    memset(j, 0, sizeof(*j));
    j->bA = bodyA; j->bB = bodyB;
    j->laA = V(lax, lay); j->laB = V(lbx, lby);
    j->refAngle = refAngle; j->enableLimit = enableLimit; j->lower = lower; j->upper = upper;
    j->enableMotor = enableMotor; j->motorSpeed = motorSpeed; j->maxMotorTorque = maxMotorTorque;
    j->collideConnected = collideConnected;
    const int jid = w->nj++;
    /* CreateJoint adds (jointID, other) to both bodies' joint lists (AabbTreeWorld.cpp:1132-1157). */
    iv_push(&w->b[bodyA].jids, jid); iv_push(&w->b[bodyA].jother, bodyB);
    if (bodyB != bodyA) { iv_push(&w->b[bodyB].jids, jid); iv_push(&w->b[bodyB].jother, bodyA); }
    return jid;
}

/* ------------------------------------------------------------------------- */
/* AABBs (AABB.cpp:51-62, detail/AABB.hpp, Interval.hpp).                     */
/* ------------------------------------------------------------------------- */
static inline void aabb_empty(real* a) { a[0] = RINF; a[1] = RINF; a[2] = -RINF; a[3] = -RINF; }
static inline void aabb_include(real* a, v2 p) {
    /* Interval::Include: {min(v, min), max(v, max)} */
    a[0] = (a[0] < p.x) ? a[0] : p.x;  /* std::min(v, GetMin()) returns v unless GetMin() < v */
    a[2] = (p.x < a[2]) ? a[2] : p.x;  /* std::max(v, GetMax()) returns v unless v < GetMax() */
    a[1] = (a[1] < p.y) ? a[1] : p.y;
    a[3] = (p.y < a[3]) ? a[3] : p.y;
}
/* Fatten = ExpandEqually (Interval.hpp:210-222). */
static inline void aabb_fatten(real* a, real amount) {
    a[0] = a[0] - amount; a[2] = a[2] + amount;
    a[1] = a[1] - amount; a[3] = a[3] + amount;
}
/* GetDisplacedAABB -> Interval::Expand (Interval.hpp:186-200). */
static inline void aabb_displace(real* a, v2 d) {
    if (d.x < R(0)) a[0] += d.x; else a[2] += d.x;
    if (d.y < R(0)) a[1] += d.y; else a[3] += d.y;
}
/* ComputeAABB(proxy, xf0, xf1) (AABB.cpp:51-62). */
static void compute_aabb2(const dproxy* dp, xf_t x0, xf_t x1, real* out) {
    aabb_empty(out);
    for (int i = 0; i < dp->count; ++i) {
        aabb_include(out, xform(dp->v[i], x0));
        aabb_include(out, xform(dp->v[i], x1));
    }
    aabb_fatten(out, dp->r);
}
/* TestOverlap -> IsIntersecting (Interval.hpp:292-298). */
static inline int aabb_overlap(const real* a, const real* b) {
    {
        const real maxOfMins = (a[0] < b[0]) ? b[0] : a[0];
        const real minOfMaxs = (b[2] < a[2]) ? b[2] : a[2];
        if (!(minOfMaxs >= maxOfMins)) return 0;
    }
    {
        const real maxOfMins = (a[1] < b[1]) ? b[1] : a[1];
        const real minOfMaxs = (b[3] < a[3]) ? b[3] : a[3];
        if (!(minOfMaxs >= maxOfMins)) return 0;
    }
    return 1;
}
/* Contains -> IsEntirelyEnclosing (Interval.hpp:324-327). */
static inline int aabb_contains(const real* a, const real* b) {
    return a[0] <= b[0] && a[2] >= b[2] && a[1] <= b[1] && a[3] >= b[3];
}

/* ------------------------------------------------------------------------- */
/* Narrowphase: CollideShapes (Manifold.cpp:393-438) and helpers.             */
/* ------------------------------------------------------------------------- */
typedef struct { v2 v; unsigned char tA, iA, tB, iB; } clipv;
enum { CF_VERTEX = 0, CF_FACE = 1 };
#define INVALID_V 255

static manifold man_empty(void) { manifold m; memset(&m, 0, sizeof(m)); m.type = M_UNSET; return m; }
static void set_cf(mpt* p, int tA, int iA, int tB, int iB) {
    p->tA = (unsigned char)tA; p->iA = (unsigned char)iA; p->tB = (unsigned char)tB; p->iB = (unsigned char)iB;
}
/* Manifold::GetForCircles (Manifold.hpp:168-171). */
static manifold man_circles(v2 vA, int iA, v2 vB, int iB) {
    manifold m = man_empty();
    m.type = M_CIRCLES; m.ln = V(R(0), R(0)); m.lp = vA; m.count = 1;
    m.p[0].lp = vB; set_cf(&m.p[0], CF_VERTEX, iA, CF_VERTEX, iB);
    return m;
}
static manifold man_face(int type, v2 ln, v2 lp) {
    manifold m = man_empty();
    m.type = type; m.ln = ln; m.lp = lp; m.count = 0;
    return m;
}
static void man_add(manifold* m, v2 lp, int tA, int iA, int tB, int iB) {
    mpt* p = &m->p[m->count++];
    p->lp = lp; set_cf(p, tA, iA, tB, iB); p->ni = R(0); p->ti = R(0);
}

/* ClipSegmentToLine (Manifold.cpp:61-102). */
static int clip_segment(const clipv* vin, int nin, v2 normal, real offset, int indexA, clipv* vout) {
    int n = 0;
    if (nin == 2) {
        const real d0 = dot(normal, vin[0].v) - offset;
        const real d1 = dot(normal, vin[1].v) - offset;
        if (d0 <= R(0) || almost_zero(d0)) vout[n++] = vin[0];
        if (d1 <= R(0) || almost_zero(d1)) vout[n++] = vin[1];
        if (n < 2 && (signbit(d0) != signbit(d1))) {
            const real interp = d0 / (d0 - d1);
            const v2 vertex = vadd(vin[0].v, vmul(vsub(vin[1].v, vin[0].v), interp));
            clipv cv;
            cv.v = vertex; cv.tA = CF_VERTEX; cv.iA = (unsigned char)indexA; cv.tB = CF_FACE; cv.iB = vin[0].iB;
            vout[n++] = cv;
        }
    }
    return n;
}

/* GetMinSeparationInfo (ShapeSeparation.cpp:36-58). */
static real min_sep_info(v2 origin, v2 dir, const v2* verts, int n, int* first, int* second) {
    real minSep = RINF;
    *first = INVALID_V; *second = INVALID_V;
    for (int i = 0; i < n; ++i) {
        const real s = dot(dir, vsub(verts[i], origin));
        if (minSep > s) { minSep = s; *first = i; *second = INVALID_V; }
        else if (minSep == s) { *second = i; }
    }
    return minSep;
}
typedef struct { real distance; int firstShape; int second0, second1; } sepinfo;
/* GetMaxSeparation4x4 (ShapeSeparation.cpp:62-101). */
static sepinfo max_sep_4x4(const dproxy* p1, xf_t xf1, const dproxy* p2, xf_t xf2) {
    sepinfo r; r.distance = -RINF; r.firstShape = INVALID_V; r.second0 = INVALID_V; r.second1 = INVALID_V;
    const xf_t xf = mult(xf1, xf2);
    v2 verts[4];
    for (int i = 0; i < 4; ++i) verts[i] = xform(p2->v[i], xf);
    for (int i = 0; i < 4; ++i) {
        int f, s;
        const real d = min_sep_info(p1->v[i], p1->n[i], verts, 4, &f, &s);
        if (r.distance < d) { r.distance = d; r.second0 = f; r.second1 = s; r.firstShape = i; }
    }
    return r;
}
/* GetMaxSeparation (ShapeSeparation.cpp:103-124). */
static sepinfo max_sep(const dproxy* p1, xf_t xf1, const dproxy* p2, xf_t xf2) {
    sepinfo r; r.distance = -RINF; r.firstShape = INVALID_V; r.second0 = INVALID_V; r.second1 = INVALID_V;
    const xf_t xf = mult(xf2, xf1);
    for (int i = 0; i < p1->count; ++i) {
        const v2 origin = xform(p1->v[i], xf);
        const v2 normal = rotate(p1->n[i], xf.q);
        int f, s;
        const real d = min_sep_info(origin, normal, p2->v, p2->count, &f, &s);
        if (r.distance < d) { r.distance = d; r.second0 = f; r.second1 = s; r.firstShape = i; }
    }
    return r;
}

/* GetMostAntiParallelEdge (Manifold.cpp:124-141). */
static void most_anti_parallel_edge(v2 n0, xf_t xf0, const dproxy* s1, xf_t xf1, int first, int second,
                                    int* e0, int* e1) {
    if (second == INVALID_V) {
        const v2 normal = invrotate(rotate(n0, xf0.q), xf1.q);
        const int count = s1->count;
        const int prev = (first == 0) ? count - 1 : first - 1;
        const real prevDot = dot(normal, s1->n[prev]);
        const real currDot = dot(normal, s1->n[first]);
        if (prevDot < currDot) { *e0 = prev; *e1 = first; }
        else { *e0 = first; *e1 = (first + 1) % count; }
        return;
    }
    if ((second > first) && ((first + 1) == second)) { *e0 = first; *e1 = second; }
    else { *e0 = second; *e1 = first; }
}

/* GetManifold for two polygons (Manifold.cpp:162-291). */
static manifold get_manifold_poly(int flipped, const dproxy* s0, xf_t xf0, int idx0,
                                  const dproxy* s1, xf_t xf1, int sec0, int sec1,
                                  real maxCirclesRatio) {
    const real r0 = s0->r, r1 = s1->r;
    const real totalRadius = r0 + r1;
    const int idx0Next = (idx0 + 1) % s0->count;
    const v2 s0_rel_v0 = s0->v[idx0];
    const v2 s0_rel_v1 = s0->v[idx0Next];
    const v2 s0_abs_v0 = xform(s0_rel_v0, xf0);
    const v2 s0_abs_v1 = xform(s0_rel_v1, xf0);
    const real s0_len_edge0 = mag2(vsub(s0_rel_v1, s0_rel_v0));
    const v2 s0_rel_n0 = s0->n[idx0];
    const v2 s0_rel_e0_dir = revperp(s0_rel_n0);
    int e1f, e1s;
    most_anti_parallel_edge(s0_rel_n0, xf0, s1, xf1, sec0, sec1, &e1f, &e1s);
    const v2 s1_rel_v0 = s1->v[e1f];
    const v2 s1_abs_v0 = xform(s1_rel_v0, xf1);
    const v2 s1_rel_v1 = s1->v[e1s];
    const v2 s1_abs_v1 = xform(s1_rel_v1, xf1);
    {
        const v2 s0_abs_e0_dir = rotate(s0_rel_e0_dir, xf0.q);
        /* GetClipPoints (Manifold.cpp:143-158) */
        clipv ie[2];
        ie[0].v = s1_abs_v0; ie[0].tA = CF_FACE; ie[0].iA = (unsigned char)idx0; ie[0].tB = CF_VERTEX; ie[0].iB = (unsigned char)e1f;
        ie[1].v = s1_abs_v1; ie[1].tA = CF_FACE; ie[1].iA = (unsigned char)idx0; ie[1].tB = CF_VERTEX; ie[1].iB = (unsigned char)e1s;
        const real dp_v0_e0 = -dot(s0_abs_e0_dir, s0_abs_v0);
        const real dp_v1_e0 = +dot(s0_abs_e0_dir, s0_abs_v1);
        clipv pts[2], cps[2];
        const int np = clip_segment(ie, 2, vneg(s0_abs_e0_dir), dp_v0_e0, idx0, pts);
        const int nc = clip_segment(pts, np, s0_abs_e0_dir, dp_v1_e0, idx0Next, cps);
        if (nc == 2) {
            const v2 abs_normal = fwdperp(s0_abs_e0_dir);
            const v2 rel_midpoint = vdiv(vadd(s0_rel_v0, s0_rel_v1), R(2));
            const real abs_offset = dot(abs_normal, s0_abs_v0);
            const v2 normal = fwdperp(s0_rel_e0_dir);
            manifold m = man_face(flipped ? M_FACEB : M_FACEA, normal, rel_midpoint);
            for (int k = 0; k < 2; ++k) {
                if ((dot(abs_normal, cps[k].v) - abs_offset) <= totalRadius) {
                    const v2 lp = invxform(cps[k].v, xf1);
                    if (!flipped) man_add(&m, lp, cps[k].tA, cps[k].iA, cps[k].tB, cps[k].iB);
                    else man_add(&m, lp, cps[k].tB, cps[k].iB, cps[k].tA, cps[k].iA);
                }
            }
            if (m.count > 0) return m;
        }
    }
    const real totalRadiusSquared = totalRadius * totalRadius;
    const real mcr = maxCirclesRatio * r0;
    const int mustUseFace = s0_len_edge0 > (mcr * mcr);
    const v2 fn = fwdperp(s0_rel_e0_dir);
    /* four vertex-vertex tests in the reference's order */
    const v2 a_rel[4] = {s0_rel_v0, s0_rel_v1, s0_rel_v0, s0_rel_v1};
    const v2 a_abs[4] = {s0_abs_v0, s0_abs_v1, s0_abs_v0, s0_abs_v1};
    const int a_idx[4] = {idx0, idx0Next, idx0, idx0Next};
    const v2 b_rel[4] = {s1_rel_v0, s1_rel_v1, s1_rel_v1, s1_rel_v0};
    const v2 b_abs[4] = {s1_abs_v0, s1_abs_v1, s1_abs_v1, s1_abs_v0};
    const int b_idx[4] = {e1f, e1s, e1s, e1f};
    for (int k = 0; k < 4; ++k) {
        if (mag2(vsub(a_abs[k], b_abs[k])) <= totalRadiusSquared) {
            if (mustUseFace) {
                manifold m = man_face(flipped ? M_FACEB : M_FACEA, fn, a_rel[k]);
                if (!flipped) man_add(&m, b_rel[k], CF_FACE, a_idx[k], CF_VERTEX, b_idx[k]);
                else man_add(&m, b_rel[k], CF_VERTEX, b_idx[k], CF_FACE, a_idx[k]);
                return m;
            }
            return !flipped ? man_circles(a_rel[k], a_idx[k], b_rel[k], b_idx[k])
                            : man_circles(b_rel[k], b_idx[k], a_rel[k], a_idx[k]);
        }
    }
    return man_empty();
}

/* GetManifold for polygon vs circle (Manifold.cpp:293-372). */
static manifold get_manifold_circle(int flipped, real totalRadius, const dproxy* shape, xf_t sxf,
                                    v2 point, xf_t xfm) {
    const int vc = shape->count;
    const v2 cLocal = invxform(xform(point, xfm), sxf);
    int indexOfMax = 0;
    real maxSeparation = -RMAXV;
    for (int i = 0; i < vc; ++i) {
        const real s = dot(shape->n[i], vsub(cLocal, shape->v[i]));
        if (s > totalRadius) return man_empty();
        if (maxSeparation < s) { maxSeparation = s; indexOfMax = i; }
    }
    const int indexOfMax2 = (indexOfMax + 1) % vc;
    const v2 v1 = shape->v[indexOfMax];
    const v2 v2_ = shape->v[indexOfMax2];
    if (maxSeparation < R(0)) {
        const v2 faceCenter = vdiv(vadd(v1, v2_), R(2));
        manifold m = man_face(flipped ? M_FACEB : M_FACEA, shape->n[indexOfMax], faceCenter);
        if (!flipped) man_add(&m, point, CF_FACE, indexOfMax, CF_VERTEX, 0);
        else man_add(&m, point, CF_VERTEX, 0, CF_FACE, indexOfMax);
        return m;
    }
    const v2 cLocalV1 = vsub(cLocal, v1);
    if (dot(cLocalV1, vsub(v2_, v1)) <= R(0)) {
        if (mag2(cLocalV1) > totalRadius * totalRadius) return man_empty();
        return !flipped ? man_circles(v1, indexOfMax, point, 0) : man_circles(point, 0, v1, indexOfMax);
    }
    const v2 cLocalV2 = vsub(cLocal, v2_);
    if (dot(cLocalV2, vsub(v1, v2_)) <= R(0)) {
        if (mag2(cLocalV2) > totalRadius * totalRadius) return man_empty();
        return !flipped ? man_circles(v2_, indexOfMax2, point, 0) : man_circles(point, 0, v2_, indexOfMax2);
    }
    const v2 faceCenter = vdiv(vadd(v1, v2_), R(2));
    if (dot(vsub(cLocal, faceCenter), shape->n[indexOfMax]) > totalRadius) return man_empty();
    manifold m = man_face(flipped ? M_FACEB : M_FACEA, shape->n[indexOfMax], faceCenter);
    if (!flipped) man_add(&m, point, CF_FACE, indexOfMax, CF_VERTEX, 0);
    else man_add(&m, point, CF_VERTEX, 0, CF_FACE, indexOfMax);
    return m;
}

/* CollideShapes (Manifold.cpp:393-438). */
static manifold collide_shapes(const dproxy* A, xf_t xfA, const dproxy* B, xf_t xfB,
                               real linearSlop, real maxCirclesRatio) {
    const real totalRadius = A->r + B->r;
    if (A->count == 1 && B->count == 1) {
        /* GetManifold(locationA, xfA, locationB, xfB, totalRadius) (Manifold.cpp:374-386) */
        const v2 pA = xform(A->v[0], xfA);
        const v2 pB = xform(B->v[0], xfB);
        const real lenSq = mag2(vsub(pB, pA));
        const real totSq = totalRadius * totalRadius;
        if (lenSq > totSq) return man_empty();
        return man_circles(A->v[0], 0, B->v[0], 0);
    }
    if (A->count == 1) return get_manifold_circle(1, totalRadius, B, xfB, A->v[0], xfA);
    if (B->count == 1) return get_manifold_circle(0, totalRadius, A, xfA, B->v[0], xfB);
    const int do4x4 = (A->count == 4) && (B->count == 4);
    const sepinfo sa = do4x4 ? max_sep_4x4(A, xfA, B, xfB) : max_sep(A, xfA, B, xfB);
    if (sa.distance > totalRadius) return man_empty();
    const sepinfo sb = do4x4 ? max_sep_4x4(B, xfB, A, xfA) : max_sep(B, xfB, A, xfA);
    if (sb.distance > totalRadius) return man_empty();
    const real k_tol = linearSlop / R(10);
    return (sb.distance > (sa.distance + k_tol))
               ? get_manifold_poly(1, B, xfB, sb.firstShape, A, xfA, sb.second0, sb.second1, maxCirclesRatio)
               : get_manifold_poly(0, A, xfA, sa.firstShape, B, xfB, sa.second0, sa.second1, maxCirclesRatio);
}

void or_collide(int kindA, int nA, const real* xyA, real rA, const real* xfA4, int kindB, int nB,
                const real* xyB, real rB, const real* xfB4, real linearSlop, real maxCirclesRatio,
                int* type_count2, int* feat8, real* fout8) {
    (void)kindA; (void)kindB;
    dproxy a, b;
    memset(&a, 0, sizeof(a)); memset(&b, 0, sizeof(b));
    a.count = nA; b.count = nB; a.r = rA; b.r = rB;
    for (int i = 0; i < nA; ++i) a.v[i] = V(xyA[2 * i], xyA[2 * i + 1]);
    for (int i = 0; i < nB; ++i) b.v[i] = V(xyB[2 * i], xyB[2 * i + 1]);
    make_normals(&a); make_normals(&b);
    xf_t xa, xb;
    xa.p = V(xfA4[0], xfA4[1]); xa.q = V(xfA4[2], xfA4[3]);
    xb.p = V(xfB4[0], xfB4[1]); xb.q = V(xfB4[2], xfB4[3]);
    const manifold m = collide_shapes(&a, xa, &b, xb, linearSlop, maxCirclesRatio);
    type_count2[0] = m.type; type_count2[1] = m.count;
    for (int k = 0; k < 2; ++k) {
        feat8[4 * k + 0] = m.p[k].tA; feat8[4 * k + 1] = m.p[k].iA;
        feat8[4 * k + 2] = m.p[k].tB; feat8[4 * k + 3] = m.p[k].iB;
    }
    fout8[0] = m.ln.x; fout8[1] = m.ln.y; fout8[2] = m.lp.x; fout8[3] = m.lp.y;
    fout8[4] = m.p[0].lp.x; fout8[5] = m.p[0].lp.y; fout8[6] = m.p[1].lp.x; fout8[7] = m.p[1].lp.y;
}

/* ------------------------------------------------------------------------- */
/* Contact maintenance.                                                       */
/* ------------------------------------------------------------------------- */
static int kv_find(const ivec* ids, int64_t id) {
    for (int i = 0; i < ids->n; ++i) if (ids->a[i] == id) return i;
    return -1;
}

static int sensor_touching(const dproxy* A, xf_t xfA, const dproxy* B, xf_t xfB, int maxIters);

/* AabbTreeWorld::Update(ContactID) (AabbTreeWorld.cpp:2587-2721). */
static void contact_update(or_world* w, int cid, const or_stepconf* conf) {
    contact_t* c = &w->c[cid];
    const manifold old = c->m;
    const body_t* bA = &w->b[c->bA];
    const body_t* bB = &w->b[c->bB];
    const shape_t* sA = &w->s[c->sA];
    const shape_t* sB = &w->s[c->sB];
    int newTouching;
    if (c->sensor) {
        /* TestOverlap (:2622-2625); sensors make no manifold (:2634) */
        newTouching = sensor_touching(&sA->dp, bA->xf, &sB->dp, bB->xf, conf->maxDistanceIters);
        c->m = man_empty();
    } else {
        manifold nm = collide_shapes(&sA->dp, bA->xf, &sB->dp, bB->xf, conf->linearSlop, conf->maxCirclesRatio);
        const int oldn = old.count, newn = nm.count;
        newTouching = newn > 0;
        int found[2] = {0, newn < 2};
        for (int i = 0; i < newn; ++i) {
            for (int j = 0; j < oldn; ++j) {
                if (nm.p[i].tA == old.p[j].tA && nm.p[i].iA == old.p[j].iA &&
                    nm.p[i].tB == old.p[j].tB && nm.p[i].iB == old.p[j].iB) {
                    found[i] = 1;
                    nm.p[i].ni = old.p[j].ni; nm.p[i].ti = old.p[j].ti;
                    break;
                }
            }
        }
        for (int i = 0; i < newn; ++i) {
            if (!found[i]) {
                real least = RINF;
                for (int j = 0; j < oldn; ++j) {
                    const real sq = mag2(vsub(old.p[j].lp, nm.p[i].lp));
                    if (least > sq) { least = sq; nm.p[i].ni = old.p[j].ni; nm.p[i].ti = old.p[j].ti; }
                }
            }
        }
        c->m = nm;
    }
    c->needsUpdate = 0;
    if (!c->touching && newTouching) record_event(w, 1, c);
    else if (c->touching && !newTouching) record_event(w, 2, c);
    c->touching = newTouching;
    if (!c->sensor && newTouching) {
        const real ni[2] = {old.p[0].ni, old.p[1].ni}, ti[2] = {old.p[0].ti, old.p[1].ti};
        record_solve_call(w, 3, c, old.count, 0, ni, ti);
    }
}

/* InternalDestroy(ContactID) (AabbTreeWorld.cpp:2245-2279). */
static void contact_destroy(or_world* w, int cid) {
    contact_t* c = &w->c[cid];
    body_t* bA = &w->b[c->bA];
    body_t* bB = &w->b[c->bB];
    int k = kv_find(&bA->cids, cid);
    if (k >= 0) { iv_erase_at(&bA->cids, k); iv_erase_at(&bA->ckeys, k); }
    k = kv_find(&bB->cids, cid);
    if (k >= 0) { iv_erase_at(&bB->cids, k); iv_erase_at(&bB->ckeys, k); }
    if (c->touching) record_event(w, 2, c);
    if (c->m.count > 0 && !c->sensor) { body_set_awake(bA); body_set_awake(bB); }
    c->alive = 0;
    iv_push(&w->cfree, cid);
}

/* DestroyContacts (AabbTreeWorld.cpp:2290-2331), overlap pass only. */
static int destroy_contacts(or_world* w) {
    int n = 0, out = 0;
    for (int i = 0; i < w->wcids.n; ++i) {
        const int cid = (int)w->wcids.a[i];
        const contact_t* c = &w->c[cid];
        if (!aabb_overlap(w->p[c->pA].aabb, w->p[c->pB].aabb)) {
            contact_destroy(w, cid);
            ++n;
        } else {
            w->wcids.a[out] = w->wcids.a[i];
            w->wkeys.a[out] = w->wkeys.a[i];
            ++out;
        }
    }
    w->wcids.n = out; w->wkeys.n = out;
    return n;
}

/* UpdateContacts (AabbTreeWorld.cpp:2333-2415). */
static int update_contacts(or_world* w, const or_stepconf* conf) {
    int n = 0;
    for (int i = 0; i < w->wcids.n; ++i) {
        const int cid = (int)w->wcids.a[i];
        if (w->c[cid].needsUpdate) { contact_update(w, cid, conf); ++n; }
    }
    return n;
}

/* Static median-split BVH over the fat AABBs: the same query result set as
 * DynamicTree::Query (DynamicTree.cpp:673-700); FindContacts sorts and
 * de-duplicates the results, so the traversal order does not matter. */
typedef struct { real box[4]; int left, right, leaf; } bnode;
typedef struct { bnode* n; int nn; int* idx; } bvh_t;
static or_world* g_sort_world;
static int g_sort_axis;
static int cmp_proxy_center(const void* a, const void* b) {
    const proxy_t* pa = &g_sort_world->p[*(const int*)a];
    const proxy_t* pb = &g_sort_world->p[*(const int*)b];
    const real ca = pa->aabb[g_sort_axis] + pa->aabb[g_sort_axis + 2];
    const real cb = pb->aabb[g_sort_axis] + pb->aabb[g_sort_axis + 2];
    return (ca < cb) ? -1 : (ca > cb) ? 1 : (*(const int*)a - *(const int*)b);
}
static int bvh_build(or_world* w, bvh_t* t, int* idx, int n) {
    const int me = t->nn++;
    bnode* nd = &t->n[me];
    aabb_empty(nd->box);
    for (int i = 0; i < n; ++i) {
        const real* a = w->p[idx[i]].aabb;
        nd->box[0] = minr(nd->box[0], a[0]); nd->box[1] = minr(nd->box[1], a[1]);
        nd->box[2] = maxr(nd->box[2], a[2]); nd->box[3] = maxr(nd->box[3], a[3]);
    }
    if (n == 1) { nd->leaf = idx[0]; nd->left = nd->right = -1; return me; }
    nd->leaf = -1;
    g_sort_world = w;
    g_sort_axis = ((nd->box[2] - nd->box[0]) >= (nd->box[3] - nd->box[1])) ? 0 : 1;
    qsort(idx, (size_t)n, sizeof(int), cmp_proxy_center);
    const int h = n / 2;
    const int l = bvh_build(w, t, idx, h);
    const int r = bvh_build(w, t, idx + h, n - h);
    t->n[me].left = l; t->n[me].right = r;
    return me;
}

typedef struct { uint64_t key; int pmin, pmax; } pkey;
static int cmp_pkey(const void* a, const void* b) {
    const uint64_t ka = ((const pkey*)a)->key, kb = ((const pkey*)b)->key;
    return (ka < kb) ? -1 : (ka > kb) ? 1 : 0;
}

/* FindContacts (AabbTreeWorld.cpp:709-751) + AddContacts (:2423-2547). */
static int find_and_add_contacts(or_world* w, const or_stepconf* conf) {
    if (w->proxiesForContacts.n == 0 || w->np == 0) { iv_free(&w->proxiesForContacts); return 0; }
    bvh_t t;
    t.n = (bnode*)malloc(sizeof(bnode) * (size_t)(2 * w->np));
    t.nn = 0;
    int* idx = (int*)malloc(sizeof(int) * (size_t)w->np);
    int live = 0;
    for (int i = 0; i < w->np; ++i) if (w->p[i].body >= 0) idx[live++] = i;
    const int root = live ? bvh_build(w, &t, idx, live) : -1;
    pkey* keys = NULL; int nk = 0, capk = 0;
    int* stack = (int*)malloc(sizeof(int) * (size_t)(2 * w->np + 8));
    for (int q = 0; q < w->proxiesForContacts.n; ++q) {
        const int pid = (int)w->proxiesForContacts.a[q];
        const proxy_t* pp = &w->p[pid];
        if (pp->body < 0 || root < 0) continue;
        int sp = 0;
        stack[sp++] = root;
        while (sp) {
            const bnode* nd = &t.n[stack[--sp]];
            if (!aabb_overlap(nd->box, pp->aabb)) continue;
            if (nd->leaf >= 0) {
                const int other = nd->leaf;
                if (other != pid && w->p[other].body != pp->body) {
                    GROW(keys, nk, capk, pkey);
                    keys[nk].key = make_key(pid, other);
                    keys[nk].pmin = pid < other ? pid : other;
                    keys[nk].pmax = pid < other ? other : pid;
                    ++nk;
                }
            } else {
                stack[sp++] = nd->left;
                stack[sp++] = nd->right;
            }
        }
    }
    free(stack); free(idx); free(t.n);
    iv_free(&w->proxiesForContacts);
    qsort(keys, (size_t)nk, sizeof(pkey), cmp_pkey);
    int added = 0;
    for (int i = 0; i < nk; ++i) {
        if (i > 0 && keys[i].key == keys[i - 1].key) continue;
        const proxy_t* pa = &w->p[keys[i].pmin];
        const proxy_t* pb = &w->p[keys[i].pmax];
        body_t* bA = &w->b[pa->body];
        body_t* bB = &w->b[pb->body];
        const shape_t* sA = &w->s[pa->shape];
        const shape_t* sB = &w->s[pb->shape];
        if (!(is_accelerable(bA) || is_accelerable(bB))) continue;
        /* ShouldCollide(jointBuffer, bodyJoints, A, B) (AabbTreeWorld.cpp:479-490) */
        int jointBlocks = 0;
        for (int k = 0; k < bA->jids.n; ++k) {
            if (bA->jother.a[k] == pb->body && !w->j[bA->jids.a[k]].collideConnected) { jointBlocks = 1; break; }
        }
        if (jointBlocks) continue;
        /* ShouldCollide(Filter, Filter) (Filter.hpp:81-88) */
        if ((sA->group == sB->group) && (sA->group != 0)) {
            if (!(sA->group > 0)) continue;
        } else if (!(((sA->mask & sB->cat) != 0) && ((sB->mask & sA->cat) != 0))) {
            continue;
        }
        /* already exists? search the body with fewer contacts */
        const ivec* kl = (bA->ckeys.n < bB->ckeys.n) ? &bA->ckeys : &bB->ckeys;
        int exists = 0;
        for (int k = 0; k < kl->n; ++k) if ((uint64_t)kl->a[k] == keys[i].key) { exists = 1; break; }
        if (exists) continue;
        int cid;
        if (w->cfree.n) { cid = (int)w->cfree.a[--w->cfree.n]; }
        else { GROW(w->c, w->nc, w->capc, contact_t); cid = w->nc++; }
        contact_t* c = &w->c[cid];
        memset(c, 0, sizeof(*c));
        c->alive = 1;
        c->key = keys[i].key;
        c->pA = keys[i].pmin; c->pB = keys[i].pmax;
        c->bA = pa->body; c->sA = pa->shape; c->cA = pa->child;
        c->bB = pb->body; c->sB = pb->shape; c->cB = pb->child;
        c->impenetrable = is_impenetrable(bA) || is_impenetrable(bB);
        c->sensor = sA->sensor || sB->sensor;
        c->friction = RSQRT(sA->friction * sB->friction); /* MixFriction (Contact.hpp:57-60) */
        c->restitution = (sA->restitution > sB->restitution) ? sA->restitution : sB->restitution;
        c->tangentSpeed = R(0);
        c->m = man_empty();
        c->needsUpdate = 1;
        iv_push(&w->wkeys, (int64_t)c->key); iv_push(&w->wcids, cid);
        iv_push(&bA->ckeys, (int64_t)c->key); iv_push(&bA->cids, cid);
        iv_push(&bB->ckeys, (int64_t)c->key); iv_push(&bB->cids, cid);
        if (!c->sensor) {
            if (is_speedable(bA)) bA->flags |= BF_AWAKE;
            if (is_speedable(bB)) bB->flags |= BF_AWAKE;
        }
        contact_update(w, cid, conf);
        ++added;
    }
    free(keys);
    return added;
}

/* GetTransform0(sweep) (Sweep.hpp).  The body's transformation is always
 * GetTransform1(sweep) (Body::SetSweep / SetPosition1), so when pos0 equals pos1
 * the stored transformation is that same value; taking it keeps a transformation
 * set by or_set_body_xf (identical transforms injected on both sides of a
 * parity check). */
static xf_t xf0_of(const body_t* b) {
    if (b->pos0.lin.x == b->pos1.lin.x && b->pos0.lin.y == b->pos1.lin.y && b->pos0.ang == b->pos1.ang) return b->xf;
    return get_xf(b->pos0, b->lc);
}

/* CreateProxies (AabbTreeWorld.cpp:557-579). */
static void create_proxies(or_world* w, int body, int shape, const or_stepconf* conf) {
    body_t* b = &w->b[body];
    const xf_t x0 = xf0_of(b);
    const xf_t x1 = b->xf;
    const v2 disp = vmul(vsub(x1.p, x0.p), conf->displaceMultiplier);
    GROW(w->p, w->np, w->capp, proxy_t);
    proxy_t* p = &w->p[w->np];
    p->body = body; p->shape = shape; p->child = 0;
    compute_aabb2(&w->s[shape].dp, x0, x1, p->aabb);
    aabb_fatten(p->aabb, conf->aabbExtension);
    aabb_displace(p->aabb, disp);
    iv_push(&b->proxies, w->np);
    iv_push(&w->proxiesForContacts, w->np);
    w->np++;
}

/* AabbTreeWorld::Synchronize (AabbTreeWorld.cpp:2564-2585). */
static int synchronize(or_world* w, int body, const or_stepconf* conf) {
    body_t* b = &w->b[body];
    const xf_t x0 = xf0_of(b);
    const xf_t x1 = b->xf;
    const v2 disp = vmul(vsub(x1.p, x0.p), conf->displaceMultiplier);
    int n = 0;
    for (int k = 0; k < b->proxies.n; ++k) {
        proxy_t* p = &w->p[b->proxies.a[k]];
        real aabb[4];
        compute_aabb2(&w->s[p->shape].dp, x0, x1, aabb);
        if (!aabb_contains(p->aabb, aabb)) {
            aabb_fatten(aabb, conf->aabbExtension);
            aabb_displace(aabb, disp);
            memcpy(p->aabb, aabb, sizeof(aabb));
            iv_push(&w->proxiesForContacts, b->proxies.a[k]);
            ++n;
        }
    }
    return n;
}

/* ------------------------------------------------------------------------- */
/* Solver (ContactSolver.cpp, VelocityConstraint.cpp, RevoluteJointConf.cpp). */
/* ------------------------------------------------------------------------- */
typedef struct { pos_t pos; pos_t vel; v2 lc; real invM, invI; } bc_t;
typedef struct {
    v2 rA, rB;
    real ni, ti, nm, tm, vb;
} vcp_t;
typedef struct {
    int bA, bB;
    v2 n;
    real friction, restitution, tangentSpeed;
    int count;
    vcp_t p[2];
    real K[3];  /* k00 k11 k01 */
    real NM[3]; /* normal mass 2x2: m00 m11 m01 */
} vc_t;

/* GetContactRelVelocity (d2/Math.cpp). */
static inline v2 rel_vel(pos_t va, v2 rA, pos_t vb, v2 rB) {
    const v2 velBrot = vmul(revperp(rB), vb.ang);
    const v2 velArot = vmul(revperp(rA), va.ang);
    return vsub(vadd(vb.lin, velBrot), vadd(va.lin, velArot));
}

/* GetWorldManifold (WorldManifold.cpp:111-132). */
typedef struct { v2 n; int count; v2 pt[2]; real ni[2], ti[2], sep[2]; } wman_t;
static wman_t world_manifold(const manifold* m, xf_t xfA, real rA, xf_t xfB, real rB) {
    wman_t wm; memset(&wm, 0, sizeof(wm));
    if (m->type == M_CIRCLES) {
        const v2 pA = xform(m->lp, xfA);
        const v2 pB = xform(m->p[0].lp, xfB);
        const v2 n = unit_vector(vsub(pB, pA), V(R(1), R(0)));
        const v2 cA = vadd(pA, vmul(n, rA));
        const v2 cB = vsub(pB, vmul(n, rB));
        wm.n = n; wm.count = 1;
        wm.pt[0] = vdiv(vadd(cA, cB), R(2));
        wm.ni[0] = m->p[0].ni; wm.ti[0] = m->p[0].ti;
        wm.sep[0] = dot(vsub(cB, cA), n);
    } else if (m->type == M_FACEA) {
        const v2 n = urotate(m->ln, xfA.q);
        const v2 planePoint = xform(m->lp, xfA);
        wm.n = n; wm.count = m->count;
        for (int i = 0; i < m->count; ++i) {
            const v2 clip = xform(m->p[i].lp, xfB);
            const v2 cA = vadd(clip, vmul(n, (rA - dot(vsub(clip, planePoint), n))));
            const v2 cB = vsub(clip, vmul(n, rB));
            wm.pt[i] = vdiv(vadd(cA, cB), R(2));
            wm.ni[i] = m->p[i].ni; wm.ti[i] = m->p[i].ti;
            wm.sep[i] = dot(vsub(cB, cA), n);
        }
    } else if (m->type == M_FACEB) {
        const v2 n = urotate(m->ln, xfB.q);
        const v2 planePoint = xform(m->lp, xfB);
        wm.n = vneg(n); wm.count = m->count;
        for (int i = 0; i < m->count; ++i) {
            const v2 clip = xform(m->p[i].lp, xfA);
            const v2 cB = vadd(clip, vmul(n, (rB - dot(vsub(clip, planePoint), n))));
            const v2 cA = vsub(clip, vmul(n, rA));
            wm.pt[i] = vdiv(vadd(cA, cB), R(2));
            wm.ni[i] = m->p[i].ni; wm.ti[i] = m->p[i].ti;
            wm.sep[i] = dot(vsub(cA, cB), n);
        }
    }
    return wm;
}

/* VelocityConstraint ctor + GetPoint + ComputeK (VelocityConstraint.cpp:38-185). */
static void make_vc(vc_t* vc, const contact_t* c, const wman_t* wm, const bc_t* bcs, const or_stepconf* conf) {
    memset(vc, 0, sizeof(*vc));
    vc->bA = c->bA; vc->bB = c->bB;
    vc->n = wm->n;
    vc->friction = c->friction; vc->restitution = c->restitution; vc->tangentSpeed = c->tangentSpeed;
    const bc_t* A = &bcs[c->bA];
    const bc_t* B = &bcs[c->bB];
    const real invMass = A->invM + B->invM;
    const v2 tangent = fwdperp(vc->n);
    for (int j = 0; j < wm->count; ++j) {
        vcp_t* p = &vc->p[vc->count];
        const v2 relA = vsub(wm->pt[j], A->pos.lin);
        const v2 relB = vsub(wm->pt[j], B->pos.lin);
        p->ni = wm->ni[j] * conf->dtRatio;
        p->ti = wm->ti[j] * conf->dtRatio;
        {
            const v2 dv = rel_vel(A->vel, relA, B->vel, relB);
            const real vn = dot(dv, vc->n);
            p->vb = (vn < -conf->velocityThreshold) ? -vc->restitution * vn : R(0);
        }
        p->rA = relA; p->rB = relB;
        {
            const real crA = cross(relA, vc->n), crB = cross(relB, vc->n);
            const real iA = A->invI * (crA * crA);
            const real iB = B->invI * (crB * crB);
            const real value = invMass + iA + iB;
            p->nm = (value != R(0)) ? R(1) / value : R(0);
        }
        {
            const real crA = cross(relA, tangent), crB = cross(relB, tangent);
            const real iA = A->invI * (crA * crA);
            const real iB = B->invI * (crB * crB);
            const real value = invMass + iA + iB;
            p->tm = (value != R(0)) ? R(1) / value : R(0);
        }
        vc->count++;
    }
    if (conf->doBlocksolve && vc->count == 2) {
        const real rnA0 = cross(vc->p[0].rA, vc->n), rnB0 = cross(vc->p[0].rB, vc->n);
        const real rnA1 = cross(vc->p[1].rA, vc->n), rnB1 = cross(vc->p[1].rB, vc->n);
        const real iMA0 = A->invI * (rnA0 * rnA0);
        const real iMA1 = A->invI * (rnA1 * rnA1);
        const real iMB0 = B->invI * (rnB0 * rnB0);
        const real iMB1 = B->invI * (rnB1 * rnB1);
        const real iMA = (A->invI * rnA0 * rnA1);
        const real iMB = (B->invI * rnB0 * rnB1);
        const real k00 = invMass + iMA0 + iMB0;
        const real k11 = invMass + iMA1 + iMB1;
        const real k01 = invMass + iMA + iMB;
        const real k00_sq = k00 * k00;
        const real k00_k11 = k00 * k11;
        const real k01_sq = k01 * k01;
        const real k_diff = k00_k11 - k01_sq;
        const real maxCondNum = R(1000.0f);
        if (k00_sq < maxCondNum * k_diff) {
            vc->K[0] = k00; vc->K[1] = k11; vc->K[2] = k01;
            /* Invert(Matrix22) (Math.hpp:430-442): cp = Cross(row0, row1) */
            const real cp = cross(V(k00, k01), V(k01, k11));
            if (!almost_zero(cp)) {
                const real inv = R(1) / cp;
                vc->NM[0] = k11 * inv;      /* [0][0] */
                vc->NM[2] = -k01 * inv;     /* [0][1] */
                vc->NM[1] = k00 * inv;      /* [1][1] */
            }
        } else {
            memset(&vc->p[1], 0, sizeof(vc->p[1]));
            vc->count = 1;
        }
    }
}

static inline void apply_imp(bc_t* b, v2 P, real L, int sign) {
    if (sign < 0) {
        b->vel.lin = vsub(b->vel.lin, vmul(P, b->invM));
        b->vel.ang = b->vel.ang - b->invI * L;
    } else {
        b->vel.lin = vadd(b->vel.lin, vmul(P, b->invM));
        b->vel.ang = b->vel.ang + b->invI * L;
    }
}

/* CalcWarmStartVelocityDeltas + WarmStartVelocities (AabbTreeWorld.cpp:227-274). */
static void warm_start(const vc_t* vc, bc_t* bcs) {
    pos_t dA = {{R(0), R(0)}, R(0)}, dB = {{R(0), R(0)}, R(0)};
    const v2 n = vc->n, t = fwdperp(vc->n);
    bc_t* A = &bcs[vc->bA];
    bc_t* B = &bcs[vc->bB];
    for (int j = 0; j < vc->count; ++j) {
        const vcp_t* p = &vc->p[j];
        const v2 P = vadd(vmul(n, p->ni), vmul(t, p->ti));
        const real LA = cross(p->rA, P);
        const real LB = cross(p->rB, P);
        dA.lin = vsub(dA.lin, vmul(P, A->invM)); dA.ang = dA.ang - A->invI * LA;
        dB.lin = vadd(dB.lin, vmul(P, B->invM)); dB.ang = dB.ang + B->invI * LB;
    }
    A->vel.lin = vadd(A->vel.lin, dA.lin); A->vel.ang = A->vel.ang + dA.ang;
    B->vel.lin = vadd(B->vel.lin, dB.lin); B->vel.ang = B->vel.ang + dB.ang;
}

/* BlockSolveUpdate (ContactSolver.cpp:100-111). */
static real block_update(vc_t* vc, bc_t* bcs, real x0, real x1) {
    bc_t* A = &bcs[vc->bA];
    bc_t* B = &bcs[vc->bB];
    const real d0 = x0 - vc->p[0].ni, d1 = x1 - vc->p[1].ni;
    /* GetVelocityDelta (ContactSolver.cpp:69-98) */
    const v2 P0 = vmul(vc->n, d0);
    const v2 P1 = vmul(vc->n, d1);
    const v2 P = vadd(P0, P1);
    const real LA = cross(vc->p[0].rA, P0) + cross(vc->p[1].rA, P1);
    const real LB = cross(vc->p[0].rB, P0) + cross(vc->p[1].rB, P1);
    const v2 dvAl = vneg(vmul(P, A->invM)); const real dvAa = -(A->invI * LA);
    const v2 dvBl = vmul(P, B->invM); const real dvBa = +(B->invI * LB);
    A->vel.lin = vadd(A->vel.lin, dvAl); A->vel.ang = A->vel.ang + dvAa;
    B->vel.lin = vadd(B->vel.lin, dvBl); B->vel.ang = B->vel.ang + dvBa;
    vc->p[0].ni = x0; vc->p[1].ni = x1;
    return maxr(fabs(x0), fabs(x1));
}

/* BlockSolveNormalConstraint (ContactSolver.cpp:245-335). */
static real block_solve(vc_t* vc, bc_t* bcs) {
    const v2 n = vc->n;
    const bc_t* A = &bcs[vc->bA];
    const bc_t* B = &bcs[vc->bB];
    const v2 dv0 = rel_vel(A->vel, vc->p[0].rA, B->vel, vc->p[0].rB);
    const v2 dv1 = rel_vel(A->vel, vc->p[1].rA, B->vel, vc->p[1].rB);
    const real vn0 = dot(dv0, n), vn1 = dot(dv1, n);
    const real b0 = vn0 - vc->p[0].vb, b1 = vn1 - vc->p[1].vb;
    /* b - Transform(impulses, K): K * x with rows (k00 k01), (k01 k11) */
    const real a0 = vc->p[0].ni, a1 = vc->p[1].ni;
    real Kx0 = R(0); Kx0 += vc->K[0] * a0; Kx0 += vc->K[2] * a1;
    real Kx1 = R(0); Kx1 += vc->K[2] * a0; Kx1 += vc->K[1] * a1;
    const real bp0 = b0 - Kx0, bp1 = b1 - Kx1;
    /* Case 1: x = -NM * b' */
    {
        real m0 = R(0); m0 += vc->NM[0] * bp0; m0 += vc->NM[2] * bp1;
        real m1 = R(0); m1 += vc->NM[2] * bp0; m1 += vc->NM[1] * bp1;
        const real x0 = -m0, x1 = -m1;
        if (x0 >= R(0) && x1 >= R(0)) return block_update(vc, bcs, x0, x1);
    }
    /* Case 2 */
    {
        const real x0 = -vc->p[0].nm * bp0;
        const real vn2 = vc->K[2] * x0 + bp1;
        if (x0 >= R(0) && vn2 >= R(0)) return block_update(vc, bcs, x0, R(0));
    }
    /* Case 3 */
    {
        const real x1 = -vc->p[1].nm * bp1;
        const real vn1b = vc->K[2] * x1 + bp0;
        if (x1 >= R(0) && vn1b >= R(0)) return block_update(vc, bcs, R(0), x1);
    }
    /* Case 4 */
    if (bp0 >= R(0) && bp1 >= R(0)) return block_update(vc, bcs, R(0), R(0));
    return R(0);
}

/* SeqSolveNormalConstraint (ContactSolver.cpp:337-393) with dir = normal, and
 * SolveTangentConstraint (:395-454) with dir = tangent. */
static real seq_solve(vc_t* vc, bc_t* bcs, int tangentPass) {
    real maxInc = R(0);
    const v2 dir = tangentPass ? fwdperp(vc->n) : vc->n;
    bc_t* A = &bcs[vc->bA];
    bc_t* B = &bcs[vc->bB];
    pos_t vA = A->vel, vB = B->vel;
    for (int k = (vc->count == 2) ? 1 : 0; k >= 0; --k) {
        vcp_t* p = &vc->p[k];
        const v2 cv = rel_vel(vA, p->rA, vB, p->rB);
        real newImp, oldImp;
        if (tangentPass) {
            const real dvel = vc->tangentSpeed - dot(cv, dir);
            const real lambda = p->tm * dvel;
            const real maxImp = vc->friction * p->ni;
            oldImp = p->ti;
            newImp = clampr(oldImp + lambda, -maxImp, maxImp);
        } else {
            const real dvel = dot(cv, dir);
            const real lambda = p->nm * (p->vb - dvel);
            oldImp = p->ni;
            newImp = maxr(oldImp + lambda, R(0));
        }
        const real inc = newImp - oldImp;
        const v2 P = vmul(dir, inc);
        const real LA = cross(p->rA, P);
        const real LB = cross(p->rB, P);
        vA.lin = vsub(vA.lin, vmul(P, A->invM)); vA.ang = vA.ang - A->invI * LA;
        vB.lin = vadd(vB.lin, vmul(P, B->invM)); vB.ang = vB.ang + B->invI * LB;
        maxInc = maxr(maxInc, fabs(inc));
        if (tangentPass) p->ti = oldImp + inc; else p->ni = oldImp + inc;
    }
    A->vel = vA;
    B->vel = vB;
    return maxInc;
}

/* GaussSeidel::SolveVelocityConstraint (ContactSolver.cpp:481-492). */
static real solve_vc(vc_t* vc, bc_t* bcs) {
    real m = R(0);
    m = maxr(m, seq_solve(vc, bcs, 1));
    const int useSeq = (vc->count == 1) || (vc->K[0] == R(0) && vc->K[1] == R(0) && vc->K[2] == R(0));
    m = maxr(m, useSeq ? seq_solve(vc, bcs, 0) : block_solve(vc, bcs));
    return m;
}

/* GetPSM (PositionSolverManifold.cpp:103-121). */
typedef struct { v2 n, pt; real sep; } psm_t;
static psm_t get_psm(const manifold* m, int idx, xf_t xfA, xf_t xfB) {
    psm_t r;
    if (m->type == M_CIRCLES) {
        const v2 pA = xform(m->lp, xfA);
        const v2 pB = xform(m->p[idx].lp, xfB);
        const v2 delta = vsub(pB, pA);
        r.n = unit_vector(delta, V(R(0), R(0)));
        r.pt = vdiv(vadd(pA, pB), R(2));
        r.sep = dot(delta, r.n);
    } else if (m->type == M_FACEA) {
        const v2 planePoint = xform(m->lp, xfA);
        r.n = urotate(m->ln, xfA.q);
        r.pt = xform(m->p[idx].lp, xfB);
        r.sep = dot(vsub(r.pt, planePoint), r.n);
    } else {
        const v2 planePoint = xform(m->lp, xfB);
        const v2 n = urotate(m->ln, xfB.q);
        r.pt = xform(m->p[idx].lp, xfA);
        r.sep = dot(vsub(r.pt, planePoint), n);
        r.n = vneg(n);
    }
    return r;
}

typedef struct { const manifold* m; int bA, bB; real totalRadius; } pc_t;
typedef struct { pos_t a, b; real sep; } psol_t;

/* solver_fn lambda of GaussSeidel::SolvePositionConstraint (ContactSolver.cpp:521-551). */
static psol_t pos_solver_fn(psm_t psm, v2 pA, v2 pB, real invMassA, real invIA, real invMassB, real invIB,
                            real totalRadius, const or_stepconf* conf) {
    const real invMassTotal = invMassA + invMassB;
    const real separation = psm.sep - totalRadius;
    const v2 rA = vsub(psm.pt, pA);
    const v2 rB = vsub(psm.pt, pB);
    const real cA = cross(rA, psm.n), cB = cross(rB, psm.n);
    const real K = invMassTotal + invIA * (cA * cA) + invIB * (cB * cB);
    const real C = -clampr(conf->regResolutionRate * (separation + conf->linearSlop), -conf->maxLinearCorrection, R(0));
    const v2 P = vdiv(vmul(psm.n, C), K);
    const real LA = cross(rA, P);
    const real LB = cross(rB, P);
    psol_t s;
    s.a.lin = vneg(vmul(P, invMassA)); s.a.ang = -(invIA * LA);
    s.b.lin = vmul(P, invMassB); s.b.ang = +(invIB * LB);
    s.sep = separation;
    return s;
}

static inline pos_t padd(pos_t a, pos_t b) { pos_t r; r.lin = vadd(a.lin, b.lin); r.ang = a.ang + b.ang; return r; }

/* GaussSeidel::SolvePositionConstraint (ContactSolver.cpp:494-643). */
static real solve_pc(const pc_t* pc, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[pc->bA];
    bc_t* B = &bcs[pc->bB];
    const real iMA = A->invM, iIA = A->invI, iMB = B->invM, iIB = B->invI;
    pos_t posA = A->pos, posB = B->pos;
    real minSep = RINF;
    const int count = pc->m->count;
    if (count == 1) {
        const psm_t psm0 = get_psm(pc->m, 0, get_xf(posA, A->lc), get_xf(posB, B->lc));
        const psol_t s = pos_solver_fn(psm0, posA.lin, posB.lin, iMA, iIA, iMB, iIB, pc->totalRadius, conf);
        posA = padd(posA, s.a); posB = padd(posB, s.b);
        minSep = R(0) + s.sep;
    } else if (count == 2) {
        const xf_t xfA = get_xf(posA, A->lc), xfB = get_xf(posB, B->lc);
        const psm_t psm0 = get_psm(pc->m, 0, xfA, xfB);
        const psm_t psm1 = get_psm(pc->m, 1, xfA, xfB);
        if (almost_equal(psm0.sep, psm1.sep)) {
            const psol_t s0 = pos_solver_fn(psm0, posA.lin, posB.lin, iMA, iIA, iMB, iIB, pc->totalRadius, conf);
            const psol_t s1 = pos_solver_fn(psm1, posA.lin, posB.lin, iMA, iIA, iMB, iIB, pc->totalRadius, conf);
            posA = padd(padd(posA, s0.a), s1.a);
            posB = padd(padd(posB, s0.b), s1.b);
            minSep = s0.sep;
        } else if (psm0.sep < psm1.sep) {
            const psol_t s0 = pos_solver_fn(psm0, posA.lin, posB.lin, iMA, iIA, iMB, iIB, pc->totalRadius, conf);
            posA = padd(posA, s0.a); posB = padd(posB, s0.b);
            const psm_t p1 = get_psm(pc->m, 1, get_xf(posA, A->lc), get_xf(posB, B->lc));
            const psol_t s1 = pos_solver_fn(p1, posA.lin, posB.lin, iMA, iIA, iMB, iIB, pc->totalRadius, conf);
            posA = padd(posA, s1.a); posB = padd(posB, s1.b);
            minSep = s0.sep;
        } else if (psm1.sep < psm0.sep) {
            const psol_t s1 = pos_solver_fn(psm1, posA.lin, posB.lin, iMA, iIA, iMB, iIB, pc->totalRadius, conf);
            posA = padd(posA, s1.a); posB = padd(posB, s1.b);
            const psm_t p0 = get_psm(pc->m, 0, get_xf(posA, A->lc), get_xf(posB, B->lc));
            const psol_t s0 = pos_solver_fn(p0, posA.lin, posB.lin, iMA, iIA, iMB, iIB, pc->totalRadius, conf);
            posA = padd(posA, s0.a); posB = padd(posB, s0.b);
            minSep = s1.sep;
        }
    }
    A->pos = posA;
    B->pos = posB;
    return minSep;
}

/* Revolute joint InitVelocity (RevoluteJointConf.cpp:127-225), no motor/limit
 * beyond what the reference supports. */
static void rj_init_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    const real iMA = A->invM, iIA = A->invI, iMB = B->invM, iIB = B->invI;
    const real aA = A->pos.ang, aB = B->pos.ang;
    pos_t vA = A->vel, vB = B->vel;
    const v2 qA = unit_from_angle(aA), qB = unit_from_angle(aB);
    j->rA = rotate(vsub(j->laA, A->lc), qA);
    j->rB = rotate(vsub(j->laB, B->lc), qB);
    const real totInvI = iIA + iIB;
    const int fixedRotation = (totInvI == R(0));
    /* GetMat33 (RevoluteJointConf.cpp:35-63) */
    {
        const v2 rA = j->rA, rB = j->rB;
        const real exx = iMA + ((rA.y * rA.y) * iIA) + iMB + ((rB.y * rB.y) * iIB);
        const real eyx = (-rA.y * rA.x * iIA) + (-rB.y * rB.x * iIB);
        const real ezx = (-rA.y * iIA) + (-rB.y * iIB);
        const real eyy = iMA + ((rA.x * rA.x) * iIA) + iMB + ((rB.x * rB.x) * iIB);
        const real ezy = (rA.x * iIA) + (rB.x * iIB);
        j->mass[0][0] = exx; j->mass[1][0] = eyx; j->mass[2][0] = ezx;
        j->mass[0][1] = eyx; j->mass[1][1] = eyy; j->mass[2][1] = ezy;
        j->mass[0][2] = ezx; j->mass[1][2] = ezy; j->mass[2][2] = totInvI;
    }
    j->angularMass = (totInvI > R(0)) ? R(1) / totInvI : R(0);
    if (!j->enableMotor || fixedRotation) j->motorImpulse = R(0);
    if (j->enableLimit && !fixedRotation) {
        const real jointAngle = aB - aA - j->refAngle;
        if (fabs(j->upper - j->lower) < (conf->angularSlop * R(2))) j->limitState = LS_EQUAL;
        else if (jointAngle <= j->lower) { if (j->limitState != LS_LOWER) { j->limitState = LS_LOWER; j->imp[2] = R(0); } }
        else if (jointAngle >= j->upper) { if (j->limitState != LS_UPPER) { j->limitState = LS_UPPER; j->imp[2] = R(0); } }
        else { j->limitState = LS_INACTIVE; j->imp[2] = R(0); }
    } else {
        j->limitState = LS_INACTIVE;
    }
    if (conf->doWarmStart) {
        j->imp[0] *= conf->dtRatio; j->imp[1] *= conf->dtRatio; j->imp[2] *= conf->dtRatio;
        j->motorImpulse *= conf->dtRatio;
        const v2 P = V(j->imp[0], j->imp[1]);
        const real L = j->motorImpulse + j->imp[2];
        const real LA = cross(j->rA, P) + L;
        const real LB = cross(j->rB, P) + L;
        vA.lin = vsub(vA.lin, vmul(P, iMA)); vA.ang = vA.ang - iIA * LA;
        vB.lin = vadd(vB.lin, vmul(P, iMB)); vB.ang = vB.ang + iIB * LB;
    } else {
        j->imp[0] = j->imp[1] = j->imp[2] = R(0);
        j->motorImpulse = R(0);
    }
    A->vel = vA;
    B->vel = vB;
}

/* Solve22 (Math.hpp:462-474) on the upper 2x2 of a Mat33 (column-major here). */
static v2 solve22(real m[3][3], v2 b) {
    const real xx = m[0][0], xy = m[1][0], yx = m[0][1], yy = m[1][1];
    const real cp = xx * yy - xy * yx;
    const real det = (cp != R(0)) ? (R(1) / cp) : cp;
    return V(det * (yy * b.x - xy * b.y), det * (xx * b.y - yx * b.x));
}

/* Revolute SolveVelocity (RevoluteJointConf.cpp:228-330), point constraint and
 * motor; limits are restated for the inactive state only. */
static int rj_solve_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    const pos_t oA = A->vel, oB = B->vel;
    pos_t vA = oA, vB = oB;
    const real iMA = A->invM, iIA = A->invI, iMB = B->invM, iIB = B->invI;
    const int fixedRotation = (iIA + iIB == R(0));
    if (j->enableMotor && (j->limitState != LS_EQUAL) && !fixedRotation) {
        const real impulse = -j->angularMass * (vB.ang - vA.ang - j->motorSpeed);
        const real oldImpulse = j->motorImpulse;
        const real maxImpulse = conf->deltaTime * j->maxMotorTorque;
        j->motorImpulse = clampr(j->motorImpulse + impulse, -maxImpulse, maxImpulse);
        const real inc = j->motorImpulse - oldImpulse;
        vA.ang -= iIA * inc;
        vB.ang += iIB * inc;
    }
    const v2 vb = vadd(vB.lin, vmul(revperp(j->rB), vB.ang));
    const v2 va = vadd(vA.lin, vmul(revperp(j->rA), vA.ang));
    const v2 vDelta = vsub(vb, va);
    {
        const v2 impulse = solve22(j->mass, vneg(vDelta));
        j->imp[0] += impulse.x;
        j->imp[1] += impulse.y;
        const v2 P = impulse;
        const real LA = cross(j->rA, P);
        const real LB = cross(j->rB, P);
        vA.lin = vsub(vA.lin, vmul(P, iMA)); vA.ang = vA.ang - iIA * LA;
        vB.lin = vadd(vB.lin, vmul(P, iMB)); vB.ang = vB.ang + iIB * LB;
    }
    if (vA.lin.x != oA.lin.x || vA.lin.y != oA.lin.y || vA.ang != oA.ang ||
        vB.lin.x != oB.lin.x || vB.lin.y != oB.lin.y || vB.ang != oB.ang) {
        A->vel = vA;
        B->vel = vB;
        return 0;
    }
    return 1;
}

/* Revolute SolvePosition (RevoluteJointConf.cpp:333-431), point constraint. */
static int rj_solve_position(const joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t posA = A->pos, posB = B->pos;
    const real iIA = A->invI, iIB = B->invI;
    const real angularError = R(0);
    real positionError;
    {
        const v2 qA = unit_from_angle(posA.ang), qB = unit_from_angle(posB.ang);
        const v2 rA = rotate(vsub(j->laA, A->lc), qA);
        const v2 rB = rotate(vsub(j->laB, B->lc), qB);
        const v2 C = vsub(vadd(posB.lin, rB), vadd(posA.lin, rA));
        positionError = mag2(C);
        const real iMA = A->invM, iMB = B->invM;
        const real exx = iMA + (iIA * (rA.y * rA.y)) + iMB + (iIB * (rB.y * rB.y));
        const real exy = (-iIA * rA.x * rA.y) + (-iIB * rB.x * rB.y);
        const real eyy = iMA + (iIA * (rA.x * rA.x)) + iMB + (iIB * (rB.x * rB.x));
        /* Solve(K, C) (Math.hpp:410-426): cp = Cross(col0, col1) */
        const real cp = cross(V(exx, exy), V(exy, eyy));
        v2 x = V(R(0), R(0));
        if (!almost_zero(cp)) {
            const real inv = R(1) / cp;
            x = V((eyy * C.x - exy * C.y) * inv, (exx * C.y - exy * C.x) * inv);
        }
        const v2 P = vneg(x);
        posA.lin = vsub(posA.lin, vmul(P, iMA)); posA.ang = posA.ang - iIA * cross(rA, P);
        posB.lin = vadd(posB.lin, vmul(P, iMB)); posB.ang = posB.ang + iIB * cross(rB, P);
    }
    A->pos = posA;
    B->pos = posB;
    return (positionError <= conf->linearSlop * conf->linearSlop) && (angularError <= conf->angularSlop);
}

/* ------------------------------------------------------------------------- */
/* Islands and the regular phase (AabbTreeWorld.cpp:1358-1683).               */
/* ------------------------------------------------------------------------- */
typedef struct {
    ivec bodies, contacts, joints;
} island_t;

/* ------------------------------------------------------------------------- */
/* Other joint types (DistanceJointConf.cpp, RopeJointConf.cpp,               */
/* WeldJointConf.cpp, FrictionJointConf.cpp, MotorJointConf.cpp).             */
/* ------------------------------------------------------------------------- */
/* Position / Velocity operator!= (Position.hpp, Velocity.hpp). */
static inline int pos_ne(pos_t a, pos_t b) {
    return !(a.lin.x == b.lin.x && a.lin.y == b.lin.y && a.ang == b.ang);
}
/* UnitVec::Get(x, y) (UnitVec.hpp:175-235): the direction and the magnitude. */
static v2 unit_len(v2 v, real* len) {
    const real m2 = v.x * v.x + v.y * v.y;
    if (isnormal(m2)) {
        const real m = RSQRT(m2);
        const real inv = R(1) / m;
        *len = m;
        return V(v.x * inv, v.y * inv);
    }
    const real m = RHYPOT(v.x, v.y);
    if (!isnormal(m)) { *len = R(0); return V(R(0), R(0)); }
    *len = m;
    return V(v.x / m, v.y / m);
}
/* Velocity / Position -= {invMass * P, invRotI * L} and += (Velocity.hpp, Position.hpp). */
static inline void sub_imp(pos_t* p, real iM, v2 P, real iI, real L) {
    p->lin = vsub(p->lin, vmul(P, iM)); p->ang = p->ang - iI * L;
}
static inline void add_imp(pos_t* p, real iM, v2 P, real iI, real L) {
    p->lin = vadd(p->lin, vmul(P, iM)); p->ang = p->ang + iI * L;
}
/* linear velocity + GetRevPerpendicular(r) * angular velocity */
static inline v2 point_vel(pos_t v, v2 r) { return vadd(v.lin, vmul(revperp(r), v.ang)); }
/* Matrix * vector, each row accumulated from zero (Vector.hpp:455-470); m[b][a]. */
static inline v2 mat22_mul(real m[2][2], v2 v) {
    real x = R(0); x += m[0][0] * v.x; x += m[0][1] * v.y;
    real y = R(0); y += m[1][0] * v.x; y += m[1][1] * v.y;
    return V(x, y);
}
/* Invert(Matrix22) (Math.hpp:430-442). */
static void mat22_invert(real k[2][2], real out[2][2]) {
    const real cp = cross(V(k[0][0], k[0][1]), V(k[1][0], k[1][1]));
    if (!almost_zero(cp)) {
        const real inv = R(1) / cp;
        out[0][0] = k[1][1] * inv; out[0][1] = -k[0][1] * inv;
        out[1][0] = -k[1][0] * inv; out[1][1] = k[0][0] * inv;
    } else {
        out[0][0] = out[0][1] = out[1][0] = out[1][1] = R(0);
    }
}
/* Vec3 Dot and Cross (Math.hpp:320-333, :397-409). */
static inline real dot3(const real* a, const real* b) { real r = R(0); r += a[0] * b[0]; r += a[1] * b[1]; r += a[2] * b[2]; return r; }
static inline void cross3(const real* a, const real* b, real* o) {
    const real x = a[1] * b[2] - a[2] * b[1], y = a[2] * b[0] - a[0] * b[2], z = a[0] * b[1] - a[1] * b[0];
    o[0] = x; o[1] = y; o[2] = z;
}
/* Solve33 / Solve22 / GetInverse22 / GetSymInverse33 (Math.hpp:447-512); K[i] is the i-th Vec3. */
static void solve33(real K[3][3], const real* b, real* o) {
    real c[3];
    cross3(K[1], K[2], c);
    const real dp = dot3(K[0], c);
    const real det = (dp != R(0)) ? (R(1) / dp) : dp;
    real t[3];
    const real x = det * dot3(b, c);
    cross3(b, K[2], t);
    const real y = det * dot3(K[0], t);
    cross3(K[1], b, t);
    const real z = det * dot3(K[0], t);
    o[0] = x; o[1] = y; o[2] = z;
}
static v2 solve22k(real K[3][3], v2 b) {
    const real xx = K[0][0], xy = K[1][0], yx = K[0][1], yy = K[1][1];
    const real cp = xx * yy - xy * yx;
    const real det = (cp != R(0)) ? (R(1) / cp) : cp;
    return V(det * (yy * b.x - xy * b.y), det * (xx * b.y - yx * b.x));
}
static void inverse22(real K[3][3], real o[3][3]) {
    const real a = K[0][0], b = K[1][0], c = K[0][1], d = K[1][1];
    real det = (a * d) - (b * c);
    if (det != R(0)) det = R(1) / det;
    o[0][0] = det * d; o[0][1] = -det * c; o[0][2] = R(0);
    o[1][0] = -det * b; o[1][1] = det * a; o[1][2] = R(0);
    o[2][0] = R(0); o[2][1] = R(0); o[2][2] = R(0);
}
static void sym_inverse33(real K[3][3], real o[3][3]) {
    real c[3];
    cross3(K[1], K[2], c);
    const real invDet = dot3(K[0], c);
    const real det = (invDet != R(0)) ? (R(1) / invDet) : invDet;
    const real a11 = K[0][0], a12 = K[1][0], a13 = K[2][0], a22 = K[1][1], a23 = K[2][1], a33 = K[2][2];
    const real ex_y = det * (a13 * a23 - a12 * a33);
    const real ey_z = det * (a13 * a12 - a11 * a23);
    const real ex_z = det * (a12 * a23 - a13 * a22);
    o[0][0] = det * (a22 * a33 - a23 * a23); o[0][1] = ex_y; o[0][2] = ex_z;
    o[1][0] = ex_y; o[1][1] = det * (a11 * a33 - a13 * a13); o[1][2] = ey_z;
    o[2][0] = ex_z; o[2][1] = ey_z; o[2][2] = det * (a11 * a22 - a12 * a12);
}
/* GetMat33 of the weld joint (WeldJointConf.cpp:36-62). */
static void weld_k(real iMA, v2 rA, real iIA, real iMB, v2 rB, real iIB, real K[3][3]) {
    const real exx = iMA + (rA.y * rA.y) * iIA + iMB + (rB.y * rB.y) * iIB;
    const real eyx = -rA.y * rA.x * iIA + -rB.y * rB.x * iIB;
    const real ezx = -rA.y * iIA + -rB.y * iIB;
    const real eyy = iMA + (rA.x * rA.x) * iIA + iMB + (rB.x * rB.x) * iIB;
    const real ezy = rA.x * iIA + rB.x * iIB;
    const real ezz = iIA + iIB;
    K[0][0] = exx; K[1][0] = eyx; K[2][0] = ezx;
    K[0][1] = eyx; K[1][1] = eyy; K[2][1] = ezy;
    K[0][2] = ezx; K[1][2] = ezy; K[2][2] = ezz;
}
static inline v2 anchor_r(v2 la, const bc_t* b) { return rotate(vsub(la, b->lc), unit_from_angle(b->pos.ang)); }

/* DistanceJointConf InitVelocity / SolveVelocity / SolvePosition (DistanceJointConf.cpp:79-247). */
static void dj_init_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t vA = A->vel, vB = B->vel;
    j->rA = anchor_r(j->laA, A);
    j->rB = anchor_r(j->laB, B);
    real length;
    j->u = unit_len(vsub(vadd(B->pos.lin, j->rB), vadd(A->pos.lin, j->rA)), &length);
    const real crAu = cross(j->rA, j->u), crBu = cross(j->rB, j->u);
    real invMass = A->invM + A->invI * (crAu * crAu) + B->invM + B->invI * (crBu * crBu);
    j->jmass = (invMass != R(0)) ? R(1) / invMass : R(0);
    const real frequency = j->extra[1], dampingRatio = j->extra[2];
    if (frequency > R(0)) {
        const real Pi = R(3.14159265358979323846264338327950288L);
        const real C = length - j->extra[0];
        const real omega = R(2) * Pi * frequency;
        const real d = R(2) * j->jmass * dampingRatio * omega;
        const real k = j->jmass * (omega * omega);
        const real h = conf->deltaTime;
        const real gamma = h * (d + h * k);
        j->invGamma = (gamma != R(0)) ? R(1) / gamma : R(0);
        j->bias = C * h * k * j->invGamma;
        invMass += j->invGamma;
        j->jmass = (invMass != R(0)) ? R(1) / invMass : R(0);
    } else {
        j->invGamma = R(0);
        j->bias = R(0);
    }
    if (conf->doWarmStart) {
        j->imp[0] *= conf->dtRatio;
        const v2 P = vmul(j->u, j->imp[0]);
        sub_imp(&vA, A->invM, P, A->invI, cross(j->rA, P));
        add_imp(&vB, B->invM, P, B->invI, cross(j->rB, P));
    } else {
        j->imp[0] = R(0);
    }
    A->vel = vA; B->vel = vB;
}
static int dj_solve_velocity(joint_t* j, bc_t* bcs) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t vA = A->vel, vB = B->vel;
    const real Cdot = dot(j->u, vsub(point_vel(vB, j->rB), point_vel(vA, j->rA)));
    const real impulse = -j->jmass * (Cdot + j->bias + j->invGamma * j->imp[0]);
    j->imp[0] += impulse;
    const v2 P = vmul(j->u, impulse);
    sub_imp(&vA, A->invM, P, A->invI, cross(j->rA, P));
    add_imp(&vB, B->invM, P, B->invI, cross(j->rB, P));
    A->vel = vA; B->vel = vB;
    return impulse == R(0);
}
static int dj_solve_position(const joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    if (j->extra[1] > R(0)) return 1;
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t pA = A->pos, pB = B->pos;
    const v2 rA = anchor_r(j->laA, A), rB = anchor_r(j->laB, B);
    real length;
    const v2 u = unit_len(vsub(vadd(pB.lin, rB), vadd(pA.lin, rA)), &length);
    const real C = clampr(length - j->extra[0], -conf->maxLinearCorrection, conf->maxLinearCorrection);
    const real impulse = -j->jmass * C;
    const v2 P = vmul(u, impulse);
    sub_imp(&pA, A->invM, P, A->invI, cross(rA, P));
    add_imp(&pB, B->invM, P, B->invI, cross(rB, P));
    A->pos = pA; B->pos = pB;
    return fabs(C) < conf->linearSlop;
}

/* RopeJointConf InitVelocity / SolveVelocity / SolvePosition (RopeJointConf.cpp:78-214). */
static void rope_init_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t vA = A->vel, vB = B->vel;
    j->rA = anchor_r(j->laA, A);
    j->rB = anchor_r(j->laB, B);
    const v2 uv = unit_len(vsub(vadd(B->pos.lin, j->rB), vadd(A->pos.lin, j->rA)), &j->length);
    const real C = j->length - j->extra[0];
    j->limitState = (C > R(0)) ? LS_UPPER : LS_INACTIVE;
    if (j->length > conf->linearSlop) {
        j->u = uv;
    } else {
        j->u = V(R(0), R(0));
        j->jmass = R(0);
        j->imp[0] = R(0);
        return;
    }
    const real crA = cross(j->rA, j->u), crB = cross(j->rB, j->u);
    const real invMass = A->invM + B->invM + A->invI * (crA * crA) + B->invI * (crB * crB);
    j->jmass = (invMass != R(0)) ? R(1) / invMass : R(0);
    if (conf->doWarmStart) {
        j->imp[0] *= conf->dtRatio;
        const v2 P = vmul(j->u, j->imp[0]);
        sub_imp(&vA, A->invM, P, A->invI, cross(j->rA, P));
        add_imp(&vB, B->invM, P, B->invI, cross(j->rB, P));
    } else {
        j->imp[0] = R(0);
    }
    A->vel = vA; B->vel = vB;
}
static int rope_solve_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t vA = A->vel, vB = B->vel;
    const v2 vpA = point_vel(vA, j->rA), vpB = point_vel(vB, j->rB);
    const real C = j->length - j->extra[0];
    const real inv_h = (conf->deltaTime != R(0)) ? R(1) / conf->deltaTime : R(0);
    const real Cdot = dot(j->u, vsub(vpB, vpA)) + ((C < R(0)) ? inv_h * C : R(0));
    real local = -j->jmass * Cdot;
    const real old = j->imp[0];
    j->imp[0] = minr(R(0), j->imp[0] + local);
    local = j->imp[0] - old;
    const v2 P = vmul(j->u, local);
    sub_imp(&vA, A->invM, P, A->invI, cross(j->rA, P));
    add_imp(&vB, B->invM, P, B->invI, cross(j->rB, P));
    A->vel = vA; B->vel = vB;
    return local == R(0);
}
static int rope_solve_position(const joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t pA = A->pos, pB = B->pos;
    const v2 rA = anchor_r(j->laA, A), rB = anchor_r(j->laB, B);
    real length;
    const v2 uv = unit_len(vsub(vadd(pB.lin, rB), vadd(pA.lin, rA)), &length);
    const real C = clampr(length - j->extra[0], R(0), conf->maxLinearCorrection);
    const real local = -j->jmass * C;
    const v2 P = vmul(uv, local);
    sub_imp(&pA, A->invM, P, A->invI, cross(rA, P));
    add_imp(&pB, B->invM, P, B->invI, cross(rB, P));
    A->pos = pA; B->pos = pB;
    return (length - j->extra[0]) < conf->linearSlop;
}

/* WeldJointConf InitVelocity / SolveVelocity / SolvePosition (WeldJointConf.cpp:133-376). */
static void weld_init_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t vA = A->vel, vB = B->vel;
    const real iMA = A->invM, iIA = A->invI, iMB = B->invM, iIB = B->invI;
    j->rA = anchor_r(j->laA, A);
    j->rB = anchor_r(j->laB, B);
    real K[3][3];
    weld_k(iMA, j->rA, iIA, iMB, j->rB, iIB, K);
    const real frequency = j->extra[1], dampingRatio = j->extra[2];
    if (frequency > R(0)) {
        inverse22(K, j->mass);
        real invRotInertia = iIA + iIB;
        const real rotInertia = (invRotInertia > R(0)) ? R(1) / invRotInertia : R(0);
        const real C = B->pos.ang - A->pos.ang - j->extra[0];
        const real Pi = R(3.14159265358979323846264338327950288L);
        const real omega = R(2) * Pi * frequency;
        const real d = R(2) * rotInertia * dampingRatio * omega;
        const real k = rotInertia * omega * omega;
        const real h = conf->deltaTime;
        const real invGamma = h * (d + h * k);
        j->invGamma = (invGamma != R(0)) ? R(1) / invGamma : R(0); /* the joint's gamma */
        j->bias = C * h * k * j->invGamma;
        invRotInertia += j->invGamma;
        j->mass[2][2] = (invRotInertia != R(0)) ? R(1) / invRotInertia : R(0);
    } else if (K[2][2] == R(0)) {
        inverse22(K, j->mass);
        j->invGamma = R(0);
        j->bias = R(0);
    } else {
        sym_inverse33(K, j->mass);
        j->invGamma = R(0);
        j->bias = R(0);
    }
    if (conf->doWarmStart) {
        j->imp[0] *= conf->dtRatio; j->imp[1] *= conf->dtRatio; j->imp[2] *= conf->dtRatio;
        const v2 P = V(j->imp[0], j->imp[1]);
        const real L = j->imp[2];
        sub_imp(&vA, iMA, P, iIA, L + cross(j->rA, P));
        add_imp(&vB, iMB, P, iIB, L + cross(j->rB, P));
    } else {
        j->imp[0] = j->imp[1] = j->imp[2] = R(0);
    }
    A->vel = vA; B->vel = vB;
}
static int weld_solve_velocity(joint_t* j, bc_t* bcs) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    const pos_t oA = A->vel, oB = B->vel;
    pos_t vA = oA, vB = oB;
    const real iMA = A->invM, iIA = A->invI, iMB = B->invM, iIB = B->invI;
    if (j->extra[1] > R(0)) {
        const real Cdot2 = vB.ang - vA.ang;
        const real gamma = j->invGamma * j->imp[2];
        const real impulse2 = -j->mass[2][2] * (Cdot2 + j->bias + gamma);
        j->imp[2] += impulse2;
        vA.ang -= iIA * impulse2;
        vB.ang += iIB * impulse2;
        const v2 Cdot1 = vsub(point_vel(vB, j->rB), point_vel(vA, j->rA));
        /* Transform(Vec2, Mat33) (Math.hpp:522-527) */
        const v2 t = V(j->mass[0][0] * Cdot1.x + j->mass[1][0] * Cdot1.y,
                       j->mass[0][1] * Cdot1.x + j->mass[1][1] * Cdot1.y);
        const v2 impulse1 = vneg(t);
        j->imp[0] += impulse1.x;
        j->imp[1] += impulse1.y;
        const v2 P = impulse1;
        sub_imp(&vA, iMA, P, iIA, cross(j->rA, P));
        add_imp(&vB, iMB, P, iIB, cross(j->rB, P));
    } else {
        const v2 Cdot1 = vsub(point_vel(vB, j->rB), point_vel(vA, j->rA));
        const real Cdot2 = vB.ang - vA.ang;
        const real Cdot[3] = {Cdot1.x, Cdot1.y, Cdot2};
        real imp3[3];
        for (int b = 0; b < 3; ++b) imp3[b] = -dot3(j->mass[b], Cdot); /* -(mass * Cdot) */
        j->imp[0] += imp3[0]; j->imp[1] += imp3[1]; j->imp[2] += imp3[2];
        const v2 P = V(imp3[0], imp3[1]);
        const real L = imp3[2];
        sub_imp(&vA, iMA, P, iIA, L + cross(j->rA, P));
        add_imp(&vB, iMB, P, iIB, L + cross(j->rB, P));
    }
    const int changed = pos_ne(vA, oA) || pos_ne(vB, oB);
    if (changed) { A->vel = vA; B->vel = vB; }
    return !changed;
}
static int weld_solve_position(const joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t pA = A->pos, pB = B->pos;
    const real iMA = A->invM, iIA = A->invI, iMB = B->invM, iIB = B->invI;
    const v2 rA = anchor_r(j->laA, A), rB = anchor_r(j->laB, B);
    real positionError, angularError;
    real K[3][3];
    weld_k(iMA, rA, iIA, iMB, rB, iIB, K);
    const v2 C1 = vsub(vadd(pB.lin, rB), vadd(pA.lin, rA));
    if (j->extra[1] > R(0)) {
        positionError = RSQRT(mag2(C1));
        angularError = R(0);
        const v2 P = vneg(solve22k(K, C1));
        sub_imp(&pA, iMA, P, iIA, cross(rA, P));
        add_imp(&pB, iMB, P, iIB, cross(rB, P));
    } else {
        const real C2 = pB.ang - pA.ang - j->extra[0];
        positionError = RSQRT(mag2(C1));
        angularError = fabs(C2);
        const real C[3] = {C1.x, C1.y, C2};
        real imp3[3];
        if (K[2][2] > R(0)) {
            real s[3];
            solve33(K, C, s);
            imp3[0] = -s[0]; imp3[1] = -s[1]; imp3[2] = -s[2];
        } else {
            const v2 i2 = vneg(solve22k(K, C1));
            imp3[0] = i2.x; imp3[1] = i2.y; imp3[2] = R(0);
        }
        const v2 P = V(imp3[0], imp3[1]);
        const real L = imp3[2];
        sub_imp(&pA, iMA, P, iIA, L + cross(rA, P));
        add_imp(&pB, iMB, P, iIB, L + cross(rB, P));
    }
    A->pos = pA; B->pos = pB;
    return (positionError <= conf->linearSlop) && (angularError <= conf->angularSlop);
}

/* FrictionJointConf (FrictionJointConf.cpp:90-239) and MotorJointConf
 * (MotorJointConf.cpp:89-235): a 2x2 linear and a scalar angular friction. */
static void fm_init_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf, int motor) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t vA = A->vel, vB = B->vel;
    const real iMA = A->invM, iIA = A->invI, iMB = B->invM, iIB = B->invI;
    if (motor) {
        j->rA = rotate(vsub(V(j->extra[0], j->extra[1]), A->lc), unit_from_angle(A->pos.ang));
        j->rB = rotate(vneg(B->lc), unit_from_angle(B->pos.ang));
    } else {
        j->rA = anchor_r(j->laA, A);
        j->rB = anchor_r(j->laB, B);
    }
    const v2 rA = j->rA, rB = j->rB;
    real K[2][2];
    if (motor) {
        K[0][0] = iMA + iMB + iIA * (rA.y * rA.y) + iIB * (rB.y * rB.y);
        K[0][1] = -iIA * rA.x * rA.y + -iIB * rB.x * rB.y;
        K[1][1] = iMA + iMB + iIA * (rA.x * rA.x) + iIB * (rB.x * rB.x);
    } else {
        K[0][0] = iMA + iIA * (rA.y * rA.y) + iMB + iIB * (rB.y * rB.y);
        K[0][1] = -iIA * rA.x * rA.y + -iIB * rB.x * rB.y;
        K[1][1] = iMA + iIA * (rA.x * rA.x) + iMB + iIB * (rB.x * rB.x);
    }
    K[1][0] = K[0][1];
    mat22_invert(K, j->lm);
    const real invRotInertia = iIA + iIB;
    j->angularMass = (invRotInertia > R(0)) ? R(1) / invRotInertia : R(0);
    if (motor) {
        j->linErr = vsub(vadd(B->pos.lin, rB), vadd(A->pos.lin, rA));
        j->angErr = (B->pos.ang - A->pos.ang) - j->extra[2];
    }
    if (conf->doWarmStart) {
        j->imp[0] *= conf->dtRatio; j->imp[1] *= conf->dtRatio; j->imp[2] *= conf->dtRatio;
        const v2 P = V(j->imp[0], j->imp[1]);
        sub_imp(&vA, iMA, P, iIA, cross(rA, P) + j->imp[2]);
        add_imp(&vB, iMB, P, iIB, cross(rB, P) + j->imp[2]);
    } else {
        j->imp[0] = j->imp[1] = j->imp[2] = R(0);
    }
    A->vel = vA; B->vel = vB;
}
/* The linear impulse, clamped to h * maxForce in magnitude. */
static v2 clamp_linear(joint_t* j, v2 impulse, real maxImpulse) {
    const v2 old = V(j->imp[0], j->imp[1]);
    v2 li = vadd(old, impulse);
    if (mag2(li) > maxImpulse * maxImpulse) li = vmul(unit_vector(li, V(R(0), R(0))), maxImpulse);
    j->imp[0] = li.x; j->imp[1] = li.y;
    return vsub(li, old);
}
static int friction_solve_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t vA = A->vel, vB = B->vel;
    const real iIA = A->invI, iIB = B->invI;
    const real h = conf->deltaTime;
    const real maxForce = j->extra[0], maxTorque = j->extra[1];
    int solved = 1;
    {
        const real angularImpulse = -j->angularMass * (vB.ang - vA.ang);
        const real old = j->imp[2];
        const real maxAng = h * maxTorque;
        j->imp[2] = clampr(j->imp[2] + angularImpulse, -maxAng, maxAng);
        const real inc = j->imp[2] - old;
        if (inc != R(0)) solved = 0;
        vA.ang -= iIA * inc;
        vB.ang += iIB * inc;
    }
    {
        const v2 impulse = vneg(mat22_mul(j->lm, vsub(point_vel(vB, j->rB), point_vel(vA, j->rA))));
        const v2 inc = clamp_linear(j, impulse, h * maxForce);
        const real angA = cross(j->rA, inc), angB = cross(j->rB, inc);
        if (inc.x != R(0) || inc.y != R(0)) solved = 0;
        sub_imp(&vA, A->invM, inc, iIA, angA);
        add_imp(&vB, B->invM, inc, iIB, angB);
    }
    A->vel = vA; B->vel = vB;
    return solved;
}
static int motor_solve_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t vA = A->vel, vB = B->vel;
    const real iMA = A->invM, iIA = A->invI, iMB = B->invM, iIB = B->invI;
    const real h = conf->deltaTime;
    const real inv_h = (h != R(0)) ? R(1) / h : R(0);
    const real maxForce = j->extra[3], maxTorque = j->extra[4], cf = j->extra[5];
    int solved = 1;
    {
        const real Cdot = (vB.ang - vA.ang) + inv_h * cf * j->angErr;
        const real angularImpulse = -j->angularMass * Cdot;
        const real old = j->imp[2];
        const real maxAng = h * maxTorque;
        const real nw = clampr(old + angularImpulse, -maxAng, maxAng);
        j->imp[2] = nw;
        const real inc = nw - old;
        if (inc != R(0)) {
            sub_imp(&vA, R(0), V(R(0), R(0)), iIA, inc);
            add_imp(&vB, R(0), V(R(0), R(0)), iIB, inc);
            solved = 0;
        }
    }
    {
        const v2 Cdot = vadd(vsub(point_vel(vB, j->rB), point_vel(vA, j->rA)), vmul(j->linErr, inv_h * cf));
        const v2 impulse = vneg(mat22_mul(j->lm, Cdot));
        const v2 inc = clamp_linear(j, impulse, h * maxForce);
        const real angA = cross(j->rA, inc), angB = cross(j->rB, inc);
        if (inc.x != R(0) || inc.y != R(0) || angA != R(0) || angB != R(0)) {
            sub_imp(&vA, iMA, inc, iIA, angA);
            add_imp(&vB, iMB, inc, iIB, angB);
            solved = 0;
        }
    }
    if (solved) return 1;
    A->vel = vA; B->vel = vB;
    return 0;
}

/* Solve(Matrix22, Vector2) (Math.hpp:412-425): rows k[0], k[1]. */
static v2 solve22m(real k[2][2], v2 b) {
    const real cp = cross(V(k[0][0], k[0][1]), V(k[1][0], k[1][1]));
    if (!almost_zero(cp)) {
        const real inverse = R(1) / cp;
        return V((k[1][1] * b.x - k[1][0] * b.y) * inverse, (k[0][0] * b.y - k[0][1] * b.x) * inverse);
    }
    return V(R(0), R(0));
}
/* std::max / std::min as the reference calls them: (a < b) ? b : a and (b < a) ? b : a. */
static inline real stdmax(real a, real b) { return (a < b) ? b : a; }
static inline real stdmin(real a, real b) { return (b < a) ? b : a; }
/* Velocity / Position -= and += {invMass * P, invRotI * L} with the scaling first (Velocity.hpp). */

/* PrismaticJointConf InitVelocity / SolveVelocity / SolvePosition
 * (PrismaticJointConf.cpp:95-449); extra = localXAxisA.xy referenceAngle
 * lowerTranslation upperTranslation motorSpeed maxMotorForce. */
static void pj_init_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t vA = A->vel, vB = B->vel;
    const real iMA = A->invM, iIA = A->invI, iMB = B->invM, iIB = B->invI;
    const v2 qA = unit_from_angle(A->pos.ang);
    const v2 rA = anchor_r(j->laA, A), rB = anchor_r(j->laB, B);
    const v2 d = vsub(vadd(vsub(B->pos.lin, A->pos.lin), rB), rA);
    const v2 xaxis = V(j->extra[0], j->extra[1]);
    j->axis = urotate(xaxis, qA);
    j->a1 = cross(vadd(d, rA), j->axis);
    j->a2 = cross(rB, j->axis);
    const real invRotMassA = iIA * (j->a1 * j->a1);
    const real invRotMassB = iIB * (j->a2 * j->a2);
    const real totalInvMass = iMA + iMB + invRotMassA + invRotMassB;
    j->jmass = (totalInvMass > R(0)) ? R(1) / totalInvMass : R(0);
    {
        j->perp = urotate(revperp(xaxis), qA);
        j->s1 = cross(vadd(d, rA), j->perp);
        j->s2 = cross(rB, j->perp);
        const real invRotMassA2 = iIA * (j->s1 * j->s1);
        const real invRotMassB2 = iIB * (j->s2 * j->s2);
        const real k11 = iMA + iMB + invRotMassA2 + invRotMassB2;
        const real k12 = iIA * j->s1 + iIB * j->s2;
        const real k13 = iIA * j->s1 * j->a1 + iIB * j->s2 * j->a2;
        const real totalInvRotInertia = iIA + iIB;
        const real k22 = (totalInvRotInertia == R(0)) ? R(1) : totalInvRotInertia;
        const real k23 = iIA * j->a1 + iIB * j->a2;
        const real k33 = totalInvMass;
        j->mass[0][0] = k11; j->mass[0][1] = k12; j->mass[0][2] = k13;
        j->mass[1][0] = k12; j->mass[1][1] = k22; j->mass[1][2] = k23;
        j->mass[2][0] = k13; j->mass[2][1] = k23; j->mass[2][2] = k33;
    }
    const real lower = j->extra[3], upper = j->extra[4];
    if (j->enableLimit) {
        const real jointTranslation = dot(j->axis, d);
        if (fabs(upper - lower) < (conf->linearSlop * R(2))) {
            j->limitState = LS_EQUAL;
        } else if (jointTranslation <= lower) {
            if (j->limitState != LS_LOWER) { j->limitState = LS_LOWER; j->imp[2] = R(0); }
        } else if (jointTranslation >= upper) {
            if (j->limitState != LS_UPPER) { j->limitState = LS_UPPER; j->imp[2] = R(0); }
        } else {
            j->limitState = LS_INACTIVE;
            j->imp[2] = R(0);
        }
    } else {
        j->limitState = LS_INACTIVE;
        j->imp[2] = R(0);
    }
    if (!j->enableMotor) j->motorImpulse = R(0);
    if (conf->doWarmStart) {
        j->imp[0] *= conf->dtRatio; j->imp[1] *= conf->dtRatio; j->imp[2] *= conf->dtRatio;
        j->motorImpulse *= conf->dtRatio;
        const v2 Px = vmul(j->perp, j->imp[0]);
        const real Pxs1 = j->imp[0] * j->s1;
        const real Pxs2 = j->imp[0] * j->s2;
        const real PzLength = j->motorImpulse + j->imp[2];
        const v2 Pz = vmul(j->axis, PzLength);
        const v2 P = vadd(Px, Pz);
        const real L = j->imp[1];
        const real LA = L + (Pxs1 + PzLength * j->a1);
        const real LB = L + (Pxs2 + PzLength * j->a2);
        sub_imp(&vA, iMA, P, iIA, LA);
        add_imp(&vB, iMB, P, iIB, LB);
    } else {
        j->imp[0] = j->imp[1] = j->imp[2] = R(0);
        j->motorImpulse = R(0);
    }
    A->vel = vA; B->vel = vB;
}
static int pj_solve_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    const pos_t oldA = A->vel, oldB = B->vel;
    pos_t vA = oldA, vB = oldB;
    const real iMA = A->invM, iIA = A->invI, iMB = B->invM, iIB = B->invI;
    if (j->enableMotor && j->limitState != LS_EQUAL) {
        const real vDot = dot(j->axis, vsub(vB.lin, vA.lin));
        const real Cdot = vDot + (j->a2 * vB.ang - j->a1 * vA.ang);
        real impulse = j->jmass * (j->extra[5] - Cdot);
        const real oldImpulse = j->motorImpulse;
        const real maxImpulse = conf->deltaTime * j->extra[6];
        j->motorImpulse = clampr(j->motorImpulse + impulse, -maxImpulse, maxImpulse);
        impulse = j->motorImpulse - oldImpulse;
        const v2 P = vmul(j->axis, impulse);
        const real LA = impulse * j->a1, LB = impulse * j->a2;
        sub_imp(&vA, iMA, P, iIA, LA);
        add_imp(&vB, iMB, P, iIB, LB);
    }
    const v2 velDelta = vsub(vB.lin, vA.lin);
    const real sRotSpeed = j->s2 * vB.ang - j->s1 * vA.ang;
    const v2 Cdot1 = V(dot(j->perp, velDelta) + sRotSpeed, vB.ang - vA.ang);
    if (j->enableLimit && j->limitState != LS_INACTIVE) {
        const real deltaDot = dot(j->axis, velDelta);
        const real aRotSpeed = j->a2 * vB.ang - j->a1 * vA.ang;
        const real Cdot2 = deltaDot + aRotSpeed;
        const real negCdot[3] = {-Cdot1.x, -Cdot1.y, -Cdot2};
        const real f1[3] = {j->imp[0], j->imp[1], j->imp[2]};
        real add[3];
        solve33(j->mass, negCdot, add);
        j->imp[0] += add[0]; j->imp[1] += add[1]; j->imp[2] += add[2];
        if (j->limitState == LS_LOWER) j->imp[2] = stdmax(j->imp[2], R(0));
        else if (j->limitState == LS_UPPER) j->imp[2] = stdmin(j->imp[2], R(0));
        const real dz = j->imp[2] - f1[2];
        const v2 b = V(-Cdot1.x - dz * j->mass[2][0], -Cdot1.y - dz * j->mass[2][1]);
        const v2 s22 = solve22k(j->mass, b);
        const v2 f2r = V(s22.x + f1[0], s22.y + f1[1]);
        j->imp[0] = f2r.x; j->imp[1] = f2r.y;
        const real df[3] = {j->imp[0] - f1[0], j->imp[1] - f1[1], j->imp[2] - f1[2]};
        const v2 P = vadd(vmul(j->perp, df[0]), vmul(j->axis, df[2]));
        const real LA = df[0] * j->s1 + df[1] + df[2] * j->a1;
        const real LB = df[0] * j->s2 + df[1] + df[2] * j->a2;
        sub_imp(&vA, iMA, P, iIA, LA);
        add_imp(&vB, iMB, P, iIB, LB);
    } else {
        const v2 df = solve22k(j->mass, vneg(Cdot1));
        j->imp[0] += df.x; j->imp[1] += df.y;
        const v2 P = vmul(j->perp, df.x);
        const real LA = df.x * j->s1 + df.y;
        const real LB = df.x * j->s2 + df.y;
        sub_imp(&vA, iMA, P, iIA, LA);
        add_imp(&vB, iMB, P, iIB, LB);
    }
    if (pos_ne(vA, oldA) || pos_ne(vB, oldB)) {
        A->vel = vA; B->vel = vB;
        return 0;
    }
    return 1;
}
static int pj_solve_position(const joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t pA = A->pos, pB = B->pos;
    const real iMA = A->invM, iIA = A->invI, iMB = B->invM, iIB = B->invI;
    const v2 qA = unit_from_angle(pA.ang);
    const v2 rA = anchor_r(j->laA, A), rB = anchor_r(j->laB, B);
    const v2 d = vsub(vadd(pB.lin, rB), vadd(pA.lin, rA));
    const v2 xaxis = V(j->extra[0], j->extra[1]);
    const v2 axis = urotate(xaxis, qA);
    const real a1 = cross(vadd(d, rA), axis), a2 = cross(rB, axis);
    const v2 perp = urotate(revperp(xaxis), qA);
    const real s1 = cross(vadd(d, rA), perp), s2 = cross(rB, perp);
    const v2 C1 = V(dot(perp, d), pB.ang - pA.ang - j->extra[2]);
    real linearError = fabs(C1.x);
    const real angularError = fabs(C1.y);
    int active = 0;
    real C2 = R(0);
    const real lower = j->extra[3], upper = j->extra[4];
    if (j->enableLimit) {
        const real translation = dot(axis, d);
        if (fabs(upper - lower) < (R(2) * conf->linearSlop)) {
            C2 = clampr(translation, -conf->maxLinearCorrection, conf->maxLinearCorrection);
            linearError = stdmax(linearError, fabs(translation));
            active = 1;
        } else if (translation <= lower) {
            C2 = clampr(translation - lower + conf->linearSlop, -conf->maxLinearCorrection, R(0));
            linearError = stdmax(linearError, lower - translation);
            active = 1;
        } else if (translation >= upper) {
            C2 = clampr(translation - upper - conf->linearSlop, R(0), conf->maxLinearCorrection);
            linearError = stdmax(linearError, translation - upper);
            active = 1;
        }
    }
    real impulse[3];
    if (active) {
        const real k11 = iMA + iIA * (s1 * s1) + iMB + iIB * (s2 * s2);
        const real k12 = iIA * s1 + iIB * s2;
        const real k13 = iIA * s1 * a1 + iIB * s2 * a2;
        real k22 = iIA + iIB;
        if (k22 == R(0)) k22 = R(1);
        const real k23 = iIA * a1 + iIB * a2;
        const real k33 = iMA + iIA * (a1 * a1) + iMB + iIB * (a2 * a2);
        real K[3][3] = {{k11, k12, k13}, {k12, k22, k23}, {k13, k23, k33}};
        const real negC[3] = {-C1.x, -C1.y, -C2};
        solve33(K, negC, impulse);
    } else {
        const real k11 = iMA + iIA * s1 * s1 + iMB + iIB * s2 * s2;
        const real k12 = iIA * s1 + iIB * s2;
        real k22 = iIA + iIB;
        if (k22 == R(0)) k22 = R(1);
        real K[2][2] = {{k11, k12}, {k12, k22}};
        const v2 i1 = solve22m(K, vneg(C1));
        impulse[0] = i1.x; impulse[1] = i1.y; impulse[2] = R(0);
    }
    const v2 P = vadd(vmul(perp, impulse[0]), vmul(axis, impulse[2]));
    const real LA = impulse[0] * s1 + impulse[1] + impulse[2] * a1;
    const real LB = impulse[0] * s2 + impulse[1] + impulse[2] * a2;
    sub_imp(&pA, iMA, P, iIA, LA);
    add_imp(&pB, iMB, P, iIB, LB);
    A->pos = pA; B->pos = pB;
    return (linearError <= conf->linearSlop) && (angularError <= conf->angularSlop);
}

/* WheelJointConf InitVelocity / SolveVelocity / SolvePosition
 * (WheelJointConf.cpp:80-311); extra = localXAxisA.xy motorSpeed maxMotorTorque
 * frequency dampingRatio. */
static void wj_init_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t vA = A->vel, vB = B->vel;
    const real iMA = A->invM, iIA = A->invI, iMB = B->invM, iIB = B->invI;
    const v2 qA = unit_from_angle(A->pos.ang);
    const v2 rA = anchor_r(j->laA, A), rB = anchor_r(j->laB, B);
    const v2 dd = vsub(vadd(B->pos.lin, rB), vadd(A->pos.lin, rA));
    const v2 xaxis = V(j->extra[0], j->extra[1]);
    {
        j->perp = urotate(revperp(xaxis), qA);  /* ay */
        j->s1 = cross(vadd(dd, rA), j->perp);   /* sAy */
        j->s2 = cross(rB, j->perp);             /* sBy */
        const real invRotMassA = iIA * (j->s1 * j->s1);
        const real invRotMassB = iIB * (j->s2 * j->s2);
        const real invMass = iMA + iMB + invRotMassA + invRotMassB;
        j->jmass = (invMass > R(0)) ? R(1) / invMass : R(0);
    }
    j->springMass = R(0);
    j->bias = R(0);
    j->gamma = R(0);
    const real frequency = j->extra[4], dampingRatio = j->extra[5];
    if (frequency > R(0)) {
        j->axis = urotate(xaxis, qA);           /* ax */
        j->a1 = cross(vadd(dd, rA), j->axis);   /* sAx */
        j->a2 = cross(rB, j->axis);             /* sBx */
        const real invRotMassA = iIA * (j->a1 * j->a1);
        const real invRotMassB = iIB * (j->a2 * j->a2);
        const real invMass = iMA + iMB + invRotMassA + invRotMassB;
        if (invMass > R(0)) {
            j->springMass = R(1) / invMass;
            const real C = dot(dd, j->axis);
            const real Pi = R(3.14159265358979323846264338327950288L);
            const real omega = R(2) * Pi * frequency;
            const real d = R(2) * j->springMass * dampingRatio * omega;
            const real k = j->springMass * omega * omega;
            const real h = conf->deltaTime;
            const real invGamma = h * (d + h * k);
            j->gamma = (invGamma > R(0)) ? R(1) / invGamma : R(0);
            j->bias = C * h * k * j->gamma;
            const real totalInvMass = invMass + j->gamma;
            j->springMass = (totalInvMass > R(0)) ? R(1) / totalInvMass : R(0);
        }
    } else {
        j->springImp = R(0);
        j->axis = V(R(0), R(0));
        j->a1 = R(0);
        j->a2 = R(0);
    }
    if (j->enableMotor) {
        const real invRotInertia = iIA + iIB;
        j->angularMass = (invRotInertia > R(0)) ? R(1) / invRotInertia : R(0);
    } else {
        j->angularMass = R(0);
        j->angImp = R(0);
    }
    if (conf->doWarmStart) {
        j->imp[0] *= conf->dtRatio;
        j->springImp *= conf->dtRatio;
        j->angImp *= conf->dtRatio;
        const v2 P = vadd(vmul(j->perp, j->imp[0]), vmul(j->axis, j->springImp));
        const real LA = (j->imp[0] * j->s1 + j->springImp * j->a1) + j->angImp;
        const real LB = (j->imp[0] * j->s2 + j->springImp * j->a2) + j->angImp;
        sub_imp(&vA, iMA, P, iIA, LA);
        add_imp(&vB, iMB, P, iIB, LB);
    } else {
        j->imp[0] = R(0);
        j->springImp = R(0);
        j->angImp = R(0);
    }
    A->vel = vA; B->vel = vB;
}
static int wj_solve_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    const pos_t oldA = A->vel, oldB = B->vel;
    pos_t vA = oldA, vB = oldB;
    const real iMA = A->invM, iIA = A->invI, iMB = B->invM, iIB = B->invI;
    {
        const real d = dot(j->axis, vsub(vB.lin, vA.lin));
        const real Cdot = d + j->a2 * vB.ang - j->a1 * vA.ang;
        const real impulse = -j->springMass * (Cdot + j->bias + j->gamma * j->springImp);
        j->springImp += impulse;
        const v2 P = vmul(j->axis, impulse);
        const real LA = impulse * j->a1, LB = impulse * j->a2;
        sub_imp(&vA, iMA, P, iIA, LA);
        add_imp(&vB, iMB, P, iIB, LB);
    }
    {
        const real Cdot = vB.ang - vA.ang - j->extra[2];
        real impulse = -j->angularMass * Cdot;
        const real oldImpulse = j->angImp;
        const real maxImpulse = conf->deltaTime * j->extra[3];
        j->angImp = clampr(j->angImp + impulse, -maxImpulse, maxImpulse);
        impulse = j->angImp - oldImpulse;
        vA.ang -= iIA * impulse;
        vB.ang += iIB * impulse;
    }
    {
        const real d = dot(j->perp, vsub(vB.lin, vA.lin));
        const real Cdot = d + j->s2 * vB.ang - j->s1 * vA.ang;
        const real impulse = -j->jmass * Cdot;
        j->imp[0] += impulse;
        const v2 P = vmul(j->perp, impulse);
        const real LA = impulse * j->s1, LB = impulse * j->s2;
        sub_imp(&vA, iMA, P, iIA, LA);
        add_imp(&vB, iMB, P, iIB, LB);
    }
    if (pos_ne(vA, oldA) || pos_ne(vB, oldB)) {
        A->vel = vA; B->vel = vB;
        return 0;
    }
    return 1;
}
static int wj_solve_position(const joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t pA = A->pos, pB = B->pos;
    const real iMA = A->invM, iIA = A->invI, iMB = B->invM, iIB = B->invI;
    const v2 qA = unit_from_angle(pA.ang);
    const v2 rA = anchor_r(j->laA, A), rB = anchor_r(j->laB, B);
    const v2 d = vadd(vsub(pB.lin, pA.lin), vsub(rB, rA));
    const v2 ay = urotate(revperp(V(j->extra[0], j->extra[1])), qA);
    const real sAy = cross(vadd(d, rA), ay);
    const real sBy = cross(rB, ay);
    const real C = dot(d, ay);
    /* the effective mass uses sAy and sBy as InitVelocity left them */
    const real invRotMassA = iIA * (j->s1 * j->s1);
    const real invRotMassB = iIB * (j->s2 * j->s2);
    const real k = iMA + iMB + invRotMassA + invRotMassB;
    const real impulse = (k != R(0)) ? -(C / k) : R(0);
    const v2 P = vmul(ay, impulse);
    const real LA = impulse * sAy, LB = impulse * sBy;
    sub_imp(&pA, iMA, P, iIA, LA);
    add_imp(&pB, iMB, P, iIB, LB);
    A->pos = pA; B->pos = pB;
    return fabs(C) <= conf->linearSlop;
}

/* PulleyJointConf InitVelocity / SolveVelocity / SolvePosition
 * (PulleyJointConf.cpp:93-241); extra = groundAnchorA.xy groundAnchorB.xy
 * lengthA lengthB ratio. */
static void pu_init_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t vA = A->vel, vB = B->vel;
    const real iMA = A->invM, iIA = A->invI, iMB = B->invM, iIB = B->invI;
    const real ratio = j->extra[6];
    j->rA = anchor_r(j->laA, A);
    j->rB = anchor_r(j->laB, B);
    const v2 pulleyAxisA = vsub(vadd(A->pos.lin, j->rA), V(j->extra[0], j->extra[1]));
    const v2 pulleyAxisB = vsub(vadd(B->pos.lin, j->rB), V(j->extra[2], j->extra[3]));
    j->u = unit_vector(pulleyAxisA, V(R(0), R(0)));
    j->u2 = unit_vector(pulleyAxisB, V(R(0), R(0)));
    const real ruA = cross(j->rA, j->u);
    const real ruB = cross(j->rB, j->u2);
    const real totInvMassA = iMA + (iIA * (ruA * ruA));
    const real totInvMassB = iMB + (iIB * (ruB * ruB));
    const real totalInvMass = totInvMassA + ratio * ratio * totInvMassB;
    j->jmass = (totalInvMass > R(0)) ? R(1) / totalInvMass : R(0);
    if (conf->doWarmStart) {
        j->imp[0] *= conf->dtRatio;
        const v2 PA = vmul(j->u, -(j->imp[0]));
        const v2 PB = vmul(j->u2, (-ratio * j->imp[0]));
        add_imp(&vA, iMA, PA, iIA, cross(j->rA, PA));
        add_imp(&vB, iMB, PB, iIB, cross(j->rB, PB));
    } else {
        j->imp[0] = R(0);
    }
    A->vel = vA; B->vel = vB;
}
static int pu_solve_velocity(joint_t* j, bc_t* bcs) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t vA = A->vel, vB = B->vel;
    const real iMA = A->invM, iIA = A->invI, iMB = B->invM, iIB = B->invI;
    const real ratio = j->extra[6];
    const v2 vpA = point_vel(vA, j->rA);
    const v2 vpB = point_vel(vB, j->rB);
    const real Cdot = -dot(j->u, vpA) - ratio * dot(j->u2, vpB);
    const real impulse = -j->jmass * Cdot;
    j->imp[0] += impulse;
    const v2 PA = vmul(j->u, -impulse);
    const v2 PB = vmul(j->u2, -ratio * impulse);
    add_imp(&vA, iMA, PA, iIA, cross(j->rA, PA));
    add_imp(&vB, iMB, PB, iIB, cross(j->rB, PB));
    A->vel = vA; B->vel = vB;
    return impulse == R(0);
}
static int pu_solve_position(const joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    pos_t pA = A->pos, pB = B->pos;
    const real iMA = A->invM, iIA = A->invI, iMB = B->invM, iIB = B->invI;
    const real ratio = j->extra[6];
    const v2 rA = anchor_r(j->laA, A), rB = anchor_r(j->laB, B);
    real lengthA, lengthB;
    const v2 uA = unit_len(vsub(vadd(pA.lin, rA), V(j->extra[0], j->extra[1])), &lengthA);
    const v2 uB = unit_len(vsub(vadd(pB.lin, rB), V(j->extra[2], j->extra[3])), &lengthB);
    const real ruA = cross(rA, uA);
    const real ruB = cross(rB, uB);
    const real totalInvMassA = iMA + iIA * (ruA * ruA);
    const real totalInvMassB = iMB + iIB * (ruB * ruB);
    const real totalInvMass = totalInvMassA + (ratio * ratio) * totalInvMassB;
    const real mass = (totalInvMass > R(0)) ? R(1) / totalInvMass : R(0);
    const real srcLengthRatio = j->extra[4] + ratio * j->extra[5];
    const real dstLengthRatio = lengthA + ratio * lengthB;
    const real C = srcLengthRatio - dstLengthRatio;
    const real linearError = fabs(C);
    const real impulse = -mass * C;
    const v2 PA = vmul(uA, -impulse);
    const v2 PB = vmul(uB, -ratio * impulse);
    add_imp(&pA, iMA, PA, iIA, cross(rA, PA));
    add_imp(&pB, iMB, PB, iIB, cross(rB, PB));
    A->pos = pA; B->pos = pB;
    return linearError < conf->linearSlop;
}

/* TargetJointConf InitVelocity / SolveVelocity (TargetJointConf.cpp:51-184);
 * the joint has only body B (bA == bB here); extra = target.xy maxForce
 * frequency dampingRatio. */
static void tj_init_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* B = &bcs[j->bB];
    const pos_t posB = B->pos;
    pos_t vB = B->vel;
    const v2 qB = unit_from_angle(posB.ang);
    const real iM = B->invM, iI = B->invI;
    const real mass = (iM != R(0)) ? (R(1) / iM) : R(0);
    const real Pi = R(3.14159265358979323846264338327950288L);
    const real omega = R(2) * Pi * j->extra[3];
    const real d = R(2) * mass * j->extra[4] * omega;
    const real k = mass * (omega * omega);
    const real h = conf->deltaTime;
    const real tmp = d + h * k;
    const real invGamma = h * tmp;
    j->gamma = (invGamma != R(0)) ? R(1) / invGamma : R(0);
    const real beta = h * k * j->gamma;
    j->rB = rotate(vsub(j->laB, B->lc), qB);
    {
        /* GetEffectiveMassMatrix (TargetJointConf.cpp:51-72) */
        const real exx = iM + (iI * (j->rB.y * j->rB.y)) + j->gamma;
        const real exy = -iI * j->rB.x * j->rB.y;
        const real eyy = iM + (iI * (j->rB.x * j->rB.x)) + j->gamma;
        real K[2][2] = {{exx, exy}, {exy, eyy}};
        mat22_invert(K, j->lm);
    }
    j->linErr = vmul(vsub(vadd(posB.lin, j->rB), V(j->extra[0], j->extra[1])), beta);
    const real DampingAmount = R(0.98f);
    vB.ang *= DampingAmount;
    if (conf->doWarmStart) {
        j->imp[0] *= conf->dtRatio; j->imp[1] *= conf->dtRatio;
        const v2 P = V(j->imp[0], j->imp[1]);
        add_imp(&vB, iM, P, iI, cross(j->rB, P));
    } else {
        j->imp[0] = j->imp[1] = R(0);
    }
    B->vel = vB;
}
static int tj_solve_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* B = &bcs[j->bB];
    pos_t vB = B->vel;
    const v2 Cdot = point_vel(vB, j->rB);
    const v2 ev = vadd(Cdot, vadd(j->linErr, vmul(V(j->imp[0], j->imp[1]), j->gamma)));
    const v2 oldImpulse = V(j->imp[0], j->imp[1]);
    const v2 addImpulse = mat22_mul(j->lm, vneg(ev));
    v2 impulse = vadd(oldImpulse, addImpulse);
    const real maxImpulse = conf->deltaTime * j->extra[2];
    if (mag2(impulse) > maxImpulse * maxImpulse) impulse = vmul(unit_vector(impulse, V(R(0), R(0))), maxImpulse);
    j->imp[0] = impulse.x; j->imp[1] = impulse.y;
    const v2 inc = vsub(impulse, oldImpulse);
    add_imp(&vB, B->invM, inc, B->invI, cross(j->rB, inc));
    B->vel = vB;
    return inc.x == R(0) && inc.y == R(0);
}

/* Joint dispatch (JointConf visitors, Joint.cpp). */
/* GearJointConf InitVelocity / SolveVelocity / SolvePosition
 * (GearJointConf.cpp:170-261, :263-300, :302-474). */
static void gear_init_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    bc_t* C = &bcs[j->bC];
    bc_t* D = &bcs[j->bD];
    pos_t velA = A->vel, velB = B->vel, velC = C->vel, velD = D->vel;
    real invMass = R(0);
    if (j->gAC == 1) {
        const v2 qA = unit_from_angle(A->pos.ang), qC = unit_from_angle(C->pos.ang);
        const v2 u = rotate(j->gAxAC, qC);
        const v2 rC = rotate(vsub(j->gLaAC, C->lc), qC);
        const v2 rA = rotate(vsub(j->gLbAC, A->lc), qA);
        j->JvAC = vmul(u, R(1));
        j->JwC = cross(rC, u);
        j->JwA = cross(rA, u);
        const real invRotMassC = C->invI * (j->JwC * j->JwC);
        const real invRotMassA = A->invI * (j->JwA * j->JwA);
        const real invLinMass = ((C->invM + A->invM) + invRotMassC) + invRotMassA;
        invMass += invLinMass;
    } else {
        j->JvAC = V(R(0), R(0));
        j->JwA = R(1);
        j->JwC = R(1);
        invMass += A->invI + C->invI;
    }
    if (j->gBD == 1) {
        const v2 qB = unit_from_angle(B->pos.ang), qD = unit_from_angle(D->pos.ang);
        const v2 u = rotate(j->gAxBD, qD);
        const v2 rD = rotate(vsub(j->gLaBD, D->lc), qD);
        const v2 rB = rotate(vsub(j->gLbBD, B->lc), qB);
        j->JvBD = vmul(u, j->ratio);
        j->JwD = j->ratio * cross(rD, u);
        j->JwB = j->ratio * cross(rB, u);
        const real invRotMassD = D->invI * (j->JwD * j->JwD);
        const real invRotMassB = B->invI * (j->JwB * j->JwB);
        const real invLinMass = ((j->ratio * j->ratio) * (D->invM + B->invM) + invRotMassD) + invRotMassB;
        invMass += invLinMass;
    } else {
        j->JvBD = V(R(0), R(0));
        j->JwB = j->ratio;
        j->JwD = j->ratio;
        invMass += (j->ratio * j->ratio) * (B->invI + D->invI);
    }
    j->gmass = (invMass > R(0)) ? R(1) / invMass : R(0);
    if (conf->doWarmStart) {
        const real imp = j->gimp;
        velA.lin = vadd(velA.lin, vmul(j->JvAC, A->invM * imp)); velA.ang = velA.ang + (A->invI * imp) * j->JwA;
        velB.lin = vadd(velB.lin, vmul(j->JvBD, B->invM * imp)); velB.ang = velB.ang + (B->invI * imp) * j->JwB;
        velC.lin = vsub(velC.lin, vmul(j->JvAC, C->invM * imp)); velC.ang = velC.ang - (C->invI * imp) * j->JwC;
        velD.lin = vsub(velD.lin, vmul(j->JvBD, D->invM * imp)); velD.ang = velD.ang - (D->invI * imp) * j->JwD;
    } else {
        j->gimp = R(0);
    }
    A->vel = velA; B->vel = velB; C->vel = velC; D->vel = velD;
}

static int gear_solve_velocity(joint_t* j, bc_t* bcs) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    bc_t* C = &bcs[j->bC];
    bc_t* D = &bcs[j->bD];
    pos_t velA = A->vel, velB = B->vel, velC = C->vel, velD = D->vel;
    const real acDot = dot(j->JvAC, vsub(velA.lin, velC.lin));
    const real bdDot = dot(j->JvBD, vsub(velB.lin, velD.lin));
    const real Cdot = ((acDot + bdDot) + (j->JwA * velA.ang - j->JwC * velC.ang)) + (j->JwB * velB.ang - j->JwD * velD.ang);
    const real impulse = -j->gmass * Cdot;
    j->gimp += impulse;
    velA.lin = vadd(velA.lin, vmul(j->JvAC, A->invM * impulse)); velA.ang = velA.ang + (A->invI * impulse) * j->JwA;
    velB.lin = vadd(velB.lin, vmul(j->JvBD, B->invM * impulse)); velB.ang = velB.ang + (B->invI * impulse) * j->JwB;
    velC.lin = vsub(velC.lin, vmul(j->JvAC, C->invM * impulse)); velC.ang = velC.ang - (C->invI * impulse) * j->JwC;
    velD.lin = vsub(velD.lin, vmul(j->JvBD, D->invM * impulse)); velD.ang = velD.ang - (D->invI * impulse) * j->JwD;
    A->vel = velA; B->vel = velB; C->vel = velC; D->vel = velD;
    return impulse == R(0);
}

/* Cap(Position, ConstraintSolverConf) (d2/Math.cpp:63-71). */
static pos_t cap_position(pos_t p, const or_stepconf* conf) {
    const real lsq = mag2(p.lin);
    if (lsq > conf->maxLinearCorrection * conf->maxLinearCorrection) p.lin = vmul(p.lin, conf->maxLinearCorrection / RSQRT(lsq));
    p.ang = clampr(p.ang, -conf->maxAngularCorrection, conf->maxAngularCorrection);
    return p;
}

static int gear_solve_position(const joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    bc_t* A = &bcs[j->bA];
    bc_t* B = &bcs[j->bB];
    bc_t* C = &bcs[j->bC];
    bc_t* D = &bcs[j->bD];
    const pos_t posA = A->pos, posB = B->pos, posC = C->pos, posD = D->pos;
    if (!isfinite(j->constant)) return 1;
    v2 JvAC = V(R(0), R(0)), JvBD = V(R(0), R(0));
    real JwA = R(0), JwB = R(0), JwC = R(0), JwD = R(0), coordA = R(0), coordB = R(0), invMass = R(0);
    if (j->gAC == 1) {
        const v2 qA = unit_from_angle(posA.ang), qC = unit_from_angle(posC.ang);
        const v2 u = rotate(j->gAxAC, qC);
        const v2 rC = rotate(vsub(j->gLaAC, C->lc), qC);
        const v2 rA = rotate(vsub(j->gLbAC, A->lc), qA);
        JvAC = vmul(u, R(1));
        JwC = cross(rC, u);
        JwA = cross(rA, u);
        const real invLinMass = C->invM + A->invM;
        const real invRotMassC = C->invI * (JwC * JwC);
        const real invRotMassA = A->invI * (JwA * JwA);
        invMass += (invLinMass + invRotMassC) + invRotMassA;
        const v2 pC = vsub(j->gLaAC, C->lc);
        const v2 pA = invrotate(vadd(rA, vsub(posA.lin, posC.lin)), qC);
        coordA = dot(vsub(pA, pC), j->gAxAC);
    } else {
        JwA = R(1);
        JwC = R(1);
        invMass += A->invI + C->invI;
        coordA = (posA.ang - posC.ang) - j->gRefAC;
    }
    if (j->gBD == 1) {
        const v2 qB = unit_from_angle(posB.ang), qD = unit_from_angle(posD.ang);
        const v2 u = rotate(j->gAxBD, qD);
        const v2 rD = rotate(vsub(j->gLaBD, D->lc), qD);
        const v2 rB = rotate(vsub(j->gLbBD, B->lc), qB);
        JvBD = vmul(u, j->ratio);
        JwD = j->ratio * cross(rD, u);
        JwB = j->ratio * cross(rB, u);
        const real invLinMass = (j->ratio * j->ratio) * (D->invM + B->invM);
        const real invRotMassD = D->invI * (JwD * JwD);
        const real invRotMassB = B->invI * (JwB * JwB);
        invMass += (invLinMass + invRotMassD) + invRotMassB;
        const v2 pD = vsub(j->gLaBD, D->lc);
        const v2 pB = invrotate(vadd(rB, vsub(posB.lin, posD.lin)), qD);
        coordB = dot(vsub(pB, pD), j->gAxBD);
    } else {
        JwB = j->ratio;
        JwD = j->ratio;
        invMass += (j->ratio * j->ratio) * (B->invI + D->invI);
        coordB = (posB.ang - posD.ang) - j->gRefBD;
    }
    const real Cv = ((coordA + j->ratio * coordB) - j->constant) * conf->regResolutionRate;
    const real impulse = (invMass > R(0)) ? -Cv / invMass : R(0);
    pos_t dA, dB, dC, dD;
    dA.lin = vmul(JvAC, A->invM * impulse); dA.ang = (A->invI * impulse) * JwA;
    dC.lin = vmul(JvAC, C->invM * impulse); dC.ang = (C->invI * impulse) * JwC;
    dB.lin = vmul(JvBD, B->invM * impulse); dB.ang = (B->invI * impulse) * JwB;
    dD.lin = vmul(JvBD, D->invM * impulse); dD.ang = (D->invI * impulse) * JwD;
    dA = cap_position(dA, conf); dC = cap_position(dC, conf);
    dB = cap_position(dB, conf); dD = cap_position(dD, conf);
    A->pos.lin = vadd(posA.lin, dA.lin); A->pos.ang = posA.ang + dA.ang;
    B->pos.lin = vadd(posB.lin, dB.lin); B->pos.ang = posB.ang + dB.ang;
    C->pos.lin = vsub(posC.lin, dC.lin); C->pos.ang = posC.ang - dC.ang;
    D->pos.lin = vsub(posD.lin, dD.lin); D->pos.ang = posD.ang - dD.ang;
    real lin = R(0), ang = R(0);
    lin = maxr(lin, mag2(dA.lin)); lin = maxr(lin, mag2(dB.lin)); lin = maxr(lin, mag2(dC.lin)); lin = maxr(lin, mag2(dD.lin));
    ang = maxr(ang, fabs(dA.ang)); ang = maxr(ang, fabs(dB.ang)); ang = maxr(ang, fabs(dC.ang)); ang = maxr(ang, fabs(dD.ang));
    return (lin <= conf->linearSlop * conf->linearSlop) && (ang <= conf->angularSlop);
}

static void joint_init_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    switch (j->type) {
    case OR_JOINT_DISTANCE: dj_init_velocity(j, bcs, conf); break;
    case OR_JOINT_ROPE: rope_init_velocity(j, bcs, conf); break;
    case OR_JOINT_WELD: weld_init_velocity(j, bcs, conf); break;
    case OR_JOINT_FRICTION: fm_init_velocity(j, bcs, conf, 0); break;
    case OR_JOINT_MOTOR: fm_init_velocity(j, bcs, conf, 1); break;
    case OR_JOINT_PRISMATIC: pj_init_velocity(j, bcs, conf); break;
    case OR_JOINT_WHEEL: wj_init_velocity(j, bcs, conf); break;
    case OR_JOINT_PULLEY: pu_init_velocity(j, bcs, conf); break;
    case OR_JOINT_TARGET: tj_init_velocity(j, bcs, conf); break;
    case OR_JOINT_GEAR: gear_init_velocity(j, bcs, conf); break;
    default: rj_init_velocity(j, bcs, conf); break;
    }
}
static int joint_solve_velocity(joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    switch (j->type) {
    case OR_JOINT_DISTANCE: return dj_solve_velocity(j, bcs);
    case OR_JOINT_ROPE: return rope_solve_velocity(j, bcs, conf);
    case OR_JOINT_WELD: return weld_solve_velocity(j, bcs);
    case OR_JOINT_FRICTION: return friction_solve_velocity(j, bcs, conf);
    case OR_JOINT_MOTOR: return motor_solve_velocity(j, bcs, conf);
    case OR_JOINT_PRISMATIC: return pj_solve_velocity(j, bcs, conf);
    case OR_JOINT_WHEEL: return wj_solve_velocity(j, bcs, conf);
    case OR_JOINT_PULLEY: return pu_solve_velocity(j, bcs);
    case OR_JOINT_TARGET: return tj_solve_velocity(j, bcs, conf);
    case OR_JOINT_GEAR: return gear_solve_velocity(j, bcs);
    default: return rj_solve_velocity(j, bcs, conf);
    }
}
static int joint_solve_position(const joint_t* j, bc_t* bcs, const or_stepconf* conf) {
    switch (j->type) {
    case OR_JOINT_DISTANCE: return dj_solve_position(j, bcs, conf);
    case OR_JOINT_ROPE: return rope_solve_position(j, bcs, conf);
    case OR_JOINT_WELD: return weld_solve_position(j, bcs, conf);
    case OR_JOINT_FRICTION: case OR_JOINT_MOTOR: case OR_JOINT_TARGET: return 1;
    case OR_JOINT_PRISMATIC: return pj_solve_position(j, bcs, conf);
    case OR_JOINT_WHEEL: return wj_solve_position(j, bcs, conf);
    case OR_JOINT_PULLEY: return pu_solve_position(j, bcs, conf);
    case OR_JOINT_GEAR: return gear_solve_position(j, bcs, conf);
    default: return rj_solve_position(j, bcs, conf);
    }
}

/* GetBodyConstraint (BodyConstraint.hpp:157-167): position 1 and
 * Cap(GetVelocity(body, h)) (Body.cpp:290-309, Velocity.cpp:26-45). */
static void make_bc(bc_t* bc, const body_t* b, real h, const or_stepconf* conf) {
    bc->invM = b->invM; bc->invI = b->invI; bc->lc = b->lc; bc->pos = b->pos1;
    pos_t v = b->vel;
    if (is_accelerable(b)) {
        v.lin = vadd(v.lin, vmul(b->la, h));
        v.ang = v.ang + h * b->aa;
        v.lin = vdiv(v.lin, R(1) + h * b->ldamp);
        v.ang = v.ang / (R(1) + h * b->adamp);
    }
    {
        const v2 translation = vmul(v.lin, h);
        const real lsq = mag2(translation);
        if (lsq > conf->maxTranslation * conf->maxTranslation) {
            const real ratio = conf->maxTranslation / RSQRT(lsq);
            v.lin = vmul(v.lin, ratio);
        }
        const real absRot = fabs(h * v.ang);
        if (absRot > conf->maxRotation) {
            const real ratio = conf->maxRotation / absRot;
            v.ang = v.ang * ratio;
        }
    }
    bc->vel = v;
}

/* Island constraint order set by or_set_solve_order (test infrastructure). */
typedef struct { int64_t rank; int joint, idx; } ord_item;
static int cmp_ord(const void* a, const void* b) {
    const ord_item* x = (const ord_item*)a;
    const ord_item* y = (const ord_item*)b;
    if (x->rank != y->rank) return (x->rank < y->rank) ? -1 : 1;
    if (x->joint != y->joint) return x->joint - y->joint;
    return x->idx - y->idx;
}
static int64_t contact_rank(const or_world* w, const contact_t* c) {
    const int a = c->sA < c->sB ? c->sA : c->sB, b = c->sA < c->sB ? c->sB : c->sA;
    const int64_t key = ((int64_t)a << 32) | (int64_t)b;
    int lo = 0, hi = w->order_ckeys.n;
    while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if (w->order_ckeys.a[mid] < key) lo = mid + 1; else hi = mid;
    }
    if (lo < w->order_ckeys.n && w->order_ckeys.a[lo] == key) return w->order_crank.a[lo];
    return INT64_MAX / 2; /* not listed: after every listed constraint, in island order */
}
static ord_item* island_order(const or_world* w, const island_t* isl) {
    const int nc = isl->contacts.n, nj = isl->joints.n;
    ord_item* o = (ord_item*)malloc(sizeof(ord_item) * (size_t)(nc + nj + 1));
    for (int i = 0; i < nc; ++i) {
        o[i].rank = contact_rank(w, &w->c[isl->contacts.a[i]]);
        o[i].joint = 0; o[i].idx = i;
    }
    for (int i = 0; i < nj; ++i) {
        const int jid = (int)isl->joints.a[i];
        const int64_t r = (jid < w->order_jrank.n) ? w->order_jrank.a[jid] : -1;
        o[nc + i].rank = (r >= 0) ? r : INT64_MAX / 2;
        o[nc + i].joint = 1; o[nc + i].idx = i;
    }
    qsort(o, (size_t)(nc + nj), sizeof(ord_item), cmp_ord);
    return o;
}

static void solve_island(or_world* w, const or_stepconf* conf, island_t* isl, bc_t* bcs,
                         or_stepstats* st) {
    const real h = conf->deltaTime;
    /* pos0 <- pos1 (:1574-1580) */
    for (int i = 0; i < isl->bodies.n; ++i) {
        body_t* b = &w->b[isl->bodies.a[i]];
        b->pos0 = b->pos1;
    }
    for (int i = 0; i < isl->bodies.n; ++i) {
        const int id = (int)isl->bodies.a[i];
        make_bc(&bcs[id], &w->b[id], h, conf);
    }
    const int nc = isl->contacts.n;
    pc_t* pcs = (pc_t*)malloc(sizeof(pc_t) * (size_t)(nc + 1));
    vc_t* vcs = (vc_t*)malloc(sizeof(vc_t) * (size_t)(nc + 1));
    for (int i = 0; i < nc; ++i) {
        const contact_t* c = &w->c[isl->contacts.a[i]];
        const real rA = w->s[c->sA].dp.r, rB = w->s[c->sB].dp.r;
        pcs[i].m = &c->m; pcs[i].bA = c->bA; pcs[i].bB = c->bB; pcs[i].totalRadius = rA + rB;
    }
    for (int i = 0; i < nc; ++i) {
        const contact_t* c = &w->c[isl->contacts.a[i]];
        const bc_t* A = &bcs[c->bA];
        const bc_t* B = &bcs[c->bB];
        const real rA = w->s[c->sA].dp.r, rB = w->s[c->sB].dp.r;
        const xf_t xfA = get_xf(A->pos, A->lc), xfB = get_xf(B->pos, B->lc);
        const wman_t wm = world_manifold(&c->m, xfA, rA, xfB, rB);
        make_vc(&vcs[i], c, &wm, bcs, conf);
    }
    /* With a solve order set (or_set_solve_order), every pass visits the island's
     * contacts and joints interleaved in that order instead of the reference's
     * (contacts in island order, joints before contacts in each iteration). */
    const int nj = isl->joints.n;
    ord_item* ord = (w->order_crank.n || w->order_jrank.n) ? island_order(w, isl) : NULL;
    if (ord) {
        for (int q = 0; q < nc + nj; ++q) {
            if (ord[q].joint) joint_init_velocity(&w->j[isl->joints.a[ord[q].idx]], bcs, conf);
            else if (conf->doWarmStart) warm_start(&vcs[ord[q].idx], bcs);
        }
    } else {
        if (conf->doWarmStart) {
            for (int i = 0; i < nc; ++i) warm_start(&vcs[i], bcs);
        }
        for (int i = 0; i < nj; ++i) joint_init_velocity(&w->j[isl->joints.a[i]], bcs, conf);
    }

    int velIters = conf->regVelocityIters;
    real maxInc = R(0);
    for (int it = 0; it < conf->regVelocityIters; ++it) {
        int jointsOkay = 1;
        real newInc = R(0);
        if (ord) {
            for (int q = 0; q < nc + nj; ++q) {
                if (ord[q].joint) jointsOkay &= joint_solve_velocity(&w->j[isl->joints.a[ord[q].idx]], bcs, conf);
                else newInc = maxr(newInc, solve_vc(&vcs[ord[q].idx], bcs));
            }
        } else {
            for (int i = 0; i < nj; ++i) jointsOkay &= joint_solve_velocity(&w->j[isl->joints.a[i]], bcs, conf);
            for (int i = 0; i < nc; ++i) newInc = maxr(newInc, solve_vc(&vcs[i], bcs));
        }
        maxInc = maxr(maxInc, newInc);
        if (jointsOkay && (newInc <= conf->regMinMomentum)) { velIters = it + 1; break; }
    }
    /* IntegratePositions (:176-188) */
    for (int i = 0; i < isl->bodies.n; ++i) {
        bc_t* bc = &bcs[isl->bodies.a[i]];
        const v2 tr = vmul(bc->vel.lin, h);
        const real rot = h * bc->vel.ang;
        bc->pos.lin = vadd(bc->pos.lin, tr);
        bc->pos.ang = bc->pos.ang + rot;
    }
    int solved = 0, posIters = conf->regPositionIters;
    real minSepIsland = RINF;
    for (int it = 0; it < conf->regPositionIters; ++it) {
        real minSep = RINF;
        int jointsOkay = 1;
        if (ord) {
            for (int q = 0; q < nc + nj; ++q) {
                if (ord[q].joint) jointsOkay &= joint_solve_position(&w->j[isl->joints.a[ord[q].idx]], bcs, conf);
                else minSep = minr(minSep, solve_pc(&pcs[ord[q].idx], bcs, conf));
            }
        } else {
            for (int i = 0; i < nc; ++i) minSep = minr(minSep, solve_pc(&pcs[i], bcs, conf));
        }
        minSepIsland = minr(minSepIsland, minSep);
        const int contactsOkay = (minSep >= conf->regMinSeparation);
        if (!ord) {
            for (int i = 0; i < nj; ++i) jointsOkay &= joint_solve_position(&w->j[isl->joints.a[i]], bcs, conf);
        }
        if (contactsOkay && jointsOkay) { posIters = it + 1; solved = 1; break; }
    }
    free(ord);
    /* AssignImpulses (:196-220) */
    for (int i = 0; i < nc; ++i) {
        contact_t* c = &w->c[isl->contacts.a[i]];
        for (int k = 0; k < vcs[i].count; ++k) { c->m.p[k].ni = vcs[i].p[k].ni; c->m.p[k].ti = vcs[i].p[k].ti; }
    }
    /* Report to PostSolveContact after the write-back (:1669-1672) */
    const int post_iter = solved ? posIters - 1 : 255;  /* StepConf::InvalidIteration */
    /* write back (:1652-1664) */
    for (int i = 0; i < isl->bodies.n; ++i) {
        const int id = (int)isl->bodies.a[i];
        body_t* b = &w->b[id];
        const bc_t* bc = &bcs[id];
        b->vel = bc->vel;
        if (b->pos1.lin.x != bc->pos.lin.x || b->pos1.lin.y != bc->pos.lin.y || b->pos1.ang != bc->pos.ang) {
            body_set_pos1(b, bc->pos);
            for (int k = 0; k < b->cids.n; ++k) w->c[b->cids.a[k]].needsUpdate = 1;
        }
    }
    for (int i = 0; i < nc; ++i) {
        const real ni[2] = {vcs[i].p[0].ni, vcs[i].p[1].ni}, ti[2] = {vcs[i].p[0].ti, vcs[i].p[1].ti};
        record_solve_call(w, 4, &w->c[isl->contacts.a[i]], vcs[i].count, post_iter, ni, ti);
    }
    /* UpdateUnderActiveTimes + Sleepem (:403-429) */
    real minUat = RINF;
    for (int i = 0; i < isl->bodies.n; ++i) {
        body_t* b = &w->b[isl->bodies.a[i]];
        if (is_speedable(b)) {
            const real lin2 = mag2(b->vel.lin);
            const real ang2 = b->vel.ang * b->vel.ang;
            const int under = (ang2 <= conf->angularSleepTolerance * conf->angularSleepTolerance) &&
                              (lin2 <= conf->linearSleepTolerance * conf->linearSleepTolerance);
            const int sleepable = (b->flags & BF_ALLOW_SLEEP) != 0;
            const real t = (sleepable && under) ? b->uat + conf->deltaTime : R(0);
            b->uat = t;
            minUat = minr(minUat, t);
        }
    }
    if ((minUat >= conf->minStillTimeToSleep) && solved) {
        for (int i = 0; i < isl->bodies.n; ++i) st->regBodiesSlept += body_unawaken(&w->b[isl->bodies.a[i]]);
    }
    if (solved) st->regIslandsSolved++;
    st->regSumPosIters += posIters;
    st->regSumVelIters += velIters;
    st->regMinSeparation = minr(st->regMinSeparation, minSepIsland);
    st->regMaxIncImpulse = maxr(st->regMaxIncImpulse, maxInc);
    free(pcs); free(vcs);
}

/* SolveReg (AabbTreeWorld.cpp:1472-1561) with AddToIsland (:1358-1470). */
static void solve_reg(or_world* w, const or_stepconf* conf, or_stepstats* st) {
    unsigned char* ib = (unsigned char*)calloc((size_t)w->nb + 1, 1);
    unsigned char* ic = (unsigned char*)calloc((size_t)w->nc + 1, 1);
    unsigned char* ij = (unsigned char*)calloc((size_t)w->nj + 1, 1);
    bc_t* bcs = (bc_t*)calloc((size_t)w->nb + 1, sizeof(bc_t));
    int* stack = (int*)malloc(sizeof(int) * (size_t)(w->nb + 1));
    island_t isl;
    memset(&isl, 0, sizeof(isl));
    for (int seed = 0; seed < w->nb; ++seed) {
        body_t* sb = &w->b[seed];
        if (ib[seed]) continue;
        if (!((sb->flags & BF_AWAKE) && (sb->flags & BF_ENABLED))) continue;
        st->regIslandsFound++;
        isl.bodies.n = isl.contacts.n = isl.joints.n = 0;
        int sp = 0;
        stack[sp++] = seed;
        ib[seed] = 1;
        while (sp) {
            const int id = stack[--sp];
            body_t* b = &w->b[id];
            iv_push(&isl.bodies, id);
            if (!is_speedable(b)) continue;
            b->flags |= BF_AWAKE;
            for (int k = 0; k < b->cids.n; ++k) {
                const int cid = (int)b->cids.a[k];
                if (ic[cid]) continue;
                const contact_t* c = &w->c[cid];
                if (c->touching && !c->sensor) {
                    const int other = (c->bA == id) ? c->bB : c->bA;
                    iv_push(&isl.contacts, cid);
                    ic[cid] = 1;
                    if (!ib[other]) { ib[other] = 1; stack[sp++] = other; }
                }
            }
            for (int k = 0; k < b->jids.n; ++k) {
                const int jid = (int)b->jids.a[k];
                if (ij[jid]) continue;
                const int other = (int)b->jother.a[k];
                if (w->b[other].flags & BF_ENABLED) {
                    ij[jid] = 1;
                    iv_push(&isl.joints, jid);
                    if (!ib[other]) { ib[other] = 1; stack[sp++] = other; }
                }
            }
        }
        for (int i = 0; i < isl.bodies.n; ++i) {
            const int id = (int)isl.bodies.a[i];
            if (!is_speedable(&w->b[id])) ib[id] = 0;
        }
        solve_island(w, conf, &isl, bcs, st);
    }
    for (int id = 0; id < w->nb; ++id) {
        if (ib[id] && is_speedable(&w->b[id])) st->regProxiesMoved += synchronize(w, id, conf);
    }
    st->regContactsUpdated += update_contacts(w, conf);
    st->regContactsAdded += find_and_add_contacts(w, conf);
    iv_free(&isl.bodies); iv_free(&isl.contacts); iv_free(&isl.joints);
    free(ib); free(ic); free(ij); free(bcs); free(stack);
}

/* ------------------------------------------------------------------------- */
/* Time of impact: Distance (GJK), separation scenarios, GetToiViaSat, and the */
/* TOI phase of the step (StepConf::doToi).                                   */
/* ------------------------------------------------------------------------- */
/* Position arithmetic (d2/Position.hpp) and GetPosition (d2/Math.cpp:30-60):
 * pos0 + (pos1 - pos0) * beta. */
static pos_t plerp(pos_t p0, pos_t p1, real beta) {
    pos_t d, s;
    d.lin = vsub(p1.lin, p0.lin); d.ang = p1.ang - p0.ang;
    s.lin = vmul(d.lin, beta); s.ang = d.ang * beta;
    return padd(p0, s);
}

/* Sweep (d2/Sweep.hpp:43-92). */
typedef struct { pos_t p0, p1; v2 lc; real a0; } sweep_t;
static sweep_t body_sweep(const body_t* b) { sweep_t s; s.p0 = b->pos0; s.p1 = b->pos1; s.lc = b->lc; s.a0 = b->alpha0; return s; }
/* Body::SetSweep (Body.hpp:697-702). */
static void body_set_sweep(body_t* b, sweep_t s) { b->pos0 = s.p0; b->pos1 = s.p1; b->lc = s.lc; b->alpha0 = s.a0; b->xf = get_xf(s.p1, s.lc); }
/* GetTransformation(sweep, beta) (d2/Math.hpp:251-254). */
static inline xf_t sweep_xf(const sweep_t* s, real beta) { return get_xf(plerp(s->p0, s->p1, beta), s->lc); }
/* Advance0 (Sweep.cpp:27-31) on a body (Body.hpp:722-730). */
static void body_advance0(body_t* b, real alpha) {
    const real beta = (alpha - b->alpha0) / (R(1) - b->alpha0);
    b->pos0 = plerp(b->pos0, b->pos1, beta);
    b->alpha0 = alpha;
}
/* Advance (Body.hpp:1004-1009): Advance0 then position 1 = position 0. */
static void body_advance(body_t* b, real alpha) { body_advance0(b, alpha); body_set_pos1(b, b->pos0); }
/* GetNormalized(Angle) (Math.cpp:33-91, default branch). */
static real angle_normalized(real a) {
    const real Pi = R(3.14159265358979323846264338327950288L);
    const real twoPi = R(2) * Pi;
    const real rTwoPi = R(1) / twoPi;
#ifdef OR_DOUBLE
    a = a - trunc(a * rTwoPi) * twoPi;
#else
    a = a - truncf(a * rTwoPi) * twoPi;
#endif
    if (a >= Pi) a -= Pi * R(2);
    else if (a < -Pi) a += Pi * R(2);
    return a;
}
/* GetNormalized(Sweep) (d2/Math.hpp:160-167). */
static sweep_t sweep_normalized(sweep_t s) {
    const real a0 = angle_normalized(s.p0.ang);
    const real d = s.p0.ang - a0;
    s.p0.ang = a0;
    s.p1.ang -= d;
    return s;
}

/* SimplexEdge (SimplexEdge.hpp:40-87) and Simplex (Simplex.cpp). */
typedef struct { v2 pA; int iA; v2 pB; int iB; } sedge;
typedef struct { int n; sedge e[3]; real c[3]; } simplex_t;
typedef struct { int n; int ia[3], ib[3]; real metric; } scache; /* Simplex::Cache */

static inline sedge make_sedge(const dproxy* A, xf_t xfA, int ia, const dproxy* B, xf_t xfB, int ib) {
    sedge e;
    e.pA = xform(A->v[ia], xfA); e.iA = ia;
    e.pB = xform(B->v[ib], xfB); e.iB = ib;
    return e;
}
static inline v2 sdelta(const sedge* e) { return vsub(e->pB, e->pA); }

static simplex_t simplex1(sedge s0) { simplex_t r; memset(&r, 0, sizeof(r)); r.n = 1; r.e[0] = s0; r.c[0] = R(1); return r; }
static simplex_t simplex2(sedge s0, sedge s1, real c0, real c1) {
    simplex_t r; memset(&r, 0, sizeof(r)); r.n = 2; r.e[0] = s0; r.e[1] = s1; r.c[0] = c0; r.c[1] = c1; return r;
}
/* Simplex::Get (Simplex.cpp:55-169). */
static simplex_t simplex_get(const sedge* s, int n) {
    if (n == 1) return simplex1(s[0]);
    if (n == 2) {
        const v2 w1 = sdelta(&s[0]), w2 = sdelta(&s[1]);
        const v2 e12 = vsub(w2, w1);
        const real d12_2 = -dot(w1, e12);
        if (d12_2 <= R(0)) return simplex1(s[0]);
        const real d12_1 = dot(w2, e12);
        if (d12_1 <= R(0)) return simplex1(s[1]);
        const real inv_sum = R(1) / (d12_1 + d12_2);
        return simplex2(s[0], s[1], d12_1 * inv_sum, d12_2 * inv_sum);
    }
    const v2 w1 = sdelta(&s[0]), w2 = sdelta(&s[1]), w3 = sdelta(&s[2]);
    const v2 e12 = vsub(w2, w1);
    const real d12_1 = dot(w2, e12);
    const real d12_2 = -dot(w1, e12);
    const v2 e13 = vsub(w3, w1);
    const real d13_1 = dot(w3, e13);
    const real d13_2 = -dot(w1, e13);
    const v2 e23 = vsub(w3, w2);
    const real d23_1 = dot(w3, e23);
    const real d23_2 = -dot(w2, e23);
    if ((d12_2 <= R(0)) && (d13_2 <= R(0))) return simplex1(s[0]);
    if ((d12_1 <= R(0)) && (d23_2 <= R(0))) return simplex1(s[1]);
    if ((d13_1 <= R(0)) && (d23_1 <= R(0))) return simplex1(s[2]);
    const real n123 = cross(e12, e13);
    const real d123_3 = n123 * cross(w1, w2);
    if ((d12_1 > R(0)) && (d12_2 > R(0)) && (d123_3 <= R(0))) {
        const real inv_sum = R(1) / (d12_1 + d12_2);
        return simplex2(s[0], s[1], d12_1 * inv_sum, d12_2 * inv_sum);
    }
    const real d123_2 = n123 * cross(w3, w1);
    if ((d13_1 > R(0)) && (d13_2 > R(0)) && (d123_2 <= R(0))) {
        const real inv_sum = R(1) / (d13_1 + d13_2);
        return simplex2(s[0], s[2], d13_1 * inv_sum, d13_2 * inv_sum);
    }
    const real d123_1 = n123 * cross(w2, w3);
    if ((d23_1 > R(0)) && (d23_2 > R(0)) && (d123_1 <= R(0))) {
        const real inv_sum = R(1) / (d23_1 + d23_2);
        return simplex2(s[2], s[1], d23_2 * inv_sum, d23_1 * inv_sum);
    }
    const real inv_sum = R(1) / (d123_1 + d123_2 + d123_3);
    simplex_t r;
    memset(&r, 0, sizeof(r));
    r.n = 3; r.e[0] = s[0]; r.e[1] = s[1]; r.e[2] = s[2];
    r.c[0] = d123_1 * inv_sum; r.c[1] = d123_2 * inv_sum; r.c[2] = d123_3 * inv_sum;
    return r;
}
/* Simplex::CalcMetric (Simplex.cpp:171-192). */
static real simplex_metric(const sedge* s, int n) {
    if (n == 2) return RSQRT(mag2(vsub(sdelta(&s[1]), sdelta(&s[0]))));
    if (n == 3) return cross(vsub(sdelta(&s[1]), sdelta(&s[0])), vsub(sdelta(&s[2]), sdelta(&s[0])));
    return R(0);
}
/* CalcSearchDirection (Simplex.cpp:37-53). */
static v2 search_direction(const sedge* s, int n) {
    if (n == 1) return vneg(sdelta(&s[0]));
    if (n == 2) {
        const v2 e12 = vsub(sdelta(&s[1]), sdelta(&s[0]));
        const v2 e0 = sdelta(&s[0]);
        const real sgn = cross(e12, vneg(e0));
        return (sgn > R(0)) ? revperp(e12) : fwdperp(e12);
    }
    return V(R(0), R(0));
}
/* GetSupportIndex (DistanceProxy.hpp:233-249). */
static int support_index(const dproxy* p, v2 dir) {
    int index = 255;
    real maxValue = -RINF;
    for (int i = 0; i < p->count; ++i) {
        const real value = dot(p->v[i], dir);
        if (maxValue < value) { maxValue = value; index = i; }
    }
    return index;
}

enum { DIST_HITMAX = 1, DIST_MAXPOINTS = 2, DIST_UNFIT = 3, DIST_DUPLICATE = 4 };
typedef struct { simplex_t s; int iters, state; } dist_out;
/* Distance (Distance.cpp:96-196) with the cache of the previous call. */
static dist_out gjk_distance(const dproxy* A, xf_t xfA, const dproxy* B, xf_t xfB, const scache* cache,
                             int maxIters) {
    int sa[3], sb[3], sn = cache->n;
    sedge edges[3];
    int ne = cache->n;
    for (int k = 0; k < sn; ++k) {
        sa[k] = cache->ia[k]; sb[k] = cache->ib[k];
        edges[k] = make_sedge(A, xfA, sa[k], B, xfB, sb[k]);
    }
    if (ne > 1) {
        const real metric1 = cache->metric;
        const real metric2 = simplex_metric(edges, ne);
        if ((metric2 < (metric1 / R(2))) || (metric2 > (metric1 * R(2))) || (metric2 < R(0)) || almost_zero(metric2)) ne = 0;
    }
    if (ne == 0) {
        edges[0] = make_sedge(A, xfA, 0, B, xfB, 0);
        ne = 1;
        sn = 1; sa[0] = 0; sb[0] = 0;
    }
    dist_out out;
    memset(&out, 0, sizeof(out));
    out.state = DIST_HITMAX;
    int iter = 0;
    while (iter < maxIters) {
        ++iter;
        out.s = simplex_get(edges, ne);
        ne = out.s.n;
        for (int k = 0; k < ne; ++k) edges[k] = out.s.e[k];
        if (ne == 3) { out.state = DIST_MAXPOINTS; break; }
        const v2 d = search_direction(edges, ne);
        if (almost_zero(mag2(d))) { out.state = DIST_UNFIT; break; }
        const int ia = support_index(A, invrotate(vneg(d), xfA.q));
        const int ib = support_index(B, invrotate(d, xfB.q));
        int dup = 0;
        for (int k = 0; k < sn; ++k) if (sa[k] == ia && sb[k] == ib) dup = 1;
        if (dup) { out.state = DIST_DUPLICATE; break; }
        edges[ne++] = make_sedge(A, xfA, ia, B, xfB, ib);
        sn = ne;
        for (int k = 0; k < ne; ++k) { sa[k] = edges[k].iA; sb[k] = edges[k].iB; }
    }
    out.iters = iter;
    return out;
}
/* GetWitnessPoints (Distance.cpp:71-94). */
static void witness_points(const simplex_t* s, v2* pA, v2* pB) {
    v2 a = V(R(0), R(0)), b = V(R(0), R(0));
    for (int i = 0; i < s->n; ++i) {
        a = vadd(a, vmul(s->e[i].pA, s->c[i]));
        b = vadd(b, vmul(s->e[i].pB, s->c[i]));
    }
    *pA = a; *pB = b;
}

/* TestOverlap (Distance.cpp:205-216) >= 0: GJK Distance from an empty cache
 * (GetDistanceConf(StepConf), DistanceConf.cpp:36-41), then the total vertex
 * radius squared less the squared distance of the witness points. */
static int sensor_touching(const dproxy* A, xf_t xfA, const dproxy* B, xf_t xfB, int maxIters) {
    scache cache;
    memset(&cache, 0, sizeof(cache));
    const dist_out di = gjk_distance(A, xfA, B, xfB, &cache, maxIters);
    v2 pa, pb;
    witness_points(&di.s, &pa, &pb);
    const real d2 = mag2(vsub(pb, pa));
    const real tr = A->r + B->r;
    return (tr * tr - d2) >= R(0);
}

/* SeparationScenario (SeparationScenario.cpp). */
enum { SEP_POINTS = 0, SEP_FACE_A = 1, SEP_FACE_B = 2 };
typedef struct { int type; v2 axis; v2 lp; } sepfn;
typedef struct { real dist; int ia, ib; } lenidx;

static sepfn separation_scenario(const scache* c, const dproxy* A, xf_t xfA, const dproxy* B, xf_t xfB) {
    sepfn f;
    memset(&f, 0, sizeof(f));
    const int type = (c->n < 2) ? SEP_POINTS : ((c->ia[0] == c->ia[1]) ? SEP_FACE_B : SEP_FACE_A);
    if (type == SEP_FACE_B) {
        const v2 lB1 = B->v[c->ib[0]], lB2 = B->v[c->ib[1]];
        const v2 axis = unit_vector(fwdperp(vsub(lB2, lB1)), V(R(0), R(0)));
        const v2 normal = urotate(axis, xfB.q);
        const v2 lp = vdiv(vadd(lB1, lB2), R(2));
        const v2 pB = xform(lp, xfB);
        const v2 pA = xform(A->v[c->ia[0]], xfA);
        f.type = SEP_FACE_B; f.lp = lp;
        f.axis = (dot(vsub(pA, pB), normal) < R(0)) ? vneg(axis) : axis;
        return f;
    }
    if (type == SEP_FACE_A) {
        const v2 lA1 = A->v[c->ia[0]], lA2 = A->v[c->ia[1]];
        const v2 axis = unit_vector(fwdperp(vsub(lA2, lA1)), V(R(0), R(0)));
        const v2 normal = urotate(axis, xfA.q);
        const v2 lp = vdiv(vadd(lA1, lA2), R(2));
        const v2 pA = xform(lp, xfA);
        const v2 pB = xform(B->v[c->ib[0]], xfB);
        f.type = SEP_FACE_A; f.lp = lp;
        f.axis = (dot(vsub(pB, pA), normal) < R(0)) ? vneg(axis) : axis;
        return f;
    }
    const v2 pA = xform(A->v[c->ia[0]], xfA);
    const v2 pB = xform(B->v[c->ib[0]], xfB);
    f.type = SEP_POINTS;
    f.axis = unit_vector(vsub(pB, pA), V(R(0), R(0)));
    return f;
}
/* FindMinSeparation (SeparationScenario.cpp:29-77). */
static lenidx find_min_separation(const sepfn* f, const dproxy* A, xf_t xfA, const dproxy* B, xf_t xfB) {
    lenidx r;
    if (f->type == SEP_POINTS) {
        const v2 dirA = invrotate(f->axis, xfA.q);
        const v2 dirB = invrotate(vneg(f->axis), xfB.q);
        r.ia = support_index(A, dirA);
        r.ib = support_index(B, dirB);
        const v2 delta = vsub(xform(B->v[r.ib], xfB), xform(A->v[r.ia], xfA));
        r.dist = dot(delta, f->axis);
    } else if (f->type == SEP_FACE_A) {
        const v2 normal = urotate(f->axis, xfA.q);
        const v2 pA = xform(f->lp, xfA);
        r.ia = 255;
        r.ib = support_index(B, invrotate(vneg(normal), xfB.q));
        const v2 delta = vsub(xform(B->v[r.ib], xfB), pA);
        r.dist = dot(delta, normal);
    } else {
        const v2 normal = urotate(f->axis, xfB.q);
        r.ia = support_index(A, invrotate(vneg(normal), xfA.q));
        r.ib = 255;
        const v2 pB = xform(f->lp, xfB);
        const v2 delta = vsub(xform(A->v[r.ia], xfA), pB);
        r.dist = dot(delta, normal);
    }
    return r;
}
/* Evaluate (SeparationScenario.cpp:79-119). */
static real sep_evaluate(const sepfn* f, const dproxy* A, xf_t xfA, const dproxy* B, xf_t xfB, int ia, int ib) {
    if (f->type == SEP_POINTS) {
        const v2 delta = vsub(xform(B->v[ib], xfB), xform(A->v[ia], xfA));
        return dot(delta, f->axis);
    }
    if (f->type == SEP_FACE_A) {
        const v2 normal = urotate(f->axis, xfA.q);
        const v2 pA = xform(f->lp, xfA);
        const v2 delta = vsub(xform(B->v[ib], xfB), pA);
        return dot(delta, normal);
    }
    const v2 normal = urotate(f->axis, xfB.q);
    const v2 pB = xform(f->lp, xfB);
    const v2 delta = vsub(xform(A->v[ia], xfA), pB);
    return dot(delta, normal);
}

/* ToiOutput::State (ToiOutput.hpp). */
enum {
    TOI_UNKNOWN = 0, TOI_OVERLAPPED, TOI_TOUCHING, TOI_SEPARATED, TOI_MAX_ROOT_ITERS, TOI_NEXT_AFTER,
    TOI_MAX_TOI_ITERS, TOI_BELOW_MIN_TARGET, TOI_MAX_DIST_ITERS, TOI_TARGET_DEPTH_EXCEEDS_TOTAL_RADIUS,
    TOI_MIN_TARGET_SQUARED_OVERFLOW, TOI_MAX_TARGET_SQUARED_OVERFLOW, TOI_NOT_FINITE
};
typedef struct { real time; int state, toi_iters, max_dist_iters, max_root_iters; } toi_out;

/* GetToiViaSat (TimeOfImpact.cpp:37-253). */
static toi_out toi_via_sat(const dproxy* A, const sweep_t* sA, const dproxy* B, const sweep_t* sB,
                           const or_stepconf* conf) {
    toi_out o;
    memset(&o, 0, sizeof(o));
    const real totalRadius = A->r + B->r;
    if (conf->targetDepth > totalRadius) { o.state = TOI_TARGET_DEPTH_EXCEEDS_TOTAL_RADIUS; return o; }
    const real target = totalRadius - conf->targetDepth;
    const real maxTarget = maxr(target + conf->tolerance, R(0));
    const real minTarget = maxr(target - conf->tolerance, R(0));
    const real minTargetSquared = minTarget * minTarget;
    if (!isfinite(minTargetSquared) && isfinite(minTarget)) { o.state = TOI_MIN_TARGET_SQUARED_OVERFLOW; return o; }
    const real maxTargetSquared = maxTarget * maxTarget;
    if (!isfinite(maxTargetSquared) && isfinite(maxTarget)) { o.state = TOI_MAX_TARGET_SQUARED_OVERFLOW; return o; }
    real timeLo = R(0);
    xf_t loA = sweep_xf(sA, timeLo), loB = sweep_xf(sB, timeLo);
    scache cache;
    memset(&cache, 0, sizeof(cache));
    while (o.toi_iters < conf->maxToiIters) {
        const dist_out di = gjk_distance(A, loA, B, loB, &cache, conf->maxDistanceIters);
        ++o.toi_iters;
        if (di.iters > o.max_dist_iters) o.max_dist_iters = di.iters;
        if (di.state == DIST_HITMAX) { o.time = timeLo; o.state = TOI_MAX_DIST_ITERS; return o; }
        /* Simplex::GetCache (Simplex.hpp:156-159) */
        cache.n = di.s.n;
        for (int k = 0; k < di.s.n; ++k) { cache.ia[k] = di.s.e[k].iA; cache.ib[k] = di.s.e[k].iB; }
        cache.metric = simplex_metric(di.s.e, di.s.n);
        v2 wA, wB;
        witness_points(&di.s, &wA, &wB);
        const real distSquared = mag2(vsub(wB, wA));
        if (distSquared < minTargetSquared) { o.time = timeLo; o.state = TOI_OVERLAPPED; return o; }
        if (distSquared <= maxTargetSquared) { o.time = timeLo; o.state = TOI_TOUCHING; return o; }
        const sepfn fcn = separation_scenario(&cache, A, loA, B, loB);
        real timeHi = R(1); /* conf.timeMax */
        xf_t hiA = sweep_xf(sA, timeHi), hiB = sweep_xf(sB, timeHi);
        for (int pb = 0; pb < 254; ++pb) { /* MaxShapeVertices */
            const lenidx hs = find_min_separation(&fcn, A, hiA, B, hiB);
            if (hs.dist > maxTarget) { o.time = timeHi; o.state = TOI_SEPARATED; return o; }
            if (hs.dist >= minTarget) {
                if (timeHi == timeLo) { o.time = timeHi; o.state = TOI_SEPARATED; return o; }
                timeLo = timeHi; loA = hiA; loB = hiB;
                break;
            }
            const real loEval = sep_evaluate(&fcn, A, loA, B, loB, hs.ia, hs.ib);
            if (loEval <= maxTarget) {
                o.time = timeLo; o.state = (loEval < minTarget) ? TOI_BELOW_MIN_TARGET : TOI_TOUCHING;
                return o;
            }
            real a1 = timeLo, a2 = timeHi, s1 = loEval, s2 = hs.dist;
            int roots = 0;
            real t = timeLo;
            for (;;) {
                if (roots == conf->maxToiRootIters) {
                    if (roots > o.max_root_iters) o.max_root_iters = roots;
                    o.time = t; o.state = TOI_MAX_ROOT_ITERS; return o;
                }
                if (RNEXT(a1, a2) >= a2) {
                    if (roots > o.max_root_iters) o.max_root_iters = roots;
                    o.time = t; o.state = TOI_NEXT_AFTER; return o;
                }
                /* Secant / Bisect (Math.hpp:92-108) */
                t = (roots & 1) ? (a1 + (target - s1) * (a2 - a1) / (s2 - s1)) : ((a1 + a2) / R(2));
                ++roots;
                const xf_t tA = sweep_xf(sA, t), tB = sweep_xf(sB, t);
                const real sv = sep_evaluate(&fcn, A, tA, B, tB, hs.ia, hs.ib);
                if (fabs(sv - target) <= conf->tolerance) {
                    timeHi = t; hiA = tA; hiB = tB;
                    break;
                }
                if (sv > target) { a1 = t; s1 = sv; } else { a2 = t; s2 = sv; }
            }
            if (roots > o.max_root_iters) o.max_root_iters = roots;
        }
    }
    o.time = timeLo;
    o.state = TOI_MAX_TOI_ITERS;
    return o;
}

/* AabbTreeWorld::UpdateContactTOIs (AabbTreeWorld.cpp:1685-1750). */
static void update_contact_tois(or_world* w, const or_stepconf* conf, or_stepstats* st) {
    for (int i = 0; i < w->wcids.n; ++i) {
        contact_t* c = &w->c[w->wcids.a[i]];
        if (c->toiValid) continue;
        if (c->sensor || !c->impenetrable) continue;
        if (c->toiCount >= conf->maxSubSteps) { st->toiContactsAtMaxSubSteps++; continue; }
        body_t* bA = &w->b[c->bA];
        body_t* bB = &w->b[c->bB];
        if (!(bA->flags & BF_AWAKE) && !(bB->flags & BF_AWAKE)) continue;
        const real alpha0 = maxr(bA->alpha0, bB->alpha0);
        body_advance0(bA, alpha0);
        body_advance0(bB, alpha0);
        const sweep_t sA = sweep_normalized(body_sweep(bA));
        const sweep_t sB = sweep_normalized(body_sweep(bB));
        const toi_out o = toi_via_sat(&w->s[c->sA].dp, &sA, &w->s[c->sB].dp, &sB, conf);
        c->toi = (o.state == TOI_TOUCHING) ? minr(alpha0 + (R(1) - alpha0) * o.time, R(1)) : R(1);
        c->toiValid = 1;
        if (o.max_dist_iters > st->toiMaxDistIters) st->toiMaxDistIters = o.max_dist_iters;
        if (o.toi_iters > st->toiMaxToiIters) st->toiMaxToiIters = o.toi_iters;
        if (o.max_root_iters > st->toiMaxRootIters) st->toiMaxRootIters = o.max_root_iters;
        st->toiContactsUpdatedToi++;
    }
}

/* FlagForUpdating(contacts of a body) (AabbTreeWorld.cpp). */
static void flag_body_contacts(or_world* w, const body_t* b) {
    for (int k = 0; k < b->cids.n; ++k) w->c[b->cids.a[k]].needsUpdate = 1;
}

/* AabbTreeWorld::SolveToiViaGS (AabbTreeWorld.cpp:1957-2059). */
static void solve_toi_island(or_world* w, const or_stepconf* conf, island_t* isl, or_stepstats* st,
                             int* posIters, int* velIters) {
    bc_t* bcs = (bc_t*)calloc((size_t)w->nb + 1, sizeof(bc_t));
    for (int i = 0; i < isl->bodies.n; ++i) {
        const int id = (int)isl->bodies.a[i];
        make_bc(&bcs[id], &w->b[id], R(0), conf);
    }
    const int nc = isl->contacts.n;
    pc_t* pcs = (pc_t*)malloc(sizeof(pc_t) * (size_t)(nc + 1));
    vc_t* vcs = (vc_t*)malloc(sizeof(vc_t) * (size_t)(nc + 1));
    for (int i = 0; i < nc; ++i) {
        const contact_t* c = &w->c[isl->contacts.a[i]];
        pcs[i].m = &c->m; pcs[i].bA = c->bA; pcs[i].bB = c->bB;
        pcs[i].totalRadius = w->s[c->sA].dp.r + w->s[c->sB].dp.r;
    }
    /* GetToiConstraintSolverConf (ConstraintSolverConf.cpp:37-45) */
    or_stepconf ps = *conf;
    ps.regResolutionRate = conf->toiResolutionRate;
    real minSepAll = RINF;
    int solved = 0;
    *posIters = conf->toiPositionIters;
    for (int it = 0; it < conf->toiPositionIters; ++it) {
        real minSep = RINF;
        for (int i = 0; i < nc; ++i) minSep = minr(minSep, solve_pc(&pcs[i], bcs, &ps));
        minSepAll = minr(minSepAll, minSep);
        if (minSep >= conf->toiMinSeparation) { *posIters = it + 1; solved = 1; break; }
    }
    for (int i = 0; i < isl->bodies.n; ++i) {
        const int id = (int)isl->bodies.a[i];
        w->b[id].pos0 = bcs[id].pos; /* SetPosition0: the sweep only */
    }
    /* GetToiVelocityConstraintConf (VelocityConstraint.cpp:207-210): dtRatio 0 */
    or_stepconf vcf = *conf;
    vcf.dtRatio = R(0);
    for (int i = 0; i < nc; ++i) {
        const contact_t* c = &w->c[isl->contacts.a[i]];
        const bc_t* A = &bcs[c->bA];
        const bc_t* B = &bcs[c->bB];
        const real rA = w->s[c->sA].dp.r, rB = w->s[c->sB].dp.r;
        const wman_t wm = world_manifold(&c->m, get_xf(A->pos, A->lc), rA, get_xf(B->pos, B->lc), rB);
        make_vc(&vcs[i], c, &wm, bcs, &vcf);
    }
    real maxInc = R(0);
    *velIters = conf->toiVelocityIters;
    for (int it = 0; it < conf->toiVelocityIters; ++it) {
        real newInc = R(0);
        for (int i = 0; i < nc; ++i) newInc = maxr(newInc, solve_vc(&vcs[i], bcs));
        if (newInc <= conf->toiMinMomentum) { *velIters = it + 1; break; }
        maxInc = maxr(maxInc, newInc);
    }
    const real h = conf->deltaTime;
    for (int i = 0; i < isl->bodies.n; ++i) {
        bc_t* bc = &bcs[isl->bodies.a[i]];
        const v2 tr = vmul(bc->vel.lin, h);
        const real rot = h * bc->vel.ang;
        bc->pos.lin = vadd(bc->pos.lin, tr);
        bc->pos.ang = bc->pos.ang + rot;
    }
    for (int i = 0; i < isl->bodies.n; ++i) {
        const int id = (int)isl->bodies.a[i];
        body_t* b = &w->b[id];
        b->vel = bcs[id].vel;
        if (pos_ne(b->pos1, bcs[id].pos)) {
            body_set_pos1(b, bcs[id].pos);
            flag_body_contacts(w, b);
        }
    }
    /* Report to PostSolveContact (AabbTreeWorld.cpp:2053-2055) */
    for (int i = 0; i < nc; ++i) {
        const real ni[2] = {vcs[i].p[0].ni, vcs[i].p[1].ni}, ti[2] = {vcs[i].p[0].ti, vcs[i].p[1].ti};
        record_solve_call(w, 4, &w->c[isl->contacts.a[i]], vcs[i].count, *posIters, ni, ti);
    }
    if (solved) st->toiIslandsSolved++;
    st->toiMinSeparation = minr(st->toiMinSeparation, minSepAll);
    st->toiMaxIncImpulse = maxr(st->toiMaxIncImpulse, maxInc);
    free(pcs); free(vcs); free(bcs);
}

/* AabbTreeWorld::ProcessContactsForTOI (AabbTreeWorld.cpp:2061-2142). */
static void process_contacts_for_toi(or_world* w, int id, island_t* isl, real toi, const or_stepconf* conf,
                                     int* updated, int* skipped) {
    body_t* body = &w->b[id];
    const int bodyImpenetrable = is_impenetrable(body);
    for (int k = 0; k < w->b[id].cids.n; ++k) {
        const int cid = (int)w->b[id].cids.a[k];
        contact_t* c = &w->c[cid];
        if (c->islanded || c->sensor) continue;
        const int otherId = (c->bA == id) ? c->bB : c->bA;
        body_t* other = &w->b[otherId];
        if (!(bodyImpenetrable || is_impenetrable(other))) continue;
        const int otherIslanded = other->islanded;
        const sweep_t backup = body_sweep(other);
        if (!otherIslanded) {
            body_advance(other, toi);
            if (pos_ne(other->pos0, backup.p0) || pos_ne(other->pos1, backup.p1)) flag_body_contacts(w, other);
        }
        if (c->needsUpdate) { contact_update(w, cid, conf); ++*updated; }
        else ++*skipped;
        if (!c->touching) { body_set_sweep(other, backup); continue; }
        iv_push(&isl->contacts, cid);
        c->islanded = 1;
        if (!otherIslanded) {
            if (is_speedable(other)) other->flags |= BF_AWAKE;
            iv_push(&isl->bodies, otherId);
            other->islanded = 1;
        }
    }
}

/* AabbTreeWorld::SolveToi(ContactID, StepConf) (AabbTreeWorld.cpp:1833-1955). */
static void solve_toi_contact(or_world* w, int cid, const or_stepconf* conf, island_t* isl, or_stepstats* st) {
    contact_t* c = &w->c[cid];
    const real toi = c->toi;
    const int idA = c->bA, idB = c->bB;
    body_t* bA = &w->b[idA];
    body_t* bB = &w->b[idB];
    int updated = 0, skipped = 0;
    {
        const sweep_t backupA = body_sweep(bA), backupB = body_sweep(bB);
        body_advance(bA, toi);
        if (pos_ne(bA->pos0, backupA.p0) || pos_ne(bA->pos1, backupA.p1)) flag_body_contacts(w, bA);
        body_advance(bB, toi);
        if (pos_ne(bB->pos0, backupB.p0) || pos_ne(bB->pos1, backupB.p1)) flag_body_contacts(w, bB);
        if (c->needsUpdate) { contact_update(w, cid, conf); ++updated; }
        c->toiValid = 0;
        c->toiCount++;
        if (!c->touching) {
            body_set_sweep(bA, backupA);
            body_set_sweep(bB, backupB);
            st->toiContactsUpdatedTouching += updated;
            st->toiContactsSkippedTouching += updated ? 0 : 1;
            return;
        }
    }
    if (is_speedable(bA)) bA->flags |= BF_AWAKE;
    if (is_speedable(bB)) bB->flags |= BF_AWAKE;
    isl->bodies.n = isl->contacts.n = isl->joints.n = 0;
    bA->islanded = 1; bB->islanded = 1; c->islanded = 1;
    iv_push(&isl->bodies, idA);
    iv_push(&isl->bodies, idB);
    iv_push(&isl->contacts, cid);
    if (is_accelerable(bA)) process_contacts_for_toi(w, idA, isl, toi, conf, &updated, &skipped);
    if (is_accelerable(bB)) process_contacts_for_toi(w, idB, isl, toi, conf, &updated, &skipped);
    /* RemoveUnspeedablesFromIslanded */
    for (int i = 0; i < isl->bodies.n; ++i) {
        body_t* b = &w->b[isl->bodies.a[i]];
        if (!is_speedable(b)) b->islanded = 0;
    }
    or_stepconf sub = *conf;
    sub.deltaTime = (R(1) - toi) * conf->deltaTime;
    int posIters = 0, velIters = 0;
    solve_toi_island(w, &sub, isl, st, &posIters, &velIters);
    st->toiSumPosIters += posIters;
    st->toiSumVelIters += velIters;
    if (posIters > 0 || velIters > 0) st->toiIslandsFound++;
    st->toiContactsUpdatedTouching += updated;
    st->toiContactsSkippedTouching += skipped;
}

/* AabbTreeWorld::SolveToi(StepConf) (AabbTreeWorld.cpp:1752-1831), no sub-stepping. */
static void solve_toi(or_world* w, const or_stepconf* conf, or_stepstats* st) {
    island_t isl;
    memset(&isl, 0, sizeof(isl));
    for (;;) {
        update_contact_tois(w, conf, st);
        /* GetSoonestContact (AabbTreeWorld.cpp:2870-2890) */
        int next = -1;
        real minToi = R(1);
        for (int i = 0; i < w->wcids.n; ++i) {
            const contact_t* c = &w->c[w->wcids.a[i]];
            if (c->toiValid && minToi > c->toi) { minToi = c->toi; next = (int)w->wcids.a[i]; }
        }
        if (next < 0) {
            /* e_stepComplete, ResetBodiesForSolveTOI, ResetContactsForSolveTOI (:1770-1777) */
            w->step_incomplete = 0;
            for (int id = 0; id < w->nb; ++id) { w->b[id].alpha0 = R(0); w->b[id].islanded = 0; }
            for (int i = 0; i < w->wcids.n; ++i) {
                contact_t* c = &w->c[w->wcids.a[i]];
                c->toiValid = 0; c->toiCount = 0; c->islanded = 0;
            }
            break;
        }
        st->toiContactsFound++;
        if (!w->c[next].islanded) solve_toi_contact(w, next, conf, &isl, st);
        for (int id = 0; id < w->nb; ++id) {
            body_t* b = &w->b[id];
            if (!b->islanded) continue;
            b->islanded = 0;
            if (is_accelerable(b)) {
                st->toiProxiesMoved += synchronize(w, id, conf);
                for (int k = 0; k < b->cids.n; ++k) {
                    contact_t* c = &w->c[b->cids.a[k]];
                    c->toiValid = 0;
                    c->islanded = 0;
                }
            }
        }
        st->toiContactsAdded += find_and_add_contacts(w, conf);
        if (w->sub_stepping) {  /* one event per Step (:1819-1823) */
            w->step_incomplete = 1;
            break;
        }
    }
    {
        const int upd = update_contacts(w, conf); /* UpdateContacts: updated and skipped counts */
        st->toiContactsUpdatedTouching += upd;
        st->toiContactsSkippedTouching += w->wcids.n - upd;
    }
    iv_free(&isl.bodies); iv_free(&isl.contacts); iv_free(&isl.joints);
}

/* Stand-alone entry points for known-answer tests. */
static void load_dproxy(dproxy* p, int n, const real* xy, real r) {
    memset(p, 0, sizeof(*p));
    p->count = n > OR_MAXV ? OR_MAXV : n;
    p->r = r;
    for (int i = 0; i < p->count; ++i) p->v[i] = V(xy[2 * i], xy[2 * i + 1]);
    make_normals(p);
}
real or_time_of_impact(int kindA, int nA, const real* xyA, real rA, const real* sweepA7, const real* lcA2,
                       int kindB, int nB, const real* xyB, real rB, const real* sweepB7, const real* lcB2,
                       const or_stepconf* conf, int* iout4) {
    (void)kindA; (void)kindB;
    dproxy a, b;
    load_dproxy(&a, nA, xyA, rA);
    load_dproxy(&b, nB, xyB, rB);
    sweep_t sa, sb;
    sa.p0.lin = V(sweepA7[0], sweepA7[1]); sa.p0.ang = sweepA7[2];
    sa.p1.lin = V(sweepA7[3], sweepA7[4]); sa.p1.ang = sweepA7[5]; sa.a0 = sweepA7[6];
    sa.lc = V(lcA2[0], lcA2[1]);
    sb.p0.lin = V(sweepB7[0], sweepB7[1]); sb.p0.ang = sweepB7[2];
    sb.p1.lin = V(sweepB7[3], sweepB7[4]); sb.p1.ang = sweepB7[5]; sb.a0 = sweepB7[6];
    sb.lc = V(lcB2[0], lcB2[1]);
    const toi_out o = toi_via_sat(&a, &sa, &b, &sb, conf);
    iout4[0] = o.state; iout4[1] = o.toi_iters; iout4[2] = o.max_dist_iters; iout4[3] = o.max_root_iters;
    return o.time;
}
void or_distance(int kindA, int nA, const real* xyA, real rA, const real* xfA4, int kindB, int nB,
                 const real* xyB, real rB, const real* xfB4, int maxIters, int* iout3, real* fout4) {
    (void)kindA; (void)kindB;
    dproxy a, b;
    load_dproxy(&a, nA, xyA, rA);
    load_dproxy(&b, nB, xyB, rB);
    xf_t xa, xb;
    xa.p = V(xfA4[0], xfA4[1]); xa.q = V(xfA4[2], xfA4[3]);
    xb.p = V(xfB4[0], xfB4[1]); xb.q = V(xfB4[2], xfB4[3]);
    scache cache;
    memset(&cache, 0, sizeof(cache));
    const dist_out d = gjk_distance(&a, xa, &b, xb, &cache, maxIters);
    v2 pA, pB;
    witness_points(&d.s, &pA, &pB);
    iout3[0] = d.state; iout3[1] = d.iters; iout3[2] = d.s.n;
    fout4[0] = pA.x; fout4[1] = pA.y; fout4[2] = pB.x; fout4[3] = pB.y;
}

/* Step(AabbTreeWorld&, StepConf) (AabbTreeWorld.cpp:2144-2219). */
void or_step(or_world* w, const or_stepconf* conf, or_stepstats* st) {
    or_stepstats local;
    if (!st) st = &local;
    memset(st, 0, sizeof(*st));
    w->events.n = 0;
    w->solve_calls.n = 0;
    st->regMinSeparation = RINF;
    for (int i = 0; i < w->fixturesForProxies.n; ++i) {
        const int body = (int)(w->fixturesForProxies.a[i] >> 32);
        const int shape = (int)(w->fixturesForProxies.a[i] & 0xffffffff);
        create_proxies(w, body, shape, conf);
        st->preProxiesCreated++;
    }
    w->fixturesForProxies.n = 0;
    for (int i = 0; i < w->bodiesForSync.n; ++i) st->preProxiesMoved += synchronize(w, (int)w->bodiesForSync.a[i], conf);
    w->bodiesForSync.n = 0;
    st->preContactsDestroyed = destroy_contacts(w);
    st->preContactsUpdated = update_contacts(w, conf);
    st->preContactsAdded = find_and_add_contacts(w, conf);
    st->toiMinSeparation = RINF;
    if (conf->deltaTime != R(0)) {
        w->inv_dt0 = R(1) / conf->deltaTime;
        if (!w->step_incomplete) solve_reg(w, conf, st);  /* IsStepComplete (:2206-2209) */
        if (conf->doToi) solve_toi(w, conf, st);
    }
}

void or_set_sub_stepping(or_world* w, int flag) { w->sub_stepping = flag != 0; }
int or_is_step_complete(const or_world* w) { return !w->step_incomplete; }

/* StepConf defaults (StepConf.hpp:59-161, Settings.hpp). */
void or_default_conf(or_stepconf* c) {
    const real Pi = R(3.14159265358979323846264338327950288L);
    const real linearSlop = R(0.005);
    memset(c, 0, sizeof(*c));
    c->deltaTime = R(1) / R(60);
    c->dtRatio = R(1);
    c->minStillTimeToSleep = R(1) / R(2);
    c->linearSlop = linearSlop;
    c->angularSlop = (Pi * R(2)) / R(180);
    c->regResolutionRate = R(2) / R(10);
    c->regMinSeparation = -linearSlop * R(3);
    c->regMinMomentum = R(0) / R(100);
    c->velocityThreshold = R(1);
    c->maxTranslation = R(2);
    c->maxRotation = R(179) * ((R(1) * Pi) / R(180));
    c->maxLinearCorrection = R(0.2);
    c->maxAngularCorrection = R(8.0f / 180.0f) * Pi;
    c->linearSleepTolerance = R(0.01);
    c->angularSleepTolerance = R((Pi * R(2)) / R(180));
    c->displaceMultiplier = R(2);
    c->aabbExtension = linearSlop * R(20);
    c->maxCirclesRatio = R(10);
    c->regVelocityIters = 8;
    c->regPositionIters = 3;
    c->doWarmStart = 1;
    c->doBlocksolve = 1;
    c->toiResolutionRate = R(75) / R(100);
    c->toiMinSeparation = -linearSlop * R(1.5f);
    c->toiMinMomentum = R(0) / R(100);
    c->targetDepth = linearSlop * R(3);
    c->tolerance = linearSlop / R(4);
    c->toiVelocityIters = 8;
    c->toiPositionIters = 20;
    c->maxToiRootIters = 30;
    c->maxToiIters = 20;
    c->maxDistanceIters = 20;
    c->maxSubSteps = 8;
    c->doToi = 0; /* the reference's default is true; callers opt in */
}

/* ------------------------------------------------------------------------- */
/* Queries.                                                                   */
/* ------------------------------------------------------------------------- */
int or_body_count(const or_world* w) { return w->nb; }
void or_get_body(const or_world* w, int id, real* o, int* awake) {
    const body_t* b = &w->b[id];
    o[0] = b->pos1.lin.x; o[1] = b->pos1.lin.y; o[2] = b->pos1.ang;
    o[3] = b->vel.lin.x; o[4] = b->vel.lin.y; o[5] = b->vel.ang;
    o[6] = b->xf.p.x; o[7] = b->xf.p.y; o[8] = b->xf.q.x; o[9] = b->xf.q.y;
    o[10] = b->invM; o[11] = b->invI; o[12] = b->uat;
    if (awake) *awake = (b->flags & BF_AWAKE) ? 1 : 0;
}
void or_get_local_center(const or_world* w, int id, real* o) { o[0] = w->b[id].lc.x; o[1] = w->b[id].lc.y; }
/* SetTransformation-like state override used by tests; queues proxy sync. */
void or_set_body_state(or_world* w, int id, real px, real py, real angle, real vx, real vy, real av) {
    body_t* b = &w->b[id];
    pos_t p; p.lin = V(px, py); p.ang = angle;
    b->pos0 = p;
    body_set_pos1(b, p);
    b->vel.lin = V(vx, vy); b->vel.ang = av;
    for (int k = 0; k < b->cids.n; ++k) w->c[b->cids.a[k]].needsUpdate = 1;
    iv_push(&w->bodiesForSync, id);
}
static int cmp_i64pair(const void* a, const void* b) {
    const int64_t* x = (const int64_t*)a;
    const int64_t* y = (const int64_t*)b;
    return (x[0] < y[0]) ? -1 : (x[0] > y[0]) ? 1 : 0;
}
void or_set_solve_order(or_world* w, int n, const int* items3) {
    w->order_ckeys.n = w->order_crank.n = w->order_jrank.n = 0;
    if (n <= 0) return;
    int64_t* pairs = (int64_t*)malloc(sizeof(int64_t) * 2 * (size_t)n);
    int np = 0;
    for (int i = 0; i < n; ++i) {
        const int kind = items3[3 * i], a = items3[3 * i + 1], b = items3[3 * i + 2];
        if (kind == 0) {
            const int lo = a < b ? a : b, hi = a < b ? b : a;
            pairs[2 * np] = ((int64_t)lo << 32) | (int64_t)hi;
            pairs[2 * np + 1] = i;
            ++np;
        } else {
            while (w->order_jrank.n <= a) iv_push(&w->order_jrank, -1);
            w->order_jrank.a[a] = i;
        }
    }
    qsort(pairs, (size_t)np, 2 * sizeof(int64_t), cmp_i64pair);
    for (int i = 0; i < np; ++i) {
        iv_push(&w->order_ckeys, pairs[2 * i]);
        iv_push(&w->order_crank, pairs[2 * i + 1]);
    }
    free(pairs);
}

void or_set_body_xf(or_world* w, int id, real px, real py, real c, real sn) {
    body_t* b = &w->b[id];
    b->xf.p = V(px, py);
    b->xf.q = V(c, sn);
}
int or_contact_count(const or_world* w) { return w->wcids.n; }
void or_get_contact(const or_world* w, int k, int* io, real* fo, int* feat) {
    const int cid = (int)w->wcids.a[k];
    const contact_t* c = &w->c[cid];
    io[0] = cid; io[1] = c->pA; io[2] = c->pB; io[3] = c->bA; io[4] = c->sA; io[5] = c->cA;
    io[6] = c->bB; io[7] = c->sB; io[8] = c->cB; io[9] = c->touching; io[10] = c->m.type; io[11] = c->m.count;
    fo[0] = c->m.ln.x; fo[1] = c->m.ln.y; fo[2] = c->m.lp.x; fo[3] = c->m.lp.y;
    for (int i = 0; i < 2; ++i) {
        fo[4 + 4 * i] = c->m.p[i].lp.x; fo[5 + 4 * i] = c->m.p[i].lp.y;
        fo[6 + 4 * i] = c->m.p[i].ni; fo[7 + 4 * i] = c->m.p[i].ti;
        feat[4 * i + 0] = c->m.p[i].tA; feat[4 * i + 1] = c->m.p[i].iA;
        feat[4 * i + 2] = c->m.p[i].tB; feat[4 * i + 3] = c->m.p[i].iB;
    }
}
int or_proxy_count(const or_world* w) { return w->np; }
void or_get_proxy(const or_world* w, int p, int* bsc, real* aabb) {
    bsc[0] = w->p[p].body; bsc[1] = w->p[p].shape; bsc[2] = w->p[p].child;
    memcpy(aabb, w->p[p].aabb, 4 * sizeof(real));
}

/* RayCast(radius, location, input) (RayCastOutput.cpp:41-71). */
static int ray_circle(real radius, v2 loc, v2 p1, v2 p2, real maxF, real* frac, v2* normal) {
    const v2 s = vsub(p1, loc);
    const real b = mag2(s) - radius * radius;
    const v2 seg = vsub(p2, p1);
    const real c = dot(s, seg);
    const real rr = mag2(seg);
    const real sigma = (c * c) - rr * b;
    if ((sigma < R(0)) || almost_zero(rr)) return 0;
    const real a = -(c + RSQRT(sigma));
    const real f = a / rr;
    if ((f >= R(0)) && (f <= maxF)) {
        *frac = f;
        *normal = unit_vector(vadd(s, vmul(seg, f)), V(R(0), R(0)));
        return 1;
    }
    return 0;
}

/* RayCast(DistanceProxy, input, transform) (RayCastOutput.cpp:132-233). */
static int ray_proxy(const dproxy* P, xf_t xf, v2 p1, v2 p2, real maxF, real* frac, v2* normal) {
    const real radius = P->r;
    v2 v0 = P->v[0];
    if (P->count == 1) return ray_circle(radius, xform(v0, xf), p1, p2, maxF, frac, normal);
    const v2 r0 = invxform(p1, xf), r1 = invxform(p2, xf);
    const v2 ray = vsub(r1, r0);
    real minT = RNEXT(maxF, R(2));
    v2 found = V(R(0), R(0));
    for (int i = 0; i < P->count; ++i) {
        real cf;
        v2 cn;
        if (ray_circle(radius, v0, r0, r1, maxF, &cf, &cn) && (minT > cf)) { minT = cf; found = cn; }
        const v2 v1 = P->v[(i + 1) % P->count];
        const v2 edge = vsub(v1, v0);
        const real rxe = cross(ray, edge);
        if (!almost_zero(rxe)) {
            const v2 n = P->n[i];
            const v2 q = vsub(vadd(v0, vmul(n, radius)), r0);
            const real inv = R(1) / rxe;
            const real t = cross(q, edge) * inv;
            const real u = cross(q, ray) * inv;
            if ((t >= R(0)) && (t <= R(1)) && (u >= R(0)) && (u <= R(1)) && (minT > t)) { minT = t; found = n; }
        }
        v0 = v1;
    }
    if (minT <= maxF) {
        *frac = minT;
        *normal = rotate(found, xf.q);
        return 1;
    }
    return 0;
}

/* RayCast(World, input, callback) (RayCastOutput.cpp:301-337) with a callback
 * that answers ResetRay: every shape with a proxy that the ray hits.  Up to cap
 * hits in shape order into shapes and hit5 (fraction, point = p1 + (p2 - p1) *
 * fraction, normal); returns how many there were.  The tree walk only prunes:
 * a shape the ray hits lies inside its fat AABB. */
int or_raycast(const or_world* w, real p1x, real p1y, real p2x, real p2y, real maxF, int cap, int* shapes,
               real* hit5) {
    const v2 p1 = V(p1x, p1y), p2 = V(p2x, p2y);
    int n = 0;
    for (int p = 0; p < w->np; ++p) {
        const int s = w->p[p].shape;
        real f;
        v2 nrm;
        if (!ray_proxy(&w->s[s].dp, w->b[w->p[p].body].xf, p1, p2, maxF, &f, &nrm)) continue;
        if (n < cap) {
            /* insertion in shape order */
            int k = n;
            while (k > 0 && shapes[k - 1] > s) {
                shapes[k] = shapes[k - 1];
                for (int q = 0; q < 5; ++q) hit5[5 * k + q] = hit5[5 * (k - 1) + q];
                --k;
            }
            const v2 pt = vadd(p1, vmul(vsub(p2, p1), f));
            shapes[k] = s;
            hit5[5 * k] = f; hit5[5 * k + 1] = pt.x; hit5[5 * k + 2] = pt.y;
            hit5[5 * k + 3] = nrm.x; hit5[5 * k + 4] = nrm.y;
        }
        ++n;
    }
    return n;
}

/* The PreSolveContact / PostSolveContact calls of the last or_step, in call
 * order: up to cap records of 5 ints (kind 3 or 4, lower shape, higher shape,
 * point count, iteration) into ints and 4 doubles (normal and tangent impulse
 * of both points) into imp; returns how many calls there were. */
int or_solve_calls(const or_world* w, int* ints, double* imp, int cap) {
    const int n = w->solve_calls.n / 9;
    for (int i = 0; i < n && i < cap; ++i) {
        const int64_t* r = w->solve_calls.a + 9 * i;
        for (int k = 0; k < 5; ++k) ints[5 * i + k] = (int)r[k];
        for (int k = 0; k < 4; ++k) memcpy(&imp[4 * i + k], &r[5 + k], sizeof(double));
    }
    return n;
}

/* The contact listener calls of the last or_step: up to cap (kind, shape,
 * shape) triples into out; returns how many there were. */
int or_events(const or_world* w, int* out, int cap) {
    const int n = w->events.n / 3;
    for (int i = 0; i < n && i < cap; ++i)
        for (int k = 0; k < 3; ++k) out[3 * i + k] = (int)w->events.a[3 * i + k];
    return n;
}
