// prgpu_toi.cuh -- time of impact: sweeps, GJK distance, separation scenarios
// and the conservative-advancement root finder (GetToiViaSat).
//
// Restates Sweep.cpp, d2/Math.hpp (GetTransformation of a sweep, GetNormalized),
// Math.cpp:33-91 (angle normalisation), Simplex.cpp, Distance.cpp:71-196,
// SeparationScenario.cpp and TimeOfImpact.cpp:37-253 in float with the
// reference's operation order.  One call runs on one thread; the phase kernels
// (prgpu_toi.cu) give each contact or each world its own thread.
#pragma once

#include "prgpu_collide.cuh"

namespace prgpu {

// Position (x, y, angle) arithmetic (d2/Position.hpp).
struct Pos {
    float x, y, a;
};
PR_HD Pos mkpos(float x, float y, float a) { Pos p; p.x = x; p.y = y; p.a = a; return p; }
PR_HD bool pos_ne(Pos p, Pos q) { return !(p.x == q.x && p.y == q.y && p.a == q.a); }
// GetPosition (d2/Math.cpp:30-60): pos0 + (pos1 - pos0) * beta.
PR_HD Pos plerp(Pos p0, Pos p1, float beta) {
    const float dx = p1.x - p0.x, dy = p1.y - p0.y, da = p1.a - p0.a;
    const float sx = dx * beta, sy = dy * beta, sa = da * beta;
    return mkpos(p0.x + sx, p0.y + sy, p0.a + sa);
}

// Sweep (d2/Sweep.hpp:43-92): positions at alpha0 and 1, local centre.
struct Sweep {
    Pos p0, p1;
    V2 lc;
    float a0;
};
// GetTransformation(sweep, beta) (d2/Math.hpp:251-254).
PR_HD Xf sweep_xf(const Sweep& s, float beta) {
    const Pos p = plerp(s.p0, s.p1, beta);
    return get_xf(p.x, p.y, p.a, s.lc);
}
// Advance0 (Sweep.cpp:27-31).
PR_HD void sweep_advance0(Sweep& s, float alpha) {
    const float beta = (alpha - s.a0) / (1.0f - s.a0);
    s.p0 = plerp(s.p0, s.p1, beta);
    s.a0 = alpha;
}
// GetNormalized(Angle) (Math.cpp:33-91, the default branch).
PR_HD float angle_normalized(float a) {
    const float Pi = 3.14159265358979323846264338327950288f;
    const float twoPi = 2.0f * Pi;
    const float rTwoPi = 1.0f / twoPi;
    a = a - truncf(a * rTwoPi) * twoPi;
    if (a >= Pi) a -= Pi * 2.0f;
    else if (a < -Pi) a += Pi * 2.0f;
    return a;
}
// GetNormalized(Sweep) (d2/Math.hpp:160-167).
PR_HD Sweep sweep_normalized(Sweep s) {
    const float a0 = angle_normalized(s.p0.a);
    const float d = s.p0.a - a0;
    s.p0.a = a0;
    s.p1.a -= d;
    return s;
}

// ---- Simplex (SimplexEdge.hpp, Simplex.cpp) ---------------------------------
struct SEdge {
    V2 pA, pB;
    int iA, iB;
};
struct Simplex {
    int n;
    SEdge e[3];
    float c[3];
};
// Simplex::Cache: index pairs of the last simplex and its metric.
struct SCache {
    int n;
    int ia[3], ib[3];
    float metric;
};

PR_HD SEdge make_sedge(const Proxy& A, Xf xfA, int ia, const Proxy& B, Xf xfB, int ib) {
    SEdge e;
    e.pA = xform(A.vtx(ia), xfA); e.iA = ia;
    e.pB = xform(B.vtx(ib), xfB); e.iB = ib;
    return e;
}
PR_HD V2 sdelta(const SEdge& e) { return e.pB - e.pA; }
PR_HD Simplex simplex1(const SEdge& s0) {
    Simplex r;
    r.n = 1; r.e[0] = s0; r.c[0] = 1.0f; r.c[1] = r.c[2] = 0.f;
    r.e[1] = r.e[2] = s0;
    return r;
}
PR_HD Simplex simplex2(const SEdge& s0, const SEdge& s1, float c0, float c1) {
    Simplex r;
    r.n = 2; r.e[0] = s0; r.e[1] = s1; r.e[2] = s1; r.c[0] = c0; r.c[1] = c1; r.c[2] = 0.f;
    return r;
}
// Simplex::Get (Simplex.cpp:55-169).
PR_HD Simplex simplex_get(const SEdge* s, int n) {
    if (n == 1) return simplex1(s[0]);
    if (n == 2) {
        const V2 w1 = sdelta(s[0]), w2 = sdelta(s[1]);
        const V2 e12 = w2 - w1;
        const float d12_2 = -dot(w1, e12);
        if (d12_2 <= 0.f) return simplex1(s[0]);
        const float d12_1 = dot(w2, e12);
        if (d12_1 <= 0.f) return simplex1(s[1]);
        const float inv_sum = 1.0f / (d12_1 + d12_2);
        return simplex2(s[0], s[1], d12_1 * inv_sum, d12_2 * inv_sum);
    }
    const V2 w1 = sdelta(s[0]), w2 = sdelta(s[1]), w3 = sdelta(s[2]);
    const V2 e12 = w2 - w1;
    const float d12_1 = dot(w2, e12);
    const float d12_2 = -dot(w1, e12);
    const V2 e13 = w3 - w1;
    const float d13_1 = dot(w3, e13);
    const float d13_2 = -dot(w1, e13);
    const V2 e23 = w3 - w2;
    const float d23_1 = dot(w3, e23);
    const float d23_2 = -dot(w2, e23);
    if ((d12_2 <= 0.f) && (d13_2 <= 0.f)) return simplex1(s[0]);
    if ((d12_1 <= 0.f) && (d23_2 <= 0.f)) return simplex1(s[1]);
    if ((d13_1 <= 0.f) && (d23_1 <= 0.f)) return simplex1(s[2]);
    const float n123 = cross(e12, e13);
    const float d123_3 = n123 * cross(w1, w2);
    if ((d12_1 > 0.f) && (d12_2 > 0.f) && (d123_3 <= 0.f)) {
        const float inv_sum = 1.0f / (d12_1 + d12_2);
        return simplex2(s[0], s[1], d12_1 * inv_sum, d12_2 * inv_sum);
    }
    const float d123_2 = n123 * cross(w3, w1);
    if ((d13_1 > 0.f) && (d13_2 > 0.f) && (d123_2 <= 0.f)) {
        const float inv_sum = 1.0f / (d13_1 + d13_2);
        return simplex2(s[0], s[2], d13_1 * inv_sum, d13_2 * inv_sum);
    }
    const float d123_1 = n123 * cross(w2, w3);
    if ((d23_1 > 0.f) && (d23_2 > 0.f) && (d123_1 <= 0.f)) {
        const float inv_sum = 1.0f / (d23_1 + d23_2);
        return simplex2(s[2], s[1], d23_2 * inv_sum, d23_1 * inv_sum);
    }
    const float inv_sum = 1.0f / (d123_1 + d123_2 + d123_3);
    Simplex r;
    r.n = 3; r.e[0] = s[0]; r.e[1] = s[1]; r.e[2] = s[2];
    r.c[0] = d123_1 * inv_sum; r.c[1] = d123_2 * inv_sum; r.c[2] = d123_3 * inv_sum;
    return r;
}
// Simplex::CalcMetric (Simplex.cpp:171-192).
PR_HD float simplex_metric(const SEdge* s, int n) {
    if (n == 2) return sqrtf(mag2(sdelta(s[1]) - sdelta(s[0])));
    if (n == 3) return cross(sdelta(s[1]) - sdelta(s[0]), sdelta(s[2]) - sdelta(s[0]));
    return 0.f;
}
// CalcSearchDirection (Simplex.cpp:37-53).
PR_HD V2 search_direction(const SEdge* s, int n) {
    if (n == 1) return -sdelta(s[0]);
    if (n == 2) {
        const V2 e12 = sdelta(s[1]) - sdelta(s[0]);
        const V2 e0 = sdelta(s[0]);
        const float sgn = cross(e12, -e0);
        return (sgn > 0.f) ? revperp(e12) : fwdperp(e12);
    }
    return mk(0.f, 0.f);
}
// GetSupportIndex (DistanceProxy.hpp:233-249).  Where no vertex beats -inf (a
// NaN direction) this returns vertex 0 rather than the invalid index, so that no
// caller reads past the shape's vertices.
PR_HD int support_index(const Proxy& p, V2 dir) {
    int index = 0;
    float maxValue = -PR_INF;
    for (int i = 0; i < p.count; ++i) {
        const float value = dot(p.vtx(i), dir);
        if (maxValue < value) { maxValue = value; index = i; }
    }
    return index;
}

// DistanceOutput::State (Distance.hpp).
enum { DIST_HITMAX = 1, DIST_MAXPOINTS = 2, DIST_UNFIT = 3, DIST_DUPLICATE = 4 };
struct DistOut {
    Simplex s;
    int iters, state;
};
// Distance (Distance.cpp:96-196), seeded from the cache of the previous call.
PR_HD DistOut gjk_distance(const Proxy& A, Xf xfA, const Proxy& B, Xf xfB, const SCache& cache, int maxIters) {
    int sa[3] = {0, 0, 0}, sb[3] = {0, 0, 0};
    int sn = cache.n;
    SEdge edges[3];
    int ne = cache.n;
    for (int k = 0; k < sn; ++k) {
        sa[k] = cache.ia[k]; sb[k] = cache.ib[k];
        edges[k] = make_sedge(A, xfA, sa[k], B, xfB, sb[k]);
    }
    if (ne > 1) {
        const float metric1 = cache.metric;
        const float metric2 = simplex_metric(edges, ne);
        if ((metric2 < (metric1 / 2.0f)) || (metric2 > (metric1 * 2.0f)) || (metric2 < 0.f) || almost_zero(metric2))
            ne = 0;
    }
    if (ne == 0) {
        edges[0] = make_sedge(A, xfA, 0, B, xfB, 0);
        ne = 1;
        sn = 1; sa[0] = 0; sb[0] = 0;
    }
    DistOut out;
    out.s = simplex1(edges[0]);
    out.s.n = 0;
    out.state = DIST_HITMAX;
    int iter = 0;
    while (iter < maxIters) {
        ++iter;
        out.s = simplex_get(edges, ne);
        ne = out.s.n;
        for (int k = 0; k < ne; ++k) edges[k] = out.s.e[k];
        if (ne == 3) { out.state = DIST_MAXPOINTS; break; }
        const V2 d = search_direction(edges, ne);
        if (almost_zero(mag2(d))) { out.state = DIST_UNFIT; break; }
        const int ia = support_index(A, invrotate(-d, xfA.q));
        const int ib = support_index(B, invrotate(d, xfB.q));
        bool dup = false;
        for (int k = 0; k < sn; ++k) dup = dup || (sa[k] == ia && sb[k] == ib);
        if (dup) { out.state = DIST_DUPLICATE; break; }
        edges[ne++] = make_sedge(A, xfA, ia, B, xfB, ib);
        sn = ne;
        for (int k = 0; k < ne; ++k) { sa[k] = edges[k].iA; sb[k] = edges[k].iB; }
    }
    out.iters = iter;
    return out;
}
// GetWitnessPoints (Distance.cpp:71-94).
PR_HD void witness_points(const Simplex& s, V2& pA, V2& pB) {
    V2 a = mk(0.f, 0.f), b = mk(0.f, 0.f);
    for (int i = 0; i < s.n; ++i) {
        a = a + s.e[i].pA * s.c[i];
        b = b + s.e[i].pB * s.c[i];
    }
    pA = a; pB = b;
}

// ---- SeparationScenario (SeparationScenario.cpp) ----------------------------
enum { SEP_POINTS = 0, SEP_FACE_A = 1, SEP_FACE_B = 2 };
struct SepFn {
    int type;
    V2 axis, lp;
};
struct LenIdx {
    float dist;
    int ia, ib;
};
// GetSeparationScenario (SeparationScenario.cpp:148-205).
PR_HD SepFn separation_scenario(const SCache& c, const Proxy& A, Xf xfA, const Proxy& B, Xf xfB) {
    SepFn f;
    f.lp = mk(0.f, 0.f);
    const int type = (c.n < 2) ? SEP_POINTS : ((c.ia[0] == c.ia[1]) ? SEP_FACE_B : SEP_FACE_A);
    if (type == SEP_FACE_B) {
        const V2 lB1 = B.vtx(c.ib[0]), lB2 = B.vtx(c.ib[1]);
        const V2 axis = unit_vector(fwdperp(lB2 - lB1), mk(0.f, 0.f));
        const V2 normal = urotate(axis, xfB.q);
        const V2 lp = vdiv(lB1 + lB2, 2.0f);
        const V2 pB = xform(lp, xfB);
        const V2 pA = xform(A.vtx(c.ia[0]), xfA);
        f.type = SEP_FACE_B; f.lp = lp;
        f.axis = (dot(pA - pB, normal) < 0.f) ? -axis : axis;
        return f;
    }
    if (type == SEP_FACE_A) {
        const V2 lA1 = A.vtx(c.ia[0]), lA2 = A.vtx(c.ia[1]);
        const V2 axis = unit_vector(fwdperp(lA2 - lA1), mk(0.f, 0.f));
        const V2 normal = urotate(axis, xfA.q);
        const V2 lp = vdiv(lA1 + lA2, 2.0f);
        const V2 pA = xform(lp, xfA);
        const V2 pB = xform(B.vtx(c.ib[0]), xfB);
        f.type = SEP_FACE_A; f.lp = lp;
        f.axis = (dot(pB - pA, normal) < 0.f) ? -axis : axis;
        return f;
    }
    const V2 pA = xform(A.vtx(c.ia[0]), xfA);
    const V2 pB = xform(B.vtx(c.ib[0]), xfB);
    f.type = SEP_POINTS;
    f.axis = unit_vector(pB - pA, mk(0.f, 0.f));
    return f;
}
// FindMinSeparation (SeparationScenario.cpp:29-77).
PR_HD LenIdx find_min_separation(const SepFn& f, const Proxy& A, Xf xfA, const Proxy& B, Xf xfB) {
    LenIdx r;
    if (f.type == SEP_POINTS) {
        r.ia = support_index(A, invrotate(f.axis, xfA.q));
        r.ib = support_index(B, invrotate(-f.axis, xfB.q));
        r.dist = dot(xform(B.vtx(r.ib), xfB) - xform(A.vtx(r.ia), xfA), f.axis);
    } else if (f.type == SEP_FACE_A) {
        const V2 normal = urotate(f.axis, xfA.q);
        const V2 pA = xform(f.lp, xfA);
        r.ia = (int)kInvalidV;
        r.ib = support_index(B, invrotate(-normal, xfB.q));
        r.dist = dot(xform(B.vtx(r.ib), xfB) - pA, normal);
    } else {
        const V2 normal = urotate(f.axis, xfB.q);
        r.ia = support_index(A, invrotate(-normal, xfA.q));
        r.ib = (int)kInvalidV;
        const V2 pB = xform(f.lp, xfB);
        r.dist = dot(xform(A.vtx(r.ia), xfA) - pB, normal);
    }
    return r;
}
// Evaluate (SeparationScenario.cpp:79-119).
PR_HD float sep_evaluate(const SepFn& f, const Proxy& A, Xf xfA, const Proxy& B, Xf xfB, int ia, int ib) {
    if (f.type == SEP_POINTS) return dot(xform(B.vtx(ib), xfB) - xform(A.vtx(ia), xfA), f.axis);
    if (f.type == SEP_FACE_A) {
        const V2 normal = urotate(f.axis, xfA.q);
        return dot(xform(B.vtx(ib), xfB) - xform(f.lp, xfA), normal);
    }
    const V2 normal = urotate(f.axis, xfB.q);
    return dot(xform(A.vtx(ia), xfA) - xform(f.lp, xfB), normal);
}

// ToiOutput::State (ToiOutput.hpp), numbered as the C ABI reports it.
enum {
    TOI_UNKNOWN = 0, TOI_OVERLAPPED, TOI_TOUCHING, TOI_SEPARATED, TOI_MAX_ROOT_ITERS, TOI_NEXT_AFTER,
    TOI_MAX_TOI_ITERS, TOI_BELOW_MIN_TARGET, TOI_MAX_DIST_ITERS, TOI_TARGET_DEPTH_EXCEEDS_TOTAL_RADIUS,
    TOI_MIN_TARGET_SQUARED_OVERFLOW, TOI_MAX_TARGET_SQUARED_OVERFLOW
};
struct ToiLimits {
    float targetDepth, tolerance;
    int maxRootIters, maxToiIters, maxDistIters;
};
struct ToiOut {
    float time;
    int state, toi_iters, max_dist_iters, max_root_iters;
};

// GetToiViaSat (TimeOfImpact.cpp:37-253) with timeMax = 1.
PR_HD ToiOut toi_via_sat(const Proxy& A, const Sweep& sA, const Proxy& B, const Sweep& sB, const ToiLimits& L) {
    ToiOut o;
    o.time = 0.f; o.state = TOI_UNKNOWN; o.toi_iters = 0; o.max_dist_iters = 0; o.max_root_iters = 0;
    const float totalRadius = A.r + B.r;
    if (L.targetDepth > totalRadius) { o.state = TOI_TARGET_DEPTH_EXCEEDS_TOTAL_RADIUS; return o; }
    const float target = totalRadius - L.targetDepth;
    const float maxTarget = maxf_(target + L.tolerance, 0.f);
    const float minTarget = maxf_(target - L.tolerance, 0.f);
    const float minTargetSquared = minTarget * minTarget;
    if (!isfinite(minTargetSquared) && isfinite(minTarget)) { o.state = TOI_MIN_TARGET_SQUARED_OVERFLOW; return o; }
    const float maxTargetSquared = maxTarget * maxTarget;
    if (!isfinite(maxTargetSquared) && isfinite(maxTarget)) { o.state = TOI_MAX_TARGET_SQUARED_OVERFLOW; return o; }
    float timeLo = 0.f;
    Xf loA = sweep_xf(sA, timeLo), loB = sweep_xf(sB, timeLo);
    SCache cache;
    cache.n = 0; cache.metric = 0.f;
    cache.ia[0] = cache.ia[1] = cache.ia[2] = 0;
    cache.ib[0] = cache.ib[1] = cache.ib[2] = 0;
    while (o.toi_iters < L.maxToiIters) {
        const DistOut di = gjk_distance(A, loA, B, loB, cache, L.maxDistIters);
        ++o.toi_iters;
        if (di.iters > o.max_dist_iters) o.max_dist_iters = di.iters;
        if (di.state == DIST_HITMAX) { o.time = timeLo; o.state = TOI_MAX_DIST_ITERS; return o; }
        cache.n = di.s.n;  // Simplex::GetCache (Simplex.hpp:156-159)
        for (int k = 0; k < di.s.n; ++k) { cache.ia[k] = di.s.e[k].iA; cache.ib[k] = di.s.e[k].iB; }
        cache.metric = simplex_metric(di.s.e, di.s.n);
        V2 wA, wB;
        witness_points(di.s, wA, wB);
        const float distSquared = mag2(wB - wA);
        if (distSquared < minTargetSquared) { o.time = timeLo; o.state = TOI_OVERLAPPED; return o; }
        if (distSquared <= maxTargetSquared) { o.time = timeLo; o.state = TOI_TOUCHING; return o; }
        const SepFn fcn = separation_scenario(cache, A, loA, B, loB);
        float timeHi = 1.0f;
        Xf hiA = sweep_xf(sA, timeHi), hiB = sweep_xf(sB, timeHi);
        for (int pb = 0; pb < 254; ++pb) {  // MaxShapeVertices
            const LenIdx hs = find_min_separation(fcn, A, hiA, B, hiB);
            if (hs.dist > maxTarget) { o.time = timeHi; o.state = TOI_SEPARATED; return o; }
            if (hs.dist >= minTarget) {
                if (timeHi == timeLo) { o.time = timeHi; o.state = TOI_SEPARATED; return o; }
                timeLo = timeHi; loA = hiA; loB = hiB;
                break;
            }
            const float loEval = sep_evaluate(fcn, A, loA, B, loB, hs.ia, hs.ib);
            if (loEval <= maxTarget) {
                o.time = timeLo;
                o.state = (loEval < minTarget) ? TOI_BELOW_MIN_TARGET : TOI_TOUCHING;
                return o;
            }
            float a1 = timeLo, a2 = timeHi, s1 = loEval, s2 = hs.dist;
            int roots = 0;
            float t = timeLo;
            for (;;) {
                if (roots == L.maxRootIters) {
                    if (roots > o.max_root_iters) o.max_root_iters = roots;
                    o.time = t; o.state = TOI_MAX_ROOT_ITERS; return o;
                }
                if (nextafterf(a1, a2) >= a2) {
                    if (roots > o.max_root_iters) o.max_root_iters = roots;
                    o.time = t; o.state = TOI_NEXT_AFTER; return o;
                }
                // Secant on odd counts, bisection on even (Math.hpp:92-108)
                t = (roots & 1) ? (a1 + (target - s1) * (a2 - a1) / (s2 - s1)) : ((a1 + a2) / 2.0f);
                ++roots;
                const Xf tA = sweep_xf(sA, t), tB = sweep_xf(sB, t);
                const float sv = sep_evaluate(fcn, A, tA, B, tB, hs.ia, hs.ib);
                if (fabsf(sv - target) <= L.tolerance) {
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

}  // namespace prgpu
