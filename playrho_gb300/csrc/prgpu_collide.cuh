// prgpu_collide.cuh -- narrowphase: CollideShapes and the manifold it produces.
//
// Restates Manifold.cpp:61-438 and ShapeSeparation.cpp:36-124 for the shape
// kinds the world step supports (disk = 1 vertex, edge = 2, polygon = 3..16).
// Contact features are packed as typeA | indexA << 8 | typeB << 16 | indexB << 24.
#pragma once

#include "prgpu_math.cuh"

namespace prgpu {

constexpr int kMaxVerts = 16;
constexpr unsigned kInvalidV = 255u;
enum { M_UNSET = 0, M_CIRCLES = 1, M_FACEA = 2, M_FACEB = 3 };
enum { CF_VERTEX = 0u, CF_FACE = 1u };

PR_HD uint32_t cf_pack(unsigned tA, unsigned iA, unsigned tB, unsigned iB) {
    return (tA & 0xffu) | ((iA & 0xffu) << 8) | ((tB & 0xffu) << 16) | ((iB & 0xffu) << 24);
}
// Flip (ContactFeature.hpp:114-117).
PR_HD uint32_t cf_flip(uint32_t c) { return ((c >> 16) & 0xffffu) | ((c & 0xffffu) << 16); }

// DistanceProxy (DistanceProxy.hpp) as a view of the shape's vertex records
// in device memory: vertex xy and outward edge normal zw, count <= kMaxVerts.
// The collision routines read the vertices where they lie rather than copying
// them into per-thread (local) memory.
struct Proxy {
    int count;
    float r;
    const float4* vn;
    PR_HD V2 vtx(int i) const { const float4 q = vn[i]; return mk(q.x, q.y); }
    PR_HD V2 nrm(int i) const { const float4 q = vn[i]; return mk(q.z, q.w); }
};

struct Man {
    int type;
    int count;
    V2 ln, lp;
    V2 plp[2];
    uint32_t cf[2];
    float ni[2], ti[2];
};

PR_HD Man man_empty() {
    Man m;
    m.type = M_UNSET; m.count = 0;
    m.ln = mk(0.f, 0.f); m.lp = mk(0.f, 0.f);
    m.plp[0] = m.plp[1] = mk(0.f, 0.f);
    m.cf[0] = m.cf[1] = cf_pack(CF_VERTEX, kInvalidV, CF_VERTEX, kInvalidV);
    m.ni[0] = m.ni[1] = m.ti[0] = m.ti[1] = 0.f;
    return m;
}
// Manifold::GetForCircles (Manifold.hpp:168-171).
PR_HD Man man_circles(V2 vA, unsigned iA, V2 vB, unsigned iB) {
    Man m = man_empty();
    m.type = M_CIRCLES; m.lp = vA; m.count = 1;
    m.plp[0] = vB; m.cf[0] = cf_pack(CF_VERTEX, iA, CF_VERTEX, iB);
    return m;
}
PR_HD Man man_face(int type, V2 ln, V2 lp) {
    Man m = man_empty();
    m.type = type; m.ln = ln; m.lp = lp;
    return m;
}
PR_HD void man_add(Man& m, V2 lp, uint32_t cf) {
    m.plp[m.count] = lp; m.cf[m.count] = cf; m.ni[m.count] = 0.f; m.ti[m.count] = 0.f;
    ++m.count;
}

struct ClipV {
    V2 v;
    uint32_t cf;
};

// ClipSegmentToLine (Manifold.cpp:61-102).
PR_HD int clip_segment(const ClipV* vin, int nin, V2 normal, float offset, unsigned indexA, ClipV* vout) {
    int n = 0;
    if (nin == 2) {
        const float d0 = dot(normal, vin[0].v) - offset;
        const float d1 = dot(normal, vin[1].v) - offset;
        if (d0 <= 0.f || almost_zero(d0)) vout[n++] = vin[0];
        if (d1 <= 0.f || almost_zero(d1)) vout[n++] = vin[1];
        if (n < 2 && (signbit(d0) != signbit(d1))) {
            const float interp = d0 / (d0 - d1);
            ClipV cv;
            cv.v = vin[0].v + (vin[1].v - vin[0].v) * interp;
            cv.cf = cf_pack(CF_VERTEX, indexA, CF_FACE, (vin[0].cf >> 24) & 0xffu);
            vout[n++] = cv;
        }
    }
    return n;
}

// GetMinSeparationInfo (ShapeSeparation.cpp:36-58).
PR_HD float min_sep_info(V2 origin, V2 dir, const V2* verts, int n, unsigned& first, unsigned& second) {
    float minSep = PR_INF;
    first = kInvalidV; second = kInvalidV;
    for (int i = 0; i < n; ++i) {
        const float s = dot(dir, verts[i] - origin);
        if (minSep > s) { minSep = s; first = (unsigned)i; second = kInvalidV; }
        else if (minSep == s) { second = (unsigned)i; }
    }
    return minSep;
}

// The same over a shape's own vertices.
PR_HD float min_sep_info(V2 origin, V2 dir, const Proxy& p, unsigned& first, unsigned& second) {
    float minSep = PR_INF;
    first = kInvalidV; second = kInvalidV;
    for (int i = 0; i < p.count; ++i) {
        const float s = dot(dir, p.vtx(i) - origin);
        if (minSep > s) { minSep = s; first = (unsigned)i; second = kInvalidV; }
        else if (minSep == s) { second = (unsigned)i; }
    }
    return minSep;
}

struct SepInfo {
    float distance;
    unsigned firstShape, second0, second1;
};

// GetMaxSeparation4x4 (ShapeSeparation.cpp:62-101).
PR_HD SepInfo max_sep_4x4(const Proxy& p1, Xf xf1, const Proxy& p2, Xf xf2) {
    SepInfo r; r.distance = -PR_INF; r.firstShape = kInvalidV; r.second0 = kInvalidV; r.second1 = kInvalidV;
    const Xf xf = mult(xf1, xf2);
    V2 verts[4];
    for (int i = 0; i < 4; ++i) verts[i] = xform(p2.vtx(i), xf);
    for (int i = 0; i < 4; ++i) {
        unsigned f, s;
        const float d = min_sep_info(p1.vtx(i), p1.nrm(i), verts, 4, f, s);
        if (r.distance < d) { r.distance = d; r.second0 = f; r.second1 = s; r.firstShape = (unsigned)i; }
    }
    return r;
}

// GetMaxSeparation (ShapeSeparation.cpp:103-124).
PR_HD SepInfo max_sep(const Proxy& p1, Xf xf1, const Proxy& p2, Xf xf2) {
    SepInfo r; r.distance = -PR_INF; r.firstShape = kInvalidV; r.second0 = kInvalidV; r.second1 = kInvalidV;
    const Xf xf = mult(xf2, xf1);
    for (int i = 0; i < p1.count; ++i) {
        const V2 origin = xform(p1.vtx(i), xf);
        const V2 normal = rotate(p1.nrm(i), xf.q);
        unsigned f, s;
        const float d = min_sep_info(origin, normal, p2, f, s);
        if (r.distance < d) { r.distance = d; r.second0 = f; r.second1 = s; r.firstShape = (unsigned)i; }
    }
    return r;
}

// GetMostAntiParallelEdge (Manifold.cpp:124-141).
PR_HD void most_anti_parallel_edge(V2 n0, Xf xf0, const Proxy& s1, Xf xf1, unsigned first, unsigned second,
                                   unsigned& e0, unsigned& e1) {
    if (second == kInvalidV) {
        const V2 normal = invrotate(rotate(n0, xf0.q), xf1.q);
        const unsigned count = (unsigned)s1.count;
        const unsigned prev = (first == 0u) ? count - 1u : first - 1u;
        const float prevDot = dot(normal, s1.nrm(prev));
        const float currDot = dot(normal, s1.nrm(first));
        if (prevDot < currDot) { e0 = prev; e1 = first; }
        else { e0 = first; e1 = (first + 1u) % count; }
        return;
    }
    if ((second > first) && ((first + 1u) == second)) { e0 = first; e1 = second; }
    else { e0 = second; e1 = first; }
}

// The features a polygon-polygon manifold was built from: the reference face
// idx0 of s0 (shape B of the contact when flipped) and the incident edge
// (e1f, e1s) of s1.  The adjoint differentiates the clipped points through them.
struct PolyPick {
    unsigned flipped, idx0, e1f, e1s;
};

// GetManifold for two polygons (Manifold.cpp:162-291).
PR_HD Man manifold_poly(bool flipped, const Proxy& s0, Xf xf0, unsigned idx0, const Proxy& s1, Xf xf1,
                        unsigned sec0, unsigned sec1, float maxCirclesRatio, PolyPick* pick = nullptr) {
    const float r0 = s0.r, r1 = s1.r;
    const float totalRadius = r0 + r1;
    const unsigned idx0Next = (idx0 + 1u) % (unsigned)s0.count;
    const V2 s0_rel_v0 = s0.vtx(idx0);
    const V2 s0_rel_v1 = s0.vtx(idx0Next);
    const V2 s0_abs_v0 = xform(s0_rel_v0, xf0);
    const V2 s0_abs_v1 = xform(s0_rel_v1, xf0);
    const float s0_len_edge0 = mag2(s0_rel_v1 - s0_rel_v0);
    const V2 s0_rel_n0 = s0.nrm(idx0);
    const V2 s0_rel_e0_dir = revperp(s0_rel_n0);
    unsigned e1f, e1s;
    most_anti_parallel_edge(s0_rel_n0, xf0, s1, xf1, sec0, sec1, e1f, e1s);
    if (pick) { pick->flipped = flipped ? 1u : 0u; pick->idx0 = idx0; pick->e1f = e1f; pick->e1s = e1s; }
    const V2 s1_rel_v0 = s1.vtx(e1f);
    const V2 s1_abs_v0 = xform(s1_rel_v0, xf1);
    const V2 s1_rel_v1 = s1.vtx(e1s);
    const V2 s1_abs_v1 = xform(s1_rel_v1, xf1);
    {
        const V2 s0_abs_e0_dir = rotate(s0_rel_e0_dir, xf0.q);
        ClipV ie[2];
        ie[0].v = s1_abs_v0; ie[0].cf = cf_pack(CF_FACE, idx0, CF_VERTEX, e1f);
        ie[1].v = s1_abs_v1; ie[1].cf = cf_pack(CF_FACE, idx0, CF_VERTEX, e1s);
        const float dp_v0_e0 = -dot(s0_abs_e0_dir, s0_abs_v0);
        const float dp_v1_e0 = +dot(s0_abs_e0_dir, s0_abs_v1);
        ClipV pts[2], cps[2];
        const int np = clip_segment(ie, 2, -s0_abs_e0_dir, dp_v0_e0, idx0, pts);
        const int nc = clip_segment(pts, np, s0_abs_e0_dir, dp_v1_e0, idx0Next, cps);
        if (nc == 2) {
            const V2 abs_normal = fwdperp(s0_abs_e0_dir);
            const V2 rel_midpoint = vdiv(s0_rel_v0 + s0_rel_v1, 2.0f);
            const float abs_offset = dot(abs_normal, s0_abs_v0);
            const V2 normal = fwdperp(s0_rel_e0_dir);
            Man m = man_face(flipped ? M_FACEB : M_FACEA, normal, rel_midpoint);
            for (int k = 0; k < 2; ++k) {
                if ((dot(abs_normal, cps[k].v) - abs_offset) <= totalRadius) {
                    man_add(m, invxform(cps[k].v, xf1), flipped ? cf_flip(cps[k].cf) : cps[k].cf);
                }
            }
            if (m.count > 0) return m;
        }
    }
    const float totalRadiusSquared = totalRadius * totalRadius;
    const float mcr = maxCirclesRatio * r0;
    const bool mustUseFace = s0_len_edge0 > (mcr * mcr);
    const V2 fn = fwdperp(s0_rel_e0_dir);
    for (int k = 0; k < 4; ++k) {
        const V2 a_rel = (k == 0 || k == 2) ? s0_rel_v0 : s0_rel_v1;
        const V2 a_abs = (k == 0 || k == 2) ? s0_abs_v0 : s0_abs_v1;
        const unsigned a_idx = (k == 0 || k == 2) ? idx0 : idx0Next;
        const V2 b_rel = (k == 0 || k == 3) ? s1_rel_v0 : s1_rel_v1;
        const V2 b_abs = (k == 0 || k == 3) ? s1_abs_v0 : s1_abs_v1;
        const unsigned b_idx = (k == 0 || k == 3) ? e1f : e1s;
        if (mag2(a_abs - b_abs) <= totalRadiusSquared) {
            if (mustUseFace) {
                Man m = man_face(flipped ? M_FACEB : M_FACEA, fn, a_rel);
                man_add(m, b_rel, flipped ? cf_pack(CF_VERTEX, b_idx, CF_FACE, a_idx)
                                          : cf_pack(CF_FACE, a_idx, CF_VERTEX, b_idx));
                return m;
            }
            return !flipped ? man_circles(a_rel, a_idx, b_rel, b_idx) : man_circles(b_rel, b_idx, a_rel, a_idx);
        }
    }
    return man_empty();
}

// GetManifold for polygon vs circle (Manifold.cpp:293-372).
PR_HD Man manifold_circle(bool flipped, float totalRadius, const Proxy& shape, Xf sxf, V2 point, Xf xfm) {
    const int vc = shape.count;
    const V2 cLocal = invxform(xform(point, xfm), sxf);
    unsigned indexOfMax = 0;
    float maxSeparation = -3.40282347e+38f;
    for (int i = 0; i < vc; ++i) {
        const float s = dot(shape.nrm(i), cLocal - shape.vtx(i));
        if (s > totalRadius) return man_empty();
        if (maxSeparation < s) { maxSeparation = s; indexOfMax = (unsigned)i; }
    }
    const unsigned indexOfMax2 = (indexOfMax + 1u) % (unsigned)vc;
    const V2 v1 = shape.vtx(indexOfMax);
    const V2 v2 = shape.vtx(indexOfMax2);
    const uint32_t cfFace = flipped ? cf_pack(CF_VERTEX, 0, CF_FACE, indexOfMax) : cf_pack(CF_FACE, indexOfMax, CF_VERTEX, 0);
    if (maxSeparation < 0.f) {
        Man m = man_face(flipped ? M_FACEB : M_FACEA, shape.nrm(indexOfMax), vdiv(v1 + v2, 2.0f));
        man_add(m, point, cfFace);
        return m;
    }
    const V2 cLocalV1 = cLocal - v1;
    if (dot(cLocalV1, v2 - v1) <= 0.f) {
        if (mag2(cLocalV1) > totalRadius * totalRadius) return man_empty();
        return !flipped ? man_circles(v1, indexOfMax, point, 0) : man_circles(point, 0, v1, indexOfMax);
    }
    const V2 cLocalV2 = cLocal - v2;
    if (dot(cLocalV2, v1 - v2) <= 0.f) {
        if (mag2(cLocalV2) > totalRadius * totalRadius) return man_empty();
        return !flipped ? man_circles(v2, indexOfMax2, point, 0) : man_circles(point, 0, v2, indexOfMax2);
    }
    const V2 faceCenter = vdiv(v1 + v2, 2.0f);
    if (dot(cLocal - faceCenter, shape.nrm(indexOfMax)) > totalRadius) return man_empty();
    Man m = man_face(flipped ? M_FACEB : M_FACEA, shape.nrm(indexOfMax), faceCenter);
    man_add(m, point, cfFace);
    return m;
}

// CollideShapes (Manifold.cpp:393-438).
PR_HD Man collide_shapes(const Proxy& A, Xf xfA, const Proxy& B, Xf xfB, float linearSlop, float maxCirclesRatio,
                         PolyPick* pick = nullptr) {
    const float totalRadius = A.r + B.r;
    if (A.count == 1 && B.count == 1) {
        const V2 pA = xform(A.vtx(0), xfA);
        const V2 pB = xform(B.vtx(0), xfB);
        const float lenSq = mag2(pB - pA);
        const float totSq = totalRadius * totalRadius;
        if (lenSq > totSq) return man_empty();
        return man_circles(A.vtx(0), 0, B.vtx(0), 0);
    }
    if (A.count == 1) return manifold_circle(true, totalRadius, B, xfB, A.vtx(0), xfA);
    if (B.count == 1) return manifold_circle(false, totalRadius, A, xfA, B.vtx(0), xfB);
    const bool do4x4 = (A.count == 4) && (B.count == 4);
    const SepInfo sa = do4x4 ? max_sep_4x4(A, xfA, B, xfB) : max_sep(A, xfA, B, xfB);
    if (sa.distance > totalRadius) return man_empty();
    const SepInfo sb = do4x4 ? max_sep_4x4(B, xfB, A, xfA) : max_sep(B, xfB, A, xfA);
    if (sb.distance > totalRadius) return man_empty();
    // Non-finite transforms leave no separating feature; report no contact instead
    // of indexing with the invalid-vertex marker.
    if (sa.firstShape >= (unsigned)A.count || sa.second0 >= (unsigned)B.count ||
        sb.firstShape >= (unsigned)B.count || sb.second0 >= (unsigned)A.count ||
        (sa.second1 != kInvalidV && sa.second1 >= (unsigned)B.count) ||
        (sb.second1 != kInvalidV && sb.second1 >= (unsigned)A.count))
        return man_empty();
    const float k_tol = linearSlop / 10.0f;
    return (sb.distance > (sa.distance + k_tol))
               ? manifold_poly(true, B, xfB, sb.firstShape, A, xfA, sb.second0, sb.second1, maxCirclesRatio, pick)
               : manifold_poly(false, A, xfA, sa.firstShape, B, xfB, sa.second0, sa.second1, maxCirclesRatio, pick);
}

// Warm-start transfer of AabbTreeWorld::Update (AabbTreeWorld.cpp:2644-2678):
// impulses follow matching contact features, else the nearest old point.
// src (optional) receives, for each new point, the old point its impulses came
// from (-1: none).
PR_HD void transfer_impulses(Man& nm, const Man& old, int* src = nullptr) {
    bool found[2] = {false, nm.count < 2};
    int from[2] = {-1, -1};
    for (int i = 0; i < nm.count; ++i) {
        for (int j = 0; j < old.count; ++j) {
            if (nm.cf[i] == old.cf[j]) {
                found[i] = true;
                nm.ni[i] = old.ni[j]; nm.ti[i] = old.ti[j];
                from[i] = j;
                break;
            }
        }
    }
    for (int i = 0; i < nm.count; ++i) {
        if (!found[i]) {
            float least = PR_INF;
            for (int j = 0; j < old.count; ++j) {
                const float sq = mag2(old.plp[j] - nm.plp[i]);
                if (least > sq) { least = sq; nm.ni[i] = old.ni[j]; nm.ti[i] = old.ti[j]; from[i] = j; }
            }
        }
    }
    if (src) { src[0] = from[0]; src[1] = from[1]; }
}

}  // namespace prgpu
