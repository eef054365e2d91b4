// prgpu_csolve.cuh -- the per-constraint contact solver steps, shared by the
// regular phase's sweeps (prgpu_solver.cu) and the time-of-impact islands
// (prgpu_toi.cu).  Each is templated on a body-state accessor BS with vel /
// set_vel / pos / set_pos / mass / writable.
#pragma once

#include "prgpu_collide.cuh"
#include "prgpu_internal.cuh"

namespace prgpu {

// ---- per-constraint solver steps --------------------------------------------

// A contact's manifold as the constraint builders read it from slot storage.
struct ManRec {
    int type, count;
    V2 ln, lp;
    V2 plp[2];
    float pni[2], pti[2];
};
__device__ __forceinline__ ManRec load_manrec(const DW& d, uint32_t slot) {
    ManRec m;
    const uint32_t meta = d.m_meta[slot];
    m.type = (int)(meta & 0xfu);
    m.count = (int)((meta >> 4) & 0xfu);
    const float4 h = d.m_head[slot];
    const float4 q0 = d.m_p0[slot], q1 = d.m_p1[slot];
    m.ln = mk(h.x, h.y); m.lp = mk(h.z, h.w);
    m.plp[0] = mk(q0.x, q0.y); m.plp[1] = mk(q1.x, q1.y);
    m.pni[0] = q0.z; m.pni[1] = q1.z; m.pti[0] = q0.w; m.pti[1] = q1.w;
    return m;
}

// GetWorldManifold (WorldManifold.cpp:111-132) and the VelocityConstraint
// constructor with GetPoint and ComputeK (VelocityConstraint.cpp:38-185) for
// bodies at pA / pB (centre x, y, angle) moving at vA / vB; stored impulses are
// scaled by dtRatio.  Body indices and the island are the caller's to fill in.
__device__ __forceinline__ VC make_contact_vc(const ManRec& m, float4 pA, float4 pB, float4 mA, float4 mB, float4 vA,
                                              float4 vB, float rA, float rB, float2 mat, float dtRatio,
                                              const DConf& c, float tangentSpeed = 0.f) {
    const Xf xfA = get_xf(pA.x, pA.y, pA.z, mk(mA.z, mA.w));
    const Xf xfB = get_xf(pB.x, pB.y, pB.z, mk(mB.z, mB.w));
    const int type = m.type, count = m.count;
    V2 n = mk(0.f, 0.f);
    V2 wpt[2] = {mk(0.f, 0.f), mk(0.f, 0.f)};
    if (type == M_CIRCLES) {
        const V2 a = xform(m.lp, xfA), b = xform(m.plp[0], xfB);
        n = unit_vector(b - a, mk(1.f, 0.f));
        const V2 cA = a + n * rA, cB = b - n * rB;
        wpt[0] = vdiv(cA + cB, 2.0f);
    } else if (type == M_FACEA) {
        n = urotate(m.ln, xfA.q);
        const V2 planePoint = xform(m.lp, xfA);
        for (int i = 0; i < count; ++i) {
            const V2 clip = xform(m.plp[i], xfB);
            const V2 cA = clip + n * (rA - dot(clip - planePoint, n));
            const V2 cB = clip - n * rB;
            wpt[i] = vdiv(cA + cB, 2.0f);
        }
    } else if (type == M_FACEB) {
        const V2 nb = urotate(m.ln, xfB.q);
        const V2 planePoint = xform(m.lp, xfB);
        for (int i = 0; i < count; ++i) {
            const V2 clip = xform(m.plp[i], xfA);
            const V2 cB = clip + nb * (rB - dot(clip - planePoint, nb));
            const V2 cA = clip - nb * rA;
            wpt[i] = vdiv(cA + cB, 2.0f);
        }
        n = -nb;
    }
    VC vc;
    vc.nx = n.x; vc.ny = n.y; vc.friction = mat.x; vc.tangentSpeed = tangentSpeed;
    vc.bA = vc.bB = 0u; vc.island = 0u;
    const float invMass = mA.x + mB.x;
    const V2 tangent = fwdperp(n);
    const V2 velA = mk(vA.x, vA.y), velB = mk(vB.x, vB.y);
    float rr[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
    float nm[2] = {0.f, 0.f}, tm[2] = {0.f, 0.f}, vb[2] = {0.f, 0.f}, ni[2] = {0.f, 0.f}, ti[2] = {0.f, 0.f};
    for (int j = 0; j < count; ++j) {
        const V2 relA = wpt[j] - mk(pA.x, pA.y);
        const V2 relB = wpt[j] - mk(pB.x, pB.y);
        ni[j] = m.pni[j] * dtRatio;
        ti[j] = m.pti[j] * dtRatio;
        {
            const V2 dv = (velB + revperp(relB) * vB.z) - (velA + revperp(relA) * vA.z);
            const float vn = dot(dv, n);
            vb[j] = (vn < -c.velocityThreshold) ? -mat.y * vn : 0.f;
        }
        {
            const float crA = cross(relA, n), crB = cross(relB, n);
            const float value = invMass + mA.y * (crA * crA) + mB.y * (crB * crB);
            nm[j] = (value != 0.f) ? 1.0f / value : 0.f;
        }
        {
            const float crA = cross(relA, tangent), crB = cross(relB, tangent);
            const float value = invMass + mA.y * (crA * crA) + mB.y * (crB * crB);
            tm[j] = (value != 0.f) ? 1.0f / value : 0.f;
        }
        rr[j][0] = relA.x; rr[j][1] = relA.y; rr[j][2] = relB.x; rr[j][3] = relB.y;
    }
    int cnt = count;
    float k00 = 0.f, k11 = 0.f, k01 = 0.f, m00 = 0.f, m11 = 0.f, m01 = 0.f;
    if (c.doBlocksolve && count == 2) {
        const V2 rA0 = mk(rr[0][0], rr[0][1]), rB0 = mk(rr[0][2], rr[0][3]);
        const V2 rA1 = mk(rr[1][0], rr[1][1]), rB1 = mk(rr[1][2], rr[1][3]);
        const float rnA0 = cross(rA0, n), rnB0 = cross(rB0, n);
        const float rnA1 = cross(rA1, n), rnB1 = cross(rB1, n);
        const float kk00 = invMass + mA.y * (rnA0 * rnA0) + mB.y * (rnB0 * rnB0);
        const float kk11 = invMass + mA.y * (rnA1 * rnA1) + mB.y * (rnB1 * rnB1);
        const float kk01 = invMass + (mA.y * rnA0 * rnA1) + (mB.y * rnB0 * rnB1);
        const float k_diff = kk00 * kk11 - kk01 * kk01;
        if (kk00 * kk00 < 1000.0f * k_diff) {
            k00 = kk00; k11 = kk11; k01 = kk01;
            const float cp = cross(mk(kk00, kk01), mk(kk01, kk11));
            if (!almost_zero(cp)) {
                const float inv = 1.0f / cp;
                m00 = kk11 * inv; m01 = -kk01 * inv; m11 = kk00 * inv;
            }
        } else {
            cnt = 1;
        }
    }
    vc.count = (uint32_t)cnt;
    vc.rA0x = rr[0][0]; vc.rA0y = rr[0][1]; vc.rB0x = rr[0][2]; vc.rB0y = rr[0][3];
    vc.nm0 = nm[0]; vc.tm0 = tm[0]; vc.vb0 = vb[0]; vc.ni0 = ni[0]; vc.ti0 = ti[0];
    if (cnt == 2) {
        vc.rA1x = rr[1][0]; vc.rA1y = rr[1][1]; vc.rB1x = rr[1][2]; vc.rB1y = rr[1][3];
        vc.nm1 = nm[1]; vc.tm1 = tm[1]; vc.vb1 = vb[1]; vc.ni1 = ni[1]; vc.ti1 = ti[1];
    } else {
        vc.rA1x = vc.rA1y = vc.rB1x = vc.rB1y = 0.f;
        vc.nm1 = vc.tm1 = vc.vb1 = vc.ni1 = vc.ti1 = 0.f;
    }
    vc.k00 = k00; vc.k11 = k11; vc.k01 = k01; vc.m00 = m00; vc.m11 = m11; vc.m01 = m01;
    return vc;
}

// PositionConstraint (PositionConstraint.hpp) of a contact: its local manifold.
__device__ __forceinline__ PC make_contact_pc(const ManRec& m, float totalRadius, uint32_t bA, uint32_t bB) {
    PC pcs;
    pcs.lnx = m.ln.x; pcs.lny = m.ln.y; pcs.lpx = m.lp.x; pcs.lpy = m.lp.y;
    pcs.p0x = m.plp[0].x; pcs.p0y = m.plp[0].y; pcs.p1x = m.plp[1].x; pcs.p1y = m.plp[1].y;
    pcs.totalRadius = totalRadius;
    pcs.type = (uint32_t)m.type; pcs.count = (uint32_t)m.count; pcs.bA = bA; pcs.bB = bB;
    pcs.island = 0u; pcs.pad0 = pcs.pad1 = 0u;
    return pcs;
}

// WarmStartVelocities (AabbTreeWorld.cpp:227-274).
template <class BS>
__device__ void warm_start(const DW& d, const BS& bs, const VC& vc) {
    const float4 mA = bs.mass(vc.bA), mB = bs.mass(vc.bB);
    const V2 n = mk(vc.nx, vc.ny), t = fwdperp(n);
    float dAx = 0.f, dAy = 0.f, dAw = 0.f, dBx = 0.f, dBy = 0.f, dBw = 0.f;
    for (uint32_t j = 0; j < vc.count; ++j) {
        const float ni = j ? vc.ni1 : vc.ni0, ti = j ? vc.ti1 : vc.ti0;
        const V2 rA = j ? mk(vc.rA1x, vc.rA1y) : mk(vc.rA0x, vc.rA0y);
        const V2 rB = j ? mk(vc.rB1x, vc.rB1y) : mk(vc.rB0x, vc.rB0y);
        const V2 P = n * ni + t * ti;
        const float LA = cross(rA, P), LB = cross(rB, P);
        dAx = dAx - P.x * mA.x; dAy = dAy - P.y * mA.x; dAw = dAw - mA.y * LA;
        dBx = dBx + P.x * mB.x; dBy = dBy + P.y * mB.x; dBw = dBw + mB.y * LB;
    }
    if (bs.writable(vc.bA)) {
        float4 v = bs.vel(vc.bA);
        v.x = v.x + dAx; v.y = v.y + dAy; v.z = v.z + dAw;
        bs.set_vel(vc.bA, v);
    }
    if (bs.writable(vc.bB)) {
        float4 v = bs.vel(vc.bB);
        v.x = v.x + dBx; v.y = v.y + dBy; v.z = v.z + dBw;
        bs.set_vel(vc.bB, v);
    }
}

__device__ __forceinline__ V2 rel_vel(float4 va, V2 rA, float4 vb, V2 rB) {
    return (mk(vb.x, vb.y) + revperp(rB) * vb.z) - (mk(va.x, va.y) + revperp(rA) * va.z);
}

// GaussSeidel::SolveVelocityConstraint (ContactSolver.cpp:245-492).
// kTrack: also return the largest impulse change, as the reference's solver
// reports it (|increment| per sequential point, |new impulse| per block update);
// the time-of-impact loop's early exit reads it.
template <class BS, bool kTrack = false>
__device__ float solve_contact_velocity(const DW& d, const BS& bs, VC& vc) {
    float mx = 0.f;
    const float4 mA = bs.mass(vc.bA), mB = bs.mass(vc.bB);
    float4 vA = bs.vel(vc.bA), vB = bs.vel(vc.bB);
    const V2 n = mk(vc.nx, vc.ny);
    const V2 rA0 = mk(vc.rA0x, vc.rA0y), rB0 = mk(vc.rB0x, vc.rB0y);
    const V2 rA1 = mk(vc.rA1x, vc.rA1y), rB1 = mk(vc.rB1x, vc.rB1y);
    // tangent then normal, point 1 before point 0 (ContactSolver.cpp:337-454)
    for (int pass = 0; pass < 2; ++pass) {
        const bool tangentPass = pass == 0;
        if (!tangentPass && vc.count == 2 && !(vc.k00 == 0.f && vc.k11 == 0.f && vc.k01 == 0.f)) {
            // BlockSolveNormalConstraint (ContactSolver.cpp:245-335)
            const V2 dv0 = rel_vel(vA, rA0, vB, rB0), dv1 = rel_vel(vA, rA1, vB, rB1);
            const float vn0 = dot(dv0, n), vn1 = dot(dv1, n);
            const float b0 = vn0 - vc.vb0, b1 = vn1 - vc.vb1;
            const float a0 = vc.ni0, a1 = vc.ni1;
            float Kx0 = 0.f; Kx0 += vc.k00 * a0; Kx0 += vc.k01 * a1;
            float Kx1 = 0.f; Kx1 += vc.k01 * a0; Kx1 += vc.k11 * a1;
            const float bp0 = b0 - Kx0, bp1 = b1 - Kx1;
            float x0 = 0.f, x1 = 0.f;
            bool apply = false;
            {
                float q0 = 0.f; q0 += vc.m00 * bp0; q0 += vc.m01 * bp1;
                float q1 = 0.f; q1 += vc.m01 * bp0; q1 += vc.m11 * bp1;
                x0 = -q0; x1 = -q1;
                apply = (x0 >= 0.f && x1 >= 0.f);
            }
            if (!apply) {
                x0 = -vc.nm0 * bp0; x1 = 0.f;
                const float vn2 = vc.k01 * x0 + bp1;
                apply = (x0 >= 0.f && vn2 >= 0.f);
            }
            if (!apply) {
                x0 = 0.f; x1 = -vc.nm1 * bp1;
                const float vn1b = vc.k01 * x1 + bp0;
                apply = (x1 >= 0.f && vn1b >= 0.f);
            }
            if (!apply) {
                x0 = 0.f; x1 = 0.f;
                apply = (bp0 >= 0.f && bp1 >= 0.f);
            }
            if (apply) {
                const float d0 = x0 - vc.ni0, d1 = x1 - vc.ni1;
                const V2 P0 = n * d0, P1 = n * d1;
                const V2 P = P0 + P1;
                const float LA = cross(rA0, P0) + cross(rA1, P1);
                const float LB = cross(rB0, P0) + cross(rB1, P1);
                vA.x = vA.x + (-(P.x * mA.x)); vA.y = vA.y + (-(P.y * mA.x)); vA.z = vA.z + (-(mA.y * LA));
                vB.x = vB.x + P.x * mB.x; vB.y = vB.y + P.y * mB.x; vB.z = vB.z + mB.y * LB;
                vc.ni0 = x0; vc.ni1 = x1;
                if (kTrack) mx = maxf_(mx, maxf_(fabsf(x0), fabsf(x1)));
            }
            continue;
        }
        const V2 dir = tangentPass ? fwdperp(n) : n;
        for (int k = (vc.count == 2) ? 1 : 0; k >= 0; --k) {
            const V2 rA = k ? rA1 : rA0, rB = k ? rB1 : rB0;
            const V2 cv = rel_vel(vA, rA, vB, rB);
            float oldImp, newImp;
            if (tangentPass) {
                const float dvel = vc.tangentSpeed - dot(cv, dir);
                const float lambda = (k ? vc.tm1 : vc.tm0) * dvel;
                const float maxImp = vc.friction * (k ? vc.ni1 : vc.ni0);
                oldImp = k ? vc.ti1 : vc.ti0;
                newImp = clampf_(oldImp + lambda, -maxImp, maxImp);
            } else {
                const float dvel = dot(cv, dir);
                const float lambda = (k ? vc.nm1 : vc.nm0) * ((k ? vc.vb1 : vc.vb0) - dvel);
                oldImp = k ? vc.ni1 : vc.ni0;
                newImp = maxf_(oldImp + lambda, 0.f);
            }
            const float inc = newImp - oldImp;
            const V2 P = dir * inc;
            const float LA = cross(rA, P), LB = cross(rB, P);
            vA.x = vA.x - P.x * mA.x; vA.y = vA.y - P.y * mA.x; vA.z = vA.z - mA.y * LA;
            vB.x = vB.x + P.x * mB.x; vB.y = vB.y + P.y * mB.x; vB.z = vB.z + mB.y * LB;
            if (kTrack) mx = maxf_(mx, fabsf(inc));
            const float nv = oldImp + inc;
            if (tangentPass) { if (k) vc.ti1 = nv; else vc.ti0 = nv; }
            else { if (k) vc.ni1 = nv; else vc.ni0 = nv; }
        }
    }
    if (bs.writable(vc.bA)) bs.set_vel(vc.bA, vA);
    if (bs.writable(vc.bB)) bs.set_vel(vc.bB, vB);
    return mx;
}

struct PSM {
    V2 n, pt;
    float sep;
};
// GetPSM (PositionSolverManifold.cpp:103-121).
__device__ __forceinline__ PSM get_psm(const PC& pc, int idx, Xf xfA, Xf xfB) {
    PSM r;
    const V2 lp = mk(pc.lpx, pc.lpy), ln = mk(pc.lnx, pc.lny);
    const V2 plp = idx ? mk(pc.p1x, pc.p1y) : mk(pc.p0x, pc.p0y);
    if (pc.type == M_CIRCLES) {
        const V2 a = xform(lp, xfA), b = xform(plp, xfB);
        const V2 delta = b - a;
        r.n = unit_vector(delta, mk(0.f, 0.f));
        r.pt = vdiv(a + b, 2.0f);
        r.sep = dot(delta, r.n);
    } else if (pc.type == M_FACEA) {
        const V2 planePoint = xform(lp, xfA);
        r.n = urotate(ln, xfA.q);
        r.pt = xform(plp, xfB);
        r.sep = dot(r.pt - planePoint, r.n);
    } else {
        const V2 planePoint = xform(lp, xfB);
        const V2 nb = urotate(ln, xfB.q);
        r.pt = xform(plp, xfA);
        r.sep = dot(r.pt - planePoint, nb);
        r.n = -nb;
    }
    return r;
}

struct PosSol {
    float ax, ay, aa, bx, by, ba, sep;
};
// solver_fn of GaussSeidel::SolvePositionConstraint (ContactSolver.cpp:521-551).
// `rate`: regResolutionRate in the regular phase, toiResolutionRate in TOI islands.
__device__ __forceinline__ PosSol pos_solver_fn(const PSM& psm, V2 pA, V2 pB, float4 mA, float4 mB, float totalRadius,
                                                const DConf& c, float rate) {
    const float invMassTotal = mA.x + mB.x;
    const float separation = psm.sep - totalRadius;
    const V2 rA = psm.pt - pA, rB = psm.pt - pB;
    const float cA = cross(rA, psm.n), cB = cross(rB, psm.n);
    const float K = invMassTotal + mA.y * (cA * cA) + mB.y * (cB * cB);
    const float C = -clampf_(rate * (separation + c.linearSlop), -c.maxLinearCorrection, 0.f);
    const V2 P = vdiv(psm.n * C, K);
    const float LA = cross(rA, P), LB = cross(rB, P);
    PosSol s;
    s.ax = -(P.x * mA.x); s.ay = -(P.y * mA.x); s.aa = -(mA.y * LA);
    s.bx = P.x * mB.x; s.by = P.y * mB.x; s.ba = +(mB.y * LB);
    s.sep = separation;
    return s;
}

// GaussSeidel::SolvePositionConstraint (ContactSolver.cpp:494-643); returns the
// separation the reference reports for this constraint.
template <class BS>
__device__ float solve_contact_position(const DW& d, const BS& bs, const PC& pc, float rate) {
    const DConf& c = *d.conf;
    const float4 mA = bs.mass(pc.bA), mB = bs.mass(pc.bB);
    float4 pA = bs.pos(pc.bA), pB = bs.pos(pc.bB);
    const V2 lcA = mk(mA.z, mA.w), lcB = mk(mB.z, mB.w);
    float minSep = __int_as_float(0x7f800000);
    auto add = [](float4& p, float x, float y, float a) { p.x = p.x + x; p.y = p.y + y; p.z = p.z + a; };
    if (pc.count == 1u) {
        const PSM psm0 = get_psm(pc, 0, get_xf(pA.x, pA.y, pA.z, lcA), get_xf(pB.x, pB.y, pB.z, lcB));
        const PosSol s = pos_solver_fn(psm0, mk(pA.x, pA.y), mk(pB.x, pB.y), mA, mB, pc.totalRadius, c, rate);
        add(pA, s.ax, s.ay, s.aa); add(pB, s.bx, s.by, s.ba);
        minSep = 0.f + s.sep;
    } else if (pc.count == 2u) {
        const Xf xfA = get_xf(pA.x, pA.y, pA.z, lcA), xfB = get_xf(pB.x, pB.y, pB.z, lcB);
        const PSM psm0 = get_psm(pc, 0, xfA, xfB);
        const PSM psm1 = get_psm(pc, 1, xfA, xfB);
        if (almost_equal(psm0.sep, psm1.sep)) {
            const PosSol s0 = pos_solver_fn(psm0, mk(pA.x, pA.y), mk(pB.x, pB.y), mA, mB, pc.totalRadius, c, rate);
            const PosSol s1 = pos_solver_fn(psm1, mk(pA.x, pA.y), mk(pB.x, pB.y), mA, mB, pc.totalRadius, c, rate);
            add(pA, s0.ax, s0.ay, s0.aa); add(pA, s1.ax, s1.ay, s1.aa);
            add(pB, s0.bx, s0.by, s0.ba); add(pB, s1.bx, s1.by, s1.ba);
            minSep = s0.sep;
        } else if (psm0.sep < psm1.sep || psm1.sep < psm0.sep) {
            const int first = (psm0.sep < psm1.sep) ? 0 : 1;
            const PSM pf = first ? psm1 : psm0;
            const PosSol s0 = pos_solver_fn(pf, mk(pA.x, pA.y), mk(pB.x, pB.y), mA, mB, pc.totalRadius, c, rate);
            add(pA, s0.ax, s0.ay, s0.aa); add(pB, s0.bx, s0.by, s0.ba);
            const PSM ps = get_psm(pc, 1 - first, get_xf(pA.x, pA.y, pA.z, lcA), get_xf(pB.x, pB.y, pB.z, lcB));
            const PosSol s1 = pos_solver_fn(ps, mk(pA.x, pA.y), mk(pB.x, pB.y), mA, mB, pc.totalRadius, c, rate);
            add(pA, s1.ax, s1.ay, s1.aa); add(pB, s1.bx, s1.by, s1.ba);
            minSep = s0.sep;
        }
    }
    if (bs.writable(pc.bA)) bs.set_pos(pc.bA, pA);
    if (bs.writable(pc.bB)) bs.set_pos(pc.bB, pB);
    return minSep;
}

}  // namespace prgpu
