// prgpu_diff.cuh -- differentiable restatement of the per-contact pieces of the
// regular step, for the adjoint (StepAdjoint) and the FP64 tangent.
//
// Each piece is written once, templated on its scalar type T, in exactly the
// operation order of the forward kernels (prgpu_solver.cu), so that
//   T = float  recomputes the forward's values bit for bit (a replay check),
//   T = Tan    carries an FP64 tangent along the forward's float values
//              (forward-mode: the tangent kernel).
// The reverse mode is written out by hand for each piece (*_vjp, in float): the
// adjoint kernels' local vector-Jacobian products, which the dot-product test
// checks against the tangent.
// Branches (clamps, block-solver cases, the position solver's point order,
// conditioning of K, vb's restitution threshold) are taken on the float values,
// so they are those of the forward pass: the derivative is that of the forward
// map with its active branches frozen.
#pragma once

#include "prgpu_collide.cuh"
#include "prgpu_internal.cuh"

namespace prgpu {
namespace diff {

// ---- scalar types ---------------------------------------------------------------
// value (float) with an FP64 tangent
struct Tan {
    float v;
    double d;
};

__device__ __forceinline__ float val(float x) { return x; }
__device__ __forceinline__ float val(const Tan& x) { return x.v; }

template <class T> __device__ __forceinline__ T C(float c);
template <> __device__ __forceinline__ float C<float>(float c) { return c; }
template <> __device__ __forceinline__ Tan C<Tan>(float c) { return Tan{c, 0.0}; }

__device__ __forceinline__ Tan operator+(const Tan& a, const Tan& b) { return Tan{a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Tan operator-(const Tan& a, const Tan& b) { return Tan{a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Tan operator*(const Tan& a, const Tan& b) {
    return Tan{a.v * b.v, a.d * (double)b.v + (double)a.v * b.d};
}
__device__ __forceinline__ Tan operator/(const Tan& a, const Tan& b) {
    const double bv = b.v;
    return Tan{a.v / b.v, (a.d * bv - (double)a.v * b.d) / (bv * bv)};
}
__device__ __forceinline__ Tan operator-(const Tan& a) { return Tan{-a.v, -a.d}; }
__device__ __forceinline__ Tan sqrt_(const Tan& a) {
    const float r = sqrtf(a.v);
    return Tan{r, a.d * 0.5 / (double)r};
}
__device__ __forceinline__ Tan hypot_(const Tan& a, const Tan& b) {
    const float h = hypotf(a.v, b.v);
    return Tan{h, ((double)a.v * a.d + (double)b.v * b.d) / h};
}
__device__ __forceinline__ void sincos_(const Tan& a, Tan& s, Tan& c) {
    float sv, cv;
    sincosf(a.v, &sv, &cv);
    s = Tan{sv, (double)cv * a.d};
    c = Tan{cv, -(double)sv * a.d};
}

__device__ __forceinline__ float sqrt_(float a) { return sqrtf(a); }
__device__ __forceinline__ float hypot_(float a, float b) { return hypotf(a, b); }
__device__ __forceinline__ void sincos_(float a, float& s, float& c) { sincosf(a, &s, &c); }

// mixed operands: a float is a constant
template <class T> __device__ __forceinline__ T operator+(const T& a, float b) { return a + C<T>(b); }
template <class T> __device__ __forceinline__ T operator+(float a, const T& b) { return C<T>(a) + b; }
template <class T> __device__ __forceinline__ T operator-(const T& a, float b) { return a - C<T>(b); }
template <class T> __device__ __forceinline__ T operator-(float a, const T& b) { return C<T>(a) - b; }
template <class T> __device__ __forceinline__ T operator*(const T& a, float b) { return a * C<T>(b); }
template <class T> __device__ __forceinline__ T operator*(float a, const T& b) { return C<T>(a) * b; }
template <class T> __device__ __forceinline__ T operator/(const T& a, float b) { return a / C<T>(b); }
template <class T> __device__ __forceinline__ T operator/(float a, const T& b) { return C<T>(a) / b; }

// ---- 2-D vectors (operation order of prgpu_math.cuh) -----------------------------
template <class T>
struct V {
    T x, y;
};
template <class T> __device__ __forceinline__ V<T> mkv(T x, T y) { return V<T>{x, y}; }
template <class T> __device__ __forceinline__ V<T> cv(float x, float y) { return V<T>{C<T>(x), C<T>(y)}; }
template <class T> __device__ __forceinline__ V<T> add(const V<T>& a, const V<T>& b) { return {a.x + b.x, a.y + b.y}; }
template <class T> __device__ __forceinline__ V<T> sub(const V<T>& a, const V<T>& b) { return {a.x - b.x, a.y - b.y}; }
template <class T> __device__ __forceinline__ V<T> neg(const V<T>& a) { return {-a.x, -a.y}; }
template <class T> __device__ __forceinline__ V<T> scale(const V<T>& a, const T& s) { return {a.x * s, a.y * s}; }
template <class T> __device__ __forceinline__ V<T> vdivt(const V<T>& a, float s) {
    const float inv = 1.0f / s;
    return {a.x * inv, a.y * inv};
}
template <class T> __device__ __forceinline__ T dott(const V<T>& a, const V<T>& b) {
    T r = C<T>(0.0f);
    r = r + a.x * b.x;
    r = r + a.y * b.y;
    return r;
}
template <class T> __device__ __forceinline__ T crosst(const V<T>& a, const V<T>& b) {
    const T m = a.x * b.y;
    const T s = a.y * b.x;
    return m - s;
}
template <class T> __device__ __forceinline__ V<T> revperpt(const V<T>& a) { return {-a.y, a.x}; }
template <class T> __device__ __forceinline__ V<T> fwdperpt(const V<T>& a) { return {a.y, -a.x}; }
template <class T> __device__ __forceinline__ V<T> rotatet(const V<T>& v, const V<T>& q) {
    return {(q.x * v.x) - (q.y * v.y), (q.y * v.x) + (q.x * v.y)};
}
template <class T> __device__ __forceinline__ V<T> urotatet(const V<T>& u, const V<T>& a) {
    return {u.x * a.x - u.y * a.y, u.y * a.x + u.x * a.y};
}
template <class T>
struct XfT {
    V<T> p, q;
};
template <class T> __device__ __forceinline__ V<T> xformt(const V<T>& v, const XfT<T>& t) {
    return add(rotatet(v, t.q), t.p);
}
// GetTransformation(Position, localCenter)
template <class T> __device__ __forceinline__ XfT<T> get_xft(const T& px, const T& py, const T& ang, float lcx, float lcy) {
    T s, c;
    sincos_(ang, s, c);
    XfT<T> t;
    t.q = V<T>{c, s};
    t.p = sub(V<T>{px, py}, rotatet(cv<T>(lcx, lcy), t.q));
    return t;
}
template <class T> __device__ __forceinline__ V<T> unit_vectort(const V<T>& v, V<T> fallback) {
    const T m2 = v.x * v.x + v.y * v.y;
    if (is_normal_f(val(m2))) {
        const T m = sqrt_(m2);
        const T inv = 1.0f / m;
        return {v.x * inv, v.y * inv};
    }
    const T m = hypot_(v.x, v.y);
    if (!is_normal_f(val(m))) return fallback;
    return {v.x / m, v.y / m};
}
template <class T> __device__ __forceinline__ T clampt(const T& v, const T& lo, const T& hi) {
    return (val(v) < val(lo)) ? lo : ((val(hi) < val(v)) ? hi : v);
}
template <class T> __device__ __forceinline__ T maxt(const T& a, const T& b) { return (val(a) < val(b)) ? b : a; }

// ---- constants of one contact for the differentiable pieces ------------------------
struct ContactK {
    float4 mA, mB;        // invM invI lcx lcy of both bodies
    float rA, rB;         // vertex radii
    float restitution;
    uint32_t type, count; // manifold type and point count (before conditioning)
    float lnx, lny, lpx, lpy, p0x, p0y, p1x, p1y;  // local manifold
    uint32_t writableA, writableB;
    double dp[4];         // tangents of p0x p0y p1x p1y (the tangent pass; zero elsewhere)
};

// A manifold point coordinate as T: its float value, with its tangent under Tan.
template <class T> __device__ __forceinline__ T kpt(float v, double d);
template <> __device__ __forceinline__ float kpt<float>(float v, double) { return v; }
template <> __device__ __forceinline__ Tan kpt<Tan>(float v, double d) { return Tan{v, d}; }

// Velocity-constraint geometry (the values VelocityConstraint holds).
template <class T>
struct Geom {
    V<T> n;
    V<T> rA[2], rB[2];
    T nm[2], tm[2], vb[2];
    T k00, k11, k01, m00, m11, m01;
    T mu;
    int cnt;
};

// Body state of a contact's two bodies: x y angle (centre of mass), vx vy w.
template <class T>
struct Pair3 {
    T ax, ay, az, bx, by, bz;
};

// GetWorldManifold + VelocityConstraint (VelocityConstraint.cpp:38-185), as
// k_build_constraints computes them.
template <class T>
__device__ Geom<T> build_geom(const ContactK& k, const Pair3<T>& p, const Pair3<T>& v, const T& mu, const DConf& c) {
    Geom<T> g;
    const XfT<T> xfA = get_xft(p.ax, p.ay, p.az, k.mA.z, k.mA.w);
    const XfT<T> xfB = get_xft(p.bx, p.by, p.bz, k.mB.z, k.mB.w);
    const V<T> ln = cv<T>(k.lnx, k.lny), lp = cv<T>(k.lpx, k.lpy);
    const V<T> plp[2] = {V<T>{kpt<T>(k.p0x, k.dp[0]), kpt<T>(k.p0y, k.dp[1])},
                         V<T>{kpt<T>(k.p1x, k.dp[2]), kpt<T>(k.p1y, k.dp[3])}};
    const int count = (int)k.count;
    V<T> n = cv<T>(0.f, 0.f);
    V<T> wpt[2] = {cv<T>(0.f, 0.f), cv<T>(0.f, 0.f)};
    if (k.type == M_CIRCLES) {
        const V<T> a = xformt(lp, xfA), b = xformt(plp[0], xfB);
        n = unit_vectort(sub(b, a), cv<T>(1.f, 0.f));
        const V<T> cA = add(a, scale(n, C<T>(k.rA))), cB = sub(b, scale(n, C<T>(k.rB)));
        wpt[0] = vdivt(add(cA, cB), 2.0f);
    } else if (k.type == M_FACEA) {
        n = urotatet(ln, xfA.q);
        const V<T> planePoint = xformt(lp, xfA);
        for (int i = 0; i < count; ++i) {
            const V<T> clip = xformt(plp[i], xfB);
            const V<T> cA = add(clip, scale(n, k.rA - dott(sub(clip, planePoint), n)));
            const V<T> cB = sub(clip, scale(n, C<T>(k.rB)));
            wpt[i] = vdivt(add(cA, cB), 2.0f);
        }
    } else if (k.type == M_FACEB) {
        const V<T> nb = urotatet(ln, xfB.q);
        const V<T> planePoint = xformt(lp, xfB);
        for (int i = 0; i < count; ++i) {
            const V<T> clip = xformt(plp[i], xfA);
            const V<T> cB = add(clip, scale(nb, k.rB - dott(sub(clip, planePoint), nb)));
            const V<T> cA = sub(clip, scale(nb, C<T>(k.rA)));
            wpt[i] = vdivt(add(cA, cB), 2.0f);
        }
        n = neg(nb);
    }
    g.n = n;
    g.mu = mu;
    const float invMass = k.mA.x + k.mB.x;
    const V<T> tangent = fwdperpt(n);
    const V<T> velA = V<T>{v.ax, v.ay}, velB = V<T>{v.bx, v.by};
    for (int j = 0; j < 2; ++j) {
        g.rA[j] = g.rB[j] = cv<T>(0.f, 0.f);
        g.nm[j] = g.tm[j] = g.vb[j] = C<T>(0.f);
    }
    for (int j = 0; j < count; ++j) {
        const V<T> relA = sub(wpt[j], V<T>{p.ax, p.ay});
        const V<T> relB = sub(wpt[j], V<T>{p.bx, p.by});
        {
            const V<T> dv = sub(add(velB, scale(revperpt(relB), v.bz)), add(velA, scale(revperpt(relA), v.az)));
            const T vn = dott(dv, n);
            g.vb[j] = (val(vn) < -c.velocityThreshold) ? (-k.restitution) * vn : C<T>(0.f);
        }
        {
            const T crA = crosst(relA, n), crB = crosst(relB, n);
            const T value = invMass + k.mA.y * (crA * crA) + k.mB.y * (crB * crB);
            g.nm[j] = (val(value) != 0.f) ? 1.0f / value : C<T>(0.f);
        }
        {
            const T crA = crosst(relA, tangent), crB = crosst(relB, tangent);
            const T value = invMass + k.mA.y * (crA * crA) + k.mB.y * (crB * crB);
            g.tm[j] = (val(value) != 0.f) ? 1.0f / value : C<T>(0.f);
        }
        g.rA[j] = relA;
        g.rB[j] = relB;
    }
    int cnt = count;
    g.k00 = g.k11 = g.k01 = g.m00 = g.m11 = g.m01 = C<T>(0.f);
    if (c.doBlocksolve && count == 2) {
        const T rnA0 = crosst(g.rA[0], n), rnB0 = crosst(g.rB[0], n);
        const T rnA1 = crosst(g.rA[1], n), rnB1 = crosst(g.rB[1], n);
        const T kk00 = invMass + k.mA.y * (rnA0 * rnA0) + k.mB.y * (rnB0 * rnB0);
        const T kk11 = invMass + k.mA.y * (rnA1 * rnA1) + k.mB.y * (rnB1 * rnB1);
        const T kk01 = invMass + (k.mA.y * rnA0 * rnA1) + (k.mB.y * rnB0 * rnB1);
        const T k_diff = kk00 * kk11 - kk01 * kk01;
        if (val(kk00 * kk00) < val(1000.0f * k_diff)) {
            g.k00 = kk00; g.k11 = kk11; g.k01 = kk01;
            const T cp = crosst(V<T>{kk00, kk01}, V<T>{kk01, kk11});
            if (!almost_zero(val(cp))) {
                const T inv = 1.0f / cp;
                g.m00 = kk11 * inv; g.m01 = (-kk01) * inv; g.m11 = kk00 * inv;
            }
        } else {
            cnt = 1;
        }
    }
    if (cnt < 2) {
        g.rA[1] = g.rB[1] = cv<T>(0.f, 0.f);
        g.nm[1] = g.tm[1] = g.vb[1] = C<T>(0.f);
    }
    g.cnt = cnt;
    return g;
}

template <class T>
struct Imp {
    T ni0, ti0, ni1, ti1;
};

// WarmStartVelocities (AabbTreeWorld.cpp:227-274): velocities after applying
// the stored impulses.
template <class T>
__device__ void warm_start_t(const ContactK& k, const Geom<T>& g, Pair3<T>& vel, const Imp<T>& im) {
    const V<T> n = g.n, t = fwdperpt(n);
    T dAx = C<T>(0.f), dAy = C<T>(0.f), dAw = C<T>(0.f), dBx = C<T>(0.f), dBy = C<T>(0.f), dBw = C<T>(0.f);
    for (int j = 0; j < g.cnt; ++j) {
        const T ni = j ? im.ni1 : im.ni0, ti = j ? im.ti1 : im.ti0;
        const V<T> P = add(scale(n, ni), scale(t, ti));
        const T LA = crosst(g.rA[j], P), LB = crosst(g.rB[j], P);
        dAx = dAx - P.x * k.mA.x; dAy = dAy - P.y * k.mA.x; dAw = dAw - k.mA.y * LA;
        dBx = dBx + P.x * k.mB.x; dBy = dBy + P.y * k.mB.x; dBw = dBw + k.mB.y * LB;
    }
    if (k.writableA) { vel.ax = vel.ax + dAx; vel.ay = vel.ay + dAy; vel.az = vel.az + dAw; }
    if (k.writableB) { vel.bx = vel.bx + dBx; vel.by = vel.by + dBy; vel.bz = vel.bz + dBw; }
}

template <class T>
__device__ __forceinline__ V<T> rel_velt(const T& vax, const T& vay, const T& vaw, const V<T>& rA, const T& vbx,
                                         const T& vby, const T& vbw, const V<T>& rB) {
    return sub(add(V<T>{vbx, vby}, scale(revperpt(rB), vbw)), add(V<T>{vax, vay}, scale(revperpt(rA), vaw)));
}

// GaussSeidel::SolveVelocityConstraint (ContactSolver.cpp:245-492) as
// solve_contact_velocity computes it; updates vel (for writable bodies) and im.
template <class T>
__device__ void solve_velocity_t(const ContactK& k, const Geom<T>& g, Pair3<T>& vel, Imp<T>& im) {
    T vAx = vel.ax, vAy = vel.ay, vAw = vel.az, vBx = vel.bx, vBy = vel.by, vBw = vel.bz;
    const V<T> n = g.n;
    const float mAx = k.mA.x, mAy = k.mA.y, mBx = k.mB.x, mBy = k.mB.y;
    for (int pass = 0; pass < 2; ++pass) {
        const bool tangentPass = pass == 0;
        if (!tangentPass && g.cnt == 2 &&
            !(val(g.k00) == 0.f && val(g.k11) == 0.f && val(g.k01) == 0.f)) {
            const V<T> dv0 = rel_velt(vAx, vAy, vAw, g.rA[0], vBx, vBy, vBw, g.rB[0]);
            const V<T> dv1 = rel_velt(vAx, vAy, vAw, g.rA[1], vBx, vBy, vBw, g.rB[1]);
            const T vn0 = dott(dv0, n), vn1 = dott(dv1, n);
            const T b0 = vn0 - g.vb[0], b1 = vn1 - g.vb[1];
            const T a0 = im.ni0, a1 = im.ni1;
            T Kx0 = C<T>(0.f); Kx0 = Kx0 + g.k00 * a0; Kx0 = Kx0 + g.k01 * a1;
            T Kx1 = C<T>(0.f); Kx1 = Kx1 + g.k01 * a0; Kx1 = Kx1 + g.k11 * a1;
            const T bp0 = b0 - Kx0, bp1 = b1 - Kx1;
            T x0 = C<T>(0.f), x1 = C<T>(0.f);
            bool apply = false;
            {
                T q0 = C<T>(0.f); q0 = q0 + g.m00 * bp0; q0 = q0 + g.m01 * bp1;
                T q1 = C<T>(0.f); q1 = q1 + g.m01 * bp0; q1 = q1 + g.m11 * bp1;
                x0 = -q0; x1 = -q1;
                apply = (val(x0) >= 0.f && val(x1) >= 0.f);
            }
            if (!apply) {
                x0 = -(g.nm[0] * bp0); x1 = C<T>(0.f);
                const T vn2 = g.k01 * x0 + bp1;
                apply = (val(x0) >= 0.f && val(vn2) >= 0.f);
            }
            if (!apply) {
                x0 = C<T>(0.f); x1 = -(g.nm[1] * bp1);
                const T vn1b = g.k01 * x1 + bp0;
                apply = (val(x1) >= 0.f && val(vn1b) >= 0.f);
            }
            if (!apply) {
                x0 = C<T>(0.f); x1 = C<T>(0.f);
                apply = (val(bp0) >= 0.f && val(bp1) >= 0.f);
            }
            if (apply) {
                const T d0 = x0 - im.ni0, d1 = x1 - im.ni1;
                const V<T> P0 = scale(n, d0), P1 = scale(n, d1);
                const V<T> P = add(P0, P1);
                const T LA = crosst(g.rA[0], P0) + crosst(g.rA[1], P1);
                const T LB = crosst(g.rB[0], P0) + crosst(g.rB[1], P1);
                vAx = vAx + (-(P.x * mAx)); vAy = vAy + (-(P.y * mAx)); vAw = vAw + (-(mAy * LA));
                vBx = vBx + P.x * mBx; vBy = vBy + P.y * mBx; vBw = vBw + mBy * LB;
                im.ni0 = x0; im.ni1 = x1;
            }
            continue;
        }
        const V<T> dir = tangentPass ? fwdperpt(n) : n;
        for (int j = (g.cnt == 2) ? 1 : 0; j >= 0; --j) {
            const V<T> rA = g.rA[j], rB = g.rB[j];
            const V<T> cvel = rel_velt(vAx, vAy, vAw, rA, vBx, vBy, vBw, rB);
            T oldImp, newImp;
            if (tangentPass) {
                const T dvel = C<T>(0.f) - dott(cvel, dir);
                const T lambda = g.tm[j] * dvel;
                const T maxImp = g.mu * (j ? im.ni1 : im.ni0);
                oldImp = j ? im.ti1 : im.ti0;
                newImp = clampt(oldImp + lambda, -maxImp, maxImp);
            } else {
                const T dvel = dott(cvel, dir);
                const T lambda = g.nm[j] * (g.vb[j] - dvel);
                oldImp = j ? im.ni1 : im.ni0;
                newImp = maxt(oldImp + lambda, C<T>(0.f));
            }
            const T inc = newImp - oldImp;
            const V<T> P = scale(dir, inc);
            const T LA = crosst(rA, P), LB = crosst(rB, P);
            vAx = vAx - P.x * mAx; vAy = vAy - P.y * mAx; vAw = vAw - mAy * LA;
            vBx = vBx + P.x * mBx; vBy = vBy + P.y * mBx; vBw = vBw + mBy * LB;
            const T nv = oldImp + inc;
            if (tangentPass) { if (j) im.ti1 = nv; else im.ti0 = nv; }
            else { if (j) im.ni1 = nv; else im.ni0 = nv; }
        }
    }
    if (k.writableA) { vel.ax = vAx; vel.ay = vAy; vel.az = vAw; }
    if (k.writableB) { vel.bx = vBx; vel.by = vBy; vel.bz = vBw; }
}

// ---- reverse of solve_velocity_t, written out ----------------------------------------
// The velocity solve is the innermost loop of the adjoint (every velocity
// iteration of every contact), so its vector-Jacobian product is written by hand
// rather than taped: the forward is recomputed from its inputs, keeping the
// state before each of its (at most four) sub-steps and the branch each took,
// and the sub-steps are then reversed in the opposite order.  Checked against
// the FP64 tangent (solve_velocity_t<Tan>) by the dot-product test.
struct GeomBar {
    float n[2];
    float rA[2][2], rB[2][2];
    float nm[2], tm[2], vb[2];
    float k00, k11, k01, m00, m11, m01, mu;
};

struct VelSub {
    float vA[3], vB[3];  // state before the sub-step
    float im[4];         // ni0 ti0 ni1 ti1 before the sub-step
    int kind;            // 0 tangent, 1 normal, 2 block
    int j;               // point (sequential sub-steps)
    int branch;          // clamp taken (sequential) or block case (0: none applied)
};

// relative velocity at (rA, rB) and its reverse
__device__ __forceinline__ void relvel_f(const float* vA, const float* vB, const float* rA, const float* rB, float* cv) {
    cv[0] = (vB[0] + (-rB[1]) * vB[2]) - (vA[0] + (-rA[1]) * vA[2]);
    cv[1] = (vB[1] + rB[0] * vB[2]) - (vA[1] + rA[0] * vA[2]);
}
__device__ __forceinline__ void relvel_bar(const float* vA, const float* vB, const float* rA, const float* rB,
                                           const float* cb, float* vbA, float* vbB, float* rbA, float* rbB) {
    vbB[0] += cb[0]; vbB[1] += cb[1]; vbB[2] += cb[0] * (-rB[1]) + cb[1] * rB[0];
    rbB[0] += cb[1] * vB[2]; rbB[1] -= cb[0] * vB[2];
    vbA[0] -= cb[0]; vbA[1] -= cb[1]; vbA[2] -= cb[0] * (-rA[1]) + cb[1] * rA[0];
    rbA[0] -= cb[1] * vA[2]; rbA[1] += cb[0] * vA[2];
}

// vbA/vbB/ib on entry: adjoints of the solve's outputs (vbA/vbB zero for bodies the
// solve does not store); on exit: adjoints of its inputs.  gb accumulates.
__device__ inline void solve_velocity_vjp(const ContactK& k, const Geom<float>& g, const Pair3<float>& vin, const Imp<float>& iin,
                                   float* vbA, float* vbB, float* ib, GeomBar& gb) {
    const float mAx = k.mA.x, mAy = k.mA.y, mBx = k.mB.x, mBy = k.mB.y;
    const float n[2] = {val(g.n.x), val(g.n.y)};
    const float t[2] = {n[1], -n[0]};
    float rA[2][2], rB[2][2];
    for (int j = 0; j < 2; ++j) {
        rA[j][0] = g.rA[j].x; rA[j][1] = g.rA[j].y; rB[j][0] = g.rB[j].x; rB[j][1] = g.rB[j].y;
    }
    // forward, keeping the sub-steps
    VelSub sub[4];
    int ns = 0;
    float vA[3] = {vin.ax, vin.ay, vin.az}, vB[3] = {vin.bx, vin.by, vin.bz};
    float im[4] = {iin.ni0, iin.ti0, iin.ni1, iin.ti1};
    auto save = [&](int kind, int j) -> VelSub& {
        VelSub& s = sub[ns++];
        for (int q = 0; q < 3; ++q) { s.vA[q] = vA[q]; s.vB[q] = vB[q]; }
        for (int q = 0; q < 4; ++q) s.im[q] = im[q];
        s.kind = kind; s.j = j; s.branch = 0;
        return s;
    };
    auto apply_P = [&](const float* P, float LA, float LB) {
        vA[0] = vA[0] - P[0] * mAx; vA[1] = vA[1] - P[1] * mAx; vA[2] = vA[2] - mAy * LA;
        vB[0] = vB[0] + P[0] * mBx; vB[1] = vB[1] + P[1] * mBx; vB[2] = vB[2] + mBy * LB;
    };
    const bool block = g.cnt == 2 && !(g.k00 == 0.f && g.k11 == 0.f && g.k01 == 0.f);
    for (int pass = 0; pass < 2; ++pass) {
        const bool tangentPass = pass == 0;
        if (!tangentPass && block) {
            VelSub& s = save(2, 0);
            float dv0[2], dv1[2];
            relvel_f(vA, vB, rA[0], rB[0], dv0);
            relvel_f(vA, vB, rA[1], rB[1], dv1);
            float vn0 = 0.f; vn0 += dv0[0] * n[0]; vn0 += dv0[1] * n[1];
            float vn1 = 0.f; vn1 += dv1[0] * n[0]; vn1 += dv1[1] * n[1];
            const float b0 = vn0 - g.vb[0], b1 = vn1 - g.vb[1];
            const float a0 = im[0], a1 = im[2];
            float Kx0 = 0.f; Kx0 += g.k00 * a0; Kx0 += g.k01 * a1;
            float Kx1 = 0.f; Kx1 += g.k01 * a0; Kx1 += g.k11 * a1;
            const float bp0 = b0 - Kx0, bp1 = b1 - Kx1;
            float x0, x1;
            int cs = 0;
            {
                float q0 = 0.f; q0 += g.m00 * bp0; q0 += g.m01 * bp1;
                float q1 = 0.f; q1 += g.m01 * bp0; q1 += g.m11 * bp1;
                x0 = -q0; x1 = -q1;
                if (x0 >= 0.f && x1 >= 0.f) cs = 1;
            }
            if (!cs) {
                x0 = -g.nm[0] * bp0; x1 = 0.f;
                const float vn2 = g.k01 * x0 + bp1;
                if (x0 >= 0.f && vn2 >= 0.f) cs = 2;
            }
            if (!cs) {
                x0 = 0.f; x1 = -g.nm[1] * bp1;
                const float vn1b = g.k01 * x1 + bp0;
                if (x1 >= 0.f && vn1b >= 0.f) cs = 3;
            }
            if (!cs) {
                x0 = 0.f; x1 = 0.f;
                if (bp0 >= 0.f && bp1 >= 0.f) cs = 4;
            }
            s.branch = cs;
            if (cs) {
                const float d0 = x0 - im[0], d1 = x1 - im[2];
                const float P0[2] = {n[0] * d0, n[1] * d0}, P1[2] = {n[0] * d1, n[1] * d1};
                const float P[2] = {P0[0] + P1[0], P0[1] + P1[1]};
                const float LA = (rA[0][0] * P0[1] - rA[0][1] * P0[0]) + (rA[1][0] * P1[1] - rA[1][1] * P1[0]);
                const float LB = (rB[0][0] * P0[1] - rB[0][1] * P0[0]) + (rB[1][0] * P1[1] - rB[1][1] * P1[0]);
                vA[0] = vA[0] + (-(P[0] * mAx)); vA[1] = vA[1] + (-(P[1] * mAx)); vA[2] = vA[2] + (-(mAy * LA));
                vB[0] = vB[0] + P[0] * mBx; vB[1] = vB[1] + P[1] * mBx; vB[2] = vB[2] + mBy * LB;
                im[0] = x0; im[2] = x1;
            }
            continue;
        }
        const float* dir = tangentPass ? t : n;
        for (int j = (g.cnt == 2) ? 1 : 0; j >= 0; --j) {
            VelSub& s = save(tangentPass ? 0 : 1, j);
            float cv[2];
            relvel_f(vA, vB, rA[j], rB[j], cv);
            float dd = 0.f; dd += cv[0] * dir[0]; dd += cv[1] * dir[1];
            float oldImp, newImp;
            if (tangentPass) {
                const float dvel = 0.f - dd;
                const float lambda = g.tm[j] * dvel;
                const float maxImp = g.mu * im[2 * j];
                oldImp = im[2 * j + 1];
                const float sv = oldImp + lambda;
                if (sv < -maxImp) { newImp = -maxImp; s.branch = 1; }
                else if (maxImp < sv) { newImp = maxImp; s.branch = 2; }
                else { newImp = sv; s.branch = 0; }
            } else {
                const float lambda = g.nm[j] * (g.vb[j] - dd);
                oldImp = im[2 * j];
                const float sv = oldImp + lambda;
                if (sv < 0.f) { newImp = 0.f; s.branch = 1; } else { newImp = sv; s.branch = 0; }
            }
            const float inc = newImp - oldImp;
            const float P[2] = {dir[0] * inc, dir[1] * inc};
            const float LA = rA[j][0] * P[1] - rA[j][1] * P[0], LB = rB[j][0] * P[1] - rB[j][1] * P[0];
            apply_P(P, LA, LB);
            if (tangentPass) im[2 * j + 1] = oldImp + inc; else im[2 * j] = oldImp + inc;
        }
    }
    // reverse
    float nb[2] = {0.f, 0.f};
    for (int q = ns - 1; q >= 0; --q) {
        const VelSub& s = sub[q];
        if (s.kind == 2) {
            if (!s.branch) continue;
            // recompute the block step's values from its inputs
            float dv0[2], dv1[2];
            relvel_f(s.vA, s.vB, rA[0], rB[0], dv0);
            relvel_f(s.vA, s.vB, rA[1], rB[1], dv1);
            float vn0 = 0.f; vn0 += dv0[0] * n[0]; vn0 += dv0[1] * n[1];
            float vn1 = 0.f; vn1 += dv1[0] * n[0]; vn1 += dv1[1] * n[1];
            const float b0 = vn0 - g.vb[0], b1 = vn1 - g.vb[1];
            const float a0 = s.im[0], a1 = s.im[2];
            float Kx0 = 0.f; Kx0 += g.k00 * a0; Kx0 += g.k01 * a1;
            float Kx1 = 0.f; Kx1 += g.k01 * a0; Kx1 += g.k11 * a1;
            const float bp0 = b0 - Kx0, bp1 = b1 - Kx1;
            float x0 = 0.f, x1 = 0.f;
            if (s.branch == 1) {
                float q0 = 0.f; q0 += g.m00 * bp0; q0 += g.m01 * bp1;
                float q1 = 0.f; q1 += g.m01 * bp0; q1 += g.m11 * bp1;
                x0 = -q0; x1 = -q1;
            } else if (s.branch == 2) {
                x0 = -g.nm[0] * bp0;
            } else if (s.branch == 3) {
                x1 = -g.nm[1] * bp1;
            }
            const float d0 = x0 - a0, d1 = x1 - a1;
            const float P0[2] = {n[0] * d0, n[1] * d0}, P1[2] = {n[0] * d1, n[1] * d1};
            // velocities
            float Pb[2] = {-mAx * vbA[0] + mBx * vbB[0], -mAx * vbA[1] + mBx * vbB[1]};
            const float LAb = -mAy * vbA[2], LBb = mBy * vbB[2];
            float P0b[2] = {Pb[0], Pb[1]}, P1b[2] = {Pb[0], Pb[1]};
            gb.rA[0][0] += LAb * P0[1]; gb.rA[0][1] -= LAb * P0[0]; P0b[0] -= LAb * rA[0][1]; P0b[1] += LAb * rA[0][0];
            gb.rA[1][0] += LAb * P1[1]; gb.rA[1][1] -= LAb * P1[0]; P1b[0] -= LAb * rA[1][1]; P1b[1] += LAb * rA[1][0];
            gb.rB[0][0] += LBb * P0[1]; gb.rB[0][1] -= LBb * P0[0]; P0b[0] -= LBb * rB[0][1]; P0b[1] += LBb * rB[0][0];
            gb.rB[1][0] += LBb * P1[1]; gb.rB[1][1] -= LBb * P1[0]; P1b[0] -= LBb * rB[1][1]; P1b[1] += LBb * rB[1][0];
            nb[0] += d0 * P0b[0] + d1 * P1b[0];
            nb[1] += d0 * P0b[1] + d1 * P1b[1];
            const float d0b = n[0] * P0b[0] + n[1] * P0b[1];
            const float d1b = n[0] * P1b[0] + n[1] * P1b[1];
            const float x0b = ib[0] + d0b, x1b = ib[2] + d1b;
            float a0b = -d0b, a1b = -d1b;
            float bp0b = 0.f, bp1b = 0.f;
            if (s.branch == 1) {
                const float q0b = -x0b, q1b = -x1b;
                gb.m00 += q0b * bp0; gb.m01 += q0b * bp1 + q1b * bp0; gb.m11 += q1b * bp1;
                bp0b = q0b * g.m00 + q1b * g.m01;
                bp1b = q0b * g.m01 + q1b * g.m11;
            } else if (s.branch == 2) {
                gb.nm[0] -= x0b * bp0;
                bp0b = -x0b * g.nm[0];
            } else if (s.branch == 3) {
                gb.nm[1] -= x1b * bp1;
                bp1b = -x1b * g.nm[1];
            }
            const float Kx0b = -bp0b, Kx1b = -bp1b;
            gb.k00 += Kx0b * a0; gb.k01 += Kx0b * a1 + Kx1b * a0; gb.k11 += Kx1b * a1;
            a0b += Kx0b * g.k00 + Kx1b * g.k01;
            a1b += Kx0b * g.k01 + Kx1b * g.k11;
            const float vn0b = bp0b, vn1b = bp1b;
            gb.vb[0] -= bp0b; gb.vb[1] -= bp1b;
            const float dv0b[2] = {vn0b * n[0], vn0b * n[1]}, dv1b[2] = {vn1b * n[0], vn1b * n[1]};
            nb[0] += vn0b * dv0[0] + vn1b * dv1[0];
            nb[1] += vn0b * dv0[1] + vn1b * dv1[1];
            relvel_bar(s.vA, s.vB, rA[0], rB[0], dv0b, vbA, vbB, gb.rA[0], gb.rB[0]);
            relvel_bar(s.vA, s.vB, rA[1], rB[1], dv1b, vbA, vbB, gb.rA[1], gb.rB[1]);
            ib[0] = a0b; ib[2] = a1b;
            continue;
        }
        const bool tangentPass = s.kind == 0;
        const int j = s.j;
        const float* dir = tangentPass ? t : n;
        float cv[2];
        relvel_f(s.vA, s.vB, rA[j], rB[j], cv);
        float dd = 0.f; dd += cv[0] * dir[0]; dd += cv[1] * dir[1];
        const int ci = tangentPass ? 2 * j + 1 : 2 * j;  // impulse this sub-step updates
        const float oldImp = s.im[ci];
        float newImp, lambda, maxImp = 0.f;
        if (tangentPass) {
            lambda = g.tm[j] * (0.f - dd);
            maxImp = g.mu * s.im[2 * j];
            newImp = (s.branch == 1) ? -maxImp : (s.branch == 2) ? maxImp : oldImp + lambda;
        } else {
            lambda = g.nm[j] * (g.vb[j] - dd);
            newImp = (s.branch == 1) ? 0.f : oldImp + lambda;
        }
        const float inc = newImp - oldImp;
        const float P[2] = {dir[0] * inc, dir[1] * inc};
        // velocities
        float Pb[2] = {-mAx * vbA[0] + mBx * vbB[0], -mAx * vbA[1] + mBx * vbB[1]};
        const float LAb = -mAy * vbA[2], LBb = mBy * vbB[2];
        gb.rA[j][0] += LAb * P[1]; gb.rA[j][1] -= LAb * P[0]; Pb[0] -= LAb * rA[j][1]; Pb[1] += LAb * rA[j][0];
        gb.rB[j][0] += LBb * P[1]; gb.rB[j][1] -= LBb * P[0]; Pb[0] -= LBb * rB[j][1]; Pb[1] += LBb * rB[j][0];
        float dirb[2] = {inc * Pb[0], inc * Pb[1]};
        float incb = dir[0] * Pb[0] + dir[1] * Pb[1];
        // the stored impulse is old + inc
        incb += ib[ci];
        float oldb = ib[ci];
        const float newb = incb;
        oldb -= incb;
        float sb = 0.f, maxb = 0.f;
        if (tangentPass) {
            if (s.branch == 1) maxb = -newb; else if (s.branch == 2) maxb = newb; else sb = newb;
        } else {
            sb = (s.branch == 1) ? 0.f : newb;
        }
        oldb += sb;
        const float lamb = sb;
        float cvb[2];
        if (tangentPass) {
            gb.mu += maxb * s.im[2 * j];
            ib[2 * j] += maxb * g.mu;
            gb.tm[j] += lamb * (0.f - dd);
            const float dvelb = lamb * g.tm[j];  // dvel = 0 - dd
            cvb[0] = -dvelb * dir[0]; cvb[1] = -dvelb * dir[1];
            dirb[0] -= dvelb * cv[0]; dirb[1] -= dvelb * cv[1];
        } else {
            gb.nm[j] += lamb * (g.vb[j] - dd);
            gb.vb[j] += lamb * g.nm[j];
            const float ddb = -lamb * g.nm[j];
            cvb[0] = ddb * dir[0]; cvb[1] = ddb * dir[1];
            dirb[0] += ddb * cv[0]; dirb[1] += ddb * cv[1];
        }
        ib[ci] = oldb;
        relvel_bar(s.vA, s.vB, rA[j], rB[j], cvb, vbA, vbB, gb.rA[j], gb.rB[j]);
        if (tangentPass) { nb[0] -= dirb[1]; nb[1] += dirb[0]; }
        else { nb[0] += dirb[0]; nb[1] += dirb[1]; }
        (void)lambda;
    }
    gb.n[0] += nb[0]; gb.n[1] += nb[1];
}

// GetPSM (PositionSolverManifold.cpp:103-121)
template <class T>
struct PSMt {
    V<T> n, pt;
    T sep;
};
template <class T>
__device__ PSMt<T> get_psmt(const ContactK& k, int idx, const XfT<T>& xfA, const XfT<T>& xfB) {
    PSMt<T> r;
    const V<T> lp = cv<T>(k.lpx, k.lpy), ln = cv<T>(k.lnx, k.lny);
    const V<T> plp = idx ? V<T>{kpt<T>(k.p1x, k.dp[2]), kpt<T>(k.p1y, k.dp[3])}
                         : V<T>{kpt<T>(k.p0x, k.dp[0]), kpt<T>(k.p0y, k.dp[1])};
    if (k.type == M_CIRCLES) {
        const V<T> a = xformt(lp, xfA), b = xformt(plp, xfB);
        const V<T> delta = sub(b, a);
        r.n = unit_vectort(delta, cv<T>(0.f, 0.f));
        r.pt = vdivt(add(a, b), 2.0f);
        r.sep = dott(delta, r.n);
    } else if (k.type == M_FACEA) {
        const V<T> planePoint = xformt(lp, xfA);
        r.n = urotatet(ln, xfA.q);
        r.pt = xformt(plp, xfB);
        r.sep = dott(sub(r.pt, planePoint), r.n);
    } else {
        const V<T> planePoint = xformt(lp, xfB);
        const V<T> nb = urotatet(ln, xfB.q);
        r.pt = xformt(plp, xfA);
        r.sep = dott(sub(r.pt, planePoint), nb);
        r.n = neg(nb);
    }
    return r;
}

// solver_fn of GaussSeidel::SolvePositionConstraint (ContactSolver.cpp:521-551):
// position increments of both bodies.
template <class T>
__device__ void pos_solver_fnt(const PSMt<T>& psm, const V<T>& pA, const V<T>& pB, const ContactK& k, const DConf& c,
                               T out[6], T& separation) {
    const float invMassTotal = k.mA.x + k.mB.x;
    separation = psm.sep - (k.rA + k.rB);
    const V<T> rA = sub(psm.pt, pA), rB = sub(psm.pt, pB);
    const T cA = crosst(rA, psm.n), cB = crosst(rB, psm.n);
    const T K = invMassTotal + k.mA.y * (cA * cA) + k.mB.y * (cB * cB);
    const T C_ = -clampt(c.regResolutionRate * (separation + c.linearSlop), C<T>(-c.maxLinearCorrection), C<T>(0.f));
    const V<T> nC = scale(psm.n, C_);
    const T invK = 1.0f / K;
    const V<T> P = V<T>{nC.x * invK, nC.y * invK};
    const T LA = crosst(rA, P), LB = crosst(rB, P);
    out[0] = -(P.x * k.mA.x); out[1] = -(P.y * k.mA.x); out[2] = -(k.mA.y * LA);
    out[3] = P.x * k.mB.x; out[4] = P.y * k.mB.x; out[5] = (k.mB.y * LB);
}

// GaussSeidel::SolvePositionConstraint (ContactSolver.cpp:494-643) as
// solve_contact_position computes it; updates the positions of writable bodies.
template <class T>
__device__ void solve_position_t(const ContactK& k, const DConf& c, Pair3<T>& pos) {
    T pAx = pos.ax, pAy = pos.ay, pAz = pos.az, pBx = pos.bx, pBy = pos.by, pBz = pos.bz;
    auto apply = [&](const T* s) {
        pAx = pAx + s[0]; pAy = pAy + s[1]; pAz = pAz + s[2];
        pBx = pBx + s[3]; pBy = pBy + s[4]; pBz = pBz + s[5];
    };
    T s0[6], s1[6], sep0, sep1;
    if (k.count == 1u) {
        const PSMt<T> psm0 = get_psmt(k, 0, get_xft(pAx, pAy, pAz, k.mA.z, k.mA.w), get_xft(pBx, pBy, pBz, k.mB.z, k.mB.w));
        pos_solver_fnt(psm0, V<T>{pAx, pAy}, V<T>{pBx, pBy}, k, c, s0, sep0);
        apply(s0);
    } else if (k.count == 2u) {
        const XfT<T> xfA = get_xft(pAx, pAy, pAz, k.mA.z, k.mA.w), xfB = get_xft(pBx, pBy, pBz, k.mB.z, k.mB.w);
        const PSMt<T> psm0 = get_psmt(k, 0, xfA, xfB);
        const PSMt<T> psm1 = get_psmt(k, 1, xfA, xfB);
        if (almost_equal(val(psm0.sep), val(psm1.sep))) {
            pos_solver_fnt(psm0, V<T>{pAx, pAy}, V<T>{pBx, pBy}, k, c, s0, sep0);
            pos_solver_fnt(psm1, V<T>{pAx, pAy}, V<T>{pBx, pBy}, k, c, s1, sep1);
            pAx = pAx + s0[0]; pAy = pAy + s0[1]; pAz = pAz + s0[2];
            pAx = pAx + s1[0]; pAy = pAy + s1[1]; pAz = pAz + s1[2];
            pBx = pBx + s0[3]; pBy = pBy + s0[4]; pBz = pBz + s0[5];
            pBx = pBx + s1[3]; pBy = pBy + s1[4]; pBz = pBz + s1[5];
        } else if (val(psm0.sep) < val(psm1.sep) || val(psm1.sep) < val(psm0.sep)) {
            const int first = (val(psm0.sep) < val(psm1.sep)) ? 0 : 1;
            const PSMt<T> pf = first ? psm1 : psm0;
            pos_solver_fnt(pf, V<T>{pAx, pAy}, V<T>{pBx, pBy}, k, c, s0, sep0);
            apply(s0);
            const PSMt<T> ps = get_psmt(k, 1 - first, get_xft(pAx, pAy, pAz, k.mA.z, k.mA.w),
                                        get_xft(pBx, pBy, pBz, k.mB.z, k.mB.w));
            pos_solver_fnt(ps, V<T>{pAx, pAy}, V<T>{pBx, pBy}, k, c, s1, sep1);
            apply(s1);
        }
    }
    if (k.writableA) { pos.ax = pAx; pos.ay = pAy; pos.az = pAz; }
    if (k.writableB) { pos.bx = pBx; pos.by = pBy; pos.bz = pBz; }
}

// ---- hand-written reverse of the position solver -----------------------------------
// q̄ += (d rotate(v, q) / dq)^T ō for a constant v (rotatet and urotatet alike).
__device__ __forceinline__ void rot_qbar(float vx, float vy, float ox, float oy, float& qx, float& qy) {
    qx += ox * vx + oy * vy;
    qy += oy * vx - ox * vy;
}

// Adjoints of one body's transformation (p = position - rotate(lc, q), q = (cos a,
// sin a)) turned into adjoints of its position (x, y, angle).
__device__ __forceinline__ void xf_bar_to_pos(float pbx, float pby, float qbx, float qby, float lcx, float lcy,
                                              float s, float c, float* out) {
    out[0] += pbx;
    out[1] += pby;
    rot_qbar(lcx, lcy, -pbx, -pby, qbx, qby);
    out[2] += qbx * -s + qby * c;
}

// Reverse of v = rotate(l, q) onto l, for a constant q: l̄ += rotate^T(v̄, q).
__device__ __forceinline__ void rot_lbar(float qx, float qy, float vbx, float vby, float* lb) {
    lb[0] += qx * vbx + qy * vby;
    lb[1] += qx * vby - qy * vbx;
}

// Reverse of one point of GaussSeidel::SolvePositionConstraint: given the body
// positions p the point starts from and the adjoints sb of its increments s(p),
// adds (ds/dp)^T sb to pb, and the adjoint of the manifold point's local
// coordinates to lb[2 idx], lb[2 idx + 1].  Forward values are recomputed in the
// forward's order.
__device__ inline void pos_point_vjp(const ContactK& k, const DConf& c, int idx, const float* p, const float* sb,
                                     float* pb, float* lb) {
    // forward: transformations, the point's manifold and the solver function
    float sA, cA, sB, cB;
    sincosf(p[2], &sA, &cA);
    sincosf(p[5], &sB, &cB);
    const XfT<float> xfA = get_xft(p[0], p[1], p[2], k.mA.z, k.mA.w);
    const XfT<float> xfB = get_xft(p[3], p[4], p[5], k.mB.z, k.mB.w);
    const PSMt<float> psm = get_psmt(k, idx, xfA, xfB);
    const float invMassTotal = k.mA.x + k.mB.x;
    const float separation = psm.sep - (k.rA + k.rB);
    const float rAx = psm.pt.x - p[0], rAy = psm.pt.y - p[1];
    const float rBx = psm.pt.x - p[3], rBy = psm.pt.y - p[4];
    const float crA = rAx * psm.n.y - rAy * psm.n.x, crB = rBx * psm.n.y - rBy * psm.n.x;
    const float K = invMassTotal + k.mA.y * (crA * crA) + k.mB.y * (crB * crB);
    const float x = c.regResolutionRate * (separation + c.linearSlop);
    const bool active = !(x < -c.maxLinearCorrection) && !(0.f < x);
    const float Cv = -clampt(x, -c.maxLinearCorrection, 0.f);
    const float nCx = psm.n.x * Cv, nCy = psm.n.y * Cv;
    const float invK = 1.0f / K;
    const float Px = nCx * invK, Py = nCy * invK;
    // reverse of the solver function
    float Pbx = -k.mA.x * sb[0] + k.mB.x * sb[3];
    float Pby = -k.mA.x * sb[1] + k.mB.x * sb[4];
    const float LAb = -k.mA.y * sb[2], LBb = k.mB.y * sb[5];
    float rAbx = LAb * Py, rAby = -LAb * Px, rBbx = LBb * Py, rBby = -LBb * Px;
    Pbx += -LAb * rAy - LBb * rBy;
    Pby += LAb * rAx + LBb * rBx;
    const float nCbx = Pbx * invK, nCby = Pby * invK;
    const float invKb = Pbx * nCx + Pby * nCy;
    const float Kb = -invKb * invK * invK;
    float nbx = nCbx * Cv, nby = nCby * Cv;
    const float Cb = nCbx * psm.n.x + nCby * psm.n.y;
    const float sepb = active ? -Cb * c.regResolutionRate : 0.f;
    const float crAb = Kb * 2.f * k.mA.y * crA, crBb = Kb * 2.f * k.mB.y * crB;
    rAbx += crAb * psm.n.y; rAby -= crAb * psm.n.x;
    rBbx += crBb * psm.n.y; rBby -= crBb * psm.n.x;
    nbx += -crAb * rAy - crBb * rBy;
    nby += crAb * rAx + crBb * rBx;
    const float ptbx = rAbx + rBbx, ptby = rAby + rBby;
    pb[0] -= rAbx; pb[1] -= rAby; pb[3] -= rBbx; pb[4] -= rBby;
    // reverse of the manifold point (GetPSM) onto both transformations
    float xApx = 0.f, xApy = 0.f, qAx = 0.f, qAy = 0.f, xBpx = 0.f, xBpy = 0.f, qBx = 0.f, qBy = 0.f;
    const float plx = idx ? k.p1x : k.p0x, ply = idx ? k.p1y : k.p0y;
    if (k.type == M_CIRCLES) {
        const V<float> a = xformt(cv<float>(k.lpx, k.lpy), xfA), b = xformt(cv<float>(plx, ply), xfB);
        const float dx = b.x - a.x, dy = b.y - a.y;
        const float m2 = dx * dx + dy * dy;
        float dbx = sepb * psm.n.x, dby = sepb * psm.n.y;
        const float ntx = nbx + sepb * dx, nty = nby + sepb * dy;
        const float m = is_normal_f(m2) ? sqrtf(m2) : hypotf(dx, dy);
        if (is_normal_f(m)) {  // n = delta / |delta|; otherwise n is the constant fallback
            const float dn = ntx * psm.n.x + nty * psm.n.y;
            dbx += (ntx - psm.n.x * dn) / m;
            dby += (nty - psm.n.y * dn) / m;
        }
        const float abx = 0.5f * ptbx - dbx, aby = 0.5f * ptby - dby;
        const float bbx = 0.5f * ptbx + dbx, bby = 0.5f * ptby + dby;
        xApx += abx; xApy += aby; rot_qbar(k.lpx, k.lpy, abx, aby, qAx, qAy);
        xBpx += bbx; xBpy += bby; rot_qbar(plx, ply, bbx, bby, qBx, qBy);
    } else if (k.type == M_FACEA) {
        const V<float> pp = xformt(cv<float>(k.lpx, k.lpy), xfA);
        const float dx = psm.pt.x - pp.x, dy = psm.pt.y - pp.y;
        const float dbx = sepb * psm.n.x, dby = sepb * psm.n.y;
        const float ntx = nbx + sepb * dx, nty = nby + sepb * dy;
        const float ptx = ptbx + dbx, pty = ptby + dby;
        xApx -= dbx; xApy -= dby; rot_qbar(k.lpx, k.lpy, -dbx, -dby, qAx, qAy);
        rot_qbar(k.lnx, k.lny, ntx, nty, qAx, qAy);
        xBpx += ptx; xBpy += pty; rot_qbar(plx, ply, ptx, pty, qBx, qBy);
        rot_lbar(xfB.q.x, xfB.q.y, ptx, pty, lb + 2 * idx);
    } else {
        const V<float> pp = xformt(cv<float>(k.lpx, k.lpy), xfB);
        const float dx = psm.pt.x - pp.x, dy = psm.pt.y - pp.y;
        // n = -nb
        const float nbn_x = -psm.n.x, nbn_y = -psm.n.y;
        const float dbx = sepb * nbn_x, dby = sepb * nbn_y;
        const float ntx = -nbx + sepb * dx, nty = -nby + sepb * dy;
        const float ptx = ptbx + dbx, pty = ptby + dby;
        xBpx -= dbx; xBpy -= dby; rot_qbar(k.lpx, k.lpy, -dbx, -dby, qBx, qBy);
        rot_qbar(k.lnx, k.lny, ntx, nty, qBx, qBy);
        xApx += ptx; xApy += pty; rot_qbar(plx, ply, ptx, pty, qAx, qAy);
        rot_lbar(xfA.q.x, xfA.q.y, ptx, pty, lb + 2 * idx);
    }
    xf_bar_to_pos(xApx, xApy, qAx, qAy, k.mA.z, k.mA.w, sA, cA, pb);
    xf_bar_to_pos(xBpx, xBpy, qBx, qBy, k.mB.z, k.mB.w, sB, cB, pb + 3);
}

// Reverse of solve_position_t in float: yb = adjoints of the output positions
// (zero for a body the solve does not store); pb = adjoints of the inputs; lb
// (p0x p0y p1x p1y) accumulates the adjoints of the manifold's local points.
__device__ inline void solve_position_vjp(const ContactK& k, const DConf& c, const float* p, const float* yb, float* pb,
                                          float* lb) {
    for (int i = 0; i < 6; ++i) pb[i] = yb[i];
    if (k.count == 1u) {
        pos_point_vjp(k, c, 0, p, yb, pb, lb);
    } else if (k.count == 2u) {
        const XfT<float> xfA = get_xft(p[0], p[1], p[2], k.mA.z, k.mA.w), xfB = get_xft(p[3], p[4], p[5], k.mB.z, k.mB.w);
        const float sep0 = get_psmt(k, 0, xfA, xfB).sep, sep1 = get_psmt(k, 1, xfA, xfB).sep;
        if (almost_equal(sep0, sep1)) {
            pos_point_vjp(k, c, 0, p, yb, pb, lb);
            pos_point_vjp(k, c, 1, p, yb, pb, lb);
        } else if (sep0 < sep1 || sep1 < sep0) {
            // p1 = p + s_first(p); p2 = p1 + s_second(p1)
            const int first = (sep0 < sep1) ? 0 : 1;
            Pair3<float> q{p[0], p[1], p[2], p[3], p[4], p[5]};
            const PSMt<float> pf = get_psmt(k, first, xfA, xfB);
            float s0[6], sp;
            pos_solver_fnt(pf, V<float>{q.ax, q.ay}, V<float>{q.bx, q.by}, k, c, s0, sp);
            const float p1[6] = {q.ax + s0[0], q.ay + s0[1], q.az + s0[2], q.bx + s0[3], q.by + s0[4], q.bz + s0[5]};
            float b1[6];
            for (int i = 0; i < 6; ++i) b1[i] = yb[i];
            pos_point_vjp(k, c, 1 - first, p1, yb, b1, lb);
            for (int i = 0; i < 6; ++i) pb[i] = b1[i];
            pos_point_vjp(k, c, first, p, b1, pb, lb);
        }
    }
}

// ---- revolute joints (RevoluteJointConf.cpp:127-431), point rows only ---------------
// The differentiated step takes joints without motor and limit: the angular
// impulse then stays zero and only the 2-row point constraint acts.
struct JointK {
    float4 mA, mB;  // invM invI lcx lcy of both bodies
    float4 an;      // local anchors on A (x, y) and B (z, w)
    uint32_t writableA, writableB;
};

// InitVelocity's geometry (RevoluteJointConf.cpp:127-186): world anchors relative
// to the centres and the upper 2x2 of the mass matrix.
template <class T>
struct JGeom {
    V<T> rA, rB;
    T exx, eyx, eyy;
};
constexpr int kJointGeomWords = 7;

template <class T>
__device__ JGeom<T> joint_geom_t(const JointK& k, const T& angA, const T& angB) {
    T sA, cA, sB, cB;
    sincos_(angA, sA, cA);
    sincos_(angB, sB, cB);
    JGeom<T> g;
    g.rA = rotatet(cv<T>(k.an.x - k.mA.z, k.an.y - k.mA.w), V<T>{cA, sA});
    g.rB = rotatet(cv<T>(k.an.z - k.mB.z, k.an.w - k.mB.w), V<T>{cB, sB});
    const float iMA = k.mA.x, iIA = k.mA.y, iMB = k.mB.x, iIB = k.mB.y;
    g.exx = iMA + ((g.rA.y * g.rA.y) * iIA) + iMB + ((g.rB.y * g.rB.y) * iIB);
    g.eyx = (-g.rA.y * g.rA.x * iIA) + (-g.rB.y * g.rB.x * iIB);
    g.eyy = iMA + ((g.rA.x * g.rA.x) * iIA) + iMB + ((g.rB.x * g.rB.x) * iIB);
    return g;
}

// Warm start of InitVelocity: the stored impulse (ix, iy) scaled by dtRatio is
// applied to both bodies and becomes the impulse the iterations start from.
template <class T>
__device__ void joint_warm_t(const JointK& k, const JGeom<T>& g, float dtRatio, Pair3<T>& v, T& ix, T& iy) {
    ix = ix * dtRatio;
    iy = iy * dtRatio;
    const V<T> P{ix, iy};
    const T LA = crosst(g.rA, P), LB = crosst(g.rB, P);
    const float iMA = k.mA.x, iIA = k.mA.y, iMB = k.mB.x, iIB = k.mB.y;
    v.ax = v.ax - P.x * iMA; v.ay = v.ay - P.y * iMA; v.az = v.az - iIA * LA;
    v.bx = v.bx + P.x * iMB; v.by = v.by + P.y * iMB; v.bz = v.bz + iIB * LB;
}

// SolveVelocity's point rows (RevoluteJointConf.cpp:228-331): Solve22 on the
// upper 2x2 of the mass matrix.
template <class T>
__device__ void joint_velocity_t(const JointK& k, const JGeom<T>& g, Pair3<T>& v, T& ix, T& iy) {
    const V<T> vb{v.bx + (-g.rB.y) * v.bz, v.by + g.rB.x * v.bz};
    const V<T> va{v.ax + (-g.rA.y) * v.az, v.ay + g.rA.x * v.az};
    const V<T> vd = sub(vb, va);
    const T cp = g.exx * g.eyy - g.eyx * g.eyx;
    const T det = (val(cp) != 0.f) ? (1.0f / cp) : cp;
    const V<T> bb = neg(vd);
    const V<T> P{det * (g.eyy * bb.x - g.eyx * bb.y), det * (g.exx * bb.y - g.eyx * bb.x)};
    ix = ix + P.x;
    iy = iy + P.y;
    const T LA = crosst(g.rA, P), LB = crosst(g.rB, P);
    const float iMA = k.mA.x, iIA = k.mA.y, iMB = k.mB.x, iIB = k.mB.y;
    v.ax = v.ax - P.x * iMA; v.ay = v.ay - P.y * iMA; v.az = v.az - iIA * LA;
    v.bx = v.bx + P.x * iMB; v.by = v.by + P.y * iMB; v.bz = v.bz + iIB * LB;
}

// SolvePosition's point rows (RevoluteJointConf.cpp:333-431); updates the
// positions of writable bodies.
template <class T>
__device__ void joint_position_t(const JointK& k, Pair3<T>& p) {
    const JGeom<T> g = joint_geom_t(k, p.az, p.bz);
    const V<T> Cp = sub(add(V<T>{p.bx, p.by}, g.rB), add(V<T>{p.ax, p.ay}, g.rA));
    const float iMA = k.mA.x, iIA = k.mA.y, iMB = k.mB.x, iIB = k.mB.y;
    const T exx = iMA + (iIA * (g.rA.y * g.rA.y)) + iMB + (iIB * (g.rB.y * g.rB.y));
    const T exy = (-iIA * g.rA.x * g.rA.y) + (-iIB * g.rB.x * g.rB.y);
    const T eyy = iMA + (iIA * (g.rA.x * g.rA.x)) + iMB + (iIB * (g.rB.x * g.rB.x));
    const T cp = crosst(V<T>{exx, exy}, V<T>{exy, eyy});
    V<T> x{C<T>(0.f), C<T>(0.f)};
    if (!almost_zero(val(cp))) {
        const T inv = 1.0f / cp;
        x = V<T>{(eyy * Cp.x - exy * Cp.y) * inv, (exx * Cp.y - exy * Cp.x) * inv};
    }
    const V<T> P = neg(x);
    const T nax = p.ax - P.x * iMA, nay = p.ay - P.y * iMA, naz = p.az - iIA * crosst(g.rA, P);
    const T nbx = p.bx + P.x * iMB, nby = p.by + P.y * iMB, nbz = p.bz + iIB * crosst(g.rB, P);
    if (k.writableA) { p.ax = nax; p.ay = nay; p.az = naz; }
    if (k.writableB) { p.bx = nbx; p.by = nby; p.bz = nbz; }
}

// Reverse of joint_velocity_t in float.  vbA/vbB/ib on entry: adjoints of the
// outputs (vbA/vbB zero for bodies the solve does not store); on exit: adjoints
// of the inputs.  gb[0..6] (rA rB exx eyx eyy) accumulates.
__device__ inline void joint_velocity_vjp(const JointK& k, const JGeom<float>& g, const Pair3<float>& v, float* vbA,
                                          float* vbB, float* ib, float* gb) {
    const float iMA = k.mA.x, iIA = k.mA.y, iMB = k.mB.x, iIB = k.mB.y;
    const float vbx = v.bx + (-g.rB.y) * v.bz, vby = v.by + g.rB.x * v.bz;
    const float vax = v.ax + (-g.rA.y) * v.az, vay = v.ay + g.rA.x * v.az;
    const float bbx = -(vbx - vax), bby = -(vby - vay);
    const float cp = g.exx * g.eyy - g.eyx * g.eyx;
    const float det = (cp != 0.f) ? (1.0f / cp) : cp;
    const float ux = g.eyy * bbx - g.eyx * bby, uy = g.exx * bby - g.eyx * bbx;
    const float Px = det * ux, Py = det * uy;
    float Pbx = -iMA * vbA[0] + iMB * vbB[0] + ib[0];
    float Pby = -iMA * vbA[1] + iMB * vbB[1] + ib[1];
    const float LAb = -iIA * vbA[2], LBb = iIB * vbB[2];
    float rAbx = LAb * Py, rAby = -LAb * Px, rBbx = LBb * Py, rBby = -LBb * Px;
    Pbx += -LAb * g.rA.y - LBb * g.rB.y;
    Pby += LAb * g.rA.x + LBb * g.rB.x;
    const float ubx = det * Pbx, uby = det * Pby;
    const float detb = Pbx * ux + Pby * uy;
    const float cpb = (cp != 0.f) ? -detb * det * det : detb;
    gb[4] += cpb * g.eyy + uby * bby;
    gb[6] += cpb * g.exx + ubx * bbx;
    gb[5] += -2.f * cpb * g.eyx - ubx * bby - uby * bbx;
    const float bbbx = g.eyy * ubx - g.eyx * uby, bbby = g.exx * uby - g.eyx * ubx;
    // vd = vb - va = -bb
    const float vbbx = -bbbx, vbby = -bbby;
    vbB[0] += vbbx; vbB[1] += vbby; vbB[2] += -vbbx * g.rB.y + vbby * g.rB.x;
    rBby += -vbbx * v.bz; rBbx += vbby * v.bz;
    vbA[0] -= vbbx; vbA[1] -= vbby; vbA[2] -= -vbbx * g.rA.y + vbby * g.rA.x;
    rAby -= -vbbx * v.az; rAbx -= vbby * v.az;
    gb[0] += rAbx; gb[1] += rAby; gb[2] += rBbx; gb[3] += rBby;
}

// Reverse of joint_position_t in float: yb = adjoints of the output positions
// (zero for a body the solve does not store); pb = adjoints of the inputs.
__device__ inline void joint_position_vjp(const JointK& k, const float* p, const float* yb, float* pb) {
    const float iMA = k.mA.x, iIA = k.mA.y, iMB = k.mB.x, iIB = k.mB.y;
    for (int i = 0; i < 6; ++i) pb[i] = yb[i];
    float sA, cA, sB, cB;
    sincosf(p[2], &sA, &cA);
    sincosf(p[5], &sB, &cB);
    const JGeom<float> g = joint_geom_t(k, p[2], p[5]);
    const float lAx = k.an.x - k.mA.z, lAy = k.an.y - k.mA.w, lBx = k.an.z - k.mB.z, lBy = k.an.w - k.mB.w;
    const float Cx = (p[3] + g.rB.x) - (p[0] + g.rA.x), Cy = (p[4] + g.rB.y) - (p[1] + g.rA.y);
    const float exx = iMA + (iIA * (g.rA.y * g.rA.y)) + iMB + (iIB * (g.rB.y * g.rB.y));
    const float exy = (-iIA * g.rA.x * g.rA.y) + (-iIB * g.rB.x * g.rB.y);
    const float eyy = iMA + (iIA * (g.rA.x * g.rA.x)) + iMB + (iIB * (g.rB.x * g.rB.x));
    const float cp = exx * eyy - exy * exy;
    const bool solved = !almost_zero(cp);
    const float inv = solved ? 1.0f / cp : 0.f;
    const float ux = eyy * Cx - exy * Cy, uy = exx * Cy - exy * Cx;
    const float Px = solved ? -(ux * inv) : 0.f, Py = solved ? -(uy * inv) : 0.f;
    float Pbx = -iMA * yb[0] + iMB * yb[3], Pby = -iMA * yb[1] + iMB * yb[4];
    const float cAb = -iIA * yb[2], cBb = iIB * yb[5];
    float rAbx = cAb * Py, rAby = -cAb * Px, rBbx = cBb * Py, rBby = -cBb * Px;
    Pbx += -cAb * g.rA.y - cBb * g.rB.y;
    Pby += cAb * g.rA.x + cBb * g.rB.x;
    float Cbx = 0.f, Cby = 0.f, exxb = 0.f, exyb = 0.f, eyyb = 0.f;
    if (solved) {
        const float xbx = -Pbx, xby = -Pby;
        const float invb = xbx * ux + xby * uy;
        const float ubx = inv * xbx, uby = inv * xby;
        Cbx = eyy * ubx - exy * uby;
        Cby = exx * uby - exy * ubx;
        eyyb += ubx * Cx; exxb += uby * Cy; exyb += -ubx * Cy - uby * Cx;
        const float cpb = -invb * inv * inv;
        exxb += cpb * eyy; eyyb += cpb * exx; exyb += -2.f * cpb * exy;
    }
    rAby += 2.f * iIA * g.rA.y * exxb; rBby += 2.f * iIB * g.rB.y * exxb;
    rAbx += -iIA * g.rA.y * exyb; rAby += -iIA * g.rA.x * exyb;
    rBbx += -iIB * g.rB.y * exyb; rBby += -iIB * g.rB.x * exyb;
    rAbx += 2.f * iIA * g.rA.x * eyyb; rBbx += 2.f * iIB * g.rB.x * eyyb;
    pb[3] += Cbx; pb[4] += Cby; rBbx += Cbx; rBby += Cby;
    pb[0] -= Cbx; pb[1] -= Cby; rAbx -= Cbx; rAby -= Cby;
    float qAx = 0.f, qAy = 0.f, qBx = 0.f, qBy = 0.f;
    rot_qbar(lAx, lAy, rAbx, rAby, qAx, qAy);
    rot_qbar(lBx, lBy, rBbx, rBby, qBx, qBy);
    pb[2] += qAx * -sA + qAy * cA;
    pb[5] += qBx * -sB + qBy * cB;
}

// ---- hand-written reverse of the once-per-step pieces -------------------------------
// Geometry adjoints in the packed order of pack_geom: n rA0 rB0 rA1 rB1 nm0 tm0 nm1
// tm1 vb0 vb1 k00 k11 k01 m00 m11 m01 mu.
enum : int { GB_N = 0, GB_RA0 = 2, GB_RB0 = 4, GB_RA1 = 6, GB_RB1 = 8, GB_NM = 10, GB_VB = 14, GB_K00 = 16,
             GB_K11 = 17, GB_K01 = 18, GB_M00 = 19, GB_M11 = 20, GB_M01 = 21, GB_MU = 22 };

__device__ __forceinline__ int gb_ra(int j) { return j ? GB_RA1 : GB_RA0; }
__device__ __forceinline__ int gb_rb(int j) { return j ? GB_RB1 : GB_RB0; }

// Reverse of warm_start_t: the velocity change does not depend on the
// velocities, whose adjoints vbA/vbB (zero for bodies not stored) pass through;
// adds the impulses' adjoints to ib and the geometry's to gb (packed order).
__device__ inline void warm_start_vjp(const ContactK& k, const Geom<float>& g, const Imp<float>& im, const float* vbA,
                                      const float* vbB, float* ib, float* gb) {
    const float nx = g.n.x, ny = g.n.y, tx = ny, ty = -nx;
    float nbx = 0.f, nby = 0.f, tbx = 0.f, tby = 0.f;
    for (int j = 0; j < g.cnt; ++j) {
        const float ni = j ? im.ni1 : im.ni0, ti = j ? im.ti1 : im.ti0;
        const float Px = nx * ni + tx * ti, Py = ny * ni + ty * ti;
        float Pbx = -k.mA.x * vbA[0] + k.mB.x * vbB[0];
        float Pby = -k.mA.x * vbA[1] + k.mB.x * vbB[1];
        const float LAb = -k.mA.y * vbA[2], LBb = k.mB.y * vbB[2];
        const V<float> rA = g.rA[j], rB = g.rB[j];
        gb[gb_ra(j)] += LAb * Py; gb[gb_ra(j) + 1] += -LAb * Px;
        gb[gb_rb(j)] += LBb * Py; gb[gb_rb(j) + 1] += -LBb * Px;
        Pbx += -LAb * rA.y - LBb * rB.y;
        Pby += LAb * rA.x + LBb * rB.x;
        ib[2 * j] += Pbx * nx + Pby * ny;
        ib[2 * j + 1] += Pbx * tx + Pby * ty;
        nbx += Pbx * ni; nby += Pby * ni;
        tbx += Pbx * ti; tby += Pby * ti;
    }
    // t = (n.y, -n.x)
    gb[GB_N] += nbx - tby;
    gb[GB_N + 1] += nby + tbx;
}

// Reverse of build_geom in float: from the geometry's adjoints gb (packed order)
// to the adjoints of the positions (pb) and velocities (vb) it was built from
// (x y angle of A then B) and of the friction (*mub); lb (p0x p0y p1x p1y)
// accumulates the adjoints of the manifold's local points.
__device__ inline void build_geom_vjp(const ContactK& k, const Pair3<float>& p, const Pair3<float>& v, float mu,
                                      const DConf& c, const float* gb, float* pb, float* vb, float* mub, float* lb) {
    for (int i = 0; i < 6; ++i) pb[i] = vb[i] = 0.f;
    *mub = gb[GB_MU];
    // forward values
    float sA, cA, sB, cB;
    sincosf(p.az, &sA, &cA);
    sincosf(p.bz, &sB, &cB);
    const XfT<float> xfA = get_xft(p.ax, p.ay, p.az, k.mA.z, k.mA.w);
    const XfT<float> xfB = get_xft(p.bx, p.by, p.bz, k.mB.z, k.mB.w);
    const Geom<float> g = build_geom(k, p, v, mu, c);
    const V<float> ln = cv<float>(k.lnx, k.lny), lp = cv<float>(k.lpx, k.lpy);
    const V<float> plp[2] = {cv<float>(k.p0x, k.p0y), cv<float>(k.p1x, k.p1y)};
    const float iA = k.mA.y, iB = k.mB.y;
    const V<float> n = g.n, t = fwdperpt(n);
    // the points kept (g.cnt of them): rA = world point - centre of A, rB likewise
    const V<float>* relA = g.rA;
    const V<float>* relB = g.rB;
    // reverse
    float nbx = gb[GB_N], nby = gb[GB_N + 1], tbx = 0.f, tby = 0.f;
    V<float> rAb[2] = {{0.f, 0.f}, {0.f, 0.f}}, rBb[2] = {{0.f, 0.f}, {0.f, 0.f}};
    for (int j = 0; j < g.cnt; ++j) {
        rAb[j] = V<float>{gb[gb_ra(j)], gb[gb_ra(j) + 1]};
        rBb[j] = V<float>{gb[gb_rb(j)], gb[gb_rb(j) + 1]};
    }
    auto cross_bar = [&](const V<float>& r, const V<float>& q, float cb, V<float>& rb, float& qbx, float& qby) {
        // cross(r, q) = r.x q.y - r.y q.x
        rb.x += cb * q.y; rb.y -= cb * q.x;
        qbx -= cb * r.y; qby += cb * r.x;
    };
    if (c.doBlocksolve && g.cnt == 2 && !(g.k00 == 0.f && g.k11 == 0.f && g.k01 == 0.f)) {
        const float rnA0 = crosst(relA[0], n), rnB0 = crosst(relB[0], n);
        const float rnA1 = crosst(relA[1], n), rnB1 = crosst(relB[1], n);
        const float kk00 = g.k00, kk11 = g.k11, kk01 = g.k01;
        float k00b = gb[GB_K00], k11b = gb[GB_K11], k01b = gb[GB_K01];
        const float cp = crosst(V<float>{kk00, kk01}, V<float>{kk01, kk11});
        if (!almost_zero(cp)) {
            const float inv = 1.0f / cp;
            const float invb = gb[GB_M00] * kk11 - gb[GB_M01] * kk01 + gb[GB_M11] * kk00;
            k11b += gb[GB_M00] * inv; k01b -= gb[GB_M01] * inv; k00b += gb[GB_M11] * inv;
            const float cpb = -invb * inv * inv;
            k00b += cpb * kk11; k11b += cpb * kk00; k01b -= 2.f * cpb * kk01;
        }
        const float rnA0b = k00b * 2.f * iA * rnA0 + k01b * iA * rnA1;
        const float rnA1b = k11b * 2.f * iA * rnA1 + k01b * iA * rnA0;
        const float rnB0b = k00b * 2.f * iB * rnB0 + k01b * iB * rnB1;
        const float rnB1b = k11b * 2.f * iB * rnB1 + k01b * iB * rnB0;
        cross_bar(relA[0], n, rnA0b, rAb[0], nbx, nby);
        cross_bar(relB[0], n, rnB0b, rBb[0], nbx, nby);
        cross_bar(relA[1], n, rnA1b, rAb[1], nbx, nby);
        cross_bar(relB[1], n, rnB1b, rBb[1], nbx, nby);
    }
    V<float> wptb[2] = {{0.f, 0.f}, {0.f, 0.f}};
    for (int j = 0; j < g.cnt; ++j) {
        const V<float> ra = relA[j], rb = relB[j];
        // velocity bias
        const V<float> dv = rel_velt(v.ax, v.ay, v.az, ra, v.bx, v.by, v.bz, rb);
        const float vn = dott(dv, n);
        if (vn < -c.velocityThreshold) {
            const float vnb = -k.restitution * gb[GB_VB + j];
            const float dvbx = vnb * n.x, dvby = vnb * n.y;
            nbx += vnb * dv.x; nby += vnb * dv.y;
            vb[3] += dvbx; vb[4] += dvby; vb[5] += -dvbx * rb.y + dvby * rb.x;
            rBb[j].x += dvby * v.bz; rBb[j].y -= dvbx * v.bz;
            vb[0] -= dvbx; vb[1] -= dvby; vb[2] -= -dvbx * ra.y + dvby * ra.x;
            rAb[j].x -= dvby * v.az; rAb[j].y += dvbx * v.az;
        }
        // normal and tangent mass
        const float nm = g.nm[j], tm = g.tm[j];
        if (nm != 0.f) {
            const float valb = -gb[GB_NM + 2 * j] * nm * nm;
            const float crA = crosst(ra, n), crB = crosst(rb, n);
            cross_bar(ra, n, valb * 2.f * iA * crA, rAb[j], nbx, nby);
            cross_bar(rb, n, valb * 2.f * iB * crB, rBb[j], nbx, nby);
        }
        if (tm != 0.f) {
            const float valb = -gb[GB_NM + 2 * j + 1] * tm * tm;
            const float crA = crosst(ra, t), crB = crosst(rb, t);
            cross_bar(ra, t, valb * 2.f * iA * crA, rAb[j], tbx, tby);
            cross_bar(rb, t, valb * 2.f * iB * crB, rBb[j], tbx, tby);
        }
    }
    // relA = wpt - pA, relB = wpt - pB (points that conditioning dropped carry none)
    for (int j = 0; j < g.cnt; ++j) {
        wptb[j] = add(rAb[j], rBb[j]);
        pb[0] -= rAb[j].x; pb[1] -= rAb[j].y;
        pb[3] -= rBb[j].x; pb[4] -= rBb[j].y;
    }
    // t = fwdperp(n) = (n.y, -n.x)
    nbx += -tby;
    nby += tbx;
    // world manifold onto the two transformations
    float xApx = 0.f, xApy = 0.f, qAx = 0.f, qAy = 0.f, xBpx = 0.f, xBpy = 0.f, qBx = 0.f, qBy = 0.f;
    if (k.type == M_CIRCLES) {
        const V<float> a = xformt(lp, xfA), b = xformt(plp[0], xfB);
        const float dx = b.x - a.x, dy = b.y - a.y;
        // wpt = (a + n rA + b - n rB) / 2
        const float hx = 0.5f * wptb[0].x, hy = 0.5f * wptb[0].y;
        float abx = hx, aby = hy, bbx = hx, bby = hy;
        nbx += hx * (k.rA - k.rB); nby += hy * (k.rA - k.rB);
        const float m2 = dx * dx + dy * dy;
        const float m = is_normal_f(m2) ? sqrtf(m2) : hypotf(dx, dy);
        if (is_normal_f(m)) {
            const float dn = nbx * n.x + nby * n.y;
            const float dbx = (nbx - n.x * dn) / m, dby = (nby - n.y * dn) / m;
            abx -= dbx; aby -= dby; bbx += dbx; bby += dby;
        }
        xApx += abx; xApy += aby; rot_qbar(lp.x, lp.y, abx, aby, qAx, qAy);
        xBpx += bbx; xBpy += bby; rot_qbar(plp[0].x, plp[0].y, bbx, bby, qBx, qBy);
    } else if (k.type == M_FACEA || k.type == M_FACEB) {
        const bool fa = k.type == M_FACEA;
        // reference side r (the face), incident side i (the clipped points)
        const V<float> nn = fa ? n : neg(n);
        float nnbx = fa ? nbx : -nbx, nnby = fa ? nby : -nby;
        const XfT<float>& xr = fa ? xfA : xfB;
        const XfT<float>& xi = fa ? xfB : xfA;
        const V<float> pp = xformt(lp, xr);
        const float rr = fa ? k.rA : k.rB, ri = fa ? k.rB : k.rA;
        float ppbx = 0.f, ppby = 0.f, xipx = 0.f, xipy = 0.f, qix = 0.f, qiy = 0.f;
        for (int i = 0; i < g.cnt; ++i) {
            const V<float> clip = xformt(plp[i], xi);
            const float ex = clip.x - pp.x, ey = clip.y - pp.y;
            const float s = rr - (ex * nn.x + ey * nn.y);
            // wpt = (clip + nn s + clip - nn ri) / 2
            const float hx = 0.5f * wptb[i].x, hy = 0.5f * wptb[i].y;
            float clbx = 2.f * hx, clby = 2.f * hy;
            nnbx += hx * (s - ri); nnby += hy * (s - ri);
            const float sb = hx * nn.x + hy * nn.y;
            // s = rr - dot(clip - pp, nn)
            clbx -= sb * nn.x; clby -= sb * nn.y;
            ppbx += sb * nn.x; ppby += sb * nn.y;
            nnbx -= sb * ex; nnby -= sb * ey;
            xipx += clbx; xipy += clby; rot_qbar(plp[i].x, plp[i].y, clbx, clby, qix, qiy);
            rot_lbar(xi.q.x, xi.q.y, clbx, clby, lb + 2 * i);
        }
        float xrpx = ppbx, xrpy = ppby, qrx = 0.f, qry = 0.f;
        rot_qbar(lp.x, lp.y, ppbx, ppby, qrx, qry);
        rot_qbar(ln.x, ln.y, nnbx, nnby, qrx, qry);  // nn = urotate(ln, q of the face's body)
        if (fa) { xApx = xrpx; xApy = xrpy; qAx = qrx; qAy = qry; xBpx = xipx; xBpy = xipy; qBx = qix; qBy = qiy; }
        else { xBpx = xrpx; xBpy = xrpy; qBx = qrx; qBy = qry; xApx = xipx; xApy = xipy; qAx = qix; qAy = qiy; }
    }
    xf_bar_to_pos(xApx, xApy, qAx, qAy, k.mA.z, k.mA.w, sA, cA, pb);
    xf_bar_to_pos(xBpx, xBpy, qBx, qBy, k.mB.z, k.mB.w, sB, cB, pb + 3);
}

// Reverse of joint_warm_t: velocity adjoints pass through; ib gets the stored
// impulse's adjoint, gb[0..3] (rA rB) accumulates.
__device__ inline void joint_warm_vjp(const JointK& k, const JGeom<float>& g, float dtRatio, float ix, float iy,
                                      const float* vbA, const float* vbB, const float* lb, float* ib, float* gb) {
    const float Px = ix * dtRatio, Py = iy * dtRatio;
    float Pbx = -k.mA.x * vbA[0] + k.mB.x * vbB[0] + lb[0];
    float Pby = -k.mA.x * vbA[1] + k.mB.x * vbB[1] + lb[1];
    const float LAb = -k.mA.y * vbA[2], LBb = k.mB.y * vbB[2];
    gb[0] += LAb * Py; gb[1] -= LAb * Px; gb[2] += LBb * Py; gb[3] -= LBb * Px;
    Pbx += -LAb * g.rA.y - LBb * g.rB.y;
    Pby += LAb * g.rA.x + LBb * g.rB.x;
    ib[0] = Pbx * dtRatio;
    ib[1] = Pby * dtRatio;
}

// Reverse of joint_geom_t: adjoints of the two angles from gb[0..6].
__device__ inline void joint_geom_vjp(const JointK& k, float angA, float angB, const float* gb, float* aAb, float* aBb) {
    const JGeom<float> g = joint_geom_t(k, angA, angB);
    const float iA = k.mA.y, iB = k.mB.y;
    float rAbx = gb[0], rAby = gb[1], rBbx = gb[2], rBby = gb[3];
    const float exxb = gb[4], eyxb = gb[5], eyyb = gb[6];
    rAby += exxb * 2.f * iA * g.rA.y; rBby += exxb * 2.f * iB * g.rB.y;
    rAbx += -eyxb * iA * g.rA.y; rAby += -eyxb * iA * g.rA.x;
    rBbx += -eyxb * iB * g.rB.y; rBby += -eyxb * iB * g.rB.x;
    rAbx += eyyb * 2.f * iA * g.rA.x; rBbx += eyyb * 2.f * iB * g.rB.x;
    float sA, cA, sB, cB;
    sincosf(angA, &sA, &cA);
    sincosf(angB, &sB, &cB);
    float qAx = 0.f, qAy = 0.f, qBx = 0.f, qBy = 0.f;
    rot_qbar(k.an.x - k.mA.z, k.an.y - k.mA.w, rAbx, rAby, qAx, qAy);
    rot_qbar(k.an.z - k.mB.z, k.an.w - k.mB.w, rBbx, rBby, qBx, qBy);
    *aAb = qAx * -sA + qAy * cA;
    *aBb = qBx * -sB + qBy * cB;
}

template <class T>
__device__ __forceinline__ void pack_jgeom(const JGeom<T>& g, float* out) {
    out[0] = val(g.rA.x); out[1] = val(g.rA.y); out[2] = val(g.rB.x); out[3] = val(g.rB.y);
    out[4] = val(g.exx); out[5] = val(g.eyx); out[6] = val(g.eyy);
}

// Body velocity at the start of the solve (k_body_begin): acceleration,
// damping, then the translation and rotation caps.
template <class T>
__device__ void integrate_velocity_t(bool accelerable, float4 a, float2 dm, const DConf& c, T& vx, T& vy, T& vw) {
    const float h = c.deltaTime;
    if (accelerable) {
        vx = vx + a.x * h;
        vy = vy + a.y * h;
        vw = vw + h * a.z;
        const float linv = 1.0f / (1.0f + h * dm.x);
        vx = vx * linv;
        vy = vy * linv;
        vw = vw / (1.0f + h * dm.y);
    }
    const T tx = vx * h, ty = vy * h;
    T lsq = C<T>(0.f);
    lsq = lsq + tx * tx;
    lsq = lsq + ty * ty;
    if (val(lsq) > c.maxTranslation * c.maxTranslation) {
        const T ratio = c.maxTranslation / sqrt_(lsq);
        vx = vx * ratio;
        vy = vy * ratio;
    }
    const float absRot = fabsf(h * val(vw));
    if (absRot > c.maxRotation) {
        // |h w| is clamped to maxRotation: the result keeps w's sign only
        const T ratio = C<T>(c.maxRotation / absRot);
        vw = C<T>(val(vw) * val(ratio));
    }
}

// Reverse of integrate_velocity_t in float: b holds the adjoints of the output
// velocity on entry and of the input velocity on exit (the rotation cap holds
// |h w| at a constant).
__device__ inline void integrate_velocity_vjp(bool accelerable, float4 a, float2 dm, const DConf& c, float vx, float vy,
                                              float vw, float* b) {
    const float h = c.deltaTime;
    float linv = 1.0f;
    if (accelerable) {
        vx = vx + a.x * h;
        vy = vy + a.y * h;
        vw = vw + h * a.z;
        linv = 1.0f / (1.0f + h * dm.x);
        vx = vx * linv;
        vy = vy * linv;
        vw = vw / (1.0f + h * dm.y);
    }
    const float tx = vx * h, ty = vy * h;
    float lsq = 0.f;
    lsq = lsq + tx * tx;
    lsq = lsq + ty * ty;
    if (lsq > c.maxTranslation * c.maxTranslation) {
        // out = u maxT / |h u|
        const float ratio = c.maxTranslation / sqrtf(lsq);
        const float kb = -ratio * h * h / lsq * (b[0] * vx + b[1] * vy);
        b[0] = ratio * b[0] + kb * vx;
        b[1] = ratio * b[1] + kb * vy;
    }
    if (fabsf(h * vw) > c.maxRotation) b[2] = 0.f;
    if (accelerable) {
        b[0] *= linv;
        b[1] *= linv;
        b[2] = b[2] / (1.0f + h * dm.y);
    }
}

}  // namespace diff
}  // namespace prgpu
