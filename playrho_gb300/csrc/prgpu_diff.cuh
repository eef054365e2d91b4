// prgpu_diff.cuh -- differentiable restatement of the per-contact pieces of the
// regular step, for the adjoint (StepAdjoint) and the FP64 tangent.
//
// Each piece is written once, templated on its scalar type T, in exactly the
// operation order of the forward kernels (prgpu_solver.cu), so that
//   T = float  recomputes the forward's values bit for bit (a replay check),
//   T = Tan    carries an FP64 tangent along the forward's float values
//              (forward-mode: the tangent kernel),
//   T = AD     records a per-thread tape of local partial derivatives that a
//              reverse sweep turns into a vector-Jacobian product (reverse-mode:
//              the adjoint kernels).
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
constexpr int kTapeNodes = 400;

// Per-thread tape: node k = a local result with up to two parents and the
// partial derivative with respect to each.
struct Tape {
    double pa[kTapeNodes], pb[kTapeNodes], adj[kTapeNodes];
    int16_t ia[kTapeNodes], ib[kTapeNodes];
    int n;
    bool overflow;
    __device__ void reset() { n = 0; overflow = false; }
    __device__ int push(int a, double da, int b, double db) {
        if (n >= kTapeNodes) { overflow = true; return -1; }
        ia[n] = (int16_t)a; pa[n] = da; ib[n] = (int16_t)b; pb[n] = db; adj[n] = 0.0;
        return n++;
    }
    // adjoints of every node from those seeded on the outputs
    __device__ void backward() {
        for (int k = n - 1; k >= 0; --k) {
            const double g = adj[k];
            if (g == 0.0) continue;
            if (ia[k] >= 0) adj[ia[k]] += pa[k] * g;
            if (ib[k] >= 0) adj[ib[k]] += pb[k] * g;
        }
    }
};

struct AD {
    float v;
    int i;     // tape node, -1 for a constant
    Tape* t;
};

// value (float) with an FP64 tangent
struct Tan {
    float v;
    double d;
};

__device__ __forceinline__ float val(float x) { return x; }
__device__ __forceinline__ float val(const AD& x) { return x.v; }
__device__ __forceinline__ float val(const Tan& x) { return x.v; }

template <class T> __device__ __forceinline__ T C(float c);
template <> __device__ __forceinline__ float C<float>(float c) { return c; }
template <> __device__ __forceinline__ AD C<AD>(float c) { return AD{c, -1, nullptr}; }
template <> __device__ __forceinline__ Tan C<Tan>(float c) { return Tan{c, 0.0}; }

__device__ __forceinline__ AD rec(float v, const AD& a, double da, const AD& b, double db) {
    Tape* t = a.t ? a.t : b.t;
    if (!t || (a.i < 0 && b.i < 0)) return AD{v, -1, t};
    return AD{v, t->push(a.i, da, b.i, db), t};
}
__device__ __forceinline__ AD rec1(float v, const AD& a, double da) {
    if (!a.t || a.i < 0) return AD{v, -1, a.t};
    return AD{v, a.t->push(a.i, da, -1, 0.0), a.t};
}

__device__ __forceinline__ AD operator+(const AD& a, const AD& b) { return rec(a.v + b.v, a, 1.0, b, 1.0); }
__device__ __forceinline__ AD operator-(const AD& a, const AD& b) { return rec(a.v - b.v, a, 1.0, b, -1.0); }
__device__ __forceinline__ AD operator*(const AD& a, const AD& b) { return rec(a.v * b.v, a, (double)b.v, b, (double)a.v); }
__device__ __forceinline__ AD operator/(const AD& a, const AD& b) {
    const double bv = b.v;
    return rec(a.v / b.v, a, 1.0 / bv, b, -(double)a.v / (bv * bv));
}
__device__ __forceinline__ AD operator-(const AD& a) { return rec1(-a.v, a, -1.0); }
__device__ __forceinline__ AD sqrt_(const AD& a) {
    const float r = sqrtf(a.v);
    return rec1(r, a, 0.5 / (double)r);
}
__device__ __forceinline__ AD hypot_(const AD& a, const AD& b) {
    const float h = hypotf(a.v, b.v);
    return rec(h, a, (double)a.v / h, b, (double)b.v / h);
}
__device__ __forceinline__ void sincos_(const AD& a, AD& s, AD& c) {
    float sv, cv;
    sincosf(a.v, &sv, &cv);
    s = rec1(sv, a, (double)cv);
    c = rec1(cv, a, -(double)sv);
}

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
};

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
    const V<T> plp[2] = {cv<T>(k.p0x, k.p0y), cv<T>(k.p1x, k.p1y)};
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
    const V<T> plp = idx ? cv<T>(k.p1x, k.p1y) : cv<T>(k.p0x, k.p0y);
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

}  // namespace diff
}  // namespace prgpu
