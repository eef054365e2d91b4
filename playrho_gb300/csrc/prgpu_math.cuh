// prgpu_math.cuh -- 2-D value types and the arithmetic of the PlayRho world step.
//
// Every helper keeps the reference's order of floating-point operations (the
// files named beside each one); the library is compiled with --fmad=false so
// that a*b+c stays two rounded operations, as in the reference's x86-64 build.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define PR_HD __host__ __device__ __forceinline__
#define PR_INF (__builtin_huge_valf())

namespace prgpu {

struct V2 {
    float x, y;
};

PR_HD V2 mk(float x, float y) { V2 r; r.x = x; r.y = y; return r; }
PR_HD V2 operator+(V2 a, V2 b) { return mk(a.x + b.x, a.y + b.y); }
PR_HD V2 operator-(V2 a, V2 b) { return mk(a.x - b.x, a.y - b.y); }
PR_HD V2 operator-(V2 a) { return mk(-a.x, -a.y); }
// Vector * scalar (Vector.hpp:497-504).
PR_HD V2 operator*(V2 a, float s) { return mk(a.x * s, a.y * s); }
// Vector / scalar multiplies by the reciprocal (Vector.hpp:511-519).
PR_HD V2 vdiv(V2 a, float s) { const float inv = 1.0f / s; return mk(a.x * inv, a.y * inv); }
// Dot accumulates from zero (Math.hpp:320-333).
PR_HD float dot(V2 a, V2 b) { float r = 0.0f; r += a.x * b.x; r += a.y * b.y; return r; }
// Cross (Math.hpp:365-386).
PR_HD float cross(V2 a, V2 b) { const float m = a.x * b.y; const float s = a.y * b.x; return m - s; }
// GetMagnitudeSquared (Math.hpp:274-283).
PR_HD float mag2(V2 a) { float r = 0.0f; r += a.x * a.x; r += a.y * a.y; return r; }
// GetRevPerpendicular / GetFwdPerpendicular (UnitVec.hpp:364-378).
PR_HD V2 revperp(V2 a) { return mk(-a.y, a.x); }
PR_HD V2 fwdperp(V2 a) { return mk(a.y, -a.x); }
// Rotate / InverseRotate of a vector by a unit vector (d2/Math.hpp).
PR_HD V2 rotate(V2 v, V2 q) { return mk((q.x * v.x) - (q.y * v.y), (q.y * v.x) + (q.x * v.y)); }
PR_HD V2 invrotate(V2 v, V2 q) { return mk((q.x * v.x) + (q.y * v.y), (q.x * v.y) - (q.y * v.x)); }
// UnitVec::Rotate (UnitVec.hpp:353-358).
PR_HD V2 urotate(V2 u, V2 a) { return mk(u.x * a.x - u.y * a.y, u.y * a.x + u.x * a.y); }

struct Xf {
    V2 p;
    V2 q;  // (cos, sin)
};
PR_HD V2 xform(V2 v, Xf t) { return rotate(v, t.q) + t.p; }
PR_HD V2 invxform(V2 v, Xf t) { return invrotate(v - t.p, t.q); }
// MulT (d2/Math.hpp).
PR_HD Xf mult(Xf A, Xf B) {
    Xf r;
    r.p = invrotate(B.p - A.p, A.q);
    r.q = urotate(B.q, mk(A.q.x, -A.q.y));
    return r;
}

PR_HD bool is_normal_f(float v) {
    const float a = fabsf(v);
    return a >= 1.17549435e-38f && a <= 3.40282347e+38f;
}
PR_HD bool almost_zero(float v) { return fabsf(v) < 1.17549435e-38f; }
// AlmostEqual with 4 ULP (Math.hpp:186-194).
PR_HD bool almost_equal(float a, float b) {
    int ulp = 4;
    for (; (a != b) && (ulp > 0); --ulp) a = nextafterf(a, b);
    return a == b;
}
PR_HD float clampf_(float v, float lo, float hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }
PR_HD float maxf_(float a, float b) { return (a < b) ? b : a; }
PR_HD float minf_(float a, float b) { return (b < a) ? b : a; }

// UnitVec::Get(x, y, fallback) (UnitVec.hpp:175-235).
PR_HD V2 unit_vector(V2 v, V2 fallback) {
    const float m2 = v.x * v.x + v.y * v.y;
    if (is_normal_f(m2)) {
        const float m = sqrtf(m2);
        const float inv = 1.0f / m;
        return mk(v.x * inv, v.y * inv);
    }
    const float m = hypotf(v.x, v.y);
    if (!is_normal_f(m)) return fallback;
    return mk(v.x / m, v.y / m);
}

// UnitVec::Get(angle) (UnitVec.cpp:27-30).
PR_HD V2 unit_from_angle(float a) {
    float s, c;
#ifdef __CUDA_ARCH__
    sincosf(a, &s, &c);
#else
    s = sinf(a);
    c = cosf(a);
#endif
    return mk(c, s);
}

// GetTransformation(Position, localCenter) (d2/Math.hpp).
PR_HD Xf get_xf(float px, float py, float angle, V2 lc) {
    Xf t;
    t.q = unit_from_angle(angle);
    t.p = mk(px, py) - rotate(lc, t.q);
    return t;
}

}  // namespace prgpu
