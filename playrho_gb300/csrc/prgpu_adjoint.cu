// prgpu_adjoint.cu -- StepAdjoint: reverse-mode gradients of a window of world
// steps, and the FP64 forward-mode tangent of the same window.
//
// A recorded step (d.tape set) runs the ordinary solver kernels, which also
// write what each constraint step starts from (prgpu_solver.cu sweep_*), the
// body state at the start of the solve, each world's sweep layout, the impulse
// sources of the post-solve contact update and the slots created
// (prgpu_tape.cuh).  From that record the step is walked backwards, turning
// adjoints of its outputs into adjoints of its inputs (body positions and
// velocities, stored contact and joint impulses, shape friction):
//
//  * k_adj_transfer, k_adj_prep: the post-solve contact update, sleep and the
//    impulse store, backwards; the constraints' geometry values;
//  * k_adj_sweeps, one block per world: the position iterations colour by
//    colour in reverse, position integration, the velocity iterations in
//    reverse (a block barrier separates two colours);
//  * k_adj_local, every constraint at once: warm start and constraint set-up;
//  * k_adj_bodies, every body: the velocity integration at the step's start.
//
// Every local vector-Jacobian product is written out by hand (prgpu_diff.cuh,
// *_vjp), in float.  k_tan_world walks the same record forwards with FP64
// tangents (Tan) from the templated restatement of each piece: the tangent
// kernel the dot-product test checks the adjoint against.
//
// Both passes take the forward's branches as recorded (contact set, clamps,
// block cases, island early exits, sleep), and each manifold's local geometry
// as constant within a step.  Revolute joints enter through their point rows.
#include <algorithm>

#include "prgpu_contact_ops.cuh"
#include "prgpu_kernels.cuh"
#include "prgpu_tape.cuh"

namespace prgpu {

using diff::Tan;

// ---- recording --------------------------------------------------------------------
__global__ void k_tape_body_start(DW d) {
    GRID_LOOP(b, d.n_bodies) {
        d.tape->p0[b] = d.b_pos1[b];
        d.tape->v0[b] = d.b_vel[b];
        d.tape->slept[b] = 0u;
    }
}

__global__ void k_tape_body_flags(DW d) {
    GRID_LOOP(b, d.n_bodies) d.tape->flags[b] = d.b_flags[b];
}

// grid-wide solve: constraints recorded after k_build_constraints
__global__ void k_tape_constraints(DW d) {
    GRID_LOOP(t, d.cnt->n_active) tape_constraint(d, t);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        StepTape* tp = d.tape;
        for (int k = 0; k <= kSerialColour + 1; ++k) tp->hdr[k] = d.cnt->colour_off[k];
        tp->hdr[kSerialColour + 2] = d.cnt->n_colours;
        tp->hdr[kSerialColour + 3] = d.cnt->n_active;
    }
}

void launch_tape_body_start(const DW& d, const Launch& L, cudaStream_t s) { k_tape_body_start<<<L.grid, L.threads, 0, s>>>(d); }
void launch_tape_body_flags(const DW& d, const Launch& L, cudaStream_t s) { k_tape_body_flags<<<L.grid, L.threads, 0, s>>>(d); }
void launch_tape_constraints(const DW& d, const Launch& L, cudaStream_t s) {
    k_tape_constraints<<<L.grid, L.threads, 0, s>>>(d);
}

// ---- helpers ------------------------------------------------------------------------
// One colour of world w's recorded sweeps, forwards or backwards, by one warp;
// the serial colour (the leftovers) runs on lane 0 in sweep order.
template <class F>
__device__ __forceinline__ void world_pass(uint32_t base, const uint32_t* off, int col, bool reverse, uint32_t lane,
                                           F&& f) {
    const uint32_t lo = base + off[col], hi = base + off[col + 1];
    if (lo == hi) return;
    if (col == kSerialColour) {
        if (lane == 0) {
            if (reverse) for (uint32_t t = hi; t-- > lo;) f(t);
            else for (uint32_t t = lo; t < hi; ++t) f(t);
        }
    } else {
        for (uint32_t t = lo + lane; t < hi; t += 32u) f(t);
    }
    __syncwarp();
}

// One colour of world w's recorded sweeps, backwards, by a block; the serial
// colour (the leftovers) runs on thread 0 in reverse sweep order.
template <class F>
__device__ __forceinline__ void block_pass(uint32_t base, const uint32_t* off, int col, F&& f) {
    const uint32_t lo = base + off[col], hi = base + off[col + 1];
    if (lo == hi) return;
    if (col == kSerialColour) {
        if (threadIdx.x == 0)
            for (uint32_t t = hi; t-- > lo;) f(t);
    } else {
        for (uint32_t t = lo + threadIdx.x; t < hi; t += blockDim.x) f(t);
    }
    __syncthreads();
}

// Recorded constraints of the step: the worlds' segments of sweep order are
// contiguous, so they are the positions [0, T).
__device__ __forceinline__ uint32_t recorded_constraints(const DW& d, const StepTape* tp) {
    const uint32_t w = d.n_worlds - 1u;
    return tp->wseg[2 * w] + tp->wseg[2 * w + 1];
}

// ---- manifold points that move with the bodies ----------------------------------------
// A point that ClipSegmentToLine (Manifold.cpp:61-102) made lies where the
// incident edge meets a side plane of the reference face, so its coordinates in
// the incident shape's frame depend on both bodies' positions at the collision,
// which are the positions the step starts from.  The rest of every manifold's
// local geometry (shape vertices, face normals, face centres) is constant.

// The clipped point in the incident shape's frame: the incident edge a-b (in its
// frame, transformation xi) meets the plane through the reference vertex vs with
// normal -e (side 0) or +e (side 1), e being the reference edge direction in
// its frame (transformation xr).
template <class T>
__device__ diff::V<T> clip_point_t(V2 a, V2 b, V2 vs, V2 e, bool side1, const diff::XfT<T>& xr,
                                   const diff::XfT<T>& xi) {
    using namespace diff;
    const V<T> A = xformt(cv<T>(a.x, a.y), xi), B = xformt(cv<T>(b.x, b.y), xi);
    const V<T> E = rotatet(cv<T>(e.x, e.y), xr.q);
    const V<T> N = side1 ? E : neg(E);
    const T off = dott(N, xformt(cv<T>(vs.x, vs.y), xr));
    const T da = dott(N, A) - off, db = dott(N, B) - off;
    const T f = da / (da - db);
    const V<T> D = sub(add(A, scale(sub(B, A), f)), xi.p);
    return V<T>{xi.q.x * D.x + xi.q.y * D.y, xi.q.x * D.y - xi.q.y * D.x};
}

struct MovingPoints {
    int n;              // clipped points (0: the contact's local geometry is constant)
    int idx[2];         // their index in the manifold
    bool side1[2];
    V2 vs[2];           // the side plane's reference vertex
    V2 a, b, e;         // incident edge, reference edge direction (own frames)
    bool flipped;       // the reference face is shape B's
};

// The contact's clipped points, found by colliding its shapes again at the
// recorded step-start positions; that must give back the recorded manifold bit
// for bit, else a replay mismatch is counted and the points are taken as fixed.
__device__ MovingPoints moving_points(const DW& d, const StepTape* tp, uint32_t t, const PC& pc) {
    MovingPoints m;
    m.n = 0;
    if (pc.type == M_CIRCLES) return m;
    const uint2 pr = tp->prox[t];
    Proxy A, B;
    load_proxy(d, pr.x, A);
    load_proxy(d, pr.y, B);
    if (A.count < 2 || B.count < 2) return m;  // a disk's manifold is fixed in both frames
    const float4 pa = tp->p0[pc.bA], pb = tp->p0[pc.bB];
    const float4 ma = d.b_mass[pc.bA], mb = d.b_mass[pc.bB];
    const Xf xfA = get_xf(pa.x, pa.y, pa.z, mk(ma.z, ma.w)), xfB = get_xf(pb.x, pb.y, pb.z, mk(mb.z, mb.w));
    PolyPick pick;
    const Man man = collide_shapes(A, xfA, B, xfB, d.conf->linearSlop, d.conf->maxCirclesRatio, &pick);
    bool same = (uint32_t)man.type == pc.type && (uint32_t)man.count == pc.count && man.ln.x == pc.lnx &&
                man.ln.y == pc.lny && man.lp.x == pc.lpx && man.lp.y == pc.lpy && man.plp[0].x == pc.p0x &&
                man.plp[0].y == pc.p0y;
    if (same && man.count == 2) same = man.plp[1].x == pc.p1x && man.plp[1].y == pc.p1y;
    if (!same) {
        atomicAdd(&tp->hdr[kTapeHdrMismatch], 1u);
        return m;
    }
    const Proxy& s0 = pick.flipped ? B : A;
    const Proxy& s1 = pick.flipped ? A : B;
    for (int i = 0; i < man.count; ++i) {
        const uint32_t c = pick.flipped ? cf_flip(man.cf[i]) : man.cf[i];
        if ((c & 0xffu) != CF_VERTEX || ((c >> 16) & 0xffu) != CF_FACE) continue;  // a shape vertex
        const unsigned side = (c >> 8) & 0xffu;
        m.idx[m.n] = i;
        m.side1[m.n] = side != pick.idx0;
        m.vs[m.n] = s0.vtx(side);
        ++m.n;
    }
    m.a = s1.vtx(pick.e1f);
    m.b = s1.vtx(pick.e1s);
    m.e = revperp(s0.nrm(pick.idx0));
    m.flipped = pick.flipped != 0u;
    return m;
}

// Tangents of the local points (p0x p0y p1x p1y) for tangents dA, dB of the
// step-start positions (x y angle) of bodies A and B.
__device__ void moving_points_tan(const DW& d, const StepTape* tp, const PC& pc, const MovingPoints& m,
                                  const double* dA, const double* dB, double* out) {
    out[0] = out[1] = out[2] = out[3] = 0.0;
    const float4 pa = tp->p0[pc.bA], pb = tp->p0[pc.bB];
    const float4 ma = d.b_mass[pc.bA], mb = d.b_mass[pc.bB];
    const diff::XfT<Tan> xfA = diff::get_xft(Tan{pa.x, dA[0]}, Tan{pa.y, dA[1]}, Tan{pa.z, dA[2]}, ma.z, ma.w);
    const diff::XfT<Tan> xfB = diff::get_xft(Tan{pb.x, dB[0]}, Tan{pb.y, dB[1]}, Tan{pb.z, dB[2]}, mb.z, mb.w);
    for (int k = 0; k < m.n; ++k) {
        const diff::V<Tan> q = m.flipped ? clip_point_t(m.a, m.b, m.vs[k], m.e, m.side1[k], xfB, xfA)
                                         : clip_point_t(m.a, m.b, m.vs[k], m.e, m.side1[k], xfA, xfB);
        out[2 * m.idx[k]] = q.x.d;
        out[2 * m.idx[k] + 1] = q.y.d;
    }
}

// Reverse: pb (x y angle of A, then B) += J^T lb, J the local points' Jacobian.
// In the incident frame the clipped point is a + f (b - a) (clip_point_t with
// the incident transformation taken out), so only the scalar
// f = da / (da - db) moves, da and db being the side plane's signed distances
// N.(Aw - Vw) and N.(Bw - Vw) of the incident edge's world points Aw, Bw, with
// Vw the plane's world vertex and N = +-R_r e its normal.  The adjoint of f is
// lb.(b - a); with rp(v) = (-v.y, v.x), d/d(angle) of a rotated vector R v is
// rp(R v), so:
//   incident centre  (da_bar + db_bar) N
//   incident angle   da_bar N.rp(Aw - Pi) + db_bar N.rp(Bw - Pi)
//   reference centre -(da_bar + db_bar) N
//   reference angle  da_bar (rp(N).(Aw - Vw) - N.rp(Vw - Pr)) + db_bar (rp(N).(Bw - Vw) - N.rp(Vw - Pr))
// (Pi, Pr the bodies' centres).  One pass instead of a forward-mode evaluation
// per position coordinate.  The distances are small differences of world
// coordinates, so the pass runs in FP64 from each body's (float) rotation;
// moving_points_tan keeps the forward-mode form for the tangent that checks it.
__device__ void moving_points_vjp(const DW& d, const StepTape* tp, const PC& pc, const MovingPoints& m,
                                  const float* lb, float* pb) {
    struct D2 { double x, y; };
    auto sub2 = [](D2 u, D2 v) { return D2{u.x - v.x, u.y - v.y}; };
    auto dot2 = [](D2 u, D2 v) { return u.x * v.x + u.y * v.y; };
    auto rp2 = [](D2 u) { return D2{-u.y, u.x}; };
    // R v + P - R lc: the world point of local point v of a body at centre P
    auto world = [](V2 v, V2 q, D2 P, V2 lc) {
        const double x = (double)v.x - lc.x, y = (double)v.y - lc.y;
        return D2{P.x + (q.x * x - q.y * y), P.y + (q.y * x + q.x * y)};
    };
    const float4 pa = tp->p0[pc.bA], pbb = tp->p0[pc.bB];
    const float4 ma = d.b_mass[pc.bA], mb = d.b_mass[pc.bB];
    const float4& pr = m.flipped ? pbb : pa;  // reference body
    const float4& pi = m.flipped ? pa : pbb;  // incident body
    const float4& mr = m.flipped ? mb : ma;
    const float4& mi = m.flipped ? ma : mb;
    const V2 qr = unit_from_angle(pr.z), qi = unit_from_angle(pi.z);
    const D2 Pr{pr.x, pr.y}, Pi{pi.x, pi.y};
    float* gr = m.flipped ? pb + 3 : pb;  // reference body's x y angle
    float* gi = m.flipped ? pb : pb + 3;  // incident body's
    const D2 Aw = world(m.a, qi, Pi, mk(mi.z, mi.w)), Bw = world(m.b, qi, Pi, mk(mi.z, mi.w));
    const D2 E{(double)qr.x * m.e.x - (double)qr.y * m.e.y, (double)qr.y * m.e.x + (double)qr.x * m.e.y};
    const D2 ba{(double)m.b.x - m.a.x, (double)m.b.y - m.a.y};
    for (int k = 0; k < m.n; ++k) {
        const D2 N = m.side1[k] ? E : D2{-E.x, -E.y};
        const D2 Vw = world(m.vs[k], qr, Pr, mk(mr.z, mr.w));
        const D2 u = sub2(Aw, Vw), w = sub2(Bw, Vw);
        const double da = dot2(N, u), db = dot2(N, w), den = da - db;
        if (den == 0.0) continue;  // no crossing: ClipSegmentToLine made no point here
        const int i = m.idx[k];
        const double fbar = lb[2 * i] * ba.x + lb[2 * i + 1] * ba.y;
        const double den2 = den * den;
        const double dab = -fbar * db / den2, dbb = fbar * da / den2;
        const double s = dab + dbb;
        const D2 rN = rp2(N), rV = rp2(sub2(Vw, Pr));
        gi[0] += (float)(s * N.x);
        gi[1] += (float)(s * N.y);
        gi[2] += (float)(dab * dot2(N, rp2(sub2(Aw, Pi))) + dbb * dot2(N, rp2(sub2(Bw, Pi))));
        gr[0] -= (float)(s * N.x);
        gr[1] -= (float)(s * N.y);
        gr[2] += (float)(dab * (dot2(rN, u) - dot2(N, rV)) + dbb * (dot2(rN, w) - dot2(N, rV)));
    }
}

// ---- joints ---------------------------------------------------------------------------
__device__ void adj_joint_position(const DW& d, const StepTape* tp, const AdjState& a, uint32_t t, uint32_t j, int it) {
    const float4* r = tp->pos + 2 * ((size_t)it * tp->kcap + t);
    if (r[0].w == 0.f) return;  // island already within tolerance
    const uint32_t A = d.j_bodies[2 * j], B = d.j_bodies[2 * j + 1];
    const diff::JointK k = joint_k(d, j);
    const float p[6] = {r[0].x, r[0].y, r[0].z, r[1].x, r[1].y, r[1].z};
    float yb[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, pb[6];
    if (k.writableA) { const float4 g = a.pbar[A]; yb[0] = g.x; yb[1] = g.y; yb[2] = g.z; }
    if (k.writableB) { const float4 g = a.pbar[B]; yb[3] = g.x; yb[4] = g.y; yb[5] = g.z; }
    diff::joint_position_vjp(k, p, yb, pb);
    if (k.writableA) a.pbar[A] = make_float4(pb[0], pb[1], pb[2], 0.f);
    if (k.writableB) a.pbar[B] = make_float4(pb[3], pb[4], pb[5], 0.f);
}

__device__ void adj_joint_velocity(const DW& d, const StepTape* tp, const AdjState& a, uint32_t t, uint32_t j, int it) {
    const float4* r = tp->vel + 3 * ((size_t)it * tp->kcap + t);
    const uint32_t A = d.j_bodies[2 * j], B = d.j_bodies[2 * j + 1];
    const diff::JointK k = joint_k(d, j);
    const float* gv = a.gval + (size_t)t * kGeomWords;
    diff::JGeom<float> g;
    g.rA = {gv[0], gv[1]}; g.rB = {gv[2], gv[3]};
    g.exx = gv[4]; g.eyx = gv[5]; g.eyy = gv[6];
    const diff::Pair3<float> v{r[0].x, r[0].y, r[0].z, r[1].x, r[1].y, r[1].z};
    float vbA[3] = {0.f, 0.f, 0.f}, vbB[3] = {0.f, 0.f, 0.f};
    if (k.writableA) { const float4 q = a.vbar[A]; vbA[0] = q.x; vbA[1] = q.y; vbA[2] = q.z; }
    if (k.writableB) { const float4 q = a.vbar[B]; vbB[0] = q.x; vbB[1] = q.y; vbB[2] = q.z; }
    const float4 l = a.lbar[t];
    float ib[2] = {l.x, l.y};
    float gb[diff::kJointGeomWords] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    diff::joint_velocity_vjp(k, g, v, vbA, vbB, ib, gb);
    if (k.writableA) a.vbar[A] = make_float4(vbA[0], vbA[1], vbA[2], 0.f);
    if (k.writableB) a.vbar[B] = make_float4(vbB[0], vbB[1], vbB[2], 0.f);
    a.lbar[t] = make_float4(ib[0], ib[1], 0.f, 0.f);
    float* gbar = a.gbar + (size_t)t * kGeomWords;
    for (int q = 0; q < diff::kJointGeomWords; ++q) gbar[q] += gb[q];
}

// ---- adjoint ------------------------------------------------------------------------
// Reverse of the post-solve contact update: manifold impulse adjoints go back
// to the points they were copied from; slots created by the step had none.
__global__ void k_adj_transfer(DW d, const StepTape* tp, AdjState a, uint32_t n_slots) {
    GRID_LOOP(s, n_slots) {
        const int8_t s0 = tp->src[2 * (size_t)s], s1 = tp->src[2 * (size_t)s + 1];
        const float4 m = a.mbar[s];
        float4 o = m;
        if (tp->created[s]) {
            o = make_float4(0.f, 0.f, 0.f, 0.f);
        } else if (s0 != -2) {
            o = make_float4(0.f, 0.f, 0.f, 0.f);
            if (s0 == 0) { o.x += m.x; o.y += m.y; } else if (s0 == 1) { o.z += m.x; o.w += m.y; }
            if (s1 == 0) { o.x += m.z; o.y += m.w; } else if (s1 == 1) { o.z += m.z; o.w += m.w; }
        }
        a.mtmp[s] = o;
    }
}

// The step's end, backwards: sleep zeroed the slept bodies' velocities; the
// stored impulses were the iterations' final ones.  Also the constraints'
// geometry values, which the sweeps' products need.
__global__ void k_adj_prep(DW d, const StepTape* tp, AdjState a) {
    GRID_LOOP(b, d.n_bodies) {
        if (tp->slept[b]) a.vbar[b] = make_float4(0.f, 0.f, 0.f, 0.f);
        a.vibar[b] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (tp->flags[b] & BF_SOLVED) {
            float vx = tp->v0[b].x, vy = tp->v0[b].y, vw = tp->v0[b].z;
            start_velocity(d, b, vx, vy, vw);
            a.vi[b] = make_float4(vx, vy, vw, 0.f);
        } else {
            a.vi[b] = tp->v0[b];
        }
    }
    const uint32_t T = recorded_constraints(d, tp);
    GRID_LOOP(t, T) {
        const uint32_t slot = tp->t_id[t];
        float* gb = a.gbar + (size_t)t * kGeomWords;
        for (int q = 0; q < kGeomWords; ++q) gb[q] = 0.f;
        if (slot & 0x80000000u) {  // joint: its stored impulse and its geometry
            const uint32_t j = slot & 0x7fffffffu;
            a.lbar[t] = a.jbar[j];
            a.jbar[j] = make_float4(0.f, 0.f, 0.f, 0.f);
            const diff::JGeom<float> g =
                diff::joint_geom_t(joint_k(d, j), tp->p0[d.j_bodies[2 * j]].z, tp->p0[d.j_bodies[2 * j + 1]].z);
            diff::pack_jgeom(g, a.gval + (size_t)t * kGeomWords);
            continue;
        }
        a.lbar[t] = a.mbar[slot];
        a.mbar[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
        const PC& pc = tp->pc[t];
        const diff::Geom<float> g = replay_geom(d, tp, t, contact_k(d, pc, tp->cinfo[t]), tp->cinfo[t].z);
        pack_geom(g, a.gval + (size_t)t * kGeomWords);
    }
}

// The iterated part of world w's solve, backwards, by one block: the position
// iterations colour by colour in reverse, position integration, then the
// velocity iterations in reverse.  A block barrier separates two colours.
// kWide: the instance for blocks of kAdjSweepMaxThreads, held to 64 registers so
// that two blocks fit on a multiprocessor.
template <bool kWide>
__global__ void __launch_bounds__(kAdjSweepMaxThreads, kWide ? 2 : 1) k_adj_sweeps(DW d, const StepTape* tp, AdjState a) {
    const DConf& c = *d.conf;
    const float h = c.deltaTime;
    const uint32_t w = blockIdx.x;
    const uint32_t b0 = d.w_body_off[w], b1 = d.w_body_off[w + 1];
    const uint32_t base = tp->wseg[2 * w], n = tp->wseg[2 * w + 1];
    // the world's colour table, and the highest parallel colour in use
    __shared__ uint32_t off[kColStride];
    for (uint32_t q = threadIdx.x; q < (uint32_t)kColStride; q += blockDim.x)
        off[q] = tp->wcol[(size_t)w * kColStride + q];
    __syncthreads();
    int top = 0;
    for (int q = 0; q < kMaxColours; ++q)
        if (off[q + 1] > off[q]) top = q + 1;
    // colours in reverse sweep order: the serial one, then top-1 .. 0
    auto prev_col = [&](int col) { return col == kSerialColour ? top - 1 : col - 1; };
    if (n) {
        for (int it = tp->ip - 1; it >= 0; --it) {
            for (int col = kSerialColour; col >= 0; col = prev_col(col)) {
                block_pass(base, off, col, [&](uint32_t t) {
                    const uint32_t id = tp->t_id[t];
                    if (id & 0x80000000u) { adj_joint_position(d, tp, a, t, id & 0x7fffffffu, it); return; }
                    const float4* r = tp->pos + 2 * ((size_t)it * tp->kcap + t);
                    if (r[0].w == 0.f) return;  // island already within tolerance
                    const PC& pc = tp->pc[t];
                    const diff::ContactK k = contact_k(d, pc, tp->cinfo[t]);
                    const float p[6] = {r[0].x, r[0].y, r[0].z, r[1].x, r[1].y, r[1].z};
                    float yb[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, pb[6];
                    if (k.writableA) { const float4 g = a.pbar[pc.bA]; yb[0] = g.x; yb[1] = g.y; yb[2] = g.z; }
                    if (k.writableB) { const float4 g = a.pbar[pc.bB]; yb[3] = g.x; yb[4] = g.y; yb[5] = g.z; }
                    diff::solve_position_vjp(k, c, p, yb, pb, a.gbar + (size_t)t * kGeomWords + kLocalPts);
                    // bodies that are not dynamic are not differentiated (and can be
                    // shared within a colour)
                    if (k.writableA) a.pbar[pc.bA] = make_float4(pb[0], pb[1], pb[2], 0.f);
                    if (k.writableB) a.pbar[pc.bB] = make_float4(pb[3], pb[4], pb[5], 0.f);
                });
            }
        }
    }
    // position integration p1 = p0 + h v
    for (uint32_t b = b0 + threadIdx.x; b < b1; b += blockDim.x) {
        if (!(tp->flags[b] & BF_SOLVED)) continue;
        const float4 pb = a.pbar[b];
        float4 vb = a.vbar[b];
        vb.x += h * pb.x; vb.y += h * pb.y; vb.z += h * pb.z;
        a.vbar[b] = vb;
    }
    __syncthreads();
    if (n) {
        for (int it = tp->iv - 1; it >= 0; --it) {
            for (int col = kSerialColour; col >= 0; col = prev_col(col)) {
                block_pass(base, off, col, [&](uint32_t t) {
                    const uint32_t id = tp->t_id[t];
                    if (id & 0x80000000u) { adj_joint_velocity(d, tp, a, t, id & 0x7fffffffu, it); return; }
                    const float4* r = tp->vel + 3 * ((size_t)it * tp->kcap + t);
                    const PC& pc = tp->pc[t];
                    const diff::ContactK k = contact_k(d, pc, tp->cinfo[t]);
                    const diff::Geom<float> g = unpack_geom(a.gval + (size_t)t * kGeomWords);
                    const diff::Pair3<float> vin{r[0].x, r[0].y, r[0].z, r[1].x, r[1].y, r[1].z};
                    const diff::Imp<float> iin{r[2].x, r[2].y, r[2].z, r[2].w};
                    const float4 ga = a.vbar[pc.bA], gbv = a.vbar[pc.bB], gl = a.lbar[t];
                    float vbA[3] = {0.f, 0.f, 0.f}, vbB[3] = {0.f, 0.f, 0.f};
                    if (k.writableA) { vbA[0] = ga.x; vbA[1] = ga.y; vbA[2] = ga.z; }
                    if (k.writableB) { vbB[0] = gbv.x; vbB[1] = gbv.y; vbB[2] = gbv.z; }
                    float ib[4] = {gl.x, gl.y, gl.z, gl.w};
                    diff::GeomBar gb = {};
                    diff::solve_velocity_vjp(k, g, vin, iin, vbA, vbB, ib, gb);
                    if (k.writableA) a.vbar[pc.bA] = make_float4(vbA[0], vbA[1], vbA[2], 0.f);
                    if (k.writableB) a.vbar[pc.bB] = make_float4(vbB[0], vbB[1], vbB[2], 0.f);
                    a.lbar[t] = make_float4(ib[0], ib[1], ib[2], ib[3]);
                    float* gbar = a.gbar + (size_t)t * kGeomWords;
                    gbar[0] += gb.n[0]; gbar[1] += gb.n[1];
                    for (int j = 0; j < 2; ++j) {
                        gbar[2 + 4 * j] += gb.rA[j][0]; gbar[3 + 4 * j] += gb.rA[j][1];
                        gbar[4 + 4 * j] += gb.rB[j][0]; gbar[5 + 4 * j] += gb.rB[j][1];
                    }
                    gbar[10] += gb.nm[0]; gbar[11] += gb.tm[0]; gbar[12] += gb.nm[1]; gbar[13] += gb.tm[1];
                    gbar[14] += gb.vb[0]; gbar[15] += gb.vb[1];
                    gbar[16] += gb.k00; gbar[17] += gb.k11; gbar[18] += gb.k01;
                    gbar[19] += gb.m00; gbar[20] += gb.m11; gbar[21] += gb.m01; gbar[22] += gb.mu;
                });
            }
        }
    }
}

// Warm start and constraint set-up, backwards, for every recorded constraint at
// once: the warm start's velocity change does not depend on the velocities, and
// the set-up reads the state at the start of the solve, so neither pass has an
// order.
__global__ void k_adj_local(DW d, const StepTape* tp, AdjState a) {
    const DConf& c = *d.conf;
    const uint32_t T = recorded_constraints(d, tp);
    GRID_LOOP(t, T) {
        const uint32_t slot = tp->t_id[t];
        float* gbar = a.gbar + (size_t)t * kGeomWords;
        const float* gv = a.gval + (size_t)t * kGeomWords;
        if (slot & 0x80000000u) {  // joint
            const uint32_t j = slot & 0x7fffffffu;
            const uint32_t A = d.j_bodies[2 * j], B = d.j_bodies[2 * j + 1];
            const diff::JointK k = joint_k(d, j);
            if (c.doWarmStart) {  // else the impulses restart from zero; velocities untouched
                diff::JGeom<float> g;
                g.rA = {gv[0], gv[1]}; g.rB = {gv[2], gv[3]};
                g.exx = gv[4]; g.eyx = gv[5]; g.eyy = gv[6];
                const float4 i0 = tp->imp0[t], l = a.lbar[t];
                float vbA[3] = {0.f, 0.f, 0.f}, vbB[3] = {0.f, 0.f, 0.f};
                if (k.writableA) { const float4 q = a.vbar[A]; vbA[0] = q.x; vbA[1] = q.y; vbA[2] = q.z; }
                if (k.writableB) { const float4 q = a.vbar[B]; vbB[0] = q.x; vbB[1] = q.y; vbB[2] = q.z; }
                const float lb[2] = {l.x, l.y};
                float ib[2];
                diff::joint_warm_vjp(k, g, c.dtRatio, i0.x, i0.y, vbA, vbB, lb, ib, gbar);
                a.jbar[j] = make_float4(ib[0], ib[1], 0.f, 0.f);
            }
            float aAb, aBb;
            diff::joint_geom_vjp(k, tp->p0[A].z, tp->p0[B].z, gbar, &aAb, &aBb);
            if (k.writableA) atomicAdd(a.pvacc + 6 * (size_t)A + 2, (double)aAb);
            if (k.writableB) atomicAdd(a.pvacc + 6 * (size_t)B + 2, (double)aBb);
            continue;
        }
        const PC& pc = tp->pc[t];
        const float4 ci = tp->cinfo[t];
        const diff::ContactK k = contact_k(d, pc, ci);
        float4 li = a.lbar[t];  // adjoint of the impulses the first iteration started from
        if (c.doWarmStart) {
            const float4 i0 = tp->imp0[t];
            const diff::Imp<float> im{i0.x, i0.y, i0.z, i0.w};
            float vbA[3] = {0.f, 0.f, 0.f}, vbB[3] = {0.f, 0.f, 0.f};
            if (k.writableA) { const float4 q = a.vbar[pc.bA]; vbA[0] = q.x; vbA[1] = q.y; vbA[2] = q.z; }
            if (k.writableB) { const float4 q = a.vbar[pc.bB]; vbB[0] = q.x; vbB[1] = q.y; vbB[2] = q.z; }
            float ib[4] = {0.f, 0.f, 0.f, 0.f};
            diff::warm_start_vjp(k, unpack_geom(gv), im, vbA, vbB, ib, gbar);
            li.x += ib[0]; li.y += ib[1]; li.z += ib[2]; li.w += ib[3];
        }
        // VelocityConstraint's impulses are the stored ones times dtRatio
        float4 m = a.mbar[slot];
        m.x += li.x * c.dtRatio; m.y += li.y * c.dtRatio; m.z += li.z * c.dtRatio; m.w += li.w * c.dtRatio;
        a.mbar[slot] = m;
        // constraint set-up: geometry from the positions and velocities at the
        // start of the solve and the contact's friction
        const float4 pa = tp->p0[pc.bA], pb = tp->p0[pc.bB], va = a.vi[pc.bA], vb = a.vi[pc.bB];
        const diff::Pair3<float> p{pa.x, pa.y, pa.z, pb.x, pb.y, pb.z};
        const diff::Pair3<float> v{va.x, va.y, va.z, vb.x, vb.y, vb.z};
        float pbar[6], vbar[6], mub;
        diff::build_geom_vjp(k, p, v, ci.z, c, gbar, pbar, vbar, &mub, gbar + kLocalPts);
        // clipped manifold points moved with the positions the step started from
        const MovingPoints mp = moving_points(d, tp, t, pc);
        if (mp.n) moving_points_vjp(d, tp, pc, mp, gbar + kLocalPts, pbar);
        // summed per body in FP64 (k_adj_bodies folds the sums in): the order of
        // the atomics then leaves the float result unchanged, so the reverse pass
        // gives the same gradients on every run
        double* accA = a.pvacc + 6 * (size_t)pc.bA;
        double* accB = a.pvacc + 6 * (size_t)pc.bB;
        for (int q = 0; q < 3; ++q) {
            atomicAdd(accA + q, (double)pbar[q]);
            atomicAdd(accB + q, (double)pbar[3 + q]);
            atomicAdd(accA + 3 + q, (double)vbar[q]);
            atomicAdd(accB + 3 + q, (double)vbar[3 + q]);
        }
        // MixFriction: sqrt(fA fB)
        if (mub != 0.f && ci.z > 0.f) {
            const uint2 pr = tp->prox[t];
            const float fa = d.s_mat[pr.x].x, fb = d.s_mat[pr.y].x;
            atomicAdd(&a.fbar[pr.x], mub * fb / (2.0f * ci.z));
            atomicAdd(&a.fbar[pr.y], mub * fa / (2.0f * ci.z));
        }
    }
}

// velocity at the start of the solve from the velocity the step started with
__global__ void k_adj_bodies(DW d, const StepTape* tp, AdjState a) {
    GRID_LOOP(b, d.n_bodies) {
        // k_adj_local's FP64 sums: position adjoints added to the sweeps', the
        // start-velocity adjoints as they are; cleared for the next step
        double* acc = a.pvacc + 6 * (size_t)b;
        float4 p = a.pbar[b];
        p.x = (float)((double)p.x + acc[0]);
        p.y = (float)((double)p.y + acc[1]);
        p.z = (float)((double)p.z + acc[2]);
        a.pbar[b] = p;
        a.vibar[b] = make_float4((float)acc[3], (float)acc[4], (float)acc[5], 0.f);
        for (int q = 0; q < 6; ++q) acc[q] = 0.0;
        if (!(tp->flags[b] & BF_SOLVED)) continue;
        const float4 v0 = tp->v0[b];
        const float4 g1 = a.vbar[b], g2 = a.vibar[b];
        float bar[3] = {g1.x + g2.x, g1.y + g2.y, g1.z + g2.z};
        diff::integrate_velocity_vjp(is_accelerable(d.b_flags[b]), d.b_acc[b], d.b_damp[b], *d.conf, v0.x, v0.y, v0.z,
                                     bar);
        a.vbar[b] = make_float4(bar[0], bar[1], bar[2], 0.f);
    }
}

// ---- tangent (FP64 forward mode) ------------------------------------------------------
__device__ diff::Geom<Tan> geom_tan(const float* gv, const double* gd) {
    diff::Geom<Tan> g;
    auto T = [&](int q) { return Tan{gv[q], gd[q]}; };
    g.n = {T(0), T(1)};
    for (int j = 0; j < 2; ++j) {
        g.rA[j] = {T(2 + 4 * j), T(3 + 4 * j)};
        g.rB[j] = {T(4 + 4 * j), T(5 + 4 * j)};
    }
    g.nm[0] = T(10); g.tm[0] = T(11); g.nm[1] = T(12); g.tm[1] = T(13);
    g.vb[0] = T(14); g.vb[1] = T(15);
    g.k00 = T(16); g.k11 = T(17); g.k01 = T(18); g.m00 = T(19); g.m11 = T(20); g.m01 = T(21);
    g.mu = T(22);
    g.cnt = __float_as_int(gv[23]);
    return g;
}

__device__ __forceinline__ diff::JGeom<Tan> jgeom_tan(const float* gv, const double* gd) {
    diff::JGeom<Tan> g;
    g.rA = {Tan{gv[0], gd[0]}, Tan{gv[1], gd[1]}};
    g.rB = {Tan{gv[2], gd[2]}, Tan{gv[3], gd[3]}};
    g.exx = Tan{gv[4], gd[4]}; g.eyx = Tan{gv[5], gd[5]}; g.eyy = Tan{gv[6], gd[6]};
    return g;
}

__global__ void k_tan_transfer(DW d, const StepTape* tp, TanState s, uint32_t n_slots) {
    GRID_LOOP(q, n_slots) {
        const int8_t s0 = tp->src[2 * (size_t)q], s1 = tp->src[2 * (size_t)q + 1];
        const double* m = s.mdot + 4 * (size_t)q;
        double o[4] = {m[0], m[1], m[2], m[3]};
        if (tp->created[q]) {
            o[0] = o[1] = o[2] = o[3] = 0.0;
        } else if (s0 != -2) {
            o[0] = (s0 >= 0) ? m[2 * s0] : 0.0; o[1] = (s0 >= 0) ? m[2 * s0 + 1] : 0.0;
            o[2] = (s1 >= 0) ? m[2 * s1] : 0.0; o[3] = (s1 >= 0) ? m[2 * s1 + 1] : 0.0;
        }
        for (int k = 0; k < 4; ++k) s.mtmp[4 * (size_t)q + k] = o[k];
    }
}

__global__ void __launch_bounds__(32) k_tan_world(DW d, const StepTape* tp, TanState s, float* gval) {
    const DConf& c = *d.conf;
    const float h = c.deltaTime;
    const uint32_t w = blockIdx.x, lane = threadIdx.x;
    const uint32_t b0 = d.w_body_off[w], b1 = d.w_body_off[w + 1];
    const uint32_t base = tp->wseg[2 * w], n = tp->wseg[2 * w + 1];
    const uint32_t* off = tp->wcol + (size_t)w * kColStride;
    for (uint32_t b = b0 + lane; b < b1; b += 32u) {
        double* vi = s.vidot + 3 * (size_t)b;
        const double* v = s.vdot + 3 * (size_t)b;
        if (tp->flags[b] & BF_SOLVED) {
            const float4 v0 = tp->v0[b];
            Tan vx{v0.x, v[0]}, vy{v0.y, v[1]}, vw{v0.z, v[2]};
            start_velocity(d, b, vx, vy, vw);
            vi[0] = vx.d; vi[1] = vy.d; vi[2] = vw.d;
        } else {
            vi[0] = v[0]; vi[1] = v[1]; vi[2] = v[2];
        }
    }
    __syncwarp();
    // constraint geometry and its tangent; the iterations start from the stored impulses
    for (uint32_t t = base + lane; t < base + n; t += 32u) {
        const uint32_t slot = tp->t_id[t];
        if (slot & 0x80000000u) {  // joint: geometry from the angles; the stored impulse
            const uint32_t j = slot & 0x7fffffffu;
            const uint32_t A = d.j_bodies[2 * j], B = d.j_bodies[2 * j + 1];
            const diff::JGeom<Tan> g = diff::joint_geom_t(joint_k(d, j), Tan{tp->p0[A].z, s.pdot[3 * (size_t)A + 2]},
                                                          Tan{tp->p0[B].z, s.pdot[3 * (size_t)B + 2]});
            diff::pack_jgeom(g, gval + (size_t)t * kGeomWords);
            double* gd = s.gdot + (size_t)t * kGeomWords;
            gd[0] = g.rA.x.d; gd[1] = g.rA.y.d; gd[2] = g.rB.x.d; gd[3] = g.rB.y.d;
            gd[4] = g.exx.d; gd[5] = g.eyx.d; gd[6] = g.eyy.d;
            double* l = s.ldot + 4 * (size_t)t;
            l[0] = c.doWarmStart ? s.jdot[2 * (size_t)j] : 0.0;
            l[1] = c.doWarmStart ? s.jdot[2 * (size_t)j + 1] : 0.0;
            l[2] = l[3] = 0.0;
            continue;
        }
        const PC& pc = tp->pc[t];
        const float4 ci = tp->cinfo[t];
        diff::ContactK k = contact_k(d, pc, ci);
        const float4 pa = tp->p0[pc.bA], pb = tp->p0[pc.bB];
        float vax = tp->v0[pc.bA].x, vay = tp->v0[pc.bA].y, vaw = tp->v0[pc.bA].z;
        float vbx = tp->v0[pc.bB].x, vby = tp->v0[pc.bB].y, vbw = tp->v0[pc.bB].z;
        if (tp->flags[pc.bA] & BF_SOLVED) start_velocity(d, pc.bA, vax, vay, vaw);
        if (tp->flags[pc.bB] & BF_SOLVED) start_velocity(d, pc.bB, vbx, vby, vbw);
        const double* dpa = s.pdot + 3 * (size_t)pc.bA;
        const double* dpb = s.pdot + 3 * (size_t)pc.bB;
        const double* dva = s.vidot + 3 * (size_t)pc.bA;
        const double* dvb = s.vidot + 3 * (size_t)pc.bB;
        const uint2 pr = tp->prox[t];
        double mud = 0.0;
        if (ci.z > 0.f) {
            const float fa = d.s_mat[pr.x].x, fb = d.s_mat[pr.y].x;
            mud = (fb * s.fdot[pr.x] + fa * s.fdot[pr.y]) / (2.0 * ci.z);
        }
        double* gd = s.gdot + (size_t)t * kGeomWords;
        const MovingPoints mp = moving_points(d, tp, t, pc);
        if (mp.n) moving_points_tan(d, tp, pc, mp, dpa, dpb, k.dp);
        for (int q = 0; q < 4; ++q) gd[kLocalPts + q] = k.dp[q];
        const diff::Pair3<Tan> p{{pa.x, dpa[0]}, {pa.y, dpa[1]}, {pa.z, dpa[2]}, {pb.x, dpb[0]}, {pb.y, dpb[1]}, {pb.z, dpb[2]}};
        const diff::Pair3<Tan> v{{vax, dva[0]}, {vay, dva[1]}, {vaw, dva[2]}, {vbx, dvb[0]}, {vby, dvb[1]}, {vbw, dvb[2]}};
        const diff::Geom<Tan> g = diff::build_geom(k, p, v, Tan{ci.z, mud}, c);
        pack_geom(g, gval + (size_t)t * kGeomWords);
        gd[0] = g.n.x.d; gd[1] = g.n.y.d;
        for (int j = 0; j < 2; ++j) {
            gd[2 + 4 * j] = g.rA[j].x.d; gd[3 + 4 * j] = g.rA[j].y.d;
            gd[4 + 4 * j] = g.rB[j].x.d; gd[5 + 4 * j] = g.rB[j].y.d;
        }
        gd[10] = g.nm[0].d; gd[11] = g.tm[0].d; gd[12] = g.nm[1].d; gd[13] = g.tm[1].d;
        gd[14] = g.vb[0].d; gd[15] = g.vb[1].d; gd[16] = g.k00.d; gd[17] = g.k11.d; gd[18] = g.k01.d;
        gd[19] = g.m00.d; gd[20] = g.m11.d; gd[21] = g.m01.d; gd[22] = g.mu.d; gd[23] = 0.0;
        const double* m = s.mdot + 4 * (size_t)slot;
        double* l = s.ldot + 4 * (size_t)t;
        for (int q = 0; q < 4; ++q) l[q] = m[q] * c.dtRatio;
    }
    // velocities after integration
    for (uint32_t b = b0 + lane; b < b1; b += 32u) {
        double* v = s.vdot + 3 * (size_t)b;
        const double* vi = s.vidot + 3 * (size_t)b;
        v[0] = vi[0]; v[1] = vi[1]; v[2] = vi[2];
    }
    __syncwarp();
    auto body_pair = [&](uint32_t A, uint32_t B, float4 ra, float4 rb, const double* basev) {
        const double* a3 = basev + 3 * (size_t)A;
        const double* b3 = basev + 3 * (size_t)B;
        return diff::Pair3<Tan>{{ra.x, a3[0]}, {ra.y, a3[1]}, {ra.z, a3[2]}, {rb.x, b3[0]}, {rb.y, b3[1]}, {rb.z, b3[2]}};
    };
    auto store_pair = [&](const auto& k, uint32_t A, uint32_t B, const diff::Pair3<Tan>& v, double* basev) {
        if (k.writableA) { double* a3 = basev + 3 * (size_t)A; a3[0] = v.ax.d; a3[1] = v.ay.d; a3[2] = v.az.d; }
        if (k.writableB) { double* b3 = basev + 3 * (size_t)B; b3[0] = v.bx.d; b3[1] = v.by.d; b3[2] = v.bz.d; }
    };
    auto joint_step = [&](uint32_t t, uint32_t j, const float4* r, bool position, bool warm) {
        const uint32_t A = d.j_bodies[2 * j], B = d.j_bodies[2 * j + 1];
        const diff::JointK k = joint_k(d, j);
        double* basev = position ? s.pdot : s.vdot;
        diff::Pair3<Tan> v = body_pair(A, B, r[0], r[1], basev);
        if (position) {
            diff::joint_position_t(k, v);
        } else {
            double* l = s.ldot + 4 * (size_t)t;
            const float4 i = warm ? tp->imp0[t] : r[2];
            Tan ix{i.x, l[0]}, iy{i.y, l[1]};
            const diff::JGeom<Tan> g = jgeom_tan(gval + (size_t)t * kGeomWords, s.gdot + (size_t)t * kGeomWords);
            if (warm) diff::joint_warm_t(k, g, c.dtRatio, v, ix, iy);
            else diff::joint_velocity_t(k, g, v, ix, iy);
            l[0] = ix.d; l[1] = iy.d;
        }
        store_pair(k, A, B, v, basev);
    };
    if (n && c.doWarmStart) {
        for (int col = 0; col <= kSerialColour; ++col) {
            world_pass(base, off, col, false, lane, [&](uint32_t t) {
                const uint32_t id = tp->t_id[t];
                if (id & 0x80000000u) { joint_step(t, id & 0x7fffffffu, tp->warm + 2 * (size_t)t, false, true); return; }
                const PC& pc = tp->pc[t];
                const diff::ContactK k = contact_k(d, pc, tp->cinfo[t]);
                const float4* r = tp->warm + 2 * (size_t)t;
                diff::Pair3<Tan> v = body_pair(pc.bA, pc.bB, r[0], r[1], s.vdot);
                const float4 i0 = tp->imp0[t];
                const double* l = s.ldot + 4 * (size_t)t;
                const diff::Imp<Tan> im{{i0.x, l[0]}, {i0.y, l[1]}, {i0.z, l[2]}, {i0.w, l[3]}};
                diff::warm_start_t(k, geom_tan(gval + (size_t)t * kGeomWords, s.gdot + (size_t)t * kGeomWords), v, im);
                store_pair(k, pc.bA, pc.bB, v, s.vdot);
            });
        }
    }
    if (n) {
        for (int it = 0; it < tp->iv; ++it) {
            for (int col = 0; col <= kSerialColour; ++col) {
                world_pass(base, off, col, false, lane, [&](uint32_t t) {
                    const float4* r = tp->vel + 3 * ((size_t)it * tp->kcap + t);
                    const uint32_t id = tp->t_id[t];
                    if (id & 0x80000000u) { joint_step(t, id & 0x7fffffffu, r, false, false); return; }
                    const PC& pc = tp->pc[t];
                    const diff::ContactK k = contact_k(d, pc, tp->cinfo[t]);
                    diff::Pair3<Tan> v = body_pair(pc.bA, pc.bB, r[0], r[1], s.vdot);
                    double* l = s.ldot + 4 * (size_t)t;
                    diff::Imp<Tan> im{{r[2].x, l[0]}, {r[2].y, l[1]}, {r[2].z, l[2]}, {r[2].w, l[3]}};
                    diff::solve_velocity_t(k, geom_tan(gval + (size_t)t * kGeomWords, s.gdot + (size_t)t * kGeomWords), v,
                                           im);
                    store_pair(k, pc.bA, pc.bB, v, s.vdot);
                    l[0] = im.ni0.d; l[1] = im.ti0.d; l[2] = im.ni1.d; l[3] = im.ti1.d;
                });
            }
        }
    }
    for (uint32_t b = b0 + lane; b < b1; b += 32u) {
        if (!(tp->flags[b] & BF_SOLVED)) continue;
        double* p = s.pdot + 3 * (size_t)b;
        const double* v = s.vdot + 3 * (size_t)b;
        p[0] += (double)h * v[0]; p[1] += (double)h * v[1]; p[2] += (double)h * v[2];
    }
    __syncwarp();
    if (n) {
        for (int it = 0; it < tp->ip; ++it) {
            for (int col = 0; col <= kSerialColour; ++col) {
                world_pass(base, off, col, false, lane, [&](uint32_t t) {
                    const float4* r = tp->pos + 2 * ((size_t)it * tp->kcap + t);
                    if (r[0].w == 0.f) return;
                    const uint32_t id = tp->t_id[t];
                    if (id & 0x80000000u) { joint_step(t, id & 0x7fffffffu, r, true, false); return; }
                    const PC& pc = tp->pc[t];
                    diff::ContactK k = contact_k(d, pc, tp->cinfo[t]);
                    const double* gd = s.gdot + (size_t)t * kGeomWords + kLocalPts;
                    k.dp[0] = gd[0]; k.dp[1] = gd[1]; k.dp[2] = gd[2]; k.dp[3] = gd[3];
                    diff::Pair3<Tan> p = body_pair(pc.bA, pc.bB, r[0], r[1], s.pdot);
                    diff::solve_position_t(k, c, p);
                    store_pair(k, pc.bA, pc.bB, p, s.pdot);
                });
            }
        }
    }
    // stored impulses; slept bodies stop
    for (uint32_t t = base + lane; t < base + n; t += 32u) {
        const uint32_t slot = tp->t_id[t];
        const double* l = s.ldot + 4 * (size_t)t;
        if (slot & 0x80000000u) {
            const uint32_t j = slot & 0x7fffffffu;
            s.jdot[2 * (size_t)j] = l[0];
            s.jdot[2 * (size_t)j + 1] = l[1];
            continue;
        }
        double* m = s.mdot + 4 * (size_t)slot;
        for (int q = 0; q < 4; ++q) m[q] = l[q];
    }
    for (uint32_t b = b0 + lane; b < b1; b += 32u) {
        if (!tp->slept[b]) continue;
        double* v = s.vdot + 3 * (size_t)b;
        v[0] = v[1] = v[2] = 0.0;
    }
}

// ---- launchers ------------------------------------------------------------------------
uint32_t adj_parallel_grid() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) return 0;
    return (uint32_t)sms * 8u;
}

uint32_t adj_sweep_threads(uint32_t most, uint32_t n_worlds) {
    // by the largest world: worlds of up to 256 bodies have a few dozen
    // constraints a colour (one warp, whose barriers are the cheapest)
    const uint32_t t = most > 4096u ? kAdjSweepMaxThreads : most > 256u ? 128u : 32u;
    if (t < kAdjSweepMaxThreads) return t;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) return t;
    // the wide instance while every world's block is resident at once with it (a
    // second wave of blocks would double the pass), else half the block
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_adj_sweeps<true>, (int)t, 0) != cudaSuccess) return t;
    return (uint32_t)b * (uint32_t)sms >= n_worlds ? t : t / 2u;
}

cudaError_t launch_adj_step(const DW& d, const StepTape* tp, const AdjState& a, uint32_t n_slots, cudaStream_t s) {
    k_adj_transfer<<<a.grid, 256, 0, s>>>(d, tp, a, n_slots);
    cudaMemcpyAsync(a.mbar, a.mtmp, sizeof(float4) * n_slots, cudaMemcpyDeviceToDevice, s);
    k_adj_prep<<<a.grid, 256, 0, s>>>(d, tp, a);
    if (a.sweep_threads == kAdjSweepMaxThreads) k_adj_sweeps<true><<<d.n_worlds, a.sweep_threads, 0, s>>>(d, tp, a);
    else k_adj_sweeps<false><<<d.n_worlds, a.sweep_threads, 0, s>>>(d, tp, a);
    k_adj_local<<<a.grid, 256, 0, s>>>(d, tp, a);
    k_adj_bodies<<<a.grid, 256, 0, s>>>(d, tp, a);
    return cudaGetLastError();
}

cudaError_t launch_tan_step(const DW& d, const StepTape* tp, const TanState& t, float* gval, uint32_t n_slots,
                            cudaStream_t s) {
    k_tan_world<<<d.n_worlds, 32, 0, s>>>(d, tp, t, gval);
    k_tan_transfer<<<256, 256, 0, s>>>(d, tp, t, n_slots);
    cudaMemcpyAsync(t.mdot, t.mtmp, sizeof(double) * 4 * n_slots, cudaMemcpyDeviceToDevice, s);
    return cudaGetLastError();
}

}  // namespace prgpu
