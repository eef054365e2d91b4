// prgpu_adjoint.cu -- StepAdjoint: reverse-mode gradients of a window of world
// steps, and the FP64 forward-mode tangent of the same window.
//
// A recorded step (d.tape set) runs the ordinary grid-wide kernels, which also
// write what each contact step starts from (prgpu_solver.cu sweep_*), the
// body state at the start of the solve, the impulse sources of the post-solve
// contact update and the slots created.  From that record:
//
//  * k_adj_step walks the step backwards -- sleep, impulse store, the position
//    iterations colour by colour in reverse, position integration, the velocity
//    iterations in reverse, warm start, the constraint set-up and the velocity
//    integration -- turning adjoints of the step's outputs into adjoints of its
//    inputs (body positions and velocities, stored contact impulses, shape
//    friction).  Each contact step's vector-Jacobian product comes from a
//    per-thread tape of its local partial derivatives (prgpu_diff.cuh).
//  * k_tan_step walks it forwards with FP64 tangents (Tan), the tangent kernel
//    a dot-product test checks the adjoint against.
//
// Both take the forward's branches as recorded (contact set, clamps, block
// cases, island early exits, sleep), and the manifold's local geometry as
// constant within a step; joints are not part of the differentiated step.
#include <cooperative_groups.h>

#include <algorithm>

#include "prgpu_diff.cuh"
#include "prgpu_kernels.cuh"

namespace prgpu {

using diff::AD;
using diff::Tan;
using diff::Tape;

constexpr int kGeomWords = 24;  // n rA0 rB0 rA1 rB1 nm0 tm0 nm1 tm1 vb0 vb1 k00 k11 k01 m00 m11 m01 mu cnt

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

__device__ diff::ContactK contact_k(const DW& d, const PC& pc, float4 ci) {
    diff::ContactK k;
    k.mA = d.b_mass[pc.bA];
    k.mB = d.b_mass[pc.bB];
    k.rA = ci.x; k.rB = ci.y; k.restitution = ci.w;
    k.type = pc.type; k.count = pc.count;
    k.lnx = pc.lnx; k.lny = pc.lny; k.lpx = pc.lpx; k.lpy = pc.lpy;
    k.p0x = pc.p0x; k.p0y = pc.p0y; k.p1x = pc.p1x; k.p1y = pc.p1y;
    k.writableA = is_accelerable(d.b_flags[pc.bA]) ? 1u : 0u;
    k.writableB = is_accelerable(d.b_flags[pc.bB]) ? 1u : 0u;
    return k;
}

// velocity of body b at the start of the solve (after k_body_begin)
template <class T>
__device__ void start_velocity(const DW& d, uint32_t b, T& vx, T& vy, T& vw) {
    diff::integrate_velocity_t(is_accelerable(d.b_flags[b]), d.b_acc[b], d.b_damp[b], *d.conf, vx, vy, vw);
}

template <class T>
__device__ void pack_geom(const diff::Geom<T>& g, float* out) {
    out[0] = diff::val(g.n.x); out[1] = diff::val(g.n.y);
    for (int j = 0; j < 2; ++j) {
        out[2 + 4 * j] = diff::val(g.rA[j].x); out[3 + 4 * j] = diff::val(g.rA[j].y);
        out[4 + 4 * j] = diff::val(g.rB[j].x); out[5 + 4 * j] = diff::val(g.rB[j].y);
    }
    out[10] = diff::val(g.nm[0]); out[11] = diff::val(g.tm[0]); out[12] = diff::val(g.nm[1]); out[13] = diff::val(g.tm[1]);
    out[14] = diff::val(g.vb[0]); out[15] = diff::val(g.vb[1]);
    out[16] = diff::val(g.k00); out[17] = diff::val(g.k11); out[18] = diff::val(g.k01);
    out[19] = diff::val(g.m00); out[20] = diff::val(g.m11); out[21] = diff::val(g.m01);
    out[22] = diff::val(g.mu); out[23] = __int_as_float(g.cnt);
}

// The geometry recomputed from the recorded state, in float: equal bit for bit
// to what k_build_constraints stored (the count of differences goes to hdr).
__device__ diff::Geom<float> replay_geom(const DW& d, const StepTape* tp, uint32_t t, const diff::ContactK& k,
                                         float mu) {
    const PC& pc = tp->pc[t];
    const float4 pa = tp->p0[pc.bA], pb = tp->p0[pc.bB];
    float vax = tp->v0[pc.bA].x, vay = tp->v0[pc.bA].y, vaw = tp->v0[pc.bA].z;
    float vbx = tp->v0[pc.bB].x, vby = tp->v0[pc.bB].y, vbw = tp->v0[pc.bB].z;
    if (tp->flags[pc.bA] & BF_SOLVED) start_velocity(d, pc.bA, vax, vay, vaw);
    if (tp->flags[pc.bB] & BF_SOLVED) start_velocity(d, pc.bB, vbx, vby, vbw);
    const diff::Pair3<float> p{pa.x, pa.y, pa.z, pb.x, pb.y, pb.z};
    const diff::Pair3<float> v{vax, vay, vaw, vbx, vby, vbw};
    return diff::build_geom(k, p, v, mu, *d.conf);
}

__global__ void k_tape_constraints(DW d) {
    StepTape* tp = d.tape;
    const uint32_t n = d.cnt->n_active;
    uint32_t bad = 0;
    GRID_LOOP(t, n) {
        const uint32_t id = d.t_id[t];
        tp->t_id[t] = id;
        if (id & 0x80000000u) continue;
        const PC pc = d.pc[t];
        tp->pc[t] = pc;
        const uint2 pr = d.cs_proxy[id];
        const float2 mat = d.cs_mat[id];
        const float4 ci = make_float4(d.s_radius[pr.x], d.s_radius[pr.y], mat.x, mat.y);
        tp->cinfo[t] = ci;
        tp->prox[t] = pr;
        const float4 e = d.vc0[t].q[3];
        const uint32_t count = __float_as_uint(d.vc0[t].q[2].w);
        const float4 i1 = (count == 2u) ? d.vc1[t].q[3] : make_float4(0.f, 0.f, 0.f, 0.f);
        tp->imp0[t] = make_float4(e.x, e.y, i1.x, i1.y);
        // replay check of the differentiable restatement
        const diff::Geom<float> g = replay_geom(d, tp, t, contact_k(d, pc, ci), mat.x);
        const float4 a = d.vc0[t].q[0], b = d.vc0[t].q[1], c2 = d.vc0[t].q[2];
        bool same = (unsigned)g.cnt == count && g.n.x == a.x && g.n.y == a.y && g.rA[0].x == b.x && g.rA[0].y == b.y &&
                    g.rB[0].x == b.z && g.rB[0].y == b.w && g.nm[0] == c2.x && g.tm[0] == c2.y && g.vb[0] == c2.z;
        if (count == 2u) {
            const float4 f = d.vc1[t].q[0], gg = d.vc1[t].q[1], h = d.vc1[t].q[2], i = d.vc1[t].q[3];
            same = same && g.rA[1].x == f.x && g.rA[1].y == f.y && g.rB[1].x == f.z && g.rB[1].y == f.w &&
                   g.nm[1] == gg.x && g.tm[1] == gg.y && g.vb[1] == gg.z && g.k00 == gg.w && g.k11 == h.x &&
                   g.k01 == h.y && g.m00 == h.z && g.m11 == h.w && g.m01 == i.z;
        }
        if (!same) ++bad;
    }
    if (bad) atomicAdd(&tp->hdr[kSerialColour + 2 + 3], bad);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int k = 0; k <= kSerialColour + 1; ++k) tp->hdr[k] = d.cnt->colour_off[k];
        tp->hdr[kSerialColour + 2] = d.cnt->n_colours;
        tp->hdr[kSerialColour + 3] = n;
    }
}

void launch_tape_body_start(const DW& d, const Launch& L, cudaStream_t s) { k_tape_body_start<<<L.grid, L.threads, 0, s>>>(d); }
void launch_tape_body_flags(const DW& d, const Launch& L, cudaStream_t s) { k_tape_body_flags<<<L.grid, L.threads, 0, s>>>(d); }
void launch_tape_constraints(const DW& d, const Launch& L, cudaStream_t s) {
    k_tape_constraints<<<L.grid, L.threads, 0, s>>>(d);
}

// ---- adjoint ----------------------------------------------------------------------

__device__ __forceinline__ AD leaf(Tape& tp, float v) { return AD{v, tp.push(-1, 0.0, -1, 0.0), &tp}; }
__device__ __forceinline__ void seed(Tape& tp, const AD& x, float g) {
    if (x.i >= 0 && g != 0.f) tp.adj[x.i] += (double)g;
}
__device__ __forceinline__ float gadj(const Tape& tp, int i) { return (float)tp.adj[i]; }

__device__ diff::Geom<AD> geom_leaves(Tape& tp, const float* gv) {
    diff::Geom<AD> g;
    g.n = {leaf(tp, gv[0]), leaf(tp, gv[1])};
    for (int j = 0; j < 2; ++j) {
        g.rA[j] = {leaf(tp, gv[2 + 4 * j]), leaf(tp, gv[3 + 4 * j])};
        g.rB[j] = {leaf(tp, gv[4 + 4 * j]), leaf(tp, gv[5 + 4 * j])};
    }
    g.nm[0] = leaf(tp, gv[10]); g.tm[0] = leaf(tp, gv[11]); g.nm[1] = leaf(tp, gv[12]); g.tm[1] = leaf(tp, gv[13]);
    g.vb[0] = leaf(tp, gv[14]); g.vb[1] = leaf(tp, gv[15]);
    g.k00 = leaf(tp, gv[16]); g.k11 = leaf(tp, gv[17]); g.k01 = leaf(tp, gv[18]);
    g.m00 = leaf(tp, gv[19]); g.m11 = leaf(tp, gv[20]); g.m01 = leaf(tp, gv[21]);
    g.mu = leaf(tp, gv[22]);
    g.cnt = __float_as_int(gv[23]);
    return g;
}

// Colour-ordered loop over one colour of the recorded step, forwards or backwards;
// the serial colour (the leftovers) runs on one thread in sweep order.
template <class F>
__device__ void colour_pass(const DW& d, const uint32_t* hdr, uint32_t col, bool reverse, F&& f) {
    const uint32_t ncol = hdr[kSerialColour + 2];
    const bool serial = (col == ncol);
    const uint32_t lo = serial ? hdr[kSerialColour] : hdr[col];
    const uint32_t hi = serial ? hdr[kSerialColour + 1] : hdr[col + 1];
    if (lo == hi) return;
    if (serial) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            if (reverse) for (uint32_t t = hi; t-- > lo;) f(t);
            else for (uint32_t t = lo; t < hi; ++t) f(t);
        }
    } else {
        GRID_LOOP(i, hi - lo) f(lo + i);
    }
    grid_barrier(d.cnt);
}

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

__global__ void __launch_bounds__(128) k_adj_step(DW d, const StepTape* tp, AdjState a) {
    const DConf& c = *d.conf;
    const uint32_t* hdr = tp->hdr;
    const uint32_t ncol = hdr[kSerialColour + 2];
    const uint32_t n = hdr[kSerialColour + 3];
    const float h = c.deltaTime;
    Tape tap;  // one per thread, reused by every local derivative below
    // sleep zeroed these velocities; the stored impulses were the final ones
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
    GRID_LOOP(t, n) {
        const uint32_t slot = tp->t_id[t];
        float* gb = a.gbar + (size_t)t * kGeomWords;
        for (int q = 0; q < kGeomWords; ++q) gb[q] = 0.f;
        if (slot & 0x80000000u) continue;
        a.lbar[t] = a.mbar[slot];
        a.mbar[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
        const PC& pc = tp->pc[t];
        const diff::Geom<float> g = replay_geom(d, tp, t, contact_k(d, pc, tp->cinfo[t]), tp->cinfo[t].z);
        pack_geom(g, a.gval + (size_t)t * kGeomWords);
    }
    grid_barrier(d.cnt);
    // position iterations, last first, colours in reverse
    for (int it = tp->ip - 1; it >= 0; --it) {
        for (int col = (int)ncol; col >= 0; --col) {
            colour_pass(d, hdr, (uint32_t)col, true, [&](uint32_t t) {
                if (tp->t_id[t] & 0x80000000u) return;
                const float4* r = tp->pos + 2 * ((size_t)it * tp->kcap + t);
                if (r[0].w == 0.f) return;  // island already within tolerance
                const PC& pc = tp->pc[t];
                const diff::ContactK k = contact_k(d, pc, tp->cinfo[t]);
                tap.reset();
                diff::Pair3<AD> p{leaf(tap, r[0].x), leaf(tap, r[0].y), leaf(tap, r[0].z),
                                  leaf(tap, r[1].x), leaf(tap, r[1].y), leaf(tap, r[1].z)};
                diff::solve_position_t(k, c, p);
                const float4 ga = a.pbar[pc.bA], gb = a.pbar[pc.bB];
                if (k.writableA) { seed(tap, p.ax, ga.x); seed(tap, p.ay, ga.y); seed(tap, p.az, ga.z); }
                if (k.writableB) { seed(tap, p.bx, gb.x); seed(tap, p.by, gb.y); seed(tap, p.bz, gb.z); }
                tap.backward();
                if (tap.overflow) atomicAdd(a.err, 1u);
                // bodies that are not dynamic can be shared within a colour: their
                // adjoints are not carried (their states are not differentiated)
                if (k.writableA) a.pbar[pc.bA] = make_float4(gadj(tap, 0), gadj(tap, 1), gadj(tap, 2), 0.f);
                if (k.writableB) a.pbar[pc.bB] = make_float4(gadj(tap, 3), gadj(tap, 4), gadj(tap, 5), 0.f);
            });
        }
    }
    // position integration p1 = p0 + h v
    GRID_LOOP(b, d.n_bodies) {
        if (!(tp->flags[b] & BF_SOLVED)) continue;
        const float4 pb = a.pbar[b];
        float4 vb = a.vbar[b];
        vb.x += h * pb.x; vb.y += h * pb.y; vb.z += h * pb.z;
        a.vbar[b] = vb;
    }
    grid_barrier(d.cnt);
    // velocity iterations, last first, colours in reverse
    for (int it = tp->iv - 1; it >= 0; --it) {
        for (int col = (int)ncol; col >= 0; --col) {
            colour_pass(d, hdr, (uint32_t)col, true, [&](uint32_t t) {
                if (tp->t_id[t] & 0x80000000u) return;
                const float4* r = tp->vel + 3 * ((size_t)it * tp->kcap + t);
                const PC& pc = tp->pc[t];
                const diff::ContactK k = contact_k(d, pc, tp->cinfo[t]);
                tap.reset();
                diff::Pair3<AD> v{leaf(tap, r[0].x), leaf(tap, r[0].y), leaf(tap, r[0].z),
                                  leaf(tap, r[1].x), leaf(tap, r[1].y), leaf(tap, r[1].z)};
                diff::Imp<AD> im{leaf(tap, r[2].x), leaf(tap, r[2].y), leaf(tap, r[2].z), leaf(tap, r[2].w)};
                const diff::Geom<AD> g = geom_leaves(tap, a.gval + (size_t)t * kGeomWords);
                diff::solve_velocity_t(k, g, v, im);
                const float4 ga = a.vbar[pc.bA], gb = a.vbar[pc.bB], gl = a.lbar[t];
                if (k.writableA) { seed(tap, v.ax, ga.x); seed(tap, v.ay, ga.y); seed(tap, v.az, ga.z); }
                if (k.writableB) { seed(tap, v.bx, gb.x); seed(tap, v.by, gb.y); seed(tap, v.bz, gb.z); }
                seed(tap, im.ni0, gl.x); seed(tap, im.ti0, gl.y); seed(tap, im.ni1, gl.z); seed(tap, im.ti1, gl.w);
                tap.backward();
                if (tap.overflow) atomicAdd(a.err, 1u);
                if (k.writableA) a.vbar[pc.bA] = make_float4(gadj(tap, 0), gadj(tap, 1), gadj(tap, 2), 0.f);
                if (k.writableB) a.vbar[pc.bB] = make_float4(gadj(tap, 3), gadj(tap, 4), gadj(tap, 5), 0.f);
                a.lbar[t] = make_float4(gadj(tap, 6), gadj(tap, 7), gadj(tap, 8), gadj(tap, 9));
                float* gbar = a.gbar + (size_t)t * kGeomWords;
                for (int q = 0; q < kGeomWords - 1; ++q) gbar[q] += gadj(tap, 10 + q);
            });
        }
    }
    // warm start
    for (int col = (int)ncol; col >= 0; --col) {
        colour_pass(d, hdr, (uint32_t)col, true, [&](uint32_t t) {
            const uint32_t slot = tp->t_id[t];
            if (slot & 0x80000000u) return;
            const PC& pc = tp->pc[t];
            float4 li = a.lbar[t];  // adjoint of the impulses the first iteration started from
            if (c.doWarmStart) {
                const float4* r = tp->warm + 2 * (size_t)t;
                const diff::ContactK k = contact_k(d, pc, tp->cinfo[t]);
                const float4 i0 = tp->imp0[t];
                tap.reset();
                diff::Pair3<AD> v{leaf(tap, r[0].x), leaf(tap, r[0].y), leaf(tap, r[0].z),
                                  leaf(tap, r[1].x), leaf(tap, r[1].y), leaf(tap, r[1].z)};
                const diff::Imp<AD> im{leaf(tap, i0.x), leaf(tap, i0.y), leaf(tap, i0.z), leaf(tap, i0.w)};
                const diff::Geom<AD> g = geom_leaves(tap, a.gval + (size_t)t * kGeomWords);
                diff::warm_start_t(k, g, v, im);
                const float4 ga = a.vbar[pc.bA], gb = a.vbar[pc.bB];
                if (k.writableA) { seed(tap, v.ax, ga.x); seed(tap, v.ay, ga.y); seed(tap, v.az, ga.z); }
                if (k.writableB) { seed(tap, v.bx, gb.x); seed(tap, v.by, gb.y); seed(tap, v.bz, gb.z); }
                tap.backward();
                if (tap.overflow) atomicAdd(a.err, 1u);
                if (k.writableA) a.vbar[pc.bA] = make_float4(gadj(tap, 0), gadj(tap, 1), gadj(tap, 2), 0.f);
                if (k.writableB) a.vbar[pc.bB] = make_float4(gadj(tap, 3), gadj(tap, 4), gadj(tap, 5), 0.f);
                li.x += gadj(tap, 6); li.y += gadj(tap, 7); li.z += gadj(tap, 8); li.w += gadj(tap, 9);
                float* gbar = a.gbar + (size_t)t * kGeomWords;
                for (int q = 0; q < kGeomWords - 1; ++q) gbar[q] += gadj(tap, 10 + q);
            }
            // VelocityConstraint's impulses are the stored ones times dtRatio
            float4 m = a.mbar[slot];
            m.x += li.x * c.dtRatio; m.y += li.y * c.dtRatio; m.z += li.z * c.dtRatio; m.w += li.w * c.dtRatio;
            a.mbar[slot] = m;
        });
    }
    // constraint set-up: geometry from the positions and velocities at the
    // start of the solve and the contact's friction
    GRID_LOOP(t, n) {
        const uint32_t slot = tp->t_id[t];
        if (slot & 0x80000000u) continue;
        const PC& pc = tp->pc[t];
        const float4 ci = tp->cinfo[t];
        const diff::ContactK k = contact_k(d, pc, ci);
        const float4 pa = tp->p0[pc.bA], pb = tp->p0[pc.bB], va = a.vi[pc.bA], vb = a.vi[pc.bB];
        tap.reset();
        const diff::Pair3<AD> p{leaf(tap, pa.x), leaf(tap, pa.y), leaf(tap, pa.z), leaf(tap, pb.x), leaf(tap, pb.y),
                                leaf(tap, pb.z)};
        const diff::Pair3<AD> v{leaf(tap, va.x), leaf(tap, va.y), leaf(tap, va.z), leaf(tap, vb.x), leaf(tap, vb.y),
                                leaf(tap, vb.z)};
        const AD mu = leaf(tap, ci.z);
        const diff::Geom<AD> g = diff::build_geom(k, p, v, mu, c);
        const float* gb = a.gbar + (size_t)t * kGeomWords;
        seed(tap, g.n.x, gb[0]); seed(tap, g.n.y, gb[1]);
        for (int j = 0; j < 2; ++j) {
            seed(tap, g.rA[j].x, gb[2 + 4 * j]); seed(tap, g.rA[j].y, gb[3 + 4 * j]);
            seed(tap, g.rB[j].x, gb[4 + 4 * j]); seed(tap, g.rB[j].y, gb[5 + 4 * j]);
        }
        seed(tap, g.nm[0], gb[10]); seed(tap, g.tm[0], gb[11]); seed(tap, g.nm[1], gb[12]); seed(tap, g.tm[1], gb[13]);
        seed(tap, g.vb[0], gb[14]); seed(tap, g.vb[1], gb[15]);
        seed(tap, g.k00, gb[16]); seed(tap, g.k11, gb[17]); seed(tap, g.k01, gb[18]);
        seed(tap, g.m00, gb[19]); seed(tap, g.m11, gb[20]); seed(tap, g.m01, gb[21]);
        seed(tap, g.mu, gb[22]);
        tap.backward();
        if (tap.overflow) atomicAdd(a.err, 1u);
        atomicAdd(&a.pbar[pc.bA].x, gadj(tap, 0)); atomicAdd(&a.pbar[pc.bA].y, gadj(tap, 1));
        atomicAdd(&a.pbar[pc.bA].z, gadj(tap, 2));
        atomicAdd(&a.pbar[pc.bB].x, gadj(tap, 3)); atomicAdd(&a.pbar[pc.bB].y, gadj(tap, 4));
        atomicAdd(&a.pbar[pc.bB].z, gadj(tap, 5));
        atomicAdd(&a.vibar[pc.bA].x, gadj(tap, 6)); atomicAdd(&a.vibar[pc.bA].y, gadj(tap, 7));
        atomicAdd(&a.vibar[pc.bA].z, gadj(tap, 8));
        atomicAdd(&a.vibar[pc.bB].x, gadj(tap, 9)); atomicAdd(&a.vibar[pc.bB].y, gadj(tap, 10));
        atomicAdd(&a.vibar[pc.bB].z, gadj(tap, 11));
        // MixFriction: sqrt(fA fB)
        const float mub = gadj(tap, 12);
        if (mub != 0.f && ci.z > 0.f) {
            const uint2 pr = tp->prox[t];
            const float fa = d.s_mat[pr.x].x, fb = d.s_mat[pr.y].x;
            atomicAdd(&a.fbar[pr.x], mub * fb / (2.0f * ci.z));
            atomicAdd(&a.fbar[pr.y], mub * fa / (2.0f * ci.z));
        }
    }
    grid_barrier(d.cnt);
    // velocity at the start of the solve from the velocity the step started with
    GRID_LOOP(b, d.n_bodies) {
        if (!(tp->flags[b] & BF_SOLVED)) continue;
        const float4 v0 = tp->v0[b];
        const float4 g1 = a.vbar[b], g2 = a.vibar[b];
        tap.reset();
        AD vx = leaf(tap, v0.x), vy = leaf(tap, v0.y), vw = leaf(tap, v0.z);
        start_velocity(d, b, vx, vy, vw);
        seed(tap, vx, g1.x + g2.x); seed(tap, vy, g1.y + g2.y); seed(tap, vw, g1.z + g2.z);
        tap.backward();
        a.vbar[b] = make_float4(gadj(tap, 0), gadj(tap, 1), gadj(tap, 2), 0.f);
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

__global__ void __launch_bounds__(128) k_tan_step(DW d, const StepTape* tp, TanState s, float* gval) {
    const DConf& c = *d.conf;
    const uint32_t* hdr = tp->hdr;
    const uint32_t ncol = hdr[kSerialColour + 2];
    const uint32_t n = hdr[kSerialColour + 3];
    const float h = c.deltaTime;
    GRID_LOOP(b, d.n_bodies) {
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
    grid_barrier(d.cnt);
    // constraint geometry and its tangent; the iterations start from the stored impulses
    GRID_LOOP(t, n) {
        const uint32_t slot = tp->t_id[t];
        if (slot & 0x80000000u) continue;
        const PC& pc = tp->pc[t];
        const float4 ci = tp->cinfo[t];
        const diff::ContactK k = contact_k(d, pc, ci);
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
        const diff::Pair3<Tan> p{{pa.x, dpa[0]}, {pa.y, dpa[1]}, {pa.z, dpa[2]}, {pb.x, dpb[0]}, {pb.y, dpb[1]}, {pb.z, dpb[2]}};
        const diff::Pair3<Tan> v{{vax, dva[0]}, {vay, dva[1]}, {vaw, dva[2]}, {vbx, dvb[0]}, {vby, dvb[1]}, {vbw, dvb[2]}};
        const diff::Geom<Tan> g = diff::build_geom(k, p, v, Tan{ci.z, mud}, c);
        float* gv = gval + (size_t)t * kGeomWords;
        pack_geom(g, gv);
        double* gd = s.gdot + (size_t)t * kGeomWords;
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
    GRID_LOOP(b, d.n_bodies) {
        double* v = s.vdot + 3 * (size_t)b;
        const double* vi = s.vidot + 3 * (size_t)b;
        v[0] = vi[0]; v[1] = vi[1]; v[2] = vi[2];
    }
    grid_barrier(d.cnt);
    auto body_pair = [&](uint32_t A, uint32_t B, float4 ra, float4 rb, const double* base) {
        const double* a3 = base + 3 * (size_t)A;
        const double* b3 = base + 3 * (size_t)B;
        return diff::Pair3<Tan>{{ra.x, a3[0]}, {ra.y, a3[1]}, {ra.z, a3[2]}, {rb.x, b3[0]}, {rb.y, b3[1]}, {rb.z, b3[2]}};
    };
    auto store_pair = [&](const diff::ContactK& k, uint32_t A, uint32_t B, const diff::Pair3<Tan>& v, double* base) {
        if (k.writableA) { double* a3 = base + 3 * (size_t)A; a3[0] = v.ax.d; a3[1] = v.ay.d; a3[2] = v.az.d; }
        if (k.writableB) { double* b3 = base + 3 * (size_t)B; b3[0] = v.bx.d; b3[1] = v.by.d; b3[2] = v.bz.d; }
    };
    if (c.doWarmStart) {
        for (uint32_t col = 0; col <= ncol; ++col) {
            colour_pass(d, hdr, col, false, [&](uint32_t t) {
                if (tp->t_id[t] & 0x80000000u) return;
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
    for (int it = 0; it < tp->iv; ++it) {
        for (uint32_t col = 0; col <= ncol; ++col) {
            colour_pass(d, hdr, col, false, [&](uint32_t t) {
                if (tp->t_id[t] & 0x80000000u) return;
                const PC& pc = tp->pc[t];
                const diff::ContactK k = contact_k(d, pc, tp->cinfo[t]);
                const float4* r = tp->vel + 3 * ((size_t)it * tp->kcap + t);
                diff::Pair3<Tan> v = body_pair(pc.bA, pc.bB, r[0], r[1], s.vdot);
                double* l = s.ldot + 4 * (size_t)t;
                diff::Imp<Tan> im{{r[2].x, l[0]}, {r[2].y, l[1]}, {r[2].z, l[2]}, {r[2].w, l[3]}};
                diff::solve_velocity_t(k, geom_tan(gval + (size_t)t * kGeomWords, s.gdot + (size_t)t * kGeomWords), v, im);
                store_pair(k, pc.bA, pc.bB, v, s.vdot);
                l[0] = im.ni0.d; l[1] = im.ti0.d; l[2] = im.ni1.d; l[3] = im.ti1.d;
            });
        }
    }
    GRID_LOOP(b, d.n_bodies) {
        if (!(tp->flags[b] & BF_SOLVED)) continue;
        double* p = s.pdot + 3 * (size_t)b;
        const double* v = s.vdot + 3 * (size_t)b;
        p[0] += (double)h * v[0]; p[1] += (double)h * v[1]; p[2] += (double)h * v[2];
    }
    grid_barrier(d.cnt);
    for (int it = 0; it < tp->ip; ++it) {
        for (uint32_t col = 0; col <= ncol; ++col) {
            colour_pass(d, hdr, col, false, [&](uint32_t t) {
                if (tp->t_id[t] & 0x80000000u) return;
                const float4* r = tp->pos + 2 * ((size_t)it * tp->kcap + t);
                if (r[0].w == 0.f) return;
                const PC& pc = tp->pc[t];
                const diff::ContactK k = contact_k(d, pc, tp->cinfo[t]);
                diff::Pair3<Tan> p = body_pair(pc.bA, pc.bB, r[0], r[1], s.pdot);
                diff::solve_position_t(k, c, p);
                store_pair(k, pc.bA, pc.bB, p, s.pdot);
            });
        }
    }
    // stored impulses; slept bodies stop
    GRID_LOOP(t, n) {
        const uint32_t slot = tp->t_id[t];
        if (slot & 0x80000000u) continue;
        const double* l = s.ldot + 4 * (size_t)t;
        double* m = s.mdot + 4 * (size_t)slot;
        for (int q = 0; q < 4; ++q) m[q] = l[q];
    }
    GRID_LOOP(b, d.n_bodies) {
        if (!tp->slept[b]) continue;
        double* v = s.vdot + 3 * (size_t)b;
        v[0] = v[1] = v[2] = 0.0;
    }
}

// ---- launchers ------------------------------------------------------------------------
namespace {
template <class K, class... Args>
cudaError_t launch_coop_small(K kernel, int grid, int threads, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}
}  // namespace

int adj_grid(int sm_count) {
    int a = 0, b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_adj_step, 128, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_tan_step, 128, 0);
    const int per = std::min(std::min(a, b), 2);
    return per < 1 ? 0 : per * sm_count;
}

cudaError_t launch_adj_step(const DW& d, const StepTape* tp, const AdjState& a, uint32_t n_slots, int grid,
                            cudaStream_t s) {
    k_adj_transfer<<<256, 256, 0, s>>>(d, tp, a, n_slots);
    cudaMemcpyAsync(a.mbar, a.mtmp, sizeof(float4) * n_slots, cudaMemcpyDeviceToDevice, s);
    return launch_coop_small(k_adj_step, grid, 128, s, d, tp, a);
}

cudaError_t launch_tan_step(const DW& d, const StepTape* tp, const TanState& t, float* gval, uint32_t n_slots,
                            int grid, cudaStream_t s) {
    cudaError_t e = launch_coop_small(k_tan_step, grid, 128, s, d, tp, t, gval);
    if (e != cudaSuccess) return e;
    k_tan_transfer<<<256, 256, 0, s>>>(d, tp, t, n_slots);
    return cudaMemcpyAsync(t.mdot, t.mtmp, sizeof(double) * 4 * n_slots, cudaMemcpyDeviceToDevice, s);
}

}  // namespace prgpu
