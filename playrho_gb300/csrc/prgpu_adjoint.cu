// prgpu_adjoint.cu -- StepAdjoint: reverse-mode gradients of a window of world
// steps, and the FP64 forward-mode tangent of the same window.
//
// A recorded step (d.tape set) runs the ordinary solver kernels, which also
// write what each contact step starts from (prgpu_solver.cu sweep_*), the body
// state at the start of the solve, each world's sweep layout, the impulse
// sources of the post-solve contact update and the slots created
// (prgpu_tape.cuh).  From that record, one warp per world:
//
//  * k_adj_world walks the step backwards -- sleep, impulse store, the position
//    iterations colour by colour in reverse, position integration, the velocity
//    iterations in reverse, warm start, the constraint set-up and the velocity
//    integration -- turning adjoints of the step's outputs into adjoints of its
//    inputs (body positions and velocities, stored contact impulses, shape
//    friction).  The vector-Jacobian products of the iterated pieces, the
//    velocity and position solves, are written out (solve_velocity_vjp,
//    solve_position_vjp); the others, run once per contact and step, come from a
//    per-thread tape of partial derivatives in shared memory (prgpu_diff.cuh).
//  * k_tan_world walks it forwards with FP64 tangents (Tan), the tangent kernel
//    a dot-product test checks the adjoint against.
//
// Worlds are independent, so a warp barrier separates two colours.  Both passes
// take the forward's branches as recorded (contact set, clamps, block cases,
// island early exits, sleep), and the manifold's local geometry as constant
// within a step; joints are not part of the differentiated step.
#include <algorithm>

#include "prgpu_kernels.cuh"
#include "prgpu_tape.cuh"

namespace prgpu {

using diff::AD;
using diff::Tan;
using diff::Tape;

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
__device__ __forceinline__ AD leaf(Tape& tp, float v) { return AD{v, tp.push(-1, 0.f, -1, 0.f), &tp}; }
__device__ __forceinline__ void seed(Tape& tp, const AD& x, float g) {
    if (x.i >= 0 && g != 0.f) tp.grad(x.i) += g;
}
__device__ __forceinline__ float gadj(const Tape& tp, int i) { return tp.grad(i); }

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

__global__ void __launch_bounds__(32) k_adj_world(DW d, const StepTape* tp, AdjState a) {
    extern __shared__ float4 s_tapes[];  // the warp's 32 tapes
    Tape tap;
    tap.init(s_tapes, threadIdx.x);
    const DConf& c = *d.conf;
    const float h = c.deltaTime;
    const uint32_t w = blockIdx.x, lane = threadIdx.x;
    const uint32_t b0 = d.w_body_off[w], b1 = d.w_body_off[w + 1];
    const uint32_t base = tp->wseg[2 * w], n = tp->wseg[2 * w + 1];
    // the world's colour table, and the highest parallel colour in use
    __shared__ uint32_t off[kColStride];
    for (uint32_t q = lane; q < (uint32_t)kColStride; q += 32u) off[q] = tp->wcol[(size_t)w * kColStride + q];
    __syncwarp();
    int top = 0;
    for (int q = 0; q < kMaxColours; ++q)
        if (off[q + 1] > off[q]) top = q + 1;
    // colours in reverse sweep order: the serial one, then top-1 .. 0
    auto prev_col = [&](int col) { return col == kSerialColour ? top - 1 : col - 1; };
    // sleep zeroed these velocities; the stored impulses were the final ones
    for (uint32_t b = b0 + lane; b < b1; b += 32u) {
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
    for (uint32_t t = base + lane; t < base + n; t += 32u) {
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
    __syncwarp();
    if (n) {
        // position iterations, last first, colours in reverse
        for (int it = tp->ip - 1; it >= 0; --it) {
            for (int col = kSerialColour; col >= 0; col = prev_col(col)) {
                world_pass(base, off, col, true, lane, [&](uint32_t t) {
                    if (tp->t_id[t] & 0x80000000u) return;
                    const float4* r = tp->pos + 2 * ((size_t)it * tp->kcap + t);
                    if (r[0].w == 0.f) return;  // island already within tolerance
                    const PC& pc = tp->pc[t];
                    const diff::ContactK k = contact_k(d, pc, tp->cinfo[t]);
                    const float p[6] = {r[0].x, r[0].y, r[0].z, r[1].x, r[1].y, r[1].z};
                    float yb[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, pb[6];
                    if (k.writableA) { const float4 g = a.pbar[pc.bA]; yb[0] = g.x; yb[1] = g.y; yb[2] = g.z; }
                    if (k.writableB) { const float4 g = a.pbar[pc.bB]; yb[3] = g.x; yb[4] = g.y; yb[5] = g.z; }
                    diff::solve_position_vjp(k, c, p, yb, pb);
                    // bodies that are not dynamic are not differentiated (and can be
                    // shared within a colour)
                    if (k.writableA) a.pbar[pc.bA] = make_float4(pb[0], pb[1], pb[2], 0.f);
                    if (k.writableB) a.pbar[pc.bB] = make_float4(pb[3], pb[4], pb[5], 0.f);
                });
            }
        }
    }
    // position integration p1 = p0 + h v
    for (uint32_t b = b0 + lane; b < b1; b += 32u) {
        if (!(tp->flags[b] & BF_SOLVED)) continue;
        const float4 pb = a.pbar[b];
        float4 vb = a.vbar[b];
        vb.x += h * pb.x; vb.y += h * pb.y; vb.z += h * pb.z;
        a.vbar[b] = vb;
    }
    __syncwarp();
    if (n) {
        // velocity iterations, last first, colours in reverse
        for (int it = tp->iv - 1; it >= 0; --it) {
            for (int col = kSerialColour; col >= 0; col = prev_col(col)) {
                world_pass(base, off, col, true, lane, [&](uint32_t t) {
                    if (tp->t_id[t] & 0x80000000u) return;
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
        // warm start
        for (int col = kSerialColour; col >= 0; col = prev_col(col)) {
            world_pass(base, off, col, true, lane, [&](uint32_t t) {
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
        for (uint32_t t = base + lane; t < base + n; t += 32u) {
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
        __syncwarp();
    }
    // velocity at the start of the solve from the velocity the step started with
    for (uint32_t b = b0 + lane; b < b1; b += 32u) {
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
        pack_geom(g, gval + (size_t)t * kGeomWords);
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
    auto store_pair = [&](const diff::ContactK& k, uint32_t A, uint32_t B, const diff::Pair3<Tan>& v, double* basev) {
        if (k.writableA) { double* a3 = basev + 3 * (size_t)A; a3[0] = v.ax.d; a3[1] = v.ay.d; a3[2] = v.az.d; }
        if (k.writableB) { double* b3 = basev + 3 * (size_t)B; b3[0] = v.bx.d; b3[1] = v.by.d; b3[2] = v.bz.d; }
    };
    if (n && c.doWarmStart) {
        for (int col = 0; col <= kSerialColour; ++col) {
            world_pass(base, off, col, false, lane, [&](uint32_t t) {
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
    if (n) {
        for (int it = 0; it < tp->iv; ++it) {
            for (int col = 0; col <= kSerialColour; ++col) {
                world_pass(base, off, col, false, lane, [&](uint32_t t) {
                    if (tp->t_id[t] & 0x80000000u) return;
                    const PC& pc = tp->pc[t];
                    const diff::ContactK k = contact_k(d, pc, tp->cinfo[t]);
                    const float4* r = tp->vel + 3 * ((size_t)it * tp->kcap + t);
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
    }
    // stored impulses; slept bodies stop
    for (uint32_t t = base + lane; t < base + n; t += 32u) {
        const uint32_t slot = tp->t_id[t];
        if (slot & 0x80000000u) continue;
        const double* l = s.ldot + 4 * (size_t)t;
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
int adj_setup() {
    const int bytes = 32 * diff::kTapeBytes;
    if (cudaFuncSetAttribute(k_adj_world, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess) return 0;
    int a = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_adj_world, 32, bytes);
    return a;
}

cudaError_t launch_adj_step(const DW& d, const StepTape* tp, const AdjState& a, uint32_t n_slots, cudaStream_t s) {
    k_adj_transfer<<<256, 256, 0, s>>>(d, tp, a, n_slots);
    cudaMemcpyAsync(a.mbar, a.mtmp, sizeof(float4) * n_slots, cudaMemcpyDeviceToDevice, s);
    k_adj_world<<<d.n_worlds, 32, 32 * diff::kTapeBytes, s>>>(d, tp, a);
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
