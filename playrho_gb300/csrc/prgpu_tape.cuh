// prgpu_tape.cuh -- recording a world step for the adjoint: what one contact
// of a recorded step keeps, shared by the grid-wide and the per-world solvers
// (which call tape_constraint right after building the constraint at t).
#pragma once

#include "prgpu_diff.cuh"
#include "prgpu_kernels.cuh"

namespace prgpu {

// n rA0 rB0 rA1 rB1 nm0 tm0 nm1 tm1 vb0 vb1 k00 k11 k01 m00 m11 m01 mu cnt, then
// the manifold's local points p0 p1 (words kLocalPts..+3: their adjoints in gbar,
// their tangents in gdot)
constexpr int kGeomWords = kAdjGeomWords;
constexpr int kLocalPts = 24;
constexpr int kTapeHdrMismatch = kSerialColour + 5;  // hdr word counting replay mismatches

__device__ __forceinline__ diff::ContactK contact_k(const DW& d, const PC& pc, float4 ci) {
    diff::ContactK k;
    k.mA = d.b_mass[pc.bA];
    k.mB = d.b_mass[pc.bB];
    k.rA = ci.x; k.rB = ci.y; k.restitution = ci.w;
    k.type = pc.type; k.count = pc.count;
    k.lnx = pc.lnx; k.lny = pc.lny; k.lpx = pc.lpx; k.lpy = pc.lpy;
    k.p0x = pc.p0x; k.p0y = pc.p0y; k.p1x = pc.p1x; k.p1y = pc.p1y;
    k.writableA = is_accelerable(d.b_flags[pc.bA]) ? 1u : 0u;
    k.writableB = is_accelerable(d.b_flags[pc.bB]) ? 1u : 0u;
    k.dp[0] = k.dp[1] = k.dp[2] = k.dp[3] = 0.0;
    return k;
}

// velocity of body b at the start of the solve (after k_body_begin)
template <class T>
__device__ __forceinline__ void start_velocity(const DW& d, uint32_t b, T& vx, T& vy, T& vw) {
    diff::integrate_velocity_t(is_accelerable(d.b_flags[b]), d.b_acc[b], d.b_damp[b], *d.conf, vx, vy, vw);
}

template <class T>
__device__ __forceinline__ void pack_geom(const diff::Geom<T>& g, float* out) {
    using diff::val;
    out[0] = val(g.n.x); out[1] = val(g.n.y);
    for (int j = 0; j < 2; ++j) {
        out[2 + 4 * j] = val(g.rA[j].x); out[3 + 4 * j] = val(g.rA[j].y);
        out[4 + 4 * j] = val(g.rB[j].x); out[5 + 4 * j] = val(g.rB[j].y);
    }
    out[10] = val(g.nm[0]); out[11] = val(g.tm[0]); out[12] = val(g.nm[1]); out[13] = val(g.tm[1]);
    out[14] = val(g.vb[0]); out[15] = val(g.vb[1]);
    out[16] = val(g.k00); out[17] = val(g.k11); out[18] = val(g.k01);
    out[19] = val(g.m00); out[20] = val(g.m11); out[21] = val(g.m01);
    out[22] = val(g.mu); out[23] = __int_as_float(g.cnt);
}

__device__ __forceinline__ diff::Geom<float> unpack_geom(const float* gv) {
    diff::Geom<float> g;
    g.n = {gv[0], gv[1]};
    for (int j = 0; j < 2; ++j) {
        g.rA[j] = {gv[2 + 4 * j], gv[3 + 4 * j]};
        g.rB[j] = {gv[4 + 4 * j], gv[5 + 4 * j]};
    }
    g.nm[0] = gv[10]; g.tm[0] = gv[11]; g.nm[1] = gv[12]; g.tm[1] = gv[13];
    g.vb[0] = gv[14]; g.vb[1] = gv[15];
    g.k00 = gv[16]; g.k11 = gv[17]; g.k01 = gv[18]; g.m00 = gv[19]; g.m11 = gv[20]; g.m01 = gv[21];
    g.mu = gv[22];
    g.cnt = __float_as_int(gv[23]);
    return g;
}

// The geometry recomputed from the recorded state, in float.
__device__ __forceinline__ diff::Geom<float> replay_geom(const DW& d, const StepTape* tp, uint32_t t,
                                                         const diff::ContactK& k, float mu) {
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

// Records the constraint just built at t (vc0/vc1/pc) and checks that the
// differentiable restatement rebuilds it bit for bit; returns whether it did.
static __device__ __noinline__ bool tape_constraint(const DW& d, uint32_t t) {
    StepTape* tp = d.tape;
    const uint32_t id = d.t_id[t];
    tp->t_id[t] = id;
    if (id & 0x80000000u) return true;
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
    if (!same) atomicAdd(&tp->hdr[kTapeHdrMismatch], 1u);
    return same;
}

// ---- joints (revolute, point rows) ------------------------------------------------
__device__ __forceinline__ diff::JointK joint_k(const DW& d, uint32_t j) {
    diff::JointK k;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    k.mA = d.b_mass[a];
    k.mB = d.b_mass[b];
    k.an = d.j_anchor[j];
    k.writableA = is_accelerable(d.b_flags[a]) ? 1u : 0u;
    k.writableB = is_accelerable(d.b_flags[b]) ? 1u : 0u;
    return k;
}

// What a joint's warm start starts from: both velocities and the stored impulse.
__device__ __forceinline__ void tape_joint_warm(const DW& d, uint32_t t, uint32_t j, float4 vA, float4 vB) {
    StepTape* tp = d.tape;
    tp->warm[2 * (size_t)t] = vA;
    tp->warm[2 * (size_t)t + 1] = vB;
    const float4 i = d.j_imp[j];
    tp->imp0[t] = make_float4(i.x, i.y, 0.f, 0.f);
}

// After the warm start: the geometry the joint stored must be the one the
// differentiable restatement computes from the recorded positions, bit for bit.
static __device__ __noinline__ void tape_joint_check(const DW& d, uint32_t j) {
    StepTape* tp = d.tape;
    const diff::JointK k = joint_k(d, j);
    const diff::JGeom<float> g =
        diff::joint_geom_t(k, tp->p0[d.j_bodies[2 * j]].z, tp->p0[d.j_bodies[2 * j + 1]].z);
    const float4 r = d.j_r[j], m0 = d.j_m0[j];
    const bool same = g.rA.x == r.x && g.rA.y == r.y && g.rB.x == r.z && g.rB.y == r.w && g.exx == m0.x &&
                      g.eyx == m0.y && g.eyy == m0.w;
    if (!same) atomicAdd(&tp->hdr[kTapeHdrMismatch], 1u);
}

// The per-world layout of a recorded step: world w's constraints are the sweep
// positions [wseg[2w], wseg[2w] + wseg[2w+1]) with colour offsets wcol[w*kColStride..].
__device__ __forceinline__ void tape_world(const DW& d, uint32_t w, uint32_t base, uint32_t n, const uint32_t* col_off,
                                           uint32_t rank, uint32_t size) {
    StepTape* tp = d.tape;
    if (rank == 0) { tp->wseg[2 * w] = base; tp->wseg[2 * w + 1] = n; }
    for (uint32_t c = rank; c < (uint32_t)kColStride; c += size) tp->wcol[(size_t)w * kColStride + c] = col_off[c];
}

}  // namespace prgpu
