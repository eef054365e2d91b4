// prgpu_contact_ops.cuh -- per-proxy and per-contact operations shared by the
// step's contact maintenance (prgpu_contacts.cu) and its time-of-impact phase
// (prgpu_toi.cu): shape and transform loads, swept and fat AABBs, the moved-proxy
// list, manifolds in slot storage and the contact Update.
#pragma once

#include <cooperative_groups.h>

#include "prgpu_collide.cuh"
#include "prgpu_toi.cuh"
#include "prgpu_internal.cuh"

namespace prgpu {

__device__ __forceinline__ void load_proxy(const DW& d, uint32_t p, Proxy& out) {
    const uint4 rec = d.s_rec[p];
    const int nv = (int)((rec.x >> 8) & 0xffu);
    out.count = nv < kMaxVerts ? nv : kMaxVerts;
    out.r = __uint_as_float(rec.z);
    out.vn = d.verts + rec.y;
}

__device__ __forceinline__ Xf load_xf(const DW& d, uint32_t b) {
    const float4 x = d.b_xf[b];
    Xf t;
    t.p = mk(x.x, x.y);
    t.q = mk(x.z, x.w);
    return t;
}

__device__ __forceinline__ Xf xf0_of(const DW& d, uint32_t b) {
    const float4 p0 = d.b_pos0[b];
    const float4 m = d.b_mass[b];
    return get_xf(p0.x, p0.y, p0.z, mk(m.z, m.w));
}

// AABB helpers (AABB.cpp:51-62, Interval.hpp).
struct Box {
    float x0, y0, x1, y1;
};
__device__ __forceinline__ void box_include(Box& a, V2 p) {
    a.x0 = (a.x0 < p.x) ? a.x0 : p.x;
    a.x1 = (p.x < a.x1) ? a.x1 : p.x;
    a.y0 = (a.y0 < p.y) ? a.y0 : p.y;
    a.y1 = (p.y < a.y1) ? a.y1 : p.y;
}
__device__ __forceinline__ void box_fatten(Box& a, float r) {
    a.x0 = a.x0 - r; a.x1 = a.x1 + r;
    a.y0 = a.y0 - r; a.y1 = a.y1 + r;
}
__device__ __forceinline__ void box_displace(Box& a, V2 dsp) {
    if (dsp.x < 0.f) a.x0 += dsp.x; else a.x1 += dsp.x;
    if (dsp.y < 0.f) a.y0 += dsp.y; else a.y1 += dsp.y;
}
__device__ __forceinline__ bool overlap4(float4 a, float4 b) {
    {
        const float maxOfMins = (a.x < b.x) ? b.x : a.x;
        const float minOfMaxs = (b.z < a.z) ? b.z : a.z;
        if (!(minOfMaxs >= maxOfMins)) return false;
    }
    {
        const float maxOfMins = (a.y < b.y) ? b.y : a.y;
        const float minOfMaxs = (b.w < a.w) ? b.w : a.w;
        if (!(minOfMaxs >= maxOfMins)) return false;
    }
    return true;
}
__device__ __forceinline__ bool contains4(float4 a, Box b) {
    return a.x <= b.x0 && a.z >= b.x1 && a.y <= b.y0 && a.w >= b.y1;
}
// ComputeAABB(proxy, xf0, xf1) reading the shape from global memory.
__device__ __forceinline__ Box swept_aabb(const DW& d, uint32_t p, Xf x0, Xf x1) {
    Box a;
    a.x0 = __int_as_float(0x7f800000); a.y0 = a.x0;
    a.x1 = -a.x0; a.y1 = -a.x0;
    const uint4 rec = d.s_rec[p];
    const int nv = (int)((rec.x >> 8) & 0xffu);
    for (int i = 0; i < nv; ++i) {
        const float4 v = d.verts[rec.y + i];
        const V2 lv = mk(v.x, v.y);
        box_include(a, xform(lv, x0));
        box_include(a, xform(lv, x1));
    }
    box_fatten(a, __uint_as_float(rec.z));
    return a;
}

__device__ __forceinline__ void append_moved(const DW& d, uint32_t p) {
    cooperative_groups::coalesced_group g = cooperative_groups::coalesced_threads();
    uint32_t base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(&d.cnt->n_moved, g.size());
    base = g.shfl(base, 0);
    d.moved_list[base + g.thread_rank()] = p;
}

// Re-fattens and displaces the swept AABB of proxy p into its tree AABB.
__device__ __forceinline__ float4 fat_box(const DW& d, Box a, Xf x0, Xf x1) {
    box_fatten(a, d.conf->aabbExtension);
    const V2 disp = (x1.p - x0.p) * d.conf->displaceMultiplier;
    box_displace(a, disp);
    return make_float4(a.x0, a.y0, a.x1, a.y1);
}

// ---- manifolds in slot storage ---------------------------------------------
__device__ __forceinline__ Man load_manifold(const DW& d, uint32_t slot) {
    Man m;
    const uint32_t meta = d.m_meta[slot];
    m.type = (int)(meta & 0xfu);
    m.count = (int)((meta >> 4) & 0xfu);
    const float4 h = d.m_head[slot];
    m.ln = mk(h.x, h.y);
    m.lp = mk(h.z, h.w);
    const float4 p0 = d.m_p0[slot], p1 = d.m_p1[slot];
    m.plp[0] = mk(p0.x, p0.y); m.ni[0] = p0.z; m.ti[0] = p0.w;
    m.plp[1] = mk(p1.x, p1.y); m.ni[1] = p1.z; m.ti[1] = p1.w;
    const uint2 cf = d.m_cf[slot];
    m.cf[0] = cf.x; m.cf[1] = cf.y;
    return m;
}
__device__ __forceinline__ void store_manifold(const DW& d, uint32_t slot, const Man& m) {
    d.m_meta[slot] = (uint32_t)m.type | ((uint32_t)m.count << 4);
    d.m_head[slot] = make_float4(m.ln.x, m.ln.y, m.lp.x, m.lp.y);
    d.m_p0[slot] = make_float4(m.plp[0].x, m.plp[0].y, m.ni[0], m.ti[0]);
    d.m_p1[slot] = make_float4(m.plp[1].x, m.plp[1].y, m.ni[1], m.ti[1]);
    d.m_cf[slot] = make_uint2(m.cf[0], m.cf[1]);
}

// A sensor contact's touching state: TestOverlap (Distance.cpp:205-216) >= 0,
// i.e. GJK Distance from an empty cache with StepConf::maxDistanceIters
// (GetDistanceConf, DistanceConf.cpp:36-41), then the total vertex radius squared
// less the squared distance of the witness points.
static __device__ __noinline__ bool sensor_touching(const DW& d, uint2 pr, uint2 bd) {
    Proxy A, B;
    load_proxy(d, pr.x, A);
    load_proxy(d, pr.y, B);
    SCache cache;
    cache.n = 0;
    cache.metric = 0.f;
    const DistOut di = gjk_distance(A, load_xf(d, bd.x), B, load_xf(d, bd.y), cache, d.conf->maxDistanceIters);
    V2 wa, wb;
    witness_points(di.s, wa, wb);
    const float tr = A.r + B.r;
    return (tr * tr - mag2(wb - wa)) >= 0.f;
}

// AabbTreeWorld::Update (AabbTreeWorld.cpp:2587-2721) without listeners.
// src2 (optional): where the new manifold's points took their impulses from.
// kSensors false: the caller passes no sensor contact, and the GJK of the
// sensor test stays out of its kernel (its registers would cost the bulk
// update pass its occupancy).
template <bool kSensors = true>
static __device__ void update_contact(const DW& d, uint32_t slot, int8_t* src2 = nullptr) {
    const uint2 pr = d.cs_proxy[slot];
    const uint2 bd = d.cs_body[slot];
    uint32_t flags = d.cs_flags[slot];
    bool touching = false;
    int src[2] = {-1, -1};
    if (kSensors && (flags & CF_SENSOR)) {
        touching = sensor_touching(d, pr, bd);  // sensors make no manifold (:2634)
        store_manifold(d, slot, man_empty());
    } else {
        Proxy A, B;
        load_proxy(d, pr.x, A);
        load_proxy(d, pr.y, B);
        const Man old = load_manifold(d, slot);
        Man nm = collide_shapes(A, load_xf(d, bd.x), B, load_xf(d, bd.y), d.conf->linearSlop, d.conf->maxCirclesRatio);
        touching = nm.count > 0;
        transfer_impulses(nm, old, src);
        store_manifold(d, slot, nm);
    }
    if (src2) { src2[0] = (int8_t)src[0]; src2[1] = (int8_t)src[1]; }
    flags &= ~CF_NEEDS_UPDATE;
    flags = touching ? (flags | CF_TOUCHING) : (flags & ~CF_TOUCHING);
    d.cs_flags[slot] = flags;
    // which phases of this step updated the contact (the listener replay)
    const uint32_t tag = d.cnt->step_no << 3, old = d.cs_upd[slot];
    d.cs_upd[slot] = (((old & ~7u) == tag) ? old : tag) | d.cnt->upd_phase;
}

}  // namespace prgpu
