// prgpu_query.cu -- spatial queries over the broad-phase tree the step keeps:
// Query (DynamicTree.cpp:673-710) and RayCast (RayCastOutput.cpp:241-337) of
// one world, walked on the world's subtree of the batch LBVH (prgpu_contacts.cu),
// whose leaves hold the proxies' fat AABBs as the reference's tree does.
//
// One thread walks the tree for one query or ray with a stack of node indices;
// a batch of queries or rays runs as one launch.  A walk that would overflow
// its stack (a tree deeper than kWalkStack levels) stops and sets *status,
// which the host turns into an error of that call.
#include <cuda_runtime.h>

#include <algorithm>

#include "prgpu_contact_ops.cuh"
#include "prgpu_kernels.cuh"

namespace prgpu {

namespace {

constexpr int kWalkStack = 96;

__device__ __forceinline__ bool box_overlap(float4 a, float4 q) {
    // TestOverlap(AABB, AABB) (AABB.hpp): max of the mins <= min of the maxes on both axes
    const float maxOfMinsX = (a.x < q.x) ? q.x : a.x, minOfMaxsX = (q.z < a.z) ? q.z : a.z;
    const float maxOfMinsY = (a.y < q.y) ? q.y : a.y, minOfMaxsY = (q.w < a.w) ? q.w : a.w;
    return (minOfMaxsX >= maxOfMinsX) && (minOfMaxsY >= maxOfMinsY);
}

__device__ __forceinline__ float4 node_box(const DW& d, uint32_t node) {
    return (node & kLeafBit) ? d.l_leaf_box[node & ~kLeafBit] : d.l_node_box[node];
}

// Walks world w's subtree; calls leaf(shape) for each leaf whose box passes
// keep(box), children of branches whose box passes keep(box).  Returns false on
// stack overflow.
template <class Keep, class Leaf>
__device__ bool walk_tree(const DW& d, uint32_t w, Keep&& keep, Leaf&& leaf) {
    const uint32_t root = d.w_root[w];
    if (root == kNone) return true;
    uint32_t stack[kWalkStack];
    int sp = 0;
    stack[sp++] = root;
    while (sp > 0) {
        const uint32_t node = stack[--sp];
        if (!keep(node_box(d, node))) continue;
        if (node & kLeafBit) {
            const uint32_t shape = d.l_idx[node & ~kLeafBit];
            if (!(d.s_meta[shape] & kShapeNoProxy)) leaf(shape);
            continue;
        }
        if (sp + 2 > kWalkStack) return false;
        stack[sp++] = d.l_right[node];
        stack[sp++] = d.l_left[node];
    }
    return true;
}

// RayCast(radius, location, input) (RayCastOutput.cpp:41-71): the ray p1 -> p2
// (up to fraction maxF) against a circle.
__device__ bool ray_circle(float radius, V2 loc, V2 p1, V2 p2, float maxF, float& frac, V2& normal) {
    const V2 s = p1 - loc;
    const float b = mag2(s) - radius * radius;
    const V2 seg = p2 - p1;
    const float c = dot(s, seg);
    const float rr = mag2(seg);
    const float sigma = (c * c) - rr * b;
    if ((sigma < 0.f) || almost_zero(rr)) return false;
    const float a = -(c + sqrtf(sigma));
    const float f = a / rr;
    if ((f >= 0.f) && (f <= maxF)) {
        frac = f;
        normal = unit_vector(s + seg * f, mk(0.f, 0.f));
        return true;
    }
    return false;
}

// RayCast(DistanceProxy, input, transform) (RayCastOutput.cpp:132-233): a disk
// (one vertex) as a circle in world space; a polygon or edge in its own frame,
// each vertex as a circle of the vertex radius and each edge pushed out along
// its normal by that radius; the nearest crossing within maxF.
__device__ bool ray_shape(const Proxy& P, Xf xf, V2 p1, V2 p2, float maxF, float& frac, V2& normal) {
    const float radius = P.r;
    V2 v0 = P.vtx(0);
    if (P.count == 1) return ray_circle(radius, xform(v0, xf), p1, p2, maxF, frac, normal);
    const V2 r0 = invxform(p1, xf), r1 = invxform(p2, xf);
    const V2 ray = r1 - r0;
    float minT = nextafterf(maxF, 2.0f);
    V2 found = mk(0.f, 0.f);
    for (int i = 0; i < P.count; ++i) {
        float cf;
        V2 cn;
        if (ray_circle(radius, v0, r0, r1, maxF, cf, cn) && (minT > cf)) {
            minT = cf;
            found = cn;
        }
        const V2 v1 = P.vtx((i + 1 < P.count) ? i + 1 : 0);
        const V2 edge = v1 - v0;
        const float rxe = cross(ray, edge);
        if (!almost_zero(rxe)) {
            const V2 n = P.nrm(i);
            const V2 q = (v0 + n * radius) - r0;
            const float inv = 1.0f / rxe;
            const float t = cross(q, edge) * inv;
            const float u = cross(q, ray) * inv;
            if ((t >= 0.f) && (t <= 1.f) && (u >= 0.f) && (u <= 1.f) && (minT > t)) {
                minT = t;
                found = n;
            }
        }
        v0 = v1;
    }
    if (minT <= maxF) {
        frac = minT;
        normal = rotate(found, xf.q);
        return true;
    }
    return false;
}

// Query: world-local IDs of the shapes whose fat AABB overlaps the query box,
// up to cap per query (count holds the full number).
__global__ void k_query_boxes(DW d, uint32_t n, const uint32_t* worlds, const float4* boxes, uint32_t cap,
                              uint32_t* counts, uint32_t* out, uint32_t* status) {
    GRID_LOOP(k, n) {
        const uint32_t w = worlds[k];
        const float4 q = boxes[k];
        const uint32_t base = d.w_shape_off[w];
        uint32_t found = 0;
        uint32_t* dst = out + (size_t)k * cap;
        const bool ok = walk_tree(
            d, w, [&](float4 box) { return box_overlap(box, q); },
            [&](uint32_t shape) {
                if (found < cap) dst[found] = shape - base;
                ++found;
            });
        if (!ok) atomicOr(status, 1u);
        counts[k] = found;
    }
}

// RayCast of a world with the callback that clips the ray to every hit
// (RayCastOpcode::ClipRay): the nearest hit of each ray (ties: the lower shape
// ID), as shape (world-local, -1 none) and (fraction, point x y, normal x y).
__global__ void k_ray_nearest(DW d, uint32_t n, const uint32_t* worlds, const float* rays5, int32_t* shape_out,
                              float* hit5, uint32_t* status) {
    GRID_LOOP(k, n) {
        const uint32_t w = worlds[k];
        const float* r = rays5 + 5 * (size_t)k;
        const V2 p1 = mk(r[0], r[1]), p2 = mk(r[2], r[3]);
        const float maxF0 = r[4];
        const V2 delta = p2 - p1;
        // separating axis of the segment (RayCastOutput.cpp:243-244, 266-271)
        const V2 v = revperp(unit_vector(delta, mk(0.f, 0.f)));
        const V2 av = mk(fabsf(v.x), fabsf(v.y));
        float maxF = maxF0;
        int32_t best = -1;
        float bf = 0.f;
        V2 bn = mk(0.f, 0.f);
        const uint32_t base = d.w_shape_off[w];
        const bool ok = walk_tree(
            d, w,
            [&](float4 box) {
                const V2 e = p1 + delta * maxF;  // GetAABB(RayCastInput) (AABB.cpp:107-112)
                const float4 sbox = make_float4(fminf(p1.x, e.x), fminf(p1.y, e.y), fmaxf(p1.x, e.x), fmaxf(p1.y, e.y));
                if (!box_overlap(box, sbox)) return false;
                const V2 ctr = mk(0.5f * (box.x + box.z), 0.5f * (box.y + box.w));
                const V2 ext = mk(0.5f * (box.z - box.x), 0.5f * (box.w - box.y));
                return !(fabsf(dot(v, p1 - ctr)) - dot(av, ext) > 0.f);
            },
            [&](uint32_t shape) {
                Proxy P;
                load_proxy(d, shape, P);
                float f;
                V2 nrm;
                if (!ray_shape(P, load_xf(d, d.s_body[shape]), p1, p2, maxF, f, nrm)) return;
                const int32_t id = (int32_t)(shape - base);
                if (best < 0 || f < bf || (f == bf && id < best)) {
                    best = id;
                    bf = f;
                    bn = nrm;
                }
                maxF = f;  // ClipRay
            });
        if (!ok) atomicOr(status, 1u);
        shape_out[k] = best;
        float* h = hit5 + 5 * (size_t)k;
        const V2 pt = p1 + delta * bf;
        h[0] = (best >= 0) ? bf : 0.f;
        h[1] = (best >= 0) ? pt.x : 0.f;
        h[2] = (best >= 0) ? pt.y : 0.f;
        h[3] = bn.x;
        h[4] = bn.y;
    }
}

// RayCast of a world with the callback that keeps the whole ray
// (RayCastOpcode::ResetRay): every hit of one ray, up to cap, as shape and
// (fraction, point x y, normal x y); *count holds the full number.
__global__ void k_ray_all(DW d, uint32_t w, float p1x, float p1y, float p2x, float p2y, float maxF, uint32_t cap,
                          uint32_t* count, int32_t* shapes, float* hit5, uint32_t* status) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const V2 p1 = mk(p1x, p1y), p2 = mk(p2x, p2y);
    const V2 delta = p2 - p1;
    const V2 v = revperp(unit_vector(delta, mk(0.f, 0.f)));
    const V2 av = mk(fabsf(v.x), fabsf(v.y));
    const V2 e = p1 + delta * maxF;
    const float4 sbox = make_float4(fminf(p1.x, e.x), fminf(p1.y, e.y), fmaxf(p1.x, e.x), fmaxf(p1.y, e.y));
    const uint32_t base = d.w_shape_off[w];
    uint32_t found = 0;
    const bool ok = walk_tree(
        d, w,
        [&](float4 box) {
            if (!box_overlap(box, sbox)) return false;
            const V2 ctr = mk(0.5f * (box.x + box.z), 0.5f * (box.y + box.w));
            const V2 ext = mk(0.5f * (box.z - box.x), 0.5f * (box.w - box.y));
            return !(fabsf(dot(v, p1 - ctr)) - dot(av, ext) > 0.f);
        },
        [&](uint32_t shape) {
            Proxy P;
            load_proxy(d, shape, P);
            float f;
            V2 nrm;
            if (!ray_shape(P, load_xf(d, d.s_body[shape]), p1, p2, maxF, f, nrm)) return;
            if (found < cap) {
                const V2 pt = p1 + delta * f;
                shapes[found] = (int32_t)(shape - base);
                float* h = hit5 + 5 * (size_t)found;
                h[0] = f; h[1] = pt.x; h[2] = pt.y; h[3] = nrm.x; h[4] = nrm.y;
            }
            ++found;
        });
    if (!ok) atomicOr(status, 1u);
    *count = found;
}

}  // namespace

void launch_query_boxes(const DW& d, const Launch& L, uint32_t n, const uint32_t* worlds, const float4* boxes,
                        uint32_t cap, uint32_t* counts, uint32_t* out, uint32_t* status, cudaStream_t s) {
    const int grid = (int)std::min<uint32_t>((n + 127u) / 128u, (uint32_t)L.grid);
    k_query_boxes<<<grid > 0 ? grid : 1, 128, 0, s>>>(d, n, worlds, boxes, cap, counts, out, status);
}

void launch_ray_nearest(const DW& d, const Launch& L, uint32_t n, const uint32_t* worlds, const float* rays5,
                        int32_t* shape_out, float* hit5, uint32_t* status, cudaStream_t s) {
    const int grid = (int)std::min<uint32_t>((n + 127u) / 128u, (uint32_t)L.grid);
    k_ray_nearest<<<grid > 0 ? grid : 1, 128, 0, s>>>(d, n, worlds, rays5, shape_out, hit5, status);
}

void launch_ray_all(const DW& d, uint32_t w, const float* ray5, uint32_t cap, uint32_t* count, int32_t* shapes,
                    float* hit5, uint32_t* status, cudaStream_t s) {
    k_ray_all<<<1, 32, 0, s>>>(d, w, ray5[0], ray5[1], ray5[2], ray5[3], ray5[4], cap, count, shapes, hit5, status);
}

}  // namespace prgpu
