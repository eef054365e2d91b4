// prgpu_contacts.cu -- proxies, broadphase (LBVH) and contact maintenance.
//
// Restates the contact bookkeeping of AabbTreeWorld.cpp for a batch of worlds:
//  * CreateProxies / Synchronize (:557-579, :2564-2585): each proxy keeps its
//    persistent fat AABB, rewritten only when the swept AABB escapes it;
//  * DestroyContacts (:2290-2331): contacts whose fat AABBs stop overlapping;
//  * UpdateContacts / Update (:2333-2415, :2587-2721): CollideShapes for
//    contacts of bodies that moved, with warm-start transfer;
//  * FindContacts + AddContacts (:709-751, :2423-2547): the DynamicTree query
//    becomes an LBVH rebuilt from 30-bit Morton codes (world index above the
//    code, so every world is one subtree) with per-thread stack traversal.
// The live contact set is a key-sorted list of (ContactKey, slot) pairs;
// contact data stays in its slot for the contact's lifetime.
#include <cooperative_groups.h>

#include "prgpu_collide.cuh"
#include "prgpu_contact_ops.cuh"
#include "prgpu_kernels.cuh"

namespace cg = cooperative_groups;

namespace prgpu {

namespace {

// Pre-step proxy maintenance: CreateProxies for new shapes and Synchronize of
// bodies whose state the host changed (AabbTreeWorld.cpp:2159-2182).
__global__ void k_pre_proxies(DW d) {
    GRID_LOOP(p, d.n_shapes) {
        const uint32_t state = d.p_moved[p];
        const uint32_t b = d.s_body[p];
        const uint32_t bf = d.b_flags[b];
        uint32_t moved = 0;
        if (d.s_meta[p] & kShapeNoProxy) {
            // no proxy: an inverted box, which overlaps nothing and leaves every
            // union it enters unchanged
            const float inf = __int_as_float(0x7f800000);
            d.p_aabb[p] = make_float4(inf, inf, -inf, -inf);
        } else if (state == 2u) {
            const Xf x0 = xf0_of(d, b), x1 = load_xf(d, b);
            d.p_aabb[p] = fat_box(d, swept_aabb(d, p, x0, x1), x0, x1);
            moved = 1u;
        } else if (bf & BF_DIRTY) {
            const Xf x0 = xf0_of(d, b), x1 = load_xf(d, b);
            const Box a = swept_aabb(d, p, x0, x1);
            if (!contains4(d.p_aabb[p], a)) {
                d.p_aabb[p] = fat_box(d, a, x0, x1);
                moved = 1u;
            }
        }
        d.p_moved[p] = moved;
        if (moved) append_moved(d, p);
    }
}

// Post-solve Synchronize of the proxies of islanded speedable bodies
// (AabbTreeWorld.cpp:1532-1544, :2564-2585).
__global__ void k_synchronize(DW d) {
    GRID_LOOP(p, d.n_shapes) {
        const uint32_t b = d.s_body[p];
        const uint32_t bf = d.b_flags[b];
        uint32_t moved = 0;
        if ((bf & BF_SOLVED) && is_speedable(bf)) {
            const Xf x0 = xf0_of(d, b), x1 = load_xf(d, b);
            const Box a = swept_aabb(d, p, x0, x1);
            if (!contains4(d.p_aabb[p], a)) {
                d.p_aabb[p] = fat_box(d, a, x0, x1);
                moved = 1u;
            }
        }
        d.p_moved[p] = moved;
        if (moved) append_moved(d, p);
    }
}

__global__ void k_moved_done(DW d) {
    Counters* c = d.cnt;
    c->st_proxies_moved += c->n_moved;
    c->need_find = c->n_moved > 0u ? 1u : 0u;
    c->n_new = 0u;
}

// Work class of a contact update: its shapes' vertex counts (1 a disk, 2 an
// edge, up to 8 told apart, in either order) and whether it touched after its
// last update, which decides whether the narrowphase stops after the
// separation tests or goes on to clip a manifold.
constexpr uint32_t kUpdClasses = 128;
constexpr uint32_t kUpdThreads = 256;
constexpr uint32_t kUpdPerThread = 4;
constexpr uint32_t kUpdWindow = kUpdThreads * kUpdPerThread;
__device__ __forceinline__ uint32_t update_class(const DW& d, uint32_t slot, uint32_t f) {
    const uint2 pr = d.cs_proxy[slot];
    const uint32_t na = min(max((d.s_rec[pr.x].x >> 8) & 0xffu, 1u), 8u) - 1u;
    const uint32_t nb = min(max((d.s_rec[pr.y].x >> 8) & 0xffu, 1u), 8u) - 1u;
    return ((f & CF_TOUCHING) ? 64u : 0u) | (min(na, nb) << 3) | max(na, nb);
}

// Each contact's update touches only its own slot, so the pass walks the slots
// in ascending order (live ones by their flag) rather than the key-ordered live
// list: the slot-indexed records are then read in coalesced runs.  A block takes
// a window of kUpdWindow slots at a time, sorts the ones that need an update by
// work class in shared memory (a counting sort) and deals the sorted list out in
// runs of 32, so that a warp's lanes run the same narrowphase case, no lane
// idles on a contact that needs no update, and each warp gets runs from all over
// the list (the block waits for its slowest warp at the end of each window).
// Four blocks a multiprocessor (64 registers) measured faster than three (80
// registers, no spills) and than five (48, spilling).
__global__ void __launch_bounds__(kUpdThreads, 4) k_update_contacts(DW d, uint32_t body_mask) {
    __shared__ uint32_t s_at[kUpdClasses];            // per class: count, then first position
    __shared__ uint32_t s_wsum[kUpdClasses / 32u];
    __shared__ uint32_t s_slot[kUpdWindow];
    uint32_t updated = 0;
    // the post-solve pass of a recorded step notes each update's impulse sources
    int8_t* rec = (d.tape && body_mask == BF_MOVED) ? d.tape->src : nullptr;
    // The pre-phase pass updates the contacts of bodies the host changed; a contact
    // flagged CF_NEEDS_UPDATE at creation is updated there and then, so with no
    // body changed there is nothing to do.
    if (body_mask == BF_DIRTY && !d.cnt->dirty_any) return;
    const uint32_t hw = d.cnt->high_water, t = threadIdx.x, lane = t & 31u;
    for (uint32_t base = blockIdx.x * kUpdWindow; base < hw; base += gridDim.x * kUpdWindow) {
        if (t < kUpdClasses) s_at[t] = 0u;
        __syncthreads();
        uint32_t pick[kUpdPerThread];  // class << 16 | rank within the class, or kNone
#pragma unroll
        for (uint32_t k = 0; k < kUpdPerThread; ++k) {
            const uint32_t slot = base + k * kUpdThreads + t;
            pick[k] = kNone;
            if (slot < hw) {
                const uint32_t f = d.cs_flags[slot];
                if ((f & (CF_LIVE | CF_SENSOR)) == CF_LIVE) {
                    const uint2 bd = d.cs_body[slot];
                    if ((f & CF_NEEDS_UPDATE) || (d.b_flags[bd.x] & body_mask) || (d.b_flags[bd.y] & body_mask)) {
                        const uint32_t cls = update_class(d, slot, f);
                        pick[k] = (cls << 16) | atomicAdd(&s_at[cls], 1u);
                    }
                }
            }
        }
        __syncthreads();
        // exclusive scan of the class counts: warp scans, then the warps' totals
        uint32_t cnt = 0u, incl = 0u;
        if (t < kUpdClasses) {
            cnt = incl = s_at[t];
            for (uint32_t o = 1u; o < 32u; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            if (lane == 31u) s_wsum[t >> 5] = incl;
        }
        __syncthreads();
        uint32_t total = 0u, before = 0u;
        for (uint32_t k = 0; k < kUpdClasses / 32u; ++k) {
            if (k < (t >> 5)) before += s_wsum[k];
            total += s_wsum[k];
        }
        if (t < kUpdClasses) s_at[t] = before + incl - cnt;
        __syncthreads();
#pragma unroll
        for (uint32_t k = 0; k < kUpdPerThread; ++k)
            if (pick[k] != kNone) s_slot[s_at[pick[k] >> 16] + (pick[k] & 0xffffu)] = base + k * kUpdThreads + t;
        __syncthreads();
        for (uint32_t e = t; e < total; e += kUpdThreads) {
            const uint32_t sl = s_slot[e];
            update_contact<false>(d, sl, rec ? rec + 2 * (size_t)sl : nullptr);
            ++updated;
        }
        __syncthreads();  // s_at and s_slot are refilled for the next window
    }
    if (updated) atomicAdd(&d.cnt->st_contacts_updated, updated);
}

// The sensor contacts of the same pass (TestOverlap instead of CollideShapes).
__global__ void k_update_sensors(DW d, uint32_t body_mask) {
    if (body_mask == BF_DIRTY && !d.cnt->dirty_any) return;
    uint32_t updated = 0;
    GRID_LOOP(slot, d.cnt->high_water) {
        const uint32_t f = d.cs_flags[slot];
        if ((f & (CF_LIVE | CF_SENSOR)) != (CF_LIVE | CF_SENSOR)) continue;
        const uint2 bd = d.cs_body[slot];
        if ((f & CF_NEEDS_UPDATE) || (d.b_flags[bd.x] & body_mask) || (d.b_flags[bd.y] & body_mask)) {
            update_contact<true>(d, slot);
            ++updated;
        }
    }
    if (updated) atomicAdd(&d.cnt->st_contacts_updated, updated);
}

// ---- DestroyContacts (overlap pass) ----------------------------------------
__global__ void k_destroy_flags(DW d) {
    GRID_LOOP(i, d.cnt->n_live) {
        const uint32_t slot = d.c_slot[i];
        const uint2 pr = d.cs_proxy[slot];
        const bool keep = overlap4(d.p_aabb[pr.x], d.p_aabb[pr.y]);
        d.flags[i] = keep ? 1u : 0u;
        if (!keep) {
            // InternalDestroy (AabbTreeWorld.cpp:2270-2276): a touching contact
            // that goes away wakes both bodies and resets their sleep timers.
            const uint32_t meta = d.m_meta[slot];
            if (((meta >> 4) & 0xfu) > 0u && !(d.cs_flags[slot] & CF_SENSOR)) {
                const uint2 bd = d.cs_body[slot];
                if (is_speedable(d.b_flags[bd.x])) { atomicOr(&d.b_flags[bd.x], BF_AWAKE); d.b_uat[bd.x] = 0.f; }
                if (is_speedable(d.b_flags[bd.y])) { atomicOr(&d.b_flags[bd.y], BF_AWAKE); d.b_uat[bd.y] = 0.f; }
            }
        }
    }
}

__global__ void k_destroy_scatter(DW d) {
    const uint32_t top = d.cnt->free_top;
    GRID_LOOP(i, d.cnt->n_live) {
        const uint32_t slot = d.c_slot[i];
        const uint32_t s = d.scan[i];
        if (d.flags[i]) {
            d.c_key_alt[s] = d.c_key[i];
            d.c_slot_alt[s] = slot;
        } else {
            d.free_stack[top + (i - s)] = slot;
            d.cs_flags[slot] = 0u;
        }
    }
}

__global__ void k_destroy_done(DW d) {
    Counters* c = d.cnt;
    const uint32_t kept = c->scan_total;
    const uint32_t destroyed = c->n_live - kept;
    c->free_top += destroyed;
    c->n_live = kept;
    c->st_contacts_destroyed += destroyed;
}

__global__ void k_copy_live(DW d) {
    GRID_LOOP(i, d.cnt->n_live) {
        d.c_key[i] = d.c_key_alt[i];
        d.c_slot[i] = d.c_slot_alt[i];
    }
}

// ---- LBVH -------------------------------------------------------------------
__device__ __forceinline__ uint32_t part1by1(uint32_t x) {
    x &= 0x0000ffffu;
    x = (x | (x << 8)) & 0x00ff00ffu;
    x = (x | (x << 4)) & 0x0f0f0f0fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}

__global__ void k_lbvh_bounds_reset(DW d) {
    if (!d.cnt->need_find || !d.cnt->lbvh_rebuild) return;
    GRID_LOOP(w, d.n_worlds) {
        const uint32_t inf = float_to_ordered(__int_as_float(0x7f800000));
        const uint32_t ninf = float_to_ordered(-__int_as_float(0x7f800000));
        d.w_bounds[w] = make_float4(__uint_as_float(inf), __uint_as_float(inf), __uint_as_float(ninf),
                                    __uint_as_float(ninf));
        d.w_root[w] = kNone;
    }
}

__global__ void k_lbvh_bounds(DW d) {
    if (!d.cnt->need_find || !d.cnt->lbvh_rebuild) return;
    GRID_LOOP(p, d.n_shapes) {
        if (d.s_meta[p] & kShapeNoProxy) continue;
        const float4 a = d.p_aabb[p];
        const float cx = 0.5f * (a.x + a.z), cy = 0.5f * (a.y + a.w);
        const uint32_t w = d.b_world[d.s_body[p]];
        uint32_t* wb = reinterpret_cast<uint32_t*>(&d.w_bounds[w]);
        atomicMin(&wb[0], float_to_ordered(cx));
        atomicMin(&wb[1], float_to_ordered(cy));
        atomicMax(&wb[2], float_to_ordered(cx));
        atomicMax(&wb[3], float_to_ordered(cy));
    }
}

__global__ void k_lbvh_morton(DW d) {
    if (!d.cnt->need_find || !d.cnt->lbvh_rebuild) return;
    GRID_LOOP(p, d.n_shapes) {
        const float4 a = d.p_aabb[p];
        // a shape without a proxy (inverted box) sorts to its world's corner
        const bool none = (d.s_meta[p] & kShapeNoProxy) != 0u;
        const float cx = none ? 0.f : 0.5f * (a.x + a.z), cy = none ? 0.f : 0.5f * (a.y + a.w);
        const uint32_t w = d.b_world[d.s_body[p]];
        const uint32_t* wb = reinterpret_cast<const uint32_t*>(&d.w_bounds[w]);
        const float bx0 = ordered_to_float(wb[0]), by0 = ordered_to_float(wb[1]);
        const float bx1 = ordered_to_float(wb[2]), by1 = ordered_to_float(wb[3]);
        const float ex = fmaxf(bx1 - bx0, 1e-30f), ey = fmaxf(by1 - by0, 1e-30f);
        const float nx = fminf(fmaxf((cx - bx0) / ex, 0.f), 1.f);
        const float ny = fminf(fmaxf((cy - by0) / ey, 0.f), 1.f);
        const uint32_t qx = min((uint32_t)(nx * 32767.f), 32767u);
        const uint32_t qy = min((uint32_t)(ny * 32767.f), 32767u);
        const uint32_t morton = (part1by1(qx) << 1) | part1by1(qy);
        d.l_key[p] = ((uint64_t)w << 30) | (uint64_t)morton;
        d.l_idx[p] = p;
    }
}

__device__ __forceinline__ int lb_delta(const uint64_t* __restrict__ keys, int n, int i, long long j) {
    if (j < 0 || j >= n) return -1;
    const uint64_t a = keys[i], b = keys[(int)j];
    if (a == b) return 64 + __clz((uint32_t)i ^ (uint32_t)j);
    return __clzll((long long)(a ^ b));
}

// Karras (2012) radix-tree construction over the sorted keys.
__global__ void k_lbvh_internal(DW d) {
    if (!d.cnt->need_find || !d.cnt->lbvh_rebuild) return;
    const int n = (int)d.n_shapes;
    const uint64_t* keys = d.l_key;
    GRID_LOOP(ui, (uint32_t)(n - 1)) {
        const int i = (int)ui;
        const int dir = (lb_delta(keys, n, i, i + 1) - lb_delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
        const int dmin = lb_delta(keys, n, i, (long long)i - dir);
        long long lmax = 2;
        for (int g = 0; g < 40 && lb_delta(keys, n, i, i + lmax * dir) > dmin; ++g) lmax *= 2;
        long long l = 0;
        for (long long t = lmax / 2; t >= 1; t /= 2) {
            if (lb_delta(keys, n, i, i + (l + t) * dir) > dmin) l += t;
        }
        const long long j = i + l * dir;
        const int dnode = lb_delta(keys, n, i, j);
        long long s = 0;
        long long t = l;
        for (int g = 0; g < 64; ++g) {
            t = (t + 1) / 2;
            if (lb_delta(keys, n, i, i + (s + t) * dir) > dnode) s += t;
            if (t <= 1) break;
        }
        const int gamma = (int)(i + s * dir + min(dir, 0));
        const int lo = (int)min((long long)i, j), hi = (int)max((long long)i, j);
        const uint32_t left = (lo == gamma) ? ((uint32_t)gamma | kLeafBit) : (uint32_t)gamma;
        const uint32_t right = (hi == gamma + 1) ? ((uint32_t)(gamma + 1) | kLeafBit) : (uint32_t)(gamma + 1);
        d.l_left[i] = left;
        d.l_right[i] = right;
        d.l_range[2 * i] = (uint32_t)lo;
        d.l_range[2 * i + 1] = (uint32_t)hi;
        d.l_parent[(left & kLeafBit) ? (uint32_t)(n - 1) + (left & ~kLeafBit) : left] = (uint32_t)i;
        d.l_parent[(right & kLeafBit) ? (uint32_t)(n - 1) + (right & ~kLeafBit) : right] = (uint32_t)i;
        d.l_visit[i] = 0u;
        if (i == 0) d.l_parent[0] = kNone;
    }
}

__global__ void k_lbvh_leaves(DW d) {
    if (!d.cnt->need_find) return;
    const bool rebuild = d.cnt->lbvh_rebuild != 0u;
    GRID_LOOP(k, d.n_shapes) {
        const uint32_t p = d.l_idx[k];
        d.l_leaf_box[k] = d.p_aabb[p];
        if (rebuild) {
            d.l_inv[p] = k;
            if (k + 1 < d.n_shapes) d.l_visit[k] = 0u;  // refit counters (internal nodes)
        }
    }
}

// Bottom-up box computation of a rebuilt tree: the second child to arrive at a
// node computes its box.
__global__ void k_lbvh_refit(DW d) {
    if (!d.cnt->need_find || !d.cnt->lbvh_rebuild) return;
    const uint32_t n = d.n_shapes;
    if (n < 2) return;
    GRID_LOOP(k, n) {
        uint32_t node = d.l_parent[(n - 1) + k];
        for (int guard = 0; guard < 256 && node != kNone; ++guard) {
            __threadfence();
            if (atomicAdd(&d.l_visit[node], 1u) == 0u) break;
            const uint32_t l = d.l_left[node], r = d.l_right[node];
            const float4 a = (l & kLeafBit) ? d.l_leaf_box[l & ~kLeafBit] : __ldcg(&d.l_node_box[l]);
            const float4 b = (r & kLeafBit) ? d.l_leaf_box[r & ~kLeafBit] : __ldcg(&d.l_node_box[r]);
            d.l_node_box[node] = make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fmaxf(a.z, b.z), fmaxf(a.w, b.w));
            __threadfence();
            node = d.l_parent[node];
        }
    }
}

__device__ __forceinline__ void atomic_min_box(float* a, float v) {
    // ordered as signed integers when v >= 0, as unsigned (reversed) when v < 0
    if (v >= 0.f) atomicMin(reinterpret_cast<int*>(a), __float_as_int(v));
    else atomicMax(reinterpret_cast<unsigned int*>(a), __float_as_uint(v));
}
__device__ __forceinline__ void atomic_max_box(float* a, float v) {
    if (v >= 0.f) atomicMax(reinterpret_cast<int*>(a), __float_as_int(v));
    else atomicMin(reinterpret_cast<unsigned int*>(a), __float_as_uint(v));
}

// Refit between rebuilds: only the proxies that moved have new boxes, so each
// moved leaf widens its ancestors (atomic min/max per side) until one already
// contains its box.  Node boxes then still contain every leaf below them, so a
// search returns exactly the same pairs as over tight boxes; they only stay as
// wide as the widest box seen since the rebuild.  An ancestor that contained the
// box because another leaf widened it is widened above by that leaf's own walk,
// and boxes are convex, so every ancestor ends up containing every moved leaf.
__global__ void k_lbvh_expand(DW d) {
    if (!d.cnt->need_find || d.cnt->lbvh_rebuild) return;
    const uint32_t n = d.n_shapes;
    if (n < 2) return;
    GRID_LOOP(m, d.cnt->n_moved) {
        const uint32_t p = d.moved_list[m];
        const float4 b = d.p_aabb[p];
        uint32_t node = d.l_parent[(n - 1) + d.l_inv[p]];
        for (int guard = 0; guard < 256 && node != kNone; ++guard) {
            const float4 nb = __ldcg(&d.l_node_box[node]);
            if (nb.x <= b.x && nb.y <= b.y && nb.z >= b.z && nb.w >= b.w) break;
            float* f = reinterpret_cast<float*>(&d.l_node_box[node]);
            if (b.x < nb.x) atomic_min_box(f + 0, b.x);
            if (b.y < nb.y) atomic_min_box(f + 1, b.y);
            if (b.z > nb.z) atomic_max_box(f + 2, b.z);
            if (b.w > nb.w) atomic_max_box(f + 3, b.w);
            node = d.l_parent[node];
        }
    }
}

// Row starts of the sorted live list by smaller proxy: c_first[p] is the first
// entry whose key's smaller proxy is >= p (c_first[S] = n_live), so the live
// contacts whose smaller proxy is p are the entries [c_first[p], c_first[p+1]).
__global__ void k_contact_rows(DW d) {
    if (!d.cnt->need_find) return;
    const uint32_t nl = d.cnt->n_live, kb = d.key_bits, ns = d.n_shapes;
    GRID_LOOP(i, nl + 1u) {
        const uint32_t lo = (i < nl) ? (uint32_t)(d.c_key[i] >> kb) : ns;
        const uint32_t from = (i > 0u) ? (uint32_t)(d.c_key[i - 1u] >> kb) + 1u : 0u;
        for (uint32_t p = from; p <= lo && p <= ns; ++p) d.c_first[p] = i;
    }
}

// Root of each world's subtree: the highest node whose leaves all belong to it.
__global__ void k_lbvh_roots(DW d) {
    if (!d.cnt->need_find || !d.cnt->lbvh_rebuild) return;
    const uint32_t n = d.n_shapes;
    GRID_LOOP(i, n) {
        // leaf i: a world with a single proxy has that leaf as its root
        const uint32_t w = (uint32_t)(d.l_key[i] >> 30);
        if (d.w_shape_off[w + 1] - d.w_shape_off[w] == 1u) d.w_root[w] = i | kLeafBit;
        if (i + 1 < n) {
            const uint32_t lo = d.l_range[2 * i], hi = d.l_range[2 * i + 1];
            const uint32_t wl = (uint32_t)(d.l_key[lo] >> 30), wh = (uint32_t)(d.l_key[hi] >> 30);
            if (wl == wh) {
                const uint32_t p = d.l_parent[i];
                bool root = (p == kNone);
                if (!root) {
                    const uint32_t plo = d.l_range[2 * p], phi = d.l_range[2 * p + 1];
                    root = (d.l_key[plo] >> 30) != (d.l_key[phi] >> 30);
                }
                if (root) d.w_root[wl] = i;
            }
        }
    }
}

// ShouldCollide over joints (AabbTreeWorld.cpp:479-490) and filters (Filter.hpp:81-88),
// plus EitherIsAccelerable (:474-477).
__device__ __forceinline__ bool should_collide(const DW& d, uint32_t pa, uint32_t pb, uint32_t ba, uint32_t bb) {
    if (!(is_accelerable(d.b_flags[ba]) || is_accelerable(d.b_flags[bb]))) return false;
    for (uint32_t j = d.b_jnt_off[ba]; j < d.b_jnt_off[ba + 1]; ++j) {
        if (d.b_jnt_other[j] == bb && !d.b_jnt_cc[j]) return false;
    }
    const int ga = d.s_group[pa], gb = d.s_group[pb];
    if (ga == gb && ga != 0) return ga > 0;
    const uint32_t fa = d.s_filter[pa], fb = d.s_filter[pb];
    return (((fa >> 16) & (fb & 0xffffu)) != 0u) && (((fb >> 16) & (fa & 0xffffu)) != 0u);
}

__device__ __forceinline__ uint32_t lower_bound_u64(const uint64_t* a, uint32_t n, uint64_t key) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// FindContacts + the AddContacts filters for every moved proxy; keys of pairs
// that pass and are not yet contacts are appended to n_key.
__global__ void __launch_bounds__(128) k_find_pairs(DW d) {
    const uint32_t kb = d.key_bits;
    GRID_LOOP(m, d.cnt->n_moved) {
        const uint32_t p = d.moved_list[m];
        const uint32_t bp = d.s_body[p];
        const uint32_t w = d.b_world[bp];
        const uint32_t root = d.w_root[w];
        if (root == kNone || (root & kLeafBit)) continue;
        const float4 box = d.p_aabb[p];
        uint32_t stack[64];
        int sp = 0;
        if (overlap4(__ldcg(&d.l_node_box[root]), box)) stack[sp++] = root;
        while (sp > 0) {
            const uint32_t node = stack[--sp];
            const uint32_t ch[2] = {d.l_left[node], d.l_right[node]};
            for (int c = 0; c < 2; ++c) {
                const uint32_t x = ch[c];
                if (x & kLeafBit) {
                    const uint32_t k = x & ~kLeafBit;
                    if (!overlap4(d.l_leaf_box[k], box)) continue;
                    const uint32_t q = d.l_idx[k];
                    if (q == p) continue;
                    const uint32_t bq = d.s_body[q];
                    if (bq == bp) continue;
                    if (d.p_moved[q] && q < p) continue;  // emitted by q's own query
                    const uint32_t lo = min(p, q), hi = max(p, q);
                    if (!should_collide(d, lo, hi, d.s_body[lo], d.s_body[hi])) continue;
                    const uint64_t key = ((uint64_t)lo << kb) | (uint64_t)hi;
                    // already a contact: a short scan of lo's row of the live list
                    bool live = false;
                    for (uint32_t at = d.c_first[lo], end = d.c_first[lo + 1u]; at < end; ++at) {
                        const uint64_t k2 = d.c_key[at];
                        if (k2 >= key) { live = (k2 == key); break; }
                    }
                    if (live) continue;
                    cg::coalesced_group g = cg::coalesced_threads();
                    uint32_t base = 0;
                    if (g.thread_rank() == 0) base = atomicAdd(&d.cnt->n_new, g.size());
                    base = g.shfl(base, 0);
                    const uint32_t idx = base + g.thread_rank();
                    if (idx < d.cand_cap) {
                        d.n_key[idx] = key;
                        d.n_val[idx] = idx;
                    } else {
                        set_error(d.cnt, PR_ECAPACITY, 10u);
                    }
                } else if (overlap4(__ldcg(&d.l_node_box[x]), box)) {
                    if (sp < 64) stack[sp++] = x;
                    else set_error(d.cnt, PR_ECAPACITY, 11u);
                }
            }
        }
    }
}

__global__ void k_pairs_done(DW d) {
    Counters* c = d.cnt;
    if (c->n_new > d.cand_cap) c->n_new = d.cand_cap;
}

// AddContacts (AabbTreeWorld.cpp:2496-2541): slot allocation (free stack top
// first), contact initialisation, wake-up, and the first Update.
__global__ void k_new_contacts(DW d) {
    const uint32_t ft = d.cnt->free_top;
    const uint32_t hw = d.cnt->high_water;
    const uint64_t seq = d.cnt->seq_next;
    const uint32_t kb = d.key_bits;
    const uint64_t mask = (1ull << kb) - 1ull;
    GRID_LOOP(i, d.cnt->n_new) {
        const uint64_t key = d.n_key[i];
        const uint32_t pa = (uint32_t)(key >> kb), pb = (uint32_t)(key & mask);
        const uint32_t slot = (i < ft) ? d.free_stack[ft - 1u - i] : hw + (i - ft);
        if (slot >= d.contact_cap) {
            set_error(d.cnt, PR_ECAPACITY, 12u);
            d.n_val[i] = 0u;
            continue;
        }
        const uint32_t ba = d.s_body[pa], bb = d.s_body[pb];
        const uint32_t fa = d.b_flags[ba], fb = d.b_flags[bb];
        d.cs_proxy[slot] = make_uint2(pa, pb);
        d.cs_body[slot] = make_uint2(ba, bb);
        const bool sensor = ((d.s_meta[pa] | d.s_meta[pb]) & kShapeSensor) != 0u;
        uint32_t flags = CF_NEEDS_UPDATE | CF_LIVE;
        if (is_impenetrable(fa) || is_impenetrable(fb)) flags |= CF_IMPENETRABLE;
        if (sensor) flags |= CF_SENSOR;
        d.cs_flags[slot] = flags;
        const float2 ma = d.s_mat[pa], mb = d.s_mat[pb];
        d.cs_mat[slot] = make_float2(sqrtf(ma.x * mb.x), (ma.y > mb.y) ? ma.y : mb.y);
        d.cs_tspeed[slot] = 0.f;
        d.cs_colour[slot] = kNone;
        // AddContacts appends in key order to the world's and both bodies' contact lists
        d.cs_seq[slot] = seq + i;
        d.cs_prio[slot] = contact_prio(d, pa, pb);
        d.cs_upd[slot] = 0u;
        d.cs_toi_ep[slot] = 0u;
        d.cs_toi_at[slot] = 0u;
        if (d.cs_post_tag) d.cs_post_tag[slot] = make_uint2(0u, 0u);
        store_manifold(d, slot, man_empty());
        if (!sensor) {
            if (is_speedable(fa)) atomicOr(&d.b_flags[ba], BF_AWAKE);
            if (is_speedable(fb)) atomicOr(&d.b_flags[bb], BF_AWAKE);
        }
        update_contact(d, slot);
        if (d.tape) d.tape->created[slot] = 1u;  // starts without impulses
        d.n_val[i] = slot;
    }
}

__global__ void k_new_done(DW d) {
    Counters* c = d.cnt;
    const uint32_t nn = c->n_new;
    const uint32_t from_stack = min(nn, c->free_top);
    c->free_top -= from_stack;
    c->high_water += nn - from_stack;
    c->seq_next += nn;
    if (c->high_water > d.contact_cap) { set_error(c, PR_ECAPACITY, 13u); c->high_water = d.contact_cap; }
    c->st_contacts_added += nn;
}

// Merge of the live list with the (sorted) new keys: each element's output
// position is its own index plus its rank in the other list.
__global__ void k_merge(DW d) {
    const uint32_t na = d.cnt->n_live, nb = d.cnt->n_new;
    GRID_LOOP(i, na + nb) {
        if (i < na) {
            const uint64_t a = d.c_key[i];
            const uint32_t pos = i + lower_bound_u64(d.n_key, nb, a);
            if (pos >= d.contact_cap) { set_error(d.cnt, PR_ECAPACITY, 14u); continue; }
            d.c_key_alt[pos] = a;
            d.c_slot_alt[pos] = d.c_slot[i];
        } else {
            const uint32_t j = i - na;
            const uint64_t b = d.n_key[j];
            const uint32_t pos = j + lower_bound_u64(d.c_key, na, b);
            if (pos >= d.contact_cap) { set_error(d.cnt, PR_ECAPACITY, 14u); continue; }
            d.c_key_alt[pos] = b;
            d.c_slot_alt[pos] = d.n_val[j];
        }
    }
}

__global__ void k_merge_done(DW d) {
    Counters* c = d.cnt;
    c->n_live = min(c->n_live + c->n_new, d.contact_cap);
    c->n_new = 0u;
    c->need_find = 0u;
}

__global__ void k_copy_u64u32(const uint64_t* ka, const uint32_t* va, uint64_t* kb, uint32_t* vb, const uint32_t* n) {
    GRID_LOOP(i, *n) {
        kb[i] = ka[i];
        vb[i] = va[i];
    }
}

// The tree is rebuilt from fresh Morton codes every kRebuildEvery searches and
// refitted in between: a refitted tree's node boxes still contain their leaves,
// so queries return exactly the same pairs, only the traversal may visit more
// nodes as bodies drift from their Morton order.
constexpr uint32_t kRebuildEvery = 8;

__global__ void k_set_lbvh_count(DW d, uint32_t* n_out) {
    Counters* c = d.cnt;
    if (!c->need_find) {
        c->lbvh_rebuild = 0u;
        *n_out = 0u;
        return;
    }
    const bool rebuild = (c->lbvh_age == 0u) || (c->lbvh_age >= kRebuildEvery);
    c->lbvh_rebuild = rebuild ? 1u : 0u;
    c->lbvh_age = rebuild ? 1u : c->lbvh_age + 1u;
    *n_out = rebuild ? d.n_shapes : 0u;
}

// Initial transforms from positions (device sin/cos), pos0 = pos1.
__global__ void k_init_bodies(DW d) {
    GRID_LOOP(b, d.n_bodies) {
        const float4 p = d.b_pos1[b];
        const float4 m = d.b_mass[b];
        const Xf x = get_xf(p.x, p.y, p.z, mk(m.z, m.w));
        d.b_xf[b] = make_float4(x.p.x, x.p.y, x.q.x, x.q.y);
        d.b_pos0[b] = p;
    }
}

}  // namespace

void launch_init_bodies(const DW& d, const Launch& L, cudaStream_t s) {
    k_init_bodies<<<L.grid, L.threads, 0, s>>>(d);
}

void launch_pre_proxies(const DW& d, const Launch& L, cudaStream_t s) {
    cudaMemsetAsync(&d.cnt->n_moved, 0, sizeof(uint32_t), s);
    k_pre_proxies<<<L.grid, L.threads, 0, s>>>(d);
    k_moved_done<<<1, 1, 0, s>>>(d);
}

void launch_synchronize(const DW& d, const Launch& L, cudaStream_t s) {
    cudaMemsetAsync(&d.cnt->n_moved, 0, sizeof(uint32_t), s);
    k_synchronize<<<L.grid, L.threads, 0, s>>>(d);
    k_moved_done<<<1, 1, 0, s>>>(d);
}

void launch_destroy_contacts(const DW& d, const Launch& L, cudaStream_t s) {
    k_destroy_flags<<<L.grid, L.threads, 0, s>>>(d);
    scan_exclusive(L.prims, d.flags, d.scan, &d.cnt->n_live, &d.cnt->scan_total, d.partial, s);
    k_destroy_scatter<<<L.grid, L.threads, 0, s>>>(d);
    k_destroy_done<<<1, 1, 0, s>>>(d);
    k_copy_live<<<L.grid, L.threads, 0, s>>>(d);
}

__global__ void k_set_upd_phase(DW d, uint32_t phase) { d.cnt->upd_phase = phase; }

void launch_set_upd_phase(const DW& d, uint32_t phase, cudaStream_t s) { k_set_upd_phase<<<1, 1, 0, s>>>(d, phase); }

void launch_update_contacts(const DW& d, const Launch& L, uint32_t body_mask, cudaStream_t s) {
    k_update_contacts<<<L.grid, kUpdThreads, 0, s>>>(d, body_mask);
    if (L.sensors) k_update_sensors<<<L.grid, L.threads, 0, s>>>(d, body_mask);
}

void launch_find_contacts(const DW& d, const Launch& L, cudaStream_t s) {
    // LBVH over all proxies (skipped on the device when nothing moved)
    uint32_t* n_lbvh = &d.cnt->pad[0];
    k_set_lbvh_count<<<1, 1, 0, s>>>(d, n_lbvh);
    k_lbvh_bounds_reset<<<L.grid, L.threads, 0, s>>>(d);
    k_lbvh_bounds<<<L.grid, L.threads, 0, s>>>(d);
    k_lbvh_morton<<<L.grid, L.threads, 0, s>>>(d);
    const bool alt = radix_sort(L.prims, d.l_key, d.l_key_alt, d.l_idx, d.l_idx_alt, n_lbvh, 30 + (int)d.world_bits,
                                d.hist, d.cnt, s);
    if (alt) k_copy_u64u32<<<L.grid, L.threads, 0, s>>>(d.l_key_alt, d.l_idx_alt, d.l_key, d.l_idx, n_lbvh);
    k_lbvh_internal<<<L.grid, L.threads, 0, s>>>(d);
    k_lbvh_leaves<<<L.grid, L.threads, 0, s>>>(d);
    k_lbvh_refit<<<L.grid, L.threads, 0, s>>>(d);
    k_lbvh_expand<<<L.grid, L.threads, 0, s>>>(d);
    k_lbvh_roots<<<L.grid, L.threads, 0, s>>>(d);
    k_contact_rows<<<L.grid, L.threads, 0, s>>>(d);
    // query moved proxies, filter, sort the new keys, create and merge
    k_find_pairs<<<L.grid * 2, 128, 0, s>>>(d);
    k_pairs_done<<<1, 1, 0, s>>>(d);
    const bool alt2 = radix_sort(L.prims, d.n_key, d.n_key_alt, d.n_val, d.n_val_alt, &d.cnt->n_new,
                                 2 * (int)d.key_bits, d.hist, d.cnt, s);
    if (alt2) k_copy_u64u32<<<L.grid, L.threads, 0, s>>>(d.n_key_alt, d.n_val_alt, d.n_key, d.n_val, &d.cnt->n_new);
    k_new_contacts<<<L.grid, L.threads, 0, s>>>(d);
    k_new_done<<<1, 1, 0, s>>>(d);
    k_merge<<<L.grid, L.threads, 0, s>>>(d);
    k_merge_done<<<1, 1, 0, s>>>(d);
    k_copy_live<<<L.grid, L.threads, 0, s>>>(d);
}

}  // namespace prgpu
