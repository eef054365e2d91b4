// prgpu_solver.cu -- islands, constraint colouring and the Gauss-Seidel solve.
//
// Restates SolveReg / SolveRegIslandViaGS (AabbTreeWorld.cpp:1472-1683) for a
// batch of worlds:
//  * islands are connected components over touching non-sensor contacts and
//    joints between speedable bodies (AddToIsland, :1358-1470), found by a
//    lock-free union-find; an island is solved when any body in it is awake;
//  * the sequential contact order of the reference becomes colour order: the
//    active contacts and joints are coloured so that no two constraints of a
//    colour share a dynamic body, and each colour is swept in parallel;
//  * the position loop keeps the reference's per-island early exit
//    (regMinSeparation, :1628-1644) through per-island, per-iteration minima;
//  * sleep follows UpdateUnderActiveTimes / Sleepem (:403-429).
// The velocity loop's early exit (regMinMomentum) only stops iterations that
// change nothing, so every island runs regVelocityIters sweeps.
//
// PRGPU_SOLVER_PART selects what a translation unit compiles, so that the
// k_world_solve instances (by far the longest to compile) build in parallel
// with the rest: 0 (this file) everything but k_world_solve; 1, 2 and 3
// (prgpu_solver_full.cu, prgpu_solver_lean.cu, prgpu_solver_tape.cu) the
// instance with joint and recording code, the one with neither, and the one
// that records but has no joint code, each with its launch helpers.
#ifndef PRGPU_SOLVER_PART
#define PRGPU_SOLVER_PART 0
#endif

#include <cooperative_groups.h>

#include <algorithm>
#include <mutex>

#include "prgpu_collide.cuh"
#include "prgpu_kernels.cuh"
#include "prgpu_csolve.cuh"
#include "prgpu_tape.cuh"

namespace prgpu {

namespace {

// ---- islands ----------------------------------------------------------------
__device__ __forceinline__ uint32_t uf_find(uint32_t* parent, uint32_t x) {
    for (int g = 0; g < 1 << 20; ++g) {
        const uint32_t p = __ldcg(&parent[x]);
        if (p == x) return x;
        x = p;
    }
    return x;
}

// The root of x for the unions, halving the path on the way (each node visited
// is pointed at its grandparent).  Only non-roots are written and a node stays a
// non-root once hooked, so these plain stores never meet the hooking CAS on a
// root; every value written is an ancestor in the same set (possibly a stale
// one), so any interleaving ends with the same sets, and, hooking larger roots
// under smaller ones, the same roots.  (The flattening pass writes each body's
// root and must not race with such stores: it uses uf_find.)
__device__ __forceinline__ uint32_t uf_find_halving(uint32_t* parent, uint32_t x) {
    for (int g = 0; g < 1 << 20; ++g) {
        const uint32_t p = __ldcg(&parent[x]);
        if (p == x) return x;
        const uint32_t gp = __ldcg(&parent[p]);
        if (gp == p) return p;
        __stcg(&parent[x], gp);
        x = gp;
    }
    return x;
}

__device__ __forceinline__ void uf_union(uint32_t* parent, uint32_t a, uint32_t b, Counters* c) {
    for (int g = 0; g < 1 << 16; ++g) {
        uint32_t ra = uf_find_halving(parent, a), rb = uf_find_halving(parent, b);
        if (ra == rb) return;
        if (ra < rb) { const uint32_t t = ra; ra = rb; rb = t; }
        // hook the larger root under the smaller one: labels end as component minima
        if (atomicCAS(&parent[ra], ra, rb) == ra) return;
    }
    set_error(c, PR_ETIMEOUT, 20u);
}

#if PRGPU_SOLVER_PART == 0
__global__ void k_isl_init(DW d) {
    GRID_LOOP(b, d.n_bodies) {
        d.b_island[b] = b;
        d.isl_awake[b] = 0u;
        d.b_flags[b] &= ~(BF_SOLVED | BF_MOVED);
    }
}

__device__ __forceinline__ bool island_edge_body(uint32_t f) { return is_speedable(f) && (f & BF_ENABLED); }

// The first index of the sorted live list whose key is >= key, by a warp: each
// round the 32 lanes probe 32 evenly spaced entries and the range shrinks to the
// gap where the keys cross.
__device__ __forceinline__ uint32_t live_lower_bound(const uint64_t* keys, uint32_t n, uint64_t key, uint32_t lane) {
    uint32_t lo = 0, hi = n;  // the answer lies in [lo, hi]
    while (hi - lo > 32u) {
        const uint32_t step = (hi - lo) / 32u;
        const bool less = keys[lo + (lane + 1u) * step - 1u] < key;
        const uint32_t k = __popc(__ballot_sync(0xffffffffu, less));
        const uint32_t nhi = (k < 32u) ? lo + (k + 1u) * step - 1u : hi;
        lo += k * step;
        hi = nhi;
    }
    const bool less = lo + lane < hi && keys[lo + lane] < key;
    return lo + __popc(__ballot_sync(0xffffffffu, less));
}

// Union-find in shared memory, with the rules of uf_find_halving / uf_union:
// only non-roots are rewritten, larger roots are hooked under smaller ones.
__device__ __forceinline__ uint32_t s_find(volatile uint32_t* p, uint32_t x) {
    for (int g = 0; g < 1 << 20; ++g) {
        const uint32_t q = p[x];
        if (q == x) return x;
        const uint32_t r = p[q];
        if (r == q) return q;
        p[x] = r;
        x = r;
    }
    return x;
}

__device__ __forceinline__ void s_union(uint32_t* p, uint32_t a, uint32_t b, Counters* c) {
    for (int g = 0; g < 1 << 16; ++g) {
        uint32_t ra = s_find(p, a), rb = s_find(p, b);
        if (ra == rb) return;
        if (ra < rb) { const uint32_t t = ra; ra = rb; rb = t; }
        if (atomicCAS(&p[ra], ra, rb) == ra) return;
    }
    set_error(c, PR_ETIMEOUT, 21u);
}

// Islands over contacts, one block a world of at most kIslSmemBodiesMax bodies.
// The live list is sorted by key and proxies are numbered world by world, so
// world w's contacts are the entries whose smaller proxy is one of its shapes:
// one range of the list.  The block unions them in shared memory and writes each
// body's root; the roots are component minima, as the global union leaves them,
// so the joints' unions (k_isl_union) and the flattening that follow see the same
// sets and labels.  Larger worlds are left to k_isl_union.


__global__ void __launch_bounds__(256) k_isl_world(DW d) {
    __shared__ uint32_t s_par[kIslSmemBodiesMax];
    __shared__ uint32_t s_rng[2];
    const uint32_t w = blockIdx.x;
    const uint32_t b0 = d.w_body_off[w], nb = d.w_body_off[w + 1] - b0;
    if (nb > kIslSmemBodiesMax) return;
    if (threadIdx.x < 64u) {  // warp 0 finds the world's first entry, warp 1 the next world's
        const uint32_t lane = threadIdx.x & 31u, which = threadIdx.x >> 5;
        const uint64_t key = (uint64_t)d.w_shape_off[w + which] << d.key_bits;
        const uint32_t at = live_lower_bound(d.c_key, d.cnt->n_live, key, lane);
        if (lane == 0) s_rng[which] = at;
    }
    for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) s_par[i] = i;
    __syncthreads();
    for (uint32_t i = s_rng[0] + threadIdx.x; i < s_rng[1]; i += blockDim.x) {
        const uint32_t slot = d.c_slot[i];
        if (!contact_solvable(d.cs_flags[slot])) continue;
        const uint2 bd = d.cs_body[slot];
        if (!(island_edge_body(d.b_flags[bd.x]) && island_edge_body(d.b_flags[bd.y]))) continue;
        if (bd.x - b0 >= nb || bd.y - b0 >= nb) {  // a contact of another world's bodies: not made
            set_error(d.cnt, PR_EINVAL, 22u);
            continue;
        }
        s_union(s_par, bd.x - b0, bd.y - b0, d.cnt);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) d.b_island[b0 + i] = b0 + s_find(s_par, i);
}

// Joints, and (big_worlds) the contacts of worlds above kIslSmemBodiesMax bodies,
// taken by slot (a free slot's flags are 0, never solvable): the union order
// does not change the components or their labels.
__global__ void k_isl_union(DW d, bool big_worlds) {
    const uint32_t hw = big_worlds ? d.cnt->high_water : 0u;
    GRID_LOOP(i, hw + d.n_joints) {
        uint32_t a, b;
        if (i < hw) {
            if (!contact_solvable(d.cs_flags[i])) continue;
            const uint2 bd = d.cs_body[i];
            a = bd.x; b = bd.y;
            const uint32_t w = d.b_world[a];
            if (d.w_body_off[w + 1] - d.w_body_off[w] <= kIslSmemBodiesMax) continue;  // done by k_isl_world
        } else {
            const uint32_t j = i - hw;
            a = d.j_bodies[2 * j]; b = d.j_bodies[2 * j + 1];
        }
        if (island_edge_body(d.b_flags[a]) && island_edge_body(d.b_flags[b])) uf_union(d.b_island, a, b, d.cnt);
    }
}

__global__ void k_isl_flatten(DW d) {
    GRID_LOOP(b, d.n_bodies) {
        const uint32_t r = uf_find(d.b_island, b);
        d.b_island[b] = r;
        const uint32_t f = d.b_flags[b];
        if (island_edge_body(f) && (f & BF_AWAKE)) d.isl_awake[r] = 1u;
    }
}

// pos0 <- pos1, GetBodyConstraint: Cap(GetVelocity(body, h)) (Body.cpp:290-309,
// Velocity.cpp:26-45), per-island state reset.
__global__ void k_body_begin(DW d) {
    const DConf& c = *d.conf;
    const float h = c.deltaTime;
    const int np = c.regPositionIters;
    uint32_t found = 0, solved = 0;
    GRID_LOOP(b, d.n_bodies) {
        const uint32_t f = d.b_flags[b];
        const uint32_t r = d.b_island[b];
        if (!island_edge_body(f) || !d.isl_awake[r]) continue;
        if (d.w_incomplete[d.b_world[b]]) continue;  // !IsStepComplete: no SolveReg (AabbTreeWorld.cpp:2206-2209)
        d.b_flags[b] = f | BF_SOLVED | BF_AWAKE;
        if (is_accelerable(f)) ++solved;
        const float4 p = d.b_pos1[b];
        d.b_pos0[b] = p;
        float4 v = d.b_vel[b];
        if (is_accelerable(f)) {
            const float4 a = d.b_acc[b];
            const float2 dm = d.b_damp[b];
            v.x = v.x + a.x * h;
            v.y = v.y + a.y * h;
            v.z = v.z + h * a.z;
            const float linv = 1.0f / (1.0f + h * dm.x);
            v.x = v.x * linv;
            v.y = v.y * linv;
            v.z = v.z / (1.0f + h * dm.y);
        }
        {
            const float tx = v.x * h, ty = v.y * h;
            float lsq = 0.f;
            lsq += tx * tx;
            lsq += ty * ty;
            if (lsq > c.maxTranslation * c.maxTranslation) {
                const float ratio = c.maxTranslation / sqrtf(lsq);
                v.x = v.x * ratio;
                v.y = v.y * ratio;
            }
            const float absRot = fabsf(h * v.z);
            if (absRot > c.maxRotation) {
                const float ratio = c.maxRotation / absRot;
                v.z = v.z * ratio;
            }
        }
        d.b_vel[b] = v;
        if (r == b) {
            ++found;
            for (int k = 0; k < np && k < kMaxPosIters; ++k) {
                d.isl_sep[(size_t)b * kMaxPosIters + k] = __int_as_float(0x7f800000);
                d.isl_jok[(size_t)b * kMaxPosIters + k] = 1u;
            }
            d.isl_uat[b] = __int_as_float(0x7f800000);
        }
    }
    if (found) atomicAdd(&d.cnt->st_islands_found, found);
    // body-steps: one per dynamic body of an awake island (warp sums, one atomic a warp)
    solved = __reduce_add_sync(0xffffffffu, solved);
    if ((threadIdx.x & 31u) == 0u && solved) {
        atomicAdd(&d.cnt->st_bodies_solved, solved);
        atomicAdd(reinterpret_cast<unsigned long long*>(&d.cnt->body_steps), (unsigned long long)solved);
    }
}
#endif

// ---- active constraints and colouring ---------------------------------------
#if PRGPU_SOLVER_PART == 0
__global__ void k_active_flags(DW d) {
    const uint32_t nl = d.cnt->n_live;
    GRID_LOOP(i, nl + d.n_joints) {
        uint32_t on = 0;
        if (i < nl) {
            const uint32_t slot = d.c_slot[i];
            if (contact_solvable(d.cs_flags[slot])) {
                const uint2 bd = d.cs_body[slot];
                on = ((d.b_flags[bd.x] | d.b_flags[bd.y]) & BF_SOLVED) ? 1u : 0u;
            }
        } else {
            const uint32_t j = i - nl;
            const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
            const uint32_t fa = d.b_flags[a], fb = d.b_flags[b];
            on = (((fa | fb) & BF_SOLVED) && (fa & BF_ENABLED) && (fb & BF_ENABLED)) ? 1u : 0u;
        }
        d.flags[i] = on;
    }
}

__global__ void k_active_scatter(DW d) {
    const uint32_t nl = d.cnt->n_live;
    GRID_LOOP(i, nl + d.n_joints) {
        if (!d.flags[i]) continue;
        const uint32_t k = d.scan[i];
        d.k_list[k] = (i < nl) ? d.c_slot[i] : ((i - nl) | kJointBit);
    }
}

__global__ void k_active_done(DW d, uint32_t* n_bodies_count) {
    Counters* c = d.cnt;
    c->n_active = c->scan_total;
    const uint32_t nl = c->n_live;
    c->n_active_c = nl ? d.scan[nl - 1] + d.flags[nl - 1] : 0u;
    c->n_colours = 0u;
    c->colour_remaining = 0u;
    for (int k = 0; k < kSerialColour + 2; ++k) { c->colour_cnt[k] = 0u; c->colour_off[k] = 0u; }
    *n_bodies_count = d.n_bodies;
}
#endif

__device__ __forceinline__ void constraint_bodies(const DW& d, uint32_t id, uint32_t& a, uint32_t& b) {
    if (id & kJointBit) {
        const uint32_t j = id & ~kJointBit;
        a = d.j_bodies[2 * j]; b = d.j_bodies[2 * j + 1];
    } else {
        const uint2 bd = d.cs_body[id];
        a = bd.x; b = bd.y;
    }
}

// Every body a constraint reads and writes: the two of a contact or joint, four
// of a gear joint (its own A and B, and the coupled joints' C and D), each once.
__device__ __forceinline__ int constraint_body_set(const DW& d, uint32_t id, uint32_t (&bs)[4]) {
    uint32_t a, b;
    constraint_bodies(d, id, a, b);
    int n = 0;
    bs[n++] = a;
    if (b != a) bs[n++] = b;
    if ((id & kJointBit) && ((d.j_flags[id & ~kJointBit] >> 8) & 0xffu) == 10u) {
        const float4 g0 = d.j_gear[5 * (id & ~kJointBit)];
        const uint32_t c = __float_as_uint(g0.x), e = __float_as_uint(g0.y);
        bool dup = false;
        for (int i = 0; i < n; ++i) dup |= (bs[i] == c);
        if (!dup) bs[n++] = c;
        dup = false;
        for (int i = 0; i < n; ++i) dup |= (bs[i] == e);
        if (!dup) bs[n++] = e;
    }
    return n;
}

#if PRGPU_SOLVER_PART == 0
// Colouring resources are the dynamic bodies: only they change under a constraint.
__global__ void k_inc_count(DW d) {
    GRID_LOOP(k, d.cnt->n_active) {
        uint32_t bs[4];
        const int n = constraint_body_set(d, d.k_list[k], bs);
        for (int e = 0; e < n; ++e)
            if (is_accelerable(d.b_flags[bs[e]])) atomicAdd(&d.inc_cur[bs[e]], 1u);
        d.k_colour[k] = kNone;
    }
}

__global__ void k_inc_fill(DW d) {
    GRID_LOOP(k, d.cnt->n_active) {
        uint32_t bs[4];
        const int n = constraint_body_set(d, d.k_list[k], bs);
        for (int e = 0; e < n; ++e)
            if (is_accelerable(d.b_flags[bs[e]])) d.inc_list[d.inc_off[bs[e]] + atomicAdd(&d.inc_cur[bs[e]], 1u)] = k;
    }
}
#endif

// Speculative greedy colouring (Gebremedhin-Manne style), deterministic:
// each round every uncoloured constraint picks the lowest colour unused by its
// coloured neighbours; among uncoloured neighbours with the same pick, the
// one of highest priority keeps it.  Rounds repeat until all are coloured; what is left
// after kMaxColourRounds, or needs a 65th colour, goes to the serial colour.
constexpr int kMaxColourRounds = 64;

// Conflict priority: a hash of the constraint index (ties broken by index).
// Index order alone follows the key order, which in stacked scenes is spatial,
// so conflicts would chain across a whole stack; hashed priorities resolve them
// in a logarithmic number of rounds and stay deterministic.
// The hash is of world-local identifiers (proxy pair of a contact, body pair of
// a joint), so a world is coloured the same whether it is stepped alone or in
// a batch; ties fall back to the constraint index, whose order within a world
// is also the same in both cases.
__device__ __forceinline__ bool colour_beats(const DW& d, uint32_t o, uint32_t k) {
    const uint32_t a = d.k_prio[o], b = d.k_prio[k];
    return (a < b) || (a == b && o < k);
}

__device__ __forceinline__ uint32_t constraint_prio(const DW& d, uint32_t id) {
    if (id & 0x80000000u) {
        const uint32_t j = id & 0x7fffffffu;
        const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
        const uint32_t base = d.w_body_off[d.b_world[a]];
        return prio_mix32(((a - base) * 0x9E3779B1u) ^ prio_mix32((b - base) + 0x7F4A7C15u) ^ 0xA5A5A5A5u);
    }
    return d.cs_prio[id];  // contact_prio of the slot's proxy pair, kept since its creation
}

__device__ __forceinline__ uint32_t colour_hint(const DW& d, uint32_t id) {
    return (id & kJointBit) ? d.j_colour[id & ~kJointBit] : d.cs_colour[id];
}

// Puts the serial colour's constraints in ascending index order, so their
// one-thread Gauss-Seidel order does not depend on scatter atomics.  The
// serial colour holds the few constraints the colouring gave up on.
__device__ void sort_serial(uint32_t* a, uint32_t n) {
    for (uint32_t i = 1; i < n; ++i) {
        const uint32_t v = a[i];
        uint32_t j = i;
        while (j > 0 && a[j - 1] > v) { a[j] = a[j - 1]; --j; }
        a[j] = v;
    }
}

// Two barriers per round.  Phase T (colour_pick): every uncoloured constraint
// picks a tentative colour from its neighbours' committed colours (in the first
// round the colour it had last step, if still free); constraints coloured
// earlier mark their tentative slot as settled.  Phase C (colour_keep): a
// constraint keeps its pick unless an uncoloured neighbour of higher priority
// picked the same colour, and commits it at once (phase C reads only tentative
// picks, never commits).  Each round depends only on the previous one, so the
// colouring is the same whether a world is coloured by the whole grid (k_colour)
// or by one CTA or warp of its own (k_world_solve).
constexpr uint32_t kSettled = 0xffffffffu;

__device__ __forceinline__ void colour_init(const DW& d, uint32_t k) {
    d.k_prio[k] = constraint_prio(d, d.k_list[k]);
    d.k_tent[k] = kSettled;
}

__device__ __forceinline__ void colour_pick(const DW& d, uint32_t k, int round) {
    const uint32_t ck = d.k_colour[k];
    if (ck != kNone) {
        if (d.k_tent[k] != kSettled) d.k_tent[k] = kSettled;
        return;
    }
    const uint32_t id = d.k_list[k];
    uint32_t bs[4];
    // In round 0 no constraint is committed yet (k_inc_count cleared them all),
    // so no colour is forbidden and the neighbours need not be read.
    const int nb = (round == 0) ? 0 : constraint_body_set(d, id, bs);
    uint64_t forbid = 0;
    for (int e = 0; e < nb; ++e) {
        const uint32_t x = bs[e];
        if (!is_accelerable(d.b_flags[x])) continue;
        for (uint32_t t = d.inc_off[x]; t < d.inc_off[x + 1]; ++t) {
            const uint32_t c = __ldcg(&d.k_colour[d.inc_list[t]]);
            if (c < (uint32_t)kMaxColours) forbid |= 1ull << c;
        }
    }
    uint32_t t;
    const uint32_t hint = (round == 0) ? colour_hint(d, id) : kNone;
    if (hint < (uint32_t)kMaxColours && !((forbid >> hint) & 1ull)) t = hint;
    else if (forbid == ~0ull) t = (uint32_t)kSerialColour;
    else t = (uint32_t)(__ffsll((long long)~forbid) - 1);
    if (t == (uint32_t)kSerialColour) { d.k_colour[k] = t; d.k_tent[k] = kSettled; }
    else d.k_tent[k] = t;
}

// Returns whether k is still uncoloured after this round.
__device__ __forceinline__ bool colour_keep(const DW& d, uint32_t k) {
    if (d.k_colour[k] != kNone) return false;
    const uint32_t t = __ldcg(&d.k_tent[k]);
    uint32_t bs[4];
    const int nb = constraint_body_set(d, d.k_list[k], bs);
    for (int e = 0; e < nb; ++e) {
        const uint32_t x = bs[e];
        if (!is_accelerable(d.b_flags[x])) continue;
        for (uint32_t q = d.inc_off[x]; q < d.inc_off[x + 1]; ++q) {
            const uint32_t o = d.inc_list[q];
            if (o != k && __ldcg(&d.k_tent[o]) == t && colour_beats(d, o, k)) return true;
        }
    }
    d.k_colour[k] = t;
    return false;
}

#if PRGPU_SOLVER_PART == 0
__global__ void k_colour(DW d) {
    const uint32_t n = d.cnt->n_active;
    uint32_t* rem = &d.cnt->pad[4];  // triple-buffered per-round counters
    GRID_LOOP(k, n) colour_init(d, k);
    if (blockIdx.x == 0 && threadIdx.x == 0) { rem[0] = 0u; rem[1] = 0u; rem[2] = 0u; }
    grid_barrier(d.cnt);
    for (int round = 0; round < kMaxColourRounds; ++round) {
        if (blockIdx.x == 0 && threadIdx.x == 0) rem[(round + 1) % 3] = 0u;
        GRID_LOOP(k, n) colour_pick(d, k, round);
        grid_barrier(d.cnt);
        uint32_t left = 0;
        GRID_LOOP(k, n) left += colour_keep(d, k) ? 1u : 0u;
        if (left) atomicAdd(&rem[round % 3], left);
        grid_barrier(d.cnt);
        if (*((volatile uint32_t*)&rem[round % 3]) == 0u) break;
    }
    GRID_LOOP(k, n) {
        if (d.k_colour[k] == kNone) d.k_colour[k] = (uint32_t)kSerialColour;
        atomicAdd(&d.cnt->colour_cnt[d.k_colour[k]], 1u);
    }
    grid_barrier(d.cnt);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        Counters* c = d.cnt;
        uint32_t off = 0, used = 0;
        for (int k = 0; k <= kSerialColour; ++k) {
            c->colour_off[k] = off;
            off += c->colour_cnt[k];
            if (k < kSerialColour && c->colour_cnt[k]) used = (uint32_t)k + 1u;
            c->colour_cnt[k] = 0u;  // reused as scatter cursors
        }
        c->colour_off[kSerialColour + 1] = off;
        c->n_colours = used;
    }
    grid_barrier(d.cnt);
    GRID_LOOP(k, n) {
        const uint32_t c = d.k_colour[k];
        d.k_order[d.cnt->colour_off[c] + atomicAdd(&d.cnt->colour_cnt[c], 1u)] = k;
        // remembered as next step's first choice
        const uint32_t id = d.k_list[k];
        const uint32_t keep = (c < (uint32_t)kMaxColours) ? c : kNone;
        if (id & kJointBit) d.j_colour[id & ~kJointBit] = keep;
        else d.cs_colour[id] = keep;
    }
    grid_barrier(d.cnt);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const uint32_t lo = d.cnt->colour_off[kSerialColour], hi = d.cnt->colour_off[kSerialColour + 1];
        if (hi > lo) sort_serial(d.k_order + lo, hi - lo);
    }
}
#endif

// ---- constraint construction --------------------------------------------------
// GetWorldManifold (WorldManifold.cpp:111-132), VelocityConstraint ctor +
// GetPoint + ComputeK (VelocityConstraint.cpp:38-185), PositionConstraint.
// ---- velocity constraint records -------------------------------------------------
__device__ __forceinline__ void store_vc(const DW& d, uint32_t t, const VC& v) {
    float4* r0 = d.vc0[t].q;
    r0[0] = make_float4(v.nx, v.ny, v.friction, v.tangentSpeed);
    r0[1] = make_float4(v.rA0x, v.rA0y, v.rB0x, v.rB0y);
    r0[2] = make_float4(v.nm0, v.tm0, v.vb0, __uint_as_float(v.count));
    r0[3] = make_float4(v.ni0, v.ti0, __uint_as_float(v.bA), __uint_as_float(v.bB));
    if (v.count == 2u) {
        float4* r1 = d.vc1[t].q;
        r1[0] = make_float4(v.rA1x, v.rA1y, v.rB1x, v.rB1y);
        r1[1] = make_float4(v.nm1, v.tm1, v.vb1, v.k00);
        r1[2] = make_float4(v.k11, v.k01, v.m00, v.m11);
        r1[3] = make_float4(v.ni1, v.ti1, v.m01, 0.f);
    }
}

__device__ __forceinline__ VC load_vc(const DW& d, uint32_t t) {
    const float4* r0 = d.vc0[t].q;
    const float4 a = r0[0], b = r0[1], c = r0[2], e = r0[3];
    VC v;
    v.nx = a.x; v.ny = a.y; v.friction = a.z; v.tangentSpeed = a.w;
    v.rA0x = b.x; v.rA0y = b.y; v.rB0x = b.z; v.rB0y = b.w;
    v.nm0 = c.x; v.tm0 = c.y; v.vb0 = c.z; v.count = __float_as_uint(c.w);
    v.ni0 = e.x; v.ti0 = e.y; v.bA = __float_as_uint(e.z); v.bB = __float_as_uint(e.w);
    v.island = 0u;
    if (v.count == 2u) {
        const float4* r1 = d.vc1[t].q;
        const float4 f = r1[0], g = r1[1], h = r1[2], i = r1[3];
        v.rA1x = f.x; v.rA1y = f.y; v.rB1x = f.z; v.rB1y = f.w;
        v.nm1 = g.x; v.tm1 = g.y; v.vb1 = g.z; v.k00 = g.w;
        v.k11 = h.x; v.k01 = h.y; v.m00 = h.z; v.m11 = h.w;
        v.ni1 = i.x; v.ti1 = i.y; v.m01 = i.z;
    } else {
        v.rA1x = v.rA1y = v.rB1x = v.rB1y = 0.f;
        v.nm1 = v.tm1 = v.vb1 = 0.f;
        v.k00 = v.k11 = v.k01 = v.m00 = v.m11 = v.m01 = 0.f;
        v.ni1 = v.ti1 = 0.f;
    }
    return v;
}

// Writes back the accumulated impulses of the constraint at t.
__device__ __forceinline__ void store_vc_impulses(const DW& d, uint32_t t, const VC& v) {
    reinterpret_cast<float2*>(d.vc0[t].q)[6] = make_float2(v.ni0, v.ti0);
    if (v.count == 2u) reinterpret_cast<float2*>(d.vc1[t].q)[6] = make_float2(v.ni1, v.ti1);
}

// Builds the constraint at sweep position t (vc0/vc1[t], pc[t]) for constraint k.
__device__ void build_constraint(const DW& d, uint32_t t, uint32_t k) {
    const DConf& c = *d.conf;
    const uint32_t id = d.k_list[k];
    d.t_id[t] = id;
    if (id & kJointBit) return;
    const uint32_t slot = id;
    const uint2 bd = d.cs_body[slot];
    const uint2 pr = d.cs_proxy[slot];
    const float rA = d.s_radius[pr.x], rB = d.s_radius[pr.y];
    const ManRec m = load_manrec(d, slot);
    VC vc = make_contact_vc(m, d.b_pos1[bd.x], d.b_pos1[bd.y], d.b_mass[bd.x], d.b_mass[bd.y], d.b_vel[bd.x],
                            d.b_vel[bd.y], rA, rB, d.cs_mat[slot], c.dtRatio, c, d.cs_tspeed[slot]);
    vc.bA = bd.x; vc.bB = bd.y;
    vc.island = is_speedable(d.b_flags[bd.x]) ? d.b_island[bd.x] : d.b_island[bd.y];
    store_vc(d, t, vc);
    PC pcs = make_contact_pc(m, rA + rB, bd.x, bd.y);
    pcs.island = vc.island;
    d.pc[t] = pcs;
}

#if PRGPU_SOLVER_PART == 0
// Constraints are stored in sweep order: position t of k_order.
__global__ void k_build_constraints(DW d) {
    GRID_LOOP(t, d.cnt->n_active) build_constraint(d, t, d.k_order[t]);
}
#endif

// Per-constraint solver steps: prgpu_csolve.cuh.

// ---- revolute joints (RevoluteJointConf.cpp:127-431) --------------------------
template <class BS>
__device__ void revolute_init_velocity(const DW& d, const BS& bs, uint32_t j) {
    const DConf& c = *d.conf;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    const float iMA = mA.x, iIA = mA.y, iMB = mB.x, iIB = mB.y;
    const float4 pA = bs.pos(a), pB = bs.pos(b);
    float4 vA = bs.vel(a), vB = bs.vel(b);
    const float4 an = d.j_anchor[j];
    const float4 prm = d.j_param[j];
    const uint32_t jf = d.j_flags[j];
    const V2 qA = unit_from_angle(pA.z), qB = unit_from_angle(pB.z);
    const V2 rA = rotate(mk(an.x, an.y) - mk(mA.z, mA.w), qA);
    const V2 rB = rotate(mk(an.z, an.w) - mk(mB.z, mB.w), qB);
    const float totInvI = iIA + iIB;
    const bool fixedRotation = (totInvI == 0.f);
    const float exx = iMA + ((rA.y * rA.y) * iIA) + iMB + ((rB.y * rB.y) * iIB);
    const float eyx = (-rA.y * rA.x * iIA) + (-rB.y * rB.x * iIB);
    const float ezx = (-rA.y * iIA) + (-rB.y * iIB);
    const float eyy = iMA + ((rA.x * rA.x) * iIA) + iMB + ((rB.x * rB.x) * iIB);
    const float ezy = (rA.x * iIA) + (rB.x * iIB);
    const float angularMass = (totInvI > 0.f) ? 1.0f / totInvI : 0.f;
    float4 imp = d.j_imp[j];  // x y z limitState
    float4 m1 = d.j_m1[j];    // ey.z ez.z angularMass motorImpulse
    float motorImpulse = m1.w;
    const bool enableMotor = (jf & 2u) != 0u, enableLimit = (jf & 1u) != 0u;
    if (!enableMotor || fixedRotation) motorImpulse = 0.f;
    int limitState = (int)imp.w;
    if (enableLimit && !fixedRotation) {
        const float jointAngle = pB.z - pA.z - prm.x;
        if (fabsf(prm.z - prm.y) < (c.angularSlop * 2.0f)) limitState = 3;
        else if (jointAngle <= prm.y) { if (limitState != 1) { limitState = 1; imp.z = 0.f; } }
        else if (jointAngle >= prm.z) { if (limitState != 2) { limitState = 2; imp.z = 0.f; } }
        else { limitState = 0; imp.z = 0.f; }
    } else {
        limitState = 0;
    }
    if (c.doWarmStart) {
        imp.x *= c.dtRatio; imp.y *= c.dtRatio; imp.z *= c.dtRatio;
        motorImpulse *= c.dtRatio;
        const V2 P = mk(imp.x, imp.y);
        const float L = motorImpulse + imp.z;
        const float LA = cross(rA, P) + L, LB = cross(rB, P) + L;
        vA.x = vA.x - P.x * iMA; vA.y = vA.y - P.y * iMA; vA.z = vA.z - iIA * LA;
        vB.x = vB.x + P.x * iMB; vB.y = vB.y + P.y * iMB; vB.z = vB.z + iIB * LB;
    } else {
        imp.x = imp.y = imp.z = 0.f;
        motorImpulse = 0.f;
    }
    imp.w = (float)limitState;
    d.j_imp[j] = imp;
    d.j_r[j] = make_float4(rA.x, rA.y, rB.x, rB.y);
    d.j_m0[j] = make_float4(exx, eyx, ezx, eyy);
    d.j_m1[j] = make_float4(ezy, totInvI, angularMass, motorImpulse);
    if (bs.writable(a)) bs.set_vel(a, vA);
    if (bs.writable(b)) bs.set_vel(b, vB);
}

template <class BS>
__device__ void revolute_solve_velocity(const DW& d, const BS& bs, uint32_t j) {
    const DConf& c = *d.conf;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    const float iMA = mA.x, iIA = mA.y, iMB = mB.x, iIB = mB.y;
    float4 vA = bs.vel(a), vB = bs.vel(b);
    const float4 r = d.j_r[j];
    const float4 m0 = d.j_m0[j];
    float4 m1 = d.j_m1[j];
    float4 imp = d.j_imp[j];
    const uint32_t jf = d.j_flags[j];
    const float4 prm = d.j_param[j];
    const V2 rA = mk(r.x, r.y), rB = mk(r.z, r.w);
    const bool fixedRotation = (iIA + iIB == 0.f);
    if ((jf & 2u) && ((int)imp.w != 3) && !fixedRotation) {
        const float impulse = -m1.z * (vB.z - vA.z - prm.w);
        const float oldImpulse = m1.w;
        const float maxImpulse = c.deltaTime * d.j_maxtorque[j];
        m1.w = clampf_(m1.w + impulse, -maxImpulse, maxImpulse);
        const float inc = m1.w - oldImpulse;
        vA.z -= iIA * inc;
        vB.z += iIB * inc;
    }
    const V2 vb = mk(vB.x, vB.y) + revperp(rB) * vB.z;
    const V2 va = mk(vA.x, vA.y) + revperp(rA) * vA.z;
    const V2 vd = vb - va;
    {
        // Solve22 (Math.hpp:462-474) on the upper 2x2 of the 3x3 mass
        const float xx = m0.x, xy = m0.y, yx = m0.y, yy = m0.w;
        const float cp = xx * yy - xy * yx;
        const float det = (cp != 0.f) ? (1.0f / cp) : cp;
        const V2 bb = -vd;
        const V2 P = mk(det * (yy * bb.x - xy * bb.y), det * (xx * bb.y - yx * bb.x));
        imp.x += P.x;
        imp.y += P.y;
        const float LA = cross(rA, P), LB = cross(rB, P);
        vA.x = vA.x - P.x * iMA; vA.y = vA.y - P.y * iMA; vA.z = vA.z - iIA * LA;
        vB.x = vB.x + P.x * iMB; vB.y = vB.y + P.y * iMB; vB.z = vB.z + iIB * LB;
    }
    d.j_imp[j] = imp;
    d.j_m1[j] = m1;
    if (bs.writable(a)) bs.set_vel(a, vA);
    if (bs.writable(b)) bs.set_vel(b, vB);
}

// Returns whether the joint is within tolerance.
template <class BS>
__device__ bool revolute_solve_position(const DW& d, const BS& bs, uint32_t j) {
    const DConf& c = *d.conf;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    const float iMA = mA.x, iIA = mA.y, iMB = mB.x, iIB = mB.y;
    float4 pA = bs.pos(a), pB = bs.pos(b);
    const float4 an = d.j_anchor[j];
    const V2 qA = unit_from_angle(pA.z), qB = unit_from_angle(pB.z);
    const V2 rA = rotate(mk(an.x, an.y) - mk(mA.z, mA.w), qA);
    const V2 rB = rotate(mk(an.z, an.w) - mk(mB.z, mB.w), qB);
    const V2 C = (mk(pB.x, pB.y) + rB) - (mk(pA.x, pA.y) + rA);
    const float positionError = mag2(C);
    const float exx = iMA + (iIA * (rA.y * rA.y)) + iMB + (iIB * (rB.y * rB.y));
    const float exy = (-iIA * rA.x * rA.y) + (-iIB * rB.x * rB.y);
    const float eyy = iMA + (iIA * (rA.x * rA.x)) + iMB + (iIB * (rB.x * rB.x));
    const float cp = cross(mk(exx, exy), mk(exy, eyy));
    V2 x = mk(0.f, 0.f);
    if (!almost_zero(cp)) {
        const float inv = 1.0f / cp;
        x = mk((eyy * C.x - exy * C.y) * inv, (exx * C.y - exy * C.x) * inv);
    }
    const V2 P = -x;
    pA.x = pA.x - P.x * iMA; pA.y = pA.y - P.y * iMA; pA.z = pA.z - iIA * cross(rA, P);
    pB.x = pB.x + P.x * iMB; pB.y = pB.y + P.y * iMB; pB.z = pB.z + iIB * cross(rB, P);
    if (bs.writable(a)) bs.set_pos(a, pA);
    if (bs.writable(b)) bs.set_pos(b, pB);
    return (positionError <= c.linearSlop * c.linearSlop) && (0.f <= c.angularSlop);
}

// ---- the other joint kinds (DistanceJointConf.cpp, RopeJointConf.cpp,
// WeldJointConf.cpp, FrictionJointConf.cpp, MotorJointConf.cpp) ----------------
// Solver state in j_m0 / j_m1 / j_imp by kind:
//   distance, rope: m0 = u.x u.y mass invGamma, m1 = bias length - -, imp.x
//   weld:           m0 = mass00 mass01 mass02 mass11, m1 = mass12 mass22 gamma bias, imp.xyz
//   friction:       m0 = linearMass00 01 11 angularMass, imp = linear xy, angular z
//   motor:          friction's, and m1 = linearError xy, angularError
//   prismatic:      r = axis perp, m0 = a1 a2 s1 s2, m1 = K11 K12 K13 K22,
//                   m2 = K23 K33 motorMass motorImpulse, imp.xyz, limitState
//   wheel:          r = ax ay, m0 = sAx sBx sAy sBy, m1 = mass springMass bias gamma,
//                   m2.x = angularMass, imp = impulse springImpulse angularImpulse
//   pulley:         r = rA rB, m0 = uA uB, m1.x = mass, imp.x
//   target:         r.zw = rB, m0 = mass22 (00 01 11) gamma, m1.xy = C, imp.xy
enum : uint32_t { JK_REVOLUTE = 0, JK_DISTANCE = 1, JK_ROPE = 2, JK_WELD = 3, JK_FRICTION = 4, JK_MOTOR = 5,
                  JK_PRISMATIC = 6, JK_WHEEL = 7, JK_PULLEY = 8, JK_TARGET = 9, JK_GEAR = 10 };
__device__ __forceinline__ uint32_t joint_kind(const DW& d, uint32_t j) { return (d.j_flags[j] >> 8) & 0xffu; }

// UnitVec::Get(x, y) (UnitVec.hpp:175-235): direction and magnitude.
__device__ __forceinline__ V2 unit_len(V2 v, float& len) {
    const float m2 = v.x * v.x + v.y * v.y;
    if (is_normal_f(m2)) {
        const float m = sqrtf(m2);
        const float inv = 1.0f / m;
        len = m;
        return mk(v.x * inv, v.y * inv);
    }
    const float m = hypotf(v.x, v.y);
    if (!is_normal_f(m)) { len = 0.f; return mk(0.f, 0.f); }
    len = m;
    return mk(v.x / m, v.y / m);
}
// Velocity / Position -= and += {invMass * P, invRotI * L}.
__device__ __forceinline__ void sub_imp(float4& s, float iM, V2 P, float iI, float L) {
    s.x = s.x - P.x * iM; s.y = s.y - P.y * iM; s.z = s.z - iI * L;
}
__device__ __forceinline__ void add_imp(float4& s, float iM, V2 P, float iI, float L) {
    s.x = s.x + P.x * iM; s.y = s.y + P.y * iM; s.z = s.z + iI * L;
}
__device__ __forceinline__ V2 point_vel(float4 v, V2 r) { return mk(v.x, v.y) + revperp(r) * v.z; }
__device__ __forceinline__ V2 anchor_r(V2 la, float4 m, float angle) {
    return rotate(la - mk(m.z, m.w), unit_from_angle(angle));
}
// Matrix * vector, rows accumulated from zero (Vector.hpp:455-470), for a
// symmetric 2x2 (a b; b c).
__device__ __forceinline__ V2 sym22_mul(float a, float b, float c, V2 v) {
    float x = 0.f; x += a * v.x; x += b * v.y;
    float y = 0.f; y += b * v.x; y += c * v.y;
    return mk(x, y);
}
__device__ __forceinline__ float dot3(const float* a, const float* b) {
    float r = 0.f; r += a[0] * b[0]; r += a[1] * b[1]; r += a[2] * b[2]; return r;
}
__device__ __forceinline__ void cross3(const float* a, const float* b, float* o) {
    const float x = a[1] * b[2] - a[2] * b[1], y = a[2] * b[0] - a[0] * b[2], z = a[0] * b[1] - a[1] * b[0];
    o[0] = x; o[1] = y; o[2] = z;
}
// GetMat33 of the weld joint (WeldJointConf.cpp:36-62); K[i] is the i-th Vec3.
__device__ __forceinline__ void weld_k(float iMA, V2 rA, float iIA, float iMB, V2 rB, float iIB, float K[3][3]) {
    const float exx = iMA + (rA.y * rA.y) * iIA + iMB + (rB.y * rB.y) * iIB;
    const float eyx = -rA.y * rA.x * iIA + -rB.y * rB.x * iIB;
    const float ezx = -rA.y * iIA + -rB.y * iIB;
    const float eyy = iMA + (rA.x * rA.x) * iIA + iMB + (rB.x * rB.x) * iIB;
    const float ezy = rA.x * iIA + rB.x * iIB;
    const float ezz = iIA + iIB;
    K[0][0] = exx; K[1][0] = eyx; K[2][0] = ezx;
    K[0][1] = eyx; K[1][1] = eyy; K[2][1] = ezy;
    K[0][2] = ezx; K[1][2] = ezy; K[2][2] = ezz;
}
// Solve22 / Solve33 (Math.hpp:447-475).
__device__ __forceinline__ V2 solve22k(const float K[3][3], V2 b) {
    const float xx = K[0][0], xy = K[1][0], yx = K[0][1], yy = K[1][1];
    const float cp = xx * yy - xy * yx;
    const float det = (cp != 0.f) ? (1.0f / cp) : cp;
    return mk(det * (yy * b.x - xy * b.y), det * (xx * b.y - yx * b.x));
}
__device__ __forceinline__ void solve33(const float K[3][3], const float* b, float* o) {
    float c[3], t[3];
    cross3(K[1], K[2], c);
    const float dp = dot3(K[0], c);
    const float det = (dp != 0.f) ? (1.0f / dp) : dp;
    const float x = det * dot3(b, c);
    cross3(b, K[2], t);
    const float y = det * dot3(K[0], t);
    cross3(K[1], b, t);
    const float z = det * dot3(K[0], t);
    o[0] = x; o[1] = y; o[2] = z;
}

template <class BS>
__device__ void distance_init_velocity(const DW& d, const BS& bs, uint32_t j, bool rope) {
    const DConf& c = *d.conf;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    const float4 pA = bs.pos(a), pB = bs.pos(b);
    float4 vA = bs.vel(a), vB = bs.vel(b);
    const float4 an = d.j_anchor[j], e = d.j_extra[2 * j];
    const V2 rA = anchor_r(mk(an.x, an.y), mA, pA.z), rB = anchor_r(mk(an.z, an.w), mB, pB.z);
    float length;
    V2 u = unit_len((mk(pB.x, pB.y) + rB) - (mk(pA.x, pA.y) + rA), length);
    float4 imp = d.j_imp[j];
    float jmass = 0.f, invGamma = 0.f, bias = 0.f;
    bool warm = c.doWarmStart != 0;
    if (rope) {
        // RopeJointConf InitVelocity (RopeJointConf.cpp:78-131)
        if (!(length > c.linearSlop)) {
            u = mk(0.f, 0.f);
            imp.x = 0.f;
            warm = false;
        } else {
            const float crA = cross(rA, u), crB = cross(rB, u);
            const float invMass = mA.x + mB.x + mA.y * (crA * crA) + mB.y * (crB * crB);
            jmass = (invMass != 0.f) ? 1.0f / invMass : 0.f;
        }
    } else {
        // DistanceJointConf InitVelocity (DistanceJointConf.cpp:79-146)
        const float crAu = cross(rA, u), crBu = cross(rB, u);
        float invMass = mA.x + mA.y * (crAu * crAu) + mB.x + mB.y * (crBu * crBu);
        jmass = (invMass != 0.f) ? 1.0f / invMass : 0.f;
        if (e.y > 0.f) {
            const float Pi = 3.14159265358979323846264338327950288f;
            const float C = length - e.x;
            const float omega = 2.0f * Pi * e.y;
            const float dd = 2.0f * jmass * e.z * omega;
            const float k = jmass * (omega * omega);
            const float h = c.deltaTime;
            const float gamma = h * (dd + h * k);
            invGamma = (gamma != 0.f) ? 1.0f / gamma : 0.f;
            bias = C * h * k * invGamma;
            invMass += invGamma;
            jmass = (invMass != 0.f) ? 1.0f / invMass : 0.f;
        }
    }
    if (warm) {
        imp.x *= c.dtRatio;
        const V2 P = u * imp.x;
        sub_imp(vA, mA.x, P, mA.y, cross(rA, P));
        add_imp(vB, mB.x, P, mB.y, cross(rB, P));
    } else if (!rope || length > c.linearSlop) {
        imp.x = 0.f;
    }
    d.j_imp[j] = imp;
    d.j_r[j] = make_float4(rA.x, rA.y, rB.x, rB.y);
    d.j_m0[j] = make_float4(u.x, u.y, jmass, invGamma);
    d.j_m1[j] = make_float4(bias, length, 0.f, 0.f);
    if (bs.writable(a)) bs.set_vel(a, vA);
    if (bs.writable(b)) bs.set_vel(b, vB);
}

template <class BS>
__device__ void distance_solve_velocity(const DW& d, const BS& bs, uint32_t j, bool rope) {
    const DConf& c = *d.conf;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    float4 vA = bs.vel(a), vB = bs.vel(b);
    const float4 r = d.j_r[j], m0 = d.j_m0[j], m1 = d.j_m1[j];
    float4 imp = d.j_imp[j];
    const V2 rA = mk(r.x, r.y), rB = mk(r.z, r.w), u = mk(m0.x, m0.y);
    V2 P;
    if (rope) {
        // RopeJointConf SolveVelocity (RopeJointConf.cpp:133-171)
        const float C = m1.y - d.j_extra[2 * j].x;
        const float inv_h = (c.deltaTime != 0.f) ? 1.0f / c.deltaTime : 0.f;
        const float Cdot = dot(u, point_vel(vB, rB) - point_vel(vA, rA)) + ((C < 0.f) ? inv_h * C : 0.f);
        float local = -m0.z * Cdot;
        const float old = imp.x;
        imp.x = minf_(0.f, imp.x + local);
        local = imp.x - old;
        P = u * local;
    } else {
        // DistanceJointConf SolveVelocity (DistanceJointConf.cpp:148-182)
        const float Cdot = dot(u, point_vel(vB, rB) - point_vel(vA, rA));
        const float impulse = -m0.z * (Cdot + m1.x + m0.w * imp.x);
        imp.x += impulse;
        P = u * impulse;
    }
    sub_imp(vA, mA.x, P, mA.y, cross(rA, P));
    add_imp(vB, mB.x, P, mB.y, cross(rB, P));
    d.j_imp[j] = imp;
    if (bs.writable(a)) bs.set_vel(a, vA);
    if (bs.writable(b)) bs.set_vel(b, vB);
}

template <class BS>
__device__ bool distance_solve_position(const DW& d, const BS& bs, uint32_t j, bool rope) {
    const DConf& c = *d.conf;
    const float4 e = d.j_extra[2 * j];
    if (!rope && e.y > 0.f) return true;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    float4 pA = bs.pos(a), pB = bs.pos(b);
    const float4 an = d.j_anchor[j];
    const V2 rA = anchor_r(mk(an.x, an.y), mA, pA.z), rB = anchor_r(mk(an.z, an.w), mB, pB.z);
    float length;
    const V2 u = unit_len((mk(pB.x, pB.y) + rB) - (mk(pA.x, pA.y) + rA), length);
    const float C = rope ? clampf_(length - e.x, 0.f, c.maxLinearCorrection)
                         : clampf_(length - e.x, -c.maxLinearCorrection, c.maxLinearCorrection);
    const float impulse = -d.j_m0[j].z * C;
    const V2 P = u * impulse;
    sub_imp(pA, mA.x, P, mA.y, cross(rA, P));
    add_imp(pB, mB.x, P, mB.y, cross(rB, P));
    if (bs.writable(a)) bs.set_pos(a, pA);
    if (bs.writable(b)) bs.set_pos(b, pB);
    return rope ? ((length - e.x) < c.linearSlop) : (fabsf(C) < c.linearSlop);
}

// WeldJointConf (WeldJointConf.cpp:133-376).
template <class BS>
__device__ void weld_init_velocity(const DW& d, const BS& bs, uint32_t j) {
    const DConf& c = *d.conf;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    const float iMA = mA.x, iIA = mA.y, iMB = mB.x, iIB = mB.y;
    const float4 pA = bs.pos(a), pB = bs.pos(b);
    float4 vA = bs.vel(a), vB = bs.vel(b);
    const float4 an = d.j_anchor[j], e = d.j_extra[2 * j];
    const V2 rA = anchor_r(mk(an.x, an.y), mA, pA.z), rB = anchor_r(mk(an.z, an.w), mB, pB.z);
    float K[3][3];
    weld_k(iMA, rA, iIA, iMB, rB, iIB, K);
    float m00, m01, m02 = 0.f, m11, m12 = 0.f, m22 = 0.f, gamma = 0.f, bias = 0.f;
    if (e.y > 0.f || K[2][2] == 0.f) {
        // GetInverse22 (Math.hpp:478-490)
        const float aa = K[0][0], bb = K[1][0], cc = K[0][1], dd = K[1][1];
        float det = (aa * dd) - (bb * cc);
        if (det != 0.f) det = 1.0f / det;
        m00 = det * dd; m01 = -det * cc; m11 = det * aa;
        if (e.y > 0.f) {
            float invRotInertia = iIA + iIB;
            const float rotInertia = (invRotInertia > 0.f) ? 1.0f / invRotInertia : 0.f;
            const float C = pB.z - pA.z - e.x;
            const float Pi = 3.14159265358979323846264338327950288f;
            const float omega = 2.0f * Pi * e.y;
            const float damp = 2.0f * rotInertia * e.z * omega;
            const float k = rotInertia * omega * omega;
            const float h = c.deltaTime;
            const float invGamma = h * (damp + h * k);
            gamma = (invGamma != 0.f) ? 1.0f / invGamma : 0.f;
            bias = C * h * k * gamma;
            invRotInertia += gamma;
            m22 = (invRotInertia != 0.f) ? 1.0f / invRotInertia : 0.f;
        }
    } else {
        // GetSymInverse33 (Math.hpp:493-512)
        float cr[3];
        cross3(K[1], K[2], cr);
        const float invDet = dot3(K[0], cr);
        const float det = (invDet != 0.f) ? (1.0f / invDet) : invDet;
        const float a11 = K[0][0], a12 = K[1][0], a13 = K[2][0], a22 = K[1][1], a23 = K[2][1], a33 = K[2][2];
        m01 = det * (a13 * a23 - a12 * a33);
        m12 = det * (a13 * a12 - a11 * a23);
        m02 = det * (a12 * a23 - a13 * a22);
        m00 = det * (a22 * a33 - a23 * a23);
        m11 = det * (a11 * a33 - a13 * a13);
        m22 = det * (a11 * a22 - a12 * a12);
    }
    float4 imp = d.j_imp[j];
    if (c.doWarmStart) {
        imp.x *= c.dtRatio; imp.y *= c.dtRatio; imp.z *= c.dtRatio;
        const V2 P = mk(imp.x, imp.y);
        const float L = imp.z;
        sub_imp(vA, iMA, P, iIA, L + cross(rA, P));
        add_imp(vB, iMB, P, iIB, L + cross(rB, P));
    } else {
        imp.x = imp.y = imp.z = 0.f;
    }
    d.j_imp[j] = imp;
    d.j_r[j] = make_float4(rA.x, rA.y, rB.x, rB.y);
    d.j_m0[j] = make_float4(m00, m01, m02, m11);
    d.j_m1[j] = make_float4(m12, m22, gamma, bias);
    if (bs.writable(a)) bs.set_vel(a, vA);
    if (bs.writable(b)) bs.set_vel(b, vB);
}

template <class BS>
__device__ void weld_solve_velocity(const DW& d, const BS& bs, uint32_t j) {
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    const float iMA = mA.x, iIA = mA.y, iMB = mB.x, iIB = mB.y;
    const float4 oA = bs.vel(a), oB = bs.vel(b);
    float4 vA = oA, vB = oB;
    const float4 r = d.j_r[j], m0 = d.j_m0[j], m1 = d.j_m1[j];
    const V2 rA = mk(r.x, r.y), rB = mk(r.z, r.w);
    float4 imp = d.j_imp[j];
    if (d.j_extra[2 * j].y > 0.f) {
        const float Cdot2 = vB.z - vA.z;
        const float gamma = m1.z * imp.z;
        const float impulse2 = -m1.y * (Cdot2 + m1.w + gamma);
        imp.z += impulse2;
        vA.z -= iIA * impulse2;
        vB.z += iIB * impulse2;
        const V2 Cdot1 = point_vel(vB, rB) - point_vel(vA, rA);
        // Transform(Vec2, Mat33) (Math.hpp:522-527)
        const V2 impulse1 = -mk(m0.x * Cdot1.x + m0.y * Cdot1.y, m0.y * Cdot1.x + m0.w * Cdot1.y);
        imp.x += impulse1.x;
        imp.y += impulse1.y;
        sub_imp(vA, iMA, impulse1, iIA, cross(rA, impulse1));
        add_imp(vB, iMB, impulse1, iIB, cross(rB, impulse1));
    } else {
        const V2 Cdot1 = point_vel(vB, rB) - point_vel(vA, rA);
        const float Cdot[3] = {Cdot1.x, Cdot1.y, vB.z - vA.z};
        const float row0[3] = {m0.x, m0.y, m0.z}, row1[3] = {m0.y, m0.w, m1.x}, row2[3] = {m0.z, m1.x, m1.y};
        const float ix = -dot3(row0, Cdot), iy = -dot3(row1, Cdot), iz = -dot3(row2, Cdot);
        imp.x += ix; imp.y += iy; imp.z += iz;
        const V2 P = mk(ix, iy);
        sub_imp(vA, iMA, P, iIA, iz + cross(rA, P));
        add_imp(vB, iMB, P, iIB, iz + cross(rB, P));
    }
    d.j_imp[j] = imp;
    if (bs.writable(a)) bs.set_vel(a, vA);
    if (bs.writable(b)) bs.set_vel(b, vB);
}

template <class BS>
__device__ bool weld_solve_position(const DW& d, const BS& bs, uint32_t j) {
    const DConf& c = *d.conf;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    const float iMA = mA.x, iIA = mA.y, iMB = mB.x, iIB = mB.y;
    float4 pA = bs.pos(a), pB = bs.pos(b);
    const float4 an = d.j_anchor[j], e = d.j_extra[2 * j];
    const V2 rA = anchor_r(mk(an.x, an.y), mA, pA.z), rB = anchor_r(mk(an.z, an.w), mB, pB.z);
    float K[3][3];
    weld_k(iMA, rA, iIA, iMB, rB, iIB, K);
    const V2 C1 = (mk(pB.x, pB.y) + rB) - (mk(pA.x, pA.y) + rA);
    const float positionError = sqrtf(mag2(C1));
    float angularError = 0.f;
    if (e.y > 0.f) {
        const V2 P = -solve22k(K, C1);
        sub_imp(pA, iMA, P, iIA, cross(rA, P));
        add_imp(pB, iMB, P, iIB, cross(rB, P));
    } else {
        const float C2 = pB.z - pA.z - e.x;
        angularError = fabsf(C2);
        const float Cv[3] = {C1.x, C1.y, C2};
        float im[3];
        if (K[2][2] > 0.f) {
            float s[3];
            solve33(K, Cv, s);
            im[0] = -s[0]; im[1] = -s[1]; im[2] = -s[2];
        } else {
            const V2 i2 = -solve22k(K, C1);
            im[0] = i2.x; im[1] = i2.y; im[2] = 0.f;
        }
        const V2 P = mk(im[0], im[1]);
        sub_imp(pA, iMA, P, iIA, im[2] + cross(rA, P));
        add_imp(pB, iMB, P, iIB, im[2] + cross(rB, P));
    }
    if (bs.writable(a)) bs.set_pos(a, pA);
    if (bs.writable(b)) bs.set_pos(b, pB);
    return (positionError <= c.linearSlop) && (angularError <= c.angularSlop);
}

// FrictionJointConf (FrictionJointConf.cpp:90-239) and MotorJointConf
// (MotorJointConf.cpp:89-235).
template <class BS>
__device__ void friction_init_velocity(const DW& d, const BS& bs, uint32_t j, bool motor) {
    const DConf& c = *d.conf;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    const float iMA = mA.x, iIA = mA.y, iMB = mB.x, iIB = mB.y;
    const float4 pA = bs.pos(a), pB = bs.pos(b);
    float4 vA = bs.vel(a), vB = bs.vel(b);
    const float4 an = d.j_anchor[j], e = d.j_extra[2 * j];
    V2 rA, rB;
    if (motor) {
        rA = rotate(mk(e.x, e.y) - mk(mA.z, mA.w), unit_from_angle(pA.z));
        rB = rotate(-mk(mB.z, mB.w), unit_from_angle(pB.z));
    } else {
        rA = anchor_r(mk(an.x, an.y), mA, pA.z);
        rB = anchor_r(mk(an.z, an.w), mB, pB.z);
    }
    float exx, exy, eyy;
    if (motor) {
        exx = iMA + iMB + iIA * (rA.y * rA.y) + iIB * (rB.y * rB.y);
        eyy = iMA + iMB + iIA * (rA.x * rA.x) + iIB * (rB.x * rB.x);
    } else {
        exx = iMA + iIA * (rA.y * rA.y) + iMB + iIB * (rB.y * rB.y);
        eyy = iMA + iIA * (rA.x * rA.x) + iMB + iIB * (rB.x * rB.x);
    }
    exy = -iIA * rA.x * rA.y + -iIB * rB.x * rB.y;
    // Invert(Matrix22) (Math.hpp:430-442)
    float l00 = 0.f, l01 = 0.f, l11 = 0.f;
    {
        const float cp = cross(mk(exx, exy), mk(exy, eyy));
        if (!almost_zero(cp)) {
            const float inv = 1.0f / cp;
            l00 = eyy * inv; l01 = -exy * inv; l11 = exx * inv;
        }
    }
    const float invRotInertia = iIA + iIB;
    const float angularMass = (invRotInertia > 0.f) ? 1.0f / invRotInertia : 0.f;
    float4 imp = d.j_imp[j];
    if (c.doWarmStart) {
        imp.x *= c.dtRatio; imp.y *= c.dtRatio; imp.z *= c.dtRatio;
        const V2 P = mk(imp.x, imp.y);
        sub_imp(vA, iMA, P, iIA, cross(rA, P) + imp.z);
        add_imp(vB, iMB, P, iIB, cross(rB, P) + imp.z);
    } else {
        imp.x = imp.y = imp.z = 0.f;
    }
    d.j_imp[j] = imp;
    d.j_r[j] = make_float4(rA.x, rA.y, rB.x, rB.y);
    d.j_m0[j] = make_float4(l00, l01, l11, angularMass);
    if (motor) {
        const V2 le = (mk(pB.x, pB.y) + rB) - (mk(pA.x, pA.y) + rA);
        d.j_m1[j] = make_float4(le.x, le.y, (pB.z - pA.z) - e.z, 0.f);
    }
    if (bs.writable(a)) bs.set_vel(a, vA);
    if (bs.writable(b)) bs.set_vel(b, vB);
}

template <class BS>
__device__ void friction_solve_velocity(const DW& d, const BS& bs, uint32_t j, bool motor) {
    const DConf& c = *d.conf;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    const float iMA = mA.x, iIA = mA.y, iMB = mB.x, iIB = mB.y;
    float4 vA = bs.vel(a), vB = bs.vel(b);
    const float4 r = d.j_r[j], m0 = d.j_m0[j], e0 = d.j_extra[2 * j], e1 = d.j_extra[2 * j + 1];
    const V2 rA = mk(r.x, r.y), rB = mk(r.z, r.w);
    float4 imp = d.j_imp[j];
    const float h = c.deltaTime;
    const float inv_h = (h != 0.f) ? 1.0f / h : 0.f;
    const float maxForce = motor ? e0.w : e0.x, maxTorque = motor ? e1.x : e0.y, cf = e1.y;
    const float4 err = motor ? d.j_m1[j] : make_float4(0.f, 0.f, 0.f, 0.f);
    {
        const float Cdot = motor ? (vB.z - vA.z) + inv_h * cf * err.z : (vB.z - vA.z);
        const float angularImpulse = -m0.w * Cdot;
        const float old = imp.z;
        const float maxAng = h * maxTorque;
        imp.z = clampf_(old + angularImpulse, -maxAng, maxAng);
        const float inc = imp.z - old;
        if (!motor || inc != 0.f) {
            vA.z -= iIA * inc;
            vB.z += iIB * inc;
        }
    }
    {
        V2 Cdot = point_vel(vB, rB) - point_vel(vA, rA);
        if (motor) Cdot = Cdot + mk(err.x, err.y) * (inv_h * cf);
        const V2 impulse = -sym22_mul(m0.x, m0.y, m0.z, Cdot);
        const V2 old = mk(imp.x, imp.y);
        V2 li = old + impulse;
        const float maxImpulse = h * maxForce;
        if (mag2(li) > maxImpulse * maxImpulse) li = unit_vector(li, mk(0.f, 0.f)) * maxImpulse;
        imp.x = li.x; imp.y = li.y;
        const V2 inc = li - old;
        const float angA = cross(rA, inc), angB = cross(rB, inc);
        if (!motor || inc.x != 0.f || inc.y != 0.f || angA != 0.f || angB != 0.f) {
            sub_imp(vA, iMA, inc, iIA, angA);
            add_imp(vB, iMB, inc, iIB, angB);
        }
    }
    d.j_imp[j] = imp;
    if (bs.writable(a)) bs.set_vel(a, vA);
    if (bs.writable(b)) bs.set_vel(b, vB);
}

// Whether a velocity or position changed (Velocity / Position operator!=).
__device__ __forceinline__ bool state_ne(float4 a, float4 b) { return !(a.x == b.x && a.y == b.y && a.z == b.z); }

// PrismaticJointConf (PrismaticJointConf.cpp:95-449); extra = localXAxisA.xy
// referenceAngle lowerTranslation upperTranslation motorSpeed maxMotorForce.
template <class BS>
__device__ void prismatic_init_velocity(const DW& d, const BS& bs, uint32_t j) {
    const DConf& c = *d.conf;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    const float iMA = mA.x, iIA = mA.y, iMB = mB.x, iIB = mB.y;
    const float4 pA = bs.pos(a), pB = bs.pos(b);
    float4 vA = bs.vel(a), vB = bs.vel(b);
    const float4 an = d.j_anchor[j], e0 = d.j_extra[2 * j], e1 = d.j_extra[2 * j + 1];
    const uint32_t jf = d.j_flags[j];
    const V2 qA = unit_from_angle(pA.z);
    const V2 rA = anchor_r(mk(an.x, an.y), mA, pA.z), rB = anchor_r(mk(an.z, an.w), mB, pB.z);
    const V2 dd = ((mk(pB.x, pB.y) - mk(pA.x, pA.y)) + rB) - rA;
    const V2 xaxis = mk(e0.x, e0.y);
    const V2 axis = urotate(xaxis, qA);
    const float a1 = cross(dd + rA, axis), a2 = cross(rB, axis);
    const float invRotMassA = iIA * (a1 * a1), invRotMassB = iIB * (a2 * a2);
    const float totalInvMass = iMA + iMB + invRotMassA + invRotMassB;
    const float motorMass = (totalInvMass > 0.f) ? 1.0f / totalInvMass : 0.f;
    const V2 perp = urotate(revperp(xaxis), qA);
    const float s1 = cross(dd + rA, perp), s2 = cross(rB, perp);
    const float invRotMassA2 = iIA * (s1 * s1), invRotMassB2 = iIB * (s2 * s2);
    const float k11 = iMA + iMB + invRotMassA2 + invRotMassB2;
    const float k12 = iIA * s1 + iIB * s2;
    const float k13 = iIA * s1 * a1 + iIB * s2 * a2;
    const float totalInvRotInertia = iIA + iIB;
    const float k22 = (totalInvRotInertia == 0.f) ? 1.0f : totalInvRotInertia;
    const float k23 = iIA * a1 + iIB * a2;
    const float k33 = totalInvMass;
    float4 imp = d.j_imp[j];
    float motorImpulse = d.j_m2[j].w;
    int limitState = (int)imp.w;
    const float lower = e0.w, upper = e1.x;
    if (jf & 1u) {
        const float jointTranslation = dot(axis, dd);
        if (fabsf(upper - lower) < (c.linearSlop * 2.0f)) limitState = 3;
        else if (jointTranslation <= lower) { if (limitState != 1) { limitState = 1; imp.z = 0.f; } }
        else if (jointTranslation >= upper) { if (limitState != 2) { limitState = 2; imp.z = 0.f; } }
        else { limitState = 0; imp.z = 0.f; }
    } else {
        limitState = 0;
        imp.z = 0.f;
    }
    if (!(jf & 2u)) motorImpulse = 0.f;
    if (c.doWarmStart) {
        imp.x *= c.dtRatio; imp.y *= c.dtRatio; imp.z *= c.dtRatio;
        motorImpulse *= c.dtRatio;
        const V2 Px = perp * imp.x;
        const float Pxs1 = imp.x * s1, Pxs2 = imp.x * s2;
        const float PzLength = motorImpulse + imp.z;
        const V2 P = Px + axis * PzLength;
        const float L = imp.y;
        const float LA = L + (Pxs1 + PzLength * a1);
        const float LB = L + (Pxs2 + PzLength * a2);
        sub_imp(vA, iMA, P, iIA, LA);
        add_imp(vB, iMB, P, iIB, LB);
    } else {
        imp.x = imp.y = imp.z = 0.f;
        motorImpulse = 0.f;
    }
    imp.w = (float)limitState;
    d.j_imp[j] = imp;
    d.j_r[j] = make_float4(axis.x, axis.y, perp.x, perp.y);
    d.j_m0[j] = make_float4(a1, a2, s1, s2);
    d.j_m1[j] = make_float4(k11, k12, k13, k22);
    d.j_m2[j] = make_float4(k23, k33, motorMass, motorImpulse);
    if (bs.writable(a)) bs.set_vel(a, vA);
    if (bs.writable(b)) bs.set_vel(b, vB);
}

template <class BS>
__device__ void prismatic_solve_velocity(const DW& d, const BS& bs, uint32_t j) {
    const DConf& c = *d.conf;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    const float iMA = mA.x, iIA = mA.y, iMB = mB.x, iIB = mB.y;
    const float4 oldA = bs.vel(a), oldB = bs.vel(b);
    float4 vA = oldA, vB = oldB;
    const float4 r = d.j_r[j], m0 = d.j_m0[j], m1 = d.j_m1[j], e1 = d.j_extra[2 * j + 1];
    float4 m2 = d.j_m2[j];
    float4 imp = d.j_imp[j];
    const uint32_t jf = d.j_flags[j];
    const int limitState = (int)imp.w;
    const V2 axis = mk(r.x, r.y), perp = mk(r.z, r.w);
    const float a1 = m0.x, a2 = m0.y, s1 = m0.z, s2 = m0.w;
    if ((jf & 2u) && limitState != 3) {
        const float vDot = dot(axis, mk(vB.x, vB.y) - mk(vA.x, vA.y));
        const float Cdot = vDot + (a2 * vB.z - a1 * vA.z);
        float impulse = m2.z * (e1.y - Cdot);
        const float oldImpulse = m2.w;
        const float maxImpulse = c.deltaTime * e1.z;
        m2.w = clampf_(m2.w + impulse, -maxImpulse, maxImpulse);
        impulse = m2.w - oldImpulse;
        const V2 P = axis * impulse;
        sub_imp(vA, iMA, P, iIA, impulse * a1);
        add_imp(vB, iMB, P, iIB, impulse * a2);
        d.j_m2[j] = m2;
    }
    float K[3][3] = {{m1.x, m1.y, m1.z}, {m1.y, m1.w, m2.x}, {m1.z, m2.x, m2.y}};
    const V2 velDelta = mk(vB.x, vB.y) - mk(vA.x, vA.y);
    const float sRotSpeed = s2 * vB.z - s1 * vA.z;
    const V2 Cdot1 = mk(dot(perp, velDelta) + sRotSpeed, vB.z - vA.z);
    if ((jf & 1u) && limitState != 0) {
        const float deltaDot = dot(axis, velDelta);
        const float aRotSpeed = a2 * vB.z - a1 * vA.z;
        const float Cdot2 = deltaDot + aRotSpeed;
        const float negCdot[3] = {-Cdot1.x, -Cdot1.y, -Cdot2};
        const float4 f1 = imp;
        float add[3];
        solve33(K, negCdot, add);
        imp.x += add[0]; imp.y += add[1]; imp.z += add[2];
        if (limitState == 1) imp.z = maxf_(imp.z, 0.f);
        else if (limitState == 2) imp.z = minf_(imp.z, 0.f);
        const float dz = imp.z - f1.z;
        const V2 bb = mk(-Cdot1.x - dz * K[2][0], -Cdot1.y - dz * K[2][1]);
        const V2 s22 = solve22k(K, bb);
        imp.x = s22.x + f1.x; imp.y = s22.y + f1.y;
        const float dx = imp.x - f1.x, dy = imp.y - f1.y, dzz = imp.z - f1.z;
        const V2 P = perp * dx + axis * dzz;
        const float LA = dx * s1 + dy + dzz * a1;
        const float LB = dx * s2 + dy + dzz * a2;
        sub_imp(vA, iMA, P, iIA, LA);
        add_imp(vB, iMB, P, iIB, LB);
    } else {
        const V2 df = solve22k(K, -Cdot1);
        imp.x += df.x; imp.y += df.y;
        const V2 P = perp * df.x;
        sub_imp(vA, iMA, P, iIA, df.x * s1 + df.y);
        add_imp(vB, iMB, P, iIB, df.x * s2 + df.y);
    }
    d.j_imp[j] = imp;
    if (state_ne(vA, oldA) || state_ne(vB, oldB)) {
        if (bs.writable(a)) bs.set_vel(a, vA);
        if (bs.writable(b)) bs.set_vel(b, vB);
    }
}

template <class BS>
__device__ bool prismatic_solve_position(const DW& d, const BS& bs, uint32_t j) {
    const DConf& c = *d.conf;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    const float iMA = mA.x, iIA = mA.y, iMB = mB.x, iIB = mB.y;
    float4 pA = bs.pos(a), pB = bs.pos(b);
    const float4 an = d.j_anchor[j], e0 = d.j_extra[2 * j], e1 = d.j_extra[2 * j + 1];
    const V2 qA = unit_from_angle(pA.z);
    const V2 rA = anchor_r(mk(an.x, an.y), mA, pA.z), rB = anchor_r(mk(an.z, an.w), mB, pB.z);
    const V2 dd = (mk(pB.x, pB.y) + rB) - (mk(pA.x, pA.y) + rA);
    const V2 xaxis = mk(e0.x, e0.y);
    const V2 axis = urotate(xaxis, qA);
    const float a1 = cross(dd + rA, axis), a2 = cross(rB, axis);
    const V2 perp = urotate(revperp(xaxis), qA);
    const float s1 = cross(dd + rA, perp), s2 = cross(rB, perp);
    const V2 C1 = mk(dot(perp, dd), pB.z - pA.z - e0.z);
    float linearError = fabsf(C1.x);
    const float angularError = fabsf(C1.y);
    bool active = false;
    float C2 = 0.f;
    const float lower = e0.w, upper = e1.x;
    if (d.j_flags[j] & 1u) {
        const float translation = dot(axis, dd);
        if (fabsf(upper - lower) < (2.0f * c.linearSlop)) {
            C2 = clampf_(translation, -c.maxLinearCorrection, c.maxLinearCorrection);
            linearError = maxf_(linearError, fabsf(translation));
            active = true;
        } else if (translation <= lower) {
            C2 = clampf_(translation - lower + c.linearSlop, -c.maxLinearCorrection, 0.f);
            linearError = maxf_(linearError, lower - translation);
            active = true;
        } else if (translation >= upper) {
            C2 = clampf_(translation - upper - c.linearSlop, 0.f, c.maxLinearCorrection);
            linearError = maxf_(linearError, translation - upper);
            active = true;
        }
    }
    float impulse[3];
    if (active) {
        const float k11 = iMA + iIA * (s1 * s1) + iMB + iIB * (s2 * s2);
        const float k12 = iIA * s1 + iIB * s2;
        const float k13 = iIA * s1 * a1 + iIB * s2 * a2;
        float k22 = iIA + iIB;
        if (k22 == 0.f) k22 = 1.0f;
        const float k23 = iIA * a1 + iIB * a2;
        const float k33 = iMA + iIA * (a1 * a1) + iMB + iIB * (a2 * a2);
        const float K[3][3] = {{k11, k12, k13}, {k12, k22, k23}, {k13, k23, k33}};
        const float negC[3] = {-C1.x, -C1.y, -C2};
        solve33(K, negC, impulse);
    } else {
        const float k11 = iMA + iIA * s1 * s1 + iMB + iIB * s2 * s2;
        const float k12 = iIA * s1 + iIB * s2;
        float k22 = iIA + iIB;
        if (k22 == 0.f) k22 = 1.0f;
        // Solve(Matrix22, Vector2) (Math.hpp:412-425)
        const V2 bneg = -C1;
        const float cp = cross(mk(k11, k12), mk(k12, k22));
        impulse[0] = impulse[1] = impulse[2] = 0.f;
        if (!almost_zero(cp)) {
            const float inverse = 1.0f / cp;
            impulse[0] = (k22 * bneg.x - k12 * bneg.y) * inverse;
            impulse[1] = (k11 * bneg.y - k12 * bneg.x) * inverse;
        }
    }
    const V2 P = perp * impulse[0] + axis * impulse[2];
    const float LA = impulse[0] * s1 + impulse[1] + impulse[2] * a1;
    const float LB = impulse[0] * s2 + impulse[1] + impulse[2] * a2;
    sub_imp(pA, iMA, P, iIA, LA);
    add_imp(pB, iMB, P, iIB, LB);
    if (bs.writable(a)) bs.set_pos(a, pA);
    if (bs.writable(b)) bs.set_pos(b, pB);
    return (linearError <= c.linearSlop) && (angularError <= c.angularSlop);
}

// WheelJointConf (WheelJointConf.cpp:80-311); extra = localXAxisA.xy motorSpeed
// maxMotorTorque frequency dampingRatio.
template <class BS>
__device__ void wheel_init_velocity(const DW& d, const BS& bs, uint32_t j) {
    const DConf& c = *d.conf;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    const float iMA = mA.x, iIA = mA.y, iMB = mB.x, iIB = mB.y;
    const float4 pA = bs.pos(a), pB = bs.pos(b);
    float4 vA = bs.vel(a), vB = bs.vel(b);
    const float4 an = d.j_anchor[j], e0 = d.j_extra[2 * j], e1 = d.j_extra[2 * j + 1];
    const V2 qA = unit_from_angle(pA.z);
    const V2 rA = anchor_r(mk(an.x, an.y), mA, pA.z), rB = anchor_r(mk(an.z, an.w), mB, pB.z);
    const V2 dd = (mk(pB.x, pB.y) + rB) - (mk(pA.x, pA.y) + rA);
    const V2 xaxis = mk(e0.x, e0.y);
    const V2 ay = urotate(revperp(xaxis), qA);
    const float sAy = cross(dd + rA, ay), sBy = cross(rB, ay);
    float mass;
    {
        const float invMass = iMA + iMB + iIA * (sAy * sAy) + iIB * (sBy * sBy);
        mass = (invMass > 0.f) ? 1.0f / invMass : 0.f;
    }
    float4 imp = d.j_imp[j];  // impulse springImpulse angularImpulse
    float springMass = 0.f, bias = 0.f, gamma = 0.f;
    V2 ax = mk(0.f, 0.f);
    float sAx = 0.f, sBx = 0.f;
    const float frequency = e1.x, dampingRatio = e1.y;
    if (frequency > 0.f) {
        ax = urotate(xaxis, qA);
        sAx = cross(dd + rA, ax);
        sBx = cross(rB, ax);
        const float invMass = iMA + iMB + iIA * (sAx * sAx) + iIB * (sBx * sBx);
        if (invMass > 0.f) {
            springMass = 1.0f / invMass;
            const float C = dot(dd, ax);
            const float Pi = 3.14159265358979323846264338327950288f;
            const float omega = 2.0f * Pi * frequency;
            const float dc = 2.0f * springMass * dampingRatio * omega;
            const float k = springMass * omega * omega;
            const float h = c.deltaTime;
            const float invGamma = h * (dc + h * k);
            gamma = (invGamma > 0.f) ? 1.0f / invGamma : 0.f;
            bias = C * h * k * gamma;
            const float totalInvMass = invMass + gamma;
            springMass = (totalInvMass > 0.f) ? 1.0f / totalInvMass : 0.f;
        }
    } else {
        imp.y = 0.f;
    }
    float angularMass = 0.f;
    if (d.j_flags[j] & 2u) {
        const float invRotInertia = iIA + iIB;
        angularMass = (invRotInertia > 0.f) ? 1.0f / invRotInertia : 0.f;
    } else {
        imp.z = 0.f;
    }
    if (c.doWarmStart) {
        imp.x *= c.dtRatio; imp.y *= c.dtRatio; imp.z *= c.dtRatio;
        const V2 P = ay * imp.x + ax * imp.y;
        const float LA = (imp.x * sAy + imp.y * sAx) + imp.z;
        const float LB = (imp.x * sBy + imp.y * sBx) + imp.z;
        sub_imp(vA, iMA, P, iIA, LA);
        add_imp(vB, iMB, P, iIB, LB);
    } else {
        imp.x = imp.y = imp.z = 0.f;
    }
    d.j_imp[j] = imp;
    d.j_r[j] = make_float4(ax.x, ax.y, ay.x, ay.y);
    d.j_m0[j] = make_float4(sAx, sBx, sAy, sBy);
    d.j_m1[j] = make_float4(mass, springMass, bias, gamma);
    d.j_m2[j] = make_float4(angularMass, 0.f, 0.f, 0.f);
    if (bs.writable(a)) bs.set_vel(a, vA);
    if (bs.writable(b)) bs.set_vel(b, vB);
}

template <class BS>
__device__ void wheel_solve_velocity(const DW& d, const BS& bs, uint32_t j) {
    const DConf& c = *d.conf;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    const float iMA = mA.x, iIA = mA.y, iMB = mB.x, iIB = mB.y;
    const float4 oldA = bs.vel(a), oldB = bs.vel(b);
    float4 vA = oldA, vB = oldB;
    const float4 r = d.j_r[j], m0 = d.j_m0[j], m1 = d.j_m1[j], e0 = d.j_extra[2 * j];
    const float angularMass = d.j_m2[j].x;
    float4 imp = d.j_imp[j];
    const V2 ax = mk(r.x, r.y), ay = mk(r.z, r.w);
    const float sAx = m0.x, sBx = m0.y, sAy = m0.z, sBy = m0.w;
    {
        const float dv = dot(ax, mk(vB.x, vB.y) - mk(vA.x, vA.y));
        const float Cdot = dv + sBx * vB.z - sAx * vA.z;
        const float impulse = -m1.y * (Cdot + m1.z + m1.w * imp.y);
        imp.y += impulse;
        const V2 P = ax * impulse;
        sub_imp(vA, iMA, P, iIA, impulse * sAx);
        add_imp(vB, iMB, P, iIB, impulse * sBx);
    }
    {
        const float Cdot = vB.z - vA.z - e0.z;
        float impulse = -angularMass * Cdot;
        const float oldImpulse = imp.z;
        const float maxImpulse = c.deltaTime * e0.w;
        imp.z = clampf_(imp.z + impulse, -maxImpulse, maxImpulse);
        impulse = imp.z - oldImpulse;
        vA.z -= iIA * impulse;
        vB.z += iIB * impulse;
    }
    {
        const float dv = dot(ay, mk(vB.x, vB.y) - mk(vA.x, vA.y));
        const float Cdot = dv + sBy * vB.z - sAy * vA.z;
        const float impulse = -m1.x * Cdot;
        imp.x += impulse;
        const V2 P = ay * impulse;
        sub_imp(vA, iMA, P, iIA, impulse * sAy);
        add_imp(vB, iMB, P, iIB, impulse * sBy);
    }
    d.j_imp[j] = imp;
    if (state_ne(vA, oldA) || state_ne(vB, oldB)) {
        if (bs.writable(a)) bs.set_vel(a, vA);
        if (bs.writable(b)) bs.set_vel(b, vB);
    }
}

template <class BS>
__device__ bool wheel_solve_position(const DW& d, const BS& bs, uint32_t j) {
    const DConf& c = *d.conf;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    const float iMA = mA.x, iIA = mA.y, iMB = mB.x, iIB = mB.y;
    float4 pA = bs.pos(a), pB = bs.pos(b);
    const float4 an = d.j_anchor[j], e0 = d.j_extra[2 * j], m0 = d.j_m0[j];
    const V2 qA = unit_from_angle(pA.z);
    const V2 rA = anchor_r(mk(an.x, an.y), mA, pA.z), rB = anchor_r(mk(an.z, an.w), mB, pB.z);
    const V2 dd = (mk(pB.x, pB.y) - mk(pA.x, pA.y)) + (rB - rA);
    const V2 ay = urotate(revperp(mk(e0.x, e0.y)), qA);
    const float sAy = cross(dd + rA, ay), sBy = cross(rB, ay);
    const float C = dot(dd, ay);
    // the effective mass uses sAy and sBy as InitVelocity left them
    const float k = iMA + iMB + iIA * (m0.z * m0.z) + iIB * (m0.w * m0.w);
    const float impulse = (k != 0.f) ? -(C / k) : 0.f;
    const V2 P = ay * impulse;
    sub_imp(pA, iMA, P, iIA, impulse * sAy);
    add_imp(pB, iMB, P, iIB, impulse * sBy);
    if (bs.writable(a)) bs.set_pos(a, pA);
    if (bs.writable(b)) bs.set_pos(b, pB);
    return fabsf(C) <= c.linearSlop;
}

// PulleyJointConf (PulleyJointConf.cpp:93-241); extra = groundAnchorA.xy
// groundAnchorB.xy lengthA lengthB ratio.
template <class BS>
__device__ void pulley_init_velocity(const DW& d, const BS& bs, uint32_t j) {
    const DConf& c = *d.conf;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    const float iMA = mA.x, iIA = mA.y, iMB = mB.x, iIB = mB.y;
    const float4 pA = bs.pos(a), pB = bs.pos(b);
    float4 vA = bs.vel(a), vB = bs.vel(b);
    const float4 an = d.j_anchor[j], e0 = d.j_extra[2 * j], e1 = d.j_extra[2 * j + 1];
    const float ratio = e1.z;
    const V2 rA = anchor_r(mk(an.x, an.y), mA, pA.z), rB = anchor_r(mk(an.z, an.w), mB, pB.z);
    const V2 uA = unit_vector((mk(pA.x, pA.y) + rA) - mk(e0.x, e0.y), mk(0.f, 0.f));
    const V2 uB = unit_vector((mk(pB.x, pB.y) + rB) - mk(e0.z, e0.w), mk(0.f, 0.f));
    const float ruA = cross(rA, uA), ruB = cross(rB, uB);
    const float totInvMassA = iMA + (iIA * (ruA * ruA));
    const float totInvMassB = iMB + (iIB * (ruB * ruB));
    const float totalInvMass = totInvMassA + ratio * ratio * totInvMassB;
    const float mass = (totalInvMass > 0.f) ? 1.0f / totalInvMass : 0.f;
    float4 imp = d.j_imp[j];
    if (c.doWarmStart) {
        imp.x *= c.dtRatio;
        const V2 PA = uA * (-imp.x);
        const V2 PB = uB * (-ratio * imp.x);
        add_imp(vA, iMA, PA, iIA, cross(rA, PA));
        add_imp(vB, iMB, PB, iIB, cross(rB, PB));
    } else {
        imp.x = 0.f;
    }
    d.j_imp[j] = imp;
    d.j_r[j] = make_float4(rA.x, rA.y, rB.x, rB.y);
    d.j_m0[j] = make_float4(uA.x, uA.y, uB.x, uB.y);
    d.j_m1[j] = make_float4(mass, 0.f, 0.f, 0.f);
    if (bs.writable(a)) bs.set_vel(a, vA);
    if (bs.writable(b)) bs.set_vel(b, vB);
}

template <class BS>
__device__ void pulley_solve_velocity(const DW& d, const BS& bs, uint32_t j) {
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    float4 vA = bs.vel(a), vB = bs.vel(b);
    const float4 r = d.j_r[j], m0 = d.j_m0[j];
    const float ratio = d.j_extra[2 * j + 1].z;
    float4 imp = d.j_imp[j];
    const V2 rA = mk(r.x, r.y), rB = mk(r.z, r.w), uA = mk(m0.x, m0.y), uB = mk(m0.z, m0.w);
    const float Cdot = -dot(uA, point_vel(vA, rA)) - ratio * dot(uB, point_vel(vB, rB));
    const float impulse = -d.j_m1[j].x * Cdot;
    imp.x += impulse;
    const V2 PA = uA * (-impulse);
    const V2 PB = uB * (-ratio * impulse);
    add_imp(vA, mA.x, PA, mA.y, cross(rA, PA));
    add_imp(vB, mB.x, PB, mB.y, cross(rB, PB));
    d.j_imp[j] = imp;
    if (bs.writable(a)) bs.set_vel(a, vA);
    if (bs.writable(b)) bs.set_vel(b, vB);
}

template <class BS>
__device__ bool pulley_solve_position(const DW& d, const BS& bs, uint32_t j) {
    const DConf& c = *d.conf;
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b);
    const float iMA = mA.x, iIA = mA.y, iMB = mB.x, iIB = mB.y;
    float4 pA = bs.pos(a), pB = bs.pos(b);
    const float4 an = d.j_anchor[j], e0 = d.j_extra[2 * j], e1 = d.j_extra[2 * j + 1];
    const float ratio = e1.z;
    const V2 rA = anchor_r(mk(an.x, an.y), mA, pA.z), rB = anchor_r(mk(an.z, an.w), mB, pB.z);
    float lengthA, lengthB;
    const V2 uA = unit_len((mk(pA.x, pA.y) + rA) - mk(e0.x, e0.y), lengthA);
    const V2 uB = unit_len((mk(pB.x, pB.y) + rB) - mk(e0.z, e0.w), lengthB);
    const float ruA = cross(rA, uA), ruB = cross(rB, uB);
    const float totalInvMassA = iMA + iIA * (ruA * ruA);
    const float totalInvMassB = iMB + iIB * (ruB * ruB);
    const float totalInvMass = totalInvMassA + (ratio * ratio) * totalInvMassB;
    const float mass = (totalInvMass > 0.f) ? 1.0f / totalInvMass : 0.f;
    const float srcLengthRatio = e1.x + ratio * e1.y;
    const float dstLengthRatio = lengthA + ratio * lengthB;
    const float C = srcLengthRatio - dstLengthRatio;
    const float impulse = -mass * C;
    const V2 PA = uA * (-impulse);
    const V2 PB = uB * (-ratio * impulse);
    add_imp(pA, iMA, PA, iIA, cross(rA, PA));
    add_imp(pB, iMB, PB, iIB, cross(rB, PB));
    if (bs.writable(a)) bs.set_pos(a, pA);
    if (bs.writable(b)) bs.set_pos(b, pB);
    return fabsf(C) < c.linearSlop;
}

// TargetJointConf (TargetJointConf.cpp:51-184): body B only (body A is the same
// index and untouched); extra = target.xy maxForce frequency dampingRatio.
template <class BS>
__device__ void target_init_velocity(const DW& d, const BS& bs, uint32_t j) {
    const DConf& c = *d.conf;
    const uint32_t b = d.j_bodies[2 * j + 1];
    const float4 mB = bs.mass(b);
    const float iM = mB.x, iI = mB.y;
    const float4 pB = bs.pos(b);
    float4 vB = bs.vel(b);
    const float4 an = d.j_anchor[j], e0 = d.j_extra[2 * j], e1 = d.j_extra[2 * j + 1];
    const float mass = (iM != 0.f) ? (1.0f / iM) : 0.f;
    const float Pi = 3.14159265358979323846264338327950288f;
    const float omega = 2.0f * Pi * e0.w;
    const float dc = 2.0f * mass * e1.x * omega;
    const float k = mass * (omega * omega);
    const float h = c.deltaTime;
    const float tmp = dc + h * k;
    const float invGamma = h * tmp;
    const float gamma = (invGamma != 0.f) ? 1.0f / invGamma : 0.f;
    const float beta = h * k * gamma;
    const V2 rB = anchor_r(mk(an.z, an.w), mB, pB.z);
    // GetEffectiveMassMatrix (TargetJointConf.cpp:51-72), then Invert(Matrix22)
    const float exx = iM + (iI * (rB.y * rB.y)) + gamma;
    const float exy = -iI * rB.x * rB.y;
    const float eyy = iM + (iI * (rB.x * rB.x)) + gamma;
    float l00 = 0.f, l01 = 0.f, l11 = 0.f;
    {
        const float cp = cross(mk(exx, exy), mk(exy, eyy));
        if (!almost_zero(cp)) {
            const float inv = 1.0f / cp;
            l00 = eyy * inv; l01 = -exy * inv; l11 = exx * inv;
        }
    }
    const V2 C = ((mk(pB.x, pB.y) + rB) - mk(e0.x, e0.y)) * beta;
    vB.z *= 0.98f;
    float4 imp = d.j_imp[j];
    if (c.doWarmStart) {
        imp.x *= c.dtRatio; imp.y *= c.dtRatio;
        const V2 P = mk(imp.x, imp.y);
        add_imp(vB, iM, P, iI, cross(rB, P));
    } else {
        imp.x = imp.y = 0.f;
    }
    d.j_imp[j] = imp;
    d.j_r[j] = make_float4(0.f, 0.f, rB.x, rB.y);
    d.j_m0[j] = make_float4(l00, l01, l11, gamma);
    d.j_m1[j] = make_float4(C.x, C.y, 0.f, 0.f);
    if (bs.writable(b)) bs.set_vel(b, vB);
}

template <class BS>
__device__ void target_solve_velocity(const DW& d, const BS& bs, uint32_t j) {
    const DConf& c = *d.conf;
    const uint32_t b = d.j_bodies[2 * j + 1];
    const float4 mB = bs.mass(b);
    float4 vB = bs.vel(b);
    const float4 r = d.j_r[j], m0 = d.j_m0[j], m1 = d.j_m1[j];
    float4 imp = d.j_imp[j];
    const V2 rB = mk(r.z, r.w);
    const V2 oldImpulse = mk(imp.x, imp.y);
    const V2 ev = point_vel(vB, rB) + (mk(m1.x, m1.y) + oldImpulse * m0.w);
    const V2 add = sym22_mul(m0.x, m0.y, m0.z, -ev);
    V2 impulse = oldImpulse + add;
    const float maxImpulse = c.deltaTime * d.j_extra[2 * j].z;
    if (mag2(impulse) > maxImpulse * maxImpulse) impulse = unit_vector(impulse, mk(0.f, 0.f)) * maxImpulse;
    imp.x = impulse.x; imp.y = impulse.y;
    const V2 inc = impulse - oldImpulse;
    add_imp(vB, mB.x, inc, mB.y, cross(rB, inc));
    d.j_imp[j] = imp;
    if (bs.writable(b)) bs.set_vel(b, vB);
}

// GearJointConf (GearJointConf.cpp:170-474): bodies A and B (the joint's) and C
// and D (the coupled joints' first bodies); the coupling of A to C (and of B
// to D) is through a revolute joint's angle or a prismatic joint's translation.
// Solver state: JvAC JvBD in j_r, JwA JwB JwC JwD in j_m0, mass in j_m1.x,
// impulse in j_imp.x.
struct GearData {
    uint32_t c, d;
    bool prisAC, prisBD;
    float ratio, constant, refAC, refBD;
    V2 laAC, lbAC, axAC, laBD, lbBD, axBD;
};
__device__ __forceinline__ GearData load_gear(const DW& d, uint32_t j) {
    const float4 g0 = d.j_gear[5 * j], g1 = d.j_gear[5 * j + 1], g2 = d.j_gear[5 * j + 2];
    const float4 g3 = d.j_gear[5 * j + 3], g4 = d.j_gear[5 * j + 4];
    GearData g;
    g.c = __float_as_uint(g0.x); g.d = __float_as_uint(g0.y);
    g.prisAC = __float_as_uint(g0.z) != 0u; g.prisBD = __float_as_uint(g0.w) != 0u;
    g.ratio = g1.x; g.constant = g1.y; g.refAC = g1.z; g.refBD = g1.w;
    g.laAC = mk(g2.x, g2.y); g.lbAC = mk(g2.z, g2.w); g.axAC = mk(g3.x, g3.y);
    g.laBD = mk(g3.z, g3.w); g.lbBD = mk(g4.x, g4.y); g.axBD = mk(g4.z, g4.w);
    return g;
}
// v += sign * {(iM * imp) * Jv, (iI * imp) * Jw}
__device__ __forceinline__ void gear_add(float4& v, V2 Jv, float iM, float iI, float Jw, float imp, bool add) {
    const V2 l = Jv * (iM * imp);
    const float a = (iI * imp) * Jw;
    if (add) { v.x = v.x + l.x; v.y = v.y + l.y; v.z = v.z + a; }
    else { v.x = v.x - l.x; v.y = v.y - l.y; v.z = v.z - a; }
}

template <class BS>
__device__ void gear_init_velocity(const DW& d, const BS& bs, uint32_t j) {
    const DConf& c = *d.conf;
    const GearData g = load_gear(d, j);
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b), mC = bs.mass(g.c), mD = bs.mass(g.d);
    float4 vA = bs.vel(a), vB = bs.vel(b), vC = bs.vel(g.c), vD = bs.vel(g.d);
    V2 JvAC = mk(0.f, 0.f), JvBD = mk(0.f, 0.f);
    float JwA, JwB, JwC, JwD, invMass = 0.f;
    if (g.prisAC) {
        const V2 qA = unit_from_angle(bs.pos(a).z), qC = unit_from_angle(bs.pos(g.c).z);
        const V2 u = rotate(g.axAC, qC);
        const V2 rC = rotate(g.laAC - mk(mC.z, mC.w), qC);
        const V2 rA = rotate(g.lbAC - mk(mA.z, mA.w), qA);
        JvAC = u * 1.0f;
        JwC = cross(rC, u);
        JwA = cross(rA, u);
        const float invRotMassC = mC.y * (JwC * JwC);
        const float invRotMassA = mA.y * (JwA * JwA);
        invMass += ((mC.x + mA.x) + invRotMassC) + invRotMassA;
    } else {
        JwA = 1.0f; JwC = 1.0f;
        invMass += mA.y + mC.y;
    }
    if (g.prisBD) {
        const V2 qB = unit_from_angle(bs.pos(b).z), qD = unit_from_angle(bs.pos(g.d).z);
        const V2 u = rotate(g.axBD, qD);
        const V2 rD = rotate(g.laBD - mk(mD.z, mD.w), qD);
        const V2 rB = rotate(g.lbBD - mk(mB.z, mB.w), qB);
        JvBD = u * g.ratio;
        JwD = g.ratio * cross(rD, u);
        JwB = g.ratio * cross(rB, u);
        const float invRotMassD = mD.y * (JwD * JwD);
        const float invRotMassB = mB.y * (JwB * JwB);
        invMass += ((g.ratio * g.ratio) * (mD.x + mB.x) + invRotMassD) + invRotMassB;
    } else {
        JwB = g.ratio; JwD = g.ratio;
        invMass += (g.ratio * g.ratio) * (mB.y + mD.y);
    }
    const float mass = (invMass > 0.f) ? 1.0f / invMass : 0.f;
    float4 imp = d.j_imp[j];
    if (c.doWarmStart) {
        gear_add(vA, JvAC, mA.x, mA.y, JwA, imp.x, true);
        gear_add(vB, JvBD, mB.x, mB.y, JwB, imp.x, true);
        gear_add(vC, JvAC, mC.x, mC.y, JwC, imp.x, false);
        gear_add(vD, JvBD, mD.x, mD.y, JwD, imp.x, false);
    } else {
        imp.x = 0.f;
    }
    d.j_imp[j] = imp;
    d.j_r[j] = make_float4(JvAC.x, JvAC.y, JvBD.x, JvBD.y);
    d.j_m0[j] = make_float4(JwA, JwB, JwC, JwD);
    d.j_m1[j] = make_float4(mass, 0.f, 0.f, 0.f);
    if (bs.writable(a)) bs.set_vel(a, vA);
    if (bs.writable(b)) bs.set_vel(b, vB);
    if (bs.writable(g.c)) bs.set_vel(g.c, vC);
    if (bs.writable(g.d)) bs.set_vel(g.d, vD);
}

template <class BS>
__device__ void gear_solve_velocity(const DW& d, const BS& bs, uint32_t j) {
    const float4 g0 = d.j_gear[5 * j];
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const uint32_t cc = __float_as_uint(g0.x), dd = __float_as_uint(g0.y);
    const float4 mA = bs.mass(a), mB = bs.mass(b), mC = bs.mass(cc), mD = bs.mass(dd);
    float4 vA = bs.vel(a), vB = bs.vel(b), vC = bs.vel(cc), vD = bs.vel(dd);
    const float4 r = d.j_r[j], w = d.j_m0[j];
    const V2 JvAC = mk(r.x, r.y), JvBD = mk(r.z, r.w);
    const float acDot = dot(JvAC, mk(vA.x, vA.y) - mk(vC.x, vC.y));
    const float bdDot = dot(JvBD, mk(vB.x, vB.y) - mk(vD.x, vD.y));
    const float Cdot = ((acDot + bdDot) + (w.x * vA.z - w.z * vC.z)) + (w.y * vB.z - w.w * vD.z);
    const float impulse = -d.j_m1[j].x * Cdot;
    float4 imp = d.j_imp[j];
    imp.x += impulse;
    gear_add(vA, JvAC, mA.x, mA.y, w.x, impulse, true);
    gear_add(vB, JvBD, mB.x, mB.y, w.y, impulse, true);
    gear_add(vC, JvAC, mC.x, mC.y, w.z, impulse, false);
    gear_add(vD, JvBD, mD.x, mD.y, w.w, impulse, false);
    d.j_imp[j] = imp;
    if (bs.writable(a)) bs.set_vel(a, vA);
    if (bs.writable(b)) bs.set_vel(b, vB);
    if (bs.writable(cc)) bs.set_vel(cc, vC);
    if (bs.writable(dd)) bs.set_vel(dd, vD);
}

// Cap(Position, ConstraintSolverConf) (d2/Math.cpp:63-71).
__device__ __forceinline__ void cap_position(float& x, float& y, float& a, const DConf& c) {
    float lsq = 0.f;
    lsq += x * x;
    lsq += y * y;
    if (lsq > c.maxLinearCorrection * c.maxLinearCorrection) {
        const float s = c.maxLinearCorrection / sqrtf(lsq);
        x = x * s; y = y * s;
    }
    a = (a < -c.maxAngularCorrection) ? -c.maxAngularCorrection : ((c.maxAngularCorrection < a) ? c.maxAngularCorrection : a);
}

template <class BS>
__device__ bool gear_solve_position(const DW& d, const BS& bs, uint32_t j) {
    const DConf& c = *d.conf;
    const GearData g = load_gear(d, j);
    const uint32_t a = d.j_bodies[2 * j], b = d.j_bodies[2 * j + 1];
    const float4 mA = bs.mass(a), mB = bs.mass(b), mC = bs.mass(g.c), mD = bs.mass(g.d);
    const float4 pA = bs.pos(a), pB = bs.pos(b), pC = bs.pos(g.c), pD = bs.pos(g.d);
    if (!isfinite(g.constant)) return true;
    V2 JvAC = mk(0.f, 0.f), JvBD = mk(0.f, 0.f);
    float JwA, JwB, JwC, JwD, coordA, coordB, invMass = 0.f;
    if (g.prisAC) {
        const V2 qA = unit_from_angle(pA.z), qC = unit_from_angle(pC.z);
        const V2 u = rotate(g.axAC, qC);
        const V2 rC = rotate(g.laAC - mk(mC.z, mC.w), qC);
        const V2 rA = rotate(g.lbAC - mk(mA.z, mA.w), qA);
        JvAC = u * 1.0f;
        JwC = cross(rC, u);
        JwA = cross(rA, u);
        const float invLinMass = mC.x + mA.x;
        const float invRotMassC = mC.y * (JwC * JwC);
        const float invRotMassA = mA.y * (JwA * JwA);
        invMass += (invLinMass + invRotMassC) + invRotMassA;
        const V2 pc = g.laAC - mk(mC.z, mC.w);
        const V2 pa = invrotate(rA + (mk(pA.x, pA.y) - mk(pC.x, pC.y)), qC);
        coordA = dot(pa - pc, g.axAC);
    } else {
        JwA = 1.0f; JwC = 1.0f;
        invMass += mA.y + mC.y;
        coordA = (pA.z - pC.z) - g.refAC;
    }
    if (g.prisBD) {
        const V2 qB = unit_from_angle(pB.z), qD = unit_from_angle(pD.z);
        const V2 u = rotate(g.axBD, qD);
        const V2 rD = rotate(g.laBD - mk(mD.z, mD.w), qD);
        const V2 rB = rotate(g.lbBD - mk(mB.z, mB.w), qB);
        JvBD = u * g.ratio;
        JwD = g.ratio * cross(rD, u);
        JwB = g.ratio * cross(rB, u);
        const float invLinMass = (g.ratio * g.ratio) * (mD.x + mB.x);
        const float invRotMassD = mD.y * (JwD * JwD);
        const float invRotMassB = mB.y * (JwB * JwB);
        invMass += (invLinMass + invRotMassD) + invRotMassB;
        const V2 pd = g.laBD - mk(mD.z, mD.w);
        const V2 pb = invrotate(rB + (mk(pB.x, pB.y) - mk(pD.x, pD.y)), qD);
        coordB = dot(pb - pd, g.axBD);
    } else {
        JwB = g.ratio; JwD = g.ratio;
        invMass += (g.ratio * g.ratio) * (mB.y + mD.y);
        coordB = (pB.z - pD.z) - g.refBD;
    }
    const float C = ((coordA + g.ratio * coordB) - g.constant) * c.regResolutionRate;
    const float impulse = (invMass > 0.f) ? -C / invMass : 0.f;
    float dAx = (mA.x * impulse) * JvAC.x, dAy = (mA.x * impulse) * JvAC.y, dAa = (mA.y * impulse) * JwA;
    float dCx = (mC.x * impulse) * JvAC.x, dCy = (mC.x * impulse) * JvAC.y, dCa = (mC.y * impulse) * JwC;
    float dBx = (mB.x * impulse) * JvBD.x, dBy = (mB.x * impulse) * JvBD.y, dBa = (mB.y * impulse) * JwB;
    float dDx = (mD.x * impulse) * JvBD.x, dDy = (mD.x * impulse) * JvBD.y, dDa = (mD.y * impulse) * JwD;
    cap_position(dAx, dAy, dAa, c);
    cap_position(dCx, dCy, dCa, c);
    cap_position(dBx, dBy, dBa, c);
    cap_position(dDx, dDy, dDa, c);
    if (bs.writable(a)) bs.set_pos(a, make_float4(pA.x + dAx, pA.y + dAy, pA.z + dAa, pA.w));
    if (bs.writable(b)) bs.set_pos(b, make_float4(pB.x + dBx, pB.y + dBy, pB.z + dBa, pB.w));
    if (bs.writable(g.c)) bs.set_pos(g.c, make_float4(pC.x - dCx, pC.y - dCy, pC.z - dCa, pC.w));
    if (bs.writable(g.d)) bs.set_pos(g.d, make_float4(pD.x - dDx, pD.y - dDy, pD.z - dDa, pD.w));
    auto msq = [](float x, float y) { float r = 0.f; r += x * x; r += y * y; return r; };
    float lin = 0.f, ang = 0.f;
    lin = maxf_(lin, msq(dAx, dAy)); lin = maxf_(lin, msq(dBx, dBy));
    lin = maxf_(lin, msq(dCx, dCy)); lin = maxf_(lin, msq(dDx, dDy));
    ang = maxf_(ang, fabsf(dAa)); ang = maxf_(ang, fabsf(dBa));
    ang = maxf_(ang, fabsf(dCa)); ang = maxf_(ang, fabsf(dDa));
    return (lin <= c.linearSlop * c.linearSlop) && (ang <= c.angularSlop);
}

// Joint dispatch on the kind (the JointConf visitors of Joint.cpp).
template <class BS>
__device__ __noinline__ void joint_init_velocity(const DW& d, const BS& bs, uint32_t j) {
    switch (joint_kind(d, j)) {
    case JK_DISTANCE: distance_init_velocity(d, bs, j, false); break;
    case JK_ROPE: distance_init_velocity(d, bs, j, true); break;
    case JK_WELD: weld_init_velocity(d, bs, j); break;
    case JK_FRICTION: friction_init_velocity(d, bs, j, false); break;
    case JK_MOTOR: friction_init_velocity(d, bs, j, true); break;
    case JK_PRISMATIC: prismatic_init_velocity(d, bs, j); break;
    case JK_WHEEL: wheel_init_velocity(d, bs, j); break;
    case JK_PULLEY: pulley_init_velocity(d, bs, j); break;
    case JK_TARGET: target_init_velocity(d, bs, j); break;
    case JK_GEAR: gear_init_velocity(d, bs, j); break;
    default: revolute_init_velocity(d, bs, j); break;
    }
}
template <class BS>
__device__ __noinline__ void joint_solve_velocity(const DW& d, const BS& bs, uint32_t j) {
    switch (joint_kind(d, j)) {
    case JK_DISTANCE: distance_solve_velocity(d, bs, j, false); break;
    case JK_ROPE: distance_solve_velocity(d, bs, j, true); break;
    case JK_WELD: weld_solve_velocity(d, bs, j); break;
    case JK_FRICTION: friction_solve_velocity(d, bs, j, false); break;
    case JK_MOTOR: friction_solve_velocity(d, bs, j, true); break;
    case JK_PRISMATIC: prismatic_solve_velocity(d, bs, j); break;
    case JK_WHEEL: wheel_solve_velocity(d, bs, j); break;
    case JK_PULLEY: pulley_solve_velocity(d, bs, j); break;
    case JK_TARGET: target_solve_velocity(d, bs, j); break;
    case JK_GEAR: gear_solve_velocity(d, bs, j); break;
    default: revolute_solve_velocity(d, bs, j); break;
    }
}
// Returns whether the joint is within tolerance.
template <class BS>
__device__ __noinline__ bool joint_solve_position(const DW& d, const BS& bs, uint32_t j) {
    switch (joint_kind(d, j)) {
    case JK_DISTANCE: return distance_solve_position(d, bs, j, false);
    case JK_ROPE: return distance_solve_position(d, bs, j, true);
    case JK_WELD: return weld_solve_position(d, bs, j);
    case JK_FRICTION: case JK_MOTOR: case JK_TARGET: return true;
    case JK_PRISMATIC: return prismatic_solve_position(d, bs, j);
    case JK_WHEEL: return wheel_solve_position(d, bs, j);
    case JK_PULLEY: return pulley_solve_position(d, bs, j);
    case JK_GEAR: return gear_solve_position(d, bs, j);
    default: return revolute_solve_position(d, bs, j);
    }
}

__device__ __forceinline__ uint32_t joint_island(const DW& d, uint32_t j) {
    const uint32_t a = d.j_bodies[2 * j];
    return is_speedable(d.b_flags[a]) ? d.b_island[a] : d.b_island[d.j_bodies[2 * j + 1]];
}

// ---- body state during the sweeps ---------------------------------------------
// The sweeps read and write body velocities and positions through one of two
// accessors.  GlobalBodies works on the batch arrays in HBM (the grid-wide
// solve, and worlds too large for shared memory).  SharedBodies works on a
// copy of one world's velocities and positions in the CTA's shared memory,
// staged in before the sweeps and written back after; inverse masses and flags,
// which the sweeps only read, stay in global memory behind the L1 cache.
// Both run the same arithmetic, so results do not depend on the accessor.
//
// Per-island position-iteration state (the minimum separation and the joint
// tolerance of iteration `it`, and whether the island already reached the
// tolerance) follows the same split.
struct GlobalBodies {
    const DW& d;
    __device__ __forceinline__ float4 vel(uint32_t b) const { return d.b_vel[b]; }
    __device__ __forceinline__ void set_vel(uint32_t b, float4 v) const { d.b_vel[b] = v; }
    __device__ __forceinline__ float4 pos(uint32_t b) const { return d.b_pos1[b]; }
    __device__ __forceinline__ void set_pos(uint32_t b, float4 p) const { d.b_pos1[b] = p; }
    __device__ __forceinline__ float4 mass(uint32_t b) const { return d.b_mass[b]; }
    __device__ __forceinline__ bool writable(uint32_t b) const { return is_accelerable(d.b_flags[b]); }
    // Whether island L reached the position tolerance before iteration `it`.
    __device__ __forceinline__ bool island_done(uint32_t L, int it) const {
        const float thr = d.conf->regMinSeparation;
        for (int k = 0; k < it; ++k) {
            const size_t at = (size_t)L * kMaxPosIters + k;
            if (__ldcg(&d.isl_sep[at]) >= thr && __ldcg(&d.isl_jok[at])) return true;
        }
        return false;
    }
    __device__ __forceinline__ void island_sep(uint32_t L, int it, float sep) const {
        atomic_min_float(&d.isl_sep[(size_t)L * kMaxPosIters + it], sep);
    }
    __device__ __forceinline__ void island_joint_fail(uint32_t L, int it) const {
        d.isl_jok[(size_t)L * kMaxPosIters + it] = 0u;
    }
};

// Shared-memory words per staged body: velocity and position (2 x float4),
// island separation, joint tolerance and done flag.
constexpr uint32_t kStageBytesPerBody = 44;

struct SharedBodies {
    const DW& d;
    uint32_t base;   // first body of the world
    float4* v;       // [nb] velocities
    float4* p;       // [nb] positions
    float* sep;      // [nb] by island root: min separation of the current position iteration
    uint32_t* jok;   // [nb] by island root: joints within tolerance in the current iteration
    uint32_t* done;  // [nb] by island root: tolerance reached in an earlier iteration
    __device__ __forceinline__ float4 vel(uint32_t b) const { return v[b - base]; }
    __device__ __forceinline__ void set_vel(uint32_t b, float4 x) const { v[b - base] = x; }
    __device__ __forceinline__ float4 pos(uint32_t b) const { return p[b - base]; }
    __device__ __forceinline__ void set_pos(uint32_t b, float4 x) const { p[b - base] = x; }
    __device__ __forceinline__ float4 mass(uint32_t b) const { return __ldg(&d.b_mass[b]); }
    __device__ __forceinline__ bool writable(uint32_t b) const { return is_accelerable(__ldg(&d.b_flags[b])); }
    __device__ __forceinline__ bool island_done(uint32_t L, int) const { return done[L - base] != 0u; }
    __device__ __forceinline__ void island_sep(uint32_t L, int, float s) const { atomic_min_float(&sep[L - base], s); }
    __device__ __forceinline__ void island_joint_fail(uint32_t L, int) const { jok[L - base] = 0u; }
};

// Non-binding prefetch of the line holding p into L1.
__device__ __forceinline__ void prefetch_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

// ---- per-constraint sweep steps (t = position in sweep order) -------------------
// When the step is recorded for the adjoint (d.tape), each contact step also
// writes the body state (and impulses) it starts from.  kMode says which of the
// joint code (kModeJoints) and the recording code (kModeTape) the instance
// carries: the caller guarantees a step needs no more, and the code left out
// costs the contact sweeps no registers.
constexpr int kModeJoints = 1, kModeTape = 2, kModeAll = kModeJoints | kModeTape;
template <int kMode = kModeAll, class BS>
__device__ __forceinline__ void sweep_warm(const DW& d, const BS& bs, uint32_t t) {
    const uint32_t id = d.t_id[t];
    if ((kMode & kModeJoints) && (id & kJointBit)) {
        const uint32_t j = id & ~kJointBit;
        if (d.tape) tape_joint_warm(d, t, j, bs.vel(d.j_bodies[2 * j]), bs.vel(d.j_bodies[2 * j + 1]));
        joint_init_velocity(d, bs, j);
        if (d.tape) tape_joint_check(d, j);
    } else if (d.conf->doWarmStart) {
        const VC vc = load_vc(d, t);
        if ((kMode & kModeTape) && d.tape) {
            d.tape->warm[2 * (size_t)t] = bs.vel(vc.bA);
            d.tape->warm[2 * (size_t)t + 1] = bs.vel(vc.bB);
        }
        warm_start(d, bs, vc);
    }
}

template <int kMode = kModeAll, class BS>
__device__ __forceinline__ void sweep_velocity(const DW& d, const BS& bs, uint32_t t, int it) {
    const uint32_t id = d.t_id[t];
    if ((kMode & kModeJoints) && (id & kJointBit)) {
        const uint32_t j = id & ~kJointBit;
        if (d.tape) {
            float4* r = d.tape->vel + 3 * ((size_t)it * d.tape->kcap + t);
            r[0] = bs.vel(d.j_bodies[2 * j]);
            r[1] = bs.vel(d.j_bodies[2 * j + 1]);
            const float4 i = d.j_imp[j];
            r[2] = make_float4(i.x, i.y, 0.f, 0.f);
        }
        joint_solve_velocity(d, bs, j);
    } else {
        VC vc = load_vc(d, t);
        if ((kMode & kModeTape) && d.tape) {
            float4* r = d.tape->vel + 3 * ((size_t)it * d.tape->kcap + t);
            r[0] = bs.vel(vc.bA);
            r[1] = bs.vel(vc.bB);
            r[2] = make_float4(vc.ni0, vc.ti0, vc.ni1, vc.ti1);
        }
        solve_contact_velocity(d, bs, vc);
        store_vc_impulses(d, t, vc);
    }
}

template <int kMode = kModeAll, class BS>
__device__ __forceinline__ void sweep_position(const DW& d, const BS& bs, uint32_t t, int it) {
    const uint32_t id = d.t_id[t];
    if ((kMode & kModeJoints) && (id & kJointBit)) {
        const uint32_t j = id & ~kJointBit;
        const uint32_t L = joint_island(d, j);
        const bool done = bs.island_done(L, it);
        if (d.tape) {
            float4* r = d.tape->pos + 2 * ((size_t)it * d.tape->kcap + t);
            float4 a = bs.pos(d.j_bodies[2 * j]);
            a.w = done ? 0.f : 1.f;
            r[0] = a;
            r[1] = bs.pos(d.j_bodies[2 * j + 1]);
        }
        if (done) return;
        if (!joint_solve_position(d, bs, j)) bs.island_joint_fail(L, it);
    } else {
        const PC pc = d.pc[t];
        const bool done = bs.island_done(pc.island, it);
        if ((kMode & kModeTape) && d.tape) {
            float4* r = d.tape->pos + 2 * ((size_t)it * d.tape->kcap + t);
            float4 a = bs.pos(pc.bA);
            a.w = done ? 0.f : 1.f;
            r[0] = a;
            r[1] = bs.pos(pc.bB);
        }
        if (done) return;
        const float sep = solve_contact_position(d, bs, pc, d.conf->regResolutionRate);
        bs.island_sep(pc.island, it, sep);
    }
}

// AssignImpulses (AabbTreeWorld.cpp:196-220)
__device__ __forceinline__ void store_impulses(const DW& d, uint32_t t) {
    const uint32_t slot = d.t_id[t];
    if (slot & kJointBit) return;
    const float4 e = d.vc0[t].q[3];
    const uint32_t count = __float_as_uint(d.vc0[t].q[2].w);
    float4 p0 = d.m_p0[slot];
    p0.z = e.x; p0.w = e.y;
    d.m_p0[slot] = p0;
    if (count == 2u) {
        const float4 i = d.vc1[t].q[3];
        float4 p1 = d.m_p1[slot];
        p1.z = i.x; p1.w = i.y;
        d.m_p1[slot] = p1;
    }
}

#if PRGPU_SOLVER_PART == 0
// Solve records for the PostSolveContact replay (Report, AabbTreeWorld.cpp:
// 196-205, called at :1669-1672): each solved contact's velocity-constraint
// impulses (GetContactImpulses: the points left after conditioning) and the
// iteration argument of its island: the position iteration that reached the
// tolerance, else StepConf::InvalidIteration (255).
__global__ void k_post_record(DW d) {
    const DConf& c = *d.conf;
    const int np = min(c.regPositionIters, kMaxPosIters);
    const uint32_t step = d.cnt->step_no;
    GRID_LOOP(t, d.cnt->n_active) {
        const uint32_t slot = d.t_id[t];
        if (slot & kJointBit) continue;
        const float4 e = d.vc0[t].q[3];
        const uint32_t count = __float_as_uint(d.vc0[t].q[2].w);
        const float4 i = (count == 2u) ? d.vc1[t].q[3] : make_float4(0.f, 0.f, 0.f, 0.f);
        const uint32_t L = d.pc[t].island;
        uint32_t iter = 255u;
        for (int k = 0; k < np; ++k) {
            const size_t at = (size_t)L * kMaxPosIters + k;
            if (d.isl_sep[at] >= c.regMinSeparation && d.isl_jok[at]) { iter = (uint32_t)k; break; }
        }
        d.cs_post[slot] = make_float4(e.x, e.y, i.x, i.y);
        d.cs_post_tag[slot] = make_uint2(step, count | (iter << 8));
    }
}
#endif

// IntegratePositions (AabbTreeWorld.cpp:176-188)
template <class BS>
__device__ __forceinline__ void integrate_body(const DW& d, const BS& bs, uint32_t b) {
    if (!(d.b_flags[b] & BF_SOLVED)) return;
    const float h = d.conf->deltaTime;
    const float4 v = bs.vel(b);
    float4 p = bs.pos(b);
    const float tx = v.x * h, ty = v.y * h, rot = h * v.z;
    p.x = p.x + tx; p.y = p.y + ty; p.z = p.z + rot;
    bs.set_pos(b, p);
}

#if PRGPU_SOLVER_PART == 0
// The whole regular-phase solve of a step over the batch: warm start, velocity
// sweeps, position integration, position sweeps, impulse store.  One
// cooperative launch; a bounded grid barrier separates colours; the serial
// colour runs on one thread.
__global__ void k_solve(DW d) {
    const DConf& c = *d.conf;
    const uint32_t* off = d.cnt->colour_off;
    const uint32_t ncol = d.cnt->n_colours;
    const bool lead = (blockIdx.x == 0 && threadIdx.x == 0);
    auto sweep = [&](uint32_t col, auto&& f) {
        const bool serial = (col == ncol);
        const uint32_t lo = serial ? off[kSerialColour] : off[col];
        const uint32_t hi = serial ? off[kSerialColour + 1] : off[col + 1];
        if (lo == hi) return;
        if (serial) {
            if (lead) for (uint32_t t = lo; t < hi; ++t) f(t);
        } else {
            GRID_LOOP(i, hi - lo) f(lo + i);
        }
        grid_barrier(d.cnt);
    };
    const GlobalBodies bs{d};
    for (uint32_t col = 0; col <= ncol; ++col) sweep(col, [&](uint32_t t) { sweep_warm(d, bs, t); });
    for (int it = 0; it < c.regVelocityIters; ++it)
        for (uint32_t col = 0; col <= ncol; ++col) sweep(col, [&](uint32_t t) { sweep_velocity(d, bs, t, it); });
    GRID_LOOP(b, d.n_bodies) integrate_body(d, bs, b);
    grid_barrier(d.cnt);
    for (int it = 0; it < c.regPositionIters && it < kMaxPosIters; ++it)
        for (uint32_t col = 0; col <= ncol; ++col) sweep(col, [&](uint32_t t) { sweep_position(d, bs, t, it); });
    GRID_LOOP(t, d.cnt->n_active) store_impulses(d, t);
}
#endif

// ---- one group of threads per world --------------------------------------------
// For batches of many worlds, a CTA (large worlds) or a warp (small ones) does
// all of one world's solve: colouring (the same rounds as k_colour, with group
// barriers), bucketing by colour, constraint construction and the sweeps, with
// a group barrier between two colours instead of a grid barrier.
//
// The active constraint lists are world-major (contact keys sort by proxy, and
// proxies are numbered world by world; joints likewise), so world w owns the
// contacts k in [w_kc[w], w_kc[w+1]) and the joints k in [w_kj[w], w_kj[w+1]).
__device__ __forceinline__ uint32_t constraint_world(const DW& d, uint32_t id) {
    uint32_t a, b;
    constraint_bodies(d, id, a, b);
    return d.b_world[a];
}

#if PRGPU_SOLVER_PART == 0
__global__ void k_world_ranges(DW d) {
    const uint32_t nc = d.cnt->n_active_c, na = d.cnt->n_active;
    GRID_LOOP(w, d.n_worlds + 1) {
        uint32_t lo = 0, hi = nc;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (constraint_world(d, d.k_list[mid]) < w) lo = mid + 1; else hi = mid;
        }
        d.w_kc[w] = lo;
        lo = nc; hi = na;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (constraint_world(d, d.k_list[mid]) < w) lo = mid + 1; else hi = mid;
        }
        d.w_kj[w] = lo;
    }
}
#endif

struct BlockGroup {
    __device__ __forceinline__ static void sync() { __syncthreads(); }
    __device__ __forceinline__ static bool any(bool p) { return __syncthreads_or(p) != 0; }
};
struct WarpGroup {
    __device__ __forceinline__ static void sync() { __syncwarp(); }
    __device__ __forceinline__ static bool any(bool p) {
        __syncwarp();
        return __any_sync(0xffffffffu, p) != 0;
    }
};
// kGroupThreads consecutive threads of a CTA on a named barrier of their own
// (1 + group index; barrier 0 is __syncthreads'), so that the CTA's groups sweep
// different worlds and one world's barrier waits overlap another's loads.
constexpr uint32_t kGroupThreads = 64;
struct SubGroup {
    __device__ __forceinline__ static uint32_t bar() { return 1u + threadIdx.x / kGroupThreads; }
    __device__ __forceinline__ static void sync() {
        asm volatile("bar.sync %0, %1;" ::"r"(bar()), "n"(kGroupThreads) : "memory");
    }
    __device__ __forceinline__ static bool any(bool p) {
        uint32_t r;
        asm volatile(
            "{\n .reg .pred ps, pd;\n setp.ne.u32 ps, %1, 0;\n bar.red.or.pred pd, %2, %3, ps;\n"
            " selp.u32 %0, 1, 0, pd;\n}"
            : "=r"(r)
            : "r"((uint32_t)p), "r"(bar()), "n"(kGroupThreads)
            : "memory");
        return r != 0u;
    }
};

// The sweeps of one world by one group, over its segment [base, base + n) of
// sweep order with colour offsets col_off; after_position(it) runs after each
// position iteration.
template <int kMode, class G, class BS, class F>
__device__ void sweeps(const DW& d, const BS& bs, uint32_t w, uint32_t rank, uint32_t size, uint32_t base,
                       uint32_t n, const uint32_t* col_off, F&& after_position) {
    const DConf& c = *d.conf;
    // parallel colours in use: 0 .. top-1 (then the serial colour, often empty)
    int top = 0;
    for (int q = 0; q < kMaxColours; ++q)
        if (col_off[q + 1] > col_off[q]) top = q + 1;
    const bool serial = col_off[kSerialColour + 1] > col_off[kSerialColour];
    // The colour after col in sweep order (the first one again after the last).
    auto next_col = [&](int col) { return (col + 1 < top) ? col + 1 : 0; };
    // Starts the loads of colour col's records for this thread (the constraint
    // ids and the records at `rec`, `stride` bytes apart), so that they arrive
    // while the current colour is solved.
    auto prefetch = [&](int col, const void* rec, size_t stride) {
        for (uint32_t t = base + col_off[col] + rank; t < base + col_off[col + 1]; t += size) {
            prefetch_l1(d.t_id + t);
            prefetch_l1(static_cast<const char*>(rec) + (size_t)t * stride);
        }
    };
    // Runs f(t) over colour col of this world, then synchronises the group.
    auto sweep = [&](int col, auto&& f) {
        const uint32_t lo = base + col_off[col], hi = base + col_off[col + 1];
        if (lo == hi) return;
        if (col == kSerialColour) {
            if (rank == 0) for (uint32_t t = lo; t < hi; ++t) f(t);
        } else {
            for (uint32_t t = lo + rank; t < hi; t += size) f(t);
        }
        G::sync();
    };
    // One pass over the world's colours; each parallel colour first prefetches the next.
    auto pass = [&](const void* rec, size_t stride, auto&& f) {
        for (int col = 0; col < top; ++col) {
            if (top > 1) prefetch(next_col(col), rec, stride);
            sweep(col, f);
        }
        if (serial) sweep(kSerialColour, f);
    };
    if (n) {
        pass(d.vc0, sizeof(VCRec), [&](uint32_t t) { sweep_warm<kMode>(d, bs, t); });
        for (int it = 0; it < c.regVelocityIters; ++it)
            pass(d.vc0, sizeof(VCRec), [&](uint32_t t) { sweep_velocity<kMode>(d, bs, t, it); });
    }
    for (uint32_t b = d.w_body_off[w] + rank; b < d.w_body_off[w + 1]; b += size) integrate_body(d, bs, b);
    G::sync();
    if (n) {
        for (int it = 0; it < c.regPositionIters && it < kMaxPosIters; ++it) {
            pass(d.pc, sizeof(PC), [&](uint32_t t) { sweep_position<kMode>(d, bs, t, it); });
            after_position(it);
        }
        for (uint32_t t = base + rank; t < base + n; t += size) store_impulses(d, t);
    }
    G::sync();
}

// col_cnt / col_off: kColStride words of shared memory owned by the group.
template <class G, int kMode>
__device__ void solve_world(const DW& d, uint32_t w, uint32_t rank, uint32_t size, uint32_t* col_cnt,
                            uint32_t* col_off, void* stage, uint32_t stage_cap) {
    const DConf& c = *d.conf;
    const uint32_t c0 = d.w_kc[w], c1 = d.w_kc[w + 1], j0 = d.w_kj[w], j1 = d.w_kj[w + 1];
    const uint32_t ncw = c1 - c0, n = ncw + (j1 - j0);
    const uint32_t base = c0 + (j0 - d.cnt->n_active_c);  // this world's segment of sweep order
    auto kof = [&](uint32_t i) { return (i < ncw) ? c0 + i : j0 + (i - ncw); };
    if (n) {
        // colouring
        for (uint32_t i = rank; i < n; i += size) colour_init(d, kof(i));
        for (uint32_t i = rank; i < (uint32_t)kColStride; i += size) col_cnt[i] = 0u;
        G::sync();
        for (int round = 0; round < kMaxColourRounds; ++round) {
            for (uint32_t i = rank; i < n; i += size) colour_pick(d, kof(i), round);
            G::sync();
            bool left = false;
            for (uint32_t i = rank; i < n; i += size) left |= colour_keep(d, kof(i));
            if (!G::any(left)) break;
        }
        // buckets by colour; what is left goes to the serial colour
        for (uint32_t i = rank; i < n; i += size) {
            const uint32_t k = kof(i);
            uint32_t col = d.k_colour[k];
            if (col == kNone) { col = (uint32_t)kSerialColour; d.k_colour[k] = col; }
            atomicAdd(&col_cnt[col], 1u);
        }
        G::sync();
        if (rank == 0) {
            uint32_t o = 0, used = 0;
            for (int k = 0; k <= kSerialColour; ++k) {
                col_off[k] = o;
                o += col_cnt[k];
                if (k < kSerialColour && col_cnt[k]) used = (uint32_t)k + 1u;
                col_cnt[k] = 0u;
            }
            col_off[kSerialColour + 1] = o;
            if (used) atomicMax(&d.cnt->n_colours, used);
            const uint32_t nser = o - col_off[kSerialColour];
            if (nser) atomicAdd(&d.cnt->colour_off[kSerialColour + 1], nser);
        }
        G::sync();
        for (uint32_t i = rank; i < n; i += size) {
            const uint32_t k = kof(i);
            const uint32_t col = d.k_colour[k];
            d.k_order[base + col_off[col] + atomicAdd(&col_cnt[col], 1u)] = k;
            // remembered as next step's first choice
            const uint32_t id = d.k_list[k];
            const uint32_t keep = (col < (uint32_t)kMaxColours) ? col : kNone;
            if (id & kJointBit) d.j_colour[id & ~kJointBit] = keep;
            else d.cs_colour[id] = keep;
        }
        G::sync();
        if (rank == 0 && col_off[kSerialColour + 1] > col_off[kSerialColour])
            sort_serial(d.k_order + base + col_off[kSerialColour], col_off[kSerialColour + 1] - col_off[kSerialColour]);
        G::sync();
        for (uint32_t t = base + rank; t < base + n; t += size) build_constraint(d, t, d.k_order[t]);
        G::sync();
    }
    if ((kMode & kModeTape) && d.tape) {  // recorded for the adjoint
        for (uint32_t t = base + rank; t < base + n; t += size) tape_constraint(d, t);
        tape_world(d, w, base, n, col_off, rank, size);
    }
    const uint32_t b0 = d.w_body_off[w], nb = d.w_body_off[w + 1] - b0;
    if (nb <= stage_cap) {
        // stage the world's velocities and positions in shared memory
        float4* sv = reinterpret_cast<float4*>(stage);
        float4* sp = sv + stage_cap;
        float* ssep = reinterpret_cast<float*>(sp + stage_cap);
        uint32_t* sjok = reinterpret_cast<uint32_t*>(ssep + stage_cap);
        uint32_t* sdone = sjok + stage_cap;
        for (uint32_t i = rank; i < nb; i += size) {
            sv[i] = d.b_vel[b0 + i];
            sp[i] = d.b_pos1[b0 + i];
            ssep[i] = __int_as_float(0x7f800000);
            sjok[i] = 1u;
            sdone[i] = 0u;
        }
        G::sync();
        const SharedBodies bs{d, b0, sv, sp, ssep, sjok, sdone};
        // after each position iteration: publish the islands' figures for the
        // sleep pass, fold them into the early-exit flags and reset them
        auto island_pass = [&](int it) {
            const float thr = c.regMinSeparation;
            for (uint32_t i = rank; i < nb; i += size) {
                if (d.b_island[b0 + i] != b0 + i || !(d.b_flags[b0 + i] & BF_SOLVED)) continue;
                const size_t at = (size_t)(b0 + i) * kMaxPosIters + it;
                d.isl_sep[at] = ssep[i];
                d.isl_jok[at] = sjok[i];
                if (ssep[i] >= thr && sjok[i]) sdone[i] = 1u;
                ssep[i] = __int_as_float(0x7f800000);
                sjok[i] = 1u;
            }
            G::sync();
        };
        sweeps<kMode, G>(d, bs, w, rank, size, base, n, col_off, island_pass);
        for (uint32_t i = rank; i < nb; i += size) {
            d.b_vel[b0 + i] = sv[i];
            d.b_pos1[b0 + i] = sp[i];
        }
    } else {
        const GlobalBodies bs{d};
        sweeps<kMode, G>(d, bs, w, rank, size, base, n, col_off, [](int) {});
    }
    G::sync();  // the group's shared words are reused by its next world
}

#if PRGPU_SOLVER_PART != 0
// Persistent CTAs take worlds from a queue ordered by decreasing body count.
// The first n_world_big entries are solved by a whole CTA each; once a CTA
// meets a smaller world, each of its groups of kGroupThreads threads takes
// worlds on its own up to n_world_mid, and then each of its warps.
// kMode: the joint and recording code the instance carries (sweep_warm).
#ifndef PRGPU_WORLD_SOLVE_MIN_BLOCKS
#define PRGPU_WORLD_SOLVE_MIN_BLOCKS 4
#endif
template <int kMode>
__global__ void __launch_bounds__(256, PRGPU_WORLD_SOLVE_MIN_BLOCKS) k_world_solve(DW d) {
    extern __shared__ float4 s_stage[];  // d.stage_bytes: body state of the world(s) being solved
    __shared__ uint32_t s_w;
    __shared__ uint32_t s_col[8][2][kColStride];
    uint32_t qi;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_w = atomicAdd(&d.cnt->world_queue, 1u);
        __syncthreads();
        qi = s_w;
        if (qi >= d.n_worlds) return;
        if (qi >= d.n_world_big) break;
        solve_world<BlockGroup, kMode>(d, d.w_order[qi], threadIdx.x, blockDim.x, s_col[0][0], s_col[0][1], s_stage,
                                d.stage_bytes / kStageBytesPerBody);
    }
    // each warp owns an eighth of the staging area, a group its warps' parts
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t part = d.stage_bytes / 8u;
    constexpr uint32_t gwarps = kGroupThreads / 32u;
    const uint32_t grp = threadIdx.x / kGroupThreads, grank = threadIdx.x % kGroupThreads;
    if (d.n_world_mid > d.n_world_big) {
        __shared__ uint32_t s_gq[256u / kGroupThreads];
        auto gnext = [&]() {
            SubGroup::sync();
            if (grank == 0) s_gq[grp] = atomicAdd(&d.cnt->world_queue, 1u);
            SubGroup::sync();
            return s_gq[grp];
        };
        if (grp != 0) qi = gnext();  // group 0 keeps the entry the CTA took
        void* gstage = reinterpret_cast<char*>(s_stage) + (size_t)(grp * gwarps) * part;
        while (qi < d.n_world_mid) {
            solve_world<SubGroup, kMode>(d, d.w_order[qi], grank, kGroupThreads, s_col[grp * gwarps][0],
                                  s_col[grp * gwarps][1], gstage, gwarps * part / kStageBytesPerBody);
            qi = gnext();
        }
        // the group's first warp keeps the group's entry
    }
    void* stage = reinterpret_cast<char*>(s_stage) + (size_t)warp * part;
    auto next = [&]() {
        uint32_t x = 0u;
        if (lane == 0) x = atomicAdd(&d.cnt->world_queue, 1u);
        return __shfl_sync(0xffffffffu, x, 0);
    };
    // warp 0 (of the CTA, or of each group) keeps the entry its CTA or group took
    if ((d.n_world_mid > d.n_world_big) ? (warp % gwarps != 0) : (warp != 0)) qi = next();
    while (qi < d.n_worlds) {
        solve_world<WarpGroup, kMode>(d, d.w_order[qi], lane, 32u, s_col[warp][0], s_col[warp][1], stage,
                               part / kStageBytesPerBody);
        qi = next();
    }
}
#endif

#if PRGPU_SOLVER_PART == 0
// Write-back bookkeeping, transforms and under-active times
// (AabbTreeWorld.cpp:1652-1679, :403-417).
__global__ void k_body_end(DW d) {
    const DConf& c = *d.conf;
    GRID_LOOP(b, d.n_bodies) {
        uint32_t f = d.b_flags[b];
        if (!(f & BF_SOLVED)) continue;
        const float4 p = d.b_pos1[b], p0 = d.b_pos0[b];
        if (p.x != p0.x || p.y != p0.y || p.z != p0.z) {
            f |= BF_MOVED;
            const float4 m = d.b_mass[b];
            const Xf x = get_xf(p.x, p.y, p.z, mk(m.z, m.w));
            d.b_xf[b] = make_float4(x.p.x, x.p.y, x.q.x, x.q.y);
        }
        d.b_flags[b] = f;
        const float4 v = d.b_vel[b];
        float lin2 = 0.f;
        lin2 += v.x * v.x;
        lin2 += v.y * v.y;
        const float ang2 = v.z * v.z;
        const bool under = (ang2 <= c.angularSleepTolerance * c.angularSleepTolerance) &&
                           (lin2 <= c.linearSleepTolerance * c.linearSleepTolerance);
        const float t = ((f & BF_ALLOW_SLEEP) && under) ? d.b_uat[b] + c.deltaTime : 0.f;
        d.b_uat[b] = t;
        atomic_min_float(&d.isl_uat[d.b_island[b]], t);
    }
}

__global__ void k_sleep(DW d) {
    const DConf& c = *d.conf;
    const int np = min(c.regPositionIters, kMaxPosIters);
    uint32_t slept = 0, solved_roots = 0, iters = 0;
    GRID_LOOP(b, d.n_bodies) {
        const uint32_t f = d.b_flags[b];
        if (!(f & BF_SOLVED)) continue;
        const uint32_t L = d.b_island[b];
        // solved: tolerance reached within the position iterations
        int done_at = -1;
        for (int k = 0; k < np; ++k) {
            const size_t at = (size_t)L * kMaxPosIters + k;
            if (d.isl_sep[at] >= c.regMinSeparation && d.isl_jok[at]) { done_at = k; break; }
        }
        if (L == b) {
            if (done_at >= 0) ++solved_roots;
            iters += (done_at >= 0) ? (uint32_t)(done_at + 1) : (uint32_t)np;
            const float ms = d.isl_sep[(size_t)L * kMaxPosIters];
            if (ms < __int_as_float(0x7f800000)) atomic_min_float(&d.cnt->st_min_separation, ms);
        }
        if (d.isl_uat[L] >= c.minStillTimeToSleep && done_at >= 0) {
            if ((f & BF_AWAKE) && (f & BF_ALLOW_SLEEP)) {
                d.b_flags[b] = f & ~BF_AWAKE;
                d.b_uat[b] = 0.f;
                d.b_vel[b] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (d.tape) d.tape->slept[b] = 1u;
                ++slept;
            }
        }
    }
    if (slept) atomicAdd(&d.cnt->st_bodies_slept, slept);
    if (solved_roots) atomicAdd(&d.cnt->st_islands_solved, solved_roots);
    if (iters) atomicAdd(&d.cnt->st_sum_pos_iters, iters);
}

__global__ void k_step_reset(DW d) {
    Counters* c = d.cnt;
    c->step_no += 1u;
    c->upd_phase = kUpdPre;
    c->st_contacts_added = 0u;
    c->st_contacts_destroyed = 0u;
    c->st_contacts_updated = 0u;
    c->st_islands_found = 0u;
    c->st_islands_solved = 0u;
    c->st_bodies_slept = 0u;
    c->st_proxies_moved = 0u;
    c->st_sum_pos_iters = 0u;
    c->st_min_separation = __int_as_float(0x7f800000);
    c->st_max_inc_impulse = 0.f;
    c->st_bodies_solved = 0u;
    c->bar_count = 0u;
    c->st_toi_found = 0u;
    c->st_toi_islands_found = 0u;
    c->st_toi_islands_solved = 0u;
    c->st_toi_sum_pos_iters = 0u;
    c->st_toi_sum_vel_iters = 0u;
    c->st_toi_updated_toi = 0u;
    c->st_toi_at_max_substeps = 0u;
    c->st_toi_updated_touching = 0u;
    c->st_toi_skipped_touching = 0u;
    c->st_toi_contacts_added = 0u;
    c->st_toi_proxies_moved = 0u;
    c->st_toi_max_dist_iters = 0u;
    c->st_toi_max_toi_iters = 0u;
    c->st_toi_max_root_iters = 0u;
    c->st_toi_min_separation = __int_as_float(0x7f800000);
    c->st_toi_max_inc_impulse = 0.f;
    c->toi_rounds = 0u;
}

__global__ void k_items_count(DW d, uint32_t* n_items) { *n_items = d.cnt->n_live + d.n_joints; }

__global__ void k_inc_off_tail(DW d) { d.inc_off[d.n_bodies] = d.cnt->pad[3]; }

__global__ void k_clear_dirty(DW d) {
    if (!d.cnt->dirty_any) return;
    GRID_LOOP(b, d.n_bodies) d.b_flags[b] &= ~BF_DIRTY;
}

__global__ void k_dirty_done(DW d) { d.cnt->dirty_any = 0u; }

template <typename K>
void launch_coop(K kernel, const DW& d, const Launch& L, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)L.coop_grid);
    cfg.blockDim = dim3((unsigned)L.coop_threads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, d);
}

#endif
}  // namespace

#if PRGPU_SOLVER_PART == 0
int coop_blocks_per_sm(int threads) {
    int a = 0, b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_solve, threads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_colour, threads, 0);
    return a < b ? a : b;
}

void launch_reset_step(const DW& d, const Launch& L, cudaStream_t s) {
    (void)L;
    k_step_reset<<<1, 1, 0, s>>>(d);
}

void launch_clear_dirty(const DW& d, const Launch& L, cudaStream_t s) {
    k_clear_dirty<<<L.grid, L.threads, 0, s>>>(d);
    k_dirty_done<<<1, 1, 0, s>>>(d);
}

void launch_islands_colour(const DW& d, const Launch& L, cudaStream_t s) {
    k_isl_init<<<L.grid, L.threads, 0, s>>>(d);
    k_isl_world<<<d.n_worlds, 256, 0, s>>>(d);
    k_isl_union<<<L.grid, L.threads, 0, s>>>(d, L.isl_big_worlds);
    k_isl_flatten<<<L.grid, L.threads, 0, s>>>(d);
    if (d.tape) launch_tape_body_start(d, L, s);
    k_body_begin<<<L.grid, L.threads, 0, s>>>(d);
    if (d.tape) launch_tape_body_flags(d, L, s);
    // active constraints in live-list order (contacts), then joints
    uint32_t* n_items = &d.cnt->pad[1];
    uint32_t* n_bodies = &d.cnt->pad[2];
    k_active_flags<<<L.grid, L.threads, 0, s>>>(d);
    k_items_count<<<1, 1, 0, s>>>(d, n_items);
    scan_exclusive(L.prims, d.flags, d.scan, n_items, &d.cnt->scan_total, d.partial, s);
    k_active_scatter<<<L.grid, L.threads, 0, s>>>(d);
    k_active_done<<<1, 1, 0, s>>>(d, n_bodies);
    cudaMemsetAsync(d.inc_cur, 0, sizeof(uint32_t) * (d.n_bodies + 1), s);
    k_inc_count<<<L.grid, L.threads, 0, s>>>(d);
    scan_exclusive(L.prims, d.inc_cur, d.inc_off, n_bodies, &d.cnt->pad[3], d.partial, s);
    k_inc_off_tail<<<1, 1, 0, s>>>(d);
    cudaMemsetAsync(d.inc_cur, 0, sizeof(uint32_t) * (d.n_bodies + 1), s);
    k_inc_fill<<<L.grid, L.threads, 0, s>>>(d);
    if (L.per_world) k_world_ranges<<<L.grid, L.threads, 0, s>>>(d);
    else launch_coop(k_colour, d, L, s);
}

void launch_build_constraints(const DW& d, const Launch& L, cudaStream_t s) {
    // per world, k_world_solve builds the constraints once it has coloured them
    if (!L.per_world) k_build_constraints<<<L.grid, L.threads, 0, s>>>(d);
    if (d.tape && !L.per_world) launch_tape_constraints(d, L, s);  // per world, k_world_solve records
}

void launch_solve_sweeps(const DW& d, const Launch& L, cudaStream_t s) {
    if (!L.per_world) {
        launch_coop(k_solve, d, L, s);
        return;
    }
    cudaMemsetAsync(&d.cnt->world_queue, 0, sizeof(uint32_t), s);
    if (d.n_joints) world_solve_full_launch(d, (unsigned)L.world_grid, s);
    else if (d.tape) world_solve_tape_launch(d, (unsigned)L.world_grid, s);
    else world_solve_lean_launch(d, (unsigned)L.world_grid, s);
}

int world_blocks_per_sm(uint32_t stage_bytes) {
    // The attribute is per function and per process: keep it at the largest
    // size any batch asked for, so every batch's launches stay valid.
    static std::mutex mu;
    static uint32_t set_bytes = 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (stage_bytes > set_bytes) {
            if (!world_solve_full_allow_smem(stage_bytes) || !world_solve_lean_allow_smem(stage_bytes) ||
                !world_solve_tape_allow_smem(stage_bytes))
                return 0;
            set_bytes = stage_bytes;
        }
    }
    // both instances have the same launch bounds; the grid is sized for the smaller residency
    const int a = world_solve_full_blocks_per_sm(stage_bytes), b = world_solve_lean_blocks_per_sm(stage_bytes);
    const int c = world_solve_tape_blocks_per_sm(stage_bytes);
    return std::min(a, std::min(b, c));
}

void launch_post_record(const DW& d, const Launch& L, cudaStream_t s) { k_post_record<<<L.grid, L.threads, 0, s>>>(d); }

void launch_solve_finish(const DW& d, const Launch& L, cudaStream_t s) {
    k_body_end<<<L.grid, L.threads, 0, s>>>(d);
    k_sleep<<<L.grid, L.threads, 0, s>>>(d);
}

void launch_solve(const DW& d, const Launch& L, cudaStream_t s) {
    launch_islands_colour(d, L, s);
    launch_build_constraints(d, L, s);
    launch_solve_sweeps(d, L, s);
    launch_solve_finish(d, L, s);
}
#else
// The one k_world_solve instance this translation unit compiles, and its launch
// helpers (declared in prgpu_kernels.cuh).
#if PRGPU_SOLVER_PART == 1
#define PRGPU_WS_MODE kModeAll
#define PRGPU_WS_NAME(x) world_solve_full_##x
#elif PRGPU_SOLVER_PART == 2
#define PRGPU_WS_MODE 0
#define PRGPU_WS_NAME(x) world_solve_lean_##x
#else
#define PRGPU_WS_MODE kModeTape
#define PRGPU_WS_NAME(x) world_solve_tape_##x
#endif

void PRGPU_WS_NAME(launch)(const DW& d, unsigned grid, cudaStream_t s) {
    k_world_solve<PRGPU_WS_MODE><<<grid, 256, d.stage_bytes, s>>>(d);
}

bool PRGPU_WS_NAME(allow_smem)(uint32_t stage_bytes) {
    return cudaFuncSetAttribute(k_world_solve<PRGPU_WS_MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)stage_bytes) == cudaSuccess;
}

int PRGPU_WS_NAME(blocks_per_sm)(uint32_t stage_bytes) {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_world_solve<PRGPU_WS_MODE>, 256, stage_bytes);
    return n;
}
#endif

}  // namespace prgpu
