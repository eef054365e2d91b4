// prgpu_toi.cu -- the time-of-impact phase of the world step (StepConf::doToi).
//
// Restates AabbTreeWorld::SolveToi (AabbTreeWorld.cpp:1685-2142) for a batch of
// worlds.  The reference handles one TOI event at a time per world: compute the
// time of impact of every impenetrable contact that lacks one, take the soonest,
// advance its two bodies to that time, gather the touching contacts they have
// with impenetrable bodies into a small island, re-solve that island for the rest
// of the step, synchronise the moved proxies, look for new contacts, and repeat.
// The GPU keeps that per-world sequence exactly and runs the worlds side by side:
//  * round 0 computes the times of impact of all contacts in parallel, one
//    thread per contact (every body still has alpha0 = 0, so the order in which
//    the reference visits them cannot matter);
//  * each further round is one event per world, solved by one warp per world:
//    the lanes gather the world's contacts that need a time of impact (in
//    contact-list order) and compute them side by side, find the soonest event,
//    and gather the event bodies' contacts; lane 0 runs the sequential parts
//    (advancing sweeps, CollideShapes, the island's position and velocity
//    iterations) with the island held in shared memory;
//  * between rounds the batch's broadphase (LBVH refit + query + AddContacts)
//    runs for the proxies the round moved.
// Contact-list order is the order contacts were created (cs_seq), as the
// reference appends new contacts to the world's and each body's list.
//
// Scans stay short: only impenetrable contacts (one body static, kinematic or a
// bullet) can have a time of impact, so the phase keeps a key-sorted list of
// them (rebuilt when a round adds contacts) and scans a world's slice of it.
// The reference's per-contact flags that the phase raises on every contact of a
// body (FlagForUpdating, ResetBodyContactsForSolveTOI) become per-body epochs of
// a per-world counter: a contact needs an update when one of its bodies moved
// after its last update, and its time of impact is void when one of its bodies
// was reset after it was computed.
#include <cooperative_groups.h>

#include "prgpu_contact_ops.cuh"
#include "prgpu_csolve.cuh"
#include "prgpu_kernels.cuh"
#include "prgpu_toi.cuh"

namespace prgpu {

namespace {

constexpr int kToiWarps = 4;             // worlds solved by one block of the round kernel
constexpr uint32_t kToiIslandContacts = 48;
constexpr uint32_t kToiIslandBodies = kToiIslandContacts + 1;
constexpr uint32_t kToiBatch = 64;       // contacts gathered and ordered at once by a warp
constexpr unsigned kFull = 0xffffffffu;

// Contacts whose times of impact a warp computes together: their sweeps are
// recorded in contact-list order (the Advance0 of each contact sees the ones
// before it), then the lanes run GetToiViaSat on them side by side.
struct ToiBatch {
    uint32_t slot[kToiBatch];
    uint64_t seq[kToiBatch];
    Sweep sA[kToiBatch], sB[kToiBatch];
    float alpha0[kToiBatch];
};

// An event's island and its solver state, in one warp's shared memory.  The
// velocity constraints are built only after the contacts have been gathered and
// the missing times of impact computed, so they share their memory with those.
struct ToiScratch {
    union {
        VC vc[kToiIslandContacts];
        ToiBatch batch;
    };
    float4 bp[kToiIslandBodies];   // body constraint position (x, y, angle)
    float4 bv[kToiIslandBodies];   // body constraint velocity
    float4 bm[kToiIslandBodies];   // invMass invRotI localCentre
    uint32_t bf[kToiIslandBodies]; // body flags
    uint32_t isl_b[kToiIslandBodies];
    uint32_t isl_c[kToiIslandContacts];
    Sweep backup;
    uint32_t nb, nc, updated, skipped, ep;
};

// Body-state accessor of the shared solver steps over an island (local indices).
struct ToiBodies {
    ToiScratch* s;
    __device__ __forceinline__ float4 vel(uint32_t b) const { return s->bv[b]; }
    __device__ __forceinline__ void set_vel(uint32_t b, float4 v) const { s->bv[b] = v; }
    __device__ __forceinline__ float4 pos(uint32_t b) const { return s->bp[b]; }
    __device__ __forceinline__ void set_pos(uint32_t b, float4 p) const { s->bp[b] = p; }
    __device__ __forceinline__ float4 mass(uint32_t b) const { return s->bm[b]; }
    __device__ __forceinline__ bool writable(uint32_t b) const { return is_accelerable(s->bf[b]); }
};

PR_HD ToiLimits toi_limits(const DConf& c) {
    ToiLimits L;
    L.targetDepth = c.targetDepth;
    L.tolerance = c.tolerance;
    L.maxRootIters = c.maxToiRootIters;
    L.maxToiIters = c.maxToiIters;
    L.maxDistIters = c.maxDistanceIters;
    return L;
}

// One out-of-line copy each of the two largest routines the phase calls from
// several places, to keep the round kernel's code small.
__device__ __noinline__ ToiOut toi_of(const Proxy& A, const Sweep& sA, const Proxy& B, const Sweep& sB,
                                      const ToiLimits& L) {
    return toi_via_sat(A, sA, B, sB, L);
}
// Update (AabbTreeWorld.cpp:2587-2721) inside the phase; stamps the contact
// with the world's current epoch.
__device__ __noinline__ void toi_update(const DW& d, uint32_t slot, uint32_t ep) {
    update_contact(d, slot);
    d.cs_toi_ep[slot] = ep;
}

__device__ __forceinline__ uint32_t toi_count(uint32_t f) { return (f & kToiCountMask) >> kToiCountShift; }

// NeedsUpdating: flagged, or a body moved since the contact's last update.
__device__ __forceinline__ bool toi_needs_update(const DW& d, uint32_t slot) {
    if (d.cs_flags[slot] & CF_NEEDS_UPDATE) return true;
    const uint2 bd = d.cs_body[slot];
    const uint32_t e = d.cs_toi_ep[slot];
    return d.b_toi_ep[bd.x] > e || d.b_toi_ep[bd.y] > e;
}
// HasValidToi: computed, and neither body reset since.
__device__ __forceinline__ bool toi_valid(const DW& d, uint32_t slot) {
    if (!(d.cs_flags[slot] & CF_TOI_VALID)) return false;
    const uint2 bd = d.cs_body[slot];
    const uint32_t at = d.cs_toi_at[slot];
    return at >= d.b_toi_rst[bd.x] && at >= d.b_toi_rst[bd.y];
}

__device__ __forceinline__ Sweep body_sweep(const DW& d, uint32_t b) {
    const float4 p0 = d.b_pos0[b], p1 = d.b_pos1[b], m = d.b_mass[b];
    Sweep s;
    s.p0 = mkpos(p0.x, p0.y, p0.z);
    s.p1 = mkpos(p1.x, p1.y, p1.z);
    s.lc = mk(m.z, m.w);
    s.a0 = d.b_alpha0[b];
    return s;
}
// Body::SetSweep (Body.hpp:697-702): the sweep and the cached transformation.
__device__ __forceinline__ void body_set_sweep(const DW& d, uint32_t b, const Sweep& s) {
    const float w0 = d.b_pos0[b].w, w1 = d.b_pos1[b].w;
    d.b_pos0[b] = make_float4(s.p0.x, s.p0.y, s.p0.a, w0);
    d.b_pos1[b] = make_float4(s.p1.x, s.p1.y, s.p1.a, w1);
    d.b_alpha0[b] = s.a0;
    const Xf xf = get_xf(s.p1.x, s.p1.y, s.p1.a, s.lc);
    d.b_xf[b] = make_float4(xf.p.x, xf.p.y, xf.q.x, xf.q.y);
}
// Advance (Body.hpp:1004-1009): Advance0, then position 1 = position 0.  When
// either position changed, every contact of the body needs an update
// (FlagForUpdating): the body takes a new epoch.
__device__ __forceinline__ void body_advance(const DW& d, uint32_t b, float alpha, Sweep& backup, uint32_t& ep) {
    backup = body_sweep(d, b);
    Sweep s = backup;
    sweep_advance0(s, alpha);
    s.p1 = s.p0;
    body_set_sweep(d, b, s);
    if (pos_ne(s.p0, backup.p0) || pos_ne(s.p1, backup.p1)) d.b_toi_ep[b] = ++ep;
}

// Both bodies' sweeps advanced to the later alpha0 (AabbTreeWorld.cpp:1717-1723);
// the normalised sweeps GetToiViaSat is given.
__device__ __forceinline__ float advance_pair(const DW& d, uint2 bd, Sweep& nA, Sweep& nB) {
    Sweep sA = body_sweep(d, bd.x), sB = body_sweep(d, bd.y);
    const float alpha0 = maxf_(sA.a0, sB.a0);
    sweep_advance0(sA, alpha0);
    d.b_pos0[bd.x] = make_float4(sA.p0.x, sA.p0.y, sA.p0.a, d.b_pos0[bd.x].w);
    d.b_alpha0[bd.x] = alpha0;
    sweep_advance0(sB, alpha0);
    d.b_pos0[bd.y] = make_float4(sB.p0.x, sB.p0.y, sB.p0.a, d.b_pos0[bd.y].w);
    d.b_alpha0[bd.y] = alpha0;
    nA = sweep_normalized(sA);
    nB = sweep_normalized(sB);
    return alpha0;
}

// The time of impact of a contact from its advanced sweeps (:1725-1748).
__device__ __forceinline__ void store_toi(const DW& d, uint32_t slot, const Sweep& sA, const Sweep& sB, float alpha0,
                                          uint32_t ep, const ToiLimits& L, int& mdist, int& mtoi, int& mroot) {
    const uint2 pr = d.cs_proxy[slot];
    Proxy A, B;
    load_proxy(d, pr.x, A);
    load_proxy(d, pr.y, B);
    const ToiOut o = toi_of(A, sA, B, sB, L);
    d.cs_toi[slot] = (o.state == TOI_TOUCHING) ? minf_(alpha0 + (1.0f - alpha0) * o.time, 1.0f) : 1.0f;
    d.cs_toi_at[slot] = ep;
    d.cs_flags[slot] |= CF_TOI_VALID;
    mdist = max(mdist, o.max_dist_iters);
    mtoi = max(mtoi, o.toi_iters);
    mroot = max(mroot, o.max_root_iters);
}

// The filter of UpdateContactTOIs (AabbTreeWorld.cpp:1692-1715) for a contact
// of the impenetrable list: 1 compute, 2 at the sub-step limit, 0 skip.
__device__ __forceinline__ int toi_candidate(const DW& d, uint32_t slot, int maxSubSteps) {
    const uint32_t f = d.cs_flags[slot];
    if ((f & (CF_SENSOR | CF_DISABLED)) || !(f & CF_IMPENETRABLE)) return 0;
    if (toi_valid(d, slot)) return 0;
    if ((int)toi_count(f) >= maxSubSteps) return 2;
    const uint2 bd = d.cs_body[slot];
    if (!(d.b_flags[bd.x] & BF_AWAKE) && !(d.b_flags[bd.y] & BF_AWAKE)) return 0;
    return 1;
}

__device__ __forceinline__ void toi_iter_stats(const DW& d, int mdist, int mtoi, int mroot) {
    if (mdist) atomicMax(&d.cnt->st_toi_max_dist_iters, (uint32_t)mdist);
    if (mtoi) atomicMax(&d.cnt->st_toi_max_toi_iters, (uint32_t)mtoi);
    if (mroot) atomicMax(&d.cnt->st_toi_max_root_iters, (uint32_t)mroot);
}

// ---- phase set-up, the impenetrable list and round 0 -----------------------------

// Every body starts the phase with alpha0 = 0 (ResetBodiesForSolveTOI ended the
// last one), no epochs, no proxy marked moved; every world at epoch 1.
// A world whose last phase sub-stepping stopped after an event continues that
// phase: its bodies' alpha0, the epochs and the contacts' times of impact stay.
__global__ void k_toi_begin(DW d) {
    GRID_LOOP(b, d.n_bodies) {
        if (d.w_incomplete[d.b_world[b]]) continue;
        d.b_alpha0[b] = 0.f;
        d.b_toi_ep[b] = 0u;
        d.b_toi_rst[b] = 0u;
    }
    GRID_LOOP(i, d.cnt->n_live) {
        const uint32_t s = d.c_slot[i];
        if (d.w_incomplete[d.b_world[d.cs_body[s].x]]) continue;
        d.cs_toi_ep[s] = 0u;
        d.cs_toi_at[s] = 0u;
    }
    GRID_LOOP(p, d.n_shapes) d.p_moved[p] = 0u;
    GRID_LOOP(w, d.n_worlds) {
        d.w_toi[w] = 0u;
        if (!d.w_incomplete[w]) d.w_toi_ep[w] = 1u;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        d.cnt->n_moved = 0u;
        d.cnt->toi_rounds = 0u;
        d.cnt->toi_events = 0u;
        d.cnt->toi_rebuild = 1u;
    }
}

// The impenetrable list: live contacts with an impenetrable body, key-sorted
// (a stable compaction of the live list), rebuilt when contacts were added.
__global__ void k_toi_list_flags(DW d) {
    Counters* c = d.cnt;
    const bool rebuild = c->toi_rebuild != 0u;
    if (blockIdx.x == 0 && threadIdx.x == 0) c->toi_scan_n = rebuild ? c->n_live : 0u;
    if (!rebuild) return;
    GRID_LOOP(i, c->n_live) {
        const uint32_t f = d.cs_flags[d.c_slot[i]];
        d.flags[i] = ((f & CF_IMPENETRABLE) && !(f & CF_SENSOR)) ? 1u : 0u;
    }
}
__global__ void k_toi_list_scatter(DW d) {
    if (!d.cnt->toi_rebuild) return;
    GRID_LOOP(i, d.cnt->n_live) {
        if (d.flags[i]) {
            d.t_key[d.scan[i]] = d.c_key[i];
            d.t_slot[d.scan[i]] = d.c_slot[i];
        }
    }
}
__global__ void k_toi_list_done(DW d) {
    Counters* c = d.cnt;
    if (c->toi_rebuild) c->n_imp = c->toi_imp_total;
    c->toi_rebuild = 0u;
}

// UpdateContactTOIs of the first loop iteration, one thread per impenetrable
// contact.  alpha0 is 0 for every body, so the Advance0 each contact applies to
// its two bodies is the same idempotent update whichever thread stores it.
__global__ void k_toi_first(DW d) {
    const DConf& c = *d.conf;
    const ToiLimits L = toi_limits(c);
    uint32_t updated = 0, at_max = 0;
    int mdist = 0, mtoi = 0, mroot = 0;
    GRID_LOOP(i, d.cnt->n_imp) {
        const uint32_t slot = d.t_slot[i];
        if (d.w_incomplete[d.b_world[d.cs_body[slot].x]]) continue;  // its round computes them in list order
        const int k = toi_candidate(d, slot, c.maxSubSteps);
        if (k == 2) ++at_max;
        if (k != 1) continue;
        Sweep sA, sB;
        const float alpha0 = advance_pair(d, d.cs_body[slot], sA, sB);
        store_toi(d, slot, sA, sB, alpha0, 1u, L, mdist, mtoi, mroot);
        ++updated;
    }
    if (updated) atomicAdd(&d.cnt->st_toi_updated_toi, updated);
    if (at_max) atomicAdd(&d.cnt->st_toi_at_max_substeps, at_max);
    toi_iter_stats(d, mdist, mtoi, mroot);
}

// ---- one event per world per round --------------------------------------------

__device__ __forceinline__ uint32_t lower_bound_key(const uint64_t* a, uint32_t n, uint64_t key) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// A world's slice of a key-sorted contact list (keys start with the smaller
// proxy index and a world's proxies are contiguous).
struct Seg {
    const uint32_t* slots;
    uint32_t c0, c1;
};
__device__ __forceinline__ Seg world_slice(const DW& d, uint32_t w, const uint64_t* keys, const uint32_t* slots,
                                           uint32_t n) {
    Seg s;
    s.slots = slots;
    s.c0 = lower_bound_key(keys, n, (uint64_t)d.w_shape_off[w] << d.key_bits);
    s.c1 = lower_bound_key(keys, n, (uint64_t)d.w_shape_off[w + 1] << d.key_bits);
    return s;
}

// The contact of the slice with the smallest creation sequence >= lo that
// passes pred (kNone if there is none); all lanes get the answer.
template <class Pred>
__device__ __forceinline__ uint32_t warp_first_in_list(const DW& d, Seg sg, uint64_t lo, uint32_t lane, Pred pred,
                                                       uint64_t& seq_out) {
    uint64_t best = ~0ull;
    uint32_t bslot = kNone;
    for (uint32_t i = sg.c0 + lane; i < sg.c1; i += 32u) {
        const uint32_t slot = sg.slots[i];
        const uint64_t q = d.cs_seq[slot];
        if (q >= lo && q < best && pred(slot)) { best = q; bslot = slot; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t ob = __shfl_xor_sync(kFull, best, o);
        const uint32_t os = __shfl_xor_sync(kFull, bslot, o);
        if (ob < best) { best = ob; bslot = os; }
    }
    seq_out = best;
    return bslot;
}

// Gathers the slice's contacts that pass pred into (slot, seq) ordered by
// creation sequence, i.e. in contact-list order.  Returns how many pass; only the
// first kToiBatch are stored, so a larger count means the list is incomplete.
template <class Pred>
__device__ uint32_t warp_gather_in_list_order(const DW& d, Seg sg, uint32_t lane, Pred pred, uint32_t* slots,
                                              uint64_t* seqs) {
    uint32_t n = 0;
    for (uint32_t base = sg.c0; base < sg.c1; base += 32u) {
        const uint32_t i = base + lane;
        uint32_t slot = kNone;
        bool take = false;
        if (i < sg.c1) {
            slot = sg.slots[i];
            take = pred(slot);
        }
        const unsigned m = __ballot_sync(kFull, take);
        if (take) {
            const uint32_t at = n + (uint32_t)__popc(m & ((1u << lane) - 1u));
            if (at < kToiBatch) { slots[at] = slot; seqs[at] = d.cs_seq[slot]; }
        }
        n += (uint32_t)__popc(m);
    }
    __syncwarp();
    // rank sort by sequence (sequences are unique): each lane places two entries
    const uint32_t k = min(n, kToiBatch);
    uint32_t ms[2] = {kNone, kNone}, rk[2] = {0, 0};
    uint64_t mq[2] = {0, 0};
    for (int e = 0; e < 2; ++e) {
        const uint32_t j = lane + 32u * (uint32_t)e;
        if (j < k) {
            ms[e] = slots[j]; mq[e] = seqs[j];
            for (uint32_t o = 0; o < k; ++o) rk[e] += (seqs[o] < mq[e]) ? 1u : 0u;
        }
    }
    __syncwarp();
    for (int e = 0; e < 2; ++e)
        if (ms[e] != kNone) { slots[rk[e]] = ms[e]; seqs[rk[e]] = mq[e]; }
    __syncwarp();
    return n;
}

// UpdateContactTOIs (AabbTreeWorld.cpp:1685-1750) for the world's contacts
// without a time of impact, in contact-list order: lane 0 advances the sweeps
// (cheap and order-dependent), then every lane computes times of impact.  Up
// to kToiBatch such contacts are gathered at once (the usual case after an
// event); beyond that lane 0 takes them one by one.
__device__ void toi_update_world(const DW& d, Seg imp, ToiScratch& S, uint32_t lane) {
    const DConf& c = *d.conf;
    const ToiLimits L = toi_limits(c);
    uint32_t at_max = 0;
    for (uint32_t i = imp.c0 + lane; i < imp.c1; i += 32u)
        if (toi_candidate(d, imp.slots[i], c.maxSubSteps) == 2) ++at_max;
    if (at_max) atomicAdd(&d.cnt->st_toi_at_max_substeps, at_max);
    int mdist = 0, mtoi = 0, mroot = 0;
    uint32_t updated = 0;
    ToiBatch& B = S.batch;
    const uint32_t ep = S.ep;
    auto missing = [&](uint32_t s) { return toi_candidate(d, s, c.maxSubSteps) == 1; };
    const uint32_t n = warp_gather_in_list_order(d, imp, lane, missing, B.slot, B.seq);
    if (n > kToiBatch) {
        for (uint32_t guard = 0; guard <= imp.c1 - imp.c0; ++guard) {  // each pass gives one contact a time
            uint64_t q;
            const uint32_t slot = warp_first_in_list(d, imp, 0, lane, missing, q);
            if (slot == kNone) break;
            if (lane == 0) {
                Sweep sA, sB;
                const float alpha0 = advance_pair(d, d.cs_body[slot], sA, sB);
                store_toi(d, slot, sA, sB, alpha0, ep, L, mdist, mtoi, mroot);
                ++updated;
            }
            __syncwarp();
        }
    } else if (n > 0) {
        if (lane == 0)
            for (uint32_t j = 0; j < n; ++j) B.alpha0[j] = advance_pair(d, d.cs_body[B.slot[j]], B.sA[j], B.sB[j]);
        __syncwarp();
        for (uint32_t j = lane; j < n; j += 32u) {
            store_toi(d, B.slot[j], B.sA[j], B.sB[j], B.alpha0[j], ep, L, mdist, mtoi, mroot);
            ++updated;
        }
        __syncwarp();
    }
    if (updated) atomicAdd(&d.cnt->st_toi_updated_toi, updated);
    toi_iter_stats(d, mdist, mtoi, mroot);
}

__device__ __forceinline__ uint32_t island_local(const ToiScratch& S, uint32_t b) {
    for (uint32_t i = 0; i < S.nb; ++i)
        if (S.isl_b[i] == b) return i;
    return kNone;
}

// GetBodyConstraint (BodyConstraint.hpp:157-167) at h: velocity integrated,
// damped and capped as in the regular phase.
__device__ __forceinline__ float4 constraint_velocity(const DW& d, uint32_t b, float h) {
    const DConf& c = *d.conf;
    const uint32_t f = d.b_flags[b];
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
    return v;
}

// SolveToiViaGS (AabbTreeWorld.cpp:1957-2059) on lane 0: position iterations
// at toiResolutionRate, the leap to the new position 0, velocity iterations
// without warm starting, integration over the rest of the step.
__device__ void toi_solve_island(const DW& d, ToiScratch& S, float toi) {
    const DConf& c = *d.conf;
    const float h = (1.0f - toi) * c.deltaTime;
    for (uint32_t i = 0; i < S.nb; ++i) {
        const uint32_t g = S.isl_b[i];
        S.bp[i] = d.b_pos1[g];
        S.bm[i] = d.b_mass[g];
        S.bf[i] = d.b_flags[g];
        S.bv[i] = constraint_velocity(d, g, 0.f);
    }
    const ToiBodies bs{&S};
    const float inf = __int_as_float(0x7f800000);
    float minSepAll = inf;
    bool solved = false;
    int posIters = c.toiPositionIters;
    for (int it = 0; it < c.toiPositionIters; ++it) {
        float minSep = inf;
        for (uint32_t k = 0; k < S.nc; ++k) {
            const uint32_t slot = S.isl_c[k];
            const uint2 bd = d.cs_body[slot], pr = d.cs_proxy[slot];
            const uint32_t la = island_local(S, bd.x), lb = island_local(S, bd.y);
            if (la == kNone || lb == kNone) { set_error(d.cnt, PR_ESTATE, 41u); return; }
            const PC pc = make_contact_pc(load_manrec(d, slot), d.s_radius[pr.x] + d.s_radius[pr.y], la, lb);
            minSep = minf_(minSep, solve_contact_position(d, bs, pc, c.toiResolutionRate));
        }
        minSepAll = minf_(minSepAll, minSep);
        if (minSep >= c.toiMinSeparation) { posIters = it + 1; solved = true; break; }
    }
    for (uint32_t i = 0; i < S.nb; ++i) {  // SetPosition0: the sweep only
        const uint32_t g = S.isl_b[i];
        d.b_pos0[g] = make_float4(S.bp[i].x, S.bp[i].y, S.bp[i].z, d.b_pos0[g].w);
    }
    for (uint32_t k = 0; k < S.nc; ++k) {  // GetToiVelocityConstraintConf: dtRatio 0
        const uint32_t slot = S.isl_c[k];
        const uint2 bd = d.cs_body[slot], pr = d.cs_proxy[slot];
        const uint32_t la = island_local(S, bd.x), lb = island_local(S, bd.y);
        if (la == kNone || lb == kNone) { set_error(d.cnt, PR_ESTATE, 41u); return; }
        VC vc = make_contact_vc(load_manrec(d, slot), S.bp[la], S.bp[lb], S.bm[la], S.bm[lb], S.bv[la], S.bv[lb],
                                d.s_radius[pr.x], d.s_radius[pr.y], d.cs_mat[slot], 0.f, c, d.cs_tspeed[slot]);
        vc.bA = la; vc.bB = lb;
        S.vc[k] = vc;
    }
    float maxInc = 0.f;
    int velIters = c.toiVelocityIters;
    for (int it = 0; it < c.toiVelocityIters; ++it) {
        float newInc = 0.f;
        for (uint32_t k = 0; k < S.nc; ++k) newInc = maxf_(newInc, solve_contact_velocity<ToiBodies, true>(d, bs, S.vc[k]));
        if (newInc <= c.toiMinMomentum) { velIters = it + 1; break; }
        maxInc = maxf_(maxInc, newInc);
    }
    for (uint32_t i = 0; i < S.nb; ++i) {  // IntegratePositions, then the write-back
        float4 p = S.bp[i];
        const float4 v = S.bv[i];
        const float tx = v.x * h, ty = v.y * h, rot = h * v.z;
        p.x = p.x + tx; p.y = p.y + ty; p.z = p.z + rot;
        const uint32_t g = S.isl_b[i];
        d.b_vel[g] = make_float4(v.x, v.y, v.z, d.b_vel[g].w);
        const float4 p1 = d.b_pos1[g];
        if (pos_ne(mkpos(p1.x, p1.y, p1.z), mkpos(p.x, p.y, p.z))) {
            d.b_pos1[g] = make_float4(p.x, p.y, p.z, p1.w);
            const Xf xf = get_xf(p.x, p.y, p.z, mk(S.bm[i].z, S.bm[i].w));
            d.b_xf[g] = make_float4(xf.p.x, xf.p.y, xf.q.x, xf.q.y);
            d.b_toi_ep[g] = ++S.ep;  // FlagForUpdating of its contacts
        }
    }
    Counters* cn = d.cnt;
    if (solved) atomicAdd(&cn->st_toi_islands_solved, 1u);
    if (posIters > 0 || velIters > 0) atomicAdd(&cn->st_toi_islands_found, 1u);
    atomicAdd(&cn->st_toi_sum_pos_iters, (uint32_t)posIters);
    atomicAdd(&cn->st_toi_sum_vel_iters, (uint32_t)velIters);
    atomic_min_float(&cn->st_toi_min_separation, minSepAll);
    atomic_max_nonneg_float(&cn->st_toi_max_inc_impulse, maxInc);
}

// One contact of ProcessContactsForTOI (AabbTreeWorld.cpp:2084-2137) for body
// x, on lane 0.  Returns false on island overflow.
__device__ bool toi_process_contact(const DW& d, uint32_t x, bool impX, uint32_t slot, float toi, ToiScratch& S) {
    const uint32_t f0 = d.cs_flags[slot];
    const uint2 bd = d.cs_body[slot];
    const uint32_t other = (bd.x == x) ? bd.y : bd.x;
    const uint32_t fo = d.b_flags[other];
    if ((f0 & (CF_TOI_ISL | CF_SENSOR)) || !(impX || is_impenetrable(fo))) return true;
    const bool otherIslanded = (fo & BF_TOI_ISL) != 0u;
    if (!otherIslanded) body_advance(d, other, toi, S.backup, S.ep);
    else S.backup = body_sweep(d, other);
    if (toi_needs_update(d, slot)) {
        toi_update(d, slot, S.ep);
        ++S.updated;
    } else {
        ++S.skipped;
    }
    const uint32_t f = d.cs_flags[slot];
    if (!(f & CF_TOUCHING) || (f & CF_DISABLED)) {  // not touching, or disabled by SetContact
        body_set_sweep(d, other, S.backup);
        return true;
    }
    if (S.nc >= kToiIslandContacts) return false;
    S.isl_c[S.nc++] = slot;
    d.cs_flags[slot] = f | CF_TOI_ISL;
    if (!otherIslanded) {
        d.b_flags[other] = fo | BF_TOI_ISL | (is_speedable(fo) ? BF_AWAKE : 0u);
        S.isl_b[S.nb++] = other;
    }
    return true;
}

// ProcessContactsForTOI (AabbTreeWorld.cpp:2061-2142) for body x, walking its
// contacts in its contact-list order.  Only contacts with an impenetrable body
// take part unless x is itself impenetrable (a bullet), so a non-bullet walks
// the impenetrable list and a bullet all of its world's contacts.  Returns false
// on island overflow.
__device__ bool toi_process_contacts(const DW& d, Seg all, Seg imp, uint32_t x, float toi, ToiScratch& S,
                                     uint32_t lane) {
    const bool impX = is_impenetrable(d.b_flags[x]);
    const Seg sg = impX ? all : imp;
    auto touches_x = [&](uint32_t s) {
        const uint2 bd = d.cs_body[s];
        return bd.x == x || bd.y == x;
    };
    // the body's list, gathered once (the island solve reuses this memory later)
    const uint32_t n = warp_gather_in_list_order(d, sg, lane, touches_x, S.batch.slot, S.batch.seq);
    uint32_t ok = 1u;
    if (n <= kToiBatch) {
        if (lane == 0)
            for (uint32_t j = 0; j < n && ok; ++j) ok = toi_process_contact(d, x, impX, S.batch.slot[j], toi, S);
        ok = __shfl_sync(kFull, ok, 0);
        __syncwarp();
        return ok != 0u;
    }
    // more contacts than one gather holds: take them one scan at a time
    uint64_t lo = 0;
    for (uint32_t guard = 0; guard <= sg.c1 - sg.c0 && ok; ++guard) {  // each pass takes a later contact
        uint64_t q;
        const uint32_t slot = warp_first_in_list(d, sg, lo, lane, touches_x, q);
        if (slot == kNone) break;
        lo = q + 1;
        if (lane == 0) ok = toi_process_contact(d, x, impX, slot, toi, S);
        ok = __shfl_sync(kFull, ok, 0);
        __syncwarp();
    }
    return ok != 0u;
}

// SolveToi(ContactID) (AabbTreeWorld.cpp:1833-1955) for the world's soonest
// contact; returns false if the island overflowed its shared-memory capacity.
__device__ bool toi_event(const DW& d, Seg all, Seg imp, uint32_t next, ToiScratch& S, uint32_t lane) {
    const uint2 bd = d.cs_body[next];
    const float toi = d.cs_toi[next];
    uint32_t go = 0;
    if (lane == 0) {
        Sweep bkA, bkB;
        body_advance(d, bd.x, toi, bkA, S.ep);
        body_advance(d, bd.y, toi, bkB, S.ep);
        uint32_t updated = 0;
        if (toi_needs_update(d, next)) {
            toi_update(d, next, S.ep);
            updated = 1;
        }
        uint32_t f = d.cs_flags[next];
        const uint32_t n = min(toi_count(f) + 1u, 255u);
        f = (f & ~(CF_TOI_VALID | kToiCountMask)) | (n << kToiCountShift);
        if (!(f & CF_TOUCHING)) {
            d.cs_flags[next] = f;
            body_set_sweep(d, bd.x, bkA);
            body_set_sweep(d, bd.y, bkB);
            atomicAdd(&d.cnt->st_toi_updated_touching, updated);
            atomicAdd(&d.cnt->st_toi_skipped_touching, updated ? 0u : 1u);
        } else {
            d.cs_flags[next] = f | CF_TOI_ISL;
            const uint32_t fa = d.b_flags[bd.x], fb = d.b_flags[bd.y];
            d.b_flags[bd.x] = fa | BF_TOI_ISL | (is_speedable(fa) ? BF_AWAKE : 0u);
            d.b_flags[bd.y] = fb | BF_TOI_ISL | (is_speedable(fb) ? BF_AWAKE : 0u);
            S.isl_b[0] = bd.x; S.isl_b[1] = bd.y; S.nb = 2;
            S.isl_c[0] = next; S.nc = 1;
            S.updated = updated; S.skipped = 0;
            go = 1;
        }
    }
    go = __shfl_sync(kFull, go, 0);
    __syncwarp();
    if (!go) return true;
    if (is_accelerable(d.b_flags[bd.x]) && !toi_process_contacts(d, all, imp, bd.x, toi, S, lane)) return false;
    if (is_accelerable(d.b_flags[bd.y]) && !toi_process_contacts(d, all, imp, bd.y, toi, S, lane)) return false;
    if (lane == 0) {
        for (uint32_t i = 0; i < S.nb; ++i) {  // RemoveUnspeedablesFromIslanded
            const uint32_t g = S.isl_b[i];
            if (!is_speedable(d.b_flags[g])) d.b_flags[g] &= ~BF_TOI_ISL;
        }
        toi_solve_island(d, S, toi);
        atomicAdd(&d.cnt->st_toi_updated_touching, S.updated);
        atomicAdd(&d.cnt->st_toi_skipped_touching, S.skipped);
    }
    __syncwarp();
    return true;
}

// Synchronize (AabbTreeWorld.cpp:2564-2585) of the proxies of body b, as the
// TOI loop does for each accelerable islanded body (:1805-1812).
__device__ __forceinline__ uint32_t toi_sync_body(const DW& d, uint32_t b) {
    uint32_t moved = 0;
    for (uint32_t k = d.b_shape_off[b]; k < d.b_shape_off[b + 1]; ++k) {
        const uint32_t p = d.b_shapes[k];
        const Xf x0 = xf0_of(d, b), x1 = load_xf(d, b);
        const Box a = swept_aabb(d, p, x0, x1);
        if (!contains4(d.p_aabb[p], a)) {
            d.p_aabb[p] = fat_box(d, a, x0, x1);
            d.p_moved[p] = 1u;
            const uint32_t at = atomicAdd(&d.cnt->n_moved, 1u);
            d.moved_list[at] = p;
            ++moved;
        }
    }
    return moved;
}

// One iteration of the reference's TOI loop (AabbTreeWorld.cpp:1758-1826) for
// world w: missing times of impact, the soonest event, its island, then the
// islanded bodies' proxies and contacts.
__device__ void toi_world_round(const DW& d, uint32_t w, ToiScratch& S, bool first, uint32_t lane) {
    const Seg imp = world_slice(d, w, d.t_key, d.t_slot, d.cnt->n_imp);
    if (lane == 0) { S.ep = d.w_toi_ep[w]; S.nb = 0; S.nc = 0; }
    __syncwarp();
    // round 0 of a continued phase: its missing times of impact in list order
    if (!first || d.w_incomplete[w]) toi_update_world(d, imp, S, lane);
    // GetSoonestContact (AabbTreeWorld.cpp:2870-2890): the smallest time below 1,
    // the earliest in the contact list among equal times
    float best = 1.0f;
    uint64_t bseq = ~0ull;
    uint32_t next = kNone;
    for (uint32_t i = imp.c0 + lane; i < imp.c1; i += 32u) {
        const uint32_t slot = imp.slots[i];
        if (!toi_valid(d, slot)) continue;
        const float t = d.cs_toi[slot];
        const uint64_t q = d.cs_seq[slot];
        if (t < best || (t == best && next != kNone && q < bseq)) { best = t; bseq = q; next = slot; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(kFull, best, o);
        const uint64_t oq = __shfl_xor_sync(kFull, bseq, o);
        const uint32_t on = __shfl_xor_sync(kFull, next, o);
        if (on != kNone && (next == kNone || ob < best || (ob == best && oq < bseq))) {
            best = ob; bseq = oq; next = on;
        }
    }
    if (next == kNone) {
        // no more events: ResetBodiesForSolveTOI and ResetContactsForSolveTOI
        // (only impenetrable contacts carry TOI bits; the epochs restart next phase)
        for (uint32_t b = d.w_body_off[w] + lane; b < d.w_body_off[w + 1]; b += 32u) d.b_alpha0[b] = 0.f;
        for (uint32_t i = imp.c0 + lane; i < imp.c1; i += 32u)
            d.cs_flags[imp.slots[i]] &= ~(CF_TOI_VALID | CF_TOI_ISL | kToiCountMask);
        if (lane == 0) { d.w_toi[w] = 1u; d.w_incomplete[w] = 0u; }  // e_stepComplete
        return;
    }
    if (lane == 0) {
        atomicAdd(&d.cnt->st_toi_found, 1u);
        atomicAdd(&d.cnt->toi_events, 1u);
    }
    if (!(d.cs_flags[next] & CF_TOI_ISL)) {
        const Seg all = world_slice(d, w, d.c_key, d.c_slot, d.cnt->n_live);
        if (!toi_event(d, all, imp, next, S, lane)) {
            if (lane == 0) set_error(d.cnt, PR_ECAPACITY, 40u);
            return;
        }
    }
    // the islanded bodies: accelerable ones synchronise their proxies and void
    // their contacts' times of impact (one new epoch for all); the event's
    // contacts leave the island
    uint32_t moved = 0;
    const uint32_t rst = S.ep + 1u;
    for (uint32_t i = lane; i < S.nb; i += 32u) {
        const uint32_t g = S.isl_b[i];
        const uint32_t f = d.b_flags[g];
        if ((f & BF_TOI_ISL) && is_accelerable(f)) {
            moved += toi_sync_body(d, g);
            d.b_toi_rst[g] = rst;
        }
    }
    if (moved) atomicAdd(&d.cnt->st_toi_proxies_moved, moved);
    __syncwarp();
    if (lane == 0) {
        for (uint32_t i = 0; i < S.nc; ++i) d.cs_flags[S.isl_c[i]] &= ~CF_TOI_ISL;
        for (uint32_t i = 0; i < S.nb; ++i) d.b_flags[S.isl_b[i]] &= ~BF_TOI_ISL;
        d.w_toi_ep[w] = rst;
        // sub-stepping: one event per Step (AabbTreeWorld.cpp:1819-1823); the contact
        // search after it runs with this round's
        if (d.cnt->sub_stepping) { d.w_toi[w] = 1u; d.w_incomplete[w] = 1u; }
    }
    __syncwarp();
}

__global__ void __launch_bounds__(kToiWarps * 32) k_toi_round(DW d) {
    __shared__ ToiScratch scratch[kToiWarps];
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const bool first = d.cnt->toi_rounds == 1u;
    if (d.cnt->err) return;
    for (uint32_t w = blockIdx.x * kToiWarps + wid; w < d.n_worlds; w += gridDim.x * kToiWarps) {
        if (d.w_toi[w]) continue;
        toi_world_round(d, w, scratch[wid], first, lane);
    }
}

// Before a round: the proxies the last round moved are no longer "moved".
__global__ void k_toi_clear_moved(DW d) {
    GRID_LOOP(i, d.cnt->n_moved) d.p_moved[d.moved_list[i]] = 0u;
}
__global__ void k_toi_round_reset(DW d) {
    Counters* c = d.cnt;
    c->n_moved = 0u;
    c->toi_events = 0u;
    c->toi_rounds += 1u;
}
__global__ void k_toi_moved_done(DW d) {
    Counters* c = d.cnt;
    c->need_find = c->n_moved > 0u ? 1u : 0u;
    c->n_new = 0u;
    c->toi_added_base = c->st_contacts_added;
}
// Contacts the round's search added; when there are any, the impenetrable list
// is rebuilt before the next round.
__global__ void k_toi_added(DW d) {
    Counters* c = d.cnt;
    const uint32_t added = c->st_contacts_added - c->toi_added_base;
    c->st_toi_contacts_added += added;
    c->toi_rebuild = added ? 1u : 0u;
}

// The final UpdateContacts of SolveToi (AabbTreeWorld.cpp:1827-1829).
__global__ void k_toi_update_contacts(DW d) {
    uint32_t updated = 0, skipped = 0;
    GRID_LOOP(i, d.cnt->n_live) {
        const uint32_t slot = d.c_slot[i];
        if (toi_needs_update(d, slot)) {
            update_contact(d, slot);
            d.cs_toi_ep[slot] = d.w_toi_ep[d.b_world[d.cs_body[slot].x]];  // up to date for a continued phase
            ++updated;
        } else {
            ++skipped;
        }
    }
    if (updated) atomicAdd(&d.cnt->st_toi_updated_touching, updated);
    if (skipped) atomicAdd(&d.cnt->st_toi_skipped_touching, skipped);
}

// ---- GetToiViaSat over a batch of pairs (the C ABI's prgpu_time_of_impact) ----
__global__ void k_toi_pairs(uint32_t n, const float4* vtx, const uint32_t* meta, const float* sweeps,
                            ToiLimits L, float* time, int32_t* iout) {
    GRID_LOOP(i, n) {
        Proxy P[2];
        Sweep S[2];
        for (int k = 0; k < 2; ++k) {
            const uint32_t m = meta[2 * i + k];  // vertex offset << 8 | count
            P[k].count = (int)(m & 0xffu);
            P[k].vn = vtx + (m >> 8);
            P[k].r = sweeps[(2 * i + k) * 10 + 9];
            const float* s = sweeps + (2 * i + k) * 10;
            S[k].p0 = mkpos(s[0], s[1], s[2]);
            S[k].p1 = mkpos(s[3], s[4], s[5]);
            S[k].a0 = s[6];
            S[k].lc = mk(s[7], s[8]);
        }
        const ToiOut o = toi_via_sat(P[0], S[0], P[1], S[1], L);
        time[i] = o.time;
        iout[4 * i + 0] = o.state;
        iout[4 * i + 1] = o.toi_iters;
        iout[4 * i + 2] = o.max_dist_iters;
        iout[4 * i + 3] = o.max_root_iters;
    }
}

// The impenetrable list, rebuilt when toi_rebuild is set.
void launch_toi_list(const DW& d, const Launch& L, cudaStream_t s) {
    k_toi_list_flags<<<L.grid, L.threads, 0, s>>>(d);
    scan_exclusive(L.prims, d.flags, d.scan, &d.cnt->toi_scan_n, &d.cnt->toi_imp_total, d.partial, s);
    k_toi_list_scatter<<<L.grid, L.threads, 0, s>>>(d);
    k_toi_list_done<<<1, 1, 0, s>>>(d);
}

}  // namespace

void launch_toi_begin(const DW& d, const Launch& L, cudaStream_t s) {
    launch_set_upd_phase(d, kUpdToi, s);
    k_toi_begin<<<L.grid, L.threads, 0, s>>>(d);
    launch_toi_list(d, L, s);
    k_toi_first<<<L.grid, L.threads, 0, s>>>(d);
}

void launch_toi_round(const DW& d, const Launch& L, cudaStream_t s) {
    k_toi_clear_moved<<<L.grid, L.threads, 0, s>>>(d);
    k_toi_round_reset<<<1, 1, 0, s>>>(d);
    const int blocks = (int)std::min<uint32_t>((d.n_worlds + kToiWarps - 1) / kToiWarps, (uint32_t)L.grid);
    k_toi_round<<<blocks, kToiWarps * 32, 0, s>>>(d);
    k_toi_moved_done<<<1, 1, 0, s>>>(d);
    launch_find_contacts(d, L, s);
    k_toi_added<<<1, 1, 0, s>>>(d);
    launch_toi_list(d, L, s);
}

void launch_toi_end(const DW& d, const Launch& L, cudaStream_t s) {
    k_toi_update_contacts<<<L.grid, L.threads, 0, s>>>(d);
}

cudaError_t launch_toi_pairs(uint32_t n, const float4* vtx, const uint32_t* meta, const float* sweeps,
                             const DConf& c, float* time, int32_t* iout, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const int blocks = (int)std::min<uint32_t>((n + 127) / 128, 4096u);
    k_toi_pairs<<<blocks, 128, 0, s>>>(n, vtx, meta, sweeps, toi_limits(c), time, iout);
    return cudaGetLastError();
}

}  // namespace prgpu
