// prgpu_internal.cuh -- device data layout of a batch of worlds and the shared
// device primitives (bounded grid barrier, ordered float atomics, scans, sort).
//
// Layout in HBM: every world of a batch is flattened into one structure of
// arrays.  Bodies, shapes (one proxy each) and joints of world w occupy the
// contiguous ranges [body_off[w], body_off[w+1]) etc., in creation order, so a
// global proxy index orders proxies exactly as the reference's tree leaf IDs
// order them within a world (leaf k of a tree built without removals has ID
// 0, 1, 3, 5, ...; the ranks are what ContactKey compares).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "prgpu_math.cuh"

namespace prgpu {

// Status codes of the C ABI (include/prgpu.h).
enum {
    PR_OK = 0,
    PR_EINVAL = 1,
    PR_ECUDA = 2,
    PR_ECAPACITY = 3,
    PR_ETIMEOUT = 4,
    PR_ENOTREADY = 5,
    PR_ESTATE = 6,
};

// Body flags (device).
enum : uint32_t {
    BF_TYPE_MASK = 3u,        // 0 static, 1 kinematic, 2 dynamic
    BF_AWAKE = 1u << 2,
    BF_ALLOW_SLEEP = 1u << 3,
    BF_FIXED_ROT = 1u << 4,
    BF_ENABLED = 1u << 5,
    BF_BULLET = 1u << 6,      // BodyConf::bullet: impenetrable, sub-stepped against every body
    BF_SOLVED = 1u << 8,      // in an awake island this step
    BF_MOVED = 1u << 9,       // pos1 changed in this step's solve
    BF_DIRTY = 1u << 10,      // state set by the host since the last step
    BF_TOI_ISL = 1u << 11,    // in the island of the current time-of-impact event
};

// Contact slot flags.
enum : uint32_t {
    CF_TOUCHING = 1u,
    CF_SENSOR = 2u,
    CF_NEEDS_UPDATE = 4u,
    CF_IMPENETRABLE = 8u,
    CF_TOI_VALID = 16u,       // cs_toi holds this step's time of impact (Contact::e_toiFlag)
    CF_TOI_ISL = 32u,         // in the island of the current time-of-impact event
    CF_DISABLED = 64u,        // Contact::e_enabledFlag unset (SetContact): not solved, not in islands
    CF_LIVE = 128u,           // the slot holds a live contact
};
// Phases of a step in which contacts are updated (AabbTreeWorld::Update): the
// pre-phase (UpdateContacts and AddContacts of Step), the regular phase's
// post-solve pass (SolveReg) and the time-of-impact phase.
enum : uint32_t { kUpdPre = 1u, kUpdPost = 2u, kUpdToi = 4u };

// A touching, enabled, non-sensor contact: one the islands and the solver take
// (AddToIsland, AabbTreeWorld.cpp:1433).
PR_HD bool contact_solvable(uint32_t f) { return (f & (CF_TOUCHING | CF_SENSOR | CF_DISABLED)) == CF_TOUCHING; }
// Shape meta word: kind | vertex count << 8 | these bits.
constexpr uint32_t kShapeSensor = 1u << 16;
constexpr uint32_t kShapeNoProxy = 1u << 17;  // the shape's body was disabled at creation: no proxy

// Bits 8..15 of the contact flags count the contact's TOI sub-steps this step.
constexpr uint32_t kToiCountShift = 8u;
constexpr uint32_t kToiCountMask = 0xffu << kToiCountShift;

PR_HD uint32_t body_type(uint32_t f) { return f & BF_TYPE_MASK; }
PR_HD bool is_speedable(uint32_t f) { return (f & BF_TYPE_MASK) != 0u; }
PR_HD bool is_accelerable(uint32_t f) { return (f & BF_TYPE_MASK) == 2u; }
// Body::GetFlags (Body.cpp:32-66): static and kinematic bodies, and bullets.
PR_HD bool is_impenetrable(uint32_t f) { return !is_accelerable(f) || (f & BF_BULLET) != 0u; }

constexpr int kMaxColours = 64;      // colours 0..63 solved in parallel
constexpr int kSerialColour = 64;    // leftover constraints solved by one thread
constexpr int kMaxPosIters = 32;
constexpr int kColStride = kSerialColour + 2;  // colour table of one world: offsets 0..65
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr uint32_t kJointBit = 0x80000000u;  // constraint id of a joint (else a contact slot)
constexpr uint32_t kNone = 0xffffffffu;

// Velocity constraint of one contact (VelocityConstraint.hpp) as the solver
// holds it in registers.  Point-1 and block-solver fields are zero unless
// count == 2.
struct VC {
    float nx, ny, friction, tangentSpeed;
    float rA0x, rA0y, rB0x, rB0y;
    float rA1x, rA1y, rB1x, rB1y;
    float nm0, tm0, nm1, tm1;
    float vb0, vb1, k00, k11;
    float k01, m00, m11, m01;
    float ni0, ti0, ni1, ti1;
    uint32_t bA, bB, count, island;
};

// In memory a velocity constraint is two 64-byte records at its sweep
// position t: VC0 holds what every contact needs, VC1 the second point and
// the 2x2 block-solver matrices, read only when count == 2.  A one-point
// contact so streams 64 bytes a sweep and a two-point one 128.
//   VC0: nx ny friction tangentSpeed | rA0 rB0 | nm0 tm0 vb0 count | ni0 ti0 bA bB
//   VC1: rA1 rB1 | nm1 tm1 vb1 k00 | k11 k01 m00 m11 | ni1 ti1 m01 -
struct __align__(16) VCRec {
    float4 q[4];
};

// Position constraint of one contact (PositionConstraint.hpp), 64 bytes.
struct __align__(16) PC {
    float lnx, lny, lpx, lpy;
    float p0x, p0y, p1x, p1y;
    float totalRadius;
    uint32_t type, count, bA;
    uint32_t bB, island, pad0, pad1;
};

// What one recorded step keeps for the adjoint and tangent passes (device
// arrays; K = constraint capacity, C = contact slots, N = bodies).
struct StepTape {
    float4* p0;        // [N] centre of mass x y angle at the start of the solve
    float4* v0;        // [N] velocity at the start of the solve (before k_body_begin)
    uint32_t* flags;   // [N] body flags after k_body_begin (BF_SOLVED: solved this step)
    uint8_t* slept;    // [N] put to sleep (velocity zeroed) by this step
    uint32_t* t_id;    // [K] constraint id at each sweep position (contact slot)
    PC* pc;            // [K] position constraint (local manifold, bodies, island)
    float4* cinfo;     // [K] vertex radius A, B, friction, restitution
    uint2* prox;       // [K] the contact's two proxies (shapes)
    float4* imp0;      // [K] impulses as built (ni0 ti0 ni1 ti1), before warm start
    float4* warm;      // [K*2] velocities of A and B before warm start
    float4* vel;       // [iv*K*3] velocities of A, B and impulses before each velocity solve
    float4* pos;       // [ip*K*2] positions of A and B before each position solve (A.w: 1 if solved)
    int8_t* src;       // [C*2] after the post-solve update: old point each new point took its
                       //       impulses from (-1 none; -2 slot not updated)
    uint8_t* created;  // [C] slot created by this step's post-solve contact search
    uint32_t* hdr;     // [kSerialColour + 2 + 4] colour offsets, n_colours, n_active, replay mismatches
    uint32_t* wseg;    // [W*2] first sweep position and constraint count of each world
    uint32_t* wcol;    // [W*kColStride] colour offsets of each world (relative to its first position)
    int iv, ip;        // velocity and position iterations recorded
    uint32_t kcap;
};

// Device counters and small per-step state.
struct Counters {
    uint32_t n_live;          // live contacts (sorted key list length)
    uint32_t n_new;           // new contacts found this pass
    uint32_t n_moved;         // proxies whose fat AABB moved this pass
    uint32_t n_destroyed;
    uint32_t free_top;        // entries on the free-slot stack
    uint32_t high_water;      // slots ever used
    uint32_t n_active;        // active constraints this step (contacts then joints)
    uint32_t n_active_c;
    uint32_t n_active_j;
    uint32_t n_colours;       // parallel colours used
    uint32_t colour_off[kSerialColour + 2];
    uint32_t colour_cnt[kSerialColour + 2];
    uint32_t colour_remaining;
    uint32_t err;             // first error status raised on the device
    uint32_t err_where;
    uint32_t bar_count;
    uint32_t bar_gen;
    uint32_t need_find;
    uint32_t step_no;         // steps begun (tags the contact updates and solve records of a step)
    uint32_t wait_limit;      // spins a grid-barrier wait may take (0: the default, 2^24)
    uint32_t sub_stepping;    // SetSubStepping: the TOI phase stops after one event per world
    uint32_t upd_phase;       // phase bit the contact updates are tagged with (kUpd*)
    uint32_t dirty_any;       // some body carries BF_DIRTY (host-set state since the last step)
    // StepStats counters (StepStats.hpp)
    uint32_t st_contacts_added;
    uint32_t st_contacts_destroyed;
    uint32_t st_contacts_updated;
    uint32_t st_islands_found;
    uint32_t st_islands_solved;
    uint32_t st_bodies_slept;
    uint32_t st_proxies_moved;
    uint32_t st_sum_pos_iters;
    float st_min_separation;
    float st_max_inc_impulse;
    uint32_t scan_total;
    uint32_t pad[7];
    uint32_t world_queue;     // next entry of w_order for the per-world sweep kernel
    uint32_t lbvh_age;        // searches since the tree was last rebuilt (0: no tree yet)
    uint32_t lbvh_rebuild;    // this search rebuilds the tree (else refits it)
    // time-of-impact phase
    uint32_t toi_events;      // worlds that solved an event in the current round
    uint32_t toi_rounds;      // rounds run this step
    uint32_t toi_added_base;  // st_contacts_added before the current round's contact search
    uint32_t toi_rebuild;     // rebuild the impenetrable list before the next round
    uint32_t toi_scan_n;      // entries the list's compaction scans
    uint32_t toi_imp_total;
    uint32_t n_imp;           // impenetrable contacts listed
    // ToiStepStats counters (StepStats.hpp:117-151)
    uint32_t st_toi_found;
    uint32_t st_toi_islands_found;
    uint32_t st_toi_islands_solved;
    uint32_t st_toi_sum_pos_iters;
    uint32_t st_toi_sum_vel_iters;
    uint32_t st_toi_updated_toi;
    uint32_t st_toi_at_max_substeps;
    uint32_t st_toi_updated_touching;
    uint32_t st_toi_skipped_touching;
    uint32_t st_toi_contacts_added;
    uint32_t st_toi_proxies_moved;
    uint32_t st_toi_max_dist_iters;
    uint32_t st_toi_max_toi_iters;
    uint32_t st_toi_max_root_iters;
    float st_toi_min_separation;
    float st_toi_max_inc_impulse;
    uint64_t seq_next;        // creation sequence number of the next new contact
    uint32_t st_bodies_solved;  // dynamic bodies of the awake islands this step (body-steps)
    uint32_t pad_solved;
    uint64_t body_steps;      // st_bodies_solved summed over every step since creation
};

// Solver / step configuration in device memory (mirrors prgpu_step_conf).
struct DConf {
    float deltaTime, dtRatio, minStillTimeToSleep, linearSlop, angularSlop;
    float regResolutionRate, regMinSeparation, regMinMomentum, velocityThreshold;
    float maxTranslation, maxRotation, maxLinearCorrection, maxAngularCorrection;
    float linearSleepTolerance, angularSleepTolerance, displaceMultiplier;
    float aabbExtension, maxCirclesRatio;
    int regVelocityIters, regPositionIters, doWarmStart, doBlocksolve;
    float toiResolutionRate, toiMinSeparation, toiMinMomentum, targetDepth, tolerance;
    int toiVelocityIters, toiPositionIters, maxToiRootIters, maxToiIters, maxDistanceIters;
    int maxSubSteps, doToi;
};

// All device pointers of one batch.  Passed to kernels by value.
struct DW {
    uint32_t n_worlds, n_bodies, n_shapes, n_joints, n_verts;
    uint32_t contact_cap, cand_cap, key_bits, world_bits;
    // worlds
    const uint32_t* w_body_off;
    const uint32_t* w_shape_off;
    uint32_t* w_root;        // LBVH root of each world (internal index or leaf | kLeafBit)
    const uint32_t* w_order; // worlds by decreasing body count (work order of per-world sweeps)
    uint32_t* w_kc;          // [n_worlds + 1] first active contact (index into k_list) of each world
    uint32_t* w_kj;          // [n_worlds + 1] first active joint of each world
    uint32_t* w_toi;         // [n_worlds] time-of-impact loop of the world finished this step (1)
    uint32_t* w_toi_ep;      // [n_worlds] the world's epoch counter in the TOI phase
    uint32_t* w_incomplete;  // [n_worlds] !IsStepComplete: sub-stepping stopped the world's TOI phase
                             //   after an event; its next step skips the regular phase
    uint32_t n_world_big;    // leading entries of w_order swept by a whole CTA,
    uint32_t n_world_mid;    //   then up to n_world_mid by groups of kGroupThreads threads (the rest by a warp)
    uint32_t stage_bytes;    // dynamic shared memory of the per-world solver (world body state)
    StepTape* tape;          // recording for the adjoint (device struct), else null
    float4* w_bounds;        // centroid bounds for Morton codes (ordered-int encoded)
    // bodies
    float4* b_pos1;          // cx cy angle -
    float4* b_pos0;
    float4* b_vel;           // vx vy w -
    float4* b_xf;            // px py c s
    float4* b_mass;          // invM invI lcx lcy
    float4* b_acc;           // ax ay aa -
    float2* b_damp;
    uint32_t* b_flags;
    float* b_uat;
    float* b_alpha0;         // Sweep::alpha0 (non-zero only inside the time-of-impact phase)
    uint32_t* b_toi_ep;      // TOI phase: epoch of the body's last position change (0: none)
    uint32_t* b_toi_rst;     // TOI phase: epoch at which its contacts' times of impact were voided
    const uint32_t* b_shape_off;  // body -> shapes CSR
    const uint32_t* b_shapes;
    uint32_t* b_world;
    uint32_t* b_island;      // union-find parent / island root
    uint32_t* b_jnt_off;     // body -> joints CSR (for joint collision filtering)
    uint32_t* b_jnt_other;
    uint32_t* b_jnt_cc;      // collideConnected of that joint
    // per-island data, indexed by the island's root body
    uint32_t* isl_awake;
    float* isl_sep;          // [n_bodies * kMaxPosIters] min separation per position iteration
    uint32_t* isl_jok;       // [n_bodies * kMaxPosIters] joints within tolerance
    float* isl_uat;          // min under-active time
    // shapes / proxies
    uint32_t* s_body;
    uint32_t* s_meta;        // kind | nverts << 8
    uint32_t* s_voff;
    float* s_radius;
    uint4* s_rec;            // meta, voff, radius (bits), body: the narrowphase's one 16-byte load
    float2* s_mat;           // friction restitution
    uint32_t* s_filter;      // category | mask << 16
    int32_t* s_group;        // group index; bit 30 = sensor
    float4* verts;           // vx vy nx ny
    float4* p_aabb;          // fat AABB: minx miny maxx maxy
    uint32_t* p_moved;       // 1 if the proxy's fat AABB moved this pass
    uint32_t* moved_list;
    // joints
    uint32_t* j_bodies;      // [2*J]
    float4* j_anchor;        // laA.xy laB.xy
    float4* j_param;         // ref lower upper motorSpeed
    float* j_maxtorque;
    uint32_t* j_flags;       // enableLimit | enableMotor << 1 | collideConnected << 2 | kind << 8
    const float4* j_extra;   // [2J] the other kinds' parameters (PRGPU_JOINT_* layouts)
    // [5J] gear joints: C D typeAC typeBD (bits) | ratio constant refAngleAC refAngleBD |
    // localAnchorA.xy localAnchorB.xy of AC | localXAxisA.xy of AC, localAnchorA.xy of BD |
    // localAnchorB.xy localXAxisA.xy of BD
    const float4* j_gear;
    float4* j_r;             // rA.xy rB.xy
    float4* j_m0;            // mass ex.x ex.y ex.z ey.y
    float4* j_m1;            // ey.z ez.z angularMass motorImpulse
    float4* j_m2;            // the other kinds' further solver state
    float4* j_imp;           // impulse xyz, limitState
    // contacts (slot storage)
    uint64_t* c_key;         // sorted live keys
    uint32_t* c_slot;
    uint64_t* c_key_alt;     // ping-pong buffers
    uint32_t* c_slot_alt;
    uint32_t* free_stack;
    uint2* cs_proxy;         // proxy min, proxy max
    uint2* cs_body;
    uint32_t* cs_flags;
    float2* cs_mat;          // friction restitution
    float* cs_tspeed;        // tangent speed (Contact::GetTangentSpeed; SetContact)
    uint32_t* cs_upd;        // (step_no << 3) | phases of that step in which the contact was updated
    float4* cs_post;         // solve records (while listening): impulses ni0 ti0 ni1 ti1 of the
    uint2* cs_post_tag;      //   velocity constraint; (step_no, count | iteration << 8); null: off
    uint32_t* cs_colour;     // colour the contact had in the last step (first choice next step)
    float* cs_toi;           // time of impact (valid with CF_TOI_VALID)
    uint64_t* cs_seq;        // creation sequence: orders a world's contacts as its contact list does
    uint32_t* cs_prio;       // colouring priority (a hash of the world-local proxy pair), set at creation
    uint32_t* cs_toi_ep;     // TOI phase: epoch of the contact's last Update
    uint32_t* cs_toi_at;     // TOI phase: epoch at which its time of impact was computed
    uint64_t* t_key;         // TOI phase: key-sorted list of the impenetrable contacts
    uint32_t* t_slot;
    uint32_t* j_colour;      // same for joints
    float4* m_head;          // ln.xy lp.xy
    float4* m_p0;            // lp.xy ni ti
    float4* m_p1;
    uint32_t* m_meta;        // type | count << 4
    uint2* m_cf;             // contact features of the two points
    // new-contact scratch
    uint64_t* n_key;
    uint64_t* n_key_alt;
    uint32_t* n_val;
    uint32_t* n_val_alt;
    // LBVH
    uint64_t* l_key;
    uint64_t* l_key_alt;
    uint32_t* l_idx;
    uint32_t* l_idx_alt;
    float4* l_leaf_box;
    float4* l_node_box;
    uint32_t* l_left;
    uint32_t* l_right;
    uint32_t* l_parent;      // [2S]: internal i at i, leaf k at S + k
    uint32_t* l_range;       // [2*(S-1)] first last
    uint32_t* l_visit;
    uint32_t* l_inv;         // [S] leaf of each proxy (written when the tree is rebuilt)
    uint32_t* c_first;       // [S+1] first live-list entry whose smaller proxy is >= p (each search)
    // constraints of this step
    uint32_t* k_list;        // active constraint ids (slot for contacts, joint id + J flag)
    uint32_t* k_colour;
    uint32_t* k_tent;
    uint32_t* k_prio;        // colouring priority (hash of world-local identifiers)
    uint32_t* k_order;       // constraint indices bucketed by colour (the sweep order)
    uint32_t* t_id;          // constraint id (k_list entry) at each sweep position; vc/pc share its indexing
    uint32_t* inc_off;       // body -> active constraint incidence CSR
    uint32_t* inc_cur;
    uint32_t* inc_list;
    VCRec* vc0;              // [contact capacity] velocity constraints in sweep order, first record
    VCRec* vc1;              // second record (two-point contacts)
    PC* pc;
    // scan scratch
    uint32_t* flags;
    uint32_t* scan;
    uint32_t* partial;
    uint32_t* hist;
    Counters* cnt;
    const DConf* conf;
};

// ---------------------------------------------------------------------------
// Device helpers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t float_to_ordered(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ordered_to_float(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}
__device__ __forceinline__ void atomic_min_float(float* addr, float v) {
    // Works for any sign: the ordered encoding is only used transiently in a CAS loop.
    unsigned int* a = reinterpret_cast<unsigned int*>(addr);
    unsigned int old = *a;
    for (int i = 0; i < 1 << 20; ++i) {
        const float cur = __uint_as_float(old);
        if (!(v < cur)) return;
        const unsigned int prev = atomicCAS(a, old, __float_as_uint(v));
        if (prev == old) return;
        old = prev;
    }
}
__device__ __forceinline__ void atomic_max_nonneg_float(float* addr, float v) {
    // For non-negative finite floats the IEEE bit pattern orders like the value.
    atomicMax(reinterpret_cast<unsigned int*>(addr), __float_as_uint(v));
}

// Colouring priorities hash world-local identifiers, so that a world is
// coloured the same whether it is stepped alone or in a batch.
__device__ __forceinline__ uint32_t prio_mix32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return h;
}
// The priority of the contact of proxies pa < pb (global indices).
__device__ __forceinline__ uint32_t contact_prio(const DW& d, uint32_t pa, uint32_t pb) {
    const uint32_t base = d.w_shape_off[d.b_world[d.s_body[pa]]];
    return prio_mix32(((pa - base) * 0x9E3779B1u) ^ prio_mix32(pb - base));
}

__device__ __forceinline__ void set_error(Counters* c, uint32_t code, uint32_t where) {
    if (atomicCAS(&c->err, 0u, code) == 0u) c->err_where = where;
}

// Bounded grid-wide barrier for cooperative launches.  Every spin is bounded:
// after the limit the barrier records PR_ETIMEOUT and returns; once an error is
// set all later barriers return at once so the kernel drains quickly.
__device__ __forceinline__ void grid_barrier(Counters* c) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile uint32_t* vgen = &c->bar_gen;
        volatile uint32_t* verr = &c->err;
        if (*verr == 0u) {
            const uint32_t g = *vgen;
            __threadfence();
            const uint32_t arrived = atomicAdd(&c->bar_count, 1u);
            if (arrived == gridDim.x - 1u) {
                c->bar_count = 0u;
                __threadfence();
                atomicAdd(&c->bar_gen, 1u);
            } else {
                const uint32_t limit = c->wait_limit ? c->wait_limit - 1u : (1u << 24);
                uint32_t spins = 0;
                while (*vgen == g) {
                    if (spins++ >= limit) {
                        set_error(c, PR_ETIMEOUT, 900u);
                        break;
                    }
                    if (*verr != 0u) break;
                    __nanosleep(64);
                }
            }
            __threadfence();
        }
    }
    __syncthreads();
}

// Grid-stride range over a count held in device memory.
#define GRID_LOOP(i, n) \
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

// ---------------------------------------------------------------------------
// Host-side primitives implemented in prgpu_prims.cu.
// ---------------------------------------------------------------------------
struct Prims {
    int sm_count;
    int grid;  // blocks for chunked primitives (<= 1024)
};

// Exclusive scan of in[0..*n) into out; *total receives the sum.
void scan_exclusive(const Prims& P, const uint32_t* in, uint32_t* out, const uint32_t* n, uint32_t* total,
                    uint32_t* partial, cudaStream_t s);
// Stable LSD radix sort of (key, val) pairs by the low `bits` bits of the keys.
// Returns true when the sorted result ended in the *_alt buffers.  hist holds
// kRadix * (radix_coop_grid(P) + 1) words; cnt's grid barrier separates passes.
bool radix_sort(const Prims& P, uint64_t* keys, uint64_t* keys_alt, uint32_t* vals, uint32_t* vals_alt,
                const uint32_t* n, int bits, uint32_t* hist, Counters* cnt, cudaStream_t s);
// Blocks of the cooperative sort launch (all resident at once, at most P.grid).
int radix_coop_grid(const Prims& P);

}  // namespace prgpu
