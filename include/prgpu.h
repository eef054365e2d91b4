/*
 * prgpu.h -- C ABI of the GB300 world step for PlayRho worlds.
 *
 * One handle holds a batch of one or more independent 2-D worlds resident in
 * GPU memory.  Every entry point returns an int status (PRGPU_OK = 0) and takes
 * plain pointers and sizes; host buffers belong to the caller, device buffers
 * to the handle.  The C++ world type of the PlayRho drop-in (GpuWorld) and the
 * Python bindings sit on top of these calls.
 *
 * Reference interfaces each entry point replaces (PlayRho 2.0.0 paths):
 *   prgpu_default_step_conf     StepConf defaults, Library/include/playrho/StepConf.hpp:59-161
 *   prgpu_world_create          World{} + CreateBody/CreateShape/Attach/CreateJoint,
 *                               Library/include/playrho/d2/World.hpp:739-745, :521-526;
 *                               Library/source/playrho/d2/AabbTreeWorld.cpp:1019-1044, :1132-1157, :1234-1257
 *   prgpu_step                  Step(World&, const StepConf&), World.hpp:917-920 ->
 *                               Step(AabbTreeWorld&, const StepConf&), AabbTreeWorld.cpp:2144-2219
 *   prgpu_step_n                a loop of Step calls (no per-step host synchronisation)
 *   prgpu_download_bodies       GetBody(World, BodyID) / GetTransformation / GetVelocity,
 *                               World.hpp (GetBody), AabbTreeWorld.cpp:2850
 *   prgpu_upload_body_states    SetBody(World, BodyID, Body), AabbTreeWorld.cpp:2723-2795
 *   prgpu_download_contacts     GetContacts(World) + GetContact + GetManifold,
 *                               World.hpp:563-591, AabbTreeWorld.cpp:2860-2865
 *   prgpu_download_proxies      GetTree(World) leaf AABBs, World.hpp:937
 *   prgpu_convex_hull           PolygonShapeConf::Set -> GetConvexHullAsVector,
 *                               PolygonShapeConf.cpp:120-133, DistanceProxy.cpp:62-105
 *   prgpu_time_of_impact        GetToiViaSat(proxyA, sweepA, proxyB, sweepB, ToiConf),
 *                               Library/include/playrho/d2/TimeOfImpact.hpp, TimeOfImpact.cpp:37-253
 *   prgpu_query_aabb(s)         Query(GetTree(World), AABB, callback), DynamicTree.cpp:673-710
 *   prgpu_raycast(_all)         RayCast(World, RayCastInput, callback), RayCastOutput.cpp:301-337
 *   prgpu_download_contact_seq  the contact-list (creation) order of GetContacts(World)
 *   prgpu_download_contact_state  ContactID + GetContact (enabled, friction, restitution,
 *                               tangent speed), AabbTreeWorld.cpp:2797-2832
 *   prgpu_set_contact           SetContact(World, ContactID, Contact), AabbTreeWorld.cpp:2797-2832
 *   prgpu_set_manifold          SetManifold(World, ContactID, Manifold), AabbTreeWorld.cpp:2834-2848
 *   prgpu_set_solve_records,    the arguments of the PreSolveContact / PostSolveContact
 *   prgpu_download_solve_records  listeners, AabbTreeWorld.cpp:2716-2720, :1669-1672
 *   prgpu_set_capacity_growth   the unbounded growth of the reference's contact containers
 *   prgpu_set_sub_stepping,     SetSubStepping(World, bool) / IsStepComplete(World),
 *   prgpu_get_step_complete     AabbTreeWorld.cpp:1819-1823, :2206-2209
 * The remaining entry points (schedule, autotuner, StepAdjoint, sweep order, body
 * steps, wait limit, allocation-free download) have no reference counterpart.
 */
#ifndef PRGPU_H
#define PRGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PRGPU_ABI_VERSION 5

enum prgpu_status {
    PRGPU_OK = 0,
    PRGPU_EINVAL = 1,      /* invalid argument (reference: InvalidArgument / OutOfRange) */
    PRGPU_ECUDA = 2,       /* CUDA runtime error (message via prgpu_last_error) */
    PRGPU_ECAPACITY = 3,   /* a device buffer overflowed (reference: LengthError) */
    PRGPU_ETIMEOUT = 4,    /* a bounded device wait gave up */
    PRGPU_ENOTREADY = 5,   /* no GPU or the library was built without one */
    PRGPU_ESTATE = 6       /* call not valid in the handle's state (reference: WrongState) */
};

enum prgpu_body_type { PRGPU_STATIC = 0, PRGPU_KINEMATIC = 1, PRGPU_DYNAMIC = 2 };
enum prgpu_shape_kind { PRGPU_DISK = 0, PRGPU_POLYGON = 1, PRGPU_EDGE = 2 };
/* body flags (BodyConf booleans) */
enum {
    PRGPU_BODY_ALLOW_SLEEP = 1,
    PRGPU_BODY_AWAKE = 2,
    PRGPU_BODY_FIXED_ROTATION = 4,
    PRGPU_BODY_ENABLED = 8,
    PRGPU_BODY_BULLET = 16      /* impenetrable: time-of-impact sub-stepping against every body */
};

typedef struct prgpu_world prgpu_world;

/* StepConf fields the step reads (StepConf.hpp:165-392): the regular phase's,
 * then the time-of-impact phase's.  doToi = 1 (the reference's default) runs the
 * TOI phase after the regular one; sub-stepping (one TOI event per Step) is not
 * offered: every step resolves all of its events. */
typedef struct prgpu_step_conf {
    float deltaTime, dtRatio, minStillTimeToSleep, linearSlop, angularSlop;
    float regResolutionRate, regMinSeparation, regMinMomentum, velocityThreshold;
    float maxTranslation, maxRotation, maxLinearCorrection, maxAngularCorrection;
    float linearSleepTolerance, angularSleepTolerance, displaceMultiplier;
    float aabbExtension, maxCirclesRatio;
    int32_t regVelocityIters, regPositionIters, doWarmStart, doBlocksolve;
    float toiResolutionRate, toiMinSeparation, toiMinMomentum, targetDepth, tolerance;
    int32_t toiVelocityIters, toiPositionIters, maxToiRootIters, maxToiIters, maxDistanceIters;
    int32_t maxSubSteps, doToi;
} prgpu_step_conf;

/* Subset of StepStats (StepStats.hpp:41-191), summed over the batch; the toi*
 * fields are ToiStepStats (StepStats.hpp:117-151). */
typedef struct prgpu_step_stats {
    uint32_t contactsAdded, contactsDestroyed, contactsUpdated;
    uint32_t islandsFound, islandsSolved, bodiesSlept, proxiesMoved, sumPosIters;
    uint32_t liveContacts, activeConstraints, colours, serialConstraints;
    float minSeparation, maxIncImpulse;
    uint32_t toiIslandsFound, toiIslandsSolved, toiContactsFound, toiContactsAtMaxSubSteps;
    uint32_t toiContactsUpdatedToi, toiContactsUpdatedTouching, toiContactsSkippedTouching;
    uint32_t toiContactsAdded, toiProxiesMoved, toiSumPosIters, toiSumVelIters;
    uint32_t toiMaxDistIters, toiMaxToiIters, toiMaxRootIters, toiRounds;
    float toiMinSeparation, toiMaxIncImpulse;
    uint32_t bodiesSolved;  /* dynamic bodies of the awake islands the step advanced (body-steps) */
} prgpu_step_stats;

/* A batch of worlds in creation order, flattened world-major.  Body indices in
 * shape_body / joint_bodies are global (into the flattened body arrays); each
 * world's bodies, shapes and joints are contiguous.  Polygon vertices must
 * already be in the order the reference's shape configuration stores them
 * (prgpu_convex_hull gives that order).  Mass data is derived from the shapes
 * as Attach(world, body, shape, resetMassData = true) does after each shape. */
typedef struct prgpu_batch_desc {
    uint32_t n_worlds;
    const uint32_t* world_body_count;   /* [n_worlds] */
    const uint32_t* world_shape_count;  /* [n_worlds] */
    const uint32_t* world_joint_count;  /* [n_worlds] */
    uint32_t n_bodies;
    const int32_t* body_type;           /* [n_bodies] */
    const float* body_pos;              /* [n_bodies*3] x y angle */
    const float* body_vel;              /* [n_bodies*3] vx vy w */
    const float* body_acc;              /* [n_bodies*3] ax ay alpha */
    const float* body_damp;             /* [n_bodies*2] linear angular */
    const uint32_t* body_flags;         /* [n_bodies] PRGPU_BODY_* */
    uint32_t n_shapes;
    const uint32_t* shape_body;         /* [n_shapes] */
    const int32_t* shape_kind;          /* [n_shapes] */
    const uint32_t* shape_voff;         /* [n_shapes] first vertex */
    const uint32_t* shape_nv;           /* [n_shapes] vertex count (disk 1, edge 2, polygon 3..16) */
    const float* shape_radius;          /* [n_shapes] vertex radius (disk radius) */
    const float* shape_density;
    const float* shape_friction;
    const float* shape_restitution;
    const int32_t* shape_filter;        /* [n_shapes*4] category mask group sensor */
    uint32_t n_verts;
    const float* verts;                 /* [n_verts*2] */
    uint32_t n_joints;                  /* joints (kinds in joint_type) */
    const uint32_t* joint_bodies;       /* [n_joints*2] */
    const float* joint_anchors;         /* [n_joints*4] localAnchorA.xy localAnchorB.xy */
    const float* joint_params;          /* [n_joints*6] refAngle lower upper motorSpeed maxMotorTorque - */
    const int32_t* joint_flags;         /* [n_joints*3] enableLimit enableMotor collideConnected */
    uint32_t contact_capacity;          /* 0: automatic */
    uint32_t candidate_capacity;        /* 0: automatic */
    const float* body_mass;             /* [n_bodies*4] optional invMass invRotInertia localCenter.xy of each
                                           dynamic body (SetMassData, Body.cpp); NULL: from the shapes */
    const int32_t* joint_type;          /* [n_joints] PRGPU_JOINT_*; NULL: every joint is revolute */
    const float* joint_extra;           /* [n_joints*8] parameters of the other kinds (below) */
    const int32_t* shape_owner;         /* [n_shapes] optional (ABI 4): for a child of a multi-child shape
                                           (ChainShapeConf: its edges; MultiShapeConf: its convex hulls),
                                           the index of the shape's first child, else -1.  The children
                                           of one shape are consecutive, on one body, each a shape of the
                                           batch with its own proxy (child order = proxy order); the mass
                                           data counts them as the one shape (ChainShapeConf.cpp:113-147,
                                           MultiShapeConf.cpp:35-57).  NULL: every shape has one child. */
} prgpu_batch_desc;

/* Joint kinds and their joint_extra parameters (the reference's JointConf types;
 * joint_anchors are localAnchorA.xy localAnchorB.xy, joint_flags[2] collideConnected):
 *   REVOLUTE   RevoluteJointConf: joint_params, joint_flags (extra unused)
 *   DISTANCE   DistanceJointConf: length frequency dampingRatio
 *   ROPE       RopeJointConf:     maxLength
 *   WELD       WeldJointConf:     referenceAngle frequency dampingRatio
 *   FRICTION   FrictionJointConf: maxForce maxTorque
 *   MOTOR      MotorJointConf:    linearOffset.x linearOffset.y angularOffset maxForce maxTorque
 *                                 correctionFactor (anchors unused)
 *   PRISMATIC  PrismaticJointConf: localXAxisA.x .y referenceAngle lowerTranslation
 *                                 upperTranslation motorSpeed maxMotorForce; joint_flags[0]
 *                                 enableLimit, joint_flags[1] enableMotor
 *   WHEEL      WheelJointConf:    localXAxisA.x .y motorSpeed maxMotorTorque frequency
 *                                 dampingRatio; joint_flags[1] enableMotor
 *   PULLEY     PulleyJointConf:   groundAnchorA.x .y groundAnchorB.x .y lengthA lengthB ratio
 *   TARGET     TargetJointConf:   target.x .y maxForce frequency dampingRatio; the joint has
 *                                 body B only: joint_bodies gives it twice (localAnchorA unused)
 *   GEAR       GearJointConf:     joint1 joint2 ratio [constant use-constant]: couples two
 *                                 earlier revolute or prismatic joints of the same world
 *                                 (global joint indices) as GetGearJointConf(world, joint1,
 *                                 joint2, ratio) does (GearJointConf.cpp:66-160); joint_bodies
 *                                 are joint1's and joint2's second bodies (A, B), their first
 *                                 bodies (C, D) take part too.  The constant is the joints'
 *                                 coordinates at creation unless extra[4] != 0, which gives it
 *                                 in extra[3] (a GearJointConf made earlier).
 * The axis of a prismatic or wheel joint is normalised as UnitVec::Get does. */
enum prgpu_joint_kind {
    PRGPU_JOINT_REVOLUTE = 0, PRGPU_JOINT_DISTANCE = 1, PRGPU_JOINT_ROPE = 2, PRGPU_JOINT_WELD = 3,
    PRGPU_JOINT_FRICTION = 4, PRGPU_JOINT_MOTOR = 5, PRGPU_JOINT_PRISMATIC = 6, PRGPU_JOINT_WHEEL = 7,
    PRGPU_JOINT_PULLEY = 8, PRGPU_JOINT_TARGET = 9, PRGPU_JOINT_GEAR = 10
};

int prgpu_abi_version(void);
int prgpu_default_step_conf(prgpu_step_conf* out);
/* Creates the batch on `device` (the first step creates proxies and contacts, as
 * the reference's first Step does). */
int prgpu_world_create(const prgpu_batch_desc* desc, int device, prgpu_world** out);
int prgpu_world_destroy(prgpu_world* w);
/* One world step of every world in the batch; synchronous like Step(World&).
 * stats may be NULL. */
int prgpu_step(prgpu_world* w, const prgpu_step_conf* conf, prgpu_step_stats* stats);
/* n steps replayed from a captured CUDA graph without host synchronisation;
 * returns after the last one has finished. */
int prgpu_step_n(prgpu_world* w, const prgpu_step_conf* conf, int n);
/* One step launched phase by phase (no graph) with CUDA events between the
 * phases; phase_ms[k] receives the device time of phase k:
 *   0 pre-step contact maintenance, 1 islands + colouring, 2 constraint set-up,
 *   3 Gauss-Seidel sweeps (velocity + position), 4 write-back + sleep,
 *   5 proxy synchronisation + contact update, 6 new-contact search. */
int prgpu_step_profiled(prgpu_world* w, const prgpu_step_conf* conf, float* phase_ms, int n_phases,
                        prgpu_step_stats* stats);
/* Device times of the phases of the last step replayed from the captured graph
 * (same phase numbering as prgpu_step_profiled; entry 7 is the whole step),
 * from CUDA events the graph records between its phases.  Waits for the step. */
int prgpu_last_step_phase_ms(prgpu_world* w, float* phase_ms, int n_phases);
/* Number of kernel launches in one captured step. */
int prgpu_graph_kernel_count(prgpu_world* w, uint32_t* n_kernels);
/* How the colour sweeps of the regular solve are scheduled.  GRID: one
 * cooperative launch over the whole batch, a grid barrier between colours.
 * PER_WORLD: one CTA per world, worlds taken from a queue largest first, a
 * block barrier between colours.  AUTO: PER_WORLD for batches of 64 worlds or
 * more.  Both give the same results bit for bit.  No reference counterpart
 * (the reference solves island by island on one thread). */
enum { PRGPU_SWEEPS_AUTO = 0, PRGPU_SWEEPS_GRID = 1, PRGPU_SWEEPS_PER_WORLD = 2 };
int prgpu_set_sweep_mode(prgpu_world* w, int mode);
int prgpu_get_sweep_mode(prgpu_world* w, int* mode);
/* In PER_WORLD mode, worlds of at most this many bodies are swept by one warp
 * (eight worlds at a time per CTA), larger ones by a whole CTA.  Default 256. */
int prgpu_set_warp_world_max_bodies(prgpu_world* w, uint32_t max_bodies);
int prgpu_get_warp_world_max_bodies(prgpu_world* w, uint32_t* max_bodies);
/* In PER_WORLD mode, worlds larger than the warp limit and of at most this many
 * bodies are swept by groups of 64 threads (four worlds at a time per CTA, each
 * group on a named barrier of its own); larger ones by a whole CTA.  0 (the
 * default): no groups.  Results do not depend on it. */
int prgpu_set_group_world_max_bodies(prgpu_world* w, uint32_t max_bodies);
int prgpu_get_group_world_max_bodies(prgpu_world* w, uint32_t* max_bodies);
/* A sweep schedule and its measured device time per step. */
/* Shared memory (bytes, a multiple of 128) in which the per-world solver
 * keeps the velocities and positions of the world it sweeps, 44 bytes a body
 * (a warp gets an eighth); larger worlds are swept in global memory.  0 (the
 * default) disables staging.  Results do not depend on it. */
int prgpu_set_stage_bytes(prgpu_world* w, uint32_t bytes);
int prgpu_get_stage_bytes(prgpu_world* w, uint32_t* bytes);
typedef struct prgpu_schedule {
    int32_t sweep_mode;               /* PRGPU_SWEEPS_GRID or PRGPU_SWEEPS_PER_WORLD */
    uint32_t warp_world_max_bodies;
    uint32_t stage_bytes;
    float step_ms;
    uint32_t group_world_max_bodies;  /* ABI 5 */
} prgpu_schedule;
/* Autotuner: times every candidate schedule over steps_per_candidate steps
 * (after one untimed step that captures it), times the 3 fastest once more,
 * and keeps the fastest (each candidate by its faster timing).  A batch of one
 * world has 1 candidate, a batch of several 22 (25 timings).  The schedules give
 * identical results, so the only effect on the simulation is that the world
 * advances (1 + steps_per_candidate) steps per timing, as with prgpu_step_n.
 * No reference counterpart. */
int prgpu_autotune(prgpu_world* w, const prgpu_step_conf* conf, int steps_per_candidate, prgpu_schedule* best);
/* StepAdjoint: gradients of a loss of the state after a window of steps with
 * respect to the state before it and to the shapes' friction.  No reference
 * counterpart.  The derivative is that of the step with its discrete decisions
 * frozen as the forward pass took them (contact set, clamps, block-solver cases,
 * island early exits, sleep) and each manifold's local geometry held constant
 * within a step.  Revolute joints take part through their point rows; joints with
 * a limit or a motor are rejected (PRGPU_EINVAL).
 *   prgpu_adjoint_begin     opens a window; the state is checkpointed every
 *                           checkpoint_every steps (device copies of the whole batch)
 *   prgpu_adjoint_forward   n steps with one StepConf, as prgpu_step_n; the steps
 *                           of the window's last segment (as of this call) are
 *                           recorded as they run
 *   prgpu_adjoint_backward  from d(loss)/d(final state) -- positions x y angle of
 *                           each body's centre of mass and velocities, [n_bodies*3],
 *                           either may be NULL -- to d(loss)/d(state at the window's
 *                           start) and d(loss)/d(friction of each shape) [n_shapes];
 *                           each segment is re-run from its checkpoint to record it
 *                           (the last one only if the forward pass did not record
 *                           it), then walked backwards; the batch is left at the
 *                           window's end.  The position and velocity gradients are
 *                           the same on every run (friction gradients are summed
 *                           with float atomics and may differ in the last bits)
 *   prgpu_adjoint_tangent   the FP64 forward-mode derivative along the same window
 *                           (tangents of the start state and friction in, of the
 *                           final state out), for dot-product tests of the adjoint
 *   prgpu_adjoint_info      steps in the window, recorded steps whose constraint
 *                           set-up the differentiable restatement did not reproduce
 *                           bit for bit, or whose re-run did not end where the
 *                           forward went on (0 expected), and a count kept at 0
 *                           (the reverse pass keeps no bounded local tapes)
 *   prgpu_adjoint_end       closes the window; its device memory stays cached
 *                           for the next window of the same sizes
 *   prgpu_adjoint_trim      frees the cached memory of closed windows
 * Host calls that change bodies (prgpu_upload_body_states) inside a window are
 * not recorded and make the gradients meaningless. */
int prgpu_adjoint_begin(prgpu_world* w, int checkpoint_every);
int prgpu_adjoint_forward(prgpu_world* w, const prgpu_step_conf* conf, int n_steps);
int prgpu_adjoint_backward(prgpu_world* w, const float* dl_dpos3, const float* dl_dvel3, float* dl_dpos3_start,
                           float* dl_dvel3_start, float* dl_dfriction);
int prgpu_adjoint_tangent(prgpu_world* w, const double* dpos3_start, const double* dvel3_start, const double* dfriction,
                          double* dpos3_end, double* dvel3_end);
int prgpu_adjoint_info(prgpu_world* w, int* steps, uint32_t* replay_mismatches, uint32_t* tape_overflows);
int prgpu_adjoint_end(prgpu_world* w);
int prgpu_adjoint_trim(void);
/* Host time (ms) of the window's forward steps (the recording of the last
 * segment included) and of the last backward pass's recording (segments re-run
 * from their checkpoints) and reverse kernels. */
int prgpu_adjoint_profile(prgpu_world* w, double* forward_ms, double* record_ms, double* reverse_ms);
/* Enqueues n steps on the handle's stream and returns at once.  A device error
 * raised by an earlier step (capacity overflow, a bounded wait that gave up) is
 * returned by the next prgpu_step_async once that step has finished, and by
 * prgpu_synchronize, which waits for all of them. */
int prgpu_step_async(prgpu_world* w, const prgpu_step_conf* conf, int n);
int prgpu_synchronize(prgpu_world* w);
/* Body-steps since the handle was created: the dynamic bodies of awake islands
 * summed over every step the device ran (sleeping and static bodies are not
 * counted).  Waits for the handle's work.  No reference counterpart (the
 * throughput unit of the batched step). */
int prgpu_get_body_steps(prgpu_world* w, uint64_t* total);
int prgpu_get_counts(prgpu_world* w, uint32_t* n_worlds, uint32_t* n_bodies, uint32_t* n_shapes,
                     uint32_t* n_joints, uint32_t* n_contacts);
/* Body state; any pointer may be NULL.  flags: bit0 awake.  mass: invM invI lcx lcy. */
int prgpu_download_bodies(prgpu_world* w, float* pos3, float* vel3, float* xf4, float* mass4,
                          float* under_active, uint32_t* flags);
/* Sets positions (x y angle of the centre of mass) and velocities of bodies
 * [first, first+count); unchanged transforms are left alone, changed ones are
 * re-synchronised before the next step (SetBody semantics). */
int prgpu_upload_body_states(prgpu_world* w, uint32_t first, uint32_t count, const float* pos3, const float* vel3);
/* Live contacts in ContactKey order.  Any array may be NULL; n_out receives the count.
 *   proxies2: proxy min, proxy max (global shape indices)   bodies2: body A, body B
 *   flags: bit0 touching, bit1 sensor                        meta2: manifold type, point count
 *   head4: local normal xy, local point xy                   pts8: per point local xy, normal and
 *   tangent impulse                                          features2: packed ContactFeature of each point
 *   (typeA | indexA << 8 | typeB << 16 | indexB << 24) */
int prgpu_download_contacts(prgpu_world* w, uint32_t capacity, uint32_t* n_out, uint32_t* proxies2,
                            uint32_t* bodies2, uint32_t* flags, int32_t* meta2, float* head4, float* pts8,
                            uint32_t* features2);
/* Query(tree, aabb, callback) over one world's broadphase tree (DynamicTree.cpp:673-710):
 * the world-local shape IDs whose fat AABB overlaps `aabb` (minx miny maxx maxy), by
 * TestOverlap, in ascending order (the reference visits them in tree order).  The
 * walk runs on the world's subtree of the step's LBVH.  Valid after the first step,
 * which creates the proxies; more than `capacity` overlaps returns PRGPU_ECAPACITY
 * with *n_out set. */
int prgpu_query_aabb(prgpu_world* w, uint32_t world, const float* aabb4, uint32_t capacity, uint32_t* n_out,
                     uint32_t* shapes);
/* n queries at once, one thread per query: query k takes worlds[k] and
 * aabb4[4k..4k+3]; counts[k] = its number of overlaps and shapes[k*capacity ..]
 * its first min(counts[k], capacity) shape IDs, ascending.  shapes may be NULL
 * (counts only); PRGPU_ECAPACITY if a query has more than capacity overlaps. */
int prgpu_query_aabbs(prgpu_world* w, uint32_t n, const uint32_t* worlds, const float* aabb4, uint32_t capacity,
                      uint32_t* counts, uint32_t* shapes);
/* RayCast(World, RayCastInput, callback) (RayCastOutput.cpp:241-337) with a
 * callback that answers RayCastOpcode::ClipRay to every hit, for n rays at once:
 * ray k in worlds[k] from p1 to p2 up to maxFraction (rays5[5k..] = p1x p1y p2x
 * p2y maxFraction).  shapes[k] = the world-local shape of its nearest hit (-1:
 * none; ties go to the lower shape ID, where the reference's answer depends on
 * its tree order) and hits5[5k..] = fraction, point x y (p1 + (p2 - p1) *
 * fraction), normal x y, as the shape RayCast (RayCastOutput.cpp:41-233)
 * computes them.  Valid after the first step. */
int prgpu_raycast(prgpu_world* w, uint32_t n, const uint32_t* worlds, const float* rays5, int32_t* shapes,
                  float* hits5);
/* The same ray with a callback that answers RayCastOpcode::ResetRay: every shape
 * the ray hits, ascending by shape ID, with hits5 as above; *n_out = their
 * number; PRGPU_ECAPACITY if more than capacity (shapes and hits5 may be NULL to
 * count). */
int prgpu_raycast_all(prgpu_world* w, uint32_t world, const float* ray5, uint32_t capacity, uint32_t* n_out,
                      int32_t* shapes, float* hits5);
/* The creation sequence number of each live contact, in the order of
 * prgpu_download_contacts.  Sorting a world's contacts by it gives the order of the
 * reference's contact list (AabbTreeWorld::m_contacts), the order in which Step
 * updates contacts and calls the BeginContact / EndContact listeners
 * (AabbTreeWorld.cpp:2333-2415, 2703-2714); a contact destroyed and created again
 * gets a new number. */
int prgpu_download_contact_seq(prgpu_world* w, uint32_t capacity, uint32_t* n_out, uint64_t* seq);
/* prgpu_download_contacts for callers that must not allocate device memory once
 * running (a real-time loop that forbids allocation in its steady state, or a
 * process whose device memory is held by another framework's caching allocator,
 * where a new allocation fails or stalls).  It has no counterpart in the
 * reference; it exists for those callers only.  Same arguments and results as
 * prgpu_download_contacts, but the device gather goes through one fixed array
 * of at most 65,536 contacts (84 bytes each, 5.5 MB) that the library declares
 * in device memory: every GPU that loads the library holds that array until the
 * process exits, and no cudaMalloc, cudaFree or allocating library routine is
 * called.  More live contacts than that limit returns PRGPU_ECAPACITY with a
 * message.  The first call on a device looks up the array's device address
 * (with that device current), so make it before any stream capture.  All calls
 * share the one array and it keeps the last call's contents: calls whose work
 * overlaps on the GPU (several handles or threads at once) race on it. */
int prgpu_download_contacts_noalloc(prgpu_world* w, uint32_t capacity, uint32_t* n_out, uint32_t* proxies2,
                                    uint32_t* bodies2, uint32_t* flags, int32_t* meta2, float* head4, float* pts8,
                                    uint32_t* features2);
/* Contact identities and the contact fields a caller may change, for every live
 * contact in the order of prgpu_download_contacts:
 *   slots[i]   the contact's slot: its ContactID, stable for the contact's life and
 *              reused after it is destroyed, as the reference's ObjectPool reuses IDs
 *              (AabbTreeWorld.cpp:2423-2547 AddContacts, :2290-2331 DestroyContacts)
 *   mat4[4i..] friction, restitution, tangent speed, enabled (1 or 0) (Contact.hpp)
 * Either array may be NULL. */
int prgpu_download_contact_state(prgpu_world* w, uint32_t capacity, uint32_t* n_out, uint32_t* slots, float* mat4);
/* Capacity growth (off by default).  The reference's contact containers grow
 * without bound; a batch holds contact_capacity contacts and candidate_capacity
 * new pairs per search, and a step that runs out raises PRGPU_ECAPACITY with its
 * state already advanced without the contacts it could not hold.  With growth on,
 * prgpu_step and prgpu_step_n keep the state before each step on the device (one
 * copy of the batch's persistent arrays), and a step that runs out is undone,
 * both capacities double (up to 16 times) and the step runs again, with the same
 * result as with the larger capacities from the start.  prgpu_step_async and
 * prgpu_step_profiled do not grow.  Not inside an adjoint window. */
int prgpu_set_capacity_growth(prgpu_world* w, int enabled);
int prgpu_get_capacities(prgpu_world* w, uint32_t* contacts, uint32_t* candidates);
/* SetSubStepping(World, flag) (AabbTreeWorld.hpp; the TOI loop's break at
 * AabbTreeWorld.cpp:1819-1823): with it on, each world's time-of-impact phase
 * stops after one event and the world's step is left incomplete; the next step
 * skips that world's regular phase (IsStepComplete, :2206-2209) and continues its
 * time-of-impact phase, until a phase finds no event.  Off by default. */
int prgpu_set_sub_stepping(prgpu_world* w, int enabled);
/* IsStepComplete(World) for one world of the batch: 1, or 0 while sub-stepping
 * left its time-of-impact phase unfinished. */
int prgpu_get_step_complete(prgpu_world* w, uint32_t world, int* complete);
/* Spins a grid-wide barrier wait may take before it gives up, records
 * PRGPU_ETIMEOUT in the device error word and lets the kernel drain (0 restores
 * the default of 2^24; 1 gives up at the first wait).  For failure tests of the
 * bounded waits. */
int prgpu_set_wait_limit(prgpu_world* w, uint32_t spins);
/* Records for the PreSolveContact / PostSolveContact listeners
 * (ContactManifoldFunction, ContactImpulsesFunction; called by the reference at
 * AabbTreeWorld.cpp:2716-2720 and :1669-1672).  Enabling keeps, for every contact
 * the regular phase solves, its velocity constraint's impulses and its island's
 * iteration argument; it allocates 24 bytes per contact slot on first use and
 * re-captures the step.  Off by default. */
int prgpu_set_solve_records(prgpu_world* w, int enabled);
/* The live contacts the last step updated (AabbTreeWorld::Update) or solved, in no
 * particular order (*n_out of them; with every array NULL only *n_out is set):
 *   slots[i]     the contact's slot
 *   info[i]      bits 0-2: phases that updated it (1: the step's pre-phase,
 *                UpdateContacts and AddContacts, :2186-2198; 2: the regular phase's
 *                post-solve pass, :1549-1557; 4: the time-of-impact phase);
 *                bit 3: solved by the regular phase (needs prgpu_set_solve_records);
 *                bits 4-7: its velocity constraint's point count; bits 8-15: the
 *                iteration argument (the position iteration at which the island
 *                reached tolerance, else 255 = StepConf::InvalidIteration)
 *   imp4[4i..]   the solved normal and tangent impulses of points 0 and 1
 *                (GetContactImpulses, ContactImpulsesList.cpp:28-38)
 * PRGPU_ECAPACITY (with *n_out set) if there are more than capacity records. */
int prgpu_download_solve_records(prgpu_world* w, uint32_t capacity, uint32_t* n_out, uint32_t* slots, uint32_t* info,
                                 float* imp4);
/* SetContact(World&, ContactID, Contact) (AabbTreeWorld.cpp:2797-2832) for the
 * fields the step reads: a disabled contact stays out of the islands and the
 * solver (AabbTreeWorld.cpp:1433) and out of the time-of-impact phase
 * (:1696, :2106) until it is enabled again; friction, restitution and tangent
 * speed are used from the next step's velocity constraints (:321-357).
 * PRGPU_EINVAL if the slot holds no live contact. */
int prgpu_set_contact(prgpu_world* w, uint32_t slot, int enabled, float friction, float restitution,
                      float tangent_speed);
/* SetManifold(World&, ContactID, Manifold) (AabbTreeWorld.cpp:2834-2848): the
 * manifold's type and point count must stay (else PRGPU_EINVAL); head4 = local
 * normal xy, local point xy; pts8 = per point local xy, normal and tangent impulse.
 * The contact features are kept. */
int prgpu_set_manifold(prgpu_world* w, uint32_t slot, int32_t type, int32_t count, const float* head4,
                       const float* pts8);
/* Fat (tree) AABB of every proxy: minx miny maxx maxy.  A shape without a proxy
 * (its body was created disabled, AabbTreeWorld.cpp:1040) reports an empty box
 * (min +inf, max -inf). */
int prgpu_download_proxies(prgpu_world* w, float* aabb4);
/* The order in which the last step's regular-phase solve swept its constraints
 * (warm start, velocity and position iterations all follow it), world by world:
 * items3[3t..3t+2] = (0, shape A, shape B) for the contact of two shapes (global
 * shape indices, lower first) or (1, joint, 0) for a joint (global joint index).
 * No reference counterpart: the reference solves each island in its own order
 * (ContactSolver.cpp, AabbTreeWorld.cpp:1563-1683); this order is a valid
 * Gauss-Seidel order of the same constraints (graph colours), reported so that
 * parity checks can replay it.  Valid after a step without the time-of-impact
 * phase, until the next step.  With items3 NULL only *n_out is set. */
int prgpu_download_sweep_order(prgpu_world* w, uint32_t capacity, uint32_t* n_out, int32_t* items3);
/* Runs the host-side part of prgpu_world_create (validation, mass data as
 * Attach(..., resetMassData = true) leaves it) without a GPU: centre-of-mass
 * positions, velocities and invM invI lcx lcy of every body.  Any output may be NULL. */
int prgpu_prepare_bodies(const prgpu_batch_desc* desc, float* pos3, float* vel3, float* mass4);
/* Copies the last error message into buf. */
int prgpu_last_error(prgpu_world* w, char* buf, int len);
/* Vertex order of PolygonShapeConf::Set (VertexSet de-duplication + gift wrap);
 * returns the hull vertex count written to out_xy (capacity n). */
int prgpu_convex_hull(const float* xy, int n, float linear_slop, float* out_xy);
/* GetToiViaSat on the GPU for n pairs of convex shapes moving over sweeps, with
 * conf's targetDepth, tolerance, maxToiRootIters, maxToiIters and
 * maxDistanceIters.  Pair i is shapes 2i (A) and 2i+1 (B):
 *   nverts[2n]       vertex count (disk 1, edge 2, polygon 3..16)
 *   verts            the shapes' vertices, x y pairs, one shape after another
 *   radius[2n]       vertex radius
 *   sweeps[2n*9]     pos0 x y angle, pos1 x y angle, alpha0, localCenter x y
 * time_out[n] receives the time in [0, 1]; iout4[n*4] receives the ToiOutput
 * state (0 unknown 1 overlapped 2 touching 3 separated 4 maxRootIters
 * 5 nextAfter 6 maxToiIters 7 belowMinTarget 8 maxDistIters
 * 9 targetDepthExceedsTotalRadius 10 minTargetSquaredOverflow
 * 11 maxTargetSquaredOverflow), TOI iterations, the most distance iterations
 * and the most root-finder iterations.  Host buffers; runs on `device`. */
int prgpu_time_of_impact(int device, uint32_t n, const uint32_t* nverts, const float* verts, const float* radius,
                         const float* sweeps, const prgpu_step_conf* conf, float* time_out, int32_t* iout4);

#ifdef __cplusplus
}
#endif
#endif
