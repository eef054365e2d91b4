/*
 * playrho_oracle.h -- CPU restatement of the PlayRho 2.0.0 world step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA world step is checked
 * against: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * may load it.  Nothing in the shipped library links or calls it.
 *
 * It restates, in plain C, the reference's regular-phase Step for disks, convex
 * polygons, edges and revolute joints (file:line citations are on each function
 * in playrho_oracle.c).  It follows the reference's operation order closely so
 * that the FP32 build reproduces the reference's FP32 results, and it builds a
 * second time with OR_DOUBLE for the FP64 oracle.
 *
 * Pinning: tests/test_oracle_kat.py checks it against the known-answer values
 * transcribed from the reference's own unit tests and HelloWorld expected
 * output; tests/test_oracle_vs_reference.py checks it against the reference
 * compiled from source (oracle/ref) whenever that build is available.
 */
#ifndef PLAYRHO_ORACLE_H
#define PLAYRHO_ORACLE_H

#ifdef OR_DOUBLE
typedef double or_real;
#else
typedef float or_real;
#endif

#ifdef __cplusplus
extern "C" {
#endif

enum { OR_STATIC = 0, OR_KINEMATIC = 1, OR_DYNAMIC = 2 };
enum { OR_SHAPE_DISK = 0, OR_SHAPE_POLYGON = 1, OR_SHAPE_EDGE = 2 };
enum { OR_MAXV = 16 };

/* Body flags accepted by or_add_body (subset of BodyConf booleans). */
enum {
    OR_BF_ALLOW_SLEEP = 1u,
    OR_BF_AWAKE = 2u,
    OR_BF_FIXED_ROTATION = 4u,
    OR_BF_ENABLED = 8u,
    OR_BF_BULLET = 16u, /* BodyConf::bullet: the body is impenetrable (TOI against every body) */
};

/* Mirrors the StepConf fields the step reads (StepConf.hpp:165-392): the
 * regular phase's, then the TOI phase's. */
typedef struct or_stepconf {
    or_real deltaTime, dtRatio, minStillTimeToSleep, linearSlop, angularSlop;
    or_real regResolutionRate, regMinSeparation, regMinMomentum, velocityThreshold;
    or_real maxTranslation, maxRotation, maxLinearCorrection, maxAngularCorrection;
    or_real linearSleepTolerance, angularSleepTolerance, displaceMultiplier;
    or_real aabbExtension, maxCirclesRatio;
    int regVelocityIters, regPositionIters, doWarmStart, doBlocksolve;
    or_real toiResolutionRate, toiMinSeparation, toiMinMomentum, targetDepth, tolerance;
    int toiVelocityIters, toiPositionIters, maxToiRootIters, maxToiIters, maxDistanceIters;
    int maxSubSteps, doToi;
} or_stepconf;

/* Subset of StepStats (StepStats.hpp:41-191) the oracle counts. */
typedef struct or_stepstats {
    int preProxiesCreated, preProxiesMoved, preContactsDestroyed, preContactsAdded;
    int preContactsUpdated, regIslandsFound, regIslandsSolved, regContactsAdded;
    int regContactsUpdated, regProxiesMoved, regBodiesSlept, regSumPosIters, regSumVelIters;
    or_real regMinSeparation, regMaxIncImpulse;
    /* ToiStepStats (StepStats.hpp:117-151) */
    int toiIslandsFound, toiIslandsSolved, toiContactsFound, toiContactsAtMaxSubSteps;
    int toiContactsUpdatedToi, toiContactsUpdatedTouching, toiContactsSkippedTouching;
    int toiContactsAdded, toiProxiesMoved, toiSumPosIters, toiSumVelIters;
    int toiMaxDistIters, toiMaxToiIters, toiMaxRootIters;
    or_real toiMinSeparation, toiMaxIncImpulse;
} or_stepstats;

typedef struct or_world or_world;

or_world* or_world_create(void);
void or_world_destroy(or_world* w);

/* Creates a body; returns its BodyID (creation order). */
int or_add_body(or_world* w, int type, or_real px, or_real py, or_real angle,
                or_real vx, or_real vy, or_real av, or_real ax, or_real ay, or_real aa,
                or_real linDamp, or_real angDamp, unsigned flags);
/* Creates a shape and attaches it to body; verts are already in the order the
 * reference's shape configuration stores them (hull order for polygons).
 * Returns the ShapeID. */
int or_add_shape(or_world* w, int body, int kind, int nverts, const or_real* xy,
                 or_real radius, or_real density, or_real friction, or_real restitution,
                 unsigned categoryBits, unsigned maskBits, int groupIndex, int sensor);
/* ResetMassData (WorldBody.cpp:360-400). */
void or_reset_mass(or_world* w, int body);
/* Marks shape as a child of the multi-child shape whose first child is owner
 * (kind 1: ChainShapeConf, its children edges; 2: MultiShapeConf, convex hulls);
 * the children of one shape are added consecutively, before or_reset_mass. */
void or_set_shape_owner(or_world* w, int shape, int owner, int kind);
/* Revolute joint (RevoluteJointConf).  Returns JointID. */
int or_add_revolute(or_world* w, int bodyA, int bodyB, or_real lax, or_real lay,
                    or_real lbx, or_real lby, or_real refAngle, int enableLimit,
                    or_real lower, or_real upper, int enableMotor, or_real motorSpeed,
                    or_real maxMotorTorque, int collideConnected);

/* StepConf defaults, except doToi = 0: callers ask for the TOI phase explicitly. */
/* Joint kinds of or_add_joint and their parameters extra8[]:
 *   OR_JOINT_DISTANCE  length frequency dampingRatio      (DistanceJointConf)
 *   OR_JOINT_ROPE      maxLength                          (RopeJointConf)
 *   OR_JOINT_WELD      referenceAngle frequency dampingRatio (WeldJointConf)
 *   OR_JOINT_FRICTION  maxForce maxTorque                 (FrictionJointConf)
 *   OR_JOINT_MOTOR     linearOffset.x .y angularOffset maxForce maxTorque
 *                      correctionFactor (no anchors)      (MotorJointConf)
 *   OR_JOINT_PRISMATIC localXAxisA.x .y referenceAngle lowerTranslation
 *                      upperTranslation motorSpeed maxMotorForce (PrismaticJointConf)
 *   OR_JOINT_WHEEL     localXAxisA.x .y motorSpeed maxMotorTorque frequency
 *                      dampingRatio                       (WheelJointConf)
 *   OR_JOINT_PULLEY    groundAnchorA.x .y groundAnchorB.x .y lengthA lengthB ratio
 *                                                         (PulleyJointConf)
 *   OR_JOINT_TARGET    target.x .y maxForce frequency dampingRatio; bodyA == bodyB
 *                      stands for the reference's invalid body A (TargetJointConf)
 * The axis of a prismatic or wheel joint is normalised as UnitVec::Get does;
 * or_joint_enable sets their enableLimit / enableMotor. */
enum { OR_JOINT_REVOLUTE = 0, OR_JOINT_DISTANCE = 1, OR_JOINT_ROPE = 2, OR_JOINT_WELD = 3,
       OR_JOINT_FRICTION = 4, OR_JOINT_MOTOR = 5, OR_JOINT_PRISMATIC = 6, OR_JOINT_WHEEL = 7,
       OR_JOINT_PULLEY = 8, OR_JOINT_TARGET = 9, OR_JOINT_GEAR = 10 };
int or_add_joint(or_world* w, int type, int bodyA, int bodyB, or_real lax, or_real lay, or_real lbx,
                 or_real lby, int collideConnected, const or_real* extra8);
void or_joint_enable(or_world* w, int jid, int enableLimit, int enableMotor);
/* GearJointConf from GetGearJointConf(world, joint1, joint2, ratio)
 * (GearJointConf.cpp:66-160): couples the two joints (revolute or prismatic) so
 * that coordinate1 + ratio * coordinate2 stays at its value now.  Returns JointID. */
int or_add_gear(or_world* w, int joint1, int joint2, or_real ratio);

void or_default_conf(or_stepconf* conf);
void or_step(or_world* w, const or_stepconf* conf, or_stepstats* stats);
/* SetSubStepping / IsStepComplete (AabbTreeWorld.cpp:1819-1823, :2206-2209). */
void or_set_sub_stepping(or_world* w, int flag);
int or_is_step_complete(const or_world* w);
/* BeginContact (kind 1) and EndContact (kind 2) listener calls of the last
 * or_step, in call order, as (kind, lower shape ID, higher shape ID) triples. */
int or_events(const or_world* w, int* out, int cap);
/* PreSolveContact (kind 3) / PostSolveContact (kind 4) calls of the last step:
 * per call 5 ints (kind, lower shape, higher shape, point count, iteration) and
 * 4 doubles (normal and tangent impulse of points 0 and 1). */
int or_solve_calls(const or_world* w, int* ints, double* imp, int cap);
/* Every shape the ray p1 -> p2 (up to maxF) hits, in shape order: shapes[k] and
 * hit5[5k..] = fraction, point xy, normal xy; returns the number of hits. */
int or_raycast(const or_world* w, or_real p1x, or_real p1y, or_real p2x, or_real p2y, or_real maxF, int cap,
               int* shapes, or_real* hit5);

/* Body queries. */
int or_body_count(const or_world* w);
/* out[0..12] = pos1.x pos1.y pos1.a vel.x vel.y vel.a xf.p.x xf.p.y xf.q.c xf.q.s
 *              invMass invRotI underActiveTime ; flags -> *awake */
void or_get_body(const or_world* w, int body, or_real* out13, int* awake);
void or_set_body_state(or_world* w, int body, or_real px, or_real py, or_real angle,
                       or_real vx, or_real vy, or_real av);
void or_get_local_center(const or_world* w, int body, or_real* out2);
/* Test hook with no reference counterpart: replaces the body's transformation
 * (p, q = cos sin) without touching its sweep, so that a parity check can give
 * this world exactly the transformation another implementation computed from the
 * same angle (the two sides' sin/cos may round differently).  Used on a body at
 * rest in its sweep (pos0 == pos1) before the first step. */
void or_set_body_xf(or_world* w, int body, or_real px, or_real py, or_real c, or_real s);
/* Test hook with no reference counterpart: from the next step on, each island's
 * warm start, velocity iterations and position iterations visit its contacts and
 * joints interleaved in the order of items3 (n triples: (0, shape A, shape B) for
 * the contact of two shapes, (1, joint, 0) for a joint) instead of the
 * reference's order.  Used to check a solver that sweeps constraints in another
 * valid Gauss-Seidel order (graph colours) against the same arithmetic in the
 * same order.  n = 0 restores the reference's order. */
void or_set_solve_order(or_world* w, int n, const int* items3);

/* Contact queries.  Contacts are reported in the world's container order. */
int or_contact_count(const or_world* w);
/* iout[0..11]: contactID proxyMin proxyMax bodyA shapeA childA bodyB shapeB childB
 *              touching manifoldType pointCount
 * fout[0..11]: ln.x ln.y lp.x lp.y  p0.lx p0.ly p0.ni p0.ti  p1.lx p1.ly p1.ni p1.ti
 * feat[0..7] : p0.typeA p0.indexA p0.typeB p0.indexB  p1.(same) */
void or_get_contact(const or_world* w, int k, int* iout12, or_real* fout12, int* feat8);
/* Fat AABB of proxy p (tree AABB): minx miny maxx maxy. */
int or_proxy_count(const or_world* w);
void or_get_proxy(const or_world* w, int p, int* body_shape_child3, or_real* aabb4);

/* Stand-alone narrowphase (CollideShapes, Manifold.cpp:393-438) on two shapes in
 * the oracle's shape format, for known-answer tests.  iout: type count
 * feat[8]; fout: ln.x ln.y lp.x lp.y p0.lx p0.ly p1.lx p1.ly */
void or_collide(int kindA, int nA, const or_real* xyA, or_real rA, const or_real* xfA4,
                int kindB, int nB, const or_real* xyB, or_real rB, const or_real* xfB4,
                or_real linearSlop, or_real maxCirclesRatio,
                int* type_count2, int* feat8, or_real* fout8);

/* Stand-alone GetToiViaSat (TimeOfImpact.cpp:37-253) for two shapes moving over
 * sweeps sweepN[7] = pos0.x pos0.y pos0.a pos1.x pos1.y pos1.a alpha0 with the
 * body's local centre lcN[2].  conf supplies targetDepth, tolerance and the
 * iteration limits.  iout: state toi_iters max_dist_iters max_root_iters;
 * returns the time (unit interval). */
or_real or_time_of_impact(int kindA, int nA, const or_real* xyA, or_real rA, const or_real* sweepA7,
                          const or_real* lcA2, int kindB, int nB, const or_real* xyB, or_real rB,
                          const or_real* sweepB7, const or_real* lcB2, const or_stepconf* conf, int* iout4);
/* Stand-alone Distance (Distance.cpp:96-196) from an empty cache: iout: state
 * iterations simplex-size; fout: witness point A.xy, witness point B.xy. */
void or_distance(int kindA, int nA, const or_real* xyA, or_real rA, const or_real* xfA4,
                 int kindB, int nB, const or_real* xyB, or_real rB, const or_real* xfB4,
                 int maxIters, int* iout3, or_real* fout4);

#ifdef __cplusplus
}
#endif
#endif
