// GpuWorld.cpp -- PlayRho value types to and from the HostWorld records, and the
// free functions World's WorldModel<GpuWorld> calls.
#include "GpuWorld.hpp"

#include <algorithm>
#include <cmath>
#include <string>

#include "playrho/InvalidArgument.hpp"
#include "playrho/LengthError.hpp"
#include "playrho/OutOfRange.hpp"
#include "playrho/WrongState.hpp"
#include "playrho/d2/DiskShapeConf.hpp"
#include "playrho/d2/EdgeShapeConf.hpp"
#include "playrho/d2/PolygonShapeConf.hpp"
#include "playrho/d2/ChainShapeConf.hpp"
#include "playrho/d2/MultiShapeConf.hpp"
#include "playrho/d2/DistanceJointConf.hpp"
#include "playrho/d2/FrictionJointConf.hpp"
#include "playrho/d2/GearJointConf.hpp"
#include "playrho/d2/MotorJointConf.hpp"
#include "playrho/d2/PrismaticJointConf.hpp"
#include "playrho/d2/PulleyJointConf.hpp"
#include "playrho/d2/RevoluteJointConf.hpp"
#include "playrho/d2/RopeJointConf.hpp"
#include "playrho/d2/TargetJointConf.hpp"
#include "playrho/d2/WeldJointConf.hpp"
#include "playrho/d2/WheelJointConf.hpp"

namespace playrho::d2 {

namespace {

float F(Real v) { return static_cast<float>(v); }

// The C ABI's status codes as the reference's exception types.
[[noreturn]] void Rethrow(const prgpu::Error& e) {
    switch (e.code) {
    case PRGPU_EINVAL: throw InvalidArgument(e.what());
    case PRGPU_ECAPACITY: throw LengthError(e.what());
    case PRGPU_ESTATE: throw WrongState(e.what());
    default: throw std::runtime_error(e.what());
    }
}

template <class F_>
auto Guard(F_&& f) -> decltype(f()) {
    try {
        return f();
    } catch (const prgpu::Error& e) {
        Rethrow(e);
    }
}

void CheckUnlocked(const GpuWorld& w) {
    if (w.locked) throw WrongState("world is locked");
}

// Body -> HostBody over `base` (the current record), keeping base's position or
// velocity where `value` leaves them as `before` had them, so that a
// GetBody/SetBody round trip uploads nothing.
prgpu::HostBody ToHost(const Body& value, const Body* before, const prgpu::HostBody& base) {
    prgpu::HostBody h = base;
    h.type = static_cast<int32_t>(GetType(value));
    const auto loc = GetLocation(value);
    const auto ang = GetAngle(value);
    const bool moved = !before || GetLocation(*before) != loc || GetAngle(*before) != ang;
    if (moved) {
        h.x = F(StripUnit(GetX(loc)));
        h.y = F(StripUnit(GetY(loc)));
        h.angle = F(StripUnit(ang));
    }
    const auto vel = GetVelocity(value);
    const bool vchanged = !before || GetVelocity(*before) != vel;
    if (vchanged) {
        h.vx = F(StripUnit(GetX(vel.linear)));
        h.vy = F(StripUnit(GetY(vel.linear)));
        h.w = F(StripUnit(vel.angular));
    }
    const auto acc = GetAcceleration(value);
    h.ax = F(StripUnit(GetX(acc.linear)));
    h.ay = F(StripUnit(GetY(acc.linear)));
    h.aa = F(StripUnit(acc.angular));
    h.linear_damping = F(StripUnit(GetLinearDamping(value)));
    h.angular_damping = F(StripUnit(GetAngularDamping(value)));
    uint32_t flags = 0;
    if (IsSleepingAllowed(value)) flags |= PRGPU_BODY_ALLOW_SLEEP;
    if (IsAwake(value)) flags |= PRGPU_BODY_AWAKE;
    if (IsFixedRotation(value)) flags |= PRGPU_BODY_FIXED_ROTATION;
    if (IsEnabled(value)) flags |= PRGPU_BODY_ENABLED;
    if (IsImpenetrable(value) && GetType(value) == BodyType::Dynamic) flags |= PRGPU_BODY_BULLET;
    h.flags = flags;
    // the mass data the reference computed (ResetMassData / SetMassData)
    h.explicit_mass = true;
    h.inv_mass = F(StripUnit(GetInvMass(value)));
    h.inv_rot_inertia = F(StripUnit(GetInvRotInertia(value)));
    const auto lc = GetLocalCenter(value);
    h.lcx = F(StripUnit(GetX(lc)));
    h.lcy = F(StripUnit(GetY(lc)));
    h.shapes.clear();
    for (const auto& s : GetShapes(value)) h.shapes.push_back(to_underlying(s));
    return h;
}

prgpu::HostShape ToHost(const Shape& shape) {
    prgpu::HostShape h;
    auto base = [&h](const auto& conf) {
        h.friction = F(conf.friction);
        h.restitution = F(conf.restitution);
        h.density = F(StripUnit(conf.density));
        h.category = static_cast<int32_t>(conf.filter.categoryBits);
        h.mask = static_cast<int32_t>(conf.filter.maskBits);
        h.group = static_cast<int32_t>(conf.filter.groupIndex);
        h.sensor = conf.isSensor ? 1 : 0;
    };
    if (const auto* c = TypeCast<DiskShapeConf>(&shape)) {
        base(*c);
        h.kind = PRGPU_DISK;
        h.radius = F(StripUnit(c->vertexRadius));
        h.verts = {F(StripUnit(GetX(c->location))), F(StripUnit(GetY(c->location)))};
    } else if (const auto* c = TypeCast<PolygonShapeConf>(&shape)) {
        base(*c);
        h.kind = PRGPU_POLYGON;
        h.radius = F(StripUnit(c->vertexRadius));
        for (const auto& v : c->ngon.GetVertices()) {
            h.verts.push_back(F(StripUnit(GetX(v))));
            h.verts.push_back(F(StripUnit(GetY(v))));
        }
    } else if (const auto* c = TypeCast<EdgeShapeConf>(&shape)) {
        base(*c);
        h.kind = PRGPU_EDGE;
        h.radius = F(StripUnit(c->vertexRadius));
        h.verts = {F(StripUnit(GetX(c->GetVertexA()))), F(StripUnit(GetY(c->GetVertexA()))),
                   F(StripUnit(GetX(c->GetVertexB()))), F(StripUnit(GetY(c->GetVertexB())))};
    } else if (TypeCast<ChainShapeConf>(&shape) || TypeCast<MultiShapeConf>(&shape)) {
        // each child (an edge of a chain, a convex hull of a multi shape) becomes a
        // shape of the batch with its own proxy, as the reference gives each child one
        const bool chain = TypeCast<ChainShapeConf>(&shape) != nullptr;
        if (chain) base(*TypeCast<ChainShapeConf>(&shape));
        else base(*TypeCast<MultiShapeConf>(&shape));
        h.kind = chain ? PRGPU_EDGE : PRGPU_POLYGON;
        const auto n = GetChildCount(shape);
        if (n == 0) throw InvalidArgument("GpuWorld: a shape without children");
        for (ChildCounter i = 0; i < n; ++i) {
            const auto child = GetChild(shape, i);
            const auto nv = child.GetVertexCount();
            if ((chain && nv != 2) || (!chain && nv < 3))
                throw InvalidArgument("GpuWorld: chain children must be edges, multi-shape children polygons");
            h.radius = F(StripUnit(child.GetVertexRadius()));
            std::vector<float> v;
            for (auto k = decltype(nv){0}; k < nv; ++k) {
                v.push_back(F(StripUnit(GetX(child.GetVertex(k)))));
                v.push_back(F(StripUnit(GetY(child.GetVertex(k)))));
            }
            h.children.push_back(std::move(v));
        }
    } else {
        throw InvalidArgument("GpuWorld: only disk, polygon, edge, chain and multi shapes are stepped on the GPU");
    }
    return h;
}

// The joint kinds the GPU steps, with their parameters in HostJoint::extra in the
// order prgpu.h gives (DistanceJointConf.hpp:102-116, RopeJointConf.hpp:89-95,
// WeldJointConf.hpp:104-119, FrictionJointConf.hpp:97-106, MotorJointConf.hpp:114-129,
// PrismaticJointConf.hpp:131-159, WheelJointConf.hpp:132-150, PulleyJointConf.hpp:100-126,
// TargetJointConf.hpp:119-140).
prgpu::HostJoint ToHost(const Joint& joint) {
    prgpu::HostJoint h;
    const auto common = [&h](const auto& c) {
        h.body_a = to_underlying(c.bodyA);
        h.body_b = to_underlying(c.bodyB);
        h.collide_connected = c.collideConnected ? 1 : 0;
    };
    const auto anchors = [&h](const auto& c) {
        h.anchor_a[0] = F(StripUnit(GetX(c.localAnchorA))); h.anchor_a[1] = F(StripUnit(GetY(c.localAnchorA)));
        h.anchor_b[0] = F(StripUnit(GetX(c.localAnchorB))); h.anchor_b[1] = F(StripUnit(GetY(c.localAnchorB)));
    };
    if (const auto* c = TypeCast<RevoluteJointConf>(&joint)) {
        common(*c); anchors(*c);
        h.kind = PRGPU_JOINT_REVOLUTE;
        h.reference_angle = F(StripUnit(c->referenceAngle));
        h.lower = F(StripUnit(c->lowerAngle));
        h.upper = F(StripUnit(c->upperAngle));
        h.motor_speed = F(StripUnit(c->motorSpeed));
        h.max_motor_torque = F(StripUnit(c->maxMotorTorque));
        h.enable_limit = c->enableLimit ? 1 : 0;
        h.enable_motor = c->enableMotor ? 1 : 0;
    } else if (const auto* c = TypeCast<DistanceJointConf>(&joint)) {
        common(*c); anchors(*c);
        h.kind = PRGPU_JOINT_DISTANCE;
        h.extra[0] = F(StripUnit(c->length));
        h.extra[1] = F(StripUnit(Frequency{c->frequency}));
        h.extra[2] = F(c->dampingRatio);
    } else if (const auto* c = TypeCast<RopeJointConf>(&joint)) {
        common(*c); anchors(*c);
        h.kind = PRGPU_JOINT_ROPE;
        h.extra[0] = F(StripUnit(c->maxLength));
    } else if (const auto* c = TypeCast<WeldJointConf>(&joint)) {
        common(*c); anchors(*c);
        h.kind = PRGPU_JOINT_WELD;
        h.extra[0] = F(StripUnit(c->referenceAngle));
        h.extra[1] = F(StripUnit(Frequency{c->frequency}));
        h.extra[2] = F(c->dampingRatio);
    } else if (const auto* c = TypeCast<FrictionJointConf>(&joint)) {
        common(*c); anchors(*c);
        h.kind = PRGPU_JOINT_FRICTION;
        h.extra[0] = F(StripUnit(Force{c->maxForce}));
        h.extra[1] = F(StripUnit(Torque{c->maxTorque}));
    } else if (const auto* c = TypeCast<MotorJointConf>(&joint)) {
        common(*c);
        h.kind = PRGPU_JOINT_MOTOR;
        h.extra[0] = F(StripUnit(GetX(c->linearOffset)));
        h.extra[1] = F(StripUnit(GetY(c->linearOffset)));
        h.extra[2] = F(StripUnit(c->angularOffset));
        h.extra[3] = F(StripUnit(Force{c->maxForce}));
        h.extra[4] = F(StripUnit(Torque{c->maxTorque}));
        h.extra[5] = F(c->correctionFactor);
    } else if (const auto* c = TypeCast<PrismaticJointConf>(&joint)) {
        common(*c); anchors(*c);
        h.kind = PRGPU_JOINT_PRISMATIC;
        h.extra[0] = F(GetX(c->localXAxisA));
        h.extra[1] = F(GetY(c->localXAxisA));
        h.extra[2] = F(StripUnit(c->referenceAngle));
        h.extra[3] = F(StripUnit(c->lowerTranslation));
        h.extra[4] = F(StripUnit(c->upperTranslation));
        h.extra[5] = F(StripUnit(c->motorSpeed));
        h.extra[6] = F(StripUnit(c->maxMotorForce));
        h.enable_limit = c->enableLimit ? 1 : 0;
        h.enable_motor = c->enableMotor ? 1 : 0;
    } else if (const auto* c = TypeCast<WheelJointConf>(&joint)) {
        common(*c); anchors(*c);
        h.kind = PRGPU_JOINT_WHEEL;
        h.extra[0] = F(GetX(c->localXAxisA));
        h.extra[1] = F(GetY(c->localXAxisA));
        h.extra[2] = F(StripUnit(c->motorSpeed));
        h.extra[3] = F(StripUnit(c->maxMotorTorque));
        h.extra[4] = F(StripUnit(Frequency{c->frequency}));
        h.extra[5] = F(c->dampingRatio);
        h.enable_motor = c->enableMotor ? 1 : 0;
    } else if (const auto* c = TypeCast<PulleyJointConf>(&joint)) {
        common(*c); anchors(*c);
        h.kind = PRGPU_JOINT_PULLEY;
        h.extra[0] = F(StripUnit(GetX(c->groundAnchorA))); h.extra[1] = F(StripUnit(GetY(c->groundAnchorA)));
        h.extra[2] = F(StripUnit(GetX(c->groundAnchorB))); h.extra[3] = F(StripUnit(GetY(c->groundAnchorB)));
        h.extra[4] = F(StripUnit(c->lengthA));
        h.extra[5] = F(StripUnit(c->lengthB));
        h.extra[6] = F(c->ratio);
    } else if (const auto* c = TypeCast<TargetJointConf>(&joint)) {
        // body B only: the GPU side holds it as both bodies (its body A is InvalidBodyID)
        if (c->bodyB == InvalidBodyID) throw InvalidArgument("GpuWorld: target joint without body B");
        h.body_a = h.body_b = to_underlying(c->bodyB);
        h.collide_connected = c->collideConnected ? 1 : 0;
        h.anchor_b[0] = F(StripUnit(GetX(c->localAnchorB))); h.anchor_b[1] = F(StripUnit(GetY(c->localAnchorB)));
        h.kind = PRGPU_JOINT_TARGET;
        h.extra[0] = F(StripUnit(GetX(c->target))); h.extra[1] = F(StripUnit(GetY(c->target)));
        h.extra[2] = F(StripUnit(Force{c->maxForce}));
        h.extra[3] = F(StripUnit(Frequency{c->frequency}));
        h.extra[4] = F(Real{c->dampingRatio});
    } else {
        throw InvalidArgument("GpuWorld: joint type not stepped on the GPU");
    }
    return h;
}

prgpu_step_conf ToAbi(const StepConf& c) {
    prgpu_step_conf s{};
    prgpu_default_step_conf(&s);
    s.deltaTime = F(StripUnit(c.deltaTime));
    s.dtRatio = F(c.dtRatio);
    s.minStillTimeToSleep = F(StripUnit(c.minStillTimeToSleep));
    s.linearSlop = F(StripUnit(Length{c.linearSlop}));
    s.angularSlop = F(StripUnit(Angle{c.angularSlop}));
    s.regResolutionRate = F(c.regResolutionRate);
    s.regMinSeparation = F(StripUnit(c.regMinSeparation));
    s.regMinMomentum = F(StripUnit(c.regMinMomentum));
    s.velocityThreshold = F(StripUnit(c.velocityThreshold));
    s.maxTranslation = F(StripUnit(c.maxTranslation));
    s.maxRotation = F(StripUnit(c.maxRotation));
    s.maxLinearCorrection = F(StripUnit(c.maxLinearCorrection));
    s.maxAngularCorrection = F(StripUnit(c.maxAngularCorrection));
    s.linearSleepTolerance = F(StripUnit(c.linearSleepTolerance));
    s.angularSleepTolerance = F(StripUnit(c.angularSleepTolerance));
    s.displaceMultiplier = F(c.displaceMultiplier);
    s.aabbExtension = F(StripUnit(c.aabbExtension));
    s.maxCirclesRatio = F(c.maxCirclesRatio);
    s.regVelocityIters = static_cast<int32_t>(c.regVelocityIters);
    s.regPositionIters = static_cast<int32_t>(c.regPositionIters);
    s.doWarmStart = c.doWarmStart ? 1 : 0;
    s.doBlocksolve = c.doBlocksolve ? 1 : 0;
    s.toiResolutionRate = F(c.toiResolutionRate);
    s.toiMinSeparation = F(StripUnit(c.toiMinSeparation));
    s.toiMinMomentum = F(StripUnit(c.toiMinMomentum));
    s.targetDepth = F(StripUnit(Length{c.targetDepth}));
    s.tolerance = F(StripUnit(Length{c.tolerance}));
    s.toiVelocityIters = static_cast<int32_t>(c.toiVelocityIters);
    s.toiPositionIters = static_cast<int32_t>(c.toiPositionIters);
    s.maxToiRootIters = static_cast<int32_t>(c.maxToiRootIters);
    s.maxToiIters = static_cast<int32_t>(c.maxToiIters);
    s.maxDistanceIters = static_cast<int32_t>(c.maxDistanceIters);
    s.maxSubSteps = static_cast<int32_t>(c.maxSubSteps);
    s.doToi = c.doToi ? 1 : 0;
    return s;
}

// The GPU's state of body id into the PlayRho body (Sweep, velocity, sleep).
void Mirror(GpuWorld& w, uint32_t id) {
    const prgpu::HostBody& h = w.host.GetBody(id);
    Body& b = w.bodies[id];
    const auto lc = GetLocalCenter(b);
    const Position p{Length2{Real(h.cx) * Meter, Real(h.cy) * Meter}, Real(h.angle) * Radian};
    b.SetSweep(Sweep{p, lc});
    b.JustSetVelocity(Velocity{LinearVelocity2{Real(h.vx) * MeterPerSecond, Real(h.vy) * MeterPerSecond},
                               Real(h.w) * RadianPerSecond});
    if (h.flags & PRGPU_BODY_AWAKE) b.SetAwakeFlag(); else b.UnsetAwakeFlag();
    b.SetUnderActiveTime(Real(h.under_active_time) * Second);
}

template <class ID>
void CheckRange(ID id, uint32_t range, const char* what) {
    if (to_underlying(id) >= range) throw OutOfRange<ID>(id, what);
}

}  // namespace

GpuWorld::GpuWorld(const WorldConf& c, int device) : conf(c), host(device) {}

void GpuWorld::Refresh() const {
    if (contactsValid) return;
    auto& self = const_cast<GpuWorld&>(*this);
    const auto& hc = Guard([&]() -> const std::vector<prgpu::HostContact>& { return self.host.Contacts(); });
    keyedContacts.clear(); contacts.clear(); manifolds.clear(); contactSeq.clear(); contactIndex.clear();
    for (size_t k = 0; k < hc.size(); ++k) {
        const auto& c = hc[k];
        Contact ct{Contactable{BodyID(c.body_a), ShapeID(c.shape_a), ChildCounter(c.child_a)},
                   Contactable{BodyID(c.body_b), ShapeID(c.shape_b), ChildCounter(c.child_b)}};
        ct.SetFriction(Real(c.friction));
        ct.SetRestitution(Real(c.restitution));
        ct.SetTangentSpeed(Real(c.tangent_speed) * MeterPerSecond);
        if (c.enabled) ct.SetEnabled(); else ct.UnsetEnabled();
        if (c.touching) ct.SetTouching(); else ct.UnsetTouching();
        if (c.sensor) ct.SetSensor();
        keyedContacts.emplace_back(ContactKey{c.proxy_a, c.proxy_b}, ContactID(static_cast<ContactID::underlying_type>(c.slot)));
        if (contactIndex.size() <= c.slot) contactIndex.resize(c.slot + 1, -1);
        contactIndex[c.slot] = static_cast<int32_t>(k);
        contactSeq.push_back(c.seq);
        contacts.push_back(ct);
        Manifold m;
        const auto ln = UnitVec::Get(Real(c.local_normal[0]), Real(c.local_normal[1])).first;
        const Length2 lp{Real(c.local_point[0]) * Meter, Real(c.local_point[1]) * Meter};
        auto pt = [&](int j) {
            const uint32_t f = c.feature[j];
            return Manifold::Point{Length2{Real(c.point[j][0]) * Meter, Real(c.point[j][1]) * Meter},
                                   ContactFeature{ContactFeature::Type(f & 0xffu), ContactFeature::Index((f >> 8) & 0xffu),
                                                  ContactFeature::Type((f >> 16) & 0xffu),
                                                  ContactFeature::Index((f >> 24) & 0xffu)},
                                   Real(c.normal_impulse[j]) * NewtonSecond, Real(c.tangent_impulse[j]) * NewtonSecond};
        };
        if (c.type == 1 && c.count >= 1) {  // circles
            const auto p0 = pt(0);
            m = Manifold::GetForCircles(lp, p0.contactFeature.indexA, p0.localPoint, p0.contactFeature.indexB);
            m.SetImpulses(0, p0.normalImpulse, p0.tangentImpulse);
        } else if (c.type == 2) {  // face A
            m = (c.count == 0) ? Manifold::GetForFaceA(ln, lp)
                : (c.count == 1) ? Manifold::GetForFaceA(ln, lp, pt(0)) : Manifold::GetForFaceA(ln, lp, pt(0), pt(1));
        } else if (c.type == 3) {  // face B
            m = (c.count == 0) ? Manifold::GetForFaceB(ln, lp)
                : (c.count == 1) ? Manifold::GetForFaceB(ln, lp, pt(0)) : Manifold::GetForFaceB(ln, lp, pt(0), pt(1));
        }
        manifolds.push_back(m);
    }
    contactsValid = true;
}

// ---- listeners ------------------------------------------------------------------
void SetShapeDestructionListener(GpuWorld& w, ShapeFunction l) noexcept { w.shapeDestructionListener = std::move(l); }
void SetDetachListener(GpuWorld& w, BodyShapeFunction l) noexcept { w.detachListener = std::move(l); }
void SetJointDestructionListener(GpuWorld& w, JointFunction l) noexcept { w.jointDestructionListener = std::move(l); }
void SetBeginContactListener(GpuWorld& w, ContactFunction l) noexcept { w.beginContactListener = std::move(l); }
void SetEndContactListener(GpuWorld& w, ContactFunction l) noexcept { w.endContactListener = std::move(l); }
void SetPreSolveContactListener(GpuWorld& w, ContactManifoldFunction l) noexcept { w.preSolveContactListener = std::move(l); }
void SetPostSolveContactListener(GpuWorld& w, ContactImpulsesFunction l) noexcept { w.postSolveContactListener = std::move(l); }

// ---- world ----------------------------------------------------------------------
bool operator==(const GpuWorld& lhs, const GpuWorld& rhs) noexcept {
    return lhs.bodies == rhs.bodies && lhs.shapes == rhs.shapes && lhs.joints == rhs.joints;
}

std::optional<pmr::StatsResource::Stats> GetResourceStats(const GpuWorld&) noexcept { return std::nullopt; }

void Clear(GpuWorld& w) noexcept {
    w.host.Clear();
    w.bodies.clear(); w.shapes.clear(); w.joints.clear();
    w.Invalidate();
}

namespace {

// The live contacts by creation number, with what the listeners may ask about.
std::vector<std::pair<uint32_t, GpuWorld::Snapshot>> TakeSnapshot(const GpuWorld& w) {
    w.Refresh();
    std::vector<std::pair<uint32_t, GpuWorld::Snapshot>> out;
    out.reserve(w.contacts.size());
    for (size_t k = 0; k < w.contacts.size(); ++k) {
        out.emplace_back(static_cast<uint32_t>(to_underlying(std::get<ContactID>(w.keyedContacts[k]))),
                         GpuWorld::Snapshot{w.contactSeq[k], IsTouching(w.contacts[k]), w.contacts[k], w.manifolds[k]});
    }
    std::sort(out.begin(), out.end(), [](const auto& a, const auto& b) { return a.second.seq < b.second.seq; });
    return out;
}

// The contact listener calls of the step just run, in the reference's order
// (Step, AabbTreeWorld.cpp:2144-2219), from the contacts before and after it and
// the GPU's records of which phase updated or solved each contact:
//  1. EndContact for each touching contact the step destroyed (DestroyContacts ->
//     InternalDestroy, :2245-2253, :2290-2331);
//  2. the pre-phase's UpdateContacts and AddContacts (:2186-2198), then
//  3. PostSolveContact for each contact the regular phase solved (:1669-1672),
//  4. the post-solve UpdateContacts and AddContacts (:1549-1557), and
//  5. the time-of-impact phase's updates (:1879, :2098):
//     for each contact updated in a phase, in contact-list (creation) order, its
//     BeginContact / EndContact if its touching state changed (attributed to the
//     last phase that updated it), then PreSolveContact with the manifold before
//     that update if it touches and is not a sensor (Update, :2703-2720).
// The manifold before the post-solve update carries the solved impulses
// (AssignImpulses, :196-220); before a time-of-impact update, the manifold
// after the step is passed.
void CallContactListeners(GpuWorld& w, std::vector<std::pair<uint32_t, GpuWorld::Snapshot>>& before) {
    auto after = TakeSnapshot(w);
    std::vector<prgpu::HostSolveRecord> recs;
    if (w.preSolveContactListener || w.postSolveContactListener || w.beginContactListener || w.endContactListener)
        recs = Guard([&] { return w.host.SolveRecords(); });
    std::vector<const prgpu::HostSolveRecord*> by_slot;
    for (const auto& r : recs) {
        if (r.slot >= by_slot.size()) by_slot.resize(r.slot + 1, nullptr);
        by_slot[r.slot] = &r;
    }
    auto record = [&](uint32_t slot) -> const prgpu::HostSolveRecord* {
        return slot < by_slot.size() ? by_slot[slot] : nullptr;
    };
    // before-step state of each contact in `after` (nullptr: created by this step)
    std::vector<const GpuWorld::Snapshot*> prior(after.size(), nullptr);
    {
        size_t i = 0;
        for (size_t k = 0; k < after.size(); ++k) {
            while (i < before.size() && before[i].second.seq < after[k].second.seq) ++i;
            if (i < before.size() && before[i].second.seq == after[k].second.seq) prior[k] = &before[i].second;
        }
    }
    struct Call {
        int kind;  // 1 begin, 2 end, 3 pre-solve, 4 post-solve
        ContactID id;
        Manifold manifold;
        ContactImpulsesList impulses;
        unsigned iter;
    };
    std::vector<Call> calls;
    size_t j = 0;
    for (const auto& e : before) {  // destroyed: in `before`, not in `after`
        while (j < after.size() && after[j].second.seq < e.second.seq) ++j;
        const bool alive = j < after.size() && after[j].second.seq == e.second.seq;
        if (!alive && e.second.touching) calls.push_back(Call{2, ContactID(e.first), {}, {}, 0u});
    }
    auto last_phase = [](uint32_t phases) { return phases & 4u ? 4u : phases & 2u ? 2u : phases & 1u ? 1u : 0u; };
    auto phase_pass = [&](uint32_t phase) {
        for (size_t k = 0; k < after.size(); ++k) {
            const auto& e = after[k];
            const auto* r = record(e.first);
            const uint32_t phases = r ? r->phases : 0u;
            const bool was = prior[k] && prior[k]->touching;
            const bool changed = e.second.touching != was;
            // a change without a record (none is expected) is reported with the post-solve pass
            const bool here = (phases & phase) != 0u;
            if (changed && (last_phase(phases) == phase || (phases == 0u && phase == 2u)))
                calls.push_back(Call{e.second.touching ? 1 : 2, ContactID(e.first), {}, {}, 0u});
            if (!here || !e.second.touching || IsSensor(e.second.contact)) continue;
            Manifold old;
            if (phase == 4u) {
                old = e.second.manifold;
            } else if (prior[k]) {
                old = prior[k]->manifold;
                if (phase == 2u && r && r->solved) {
                    const auto n = std::min<std::size_t>(old.GetPointCount(), static_cast<std::size_t>(r->count));
                    for (std::size_t q = 0; q < n; ++q)
                        old.SetImpulses(q, Real(r->normal_impulse[q]) * NewtonSecond,
                                        Real(r->tangent_impulse[q]) * NewtonSecond);
                }
            }
            calls.push_back(Call{3, ContactID(e.first), old, {}, 0u});
        }
    };
    phase_pass(1u);
    for (const auto& e : after) {
        const auto* r = record(e.first);
        if (!r || !r->solved) continue;
        ContactImpulsesList imp;
        for (int q = 0; q < r->count && q < 2; ++q)
            imp.AddEntry(Real(r->normal_impulse[q]) * NewtonSecond, Real(r->tangent_impulse[q]) * NewtonSecond);
        calls.push_back(Call{4, ContactID(e.first), {}, imp, r->iter});
    }
    phase_pass(2u);
    phase_pass(4u);
    w.replaying = &before;
    w.locked = true;
    try {
        for (const auto& c : calls) {
            switch (c.kind) {
            case 1: if (w.beginContactListener) w.beginContactListener(c.id); break;
            case 2: if (w.endContactListener) w.endContactListener(c.id); break;
            case 3: if (w.preSolveContactListener) w.preSolveContactListener(c.id, c.manifold); break;
            default: if (w.postSolveContactListener) w.postSolveContactListener(c.id, c.impulses, c.iter); break;
            }
        }
    } catch (...) {
        w.locked = false;
        w.replaying = nullptr;
        throw;
    }
    w.locked = false;
    w.replaying = nullptr;
    before = std::move(after);
}

}  // namespace

StepStats Step(GpuWorld& w, const StepConf& conf) {
    CheckUnlocked(w);
    StepStats stats;
    const auto sc = ToAbi(conf);
    const bool listen = static_cast<bool>(w.beginContactListener) || static_cast<bool>(w.endContactListener) ||
                        static_cast<bool>(w.preSolveContactListener) || static_cast<bool>(w.postSolveContactListener);
    w.host.SetSolveRecords(static_cast<bool>(w.postSolveContactListener) ||
                           static_cast<bool>(w.preSolveContactListener));
    // the contacts before the step (kept from the last step while listeners are set)
    if (listen && !w.listening) {
        w.previous = w.host.HasGpuBatch() ? TakeSnapshot(w) : decltype(w.previous){};
        w.listening = true;
    }
    if (!listen) {
        w.previous.clear();
        w.listening = false;
    }
    if (w.host.NeedsRebuild()) w.previous.clear();  // a rebuilt batch finds its contacts anew
    const prgpu_step_stats s = Guard([&] { return w.host.Step(sc); });
    for (uint32_t id = 0; id < w.host.BodyRange(); ++id)
        if (w.host.BodyAlive(id)) Mirror(w, id);
    w.Invalidate();
    if (listen) CallContactListeners(w, w.previous);
    if (conf.deltaTime != 0_s) w.invDeltaTime = Real(1) / conf.deltaTime;
    stats.pre.contactsAdded = s.contactsAdded;
    stats.pre.contactsDestroyed = s.contactsDestroyed;
    stats.pre.contactsUpdated = s.contactsUpdated;
    stats.pre.proxiesMoved = s.proxiesMoved;
    stats.reg.islandsFound = s.islandsFound;
    stats.reg.islandsSolved = s.islandsSolved;
    stats.reg.bodiesSlept = s.bodiesSlept;
    stats.reg.sumPosIters = s.sumPosIters;
    stats.reg.minSeparation = Real(s.minSeparation) * Meter;
    stats.reg.maxIncImpulse = Real(s.maxIncImpulse) * NewtonSecond;
    stats.toi.islandsFound = s.toiIslandsFound;
    stats.toi.islandsSolved = s.toiIslandsSolved;
    stats.toi.contactsFound = s.toiContactsFound;
    stats.toi.contactsAtMaxSubSteps = s.toiContactsAtMaxSubSteps;
    stats.toi.contactsUpdatedToi = s.toiContactsUpdatedToi;
    stats.toi.contactsUpdatedTouching = s.toiContactsUpdatedTouching;
    stats.toi.contactsSkippedTouching = s.toiContactsSkippedTouching;
    stats.toi.contactsAdded = s.toiContactsAdded;
    stats.toi.proxiesMoved = s.toiProxiesMoved;
    stats.toi.sumPosIters = s.toiSumPosIters;
    stats.toi.sumVelIters = s.toiSumVelIters;
    stats.toi.maxDistIters = static_cast<ToiStepStats::dist_iter_type>(s.toiMaxDistIters);
    stats.toi.maxToiIters = static_cast<ToiStepStats::toi_iter_type>(s.toiMaxToiIters);
    stats.toi.maxRootIters = static_cast<ToiStepStats::root_iter_type>(s.toiMaxRootIters);
    stats.toi.minSeparation = Real(s.toiMinSeparation) * Meter;
    stats.toi.maxIncImpulse = Real(s.toiMaxIncImpulse) * NewtonSecond;
    return stats;
}

bool IsStepComplete(const GpuWorld& w) noexcept {
    try {
        return const_cast<GpuWorld&>(w).host.StepComplete();
    } catch (...) {
        return true;
    }
}
bool GetSubStepping(const GpuWorld& w) noexcept { return w.subStepping; }
void SetSubStepping(GpuWorld& w, bool flag) noexcept {
    w.subStepping = flag;
    try {
        w.host.SetSubStepping(flag);  // also kept for the next batch the host builds
    } catch (...) {
    }
}

const DynamicTree& GetTree(const GpuWorld& w) noexcept {
    if (!w.treeValid) {
        w.tree.Clear();
        std::vector<float> aabb;
        std::vector<uint32_t> bs;
        try {
            const_cast<GpuWorld&>(w).host.Proxies(aabb, bs);
        } catch (...) {
            aabb.clear(); bs.clear();
        }
        for (size_t k = 0; k < bs.size() / 3; ++k) {
            const AABB box{LengthInterval{Real(aabb[4 * k]) * Meter, Real(aabb[4 * k + 2]) * Meter},
                           LengthInterval{Real(aabb[4 * k + 1]) * Meter, Real(aabb[4 * k + 3]) * Meter}};
            w.tree.CreateLeaf(box, Contactable{BodyID(bs[3 * k]), ShapeID(bs[3 * k + 1]), ChildCounter(bs[3 * k + 2])});
        }
        w.treeValid = true;
    }
    return w.tree;
}

bool IsLocked(const GpuWorld& w) noexcept { return w.locked; }

void ShiftOrigin(GpuWorld& w, const Length2& newOrigin) {
    CheckUnlocked(w);
    for (uint32_t id = 0; id < w.bodies.size(); ++id) {
        if (!w.host.BodyAlive(id)) continue;
        Body b = w.bodies[id];
        SetLocation(b, GetLocation(b) - newOrigin);
        SetBody(w, BodyID(id), b);
    }
}

Interval<Positive<Length>> GetVertexRadiusInterval(const GpuWorld& w) noexcept { return w.conf.vertexRadius; }
Frequency GetInvDeltaTime(const GpuWorld& w) noexcept { return w.invDeltaTime; }

// ---- bodies ---------------------------------------------------------------------
BodyCounter GetBodyRange(const GpuWorld& w) noexcept { return static_cast<BodyCounter>(w.bodies.size()); }

std::vector<BodyID> GetBodies(const GpuWorld& w) {
    std::vector<BodyID> out;
    for (uint32_t id = 0; id < w.bodies.size(); ++id)
        if (w.host.BodyAlive(id)) out.push_back(BodyID(id));
    return out;
}

std::vector<BodyID> GetBodiesForProxies(const GpuWorld&) { return {}; }

BodyID CreateBody(GpuWorld& w, const Body& body) {
    CheckUnlocked(w);
    if (w.bodies.size() >= MaxBodies) throw LengthError("CreateBody: too many bodies");
    for (const auto& s : GetShapes(body)) CheckRange(s, static_cast<uint32_t>(w.shapes.size()), "shape ID out of range");
    const uint32_t id = Guard([&] { return w.host.CreateBody(ToHost(body, nullptr, prgpu::HostBody{})); });
    if (id >= w.bodies.size()) w.bodies.resize(id + 1);
    w.bodies[id] = body;
    w.Invalidate();
    return BodyID(id);
}

Body GetBody(const GpuWorld& w, BodyID id) {
    CheckRange(id, static_cast<uint32_t>(w.bodies.size()), "body ID out of range");
    if (!w.host.BodyAlive(to_underlying(id))) throw WasDestroyed<BodyID>(id, "body was destroyed");
    return w.bodies[to_underlying(id)];
}

void SetBody(GpuWorld& w, BodyID id, const Body& value) {
    CheckUnlocked(w);
    const uint32_t i = to_underlying(id);
    CheckRange(id, static_cast<uint32_t>(w.bodies.size()), "body ID out of range");
    if (!w.host.BodyAlive(i)) throw WasDestroyed<BodyID>(id, "body was destroyed");
    for (const auto& s : GetShapes(value)) CheckRange(s, static_cast<uint32_t>(w.shapes.size()), "shape ID out of range");
    Guard([&] { w.host.SetBody(i, ToHost(value, &w.bodies[i], w.host.GetBody(i))); return 0; });
    w.bodies[i] = value;
    w.Invalidate();
}

void Destroy(GpuWorld& w, BodyID id) {
    CheckUnlocked(w);
    const uint32_t i = to_underlying(id);
    CheckRange(id, static_cast<uint32_t>(w.bodies.size()), "body ID out of range");
    for (const auto& bj : GetJoints(w, id)) {
        if (w.jointDestructionListener) w.jointDestructionListener(std::get<1>(bj));
        w.joints[to_underlying(std::get<1>(bj))] = Joint{};
    }
    if (w.detachListener)
        for (const auto& s : GetShapes(w.bodies[i])) w.detachListener(std::make_pair(id, s));
    Guard([&] { w.host.DestroyBody(i); return 0; });
    w.bodies[i] = Body{};
    w.Invalidate();
}

std::vector<std::pair<BodyID, JointID>> GetJoints(const GpuWorld& w, BodyID id) {
    std::vector<std::pair<BodyID, JointID>> out;
    const uint32_t i = to_underlying(id);
    for (uint32_t j = 0; j < w.joints.size(); ++j) {
        if (!w.host.JointAlive(j)) continue;
        const auto& h = w.host.GetJoint(j);
        if (h.kind == PRGPU_JOINT_TARGET) {
            if (h.body_b == i) out.emplace_back(InvalidBodyID, JointID(j));
        } else if (h.body_a == i) {
            out.emplace_back(BodyID(h.body_b), JointID(j));
        } else if (h.body_b == i) {
            out.emplace_back(BodyID(h.body_a), JointID(j));
        }
    }
    return out;
}

std::vector<std::tuple<ContactKey, ContactID>> GetContacts(const GpuWorld& w, BodyID id) {
    w.Refresh();
    std::vector<std::tuple<ContactKey, ContactID>> out;
    for (size_t k = 0; k < w.contacts.size(); ++k) {
        if (GetBodyA(w.contacts[k]) == id || GetBodyB(w.contacts[k]) == id)
            out.emplace_back(std::get<0>(w.keyedContacts[k]), std::get<1>(w.keyedContacts[k]));
    }
    return out;
}

std::vector<ShapeID> GetShapes(const GpuWorld& w, BodyID id) { return GetShapes(GetBody(w, id)); }

// ---- joints ---------------------------------------------------------------------
JointCounter GetJointRange(const GpuWorld& w) noexcept { return static_cast<JointCounter>(w.joints.size()); }

std::vector<JointID> GetJoints(const GpuWorld& w) {
    std::vector<JointID> out;
    for (uint32_t j = 0; j < w.joints.size(); ++j)
        if (w.host.JointAlive(j)) out.push_back(JointID(j));
    return out;
}

namespace {

// A GearJointConf (GearJointConf.hpp) for the GPU: the two joints it couples are
// found among the world's joints by their bodies (the gear's A and B are their
// second bodies, C and D their first) and kinds (revolute or prismatic, as the
// conf's type data say); ratio and constant are the conf's own.
prgpu::HostJoint GearToHost(const GpuWorld& w, const GearJointConf& c) {
    auto find = [&](BodyID first, BodyID second, bool prismatic) -> uint32_t {
        for (uint32_t j = 0; j < w.joints.size(); ++j) {
            if (!w.host.JointAlive(j)) continue;
            const auto& h = w.host.GetJoint(j);
            const bool kindOk = prismatic ? (h.kind == PRGPU_JOINT_PRISMATIC) : (h.kind == PRGPU_JOINT_REVOLUTE);
            if (kindOk && h.body_a == to_underlying(first) && h.body_b == to_underlying(second)) return j;
        }
        throw InvalidArgument("GpuWorld: no revolute or prismatic joint that the gear joint couples");
    };
    const bool prisAC = std::holds_alternative<GearJointConf::PrismaticData>(c.typeDataAC);
    const bool prisBD = std::holds_alternative<GearJointConf::PrismaticData>(c.typeDataBD);
    if (std::holds_alternative<std::monostate>(c.typeDataAC) || std::holds_alternative<std::monostate>(c.typeDataBD))
        throw InvalidArgument("GpuWorld: gear joint without coupled joint data");
    prgpu::HostJoint h;
    h.kind = PRGPU_JOINT_GEAR;
    h.body_a = to_underlying(GetBodyA(c));
    h.body_b = to_underlying(GetBodyB(c));
    h.collide_connected = c.collideConnected ? 1 : 0;
    h.extra[0] = static_cast<float>(find(c.bodyC, GetBodyA(c), prisAC));
    h.extra[1] = static_cast<float>(find(c.bodyD, GetBodyB(c), prisBD));
    h.extra[2] = F(c.ratio);
    h.extra[3] = F(c.constant);
    h.extra[4] = 1.f;  // keep the conf's constant
    return h;
}

prgpu::HostJoint ToHost(const GpuWorld& w, const Joint& def) {
    if (const auto* c = TypeCast<GearJointConf>(&def)) return GearToHost(w, *c);
    return ToHost(def);
}

}  // namespace

JointID CreateJoint(GpuWorld& w, const Joint& def) {
    CheckUnlocked(w);
    if (w.joints.size() >= MaxJoints) throw LengthError("CreateJoint: too many joints");
    const uint32_t id = Guard([&] { return w.host.CreateJoint(ToHost(w, def)); });
    if (id >= w.joints.size()) w.joints.resize(id + 1);
    w.joints[id] = def;
    w.Invalidate();
    return JointID(id);
}

Joint GetJoint(const GpuWorld& w, JointID id) {
    CheckRange(id, static_cast<uint32_t>(w.joints.size()), "joint ID out of range");
    if (!w.host.JointAlive(to_underlying(id))) throw WasDestroyed<JointID>(id, "joint was destroyed");
    return w.joints[to_underlying(id)];
}

void SetJoint(GpuWorld& w, JointID id, const Joint& def) {
    CheckUnlocked(w);
    CheckRange(id, static_cast<uint32_t>(w.joints.size()), "joint ID out of range");
    Guard([&] { w.host.SetJoint(to_underlying(id), ToHost(w, def)); return 0; });
    w.joints[to_underlying(id)] = def;
    w.Invalidate();
}

void Destroy(GpuWorld& w, JointID id) {
    CheckUnlocked(w);
    CheckRange(id, static_cast<uint32_t>(w.joints.size()), "joint ID out of range");
    Guard([&] { w.host.DestroyJoint(to_underlying(id)); return 0; });
    w.joints[to_underlying(id)] = Joint{};
    w.Invalidate();
}

// ---- shapes ---------------------------------------------------------------------
ShapeCounter GetShapeRange(const GpuWorld& w) noexcept { return static_cast<ShapeCounter>(w.shapes.size()); }

ShapeID CreateShape(GpuWorld& w, const Shape& def) {
    CheckUnlocked(w);
    if (w.shapes.size() >= MaxShapes) throw LengthError("CreateShape: too many shapes");
    const auto& lim = w.conf.vertexRadius;
    for (ChildCounter i = 0; i < GetChildCount(def); ++i) {
        const auto vr = GetVertexRadius(def, i);
        if (vr < lim.GetMin() || vr > lim.GetMax())
            throw InvalidArgument("CreateShape: vertex radius out of the world's range");
    }
    const uint32_t id = Guard([&] { return w.host.CreateShape(ToHost(def)); });
    if (id >= w.shapes.size()) w.shapes.resize(id + 1);
    w.shapes[id] = def;
    w.Invalidate();
    return ShapeID(id);
}

Shape GetShape(const GpuWorld& w, ShapeID id) {
    CheckRange(id, static_cast<uint32_t>(w.shapes.size()), "shape ID out of range");
    if (!w.host.ShapeAlive(to_underlying(id))) throw WasDestroyed<ShapeID>(id, "shape was destroyed");
    return w.shapes[to_underlying(id)];
}

void SetShape(GpuWorld& w, ShapeID id, const Shape& def) {
    CheckUnlocked(w);
    CheckRange(id, static_cast<uint32_t>(w.shapes.size()), "shape ID out of range");
    Guard([&] { w.host.SetShape(to_underlying(id), ToHost(def)); return 0; });
    w.shapes[to_underlying(id)] = def;
    w.Invalidate();
}

void Destroy(GpuWorld& w, ShapeID id) {
    CheckUnlocked(w);
    CheckRange(id, static_cast<uint32_t>(w.shapes.size()), "shape ID out of range");
    if (w.shapeDestructionListener) w.shapeDestructionListener(id);
    Guard([&] { w.host.DestroyShape(to_underlying(id)); return 0; });
    for (uint32_t b = 0; b < w.bodies.size(); ++b)
        if (w.host.BodyAlive(b)) {
            Body body = w.bodies[b];
            if (body.Detach(id)) w.bodies[b] = body;
        }
    w.shapes[to_underlying(id)] = Shape{};
    w.Invalidate();
}

// ---- contacts -------------------------------------------------------------------
namespace {

// Position of a live contact by ID; -1 with *old set for a contact the last step
// destroyed, while that step's listeners run (they may still ask about it).
int32_t ContactAt(const GpuWorld& w, ContactID id, const GpuWorld::Snapshot** old) {
    w.Refresh();
    *old = nullptr;
    const auto slot = to_underlying(id);
    if (slot < w.contactIndex.size() && w.contactIndex[slot] >= 0) return w.contactIndex[slot];
    if (w.replaying) {
        for (const auto& e : *w.replaying)
            if (e.first == slot) { *old = &e.second; return -1; }
    }
    if (slot >= w.contactIndex.size()) throw OutOfRange<ContactID>(id, "contact ID out of range");
    throw WasDestroyed<ContactID>(id, "contact was destroyed");
}

}  // namespace

ContactCounter GetContactRange(const GpuWorld& w) noexcept {
    try {
        w.Refresh();
    } catch (...) {
        return 0;
    }
    return static_cast<ContactCounter>(w.contactIndex.size());
}

std::vector<KeyedContactID> GetContacts(const GpuWorld& w) {
    w.Refresh();
    return w.keyedContacts;
}

Contact GetContact(const GpuWorld& w, ContactID id) {
    const GpuWorld::Snapshot* old;
    const auto k = ContactAt(w, id, &old);
    return old ? old->contact : w.contacts[static_cast<size_t>(k)];
}

// SetContact (AabbTreeWorld.cpp:2797-2832): the contactables and the sensor
// state stay; enabled, friction, restitution and tangent speed are taken into
// the next step.
void SetContact(GpuWorld& w, ContactID id, const Contact& value) {
    CheckUnlocked(w);
    const GpuWorld::Snapshot* old;
    const auto k = ContactAt(w, id, &old);
    if (old) throw WasDestroyed<ContactID>(id, "contact was destroyed");
    const auto& elem = w.contacts[static_cast<size_t>(k)];
    if (elem.GetContactableA() != value.GetContactableA()) throw InvalidArgument("cannot change contactable A");
    if (elem.GetContactableB() != value.GetContactableB()) throw InvalidArgument("cannot change contactable B");
    if (IsSensor(elem) != IsSensor(value))
        throw InvalidArgument("change shape A or B being a sensor to change sensor state");
    Guard([&] {
        w.host.SetContact(to_underlying(id), IsEnabled(value), F(GetFriction(value)), F(GetRestitution(value)),
                          F(GetTangentSpeed(value) / MeterPerSecond));
    });
    w.Invalidate();
}

Manifold GetManifold(const GpuWorld& w, ContactID id) {
    const GpuWorld::Snapshot* old;
    const auto k = ContactAt(w, id, &old);
    return old ? old->manifold : w.manifolds[static_cast<size_t>(k)];
}

// SetManifold (AabbTreeWorld.cpp:2834-2848): same type and point count.
void SetManifold(GpuWorld& w, ContactID id, const Manifold& value) {
    CheckUnlocked(w);
    const GpuWorld::Snapshot* old;
    const auto k = ContactAt(w, id, &old);
    if (old) throw WasDestroyed<ContactID>(id, "contact was destroyed");
    const auto& m = w.manifolds[static_cast<size_t>(k)];
    if (m.GetType() != value.GetType()) throw InvalidArgument("cannot change manifold type");
    if (m.GetPointCount() != value.GetPointCount()) throw InvalidArgument("cannot change manifold point count");
    float head[4] = {F(GetX(value.GetLocalNormal())), F(GetY(value.GetLocalNormal())),
                     F(GetX(value.GetLocalPoint()) / Meter), F(GetY(value.GetLocalPoint()) / Meter)};
    float pts[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (auto j = 0; j < static_cast<int>(value.GetPointCount()); ++j) {
        const auto p = value.GetPoint(j);
        pts[4 * j] = F(GetX(p.localPoint) / Meter);
        pts[4 * j + 1] = F(GetY(p.localPoint) / Meter);
        pts[4 * j + 2] = F(p.normalImpulse / NewtonSecond);
        pts[4 * j + 3] = F(p.tangentImpulse / NewtonSecond);
    }
    const int type = (value.GetType() == Manifold::e_circles) ? 1 : (value.GetType() == Manifold::e_faceA) ? 2
                   : (value.GetType() == Manifold::e_faceB) ? 3 : 0;
    Guard([&] {
        w.host.SetManifold(to_underlying(id), type, static_cast<int32_t>(value.GetPointCount()), head, pts);
    });
    w.Invalidate();
}

}  // namespace playrho::d2
