// ref_scene.hpp -- the scene records read by the reference drivers (ref_driver,
// ref_bench): each line builds part of a World through the reference's public
// API (CreateBody, CreateShape, Attach, CreateJoint) or changes the StepConf.
//   conf <StepConf field> <value> ...        overrides of StepConf defaults
//   body type px py angle vx vy av ax ay aa linDamp angDamp flags
//        (flags: 1 allow sleep, 2 awake, 4 fixed rotation, 8 enabled, 16 bullet)
//   shape body kind nverts radius density friction restitution cat mask group sensor x0 y0 ...
//   joint bodyA bodyB lax lay lbx lby refAngle enableLimit lower upper enableMotor
//         motorSpeed maxMotorTorque collideConnected
//   jointx kind bodyA bodyB lax lay lbx lby collideConnected enableLimit enableMotor e0..e7
#pragma once
#include <playrho/d2/World.hpp>
#include <playrho/d2/WorldBody.hpp>
#include <playrho/d2/WorldContact.hpp>
#include <playrho/d2/WorldShape.hpp>
#include <playrho/d2/WorldJoint.hpp>
#include <playrho/d2/WorldMisc.hpp>
#include <playrho/d2/DiskShapeConf.hpp>
#include <playrho/d2/EdgeShapeConf.hpp>
#include <playrho/d2/PolygonShapeConf.hpp>
#include <playrho/d2/ChainShapeConf.hpp>
#include <playrho/d2/MultiShapeConf.hpp>
#include <playrho/d2/RevoluteJointConf.hpp>
#include <playrho/d2/DistanceJointConf.hpp>
#include <playrho/d2/RopeJointConf.hpp>
#include <playrho/d2/WeldJointConf.hpp>
#include <playrho/d2/FrictionJointConf.hpp>
#include <playrho/d2/MotorJointConf.hpp>
#include <playrho/d2/PrismaticJointConf.hpp>
#include <playrho/d2/WheelJointConf.hpp>
#include <playrho/d2/PulleyJointConf.hpp>
#include <playrho/d2/TargetJointConf.hpp>
#include <playrho/d2/GearJointConf.hpp>
#include <playrho/d2/Joint.hpp>
#include <playrho/StepConf.hpp>

#include <cstdio>
#include <cstdlib>
#include <istream>
#include <string>
#include <vector>

namespace refscene {

using namespace playrho;
using namespace playrho::d2;

inline Real rd(std::istream& in)
{
    std::string t;
    in >> t;
    return static_cast<Real>(std::strtod(t.c_str(), nullptr));
}

inline void hex(double v) { std::printf(" %a", v); }

inline void setConf(StepConf& c, const std::string& k, Real v)
{
    if (k == "deltaTime") c.deltaTime = v * 1_s;
    else if (k == "dtRatio") c.dtRatio = v;
    else if (k == "minStillTimeToSleep") c.minStillTimeToSleep = v * 1_s;
    else if (k == "linearSlop") c.linearSlop = v * 1_m;
    else if (k == "angularSlop") c.angularSlop = v * 1_rad;
    else if (k == "regResolutionRate") c.regResolutionRate = v;
    else if (k == "regMinSeparation") c.regMinSeparation = v * 1_m;
    else if (k == "regMinMomentum") c.regMinMomentum = v * 1_Ns;
    else if (k == "velocityThreshold") c.velocityThreshold = v * 1_mps;
    else if (k == "maxTranslation") c.maxTranslation = v * 1_m;
    else if (k == "maxRotation") c.maxRotation = v * 1_rad;
    else if (k == "maxLinearCorrection") c.maxLinearCorrection = v * 1_m;
    else if (k == "maxAngularCorrection") c.maxAngularCorrection = v * 1_rad;
    else if (k == "linearSleepTolerance") c.linearSleepTolerance = v * 1_mps;
    else if (k == "angularSleepTolerance") c.angularSleepTolerance = v * 1_rad / 1_s;
    else if (k == "displaceMultiplier") c.displaceMultiplier = v;
    else if (k == "aabbExtension") c.aabbExtension = v * 1_m;
    else if (k == "maxCirclesRatio") c.maxCirclesRatio = v;
    else if (k == "regVelocityIters") c.regVelocityIters = static_cast<StepConf::iteration_type>(v);
    else if (k == "regPositionIters") c.regPositionIters = static_cast<StepConf::iteration_type>(v);
    else if (k == "doWarmStart") c.doWarmStart = v != 0;
    else if (k == "doBlocksolve") c.doBlocksolve = v != 0;
    else if (k == "doToi") c.doToi = v != 0;
    else { std::fprintf(stderr, "unknown conf key %s\n", k.c_str()); std::exit(2); }
}


// Applies one scene record (tag already read from `in`); false if the tag is not one.
inline bool ApplyRecord(World& world, StepConf& conf, const std::string& tag, std::istream& in)
{
    if (tag == "conf") {
        std::string k;
        while (in >> k) setConf(conf, k, rd(in));
        return true;
    }
    if (tag == "body") {
        int type = 0; in >> type;
        const auto px = rd(in), py = rd(in), a = rd(in), vx = rd(in), vy = rd(in), av = rd(in);
        const auto ax = rd(in), ay = rd(in), aa = rd(in), ld = rd(in), ad = rd(in);
        unsigned flags = 0; in >> flags;
        auto bc = BodyConf{};
        bc.Use(type == 2 ? BodyType::Dynamic : type == 1 ? BodyType::Kinematic : BodyType::Static);
        bc.UseLocation(Length2{px * 1_m, py * 1_m});
        bc.UseAngle(a * 1_rad);
        bc.UseLinearVelocity(LinearVelocity2{vx * 1_mps, vy * 1_mps});
        bc.UseAngularVelocity(av * 1_rad / 1_s);
        bc.UseLinearAcceleration(LinearAcceleration2{ax * 1_mps2, ay * 1_mps2});
        bc.UseAngularAcceleration(aa * 1_rad / (1_s * 1_s));
        bc.UseLinearDamping(ld * 1_Hz);
        bc.UseAngularDamping(ad * 1_Hz);
        bc.UseAllowSleep((flags & 1u) != 0);
        bc.UseAwake((flags & 2u) != 0);
        bc.UseFixedRotation((flags & 4u) != 0);
        bc.UseEnabled((flags & 8u) != 0);
        bc.UseBullet((flags & 16u) != 0);
        CreateBody(world, bc);
    }
    else if (tag == "shape") {
        int body = 0, kind = 0, nv = 0;
        in >> body >> kind >> nv;
        auto radius = rd(in);
        const auto density = rd(in), friction = rd(in), restitution = rd(in);
        // Scenes carry float32 values; in the Real = double build a 0.01f skin is
        // just under the world's minimum vertex radius, so it is raised to it.
        const auto minRadius = GetVertexRadiusInterval(world).GetMin() / 1_m;
        if (kind != 0 && radius < minRadius) radius = static_cast<Real>(minRadius);
        unsigned cat = 0, mask = 0; int group = 0, sensor = 0;
        in >> cat >> mask >> group >> sensor;
        std::vector<Length2> v;
        for (int i = 0; i < nv; ++i) { const auto x = rd(in); const auto y = rd(in); v.push_back(Length2{x * 1_m, y * 1_m}); }
        auto filter = Filter{};
        filter.categoryBits = static_cast<Filter::bits_type>(cat);
        filter.maskBits = static_cast<Filter::bits_type>(mask);
        filter.groupIndex = static_cast<Filter::index_type>(group);
        ShapeID sid;
        if (kind == 0) {
            auto c = DiskShapeConf{};
            c.UseRadius(radius * 1_m).UseLocation(v.at(0));
            c.UseDensity(density * 1_kgpm2).UseFriction(friction).UseRestitution(restitution);
            c.UseFilter(filter).UseIsSensor(sensor != 0);
            sid = CreateShape(world, c);
        }
        else if (kind == 1) {
            auto c = PolygonShapeConf{};
            c.UseVertices(v);
            c.UseVertexRadius(radius * 1_m);
            c.UseDensity(density * 1_kgpm2).UseFriction(friction).UseRestitution(restitution);
            c.UseFilter(filter).UseIsSensor(sensor != 0);
            sid = CreateShape(world, c);
        }
        else {
            auto c = EdgeShapeConf{v.at(0), v.at(1)};
            c.UseVertexRadius(radius * 1_m);
            c.UseDensity(density * 1_kgpm2).UseFriction(friction).UseRestitution(restitution);
            c.UseFilter(filter).UseIsSensor(sensor != 0);
            sid = CreateShape(world, c);
        }
        Attach(world, BodyID(static_cast<BodyID::underlying_type>(body)), sid, true);
    }
    else if (tag == "chain" || tag == "multi") {
        // chain body nv radius density friction restitution cat mask group sensor x0 y0 ...
        // multi body nhulls radius density friction restitution cat mask group sensor
        //       (nv x0 y0 ...) per hull
        int body = 0, n = 0;
        in >> body >> n;
        auto radius = rd(in);
        const auto density = rd(in), friction = rd(in), restitution = rd(in);
        const auto minRadius = GetVertexRadiusInterval(world).GetMin() / 1_m;
        if (radius < minRadius) radius = static_cast<Real>(minRadius);
        unsigned cat = 0, mask = 0; int group = 0, sensor = 0;
        in >> cat >> mask >> group >> sensor;
        auto filter = Filter{};
        filter.categoryBits = static_cast<Filter::bits_type>(cat);
        filter.maskBits = static_cast<Filter::bits_type>(mask);
        filter.groupIndex = static_cast<Filter::index_type>(group);
        ShapeID sid;
        if (tag == "chain") {
            std::vector<Length2> v;
            for (int i = 0; i < n; ++i) { const auto x = rd(in); const auto y = rd(in); v.push_back(Length2{x * 1_m, y * 1_m}); }
            auto c = ChainShapeConf{};
            c.Set(v);
            c.vertexRadius = radius * 1_m;
            c.UseDensity(density * 1_kgpm2).UseFriction(friction).UseRestitution(restitution);
            c.UseFilter(filter).UseIsSensor(sensor != 0);
            sid = CreateShape(world, c);
        }
        else {
            auto c = MultiShapeConf{};
            for (int k = 0; k < n; ++k) {
                int nv = 0; in >> nv;
                auto vs = VertexSet{};
                for (int i = 0; i < nv; ++i) { const auto x = rd(in); const auto y = rd(in); vs.add(Length2{x * 1_m, y * 1_m}); }
                c.AddConvexHull(vs, radius * 1_m);
            }
            c.UseDensity(density * 1_kgpm2).UseFriction(friction).UseRestitution(restitution);
            c.UseFilter(filter).UseIsSensor(sensor != 0);
            sid = CreateShape(world, c);
        }
        Attach(world, BodyID(static_cast<BodyID::underlying_type>(body)), sid, true);
    }
    else if (tag == "joint") {
        int a = 0, b = 0; in >> a >> b;
        auto j = RevoluteJointConf{};
        j.bodyA = BodyID(static_cast<BodyID::underlying_type>(a));
        j.bodyB = BodyID(static_cast<BodyID::underlying_type>(b));
        const auto lax = rd(in), lay = rd(in), lbx = rd(in), lby = rd(in), ref = rd(in);
        j.localAnchorA = Length2{lax * 1_m, lay * 1_m};
        j.localAnchorB = Length2{lbx * 1_m, lby * 1_m};
        j.referenceAngle = ref * 1_rad;
        int en = 0; in >> en; j.enableLimit = en != 0;
        j.lowerAngle = rd(in) * 1_rad; j.upperAngle = rd(in) * 1_rad;
        in >> en; j.enableMotor = en != 0;
        j.motorSpeed = rd(in) * 1_rad / 1_s;
        j.maxMotorTorque = rd(in) * 1_Nm;
        in >> en; j.collideConnected = en != 0;
        CreateJoint(world, Joint{j});
    }
    else if (tag == "jointx") {
        // jointx kind bodyA bodyB lax lay lbx lby collideConnected enableLimit enableMotor e0..e7
        int kind = 0, a = 0, b = 0; in >> kind >> a >> b;
        const auto lax = rd(in), lay = rd(in), lbx = rd(in), lby = rd(in);
        int cc = 0, el = 0, em = 0; in >> cc >> el >> em;
        Real e[8];
        for (auto& x : e) x = rd(in);
        const auto bA = BodyID(static_cast<BodyID::underlying_type>(a));
        const auto bB = BodyID(static_cast<BodyID::underlying_type>(b));
        const auto laA = Length2{lax * 1_m, lay * 1_m}, laB = Length2{lbx * 1_m, lby * 1_m};
        if (kind == 1) {
            auto j = DistanceJointConf{bA, bB, laA, laB, e[0] * 1_m};
            j.frequency = e[1] * 1_Hz; j.dampingRatio = e[2]; j.collideConnected = cc != 0;
            CreateJoint(world, Joint{j});
        } else if (kind == 2) {
            auto j = RopeJointConf{bA, bB};
            j.localAnchorA = laA; j.localAnchorB = laB; j.maxLength = e[0] * 1_m; j.collideConnected = cc != 0;
            CreateJoint(world, Joint{j});
        } else if (kind == 3) {
            auto j = WeldJointConf{};
            j.bodyA = bA; j.bodyB = bB; j.localAnchorA = laA; j.localAnchorB = laB;
            j.referenceAngle = e[0] * 1_rad; j.frequency = e[1] * 1_Hz; j.dampingRatio = e[2];
            j.collideConnected = cc != 0;
            CreateJoint(world, Joint{j});
        } else if (kind == 4) {
            auto j = FrictionJointConf{};
            j.bodyA = bA; j.bodyB = bB; j.localAnchorA = laA; j.localAnchorB = laB;
            j.maxForce = e[0] * 1_N; j.maxTorque = e[1] * 1_Nm; j.collideConnected = cc != 0;
            CreateJoint(world, Joint{j});
        } else if (kind == 5) {
            auto j = MotorJointConf{};
            j.bodyA = bA; j.bodyB = bB; j.linearOffset = Length2{e[0] * 1_m, e[1] * 1_m};
            j.angularOffset = e[2] * 1_rad; j.maxForce = e[3] * 1_N; j.maxTorque = e[4] * 1_Nm;
            j.correctionFactor = e[5]; j.collideConnected = cc != 0;
            CreateJoint(world, Joint{j});
        } else if (kind == 6) {
            const auto axis = std::get<UnitVec>(UnitVec::Get(e[0], e[1]));
            auto j = PrismaticJointConf{bA, bB, laA, laB, axis, e[2] * 1_rad};
            j.enableLimit = el != 0; j.lowerTranslation = e[3] * 1_m; j.upperTranslation = e[4] * 1_m;
            j.enableMotor = em != 0; j.motorSpeed = e[5] * 1_rad / 1_s; j.maxMotorForce = e[6] * 1_N;
            j.collideConnected = cc != 0;
            CreateJoint(world, Joint{j});
        } else if (kind == 7) {
            const auto axis = std::get<UnitVec>(UnitVec::Get(e[0], e[1]));
            auto j = WheelJointConf{bA, bB, laA, laB, axis};
            j.enableMotor = em != 0; j.motorSpeed = e[2] * 1_rad / 1_s; j.maxMotorTorque = e[3] * 1_Nm;
            j.frequency = e[4] * 1_Hz; j.dampingRatio = e[5]; j.collideConnected = cc != 0;
            CreateJoint(world, Joint{j});
        } else if (kind == 8) {
            auto j = PulleyJointConf{bA, bB, Length2{e[0] * 1_m, e[1] * 1_m}, Length2{e[2] * 1_m, e[3] * 1_m},
                                     laA, laB, e[4] * 1_m, e[5] * 1_m};
            j.ratio = e[6]; j.collideConnected = cc != 0;
            CreateJoint(world, Joint{j});
        } else if (kind == 10) {
            // the gear couples two existing joints (e0, e1) with ratio e2
            const auto j1 = JointID(static_cast<JointID::underlying_type>(e[0]));
            const auto j2 = JointID(static_cast<JointID::underlying_type>(e[1]));
            CreateJoint(world, Joint{GetGearJointConf(world, j1, j2, e[2])});
        } else if (kind == 9) {
            // the target joint has body B only (its body A is InvalidBodyID)
            auto j = TargetJointConf{bB};
            j.localAnchorB = laB; j.target = Length2{e[0] * 1_m, e[1] * 1_m};
            j.maxForce = e[2] * 1_N; j.frequency = e[3] * 1_Hz; j.dampingRatio = e[4];
            j.collideConnected = cc != 0;
            CreateJoint(world, Joint{j});
        }
    }
    else {
        return false;
    }
    return true;
}

} // namespace refscene
