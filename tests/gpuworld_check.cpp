// gpuworld_check.cpp -- the reference's HelloWorld program with one change:
// the World is constructed over GpuWorld.  Everything else goes through
// PlayRho's own World API (CreateShape, CreateBody with BodyConf::Use(shape),
// Step with the default StepConf, GetTransformation, ...).  Then one joint of
// each kind the GPU steps is made through CreateJoint on a second world and the
// joint GpuWorld hands to the GPU side is printed.
//
// Prints, one per line:
//   bodies N / shapes N / mass <invMass> <invRotI> / type T     after set-up
//   joint <kind> <collide> <anchorA.x> <anchorB.y> <extra0..6> <limit> <motor> <bodyA> <bodyB>
//                                                               per joint kind
//   joint_rejected <what>                                       for a kind the GPU does not step
//   step <i> <x> <y> <angle>                                    per step (needs a GPU)
//   error <what>                                                when stepping fails
#include <cstdio>
#include <exception>
#include <optional>

#include "playrho/d2/BasicAPI.hpp"
#include "playrho/d2/ChainShapeConf.hpp"
#include "playrho/d2/MultiShapeConf.hpp"

#include <cmath>
#include <utility>
#include <vector>
#include "playrho/d2/GearJointConf.hpp"
#include "playrho/d2/PrismaticJointConf.hpp"
#include "playrho/d2/PulleyJointConf.hpp"
#include "playrho/d2/TargetJointConf.hpp"
#include "playrho/d2/WheelJointConf.hpp"

#include "GpuWorld.hpp"

namespace {

void CheckJoints() {
    using namespace playrho;
    using namespace playrho::d2;
    auto world = World{GpuWorld{}};
    const auto disk = CreateShape(world, DiskShapeConf{}.UseRadius(0.5_m));
    const auto a = CreateBody(world, BodyConf{}.Use(BodyType::Dynamic).Use(disk).UseLocation(Length2{0_m, 0_m}));
    const auto b = CreateBody(world, BodyConf{}.Use(BodyType::Dynamic).Use(disk).UseLocation(Length2{2_m, 0_m}));
    const auto anchorA = Length2{0.25_m, 0_m};
    const auto anchorB = Length2{-0.25_m, 0.5_m};
    auto distance = DistanceJointConf{a, b};
    distance.localAnchorA = anchorA; distance.localAnchorB = anchorB;
    distance.length = 1.5_m; distance.frequency = 4_Hz; distance.dampingRatio = 0.5f;
    auto rope = RopeJointConf{a, b};
    rope.localAnchorA = anchorA; rope.localAnchorB = anchorB; rope.maxLength = 2.5_m;
    rope.collideConnected = true;
    auto weld = WeldJointConf{a, b};
    weld.localAnchorA = anchorA; weld.localAnchorB = anchorB;
    weld.referenceAngle = 0.25_rad; weld.frequency = 2_Hz; weld.dampingRatio = 0.75f;
    auto friction = FrictionJointConf{a, b};
    friction.localAnchorA = anchorA; friction.localAnchorB = anchorB;
    friction.maxForce = 3_N; friction.maxTorque = 1.5_Nm;
    auto motor = MotorJointConf{a, b};
    motor.linearOffset = Length2{1_m, -0.5_m}; motor.angularOffset = 0.125_rad;
    motor.maxForce = 10_N; motor.maxTorque = 5_Nm; motor.correctionFactor = 0.25f;
    auto revolute = RevoluteJointConf{a, b};
    revolute.localAnchorA = anchorA; revolute.localAnchorB = anchorB;
    auto prismatic = PrismaticJointConf{a, b, anchorA, anchorB, UnitVec::GetUp(), 0.5_rad};
    prismatic.enableLimit = true; prismatic.lowerTranslation = -1_m; prismatic.upperTranslation = 2_m;
    prismatic.enableMotor = true; prismatic.motorSpeed = 3_rad / 1_s; prismatic.maxMotorForce = 7_N;
    auto wheel = WheelJointConf{a, b, anchorA, anchorB, UnitVec::GetUp()};
    wheel.enableMotor = true; wheel.motorSpeed = -2_rad / 1_s; wheel.maxMotorTorque = 6_Nm;
    wheel.frequency = 4_Hz; wheel.dampingRatio = 0.5f;
    auto pulley = PulleyJointConf{a, b, Length2{-1_m, 5_m}, Length2{2_m, 5_m}, anchorA, anchorB, 4_m, 3_m};
    pulley.ratio = 1.5f;
    auto target = TargetJointConf{b};
    target.localAnchorB = anchorB; target.target = Length2{3_m, 4_m}; target.maxForce = 9_N;
    target.frequency = 3_Hz; target.dampingRatio = 0.25f;
    for (const auto& def : {Joint{revolute}, Joint{distance}, Joint{rope}, Joint{weld}, Joint{friction},
                            Joint{motor}, Joint{prismatic}, Joint{wheel}, Joint{pulley}, Joint{target}}) {
        const auto id = CreateJoint(world, def);
        const auto& h = TypeCast<const GpuWorld&>(world).host.GetJoint(to_underlying(id));
        std::printf("joint %d %d %a %a", h.kind, h.collide_connected, static_cast<double>(h.anchor_a[0]),
                    static_cast<double>(h.anchor_b[1]));
        for (auto k = 0; k < 7; ++k) std::printf(" %a", static_cast<double>(h.extra[k]));
        std::printf(" %d %d %u %u", h.enable_limit, h.enable_motor, h.body_a, h.body_b);
        std::printf("\n");
    }
    // a gear coupling the revolute joint (ID 0) and the prismatic one (ID 6), made
    // by the reference's own GetGearJointConf: GpuWorld finds the two joints
    const auto gear = CreateJoint(world, Joint{GetGearJointConf(world, JointID(0), JointID(6), 2.0f)});
    const auto& gh = TypeCast<const GpuWorld&>(world).host.GetJoint(to_underlying(gear));
    std::printf("gear %d %g %g %g %d\n", gh.kind, double(gh.extra[0]), double(gh.extra[1]), double(gh.extra[2]),
                int(gh.extra[4]));
    try {
        CreateJoint(world, Joint{GearJointConf{}});
    } catch (const InvalidArgument& e) {
        std::printf("joint_rejected %s\n", e.what());
    }
}

// The same calls on a world of either kind: a box and a disk dropped on a ground
// box, the BeginContact / EndContact listeners recording (step, begin?, lower
// shape, higher shape), the box-ground contact's ID followed through the run,
// and SetContact on it: a tangent speed of 2 m/s with friction 0.8 from step 20
// (a conveyor belt), disabled from step 45 (the box sinks through the ground).
// Prints "<tag> event ...", "<tag> call ...", "<tag> pre ...", "<tag> post ...",
// "<tag> id ..." and "<tag> pos ..." lines; StepConf::doToi as given.
void Conveyor(playrho::d2::World& world, const char* tag, bool doToi) {
    using namespace playrho;
    using namespace playrho::d2;
    const auto ground = CreateShape(world, PolygonShapeConf{}.SetAsBox(20_m, 1_m));
    CreateBody(world, BodyConf{}.Use(ground).UseLocation(Length2{0_m, -1_m}));
    const auto boxShape = CreateShape(world, PolygonShapeConf{}.SetAsBox(0.5_m, 0.5_m).UseDensity(1_kgpm2).UseFriction(0.5f));
    const auto box = CreateBody(world, BodyConf{}.Use(BodyType::Dynamic).Use(boxShape)
                                           .UseLocation(Length2{0_m, 0.75_m}).UseLinearAcceleration(EarthlyGravity));
    const auto diskShape = CreateShape(world, DiskShapeConf{}.UseRadius(0.4_m).UseDensity(1_kgpm2));
    CreateBody(world, BodyConf{}.Use(BodyType::Dynamic).Use(diskShape).UseLocation(Length2{3_m, 1.5_m})
                          .UseLinearAcceleration(EarthlyGravity));
    auto step = 0;
    auto event = [&world, &step, tag](const char* kind, ContactID id) {
        const auto& c = GetContact(world, id);
        const auto a = to_underlying(GetShapeA(c)), b = to_underlying(GetShapeB(c));
        std::printf("%s event %d %s %u %u\n", tag, step, kind, unsigned(a < b ? a : b), unsigned(a < b ? b : a));
        std::printf("%s call %d %s %u %u\n", tag, step, kind, unsigned(a < b ? a : b), unsigned(a < b ? b : a));
    };
    SetBeginContactListener(world, [event](ContactID id) { event("begin", id); });
    SetEndContactListener(world, [event](ContactID id) { event("end", id); });
    // PreSolveContact / PostSolveContact: "<tag> call <step> <kind> <lower> <higher>"
    // for the order of all listener calls, and "<tag> pre|post <step> <lower>
    // <higher> <count> [<iteration>] <ni0 ti0 ni1 ti1>" with their arguments
    auto shapes = [&world](ContactID id) {
        const auto& c = GetContact(world, id);
        const auto a = to_underlying(GetShapeA(c)), b = to_underlying(GetShapeB(c));
        return std::pair<unsigned, unsigned>(unsigned(a < b ? a : b), unsigned(a < b ? b : a));
    };
    SetPreSolveContactListener(world, [&step, tag, shapes](ContactID id, const Manifold& old) {
        const auto sh = shapes(id);
        std::printf("%s call %d pre %u %u\n", tag, step, sh.first, sh.second);
        std::printf("%s pre %d %u %u %d", tag, step, sh.first, sh.second, int(old.GetPointCount()));
        for (auto k = 0u; k < 2u; ++k) {
            const bool has = k < old.GetPointCount();
            std::printf(" %a %a", has ? double(StripUnit(old.GetPoint(k).normalImpulse)) : 0.0,
                        has ? double(StripUnit(old.GetPoint(k).tangentImpulse)) : 0.0);
        }
        std::printf("\n");
    });
    SetPostSolveContactListener(world, [&step, tag, shapes](ContactID id, const ContactImpulsesList& imp, unsigned it) {
        const auto sh = shapes(id);
        std::printf("%s call %d post %u %u\n", tag, step, sh.first, sh.second);
        std::printf("%s post %d %u %u %d %u", tag, step, sh.first, sh.second, int(imp.GetCount()), it);
        for (auto k = 0u; k < 2u; ++k) {
            const bool has = k < imp.GetCount();
            std::printf(" %a %a", has ? double(StripUnit(imp.GetEntryNormal(k))) : 0.0,
                        has ? double(StripUnit(imp.GetEntryTanget(k))) : 0.0);
        }
        std::printf("\n");
    });
    auto conf = StepConf{};
    conf.doToi = doToi;
    auto boxContact = std::optional<ContactID>{};
    for (step = 1; step <= 60; ++step) {
        Step(world, conf);
        for (const auto& kc : GetContacts(world)) {
            const auto id = std::get<ContactID>(kc);
            const auto& c = GetContact(world, id);
            if ((GetBodyA(c) == box || GetBodyB(c) == box) && IsTouching(c) && !boxContact) {
                boxContact = id;
                std::printf("%s id %d\n", tag, step);
            }
        }
        if (boxContact) {
            // the ID stays the contact's own while it lives
            const auto& c = GetContact(world, *boxContact);
            if (GetBodyA(c) != box && GetBodyB(c) != box) std::printf("%s id_changed %d\n", tag, step);
            if (step == 20) {
                auto m = GetContact(world, *boxContact);
                m.SetTangentSpeed(2_mps);
                m.SetFriction(0.8f);
                SetContact(world, *boxContact, m);
            }
            if (step == 45) {
                auto m = GetContact(world, *boxContact);
                m.UnsetEnabled();
                SetContact(world, *boxContact, m);
            }
        }
        const auto xf = GetTransformation(world, box);
        std::printf("%s pos %d %a %a %a\n", tag, step, double(StripUnit(GetX(xf.p))), double(StripUnit(GetY(xf.p))),
                    double(StripUnit(GetAngle(xf.q))));
    }
}

// Multi-child shapes: a ChainShapeConf terrain and two bodies of MultiShapeConf
// hulls and a disk falling onto it, 30 steps.  Prints "<tag> tcontact <step>
// <shapeA> <childA> <shapeB> <childB> <touching>" for every contact at steps 1,
// 10, 20 and 30 (lower shape first), "<tag> tpos <step> <body> x y angle" every 5
// steps and "<tag> tmass <body> invMass invRotInertia" once.
void Terrain(playrho::d2::World& world, const char* tag) {
    using namespace playrho;
    using namespace playrho::d2;
    auto chain = ChainShapeConf{};
    std::vector<Length2> pts;
    for (int i = 0; i <= 20; ++i) {
        const auto x = Real(-10 + i);
        pts.push_back(Length2{x * 1_m, Real(0.6) * Real(std::sin(double(x) * 0.7)) * 1_m});
    }
    chain.Set(pts);
    chain.UseFriction(0.6f);
    const auto ground = CreateShape(world, chain);
    CreateBody(world, BodyConf{}.Use(ground));
    auto hull = [](std::initializer_list<Length2> pts) {
        auto vs = VertexSet{};
        for (const auto& p : pts) vs.add(p);
        return vs;
    };
    auto l = MultiShapeConf{};
    l.AddConvexHull(hull({Length2{-0.6_m, -0.2_m}, Length2{0.6_m, -0.2_m}, Length2{0.6_m, 0.2_m},
                          Length2{-0.6_m, 0.2_m}}));
    l.AddConvexHull(hull({Length2{-0.6_m, 0.2_m}, Length2{-0.2_m, 0.2_m}, Length2{-0.2_m, 0.9_m},
                          Length2{-0.6_m, 0.9_m}}));
    l.UseDensity(1_kgpm2).UseFriction(0.5f);
    const auto lshape = CreateShape(world, l);
    std::vector<BodyID> bodies;
    bodies.push_back(CreateBody(world, BodyConf{}.Use(BodyType::Dynamic).Use(lshape)
                                           .UseLocation(Length2{-5_m, 3_m}).UseAngle(0.3_rad)
                                           .UseLinearAcceleration(EarthlyGravity)));
    bodies.push_back(CreateBody(world, BodyConf{}.Use(BodyType::Dynamic).Use(lshape)
                                           .UseLocation(Length2{4_m, 2.5_m}).UseAngle(-1.1_rad)
                                           .UseLinearAcceleration(EarthlyGravity)));
    const auto disk = CreateShape(world, DiskShapeConf{}.UseRadius(0.35_m).UseDensity(1_kgpm2));
    bodies.push_back(CreateBody(world, BodyConf{}.Use(BodyType::Dynamic).Use(disk)
                                           .UseLocation(Length2{0.3_m, 2_m}).UseLinearAcceleration(EarthlyGravity)));
    for (const auto& b : bodies)
        std::printf("%s tmass %u %a %a\n", tag, unsigned(to_underlying(b)), double(StripUnit(GetInvMass(world, b))),
                    double(StripUnit(GetInvRotInertia(world, b))));
    auto conf = StepConf{};
    conf.doToi = false;
    for (auto step = 1; step <= 30; ++step) {
        Step(world, conf);
        if (step == 1 || step == 10 || step == 20 || step == 30) {
            for (const auto& kc : GetContacts(world)) {
                const auto& c = GetContact(world, std::get<ContactID>(kc));
                auto a = std::make_pair(unsigned(to_underlying(GetShapeA(c))), unsigned(GetChildIndexA(c)));
                auto b = std::make_pair(unsigned(to_underlying(GetShapeB(c))), unsigned(GetChildIndexB(c)));
                if (b < a) std::swap(a, b);
                std::printf("%s tcontact %d %u %u %u %u %d\n", tag, step, a.first, a.second, b.first, b.second,
                            IsTouching(c) ? 1 : 0);
            }
        }
        if (step % 5 == 0 && step <= 30) {
            for (const auto& b : bodies) {
                const auto xf = GetTransformation(world, b);
                std::printf("%s tpos %d %u %a %a %a\n", tag, step, unsigned(to_underlying(b)),
                            double(StripUnit(GetX(xf.p))), double(StripUnit(GetY(xf.p))),
                            double(StripUnit(GetAngle(xf.q))));
            }
        }
    }
}

} // namespace

int main() {
    using namespace playrho;
    using namespace playrho::d2;
    constexpr auto boxX = +0_m;
    constexpr auto boxY = -10_m;
    constexpr auto boxWidth = 50_m;
    constexpr auto bodyHeight = 10_m;
    constexpr auto maxSteps = 60;
    constexpr auto ballStart = Length2{0_m, 4_m};
    auto world = World{GpuWorld{}};
    const auto box = CreateShape(world, PolygonShapeConf{}.SetAsBox(boxWidth, bodyHeight));
    CreateBody(world, BodyConf{}.Use(box).UseLocation(Length2{boxX, boxY}));
    const auto diskShape = CreateShape(world, DiskShapeConf{}.UseRadius(1_m));
    const auto ball = CreateBody(world, BodyConf{}
                                            .Use(BodyType::Dynamic)
                                            .Use(diskShape)
                                            .UseLocation(ballStart)
                                            .UseLinearAcceleration(EarthlyGravity));
    std::printf("bodies %u\n", static_cast<unsigned>(GetBodies(world).size()));
    std::printf("shapes %u\n", static_cast<unsigned>(GetShapeRange(world)));
    std::printf("mass %a %a\n", static_cast<double>(StripUnit(GetInvMass(world, ball))),
                static_cast<double>(StripUnit(GetInvRotInertia(world, ball))));
    std::printf("type %d\n", static_cast<int>(GetType(world, ball)));
    CheckJoints();
    {
        auto ref = World{};
        Conveyor(ref, "ref", true);
        auto ref2 = World{};
        Conveyor(ref2, "rnt", false);
        auto ref3 = World{};
        Terrain(ref3, "ref");
    }
    const auto conf = StepConf{};
    try {
        for (auto i = 0; i < maxSteps; ++i) {
            Step(world, conf);
            const auto transformation = GetTransformation(world, ball);
            const auto location = GetLocation(transformation);
            const auto angle = GetAngle(transformation);
            std::printf("step %d %a %a %a\n", i, static_cast<double>(StripUnit(GetX(location))),
                        static_cast<double>(StripUnit(GetY(location))), static_cast<double>(StripUnit(angle)));
        }
        auto gpu = World{GpuWorld{}};
        Conveyor(gpu, "gpu", true);
        auto gpu2 = World{GpuWorld{}};
        Conveyor(gpu2, "gnt", false);
        auto gpu3 = World{GpuWorld{}};
        Terrain(gpu3, "gpu");
    } catch (const std::exception& e) {
        std::printf("error %s\n", e.what());
        return 3;
    }
    return 0;
}
