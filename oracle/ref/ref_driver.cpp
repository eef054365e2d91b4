// ref_driver.cpp -- runs a scene through the PlayRho reference's public API
// (World, CreateBody, CreateShape, Attach, CreateJoint, Step, Get*) and prints
// the resulting state with hexadecimal floats.  Used only as a checker of the
// oracle in the container where the reference sources are present.
//
// Input (stdin), one record per line:
//   conf <StepConf field> <value> ...        overrides of StepConf defaults
//   body type px py angle vx vy av ax ay aa linDamp angDamp flags
//        (flags: 1 allow sleep, 2 awake, 4 fixed rotation, 8 enabled, 16 bullet)
//   shape body kind nverts radius density friction restitution cat mask group sensor x0 y0 ...
//   joint bodyA bodyB lax lay lbx lby refAngle enableLimit lower upper enableMotor
//         motorSpeed maxMotorTorque collideConnected
//   step N            (runs N steps; may repeat)
//   dump              (prints bodies, contacts and proxies)
//   ray x1 y1 x2 y2 maxFraction   (prints every shape the ray hits)
//   substep 0|1       (SetSubStepping)
//   defaults          (prints the StepConf defaults)
#include "ref_scene.hpp"

#include <playrho/d2/DynamicTree.hpp>
#include <playrho/d2/RayCastOutput.hpp>

#include <algorithm>
#include <cstdio>
#include <iostream>
#include <map>
#include <sstream>
#include <string>

using namespace playrho;
using namespace playrho::d2;

namespace {

using refscene::hex;
using refscene::rd;

void printDefaults()
{
    const auto c = StepConf{};
    std::printf("defaults");
    hex(c.deltaTime / 1_s); hex(c.dtRatio); hex(c.minStillTimeToSleep / 1_s); hex(c.linearSlop / 1_m);
    hex(c.angularSlop / 1_rad); hex(c.regResolutionRate); hex(c.regMinSeparation / 1_m);
    hex(c.regMinMomentum / 1_Ns); hex(c.velocityThreshold / 1_mps); hex(c.maxTranslation / 1_m);
    hex(c.maxRotation / 1_rad); hex(c.maxLinearCorrection / 1_m); hex(c.maxAngularCorrection / 1_rad);
    hex(c.linearSleepTolerance / 1_mps); hex(c.angularSleepTolerance / (1_rad / 1_s));
    hex(c.displaceMultiplier); hex(c.aabbExtension / 1_m); hex(c.maxCirclesRatio);
    std::printf(" %d %d %d %d\n", int(c.regVelocityIters), int(c.regPositionIters), int(c.doWarmStart),
                int(c.doBlocksolve));
}

void dump(const World& world, const StepStats& st)
{
    std::printf("complete %d\n", IsStepComplete(world) ? 1 : 0);
    std::printf("stats %u %u %u %u %u %u %u %u %u",
                unsigned(st.pre.proxiesCreated), unsigned(st.pre.contactsDestroyed),
                unsigned(st.pre.contactsAdded), unsigned(st.reg.islandsFound),
                unsigned(st.reg.islandsSolved), unsigned(st.reg.contactsAdded),
                unsigned(st.reg.bodiesSlept), unsigned(st.reg.sumPosIters), unsigned(st.reg.sumVelIters));
    hex(st.reg.minSeparation / 1_m); hex(st.reg.maxIncImpulse / 1_Ns);
    std::printf("\n");
    std::printf("toistats %u %u %u %u %u %u %u %u %u %u %u %u %u %u",
                unsigned(st.toi.islandsFound), unsigned(st.toi.islandsSolved), unsigned(st.toi.contactsFound),
                unsigned(st.toi.contactsAtMaxSubSteps), unsigned(st.toi.contactsUpdatedToi),
                unsigned(st.toi.contactsUpdatedTouching), unsigned(st.toi.contactsSkippedTouching),
                unsigned(st.toi.contactsAdded), unsigned(st.toi.proxiesMoved), unsigned(st.toi.sumPosIters),
                unsigned(st.toi.sumVelIters), unsigned(st.toi.maxDistIters), unsigned(st.toi.maxToiIters),
                unsigned(st.toi.maxRootIters));
    hex(st.toi.minSeparation / 1_m); hex(st.toi.maxIncImpulse / 1_Ns);
    std::printf("\n");
    const auto nb = GetBodyRange(world);
    for (auto i = decltype(nb){0}; i < nb; ++i) {
        const auto id = BodyID(i);
        const auto& b = GetBody(world, id);
        const auto sw = GetSweep(b);
        const auto v = GetVelocity(b);
        const auto xf = GetTransformation(b);
        std::printf("body %u", unsigned(i));
        hex(GetX(sw.pos1.linear) / 1_m); hex(GetY(sw.pos1.linear) / 1_m); hex(sw.pos1.angular / 1_rad);
        hex(GetX(v.linear) / 1_mps); hex(GetY(v.linear) / 1_mps); hex(v.angular / (1_rad / 1_s));
        hex(GetX(xf.p) / 1_m); hex(GetY(xf.p) / 1_m); hex(GetX(xf.q)); hex(GetY(xf.q));
        hex(StripUnit(GetInvMass(b))); hex(StripUnit(GetInvRotInertia(b)));
        hex(GetUnderActiveTime(b) / 1_s);
        std::printf(" %d\n", IsAwake(b) ? 1 : 0);
    }
    // Proxies in leaf-ID order; leaf IDs are mapped to their rank (creation order).
    const auto& tree = GetTree(world);
    std::map<DynamicTree::Size, int> rank;
    {
        int r = 0;
        for (auto i = DynamicTree::Size{0}; i < tree.GetNodeCapacity(); ++i) {
            if (DynamicTree::IsLeaf(tree.GetHeight(i))) rank[i] = r++;
        }
        for (const auto& e : rank) {
            const auto leaf = tree.GetLeafData(e.first);
            const auto aabb = tree.GetAABB(e.first);
            std::printf("proxy %d %u %u %u", e.second, unsigned(to_underlying(leaf.bodyId)),
                        unsigned(to_underlying(leaf.shapeId)), unsigned(leaf.childId));
            hex(aabb.ranges[0].GetMin() / 1_m); hex(aabb.ranges[1].GetMin() / 1_m);
            hex(aabb.ranges[0].GetMax() / 1_m); hex(aabb.ranges[1].GetMax() / 1_m);
            std::printf("\n");
        }
    }
    const auto contacts = GetContacts(world);
    int k = 0;
    for (const auto& kc : contacts) {
        const auto key = std::get<ContactKey>(kc);
        const auto cid = std::get<ContactID>(kc);
        const auto c = GetContact(world, cid);
        const auto m = GetManifold(world, cid);
        std::printf("contact %d %u %d %d %u %u %u %u %u %u %d %d %d", k++, unsigned(to_underlying(cid)),
                    rank[key.GetMin()], rank[key.GetMax()],
                    unsigned(to_underlying(GetBodyA(c))), unsigned(to_underlying(GetShapeA(c))),
                    unsigned(GetChildIndexA(c)), unsigned(to_underlying(GetBodyB(c))),
                    unsigned(to_underlying(GetShapeB(c))), unsigned(GetChildIndexB(c)),
                    IsTouching(c) ? 1 : 0, int(m.GetType()), int(m.GetPointCount()));
        hex(GetX(m.GetLocalNormal())); hex(GetY(m.GetLocalNormal()));
        hex(GetX(m.GetLocalPoint()) / 1_m); hex(GetY(m.GetLocalPoint()) / 1_m);
        for (auto i = 0; i < 2; ++i) {
            const auto p = (i < m.GetPointCount()) ? m.GetPoint(i) : Manifold::Point{};
            hex(GetX(p.localPoint) / 1_m); hex(GetY(p.localPoint) / 1_m);
            hex(p.normalImpulse / 1_Ns); hex(p.tangentImpulse / 1_Ns);
        }
        for (auto i = 0; i < 2; ++i) {
            const auto p = (i < m.GetPointCount()) ? m.GetPoint(i) : Manifold::Point{};
            std::printf(" %d %d %d %d", int(p.contactFeature.typeA), int(p.contactFeature.indexA),
                        int(p.contactFeature.typeB), int(p.contactFeature.indexB));
        }
        std::printf("\n");
    }
}

} // namespace

int main()
{
    auto world = World{};
    // BeginContact / EndContact calls as "ev kind lowerShape higherShape" lines
    const auto event = [&world](int kind, ContactID id) {
        const auto& c = GetContact(world, id);
        const auto a = to_underlying(GetShapeA(c)), b = to_underlying(GetShapeB(c));
        std::printf("ev %d %u %u\n", kind, static_cast<unsigned>(a < b ? a : b), static_cast<unsigned>(a < b ? b : a));
    };
    SetBeginContactListener(world, [event](ContactID id) { event(1, id); });
    SetEndContactListener(world, [event](ContactID id) { event(2, id); });
    // PreSolveContact / PostSolveContact calls as "solve kind lowerShape higherShape
    // count iteration ni0 ti0 ni1 ti1" lines (kind 3: the manifold before the
    // update; kind 4: the solved impulses and the iteration argument)
    const auto solveCall = [&world](int kind, ContactID id, int count, unsigned iter, const double* imp) {
        const auto& c = GetContact(world, id);
        const auto a = to_underlying(GetShapeA(c)), b = to_underlying(GetShapeB(c));
        std::printf("solve %d %u %u %d %u", kind, static_cast<unsigned>(a < b ? a : b),
                    static_cast<unsigned>(a < b ? b : a), count, iter);
        for (int k = 0; k < 4; ++k) hex(imp[k]);
        std::printf("\n");
    };
    SetPreSolveContactListener(world, [solveCall](ContactID id, const Manifold& old) {
        double imp[4] = {0, 0, 0, 0};
        const auto n = int(old.GetPointCount());
        for (int k = 0; k < n; ++k) {
            imp[2 * k] = double(old.GetPoint(k).normalImpulse / 1_Ns);
            imp[2 * k + 1] = double(old.GetPoint(k).tangentImpulse / 1_Ns);
        }
        solveCall(3, id, n, 0u, imp);
    });
    SetPostSolveContactListener(world, [solveCall](ContactID id, const ContactImpulsesList& ci, unsigned iter) {
        double imp[4] = {0, 0, 0, 0};
        const auto n = int(ci.GetCount());
        for (int k = 0; k < n; ++k) {
            imp[2 * k] = double(ci.GetEntryNormal(k) / 1_Ns);
            imp[2 * k + 1] = double(ci.GetEntryTanget(k) / 1_Ns);
        }
        solveCall(4, id, n, iter, imp);
    });
    auto conf = StepConf{};
    conf.doToi = false;
    auto stats = StepStats{};
    std::string line;
    while (std::getline(std::cin, line)) {
        std::istringstream in(line);
        std::string tag;
        if (!(in >> tag)) continue;
        if (tag == "defaults") {
            printDefaults();
        }
        else if (refscene::ApplyRecord(world, conf, tag, in)) {
        }
        else if (tag == "step") {
            int n = 0; in >> n;
            for (int i = 0; i < n; ++i) stats = Step(world, conf);
        }
        else if (tag == "substep") {
            int flag = 0; in >> flag;
            SetSubStepping(world, flag != 0);
        }
        else if (tag == "ray") {
            // RayCast(World, RayCastInput, callback) answering ResetRay: every hit as
            // "rayhit shape point.x point.y normal.x normal.y", then "rayend"
            double x1, y1, x2, y2, f;
            in >> x1 >> y1 >> x2 >> y2 >> f;
            auto input = RayCastInput{};
            input.p1 = Length2{Real(x1) * Meter, Real(y1) * Meter};
            input.p2 = Length2{Real(x2) * Meter, Real(y2) * Meter};
            input.maxFraction = UnitInterval<Real>(Real(f));
            RayCast(world, input, [](BodyID, ShapeID shape, ChildCounter, const Length2& pt, const UnitVec& n) {
                std::printf("rayhit %u", static_cast<unsigned>(to_underlying(shape)));
                hex(double(StripUnit(GetX(pt)))); hex(double(StripUnit(GetY(pt))));
                hex(double(GetX(n))); hex(double(GetY(n)));
                std::printf("\n");
                return RayCastOpcode::ResetRay;
            });
            std::printf("rayend\n");
            std::fflush(stdout);
        }
        else if (tag == "dump") {
            dump(world, stats);
            std::printf("end\n");
            std::fflush(stdout);
        }
    }
    return 0;
}
