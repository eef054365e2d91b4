// gpuworld_check.cpp -- the reference's HelloWorld program with two changes:
// the World is constructed over GpuWorld, and the step configuration turns off
// TOI (the GPU step is the regular phase).  Everything else goes through
// PlayRho's own World API (CreateShape, CreateBody with BodyConf::Use(shape),
// Step, GetTransformation, ...).
//
// Prints, one per line:
//   bodies N / shapes N / mass <invMass> <invRotI> / type T     after set-up
//   step <i> <x> <y> <angle>                                    per step (needs a GPU)
//   error <what>                                                when stepping fails
#include <cstdio>
#include <exception>

#include "playrho/d2/BasicAPI.hpp"

#include "GpuWorld.hpp"

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
    auto conf = StepConf{};
    conf.doToi = false;
    try {
        for (auto i = 0; i < maxSteps; ++i) {
            Step(world, conf);
            const auto transformation = GetTransformation(world, ball);
            const auto location = GetLocation(transformation);
            const auto angle = GetAngle(transformation);
            std::printf("step %d %a %a %a\n", i, static_cast<double>(StripUnit(GetX(location))),
                        static_cast<double>(StripUnit(GetY(location))), static_cast<double>(StripUnit(angle)));
        }
    } catch (const std::exception& e) {
        std::printf("error %s\n", e.what());
        return 3;
    }
    return 0;
}
