// ref_bench.cpp -- times the PlayRho reference's own Step(World&, const StepConf&)
// over many independent worlds: the CPU baseline of the batched world step.  It is
// the reference's unmodified library (compiled from its sources by
// oracle/ref/Makefile) driven through its public API; nothing of the GPU path is
// involved.
//
// Input (stdin): the scene records of ref_scene.hpp for one world after another,
// each world introduced by a line "world"; then any of
//   run S     steps every world S times, untimed (settling, warm-up)
//   ready     prints "ready <worlds> <dynamic bodies>" and waits for a line "go", so
//             that several processes can start their timed steps together
//   time K    steps every world K times, timing each Step call, and prints
//             "result <seconds> <body-steps> <steps>"
// A body-step is one awake dynamic body advanced one step: before each timed Step
// the world's awake, enabled, dynamic bodies are counted (outside the timed
// calls); sleeping and static bodies are not counted.
#include "ref_scene.hpp"

#include <chrono>
#include <iostream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

using namespace playrho;
using namespace playrho::d2;

namespace {

std::size_t AwakeDynamicBodies(const World& world)
{
    std::size_t n = 0;
    for (const auto& id : GetBodies(world)) {
        const auto& b = GetBody(world, id);
        if (GetType(b) == BodyType::Dynamic && IsAwake(b) && IsEnabled(b)) ++n;
    }
    return n;
}

std::size_t DynamicBodies(const World& world)
{
    std::size_t n = 0;
    for (const auto& id : GetBodies(world)) {
        if (GetType(GetBody(world, id)) == BodyType::Dynamic) ++n;
    }
    return n;
}

} // namespace

int main()
{
    std::ios::sync_with_stdio(false);
    std::vector<std::unique_ptr<World>> worlds;
    auto conf = StepConf{};
    conf.doToi = false;
    std::string line;
    while (std::getline(std::cin, line)) {
        std::istringstream in(line);
        std::string tag;
        if (!(in >> tag)) continue;
        if (tag == "world") {
            worlds.push_back(std::make_unique<World>());
        }
        else if (tag == "run") {
            int n = 0; in >> n;
            for (int i = 0; i < n; ++i)
                for (auto& w : worlds) Step(*w, conf);
        }
        else if (tag == "ready") {
            std::size_t nb = 0;
            for (auto& w : worlds) nb += DynamicBodies(*w);
            std::printf("ready %zu %zu\n", worlds.size(), nb);
            std::fflush(stdout);
            std::string go;
            while (std::getline(std::cin, go) && go != "go") {}
        }
        else if (tag == "time") {
            int n = 0; in >> n;
            double seconds = 0.0;
            unsigned long long body_steps = 0;
            for (int i = 0; i < n; ++i) {
                for (auto& w : worlds) {
                    body_steps += AwakeDynamicBodies(*w);
                    const auto t0 = std::chrono::steady_clock::now();
                    Step(*w, conf);
                    const auto t1 = std::chrono::steady_clock::now();
                    seconds += std::chrono::duration<double>(t1 - t0).count();
                }
            }
            std::printf("result %.9f %llu %d\n", seconds, body_steps, n);
            std::fflush(stdout);
        }
        else if (worlds.empty()) {
            std::fprintf(stderr, "record before the first 'world' line: %s\n", tag.c_str());
            return 2;
        }
        else if (!refscene::ApplyRecord(*worlds.back(), conf, tag, in)) {
            std::fprintf(stderr, "unknown record %s\n", tag.c_str());
            return 2;
        }
    }
    return 0;
}
