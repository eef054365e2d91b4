// host_world_check.cpp -- drives prgpu::HostWorld (the C++ host layer) the way
// a PlayRho program drives a World: CreateBody, CreateShape + attach, CreateJoint,
// Step, GetBody, SetBody.  Reads a scene in the reference driver's text form on
// stdin (body / shape / joint / jointx lines, hexadecimal floats), then commands:
//   step N                 N steps with the default StepConf
//   teleport B x y         SetBody of body B with a new location (velocities kept)
//   destroy_body B         Destroy(BodyID)
//   dump                   one line per body: "b x y angle vx vy w awake" (hex floats)
//   contacts               one line per contact: "c proxyA proxyB bodyA bodyB touching count"
// Output goes to stdout; errors exit non-zero with the status code.
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "host_world.hpp"

using prgpu::HostBody;
using prgpu::HostJoint;
using prgpu::HostShape;
using prgpu::HostWorld;

static float hexf(const std::string& s) { return std::strtof(s.c_str(), nullptr); }

int main() {
    HostWorld world;
    std::vector<uint32_t> body_ids;
    prgpu_step_conf conf;
    prgpu_default_step_conf(&conf);
    conf.doToi = 0;  // compared with the batch API's regular-phase steps
    std::string line;
    try {
        while (std::getline(std::cin, line)) {
            std::istringstream in(line);
            std::string cmd;
            in >> cmd;
            if (cmd == "body") {
                HostBody b;
                std::string v[11];
                in >> b.type;
                for (auto& x : v) in >> x;
                in >> b.flags;
                b.x = hexf(v[0]); b.y = hexf(v[1]); b.angle = hexf(v[2]);
                b.vx = hexf(v[3]); b.vy = hexf(v[4]); b.w = hexf(v[5]);
                b.ax = hexf(v[6]); b.ay = hexf(v[7]); b.aa = hexf(v[8]);
                b.linear_damping = hexf(v[9]); b.angular_damping = hexf(v[10]);
                body_ids.push_back(world.CreateBody(b));
            } else if (cmd == "shape") {
                uint32_t body, nv;
                HostShape s;
                std::string r, dens, fr, rest;
                in >> body >> s.kind >> nv >> r >> dens >> fr >> rest >> s.category >> s.mask >> s.group >> s.sensor;
                s.radius = hexf(r); s.density = hexf(dens); s.friction = hexf(fr); s.restitution = hexf(rest);
                for (uint32_t i = 0; i < 2 * nv; ++i) {
                    std::string x;
                    in >> x;
                    s.verts.push_back(hexf(x));
                }
                const uint32_t sid = world.CreateShape(s);
                HostBody b = world.GetBody(body_ids.at(body));
                b.shapes.push_back(sid);  // Attach(world, body, shape)
                world.SetBody(body_ids.at(body), b);
            } else if (cmd == "joint") {
                HostJoint j;
                uint32_t a, b;
                std::string an[4], ref, lo, up, ms, mt;
                in >> a >> b >> an[0] >> an[1] >> an[2] >> an[3] >> ref >> j.enable_limit >> lo >> up >> j.enable_motor >>
                    ms >> mt >> j.collide_connected;
                j.body_a = body_ids.at(a); j.body_b = body_ids.at(b);
                j.anchor_a[0] = hexf(an[0]); j.anchor_a[1] = hexf(an[1]);
                j.anchor_b[0] = hexf(an[2]); j.anchor_b[1] = hexf(an[3]);
                j.reference_angle = hexf(ref); j.lower = hexf(lo); j.upper = hexf(up);
                j.motor_speed = hexf(ms); j.max_motor_torque = hexf(mt);
                world.CreateJoint(j);
            } else if (cmd == "jointx") {
                HostJoint j;
                uint32_t a, b;
                std::string an[4], e[8];
                in >> j.kind >> a >> b >> an[0] >> an[1] >> an[2] >> an[3] >> j.collide_connected >> j.enable_limit >>
                    j.enable_motor;
                for (auto& x : e) in >> x;
                j.body_a = body_ids.at(a); j.body_b = body_ids.at(b);
                j.anchor_a[0] = hexf(an[0]); j.anchor_a[1] = hexf(an[1]);
                j.anchor_b[0] = hexf(an[2]); j.anchor_b[1] = hexf(an[3]);
                for (int k = 0; k < 8; ++k) j.extra[k] = hexf(e[k]);
                world.CreateJoint(j);
            } else if (cmd == "step") {
                int n = 0;
                in >> n;
                for (int i = 0; i < n; ++i) world.Step(conf);
            } else if (cmd == "teleport") {
                uint32_t b;
                std::string x, y;
                in >> b >> x >> y;
                HostBody body = world.GetBody(body_ids.at(b));
                body.x = hexf(x); body.y = hexf(y);
                world.SetBody(body_ids.at(b), body);
            } else if (cmd == "destroy_body") {
                uint32_t b;
                in >> b;
                world.DestroyBody(body_ids.at(b));
            } else if (cmd == "dump") {
                for (uint32_t i = 0; i < body_ids.size(); ++i) {
                    if (!world.BodyAlive(body_ids[i])) continue;
                    const HostBody& b = world.GetBody(body_ids[i]);
                    std::printf("b %u %a %a %a %a %a %a %d\n", i, b.x, b.y, b.angle, b.vx, b.vy, b.w,
                                (b.flags & PRGPU_BODY_AWAKE) ? 1 : 0);
                }
            } else if (cmd == "contacts") {
                for (const auto& c : world.Contacts())
                    std::printf("c %u %u %u %u %d %d\n", c.proxy_a, c.proxy_b, c.body_a, c.body_b, c.touching ? 1 : 0,
                                c.count);
            }
        }
    } catch (const prgpu::Error& e) {
        std::fprintf(stderr, "error %d: %s\n", e.code, e.what());
        return 10 + e.code;
    }
    return 0;
}
