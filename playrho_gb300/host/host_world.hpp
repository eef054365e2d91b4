// host_world.hpp -- the host side of one GPU-stepped world, in plain C++17 over
// the C ABI of include/prgpu.h (no PlayRho headers needed).
//
// HostWorld keeps what the reference's AabbTreeWorld keeps on the host for the
// world-step path -- bodies, shapes, joints in ID-indexed pools with free lists
// (Library/source/playrho/d2/AabbTreeWorld.cpp:1019-1044 CreateBody, :1132-1157
// CreateShape, :1234-1257 CreateJoint; ObjectPool.hpp) -- and mirrors the body
// states the GPU computes.  The GPU batch (one world) is built on the first
// Step after the set of bodies, shapes, joints or attachments changed; body
// position and velocity changes between steps are uploaded in place
// (SetBody, AabbTreeWorld.cpp:2723-2795), other body changes rebuild the batch.
// IDs are stable while an entity lives and are reused after it is destroyed, as
// the reference's pools reuse them.
//
// The C++ drop-in (GpuWorld.hpp) converts PlayRho's Body/Shape/Joint values
// to and from these records; tests drive HostWorld directly on a GPU machine.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "prgpu.h"

namespace prgpu {

// Body as the step sees it: origin location and angle (Transformation), velocity,
// acceleration, damping, flags (PRGPU_BODY_*), mass data, under-active time and
// the shapes attached to it (Body.hpp:486-522, GetShapes :1460).
struct HostBody {
    int32_t type = PRGPU_STATIC;
    float x = 0.f, y = 0.f, angle = 0.f;
    float vx = 0.f, vy = 0.f, w = 0.f;
    float ax = 0.f, ay = 0.f, aa = 0.f;
    float linear_damping = 0.f, angular_damping = 0.f;
    uint32_t flags = PRGPU_BODY_ALLOW_SLEEP | PRGPU_BODY_AWAKE | PRGPU_BODY_ENABLED;
    // mass data: invMass, invRotInertia, local centre (SetMassData); only read
    // for dynamic bodies when explicit_mass is set, else derived from the shapes
    bool explicit_mass = false;
    float inv_mass = 0.f, inv_rot_inertia = 0.f, lcx = 0.f, lcy = 0.f;
    float under_active_time = 0.f;
    std::vector<uint32_t> shapes;
    float cx = 0.f, cy = 0.f;  // centre of mass the GPU holds (set by a step; read-only)
};

// Shape configuration (DiskShapeConf / PolygonShapeConf / EdgeShapeConf +
// BaseShapeConf): vertices in the body frame (disk: its centre; polygon: in the
// order PolygonShapeConf stores them), vertex radius, material and filter.
struct HostShape {
    int32_t kind = PRGPU_DISK;
    std::vector<float> verts;  // x0 y0 x1 y1 ...
    // a shape of several children (ChainShapeConf: edges, MultiShapeConf: convex
    // hulls): each child's vertices, kind then being the children's kind; each
    // child becomes a shape of the batch with its own proxy (prgpu_batch_desc::shape_owner)
    std::vector<std::vector<float>> children;
    float radius = 0.f, density = 0.f, friction = 0.2f, restitution = 0.f;
    int32_t category = 1, mask = 0xffff, group = 0, sensor = 0;
};

// RevoluteJointConf (RevoluteJointConf.hpp): bodies, local anchors, limits, motor.
struct HostJoint {
    int32_t kind = PRGPU_JOINT_REVOLUTE;                         // prgpu_joint_kind
    uint32_t body_a = 0, body_b = 0;
    float anchor_a[2] = {0.f, 0.f}, anchor_b[2] = {0.f, 0.f};
    float reference_angle = 0.f, lower = 0.f, upper = 0.f, motor_speed = 0.f, max_motor_torque = 0.f;
    int32_t enable_limit = 0, enable_motor = 0, collide_connected = 0;
    float extra[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};   // the other kinds' parameters (prgpu.h);
                                                                 // a gear's coupled joints by joint ID
};

// A live contact after the last step (Contact.hpp + Manifold.hpp).
struct HostContact {
    uint32_t slot = 0;                                           // ContactID: stable for the contact's life
    uint64_t seq = 0;                                            // creation number (contact-list order)
    uint32_t body_a = 0, body_b = 0, shape_a = 0, shape_b = 0;  // IDs of the host pools
    uint32_t child_a = 0, child_b = 0;                           // child indices of the shapes
    uint32_t proxy_a = 0, proxy_b = 0;                           // tree leaf IDs (ContactKey)
    bool touching = false, sensor = false;
    int32_t type = 0, count = 0;                                 // Manifold::Type, point count
    float local_normal[2] = {0.f, 0.f}, local_point[2] = {0.f, 0.f};
    float point[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    float normal_impulse[2] = {0.f, 0.f}, tangent_impulse[2] = {0.f, 0.f};
    uint32_t feature[2] = {0u, 0u};                              // typeA | indexA << 8 | typeB << 16 | indexB << 24
    float friction = 0.f, restitution = 0.f, tangent_speed = 0.f;
    bool enabled = true;
};

// What the last step did to one live contact (prgpu_download_solve_records):
// the phases that updated it (1 pre-phase, 2 post-solve pass, 4 time-of-impact
// phase) and, if the regular phase solved it, its velocity constraint's impulses
// and its island's iteration argument.
struct HostSolveRecord {
    uint32_t slot = 0;
    uint32_t phases = 0;
    bool solved = false;
    int32_t count = 0;     // velocity-constraint points
    uint32_t iter = 255;   // StepConf::InvalidIteration unless the island reached tolerance
    float normal_impulse[2] = {0.f, 0.f}, tangent_impulse[2] = {0.f, 0.f};
};

// Errors carry the C ABI's status code; the drop-in maps them onto the
// reference's exception types.
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& what) : std::runtime_error(what), code(c) {}
};

class HostWorld {
public:
    explicit HostWorld(int device = 0) : device_(device) {}
    HostWorld(const HostWorld& other);
    HostWorld& operator=(const HostWorld& other);
    ~HostWorld();

    // bodies
    uint32_t CreateBody(const HostBody& b);
    const HostBody& GetBody(uint32_t id) const;
    void SetBody(uint32_t id, const HostBody& b);
    void DestroyBody(uint32_t id);
    bool BodyAlive(uint32_t id) const { return id < bodies_.size() && body_live_[id]; }
    uint32_t BodyRange() const { return (uint32_t)bodies_.size(); }
    // shapes
    uint32_t CreateShape(const HostShape& s);
    const HostShape& GetShape(uint32_t id) const;
    void SetShape(uint32_t id, const HostShape& s);
    void DestroyShape(uint32_t id);
    bool ShapeAlive(uint32_t id) const { return id < shapes_.size() && shape_live_[id]; }
    uint32_t ShapeRange() const { return (uint32_t)shapes_.size(); }
    // joints
    uint32_t CreateJoint(const HostJoint& j);
    const HostJoint& GetJoint(uint32_t id) const;
    void SetJoint(uint32_t id, const HostJoint& j);
    void DestroyJoint(uint32_t id);
    bool JointAlive(uint32_t id) const { return id < joints_.size() && joint_live_[id]; }
    uint32_t JointRange() const { return (uint32_t)joints_.size(); }

    // One world step on the GPU (Step(World&, StepConf), doToi = false).
    prgpu_step_stats Step(const prgpu_step_conf& conf);
    // Live contacts after the last step, in ContactKey order.
    const std::vector<HostContact>& Contacts();
    // SetContact / SetManifold on a live contact's slot (prgpu_set_contact, prgpu_set_manifold).
    void SetContact(uint32_t slot, bool enabled, float friction, float restitution, float tangent_speed);
    void SetManifold(uint32_t slot, int32_t type, int32_t count, const float head4[4], const float pts8[8]);
    // Keep solve records from the next step on (prgpu_set_solve_records), across rebuilds.
    void SetSolveRecords(bool enabled);
    // SetSubStepping / IsStepComplete (prgpu_set_sub_stepping, prgpu_get_step_complete).
    void SetSubStepping(bool enabled);
    bool StepComplete();
    // The live contacts the last step updated or solved.
    std::vector<HostSolveRecord> SolveRecords();
    // Fat AABB (minx miny maxx maxy) and (body, shape, child) of every proxy, by leaf ID order.
    void Proxies(std::vector<float>& aabb4, std::vector<uint32_t>& body_shape_child3);
    // The GPU shape (proxy) index of a shape's child, or ~0u (after a step).
    uint32_t ProxyOf(uint32_t shape, uint32_t child) const;
    void Clear();
    bool HasGpuBatch() const { return gpu_ != nullptr; }
    // The next Step rebuilds the GPU batch (entities changed since the last one).
    bool NeedsRebuild() const { return gpu_ == nullptr || rebuild_; }

private:
    void Build();         // (re)creates the GPU batch from the pools
    void UploadStates();  // position / velocity changes since the last step
    void Pull();          // body states after a step
    void Drop();
    void Check(int rc, const char* what) const;

    int device_ = 0;
    std::vector<HostBody> bodies_;
    std::vector<HostShape> shapes_;
    std::vector<HostJoint> joints_;
    std::vector<bool> body_live_, shape_live_, joint_live_;
    std::vector<uint32_t> body_free_, shape_free_, joint_free_;
    // GPU batch and the maps between its indices and the pools' IDs
    prgpu_world* gpu_ = nullptr;
    bool rebuild_ = true;
    std::vector<uint32_t> gpu_body_;          // GPU body index -> body ID
    std::vector<uint32_t> body_gpu_;          // body ID -> GPU body index (or ~0)
    std::vector<uint32_t> proxy_body_, proxy_shape_, proxy_child_;  // GPU shape (proxy) index -> IDs
    std::vector<float> lc_;                   // local centre per GPU body (x y)
    std::vector<bool> state_dirty_;           // body ID -> position/velocity set since the last step
    bool contacts_valid_ = false;
    std::vector<HostContact> contacts_;
    bool solve_records_ = false;
    bool sub_stepping_ = false;
};

}  // namespace prgpu
